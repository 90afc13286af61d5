// gas.cuh — trace-gas absorption tables and the per-layer absorption depth
// (rt_absorption.c, rt_atm.c:437-548).
//
// Six gases (H2O, O3, O2, CO2, NO2, CH4).  An AFGL atmosphere gives, on an
// ascending altitude grid, the number density n_g = mr_g * 1e-6 * n_total of
// every gas; a layered cross-section table gives sigma_g(table level,
// wavelength), where table level i sits at the altitude of AFGL level i.
// Columns are trapezoids on the AFGL grid with the cut layer interpolated
// linearly; sigma is linear in altitude and in wavelength.  The same
// functions serve the host (column depths for reporting) and the device
// (per-layer depths folded into the level grid), on host or device copies of
// the tables.
#pragma once
#include <cmath>
#include "../../include/ocrt_gb300.h"
#include "common.cuh"

#define OCRT_NGAS 6

struct GasDev {
    int nlev;                          // AFGL levels, altitude ascending
    const double *z;                   // [nlev] km
    const double *nd;                  // [OCRT_NGAS][nlev] number density, cm^-3
    double col_default[OCRT_NGAS];     // integrated AFGL column, molecules/cm^2
    double col_eff[OCRT_NGAS];         // column in use (default or caller's)
    int overridden[OCRT_NGAS];
    int avail[OCRT_NGAS], nwl[OCRT_NGAS], nlay[OCRT_NGAS];
    const double *wl[OCRT_NGAS];       // [nwl] nm, increasing
    const double *sig[OCRT_NGAS];      // [nlay][nwl] cm^2/molecule
};

// sigma of gas q at table level `layer` (clamped) and wavelength wl; NaN
// outside the table's grid, 0 for a gas without a table
// (rt_xsec_interp_layer, rt_absorption.c:347-371).
__host__ __device__ inline double gas_sigma_level(const GasDev &G, int q, int layer, double wl)
{
    if (!G.avail[q] || G.nwl[q] < 2) return 0.0;
    const int n = G.nwl[q];
    if (layer < 0) layer = 0;
    if (layer >= G.nlay[q]) layer = G.nlay[q] - 1;
    const double *w = G.wl[q];
    const double *s = G.sig[q] + (size_t)layer * n;
    if (wl < w[0] || wl > w[n - 1]) return NAN;
    if (wl == w[0]) return s[0];
    if (wl == w[n - 1]) return s[n - 1];
    int a = 0, b = n - 1;
    while (b - a > 1) {
        const int c = (a + b) / 2;
        if (w[c] <= wl) a = c; else b = c;
    }
    const double t = (wl - w[a]) / (w[b] - w[a]);
    return (1.0 - t) * s[a] + t * s[b];
}

// sigma of gas q at altitude z: linear between the bracketing table levels
// placed at the AFGL altitudes (rt_xsec_interp_layer_z, rt_absorption.c:378-412).
__host__ __device__ inline double gas_sigma(const GasDev &G, int q, double z, double wl)
{
    if (!G.avail[q]) return 0.0;
    const int nl = G.nlay[q];
    if (nl == 1 || z <= G.z[0]) return gas_sigma_level(G, q, 0, wl);
    if (z >= G.z[nl - 1]) return gas_sigma_level(G, q, nl - 1, wl);
    int a = 0, b = nl - 1;
    while (b - a > 1) {
        const int c = (a + b) / 2;
        if (G.z[c] <= z) a = c; else b = c;
    }
    const double dz = G.z[b] - G.z[a];
    if (dz <= 0.0) return gas_sigma_level(G, q, a, wl);
    const double t = (z - G.z[a]) / dz;
    return (1.0 - t) * gas_sigma_level(G, q, a, wl) + t * gas_sigma_level(G, q, b, wl);
}

// Column of gas q above altitude z, molecules/cm^2
// (rt_afgl_cumulative_column, rt_absorption.c:425-453).
__host__ __device__ inline double gas_column_above(const GasDev &G, int q, double z)
{
    const double *n = G.nd + (size_t)q * G.nlev;
    double cum = 0.0;
    for (int i = 0; i + 1 < G.nlev; ++i) {
        const double z1 = G.z[i], z2 = G.z[i + 1];
        if (z2 <= z) continue;
        const double lo = z1 < z ? z : z1;
        if (z2 <= lo) continue;
        const double f1 = (lo - z1) / (z2 - z1);
        const double n_lo = (1.0 - f1) * n[i] + f1 * n[i + 1];
        const double n_hi = n[i + 1];           // the layer top: fraction exactly 1
        cum += 0.5 * (n_lo + n_hi) * ((z2 - lo) * 1.0e5);
    }
    return cum;
}

// Column of gas q between z_lo and z_hi (rt_afgl_layer_column, rt_absorption.c:455-461).
__host__ __device__ inline double gas_column(const GasDev &G, int q, double z_lo, double z_hi)
{
    if (z_hi <= z_lo) return 0.0;
    return gas_column_above(G, q, z_lo) - gas_column_above(G, q, z_hi);
}

// Absorption depth of the solver layer spanning altitudes z_a, z_b at wl: the
// sum over gases of sigma(z_mid) times the layer column, a caller's column
// spread in proportion to the AFGL layer column (rt_atm.c:451-499).
__host__ __device__ inline double gas_layer_depth(const GasDev &G, double z_a, double z_b, double wl)
{
    double z_hi = z_a, z_lo = z_b;
    if (z_lo > z_hi) { const double t = z_lo; z_lo = z_hi; z_hi = t; }
    const double z_mid = 0.5 * (z_lo + z_hi);
    double dt = 0.0;
    for (int q = 0; q < OCRT_NGAS; ++q) {
        double N;
        if (G.overridden[q]) {
            const double nd = G.col_default[q];
            N = nd > 0.0 ? G.col_eff[q] * (gas_column(G, q, z_lo, z_hi) / nd) : 0.0;
        } else {
            N = gas_column(G, q, z_lo, z_hi);
        }
        dt += gas_sigma(G, q, z_mid, wl) * N;
    }
    return dt;
}

// The library's absorption state: host tables (for column depths) and one
// device allocation holding the same tables plus a device copy of GasDev.
struct ocrt_gas {
    GasDev host;                       // pointers into the host vectors below
    GasDev *dev;                       // device copy, pointers into dbuf
    void *dbuf;
    double *hbuf;                      // host tables, one allocation
};

__global__ void k_gas_apply(PixDev *px, int P, double *h, double *ch, double *xd, double *yd, const double *z,
                            double *tabs);
