/*
 * ocrt_oracle.c — FP64 CPU restatement of the OCRT SOS solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GB300
 * library and the timed CPU "port" baseline; the product never links it.
 * It is pinned against the reference C solver built from its own sources
 * (oracle/Makefile -> oracle/_ref) and against the reference's published
 * golden values (tests/golden/).
 *
 * Every routine restates one reference routine; the reference file:line is
 * given beside it (paths relative to code/OCRT_C/src/).  The layout is this
 * oracle's own: directions are kept in signed-ring arrays indexed j+n, fields
 * as [level][signed direction], exactly the mathematical objects of the
 * reference, not its packing.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/ocrt_gb300.h"

int ocrt_oracle_solve_case_layers(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                                  const ocrt_layers *layers, ocrt_result *out, ocrt_diag *diag);
static int solve_impl(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                      const ocrt_layers *layers, ocrt_lut *lut, ocrt_result *out, ocrt_diag *diag);

#define PI 3.14159265358979323846

/* Hooks of the coupled atmosphere-ocean driver (ocean.c) into the atmosphere
 * solve, thread-local so that batched oracle solves stay independent:
 *   bottom_only: the solar primary and the surface seeds are dropped, only
 *     the bottom source drives the field (rt_solver.c:949-954,
 *     rt_surface_boundary.c:553-569);
 *   ext_*: upward radiance per mode and ring node emitted at the bottom of
 *     the atmosphere, attenuated upward and added to order 1 and the total
 *     (rt_surface_boundary.c:495-527);
 *   boa_*: the converged downward total at the bottom per mode and ring node
 *     (rt_solver.c:1050-1076);
 *   mu / w / n: the ring of the solve. */
typedef struct {
    int bottom_only;
    const double *ext_I, *ext_Q, *ext_U;
    int ext_mmax;
    double *boa_I, *boa_Q, *boa_U;
    double mu[260], w[260];
    int n;
} atm_hooks_t;
static _Thread_local atm_hooks_t *g_atm_hooks;
#define DEPOL 0.0279                  /* rt_solver.c:646 */
#define Z_TOP_KM 100.0                /* rt_atm.c:219, 306 */
#define MAX_RING 130
#define MAX_M1 256                    /* Fourier modes 0..255 */
#define DEDUP_TOL 1.0e-12             /* rt_angle_grid.h:12 */

/* ======================================================================
 * Quadrature: Gauss-Legendre positive nodes, Newton from a Tricomi guess
 * (rt_quadrature.c:20-61).  Nodes ascending, weights sum to 1.
 * ==================================================================== */
static void legendre_pair(int order, double t, double *p_n, double *p_nm1)
{
    double a = 1.0, b = t;
    for (int k = 1; k < order; ++k) {
        const double c = ((2.0 * k + 1.0) * t * b - (double)k * a) / (double)(k + 1);
        a = b;
        b = c;
    }
    *p_n = b;
    *p_nm1 = a;
}

int ocrt_oracle_gauss(int n, double *mu, double *w)
{
    if (n < 1 || !mu || !w) return -1;
    const int order = 2 * n;
    for (int k = 1; k <= n; ++k) {
        double t = cos(PI * ((double)k - 0.25) / ((double)order + 0.5));
        double pn = 0.0, pm = 0.0, dp = 1.0;
        int ok = 0;
        for (int it = 0; it < 100; ++it) {
            legendre_pair(order, t, &pn, &pm);
            dp = (double)order * (t * pn - pm) / (t * t - 1.0);
            const double step = -pn / dp;
            t += step;
            if (fabs(step) < 1.0e-15 * (fabs(t) + 1.0)) { ok = 1; break; }
        }
        if (!ok) return -2;
        legendre_pair(order, t, &pn, &pm);
        dp = (double)order * (t * pn - pm) / (t * t - 1.0);
        mu[n - k] = t;
        w[n - k] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
    return 0;
}

/* Sorted insertion of a zero-weight node with de-duplication
 * (rt_angle_grid.c:37-73).  Returns the ring index (0-based) of mu_new. */
static int ring_insert(double *mu, double *w, int *n_total, double mu_new)
{
    int lo = 0, hi = *n_total;
    while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (mu[mid] < mu_new) lo = mid + 1; else hi = mid;
    }
    if (lo > 0 && fabs(mu[lo - 1] - mu_new) < DEDUP_TOL) return lo - 1;
    if (lo < *n_total && fabs(mu[lo] - mu_new) < DEDUP_TOL) return lo;
    for (int i = *n_total; i > lo; --i) { mu[i] = mu[i - 1]; w[i] = w[i - 1]; }
    mu[lo] = mu_new;
    w[lo] = 0.0;
    *n_total += 1;
    return lo;
}

/* ======================================================================
 * Rayleigh optical depth, Bodhaine et al. 1999 (rt_rayleigh.c:46-52,
 * 84-96, 137-146, 198-238): CO2 360 ppm, latitude 45 deg, sea level.
 * ==================================================================== */
static double gravity_wgs84(double lat_deg, double z_m)
{
    const double lat = lat_deg * PI / 180.0;
    const double s1 = sin(lat) * sin(lat);
    const double s2 = sin(2.0 * lat) * sin(2.0 * lat);
    return 9.780327 * (1.0 + 0.0053024 * s1 - 0.0000058 * s2) - 3.086e-6 * z_m;
}

double ocrt_oracle_tau_rayleigh(double wl_nm, double p_hpa)
{
    const double co2 = 360.0;
    const double um = wl_nm / 1000.0;
    const double inv2 = 1.0 / (um * um);
    const double fn2 = 1.034 + 3.17e-4 * inv2;
    const double fo2 = 1.096 + 1.385e-3 * inv2 + 1.448e-4 * inv2 * inv2;
    const double xc = co2 / 1.0e4;
    const double king = (78.084 * fn2 + 20.946 * fo2 + 0.934 * 1.0 + xc * 1.15) /
                        (78.084 + 20.946 + 0.934 + xc);
    const double n300 = (8060.51 + 2480990.0 / (132.274 - inv2) +
                         17455.7 / (39.32957 - inv2)) * 1.0e-8;
    const double nm1 = n300 * (1.0 + 0.54 * (co2 * 1.0e-6 - 0.0003));
    const double nn = (1.0 + nm1) * (1.0 + nm1);
    const double avo = 6.0221367e23;
    const double ns = (avo / 22.4141) * (273.15 / 288.15) * 1.0e-3;
    const double wl_cm = wl_nm * 1.0e-7;
    const double wl4 = wl_cm * wl_cm * wl_cm * wl_cm;
    const double sigma = 24.0 * PI * PI * PI * (nn - 1.0) * (nn - 1.0) /
                         (wl4 * ns * ns * (nn + 2.0) * (nn + 2.0)) * king;
    const double ma = 15.0556 * (co2 * 1.0e-6) + 28.9595;
    const double g = 100.0 * gravity_wgs84(45.0, 5517.56);
    return sigma * (p_hpa * 1000.0) * avo / (ma * g);
}

/* ======================================================================
 * Altitude mapping: US Standard Atmosphere 1962 column fractions
 * (rt_molecular_profile.c:9-105) and the finite exponential aerosol profile
 * (rt_atm.c:44-51).
 * ==================================================================== */
static const double US62_Z[8] = {0.0, 11.0, 20.0, 32.0, 47.0, 51.0, 71.0, 84.852};
static const double US62_P[8] = {101325.0, 22632.1, 5474.89, 868.019,
                                 110.906, 66.9389, 3.95642, 0.3734};

static double us62_pressure(double z)
{
    if (z <= US62_Z[0]) return US62_P[0];
    if (z >= US62_Z[7]) return US62_P[7];
    int lo = 0, hi = 7;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (z < US62_Z[mid]) hi = mid; else lo = mid;
    }
    const double t = (z - US62_Z[lo]) / (US62_Z[hi] - US62_Z[lo]);
    const double a = log(US62_P[lo]), b = log(US62_P[hi]);
    return exp(a + t * (b - a));
}

static double clamp01(double x) { return x <= 0.0 ? 0.0 : (x >= 1.0 ? 1.0 : x); }

static double us62_fraction_above_raw(double z)
{
    if (z <= 0.0) return 1.0;
    const double g0 = gravity_wgs84(45.0, 0.0);
    if (z >= US62_Z[7]) {
        const double gt = gravity_wgs84(45.0, US62_Z[7] * 1000.0);
        return clamp01((US62_P[7] / gt) / (US62_P[0] / g0));
    }
    const double gz = gravity_wgs84(45.0, z * 1000.0);
    return clamp01((us62_pressure(z) / gz) / (US62_P[0] / g0));
}

static double us62_grid_fraction_above(double z)
{
    if (z <= 0.0) return 1.0;
    if (z >= US62_Z[7]) return 0.0;
    const double ft = us62_fraction_above_raw(US62_Z[7]);
    return clamp01((us62_fraction_above_raw(z) - ft) / (1.0 - ft));
}

static double exp_fraction_above(double z, double z_top, double h)
{
    if (z <= 0.0) return 1.0;
    if (z >= z_top) return 0.0;
    const double et = exp(-z_top / h);
    return (exp(-z / h) - et) / (1.0 - et);
}

/* Molecular column fraction above z for the selected profile. */
static double ray_fraction_above(double z, int profile, double h_km)
{
    return profile == OCRT_PROFILE_EXPONENTIAL ? exp_fraction_above(z, Z_TOP_KM, h_km)
                                               : us62_grid_fraction_above(z);
}

static double altitude_from_ray_fraction(double f, int profile, double h_km)
{
    const double ztop = profile == OCRT_PROFILE_EXPONENTIAL ? Z_TOP_KM : US62_Z[7];
    if (f >= 1.0) return 0.0;
    if (f <= 0.0) return ztop;
    double lo = 0.0, hi = ztop;
    for (int it = 0; it < 64; ++it) {       /* rt_molecular_profile.c:92-102 */
        const double mid = 0.5 * (lo + hi);
        if (ray_fraction_above(mid, profile, h_km) > f) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

/* ======================================================================
 * Medium: uniform-tau levels with direct-beam attenuation and the aerosol /
 * molecular scattering fractions per level (rt_atm.c:177-400).
 * ==================================================================== */
typedef struct {
    int nt;
    double tau_total;
    double *h, *ch, *xdel, *ydel, *z;
    double *tabs;                     /* [nt] gas absorption per layer, NULL without gas */
} medium_t;

static void medium_free(medium_t *md)
{
    free(md->h); free(md->ch); free(md->xdel); free(md->ydel); free(md->z); free(md->tabs);
    memset(md, 0, sizeof(*md));
}

static int medium_build(medium_t *md, int nt, double tau_r, double tau_a,
                        double ssa_a, double mu0, double aer_h_km,
                        int profile, double ray_h_km)
{
    memset(md, 0, sizeof(*md));
    md->nt = nt;
    md->h = calloc(nt + 1, sizeof(double));
    md->ch = calloc(nt + 1, sizeof(double));
    md->xdel = calloc(nt + 1, sizeof(double));
    md->ydel = calloc(nt + 1, sizeof(double));
    md->z = calloc(nt + 1, sizeof(double));
    if (!md->h || !md->ch || !md->xdel || !md->ydel || !md->z) { medium_free(md); return -3; }
    const double tau = tau_r + tau_a;
    md->tau_total = tau;
    for (int k = 0; k <= nt; ++k) {
        md->h[k] = (double)k * tau / (double)nt;
        md->ch[k] = 0.5 * exp(-md->h[k] / mu0);
        md->xdel[k] = 0.0;
        md->ydel[k] = 1.0;
        md->z[k] = k == 0 ? Z_TOP_KM
                          : altitude_from_ray_fraction(md->h[k] / tau, profile, ray_h_km);
    }
    if (tau_a <= 0.0) return 0;

    /* Aerosol + Rayleigh: altitude of every level by bisection on the mixed
     * column above, then per-layer scattering fractions (rt_atm.c:313-383). */
    const double ah = aer_h_km > 0.0 ? aer_h_km : 2.0;
    if (tau_r == 0.0) { md->xdel[0] = ssa_a; md->ydel[0] = 0.0; }
    else { md->xdel[0] = 0.0; md->ydel[0] = 1.0; }
    double z_prev = Z_TOP_KM, ray_prev = 0.0, aer_prev = 0.0;
    md->z[0] = Z_TOP_KM;
    for (int j = 1; j <= nt; ++j) {
        double zj = 0.0;
        if (j < nt) {
            double lo = 0.0, hi = z_prev;
            for (int it = 0; it < 64; ++it) {
                const double mid = 0.5 * (lo + hi);
                const double above = tau_r * ray_fraction_above(mid, profile, ray_h_km) +
                                     tau_a * exp_fraction_above(mid, Z_TOP_KM, ah);
                if (above > md->h[j]) lo = mid; else hi = mid;
            }
            zj = 0.5 * (lo + hi);
        }
        md->z[j] = zj;
        const double ray_j = tau_r * ray_fraction_above(zj, profile, ray_h_km);
        const double aer_j = tau_a * exp_fraction_above(zj, Z_TOP_KM, ah);
        const double dr = ray_j - ray_prev, da = aer_j - aer_prev, dt = dr + da;
        if (dt > 0.0) { md->xdel[j] = da * ssa_a / dt; md->ydel[j] = dr / dt; }
        else { md->xdel[j] = 0.0; md->ydel[j] = tau_r > 0.0 ? 1.0 : 0.0; }
        z_prev = zj; ray_prev = ray_j; aer_prev = aer_j;
    }
    return 0;
}

/* ======================================================================
 * Trace-gas absorption (rt_absorption.c, rt_atm.c:437-548).  AFGL level
 * profiles give per-gas number densities; layered cross-section tables
 * sigma(AFGL level, wavelength) are interpolated linearly in altitude and
 * wavelength; columns are trapezoids on the AFGL grid.  The per-layer
 * absorption depth of every solver layer is added to h[] and the scattering
 * fractions are rescaled by dtau_old / dtau_new.
 * ==================================================================== */
#define NGAS 6
static const char *const GAS_NAMES[NGAS] = {"h2o", "o3", "o2", "co2", "no2", "ch4"};   /* rt_absorption.c:38 */
static const char *const AFGL_NAMES[7] = {"usstd76", "tropical", "mlsumm", "mlwint",
                                          "sasumm", "sawint", "userdef"};             /* :40-42 */

typedef struct {
    int avail, nwl, nlay;
    double *wl, *sig;                 /* sig[layer * nwl + i] */
} xsec_t;

struct ocrt_gas {
    int nlev;
    double *z, *ntot, *mr[NGAS];
    double col_default[NGAS], col_eff[NGAS];
    int overridden[NGAS];
    xsec_t xs[NGAS];
};

/* Whole file as a NUL-terminated buffer; NULL if it cannot be read. */
static char *slurp(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    size_t cap = 1 << 16, len = 0;
    char *b = malloc(cap);
    while (b) {
        if (len + 4096 + 1 > cap) { char *nb = realloc(b, cap *= 2); if (!nb) { free(b); b = NULL; break; } b = nb; }
        const size_t r = fread(b + len, 1, 4096, f);
        len += r;
        if (r == 0) break;
    }
    fclose(f);
    if (b) b[len] = 0;
    return b;
}

/* Next line of a buffer, NUL-terminated in place; NULL at the end. */
static char *next_line(char **cur)
{
    char *s = *cur;
    if (!s || !*s) return NULL;
    char *e = strchr(s, '\n');
    if (e) { *e = 0; *cur = e + 1; } else *cur = s + strlen(s);
    return s;
}

/* Data lines skip '#' comments and empty lines (rt_absorption.c:68-72). */
static int is_skip(const char *l) { return l[0] == '#' || l[0] == 0 || l[0] == '\r'; }

/* AFGL loader (rt_afgl_load, rt_absorption.c:48-175): z P T n_total and six
 * mixing ratios (ppmv) per level, default columns by trapezoids (:160-172). */
static int afgl_load(struct ocrt_gas *g, const char *dir, int profile)
{
    char path[1024];
    snprintf(path, sizeof(path), "%s/afgl_%s.dat", dir, AFGL_NAMES[profile]);
    char *buf = slurp(path);
    if (!buf) return -2;
    int cap = 64, n = 0;
    double *rows = malloc(sizeof(double) * 10 * cap);
    char *cur = buf, *l;
    int bad = 0;
    while (rows && (l = next_line(&cur))) {
        if (is_skip(l)) continue;
        double v[10];
        if (sscanf(l, "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5],
                   &v[6], &v[7], &v[8], &v[9]) != 10) {
            /* blank-looking lines are skipped; any other malformed row is an error */
            const char *q = l;
            while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
            if (*q) bad = 1;
            continue;
        }
        if (n == cap) { double *nr = realloc(rows, sizeof(double) * 10 * (cap *= 2)); if (!nr) { free(rows); rows = NULL; break; } rows = nr; }
        memcpy(rows + 10 * n, v, sizeof(v));
        ++n;
    }
    free(buf);
    if (!rows) return -3;
    if (bad || n < 2) { free(rows); return -1; }
    g->nlev = n;
    g->z = malloc(sizeof(double) * n);
    g->ntot = malloc(sizeof(double) * n);
    for (int k = 0; k < NGAS; ++k) g->mr[k] = malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) {
        g->z[i] = rows[10 * i];
        g->ntot[i] = rows[10 * i + 3];
        for (int k = 0; k < NGAS; ++k) g->mr[k][i] = rows[10 * i + 4 + k];
    }
    free(rows);
    for (int k = 0; k < NGAS; ++k) {
        double col = 0.0;
        for (int i = 0; i + 1 < n; ++i) {
            const double n1 = g->mr[k][i] * 1e-6 * g->ntot[i];
            const double n2 = g->mr[k][i + 1] * 1e-6 * g->ntot[i + 1];
            col += 0.5 * (n1 + n2) * ((g->z[i + 1] - g->z[i]) * 1.0e5);
        }
        g->col_default[k] = col;
    }
    return 0;
}

/* Cross-section table (rt_xsec_load, rt_absorption.c:192-333).  Header tag
 * "n_layers" selects the layered form: a wavelength row, then one sigma row
 * per AFGL level; otherwise rows of (wavelength, sigma).  The grid must be
 * increasing and cover 330-1100 nm (rt_spectral_contract.h); a table that
 * fails to load leaves the gas out. */
static void xsec_load(xsec_t *x, const char *dir, int gas)
{
    memset(x, 0, sizeof(*x));
    char path[1024];
    snprintf(path, sizeof(path), "%s/xsec_%s.dat", dir, GAS_NAMES[gas]);
    char *buf = slurp(path);
    if (!buf) return;
    int nlay = 1;
    char *cur = buf, *l;
    while ((l = next_line(&cur))) {
        if (l[0] != '#') continue;
        const char *p = strstr(l, "n_layers");
        if (p) { sscanf(p, "n_layers = %d", &nlay); if (nlay < 1) nlay = 1; }
    }
    for (char *q = buf; q < cur; ++q) if (*q == 0) *q = '\n';   /* restore the lines */
    cur = buf;
    int ok = 1;
    if (nlay == 1) {
        int cap = 1024, n = 0;
        x->wl = malloc(sizeof(double) * cap);
        x->sig = malloc(sizeof(double) * cap);
        while ((l = next_line(&cur))) {
            if (is_skip(l)) continue;
            double a, b;
            if (sscanf(l, "%lf %lf", &a, &b) != 2) continue;
            if (n == cap) { cap *= 2; x->wl = realloc(x->wl, sizeof(double) * cap); x->sig = realloc(x->sig, sizeof(double) * cap); }
            x->wl[n] = a; x->sig[n] = b; ++n;
        }
        x->nwl = n; x->nlay = 1;
    } else {
        int row = -1;
        while ((l = next_line(&cur))) {
            if (is_skip(l)) continue;
            if (row < 0) {
                int cnt = 0;
                for (char *p = l, *e; ; p = e) { strtod(p, &e); if (e == p) break; ++cnt; }
                if (cnt < 2) { ok = 0; break; }
                x->nwl = cnt; x->nlay = nlay;
                x->wl = malloc(sizeof(double) * cnt);
                x->sig = calloc((size_t)cnt * nlay, sizeof(double));
                char *p = l, *e;
                for (int i = 0; i < cnt; ++i, p = e) x->wl[i] = strtod(p, &e);
                row = 0;
            } else if (row < nlay) {
                char *p = l, *e;
                for (int i = 0; i < x->nwl; ++i, p = e) {
                    const double v = strtod(p, &e);
                    if (e == p) break;
                    x->sig[(size_t)row * x->nwl + i] = v;
                }
                ++row;
            }
        }
        if (row < 0) ok = 0;
    }
    free(buf);
    if (ok && x->nwl >= 2) {
        for (int i = 0; i < x->nwl; ++i)
            if (!isfinite(x->wl[i]) || (i > 0 && !(x->wl[i] > x->wl[i - 1]))) ok = 0;
        if (ok && !(x->wl[0] <= 330.0 + 1e-9 && x->wl[x->nwl - 1] >= 1100.0 - 1e-9)) ok = 0;
    } else ok = 0;
    if (!ok) { free(x->wl); free(x->sig); memset(x, 0, sizeof(*x)); return; }
    x->avail = 1;
}

static void gas_free(struct ocrt_gas *g)
{
    if (!g) return;
    free(g->z); free(g->ntot);
    for (int k = 0; k < NGAS; ++k) { free(g->mr[k]); free(g->xs[k].wl); free(g->xs[k].sig); }
    free(g);
}

/* rt_absorption_init (rt_absorption.c:486-533). */
int ocrt_oracle_gas_create(const char *afgl_dir, const char *xsec_dir, int profile,
                           const double *override, ocrt_gas **out)
{
    if (!afgl_dir || !xsec_dir || !out || profile < 0 || profile > 6) return -1;
    *out = NULL;
    struct ocrt_gas *g = calloc(1, sizeof(*g));
    if (!g) return -3;
    int rc = afgl_load(g, afgl_dir, profile);
    if (rc) { gas_free(g); return rc == -3 ? -3 : -1; }
    for (int k = 0; k < NGAS; ++k) {
        xsec_load(&g->xs[k], xsec_dir, k);
        /* the reference reads the altitude of table level i from AFGL level i */
        if (g->xs[k].avail && g->xs[k].nlay > g->nlev) { gas_free(g); return -1; }
        if (override && override[k] >= 0.0) { g->col_eff[k] = override[k]; g->overridden[k] = 1; }
        else g->col_eff[k] = g->col_default[k];
    }
    *out = g;
    return 0;
}

void ocrt_oracle_gas_destroy(ocrt_gas *g) { gas_free(g); }

/* sigma at (table level, wavelength) (rt_xsec_interp_layer, rt_absorption.c:347-371). */
static double xsec_at(const xsec_t *x, int layer, double wl)
{
    if (!x->avail || x->nwl < 2) return 0.0;
    if (layer < 0) layer = 0;
    if (layer >= x->nlay) layer = x->nlay - 1;
    const double *s = x->sig + (size_t)layer * x->nwl;
    const int n = x->nwl;
    if (wl < x->wl[0] || wl > x->wl[n - 1]) return NAN;
    if (wl == x->wl[0]) return s[0];
    if (wl == x->wl[n - 1]) return s[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (x->wl[mid] <= wl) lo = mid; else hi = mid; }
    const double t = (wl - x->wl[lo]) / (x->wl[hi] - x->wl[lo]);
    return (1.0 - t) * s[lo] + t * s[hi];
}

/* sigma at (altitude, wavelength), linear between bracketing AFGL levels
 * (rt_xsec_interp_layer_z, rt_absorption.c:378-412). */
static double xsec_at_z(const xsec_t *x, const double *zg, double z, double wl)
{
    if (!x->avail) return 0.0;
    const int nl = x->nlay;
    if (nl == 1) return xsec_at(x, 0, wl);
    if (z <= zg[0]) return xsec_at(x, 0, wl);
    if (z >= zg[nl - 1]) return xsec_at(x, nl - 1, wl);
    int lo = 0, hi = nl - 1;
    while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (zg[mid] <= z) lo = mid; else hi = mid; }
    const double dz = zg[hi] - zg[lo];
    if (dz <= 0.0) return xsec_at(x, lo, wl);
    const double t = (z - zg[lo]) / dz;
    return (1.0 - t) * xsec_at(x, lo, wl) + t * xsec_at(x, hi, wl);
}

/* Column above z (molecules/cm^2), trapezoids with the cut layer
 * interpolated (rt_afgl_cumulative_column, rt_absorption.c:425-453). */
static double col_above(const struct ocrt_gas *g, int k, double z)
{
    double cum = 0.0;
    for (int i = 0; i + 1 < g->nlev; ++i) {
        const double z1 = g->z[i], z2 = g->z[i + 1];
        if (z2 <= z) continue;
        const double a = z1 < z ? z : z1, b = z2;
        if (b <= a) continue;
        const double f1 = (a - z1) / (z2 - z1), f2 = (b - z1) / (z2 - z1);
        const double n1 = g->mr[k][i] * 1e-6 * g->ntot[i];
        const double n2 = g->mr[k][i + 1] * 1e-6 * g->ntot[i + 1];
        const double nlo = (1.0 - f1) * n1 + f1 * n2, nhi = (1.0 - f2) * n1 + f2 * n2;
        cum += 0.5 * (nlo + nhi) * ((b - a) * 1.0e5);
    }
    return cum;
}

/* Column in [z_lo, z_hi] (rt_afgl_layer_column, rt_absorption.c:455-461). */
static double col_layer(const struct ocrt_gas *g, int k, double zlo, double zhi)
{
    if (zhi <= zlo) return 0.0;
    return col_above(g, k, zlo) - col_above(g, k, zhi);
}

/* Column absorption depth of one gas (rt_absorption_tau_per_gas, :556-590). */
static double gas_tau_one(const struct ocrt_gas *g, int k, double wl)
{
    const xsec_t *x = &g->xs[k];
    if (!x->avail || g->nlev < 2) return 0.0;
    const double ndef = g->col_default[k];
    const int ov = g->overridden[k] && ndef > 0.0;
    const double scale = ov ? g->col_eff[k] / ndef : 1.0;
    double tau = 0.0;
    for (int i = 0; i + 1 < g->nlev; ++i) {
        const double zlo = g->z[i], zhi = g->z[i + 1];
        const double sig = xsec_at_z(x, g->z, 0.5 * (zlo + zhi), wl);
        double nl = col_layer(g, k, zlo, zhi);
        if (ov) nl *= scale;
        tau += sig * nl;
    }
    return tau;
}

int ocrt_oracle_gas_tau(const ocrt_gas *g, double wl, double *per_gas, double *total)
{
    if (!g) return -1;
    double t = 0.0;
    for (int k = 0; k < NGAS; ++k) {
        const double v = gas_tau_one(g, k, wl);
        if (per_gas) per_gas[k] = v;
        t += v;
    }
    if (total) *total = t;
    return 0;
}

int ocrt_oracle_gas_columns(const ocrt_gas *g, double *eff, double *def, int *ov)
{
    if (!g) return -1;
    for (int k = 0; k < NGAS; ++k) {
        if (eff) eff[k] = g->col_eff[k];
        if (def) def[k] = g->col_default[k];
        if (ov) ov[k] = g->overridden[k];
    }
    return 0;
}

/* Fold the gas into the medium (rt_atm_apply_gas_absorption, rt_atm.c:437-548). */
static int medium_apply_gas(medium_t *md, const struct ocrt_gas *g, double wl, double mu0)
{
    const int nt = md->nt;
    if (!(mu0 > 0.0)) return -1;
    md->tabs = calloc(nt, sizeof(double));
    double *hold = malloc(sizeof(double) * (nt + 1));
    if (!md->tabs || !hold) { free(hold); return -3; }
    for (int k = 0; k < nt; ++k) {
        double zhi = md->z[k], zlo = md->z[k + 1];
        if (zlo > zhi) { const double t = zlo; zlo = zhi; zhi = t; }
        const double zmid = 0.5 * (zlo + zhi);
        double dt = 0.0;
        for (int q = 0; q < NGAS; ++q) {
            double N;
            if (g->overridden[q]) {
                const double ndef = g->col_default[q];
                N = ndef > 0.0 ? g->col_eff[q] * (col_layer(g, q, zlo, zhi) / ndef) : 0.0;
            } else N = col_layer(g, q, zlo, zhi);
            dt += xsec_at_z(&g->xs[q], g->z, zmid, wl) * N;
        }
        md->tabs[k] = dt;
    }
    for (int k = 0; k <= nt; ++k) hold[k] = md->h[k];
    double cum = 0.0;
    for (int k = 0; k <= nt; ++k) {
        md->h[k] = hold[k] + cum;
        md->ch[k] = 0.5 * exp(-md->h[k] / mu0);
        if (k < nt) cum += md->tabs[k];
    }
    for (int k = 1; k <= nt; ++k) {
        const double dold = hold[k] - hold[k - 1], dnew = dold + md->tabs[k - 1];
        if (dnew > 0.0 && dold > 0.0) {
            md->xdel[k] = md->xdel[k] * dold / dnew;
            md->ydel[k] = md->ydel[k] * dold / dnew;
        }
    }
    md->tau_total = md->h[nt];
    free(hold);
    return 0;
}

/* ======================================================================
 * Angular basis: normalised associated Legendre P_l^m and the spin-2 pair
 * R_l^m, T_l^m by three-term recurrence (rt_angular_basis.c:19-124).
 * Arrays are [l] for one direction cosine.
 * ==================================================================== */
static double diag_norm(int m)
{
    double v = 1.0;
    for (int i = 1; i <= m; ++i) v *= sqrt((double)(i + m) / (double)i) * 0.5;
    return v;
}

static void basis_scalar(int L, int m, double x, double *p)
{
    for (int l = 0; l <= L; ++l) p[l] = 0.0;
    if (m == 0) { p[0] = 1.0; p[1] = x; p[2] = 0.5 * (3.0 * x * x - 1.0); }
    else if (m == 1) { p[1] = sqrt(0.5 * (1.0 - x * x)); p[2] = x * p[1] * sqrt(3.0); }
    else { p[m - 1] = 0.0; p[m] = diag_norm(m) * pow(1.0 - x * x, 0.5 * (double)m); }
    const int l0 = m < 2 ? 2 : m;
    for (int l = l0; l < L; ++l) {
        const double f = (2.0 * l + 1.0) / sqrt((double)(l + m + 1) * (double)(l - m + 1));
        const double b = sqrt((double)(l + m) * (double)(l - m)) / (2.0 * l + 1.0);
        p[l + 1] = f * (x * p[l] - b * p[l - 1]);
    }
}

static void basis_spin2(int L, int m, double x, double *r, double *t)
{
    for (int l = 0; l <= L; ++l) { r[l] = 0.0; t[l] = 0.0; }
    if (m == 0) {
        r[2] = 3.0 * (1.0 - x * x) / (2.0 * sqrt(6.0));
    } else if (m == 1) {
        const double s = sqrt(1.0 - x * x);
        r[2] = -x * s * 0.5;
        t[2] = -s * 0.5;
    } else {
        const double sn = diag_norm(m) * sqrt((double)m / (double)(m + 1)) *
                          sqrt((double)(m - 1) / (double)(m + 2));
        const double env = pow(1.0 - x * x, 0.5 * (double)m - 1.0);
        r[m] = sn * (1.0 + x * x) * env;
        t[m] = sn * 2.0 * x * env;
    }
    const int l0 = m < 2 ? 2 : m;
    for (int l = l0; l < L; ++l) {
        const double sc = (double)(l + 1) * (double)(2 * l + 1) /
            sqrt((double)(l + 3) * (double)(l - 1) * (double)(l + m + 1) * (double)(l - m + 1));
        const double dc = sqrt((double)(l + 2) * (double)(l - 2) * (double)(l + m) * (double)(l - m)) /
                          ((double)l * (double)(2 * l + 1));
        const double cc = 2.0 * (double)m / ((double)l * (double)(l + 1));
        r[l + 1] = sc * (x * r[l] - cc * t[l] - dc * r[l - 1]);
        t[l + 1] = sc * (x * t[l] - cc * r[l] - dc * t[l - 1]);
    }
}

/* ======================================================================
 * Per-mode angular state: the six particle phase tables over
 * (row j in 0..n) x (column k in -n..n) (rt_angular_basis.c:278-357) and the
 * molecular l=2 basis values xpl/xrl/xtl (rt_angular_basis.c:366-396).
 * Row 0 / column 0 is the solar slot mu = -mu0.
 * ==================================================================== */
typedef struct {
    int n, L, m;
    double *P, *R, *T;              /* [(L+1)][2n+1] basis at the signed ring */
    double *pfm, *gr, *gt, *arr, *art, *att;   /* [(n+1)][2n+1] */
    double *xpl, *xrl, *xtl;        /* [2n+1] */
} mode_t_;

#define RIDX(n, j) ((j) + (n))
#define TAB(tab, n, j, k) ((tab)[(size_t)(j) * (size_t)(2 * (n) + 1) + (size_t)((k) + (n))])

static void mode_free(mode_t_ *md)
{
    free(md->P); free(md->R); free(md->T);
    free(md->pfm); free(md->gr); free(md->gt); free(md->arr); free(md->art); free(md->att);
    free(md->xpl); free(md->xrl); free(md->xtl);
    memset(md, 0, sizeof(*md));
}

static int mode_alloc(mode_t_ *md, int n, int L)
{
    memset(md, 0, sizeof(*md));
    md->n = n; md->L = L;
    const size_t nd = (size_t)(2 * n + 1);
    const size_t nb = (size_t)(L + 1) * nd, nk = (size_t)(n + 1) * nd;
    md->P = calloc(nb, sizeof(double)); md->R = calloc(nb, sizeof(double));
    md->T = calloc(nb, sizeof(double));
    md->pfm = calloc(nk, sizeof(double)); md->gr = calloc(nk, sizeof(double));
    md->gt = calloc(nk, sizeof(double)); md->arr = calloc(nk, sizeof(double));
    md->art = calloc(nk, sizeof(double)); md->att = calloc(nk, sizeof(double));
    md->xpl = calloc(nd, sizeof(double)); md->xrl = calloc(nd, sizeof(double));
    md->xtl = calloc(nd, sizeof(double));
    if (!md->P || !md->R || !md->T || !md->pfm || !md->gr || !md->gt || !md->arr ||
        !md->art || !md->att || !md->xpl || !md->xrl || !md->xtl) { mode_free(md); return -3; }
    return 0;
}

/* Tabulated P11 at a scattering-angle cosine, linear in the angle in
 * degrees, clamped to the end values (rt_solver.c:190-202, rt_ipss.c:131-146). */
static double aer_p11_table(const ocrt_aerosol *a, double cth)
{
    if (cth > 1.0) cth = 1.0; else if (cth < -1.0) cth = -1.0;
    const double t = acos(cth) * 180.0 / PI;
    const double *th = a->theta_phase, *P = a->P11_phase;
    const int n = a->n_ang_phase;
    if (t <= th[0]) return P[0];
    if (t >= th[n - 1]) return P[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (th[mid] <= t) lo = mid; else hi = mid; }
    return P[lo] + (t - th[lo]) / (th[hi] - th[lo]) * (P[hi] - P[lo]);
}

/* rm: signed ring [2n+1] (index j+n), moments may be NULL (pure Rayleigh). */
static void mode_build(mode_t_ *md, int m, const double *rm,
                       const ocrt_aerosol *aer)
{
    const int n = md->n, L = md->L, nd = 2 * n + 1;
    md->m = m;
    double *bp = malloc(sizeof(double) * 3 * (L + 1));
    double *br = bp + (L + 1), *bt = br + (L + 1);
    for (int j = -n; j <= n; ++j) {
        basis_scalar(L, m, rm[RIDX(n, j)], bp);
        basis_spin2(L, m, rm[RIDX(n, j)], br, bt);
        for (int l = 0; l <= L; ++l) {
            md->P[(size_t)l * nd + RIDX(n, j)] = bp[l];
            md->R[(size_t)l * nd + RIDX(n, j)] = br[l];
            md->T[(size_t)l * nd + RIDX(n, j)] = bt[l];
        }
        md->xpl[RIDX(n, j)] = bp[2];
        md->xrl[RIDX(n, j)] = br[2];
        md->xtl[RIDX(n, j)] = bt[2];
    }
    free(bp);
    const size_t nk = (size_t)(n + 1) * nd;
    memset(md->pfm, 0, nk * sizeof(double)); memset(md->gr, 0, nk * sizeof(double));
    memset(md->gt, 0, nk * sizeof(double)); memset(md->arr, 0, nk * sizeof(double));
    memset(md->art, 0, nk * sizeof(double)); memset(md->att, 0, nk * sizeof(double));
    if (!aer) return;
    const int La = aer->L_max;
    for (int j = 0; j <= n; ++j) {
        for (int k = -n; k <= n; ++k) {
            double s_p = 0, s_r = 0, s_t = 0, s_rr = 0, s_rt = 0, s_tt = 0;
            for (int l = m; l <= L; ++l) {
                const double be = l <= La ? aer->beta[l] : 0.0;
                const double ga = l <= La ? aer->gamma[l] : 0.0;
                const double al = l <= La ? aer->alpha[l] : 0.0;
                const double ze = l <= La ? aer->zeta[l] : 0.0;
                const double pj = md->P[(size_t)l * nd + RIDX(n, j)], pk = md->P[(size_t)l * nd + RIDX(n, k)];
                const double rj = md->R[(size_t)l * nd + RIDX(n, j)], rk = md->R[(size_t)l * nd + RIDX(n, k)];
                const double tj = md->T[(size_t)l * nd + RIDX(n, j)], tk = md->T[(size_t)l * nd + RIDX(n, k)];
                s_p += pj * pk * be;
                s_r += pj * rk * ga;
                s_t += pj * tk * ga;
                s_tt += tj * tk * al + rj * rk * ze;
                s_rr += tj * tk * ze + rj * rk * al;
                s_rt += tj * rk * al + rj * tk * ze;
            }
            TAB(md->pfm, n, j, k) = s_p; TAB(md->gr, n, j, k) = s_r; TAB(md->gt, n, j, k) = s_t;
            TAB(md->arr, n, j, k) = s_rr; TAB(md->art, n, j, k) = s_rt; TAB(md->att, n, j, k) = s_tt;
        }
    }
    if (aer->use_value_kernel && aer->n_ang_phase > 1) {
        /* value kernel (rt_solver.c:188-235): the I-I table by direct azimuth
         * integration of the tabulated P11 over 720 midpoints */
        for (int j = 0; j <= n; ++j) {
            const double mj = rm[RIDX(n, j)], sj = sqrt(fmax(0.0, 1.0 - mj * mj));
            for (int k = -n; k <= n; ++k) {
                const double mk = rm[RIDX(n, k)], sk = sqrt(fmax(0.0, 1.0 - mk * mk));
                double acc = 0.0;
                for (int q = 0; q < 720; ++q) {
                    const double phi = 2.0 * PI * ((double)q + 0.5) / 720.0;
                    acc += aer_p11_table(aer, mj * mk + sj * sk * cos(phi)) * cos((double)m * phi);
                }
                TAB(md->pfm, n, j, k) = acc / 720.0;
            }
        }
    }
}

/* ======================================================================
 * Solve context for one pixel.
 * ==================================================================== */
typedef struct {
    int n;                 /* ring size (positive directions) */
    int view_idx;          /* 1-based ring index of mu_view, 0 if interpolated */
    double mu0, mu_view;
    double rm[2 * MAX_RING + 1], gb[2 * MAX_RING + 1];
    double beta0, beta2, gamma2, alpha2;
    medium_t md;
    double *Tr;            /* [2n+1][nt] layer transmission */
    double *Ca, *Cb;       /* [2n+1][nt] linear-source weights on J_out, J_in */
} ctx_t;

#define F(buf, c, k, j) ((buf)[(size_t)(k) * (size_t)(2 * (c)->n + 1) + (size_t)((j) + (c)->n)])

/* Transport coefficients of the linear-in-tau formal solution
 * (rt_layer_transport.c:36-99, 107-208), regrouped as
 *   I_k = T I_up + Ca J_k + Cb J_up,
 *   G = (1-T)|mu|/dtau - T,  Ca = (1-T-G)/2,  Cb = G/2,
 * which is the reference's slope/intercept expression expanded. */
static int transport_prepare(ctx_t *c)
{
    const int n = c->n, nt = c->md.nt, nd = 2 * n + 1;
    c->Tr = malloc(sizeof(double) * (size_t)nd * nt);
    c->Ca = malloc(sizeof(double) * (size_t)nd * nt);
    c->Cb = malloc(sizeof(double) * (size_t)nd * nt);
    if (!c->Tr || !c->Ca || !c->Cb) return -3;
    for (int j = -n; j <= n; ++j) {
        for (int l = 0; l < nt; ++l) {
            const size_t i = (size_t)RIDX(n, j) * nt + l;
            if (j == 0) { c->Tr[i] = c->Ca[i] = c->Cb[i] = 0.0; continue; }
            const double am = fabs(c->rm[RIDX(n, j)]);
            const double dtau = c->md.h[l + 1] - c->md.h[l];
            const double T = exp(-dtau / am);
            const double G = (1.0 - T) * am / dtau - T;
            c->Tr[i] = T;
            c->Ca[i] = 0.5 * (1.0 - T - G);
            c->Cb[i] = 0.5 * G;
        }
    }
    return 0;
}

/* Up sweep from the surface BC, down sweep from a zero top BC. */
static int transport(const ctx_t *c, const double *J, const double *bc, double *I)
{
    const int n = c->n, nt = c->md.nt;
    for (int k = 0; k <= nt; ++k) F(I, c, k, 0) = NAN;
    for (int j = -n; j <= n; ++j) {
        if (j == 0) continue;
        const double *T = c->Tr + (size_t)RIDX(n, j) * nt;
        const double *A = c->Ca + (size_t)RIDX(n, j) * nt;
        const double *B = c->Cb + (size_t)RIDX(n, j) * nt;
        if (j > 0) {
            double run = bc ? bc[j - 1] : 0.0;
            F(I, c, nt, j) = run;
            for (int k = nt - 1; k >= 0; --k) {
                const double jo = F(J, c, k, j), ji = F(J, c, k + 1, j);
                if (!isfinite(jo) || !isfinite(ji)) return -2;
                run = T[k] * run + A[k] * jo + B[k] * ji;
                F(I, c, k, j) = run;
            }
        } else {
            double run = 0.0;
            F(I, c, 0, j) = run;
            for (int k = 1; k <= nt; ++k) {
                const double jo = F(J, c, k, j), ji = F(J, c, k - 1, j);
                if (!isfinite(jo) || !isfinite(ji)) return -2;
                run = T[k - 1] * run + A[k - 1] * jo + B[k - 1] * ji;
                F(I, c, k, j) = run;
            }
        }
    }
    return 0;
}

/* Direct-beam primary source (rt_primary_source.c:17-198; beam_q = 0). */
static void primary_source(const ctx_t *c, const mode_t_ *md, double *JI, double *JQ, double *JU)
{
    const int n = c->n, nt = c->md.nt, m = md->m;
    const int mol = m <= 2;
    const double b0 = m == 0 ? c->beta0 : 0.0;
    const double p0 = md->xpl[RIDX(n, 0)];
    for (int k = 0; k <= nt; ++k) {
        const double beam = c->md.ch[k], x = c->md.xdel[k], y = c->md.ydel[k];
        for (int j = -n; j <= n; ++j) {
            const double pj = md->xpl[RIDX(n, j)];
            const double mi = b0 + c->beta2 * pj * p0;
            const double mq = mol ? c->gamma2 * md->xrl[RIDX(n, j)] * p0 : 0.0;
            const double mu = mol ? c->gamma2 * md->xtl[RIDX(n, j)] * p0 : 0.0;
            F(JI, c, k, j) = beam * (x * TAB(md->pfm, n, 0, j) + y * mi);
            F(JQ, c, k, j) = beam * (x * TAB(md->gr, n, 0, j) + y * mq);
            F(JU, c, k, j) = -beam * (x * TAB(md->gt, n, 0, j) + y * mu);
        }
        F(JI, c, k, 0) = F(JQ, c, k, 0) = F(JU, c, k, 0) = NAN;
    }
}

/* Multiple-scattering source: the vector contraction of
 * rt_sos_operator.c:206-424.  The 18 aerosol and 18 molecular direction-pair
 * coefficients are formed once per (outgoing, incoming) pair from the phase
 * tables; the level loop is innermost over transposed field planes. */
static int ms_source(const ctx_t *c, const mode_t_ *md,
                     const double *I, const double *Q, const double *U,
                     double *JI, double *JQ, double *JU)
{
    const int n = c->n, nt = c->md.nt, m = md->m, K = nt + 1;
    const int mol = m <= 2;
    const double b0 = m == 0 ? c->beta0 : 0.0, b2 = c->beta2, g2 = c->gamma2, a2 = c->alpha2;
    const double *xp = md->xpl + n, *xr = md->xrl + n, *xt = md->xtl + n;
    for (int k = 0; k <= nt; ++k)
        for (int j = -n; j <= n; ++j)
            if (j != 0 && (!isfinite(F(I, c, k, j)) || !isfinite(F(Q, c, k, j)) ||
                           !isfinite(F(U, c, k, j)))) return -2;
    double *pl = malloc(sizeof(double) * (size_t)K * (6 * n + 6));
    if (!pl) return -3;
    double *acc = pl + (size_t)6 * n * K;
#define PLANE(comp, i) (pl + ((size_t)(comp) * n + (size_t)((i) - 1)) * K)
    for (int i = 1; i <= n; ++i)
        for (int k = 0; k <= nt; ++k) {
            PLANE(0, i)[k] = F(I, c, k, i); PLANE(1, i)[k] = F(I, c, k, -i);
            PLANE(2, i)[k] = F(Q, c, k, i); PLANE(3, i)[k] = F(Q, c, k, -i);
            PLANE(4, i)[k] = F(U, c, k, i); PLANE(5, i)[k] = F(U, c, k, -i);
        }
    const double *xd = c->md.xdel, *yd = c->md.ydel;
    for (int o = 1; o <= n; ++o) {
        memset(acc, 0, sizeof(double) * 6 * (size_t)K);
        double *Iu_ = acc, *Id_ = acc + K, *Qu_ = acc + 2 * K, *Qd_ = acc + 3 * K, *Uu_ = acc + 4 * K, *Ud_ = acc + 5 * K;
        for (int i = 1; i <= n; ++i) {
            const double w = c->gb[RIDX(n, i)];
            if (w == 0.0) continue;
            const double pa[18] = {
                TAB(md->pfm, n, i, o), TAB(md->pfm, n, i, -o), TAB(md->gt, n, i, o), TAB(md->gt, n, i, -o),
                TAB(md->gt, n, o, i), TAB(md->gt, n, o, -i), TAB(md->gr, n, i, o), TAB(md->gr, n, i, -o),
                TAB(md->gr, n, o, i), TAB(md->gr, n, o, -i), TAB(md->arr, n, i, o), TAB(md->arr, n, i, -o),
                TAB(md->art, n, i, o), TAB(md->art, n, i, -o), TAB(md->art, n, o, i), TAB(md->art, n, o, -i),
                TAB(md->att, n, i, o), TAB(md->att, n, i, -o)};
            double pm[18] = {0};
            if (mol) {
                const double v[18] = {
                    b0 + b2 * xp[i] * xp[o], b0 + b2 * xp[i] * xp[-o], g2 * xp[i] * xt[o], g2 * xp[i] * xt[-o],
                    g2 * xp[o] * xt[i], g2 * xp[o] * xt[-i], g2 * xp[i] * xr[o], g2 * xp[i] * xr[-o],
                    g2 * xp[o] * xr[i], g2 * xp[o] * xr[-i], a2 * xr[i] * xr[o], a2 * xr[i] * xr[-o],
                    a2 * xt[i] * xr[o], a2 * xt[i] * xr[-o], a2 * xt[o] * xr[i], a2 * xt[o] * xr[-i],
                    a2 * xt[i] * xt[o], a2 * xt[i] * xt[-o]};
                memcpy(pm, v, sizeof(v));
            }
            const double *iu_ = PLANE(0, i), *id_ = PLANE(1, i), *qu_ = PLANE(2, i), *qd_ = PLANE(3, i);
            const double *uu_ = PLANE(4, i), *ud_ = PLANE(5, i);
            for (int k = 0; k < K; ++k) {
                const double x = xd[k], y = yd[k];
                const double ii_s = x * pa[0] + y * pm[0], ii_c = x * pa[1] + y * pm[1];
                const double iu_s = x * pa[2] + y * pm[2], iu_c = x * pa[3] + y * pm[3];
                const double iuT_s = x * pa[4] + y * pm[4], iuT_c = x * pa[5] + y * pm[5];
                const double iq_s = x * pa[6] + y * pm[6], iq_c = x * pa[7] + y * pm[7];
                const double iqT_s = x * pa[8] + y * pm[8], iqT_c = x * pa[9] + y * pm[9];
                const double qq_s = x * pa[10] + y * pm[10], qq_c = x * pa[11] + y * pm[11];
                const double qu_s = x * pa[12] + y * pm[12], qu_c = x * pa[13] + y * pm[13];
                const double quT_s = x * pa[14] + y * pm[14], quT_c = x * pa[15] + y * pm[15];
                const double uu_s = x * pa[16] + y * pm[16], uu_c = x * pa[17] + y * pm[17];
                const double iu = iu_[k], id = id_[k], qu = qu_[k], qd = qd_[k], uu = uu_[k], ud = ud_[k];
                Iu_[k] += w * (iu * ii_s + qu * iqT_s - uu * iuT_s + id * ii_c + qd * iqT_c - ud * iuT_c);
                Id_[k] += w * (iu * ii_c + qu * iqT_c + uu * iuT_c + id * ii_s + qd * iqT_s + ud * iuT_s);
                Qu_[k] += w * (iu * iq_s + qu * qq_s - uu * qu_s + id * iq_c + qd * qq_c + ud * qu_c);
                Qd_[k] += w * (iu * iq_c + qu * qq_c - uu * qu_c + id * iq_s + qd * qq_s + ud * qu_s);
                Uu_[k] -= w * (iu * iu_s + qu * quT_s - uu * uu_s - id * iu_c + qd * quT_c - ud * uu_c);
                Ud_[k] -= w * (iu * iu_c - qu * quT_c - uu * uu_c - id * iu_s - qd * quT_s - ud * uu_s);
            }
        }
        for (int k = 0; k <= nt; ++k) {
            F(JI, c, k, o) = Iu_[k]; F(JI, c, k, -o) = Id_[k];
            F(JQ, c, k, o) = Qu_[k]; F(JQ, c, k, -o) = Qd_[k];
            F(JU, c, k, o) = Uu_[k]; F(JU, c, k, -o) = Ud_[k];
        }
    }
    for (int k = 0; k <= nt; ++k) F(JI, c, k, 0) = F(JQ, c, k, 0) = F(JU, c, k, 0) = NAN;
#undef PLANE
    free(pl);
    return 0;
}

/* ======================================================================
 * Surface: Fresnel core and Cox-Munk Mueller BRDF (shared/surface.c:57-64,
 * 385-455, 514-619), rotations (shared/mat3.h:45-55).
 * ==================================================================== */
static double slope_variance(double ws, int sigma_type)
{
    if (sigma_type == 1) return 0.003 + 0.00512 * fmax(0.01, ws);
    const double s = 0.0731 * sqrt(fmax(0.0, ws));
    return fmax(s * s, 1e-10);
}

static void fresnel_R(double mu_i, double nw, int qconv, double *M)
{
    for (int i = 0; i < 9; ++i) M[i] = 0.0;
    const double st2 = (1.0 / nw) * (1.0 / nw) * fmax(0.0, 1.0 - mu_i * mu_i);
    if (st2 >= 1.0) { M[0] = M[4] = M[8] = 1.0; return; }
    const double mt = sqrt(1.0 - st2);
    const double rs = (mu_i - nw * mt) / (mu_i + nw * mt);
    const double rp = (nw * mu_i - mt) / (nw * mu_i + mt);
    const double Rs = rs * rs, Rp = rp * rp;
    const double q = qconv == 1 ? 0.5 * (Rp - Rs) : 0.5 * (Rs - Rp);
    M[0] = 0.5 * (Rs + Rp); M[1] = q; M[3] = q; M[4] = 0.5 * (Rs + Rp); M[8] = rs * rp;
}

static void rot_L(double c, double s, double *L)
{
    const double c2 = c * c - s * s, s2 = 2.0 * c * s;
    for (int i = 0; i < 9; ++i) L[i] = 0.0;
    L[0] = 1.0; L[4] = c2; L[5] = -s2; L[7] = s2; L[8] = c2;
}

static void mul3(const double *A, const double *B, double *C)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += A[i * 3 + k] * B[k * 3 + j];
            C[i * 3 + j] = s;
        }
}

void ocrt_oracle_coxmunk_R(double mu_out, double mu_in_dn, double cphi, double sphi,
                           double ws, int sigma_type, double nw, int qconv, double *R)
{
    for (int i = 0; i < 9; ++i) R[i] = 0.0;
    const double s2v = slope_variance(ws, sigma_type);
    const double mi = -mu_in_dn;
    const double s1 = sqrt(fmax(0.0, 1.0 - mu_out * mu_out));
    const double s2 = sqrt(fmax(0.0, 1.0 - mi * mi));
    double cT = mu_out * mi + s1 * s2 * cphi;
    cT = cT > 1.0 ? 1.0 : (cT < -1.0 ? -1.0 : cT);
    const double cw = sqrt(fmax(0.0, 0.5 * (1.0 - cT)));
    if (cw <= 1e-6) return;
    const double cb = (mu_out + mu_in_dn) / (2.0 * cw);
    if (cb <= 1e-6) return;
    const double sT = sqrt(fmax(0.0, 1.0 - cT * cT));
    const double den = fmax(1e-12, sT);
    const double pole = 1.0e-8;        /* surface.c:57 pole limit */
    double c1, si1, c2, si2;
    if (s2 <= pole) { c1 = -copysign(1.0, mi) * cphi; si1 = sphi; }
    else {
        c1 = (mu_out - mi * cT) / (den * fmax(1e-12, s2));
        si1 = s1 * sphi / den;
        const double nn = sqrt(c1 * c1 + si1 * si1);
        if (nn < 1e-12) { c1 = 1.0; si1 = 0.0; } else { c1 /= nn; si1 /= nn; }
    }
    if (s1 <= pole) { c2 = -copysign(1.0, mu_out) * cphi; si2 = sphi; }
    else {
        c2 = (mi - mu_out * cT) / (den * fmax(1e-12, s1));
        si2 = s2 * sphi / den;
        const double nn = sqrt(c2 * c2 + si2 * si2);
        if (nn < 1e-12) { c2 = 1.0; si2 = 0.0; } else { c2 /= nn; si2 /= nn; }
    }
    double MF[9];
    fresnel_R(cw, nw, qconv, MF);
    const double cb2 = cb * cb;
    const double tb2 = (1.0 - cb2) / fmax(cb2, 1e-8);
    const double Pslope = (1.0 / (PI * s2v)) * exp(-tb2 / s2v);
    const double sl = sqrt(s2v);
    double li = 0.0, lv = 0.0;
    if (mu_in_dn < 1.0 - 1e-10) {
        const double si = sqrt(fmax(1e-20, 1.0 - mu_in_dn * mu_in_dn));
        const double nu = (mu_in_dn / si) / sl;
        if (nu <= 20.0) li = 0.5 * (exp(-nu * nu) / (nu * sqrt(PI)) - erfc(nu));
    }
    if (mu_out < 1.0 - 1e-10) {
        const double sv = sqrt(fmax(1e-20, 1.0 - mu_out * mu_out));
        const double nu = (mu_out / sv) / sl;
        if (nu <= 20.0) lv = 0.5 * (exp(-nu * nu) / (nu * sqrt(PI)) - erfc(nu));
    }
    const double S = 1.0 / (1.0 + li + lv);
    const double brdf = (Pslope * S) / (4.0 * mu_in_dn * mu_out * cb2 * cb2);
    double L1[9], L2[9], A[9], B[9];
    rot_L(c1, si1, L1);
    rot_L(c2, si2, L2);
    mul3(MF, L1, A);
    mul3(L2, A, B);
    for (int i = 0; i < 9; ++i) R[i] = B[i] * brdf;
}

/* Azimuthal Fourier projection of the Cox-Munk Mueller kernel for all modes
 * 0..M at once (shared/surface.c:839-909; the all-mode build of
 * surface.c:1005-1057).  out[m][o][i][9]. */
static void coxmunk_fourier_allm(const double *mu_o, int no, const double *mu_i, int ni,
                                 int M, int nphi, double ws, int st, double nw, int qc,
                                 double *out)
{
    static const int cos_entry[9] = {1, 1, 0, 1, 1, 0, 0, 0, 1};
    const double dphi = 2.0 * PI / (double)nphi;
    double *cm = malloc(sizeof(double) * (size_t)nphi * (M + 1) * 2);
    double *sm = cm + (size_t)nphi * (M + 1);
    for (int p = 0; p < nphi; ++p) {
        const double phi = (p + 0.5) * dphi;
        for (int m = 0; m <= M; ++m) {
            cm[(size_t)p * (M + 1) + m] = cos(m * phi);
            sm[(size_t)p * (M + 1) + m] = sin(m * phi);
        }
    }
    const size_t slab = (size_t)no * ni * 9;
    memset(out, 0, sizeof(double) * slab * (M + 1));
    for (int o = 0; o < no; ++o)
        for (int i = 0; i < ni; ++i) {
            for (int p = 0; p < nphi; ++p) {
                const double phi = (p + 0.5) * dphi;
                double R[9];
                ocrt_oracle_coxmunk_R(mu_o[o], mu_i[i], cos(phi), sin(phi), ws, st, nw, qc, R);
                for (int m = 0; m <= M; ++m) {
                    double *dst = out + (size_t)m * slab + ((size_t)o * ni + i) * 9;
                    const double cw = cm[(size_t)p * (M + 1) + m], sw = sm[(size_t)p * (M + 1) + m];
                    for (int e = 0; e < 9; ++e) dst[e] += R[e] * (cos_entry[e] ? cw : sw);
                }
            }
            for (int m = 0; m <= M; ++m) {
                const double norm = m == 0 ? 1.0 / (2.0 * PI) : 1.0 / PI;
                double *dst = out + (size_t)m * slab + ((size_t)o * ni + i) * 9;
                for (int e = 0; e < 9; ++e) dst[e] *= dphi * norm;
                if (m > 0) { dst[2] = -dst[2]; dst[5] = -dst[5]; }
            }
        }
    free(cm);
}

/* Direct sunglint reflectance (shared/surface.c:1813-1907). */
static void sunglint_rho(double mu_v, double phi_v, double mu0, double ws, int st,
                         double nw, double tau, int qc, double *g)
{
    const double dphi = phi_v;
    const double trans = exp(-tau / mu0) * exp(-tau / mu_v);
    if (ws < 1e-6) {
        const double fov = 0.5 * PI / 180.0;
        const double s0 = sqrt(fmax(0.0, 1.0 - mu0 * mu0));
        const double smu = fov * fmax(s0, 1e-3), sph = fov;
        double de = dphi;
        while (de > PI) de -= 2.0 * PI;
        while (de < -PI) de += 2.0 * PI;
        const double dm = mu_v - mu0;
        const double ex = -0.5 * (dm * dm / (smu * smu) + de * de / (sph * sph));
        if (ex < -50.0) { g[0] = g[1] = g[2] = 0.0; return; }
        double MF[9];
        fresnel_R(mu0, nw, qc, MF);
        const double den = fmax(2.0 * mu0 * s0 * mu0 * mu_v, 1e-12);
        const double r = 4.0 * PI * trans / den * exp(ex);
        g[0] = MF[0] * r; g[1] = MF[3] * r; g[2] = MF[6] * r;
        return;
    }
    double R[9];
    ocrt_oracle_coxmunk_R(mu_v, mu0, cos(dphi), sin(dphi), ws, st, nw, qc, R);
    g[0] = PI * R[0] * trans; g[1] = PI * R[3] * trans; g[2] = PI * R[6] * trans;
}

/* ======================================================================
 * IPSS spherical single-scatter correction (rt_ipss.c:24-644), surface
 * anchor, phase-weighted source when aerosol scatters.
 * ==================================================================== */
typedef struct {
    int nl;
    double Re, H, mu0, depol;
    double *he, *beta, *wsrc, *wray, *waer, *above;
    double *seg, *ts, *lt, *ltau;
    int *llay, ln;
    const ocrt_aerosol *aer;
} ipss_t;

static void ipss_free(ipss_t *g)
{
    free(g->he); free(g->beta); free(g->wsrc); free(g->wray); free(g->waer); free(g->above);
    free(g->seg); free(g->ts); free(g->lt); free(g->ltau); free(g->llay);
    memset(g, 0, sizeof(*g));
}

static int ipss_init(ipss_t *g, const medium_t *md, double mu0, const ocrt_aerosol *aer)
{
    memset(g, 0, sizeof(*g));
    const int nt = md->nt;
    g->nl = nt; g->Re = 6371.0; g->mu0 = mu0; g->depol = DEPOL;
    g->he = malloc(sizeof(double) * (nt + 1));
    g->beta = malloc(sizeof(double) * nt);
    g->wsrc = malloc(sizeof(double) * nt);
    g->wray = malloc(sizeof(double) * nt);
    g->waer = malloc(sizeof(double) * nt);
    g->above = malloc(sizeof(double) * (nt + 1));
    g->seg = malloc(sizeof(double) * nt);
    g->ts = malloc(sizeof(double) * (2 * nt + 8));
    g->lt = malloc(sizeof(double) * (2 * nt + 8));
    g->ltau = malloc(sizeof(double) * (2 * nt + 8));
    g->llay = malloc(sizeof(int) * (2 * nt + 8));
    for (int k = 0; k <= nt; ++k) g->he[k] = md->z[nt - k];
    g->H = g->he[nt];
    int have_aer = 0;
    for (int j = 0; j < nt; ++j) {
        const int k = nt - 1 - j;
        const double dz = g->he[j + 1] - g->he[j];
        const double dtau = md->h[k + 1] - md->h[k];
        if (!(dz > 0.0)) return -2;
        g->beta[j] = dtau > 0.0 ? dtau / dz : 0.0;
        g->wray[j] = md->ydel[k + 1] > 0.0 ? md->ydel[k + 1] : 0.0;
        g->waer[j] = md->xdel[k + 1] > 0.0 ? md->xdel[k + 1] : 0.0;
        if (md->xdel[k + 1] > 0.0) have_aer = 1;
        /* phase-free source weight: the layer's scattering fraction of its
         * extinction, 1 without gas (rt_ipss.c:64-70) */
        double ta = md->tabs ? md->tabs[k] : 0.0;
        if (ta < 0.0) ta = 0.0;
        if (ta > dtau) ta = dtau;
        g->wsrc[j] = dtau > 0.0 ? (dtau - ta) / dtau : 0.0;
    }
    g->aer = (have_aer && aer) ? aer : NULL;
    g->above[nt] = 0.0;
    for (int j = nt - 1; j >= 0; --j) g->above[j] = g->above[j + 1] + g->beta[j] * (g->he[j + 1] - g->he[j]);
    return 0;
}

static int ipss_layer_of(const ipss_t *g, double h)
{
    if (h <= g->he[0]) return 0;
    if (h >= g->he[g->nl]) return g->nl - 1;
    int lo = 0, hi = g->nl;
    while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (g->he[mid] <= h) lo = mid; else hi = mid; }
    return lo > g->nl - 1 ? g->nl - 1 : lo;
}

/* Slant depth toward the sun from rB; INFINITY when shadowed (rt_ipss.c:233-329). */
static double ipss_tau_sun(ipss_t *g, const double *r0)
{
    const int nl = g->nl;
    const double sn = sqrt(fmax(0.0, 1.0 - g->mu0 * g->mu0));
    double u[3] = {-sn, 0.0, g->mu0};
    const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    u[0] /= un; u[1] /= un; u[2] /= un;
    const double b = r0[0] * u[0] + r0[1] * u[1] + r0[2] * u[2];
    const double c0 = r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2];
    double tstop = INFINITY;
    int hit = 0;
    const double dg = b * b - (c0 - g->Re * g->Re);
    if (dg >= 0.0) {
        const double sq = sqrt(dg);
        const double cand[2] = {-b - sq, -b + sq};
        for (int i = 0; i < 2; ++i)
            if (cand[i] > 1e-9 && cand[i] < tstop) { tstop = cand[i]; hit = 1; }
    }
    if (hit) return INFINITY;
    const int cap = 2 * nl + 8;
    int cnt = 0;
    g->ts[cnt++] = 0.0;
    for (int k = nl; k >= 0; --k) {
        const double R = g->Re + g->he[k], d = b * b - (c0 - R * R);
        if (d < 0.0) continue;
        const double t = -b - sqrt(d);
        if (t > 1e-9 && t <= tstop && cnt < cap) g->ts[cnt++] = t;
    }
    for (int k = 0; k <= nl; ++k) {
        const double R = g->Re + g->he[k], d = b * b - (c0 - R * R);
        if (d < 0.0) continue;
        const double t = -b + sqrt(d);
        if (t > 1e-9 && t <= tstop && cnt < cap) g->ts[cnt++] = t;
    }
    int mm = 0;
    for (int i = 0; i < cnt; ++i)
        if (i == 0 || g->ts[i] > g->ts[mm - 1] + 1e-12) g->ts[mm++] = g->ts[i];
    double tau = 0.0;
    for (int i = 0; i + 1 < mm; ++i) {
        const double ta = g->ts[i], tb = g->ts[i + 1], tm = 0.5 * (ta + tb);
        const double hm = sqrt(tm * tm + 2.0 * b * tm + c0) - g->Re;
        if (hm < 0.0 || hm > g->he[nl]) continue;
        int lo = 0, hi = nl;
        while (hi - lo > 1) { const int mid = (lo + hi) / 2; if (g->he[mid] <= hm) lo = mid; else hi = mid; }
        if (lo > nl - 1) lo = nl - 1;
        tau += (tb - ta) * g->beta[lo];
    }
    return tau;
}

static double ipss_phase_aer(const ipss_t *g, double ct)
{
    const ocrt_aerosol *a = g->aer;
    if (a->use_value_kernel && a->n_ang_phase > 1) return aer_p11_table(a, ct);
    double p0 = 1.0, p1 = ct, s = a->beta[0];
    if (a->L_max >= 1) s += a->beta[1] * p1;
    for (int l = 2; l <= a->L_max; ++l) {
        const double p2 = ((2.0 * l - 1.0) * ct * p1 - (l - 1.0) * p0) / l;
        s += a->beta[l] * p2; p0 = p1; p1 = p2;
    }
    return s > 0.0 ? s : 0.0;
}

static double ipss_kappa(ipss_t *g, double vza, double raa)
{
    const int nl = g->nl;
    const double tv = vza * PI / 180.0, fp = (180.0 - raa) * PI / 180.0;
    if (g->aer) {
        const double sn = sqrt(fmax(0.0, 1.0 - g->mu0 * g->mu0));
        const double ct = sn * sin(tv) * cos(fp) - g->mu0 * cos(tv);
        const double d = (g->depol >= 0.0 && g->depol < 1.0) ? g->depol : 0.0;
        const double PR = 1.0 + (1.0 - d) / (2.0 + d) * 0.5 * (3.0 * ct * ct - 1.0);
        const double PA = ipss_phase_aer(g, ct);
        for (int j = 0; j < nl; ++j) g->wsrc[j] = g->wray[j] * PR + g->waer[j] * PA;
    }
    /* plane-parallel single scatter (rt_ipss.c:595-615) */
    const double mv = cos(tv);
    double Ipp = 0.0;
    if (mv > 0.0) {
        const double C = 1.0 / mv + 1.0 / g->mu0;
        for (int j = 0; j < nl; ++j) {
            if (!(g->beta[j] > 0.0)) continue;
            Ipp += g->wsrc[j] / (mv * C) * (exp(-C * g->above[j + 1]) - exp(-C * g->above[j]));
        }
    }
    /* spherical single scatter along the pixel-anchored line of sight */
    const double u[3] = {sin(tv) * cos(fp), sin(tv) * sin(fp), cos(tv)};
    const double Rt = g->Re + g->H;
    const double bq = g->Re * u[2];
    const double disc = bq * bq + Rt * Rt - g->Re * g->Re;
    double Iss = 0.0;
    if (disc > 0.0) {
        const double s = -bq + sqrt(disc);
        if (s > 0.0) {
            const double rA[3] = {s * u[0], s * u[1], g->Re + s * u[2]};
            const double dmax = s;
            const double b = -(rA[0] * u[0] + rA[1] * u[1] + rA[2] * u[2]);
            const double c0 = rA[0] * rA[0] + rA[1] * rA[1] + rA[2] * rA[2];
            const int cap = 2 * nl + 8;
            int cnt = 0;
            g->lt[cnt++] = 0.0;
            for (int k = nl; k >= 0; --k) {
                const double R = g->Re + g->he[k], d = b * b - (c0 - R * R);
                if (d < 0.0) continue;
                const double t = -b - sqrt(d);
                if (t > 1e-12 && t <= dmax && cnt < cap) g->lt[cnt++] = t;
            }
            for (int k = 0; k <= nl; ++k) {
                const double R = g->Re + g->he[k], d = b * b - (c0 - R * R);
                if (d < 0.0) continue;
                const double t = -b + sqrt(d);
                if (t > 1e-12 && t <= dmax && cnt < cap) g->lt[cnt++] = t;
            }
            if (cnt < cap) g->lt[cnt++] = dmax;
            int mm = 0;
            for (int i = 0; i < cnt; ++i)
                if (i == 0 || g->lt[i] > g->lt[mm - 1] + 1e-12) g->lt[mm++] = g->lt[i];
            double tau = 0.0;
            for (int i = 0; i + 1 < mm; ++i) {
                const double tm = 0.5 * (g->lt[i] + g->lt[i + 1]);
                const double rmid = sqrt(tm * tm + 2.0 * b * tm + c0);
                const int j = ipss_layer_of(g, rmid - g->Re);
                g->llay[i] = j; g->ltau[i] = tau;
                tau += (g->lt[i + 1] - g->lt[i]) * g->beta[j];
            }
            g->ln = mm;
            const double xq = 1.0 / sqrt(3.0);     /* 2-point Gauss-Legendre per panel */
            for (int i = 0; i + 1 < mm; ++i) {
                const int j = g->llay[i];
                if (!(g->beta[j] > 0.0)) continue;
                const double sa = g->lt[i], sb = g->lt[i + 1];
                const double half = 0.5 * (sb - sa), mid = 0.5 * (sa + sb);
                for (int q = 0; q < 2; ++q) {
                    const double sq = mid + half * (q == 0 ? -xq : xq);
                    const double rB[3] = {rA[0] - sq * u[0], rA[1] - sq * u[1], rA[2] - sq * u[2]};
                    const double hB = sqrt(rB[0] * rB[0] + rB[1] * rB[1] + rB[2] * rB[2]) - g->Re;
                    if (hB < 0.0 || hB > g->H) continue;
                    const double tview = g->ltau[i] + (sq - sa) * g->beta[j];
                    const double tsun = ipss_tau_sun(g, rB);
                    if (!isfinite(tsun)) continue;
                    Iss += half * g->beta[j] * g->wsrc[j] * exp(-tview - tsun);
                }
            }
        }
    }
    if (!(Ipp > 1.0e-300) || !isfinite(Iss)) return 1.0;
    return Iss / Ipp;
}

/* ======================================================================
 * Single-pixel solve (rt_solver.c:618-1436 with rt_solver_sos_pol
 * :1987-2212 and rt_solver_sos_pol_with_surface :2923-3150).
 * ==================================================================== */
static double sup_norm(const ctx_t *c, const double *X)
{
    double mx = 0.0;
    for (int k = 0; k <= c->md.nt; ++k)
        for (int j = -c->n; j <= c->n; ++j) {
            if (j == 0) continue;
            const double a = fabs(F(X, c, k, j));
            if (a > mx) mx = a;
        }
    return mx;
}

static double interp_pos(const double *mu_pos, const double *vals, int n, double mu)
{
    int jh = 1;
    while (jh < n && mu_pos[jh - 1] < mu) jh++;
    int jl = jh - 1;
    if (jl < 1) { jl = 1; jh = 2; }
    if (jh > n) { jh = n; jl = n - 1; }
    const double t = (mu - mu_pos[jl - 1]) / (mu_pos[jh - 1] - mu_pos[jl - 1]);
    return (1.0 - t) * vals[jl - 1] + t * vals[jh - 1];
}

/* Monotone cubic (PCHIP) sample of ring values at mu (rt_solver.c:435-481,
 * the Fritsch-Carlson method with the weighted-harmonic interior slope and
 * the three-point one-sided edge slope with its monotonicity clamp).  The
 * bracket is that of interp_pos; outside the node range, or with fewer than
 * four nodes, the linear sample is returned. */
static double pchip_slope_interior(double h0, double h1, double s0, double s1)
{
    if (s0 == 0.0 || s1 == 0.0 || (s0 > 0.0) != (s1 > 0.0)) return 0.0;
    const double w1 = 2.0 * h1 + h0, w2 = h1 + 2.0 * h0;
    return (w1 + w2) / (w1 / s0 + w2 / s1);
}

static double pchip_slope_edge(double h0, double h1, double s0, double s1)
{
    double d = ((2.0 * h0 + h1) * s0 - h0 * s1) / (h0 + h1);
    if (d == 0.0 || s0 == 0.0 || (d > 0.0) != (s0 > 0.0)) {
        if (s0 == 0.0 || (d > 0.0) != (s0 > 0.0)) d = 0.0;
    } else if (((s0 > 0.0) != (s1 > 0.0)) && fabs(d) > 3.0 * fabs(s0)) {
        d = 3.0 * s0;
    }
    return d;
}

static double pchip_pos(const double *mu_pos, const double *vals, int n, double mu)
{
    int jh = 1;
    while (jh < n && mu_pos[jh - 1] < mu) jh++;
    const int jl = jh - 1;
    if (jl < 1 || jh > n || n < 4) return interp_pos(mu_pos, vals, n, mu);
    const double x1 = mu_pos[jl - 1], x2 = mu_pos[jh - 1], y1 = vals[jl - 1], y2 = vals[jh - 1];
    const double h = x2 - x1, sl = (y2 - y1) / h;
    double d1, d2;
    if (jl == 1) {
        const double x3 = mu_pos[jh], s2 = (vals[jh] - y2) / (x3 - x2);
        d1 = pchip_slope_edge(h, x3 - x2, sl, s2);
        d2 = pchip_slope_interior(h, x3 - x2, sl, s2);
    } else if (jh == n) {
        const double x0 = mu_pos[jl - 2], s0 = (y1 - vals[jl - 2]) / (x1 - x0);
        d1 = pchip_slope_interior(x1 - x0, h, s0, sl);
        d2 = pchip_slope_edge(h, x1 - x0, sl, s0);
    } else {
        const double x0 = mu_pos[jl - 2], x3 = mu_pos[jh];
        const double s0 = (y1 - vals[jl - 2]) / (x1 - x0), s2 = (vals[jh] - y2) / (x3 - x2);
        d1 = pchip_slope_interior(x1 - x0, h, s0, sl);
        d2 = pchip_slope_interior(h, x3 - x2, sl, s2);
    }
    const double t = (mu - x1) / h, t2 = t * t, t3 = t2 * t;
    return (2.0 * t3 - 3.0 * t2 + 1.0) * y1 + (t3 - 2.0 * t2 + t) * h * d1 + (-2.0 * t3 + 3.0 * t2) * y2 +
           (t3 - t2) * h * d2;
}

static double recon_cos(const double *v, int M, double dphi)
{
    const double phi = dphi + PI;
    double s = v[0];
    for (int m = 1; m <= M; ++m) s += 2.0 * v[m] * cos((double)m * phi);
    return s;
}

static double recon_sin(const double *v, int M, double dphi)
{
    if (M < 1) return 0.0;
    const double phi = dphi + PI;
    double s = 0.0;
    for (int m = 1; m <= M; ++m) s += 2.0 * v[m] * sin((double)m * phi);
    return s;
}

/* Flat-Fresnel reflected direct beam scattered once by the atmosphere
 * (rt_surface_boundary.c:210-428). */
static int flat_reflected_beam(const ctx_t *c, const mode_t_ *md, const ocrt_aerosol *aer,
                               double nw, int qc, double *tot[3], double *o1[3])
{
    const int n = c->n, nt = c->md.nt, m = md->m, nd = 2 * n + 1;
    const size_t cnt = (size_t)(nt + 1) * nd;
    const double mu0 = c->mu0, n2 = nw * nw;
    const double tn = sqrt(n2 - 1.0 + mu0 * mu0);
    const double rp = (n2 * mu0 - tn) / (n2 * mu0 + tn), rs = (mu0 - tn) / (mu0 + tn);
    const double RI = (rp * rp + rs * rs) / 2.0;
    const double RQ = qc == 1 ? (rp * rp - rs * rs) / 2.0 : (rs * rs - rp * rp) / 2.0;
    const double sb = 0.5 * exp(-2.0 * c->md.h[nt] / mu0);
    const double bP = md->xpl[RIDX(n, 0)], bR = md->xrl[RIDX(n, 0)];
    const double b0 = m == 0 ? c->beta0 : 0.0;
    const int mol = m <= 2;
    double *S = calloc(cnt * 6, sizeof(double));
    if (!S) return -3;
    double *SI = S, *SQ = S + cnt, *SU = S + 2 * cnt, *FI = S + 3 * cnt, *FQ = S + 4 * cnt, *FU = S + 5 * cnt;
    const int L = md->L;
    for (int layer = 0; layer < nt; ++layer) {
        const double yt = c->md.ydel[layer], xt_ = c->md.xdel[layer];
        const double yb = c->md.ydel[layer + 1], xb = c->md.xdel[layer + 1];
        const double btop = sb * exp(c->md.h[layer] / mu0), bbot = sb * exp(c->md.h[layer + 1] / mu0);
        for (int d = 1; d <= n; ++d) {
            double K[2][6];
            for (int side = 0; side < 2; ++side) {
                const int jd = side == 0 ? -d : d;     /* top kernel uses the mirrored direction */
                const double p = md->xpl[RIDX(n, jd)], r = md->xrl[RIDX(n, jd)], t = md->xtl[RIDX(n, jd)];
                double pRT = 0.0, pTR = 0.0;
                if (aer) {
                    for (int l = m; l <= L; ++l) {
                        const double Pj = md->P[(size_t)l * nd + RIDX(n, jd)];
                        const double Rj = md->R[(size_t)l * nd + RIDX(n, jd)];
                        const double Tj = md->T[(size_t)l * nd + RIDX(n, jd)];
                        const double R0 = md->R[(size_t)l * nd + RIDX(n, 0)];
                        const double T0 = md->T[(size_t)l * nd + RIDX(n, 0)];
                        const double ga = l <= aer->L_max ? aer->gamma[l] : 0.0;
                        const double al = l <= aer->L_max ? aer->alpha[l] : 0.0;
                        const double ze = l <= aer->L_max ? aer->zeta[l] : 0.0;
                        pRT += Pj * R0 * ga;
                        pTR += Tj * R0 * al + Rj * T0 * ze;
                    }
                }
                const double xx = side == 0 ? xt_ : xb, yy = side == 0 ? yt : yb;
                K[side][0] = TAB(md->pfm, n, 0, jd) * xx + (mol ? b0 + c->beta2 * p * bP : 0.0) * yy;
                K[side][1] = TAB(md->gr, n, 0, jd) * xx + (mol ? c->gamma2 * r * bP : 0.0) * yy;
                K[side][2] = TAB(md->gt, n, 0, jd) * xx + (mol ? c->gamma2 * t * bP : 0.0) * yy;
                K[side][3] = pRT * xx + (mol ? c->gamma2 * bR * p : 0.0) * yy;
                K[side][4] = TAB(md->arr, n, 0, jd) * xx + (mol ? c->alpha2 * bR * r : 0.0) * yy;
                K[side][5] = pTR * xx + (mol ? c->alpha2 * t * bR : 0.0) * yy;
            }
            F(SI, c, layer, d) = btop * (RI * K[0][0] + RQ * K[0][3]);
            F(SQ, c, layer, d) = btop * (RI * K[0][1] + RQ * K[0][4]);
            F(SU, c, layer, d) = btop * (RI * K[0][2] + RQ * K[0][5]);
            F(SI, c, layer + 1, -d) = bbot * (RI * K[1][0] + RQ * K[1][3]);
            F(SQ, c, layer + 1, -d) = bbot * (RI * K[1][1] + RQ * K[1][4]);
            F(SU, c, layer + 1, -d) = bbot * (RI * K[1][2] + RQ * K[1][5]);
        }
    }
    for (int k = 0; k <= nt; ++k) F(SI, c, k, 0) = F(SQ, c, k, 0) = F(SU, c, k, 0) = NAN;
    int rc = transport(c, SI, NULL, FI);
    if (!rc) rc = transport(c, SQ, NULL, FQ);
    if (!rc) rc = transport(c, SU, NULL, FU);
    if (!rc) {
        double *fs[3] = {FI, FQ, FU};
        for (int s = 0; s < 3; ++s)
            for (int k = 0; k <= nt; ++k)
                for (int j = -n; j <= n; ++j) {
                    if (j == 0) continue;
                    F(tot[s], c, k, j) += F(fs[s], c, k, j);
                    F(o1[s], c, k, j) += F(fs[s], c, k, j);
                }
    }
    free(S);
    return rc ? -2 : 0;
}

static int check_args(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer)
{
    if (!cs || !op) return -1;
    if (!(cs->wavelength_nm >= 330.0 - 1e-9 && cs->wavelength_nm <= 1100.0 + 1e-9)) return -1;
    if (cs->sza_deg < 0.0 || cs->sza_deg >= 90.0) return -1;
    if (cs->vza_deg < 0.0 || cs->vza_deg >= 90.0) return -1;
    if (op->fourier_m_max < 0 || op->fourier_m_max > 255) return -1;
    if (op->n_mu < 2 || op->n_mu > 64 || op->n_layers < 2) return -1;
    if (op->max_orders < 1 || !(op->tolerance > 0.0)) return -1;
    if (aer) {
        if (aer->tau_a < 0.0 || aer->ssa_a < 0.0 || aer->ssa_a > 1.0 || aer->L_max < 2) return -1;
        if (!aer->beta || !aer->gamma || !aer->alpha || !aer->zeta) return -1;
    }
    if (cs->surface != OCRT_SURFACE_BLACK && cs->surface != OCRT_SURFACE_BLACK_FRESNEL_OCEAN &&
        cs->surface != OCRT_SURFACE_FLAT) return -5;
    if ((cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN || cs->surface == OCRT_SURFACE_FLAT) &&
        !(cs->n_water > 0.0)) return -1;
    return 0;
}

/* Per-layer overrides (no reference counterpart; the parameters of the
 * adjoint).  Layer l (0-based) spans levels l..l+1.  dtau replaces the uniform
 * optical-depth grid by h[k] = sum_{l<k} dtau[l]; ssa[l] rescales level l+1's
 * scattering fractions (xdel, ydel) so that xdel + ydel = ssa[l], keeping the
 * aerosol/molecular split of that layer.  The level altitudes, and with them
 * the mixing fractions, stay those of the uniform grid; IPSS is not allowed
 * with overrides (it would need the altitudes of the new grid). */
static int apply_layers(medium_t *md, const ocrt_layers *ly, double mu0)
{
    const int nt = md->nt;
    if (ly->n_layers != nt) return -1;
    if (ly->dtau) {
        double h = 0.0;
        md->h[0] = 0.0;
        for (int l = 0; l < nt; ++l) {
            if (!(ly->dtau[l] > 0.0) || !isfinite(ly->dtau[l])) return -1;
            h += ly->dtau[l];
            md->h[l + 1] = h;
        }
        md->tau_total = h;
        for (int k = 0; k <= nt; ++k) md->ch[k] = 0.5 * exp(-md->h[k] / mu0);
    }
    if (ly->ssa) {
        for (int l = 0; l < nt; ++l) {
            const double w = ly->ssa[l], w0 = md->xdel[l + 1] + md->ydel[l + 1];
            if (!(w >= 0.0 && w <= 1.0) || !(w0 > 0.0)) return -1;
            md->xdel[l + 1] *= w / w0;
            md->ydel[l + 1] *= w / w0;
        }
    }
    return 0;
}

int ocrt_oracle_solve_case(const ocrt_case *cs, const ocrt_opts *op,
                           const ocrt_aerosol *aer_in, ocrt_result *out, ocrt_diag *diag)
{
    return ocrt_oracle_solve_case_layers(cs, op, aer_in, NULL, out, diag);
}

int ocrt_oracle_solve_case_layers(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                                  const ocrt_layers *layers, ocrt_result *out, ocrt_diag *diag)
{
    return solve_impl(cs, op, aer_in, layers, NULL, out, diag);
}

/* Angle-grid LUT (rt_solve_case_pol_lut, rt_solver.c:870-900, 1025-1045,
 * 1276-1424). */
int ocrt_oracle_solve_case_lut(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                               ocrt_result *out, ocrt_lut *lut)
{
    if (!lut || lut->n_vza <= 0 || lut->n_raa <= 0 || !lut->vza_deg || !lut->raa_deg || !lut->rho_I ||
        !lut->rho_Q || !lut->rho_U) return -1;
    for (int i = 0; i < lut->n_vza; ++i)
        if (!(lut->vza_deg[i] >= 0.0 && lut->vza_deg[i] < 90.0)) return -1;
    return solve_impl(cs, op, aer_in, NULL, lut, out, NULL);
}

static int solve_impl(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                      const ocrt_layers *layers, ocrt_lut *lut, ocrt_result *out, ocrt_diag *diag)
{
    int rc = check_args(cs, op, aer_in);
    if (rc) return rc;
    if (!out) return -1;
    if (layers && op->pssa) return -5;
    memset(out, 0, sizeof(*out));
    const ocrt_aerosol *aer = (aer_in && aer_in->tau_a > 0.0) ? aer_in : NULL;

    ctx_t *c = calloc(1, sizeof(ctx_t));
    if (!c) return -3;
    c->mu0 = cos(cs->sza_deg * PI / 180.0);
    c->mu_view = cos(cs->vza_deg * PI / 180.0);
    const double dphi = cs->raa_deg * PI / 180.0;

    double tau_r;
    if (!(cs->pressure_hpa > 0.0)) tau_r = 0.0;
    else if (op->tau_r_source == OCRT_TAU_R_FROM_INPUT) {
        if (cs->tau_r_input <= 0.0) { free(c); return -1; }
        tau_r = cs->tau_r_input;
    } else tau_r = ocrt_oracle_tau_rayleigh(cs->wavelength_nm, cs->pressure_hpa);
    out->tau_R_total = tau_r;

    /* ring: Gauss nodes plus the view direction as a zero-weight node */
    double mu_r[MAX_RING], w_r[MAX_RING];
    int nr = op->n_mu;
    if (ocrt_oracle_gauss(op->n_mu, mu_r, w_r)) { free(c); return -1; }
    c->view_idx = 0;
    if (op->view_as_node) c->view_idx = ring_insert(mu_r, w_r, &nr, c->mu_view) + 1;
    const int n = nr, nt = op->n_layers, nd = 2 * n + 1, M = op->fourier_m_max;
    c->n = n;
    if (g_atm_hooks) {
        g_atm_hooks->n = n;
        for (int j = 0; j < n; ++j) { g_atm_hooks->mu[j] = mu_r[j]; g_atm_hooks->w[j] = w_r[j]; }
    }
    c->rm[RIDX(n, 0)] = -c->mu0; c->gb[RIDX(n, 0)] = 0.0;
    for (int j = 1; j <= n; ++j) {
        c->rm[RIDX(n, j)] = mu_r[j - 1]; c->rm[RIDX(n, -j)] = -mu_r[j - 1];
        c->gb[RIDX(n, j)] = c->gb[RIDX(n, -j)] = w_r[j - 1];
    }
    /* molecular moments (rt_molecular_phase.c:5-20) */
    const double A = 2.0 * (1.0 - DEPOL) / (2.0 + DEPOL);
    c->beta0 = 1.0; c->beta2 = 0.5 * A; c->gamma2 = -A * sqrt(1.5); c->alpha2 = 3.0 * A;

    if (aer) {
        if (!(tau_r >= 0.0 && tau_r + aer->tau_a > 0.0)) { free(c); return -1; }
        rc = medium_build(&c->md, nt, tau_r, aer->tau_a, aer->ssa_a, c->mu0, op->aer_h_km,
                          op->rayleigh_profile, op->rayleigh_h_km);
    } else {
        if (!(tau_r > 0.0)) { free(c); return -1; }
        rc = medium_build(&c->md, nt, tau_r, 0.0, 1.0, c->mu0, op->aer_h_km,
                          op->rayleigh_profile, op->rayleigh_h_km);
    }
    if (!rc && op->gas) rc = medium_apply_gas(&c->md, op->gas, cs->wavelength_nm, c->mu0);
    if (!rc && layers) rc = apply_layers(&c->md, layers, c->mu0);
    if (rc) { medium_free(&c->md); free(c); return rc; }
    if ((rc = transport_prepare(c))) goto done;

    int L = M > 2 ? M : 2;
    if (aer && aer->L_max > L) L = aer->L_max;
    mode_t_ md;
    if ((rc = mode_alloc(&md, n, L))) goto done;

    const size_t cnt = (size_t)(nt + 1) * nd;
    double *buf = calloc(cnt * 18, sizeof(double));
    if (!buf) { mode_free(&md); rc = -3; goto done; }
    double *Js[3] = {buf, buf + cnt, buf + 2 * cnt};
    double *Pr[3] = {buf + 3 * cnt, buf + 4 * cnt, buf + 5 * cnt};
    double *Tt[3] = {buf + 6 * cnt, buf + 7 * cnt, buf + 8 * cnt};
    double *Ip[3] = {buf + 9 * cnt, buf + 10 * cnt, buf + 11 * cnt};
    double *Ic[3] = {buf + 12 * cnt, buf + 13 * cnt, buf + 14 * cnt};
    double *O1[3] = {buf + 15 * cnt, buf + 16 * cnt, buf + 17 * cnt};

    const int surf_on = cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN || cs->surface == OCRT_SURFACE_FLAT;
    const int flat = cs->surface == OCRT_SURFACE_FLAT ||
                     (cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && cs->wind_speed <= 0.0);
    const int rough = surf_on && !flat;
    double *mu_pos = malloc(sizeof(double) * n);
    for (int j = 1; j <= n; ++j) mu_pos[j - 1] = c->rm[RIDX(n, j)];
    /* rough-surface Fourier kernels for all modes: ring x ring and ring x sun */
    double *Kr = NULL, *Ks = NULL;
    const int nphi = op->n_phi_surface > 0 ? op->n_phi_surface : 1024;
    if (rough) {
        Kr = malloc(sizeof(double) * (size_t)(M + 1) * n * n * 9);
        Ks = malloc(sizeof(double) * (size_t)(M + 1) * n * 9);
        coxmunk_fourier_allm(mu_pos, n, mu_pos, n, M, nphi, cs->wind_speed, cs->sigma_type,
                             cs->n_water, cs->q_convention, Kr);
        coxmunk_fourier_allm(mu_pos, n, &c->mu0, 1, M, nphi, cs->wind_speed, cs->sigma_type,
                             cs->n_water, cs->q_convention, Ks);
    }
    double *I_dn_boa = calloc((size_t)(M + 1) * n, sizeof(double));
    const int nvg = lut ? lut->n_vza : 0;
    double *lut_samp = lut ? calloc((size_t)(M + 1) * nvg * 3, sizeof(double)) : NULL;   /* [m][iv][IQU] */
    double *vI = calloc((size_t)(M + 1) * 3, sizeof(double));
    double *vQ = vI + (M + 1), *vU = vQ + (M + 1);
    double *seed = rough ? calloc(cnt * 3, sizeof(double)) : NULL;
    int max_orders_seen = 0, all_conv = 1, order_modes = 0;

    for (int m = 0; m <= M && !rc; ++m) {
        mode_build(&md, m, c->rm, aer);
        primary_source(c, &md, Js[0], Js[1], Js[2]);
        for (int s = 0; s < 3 && !rc; ++s) if (transport(c, Js[s], NULL, Pr[s])) rc = -2;
        if (rc) break;
        const int bottom_only = g_atm_hooks && g_atm_hooks->bottom_only;
        if (bottom_only)
            for (int s = 0; s < 3; ++s)
                for (int k = 0; k <= nt; ++k)
                    for (int j = -n; j <= n; ++j) if (j) F(Pr[s], c, k, j) = 0.0;
        for (int s = 0; s < 3; ++s) { memcpy(Tt[s], Pr[s], cnt * sizeof(double)); memset(O1[s], 0, cnt * sizeof(double)); }
        int orders = 1, conv = 0;
        double resid = 0.0;
        const double *Krm = rough ? Kr + (size_t)m * n * n * 9 : NULL;
        if (surf_on && !bottom_only) {
            if (flat) {
                if ((rc = flat_reflected_beam(c, &md, aer, cs->n_water, cs->q_convention, Tt, O1))) break;
            } else {
                /* rough direct-beam seed (rt_surface_boundary.c:430-493) */
                const double *Ksm = Ks + (size_t)m * n * 9;
                const double tdn = exp(-c->md.h[nt] / c->mu0);
                const double fs = (m == 0 ? PI : 0.5 * PI) * c->mu0;
                for (int k = 0; k <= nt; ++k) {
                    const double up = c->md.h[nt] - c->md.h[k];
                    for (int o = 1; o <= n; ++o) {
                        const double f = fs * tdn * exp(-up / mu_pos[o - 1]);
                        const double v[3] = {Ksm[(o - 1) * 9 + 0] * f, Ksm[(o - 1) * 9 + 3] * f,
                                             Ksm[(o - 1) * 9 + 6] * f};
                        for (int s = 0; s < 3; ++s) {
                            F(Tt[s], c, k, o) += v[s];
                            F(O1[s], c, k, o) += v[s];
                            seed[(size_t)s * cnt + (size_t)k * nd + RIDX(n, o)] = v[s];
                        }
                    }
                }
            }
        }
        if (g_atm_hooks && g_atm_hooks->ext_I && m <= g_atm_hooks->ext_mmax) {
            const double *ex[3] = {g_atm_hooks->ext_I, g_atm_hooks->ext_Q, g_atm_hooks->ext_U};
            for (int k = 0; k <= nt; ++k) {
                const double up = c->md.h[nt] - c->md.h[k];
                for (int o = 1; o <= n; ++o) {
                    const double att = exp(-up / mu_pos[o - 1]);
                    for (int s = 0; s < 3; ++s) {
                        const double v = ex[s][(size_t)m * n + o - 1] * att;
                        F(Tt[s], c, k, o) += v;
                        F(O1[s], c, k, o) += v;
                    }
                }
            }
        }
        if (op->max_orders > 1) {
            for (int s = 0; s < 3; ++s)
                for (size_t i = 0; i < cnt; ++i) Ip[s][i] = Pr[s][i] + O1[s][i];
            double bc[3][MAX_RING];
            for (int it = 2; it <= op->max_orders; ++it) {
                if ((rc = ms_source(c, &md, Ip[0], Ip[1], Ip[2], Js[0], Js[1], Js[2]))) break;
                if (surf_on) {
                    /* surface boundary operator (rt_surface_boundary.c:137-208) */
                    const double fw = flat ? 2.0 * PI : (m == 0 ? 2.0 * PI : PI);
                    for (int o = 1; o <= n; ++o) {
                        double si = 0, sq = 0, su = 0;
                        if (flat) {
                            const double wo = c->gb[RIDX(n, o)];
                            double MF[9];
                            fresnel_R(mu_pos[o - 1], cs->n_water, cs->q_convention, MF);
                            const double ii = F(Ip[0], c, nt, -o), qq = F(Ip[1], c, nt, -o), uu = F(Ip[2], c, nt, -o);
                            if (wo == 0.0) {
                                si = MF[0] * ii + MF[1] * qq + MF[2] * uu;
                                sq = MF[3] * ii + MF[4] * qq + MF[5] * uu;
                                su = MF[6] * ii + MF[7] * qq + MF[8] * uu;
                            } else {
                                const double dd = 1.0 / (2.0 * PI * mu_pos[o - 1] * wo);
                                const double pw = fw * mu_pos[o - 1] * wo;
                                si = pw * (dd * MF[0] * ii + dd * MF[1] * qq + dd * MF[2] * uu);
                                sq = pw * (dd * MF[3] * ii + dd * MF[4] * qq + dd * MF[5] * uu);
                                su = pw * (dd * MF[6] * ii + dd * MF[7] * qq + dd * MF[8] * uu);
                            }
                        } else {
                            for (int i = 1; i <= n; ++i) {
                                const double wi = c->gb[RIDX(n, i)];
                                if (wi == 0.0) continue;
                                const double pw = fw * mu_pos[i - 1] * wi;
                                const double *R = Krm + ((size_t)(o - 1) * n + (i - 1)) * 9;
                                const double ii = F(Ip[0], c, nt, -i), qq = F(Ip[1], c, nt, -i), uu = F(Ip[2], c, nt, -i);
                                si += pw * (R[0] * ii + R[1] * qq + R[2] * uu);
                                sq += pw * (R[3] * ii + R[4] * qq + R[5] * uu);
                                su += pw * (R[6] * ii + R[7] * qq + R[8] * uu);
                            }
                        }
                        bc[0][o - 1] = si; bc[1][o - 1] = sq; bc[2][o - 1] = su;
                    }
                }
                for (int s = 0; s < 3 && !rc; ++s)
                    if (transport(c, Js[s], surf_on ? bc[s] : NULL, Ic[s])) rc = -2;
                if (rc) break;
                for (int s = 0; s < 3; ++s)
                    for (int k = 0; k <= nt; ++k)
                        for (int j = -n; j <= n; ++j)
                            if (j) F(Tt[s], c, k, j) += F(Ic[s], c, k, j);
                orders = it;
                double mi = 0, mt = 0;
                for (int s = 0; s < 3; ++s) {
                    const double a = sup_norm(c, Ic[s]), b = sup_norm(c, Tt[s]);
                    if (a > mi) mi = a;
                    if (b > mt) mt = b;
                }
                resid = mt > 0.0 ? mi / mt : 0.0;
                if (resid < op->tolerance) { conv = 1; break; }
                for (int s = 0; s < 3; ++s) memcpy(Ip[s], Ic[s], cnt * sizeof(double));
            }
        } else {
            conv = 1;
        }
        if (rc) break;
        if (rough)
            for (int s = 0; s < 3; ++s)
                for (int k = 0; k <= nt; ++k)
                    for (int o = 1; o <= n; ++o)
                        F(Tt[s], c, k, o) -= seed[(size_t)s * cnt + (size_t)k * nd + RIDX(n, o)];
        if (g_atm_hooks && g_atm_hooks->boa_I)
            for (int j = 1; j <= n; ++j) {
                g_atm_hooks->boa_I[(size_t)m * n + j - 1] = F(Tt[0], c, nt, -j);
                g_atm_hooks->boa_Q[(size_t)m * n + j - 1] = F(Tt[1], c, nt, -j);
                g_atm_hooks->boa_U[(size_t)m * n + j - 1] = F(Tt[2], c, nt, -j);
            }
        if (orders > max_orders_seen) max_orders_seen = orders;
        if (!conv) all_conv = 0;
        order_modes += orders;
        if (diag) {
            if (diag->orders_per_m) diag->orders_per_m[m] = orders;
            if (diag->residual_per_m) diag->residual_per_m[m] = resid;
        }
        /* TOA sample at the view (rt_solver.c:1010-1024) */
        if (c->view_idx > 0) {
            vI[m] = F(Tt[0], c, 0, c->view_idx); vQ[m] = F(Tt[1], c, 0, c->view_idx);
            vU[m] = F(Tt[2], c, 0, c->view_idx);
        } else {
            double tmp[3][MAX_RING];
            for (int s = 0; s < 3; ++s) for (int j = 1; j <= n; ++j) tmp[s][j - 1] = F(Tt[s], c, 0, j);
            vI[m] = interp_pos(mu_pos, tmp[0], n, c->mu_view);
            vQ[m] = interp_pos(mu_pos, tmp[1], n, c->mu_view);
            vU[m] = interp_pos(mu_pos, tmp[2], n, c->mu_view);
        }
        for (int j = 1; j <= n; ++j) I_dn_boa[(size_t)m * n + j - 1] = F(Tt[0], c, nt, -j);
        if (lut) {
            double tmp[3][MAX_RING];
            for (int st = 0; st < 3; ++st) for (int j = 1; j <= n; ++j) tmp[st][j - 1] = F(Tt[st], c, 0, j);
            for (int iv = 0; iv < nvg; ++iv) {
                const double mug = cos(lut->vza_deg[iv] * PI / 180.0);
                for (int st = 0; st < 3; ++st)
                    lut_samp[((size_t)m * nvg + iv) * 3 + st] = pchip_pos(mu_pos, tmp[st], n, mug);
            }
        }
        if (diag) {
            if (diag->view_I_m) diag->view_I_m[m] = vI[m];
            if (diag->view_Q_m) diag->view_Q_m[m] = vQ[m];
            if (diag->view_U_m) diag->view_U_m[m] = vU[m];
        }
    }
    if (!rc) {
        const double I = recon_cos(vI, M, dphi), Q = recon_cos(vQ, M, dphi), U = recon_sin(vU, M, dphi);
        out->I_TOA = I; out->Q_TOA = Q; out->U_TOA = U;
        out->rho_I = I / c->mu0; out->rho_Q = Q / c->mu0; out->rho_U = U / c->mu0;
        out->kappa_ipss = 1.0;
        double tau_dir = -1.0;
        ipss_t g;
        int ipss_ready = 0;
        memset(&g, 0, sizeof(g));
        if (op->pssa) {
            if (ipss_init(&g, &c->md, c->mu0, aer) == 0) {
                ipss_ready = 1;
                const double rB[3] = {0.0, 0.0, g.Re};
                const double ts = ipss_tau_sun(&g, rB);
                tau_dir = isfinite(ts) ? ts : -1.0;
                const double kap = ipss_kappa(&g, cs->vza_deg, cs->raa_deg);
                out->kappa_ipss = kap;
                out->rho_I *= kap; out->rho_Q *= kap; out->rho_U *= kap;
                out->I_TOA *= kap; out->Q_TOA *= kap; out->U_TOA *= kap;
            } else rc = -1;
        }
        const double tau_t = c->md.h[nt];
        if (!rc && cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN) {
            const double phi_v = (cs->raa_deg - 180.0) * PI / 180.0;
            const double mv = cs->vza_deg > 0.0 ? c->mu_view : 1.0;
            double g[3];
            sunglint_rho(mv, phi_v, c->mu0, cs->wind_speed, cs->sigma_type, cs->n_water, tau_t,
                         cs->q_convention, g);
            if (tau_dir >= 0.0) {
                const double cg = exp(-(tau_dir - tau_t / c->mu0));
                g[0] *= cg; g[1] *= cg; g[2] *= cg;
            }
            if (cs->decouple_sunglint == 0) { out->rho_I += g[0]; out->rho_Q += g[1]; out->rho_U += -g[2]; }
            if (cs->wind_speed > 0.0) {
                out->T_sg_up_dir = g[0] * c->mu0;
                out->rho_glint_direct_I = g[0]; out->rho_glint_direct_Q = g[1]; out->rho_glint_direct_U = g[2];
            }
        }
        out->n_orders_used = max_orders_seen;
        out->converged = all_conv;
        out->order_modes = order_modes;
        /* transmittances (rt_solver.c:1195-1275) */
        out->T_dir_dn = tau_dir >= 0.0 ? exp(-tau_dir) : exp(-tau_t / c->mu0);
        double fd = 0.0;
        for (int j = 1; j <= n; ++j) fd += mu_pos[j - 1] * c->gb[RIDX(n, j)] * I_dn_boa[j - 1];
        fd *= 2.0 * PI;
        out->T_diff_dn_hemi = fd / (PI * c->mu0);
        out->T_total_dn_hemi = out->T_dir_dn + out->T_diff_dn_hemi;
        double *vdn = calloc(M + 1, sizeof(double));
        for (int m = 0; m <= M; ++m) vdn[m] = interp_pos(mu_pos, I_dn_boa + (size_t)m * n, n, c->mu_view);
        out->T_diff_dn_dir = 2.0 * PI * c->mu_view * recon_cos(vdn, M, dphi) / (PI * c->mu0);
        free(vdn);
        out->T_total_up_dir = out->rho_I * c->mu0;
        out->T_dir_up_view = exp(-tau_t / (c->mu_view > 0.0 ? c->mu_view : 1.0));
        if (!rc && lut) {
            /* per grid direction: Fourier sums, rho, kappa, direct glint (rt_solver.c:1276-1424) */
            lut->T_dir_dn = out->T_dir_dn;
            lut->T_diff_dn_hemi = out->T_diff_dn_hemi;
            const double cglint = (ipss_ready && tau_dir >= 0.0) ? exp(-(tau_dir - tau_t / c->mu0)) : 1.0;
            double pm[3][MAX_M1], dnm[MAX_M1];
            for (int iv = 0; iv < nvg; ++iv) {
                const double mug = cos(lut->vza_deg[iv] * PI / 180.0);
                for (int m = 0; m <= M; ++m) {
                    for (int st = 0; st < 3; ++st) pm[st][m] = lut_samp[((size_t)m * nvg + iv) * 3 + st];
                    dnm[m] = interp_pos(mu_pos, I_dn_boa + (size_t)m * n, n, mug);
                }
                for (int ir = 0; ir < lut->n_raa; ++ir) {
                    const double raa = lut->raa_deg[ir], ph = raa * PI / 180.0;
                    double rI = recon_cos(pm[0], M, ph) / c->mu0;
                    double rQ = recon_cos(pm[1], M, ph) / c->mu0;
                    double rU = recon_sin(pm[2], M, ph) / c->mu0;
                    if (ipss_ready) {
                        const double kg = ipss_kappa(&g, lut->vza_deg[iv], raa);
                        rI *= kg; rQ *= kg; rU *= kg;
                    }
                    double sgI = 0.0;
                    if (cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && cs->wind_speed > 0.0) {
                        const double phv = (raa - 180.0) * PI / 180.0;
                        const double mvu = lut->vza_deg[iv] > 0.0 ? mug : 1.0;
                        double gl[3];
                        sunglint_rho(mvu, phv, c->mu0, cs->wind_speed, cs->sigma_type, cs->n_water, tau_t,
                                     cs->q_convention, gl);
                        gl[0] *= cglint; gl[1] *= cglint; gl[2] *= cglint;
                        if (cs->decouple_sunglint == 0) { rI += gl[0]; rQ += gl[1]; rU += -gl[2]; }
                        sgI = gl[0];
                    }
                    const int idx = iv * lut->n_raa + ir;
                    lut->rho_I[idx] = rI; lut->rho_Q[idx] = rQ; lut->rho_U[idx] = rU;
                    if (lut->T_diff_dn_dir)
                        lut->T_diff_dn_dir[idx] = 2.0 * PI * mug * recon_cos(dnm, M, ph) / (PI * c->mu0);
                    if (lut->T_sg_up_dir) lut->T_sg_up_dir[idx] = sgI * c->mu0;
                    if (lut->T_total_up_dir) lut->T_total_up_dir[idx] = rI * c->mu0;
                }
            }
        }
        ipss_free(&g);
    }
    free(lut_samp); free(seed); free(vI); free(I_dn_boa); free(Kr); free(Ks); free(mu_pos); free(buf);
    mode_free(&md);
done:
    free(c->Tr); free(c->Ca); free(c->Cb);
    medium_free(&c->md);
    free(c);
    return rc;
}

/* Profile values of the per-layer parameters (the defaults that ocrt_layers
 * overrides): dtau[l] = h[l+1] - h[l], ssa[l] = xdel[l+1] + ydel[l+1]. */
int ocrt_oracle_layer_defaults(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                               double *dtau, double *ssa)
{
    int rc = check_args(cs, op, aer_in);
    if (rc) return rc;
    const ocrt_aerosol *aer = (aer_in && aer_in->tau_a > 0.0) ? aer_in : NULL;
    double tau_r;
    if (!(cs->pressure_hpa > 0.0)) tau_r = 0.0;
    else if (op->tau_r_source == OCRT_TAU_R_FROM_INPUT) tau_r = cs->tau_r_input;
    else tau_r = ocrt_oracle_tau_rayleigh(cs->wavelength_nm, cs->pressure_hpa);
    medium_t md;
    const double mu0 = cos(cs->sza_deg * PI / 180.0);
    rc = medium_build(&md, op->n_layers, tau_r, aer ? aer->tau_a : 0.0, aer ? aer->ssa_a : 1.0, mu0,
                      op->aer_h_km, op->rayleigh_profile, op->rayleigh_h_km);
    if (!rc && op->gas) rc = medium_apply_gas(&md, op->gas, cs->wavelength_nm, mu0);
    if (rc) { medium_free(&md); return rc; }
    for (int l = 0; l < op->n_layers; ++l) {
        if (dtau) dtau[l] = md.h[l + 1] - md.h[l];
        if (ssa) ssa[l] = md.xdel[l + 1] + md.ydel[l + 1];
    }
    medium_free(&md);
    return 0;
}

/* Per-layer gas absorption depths and level altitudes of one case
 * (atm->tau_abs_layer and atm->z_km_level after rt_atm_apply_gas_absorption). */
int ocrt_oracle_layer_gas(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                          double *tau_abs, double *z_km)
{
    int rc = check_args(cs, op, aer_in);
    if (rc) return rc;
    const ocrt_aerosol *aer = (aer_in && aer_in->tau_a > 0.0) ? aer_in : NULL;
    double tau_r;
    if (!(cs->pressure_hpa > 0.0)) tau_r = 0.0;
    else if (op->tau_r_source == OCRT_TAU_R_FROM_INPUT) tau_r = cs->tau_r_input;
    else tau_r = ocrt_oracle_tau_rayleigh(cs->wavelength_nm, cs->pressure_hpa);
    if (!aer && !(tau_r > 0.0)) return -1;
    medium_t md;
    const double mu0 = cos(cs->sza_deg * PI / 180.0);
    rc = medium_build(&md, op->n_layers, tau_r, aer ? aer->tau_a : 0.0, aer ? aer->ssa_a : 1.0, mu0,
                      op->aer_h_km, op->rayleigh_profile, op->rayleigh_h_km);
    if (!rc && op->gas) rc = medium_apply_gas(&md, op->gas, cs->wavelength_nm, mu0);
    if (rc) { medium_free(&md); return rc; }
    for (int l = 0; l < op->n_layers; ++l)
        if (tau_abs) tau_abs[l] = md.tabs ? md.tabs[l] : 0.0;
    for (int k = 0; k <= op->n_layers; ++k)
        if (z_km) z_km[k] = md.z[k];
    medium_free(&md);
    return 0;
}

/* OpenMP pixel loop (the reference's batch pattern rt_io.c:197-199). */
int ocrt_oracle_solve_batch(int n, const ocrt_case *cases, const ocrt_opts *opts, int opts_per_case,
                            const ocrt_aerosol *aer, int aer_per_case, ocrt_result *out,
                            int n_threads)
{
    if (n < 0 || (n > 0 && (!cases || !opts || !out))) return -1;
    int rc_all = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; ++i) {
        const ocrt_opts *o = opts_per_case ? opts + i : opts;
        const ocrt_aerosol *a = aer ? (aer_per_case ? aer + i : aer) : NULL;
        const int rc = ocrt_oracle_solve_case(cases + i, o, a, out + i, NULL);
        if (rc) {
#pragma omp critical
            rc_all = rc;
        }
    }
    return rc_all;
}

int ocrt_oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* sizeof of every ABI struct, so the ctypes mirror can be checked without a GPU. */
void ocrt_oracle_abi_sizes(size_t *out)
{
    out[0] = sizeof(ocrt_case);
    out[1] = sizeof(ocrt_opts);
    out[2] = sizeof(ocrt_aerosol);
    out[3] = sizeof(ocrt_result);
    out[4] = sizeof(ocrt_diag);
}
#include "ocean.c"
