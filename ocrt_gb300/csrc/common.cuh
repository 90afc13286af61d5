// common.cuh — device data model shared by the GB300 SOS kernels.
//
// Work decomposition: a batch holds P pixels that share the Gauss order N.
// Every (pixel, Fourier mode m) pair is an independent SOS problem ("task").
// Tasks are processed in waves sized to the workspace; a wave is a contiguous
// pixel range, so all setup that is per pixel-and-mode is built per wave.
//
// Direction ring of a pixel (internal order, not the reference's sorted
// order): slots 0..N-1 are the Gauss nodes in ascending mu, slots N..N+E-1
// zero-weight directions (rt_angle_grid.c:37-73): in the atmosphere E = 1, the
// view node when one is inserted; in the water column E = 4, the refracted
// view, nadir, refracted sun and air-side sun directions (rt_water_rt.c:5236-
// 5298).  NR = N + E is the padded ring width.  Field columns:
//     Gauss slot g < N:        c = s * 2N + h * N + g
//     zero-weight slot g >= N: c = 6N + 6(g - N) + 2s + h
// (s in {I,Q,U}, h = 0 up / 1 down), so the weighted inputs of the source
// contraction are exactly columns [0, 6N) -- six 16-byte aligned blocks of N --
// and the zero-weight columns follow.  Field rows are levels k = 0 (TOA) .. nt.
// Source operators are stored output-major, Aop[c_out][c_in] with c_in in
// [0, 6N) contiguous and NP >= 6N + 6 output rows (multiple of 16).
#pragma once
#include <cstdint>
#include <cstring>

#define OCRT_PI 3.14159265358979323846
#define OCRT_MAX_N 64
#define OCRT_MAX_M 255
#define OCRT_DEPOL 0.0279
#define OCRT_ZTOP_KM 100.0
#define OCRT_DEPOL_WATER 0.039   // pure seawater (rt_water_rt.c:2121)
#define OCRT_MAX_EXTRA 4        // zero-weight ring slots

struct GasDev;

struct PixDev {
    // ---- inputs (host) ----
    double sza_deg, vza_deg, raa_deg, wavelength_nm;
    double pressure_hpa, tau_r_input;
    double tau_a, ssa_a, aer_h_km, ray_h_km;
    double n_water, wind;
    double tol;
    int surface, sigma_type, q_conv, decouple;
    int nt, M, L, L_aer, max_orders;
    int tau_r_source, profile, pssa, view_as_node, nphi;
    int mom_off;            // offset into the moment arrays, -1 without aerosol
    int task0;              // first task of this pixel
    long long lev_off;      // offset of level arrays (nt+1 entries)
    long long coef_off;     // offset of transport coefficients (nt * NR entries)
    long long lay_off;      // offset of the per-layer override arrays (nt entries), -1 = none
    int has_dtau, has_ssa;  // which overrides are present
    int lut_nv, lut_nr;     // angle-grid LUT size (0 = no LUT)
    long long lut_vo, lut_ro, lut_oo;   // offsets of the grid vza, grid raa and the LUT outputs
    const GasDev *gas;      // device gas tables, nullptr = no gas absorption
    // ---- coupled atmosphere-ocean (ocrt_gb_solve_ocean) ----
    int medium;             // 0 atmosphere, 1 water column (top boundary = internal reflection)
    int bottom_only;        // atmosphere driven only by ext_bottom (no solar primary, no seeds)
    long long ext_off;      // offset of this pixel's [M+1][NR][3] ext_bottom (atmosphere) or
                            // skylight top source (water, [M+1][N][3]) in BatchBufs::ext; -1 = none
    int ext_mmax;           // last mode the boundary source holds
    double depol;           // molecular depolarisation: 0.0279 air, 0.039 water
    double beam_q;          // incident-beam polarisation Q/I (water: Fresnel transmission)
    double xmu[OCRT_MAX_EXTRA];   // cosines of the zero-weight slots N.. (water: set by the host)
    double w_tau, w_omega_w, w_omega_p;   // water: optical depth, pure-water and hydrosol albedo
    // ---- aerosol value kernel (rt_solver.c:188-235): tabulated P11, ascending angle ----
    int vk_n;               // table entries; 0 = the I-I aerosol table from the moments
    long long vk_off;       // offset of the table in the group's angle / P11 arrays
    // ---- derived on device (k_pixel_setup) ----
    double mu0, mu_view, tau_r, tau_total;
    int n_ring, view_slot;  // view_slot: ring slot holding mu_view, -1 = interpolate
    int flat, rough, surf_on;
    int pad_;
};

struct TaskDev {
    int pix, m, K, has_mol;
    long long fld_off;      // wave-relative offset of F/J/Tot (K * LDC entries)
    long long op_off;       // wave-relative offset of the aerosol operator (NP * CIN)
    long long mol_off;      // wave-relative offset of the molecular operator factor U [COUT][24], -1 if none
    long long uv_off;       // wave-relative offset of the dense molecular operator U V [NP][CIN], -1 if none
    long long srf_off;      // wave-relative offset of the surface kernels (NR*N*9 + NR*9), -1 if none
    long long tail_off;     // wave-relative offset of the total's tails at the TOA and BOA (2 * LDC entries)
};

// Per-task mutable SOS state.
struct TaskState {
    int active, orders, converged, pad_;
    double resid;
};

// Per-task extracted outputs (TOA view up, BOA down) for the finaliser.
struct TaskOut {
    double vI, vQ, vU;      // TOA upwelling at mu_view (seed removed)
    double dn_view;         // BOA diffuse downward I at mu_view
    double fdn;             // sum_g mu_g w_g I_dn(BOA, g): hemispheric diffuse flux / 2pi
};

struct Geom {
    int N, E, NR, LDC;      // E zero-weight slots, NR = N + E; LDC: field row stride (floats, multiple of 32)
    int CIN;                // 6N weighted input columns (operator row stride)
    int COUT;               // 6N + 6E output columns
    int NP;                 // operator rows, COUT rounded up to 16
    // 1: the order totals are kept at every level (the adjoint reads them,
    // the coupled ocean reads level 1); 0: only at the TOA and BOA output
    // levels, the interior ones neither read nor written
    int tot_all;
};

__host__ __device__ inline Geom make_geom(int N, int E = 1)
{
    Geom g;
    g.N = N;
    g.E = E;
    g.NR = N + E;
    g.CIN = 6 * N;
    g.COUT = 6 * N + 6 * E;
    // field rows start on 128-byte lines: the scan and the source contraction
    // read rows in runs of 32 columns, and a run that straddles two lines
    // costs DRAM two lines
    g.LDC = (g.COUT + 31) & ~31;
    g.NP = (g.COUT + 15) & ~15;
    g.tot_all = 1;
    return g;
}

__host__ __device__ inline int col_of(const Geom &g, int s, int h, int slot)
{
    return slot < g.N ? s * 2 * g.N + h * g.N + slot : 6 * g.N + 6 * (slot - g.N) + 2 * s + h;
}

// Field column -> (Stokes s, hemisphere h, ring slot g); columns past the
// zero-weight block decode to slot NR (never a valid ring slot).
__host__ __device__ inline void decode_col(const Geom &G, int c, int &s, int &h, int &g)
{
    const int N = G.N;
    if (c < 6 * N) {
        s = c / (2 * N);
        const int r = c - s * 2 * N;
        h = r / N;
        g = r - h * N;
    } else if (c < G.COUT) {
        const int v = c - 6 * N, e = v / 6, r = v - 6 * e;
        s = r >> 1; h = r & 1; g = N + e;
    } else {
        s = 0; h = 0; g = G.NR;
    }
}

// Cosine of ring slot g (Gauss node or zero-weight direction); slots past the
// pixel's ring get 1 so that every coefficient stays finite.
__host__ __device__ inline double ring_mu(const PixDev &d, const double *gmu, int N, int g)
{
    if (g >= d.n_ring) return 1.0;
    return g < N ? gmu[g] : d.xmu[g - N];
}

// Input column (weighted Gauss direction) -> field column: the identity.
__host__ __device__ inline int in_to_col(const Geom &g, int cin)
{
    (void)g;
    return cin;
}

// Order totals are kept as unevaluated FP32 pairs (hi + lo, ~48-bit
// significand): FP64 issues at a small fraction of the FP32 rate on this part,
// and the totals are touched at every order, level and column.
// df_add(a, b) = a + b with TwoSum on the heads and the tails folded in.
__host__ __device__ inline float2 df_add(float2 a, float b)
{
    const float s = a.x + b;
    const float bp = s - a.x;
    const float e = (a.x - (s - bp)) + (b - bp);
    const float t = e + a.y;
    const float hi = s + t;
    return make_float2(hi, t - (hi - s));
}

__host__ __device__ inline double df_value(float2 a) { return (double)a.x + (double)a.y; }

// tf32 rounding (to nearest, ties away from zero) of an FP32 value: the
// tensor-core contraction splits each operand into hi = RN_tf32(v) and
// lo = RN_tf32(v - hi), so each part is exact as an MMA operand and hi + lo
// carries v to ~2^-22 relative.
__host__ __device__ inline float round_tf32f(float v)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
#else
    unsigned u; memcpy(&u, &v, 4); u = (u + 0x1000u) & 0xFFFFE000u; float r; memcpy(&r, &u, 4); return r;
#endif
}

// Operator entry (row, cin) into the pre-split tensor-core tiles of one
// operator: per 32-column K tile kt, a tf32 hi tile then a lo tile of NP rows
// x 128 bytes in the SWIZZLE_128B K-major layout the MMA reads (16-byte chunk
// j of row r at chunk position j ^ (r % 8)), so a tile is one bulk copy.
__device__ inline void tile_put_rows(float *T, int nrows, int row, int col, float v)
{
    const int kt = col >> 5, kc = col & 31;
    float *hi = T + (size_t)kt * 2 * nrows * 32;
    const int off = row * 32 + (((kc >> 2) ^ (row & 7)) << 2) + (kc & 3);
    const float h = round_tf32f(v);
    hi[off] = h;
    hi[(size_t)nrows * 32 + off] = round_tf32f(v - h);
}
// forward operators: NP rows (outputs), K = CIN
__device__ inline void tile_put(float *T, const Geom &G, int row, int cin, float v)
{
    tile_put_rows(T, G.NP, row, cin, v);
}

#ifdef __CUDACC__
// Per-thread asynchronous global -> shared copies (cp.async, cached in L1).
__device__ inline void cp_async4(float *dst_smem, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ inline void cp_async8(float2 *dst_smem, const float2 *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ inline void cp_async16_cg(float4 *dst_smem, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ inline void cp_async16_ca(float4 *dst_smem, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
#endif

