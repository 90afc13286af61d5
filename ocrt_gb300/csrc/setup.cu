// setup.cu — per-batch and per-wave setup kernels.
//
//   k_gauss          Gauss-Legendre nodes, FP64 Newton       (rt_quadrature.c:20-61)
//   k_pixel_setup    mu0, view slot, Rayleigh depth           (rt_solver.c:618-677)
//   k_levels         h, ch, xdel, ydel, z per level, FP64     (rt_atm.c:177-400)
//   k_coef           linear-source transport weights          (rt_layer_transport.c:36-99)
//   k_basis_gauss    GSF basis at the Gauss nodes per m, FP64 (rt_angular_basis.c:126-276)
//   k_basis_pix      GSF basis at -mu0 and mu_view per task, FP64
//   k_tables         phase tables -> packed source operators  (rt_angular_basis.c:278-357,
//                    rt_sos_operator.c:50-182, rt_primary_source.c:17-198)
//   k_coxmunk        rough-surface Fourier kernels, all m     (shared/surface.c:514-909)
//   k_flat_fresnel   flat-surface diagonal Mueller kernels    (rt_surface_boundary.c:86-103)
#include "kernels.cuh"
#include "physics.cuh"
#include "tables.cuh"

__global__ void k_gauss(int N, double *mu, double *w, float *pw)
{
    const int k = threadIdx.x + 1;               // 1..N (largest root first)
    if (k > N) return;
    const int order = 2 * N;
    double t = cos(OCRT_PI * ((double)k - 0.25) / ((double)order + 0.5));
    double pn = 0, pm = 0, dp = 1;
    for (int it = 0; it < 100; ++it) {
        double a = 1.0, b = t;
        for (int q = 1; q < order; ++q) { const double c = ((2.0 * q + 1.0) * t * b - (double)q * a) / (double)(q + 1); a = b; b = c; }
        pn = b; pm = a;
        dp = (double)order * (t * pn - pm) / (t * t - 1.0);
        const double step = -pn / dp;
        t += step;
        if (fabs(step) < 1.0e-15 * (fabs(t) + 1.0)) break;
    }
    double a = 1.0, b = t;
    for (int q = 1; q < order; ++q) { const double c = ((2.0 * q + 1.0) * t * b - (double)q * a) / (double)(q + 1); a = b; b = c; }
    dp = (double)order * (t * b - a) / (t * t - 1.0);
    mu[N - k] = t;
    w[N - k] = 2.0 / ((1.0 - t * t) * dp * dp);
    // surface-operator weights (2 pi or pi) mu w, rounded once (rt_surface_boundary.c:137-208)
    if (pw) {
        pw[N - k] = (float)(2.0 * OCRT_PI * t * w[N - k]);
        pw[N + N - k] = (float)(OCRT_PI * t * w[N - k]);
    }
}

__global__ void k_pixel_setup(PixDev *px, int P, int N, const double *gmu)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    PixDev &d = px[p];
    if (d.medium == 1) {
        // water column: the host sets mu0 (refracted sun), mu_view (refracted
        // view), the zero-weight slots and the optical depth; no surface below
        d.view_slot = N;
        d.surf_on = d.flat = d.rough = 0;
        return;
    }
    d.mu0 = cos(d.sza_deg * OCRT_PI / 180.0);
    d.mu_view = cos(d.vza_deg * OCRT_PI / 180.0);
    d.xmu[0] = d.mu_view;
    double tr;
    if (!(d.pressure_hpa > 0.0)) tr = 0.0;
    else if (d.tau_r_source == 1) tr = d.tau_r_input;
    else tr = bodhaine_tau(d.wavelength_nm, d.pressure_hpa);
    d.tau_r = tr;
    d.tau_total = tr + (d.mom_off >= 0 ? d.tau_a : 0.0);
    // view node: sorted insertion with de-duplication (rt_angle_grid.c:37-73)
    d.view_slot = -1;
    d.n_ring = N;
    if (d.view_as_node) {
        int lo = 0, hi = N;
        while (lo < hi) { const int mid = (lo + hi) >> 1; if (gmu[mid] < d.mu_view) lo = mid + 1; else hi = mid; }
        if (lo > 0 && fabs(gmu[lo - 1] - d.mu_view) < 1.0e-12) d.view_slot = lo - 1;
        else if (lo < N && fabs(gmu[lo] - d.mu_view) < 1.0e-12) d.view_slot = lo;
        else { d.view_slot = N; d.n_ring = N + 1; }
    }
    const int bfo = d.surface == 2, flat_s = d.surface == 3;
    d.surf_on = bfo || flat_s;
    d.flat = flat_s || (bfo && d.wind <= 0.0);
    d.rough = d.surf_on && !d.flat;
}

// One thread per (pixel, level).  Altitude of each level by 64-step
// bisection on the column above (rt_molecular_profile.c:84-105, rt_atm.c:313-355);
// every level brackets [0, 100 km] independently.
__global__ void k_levels(const PixDev *px, int P, double *h, double *ch, double *xd, double *yd, double *z)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    if (d.medium == 1) return;
    const int nt = d.nt;
    const double tau = d.tau_total, tr = d.tau_r;
    const int aer = d.mom_off >= 0 && d.tau_a > 0.0;
    const double ta = aer ? d.tau_a : 0.0;
    const double ah = d.aer_h_km > 0.0 ? d.aer_h_km : 2.0;
    AboveEval E;
    above_init(E, d.profile, d.ray_h_km, ah);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nt; k += gridDim.x * blockDim.x) {
        const long long o = d.lev_off + k;
        const double hk = (double)k * tau / (double)nt;
        h[o] = hk;
        ch[o] = 0.5 * exp(-hk / d.mu0);
        double zk;
        if (k == 0) zk = OCRT_ZTOP_KM;
        else if (k == nt && aer) zk = 0.0;
        else {
            const double ztop = (!aer && d.profile == 0) ? 84.852 : OCRT_ZTOP_KM;
            const double f = hk / tau;
            if (!aer && f >= 1.0) zk = 0.0;
            else {
                double lo = 0.0, hi = aer ? OCRT_ZTOP_KM : ztop;
                const double target = aer ? hk : f;
                auto above_at = [&](double zz) {
                    return aer ? tr * above_ray(E, zz) + ta * above_exp(zz, ah, E.et_a) : above_ray(E, zz);
                };
                // Illinois steps (regula falsi that halves the value of an end
                // kept twice) narrow the bracket while keeping the bisection's
                // invariant above(lo) > target >= above(hi), until it is ~1e-12
                // wide relative; the bisection below then ends, as a full
                // 64-step bisection from [0, top] does, on the two adjacent
                // doubles around the crossing, in ~26 evaluations of the
                // column fraction instead of ~58.  Where the computed fraction
                // is not monotone in its last bits the two can end a few ulps
                // apart (1.2e-15 relative at most over 60k levels of random
                // profiles, 99.5% identical).
                double flo = above_at(lo) - target, fhi = above_at(hi) - target;
                int side = 0;
                for (int it = 0; it < 40 && hi - lo > 1e-12 * hi; ++it) {
                    double c = hi - fhi * (hi - lo) / (fhi - flo);
                    if (!(c > lo && c < hi)) c = 0.5 * (lo + hi);
                    const double fc = above_at(c) - target;
                    if (fc > 0.0) { lo = c; flo = fc; if (side < 0) fhi *= 0.5; side = -1; }
                    else { hi = c; fhi = fc; if (side > 0) flo *= 0.5; side = 1; }
                }
                // Once the midpoint equals an end, every later step leaves
                // 0.5 (lo + hi) at that midpoint, so the loop can stop there.
                zk = 0.5 * (lo + hi);
                for (int it = 0; it < 64; ++it) {
                    const double mid = 0.5 * (lo + hi);
                    zk = mid;
                    if (mid == lo || mid == hi) break;
                    if (above_at(mid) > target) lo = mid; else hi = mid;
                    zk = 0.5 * (lo + hi);
                }
            }
        }
        z[o] = zk;
        double x = 0.0, y = 1.0;
        if (aer) {
            if (k == 0) { x = tr == 0.0 ? d.ssa_a : 0.0; y = tr == 0.0 ? 0.0 : 1.0; }
        }
        xd[o] = x;
        yd[o] = y;
    }
}

// Levels of a homogeneous water column (build_inwater_atm, rt_water_rt.c:2163-
// 2176): h_k = k tau / nt from the surface down, direct beam exp(-h/mu_sw)/2,
// hydrosol and pure-water scattering fractions constant.
__global__ void k_levels_water(const PixDev *px, int P, double *h, double *ch, double *xd, double *yd, double *z)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    if (d.medium != 1) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= d.nt; k += gridDim.x * blockDim.x) {
        const long long o = d.lev_off + k;
        const double hk = (double)k * d.w_tau / (double)d.nt;
        h[o] = hk;
        ch[o] = 0.5 * exp(-hk / d.mu0);
        xd[o] = d.w_omega_p;
        yd[o] = d.w_omega_w;
        z[o] = 0.0;
    }
}

// Layer scattering fractions once every level altitude is known.
__global__ void k_level_mix(const PixDev *px, int P, const double *z, double *xd, double *yd)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    if (d.medium == 1 || !(d.mom_off >= 0 && d.tau_a > 0.0)) return;
    const double tr = d.tau_r, ta = d.tau_a, ah = d.aer_h_km > 0.0 ? d.aer_h_km : 2.0;
    for (int k = 1 + blockIdx.x * blockDim.x + threadIdx.x; k <= d.nt; k += gridDim.x * blockDim.x) {
        const long long o = d.lev_off + k;
        const double zj = z[o], zp = z[o - 1];
        const double rj = tr * ray_above(zj, d.profile, d.ray_h_km);
        const double aj = ta * exp_above(zj, OCRT_ZTOP_KM, ah);
        const double rp = k == 1 ? 0.0 : tr * ray_above(zp, d.profile, d.ray_h_km);
        const double ap = k == 1 ? 0.0 : ta * exp_above(zp, OCRT_ZTOP_KM, ah);
        const double dr = rj - rp, da = aj - ap, dt = dr + da;
        if (dt > 0.0) { xd[o] = da * d.ssa_a / dt; yd[o] = dr / dt; }
        else { xd[o] = 0.0; yd[o] = tr > 0.0 ? 1.0 : 0.0; }
    }
}

// Transport weights per (pixel, layer, ring slot):
//   I_k = T I_up + Ca J_k + Cb J_up,  G = (1-T)|mu|/dtau - T, Ca = (1-T-G)/2, Cb = G/2
// (the reference's slope/intercept form of rt_layer_transport.c:89-99 expanded,
// which keeps every weight non-negative).  Computed in FP64, stored FP32.
__global__ void k_coef(const PixDev *px, int P, int N, int NR, const double *gmu, const double *h,
                       float *Tc, float *Ca, float *Cb)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int total = d.nt * NR;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int layer = e / NR, g = e - layer * NR;
        const long long o = d.coef_off + e;
        const double am = ring_mu(d, gmu, N, g);
        const double dtau = h[d.lev_off + layer + 1] - h[d.lev_off + layer];
        const double x = dtau / am;
        const double T = exp(-x);
        const double G = -expm1(-x) / x - T;
        Tc[o] = (float)T;
        Ca[o] = (float)(0.5 * (1.0 - T - G));
        Cb[o] = (float)(0.5 * G);
    }
}

// The transport weights regrouped in quads for k_scan4 and k_scan_tma: per
// (layer, quad of ring slots g = 4q..4q+3) the four T, then the four Ca, then
// the four Cb, so that one 16-byte copy brings one weight of four columns and
// one layer is a row of coef_quad_width(NR) floats; slots past NR are zero.
__global__ void k_coef_quads(const PixDev *px, int P, int N, int NR, const float *Tc, const float *Ca, const float *Cb,
                             float *Cq)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int NRq = (NR + 3) & ~3, total = d.nt * NRq;
    const long long qo = coef_quad_off(d.coef_off, N, NR);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int layer = e / NRq, g = e - layer * NRq;
        const long long src = d.coef_off + (long long)layer * NR + g;
        const long long dst = qo + (long long)layer * 3 * NRq + (g >> 2) * 12 + (g & 3);
        const bool in = g < NR;
        Cq[dst] = in ? Tc[src] : 0.f;
        Cq[dst + 4] = in ? Ca[src] : 0.f;
        Cq[dst + 8] = in ? Cb[src] : 0.f;
    }
}

// GSF basis at the Gauss nodes for every mode: B[(m*(L+1) + l)*N + g], 3 arrays.
// Per-layer overrides (ocrt_layers): optical depths replace the uniform level
// grid (prefix sum in FP64, one thread per pixel) and the layer albedos
// rescale the scattering fractions of the layer's bottom level.  Runs after
// k_level_mix, so the mixing fractions stay those of the uniform grid.
__global__ void k_layers_apply(PixDev *px, int P, const double *ldt, const double *lss, double *h, double *ch,
                               double *xd, double *yd, int *err)
{
    const int p = blockIdx.x;
    if (p >= P) return;
    PixDev &d = px[p];
    if (d.lay_off < 0) return;
    const int nt = d.nt;
    double *hh = h + d.lev_off;
    if (d.has_dtau) {
        if (threadIdx.x == 0) {
            double acc = 0.0;
            hh[0] = 0.0;
            for (int l = 0; l < nt; ++l) { acc += ldt[d.lay_off + l]; hh[l + 1] = acc; }
            d.tau_total = acc;
        }
        __syncthreads();
        for (int k = threadIdx.x; k <= nt; k += blockDim.x) ch[d.lev_off + k] = 0.5 * exp(-hh[k] / d.mu0);
    }
    if (d.has_ssa) {
        for (int l = threadIdx.x; l < nt; l += blockDim.x) {
            const long long o = d.lev_off + l + 1;
            const double w = lss[d.lay_off + l], w0 = xd[o] + yd[o];
            if (!(w0 > 0.0)) { atomicExch(err, OCRT_ERR_ARGS); continue; }
            xd[o] *= w / w0;
            yd[o] *= w / w0;
        }
    }
}

// Derivatives of the transport coefficients with respect to the layer optical
// depth, for the adjoint.  With x = dtau/mu: T = e^-x, G = (1-T)/x - T,
// Ca = (1 - T - G)/2, Cb = G/2; dT/dx = -T, dG/dx = T + T/x - (1-T)/x^2 (its
// Taylor series below x = 1e-2, where the closed form cancels), and
// d/ddtau = (1/mu) d/dx.
__global__ void k_coef_deriv(const PixDev *px, int P, int N, const double *gmu, const double *h,
                             float *dTc, float *dCa, float *dCb)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int NR = N + 1;
    const int total = d.nt * NR;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int layer = e / NR, g = e - layer * NR;
        const long long o = d.coef_off + e;
        double am = g < N ? gmu[g] : d.mu_view;
        if (g >= d.n_ring) am = 1.0;
        const double dtau = h[d.lev_off + layer + 1] - h[d.lev_off + layer];
        const double x = dtau / am;
        const double T = exp(-x);
        double Gp;
        if (x < 1e-2)
            Gp = 0.5 + x * (-2.0 / 3.0 + x * (3.0 / 8.0 + x * (-2.0 / 15.0 + x * (5.0 / 144.0 - x / 140.0))));
        else
            Gp = T + T / x + expm1(-x) / (x * x);
        dTc[o] = (float)(-T / am);
        dCa[o] = (float)(0.5 * (T - Gp) / am);
        dCb[o] = (float)(0.5 * Gp / am);
    }
}

__global__ void k_basis_gauss(int N, int M, int L, const double *gmu, float *Bp, float *Br, float *Bt,
                              const double *gcoef)
{
    const int m = blockIdx.x, g = threadIdx.x;
    if (m > M || g >= N) return;
    const size_t base = (size_t)m * (L + 1) * N;
    gsf_recur(L, m, gmu[g], [&](int l, double P, double R, double T) {
        Bp[base + (size_t)l * N + g] = (float)P;
        Br[base + (size_t)l * N + g] = (float)R;
        Bt[base + (size_t)l * N + g] = (float)T;
    }, gcoef ? gcoef + (size_t)m * (L + 1) * 5 : nullptr);
}

// Step coefficients of the GSF recurrences for every (m, l) of a group:
// gcoef[(m * (L + 1) + l) * 5 ..] = gsf_step_coefs(l, m) for max(2, m) <= l < L.
__global__ void k_gsf_coefs(int M, int L, double *gcoef)
{
    const int m = blockIdx.x;
    if (m > M) return;
    const int l0 = m < 2 ? 2 : m;
    for (int l = l0 + threadIdx.x; l < L; l += blockDim.x)
        gsf_step_coefs(l, m, gcoef + ((size_t)m * (L + 1) + l) * 5);
}

// GSF basis at the solar direction (-mu0) and at the E zero-weight slots for
// every task of a wave: Bx[((t*(1+E) + which)*3 + comp)*(L+1) + l], which 0 =
// sun, 1 + e = slot N + e.
__global__ void k_basis_pix(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, int L, int E, float *Bx,
                            const double *gcoef)
{
    const int W = 1 + E, per = blockDim.x / W;
    if ((int)threadIdx.x >= per * W) return;
    const int tl = blockIdx.x * per + threadIdx.x / W;
    const int which = threadIdx.x % W;
    if (tl >= nt_tasks) return;
    const TaskDev tk = tasks[t0 + tl];
    const PixDev &d = px[tk.pix];
    const double x = which == 0 ? -d.mu0 : d.xmu[which - 1];
    float *dst = Bx + ((size_t)tl * W + which) * 3 * (L + 1);
    for (int l = 0; l <= L; ++l) { dst[l] = 0.f; dst[L + 1 + l] = 0.f; dst[2 * (L + 1) + l] = 0.f; }
    gsf_recur(d.L, tk.m, x, [&](int l, double P, double R, double T) {
        dst[l] = (float)P; dst[L + 1 + l] = (float)R; dst[2 * (L + 1) + l] = (float)T;
    }, gcoef ? gcoef + (size_t)tk.m * (L + 1) * 5 : nullptr);
}

// One block per task.  Phase tables by contraction over l in FP32 with the
// even/odd parity split giving the mirrored columns; then the packed aerosol
// operator (and molecular operator for m <= 2), the primary-source vectors and
// the flat-surface reflected-beam vectors.  With sprod (k_tables_tc has run)
// only the second part: the tensor-core kernel wrote the aerosol operator and
// the sun-outgoing products of the Gauss slots.
__global__ void __launch_bounds__(256, 2) k_tables(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, Geom G, int L,
                         const float *Bp, const float *Br, const float *Bt, const float *Bx,
                         const double *gw,
                         const double *mb, const double *mg, const double *ma, const double *mz,
                         float *ops, float *pvec, float *fvec, float *opt, int plain,
                         const float *V, int vp0, long long vstride, const float *sprod)
{
    const int tl = blockIdx.x;
    if (tl >= nt_tasks) return;
    const TaskDev tk = tasks[t0 + tl];
    const PixDev &d = px[tk.pix];
    const int m = tk.m, N = G.N, n = d.n_ring, Lp = d.L;
    const int aer = d.mom_off >= 0 && d.tau_a > 0.0;
    const int La = aer ? d.L_aer : -1;
    const float *bx = Bx + (size_t)tl * (1 + G.E) * 3 * (L + 1);        // [which][comp][l]
    const size_t gb = (size_t)m * (L + 1) * N;
    // basis accessor: slot s in 0..N-1 Gauss, s >= N zero-weight slot, s == -1 solar
    auto basis = [&](int comp, int s, int l) -> float {
        if (s < 0) return bx[(size_t)(0 * 3 + comp) * (L + 1) + l];
        if (s >= N) return bx[(size_t)((1 + s - N) * 3 + comp) * (L + 1) + l];
        const float *B = comp == 0 ? Bp : (comp == 1 ? Br : Bt);
        return B[gb + (size_t)l * N + s];
    };
    // molecular l = 2 basis with mirror parity p(-x) = (-1)^m p(x), t(-x) = -(-1)^m t(x)
    const float par = (m & 1) ? -1.f : 1.f;
    const double A = 2.0 * (1.0 - d.depol) / (2.0 + d.depol);
    const float b0 = m == 0 ? 1.f : 0.f, b2 = (float)(0.5 * A), g2 = (float)(-A * sqrt(1.5)), a2 = (float)(3.0 * A);
    const int mol = m <= 2;
    // aerosol value kernel: the I-I table of this mode from k_value_pfm
    const float *Vm = (V && d.vk_n > 1) ? V + (size_t)(tk.pix - vp0) * vstride + (size_t)m * (N + 1) * 2 * G.NR
                                        : nullptr;
    float *Aop = ops + tk.op_off;
    float *Atile = opt ? opt + 2 * tk.op_off : nullptr;     // tensor-core tiles of the aerosol operator
    float *Bop = tk.mol_off >= 0 ? ops + tk.mol_off : nullptr;
    // aerosol moments in FP32 shared memory (read at every l of every pair)
    extern __shared__ float smom[];                               // [4][Lp + 1]
    for (int l = threadIdx.x; l <= Lp; l += blockDim.x) {
        const bool in = l <= La;
        smom[l] = in ? (float)mb[d.mom_off + l] : 0.f;
        smom[(Lp + 1) + l] = in ? (float)mg[d.mom_off + l] : 0.f;
        smom[2 * (Lp + 1) + l] = in ? (float)ma[d.mom_off + l] : 0.f;
        smom[3 * (Lp + 1) + l] = in ? (float)mz[d.mom_off + l] : 0.f;
    }
    __syncthreads();

    // ---- operator pairs (o ring slot, i Gauss) ----
    // A thread takes the two pairs (o, i) and (o, i + hN), hN = ceil(N / 2), so
    // both share the outgoing factors; block y of the task takes the (o, i)
    // slots [y * blockDim, (y + 1) * blockDim) of n * hN.  Every pair product
    // is (incoming basis) x (outgoing basis x moment); the eight outgoing
    // factors Y_k(o, l) and the incoming bases X_c(i, l) are staged in shared
    // memory TB_LC moments at a time, so a pair costs 13 FMAs per moment.  l
    // starts at m and chunks are even, so the parity of l + m is the parity of
    // the chunk offset.
    float *Ys = smom + 4 * (L + 1);                               // [8][PO][TB_LC]
    const int PO = tables_orows(blockDim.x, N);
    float *Xs = Ys + 8 * PO * TB_LC;                              // [3][TB_LC][N]
    const int hN = (N + 1) / 2;
    const int nslot = n * hN, e0 = blockIdx.y * blockDim.x;
    if (!sprod && e0 < nslot) {
    const int e1 = min(e0 + (int)blockDim.x, nslot);
    const int o_lo = e0 / hN, nor = (e1 - 1) / hN - o_lo + 1;
    const int e = e0 + threadIdx.x;
    const bool mine = e < e1;
    const int o = mine ? e / hN : o_lo, i0 = mine ? e - o * hN : 0, i1 = i0 + hN;
    const bool mine1 = mine && i1 < N;
    const int os = o;    // ring slot (the view node, when inserted, is slot N)
    // Y_k = basis(comp_k) x moment(mom_k), one nibble per k (k = 0 lowest):
    // comp {P, R, T, T, R, T, R, P}, moment {beta, gamma, gamma, zeta, alpha, alpha, zeta, gamma}
    // with moments 0 beta, 1 gamma, 2 alpha, 3 zeta
    constexpr unsigned ycomp = 0x01212210u, ymom = 0x13223110u;
    // accumulators 0..8: [row i, col o] products, 9..12: transposed pair; even
    // (E) / odd (O) in l+m; the second pair's in E1 / O1
    float E[13], O[13], E1[13], O1[13];
#pragma unroll
    for (int q = 0; q < 13; ++q) { E[q] = 0.f; O[q] = 0.f; E1[q] = 0.f; O1[q] = 0.f; }
    const int ia = i0, ib = mine1 ? i1 : i0;
    for (int l0 = m; l0 <= Lp; l0 += TB_LC) {
        __syncthreads();
        // Y: one (outgoing row, moment) per thread, all eight factors
        for (int x = threadIdx.x; x < nor * TB_LC; x += blockDim.x) {
            const int oo = x / TB_LC, lc = x % TB_LC, l = l0 + lc;
            float bc[3] = {0.f, 0.f, 0.f}, mo[4] = {0.f, 0.f, 0.f, 0.f};
            if (l <= Lp) {
#pragma unroll
                for (int c = 0; c < 3; ++c) bc[c] = basis(c, o_lo + oo, l);
#pragma unroll
                for (int q = 0; q < 4; ++q) mo[q] = smom[q * (Lp + 1) + l];
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                Ys[(k * PO + oo) * TB_LC + lc] = bc[(ycomp >> (4 * k)) & 15] * mo[(ymom >> (4 * k)) & 15];
        }
        // X: the Gauss bases of moments l0 .. l0 + TB_LC - 1 are contiguous rows of Bp / Br / Bt
        const int xe = min(TB_LC, Lp + 1 - l0) * N;
        for (int x = threadIdx.x; x < TB_LC * N; x += blockDim.x) {
            const size_t gsrc = gb + (size_t)l0 * N + x;
            const bool in = x < xe;
            Xs[x] = in ? Bp[gsrc] : 0.f;
            Xs[TB_LC * N + x] = in ? Br[gsrc] : 0.f;
            Xs[2 * TB_LC * N + x] = in ? Bt[gsrc] : 0.f;
        }
        __syncthreads();
        if (mine) {
            const float *yb = Ys + (o - o_lo) * TB_LC;
#pragma unroll
            for (int lc = 0; lc < TB_LC; lc += 4) {
                float4 y[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) y[k] = *reinterpret_cast<const float4 *>(yb + k * PO * TB_LC + lc);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    float Y[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) Y[k] = u == 0 ? y[k].x : u == 1 ? y[k].y : u == 2 ? y[k].z : y[k].w;
                    const float *xr = Xs + (lc + u) * N;
                    {
                        const float Pi = xr[ia], Ri = xr[TB_LC * N + ia], Ti = xr[2 * TB_LC * N + ia];
                        float *A = (u & 1) ? O : E;
                        A[0] = fmaf(Pi, Y[0], A[0]);  A[1] = fmaf(Pi, Y[1], A[1]);  A[2] = fmaf(Pi, Y[2], A[2]);
                        A[3] = fmaf(Ti, Y[3], A[3]);  A[4] = fmaf(Ri, Y[4], A[4]);  A[5] = fmaf(Ti, Y[4], A[5]);
                        A[6] = fmaf(Ri, Y[3], A[6]);  A[7] = fmaf(Ti, Y[5], A[7]);  A[8] = fmaf(Ri, Y[6], A[8]);
                        A[9] = fmaf(Ti, Y[7], A[9]);  A[10] = fmaf(Ri, Y[7], A[10]);
                        A[11] = fmaf(Ri, Y[5], A[11]); A[12] = fmaf(Ti, Y[6], A[12]);
                    }
                    {
                        const float Pi = xr[ib], Ri = xr[TB_LC * N + ib], Ti = xr[2 * TB_LC * N + ib];
                        float *A = (u & 1) ? O1 : E1;
                        A[0] = fmaf(Pi, Y[0], A[0]);  A[1] = fmaf(Pi, Y[1], A[1]);  A[2] = fmaf(Pi, Y[2], A[2]);
                        A[3] = fmaf(Ti, Y[3], A[3]);  A[4] = fmaf(Ri, Y[4], A[4]);  A[5] = fmaf(Ti, Y[4], A[5]);
                        A[6] = fmaf(Ri, Y[3], A[6]);  A[7] = fmaf(Ti, Y[5], A[7]);  A[8] = fmaf(Ri, Y[6], A[8]);
                        A[9] = fmaf(Ti, Y[7], A[9]);  A[10] = fmaf(Ri, Y[7], A[10]);
                        A[11] = fmaf(Ri, Y[5], A[11]); A[12] = fmaf(Ti, Y[6], A[12]);
                    }
                }
            }
        }
    }
    // tables: value at +col = S, at -col = sigma * D with sigma from the column basis
    auto emit = [&](const float *Ea, const float *Oa, int i) {
        float S[13], D[13], c[18];
#pragma unroll
        for (int q = 0; q < 13; ++q) { S[q] = Ea[q] + Oa[q]; D[q] = Ea[q] - Oa[q]; }
        pair_coefs(S, D, c);
        if (Vm) {                                           // the value kernel's table instead
            c[0] = Vm[(size_t)(1 + i) * 2 * G.NR + os];
            c[1] = Vm[(size_t)(1 + i) * 2 * G.NR + G.NR + os];
        }
        const float w = (float)gw[i];
        if (plain) put_pair([&](int r, int ci, float v) { Aop[(size_t)r * G.CIN + ci] = v; }, G, os, i, w, c);
        if (Atile) put_pair([&](int r, int ci, float v) { tile_put(Atile, G, r, ci, v); }, G, os, i, w, c);
    };
    if (mine) emit(E, O, i0);
    if (mine1) emit(E1, O1, i1);
    }
    if (blockIdx.y != 0) return;
    // tile rows no pair writes: the rows of unused zero-weight slots (the view
    // when it is a Gauss node), and the padding rows COUT .. NP - 1
    if (Atile && !sprod) {
        const int nz0 = 6 * (G.NR - n), nz = nz0 + (G.NP - G.COUT);
        for (int e = threadIdx.x; e < nz * G.CIN; e += blockDim.x) {
            const int q = e / G.CIN, ci = e - q * G.CIN;
            tile_put(Atile, G, q < nz0 ? 6 * N + 6 * (n - N) + q : G.COUT + (q - nz0), ci, 0.f);
        }
    }
    // ---- molecular operator (m <= 2) in factored form U[c_out][24] ----
    // Every molecular entry is (function of the outgoing direction) x
    // w_i f(mu_i), f in {1, P2m, R2m, T2m}; U holds the outgoing factors for
    // input block b = 2s + h and functional f at column 4b + f.  The sign
    // pattern is that of the pair contraction in rt_sos_operator.c:387-406.
    if (Bop && mol) {
        for (int e = threadIdx.x; e < n * 6; e += blockDim.x) {
            const int o = e / 6, ob = e - o * 6;
            const float po = basis(0, o, 2), ro = basis(1, o, 2), to = basis(2, o, 2);
            const float sr = par, st = -par;                 // r(-x) = sr r(x), t(-x) = st t(x)
            const float pm = par * po, rm = sr * ro, tm = st * to;
            float u[24];
#pragma unroll
            for (int q = 0; q < 24; ++q) u[q] = 0.f;
            // u[4*ib + f], ib = 2*s_in + h_in, f: 0 const, 1 P, 2 R, 3 T
            switch (ob) {
            case 0:   // I up
                u[0] = b0; u[1] = b2 * po; u[8 + 2] = g2 * po; u[16 + 3] = -g2 * po;
                u[4] = b0; u[4 + 1] = b2 * pm; u[12 + 2] = g2 * po * sr; u[20 + 3] = -g2 * po * st;
                break;
            case 1:   // I down
                u[0] = b0; u[1] = b2 * pm; u[8 + 2] = g2 * po * sr; u[16 + 3] = g2 * po * st;
                u[4] = b0; u[4 + 1] = b2 * po; u[12 + 2] = g2 * po; u[20 + 3] = g2 * po;
                break;
            case 2:   // Q up
                u[1] = g2 * ro; u[8 + 2] = a2 * ro; u[16 + 3] = -a2 * ro;
                u[4 + 1] = g2 * rm; u[12 + 2] = a2 * rm; u[20 + 3] = a2 * rm;
                break;
            case 3:   // Q down
                u[1] = g2 * rm; u[8 + 2] = a2 * rm; u[16 + 3] = -a2 * rm;
                u[4 + 1] = g2 * ro; u[12 + 2] = a2 * ro; u[20 + 3] = a2 * ro;
                break;
            case 4:   // U up
                u[1] = -g2 * to; u[8 + 2] = -a2 * to; u[16 + 3] = a2 * to;
                u[4 + 1] = g2 * tm; u[12 + 2] = -a2 * to * sr; u[20 + 3] = a2 * tm;
                break;
            default:  // U down
                u[1] = -g2 * tm; u[8 + 2] = a2 * to * sr; u[16 + 3] = a2 * tm;
                u[4 + 1] = g2 * to; u[12 + 2] = a2 * to; u[20 + 3] = a2 * to;
                break;
            }
            const int c = col_of(G, ob >> 1, ob & 1, o);
#pragma unroll
            for (int q = 0; q < 24; ++q) Bop[(size_t)c * 24 + q] = u[q];
        }
        // rows of unused zero-weight slots (the view when it is a Gauss node; the
        // buffer is not cleared between waves on the tensor-core path)
        for (int e = threadIdx.x; e < 6 * (G.NR - n) * 24; e += blockDim.x)
            Bop[(size_t)(6 * N + 6 * (n - N)) * 24 + e] = 0.f;
    }

    // ---- solar row: primary-source vectors and flat reflected-beam vectors ----
    // pvec[tl][2][LDC]: [0] aerosol part, [1] molecular part of J1 / (ch * fraction)
    float *pv = pvec + (size_t)tl * 2 * G.LDC;
    float *fv = fvec ? fvec + (size_t)tl * 2 * 2 * 6 * G.NR : nullptr;   // [side][aer/mol][6][NR]
    // with sprod, the zero-weight slots' sun-outgoing products are summed by a
    // warp each (lane: l = m + lane + 32 j, whose parity is the lane's), into
    // vprod[e] = {S[8], D[8]}
    __shared__ float vprod[4][16];
    if (sprod) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
        for (int e = warp; e < n - N && e < 4; e += nwarp) {
            const int os = N + e;
            float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int l = m + lane; l <= Lp; l += 32) {
                const float be = smom[l], ga = smom[(Lp + 1) + l];
                const float al = smom[2 * (Lp + 1) + l], ze = smom[3 * (Lp + 1) + l];
                const float P0 = basis(0, -1, l), R0 = basis(1, -1, l), T0 = basis(2, -1, l);
                const float Po = basis(0, os, l), Ro = basis(1, os, l), To = basis(2, os, l);
                a[0] += P0 * Po * be; a[1] += P0 * Ro * ga; a[2] += P0 * To * ga; a[3] += T0 * To * ze;
                a[4] += R0 * Ro * al; a[5] += Po * R0 * ga; a[6] += To * R0 * al; a[7] += Ro * T0 * ze;
            }
            const float sg = (lane & 1) ? -1.f : 1.f;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float sv = a[q], dv = sg * a[q];
#pragma unroll
                for (int k = 16; k >= 1; k >>= 1) {
                    sv += __shfl_xor_sync(0xffffffffu, sv, k);
                    dv += __shfl_xor_sync(0xffffffffu, dv, k);
                }
                if (lane == 0) { vprod[e][q] = sv; vprod[e][8 + q] = dv; }
            }
        }
        __syncthreads();
    }
    for (int o = threadIdx.x; o < n; o += blockDim.x) {
        const int os = o;
        // the eight sun-outgoing products (0 sun incoming): sums over l of
        //   0 P0 Po beta   1 P0 Ro gamma   2 P0 To gamma   3 T0 To zeta
        //   4 R0 Ro alpha  5 R0 Po gamma   6 R0 To alpha   7 T0 Ro zeta
        // S over all l, D with the sign (-1)^(l+m); from k_tables_tc for the
        // Gauss slots when it ran, else summed here
        float S[8], D[8];
        if (sprod) {
            const float *sp = o < N ? sprod + ((size_t)tl * N + o) * 16 : vprod[o - N];
#pragma unroll
            for (int q = 0; q < 8; ++q) { S[q] = sp[q]; D[q] = sp[8 + q]; }
        } else {
            float E[8] = {0}, O[8] = {0};
            for (int l = m; l <= Lp; ++l) {
                const float be = smom[l], ga = smom[(Lp + 1) + l];
                const float al = smom[2 * (Lp + 1) + l], ze = smom[3 * (Lp + 1) + l];
                const float P0 = basis(0, -1, l), R0 = basis(1, -1, l), T0 = basis(2, -1, l);
                const float Po = basis(0, os, l), Ro = basis(1, os, l), To = basis(2, os, l);
                const float v[8] = {P0 * Po * be, P0 * Ro * ga, P0 * To * ga, T0 * To * ze,
                                    R0 * Ro * al, Po * R0 * ga, To * R0 * al, Ro * T0 * ze};
                const bool ev = ((l + m) & 1) == 0;
#pragma unroll
                for (int q = 0; q < 8; ++q) (ev ? E[q] : O[q]) += v[q];
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) { S[q] = E[q] + O[q]; D[q] = E[q] - O[q]; }
        }
        // row 0 (solar) tables at column +o (S) and -o (sigma D)
        const float pfmP = Vm ? Vm[os] : S[0], pfmM = Vm ? Vm[G.NR + os] : D[0];
        const float grP = S[1], grM = D[1];
        const float gtP = S[2], gtM = -D[2];
        const float arrP = S[3] + S[4], arrM = -D[3] + D[4];
        // T_o R_0 alpha (sigma -) + R_o T_0 zeta (sigma +)
        const float quP = S[6] + S[7], quM = -D[6] + D[7];
        // primary source (rt_primary_source.c:59-77, 163-177), U sign folded in
        const float p0 = basis(0, -1, 2);
        const float po = basis(0, os, 2), ro = basis(1, os, 2), to = basis(2, os, 2);
        const float pmo = par * po, rmo = par * ro, tmo = -par * to;
        pv[col_of(G, 0, 0, os)] = pfmP;  pv[col_of(G, 0, 1, os)] = pfmM;
        pv[col_of(G, 1, 0, os)] = grP;   pv[col_of(G, 1, 1, os)] = grM;
        pv[col_of(G, 2, 0, os)] = -gtP;  pv[col_of(G, 2, 1, os)] = -gtM;
        float *pm = pv + G.LDC;
        pm[col_of(G, 0, 0, os)] = b0 + b2 * po * p0;
        pm[col_of(G, 0, 1, os)] = b0 + b2 * pmo * p0;
        pm[col_of(G, 1, 0, os)] = mol ? g2 * ro * p0 : 0.f;
        pm[col_of(G, 1, 1, os)] = mol ? g2 * rmo * p0 : 0.f;
        pm[col_of(G, 2, 0, os)] = mol ? -g2 * to * p0 : 0.f;
        pm[col_of(G, 2, 1, os)] = mol ? -g2 * tmo * p0 : 0.f;
        if (d.beam_q != 0.0) {
            // partially polarised incident beam (1, q, 0): the Q-incident solar
            // column of the phase matrix, aerosol and molecular parts
            // (rt_primary_source.c:31-55, 72-78, 106-148, 173-182)
            const float bq = (float)d.beam_q, r0s = basis(1, -1, 2);
            pv[col_of(G, 0, 0, os)] += bq * S[5];
            pv[col_of(G, 0, 1, os)] += bq * D[5];
            pv[col_of(G, 1, 0, os)] += bq * arrP;
            pv[col_of(G, 1, 1, os)] += bq * arrM;
            pv[col_of(G, 2, 0, os)] += -bq * quP;
            pv[col_of(G, 2, 1, os)] += -bq * quM;
            if (mol) {
                pm[col_of(G, 0, 0, os)] += bq * g2 * po * r0s;
                pm[col_of(G, 0, 1, os)] += bq * g2 * pmo * r0s;
                pm[col_of(G, 1, 0, os)] += bq * a2 * ro * r0s;
                pm[col_of(G, 1, 1, os)] += bq * a2 * rmo * r0s;
                pm[col_of(G, 2, 0, os)] += -bq * a2 * to * r0s;
                pm[col_of(G, 2, 1, os)] += -bq * a2 * tmo * r0s;
            }
        }
        if (fv) {
            // flat-surface reflected beam kernels (rt_surface_boundary.c:246-360):
            // side 0 ("top", upward outputs) uses column -o, side 1 uses +o.
            // comps: P, R, T, RT(transpose gr), RR, TR(transpose art)
            const float r0 = basis(1, -1, 2);
            for (int side = 0; side < 2; ++side) {
                const bool neg = side == 0;
                float *fa = fv + ((size_t)(side * 2 + 0) * 6) * G.NR;
                float *fm = fv + ((size_t)(side * 2 + 1) * 6) * G.NR;
                fa[0 * G.NR + os] = neg ? pfmM : pfmP;
                fa[1 * G.NR + os] = neg ? grM : grP;
                fa[2 * G.NR + os] = neg ? gtM : gtP;
                fa[3 * G.NR + os] = neg ? D[5] : S[5];
                fa[4 * G.NR + os] = neg ? arrM : arrP;
                fa[5 * G.NR + os] = neg ? quM : quP;
                const float pd = neg ? pmo : po, rd = neg ? rmo : ro, td = neg ? tmo : to;
                fm[0 * G.NR + os] = mol ? b0 + b2 * pd * p0 : 0.f;
                fm[1 * G.NR + os] = mol ? g2 * rd * p0 : 0.f;
                fm[2 * G.NR + os] = mol ? g2 * td * p0 : 0.f;
                fm[3 * G.NR + os] = mol ? g2 * r0 * pd : 0.f;
                fm[4 * G.NR + os] = mol ? a2 * r0 * rd : 0.f;
                fm[5 * G.NR + os] = mol ? a2 * td * r0 : 0.f;
            }
        }
    }
}

// Rough-surface Fourier kernels for one (pixel, outgoing slot o, incoming
// slot i) per block, all modes at once.  Incoming slot N is the sun.
// Mueller values on the azimuth grid in FP32 (half grid: the mirror symmetry
// phi -> 2pi - phi flips exactly the sin entries), projection onto cos/sin
// mphi in FP32, normalisation dphi/(2pi or pi) and the m>0 IU/QU sign of
// shared/surface.c:896-906 applied at the end.
#define CM_MG 5

// DW = true additionally writes srfW = dR_m/dW.  Only the slope-distribution
// factor of R depends on the wind: R = brdf * (Fresnel, rotations) with
// brdf ~ exp(-tan^2(beta)/s2) / (pi s2 (1 + lam)), so
//   dR/dW = ds2/dW * R * [ -1/s2 + tan^2(beta)/s2^2 - (dlam/ds2)/(1 + lam) ]
// and dR_m/dW = a R_m + b P_m[R tan^2(beta)] with per-pair constants a, b and
// P_m the same azimuth projection.
// One (pixel p, outgoing slot o, incoming slot i) pair, all modes, by the
// whole block.  tab: cos/sin(m phi_q) rows [(m * 2 + kind) * half + q] of a
// table built for Mtab modes, followed by the cos phi, sin phi, sin^2(phi/2)
// rows; SMT = the table is in shared memory (else read through the read-only
// cache).  sm_R holds R (and R tan^2(beta) when DW) on the half grid.  Ends with
// a block barrier so the caller can reuse sm_R.
// mirror: o and i are both Gauss slots and the pair (i, o) is written here
// too.  Swapping mu_out and mu_in leaves the facet geometry, Fresnel matrix,
// slope density and shadowing unchanged and turns the two rotations into
// each other's transposes, so R(i <- o) = R(o <- i)^T at every azimuth, and
// so for every Fourier coefficient.
template <bool DW, bool SMT>
__device__ __forceinline__ void coxmunk_pair(int p, int o, int i, const TaskDev *tasks, const PixDev &d,
                                             const int *pix_task0, const Geom &G, const double *gmu,
                                             const float *tab, int Mtab, const double *lamv, const double *lamd,
                                             float *srf, float *srfW, float *sm_R, bool mirror)
{
    // Per-pair scalars are formed in FP32 (FP64 issues at a small fraction of
    // the FP32 rate on this part and every thread of the block needs them).
    const int N = G.N;
    const int os = o;
    const float fmo = (float)(os < N ? gmu[os] : d.mu_view);
    const float fmi = (float)(i < N ? gmu[i] : d.mu0);
    const float fs2 = d.sigma_type == 1 ? 0.003f + 0.00512f * fmaxf(0.01f, (float)d.wind)
                                        : fmaxf(0.0731f * 0.0731f * fmaxf(0.f, (float)d.wind), 1e-10f);
    // Sancer shadowing terms, precomputed per (pixel, slot); slot N+1 is the sun
    const double *lp = lamv + (size_t)p * (N + 2);
    const float flam = (float)lp[i < N ? i : N + 1] + (float)lp[os];
    const int nphi = d.nphi, half = nphi / 2, hs = half + 1;
    const float *ptab = tab + (size_t)(Mtab + 1) * 2 * half;       // [cos, sin, sin^2(phi/2)][half]
    auto ld = [&](const float *a) -> float { return SMT ? *a : __ldg(a); };
    const float fnw = (float)d.n_water;
    float *sm_T = sm_R + 9 * hs;
    for (int q = threadIdx.x; q < half; q += blockDim.x) {
        float R[9], tb2 = 0.f;
        coxmunk_R<float>(fmo, fmi, ld(ptab + q), ld(ptab + half + q), ld(ptab + 2 * half + q), fs2, flam, fnw,
                         d.q_conv, R, DW ? &tb2 : nullptr);
#pragma unroll
        for (int e = 0; e < 9; ++e) sm_R[e * hs + q] = R[e];
        if (DW) {
#pragma unroll
            for (int e = 0; e < 9; ++e) sm_T[e * hs + q] = R[e] * tb2;
        }
    }
    float ca = 0.f, cb = 0.f;
    if (DW) {
        const float ds2 = (float)slope_variance_dw(d.wind, d.sigma_type);
        const double *ldv = lamd + (size_t)p * (N + 2);
        const float dlam = (float)ldv[i < N ? i : N + 1] + (float)ldv[os];
        ca = ds2 * (-1.f / fs2 - dlam / (1.f + flam));
        cb = ds2 / (fs2 * fs2);
    }
    __syncthreads();
    // Projection onto cos/sin(m phi).  Work item = (cos or sin entry group,
    // group of CM_MG modes), one warp per item; the 32 lanes stride the
    // azimuth nodes, so every table and Mueller load of a warp is one
    // contiguous run, and each lane keeps a 5 x CM_MG register tile.  The
    // lane partials are summed with shuffles.
    const int M = d.M;
    const int nmg = (M + CM_MG) / CM_MG;
    const int items = 2 * nmg;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int task_first = pix_task0[p];
    // normalisation x2 (half grid) x dphi / (2 pi) for m = 0 and dphi / pi for m > 0, dphi = 2 pi / nphi
    const float scale0 = 2.f / (float)nphi, scale1 = 4.f / (float)nphi;
    const int ecos[5] = {0, 1, 3, 4, 8}, esin[5] = {2, 5, 6, 7, 7};
    constexpr int AT = DW ? 5 : 1;
    for (int item = warp; item < items; item += nwarp) {
        const int kind = item & 1, mg = item >> 1;  // kind 0: cos entries, 1: sin entries
        const int ne = kind == 0 ? 5 : 4;
        float acc[5][CM_MG], acct[AT][CM_MG];
#pragma unroll
        for (int a = 0; a < 5; ++a)
#pragma unroll
            for (int b = 0; b < CM_MG; ++b) acc[a][b] = 0.f;
#pragma unroll
        for (int a = 0; a < AT; ++a)
#pragma unroll
            for (int b = 0; b < CM_MG; ++b) acct[a][b] = 0.f;
        const float *tb[CM_MG];
#pragma unroll
        for (int b = 0; b < CM_MG; ++b) {
            const int m = min(CM_MG * mg + b, M);
            tb[b] = tab + ((size_t)m * 2 + kind) * half;
        }
        int ro[5];
#pragma unroll
        for (int a = 0; a < 5; ++a) ro[a] = (kind == 0 ? ecos[a] : esin[a]) * hs;
        for (int q = lane; q < half; q += 32) {
            float tv[CM_MG], rv[5];
#pragma unroll
            for (int b = 0; b < CM_MG; ++b) tv[b] = ld(tb[b] + q);
#pragma unroll
            for (int a = 0; a < 5; ++a) rv[a] = sm_R[ro[a] + q];
#pragma unroll
            for (int a = 0; a < 5; ++a)
#pragma unroll
                for (int b = 0; b < CM_MG; ++b) acc[a][b] = fmaf(rv[a], tv[b], acc[a][b]);
            if (DW) {
#pragma unroll
                for (int a = 0; a < AT; ++a) rv[a] = sm_T[ro[a] + q];
#pragma unroll
                for (int a = 0; a < AT; ++a)
#pragma unroll
                    for (int b = 0; b < CM_MG; ++b) acct[a][b] = fmaf(rv[a], tv[b], acct[a][b]);
            }
        }
#pragma unroll
        for (int a = 0; a < 5; ++a)
#pragma unroll
            for (int b = 0; b < CM_MG; ++b)
#pragma unroll
                for (int o2 = 16; o2 > 0; o2 >>= 1) acc[a][b] += __shfl_xor_sync(0xffffffffu, acc[a][b], o2);
#pragma unroll
        for (int a = 0; a < AT; ++a)
#pragma unroll
            for (int b = 0; b < CM_MG; ++b)
#pragma unroll
                for (int o2 = 16; o2 > 0; o2 >>= 1) acct[a][b] += __shfl_xor_sync(0xffffffffu, acct[a][b], o2);
        // lane (a * CM_MG + b) stores entry a of mode CM_MG * mg + b
#pragma unroll
        for (int a = 0; a < 5; ++a)
#pragma unroll
            for (int b = 0; b < CM_MG; ++b) {
                const int m = CM_MG * mg + b;
                if (lane != a * CM_MG + b || a >= ne || m > M) continue;
                const int e = kind == 0 ? ecos[a] : esin[a];
                float sc = m == 0 ? scale0 : scale1;
                if (m > 0 && (e == 2 || e == 5)) sc = -sc;
                const TaskDev &tk = tasks[task_first + m];
                const size_t off = i < N ? ((size_t)os * N + i) * 9 + e : (size_t)G.NR * N * 9 + (size_t)os * 9 + e;
                srf[tk.srf_off + off] = acc[a][b] * sc;
                if (DW) srfW[tk.srf_off + off] = (ca * acc[a][b] + cb * acct[AT == 5 ? a : 0][b]) * sc;
                if (mirror) {
                    // entry (r, c) of the pair is entry (c, r) of the reciprocal pair
                    const int et = (e % 3) * 3 + e / 3;
                    float st = m == 0 ? scale0 : scale1;
                    if (m > 0 && (et == 2 || et == 5)) st = -st;
                    const size_t offt = ((size_t)i * N + os) * 9 + et;
                    srf[tk.srf_off + offt] = acc[a][b] * st;
                    if (DW) srfW[tk.srf_off + offt] = (ca * acc[a][b] + cb * acct[AT == 5 ? a : 0][b]) * st;
                }
            }
    }
    __syncthreads();
}

// Grid (N + 1 incoming, NR outgoing, pixels): one pair per block, table in global memory.
__global__ void k_coxmunk(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                          const double *gmu, const float *cs_tab, int Mtab, const double *lamv, float *srf)
{
    extern __shared__ float sm_R[];
    const int p = p0 + blockIdx.z;
    const PixDev &d = px[p];
    if (!d.rough || (int)blockIdx.y >= d.n_ring) return;
    const int o = blockIdx.y, i = blockIdx.x;
    if (o < G.N && i < G.N && o > i) return;      // written by the reciprocal block (i, o)
    coxmunk_pair<false, false>(p, o, i, tasks, d, pix_task0, G, gmu, cs_tab, Mtab, lamv, nullptr, srf, nullptr, sm_R,
                               o < G.N && i < G.N && o < i);
}

__global__ void k_coxmunk_dw(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                             const double *gmu, const float *cs_tab, int Mtab, const double *lamv,
                             const double *lamd, float *srf, float *srfW)
{
    extern __shared__ float sm_R[];
    const int p = p0 + blockIdx.z;
    const PixDev &d = px[p];
    if (!d.rough || (int)blockIdx.y >= d.n_ring) return;
    const int o = blockIdx.y, i = blockIdx.x;
    if (o < G.N && i < G.N && o > i) return;      // written by the reciprocal block (i, o)
    coxmunk_pair<true, false>(p, o, i, tasks, d, pix_task0, G, gmu, cs_tab, Mtab, lamv, lamd, srf, srfW, sm_R,
                              o < G.N && i < G.N && o < i);
}

// cos / sin(m phi_q) on the half azimuth grid for m = 0..M, followed by the
// rows cos(phi), sin(phi), sin^2(phi/2) used by the Mueller evaluation; all
// evaluated in FP64 (grid launch: M + 2 blocks).
__global__ void k_cs_table(int M, int nphi, float *cs)
{
    const int half = nphi / 2;
    const int m = blockIdx.x;
    const double dphi = 2.0 * OCRT_PI / (double)nphi;
    for (int q = threadIdx.x; q < half; q += blockDim.x) {
        const double phi = (q + 0.5) * dphi;
        if (m <= M) {
            cs[((size_t)m * 2 + 0) * half + q] = (float)cos(m * phi);
            cs[((size_t)m * 2 + 1) * half + q] = (float)sin(m * phi);
        } else {
            float *pt = cs + (size_t)(M + 1) * 2 * half;
            const double sh = sin(0.5 * phi);
            pt[q] = (float)cos(phi);
            pt[half + q] = (float)sin(phi);
            pt[2 * half + q] = (float)(sh * sh);
        }
    }
}

// Sancer shadowing term lambda(mu) (shared/surface.c:578-598) of every ring
// slot and of the sun, once per rough pixel: lam[p*(N+2) + slot], slot N+1 = sun.
__global__ void k_sancer(const PixDev *px, int P, int N, const double *gmu, double *lam, double *lamd)
{
    const int p = blockIdx.x, s = threadIdx.x;
    if (p >= P || s > N + 1) return;
    const PixDev &d = px[p];
    if (!d.rough) return;
    const double mu = s < N ? gmu[s] : (s == N ? d.mu_view : d.mu0);
    const double slen = sqrt(slope_variance(d.wind, d.sigma_type));
    lam[(size_t)p * (N + 2) + s] = sancer_lambda(mu, slen);
    if (lamd) lamd[(size_t)p * (N + 2) + s] = sancer_lambda_ds2(mu, slen);
}

// Direct-beam attenuation from the surface to level k along slot g,
// exp(-(tau - h_k)/mu_g), FP64, once per pixel (shared by every mode):
// E[lev_off*NR + k*NR + g].
__global__ void k_seed_att(const PixDev *px, int P, int N, const double *gmu, const double *h, float *E)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    if (!d.rough) return;
    const int NR = N + 1, total = (d.nt + 1) * NR;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int k = e / NR, g = e - k * NR;
        double am = g < N ? gmu[g] : d.mu_view;
        if (g >= d.n_ring) am = 1.0;
        E[d.lev_off * NR + e] = (float)exp(-(d.tau_total - h[d.lev_off + k]) / am);
    }
}

// FP32 copies of the per-level scattering fractions and direct beam, read at
// every (level, column) by the order-loop kernels.
__global__ void k_level_float(const PixDev *px, int P, const double *xd, const double *yd, const double *ch, float *lvf)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= d.nt; k += gridDim.x * blockDim.x) {
        const long long o = d.lev_off + k;
        lvf[3 * o + 0] = (float)xd[o];
        lvf[3 * o + 1] = (float)yd[o];
        lvf[3 * o + 2] = (float)ch[o];
    }
}

// Flat Fresnel Mueller per ring slot of every pixel: frs[(p*NR + slot)*9].
__global__ void k_flat_fresnel(const PixDev *px, int P, int N, const double *gmu, float *frs)
{
    const int p = blockIdx.x, s = threadIdx.x;
    if (p >= P || s > N) return;
    const PixDev &d = px[p];
    if (!d.flat || s >= d.n_ring) return;
    const int os = s;
    const double mu = os < N ? gmu[os] : d.mu_view;
    double M[9];
    fresnel_R<double>(mu, d.n_water, d.q_conv, M);
    for (int e = 0; e < 9; ++e) frs[((size_t)p * (N + 1) + os) * 9 + e] = (float)M[e];
}

size_t coxmunk_smem_bytes(int nphi, bool dw)
{
    return sizeof(float) * 9 * (size_t)(nphi / 2 + 1) * (dw ? 2 : 1);
}
