// lut.cu — angle-grid LUT mode (rt_solve_case_pol_lut, rt_solver.c:870-900,
// 1025-1045, 1276-1424): one SOS per case, then the TOA reflectance at every
// (vza, raa) of a grid.
//
//   k_lut_sample  per task (pixel, Fourier mode), after its orders: the TOA
//                 upwelling total at every grid vza by monotone cubic (PCHIP)
//                 interpolation over the ring nodes in ascending mu, and the
//                 BOA downward I by linear interpolation (FP64)
//   k_lut_final   per (pixel, grid point): Fourier sums over the modes,
//                 rho = X / mu0, IPSS kappa of the direction, the direct
//                 sunglint (rough ocean) and the directional transmittances
#include "kernels.cuh"
#include "physics.cuh"

namespace {

// Fritsch-Carlson slopes in the weighted-harmonic (interior) and three-point
// one-sided (edge, with the monotonicity clamp) forms.
__device__ inline double slope_interior(double h0, double h1, double s0, double s1)
{
    if (s0 == 0.0 || s1 == 0.0 || (s0 > 0.0) != (s1 > 0.0)) return 0.0;
    const double w1 = 2.0 * h1 + h0, w2 = h1 + 2.0 * h0;
    return (w1 + w2) / (w1 / s0 + w2 / s1);
}

__device__ inline double slope_edge(double h0, double h1, double s0, double s1)
{
    double d = ((2.0 * h0 + h1) * s0 - h0 * s1) / (h0 + h1);
    if (d == 0.0 || s0 == 0.0 || (d > 0.0) != (s0 > 0.0)) {
        if (s0 == 0.0 || (d > 0.0) != (s0 > 0.0)) d = 0.0;
    } else if (((s0 > 0.0) != (s1 > 0.0)) && fabs(d) > 3.0 * fabs(s0)) {
        d = 3.0 * s0;
    }
    return d;
}

__device__ inline double lin_sample(const double *x, const double *y, int n, double mu)
{
    int jh = 1;
    while (jh < n && x[jh - 1] < mu) jh++;
    int jl = jh - 1;
    if (jl < 1) { jl = 1; jh = 2; }
    if (jh > n) { jh = n; jl = n - 1; }
    const double t = (mu - x[jl - 1]) / (x[jh - 1] - x[jl - 1]);
    return (1.0 - t) * y[jl - 1] + t * y[jh - 1];
}

__device__ inline double pchip_sample(const double *x, const double *y, int n, double mu)
{
    int jh = 1;
    while (jh < n && x[jh - 1] < mu) jh++;
    const int jl = jh - 1;
    if (jl < 1 || jh > n || n < 4) return lin_sample(x, y, n, mu);
    const double x1 = x[jl - 1], x2 = x[jh - 1], y1 = y[jl - 1], y2 = y[jh - 1];
    const double h = x2 - x1, sl = (y2 - y1) / h;
    double d1, d2;
    if (jl == 1) {
        const double x3 = x[jh], s2 = (y[jh] - y2) / (x3 - x2);
        d1 = slope_edge(h, x3 - x2, sl, s2);
        d2 = slope_interior(h, x3 - x2, sl, s2);
    } else if (jh == n) {
        const double x0 = x[jl - 2], s0 = (y1 - y[jl - 2]) / (x1 - x0);
        d1 = slope_interior(x1 - x0, h, s0, sl);
        d2 = slope_edge(h, x1 - x0, sl, s0);
    } else {
        const double x0 = x[jl - 2], x3 = x[jh];
        const double s0 = (y1 - y[jl - 2]) / (x1 - x0), s2 = (y[jh] - y2) / (x3 - x2);
        d1 = slope_interior(x1 - x0, h, s0, sl);
        d2 = slope_interior(h, x3 - x2, sl, s2);
    }
    const double t = (mu - x1) / h, t2 = t * t, t3 = t2 * t;
    return (2.0 * t3 - 3.0 * t2 + 1.0) * y1 + (t3 - 2.0 * t2 + t) * h * d1 + (-2.0 * t3 + 3.0 * t2) * y2 +
           (t3 - t2) * h * d2;
}

} // namespace

__global__ void k_lut_sample(BatchBufs B, WaveBufs W, LutBufs Lb, Geom G, int t0, int nw)
{
    const int tl = blockIdx.x;
    if (tl >= nw) return;
    const int tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    if (d.lut_nv <= 0) return;
    const int N = G.N, n = d.n_ring;
    __shared__ double xr[OCRT_MAX_N + 1], yr[4][OCRT_MAX_N + 1];
    // ring in ascending mu: the Gauss nodes with the view node inserted at its place
    int vpos = -1;
    if (d.view_slot == N) {
        vpos = 0;
        while (vpos < N && B.gmu[vpos] < d.mu_view) ++vpos;
    }
    const float fs_tdn = d.rough ? (float)((tk.m == 0 ? OCRT_PI : 0.5 * OCRT_PI) * d.mu0 *
                                           exp(-d.tau_total / d.mu0)) : 0.f;
    const float *Rs = d.rough ? W.srf + tk.srf_off + (size_t)G.NR * G.N * 9 : nullptr;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        int slot;
        if (vpos < 0) slot = j;
        else slot = j < vpos ? j : (j == vpos ? N : j - 1);
        xr[j] = slot < N ? B.gmu[slot] : d.mu_view;
        for (int s = 0; s < 3; ++s) {
            double v = tot_value(W, tk, G, 0, d.nt, col_of(G, s, 0, slot));
            if (d.rough) v -= (double)(fs_tdn * B.Eatt[d.lev_off * G.NR + slot] * Rs[slot * 9 + s * 3]);
            yr[s][j] = v;
        }
        yr[3][j] = tot_value(W, tk, G, d.nt, d.nt, col_of(G, 0, 1, slot));
    }
    __syncthreads();
    for (int iv = threadIdx.x; iv < d.lut_nv; iv += blockDim.x) {
        const double mug = cos(Lb.vza[d.lut_vo + iv] * OCRT_PI / 180.0);
        double *o = Lb.samp + ((size_t)tg * Lb.nvmax + iv) * 4;
        for (int s = 0; s < 3; ++s) o[s] = pchip_sample(xr, yr[s], n, mug);
        o[3] = lin_sample(xr, yr[3], n, mug);
    }
}

__global__ void k_lut_final(const PixDev *px, int P, LutBufs Lb, const int *pix_task0)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int npts = d.lut_nv * d.lut_nr;
    const int M = d.M;
    const double mu0 = d.mu0, tau = d.tau_total;
    const double td = d.pssa ? Lb.tau_dir[p] : -1.0;
    const double cglint = td >= 0.0 ? exp(-(td - tau / mu0)) : 1.0;
    for (int pt = blockIdx.x * blockDim.x + threadIdx.x; pt < npts; pt += gridDim.x * blockDim.x) {
        const int iv = pt / d.lut_nr, ir = pt - iv * d.lut_nr;
        const double vza = Lb.vza[d.lut_vo + iv], raa = Lb.raa[d.lut_ro + ir];
        const double mug = cos(vza * OCRT_PI / 180.0);
        const double phi = raa * OCRT_PI / 180.0 + OCRT_PI;
        double I = 0.0, Q = 0.0, U = 0.0, Dn = 0.0;
        for (int m = 0; m <= M; ++m) {
            const double *s = Lb.samp + ((size_t)(pix_task0[p] + m) * Lb.nvmax + iv) * 4;
            const double cm = m == 0 ? 1.0 : 2.0 * cos((double)m * phi);
            const double sm = m == 0 ? 0.0 : 2.0 * sin((double)m * phi);
            I += cm * s[0]; Q += cm * s[1]; U += sm * s[2]; Dn += cm * s[3];
        }
        double rI = I / mu0, rQ = Q / mu0, rU = U / mu0;
        if (d.pssa) {
            const double kg = Lb.kappa[d.lut_oo + pt];
            rI *= kg; rQ *= kg; rU *= kg;
        }
        double sgI = 0.0;
        if (d.surface == 2 && d.wind > 0.0) {
            const double phv = (raa - 180.0) * OCRT_PI / 180.0;
            const double mvu = vza > 0.0 ? mug : 1.0;
            double g[3];
            sunglint(d, mvu, phv, tau, g);
            g[0] *= cglint; g[1] *= cglint; g[2] *= cglint;
            if (!d.decouple) { rI += g[0]; rQ += g[1]; rU += -g[2]; }
            sgI = g[0];
        }
        const long long o = d.lut_oo + pt;
        Lb.out[0 * Lb.ntot + o] = rI;
        Lb.out[1 * Lb.ntot + o] = rQ;
        Lb.out[2 * Lb.ntot + o] = rU;
        Lb.out[3 * Lb.ntot + o] = 2.0 * OCRT_PI * mug * Dn / (OCRT_PI * mu0);
        Lb.out[4 * Lb.ntot + o] = sgI * mu0;
        Lb.out[5 * Lb.ntot + o] = rI * mu0;
    }
}
