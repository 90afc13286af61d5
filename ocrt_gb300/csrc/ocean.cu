// ocean.cu — device kernels of the coupled atmosphere-ocean solve
// (rt_solve_case_ocean, rt_solver.c:3468-6660).
//
//   k_edges         per task and ring slot: the order totals at the top (k = 0,
//                   upward and downward), at level 1 and at the bottom (k = nt,
//                   downward), double-float where the solve keeps them so
//   k_rww           water-side internal reflection Fourier kernels of the water
//                   column's top boundary (shared/surface.c:1136-1238, 1386-1449)
//   k_taw_direct    slope-integrated air->water irradiance transmittance of the
//                   sun and of every atmosphere ring direction (surface.c:144-179)
//   k_couple_aw     skylight transmitted into the water: the air->water Fourier
//                   kernels on 128 azimuths contracted with the atmosphere's
//                   bottom field (rt_air_water_coupling.c:244-311, surface.c:1476-1720)
//   k_couple_wa     water-leaving radiance on the atmosphere ring and at the view:
//                   the water->air Fourier kernels on a composite water-mu grid
//                   contracted with the upwelling field at the surface
//                   (rt_air_water_coupling.c:598-737, surface.c:648-764, 1731-1811)
//   k_ocean_final   TOA, water-leaving and in-water outputs of each pixel
//                   (rt_solver.c:6314-6647, rt_water_rt.c:6263-7558)
//
// The interface operators are evaluated in FP32 on the CUDA cores (their
// Mueller entries are FP32 expressions of the geometry; the tilt of a facet is
// formed from its normal's components, free of the 1 - cos^2 cancellation);
// quadrature sums over many terms accumulate in FP64.
#include "kernels.cuh"
#include "physics.cuh"

namespace {

__device__ __forceinline__ float sancer_f(float mu, float slen)
{
    if (!(mu < 1.f - 1e-7f)) return 0.f;
    const float s = sqrtf(fmaxf(1e-20f, 1.f - mu * mu));
    const float nu = (mu / s) / slen;
    if (nu > 20.f) return 0.f;
    return 0.5f * (expf(-nu * nu) / (nu * 1.7724538509f) - erfcf(nu));
}

// Stokes rotation pair between the meridian planes of incoming (cosine ma,
// sine sa) and outgoing (mb, sb) propagation directions with scattering
// cosine cT, including the pole limits (shared/surface.c:547-572).
__device__ __forceinline__ void rot_pair_f(float ma, float sa, float mb, float sb, float cT, float cphi, float sphi,
                                           float &c1, float &s1, float &c2, float &s2)
{
    const float den = fmaxf(1e-12f, sqrtf(fmaxf(0.f, 1.f - cT * cT)));
    const float pole = 1e-8f;
    if (sa <= pole) { c1 = -copysignf(1.f, ma) * cphi; s1 = sphi; }
    else {
        c1 = (mb - ma * cT) / (den * fmaxf(1e-12f, sa)); s1 = sb * sphi / den;
        const float r = sqrtf(c1 * c1 + s1 * s1);
        if (r < 1e-12f) { c1 = 1.f; s1 = 0.f; } else { c1 /= r; s1 /= r; }
    }
    if (sb <= pole) { c2 = -copysignf(1.f, mb) * cphi; s2 = sphi; }
    else {
        c2 = (ma - mb * cT) / (den * fmaxf(1e-12f, sb)); s2 = sa * sphi / den;
        const float r = sqrtf(c2 * c2 + s2 * s2);
        if (r < 1e-12f) { c2 = 1.f; s2 = 0.f; } else { c2 /= r; s2 /= r; }
    }
}

// out = L2 * MT * L1 for MT = [[f0, f1, 0], [f1, f0, 0], [0, 0, f8]]
__device__ __forceinline__ void rotate_f(float f0, float f1, float f8, float c1, float s1, float c2, float s2,
                                         float *R)
{
    const float a1 = c1 * c1 - s1 * s1, b1 = 2.f * c1 * s1, a2 = c2 * c2 - s2 * s2, b2 = 2.f * c2 * s2;
    const float A01 = f1 * a1, A02 = -f1 * b1, A11 = f0 * a1, A12 = -f0 * b1, A21 = f8 * b1, A22 = f8 * a1;
    R[0] = f0; R[1] = A01; R[2] = A02;
    R[3] = a2 * f1; R[4] = a2 * A11 - b2 * A21; R[5] = a2 * A12 - b2 * A22;
    R[6] = b2 * f1; R[7] = b2 * A11 + a2 * A21; R[8] = b2 * A12 + a2 * A22;
}

// Air -> water facet transmission Mueller, incident air cosine mu_i (sine si),
// refracted water cosine mu_o (sine so) (shared/surface.c:80-119, 1476-1568).
// The sines come from the caller's FP64 cosines: near the pole an FP32
// 1 - mu^2 loses the tilt and flips the rotation onto its pole limit.
__device__ void taw_mueller(float mu_i, float si, float mu_o, float so, float cphi, float sphi, float s2v, float n,
                            int qc, float *T)
{
#pragma unroll
    for (int e = 0; e < 9; ++e) T[e] = 0.f;
    if (mu_i <= 1e-9f || mu_o <= 1e-9f) return;
    // half vector h ~ -(i + n o), i = (si, 0, mu_i), o = (so cphi, so sphi, -mu_o)
    float hx = -(si + n * so * cphi), hy = -(n * so * sphi), hz = n * mu_o - mu_i;
    const float hh = hx * hx + hy * hy, hn2 = hh + hz * hz;
    if (hn2 < 1e-24f) return;
    const float inv = rsqrtf(hn2);
    if (hz < 0.f) { hx = -hx; hy = -hy; hz = -hz; }
    const float ih = (si * hx + mu_i * hz) * inv;
    const float oh = (so * cphi * hx + so * sphi * hy - mu_o * hz) * inv;
    const float hzn = hz * inv;
    if (ih <= 0.f || hzn <= 1e-9f) return;
    const float tan2 = hh / (hz * hz);
    const float cos2 = hzn * hzn;
    const float D = expf(-tan2 / s2v) / (3.14159265f * s2v * cos2 * cos2);
    float den = ih + n * oh;
    den *= den;
    if (den < 1e-12f) return;
    const float sti = sqrtf(fmaxf(0.f, 1.f - ih * ih)), stt = sti / n;
    float Ts = 0.f, Tp = 0.f;
    if (stt < 1.f) {
        const float ctt = sqrtf(fmaxf(0.f, 1.f - stt * stt));
        const float rs = (ih - n * ctt) / (ih + n * ctt), rp = (n * ih - ctt) / (n * ih + ctt);
        Ts = 1.f - rs * rs; Tp = 1.f - rp * rp;
    }
    const float common = (fabsf(ih) * fabsf(oh)) / (mu_i * mu_o) * (n * n * D) / den;
    const float fs = common * Ts, fp = common * Tp, fsp = common * sqrtf(fmaxf(0.f, Ts * Tp));
    const float f1 = qc == 1 ? 0.5f * (fp - fs) : 0.5f * (fs - fp);
    // rotations on the photon propagation directions (both cosines negative,
    // azimuth shifted by pi), surface.c:1517-1557
    const float cr = -cphi, sr = -sphi, mis = -mu_i, mos = -mu_o;
    float cP = mis * mos + si * so * cr;
    cP = fminf(1.f, fmaxf(-1.f, cP));
    float c1, s1, c2, s2;
    rot_pair_f(mis, si, mos, so, cP, cr, sr, c1, s1, c2, s2);
    rotate_f(0.5f * (fs + fp), f1, fsp, c1, s1, c2, s2, T);
}

// Water -> air facet transmission Mueller, air cosine mu2 (sine s2), upwelling
// water cosine mu1 (sine s1) (shared/surface.c:648-764); the facet tilt from
// the normal N = n p1 - p2: tan^2(beta) = |N_h|^2 / N_z^2.  Sines as for
// taw_mueller.
__device__ void twa_mueller(float mu2, float s2, float mu1, float s1, float cphi, float sphi, float s2v, float slen,
                            float n, int qc, float *T)
{
#pragma unroll
    for (int e = 0; e < 9; ++e) T[e] = 0.f;
    if (mu1 <= 1e-9f || mu2 <= 1e-9f) return;
    float cP = mu1 * mu2 + s1 * s2 * cphi;
    cP = fminf(1.f, fmaxf(-1.f, cP));
    const float Nz = n * mu1 - mu2;
    const float Nhx = n * s1 - s2 * cphi, Nhy = s2 * sphi;
    const float Nh2 = Nhx * Nhx + Nhy * Nhy;
    const float Nsq = Nh2 + Nz * Nz;
    if (Nsq <= 1e-12f) return;
    const float Nm = sqrtf(Nsq);
    const float cb = Nz / Nm, cw = (n - cP) / Nm;
    if (cb <= 1e-6f || cw <= 1e-6f) return;
    const float st2 = n * n * fmaxf(0.f, 1.f - cw * cw);
    if (st2 >= 1.f) return;
    const float maf = sqrtf(1.f - st2);
    const float rs = (n * cw - maf) / (n * cw + maf), rp = (cw - n * maf) / (cw + n * maf);
    const float ts = 1.f + rs, tp = n * (1.f + rp);
    const float cb2 = cb * cb, tb2 = Nh2 / (Nz * Nz);
    const float P = expf(-tb2 / s2v) / (3.14159265f * s2v);
    const float S = 1.f / (1.f + sancer_f(mu1, slen) + sancer_f(mu2, slen));
    const float common = (maf * maf) / (n * mu1 * mu2 * Nsq) * (P / (cb2 * cb2)) * S;
    const float fs = common * ts * ts, fp = common * tp * tp, fsp = common * ts * tp;
    const float f1 = qc == 1 ? 0.5f * (fp - fs) : 0.5f * (fs - fp);
    float c1, si1, c2, si2;
    rot_pair_f(mu1, s1, mu2, s2, cP, cphi, sphi, c1, si1, c2, si2);
    rotate_f(0.5f * (fs + fp), f1, fsp, c1, si1, c2, si2, T);
}

// Shared-memory table of cos(m phi_q), sin(m phi_q) on the midpoint grid
// phi_q = (q + 1/2) 2 pi / nphi for m <= M: cs[(m * nphi + q) * 2 + {0, 1}].
__device__ void fill_cs(float *cs, int M, int nphi)
{
    for (int x = threadIdx.x; x < (M + 1) * nphi; x += blockDim.x) {
        const int m = x / nphi, q = x - m * nphi;
        float s, c;
        // m (2q + 1) / nphi reduced exactly before the pi-scaled sincos
        const long long num = (long long)m * (2 * q + 1) % (2LL * nphi);
        sincospif((float)num / (float)nphi, &s, &c);
        cs[2 * x] = c; cs[2 * x + 1] = s;
    }
}

// Fourier coefficients of one kernel sampled by the block in Rq[nphi][9]:
// out[m][e] = (dphi / (2 pi or pi)) sum_q Rq[q][e] {cos, sin}(m phi_q), with
// the incoming-U column of m > 0 negated when fold_u (T_aw, T_wa: surface.c
// :1680-1684, 1722-1729).  Ends with a block barrier.
__device__ void project_block(const float *Rq, const float *cs, int nphi, int M, bool fold_u, float *out)
{
    const float dphi = 6.28318530718f / (float)nphi;
    for (int o = threadIdx.x; o < (M + 1) * 9; o += blockDim.x) {
        const int m = o / 9, e = o - 9 * m;
        const int sin_e = (e == 2 || e == 5 || e == 6 || e == 7);
        const float *t = cs + (size_t)m * nphi * 2 + sin_e;
        float acc = 0.f;
        for (int q = 0; q < nphi; ++q) acc = fmaf(Rq[q * 9 + e], t[2 * q], acc);
        float v = acc * dphi * (m == 0 ? 0.159154943092f : 0.318309886184f);
        if (fold_u && m > 0 && (e == 2 || e == 5)) v = -v;
        out[o] = v;
    }
    __syncthreads();
}

} // namespace

// Totals at the surface-side levels for every (task, ring slot) of a wave.
__global__ void k_edges(BatchBufs B, WaveBufs W, Geom G, int t0, int nw, double *edge)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nw * G.NR) return;
    const int tl = x / G.NR, g = x - tl * G.NR, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    double *e = edge + ((size_t)tg * G.NR + g) * OCRT_EDGE;
    if (g >= d.n_ring) {
        for (int q = 0; q < OCRT_EDGE; ++q) e[q] = 0.0;
        return;
    }
    const int nt = d.nt;
    const float *Tot = W.Tot + tk.fld_off;
    const bool seed = d.rough && !d.bottom_only;
    float fs_tdn = 0.f;
    if (seed) fs_tdn = (float)((tk.m == 0 ? OCRT_PI : 0.5 * OCRT_PI) * d.mu0 * exp(-d.tau_total / d.mu0));
    for (int s = 0; s < 3; ++s) {
        double u = tot_value(W, tk, G, 0, nt, col_of(G, s, 0, g));
        if (seed) {
            const float *Rs = W.srf + tk.srf_off + (size_t)G.NR * G.N * 9;
            u -= (double)(fs_tdn * B.Eatt[(d.lev_off + 0) * G.NR + g] * Rs[g * 9 + s * 3]);
        }
        e[s] = u;
        e[3 + s] = tot_value(W, tk, G, nt, nt, col_of(G, s, 1, g));
    }
    e[6] = tot_value(W, tk, G, 0, nt, col_of(G, 0, 1, g));
    e[7] = nt >= 1 ? (double)Tot[(size_t)1 * G.LDC + col_of(G, 0, 0, g)] : 0.0;
    e[8] = nt >= 1 ? (double)Tot[(size_t)1 * G.LDC + col_of(G, 0, 1, g)] : 0.0;
    e[9] = e[10] = e[11] = 0.0;
}

// Water-side internal-reflection Fourier kernels R_m[o][i][9] of every water
// pixel of a wave: outgoing (downward) ring slot o, incoming (upward) Gauss
// node i, modes 0..M on nphi midpoint azimuths, no U fold (surface.c:1386-1449).
// One block per (o, pixel); the block samples the azimuths of one pair at a
// time and projects them.
__global__ void k_rww(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                      const double *gmu, int nphi, float *srf)
{
    const int o = blockIdx.x, p = p0 + blockIdx.y;
    const PixDev &d = px[p];
    if (d.medium != 1 || o >= d.n_ring) return;
    const int N = G.N, M = d.M;
    extern __shared__ float sm[];
    float *cs = sm;                                  // [(M+1) nphi 2]
    float *Rq = cs + (size_t)(M + 1) * nphi * 2;     // [nphi][9]
    float *out = Rq + (size_t)nphi * 9;              // [(M+1) 9]
    fill_cs(cs, M, nphi);
    const float s2v = (float)slope_variance(d.wind, d.sigma_type), slen = sqrtf(s2v);
    const float mo = (float)ring_mu(d, gmu, N, o), nw = (float)d.n_water;
    const float lo = sancer_f(mo, slen);
    const float dphi = 6.28318530718f / (float)nphi;
    __syncthreads();
    for (int i = 0; i < N; ++i) {
        const float mi = (float)gmu[i];
        const float lam = lo + sancer_f(mi, slen);
        for (int q = threadIdx.x; q < nphi; q += blockDim.x) {
            const float phi = (q + 0.5f) * dphi;
            float sp, cp;
            sincosf(phi, &sp, &cp);
            const float sh = sinf(0.5f * phi);
            coxmunk_R<float>(mo, mi, cp, sp, sh * sh, s2v, lam, nw, d.q_conv, Rq + q * 9, nullptr, true);
        }
        __syncthreads();
        project_block(Rq, cs, nphi, M, false, out);
        for (int x = threadIdx.x; x < (M + 1) * 9; x += blockDim.x) {
            const int m = x / 9, e = x - 9 * m;
            const TaskDev tk = tasks[pix_task0[p] + m];
            srf[tk.srf_off + ((size_t)o * N + i) * 9 + e] = out[x];
        }
        __syncthreads();
    }
}

// Slope-integrated air->water irradiance transmittance (101 x 101 trapezoid
// over +-6 sigma, surface.c:144-179) of the sun (slot -1, stored at [na]) and
// of every atmosphere ring slot: td[p * (NRa + 1) + slot].  One block each.
__global__ void k_taw_direct(const OceanPix *op, int P, const PixDev *pxa, const double *gmu, int N, int NRa, double *td)
{
    const int p = blockIdx.y, slot = (int)blockIdx.x - 1;
    if (p >= P) return;
    const OceanPix &o = op[p];
    const PixDev &da = pxa[o.pa];
    double mu;
    if (slot < 0) mu = o.mu_sa;
    else if (slot < N) mu = gmu[slot];      // zero-weight ring slots are never weighted
    else return;
    double *dst = td + (size_t)p * (NRa + 1) + (slot < 0 ? NRa : slot);
    const double s2v = slope_variance(o.wind, o.st), nw = o.nw;
    const double ss = sqrt(fmax(0.0, 1.0 - mu * mu));
    __shared__ double red[32];
    if (mu <= 1e-9) { if (threadIdx.x == 0) *dst = 0.0; return; }
    const double L = 6.0 * sqrt(s2v);
    const int NQ = 101;
    const double dz = 2.0 * L / (double)(NQ - 1);
    double acc = 0.0;
    for (int x = threadIdx.x; x < NQ * NQ; x += blockDim.x) {
        const int i = x / NQ, j = x - i * NQ;
        const double zx = -L + i * dz, zy = -L + j * dz;
        const double wx = (i == 0 || i == NQ - 1) ? 0.5 : 1.0, wy = (j == 0 || j == NQ - 1) ? 0.5 : 1.0;
        const double proj = mu + zx * ss;
        if (proj <= 0.0) continue;
        const float r2 = (float)(zx * zx + zy * zy);
        const float cti = (float)proj * rsqrtf(1.f + r2);
        const float stt = sqrtf(fmaxf(0.f, 1.f - cti * cti)) / (float)nw;
        const float ctt = sqrtf(fmaxf(0.f, 1.f - stt * stt));
        const float nf = (float)nw;
        const float rs = (cti - nf * ctt) / (cti + nf * ctt), rp = (nf * cti - ctt) / (nf * cti + ctt);
        const float TF = 1.f - 0.5f * (rs * rs + rp * rp);
        const float pd = expf(-r2 / (float)s2v);
        acc += wx * wy * (double)pd * proj * (double)TF;
    }
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[w];
        t *= dz * dz / (OCRT_PI * s2v) / mu;
        *dst = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    }
}

// Per-pixel scalars of the coupling (rt_solver.c:3737-3770, 4258-4357,
// 4603-4646): direct transmittance, flux at the bottom of the atmosphere, the
// refracted beam's flux in the water F_w = F_boa mu0 T_aw(mu0) / mu_w, and the
// diffuse irradiance just above (incident) and below (transmitted) the surface
// from the atmosphere's bottom field at m = 0.
__global__ void k_ocean_prep(OceanPix *op, int P, const int *task0_a, const double *gmu, const double *gw, int N,
                             int NRa, const double *edge_a, const double *td)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    OceanPix &o = op[p];
    o.T_dir = (o.mu_sa > 0.0 && o.tau_atm > 0.0) ? exp(-o.tau_atm / o.mu_sa) : 1.0;
    o.F_boa = OCRT_PI * o.T_dir;
    double Taw = td[(size_t)p * (NRa + 1) + NRa];
    Taw = Taw < 0.0 ? 0.0 : (Taw > 1.0 ? 1.0 : Taw);
    o.F_w = o.F_boa * o.mu_sa * Taw / o.mu_sw;
    double ew = 0.0, ea = 0.0;
    const double *e0 = edge_a + (size_t)task0_a[o.pa] * NRa * OCRT_EDGE;     // mode 0 of the pixel
    for (int j = 0; j < N; ++j) {
        const double muL = gw[j] * gmu[j] * e0[(size_t)j * OCRT_EDGE + 3];
        ew += muL * td[(size_t)p * (NRa + 1) + j];
        ea += muL;
    }
    o.Ed_sky_w = ew * 2.0 * OCRT_PI;
    o.Ed_sky_a = ea * 2.0 * OCRT_PI;
}

// Skylight transmitted into the water, per (water Gauss node iw, pixel):
//   top[m][iw][s] = (-1)^m (pi / F_w) sum_ja (2 pi or pi) mu_a w_a T_aw^m(iw, ja) . S_boa^m(ja)
// the T_aw kernels on 128 azimuths with the incoming-U fold, odd modes turned
// to the water's azimuth base, the whole on the water solve's F_w scale
// (rt_solver.c:4164-4225, 4636-4646; rt_air_water_coupling.c:244-311).
__global__ void k_couple_aw(const OceanPix *op, int P, const int *task0_a, const double *gmu, const double *gw,
                            int N, int NRa, const double *edge_a, double *top)
{
    const int iw = blockIdx.x, p = blockIdx.y;
    if (p >= P || iw >= N) return;
    const OceanPix &o = op[p];
    const int M = o.M, nphi = 128;
    extern __shared__ float sm[];
    float *cs = sm;
    float *Rq = cs + (size_t)(M + 1) * nphi * 2;
    float *out = Rq + (size_t)nphi * 9;
    double *acc = reinterpret_cast<double *>(out + (((M + 1) * 9 + 1) & ~1));
    fill_cs(cs, M, nphi);
    for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) acc[x] = 0.0;
    const float s2v = (float)slope_variance(o.wind, o.st), nw = (float)o.nw;
    const float muw = (float)gmu[iw], sw = (float)sqrt(fmax(0.0, 1.0 - gmu[iw] * gmu[iw]));
    const float dphi = 6.28318530718f / (float)nphi;
    __syncthreads();
    for (int ja = 0; ja < N; ++ja) {
        const float mua = (float)gmu[ja], sa = (float)sqrt(fmax(0.0, 1.0 - gmu[ja] * gmu[ja]));
        for (int q = threadIdx.x; q < nphi; q += blockDim.x) {
            const float phi = (q + 0.5f) * dphi;
            float sp, cp;
            sincosf(phi, &sp, &cp);
            taw_mueller(mua, sa, muw, sw, cp, sp, s2v, nw, o.qc, Rq + q * 9);
        }
        __syncthreads();
        project_block(Rq, cs, nphi, M, true, out);
        for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) {
            const int m = x / 3, s = x - 3 * m;
            const double *eb = edge_a + ((size_t)(task0_a[o.pa] + m) * NRa + ja) * OCRT_EDGE;
            const double wj = (m == 0 ? 2.0 * OCRT_PI : OCRT_PI) * gmu[ja] * gw[ja];
            const float *T = out + m * 9 + s * 3;
            acc[x] += wj * ((double)T[0] * eb[3] + (double)T[1] * eb[4] + (double)T[2] * eb[5]);
        }
        __syncthreads();
    }
    const double scale = OCRT_PI / o.F_w;
    for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) {
        const int m = x / 3;
        top[(size_t)o.top_off + ((size_t)m * N + iw) * 3 + (x - 3 * m)] = ((m & 1) ? -scale : scale) * acc[x];
    }
}

// Unscattered skylight in the water column as a field: on the downward Gauss
// columns F[k] = top[m][c] exp(-h_k / mu_c), zero elsewhere.  The source pass
// applied to it gives the skylight's first-scatter source, equal to the
// reference's diffuse-top primary (rt_water_rt.c:681-913).  One block per task.
__global__ void k_dtop_field(BatchBufs B, WaveBufs W, Geom G, int t0)
{
    const int tl = blockIdx.x, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    float *F = W.F + tk.fld_off;
    const bool on = d.medium == 1 && d.ext_off >= 0 && tk.m <= d.ext_mmax;
    const double *top = on ? B.ext + d.ext_off + (size_t)tk.m * G.N * 3 : nullptr;
    for (int x = threadIdx.x; x < (d.nt + 1) * G.LDC; x += blockDim.x) {
        const int k = x / G.LDC, c = x - k * G.LDC;
        float v = 0.f;
        if (on && c < 6 * G.N) {
            const int s = c / (2 * G.N), r = c - s * 2 * G.N, h = r / G.N, g = r - h * G.N;
            if (h == 1) v = (float)(top[g * 3 + s] * exp(-B.h[d.lev_off + k] / B.gmu[g]));
        }
        F[x] = v;
    }
}

// Water modes that the reference's mode loop reaches: from m = 3 on it stops
// after two consecutive modes whose view amplitude is below tolerance x the
// running maximum (rt_water_rt.c:6148-6169); the stopping mode keeps its view
// sample but not its node values.  m_view / m_nodes: last mode of each.
__global__ void k_water_modes(OceanPix *op, int P, const PixDev *pxw, const int *task0_w, int NRw, const double *edge_w)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    OceanPix &o = op[p];
    const PixDev &dw = pxw[o.pw];
    const int vs = dw.view_slot;
    double amax = 0.0;
    int streak = 0, mv = o.m_loop, mn = o.m_loop;
    for (int m = 0; m <= o.m_loop; ++m) {
        const double *e = edge_w + ((size_t)(task0_w[o.pw] + m) * NRw + vs) * OCRT_EDGE;
        const double amp = fmax(fabs(e[0]), fmax(fabs(e[1]), fabs(e[2])));
        if (amp > amax) amax = amp;
        if (m >= 3 && amax > 0.0) {
            streak = amp < dw.tol * amax ? streak + 1 : 0;
            if (streak >= 2) { mv = m; mn = m - 1; break; }
        }
    }
    o.m_view = mv;
    o.m_nodes = mn;
}

// Water-leaving radiance above the surface by the rough water->air operator
// (rt_air_water_coupling.c:598-737): per air direction a composite water-mu
// grid (1024-point trapezoid window of +-0.3 around the reverse-Snell cosine,
// Gauss-Legendre 96 outside it), T_wa rows on 128 azimuths with the U fold,
// the upwelling field at the surface interpolated linearly on the sorted,
// de-duplicated water ring.  Block (ja, p): ja < NRa an atmosphere ring slot
// (the pass-3 bottom source, modes 0..min(M, m_nodes)), ja == NRa the view
// (modes 0..m_nodes).  Results on the water solve's F_w scale (x F_w / pi),
// which pass 3 carries to the TOA unchanged (rt_water_rt.c:7438-7440).
__global__ void k_couple_wa(const OceanPix *op, int P, const PixDev *pxa, const PixDev *pxw, const int *task0_w,
                            const double *gmu, int N, int NRa, int NRw, const double *edge_w, const double *glo,
                            double *ext3, double *view)
{
    const int ja = blockIdx.x, p = blockIdx.y;
    if (p >= P) return;
    const OceanPix &o = op[p];
    const PixDev &da = pxa[o.pa];
    const PixDev &dw = pxw[o.pw];
    double mua;
    int M;
    if (ja < NRa) {
        if (ja >= da.n_ring) return;
        mua = ring_mu(da, gmu, N, ja);
        M = min(o.M, o.m_nodes);
    } else {
        mua = o.mu_va;
        M = o.m_nodes;
    }
    const int nphi = 128, NWIN = 1024, NGLO = 96, NTOT = NWIN + NGLO;
    extern __shared__ float sm[];
    float *cs = sm;
    float *Rq = cs + (size_t)(M + 1) * nphi * 2;
    float *out = Rq + (size_t)nphi * 9;
    double *acc = reinterpret_cast<double *>(out + (((M + 1) * 9 + 1) & ~1));
    double *wmu = acc + 3 * (M + 1);                 // sorted unique water cosines
    int *wsrc = reinterpret_cast<int *>(wmu + NRw);  // their ring slots
    __shared__ int nu_s;
    fill_cs(cs, M, nphi);
    for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) acc[x] = 0.0;
    if (threadIdx.x == 0) {
        const int n = dw.n_ring;
        int ord[OCRT_MAX_N + OCRT_MAX_EXTRA];
        for (int a = 0; a < n; ++a) ord[a] = a;
        for (int a = 1; a < n; ++a) {
            const int k = ord[a];
            const double mk = ring_mu(dw, gmu, N, k);
            int b = a - 1;
            while (b >= 0 && ring_mu(dw, gmu, N, ord[b]) > mk) { ord[b + 1] = ord[b]; --b; }
            ord[b + 1] = k;
        }
        int w = 0;
        for (int a = 0; a < n; ++a) {
            const double m = ring_mu(dw, gmu, N, ord[a]);
            if (w > 0 && fabs(m - wmu[w - 1]) < 1e-12) continue;
            wmu[w] = m; wsrc[w] = ord[a]; ++w;
        }
        nu_s = w;
    }
    const float s2v = (float)slope_variance(o.wind, o.st), slen = sqrtf(s2v), nw = (float)o.nw;
    const double mws = sqrt(fmax(0.0, 1.0 - (1.0 - mua * mua) / (o.nw * o.nw)));
    const float sva = (float)sqrt(fmax(0.0, 1.0 - mua * mua));
    double lo = mws - 0.30, hi = mws + 0.30;
    if (lo < 1e-6) lo = 1e-6;
    if (hi > 1.0 - 1e-9) hi = 1.0 - 1e-9;
    const double hstep = (hi - lo) / (double)(NWIN - 1);
    const float dphi = 6.28318530718f / (float)nphi;
    __syncthreads();
    const int nu = nu_s;
    const double *ew = edge_w + (size_t)task0_w[o.pw] * NRw * OCRT_EDGE;
    for (int i = 0; i < NTOT; ++i) {
        double xi, wi;
        if (i < NWIN) { xi = lo + hstep * (double)i; wi = ((i == 0 || i == NWIN - 1) ? 0.5 : 1.0) * hstep; }
        else { xi = glo[i - NWIN]; wi = (xi > lo && xi < hi) ? 0.0 : glo[NGLO + i - NWIN]; }
        if (wi == 0.0) continue;
        const float sxi = (float)sqrt(fmax(0.0, 1.0 - xi * xi));
        for (int q = threadIdx.x; q < nphi; q += blockDim.x) {
            const float phi = (q + 0.5f) * dphi;
            float sp, cp;
            sincosf(phi, &sp, &cp);
            twa_mueller((float)mua, sva, (float)xi, sxi, cp, sp, s2v, slen, nw, o.qc, Rq + q * 9);
        }
        __syncthreads();
        project_block(Rq, cs, nphi, M, true, out);
        // linear interpolation (end pairs extrapolate) on the sorted ring
        int hi_i = 1;
        while (hi_i < nu && wmu[hi_i] < xi) hi_i++;
        int lo_i = hi_i - 1;
        if (hi_i >= nu) { hi_i = nu - 1; lo_i = nu - 2; }
        if (lo_i < 0) { lo_i = 0; hi_i = 1; }
        const double t = (xi - wmu[lo_i]) / (wmu[hi_i] - wmu[lo_i]);
        for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) {
            const int m = x / 3, s = x - 3 * m;
            const float *T = out + m * 9 + s * 3;
            const double *ea = ew + ((size_t)m * NRw + wsrc[lo_i]) * OCRT_EDGE;
            const double *eb = ew + ((size_t)m * NRw + wsrc[hi_i]) * OCRT_EDGE;
            double v = 0.0;
            for (int u = 0; u < 3; ++u) v += (double)T[u] * ((1.0 - t) * ea[u] + t * eb[u]);
            acc[x] += (m == 0 ? 2.0 * OCRT_PI : OCRT_PI) * xi * wi * v;
        }
        __syncthreads();
    }
    const double f = o.F_w / OCRT_PI;
    for (int x = threadIdx.x; x < 3 * (M + 1); x += blockDim.x) {
        if (ja < NRa) ext3[(size_t)o.ext_off + ((size_t)(x / 3) * NRa + ja) * 3 + (x % 3)] = f * acc[x];
        else view[(size_t)p * 3 * (OCRT_MAX_M + 1) + x] = f * acc[x];
    }
}

// Outputs of each coupled pixel (rt_solver.c:6314-6647, rt_water_rt.c:6263-7558).
// The water fields are on the pi-normalised scale; f = F_w / pi converts them.
__global__ void k_ocean_final(const OceanPix *op, int P, const PixDev *pxa, const PixDev *pxw, const int *task0_w,
                              const double *gmu, const double *gw, int N, int NRw, const double *edge_w,
                              const double *view, const double *top, const ocrt_result *r1, const ocrt_result *rw,
                              const ocrt_result *r3, ocrt_result *out, ocrt_ocean_result *wout)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const OceanPix &o = op[p];
    const PixDev &da = pxa[o.pa];
    const PixDev &dw = pxw[o.pw];
    const double mu0 = o.mu_sa, f = o.F_w / OCRT_PI;
    const double phi = o.raa_deg * OCRT_PI / 180.0 + OCRT_PI;
    ocrt_result R = r1[o.pa];
    const ocrt_result &R3 = r3[o.pa];
    ocrt_ocean_result Wr;
    memset(&Wr, 0, sizeof(Wr));
    // TOA: atmosphere path (pass 1) + water-leaving light carried up (pass 3)
    Wr.rho_atm_I = R.I_TOA / mu0; Wr.rho_atm_Q = R.Q_TOA / mu0; Wr.rho_atm_U = R.U_TOA / mu0;
    Wr.rho_water_I = R3.I_TOA / mu0; Wr.rho_water_Q = R3.Q_TOA / mu0; Wr.rho_water_U = R3.U_TOA / mu0;
    // the glint stays out of rho (reported apart, rt_solver.c:6624-6643)
    const double gI = R.rho_glint_direct_I, gQ = R.rho_glint_direct_Q, gU = R.rho_glint_direct_U;
    R.I_TOA += R3.I_TOA; R.Q_TOA += R3.Q_TOA; R.U_TOA += R3.U_TOA;
    R.rho_I = Wr.rho_atm_I + Wr.rho_water_I;
    R.rho_Q = Wr.rho_atm_Q + Wr.rho_water_Q;
    R.rho_U = Wr.rho_atm_U + Wr.rho_water_U;
    R.rho_glint_direct_I = gI; R.rho_glint_direct_Q = gQ; R.rho_glint_direct_U = -gU;
    R.T_dir_dn = o.T_dir;
    R.T_total_dn_hemi = R.T_dir_dn + R.T_diff_dn_hemi;
    R.T_dir_up_view = exp(-o.tau_atm / (o.mu_va > 0.0 ? o.mu_va : 1.0));
    R.order_modes += R3.order_modes;
    // water column: view sample at 0- per mode, fluxes from m = 0
    const double *e0 = edge_w + (size_t)task0_w[o.pw] * NRw * OCRT_EDGE;
    double vi = 0.0, vq = 0.0, vu = 0.0;
    for (int m = 0; m <= o.m_view; ++m) {
        const double *e = e0 + ((size_t)m * NRw + dw.view_slot) * OCRT_EDGE;
        const double c = m == 0 ? 1.0 : 2.0 * cos(m * phi), s = m == 0 ? 0.0 : 2.0 * sin(m * phi);
        vi += c * e[0]; vq += c * e[1]; vu += s * e[2];
    }
    double Edd = 0.0, Eud = 0.0, Ed1 = 0.0, Eu1 = 0.0;
    for (int j = 0; j < N; ++j) {
        const double *e = e0 + (size_t)j * OCRT_EDGE;
        const double mw = gmu[j] * gw[j];
        Eud += e[0] * mw; Edd += e[6] * mw; Eu1 += e[7] * mw; Ed1 += e[8] * mw;
    }
    const double Ed_w = o.F_w * o.mu_sw + 2.0 * OCRT_PI * Edd * f;
    const double Eu_w = 2.0 * OCRT_PI * Eud * f;
    const double tau1 = dw.w_tau / (double)dw.nt, z1 = tau1 / o.ext_w;
    const double Ed1_w = o.F_w * o.mu_sw * exp(-tau1 / o.mu_sw) + 2.0 * OCRT_PI * Ed1 * f;
    const double Eu1_w = 2.0 * OCRT_PI * Eu1 * f;
    double Kd = (Ed1_w > 0.0 && Ed_w > 0.0) ? -log(Ed1_w / Ed_w) / fmax(z1, 1e-12) : 0.0;
    const double Ku = (Eu1_w > 0.0 && Eu_w > 0.0) ? -log(Eu1_w / Eu_w) / fmax(z1, 1e-12) : 0.0;
    // Kd with the unscattered skylight re-added (rt_solver.c:3419-3466)
    {
        double q0 = 0.0, q1 = 0.0;
        const double *tp = top + o.top_off;
        for (int c = 0; c < N; ++c) {
            const double I0 = tp[c * 3];
            if (!(gw[c] > 0.0) || !isfinite(I0)) continue;
            q0 += I0 * gmu[c] * gw[c];
            q1 += I0 * gmu[c] * gw[c] * exp(-tau1 / gmu[c]);
        }
        if (q0 > 0.0 && q1 > 0.0 && Ed1_w > 0.0 && tau1 > 0.0 && z1 > 0.0) {
            const double sc = 2.0 * OCRT_PI * f;
            const double E0 = Ed_w + sc * q0, E1 = Ed1_w + sc * q1;
            if (E0 > 0.0 && E1 > 0.0) {
                const double kd = -log(E1 / E0) / z1;
                if (isfinite(kd)) Kd = kd;
            }
        }
    }
    // view above the surface
    const double *va = view + (size_t)p * 3 * (OCRT_MAX_M + 1);
    double ai = 0.0, aq = 0.0, au = 0.0;
    for (int m = 0; m <= o.m_nodes; ++m) {
        const double c = m == 0 ? 1.0 : 2.0 * cos(m * phi), s = m == 0 ? 0.0 : 2.0 * sin(m * phi);
        ai += c * va[3 * m]; aq += c * va[3 * m + 1]; au += s * va[3 * m + 2];
    }
    Wr.Lu_0minus_I = vi * f; Wr.Lu_0minus_Q = vq * f; Wr.Lu_0minus_U = vu * f;
    Wr.Lu_0plus_I = ai; Wr.Lu_0plus_Q = aq; Wr.Lu_0plus_U = au;
    Wr.Ed_0minus = Ed_w + o.Ed_sky_w;
    Wr.Eu_0minus = Eu_w;
    Wr.Ed_0plus = o.F_boa * mu0 + o.Ed_sky_a;
    Wr.Ed_0minus_direct = o.F_w * o.mu_sw;
    Wr.Ed_0plus_direct = o.F_boa * mu0;
    Wr.Rrs_0plus_I = Wr.Lu_0plus_I / Wr.Ed_0plus; Wr.Rrs_0plus_Q = Wr.Lu_0plus_Q / Wr.Ed_0plus;
    Wr.Rrs_0plus_U = Wr.Lu_0plus_U / Wr.Ed_0plus;
    Wr.rrs_0minus_I = Wr.Lu_0minus_I / Wr.Ed_0minus; Wr.rrs_0minus_Q = Wr.Lu_0minus_Q / Wr.Ed_0minus;
    Wr.rrs_0minus_U = Wr.Lu_0minus_U / Wr.Ed_0minus;
    Wr.Kd_0minus = Kd; Wr.Ku_0minus = Ku;
    Wr.tau_water = dw.w_tau; Wr.depth_water_m = dw.w_tau / o.ext_w;
    Wr.n_layers_water = dw.nt; Wr.n_ring_water = o.n_ring_unique;
    Wr.orders_water = rw[o.pw].n_orders_used; Wr.converged_water = rw[o.pw].converged;
    R.n_orders_used = Wr.orders_water; R.converged = Wr.converged_water;
    R.order_modes += rw[o.pw].order_modes;
    (void)da;
    out[p] = R;
    wout[p] = Wr;
}
