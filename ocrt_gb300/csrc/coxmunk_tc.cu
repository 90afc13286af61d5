// coxmunk_tc.cu — Cox-Munk Fourier kernels (shared/surface.c:839-1135) with the
// azimuth projection on the tcgen05 tensor cores.
//
// For one pixel, a CTA takes CMT_P (outgoing slot, incoming slot) pairs.  The
// 9 Mueller entries of every pair form 9 rows of the A operand (126 of the 128
// rows; the last two are zero) and the half azimuth grid is the K dimension:
//   D[(pair, e)][n] = sum_q R_e(phi_q) B[n][q],
// with B[n] = cos(n phi) for n < NM and sin((n - NM) phi) for NM <= n < 2 NM
// (NM = M + 1 rounded up to 8), so D holds every cos and sin coefficient of
// every entry; the epilogue keeps cos for the entries 0, 1, 3, 4, 8 and sin for
// 2, 5, 6, 7.  The wind-derivative variant adds a second A operand, R tan^2(beta),
// into a second accumulator.
//
// K is swept in chunks of 32 azimuth nodes (one 128-byte swizzle row).  For a
// chunk every one of the 448 threads evaluates one Mueller matrix on the CUDA
// cores (FP32, the same coxmunk_R as the CUDA-core kernel) and stores the tf32 (hi, lo)
// split into the SWIZZLE_128B K-major A tiles, while a TMA bulk copy brings the
// chunk's B tiles (the cos/sin table already split and swizzled once per
// group by k_cs_tiles).  One thread then issues the three kind::tf32 MMAs per
// 8-node slice (hi*hi + hi*lo + lo*hi).  Two stages in the plain variant: the
// MMAs of chunk c run while chunk c + 1 is evaluated.  The wind-derivative
// variant's stage (four A tiles) is too large for two stages at two CTAs per
// SM, so it keeps one: a CTA's MMAs and its next chunk's evaluation
// alternate, and the second CTA on the SM fills the gaps (two CTAs of one
// stage ran faster than one CTA of two: the evaluation, not the MMA, is the
// long phase).  Gauss-Gauss pairs are evaluated once per
// reciprocal couple and written both ways, as in k_coxmunk.  Every wait is
// bounded by TC_WAIT_NS.
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"
#include "physics.cuh"
#include "tcgen05.cuh"

using namespace tcg;

#define CMT_P 14            // pairs per CTA (9 rows each)
#define CMT_THREADS 224     // CMT_P x CMT_KC / 2: two Mueller evaluations per thread and chunk
#define CMT_THREADS_DW 448  // CMT_P x CMT_KC: one Mueller evaluation per thread and chunk
#define CMT_KC 32           // azimuth nodes per chunk

// Pair constants of the Mueller evaluation (coxmunk_R in physics.cuh with
// mu_out = mo, mu_in = -mi): everything that does not depend on the azimuth.
struct CmPair {
    float mo, mi, s1, s2, musum, A2, d12, s4, s12, inv_s1, inv_s2, inv_A2, inv_musum, inv_sig2, kfac, nw, inv_nw2;
    int pole1, pole2;
};

__device__ inline CmPair cm_pair(float mu_out, float mu_in_dn, float sig2, float lam, float nw)
{
    CmPair c;
    c.mo = mu_out;
    c.mi = -mu_in_dn;
    c.s1 = sqrtf(fmaxf(0.f, 1.f - mu_out * mu_out));
    c.s2 = sqrtf(fmaxf(0.f, 1.f - c.mi * c.mi));
    c.musum = mu_out + mu_in_dn;
    c.A2 = c.musum * c.musum;
    c.d12 = (c.s1 - c.s2) * (c.s1 - c.s2);
    c.s4 = 4.f * c.s1 * c.s2;
    c.s12 = c.s1 * c.s2;
    c.inv_s1 = 1.f / fmaxf(1e-12f, c.s1);
    c.inv_s2 = 1.f / fmaxf(1e-12f, c.s2);
    c.inv_A2 = 1.f / c.A2;
    c.inv_musum = 1.f / c.musum;
    c.inv_sig2 = 1.f / sig2;
    c.kfac = ((1.f / (float)OCRT_PI / sig2) / (1.f + lam)) / (4.f * mu_in_dn * mu_out);
    c.nw = nw;
    c.inv_nw2 = (1.f / nw) * (1.f / nw);
    c.pole1 = c.s1 <= 1e-8f;
    c.pole2 = c.s2 <= 1e-8f;
    return c;
}

// Cox-Munk reflection Mueller matrix at one azimuth (the formulas of coxmunk_R:
// facet geometry in the cancellation-free form, Sancer shadowing, Fresnel at
// the facet angle, L2 MF L1 rotations), with the pair constants hoisted and the
// per-azimuth divisions turned into two reciprocals, two Fresnel quotients and
// two reciprocal square roots.  tb2 = tan^2(beta) of the facet.
__device__ inline void cm_mueller(const CmPair &c, float cphi, float sphi, float shalf2, int qconv, float *R, float &tb2)
{
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = 0.f;
    tb2 = 0.f;
    float cT = c.mo * c.mi + c.s12 * cphi;
    cT = fminf(1.f, fmaxf(-1.f, cT));
    const float Bt = c.d12 + c.s4 * shalf2;
    const float cw = 0.5f * sqrtf(c.A2 + Bt);
    if (cw <= 1e-6f) return;
    const float inv_cb = 2.f * cw * c.inv_musum;             // 1 / cos(beta)
    if (inv_cb >= 1e6f) return;
    const float sT = sqrtf(fmaxf(0.f, 1.f - cT * cT));
    const float inv_den = 1.f / fmaxf(1e-12f, sT);
    float c1, si1, c2, si2;
    if (c.pole2) { c1 = -copysignf(1.f, c.mi) * cphi; si1 = sphi; }
    else {
        const float u = (c.mo - c.mi * cT) * c.inv_s2, v = c.s1 * sphi, n2 = u * u + v * v;
        if (n2 * inv_den * inv_den < 1e-24f) { c1 = 1.f; si1 = 0.f; }
        else { const float r = rsqrtf(n2); c1 = u * r; si1 = v * r; }
    }
    if (c.pole1) { c2 = -copysignf(1.f, c.mo) * cphi; si2 = sphi; }
    else {
        const float u = (c.mi - c.mo * cT) * c.inv_s1, v = c.s2 * sphi, n2 = u * u + v * v;
        if (n2 * inv_den * inv_den < 1e-24f) { c2 = 1.f; si2 = 0.f; }
        else { const float r = rsqrtf(n2); c2 = u * r; si2 = v * r; }
    }
    // Fresnel at the facet angle cos(omega) = cw
    float f0 = 1.f, f1 = 0.f, f8 = 1.f;
    const float st2 = c.inv_nw2 * fmaxf(0.f, 1.f - cw * cw);
    if (st2 < 1.f) {
        const float mt = sqrtf(1.f - st2);
        const float rs = __fdividef(cw - c.nw * mt, cw + c.nw * mt);
        const float rp = __fdividef(c.nw * cw - mt, c.nw * cw + mt);
        const float Rs = rs * rs, Rp = rp * rp;
        f0 = 0.5f * (Rs + Rp);
        f1 = qconv == 1 ? 0.5f * (Rp - Rs) : 0.5f * (Rs - Rp);
        f8 = rs * rp;
    }
    tb2 = Bt * c.inv_A2;
    const float ib2 = inv_cb * inv_cb;
    const float brdf = c.kfac * expf(-tb2 * c.inv_sig2) * ib2 * ib2;
    const float a1 = c1 * c1 - si1 * si1, b1 = 2.f * c1 * si1;
    const float a2 = c2 * c2 - si2 * si2, b2 = 2.f * c2 * si2;
    const float A01 = f1 * a1, A02 = -f1 * b1, A11 = f0 * a1, A12 = -f0 * b1, A21 = f8 * b1, A22 = f8 * a1;
    R[0] = f0 * brdf; R[1] = A01 * brdf; R[2] = A02 * brdf;
    R[3] = (a2 * f1) * brdf; R[4] = (a2 * A11 - b2 * A21) * brdf; R[5] = (a2 * A12 - b2 * A22) * brdf;
    R[6] = (b2 * f1) * brdf; R[7] = (b2 * A11 + a2 * A21) * brdf; R[8] = (b2 * A12 + a2 * A22) * brdf;
}

// B tiles of every chunk, split into tf32 (hi, lo) and laid out exactly as the
// kernel's shared-memory B operand: tiles[c] = hi [NN rows x 128 B, swizzled]
// then lo.  One block per chunk.
__global__ void k_cs_tiles(int Mtab, int nphi, const float *cs_tab, float *tiles)
{
    const int c = blockIdx.x, half = nphi / 2;
    const int NM = (Mtab + 1 + 7) & ~7, NN = 2 * NM;
    unsigned char *hi = reinterpret_cast<unsigned char *>(tiles) + (size_t)c * 2 * NN * 128;
    unsigned char *lo = hi + (size_t)NN * 128;
    for (int x = threadIdx.x; x < NN * (CMT_KC / 4); x += blockDim.x) {
        const int n = x >> 3, ch = x & 7;
        const int m = n < NM ? n : n - NM, kind = n < NM ? 0 : 1;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (m <= Mtab) v = *reinterpret_cast<const float4 *>(cs_tab + ((size_t)m * 2 + kind) * half + c * CMT_KC + ch * 4);
        const uint32_t off = (uint32_t)n * 128u + ((uint32_t)(ch ^ (n & 7)) << 4);
        float4 h, l;
        h.x = round_tf32f(v.x); l.x = round_tf32f(v.x - h.x);
        h.y = round_tf32f(v.y); l.y = round_tf32f(v.y - h.y);
        h.z = round_tf32f(v.z); l.z = round_tf32f(v.z - h.z);
        h.w = round_tf32f(v.w); l.w = round_tf32f(v.w - h.w);
        *reinterpret_cast<float4 *>(hi + off) = h;
        *reinterpret_cast<float4 *>(lo + off) = l;
    }
}

__global__ void __launch_bounds__(CMT_THREADS_DW)
k_coxmunk_tc(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G, const double *gmu,
             const float *cs_tab, const float *cs_tiles, int Mtab, const double *lamv, const double *lamd,
             float *srf, float *srfW, const short2 *pairs, int npairs, int dw, int *err)
{
    extern __shared__ unsigned char smem_raw[];
    const int p = p0 + blockIdx.y;
    const PixDev &d = px[p];
    const int N = G.N, M = d.M, nphi = d.nphi, half = nphi / 2;
    const int pr0 = blockIdx.x * CMT_P;
    if (!d.rough || pr0 >= npairs) return;
    const int NM = (Mtab + 1 + 7) & ~7, NN = 2 * NM;
    const uint32_t A_BYTES = 128 * CMT_KC * 4, B_BYTES = (uint32_t)NN * CMT_KC * 4;
    const uint32_t STAGE = (dw ? 4u : 2u) * A_BYTES + 2u * B_BYTES;
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int NSTG = dw ? 1 : 2;                                 // operand stages (see above)
    uint64_t *mma_done = (uint64_t *)(base + NSTG * STAGE);      // [2]
    uint64_t *fin = mma_done + 2;
    uint64_t *bfull = fin + 1;                                   // [2] B tiles of the stage landed
    uint32_t *tslot = (uint32_t *)(bfull + 2);
    volatile int *abort_flag = (volatile int *)(tslot + 1);
    float *pf = (float *)(tslot + 2);                            // per pair: ca, cb (wind derivative)
    int *pio = (int *)(pf + 2 * CMT_P);                          // per pair: outgoing slot, incoming slot, mirror
    CmPair *pc = (CmPair *)(pio + 3 * CMT_P);                    // per pair: Mueller constants
    long long *soff = (long long *)(((uintptr_t)(pc + CMT_P) + 7) & ~(uintptr_t)7);        // [M + 1]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&mma_done[0], 1);
        mbar_init(&mma_done[1], 1);
        mbar_init(fin, 1);
        mbar_init(&bfull[0], 1);
        mbar_init(&bfull[1], 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // per-pair scalars (FP32, as in the CUDA-core kernel)
    if (tid < CMT_P) {
        const int q = pr0 + tid;
        int o = G.NR, i = 0;
        if (q < npairs) { o = pairs[q].x; i = pairs[q].y; }
        const bool ok = o < d.n_ring;
        const float fmo = ok ? (float)(o < N ? gmu[o] : d.mu_view) : 0.5f;
        const float fmi = (float)(i < N ? gmu[i] : d.mu0);
        const float fs2 = d.sigma_type == 1 ? 0.003f + 0.00512f * fmaxf(0.01f, (float)d.wind)
                                            : fmaxf(0.0731f * 0.0731f * fmaxf(0.f, (float)d.wind), 1e-10f);
        const double *lp = lamv + (size_t)p * (N + 2);
        const float flam = ok ? (float)lp[i < N ? i : N + 1] + (float)lp[o] : 0.f;
        float ca = 0.f, cb = 0.f;
        if (dw && ok) {
            const float ds2 = (float)slope_variance_dw(d.wind, d.sigma_type);
            const double *ldv = lamd + (size_t)p * (N + 2);
            const float dlam = (float)ldv[i < N ? i : N + 1] + (float)ldv[o];
            ca = ds2 * (-1.f / fs2 - dlam / (1.f + flam));
            cb = ds2 / (fs2 * fs2);
        }
        pf[2 * tid] = ca;
        pf[2 * tid + 1] = cb;
        pc[tid] = cm_pair(fmo, fmi, fs2, flam, (float)d.n_water);
        pio[3 * tid] = ok ? o : -1;
        pio[3 * tid + 1] = i;
        pio[3 * tid + 2] = ok && o < N && i < N && o < i;
    }
    const int task_first = pix_task0[p];
    for (int m = tid; m <= M; m += blockDim.x) soff[m] = tasks[task_first + m].srf_off;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const float *ptab = cs_tab + (size_t)(Mtab + 1) * 2 * half;     // [cos, sin, sin^2(phi/2)][half]
    const int qc = d.q_conv;
    auto split_st = [&](unsigned char *hi, unsigned char *lo, uint32_t off, float v) {
        const float h = round_tf32f(v);
        *reinterpret_cast<float *>(hi + off) = h;
        *reinterpret_cast<float *>(lo + off) = round_tf32f(v - h);
    };
    const uint32_t idesc = idesc_tf32(128, NN);
    const int nchunk = half / CMT_KC;
    for (int c = 0; c < nchunk; ++c) {
        const int s = dw ? 0 : (c & 1);
        unsigned char *sp = base + (size_t)s * STAGE;
        unsigned char *aH = sp, *aL = sp + A_BYTES;
        unsigned char *tH = sp + 2 * A_BYTES, *tL = sp + 3 * A_BYTES;             // R tan^2(beta) (wind derivative)
        unsigned char *bH = sp + (dw ? 4 : 2) * A_BYTES, *bL = bH + B_BYTES;
        if (c >= NSTG) {
            // every thread waits (bounded) for the MMAs that read this stage
            // NSTG chunks ago; the barrier makes the abort decision block-uniform
            if (!mbar_wait(&mma_done[s], ((c / NSTG) - 1) & 1)) *abort_flag = 1;
            __syncthreads();
            if (*abort_flag) break;
        }
        const int q0 = c * CMT_KC;
        // B: the chunk's cos/sin tiles by one bulk copy (the stage is free: its
        // previous MMAs completed before the wait above)
        if (tid == 0) {
            mbar_expect_tx(&bfull[s], 2 * B_BYTES);
            bulk_g2s(bH, cs_tiles + (size_t)c * 2 * NN * CMT_KC, 2 * B_BYTES, &bfull[s]);
        }
        // A: Mueller entries of (pair, node); row = 9 pair + entry, K = node in the chunk
        for (int x = tid; x < CMT_P * CMT_KC; x += blockDim.x) {
            const int pp = x / CMT_KC, qq = x - pp * CMT_KC, q = q0 + qq;
            float R[9], tb2 = 0.f;
            if (pio[3 * pp] >= 0) {
                cm_mueller(pc[pp], ptab[q], ptab[half + q], ptab[2 * half + q], qc, R, tb2);
            } else {
#pragma unroll
                for (int e = 0; e < 9; ++e) R[e] = 0.f;
            }
#pragma unroll
            for (int e = 0; e < 9; ++e) {
                const int row = 9 * pp + e;
                const uint32_t off = (uint32_t)row * 128u + ((uint32_t)((qq >> 2) ^ (row & 7)) << 4) + (uint32_t)(qq & 3) * 4u;
                split_st(aH, aL, off, R[e]);
                if (dw) split_st(tH, tL, off, R[e] * tb2);
            }
        }
        // rows 126 and 127 are zero
        for (int x = tid; x < 2 * CMT_KC; x += blockDim.x) {
            const int row = 126 + x / CMT_KC, qq = x % CMT_KC;
            const uint32_t off = (uint32_t)row * 128u + ((uint32_t)((qq >> 2) ^ (row & 7)) << 4) + (uint32_t)(qq & 3) * 4u;
            split_st(aH, aL, off, 0.f);
            if (dw) split_st(tH, tL, off, 0.f);
        }
        // generic-proxy stores made visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            const bool bok = mbar_wait(&bfull[s], (c / NSTG) & 1);
            if (!bok) *abort_flag = 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa_h = smem_u32(aH), sa_l = smem_u32(aL), st_h = smem_u32(tH), st_l = smem_u32(tL);
            const uint32_t sb_h = smem_u32(bH), sb_l = smem_u32(bL);
            for (int kk = 0; bok && kk < CMT_KC / 8; ++kk) {
                const uint32_t off = kk * 32;
                const uint64_t bh = sdesc_sw128(sb_h + off), bl = sdesc_sw128(sb_l + off);
                const uint32_t acc0 = (c > 0 || kk > 0) ? 1u : 0u;
                umma_tf32(tmem, sdesc_sw128(sa_h + off), bh, idesc, acc0);
                umma_tf32(tmem, sdesc_sw128(sa_h + off), bl, idesc, 1u);
                umma_tf32(tmem, sdesc_sw128(sa_l + off), bh, idesc, 1u);
                if (dw) {
                    umma_tf32(tmem + (uint32_t)NN, sdesc_sw128(st_h + off), bh, idesc, acc0);
                    umma_tf32(tmem + (uint32_t)NN, sdesc_sw128(st_h + off), bl, idesc, 1u);
                    umma_tf32(tmem + (uint32_t)NN, sdesc_sw128(st_l + off), bh, idesc, 1u);
                }
            }
            umma_commit(&mma_done[s]);
        }
    }
    if (tid == 0) umma_commit(fin);
    if (!mbar_wait(fin, 0)) *abort_flag = 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    const bool done = !*abort_flag;                                  // block-uniform
    if (warp < 4 && done) {
        // epilogue: lane = row (pair, entry) of the warp's TMEM lane quadrant
        const int row = warp * 32 + lane;
        const int pp = row / 9, e = row - pp * 9;
        const bool live = row < 9 * CMT_P && pio[3 * pp] >= 0;
        const int o = live ? pio[3 * pp] : 0, i = live ? pio[3 * pp + 1] : 0;
        const bool mirror = live && pio[3 * pp + 2];
        const int kind = (e == 2 || e == 5 || e == 6 || e == 7) ? 1 : 0;
        const int et = (e % 3) * 3 + e / 3;
        const float ca = live ? pf[2 * pp] : 0.f, cb = live ? pf[2 * pp + 1] : 0.f;
        // normalisation x2 (half grid) x dphi / (2 pi) for m = 0 and dphi / pi for m > 0
        const float scale0 = 2.f / (float)nphi, scale1 = 4.f / (float)nphi;
        const size_t offp = i < N ? ((size_t)o * N + i) * 9 + e : (size_t)G.NR * N * 9 + (size_t)o * 9 + e;
        const size_t offt = ((size_t)i * N + o) * 9 + et;
        const uint32_t tb = tmem + ((uint32_t)(warp * 32) << 16);
        for (int cb16 = 0; cb16 < NN / 16; ++cb16) {
            float v[16], vt[16];
            tmem_ld16(tb + (uint32_t)(cb16 * 16), v);
            if (dw) tmem_ld16(tb + (uint32_t)(NN + cb16 * 16), vt);
            if (!live) continue;
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) {
                const int n = cb16 * 16 + jj;
                const int m = n < NM ? n : n - NM, nk = n < NM ? 0 : 1;
                if (nk != kind || m > M) continue;
                float sc = m == 0 ? scale0 : scale1;
                if (m > 0 && (e == 2 || e == 5)) sc = -sc;
                srf[soff[m] + offp] = v[jj] * sc;
                if (dw) srfW[soff[m] + offp] = (ca * v[jj] + cb * vt[jj]) * sc;
                if (mirror) {
                    float st = m == 0 ? scale0 : scale1;
                    if (m > 0 && (et == 2 || et == 5)) st = -st;
                    srf[soff[m] + offt] = v[jj] * st;
                    if (dw) srfW[soff[m] + offt] = (ca * v[jj] + cb * vt[jj]) * st;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *abort_flag) atomicExch(err, OCRT_ERR_DEVICE);
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
    }
}

size_t coxmunk_tc_smem_bytes(int Mtab, bool dw)
{
    const size_t NN = 2 * (size_t)((Mtab + 1 + 7) & ~7);
    const size_t stage = (dw ? 4 : 2) * (size_t)128 * CMT_KC * 4 + 2 * NN * CMT_KC * 4;
    return 1024 + (dw ? 1 : 2) * stage + 64 + 2 * 4 * CMT_P + 3 * 4 * CMT_P + sizeof(CmPair) * CMT_P + 16 + 8 * ((size_t)Mtab + 1);
}

size_t coxmunk_tc_tiles_floats(int Mtab, int nphi)
{
    const size_t NN = 2 * (size_t)((Mtab + 1 + 7) & ~7);
    return (size_t)(nphi / 2 / CMT_KC) * 2 * NN * CMT_KC;
}

bool coxmunk_tc_supported(int Mtab, int nphi, bool dw)
{
    return Mtab <= 63 && nphi % (2 * CMT_KC) == 0 && coxmunk_tc_smem_bytes(Mtab, dw) <= 227 * 1024;
}

int coxmunk_tc_pairs_per_cta() { return CMT_P; }

int coxmunk_tc_threads(bool dw) { (void)dw; return CMT_THREADS_DW; }
