// tables_tc.cu — phase-kernel Fourier tables and the packed aerosol operator
// (rt_angular_basis.c:278-357, rt_sos_operator.c:50-182) with the sums over
// the moment index on the tcgen05 tensor cores.
//
// Every table entry of a task (pixel, mode m) is a sum over l = m .. L of
//     (outgoing basis comp_o(l)) x (incoming basis c_i(l)) x (moment q(l)),
// so one GEMM per task gives all of them:
//     D[row][col] = sum_l A[row][l] B[col][l]
//   rows (A, 128): the outgoing bases P, R, T of Gauss slot d at row
//     32 comp + d (rows 0..95, the same for every pixel: pre-split once per
//     group by k_basis_perm and brought by bulk copies), then in rows 96 + x
//     (x = 3 which + comp) the sun (which 0) and the zero-weight slots
//     (which 1 + e) of the pixel;
//   cols (B, 256): the eight (incoming basis, moment) types
//     0 P beta  1 P gamma  2 R gamma  3 T gamma  4 R alpha  5 T alpha
//     6 R zeta  7 T zeta
//     of incoming Gauss slot i at column 32 type + i;
//   K: l swept in chunks of 32 with the even l + m in the first 16 positions
//     of a chunk and the odd ones in the last 16, so the first two 8-deep MMA
//     steps of a chunk sum E (even l + m) into TMEM columns 0..255 and the last
//     two O into columns 256..511; the tables need S = E + O and D = E - O.
// 13 of the 24 (outgoing comp, type) products of a slot pair are tables
// (pair_coefs in tables.cuh); the sun rows give the eight sun-outgoing
// products of every Gauss slot for the primary source, which k_tables
// finishes with the molecular parts.
//
// Operands are 3xTF32 (hi*hi + hi*lo + lo*hi, each split rounded to nearest)
// in SWIZZLE_128B K-major tiles.  Warp roles, one CTA per SM, persistent over
// the tasks blockIdx.x, + gridDim.x, ...:
//   warps 0..7 (main): put the task's moments in the chunk order, then per
//     chunk write the pixel rows of A and the B tile (B = Gauss basis x
//     moment, split), while a bulk copy brings the Gauss rows of A; thread 0
//     issues the chunk's 12 MMAs and commits them;
//   warps 8..15 (epilogue): once a task's MMAs are complete, move the
//     accumulators to a product table in shared memory (slot, product,
//     incoming slot) and release TMEM, then write the operator from the
//     table — a warp per outgoing slot, a lane per incoming Gauss slot, so
//     each store of a warp fills one 128-byte row of a pre-split operator
//     tile — while the main warps already run the next task.
// Every wait is bounded by TC_WAIT_NS and ends in OCRT_ERR_DEVICE.
#include <cuda.h>
#include <cstdint>
#include <type_traits>
#include "kernels.cuh"
#include "tables.cuh"
#include "tcgen05.cuh"

using namespace tcg;

#define TT_MW 8                                    // main warps
#define TT_EW 8                                    // epilogue warps
#define TT_THREADS ((TT_MW + TT_EW) * 32)
#define TT_KC 32                                   // moments per chunk (one 128-byte swizzle row)
#define TT_GROWS 96                                // Gauss rows of A
#define TT_A_BYTES (128u * TT_KC * 4u)             // A tile, hi or lo
#define TT_B_BYTES (256u * TT_KC * 4u)             // B tile, hi or lo
#define TT_AG_FLOATS (TT_GROWS * TT_KC)            // the Gauss rows of one A tile, hi or lo
#define TT_STAGE (2u * TT_A_BYTES + 2u * TT_B_BYTES)
#define TT_PS 33                                   // product-table row stride (floats)

__host__ __device__ inline int tt_kpad(int L) { return (L + 1 + TT_KC - 1) & ~(TT_KC - 1); }

// chunk position kk (0..31) -> offset of l from the chunk's first moment
__device__ __forceinline__ int tt_loff(int kk) { return kk < 16 ? 2 * kk : 2 * (kk - 16) + 1; }

// byte offset of element (row, kk) in a K-major SWIZZLE_128B tile
__device__ __forceinline__ uint32_t tt_swz(int row, int kk)
{
    return (uint32_t)row * 128u + ((uint32_t)((kk >> 2) ^ (row & 7)) << 4) + (uint32_t)(kk & 3) * 4u;
}

// Gauss bases of every mode in the chunk order of the K dimension, per group:
//   GT[((m * 3 + comp) * N + g) * Kp + 32 c + kk] = basis_comp(mu_g) at
//     l = m + 32 c + loff(kk), zero past L (the B side, multiplied by the
//     pixel's moments in the kernel);
//   AT[((m * nchx + c) * 2 + h) * 96 * 32 ...]: the same values as the Gauss
//     rows (32 comp + g) of the A tile of chunk c, split (h = 0 hi, 1 lo) and
//     swizzled, one bulk copy each.
__global__ void k_basis_perm(int N, int M, int L, const float *Bp, const float *Br, const float *Bt, float *GT,
                             float *AT)
{
    const int m = blockIdx.y;
    if (m > M) return;
    const int Kp = tt_kpad(L), nchx = Kp / TT_KC;
    const size_t per = (size_t)3 * N * Kp;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < per; e += (size_t)gridDim.x * blockDim.x) {
        const int kp = (int)(e % Kp);
        const size_t r = e / Kp;
        const int g = (int)(r % N), comp = (int)(r / N);
        const int l = m + 32 * (kp >> 5) + tt_loff(kp & 31);
        float v = 0.f;
        if (l <= L) {
            const float *B = comp == 0 ? Bp : (comp == 1 ? Br : Bt);
            v = B[((size_t)m * (L + 1) + l) * N + g];
        }
        GT[(size_t)m * per + e] = v;
    }
    const size_t pa = (size_t)nchx * TT_GROWS * TT_KC;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < pa; e += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(e / (TT_GROWS * TT_KC)), x = (int)(e % (TT_GROWS * TT_KC));
        const int row = x >> 5, kk = x & 31, comp = row >> 5, g = row & 31;
        const int l = m + 32 * c + tt_loff(kk);
        float v = 0.f;
        if (g < N && l <= L) {
            const float *B = comp == 0 ? Bp : (comp == 1 ? Br : Bt);
            v = B[((size_t)m * (L + 1) + l) * N + g];
        }
        float *hi = AT + (((size_t)m * nchx + c) * 2) * TT_AG_FLOATS;
        const uint32_t off = tt_swz(row, kk) >> 2;
        const float h = round_tf32f(v);
        hi[off] = h;
        hi[TT_AG_FLOATS + off] = round_tf32f(v - h);
    }
}

// incoming basis and moment of B type b
__device__ __forceinline__ int tt_cin(int b) { return b < 2 ? 0 : ((b & 1) ? 2 : 1); }
__device__ __forceinline__ int tt_mom(int b) { return b == 0 ? 0 : (b < 4 ? 1 : (b < 6 ? 2 : 3)); }

// pair product index (tables.cuh numbering) of (outgoing comp, B type), -1 if unused
//   P: 0 P beta -> 0, 2 R gamma -> 10, 3 T gamma -> 9
//   R: 1 P gamma -> 1, 4 R alpha -> 4, 5 T alpha -> 5, 6 R zeta -> 8, 7 T zeta -> 12
//   T: 1 P gamma -> 2, 4 R alpha -> 11, 5 T alpha -> 7, 6 R zeta -> 6, 7 T zeta -> 3
__constant__ signed char tt_prod[3][8] = {{0, -1, 10, 9, -1, -1, -1, -1},
                                          {-1, 1, -1, -1, 4, 5, 8, 12},
                                          {-1, 2, -1, -1, 11, 7, 6, 3}};
// sun-outgoing product index (k_tables' solar-row numbering) of (sun comp, B type), -1 if unused
//   0 P0 Po beta   1 P0 Ro gamma  2 P0 To gamma  3 T0 To zeta
//   4 R0 Ro alpha  5 R0 Po gamma  6 R0 To alpha  7 T0 Ro zeta
__constant__ signed char tt_sun[3][8] = {{0, -1, 1, 2, -1, -1, -1, -1},
                                         {-1, 5, -1, -1, 4, 6, -1, -1},
                                         {-1, -1, -1, -1, -1, -1, 7, 3}};

__device__ __forceinline__ void tt_bar(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// 32x32b TMEM loads of 16 columns without the wait (tcgen05.wait::ld after a batch)
__device__ __forceinline__ void tt_ld16(uint32_t taddr, uint32_t *r)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

size_t tables_tc_ptab_bytes(const Geom &G) { return (size_t)(G.N + G.E) * 26 * TT_PS * 4; }

__global__ void __launch_bounds__(TT_THREADS, 1)
k_tables_tc(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, Geom G, int L, const float *GT,
            const float *AT, const float *Bx, const double *gw, const double *mb, const double *mg, const double *ma,
            const double *mz, float *ops, float *opt, int plain, const float *V, int vp0, long long vstride,
            float *sprod, int *err)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int Kp = tt_kpad(L), nchx = Kp / TT_KC;
    const int N = G.N, E = G.E, nxr = 3 * (E + 1);
    unsigned char *aH = base, *aL = base + TT_A_BYTES, *bH = base + 2 * TT_A_BYTES, *bL = bH + TT_B_BYTES;
    float *ptab = (float *)(base + TT_STAGE);                             // [N + E][26][TT_PS]
    float *smp = ptab + (size_t)(N + E) * 26 * TT_PS;                     // [4][Kp] moments in the chunk order
    uint64_t *bars = (uint64_t *)(((uintptr_t)(smp + 4 * Kp) + 7) & ~(uintptr_t)7);
    uint64_t *afull = bars, *empty = bars + 1, *acc_full = bars + 2, *acc_empty = bars + 3, *fin = bars + 4;
    uint32_t *tslot = (uint32_t *)(bars + 5);
    // abort flags, one per warp group: each is written only by its own group
    // before one of the group's barriers and read only after it, so every
    // thread of a group takes the same branch; a failure in the other group
    // reaches a group through a bounded wait that runs out
    volatile int *abort_main = (volatile int *)(tslot + 1), *abort_epi = abort_main + 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(afull, 1);
        mbar_init(empty, 1);
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, TT_EW * 32);
        mbar_init(fin, 1);
        *abort_main = 0;
        *abort_epi = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    if (warp < TT_MW) {
        // ================= main warps: operands and MMAs =================
        const uint32_t idesc = idesc_tf32(128, 256);
        unsigned gc = 0, ntask = 0;
        bool stop = false;
        for (int tl = blockIdx.x; tl < nt_tasks && !stop; tl += gridDim.x, ++ntask) {
            const TaskDev tk = tasks[t0 + tl];
            const PixDev &d = px[tk.pix];
            const int m = tk.m, Lp = d.L;
            const int aer = d.mom_off >= 0 && d.tau_a > 0.0;
            const int Lm = min(Lp, aer ? d.L_aer : -1);               // last l with a moment
            const int nch = max(1, (Lp + 1 - m + TT_KC - 1) / TT_KC);
            for (int x = tid; x < 4 * nch * TT_KC; x += TT_MW * 32) {
                const int q = x / (nch * TT_KC), kp = x - q * (nch * TT_KC);
                const int l = m + 32 * (kp >> 5) + tt_loff(kp & 31);
                float v = 0.f;
                if (l <= Lm) {
                    const double *mm = q == 0 ? mb : (q == 1 ? mg : (q == 2 ? ma : mz));
                    v = (float)mm[d.mom_off + l];
                }
                smp[q * Kp + kp] = v;
            }
            const float *gtm = GT + (size_t)m * 3 * N * Kp;
            const float *atm = AT + (size_t)m * nchx * 2 * TT_AG_FLOATS;
            const float *bx = Bx + (size_t)tl * (1 + E) * 3 * (L + 1);
            // this thread's inputs of a chunk (K position lane): the Gauss bases
            // of its four incoming slots i = warp + 8 u (B rows 32 type + i) and
            // the sun / zero-weight bases of its four spare A rows, loaded one
            // chunk ahead
            float xg[3][4], xs[4];
            auto load_inputs = [&](int c) {
                const int kp = 32 * c + lane, lq = m + 32 * c + tt_loff(lane);
#pragma unroll
                for (int comp = 0; comp < 3; ++comp)
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int i = warp + 8 * u;
                        xg[comp][u] = i < N ? gtm[((size_t)comp * N + i) * Kp + kp] : 0.f;
                    }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int x = warp + 8 * u;
                    float v = 0.f;
                    if (x < nxr && lq <= L) {
                        const int which = x / 3, cm = x - 3 * which;
                        v = bx[((size_t)which * 3 + cm) * (L + 1) + lq];
                    }
                    xs[u] = v;
                }
            };
            load_inputs(0);
            for (int cc = 0; cc < nch; ++cc, ++gc) {
                // the stage is free once the previous chunk's MMAs completed
                if (gc >= 1 && !mbar_wait(empty, (gc - 1) & 1)) *abort_main = 1;
                tt_bar(2, TT_MW * 32);                                // also: smp written
                if (*abort_main) { stop = true; break; }
                if (tid == 0) {
                    mbar_expect_tx(afull, 2 * TT_AG_FLOATS * 4);
                    bulk_g2s(aH, atm + (size_t)cc * 2 * TT_AG_FLOATS, TT_AG_FLOATS * 4, afull);
                    bulk_g2s(aL, atm + (size_t)cc * 2 * TT_AG_FLOATS + TT_AG_FLOATS, TT_AG_FLOATS * 4, afull);
                }
                const int kp = 32 * cc + lane;
                float mom[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) mom[q] = smp[q * Kp + kp];
                auto put = [&](unsigned char *hi, unsigned char *lo, int row, float v) {
                    const uint32_t off = tt_swz(row, lane);
                    const float h = round_tf32f(v);
                    *reinterpret_cast<float *>(hi + off) = h;
                    *reinterpret_cast<float *>(lo + off) = round_tf32f(v - h);
                };
                // A rows 96..127: the sun and the zero-weight slots
#pragma unroll
                for (int u = 0; u < 4; ++u) put(aH, aL, TT_GROWS + warp + 8 * u, xs[u]);
                // B: row = warp + 8 j = 32 type + i, type = j >> 2, i = warp + 8 (j & 3)
#pragma unroll
                for (int j = 0; j < 32; ++j) put(bH, bL, warp + 8 * j, xg[tt_cin(j >> 2)][j & 3] * mom[tt_mom(j >> 2)]);
                if (cc + 1 < nch) load_inputs(cc + 1);
                // generic-proxy stores made visible to the tensor cores
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tt_bar(2, TT_MW * 32);
                if (tid == 0) {
                    bool ok = mbar_wait(afull, gc & 1);
                    // TMEM drained by the epilogue before the task's first MMA
                    if (ok && cc == 0 && ntask > 0) ok = mbar_wait(acc_empty, (ntask - 1) & 1);
                    if (!ok) {
                        *abort_main = 1;                             // read after the next barrier
                    } else {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t sa_h = smem_u32(aH), sa_l = smem_u32(aL), sb_h = smem_u32(bH), sb_l = smem_u32(bL);
#pragma unroll
                        for (int kk = 0; kk < TT_KC / 8; ++kk) {
                            const uint32_t off = kk * 32, dcol = kk < 2 ? 0u : 256u;
                            const uint32_t acc0 = (cc > 0 || (kk & 1)) ? 1u : 0u;
                            const uint64_t ah = sdesc_sw128(sa_h + off), bh = sdesc_sw128(sb_h + off);
                            umma_tf32(tmem + dcol, ah, bh, idesc, acc0);
                            umma_tf32(tmem + dcol, ah, sdesc_sw128(sb_l + off), idesc, 1u);
                            umma_tf32(tmem + dcol, sdesc_sw128(sa_l + off), bh, idesc, 1u);
                        }
                        umma_commit(empty);
                        if (cc == nch - 1) umma_commit(acc_full);
                    }
                }
            }
        }
        // every MMA this thread issued has completed before TMEM is released
        if (tid == 0) {
            umma_commit(fin);
            if (!mbar_wait(fin, 0)) *abort_main = 1;
        }
    } else {
        // ================= epilogue warps =================
        const int ew = warp - TT_MW;
        const int qd = warp & 3, hf = ew >> 2;
        // TMEM row of this thread: qd < 3 -> Gauss slot lane, comp qd; qd 3 -> spare row lane
        const int x = lane;
        int role = -1, o_row = 0, cm = qd;           // 0: ring slot o_row, 1: the sun
        if (qd < 3) {
            if (lane < N) { role = 0; o_row = lane; }
        } else if (x < nxr) {
            const int which = x / 3;
            cm = x - 3 * which;
            if (which == 0) role = 1;
            else { role = 0; o_row = N + which - 1; }
        }
        const uint32_t tb = tmem + ((uint32_t)(qd * 32) << 16);
        // per lane (incoming Gauss slot i = lane): the operator-tile column of each input block
        int kofs[6], kcs[6];
#pragma unroll
        for (int ib = 0; ib < 6; ++ib) {
            const int cin = ib * N + lane;
            kofs[ib] = (cin >> 5) * 2 * G.NP * 32;
            kcs[ib] = cin & 31;
        }
        const float wi = lane < N ? (float)gw[lane] : 0.f;
        unsigned t = 0;
        for (int tl = blockIdx.x; tl < nt_tasks; tl += gridDim.x, ++t) {
            const bool ok = mbar_wait(acc_full, t & 1);
            if (!ok) *abort_epi = 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            tt_bar(1, TT_EW * 32);
            if (*abort_epi) break;
            const TaskDev tk = tasks[t0 + tl];
            const PixDev &d = px[tk.pix];
            const int m = tk.m, n = d.n_ring;
            // ---- accumulators -> product table (ring slots) and sun products ----
#pragma unroll 1
            for (int bb = 0; bb < 4; ++bb) {
                const int b = hf * 4 + bb;
                uint32_t e[32], od[32];
                tt_ld16(tb + (uint32_t)(b * 32), e);
                tt_ld16(tb + (uint32_t)(b * 32 + 16), e + 16);
                tt_ld16(tb + (uint32_t)(256 + b * 32), od);
                tt_ld16(tb + (uint32_t)(256 + b * 32 + 16), od + 16);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (role == 0) {
                    const int pi = tt_prod[cm][b];
                    if (pi >= 0) {
                        float *pt = ptab + (size_t)(o_row * 26 + pi) * TT_PS;
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (i < N) {
                                const float ev = __uint_as_float(e[i]), ov = __uint_as_float(od[i]);
                                pt[i] = ev + ov;
                                pt[13 * TT_PS + i] = ev - ov;
                            }
                    }
                } else if (role == 1) {
                    const int pi = tt_sun[cm][b];
                    if (pi >= 0) {
                        float *spd = sprod + (size_t)tl * N * 16;
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (i < N) {
                                const float ev = __uint_as_float(e[i]), ov = __uint_as_float(od[i]);
                                spd[i * 16 + pi] = ev + ov;
                                spd[i * 16 + 8 + pi] = ev - ov;
                            }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(acc_empty);                                  // TMEM free for the next task
            tt_bar(1, TT_EW * 32);                                   // product table complete
            // ---- operator entries: a warp per outgoing slot, lane = incoming Gauss slot ----
            const float *Vm = (V && d.vk_n > 1) ? V + (size_t)(tk.pix - vp0) * vstride + (size_t)m * (N + 1) * 2 * G.NR
                                                : nullptr;
            float *Aop = ops + tk.op_off;
            float *Atile = opt ? opt + 2 * tk.op_off : nullptr;
            if (lane < N) {
                // items (outgoing slot o, output Stokes component so): the 12
                // entries of a pair in the rows of so need 3 (I) or 5 (Q, U) of
                // the 13 products, so the 3 n items share the warps evenly
                for (int item = ew; item < 3 * n; item += TT_EW) {
                    const int o = item / 3, so = item - 3 * o;
                    const float *pt = ptab + (size_t)o * 26 * TT_PS + lane;
                    int rowv[6];
#pragma unroll
                    for (int ob = 0; ob < 6; ++ob) rowv[ob] = col_of(G, ob >> 1, ob & 1, o);
                    // Gauss rows with N a multiple of 8 all have row % 8 == o % 8:
                    // the swizzled column of an input block is then fixed per slot
                    const bool uni = o < N && (N & 7) == 0;
                    int swu[6];
#pragma unroll
                    for (int ib = 0; ib < 6; ++ib) swu[ib] = (((kcs[ib] >> 2) ^ (o & 7)) << 2) + (kcs[ib] & 3);
                    auto put_rows = [&](auto so_c) {
                        constexpr int SO = decltype(so_c)::value;
                        // the products this component needs (the others are not read)
                        float S[13], D[13], c[18];
#pragma unroll
                        for (int q = 0; q < 13; ++q) { S[q] = pt[q * TT_PS]; D[q] = pt[(13 + q) * TT_PS]; }
                        pair_coefs(S, D, c);
                        if (SO == 0 && Vm) {                         // the value kernel's table instead
                            c[0] = Vm[(size_t)(1 + lane) * 2 * G.NR + o];
                            c[1] = Vm[(size_t)(1 + lane) * 2 * G.NR + G.NR + o];
                        }
                        if (Atile)
                            put_pair_places([&](int ob, int ib, int q, bool neg) {
                                if ((ob >> 1) != SO) return;
                                const float v = wi * c[q], h = round_tf32f(v), l = round_tf32f(v - h);
                                const int row = rowv[ob], kc = kcs[ib];
                                const int sw = uni ? swu[ib] : ((((kc >> 2) ^ (row & 7)) << 2) + (kc & 3));
                                float *p = Atile + kofs[ib] + row * 32 + sw;
                                p[0] = neg ? -h : h;                 // the split of -v is minus the split of v
                                p[G.NP * 32] = neg ? -l : l;
                            });
                        if (plain)
                            put_pair_places([&](int ob, int ib, int q, bool neg) {
                                if ((ob >> 1) != SO) return;
                                Aop[(size_t)rowv[ob] * G.CIN + ib * N + lane] = neg ? -wi * c[q] : wi * c[q];
                            });
                    };
                    if (so == 0) put_rows(std::integral_constant<int, 0>());
                    else if (so == 1) put_rows(std::integral_constant<int, 1>());
                    else put_rows(std::integral_constant<int, 2>());
                }
            }
            // tile rows no pair writes: unused zero-weight slots and the padding rows COUT .. NP - 1
            if (Atile) {
                const int nz0 = 6 * (G.NR - n), nz = nz0 + (G.NP - G.COUT), nkt = G.CIN / 32;
                for (int y = ew; y < nz * nkt; y += TT_EW) {
                    const int q = y / nkt, kt = y - q * nkt;
                    const int row = q < nz0 ? 6 * N + 6 * (n - N) + q : G.COUT + (q - nz0);
                    float *hi = Atile + (size_t)kt * 2 * G.NP * 32 + (size_t)row * 32;
                    hi[lane] = 0.f;
                    hi[(size_t)G.NP * 32 + lane] = 0.f;
                }
            }
            // and the plain operator's rows of the unused slots (its buffer is
            // not cleared beforehand)
            if (plain) {
                float *Aop = ops + tk.op_off;
                const int nz0 = 6 * (G.NR - n), nkt = G.CIN / 32;
                for (int y = ew; y < nz0 * nkt; y += TT_EW) {
                    const int q = y / nkt, kt = y - q * nkt;
                    Aop[(size_t)(6 * N + 6 * (n - N) + q) * G.CIN + kt * 32 + lane] = 0.f;
                }
            }
            tt_bar(1, TT_EW * 32);                                   // table reads done
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && (*abort_main || *abort_epi)) atomicExch(err, OCRT_ERR_DEVICE);
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

size_t tables_tc_smem_bytes(const Geom &G, int L)
{
    return 1024 + (size_t)TT_STAGE + tables_tc_ptab_bytes(G) + 16 * (size_t)tt_kpad(L) + 64;
}

size_t tables_tc_gt_floats(int N, int M, int L) { return (size_t)(M + 1) * 3 * N * tt_kpad(L); }

size_t tables_tc_at_floats(int M, int L) { return (size_t)(M + 1) * (tt_kpad(L) / TT_KC) * 2 * TT_AG_FLOATS; }

bool tables_tc_supported(const Geom &G, int L)
{
    return G.N <= 32 && 3 * (G.E + 1) <= 32 && G.CIN % 32 == 0 && tables_tc_smem_bytes(G, L) <= 227 * 1024;
}

int tables_tc_threads() { return TT_THREADS; }

cudaError_t tables_tc_init()
{
    return cudaFuncSetAttribute(k_tables_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}
