// tc_gemm.cu — multiple-scattering source contraction on the tcgen05 tensor
// cores (rt_sos_operator.c:206-424 for modes without a molecular term, m > 2).
//
// Per item: one (task, 128-level tile).  D[128 levels][NP outputs] (FP32 in
// TMEM) = F[128 levels][6N inputs] x Aop^T, K = 6N swept in 32-element tiles
// (one 128-byte swizzle row).  Each K tile is brought in by TMA into a
// SWIZZLE_128B K-major layout, split in place into tf32 hi and lo parts, and
// contracted with three tcgen05.mma.kind::tf32 passes (hi*hi + hi*lo + lo*hi),
// which carries FP32-level accuracy on the TF32 tensor path.  The epilogue
// reads TMEM with tcgen05.ld and writes J = x_k * D.
//
// Every wait is time-bounded: on timeout the CTA records an error word,
// drains its own in-flight copies with a second bounded wait, frees TMEM and
// returns.
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"

#define TC_M 128
#define TC_KT 32
#define TC_THREADS 256
#define TC_TMEM_COLS 256
#define TC_WAIT_NS 2000000000ull

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Wait for phase `parity` of a barrier; false after TC_WAIT_NS nanoseconds.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer() - t0 > TC_WAIT_NS) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: rows of
// 128 B, 8-row groups 1024 B apart (SBO), LBO unused, version 1 (sm_100 family).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor: D F32, A/B TF32, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

} // namespace

// Split a raw FP32 tile in place into a tf32 head (kept in place) and a tf32
// tail (written to `lo`), each rounded to nearest, so x = hi + lo to ~2^-22
// relative and the MMA's own tf32 reading of either part is exact.
__device__ __forceinline__ uint32_t round_tf32(uint32_t u)
{
    return (u + 0x1000u) & 0xFFFFE000u;
}

__device__ __forceinline__ void split_tf32(uint32_t *hi, uint32_t *lo, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t u = hi[i];
        const uint32_t h = round_tf32(u);
        hi[i] = h;
        lo[i] = round_tf32(__float_as_uint(__uint_as_float(u) - __uint_as_float(h)));
    }
}

// Persistent form: a grid of about one CTA per SM pulls (task, 128-row tile)
// items from a per-order counter.  TMEM and the barriers are set up once per
// CTA; K tiles are numbered globally across the CTA's items (stage g & 1, use
// g >> 1), so thread 0 streams the next item's first two tiles in while the
// current item's epilogue drains TMEM.
//
// ADJ = false: forward source.  Rows = levels of one task's field F (map over
//   the wave's F), B operand = the task's operator Aop [NP][CIN], K = CIN,
//   epilogue J[k][c] = x_k D[k][c] for c < COUT; items = active list x tiles.
// ADJ = true: transposed source of the adjoint.  Rows = the ncot adjoint
//   fields of one task stacked (ncot * K rows of muJ), B operand = the task's
//   transposed operator AopT [CIN][KP] (KP = COUT rounded up to 32), K = KP,
//   epilogue a[row][cin] = x_k D[row][cin] for cin < CIN; items = every task of
//   the wave x tiles, skipped when none of the task's rows is still active.
template <bool ADJ>
__device__ __forceinline__ void source_tc_body(const CUtensorMap *mapF, const CUtensorMap *mapA, const BatchBufs &B,
                                               const WaveBufs &W, const AdjBufs &AB, const Geom &G, int t0, int it,
                                               int mtiles, int nw)
{
    extern __shared__ unsigned char smem_raw[];
    const int NB = ADJ ? G.CIN : G.NP;                  // MMA N (B operand rows)
    const int NKT = ADJ ? ((G.COUT + TC_KT - 1) / TC_KT) : G.CIN / TC_KT;
    const uint32_t A_BYTES = TC_M * TC_KT * 4, B_BYTES = (uint32_t)NB * TC_KT * 4;
    const uint32_t STAGE = 2 * A_BYTES + 2 * B_BYTES;
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(base + 2 * STAGE);     // full[2], empty[2], done
    uint32_t *tslot = (uint32_t *)(bars + 5);
    int *abort_flag = (int *)(tslot + 1);
    int *slot = abort_flag + 1;                          // item ring [2]: task index * mtiles + tile, or -1
    const int tid = threadIdx.x, warp = tid >> 5;
    const int n_items = (ADJ ? nw : B.active_cnt[it - 1]) * mtiles;
    const int *alist = ADJ ? nullptr : B.alist[it & 1];
    int *counter = ADJ ? &AB.awork[it] : &B.work[it * 4 + 0];

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    uint64_t *full = bars, *empty = bars + 2, *done = bars + 4;

    auto task_of = [&](int li) -> int { return ADJ ? li : alist[li]; };
    // Thread 0 only: next item with work, or -1.
    auto fetch = [&]() -> int {
        for (;;) {
            const int item = atomicAdd(counter, 1);
            if (item >= n_items) return -1;
            const int li = item / mtiles, mt = item - li * mtiles;
            const int tl = task_of(li);
            const TaskDev tk = B.tasks[t0 + tl];
            if (ADJ) {
                if (mt * TC_M >= AB.ncot * tk.K) continue;
                bool any = false;
                for (int r = 0; r < AB.ncot; ++r) any |= AB.st[tl * AB.ncot + r].active != 0;
                if (any) return item;
            } else if (mt * TC_M <= B.px[tk.pix].nt) {
                return item;
            }
        }
    };
    // Thread 0 only: TMA loads of K tile kt of `item` into stage s.
    auto issue = [&](int item, int kt, int s) {
        const int li = item / mtiles, mt = item - li * mtiles;
        const int tl = task_of(li);
        const TaskDev tk = B.tasks[t0 + tl];
        const int rowF = ADJ ? (int)(tk.fld_off * AB.ncot / G.LDC) + mt * TC_M : (int)(tk.fld_off / G.LDC) + mt * TC_M;
        const int rowA = ADJ ? tl * G.CIN : (int)(tk.op_off / G.CIN);
        unsigned char *sp = base + (size_t)s * STAGE;
        mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
        tma_load_2d(sp, mapF, &full[s], kt * TC_KT, rowF);
        tma_load_2d(sp + 2 * A_BYTES, mapA, &full[s], kt * TC_KT, rowA);
    };

    int inflight[2] = {0, 0};          // thread 0: stage holds an unconsumed load
    if (tid == 0) {
        for (int i = 0; i < 5; ++i) mbar_init(&bars[i], 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int first = fetch();
        slot[0] = first;
        slot[1] = -1;
        if (first >= 0) {
            issue(first, 0, 0); inflight[0] = 1;
            issue(first, 1, 1); inflight[1] = 1;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    constexpr uint32_t IDESC_BASE = idesc_tf32(TC_M, 16);    // N filled in below
    const uint32_t idesc = (IDESC_BASE & ~(0x3Fu << 17)) | ((uint32_t)(NB >> 3) << 17);
    uint32_t g = 0;                    // global K-tile sequence number of this CTA
    uint32_t ph_done = 0;
    bool ok = true, done_pending = false;
    for (int j = 0;; ++j) {
        __syncthreads();
        const int item = slot[j & 1];
        if (item < 0) break;
        const int li = item / mtiles, mt = item - li * mtiles;
        const TaskDev tk = B.tasks[t0 + task_of(li)];
        const PixDev &d = B.px[tk.pix];
        const int nt = d.nt, k0 = mt * TC_M;
        for (int kt = 0; kt < NKT; ++kt, ++g) {
            const int s = g & 1;
            const uint32_t use = g >> 1;
            if (!mbar_wait(&full[s], use & 1)) atomicExch(abort_flag, 1);
            __syncthreads();
            if (*abort_flag) { ok = false; break; }
            if (tid == 0) inflight[s] = 0;
            unsigned char *sp = base + (size_t)s * STAGE;
            uint32_t *ahi = (uint32_t *)sp, *alo = (uint32_t *)(sp + A_BYTES);
            uint32_t *bhi = (uint32_t *)(sp + 2 * A_BYTES), *blo = (uint32_t *)(sp + 2 * A_BYTES + B_BYTES);
            split_tf32(ahi, alo, TC_M * TC_KT);
            split_tf32(bhi, blo, NB * TC_KT);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa_hi = smem_u32(ahi), sa_lo = smem_u32(alo);
                const uint32_t sb_hi = smem_u32(bhi), sb_lo = smem_u32(blo);
#pragma unroll
                for (int kk = 0; kk < TC_KT / 8; ++kk) {
                    const uint32_t off = kk * 32;     // 8 tf32 = 32 bytes along the swizzled row
                    const uint64_t ah = sdesc_sw128(sa_hi + off), al = sdesc_sw128(sa_lo + off);
                    const uint64_t bh = sdesc_sw128(sb_hi + off), bl = sdesc_sw128(sb_lo + off);
                    umma_tf32(tmem, ah, bh, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
                    umma_tf32(tmem, ah, bl, idesc, 1u);
                    umma_tf32(tmem, al, bh, idesc, 1u);
                }
                umma_commit(&empty[s]);
                if (kt == NKT - 1) { umma_commit(done); done_pending = true; }
                // Refill this stage with K tile g + 2 (this item's, or the next item's).
                int nitem = item, nkt = kt + 2;
                if (nkt >= NKT) {
                    nkt -= NKT;
                    if (nkt == 0) slot[(j + 1) & 1] = fetch();
                    nitem = slot[(j + 1) & 1];
                }
                if (nitem >= 0) {
                    if (!mbar_wait(&empty[s], use & 1)) {
                        atomicExch(abort_flag, 1);
                    } else {
                        issue(nitem, nkt, s);
                        inflight[s] = 1;
                    }
                }
            }
        }
        if (!ok) break;
        if (mbar_wait(done, ph_done)) {
            ph_done ^= 1;
            done_pending = false;
        } else {
            atomicExch(abort_flag, 1);
        }
        __syncthreads();
        if (*abort_flag) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // Epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (one row each);
        // warps 0-3 take the even 16-column chunks, warps 4-7 the odd ones.
        const int lane = tid & 31, q = warp & 3, half = warp >> 2;
        const int row = k0 + q * 32 + lane;
        int k;
        bool live;
        float *out;
        int ncols;
        if (ADJ) {
            live = row < AB.ncot * tk.K;
            k = live ? row % tk.K : 0;
            out = AB.AF + (size_t)tk.fld_off * AB.ncot + (size_t)row * G.LDC;
            ncols = G.CIN;
        } else {
            live = row <= nt;
            k = row;
            out = W.J + tk.fld_off + (size_t)row * G.LDC;
            ncols = G.COUT;
        }
        const float x = live ? (float)B.xd[d.lev_off + k] : 0.f;
        for (int cb = half; cb < NB / 16; cb += 2) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cb * 16), v);
            if (live) {
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) {
                    const int c = cb * 16 + jj;
                    if (c < ncols) out[c] = x * v[jj];
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(B.err, OCRT_ERR_DEVICE);
            // drain this CTA's own copies and MMAs still in flight (bounded)
            for (int s = 0; s < 2; ++s)
                if (inflight[s]) mbar_wait(&full[s], ((g + (s != (int)(g & 1))) >> 1) & 1);
            if (!done_pending) umma_commit(done);
            mbar_wait(done, ph_done);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
k_source_tc(const __grid_constant__ CUtensorMap mapF, const __grid_constant__ CUtensorMap mapA,
            BatchBufs B, WaveBufs W, Geom G, int t0, int it, int mtiles)
{
    AdjBufs none{};
    source_tc_body<false>(&mapF, &mapA, B, W, none, G, t0, it, mtiles, 0);
}

// Transposed contraction of the adjoint for adjoint order `it` (work counter
// AB.awork[it]).
__global__ void __launch_bounds__(TC_THREADS, 1)
k_adj_source_tc(const __grid_constant__ CUtensorMap mapJ, const __grid_constant__ CUtensorMap mapAT,
                BatchBufs B, WaveBufs W, AdjBufs AB, Geom G, int t0, int it, int mtiles, int nw)
{
    source_tc_body<true>(&mapJ, &mapAT, B, W, AB, G, t0, it, mtiles, nw);
}

size_t tc_smem_bytes(const Geom &G)
{
    return 1024 + 2 * (2 * (size_t)TC_M * TC_KT * 4 + 2 * (size_t)G.NP * TC_KT * 4) + 128;
}

size_t tc_adj_smem_bytes(const Geom &G)
{
    return 1024 + 2 * (2 * (size_t)TC_M * TC_KT * 4 + 2 * (size_t)G.CIN * TC_KT * 4) + 128;
}

bool tc_adj_supported(const Geom &G)
{
    return (G.CIN % 16) == 0 && G.CIN <= 256 && tc_adj_smem_bytes(G) <= 227 * 1024;
}

bool tc_supported(const Geom &G)
{
    return (G.CIN % TC_KT) == 0 && G.CIN / TC_KT >= 2 && G.NP <= 256 && G.NP % 16 == 0 &&
           tc_smem_bytes(G) <= 227 * 1024;
}
