// scan_tma.cu — the order step's transport scan fed by the tensor memory
// accelerator (rt_layer_transport.c:107-208 for the recurrences,
// rt_surface_boundary.c:137-208 for the boundary condition, rt_solver.c:
// 2178-2197 for the convergence test).
//
// Per task the scan reads, for every level, the source J and the FP32 head of
// the order total, and for every layer the three transport weights of each
// ring slot; it writes the order field F and the new total.  k_scan and
// k_scan4 move those inputs with per-thread cp.async copies of 4 or 16 bytes.
// Here one producer thread moves them as whole level chunks:
//
//   * a chunk is CH consecutive levels of one transport direction h (upward
//     columns walk from the bottom, downward ones from the top);
//   * the Gauss columns of direction h in a level row are three runs of N
//     floats (Stokes s = 0, 1, 2 at s*2N + h*N), which a 4-D tensor map over
//     the field buffer ({N, 2, 3, rows}) fetches as one box {N, 1, 3, CH};
//   * the 6E zero-weight columns come as one 2-D box {ZW, CH} at column 6N;
//   * the weights come from the quad table Cq (per layer, per quad of ring
//     slots, four T then four Ca then four Cb), one 2-D box {3*NRq, CH};
//   * both directions' chunks of one step share a ring stage and complete on
//     the stage's mbarrier; NS stages are in flight.
//
// Column threads read everything from shared memory (conflict-free: the
// threads of a warp hold consecutive slots), run the recurrence, and store F
// and the total with coalesced 4-byte stores.  Per column the arithmetic is
// that of k_scan in the same order, so all scans give identical results.
//
// Every mbarrier wait is bounded by %globaltimer; after a timeout the block
// records OCRT_ERR_DEVICE, stops, waits (bounded) for the copies it issued
// and returns.
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"
#include "tcgen05.cuh"

using namespace tcg;

namespace {

// Shared-memory carve-up of one ring stage: for each direction the Gauss
// J box, the Gauss total box, the zero-weight J and total boxes and the
// weight box, each 128-byte aligned.
struct StmLayout {
    uint32_t jg, tg, jz, tz, cf, dir, stage;
};

__host__ __device__ inline uint32_t al128(uint32_t v) { return (v + 127u) & ~127u; }

// Per direction: the source J's Gauss and zero-weight boxes, the order
// total's (only where every level keeps its total, G.tot_all; otherwise the
// two output rows of the total are read directly) and the weight box.
__host__ __device__ inline StmLayout stm_layout(const Geom &G, int CH)
{
    StmLayout L;
    const uint32_t gb = al128((uint32_t)(CH * 3 * G.N * 4));
    const uint32_t zb = al128((uint32_t)(CH * scan_tma_zw(G) * 4));
    const uint32_t cb = al128((uint32_t)(CH * scan_tma_cw(G) * 4));
    if (G.tot_all) {
        L.jg = 0; L.tg = gb; L.jz = 2 * gb; L.tz = 2 * gb + zb; L.cf = 2 * gb + 2 * zb;
        L.dir = 2 * gb + 2 * zb + cb;
    } else {
        L.jg = 0; L.jz = gb; L.cf = gb + zb; L.tg = L.tz = 0;
        L.dir = gb + zb + cb;
    }
    L.stage = 2 * L.dir;
    return L;
}

// bytes the tensor copies of one stage deliver (boxes are always whole, the
// out-of-range part zero-filled), with or without the total's boxes
__host__ __device__ inline uint32_t stm_stage_tx(const Geom &G, int CH, bool tot = true)
{
    const int nt = tot ? 2 : 1;
    return 2u * (uint32_t)CH * 4u * (uint32_t)(nt * 3 * G.N + nt * scan_tma_zw(G) + scan_tma_cw(G));
}

__device__ __forceinline__ void tma2(void *dst, const CUtensorMap *m, int x, int y, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                 "[%0], [%1, {%2, %3}], [%4];"
                 ::"r"(smem_u32(dst)), "l"((uint64_t)m), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tma4(void *dst, const CUtensorMap *m, int c0, int c1, int c2, int c3, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                 "[%0], [%1, {%2, %3, %4, %5}], [%6];"
                 ::"r"(smem_u32(dst)), "l"((uint64_t)m), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
                 : "memory");
}

// Block maxima of (a, b), valid in thread 0.  One barrier: the caller
// passes a barrier between a thread 0 read of red and the next call.
__device__ inline float2 stm_maxf2(float a, float b, float2 *red)
{
    for (int o = 16; o > 0; o >>= 1) {
        a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = make_float2(a, b);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 1; i < nw; ++i) { a = fmaxf(a, red[i].x); b = fmaxf(b, red[i].y); }
    }
    return make_float2(a, b);
}

} // namespace

size_t scan_tma_smem_bytes(const Geom &G, int CH, int NS)
{
    return (size_t)stm_layout(G, CH).stage * NS + 128 /* alignment slack */ + 256 /* barriers */;
}

template <int CH, int NS>
__global__ void __launch_bounds__(256, 3) k_scan_tma(BatchBufs B, WaveBufs W, Geom G, int t0, int it,
                                                     const __grid_constant__ ScanMaps M)
{
    extern __shared__ unsigned char stm_raw[];
    __shared__ float2 redf2[32];
    __shared__ int item_nx, abort_raw;
    volatile int &abort_s = abort_raw;
    unsigned char *base = (unsigned char *)(((uintptr_t)stm_raw + 127) & ~(uintptr_t)127);
    const StmLayout Ly = stm_layout(G, CH);
    uint64_t *full = (uint64_t *)(base + (size_t)Ly.stage * NS), *empty = full + NS;
    const int tid = threadIdx.x, lane = tid & 31, nthr = blockDim.x;
    const int ncw = nthr / 32 - 1;                       // column warps; the last warp's lane 0 produces
    const bool producer = tid == nthr - 32;
    const int N = G.N, NR = G.NR, ZW = scan_tma_zw(G), CW = scan_tma_cw(G);
    const uint32_t TX = stm_stage_tx(G, CH), TXJ = stm_stage_tx(G, CH, false);
    const int n_items = B.active_cnt[it - 1];
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], ncw); }
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (producer) {
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&M.jg) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&M.tg) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&M.jz) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&M.tz) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&M.cq) : "memory");
    }
    // column of this thread
    const int c = tid;
    int s = 0, h = 0, g = 0;
    const bool col = c < G.COUT;
    if (col) decode_col(G, c, s, h, g);
    // offsets of this column's values inside a direction block of a stage
    const bool gauss = g < N;
    const uint32_t voff = gauss ? (uint32_t)(s * N + g) * 4u : (uint32_t)(c - 6 * N) * 4u;
    const uint32_t vrow = gauss ? (uint32_t)(3 * N) * 4u : (uint32_t)ZW * 4u;
    const uint32_t cofs = (uint32_t)(((g >> 2) * 12 + (g & 3)) * 4), crow = (uint32_t)CW * 4u;
    uint32_t issued = 0, consumed = 0;                   // chunks issued / consumed by this CTA (ring position)
    // The producer fetches the items: the first one here, each next one as
    // soon as the current item's chunks are all issued, and it then issues
    // the next item's first chunks into the ring slots the consumers free
    // while they finish the current item (run-ahead), so a new item's first
    // copies are in flight before the consumers reach it.  pre = chunks of
    // the current item already issued that way (producer only).
    int pre = 0;
    if (producer) item_nx = atomicAdd(&B.work[it * 4 + 2], 1);
    __syncthreads();
    for (;;) {
        // item_nx was written before the previous item's reduction barrier and
        // is rewritten only after this item's boundary-condition barrier
        const int item_c = __syncthreads_or(abort_s != 0) ? n_items : item_nx;
        if (item_c >= n_items) break;
        const int tl = B.alist[it & 1][item_c], tg = t0 + tl;
        const TaskState st = B.state[tg];
        const TaskDev tk = B.tasks[tg];
        const PixDev &d = B.px[tk.pix];
        const int nt = d.nt, nq = (nt + CH) / CH;        // ceil((nt + 1) / CH) chunks of steps j = 0 .. nt
        const int row0 = (int)(tk.fld_off / G.LDC), lay0 = (int)(d.coef_off / NR);
        // ---- producer: issue chunk q of a task (levels nt_, first field row
        // row0_, first layer lay0_) into ring position issued ----
        auto issue_of = [&](int q, int nt_, int row0_, int lay0_) -> bool {
            const uint32_t pos = issued, sl = pos % NS;
            if (pos >= (uint32_t)NS && !mbar_wait(&empty[sl], ((pos / NS) - 1) & 1)) return false;
            unsigned char *stg = base + (size_t)sl * Ly.stage;
            // the total's boxes only where every level keeps it
            const bool wt = G.tot_all != 0;
            mbar_expect_tx(&full[sl], wt ? TX : TXJ);
#pragma unroll
            for (int dd = 0; dd < 2; ++dd) {
                unsigned char *db = stg + dd * Ly.dir;
                const int r = dd == 0 ? nt_ - q * CH - CH + 1 : q * CH;      // first level row of the box
                const int ly = dd == 0 ? r : q * CH - 1;                      // first layer of the box
                tma4(db + Ly.jg, &M.jg, 0, dd, 0, row0_ + r, &full[sl]);
                if (wt) tma4(db + Ly.tg, &M.tg, 0, dd, 0, row0_ + r, &full[sl]);
                tma2(db + Ly.jz, &M.jz, 6 * N, row0_ + r, &full[sl]);
                if (wt) tma2(db + Ly.tz, &M.tz, 6 * N, row0_ + r, &full[sl]);
                tma2(db + Ly.cf, &M.cq, 0, lay0_ + ly, &full[sl]);
            }
            issued = pos + 1;
            return true;
        };
        auto issue = [&](int q) -> bool { return issue_of(q, nt, row0, lay0); };
        const int npre = nq < NS ? nq : NS;
        if (producer) {
            for (int q = pre; q < npre; ++q)
                if (!issue(q)) { abort_s = 1; break; }
        }
        // ---- boundary condition from the previous order's field (as in k_scan) ----
        const bool valid = col && g < d.n_ring;
        float *F = W.F + tk.fld_off;
        float *Tot = W.Tot + tk.fld_off;
        float *tl0 = W.Ttl + tot_tail_off(tk, G, 0, c), *tlN = W.Ttl + tot_tail_off(tk, G, nt, c);
        float lo0 = 0.f, loN = 0.f, hd0 = 0.f, hdN = 0.f;
        float bc = 0.f;
        const bool water = d.medium == 1;
        if (valid) {
            lo0 = *tl0; loN = *tlN;
            if (!G.tot_all) { hd0 = Tot[c]; hdN = Tot[(size_t)nt * G.LDC + c]; }
            if ((water && h == 1) || (!water && h == 0 && d.surf_on)) {
                if (water || d.rough) {
                    // water: internal reflection of the previous order's upward field at the
                    // top; atmosphere: rough reflection of the downward field at the bottom
                    const float *Rm = W.srf + tk.srf_off + (size_t)g * N * 9 + s * 3;
                    const float *pwm = B.pw + (tk.m == 0 ? 0 : N);
                    const float *Fr = water ? F : F + (size_t)nt * G.LDC;
                    const int hin = water ? 0 : 1;
                    float acc = 0.f;
                    for (int i = 0; i < N; ++i) {
                        const float *Ri = Rm + (size_t)i * 9;
                        acc += pwm[i] * (Ri[0] * Fr[col_of(G, 0, hin, i)] + Ri[1] * Fr[col_of(G, 1, hin, i)] +
                                         Ri[2] * Fr[col_of(G, 2, hin, i)]);
                    }
                    bc = acc;
                } else {
                    const float *Fbot = F + (size_t)nt * G.LDC;
                    const float *MF = B.frs + ((size_t)tk.pix * NR + g) * 9 + s * 3;
                    bc = MF[0] * Fbot[col_of(G, 0, 1, g)] + MF[1] * Fbot[col_of(G, 1, 1, g)] +
                         MF[2] * Fbot[col_of(G, 2, 1, g)];
                }
            }
        }
        __syncthreads();   // every boundary value is read before the first F store
        float mi = 0.f, mt = 0.f;
        int bad = 0;
        if (producer) {
            for (int q = npre > pre ? npre : pre; q < nq && !abort_s; ++q)
                if (!issue(q)) { abort_s = 1; break; }
            // run-ahead: the next item and its first chunks; the slots they
            // take are freed by the consumers' progress through this item,
            // which needs nothing more from the producer
            pre = 0;
            item_nx = abort_s ? n_items : atomicAdd(&B.work[it * 4 + 2], 1);
            if (item_nx < n_items) {
                const TaskDev tn = B.tasks[t0 + B.alist[it & 1][item_nx]];
                const PixDev &dn = B.px[tn.pix];
                const int nqn = (dn.nt + CH) / CH, npn = nqn < NS ? nqn : NS;
                const int r0n = (int)(tn.fld_off / G.LDC), l0n = (int)(dn.coef_off / NR);
                for (int q = 0; q < npn && !abort_s; ++q) {
                    if (!issue_of(q, dn.nt, r0n, l0n)) { abort_s = 1; break; }
                    pre = q + 1;
                }
            }
        } else if (tid < ncw * 32) {
            float I = (water ? h == 1 : h == 0) ? bc : 0.f, Jp = 0.f;
            for (int q = 0; q < nq; ++q) {
                const uint32_t pos = consumed, sl = pos % NS;
                const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[sl], (pos / NS) & 1));
                if (!ok) { abort_s = 1; break; }
                consumed = pos + 1;
                const unsigned char *db = base + (size_t)sl * Ly.stage + h * Ly.dir;
                const unsigned char *vj = db + (gauss ? Ly.jg : Ly.jz) + voff;
                const unsigned char *vt = db + (gauss ? Ly.tg : Ly.tz) + voff;
                const unsigned char *vc = db + Ly.cf + cofs;
                if (valid) {
#pragma unroll 4
                    for (int jj = 0; jj < CH; ++jj) {
                        const int j = q * CH + jj;
                        if (j > nt) break;
                        const int r = h == 0 ? CH - 1 - jj : jj;   // box row of level k (and of its layer)
                        const int k = h == 0 ? nt - j : j;
                        const float jv = *(const float *)(vj + r * vrow);
                        if (j > 0) {
                            const float *cw = (const float *)(vc + r * crow);
                            I = cw[0] * I + cw[4] * jv + cw[8] * Jp;
                        }
                        Jp = jv;
                        const size_t o = (size_t)k * G.LDC + c;
                        F[o] = I;
                        if (k == 0 || k == nt) {
                            const float ov = G.tot_all ? *(const float *)(vt + r * vrow) : (k == 0 ? hd0 : hdN);
                            const float2 td = df_add(make_float2(ov, k == 0 ? lo0 : loN), I);
                            Tot[o] = td.x;
                            *(k == 0 ? tl0 : tlN) = td.y;
                            mt = fmaxf(mt, fabsf(td.x));
                        } else if (G.tot_all) {
                            Tot[o] = *(const float *)(vt + r * vrow) + I;
                        }
                        mi = fmaxf(mi, fabsf(I));
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[sl]);
            }
            bad = valid && !isfinite(I);
        }
        if (bad) atomicExch(B.err, OCRT_ERR_NONFINITE);
        const float2 mm = stm_maxf2(mi, mt, redf2);
        if (tid == 0 && !abort_s) {
            TaskState ns = st;
            ns.orders = it;
            ns.resid = mm.y > 0.f ? (double)(mm.x / mm.y) : 0.0;
            if (ns.resid < d.tol) { ns.converged = 1; ns.active = 0; }
            else if (it >= d.max_orders) ns.active = 0;
            B.state[tg] = ns;
            if (ns.active) queue_next(B, it + 1, tl, tk.has_mol, nt + 1);
        }
        if (abort_s) break;
    }
    __syncthreads();
    if (abort_s) {
        if (tid == 0) atomicExch(B.err, OCRT_ERR_DEVICE);
        // copies issued but not consumed still land in this block's shared
        // memory: wait for them (bounded) before the block exits
        // (the last NS issued positions hold one phase of each stage)
        if (producer)
            for (uint32_t p = issued > (uint32_t)NS ? issued - NS : 0; p < issued; ++p)
                (void)mbar_wait(&full[p % NS], (p / NS) & 1);
    }
}

// ===========================================================================
// The adjoint's transposed transport (k_adj_scan in adjoint.cu: the same
// recurrences run the other way, nu = a + T nu', muJ = Ca nu + Cb nu', the
// adjoint total and its convergence norms) fed the same way.  Persistent:
// blocks pull (task, group of up to ADJ_RB cotangent rows) items of the
// order's active-task list (k_compact_adj) from a work counter, and a task
// with a row still active after the order is flagged for the next list; per
// ring stage and direction
// the adjoint field and the adjoint total boxes of every active row and the
// weight rows of the chunk's CH levels plus one (the transposed recurrence
// reads T and Cb of one layer and Ca of the next).  Per column and row the
// arithmetic is k_adj_scan's, in the same order.
// ===========================================================================
namespace {

struct AstLayout {
    uint32_t g, z, cf, dir, stage;   // one row's Gauss box, zero-weight box; weights; per direction
};

__host__ __device__ inline AstLayout ast_layout(const Geom &G, int CH)
{
    AstLayout L;
    L.g = al128((uint32_t)(CH * 3 * G.N * 4));
    L.z = al128((uint32_t)(CH * scan_tma_zw(G) * 4));
    L.cf = al128((uint32_t)((CH + 1) * scan_tma_cw(G) * 4));
    // per active row: field Gauss, total Gauss, field zero-weight, total zero-weight
    L.dir = ADJ_RB * (2 * L.g + 2 * L.z) + L.cf;
    L.stage = 2 * L.dir;
    return L;
}

} // namespace

size_t adj_scan_tma_smem_bytes(const Geom &G, int CH, int NS)
{
    return (size_t)ast_layout(G, CH).stage * NS + 128 + 256;
}

template <int CH, int NS>
__global__ void __launch_bounds__(256, 2) k_adj_scan_tma(BatchBufs B, AdjBufs A, Geom G, int t0, int j,
                                                         const __grid_constant__ AdjScanMaps M)
{
    extern __shared__ unsigned char ast_raw[];
    __shared__ float2 redr[32][ADJ_RB];
    __shared__ int item_s, abort_raw;
    volatile int &abort_s = abort_raw;
    unsigned char *base = (unsigned char *)(((uintptr_t)ast_raw + 127) & ~(uintptr_t)127);
    const AstLayout Ly = ast_layout(G, CH);
    uint64_t *full = (uint64_t *)(base + (size_t)Ly.stage * NS), *empty = full + NS;
    const int tid = threadIdx.x, lane = tid & 31, nthr = blockDim.x;
    const int ncw = nthr / 32 - 1;
    const bool producer = tid == nthr - 32;
    const int N = G.N, NR = G.NR, ZW = scan_tma_zw(G), CW = scan_tma_cw(G);
    const int nrg = (A.ncot + ADJ_RB - 1) / ADJ_RB;
    // items: (task of this order's active list, group of ADJ_RB rows)
    const int n_items = A.lcnt[j] * nrg;
    const int *lst = A.alist[j & 1];
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], ncw); }
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    uint32_t issued = 0, consumed = 0;                   // ring positions issued / consumed by this CTA
    __syncthreads();
    for (;;) {
    __syncthreads();
    if (tid == 0) item_s = abort_s ? n_items : atomicAdd(&A.swork[j], 1);
    __syncthreads();
    if (item_s >= n_items) break;
    const int li = item_s / nrg;
    const int tl = lst[li], r0 = (item_s - li * nrg) * ADJ_RB, tg = t0 + tl;
    const int nr = min(ADJ_RB, A.ncot - r0);
    bool act[ADJ_RB];
    int nact = 0;
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) {
        act[q] = q < nr && A.st[tl * A.ncot + r0 + q].active;
        nact += act[q] ? 1 : 0;
    }
    if (nact == 0) continue;                              // block-uniform
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt, nq = (nt + CH) / CH;
    // first level row of each active row's adjoint field: (fld_off ncot + r K LDC) / LDC
    int rrow[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q)
        rrow[q] = (int)((tk.fld_off * A.ncot) / G.LDC) + (r0 + (q < nr ? q : 0)) * tk.K;
    const int lay0 = (int)(d.coef_off / NR);
    const uint32_t TX = 2u * (uint32_t)CH * 4u * (uint32_t)nact * (uint32_t)(2 * 3 * N + 2 * ZW) +
                        2u * (uint32_t)(CH + 1) * 4u * (uint32_t)CW;
    auto issue = [&](int q) -> bool {
        const uint32_t pos = issued, sl = pos % NS;
        if (pos >= (uint32_t)NS && !mbar_wait(&empty[sl], ((pos / NS) - 1) & 1)) return false;
        unsigned char *stg = base + (size_t)sl * Ly.stage;
        mbar_expect_tx(&full[sl], TX);
#pragma unroll
        for (int dd = 0; dd < 2; ++dd) {
            unsigned char *db = stg + dd * Ly.dir;
            // direction 0 (upward columns) walks k = 0 .. nt, direction 1 k = nt .. 0
            const int r = dd == 0 ? q * CH : nt - q * CH - CH + 1;       // first level of the box
            const int ly = dd == 0 ? q * CH - 1 : nt - q * CH - CH;      // first layer of the weight box
            int slot = 0;
#pragma unroll
            for (int rq = 0; rq < ADJ_RB; ++rq) {
                if (!act[rq]) continue;
                unsigned char *rb = db + (size_t)slot * (2 * Ly.g + 2 * Ly.z);
                tma4(rb, &M.ag, 0, dd, 0, rrow[rq] + r, &full[sl]);
                tma4(rb + Ly.g, &M.tg, 0, dd, 0, rrow[rq] + r, &full[sl]);
                tma2(rb + 2 * Ly.g, &M.az, 6 * N, rrow[rq] + r, &full[sl]);
                tma2(rb + 2 * Ly.g + Ly.z, &M.tz, 6 * N, rrow[rq] + r, &full[sl]);
                ++slot;
            }
            tma2(db + ADJ_RB * (2 * Ly.g + 2 * Ly.z), &M.cq, 0, lay0 + ly, &full[sl]);
        }
        issued = pos + 1;
        return true;
    };
    if (producer) {
        for (int q = 0; q < (nq < NS ? nq : NS); ++q)
            if (!issue(q)) { abort_s = 1; break; }
    }
    // column of this thread
    const int c = tid;
    int s = 0, h = 0, g = 0;
    const bool col = c < G.COUT;
    if (col) decode_col(G, c, s, h, g);
    const bool valid = col && g < d.n_ring;
    const bool gauss = g < N;
    const uint32_t voff = gauss ? (uint32_t)(s * N + g) * 4u : (uint32_t)(c - 6 * N) * 4u;
    const uint32_t vrow = gauss ? (uint32_t)(3 * N) * 4u : (uint32_t)ZW * 4u;
    const uint32_t cofs = (uint32_t)(((g >> 2) * 12 + (g & 3)) * 4), crow = (uint32_t)CW * 4u;
    float *a[ADJ_RB], *At[ADJ_RB], *mj[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) {
        const size_t off = (size_t)tk.fld_off * A.ncot + (size_t)(r0 + (q < nr ? q : 0)) * tk.K * G.LDC;
        a[q] = A.AF + off; At[q] = A.ATot + off; mj[q] = A.AJ + off;
    }
    float mi[ADJ_RB], mt[ADJ_RB], nup[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) { mi[q] = 0.f; mt[q] = 0.f; nup[q] = 0.f; }
    if (producer) {
        for (int q = NS; q < nq && !abort_s; ++q)
            if (!issue(q)) { abort_s = 1; break; }
    } else if (tid < ncw * 32) {
        // the view columns are outputs only: the transposed source never
        // writes them, so they are cleared here once read
        const bool clear = c >= G.CIN;
        for (int q = 0; q < nq; ++q) {
            const uint32_t pos = consumed + (uint32_t)q, sl = pos % NS;
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[sl], (pos / NS) & 1));
            if (!ok) { abort_s = 1; break; }
            const unsigned char *db = base + (size_t)sl * Ly.stage + h * Ly.dir;
            const unsigned char *vc = db + ADJ_RB * (2 * Ly.g + 2 * Ly.z) + cofs;
            if (valid) {
                for (int jj = 0; jj < CH; ++jj) {
                    const int step = q * CH + jj;
                    if (step > nt) break;
                    const int k = h == 0 ? step : nt - step;
                    const int rbx = h == 0 ? jj : CH - 1 - jj;                 // box row of level k
                    // weight rows: T, Cb of layer kt and Ca of layer ka
                    const int kt = h == 0 ? k - 1 : k, ka = h == 0 ? k : k - 1;
                    const int rt = h == 0 ? jj : CH - jj, ra = h == 0 ? jj + 1 : CH - jj - 1;
                    const bool ht = kt >= 0 && kt < nt, ha = ka >= 0 && ka < nt;
                    const float tv = ht ? *(const float *)(vc + rt * crow) : 0.f;
                    const float cb = ht ? *(const float *)(vc + rt * crow + 32) : 0.f;
                    const float ca = ha ? *(const float *)(vc + ra * crow + 16) : 0.f;
                    const bool has_a = h == 0 || k > 0;
                    const size_t o = (size_t)k * G.LDC + c;
                    int slot = 0;
#pragma unroll
                    for (int rq = 0; rq < ADJ_RB; ++rq) {
                        if (!act[rq]) continue;
                        const unsigned char *rb = db + (size_t)slot * (2 * Ly.g + 2 * Ly.z);
                        ++slot;
                        const unsigned char *va = rb + (gauss ? 0 : 2 * Ly.g) + voff;
                        const unsigned char *vt = rb + (gauss ? Ly.g : 2 * Ly.g + Ly.z) + voff;
                        // order 1: a_1 is zero below the TOA row and the total
                        // starts at a_1 (neither buffer is cleared beforehand)
                        const float av = has_a && (j > 1 || k == 0) ? *(const float *)(va + rbx * vrow) : 0.f;
                        if (has_a) {
                            const float t = (j > 1 ? *(const float *)(vt + rbx * vrow) : 0.f) + av;
                            At[rq][o] = t;
                            if (clear) a[rq][o] = 0.f;
                            mi[rq] = fmaxf(mi[rq], fabsf(av));
                            mt[rq] = fmaxf(mt[rq], fabsf(t));
                        }
                        const float nu = av + tv * nup[rq];
                        mj[rq][o] = ca * nu + cb * nup[rq];
                        nup[rq] = nu;
                    }
                }
            } else if (j == 1 && c < G.LDC) {
                // columns no order writes (unused ring slots, the row
                // padding): zero once, as the transposed source reads whole
                // muJ rows
                for (int jj = 0; jj < CH; ++jj) {
                    const int step = q * CH + jj;
                    if (step > nt) break;
#pragma unroll
                    for (int rq = 0; rq < ADJ_RB; ++rq)
                        if (act[rq]) mj[rq][(size_t)step * G.LDC + c] = 0.f;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[sl]);
        }
        if (valid && h == 0 && d.surf_on)
#pragma unroll
            for (int rq = 0; rq < ADJ_RB; ++rq)
                if (act[rq]) A.bc[(size_t)(tl * A.ncot + r0 + rq) * NR * 3 + g * 3 + s] = nup[rq];
    }
    consumed += (uint32_t)nq;
    __syncthreads();
    if (abort_s) break;
    // every row's maxima in one block reduction: lane 0 of each warp stores
    // its warp's (mi, mt) per row, one barrier, thread 0 finishes (the values
    // are non-negative, so 0 starts the maximum)
#pragma unroll
    for (int rq = 0; rq < ADJ_RB; ++rq) {
        float a = mi[rq], b = mt[rq];
        for (int o = 16; o > 0; o >>= 1) {
            a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        if (lane == 0) redr[tid >> 5][rq] = make_float2(a, b);
    }
    __syncthreads();
#pragma unroll
    for (int rq = 0; rq < ADJ_RB; ++rq) {
        if (!act[rq]) continue;                    // block-uniform
        if (threadIdx.x == 0) {
            float2 mm = make_float2(0.f, 0.f);
            for (int w = 0; w < (nthr >> 5); ++w) {
                mm.x = fmaxf(mm.x, redr[w][rq].x);
                mm.y = fmaxf(mm.y, redr[w][rq].y);
            }
            const int ta = tl * A.ncot + r0 + rq;
            TaskState ns = A.st[ta];
            ns.orders = j;
            ns.resid = mm.y > 0.f ? (double)(mm.x / mm.y) : 0.0;
            if (ns.resid < d.tol) { ns.converged = 1; ns.active = 0; }
            else if (j >= d.max_orders) ns.active = 0;
            A.st[ta] = ns;
            if (ns.active) {
                atomicAdd(&A.acnt[j], 1);
                A.aflag[tl] = 1;                           // the task stays on the next order's list
            }
        }
    }
    }
    if (abort_s) {
        if (tid == 0) atomicExch(B.err, OCRT_ERR_DEVICE);
        // copies issued but not consumed still land in this block's shared
        // memory: wait for them (bounded) before the block exits
        if (producer)
            for (uint32_t p = issued > (uint32_t)NS ? issued - NS : 0; p < issued; ++p)
                (void)mbar_wait(&full[p % NS], (p / NS) & 1);
    }
}

cudaError_t adj_scan_tma_launch(int grid, cudaStream_t st, const BatchBufs &B, const AdjBufs &A, const Geom &G,
                                int t0, int j, const AdjScanMaps &M)
{
    const int th = scan_tma_threads(G);
    k_adj_scan_tma<4, 4><<<grid, th, adj_scan_tma_smem_bytes(G, 4, 4), st>>>(B, A, G, t0, j, M);
    return cudaGetLastError();
}

int adj_scan_tma_maps(const Geom &G, float *AF, float *ATot, size_t adj_floats, const float *Cq, size_t layers,
                      AdjScanMaps *M)
{
    ScanMaps f, t;
    // the field maps of the forward scan over the adjoint buffers (4-level chunks)
    if (scan_tma_maps(G, 4, AF, ATot, adj_floats, Cq, layers, &f)) return -1;
    M->ag = f.jg; M->tg = f.tg; M->az = f.jz; M->tz = f.tz;
    // weight rows: a box one row taller than the chunk
    if (scan_tma_maps(G, 5, AF, ATot, adj_floats, Cq, layers, &t)) return -1;
    M->cq = t.cq;
    return 0;
}

// ---- host: launch, function handles ----
const void *scan_tma_fn(int ch, int ns)
{
    if (ch == 8 && ns == 3) return (const void *)k_scan_tma<8, 3>;
    if (ch == 8 && ns == 4) return (const void *)k_scan_tma<8, 4>;
    if (ch == 4 && ns == 6) return (const void *)k_scan_tma<4, 6>;
    if (ch == 16 && ns == 2) return (const void *)k_scan_tma<16, 2>;
    if (ch == 8 && ns == 5) return (const void *)k_scan_tma<8, 5>;
    if (ch == 4 && ns == 10) return (const void *)k_scan_tma<4, 10>;
    return nullptr;
}

cudaError_t scan_tma_launch(int ch, int ns, int grid, cudaStream_t st, const BatchBufs &B, const WaveBufs &W,
                            const Geom &G, int t0, int it, const ScanMaps &M)
{
    const int th = scan_tma_threads(G);
    const size_t sb = scan_tma_smem_bytes(G, ch, ns);
    if (ch == 8 && ns == 3) k_scan_tma<8, 3><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else if (ch == 8 && ns == 4) k_scan_tma<8, 4><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else if (ch == 4 && ns == 6) k_scan_tma<4, 6><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else if (ch == 16 && ns == 2) k_scan_tma<16, 2><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else if (ch == 8 && ns == 5) k_scan_tma<8, 5><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else if (ch == 4 && ns == 10) k_scan_tma<4, 10><<<grid, th, sb, st>>>(B, W, G, t0, it, M);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t scan_tma_init()
{
    const int v[6][2] = {{8, 3}, {8, 4}, {4, 6}, {16, 2}, {8, 5}, {4, 10}};
    for (const auto &x : v) {
        const cudaError_t e =
            cudaFuncSetAttribute(scan_tma_fn(x[0], x[1]), cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
    }
    return cudaFuncSetAttribute(k_adj_scan_tma<4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// ---- host: tensor maps over the wave buffers ----
namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    }
    return fn;
}
} // namespace

int scan_tma_maps(const Geom &G, int CH, float *J, float *Tot, size_t fld_floats, const float *Cq, size_t layers,
                  ScanMaps *M)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) return -1;
    const cuuint64_t rows = fld_floats / G.LDC;
    const cuuint32_t es[4] = {1, 1, 1, 1};
    // Gauss columns: {g, h, s, row}
    const cuuint64_t gd[4] = {(cuuint64_t)G.N, 2, 3, rows};
    const cuuint64_t gs[3] = {(cuuint64_t)G.N * 4, (cuuint64_t)2 * G.N * 4, (cuuint64_t)G.LDC * 4};
    const cuuint32_t gb[4] = {(cuuint32_t)G.N, 1, 3, (cuuint32_t)CH};
    // zero-weight columns: {column, row}
    const cuuint64_t zd[2] = {(cuuint64_t)G.LDC, rows};
    const cuuint64_t zs[1] = {(cuuint64_t)G.LDC * 4};
    const cuuint32_t zb[2] = {(cuuint32_t)scan_tma_zw(G), (cuuint32_t)CH};
    // weights: {3 * NRq, layer}
    const cuuint64_t cd[2] = {(cuuint64_t)scan_tma_cw(G), (cuuint64_t)layers};
    const cuuint64_t cs[1] = {(cuuint64_t)scan_tma_cw(G) * 4};
    const cuuint32_t cb[2] = {(cuuint32_t)scan_tma_cw(G), (cuuint32_t)CH};
    const auto F32 = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const auto NI = CU_TENSOR_MAP_INTERLEAVE_NONE;
    const auto NSW = CU_TENSOR_MAP_SWIZZLE_NONE;
    const auto L2P = CU_TENSOR_MAP_L2_PROMOTION_NONE;
    const auto OOB = CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE;
    if (enc(&M->jg, F32, 4, J, gd, gs, gb, es, NI, NSW, L2P, OOB) != CUDA_SUCCESS) return -2;
    if (enc(&M->tg, F32, 4, Tot, gd, gs, gb, es, NI, NSW, L2P, OOB) != CUDA_SUCCESS) return -2;
    if (enc(&M->jz, F32, 2, J, zd, zs, zb, es, NI, NSW, L2P, OOB) != CUDA_SUCCESS) return -2;
    if (enc(&M->tz, F32, 2, Tot, zd, zs, zb, es, NI, NSW, L2P, OOB) != CUDA_SUCCESS) return -2;
    if (enc(&M->cq, F32, 2, (void *)Cq, cd, cs, cb, es, NI, NSW, L2P, OOB) != CUDA_SUCCESS) return -2;
    return 0;
}

bool scan_tma_supported(const Geom &G)
{
    return G.N % 4 == 0 && scan_tma_cw(G) <= 256 && scan_tma_zw(G) <= 256 && scan_tma_threads(G) <= 512 &&
           encode_fn() != nullptr;
}
