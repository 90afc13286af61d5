// tc_gemm.cu — multiple-scattering source contraction on the tcgen05 tensor
// cores (rt_sos_operator.c:206-424), aerosol operator and molecular term.
//
// Per item: one (task, 128-level tile).  D[128 levels][NP outputs] (FP32 in
// TMEM) = F[128 levels][6N inputs] x Aop^T, K = 6N swept in 32-element tiles
// (one 128-byte swizzle row), each tile as three tcgen05.mma.kind::tf32 passes
// (hi*hi + hi*lo + lo*hi) over tf32 (hi, lo) splits of both operands, which
// carry FP32-level accuracy on the TF32 tensor path.
//
// Both kernels (k_source_tc, k_adj_source_tc: 512 threads, one CTA per SM,
// persistent over items):
//   warps 8-15 producers: read the FP32 field rows of a K tile straight from
//           global memory, split each value into tf32 (hi, lo) in registers
//           and store both into the SWIZZLE_128B K-major layout of a 2-stage
//           shared-memory ring (warps 8-11 fill stage 0, warps 12-15 stage 1,
//           so each group has two tile periods to cover its load latency);
//           field rows past the task are zero and never read.  The operator
//           side arrives pre-split: the first thread of the group issues two
//           bulk copies of the operator's hi and lo tiles for that K tile
//           (written once per wave by k_tables / k_mol_dense, or by
//           k_op_transpose / k_mol_utrans for the adjoint), completing on the
//           stage's full barrier.  Warp 8 lane 0 also fetches the items.
//   warp 1  MMA issuer: one thread issues the MMAs into one of two TMEM
//           accumulators (2 x 256 columns), so the next item's MMAs run while
//           the epilogue drains the previous one;
//   warp 2  TMEM allocation owner;
//   warps 4-7 epilogue: tcgen05.ld of their 32-lane quadrant, J = x_k * D,
//           stored row-contiguous through a shared-memory transpose.
//
// Every wait is time-bounded: on timeout the CTA records an error word, waits
// (bounded) for its own MMAs to complete, frees TMEM and returns.
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"
#include "tcgen05.cuh"

#define TC_M 128
#define TC_KT 32
#define TC_FWD_THREADS 512
#define TC_PW0 8            // first producer warp of the forward kernel
#define TC_PGW 4            // producer warps per stage group
#define TC_AQ 8             // float4 chunks of a field tile per producer thread (128 rows x 8 / 128)
#define TC_BQ 14            // B-tile rows per producer thread, upper bound (224 rows)
#define TC_TMEM_COLS 512
#define TC_ACC_COLS 256
#define TC_Q 8
#define TC_TP 20             // row stride (floats) of an epilogue transpose tile: 16 columns + pad

using namespace tcg;

// ADJ = false: forward source.  A rows = levels of one task's field F, K = CIN,
//   B = the aerosol operator [NP][CIN] into one TMEM accumulator; for m <= 2
//   tasks the item runs NKT more K tiles over the same field rows with B = the
//   dense molecular operator U V (rt_sos_operator.c:387-406) into the second
//   accumulator.  Epilogue J[k][c] = x_k D_aer[k][c] + y_k D_mol[k][c] for
//   c < COUT, one write.  Items = active list x level tiles; an item takes one
//   accumulator slot, or two for m <= 2.
// ADJ = true: transposed source of the adjoint.  A rows = the ncot adjoint
//   fields of one task stacked (ncot * K rows of muJ, row stride LDC, columns
//   past LDC read as zero), B = the task's transposed operator AopT [CIN][KP]
//   and, for m <= 2, U^T [24][KP] (KP = COUT rounded up to 32), K = KP;
//   epilogue a[row][cin] = x_k D[row][cin] + y_k sum_f V[4b+f][cin]
//   D[row][CIN + 4b + f] (cin = bN + i) for cin < CIN; items = every task of
//   the wave x tiles, skipped when none of its rows is active.
// XS = true (forward form only): the A rows are the adjoint's scattered field
//   Xs = F_tot - F_last formed while loading, (Tot - F) plus the total's tail
//   at the TOA and BOA rows, in the same FP32 operations k_adj_prep applies.
template <bool ADJ, bool XS = false>
__device__ __forceinline__ void source_tc_body(const BatchBufs &B, const WaveBufs &W, const AdjBufs &AB,
                                               const Geom &G, int t0, int it, int mtiles, int nw)
{
    extern __shared__ unsigned char smem_raw[];
    // MMA N: the operator rows (NB); in the adjoint, m <= 2 tasks add 32 rows of
    // the transposed molecular factor U^T, whose product lands in TMEM columns
    // NB .. NB + 23 and is contracted with V^T in the epilogue.
    const int NB = ADJ ? G.CIN : G.NP;
    const int NBM = ADJ ? NB + 32 : NB;
    const int NKT = ADJ ? ((G.COUT + TC_KT - 1) / TC_KT) : G.CIN / TC_KT;
    const uint32_t A_BYTES = TC_M * TC_KT * 4, B_BYTES = (uint32_t)NBM * TC_KT * 4;
    const uint32_t STAGE = 2 * A_BYTES + 2 * B_BYTES;
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(base + 2 * STAGE);
    uint64_t *full = bars, *empty = bars + 2, *tfull = bars + 4, *tempty = bars + 6, *done = bars + 8;
    uint64_t *qbar = bars + 9;                           // [TC_Q]
    int *qitem = (int *)(qbar + TC_Q);                   // [TC_Q]
    uint32_t *tslot = (uint32_t *)(qitem + TC_Q);
    volatile int *abort_flag = (volatile int *)(tslot + 1);
    // epilogue transpose tiles: [4 warps][32 rows][TC_TP floats]
    float *tpose = (float *)(base + 2 * STAGE + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the adjoint's order it reads the tasks with a row still active after its
    // scan: list it + 1
    const int n_items = (ADJ ? AB.lcnt[it + 1] : B.active_cnt[it - 1]) * mtiles;
    const int *alist = ADJ ? AB.alist[(it + 1) & 1] : B.alist[it & 1];
    int *counter = ADJ ? &AB.awork[it] : &B.work[it * 4];
    auto task_of = [&](int li) -> int { return alist[li]; };

    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            // one more arrival: the bulk-copy thread's arrive.expect_tx for the B tiles
            mbar_init(&full[i], TC_PGW + 1);
            mbar_init(&empty[i], 1);
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 4);
        }
        mbar_init(done, 1);
        for (int i = 0; i < TC_Q; ++i) mbar_init(&qbar[i], 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    if (warp >= TC_PW0) {
        // ---------------- producer warps ----------------
        const int pt = tid - TC_PW0 * 32;                 // 0 .. 255
        const int grp = pt >> 7, gt = pt & 127;           // stage group, thread within the group
        // Thread gt owns 16-byte chunk ch = gt % 8 of rows r = gt / 8 + 16 i of a
        // tile; all its rows share r % 8, so their swizzled chunk position
        // (ch ^ r % 8) is one constant and row i sits 2048 i bytes further.
        const int r8 = gt >> 3, ch = gt & 7;
        const uint32_t soff = (uint32_t)r8 * 128u + ((uint32_t)(ch ^ (r8 & 7)) << 4);
        // A rows: field (forward) or stacked muJ rows (adjoint), stride LDC,
        // K columns < a_cols real; B rows: operator rows of length b_ld.
        const int a_cols = ADJ ? G.LDC : G.CIN, b_ld = ADJ ? ((G.COUT + 31) & ~31) : G.CIN;
        float4 ra[TC_AQ];
        // item operands: A rows (nra of them real), B = Bb for K tiles below
        // NKT and Bm (dense molecular operator) for NKT .. nkt - 1
        // Bt / Btm: the pre-split operator tiles (forward: aerosol, dense
        // molecular; adjoint: transposed operator with U^T rows), tile row count tr
        struct Opnd { const float *Ab, *Bt, *Btm, *Tb, *Tl; int nra, nbi, nkt, r0, nt; };
        const int tr = ADJ ? NB + 32 : NB;
        // K tile kt of the item into registers: A rows 0 .. nra - 1 of the item
        // (zero past the task and past a_cols), B rows 0 .. nbi - 1
        auto load = [&](const Opnd &o, int kt) {
            const int kk = kt < NKT ? kt : kt - NKT;
            const int col = kk * TC_KT + ch * 4;
            const bool acol = col + 4 <= a_cols;
            const float4 *pa = reinterpret_cast<const float4 *>(o.Ab + (size_t)r8 * G.LDC + col);
#pragma unroll
            for (int i = 0; i < TC_AQ; ++i)
                ra[i] = acol && r8 + 16 * i < o.nra ? __ldg(pa + (size_t)i * 4 * G.LDC) : make_float4(0.f, 0.f, 0.f, 0.f);
            if constexpr (XS) {
                const float4 *pt = reinterpret_cast<const float4 *>(o.Tb + (size_t)r8 * G.LDC + col);
#pragma unroll
                for (int i = 0; i < TC_AQ; ++i) {
                    if (!(acol && r8 + 16 * i < o.nra)) continue;
                    const float4 t = __ldg(pt + (size_t)i * 4 * G.LDC);
                    float4 x = make_float4(t.x - ra[i].x, t.y - ra[i].y, t.z - ra[i].z, t.w - ra[i].w);
                    const int k = o.r0 + r8 + 16 * i;
                    if (k == 0 || k == o.nt) {
                        const float4 lo = __ldg(reinterpret_cast<const float4 *>(o.Tl + (k == 0 ? 0 : G.LDC) + col));
                        x.x = x.x + lo.x; x.y = x.y + lo.y; x.z = x.z + lo.z; x.w = x.w + lo.w;
                    }
                    ra[i] = x;
                }
            }
        };
        // split into tf32 (hi, lo) and store at byte offset off of the hi and lo tiles
        auto put = [&](unsigned char *hi, unsigned char *lo, uint32_t off, float4 v) {
            float4 h, l;
            h.x = round_tf32f(v.x); l.x = round_tf32f(v.x - h.x);
            h.y = round_tf32f(v.y); l.y = round_tf32f(v.y - h.y);
            h.z = round_tf32f(v.z); l.z = round_tf32f(v.z - h.z);
            h.w = round_tf32f(v.w); l.w = round_tf32f(v.w - h.w);
            *reinterpret_cast<float4 *>(hi + off) = h;
            *reinterpret_cast<float4 *>(lo + off) = l;
        };
        // Item j + 1 is published as soon as item j is known, so each group
        // loads its first tile of the next item while the current item's last
        // tiles are still in the MMA pipeline.
        auto fetch_publish = [&](int jj) {                // warp 8 lane 0 only
            int item = -1;
            while (!*abort_flag) {
                const int cand = atomicAdd(counter, 1);
                if (cand >= n_items) break;
                const int li = cand / mtiles, mt = cand - li * mtiles;
                const int tl = task_of(li);
                const TaskDev tk = B.tasks[t0 + tl];
                if (ADJ) {
                    if (mt * TC_M >= AB.ncot * tk.K) continue;
                    bool any = false;
                    for (int r = 0; r < AB.ncot; ++r) any |= AB.st[tl * AB.ncot + r].active != 0;
                    if (!any) continue;
                } else if (mt * TC_M > B.px[tk.pix].nt) {
                    continue;
                }
                item = cand;
                break;
            }
            qitem[jj & (TC_Q - 1)] = item;
            mbar_arrive(&qbar[jj & (TC_Q - 1)]);
        };
        // item of queue position jj; one lane waits and the warp stays converged
        auto item_at = [&](int jj, int &item) -> bool {
            int ok = lane == 0 ? (int)mbar_wait(&qbar[jj & (TC_Q - 1)], (jj / TC_Q) & 1) : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            __syncwarp();                 // orders lane 0's acquire before the other lanes' reads
            if (ok) item = qitem[jj & (TC_Q - 1)];
            return ok != 0;
        };
        auto operands = [&](int item) -> Opnd {
            const int li = item / mtiles, mt = item - li * mtiles;
            const int tl = task_of(li);
            const TaskDev tk = B.tasks[t0 + tl];
            const int r0 = mt * TC_M;
            Opnd o;
            o.nra = min(TC_M, (ADJ ? AB.ncot * tk.K : tk.K) - r0);
            o.nbi = ADJ && tk.has_mol ? NBM : NB;
            o.Ab = ADJ ? AB.AJ + (size_t)tk.fld_off * AB.ncot + (size_t)r0 * G.LDC : W.F + tk.fld_off + (size_t)r0 * G.LDC;
            const bool dbl = !ADJ && tk.has_mol;
            o.Bt = ADJ ? AB.opsT + (size_t)tl * 2 * tr * b_ld : W.opt + 2 * tk.op_off;
            o.Btm = dbl ? W.opt + 2 * tk.uv_off : o.Bt;
            o.nkt = dbl ? 2 * NKT : NKT;
            o.Tb = XS ? W.Tot + tk.fld_off + (size_t)r0 * G.LDC : nullptr;
            o.Tl = XS ? W.Ttl + tk.tail_off : nullptr;
            o.r0 = r0;
            o.nt = tk.K - 1;
            return o;
        };
        if (pt == 0) fetch_publish(0);
        uint32_t g = 0;
        bool have = false;
        int armed = 0;               // bulk copies issued into this group's stage; parity of the last
        uint32_t armed_par = 0;           // the registers already hold this group's first tile of the item
        for (int j = 0;; ++j) {
            int item = -1;
            if (!item_at(j, item)) { *abort_flag = 1; break; }
            if (item < 0) break;
            if (pt == 0) fetch_publish(j + 1);
            const Opnd op = operands(item);
            // this group's K tiles of the item: global tile index g + kt with (g + kt) & 1 == grp
            const int kt0 = (int)((grp - (int)(g & 1)) & 1);
            if (!have && kt0 < op.nkt) load(op, kt0);
            have = false;
            bool stop = false;
            for (int kt = kt0; kt < op.nkt; kt += 2) {
                const uint32_t gg = g + (uint32_t)kt, u = gg >> 1;
                const int s = (int)(gg & 1);
                int free_ok = (u == 0 || lane != 0) ? 1 : (int)mbar_wait(&empty[s], (u - 1) & 1);
                free_ok = __shfl_sync(0xffffffffu, free_ok, 0);
                __syncwarp();
                if (!free_ok) { *abort_flag = 1; stop = true; break; }
                unsigned char *sp = base + (size_t)s * STAGE;
                if (gt == 0) {
                    // the B tiles of this K tile (its first nbi rows): two bulk
                    // copies completing on full[s]
                    const int kf = kt < NKT ? kt : kt - NKT;
                    const float *src = (kt < NKT ? op.Bt : op.Btm) + (size_t)kf * 2 * tr * TC_KT;
                    const uint32_t nb = (uint32_t)op.nbi * TC_KT * 4;
                    mbar_expect_tx(&full[s], 2 * nb);
                    armed = 1;
                    armed_par = u & 1;
                    bulk_g2s(sp + 2 * A_BYTES, src, nb, &full[s]);
                    bulk_g2s(sp + 2 * A_BYTES + B_BYTES, src + (size_t)tr * TC_KT, nb, &full[s]);
                }
#pragma unroll
                for (int i = 0; i < TC_AQ; ++i) put(sp, sp + A_BYTES, soff + 2048u * i, ra[i]);

                // generic-proxy stores made visible to the tensor cores before the stage is marked full
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
                if (kt + 2 < op.nkt) {
                    load(op, kt + 2);
                } else {
                    int nxt = -1;
                    if (!item_at(j + 1, nxt)) { *abort_flag = 1; stop = true; break; }
                    const int kt0n = (int)((grp - (int)((g + (uint32_t)op.nkt) & 1)) & 1);
                    if (nxt >= 0) {
                        const Opnd on = operands(nxt);
                        if (kt0n < on.nkt) { load(on, kt0n); have = true; }
                    }
                }
            }
            if (stop) break;
            g += (uint32_t)op.nkt;
        }
        // the last B copies into this group's stage have landed before the CTA
        // can leave (every armed stage also gets the group's four arrivals)
        if (gt == 0 && armed) mbar_wait(&full[grp], armed_par);
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        constexpr uint32_t IDESC_BASE = idesc_tf32(TC_M, 16);    // N filled in below
        uint32_t g = 0, u = 0, sc0 = 0, sc1 = 0;                 // tiles, accumulator slots, uses per slot
        for (int j = 0;; ++j) {
            if (!mbar_wait(&qbar[j & (TC_Q - 1)], (j / TC_Q) & 1)) { *abort_flag = 1; break; }
            const int item = qitem[j & (TC_Q - 1)];
            if (item < 0 || *abort_flag) break;
            const bool hm = B.tasks[t0 + task_of(item / mtiles)].has_mol;
            const int nbi = ADJ && hm ? NBM : NB;
            const bool dbl = !ADJ && hm;
            const int nkt = dbl ? 2 * NKT : NKT;
            const uint32_t idesc = (IDESC_BASE & ~(0x3Fu << 17)) | ((uint32_t)(nbi >> 3) << 17);
            const int b0 = (int)(u & 1), b1 = (int)((u + 1) & 1);
            bool ok = true;
            for (int q = 0; q < (dbl ? 2 : 1); ++q) {
                const int bq = q ? b1 : b0;
                const uint32_t n = bq ? sc1 : sc0;
                if (n >= 1 && !mbar_wait(&tempty[bq], (n - 1) & 1)) { ok = false; break; }
            }
            if (!ok) { *abort_flag = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int kt = 0; kt < nkt; ++kt, ++g) {
                const uint32_t acc = tmem + (uint32_t)((kt < NKT ? b0 : b1) * TC_ACC_COLS);
                const int kf = kt < NKT ? kt : kt - NKT;
                const int s = g & 1;
                if (!mbar_wait(&full[s], (g >> 1) & 1)) { *abort_flag = 1; ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                unsigned char *sp = base + (size_t)s * STAGE;
                const uint32_t sa_hi = smem_u32(sp), sa_lo = smem_u32(sp + A_BYTES);
                const uint32_t sb_hi = smem_u32(sp + 2 * A_BYTES), sb_lo = smem_u32(sp + 2 * A_BYTES + B_BYTES);
#pragma unroll
                for (int kk = 0; kk < TC_KT / 8; ++kk) {
                    const uint32_t off = kk * 32;     // 8 tf32 = 32 bytes along the swizzled row
                    const uint64_t ah = sdesc_sw128(sa_hi + off), al = sdesc_sw128(sa_lo + off);
                    const uint64_t bh = sdesc_sw128(sb_hi + off), bl = sdesc_sw128(sb_lo + off);
                    umma_tf32(acc, ah, bh, idesc, (kf > 0 || kk > 0) ? 1u : 0u);
                    umma_tf32(acc, ah, bl, idesc, 1u);
                    umma_tf32(acc, al, bh, idesc, 1u);
                }
                umma_commit(&empty[s]);
            }
            if (!ok) break;
            umma_commit(&tfull[b0]);
            if (dbl) umma_commit(&tfull[b1]);
            if (dbl) { ++sc0; ++sc1; } else if (b0) { ++sc1; } else { ++sc0; }
            u += dbl ? 2 : 1;
        }
        // every MMA this thread issued has completed before TMEM is released
        umma_commit(done);
        if (!mbar_wait(done, 0)) *abort_flag = 1;
    } else if (warp >= 4 && warp < 8) {
        // ---------------- epilogue ----------------
        const int q4 = warp - 4;
        uint32_t u = 0, sc0 = 0, sc1 = 0;                        // accumulator slots, uses per slot
        for (int j = 0;; ++j) {
            if (!mbar_wait(&qbar[j & (TC_Q - 1)], (j / TC_Q) & 1)) { *abort_flag = 1; break; }
            const int item = qitem[j & (TC_Q - 1)];
            if (item < 0 || *abort_flag) break;
            const int li = item / mtiles, mt = item - li * mtiles;
            const TaskDev tk = B.tasks[t0 + task_of(li)];
            const bool dbl = !ADJ && tk.has_mol;
            const int b = (int)(u & 1), b1 = (int)((u + 1) & 1);
            if (!mbar_wait(&tfull[b], (b ? sc1 : sc0) & 1) || (dbl && !mbar_wait(&tfull[b1], (b1 ? sc1 : sc0) & 1))) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const PixDev &d = B.px[tk.pix];
            const int row = mt * TC_M + q4 * 32 + lane;
            int k, ncols;
            bool live;
            float *outbase;                                  // row 0 of the item's output rows
            if (ADJ) {
                live = row < AB.ncot * tk.K;
                k = live ? row % tk.K : 0;
                outbase = AB.AF + (size_t)tk.fld_off * AB.ncot;
                ncols = G.CIN;
            } else {
                live = row <= d.nt;
                k = row;
                outbase = W.J + tk.fld_off;
                ncols = G.COUT;
            }
            const float x = live ? B.lvf[3 * (d.lev_off + k)] : 0.f;
            const float ym = dbl && live ? B.lvf[3 * (d.lev_off + k) + 1] : 0.f;
            const uint32_t tb = tmem + (uint32_t)(b * TC_ACC_COLS) + ((uint32_t)(q4 * 32) << 16);
            const uint32_t tbm = tmem + (uint32_t)(b1 * TC_ACC_COLS) + ((uint32_t)(q4 * 32) << 16);
            // adjoint, m <= 2: the rank-24 product U^T muJ of this row sits in
            // columns NB .. NB + 23
            const bool mol = ADJ && tk.has_mol;
            float t24[24];
            float y = 0.f;
            const float *Vm = B.molV + (size_t)(mol ? tk.m : 0) * 32 * G.CIN;
            if (mol) {
                float th[16];
                tmem_ld16(tb + (uint32_t)NB, t24);
                tmem_ld16(tb + (uint32_t)(NB + 16), th);
#pragma unroll
                for (int q = 0; q < 8; ++q) t24[16 + q] = th[q];
                y = live ? B.lvf[3 * (d.lev_off + k) + 1] : 0.f;
            }
            // Each 32-row x 16-column chunk goes through a shared-memory
            // transpose so the stores are row-contiguous: lane l then writes
            // 16 bytes (columns 4 (l % 4) .. +3) of rows l / 4 + 8 i, i < 4.
            float *tp = tpose + (size_t)q4 * 32 * TC_TP;
            const int row0 = mt * TC_M + q4 * 32;            // first row of this warp's quadrant
            for (int cb = 0; cb < NB / 16; ++cb) {
                float v[16];
                tmem_ld16(tb + (uint32_t)(cb * 16), v);
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) v[jj] *= x;
                if (dbl) {
                    float vm[16];
                    tmem_ld16(tbm + (uint32_t)(cb * 16), vm);
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj) v[jj] = fmaf(ym, vm[jj], v[jj]);
                }
                if (mol) {
                    // the chunk lies in input block b = 16 cb / N (N % 16 == 0);
                    // V^T: input column c = bN + i takes sum_f V[4b + f][c] t[4b + f]
                    float w4[4] = {0.f, 0.f, 0.f, 0.f};
                    const int b4 = 4 * ((cb * 16) / G.N);
#pragma unroll
                    for (int q = 0; q < 24; ++q)
                        if ((q & ~3) == b4) w4[q & 3] = t24[q];
                    for (int jj = 0; jj < 16; ++jj) {
                        const int c = cb * 16 + jj;
                        float acc = 0.f;
#pragma unroll
                        for (int f = 0; f < 4; ++f) acc = fmaf(__ldg(Vm + (size_t)(b4 + f) * G.CIN + c), w4[f], acc);
                        v[jj] = fmaf(y, acc, v[jj]);
                    }
                }
#pragma unroll
                for (int jj = 0; jj < 16; jj += 4)
                    *reinterpret_cast<float4 *>(tp + lane * TC_TP + jj) = make_float4(v[jj], v[jj + 1], v[jj + 2], v[jj + 3]);
                __syncwarp();
                const int c = cb * 16 + (lane & 3) * 4;
                if (c + 4 <= G.LDC && c < ncols) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int rl = (lane >> 2) + 8 * i, rg = row0 + rl;
                        const bool rlive = ADJ ? rg < AB.ncot * tk.K : rg <= d.nt;
                        if (!rlive) continue;
                        float *dst = outbase + (size_t)rg * G.LDC + c;
                        *reinterpret_cast<float4 *>(dst) = *reinterpret_cast<const float4 *>(tp + rl * TC_TP + (lane & 3) * 4);
                    }
                }
                __syncwarp();
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&tempty[b]);
                if (dbl) mbar_arrive(&tempty[b1]);
            }
            if (dbl) { ++sc0; ++sc1; } else if (b) { ++sc1; } else { ++sc0; }
            u += dbl ? 2 : 1;
        }
    }
    __syncthreads();
    if (tid == 0 && *abort_flag) atomicExch(B.err, OCRT_ERR_DEVICE);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 2) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
    }
}

__global__ void __launch_bounds__(TC_FWD_THREADS, 1)
k_source_tc(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int mtiles)
{
    AdjBufs none{};
    source_tc_body<false>(B, W, none, G, t0, it, mtiles, 0);
}

// The adjoint's source of the scattered field, S Xs with Xs = F_tot - F_last
// formed from the forward total and the last order while the rows load.
__global__ void __launch_bounds__(TC_FWD_THREADS, 1)
k_source_tc_xs(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int mtiles)
{
    AdjBufs none{};
    source_tc_body<false, true>(B, W, none, G, t0, it, mtiles, 0);
}

// Transposed contraction of the adjoint for adjoint order `it` (work counter
// AB.awork[it]).
__global__ void __launch_bounds__(TC_FWD_THREADS, 1)
k_adj_source_tc(BatchBufs B, WaveBufs W, AdjBufs AB, Geom G, int t0, int it, int mtiles, int nw)
{
    source_tc_body<true>(B, W, AB, G, t0, it, mtiles, nw);
}

static size_t tc_smem_for(int NBM)
{
    return 1024 + 2 * (2 * (size_t)TC_M * TC_KT * 4 + 2 * (size_t)NBM * TC_KT * 4) + 256 + 4 * 32 * TC_TP * 4;
}

int tc_fwd_threads() { return TC_FWD_THREADS; }

size_t tc_smem_bytes(const Geom &G)
{
    return tc_smem_for(G.NP);
}

size_t tc_adj_smem_bytes(const Geom &G)
{
    return tc_smem_for(G.CIN + 32);
}

bool tc_adj_supported(const Geom &G)
{
    return (G.CIN % 16) == 0 && G.CIN + 32 <= TC_ACC_COLS && G.CIN + 32 <= 16 * TC_BQ && G.N % 16 == 0 &&
           tc_adj_smem_bytes(G) <= 227 * 1024;
}

bool tc_supported(const Geom &G)
{
    return (G.CIN % TC_KT) == 0 && G.CIN / TC_KT >= 2 && G.NP <= TC_ACC_COLS && G.NP <= 16 * TC_BQ &&
           G.NP % 16 == 0 && (G.LDC % 4) == 0 && tc_smem_bytes(G) <= 227 * 1024;
}
