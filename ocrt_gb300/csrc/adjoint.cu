// adjoint.cu — gradients of the TOA reflectance with respect to the layer
// optical depths, the layer single-scattering albedos and the wind speed.
//
// The reference has no derivatives; this is the adjoint of the discrete
// system the forward solves.  For one Fourier mode the SOS computes the
// Neumann series F = sum_n L^(n-1) F_1 of the linear order operator
//     L F = Scan(S F, Rsurf F_dn(BOA)),
// S the per-level source contraction (rt_sos_operator.c:206-424), Scan the
// up/down linear-in-tau recurrences (rt_layer_transport.c:107-208) and Rsurf
// the rough-surface boundary operator (rt_surface_boundary.c:137-208).  For an
// output y = e^T F the adjoint field is a = sum_j (L^T)^j e, summed by its own
// successive orders with the same convergence test, and for any parameter p
//     dy/dp = a^T (dL/dp) F_tot + a^T dF_1/dp.
// Because L is linear and the same at every order, the forward only needs two
// checkpoints per mode: the order total F_tot and the last order's field
// (their difference is the field that was scattered), not every order.
//
//   k_adj_prep      Xs = F_tot - F_last into the field buffer (the scattered field),
//                   where a CUDA-core source pass reads it; the tensor-core pass
//                   (k_source_tc_xs) and k_adj_grad form it from the total instead
//   k_fill_all      every task active, for one extra source pass J_tot = S Xs
//   k_adj_init      a_1 = e: the output weights at the TOA view column(s)
//   k_adj_scan      transposed transport of a_j (recurrences run the other way),
//                   accumulation of the adjoint total and the residual test
//   k_adj_source    a_{j+1} = x_k A^T muJ: the transposed aerosol contraction
//   k_adj_mol       + y_k V^T (U^T muJ): the transposed rank-24 molecular term
//   k_adj_surface   + Rsurf^T mu_bc at the BOA downward columns
//   k_adj_grad      final transposed pass over the adjoint total: per-level and
//                   per-layer sums of the parameter derivatives
//   k_adj_pixel     sum over modes, chain rule to (dtau_l, ssa_l, wind), and
//                   the direct terms (removed surface seed, sunglint)
#include "kernels.cuh"
#include "physics.cuh"

namespace {

__device__ inline void decode_col_a(const Geom &G, int c, int &s, int &h, int &g) { decode_col(G, c, s, h, g); }

__device__ inline size_t adj_off(const TaskDev &tk, const Geom &G, int ncot, int r)
{
    return (size_t)tk.fld_off * ncot + (size_t)r * tk.K * G.LDC;
}

__device__ inline double block_max_a(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = l < nw ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

__device__ inline double block_sum_a(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = l < nw ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

__device__ inline float warp_sum(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Linear interpolation weights between the bracketing Gauss nodes
// (rt_solver.c:386-403), as in the forward extraction.
__device__ inline void bracket_a(const double *gmu, int n, double mu, int &lo, int &hi, double &t)
{
    int jh = 1;
    while (jh < n && gmu[jh - 1] < mu) jh++;
    int jl = jh - 1;
    if (jl < 1) { jl = 1; jh = 2; }
    if (jh > n) { jh = n; jl = n - 1; }
    lo = jl - 1; hi = jh - 1;
    t = (mu - gmu[lo]) / (gmu[hi] - gmu[lo]);
}

// Output weights of mode m for cotangent row (cI, cQ, cU):
// rho = (1/mu0) [X_0 + 2 sum_m X_m cos m(phi+pi)] for I, Q and
// (1/mu0) 2 sum_m U_m sin m(phi+pi) for U (rt_fourier.c:9-33).
__device__ inline void mode_weights(const PixDev &d, int m, const double *cot, double *w)
{
    const double phi = d.raa_deg * OCRT_PI / 180.0 + OCRT_PI;
    const double cm = m == 0 ? 1.0 : 2.0 * cos((double)m * phi);
    const double sm = m == 0 ? 0.0 : 2.0 * sin((double)m * phi);
    w[0] = cot[0] * cm / d.mu0;
    w[1] = cot[1] * cm / d.mu0;
    w[2] = cot[2] * sm / d.mu0;
}

} // namespace

// Xs = F_tot - F_last for every valid column and level.
__global__ void k_adj_prep(BatchBufs B, WaveBufs W, Geom G, int t0)
{
    const int tl = blockIdx.x, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int c = threadIdx.x;
    if (c >= G.COUT) return;
    int s, h, g;
    decode_col_a(G, c, s, h, g);
    if (g >= d.n_ring) return;
    float *F = W.F + tk.fld_off;
    const float *Tot = W.Tot + tk.fld_off;
    for (int k = 0; k <= d.nt; ++k) {
        const size_t o = (size_t)k * G.LDC + c;
        const float lo = (k == 0 || k == d.nt) ? W.Ttl[tot_tail_off(tk, G, k, c)] : 0.f;
        F[o] = (Tot[o] - F[o]) + lo;
    }
}

// Rows CIN .. CIN + 31 of a molecular task's transposed operator block:
// U^T[q][kk] = U[kk][q] for q < 24, kk < COUT (zero elsewhere), the second
// factor of the transposed rank-24 molecular term in the tcgen05 adjoint pass.
__global__ void k_mol_utrans(const TaskDev *tasks, int t0, int nw, Geom G, const float *ops, float *opsT)
{
    const int tl = blockIdx.x;
    if (tl >= nw) return;
    const TaskDev tk = tasks[t0 + tl];
    if (!tk.has_mol) return;
    const int KP = (G.COUT + 31) & ~31;
    const float *U = ops + tk.mol_off;
    float *T = opsT + (size_t)tl * 2 * (G.CIN + 32) * KP;
    for (int e = threadIdx.x; e < 32 * KP; e += blockDim.x) {
        const int q = e / KP, kk = e - q * KP;
        tile_put_rows(T, G.CIN + 32, G.CIN + q, kk, (q < 24 && kk < G.COUT) ? U[(size_t)kk * 24 + q] : 0.f);
    }
}

// Mark every task of the wave active for order index `it` (one source pass).
__global__ void k_fill_all(BatchBufs B, int t0, int nw, int it)
{
    __shared__ int nmol;
    if (threadIdx.x == 0) nmol = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nw; i += blockDim.x) {
        B.alist[it & 1][i] = i;
        if (B.tasks[t0 + i].has_mol) B.mlist[it & 1][atomicAdd(&nmol, 1)] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        B.active_cnt[it - 1] = nw;
        B.mol_cnt[it - 1] = nmol;
        for (int q = 0; q < 4; ++q) B.work[it * 4 + q] = 0;
    }
}

// Transposed operators for the tcgen05 adjoint source: entry (cin, kk) =
// Aop[kk][cin] for kk < COUT, 0 up to KP = COUT rounded up to 32, per task
// CIN + 32 rows (k_mol_utrans fills the last 32 for m <= 2), written as the
// pre-split tf32 hi/lo SWIZZLE_128B tiles the tensor-core pass copies in
// (tile_put_rows; 2 (CIN + 32) KP floats per task).  32 x 32 blocks through
// shared memory.  Grid (task, CIN/32 blocks, KP/32 blocks), 32 x 8.
__global__ void k_op_transpose(const TaskDev *tasks, int t0, int nw, Geom G, const float *ops, float *opsT)
{
    __shared__ float tile[32][33];
    const int tl = blockIdx.x;
    if (tl >= nw) return;
    const TaskDev tk = tasks[t0 + tl];
    const int KP = (G.COUT + 31) & ~31;
    const int c0 = blockIdx.y * 32, r0 = blockIdx.z * 32;
    const float *A = ops + tk.op_off;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int row = r0 + yy, cin = c0 + threadIdx.x;
        tile[yy][threadIdx.x] = (row < G.COUT && cin < G.CIN) ? A[(size_t)row * G.CIN + cin] : 0.f;
    }
    __syncthreads();
    float *T = opsT + (size_t)tl * 2 * (G.CIN + 32) * KP;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int cin = c0 + yy, kk = r0 + threadIdx.x;
        if (cin < G.CIN && kk < KP) tile_put_rows(T, G.CIN + 32, cin, kk, tile[threadIdx.x][yy]);
    }
}

// a_1 = e.  One thread per adjoint task.
__global__ void k_adj_init(BatchBufs B, AdjBufs A, Geom G, int t0, int nadj)
{
    const int ta = blockIdx.x * blockDim.x + threadIdx.x;
    if (ta >= nadj) return;
    const int tl = ta / A.ncot, r = ta - tl * A.ncot, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    TaskState st;
    st.active = 1; st.orders = 0; st.converged = 0; st.pad_ = 0; st.resid = 0.0;
    A.st[ta] = st;
    double w[3];
    mode_weights(d, tk.m, A.cot + ((size_t)tk.pix * A.ncot + r) * 3, w);
    float *a = A.AF + adj_off(tk, G, A.ncot, r);
    // The adjoint buffers are not cleared per execute: order 1 reads a_1 at
    // the TOA row alone (every other level of a_1 is zero), so that row is
    // written here in full.
    for (int c = 0; c < G.LDC; ++c) a[c] = 0.f;
    if (d.view_slot >= 0) {
        for (int s = 0; s < 3; ++s) a[col_of(G, s, 0, d.view_slot)] = (float)w[s];
    } else {
        int lo, hi; double t;
        bracket_a(B.gmu, G.N, d.mu_view, lo, hi, t);
        for (int s = 0; s < 3; ++s) {
            a[col_of(G, s, 0, lo)] += (float)((1.0 - t) * w[s]);
            a[col_of(G, s, 0, hi)] += (float)(t * w[s]);
        }
    }
}

// Transposed transport of a_j.  Up column (forward I[nt] = bc,
// I[k] = T_k I[k+1] + Ca_k J[k] + Cb_k J[k+1]):
//   nu[0] = a[0], nu[k] = a[k] + T_{k-1} nu[k-1];
//   muJ[k] = Ca_k nu[k] (k < nt) + Cb_{k-1} nu[k-1] (k > 0);  mu_bc = nu[nt].
// Down column (forward I[0] = 0, I[k] = T_{k-1} I[k-1] + Ca_{k-1} J[k] + Cb_{k-1} J[k-1]):
//   nu[nt] = a[nt], nu[k] = a[k] + T_k nu[k+1];
//   muJ[k] = Ca_{k-1} nu[k] (k > 0) + Cb_k nu[k+1] (k < nt).
__global__ void __launch_bounds__(512, 1) k_adj_scan(BatchBufs B, AdjBufs A, Geom G, int t0, int j)
{
    // One block per (task, group of up to ADJ_RB cotangent rows): the rows
    // share the transport coefficients and each thread runs its column's
    // recurrence for every active row of the group.
    __shared__ double red[32];
    const int nrg = (A.ncot + ADJ_RB - 1) / ADJ_RB;
    const int tl = blockIdx.x / nrg, r0 = (blockIdx.x - tl * nrg) * ADJ_RB, tg = t0 + tl;
    const int nr = min(ADJ_RB, A.ncot - r0);
    bool act[ADJ_RB];
    bool any = false;
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) {
        act[q] = q < nr && A.st[tl * A.ncot + r0 + q].active;
        any |= act[q];
    }
    if (!any) return;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int c = threadIdx.x, nt = d.nt, NR = G.NR;
    int s = 0, h = 0, g = 0;
    if (c < G.COUT) decode_col_a(G, c, s, h, g);
    const bool valid = c < G.COUT && g < d.n_ring;
    float *a[ADJ_RB], *mj[ADJ_RB];
    float *At[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) {
        const size_t off = adj_off(tk, G, A.ncot, r0 + (q < nr ? q : 0));
        a[q] = A.AF + off; At[q] = A.ATot + off; mj[q] = A.AJ + off;
    }
    float mi[ADJ_RB], mt[ADJ_RB], nup[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) { mi[q] = 0.f; mt[q] = 0.f; nup[q] = 0.f; }
    if (valid) {
        const float *Tc = B.Tc + d.coef_off, *Ca = B.Ca + d.coef_off, *Cb = B.Cb + d.coef_off;
        // The view columns are outputs only (zero quadrature weight): the
        // transposed source never writes them, so they are cleared here once read.
        const bool clear = c >= G.CIN;
        // Each column walks its levels in its (transposed) transport direction,
        // step j at level j (upward columns) or nt - j (downward columns), with
        // the adjoint orders, their totals and the coefficients of the next
        // SCAN_DEPTH steps in flight as cp.async copies into this thread's own
        // shared-memory slots (refilled only after the values read are used).
        extern __shared__ float scan_smem[];
        const int bs = blockDim.x;
        float *As = scan_smem;                                                   // [SCAN_DEPTH][RB][bs]
        float *Ts = As + SCAN_DEPTH * ADJ_RB * bs;                                // [SCAN_DEPTH][RB][bs]
        float *Cs = Ts + SCAN_DEPTH * ADJ_RB * bs;                                // [SCAN_DEPTH][3][bs]
        // coefficient rows of step j: upward tv, cb at k - 1 and ca at k;
        // downward tv, cb at k and ca at k - 1 (absent rows read as zero)
        auto issue = [&](int jj) {
            if (jj <= nt) {
                const int k = h == 0 ? jj : nt - jj, sl = jj & (SCAN_DEPTH - 1);
                const size_t o = (size_t)k * G.LDC + c;
                if (h == 0 || k > 0) {            // the TOA downward radiance is fixed at zero
#pragma unroll
                    for (int q = 0; q < ADJ_RB; ++q)
                        if (act[q]) {
                            cp_async4(As + (sl * ADJ_RB + q) * bs + c, a[q] + o);
                            cp_async4(Ts + (sl * ADJ_RB + q) * bs + c, At[q] + o);
                        }
                }
                const int kt = h == 0 ? k - 1 : k, ka = h == 0 ? k : k - 1;
                if (kt >= 0 && kt < nt) {
                    cp_async4(Cs + (sl * 3 + 0) * bs + c, Tc + kt * NR + g);
                    cp_async4(Cs + (sl * 3 + 2) * bs + c, Cb + kt * NR + g);
                }
                if (ka >= 0 && ka < nt) cp_async4(Cs + (sl * 3 + 1) * bs + c, Ca + ka * NR + g);
            }
            cp_async_commit();
        };
#pragma unroll
        for (int jj = 0; jj < SCAN_DEPTH; ++jj) issue(jj);
        for (int jj = 0; jj <= nt; ++jj) {
            cp_async_wait<SCAN_DEPTH - 1>();
            const int k = h == 0 ? jj : nt - jj, sl = jj & (SCAN_DEPTH - 1);
            const int kt = h == 0 ? k - 1 : k, ka = h == 0 ? k : k - 1;
            const bool has_a = h == 0 || k > 0;
            const float tv = kt >= 0 && kt < nt ? Cs[(sl * 3 + 0) * bs + c] : 0.f;
            const float cb = kt >= 0 && kt < nt ? Cs[(sl * 3 + 2) * bs + c] : 0.f;
            const float ca = ka >= 0 && ka < nt ? Cs[(sl * 3 + 1) * bs + c] : 0.f;
            const size_t o = (size_t)k * G.LDC + c;
#pragma unroll
            for (int q = 0; q < ADJ_RB; ++q) {
                if (!act[q]) continue;
                // order 1: a_1 is zero below the TOA row and the total starts
                // at a_1 (neither buffer is cleared beforehand)
                const float av = has_a && (j > 1 || k == 0) ? As[(sl * ADJ_RB + q) * bs + c] : 0.f;
                if (has_a) {
                    const float t = (j > 1 ? Ts[(sl * ADJ_RB + q) * bs + c] : 0.f) + av;
                    At[q][o] = t;
                    if (clear) a[q][o] = 0.f;
                    mi[q] = fmaxf(mi[q], fabsf(av));
                    mt[q] = fmaxf(mt[q], fabsf(t));
                }
                const float nu = av + tv * nup[q];
                mj[q][o] = ca * nu + cb * nup[q];
                nup[q] = nu;
            }
            issue(jj + SCAN_DEPTH);
        }
        cp_async_wait<0>();
        if (h == 0 && d.surf_on)
#pragma unroll
            for (int q = 0; q < ADJ_RB; ++q)
                if (act[q]) A.bc[(size_t)(tl * A.ncot + r0 + q) * NR * 3 + g * 3 + s] = nup[q];
    } else if (j == 1 && c < G.LDC) {
        // columns no order writes (unused ring slots, the row padding): zero
        // once, as the transposed source reads whole muJ rows
#pragma unroll
        for (int q = 0; q < ADJ_RB; ++q)
            if (act[q])
                for (int k = 0; k <= nt; ++k) mj[q][(size_t)k * G.LDC + c] = 0.f;
    }
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) {
        if (!act[q]) continue;                    // block-uniform
        const float bmi = (float)block_max_a(mi[q], red);
        __syncthreads();
        const float bmt = (float)block_max_a(mt[q], red);
        __syncthreads();
        if (threadIdx.x == 0) {
            const int ta = tl * A.ncot + r0 + q;
            TaskState ns = A.st[ta];
            ns.orders = j;
            ns.resid = bmt > 0.f ? (double)(bmi / bmt) : 0.0;
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

// a_{j+1}[k][cin] = x_k sum_row A[row][cin] muJ[k][row] (the transposed
// aerosol contraction; rows are the COUT outputs).  Columns past the weighted
// inputs are cleared.  Grid (adjoint task, 64-level tile, 64-column tile).
__global__ void __launch_bounds__(256) k_adj_source(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0)
{
    const int ta = blockIdx.x, tl = ta / A.ncot, r = ta - tl * A.ncot, tg = t0 + tl;
    if (!A.st[ta].active) return;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt;
    const int k0 = blockIdx.y * ST_M_TILE, c0 = blockIdx.z * ST_N_TILE;
    if (k0 > nt || c0 >= G.LDC) return;
    const size_t off = adj_off(tk, G, A.ncot, r);
    float *out = A.AF + off;
    if (c0 >= G.CIN) {
        for (int e = threadIdx.x; e < ST_M_TILE * ST_N_TILE; e += 256) {
            const int lv = e / ST_N_TILE, cc = e - lv * ST_N_TILE;
            const int k = k0 + lv, c = c0 + cc;
            if (k <= nt && c < G.LDC) out[(size_t)k * G.LDC + c] = 0.f;
        }
        return;
    }
    constexpr int KT = 16;
    __shared__ float Ms[KT][ST_M_TILE + 4];
    __shared__ float As[KT][ST_N_TILE + 4];
    const float *mj = A.AJ + off;
    const float *Aop = W.ops + tk.op_off;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4] = {{0}};
    for (int kc = 0; kc < G.COUT; kc += KT) {
        for (int idx = threadIdx.x; idx < ST_M_TILE * KT; idx += 256) {
            const int lv = idx / KT, kk = idx - lv * KT;
            const int k = k0 + lv, row = kc + kk;
            const size_t o = (size_t)k * G.LDC + row;
            Ms[kk][lv] = (k <= nt && row < G.COUT) ? mj[o] : 0.f;
        }
        for (int idx = threadIdx.x; idx < KT * ST_N_TILE; idx += 256) {
            const int kk = idx / ST_N_TILE, cc = idx - kk * ST_N_TILE;
            const int row = kc + kk, ci = c0 + cc;
            As[kk][cc] = (row < G.COUT && ci < G.CIN) ? Aop[(size_t)row * G.CIN + ci] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KT; ++kk) {
            float fr[4], ar[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) fr[i] = Ms[kk][ty + 16 * i];
#pragma unroll
            for (int q = 0; q < 4; ++q) ar[q] = As[kk][tx + 16 * q];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[i][q] = fmaf(fr[i], ar[q], acc[i][q]);
        }
        __syncthreads();
    }
    const double *xd = B.xd + d.lev_off;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int k = k0 + ty + 16 * i;
        if (k > nt) continue;
        const float x = (float)xd[k];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = c0 + tx + 16 * q;
            if (c < G.CIN) out[(size_t)k * G.LDC + c] = x * acc[i][q];
            else if (c < G.LDC) out[(size_t)k * G.LDC + c] = 0.f;
        }
    }
}

// a_{j+1}[k][bN+i] += y_k sum_f fv[f][i] zeta[k][4b+f], zeta[k][r] = sum_c U[c][r] muJ[k][c]
// (transpose of the rank-24 molecular operator of k_mol_lowrank).
// Grid (adjoint task, tile of 32 levels), 256 threads.
__global__ void __launch_bounds__(256) k_adj_mol(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0,
                                                 const float *Bp, const float *Br, const float *Bt, int L)
{
    extern __shared__ float sm[];
    const int ta = blockIdx.x, tl = ta / A.ncot, r = ta - tl * A.ncot, tg = t0 + tl;
    if (!A.st[ta].active) return;
    const TaskDev tk = B.tasks[tg];
    if (!tk.has_mol) return;
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt, N = G.N, k0 = blockIdx.y * 32;
    if (k0 > nt) return;
    const int nk = min(32, nt - k0 + 1);
    float *fv = sm;                          // [4][N]
    float *U = fv + 4 * N;                   // [COUT][24]
    float *Ms = U + G.COUT * 24;             // [32][COUT]
    float *zt = Ms + 32 * G.COUT;            // [32][25]
    const size_t gb = (size_t)tk.m * (L + 1) * N + (size_t)2 * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float w = (float)B.gw[i];
        fv[i] = w; fv[N + i] = w * Bp[gb + i]; fv[2 * N + i] = w * Br[gb + i]; fv[3 * N + i] = w * Bt[gb + i];
    }
    const float *Ug = W.ops + tk.mol_off;
    for (int e = threadIdx.x; e < G.COUT * 24; e += blockDim.x) U[e] = Ug[e];
    const size_t off = adj_off(tk, G, A.ncot, r);
    const float *mj = A.AJ + off + (size_t)k0 * G.LDC;
    for (int e = threadIdx.x; e < nk * G.COUT; e += blockDim.x) {
        const int k = e / G.COUT, c = e - k * G.COUT;
        const size_t o = (size_t)k * G.LDC + c;
        Ms[k * G.COUT + c] = mj[o];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nk * 24; e += blockDim.x) {
        const int k = e / 24, rr = e - k * 24;
        const float *mr = Ms + k * G.COUT;
        float acc = 0.f;
        for (int c = 0; c < G.COUT; ++c) acc = fmaf(U[c * 24 + rr], mr[c], acc);
        zt[k * 25 + rr] = acc;
    }
    __syncthreads();
    float *out = A.AF + off;
    for (int e = threadIdx.x; e < nk * G.CIN; e += blockDim.x) {
        const int k = e / G.CIN, ci = e - k * G.CIN, b = ci / N, i = ci - b * N;
        const float *z = zt + k * 25 + 4 * b;
        const float v = fv[i] * z[0] + fv[N + i] * z[1] + fv[2 * N + i] * z[2] + fv[3 * N + i] * z[3];
        out[(size_t)(k0 + k) * G.LDC + ci] += B.lvf[3 * (d.lev_off + k0 + k) + 1] * v;
    }
}

size_t adj_mol_smem_bytes(const Geom &G)
{
    return sizeof(float) * (4 * (size_t)G.N + (size_t)G.COUT * 24 + 32 * (size_t)G.COUT + 32 * 25);
}

// a_{j+1}[nt][(s', down, i)] += pw_i sum_{g, s} R_m(g, i)[s][s'] mu_bc[g][s]
// (transpose of the rough-surface boundary operator).  Threads over (s', i).
// Surface term of adjoint order j for the rows still active after the
// order's scan: blocks stride over the (listed task, row) items of list j + 1.
__global__ void k_adj_surface(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0, int j)
{
    const int N = G.N, NR = G.NR;
    const int e = threadIdx.x;
    if (e >= 3 * N) return;
    const int sp = e / N, i = e - sp * N;
    const int n_items = A.lcnt[j + 1] * A.ncot;
    const int *lst = A.alist[(j + 1) & 1];
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
        const int li = item / A.ncot, r = item - li * A.ncot, tl = lst[li], ta = tl * A.ncot + r, tg = t0 + tl;
        if (!A.st[ta].active) continue;
        const TaskDev tk = B.tasks[tg];
        const PixDev &d = B.px[tk.pix];
        if (!d.rough) continue;
        const float *mb = A.bc + (size_t)ta * NR * 3;
        const float *R = W.srf + tk.srf_off;
        const float pw = B.pw[(tk.m == 0 ? 0 : N) + i];
        float acc = 0.f;
        for (int g = 0; g < d.n_ring; ++g) {
            const float *Rg = R + ((size_t)g * N + i) * 9 + sp;
            acc += Rg[0] * mb[g * 3 + 0] + Rg[3] * mb[g * 3 + 1] + Rg[6] * mb[g * 3 + 2];
        }
        A.AF[adj_off(tk, G, A.ncot, r) + (size_t)d.nt * G.LDC + col_of(G, sp, 1, i)] += pw * acc;
    }
}

// List of order 1: every task of the wave.
__global__ void k_adj_list_all(AdjBufs A, int nw)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) A.alist[1][i] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) A.lcnt[1] = nw;
}

// The flagged tasks (a row active after the scan of order j) in task order
// into list j + 1 and its count; clears the flags.  One block.
__global__ void __launch_bounds__(COMPACT_THREADS) k_compact_adj(AdjBufs A, int nw, int j)
{
    __shared__ int sa[COMPACT_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (nw + COMPACT_THREADS - 1) / COMPACT_THREADS;
    const int b = min(nw, tid * per), e = min(nw, b + per);
    int na = 0;
    for (int i = b; i < e; ++i) na += A.aflag[i] ? 1 : 0;
    int xa = na;
    for (int o = 1; o < 32; o <<= 1) {
        const int ya = __shfl_up_sync(0xffffffffu, xa, o);
        if (lane >= o) xa += ya;
    }
    if (lane == 31) sa[w] = xa;
    __syncthreads();
    if (w == 0) {
        int ta = sa[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int ya = __shfl_up_sync(0xffffffffu, ta, o);
            if (lane >= o) ta += ya;
        }
        sa[lane] = ta;
        if (lane == 31) A.lcnt[j + 1] = ta;
    }
    __syncthreads();
    int oa = (w ? sa[w - 1] : 0) + xa - na;
    int *al = A.alist[(j + 1) & 1];
    for (int i = b; i < e; ++i)
        if (A.aflag[i]) {
            al[oa++] = i;
            A.aflag[i] = 0;
        }
}

// Final pass per adjoint task: the transposed transport of the adjoint total
// (the nu recurrence) fused with the per-level contractions.  With the forward
// total field F_tot and total source J_tot = S Xs + J_1:
//   lev_ssa[k] = sum_c muJ[k][c] J_tot[k][c]            (x_k, y_k and J_1 scale with the albedo)
//   lev_j1[k]  = sum_c muJ[k][c] J_1[k][c]              (J_1 ~ exp(-h_k/mu0))
//   lay[l]     = sum_c nu . (F dT + J dCa + J dCb)_l    (layer-l transport coefficients)
// plus, at the surface, mu_bc . dRsurf/dW . Xs_dn(BOA) and the seed terms.
// Each thread owns one column and walks its levels in the column's transport
// direction, so nu, muJ and the neighbouring level's J_tot are in registers
// when a level's terms are formed; each warp sums its lanes per level with
// shuffles.  The block's first half of threads takes the upward columns and
// the second half the downward ones (launch with 2 round32(3N + 3) threads),
// so every warp runs one direction.  Per-warp level sums sit in shared memory
// [warp][3][nt + 1] and are added in warp order, so the result does not
// depend on scheduling.
__global__ void __launch_bounds__(512) k_adj_grad(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0, int rb,
                                                  int xs_in_f)
{
    // One block per (task, group of rb <= ADJ_RB cotangent rows): the forward
    // totals, sources and coefficients a level's terms need are loaded once
    // for all rows of the group.
    extern __shared__ float wsum[];               // [warp][row][3][nt + 1]
    __shared__ double red[32];
    const int nrg = (A.ncot + rb - 1) / rb;
    const int tl = blockIdx.x / nrg, r0 = (blockIdx.x - tl * nrg) * rb, tg = t0 + tl;
    const int nr = min(rb, A.ncot - r0);
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt, NR = G.NR, N = G.N, L1 = nt + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float *ws = wsum + (size_t)warp * rb * 3 * L1;
    for (int x = lane; x < rb * 3 * L1; x += 32) ws[x] = 0.f;
    __syncwarp();
    const float *At[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) At[q] = A.ATot + adj_off(tk, G, A.ncot, r0 + (q < nr ? q : 0));
    const float *Tc = B.Tc + d.coef_off, *Ca = B.Ca + d.coef_off, *Cb = B.Cb + d.coef_off;
    const float *dT = A.dTc + d.coef_off, *dA = A.dCa + d.coef_off, *dB = A.dCb + d.coef_off;
    const float *lv = B.lvf + 3 * (size_t)d.lev_off;                 // x, y, ch per level
    const float *pv = W.pvec + (size_t)tl * 2 * G.LDC;
    const float *Jx = W.J + tk.fld_off;
    const float *Tot = W.Tot + tk.fld_off;
    // Threads [0, half) take the upward columns (h = 0), [half, 2 half) the
    // downward ones, so every warp runs one direction; half = round32(3N + 3).
    const int half = blockDim.x >> 1;
    const int h = threadIdx.x >= half ? 1 : 0, u = threadIdx.x - h * half;
    int s = 0, g = G.NR;
    if (u < 3 * N) { s = u / N; g = u - s * N; }
    else if (u < 3 * N + 3) { s = u - 3 * N; g = N; }
    const int c = g < N ? col_of(G, s, h, g) : 6 * N + 2 * s + h;
    const bool valid = g < d.n_ring;
    const float fa = valid ? pv[c] : 0.f, fm = valid ? pv[G.LDC + c] : 0.f;
    const bool wact = __any_sync(0xffffffffu, valid);                // warp-uniform
    float nu_prev[ADJ_RB];
#pragma unroll
    for (int q = 0; q < ADJ_RB; ++q) nu_prev[q] = 0.f;
    float jt_prev = 0.f;
    constexpr int PF = 4;
    // step j visits level k = j (upward columns: nu from the TOA down) or
    // k = nt - j (downward columns: nu from the BOA up, nu_0 = 0)
    for (int j1 = 0; wact && j1 <= nt; j1 += PF) {
        const int cnt = nt - j1 + 1 < PF ? nt - j1 + 1 : PF;
        float av[ADJ_RB][PF], tv[PF], ca[PF], cb[PF], jx[PF], tt[PF], xk[PF], yk[PF], chk[PF], lt[PF], la[PF], lb[PF];
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            tv[q] = ca[q] = cb[q] = jx[q] = tt[q] = xk[q] = yk[q] = chk[q] = lt[q] = la[q] = lb[q] = 0.f;
#pragma unroll
            for (int r = 0; r < ADJ_RB; ++r) av[r][q] = 0.f;
            if (valid && q < cnt) {
                const int k = h == 0 ? j1 + q : nt - j1 - q;
                const size_t o = (size_t)k * G.LDC + c;
#pragma unroll
                for (int r = 0; r < ADJ_RB; ++r)
                    if (r < nr) av[r][q] = At[r][o];
                jx[q] = Jx[o];
                tt[q] = Tot[o];
                xk[q] = lv[3 * k]; yk[q] = lv[3 * k + 1]; chk[q] = lv[3 * k + 2];
                if (h == 0) {
                    tv[q] = k > 0 ? Tc[(k - 1) * NR + g] : 0.f;
                    ca[q] = k < nt ? Ca[k * NR + g] : 0.f;
                    cb[q] = k > 0 ? Cb[(k - 1) * NR + g] : 0.f;
                    if (k > 0) {
                        const int e = (k - 1) * NR + g;
                        lt[q] = dT[e]; la[q] = dA[e]; lb[q] = dB[e];
                    }
                } else {
                    tv[q] = k < nt ? Tc[k * NR + g] : 0.f;
                    ca[q] = k > 0 ? Ca[(k - 1) * NR + g] : 0.f;
                    cb[q] = k < nt ? Cb[k * NR + g] : 0.f;
                    if (k < nt) {
                        const int e = k * NR + g;
                        lt[q] = dT[e]; la[q] = dA[e]; lb[q] = dB[e];
                    }
                }
            }
        }
        // per-lane contributions of the PF levels of this batch: [row][quantity][level]
        float v3[ADJ_RB][3][PF];
#pragma unroll
        for (int r = 0; r < ADJ_RB; ++r)
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
                for (int q = 0; q < PF; ++q) v3[r][x][q] = 0.f;
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            if (q >= cnt) break;                                            // warp-uniform
            const int k = h == 0 ? j1 + q : nt - j1 - q;
            // row-independent parts: J_tot at this level and the layer bracket
            // h 0 (layer k-1): F_k dT + J_{k-1} dCa + J_k dCb
            // h 1 (layer k):   F_k dT + J_{k+1} dCa + J_k dCb
            const float j1v = chk[q] * (xk[q] * fa + yk[q] * fm);
            const float jt = jx[q] + j1v;
            const float lay = tt[q] * lt[q] + jt_prev * la[q] + jt * lb[q];
            jt_prev = valid ? jt : 0.f;
#pragma unroll
            for (int r = 0; r < ADJ_RB; ++r) {
                if (r >= nr) break;                                         // block-uniform
                if (valid) {
                    const float nu = (h == 1 && k == 0) ? 0.f : av[r][q] + tv[q] * nu_prev[r];
                    // h 0: mu = Ca_k nu_k + Cb_{k-1} nu_{k-1};  h 1: mu = Ca_{k-1} nu_k + Cb_k nu_{k+1}
                    const float mu = ca[q] * nu + cb[q] * nu_prev[r];
                    v3[r][0][q] = mu * jt;
                    v3[r][1][q] = mu * j1v;
                    v3[r][2][q] = nu_prev[r] * lay;
                    nu_prev[r] = nu;
                }
            }
        }
        // Sums over the warp's 32 columns for the four levels at once: halve
        // the level set across lanes 16 and 8 apart (reduce-scatter), then
        // finish with three butterfly steps; lane 8 (2 b16 + b8) ends with
        // the total of level 2 b16 + b8, and lanes 0, 8, 16, 24 store them.
        const int b16 = (lane >> 4) & 1, b8 = (lane >> 3) & 1;
        const int qmine = 2 * b16 + b8;
        const int kmine = h == 0 ? j1 + qmine : nt - j1 - qmine;
        const int klmine = h == 0 ? kmine - 1 : kmine;
#pragma unroll
        for (int r = 0; r < ADJ_RB; ++r) {
            if (r >= nr) break;                                             // block-uniform
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                const float *v = v3[r][x];
                const float s0 = b16 ? v[0] : v[2], s1 = b16 ? v[1] : v[3];
                const float r0 = __shfl_xor_sync(0xffffffffu, s0, 16), r1 = __shfl_xor_sync(0xffffffffu, s1, 16);
                const float k0 = (b16 ? v[2] : v[0]) + r0, k1 = (b16 ? v[3] : v[1]) + r1;
                const float se = b8 ? k0 : k1;
                float tot = (b8 ? k1 : k0) + __shfl_xor_sync(0xffffffffu, se, 8);
                tot += __shfl_xor_sync(0xffffffffu, tot, 4);
                tot += __shfl_xor_sync(0xffffffffu, tot, 2);
                tot += __shfl_xor_sync(0xffffffffu, tot, 1);
                if ((lane & 7) == 0 && qmine < cnt) {
                    float *wr = ws + (size_t)r * 3 * L1;
                    if (x == 0) wr[kmine] += tot;
                    else if (x == 1) wr[L1 + kmine] += tot;
                    else if (klmine >= 0 && klmine < nt) wr[2 * L1 + klmine] += tot;
                }
            }
        }
    }
    // surface terms: wind derivative of the boundary operator and of the
    // direct-beam seed, and the seed's optical-depth dependence
    double gW[ADJ_RB], gS[ADJ_RB];
#pragma unroll
    for (int r = 0; r < ADJ_RB; ++r) { gW[r] = 0.0; gS[r] = 0.0; }
    if (valid && h == 0 && d.rough) {
        // the scattered field at the BOA: in F when k_adj_prep ran, else
        // formed as k_adj_prep forms it
        const float *Fb = W.F + tk.fld_off + (size_t)nt * G.LDC, *Tb = W.Tot + tk.fld_off + (size_t)nt * G.LDC;
        const float *Lb = W.Ttl + tk.tail_off + G.LDC;
        auto Xb = [&](int cc) -> float { return xs_in_f ? Fb[cc] : (Tb[cc] - Fb[cc]) + Lb[cc]; };
        const float *RW = A.srfW + tk.srf_off + (size_t)g * N * 9 + s * 3;
        const float *pwm = B.pw + (tk.m == 0 ? 0 : N);
        float accf = 0.f;          // FP32 like the boundary condition it differentiates
        for (int i = 0; i < N; ++i) {
            const float *Ri = RW + (size_t)i * 9;
            accf += pwm[i] * (Ri[0] * Xb(col_of(G, 0, 1, i)) + Ri[1] * Xb(col_of(G, 1, 1, i)) +
                              Ri[2] * Xb(col_of(G, 2, 1, i)));
        }
        const double acc = accf;
        const double tdn = exp(-d.tau_total / d.mu0);
        const double fs = (tk.m == 0 ? OCRT_PI : 0.5 * OCRT_PI) * d.mu0;
        const float *RsW = A.srfW + tk.srf_off + (size_t)G.NR * N * 9;
        const float *Rs = W.srf + tk.srf_off + (size_t)G.NR * N * 9;
        const double E = (double)B.Eatt[(d.lev_off + nt) * NR + g];
        const double sw = acc + fs * tdn * E * (double)RsW[g * 9 + s * 3];
        const double ss = fs * tdn * E * (double)Rs[g * 9 + s * 3];
#pragma unroll
        for (int r = 0; r < ADJ_RB; ++r) { gW[r] = nu_prev[r] * sw; gS[r] = nu_prev[r] * ss; }
    }
#pragma unroll
    for (int r = 0; r < ADJ_RB; ++r) {
        if (r >= nr) break;                       // block-uniform
        const double bW = block_sum_a(gW[r], red);
        __syncthreads();
        const double bS = block_sum_a(gS[r], red);
        __syncthreads();
        double *go = A.gout + (size_t)(tl * A.ncot + r0 + r) * A.gstride;
        for (int x = threadIdx.x; x < 3 * L1; x += blockDim.x) {
            const int q = x / L1, k = x - q * L1;
            float v = 0.f;
            for (int w = 0; w < nwarp; ++w) v += wsum[((size_t)w * rb + r) * 3 * L1 + x];
            go[(size_t)q * A.kstride + k] = v;
        }
        if (threadIdx.x == 0) {
            go[3 * A.kstride + 0] = bW;
            go[3 * A.kstride + 1] = bS;
        }
    }
}

// Per (pixel, cotangent row): sum the per-mode partials and apply the chain
// rule to the layer parameters:
//   d/ddtau_l = sum_m lay_m[l] - (1/mu0) sum_m sum_{k>l} lev_j1_m[k]
//               - (1/mu0) sum_m seed_m + (removed view seed) + (sunglint)
//   d/dssa_l  = sum_m lev_ssa_m[l+1] / ssa_l
//   d/dW      = sum_m surface_m + (removed view seed) + (sunglint)
__global__ void k_adj_pixel(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int p0, int t0)
{
    extern __shared__ double psm[];          // suffix of lev_j1 [nt + 2]
    __shared__ double dir[2];
    const int q = p0 + blockIdx.x / A.ncot, r = blockIdx.x % A.ncot;
    const PixDev &d = B.px[q];
    const int nt = d.nt, M = d.M, N = G.N, NR = G.NR;
    const double *cot = A.cot + ((size_t)q * A.ncot + r) * 3;
    auto gout = [&](int m) -> const double * {
        const int tl = d.task0 + m - t0;
        return A.gout + ((size_t)tl * A.ncot + r) * A.gstride;
    };
    for (int k = threadIdx.x; k <= nt; k += blockDim.x) {
        double v = 0.0;
        for (int m = 0; m <= M; ++m) v += gout(m)[A.kstride + k];
        psm[k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // warp 0: the suffix sums and the per-pixel terms, modes over lanes
        const unsigned full = 0xffffffffu;
        const int lane = threadIdx.x;
        // psm[k] = sum_{k' >= k} psm[k']: each lane takes a contiguous segment
        // of levels, the segment totals are combined by a warp suffix scan
        const int L1 = nt + 1, seg = (L1 + 31) / 32;
        const int k0 = min(L1, lane * seg), k1 = min(L1, k0 + seg);
        double part = 0.0;
        for (int k = k1 - 1; k >= k0; --k) part += psm[k];
        double incl = part;
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_down_sync(full, incl, o);
            if (lane + o < 32) incl += v;
        }
        double acc = __shfl_down_sync(full, incl, 1);
        if (lane == 31) acc = 0.0;
        for (int k = k1 - 1; k >= k0; --k) { acc += psm[k]; psm[k] = acc; }
        if (lane == 0) psm[nt + 1] = 0.0;
        // direct terms: the removed view seed and the sunglint
        double dt = 0.0, dw = 0.0, seed_sum = 0.0, gw_sum = 0.0;
        for (int m = lane; m <= M; m += 32) {
            seed_sum += gout(m)[3 * A.kstride + 1];
            gw_sum += gout(m)[3 * A.kstride + 0];
        }
        dt -= seed_sum / d.mu0;
        dw += gw_sum;
        if (d.rough) {
            const double tdn = exp(-d.tau_total / d.mu0);
            int cols[2]; double cw[2]; int nc;
            if (d.view_slot >= 0) { cols[0] = d.view_slot; cw[0] = 1.0; nc = 1; }
            else {
                int lo, hi; double t;
                bracket_a(B.gmu, N, d.mu_view, lo, hi, t);
                cols[0] = lo; cw[0] = 1.0 - t; cols[1] = hi; cw[1] = t; nc = 2;
            }
            for (int m = lane; m <= M; m += 32) {
                const TaskDev &tk = B.tasks[d.task0 + m];
                double w[3];
                mode_weights(d, m, cot, w);
                const double fs = (m == 0 ? OCRT_PI : 0.5 * OCRT_PI) * d.mu0;
                const float *Rs = W.srf + tk.srf_off + (size_t)NR * N * 9;
                const float *RsW = A.srfW + tk.srf_off + (size_t)NR * N * 9;
                for (int cc = 0; cc < nc; ++cc) {
                    const int gg = cols[cc];
                    const double mug = gg < N ? B.gmu[gg] : d.mu_view;
                    const double E = (double)B.Eatt[d.lev_off * NR + gg];
                    for (int s = 0; s < 3; ++s) {
                        const double sv = cw[cc] * fs * tdn * E * (double)Rs[gg * 9 + s * 3];
                        const double svw = cw[cc] * fs * tdn * E * (double)RsW[gg * 9 + s * 3];
                        dt += w[s] * sv * (1.0 / d.mu0 + 1.0 / mug);
                        dw -= w[s] * svw;
                    }
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            dt += __shfl_xor_sync(full, dt, o);
            dw += __shfl_xor_sync(full, dw, o);
        }
        if (d.rough && !d.decouple) {
            // lanes 0, 1, 2: the sunglint at W, W + h, W - h
            const double phi_v = (d.raa_deg - 180.0) * OCRT_PI / 180.0;
            const double mv = d.vza_deg > 0.0 ? d.mu_view : 1.0;
            const double hW = 1e-5 * d.wind;
            double gl[3] = {0.0, 0.0, 0.0};
            if (lane < 3) {
                PixDev dv = d;
                dv.wind = lane == 0 ? d.wind : lane == 1 ? d.wind + hW : d.wind - hW;
                sunglint(dv, mv, phi_v, d.tau_total, gl);
            }
            const double yv = cot[0] * gl[0] + cot[1] * gl[1] - cot[2] * gl[2];
            const double yp = __shfl_sync(full, yv, 1), ym = __shfl_sync(full, yv, 2);
            dt -= yv * (1.0 / d.mu0 + 1.0 / mv);
            dw += (yp - ym) / (2.0 * hW);
        }
        if (lane == 0) {
            dir[0] = dt;
            dir[1] = dw;
        }
    }
    __syncthreads();
    double *out = A.grad + ((size_t)q * A.ncot + r) * A.grad_stride;
    const double *xd = B.xd + d.lev_off, *yd = B.yd + d.lev_off;
    for (int l = threadIdx.x; l < nt; l += blockDim.x) {
        double lay = 0.0, lss = 0.0;
        for (int m = 0; m <= M; ++m) {
            const double *go = gout(m);
            lay += go[2 * A.kstride + l];
            lss += go[l + 1];
        }
        out[l] = lay - psm[l + 1] / d.mu0 + dir[0];
        const double w = xd[l + 1] + yd[l + 1];
        out[nt + l] = w > 0.0 ? lss / w : 0.0;
    }
    if (threadIdx.x == 0) out[2 * nt] = dir[1];
}
