// sos.cu — the successive-orders loop on the GPU.
//
//   k_primary      direct-beam source (rt_primary_source.c:17-198), flat-surface
//                  reflected-beam source (rt_surface_boundary.c:210-428) and the
//                  rough direct-beam seed (rt_surface_boundary.c:430-493), then
//                  the formal solution of order 1 (rt_layer_transport.c:107-208).
//   k_source_simt  aerosol part of the multiple-scattering source, J = x * (A F) over all
//                  levels (rt_sos_operator.c:206-424), tiled FP32 GEMM on CUDA cores (used
//                  where the tcgen05 kernel's shape rules do not hold).
//   k_mol_lowrank  molecular part for m <= 2, J += y * U (V F) with the rank-24 factored
//                  molecular operator.
//   k_scan         surface boundary condition (rt_surface_boundary.c:137-208),
//                  up/down formal solution, order totals (double-float at the TOA
//                  and BOA, FP32 elsewhere), FP32 sup-norm residual and the
//                  convergence test (rt_solver.c:2178-2197, 2923-3150).
//   k_extract      TOA view sample and BOA downward samples (rt_solver.c:1010-1076).
#include "kernels.cuh"
#include "physics.cuh"

// Rough direct-beam seed at level k for upward slot g, Stokes s:
// (pi or pi/2) mu0 exp(-tau/mu0) exp(-(tau-h_k)/mu_g) R_m(mu_g, mu0)[s,I]
// (rt_surface_boundary.c:430-493).  fs_tdn = (pi or pi/2) mu0 exp(-tau/mu0),
// formed once per task in FP64 and rounded; the product is FP32 like the field.
__device__ inline float rough_seed(const TaskDev &tk, const WaveBufs &W, const BatchBufs &B, const PixDev &d,
                                   const Geom &G, float fs_tdn, int k, int g, int s)
{
    const float *Rs = W.srf + tk.srf_off + (size_t)G.NR * G.N * 9;
    return fs_tdn * B.Eatt[(d.lev_off + k) * G.NR + g] * Rs[g * 9 + s * 3];
}

__device__ inline float seed_scale(const PixDev &d, const TaskDev &tk)
{
    return (float)((tk.m == 0 ? OCRT_PI : 0.5 * OCRT_PI) * d.mu0 * exp(-d.tau_total / d.mu0));
}

__global__ void __launch_bounds__(512, 1) k_primary(BatchBufs B, WaveBufs W, Geom G, int t0)
{
    const int tl = blockIdx.x, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int c = threadIdx.x;
    if (c == 0) {
        TaskState st;
        st.orders = 1;
        st.active = d.max_orders > 1;
        st.converged = d.max_orders <= 1;
        st.pad_ = 0;
        st.resid = 0.0;
        B.state[tg] = st;
        if (st.active) queue_next(B, 2, tl, tk.has_mol, d.nt + 1);
    }
    if (c >= G.COUT) return;
    int s, h, g;
    decode_col(G, c, s, h, g);
    if (g >= d.n_ring) return;
    const int nt = d.nt;
    const float *pv = W.pvec + (size_t)tl * 2 * G.LDC;
    const double aP = pv[c], mP = pv[G.LDC + c];
    float *F = W.F + tk.fld_off;
    float *Tot = W.Tot + tk.fld_off;
    const double *hh = B.h + d.lev_off;
    const float *Tc = B.Tc + d.coef_off, *Ca = B.Ca + d.coef_off, *Cb = B.Cb + d.coef_off;
    const int NR = G.NR;
    // flat reflected beam: Stokes s uses kernel components (s, s+3)
    double RI = 0, RQ = 0, sb = 0, fa1 = 0, fa2 = 0, fm1 = 0, fm2 = 0;
    if (d.flat) {
        const double n2 = d.n_water * d.n_water, mu0 = d.mu0;
        const double tn = sqrt(n2 - 1.0 + mu0 * mu0);
        const double rp = (n2 * mu0 - tn) / (n2 * mu0 + tn), rs = (mu0 - tn) / (mu0 + tn);
        RI = (rp * rp + rs * rs) / 2.0;
        RQ = d.q_conv == 1 ? (rp * rp - rs * rs) / 2.0 : (rs * rs - rp * rp) / 2.0;
        sb = 0.5 * exp(-2.0 * d.tau_total / mu0);
        const int side = h == 0 ? 0 : 1;
        const float *fv = W.fvec + (size_t)tl * 2 * 2 * 6 * NR;
        const float *fa = fv + (size_t)(side * 2 + 0) * 6 * NR;
        const float *fm = fv + (size_t)(side * 2 + 1) * 6 * NR;
        fa1 = fa[s * NR + g]; fa2 = fa[(s + 3) * NR + g];
        fm1 = fm[s * NR + g]; fm2 = fm[(s + 3) * NR + g];
    }
    int bad = 0;
    // an atmosphere driven only by a bottom source has no solar primary and no
    // surface seeds (rt_solver.c:949-954, rt_surface_boundary.c:553-569)
    const float faP = d.bottom_only ? 0.f : (float)aP, fmP = d.bottom_only ? 0.f : (float)mP;
    const float fs_tdn = d.rough ? seed_scale(d, tk) : 0.f;
    // rough direct-beam seed (rt_surface_boundary.c:430-493) on upward columns:
    // fs_tdn exp(-(tau-h_k)/mu_g) R_m(mu_g, mu0)[s, I], the attenuation per level from Eatt
    const bool seeded = d.rough && h == 0 && !d.bottom_only;
    const float rs = seeded ? W.srf[tk.srf_off + (size_t)G.NR * G.N * 9 + g * 9 + s * 3] : 0.f;
    // water column: the skylight's first-scatter source, computed into J by the
    // source pass over the unscattered skylight field (k_dtop_field)
    const float *Jdt = (d.medium == 1 && d.ext_off >= 0 && tk.m <= d.ext_mmax) ? W.J + tk.fld_off : nullptr;
    // atmosphere over the ocean: upward bottom source ext[m][g][s] attenuated
    // upward, part of order 1 and of the total (rt_surface_boundary.c:495-527)
    const bool extb = d.medium == 0 && d.ext_off >= 0 && h == 0 && tk.m <= d.ext_mmax;
    const float exv = extb ? (float)B.ext[d.ext_off + ((size_t)tk.m * G.NR + g) * 3 + s] : 0.f;
    // Step j visits level nt - j (upward) or j (downward); the per-level inputs
    // of PF steps are loaded before the dependent recurrence runs.
    constexpr int PF = 4;
    float I = 0.f, Jp = 0.f;
    for (int j0 = 0; j0 <= nt; j0 += PF) {
        const int cnt = nt - j0 + 1 < PF ? nt - j0 + 1 : PF;
        float lx[PF], ly[PF], lc[PF], tv[PF], av[PF], bv[PF], ea[PF];
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            if (q < cnt) {
                const int j = j0 + q, k = h == 0 ? nt - j : j;
                const float *lv = B.lvf + 3 * (d.lev_off + k);
                lx[q] = lv[0]; ly[q] = lv[1]; lc[q] = lv[2];
                if (j > 0) {
                    const int e = (h == 0 ? k : k - 1) * NR + g;
                    tv[q] = Tc[e]; av[q] = Ca[e]; bv[q] = Cb[e];
                }
                ea[q] = (seeded || extb) ? B.Eatt[(d.lev_off + k) * NR + g] : 0.f;
            }
        }
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            if (q < cnt) {
                const int j = j0 + q, k = h == 0 ? nt - j : j;
                float Jk = prim_source(lc[q], lx[q], ly[q], faP, fmP);
                if (Jdt) Jk = __fadd_rn(Jk, Jdt[(size_t)k * G.LDC + c]);
                if (d.flat && !d.bottom_only && ((h == 0 && k < nt) || (h == 1 && k >= 1))) {
                    const double beam = sb * exp(hh[k] / d.mu0);
                    Jk += (float)(beam * (RI * (lx[q] * fa1 + ly[q] * fm1) + RQ * (lx[q] * fa2 + ly[q] * fm2)));
                }
                if (!isfinite(Jk)) bad = 1;
                if (j > 0) I = prim_step(tv[q], I, av[q], Jk, bv[q], Jp);
                Jp = Jk;
                float2 t = make_float2(I, 0.f);
                if (seeded) t = df_add(t, __fmul_rn(__fmul_rn(fs_tdn, ea[q]), rs));
                if (extb) t = df_add(t, __fmul_rn(exv, ea[q]));
                F[(size_t)k * G.LDC + c] = t.x;
                if (G.tot_all || k == 0 || k == nt) Tot[(size_t)k * G.LDC + c] = t.x;
                if (k == 0 || k == nt) W.Ttl[tot_tail_off(tk, G, k, c)] = t.y;
            }
        }
    }
    if (bad) atomicExch(B.err, -2);
}

// Order 1 with four Gauss columns per thread (columns s*2N + h*N + 4q .. +3,
// N a multiple of 4) and one zero-weight column per thread, for groups with
// no flat surface.  Per column the arithmetic is k_primary's in the same
// order; the per-level weights come from the quad table (16-byte loads for a
// quad), and the field and total rows are written as 16-byte stores.
template <int WD>
__device__ __forceinline__ void primary_cols(const BatchBufs &B, const WaveBufs &W, const Geom &G, const TaskDev &tk,
                                             const PixDev &d, int tl, int c, int s, int h, int g, int &bad)
{
    const int nt = d.nt, NR = G.NR, N = G.N;
    const float *pv = W.pvec + (size_t)tl * 2 * G.LDC + c;
    float faP[WD], fmP[WD], rs[WD], exv[WD];
    const bool seeded = d.rough && h == 0 && !d.bottom_only;
    const bool extb = d.medium == 0 && d.ext_off >= 0 && h == 0 && tk.m <= d.ext_mmax;
    const float fs_tdn = d.rough ? seed_scale(d, tk) : 0.f;
#pragma unroll
    for (int u = 0; u < WD; ++u) {
        faP[u] = d.bottom_only ? 0.f : pv[u];
        fmP[u] = d.bottom_only ? 0.f : pv[G.LDC + u];
        rs[u] = seeded ? W.srf[tk.srf_off + (size_t)NR * N * 9 + (g + u) * 9 + s * 3] : 0.f;
        exv[u] = extb ? (float)B.ext[d.ext_off + ((size_t)tk.m * NR + g + u) * 3 + s] : 0.f;
    }
    const float *Jdt = (d.medium == 1 && d.ext_off >= 0 && tk.m <= d.ext_mmax) ? W.J + tk.fld_off + c : nullptr;
    float *Fp = W.F + tk.fld_off + c, *Tp = W.Tot + tk.fld_off + c;
    const int cw = coef_quad_width(NR);
    const float *cq = B.Cq + coef_quad_off(d.coef_off, N, NR) + (g >> 2) * 12 + (g & 3);
    const float *lvb = B.lvf + 3 * d.lev_off;
    const float *eab = B.Eatt + d.lev_off * NR + g;
    float I[WD], Jp[WD];
#pragma unroll
    for (int u = 0; u < WD; ++u) { I[u] = 0.f; Jp[u] = 0.f; }
    constexpr int PF = WD == 4 ? 2 : 4;
    for (int j0 = 0; j0 <= nt; j0 += PF) {
        const int cnt = nt - j0 + 1 < PF ? nt - j0 + 1 : PF;
        float lx[PF], ly[PF], lc[PF], tv[PF][WD], av[PF][WD], bv[PF][WD], ea[PF][WD], jd[PF][WD];
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            if (q < cnt) {
                const int j = j0 + q, k = h == 0 ? nt - j : j;
                const float *lv = lvb + 3 * k;
                lx[q] = lv[0]; ly[q] = lv[1]; lc[q] = lv[2];
                if (j > 0) {
                    const float *w = cq + (size_t)(h == 0 ? k : k - 1) * cw;
                    if (WD == 4) {
                        const float4 t4 = *reinterpret_cast<const float4 *>(w);
                        const float4 a4 = *reinterpret_cast<const float4 *>(w + 4);
                        const float4 b4 = *reinterpret_cast<const float4 *>(w + 8);
                        tv[q][0] = t4.x; tv[q][WD > 1 ? 1 : 0] = t4.y; tv[q][WD > 2 ? 2 : 0] = t4.z; tv[q][WD - 1] = t4.w;
                        av[q][0] = a4.x; av[q][WD > 1 ? 1 : 0] = a4.y; av[q][WD > 2 ? 2 : 0] = a4.z; av[q][WD - 1] = a4.w;
                        bv[q][0] = b4.x; bv[q][WD > 1 ? 1 : 0] = b4.y; bv[q][WD > 2 ? 2 : 0] = b4.z; bv[q][WD - 1] = b4.w;
                    } else {
                        tv[q][0] = w[0]; av[q][0] = w[4]; bv[q][0] = w[8];
                    }
                }
#pragma unroll
                for (int u = 0; u < WD; ++u) ea[q][u] = (seeded || extb) ? eab[(size_t)k * NR + u] : 0.f;
                if (Jdt) {
                    if (WD == 4) {
                        const float4 x = *reinterpret_cast<const float4 *>(Jdt + (size_t)k * G.LDC);
                        jd[q][0] = x.x; jd[q][WD > 1 ? 1 : 0] = x.y; jd[q][WD > 2 ? 2 : 0] = x.z; jd[q][WD - 1] = x.w;
                    } else {
                        jd[q][0] = Jdt[(size_t)k * G.LDC];
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            if (q < cnt) {
                const int j = j0 + q, k = h == 0 ? nt - j : j;
                float tx[WD], ty[WD];
#pragma unroll
                for (int u = 0; u < WD; ++u) {
                    float Jk = prim_source(lc[q], lx[q], ly[q], faP[u], fmP[u]);
                    if (Jdt) Jk = __fadd_rn(Jk, jd[q][u]);
                    if (!isfinite(Jk)) bad = 1;
                    if (j > 0) I[u] = prim_step(tv[q][u], I[u], av[q][u], Jk, bv[q][u], Jp[u]);
                    Jp[u] = Jk;
                    float2 t = make_float2(I[u], 0.f);
                    if (seeded) t = df_add(t, __fmul_rn(__fmul_rn(fs_tdn, ea[q][u]), rs[u]));
                    if (extb) t = df_add(t, __fmul_rn(exv[u], ea[q][u]));
                    tx[u] = t.x; ty[u] = t.y;
                }
                const size_t o = (size_t)k * G.LDC;
                const bool wt = G.tot_all || k == 0 || k == nt;
                if (WD == 4) {
                    const float4 v = make_float4(tx[0], tx[WD > 1 ? 1 : 0], tx[WD > 2 ? 2 : 0], tx[WD - 1]);
                    *reinterpret_cast<float4 *>(Fp + o) = v;
                    if (wt) *reinterpret_cast<float4 *>(Tp + o) = v;
                } else {
                    Fp[o] = tx[0];
                    if (wt) Tp[o] = tx[0];
                }
                if (k == 0 || k == nt) {
#pragma unroll
                    for (int u = 0; u < WD; ++u) W.Ttl[tot_tail_off(tk, G, k, c + u)] = ty[u];
                }
            }
        }
    }
}

__global__ void __launch_bounds__(128, 4) k_primary4(BatchBufs B, WaveBufs W, Geom G, int t0)
{
    const int tl = blockIdx.x, tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int tid = threadIdx.x, N = G.N, nq = 6 * N / 4;
    if (tid == 0) {
        TaskState st;
        st.orders = 1;
        st.active = d.max_orders > 1;
        st.converged = d.max_orders <= 1;
        st.pad_ = 0;
        st.resid = 0.0;
        B.state[tg] = st;
        if (st.active) queue_next(B, 2, tl, tk.has_mol, d.nt + 1);
    }
    int bad = 0;
    int s, h, g;
    if (tid < nq) {
        const int c = 4 * tid;
        decode_col(G, c, s, h, g);
        primary_cols<4>(B, W, G, tk, d, tl, c, s, h, g, bad);
    } else if (tid < nq + 6 * G.E) {
        const int c = 6 * N + (tid - nq);
        decode_col(G, c, s, h, g);
        if (g < d.n_ring) primary_cols<1>(B, W, G, tk, d, tl, c, s, h, g, bad);
    }
    if (bad) atomicExch(B.err, -2);
}

// Tiled SIMT GEMM: per task, J[k][c] = x_k * sum_i F[k][col(i)] A[i][c] + y_k * (... B ...).
// Tile 64 levels x 64 output columns, 256 threads, 4x4 outputs per thread.
#define ST_K 16
#define ST_M 64
#define ST_N 64
__global__ void __launch_bounds__(256) k_source_simt(BatchBufs B, WaveBufs W, Geom G, int t0, int it)
{
    if ((int)blockIdx.x >= B.active_cnt[it - 1]) return;
    const int tl = B.alist[it & 1][blockIdx.x], tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt;
    const int k0 = blockIdx.y * ST_M, c0 = blockIdx.z * ST_N;
    if (k0 > nt || c0 >= G.COUT) return;
    __shared__ float Fs[ST_K][ST_M + 4];
    __shared__ float As[ST_K][ST_N + 4];
    const float *F = W.F + tk.fld_off;
    const float *A = W.ops + tk.op_off;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float accA[4][4] = {{0}};
    for (int kc = 0; kc < G.CIN; kc += ST_K) {
        for (int idx = threadIdx.x; idx < ST_M * ST_K; idx += 256) {
            const int lv = idx / ST_K, kk = idx - lv * ST_K;
            const int k = k0 + lv, ci = kc + kk;
            const size_t o = (size_t)k * G.LDC + in_to_col(G, ci);
            Fs[kk][lv] = (k <= nt && ci < G.CIN) ? F[o] : 0.f;
        }
        for (int idx = threadIdx.x; idx < ST_K * ST_N; idx += 256) {
            const int cc = idx / ST_K, kk = idx - cc * ST_K;
            const int ci = kc + kk, co = c0 + cc;
            const bool ok = ci < G.CIN && co < G.NP;
            As[kk][cc] = ok ? A[(size_t)co * G.CIN + ci] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < ST_K; ++kk) {
            float fr[4], ar[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) fr[i] = Fs[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) ar[j] = As[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) accA[i][j] = fmaf(fr[i], ar[j], accA[i][j]);
        }
        __syncthreads();
    }
    float *J = W.J + tk.fld_off;
    const double *xd = B.xd + d.lev_off;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int k = k0 + ty + 16 * i;
        if (k > nt) continue;
        const float x = (float)xd[k];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tx + 16 * j;
            if (c < G.COUT) J[(size_t)k * G.LDC + c] = x * accA[i][j];
        }
    }
}

// Molecular source for m <= 2 tasks: xi[k][4b+f] = sum_i w_i f(mu_i) F[k][bN+i]
// (f in {1, P2m, R2m, T2m}), then J[k][c] += y_k sum_r U[c][r] xi[k][r].
// Grid (task in list, tile of 32 levels), 256 threads.
__global__ void __launch_bounds__(256) k_mol_lowrank(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int ltiles,
                                                     const float *Bp, const float *Br, const float *Bt, int L)
{
    extern __shared__ float sm[];
    __shared__ int item_s;
    const int n_items = B.mol_cnt[it - 1] * ltiles;
    for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) item_s = atomicAdd(&B.work[it * 4 + 1], 1);
    __syncthreads();
    const int item = item_s;
    if (item >= n_items) return;
    const int tl = B.mlist[it & 1][item / ltiles], tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt, N = G.N, k0 = (item % ltiles) * 32;
    if (k0 > nt) continue;
    const int nk = min(32, nt - k0 + 1);
    float *fv = sm;                          // [4][N]
    float *U = fv + 4 * N;                   // [COUT][24]
    float *Fs = U + G.COUT * 24;             // [32][6N]
    float *xi = Fs + 32 * G.CIN;             // [32][25]
    const size_t gb = (size_t)tk.m * (L + 1) * N + (size_t)2 * N;    // degree-2 row of mode m
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float w = (float)B.gw[i];
        fv[i] = w; fv[N + i] = w * Bp[gb + i]; fv[2 * N + i] = w * Br[gb + i]; fv[3 * N + i] = w * Bt[gb + i];
    }
    const float *Ug = W.ops + tk.mol_off;
    for (int e = threadIdx.x; e < G.COUT * 24; e += blockDim.x) U[e] = Ug[e];
    const float *F = W.F + tk.fld_off + (size_t)k0 * G.LDC;
    for (int e = threadIdx.x; e < nk * G.CIN; e += blockDim.x) {
        const int k = e / G.CIN, ci = e - k * G.CIN;
        const size_t o = (size_t)k * G.LDC + ci;
        Fs[k * G.CIN + ci] = F[o];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nk * 24; e += blockDim.x) {
        const int k = e / 24, r = e - k * 24, b = r >> 2, f = r & 3;
        const float *fr = Fs + k * G.CIN + b * N;
        const float *ff = fv + f * N;
        float acc = 0.f;
        for (int i = 0; i < N; ++i) acc = fmaf(ff[i], fr[i], acc);
        xi[k * 25 + r] = acc;
    }
    __syncthreads();
    float *J = W.J + tk.fld_off;
    for (int e = threadIdx.x; e < nk * G.COUT; e += blockDim.x) {
        const int k = e / G.COUT, c = e - k * G.COUT;
        const float *u = U + c * 24, *x = xi + k * 25;
        float acc = 0.f;
#pragma unroll
        for (int r = 0; r < 24; ++r) acc = fmaf(u[r], x[r], acc);
        J[(size_t)(k0 + k) * G.LDC + c] += B.lvf[3 * (d.lev_off + k0 + k) + 1] * acc;
    }
    }
}

// Block-wide maxima of two values at once (thread 0 holds the result).
__device__ inline float2 block_maxf2(float a, float b, float2 *red)
{
    for (int o = 16; o > 0; o >>= 1) {
        a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = make_float2(a, b);
    __syncthreads();
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        const float2 v = l < nw ? red[l] : make_float2(0.f, 0.f);
        a = v.x; b = v.y;
        for (int o = 16; o > 0; o >>= 1) {
            a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
    }
    return make_float2(a, b);
}

__device__ inline double block_max(double v, double *red)
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

__global__ void __launch_bounds__(512, 2) k_scan(BatchBufs B, WaveBufs W, Geom G, int t0, int it)
{
    __shared__ float2 redf2[32];
    extern __shared__ float scan_smem[];
    __shared__ int item_s;
    const int n_items = B.active_cnt[it - 1];
    for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) item_s = atomicAdd(&B.work[it * 4 + 2], 1);
    __syncthreads();
    if (item_s >= n_items) return;
    const int tl = B.alist[it & 1][item_s], tg = t0 + tl;
    const TaskState st = B.state[tg];
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int c = threadIdx.x, nt = d.nt, N = G.N, NR = G.NR;
    int s = 0, h = 0, g = 0;
    if (c < G.COUT) decode_col(G, c, s, h, g);
    const bool valid = c < G.COUT && g < d.n_ring;
    float *F = W.F + tk.fld_off;
    const float *J = W.J + tk.fld_off;
    float *Tot = W.Tot + tk.fld_off;
    // Each column walks its nt + 1 levels in its transport direction (step
    // j: level nt - j upward, j downward).  The J, total and coefficient
    // values of the next SCAN_DEPTH steps are in flight as cp.async copies
    // into this thread's own shared-memory slots, so the recurrence never
    // waits on a memory round trip; a slot is refilled only after the
    // values read from it have been used.
    const int bs = blockDim.x;
    float *Js = scan_smem;                                             // [SCAN_DEPTH][bs]
    float *Ts = Js + SCAN_DEPTH * bs;                                  // [SCAN_DEPTH][bs]
    float *Cs = Ts + SCAN_DEPTH * bs;                                  // [SCAN_DEPTH][3][bs]
    const float *Tc = B.Tc + d.coef_off, *Ca = B.Ca + d.coef_off, *Cb = B.Cb + d.coef_off;
    auto issue = [&](int j) {
        if (j <= nt) {
            const int k = h == 0 ? nt - j : j, sl = j & (SCAN_DEPTH - 1);
            const size_t o = (size_t)k * G.LDC + c;
            cp_async4(Js + sl * bs + c, J + o);
            if (G.tot_all || k == 0 || k == nt) cp_async4(Ts + sl * bs + c, Tot + o);
            if (j > 0) {
                const int e = (h == 0 ? k : k - 1) * NR + g;
                cp_async4(Cs + (sl * 3 + 0) * bs + c, Tc + e);
                cp_async4(Cs + (sl * 3 + 1) * bs + c, Ca + e);
                cp_async4(Cs + (sl * 3 + 2) * bs + c, Cb + e);
            }
        }
        cp_async_commit();
    };
    // tails of the TOA and BOA totals (double-float output levels)
    float *tl0 = W.Ttl + tot_tail_off(tk, G, 0, c), *tlN = W.Ttl + tot_tail_off(tk, G, nt, c);
    float lo0 = 0.f, loN = 0.f;
    // the first ring copies and the tails are in flight while the boundary
    // condition below is summed (they read J and the totals, not F)
    if (valid) {
#pragma unroll
        for (int j = 0; j < SCAN_DEPTH; ++j) issue(j);
        lo0 = *tl0; loN = *tlN;
    }
    // ---- surface boundary condition from the previous order's BOA downward field
    // (atmosphere), or the internal reflection at the water surface of the
    // previous order's upward field at the top (water column, rt_solver.c:2788-2815)
    float bc = 0.f;
    const bool water = d.medium == 1;
    if (valid && water && h == 1) {
        const float *R = W.srf + tk.srf_off + (size_t)g * N * 9 + s * 3;
        const float *pwm = B.pw + (tk.m == 0 ? 0 : N);
        float acc = 0.f;
        for (int i = 0; i < N; ++i) {
            const float *Ri = R + (size_t)i * 9;
            acc += pwm[i] * (Ri[0] * F[col_of(G, 0, 0, i)] + Ri[1] * F[col_of(G, 1, 0, i)] +
                             Ri[2] * F[col_of(G, 2, 0, i)]);
        }
        bc = acc;
    } else if (valid && h == 0 && d.surf_on) {
        const float *Fbot = F + (size_t)nt * G.LDC;
        auto Fb = [&](int col) -> float { return Fbot[col]; };
        if (d.rough) {
            const float *R = W.srf + tk.srf_off + (size_t)g * N * 9 + s * 3;
            const float *pwm = B.pw + (tk.m == 0 ? 0 : N);
            float acc = 0.f;
            for (int i = 0; i < N; ++i) {
                const float pw = pwm[i];
                const float *Ri = R + (size_t)i * 9;
                acc += pw * (Ri[0] * Fb(col_of(G, 0, 1, i)) + Ri[1] * Fb(col_of(G, 1, 1, i)) +
                             Ri[2] * Fb(col_of(G, 2, 1, i)));
            }
            bc = acc;
        } else {
            const float *MF = B.frs + ((size_t)tk.pix * NR + g) * 9 + s * 3;
            bc = MF[0] * Fb(col_of(G, 0, 1, g)) + MF[1] * Fb(col_of(G, 1, 1, g)) + MF[2] * Fb(col_of(G, 2, 1, g));
        }
    }
    __syncthreads();
    // sup norms in FP32: the order field over every level; the total over
    // the output levels (TOA and BOA), whose heads carry it to 2^-24 relative
    float mi = 0.f, mt = 0.f;
    int bad = 0;
    if (valid) {
        float I = (water ? h == 1 : h == 0) ? bc : 0.f, Jp = 0.f;
        for (int j = 0; j <= nt; ++j) {
            cp_async_wait<SCAN_DEPTH - 1>();
            const int k = h == 0 ? nt - j : j, sl = j & (SCAN_DEPTH - 1);
            const float jv = Js[sl * bs + c];
            if (j > 0)
                I = Cs[(sl * 3 + 0) * bs + c] * I + Cs[(sl * 3 + 1) * bs + c] * jv + Cs[(sl * 3 + 2) * bs + c] * Jp;
            Jp = jv;
            const size_t o = (size_t)k * G.LDC + c;
            F[o] = I;
            if (k == 0 || k == nt) {
                const float ov = Ts[sl * bs + c];
                const float2 td = df_add(make_float2(ov, k == 0 ? lo0 : loN), I);
                Tot[o] = td.x;
                *(k == 0 ? tl0 : tlN) = td.y;
                mt = fmaxf(mt, fabsf(td.x));
            } else if (G.tot_all) {
                Tot[o] = Ts[sl * bs + c] + I;
            }
            mi = fmaxf(mi, fabsf(I));
            issue(j + SCAN_DEPTH);
        }
        cp_async_wait<0>();
        bad = !isfinite(I);
    }
    if (bad) atomicExch(B.err, -2);
    const float2 mm = block_maxf2(mi, mt, redf2);
    mi = mm.x; mt = mm.y;
    if (threadIdx.x == 0) {
        TaskState ns = st;
        ns.orders = it;
        ns.resid = mt > 0.f ? (double)(mi / mt) : 0.0;
        if (ns.resid < d.tol) { ns.converged = 1; ns.active = 0; }
        else if (it >= d.max_orders) ns.active = 0;
        B.state[tg] = ns;
        if (ns.active) queue_next(B, it + 1, tl, tk.has_mol, d.nt + 1);
    }
    }
}

// The same order step as k_scan with four Gauss columns per thread.  Columns
// s*2N + h*N + 4q .. +3 share the Stokes index and the direction (N is a
// multiple of 4), so one thread runs their four recurrences side by side and
// every per-level value arrives as one 16-byte copy: J, the total's head, and
// T, Ca, Cb of the four ring slots from the quad layout of k_coef_quads.  The
// zero-weight columns (6E of them) take one thread each with 4-byte copies.
// Per column the arithmetic is k_scan's, in the same order.
__global__ void __launch_bounds__(128, 4) k_scan4(BatchBufs B, WaveBufs W, Geom G, int t0, int it)
{
    __shared__ float2 redf2[32];
    extern __shared__ float4 scan4_smem[];
    __shared__ int item_s;
    const int n_items = B.active_cnt[it - 1];
    const int tid = threadIdx.x, bs = blockDim.x, N = G.N, NR = G.NR, nq = 6 * N / 4;
    const bool quad = tid < nq, single = !quad && tid < nq + 6 * G.E;
    int s = 0, h = 0, g = 0, c = 0;
    if (quad) { c = 4 * tid; decode_col(G, c, s, h, g); }
    else if (single) { c = 6 * N + (tid - nq); decode_col(G, c, s, h, g); }
    float4 *R = scan4_smem;   // [SCAN4_DEPTH][5][bs]: J, total, T, Ca, Cb
    auto slot = [&](int sl, int f) -> float4 * { return R + ((size_t)sl * 5 + f) * bs + tid; };
    for (;;) {
    __syncthreads();
    if (tid == 0) item_s = atomicAdd(&B.work[it * 4 + 2], 1);
    __syncthreads();
    if (item_s >= n_items) return;
    const int tl = B.alist[it & 1][item_s], tg = t0 + tl;
    const TaskState st = B.state[tg];
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt;
    const bool valid = quad || (single && g < d.n_ring);
    float *F = W.F + tk.fld_off;
    const float *J = W.J + tk.fld_off;
    float *Tot = W.Tot + tk.fld_off;
    const float *Tc = B.Tc + d.coef_off, *Ca = B.Ca + d.coef_off, *Cb = B.Cb + d.coef_off;
    const float *Cq = B.Cq + coef_quad_off(d.coef_off, N, NR) + (size_t)(g >> 2) * 12;
    auto issue = [&](int j) {
        if (j <= nt) {
            const int k = h == 0 ? nt - j : j, sl = j & (SCAN4_DEPTH - 1);
            const size_t o = (size_t)k * G.LDC + c;
            const int layer = h == 0 ? k : k - 1;
            const bool wt = G.tot_all || k == 0 || k == nt;
            if (quad) {
                cp_async16_cg(slot(sl, 0), J + o);
                if (wt) cp_async16_cg(slot(sl, 1), Tot + o);
                if (j > 0) {
                    const float *q = Cq + (size_t)layer * coef_quad_width(NR);
                    cp_async16_ca(slot(sl, 2), q);
                    cp_async16_ca(slot(sl, 3), q + 4);
                    cp_async16_ca(slot(sl, 4), q + 8);
                }
            } else {
                cp_async4(&slot(sl, 0)->x, J + o);
                if (wt) cp_async4(&slot(sl, 1)->x, Tot + o);
                if (j > 0) {
                    const int e = layer * NR + g;
                    cp_async4(&slot(sl, 2)->x, Tc + e);
                    cp_async4(&slot(sl, 3)->x, Ca + e);
                    cp_async4(&slot(sl, 4)->x, Cb + e);
                }
            }
        }
        cp_async_commit();
    };
    const int ncol = quad ? 4 : 1;
    float *tl0 = W.Ttl + tot_tail_off(tk, G, 0, c), *tlN = W.Ttl + tot_tail_off(tk, G, nt, c);
    float lo0[4] = {0.f, 0.f, 0.f, 0.f}, loN[4] = {0.f, 0.f, 0.f, 0.f};
    if (valid) {
#pragma unroll
        for (int j = 0; j < SCAN4_DEPTH; ++j) issue(j);
        for (int q = 0; q < ncol; ++q) { lo0[q] = tl0[q]; loN[q] = tlN[q]; }
    }
    // boundary condition of each column (as in k_scan)
    float bc[4] = {0.f, 0.f, 0.f, 0.f};
    const bool water = d.medium == 1;
    if (valid && ((water && h == 1) || (!water && h == 0 && d.surf_on))) {
        const float *pwm = B.pw + (tk.m == 0 ? 0 : N);
        for (int q = 0; q < ncol; ++q) {
            const int gq = g + q;
            if (water || d.rough) {
                // water: internal reflection of the previous order's upward field at
                // the top; atmosphere: rough reflection of the downward field at the bottom
                const float *Rm = W.srf + tk.srf_off + (size_t)gq * N * 9 + s * 3;
                const float *Fr = water ? F : F + (size_t)nt * G.LDC;
                const int hin = water ? 0 : 1;
                float acc = 0.f;
                for (int i = 0; i < N; ++i) {
                    const float *Ri = Rm + (size_t)i * 9;
                    acc += pwm[i] * (Ri[0] * Fr[col_of(G, 0, hin, i)] + Ri[1] * Fr[col_of(G, 1, hin, i)] +
                                     Ri[2] * Fr[col_of(G, 2, hin, i)]);
                }
                bc[q] = acc;
            } else {
                const float *Fbot = F + (size_t)nt * G.LDC;
                const float *MF = B.frs + ((size_t)tk.pix * NR + gq) * 9 + s * 3;
                bc[q] = MF[0] * Fbot[col_of(G, 0, 1, gq)] + MF[1] * Fbot[col_of(G, 1, 1, gq)] +
                        MF[2] * Fbot[col_of(G, 2, 1, gq)];
            }
        }
    }
    __syncthreads();
    float mi = 0.f, mt = 0.f;
    int bad = 0;
    if (valid && quad) {
        const bool start = water ? h == 1 : h == 0;
        float4 I = start ? make_float4(bc[0], bc[1], bc[2], bc[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 Jp = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int j = 0; j <= nt; ++j) {
            cp_async_wait<SCAN4_DEPTH - 1>();
            const int k = h == 0 ? nt - j : j, sl = j & (SCAN4_DEPTH - 1);
            const float4 jv = *slot(sl, 0), ov = *slot(sl, 1);
            if (j > 0) {
                const float4 T = *slot(sl, 2), A = *slot(sl, 3), Bw = *slot(sl, 4);
                I.x = T.x * I.x + A.x * jv.x + Bw.x * Jp.x;
                I.y = T.y * I.y + A.y * jv.y + Bw.y * Jp.y;
                I.z = T.z * I.z + A.z * jv.z + Bw.z * Jp.z;
                I.w = T.w * I.w + A.w * jv.w + Bw.w * Jp.w;
            }
            Jp = jv;
            const size_t o = (size_t)k * G.LDC + c;
            *reinterpret_cast<float4 *>(F + o) = I;
            if (k == 0 || k == nt) {
                const bool top = k == 0;
                float *tp = top ? tl0 : tlN;
                const float2 a = df_add(make_float2(ov.x, top ? lo0[0] : loN[0]), I.x);
                const float2 b = df_add(make_float2(ov.y, top ? lo0[1] : loN[1]), I.y);
                const float2 e = df_add(make_float2(ov.z, top ? lo0[2] : loN[2]), I.z);
                const float2 f = df_add(make_float2(ov.w, top ? lo0[3] : loN[3]), I.w);
                tp[0] = a.y; tp[1] = b.y; tp[2] = e.y; tp[3] = f.y;
                const float4 t = make_float4(a.x, b.x, e.x, f.x);
                *reinterpret_cast<float4 *>(Tot + o) = t;
                mt = fmaxf(mt, fmaxf(fmaxf(fabsf(t.x), fabsf(t.y)), fmaxf(fabsf(t.z), fabsf(t.w))));
            } else if (G.tot_all) {
                *reinterpret_cast<float4 *>(Tot + o) = make_float4(ov.x + I.x, ov.y + I.y, ov.z + I.z, ov.w + I.w);
            }
            mi = fmaxf(mi, fmaxf(fmaxf(fabsf(I.x), fabsf(I.y)), fmaxf(fabsf(I.z), fabsf(I.w))));
            issue(j + SCAN4_DEPTH);
        }
        cp_async_wait<0>();
        bad = !(isfinite(I.x) && isfinite(I.y) && isfinite(I.z) && isfinite(I.w));
    } else if (valid) {
        float I = (water ? h == 1 : h == 0) ? bc[0] : 0.f, Jp = 0.f;
        for (int j = 0; j <= nt; ++j) {
            cp_async_wait<SCAN4_DEPTH - 1>();
            const int k = h == 0 ? nt - j : j, sl = j & (SCAN4_DEPTH - 1);
            const float jv = slot(sl, 0)->x, ov = slot(sl, 1)->x;
            if (j > 0) I = slot(sl, 2)->x * I + slot(sl, 3)->x * jv + slot(sl, 4)->x * Jp;
            Jp = jv;
            const size_t o = (size_t)k * G.LDC + c;
            F[o] = I;
            if (k == 0 || k == nt) {
                const float2 td = df_add(make_float2(ov, k == 0 ? lo0[0] : loN[0]), I);
                Tot[o] = td.x;
                *(k == 0 ? tl0 : tlN) = td.y;
                mt = fmaxf(mt, fabsf(td.x));
            } else if (G.tot_all) {
                Tot[o] = ov + I;
            }
            mi = fmaxf(mi, fabsf(I));
            issue(j + SCAN4_DEPTH);
        }
        cp_async_wait<0>();
        bad = !isfinite(I);
    }
    if (bad) atomicExch(B.err, -2);
    const float2 mm = block_maxf2(mi, mt, redf2);
    mi = mm.x; mt = mm.y;
    if (tid == 0) {
        TaskState ns = st;
        ns.orders = it;
        ns.resid = mt > 0.f ? (double)(mi / mt) : 0.0;
        if (ns.resid < d.tol) { ns.converged = 1; ns.active = 0; }
        else if (it >= d.max_orders) ns.active = 0;
        B.state[tg] = ns;
        if (ns.active) queue_next(B, it + 1, tl, tk.has_mol, d.nt + 1);
    }
    }
}

// Linear interpolation between the bracketing Gauss nodes (rt_solver.c:386-403).
__device__ inline void bracket(const double *gmu, int n, double mu, int &lo, int &hi, double &t)
{
    int jh = 1;
    while (jh < n && gmu[jh - 1] < mu) jh++;
    int jl = jh - 1;
    if (jl < 1) { jl = 1; jh = 2; }
    if (jh > n) { jh = n; jl = n - 1; }
    lo = jl - 1; hi = jh - 1;
    t = (mu - gmu[lo]) / (gmu[hi] - gmu[lo]);
}

__global__ void k_extract(BatchBufs B, WaveBufs W, Geom G, int t0, int nt_tasks)
{
    const int tl = blockIdx.x * blockDim.x + threadIdx.x;
    if (tl >= nt_tasks) return;
    const int tg = t0 + tl;
    const TaskDev tk = B.tasks[tg];
    const PixDev &d = B.px[tk.pix];
    const int nt = d.nt, N = G.N, vs = d.view_slot;
    const float fs_tdn = d.rough ? seed_scale(d, tk) : 0.f;
    auto up0 = [&](int s, int g) -> double {
        double v = tot_value(W, tk, G, 0, nt, col_of(G, s, 0, g));
        if (d.rough && !d.bottom_only) v -= (double)rough_seed(tk, W, B, d, G, fs_tdn, 0, g, s);
        return v;
    };
    auto dn = [&](int g) -> double { return tot_value(W, tk, G, nt, nt, col_of(G, 0, 1, g)); };
    TaskOut o;
    if (vs >= 0) {
        o.vI = up0(0, vs); o.vQ = up0(1, vs); o.vU = up0(2, vs);
        o.dn_view = dn(vs);
    } else {
        int lo, hi; double t;
        bracket(B.gmu, N, d.mu_view, lo, hi, t);
        o.vI = (1.0 - t) * up0(0, lo) + t * up0(0, hi);
        o.vQ = (1.0 - t) * up0(1, lo) + t * up0(1, hi);
        o.vU = (1.0 - t) * up0(2, lo) + t * up0(2, hi);
        o.dn_view = (1.0 - t) * dn(lo) + t * dn(hi);
    }
    double f = 0.0;
    for (int g = 0; g < N; ++g) f += B.gmu[g] * B.gw[g] * dn(g);
    o.fdn = f;
    B.tout[tg] = o;
}

// A graph replay runs each wave for the order count an eager execute
// recorded; this flags a replay that ends with a task still active.
__global__ void k_stop_check(const int *active_after_last, int *flag)
{
    if (threadIdx.x == 0 && *active_after_last != 0) atomicExch(flag, 1);
}

// Dense molecular operator for the tensor-core contraction:
// UV[c][bN + i] = sum_f U[c][4b + f] fv[f][i], fv[f][i] = w_i {1, P2m, R2m, T2m}(mu_i),
// so that UV F equals U (V F) of k_mol_lowrank.  Rows COUT..NP-1 are zero.
// One block per molecular task of the wave.
__global__ void k_mol_dense(const TaskDev *tasks, int t0, int nw, Geom G, int L, const float *Bp, const float *Br,
                            const float *Bt, const double *gw, const float *ops, float *opt)
{
    const int tl = blockIdx.x;
    if (tl >= nw) return;
    const TaskDev tk = tasks[t0 + tl];
    if (tk.uv_off < 0) return;
    const int N = G.N;
    __shared__ float fv[4 * OCRT_MAX_N];
    const size_t gb = (size_t)tk.m * (L + 1) * N + (size_t)2 * N;    // degree-2 row of mode m
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float w = (float)gw[i];
        fv[i] = w; fv[N + i] = w * Bp[gb + i]; fv[2 * N + i] = w * Br[gb + i]; fv[3 * N + i] = w * Bt[gb + i];
    }
    __syncthreads();
    const float *U = ops + tk.mol_off;
    float *UVt = opt + 2 * tk.uv_off;          // pre-split tensor-core tiles, padding rows included
    for (int e = threadIdx.x; e < G.NP * G.CIN; e += blockDim.x) {
        const int c = e / G.CIN, ci = e - c * G.CIN, b = ci / N, i = ci - b * N;
        float v = 0.f;
        if (c < G.COUT) {
            const float *u = U + (size_t)c * 24 + 4 * b;
            v = u[0] * fv[i] + u[1] * fv[N + i] + u[2] * fv[2 * N + i] + u[3] * fv[3 * N + i];
        }
        tile_put(UVt, G, c, ci, v);
    }
}

// Molecular input factors of the tensor-core pass, one block per mode m <= 2:
// V_m[4b + f][bN + i] = w_i f(mu_i), f in {1, P2m, R2m, T2m} at the Gauss
// nodes (the xi = V F factor of k_mol_lowrank); rows 24..31 and the entries
// outside block b are zero.  V[(m * 32 + q) * CIN + cin].
__global__ void k_mol_vtab(Geom G, int L, const float *Bp, const float *Br, const float *Bt, const double *gw,
                           float *V)
{
    const int m = blockIdx.x, N = G.N;
    const size_t gb = (size_t)m * (L + 1) * N + (size_t)2 * N;        // degree-2 row of mode m
    float *Vm = V + (size_t)m * 32 * G.CIN;
    for (int e = threadIdx.x; e < 32 * G.CIN; e += blockDim.x) {
        const int q = e / G.CIN, cin = e - q * G.CIN, b = cin / N, i = cin - b * N;
        float v = 0.f;
        if (q < 24 && (q >> 2) == b) {
            const float w = (float)gw[i];
            const int f = q & 3;
            v = f == 0 ? w : w * (f == 1 ? Bp[gb + i] : (f == 2 ? Br[gb + i] : Bt[gb + i]));
        }
        Vm[e] = v;
    }
}

// Flags -> task-ordered lists.  Queueing by completion order scatters the
// modes of one pixel over the next order's list; in task order the CTAs
// that run at the same time work on neighbouring tasks (the modes of a few
// pixels), which share the pixel's transport weights in L2, and the level
// tiles of one task's source contraction share its operator tiles.
__global__ void __launch_bounds__(COMPACT_THREADS) k_compact(BatchBufs B, int t0, int nw, int itn)
{
    __shared__ int sa[COMPACT_THREADS / 32], sm[COMPACT_THREADS / 32], sl[COMPACT_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // thread tid owns tasks [b, e)
    const int per = (nw + COMPACT_THREADS - 1) / COMPACT_THREADS;
    const int b = min(nw, tid * per), e = min(nw, b + per);
    int na = 0, nm = 0, lev = 0;
    for (int i = b; i < e; ++i) {
        const unsigned char f = B.aflag[i];
        if (f) {
            ++na;
            nm += f >> 1;
            lev += B.px[B.tasks[t0 + i].pix].nt + 1;
        }
    }
    // inclusive prefix sums over the warp, then over the warp totals
    int xa = na, xm = nm;
    for (int o = 1; o < 32; o <<= 1) {
        const int ya = __shfl_up_sync(0xffffffffu, xa, o), ym = __shfl_up_sync(0xffffffffu, xm, o);
        if (lane >= o) { xa += ya; xm += ym; }
    }
    int ls = lev;
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if (lane == 31) { sa[w] = xa; sm[w] = xm; }
    if (lane == 0) sl[w] = ls;
    __syncthreads();
    if (w == 0) {
        int ta = sa[lane], tm = sm[lane], tlv = sl[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int ya = __shfl_up_sync(0xffffffffu, ta, o), ym = __shfl_up_sync(0xffffffffu, tm, o);
            if (lane >= o) { ta += ya; tm += ym; }
        }
        for (int o = 16; o > 0; o >>= 1) tlv += __shfl_xor_sync(0xffffffffu, tlv, o);
        sa[lane] = ta; sm[lane] = tm;
        if (lane == 31) {
            B.active_cnt[itn - 1] = ta;
            B.mol_cnt[itn - 1] = tm;
        }
        if (lane == 0) B.work[itn * 4 + 3] = tlv;
    }
    __syncthreads();
    int oa = (w ? sa[w - 1] : 0) + xa - na, om = (w ? sm[w - 1] : 0) + xm - nm;
    int *al = B.alist[itn & 1], *ml = B.mlist[itn & 1];
    for (int i = b; i < e; ++i) {
        const unsigned char f = B.aflag[i];
        if (f) {
            al[oa++] = i;
            if (f >> 1) ml[om++] = i;
            B.aflag[i] = 0;
        }
    }
}
