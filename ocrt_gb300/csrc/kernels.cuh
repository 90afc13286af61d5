// kernels.cuh — kernel declarations shared by the host orchestration.
#pragma once
#include <cuda.h>
#include "common.cuh"
#include "gas.cuh"
#include "../../include/ocrt_gb300.h"

// setup.cu
__global__ void k_gauss(int N, double *mu, double *w, float *pw);
__global__ void k_pixel_setup(PixDev *px, int P, int N, const double *gmu);
__global__ void k_levels(const PixDev *px, int P, double *h, double *ch, double *xd, double *yd, double *z);
__global__ void k_levels_water(const PixDev *px, int P, double *h, double *ch, double *xd, double *yd, double *z);
__global__ void k_level_mix(const PixDev *px, int P, const double *z, double *xd, double *yd);
__global__ void k_coef(const PixDev *px, int P, int N, int NR, const double *gmu, const double *h,
                       float *Tc, float *Ca, float *Cb);
__global__ void k_coef_quads(const PixDev *px, int P, int N, int NR, const float *Tc, const float *Ca, const float *Cb,
                             float *Cq);
// gcoef (k_gsf_coefs, (M + 1) (L + 1) 5 doubles) or nullptr: the recurrences'
// step coefficients, tabulated once per group instead of per direction
__global__ void k_gsf_coefs(int M, int L, double *gcoef);
__global__ void k_basis_gauss(int N, int M, int L, const double *gmu, float *Bp, float *Br, float *Bt,
                              const double *gcoef);
__global__ void k_basis_pix(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, int L, int E, float *Bx,
                            const double *gcoef);
// k_scan: levels in flight per column (cp.async ring depth, a power of two)
// and its dynamic shared memory: J, the total's FP32 head and 3 coefficients per slot.
#define SCAN_DEPTH 8
inline size_t scan_smem_bytes(int threads) { return (size_t)SCAN_DEPTH * threads * (4 + 4 + 12); }
// k_scan4: four Gauss columns of one (Stokes, hemisphere) per thread, moved
// as 16-byte copies; the zero-weight columns one per thread.  It applies when
// N is a multiple of 4.
#define SCAN4_DEPTH 8
__host__ __device__ inline int scan4_threads(const Geom &G) { return ((6 * G.N / 4 + 6 * G.E + 31) / 32) * 32; }
inline size_t scan4_smem_bytes(int threads) { return (size_t)SCAN4_DEPTH * 5 * threads * 16; }
// Transport weights in quads (k_coef_quads): per layer, per quad of ring
// slots g = 4q..4q+3 (the ring padded to NRq = NR rounded up to 4, padding
// zero), four T, then four Ca, then four Cb: 3 * NRq floats per layer.
__host__ __device__ inline int coef_quad_width(int NR) { return 3 * ((NR + 3) & ~3); }
__host__ __device__ inline long long coef_quad_off(long long coef_off, int N, int NR)
{
    (void)N;
    return coef_off / NR * coef_quad_width(NR);
}
// k_scan_tma (scan_tma.cu): zero-weight columns fetched per level (6E rounded
// up to 4), weight-row width, block size (one thread per field column plus
// one producer warp), and the tensor maps it reads through.
__host__ __device__ inline int scan_tma_zw(const Geom &G) { return (6 * G.E + 3) & ~3; }
__host__ __device__ inline int scan_tma_cw(const Geom &G) { return coef_quad_width(G.NR); }
__host__ __device__ inline int scan_tma_threads(const Geom &G) { return ((G.COUT + 31) / 32) * 32 + 32; }
struct ScanMaps {
    CUtensorMap jg, tg;    // Gauss columns of J / the total head: {N, 2 (h), 3 (s), rows}
    CUtensorMap jz, tz;    // zero-weight columns: {LDC, rows}
    CUtensorMap cq;        // transport weights in quads: {3 * NRq, layers}
};
// k_adj_scan: cotangent rows per block (they share the transport coefficients)
#define ADJ_RB 3
inline size_t adj_scan_smem_bytes(int threads) { return (size_t)SCAN_DEPTH * threads * (ADJ_RB * (4 + 4) + 12); }
// k_tables launch shape: grid (tasks, tables_yblocks), two (outgoing, incoming)
// pairs per thread, (o, i) and (o, i + ceil(N/2)); moments are staged TB_LC at a
// time (even).
#define TB_LC 16
__host__ __device__ inline int tables_orows(int threads, int N) { return threads / ((N + 1) / 2) + 2; }
inline int tables_yblocks(int threads, int NR, int N) { return (NR * ((N + 1) / 2) + threads - 1) / threads; }
inline size_t tables_smem_bytes(int threads, int N, int L)
{
    return sizeof(float) * (4 * ((size_t)L + 1) + 8 * (size_t)tables_orows(threads, N) * TB_LC + 3 * (size_t)TB_LC * N);
}
__global__ void k_tables(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, Geom G, int L,
                         const float *Bp, const float *Br, const float *Bt, const float *Bx,
                         const double *gw,
                         const double *mb, const double *mg, const double *ma, const double *mz,
                         float *ops, float *pvec, float *fvec, float *opt, int plain,
                         const float *V, int vp0, long long vstride, const float *sprod);
// tables_tc.cu: phase tables and the aerosol operator tiles with the sums over
// l on tcgen05 (the pair part of k_tables; k_tables then runs with sprod for
// the molecular operator and the solar row).  GT: the Gauss bases in the chunk
// order, AT: the Gauss rows of the A tiles split and swizzled (k_basis_perm,
// grid (blocks, M + 1)); sprod[task][N][16]: the S and D sums of the eight
// sun-outgoing products of every Gauss slot.
__global__ void k_basis_perm(int N, int M, int L, const float *Bp, const float *Br, const float *Bt, float *GT,
                             float *AT);
__global__ void k_tables_tc(const TaskDev *tasks, int t0, int nt_tasks, const PixDev *px, Geom G, int L,
                            const float *GT, const float *AT, const float *Bx, const double *gw, const double *mb,
                            const double *mg, const double *ma, const double *mz, float *ops, float *opt, int plain,
                            const float *V, int vp0, long long vstride, float *sprod, int *err);
size_t tables_tc_smem_bytes(const Geom &G, int L);
size_t tables_tc_gt_floats(int N, int M, int L);
size_t tables_tc_at_floats(int M, int L);
bool tables_tc_supported(const Geom &G, int L);
int tables_tc_threads();
cudaError_t tables_tc_init();
// value.cu: the aerosol value kernel's I-I tables V[pixel - p0][m][row][column]
// (rows: sun, Gauss nodes; columns: ring slots at +mu, then at -mu)
__global__ void k_value_pfm(const PixDev *px, int p0, Geom G, const double *gmu, const double *vk_th,
                            const double *vk_p11, float *V, long long vstride);
size_t value_kernel_smem_bytes(int n_ang);
// coxmunk_tc.cu: Cox-Munk Fourier kernels with the azimuth projection on tcgen05.
// pairs: (outgoing slot, incoming slot) list of the ring (Gauss pairs with
// outgoing > incoming left out: the reciprocal pair writes them).
__global__ void k_coxmunk_tc(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                             const double *gmu, const float *cs_tab, const float *cs_tiles, int Mtab,
                             const double *lamv, const double *lamd, float *srf, float *srfW, const short2 *pairs,
                             int npairs, int dw, int *err);
__global__ void k_cs_tiles(int Mtab, int nphi, const float *cs_tab, float *tiles);
size_t coxmunk_tc_smem_bytes(int Mtab, bool dw);
size_t coxmunk_tc_tiles_floats(int Mtab, int nphi);
bool coxmunk_tc_supported(int Mtab, int nphi, bool dw);
int coxmunk_tc_pairs_per_cta();
int coxmunk_tc_threads(bool dw);
__global__ void k_coxmunk(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                          const double *gmu, const float *cs_tab, int Mtab, const double *lamv, float *srf);
__global__ void k_coxmunk_dw(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                             const double *gmu, const float *cs_tab, int Mtab, const double *lamv,
                             const double *lamd, float *srf, float *srfW);
__global__ void k_sancer(const PixDev *px, int P, int N, const double *gmu, double *lam, double *lamd);
__global__ void k_layers_apply(PixDev *px, int P, const double *ldt, const double *lss, double *h, double *ch,
                               double *xd, double *yd, int *err);
__global__ void k_coef_deriv(const PixDev *px, int P, int N, const double *gmu, const double *h,
                             float *dTc, float *dCa, float *dCb);
__global__ void k_cs_table(int M, int nphi, float *cs);
__global__ void k_flat_fresnel(const PixDev *px, int P, int N, const double *gmu, float *frs);
__global__ void k_seed_att(const PixDev *px, int P, int N, const double *gmu, const double *h, float *E);
__global__ void k_level_float(const PixDev *px, int P, const double *xd, const double *yd, const double *ch, float *lvf);

// sos.cu
#define ST_M_TILE 64
#define ST_N_TILE 64
struct WaveBufs {
    float *F;              // field of the current order (FP32), wave-relative by TaskDev::fld_off
    float *J;              // source of the current order
    float *Tot;            // order totals, FP32 head at every level (convergence norm, adjoint)
    float *Ttl;            // tails of the totals at the output levels: two rows per task at
                           // TaskDev::tail_off, row 0 for k = 0 and row 1 for k = nt, so
                           // (Tot, Ttl) is a double-float there
    float *ops;            // operators, wave-relative (FP32)
    float *opt;            // tensor-core path: the aerosol and dense molecular operators pre-split into
                           // tf32 (hi, lo) SWIZZLE_128B tiles at 2 x op_off / 2 x uv_off (tile_put)
    float *pvec, *fvec;    // per wave-task primary and flat-beam vectors
    float *srf;            // rough surface kernels, wave-relative
};
// The outputs read the totals only at the TOA (k = 0) and the BOA (k = nt);
// there they are double-floats (head in Tot, tail in Ttl).  Interior levels
// feed only the FP32 convergence norm and the adjoint, so they keep the FP32
// head alone, which saves the scan 8 B per element and order.
__device__ inline size_t tot_tail_off(const TaskDev &tk, const Geom &G, int k, int c)
{
    return (size_t)tk.tail_off + (k == 0 ? 0 : (size_t)G.LDC) + c;
}
__device__ inline double tot_value(const WaveBufs &W, const TaskDev &tk, const Geom &G, int k, int nt, int c)
{
    const float hi = W.Tot[(size_t)tk.fld_off + (size_t)k * G.LDC + c];
    const float lo = (k == 0 || k == nt) ? W.Ttl[tot_tail_off(tk, G, k, c)] : 0.f;
    return (double)hi + (double)lo;
}
struct BatchBufs {
    const PixDev *px;
    const TaskDev *tasks;
    TaskState *state;
    TaskOut *tout;
    const double *gmu, *gw;
    const float *pw;       // [2N]: (float)(2 pi mu_i w_i) for m = 0, then (float)(pi mu_i w_i)
    const double *h, *ch, *xd, *yd, *z;
    const float *Tc, *Ca, *Cb;
    const float *Cq;       // Gauss-slot transport weights in quads for k_scan4 (k_coef_quads), or nullptr
    const float *frs;
    const float *Eatt;     // rough direct-beam attenuation [lev_off*NR + k*NR + g]
    const float *lvf;      // [lev_off + k][3]: x_k, y_k, direct beam ch_k rounded to FP32
    int *active_cnt;       // [max_orders + 2]: tasks still active after order it
    int *mol_cnt;          // [max_orders + 2]: molecular (m <= 2) tasks still active after order it
    const double *ext;     // per-pixel boundary sources at PixDev::ext_off (coupled ocean), or nullptr
    int *alist[2];         // ping-pong active-task lists (wave-local ids); order it reads alist[it & 1]
    int *mlist[2];         // same for the molecular tasks
    int *work;             // [max_orders + 2][4] work counters of the persistent kernels
    int *err;              // device error word
    const float *molV;     // [3][32][CIN]: V_m[4b + f][bN + i] = w_i {1, P2m, R2m, T2m}(mu_i), rows 24..31 zero
                           // (the adjoint's tensor-core pass contracts the transposed molecular term with it)
    unsigned char *aflag = nullptr;  // per wave task: 1 = active in the next order, 3 = active and molecular; k_compact
                           // turns the flags into task-ordered lists.  nullptr: tasks are appended to the lists
                           // directly (in completion order).
};

// Queue wave task tl for order itn (after the order that just ran, or after
// the primary for itn = 2): a flag for k_compact, or a direct append.  The
// work counter [itn][3] sums the level rows queued (the scan autotuner's work
// measure).
__device__ inline void queue_next(const BatchBufs &B, int itn, int tl, int has_mol, int levels)
{
    if (B.aflag) {
        B.aflag[tl] = has_mol ? 3 : 1;
        return;
    }
    B.alist[itn & 1][atomicAdd(&B.active_cnt[itn - 1], 1)] = tl;
    if (has_mol) B.mlist[itn & 1][atomicAdd(&B.mol_cnt[itn - 1], 1)] = tl;
    atomicAdd(&B.work[itn * 4 + 3], levels);
}
// k_compact: the flagged tasks of a wave (nw of them) in task order into the
// lists of order itn, their counts and level rows; clears the flags.  One block.
#define COMPACT_THREADS 1024
__global__ void k_compact(BatchBufs B, int t0, int nw, int itn);

// adjoint.cu
struct AdjBufs {
    int ncot;              // cotangent rows per pixel; adjoint task = wave task * ncot + row
    float *AF;             // adjoint field a_j (wave-relative, x ncot)
    float *AJ;             // transposed-transport output muJ (FP32, like AF)
    const float *opsT;     // per wave task [CIN + 32][KP] (FP32, KP = COUT rounded up to 32): the transposed
                           // aerosol operator, then for m <= 2 the transposed molecular factor U^T (24 rows, 8 zero)
    float *ATot;           // adjoint total (FP32: it only feeds the gradients)
    float *bc;             // mu_bc per adjoint task [NR][3]
    TaskState *st;         // per adjoint task
    int *acnt;             // [max_orders + 2] adjoint tasks still active after order j
    int *awork;            // [max_orders + 2] work counters of the persistent transposed source
    // active-task lists: alist[j & 1] holds the lcnt[j] wave tasks with a row
    // active at the start of order j (in task order, k_compact_adj from aflag,
    // which the adjoint scan of order j - 1 sets); the transposed source and
    // surface of order j read list j + 1 (rows still active after the scan)
    unsigned char *aflag;
    int *alist[2];
    int *lcnt;             // [max_orders + 2]
    int *swork;            // [max_orders + 2] work counters of the persistent adjoint scan
    const double *cot;     // [P][ncot][3]
    double *gout;          // per adjoint task partials, gstride doubles (3 arrays of kstride + 2 scalars)
    int gstride, kstride;
    const float *dTc, *dCa, *dCb;   // transport-coefficient derivatives (like Tc/Ca/Cb)
    const float *srfW;     // dR_m/dW, laid out like WaveBufs::srf
    double *grad;          // [P][ncot][grad_stride]: d_dtau[nt], d_ssa[nt], d_wind
    int grad_stride;
};
__global__ void k_adj_prep(BatchBufs B, WaveBufs W, Geom G, int t0);
__global__ void k_fill_all(BatchBufs B, int t0, int nw, int it);
__global__ void k_adj_init(BatchBufs B, AdjBufs A, Geom G, int t0, int nadj);
__global__ void k_adj_scan(BatchBufs B, AdjBufs A, Geom G, int t0, int j);
__global__ void k_adj_source(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0);
__global__ void k_adj_mol(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0,
                          const float *Bp, const float *Br, const float *Bt, int L);
__global__ void k_adj_surface(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0, int j);
__global__ void k_adj_list_all(AdjBufs A, int nw);
__global__ void k_compact_adj(AdjBufs A, int nw, int j);
__global__ void k_adj_grad(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int t0, int rb, int xs_in_f);
__global__ void k_adj_pixel(BatchBufs B, WaveBufs W, AdjBufs A, Geom G, int p0, int t0);
size_t adj_mol_smem_bytes(const Geom &G);

__global__ void k_primary(BatchBufs B, WaveBufs W, Geom G, int t0);
__global__ void k_primary4(BatchBufs B, WaveBufs W, Geom G, int t0);   // N % 4 == 0, no flat surface, quad weights
// The order-1 source and transport step with the rounding sequence fixed
// (no contraction left to the compiler), so k_primary and k_primary4 give the
// same bits: J = ch (x fa + y fm), I' = T I + Ca J + Cb J'.
__device__ __forceinline__ float prim_source(float lc, float lx, float ly, float fa, float fm)
{
    return __fmul_rn(lc, __fmaf_rn(lx, fa, __fmul_rn(ly, fm)));
}
__device__ __forceinline__ float prim_step(float T, float I, float A, float J, float Bw, float Jp)
{
    return __fmaf_rn(T, I, __fmaf_rn(A, J, __fmul_rn(Bw, Jp)));
}

// lut.cu (angle-grid LUT mode)
struct LutBufs {
    const double *vza, *raa;   // grid angles in degrees, by PixDev::lut_vo / lut_ro
    double *samp;              // [task][nvmax][4]: TOA-up I, Q, U (PCHIP) and BOA-down I (linear) per grid vza
    int nvmax;
    const double *kappa;       // [lut_oo + point] IPSS kappa per grid direction
    const double *tau_dir;     // [pixel] IPSS direct slant depth (or -1)
    double *out;               // 6 planes of ntot: rho_I, rho_Q, rho_U, T_diff_dn_dir, T_sg_up_dir, T_total_up_dir
    long long ntot;
};
__global__ void k_lut_sample(BatchBufs B, WaveBufs W, LutBufs Lb, Geom G, int t0, int nw);
__global__ void k_lut_final(const PixDev *px, int P, LutBufs Lb, const int *pix_task0);
__global__ void k_ipss_lut(const PixDev *px, int P, const double *h, const double *z, const double *xd,
                           const double *yd, const double *tabs, const double *mb, const double *vk_th,
                           const double *vk_p11, const double *lut_vza, const double *lut_raa, double *lut_kappa);
__global__ void k_source_simt(BatchBufs B, WaveBufs W, Geom G, int t0, int it);

// tc_gemm.cu (tcgen05 source contraction for modes without a molecular term)
__global__ void k_source_tc(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int mtiles);
__global__ void k_source_tc_xs(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int mtiles);
__global__ void k_adj_source_tc(BatchBufs B, WaveBufs W, AdjBufs AB, Geom G, int t0, int it, int mtiles, int nw);
__global__ void k_op_transpose(const TaskDev *tasks, int t0, int nw, Geom G, const float *ops, float *opsT);
__global__ void k_mol_utrans(const TaskDev *tasks, int t0, int nw, Geom G, const float *ops, float *opsT);
__global__ void k_mol_dense(const TaskDev *tasks, int t0, int nw, Geom G, int L, const float *Bp, const float *Br,
                            const float *Bt, const double *gw, const float *ops, float *opt);
__global__ void k_mol_vtab(Geom G, int L, const float *Bp, const float *Br, const float *Bt, const double *gw,
                           float *V);
size_t coxmunk_smem_bytes(int nphi, bool dw);
size_t tc_smem_bytes(const Geom &G);
int tc_fwd_threads();          // block size of k_source_tc
bool tc_supported(const Geom &G);
size_t tc_adj_smem_bytes(const Geom &G);
bool tc_adj_supported(const Geom &G);
__global__ void k_scan(BatchBufs B, WaveBufs W, Geom G, int t0, int it);
__global__ void k_scan4(BatchBufs B, WaveBufs W, Geom G, int t0, int it);
// k_scan_tma<CH, NS> (levels per chunk, ring stages) instances: (8, 3), (8, 4), (4, 6), (16, 2)
const void *scan_tma_fn(int ch, int ns);
cudaError_t scan_tma_launch(int ch, int ns, int grid, cudaStream_t st, const BatchBufs &B, const WaveBufs &W,
                            const Geom &G, int t0, int it, const ScanMaps &M);
cudaError_t scan_tma_init();   // dynamic shared-memory limits of the instances
size_t scan_tma_smem_bytes(const Geom &G, int CH, int NS);
// tensor maps over the wave's J and total buffers (fld_floats floats) and the
// quad weight table (layers rows); 0 on success
int scan_tma_maps(const Geom &G, int CH, float *J, float *Tot, size_t fld_floats, const float *Cq, size_t layers,
                  ScanMaps *M);
bool scan_tma_supported(const Geom &G);
// the adjoint's transposed scan fed the same way (scan_tma.cu): maps over the
// adjoint field and total buffers and the weight rows in boxes of 5 levels
struct AdjScanMaps {
    CUtensorMap ag, tg;    // Gauss columns of the adjoint field / adjoint total
    CUtensorMap az, tz;    // zero-weight columns
    CUtensorMap cq;        // transport weights, 5 layers per box
};
struct AdjBufs;
int adj_scan_tma_maps(const Geom &G, float *AF, float *ATot, size_t adj_floats, const float *Cq, size_t layers,
                      AdjScanMaps *M);
size_t adj_scan_tma_smem_bytes(const Geom &G, int CH, int NS);
cudaError_t adj_scan_tma_launch(int grid, cudaStream_t st, const BatchBufs &B, const AdjBufs &A, const Geom &G,
                                int t0, int j, const AdjScanMaps &M);
__global__ void k_mol_lowrank(BatchBufs B, WaveBufs W, Geom G, int t0, int it, int ltiles,
                              const float *Bp, const float *Br, const float *Bt, int L);
inline size_t mol_smem_bytes(const Geom &G) { return sizeof(float) * (4 * G.N + G.COUT * 24 + 32 * G.CIN + 32 * 25); }
__global__ void k_extract(BatchBufs B, WaveBufs W, Geom G, int t0, int nt_tasks);
__global__ void k_stop_check(const int *active_after_last, int *flag);

// post.cu
__global__ void k_ipss(const PixDev *px, int P, const double *h, const double *z,
                       const double *xd, const double *yd, const double *tabs,
                       const double *mb, const double *vk_th, const double *vk_p11, double *kappa, double *tau_dir);
__global__ void k_finalize(const PixDev *px, int P, const TaskState *state, const TaskOut *tout,
                           const double *gmu, const double *gw, const double *h,
                           const double *kappa, const double *tau_dir, ocrt_result *res);

// ocean.cu — coupled atmosphere-ocean solve
#define OCRT_EDGE 12      // doubles per (task, ring slot) of k_edges
// One coupled pixel: its place in the three passes and the scalars of the
// interface coupling.
struct OceanPix {
    // ---- host ----
    double mu_sa, mu_va, mu_sw, mu_vw, raa_deg, nw, wind, tau_atm, ext_w;
    int st, qc, M, m_loop;        // atmosphere modes; water modes solved (min(m_max_water, L))
    int pa, pw;                   // pixel index in the atmosphere groups / the water group
    int n_ring_unique;            // distinct water directions (Gauss + zero-weight)
    long long top_off;            // skylight top source [M+1][N][3] in the water group's ext buffer
    long long ext_off;            // water-leaving bottom source [M+1][NRa][3] in the pass-3 ext buffer
    // ---- device ----
    double T_dir, F_boa, F_w, Ed_sky_w, Ed_sky_a;
    int m_view, m_nodes;          // last water mode with a view sample / with node values
};
__global__ void k_edges(BatchBufs B, WaveBufs W, Geom G, int t0, int nw, double *edge);
__global__ void k_rww(const TaskDev *tasks, const PixDev *px, int p0, const int *pix_task0, Geom G,
                      const double *gmu, int nphi, float *srf);
__global__ void k_taw_direct(const OceanPix *op, int P, const PixDev *pxa, const double *gmu, int N, int NRa, double *td);
__global__ void k_ocean_prep(OceanPix *op, int P, const int *task0_a, const double *gmu, const double *gw, int N,
                             int NRa, const double *edge_a, const double *td);
__global__ void k_couple_aw(const OceanPix *op, int P, const int *task0_a, const double *gmu, const double *gw,
                            int N, int NRa, const double *edge_a, double *top);
__global__ void k_dtop_field(BatchBufs B, WaveBufs W, Geom G, int t0);
__global__ void k_water_modes(OceanPix *op, int P, const PixDev *pxw, const int *task0_w, int NRw, const double *edge_w);
__global__ void k_couple_wa(const OceanPix *op, int P, const PixDev *pxa, const PixDev *pxw, const int *task0_w,
                            const double *gmu, int N, int NRa, int NRw, const double *edge_w, const double *glo,
                            double *ext3, double *view);
__global__ void k_ocean_final(const OceanPix *op, int P, const PixDev *pxa, const PixDev *pxw, const int *task0_w,
                              const double *gmu, const double *gw, int N, int NRw, const double *edge_w,
                              const double *view, const double *top, const ocrt_result *r1, const ocrt_result *rw,
                              const ocrt_result *r3, ocrt_result *out, ocrt_ocean_result *wout);
// shared-memory bytes of the interface-projection kernels for M modes
inline size_t iface_smem_bytes(int M, int nphi, int extra_doubles)
{
    return sizeof(float) * ((size_t)(M + 1) * nphi * 2 + (size_t)nphi * 9 + (((size_t)(M + 1) * 9 + 1) & ~(size_t)1)) +
           sizeof(double) * (size_t)extra_doubles;
}
