// api.cu — host side of the C ABI (include/ocrt_gb300.h).
//
// A plan uploads a batch, groups pixels by Gauss order N, and splits each
// group into waves of whole pixels whose per-(pixel, mode) working set fits
// the workspace budget.  Execution is asynchronous on one stream; the order
// loop polls the device-side active-task count every few orders, which is the
// only host synchronisation inside a solve.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include <algorithm>
#include <climits>
#include <functional>
#include <utility>

#include "kernels.cuh"
#include "physics.cuh"

namespace {

std::mutex g_mu;
thread_local std::string g_err;
int g_device = -1;
int g_nsm = 152;           // SM count of the device, read at init
cudaStream_t g_stream = nullptr;
std::multimap<size_t, void *> g_free;      // caching allocator: size -> block
std::map<void *, size_t> g_live;
int *g_pinned = nullptr;
int g_timing = 0;

// ---- launch-shape autotuner ----
// Kernels whose outputs are plain stores of values computed from their inputs
// (k_coxmunk, k_tables) can be launched again without changing the result, so
// on the first execute that meets a new shape key each candidate block size is
// run twice on the launching stream and the second run timed with CUDA events;
// the fastest size is kept for the rest of the process.  OCRT_GB_AUTOTUNE=0
// keeps the default of 256 threads.
struct TuneRec {
    std::string kernel;
    std::vector<int> key;
    int best = 256;
    std::vector<std::pair<int, float>> ms;
    const char *const *labels = nullptr;   // names of the choices (printed instead of their numbers)
};
std::map<std::pair<std::string, std::vector<int>>, size_t> g_tune_idx;
std::vector<TuneRec> g_tune;
const int kTuneBlocks[3] = {128, 256, 512};

bool autotune_enabled()
{
    const char *e = getenv("OCRT_GB_AUTOTUNE");
    return !(e && strcmp(e, "0") == 0);
}

enum KClass { KC_SETUP, KC_TABLES, KC_COXMUNK, KC_PRIMARY, KC_SOURCE, KC_SOURCE_TC, KC_MOL, KC_SCAN, KC_EXTRACT,
              KC_IPSS, KC_FINAL, KC_ADJ_SCAN, KC_ADJ_SOURCE, KC_ADJ_OTHER, KC_ADJ_TOTALS, KC_ADJ_GRAD, KC_N };
const char *kc_names[KC_N] = {"setup", "phase_tables", "coxmunk_fourier", "primary", "source_gemm_simt",
                              "source_gemm_tcgen05", "source_molecular", "transport_scan", "extract", "ipss",
                              "finalize", "adjoint_scan", "adjoint_source", "adjoint_other", "adjoint_forward_totals",
                              "adjoint_gradients"};

int fail(int rc, const std::string &msg)
{
    g_err = msg;
    return rc;
}

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(OCRT_ERR_DEVICE, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void *dalloc(size_t bytes)
{
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~size_t(255);
    auto it = g_free.lower_bound(bytes);
    if (it != g_free.end() && it->first <= bytes * 2) {
        void *p = it->second;
        const size_t sz = it->first;
        g_free.erase(it);
        g_live[p] = sz;
        return p;
    }
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        for (auto &kv : g_free) cudaFree(kv.second);
        g_free.clear();
        if (cudaMalloc(&p, bytes) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    }
    g_live[p] = bytes;
    return p;
}

void dfree(void *p)
{
    if (!p) return;
    auto it = g_live.find(p);
    if (it == g_live.end()) return;
    g_free.insert({it->second, p});
    g_live.erase(it);
}

int ensure_init()
{
    if (g_device >= 0) return OCRT_OK;
    return ocrt_gb_init(0);
}

int validate(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer)
{
    // rt_solver.c:627-638 plus the documented limits of this library
    if (!cs || !op) return fail(OCRT_ERR_ARGS, "null case or options");
    if (!(cs->wavelength_nm >= 330.0 - 1e-9 && cs->wavelength_nm <= 1100.0 + 1e-9))
        return fail(OCRT_ERR_ARGS, "wavelength outside [330, 1100] nm");
    if (!(cs->sza_deg >= 0.0 && cs->sza_deg < 90.0)) return fail(OCRT_ERR_ARGS, "sza outside [0, 90)");
    if (!(cs->vza_deg >= 0.0 && cs->vza_deg < 90.0)) return fail(OCRT_ERR_ARGS, "vza outside [0, 90)");
    if (!std::isfinite(cs->raa_deg)) return fail(OCRT_ERR_ARGS, "raa not finite");
    if (op->fourier_m_max < 0 || op->fourier_m_max > OCRT_MAX_M) return fail(OCRT_ERR_ARGS, "fourier_m_max outside [0, 255]");
    if (op->n_mu < 2 || op->n_mu > OCRT_MAX_N) return fail(OCRT_ERR_ARGS, "n_mu outside [2, 64]");
    if (op->n_layers < 2 || op->n_layers > 1024) return fail(OCRT_ERR_ARGS, "n_layers outside [2, 1024]");
    if (op->max_orders < 1 || !(op->tolerance > 0.0)) return fail(OCRT_ERR_ARGS, "bad SOS iteration control");
    const int nphi = op->n_phi_surface > 0 ? op->n_phi_surface : 1024;
    if (nphi < 64 || nphi > 4096 || (nphi & 1)) return fail(OCRT_ERR_ARGS, "n_phi_surface outside [64, 4096] or odd");
    if (cs->surface == OCRT_SURFACE_LAMBERT || cs->surface == OCRT_SURFACE_OCEAN)
        return fail(OCRT_ERR_UNSUPPORTED, "surface kind not on the GB300 solve path");
    if (cs->surface != OCRT_SURFACE_BLACK && cs->surface != OCRT_SURFACE_BLACK_FRESNEL_OCEAN &&
        cs->surface != OCRT_SURFACE_FLAT) return fail(OCRT_ERR_ARGS, "unknown surface kind");
    if ((cs->surface != OCRT_SURFACE_BLACK) && !(cs->n_water > 0.0)) return fail(OCRT_ERR_ARGS, "n_water <= 0");
    const bool has_aer = aer && aer->tau_a > 0.0;
    if (aer) {
        if (aer->tau_a < 0.0 || aer->ssa_a < 0.0 || aer->ssa_a > 1.0 || aer->L_max < 2 || aer->L_max > 1024)
            return fail(OCRT_ERR_ARGS, "bad aerosol expansion");
        if (!aer->beta || !aer->gamma || !aer->alpha || !aer->zeta) return fail(OCRT_ERR_ARGS, "null moment array");
        for (int l = 0; l <= aer->L_max; ++l)
            if (!std::isfinite(aer->beta[l]) || !std::isfinite(aer->gamma[l]) || !std::isfinite(aer->alpha[l]) ||
                !std::isfinite(aer->zeta[l])) return fail(OCRT_ERR_NONFINITE, "non-finite aerosol moment");
        if (aer->use_value_kernel && aer->tau_a > 0.0) {
            const int n = aer->n_ang_phase;
            if (n < 2 || n > 8192 || !aer->theta_phase || !aer->P11_phase)
                return fail(OCRT_ERR_ARGS, "value kernel: phase table of 2 .. 8192 angles required");
            for (int i = 0; i < n; ++i) {
                if (!std::isfinite(aer->theta_phase[i]) || !std::isfinite(aer->P11_phase[i]))
                    return fail(OCRT_ERR_NONFINITE, "value kernel: non-finite phase table");
                if (i && !(aer->theta_phase[i] > aer->theta_phase[i - 1]))
                    return fail(OCRT_ERR_ARGS, "value kernel: phase angles must ascend strictly");
            }
            if (cs->surface == OCRT_SURFACE_FLAT || (cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && !(cs->wind_speed > 0.0)))
                return fail(OCRT_ERR_UNSUPPORTED, "value kernel with a flat surface is not on the GB300 path");
        }
    }
    double tau_r;
    if (!(cs->pressure_hpa > 0.0)) tau_r = 0.0;
    else if (op->tau_r_source == OCRT_TAU_R_FROM_INPUT) {
        if (cs->tau_r_input <= 0.0) return fail(OCRT_ERR_ARGS, "tau_r_input <= 0 with FROM_INPUT");
        tau_r = cs->tau_r_input;
    } else tau_r = bodhaine_tau(cs->wavelength_nm, cs->pressure_hpa);
    if (has_aer) { if (!(tau_r + aer->tau_a > 0.0)) return fail(OCRT_ERR_ARGS, "zero column"); }
    else if (!(tau_r > 0.0)) return fail(OCRT_ERR_ARGS, "no scattering column (pressure <= 0 and no aerosol)");
    if (op->pssa && op->rayleigh_profile == OCRT_PROFILE_EXPONENTIAL && !(op->rayleigh_h_km > 0.0))
        return fail(OCRT_ERR_ARGS, "rayleigh_h_km <= 0");
    return OCRT_OK;
}

struct Wave {
    int p0, p1;            // pixel range within the group
    int t0, t1;            // task range
    int Kmax;
    size_t fld, ops, srf;  // element counts of the wave buffers
    bool any_rough, any_flat;
    size_t tail = 0;       // element count of the total-tail rows (2 * LDC per task)
    bool any_water = false, any_top = false;   // water-column pixels; with a skylight top source
    int n_simt = 0, n_tc = 0, n_mol = 0;   // tasks given to each source kernel
    // Last order run before every task was found converged (forward orders,
    // adjoint orders); INT_MAX when the loop ran to max_orders.  Recorded by
    // an eager execute, replayed without host polls by the captured graph.
    int fwd_stop = INT_MAX, adj_stop = INT_MAX;
};

bool force_simt_coxmunk()
{
    const char *e = getenv("OCRT_GB_COXMUNK");
    return e && strcmp(e, "simt") == 0;
}

// OCRT_GB_TABLES=simt keeps the phase tables on the CUDA cores (k_tables alone).
bool force_simt_tables()
{
    const char *e = getenv("OCRT_GB_TABLES");
    return e && strcmp(e, "simt") == 0;
}

bool force_simt()
{
    const char *e = getenv("OCRT_GB_SOURCE_KERNEL");
    return e && strcmp(e, "simt") == 0;
}

// OCRT_GB_SCAN=column keeps the one-column-per-thread scan where the
// four-column one applies (N a multiple of 4).
// Transport-scan implementations.  All run each column's recurrence with
// the same arithmetic in the same order, so any of them (and any mix across
// orders) gives identical results; they differ in how the per-level inputs
// reach the threads.
// The deeper rings (8x5, 4x10) fit three blocks per SM only where the order
// totals stay at the output levels (smaller stages).
enum ScanKind { SK_COLUMN, SK_QUAD, SK_TMA_8_3, SK_TMA_8_4, SK_TMA_4_6, SK_TMA_16_2, SK_TMA_8_5, SK_TMA_4_10, SK_N };
const char *sk_names[SK_N] = {"column", "quad", "tma8x3", "tma8x4", "tma4x6", "tma16x2", "tma8x5", "tma4x10"};
const int sk_ch[SK_N] = {0, 0, 8, 8, 4, 16, 8, 4};
const int sk_ns[SK_N] = {0, 0, 3, 4, 6, 2, 5, 10};
inline int sk_map_index(int ch) { return ch == 4 ? 0 : ch == 8 ? 1 : 2; }

// Resident blocks per SM of a chunked-scan variant at this geometry (0: does
// not fit); the persistent grid is that times the SM count.
int scan_tma_blocks(int kind, const Geom &G)
{
    static std::map<std::vector<int>, int> cache;
    const std::vector<int> key = {kind, G.N, G.E, G.tot_all};
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const void *fn = scan_tma_fn(sk_ch[kind], sk_ns[kind]);
    int nb = 0;
    const int th = scan_tma_threads(G);
    if (th > 256 ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, th, scan_tma_smem_bytes(G, sk_ch[kind], sk_ns[kind])) !=
            cudaSuccess) {
        cudaGetLastError();
        nb = 0;
    }
    cache[key] = nb;
    return nb;
}

// OCRT_GB_ADJ_SCAN=column keeps the adjoint's per-thread copy-ring scan.
bool adj_scan_column()
{
    const char *e = getenv("OCRT_GB_ADJ_SCAN");
    return e && strcmp(e, "column") == 0;
}

// OCRT_GB_PRIMARY=column keeps the one-column-per-thread order-1 kernel.
bool primary_column()
{
    const char *e = getenv("OCRT_GB_PRIMARY");
    return e && strcmp(e, "column") == 0;
}

bool scan4_allowed(int N)
{
    const char *e = getenv("OCRT_GB_SCAN");
    return N % 4 == 0 && !(e && strcmp(e, "column") == 0);
}


// OCRT_GB_SCAN names one implementation (column, quad, tma8x3, ...); unset,
// the scan autotuner picks one.  Returns -1 when unset or unknown.
int scan_forced()
{
    const char *e = getenv("OCRT_GB_SCAN");
    if (!e) return -1;
    if (strcmp(e, "tma") == 0) return SK_TMA_8_3;
    for (int k = 0; k < SK_N; ++k)
        if (strcmp(e, sk_names[k]) == 0) return k;
    return -1;
}

// Online scan autotuner.  The scan updates the order state, so a candidate
// cannot be re-run on the same input; instead, on eager executes of a shape
// key that has no choice yet, successive orders rotate through the
// candidates, each order's scan is timed with CUDA events, and the time is
// divided by the order's level-columns (the scan's work, counted on the
// device as tasks are queued).  Once every candidate has two orders the
// fastest per level-column is kept for the process.
struct ScanTune {
    std::vector<int> cand;
    double ms[SK_N] = {0}, lev[SK_N] = {0};
    int n[SK_N] = {0};
    int best = -1;
};
std::map<std::vector<int>, ScanTune> g_scan_tune;

struct Group {
    int N = 0, E = 1, P = 0, T = 0;   // E zero-weight ring slots (1 atmosphere, 4 water column)
    Geom G{};
    std::vector<int> idx;                 // case index of each pixel
    std::vector<PixDev> hpx;
    std::vector<TaskDev> htask;
    std::vector<int> hpix_task0;
    std::vector<Wave> waves;
    int Lmax = 2, Mmax = 0, max_orders = 1, nphi = 1024;
    bool any_pssa = false, any_rough = false, any_flat = false, any_gas = false, any_water = false;
    // coupled atmosphere-ocean: boundary sources read by the solve (owned by the
    // ocean plan), the edge export written after each wave's orders (k_edges)
    const double *ext = nullptr;
    double *edge = nullptr;
    int nphi_ww = 176;
    size_t nlev = 0, ncoef = 0, nmom = 0;
    size_t wave_fld = 0, wave_ops = 0, wave_srf = 0, wave_tail = 0;
    int wave_tasks = 0;
    // device
    PixDev *px = nullptr; TaskDev *tasks = nullptr; TaskState *state = nullptr; TaskOut *tout = nullptr;
    ocrt_result *res = nullptr; int *pix_task0 = nullptr;
    double *gmu = nullptr, *gw = nullptr;
    float *pw = nullptr;
    double *h = nullptr, *ch = nullptr, *xd = nullptr, *yd = nullptr, *z = nullptr;
    double *tabs = nullptr;   // per-layer gas absorption depths (level-array layout), any_gas only
    float *Tc = nullptr, *Ca = nullptr, *Cb = nullptr;
    float *Cq = nullptr;                  // transport weights in quads (k_scan4, k_scan_tma), nullptr when the column scan runs
    ScanMaps smap[3];                     // k_scan_tma tensor maps for level chunks of 4, 8, 16
    // aerosol value kernel: tables of every such pixel (ascending degrees, P11),
    // and the wave's I-I tables from k_value_pfm ([wave pixel][m][N + 1][2 NR])
    bool any_vk = false;
    int vk_nmax = 0;
    double *vk_th = nullptr, *vk_p11 = nullptr;
    float *vkV = nullptr;
    long long vk_stride = 0;
    int wave_pix = 0;
    bool smap_ok = false;
    AdjScanMaps amap;                     // k_adj_scan_tma tensor maps over the adjoint buffers
    bool amap_ok = false;
    float *Bp = nullptr, *Br = nullptr, *Bt = nullptr, *cs = nullptr, *frs = nullptr;
    double *lam = nullptr;
    float *Eatt = nullptr, *lvf = nullptr;
    double *mb = nullptr, *mg = nullptr, *ma = nullptr, *mz = nullptr;
    double *kappa = nullptr, *taudir = nullptr;
    int *active_cnt = nullptr, *mol_cnt = nullptr, *work = nullptr, *err = nullptr;
    int *alist[2] = {nullptr, nullptr}, *mlist[2] = {nullptr, nullptr};   // device-built active-task lists
    unsigned char *aflag = nullptr;       // per wave task: queued for the next order (k_compact sorts the lists)
    float *F = nullptr, *J = nullptr, *ops = nullptr;
    float *opt = nullptr;    // pre-split operator tiles of the tensor-core pass (2 x wave_ops floats)
    bool tabs_tc = false;    // phase tables on tcgen05 (k_tables_tc)
    bool keep_tot = false;   // keep the order totals at every level (set before build_group)
    float *gtab = nullptr;   // its Gauss bases in the chunk order (k_basis_perm)
    float *atab = nullptr;   // and the Gauss rows of its A tiles, split and swizzled
    double *gcoef = nullptr; // GSF recurrence step coefficients per (m, l) (k_gsf_coefs)
    float *sprod = nullptr;  // its sun-outgoing products per wave task [N][16]
    float *molV = nullptr;   // [3][32][CIN] molecular input factors V_m of the tensor-core pass
    short2 *cmpairs = nullptr;   // (outgoing, incoming) slot pairs of the tensor-core Cox-Munk kernel
    float *cstiles = nullptr;    // its cos/sin B tiles, split and swizzled
    int ncmpairs = 0;
    float *pvec = nullptr, *fvec = nullptr, *srf = nullptr, *Bx = nullptr;
    float *Tot = nullptr, *Ttl = nullptr;
    bool use_tc = false;
    // per-layer overrides and the adjoint (ocrt_gb_solve_batch_adjoint)
    bool any_layers = false;
    int ncot = 0, ntmax = 0;
    double *ldt = nullptr, *lss = nullptr, *cot = nullptr, *lamd = nullptr, *gout = nullptr,
           *grad = nullptr;
    float *dTc = nullptr, *dCa = nullptr, *dCb = nullptr, *srfW = nullptr, *AF = nullptr, *AJ = nullptr,
          *Abc = nullptr;
    float *ATot = nullptr;
    TaskState *Ast = nullptr;
    // angle-grid LUT mode
    bool any_lut = false;
    int lut_nvmax = 0, lut_ptmax = 0;
    long long lut_ntot = 0;
    double *lut_vza = nullptr, *lut_raa = nullptr, *lut_samp = nullptr, *lut_kappa = nullptr, *lut_out = nullptr;
    int *acnt = nullptr, *awork = nullptr;
    int *alcnt = nullptr, *aswork = nullptr, *adjlist[2] = {nullptr, nullptr};   // adjoint active-task lists
    float *opsT = nullptr;   // transposed aerosol operators for the tcgen05 adjoint source
    bool use_tc_adj = false;
    int gstride = 0, kstride = 0, grad_stride = 0;
};

size_t wave_budget_bytes()
{
    const char *e = getenv("OCRT_GB_WAVE_BYTES");
    if (e && *e) return (size_t)strtoull(e, nullptr, 10);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > 0) return (size_t)(fr * 0.7);
    return (size_t)8 << 30;
}

} // namespace

struct ocrt_plan {
    int n = 0;
    int ncot = 0;          // cotangent rows per pixel (adjoint plans)
    std::vector<Group> groups;
    long long launches = 0;
    double order_modes = 0;
    // per-kernel-class timing (enabled by ocrt_gb_set_timing)
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
    double ms[KC_N] = {0};
    long long cnt[KC_N] = {0};
    double flops[KC_N] = {0}, bytes[KC_N] = {0};
    bool work_done = false;
    // CUDA graph of a whole execute: captured on the second untimed execute
    // from the order counts the first one recorded, replayed from then on.
    cudaGraphExec_t gexec = nullptr;
    int executes = 0;
    bool graph_off = false;
    long long graph_launches = 0;
};

namespace {

template <class T> int up(T *&dst, const std::vector<T> &src)
{
    dst = (T *)dalloc(sizeof(T) * std::max<size_t>(src.size(), 1));
    if (!dst) return fail(OCRT_ERR_ALLOC, "device allocation failed");
    if (!src.empty()) CK(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, g_stream));
    return OCRT_OK;
}

template <class T> int alloc(T *&dst, size_t n)
{
    dst = (T *)dalloc(sizeof(T) * std::max<size_t>(n, 1));
    return dst ? OCRT_OK : fail(OCRT_ERR_ALLOC, "device allocation failed");
}

void free_group(Group &g)
{
    void *ptrs[] = {g.px, g.tasks, g.state, g.tout, g.res, g.pix_task0, g.gmu, g.gw, g.pw, g.h, g.ch, g.xd, g.yd, g.z,
                    g.tabs, g.Tc, g.Ca, g.Cb, g.Cq, g.Bp, g.Br, g.Bt, g.cs, g.frs, g.Eatt, g.lvf, g.lam, g.mb, g.mg, g.ma, g.mz, g.kappa, g.taudir,
                    g.active_cnt, g.mol_cnt, g.work, g.alist[0], g.alist[1], g.mlist[0], g.mlist[1], g.aflag,
                    g.err, g.F, g.J, g.ops, g.opt, g.molV, g.cmpairs, g.cstiles, g.pvec, g.fvec, g.srf, g.Bx, g.Tot, g.Ttl,
                    g.ldt, g.lss, g.cot, g.lamd, g.ATot, g.gout, g.grad, g.dTc, g.dCa, g.dCb, g.srfW, g.AF, g.AJ,
                    g.Abc, g.Ast, g.acnt, g.awork, g.opsT, g.alcnt, g.aswork, g.adjlist[0], g.adjlist[1],
                    g.lut_vza, g.lut_raa, g.lut_samp, g.lut_kappa, g.lut_out, g.vk_th, g.vk_p11, g.vkV, g.gtab,
                    g.atab, g.sprod, g.gcoef};
    for (void *p : ptrs) dfree(p);
}

// patch: optional per-pixel adjustment of the device record (the coupled
// ocean's pass flags, water-column geometry and source offsets), applied once
// the record is built from the case, options and aerosol.
int build_group(Group &g, const ocrt_case *cases, const ocrt_opts *opts, int opp, const ocrt_aerosol *aer, int app,
                const ocrt_layers *layers = nullptr, int ncot = 0, const double *cot = nullptr,
                const ocrt_lut *luts = nullptr, const std::function<void(int, PixDev &)> &patch = {})
{
    g.ncot = ncot;
    std::vector<double> ldt, lss, hcot, hlv, hlr;
    const Geom G = make_geom(g.N, g.E);
    g.G = G;
    // forward-only plans keep the order totals at the output levels alone
    g.G.tot_all = (ncot > 0 || g.keep_tot) ? 1 : 0;
    g.P = (int)g.idx.size();
    std::vector<double> mb, mgv, ma, mz, vth, vp11;
    size_t lev = 0, coef = 0;
    int task = 0;
    for (int q = 0; q < g.P; ++q) {
        const int i = g.idx[q];
        const ocrt_case &c = cases[i];
        const ocrt_opts &o = opp ? opts[i] : opts[0];
        const ocrt_aerosol *a = aer ? (app ? &aer[i] : &aer[0]) : nullptr;
        PixDev d;
        memset(&d, 0, sizeof(d));
        d.sza_deg = c.sza_deg; d.vza_deg = c.vza_deg; d.raa_deg = c.raa_deg; d.wavelength_nm = c.wavelength_nm;
        d.pressure_hpa = c.pressure_hpa; d.tau_r_input = c.tau_r_input;
        d.n_water = c.n_water; d.wind = c.wind_speed; d.surface = c.surface;
        d.sigma_type = c.sigma_type; d.q_conv = c.q_convention; d.decouple = c.decouple_sunglint;
        d.nt = o.n_layers; d.M = o.fourier_m_max; d.max_orders = o.max_orders; d.tol = o.tolerance;
        d.tau_r_source = o.tau_r_source; d.pssa = o.pssa; d.view_as_node = o.view_as_node;
        d.aer_h_km = o.aer_h_km; d.profile = o.rayleigh_profile; d.ray_h_km = o.rayleigh_h_km;
        d.nphi = o.n_phi_surface > 0 ? o.n_phi_surface : 1024;
        d.mom_off = -1; d.L_aer = -1;
        d.lay_off = -1;
        d.gas = o.gas ? o.gas->dev : nullptr;
        d.depol = OCRT_DEPOL; d.ext_off = -1;
        g.any_gas |= o.gas != nullptr;
        if (layers && (layers[i].dtau || layers[i].ssa)) {
            d.lay_off = (long long)std::max(ldt.size(), lss.size());
            ldt.resize(d.lay_off, 0.0); lss.resize(d.lay_off, 0.0);
            for (int l = 0; l < o.n_layers; ++l) {
                ldt.push_back(layers[i].dtau ? layers[i].dtau[l] : 0.0);
                lss.push_back(layers[i].ssa ? layers[i].ssa[l] : 0.0);
            }
            d.has_dtau = layers[i].dtau != nullptr;
            d.has_ssa = layers[i].ssa != nullptr;
            g.any_layers = true;
        }
        for (int r = 0; r < ncot; ++r)
            for (int x = 0; x < 3; ++x) hcot.push_back(cot[((size_t)i * ncot + r) * 3 + x]);
        g.ntmax = std::max(g.ntmax, o.n_layers);
        d.lut_nv = d.lut_nr = 0;
        if (luts) {
            const ocrt_lut &L = luts[i];
            d.lut_nv = L.n_vza; d.lut_nr = L.n_raa;
            d.lut_vo = (long long)hlv.size(); d.lut_ro = (long long)hlr.size(); d.lut_oo = g.lut_ntot;
            hlv.insert(hlv.end(), L.vza_deg, L.vza_deg + L.n_vza);
            hlr.insert(hlr.end(), L.raa_deg, L.raa_deg + L.n_raa);
            g.lut_ntot += (long long)L.n_vza * L.n_raa;
            g.lut_nvmax = std::max(g.lut_nvmax, L.n_vza);
            g.lut_ptmax = std::max(g.lut_ptmax, L.n_vza * L.n_raa);
            g.any_lut = true;
        }
        if (a && a->tau_a > 0.0) {
            d.mom_off = (int)mb.size(); d.L_aer = a->L_max; d.tau_a = a->tau_a; d.ssa_a = a->ssa_a;
            for (int l = 0; l <= a->L_max; ++l) {
                mb.push_back(a->beta[l]); mgv.push_back(a->gamma[l]); ma.push_back(a->alpha[l]); mz.push_back(a->zeta[l]);
            }
            if (a->use_value_kernel && a->n_ang_phase > 1) {
                d.vk_n = a->n_ang_phase;
                d.vk_off = (long long)vth.size();
                vth.insert(vth.end(), a->theta_phase, a->theta_phase + a->n_ang_phase);
                vp11.insert(vp11.end(), a->P11_phase, a->P11_phase + a->n_ang_phase);
                g.any_vk = true;
                g.vk_nmax = std::max(g.vk_nmax, d.vk_n);
            }
        }
        d.L = std::max(std::max(d.M, 2), d.L_aer);
        d.lev_off = (long long)lev; lev += d.nt + 1;
        d.coef_off = (long long)coef; coef += (size_t)d.nt * G.NR;
        d.task0 = task;
        g.hpix_task0.push_back(task);
        for (int m = 0; m <= d.M; ++m) {
            TaskDev t;
            memset(&t, 0, sizeof(t));
            t.pix = q; t.m = m; t.K = d.nt + 1; t.has_mol = m <= 2;
            g.htask.push_back(t);
        }
        task += d.M + 1;
        g.Lmax = std::max(g.Lmax, d.L);
        g.Mmax = std::max(g.Mmax, d.M);
        g.max_orders = std::max(g.max_orders, d.max_orders);
        g.nphi = std::max(g.nphi, d.nphi);
        const bool surf = c.surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN || c.surface == OCRT_SURFACE_FLAT;
        const bool flat = c.surface == OCRT_SURFACE_FLAT || (c.surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && c.wind_speed <= 0.0);
        if (patch) patch(q, d);
        g.any_rough |= surf && !flat && d.medium == 0;
        g.any_flat |= flat && d.medium == 0;
        g.any_water |= d.medium == 1;
        g.any_pssa |= o.pssa != 0;
        g.hpx.push_back(d);
    }
    g.T = task;
    g.nlev = lev; g.ncoef = coef; g.nmom = mb.size();
    // ---- waves of whole pixels under the workspace budget ----
    const size_t budget = wave_budget_bytes();
    const size_t op_elems = (size_t)G.NP * G.CIN;
    const bool tiles = tc_supported(G) && !force_simt();
    Wave w{0, 0, 0, 0, 0, 0, 0, 0, false, false};
    size_t bytes = 0;
    auto close = [&](int pend) {
        w.p1 = pend;
        w.t1 = pend < g.P ? g.hpx[pend].task0 : g.T;
        g.waves.push_back(w);
        g.wave_fld = std::max(g.wave_fld, w.fld); g.wave_ops = std::max(g.wave_ops, w.ops);
        g.wave_tail = std::max(g.wave_tail, w.tail);
        g.wave_srf = std::max(g.wave_srf, w.srf); g.wave_tasks = std::max(g.wave_tasks, w.t1 - w.t0);
        g.wave_pix = std::max(g.wave_pix, w.p1 - w.p0);
    };
    for (int q = 0; q < g.P; ++q) {
        const PixDev &d = g.hpx[q];
        const size_t K = d.nt + 1, nm = d.M + 1;
        const bool rough = (d.surface == 2 && d.wind > 0.0) || d.medium == 1;   // water: R_ww kernels
        const size_t pf = nm * K * G.LDC;
        const size_t po = (nm + 2 * std::min<size_t>(nm, 3)) * op_elems;
        const size_t ps = rough ? nm * ((size_t)G.NR * G.N * 9 + (size_t)G.NR * 9) : 0;
        size_t pb = pf * 12 + po * (tiles ? 12 : 4) + ps * 4 + nm * (4 * G.LDC + 24 * G.NR + 3 * (1 + G.E) * (g.Lmax + 1)) * 4;
        if (ncot > 0)   // adjoint fields, dR/dW, per-task partials
            pb += (size_t)ncot * (pf * 12 + nm * (G.NR * 3 * 4 + sizeof(TaskState) + (3 * K + 4) * 8)) + ps * 4 +
                  nm * (size_t)2 * (G.CIN + 32) * ((G.COUT + 31) & ~31) * 4;
        if (g.any_vk)   // the value kernel's tables of the pixel
            pb += (size_t)(g.Mmax + 1) * (G.N + 1) * 2 * G.NR * 4;
        if (q > w.p0 && bytes + pb > budget) {
            close(q);
            w = Wave{q, 0, d.task0, 0, 0, 0, 0, 0, false, false};
            bytes = 0;
        }
        TaskDev *tk = &g.htask[d.task0];
        for (size_t m = 0; m < nm; ++m) {
            tk[m].fld_off = (long long)w.fld; w.fld += K * G.LDC;
            tk[m].tail_off = (long long)w.tail; w.tail += 2 * (size_t)G.LDC;
            tk[m].op_off = (long long)w.ops; w.ops += op_elems;
            if (m <= 2) {
                tk[m].mol_off = (long long)w.ops; w.ops += op_elems;
                tk[m].uv_off = (long long)w.ops; w.ops += op_elems;
            } else {
                tk[m].mol_off = tk[m].uv_off = -1;
            }
            if (rough) { tk[m].srf_off = (long long)w.srf; w.srf += (size_t)G.NR * G.N * 9 + (size_t)G.NR * 9; }
            else tk[m].srf_off = -1;
            tk[m].has_mol = m <= 2;
        }
        w.Kmax = std::max(w.Kmax, (int)K);
        w.any_rough |= rough && d.medium == 0;
        w.any_water |= d.medium == 1;
        w.any_top |= d.medium == 1 && d.ext_off >= 0;
        w.any_flat |= (d.surface == 3 || (d.surface == 2 && d.wind <= 0.0));
        bytes += pb;
    }
    close(g.P);
    // ---- device buffers ----
    int rc;
    if ((rc = up(g.px, g.hpx)) || (rc = up(g.tasks, g.htask)) || (rc = up(g.pix_task0, g.hpix_task0)) ||
        (rc = up(g.mb, mb)) || (rc = up(g.mg, mgv)) || (rc = up(g.ma, ma)) || (rc = up(g.mz, mz)) ||
        (rc = alloc(g.state, g.T)) || (rc = alloc(g.tout, g.T)) || (rc = alloc(g.res, g.P)) ||
        (rc = alloc(g.gmu, g.N)) || (rc = alloc(g.gw, g.N)) || (rc = alloc(g.pw, 2 * (size_t)g.N)) ||
        (rc = alloc(g.h, g.nlev)) || (rc = alloc(g.ch, g.nlev)) || (rc = alloc(g.xd, g.nlev)) ||
        (rc = alloc(g.yd, g.nlev)) || (rc = alloc(g.z, g.nlev)) || (rc = alloc(g.tabs, g.any_gas ? g.nlev : 1)) ||
        (rc = alloc(g.Tc, g.ncoef)) || (rc = alloc(g.Ca, g.ncoef)) || (rc = alloc(g.Cb, g.ncoef)) ||
        (scan4_allowed(g.N) && (rc = alloc(g.Cq, g.ncoef / G.NR * (size_t)coef_quad_width(G.NR)))) ||
        (rc = alloc(g.Bp, (size_t)(g.Mmax + 1) * (g.Lmax + 1) * g.N)) ||
        (rc = alloc(g.Br, (size_t)(g.Mmax + 1) * (g.Lmax + 1) * g.N)) ||
        (rc = alloc(g.Bt, (size_t)(g.Mmax + 1) * (g.Lmax + 1) * g.N)) ||
        (rc = alloc(g.cs, (size_t)(g.Mmax + 1) * 2 * (g.nphi / 2) + 3 * (size_t)(g.nphi / 2))) ||
        (rc = alloc(g.Eatt, g.any_rough ? g.nlev * G.NR : 1)) || (rc = alloc(g.lvf, 3 * g.nlev)) ||
        (rc = alloc(g.lam, (size_t)g.P * (G.N + 2))) ||
        (rc = alloc(g.frs, (size_t)g.P * G.NR * 9)) ||
        (rc = alloc(g.kappa, g.P)) || (rc = alloc(g.taudir, g.P)) ||
        (rc = alloc(g.active_cnt, (size_t)g.max_orders + 2)) || (rc = alloc(g.mol_cnt, (size_t)g.max_orders + 2)) ||
        (rc = alloc(g.work, 4 * ((size_t)g.max_orders + 2))) || (rc = alloc(g.err, 2)) ||
        (rc = alloc(g.alist[0], g.wave_tasks)) || (rc = alloc(g.alist[1], g.wave_tasks)) ||
        (rc = alloc(g.mlist[0], g.wave_tasks)) || (rc = alloc(g.mlist[1], g.wave_tasks)) ||
        (rc = alloc(g.aflag, g.wave_tasks)) ||
        (rc = alloc(g.F, g.wave_fld)) || (rc = alloc(g.J, g.wave_fld)) ||
        (rc = alloc(g.Tot, g.wave_fld)) || (rc = alloc(g.Ttl, g.wave_tail)) ||
        (rc = alloc(g.ops, g.wave_ops)) || (rc = alloc(g.pvec, (size_t)g.wave_tasks * 2 * G.LDC)) ||
        (rc = alloc(g.fvec, g.any_flat ? (size_t)g.wave_tasks * 24 * G.NR : 1)) ||
        (rc = alloc(g.srf, g.wave_srf)) ||
        (rc = alloc(g.Bx, (size_t)g.wave_tasks * 3 * (1 + G.E) * (g.Lmax + 1))) ||
        (rc = alloc(g.gcoef, (size_t)(g.Mmax + 1) * (g.Lmax + 1) * 5)))
        return rc;
    if (g.any_layers && ((rc = up(g.ldt, ldt)) || (rc = up(g.lss, lss)))) return rc;
    if (g.any_vk) {
        g.vk_stride = (long long)(g.Mmax + 1) * (G.N + 1) * 2 * G.NR;
        if ((rc = up(g.vk_th, vth)) || (rc = up(g.vk_p11, vp11)) ||
            (rc = alloc(g.vkV, (size_t)g.wave_pix * g.vk_stride)))
            return rc;
    }
    if (g.any_lut && ((rc = up(g.lut_vza, hlv)) || (rc = up(g.lut_raa, hlr)) ||
                      (rc = alloc(g.lut_samp, (size_t)g.T * g.lut_nvmax * 4)) ||
                      (rc = alloc(g.lut_kappa, (size_t)g.lut_ntot)) || (rc = alloc(g.lut_out, 6 * (size_t)g.lut_ntot))))
        return rc;
    if (ncot > 0) {
        g.kstride = g.ntmax + 1;
        g.gstride = 3 * g.kstride + 2;
        g.grad_stride = 2 * g.ntmax + 1;
        const size_t na = (size_t)g.wave_tasks * ncot;
        if ((rc = up(g.cot, hcot)) || (rc = alloc(g.lamd, (size_t)g.P * (G.N + 2))) ||
            (rc = alloc(g.dTc, g.ncoef)) || (rc = alloc(g.dCa, g.ncoef)) || (rc = alloc(g.dCb, g.ncoef)) ||
            (rc = alloc(g.srfW, g.wave_srf)) || (rc = alloc(g.AF, g.wave_fld * ncot)) ||
            (rc = alloc(g.AJ, g.wave_fld * ncot)) ||
            (rc = alloc(g.ATot, g.wave_fld * ncot)) ||
            (rc = alloc(g.Abc, na * G.NR * 3)) || (rc = alloc(g.Ast, na)) ||
            (rc = alloc(g.acnt, (size_t)g.max_orders + 2)) || (rc = alloc(g.awork, (size_t)g.max_orders + 2)) ||
            (rc = alloc(g.alcnt, (size_t)g.max_orders + 2)) || (rc = alloc(g.aswork, (size_t)g.max_orders + 2)) ||
            (rc = alloc(g.adjlist[0], g.wave_tasks)) || (rc = alloc(g.adjlist[1], g.wave_tasks)) ||
            (rc = alloc(g.gout, na * g.gstride)) ||
            (rc = alloc(g.grad, (size_t)g.P * ncot * g.grad_stride)))
            return rc;
    }
    // ---- source kernels: tcgen05 for the aerosol contraction and the dense
    // m <= 2 molecular operator when the geometry allows it, CUDA cores
    // otherwise.  The per-order task lists themselves are built on the device
    // (k_primary, k_scan). ----
    // tensor maps of the chunked scan over this group's J / total buffers
    if (g.Cq && scan_tma_supported(G)) {
        g.smap_ok = true;
        const int chs[3] = {4, 8, 16};
        for (int i = 0; i < 3 && g.smap_ok; ++i)
            g.smap_ok = scan_tma_maps(G, chs[i], g.J, g.Tot, g.wave_fld, g.Cq, g.ncoef / G.NR, &g.smap[i]) == 0;
    }
    if (g.smap_ok && g.ncot > 0 && g.AF && !adj_scan_column())
        g.amap_ok = adj_scan_tma_maps(G, g.AF, g.ATot, g.wave_fld * g.ncot, g.Cq, g.ncoef / G.NR, &g.amap) == 0;
    g.use_tc = tc_supported(G) && !force_simt();
    if (g.use_tc && (rc = alloc(g.opt, 2 * g.wave_ops))) return rc;
    if (g.use_tc && (rc = alloc(g.molV, (size_t)3 * 32 * G.CIN))) return rc;
    g.tabs_tc = g.use_tc && tables_tc_supported(G, g.Lmax) && !force_simt_tables();
    if (g.tabs_tc && ((rc = alloc(g.gtab, tables_tc_gt_floats(G.N, g.Mmax, g.Lmax))) ||
                      (rc = alloc(g.atab, tables_tc_at_floats(g.Mmax, g.Lmax))) ||
                      (rc = alloc(g.sprod, (size_t)g.wave_tasks * G.N * 16))))
        return rc;
    // Cox-Munk pairs for the tensor-core projection: ring slots o < NR, incoming
    // Gauss slots and the sun (i = N); Gauss pairs with o > i are written by
    // their reciprocal pair
    if (g.any_rough && coxmunk_tc_supported(g.Mmax, g.nphi, ncot > 0) && !force_simt_coxmunk()) {
        std::vector<short2> pl;
        for (int o = 0; o < G.NR; ++o)
            for (int i = 0; i <= G.N; ++i)
                if (!(o < G.N && i < G.N && o > i)) pl.push_back(make_short2((short)o, (short)i));
        g.ncmpairs = (int)pl.size();
        if ((rc = up(g.cmpairs, pl)) || (rc = alloc(g.cstiles, coxmunk_tc_tiles_floats(g.Mmax, g.nphi)))) return rc;
    }
    if (g.use_tc && ncot > 0 && tc_adj_supported(G)) {
        const int KP = (G.COUT + 31) & ~31;
        if ((rc = alloc(g.opsT, (size_t)g.wave_tasks * 2 * (G.CIN + 32) * KP))) return rc;
        g.use_tc_adj = true;
    }
    for (Wave &w : g.waves) {
        w.n_simt = g.use_tc ? 0 : w.t1 - w.t0;
        w.n_tc = g.use_tc ? w.t1 - w.t0 : 0;
        w.n_mol = 0;
        for (int t = w.t0; t < w.t1; ++t) w.n_mol += g.htask[t].has_mol ? 1 : 0;
    }
    return OCRT_OK;
}

#define LAUNCH(plan, cls, ...)                                                        \
    do {                                                                              \
        cudaEvent_t e0_ = nullptr, e1_ = nullptr;                                     \
        if (g_timing) {                                                               \
            cudaEventCreate(&e0_); cudaEventCreate(&e1_); cudaEventRecord(e0_, st);   \
        }                                                                             \
        __VA_ARGS__;                                                                  \
        (plan)->launches++;                                                           \
        (plan)->cnt[cls]++;                                                           \
        if (g_timing) { cudaEventRecord(e1_, st); (plan)->ev.push_back({cls, {e0_, e1_}}); } \
        cudaError_t e_ = cudaGetLastError();                                          \
        if (e_ != cudaSuccess) return fail(OCRT_ERR_DEVICE, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

// Block size for `kernel` at shape `key`: the cached choice, else (when
// tuning is allowed: never while a graph is being captured) a measurement of
// every candidate the kernel's register and thread limits admit.
template <class F>
int tuned_block(const char *kernel, const void *fn, const std::vector<int> &key, bool may_tune, cudaStream_t st,
                F &&launch, int *bs)
{
    *bs = 256;
    if (!autotune_enabled()) return OCRT_OK;
    const auto k = std::make_pair(std::string(kernel), key);
    const auto it = g_tune_idx.find(k);
    if (it != g_tune_idx.end()) { *bs = g_tune[it->second].best; return OCRT_OK; }
    if (!may_tune) return OCRT_OK;
    cudaFuncAttributes fa;
    CK(cudaFuncGetAttributes(&fa, fn));
    TuneRec r;
    r.kernel = kernel;
    r.key = key;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(OCRT_ERR_DEVICE, "autotune: event create failed");
    }
    float best = 0.f;
    int rc = OCRT_OK;
    for (int b : kTuneBlocks) {
        if (b > fa.maxThreadsPerBlock) continue;
        launch(b);                      // first run absorbs module loading and cold caches
        cudaEventRecord(e0, st);
        launch(b);
        cudaEventRecord(e1, st);
        float t = 0.f;
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (e != cudaSuccess) { rc = fail(OCRT_ERR_DEVICE, std::string("autotune: ") + cudaGetErrorString(e)); break; }
        r.ms.push_back({b, t});
        if (r.ms.size() == 1 || t < best) { best = t; r.best = b; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    g_tune_idx[k] = g_tune.size();
    g_tune.push_back(r);
    *bs = r.best;
    return OCRT_OK;
}

LutBufs make_lut(Group &g)
{
    LutBufs L;
    L.vza = g.lut_vza; L.raa = g.lut_raa; L.samp = g.lut_samp; L.nvmax = g.lut_nvmax;
    L.kappa = g.lut_kappa; L.tau_dir = g.taudir; L.out = g.lut_out; L.ntot = g.lut_ntot;
    return L;
}

AdjBufs make_adj(Group &g)
{
    AdjBufs A;
    A.ncot = g.ncot; A.AF = g.AF; A.AJ = g.AJ; A.opsT = g.opsT; A.ATot = g.ATot; A.bc = g.Abc; A.st = g.Ast; A.acnt = g.acnt;
    A.cot = g.cot; A.gout = g.gout; A.gstride = g.gstride; A.kstride = g.kstride;
    A.dTc = g.dTc; A.dCa = g.dCa; A.dCb = g.dCb; A.srfW = g.srfW; A.grad = g.grad; A.grad_stride = g.grad_stride;
    A.awork = g.awork;
    A.aflag = g.aflag; A.alist[0] = g.adjlist[0]; A.alist[1] = g.adjlist[1]; A.lcnt = g.alcnt; A.swork = g.aswork;
    return A;
}

// Adjoint of one wave, right after its forward orders (the forward fields of
// the wave are still resident).
int run_adjoint_wave(ocrt_plan *plan, Group &g, Wave &w, const BatchBufs &B, const WaveBufs &W, cudaStream_t st,
                     int tc_grid, int mol_grid, int mtiles, int ltiles, dim3 sgrid, size_t tc_smem, bool capture)
{
    const Geom G = g.G;
    const int nw = w.t1 - w.t0, na = nw * g.ncot;
    const int scan_threads = ((G.COUT + 31) / 32) * 32;
    // the scattered field Xs = F_tot - F_last and its source S Xs = J_tot - J_1;
    // the tensor-core pass forms Xs from the total as it loads the rows, the
    // CUDA-core passes read it from F (k_adj_prep)
    const bool xs_in_f = w.n_simt > 0 || w.n_tc == 0;
    if (xs_in_f) LAUNCH(plan, KC_ADJ_TOTALS, k_adj_prep<<<nw, scan_threads, 0, st>>>(B, W, G, w.t0));
    const int it = g.max_orders + 1;
    LAUNCH(plan, KC_ADJ_TOTALS, k_fill_all<<<1, 256, 0, st>>>(B, w.t0, nw, it));
    if (w.n_simt) LAUNCH(plan, KC_ADJ_TOTALS, k_source_simt<<<sgrid, 256, 0, st>>>(B, W, G, w.t0, it));
    if (w.n_tc && xs_in_f)
        LAUNCH(plan, KC_ADJ_TOTALS, k_source_tc<<<tc_grid, tc_fwd_threads(), tc_smem, st>>>(B, W, G, w.t0, it, mtiles));
    else if (w.n_tc)
        LAUNCH(plan, KC_ADJ_TOTALS,
               k_source_tc_xs<<<tc_grid, tc_fwd_threads(), tc_smem, st>>>(B, W, G, w.t0, it, mtiles));
    if (w.n_mol && !w.n_tc)
        LAUNCH(plan, KC_ADJ_TOTALS, k_mol_lowrank<<<mol_grid, 256, mol_smem_bytes(G), st>>>(
                   B, W, G, w.t0, it, ltiles, g.Bp, g.Br, g.Bt, g.Lmax));
    // adjoint successive orders (the adjoint field, source and total are not
    // cleared: k_adj_init writes a_1's TOA row, order 1 reads no other row of
    // a_1 nor the total, and its scan zeroes the muJ columns no order writes)
    CK(cudaMemsetAsync(g.Abc, 0, sizeof(float) * (size_t)na * G.NR * 3, st));
    CK(cudaMemsetAsync(g.acnt, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
    CK(cudaMemsetAsync(g.awork, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
    CK(cudaMemsetAsync(g.alcnt, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
    CK(cudaMemsetAsync(g.aswork, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
    CK(cudaMemsetAsync(g.aflag, 0, (size_t)nw, st));
    const int KP = (G.COUT + 31) & ~31;
    const int amt = (g.ncot * w.Kmax + 127) / 128;
    if (g.use_tc_adj) {
        LAUNCH(plan, KC_ADJ_OTHER, k_op_transpose<<<dim3(nw, (G.CIN + 31) / 32, KP / 32), dim3(32, 8), 0, st>>>(
                   g.tasks, w.t0, nw, G, g.ops, g.opsT));
        if (w.n_mol) LAUNCH(plan, KC_ADJ_OTHER, k_mol_utrans<<<nw, 256, 0, st>>>(g.tasks, w.t0, nw, G, g.ops, g.opsT));
    }
    const AdjBufs A = make_adj(g);
    LAUNCH(plan, KC_ADJ_OTHER, k_adj_init<<<(na + 127) / 128, 128, 0, st>>>(B, A, G, w.t0, na));
    LAUNCH(plan, KC_ADJ_OTHER, k_adj_list_all<<<(nw + 255) / 256, 256, 0, st>>>(A, nw));
    const dim3 agrid(na, (w.Kmax + ST_M_TILE - 1) / ST_M_TILE, (G.LDC + ST_N_TILE - 1) / ST_N_TILE);
    const int surf_threads = ((3 * G.N + 31) / 32) * 32;
    if (!capture) w.adj_stop = INT_MAX;
    for (int j = 1; j <= g.max_orders; ++j) {
        const int nitem = nw * ((g.ncot + ADJ_RB - 1) / ADJ_RB);
        if (g.amap_ok)
            LAUNCH(plan, KC_ADJ_SCAN, adj_scan_tma_launch(std::min(nitem, 2 * g_nsm), st, B, A, G, w.t0, j, g.amap));
        else
            LAUNCH(plan, KC_ADJ_SCAN, k_adj_scan<<<nitem, scan_threads, adj_scan_smem_bytes(scan_threads), st>>>(
                       B, A, G, w.t0, j));
        LAUNCH(plan, KC_ADJ_SCAN, k_compact_adj<<<1, COMPACT_THREADS, 0, st>>>(A, nw, j));
        if (capture) {
            if (j == w.adj_stop) break;
        } else if ((j - 1) % 4 == 0 || j == g.max_orders) {
            CK(cudaMemcpyAsync(g_pinned, g.acnt + j, sizeof(int), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (*g_pinned == 0) { w.adj_stop = j; break; }
        }
        if (g.use_tc_adj)
            LAUNCH(plan, KC_ADJ_SOURCE, k_adj_source_tc<<<std::min(nw * amt, g_nsm), tc_fwd_threads(), tc_adj_smem_bytes(G),
                                                         st>>>(B, W, A, G, w.t0, j, amt, nw));
        else
            LAUNCH(plan, KC_ADJ_SOURCE, k_adj_source<<<agrid, 256, 0, st>>>(B, W, A, G, w.t0));
        if (w.n_mol && !g.use_tc_adj)
            LAUNCH(plan, KC_ADJ_SOURCE, k_adj_mol<<<dim3(na, ltiles), 256, adj_mol_smem_bytes(G), st>>>(
                       B, W, A, G, w.t0, g.Bp, g.Br, g.Bt, g.Lmax));
        if (w.any_rough)
            LAUNCH(plan, KC_ADJ_OTHER, k_adj_surface<<<std::min(na, 32 * g_nsm), surf_threads, 0, st>>>(B, W, A, G,
                                                                                                  w.t0, j));
    }
    if (capture && w.adj_stop != INT_MAX)
        LAUNCH(plan, KC_ADJ_OTHER, k_stop_check<<<1, 32, 0, st>>>(g.acnt + w.adj_stop, g.err + 1));
    const int grad_threads = 2 * ((3 * G.N + 3 + 31) / 32) * 32;
    // cotangent rows per block: up to ADJ_RB while the per-warp level sums fit
    const size_t row_smem = sizeof(float) * 3 * ((size_t)g.ntmax + 1) * (grad_threads / 32);
    const int grad_rb = std::max(1, std::min({ADJ_RB, g.ncot, (int)((200 * 1024) / row_smem)}));
    LAUNCH(plan, KC_ADJ_GRAD, k_adj_grad<<<nw * ((g.ncot + grad_rb - 1) / grad_rb), grad_threads, row_smem * grad_rb, st>>>(
               B, W, A, G, w.t0, grad_rb, xs_in_f ? 1 : 0));
    LAUNCH(plan, KC_ADJ_GRAD, k_adj_pixel<<<(w.p1 - w.p0) * g.ncot, 256, sizeof(double) * (g.ntmax + 2), st>>>(
               B, W, A, G, w.p0, w.t0));
    return OCRT_OK;
}

// One execute of a group.  Eager (capture == false): host polls of the active
// counts end each wave's order loop and record where it ended.  Capture: the
// same launch sequence with the recorded order counts and no host polls, for
// a CUDA graph; a device check flags a replay that ends with tasks active.
int run_group(ocrt_plan *plan, Group &g, cudaStream_t st, bool capture)
{
    const Geom G = g.G;
    const int P = g.P;
    CK(cudaMemsetAsync(g.err, 0, 2 * sizeof(int), st));
    LAUNCH(plan, KC_SETUP, k_gauss<<<1, 64, 0, st>>>(g.N, g.gmu, g.gw, g.pw));
    LAUNCH(plan, KC_SETUP, k_pixel_setup<<<(P + 127) / 128, 128, 0, st>>>(g.px, P, g.N, g.gmu));
    LAUNCH(plan, KC_SETUP, k_levels<<<dim3(2, P), 256, 0, st>>>(g.px, P, g.h, g.ch, g.xd, g.yd, g.z));
    if (g.any_water)
        LAUNCH(plan, KC_SETUP, k_levels_water<<<dim3(2, P), 256, 0, st>>>(g.px, P, g.h, g.ch, g.xd, g.yd, g.z));
    LAUNCH(plan, KC_SETUP, k_level_mix<<<dim3(2, P), 256, 0, st>>>(g.px, P, g.z, g.xd, g.yd));
    if (g.any_gas)
        LAUNCH(plan, KC_SETUP, k_gas_apply<<<P, 256, 0, st>>>(g.px, P, g.h, g.ch, g.xd, g.yd, g.z, g.tabs));
    if (g.any_layers)
        LAUNCH(plan, KC_SETUP, k_layers_apply<<<P, 256, 0, st>>>(g.px, P, g.ldt, g.lss, g.h, g.ch, g.xd, g.yd, g.err));
    LAUNCH(plan, KC_SETUP, k_coef<<<dim3(16, P), 256, 0, st>>>(g.px, P, g.N, G.NR, g.gmu, g.h, g.Tc, g.Ca, g.Cb));
    if (g.Cq)
        LAUNCH(plan, KC_SETUP, k_coef_quads<<<dim3(16, P), 256, 0, st>>>(g.px, P, g.N, G.NR, g.Tc, g.Ca, g.Cb, g.Cq));
    LAUNCH(plan, KC_SETUP, k_gsf_coefs<<<g.Mmax + 1, 128, 0, st>>>(g.Mmax, g.Lmax, g.gcoef));
    LAUNCH(plan, KC_SETUP, k_basis_gauss<<<g.Mmax + 1, 64, 0, st>>>(g.N, g.Mmax, g.Lmax, g.gmu, g.Bp, g.Br, g.Bt,
                                                                   g.gcoef));
    if (g.tabs_tc)
        LAUNCH(plan, KC_SETUP, k_basis_perm<<<dim3(8, g.Mmax + 1), 256, 0, st>>>(g.N, g.Mmax, g.Lmax, g.Bp, g.Br, g.Bt,
                                                                                g.gtab, g.atab));
    if (g.use_tc)
        LAUNCH(plan, KC_SETUP, k_mol_vtab<<<std::min(g.Mmax, 2) + 1, 256, 0, st>>>(G, g.Lmax, g.Bp, g.Br, g.Bt, g.gw,
                                                                                  g.molV));
    if (g.any_rough) {
        LAUNCH(plan, KC_SETUP, k_cs_table<<<g.Mmax + 2, 256, 0, st>>>(g.Mmax, g.nphi, g.cs));
        if (g.cstiles) LAUNCH(plan, KC_SETUP, k_cs_tiles<<<g.nphi / 64, 256, 0, st>>>(g.Mmax, g.nphi, g.cs, g.cstiles));
        LAUNCH(plan, KC_SETUP, k_seed_att<<<dim3(8, P), 256, 0, st>>>(g.px, P, g.N, g.gmu, g.h, g.Eatt));
        LAUNCH(plan, KC_SETUP, k_sancer<<<P, 128, 0, st>>>(g.px, P, g.N, g.gmu, g.lam, g.ncot ? g.lamd : nullptr));
    }
    LAUNCH(plan, KC_SETUP, k_level_float<<<dim3(2, P), 256, 0, st>>>(g.px, P, g.xd, g.yd, g.ch, g.lvf));
    if (g.any_flat) LAUNCH(plan, KC_SETUP, k_flat_fresnel<<<P, 128, 0, st>>>(g.px, P, g.N, g.gmu, g.frs));
    if (g.ncot)
        LAUNCH(plan, KC_SETUP, k_coef_deriv<<<dim3(16, P), 256, 0, st>>>(g.px, P, g.N, g.gmu, g.h, g.dTc, g.dCa, g.dCb));

    BatchBufs B;
    B.px = g.px; B.tasks = g.tasks; B.state = g.state; B.tout = g.tout;
    B.gmu = g.gmu; B.gw = g.gw; B.pw = g.pw; B.h = g.h; B.ch = g.ch; B.xd = g.xd; B.yd = g.yd; B.z = g.z;
    B.Tc = g.Tc; B.Ca = g.Ca; B.Cb = g.Cb; B.Cq = g.Cq; B.frs = g.frs; B.Eatt = g.Eatt; B.lvf = g.lvf; B.active_cnt = g.active_cnt; B.err = g.err;
    B.mol_cnt = g.mol_cnt; B.work = g.work;
    B.alist[0] = g.alist[0]; B.alist[1] = g.alist[1]; B.mlist[0] = g.mlist[0]; B.mlist[1] = g.mlist[1];
    B.molV = g.molV;
    B.ext = g.ext;
    B.aflag = g.aflag;
    WaveBufs W;
    W.F = g.F; W.J = g.J; W.Tot = g.Tot; W.Ttl = g.Ttl; W.ops = g.ops; W.opt = g.use_tc ? g.opt : nullptr;
    W.pvec = g.pvec;
    W.fvec = g.any_flat ? g.fvec : nullptr; W.srf = g.srf;
    const int scan_threads = ((G.COUT + 31) / 32) * 32;
    const int poll = 4;
    // ---- transport-scan implementation: forced, tuned, or being tuned ----
    std::vector<int> scan_cands;
    if (!g.Cq) {
        scan_cands.push_back(SK_COLUMN);
    } else {
        scan_cands.push_back(SK_QUAD);
        if (g.smap_ok)
            for (int k = SK_TMA_8_3; k < SK_N; ++k)
                if (scan_tma_blocks(k, G) > 0) scan_cands.push_back(k);
    }
    int scan_pick = -1;
    ScanTune *stune = nullptr;
    std::vector<int> stune_key;
    {
        const int forced = scan_forced();
        int kmax = 0;
        for (const Wave &w : g.waves) kmax = std::max(kmax, w.Kmax);
        const std::vector<int> key = {G.N, G.E, kmax, G.tot_all};
        const int dflt = scan_cands.size() > 1 ? scan_cands[1] : scan_cands[0];
        if (forced >= 0 && std::find(scan_cands.begin(), scan_cands.end(), forced) != scan_cands.end()) {
            scan_pick = forced;
        } else if (scan_cands.size() == 1 || !autotune_enabled()) {
            scan_pick = dflt;
        } else {
            ScanTune &t = g_scan_tune[key];
            if (t.cand.empty()) t.cand = scan_cands;
            if (t.best >= 0) scan_pick = t.best;
            else if (capture) scan_pick = dflt;
            else stune = &t;
        }
        if (stune) stune_key = key;
    }
    struct ScanTrial { int kind, it; cudaEvent_t e0, e1; };
    std::vector<ScanTrial> scan_trials;
    for (Wave &w : g.waves) {
        const int nw = w.t1 - w.t0;
        if (!capture) w.fwd_stop = INT_MAX;
        // the plain operators are read only off the forward tensor-core path; the
        // molecular factors it reads are written in full by k_tables, and
        // k_tables_tc writes every row of the plain operator it keeps
        if (!g.use_tc || (g.ncot > 0 && !g.tabs_tc)) CK(cudaMemsetAsync(g.ops, 0, sizeof(float) * w.ops, st));
        CK(cudaMemsetAsync(g.pvec, 0, sizeof(float) * (size_t)nw * 2 * G.LDC, st));
        if (g.any_flat) CK(cudaMemsetAsync(g.fvec, 0, sizeof(float) * (size_t)nw * 24 * G.NR, st));
        CK(cudaMemsetAsync(g.active_cnt, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
        CK(cudaMemsetAsync(g.mol_cnt, 0, sizeof(int) * ((size_t)g.max_orders + 2), st));
        CK(cudaMemsetAsync(g.work, 0, sizeof(int) * 4 * ((size_t)g.max_orders + 2), st));
        CK(cudaMemsetAsync(g.aflag, 0, (size_t)nw, st));
        LAUNCH(plan, KC_TABLES, k_basis_pix<<<(nw + 128 / (1 + G.E) - 1) / (128 / (1 + G.E)), 128, 0, st>>>(
                   g.tasks, w.t0, nw, g.px, g.Lmax, G.E, g.Bx, g.gcoef));
        if (g.any_vk)
            LAUNCH(plan, KC_TABLES, k_value_pfm<<<dim3(((G.N + 1) * 2 * G.NR + 127) / 128, w.p1 - w.p0), 128,
                                                  value_kernel_smem_bytes(g.vk_nmax), st>>>(
                       g.px, w.p0, G, g.gmu, g.vk_th, g.vk_p11, g.vkV, g.vk_stride));
        const int plain_ops = (!g.use_tc || g.ncot > 0) ? 1 : 0;
        int rc = 0;
        if (g.tabs_tc) {
            // the aerosol operator and the sun-outgoing products on tcgen05, then
            // the molecular operator and the solar row
            LAUNCH(plan, KC_TABLES, k_tables_tc<<<std::min(nw, g_nsm), tables_tc_threads(),
                                                  tables_tc_smem_bytes(G, g.Lmax), st>>>(
                       g.tasks, w.t0, nw, g.px, G, g.Lmax, g.gtab, g.atab, g.Bx, g.gw, g.mb, g.mg, g.ma, g.mz, g.ops, W.opt,
                       plain_ops, g.any_vk ? g.vkV : nullptr, w.p0, g.vk_stride, g.sprod, g.err));
            LAUNCH(plan, KC_TABLES, k_tables<<<dim3(nw, 1), 64, tables_smem_bytes(64, G.N, g.Lmax), st>>>(
                       g.tasks, w.t0, nw, g.px, G, g.Lmax, g.Bp, g.Br, g.Bt, g.Bx, g.gw, g.mb, g.mg, g.ma, g.mz,
                       g.ops, g.pvec, W.fvec, W.opt, plain_ops, g.any_vk ? g.vkV : nullptr, w.p0, g.vk_stride,
                       g.sprod));
        } else {
            auto tables = [&](int b) {
                k_tables<<<dim3(nw, tables_yblocks(b, G.NR, G.N)), b, tables_smem_bytes(b, G.N, g.Lmax), st>>>(
                    g.tasks, w.t0, nw, g.px, G, g.Lmax, g.Bp, g.Br, g.Bt, g.Bx, g.gw, g.mb, g.mg, g.ma, g.mz, g.ops,
                    g.pvec, W.fvec, W.opt, plain_ops, g.any_vk ? g.vkV : nullptr, w.p0, g.vk_stride, nullptr);
            };
            int tb = 256;
            rc = tuned_block("k_tables", (const void *)k_tables, {G.N, g.Lmax, g.Mmax}, !capture, st, tables, &tb);
            if (rc) return rc;
            LAUNCH(plan, KC_TABLES, tables(tb));
        }
        if (g.use_tc)
            LAUNCH(plan, KC_TABLES, k_mol_dense<<<nw, 256, 0, st>>>(g.tasks, w.t0, nw, G, g.Lmax, g.Bp, g.Br, g.Bt,
                                                                     g.gw, g.ops, g.opt));
        if (w.any_rough) {
            const bool dw = g.ncot > 0;
            const int np = w.p1 - w.p0;
            const size_t smem = coxmunk_smem_bytes(g.nphi, dw);
            auto coxmunk = [&](int b) {
                if (dw)
                    k_coxmunk_dw<<<dim3(G.N + 1, G.NR, np), b, smem, st>>>(g.tasks, g.px, w.p0, g.pix_task0, G, g.gmu,
                                                                         g.cs, g.Mmax, g.lam, g.lamd, g.srf, g.srfW);
                else
                    k_coxmunk<<<dim3(G.N + 1, G.NR, np), b, smem, st>>>(g.tasks, g.px, w.p0, g.pix_task0, G, g.gmu,
                                                                      g.cs, g.Mmax, g.lam, g.srf);
            };
            if (g.cmpairs) {
                const int per = coxmunk_tc_pairs_per_cta();
                LAUNCH(plan, KC_COXMUNK, k_coxmunk_tc<<<dim3((g.ncmpairs + per - 1) / per, np), coxmunk_tc_threads(dw),
                                                         coxmunk_tc_smem_bytes(g.Mmax, dw), st>>>(
                           g.tasks, g.px, w.p0, g.pix_task0, G, g.gmu, g.cs, g.cstiles, g.Mmax, g.lam,
                           dw ? g.lamd : nullptr, g.srf, dw ? g.srfW : nullptr, g.cmpairs, g.ncmpairs, dw ? 1 : 0,
                           g.err));
            } else {
                int cb = 256;
                rc = tuned_block(dw ? "k_coxmunk_dw" : "k_coxmunk",
                                 dw ? (const void *)k_coxmunk_dw : (const void *)k_coxmunk, {G.N, g.nphi, g.Mmax},
                                 !capture, st, coxmunk, &cb);
                if (rc) return rc;
                LAUNCH(plan, KC_COXMUNK, coxmunk(cb));
            }
        }
        if (w.any_water)
            LAUNCH(plan, KC_COXMUNK, k_rww<<<dim3(G.NR, w.p1 - w.p0), 256,
                                             iface_smem_bytes(g.Mmax, g.nphi_ww, 0), st>>>(
                       g.tasks, g.px, w.p0, g.pix_task0, G, g.gmu, g.nphi_ww, g.srf));
        const dim3 sgrid(w.n_simt, (w.Kmax + ST_M_TILE - 1) / ST_M_TILE, (G.COUT + ST_N_TILE - 1) / ST_N_TILE);
        const int mtiles = (w.Kmax + 127) / 128, ltiles = (w.Kmax + 31) / 32;
        const size_t tc_smem = tc_smem_bytes(G);
        // Persistent grids: CTAs pull (task, level tile) items from the order's
        // active list, so tasks that have converged cost nothing.
        const int tc_grid = std::min(w.n_tc * mtiles, g_nsm);
        const int mol_grid = std::min(w.n_mol * ltiles, 4 * g_nsm);
        const int scan_grid = std::min(nw, 8 * g_nsm), scan4_grid = std::min(nw, 16 * g_nsm);
        if (w.any_top) {
            // skylight first-scatter source of the water column: the source pass
            // over the unscattered skylight field, every task active, into J
            const int itd = g.max_orders + 1;
            LAUNCH(plan, KC_PRIMARY, k_dtop_field<<<nw, 256, 0, st>>>(B, W, G, w.t0));
            LAUNCH(plan, KC_PRIMARY, k_fill_all<<<1, 256, 0, st>>>(B, w.t0, nw, itd));
            if (w.n_simt) LAUNCH(plan, KC_SOURCE, k_source_simt<<<sgrid, 256, 0, st>>>(B, W, G, w.t0, itd));
            if (w.n_tc)
                LAUNCH(plan, KC_SOURCE_TC, k_source_tc<<<tc_grid, tc_fwd_threads(), tc_smem, st>>>(
                           B, W, G, w.t0, itd, mtiles));
            if (w.n_mol && !w.n_tc)
                LAUNCH(plan, KC_MOL, k_mol_lowrank<<<mol_grid, 256, mol_smem_bytes(G), st>>>(
                           B, W, G, w.t0, itd, ltiles, g.Bp, g.Br, g.Bt, g.Lmax));
            CK(cudaMemsetAsync(g.active_cnt + (itd - 1), 0, sizeof(int), st));
            CK(cudaMemsetAsync(g.mol_cnt + (itd - 1), 0, sizeof(int), st));
        }
        if (g.Cq && !w.any_flat && !primary_column())
            LAUNCH(plan, KC_PRIMARY, k_primary4<<<nw, scan4_threads(G), 0, st>>>(B, W, G, w.t0));
        else
            LAUNCH(plan, KC_PRIMARY, k_primary<<<nw, scan_threads, 0, st>>>(B, W, G, w.t0));
        LAUNCH(plan, KC_PRIMARY, k_compact<<<1, COMPACT_THREADS, 0, st>>>(B, w.t0, nw, 2));
        for (int it = 2; it <= g.max_orders; ++it) {
            if (w.n_simt)
                LAUNCH(plan, KC_SOURCE, k_source_simt<<<sgrid, 256, 0, st>>>(B, W, G, w.t0, it));
            if (w.n_tc)
                LAUNCH(plan, KC_SOURCE_TC, k_source_tc<<<tc_grid, tc_fwd_threads(), tc_smem, st>>>(
                           B, W, G, w.t0, it, mtiles));
            if (w.n_mol && !w.n_tc)
                LAUNCH(plan, KC_MOL, k_mol_lowrank<<<mol_grid, 256, mol_smem_bytes(G), st>>>(
                           B, W, G, w.t0, it, ltiles, g.Bp, g.Br, g.Bt, g.Lmax));
            {
                int kind = scan_pick;
                const bool tuning = kind < 0;
                if (tuning) kind = stune->cand[(it - 2) % stune->cand.size()];
                cudaEvent_t te0 = nullptr, te1 = nullptr;
                if (tuning) {
                    CK(cudaEventCreate(&te0));
                    CK(cudaEventCreate(&te1));
                    CK(cudaEventRecord(te0, st));
                }
                switch (kind) {
                case SK_COLUMN:
                    LAUNCH(plan, KC_SCAN, k_scan<<<scan_grid, scan_threads, scan_smem_bytes(scan_threads), st>>>(
                               B, W, G, w.t0, it));
                    break;
                case SK_QUAD:
                    LAUNCH(plan, KC_SCAN, k_scan4<<<scan4_grid, scan4_threads(G),
                                                     scan4_smem_bytes(scan4_threads(G)), st>>>(B, W, G, w.t0, it));
                    break;
                default: {
                    const int ch = sk_ch[kind], ns = sk_ns[kind];
                    const ScanMaps &sm = g.smap[sk_map_index(ch)];
                    const int grid = std::min(nw, scan_tma_blocks(kind, G) * g_nsm);
                    LAUNCH(plan, KC_SCAN, scan_tma_launch(ch, ns, grid, st, B, W, G, w.t0, it, sm));
                }
                }
                if (tuning) {
                    CK(cudaEventRecord(te1, st));
                    scan_trials.push_back({kind, it, te0, te1});
                }
                LAUNCH(plan, KC_SCAN, k_compact<<<1, COMPACT_THREADS, 0, st>>>(B, w.t0, nw, it + 1));
            }
            if (capture) {
                if (it == w.fwd_stop) break;
            } else if ((it - 1) % poll == 0 || it == g.max_orders) {
                CK(cudaMemcpyAsync(g_pinned, g.active_cnt + it, sizeof(int), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (*g_pinned == 0) { w.fwd_stop = it; break; }
            }
        }
        if (stune && !scan_trials.empty()) {
            // scan autotuner: per-candidate time over the level-columns its orders scanned
            std::vector<int> wk(4 * ((size_t)g.max_orders + 2));
            CK(cudaMemcpyAsync(wk.data(), g.work, sizeof(int) * wk.size(), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            for (const ScanTrial &t : scan_trials) {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, t.e0, t.e1) != cudaSuccess) cudaGetLastError();
                const double lev = (double)wk[(size_t)t.it * 4 + 3] * G.COUT;
                if (lev > 0 && ms > 0.f) {
                    stune->ms[t.kind] += ms;
                    stune->lev[t.kind] += lev;
                    stune->n[t.kind]++;
                }
                cudaEventDestroy(t.e0);
                cudaEventDestroy(t.e1);
            }
            scan_trials.clear();
            bool all = true;
            for (int k : stune->cand) all = all && stune->n[k] >= 2;
            if (all) {
                TuneRec r;
                r.kernel = "transport_scan";
                r.key = stune_key;
                r.labels = sk_names;
                double bestv = 0;
                for (int k : stune->cand) {
                    const double v = stune->ms[k] / stune->lev[k] * 1e6;   // ns per level-column
                    r.ms.push_back({k, (float)v});
                    if (stune->best < 0 || v < bestv) { bestv = v; stune->best = k; }
                }
                r.best = stune->best;
                g_tune_idx[std::make_pair(r.kernel, r.key)] = g_tune.size();
                g_tune.push_back(r);
                scan_pick = stune->best;
                stune = nullptr;
            }
        }
        if (capture && w.fwd_stop != INT_MAX)
            LAUNCH(plan, KC_EXTRACT, k_stop_check<<<1, 32, 0, st>>>(g.active_cnt + w.fwd_stop, g.err + 1));
        LAUNCH(plan, KC_EXTRACT, k_extract<<<(nw + 127) / 128, 128, 0, st>>>(B, W, G, w.t0, nw));
        if (g.edge)
            LAUNCH(plan, KC_EXTRACT, k_edges<<<(nw * G.NR + 127) / 128, 128, 0, st>>>(B, W, G, w.t0, nw, g.edge));
        if (g.any_lut) LAUNCH(plan, KC_EXTRACT, k_lut_sample<<<nw, 128, 0, st>>>(B, W, make_lut(g), G, w.t0, nw));
        if (g.ncot) {
            const int rc = run_adjoint_wave(plan, g, w, B, W, st, tc_grid, mol_grid, mtiles, ltiles, sgrid, tc_smem,
                                            capture);
            if (rc) return rc;
        }
    }
    if (g.any_pssa) {
        int maxnt = 0;
        for (const PixDev &d : g.hpx) maxnt = std::max(maxnt, d.nt);
        const size_t smem = sizeof(double) * (6 * (size_t)maxnt + 6) + sizeof(int) * ((size_t)maxnt + 1);
        LAUNCH(plan, KC_IPSS, k_ipss<<<P, 256, smem, st>>>(g.px, P, g.h, g.z, g.xd, g.yd,
                                                           g.any_gas ? g.tabs : nullptr, g.mb, g.vk_th, g.vk_p11,
                                                           g.kappa, g.taudir));
        if (g.any_lut)
            LAUNCH(plan, KC_IPSS, k_ipss_lut<<<dim3(std::min(g.lut_ptmax, 2048), P), 256, smem, st>>>(
                       g.px, P, g.h, g.z, g.xd, g.yd, g.any_gas ? g.tabs : nullptr, g.mb, g.vk_th, g.vk_p11,
                       g.lut_vza, g.lut_raa, g.lut_kappa));
    }
    if (g.any_lut)
        LAUNCH(plan, KC_FINAL, k_lut_final<<<dim3((g.lut_ptmax + 127) / 128, P), 128, 0, st>>>(g.px, P, make_lut(g),
                                                                                              g.pix_task0));
    LAUNCH(plan, KC_FINAL, k_finalize<<<(P + 127) / 128, 128, 0, st>>>(g.px, P, g.state, g.tout, g.gmu, g.gw, g.h,
                                                              g.kappa, g.taudir, g.res));
    return OCRT_OK;
}

} // namespace

extern "C" {

void ocrt_opts_default(ocrt_opts *o)
{
    if (!o) return;
    o->n_mu = 24; o->n_layers = 40; o->fourier_m_max = 2; o->max_orders = 20; o->tolerance = 1e-7;
    o->tau_r_source = OCRT_TAU_R_AUTO; o->pssa = 0; o->view_as_node = 1; o->aer_h_km = 2.0;
    o->rayleigh_profile = OCRT_PROFILE_US62; o->rayleigh_h_km = 8.0; o->n_phi_surface = 1024;
    o->gas = nullptr;
}

void ocrt_case_default(ocrt_case *c)
{
    if (!c) return;
    c->sza_deg = 40.0; c->vza_deg = 30.0; c->raa_deg = 90.0; c->wavelength_nm = 555.0;
    c->surface = OCRT_SURFACE_BLACK; c->pressure_hpa = 1013.25; c->tau_r_input = 0.0;
    c->n_water = 1.34; c->wind_speed = 0.0; c->sigma_type = 1; c->q_convention = 1; c->decouple_sunglint = 0;
}

int ocrt_gb_init(int device)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_device >= 0) return OCRT_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) { cudaGetLastError(); return fail(OCRT_ERR_DEVICE, "no CUDA device"); }
    if (device < 0 || device >= n) return fail(OCRT_ERR_ARGS, "device index out of range");
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
    CK(cudaMallocHost(&g_pinned, sizeof(int) * 16));
    CK(cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, device));
    CK(cudaFuncSetAttribute(k_coxmunk, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_coxmunk_dw, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_coxmunk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    CK(cudaFuncSetAttribute(k_ipss, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(tables_tc_init());
    CK(cudaFuncSetAttribute(k_value_pfm, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_scan4, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(scan_tma_init());
    CK(cudaFuncSetAttribute(k_adj_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_source_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    CK(cudaFuncSetAttribute(k_source_tc_xs, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    CK(cudaFuncSetAttribute(k_mol_lowrank, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_adj_mol, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_adj_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CK(cudaFuncSetAttribute(k_adj_source_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    g_device = device;
    return OCRT_OK;
}

void ocrt_gb_shutdown(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_device < 0) return;
    cudaStreamSynchronize(g_stream);
    for (auto &kv : g_free) cudaFree(kv.second);
    for (auto &kv : g_live) cudaFree(kv.first);
    g_free.clear(); g_live.clear();
    cudaFreeHost(g_pinned); g_pinned = nullptr;
    cudaStreamDestroy(g_stream); g_stream = nullptr;
    g_device = -1;
}

const char *ocrt_gb_last_error(void) { return g_err.c_str(); }

}   // extern "C"

namespace {

int validate_layers(const ocrt_case *cs, const ocrt_opts *op, const ocrt_layers *ly, int ncot)
{
    if ((ly || ncot > 0) && op->pssa)
        return fail(OCRT_ERR_UNSUPPORTED, "IPSS cannot be combined with layer overrides or gradients");
    if (ncot > 0) {
        const bool rough = cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && cs->wind_speed > 0.0;
        if (cs->surface != OCRT_SURFACE_BLACK && !rough)
            return fail(OCRT_ERR_UNSUPPORTED, "gradients need a black or rough (wind > 0) Fresnel surface");
    }
    if (!ly) return OCRT_OK;
    if (ly->n_layers != op->n_layers) return fail(OCRT_ERR_ARGS, "layers.n_layers differs from opts.n_layers");
    for (int l = 0; l < ly->n_layers; ++l) {
        if (ly->dtau && !(std::isfinite(ly->dtau[l]) && ly->dtau[l] > 0.0))
            return fail(OCRT_ERR_ARGS, "layer optical depth not finite and positive");
        if (ly->ssa && !(ly->ssa[l] >= 0.0 && ly->ssa[l] <= 1.0))
            return fail(OCRT_ERR_ARGS, "layer single-scattering albedo outside [0, 1]");
    }
    return OCRT_OK;
}

int validate_lut(const ocrt_lut *L)
{
    if (L->n_vza <= 0 || L->n_raa <= 0 || !L->vza_deg || !L->raa_deg || !L->rho_I || !L->rho_Q || !L->rho_U)
        return fail(OCRT_ERR_ARGS, "bad LUT grid or outputs");
    for (int i = 0; i < L->n_vza; ++i)
        if (!(L->vza_deg[i] >= 0.0 && L->vza_deg[i] < 90.0)) return fail(OCRT_ERR_ARGS, "LUT vza outside [0, 90)");
    for (int i = 0; i < L->n_raa; ++i)
        if (!std::isfinite(L->raa_deg[i])) return fail(OCRT_ERR_ARGS, "LUT raa not finite");
    return OCRT_OK;
}

int plan_create_impl(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp, const ocrt_aerosol *aer, int app,
                     const ocrt_layers *layers, int ncot, const double *cot, ocrt_plan **out,
                     const ocrt_lut *luts = nullptr)
{
    if (!out) return fail(OCRT_ERR_ARGS, "null plan pointer");
    *out = nullptr;
    if (n < 0 || (n > 0 && (!cases || !opts))) return fail(OCRT_ERR_ARGS, "bad batch arguments");
    for (int i = 0; i < n; ++i) {
        int rc = validate(&cases[i], opp ? &opts[i] : &opts[0], aer ? (app ? &aer[i] : &aer[0]) : nullptr);
        if (!rc) rc = validate_layers(&cases[i], opp ? &opts[i] : &opts[0], layers ? &layers[i] : nullptr, ncot);
        if (!rc && luts) rc = validate_lut(&luts[i]);
        if (rc) return rc;
    }
    int rc = ensure_init();
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    ocrt_plan *plan = new ocrt_plan();
    plan->n = n;
    // groups share the Gauss order and the Cox-Munk azimuth grid
    std::map<std::pair<int, int>, int> gid;
    for (int i = 0; i < n; ++i) {
        const ocrt_opts &oi = opp ? opts[i] : opts[0];
        const int N = oi.n_mu;
        const std::pair<int, int> key(N, oi.n_phi_surface > 0 ? oi.n_phi_surface : 1024);
        auto it = gid.find(key);
        if (it == gid.end()) {
            gid[key] = (int)plan->groups.size();
            plan->groups.emplace_back();
            plan->groups.back().N = N;
            it = gid.find(key);
        }
        plan->groups[it->second].idx.push_back(i);
    }
    for (Group &g : plan->groups) {
        rc = build_group(g, cases, opts, opp, aer, app, layers, ncot, cot, luts);
        if (rc) {
            for (Group &h : plan->groups) free_group(h);
            delete plan;
            return rc;
        }
    }
    if (cudaStreamSynchronize(g_stream) != cudaSuccess) {
        for (Group &h : plan->groups) free_group(h);
        delete plan;
        return fail(OCRT_ERR_DEVICE, "upload failed");
    }
    *out = plan;
    return OCRT_OK;
}

} // namespace

extern "C" {

int ocrt_gb_plan_create(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp,
                        const ocrt_aerosol *aer, int app, ocrt_plan **out)
{
    return plan_create_impl(n, cases, opts, opp, aer, app, nullptr, 0, nullptr, out);
}

namespace {

bool graphs_enabled()
{
    const char *e = getenv("OCRT_GB_GRAPH");
    return !(e && strcmp(e, "0") == 0);
}

// Record every group's launch sequence (recorded order counts, no host polls)
// into one graph on `st` and instantiate it.
int capture_plan(ocrt_plan *plan, cudaStream_t st)
{
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return OCRT_ERR_DEVICE;
    }
    plan->launches = 0;
    int rc = OCRT_OK;
    for (Group &g : plan->groups) {
        rc = run_group(plan, g, st, true);
        if (rc) break;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc == OCRT_OK && (e != cudaSuccess || !graph)) rc = OCRT_ERR_DEVICE;
    if (rc == OCRT_OK && cudaGraphInstantiate(&plan->gexec, graph, 0) != cudaSuccess) {
        plan->gexec = nullptr;
        rc = OCRT_ERR_DEVICE;
    }
    if (graph) cudaGraphDestroy(graph);
    if (rc) cudaGetLastError();
    else plan->graph_launches = plan->launches;
    return rc;
}

// Device error flags of a group after an execute: [0] a non-finite field,
// [1] a graph replay whose recorded order counts ended with tasks still
// iterating (later executes of the plan then run eagerly with host polls).
int group_flags(ocrt_plan *plan, Group &g, cudaStream_t st)
{
    int f[2] = {0, 0};
    CK(cudaMemcpyAsync(f, g.err, sizeof(f), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (f[0]) return fail(f[0], "non-finite field during the SOS iteration");
    if (f[1]) {
        if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
        plan->gexec = nullptr;
        plan->graph_off = true;
        return fail(OCRT_ERR_DEVICE, "graph replay ended with tasks still iterating; execute the plan again");
    }
    return OCRT_OK;
}

} // namespace

int ocrt_gb_plan_execute(ocrt_plan *plan, void *stream)
{
    if (!plan) return fail(OCRT_ERR_ARGS, "null plan");
    std::lock_guard<std::mutex> lk(g_mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : g_stream;
    plan->launches = 0;
    for (auto &e : plan->ev) { cudaEventDestroy(e.second.first); cudaEventDestroy(e.second.second); }
    plan->ev.clear();
    for (int c = 0; c < KC_N; ++c) { plan->ms[c] = 0; plan->cnt[c] = 0; }
    plan->work_done = false;
    const bool want_graph = !g_timing && !plan->graph_off && graphs_enabled();
    if (want_graph && plan->gexec) {
        CK(cudaGraphLaunch(plan->gexec, st));
        plan->launches = plan->graph_launches;
        plan->executes++;
        return OCRT_OK;
    }
    if (want_graph && plan->executes >= 1) {
        if (capture_plan(plan, st) == OCRT_OK) {
            CK(cudaGraphLaunch(plan->gexec, st));
            plan->launches = plan->graph_launches;
            plan->executes++;
            return OCRT_OK;
        }
        plan->graph_off = true;    // capture not possible on this stream: stay eager
        plan->launches = 0;
        for (int c = 0; c < KC_N; ++c) plan->cnt[c] = 0;
    }
    for (Group &g : plan->groups) {
        const int rc = run_group(plan, g, st, false);
        if (rc) return rc;
    }
    plan->executes++;
    return OCRT_OK;
}

int ocrt_gb_plan_results(ocrt_plan *plan, ocrt_result *out, void *stream)
{
    if (!plan || (!out && plan->n > 0)) return fail(OCRT_ERR_ARGS, "null plan or output");
    std::lock_guard<std::mutex> lk(g_mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : g_stream;
    double om = 0;
    for (Group &g : plan->groups) {
        std::vector<ocrt_result> r(g.P);
        CK(cudaMemcpyAsync(r.data(), g.res, sizeof(ocrt_result) * g.P, cudaMemcpyDeviceToHost, st));
        const int rc = group_flags(plan, g, st);
        if (rc) return rc;
        for (int q = 0; q < g.P; ++q) { out[g.idx[q]] = r[q]; om += r[q].order_modes; }
    }
    plan->order_modes = om;
    return OCRT_OK;
}

void ocrt_gb_set_timing(int enable) { g_timing = enable ? 1 : 0; }

int ocrt_gb_plan_kernel_stats(ocrt_plan *plan, int cls, const char **name, double *ms, long long *launches,
                              double *alg_flops, double *alg_bytes)
{
    if (!plan) return fail(OCRT_ERR_ARGS, "null plan");
    if (cls == -1) return KC_N;
    if (cls < 0 || cls >= KC_N) return fail(OCRT_ERR_ARGS, "kernel class out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!plan->ev.empty()) {
        CK(cudaStreamSynchronize(g_stream));
        for (auto &e : plan->ev) {
            float t = 0.f;
            if (cudaEventSynchronize(e.second.second) == cudaSuccess &&
                cudaEventElapsedTime(&t, e.second.first, e.second.second) == cudaSuccess)
                plan->ms[e.first] += t;
            cudaEventDestroy(e.second.first);
            cudaEventDestroy(e.second.second);
        }
        plan->ev.clear();
    }
    if (!plan->work_done) {
        // algorithmic work from the orders each task actually executed
        for (int c = 0; c < KC_N; ++c) { plan->flops[c] = 0; plan->bytes[c] = 0; }
        for (Group &g : plan->groups) {
            std::vector<TaskState> st(g.T);
            CK(cudaMemcpy(st.data(), g.state, sizeof(TaskState) * g.T, cudaMemcpyDeviceToHost));
            const double N = g.N, NR = g.G.NR;
            for (int t = 0; t < g.T; ++t) {
                const TaskDev &tk = g.htask[t];
                const PixDev &d = g.hpx[tk.pix];
                const double K = tk.K, nt = d.nt, ords = std::max(0, st[t].orders - 1);
                const int sc = g.use_tc ? KC_SOURCE_TC : KC_SOURCE;
                plan->flops[sc] += ords * 72.0 * N * N * K;
                plan->bytes[sc] += ords * (K * 6 * N + K * 6 * NR + 36.0 * N * NR) * 4.0;
                if (tk.has_mol && g.use_tc) {          // dense U V inside the tensor-core pass
                    plan->flops[KC_SOURCE_TC] += ords * 72.0 * N * N * K;
                    plan->bytes[KC_SOURCE_TC] += ords * (36.0 * N * NR) * 4.0;
                } else if (tk.has_mol) {               // rank-24 form on CUDA cores
                    plan->flops[KC_MOL] += ords * 2.0 * K * 24.0 * (N + 6 * NR);
                    plan->bytes[KC_MOL] += ords * (K * 6 * N + 2.0 * K * 6 * NR) * 4.0;
                }
                plan->bytes[KC_SCAN] += ords * (2.0 * 6 * N * K + N * nt) * 4.0;
                plan->flops[KC_SCAN] += ords * 6.0 * N * nt * 5.0;
                plan->bytes[KC_PRIMARY] += K * 6 * NR * 12.0;
                const double Lm = d.L - tk.m + 1;
                plan->flops[KC_TABLES] += 2.0 * 26.0 * NR * N * Lm;
                plan->bytes[KC_TABLES] += 36.0 * N * NR * 4.0 * (tk.has_mol ? 2 : 1);
            }
            for (const PixDev &d : g.hpx) {
                if (!(d.surface == 2 && d.wind > 0.0)) continue;
                // pairs evaluated: Gauss-Gauss once per reciprocal couple, the
                // view row and the sun column in full; all N^2 + N written
                const double pairs = N * (N + 1) / 2 + (NR - N) * (N + 1) + N;
                plan->flops[KC_COXMUNK] += 18.0 * pairs * d.nphi * (d.M + 1);
                plan->bytes[KC_COXMUNK] += (N * N + N) * 9.0 * (d.M + 1) * 4.0;
            }
        }
        plan->work_done = true;
    }
    if (name) *name = kc_names[cls];
    if (ms) *ms = plan->ms[cls];
    if (launches) *launches = plan->cnt[cls];
    if (alg_flops) *alg_flops = plan->flops[cls];
    if (alg_bytes) *alg_bytes = plan->bytes[cls];
    return OCRT_OK;
}

int ocrt_gb_plan_stats(const ocrt_plan *plan, double *order_modes_total, long long *kernel_launches)
{
    if (!plan) return fail(OCRT_ERR_ARGS, "null plan");
    if (order_modes_total) *order_modes_total = plan->order_modes;
    if (kernel_launches) *kernel_launches = plan->launches;
    return OCRT_OK;
}

int ocrt_gb_plan_graph_ready(const ocrt_plan *plan) { return plan && plan->gexec ? 1 : 0; }

int ocrt_gb_autotune_summary(char *buf, int len)
{
    std::lock_guard<std::mutex> lk(g_mu);
    std::string t;
    for (const TuneRec &r : g_tune) {
        t += r.kernel;
        t += " key=";
        for (size_t i = 0; i < r.key.size(); ++i) t += (i ? "," : "") + std::to_string(r.key[i]);
        t += " best=" + (r.labels ? std::string(r.labels[r.best]) : std::to_string(r.best)) + " ms:";
        for (const auto &m : r.ms) {
            char b[64];
            if (r.labels) snprintf(b, sizeof(b), " %s=%.6g", r.labels[m.first], m.second);
            else snprintf(b, sizeof(b), " %d=%.4f", m.first, m.second);
            t += b;
        }
        t += "\n";
    }
    if (buf && len > 0) {
        const size_t n = std::min(t.size(), (size_t)len - 1);
        memcpy(buf, t.data(), n);
        buf[n] = 0;
    }
    return (int)t.size();
}

void ocrt_gb_plan_destroy(ocrt_plan *plan)
{
    if (!plan) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_stream) cudaStreamSynchronize(g_stream);
    for (Group &g : plan->groups) free_group(g);
    for (auto &e : plan->ev) { cudaEventDestroy(e.second.first); cudaEventDestroy(e.second.second); }
    if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
    delete plan;
}

int ocrt_gb_solve_batch(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp,
                        const ocrt_aerosol *aer, int app, ocrt_result *out, void *stream)
{
    if (n == 0) return OCRT_OK;
    if (!out) return fail(OCRT_ERR_ARGS, "null output");
    ocrt_plan *plan = nullptr;
    int rc = ocrt_gb_plan_create(n, cases, opts, opp, aer, app, &plan);
    if (rc) return rc;
    rc = ocrt_gb_plan_execute(plan, stream);
    if (!rc) rc = ocrt_gb_plan_results(plan, out, stream);
    ocrt_gb_plan_destroy(plan);
    return rc;
}

int ocrt_gb_plan_create_adjoint(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp,
                                const ocrt_aerosol *aer, int app, const ocrt_layers *layers, int n_cot,
                                const double *cot, ocrt_plan **out)
{
    if (!out) return fail(OCRT_ERR_ARGS, "null plan pointer");
    *out = nullptr;
    if (n_cot < 0 || n_cot > 3) return fail(OCRT_ERR_ARGS, "n_cot outside [0, 3]");
    if (n_cot > 0 && !cot) return fail(OCRT_ERR_ARGS, "null cotangent array");
    const int rc = plan_create_impl(n, cases, opts, opp, aer, app, layers, n_cot, cot, out);
    if (!rc) (*out)->ncot = n_cot;
    return rc;
}

int ocrt_gb_plan_gradients(ocrt_plan *plan, ocrt_grad *grad, void *stream)
{
    if (!plan) return fail(OCRT_ERR_ARGS, "null plan");
    if (plan->ncot == 0) return fail(OCRT_ERR_ARGS, "plan has no cotangent rows");
    if (!grad) return fail(OCRT_ERR_ARGS, "null gradient array");
    const int n_cot = plan->ncot;
    for (int i = 0; i < plan->n * n_cot; ++i)
        if (!grad[i].d_dtau || !grad[i].d_ssa) return fail(OCRT_ERR_ARGS, "null gradient array");
    std::lock_guard<std::mutex> lk(g_mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : g_stream;
    for (Group &g : plan->groups) {
        std::vector<double> h((size_t)g.P * n_cot * g.grad_stride);
        CK(cudaMemcpyAsync(h.data(), g.grad, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        const int rc = group_flags(plan, g, st);
        if (rc) return rc;
        for (int q = 0; q < g.P; ++q) {
            const int i = g.idx[q], nt = g.hpx[q].nt;
            for (int r = 0; r < n_cot; ++r) {
                const double *src = h.data() + ((size_t)q * n_cot + r) * g.grad_stride;
                ocrt_grad &gr = grad[(size_t)i * n_cot + r];
                for (int l = 0; l < nt; ++l) { gr.d_dtau[l] = src[l]; gr.d_ssa[l] = src[nt + l]; }
                gr.d_wind = src[2 * nt];
            }
        }
    }
    return OCRT_OK;
}

int ocrt_gb_solve_batch_adjoint(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp,
                                const ocrt_aerosol *aer, int app, const ocrt_layers *layers, int n_cot,
                                const double *cot, ocrt_result *out, ocrt_grad *grad, void *stream)
{
    if (n == 0) return OCRT_OK;
    if (!out) return fail(OCRT_ERR_ARGS, "null output");
    if (n_cot > 0 && !grad) return fail(OCRT_ERR_ARGS, "null gradient array");
    ocrt_plan *plan = nullptr;
    int rc = ocrt_gb_plan_create_adjoint(n, cases, opts, opp, aer, app, layers, n_cot, cot, &plan);
    if (rc) return rc;
    rc = ocrt_gb_plan_execute(plan, stream);
    if (!rc) rc = ocrt_gb_plan_results(plan, out, stream);
    if (!rc && n_cot > 0) rc = ocrt_gb_plan_gradients(plan, grad, stream);
    ocrt_gb_plan_destroy(plan);
    return rc;
}

int ocrt_gb_solve_batch_lut(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp,
                            const ocrt_aerosol *aer, int app, ocrt_lut *luts, ocrt_result *out, void *stream)
{
    if (n == 0) return OCRT_OK;
    if (!out || !luts) return fail(OCRT_ERR_ARGS, "null output or LUT array");
    ocrt_plan *plan = nullptr;
    int rc = plan_create_impl(n, cases, opts, opp, aer, app, nullptr, 0, nullptr, &plan, luts);
    if (rc) return rc;
    rc = ocrt_gb_plan_execute(plan, stream);
    if (!rc) rc = ocrt_gb_plan_results(plan, out, stream);
    if (!rc) {
        std::lock_guard<std::mutex> lk(g_mu);
        cudaStream_t st = stream ? (cudaStream_t)stream : g_stream;
        for (Group &g : plan->groups) {
            std::vector<double> h(6 * (size_t)g.lut_ntot);
            if (cudaMemcpyAsync(h.data(), g.lut_out, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
                rc = fail(OCRT_ERR_DEVICE, "LUT copy failed");
                break;
            }
            for (int q = 0; q < g.P; ++q) {
                const int i = g.idx[q];
                const PixDev &d = g.hpx[q];
                ocrt_lut &L = luts[i];
                double *dst[6] = {L.rho_I, L.rho_Q, L.rho_U, L.T_diff_dn_dir, L.T_sg_up_dir, L.T_total_up_dir};
                const size_t np = (size_t)d.lut_nv * d.lut_nr;
                for (int f = 0; f < 6; ++f)
                    if (dst[f]) memcpy(dst[f], h.data() + (size_t)f * g.lut_ntot + d.lut_oo, sizeof(double) * np);
                L.T_dir_dn = out[i].T_dir_dn;
                L.T_diff_dn_hemi = out[i].T_diff_dn_hemi;
            }
        }
    }
    ocrt_gb_plan_destroy(plan);
    return rc;
}

int ocrt_gb_solve_case_lut(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer, ocrt_result *out,
                           ocrt_lut *lut)
{
    if (!cs || !out || !lut) return fail(OCRT_ERR_ARGS, "null case, output or LUT");
    ocrt_opts def;
    if (!opts) { ocrt_opts_default(&def); opts = &def; }
    return ocrt_gb_solve_batch_lut(1, cs, opts, 0, aer, 0, lut, out, nullptr);
}

int ocrt_gb_solve_case(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                       ocrt_result *out, ocrt_diag *diag)
{
    if (!cs || !out) return fail(OCRT_ERR_ARGS, "null case or output");
    ocrt_opts def;
    if (!opts) { ocrt_opts_default(&def); opts = &def; }
    ocrt_plan *plan = nullptr;
    int rc = ocrt_gb_plan_create(1, cs, opts, 0, aer, 0, &plan);
    if (rc) return rc;
    rc = ocrt_gb_plan_execute(plan, nullptr);
    if (!rc) rc = ocrt_gb_plan_results(plan, out, nullptr);
    if (!rc && diag) {
        std::lock_guard<std::mutex> lk(g_mu);
        Group &g = plan->groups[0];
        std::vector<TaskState> st(g.T);
        std::vector<TaskOut> to(g.T);
        if (cudaMemcpy(st.data(), g.state, sizeof(TaskState) * g.T, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(to.data(), g.tout, sizeof(TaskOut) * g.T, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = fail(OCRT_ERR_DEVICE, "diagnostic copy failed");
        else
            for (int m = 0; m < g.T; ++m) {
                if (diag->orders_per_m) diag->orders_per_m[m] = st[m].orders;
                if (diag->residual_per_m) diag->residual_per_m[m] = st[m].resid;
                if (diag->view_I_m) diag->view_I_m[m] = to[m].vI;
                if (diag->view_Q_m) diag->view_Q_m[m] = to[m].vQ;
                if (diag->view_U_m) diag->view_U_m[m] = to[m].vU;
            }
    }
    ocrt_gb_plan_destroy(plan);
    return rc;
}

} // extern "C"

namespace {

// Level grid of one case as the solve builds it, copied back: optical depths,
// summed scattering fractions, altitudes and gas absorption depths.
int level_profile(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer, std::vector<double> &h,
                  std::vector<double> &w, std::vector<double> &zk, std::vector<double> &ta)
{
    if (!cs || !opts) return fail(OCRT_ERR_ARGS, "null case or options");
    ocrt_plan *plan = nullptr;
    int rc = ocrt_gb_plan_create(1, cs, opts, 0, aer, 0, &plan);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        Group &g = plan->groups[0];
        cudaStream_t st = g_stream;
        const int nt = g.hpx[0].nt;
        std::vector<double> x(nt + 1), y(nt + 1);
        h.assign(nt + 1, 0.0); zk.assign(nt + 1, 0.0); ta.assign(nt + 1, 0.0); w.assign(nt, 0.0);
        k_gauss<<<1, 64, 0, st>>>(g.N, g.gmu, g.gw, g.pw);
        k_pixel_setup<<<1, 128, 0, st>>>(g.px, 1, g.N, g.gmu);
        k_levels<<<dim3(2, 1), 256, 0, st>>>(g.px, 1, g.h, g.ch, g.xd, g.yd, g.z);
        k_level_mix<<<dim3(2, 1), 256, 0, st>>>(g.px, 1, g.z, g.xd, g.yd);
        if (g.any_gas) k_gas_apply<<<1, 256, 0, st>>>(g.px, 1, g.h, g.ch, g.xd, g.yd, g.z, g.tabs);
        const size_t lb = sizeof(double) * (nt + 1);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(h.data(), g.h, lb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(x.data(), g.xd, lb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(y.data(), g.yd, lb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(zk.data(), g.z, lb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            (g.any_gas && cudaMemcpyAsync(ta.data(), g.tabs, lb, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = fail(OCRT_ERR_DEVICE, "level setup failed");
        } else {
            for (int l = 0; l < nt; ++l) w[l] = x[l + 1] + y[l + 1];
        }
    }
    ocrt_gb_plan_destroy(plan);
    return rc;
}

}  // namespace

extern "C" {

int ocrt_gb_layer_defaults(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                           double *dtau, double *ssa)
{
    std::vector<double> h, w, zk, ta;
    const int rc = level_profile(cs, opts, aer, h, w, zk, ta);
    if (rc) return rc;
    for (size_t l = 0; l < w.size(); ++l) {
        if (dtau) dtau[l] = h[l + 1] - h[l];
        if (ssa) ssa[l] = w[l];
    }
    return OCRT_OK;
}

int ocrt_gb_layer_gas(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer, double *tau_abs,
                      double *z_km)
{
    std::vector<double> h, w, zk, ta;
    const int rc = level_profile(cs, opts, aer, h, w, zk, ta);
    if (rc) return rc;
    for (size_t l = 0; l < w.size(); ++l)
        if (tau_abs) tau_abs[l] = ta[l];
    for (size_t k = 0; k < zk.size(); ++k)
        if (z_km) z_km[k] = zk[k];
    return OCRT_OK;
}

} // extern "C"

// Internal helpers for other translation units of this library (C++ linkage,
// not part of the C ABI).
int ocrt_internal_validate(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer)
{
    return validate(cs, op, aer);
}

int ocrt_internal_fail(int rc, const char *msg)
{
    return fail(rc, msg);
}

// ===================================================================
// Coupled atmosphere-ocean solve (rt_solve_case_ocean, rt_solver.c:3468-6660)
// ===================================================================
namespace {

double snell_down(double mu_air, double n)
{
    const double s2 = std::max(0.0, 1.0 - mu_air * mu_air) / (n * n);
    return s2 >= 1.0 ? 0.0 : std::sqrt(1.0 - s2);
}

// Water column of one pixel on the host: optical budget, depth policy and
// layer count (rt_water_rt.c:4405-4440, 5119-5180).
struct WaterCol {
    double ext, om_w, om_p, tau, depth;
    int nt, m_loop;
};

int water_column(const ocrt_ocean &oc, WaterCol &wc)
{
    const double bp = oc.b_particle > 0.0 ? oc.b_particle : 0.0;
    const double b_rt = oc.b_water + bp;
    wc.ext = oc.a_total + b_rt;
    if (!(wc.ext > 0.0)) return fail(OCRT_ERR_ARGS, "water column has no extinction");
    wc.om_w = oc.b_water / wc.ext;
    wc.om_p = bp / wc.ext;
    if (oc.depth_m > 0.0) {
        wc.tau = wc.ext * oc.depth_m;
    } else {
        double gp = 0.0;
        if (bp > 0.0 && oc.L_particle >= 1) gp = std::min(0.999, std::max(-0.999, oc.beta[1] / 3.0));
        const double sb = bp + oc.b_water;
        const double ge = std::min(0.999, std::max(-0.999, sb > 0.0 ? bp * gp / sb : 0.0));
        double z_req = (oc.tau_base > 0.0 ? oc.tau_base : 20.0) / wc.ext;
        const double te = oc.a_total + b_rt * std::max(0.0, 1.0 - ge);
        if (te > 0.0) z_req = std::max(z_req, -std::log(1.0e-8) / te);
        wc.tau = wc.ext * z_req;
    }
    wc.depth = wc.tau / wc.ext;
    int nt = (int)std::ceil(wc.tau / 0.05);
    if (oc.n_layers_water > 0 && (oc.depth_m > 0.0 || oc.n_layers_water > nt)) nt = oc.n_layers_water;
    wc.nt = std::max(nt, 1);
    const int Lws = std::max(bp > 0.0 ? oc.L_particle : 0, 2);
    wc.m_loop = std::min(oc.m_max_water, Lws);
    return OCRT_OK;
}

int validate_ocean(const ocrt_case &c, const ocrt_opts &o, const ocrt_ocean &oc)
{
    if (c.surface != OCRT_SURFACE_OCEAN) return fail(OCRT_ERR_ARGS, "coupled solve needs surface OCRT_SURFACE_OCEAN");
    if (!(c.wind_speed > 0.0)) return fail(OCRT_ERR_UNSUPPORTED, "coupled solve: flat interface (wind <= 0) not supported");
    if (o.pssa) return fail(OCRT_ERR_UNSUPPORTED, "coupled solve: IPSS is not applied on this path");
    if (!(oc.a_total >= 0.0) || !(oc.b_water >= 0.0) || !(oc.b_particle >= 0.0))
        return fail(OCRT_ERR_ARGS, "water absorption / scattering must be >= 0");
    if (oc.n_mu_water < 2 || oc.n_mu_water > OCRT_MAX_N) return fail(OCRT_ERR_ARGS, "n_mu_water outside [2, 64]");
    if (oc.m_max_water < 0 || oc.m_max_water > OCRT_MAX_M) return fail(OCRT_ERR_ARGS, "m_max_water outside [0, 255]");
    if (oc.max_orders_water < 1 || !(oc.tolerance_water > 0.0)) return fail(OCRT_ERR_ARGS, "bad water SOS control");
    if (oc.n_layers_water < 0 || oc.n_layers_water > 4096) return fail(OCRT_ERR_ARGS, "n_layers_water outside [0, 4096]");
    if (!oc.view_as_node) return fail(OCRT_ERR_UNSUPPORTED, "coupled solve: the water view is extracted at its node");
    if (oc.b_particle > 0.0) {
        if (oc.L_particle < 1 || oc.L_particle > 1024 || !oc.beta || !oc.gamma || !oc.alpha || !oc.zeta)
            return fail(OCRT_ERR_ARGS, "hydrosol expansion missing");
        for (int l = 0; l <= oc.L_particle; ++l)
            if (!std::isfinite(oc.beta[l]) || !std::isfinite(oc.gamma[l]) || !std::isfinite(oc.alpha[l]) ||
                !std::isfinite(oc.zeta[l])) return fail(OCRT_ERR_NONFINITE, "non-finite hydrosol moment");
    }
    return OCRT_OK;
}

int ocean_solve(int n, const ocrt_case *cases, const ocrt_opts *opts, int opp, const ocrt_aerosol *aer, int app,
                const ocrt_ocean *ocs, int ocp, ocrt_result *out, ocrt_ocean_result *wout, cudaStream_t st)
{
    if (n <= 0) return OCRT_OK;
    const int Nw = ocs[0].n_mu_water;
    std::vector<ocrt_case> ca(n);
    std::vector<ocrt_opts> oa(n), ow(n);
    std::vector<ocrt_aerosol> hyd(n);
    std::vector<WaterCol> wc(n);
    int nphi = -1;
    for (int i = 0; i < n; ++i) {
        const ocrt_opts &o = opp ? opts[i] : opts[0];
        const ocrt_ocean &oc = ocp ? ocs[i] : ocs[0];
        int rc = validate_ocean(cases[i], o, oc);
        if (rc) return rc;
        if (oc.n_mu_water != Nw) return fail(OCRT_ERR_ARGS, "coupled batch: n_mu_water must be common to the batch");
        if (aer && (app ? aer[i] : aer[0]).use_value_kernel)
            return fail(OCRT_ERR_UNSUPPORTED, "coupled solve: the aerosol value kernel is not on the GB300 path");
        const int np = o.n_phi_surface > 0 ? o.n_phi_surface : 1024;
        if (nphi >= 0 && np != nphi) return fail(OCRT_ERR_ARGS, "coupled batch: n_phi_surface must be common");
        nphi = np;
        ca[i] = cases[i];
        ca[i].surface = OCRT_SURFACE_BLACK_FRESNEL_OCEAN;
        if (!(ca[i].n_water > 0.0)) ca[i].n_water = 1.34;
        oa[i] = o;
        oa[i].n_mu = Nw;                        // shared node set (rt_solver.c:4006-4010)
        rc = validate(&ca[i], &oa[i], aer ? (app ? &aer[i] : &aer[0]) : nullptr);
        if (rc) return rc;
        if ((rc = water_column(oc, wc[i]))) return rc;
        ow[i] = oa[i];
        ow[i].n_layers = wc[i].nt;
        ow[i].fourier_m_max = wc[i].m_loop;
        ow[i].max_orders = oc.max_orders_water;
        ow[i].tolerance = oc.tolerance_water;
        ow[i].gas = nullptr;
        ow[i].pssa = 0;
        memset(&hyd[i], 0, sizeof(ocrt_aerosol));
        if (oc.b_particle > 0.0) {
            hyd[i].tau_a = 1.0; hyd[i].ssa_a = 1.0; hyd[i].L_max = oc.L_particle;
            hyd[i].beta = oc.beta; hyd[i].gamma = oc.gamma; hyd[i].alpha = oc.alpha; hyd[i].zeta = oc.zeta;
        }
    }
    int rc = ensure_init();
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    ocrt_plan plan;
    plan.n = n;
    // host side of each pixel
    std::vector<OceanPix> hop(n);
    int Ma = 0;
    for (int i = 0; i < n; ++i) Ma = std::max(Ma, oa[i].fourier_m_max);
    for (int i = 0; i < n; ++i) {
        const ocrt_case &c = cases[i];
        const ocrt_opts &o = oa[i];
        const ocrt_ocean &oc = ocp ? ocs[i] : ocs[0];
        const ocrt_aerosol *a = aer ? (app ? &aer[i] : &aer[0]) : nullptr;
        OceanPix &p = hop[i];
        memset(&p, 0, sizeof(p));
        p.mu_sa = std::cos(c.sza_deg * OCRT_PI / 180.0);
        p.mu_va = std::cos(c.vza_deg * OCRT_PI / 180.0);
        p.nw = ca[i].n_water;
        p.mu_sw = snell_down(p.mu_sa, p.nw);
        p.mu_vw = snell_down(p.mu_va, p.nw);
        p.raa_deg = c.raa_deg; p.wind = c.wind_speed; p.st = c.sigma_type; p.qc = c.q_convention;
        double tau_r = 0.0;
        if (c.pressure_hpa > 0.0)
            tau_r = o.tau_r_source == OCRT_TAU_R_FROM_INPUT ? c.tau_r_input : bodhaine_tau(c.wavelength_nm, c.pressure_hpa);
        p.tau_atm = tau_r + ((a && a->tau_a > 0.0) ? a->tau_a : 0.0);
        if (o.gas) {
            double tg = 0.0;
            if ((rc = ocrt_gb_gas_tau(o.gas, c.wavelength_nm, nullptr, &tg))) return rc;
            p.tau_atm += tg;
        }
        p.ext_w = wc[i].ext;
        p.M = o.fourier_m_max;
        p.m_loop = wc[i].m_loop;
        p.pa = i; p.pw = i;
        p.top_off = (long long)i * (Ma + 1) * Nw * 3;
        p.ext_off = (long long)i * (Ma + 1) * (Nw + 1) * 3;
        // distinct water directions: Gauss + refracted view, nadir, refracted sun, air sun
        std::vector<double> dirs;
        {
            std::vector<double> gm(Nw), gww(Nw);
            // Gauss nodes as the device builds them (only their coincidence matters here)
            for (int k = 1; k <= Nw; ++k) {
                double t = std::cos(OCRT_PI * ((double)k - 0.25) / (2.0 * Nw + 0.5));
                gm[k - 1] = t;
            }
            dirs = gm;
            for (double x : {p.mu_vw, 1.0, p.mu_sw, p.mu_sa}) {
                bool dup = false;
                for (double y : dirs) if (std::fabs(x - y) < 1e-12) dup = true;
                if (!dup) dirs.push_back(x);
            }
        }
        p.n_ring_unique = (int)dirs.size();
        (void)oc;
    }
    // ---- pass 1: atmosphere over the rough surface, bottom field exported ----
    plan.groups.resize(3);
    Group &GA = plan.groups[0], &GW = plan.groups[1], &GC = plan.groups[2];
    // the interface coupling reads the totals at level 1 (k_edges)
    GA.keep_tot = GW.keep_tot = GC.keep_tot = true;
    for (int i = 0; i < n; ++i) { GA.idx.push_back(i); GW.idx.push_back(i); GC.idx.push_back(i); }
    GA.N = GW.N = GC.N = Nw;
    GA.E = GC.E = 1;
    GW.E = OCRT_MAX_EXTRA;
    int Mw = 0;
    for (int i = 0; i < n; ++i) Mw = std::max(Mw, wc[i].m_loop);
    GW.nphi_ww = std::max(176, 2 * Mw + 16);
    const Geom GeA = make_geom(Nw, 1), GeW = make_geom(Nw, OCRT_MAX_EXTRA);
    double *d_top = nullptr, *d_ext3 = nullptr, *d_td = nullptr, *d_view = nullptr, *d_glo = nullptr;
    OceanPix *d_op = nullptr;
    ocrt_result *d_out = nullptr;
    ocrt_ocean_result *d_wout = nullptr;
    auto cleanup = [&]() {
        for (Group &g : plan.groups) { dfree(g.edge); free_group(g); }
        dfree(d_top); dfree(d_ext3); dfree(d_td); dfree(d_view); dfree(d_glo); dfree(d_op); dfree(d_out); dfree(d_wout);
    };
    auto atm_patch = [&](int bottom) {
        return [&, bottom](int q, PixDev &d) {
            if (bottom) {
                d.bottom_only = 1;
                d.ext_off = hop[q].ext_off;
                d.ext_mmax = std::min(hop[q].M, wc[q].m_loop);
            }
        };
    };
    if ((rc = build_group(GA, ca.data(), oa.data(), 1, aer, app, nullptr, 0, nullptr, nullptr, atm_patch(0)))) {
        cleanup();
        return rc;
    }
    rc = alloc(GA.edge, (size_t)GA.T * GeA.NR * OCRT_EDGE);
    if (!rc) rc = run_group(&plan, GA, st, false);
    if (rc) { cleanup(); return rc; }
    // ---- skylight into the water ----
    if ((rc = up(d_op, hop)) || (rc = alloc(d_td, (size_t)n * (GeA.NR + 1))) ||
        (rc = alloc(d_top, (size_t)n * (Ma + 1) * Nw * 3))) { cleanup(); return rc; }
    LAUNCH(&plan, KC_COXMUNK, k_taw_direct<<<dim3(Nw + 1, n), 128, 0, st>>>(d_op, n, GA.px, GA.gmu, Nw, GeA.NR, d_td));
    LAUNCH(&plan, KC_COXMUNK, k_ocean_prep<<<(n + 127) / 128, 128, 0, st>>>(d_op, n, GA.pix_task0, GA.gmu, GA.gw, Nw,
                                                                             GeA.NR, GA.edge, d_td));
    {
        const size_t smem = iface_smem_bytes(Ma, 128, 3 * (Ma + 1));
        CK(cudaFuncSetAttribute(k_couple_aw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(smem + 1024, 227 * 1024)));
        LAUNCH(&plan, KC_COXMUNK, k_couple_aw<<<dim3(Nw, n), 128, smem, st>>>(d_op, n, GA.pix_task0, GA.gmu, GA.gw, Nw,
                                                                               GeA.NR, GA.edge, d_top));
    }
    // ---- pass 2: the water column ----
    std::vector<ocrt_case> cw(n);
    for (int i = 0; i < n; ++i) {
        cw[i] = ca[i];
        cw[i].surface = OCRT_SURFACE_BLACK;
        cw[i].pressure_hpa = 0.0;
    }
    auto water_patch = [&](int q, PixDev &d) {
        const OceanPix &p = hop[q];
        const ocrt_ocean &oc = ocp ? ocs[q] : ocs[0];
        d.medium = 1;
        d.mu0 = p.mu_sw; d.mu_view = p.mu_vw;
        d.xmu[0] = p.mu_vw; d.xmu[1] = 1.0; d.xmu[2] = p.mu_sw; d.xmu[3] = p.mu_sa;
        d.n_ring = Nw + OCRT_MAX_EXTRA;
        d.view_slot = Nw;
        d.tau_total = wc[q].tau;
        d.w_tau = wc[q].tau; d.w_omega_w = wc[q].om_w; d.w_omega_p = wc[q].om_p;
        d.depol = OCRT_DEPOL_WATER;
        // flat Fresnel transmission of the sun's beam: q = T[1,0] / T[0,0] (rt_water_rt.c:5627-5641)
        {
            const double n1 = 1.0, n2 = p.nw, mi = p.mu_sa;
            const double st2 = (n1 / n2) * (n1 / n2) * std::max(0.0, 1.0 - mi * mi);
            double bq = 0.0;
            if (st2 < 1.0) {
                const double mt = std::sqrt(1.0 - st2);
                const double rs = (n1 * mi - n2 * mt) / (n1 * mi + n2 * mt), rp = (n2 * mi - n1 * mt) / (n2 * mi + n1 * mt);
                const double ts = 1.0 + rs, tp = (n1 / n2) * (1.0 + rp);
                const double Ts = ts * ts, Tp = tp * tp;
                const double qk = p.qc == 1 ? 0.5 * (Tp - Ts) : 0.5 * (Ts - Tp);
                bq = qk / (0.5 * (Ts + Tp));
            }
            d.beam_q = bq;
        }
        d.ext_off = p.top_off;
        d.ext_mmax = p.M;
        d.surface = OCRT_SURFACE_BLACK;
        d.wind = p.wind; d.n_water = p.nw; d.sigma_type = p.st; d.q_conv = p.qc;
        d.mom_off = oc.b_particle > 0.0 ? d.mom_off : -1;
        if (oc.b_particle <= 0.0) { d.L_aer = -1; d.tau_a = 0.0; }
    };
    if ((rc = build_group(GW, cw.data(), ow.data(), 1, hyd.data(), 1, nullptr, 0, nullptr, nullptr, water_patch))) {
        cleanup();
        return rc;
    }
    GW.ext = d_top;
    rc = alloc(GW.edge, (size_t)GW.T * GeW.NR * OCRT_EDGE);
    if (!rc) {
        CK(cudaFuncSetAttribute(k_rww, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)std::min<size_t>(iface_smem_bytes(GW.Mmax, GW.nphi_ww, 0) + 1024, 227 * 1024)));
        rc = run_group(&plan, GW, st, false);
    }
    if (rc) { cleanup(); return rc; }
    // ---- water-leaving radiance on the atmosphere ring and at the view ----
    {
        std::vector<double> hg(192);
        std::vector<double> xg(96), wg(96);
        // Gauss-Legendre 96 on (0, 1), as the reference's quadrature (rt_quadrature.c:20-61)
        for (int k = 1; k <= 96; ++k) {
            double t = std::cos(OCRT_PI * ((double)k - 0.25) / (192.0 + 0.5)), pn = 0, pm = 0, dp = 1;
            for (int it = 0; it < 100; ++it) {
                double a = 1.0, b = t;
                for (int q = 1; q < 192; ++q) { const double cc = ((2.0 * q + 1.0) * t * b - (double)q * a) / (double)(q + 1); a = b; b = cc; }
                pn = b; pm = a;
                dp = 192.0 * (t * pn - pm) / (t * t - 1.0);
                const double step = -pn / dp;
                t += step;
                if (std::fabs(step) < 1.0e-15 * (std::fabs(t) + 1.0)) break;
            }
            double a = 1.0, b = t;
            for (int q = 1; q < 192; ++q) { const double cc = ((2.0 * q + 1.0) * t * b - (double)q * a) / (double)(q + 1); a = b; b = cc; }
            dp = 192.0 * (t * b - a) / (t * t - 1.0);
            xg[96 - k] = t;
            wg[96 - k] = 2.0 / ((1.0 - t * t) * dp * dp);
        }
        for (int k = 0; k < 96; ++k) { hg[k] = xg[k]; hg[96 + k] = wg[k]; }
        if ((rc = up(d_glo, hg)) || (rc = alloc(d_ext3, (size_t)n * (Ma + 1) * GeA.NR * 3)) ||
            (rc = alloc(d_view, (size_t)n * 3 * (OCRT_MAX_M + 1)))) { cleanup(); return rc; }
        CK(cudaMemsetAsync(d_ext3, 0, sizeof(double) * (size_t)n * (Ma + 1) * GeA.NR * 3, st));
        CK(cudaMemsetAsync(d_view, 0, sizeof(double) * (size_t)n * 3 * (OCRT_MAX_M + 1), st));
        LAUNCH(&plan, KC_COXMUNK, k_water_modes<<<(n + 127) / 128, 128, 0, st>>>(d_op, n, GW.px, GW.pix_task0, GeW.NR,
                                                                                 GW.edge));
        const int Mc = std::max(Ma, Mw);
        const size_t extra = 3 * (size_t)(Mc + 1) + GeW.NR + (GeW.NR + 1) / 2 + 1;
        const size_t smem = iface_smem_bytes(Mc, 128, (int)extra);
        CK(cudaFuncSetAttribute(k_couple_wa, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(smem + 1024, 227 * 1024)));
        LAUNCH(&plan, KC_COXMUNK, k_couple_wa<<<dim3(GeA.NR + 1, n), 128, smem, st>>>(
                   d_op, n, GA.px, GW.px, GW.pix_task0, GA.gmu, Nw, GeA.NR, GeW.NR, GW.edge, d_glo, d_ext3, d_view));
    }
    // ---- pass 3: the atmosphere driven by the water-leaving radiance ----
    if ((rc = build_group(GC, ca.data(), oa.data(), 1, aer, app, nullptr, 0, nullptr, nullptr, atm_patch(1)))) {
        cleanup();
        return rc;
    }
    GC.ext = d_ext3;
    if ((rc = run_group(&plan, GC, st, false))) { cleanup(); return rc; }
    // ---- outputs ----
    if ((rc = alloc(d_out, n)) || (rc = alloc(d_wout, n))) { cleanup(); return rc; }
    LAUNCH(&plan, KC_FINAL, k_ocean_final<<<(n + 127) / 128, 128, 0, st>>>(
               d_op, n, GA.px, GW.px, GW.pix_task0, GA.gmu, GA.gw, Nw, GeW.NR, GW.edge, d_view, d_top, GA.res, GW.res,
               GC.res, d_out, d_wout));
    std::vector<ocrt_result> ho(n);
    std::vector<ocrt_ocean_result> hw(n);
    CK(cudaMemcpyAsync(ho.data(), d_out, sizeof(ocrt_result) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hw.data(), d_wout, sizeof(ocrt_ocean_result) * n, cudaMemcpyDeviceToHost, st));
    for (Group &g : plan.groups) {
        if ((rc = group_flags(&plan, g, st))) { cleanup(); return rc; }
    }
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i) {
        if (out) out[i] = ho[i];
        if (wout) wout[i] = hw[i];
    }
    cleanup();
    return OCRT_OK;
}

} // namespace

extern "C" {

void ocrt_ocean_default(ocrt_ocean *oc)
{
    if (!oc) return;
    memset(oc, 0, sizeof(*oc));
    oc->n_mu_water = 48; oc->m_max_water = 2; oc->max_orders_water = 20; oc->tolerance_water = 1e-7;
    oc->tau_base = 20.0; oc->view_as_node = 1;
}

int ocrt_gb_solve_batch_ocean(int n, const ocrt_case *cases, const ocrt_opts *opts, int opts_per_case,
                              const ocrt_aerosol *aer, int aer_per_case, const ocrt_ocean *oc, int oc_per_case,
                              ocrt_result *out, ocrt_ocean_result *wout, void *stream)
{
    if (n < 0 || (n > 0 && (!cases || !opts || !oc))) return fail(OCRT_ERR_ARGS, "bad batch arguments");
    const int rc = ensure_init();
    if (rc) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : g_stream;
    return ocean_solve(n, cases, opts, opts_per_case, aer, aer_per_case, oc, oc_per_case, out, wout, st);
}

int ocrt_gb_solve_ocean(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer, const ocrt_ocean *oc,
                        ocrt_result *out, ocrt_ocean_result *wout)
{
    if (!cs || !oc || !out) return fail(OCRT_ERR_ARGS, "null case, water column or output");
    ocrt_opts def;
    if (!opts) { ocrt_opts_default(&def); opts = &def; }
    return ocrt_gb_solve_batch_ocean(1, cs, opts, 0, aer, 0, oc, 0, out, wout, nullptr);
}

} // extern "C"
