// noalloc.cu — single-pixel solve that allocates no memory.
//
// Some callers cannot allocate device memory: a host application that owns
// the whole device budget through its own pool allocator and forbids any
// other cudaMalloc/cudaFree, or a latency-bound loop that cannot afford the
// implicit device synchronisation cudaMalloc/cudaFree imply.  For them,
// ocrt_gb_solve_case_noalloc solves one pixel with the CUDA-core kernels of
// the allocating path (k_source_simt and k_mol_lowrank for the source,
// k_coxmunk for the rough surface; ocrt_gb_solve_case takes the tensor-core
// kernels k_source_tc and k_coxmunk_tc where it can, so the two agree to the
// parity tolerance, not bit for bit), with every device buffer carved from
// g_noalloc_scratch, a fixed file-scope __device__ array of OCRT_NOALLOC_BYTES
// that each GPU loading this library holds until process exit.  Host staging
// uses the stack only.
//
// Contract:
//  * limits: n_mu <= 32, n_layers <= 400, fourier_m_max <= 32, aerosol
//    L_max <= 255, max_orders <= 4096, and the case's working set must fit
//    the array; larger requests are rejected with OCRT_ERR_ARGS and a message.
//  * the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (and sets the kernels' shared-memory limits) while
//    that device is current.
//  * every call synchronises its stream and polls device counters from the
//    host, so no call may be made while a stream is being captured.
//  * every call shares the one array and leaves its contents behind; each
//    call clears what must start at zero.  Calls whose GPU work overlaps
//    (different host threads, or streams that run concurrently) race on the
//    array and must be serialised by the caller.  In-process calls are
//    serialised by a mutex, and a call that fails after it has queued work
//    waits for that work before it returns.
#include <cuda_runtime.h>
#include <cstring>
#include <mutex>

#include "kernels.cuh"

int ocrt_internal_validate(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer);
int ocrt_internal_fail(int rc, const char *msg);

#define OCRT_NOALLOC_BYTES (32ull << 20)
#define NA_MAX_N 32
#define NA_MAX_LAYERS 400
#define NA_MAX_M 32
#define NA_MAX_L 255
#define NA_MAX_ORDERS 4096
#define NA_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[OCRT_NOALLOC_BYTES];

namespace {

void *g_na_base[NA_MAX_DEVICES];
std::mutex g_na_mu;

struct Carver {
    char *base;
    size_t off, cap;
    bool ok = true;
    template <class T> T *take(size_t n)
    {
        off = (off + 255) & ~size_t(255);
        T *p = (T *)(base + off);
        off += (n ? n : 1) * sizeof(T);
        if (off > cap) ok = false;
        return p;
    }
};

// Failure exits: once work is queued on the stream (enq), wait for it before
// returning, so that the next call does not reuse the array under it.
#define NA_CK(call)                                                                  \
    do {                                                                             \
        if ((call) != cudaSuccess) {                                                 \
            if (enq) (void)cudaStreamSynchronize(st);                                \
            return ocrt_internal_fail(OCRT_ERR_DEVICE, "noalloc: " #call " failed"); \
        }                                                                            \
    } while (0)
#define NA_LAUNCH(...)                                                               \
    do {                                                                             \
        __VA_ARGS__;                                                                 \
        if (cudaGetLastError() != cudaSuccess) {                                     \
            if (enq) (void)cudaStreamSynchronize(st);                                \
            return ocrt_internal_fail(OCRT_ERR_DEVICE, "noalloc: kernel launch failed"); \
        }                                                                            \
    } while (0)

} // namespace

extern "C" int ocrt_gb_solve_case_noalloc(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer_in,
                                          ocrt_result *out, void *stream)
{
    if (!cs || !opts || !out) return ocrt_internal_fail(OCRT_ERR_ARGS, "noalloc: null case, options or output");
    int rc = ocrt_internal_validate(cs, opts, aer_in);
    if (rc) return rc;
    const ocrt_aerosol *aer = (aer_in && aer_in->tau_a > 0.0) ? aer_in : nullptr;
    if (aer && aer->use_value_kernel)
        return ocrt_internal_fail(OCRT_ERR_UNSUPPORTED, "noalloc: the aerosol value kernel needs its table buffers; "
                                                        "use ocrt_gb_solve_case");
    if (opts->n_mu > NA_MAX_N || opts->n_layers > NA_MAX_LAYERS || opts->fourier_m_max > NA_MAX_M ||
        (aer && aer->L_max > NA_MAX_L) || opts->max_orders > NA_MAX_ORDERS)
        return ocrt_internal_fail(OCRT_ERR_ARGS, "noalloc: case exceeds the static-scratch limits "
                                                 "(n_mu<=32, n_layers<=400, m_max<=32, L_max<=255, max_orders<=4096)");
    cudaStream_t st = (cudaStream_t)stream;
    bool enq = false;
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NA_MAX_DEVICES) return ocrt_internal_fail(OCRT_ERR_DEVICE, "noalloc: device index too large");
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_base[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return ocrt_internal_fail(OCRT_ERR_DEVICE, "noalloc: cudaGetSymbolAddress failed");
        NA_CK(cudaFuncSetAttribute(k_coxmunk, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NA_CK(cudaFuncSetAttribute(k_ipss, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NA_CK(cudaFuncSetAttribute(k_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NA_CK(cudaFuncSetAttribute(k_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NA_CK(cudaFuncSetAttribute(k_mol_lowrank, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        g_na_base[dev] = p;
    }

    // ---- host staging (stack only) ----
    const int N = opts->n_mu, M = opts->fourier_m_max, T = M + 1, nt = opts->n_layers, K = nt + 1;
    const Geom G = make_geom(N);
    const int NR = G.NR;
    PixDev d;
    memset(&d, 0, sizeof(d));
    d.lay_off = -1;
    d.sza_deg = cs->sza_deg; d.vza_deg = cs->vza_deg; d.raa_deg = cs->raa_deg; d.wavelength_nm = cs->wavelength_nm;
    d.pressure_hpa = cs->pressure_hpa; d.tau_r_input = cs->tau_r_input;
    d.n_water = cs->n_water; d.wind = cs->wind_speed; d.surface = cs->surface;
    d.sigma_type = cs->sigma_type; d.q_conv = cs->q_convention; d.decouple = cs->decouple_sunglint;
    d.nt = nt; d.M = M; d.max_orders = opts->max_orders; d.tol = opts->tolerance;
    d.tau_r_source = opts->tau_r_source; d.pssa = opts->pssa; d.view_as_node = opts->view_as_node;
    d.aer_h_km = opts->aer_h_km; d.profile = opts->rayleigh_profile; d.ray_h_km = opts->rayleigh_h_km;
    d.nphi = opts->n_phi_surface > 0 ? opts->n_phi_surface : 1024;
    d.mom_off = -1; d.L_aer = -1;
    d.gas = opts->gas ? opts->gas->dev : nullptr;
    d.depol = OCRT_DEPOL; d.ext_off = -1;
    if (aer) { d.mom_off = 0; d.L_aer = aer->L_max; d.tau_a = aer->tau_a; d.ssa_a = aer->ssa_a; }
    d.L = M > 2 ? M : 2;
    if (d.L_aer > d.L) d.L = d.L_aer;
    d.lev_off = 0; d.coef_off = 0; d.task0 = 0;
    const int L = d.L;
    const bool surf = cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN || cs->surface == OCRT_SURFACE_FLAT;
    const bool flat = cs->surface == OCRT_SURFACE_FLAT ||
                      (cs->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && cs->wind_speed <= 0.0);
    const bool rough = surf && !flat;
    const size_t op_elems = (size_t)G.NP * G.CIN;
    const size_t srf_elems = (size_t)NR * N * 9 + (size_t)NR * 9;

    // ---- carve the static array: fixed part, then as many mode tasks per wave as fit ----
    Carver cv{(char *)g_na_base[dev], 0, OCRT_NOALLOC_BYTES};
    PixDev *px = cv.take<PixDev>(1);
    TaskDev *tasks = cv.take<TaskDev>(T);
    TaskState *state = cv.take<TaskState>(T);
    TaskOut *tout = cv.take<TaskOut>(T);
    ocrt_result *res = cv.take<ocrt_result>(1);
    int *ptask0 = cv.take<int>(1);
    double *gmu = cv.take<double>(N), *gw = cv.take<double>(N);
    float *pwt = cv.take<float>(2 * (size_t)N);
    double *h = cv.take<double>(K), *ch = cv.take<double>(K), *xd = cv.take<double>(K);
    double *yd = cv.take<double>(K), *z = cv.take<double>(K);
    double *tabs = cv.take<double>(opts->gas ? K : 1);
    float *Tc = cv.take<float>((size_t)nt * NR), *Ca = cv.take<float>((size_t)nt * NR), *Cb = cv.take<float>((size_t)nt * NR);
    const size_t nb = (size_t)T * (L + 1) * N;
    float *Bp = cv.take<float>(nb), *Br = cv.take<float>(nb), *Bt = cv.take<float>(nb);
    float *cst = cv.take<float>(rough ? (size_t)(T * 2 + 3) * (d.nphi / 2) : 1);
    float *Eatt = cv.take<float>(rough ? (size_t)K * NR : 1);
    float *lvf = cv.take<float>(3 * (size_t)K);
    double *lamv = cv.take<double>((size_t)N + 2);
    float *frs = cv.take<float>((size_t)NR * 9);
    const int La1 = aer ? aer->L_max + 1 : 1;
    double *mb = cv.take<double>(La1), *mg = cv.take<double>(La1), *ma = cv.take<double>(La1), *mz = cv.take<double>(La1);
    double *kappa = cv.take<double>(1), *taudir = cv.take<double>(1);
    int *active = cv.take<int>((size_t)opts->max_orders + 2);
    int *molcnt = cv.take<int>((size_t)opts->max_orders + 2);
    int *work = cv.take<int>(4 * ((size_t)opts->max_orders + 2));
    int *err = cv.take<int>(1);
    float *srf = cv.take<float>(rough ? (size_t)T * srf_elems : 1);
    if (!cv.ok) return ocrt_internal_fail(OCRT_ERR_ARGS, "noalloc: case exceeds the static scratch size");
    const size_t per_task = (size_t)K * G.LDC * 12 + 2 * op_elems * 4 + (size_t)4 * G.LDC * 4 +
                            (size_t)24 * NR * 4 + (size_t)6 * (L + 1) * 4 + 8 * 256;
    const size_t left = cv.cap - ((cv.off + 255) & ~size_t(255));
    int Wt = (int)(left / per_task);
    if (Wt > T) Wt = T;
    if (Wt < 1) return ocrt_internal_fail(OCRT_ERR_ARGS, "noalloc: case exceeds the static scratch size");
    float *F = cv.take<float>((size_t)Wt * K * G.LDC);
    float *J = cv.take<float>((size_t)Wt * K * G.LDC);
    float *Tot = cv.take<float>((size_t)Wt * K * G.LDC);
    float *Ttl = cv.take<float>((size_t)Wt * 2 * G.LDC);
    float *ops = cv.take<float>(2 * (size_t)Wt * op_elems);
    float *pvec = cv.take<float>((size_t)Wt * 2 * G.LDC);
    float *fvec = cv.take<float>((size_t)Wt * 24 * NR);
    float *Bx = cv.take<float>((size_t)Wt * 6 * (L + 1));
    int *alist0 = cv.take<int>((size_t)Wt), *alist1 = cv.take<int>((size_t)Wt);
    int *mlist0 = cv.take<int>((size_t)Wt), *mlist1 = cv.take<int>((size_t)Wt);
    if (!cv.ok) return ocrt_internal_fail(OCRT_ERR_ARGS, "noalloc: case exceeds the static scratch size");

    TaskDev ht[NA_MAX_M + 1];
    for (int m = 0; m < T; ++m) {
        const int q = m % Wt;
        memset(&ht[m], 0, sizeof(TaskDev));
        ht[m].pix = 0; ht[m].m = m; ht[m].K = K; ht[m].has_mol = m <= 2;
        ht[m].fld_off = (long long)q * K * G.LDC;
        ht[m].tail_off = (long long)q * 2 * G.LDC;
        ht[m].op_off = (long long)(2 * q) * (long long)op_elems;
        ht[m].mol_off = m <= 2 ? (long long)(2 * q + 1) * (long long)op_elems : -1;
        ht[m].uv_off = -1;
        ht[m].srf_off = rough ? (long long)m * (long long)srf_elems : -1;
    }
    const int zero = 0;
    enq = true;
    NA_CK(cudaMemcpyAsync(px, &d, sizeof(PixDev), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(tasks, ht, sizeof(TaskDev) * T, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(ptask0, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    if (aer) {
        NA_CK(cudaMemcpyAsync(mb, aer->beta, sizeof(double) * La1, cudaMemcpyHostToDevice, st));
        NA_CK(cudaMemcpyAsync(mg, aer->gamma, sizeof(double) * La1, cudaMemcpyHostToDevice, st));
        NA_CK(cudaMemcpyAsync(ma, aer->alpha, sizeof(double) * La1, cudaMemcpyHostToDevice, st));
        NA_CK(cudaMemcpyAsync(mz, aer->zeta, sizeof(double) * La1, cudaMemcpyHostToDevice, st));
    }
    NA_CK(cudaStreamSynchronize(st));      // host staging lives on this stack frame
    NA_CK(cudaMemsetAsync(err, 0, sizeof(int), st));

    // ---- the kernel sequence of the allocating path, CUDA-core source and Cox-Munk kernels ----
    NA_LAUNCH(k_gauss<<<1, 64, 0, st>>>(N, gmu, gw, pwt));
    NA_LAUNCH(k_pixel_setup<<<1, 32, 0, st>>>(px, 1, N, gmu));
    NA_LAUNCH(k_levels<<<dim3(2, 1), 256, 0, st>>>(px, 1, h, ch, xd, yd, z));
    NA_LAUNCH(k_level_mix<<<dim3(2, 1), 256, 0, st>>>(px, 1, z, xd, yd));
    if (opts->gas) NA_LAUNCH(k_gas_apply<<<1, 256, 0, st>>>(px, 1, h, ch, xd, yd, z, tabs));
    NA_LAUNCH(k_coef<<<dim3(16, 1), 256, 0, st>>>(px, 1, N, NR, gmu, h, Tc, Ca, Cb));
    NA_LAUNCH(k_basis_gauss<<<T, 64, 0, st>>>(N, M, L, gmu, Bp, Br, Bt, nullptr));
    if (rough) {
        NA_LAUNCH(k_cs_table<<<T + 1, 256, 0, st>>>(M, d.nphi, cst));
        NA_LAUNCH(k_seed_att<<<dim3(8, 1), 256, 0, st>>>(px, 1, N, gmu, h, Eatt));
        NA_LAUNCH(k_sancer<<<1, 128, 0, st>>>(px, 1, N, gmu, lamv, nullptr));
        NA_LAUNCH(k_coxmunk<<<dim3(N + 1, NR, 1), 256, coxmunk_smem_bytes(d.nphi, false), st>>>(
            tasks, px, 0, ptask0, G, gmu, cst, M, lamv, srf));
    }
    NA_LAUNCH(k_level_float<<<dim3(2, 1), 256, 0, st>>>(px, 1, xd, yd, ch, lvf));
    if (flat) NA_LAUNCH(k_flat_fresnel<<<1, 128, 0, st>>>(px, 1, N, gmu, frs));

    BatchBufs B;
    B.px = px; B.tasks = tasks; B.state = state; B.tout = tout; B.gmu = gmu; B.gw = gw; B.pw = pwt;
    B.h = h; B.ch = ch; B.xd = xd; B.yd = yd; B.z = z; B.Tc = Tc; B.Ca = Ca; B.Cb = Cb; B.Cq = nullptr; B.frs = frs; B.Eatt = Eatt; B.lvf = lvf;
    B.active_cnt = active; B.err = err; B.mol_cnt = molcnt; B.work = work; B.molV = nullptr;
    B.alist[0] = alist0; B.alist[1] = alist1; B.mlist[0] = mlist0; B.mlist[1] = mlist1;
    WaveBufs W;
    W.F = F; W.J = J; W.Tot = Tot; W.Ttl = Ttl; W.ops = ops; W.opt = nullptr; W.pvec = pvec; W.fvec = flat ? fvec : nullptr; W.srf = srf;
    const int scan_threads = ((G.COUT + 31) / 32) * 32;
    for (int t0 = 0; t0 < T; t0 += Wt) {
        const int nw = (T - t0) < Wt ? (T - t0) : Wt;
        const int nmol = t0 <= 2 ? ((3 - t0) < nw ? (3 - t0) : nw) : 0;   // tasks are ordered by mode
        NA_CK(cudaMemsetAsync(ops, 0, sizeof(float) * 2 * (size_t)nw * op_elems, st));
        NA_CK(cudaMemsetAsync(pvec, 0, sizeof(float) * (size_t)nw * 2 * G.LDC, st));
        if (flat) NA_CK(cudaMemsetAsync(fvec, 0, sizeof(float) * (size_t)nw * 24 * NR, st));
        NA_CK(cudaMemsetAsync(active, 0, sizeof(int) * ((size_t)opts->max_orders + 2), st));
        NA_CK(cudaMemsetAsync(molcnt, 0, sizeof(int) * ((size_t)opts->max_orders + 2), st));
        NA_CK(cudaMemsetAsync(work, 0, sizeof(int) * 4 * ((size_t)opts->max_orders + 2), st));
        NA_LAUNCH(k_basis_pix<<<(nw + 63) / 64, 128, 0, st>>>(tasks, t0, nw, px, L, 1, Bx, nullptr));
        NA_LAUNCH(k_tables<<<dim3(nw, tables_yblocks(256, G.NR, G.N)), 256, tables_smem_bytes(256, G.N, L), st>>>(
            tasks, t0, nw, px, G, L, Bp, Br, Bt, Bx, gw, mb, mg, ma, mz, ops, pvec, W.fvec, nullptr, 1, nullptr, 0, 0,
            nullptr));
        NA_LAUNCH(k_primary<<<nw, scan_threads, 0, st>>>(B, W, G, t0));
        const dim3 sgrid(nw, (K + ST_M_TILE - 1) / ST_M_TILE, (G.COUT + ST_N_TILE - 1) / ST_N_TILE);
        for (int it = 2; it <= opts->max_orders; ++it) {
            NA_LAUNCH(k_source_simt<<<sgrid, 256, 0, st>>>(B, W, G, t0, it));
            if (nmol > 0)
                NA_LAUNCH(k_mol_lowrank<<<dim3(nmol * ((K + 31) / 32)), 256, mol_smem_bytes(G), st>>>(
                    B, W, G, t0, it, (K + 31) / 32, Bp, Br, Bt, L));
            NA_LAUNCH(k_scan<<<nw, scan_threads, scan_smem_bytes(scan_threads), st>>>(B, W, G, t0, it));
            if ((it - 1) % 4 == 0 || it == opts->max_orders) {
                int left_active = 0;
                NA_CK(cudaMemcpyAsync(&left_active, active + it, sizeof(int), cudaMemcpyDeviceToHost, st));
                NA_CK(cudaStreamSynchronize(st));
                if (left_active == 0) break;
            }
        }
        NA_LAUNCH(k_extract<<<(nw + 127) / 128, 128, 0, st>>>(B, W, G, t0, nw));
    }
    if (opts->pssa) {
        const size_t smem = sizeof(double) * (6 * (size_t)nt + 6) + sizeof(int) * ((size_t)nt + 1);
        NA_LAUNCH(k_ipss<<<1, 256, smem, st>>>(px, 1, h, z, xd, yd, opts->gas ? tabs : nullptr, mb, nullptr, nullptr,
                                               kappa, taudir));
    }
    NA_LAUNCH(k_finalize<<<1, 32, 0, st>>>(px, 1, state, tout, gmu, gw, h, kappa, taudir, res));
    int dev_err = 0;
    NA_CK(cudaMemcpyAsync(out, res, sizeof(ocrt_result), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&dev_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (dev_err) return ocrt_internal_fail(dev_err, "noalloc: non-finite field during the SOS iteration");
    return OCRT_OK;
}
