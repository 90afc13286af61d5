/*
 * ocrt_gb300.h — C ABI of the GB300 successive-orders-of-scattering (SOS)
 * vector radiative-transfer solve path.
 *
 * Drop-in boundary for the solve API of the OCRT C solver
 * (code/OCRT_C/src/rt_solver.h).  Plain C types only: no CUDA or torch types
 * cross this boundary, so the library can be bound from C, ctypes, cgo or JNI.
 *
 * Conventions kept from the reference (rt_types.h:7-50, rt_solver.h):
 *   - F_sun = pi normalisation ("Convention B"): rho = I_TOA / mu_sun.
 *   - Fourier reconstruction X(phi) = X_0 + 2 sum_m X_m cos m(phi+pi),
 *     U(phi) = 2 sum_m U_m sin m(phi+pi)           (rt_fourier.c:9-33).
 *   - Return codes: 0 ok, -1 invalid arguments, -2 non-finite field,
 *     -3 allocation failure, -7 bottom-source shape (rt_solver.h:7-11).
 *     Non-convergence is not an error: converged = 0 and
 *     n_orders_used = max_orders (rt_solver.c:2193-2211).
 *   - Callers own every input and output buffer.
 */
#ifndef OCRT_GB300_H
#define OCRT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------ */
#define OCRT_OK                        0
#define OCRT_ERR_ARGS                 -1
#define OCRT_ERR_NONFINITE            -2
#define OCRT_ERR_ALLOC                -3
#define OCRT_ERR_DEVICE               -4   /* CUDA launch/runtime failure (no reference counterpart) */
#define OCRT_ERR_UNSUPPORTED          -5   /* surface/mode outside the GB300 solve path */
#define OCRT_ERR_BOTTOM_SOURCE_SHAPE  -7

/* ---- enumerations (values identical to rt_types.h:59-65, 181-184) ------ */
enum {
    OCRT_SURFACE_BLACK = 0,
    OCRT_SURFACE_LAMBERT = 1,               /* not on the solve path: -5 */
    OCRT_SURFACE_BLACK_FRESNEL_OCEAN = 2,   /* rough (wind>0) or flat (wind<=0) Fresnel over a black ocean */
    OCRT_SURFACE_FLAT = 3,                  /* exact flat Fresnel */
    OCRT_SURFACE_OCEAN = 4                  /* coupled in-water solve: ocrt_gb_solve_ocean */
};
enum { OCRT_TAU_R_AUTO = 0, OCRT_TAU_R_FROM_INPUT = 1 };
/* Altitude mapping of the uniform-optical-depth level grid.  The plane-parallel
 * solve does not depend on it; IPSS ray tracing does (rt_atm.c:205-232). */
enum { OCRT_PROFILE_US62 = 0, OCRT_PROFILE_EXPONENTIAL = 1 };

/* ---- per-case input (solve-relevant fields of rt_case_t, rt_types.h:321-360) */
typedef struct {
    double sza_deg;          /* [0, 90) */
    double vza_deg;          /* [0, 90) */
    double raa_deg;          /* public relative azimuth, degrees */
    double wavelength_nm;    /* [330, 1100] */
    int    surface;          /* OCRT_SURFACE_* */
    double pressure_hpa;     /* <= 0 => no Rayleigh (rt_types.h:327-330) */
    double tau_r_input;      /* column Rayleigh depth for OCRT_TAU_R_FROM_INPUT */
    double n_water;          /* default 1.34 */
    double wind_speed;       /* m/s; <= 0 => flat Fresnel for BLACK_FRESNEL_OCEAN */
    int    sigma_type;       /* 0 Nakajima-Tanaka, 1 OCRT floor law (default 1) */
    int    q_convention;     /* 0 legacy (Rs-Rp)/2, 1 Mishchenko (Rp-Rs)/2 (default 1) */
    int    decouple_sunglint;/* 1 => direct sunglint not added to rho */
} ocrt_case;

/* ---- trace-gas absorption state (rt_absorption_t, rt_absorption.h:66-76) --
 * Opaque; made by ocrt_gb_gas_create and named in ocrt_opts.gas the way the
 * reference's rt_options_t.abs_state names an rt_absorption_t
 * (rt_solver.c:753-759).  It must outlive every solve or plan that uses it. */
typedef struct ocrt_gas ocrt_gas;

/* ---- solver options (solve-relevant fields of rt_options_t, rt_types.h:654-795) */
typedef struct {
    int    n_mu;             /* Gauss nodes per hemisphere, default 24, max 64 */
    int    n_layers;         /* default 40, max 1024 */
    int    fourier_m_max;    /* default 2; the reference caps this at 32, this library at 255 */
    int    max_orders;       /* SOS max_iterations, default 20 */
    double tolerance;        /* SOS relative sup-norm tolerance, default 1e-7 */
    int    tau_r_source;     /* OCRT_TAU_R_* */
    int    pssa;             /* 1 => IPSS spherical correction (rt_ipss.h) */
    int    view_as_node;     /* 1 (default) => mu_view is a zero-weight ring node */
    double aer_h_km;         /* aerosol scale height, default 2 km */
    int    rayleigh_profile; /* OCRT_PROFILE_* (default US62, the reference's mapping) */
    double rayleigh_h_km;    /* scale height for OCRT_PROFILE_EXPONENTIAL */
    int    n_phi_surface;    /* Cox-Munk azimuth quadrature, default 1024 */
    const ocrt_gas *gas;     /* NULL => no gas absorption (abs_state, rt_atm.c:437) */
} ocrt_opts;

/* ---- aerosol (rt_aerosol_input_t, rt_solver.h:94-114) ------------------
 * The moment expansion drives every element of the aerosol phase matrix.
 * With use_value_kernel set, the intensity-to-intensity phase table is
 * instead the direct azimuth integral (720 midpoints) of the tabulated P11,
 * linear in the scattering angle (rt_solver.c:188-235), and IPSS weights the
 * aerosol single scattering with the same table (rt_ipss.c:81-146); the
 * polarised elements stay on the moments.  Zero-filled trailing fields give
 * the moment path. */
typedef struct {
    double tau_a;            /* column AOD at the wavelength */
    double ssa_a;            /* aerosol single-scattering albedo [0,1] */
    int    L_max;            /* >= 2 */
    const double *beta;      /* [L_max+1], beta_0 = 1 */
    const double *gamma;     /* [L_max+1] */
    const double *alpha;     /* [L_max+1] */
    const double *zeta;      /* [L_max+1] */
    int    use_value_kernel; /* 0: moment kernel; 1: value kernel from the phase table below */
    int    n_ang_phase;      /* table size (>= 2 when use_value_kernel) */
    const double *theta_phase;                     /* [n_ang_phase] scattering angles, degrees, ascending */
    const double *P11_phase, *P12_phase, *P33_phase; /* [n_ang_phase], normalised so (1/2) int P11 dmu = 1 */
} ocrt_aerosol;

/* ---- per-case output (solve-path fields of rt_result_t, rt_types.h:496-651) */
typedef struct {
    double rho_I, rho_Q, rho_U;
    double I_TOA, Q_TOA, U_TOA;
    double tau_R_total;
    int    n_orders_used;     /* max over Fourier modes */
    int    converged;         /* AND over Fourier modes */
    int    order_modes;       /* sum over modes of orders executed (work actually done) */
    double kappa_ipss;        /* IPSS factor applied (1 when off) */
    double T_dir_dn;
    double T_diff_dn_hemi;
    double T_total_dn_hemi;
    double T_diff_dn_dir;
    double T_total_up_dir;
    double T_sg_up_dir;
    double T_dir_up_view;
    double rho_glint_direct_I, rho_glint_direct_Q, rho_glint_direct_U;
} ocrt_result;

/* Optional per-mode diagnostics; every non-NULL array holds fourier_m_max+1
 * entries (sos_orders_per_m / sos_residual_per_m of rt_result_t). */
typedef struct {
    int    *orders_per_m;
    double *residual_per_m;
    double *view_I_m, *view_Q_m, *view_U_m;   /* TOA upwelling at mu_view per mode */
} ocrt_diag;

/* Fill defaults identical to rt_options_default() (rt_types.h:760-795) plus
 * the CLI case defaults of main.c:1826-1840. */
void ocrt_opts_default(ocrt_opts *opts);
void ocrt_case_default(ocrt_case *cs);

/* ---- device lifetime -------------------------------------------------- */
/* Select the CUDA device and create the library's streams, CUDA graphs cache
 * and workspace arena.  Idempotent.  Replaces no reference call (the
 * reference allocates per solve, rt_solver.h:45-48). */
int         ocrt_gb_init(int device);
void        ocrt_gb_shutdown(void);
const char *ocrt_gb_last_error(void);

/* ---- single solve ------------------------------------------------------
 * Replaces rt_solve_case_pol (rt_solver.h:84-85) when aer == NULL or
 * aer->tau_a == 0, and rt_solve_case_pol_aerosol (rt_solver.h:119-121)
 * otherwise.  Host buffers in, host result out. */
int ocrt_gb_solve_case(const ocrt_case *cs, const ocrt_opts *opts,
                       const ocrt_aerosol *aer, ocrt_result *out,
                       ocrt_diag *diag);

/* ---- batched solve -----------------------------------------------------
 * n independent pixels in one device pass.  opts / aer are either one shared
 * object (*_per_case = 0) or arrays of n (*_per_case = 1); aer may be NULL.
 * Each pixel's result equals ocrt_gb_solve_case on the same inputs.  This is
 * the GPU form of the reference's OpenMP row loop (rt_io.c:197-199).
 * stream: a cudaStream_t passed as void* (NULL = the library's stream). */
int ocrt_gb_solve_batch(int n, const ocrt_case *cases,
                        const ocrt_opts *opts, int opts_per_case,
                        const ocrt_aerosol *aer, int aer_per_case,
                        ocrt_result *out, void *stream);

/* ---- resident plans (inputs uploaded once, solved many times) -----------
 * A plan holds the device copy of a batch.  ocrt_gb_plan_execute runs the
 * full solve on device-resident inputs (no host traffic); results stay on the
 * device until ocrt_gb_plan_results copies them out.
 * The first execute runs eagerly: host polls of the device active-task counts
 * end each order loop, and the order count each wave needed is recorded.  The
 * second execute captures the same launch sequence with those counts and no
 * host polls into a CUDA graph; later executes replay the graph (one launch
 * call, no host synchronisation).  A replay that ends with a task still
 * iterating is reported by ocrt_gb_plan_results as an error and the plan goes
 * back to eager executes.  OCRT_GB_GRAPH=0, or timing enabled, keeps every
 * execute eager. */
typedef struct ocrt_plan ocrt_plan;
int  ocrt_gb_plan_create(int n, const ocrt_case *cases,
                         const ocrt_opts *opts, int opts_per_case,
                         const ocrt_aerosol *aer, int aer_per_case,
                         ocrt_plan **plan);
int  ocrt_gb_plan_execute(ocrt_plan *plan, void *stream);
int  ocrt_gb_plan_results(ocrt_plan *plan, ocrt_result *out, void *stream);
/* Device time of the last execute's kernels, and how many of this library's
 * kernels it launched. */
int  ocrt_gb_plan_stats(const ocrt_plan *plan, double *order_modes_total,
                        long long *kernel_launches);
void ocrt_gb_plan_destroy(ocrt_plan *plan);
/* 1 when the next ocrt_gb_plan_execute replays a captured CUDA graph. */
int  ocrt_gb_plan_graph_ready(const ocrt_plan *plan);

/* Launch-shape autotuner (no reference counterpart).  The Cox-Munk Fourier
 * projection and the phase-table kernels are timed at 128, 256 and 512
 * threads per block the first time a shape (N, n_phi, M / N, L, M) is met,
 * and the fastest is used from then on (OCRT_GB_AUTOTUNE=0: 256 always).
 * Writes one line per tuned shape into buf (NUL-terminated, truncated to
 * len) and returns the length of the full text. */
int  ocrt_gb_autotune_summary(char *buf, int len);

/* Per-kernel-class instrumentation (no reference counterpart).  With timing
 * enabled every launch of a plan is bracketed by CUDA events on the launching
 * stream.  ocrt_gb_plan_kernel_stats(plan, -1, ...) returns the number of
 * classes; for a class index it returns the class name, summed device time of
 * the last execute, launch count, and the algorithmic FLOPs and bytes that
 * execute performed (derived from the orders each task ran). */
void ocrt_gb_set_timing(int enable);
int  ocrt_gb_plan_kernel_stats(ocrt_plan *plan, int cls, const char **name, double *ms,
                               long long *launches, double *alg_flops, double *alg_bytes);

/* ---- single solve that allocates nothing --------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory: an application that owns the whole device budget through its own
 * pool allocator and forbids any other cudaMalloc/cudaFree, or a latency-bound
 * loop that cannot afford the implicit device synchronisation of cudaMalloc
 * and cudaFree.  Same inputs and outputs as ocrt_gb_solve_case; it runs the
 * CUDA-core source and Cox-Munk kernels of the allocating path (which takes
 * the tensor-core ones where it can), so results agree with
 * ocrt_gb_solve_case to the parity tolerance rather than bit for bit.  Every
 * device buffer lives in one fixed 32 MiB __device__ array that each GPU
 * loading this library holds until exit; no cudaMalloc, cudaFree or pinned
 * host allocation is made.  Limits: n_mu <= 32, n_layers <= 400,
 * fourier_m_max <= 32, aerosol L_max <= 255, max_orders <= 4096; larger
 * requests return OCRT_ERR_ARGS with a message.  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress) with that device
 * current.  Every call synchronises its stream and polls device counters, so
 * it must never be called while a stream is being captured.  All calls share
 * the array: each call clears what must start at zero, and calls whose GPU
 * work overlaps race on it and must be serialised by the caller (calls in
 * one process are serialised by a lock; a call that fails after queuing work
 * waits for that work before returning).  stream: a cudaStream_t as void*
 * (NULL = the default stream). */
int ocrt_gb_solve_case_noalloc(const ocrt_case *cs, const ocrt_opts *opts,
                               const ocrt_aerosol *aer, ocrt_result *out,
                               void *stream);

/* ---- angle-grid LUT mode ------------------------------------------------
 * Replaces rt_solve_case_pol_lut (rt_solver.h:207-210) and its
 * rt_lut_grid_out_t (rt_types.h:805-846): one SOS per case, then the TOA
 * reflectance at every (vza, raa) of a grid.  Per Fourier mode the upwelling
 * TOA field is sampled at each grid vza by monotone cubic (PCHIP) interpolation
 * over the ring nodes (linear outside them), the modes are summed at each raa,
 * and IPSS kappa (when pssa) and the direct sunglint (rough ocean) are applied
 * per grid direction.  Arrays are caller-allocated; outputs are row-major
 * [iv * n_raa + ir].  The case's own vza/raa give the result in `out` as usual
 * (the reference CLI passes vza = raa = 0 for a grid run). */
typedef struct {
    int n_vza;
    const double *vza_deg;     /* [n_vza], each in [0, 90) */
    int n_raa;
    const double *raa_deg;     /* [n_raa], public relative azimuth */
    double *rho_I, *rho_Q, *rho_U;                      /* [n_vza * n_raa] */
    double *T_diff_dn_dir, *T_sg_up_dir, *T_total_up_dir; /* optional (NULL to skip) */
    double T_dir_dn, T_diff_dn_hemi;                    /* filled: case-level scalars */
} ocrt_lut;

int ocrt_gb_solve_case_lut(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                           ocrt_result *out, ocrt_lut *lut);
/* n cases, each with its own grid (luts[i]); one device pass. */
int ocrt_gb_solve_batch_lut(int n, const ocrt_case *cases,
                            const ocrt_opts *opts, int opts_per_case,
                            const ocrt_aerosol *aer, int aer_per_case,
                            ocrt_lut *luts, ocrt_result *out, void *stream);

/* ---- per-layer parameters and the adjoint ------------------------------
 * No counterpart in the reference (its solve API takes no per-layer inputs
 * and has no derivatives).  Layer l (0-based, l < n_layers) spans levels l
 * and l+1 of the level grid (level 0 = TOA).
 *   dtau[l] replaces the uniform optical-depth grid: h_k = sum_{l<k} dtau[l].
 *   ssa[l]  is the single-scattering albedo of layer l: level l+1's aerosol
 *           and molecular scattering fractions (rt_atm.c:313-383) are scaled
 *           together so that they sum to ssa[l].
 * The aerosol/molecular split of every layer, and the level altitudes, stay
 * those of the profile's uniform grid.  NULL arrays keep the profile values.
 * IPSS (opts.pssa) cannot be combined with overrides or gradients. */
typedef struct {
    int n_layers;            /* must equal opts.n_layers of the case */
    const double *dtau;      /* [n_layers], each > 0, or NULL */
    const double *ssa;       /* [n_layers], each in [0, 1], or NULL */
} ocrt_layers;

/* Gradient of  c_I rho_I + c_Q rho_Q + c_U rho_U  (one cotangent row) with
 * respect to the layer optical depths, the layer single-scattering albedos
 * and the wind speed.  The caller allocates d_dtau and d_ssa (n_layers). */
typedef struct {
    double *d_dtau;
    double *d_ssa;
    double  d_wind;
} ocrt_grad;

/* Batched forward solve with optional per-layer parameters and, for each
 * pixel, n_cot cotangent rows cot[(i * n_cot + r) * 3 + {0,1,2}] for
 * (rho_I, rho_Q, rho_U); grad[i * n_cot + r] receives row r's gradient.
 * n_cot = 3 with the identity rows gives the full Jacobian.  n_cot = 0 is a
 * plain forward solve with the overrides (cot and grad may be NULL).
 * layers: NULL or n entries (one per case).  The gradient is the adjoint of
 * the converged SOS system: the forward keeps two checkpoints per Fourier
 * mode (the order total and the last order's field), and an adjoint
 * successive-orders sweep with the transposed source, transport and surface
 * operators gives every parameter derivative in one pass per cotangent row.
 * Supported surfaces: BLACK and BLACK_FRESNEL_OCEAN with wind > 0; pssa = 0.
 * Otherwise OCRT_ERR_UNSUPPORTED. */
/* Profile values of the per-layer parameters of one case, the values that a
 * NULL ocrt_layers array stands for: dtau[l] = h_{l+1} - h_l and
 * ssa[l] = the summed scattering fractions of level l+1 (rt_atm.c:177-400),
 * after the gas absorption step when opts.gas is set.
 * Both arrays hold opts.n_layers entries (either may be NULL). */
int ocrt_gb_layer_defaults(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                           double *dtau, double *ssa);

/* ---- trace-gas absorption (rt_absorption.c, rt_atm.c:437-548) -----------
 * Six gases in the reference's order (rt_absorption.h:35-37) and the seven
 * AFGL atmospheres (rt_absorption.h:24-32).  ocrt_gb_gas_create reads
 * <afgl_dir>/afgl_<profile>.dat and <xsec_dir>/xsec_<gas>.dat (the files of
 * the reference's inputs/afgl_atm and inputs/xsec), integrates the default
 * columns and uploads the profile and the cross-section tables to the device
 * once.  column_override: NULL, or six entries, each < 0 (AFGL default) or
 * the total column in molecules/cm^2 (the profile shape is kept).  A missing
 * or unusable cross-section file leaves that gas out, as in the reference
 * (rt_absorption.c:486-520); a missing AFGL file is OCRT_ERR_ARGS.
 * With opts.gas set, every solve adds the per-layer absorption depths of
 * the case's level altitudes to the optical-depth grid and scales the
 * scattering fractions by dtau_old / dtau_new (rt_atm.c:449-546); IPSS uses
 * the layer absorption for its single-scattering albedo (rt_ipss.c:64-70).
 * Layer overrides (ocrt_layers) apply on top of the gas-loaded profile. */
enum { OCRT_GAS_H2O = 0, OCRT_GAS_O3, OCRT_GAS_O2, OCRT_GAS_CO2, OCRT_GAS_NO2, OCRT_GAS_CH4, OCRT_N_GAS };
enum { OCRT_AFGL_USSTD76 = 0, OCRT_AFGL_TROPICAL, OCRT_AFGL_MLSUMM, OCRT_AFGL_MLWINT,
       OCRT_AFGL_SASUMM, OCRT_AFGL_SAWINT, OCRT_AFGL_USERDEF };
int  ocrt_gb_gas_create(const char *afgl_dir, const char *xsec_dir, int profile,
                        const double *column_override, ocrt_gas **out);
void ocrt_gb_gas_destroy(ocrt_gas *gas);
/* Column absorption depth at one wavelength, per gas and total
 * (rt_absorption_tau_per_gas / rt_absorption_tau_total, rt_absorption.c:556-600).
 * tau_per_gas: NULL or OCRT_N_GAS entries. */
int  ocrt_gb_gas_tau(const ocrt_gas *gas, double wavelength_nm, double *tau_per_gas, double *tau_total);
/* Effective and default total columns (molecules/cm^2), OCRT_N_GAS entries
 * each (either may be NULL); overridden[g] = 1 where the caller set it. */
int  ocrt_gb_gas_columns(const ocrt_gas *gas, double *column_eff, double *column_default, int *overridden);
/* Per-layer absorption depths of one case as the solve applies them
 * (tau_abs, opts.n_layers entries, zero without opts.gas) and the level
 * altitudes in km (z_km, opts.n_layers + 1 entries, level 0 = TOA). */
int  ocrt_gb_layer_gas(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                       double *tau_abs, double *z_km);

/* ---- aerosol models from .mie tables ------------------------------------
 * ocrt_gb_mie_read replaces read_mie_file (shared/mie_io.c:174-327): the
 * OPAC layout (angle count, free header, spectral rows of wavelength [um]
 * and six columns, then the P11, P12 and P33 blocks with an optional TETA
 * line naming a separate phase-wavelength grid).  ocrt_gb_mie_prepare
 * replaces rt_aerosol_runtime_prepare (rt_aerosol_runtime.c:13-285) for the
 * CLI's aerosol protocol (main.c:3296-3343, 3646-3686): the AOD given at
 * aod_ref_nm is carried to the wavelength by the table's extinction ratio,
 * SSA is interpolated linearly, P11/P12/P33 by PCHIP in wavelength; the
 * real-angle log10-linear forward-peak truncation (rt_aerosol.c:403-552) with
 * its mass-conserving tau/SSA renormalisation; vector moments to L_max from
 * a 4096-point PCHIP-densified angle grid (rt_aerosol.c:119-213, 649-774);
 * and the phase table normalised by beta_0 and ordered by ascending angle
 * for the value kernel.  The prepared aerosol (ocrt_mie_aerosol) owns the
 * arrays that the filled ocrt_aerosol points into. */
typedef struct ocrt_mie ocrt_mie;
typedef struct ocrt_mie_aerosol ocrt_mie_aerosol;
typedef struct {
    int    L_max;                /* moment order (CLI default 80) */
    int    use_loglin_trunc;     /* 1 (CLI default): log10-linear truncation */
    double loglin_mu1, loglin_mu2, loglin_threshold;   /* 0.8, 0.94, 0.1 */
    int    use_value_kernel;     /* 1 (CLI default): value kernel for the I-I table */
} ocrt_mie_opts;
typedef struct {
    double aod_ref, aod_ref_nm;          /* the given AOD and its wavelength */
    double aod_target, extinction_ratio; /* AOD at the wavelength = aod_ref * extinction_ratio */
    double ssa_raw;                      /* interpolated SSA before truncation */
    double trunc_A;                      /* truncation coefficient A (0: none) */
    double tau_a_eff, ssa_a_eff;         /* after the truncation renormalisation */
} ocrt_mie_diag;
void ocrt_mie_opts_default(ocrt_mie_opts *o);
int  ocrt_gb_mie_read(const char *path, ocrt_mie **out);
void ocrt_gb_mie_free(ocrt_mie *m);
/* Table sizes: angles, spectral wavelengths, phase wavelengths (any may be NULL). */
int  ocrt_gb_mie_shape(const ocrt_mie *m, int *n_ang, int *n_wl, int *n_phase_wl);
/* OCRT_ERR_ARGS when the wavelength or aod_ref_nm lies outside the table's
 * grids, the table does not span 0..180 degrees, or aod_ref <= 0. */
int  ocrt_gb_mie_prepare(const ocrt_mie *m, double wavelength_nm, double aod_ref, double aod_ref_nm,
                         const ocrt_mie_opts *opts, ocrt_mie_aerosol **out, ocrt_aerosol *aer,
                         ocrt_mie_diag *diag);
void ocrt_gb_mie_aerosol_free(ocrt_mie_aerosol *a);

/* ---- coupled atmosphere-ocean (rt_solve_case_ocean, rt_solver.h:145-149) -
 * Three successive-orders solves joined at a rough (Cox-Munk) air-water
 * interface, as rt_solve_case_ocean runs them (rt_solver.c:3468-6660):
 *   1. the atmosphere over the rough Fresnel surface, with the diffuse
 *      downward field at the bottom of the atmosphere exported per mode;
 *   2. the water column: the refracted direct beam (polarised by the
 *      Fresnel transmission) and the transmitted skylight as sources, the
 *      internal reflection of the upward field at the surface as the top
 *      boundary, a black bottom (rt_water_rt.c:3549-7578);
 *   3. the atmosphere again, driven only by the water-leaving radiance
 *      transmitted up through the surface as a bottom source.
 * TOA reflectance = pass 1 + pass 3; the water-leaving and in-water
 * quantities of rt_result_t go to ocrt_ocean_result.  The case's surface
 * must be OCRT_SURFACE_OCEAN with wind_speed > 0; opts.n_mu is ignored (the
 * atmosphere solves use n_mu_water nodes, as the reference does), pssa must
 * be 0 (the reference refuses IPSS on this path).
 * Water optical properties are given directly (the reference derives them
 * from its pure-water tables and constituent models, rt_water_iop.c):
 * pure-seawater scattering uses the Rayleigh-like matrix with depolarisation
 * 0.039 (rt_water_rt.c:2104-2236), hydrosol scattering a moment expansion
 * like the aerosol's. */
typedef struct {
    double a_total;          /* absorption of the water [1/m] */
    double b_water;          /* pure-seawater scattering [1/m] */
    double b_particle;       /* hydrosol scattering [1/m]; 0 = none */
    int    L_particle;       /* hydrosol expansion order (>= 1 when b_particle > 0) */
    const double *beta, *gamma, *alpha, *zeta;   /* [L_particle+1] hydrosol moments, beta_0 = 1 */
    int    n_mu_water;       /* Gauss nodes per hemisphere in the water (default 48) */
    int    m_max_water;      /* Fourier modes of the in-water solve (default 2) */
    int    max_orders_water; /* in-water SOS orders (default 20) */
    double tolerance_water;  /* in-water SOS tolerance (default 1e-7) */
    int    n_layers_water;   /* depth policy: at least this many layers, and at least
                                optical depth / 0.05; fixed depth: exactly this many
                                (0 = optical depth / 0.05) */
    double depth_m;          /* > 0: black bottom at this depth; 0 (default) = depth policy:
                                optical depth >= tau_base and 1e-8 transport attenuation */
    double tau_base;         /* base optical depth of the depth policy (default 20; the
                                reference's constituent-model path uses 15) */
    int    view_as_node;     /* 1 (default): the refracted view is a zero-weight water node */
} ocrt_ocean;

typedef struct {
    double rho_atm_I, rho_atm_Q, rho_atm_U;          /* TOA reflectance of pass 1 (atmosphere and surface) */
    double rho_water_I, rho_water_Q, rho_water_U;    /* TOA reflectance of the water-leaving light (pass 3) */
    double Lu_0minus_I, Lu_0minus_Q, Lu_0minus_U;    /* upwelling just below the surface, view direction */
    double Lu_0plus_I, Lu_0plus_Q, Lu_0plus_U;       /* water-leaving radiance just above the surface */
    double Ed_0minus, Eu_0minus, Ed_0plus;           /* irradiances (F_sun = pi units) */
    double Ed_0minus_direct, Ed_0plus_direct;
    double Rrs_0plus_I, Rrs_0plus_Q, Rrs_0plus_U;    /* Lu(0+) / Ed(0+) */
    double rrs_0minus_I, rrs_0minus_Q, rrs_0minus_U; /* Lu(0-) / Ed(0-) */
    double Kd_0minus, Ku_0minus;                     /* diffuse attenuation of the first water layer [1/m] */
    double tau_water, depth_water_m;                 /* optical and physical depth of the water column */
    int    n_layers_water, n_ring_water;             /* water layers; water directions (Gauss + zero-weight) */
    int    orders_water, converged_water;            /* max orders over modes; AND over modes */
} ocrt_ocean_result;

/* Defaults of rt_water_rt_options_default (rt_water_rt.c:1340-1410) and of a
 * pure-seawater column with no hydrosol (a_total and b_water left 0). */
void ocrt_ocean_default(ocrt_ocean *oc);
int  ocrt_gb_solve_ocean(const ocrt_case *cs, const ocrt_opts *opts, const ocrt_aerosol *aer,
                         const ocrt_ocean *oc, ocrt_result *out, ocrt_ocean_result *wout);
/* n coupled pixels in one device pass; opts / aer / oc shared or per case. */
int  ocrt_gb_solve_batch_ocean(int n, const ocrt_case *cases,
                               const ocrt_opts *opts, int opts_per_case,
                               const ocrt_aerosol *aer, int aer_per_case,
                               const ocrt_ocean *oc, int oc_per_case,
                               ocrt_result *out, ocrt_ocean_result *wout, void *stream);

int ocrt_gb_solve_batch_adjoint(int n, const ocrt_case *cases,
                                const ocrt_opts *opts, int opts_per_case,
                                const ocrt_aerosol *aer, int aer_per_case,
                                const ocrt_layers *layers, int n_cot, const double *cot,
                                ocrt_result *out, ocrt_grad *grad, void *stream);

/* Resident-plan form of the adjoint: a plan that carries layer parameters and
 * n_cot cotangent rows per pixel.  ocrt_gb_plan_execute then runs the forward
 * and the adjoint sweeps, ocrt_gb_plan_results gives the forward results and
 * ocrt_gb_plan_gradients the gradients (layout as ocrt_gb_solve_batch_adjoint);
 * ocrt_gb_plan_kernel_stats covers the adjoint kernels too. */
int ocrt_gb_plan_create_adjoint(int n, const ocrt_case *cases,
                                const ocrt_opts *opts, int opts_per_case,
                                const ocrt_aerosol *aer, int aer_per_case,
                                const ocrt_layers *layers, int n_cot, const double *cot,
                                ocrt_plan **plan);
int ocrt_gb_plan_gradients(ocrt_plan *plan, ocrt_grad *grad, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* OCRT_GB300_H */
