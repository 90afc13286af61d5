"""ctypes mirror of include/ocrt_gb300.h.

The structures below must stay field-for-field identical to the C header;
tests/test_abi.py checks the sizes against the compiled library.
"""
import ctypes as C

OCRT_OK = 0
OCRT_ERR_ARGS = -1
OCRT_ERR_NONFINITE = -2
OCRT_ERR_ALLOC = -3
OCRT_ERR_DEVICE = -4
OCRT_ERR_UNSUPPORTED = -5
OCRT_ERR_BOTTOM_SOURCE_SHAPE = -7

SURFACE_BLACK = 0
SURFACE_LAMBERT = 1
SURFACE_BLACK_FRESNEL_OCEAN = 2
SURFACE_FLAT = 3
SURFACE_OCEAN = 4

SURFACE_NAMES = {
    "black": SURFACE_BLACK,
    "lambert": SURFACE_LAMBERT,
    "black_fresnel_ocean": SURFACE_BLACK_FRESNEL_OCEAN,
    "coxmunk": SURFACE_BLACK_FRESNEL_OCEAN,
    "flat": SURFACE_FLAT,
    "ocean": SURFACE_OCEAN,
}

TAU_R_AUTO = 0
TAU_R_FROM_INPUT = 1
PROFILE_US62 = 0
PROFILE_EXPONENTIAL = 1


class Case(C.Structure):
    _fields_ = [
        ("sza_deg", C.c_double), ("vza_deg", C.c_double), ("raa_deg", C.c_double),
        ("wavelength_nm", C.c_double), ("surface", C.c_int), ("pressure_hpa", C.c_double),
        ("tau_r_input", C.c_double), ("n_water", C.c_double), ("wind_speed", C.c_double),
        ("sigma_type", C.c_int), ("q_convention", C.c_int), ("decouple_sunglint", C.c_int),
    ]


class Opts(C.Structure):
    _fields_ = [
        ("n_mu", C.c_int), ("n_layers", C.c_int), ("fourier_m_max", C.c_int),
        ("max_orders", C.c_int), ("tolerance", C.c_double), ("tau_r_source", C.c_int),
        ("pssa", C.c_int), ("view_as_node", C.c_int), ("aer_h_km", C.c_double),
        ("rayleigh_profile", C.c_int), ("rayleigh_h_km", C.c_double),
        ("n_phi_surface", C.c_int), ("gas", C.c_void_p),
    ]


class Aerosol(C.Structure):
    _fields_ = [
        ("tau_a", C.c_double), ("ssa_a", C.c_double), ("L_max", C.c_int),
        ("beta", C.POINTER(C.c_double)), ("gamma", C.POINTER(C.c_double)),
        ("alpha", C.POINTER(C.c_double)), ("zeta", C.POINTER(C.c_double)),
        ("use_value_kernel", C.c_int), ("n_ang_phase", C.c_int),
        ("theta_phase", C.POINTER(C.c_double)), ("P11_phase", C.POINTER(C.c_double)),
        ("P12_phase", C.POINTER(C.c_double)), ("P33_phase", C.POINTER(C.c_double)),
    ]


class MieOpts(C.Structure):
    _fields_ = [("L_max", C.c_int), ("use_loglin_trunc", C.c_int), ("loglin_mu1", C.c_double),
                ("loglin_mu2", C.c_double), ("loglin_threshold", C.c_double), ("use_value_kernel", C.c_int)]


class MieDiag(C.Structure):
    _fields_ = [(f, C.c_double) for f in ("aod_ref", "aod_ref_nm", "aod_target", "extinction_ratio", "ssa_raw",
                                          "trunc_A", "tau_a_eff", "ssa_a_eff")]


class Result(C.Structure):
    _fields_ = [
        ("rho_I", C.c_double), ("rho_Q", C.c_double), ("rho_U", C.c_double),
        ("I_TOA", C.c_double), ("Q_TOA", C.c_double), ("U_TOA", C.c_double),
        ("tau_R_total", C.c_double), ("n_orders_used", C.c_int), ("converged", C.c_int),
        ("order_modes", C.c_int), ("kappa_ipss", C.c_double),
        ("T_dir_dn", C.c_double), ("T_diff_dn_hemi", C.c_double),
        ("T_total_dn_hemi", C.c_double), ("T_diff_dn_dir", C.c_double),
        ("T_total_up_dir", C.c_double), ("T_sg_up_dir", C.c_double),
        ("T_dir_up_view", C.c_double),
        ("rho_glint_direct_I", C.c_double), ("rho_glint_direct_Q", C.c_double),
        ("rho_glint_direct_U", C.c_double),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("orders_per_m", C.POINTER(C.c_int)), ("residual_per_m", C.POINTER(C.c_double)),
        ("view_I_m", C.POINTER(C.c_double)), ("view_Q_m", C.POINTER(C.c_double)),
        ("view_U_m", C.POINTER(C.c_double)),
    ]


class Layers(C.Structure):
    _fields_ = [("n_layers", C.c_int), ("dtau", C.POINTER(C.c_double)), ("ssa", C.POINTER(C.c_double))]


class Grad(C.Structure):
    _fields_ = [("d_dtau", C.POINTER(C.c_double)), ("d_ssa", C.POINTER(C.c_double)), ("d_wind", C.c_double)]


class LayersHolder:
    """Keeps per-layer override arrays alive while a Layers struct points into them."""

    def __init__(self, n_layers, dtau=None, ssa=None):
        import numpy as np
        self.dtau = None if dtau is None else np.ascontiguousarray(np.asarray(dtau, dtype=np.float64))
        self.ssa = None if ssa is None else np.ascontiguousarray(np.asarray(ssa, dtype=np.float64))
        for a in (self.dtau, self.ssa):
            if a is not None and a.shape != (n_layers,):
                raise ValueError("per-layer array length differs from n_layers")
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None
        self.struct = Layers(n_layers=int(n_layers), dtau=ptr(self.dtau), ssa=ptr(self.ssa))


class Lut(C.Structure):
    _fields_ = [("n_vza", C.c_int), ("vza_deg", C.POINTER(C.c_double)),
                ("n_raa", C.c_int), ("raa_deg", C.POINTER(C.c_double)),
                ("rho_I", C.POINTER(C.c_double)), ("rho_Q", C.POINTER(C.c_double)),
                ("rho_U", C.POINTER(C.c_double)), ("T_diff_dn_dir", C.POINTER(C.c_double)),
                ("T_sg_up_dir", C.POINTER(C.c_double)), ("T_total_up_dir", C.POINTER(C.c_double)),
                ("T_dir_dn", C.c_double), ("T_diff_dn_hemi", C.c_double)]


LUT_FIELDS = ("rho_I", "rho_Q", "rho_U", "T_diff_dn_dir", "T_sg_up_dir", "T_total_up_dir")


class LutHolder:
    """A (vza, raa) grid and its caller-owned output arrays (numpy), bound to a Lut struct."""

    def __init__(self, vza_deg, raa_deg):
        import numpy as np
        self.vza = np.ascontiguousarray(np.asarray(vza_deg, dtype=np.float64))
        self.raa = np.ascontiguousarray(np.asarray(raa_deg, dtype=np.float64))
        n = self.vza.size * self.raa.size
        self.out = {k: np.zeros(n) for k in LUT_FIELDS}
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.struct = Lut(n_vza=self.vza.size, vza_deg=P(self.vza), n_raa=self.raa.size, raa_deg=P(self.raa),
                          **{k: P(v) for k, v in self.out.items()}, T_dir_dn=0.0, T_diff_dn_hemi=0.0)

    def grid(self, key):
        return self.out[key].reshape(self.vza.size, self.raa.size)


def lut_grid_reference_cli(vza_step=2.5, raa_step=2.5, vza_max=85.0):
    """The grid of the reference CLI's LUT mode (main.c:3794-3804)."""
    import numpy as np
    n_vza = int(vza_max / vza_step) + 1
    n_raa = int(360.0 / raa_step)
    return np.arange(n_vza) * vza_step, np.arange(n_raa) * raa_step


RESULT_FIELDS = [f for f, _ in Result._fields_]


def default_case(**kw):
    """CLI defaults of the reference (main.c:1826-1840)."""
    c = Case(sza_deg=40.0, vza_deg=30.0, raa_deg=90.0, wavelength_nm=555.0,
             surface=SURFACE_BLACK, pressure_hpa=1013.25, tau_r_input=0.0, n_water=1.34,
             wind_speed=0.0, sigma_type=1, q_convention=1, decouple_sunglint=0)
    for k, v in kw.items():
        if k == "surface" and isinstance(v, str):
            v = SURFACE_NAMES[v]
        setattr(c, k, v)
    return c


def default_opts(**kw):
    """rt_options_default() (rt_types.h:760-795)."""
    o = Opts(n_mu=24, n_layers=40, fourier_m_max=2, max_orders=20, tolerance=1e-7,
             tau_r_source=TAU_R_AUTO, pssa=0, view_as_node=1, aer_h_km=2.0,
             rayleigh_profile=PROFILE_US62, rayleigh_h_km=8.0, n_phi_surface=1024)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class AerosolHolder:
    """Keeps the moment arrays (and, for the value kernel, the phase table:
    ascending angles in degrees and P11, P12, P33) alive while an Aerosol
    struct points into them."""

    def __init__(self, tau_a, ssa_a, beta, gamma, alpha, zeta, phase=None, value_kernel=None):
        import numpy as np
        self.arrays = [np.ascontiguousarray(np.asarray(a, dtype=np.float64))
                       for a in (beta, gamma, alpha, zeta)]
        L = len(self.arrays[0]) - 1
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in self.arrays]
        self.struct = Aerosol(tau_a=float(tau_a), ssa_a=float(ssa_a), L_max=L,
                              beta=ptrs[0], gamma=ptrs[1], alpha=ptrs[2], zeta=ptrs[3])
        if phase is not None:
            self.phase = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in phase]
            pp = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in self.phase]
            self.struct.use_value_kernel = 1 if value_kernel is None else int(value_kernel)
            self.struct.n_ang_phase = len(self.phase[0])
            self.struct.theta_phase, self.struct.P11_phase, self.struct.P12_phase, self.struct.P33_phase = pp

    @property
    def L_max(self):
        return self.struct.L_max


def result_dict(r):
    return {f: getattr(r, f) for f in RESULT_FIELDS}


def bind_solver(lib, prefix):
    """Declare argtypes for <prefix>_solve_case / <prefix>_solve_batch."""
    f = getattr(lib, prefix + "_solve_case")
    f.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol), C.POINTER(Result),
                  C.POINTER(Diag)]
    f.restype = C.c_int
    return f


class Ocean(C.Structure):
    _fields_ = [
        ("a_total", C.c_double), ("b_water", C.c_double), ("b_particle", C.c_double),
        ("L_particle", C.c_int),
        ("beta", C.POINTER(C.c_double)), ("gamma", C.POINTER(C.c_double)),
        ("alpha", C.POINTER(C.c_double)), ("zeta", C.POINTER(C.c_double)),
        ("n_mu_water", C.c_int), ("m_max_water", C.c_int), ("max_orders_water", C.c_int),
        ("tolerance_water", C.c_double), ("n_layers_water", C.c_int), ("depth_m", C.c_double),
        ("tau_base", C.c_double), ("view_as_node", C.c_int),
    ]


class OceanResult(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "rho_atm_I", "rho_atm_Q", "rho_atm_U", "rho_water_I", "rho_water_Q", "rho_water_U",
        "Lu_0minus_I", "Lu_0minus_Q", "Lu_0minus_U", "Lu_0plus_I", "Lu_0plus_Q", "Lu_0plus_U",
        "Ed_0minus", "Eu_0minus", "Ed_0plus", "Ed_0minus_direct", "Ed_0plus_direct",
        "Rrs_0plus_I", "Rrs_0plus_Q", "Rrs_0plus_U", "rrs_0minus_I", "rrs_0minus_Q", "rrs_0minus_U",
        "Kd_0minus", "Ku_0minus", "tau_water", "depth_water_m")] + [
        (k, C.c_int) for k in ("n_layers_water", "n_ring_water", "orders_water", "converged_water")]


OCEAN_RESULT_FIELDS = [f for f, _ in OceanResult._fields_]


class OceanHolder:
    """A water column (ocrt_ocean) with its hydrosol moment arrays kept alive.

    a_total, b_water and b_particle in 1/m; moments (beta, gamma, alpha,
    zeta) of the hydrosol as for the aerosol, or None without a hydrosol.
    Remaining keywords set ocrt_ocean fields (n_mu_water, m_max_water, ...)."""

    def __init__(self, a_total, b_water, b_particle=0.0, moments=None, **kw):
        import numpy as np
        o = Ocean(a_total=float(a_total), b_water=float(b_water), b_particle=float(b_particle), L_particle=0,
                  n_mu_water=48, m_max_water=2, max_orders_water=20, tolerance_water=1e-7,
                  n_layers_water=0, depth_m=0.0, tau_base=20.0, view_as_node=1)
        self.arrays = []
        if moments is not None:
            self.arrays = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in moments]
            ptrs = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in self.arrays]
            o.L_particle = len(self.arrays[0]) - 1
            o.beta, o.gamma, o.alpha, o.zeta = ptrs
        for k, v in kw.items():
            setattr(o, k, v)
        self.struct = o


def ocean_result_dict(r):
    return {f: getattr(r, f) for f in OCEAN_RESULT_FIELDS}
