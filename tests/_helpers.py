"""Shared helpers: oracle binding, fixture loading and the parity tolerance.

Parity bar (the accuracy requirement of this path): |rho_I - ref| <= 1e-5 * |ref|,
|rho_Q - ref| <= 1e-4 and |rho_U - ref| <= 1e-4.
"""
import ctypes as C
import json
import os

import numpy as np

from ocrt_gb300 import _abi as A
from synthetic import hg_aerosol_moments

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_cases.json")

TOL_I_REL = 1e-5
TOL_QU_ABS = 1e-4


class Oracle:
    def __init__(self, path):
        self.lib = C.CDLL(path)
        self.f = A.bind_solver(self.lib, "ocrt_oracle")
        self.lib.ocrt_oracle_solve_batch.argtypes = [
            C.c_int, C.POINTER(A.Case), C.POINTER(A.Opts), C.c_int, C.POINTER(A.Aerosol), C.c_int,
            C.POINTER(A.Result), C.c_int]

        self.lib.ocrt_oracle_solve_case_layers.argtypes = [
            C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Layers), C.POINTER(A.Result),
            C.POINTER(A.Diag)]
        self.lib.ocrt_oracle_layer_defaults.argtypes = [
            C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(C.c_double),
            C.POINTER(C.c_double)]

        L = self.lib
        L.ocrt_oracle_gas_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(C.c_void_p)]
        L.ocrt_oracle_gas_destroy.argtypes = [C.c_void_p]
        L.ocrt_oracle_gas_destroy.restype = None
        L.ocrt_oracle_gas_tau.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ocrt_oracle_gas_columns.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_int)]
        L.ocrt_oracle_layer_gas.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double)]

    def gas_create(self, root, profile, override=None):
        """Oracle gas state on <root>/afgl_atm and <root>/xsec; returns the handle."""
        h = C.c_void_p()
        ov = (C.c_double * 6)(*override) if override is not None else None
        rc = self.lib.ocrt_oracle_gas_create(os.path.join(root, "afgl_atm").encode(),
                                             os.path.join(root, "xsec").encode(), profile, ov, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle gas rc {rc}")
        return h.value

    def gas_destroy(self, h):
        self.lib.ocrt_oracle_gas_destroy(h)

    def gas_tau(self, h, wl):
        per, tot = (C.c_double * 6)(), C.c_double()
        self.lib.ocrt_oracle_gas_tau(h, wl, per, C.byref(tot))
        return np.array(per[:]), tot.value

    def gas_columns(self, h):
        e, d, o = (C.c_double * 6)(), (C.c_double * 6)(), (C.c_int * 6)()
        self.lib.ocrt_oracle_gas_columns(h, e, d, o)
        return np.array(e[:]), np.array(d[:]), np.array(o[:])

    def layer_gas(self, case, opts, aer=None):
        n = opts.n_layers
        ta, z = np.zeros(n), np.zeros(n + 1)
        a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
        rc = self.lib.ocrt_oracle_layer_gas(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None,
                                            ta.ctypes.data_as(C.POINTER(C.c_double)),
                                            z.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise RuntimeError(f"oracle rc {rc}")
        return ta, z

    def layer_defaults(self, case, opts, aer=None):
        n = opts.n_layers
        dt, ss = np.zeros(n), np.zeros(n)
        a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
        rc = self.lib.ocrt_oracle_layer_defaults(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None,
                                                 dt.ctypes.data_as(C.POINTER(C.c_double)),
                                                 ss.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise RuntimeError(f"oracle rc {rc}")
        return dt, ss

    def solve_layers(self, case, opts, aer=None, dtau=None, ssa=None):
        ly = A.LayersHolder(opts.n_layers, dtau, ssa)
        r = A.Result()
        a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
        rc = self.lib.ocrt_oracle_solve_case_layers(C.byref(case), C.byref(opts),
                                                    C.byref(a) if a is not None else None,
                                                    C.byref(ly.struct), C.byref(r), None)
        if rc != 0:
            raise RuntimeError(f"oracle rc {rc}")
        return A.result_dict(r)

    def solve(self, case, opts, aer=None, diag=False):
        n = opts.fourier_m_max + 1
        arr = None
        d = None
        if diag:
            arr = {"orders_per_m": (C.c_int * n)(), "residual_per_m": (C.c_double * n)(),
                   "view_I_m": (C.c_double * n)(), "view_Q_m": (C.c_double * n)(),
                   "view_U_m": (C.c_double * n)()}
            d = A.Diag(**{k: C.cast(v, A.Diag._fields_[i][1]) for i, (k, v) in enumerate(arr.items())})
        r = A.Result()
        a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
        rc = self.f(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None, C.byref(r),
                    C.byref(d) if d is not None else None)
        if rc != 0:
            raise RuntimeError(f"oracle rc {rc}")
        out = A.result_dict(r)
        if diag:
            out.update({k: np.array(v[:]) for k, v in arr.items()})
        return out


GAS_DATA = os.path.join(HERE, "golden", "gas_data")
GAS_PROFILES = {"usstd76": 0, "tropical": 1, "mlwint": 3}


def load_gas_golden():
    with open(os.path.join(HERE, "golden", "reference_gas.json")) as fh:
        return json.load(fh)


def gas_solve_inputs(spec):
    """(case, opts, aerosol holder or None) of one gas fixture solve; opts.gas unset."""
    c = A.default_case(**spec["case"])
    o = A.default_opts(**spec["opts"])
    af = spec["aerosol"]
    aer = A.AerosolHolder(af["tau_a"], af["ssa_a"], *hg_aerosol_moments(af["g"], af["L"])) if af else None
    return c, o, aer


def load_golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def inputs_from_spec(spec):
    c = A.default_case(**spec["case"])
    o = A.default_opts(**spec["opts"])
    aer = None
    if spec.get("aerosol"):
        a = spec["aerosol"]
        aer = A.AerosolHolder(a["tau_a"], a["ssa_a"], *hg_aerosol_moments(a["g"], a["L"]))
    return c, o, aer


def assert_parity(got, ref, where="", i_rel=TOL_I_REL, qu_abs=TOL_QU_ABS):
    relI = abs(got["rho_I"] - ref["rho_I"]) / abs(ref["rho_I"])
    dQ = abs(got["rho_Q"] - ref["rho_Q"])
    dU = abs(got["rho_U"] - ref["rho_U"])
    assert relI <= i_rel, f"{where}: rho_I rel err {relI:.3e} > {i_rel}"
    assert dQ <= qu_abs, f"{where}: rho_Q abs err {dQ:.3e} > {qu_abs}"
    assert dU <= qu_abs, f"{where}: rho_U abs err {dU:.3e} > {qu_abs}"
    return relI, dQ, dU


def rho_vec(r):
    return np.array([r["rho_I"], r["rho_Q"], r["rho_U"]])


def fd_gradient(orc, case, opts, aer, dtau, ssa, cot, which, rel_step=1e-6):
    """FP64 central finite differences of cot . (rho_I, rho_Q, rho_U) on the
    oracle with a fixed order count.  which: list of ("dtau", l), ("ssa", l) or
    ("wind", None); the step is rel_step times the parameter value."""
    import copy
    out = []

    def f(kind, l, delta):
        dt, ss, cs = dtau.copy(), ssa.copy(), copy.copy(case)
        if kind == "dtau":
            dt[l] += delta
        elif kind == "ssa":
            ss[l] += delta
        else:
            cs.wind_speed = case.wind_speed + delta
        return float(np.dot(cot, rho_vec(orc.solve_layers(cs, opts, aer, dt, ss))))

    for kind, l in which:
        x = dtau[l] if kind == "dtau" else (ssa[l] if kind == "ssa" else case.wind_speed)
        h = rel_step * x
        if kind == "ssa" and x + h > 1.0:
            # albedo at its upper bound: second-order one-sided difference
            out.append((3.0 * f(kind, l, 0.0) - 4.0 * f(kind, l, -h) + f(kind, l, -2.0 * h)) / (2.0 * h))
        else:
            out.append((f(kind, l, h) - f(kind, l, -h)) / (2.0 * h))
    return np.array(out)


GOLDEN_LUT = os.path.join(HERE, "golden", "reference_lut.json")


def load_golden_lut():
    with open(GOLDEN_LUT) as fh:
        return json.load(fh)


def oracle_lut(orc, case, opts, aer, vza, raa):
    lut = A.LutHolder(vza, raa)
    f = orc.lib.ocrt_oracle_solve_case_lut
    f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Result),
                  C.POINTER(A.Lut)]
    a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
    r = A.Result()
    rc = f(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None, C.byref(r), C.byref(lut.struct))
    if rc != 0:
        raise RuntimeError(f"oracle lut rc {rc}")
    return lut


GOLDEN_OCEAN = os.path.join(HERE, "golden", "reference_ocean.json")

# reference CLI key -> (ocrt_result / ocrt_ocean_result key, relative tolerance of the
# oracle's reproduction, set by the printed precision); Kd / Ku are printed to 1e-6 absolute
OCEAN_RADIOMETRIC = ("Lu0plus", "Qu0plus", "Uu0plus", "Ed0plus", "Lu0minus", "Qu0minus", "Uu0minus", "Ed0minus",
                     "Eu0minus")
REF_OCEAN_KEYS = {
    "TOA_rho_I": ("rho_I", 1e-9), "TOA_rho_Q": ("rho_Q", 1e-9), "TOA_rho_U": ("rho_U", 1e-9),
    "TOA_rho_atm_I": ("rho_atm_I", 1e-9), "TOA_rho_atm_Q": ("rho_atm_Q", 1e-9), "TOA_rho_atm_U": ("rho_atm_U", 1e-9),
    "TOA_rho_water_direct_I": ("rho_water_I", 1e-9), "TOA_rho_water_direct_Q": ("rho_water_Q", 1e-9),
    "TOA_rho_water_direct_U": ("rho_water_U", 1e-9),
    "TOA_rho_glint_direct_I": ("rho_glint_direct_I", 1e-9),
    "T_dir_dn": ("T_dir_dn", 1e-9), "T_diff_dn_hemi": ("T_diff_dn_hemi", 1e-9), "T_diff_dn_dir": ("T_diff_dn_dir", 1e-9),
    "Lu0plus": ("Lu_0plus_I", 1e-6), "Qu0plus": ("Lu_0plus_Q", 1e-6), "Uu0plus": ("Lu_0plus_U", 1e-6),
    "Ed0plus": ("Ed_0plus", 1e-6), "Rrs0plus_I": ("Rrs_0plus_I", 1e-6), "Rrs0plus_Q": ("Rrs_0plus_Q", 1e-6),
    "Rrs0plus_U": ("Rrs_0plus_U", 1e-6),
    "Lu0minus": ("Lu_0minus_I", 1e-6), "Qu0minus": ("Lu_0minus_Q", 1e-6), "Uu0minus": ("Lu_0minus_U", 1e-6),
    "Ed0minus": ("Ed_0minus", 1e-6), "Eu0minus": ("Eu_0minus", 1e-6), "rrs0minus_I": ("rrs_0minus_I", 1e-6),
    "Kd0minus": ("Kd_0minus", 1e-5), "Ku0minus": ("Ku_0minus", 1e-5),
}


def ocean_ref_value(spec, key):
    """Reference value of a key in this library's units (F_sun = pi): the
    reference's constituent-model path reports radiances and irradiances for
    F_sun = 1."""
    v = spec["reference"][key]
    return v * (3.141592653589793 / spec["F_sun"]) if key in OCEAN_RADIOMETRIC else v


def load_golden_ocean():
    with open(GOLDEN_OCEAN) as fh:
        return json.load(fh)


def ocean_inputs_from_spec(spec, **ocean_kw):
    """(case, opts, OceanHolder) of one reference_ocean.json case: the water's
    absorption and scattering are the values the reference printed."""
    ref = spec["reference"]
    c = A.default_case(surface="ocean", sza_deg=spec["sza_deg"], vza_deg=spec["vza_deg"], raa_deg=spec["raa_deg"],
                       wavelength_nm=spec["wavelength_nm"], wind_speed=spec["wind_speed"])
    m = spec["m_max"] if spec["m_max"] is not None else 2
    o = A.default_opts(fourier_m_max=m, n_layers=spec["n_layers"] or 40)
    kw = dict(n_mu_water=spec["n_mu_water"] or 48, m_max_water=m)
    kw.update(spec.get("water_policy", {}))
    kw.update(ocean_kw)
    oc = A.OceanHolder(ref["a_total"], ref["b_total"], **kw)
    return c, o, oc


def oracle_ocean(orc, case, opts, oc, aer=None):
    f = orc.lib.ocrt_oracle_solve_ocean
    f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Ocean),
                  C.POINTER(A.Result), C.POINTER(A.OceanResult)]
    r, w = A.Result(), A.OceanResult()
    a = aer.struct if isinstance(aer, A.AerosolHolder) else aer
    rc = f(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None, C.byref(oc.struct), C.byref(r),
           C.byref(w))
    if rc != 0:
        raise RuntimeError(f"oracle ocean rc {rc}")
    return {**A.result_dict(r), **A.ocean_result_dict(w)}
