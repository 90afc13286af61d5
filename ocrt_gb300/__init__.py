"""GB300 successive-orders-of-scattering vector radiative-transfer solver.

Python face of the C-ABI library ``libocrt_gb300.so`` (include/ocrt_gb300.h).
Every solve runs in the CUDA library; there is no CPU fallback: if the shared
library is missing or no CUDA device is present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import (Aerosol, AerosolHolder, Case, Diag, Grad, Layers, LayersHolder, Lut, LutHolder, MieDiag, MieOpts,
                   Ocean, OceanHolder,
                   OceanResult, Opts, Result, default_case, default_opts, lut_grid_reference_cli, ocean_result_dict,
                   result_dict, RESULT_FIELDS)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libocrt_gb300.so")
_lib = None

EXPORTS = [
    "ocrt_opts_default", "ocrt_case_default", "ocrt_gb_init", "ocrt_gb_shutdown", "ocrt_gb_last_error",
    "ocrt_gb_solve_case", "ocrt_gb_solve_batch", "ocrt_gb_plan_create", "ocrt_gb_plan_execute",
    "ocrt_gb_plan_results", "ocrt_gb_plan_stats", "ocrt_gb_plan_destroy", "ocrt_gb_set_timing",
    "ocrt_gb_plan_kernel_stats", "ocrt_gb_solve_case_noalloc", "ocrt_gb_solve_batch_adjoint",
    "ocrt_gb_layer_defaults", "ocrt_gb_plan_create_adjoint", "ocrt_gb_plan_gradients",
    "ocrt_gb_solve_case_lut", "ocrt_gb_solve_batch_lut", "ocrt_gb_plan_graph_ready", "ocrt_gb_autotune_summary",
    "ocrt_gb_gas_create", "ocrt_gb_gas_destroy", "ocrt_gb_gas_tau", "ocrt_gb_gas_columns", "ocrt_gb_layer_gas",
    "ocrt_ocean_default", "ocrt_gb_solve_ocean", "ocrt_gb_solve_batch_ocean",
    "ocrt_mie_opts_default", "ocrt_gb_mie_read", "ocrt_gb_mie_free", "ocrt_gb_mie_shape", "ocrt_gb_mie_prepare",
    "ocrt_gb_mie_aerosol_free",
]


class OcrtError(RuntimeError):
    def __init__(self, rc, msg):
        super().__init__(f"ocrt error {rc}: {msg}")
        self.rc = rc


def lib():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OcrtError(_abi.OCRT_ERR_DEVICE,
                        f"{LIB_PATH} not built; run python -m ocrt_gb300.build")
    L = C.CDLL(LIB_PATH)
    L.ocrt_gb_init.argtypes = [C.c_int]
    L.ocrt_gb_last_error.restype = C.c_char_p
    L.ocrt_gb_solve_case.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol),
                                     C.POINTER(Result), C.POINTER(Diag)]
    L.ocrt_gb_solve_batch.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int,
                                      C.POINTER(Aerosol), C.c_int, C.POINTER(Result), C.c_void_p]
    L.ocrt_gb_plan_create.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int,
                                      C.POINTER(Aerosol), C.c_int, C.POINTER(C.c_void_p)]
    L.ocrt_gb_plan_execute.argtypes = [C.c_void_p, C.c_void_p]
    L.ocrt_gb_plan_results.argtypes = [C.c_void_p, C.POINTER(Result), C.c_void_p]
    L.ocrt_gb_plan_stats.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.ocrt_gb_plan_destroy.argtypes = [C.c_void_p]
    L.ocrt_gb_set_timing.argtypes = [C.c_int]
    L.ocrt_gb_plan_kernel_stats.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                            C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
    L.ocrt_gb_solve_batch_adjoint.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int,
                                              C.POINTER(Aerosol), C.c_int, C.POINTER(Layers), C.c_int,
                                              C.POINTER(C.c_double), C.POINTER(Result), C.POINTER(Grad), C.c_void_p]
    L.ocrt_gb_plan_create_adjoint.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int,
                                              C.POINTER(Aerosol), C.c_int, C.POINTER(Layers), C.c_int,
                                              C.POINTER(C.c_double), C.POINTER(C.c_void_p)]
    L.ocrt_gb_plan_gradients.argtypes = [C.c_void_p, C.POINTER(Grad), C.c_void_p]
    L.ocrt_gb_layer_defaults.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ocrt_gb_solve_case_lut.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol), C.POINTER(Result),
                                         C.POINTER(Lut)]
    L.ocrt_gb_solve_batch_lut.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int, C.POINTER(Aerosol),
                                          C.c_int, C.POINTER(Lut), C.POINTER(Result), C.c_void_p]
    L.ocrt_gb_plan_graph_ready.argtypes = [C.c_void_p]
    L.ocrt_gb_autotune_summary.argtypes = [C.c_char_p, C.c_int]
    L.ocrt_gb_gas_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_void_p)]
    L.ocrt_gb_gas_destroy.argtypes = [C.c_void_p]
    L.ocrt_gb_gas_destroy.restype = None
    L.ocrt_gb_gas_tau.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ocrt_gb_gas_columns.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int)]
    L.ocrt_gb_layer_gas.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ocrt_opts_default.argtypes = [C.POINTER(Opts)]
    L.ocrt_case_default.argtypes = [C.POINTER(Case)]
    L.ocrt_ocean_default.argtypes = [C.POINTER(Ocean)]
    L.ocrt_gb_solve_ocean.argtypes = [C.POINTER(Case), C.POINTER(Opts), C.POINTER(Aerosol), C.POINTER(Ocean),
                                      C.POINTER(Result), C.POINTER(OceanResult)]
    L.ocrt_gb_solve_batch_ocean.argtypes = [C.c_int, C.POINTER(Case), C.POINTER(Opts), C.c_int, C.POINTER(Aerosol),
                                            C.c_int, C.POINTER(Ocean), C.c_int, C.POINTER(Result),
                                            C.POINTER(OceanResult), C.c_void_p]
    L.ocrt_mie_opts_default.argtypes = [C.POINTER(MieOpts)]
    L.ocrt_mie_opts_default.restype = None
    L.ocrt_gb_mie_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.ocrt_gb_mie_free.argtypes = [C.c_void_p]
    L.ocrt_gb_mie_free.restype = None
    L.ocrt_gb_mie_shape.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.ocrt_gb_mie_prepare.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(MieOpts),
                                      C.POINTER(C.c_void_p), C.POINTER(Aerosol), C.POINTER(MieDiag)]
    L.ocrt_gb_mie_aerosol_free.argtypes = [C.c_void_p]
    L.ocrt_gb_mie_aerosol_free.restype = None
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise OcrtError(rc, lib().ocrt_gb_last_error().decode())


def solve_case(case, opts=None, aerosol=None, diag=False):
    """One pixel; returns a dict of ocrt_result fields (plus per-mode arrays if diag)."""
    L = lib()
    opts = opts or default_opts()
    r = Result()
    d = None
    arrs = None
    if diag:
        n = opts.fourier_m_max + 1
        arrs = {"orders_per_m": (C.c_int * n)(), "residual_per_m": (C.c_double * n)(),
                "view_I_m": (C.c_double * n)(), "view_Q_m": (C.c_double * n)(),
                "view_U_m": (C.c_double * n)()}
        d = Diag(**{k: C.cast(v, Diag._fields_[i][1]) for i, (k, v) in enumerate(arrs.items())})
    a = aerosol.struct if hasattr(aerosol, "struct") else aerosol
    _check(L.ocrt_gb_solve_case(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None,
                                C.byref(r), C.byref(d) if d is not None else None))
    out = result_dict(r)
    if diag:
        out.update({k: np.array(v[:]) for k, v in arrs.items()})
    return out


def solve_ocean(case, opts=None, ocean=None, aerosol=None):
    """One coupled atmosphere-ocean pixel (ocrt_gb_solve_ocean): a dict of
    the ocrt_result and ocrt_ocean_result fields.  ocean: an OceanHolder."""
    res = solve_batch_ocean([case], opts, [ocean], None if aerosol is None else [aerosol])
    return res[0]


def solve_batch_ocean(cases, opts, oceans, aerosols=None):
    """n coupled pixels in one device pass (ocrt_gb_solve_batch_ocean); a list
    of dicts of the ocrt_result and ocrt_ocean_result fields."""
    L = lib()
    opts = opts or default_opts()
    n, ca, oa, opp, aa, app = _arrays(cases, opts, aerosols)
    structs = [o.struct if isinstance(o, OceanHolder) else o for o in oceans]
    ocs = (Ocean * len(structs))(*structs)
    r = (Result * n)()
    w = (OceanResult * n)()
    _check(L.ocrt_gb_solve_batch_ocean(n, ca, oa, opp, aa, app, ocs, 1 if len(structs) > 1 else 0, r, w, None))
    return [{**result_dict(r[i]), **ocean_result_dict(w[i])} for i in range(n)]


def _arrays(cases, opts, aerosols):
    n = len(cases)
    ca = (Case * n)(*cases)
    if isinstance(opts, (list, tuple)):
        oa, opp = (Opts * n)(*opts), 1
    else:
        oa, opp = (Opts * 1)(opts), 0
    if aerosols is None:
        aa, app = None, 0
    elif isinstance(aerosols, (list, tuple)):
        structs = [a.struct if hasattr(a, "struct") else a for a in aerosols]
        aa, app = (Aerosol * n)(*structs), 1
    else:
        s = aerosols.struct if hasattr(aerosols, "struct") else aerosols
        aa, app = (Aerosol * 1)(s), 0
    return n, ca, oa, opp, aa, app


def solve_batch(cases, opts, aerosols=None):
    """n pixels in one device pass; returns a numpy structured view of ocrt_result."""
    L = lib()
    n, ca, oa, opp, aa, app = _arrays(cases, opts, aerosols)
    out = (Result * n)()
    _check(L.ocrt_gb_solve_batch(n, ca, oa, opp, aa, app, out, None))
    return results_to_numpy(out)


def layer_defaults(case, opts, aerosol=None):
    """Profile values (dtau[nt], ssa[nt]) of the per-layer parameters of one case."""
    L = lib()
    n = opts.n_layers
    dt, ss = np.zeros(n), np.zeros(n)
    a = aerosol.struct if hasattr(aerosol, "struct") else aerosol
    _check(L.ocrt_gb_layer_defaults(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None,
                                    dt.ctypes.data_as(C.POINTER(C.c_double)),
                                    ss.ctypes.data_as(C.POINTER(C.c_double))))
    return dt, ss


AFGL_PROFILES = ("usstd76", "tropical", "mlsumm", "mlwint", "sasumm", "sawint", "userdef")
GASES = ("h2o", "o3", "o2", "co2", "no2", "ch4")


class GasState:
    """Trace-gas absorption state (rt_absorption_t): an AFGL atmosphere and
    the six cross-section tables, resident on the device.  Set
    ``opts.gas = state.handle`` to make a solve gas-loaded; keep the object
    alive while any solve or plan uses it."""

    def __init__(self, afgl_dir, xsec_dir, profile="usstd76", column_override=None):
        L = lib()
        prof = AFGL_PROFILES.index(profile) if isinstance(profile, str) else int(profile)
        ov = None
        if column_override is not None:
            vals = [-1.0] * 6
            if isinstance(column_override, dict):
                for k, v in column_override.items():
                    vals[GASES.index(k)] = float(v)
            else:
                vals = [float(v) for v in column_override]
            ov = (C.c_double * 6)(*vals)
        h = C.c_void_p()
        _check(L.ocrt_gb_gas_create(os.fsencode(afgl_dir), os.fsencode(xsec_dir), prof, ov, C.byref(h)))
        self.handle = h.value

    def tau(self, wavelength_nm):
        """(per-gas column absorption depths [6], total) at one wavelength."""
        per, tot = (C.c_double * 6)(), C.c_double()
        _check(lib().ocrt_gb_gas_tau(self.handle, wavelength_nm, per, C.byref(tot)))
        return np.array(per[:]), tot.value

    def columns(self):
        """(effective columns [6], AFGL default columns [6], overridden [6])."""
        e, d, o = (C.c_double * 6)(), (C.c_double * 6)(), (C.c_int * 6)()
        _check(lib().ocrt_gb_gas_columns(self.handle, e, d, o))
        return np.array(e[:]), np.array(d[:]), np.array(o[:], dtype=bool)

    def close(self):
        if getattr(self, "handle", None):
            lib().ocrt_gb_gas_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def layer_gas(case, opts, aerosol=None):
    """(tau_abs[nt], z_km[nt+1]): the per-layer gas absorption depths a solve
    of this case applies and its level altitudes (level 0 = TOA)."""
    L = lib()
    n = opts.n_layers
    ta, z = np.zeros(n), np.zeros(n + 1)
    a = aerosol.struct if hasattr(aerosol, "struct") else aerosol
    _check(L.ocrt_gb_layer_gas(C.byref(case), C.byref(opts), C.byref(a) if a is not None else None,
                               ta.ctypes.data_as(C.POINTER(C.c_double)), z.ctypes.data_as(C.POINTER(C.c_double))))
    return ta, z


def _layers_array(n, opts, layers):
    if layers is None:
        return None
    structs = []
    for i, ly in enumerate(layers):
        nl = (opts[i] if isinstance(opts, (list, tuple)) else opts).n_layers
        structs.append(ly.struct if ly is not None else Layers(n_layers=nl, dtau=None, ssa=None))
    return (Layers * n)(*structs)


def _collect_grads(n, ncot, nts, call):
    ntm = max(nts)
    bufs = []
    ga = (Grad * (n * ncot))()
    for i in range(n):
        for r in range(ncot):
            a, b = np.zeros(nts[i]), np.zeros(nts[i])
            bufs.append((i, r, a, b))
            ga[i * ncot + r].d_dtau = a.ctypes.data_as(C.POINTER(C.c_double))
            ga[i * ncot + r].d_ssa = b.ctypes.data_as(C.POINTER(C.c_double))
    _check(call(ga))
    d_dtau = np.zeros((n, ncot, ntm))
    d_ssa = np.zeros((n, ncot, ntm))
    d_wind = np.zeros((n, ncot))
    for i, r, a, b in bufs:
        d_dtau[i, r, :nts[i]] = a
        d_ssa[i, r, :nts[i]] = b
        d_wind[i, r] = ga[i * ncot + r].d_wind
    return {"d_dtau": d_dtau, "d_ssa": d_ssa, "d_wind": d_wind}


def solve_batch_adjoint(cases, opts, aerosols=None, layers=None, cot=None):
    """Batched forward solve with per-layer parameters and gradients.

    layers: None or a list (one per case) of LayersHolder / None.
    cot: None (forward only) or an array [n, n_cot, 3] of cotangent rows for
    (rho_I, rho_Q, rho_U); n_cot = 3 with identity rows gives the Jacobian.
    Returns (results, grads) with grads a dict of arrays
    d_dtau [n, n_cot, nt], d_ssa [n, n_cot, nt], d_wind [n, n_cot] (None if cot is None).
    """
    L = lib()
    n, ca, oa, opp, aa, app = _arrays(cases, opts, aerosols)
    la = _layers_array(n, opts, layers)
    out = (Result * n)()
    if cot is None:
        _check(L.ocrt_gb_solve_batch_adjoint(n, ca, oa, opp, aa, app, la, 0, None, out, None, None))
        return results_to_numpy(out), None
    cot = np.ascontiguousarray(np.asarray(cot, dtype=np.float64))
    if cot.ndim != 3 or cot.shape[0] != n or cot.shape[2] != 3:
        raise ValueError("cot must have shape [n, n_cot, 3]")
    ncot = cot.shape[1]
    nts = [(opts[i] if isinstance(opts, (list, tuple)) else opts).n_layers for i in range(n)]
    cp = cot.ctypes.data_as(C.POINTER(C.c_double))
    grads = _collect_grads(n, ncot, nts,
                           lambda ga: L.ocrt_gb_solve_batch_adjoint(n, ca, oa, opp, aa, app, la, ncot, cp, out, ga,
                                                                    None))
    return results_to_numpy(out), grads


def solve_batch_lut(cases, opts, aerosols, luts):
    """Angle-grid LUT for n cases in one device pass; luts: one LutHolder per
    case (its output arrays are filled).  Returns the per-case results."""
    L = lib()
    n, ca, oa, opp, aa, app = _arrays(cases, opts, aerosols)
    la = (Lut * n)(*[x.struct for x in luts])
    out = (Result * n)()
    _check(L.ocrt_gb_solve_batch_lut(n, ca, oa, opp, aa, app, la, out, None))
    for i, x in enumerate(luts):
        x.struct.T_dir_dn, x.struct.T_diff_dn_hemi = la[i].T_dir_dn, la[i].T_diff_dn_hemi
    return results_to_numpy(out)


def solve_case_lut(case, opts, aerosol, lut):
    """Angle-grid LUT of one case (rt_solve_case_pol_lut); fills `lut` (a LutHolder)."""
    return solve_batch_lut([case], opts, [aerosol] if aerosol is not None else None, [lut])


def set_timing(enable):
    lib().ocrt_gb_set_timing(1 if enable else 0)


def autotune_summary():
    """Launch choices the autotuners picked, one dict per shape: block sizes of
    the setup kernels, and the transport-scan implementation (with its time
    per level-column in ns for each candidate)."""
    L = lib()
    n = L.ocrt_gb_autotune_summary(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.ocrt_gb_autotune_summary(buf, n + 1)
    out = []
    for line in buf.value.decode().splitlines():
        head, ms = line.split(" ms:")
        kern, key, best = head.split(" ")
        lab = lambda v: int(v) if v.lstrip("-").isdigit() else v   # noqa: E731 (block sizes or scan names)
        out.append({"kernel": kern, "key": [int(x) for x in key[4:].split(",")], "best": lab(best[5:]),
                    "ms": {lab(a): float(b) for a, b in (t.split("=") for t in ms.split())}})
    return out


def results_to_numpy(out):
    dt = np.dtype([(f, np.float64 if t is C.c_double else np.int32) for f, t in Result._fields_],
                  align=True)
    arr = np.frombuffer(out, dtype=dt, count=len(out)).copy()
    return arr


class Plan:
    """Device-resident batch: upload once, execute many times."""

    def __init__(self, cases, opts, aerosols=None, layers=None, cot=None):
        L = lib()
        self._keep = _arrays(cases, opts, aerosols)
        n, ca, oa, opp, aa, app = self._keep
        self.n = n
        self._h = C.c_void_p()
        self.ncot = 0
        if layers is None and cot is None:
            _check(L.ocrt_gb_plan_create(n, ca, oa, opp, aa, app, C.byref(self._h)))
            return
        la = _layers_array(n, opts, layers)
        self._nts = [(opts[i] if isinstance(opts, (list, tuple)) else opts).n_layers for i in range(n)]
        cp = None
        if cot is not None:
            self._cot = np.ascontiguousarray(np.asarray(cot, dtype=np.float64))
            if self._cot.ndim != 3 or self._cot.shape[0] != n or self._cot.shape[2] != 3:
                raise ValueError("cot must have shape [n, n_cot, 3]")
            self.ncot = self._cot.shape[1]
            cp = self._cot.ctypes.data_as(C.POINTER(C.c_double))
        self._la = la
        _check(L.ocrt_gb_plan_create_adjoint(n, ca, oa, opp, aa, app, la, self.ncot, cp, C.byref(self._h)))

    def gradients(self, stream=None):
        """d_dtau [n, n_cot, nt], d_ssa [n, n_cot, nt], d_wind [n, n_cot] of the last execute."""
        return _collect_grads(self.n, self.ncot, self._nts,
                              lambda ga: lib().ocrt_gb_plan_gradients(self._h, ga, stream))

    def execute(self, stream=None):
        _check(lib().ocrt_gb_plan_execute(self._h, stream))

    def results(self, stream=None):
        out = (Result * self.n)()
        _check(lib().ocrt_gb_plan_results(self._h, out, stream))
        return results_to_numpy(out)

    @property
    def graph_ready(self):
        """True when the next execute replays the captured CUDA graph."""
        return bool(lib().ocrt_gb_plan_graph_ready(self._h))

    def stats(self):
        om, nl = C.c_double(), C.c_longlong()
        _check(lib().ocrt_gb_plan_stats(self._h, C.byref(om), C.byref(nl)))
        return {"order_modes": om.value, "kernel_launches": nl.value}

    def kernel_stats(self):
        """Per kernel class: device ms of the last execute (timing must be on), launches,
        algorithmic FLOPs and bytes."""
        L = lib()
        n = L.ocrt_gb_plan_kernel_stats(self._h, -1, None, None, None, None, None)
        out = {}
        for k in range(n):
            nm, ms, nl, fl, by = C.c_char_p(), C.c_double(), C.c_longlong(), C.c_double(), C.c_double()
            _check(L.ocrt_gb_plan_kernel_stats(self._h, k, C.byref(nm), C.byref(ms), C.byref(nl), C.byref(fl),
                                               C.byref(by)))
            out[nm.value.decode()] = {"ms": ms.value, "launches": nl.value, "flops": fl.value,
                                      "bytes": by.value}
        return out

    def close(self):
        if self._h:
            lib().ocrt_gb_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MieAerosol:
    """A .mie aerosol prepared at one wavelength (ocrt_gb_mie_prepare): .struct
    is the ocrt_aerosol to pass to the solves, .diag the preparation's
    diagnostics.  The native object owning the arrays lives as long as this."""

    def __init__(self, handle, struct, diag):
        self._h, self.struct, self.diag = handle, struct, diag

    @property
    def L_max(self):
        return self.struct.L_max

    def arrays(self):
        """Moments and phase table as numpy copies."""
        s = self.struct
        L, n = s.L_max + 1, s.n_ang_phase
        out = {k: np.ctypeslib.as_array(getattr(s, k), (L,)).copy() for k in ("beta", "gamma", "alpha", "zeta")}
        for k in ("theta_phase", "P11_phase", "P12_phase", "P33_phase"):
            out[k] = np.ctypeslib.as_array(getattr(s, k), (n,)).copy()
        return out

    def __del__(self):
        if self._h and _lib is not None:
            _lib.ocrt_gb_mie_aerosol_free(self._h)
            self._h = None


class MieModel:
    """An aerosol model read from a .mie table (ocrt_gb_mie_read)."""

    def __init__(self, path):
        L = lib()
        self._h = C.c_void_p()
        _check(L.ocrt_gb_mie_read(os.fsencode(path), C.byref(self._h)))
        self.path = path

    def shape(self):
        a, w, p = C.c_int(), C.c_int(), C.c_int()
        _check(lib().ocrt_gb_mie_shape(self._h, C.byref(a), C.byref(w), C.byref(p)))
        return a.value, w.value, p.value

    def prepare(self, wavelength_nm, aod_ref, aod_ref_nm=555.0, L_max=80, value_kernel=True, loglin=True):
        """The aerosol at a wavelength, the CLI's protocol by default: AOD given
        at aod_ref_nm, log10-linear truncation, moments to L_max = 80, value
        kernel for the intensity table."""
        L = lib()
        o = MieOpts()
        L.ocrt_mie_opts_default(C.byref(o))
        o.L_max = int(L_max)
        o.use_value_kernel = 1 if value_kernel else 0
        o.use_loglin_trunc = 1 if loglin else 0
        h, aer, dg = C.c_void_p(), Aerosol(), MieDiag()
        _check(L.ocrt_gb_mie_prepare(self._h, float(wavelength_nm), float(aod_ref), float(aod_ref_nm), C.byref(o),
                                     C.byref(h), C.byref(aer), C.byref(dg)))
        return MieAerosol(h, aer, {f: getattr(dg, f) for f, _ in MieDiag._fields_})

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ocrt_gb_mie_free(self._h)
            self._h = None
