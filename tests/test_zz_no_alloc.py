"""The allocation-free single solve, called through the C ABI.

ocrt_gb_solve_case_noalloc serves callers that may not allocate device
memory (an application that owns the device budget through its own pool, or a
loop that cannot afford cudaMalloc's implicit synchronisation).  It must give
the same results as ocrt_gb_solve_case, within the parity tolerance of this
suite, on consecutive calls that share its one static scratch array, and must
reject cases larger than that array with a clear error.

This file is collected last on purpose, and passes both alone in a fresh
process and after the rest of the suite."""
import ctypes as C

import pytest

from _helpers import assert_parity

pytestmark = pytest.mark.gpu


def _noalloc(gpu):
    from ocrt_gb300 import _abi as A
    f = gpu.lib().ocrt_gb_solve_case_noalloc
    f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Result), C.c_void_p]
    f.restype = C.c_int
    return f


def _call(gpu, case, opts, aer=None):
    from ocrt_gb300 import _abi as A
    r = A.Result()
    rc = _noalloc(gpu)(C.byref(case), C.byref(opts), C.byref(aer.struct) if aer else None, C.byref(r), None)
    return rc, A.result_dict(r)


def test_noalloc_matches_solve_case_on_consecutive_calls(gpu):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.15, 0.94, *hg_aerosol_moments(0.72, 120))
    calls = [
        # a large case first: 32 streams, 400 layers, 33 modes (several mode waves in the array)
        (A.default_case(surface="black_fresnel_ocean", wind_speed=6.0, sza_deg=45.0, vza_deg=30.0, raa_deg=60.0,
                        tau_r_input=0.0945),
         A.default_opts(n_mu=32, n_layers=400, fourier_m_max=32, tau_r_source=1, max_orders=1000), aer),
        # then a different, smaller case: stale contents of the shared array must not leak into it
        (A.default_case(surface="flat", sza_deg=30.0, vza_deg=50.0, raa_deg=120.0),
         A.default_opts(n_mu=16, n_layers=40, fourier_m_max=4, pssa=1), None),
        # and the first case again
        (A.default_case(surface="black_fresnel_ocean", wind_speed=6.0, sza_deg=45.0, vza_deg=30.0, raa_deg=60.0,
                        tau_r_input=0.0945),
         A.default_opts(n_mu=32, n_layers=400, fourier_m_max=32, tau_r_source=1, max_orders=1000), aer),
    ]
    for i, (c, o, a) in enumerate(calls):
        rc, got = _call(gpu, c, o, a)
        assert rc == 0, gpu.lib().ocrt_gb_last_error()
        ref = gpu.solve_case(c, o, a)
        assert_parity(got, ref, f"noalloc call {i}")
        assert got["order_modes"] == ref["order_modes"]
        for k in ("T_diff_dn_hemi", "T_diff_dn_dir", "kappa_ipss"):
            assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref[k]) + 1e-12, (i, k)


def test_noalloc_rejects_oversized_cases(gpu):
    from ocrt_gb300 import _abi as A
    for o in (A.default_opts(n_layers=500), A.default_opts(n_mu=40), A.default_opts(fourier_m_max=40)):
        rc, _ = _call(gpu, A.default_case(), o)
        assert rc == A.OCRT_ERR_ARGS
        assert b"noalloc" in gpu.lib().ocrt_gb_last_error()
