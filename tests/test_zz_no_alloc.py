"""The allocation-free single solve, called through the C ABI.

ocrt_gb_solve_case_noalloc serves callers that may not allocate device
memory (an application that owns the device budget through its own pool, or a
loop that cannot afford cudaMalloc's implicit synchronisation).  It runs the
CUDA-core source and Cox-Munk kernels of the allocating path out of one static
scratch array, so it must give the results of ocrt_gb_solve_case and of the
FP64 oracle within the parity tolerance of this suite, on consecutive calls
that share that array; it must leave the device's free memory unchanged; and
it must reject cases larger than the array with a clear error.

This file is collected last on purpose, and passes both alone in a fresh
process and after the rest of the suite."""
import ctypes as C
import ctypes.util

import pytest

from _helpers import GAS_DATA, assert_parity

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


def _free_device_bytes():
    """cudaMemGetInfo through the CUDA runtime the library itself links."""
    rt = None
    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    if rt is None:
        pytest.skip("CUDA runtime library not found by name")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _large_case(A, aer):
    return (A.default_case(surface="black_fresnel_ocean", wind_speed=6.0, sza_deg=45.0, vza_deg=30.0, raa_deg=60.0,
                           tau_r_input=0.0945),
            A.default_opts(n_mu=32, n_layers=400, fourier_m_max=32, tau_r_source=1, max_orders=1000), aer)


def test_noalloc_matches_solve_case_and_oracle_on_consecutive_calls(gpu, oracle):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.15, 0.94, *hg_aerosol_moments(0.72, 120))
    calls = [
        # a large case first: 32 streams, 400 layers, 33 modes (several mode waves in the array)
        _large_case(A, aer),
        # then a different, smaller case: stale contents of the shared array must not leak into it
        (A.default_case(surface="flat", sza_deg=30.0, vza_deg=50.0, raa_deg=120.0),
         A.default_opts(n_mu=16, n_layers=40, fourier_m_max=4, pssa=1), None),
        # and the first case again
        _large_case(A, aer),
    ]
    for i, (c, o, a) in enumerate(calls):
        rc, got = _call(gpu, c, o, a)
        assert rc == 0, gpu.lib().ocrt_gb_last_error()
        ref = gpu.solve_case(c, o, a)
        assert_parity(got, ref, f"noalloc call {i} vs ocrt_gb_solve_case")
        assert_parity(got, oracle.solve(c, o, a), f"noalloc call {i} vs the FP64 oracle")
        assert got["order_modes"] == ref["order_modes"]
        for k in ("T_diff_dn_hemi", "T_diff_dn_dir", "kappa_ipss"):
            assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref[k]) + 1e-12, (i, k)


def test_noalloc_allocates_no_device_memory(gpu):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, 60))
    c, o, _ = _large_case(A, aer)
    o.n_layers = 100
    rc, first = _call(gpu, c, o, aer)          # warm-up: array address, kernel loading
    assert rc == 0, gpu.lib().ocrt_gb_last_error()
    before = _free_device_bytes()
    for _ in range(2):
        rc, again = _call(gpu, c, o, aer)
        assert rc == 0, gpu.lib().ocrt_gb_last_error()
        assert again["rho_I"] == first["rho_I"] and again["rho_U"] == first["rho_U"]
    assert _free_device_bytes() == before


def test_noalloc_with_gas_absorption(gpu):
    from ocrt_gb300 import _abi as A
    import os
    st = gpu.GasState(os.path.join(GAS_DATA, "afgl_atm"), os.path.join(GAS_DATA, "xsec"), "usstd76")
    try:
        c = A.default_case(surface="black_fresnel_ocean", wind_speed=4.0, wavelength_nm=600.3, sza_deg=35.0)
        o = A.default_opts(n_mu=16, n_layers=50, fourier_m_max=4, pssa=1)
        o.gas = st.handle
        rc, got = _call(gpu, c, o)
        assert rc == 0, gpu.lib().ocrt_gb_last_error()
        assert_parity(got, gpu.solve_case(c, o), "noalloc with gas")
    finally:
        st.close()


def test_noalloc_rejects_oversized_cases(gpu):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    for o in (A.default_opts(n_layers=500), A.default_opts(n_mu=40), A.default_opts(fourier_m_max=40),
              A.default_opts(max_orders=5000)):
        rc, _ = _call(gpu, A.default_case(), o)
        assert rc == A.OCRT_ERR_ARGS
        assert b"noalloc" in gpu.lib().ocrt_gb_last_error()
    aer = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, 256))
    rc, _ = _call(gpu, A.default_case(), A.default_opts(), aer)
    assert rc == A.OCRT_ERR_ARGS
    assert b"noalloc" in gpu.lib().ocrt_gb_last_error()
