"""C-ABI contract checks that need no GPU: the library loads, exports every
function include/ocrt_gb300.h declares, the ctypes mirror matches the C
struct sizes, and argument validation returns the reference's codes."""
import ctypes as C
import os
import re

import pytest

import ocrt_gb300 as og
from ocrt_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "ocrt_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ocrt_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = og.lib()
    names = header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(og.EXPORTS) <= set(names)


def test_struct_sizes_match_c(oracle):
    f = oracle.lib.ocrt_oracle_abi_sizes
    f.argtypes = [C.POINTER(C.c_size_t)]
    sizes = (C.c_size_t * 5)()
    f(sizes)
    assert list(sizes) == [C.sizeof(A.Case), C.sizeof(A.Opts), C.sizeof(A.Aerosol), C.sizeof(A.Result),
                           C.sizeof(A.Diag)]


def test_defaults_match_reference():
    lib = og.lib()
    o = A.Opts()
    lib.ocrt_opts_default(C.byref(o))
    ref = A.default_opts()
    for f, _ in A.Opts._fields_:
        assert getattr(o, f) == getattr(ref, f), f
    c = A.Case()
    lib.ocrt_case_default(C.byref(c))
    rc = A.default_case()
    for f, _ in A.Case._fields_:
        assert getattr(c, f) == getattr(rc, f), f


@pytest.mark.parametrize("field,value,code", [
    ("sza_deg", 90.0, A.OCRT_ERR_ARGS), ("vza_deg", -1.0, A.OCRT_ERR_ARGS),
    ("wavelength_nm", 320.0, A.OCRT_ERR_ARGS), ("surface", A.SURFACE_OCEAN, A.OCRT_ERR_UNSUPPORTED),
    ("surface", A.SURFACE_LAMBERT, A.OCRT_ERR_UNSUPPORTED), ("pressure_hpa", 0.0, A.OCRT_ERR_ARGS),
])
def test_invalid_case_codes_without_device(field, value, code):
    c = A.default_case(**{field: value})
    with pytest.raises(og.OcrtError) as e:
        og.solve_case(c, A.default_opts())
    assert e.value.rc == code


@pytest.mark.parametrize("field,value", [("n_mu", 1), ("n_mu", 65), ("n_layers", 1), ("fourier_m_max", 256),
                                         ("fourier_m_max", -1), ("max_orders", 0), ("tolerance", 0.0)])
def test_invalid_opts_codes(field, value):
    with pytest.raises(og.OcrtError) as e:
        og.solve_case(A.default_case(), A.default_opts(**{field: value}))
    assert e.value.rc == A.OCRT_ERR_ARGS


def test_invalid_aerosol_codes():
    import numpy as np
    bad = A.AerosolHolder(0.1, 1.5, np.ones(5), np.zeros(5), np.zeros(5), np.zeros(5))
    with pytest.raises(og.OcrtError) as e:
        og.solve_case(A.default_case(), A.default_opts(), bad)
    assert e.value.rc == A.OCRT_ERR_ARGS
    nanm = A.AerosolHolder(0.1, 0.9, np.array([1.0, np.nan, 0.1, 0.0]), np.zeros(4), np.zeros(4), np.zeros(4))
    with pytest.raises(og.OcrtError) as e:
        og.solve_case(A.default_case(), A.default_opts(), nanm)
    assert e.value.rc == A.OCRT_ERR_NONFINITE
