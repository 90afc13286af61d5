"""The .mie aerosol path on the host: the library's reader and preparation
(ocrt_gb_mie_read / ocrt_gb_mie_prepare, the CLI's protocol: AOD carried by
the extinction ratio, log10-linear truncation, vector moments to L_max, the
normalised phase table) against the reference's read_mie_file +
rt_aerosol_runtime_prepare, through the committed fixture (and the live
reference library where it is built); and the FP64 oracle's value kernel
against the reference solves of the same prepared aerosols.  No GPU: the
preparation is host code of the library."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from ocrt_gb300 import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DOC = json.load(open(os.path.join(HERE, "golden", "reference_mie.json")))
PREP = {p["name"]: p for p in DOC["prepared"]}
MIE = os.path.join(HERE, "golden", "mie")


def prepare(spec, value_kernel=True):
    import ocrt_gb300 as og
    m = og.MieModel(os.path.join(MIE, spec["model"]))
    return m.prepare(spec["wavelength_nm"], spec["aod_555"], spec["aod_ref_nm"], L_max=spec["L_max"],
                     value_kernel=value_kernel)


@pytest.mark.parametrize("spec", DOC["prepared"], ids=[p["name"] for p in DOC["prepared"]])
def test_prepare_matches_reference(spec):
    a = prepare(spec)
    ref = spec["reference"]
    s = a.struct
    assert s.tau_a == pytest.approx(ref["tau_a"], rel=1e-13)
    assert s.ssa_a == pytest.approx(ref["ssa_a"], rel=1e-13)
    assert a.diag["trunc_A"] == pytest.approx(ref["trunc_A"], rel=1e-12, abs=1e-15)
    assert a.diag["aod_target"] == pytest.approx(ref["aod_target"], rel=1e-13)
    assert s.n_ang_phase == ref["n_ang"] and s.use_value_kernel == 1
    arr = a.arrays()
    for k in ("beta", "gamma", "alpha", "zeta"):
        r = np.asarray(ref[k])
        assert np.max(np.abs(arr[k] - r)) <= 1e-12 * np.max(np.abs(r)), k
    st = ref["phase_step"]
    for k, kk in (("theta", "theta_phase"), ("P11", "P11_phase"), ("P12", "P12_phase"), ("P33", "P33_phase")):
        r = np.asarray(ref[k])
        np.testing.assert_allclose(arr[kk][::st], r, rtol=1e-12, atol=1e-15, err_msg=k)


def test_prepare_matches_live_reference():
    so = os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so")
    if not os.path.exists(so):
        pytest.skip("reference library not built here")
    lib = C.CDLL(so)
    P = C.POINTER(C.c_double)
    for spec in DOC["prepared"]:
        a = prepare(spec).arrays()
        L, n = spec["L_max"], len(a["theta_phase"])
        scal = np.zeros(8)
        mom = [np.zeros(L + 1) for _ in range(4)]
        ph = [np.zeros(n) for _ in range(4)]
        rc = lib.ocrt_ref_mie_prepare(os.path.join(MIE, spec["model"]).encode(), C.c_double(spec["wavelength_nm"]),
                                      C.c_double(spec["aod_555"]), C.c_double(555.0), L, 1, 1,
                                      scal.ctypes.data_as(P), *[x.ctypes.data_as(P) for x in mom],
                                      *[x.ctypes.data_as(P) for x in ph], n)
        assert rc == 0
        for k, r in zip(("theta_phase", "P11_phase", "P12_phase", "P33_phase"), ph):
            np.testing.assert_allclose(a[k], r, rtol=1e-12, atol=1e-15, err_msg=(spec["name"], k))


@pytest.mark.parametrize("spec", DOC["solves"], ids=[s["name"] for s in DOC["solves"]])
@pytest.mark.parametrize("kernel", ["value", "moment"])
def test_oracle_value_kernel_matches_reference(oracle, spec, kernel):
    p = PREP[spec["aerosol"]]
    a = prepare(p, value_kernel=kernel == "value")
    c = A.default_case(wavelength_nm=p["wavelength_nm"], **spec["case"])
    o = A.default_opts(**spec["opts"])
    r = A.Result()
    assert oracle.f(C.byref(c), C.byref(o), C.byref(a.struct), C.byref(r), None) == 0
    ref = spec["reference"][kernel]
    assert r.rho_I == pytest.approx(ref["rho_I"], rel=1e-10)
    assert r.rho_Q == pytest.approx(ref["rho_Q"], abs=1e-12)
    assert r.rho_U == pytest.approx(ref["rho_U"], abs=1e-12)
    assert r.order_modes == sum(ref["orders_per_m"])


def test_value_and_moment_kernels_differ_near_backscatter():
    """The fixture carries a case where the two kernels differ well beyond
    the parity bar, so the tests above tell them apart."""
    s = next(x for x in DOC["solves"] if x["name"] == "backscatter_L40")
    v, m = s["reference"]["value"]["rho_I"], s["reference"]["moment"]["rho_I"]
    assert abs(v - m) / abs(v) > 1e-3


def test_mie_errors(tmp_path):
    import ocrt_gb300 as og
    with pytest.raises(og.OcrtError):
        og.MieModel(str(tmp_path / "missing.mie"))
    bad = tmp_path / "short.mie"
    text = open(os.path.join(MIE, "synth_hg.mie")).read().splitlines()
    bad.write_text("\n".join(text[:200]) + "\n")              # cut inside the first phase block
    with pytest.raises(og.OcrtError):
        og.MieModel(str(bad))
    m = og.MieModel(os.path.join(MIE, "synth_hg.mie"))
    assert m.shape() == (441, 8, 5)
    for wl in (350.0, 1100.0):                                 # outside the spectral / phase grids
        with pytest.raises(og.OcrtError):
            m.prepare(wl, 0.1)
    with pytest.raises(og.OcrtError):
        m.prepare(555.0, 0.0)
