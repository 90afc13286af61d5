"""The .mie aerosol path on the GPU: aerosols prepared by the library from
the synthetic .mie models, solved with the value kernel (k_value_pfm: the
intensity table by direct azimuth integration of the tabulated P11) and with
the moment kernel, against the reference's own solves of the same models
(tests/golden/reference_mie.json) and against the FP64 oracle."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from _helpers import assert_parity
from ocrt_gb300 import _abi as A

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DOC = json.load(open(os.path.join(HERE, "golden", "reference_mie.json")))
PREP = {p["name"]: p for p in DOC["prepared"]}
MIE = os.path.join(HERE, "golden", "mie")


def prepared(gpu, name, value_kernel=True):
    p = PREP[name]
    return gpu.MieModel(os.path.join(MIE, p["model"])).prepare(p["wavelength_nm"], p["aod_555"], 555.0,
                                                               L_max=p["L_max"], value_kernel=value_kernel)


@pytest.mark.parametrize("spec", DOC["solves"], ids=[s["name"] for s in DOC["solves"]])
@pytest.mark.parametrize("kernel", ["value", "moment"])
def test_gpu_mie_matches_reference(gpu, spec, kernel):
    p = PREP[spec["aerosol"]]
    a = prepared(gpu, spec["aerosol"], kernel == "value")
    c = A.default_case(wavelength_nm=p["wavelength_nm"], **spec["case"])
    o = A.default_opts(**spec["opts"])
    got = gpu.solve_case(c, o, a, diag=True)
    ref = spec["reference"][kernel]
    relI, dQ, dU = assert_parity(got, ref, f"{spec['name']}/{kernel}")
    print(f"{spec['name']}/{kernel}: rho_I rel {relI:.1e} |dQ| {dQ:.1e} |dU| {dU:.1e}")
    d = np.abs(np.asarray(got["orders_per_m"]) - np.asarray(ref["orders_per_m"]))
    assert d.max() <= 1, (got["orders_per_m"], ref["orders_per_m"])


def test_gpu_value_kernel_batch_matches_oracle(gpu, oracle):
    """Mixed batch: both models at several wavelengths, rough ocean and black
    surfaces, IPSS on and off, uneven layers and modes."""
    rng = np.random.default_rng(7)
    models = [gpu.MieModel(os.path.join(MIE, f)) for f in ("synth_peaked.mie", "synth_hg.mie")]
    cases, opts, aers = [], [], []
    for i in range(8):
        wl = float(rng.choice([412.0, 490.0, 555.0, 670.0, 865.0]))
        aers.append(models[i % 2].prepare(wl, float(rng.uniform(0.05, 0.4)), 555.0, L_max=int(rng.choice([40, 80]))))
        cases.append(A.default_case(surface=["black_fresnel_ocean", "black"][i % 2], sza_deg=rng.uniform(10, 70),
                                    vza_deg=rng.uniform(0, 60), raa_deg=rng.uniform(0, 180), wavelength_nm=wl,
                                    wind_speed=rng.uniform(2, 10)))
        opts.append(A.default_opts(n_mu=16, n_layers=int(rng.choice([30, 50, 80])),
                                   fourier_m_max=int(rng.integers(4, 12)), max_orders=300, pssa=int(i % 3 == 0)))
    res = gpu.solve_batch(cases, opts, aers)
    for i in range(len(cases)):
        r = A.Result()
        assert oracle.f(C.byref(cases[i]), C.byref(opts[i]), C.byref(aers[i].struct), C.byref(r), None) == 0
        ref = A.result_dict(r)
        assert_parity({k: res[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"pixel {i}")


def test_gpu_value_kernel_unsupported_paths(gpu):
    a = prepared(gpu, "peaked_555")
    c = A.default_case(surface="flat", wavelength_nm=555.0)
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_case(c, A.default_opts(n_mu=16, n_layers=30), a)
    assert e.value.rc == A.OCRT_ERR_UNSUPPORTED
    r = A.Result()
    rc = gpu.lib().ocrt_gb_solve_case_noalloc(C.byref(A.default_case(wavelength_nm=555.0)),
                                              C.byref(A.default_opts(n_mu=16, n_layers=30)), C.byref(a.struct),
                                              C.byref(r), None)
    assert rc == A.OCRT_ERR_UNSUPPORTED
