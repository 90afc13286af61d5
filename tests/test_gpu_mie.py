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


@pytest.mark.parametrize("spec", DOC["cli"], ids=[s["name"] for s in DOC["cli"]])
def test_cli_mie_matches_reference_cli(spec):
    """The ocrt command on a .mie model (--mie, --aod-555 / --aod-865, the
    reference's aerosol protocol, gases off) against the reference CLI's line."""
    import subprocess
    root = os.path.dirname(HERE)
    binp = os.path.join(root, "ocrt_gb300", "bin", "ocrt")
    if not os.path.exists(binp):
        pytest.skip("ocrt CLI not built")
    gas_off = sum([[f"--gas-column-{g}", "0"] for g in ("h2o", "o3", "no2", "o2", "co2", "ch4")], [])
    args = [os.path.join(root, a) if a.startswith("tests/") else a for a in spec["args"]]
    env = dict(os.environ, OCRT_GB_INPUTS=os.path.join(HERE, "golden", "gas_data"))
    env.pop("OCRT_ADVANCED", None)
    r = subprocess.run([binp, *args, *gas_off], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    rho = [float(x) for x in fields[:3]]
    kv = {f.split("=")[0]: float(f.split("=")[1]) for f in fields[3:] if "=" in f}
    ref = spec["reference"]
    assert_parity({"rho_I": rho[0], "rho_Q": rho[1], "rho_U": rho[2]},
                  {"rho_I": ref["rho"][0], "rho_Q": ref["rho"][1], "rho_U": ref["rho"][2]}, spec["name"])
    for k in ("AOD_ref", "AOD_ref_nm", "AOD_band", "AOD_ext_ratio"):
        assert kv[k] == pytest.approx(ref[k], rel=1e-6), k
    assert kv["T_dir_dn"] == pytest.approx(ref["T_dir_dn"], rel=1e-6)


def test_ocrt_solve_with_mie_model(gpu):
    """ocrt_solve's aer_name as a .mie model: R3 with aod865 equals a direct
    solve of the aerosol the library prepares (AOD given at 865 nm)."""
    from ocrt_gb300.ocrt_solve import solve_reflectances
    path = os.path.join(MIE, "synth_peaked.mie")
    out = solve_reflectances(490.0, 35.0, 25.0, 70.0, 4.0, 0, 0, 0, 0.12, path, which=("R3",), gas_on=False)
    a = gpu.MieModel(path).prepare(490.0, 0.12, 865.0, L_max=80)
    c = A.default_case(surface="black_fresnel_ocean", sza_deg=35.0, vza_deg=25.0, raa_deg=70.0, wavelength_nm=490.0,
                       wind_speed=4.0, decouple_sunglint=1)
    row = out[0] if isinstance(out, list) else out
    assert a.diag["aod_ref_nm"] == 865.0 and a.struct.use_value_kernel == 1
    o = A.default_opts(n_mu=24, n_layers=400, fourier_m_max=16, max_orders=100)
    direct = gpu.solve_case(c, o, a)
    assert row["rho_RA_black_I"] == pytest.approx(direct["rho_I"], rel=1e-5)
    assert row["rho_RA_black_Q"] == pytest.approx(direct["rho_Q"], abs=1e-6)
