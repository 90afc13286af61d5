"""Gas absorption on the GPU (ocrt_gb_gas_* and opts.gas), against the
reference fixtures (tests/golden/reference_gas.json) and the oracle.

The table loader and the column depths are host FP64 code: they must give
the reference's numbers to 1e-12.  The per-layer absorption depths are
computed on the device (k_gas_apply) in FP64: 1e-12 relative against the
oracle.  Solves carry the parity bar (1e-5 relative in rho_I, 1e-4 absolute
in rho_Q and rho_U)."""
import ctypes as C

import numpy as np
import pytest

from _helpers import (GAS_DATA, GAS_PROFILES, TOL_I_REL, TOL_QU_ABS, assert_parity, fd_gradient,
                      gas_solve_inputs, load_gas_golden, oracle_lut)

pytestmark = pytest.mark.gpu

DOC = load_gas_golden()
AFGL, XSEC = GAS_DATA + "/afgl_atm", GAS_DATA + "/xsec"


@pytest.fixture(scope="module")
def states(gpu):
    hs = {}
    for key in DOC["columns"]:
        prof, oname = key.split("/")
        hs[key] = gpu.GasState(AFGL, XSEC, prof, DOC["overrides"][oname])
    yield hs
    for s in hs.values():
        s.close()


@pytest.mark.parametrize("key", list(DOC["columns"]))
def test_gas_tables_match_reference(states, key):
    eff, dflt, ov = states[key].columns()
    ref = DOC["columns"][key]
    np.testing.assert_allclose(eff, ref["eff"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(dflt, ref["default"], rtol=1e-13, atol=0)
    assert list(ov.astype(int)) == ref["overridden"]
    for wl, r in zip(DOC["wavelengths"], DOC["tau"][key]):
        per, tot = states[key].tau(wl)
        np.testing.assert_allclose(per, r["per_gas"], rtol=1e-12, atol=1e-300)
        assert tot == pytest.approx(r["total"], rel=1e-12, abs=0)


@pytest.mark.parametrize("spec", DOC["solves"], ids=[s["name"] for s in DOC["solves"]])
def test_layer_depths_match_oracle_and_reference(gpu, oracle, states, spec):
    c, o, aer = gas_solve_inputs(spec)
    o.gas = states[f"{spec['profile']}/{spec['override']}"].handle
    ta, z = gpu.layer_gas(c, o, aer)
    h = oracle.gas_create(GAS_DATA, GAS_PROFILES[spec["profile"]], DOC["overrides"][spec["override"]])
    try:
        o.gas = h
        ta0, z0 = oracle.layer_gas(c, o, aer)
    finally:
        oracle.gas_destroy(h)
    np.testing.assert_allclose(z, z0, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ta, ta0, rtol=1e-12, atol=1e-300)
    lay = next((l for l in DOC["layers"] if l["name"] == spec["name"]), None)
    if lay is not None:
        np.testing.assert_allclose(ta, lay["tau_abs"], rtol=1e-10, atol=1e-300)


def test_gas_solves_match_reference_in_one_batch(gpu, states):
    """Every fixture solve in one batched call: per-case options carry
    different gas states (and one case runs without gas)."""
    from ocrt_gb300 import _abi as A
    cases, opts, aers = [], [], []
    for spec in DOC["solves"]:
        c, o, aer = gas_solve_inputs(spec)
        o.gas = states[f"{spec['profile']}/{spec['override']}"].handle
        cases.append(c); opts.append(o); aers.append(aer)
    spec0 = DOC["solves"][0]
    c, o, aer = gas_solve_inputs(spec0)
    cases.append(c); opts.append(o); aers.append(aer)        # gas-free copy of the first case
    holder_none = A.AerosolHolder(0.0, 1.0, [1.0, 0.0, 0.0], [0.0] * 3, [0.0] * 3, [0.0] * 3)
    res = gpu.solve_batch(cases, opts, [a if a is not None else holder_none for a in aers])
    for i, spec in enumerate(DOC["solves"]):
        got = {k: float(res[k][i]) for k in ("rho_I", "rho_Q", "rho_U", "T_dir_dn", "T_diff_dn_hemi")}
        ref = spec["reference"]
        assert_parity(got, ref, spec["name"])
        assert got["T_dir_dn"] == pytest.approx(ref["T_dir_dn"], rel=1e-9, abs=1e-300), spec["name"]
        assert got["T_diff_dn_hemi"] == pytest.approx(ref["T_diff_dn_hemi"], rel=1e-5), spec["name"]
    # the gas-free copy differs from its gas-loaded twin
    assert abs(res["rho_I"][-1] - res["rho_I"][0]) > 1e-4 * abs(res["rho_I"][0])


def test_zero_columns_equal_gas_free(gpu, states):
    spec = next(s for s in DOC["solves"] if s["override"] == "all_zero")
    c, o, aer = gas_solve_inputs(spec)
    free = gpu.solve_case(c, o, aer)
    o.gas = states["usstd76/all_zero"].handle
    got = gpu.solve_case(c, o, aer)
    for k in ("rho_I", "rho_Q", "rho_U", "T_dir_dn"):
        assert got[k] == pytest.approx(free[k], rel=1e-12, abs=1e-15), k


def test_gas_layer_defaults_match_oracle(gpu, oracle, states):
    spec = DOC["solves"][1]
    c, o, aer = gas_solve_inputs(spec)
    o.gas = states["usstd76/default"].handle
    dt, ss = gpu.layer_defaults(c, o, aer)
    h = oracle.gas_create(GAS_DATA, 0)
    try:
        o.gas = h
        dt0, ss0 = oracle.layer_defaults(c, o, aer)
    finally:
        oracle.gas_destroy(h)
    np.testing.assert_allclose(dt, dt0, rtol=1e-12)
    np.testing.assert_allclose(ss, ss0, rtol=1e-12)


def test_gas_lut_matches_oracle(gpu, oracle, states):
    """LUT mode with gas and IPSS: every grid direction against the oracle."""
    from ocrt_gb300 import _abi as A
    spec = next(s for s in DOC["solves"] if s["name"] == "aer_600_mlwint_ipss")
    c, o, aer = gas_solve_inputs(spec)
    vza = np.arange(0.0, 80.1, 10.0)
    raa = np.arange(0.0, 180.1, 30.0)
    o.gas = states["mlwint/default"].handle
    lut = A.LutHolder(vza, raa)
    gpu.solve_case_lut(c, o, aer, lut)
    h = oracle.gas_create(GAS_DATA, GAS_PROFILES["mlwint"])
    try:
        o.gas = h
        ref = oracle_lut(oracle, c, o, aer, vza, raa)
    finally:
        oracle.gas_destroy(h)
    relI = np.max(np.abs(lut.out["rho_I"] - ref.out["rho_I"]) / np.abs(ref.out["rho_I"]))
    assert relI <= TOL_I_REL
    assert np.max(np.abs(lut.out["rho_Q"] - ref.out["rho_Q"])) <= TOL_QU_ABS
    assert np.max(np.abs(lut.out["rho_U"] - ref.out["rho_U"])) <= TOL_QU_ABS


def test_gas_noalloc_matches_reference(gpu, states):
    from ocrt_gb300 import _abi as A
    f = gpu.lib().ocrt_gb_solve_case_noalloc
    f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Result), C.c_void_p]
    for name in ("ray_760_ipss", "override_940_flat"):
        spec = next(s for s in DOC["solves"] if s["name"] == name)
        c, o, aer = gas_solve_inputs(spec)
        o.gas = states[f"{spec['profile']}/{spec['override']}"].handle
        r = A.Result()
        rc = f(C.byref(c), C.byref(o), C.byref(aer.struct) if aer else None, C.byref(r), None)
        assert rc == 0, gpu.lib().ocrt_gb_last_error()
        assert_parity(A.result_dict(r), spec["reference"], name)


def test_gas_graph_replay_equals_eager(gpu, states):
    spec = DOC["solves"][6]
    c, o, aer = gas_solve_inputs(spec)
    o.gas = states[f"{spec['profile']}/{spec['override']}"].handle
    plan = gpu.Plan([c], o, [aer])
    outs = []
    for _ in range(3):
        plan.execute()
        outs.append(plan.results())
    assert plan.graph_ready
    assert np.array_equal(outs[0], outs[2])
    plan.close()


def test_gas_adjoint_matches_finite_differences(gpu, oracle, states):
    """Layer gradients around the gas-loaded profile: the adjoint against FP64
    central differences of the oracle with the same gas state (layer
    overrides apply on top of the gas step)."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=5.0, sza_deg=40.0, vza_deg=50.0, raa_deg=80.0,
                       wavelength_nm=600.3)
    ok = dict(n_mu=8, n_layers=8, fourier_m_max=4)
    o_gpu = A.default_opts(max_orders=400, tolerance=1e-9, **ok)
    o_fd = A.default_opts(max_orders=200, tolerance=1e-300, **ok)
    aer = A.AerosolHolder(0.15, 0.93, *hg_aerosol_moments(0.7, 16))
    o_gpu.gas = states["usstd76/default"].handle
    h = oracle.gas_create(GAS_DATA, 0)
    try:
        o_fd.gas = h
        dt, ss = oracle.layer_defaults(c, o_fd, aer)
        cot = np.array([1.0, 0.0, 0.0])
        res, g = gpu.solve_batch_adjoint([c], o_gpu, [aer], None, cot[None, None, :])
        which = [("dtau", l) for l in range(len(dt))] + [("ssa", l) for l in range(len(ss))]
        fd = fd_gradient(oracle, c, o_fd, aer, dt, ss, cot, which)
    finally:
        oracle.gas_destroy(h)
    n = len(dt)
    for got, ref, what in ((g["d_dtau"][0, 0], fd[:n], "dtau"), (g["d_ssa"][0, 0], fd[n:], "ssa")):
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-4 * scale + 1e-8, what


def test_gas_loader_edge_cases_match_oracle(gpu, oracle, tmp_path):
    """Missing cross-section table (gas left out), a caller's column, and a
    malformed AFGL row, as in the oracle's loader."""
    import shutil
    root = tmp_path / "data"
    shutil.copytree(GAS_DATA, root)
    (root / "xsec" / "xsec_no2.dat").unlink()
    ov = [-1.0, 300.0 * 2.6868e16, -1.0, -1.0, -1.0, -1.0]
    g = gpu.GasState(str(root / "afgl_atm"), str(root / "xsec"), "tropical", ov)
    h = oracle.gas_create(str(root), GAS_PROFILES["tropical"], ov)
    try:
        for wl in DOC["wavelengths"]:
            pg, tg = g.tau(wl)
            po, to = oracle.gas_tau(h, wl)
            assert pg[4] == 0.0
            np.testing.assert_allclose(pg, po, rtol=1e-12, atol=1e-300)
            assert tg == pytest.approx(to, rel=1e-12)
    finally:
        g.close()
        oracle.gas_destroy(h)
    f = root / "afgl_atm" / "afgl_usstd76.dat"
    f.write_text(f.read_text() + "  1.0 2.0 three\n")
    with pytest.raises(gpu.OcrtError):
        gpu.GasState(str(root / "afgl_atm"), str(root / "xsec"), "usstd76")
