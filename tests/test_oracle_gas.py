"""Gas absorption in the oracle, pinned against the reference
(tests/golden/reference_gas.json, made by tests/golden/make_golden_gas.py on
the reduced tables under tests/golden/gas_data): AFGL column integrals,
column absorption depths per gas (rt_absorption.c:556-600), per-layer depths
and level altitudes of the gas-loaded grid (rt_atm.c:437-548) and full solves
with gas absorption, plane-parallel and with IPSS (rt_ipss.c:64-70)."""
import numpy as np
import pytest

from _helpers import GAS_DATA, GAS_PROFILES, gas_solve_inputs, load_gas_golden

DOC = load_gas_golden()
FIELDS = ["rho_I", "rho_Q", "rho_U", "I_TOA", "Q_TOA", "U_TOA", "T_dir_dn", "T_diff_dn_hemi", "T_total_dn_hemi",
          "T_diff_dn_dir", "T_total_up_dir", "T_sg_up_dir", "rho_glint_direct_I"]


@pytest.fixture(scope="module")
def handles(oracle):
    hs = {}
    for key in DOC["columns"]:
        prof, oname = key.split("/")
        hs[key] = oracle.gas_create(GAS_DATA, GAS_PROFILES[prof], DOC["overrides"][oname])
    yield hs
    for h in hs.values():
        oracle.gas_destroy(h)


@pytest.mark.parametrize("key", list(DOC["columns"]))
def test_columns_and_depths_match_reference(oracle, handles, key):
    eff, dflt, ov = oracle.gas_columns(handles[key])
    ref = DOC["columns"][key]
    np.testing.assert_allclose(eff, ref["eff"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(dflt, ref["default"], rtol=1e-13, atol=0)
    assert list(ov) == ref["overridden"]
    for wl, r in zip(DOC["wavelengths"], DOC["tau"][key]):
        per, tot = oracle.gas_tau(handles[key], wl)
        np.testing.assert_allclose(per, r["per_gas"], rtol=1e-12, atol=1e-300)
        assert tot == pytest.approx(r["total"], rel=1e-12, abs=0)


def test_usstd76_o3_column_is_the_documented_value(oracle, handles):
    """rt_absorption.c:22-24: the US76 O3 column is 346.9 DU."""
    _, dflt, _ = oracle.gas_columns(handles["usstd76/default"])
    assert dflt[1] / 2.6867e16 == pytest.approx(346.9, abs=0.05)


@pytest.mark.parametrize("spec", DOC["solves"], ids=[s["name"] for s in DOC["solves"]])
def test_oracle_solve_with_gas_matches_reference(oracle, spec):
    c, o, aer = gas_solve_inputs(spec)
    h = oracle.gas_create(GAS_DATA, GAS_PROFILES[spec["profile"]], DOC["overrides"][spec["override"]])
    try:
        o.gas = h
        got = oracle.solve(c, o, aer)
        ref = spec["reference"]
        for k in FIELDS:
            assert got[k] == pytest.approx(ref[k], rel=1e-9, abs=1e-15), k
        lay = next((l for l in DOC["layers"] if l["name"] == spec["name"]), None)
        if lay is not None:
            ta, z = oracle.layer_gas(c, o, aer)
            np.testing.assert_allclose(ta, lay["tau_abs"], rtol=1e-10, atol=1e-300)
            np.testing.assert_allclose(z[:-1], lay["z_top_km"], rtol=0, atol=2e-9)
            np.testing.assert_allclose(z[1:], lay["z_bot_km"], rtol=0, atol=2e-9)
    finally:
        oracle.gas_destroy(h)


def test_zero_columns_equal_gas_free(oracle):
    """All six columns at zero leave the solve as without gas (main.c:249-253)."""
    spec = next(s for s in DOC["solves"] if s["override"] == "all_zero")
    c, o, aer = gas_solve_inputs(spec)
    free = oracle.solve(c, o, aer)
    h = oracle.gas_create(GAS_DATA, 0, [0.0] * 6)
    try:
        o.gas = h
        got = oracle.solve(c, o, aer)
    finally:
        oracle.gas_destroy(h)
    for k in FIELDS:
        assert got[k] == pytest.approx(free[k], rel=1e-14, abs=1e-300), k


def test_gas_defaults_feed_the_layer_parameters(oracle):
    """Layer defaults with gas: dtau includes the absorption, ssa drops by dtau_old/dtau_new."""
    spec = DOC["solves"][1]
    c, o, aer = gas_solve_inputs(spec)
    dt0, ss0 = oracle.layer_defaults(c, o, aer)
    h = oracle.gas_create(GAS_DATA, 0)
    try:
        o.gas = h
        dt1, ss1 = oracle.layer_defaults(c, o, aer)
        ta, _ = oracle.layer_gas(c, o, aer)
        # the layer overrides at the gas-loaded defaults reproduce the gas solve
        base = oracle.solve(c, o, aer)
        o2 = gas_solve_inputs(spec)[1]
        via = oracle.solve_layers(c, o2, aer, dtau=dt1, ssa=ss1)
    finally:
        oracle.gas_destroy(h)
    np.testing.assert_allclose(dt1, dt0 + ta, rtol=1e-12)
    np.testing.assert_allclose(ss1, ss0 * dt0 / (dt0 + ta), rtol=1e-12)
    for k in ("rho_I", "rho_Q", "rho_U"):
        assert via[k] == pytest.approx(base[k], rel=1e-10, abs=1e-14), k


def test_missing_afgl_profile_is_an_error(oracle, tmp_path):
    with pytest.raises(RuntimeError):
        oracle.gas_create(str(tmp_path), 0)


def test_missing_cross_section_table_leaves_the_gas_out(oracle, tmp_path):
    """rt_absorption.c:500-515: a missing xsec file contributes zero absorption
    for that gas; the other gases are unchanged."""
    import shutil
    root = tmp_path / "data"
    shutil.copytree(GAS_DATA, root)
    (root / "xsec" / "xsec_o3.dat").unlink()
    full = oracle.gas_create(GAS_DATA, 0)
    part = oracle.gas_create(str(root), 0)
    try:
        for wl in (443.0, 600.3):
            pf, _ = oracle.gas_tau(full, wl)
            pp, tp = oracle.gas_tau(part, wl)
            assert pp[1] == 0.0
            np.testing.assert_array_equal(np.delete(pp, 1), np.delete(pf, 1))
            assert tp == pytest.approx(pf.sum() - pf[1], rel=1e-14)
    finally:
        oracle.gas_destroy(full)
        oracle.gas_destroy(part)


def test_column_override_scales_the_profile(oracle):
    """A caller's column rescales that gas's layers in proportion
    (rt_absorption.c:566-583): the depth scales by column / default."""
    h0 = oracle.gas_create(GAS_DATA, 0)
    try:
        _, dflt, _ = oracle.gas_columns(h0)
        ov = [-1.0] * 6
        ov[1] = 2.0 * dflt[1]
        h1 = oracle.gas_create(GAS_DATA, 0, ov)
        try:
            for wl in (330.0, 555.0, 600.3):
                p0, _ = oracle.gas_tau(h0, wl)
                p1, _ = oracle.gas_tau(h1, wl)
                assert p1[1] == pytest.approx(2.0 * p0[1], rel=1e-12)
                np.testing.assert_array_equal(np.delete(p1, 1), np.delete(p0, 1))
        finally:
            oracle.gas_destroy(h1)
    finally:
        oracle.gas_destroy(h0)


def test_malformed_afgl_row_is_an_error(oracle, tmp_path):
    import shutil
    root = tmp_path / "data"
    shutil.copytree(GAS_DATA, root)
    f = root / "afgl_atm" / "afgl_usstd76.dat"
    f.write_text(f.read_text() + "  1.0 2.0 three\n")
    with pytest.raises(RuntimeError):
        oracle.gas_create(str(root), 0)
