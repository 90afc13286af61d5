"""The oracle is pinned: it must reproduce the reference's published values
and every reference fixture (tests/golden/reference_cases.json) to ~1e-9."""
import os

import pytest

from _helpers import inputs_from_spec, load_golden

DOC = load_golden()
FIELDS = ["rho_I", "rho_Q", "rho_U", "I_TOA", "Q_TOA", "U_TOA", "tau_R_total", "T_dir_dn",
          "T_diff_dn_hemi", "T_total_dn_hemi", "T_diff_dn_dir", "T_total_up_dir", "T_sg_up_dir",
          "rho_glint_direct_I", "rho_glint_direct_Q", "rho_glint_direct_U"]


def _close(a, b, rel=1e-9, absol=1e-15):
    return abs(a - b) <= max(rel * abs(b), absol)


@pytest.mark.parametrize("name", ["R01", "R07"])
def test_published_recipe_values(oracle, name):
    spec = next(c for c in DOC["cases"] if c["name"] == name)
    c, o, a = inputs_from_spec(spec)
    got = oracle.solve(c, o, a)
    pub = DOC["published"][name]
    for k in ("rho_I", "rho_Q", "rho_U"):
        # published to 11 significant digits
        assert abs(got[k] - pub[k]) <= 6e-11 * max(1.0, abs(pub[k]) * 10), (k, got[k], pub[k])


@pytest.mark.parametrize("spec", DOC["cases"], ids=[c["name"] for c in DOC["cases"]])
def test_oracle_matches_reference_fixture(oracle, spec):
    c, o, a = inputs_from_spec(spec)
    got = oracle.solve(c, o, a, diag=True)
    ref = spec["reference"]
    for k in FIELDS:
        assert _close(got[k], ref[k]), (k, got[k], ref[k])
    if ref.get("kappa_ipss") is not None:
        assert _close(got["kappa_ipss"], ref["kappa_ipss"])
    assert got["order_modes"] == ref["order_modes"]
    assert list(got["orders_per_m"]) == ref["orders_per_m"]
    for m, (gi, ri) in enumerate(zip(got["view_I_m"], ref["view_I_m"])):
        assert _close(gi, ri, absol=1e-14), (m, gi, ri)


REF_SO = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                      "libocrt_ref.so")


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_vs_live_reference_random(oracle):
    import ctypes as C
    import numpy as np
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    ref = A.bind_solver(C.CDLL(REF_SO), "ocrt_ref")
    rng = np.random.default_rng(5)
    for _ in range(6):
        c = A.default_case(surface=int(rng.choice([0, 2, 3])), sza_deg=float(rng.uniform(0, 80)),
                           vza_deg=float(rng.uniform(0, 70)), raa_deg=float(rng.uniform(0, 360)),
                           wind_speed=float(rng.uniform(0.5, 12)), wavelength_nm=float(rng.uniform(400, 900)))
        o = A.default_opts(n_mu=int(rng.choice([8, 12, 16])), n_layers=int(rng.choice([10, 20, 30])),
                           fourier_m_max=int(rng.integers(0, 6)), view_as_node=int(rng.integers(0, 2)))
        aer = A.AerosolHolder(float(rng.uniform(0.01, 0.4)), float(rng.uniform(0.8, 1.0)),
                              *hg_aerosol_moments(float(rng.uniform(0.5, 0.8)), 20))
        r = A.Result()
        assert ref(C.byref(c), C.byref(o), C.byref(aer.struct), C.byref(r), None) == 0
        got = oracle.solve(c, o, aer)
        for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi", "T_diff_dn_dir"):
            assert _close(got[k], getattr(r, k), rel=1e-9, absol=1e-14), (k, got[k], getattr(r, k))


from _helpers import load_golden_lut, oracle_lut  # noqa: E402

LUTDOC = load_golden_lut()


@pytest.mark.parametrize("spec", LUTDOC["cases"], ids=[c["name"] for c in LUTDOC["cases"]])
def test_oracle_lut_matches_reference_fixture(oracle, spec):
    """Angle-grid LUT (rt_solve_case_pol_lut): PCHIP view sampling per mode,
    per-direction Fourier sums, IPSS kappa and sunglint, against the reference."""
    import numpy as np
    from ocrt_gb300 import _abi as A
    c, o, a = inputs_from_spec(spec)
    lut = oracle_lut(oracle, c, o, a, LUTDOC["vza_deg"], LUTDOC["raa_deg"])
    ref = spec["reference"]
    for k in A.LUT_FIELDS:
        got, want = lut.out[k], np.asarray(ref[k])
        scale = max(np.max(np.abs(want)), 1e-300)
        assert np.max(np.abs(got - want)) <= 1e-9 * scale + 1e-15, k
    assert _close(lut.struct.T_dir_dn, ref["T_dir_dn"])
    assert _close(lut.struct.T_diff_dn_hemi, ref["T_diff_dn_hemi"])
