"""Angle-grid LUT mode on the GPU (ocrt_gb_solve_batch_lut) against the
reference's rt_solve_case_pol_lut fixtures (tests/golden/reference_lut.json)
and the oracle, per grid direction, with the parity bar: 1e-5 relative in
rho_I, 1e-4 absolute in rho_Q and rho_U."""
import numpy as np
import pytest

from _helpers import TOL_I_REL, TOL_QU_ABS, inputs_from_spec, load_golden_lut, oracle_lut

pytestmark = pytest.mark.gpu

DOC = load_golden_lut()


def _check(got, ref, where):
    relI = np.max(np.abs(got["rho_I"] - ref["rho_I"]) / np.abs(ref["rho_I"]))
    dQ = np.max(np.abs(got["rho_Q"] - ref["rho_Q"]))
    dU = np.max(np.abs(got["rho_U"] - ref["rho_U"]))
    assert relI <= TOL_I_REL, f"{where}: rho_I rel {relI:.2e}"
    assert dQ <= TOL_QU_ABS and dU <= TOL_QU_ABS, f"{where}: Q {dQ:.2e} U {dU:.2e}"
    for k in ("T_diff_dn_dir", "T_sg_up_dir", "T_total_up_dir"):
        scale = max(np.max(np.abs(ref[k])), 1e-12)
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-5 * scale, f"{where}: {k}"


@pytest.mark.parametrize("spec", DOC["cases"], ids=[c["name"] for c in DOC["cases"]])
def test_gpu_lut_matches_reference(gpu, spec):
    from ocrt_gb300 import _abi as A
    c, o, a = inputs_from_spec(spec)
    lut = A.LutHolder(DOC["vza_deg"], DOC["raa_deg"])
    gpu.solve_case_lut(c, o, a, lut)
    ref = {k: np.asarray(v) for k, v in spec["reference"].items() if isinstance(v, list)}
    _check(lut.out, ref, spec["name"])
    assert abs(lut.struct.T_dir_dn - spec["reference"]["T_dir_dn"]) <= 1e-12


def test_gpu_lut_batch_reference_cli_grid(gpu, oracle):
    """Several cases with the reference CLI's default grid (2.5 deg steps,
    vza <= 85) in one call; each against the oracle."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    vza, raa = A.lut_grid_reference_cli()
    cases = [A.default_case(surface="black_fresnel_ocean", wind_speed=w, sza_deg=s, vza_deg=0.0, raa_deg=0.0)
             for w, s in ((3.0, 20.0), (9.0, 55.0))]
    o = A.default_opts(n_mu=16, n_layers=30, fourier_m_max=8, max_orders=300)
    aers = [A.AerosolHolder(0.15, 0.92, *hg_aerosol_moments(0.72, 30)) for _ in cases]
    luts = [A.LutHolder(vza, raa) for _ in cases]
    gpu.solve_batch_lut(cases, o, aers, luts)
    for i in range(len(cases)):
        ref = oracle_lut(oracle, cases[i], o, aers[i], vza, raa)
        _check(luts[i].out, ref.out, f"case {i}")
