"""GPU parity through the C ABI: every reference fixture, checked against the
reference's stored outputs and against the FP64 oracle, at the stated bar
(1e-5 relative in I, 1e-4 absolute in Q and U) plus tighter internal checks
on transmittances, IPSS kappa and per-mode order counts."""
import numpy as np
import pytest

from _helpers import assert_parity, inputs_from_spec, load_golden

pytestmark = pytest.mark.gpu
DOC = load_golden()


@pytest.mark.parametrize("spec", DOC["cases"], ids=[c["name"] for c in DOC["cases"]])
def test_gpu_matches_reference_fixture(gpu, oracle, spec):
    c, o, a = inputs_from_spec(spec)
    got = gpu.solve_case(c, o, a, diag=True)
    ref = spec["reference"]
    assert_parity(got, ref, spec["name"])
    # diagnostics follow the same tolerance class
    for k in ("T_diff_dn_hemi", "T_diff_dn_dir", "T_dir_dn", "T_total_dn_hemi"):
        assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref[k]) + 1e-12, (k, got[k], ref[k])
    assert abs(got["tau_R_total"] - ref["tau_R_total"]) <= 1e-12 * ref["tau_R_total"]
    orc = oracle.solve(c, o, a, diag=True)
    assert abs(got["kappa_ipss"] - orc["kappa_ipss"]) <= 1e-10
    # per-mode order counts: identical, or off by at most one order in a mode
    # whose residual sits at the tolerance (as the reference's own CPU/GPU gate
    # allows).  Checked on the modes that carry at least 1e-9 of the view
    # radiance: a mode below that is below the FP32 field's resolution of the
    # solution, and its sup-norm ratio is set by FP32 rounding of its tiny
    # surface-kernel Fourier coefficients (e.g. m >= 26 of config3_full_3,
    # 1e-13 of the total, where the reference needs 4 orders and the GPU 2).
    vm = np.abs(np.array([ref["view_I_m"], ref["view_Q_m"], ref["view_U_m"]])).max(axis=0)
    live = vm >= 1e-9 * abs(ref["I_TOA"])
    d = np.abs(np.array(got["orders_per_m"]) - np.array(ref["orders_per_m"]))[live]
    assert d.max() <= 1, (got["orders_per_m"], ref["orders_per_m"])


@pytest.mark.parametrize("m_max", [0, 1, 3, 40])
def test_gpu_modes_and_high_m(gpu, oracle, m_max):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.2, 0.93, *hg_aerosol_moments(0.75, 48))
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=7.0, sza_deg=55.0, vza_deg=35.0, raa_deg=120.0)
    o = A.default_opts(n_mu=20, n_layers=30, fourier_m_max=m_max, max_orders=300)
    got = gpu.solve_case(c, o, aer)
    ref = oracle.solve(c, o, aer)
    assert_parity(got, ref, f"m_max={m_max}")


def test_gpu_rayleigh_only_aerosol_only(gpu, oracle):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.3, 0.9, *hg_aerosol_moments(0.7, 30))
    c = A.default_case(surface="black", pressure_hpa=0.0, sza_deg=30.0)
    o = A.default_opts(n_mu=12, n_layers=20, fourier_m_max=5)
    assert_parity(gpu.solve_case(c, o, aer), oracle.solve(c, o, aer), "aerosol only")


def test_gpu_max_orders_one_and_nonconvergence(gpu, oracle):
    from ocrt_gb300 import _abi as A
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=5.0)
    for mo in (1, 3):
        o = A.default_opts(max_orders=mo)
        got = gpu.solve_case(c, o)
        ref = oracle.solve(c, o)
        assert_parity(got, ref, f"max_orders={mo}")
        assert got["n_orders_used"] == ref["n_orders_used"] == mo
        assert got["converged"] == ref["converged"]
