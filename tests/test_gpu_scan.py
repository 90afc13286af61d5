"""The four-column transport scan (k_scan4, N a multiple of 4) against the
one-column scan (k_scan, OCRT_GB_SCAN=column): per column both run the same
recurrence in the same order, so a batch, the coupled ocean solve and the
adjoint give the same numbers either way."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(A, N, n=6, seed=5):
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(seed)
    cases, opts, aers = [], [], []
    for i in range(n):
        cases.append(A.default_case(surface=["black_fresnel_ocean", "black", "flat"][i % 3],
                                    sza_deg=rng.uniform(0, 70), vza_deg=rng.uniform(0, 60), raa_deg=rng.uniform(0, 180),
                                    wavelength_nm=rng.choice([443.0, 555.0, 865.0]), wind_speed=rng.uniform(1, 10)))
        opts.append(A.default_opts(n_mu=N, n_layers=int(rng.choice([20, 37, 60])), fourier_m_max=int(rng.integers(2, 9)),
                                   max_orders=200))
        aers.append(A.AerosolHolder(rng.uniform(0.02, 0.3), 0.95, *hg_aerosol_moments(rng.uniform(0.6, 0.8), 40)))
    return cases, opts, aers


@pytest.mark.parametrize("N", [8, 24, 32])
def test_scan4_equals_column_scan(gpu, monkeypatch, N):
    from ocrt_gb300 import _abi as A
    cases, opts, aers = _batch(A, N)
    quad = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_SCAN", "column")
    col = gpu.solve_batch(cases, opts, aers)
    for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi", "order_modes"):
        np.testing.assert_allclose(quad[k], col[k], rtol=1e-12, atol=1e-15, err_msg=k)


def test_scan4_equals_column_scan_coupled_ocean(gpu, monkeypatch):
    """The water column's top boundary (internal reflection) in both scans."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="ocean", sza_deg=35.0, vza_deg=25.0, raa_deg=60.0, wavelength_nm=490.0, wind_speed=6.0)
    o = A.default_opts(fourier_m_max=4, n_layers=30)
    oc = A.OceanHolder(0.08, 0.003, 0.2, hg_aerosol_moments(0.92, 80), n_mu_water=16, m_max_water=4, depth_m=50.0,
                       n_layers_water=60, max_orders_water=200)
    quad = gpu.solve_ocean(c, o, oc)
    monkeypatch.setenv("OCRT_GB_SCAN", "column")
    col = gpu.solve_ocean(c, o, oc)
    for k in ("rho_I", "rho_Q", "rho_U", "Rrs_0plus_I", "Ed_0minus", "Lu_0minus_I", "Kd_0minus"):
        assert quad[k] == pytest.approx(col[k], rel=1e-12, abs=1e-15), k
