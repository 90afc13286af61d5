"""The transport-scan implementations against the one-column scan (k_scan,
OCRT_GB_SCAN=column): the four-column scan (k_scan4) and the chunked scans
fed by tensor-map copies (k_scan_tma with 8, 4 or 16 levels per chunk) run
each column's recurrence with the same arithmetic in the same order, so a
batch, the coupled ocean solve and the scan autotuner (which rotates the
implementations across the orders of its first execute) give the same
numbers as the column scan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(A, N, n=6, seed=5, surfaces=("black_fresnel_ocean", "black", "flat")):
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(seed)
    cases, opts, aers = [], [], []
    for i in range(n):
        cases.append(A.default_case(surface=surfaces[i % len(surfaces)],
                                    sza_deg=rng.uniform(0, 70), vza_deg=rng.uniform(0, 60), raa_deg=rng.uniform(0, 180),
                                    wavelength_nm=rng.choice([443.0, 555.0, 865.0]), wind_speed=rng.uniform(1, 10)))
        opts.append(A.default_opts(n_mu=N, n_layers=int(rng.choice([20, 37, 60])), fourier_m_max=int(rng.integers(2, 9)),
                                   max_orders=200))
        aers.append(A.AerosolHolder(rng.uniform(0.02, 0.3), 0.95, *hg_aerosol_moments(rng.uniform(0.6, 0.8), 40)))
    return cases, opts, aers


SCANS = ["quad", "tma8x3", "tma8x4", "tma4x6", "tma16x2", "tma8x5", "tma4x10"]


@pytest.mark.parametrize("N", [8, 24, 32])
@pytest.mark.parametrize("scan", SCANS)
def test_scan_equals_column_scan(gpu, monkeypatch, N, scan):
    from ocrt_gb300 import _abi as A
    cases, opts, aers = _batch(A, N)
    monkeypatch.setenv("OCRT_GB_SCAN", scan)
    quad = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_SCAN", "column")
    col = gpu.solve_batch(cases, opts, aers)
    for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi", "order_modes"):
        np.testing.assert_allclose(quad[k], col[k], rtol=1e-12, atol=1e-15, err_msg=k)


@pytest.mark.parametrize("scan", ["quad", "tma8x3", "tma8x5"])
def test_scan_equals_column_scan_coupled_ocean(gpu, monkeypatch, scan):
    """The water column's top boundary (internal reflection, four zero-weight
    ring slots) in every scan."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="ocean", sza_deg=35.0, vza_deg=25.0, raa_deg=60.0, wavelength_nm=490.0, wind_speed=6.0)
    o = A.default_opts(fourier_m_max=4, n_layers=30)
    oc = A.OceanHolder(0.08, 0.003, 0.2, hg_aerosol_moments(0.92, 80), n_mu_water=16, m_max_water=4, depth_m=50.0,
                       n_layers_water=60, max_orders_water=200)
    monkeypatch.setenv("OCRT_GB_SCAN", scan)
    quad = gpu.solve_ocean(c, o, oc)
    monkeypatch.setenv("OCRT_GB_SCAN", "column")
    col = gpu.solve_ocean(c, o, oc)
    for k in ("rho_I", "rho_Q", "rho_U", "Rrs_0plus_I", "Ed_0minus", "Lu_0minus_I", "Kd_0minus"):
        assert quad[k] == pytest.approx(col[k], rel=1e-12, abs=1e-15), k


def test_scan_autotuner_matches_column_scan(gpu, monkeypatch):
    """With no implementation named, the first execute of a new shape rotates
    the scans across its orders and keeps the fastest; the results equal the
    column scan's, and the choice is listed by the autotune summary."""
    from ocrt_gb300 import _abi as A
    monkeypatch.delenv("OCRT_GB_SCAN", raising=False)
    monkeypatch.delenv("OCRT_GB_AUTOTUNE", raising=False)
    cases, opts, aers = _batch(A, 20, n=5, seed=11)
    for o in opts:
        o.n_layers = 77          # a level count no other test uses: a fresh tuning key
        o.max_orders = 400
    tuned = gpu.solve_batch(cases, opts, aers)
    again = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_SCAN", "column")
    col = gpu.solve_batch(cases, opts, aers)
    for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi", "order_modes"):
        np.testing.assert_allclose(tuned[k], col[k], rtol=1e-12, atol=1e-15, err_msg=k)
        np.testing.assert_allclose(again[k], col[k], rtol=1e-12, atol=1e-15, err_msg=k)
    recs = [r for r in gpu.autotune_summary() if r["kernel"] == "transport_scan" and r["key"][:2] == [20, 1]]
    assert recs, gpu.autotune_summary()
    assert recs[0]["best"] in SCANS


@pytest.mark.parametrize("N", [8, 32])
def test_primary4_equals_column_primary(gpu, monkeypatch, N):
    """The four-column order-1 kernel (no flat surface in the batch: rough
    ocean with its direct-beam seeds, black) against the one-column one."""
    from ocrt_gb300 import _abi as A
    cases, opts, aers = _batch(A, N, surfaces=("black_fresnel_ocean", "black"))
    monkeypatch.setenv("OCRT_GB_SCAN", "quad")
    quad = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_PRIMARY", "column")
    col = gpu.solve_batch(cases, opts, aers)
    for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi", "order_modes"):
        np.testing.assert_allclose(quad[k], col[k], rtol=1e-12, atol=1e-15, err_msg=k)


@pytest.mark.parametrize("N", [8, 32])
def test_adjoint_scan_tma_equals_column_scan(gpu, monkeypatch, N):
    """The adjoint's transposed scan fed by tensor-map copies against its
    per-thread copy-ring form: the same recurrences in the same order, so the
    gradients agree bit for bit (3 cotangent rows, mixed geometries, two
    surfaces, uneven layers)."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(21)
    cs, aers = [], []
    for i in range(4):
        cs.append(A.default_case(surface=["black_fresnel_ocean", "black"][i % 2], sza_deg=rng.uniform(10, 70),
                                 vza_deg=rng.uniform(0, 60), raa_deg=rng.uniform(0, 180), wind_speed=rng.uniform(2, 9),
                                 wavelength_nm=float(rng.choice([443.0, 555.0]))))
        aers.append(A.AerosolHolder(rng.uniform(0.05, 0.3), 0.93, *hg_aerosol_moments(0.7, 30)))
    o = A.default_opts(n_mu=N, n_layers=37, fourier_m_max=6, max_orders=300)
    eye = np.broadcast_to(np.eye(3), (4, 3, 3)).copy()
    monkeypatch.delenv("OCRT_GB_ADJ_SCAN", raising=False)
    r1, g1 = gpu.solve_batch_adjoint(cs, o, aers, None, eye)
    monkeypatch.setenv("OCRT_GB_ADJ_SCAN", "column")
    r2, g2 = gpu.solve_batch_adjoint(cs, o, aers, None, eye)
    for k in ("d_dtau", "d_ssa", "d_wind"):
        np.testing.assert_allclose(g1[k], g2[k], rtol=1e-12, atol=1e-18, err_msg=k)
    np.testing.assert_allclose(r1["rho_I"], r2["rho_I"], rtol=1e-13)
