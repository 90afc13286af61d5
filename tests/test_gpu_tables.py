"""The phase tables and the aerosol operator on the tensor cores (k_tables_tc,
the default where the tensor-core source runs: N a multiple of 16 up to 32)
against the CUDA-core kernel (k_tables, OCRT_GB_TABLES=simt).  The sums over
the moment index run in 3xTF32 on the tensor cores and in FP32 FMAs on the
CUDA cores, so the operators differ by FP32 rounding (~1e-7 relative) and a
mode may stop one order earlier or later; the solves agree to 2e-6 relative
in I and 5e-8 absolute in Q and U.  Covered: every surface (the flat one reads
the sun-outgoing products through the reflected-beam vectors), IPSS, N = 16
and 32, the view as an inserted ring slot, the value kernel of a .mie
aerosol, the adjoint (which also takes the plain operator) and the water
column of the coupled ocean (four zero-weight slots)."""
import os

import numpy as np
import pytest

from _helpers import assert_parity

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _batch(A, N, n=8, seed=3, L=60, m_max=12):
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(seed)
    surfaces = ("black_fresnel_ocean", "black", "flat")
    cases, opts, aers = [], [], []
    for i in range(n):
        cases.append(A.default_case(surface=surfaces[i % 3], sza_deg=rng.uniform(5, 70),
                                    vza_deg=rng.uniform(0, 60), raa_deg=rng.uniform(0, 180),
                                    wavelength_nm=float(rng.choice([443.0, 555.0, 865.0])),
                                    wind_speed=rng.uniform(1, 10)))
        opts.append(A.default_opts(n_mu=N, n_layers=int(rng.choice([20, 50, 90])), fourier_m_max=m_max,
                                   max_orders=300, pssa=int(i % 2)))
        aers.append(A.AerosolHolder(rng.uniform(0.02, 0.4), rng.uniform(0.85, 0.99),
                                    *hg_aerosol_moments(rng.uniform(0.55, 0.8), L)))
    return cases, opts, aers


def _close(a, b, what):
    np.testing.assert_allclose(a["rho_I"], b["rho_I"], rtol=2e-6, atol=0, err_msg=what)
    np.testing.assert_allclose(a["rho_Q"], b["rho_Q"], rtol=0, atol=5e-8, err_msg=what)
    np.testing.assert_allclose(a["rho_U"], b["rho_U"], rtol=0, atol=5e-8, err_msg=what)


@pytest.mark.parametrize("N,L", [(32, 120), (16, 60), (32, 30)])
def test_tables_tc_matches_cuda_core_tables(gpu, oracle, monkeypatch, N, L):
    from ocrt_gb300 import _abi as A
    cases, opts, aers = _batch(A, N, L=L, m_max=min(16, L + 4))
    monkeypatch.delenv("OCRT_GB_TABLES", raising=False)
    tc = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_TABLES", "simt")
    ref = gpu.solve_batch(cases, opts, aers)
    _close(tc, ref, f"N={N} L={L}")
    # and against the FP64 oracle at the parity bar
    for i in range(0, len(cases), 3):
        o = oracle.solve(cases[i], opts[i], aers[i])
        assert_parity({k: tc[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, o, f"pixel {i}")


def test_tables_tc_modes_past_L(gpu, monkeypatch):
    """Modes m > L have no moment to sum over: the tensor-core kernel writes a
    zero operator for them, as the CUDA-core kernel does."""
    from ocrt_gb300 import _abi as A
    cases, opts, aers = _batch(A, 32, n=3, L=6, m_max=10)
    monkeypatch.delenv("OCRT_GB_TABLES", raising=False)
    tc = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_TABLES", "simt")
    ref = gpu.solve_batch(cases, opts, aers)
    _close(tc, ref, "m > L")


def test_tables_tc_value_kernel(gpu, monkeypatch):
    """A .mie aerosol with the value kernel: the I-I table comes from the
    value tables in both kernels."""
    from ocrt_gb300 import _abi as A
    mie = os.path.join(HERE, "golden", "mie", "synth_peaked.mie")
    aer = gpu.MieModel(mie).prepare(555.0, 0.2, 555.0, L_max=80)
    rng = np.random.default_rng(9)
    cases = [A.default_case(surface=["black_fresnel_ocean", "black"][i % 2], sza_deg=rng.uniform(10, 60),
                            vza_deg=rng.uniform(0, 50), raa_deg=rng.uniform(0, 180), wavelength_nm=555.0,
                            wind_speed=5.0) for i in range(4)]
    opts = [A.default_opts(n_mu=32, n_layers=60, fourier_m_max=16, max_orders=300) for _ in cases]
    aers = [aer] * len(cases)
    monkeypatch.delenv("OCRT_GB_TABLES", raising=False)
    tc = gpu.solve_batch(cases, opts, aers)
    monkeypatch.setenv("OCRT_GB_TABLES", "simt")
    ref = gpu.solve_batch(cases, opts, aers)
    _close(tc, ref, "value kernel")


def test_tables_tc_adjoint(gpu, monkeypatch):
    """Adjoint plans take the plain operator (and its transpose) as well: the
    tensor-core kernel writes both, and the gradients agree."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(17)
    cs, aers = [], []
    for i in range(3):
        cs.append(A.default_case(surface=["black_fresnel_ocean", "black"][i % 2], sza_deg=rng.uniform(10, 60),
                                 vza_deg=rng.uniform(0, 50), raa_deg=rng.uniform(0, 180), wind_speed=4.0,
                                 wavelength_nm=555.0))
        aers.append(A.AerosolHolder(0.15, 0.93, *hg_aerosol_moments(0.7, 40)))
    o = A.default_opts(n_mu=32, n_layers=30, fourier_m_max=6, max_orders=300)
    eye = np.broadcast_to(np.eye(3), (3, 3, 3)).copy()
    monkeypatch.delenv("OCRT_GB_TABLES", raising=False)
    r1, g1 = gpu.solve_batch_adjoint(cs, o, aers, None, eye)
    monkeypatch.setenv("OCRT_GB_TABLES", "simt")
    r2, g2 = gpu.solve_batch_adjoint(cs, o, aers, None, eye)
    np.testing.assert_allclose(r1["rho_I"], r2["rho_I"], rtol=2e-6)
    for k in ("d_dtau", "d_ssa", "d_wind"):
        scale = np.abs(g2[k]).max()
        assert np.abs(g1[k] - g2[k]).max() <= 1e-5 * scale, k


def test_tables_tc_coupled_ocean(gpu, monkeypatch):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="ocean", sza_deg=35.0, vza_deg=25.0, raa_deg=60.0, wavelength_nm=490.0, wind_speed=6.0)
    o = A.default_opts(fourier_m_max=4, n_layers=30, n_mu=32)
    oc = A.OceanHolder(0.08, 0.003, 0.2, hg_aerosol_moments(0.92, 80), n_mu_water=32, m_max_water=4, depth_m=50.0,
                       n_layers_water=60, max_orders_water=300)
    monkeypatch.delenv("OCRT_GB_TABLES", raising=False)
    tc = gpu.solve_ocean(c, o, oc)
    monkeypatch.setenv("OCRT_GB_TABLES", "simt")
    ref = gpu.solve_ocean(c, o, oc)
    assert tc["rho_I"] == pytest.approx(ref["rho_I"], rel=2e-6)
    # the water-leaving signal, a few percent of the TOA signal, through a
    # hydrosol peaked at g = 0.92: its sums over l cancel to ~1e-2 of their
    # terms, and the two kernels' roundings differ by ~1e-5 (the parity bar
    # for these quantities is 1e-4)
    for k in ("Rrs_0plus_I", "Ed_0minus", "Lu_0minus_I"):
        assert tc[k] == pytest.approx(ref[k], rel=3e-5), k
    for k in ("rho_Q", "rho_U"):
        assert tc[k] == pytest.approx(ref[k], abs=5e-8), k
