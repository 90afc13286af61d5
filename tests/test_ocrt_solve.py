"""ocrt_gb300.ocrt_solve keeps the reference's Python entry signatures
(code/OCRT_Python/ocrt_solve.py:131-206, :279-410) for the R2/R3 reflectances
that are on this path."""
import pytest


def test_unavailable_parts_raise():
    from ocrt_gb300.ocrt_solve import solve_reflectances
    with pytest.raises(NotImplementedError, match="R1"):
        solve_reflectances(555, 30, 30, 90, 3, 1.2, 3.5, 0.04, 0.1, "HG:0.7,0.95", which=("R1",), gas_on=False)
    with pytest.raises(NotImplementedError, match=".mie"):
        solve_reflectances(555, 30, 30, 90, 3, 0, 0, 0, 0.1, "C50", which=("R3",), gas_on=False)


@pytest.mark.gpu
def test_r2_r3_equal_direct_solves(gpu):
    from ocrt_gb300 import _abi as A
    from ocrt_gb300.ocrt_solve import solve_reflectances
    from synthetic import hg_aerosol_moments
    out = solve_reflectances(555.0, 30.0, 40.0, 90.0, 3.0, 0, 0, 0, 0.12, "HG:0.7,0.95,60", which=("R2", "R3"),
                             fourier_m_max=8, nt_atm=60, gas_on=False)
    base = dict(surface="black_fresnel_ocean", sza_deg=30.0, vza_deg=40.0, raa_deg=90.0, wavelength_nm=555.0,
                wind_speed=3.0, decouple_sunglint=1)
    r2 = gpu.solve_case(A.default_case(**base), A.default_opts(n_mu=24, n_layers=60, fourier_m_max=2,
                                                                 max_orders=100))
    r3 = gpu.solve_case(A.default_case(**base), A.default_opts(n_mu=24, n_layers=60, fourier_m_max=8,
                                                                 max_orders=100),
                        A.AerosolHolder(0.12, 0.95, *hg_aerosol_moments(0.7, 60)))
    assert out["rho_R_I"] == pytest.approx(r2["rho_I"], rel=1e-12)
    assert out["rho_RA_black_I"] == pytest.approx(r3["rho_I"], rel=1e-12)
    assert out["rho_AplusRA_I"] == pytest.approx(r3["rho_I"] - r2["rho_I"], rel=1e-9)


@pytest.mark.gpu
def test_r2_r3_with_gas_equal_direct_solves(gpu, monkeypatch):
    """gas_on=True (the default) folds the gas tables into both solves."""
    import os
    from ocrt_gb300 import _abi as A
    from ocrt_gb300 import ocrt_solve
    from synthetic import hg_aerosol_moments
    data = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gas_data")
    monkeypatch.setenv("OCRT_GB_INPUTS", data)
    ocrt_solve._STATE.pop("ab", None)
    out = ocrt_solve.solve_reflectances(760.4, 30.0, 40.0, 90.0, 3.0, 0, 0, 0, 0.12, "HG:0.7,0.95,60",
                                        which=("R2", "R3"), fourier_m_max=8, nt_atm=60)
    ocrt_solve._STATE.pop("ab", None)
    gas = gpu.GasState(data + "/afgl_atm", data + "/xsec")
    base = dict(surface="black_fresnel_ocean", sza_deg=30.0, vza_deg=40.0, raa_deg=90.0, wavelength_nm=760.4,
                wind_speed=3.0, decouple_sunglint=1)
    r2 = gpu.solve_case(A.default_case(**base), A.default_opts(n_mu=24, n_layers=60, fourier_m_max=2,
                                                                 max_orders=100, gas=gas.handle))
    r3 = gpu.solve_case(A.default_case(**base), A.default_opts(n_mu=24, n_layers=60, fourier_m_max=8,
                                                                 max_orders=100, gas=gas.handle),
                        A.AerosolHolder(0.12, 0.95, *hg_aerosol_moments(0.7, 60)))
    assert out["rho_R_I"] == pytest.approx(r2["rho_I"], rel=1e-12)
    assert out["rho_RA_black_I"] == pytest.approx(r3["rho_I"], rel=1e-12)
