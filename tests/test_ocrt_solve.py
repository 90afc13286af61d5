"""ocrt_gb300.ocrt_solve keeps the reference's Python entry signatures
(code/OCRT_Python/ocrt_solve.py:131-206, :279-410) for the R1/R2/R3
reflectances; R1 runs the coupled solve over pure seawater plus CDOM, whose
IOPs (ocrt_gb300/water_iop.py) are checked against the a_total and b_total
the reference printed for every coupled fixture."""
import os

import pytest

from _helpers import assert_parity, load_golden_ocean

HERE = os.path.dirname(os.path.abspath(__file__))
WATER = os.path.join(HERE, "golden", "water_iop")


def test_unavailable_parts_raise():
    from ocrt_gb300.ocrt_solve import solve_reflectances
    with pytest.raises(NotImplementedError, match="constituent"):
        solve_reflectances(555, 30, 30, 90, 3, 1.2, 3.5, 0.04, 0.1, "HG:0.7,0.95", which=("R1",), gas_on=False)
    import ocrt_gb300 as og
    with pytest.raises(og.OcrtError, match="cannot open"):      # data/C50.mie: the FR631 tables are not here
        solve_reflectances(555, 30, 30, 90, 3, 0, 0, 0, 0.1, "C50", which=("R3",), gas_on=False)


def test_pure_water_iops_match_reference():
    """a_w(lambda, T) + a_cdom and b_w of every coupled fixture, including a
    28 C case (the psi_T term) and a wavelength between table rows."""
    from ocrt_gb300.water_iop import PureWater
    pw = PureWater(WATER)
    for spec in load_golden_ocean()["cases"]:
        ref = spec["reference"]
        a, b = pw.iops(spec["wavelength_nm"], spec["T_water"], spec["adom440"])
        assert a == pytest.approx(ref["a_total"], rel=1e-9), spec["name"]
        assert b == pytest.approx(ref["b_total"], rel=1e-9), spec["name"]
        assert pw.a_w(spec["wavelength_nm"], spec["T_water"]) == pytest.approx(ref["a_w"], rel=1e-9)
        assert a - pw.a_w(spec["wavelength_nm"], spec["T_water"]) == pytest.approx(ref["a_dom"], rel=1e-6, abs=1e-15)


def test_pure_water_tables_do_not_extrapolate(tmp_path):
    from ocrt_gb300.water_iop import PureWater
    pw = PureWater(WATER)
    with pytest.raises(ValueError, match="outside"):
        pw.a_w(300.0)
    bad = tmp_path / "water_coef_z09_1nm.txt"
    bad.write_text("/end_header\n500 0.1 0.002\n499 0.1 0.002\n")
    with pytest.raises(ValueError, match="increasing"):
        PureWater(str(tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["R26", "R28", "warm_water_t28"])
def test_r1_matches_reference(gpu, monkeypatch, name):
    """R1 from the pure-water tables, with the reference CLI's settings of
    each fixture, reproduces the reference's coupled TOA reflectance and Rrs."""
    from ocrt_gb300 import ocrt_solve
    spec = next(s for s in load_golden_ocean()["cases"] if s["name"] == name)
    monkeypatch.setenv("OCRT_GB_WATER_IOP", WATER)
    ocrt_solve._STATE.pop("pw", None)
    m = spec["m_max"] if spec["m_max"] is not None else 2
    out = ocrt_solve.solve_reflectances(spec["wavelength_nm"], spec["sza_deg"], spec["vza_deg"], spec["raa_deg"],
                                        spec["wind_speed"], 0.0, 0.0, spec["adom440"], 0.0, "HG:0.7,0.95",
                                        which=("R1",), n_mu_water=spec["n_mu_water"] or 48, fourier_m_max=m,
                                        nt_atm=spec["n_layers"] or 40, max_it_water=20, gas_on=False,
                                        water_temperature_c=spec["T_water"])
    ocrt_solve._STATE.pop("pw", None)
    ref = spec["reference"]
    assert_parity({"rho_I": out["rho_TOA_I"], "rho_Q": out["rho_TOA_Q"], "rho_U": out["rho_TOA_U"]},
                  {"rho_I": ref["TOA_rho_I"], "rho_Q": ref["TOA_rho_Q"], "rho_U": ref["TOA_rho_U"]}, name)
    assert out["Rrs"] == pytest.approx(ref["Rrs0plus_I"], rel=1e-4)
    assert out["rrs0minus"] == pytest.approx(ref["rrs0minus_I"], rel=1e-4)


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
