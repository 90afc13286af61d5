"""The `ocrt` command-line front end (ocrt_gb300/cli/ocrt_cli.c): option
gates and modes of the reference CLI (code/OCRT_C/src/main.c), output lines in
the rt_io_print_single format and the LUT CSV of main.c:3857-3884.  Gas
absorption is on by default, as in the reference; the tests point the CLI at
the fixture tables (OCRT_GB_INPUTS) and give the library the same state."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "ocrt_gb300", "bin", "ocrt")
GAS_DATA = os.path.join(ROOT, "tests", "golden", "gas_data")


def run(*args, env=None):
    if not os.path.exists(BIN):
        pytest.skip("ocrt CLI not built")
    e = dict(os.environ)
    e.pop("OCRT_ADVANCED", None)
    e["OCRT_GB_INPUTS"] = GAS_DATA
    if env:
        e.update(env)
    return subprocess.run([BIN, *args], capture_output=True, text=True, env=e, timeout=600)


@pytest.mark.parametrize("args,msg", [
    ((), "--surface is required"),
    (("--surface", "black", "--vza", "30"), "requires BOTH --vza and --raa"),
    (("--surface", "black", "--n-mu", "32", "--vza", "1", "--raa", "2"), "OCRT_ADVANCED=1"),
    (("--surface", "black", "--sos-max-orders", "50", "--vza", "1", "--raa", "2"), "OCRT_ADVANCED=1"),
    (("--surface", "black", "--n-layers", "80", "--vza", "1", "--raa", "2"), "OCRT_ADVANCED=1"),
    (("--surface", "lambert"), "not implemented"),
    (("--surface", "ocean"), "not on this solve path"),
    (("--surface", "black", "--aer", "C50"), ".mie"),
    (("--surface", "black", "--vza", "1", "--raa", "2", "--lut-vza-step", "5"), "conflicting mode flags"),
    (("--surface", "black", "--atm-profile", "venus"), "--atm-profile must be one of"),
])
def test_cli_gates_without_device(args, msg):
    r = run(*args)
    assert r.returncode == 2
    assert msg in r.stderr


def _gas(gpu, profile="usstd76", override=None):
    return gpu.GasState(GAS_DATA + "/afgl_atm", GAS_DATA + "/xsec", profile, override)


@pytest.mark.gpu
def test_cli_single_line_equals_library(gpu):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    r = run("--surface", "black_fresnel_ocean", "--wind-speed", "5", "--sza", "40", "--vza", "55", "--raa", "90",
            "--wavelength", "555", "--aod", "0.1", "--aer-hg-g", "0.7", "--aer-ssa", "0.95", "--aer-l-max", "40",
            "--n-layers", "50", "--m-max", "8", env={"OCRT_ADVANCED": "1"})
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    rho = [float(x) for x in fields[:3]]
    kv = dict(f.split("=") for f in fields[3:] if "=" in f)
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=5.0, sza_deg=40.0, vza_deg=55.0, raa_deg=90.0)
    o = A.default_opts(n_layers=50, fourier_m_max=8)
    a = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, 40))
    gas = _gas(gpu)
    o.gas = gas.handle
    ref = gpu.solve_case(c, o, a)
    assert rho == pytest.approx([ref["rho_I"], ref["rho_Q"], ref["rho_U"]], rel=1e-9, abs=1e-14)
    assert float(kv["T_dir_dn"]) == pytest.approx(ref["T_dir_dn"], rel=1e-9)
    assert int(kv["orders"]) == ref["n_orders_used"]


@pytest.mark.gpu
def test_cli_lut_csv_equals_library(gpu, tmp_path):
    from ocrt_gb300 import _abi as A
    out = tmp_path / "lut.csv"
    r = run("--surface", "black_fresnel_ocean", "--wind-speed", "6", "--sza", "35", "--lut-vza-step", "10",
            "--lut-raa-step", "45", "--lut-vza-max", "80", "--lut-output", str(out))
    assert r.returncode == 0, r.stderr
    rows = np.genfromtxt(out, delimiter=",", names=True)
    vza, raa = A.lut_grid_reference_cli(10.0, 45.0, 80.0)
    assert len(rows) == len(vza) * len(raa)
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=6.0, sza_deg=35.0, vza_deg=0.0, raa_deg=0.0)
    lut = A.LutHolder(vza, raa)
    gas = _gas(gpu)
    gpu.solve_case_lut(c, A.default_opts(gas=gas.handle), None, lut)
    np.testing.assert_allclose(rows["rho_I"], lut.out["rho_I"], rtol=1e-9)
    np.testing.assert_allclose(rows["rho_Q"], lut.out["rho_Q"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(rows["diffuse_dn_dir"], lut.out["T_diff_dn_dir"], rtol=1e-9)


@pytest.mark.gpu
def test_cli_batch_rows(gpu, tmp_path):
    csv = tmp_path / "rows.csv"
    csv.write_text("sza,vza,raa,wavelength,wind\n30,20,60,443,3\n50,40,120,865,9\n10,5,170,555,6\n")
    r = run("--surface", "black_fresnel_ocean", "--batch", str(csv))
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 3
    from ocrt_gb300 import _abi as A
    c = A.default_case(surface="black_fresnel_ocean", sza_deg=50.0, vza_deg=40.0, raa_deg=120.0,
                       wavelength_nm=865.0, wind_speed=9.0)
    gas = _gas(gpu)
    ref = gpu.solve_case(c, A.default_opts(gas=gas.handle))
    assert float(lines[1].split()[0]) == pytest.approx(ref["rho_I"], rel=1e-9)


@pytest.mark.gpu
def test_cli_gas_columns_and_profile(gpu):
    """--atm-profile and --gas-column-* reach the solve: the CLI line equals
    the library with the same gas state; all six columns at 0 equal gas-free."""
    from ocrt_gb300 import _abi as A
    args = ("--surface", "black_fresnel_ocean", "--wind-speed", "5", "--sza", "40", "--vza", "30", "--raa", "60",
            "--wavelength", "940")
    r = run(*args, "--atm-profile", "tropical", "--pwv-g-cm", "2.5", "--gas-column-o3", "300")
    assert r.returncode == 0, r.stderr
    assert "(overridden)" in r.stderr
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=5.0, sza_deg=40.0, vza_deg=30.0, raa_deg=60.0,
                       wavelength_nm=940.0)
    gas = _gas(gpu, "tropical", {"h2o": 2.5 * 6.02214076e23 / 18.01528, "o3": 300 * 2.6868e16})
    ref = gpu.solve_case(c, A.default_opts(gas=gas.handle))
    assert float(r.stdout.split()[0]) == pytest.approx(ref["rho_I"], rel=1e-9)
    zero = sum((("--gas-column-" + g, "0") for g in ("h2o", "o3", "no2", "o2", "co2", "ch4")), ())
    r0 = run(*args, *zero)
    assert r0.returncode == 0, r0.stderr
    free = gpu.solve_case(c, A.default_opts())
    assert float(r0.stdout.split()[0]) == pytest.approx(free["rho_I"], rel=1e-12)


def test_cli_missing_gas_tables_is_an_error(tmp_path):
    r = run("--surface", "black", "--vza", "1", "--raa", "2", env={"OCRT_GB_INPUTS": str(tmp_path)})
    assert r.returncode == 1
    assert "gas absorption setup failed" in r.stderr or "no CUDA device" in r.stderr
