"""Generate tests/golden/reference_mie.json: the reference's .mie aerosol
pipeline on the synthetic models of tests/golden/mie/ (written by
make_synthetic_mie.py).

For each prepared aerosol the reference's read_mie_file and
rt_aerosol_runtime_prepare (with the CLI's log10-linear truncation options,
main.c:3646-3670) give the effective AOD and SSA, the truncation coefficient,
the vector moments and the normalised phase table (every 20th angle kept);
for each solve, rt_solve_case_pol_aerosol runs the prepared aerosol with the
value kernel (the CLI's aerosol default, main.c:3338-3341) and with the
moment kernel.  Both go through oracle/ref_driver.c in oracle/_ref.  The
reference CLI itself (oracle/_ref/ocrt, gases off) runs two whole .mie
commands whose output lines are kept.

    OCRT_REF_ROOT=<reference checkout> make -C oracle all && \\
        OCRT_REF_ROOT=<reference checkout> python tests/golden/make_golden_mie.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from ocrt_gb300 import _abi as A  # noqa: E402

OUT = os.path.join(HERE, "reference_mie.json")
MIE = os.path.join(HERE, "mie")
PHASE_STEP = 20

PREPARED = [
    {"name": "peaked_443", "model": "synth_peaked.mie", "wavelength_nm": 443.0, "aod_555": 0.15, "L_max": 80},
    {"name": "peaked_670", "model": "synth_peaked.mie", "wavelength_nm": 670.0, "aod_555": 0.15, "L_max": 80},
    {"name": "peaked_555", "model": "synth_peaked.mie", "wavelength_nm": 555.0, "aod_555": 0.2, "L_max": 80},
    {"name": "hg_555", "model": "synth_hg.mie", "wavelength_nm": 555.0, "aod_555": 0.1, "L_max": 80},
    {"name": "peaked_865_L40", "model": "synth_peaked.mie", "wavelength_nm": 865.0, "aod_555": 0.3, "L_max": 40},
]

SOLVES = [
    {"name": "rough_n16", "aerosol": "peaked_443",
     "case": {"surface": "black_fresnel_ocean", "sza_deg": 40.0, "vza_deg": 30.0, "raa_deg": 60.0, "wind_speed": 5.0},
     "opts": {"n_mu": 16, "n_layers": 60, "fourier_m_max": 8, "max_orders": 200}},
    {"name": "black_ipss_n16", "aerosol": "peaked_670",
     "case": {"surface": "black", "sza_deg": 60.0, "vza_deg": 45.0, "raa_deg": 150.0},
     "opts": {"n_mu": 16, "n_layers": 60, "fourier_m_max": 8, "max_orders": 200, "pssa": 1}},
    {"name": "hg_rough_n24", "aerosol": "hg_555",
     "case": {"surface": "black_fresnel_ocean", "sza_deg": 20.0, "vza_deg": 50.0, "raa_deg": 100.0, "wind_speed": 3.0},
     "opts": {"n_mu": 24, "n_layers": 100, "fourier_m_max": 16, "max_orders": 300}},
    {"name": "cli_protocol_555", "aerosol": "peaked_555",
     "case": {"surface": "black_fresnel_ocean", "sza_deg": 45.0, "vza_deg": 20.0, "raa_deg": 90.0, "wind_speed": 7.0},
     "opts": {"n_mu": 24, "n_layers": 400, "fourier_m_max": 16, "max_orders": 1000, "pssa": 1},
     "note": "the CLI's aerosol protocol: 400 layers, modes 0..16, L = 80, log10-linear truncation, IPSS"},
    {"name": "backscatter_L40", "aerosol": "peaked_865_L40",
     "case": {"surface": "black", "sza_deg": 30.0, "vza_deg": 28.0, "raa_deg": 178.0},
     "opts": {"n_mu": 16, "n_layers": 40, "fourier_m_max": 10, "max_orders": 200},
     "note": "near-backscatter geometry, where the moment and value kernels differ most"},
]


# the reference CLI on a .mie model (main.c's aerosol protocol); gases off
CLI_RUNS = [
    {"name": "cli_peaked_490", "args": ["--mie", "tests/golden/mie/synth_peaked.mie", "--aod-555", "0.2",
                                        "--surface", "black_fresnel_ocean", "--wind-speed", "5", "--sza", "40",
                                        "--vza", "30", "--raa", "60", "--wavelength", "490"]},
    {"name": "cli_hg_865_pssa", "args": ["--mie", "tests/golden/mie/synth_hg.mie", "--aod-865", "0.08",
                                         "--surface", "black", "--sza", "55", "--vza", "10", "--raa", "170",
                                         "--wavelength", "865", "--pssa"]},
]
GAS_OFF = sum([[f"--gas-column-{g}", "0"] for g in ("h2o", "o3", "no2", "o2", "co2", "ch4")], [])


def ref_cli(spec):
    import subprocess
    wd = os.path.join(os.environ.get("OCRT_REF_ROOT", ""), "code", "OCRT_C")
    args = [os.path.join(ROOT, "oracle", "_ref", "ocrt")] + \
        [os.path.join(ROOT, a) if a.startswith("tests/") else a for a in spec["args"]] + GAS_OFF
    r = subprocess.run(args, capture_output=True, text=True, cwd=wd, timeout=600)
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    kv = {f.split("=")[0]: float(f.split("=")[1]) for f in fields[3:] if "=" in f}
    kv["rho"] = [float(x) for x in fields[:3]]
    return kv


def ref_prepare(lib, spec):
    path = os.path.join(MIE, spec["model"]).encode()
    L = spec["L_max"]
    P = C.POINTER(C.c_double)
    scal = np.zeros(8)
    mom = [np.zeros(L + 1) for _ in range(4)]
    cap = 8192
    ph = [np.zeros(cap) for _ in range(4)]
    rc = lib.ocrt_ref_mie_prepare(path, C.c_double(spec["wavelength_nm"]), C.c_double(spec["aod_555"]),
                                  C.c_double(555.0), L, 1, 1, scal.ctypes.data_as(P),
                                  *[a.ctypes.data_as(P) for a in mom], *[a.ctypes.data_as(P) for a in ph], cap)
    assert rc == 0, (spec["name"], rc)
    n = int(scal[6])
    return scal, mom, [a[:n] for a in ph]


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so"))
    solve = A.bind_solver(lib, "ocrt_ref")
    prepared, holders = [], {}
    for spec in PREPARED:
        scal, mom, ph = ref_prepare(lib, spec)
        prepared.append({**spec, "aod_ref_nm": 555.0,
                         "reference": {"tau_a": scal[0], "ssa_a": scal[1], "trunc_A": scal[2], "ssa_raw": scal[3],
                                       "aod_target": scal[4], "extinction_ratio": scal[5], "n_ang": len(ph[0]),
                                       "beta": mom[0].tolist(), "gamma": mom[1].tolist(), "alpha": mom[2].tolist(),
                                       "zeta": mom[3].tolist(), "phase_step": PHASE_STEP,
                                       "theta": ph[0][::PHASE_STEP].tolist(), "P11": ph[1][::PHASE_STEP].tolist(),
                                       "P12": ph[2][::PHASE_STEP].tolist(), "P33": ph[3][::PHASE_STEP].tolist()}})
        holders[spec["name"]] = (scal, mom, ph)
        print(spec["name"], "tau", scal[0], "ssa", scal[1], "A", scal[2])
    rows = []
    for spec in SOLVES:
        scal, mom, ph = holders[spec["aerosol"]]
        c = A.default_case(wavelength_nm=next(p for p in PREPARED if p["name"] == spec["aerosol"])["wavelength_nm"],
                           **spec["case"])
        o = A.default_opts(**spec["opts"])
        out = {}
        for kernel, vk in (("value", 1), ("moment", 0)):
            aer = A.AerosolHolder(scal[0], scal[1], *mom, phase=ph, value_kernel=vk)
            n = o.fourier_m_max + 1
            orders = (C.c_int * n)()
            d = A.Diag(orders_per_m=C.cast(orders, C.POINTER(C.c_int)))
            r = A.Result()
            rc = solve(C.byref(c), C.byref(o), C.byref(aer.struct), C.byref(r), C.byref(d))
            assert rc == 0, (spec["name"], kernel, rc)
            res = A.result_dict(r)
            res["orders_per_m"] = list(orders[:])
            res["kappa_ipss"] = None       # not exported by the reference on this path
            out[kernel] = res
        rows.append({**spec, "reference": out})
        print(spec["name"], "value", out["value"]["rho_I"], "moment", out["moment"]["rho_I"])
    cli = []
    for spec in CLI_RUNS:
        kv = ref_cli(spec)
        cli.append({**spec, "reference": kv})
        print(spec["name"], kv["rho"])
    doc = {"source": "reference read_mie_file + rt_aerosol_runtime_prepare + rt_solve_case_pol_aerosol, "
                     "built from code/OCRT_C/src by oracle/Makefile, driven by oracle/ref_driver.c; "
                     "cli: the reference CLI (oracle/_ref/ocrt) with every gas column at 0",
           "models": "tests/golden/mie (make_synthetic_mie.py)", "prepared": prepared, "solves": rows, "cli": cli}
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
