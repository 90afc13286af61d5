"""Generate tests/golden/reference_ocean.json from the reference solver's own
command-line program on coupled atmosphere-ocean cases.

The reference CLI (oracle/_ref/ocrt, built from code/OCRT_C/src by
oracle/Makefile) runs each case with --surface ocean and the pure-seawater
water model (optionally with CDOM absorption), gases off; every key=value of
its output line is recorded.  The water absorption and scattering the
reference used (a_total, b_w) are part of that output and become the inputs
of the library's ocrt_ocean for the same case.  Recipes R26 and R28 of the
reference's manual are included with their published values.

It also writes tests/golden/water_iop/: the rows of the reference's pure-water
tables (inputs/water_iop) that bracket every case's wavelength, so that the
library's pure-water model (ocrt_gb300/water_iop.py) is checked against the
a_total and b_total the reference printed without shipping the full tables.

Only runnable where the reference sources exist (the CLI reads its tables
from code/OCRT_C/inputs); the JSON it writes is committed.

    OCRT_REF_ROOT=<reference checkout> make -C oracle ref && \\
        OCRT_REF_ROOT=<reference checkout> python tests/golden/make_golden_ocean.py
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "reference_ocean.json")
CLI = os.path.join(ROOT, "oracle", "_ref", "ocrt")
REF_WD = os.path.join(os.environ.get("OCRT_REF_ROOT", ""), "code", "OCRT_C")

GAS_OFF = sum([[f"--gas-column-{g}", "0"] for g in ("h2o", "o3", "no2", "o2", "co2", "ch4")], [])


def cases():
    out = []

    def add(name, sza, vza, raa, wl, wind, adom=0.0, n_mu_water=None, m_max=None, n_layers=None, T=20.0, note=""):
        out.append({"name": name, "sza_deg": sza, "vza_deg": vza, "raa_deg": raa, "wavelength_nm": wl,
                    "wind_speed": wind, "adom440": adom, "n_mu_water": n_mu_water, "m_max": m_max,
                    "n_layers": n_layers, "T_water": T, "note": note})

    add("R26", 40.0, 30.0, 90.0, 555.0, 3.0, note="recipe R26: pure seawater under a molecular atmosphere")
    add("R28", 40.0, 30.0, 90.0, 555.0, 3.0, adom=0.1, note="recipe R28: CDOM absorption added")
    add("blue_high_wind", 60.0, 10.0, 150.0, 443.0, 7.0)
    add("red_low_wind", 20.0, 45.0, 30.0, 670.0, 1.5)
    add("cdom_412", 35.0, 50.0, 120.0, 412.0, 5.0, adom=0.05)
    add("modes4_n24", 30.0, 40.0, 60.0, 490.0, 4.0, n_mu_water=24, m_max=4,
        note="24 water nodes shared by the atmosphere, Fourier modes 0..4 in both media")
    add("nadir_view_n16", 50.0, 0.0, 0.0, 555.0, 2.0, n_mu_water=16, m_max=3, n_layers=30)
    add("warm_water_t28", 45.0, 20.0, 100.0, 687.5, 5.0, n_mu_water=16, m_max=2, n_layers=30, T=28.0,
        note="28 C water: the temperature term of a_w; a wavelength between table rows")
    return out


def run(spec):
    args = [CLI, "--surface", "ocean", "--sza", str(spec["sza_deg"]), "--vza", str(spec["vza_deg"]),
            "--raa", str(spec["raa_deg"]), "--wavelength", str(spec["wavelength_nm"]), "--pressure", "1013.25",
            "--wind-speed", str(spec["wind_speed"]), "--n-water", "1.34", *GAS_OFF,
            "--water-model", "ocrt", "--water-temperature", str(spec["T_water"]), "--water-salinity", "35",
            "--ocrt-chl", "0", "--ocrt-tsm", "0", "--ocrt-adom440", str(spec["adom440"])]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    if spec["n_mu_water"]:
        args += ["--n-mu-water", str(spec["n_mu_water"])]
        env["OCRT_ADVANCED"] = "1"
    if spec["m_max"] is not None:
        args += ["--m-max", str(spec["m_max"]), "--water-m-max", str(spec["m_max"])]
        env["OCRT_ADVANCED"] = "1"
    if spec["n_layers"]:
        args += ["--n-layers", str(spec["n_layers"])]
    p = subprocess.run(args, cwd=REF_WD, env=env, capture_output=True, text=True, check=True)
    vals = {}
    for tok in p.stdout.split():
        if "=" in tok:
            k, v = tok.split("=", 1)
            try:
                vals[k] = float(v)
            except ValueError:
                pass
    return vals


def reduce_tables(wavelengths):
    """Copy the pure-water table rows within 2 nm of each wavelength."""
    src = os.path.join(REF_WD, "inputs", "water_iop")
    dst = os.path.join(HERE, "water_iop")
    os.makedirs(dst, exist_ok=True)
    for name in ("water_coef_z09_1nm.txt", "psi_T_rottgers2014_OCRT.txt"):
        keep = []
        with open(os.path.join(src, name)) as fh:
            body = False
            for line in fh:
                if line.startswith("/end_header"):
                    body = True
                    continue
                if not body or not line.strip() or line.startswith("#"):
                    continue
                wl = float(line.split()[0])
                if any(abs(wl - w) <= 2.0 for w in wavelengths):
                    keep.append(line)
        with open(os.path.join(dst, name), "w") as fh:
            fh.write(f"# rows of the reference's inputs/water_iop/{name} within 2 nm of the fixture wavelengths\n")
            fh.write("/end_header\n")
            fh.writelines(keep)


def main():
    if not os.path.isdir(REF_WD):
        sys.exit("set OCRT_REF_ROOT to the reference checkout")
    rows = []
    for spec in cases():
        ref = run(spec)
        # the reference's constituent-model path (any CDOM) runs with F_sun = 1,
        # a 15 optical-depth base, at least 300 layers and up to 140 orders
        # (main.c:2960-2980, rt_solver.c:3520-3545); pure seawater with F_sun = pi
        spec["F_sun"] = 1.0 if spec["adom440"] > 0.0 else 3.141592653589793
        spec["water_policy"] = ({"tau_base": 15.0, "n_layers_water": 300, "max_orders_water": 140}
                                if spec["adom440"] > 0.0 else {})
        rows.append({**spec, "reference": ref})
        print(spec["name"], ref["TOA_rho_I"], ref["Rrs0plus_I"], ref["a_total"], ref["b_total"], ref["orders"])
    doc = {
        "source": "reference CLI (oracle/_ref/ocrt) built from code/OCRT_C/src, --surface ocean, pure seawater",
        "published": {
            "R26": {"TOA_rho_I": 4.4074678104e-02, "Rrs0plus_I": 7.978506e-04, "rrs0minus_I": 1.507508e-03,
                    "source": "docs/manual/examples/verification_core_examples.json (R26)"},
            "R28": {"TOA_rho_I": 4.3515055264e-02, "Rrs0plus_I": 5.987734e-04, "rrs0minus_I": 1.132024e-03,
                    "source": "docs/manual/examples/verification_core_examples.json (R28)"},
        },
        "cases": rows,
    }
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    reduce_tables(sorted({r["wavelength_nm"] for r in rows}))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
