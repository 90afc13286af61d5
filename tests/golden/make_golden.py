"""Generate tests/golden/reference_cases.json from the reference solver.

Runs the reference C solver compiled from its own sources by oracle/Makefile
(oracle/_ref/libocrt_ref.so, via oracle/ref_driver.c) on a fixed list of
inputs and records its outputs.  Only runnable where the reference sources
exist; the JSON it writes is committed and travels with the tests.

    OCRT_REF_ROOT=<reference checkout> make -C oracle ref && python tests/golden/make_golden.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from ocrt_gb300 import _abi as A  # noqa: E402
from synthetic import batched_forward_pixels, hg_aerosol_moments  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_cases.json")


def case_list():
    cases = []

    def add(name, case, opts, aer=None, note=""):
        cases.append({"name": name, "case": case, "opts": opts, "aerosol": aer, "note": note})

    add("R01", {"surface": 0}, {}, note="recipe R01 (recipe_catalog.json), CLI defaults")
    add("R07", {"surface": 2, "wind_speed": 5.0, "decouple_sunglint": 1}, {}, note="recipe R07")
    add("R07_glint", {"surface": 2, "wind_speed": 5.0}, {})
    add("flat", {"surface": 3}, {})
    add("bfo_wind0", {"surface": 2, "wind_speed": 0.0}, {})
    add("interp_view", {"surface": 0}, {"view_as_node": 0})
    add("nadir_view_zenith_sun", {"surface": 2, "wind_speed": 3.0, "sza_deg": 0.3, "vza_deg": 0.0, "raa_deg": 10.0}, {})
    add("ipss_us62_sza75", {"surface": 2, "wind_speed": 5.0, "sza_deg": 75.0, "vza_deg": 55.0},
        {"pssa": 1, "n_layers": 100})
    add("ipss_exp8km", {"surface": 2, "wind_speed": 5.0, "vza_deg": 55.0},
        {"pssa": 1, "n_layers": 100, "rayleigh_profile": 1, "rayleigh_h_km": 8.0})
    aer40 = {"g": 0.7, "L": 40, "tau_a": 0.1, "ssa_a": 0.95}
    add("aerosol_L40", {"surface": 2, "wind_speed": 5.0}, {"n_layers": 50, "fourier_m_max": 8}, aer40)
    add("aerosol_ipss", {"surface": 2, "wind_speed": 5.0, "sza_deg": 60.0},
        {"n_layers": 50, "fourier_m_max": 4, "pssa": 1}, aer40)
    add("high_sza_low_wind", {"surface": 2, "wind_speed": 1.74, "sza_deg": 79.6, "vza_deg": 13.5, "raa_deg": 74.1,
                              "tau_r_input": 0.0945, "wavelength_nm": 555.0},
        {"n_mu": 16, "n_layers": 50, "fourier_m_max": 6, "tau_r_source": 1, "max_orders": 200},
        {"g": 0.65, "L": 30, "tau_a": 0.244, "ssa_a": 0.9})
    add("config1_rayleigh_400", {"surface": 2, "wind_speed": 5.0, "sza_deg": 40.0, "vza_deg": 55.0, "raa_deg": 90.0,
                                 "tau_r_input": 0.0945},
        {"n_mu": 24, "n_layers": 400, "fourier_m_max": 2, "tau_r_source": 1, "max_orders": 1000, "pssa": 1,
         "rayleigh_profile": 1, "rayleigh_h_km": 8.0},
        note="configuration 1: Rayleigh 0.0945 over 400 layers, exponential 8 km profile for IPSS")
    add("config2_aerosol_m32", {"surface": 2, "wind_speed": 5.0, "sza_deg": 40.0, "vza_deg": 55.0, "raa_deg": 90.0,
                                "tau_r_input": 0.0945},
        {"n_mu": 32, "n_layers": 400, "fourier_m_max": 32, "tau_r_source": 1, "max_orders": 1000, "pssa": 1},
        {"g": 0.7, "L": 120, "tau_a": 0.1, "ssa_a": 0.95},
        note="configuration 2 at the reference's mode cap m <= 32")
    p = batched_forward_pixels(8, seed=11)
    for i in range(8):
        add(f"batch_like_{i}", {"surface": 2, "wind_speed": float(p["wind"][i]), "sza_deg": float(p["sza"][i]),
                                "vza_deg": float(p["vza"][i]), "raa_deg": float(p["raa"][i]),
                                "wavelength_nm": float(p["wavelength"][i]), "tau_r_input": float(p["tau_r"][i])},
            {"n_mu": 16 + 4 * (i % 3), "n_layers": int(p["n_layers"][i]) // 4, "fourier_m_max": 8, "tau_r_source": 1,
             "max_orders": 500},
            {"g": float(p["g"][i]), "L": 60, "tau_a": float(p["aod"][i]), "ssa_a": float(p["ssa"][i])},
            note="configuration-3 distribution, reduced layers and modes")
    # configuration 3 at its full shape: the first three 400-layer and the
    # first three 200-layer pixels of the batched-forward workload's own draw
    q = batched_forward_pixels(4096)
    picked = [i for i in range(4096) if q["n_layers"][i] == 400][:3] + \
             [i for i in range(4096) if q["n_layers"][i] == 200][:3]
    for i in picked:
        add(f"config3_full_{i}", {"surface": 2, "wind_speed": float(q["wind"][i]), "sza_deg": float(q["sza"][i]),
                                  "vza_deg": float(q["vza"][i]), "raa_deg": float(q["raa"][i]),
                                  "wavelength_nm": float(q["wavelength"][i]), "tau_r_input": float(q["tau_r"][i])},
            {"n_mu": 32, "n_layers": int(q["n_layers"][i]), "fourier_m_max": 32, "tau_r_source": 1,
             "max_orders": 1000},
            {"g": float(q["g"][i]), "L": 120, "tau_a": float(q["aod"][i]), "ssa_a": float(q["ssa"][i])},
            note="configuration 3 at full shape (N 32, m <= 32, L 120), pixel i of the 4096-pixel draw")
    return cases


def build_inputs(spec):
    c = A.default_case(**spec["case"])
    o = A.default_opts(**spec["opts"])
    aer = None
    if spec["aerosol"]:
        a = spec["aerosol"]
        aer = A.AerosolHolder(a["tau_a"], a["ssa_a"], *hg_aerosol_moments(a["g"], a["L"]))
    return c, o, aer


def run(lib, prefix, spec):
    f = A.bind_solver(lib, prefix)
    c, o, aer = build_inputs(spec)
    n = o.fourier_m_max + 1
    arr = {"orders_per_m": (C.c_int * n)(), "residual_per_m": (C.c_double * n)(), "view_I_m": (C.c_double * n)(),
           "view_Q_m": (C.c_double * n)(), "view_U_m": (C.c_double * n)()}
    d = A.Diag(**{k: C.cast(v, A.Diag._fields_[i][1]) for i, (k, v) in enumerate(arr.items())})
    r = A.Result()
    rc = f(C.byref(c), C.byref(o), C.byref(aer.struct) if aer else None, C.byref(r), C.byref(d))
    out = A.result_dict(r)
    out.update({k: list(v[:]) for k, v in arr.items()})
    return rc, out


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so"))
    rows = []
    for spec in case_list():
        rc, out = run(lib, "ocrt_ref", spec)
        assert rc == 0, (spec["name"], rc)
        if spec["opts"].get("rayleigh_profile", 0) != 1 or not spec["opts"].get("pssa", 0):
            out["kappa_ipss"] = None   # the reference does not export kappa on its own IPSS path
        rows.append({**spec, "reference": out})
        print(spec["name"], out["rho_I"], out["rho_Q"], out["rho_U"], out["order_modes"])
    doc = {
        "source": "reference C solver built from code/OCRT_C/src by oracle/Makefile, driven by oracle/ref_driver.c",
        "published": {
            "R01": {"rho_I": 3.9251609571e-02, "rho_Q": 6.6709086582e-03, "rho_U": -1.2524744881e-02,
                    "source": "docs/manual/examples/verification_core_examples.json (R01)"},
            "R07": {"rho_I": 4.1798373685e-02, "rho_Q": 7.205165675e-03, "rho_U": -1.2404692357e-02,
                    "source": "docs/manual/examples/verification_core_examples.json (R07)"},
        },
        "cases": rows,
    }
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
