"""Generate tests/golden/reference_lut.json: angle-grid LUT outputs of the
reference solver (rt_solve_case_pol_lut through oracle/ref_driver.c, compiled
from the reference's own sources by oracle/Makefile).  Only runnable where the
reference sources exist; the JSON it writes is committed.

    OCRT_REF_ROOT=<reference checkout> make -C oracle ref && python tests/golden/make_golden_lut.py
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
from synthetic import hg_aerosol_moments  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_lut.json")
VZA = list(np.arange(0.0, 81.0, 10.0))
RAA = list(np.arange(0.0, 360.0, 60.0))


def lut_cases():
    aer = {"g": 0.7, "L": 24, "tau_a": 0.1, "ssa_a": 0.95}
    return [
        {"name": "lut_rough_aerosol", "case": {"surface": 2, "wind_speed": 5.0, "sza_deg": 40.0, "vza_deg": 0.0,
                                               "raa_deg": 0.0},
         "opts": {"n_mu": 16, "n_layers": 40, "fourier_m_max": 6, "max_orders": 200}, "aerosol": aer},
        {"name": "lut_rough_aerosol_ipss", "case": {"surface": 2, "wind_speed": 7.0, "sza_deg": 60.0,
                                                    "vza_deg": 0.0, "raa_deg": 0.0},
         "opts": {"n_mu": 16, "n_layers": 40, "fourier_m_max": 6, "max_orders": 200, "pssa": 1}, "aerosol": aer},
        {"name": "lut_black_rayleigh", "case": {"surface": 0, "sza_deg": 30.0, "vza_deg": 0.0, "raa_deg": 0.0},
         "opts": {"n_mu": 24, "n_layers": 40, "fourier_m_max": 2, "max_orders": 100}, "aerosol": None},
        {"name": "lut_flat_view_interp", "case": {"surface": 3, "sza_deg": 45.0, "vza_deg": 33.0, "raa_deg": 20.0},
         "opts": {"n_mu": 8, "n_layers": 20, "fourier_m_max": 4, "max_orders": 100, "view_as_node": 0},
         "aerosol": None},
    ]


def inputs(spec):
    c = A.default_case(**spec["case"])
    o = A.default_opts(**spec["opts"])
    a = None
    if spec["aerosol"]:
        x = spec["aerosol"]
        a = A.AerosolHolder(x["tau_a"], x["ssa_a"], *hg_aerosol_moments(x["g"], x["L"]))
    return c, o, a


def run(lib, fn, spec):
    c, o, a = inputs(spec)
    lut = A.LutHolder(VZA, RAA)
    r = A.Result()
    f = getattr(lib, fn)
    f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Result),
                  C.POINTER(A.Lut)]
    rc = f(C.byref(c), C.byref(o), C.byref(a.struct) if a else None, C.byref(r), C.byref(lut.struct))
    if rc:
        raise RuntimeError(f"{fn} rc {rc}")
    return {**{k: lut.out[k].tolist() for k in A.LUT_FIELDS}, "T_dir_dn": lut.struct.T_dir_dn,
            "T_diff_dn_hemi": lut.struct.T_diff_dn_hemi}


def main():
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so"))
    doc = {"vza_deg": VZA, "raa_deg": RAA, "cases": []}
    for spec in lut_cases():
        doc["cases"].append({**spec, "reference": run(ref, "ocrt_ref_solve_case_lut", spec)})
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
