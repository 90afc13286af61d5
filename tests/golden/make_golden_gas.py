"""Generate the gas-absorption fixtures: tests/golden/gas_data/ and
tests/golden/reference_gas.json.

1. gas_data/afgl_atm/: the AFGL atmospheres used by the tests, copied from the
   reference's inputs/afgl_atm (public standard-atmosphere data).
2. gas_data/xsec/: the reference's six cross-section tables (inputs/xsec)
   reduced to the wavelength columns the fixture wavelengths interpolate
   between, plus the 330 and 1100 nm grid ends the loader requires.  Values are
   copied as the original text tokens, so at the fixture wavelengths the
   reduced tables interpolate to the same numbers as the full ones (checked
   below against the reference on the full tables).
3. reference_gas.json: outputs of the reference C solver built from its own
   sources (oracle/Makefile -> oracle/_ref, oracle/ref_driver.c) on the reduced
   data: default and effective columns, column absorption depths per gas
   (rt_absorption_tau_per_gas), per-layer absorption depths and level
   altitudes of the gas-loaded atmosphere (the reference's IPSS layer-profile
   dump, rt_solver.c:783-818), and full solves with gas absorption.

Only runnable where the reference sources exist; the outputs are committed.

    OCRT_REF_ROOT=<reference checkout> make -C oracle ref && \
        OCRT_REF_ROOT=<reference checkout> python tests/golden/make_golden_gas.py
"""
import ctypes as C
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from ocrt_gb300 import _abi as A  # noqa: E402
from synthetic import hg_aerosol_moments  # noqa: E402

REF_INPUTS = os.path.join(os.environ.get("OCRT_REF_ROOT", ""), "code", "OCRT_C", "inputs")
DATA = os.path.join(HERE, "gas_data")
OUT = os.path.join(HERE, "reference_gas.json")
GASES = ("h2o", "o3", "o2", "co2", "no2", "ch4")
PROFILES = {"usstd76": 0, "tropical": 1, "mlwint": 3}
WAVELENGTHS = [330.0, 412.5, 443.0, 555.0, 600.3, 687.0, 760.4, 865.0, 940.0, 1100.0]
H2O_G_CM2 = 6.02214076e23 / 18.01528      # main.c:2726
DU = 2.6868e16                             # main.c:2730


def reduce_xsec(src, dst):
    """Keep the header and the wavelength columns bracketing WAVELENGTHS."""
    lines = open(src).read().splitlines()
    data = [i for i, l in enumerate(lines) if l and not l.startswith("#")]
    wl = [float(t) for t in lines[data[0]].split()]
    keep = {0, len(wl) - 1}
    for w in WAVELENGTHS:
        j = int(np.searchsorted(wl, w, side="right")) - 1
        keep.add(j)
        if wl[j] != w:
            keep.add(j + 1)
    keep = sorted(keep)
    out = [l for l in lines if l.startswith("#") and ("layer " not in l or "n_layers" in l)]
    out.insert(1, "# Reduced copy for tests: wavelength columns " + " ".join(f"{wl[j]:g}" for j in keep))
    for i in data:
        toks = lines[i].split()
        out.append(" ".join(toks[j] for j in keep))
    with open(dst, "w") as fh:
        fh.write("\n".join(out) + "\n")


def make_data():
    if os.path.isdir(DATA):
        shutil.rmtree(DATA)
    os.makedirs(os.path.join(DATA, "afgl_atm"))
    os.makedirs(os.path.join(DATA, "xsec"))
    for p in PROFILES:
        shutil.copy(os.path.join(REF_INPUTS, "afgl_atm", f"afgl_{p}.dat"), os.path.join(DATA, "afgl_atm"))
    for g in GASES:
        reduce_xsec(os.path.join(REF_INPUTS, "xsec", f"xsec_{g}.dat"), os.path.join(DATA, "xsec", f"xsec_{g}.dat"))


class Ref:
    def __init__(self):
        self.lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so"))
        L = self.lib
        L.ocrt_ref_gas_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_double),
                                          C.POINTER(C.c_void_p)]
        L.ocrt_ref_gas_destroy.argtypes = [C.c_void_p]
        L.ocrt_ref_gas_tau.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ocrt_ref_gas_columns.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_int)]
        self.solve = A.bind_solver(L, "ocrt_ref")

    def gas(self, root, profile, override):
        h = C.c_void_p()
        ov = (C.c_double * 6)(*override) if override is not None else None
        rc = self.lib.ocrt_ref_gas_create(os.path.join(root, "afgl_atm").encode(), os.path.join(root, "xsec").encode(),
                                          PROFILES[profile], ov, C.byref(h))
        assert rc == 0, rc
        return h

    def tau(self, h, wl):
        per, tot = (C.c_double * 6)(), C.c_double()
        self.lib.ocrt_ref_gas_tau(h, wl, per, C.byref(tot))
        return list(per[:]), tot.value

    def columns(self, h):
        e, d, o = (C.c_double * 6)(), (C.c_double * 6)(), (C.c_int * 6)()
        self.lib.ocrt_ref_gas_columns(h, e, d, o)
        return list(e[:]), list(d[:]), list(o[:])


OVERRIDES = {
    "default": None,
    "all_zero": [0.0] * 6,
    "pwv_o3_no2": [2.5 * H2O_G_CM2, 300.0 * DU, -1.0, -1.0, 0.5 * DU, -1.0],
}

SOLVES = [
    # name, profile, override, case fields, opts fields, aerosol
    ("ray_443_bfo", "usstd76", "default", {"surface": 2, "wind_speed": 5.0, "wavelength_nm": 443.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 4, "max_orders": 200, "tolerance": 1e-9}, None),
    ("aer_555_bfo", "usstd76", "default", {"surface": 2, "wind_speed": 5.0, "wavelength_nm": 555.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 6, "max_orders": 200, "tolerance": 1e-9},
     {"g": 0.7, "L": 40, "tau_a": 0.2, "ssa_a": 0.95}),
    ("ray_760_ipss", "usstd76", "default", {"surface": 2, "wind_speed": 5.0, "wavelength_nm": 760.4,
                                            "sza_deg": 60.0, "vza_deg": 45.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 4, "max_orders": 200, "tolerance": 1e-9, "pssa": 1}, None),
    ("aer_687_black_ipss_tropical", "tropical", "default", {"surface": 0, "wavelength_nm": 687.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 4, "max_orders": 200, "tolerance": 1e-9, "pssa": 1},
     {"g": 0.65, "L": 30, "tau_a": 0.15, "ssa_a": 0.9}),
    ("zero_columns_555", "usstd76", "all_zero", {"surface": 2, "wind_speed": 5.0, "wavelength_nm": 555.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 4, "max_orders": 200, "tolerance": 1e-9}, None),
    ("override_940_flat", "usstd76", "pwv_o3_no2", {"surface": 3, "wavelength_nm": 940.0},
     {"n_mu": 12, "n_layers": 60, "fourier_m_max": 4, "max_orders": 200, "tolerance": 1e-9},
     {"g": 0.7, "L": 40, "tau_a": 0.1, "ssa_a": 0.95}),
    ("aer_600_mlwint_ipss", "mlwint", "default", {"surface": 2, "wind_speed": 3.0, "wavelength_nm": 600.3,
                                                  "sza_deg": 70.0, "vza_deg": 30.0, "raa_deg": 150.0},
     {"n_mu": 16, "n_layers": 80, "fourier_m_max": 8, "max_orders": 300, "tolerance": 1e-9, "pssa": 1},
     {"g": 0.7, "L": 40, "tau_a": 0.3, "ssa_a": 0.95}),
    ("config2_like_865", "usstd76", "default", {"surface": 2, "wind_speed": 5.0, "wavelength_nm": 865.0,
                                                "sza_deg": 40.0, "vza_deg": 55.0, "raa_deg": 90.0},
     {"n_mu": 24, "n_layers": 100, "fourier_m_max": 12, "max_orders": 500, "tolerance": 1e-9},
     {"g": 0.7, "L": 80, "tau_a": 0.1, "ssa_a": 0.95}),
]


def main():
    make_data()
    ref = Ref()
    doc = {"source": "reference C solver built from code/OCRT_C/src by oracle/Makefile, driven by "
                     "oracle/ref_driver.c, on the reduced tables under tests/golden/gas_data",
           "wavelengths": WAVELENGTHS, "overrides": OVERRIDES, "columns": {}, "tau": {}, "layers": [], "solves": []}
    for prof in PROFILES:
        for oname, ov in OVERRIDES.items():
            hf = ref.gas(REF_INPUTS, prof, ov)
            hr = ref.gas(DATA, prof, ov)
            key = f"{prof}/{oname}"
            doc["columns"][key] = dict(zip(("eff", "default", "overridden"), ref.columns(hr)))
            doc["tau"][key] = []
            for wl in WAVELENGTHS:
                full, reduced = ref.tau(hf, wl), ref.tau(hr, wl)
                assert full == reduced, (key, wl, full, reduced)
                doc["tau"][key].append({"per_gas": reduced[0], "total": reduced[1]})
            ref.lib.ocrt_ref_gas_destroy(hf)
            ref.lib.ocrt_ref_gas_destroy(hr)
    for name, prof, oname, cf, of, af in SOLVES:
        h = ref.gas(DATA, prof, OVERRIDES[oname])
        c = A.default_case(**cf)
        o = A.default_opts(**of)
        o.gas = h.value
        aer = A.AerosolHolder(af["tau_a"], af["ssa_a"], *hg_aerosol_moments(af["g"], af["L"])) if af else None
        dump = None
        if of.get("pssa"):
            fd, dump = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            os.environ["OCRT_IPSS_PROFILE_DUMP"] = dump
        r = A.Result()
        rc = ref.solve(C.byref(c), C.byref(o), C.byref(aer.struct) if aer else None, C.byref(r), None)
        os.environ.pop("OCRT_IPSS_PROFILE_DUMP", None)
        assert rc == 0, (name, rc)
        out = A.result_dict(r)
        out["kappa_ipss"] = None    # the reference does not export kappa on its own IPSS path
        doc["solves"].append({"name": name, "profile": prof, "override": oname, "case": cf, "opts": of,
                              "aerosol": af, "reference": out})
        if dump:
            rows = [l.strip().split(",") for l in open(dump) if l[:1].isdigit()]
            os.unlink(dump)
            doc["layers"].append({"name": name, "z_top_km": [float(r_[1]) for r_ in rows],
                                  "z_bot_km": [float(r_[2]) for r_ in rows],
                                  "dtau": [float(r_[3]) for r_ in rows],
                                  "tau_abs": [float(r_[6]) for r_ in rows]})
        ref.lib.ocrt_ref_gas_destroy(h)
        print(name, out["rho_I"], out["rho_Q"], out["rho_U"], out["T_dir_dn"])
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
