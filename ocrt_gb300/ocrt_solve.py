"""Python entry point with the signatures of the reference's ocrt_solve.py
(code/OCRT_Python/ocrt_solve.py:131-206 `solve_reflectances`, and the
`single` / `grid` sub-commands at :279-410), running on the GB300 library.

The reference computes three reflectances per row (ocrt_solve.py:5-10):
  R1 rho_TOA      ocean + atmosphere + aerosol + water-leaving (coupled ocean)
  R2 rho_R        Rayleigh atmosphere over a black Fresnel ocean surface, glint decoupled
  R3 rho_RA_black Rayleigh + aerosol over a black Fresnel ocean surface, glint decoupled
All three are on this path.  R1 runs the coupled solve
(ocrt_gb_solve_batch_ocean) over a water column of pure seawater plus CDOM
(ocrt_gb300/water_iop.py: the reference's pure-water tables, read from
$OCRT_GB_WATER_IOP, $OCRT_GB_INPUTS/water_iop or inputs/water_iop, and a_cdom = a440
exp(-S (lambda - 440))); with CDOM the reference's constituent-path policy
applies (optical-depth base 15, at least 300 water layers, up to 140 water
orders; rt_solver.c:3520-3545).  Chlorophyll, TSM and detritus need the
constituent tables and the hydrosol .mie models and raise; a caller that has
its own water IOPs passes water_iop=(a_total, b_water).  gas_on (default True, as in the reference) loads the AFGL
US76 atmosphere and the six cross-section tables once (ocrt_solve.py:41-45)
from $OCRT_GB_INPUTS/afgl_atm and $OCRT_GB_INPUTS/xsec, or inputs/afgl_atm and
inputs/xsec under the working directory, and folds the per-layer absorption
into every solve.  The aerosol, as in the reference (ocrt_solve.py:48-53,
143-147), is the .mie model named by aer_name (a path, or a name resolved as
<name>.mie under $OCRT_GB_MIE_DIR or data/) with aod865 its AOD at 865 nm,
prepared at the row's wavelength by the library (ocrt_gb_mie_prepare: the
log10-linear truncation, moments to L = 80, the value kernel); aer_name may
instead be a synthetic expansion spec "HG:g,ssa[,L]" (Henyey-Greenstein
beta_l = (2l+1) g^l with the Rayleigh-form gamma_2/alpha_2 x 0.3), where
aod865 is the AOD at the row's wavelength.
"""
import argparse
import csv
import os
import sys

import numpy as np

from . import _abi as A
from . import GasState, solve_batch, solve_batch_ocean
from .water_iop import PureWater, default_directory

DEPOL = 0.0279
_STATE = {}
_NO_AEROSOL = A.AerosolHolder(0.0, 1.0, [1.0, 0, 0], [0] * 3, [0] * 3, [0] * 3)


def _pure_water():
    if "pw" not in _STATE:
        _STATE["pw"] = PureWater(default_directory())
    return _STATE["pw"]


def _absorption():
    """The gas state, made once per process (the reference's lazy singleton)."""
    if "ab" not in _STATE:
        root = os.environ.get("OCRT_GB_INPUTS") or "inputs"
        _STATE["ab"] = GasState(os.path.join(root, "afgl_atm"), os.path.join(root, "xsec"), "usstd76")
    return _STATE["ab"]


def _mie_model(name):
    """The .mie model of aer_name, read once per process."""
    from . import MieModel
    key = ("mie", name)
    if key not in _STATE:
        path = name
        if not os.path.exists(path):
            fn = name if name.endswith(".mie") else name + ".mie"
            path = os.path.join(os.environ.get("OCRT_GB_MIE_DIR") or "data", fn)
        _STATE[key] = MieModel(path)
    return _STATE[key]


def _hg(spec, aod, wl_nm=None, value_kernel=True):
    if not isinstance(spec, str) or not spec.upper().startswith("HG:"):
        if wl_nm is None:
            raise ValueError("a .mie aerosol needs the wavelength")
        return _mie_model(spec).prepare(wl_nm, aod, 865.0, L_max=80, value_kernel=value_kernel)
    parts = [float(x) for x in spec[3:].split(",")]
    g, ssa = parts[0], parts[1]
    L = int(parts[2]) if len(parts) > 2 else 80
    l = np.arange(L + 1, dtype=np.float64)
    beta = (2.0 * l + 1.0) * g ** l
    gamma, alpha, zeta = np.zeros(L + 1), np.zeros(L + 1), np.zeros(L + 1)
    Ar = 2.0 * (1.0 - DEPOL) / (2.0 + DEPOL)
    gamma[2], alpha[2] = 0.3 * (-Ar * np.sqrt(1.5)), 0.3 * 3.0 * Ar
    return A.AerosolHolder(aod, ssa, beta, gamma, alpha, zeta)


def _rows_to_cases(rows, which, fourier_m_max, nt_atm, pressure_hpa, max_it=100, gas=None):
    """Cases of the R2 / R3 solves of every row (ocrt_solve.py:160-177)."""
    out = []
    g = gas.handle if gas is not None else None
    for r in rows:
        base = dict(sza_deg=r["sza"], vza_deg=r["vza"], raa_deg=r["raa"], wavelength_nm=r["wl_nm"],
                    wind_speed=r["wind"], surface="black_fresnel_ocean", pressure_hpa=pressure_hpa,
                    decouple_sunglint=1)
        if "R2" in which:
            out.append(("R2", r, A.default_case(**base),
                        A.default_opts(n_mu=24, n_layers=nt_atm, fourier_m_max=2, max_orders=max_it, gas=g), None))
        if "R3" in which:
            out.append(("R3", r, A.default_case(**base),
                        A.default_opts(n_mu=24, n_layers=nt_atm, fourier_m_max=fourier_m_max, max_orders=max_it,
                                       gas=g),
                        _hg(r["aer_name"], r["aod865"], r["wl_nm"])))
    return out


def _water_column(r, n_mu_water, fourier_m_max, max_it_water):
    """The ocrt_ocean of a row's R1 solve (ocrt_solve.py:171-189 of the reference)."""
    if r.get("water_iop") is not None:
        a_tot, b_w = r["water_iop"]
        cdom = False
    else:
        if r.get("chl", 0.0) > 0.0 or r.get("tsm", 0.0) > 0.0 or r.get("det_a440", 0.0) > 0.0:
            raise NotImplementedError("R1 with chlorophyll, TSM or detritus needs the constituent tables and the "
                                      "hydrosol .mie models; pass water_iop=(a_total, b_water) instead")
        a_tot, b_w = _pure_water().iops(r["wl_nm"], r.get("T_water", 20.0), r.get("acdom440", 0.0),
                                        r.get("cdom_slope", 0.014))
        cdom = r.get("acdom440", 0.0) > 0.0
    kw = dict(n_mu_water=n_mu_water, m_max_water=fourier_m_max, max_orders_water=max_it_water)
    if cdom:
        kw.update(tau_base=15.0, n_layers_water=300, max_orders_water=140)
    return A.OceanHolder(a_tot, b_w, **kw)


def _solve_r1(rows, outs, fourier_m_max, nt_atm, pressure_hpa, gas, n_mu_water, max_it_water):
    g = gas.handle if gas is not None else None
    cases, opts, oceans, aers = [], [], [], []
    for r in rows:
        cases.append(A.default_case(sza_deg=r["sza"], vza_deg=r["vza"], raa_deg=r["raa"], wavelength_nm=r["wl_nm"],
                                    wind_speed=r["wind"], surface="ocean", pressure_hpa=pressure_hpa))
        opts.append(A.default_opts(n_layers=nt_atm, fourier_m_max=fourier_m_max, max_orders=100, gas=g))
        oceans.append(_water_column(r, n_mu_water, fourier_m_max, max_it_water))
        # the coupled solve takes the moment kernel (the value kernel is not on that path)
        aers.append(_hg(r["aer_name"], r["aod865"], r["wl_nm"], value_kernel=False) if r["aod865"] > 0.0
                    else _NO_AEROSOL)
    res = solve_batch_ocean(cases, opts, oceans, aers)
    for o, x in zip(outs, res):
        o["rho_TOA_I"], o["rho_TOA_Q"], o["rho_TOA_U"] = x["rho_I"], x["rho_Q"], x["rho_U"]
        o["Rrs"], o["Rrs_Q"], o["Rrs_U"] = x["Rrs_0plus_I"], x["Rrs_0plus_Q"], x["Rrs_0plus_U"]
        o["rrs0minus"], o["rrs0minus_Q"], o["rrs0minus_U"] = x["rrs_0minus_I"], x["rrs_0minus_Q"], x["rrs_0minus_U"]
        o["orders"], o["conv"] = x["orders_water"], x["converged_water"]


def _solve_rows(rows, which, fourier_m_max, nt_atm, pressure_hpa, gas_on, n_mu_water=48, max_it_water=500):
    which = tuple(which)
    gas = _absorption() if gas_on else None
    jobs = _rows_to_cases(rows, which, fourier_m_max, nt_atm, pressure_hpa, gas=gas)
    outs = [dict(wavelength_nm=r["wl_nm"], sza=r["sza"], vza=r["vza"], raa=r["raa"], wind=r["wind"],
                 aod865=r["aod865"], aer_model=r["aer_name"], aod_band=r["aod865"]) for r in rows]
    if "R1" in which:
        _solve_r1(rows, outs, fourier_m_max, nt_atm, pressure_hpa, gas, n_mu_water, max_it_water)
    index = {id(r): i for i, r in enumerate(rows)}
    if jobs:
        res = solve_batch([j[2] for j in jobs], [j[3] for j in jobs],
                          [j[4] if j[4] is not None else _NO_AEROSOL for j in jobs])
        for k, (tag, r, *_rest) in enumerate(jobs):
            o = outs[index[id(r)]]
            key = "rho_R" if tag == "R2" else "rho_RA_black"
            o[key + "_I"], o[key + "_Q"], o[key + "_U"] = (float(res["rho_I"][k]), float(res["rho_Q"][k]),
                                                           float(res["rho_U"][k]))
    for o in outs:
        if "R1" in which and "R2" in which:
            o["rho_RC_I"] = o["rho_TOA_I"] - o["rho_R_I"]
        if "R2" in which and "R3" in which:
            o["rho_AplusRA_I"] = o["rho_RA_black_I"] - o["rho_R_I"]
        if "R1" in which and "R3" in which:
            o["t_rho_w_I"] = o["rho_TOA_I"] - o["rho_RA_black_I"]
    return outs


def solve_reflectances(wl_nm, sza, vza, raa, wind, chl, tsm, acdom440,
                       aod865, aer_name, which=('R1', 'R2', 'R3'),
                       phyto_group='micro', tsm_species='red_clay',
                       n_mu_water=48, fourier_m_max=16, nt_atm=400,
                       max_it_water=500, pressure_hpa=1013.25,
                       gas_on=True, cdom_slope=0.014,
                       det_a440=0.0, det_slope=0.0109, water_iop=None, water_temperature_c=20.0):
    """Same signature as the reference (plus water_iop and
    water_temperature_c); see the module docstring for what is on this path.
    The water arguments only feed R1."""
    row = dict(wl_nm=wl_nm, sza=sza, vza=vza, raa=raa, wind=wind, aod865=aod865, aer_name=aer_name, chl=chl,
               tsm=tsm, acdom440=acdom440, cdom_slope=cdom_slope, det_a440=det_a440, water_iop=water_iop,
               T_water=water_temperature_c)
    out = _solve_rows([row], which, fourier_m_max, nt_atm, pressure_hpa, gas_on, n_mu_water, max_it_water)[0]
    if "R1" in which:
        out.update(chl=chl, tsm=tsm, acdom440=acdom440, adom_slope=cdom_slope, detritus_a440=det_a440,
                   detritus_slope=det_slope)
    return out


def cmd_single(a):
    out = solve_reflectances(a.wl, a.sza, a.vza, a.raa, a.wind, a.chl, a.tsm, a.acdom440, a.aod865, a.aer,
                             which=a.which, fourier_m_max=a.m_max, nt_atm=a.n_layers, pressure_hpa=a.pressure,
                             gas_on=not a.no_gas, n_mu_water=a.n_mu_water, max_it_water=a.max_it_water,
                             cdom_slope=a.cdom_slope)
    for k, v in out.items():
        print(f"{k}={v}")
    return 0


def cmd_grid(a):
    """Rows of a CSV (columns sza, vza, raa, wind, aod865, aer, optional chl,
    tsm, acdom440, and wl or one run per --bands) solved in one batched call
    per reflectance, written to --out."""
    with open(a.grid) as fh:
        src = list(csv.DictReader(fh))
    rows = []
    for r in src:
        bands = [float(r["wl"])] if "wl" in r and r["wl"] else a.bands
        for wl in bands:
            rows.append(dict(wl_nm=float(wl), sza=float(r["sza"]), vza=float(r["vza"]), raa=float(r["raa"]),
                             wind=float(r["wind"]), aod865=float(r.get("aod865", 0.0) or 0.0),
                             aer_name=r.get("aer", a.aer) or a.aer, chl=float(r.get("chl", 0.0) or 0.0),
                             tsm=float(r.get("tsm", 0.0) or 0.0), acdom440=float(r.get("acdom440", 0.0) or 0.0),
                             cdom_slope=a.cdom_slope))
    outs = _solve_rows(rows, a.which, a.m_max, a.n_layers, a.pressure, not a.no_gas, a.n_mu_water, a.max_it_water)
    keys = sorted({k for o in outs for k in o})
    with open(a.out, "w", newline="") as fh:
        w = csv.DictWriter(fh, fieldnames=keys)
        w.writeheader()
        w.writerows(outs)
    print(f"wrote {len(outs)} rows to {a.out}")
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description="GB300 OCRT reflectances (R1/R2/R3)")
    sub = ap.add_subparsers(dest="cmd", required=True)

    def common(p):
        p.add_argument("--which", nargs="+", default=["R1", "R2", "R3"], choices=["R1", "R2", "R3"])
        p.add_argument("--n-mu-water", type=int, default=48)
        p.add_argument("--max-it-water", type=int, default=500)
        p.add_argument("--cdom-slope", type=float, default=0.014)
        p.add_argument("--m-max", type=int, default=16)
        p.add_argument("--n-layers", type=int, default=400)
        p.add_argument("--pressure", type=float, default=1013.25)
        p.add_argument("--no-gas", action="store_true")
        p.add_argument("--aer", default="HG:0.7,0.95,80")

    ps = sub.add_parser("single")
    common(ps)
    for k in ("wl", "sza", "vza", "raa", "wind"):
        ps.add_argument("--" + k, type=float, required=True)
    for k in ("chl", "tsm", "acdom440", "aod865"):
        ps.add_argument("--" + k, type=float, default=0.0)
    pg = sub.add_parser("grid")
    common(pg)
    pg.add_argument("--grid", required=True)
    pg.add_argument("--out", required=True)
    pg.add_argument("--bands", type=float, nargs="+", default=[443.0, 555.0, 865.0])
    a = ap.parse_args(argv)
    return cmd_single(a) if a.cmd == "single" else cmd_grid(a)


if __name__ == "__main__":
    sys.exit(main())
