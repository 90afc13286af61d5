"""Generate tests/golden/adjoint_fd_config4.json: FP64 central finite
differences of the oracle at the adjoint benchmark's full shape.

Shape: 32 Gauss streams per hemisphere, 200 layers, aerosol moments to
L = 120 (HG g = 0.7, SSA 0.95, AOD 0.1), Fourier modes 0..32, rough Cox-Munk
ocean at 5 m/s, plane-parallel; three geometries of the adjoint workload at
443, 555 and 865 nm.  Derivatives of (rho_I, rho_Q, rho_U) with respect to
every 20th layer optical depth and single-scattering albedo (layers 0, 20,
..., 180 and 199) and the wind speed, by central differences with a relative
step of 1e-6 on the FP64 oracle with a fixed order count (tolerance 1e-300,
45 orders: every mode of these cases converges to 1e-13 within 35), so every
evaluation sums the same orders.

TEST INFRASTRUCTURE: runs the oracle (oracle/_build/liboracle.so) in a
process pool; the JSON it writes is committed and travels with the tests.

    make -C oracle oracle && python tests/golden/make_golden_adjoint.py
"""
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "adjoint_fd_config4.json")

N_MU, N_LAYERS, M_MAX, L_AER, FD_ORDERS, REL_STEP = 32, 200, 32, 120, 45, 1e-6
LAYER_SUBSET = list(range(0, N_LAYERS, 20)) + [N_LAYERS - 1]
BANDS = (443.0, 555.0, 865.0)


def _paths():
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def pixel_specs(seed=20261203 + 4):
    """Three geometries of the adjoint workload's distribution (sza U[0,70],
    vza U[0,60], raa U[0,180]), one per band."""
    rng = np.random.default_rng(seed)
    sza, vza, raa = rng.uniform(0, 70, 3), rng.uniform(0, 60, 3), rng.uniform(0, 180, 3)
    return [{"sza_deg": float(sza[i]), "vza_deg": float(vza[i]), "raa_deg": float(raa[i]),
             "wavelength_nm": BANDS[i], "wind_speed": 5.0, "tau_r_input": 0.0945 * (BANDS[i] / 555.0) ** -4.08}
            for i in range(3)]


def inputs(spec, fd):
    _paths()
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="black_fresnel_ocean", **spec)
    o = A.default_opts(n_mu=N_MU, n_layers=N_LAYERS, fourier_m_max=M_MAX, tau_r_source=A.TAU_R_FROM_INPUT,
                       max_orders=FD_ORDERS if fd else 1000, tolerance=1e-300 if fd else 1e-7)
    aer = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, L_AER))
    return c, o, aer


_ORC = None


def _oracle():
    global _ORC
    if _ORC is None:
        _paths()
        from _helpers import Oracle
        _ORC = Oracle(os.path.join(ROOT, "oracle", "_build", "liboracle.so"))
    return _ORC


def _solve(job):
    """One oracle solve with parameter `kind` (dtau/ssa/wind/None) moved by delta."""
    spec, kind, l, delta = job
    import copy
    orc = _oracle()
    c, o, aer = inputs(spec, fd=True)
    dt, ss = orc.layer_defaults(c, o, aer)
    if kind == "dtau":
        dt[l] += delta
    elif kind == "ssa":
        ss[l] += delta
    elif kind == "wind":
        c = copy.copy(c)
        c.wind_speed += delta
    r = orc.solve_layers(c, o, aer, dt, ss)
    return [r["rho_I"], r["rho_Q"], r["rho_U"]]


def main():
    _paths()
    orc = _oracle()
    params = [("dtau", l) for l in LAYER_SUBSET] + [("ssa", l) for l in LAYER_SUBSET] + [("wind", None)]
    rows = []
    ctx = mp.get_context("spawn")
    with ctx.Pool(os.cpu_count()) as pool:
        for spec in pixel_specs():
            c, o, aer = inputs(spec, fd=True)
            dt, ss = orc.layer_defaults(c, o, aer)
            jobs, steps, one_sided = [], [], []
            for kind, l in params:
                x = dt[l] if kind == "dtau" else (ss[l] if kind == "ssa" else c.wind_speed)
                h = REL_STEP * x
                steps.append(h)
                # an albedo at its upper bound (pure Rayleigh layers) takes the
                # second-order one-sided difference (3 f(0) - 4 f(-h) + f(-2h)) / 2h
                one_sided.append(kind == "ssa" and x + h > 1.0)
                jobs += [(spec, kind, l, 0.0 if one_sided[-1] else h), (spec, kind, l, -h)]
                if one_sided[-1]:
                    jobs.append((spec, kind, l, -2.0 * h))
            vals = np.array(pool.map(_solve, jobs))
            cols, j = [], 0
            for i in range(len(params)):
                if one_sided[i]:
                    cols.append((3.0 * vals[j] - 4.0 * vals[j + 1] + vals[j + 2]) / (2.0 * steps[i]))
                    j += 3
                else:
                    cols.append((vals[j] - vals[j + 1]) / (2.0 * steps[i]))
                    j += 2
            jac = np.stack(cols, axis=1)
            base = _solve((spec, None, 0, 0.0))
            rows.append({"case": spec, "rho_fd_orders": base, "jacobian": jac.tolist()})
            print(spec["wavelength_nm"], base, np.abs(jac).max(axis=1))
    doc = {
        "source": "FP64 oracle (oracle/ocrt_oracle.c), central differences, tests/golden/make_golden_adjoint.py",
        "shape": {"n_mu": N_MU, "n_layers": N_LAYERS, "fourier_m_max": M_MAX, "aerosol": {"g": 0.7, "L": L_AER,
                  "tau_a": 0.1, "ssa_a": 0.95}, "surface": "black_fresnel_ocean", "fd_orders": FD_ORDERS,
                  "rel_step": REL_STEP},
        "params": [[k, l] for k, l in params],
        "rows": ["rho_I", "rho_Q", "rho_U"],
        "pixels": rows,
    }
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
