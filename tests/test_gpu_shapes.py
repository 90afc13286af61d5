"""GPU parity at the full shapes of the benchmark configurations.

* Configuration 2 over its whole mode range (m = 0..2L+1 = 241; 32 streams,
  400 layers, aerosol moments to L = 120, IPSS on).  The reference caps the
  mode count at 32 (rt_solver.c:630), so modes 33..241 are checked against the
  FP64 oracle only; the m <= 32 truncation is pinned to the reference by the
  `config2_aerosol_m32` fixture.  Every mode's TOA view value is compared, and
  the per-mode order counts must agree within one order (the FP32 convergence
  norm against the oracle's FP64 one).
* Configuration 4 (the adjoint) at its full shape: 32 streams, 200 layers,
  L = 120, m <= 32, against FP64 central finite differences of the oracle
  (tests/golden/adjoint_fd_config4.json, made by make_golden_adjoint.py) over
  every 20th layer's optical depth and albedo plus the wind speed, for all
  three rows of the Jacobian.  Bound as in test_gpu_adjoint.py: 1e-4 of the
  largest derivative of each group.

Configuration 3 at full shape (32 streams, m <= 32, L = 120, 200 and 400
layers) is in tests/golden/reference_cases.json (`config3_full_*`) and runs
through test_gpu_parity.py against the reference's own outputs.
"""
import json
import os

import numpy as np
import pytest

from _helpers import HERE, assert_parity

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-4


def _config2(A, m_max, sza, vza, raa):
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, 120))
    c = A.default_case(surface="black_fresnel_ocean", wind_speed=5.0, sza_deg=sza, vza_deg=vza, raa_deg=raa,
                       tau_r_input=0.0945, wavelength_nm=555.0)
    o = A.default_opts(n_mu=32, n_layers=400, fourier_m_max=m_max, tau_r_source=A.TAU_R_FROM_INPUT,
                       max_orders=1000, tolerance=1e-7, pssa=1)
    return c, o, aer


@pytest.mark.parametrize("geom", [(40.0, 55.0, 90.0), (40.0, 38.0, 178.0), (30.0, 30.0, 2.0)],
                         ids=["config2_geometry", "near_backscatter", "near_glint"])
def test_config2_full_mode_range(gpu, oracle, geom):
    from ocrt_gb300 import _abi as A
    c, o, aer = _config2(A, 241, *geom)
    got = gpu.solve_case(c, o, aer, diag=True)
    ref = oracle.solve(c, o, aer, diag=True)
    relI, dQ, dU = assert_parity(got, ref, f"config 2, m <= 241, {geom}")
    print(f"config 2 m<=241 {geom}: rho_I rel {relI:.2e}, |dQ| {dQ:.2e}, |dU| {dU:.2e}, "
          f"kappa {abs(got['kappa_ipss'] - ref['kappa_ipss']):.1e}, order-modes {got['order_modes']} "
          f"(oracle {ref['order_modes']})")
    # every mode's TOA view value, against the size of the reconstructed total
    for k, tot, tol in (("view_I_m", abs(ref["I_TOA"]), 1e-5), ("view_Q_m", 1.0, 1e-4 * np.cos(np.radians(geom[0]))),
                        ("view_U_m", 1.0, 1e-4 * np.cos(np.radians(geom[0])))):
        d = np.abs(np.asarray(got[k]) - np.asarray(ref[k]))
        assert d.max() <= tol * tot, (k, int(d.argmax()), d.max())
    # the high modes carry only the surface coupling, yet must be solved
    assert np.any(np.abs(ref["view_I_m"][33:]) > 0.0)
    d = np.abs(np.asarray(got["orders_per_m"]) - np.asarray(ref["orders_per_m"]))
    assert d.max() <= 1, (list(got["orders_per_m"]), list(ref["orders_per_m"]))
    assert got["converged"] == ref["converged"] == 1


def test_config2_truncation_matches_reference_fixture(gpu):
    """The same solve cut at the reference's m <= 32 cap equals the reference."""
    from _helpers import load_golden
    from ocrt_gb300 import _abi as A
    spec = next(s for s in load_golden()["cases"] if s["name"] == "config2_aerosol_m32")
    c, o, aer = _config2(A, 32, 40.0, 55.0, 90.0)
    for k, v in spec["opts"].items():
        assert getattr(o, k) == v, k
    got = gpu.solve_case(c, o, aer, diag=True)
    assert_parity(got, spec["reference"], "config 2, m <= 32")


def _load_fd():
    with open(os.path.join(HERE, "golden", "adjoint_fd_config4.json")) as fh:
        return json.load(fh)


def test_config4_adjoint_full_shape(gpu, oracle):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    doc = _load_fd()
    sh = doc["shape"]
    aer = A.AerosolHolder(sh["aerosol"]["tau_a"], sh["aerosol"]["ssa_a"],
                          *hg_aerosol_moments(sh["aerosol"]["g"], sh["aerosol"]["L"]))
    cases = [A.default_case(surface="black_fresnel_ocean", **p["case"]) for p in doc["pixels"]]
    o = A.default_opts(n_mu=sh["n_mu"], n_layers=sh["n_layers"], fourier_m_max=sh["fourier_m_max"],
                       tau_r_source=A.TAU_R_FROM_INPUT, max_orders=1000, tolerance=1e-9)
    eye = np.broadcast_to(np.eye(3), (len(cases), 3, 3)).copy()
    res, g = gpu.solve_batch_adjoint(cases, o, [aer] * len(cases), None, eye)
    params = doc["params"]
    it = [i for i, (k, _) in enumerate(params) if k == "dtau"]
    iw = [i for i, (k, _) in enumerate(params) if k == "wind"]
    ls = [params[i][1] for i in it]
    worst = 0.0
    for p, px in enumerate(doc["pixels"]):
        jac = np.asarray(px["jacobian"])
        # the forward values themselves sit at the parity bar against the FP64 oracle
        ref = oracle.solve(cases[p], o, aer)
        assert_parity({k: res[k][p] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"pixel {p}")
        for r in range(3):
            for name, got, fd in (("d/ddtau", g["d_dtau"][p, r, ls], jac[r, it]),
                                  ("d/dssa", g["d_ssa"][p, r, ls], jac[r, [i + len(it) for i in it]]),
                                  ("d/dwind", np.array([g["d_wind"][p, r]]), jac[r, iw])):
                scale = np.max(np.abs(fd))
                err = np.max(np.abs(got - fd))
                worst = max(worst, err / max(scale, 1e-300))
                assert err <= GRAD_REL * scale + 1e-8, \
                    f"pixel {p} row {r} {name}: max err {err:.3e} vs scale {scale:.3e}"
    print(f"configuration-4 adjoint at full shape: worst error {worst:.2e} of the group maximum")
