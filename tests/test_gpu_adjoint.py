"""Per-layer parameters and the adjoint, through ocrt_gb_solve_batch_adjoint.

The reference has no derivatives, so the adjoint is checked against FP64
central finite differences (relative step 1e-6) of the oracle with the same
per-layer parameters and a fixed order count (tolerance 1e-300, so every FD
evaluation sums the same number of orders and the difference quotient is
smooth).  The GPU adjoint is that of the converged SOS system in FP32 fields.

Tolerance, per parameter group (d/ddtau, d/dssa) and for d/dwind:
    |g_gpu - g_fd| <= 1e-4 * max|g_fd| of the group  (+ 1e-8 absolute)
FP32 fields carry ~1e-6 relative error; a layer derivative is a sum of
competing terms (transport attenuation against source strength), so the
bound is taken relative to the largest derivative of its group.  Measured on
a GB300: 1e-7 .. 7e-6 of the group maximum.
"""
import numpy as np
import pytest

from _helpers import assert_parity, fd_gradient, rho_vec

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-4


def _case(A, surface="black_fresnel_ocean", wind=5.0, **kw):
    return A.default_case(surface=surface, wind_speed=wind, **kw)


def _fd_all(oracle, c, o_fd, aer, dt, ss, cot, with_wind):
    which = [("dtau", l) for l in range(len(dt))] + [("ssa", l) for l in range(len(ss))]
    if with_wind:
        which.append(("wind", None))
    g = fd_gradient(oracle, c, o_fd, aer, dt, ss, cot, which)
    n = len(dt)
    return g[:n], g[n:2 * n], (g[2 * n] if with_wind else 0.0)


def _check_grad(gg, gf, what):
    scale = np.max(np.abs(gf)) if np.ndim(gf) else abs(gf)
    err = np.max(np.abs(np.asarray(gg) - np.asarray(gf)))
    print(f"{what}: max abs err {err:.3e}, scale {scale:.3e}, rel {err / max(scale, 1e-300):.2e}")
    assert err <= GRAD_REL * scale + 1e-8, f"{what}: max err {err:.3e} vs scale {scale:.3e}"
    return err / max(scale, 1e-300)


CASES = [
    # (label, case kwargs, opts kwargs, aerosol (g, L, tau, ssa) or None)
    ("black_aerosol_simt", dict(surface="black", wind=0.0, sza_deg=35.0, vza_deg=20.0, raa_deg=60.0),
     dict(n_mu=8, n_layers=8, fourier_m_max=4), (0.7, 16, 0.15, 0.92)),
    ("rough_aerosol_tc", dict(sza_deg=40.0, vza_deg=55.0, raa_deg=90.0, wavelength_nm=555.0),
     dict(n_mu=16, n_layers=10, fourier_m_max=5), (0.7, 24, 0.1, 0.95)),
    ("rough_rayleigh_interp_view", dict(sza_deg=50.0, vza_deg=33.0, raa_deg=135.0, wavelength_nm=443.0, wind=8.0),
     dict(n_mu=8, n_layers=8, fourier_m_max=3, view_as_node=0), None),
]


@pytest.mark.parametrize("label,ck,ok,ak", CASES, ids=[c[0] for c in CASES])
def test_adjoint_matches_fp64_finite_differences(gpu, oracle, label, ck, ok, ak):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    c = _case(A, **ck)
    o_gpu = A.default_opts(max_orders=400, tolerance=1e-9, **ok)
    o_fd = A.default_opts(max_orders=200, tolerance=1e-300, **ok)
    aer = A.AerosolHolder(ak[2], ak[3], *hg_aerosol_moments(ak[0], ak[1])) if ak else None
    dt, ss = oracle.layer_defaults(c, o_gpu, aer)
    rough = c.surface == 2 and c.wind_speed > 0
    for cot in (np.array([1.0, 0.0, 0.0]), np.array([0.3, -1.0, 0.7])):
        res, g = gpu.solve_batch_adjoint([c], o_gpu, [aer] if aer else None, None, cot[None, None, :])
        fd_t, fd_s, fd_w = _fd_all(oracle, c, o_fd, aer, dt, ss, cot, rough)
        _check_grad(g["d_dtau"][0, 0], fd_t, f"{label} d/ddtau cot={cot}")
        _check_grad(g["d_ssa"][0, 0], fd_s, f"{label} d/dssa cot={cot}")
        if rough:
            _check_grad(g["d_wind"][0, 0], fd_w, f"{label} d/dwind cot={cot}")


def test_layer_overrides_forward_matches_oracle(gpu, oracle):
    """Non-uniform layer depths and albedos: forward parity with the oracle."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(7)
    c = _case(A, sza_deg=30.0, vza_deg=45.0, raa_deg=120.0)
    o = A.default_opts(n_mu=16, n_layers=12, fourier_m_max=6, max_orders=400)
    aer = A.AerosolHolder(0.2, 0.9, *hg_aerosol_moments(0.75, 30))
    dt0, ss0 = oracle.layer_defaults(c, o, aer)
    dt = dt0 * rng.uniform(0.5, 1.8, dt0.size)
    ss = ss0 * rng.uniform(0.85, 1.0, ss0.size)
    ly = A.LayersHolder(o.n_layers, dt, ss)
    res, _ = gpu.solve_batch_adjoint([c], o, [aer], [ly], None)
    ref = oracle.solve_layers(c, o, aer, dt, ss)
    assert_parity({k: res[k][0] for k in ("rho_I", "rho_Q", "rho_U")}, ref, "overrides")
    # overrides equal to the profile values reproduce the plain solve
    res2, _ = gpu.solve_batch_adjoint([c], o, [aer], [A.LayersHolder(o.n_layers, dt0, ss0)], None)
    plain = gpu.solve_case(c, o, aer)
    assert abs(res2["rho_I"][0] - plain["rho_I"]) <= 1e-6 * abs(plain["rho_I"])


def test_adjoint_with_overrides_and_batch_consistency(gpu, oracle):
    """Gradients at non-uniform parameters; the Jacobian (3 identity rows) of a
    pixel inside a mixed batch equals its rows solved alone."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    rng = np.random.default_rng(11)
    cs = [_case(A, sza_deg=25.0 + 10 * i, vza_deg=15.0 + 12 * i, raa_deg=30.0 + 40 * i, wind=3.0 + 2 * i)
          for i in range(3)]
    o_gpu = A.default_opts(n_mu=8, n_layers=8, fourier_m_max=4, max_orders=400, tolerance=1e-9)
    o_fd = A.default_opts(n_mu=8, n_layers=8, fourier_m_max=4, max_orders=200, tolerance=1e-300)
    aers = [A.AerosolHolder(0.05 + 0.05 * i, 0.9, *hg_aerosol_moments(0.65 + 0.05 * i, 20)) for i in range(3)]
    lys, pars = [], []
    for i in range(3):
        dt0, ss0 = oracle.layer_defaults(cs[i], o_gpu, aers[i])
        dt = dt0 * rng.uniform(0.6, 1.5, dt0.size)
        ss = ss0 * rng.uniform(0.9, 1.0, ss0.size)
        lys.append(A.LayersHolder(o_gpu.n_layers, dt, ss))
        pars.append((dt, ss))
    eye = np.broadcast_to(np.eye(3), (3, 3, 3)).copy()
    res, g = gpu.solve_batch_adjoint(cs, o_gpu, aers, lys, eye)
    # pixel 1, row Q against FD at its own parameters
    dt, ss = pars[1]
    fd_t, fd_s, fd_w = _fd_all(oracle, cs[1], o_fd, aers[1], dt, ss, np.array([0.0, 1.0, 0.0]), True)
    _check_grad(g["d_dtau"][1, 1], fd_t, "batch d/ddtau (Q)")
    _check_grad(g["d_ssa"][1, 1], fd_s, "batch d/dssa (Q)")
    _check_grad(g["d_wind"][1, 1], fd_w, "batch d/dwind (Q)")
    # each row alone, each pixel alone
    for i in range(3):
        for r in range(3):
            _, g1 = gpu.solve_batch_adjoint([cs[i]], o_gpu, [aers[i]], [lys[i]], eye[i:i + 1, r:r + 1])
            np.testing.assert_allclose(g1["d_dtau"][0, 0], g["d_dtau"][i, r], rtol=1e-5, atol=1e-9)
            np.testing.assert_allclose(g1["d_ssa"][0, 0], g["d_ssa"][i, r], rtol=1e-5, atol=1e-9)
            np.testing.assert_allclose(g1["d_wind"][0, 0], g["d_wind"][i, r], rtol=1e-5, atol=1e-10)


def test_adjoint_rejects_unsupported(gpu):
    from ocrt_gb300 import _abi as A
    c = A.default_case(surface="flat")
    o = A.default_opts(n_mu=8, n_layers=8)
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_batch_adjoint([c], o, None, None, np.ones((1, 1, 3)))
    assert e.value.rc == A.OCRT_ERR_UNSUPPORTED
    c = A.default_case()
    o = A.default_opts(n_mu=8, n_layers=8, pssa=1)
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_batch_adjoint([c], o, None, None, np.ones((1, 1, 3)))
    assert e.value.rc == A.OCRT_ERR_UNSUPPORTED


def test_torch_autograd_function(gpu, oracle):
    """sos_reflectance under torch.autograd: backward equals the library's
    adjoint for the same cotangent, and the oracle's FP64 finite differences."""
    torch = pytest.importorskip("torch")
    from ocrt_gb300 import _abi as A
    from ocrt_gb300.autograd import layer_parameters, sos_reflectance
    from synthetic import hg_aerosol_moments
    cs = [_case(A, sza_deg=35.0, vza_deg=40.0, raa_deg=100.0, wind=6.0),
          _case(A, sza_deg=55.0, vza_deg=20.0, raa_deg=10.0, wind=2.5)]
    o = A.default_opts(n_mu=16, n_layers=8, fourier_m_max=4, max_orders=400, tolerance=1e-9)
    aers = [A.AerosolHolder(0.12, 0.93, *hg_aerosol_moments(0.7, 24)) for _ in cs]
    dt, ss, w = layer_parameters(cs, o, aers)
    # the library's defaults equal the oracle's profile values
    dto, sso = oracle.layer_defaults(cs[0], o, aers[0])
    np.testing.assert_allclose(dt[0].numpy(), dto, rtol=1e-12)
    np.testing.assert_allclose(ss[0].numpy(), sso, rtol=1e-12)
    dt.requires_grad_(True); ss.requires_grad_(True); w.requires_grad_(True)
    rho = sos_reflectance(dt, ss, w, cs, o, aers)
    wts = torch.tensor([[1.0, 0.5, -0.25], [0.2, -1.0, 0.4]], dtype=torch.float64)
    (rho * wts).sum().backward()
    _, g = gpu.solve_batch_adjoint(cs, o, aers, None, wts.numpy()[:, None, :])
    np.testing.assert_allclose(dt.grad.numpy(), g["d_dtau"][:, 0], rtol=1e-5, atol=1e-10)
    np.testing.assert_allclose(ss.grad.numpy(), g["d_ssa"][:, 0], rtol=1e-5, atol=1e-10)
    np.testing.assert_allclose(w.grad.numpy(), g["d_wind"][:, 0], rtol=1e-5, atol=1e-12)
    o_fd = A.default_opts(n_mu=16, n_layers=8, fourier_m_max=4, max_orders=200, tolerance=1e-300)
    fd_t, fd_s, fd_w = _fd_all(oracle, cs[1], o_fd, aers[1], dto * 0 + dt[1].detach().numpy(),
                               ss[1].detach().numpy(), wts[1].numpy(), True)
    _check_grad(dt.grad[1].numpy(), fd_t, "torch d/ddtau")
    _check_grad(ss.grad[1].numpy(), fd_s, "torch d/dssa")
    _check_grad(w.grad[1].item(), fd_w, "torch d/dwind")
