"""Batched solves: uneven shapes in one call equal per-pixel solves exactly
(the GPU form of the reference's batch row-independence check) and the
oracle within the parity bar; whole-batch properties at full size."""
import numpy as np
import pytest

from _helpers import assert_parity

pytestmark = pytest.mark.gpu


def _batch(n, seed, nt_div=4, m_max=6, n_mu=16, L=40):
    from ocrt_gb300 import _abi as A
    from synthetic import batched_forward_pixels, hg_aerosol_moments
    p = batched_forward_pixels(n, seed=seed)
    cs, os_, aa = [], [], []
    for i in range(n):
        cs.append(A.default_case(surface="black_fresnel_ocean", sza_deg=p["sza"][i], vza_deg=p["vza"][i],
                                 raa_deg=p["raa"][i], wavelength_nm=p["wavelength"][i], wind_speed=p["wind"][i],
                                 tau_r_input=p["tau_r"][i]))
        os_.append(A.default_opts(n_mu=n_mu, n_layers=max(2, int(p["n_layers"][i]) // nt_div),
                                  fourier_m_max=m_max, tau_r_source=1, max_orders=500))
        aa.append(A.AerosolHolder(p["aod"][i], p["ssa"][i], *hg_aerosol_moments(p["g"][i], L)))
    return cs, os_, aa


def test_batch_equals_single_and_oracle(gpu, oracle):
    cs, os_, aa = _batch(48, seed=21)
    res = gpu.solve_batch(cs, os_, aa)
    for i in range(len(cs)):
        single = gpu.solve_case(cs[i], os_[i], aa[i])
        for k in ("rho_I", "rho_Q", "rho_U", "T_diff_dn_hemi"):
            assert res[k][i] == single[k], (i, k)
        assert res["order_modes"][i] == single["order_modes"]
        assert_parity({k: res[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, oracle.solve(cs[i], os_[i], aa[i]),
                      f"pixel {i}")


def test_batch_mixed_streams_and_surfaces(gpu, oracle):
    """Pixels with different Gauss orders, surfaces and view modes in one call."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    cs, os_, aa = [], [], []
    for i, (surf, n_mu, van) in enumerate([("black", 8, 1), ("flat", 12, 1), ("black_fresnel_ocean", 16, 0),
                                           ("black_fresnel_ocean", 8, 1), ("black", 12, 0), ("flat", 16, 0)]):
        cs.append(A.default_case(surface=surf, wind_speed=3.0 + i, sza_deg=10.0 + 11 * i, vza_deg=5.0 + 9 * i))
        os_.append(A.default_opts(n_mu=n_mu, n_layers=15 + 5 * i, fourier_m_max=i % 4 + 1, view_as_node=van))
        aa.append(A.AerosolHolder(0.05 * (i + 1), 0.9, *hg_aerosol_moments(0.6 + 0.03 * i, 20)))
    res = gpu.solve_batch(cs, os_, aa)
    for i in range(len(cs)):
        assert_parity({k: res[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, oracle.solve(cs[i], os_[i], aa[i]),
                      f"pixel {i}")


def test_batch_mirror_azimuth_symmetry(gpu):
    """rho_I, rho_Q even and rho_U odd under raa -> 360 - raa (recipes R01/R02)."""
    from ocrt_gb300 import _abi as A
    cs, os_, aa = _batch(32, seed=5)
    mir = [A.Case.from_buffer_copy(c) for c in cs]
    for c in mir:
        c.raa_deg = 360.0 - c.raa_deg
    a = gpu.solve_batch(cs, os_, aa)
    b = gpu.solve_batch(mir, os_, aa)
    np.testing.assert_allclose(a["rho_I"], b["rho_I"], rtol=1e-6)
    np.testing.assert_allclose(a["rho_Q"], b["rho_Q"], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(a["rho_U"], -b["rho_U"], rtol=1e-6, atol=1e-9)


def test_batch_invalid_row_rejected(gpu):
    cs, os_, aa = _batch(4, seed=2)
    cs[2].sza_deg = 95.0
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_batch(cs, os_, aa)
    assert e.value.rc == -1


def test_plan_reexecute_is_deterministic(gpu):
    cs, os_, aa = _batch(16, seed=9)
    plan = gpu.Plan(cs, os_, aa)
    plan.execute()
    r1 = plan.results()
    plan.execute()
    r2 = plan.results()
    assert np.array_equal(r1, r2)
    assert plan.stats()["kernel_launches"] > 0
    plan.close()


def test_tcgen05_and_cuda_core_source_agree(gpu, oracle):
    """The tcgen05 3xTF32 contraction and the CUDA-core FP32 contraction give the
    same solve within the parity bar, and both match the oracle."""
    import os
    cs, os_, aa = _batch(24, seed=33, n_mu=32, m_max=8, L=60)
    try:
        os.environ["OCRT_GB_SOURCE_KERNEL"] = "simt"
        r_simt = gpu.solve_batch(cs, os_, aa)
    finally:
        os.environ.pop("OCRT_GB_SOURCE_KERNEL", None)
    r_tc = gpu.solve_batch(cs, os_, aa)
    for i in range(len(cs)):
        ref = oracle.solve(cs[i], os_[i], aa[i])
        assert_parity({k: r_tc[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"tcgen05 pixel {i}")
        assert_parity({k: r_simt[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"simt pixel {i}")
        assert abs(r_tc["rho_I"][i] - r_simt["rho_I"][i]) <= 2e-6 * abs(r_simt["rho_I"][i])


def test_tcgen05_kernel_is_used(gpu):
    cs, os_, aa = _batch(8, seed=34, n_mu=32, m_max=6, L=40)
    gpu.set_timing(True)
    try:
        plan = gpu.Plan(cs, os_, aa)
        plan.execute()
        ks = plan.kernel_stats()
        plan.close()
    finally:
        gpu.set_timing(False)
    assert ks["source_gemm_tcgen05"]["launches"] > 0
    assert ks["source_gemm_tcgen05"]["ms"] > 0


def test_coxmunk_tensor_core_and_cuda_core_agree(gpu, oracle):
    """The Cox-Munk Fourier kernels with the azimuth projection on tcgen05
    (3xTF32) and on the CUDA cores give the same solve within the parity bar,
    and both match the oracle; rough surfaces at several winds and modes."""
    import os
    cs, os_, aa = _batch(24, seed=35, n_mu=16, m_max=12, L=40)
    try:
        os.environ["OCRT_GB_COXMUNK"] = "simt"
        r_simt = gpu.solve_batch(cs, os_, aa)
    finally:
        os.environ.pop("OCRT_GB_COXMUNK", None)
    r_tc = gpu.solve_batch(cs, os_, aa)
    for i in range(len(cs)):
        ref = oracle.solve(cs[i], os_[i], aa[i])
        assert_parity({k: r_tc[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"tcgen05 Cox-Munk pixel {i}")
        assert abs(r_tc["rho_I"][i] - r_simt["rho_I"][i]) <= 2e-6 * abs(r_simt["rho_I"][i])
        assert abs(r_tc["rho_Q"][i] - r_simt["rho_Q"][i]) <= 1e-6
        assert abs(r_tc["rho_U"][i] - r_simt["rho_U"][i]) <= 1e-6


def test_source_tensor_core_and_cuda_core_agree(gpu, oracle):
    """The tcgen05 source pass (operators as pre-split tf32 tiles, 3xTF32) and
    the CUDA-core source (FP32) give the same solve: m <= 2 tasks take the
    dense molecular tiles; half the pixels interpolate the view (no view slot:
    its operator tile rows are zero) and half carry it as a ring node."""
    import os
    from ocrt_gb300 import _abi as A
    cs, os_, aa = _batch(24, seed=36, n_mu=32, m_max=8, L=60)
    for i in range(len(cs)):
        os_[i].view_as_node = i % 2
    try:
        os.environ["OCRT_GB_SOURCE_KERNEL"] = "simt"
        r_simt = gpu.solve_batch(cs, os_, aa)
    finally:
        os.environ.pop("OCRT_GB_SOURCE_KERNEL", None)
    r_tc = gpu.solve_batch(cs, os_, aa)
    # each path carries FP32 fields (a few 1e-6 relative against FP64), so
    # both are held to the parity bar against the oracle and to each other
    for i in range(len(cs)):
        ref = oracle.solve(cs[i], os_[i], aa[i])
        for r, what in ((r_tc, "tcgen05"), (r_simt, "CUDA-core")):
            assert_parity({k: r[k][i] for k in ("rho_I", "rho_Q", "rho_U")}, ref, f"{what} source pixel {i}")
        assert abs(r_tc["rho_I"][i] - r_simt["rho_I"][i]) <= 1e-5 * abs(r_simt["rho_I"][i]), i
        assert abs(r_tc["rho_Q"][i] - r_simt["rho_Q"][i]) <= 1e-5, i
        assert abs(r_tc["rho_U"][i] - r_simt["rho_U"][i]) <= 1e-5, i
