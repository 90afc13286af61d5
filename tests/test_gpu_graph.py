"""Resident plans: the first execute runs eagerly with host polls, the second
captures the launch sequence into a CUDA graph, later ones replay it.  Graph
replays give the eager results and gradients bit for bit (the per-task
arithmetic does not depend on which CTA ran it), on the library stream and on
a caller's stream; timing keeps executes eager.  The launch-shape autotuner
only changes block sizes of kernels whose per-thread arithmetic is independent
of the block size, so its choice changes no result bit either."""
import contextlib
import ctypes as C
import os

import numpy as np
import pytest

from test_gpu_batch import _batch

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def _env(**kv):
    old = {k: os.environ.get(k) for k in kv}
    os.environ.update(kv)
    try:
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _eager(gpu, cs, os_, aa):
    with _env(OCRT_GB_GRAPH="0"):
        p = gpu.Plan(cs, os_, aa)
        p.execute()
        p.execute()
        assert not p.graph_ready
        r = p.results()
        p.close()
    return r


def test_graph_replay_equals_eager(gpu):
    cs, os_, aa = _batch(40, seed=41)
    ref = _eager(gpu, cs, os_, aa)
    plan = gpu.Plan(cs, os_, aa)
    launches = []
    for k in range(4):
        plan.execute()
        assert plan.graph_ready == (k >= 1)
        assert np.array_equal(plan.results(), ref), f"execute {k}"
        launches.append(plan.stats()["kernel_launches"])
    # the graph holds the eager sequence plus one convergence check per wave
    assert launches[1] == launches[2] == launches[3] >= launches[0]
    plan.close()


def test_graph_replay_on_caller_stream(gpu):
    torch = pytest.importorskip("torch")
    cs, os_, aa = _batch(12, seed=42, m_max=3)
    ref = _eager(gpu, cs, os_, aa)
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    plan = gpu.Plan(cs, os_, aa)
    for _ in range(3):
        plan.execute(sp)
    assert plan.graph_ready
    assert np.array_equal(plan.results(sp), ref)
    plan.close()


def test_timing_keeps_executes_eager(gpu):
    cs, os_, aa = _batch(8, seed=43, m_max=2)
    gpu.set_timing(True)
    try:
        plan = gpu.Plan(cs, os_, aa)
        for _ in range(3):
            plan.execute()
        assert not plan.graph_ready
        ks = plan.kernel_stats()
        plan.close()
    finally:
        gpu.set_timing(False)
    assert ks["transport_scan"]["launches"] > 0 and ks["transport_scan"]["ms"] > 0


def test_graph_replay_adjoint_plan(gpu):
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    cs = [A.default_case(surface="black_fresnel_ocean", wind_speed=3.0 + i, sza_deg=30.0 + 5 * i,
                         vza_deg=20.0 + 7 * i, raa_deg=40.0 + 30 * i) for i in range(4)]
    o = A.default_opts(n_mu=8, n_layers=8, fourier_m_max=4, max_orders=400, tolerance=1e-9)
    aers = [A.AerosolHolder(0.1, 0.93, *hg_aerosol_moments(0.7, 20)) for _ in range(4)]
    eye = np.broadcast_to(np.eye(3), (4, 3, 3)).copy()
    with _env(OCRT_GB_GRAPH="0"):
        p0 = gpu.Plan(cs, o, aers, cot=eye)
        p0.execute()
        r0, g0 = p0.results(), p0.gradients()
        p0.close()
    plan = gpu.Plan(cs, o, aers, cot=eye)
    for k in range(3):
        plan.execute()
        assert np.array_equal(plan.results(), r0)
        g = plan.gradients()
        for key in ("d_dtau", "d_ssa", "d_wind"):
            assert np.array_equal(g[key], g0[key]), (k, key)
    assert plan.graph_ready
    plan.close()


def test_autotune_changes_no_result(gpu):
    # the CUDA-core Cox-Munk and phase-table kernels are the autotuned ones
    # (the tensor-core kernels have a fixed shape), so this test selects them
    cs, os_, aa = _batch(16, seed=44, n_mu=16, m_max=5)
    with _env(OCRT_GB_AUTOTUNE="0", OCRT_GB_COXMUNK="simt", OCRT_GB_TABLES="simt"):
        r0 = gpu.solve_batch(cs, os_, aa)
    with _env(OCRT_GB_COXMUNK="simt", OCRT_GB_TABLES="simt"):
        r1 = gpu.solve_batch(cs, os_, aa)
    assert np.array_equal(r0, r1)
    summ = gpu.autotune_summary()
    kinds = {s["kernel"] for s in summ}
    assert "k_tables" in kinds and "k_coxmunk" in kinds
    for s in summ:
        # block sizes of the setup kernels; scan implementations by name
        if s["kernel"] == "transport_scan":
            assert s["best"] in ("quad", "tma8x3", "tma8x4", "tma4x6", "tma16x2", "tma8x5", "tma4x10")
        else:
            assert s["best"] in (128, 256, 512)
        assert s["best"] in s["ms"] and all(v > 0 for v in s["ms"].values())
        assert s["ms"][s["best"]] == min(s["ms"].values())
