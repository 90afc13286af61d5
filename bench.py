"""Benchmark: batched forward pixel-solves/s on one GB300 (configuration 3).

Workload (seeded synthetic, config["workload"]): 4096 pixels in one call with
uneven shapes -- sza U[0,80], vza U[0,70], raa U[0,180], AOD lognormal
(median 0.1, sigma 0.6), layers uniform in {50,100,200,400}, 10 bands
412-865 nm with tau_R ~ lambda^-4.08, wind U[1,12] m/s, Henyey-Greenstein
aerosol g U[0.6,0.8], SSA U[0.85,0.99], moments to L=120, 32 Gauss streams,
Fourier modes 0..32, rough Cox-Munk ocean, tolerance 1e-7.

value : pixel-solves/s from a resident plan (inputs already in HBM), K steps
        timed with CUDA events on the launching stream.
e2e   : the same metric through the C ABI call ocrt_gb_solve_batch with host
        buffers (uploads, solve, result download inside the timed region).

    python bench.py [--steps K] [--warmup W] [--impl ours|reference] [--pixels P]
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ocrt_gb300 import _abi as A  # noqa: E402
from ocrt_gb300.replicas import max_over_ranks  # noqa: E402
from synthetic import batched_forward_pixels, coupled_ocean_pixels, hg_aerosol_moments  # noqa: E402

METRIC = "pixel-solves/s"
N_MU, M_MAX, L_AER = 32, 32, 120


def workload(n_pix, seed=20261203 + 3):
    p = batched_forward_pixels(n_pix, seed=seed)
    cases, opts, aers = [], [], []
    for i in range(n_pix):
        cases.append(A.default_case(surface="black_fresnel_ocean", sza_deg=p["sza"][i], vza_deg=p["vza"][i],
                                    raa_deg=p["raa"][i], wavelength_nm=p["wavelength"][i],
                                    wind_speed=p["wind"][i], tau_r_input=p["tau_r"][i]))
        opts.append(A.default_opts(n_mu=N_MU, n_layers=int(p["n_layers"][i]), fourier_m_max=M_MAX,
                                   tau_r_source=A.TAU_R_FROM_INPUT, max_orders=1000, tolerance=1e-7))
        aers.append(A.AerosolHolder(p["aod"][i], p["ssa"][i], *hg_aerosol_moments(p["g"][i], L_AER)))
    return cases, opts, aers


ADJ_BANDS = (443.0, 555.0, 865.0)
ADJ_LAYERS = 200


def adjoint_workload(n_pix, seed=20261203 + 4):
    """Configuration 4: n_pix geometries x 3 bands, 200 layers, the fixed
    aerosol of configuration 2 (HG g=0.7 to L=120, SSA 0.95, AOD 0.1), rough
    ocean at 5 m/s, plane-parallel (IPSS is not differentiated)."""
    rng = np.random.default_rng(seed)
    sza, vza, raa = rng.uniform(0, 70, n_pix), rng.uniform(0, 60, n_pix), rng.uniform(0, 180, n_pix)
    mom = hg_aerosol_moments(0.7, L_AER)
    aer = A.AerosolHolder(0.1, 0.95, *mom)
    cases, aers = [], []
    for i in range(n_pix):
        for wl in ADJ_BANDS:
            cases.append(A.default_case(surface="black_fresnel_ocean", sza_deg=sza[i], vza_deg=vza[i],
                                        raa_deg=raa[i], wavelength_nm=wl, wind_speed=5.0,
                                        tau_r_input=0.0945 * (wl / 555.0) ** -4.08))
            aers.append(aer)
    opts = A.default_opts(n_mu=N_MU, n_layers=ADJ_LAYERS, fourier_m_max=M_MAX, tau_r_source=A.TAU_R_FROM_INPUT,
                          max_orders=1000, tolerance=1e-7)
    return cases, opts, aers


OCEAN_N, OCEAN_M, OCEAN_LAYERS_ATM, OCEAN_LAYERS_W, L_HYD = 32, 16, 400, 100, 200


def ocean_workload(n_geom):
    """Configuration 5: n_geom geometries x 8 bands; the configuration-2
    atmosphere (400 layers, HG g=0.7 aerosol to L=120, SSA 0.95, AOD 0.1) over
    a 50 m, 100-layer ocean with a forward-peaked hydrosol (HG g=0.92 to
    L=200) and pure-water scattering, Cox-Munk interface, n_water 1.34."""
    rows = coupled_ocean_pixels(n_geom)
    aer = A.AerosolHolder(0.1, 0.95, *hg_aerosol_moments(0.7, L_AER))
    hyd = hg_aerosol_moments(0.92, L_HYD)
    cases, oceans = [], []
    for r in rows:
        cases.append(A.default_case(surface="ocean", sza_deg=r["sza"], vza_deg=r["vza"], raa_deg=r["raa"],
                                    wavelength_nm=r["wavelength"], wind_speed=r["wind"], tau_r_input=r["tau_r"],
                                    n_water=1.34))
        oceans.append(A.OceanHolder(r["a"], r["b_water"], r["b_particle"], hyd, n_mu_water=OCEAN_N,
                                    m_max_water=OCEAN_M, depth_m=50.0, n_layers_water=OCEAN_LAYERS_W,
                                    max_orders_water=1000, tolerance_water=1e-7))
    opts = A.default_opts(n_mu=OCEAN_N, n_layers=OCEAN_LAYERS_ATM, fourier_m_max=OCEAN_M,
                          tau_r_source=A.TAU_R_FROM_INPUT, max_orders=1000, tolerance=1e-7)
    return cases, opts, [aer] * len(cases), oceans


def run_ocean(args, og, world):
    """Configuration-5 sub-line: coupled atmosphere-ocean pixel-bands per
    second through ocrt_gb_solve_batch_ocean with host buffers (uploads,
    the three SOS passes, the interface kernels and the result download
    inside the timed region), and the error against the FP64 oracle."""
    cases, opts, aers, oceans = ocean_workload(args.ocean_geoms)
    n = len(cases)
    og.solve_batch_ocean(cases[:8], opts, oceans[:8], aers[:8])      # warm the allocator cache
    for _ in range(max(0, min(args.warmup, 1))):
        og.solve_batch_ocean(cases, opts, oceans, aers)
    steps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(steps):
        res = og.solve_batch_ocean(cases, opts, oceans, aers)
    dt = max_over_ranks((time.perf_counter() - t0) / steps)
    out = {"metric": "coupled pixel-solves/s", "value": n * world / dt, "unit": "pixel-solves/s",
           "ms_per_step": dt * 1e3, "steps": steps, "pixel_bands": n,
           "workload": f"configuration 5: {args.ocean_geoms} geometries x 8 bands, atmosphere {OCEAN_LAYERS_ATM} "
                       f"layers (aerosol HG g=0.7 to L={L_AER}), ocean {OCEAN_LAYERS_W} layers, 50 m, hydrosol "
                       f"HG g=0.92 to L={L_HYD}, a U[0.02,0.5] b U[0.01,1.0] per m, wind U[1,12]; "
                       f"N={OCEAN_N} shared streams, Fourier modes 0..{OCEAN_M} in both media; "
                       f"IPSS off (the coupled path is plane-parallel); forward only",
           "timing": "wall clock around ocrt_gb_solve_batch_ocean with host buffers (host<->device copies, "
                     "allocation and the three SOS passes inside)",
           "water_orders_max": max(r["orders_water"] for r in res)}
    if world == 1 and not args.no_cpu and args.ocean_cpu > 0:
        lib = oracle_lib()
        f = lib.ocrt_oracle_solve_ocean
        f.argtypes = [C.POINTER(A.Case), C.POINTER(A.Opts), C.POINTER(A.Aerosol), C.POINTER(A.Ocean),
                      C.POINTER(A.Result), C.POINTER(A.OceanResult)]
        k = min(args.ocean_cpu, n)
        errs = {"rho_I": 0.0, "rho_Q": 0.0, "rho_U": 0.0, "Rrs": 0.0}
        t0 = time.perf_counter()
        for i in range(k):
            r, w = A.Result(), A.OceanResult()
            rc = f(C.byref(cases[i]), C.byref(opts), C.byref(aers[i].struct), C.byref(oceans[i].struct),
                   C.byref(r), C.byref(w))
            if rc != 0:
                raise RuntimeError(f"oracle ocean rc {rc}")
            g = res[i]
            errs["rho_I"] = max(errs["rho_I"], abs(g["rho_I"] - r.rho_I) / abs(r.rho_I))
            errs["rho_Q"] = max(errs["rho_Q"], abs(g["rho_Q"] - r.rho_Q))
            errs["rho_U"] = max(errs["rho_U"], abs(g["rho_U"] - r.rho_U))
            errs["Rrs"] = max(errs["Rrs"], abs(g["Rrs_0plus_I"] - w.Rrs_0plus_I) / abs(w.Rrs_0plus_I))
        tc = time.perf_counter() - t0
        out["rel_err_vs_fp64"] = {"pixels": k, "max_rel_err_rho_I": errs["rho_I"], "max_abs_err_rho_Q": errs["rho_Q"],
                                  "max_abs_err_rho_U": errs["rho_U"], "max_rel_err_Rrs_0plus": errs["Rrs"],
                                  "reference": "FP64 oracle on the same pixel-bands"}
        out["cpu_baseline"] = {"value": k / tc, "unit": "pixel-solves/s", "cores": 1, "kind": "port",
                               "sample": f"first {k} pixel-bands, one oracle call each, {tc:.1f} s"}
    return out


def config_dict(n_pix, world):
    return {"workload": f"configuration 3: batched forward, {n_pix} pixels/GPU, uneven layers 50-400, "
                        f"N={N_MU} streams, m<=32, aerosol L={L_AER}, rough Cox-Munk ocean",
            "pixels_per_gpu": n_pix, "n_mu": N_MU, "fourier_m_max": M_MAX, "aerosol_L": L_AER,
            "tolerance": 1e-7, "parallelism": f"replicas x{world}",
            "l2_policy": "working set (fields, totals, operators) >> 129 MB L2; no flush needed"}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "src": "fallback"}


def traffic_from_profiles(kernel, alg_bytes_per_launch):
    """DRAM bytes per launch for kernel class `kernel`: the ratio of ncu DRAM
    traffic to algorithmic bytes measured on a smaller case of the same
    kernel (profiles/dram_traffic.txt: `class ratio kernel` lines) times this
    run's algorithmic bytes per launch."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and not line.startswith("#") and parts[0] == kernel:
            return float(parts[1]) * alg_bytes_per_launch
    return None


def oracle_lib():
    """The CPU restatement compiled with the reference's floating-point flags
    (liboracle_fast.so), the timed port baseline."""
    so = os.path.join(ROOT, "oracle", "_build", "liboracle_fast.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    lib = C.CDLL(so)
    lib.ocrt_oracle_solve_batch.argtypes = [C.c_int, C.POINTER(A.Case), C.POINTER(A.Opts), C.c_int,
                                            C.POINTER(A.Aerosol), C.c_int, C.POINTER(A.Result), C.c_int]
    lib.ocrt_oracle_max_threads.restype = C.c_int
    return lib


def cpu_run(cases, opts, aers, prefer_reference):
    """Time the CPU implementation over the given pixels with every host thread."""
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libocrt_ref.so")
    lib = oracle_lib()
    threads = lib.ocrt_oracle_max_threads()
    kind, fn = "port", lib.ocrt_oracle_solve_batch
    if prefer_reference and os.path.exists(ref_so):
        try:
            rl = C.CDLL(ref_so)
            rl.ocrt_ref_solve_batch.argtypes = lib.ocrt_oracle_solve_batch.argtypes
            kind, fn = "reference", rl.ocrt_ref_solve_batch
        except OSError:
            pass
    n = len(cases)
    out = (A.Result * n)()
    t0 = time.perf_counter()
    rc = fn(n, (A.Case * n)(*cases), (A.Opts * n)(*opts), 1, (A.Aerosol * n)(*[a.struct for a in aers]), 1,
            out, threads)
    dt = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError(f"cpu baseline rc {rc}")
    return dt, threads, kind, out


def cpu_sample(cases, opts, aers, budget_s=20.0, prefer_reference=False):
    """Bounded sample: grow the pixel count until about budget_s of CPU work."""
    n = 16
    dt, threads, kind, out = cpu_run(cases[:n], opts[:n], aers[:n], prefer_reference)
    total_t, total_n = dt, n
    outs = list(out)
    while total_t < budget_s * 0.5 and total_n + n <= len(cases):
        dt, _, _, out = cpu_run(cases[total_n:total_n + n], opts[total_n:total_n + n], aers[total_n:total_n + n],
                                prefer_reference)
        total_t += dt
        total_n += n
        outs += list(out)
    return {"value": total_n / total_t, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"first {total_n} pixels of the workload, OpenMP over pixels, {total_t:.1f} s"}, outs


# ---------------------------------------------------------------- arms
def run_reference(args, rank, world):
    if rank != 0:
        return
    cases, opts, aers = workload(max(args.pixels, 256))
    for _ in range(args.warmup):
        cpu_run(cases[:4], opts[:4], aers[:4], True)
    vals = []
    base = None
    for k in range(args.steps):
        base, _ = cpu_sample(cases[k * 16:], opts[k * 16:], aers[k * 16:], budget_s=args.cpu_budget,
                             prefer_reference=True)
        vals.append(base["value"])
    v = statistics.median(vals)
    extra = {}
    if args.compare_port and base["kind"] == "reference":
        # the port on the same pixels and threads: its speed relative to the
        # reference library on this host
        n = int(base["sample"].split()[1])
        dt_r, _, _, _ = cpu_run(cases[:n], opts[:n], aers[:n], True)
        dt_p, _, _, _ = cpu_run(cases[:n], opts[:n], aers[:n], False)
        extra = {"port_time_over_reference": dt_p / dt_r, "compare_pixels": n}
    line = {"impl": "reference", **extra, "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args.pixels, world),
            "cpu_baseline": {**base, "value": v},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import torch
    import ocrt_gb300 as og
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    og.lib().ocrt_gb_init(dev)
    cases, opts, aers = workload(args.pixels)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- value: resident plan ----
    # Warm-up: the first execute runs eagerly (host polls end the order loops
    # and record their lengths, the autotuner picks block sizes), the second
    # captures the launch sequence into a CUDA graph; timed steps replay it.
    plan = og.Plan(cases, opts, aers)
    for _ in range(args.warmup):
        plan.execute(sp)
    torch.cuda.synchronize()
    graph = plan.graph_ready
    clocks = ClockSampler(dev)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    launches = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    for _ in range(args.steps):
        e0.record(stream)
        plan.execute(sp)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        launches += plan.stats()["kernel_launches"]
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    res = plan.results(sp)

    # ---- per-kernel breakdown: the same steps executed eagerly with every
    # launch bracketed by CUDA events on the launching stream ----
    og.set_timing(True)
    kstats = {}
    instr_ms = 0.0
    for _ in range(args.steps):
        e0.record(stream)
        plan.execute(sp)
        e1.record(stream)
        e1.synchronize()
        instr_ms += e0.elapsed_time(e1)
        for k, v in plan.kernel_stats().items():
            acc = kstats.setdefault(k, {"ms": 0.0, "launches": 0, "flops": 0.0, "bytes": 0.0})
            for f in acc:
                acc[f] += v[f]
    og.set_timing(False)
    res_instr = plan.results(sp)
    if not np.array_equal(res, res_instr):
        raise RuntimeError("graph replay and eager execute disagree")
    om = float(np.sum(res["order_modes"]))
    ms_step = max_over_ranks(total_ms / args.steps)
    value = args.pixels * world / (ms_step / 1e3)

    # ---- roofline of the dominant kernel ----
    # The binding roof is the one the kernel's algorithmic intensity hits first:
    # tensor (or the FP32 pipes) above the ridge point peak_flops / peak_bw, HBM below.
    pk = peaks()
    dom = max(kstats, key=lambda k: kstats[k]["ms"])
    d = kstats[dom]
    per_launch_ms = d["ms"] / max(d["launches"], 1)
    secs = d["ms"] / 1e3
    ridge = pk["bf16_tflops_sustained"] * 1e12 / (pk["hbm_gbs"] * 1e9)
    intensity = d["flops"] / d["bytes"] if d["bytes"] > 0 else float("inf")
    tensor_frac = (d["flops"] / secs / 1e12) / pk["bf16_tflops_sustained"] if d["flops"] > 0 else None
    if d["flops"] > 0 and intensity >= ridge:
        achieved = d["flops"] / secs / 1e12
        roof = {"kernel": dom, "bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops_sustained"],
                "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops_sustained"],
                "peak_source": f"{pk['src']} bf16 sustained",
                "traffic": traffic_from_profiles(dom, d["bytes"] / max(d["launches"], 1)),
                "avg_launch_ms": per_launch_ms, "alg_flops_per_launch": d["flops"] / max(d["launches"], 1),
                "intensity_flop_per_byte": intensity, "ridge_flop_per_byte": ridge}
    else:
        achieved = d["bytes"] / secs / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "peak_source": f"{pk['src']} HBM copy",
                "traffic": traffic_from_profiles(dom, d["bytes"] / max(d["launches"], 1)),
                "avg_launch_ms": per_launch_ms, "alg_bytes_per_launch": d["bytes"] / max(d["launches"], 1),
                "intensity_flop_per_byte": intensity if d["flops"] > 0 else None, "ridge_flop_per_byte": ridge,
                "tensor_frac_of_bf16": tensor_frac}
    if roof.get("traffic"):
        # DRAM bytes actually moved per launch (measured ratio x algorithmic) over the launch time
        roof["traffic_gbs"] = roof["traffic"] / (per_launch_ms / 1e3) / 1e9
        roof["traffic_frac_of_hbm"] = roof["traffic_gbs"] / pk["hbm_gbs"]
    breakdown = {k: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps,
                     "share": v["ms"] / max(sum(x["ms"] for x in kstats.values()), 1e-9),
                     "alg_bytes_per_step": v["bytes"] / args.steps, "alg_flops_per_step": v["flops"] / args.steps}
                 for k, v in sorted(kstats.items(), key=lambda kv: -kv[1]["ms"]) if v["launches"]}
    plan.close()

    # ---- e2e through the C ABI with host buffers ----
    og.solve_batch(cases, opts, aers)          # warm the allocator cache
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r_e2e = og.solve_batch(cases, opts, aers)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps)
    h2d = args.pixels * (C.sizeof(A.Case) + C.sizeof(A.Opts) + C.sizeof(A.Aerosol) + 4 * 8 * (L_AER + 1))
    d2h = args.pixels * C.sizeof(A.Result)
    e2e = {"value": args.pixels * world / t_e2e, "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    # ---- adjoint: full Jacobians (3 cotangent rows) per pixel-band ----
    adj = None
    if args.adj_pixels > 0:
        adj = run_adjoint(args, og, torch, stream, sp, barrier, world)

    # ---- configuration 5: the coupled atmosphere-ocean solve ----
    ocean = run_ocean(args, og, world) if args.ocean_geoms > 0 else None

    if rank != 0:
        return
    # ---- plain per-pixel GPU form (one solve call per pixel) ----
    nplain = min(args.plain_pixels, args.pixels)
    og.solve_case(cases[0], opts[0], aers[0])
    t0 = time.perf_counter()
    for i in range(nplain):
        og.solve_case(cases[i], opts[i], aers[i])
    plain = nplain / (time.perf_counter() - t0)

    # ---- CPU baseline (oracle port, all host threads) + error vs FP64 ----
    cpu, couts = (None, None)
    err = None
    if world == 1 and not args.no_cpu:
        cpu, couts = cpu_sample(cases, opts, aers, budget_s=args.cpu_budget)
        n = len(couts)
        relI = max(abs(res["rho_I"][i] - couts[i].rho_I) / abs(couts[i].rho_I) for i in range(n))
        dQ = max(abs(res["rho_Q"][i] - couts[i].rho_Q) for i in range(n))
        dU = max(abs(res["rho_U"][i] - couts[i].rho_U) for i in range(n))
        err = {"pixels": n, "max_rel_err_rho_I": relI, "max_abs_err_rho_Q": dQ, "max_abs_err_rho_U": dU,
               "reference": "FP64 oracle on the same pixels"}

    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args.pixels, world),
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "roofline": roof,
            "cpu_baseline": cpu, "rel_err_vs_fp64": err,
            "plain_per_pixel_gpu": {"value": plain, "unit": METRIC, "sample": f"{nplain} pixels, one "
                                    f"ocrt_gb_solve_case call each", "batched_speedup": value / world / plain},
            "order_modes_per_step": om, "kernel_breakdown": breakdown, "adjoint": adj, "coupled_ocean": ocean,
            "execute": {"graph_replay": graph, "eager_instrumented_ms_per_step": instr_ms / args.steps,
                        "autotune": [{k: s[k] for k in ("kernel", "key", "best")} for s in og.autotune_summary()]}}
    print(json.dumps(line), flush=True)


def run_adjoint(args, og, torch, stream, sp, barrier, world):
    """Configuration 4 on a resident plan: forward alone and forward + the
    3-row Jacobian, K steps each timed with CUDA events on the launching
    stream; Jacobians/s counts pixel-band Jacobians (3 outputs x 401 inputs)."""
    cases, opts, aers = adjoint_workload(args.adj_pixels)
    n = len(cases)
    eye = np.broadcast_to(np.eye(3), (n, 3, 3)).copy()

    def timed(plan):
        for _ in range(args.warmup):
            plan.execute(sp)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(args.steps):
            e0.record(stream)
            plan.execute(sp)
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        ms = max_over_ranks(tot / args.steps)
        # one eager execute with per-launch events for the breakdown
        og.set_timing(True)
        plan.execute(sp)
        ks = {k: v["ms"] for k, v in plan.kernel_stats().items()}
        og.set_timing(False)
        return ms, {k: v for k, v in sorted(ks.items(), key=lambda kv: -kv[1]) if v > 0}

    fwd = og.Plan(cases, opts, aers)
    ms_fwd, _ = timed(fwd)
    fwd.close()
    jac = og.Plan(cases, opts, aers, cot=eye)
    ms_jac, ks = timed(jac)
    g = jac.gradients(sp)
    jac.close()
    finite = bool(np.isfinite(g["d_dtau"]).all() and np.isfinite(g["d_ssa"]).all() and np.isfinite(g["d_wind"]).all())
    return {"metric": "adjoint Jacobians/s", "value": n * world / (ms_jac / 1e3), "unit": "Jacobians/s",
            "ms_per_step": ms_jac, "forward_ms_per_step": ms_fwd,
            "jacobian_cost_vs_forward": ms_jac / ms_fwd,
            "workload": f"configuration 4: {args.adj_pixels} pixels x {len(ADJ_BANDS)} bands, {ADJ_LAYERS} layers, "
                        f"N={N_MU}, m<=32, aerosol L={L_AER}, rough ocean 5 m/s, IPSS off; "
                        f"Jacobian of TOA (I,Q,U) w.r.t. {ADJ_LAYERS} dtau + {ADJ_LAYERS} ssa + wind",
            "pixel_bands": n, "gradients_finite": finite,
            "fd_check": "tests/test_gpu_adjoint.py (FP64 central differences on the oracle)",
            "kernel_ms_per_step": ks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pixels", type=int, default=4096)
    ap.add_argument("--plain-pixels", type=int, default=16)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--compare-port", action="store_true",
                    help="reference arm: also time the port on the same pixels (where the reference library exists)")
    ap.add_argument("--adj-pixels", type=int, default=1024,
                    help="configuration-4 geometries (x3 bands) for the adjoint line; 0 skips it")
    ap.add_argument("--ocean-geoms", type=int, default=128,
                    help="configuration-5 geometries (x8 bands) for the coupled-ocean line; 0 skips it")
    ap.add_argument("--ocean-cpu", type=int, default=2,
                    help="pixel-bands of the coupled line checked against (and timed on) the FP64 oracle")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
