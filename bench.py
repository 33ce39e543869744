"""BK5 operator-apply benchmark (GDoF/s) on one GB300, JSON-line contract.

Workload: the BK5/BP5 FP64 Laplacian on the deformed unit cube, Q4 with GLL
collocation (p = 4), 128 x 128 x 64 cells = 67,634,433 DoFs, mesh nodes moved
by x_d += 0.05 sin(2 pi x) sin(2 pi y) sin(2 pi z), Dirichlet boundary, src
seeded U[-1,1].  One step = one operator application vmult(dst, src) over the
whole L-vector: dst = 0, the fused gather / D / G / D^T / scatter kernel, the
constrained identity rows.  Inputs (src 541 MB, G 6.5 GB) are far larger than
the 129 MB L2, so no flush is needed between steps.

--impl reference times the CPU implementation of the same vmult (the oracle
restatement, OpenMP over all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(nx=128, ny=128, nz=64, degree=4, amplitude=0.05, seed=1)
METRIC = "BK5 GDoF/s (FP64 operator apply)"


def algorithmic_bytes(n_dofs, n_cells, degree):
    """src read + dst write + per quadrature point 6 FP64 metric terms and a 4-byte map entry."""
    n3 = (degree + 1) ** 3
    return 8 * n_dofs + 8 * n_dofs + n_cells * n3 * (48 + 4)


def algorithmic_flops(n_cells, degree):
    n = degree + 1
    return n_cells * (12 * n ** 4 + 15 * n ** 3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("MFGB_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, world


def max_over_ranks(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profile(arith: str):
    """DRAM bytes per launch of the operator kernel from the committed ncu
    summary for this workload (None if not captured)."""
    if not is_headline():
        return None
    path = os.path.join(ROOT, "profiles", "bk5fx_p4_67M.md" if arith == "df" else
                        f"bk5_{arith}_p4_67M.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def cpu_reference_apply_rate(prob, steps, warmup, src):
    """Time the oracle's OpenMP vmult on the host cores; returns GDoF/s."""
    for _ in range(warmup):
        prob.apply(src)
    t0 = time.perf_counter()
    for _ in range(steps):
        prob.apply(src)
    dt = (time.perf_counter() - t0) / steps
    return prob.n_dofs / dt / 1e9, dt


def run_reference(args, rank, world):
    """CPU implementation of the same vmult (oracle restatement; the reference's
    deal.II CPU path cannot be built here)."""
    if rank != 0:
        return
    from oracle import oracle
    w = WORKLOAD
    prob = oracle.BoxProblem(w["nx"], w["ny"], w["nz"], w["degree"], amplitude=w["amplitude"])
    src = prob.rhs(w["seed"])
    # bounded sample: at most 10 timed and 5 warm-up applies (about 0.2 s each on
    # 16 Grace cores at this size); the line reports the counts it ran
    steps = max(1, min(args.steps, 10))
    warm = max(1, min(args.warmup, 5))
    rate, dt = cpu_reference_apply_rate(prob, steps, warm, src)
    cores = oracle.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "GDoF/s",
        "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded U[-1,1] src, deformed unit-cube mesh)",
        "config": config_dict(args, prob.n_dofs, prob.n_cells),
        "cpu_baseline": {"value": rate, "unit": "GDoF/s", "cores": cores, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": f"full workload, {steps} vmult on {prob.n_dofs} DoFs"},
        "e2e": {"value": rate, "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# operator kernel thread layouts (mfgb_set_kernel_shape; 5, 6 double-float only)
SHAPE_CODES = {"column": 0, "point": 1, "tma": 2, "column_alt": 3, "tma_alt": 4, "fx": 5,
               "fx_alt": 6}
# what the arithmetic of the operator kernel is, and its accuracy against FP64
ARITH_LABEL = {
    "df": "FP64-accurate double-float on the FP32 pipes (offset accumulation, per-cell "
          "exponent scaling; ~2^-43 normwise relative, 1e-12 bar)",
    "fp64": "native FP64 (DFMA)"}


def is_headline():
    return (WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["nz"], WORKLOAD["degree"]) == (128, 128, 64, 4)


def config_dict(args, n_dofs, n_cells):
    w = WORKLOAD
    return {"workload": f"BK5 vmult p={w['degree']} {w['nx']}x{w['ny']}x{w['nz']} cells deformed "
                        f"unit cube (a={w['amplitude']}), {n_dofs} DoFs",
            "degree": w["degree"], "cells": [w["nx"], w["ny"], w["nz"]], "n_dofs": n_dofs,
            "n_cells": n_cells, "arith": args.arith, "shape": getattr(args, "shape", "auto"),
            "l2": "inputs larger than L2 (no flush)",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def run_ours(args, rank, world):
    import ctypes

    import torch

    import benchmarks_gb300 as mf
    from benchmarks_gb300 import _abi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    L = mf.lib()
    w = WORKLOAD
    if args.shape != "auto":
        _abi.check(L.mfgb_set_kernel_shape(mf._arith(args.arith), w["degree"],
                                           SHAPE_CODES[args.shape]))
    A = mf.LaplaceOperator(mf.BoxMesh(w["nx"], w["ny"], w["nz"], degree=w["degree"],
                                      amplitude=w["amplitude"]), arith=args.arith)
    n, n_cells = A.m(), A.n_cells
    arith = mf._arith(args.arith)
    src = A.rhs_uniform(w["seed"])
    dst = A.initialize_dof_vector()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    op, d_dst, d_src = A.handle, ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr())

    def step():
        # the library's vmult: dst = 0 ; cell loop (one kernel) ; constrained identity rows
        _abi.check(L.mfgb_vmult(op, d_dst, d_src, arith, sp))

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    barrier(world)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local).start() if rank == 0 else None
    torch.cuda.synchronize()
    start.record(stream)
    for k in range(args.steps):
        step()
    stop.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    total_ms = start.elapsed_time(stop)
    total_ms = max_over_ranks(total_ms, world)
    _abi.check(L.mfgb_check_device_errors(sp))  # a timed-out copy wait voids the numbers
    kernel_ms = operator_kernel_ms(L, op, d_dst, d_src, arith, sp, stream, args.steps)
    barrier(world)

    # end to end through the public vmult with pinned host buffers
    e2e_ms = float("nan")
    if args.no_e2e:
        return finish(args, rank, world, A, n, n_cells, arith, total_ms, kernel_ms, e2e_ms, clk)
    # (mfgb_vmult_host: the H2D copy of src, the apply and the D2H copy of dst,
    # pipelined over slabs of cells inside the library call)
    h_src = src.cpu().pin_memory()
    h_dst = torch.empty_like(h_src).pin_memory()
    for _ in range(3):
        A.vmult_host(h_dst, h_src)
    torch.cuda.synchronize()
    # three timed blocks, the median reported (the host link is shared with the
    # machine's other GPUs: one block under a neighbour's transfer stays visible
    # in e2e_runs_ms without setting the figure)
    e_steps = max(3, min(args.steps, 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_runs = []
    for _ in range(3):
        e0.record(stream)
        for _ in range(e_steps):
            A.vmult_host(h_dst, h_src)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_runs.append(max_over_ranks(e0.elapsed_time(e1) / e_steps, world))
    e2e_ms = sorted(e2e_runs)[1]
    # correctness guard on the timed result: the device apply of the same src
    A.vmult(dst, src)
    torch.cuda.synchronize()
    err = float(torch.linalg.norm(h_dst.cuda() - dst) / torch.linalg.norm(dst))
    assert err <= 1e-14, err
    # the link's own bound for the step: every DoF once each way at the pinned
    # copy rate with both directions busy
    from benchmarks_gb300.rates import link_rates
    link = link_rates(8 * n, 3)
    return finish(args, rank, world, A, n, n_cells, arith, total_ms, kernel_ms, e2e_ms, clk, link,
                  e2e_runs)


def operator_kernel_ms(L, op, d_dst, d_src, arith, sp, stream, steps):
    """Mean duration of the operator kernel alone (mfgb_vmult_add: the one cell-loop
    launch of vmult, dst += A src), CUDA events on the launching stream around
    every launch, over as many launches as the timed region had steps."""
    import torch

    from benchmarks_gb300 import _abi
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for _ in range(2):
        _abi.check(L.mfgb_vmult_add(op, d_dst, d_src, arith, sp))
    torch.cuda.synchronize()
    for a, b in ev:
        a.record(stream)
        _abi.check(L.mfgb_vmult_add(op, d_dst, d_src, arith, sp))
        b.record(stream)
    torch.cuda.synchronize()
    _abi.check(L.mfgb_check_device_errors(sp))
    return statistics.mean(a.elapsed_time(b) for a, b in ev)


def degree_sweep(args, degrees=(3, 4, 5, 6, 7, 8), target_dofs=4.0e7):
    """The same measurement at p = 3..8 on n^3-cell deformed cubes of about 4e7 DoFs
    (n = round((N^(1/3) - 1) / p), amplitude 0.05, seeded U[-1,1] src): GDoF/s of
    the library's vmult (CUDA events over 20 steps after 3 warm-up steps), the
    operator kernel's mean time and its algorithmic-byte HBM fraction."""
    import ctypes

    import torch

    import benchmarks_gb300 as mf
    from benchmarks_gb300 import _abi
    L = mf.lib()
    arith = mf._arith(args.arith)
    peak = measured_peaks()[0]
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    out = {}
    for p in degrees:
        nc = max(2, round((target_dofs ** (1.0 / 3.0) - 1) / p))
        A = mf.LaplaceOperator(mf.BoxMesh(nc, nc, nc, degree=p, amplitude=WORKLOAD["amplitude"]),
                               arith=args.arith)
        src = A.rhs_uniform(WORKLOAD["seed"])
        dst = A.initialize_dof_vector()
        op, d_dst, d_src = A.handle, ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr())
        for _ in range(3):
            _abi.check(L.mfgb_vmult(op, d_dst, d_src, arith, sp))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(20):
            _abi.check(L.mfgb_vmult(op, d_dst, d_src, arith, sp))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 20
        kms = operator_kernel_ms(L, op, d_dst, d_src, arith, sp, stream, 20)
        n = A.m()
        byts = algorithmic_bytes(n, A.n_cells, p)
        out[str(p)] = {"cells": [nc, nc, nc], "n_dofs": n, "GDoF/s": n / ms / 1e6,
                       "ms_per_vmult": ms, "kernel_ms": kms,
                       "hbm_frac": byts / (kms * 1e-3) / 1e9 / peak,
                       "kernel": kernel_name(p, arith)}
        del A, src, dst
    return out


def finish(args, rank, world, A, n, n_cells, arith, total_ms, kernel_ms, e2e_ms, clk, link=None,
           e2e_runs=None):
    w = WORKLOAD
    if rank != 0:
        return
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    bytes_per = algorithmic_bytes(n, n_cells, w["degree"])
    achieved = bytes_per / (kernel_ms * 1e-3) / 1e9
    flops = algorithmic_flops(n_cells, w["degree"])
    traffic = traffic_from_profile(args.arith)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        from oracle import oracle
        sample = oracle.BoxProblem(max(1, w["nx"] // 2), max(1, w["ny"] // 2), max(1, w["nz"] // 2),
                                   w["degree"], amplitude=w["amplitude"])
        s_src = sample.rhs(w["seed"])
        rate, dt = cpu_reference_apply_rate(sample, 5, 1, s_src)
        cpu = {"value": rate, "unit": "GDoF/s", "cores": oracle.num_threads(), "kind": "port",
               "cpu_model": cpu_model(),
               "sample": f"5 vmult of the oracle (OpenMP) on a {sample.nx}x{sample.ny}x{sample.nz}-"
                         f"cell p={w['degree']} mesh of the same deformed cube, "
                         f"{sample.n_dofs} DoFs"}
    line = {
        "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / 6.83 if is_headline() else None,
        "dtype": "f64",
        "arith": ARITH_LABEL[args.arith],
        "data": "synthetic (seeded U[-1,1] src, deformed unit-cube mesh)",
        "config": config_dict(args, n, n_cells),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": kernel_name(w['degree'], arith),
                     "kernel_ms": kernel_ms, "bytes_per_launch": bytes_per,
                     "flops_per_launch": flops,
                     "fp64_equiv_tflops": flops / (kernel_ms * 1e-3) / 1e12},
        "e2e": {"value": world * n / (e2e_ms * 1e-3) / 1e9, "unit": "GDoF/s",
                "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "ms_per_step": e2e_ms, "e2e_runs_ms": e2e_runs, "timing": "median of 3 blocks",
                "call": "mfgb_vmult_host (pinned host vectors)"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
    }
    if link:
        bound = world * n / (16 * n / link["both"]) / 1e9  # GDoF/s, 8 B each way a DoF
        line["e2e"]["link"] = {"h2d_gbs": link["h2d"] / 1e9, "d2h_gbs": link["d2h"] / 1e9,
                               "both_gbs": link["both"] / 1e9, "bound_gdofs": bound,
                               "frac": line["e2e"]["value"] / bound,
                               "call": "mfgb_link_rate (pinned buffers of one vector)"}
    if cpu:
        line["cpu_baseline"] = cpu
    if not args.no_degrees and world == 1 and is_headline():
        line["degrees"] = degree_sweep(args)
    if not args.no_solve and world == 1 and is_headline():
        line["bp5"] = bp5_solves(A)
        line["bk6"] = bk6_rate(A, args)
        line["bk5_gauss_like_for_like"] = gauss_like_for_like(args)
        line["batched"] = batched_solves()
        line["ceed_bk1_bk3_evector"] = bk1_bk3_rates()
        line["helmholtz_bp5"] = helmholtz_bp5(args)
        line["bp3"] = bp3_rate(args)
    print(json.dumps(line), flush=True)


def bp5_solves(A):
    """BP5 time to a 1e-10 relative residual on the bench mesh (seeded U[-1,1]
    right-hand side): FP64 CG preconditioned by the FP32 p/h-multigrid V-cycle
    against plain FP64 Jacobi-CG on the same GPU, and the error of the
    mixed-precision solution against the FP64-multigrid solution."""
    import torch

    import benchmarks_gb300 as mf
    w = WORKLOAD
    mesh = mf.BoxMesh(w["nx"], w["ny"], w["nz"], degree=w["degree"], amplitude=w["amplitude"])
    b = A.rhs_uniform(w["seed"])

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    out = {"tol": 1e-10, "workload": "same mesh, f ~ U[-1,1] (seed 1), x0 = 0"}
    sols = {}
    for prec in (32, 64):
        M, t_setup = timed(lambda: mf.MGPreconditioner(mesh, precision=prec, operator=A))
        best = None
        for _ in range(2):
            x = A.initialize_dof_vector()
            ctl = mf.ReductionControl(1000, 1e-300, 1e-10)
            _, t = timed(lambda: mf.SolverCG(ctl).solve(A, x, b, M))
            best = t if best is None else min(best, t)
        sols[prec] = x
        out[f"mg_cg_fp{prec}_vcycle"] = {"seconds": best, "setup_seconds": t_setup,
                                         "iterations": ctl.last_step(),
                                         "levels": [l["dofs"] for l in M.levels]}
        del M
    out["error_mixed_vs_fp64_mg"] = float(torch.linalg.norm(sols[32] - sols[64]) /
                                          torch.linalg.norm(sols[64]))
    # learned smoother weights (network trained by benchmarks_gb300/train_smoother.py);
    # the calibration keeps the plain smoother unless the learned one needs fewer iterations
    wpath = os.path.join(ROOT, "benchmarks_gb300", "data", "smoother_mlp.bin")
    if os.path.exists(wpath):
        from benchmarks_gb300.learned import LearnedSmoother
        S = LearnedSmoother.load(wpath)
        M = mf.MGPreconditioner(mesh, precision=32, operator=A)
        (used, its_plain, its_learned, alpha), t_cal = timed(
            lambda: S.attach(M, A, calibrate=True, reduce=1e-10))
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(1000, 1e-300, 1e-10)
        _, t = timed(lambda: mf.SolverCG(ctl).solve(A, x, b, M))
        out["mg_cg_fp32_learned"] = {
            "seconds": t, "iterations": ctl.last_step(), "used_learned_weights": used,
            "calibration_iterations_plain": its_plain,
            "calibration_iterations_learned": its_learned, "exponent": alpha,
            "calibration_seconds": t_cal,
            "error_vs_fp64_mg": float(torch.linalg.norm(x - sols[64]) / torch.linalg.norm(sols[64]))}
        del M
        # the same on a strongly deformed cube of the same size (amplitude 0.12,
        # the largest of the training range), where the smoother weights matter
        mesh2 = mf.BoxMesh(w["nx"], w["ny"], w["nz"], degree=w["degree"], amplitude=0.12)
        A2 = mf.LaplaceOperator(mesh2)
        b2 = A2.rhs_uniform(w["seed"])
        M2 = mf.MGPreconditioner(mesh2, precision=32)
        res = {}
        for name in ("plain", "learned"):
            if name == "learned":
                used2, p2, l2, alpha2 = S.attach(M2, A2, calibrate=True, reduce=1e-10)
            x = A2.initialize_dof_vector()
            ctl = mf.ReductionControl(1000, 1e-300, 1e-10)
            _, t = timed(lambda: mf.SolverCG(ctl).solve(A2, x, b2, M2))
            res[name] = {"seconds": t, "iterations": ctl.last_step()}
        res["used_learned_weights"], res["exponent"] = used2, alpha2
        out["mg_cg_fp32_learned_amplitude_0.12"] = res
        del M2, A2
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(100000, 1e-300, 1e-10)
    P = A.get_matrix_diagonal_inverse()
    _, t = timed(lambda: mf.SolverCG(ctl).solve(A, x, b, P))
    out["jacobi_cg_fp64"] = {"seconds": t, "iterations": ctl.last_step()}
    out["speedup_mg_fp32_vs_jacobi"] = t / out["mg_cg_fp32_vcycle"]["seconds"]
    out["speedup_incl_setup"] = t / (out["mg_cg_fp32_vcycle"]["seconds"] +
                                     out["mg_cg_fp32_vcycle"]["setup_seconds"])
    return out


def batched_solves(n_problems=256, n_sequential=24):
    """Batched BP5 solves: 256 independent problems (degree uniform in 2..7,
    n^3 cells with n uniform in 6..32, amplitude uniform in [0, 0.1], one
    seeded U[-1,1] right-hand side each) to a 1e-10 relative residual with the
    batched FP32-multigrid FP64 CG, against the same method run problem by
    problem (timed on the first n_sequential problems, scaled by DoFs)."""
    import numpy as np
    import torch

    import benchmarks_gb300 as mf
    meshes, seeds = mf.batch_workload(n_problems, seed=2024)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    B, t_setup = timed(lambda: mf.BatchSolver(meshes))
    b = B.rhs_uniform(seeds)
    best = None
    for _ in range(2):
        x = B.initialize_dof_vector()
        _, t = timed(lambda: B.solve(x, b, max_steps=200, reduce=1e-10))
        best = t if best is None else min(best, t)
    steps = [i["steps"] for i in B.infos]
    out = {"problems": n_problems, "n_dofs": B.n_dofs, "setup_seconds": t_setup,
           "seconds": best, "dofs_per_second": B.n_dofs / best,
           "iterations_min_mean_max": [min(steps), float(np.mean(steps)), max(steps)],
           "all_converged": all(i["converged"] for i in B.infos),
           "replans": B.replans,
           "depth_dofs": B.depth_dofs}
    seq_t, seq_dofs = 0.0, 0
    for i in range(n_sequential):
        A = mf.LaplaceOperator(meshes[i])
        M = mf.MGPreconditioner(meshes[i], precision=32)
        bi = B.split(b)[i].contiguous()
        t_best = None
        for _ in range(2):
            xi = A.initialize_dof_vector()
            ctl = mf.ReductionControl(200, 1e-300, 1e-10)
            _, t = timed(lambda: mf.SolverCG(ctl).solve(A, xi, bi, M))
            t_best = t if t_best is None else min(t_best, t)
        seq_t += t_best
        seq_dofs += A.m()
        del A, M
    out["one_by_one_dofs_per_second"] = seq_dofs / seq_t
    out["one_by_one_sample"] = f"first {n_sequential} problems, {seq_dofs} DoFs, {seq_t:.3f} s"
    out["speedup_vs_one_by_one"] = out["dofs_per_second"] / out["one_by_one_dofs_per_second"]
    del B
    return out


def bk1_bk3_rates(degree=4, target_dofs=6.7e7):
    """CEED BK1 (mass) and BK3 (Laplacian, q = p + 2) E-vector applies, the
    reference CEED_BK benchmarks' operators, at about 6.7e7 E-vector DoFs
    (nelmt * (p+1)^3) with seeded inputs; GDoF/s and the HBM fraction of the
    algorithmic bytes (E-vector in + out, JxW or G per point)."""
    import numpy as np
    import torch

    import benchmarks_gb300 as mf
    from oracle import oracle as orc  # GLL / Gauss points for the bases only
    nq, nm = degree + 2, degree + 1
    nel = int(target_dofs // nm ** 3)
    xg, _ = orc.gll(nm)
    xq, _ = orc.gauss(nq)
    basis = torch.from_numpy(orc.interpolation_matrix(xg, xq).reshape(-1)).cuda()
    dbasis = torch.from_numpy(orc.derivative_matrix(xq).reshape(-1)).cuda()
    g = torch.Generator(device="cuda").manual_seed(5)
    u = torch.rand(nel * nm ** 3, dtype=torch.float64, device="cuda", generator=g)
    y = torch.empty_like(u)
    jxw = 0.5 + torch.rand(nel * nq ** 3, dtype=torch.float64, device="cuda", generator=g)
    G = torch.rand(nel * 6 * nq ** 3, dtype=torch.float64, device="cuda", generator=g)
    peak = measured_peaks()[0]
    out = {"degree": degree, "n_q_1d": nq, "elements": nel, "evector_dofs": nel * nm ** 3}
    for name, fn, coef_bytes in (
            ("bk1", lambda a: mf.bk1_evector(degree, basis, jxw, u, y, arith=a), 8 * nq ** 3),
            ("bk3", lambda a: mf.bk3_evector(degree, basis, dbasis, G, u, y, arith=a), 48 * nq ** 3)):
        for arith in ("df", "fp64") + (("tc",) if name == "bk1" and degree <= 6 else ()):
            for _ in range(3):
                fn(arith)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                fn(arith)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 10
            byts = nel * (16 * nm ** 3 + coef_bytes)
            out[f"{name}_{arith}"] = {"GDoF/s": nel * nm ** 3 / ms / 1e6, "ms": ms,
                                      "hbm_frac": byts / (ms * 1e-3) / 1e9 / peak}
    del u, y, jxw, G
    return out


def helmholtz_bp5(args):
    """bp5_kokkos's benchmark on the bench mesh: the Helmholtz operator (mass +
    stiffness at QGauss(p+1)), its exact diagonal, Jacobi-PCG with
    ReductionControl(100, 1e-15, 1e-8), best of 4 solves from x = 0, and the
    vmult time as the best of 4 x 50 applies (bp5_kokkos/benchmark.cc:352-397),
    with the seeded U[-1,1] right-hand side."""
    import torch

    import benchmarks_gb300 as mf
    w = WORKLOAD
    mesh = mf.BoxMesh(w["nx"], w["ny"], w["nz"], degree=w["degree"], amplitude=w["amplitude"])

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    H, t_setup = timed(lambda: mf.HelmholtzOperator(mesh, arith=args.arith))
    _, t_diag = timed(H.compute_diagonal)
    P = H.get_matrix_diagonal_inverse()
    b = H.rhs_uniform(w["seed"])
    best, its, converged = None, None, True

    def solve(x, ctl):
        try:
            mf.SolverCG(ctl).solve(H, x, b, P)
        except mf.MfgbError as e:  # the reference catches NoConvergence the same way
            if e.status != mf._abi.ERR_NOT_CONVERGED:
                raise
            return False
        return True

    for _ in range(4):
        x = H.initialize_dof_vector()
        ctl = mf.ReductionControl(100, 1e-15, 1e-8)
        converged, t = timed(lambda: solve(x, ctl))
        best = t if best is None else min(best, t)
        its = ctl.last_step()
        reduction = ctl.last_value() / ctl.initial_value()
    y = H.initialize_dof_vector()
    mv = None
    for _ in range(4):
        _, t = timed(lambda: [H.vmult(y, x) for _ in range(50)])
        mv = t / 50 if mv is None else min(mv, t / 50)
    del H
    return {"n_dofs": mesh.n_dofs, "setup_seconds": t_setup, "diagonal_seconds": t_diag,
            "cg_seconds": best, "cg_iterations": its, "cg_converged": converged,
            "cg_residual_reduction": reduction, "vmult_seconds": mv,
            "vmult_GDoF/s": mesh.n_dofs / mv / 1e9}


def bp3_rate(args):
    """BP3 (Laplacian at QGauss(p+2), L-vector) apply on the bench mesh, GDoF/s."""
    import torch

    import benchmarks_gb300 as mf
    w = WORKLOAD
    A = mf.LaplaceOperator(mf.BoxMesh(w["nx"], w["ny"], w["nz"], degree=w["degree"],
                                      amplitude=w["amplitude"]), arith=args.arith, quadrature="bp3")
    u = A.rhs_uniform(1)
    y = A.initialize_dof_vector()
    for _ in range(3):
        A.vmult(y, u)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        A.vmult(y, u)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    n = A.m()
    del A
    # published: 9.396e-3 s a vmult at 67,634,433 DoFs on one GH200 (FP64 on an
    # affine cube; CEED_bp/results/1xGH200_P4.txt:648)
    return {"GDoF/s": n / ms / 1e6, "ms_per_vmult": ms, "n_q_1d": w["degree"] + 2,
            "published_gh200": 7.20, "ratio_vs_published": n / ms / 1e6 / 7.20}


def bk6_rate(A, args):
    """BK6 on the bench mesh: the vector Laplacian with 3 interleaved FP64
    components per node; GDoF/s counts the 3 components (the CEED convention)."""
    import torch
    n = A.m()
    g = torch.Generator(device="cuda").manual_seed(3)
    u = torch.rand(3 * n, dtype=torch.float64, device="cuda", generator=g)
    y = torch.empty_like(u)
    for _ in range(3):
        A.vmult_vector(y, u, arith=args.arith)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        A.vmult_vector(y, u, arith=args.arith)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    n_cells, n3 = A.n_cells, (A.degree + 1) ** 3
    bytes_per = 3 * 16 * n + n_cells * n3 * 52
    return {"GDoF/s": 3 * n / ms / 1e6, "ms_per_vmult": ms, "components": 3,
            "hbm_frac": bytes_per / (ms * 1e-3) / 1e9 / measured_peaks()[0]}


def gauss_like_for_like(args):
    """The reference's own published configuration: the BP5 variant (QGauss(5)
    on GLL nodal values, affine mesh) at cycle 20 of its scaling study,
    128 x 128 x 64 cells on [-1, 2.8]^2 x [-1, 0.9], 67,634,433 DoFs; published
    6.83 GDoF/s on one A100 (bakeoff_problems_dealii/tests/
    scaling_bp35_kokkos_kernel/results/1_GPU.out:652)."""
    import torch

    import benchmarks_gb300 as mf
    mesh = mf.BoxMesh(128, 128, 64, degree=4, amplitude=0.0, lo=(-1.0, -1.0, -1.0),
                      hi=(2.8, 2.8, 0.9))
    A = mf.LaplaceOperator(mesh, quadrature="gauss", arith=args.arith)
    u = A.rhs_uniform(1)
    y = A.initialize_dof_vector()
    for _ in range(3):
        A.vmult(y, u)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        A.vmult(y, u)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 20
    rate = A.m() / ms / 1e6
    return {"GDoF/s": rate, "ms_per_vmult": ms, "n_dofs": A.m(), "published_a100": 6.83,
            "ratio_vs_published": rate / 6.83}


def kernel_name(degree, arith):
    """Name of the operator kernel the library's shape table launches."""
    import ctypes

    import benchmarks_gb300 as mf
    shape = ctypes.c_int()
    mf.lib().mfgb_get_kernel_shape(arith, degree, ctypes.byref(shape))
    n = degree + 1
    pol = "ArithDF" if arith == 1 else "ArithF64"
    return {0: f"bk5_kernel<{n},{pol}>", 1: f"bk5_pt_kernel<{n},{pol}>",
            2: f"bk5_tma_kernel<{n},{pol}>", 3: f"bk5_kernel_mb<{n},{pol}>",
            4: f"bk5_tma_kernel<{n},alt,{pol}>", 5: f"bk5fx_tma_kernel<{n}>",
            6: f"bk5fx_tma_kernel<{n},alt>"}.get(shape.value, "bk5")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--arith", choices=["df", "fp64"], default="df")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) leg")
    ap.add_argument("--no-degrees", action="store_true", help="skip the p = 3..8 sweep")
    ap.add_argument("--no-solve", action="store_true",
                    help="skip the BP5 solve comparison and the like-for-like Gauss figure")
    ap.add_argument("--cells", type=int, nargs=3, default=None,
                    help="override the mesh (cells per direction) for sweeps and profiling")
    ap.add_argument("--degree", type=int, default=None, help="override the degree p")
    ap.add_argument("--shape", choices=["auto", *SHAPE_CODES], default="auto",
                    help="operator kernel thread layout (default: the library's table)")
    args = ap.parse_args()
    if args.cells:
        WORKLOAD.update(nx=args.cells[0], ny=args.cells[1], nz=args.cells[2])
    if args.degree:
        WORKLOAD.update(degree=args.degree)
    rank, world = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

