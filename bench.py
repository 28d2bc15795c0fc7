"""Benchmark of the batched WENO5 forward path (one JSON line on rank 0).

Workload (the batched plain-method configuration): B = 4096 inviscid Burgers
instances on periodic [-1, 1], N drawn uniformly from {1024, 2048, 4096, 8192,
16384} per instance from the seed, u0 = mean U(-0.5, 0.5) + 8-mode Fourier
series (amplitudes N(0,1)/k^2, uniform phases) + 0-3 jumps of height U(-1, 1)
(exact cell averages), WENO-JS5 (eps 1e-6) + Rusanov + SSPRK33, CFL 0.5
(theta = 1 with the Rusanov estimate), float64, fixed step count.

A "step" is one SSPRK33 step of the whole batch (one persistent kernel launch,
per-instance dt computed on the device). ``value`` = interior cells x steps /
second with the state resident in HBM (two 208 MB ping-pong buffers, larger
than the 129 MB L2, so no flush is needed). ``e2e`` runs the same steps through
the public API with host buffers: each step copies the batch from pinned host
memory, resets the plan, steps once and copies the state back.

``--impl reference`` times the CPU restatement of the reference's path
(``oracle/shocks_ref.c``, OpenMP over instances, all host threads) on a
bounded sample of the same workload: JAX, the reference's runtime, is not
installable here, so the reference itself cannot run.

Multi-GPU (torchrun): every rank runs its own full batch (rank-specific seed),
no data-path collective; the time is the max over ranks (weak scaling).
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SIZES = (1024, 2048, 4096, 8192, 16384)
BATCH = 4096
SEED = 20261203
EPS = 1.0e-6
THETA = 1.0
METRIC = "WENO5 cell-steps/s"
BYTES_PER_CELL_STEP_F64 = 16  # one read + one write of u per fused step


def workload_params(seed: int, batch: int = BATCH):
    """Per-instance sizes and initial-condition parameters from the seed."""
    rng = np.random.default_rng(seed)
    sizes = rng.choice(np.array(SIZES), size=batch)
    params = []
    for _ in range(batch):
        m = rng.uniform(-0.5, 0.5)
        k = np.arange(1, 9)
        amp = rng.normal(0.0, 1.0, size=8) / k**2
        phi = rng.uniform(0.0, 2.0 * np.pi, size=8)
        nj = int(rng.integers(0, 4))
        h = rng.uniform(-1.0, 1.0, size=nj)
        xj = rng.uniform(-1.0, 1.0, size=nj)
        params.append((m, amp, phi, h, xj))
    return sizes.astype(np.int64), params


def initial_state(sizes, params, device):
    """Exact cell averages of the workload's initial conditions, packed
    (float64), evaluated for all instances at once."""
    import torch

    sizes = np.asarray(sizes, dtype=np.int64)
    B = sizes.size
    m = torch.tensor([p[0] for p in params], dtype=torch.float64, device=device)
    amp = torch.tensor(np.stack([p[1] for p in params]), dtype=torch.float64, device=device)
    phi = torch.tensor(np.stack([p[2] for p in params]), dtype=torch.float64, device=device)
    hj = np.zeros((B, 3))
    xj = np.zeros((B, 3))
    for b, p in enumerate(params):
        hj[b, : len(p[3])] = p[3]
        xj[b, : len(p[4])] = p[4]
    hj = torch.tensor(hj, dtype=torch.float64, device=device)
    xj = torch.tensor(xj, dtype=torch.float64, device=device)
    inst = torch.repeat_interleave(torch.arange(B, device=device),
                                   torch.tensor(sizes, device=device))
    off = torch.tensor(np.concatenate([[0], np.cumsum(sizes)[:-1]]), device=device)
    local = torch.arange(int(sizes.sum()), device=device) - off[inst]
    nb = torch.tensor(sizes, dtype=torch.float64, device=device)[inst]
    hh = 2.0 / nb
    fl = -1.0 + local.double() * hh
    fr = -1.0 + (local + 1).double() * hh
    u = m[inst].clone()
    for kk in range(8):
        k = kk + 1
        ph = phi[inst, kk]
        u += amp[inst, kk] * (torch.cos(k * np.pi * fl + ph) - torch.cos(k * np.pi * fr + ph)) / (
            k * np.pi * hh)
    for j in range(3):
        u += hj[inst, j] * torch.clamp((fr - xj[inst, j]) / hh, 0.0, 1.0)
    return u


def fourier_perturbation(n: int, B: int, seed: int, device):
    """Exact cell averages of B random 8-mode Fourier series on [-1, 1] with N=n
    (amplitudes N(0,1)/k^2, uniform phases, no mean, no jumps): the adjoint
    configuration's target perturbation, one series per instance."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, 9)
    prm = [(0.0, rng.normal(0.0, 1.0, size=8) / k**2, rng.uniform(0.0, 2.0 * np.pi, size=8),
            np.zeros(0), np.zeros(0)) for _ in range(B)]
    return initial_state(np.full(B, n), prm, device)


# {{{ clocks


class ClockSampler:
    """``nvidia-smi`` samples of SM clock and throttle reasons during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), parts[4:9]))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for _, _, flags in rows:
            for nm, fl in zip(names, flags[1:]):
                if fl.lower() == "active":
                    reasons.add(nm)
        load = [r[0] for r in rows]
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


# }}}


def _profile_constants() -> dict:
    p = ROOT / "profiles" / "roofline_constants.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def _measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def _cpu_inputs(sizes, params, n_inst: int):
    """Packed initial state, offsets and cell sizes of the first *n_inst*
    instances, on the host."""
    sub_sizes = sizes[:n_inst]
    u0 = initial_state(sub_sizes, params[:n_inst], "cpu").numpy()
    off = np.zeros(n_inst + 1, dtype=np.int64)
    off[1:] = np.cumsum(sub_sizes)
    return u0, off, 2.0 / sub_sizes.astype(np.float64)


def run_cpu_sample(sizes, params, *, n_inst: int, nsteps: int, threads: int = 0):
    """Time the C restatement of the reference path on the first *n_inst*
    instances for *nsteps* steps (best of 3); returns (cell-steps/s, threads)."""
    from oracle import c_ref

    u0, off, dx = _cpu_inputs(sizes, params, n_inst)
    c_ref.run_batch(u0, off, dx, theta=THETA, eps=EPS, nsteps=1, nthreads=threads)  # warm-up
    best = None
    used = 1
    for _ in range(3):
        t0 = time.perf_counter()
        _, _, used = c_ref.run_batch(u0, off, dx, theta=THETA, eps=EPS, nsteps=nsteps,
                                     nthreads=threads)
        el = time.perf_counter() - t0
        best = el if best is None else min(best, el)
    return float(off[-1]) * nsteps / best, used


def bench_reference(args, rank: int) -> None:
    if rank != 0:
        return
    from oracle import c_ref

    sizes, params = workload_params(SEED)
    n_inst = args.cpu_instances
    u0, off, dx = _cpu_inputs(sizes, params, n_inst)
    vals = []
    used = 1
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, used = c_ref.run_batch(u0, off, dx, theta=THETA, eps=EPS, nsteps=1, nthreads=0)
        rate = float(off[-1]) / (time.perf_counter() - t0)
        if i >= args.warmup:
            vals.append(rate)
    value = float(np.median(vals))
    cells = int(off[-1])
    sample = (f"first {n_inst} of the {BATCH} seeded instances ({cells} cells), one SSPRK33 "
              f"step per timed step from the initial state, median of the timed steps")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "cell-steps/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * cells / value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": _config(args),
        "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": used, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference runs on JAX, which is not installable in this image; the "
                 "timed CPU code is the C restatement of its path (oracle/shocks_ref.c)"),
    }
    print(json.dumps(line), flush=True)


def _config(args) -> dict:
    what = {"plain": "plain WENO-JS5", "plain32": "plain WENO-JS5 (float32 state)",
            "learned": "learned-weight WENO (float64 state)",
            "learned32": "learned-weight WENO (float32 state)"}[getattr(args, "scheme", "plain")]
    return {
        "workload": f"batched {what}+Rusanov+SSPRK33 Burgers, B={args.batch}, "
                    "N~U{1024..16384}, CFL 0.5, periodic",
        "batch": args.batch,
        "sizes": list(SIZES),
        "seed": SEED,
        "eps": EPS,
        "theta": THETA,
        "precision": "float64",
        "l2": "state (2 x 208 MB ping-pong) larger than the 129 MB L2; no flush",
        "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
        "tile": args.tile,
    }


def bench_gpu(args, rank: int, world: int) -> None:
    import torch

    import pyshocks_gb300 as gb
    from pyshocks_gb300 import _lib as L
    from pyshocks_gb300.batched import BatchedSolver, HostStepper

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sizes, params = workload_params(SEED + rank, batch=args.batch)
    cells = int(np.sum(sizes))
    rec = gb.reconstruction.make_reconstruction_from_name("wenojs53", eps=EPS)
    scheme = gb.burgers.make_scheme_from_name("rusanov", rec=rec)
    u0 = initial_state(sizes, params, dev)
    if args.scheme.startswith("learned"):
        # profiling aid: the learned-weight step on the same batch (float64
        # state with the float operator, or float32 state)
        from pyshocks_gb300 import learned

        lscheme = gb.burgers.Rusanov(rec=learned.LearnedWENO(params=learned.load_default_params()))
        solver = BatchedSolver(lscheme, sizes, 2.0 / sizes.astype(np.float64), theta=THETA,
                               dtype=torch.float32 if args.scheme == "learned32" else torch.float64,
                               tile=args.tile)
    else:
        solver = BatchedSolver(scheme, sizes, 2.0 / sizes.astype(np.float64), theta=THETA,
                               dtype=torch.float32 if args.scheme == "plain32" else torch.float64,
                               tile=args.tile)
    stream = torch.cuda.Stream(device=dev)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

    def barrier():
        if dist is not None:
            dist.barrier()

    with torch.cuda.stream(stream):
        solver.reset(u0)
        # warm-up (also captures the two-step graph)
        solver.step(2 * max(1, (args.warmup + 1) // 2), graph=True)
        stream.synchronize()
        k = args.steps + (args.steps % 2)
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            torch.cuda.nvtx.range_push("timed")
            e0.record(stream)
            solver.step(k, graph=True)
            e1.record(stream)
            e1.synchronize()
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        status = solver.status()
    if status:
        raise RuntimeError(f"step kernel reported status {status}")
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    total_cells = cells * world
    value = total_cells * k / (ms_max * 1e-3)
    per_launch_s = ms * 1e-3 / k

    e2e = None
    if not args.profile:
        # e2e through the public host-buffer API (shk_host_stepper_advance):
        # every step copies the whole packed state in from pinned host memory,
        # resets and steps it, and copies the result back, with the batch in
        # chunks whose copies overlap the other chunks' steps
        hs = HostStepper(solver.scheme, sizes, 2.0 / sizes.astype(np.float64), theta=THETA,
                         dtype=solver.dtype, tile=solver.tile, ctas_per_sm=solver.ctas_per_sm,
                         chunks=args.e2e_chunks)
        host_in = u0.to(solver.dtype).cpu().pin_memory()
        host_out = torch.empty_like(host_in).pin_memory()
        ke = max(2, min(args.steps, 10))
        reps = []
        with torch.cuda.stream(stream):
            hs.advance(host_in, host_out, 1)
            stream.synchronize()
            for _ in range(3):
                barrier()
                t0 = time.perf_counter()
                f0 = torch.cuda.Event(enable_timing=True)
                f1 = torch.cuda.Event(enable_timing=True)
                f0.record(stream)
                for _ in range(ke):
                    hs.advance(host_in, host_out, 1)
                f1.record(stream)
                f1.synchronize()
                wall = time.perf_counter() - t0
                # wall clock: host calls, copies and kernels of every e2e step
                reps.append(total_cells * ke / max(wall, f0.elapsed_time(f1) * 1e-3))
        if hs.status():
            raise RuntimeError("host stepper reported a nonzero status")
        # the median of three repetitions of ke steps (a host hiccup in one of
        # them does not set the figure)
        e2e_value = float(statistics.median(reps))
        e2e = {"value": e2e_value, "unit": "cell-steps/s",
               "h2d_bytes_per_step": int(host_in.numel() * host_in.element_size()),
               "d2h_bytes_per_step": int(host_out.numel() * host_out.element_size()),
               "chunks": hs.chunks, "steps_per_repetition": ke,
               "repetitions": [float(r) for r in reps]}
        del hs

    peaks = _measured_peaks()
    consts = _profile_constants()
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)"
    if hbm_peak is None:
        hbm_peak, peak_src = 6800.0, "profiling-recipe fallback 6.8 TB/s (of fallback)"
    algo_bytes = BYTES_PER_CELL_STEP_F64 * cells
    if solver.dtype == torch.float32:  # profiling aid: float32 state, 8 B per cell-step
        algo_bytes //= 2
    achieved = algo_bytes / per_launch_s / 1e9
    traffic = None
    if "dram_bytes_per_cell_step" in consts and args.scheme == "plain":
        traffic = consts["dram_bytes_per_cell_step"] * cells  # measured on the plain FP64 step
    fp64_peak = None if args.profile else ctypes_fp_peak(L)
    fp64 = None
    if "fp64_flop_per_cell_step" in consts and fp64_peak:
        fl = consts["fp64_flop_per_cell_step"] * cells / per_launch_s
        fp64 = {"achieved": fl / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                "frac": fl / fp64_peak, "flop_per_cell_step": consts["fp64_flop_per_cell_step"],
                "peak_source": "shk_measure_fp_peak FMA chains on this GPU (of measured)"}
    elif fp64_peak:
        fp64 = {"peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                "peak_source": "shk_measure_fp_peak FMA chains on this GPU (of measured)"}

    extra = None
    if rank == 0 and not args.profile and not args.no_extra:
        adj = bench_adjoint(scheme, dev, args)
        extra = {"fp32_forward": bench_fp32(scheme, sizes, u0, stream, args),
                 "adjoint": adj,
                 "learned": bench_learned(scheme, dev, stream, args, adj),
                 "inverse_lwr": bench_inverse(dev, args)}

    cpu = None
    if rank == 0 and not args.no_cpu and not args.profile:
        rate, used = run_cpu_sample(sizes, params, n_inst=args.cpu_instances, nsteps=1)
        cpu = {"value": rate, "unit": "cell-steps/s", "cores": used, "kind": "port",
               "sample": f"first {args.cpu_instances} of the {BATCH} instances of the batch, "
                         f"one step, C restatement (oracle/shocks_ref.c), best of 3"}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "cell-steps/s",
            "n_gpus": world,
            "steps": k,
            "warmup": args.warmup,
            "ms_per_step": ms_max / k,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32" if solver.dtype == torch.float32 else "f64",
            "data": "synthetic",
            "config": _config(args),
            "clocks": clk.summary(),
            "e2e": e2e,
            "gpu_launches": k,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "kernel": (f"batched_step_kernel<{'float' if args.scheme == 'plain32' else 'double'},"
                                    "Burgers,WENOJS53,Rusanov>"
                                    if args.scheme.startswith("plain") else
                                    f"batched_step_kernel<{'float' if args.scheme == 'learned32' else 'double'},"
                                    "Burgers,LEARNED,Rusanov>"),
                         "algo_bytes_per_launch": algo_bytes, "peak_source": peak_src},
            "fp64_pipe": fp64,
            "cpu_baseline": cpu,
            "extra": extra,
        }
        print(json.dumps(line), flush=True)


def _timed_steps(solver, u0, k, stream) -> float:
    """ms per step of *k* graph-captured steps after a warm-up."""
    import torch

    with torch.cuda.stream(stream):
        solver.reset(u0)
        solver.step(4, graph=True)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.step(k, graph=True)
        e1.record(stream)
        e1.synchronize()
    if solver.status():
        raise RuntimeError(f"step kernel reported status {solver.status()}")
    return e0.elapsed_time(e1) / k


def bench_fp32(scheme, sizes, u0, stream, args) -> dict:
    """Same batch with float32 state (float64 dt and reductions): rate, and the
    error against the float64 run and the conservation drift after the
    configuration's ``--accuracy-steps`` (2000) steps from the initial state."""
    import torch

    from pyshocks_gb300.batched import BatchedSolver

    dx = 2.0 / sizes.astype(np.float64)
    k = args.steps + (args.steps % 2)
    s32 = BatchedSolver(scheme, sizes, dx, dtype=torch.float32, tile=args.tile)
    ms = _timed_steps(s32, u0, k, stream)  # ms per step
    cells = int(np.sum(sizes))
    rate = cells / (ms * 1e-3)
    nacc = args.accuracy_steps + (args.accuracy_steps % 2)
    s64 = BatchedSolver(scheme, sizes, dx)
    with torch.cuda.stream(stream):
        s32.reset(u0)
        s32.step(nacc, graph=True)
        s64.reset(u0)
        m0 = s64.reduce(0)
        s64.step(nacc, graph=True)
        diff = (s32.u.double() - s64.u).abs()
        inst = torch.repeat_interleave(torch.arange(len(sizes), device=diff.device),
                                       torch.tensor(sizes, device=diff.device))
        l1 = torch.zeros(len(sizes), dtype=torch.float64, device=diff.device).index_add_(0, inst, diff)
        l1 = l1 * torch.tensor(dx, device=diff.device)
        drift64 = ((s64.reduce(0) - m0).abs() / torch.tensor(sizes, device=diff.device)).max()
        drift32 = ((s32.reduce(0) - m0).abs() / torch.tensor(sizes, device=diff.device)).max()
        stream.synchronize()
    return {"metric": "WENO5 cell-steps/s (float32 state)", "value": rate, "unit": "cell-steps/s",
            "ms_per_step": ms, "algo_gb_per_s": 8 * rate / 1e9,
            "launch_shape": {"tile": s32.tile, "ctas_per_sm": s32.ctas_per_sm},
            "vs_float64_after_steps": nacc,
            "l1_mean": float(l1.mean()), "linf": float(diff.max()),
            "mass_drift_per_cell_max": {"float64": float(drift64), "float32": float(drift32)}}


def _adjoint_rate(scheme, dev, nsteps, dtype, B=256, n=4096, tile="auto") -> dict:
    """B Burgers instances, N=4096, initial condition 0.5 + sin(pi x) (cell averages),
    J = 1/2 |u(T) - u_target|^2, sqrt(n)-checkpointed reverse sweep. One
    gradient = one instance's full dJ/du0."""
    import torch

    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    # exact cell averages of 0.5 + sin(pi x) on [-1, 1]
    f = np.linspace(-1.0, 1.0, n + 1)
    u1 = 0.5 + (np.cos(np.pi * f[:-1]) - np.cos(np.pi * f[1:])) / (np.pi * (2.0 / n))
    u0 = torch.tensor(np.tile(u1, B), device=dev, dtype=dtype)
    solver = BatchedSolver(scheme, [n] * B, 2.0 / n, max_steps=nsteps, dtype=dtype, tile=tile)
    cs = CheckpointedSolve(solver, nsteps)
    pert = fourier_perturbation(n, B, SEED + 3, dev).to(dtype)
    target = cs.forward((u0 + 0.05 * pert).contiguous()).clone()
    cs.forward(u0)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    uT = cs.forward(u0)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g = cs.backward(uT - target)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    if solver.status() or not torch.isfinite(g).all():
        raise RuntimeError("adjoint run failed")
    return {"metric": "adjoint grads/s", "value": B / (t2 - t0), "unit": "gradients/s",
            "config": {"batch": B, "n": n, "steps": nsteps, "checkpoint_stride": cs.stride,
                       "dtype": str(dtype).replace("torch.", ""),
                       "launch_shape": {"tile": solver.tile, "ctas_per_sm": solver.ctas_per_sm}},
            "forward_s": t1 - t0, "reverse_s": t2 - t1,
            "adjoint_cell_steps_per_s": n * B * nsteps / (t2 - t1)}


def bench_adjoint(scheme, dev, args) -> dict:
    """The adjoint configuration in float64 (B=256, N=4096, 4000 steps)."""
    import torch

    return _adjoint_rate(scheme, dev, args.adjoint_steps, torch.float64, tile=args.tile)


def bench_learned(plain, dev, stream, args, adjoint_plain) -> dict:
    """Learned-weight WENO against the plain float64 kernel: forward rate on
    B=4096 x N=4096, adjoint rate on the adjoint configuration, and L1 error
    at t=0.4 against the plain float64 solution on a 4x finer grid (restricted
    by averaging) for ``--accuracy-batch`` instances (512 by default) of the
    same initial-condition family. The fine solution stays in float64: a
    float32 one raised every scheme's L1 by about 1.3e-5 (6 %), alike for all,
    which shifts the equal-error comparison; in float64 the configuration's
    4096 instances would take the fine grid about 190 s."""
    import torch

    from pyshocks_gb300 import burgers, learned
    from pyshocks_gb300.batched import BatchedSolver

    params = learned.load_default_params(device=dev)
    lrec = learned.LearnedWENO(params=params)
    lscheme = burgers.Rusanov(rec=lrec)
    uscheme = burgers.Rusanov(rec=learned.LearnedWENO(params=learned.init_params(device=dev)))
    n = 4096
    k = args.steps + (args.steps % 2)
    B = 4096
    u0 = initial_state(np.full(B, n), workload_params(SEED + 4, batch=B)[1], dev)
    rates = {}
    shapes = {}
    for name, sch, dt in (("plain_f64", plain, torch.float64),
                          ("plain_f32", plain, torch.float32),
                          ("learned_f64", lscheme, torch.float64),
                          ("learned_f32", lscheme, torch.float32)):
        s = BatchedSolver(sch, [n] * B, 2.0 / n, dtype=dt, tile=args.tile)
        shapes[name] = {"tile": s.tile, "ctas_per_sm": s.ctas_per_sm}
        rates[name] = B * n / (_timed_steps(s, u0, k, stream) * 1e-3)
        del s
    # accuracy
    Bl, r, T = args.accuracy_batch, 4, 0.4
    prm = workload_params(SEED + 5, batch=Bl)[1]

    def run(sch, nn, dt):
        """The accuracy set on nn cells to t=T: (state, mean steps taken)."""
        s = BatchedSolver(sch, [nn] * Bl, 2.0 / nn, dtype=dt, max_steps=2 * nn)
        with torch.cuda.stream(stream):
            s.reset(initial_state(np.full(Bl, nn), prm, dev), tfinal=T)
            while float(s.time().min()) < T:
                s.step(256, graph=True)
            stream.synchronize()
        if s.status():
            raise RuntimeError("accuracy run failed")
        # mean number of steps an instance takes to reach T (per-instance CFL dt)
        steps = float((s.dt_history() > 0).sum(0).double().mean())
        return s.u.double().reshape(Bl, nn), steps

    fine, _ = run(plain, n * r, torch.float64)
    # cumulative integral of the fine piecewise-constant solution at its faces
    nf = n * r
    cum = torch.cat([torch.zeros(Bl, 1, dtype=torch.float64, device=dev),
                     torch.cumsum(fine, -1) * (2.0 / nf)], -1)
    del fine

    def l1(u):
        """L1 distance to the fine solution averaged onto u's cells (exact
        cell averages of the piecewise-constant fine solution, any N), mean
        over the instances."""
        nn = u.shape[-1]
        xf = torch.arange(nn + 1, dtype=torch.float64, device=dev) * (nf / nn)
        i0 = torch.clamp(xf.floor().long(), max=nf - 1)
        w = xf - i0
        F = cum[:, i0] + w * (cum[:, i0 + 1] - cum[:, i0])
        avg = (F[:, 1:] - F[:, :-1]) / (2.0 / nn)
        return float((u - avg).abs().sum(-1).mean() * 2.0 / nn)

    runs = {"plain_f64": run(plain, n, torch.float64), "plain_f32": run(plain, n, torch.float32),
            "learned_f64": run(lscheme, n, torch.float64),
            "learned_f32": run(lscheme, n, torch.float32),
            "untrained_f64": run(uscheme, n, torch.float64)}
    err = {k_: l1(v[0]) for k_, v in runs.items()}
    iso = bench_iso_l1(plain, lscheme, run, l1, err, runs, rates, stream, dev, args, B, n, T)
    adj = {"learned_f64": _adjoint_rate(lscheme, dev, args.adjoint_steps, torch.float64, tile=args.tile),
           "learned_f32": _adjoint_rate(lscheme, dev, args.adjoint_steps, torch.float32, tile=args.tile)}
    return {
        "forward": {"unit": "cell-steps/s", "config": {"batch": B, "n": n, "steps": k},
                    "launch_shapes": shapes, **rates,
                    "speedup_learned_f64": rates["learned_f64"] / rates["plain_f64"],
                    "speedup_learned_f32": rates["learned_f32"] / rates["plain_f64"],
                    "learned_f64_vs_plain_f32": rates["learned_f64"] / rates["plain_f32"]},
        "adjoint": {"unit": "gradients/s", "plain_f64": adjoint_plain["value"],
                    "launch_shapes": {"plain_f64": adjoint_plain["config"]["launch_shape"],
                                      "learned_f64": adj["learned_f64"]["config"]["launch_shape"],
                                      "learned_f32": adj["learned_f32"]["config"]["launch_shape"]},
                    "learned_f64": adj["learned_f64"]["value"],
                    "learned_f32": adj["learned_f32"]["value"],
                    "speedup_learned_f64": adj["learned_f64"]["value"] / adjoint_plain["value"],
                    "speedup_learned_f32": adj["learned_f32"]["value"] / adjoint_plain["value"]},
        "l1_vs_fine_plain": {"config": {"batch": Bl, "n": n, "t_final": T, "fine": n * r,
                                        "fine_state": "float64"},
                             **err, "steps": {k_: v[1] for k_, v in runs.items()}},
        "iso_l1": iso,
        "note": ("learned_f64 keeps the state and its accumulation in float64 and runs the "
                 "operator in float32 (bfloat16 tensor-core network); learned_f32 also "
                 "stores the state in float32. untrained_f64: the network at initialisation "
                 "(softmax at the ideal weights) with the same trust band"),
    }


def bench_iso_l1(plain, lscheme, run, l1, err, runs, rates, stream, dev, args, B, n, T) -> dict:
    """Learned vs plain at equal L1 error. The plain scheme (float64 and
    float32 state) is run on finer grids of the same accuracy set until its L1
    against the fine solution reaches the learned scheme's L1 at N=n (a
    resolution ladder, then a log-log interpolation between the bracketing
    resolutions, rounded up to a multiple of 64 and verified by a run there).
    Time to solution is for the configuration's batch (B instances to t=T):
    B x N x (mean steps an instance takes to reach T on that grid) / the
    cell-steps/s measured at B x N (for the plain scheme, the better of that
    and its rate at B x n). The ratios are plain time / learned time."""
    import math

    import torch

    from pyshocks_gb300.batched import BatchedSolver

    target = err["learned_f64"]
    k = args.steps + (args.steps % 2)

    def rate_at(sch, nn, dt):
        s = BatchedSolver(sch, [nn] * B, 2.0 / nn, dtype=dt, tile=args.tile)
        u0 = initial_state(np.full(B, nn), workload_params(SEED + 4, batch=B)[1], dev)
        r = B * nn / (_timed_steps(s, u0, k, stream) * 1e-3)
        del s
        return r

    out = {"target_l1": target, "learned_n": n,
           "config": {"batch": B, "t_final": T, "accuracy_batch": args.accuracy_batch}}
    lsteps = runs["learned_f64"][1]
    t_learned = B * n * lsteps / rates["learned_f64"]
    out["learned_f64"] = {"n": n, "l1": target, "steps": lsteps, "rate": rates["learned_f64"],
                          "time_to_solution_s": t_learned}
    for name, dt in (("plain_f64", torch.float64), ("plain_f32", torch.float32)):
        pts = [(n, err[name])]
        nn = n
        while pts[-1][1] > target and nn < 2 * n:
            nn += n // 8
            pts.append((nn, l1(run(plain, nn, dt)[0])))
        if pts[-1][1] > target:
            raise RuntimeError(f"{name}: no grid up to {nn} cells reaches L1 {target:.3e}")
        if len(pts) == 1:
            nstar = n
        else:
            (n1, e1), (n2, e2) = pts[-2], pts[-1]
            p = math.log(e1 / e2) / math.log(n2 / n1) if e1 > e2 else 1.0
            nstar = n1 * (e1 / target) ** (1.0 / p)
            nstar = int(math.ceil(nstar / 64.0)) * 64
        u, steps = run(plain, nstar, dt)
        e = l1(u)
        while e > target:
            nstar += 64
            u, steps = run(plain, nstar, dt)
            e = l1(u)
        # the plain scheme's cost per cell-step does not depend on N, but the
        # measured rate at N* carries that size's tile fit (e.g. 4544 = 2 x 2048
        # + 448): the better of the rates at N* and at n is used (the
        # conservative choice for the learned scheme), both reported
        r_star = rate_at(plain, nstar, dt)
        r = max(r_star, rates[name])
        t = B * nstar * steps / r
        out[name] = {"n": nstar, "l1": e, "steps": steps, "rate": r, "rate_at_n": r_star,
                     f"rate_at_{n}": rates[name], "time_to_solution_s": t,
                     "ladder": [[a, b] for a, b in pts]}
        out[f"ratio_learned_f64_vs_{name}"] = t / t_learned
    return out


def bench_inverse(dev, args) -> dict:
    """The batched LWR inverse problem (learned scheme, float32 state, float64
    misfits, whole iteration in a CUDA graph): B=1024 instances with N from
    {4096..65536}; ``--inverse-steps`` SSPRK33 steps per solve (the full
    configuration has 3000) and a few timed gradient-descent iterations."""
    import torch

    from pyshocks_gb300 import burgers, learned
    from pyshocks_gb300.inverse import InverseProblem, lwr_initial_states

    rng = np.random.default_rng(SEED + 6)
    B = 1024
    sizes = rng.choice(np.array([4096, 8192, 16384, 32768, 65536]), size=B)
    rec = learned.LearnedWENO(params=learned.load_default_params(device=dev))
    prob = InverseProblem(burgers.LWRRusanov(rec=rec), sizes, 2.0 / sizes.astype(np.float64),
                          args.inverse_steps, lr=0.5)
    truth = lwr_initial_states(rng, sizes, device=dev)
    prob.observe(truth)
    guess = torch.cat([torch.full((int(m),), float(x.mean()), dtype=torch.float64, device=dev)
                       for m, x in zip(sizes, torch.split(truth, list(sizes)))])
    prob.run(guess, 1, graph=True)  # capture + warm-up
    torch.cuda.synchronize()
    iters = args.inverse_iters
    t0 = time.perf_counter()
    hist = prob.run(guess, iters, graph=True)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / iters
    j = torch.stack(hist).sum(-1).cpu().numpy()
    cells = int(sizes.sum())
    return {"config": {"batch": B, "cells": cells, "steps": args.inverse_steps,
                       "full_steps": 3000, "iterations_timed": iters},
            "s_per_iteration": dt,
            "cell_steps_per_s": 2 * cells * args.inverse_steps / dt,
            "est_s_per_iteration_full": dt * 3000 / args.inverse_steps,
            "misfit_sum": [float(x) for x in j],
            "note": "cell_steps_per_s counts the forward and the reverse sweep of each iteration"}


def profile_adjoint(args) -> None:
    """The adjoint leg alone (for ncu captures of the reverse-step kernel)."""
    import torch

    import pyshocks_gb300 as gb
    from pyshocks_gb300 import learned

    dev = torch.device("cuda", 0)
    if args.scheme.startswith("plain"):
        sch = gb.burgers.Rusanov(rec=gb.reconstruction.make_reconstruction_from_name("wenojs53", eps=EPS))
    else:
        sch = gb.burgers.Rusanov(rec=learned.LearnedWENO(params=learned.load_default_params(device=dev)))
    dtype = torch.float32 if args.scheme.endswith("32") else torch.float64
    r = _adjoint_rate(sch, dev, args.adjoint_steps, dtype, B=args.batch, tile=args.tile)
    print(json.dumps({"profile_adjoint": args.scheme, **r}), flush=True)


def ctypes_fp_peak(L):
    import ctypes

    v = ctypes.c_double()
    st = L.lib().shk_measure_fp_peak(L.SHK_F64, 4096, ctypes.byref(v))
    return float(v.value) if st == 0 else None


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-instances", type=int, default=BATCH,
                    help="instances of the batch in the CPU samples (default: all)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the float32 and adjoint measurements")
    ap.add_argument("--e2e-chunks", type=int, default=0,
                    help="chunks of the pipelined host-buffer e2e leg (0: the library default)")
    ap.add_argument("--adjoint-steps", type=int, default=4000)
    ap.add_argument("--accuracy-batch", type=int, default=512,
                    help="instances of the learned-vs-plain L1 comparison (their float64 "
                         "solution on the 4x finer grid costs about 24 s per 512)")
    ap.add_argument("--accuracy-steps", type=int, default=2000,
                    help="steps of the float32-vs-float64 comparison of the batch (full: 2000)")
    ap.add_argument("--inverse-steps", type=int, default=3000,
                    help="SSPRK33 steps per solve of the inverse-problem leg (the configuration's 3000)")
    ap.add_argument("--inverse-iters", type=int, default=2,
                    help="timed gradient-descent iterations of the inverse-problem leg (of the "
                         "configuration's 50)")
    ap.add_argument("--inverse-only", action="store_true",
                    help="run only the inverse-problem leg (one JSON line)")
    ap.add_argument("--scheme", choices=["plain", "plain32", "learned", "learned32"], default="plain",
                    help="profiling aid: time the plain step with float32 state, or the "
                         "learned-weight step (float64 state with the float operator, or "
                         "float32 state), instead of the plain float64 one")
    ap.add_argument("--tile", default="auto",
                    help="cells per work item of the batched plans, or 'auto' (autotuner: tile "
                         "and CTAs/SM timed on the batch); 0 = library default")
    ap.add_argument("--batch", type=int, default=BATCH,
                    help="profiling aid: instances of the batch (default: the workload's 4096)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="profiling aid: only the checkpointed adjoint of --scheme on --batch "
                         "instances of N=4096 for --adjoint-steps steps")
    ap.add_argument("--profile", action="store_true",
                    help="timed region only (no e2e, CPU baseline or FP peak): for ncu")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.tile != "auto":
        args.tile = int(args.tile)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        bench_reference(args, rank)
        return
    if args.profile_adjoint:
        profile_adjoint(args)
        return
    if args.inverse_only:
        import torch

        print(json.dumps({"inverse_lwr": bench_inverse(torch.device("cuda", 0), args)}), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    bench_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
