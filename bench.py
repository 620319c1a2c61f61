"""Benchmark of the MAC mr-SAV stage hot path on one or more GB300s.

Metric (cell-stage updates/s): nx*ny*(stages completed)/second.  The default
workload is the learned-preconditioner case: the 1024^2 unit-square cavity,
nu=1e-4, sdirk3_mrsav, dt=1e-4, stream-function modes k,l <= 32 (seeded
synthetic field).  ``value`` is FP32 bulk with the learned preconditioner
(FP32 transforms/stencils/Krylov vectors, FP64 reductions, FP64 defect
correction so the reference's 1e-9 Stokes and 1e-8 stage gates hold;
flexible CG at Krylov tolerance 1e-10 whose first search direction per Stokes
solve comes from the trained U-Net), with the state resident in HBM.  Beside
it: the plain FP64 path at 1e-12 (``fp64``, ``speedup_vs_fp64``), plain FP32
bulk (``plain_fp32``), the errors against the FP64 run and, for the first
step, against the CPU oracle; ``e2e`` is the same metric through the public
API (``scheme.step(model, state, dt)`` with host states), ``roofline`` the
dominant kernel against the measured HBM bandwidth, ``cpu_baseline`` the
oracle on one step.  The network is trained and judged before the timed
region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload learned1024|cavity512|ensemble256|adaptive2048|channel512]

``--workload cavity512`` is the 512^2 precision case (nu=1e-3, dt=2.5e-4,
modes <= 16) with the FP32-vs-FP64 trajectory errors over its 200 steps;
``ensemble256`` the mixed-size ensemble: 256 cavities (nx, ny drawn from
{64, 96, 128, 192, 256}, domain [0, nx/ny] x [0, 1], nu log-uniform in
[1e-4, 1e-2], psi modes k,l <= 8, sdirk2_mrsav, dt=5e-4), all members' steps
in flight at once (``Ensemble``); with N ranks the members are sharded by
cell count (``scaling: strong``).

Multi-GPU: independent replicas of the cavity, one per rank (a single cavity
does not shard; the reference has no distributed path), ``scaling: weak``.
``--impl reference`` times the CPU oracle (a NumPy/SciPy restatement of the
reference's own path, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import contextlib
import ctypes as C
import gc
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {"workload": "cavity512_sdirk3_mrsav", "nx": 512, "ny": 512, "lx": 1.0, "ly": 1.0, "nu": 1e-3,
            "dt": 2.5e-4, "scheme": "sdirk3_mrsav", "psi_modes": 16, "seed": 20261203, "stages_per_step": 4}
METRIC = "cell-stage updates/s"
L2_BYTES = 129 * 2 ** 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """SM clock and throttle-reason samples taken during the timed region.

    Reads NVML through ctypes (read-only queries: clocks, maximum clocks and
    the active clock-event reasons) every 10 ms on a background thread, so a
    timed region of a few tens of milliseconds still gets several samples;
    falls back to ``nvidia-smi -lms 200`` where NVML cannot be loaded.
    """

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
                   "hw_thermal_slowdown": 0x40}
    PERIOD_S = 0.010

    def __init__(self, index: int) -> None:
        self.index = index
        self.proc = None
        self.thread = None
        self.samples = []   # (sm_mhz, max_mhz, reasons bitmask)
        self.lines = []

    def _nvml(self):
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        if lib.nvmlInit_v2() != 0:
            return None
        dev = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(dev)) != 0:
            lib.nvmlShutdown()
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
        if reasons is None:
            lib.nvmlShutdown()
            return None
        return lib, dev, reasons

    def _loop(self, lib, dev, reasons):
        sm, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.stop.is_set():
            ok = (lib.nvmlDeviceGetClockInfo(dev, 1, C.byref(sm)) == 0          # NVML_CLOCK_SM
                  and lib.nvmlDeviceGetMaxClockInfo(dev, 1, C.byref(mx)) == 0
                  and reasons(dev, C.byref(rs)) == 0)
            if ok:
                self.samples.append((float(sm.value), float(mx.value), int(rs.value)))
            self.stop.wait(self.PERIOD_S)

    def __enter__(self):
        import threading
        h = self._nvml()
        if h is not None:
            self.nvml = h
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._loop, args=h, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.thread is not None:
            self.stop.set()
            self.thread.join(timeout=5)
            self.nvml[0].nvmlShutdown()
            return
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        for s, m, bits in self.samples:
            sm.append(s)
            mx.append(m)
            reasons.update(name for name, bit in self.REASON_BITS.items() if bits & bit)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvml" if self.samples else "nvidia-smi"}


def initial_state(pkg):
    w = WORKLOAD
    return pkg.fields.packed_curl_velocity(w["nx"], w["ny"], w["lx"], w["ly"], w["psi_modes"], w["seed"])


def cpu_baseline(w=None, steps: int = 2, threads: int = 1) -> dict:
    """The CPU oracle (restatement of the reference path) on a bounded sample:
    ``steps`` steps of workload ``w`` from its seeded field, Krylov tolerance
    1e-12 (the reference's own)."""
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    import oracle
    w = w or WORKLOAD
    g = oracle.Grid(w["nx"], w["ny"], w["lx"], w["ly"])
    model = oracle.OracleModel(g, w["nu"], backend=oracle.TensorStokesOracle(g, 1e-9, 1e-12, workers=threads))
    scheme = oracle.make_scheme(w["scheme"])
    x0 = pkg.fields.packed_curl_velocity(w["nx"], w["ny"], w["lx"], w["ly"], w["psi_modes"], w["seed"])
    state = model.state(0.0, x0, 1.0)
    t0 = time.perf_counter()
    for _ in range(steps):
        state = scheme.step(model, state, w["dt"]).state
    sec = time.perf_counter() - t0
    cells = w["nx"] * w["ny"] * w["stages_per_step"] * steps
    return {"value": cells / sec, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the {w['workload']} workload (NumPy/SciPy oracle, {threads} thread(s))",
            "seconds": sec}


def run_reference(args) -> None:
    """The reference arm: the oracle (the reference's CPU path restated in
    NumPy/SciPy; the reference itself is Python and cannot travel here) on
    the same workload and metric, with every host thread for SciPy's FFTs, a
    bounded sample of min(K, 3) steps.  Under torchrun only rank 0 runs."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = WORKLOAD if args.workload == "cavity512" else HEADLINE
    steps = max(1, min(args.steps, 3))
    base = cpu_baseline(w, steps=steps, threads=threads)
    value = base["value"]
    line = {"metric": METRIC, "value": value, "unit": "cell-stage/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * base["seconds"] / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded stream-function curl field)",
            "config": {"workload": w["workload"], **{k: w[k] for k in ("nx", "ny", "nu", "dt", "scheme",
                                                                       "psi_modes")},
                       "krylov_tolerance": 1e-12, "sample": f"{steps} steps per run"},
            "cpu_baseline": {"value": value, "unit": "cell-stage/s", "cores": threads, "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": value, "unit": "cell-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


ENSEMBLE = {"workload": "ensemble256_sdirk2_mrsav", "members": 256, "seed": 2026, "dt": 5e-4,
            "scheme": "sdirk2_mrsav", "psi_modes": 8, "stages_per_step": 2}


def run_ensemble(args) -> None:
    """The ensemble workload: FP32-bulk and FP64 ensembles from the same fields."""
    import torch
    import torch.distributed as dist
    import __graft_entry__
    from importlib import import_module
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    E = import_module(pkg.__name__ + ".ensemble")
    w = ENSEMBLE
    members = E.ensemble_members(w["members"], seed=w["seed"])
    mine = [members[i] for i in E.shard_members(members, world, rank)]
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(precision):
        ens = E.Ensemble(mine, w["scheme"], precision=precision)
        ens.seed_fields(modes=w["psi_modes"])
        for _ in range(args.warmup):
            ens.step(w["dt"])
        barrier()
        total = 0.0
        with ClockSampler(local) as clk:
            for _ in range(args.steps):
                flush.fill_(1.0)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ens.step(w["dt"])
                b.record(stream)
                b.synchronize()
                total += a.elapsed_time(b)
        return ens, total, clk.summary()

    e32, ms32, clk = timed("fp32")
    e64, ms64, _ = timed("fp64")
    # kernels per ensemble step: one eager step of a copy of the FP32 ensemble
    eager = E.Ensemble(mine, w["scheme"], precision="fp32", use_graph=False)
    for i in range(len(mine)):
        eager.set_state(i, e32.velocity(i), r=e32.r[i], t=e32.t[i])
    before = eager.launches()
    eager.step(w["dt"])
    launches_per_step = eager.launches() - before
    del eager
    err = max(float(torch.linalg.vector_norm(e32.velocity(i) - e64.velocity(i))
                    / torch.linalg.vector_norm(e64.velocity(i))) for i in range(len(mine)))
    # end to end: host states in, host states out, every step, through the
    # ensemble's pinned host block (one array per member, allocated once):
    # every member's state uploaded by one kernel, stepped, and downloaded by
    # one kernel, each reading or writing the pinned block over the host link
    e32.host_buffers()
    e32.download()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e32.upload()
        e32.step(w["dt"])
        e32.download()
    e2e_sec = time.perf_counter() - t0
    tot = torch.tensor([ms32, ms64, e2e_sec, err], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
    ms32, ms64, e2e_sec, err = (float(v) for v in tot)
    if rank == 0:
        cells = sum(m.cells for m in members) * w["stages_per_step"] * args.steps
        size_bytes = sum(m.grid().size for m in members) * 8
        launches = launches_per_step * args.steps  # of this rank; every rank runs the same kind of shard
        line = {
            "metric": METRIC, "value": cells / (ms32 / 1e3), "unit": "cell-stage/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32 / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "fp32+fp64",
            "data": "synthetic (seeded stream-function curl fields, one seed per member)",
            "config": {"workload": w["workload"], "members": w["members"], "cells": sum(m.cells for m in members),
                       "dt": w["dt"], "scheme": w["scheme"], "psi_modes": w["psi_modes"],
                       "parallelism": f"shards{world}", "l2": "flushed (256 MiB write) before every timed step",
                       "graph": "equal-shape members batched into one plan (16 at most); one CUDA graph per plan "
                                "step, all plans in flight", "plans": len(e32.units)},
            "fp64": {"value": cells / (ms64 / 1e3), "ms_per_step": ms64 / args.steps, "unit": "cell-stage/s"},
            "error_vs_fp64": {"max_rel_l2_velocity": err, "after_steps": args.warmup + args.steps},
            "clocks": clk,
            "e2e": {"value": cells / e2e_sec, "unit": "cell-stage/s", "h2d_bytes_per_step": size_bytes,
                    "d2h_bytes_per_step": size_bytes},
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


ADAPTIVE = {"workload": "adaptive2048x1024_sdirk3_mrsav", "nx": 2048, "ny": 1024, "lx": 2.0, "ly": 1.0,
            "nu": 5e-5, "psi_modes": 64, "seed": 20261205, "t_end": 0.05, "dt0": 1e-4, "rtol": 1e-5,
            "scheme": "sdirk3_mrsav", "stages_per_step": 4}


def run_adaptive(args) -> None:
    """The adaptive run: 2048x1024 on [0,2]x[0,1], nu=5e-5, psi modes <= 64,
    sdirk3_mrsav with SDIRK3(2) PI control (rtol 1e-5), dt0=1e-4 to t=0.05
    through the package's device-resident loop ``run_adaptive`` (every attempt
    one fused step), FP32 bulk and FP64; reports accepted / rejected attempts
    and the FP32 run's error against the FP64 run at t_end."""
    import torch
    import __graft_entry__
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    w = ADAPTIVE
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    x0 = pkg.fields.packed_curl_velocity(w["nx"], w["ny"], w["lx"], w["ly"], w["psi_modes"], w["seed"])
    runs = {}
    with ClockSampler(local) as clk:
        for precision in ("fp32", "fp64"):
            model = pkg.MACNavierStokes(g, w["nu"], precision=precision, use_graph=True)
            scheme = pkg.make_scheme(w["scheme"])
            ctl = pkg.StepControl(rtol=w["rtol"], pi=(0.7, 0.4))  # the reference PIController's defaults
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = pkg.run_adaptive(model, scheme, model.state(0.0, x0, 1.0), w["t_end"], w["dt0"], ctl,
                                   keep_attempts=False)
            torch.cuda.synchronize()
            runs[precision] = (res, time.perf_counter() - t0, model.vector(res.final))
        # the same FP32 run with the attempt loop itself on the device (one
        # graph launch for the whole integration, no host decision per attempt)
        model = pkg.MACNavierStokes(g, w["nu"], precision="fp32", use_graph=True)
        scheme = pkg.make_scheme(w["scheme"])
        ctl = pkg.StepControl(rtol=w["rtol"], pi=(0.7, 0.4))
        pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 1.0), 2 * w["dt0"], w["dt0"], ctl)  # capture
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dres = pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 1.0), w["t_end"], w["dt0"], ctl,
                                       history=1)
        torch.cuda.synchronize()
        dsec = time.perf_counter() - t0
        dx = model.vector(dres.final)
    if rank != 0:
        return
    res32, sec32, x32 = runs["fp32"]
    res64, sec64, x64 = runs["fp64"]
    attempts32, acc32 = res32.attempted_steps, res32.accepted_steps
    attempts64, acc64 = res64.attempted_steps, res64.accepted_steps
    cells = w["nx"] * w["ny"] * w["stages_per_step"]
    err = float(np.linalg.norm(x32 - x64) / np.linalg.norm(x64))
    line = {"metric": METRIC, "value": cells * attempts32 / sec32, "unit": "cell-stage/s", "n_gpus": world,
            "steps": attempts32, "warmup": 0, "ms_per_step": 1e3 * sec32 / attempts32, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
            "data": "synthetic (seeded stream-function curl field, psi modes <= 64)",
            "config": {"workload": w["workload"], **{k: w[k] for k in ("nx", "ny", "lx", "ly", "nu", "t_end", "dt0",
                                                                       "rtol", "scheme")},
                       "controller": "PI control (SDIRK3(2) embedded error), the reference PIController's constants",
                       "note": "wall time of the whole run_adaptive call (host decisions included)"},
            "status": res32.status, "t_end_reached": float(res32.final.t),
            "accepted": acc32, "rejected": attempts32 - acc32,
            "fp64": {"value": cells * attempts64 / sec64, "seconds": sec64, "accepted": acc64,
                     "rejected": attempts64 - acc64, "unit": "cell-stage/s"},
            "error_vs_fp64_at_t_end": {"rel_l2_velocity": err},
            "device_loop": {"value": cells * dres.attempted_steps / dsec, "seconds": dsec, "unit": "cell-stage/s",
                            "status": dres.status, "accepted": dres.accepted_steps,
                            "rejected": dres.attempted_steps - dres.accepted_steps,
                            "rel_l2_vs_host_loop": float(np.linalg.norm(dx - x32) / np.linalg.norm(x32)),
                            "note": "FP32 bulk, run_adaptive_device: every attempt, decision and retry in one "
                                    "graph launch"},
            "clocks": clk.summary(),
            "e2e": {"value": cells * attempts32 / sec32, "unit": "cell-stage/s",
                    "h2d_bytes_per_step": g.size * 8, "d2h_bytes_per_step": g.size * 8}}
    print(json.dumps(line), flush=True)


def network_info(net) -> dict:
    return {"params": net.num_params, "channels": list(net.channels), "activations": "bf16",
            "convolutions": ("3x3 forward on tcgen05 (BF16 operands, FP32 accumulator in TMEM), backward on CUDA cores"
                             if net.tensor_cores else "CUDA cores")}


def stage_rhs_columns(pkg, g, w, seeds, model):
    """Two-column stage-like Stokes right-hand sides [x, dt N(x)] of seeded
    curl fields with the workload's modes (host (size, 2) arrays)."""
    out = []
    for s in seeds:
        x = pkg.fields.packed_curl_velocity(g.nx, g.ny, g.lx, g.ly, w["psi_modes"], s)
        out.append(np.column_stack([x, w["dt"] * model.nonlinear(x).cpu().numpy()]))
    return out


def train_first_direction(pkg, g, w) -> tuple:
    """The learned preconditioner of the headline workload, trained on the GPU
    with the library's own BF16 forward/backward kernels: pairs (pressure
    right-hand side -> error of the spectral first direction) logged by plain
    FP64 Schur CG on the workload's grid and stage shift (mass 1, viscosity
    nu dt / 4, the sdirk3 stage diagonal) for seeded stage-like right-hand
    sides, restricted to the network's grid; then its output gain is set with
    plain PCG as the judge on held-out right-hand sides."""
    import torch
    from importlib import import_module
    L = import_module(pkg.__name__ + ".learned")
    t0 = time.perf_counter()
    helper = pkg.MACNavierStokes(g, w["nu"])
    mass, visc = 1.0, w["nu"] * w["dt"] / 4
    train_cols = stage_rhs_columns(pkg, g, w, range(1000, 1000 + w["train_fields"]), helper)
    rhs = [c[:, k] for c in train_cols for k in range(2)]
    pairs = L.collect_first_direction_pairs(g, rhs, mass, visc, restriction=w["restriction"])
    net = L.UNet(channels=w.get("net_channels", L.DEFAULT_CHANNELS), seed=0)
    losses = L.train(net, pairs, steps=w["train_steps"], batch=8, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    held = stage_rhs_columns(pkg, g, w, range(2000, 2000 + w["judge_fields"]), helper)
    judge = L.calibrate_gain(net, g, held, mass, visc, restriction=w["restriction"],
                             krylov_tolerance=w["krylov_tolerance"])
    info = {"pairs": int(pairs.inputs.shape[0]), "logged_on": f"{g.nx}x{g.ny}",
            "network_grid": f"{g.nx // w['restriction']}x{g.ny // w['restriction']}",
            "shift": {"mass": mass, "viscosity": visc}, "steps": len(losses),
            "loss_first": float(np.mean(losses[:5])), "loss_last": float(np.mean(losses[-5:])),
            "seconds": t_train, "judge": {"held_out_solves": len(held),
                                          "inner_iterations_per_gain": judge["iterations_per_gain"],
                                          "gain": judge["gain"]}}
    return net, info


def timed_steps(pkg, g, w, x0_host, dev, args, precision, ktol, net=None, flush=None, count_launches=False):
    """W warm-up + K timed steps of one form on device-resident state, one CUDA
    graph per step, per-step CUDA events on the launching stream, L2 flushed
    (256 MiB write) before every timed step, outside the events.  Returns the
    model, the state after W + K steps, per-step ms, inner CG iterations per
    step and (optionally) the kernel launches of one eager step."""
    import torch
    from importlib import import_module
    L = import_module(pkg.__name__ + ".learned")
    model = pkg.MACNavierStokes(g, w["nu"], precision=precision, use_graph=True, krylov_tolerance=ktol)
    if net is not None:
        L.attach(model, net)
        L.placement(model, every_iteration=False, restriction=w["restriction"])
    scheme = pkg.make_scheme(w["scheme"])
    stream = torch.cuda.current_stream()
    x = torch.from_numpy(x0_host.copy()).to(dev)
    y = torch.empty_like(x)
    pres = torch.empty((4, g.np), dtype=torch.float64, device=dev)
    t, r = 0.0, 1.0
    for _ in range(args.warmup):
        y, r, _, _, _ = scheme.step_device(model, x, t, r, w["dt"], x1=y, pres=pres, want_embedded=False)
        x, y, t = y, x, t + w["dt"]
    launches = None
    if count_launches:
        eager = pkg.MACNavierStokes(g, w["nu"], precision=precision, use_graph=False, krylov_tolerance=ktol)
        if net is not None:
            L.attach(eager, net)
            L.placement(eager, every_iteration=False, restriction=w["restriction"])
        before = eager.plan.launches
        scheme.step_device(eager, x, t, r, w["dt"], pres=torch.empty_like(pres), want_embedded=False)
        launches = eager.plan.launches - before
        del eager
    torch.cuda.synchronize()
    before = L.cg_counters(model, 2) if precision == "fp32" else None
    events = []
    with quiet_host():
        for _ in range(args.steps):
            if flush is not None:
                flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            y, r, _, _, _ = scheme.step_device(model, x, t, r, w["dt"], x1=y, pres=pres, want_embedded=False)
            b.record(stream)
            events.append((a, b))
            x, y, t = y, x, t + w["dt"]
        torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in events]
    iters = None
    if before is not None:
        after = L.cg_counters(model, 2)
        iters = {k: (sum(after[k]) - sum(before[k])) / args.steps for k in after}
    return {"model": model, "x": x, "r": r, "t": t, "ms": ms, "iterations": iters, "launches": launches}


def column_roofline(pkg, model, pass_id, reps, hbm, pk_exists, traffic_file):
    """The dominant kernel (a transform column pass over both velocity
    blocks, two right-hand sides) timed alone from a captured graph of
    ``reps`` launches, against the measured HBM bandwidth."""
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    stokes = import_module(pkg.__name__ + ".stokes")
    ms_k, bytes_k = C.c_double(), C.c_double()
    model.plan.check(lib.load().macsav_time_pass(model.plan.handle, pass_id, reps, C.byref(ms_k), C.byref(bytes_k),
                                                 stokes.stream_handle()))
    achieved = bytes_k.value / (ms_k.value * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / traffic_file
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("traffic_bytes_per_launch")
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "peak_source": "measured" if pk_exists else "fallback", "traffic": traffic,
            "bytes_per_launch": bytes_k.value, "ms_per_launch": ms_k.value}


def fp64_roofline(pkg, g, model64, dev, hbm):
    """The FP64 path's dominant kernel (the FP64 velocity column pass) against
    the FP64 rate (measured here: float64 matmul 4096^3, best of 4; the FP64
    peak is not in the measured peaks file) and against HBM."""
    import torch
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    stokes = import_module(pkg.__name__ + ".stokes")
    ms_k64, bytes_k64 = C.c_double(), C.c_double()
    model64.plan.check(lib.load().macsav_time_pass(model64.plan.handle, 3, 20, C.byref(ms_k64), C.byref(bytes_k64),
                                                   stokes.stream_handle()))

    def column_flops(block_cols: int, m: int) -> float:
        # forward and inverse transform of every column, 2.5 m log2(m) each
        return block_cols * 2 * 2.5 * m * np.log2(m)
    lu, lv = int(2 ** np.ceil(np.log2(g.ny))), int(2 ** np.ceil(np.log2(2 * g.ny)))  # DST-II, DST-I lengths
    flops64 = 2 * (column_flops(g.nx - 1, lu) + column_flops(g.nx, lv))  # two right-hand sides
    a_m = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    best = float("inf")
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a_m, a_m)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a_m
    fp64_peak = 2 * 4096 ** 3 / (best * 1e-3) / 1e12
    fp64_achieved = flops64 / (ms_k64.value * 1e-3) / 1e12
    gbs = bytes_k64.value / (ms_k64.value * 1e-3) / 1e9
    return {"kernel": "k_column_p2<double> (velocity blocks, 2 RHS)", "bound": "fp64",
            "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": fp64_achieved / fp64_peak,
            "peak_source": "measured here: float64 matmul 4096^3 (torch), best of 4",
            "flops_per_launch": flops64, "flop_convention": "2.5 m log2(m) per line and direction",
            "ms_per_launch": ms_k64.value, "bytes": {"achieved": gbs, "unit": "GB/s", "frac_of_hbm": gbs / hbm}}


@contextlib.contextmanager
def quiet_host():
    """A timed region without Python garbage collection: collected once
    before (with the device idle), none during, so no collector pause or
    allocator free lands between a step's launch and its events."""
    import torch
    gc.collect()
    torch.cuda.synchronize()
    gc.disable()
    try:
        yield
    finally:
        gc.enable()


def e2e_steps(pkg, model, w, x0_host, args, pageable: bool) -> float:
    """Seconds for K steps through the public API, ``scheme.step(model,
    state, dt)``, with host states: every step its velocity goes host ->
    device and the new state device -> host.  pinned: each step gets the
    previous step's host face arrays (the library's pinned, device-mapped
    arrays); pageable: fresh NumPy copies of them (the staging-copy path a
    caller's own arrays take)."""
    import torch
    g = model.grid
    scheme = pkg.make_scheme(w["scheme"])
    st = pkg.State(0.0, *g.unpack(x0_host), 1.0)

    def fresh(s):
        if pageable:
            return pkg.State(s.t, np.array(s.u), np.array(s.v), s.r)
        return pkg.State(s.t, s.u, s.v, s.r)  # host arrays only, no cached device vector
    for _ in range(args.warmup):
        st = scheme.step(model, fresh(st), w["dt"]).state
    torch.cuda.synchronize()
    with quiet_host():
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st = scheme.step(model, fresh(st), w["dt"]).state
        torch.cuda.synchronize()
        return time.perf_counter() - t0


HEADLINE = {"workload": "learned1024_sdirk3_mrsav", "nx": 1024, "ny": 1024, "lx": 1.0, "ly": 1.0, "nu": 1e-4,
            "dt": 1e-4, "psi_modes": 32, "seed": 20261204, "scheme": "sdirk3_mrsav", "stages_per_step": 4,
            "krylov_tolerance": 1e-10, "reference_krylov_tolerance": 1e-12, "restriction": 4,
            "net_channels": (16, 16, 16, 16), "train_fields": 32, "train_steps": 400, "judge_fields": 3}


def oracle_step(w, x0, threads: int):
    """One step of the workload by the CPU oracle (the reference's path
    restated in NumPy/SciPy) from x0; returns (seconds, new velocity)."""
    import oracle
    g = oracle.Grid(w["nx"], w["ny"], w["lx"], w["ly"])
    model = oracle.OracleModel(g, w["nu"], backend=oracle.TensorStokesOracle(
        g, 1e-9, w.get("reference_krylov_tolerance", 1e-12), workers=threads))
    scheme = oracle.make_scheme(w["scheme"])
    state = model.state(0.0, x0, 1.0)
    t0 = time.perf_counter()
    state = scheme.step(model, state, w["dt"]).state
    return time.perf_counter() - t0, model.vector(state)


def run_headline(args) -> None:
    """The headline workload: 1024^2 unit-square cavity, nu=1e-4,
    sdirk3_mrsav, dt=1e-4, psi modes k,l <= 32.  ``value`` is FP32 bulk with
    the learned preconditioner (flexible CG, Krylov tolerance 1e-10); beside
    it the plain FP64 path at 1e-12 (the reference's own setting, the only one
    at which its gates hold here), plain FP32 bulk at 1e-10, their errors
    against the FP64 run after the same steps and, for the first step, against
    the CPU oracle itself."""
    import torch
    import torch.distributed as dist
    import __graft_entry__
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    w = dict(HEADLINE)
    if args.restriction:
        w["restriction"] = args.restriction
    if args.net_channels:
        w["net_channels"] = tuple(int(c) for c in args.net_channels.split(","))
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    dev = torch.device("cuda", local)
    x0_host = pkg.fields.packed_curl_velocity(w["nx"], w["ny"], w["lx"], w["ly"], w["psi_modes"], w["seed"])
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    net, training = train_first_direction(pkg, g, w)
    barrier()
    with ClockSampler(local) as clk:
        learned = timed_steps(pkg, g, w, x0_host, dev, args, "fp32", w["krylov_tolerance"], net, flush, True)
    barrier()
    plain = timed_steps(pkg, g, w, x0_host, dev, args, "fp32", w["krylov_tolerance"], None, flush)
    barrier()
    fp64 = timed_steps(pkg, g, w, x0_host, dev, args, "fp64", w["reference_krylov_tolerance"], None, flush)
    barrier()
    tot = torch.tensor([sum(learned["ms"]), sum(plain["ms"]), sum(fp64["ms"])], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
    ms_l, ms_p, ms_64 = (float(v) for v in tot)
    cells = w["nx"] * w["ny"] * w["stages_per_step"] * args.steps * world

    def err(x):
        return float(torch.linalg.vector_norm(x - fp64["x"]) / torch.linalg.vector_norm(fp64["x"]))

    # end to end through scheme.step with host states (learned form)
    e2e_pinned = e2e_steps(pkg, learned["model"], w, x0_host, args, pageable=False)
    e2e_pageable = e2e_steps(pkg, learned["model"], w, x0_host, args, pageable=True)
    et = torch.tensor([e2e_pinned, e2e_pageable], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(et, op=dist.ReduceOp.MAX)
    face_bytes = (g.ny * (g.nx + 1) + (g.ny + 1) * g.nx) * 8
    rec_bytes = C.sizeof(lib.StageRecord)

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    roof = column_roofline(pkg, plain["model"], 0, 50, hbm, pk.exists(), "column_pass_traffic_1024.json")
    roof["kernel"] = "k_column_p2<float,1024,128> (u) + k_column_p2<float,2048,128> (v, split) (velocity blocks, 2 RHS)"
    roof64 = fp64_roofline(pkg, g, fp64["model"], dev, hbm)

    # the first step of each GPU form against the CPU oracle's first step
    first = {}
    for name, prec, ktol, with_net in (("fp64", "fp64", w["reference_krylov_tolerance"], False),
                                       ("fp32_learned", "fp32", w["krylov_tolerance"], True)):
        class _One:
            steps, warmup = 1, 0
        first[name] = timed_steps(pkg, g, w, x0_host, dev, _One, prec, ktol, net if with_net else None)["x"]
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    threads = 1
    oracle_sec, oracle_x = (None, None) if args.no_cpu_baseline else oracle_step(w, x0_host, threads)
    vs_oracle = None
    if oracle_x is not None:
        ox = torch.from_numpy(oracle_x).to(dev)
        vs_oracle = {k: float(torch.linalg.vector_norm(v - ox) / torch.linalg.vector_norm(ox))
                     for k, v in first.items()}
    cav = quick_cavity512(pkg, dev, args, flush)
    try:
        ens = quick_ensemble(pkg, flush)
    except Exception as exc:  # the headline stands on its own
        ens = {"error": f"{type(exc).__name__}: {exc}"}
    autotune = transform_choices(pkg)
    line = {
        "metric": METRIC, "value": cells / (ms_l / 1e3), "unit": "cell-stage/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_l / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+bf16 network+fp64",
        "data": "synthetic (seeded stream-function curl field, psi modes <= 32)",
        "config": {"workload": w["workload"], **{k: w[k] for k in ("nx", "ny", "nu", "dt", "scheme", "psi_modes",
                                                                   "krylov_tolerance", "reference_krylov_tolerance")},
                   "parallelism": f"replicas{world}",
                   "form": "fp32 transforms/stencils/Krylov + fp64-accurate reductions + double-float defect "
                           "correction; flexible CG with the learned first direction",
                   "learned_placement": f"first search direction of each Stokes solve, network on the "
                                        f"{w['restriction']}x{w['restriction']}-restricted residual",
                   "l2": "flushed (256 MiB write) before every timed step", "graph": "one CUDA graph per step"},
        "speedup_vs_fp64": ms_64 / ms_l,
        "error_vs_fp64": {"rel_l2_velocity": err(learned["x"]), "after_steps": args.warmup + args.steps},
        "error_vs_oracle_first_step": vs_oracle,
        "cg_iterations_per_step": learned["iterations"],
        "plain_fp32": {"value": cells / (ms_p / 1e3), "ms_per_step": ms_p / args.steps,
                       "error_vs_fp64": err(plain["x"]), "cg_iterations_per_step": plain["iterations"]},
        "fp64": {"value": cells / (ms_64 / 1e3), "ms_per_step": ms_64 / args.steps, "unit": "cell-stage/s",
                 "krylov_tolerance": w["reference_krylov_tolerance"]},
        "learned_vs_plain_fp32": ms_p / ms_l,
        "step_ms": {k: {"min": min(v["ms"]), "median": statistics.median(v["ms"]), "max": max(v["ms"])}
                    for k, v in (("learned", learned), ("plain_fp32", plain), ("fp64", fp64))},
        "network": network_info(net), "training": training,
        "clocks": clk.summary(),
        "e2e": {"value": cells / float(et[0]), "unit": "cell-stage/s", "h2d_bytes_per_step": face_bytes,
                "d2h_bytes_per_step": face_bytes + w["stages_per_step"] * rec_bytes,
                "host_memory": "the library's pinned, device-mapped state arrays fed back each step",
                "pageable": {"value": cells / float(et[1]),
                             "host_memory": "fresh pageable NumPy copies of the face arrays each step"}},
        "gpu_launches": int(learned["launches"] * args.steps),
        "roofline": roof,
        "roofline_fp64": roof64,
        "cavity512_sdirk3_mrsav": cav,
        "ensemble256_sdirk2_mrsav": ens,
        "transform_autotune": autotune,
        "launch_shapes": {"learned": learned["model"].plan.launch_shapes, "plain_fp32": plain["model"].plan.launch_shapes},
    }
    if oracle_sec is not None:
        line["cpu_baseline"] = {"value": w["nx"] * w["ny"] * w["stages_per_step"] / oracle_sec,
                                "unit": "cell-stage/s", "cores": threads, "kind": "port",
                                "sample": f"one step of the {w['workload']} workload (NumPy/SciPy oracle, "
                                          f"{threads} thread, Krylov 1e-12)"}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def transform_choices(pkg) -> dict:
    """The autotuner's choice between the shared-memory FFT and the tcgen05
    transform-matrix product (6 BF16 products) for FP32 forward transforms of
    2n rows of length n, with both times (us)."""
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    plan = stokes.Plan(pkg.MACGrid(8, 8))
    out = {}
    for kind, name in ((0, "dct2"), (1, "dst2"), (2, "dst1")):
        for n in (64, 128, 256, 511, 512):
            m, tf, tt = C.c_int(), C.c_double(), C.c_double()
            plan.check(plan.lib.macsav_transform32_autotune(plan.handle, kind, 0, 2 * n, n, C.byref(m), C.byref(tf),
                                                            C.byref(tt), stokes.stream_handle()))
            out[f"{name}_{n}"] = {"choice": "tensor" if m.value == 2 else "fft", "fft_us": round(1e3 * tf.value, 1),
                                  "tensor_us": round(1e3 * tt.value, 1)}
    return out


def quick_cavity512(pkg, dev, args, flush) -> dict:
    """The 512^2 precision case (nu=1e-3, dt=2.5e-4, modes <= 16, sdirk3_mrsav):
    FP32 bulk (plain preconditioner) and FP64 on the same K steps."""
    w = dict(WORKLOAD, restriction=1)
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    x0 = initial_state(pkg)
    a = timed_steps(pkg, g, w, x0, dev, args, "fp32", 1e-12, None, flush)
    b = timed_steps(pkg, g, w, x0, dev, args, "fp64", 1e-12, None, flush)
    import torch
    cells = w["nx"] * w["ny"] * w["stages_per_step"] * args.steps
    return {"value": cells / (sum(a["ms"]) / 1e3), "ms_per_step": sum(a["ms"]) / args.steps,
            "fp64": {"value": cells / (sum(b["ms"]) / 1e3), "ms_per_step": sum(b["ms"]) / args.steps},
            "error_vs_fp64": float(torch.linalg.vector_norm(a["x"] - b["x"]) / torch.linalg.vector_norm(b["x"])),
            "unit": "cell-stage/s"}


def quick_ensemble(pkg, flush, warmup: int = 3, steps: int = 5) -> dict:
    """The mixed-size ensemble (256 cavities, sdirk2_mrsav, FP32 bulk) on a
    few steps: throughput over all members and kernels per ensemble step."""
    import torch
    from importlib import import_module
    E = import_module(pkg.__name__ + ".ensemble")
    w = ENSEMBLE
    members = E.ensemble_members(w["members"], seed=w["seed"])
    ens = E.Ensemble(members, w["scheme"], precision="fp32")
    ens.seed_fields(modes=w["psi_modes"])
    for _ in range(warmup):
        ens.step(w["dt"])
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    total = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ens.step(w["dt"])
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b)
    eager = E.Ensemble(members, w["scheme"], precision="fp32", use_graph=False)
    eager.seed_fields(modes=w["psi_modes"])
    before = eager.launches()
    eager.step(w["dt"])
    launches = eager.launches() - before
    cells = sum(m.cells for m in members) * w["stages_per_step"] * steps
    return {"value": cells / (total / 1e3), "ms_per_step": total / steps, "unit": "cell-stage/s",
            "members": len(members), "plans": len(ens.units), "kernels_per_step": launches,
            "precision": "fp32 bulk", "steps": steps}


def profile_unet() -> None:
    """Three forward passes of the learned preconditioner's U-Net on a batch
    of 4 256x256 residual fields (the tcgen05 convolution capture of
    profiles/ comes from this)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    net = pkg.UNet(seed=0, output_gain=1.0)
    x = torch.randn(4, 256, 256, generator=torch.Generator().manual_seed(0)).cuda()
    for _ in range(3):
        y = net.forward(x)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "unet", "out_norm": float(y.norm())}))


def profile_steps(precision: str, workload: str) -> None:
    """Two eager steps of a workload (the launch lists and kernel captures of
    profiles/ come from this).  precision "learned": the headline's FP32 form
    with an (untrained) network in its first-direction placement, so that no
    training kernels precede the steps."""
    import torch
    import __graft_entry__
    from importlib import import_module
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    w = HEADLINE if workload == "learned1024" else WORKLOAD
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    ktol = w.get("krylov_tolerance", 1e-12) if precision != "fp64" else 1e-12
    model = pkg.MACNavierStokes(g, w["nu"], precision="fp64" if precision == "fp64" else "fp32", use_graph=False,
                                krylov_tolerance=ktol)
    if precision == "learned":
        L = import_module(pkg.__name__ + ".learned")
        net = L.UNet(channels=w.get("net_channels", L.DEFAULT_CHANNELS), seed=0)
        L.attach(model, net)
        L.placement(model, every_iteration=False, restriction=w["restriction"])
    scheme = pkg.make_scheme(w["scheme"])
    x = torch.from_numpy(pkg.fields.packed_curl_velocity(w["nx"], w["ny"], w["lx"], w["ly"], w["psi_modes"],
                                                         w["seed"])).to("cuda")
    t, r = 0.0, 1.0
    for _ in range(2):
        x, r, recs, _, _ = scheme.step_device(model, x, t, r, w["dt"], want_embedded=False)
        t += w["dt"]
    torch.cuda.synchronize()
    print(json.dumps({"profile": precision, "workload": w["workload"], "launches": model.plan.launches,
                      "iterations": [list(rc.iterations[:2]) for rc in recs]}))


def profile_transform32() -> None:
    """The autotuner's measurements for the FP32 row transforms at the
    solver's lengths (n = 64..512 and 1023/1024, rows = 2n: two right-hand
    sides of a square block)."""
    import torch
    import __graft_entry__
    from importlib import import_module
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    stokes = import_module(pkg.__name__ + ".stokes")
    plan = stokes.Plan(pkg.MACGrid(8, 8))
    table = []
    for kind, name in ((0, "dct2"), (1, "dst2"), (2, "dst1")):
        for n in (64, 127, 128, 255, 256, 511, 512, 1023, 1024):
            for inverse in (0, 1):
                m, tf, tt = C.c_int(), C.c_double(), C.c_double()
                plan.check(plan.lib.macsav_transform32_autotune(plan.handle, kind, inverse, 2 * n, n, C.byref(m),
                                                                C.byref(tf), C.byref(tt), stokes.stream_handle()))
                table.append({"kind": name, "n": n, "rows": 2 * n, "inverse": inverse, "fft_us": 1e3 * tf.value,
                              "tc6_us": 1e3 * tt.value if tt.value > 0 else None,
                              "chosen": "tc6" if m.value == 2 else "fft"})
    print(json.dumps({"profile": "transform32", "autotune": table}))


def profile_tgemm() -> None:
    """Three launches of the tensor-core row transform (DCT-II, 6 products)
    at n = 512 on 1024 rows, after one warm-up (for a kernel capture)."""
    import torch
    import __graft_entry__
    from importlib import import_module
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    stokes = import_module(pkg.__name__ + ".stokes")
    plan = stokes.Plan(pkg.MACGrid(8, 8))
    x = torch.randn(1024, 512, device="cuda", dtype=torch.float32)
    y = torch.empty_like(x)
    for _ in range(4):
        plan.check(plan.lib.macsav_transform32(plan.handle, 0, 0, 1024, 512, 2, stokes.dptr(x), stokes.dptr(y),
                                               stokes.stream_handle()))
    torch.cuda.synchronize()
    print(json.dumps({"profile": "tgemm", "n": 512, "rows": 1024}))


def profile_pass(workload: str, pass_id: int, reps: int = 3) -> None:
    """``reps`` launches of one transform pass (macsav_time_pass: 0 the FP32
    velocity column pass, 1 and 2 the FP32 velocity row forward and inverse
    passes, 3 the FP64 column pass, 4-6 the FP32 pressure column, forward
    and inverse row passes; pass // 10 forces a launch shape) on the
    workload's grid, after one warm-up launch, for a capture of that kernel
    and its average time per launch (graph replay)."""
    import torch
    import __graft_entry__
    from importlib import import_module
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    lib = import_module(pkg.__name__ + "._lib")
    stokes = import_module(pkg.__name__ + ".stokes")
    w = HEADLINE if workload == "learned1024" else WORKLOAD
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    model = pkg.MACNavierStokes(g, w["nu"], precision="fp64" if pass_id == 3 else "fp32")
    ms_k, bytes_k = C.c_double(), C.c_double()
    model.plan.check(lib.load().macsav_time_pass(model.plan.handle, pass_id, reps, C.byref(ms_k), C.byref(bytes_k),
                                                 stokes.stream_handle()))
    torch.cuda.synchronize()
    print(json.dumps({"profile": "pass", "pass": pass_id, "workload": w["workload"], "bytes": bytes_k.value,
                      "ms_per_launch": ms_k.value}))


CHANNEL = {"workload": "channel512_fft_stokes", "nx": 512, "ny": 512, "lx": 6.283185307179586, "ly": 1.0,
           "mass": 1.0, "nu": 1e-3, "dt": 2.5e-4, "columns": 2, "seed": 7, "cpu_nx": 128, "cpu_ny": 128}


def run_channel(args) -> None:
    """The channel MAC FFT Stokes backend (periodic x, no-slip y): repeated
    two-column solves at 512 x 512 with the sdirk3 stage shift (mass 1,
    viscosity nu dt / 4, nu = 1e-3, dt = 2.5e-4) on device-resident right-hand
    sides, after the first solve has factored the per-mode banded systems.
    Value = cells x right-hand sides solved per second; each solve's wall time
    includes the readback of its residual and divergence.  CPU baseline: the
    oracle's FFT solve (dense per-mode solves) on a 128 x 128 sample."""
    import torch
    import __graft_entry__
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    w = CHANNEL
    grid = pkg.ChannelGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    solver = pkg.FFTStokes(grid)
    rng = np.random.default_rng(w["seed"])
    f = torch.from_numpy(rng.normal(size=(w["columns"], grid.size))).to("cuda")
    visc = w["nu"] * w["dt"] / 4
    for _ in range(args.warmup):
        solver.solve_device(f, w["mass"], visc)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            vel, pres, res, div = solver.solve_device(f, w["mass"], visc)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    # the solve's own gate (FFTStokes: residual and divergence <= tolerance):
    # a timing of a wrong solve is no timing
    umax = float(vel.abs().max())
    if not (res <= 1e-9 and div <= 1e-9 * (1.0 + umax)):
        raise RuntimeError(f"channel solve failed its gate: residual {res:.3e}, divergence {div:.3e}")
    if rank != 0:
        return
    sec = statistics.median(times)
    units = grid.nx * grid.ny * w["columns"]
    line = {"metric": "channel Stokes solve: cells x right-hand sides / s", "value": units / sec,
            "unit": "cell-rhs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sec, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded normal right-hand sides)",
            "config": {"workload": w["workload"], **{k: w[k] for k in ("nx", "ny", "lx", "ly", "mass", "nu", "dt",
                                                                       "columns")},
                       "note": "median wall time of one solve call; factorisation cached after the warm-up"},
            "residual": res, "divergence": div, "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        import oracle.channel_oracle as CO
        cg_ = CO.ChannelGridOracle(w["cpu_nx"], w["cpu_ny"], w["lx"], w["ly"])
        rhs = np.random.default_rng(w["seed"]).normal(size=(cg_.size, w["columns"]))
        t0 = time.perf_counter()
        CO.fft_solve(cg_, rhs, w["mass"], visc)
        csec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": cg_.nx * cg_.ny * w["columns"] / csec, "unit": "cell-rhs/s", "cores": 1,
                                "kind": "port", "sample": f"one two-column solve on {cg_.nx} x {cg_.ny} "
                                                          "(NumPy oracle, dense per-mode solves)"}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--net-channels", default=None,
                    help="headline: the U-Net's channels per level, four comma-separated values "
                         "(16, 32 or 64 each; default the workload's own)")
    ap.add_argument("--restriction", type=int, choices=[2, 4, 8], default=None,
                    help="headline: the learned preconditioner's restriction factor (the network sees "
                         "(nx/f) x (ny/f) cell means); default the workload's own")
    ap.add_argument("--workload", choices=["learned1024", "cavity512", "ensemble256", "adaptive2048", "channel512"],
                    default="learned1024")
    ap.add_argument("--profile", choices=["fp32", "fp64", "learned", "unet", "pass0", "pass1", "pass2", "pass3",
                                          "pass", "transform32", "tgemm"],
                    default=None,
                    help="run two eager steps of the workload (or launches of one transform pass) and exit, "
                         "for ncu captures")
    ap.add_argument("--pass-id", type=int, default=0,
                    help="--profile pass: macsav_time_pass's pass (pass %% 10) and launch shape (pass // 10)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile == "unet":
        profile_unet()
        return
    if args.profile == "transform32":
        profile_transform32()
        return
    if args.profile == "tgemm":
        profile_tgemm()
        return
    if args.profile in ("pass0", "pass1", "pass2", "pass3", "pass"):
        pass_id = args.pass_id if args.profile == "pass" else int(args.profile[-1])
        profile_pass(args.workload, pass_id, args.steps if args.steps > 0 else 3)
        return
    if args.profile:
        profile_steps(args.profile, args.workload)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "ensemble256":
        run_ensemble(args)
        return
    if args.workload == "adaptive2048":
        run_adaptive(args)
        return
    if args.workload == "learned1024":
        run_headline(args)
        return
    if args.workload == "channel512":
        run_channel(args)
        return

    import torch
    import torch.distributed as dist
    import __graft_entry__
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    __graft_entry__.build()
    pkg = __graft_entry__.load_package()
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    stokes = import_module(pkg.__name__ + ".stokes")
    w = WORKLOAD
    g = pkg.MACGrid(w["nx"], w["ny"], w["lx"], w["ly"])
    x0_host = initial_state(pkg)
    dev = torch.device("cuda", local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed_device_run(precision: str):
        """W warm-up + K timed steps on device-resident state; per-step events,
        L2 flushed (256 MiB write) between timed steps outside the events."""
        model = pkg.MACNavierStokes(g, w["nu"], precision=precision, use_graph=True)
        scheme = pkg.make_scheme(w["scheme"])
        x = torch.from_numpy(x0_host.copy()).to(dev)
        y = torch.empty_like(x)
        pres = torch.empty((4, g.np), dtype=torch.float64, device=dev)
        t, r = 0.0, 0.0
        iters = []
        for _ in range(args.warmup):
            y, r, recs, _, _ = scheme.step_device(model, x, t, r, w["dt"], x1=y, pres=pres, want_embedded=False)
            x, y, t = y, x, t + w["dt"]
        # kernels per step: one eager step on a copy (same CG iteration counts)
        eager = pkg.MACNavierStokes(g, w["nu"], precision=precision, use_graph=False)
        before = eager.plan.launches
        scheme.step_device(eager, x, t, r, w["dt"], pres=pres, want_embedded=False)
        launches_per_step = eager.plan.launches - before
        del eager
        barrier()
        times = []
        with ClockSampler(local) as clk:
            for _ in range(args.steps):
                flush.fill_(1.0)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                y, r, recs, _, _ = scheme.step_device(model, x, t, r, w["dt"], x1=y, pres=pres,
                                                      want_embedded=False)
                b.record(stream)
                x, y, t = y, x, t + w["dt"]
                iters.append([tuple(rc.iterations[:2]) for rc in recs])
                times.append((a, b))
            torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in times]
        return model, scheme, x, r, sum(ms), ms, iters, launches_per_step, clk.summary()

    barrier()
    m32, s32, x32, r32, ms32, per32, it32, l32, clk32 = timed_device_run("fp32")
    barrier()
    m64, s64, x64, r64, ms64, per64, it64, l64, clk64 = timed_device_run("fp64")
    barrier()
    # both trajectories start from the same field and take the same steps
    diff = float(torch.linalg.vector_norm(x32 - x64) / torch.linalg.vector_norm(x64))

    # the workload's full run (200 steps) in both forms, the FP32-bulk error
    # against FP64 every 20 steps (outside the timed region)
    def trajectory_errors(steps: int = 200, every: int = 20) -> dict:
        """Relative L2 errors of the FP32-bulk run against the FP64 run every
        `every` steps: packed velocity, u faces, v faces and the step's
        pressure (its last stage's)."""
        ms = {p: pkg.MACNavierStokes(g, w["nu"], precision=p, use_graph=True) for p in ("fp32", "fp64")}
        sch = pkg.make_scheme(w["scheme"])
        xs = {p: torch.from_numpy(x0_host.copy()).to(dev) for p in ms}
        ys = {p: torch.empty_like(xs[p]) for p in ms}
        ps = {p: torch.empty((sch.info.n_stages, g.np), dtype=torch.float64, device=dev) for p in ms}
        rs = {p: 0.0 for p in ms}
        out = {"velocity": [], "u": [], "v": [], "p": []}

        def rel(a, b):
            return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
        for k in range(1, steps + 1):
            for p in ms:
                ys[p], rs[p], _, _, _ = sch.step_device(ms[p], xs[p], (k - 1) * w["dt"], rs[p], w["dt"], x1=ys[p],
                                                        pres=ps[p], want_embedded=False)
                xs[p], ys[p] = ys[p], xs[p]
            if k % every == 0:
                a, b = xs["fp32"], xs["fp64"]
                out["velocity"].append(rel(a, b))
                out["u"].append(rel(a[:g.nu], b[:g.nu]))
                out["v"].append(rel(a[g.nu:], b[g.nu:]))
                out["p"].append(rel(ps["fp32"][-1], ps["fp64"][-1]))
        return out

    traj = trajectory_errors() if rank == 0 else {}

    # max over ranks of the timed totals
    tot = torch.tensor([ms32, ms64], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
    ms32, ms64 = float(tot[0]), float(tot[1])
    cells = w["nx"] * w["ny"] * w["stages_per_step"] * args.steps * world
    value = cells / (ms32 / 1e3)
    value64 = cells / (ms64 / 1e3)

    # end to end through the public API with host state (H2D + D2H each step):
    # each step gets a State holding only the previous step's host arrays (no
    # cached device vector), so its velocity crosses to the device and the new
    # state comes back to host memory
    scheme = pkg.make_scheme(w["scheme"])
    st_host = pkg.State(0.0, *g.unpack(x0_host), 0.0)
    for _ in range(args.warmup):
        st_host = scheme.step(m32, pkg.State(st_host.t, st_host.u, st_host.v, st_host.r), w["dt"]).state
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fresh = pkg.State(st_host.t, st_host.u, st_host.v, st_host.r)  # host arrays only
        st_host = scheme.step(m32, fresh, w["dt"]).state
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    et = torch.tensor([e2e_sec], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(et, op=dist.ReduceOp.MAX)
    e2e_value = cells / float(et[0])
    # bytes copied per e2e step: the face arrays u (ny, nx+1) and v (ny+1, nx)
    # each way, plus the stage records read back with the step
    face_bytes = (g.ny * (g.nx + 1) + (g.ny + 1) * g.nx) * 8
    rec_bytes = C.sizeof(lib.StageRecord)

    # dominant kernel (FP32 column pass of the velocity blocks) timed alone
    ms_k, bytes_k = C.c_double(), C.c_double()
    m32.plan.check(lib.load().macsav_time_pass(m32.plan.handle, 0, 50, C.byref(ms_k), C.byref(bytes_k),
                                               stokes.stream_handle()))
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bytes_k.value / (ms_k.value * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "column_pass_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("traffic_bytes_per_launch")


    # FP64 path: its dominant kernel (the FP64 velocity column pass) against
    # the FP64 rate and against HBM.  The FP64 peak is not in the measured
    # peaks file, so it is measured here: a float64 matmul 4096^3, best of 3.
    ms_k64, bytes_k64 = C.c_double(), C.c_double()
    m64.plan.check(lib.load().macsav_time_pass(m64.plan.handle, 3, 20, C.byref(ms_k64), C.byref(bytes_k64),
                                               stokes.stream_handle()))

    def column_flops(block_cols: int, m: int) -> float:
        # forward and inverse transform of every column, 2.5 m log2(m) each
        return block_cols * 2 * 2.5 * m * np.log2(m)
    lu, lv = int(2 ** np.ceil(np.log2(g.ny))), int(2 ** np.ceil(np.log2(2 * g.ny)))  # DST-II, DST-I lengths
    flops64 = 2 * (column_flops(g.nx - 1, lu) + column_flops(g.nx, lv))  # two right-hand sides
    a_m = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    best = float("inf")
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a_m, a_m)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a_m
    fp64_peak = 2 * 4096 ** 3 / (best * 1e-3) / 1e12
    fp64_achieved = flops64 / (ms_k64.value * 1e-3) / 1e12
    roofline64 = {"kernel": "k_column_p2<double> (velocity blocks, 2 RHS)", "bound": "fp64",
                  "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": fp64_achieved / fp64_peak,
                  "peak_source": "measured here: float64 matmul 4096^3 (torch), best of 4",
                  "flops_per_launch": flops64, "flop_convention": "2.5 m log2(m) per line and direction",
                  "ms_per_launch": ms_k64.value,
                  "bytes": {"achieved": bytes_k64.value / (ms_k64.value * 1e-3) / 1e9, "unit": "GB/s",
                            "frac_of_hbm": bytes_k64.value / (ms_k64.value * 1e-3) / 1e9
                            / float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", 6800.0))
                            if (ROOT / "MEASURED_PEAKS.json").exists() else None}}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    base = None if args.no_cpu_baseline else cpu_baseline(WORKLOAD, steps=2, threads=1)
    mean_iters = float(np.mean([[a, b] for stage in it32 for (a, b) in stage]))
    line = {
        "metric": METRIC, "value": value, "unit": "cell-stage/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic (seeded stream-function curl field)",
        "config": {"workload": w["workload"], "nx": w["nx"], "ny": w["ny"], "nu": w["nu"], "dt": w["dt"],
                   "scheme": w["scheme"], "psi_modes": w["psi_modes"], "parallelism": f"replicas{world}",
                   "form": "fp32 transforms/stencils/Krylov + fp64 reductions + fp64 defect correction",
                   "preconditioner": "spectral m(DD^T)^+ + kI (the learned variant is reported under learned)",
                   "l2": "flushed (256 MiB write) before every timed step", "graph": "one CUDA graph per step"},
        "fp64": {"value": value64, "ms_per_step": ms64 / args.steps, "unit": "cell-stage/s"},
        "speedup_vs_fp64": value / value64,
        "error_vs_fp64": {"rel_l2_velocity": diff, "after_steps": args.warmup + args.steps,
                          "trajectory_200_steps_every_20": traj},
        "cg_iterations_mean": mean_iters,
        "clocks": clk32,
        "e2e": {"value": e2e_value, "unit": "cell-stage/s", "h2d_bytes_per_step": face_bytes,
                "d2h_bytes_per_step": face_bytes + w["stages_per_step"] * rec_bytes},
        "gpu_launches": int(l32 * args.steps),
        "roofline": {"kernel": "k_column_p2<float> (velocity blocks, 2 RHS)", "bound": "hbm",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": "measured" if pk.exists() else "fallback",
                     "traffic": traffic, "bytes_per_launch": bytes_k.value, "ms_per_launch": ms_k.value},
        "roofline_fp64": roofline64,
    }
    if base is not None:
        line["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
