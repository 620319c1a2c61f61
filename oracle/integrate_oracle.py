"""Restatement of the reference's fixed-step driver -- TEST INFRASTRUCTURE ONLY.

``integrate`` as in the reference's ``solver/integrate.py:47-100`` with
``solver/schedule.py:7-29``: finiteness checks on the state, per-step
diagnostics, snapshots at the nearest nodes, the failed prefix kept on an
exception, observer time excluded from ``seconds``.  The tests drive the GPU
model and the fused GPU schemes with it, as a user drives them with the
reference's own driver.  The product package never imports it.
"""
from __future__ import annotations

from collections.abc import Callable
from dataclasses import dataclass, field
from time import perf_counter, process_time

import numpy as np

from .mac_oracle import stage_diagnostics


@dataclass
class History:
    state: object
    accepted_steps: int = 0


@dataclass
class Result:
    """``solver/integrate.py:12-25``."""
    final: object
    times: list
    diagnostics: list
    stages: list = field(default_factory=list)
    final_stages: list = field(default_factory=list)
    snapshot_requests: list = field(default_factory=list)
    snapshot_times: list = field(default_factory=list)
    snapshots: list = field(default_factory=list)
    status: str = "complete"
    error: str = ""
    seconds: float = 0.0
    observer_cpu_seconds: float = 0.0
    observer_wall_seconds: float = 0.0


def schedule_nodes(initial_time: float, sequence: np.ndarray) -> np.ndarray:
    """Node times by compensated (Kahan) accumulation (schedule.py:7-19)."""
    nodes = np.empty(sequence.size + 1, dtype=float)
    nodes[0] = initial_time
    total, carry = float(initial_time), 0.0
    for k, h in enumerate(sequence, start=1):
        inc = float(h) - carry
        new = total + inc
        carry = (new - total) - inc
        total = new
        nodes[k] = total
    return nodes


def nearest_node_indices(nodes: np.ndarray, requests: list) -> list[int]:
    """Nearest node per request, the earlier one on a tie (schedule.py:22-29)."""
    out = []
    for t in requests:
        dist = np.abs(nodes - t)
        tie = 8 * np.finfo(float).eps * max(abs(t), float(np.max(np.abs(nodes))), np.finfo(float).tiny)
        out.append(int(np.flatnonzero(dist <= dist.min() + tie)[0]))
    return out


def step_sizes(T: float, *, dt: float | None = None, steps: list | None = None) -> np.ndarray:
    """``solver/integrate.py:27-44``."""
    if not np.isfinite(T) or T <= 0:
        raise ValueError("T must be positive")
    if (dt is None) == (steps is None):
        raise ValueError("Specify exactly one of dt or steps")
    if steps is not None:
        seq = np.asarray(steps, dtype=float)
        if seq.ndim != 1 or seq.size == 0 or not np.isfinite(seq).all() or np.any(seq <= 0):
            raise ValueError("Steps must be finite and positive")
        if not np.isclose(np.sum(seq), T, rtol=1e-12, atol=1e-14 * T):
            raise ValueError("Prescribed steps must sum to T")
        return seq
    if not np.isfinite(dt) or dt <= 0:
        raise ValueError("dt must be positive")
    ratio = T / dt
    nearest = round(ratio)
    if nearest > 0 and abs(ratio - nearest) <= 1e-12 * max(1, ratio):
        return np.full(nearest, dt)
    count = int(np.floor(ratio))
    return np.r_[np.full(count, dt), T - count * dt]


def state_finite(model, state) -> bool:
    """Every velocity entry of ``state`` is finite (integrate.py:67).  A state
    that carries its packed device vector is checked on the device (the
    maximum of |x| propagates NaN and Inf), without a host copy."""
    device = getattr(state, "device", None)
    if device is not None and hasattr(model, "max_abs"):
        return bool(np.isfinite(model.max_abs(device)))
    return bool(np.isfinite(model.vector(state)).all())


def integrate(model, scheme, initial, steps, snapshots: list | None = None,
              progress: Callable[[int, float, float], None] | None = None, *,
              on_accept: Callable | None = None) -> Result:
    """``solver/integrate.py:47-100``."""
    seq = np.asarray(steps, dtype=float)
    if seq.ndim != 1 or seq.size == 0 or np.any(seq <= 0) or not np.isfinite(seq).all():
        raise ValueError("Invalid step sequence")
    nodes = schedule_nodes(initial.t, seq)
    requests = [] if snapshots is None else list(snapshots)
    if any(not np.isfinite(t) or t < initial.t or t > nodes[-1] + 1e-12 for t in requests):
        raise ValueError("Snapshot time outside integration interval")
    indices = nearest_node_indices(nodes, requests)
    kept: dict = {}
    if 0 in indices:
        kept[0] = initial
    history = History(initial)
    result = Result(initial, [initial.t], [model.diagnostics(initial)])
    start = perf_counter()
    for k, dt in enumerate(seq):
        try:
            trial = scheme.step(model, history.state, float(dt))
            if not state_finite(model, trial.state) or not np.isfinite(trial.state.r):
                raise FloatingPointError("Nonfinite trial state")
            diagnostic = model.diagnostics(trial.state)
            if not all(np.isfinite(v) for v in diagnostic.values()):
                raise FloatingPointError("Nonfinite diagnostic")
            history.state = trial.state
            history.accepted_steps += 1
            result.final = trial.state
            result.times.append(trial.state.t)
            result.diagnostics.append(diagnostic)
            result.final_stages = trial.stages
            result.stages.append([stage_diagnostics(s) for s in trial.stages])
            if k + 1 in indices:
                kept[k + 1] = trial.state
            if on_accept is not None:
                wall, cpu = perf_counter(), process_time()
                try:
                    on_accept(trial.state)
                except Exception as error:
                    raise RuntimeError(f"Accepted-state observer failed: {type(error).__name__}: {error}") from error
                finally:
                    result.observer_wall_seconds += perf_counter() - wall
                    result.observer_cpu_seconds += process_time() - cpu
            if progress is not None:
                progress(k + 1, trial.state.t, perf_counter() - start - result.observer_wall_seconds)
        except Exception as error:
            result.status = "failed"
            result.error = f"{type(error).__name__}: {error}"
            break
    for request, index in zip(requests, indices):
        if index in kept:
            result.snapshot_requests.append(request)
            result.snapshot_times.append(kept[index].t)
            result.snapshots.append(kept[index])
    result.seconds = perf_counter() - start - result.observer_wall_seconds
    return result
