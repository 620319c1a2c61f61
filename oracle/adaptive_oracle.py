"""Restatement of the reference's adaptive driver -- TEST INFRASTRUCTURE ONLY.

``integrate_adaptive`` with its I and PI controllers as in the reference's
``solver/adaptivity/controller.py`` (I/PI controllers :14-70, scalar error
control :73-90, continuation :93-100, error estimate :112-123, driver
:126-398).  The tests drive the GPU model and the fused GPU schemes with it,
as a user drives them with the reference's own driver (the reference's Python
cannot travel to the GPU machine), and pin it to the reference's adaptive runs
(tests/golden/adaptive.npz).  It takes the fused step's device-formed
embedded-error inner products when a trial carries them (``_error_from_norms``)
and checks a device state's finiteness on the device; otherwise it works on
host vectors like the reference.  The product package never imports it.
"""
from __future__ import annotations

from collections.abc import Callable
from dataclasses import dataclass, field, replace
from time import perf_counter, process_time
from typing import Any, Literal

import numpy as np

from .integrate_oracle import Result, stage_diagnostics


@dataclass(frozen=True)
class IController:
    """``controller.py:14-48``."""
    atol: float = 1e-8
    rtol: float = 1e-4
    safety: float = 0.9
    min_factor: float = 0.2
    max_factor: float = 2.0
    min_step: float = 1e-10
    max_step: float = float("inf")
    max_rejections: int = 12
    max_steps: int = 1_000_000
    estimator_order: int = 3

    def __post_init__(self) -> None:
        if not np.isfinite([self.atol, self.rtol, self.safety, self.min_factor, self.max_factor,
                            self.min_step]).all():
            raise ValueError("Controller parameters must be finite")
        if self.atol < 0 or self.rtol < 0 or self.atol + self.rtol == 0:
            raise ValueError("At least one tolerance must be positive")
        if not (0 < self.safety < 1 and 0 < self.min_factor < 1 < self.max_factor):
            raise ValueError("Invalid I-controller factors")
        if self.min_step <= 0 or np.isnan(self.max_step) or self.max_step < self.min_step:
            raise ValueError("Invalid step bounds")
        if self.max_rejections < 0 or self.max_steps <= 0:
            raise ValueError("Invalid trial limits")
        if type(self.estimator_order) is not int or self.estimator_order < 2:
            raise ValueError("Invalid estimator order")

    def accepted_factor(self, error: float, previous_error: float | None) -> float:
        if error == 0:
            return self.max_factor
        return float(np.clip(self.safety * error ** (-1 / self.estimator_order), self.min_factor, self.max_factor))


@dataclass(frozen=True)
class PIController(IController):
    """``controller.py:51-70``."""
    proportional: float = 0.7
    integral: float = 0.4
    error_floor: float = 1e-14

    def __post_init__(self) -> None:
        super().__post_init__()
        if not np.isfinite([self.proportional, self.integral, self.error_floor]).all() \
                or self.proportional <= self.integral or self.integral < 0 or not 0 < self.error_floor < 1:
            raise ValueError("Invalid PI-controller parameters")

    def accepted_factor(self, error: float, previous_error: float | None) -> float:
        if previous_error is None:
            return super().accepted_factor(error, previous_error)
        current = max(error, self.error_floor)
        previous = max(previous_error, self.error_floor)
        factor = self.safety * current ** (-self.proportional / self.estimator_order) \
            * previous ** (self.integral / self.estimator_order)
        return float(np.clip(factor, self.min_factor, self.max_factor))


@dataclass(frozen=True)
class ScalarErrorControl:
    """``controller.py:73-90``: local defect of r' = -gamma r over one step."""
    atol: float
    gamma: float

    def __post_init__(self) -> None:
        if not np.isfinite([self.atol, self.gamma]).all() or self.atol <= 0 or self.gamma < 0:
            raise ValueError("Invalid scalar error controls")

    def defect(self, old_r: float, trial_r: float, step: float) -> float:
        return float(trial_r - np.exp(-self.gamma * step) * old_r)


@dataclass(frozen=True)
class AdaptiveContinuation:
    """``controller.py:93-100``."""
    step: float
    previous_error: float | None = None
    previous_u: float | None = None
    previous_r: float | None = None
    accepted_steps: int = 0
    attempted_steps: int = 0


@dataclass
class AdaptiveResult(Result):
    """``controller.py:103-109``."""
    attempts: list = field(default_factory=list)
    accepted_steps: int = 0
    attempted_steps: int = 0
    continuation: AdaptiveContinuation | None = None


def _finite(model, x) -> bool:
    if isinstance(x, np.ndarray):
        return bool(np.isfinite(x).all())
    return bool(np.isfinite(model.max_abs(x)))


def _error_from_norms(norms, controller: IController) -> float:
    """``_error`` from the step's device inner products (sq, old_sq, high_sq)."""
    sq, old_sq, high_sq = norms[:3]
    if not np.isfinite([sq, old_sq, high_sq]).all() or min(sq, old_sq, high_sq) < 0:
        return float("inf")
    scale = controller.atol + controller.rtol * max(np.sqrt(old_sq), np.sqrt(high_sq))
    return float(np.sqrt(sq) / scale)


def _error(model, old, high, low, controller: IController, error_norm) -> float:
    """Scaled embedded error (``controller.py:112-123``)."""
    difference = model.combine((1., high), (-1., low))
    sq = error_norm(difference) ** 2 if error_norm is not None else model.inner(difference, difference)
    old_sq = error_norm(old) ** 2 if error_norm is not None else model.inner(old, old)
    high_sq = error_norm(high) ** 2 if error_norm is not None else model.inner(high, high)
    if not np.isfinite([sq, old_sq, high_sq]).all() or min(sq, old_sq, high_sq) < 0:
        return float("inf")
    scale = controller.atol + controller.rtol * max(np.sqrt(old_sq), np.sqrt(high_sq))
    return float(np.sqrt(sq) / scale)


def integrate_adaptive(model, scheme, initial, T: float, initial_step: float, *,
                       controller: IController = IController(), snapshots: list | None = None,
                       error_norm: Callable[[Any], float] | None = None, strict_snapshots: bool = False,
                       progress: Callable[[int, float, float], None] | None = None,
                       on_accept: Callable[[Any], None] | None = None,
                       scalar_control: ScalarErrorControl | None = None,
                       min_step_policy: Literal["fail", "force"] = "fail", retain_history: bool = True,
                       continuation: AdaptiveContinuation | None = None,
                       on_attempt: Callable[[dict], None] | None = None,
                       on_advance: Callable[[AdaptiveResult], None] | None = None) -> AdaptiveResult:
    """``integrate_adaptive`` (``controller.py:126-398``): rejected trials never
    change the accepted state; terminal alignment, strict snapshot partitions,
    scalar control, the force floor policy and continuation as in the reference."""
    if min_step_policy not in ("fail", "force"):
        raise ValueError("Unknown min_step_policy")
    if not np.isfinite([T, initial_step, initial.t]).all() or T <= 0 or initial_step <= 0:
        raise ValueError("T and initial_step must be finite and positive")
    if initial_step < controller.min_step:
        raise ValueError("initial_step is below min_step")
    end = initial.t + T
    requests = [] if snapshots is None else list(snapshots)
    if any(not np.isfinite(t) or t < initial.t or t > end for t in requests):
        raise ValueError("Snapshot time outside integration interval")
    if strict_snapshots and requests != sorted(set(requests)):
        raise ValueError("Strict snapshot times must be distinct and increasing")
    best = [(abs(t - initial.t), initial) for t in requests]
    result = AdaptiveResult(initial, [initial.t], [model.diagnostics(initial)])
    if continuation is not None:
        if strict_snapshots:
            raise ValueError("Continuation supports natural nodes, not strict snapshot partitions")
        if not np.isfinite(continuation.step) or not controller.min_step <= continuation.step <= controller.max_step:
            raise ValueError("Invalid continuation step")
        hist = [v for v in (continuation.previous_error, continuation.previous_u, continuation.previous_r)
                if v is not None]
        if any(not np.isfinite(v) or v < 0 for v in hist) or continuation.accepted_steps < 0 \
                or continuation.attempted_steps < continuation.accepted_steps:
            raise ValueError("Invalid continuation history")
    saved = continuation or AdaptiveContinuation(min(initial_step, controller.max_step))
    step = saved.step
    result.continuation = saved
    rejections = 0
    previous_error, previous_u, previous_r = saved.previous_error, saved.previous_u, saved.previous_r
    scalar_controller = replace(controller, estimator_order=2)
    output_index = 0
    boundary_step: float | None = None
    boundary_left = 0
    if strict_snapshots and requests and requests[0] == initial.t:
        output_index = 1
    start, cpu_start = perf_counter(), process_time()
    diagnostic = None
    while result.final.t < end:
        if saved.accepted_steps + result.accepted_steps >= controller.max_steps:
            result.status, result.error = "failed", "Maximum accepted steps exceeded"
            break
        remaining = end - result.final.t
        time_tol = 8 * np.finfo(float).eps * max(abs(end), abs(result.final.t), 1.)
        proposed = min(step, remaining)
        step = proposed
        boundary_partition = output_truncated = False
        if strict_snapshots and output_index < len(requests):
            to_output = requests[output_index] - result.final.t
            if abs(to_output) <= time_tol:
                output_index += 1
                continue
            if to_output < 0:
                result.status, result.error = "failed", "Strict snapshot time was crossed"
                break
            if boundary_left:
                step = min(boundary_step, to_output)
                boundary_partition = True
            else:
                output_truncated = proposed >= to_output
                remainder = to_output - proposed
                if 0 < remainder < controller.min_step and to_output / 4 >= controller.min_step:
                    boundary_step, boundary_left = to_output / 4, 4
                    step, boundary_partition = boundary_step, True
                elif 0 < remainder < 0.5 * proposed and to_output / 2 >= controller.min_step:
                    boundary_step, boundary_left = to_output / 2, 2
                    step, boundary_partition = boundary_step, True
                else:
                    step = min(proposed, to_output)
        terminal = step == remaining
        force_floor = min_step_policy == "force" and step == controller.min_step
        if step < controller.min_step and not terminal:
            result.status, result.error = "failed", "Step below min_step"
            break
        reason = ""
        error = error_u = float("inf")
        error_r = scalar_defect = float("nan")
        trial = None
        try:
            trial = scheme.step(model, result.final, step)
            if trial.embedded_velocity is None:
                raise ValueError("Scheme does not provide an embedded velocity")
            # a fused GPU step brings the embedded-error inner products with it
            norms = getattr(trial, "embedded_norms", None) if error_norm is None else None
            device = getattr(trial.state, "device", None) if norms is not None else None
            if device is not None:
                # finiteness of the new state on the device (the maximum of
                # |x| propagates NaN and Inf), not on a host copy of it
                high = device
                high_finite = bool(np.isfinite(model.max_abs(device)))
            else:
                high = model.vector(trial.state)
                high_finite = bool(np.isfinite(high).all())
            if terminal:
                trial.state = model.state(end, high, trial.state.r)
            emb_finite = (norms[3] == 0.0) if norms is not None else _finite(model, trial.embedded_velocity)
            if not high_finite or not emb_finite or not np.isfinite(trial.state.r):
                raise FloatingPointError("Nonfinite trial state")
            if norms is not None:
                error_u = _error_from_norms(norms, controller)
            else:
                error_u = _error(model, model.vector(result.final), high, trial.embedded_velocity, controller,
                                 error_norm)
            error = error_u
            if scalar_control is not None:
                scalar_defect = scalar_control.defect(result.final.r, trial.state.r, step)
                error_r = abs(scalar_defect) / scalar_control.atol
                error = max(error_u, error_r) if np.isfinite(error_r) else float("inf")
            if not np.isfinite(error):
                reason = "nonfinite_error"
            elif error > 1. and not force_floor:
                reason = "error_exceeded"
            else:
                diagnostic = model.diagnostics(trial.state)
                if not all(np.isfinite(v) for v in diagnostic.values()):
                    raise FloatingPointError("Nonfinite diagnostic")
        except (FloatingPointError, RuntimeError, np.linalg.LinAlgError) as exc:
            reason = f"{type(exc).__name__}: {exc}"
        if reason:
            factor = min(IController.accepted_factor(controller, error_u, None), 0.8)
            if scalar_control is not None:
                se = error_r if np.isfinite(error_r) else float("inf")
                factor = min(factor, IController.accepted_factor(scalar_controller, se, None))
        else:
            factor = controller.accepted_factor(error_u, previous_u)
            if scalar_control is not None:
                factor = min(factor, scalar_controller.accepted_factor(error_r, previous_r))
        nan = float("nan")
        result.attempts.append({
            "t": float(result.final.t), "step": float(step), "error": float(error), "accepted": not bool(reason),
            "error_u": float(error_u), "error_r": float(error_r), "scalar_defect": float(scalar_defect),
            "reason": reason, "factor": float(factor), "boundary_partition": boundary_partition,
            "output_truncated": output_truncated,
            "previous_accepted_error": nan if previous_error is None else previous_error,
            "previous_accepted_error_u": nan if previous_u is None else previous_u,
            "previous_accepted_error_r": nan if previous_r is None else previous_r,
            "controller": type(controller).__name__,
            "elapsed_seconds": perf_counter() - start - result.observer_wall_seconds,
            "cpu_seconds": process_time() - cpu_start - result.observer_cpu_seconds})
        result.attempted_steps += 1
        if not retain_history:
            result.attempts[:] = result.attempts[-1:]
        if on_attempt is not None:
            w0, c0 = perf_counter(), process_time()
            try:
                on_attempt(result.attempts[-1])
            except Exception as exc:
                result.status, result.error = "failed", f"Trial observer failed: {type(exc).__name__}: {exc}"
                break
            finally:
                result.observer_cpu_seconds += process_time() - c0
                result.observer_wall_seconds += perf_counter() - w0
        if reason:
            if boundary_partition:
                boundary_step, boundary_left = None, 0
            rejections += 1
            if rejections > controller.max_rejections:
                result.status, result.error = "failed", reason or "Maximum rejections exceeded"
                break
            new_step = step * factor
            if new_step < controller.min_step:
                if min_step_policy == "force" and step > controller.min_step and not terminal:
                    step = controller.min_step
                    continue
                result.status, result.error = "failed", reason
                break
            step = new_step
            continue
        rejections = 0
        previous_error, previous_u = error, error_u
        if scalar_control is not None:
            previous_r = error_r
        result.final = trial.state
        if strict_snapshots and output_index < len(requests) and \
                abs(trial.state.t - requests[output_index]) <= 8 * np.finfo(float).eps * max(1., abs(trial.state.t)):
            output_index += 1
        result.accepted_steps += 1
        result.times.append(trial.state.t)
        result.diagnostics.append(diagnostic)
        result.final_stages = trial.stages
        result.stages.append([stage_diagnostics(s) for s in trial.stages])
        if not retain_history:
            result.times[:] = [initial.t, trial.state.t]
            result.diagnostics[:] = result.diagnostics[-1:]
            result.stages[:] = result.stages[-1:]
        for index, request in enumerate(requests):
            distance = abs(request - trial.state.t)
            if distance < best[index][0]:
                best[index] = (distance, trial.state)
        if boundary_partition:
            boundary_left -= 1
            if boundary_left:
                step = boundary_step
            else:
                boundary_step = None
                step = min(step * factor, controller.max_step)
        else:
            step = min(step * factor, controller.max_step)
        if min_step_policy == "force" and not boundary_left:
            step = max(step, controller.min_step)
        result.continuation = AdaptiveContinuation(step, previous_error, previous_u, previous_r,
                                                   saved.accepted_steps + result.accepted_steps,
                                                   saved.attempted_steps + result.attempted_steps)
        if on_accept is not None:
            w0, c0 = perf_counter(), process_time()
            try:
                on_accept(trial.state)
            except Exception as exc:
                result.status, result.error = "failed", f"Accepted-state observer failed: {type(exc).__name__}: {exc}"
                break
            finally:
                result.observer_cpu_seconds += process_time() - c0
                result.observer_wall_seconds += perf_counter() - w0
        if progress is not None:
            progress(result.accepted_steps, trial.state.t, perf_counter() - start - result.observer_wall_seconds)
        if on_advance is not None:
            w0, c0 = perf_counter(), process_time()
            try:
                on_advance(result)
            except Exception as exc:
                result.status, result.error = "failed", f"Advance observer failed: {type(exc).__name__}: {exc}"
                break
            finally:
                result.observer_cpu_seconds += process_time() - c0
                result.observer_wall_seconds += perf_counter() - w0
    for request, (_, state) in zip(requests, best):
        result.snapshot_requests.append(request)
        result.snapshot_times.append(state.t)
        result.snapshots.append(state)
    result.seconds = perf_counter() - start - result.observer_wall_seconds
    return result
