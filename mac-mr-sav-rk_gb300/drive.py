"""Device-resident time loops for the fused GPU schemes.

The reference advances a scheme with ``integrate`` / ``integrate_adaptive``
(solver/integrate.py:47-100, solver/adaptivity/controller.py:126-398); the
GPU model and the fused schemes plug into those unchanged.  This module is
the package's own loop for the common cases, built around the fused step:

* the velocity stays on the device from the first step to the last: a step
  reads the accepted velocity and writes its trial into a second buffer;
  accepting a trial swaps the two buffers and rejecting it leaves the accepted
  one untouched, so neither costs a copy, and no host state is built between
  steps;
* an adaptive attempt's error estimate comes with the step: the fused step
  forms the embedded-error inner products on the device and they come back in
  the same device-to-host transfer as the stage records, so the host's work
  per attempt is a handful of scalar operations.

``run_adaptive`` applies the reference's step-size control (the scaled
embedded error of controller.py:112-123 and the I and PI step factors of
controller.py:14-70, with its treatment of rejected attempts, of the last
step and of the step bounds), so it takes the same accepted and rejected
attempts as the reference's driver.  It leaves out what that driver offers
beyond the integration itself (snapshots, strict output partitions, scalar
error control, continuation, observers); for those, call the reference's
``integrate_adaptive`` with this package's model and scheme.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from time import perf_counter
from typing import Any

import torch

from . import _lib


@dataclass(frozen=True)
class StepControl:
    """Embedded-error step control: elementary (``pi`` None) or PI.

    The scaled error of an attempt is |x1 - x_emb|_h / (atol + rtol max(|x0|_h,
    |x1|_h)); an attempt is accepted when it is at most 1.  After an accepted
    attempt the step is multiplied by safety err^(-1/order) (I) or by
    safety err^(-kp/order) err_prev^(ki/order) (PI, errors floored at
    ``error_floor``), clipped to [min_factor, max_factor]; after a rejected one
    by the elementary factor, at most 0.8.  These are the reference's
    controllers (solver/adaptivity/controller.py:14-70) with their defaults.
    """
    atol: float = 1e-8
    rtol: float = 1e-4
    safety: float = 0.9
    min_factor: float = 0.2
    max_factor: float = 2.0
    min_step: float = 1e-10
    max_step: float = math.inf
    max_rejections: int = 12
    max_steps: int = 1_000_000
    order: int = 3
    pi: tuple[float, float] | None = None
    error_floor: float = 1e-14

    def __post_init__(self) -> None:
        vals = (self.atol, self.rtol, self.safety, self.min_factor, self.max_factor, self.min_step, self.error_floor)
        if not all(math.isfinite(v) for v in vals):
            raise ValueError("step control parameters must be finite")
        if self.atol < 0 or self.rtol < 0 or self.atol + self.rtol == 0:
            raise ValueError("at least one tolerance must be positive")
        if not (0 < self.safety < 1 and 0 < self.min_factor < 1 < self.max_factor):
            raise ValueError("need 0 < safety < 1 and 0 < min_factor < 1 < max_factor")
        if not (0 < self.min_step <= self.max_step):
            raise ValueError("need 0 < min_step <= max_step")
        if self.max_rejections < 0 or self.max_steps < 1 or not isinstance(self.order, int) or self.order < 2:
            raise ValueError("need max_rejections >= 0, max_steps >= 1 and an integer order >= 2")
        if self.pi is not None:
            kp, ki = self.pi
            if not (math.isfinite(kp) and math.isfinite(ki) and kp > ki >= 0):
                raise ValueError("PI gains need proportional > integral >= 0")
        if not 0 < self.error_floor < 1:
            raise ValueError("need 0 < error_floor < 1")

    @classmethod
    def of(cls, control: Any) -> "StepControl":
        """A ``StepControl``, or the same control read from one of the
        reference's controller objects (IController / PIController)."""
        if isinstance(control, StepControl):
            return control
        pi = None
        if hasattr(control, "proportional"):
            pi = (float(control.proportional), float(control.integral))
        return cls(atol=float(control.atol), rtol=float(control.rtol), safety=float(control.safety),
                   min_factor=float(control.min_factor), max_factor=float(control.max_factor),
                   min_step=float(control.min_step), max_step=float(control.max_step),
                   max_rejections=int(control.max_rejections), max_steps=int(control.max_steps),
                   order=int(control.estimator_order), pi=pi,
                   error_floor=float(getattr(control, "error_floor", 1e-14)))

    def error(self, diff_sq: float, old_sq: float, new_sq: float) -> float:
        """Scaled error from the squared norms |x1 - x_emb|_h^2, |x0|_h^2 and
        |x1|_h^2; infinite when one of them is not a finite square."""
        if not all(math.isfinite(v) and v >= 0 for v in (diff_sq, old_sq, new_sq)):
            return math.inf
        return math.sqrt(diff_sq) / (self.atol + self.rtol * max(math.sqrt(old_sq), math.sqrt(new_sq)))

    def _elementary(self, err: float) -> float:
        if err == 0:
            return self.max_factor
        return min(max(self.safety * err ** (-1 / self.order), self.min_factor), self.max_factor)

    def grow(self, err: float, previous: float | None) -> float:
        """Step factor after an accepted attempt (previous: the last accepted
        attempt's error, None for the first)."""
        if self.pi is None or previous is None:
            return self._elementary(err)
        kp, ki = self.pi
        factor = self.safety * max(err, self.error_floor) ** (-kp / self.order) \
            * max(previous, self.error_floor) ** (ki / self.order)
        return min(max(factor, self.min_factor), self.max_factor)

    def shrink(self, err: float) -> float:
        """Step factor after a rejected attempt."""
        return min(self._elementary(err), 0.8)


class _DeviceTrials:
    """The device buffers of one run: the accepted velocity, the trial, the
    embedded velocity and the stage pressures; accept() swaps the first two."""

    def __init__(self, model, scheme, x0: torch.Tensor, embedded: bool) -> None:
        g = model.grid
        self.model, self.scheme = model, scheme
        self.x = x0.detach().clone()
        self.y = torch.empty_like(self.x)
        self.emb = torch.empty_like(self.x) if embedded else None
        self.pres = torch.empty((scheme.info.n_stages, g.np), dtype=torch.float64, device=self.x.device)
        self.norms = (C.c_double * 4)()
        self.records = None

    def step(self, t: float, r: float, h: float) -> tuple[float | None, str]:
        """One fused step from the accepted velocity into the trial buffer.
        Returns (r1, "") or (None, the failure) when a stage check failed."""
        try:
            _, r1, self.records, _, _ = self.scheme.step_device(
                self.model, self.x, t, r, h, x1=self.y, emb=self.emb, pres=self.pres,
                want_embedded=self.emb is not None)
        except RuntimeError as exc:
            return None, f"RuntimeError: {exc}"
        if self.emb is not None:
            # formed on the device inside the step and already on the host
            _lib.check(_lib.load().macsav_step_embedded_norms(self.model.plan.handle, self.norms),
                       self.model.plan.handle)
        return r1, ""

    def accept(self) -> None:
        self.x, self.y = self.y, self.x


@dataclass
class AdaptiveRun:
    """Outcome of ``run_adaptive``: the final state (its velocity on the
    device and, through ``State``, on the host), ``status`` "complete" or
    "failed" with ``error``, the counts and, per attempt, its start time, step,
    scaled error, decision, reason and step factor."""
    final: Any
    status: str = "complete"
    error: str = ""
    accepted_steps: int = 0
    attempted_steps: int = 0
    attempts: list = field(default_factory=list)
    times: list = field(default_factory=list)
    seconds: float = 0.0

    @property
    def rejected_steps(self) -> int:
        return self.attempted_steps - self.accepted_steps


def run_adaptive(model, scheme, initial, T: float, initial_step: float, control: Any = None, *,
                 keep_attempts: bool = True) -> AdaptiveRun:
    """Integrate from ``initial`` over a span ``T`` with the fused scheme's
    embedded error controlling the step (``control``: a ``StepControl`` or a
    reference controller; default elementary control).  Every attempt is one
    fused step; the accepted velocity never leaves the device."""
    ctl = StepControl.of(control if control is not None else StepControl())
    if scheme.info.estimator_order is None:
        raise ValueError(f"{scheme.name} has no embedded velocity to control the step with")
    if not (math.isfinite(T) and math.isfinite(initial_step) and math.isfinite(initial.t)) or T <= 0 \
            or initial_step <= 0:
        raise ValueError("T and initial_step must be finite and positive")
    if initial_step < ctl.min_step:
        raise ValueError("initial_step is below min_step")
    trials = _DeviceTrials(model, scheme, model.device_vector(initial), embedded=True)
    end = initial.t + T
    t, r = float(initial.t), float(initial.r)
    h = min(initial_step, ctl.max_step)
    run = AdaptiveRun(final=initial, times=[t])
    previous: float | None = None
    rejections = 0
    start = perf_counter()
    while t < end:
        if run.accepted_steps >= ctl.max_steps:
            run.status, run.error = "failed", "Maximum accepted steps exceeded"
            break
        remaining = end - t
        h_try = min(h, remaining)
        last = h_try == remaining
        if h_try < ctl.min_step and not last:
            run.status, run.error = "failed", "Step below min_step"
            break
        r1, failure = trials.step(t, r, h_try)
        err = math.inf
        if not failure:
            diff_sq, old_sq, new_sq, emb_bad = tuple(trials.norms)
            if emb_bad != 0.0 or not math.isfinite(new_sq) or not math.isfinite(r1):
                failure = "FloatingPointError: Nonfinite trial state"
            else:
                err = ctl.error(diff_sq, old_sq, new_sq)
                failure = "nonfinite_error" if not math.isfinite(err) else ("error_exceeded" if err > 1.0 else "")
        factor = ctl.shrink(err) if failure else ctl.grow(err, previous)
        run.attempted_steps += 1
        if keep_attempts:
            run.attempts.append({"t": t, "step": h_try, "error": err, "accepted": not failure, "reason": failure,
                                 "factor": factor})
        if failure:
            rejections += 1
            if rejections > ctl.max_rejections:
                run.status, run.error = "failed", failure
                break
            h = h_try * factor
            if h < ctl.min_step:
                run.status, run.error = "failed", failure
                break
            continue
        trials.accept()
        rejections, previous = 0, err
        t = end if last else t + h_try
        r = r1
        run.accepted_steps += 1
        run.times.append(t)
        h = min(h_try * factor, ctl.max_step)
    torch.cuda.current_stream().synchronize()
    run.seconds = perf_counter() - start
    run.final = model.state(t, trials.x, r)
    return run


_REASONS = {1: "error_exceeded", 2: "nonfinite_error", 3: "FloatingPointError: Nonfinite trial state",
            5: "Step below min_step", 6: "Maximum accepted steps exceeded"}


def _reason_text(code: int, stage_status: int = 0) -> str:
    if code == 4:
        return f"RuntimeError: stage check failed (status {stage_status})"
    return _REASONS.get(code, "")


def run_adaptive_device(model, scheme, initial, T: float, initial_step: float, control: Any = None, *,
                        history: int = 4096) -> AdaptiveRun:
    """``run_adaptive`` with the whole attempt loop on the device: every
    attempt, its accept/reject decision, the retry with a smaller step and
    the next step's proposal run inside one CUDA graph launch
    (``macsav_integrate_adaptive``), so the host reads the outcome once.
    The step control and the decisions are those of ``run_adaptive`` (the
    reference's controllers, solver/adaptivity/controller.py:14-123,244-327).
    Needs an autonomous model (no body force: the device cannot evaluate
    the force's Python callable at the stage times of an attempt it chose);
    ``history`` attempts are returned in ``attempts``."""
    ctl = StepControl.of(control if control is not None else StepControl())
    if scheme.info.estimator_order is None:
        raise ValueError(f"{scheme.name} has no embedded velocity to control the step with")
    if not getattr(model.force, "zero", False):
        raise ValueError("the device-resident loop needs a model without body force; use run_adaptive")
    if not (math.isfinite(T) and math.isfinite(initial_step) and math.isfinite(initial.t)) or T <= 0 \
            or initial_step <= 0:
        raise ValueError("T and initial_step must be finite and positive")
    if initial_step < ctl.min_step:
        raise ValueError("initial_step is below min_step")
    lib = _lib.load()
    c = _lib.StepControl(ctl.atol, ctl.rtol, ctl.safety, ctl.min_factor, ctl.max_factor, ctl.min_step,
                         ctl.max_step, ctl.error_floor, ctl.pi[0] if ctl.pi else 0.0, ctl.pi[1] if ctl.pi else 0.0,
                         ctl.order, ctl.max_rejections, ctl.max_steps, 0)
    x0 = model.device_vector(initial).contiguous()
    x1 = torch.empty_like(x0)
    res = _lib.AdaptiveResult()
    hist = (_lib.AdaptiveAttempt * max(int(history), 1))()
    start = perf_counter()
    lib.macsav_plan_set_graph(model.plan.handle, 1)
    _lib.check(lib.macsav_integrate_adaptive(model.plan.handle, scheme._id, float(initial.t), float(T),
                                             float(initial_step), float(model.nu), float(scheme.gamma),
                                             C.c_void_p(x0.data_ptr()), float(initial.r), C.byref(c),
                                             C.c_void_p(x1.data_ptr()), C.byref(res), hist, int(history),
                                             C.c_void_p(torch.cuda.current_stream().cuda_stream)),
               model.plan.handle)
    run = AdaptiveRun(final=model.state(res.t, x1, res.r), accepted_steps=res.accepted_steps,
                      attempted_steps=res.attempted_steps, seconds=perf_counter() - start)
    if res.status != 0:
        run.status, run.error = "failed", _reason_text(res.reason)
    t = float(initial.t)
    run.times = [t]
    for a in hist[:min(res.attempted_steps, int(history))]:
        run.attempts.append({"t": a.t, "step": a.step, "error": a.error, "accepted": bool(a.accepted),
                             "reason": _reason_text(a.reason, a.stage_status), "factor": a.factor})
    for a, nxt in zip(run.attempts, run.attempts[1:] + [None]):
        if a["accepted"]:
            run.times.append(nxt["t"] if nxt is not None else res.t)
    return run


@dataclass
class FixedRun:
    """Outcome of ``run_fixed``: the final state, the accepted times, the last
    step's stages, and ``status`` "complete" or "failed" with ``error`` (the
    accepted prefix is kept, as the reference's integrate keeps it)."""
    final: Any
    times: list
    stages: list = field(default_factory=list)
    status: str = "complete"
    error: str = ""
    seconds: float = 0.0


def run_fixed(model, scheme, initial, steps) -> FixedRun:
    """Take steps of the given sizes with the velocity on the device
    throughout; the first failing step (a stage check, or a non-finite
    velocity or scalar) ends the run with the prefix before it."""
    seq = [float(h) for h in steps]
    if not seq or not all(math.isfinite(h) and h > 0 for h in seq):
        raise ValueError("Invalid step sequence")
    trials = _DeviceTrials(model, scheme, model.device_vector(initial), embedded=False)
    t, r = float(initial.t), float(initial.r)
    run = FixedRun(final=initial, times=[t])
    start = perf_counter()
    for h in seq:
        r1, failure = trials.step(t, r, h)
        if not failure and not (math.isfinite(r1) and math.isfinite(model.max_abs(trials.y))):
            failure = "FloatingPointError: Nonfinite trial state"
        if failure:
            run.status, run.error = "failed", failure
            break
        trials.accept()
        t, r = t + h, r1
        run.times.append(t)
        run.stages = list(trials.records)
    torch.cuda.current_stream().synchronize()
    run.seconds = perf_counter() - start
    run.final = model.state(t, trials.x, r)
    return run
