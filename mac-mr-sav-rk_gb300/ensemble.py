"""Ensembles of independent no-slip cavities stepped together on one GB300.

The reference steps one model at a time; an ensemble there is a loop of
``integrate`` calls over models (its documentation recommends process-level
parallelism over members, docs/linear-stokes-acceleration-research.md:263-277,
without implementing it).  Here every member has its own model (a plan with
device tables and buffers) and its own captured step graph, and one ensemble
step enqueues every member's step (``macsav_step_enqueue``) on the member's own
stream before it waits for any (``macsav_step_finish``).  The GPU therefore
overlaps the members' kernels, and the host waits once per ensemble step.
Each member computes exactly what a lone ``make_scheme(name).step`` computes on
it: same kernels, same launch shapes, same order, so results are bitwise equal.

``ensemble_members`` draws the mixed-size workload (grids from
{64, 96, 128, 192, 256}^2 on [0, nx/ny] x [0, 1], nu log-uniform in
[1e-4, 1e-2], one seed per member); ``shard_members`` splits members across
processes by cell count, for runs with one process per GPU and no exchange.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _lib, fields
from ._lib import StageRecord
from .grid import MACGrid
from .model import MACNavierStokes
from .schemes import make_scheme
from .stokes import dptr

SIZES = (64, 96, 128, 192, 256)


@dataclass(frozen=True)
class Member:
    """One cavity: grid nx x ny on [0, nx/ny] x [0, 1], viscosity, field seed."""
    nx: int
    ny: int
    nu: float
    seed: int

    @property
    def cells(self) -> int:
        return self.nx * self.ny

    def grid(self) -> MACGrid:
        return MACGrid(self.nx, self.ny, self.nx / self.ny, 1.0)


def ensemble_members(count: int, seed: int = 0, sizes: Sequence[int] = SIZES,
                     nu_range: tuple[float, float] = (1e-4, 1e-2)) -> list[Member]:
    """``count`` members with nx, ny uniform over ``sizes`` and nu log-uniform."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log10(nu_range[0]), np.log10(nu_range[1])
    out = []
    for i in range(count):
        nx, ny = (int(s) for s in rng.choice(np.asarray(sizes), size=2))
        out.append(Member(nx, ny, float(10.0 ** rng.uniform(lo, hi)), int(seed) * 100003 + i))
    return out


def shard_members(members: Sequence[Member], world_size: int, rank: int) -> list[int]:
    """Indices of the members that ``rank`` runs: longest-processing-time
    assignment by cell count (ties by index), so every rank gets a similar
    number of cells and the shards are disjoint and cover all members."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("need 0 <= rank < world_size")
    loads = [0] * world_size
    owner = [0] * len(members)
    for i in sorted(range(len(members)), key=lambda k: (-members[k].cells, k)):
        r = min(range(world_size), key=lambda q: (loads[q], q))
        owner[i] = r
        loads[r] += members[i].cells
    return [i for i in range(len(members)) if owner[i] == rank]


class EnsembleError(RuntimeError):
    """A member's step failed; ``index`` names it and ``__cause__`` is the
    reference's exception for the failing stage."""

    def __init__(self, index: int, error: Exception) -> None:
        super().__init__(f"ensemble member {index}: {error}")
        self.index = index


class Ensemble:
    """Members stepped concurrently with one fused scheme (see module docstring).

    ``precision`` "fp32" is the FP32-bulk Stokes form (FP64 reductions, SAV
    scalars and gates); "fp64" is the plain path.
    """

    def __init__(self, members: Sequence[Member], scheme: str = "sdirk2_mrsav", gamma: float = 1.0, *,
                 precision: str = "fp32", use_graph: bool = True, tolerance: float = 1e-9,
                 krylov_tolerance: float = 1e-12) -> None:
        if not members:
            raise ValueError("an ensemble needs at least one member")
        self.members = list(members)
        self.scheme = make_scheme(scheme, gamma)
        self.models = [MACNavierStokes(m.grid(), m.nu, precision=precision, use_graph=use_graph,
                                       tolerance=tolerance, krylov_tolerance=krylov_tolerance)
                       for m in self.members]
        self.lib = _lib.load()
        for model in self.models:
            self.lib.macsav_plan_set_graph(model.plan.handle, 1 if use_graph else 0)
        self.streams = [torch.cuda.Stream() for _ in self.members]
        n = self.scheme.info.n_stages
        self._x = [torch.zeros((2, m.grid().size), dtype=torch.float64, device="cuda") for m in self.members]
        self._pres = [torch.empty((n, m.cells), dtype=torch.float64, device="cuda") for m in self.members]
        self._cur = [0] * len(self.members)
        self.t = np.zeros(len(self.members))
        self.r = np.zeros(len(self.members))
        self.last_records: list[list[StageRecord]] = []

    def __len__(self) -> int:
        return len(self.members)

    @property
    def cells(self) -> int:
        return sum(m.cells for m in self.members)

    def set_state(self, index: int, velocity, r: float = 0.0, t: float = 0.0) -> None:
        x = self.models[index]._dev(velocity).reshape(-1)
        self._x[index][self._cur[index]].copy_(x)
        self.r[index] = float(r)
        self.t[index] = float(t)

    def seed_fields(self, modes: int = 8, r: float | None = None) -> None:
        """The seeded curl fields (psi modes k,l <= ``modes``), one per member;
        SAV schemes start from r = 1 unless ``r`` is given."""
        r0 = (1.0 if self.scheme.sav else 0.0) if r is None else r
        for i, m in enumerate(self.members):
            g = m.grid()
            self.set_state(i, fields.packed_curl_velocity(m.nx, m.ny, g.lx, g.ly, modes, m.seed), r0)

    def velocity(self, index: int) -> torch.Tensor:
        return self._x[index][self._cur[index]]

    def step(self, dt: float) -> list[list[StageRecord]]:
        """One step of every member; raises ``EnsembleError`` for the first
        failing member after all enqueued steps have finished (the states of
        the members are then left as they were before the step)."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        ready = torch.cuda.Event()
        ready.record(torch.cuda.current_stream())
        sid = self.scheme._id
        n = self.scheme.info.n_stages
        enqueued, failure = [], None
        for i, (model, stream) in enumerate(zip(self.models, self.streams)):
            stream.wait_event(ready)
            x = self._x[i]
            code = self.lib.macsav_step_enqueue(
                model.plan.handle, sid, float(self.t[i]), float(dt), float(model.nu), self.scheme.gamma,
                dptr(x[self._cur[i]]), float(self.r[i]), None, dptr(x[1 - self._cur[i]]), None,
                dptr(self._pres[i]), C.c_void_p(stream.cuda_stream))
            if code != _lib.OK:
                failure = failure or (i, code, None)
                break
            enqueued.append(i)
        records: list[list[StageRecord]] = [[] for _ in self.members]
        r1s = {}
        for i in enqueued:
            recs = (StageRecord * n)()
            r1 = C.c_double()
            code = self.lib.macsav_step_finish(self.models[i].plan.handle, recs, C.byref(r1))
            records[i] = list(recs)
            r1s[i] = float(r1.value)
            if code != _lib.OK and failure is None:
                failure = (i, code, recs)
        torch.cuda.current_stream().wait_event(self._done_event())
        self.last_records = records
        if failure is not None:
            i, code, recs = failure
            try:
                failing = next((r for r in recs if r.status), None) if recs is not None else None
                if failing is None:
                    _lib.check(code, self.models[i].plan.handle)
                self.scheme._raise(code, failing, self.models[i].plan)
            except Exception as error:  # the reference's exception for the failing stage
                raise EnsembleError(i, error) from error
        for i in enqueued:
            self._cur[i] = 1 - self._cur[i]
            self.t[i] += dt
            if self.scheme.sav:
                self.r[i] = r1s[i]
        return records

    def _done_event(self) -> torch.cuda.Event:
        ev = torch.cuda.Event()
        for stream in self.streams:
            ev.record(stream)
            torch.cuda.current_stream().wait_event(ev)
        return ev

    def run(self, steps: int, dt: float) -> None:
        for _ in range(steps):
            self.step(dt)

    def diagnostics(self) -> list[dict[str, float]]:
        """``MACNavierStokes.diagnostics`` of every member's current state."""
        keys = ("kinetic", "modified_energy", "divergence_inf", "h1_seminorm_squared", "r", "angular_momentum",
                "power", "dissipation")
        out = []
        for i, model in enumerate(self.models):
            d = model._diagnostics(self.velocity(i), float(self.r[i]), None)
            out.append(dict(zip(keys, (float(v) for v in d))))
        return out
