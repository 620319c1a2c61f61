"""Ensembles of independent no-slip cavities stepped together on one GB300.

The reference steps one model at a time; an ensemble there is a loop of
``integrate`` calls over models (its documentation recommends process-level
parallelism over members, docs/linear-stokes-acceleration-research.md:263-277,
without implementing it).  Here equal-shape members share one plan
(``macsav_plan_create_members``, up to 32 members): every stage kernel runs
once for all of them (member = blockIdx.y), the Stokes solve treats their
2 x M right-hand sides as columns with per-member shifts, and each member
keeps its own viscosity, SAV scalar, records and gates.  Every plan has its
own stream and captured step graph; one ensemble step enqueues all plans'
steps (``macsav_step_members_enqueue``) before it waits for any
(``macsav_step_members_finish``), so the shape groups overlap on the GPU and
the host waits once per ensemble step.  Each member computes exactly what a
lone ``make_scheme(name).step`` computes on it (the per-column arithmetic and
launch shapes are those of a single cavity), so results are bitwise equal.

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
from .schemes import make_scheme
from .stokes import PRECISIONS, dptr, stream_handle

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


class _Unit:
    """One plan stepping ``len(indices)`` equal-shape members together
    (``macsav_plan_create_members``), with its stream and state buffers."""

    def __init__(self, lib, members: Sequence[Member], indices: list[int], scheme, precision: str, use_graph: bool,
                 tolerance: float, krylov_tolerance: float) -> None:
        self.lib, self.indices = lib, indices
        grid = members[indices[0]].grid()
        self.grid = grid
        handle = C.c_void_p()
        code = lib.macsav_plan_create_members(C.byref(handle), grid.nx, grid.ny, float(grid.lx), float(grid.ly),
                                              PRECISIONS[precision], float(tolerance), float(krylov_tolerance), 100,
                                              len(indices))
        if code != _lib.OK:
            _lib.check(code, None)
        self.handle = handle
        lib.macsav_plan_set_graph(handle, 1 if use_graph else 0)
        M, n = len(indices), scheme.info.n_stages
        self.nus = (C.c_double * M)(*[members[i].nu for i in indices])
        self.x = torch.zeros((2, M, grid.size), dtype=torch.float64, device="cuda")
        self.pres = torch.empty((M, n, grid.np), dtype=torch.float64, device="cuda")
        self.cur = 0
        self.stream = torch.cuda.Stream()

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                torch.cuda.synchronize()
            except Exception:
                pass
            self.lib.macsav_plan_destroy(h)
            self.handle = None


class Ensemble:
    """Members stepped concurrently with one fused scheme (see module docstring).

    ``batched=True`` (default) groups equal-shape members into plans of up to
    ``max_group`` members, so each stage kernel runs once for the group;
    ``batched=False`` gives every member its own plan.  Either way every
    member's result is bitwise that of a lone step.  ``precision`` "fp32" is
    the FP32-bulk Stokes form (FP64 reductions, SAV scalars and gates);
    "fp64" is the plain path.
    """

    def __init__(self, members: Sequence[Member], scheme: str = "sdirk2_mrsav", gamma: float = 1.0, *,
                 precision: str = "fp32", use_graph: bool = True, tolerance: float = 1e-9,
                 krylov_tolerance: float = 1e-12, batched: bool = True, max_group: int = 16) -> None:
        if not members:
            raise ValueError("an ensemble needs at least one member")
        if not 1 <= max_group <= 32:
            raise ValueError("max_group must be in 1..32")
        self.members = list(members)
        self.scheme = make_scheme(scheme, gamma)
        self.lib = _lib.load()
        torch.cuda.init()
        groups: dict[tuple[int, int], list[int]] = {}
        for i, m in enumerate(self.members):
            groups.setdefault((m.nx, m.ny), []).append(i)
        size = max_group if batched else 1
        self.units = [_Unit(self.lib, self.members, idx[k:k + size], self.scheme, precision, use_graph, tolerance,
                            krylov_tolerance)
                      for idx in groups.values() for k in range(0, len(idx), size)]
        self._where = {i: (u, j) for u in self.units for j, i in enumerate(u.indices)}
        self.t = np.zeros(len(self.members))
        self.r = np.zeros(len(self.members))
        self.last_records: list[list[StageRecord]] = []
        self._host = None      # (pinned block, per-member views, mapped)
        self._tables = {}      # device pointer tables of the host copies, by slot parity

    def __len__(self) -> int:
        return len(self.members)

    @property
    def cells(self) -> int:
        return sum(m.cells for m in self.members)

    def set_state(self, index: int, velocity, r: float = 0.0, t: float = 0.0) -> None:
        unit, j = self._where[index]
        x = velocity if isinstance(velocity, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(np.asarray(velocity, dtype=np.float64)))
        # one copy straight into the member's slot (a blocking copy from host
        # memory; from a pinned buffer it runs at full link speed)
        unit.x[unit.cur, j].copy_(x.reshape(-1).to(torch.float64))
        self.r[index] = float(r)
        self.t[index] = float(t)

    def seed_fields(self, modes: int = 8, r: float | None = None) -> None:
        """The seeded curl fields (psi modes k,l <= ``modes``), one per member;
        SAV schemes start from r = 1 unless ``r`` is given."""
        r0 = (1.0 if self.scheme.sav else 0.0) if r is None else r
        for i, m in enumerate(self.members):
            g = m.grid()
            self.set_state(i, fields.packed_curl_velocity(m.nx, m.ny, g.lx, g.ly, modes, m.seed), r0)

    # ------------------------------------------------------ host boundary ---
    def host_buffers(self) -> list[np.ndarray]:
        """One host array per member (its packed velocity, float64), in one
        pinned block allocated on first use and owned by the ensemble.
        ``upload()`` moves every buffer into its member's state and
        ``download()`` fills every buffer from it, each as one kernel that
        reads or writes the pinned block over the host link
        (``macsav_copy_vectors``); where the device does not map the block,
        as one copy per member.  Either way the call returns once the data
        have arrived."""
        if self._host is None:
            sizes = [m.grid().size for m in self.members]
            block = torch.empty(sum(sizes), dtype=torch.float64, pin_memory=True)
            offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            views = [block[int(offs[i]):int(offs[i + 1])].numpy() for i in range(len(sizes))]
            ok = C.c_int()
            _lib.check(self.lib.macsav_host_mapped(block.data_ptr(), block.nbytes, C.byref(ok)), None)
            self._host = (block, views, bool(ok.value))
        return self._host[1]

    def _copy_tables(self) -> tuple[torch.Tensor, torch.Tensor, int]:
        """Device pointer tables (src, dst, n) for host -> states and
        states -> host at the current slot parity of every plan."""
        key = tuple(u.cur for u in self.units)
        hit = self._tables.get(key)
        if hit is None:
            block, views, _ = self._host
            host = [v.ctypes.data for v in views]
            slots = [0] * len(self.members)
            for u in self.units:
                for j, i in enumerate(u.indices):
                    slots[i] = u.x[u.cur, j].data_ptr()
            n = [v.size for v in views]
            t_in = torch.tensor([host, slots, n], dtype=torch.int64).to("cuda")
            t_out = torch.tensor([slots, host, n], dtype=torch.int64).to("cuda")
            hit = self._tables[key] = (t_in, t_out, max(n))
        return hit

    def _copy_all(self, upload: bool) -> None:
        if self._host is None:
            self.host_buffers()
        block, views, mapped = self._host
        if mapped:
            t_in, t_out, max_n = self._copy_tables()
            t = t_in if upload else t_out
            row = t.stride(0) * t.element_size()
            p = t.data_ptr()
            _lib.check(self.lib.macsav_copy_vectors(len(views), p, p + row, p + 2 * row, max_n, stream_handle()),
                       None)
        else:
            for i, v in enumerate(views):
                slot, h = self.velocity(i), torch.from_numpy(v)
                if upload:
                    slot.copy_(h, non_blocking=True)
                else:
                    h.copy_(slot, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    def upload(self, r=None, t=None) -> None:
        """Every member's state from its host buffer (``host_buffers``), with
        optional per-member SAV scalars ``r`` and times ``t``."""
        if r is not None and len(r) != len(self.members) or t is not None and len(t) != len(self.members):
            raise ValueError("need one r and one t per member")
        self._copy_all(True)
        if r is not None:
            self.r[:] = np.asarray(r, dtype=np.float64)
        if t is not None:
            self.t[:] = np.asarray(t, dtype=np.float64)

    def download(self) -> list[np.ndarray]:
        """Every member's packed velocity into its host buffer; returns the
        buffers."""
        self._copy_all(False)
        return self._host[1]

    def velocity(self, index: int) -> torch.Tensor:
        unit, j = self._where[index]
        return unit.x[unit.cur, j]

    def step(self, dt: float) -> list[list[StageRecord]]:
        """One step of every member; raises ``EnsembleError`` for the first
        failing member after all enqueued steps have finished (the states of
        all members are then left as they were before the step)."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        ready = torch.cuda.Event()
        ready.record(torch.cuda.current_stream())
        sid = self.scheme._id
        n = self.scheme.info.n_stages
        enqueued, failure = [], None
        for u in self.units:
            u.stream.wait_event(ready)
            M = len(u.indices)
            r0 = (C.c_double * M)(*[self.r[i] for i in u.indices])
            t0 = float(self.t[u.indices[0]])
            code = self.lib.macsav_step_members_enqueue(
                u.handle, sid, t0, float(dt), u.nus, self.scheme.gamma, dptr(u.x[u.cur]), r0, None,
                dptr(u.x[1 - u.cur]), None, dptr(u.pres), C.c_void_p(u.stream.cuda_stream))
            if code != _lib.OK:
                failure = failure or (u.indices[0], code, None, u)
                break
            enqueued.append(u)
        records: list[list[StageRecord]] = [[] for _ in self.members]
        r1s = {}
        for u in enqueued:
            M = len(u.indices)
            recs = (StageRecord * (M * n))()
            r1 = (C.c_double * M)()
            code = self.lib.macsav_step_members_finish(u.handle, recs, r1)
            for j, i in enumerate(u.indices):
                records[i] = list(recs[j * n:(j + 1) * n])
                r1s[i] = float(r1[j])
            if code != _lib.OK and failure is None:
                bad = next((i for i in u.indices if any(rc.status for rc in records[i])), u.indices[0])
                failure = (bad, code, records[bad], u)
        done = torch.cuda.Event()
        for u in self.units:
            done.record(u.stream)
            torch.cuda.current_stream().wait_event(done)
        self.last_records = records
        if failure is not None:
            i, code, recs, u = failure
            try:
                failing = next((rc for rc in recs if rc.status), None) if recs else None
                if failing is None:
                    _lib.check(code, u.handle)
                self.scheme._raise(code, failing, _PlanRef(u.handle))
            except Exception as error:  # the reference's exception for the failing stage
                raise EnsembleError(i, error) from error
        for u in enqueued:
            u.cur = 1 - u.cur
            for i in u.indices:
                self.t[i] += dt
                if self.scheme.sav:
                    self.r[i] = r1s[i]
        return records

    def run(self, steps: int, dt: float) -> None:
        for _ in range(steps):
            self.step(dt)

    def launches(self) -> int:
        """Kernel launches issued so far by all plans (eager steps only count
        their launches; a graph replay counts none)."""
        return sum(int(self.lib.macsav_plan_launches(u.handle)) for u in self.units)

    def diagnostics(self) -> list[dict[str, float]]:
        """``MACNavierStokes.diagnostics`` of every member's current state."""
        keys = ("kinetic", "modified_energy", "divergence_inf", "h1_seminorm_squared", "r", "angular_momentum",
                "power", "dissipation")
        out = []
        for i, m in enumerate(self.members):
            unit, _ = self._where[i]
            res = (C.c_double * 8)()
            x = self.velocity(i).contiguous()
            _lib.check(self.lib.macsav_diagnostics(unit.handle, dptr(x), float(self.r[i]), float(m.nu), None, res,
                                                   stream_handle()), unit.handle)
            out.append(dict(zip(keys, (float(v) for v in res))))
        return out


class _PlanRef:
    """The ``plan.handle`` view that ``FusedScheme._raise`` expects."""

    def __init__(self, handle) -> None:
        self.handle = handle
