"""Learned correction of the pressure preconditioner (flexible Schur CG).

The reference solves the pressure Schur system with SciPy's PCG and the
spectral preconditioner ``m (D D^T)^+ + k I`` (tensor_stokes.py:217-243,
313-321); it has nothing learned.  Here a small bias-free BF16 U-Net
(``UNet``, CUDA forward/backward kernels in ``csrc/unet.cu``) learns what the
spectral preconditioner misses (the wall commutator of ``S``):

    z = M r + s(r) net(r / rms(r)),   s(r) = rms(r) (r.Mr) / (r.r),

projected to mean zero, inside flexible CG (Polak-Ribiere beta) in the FP32
inner solves of the mixed-precision Stokes solve.  Training pairs come from
plain FP64 Schur CG itself: for every iteration k of a logged solve, the
residual r_k and the exact error p* - p_k of the iterate (which solves
S e = r_k); the target is that error minus M r_k, in the units above.

Plain PCG stays the fallback and the gates stay in charge: a column whose learned attempt
does not converge within ``learned_max_iterations`` restarts plain PCG from
zero, and the FP64 defect correction and the reference's closing gates decide
as before, so the network never changes the answer beyond the tolerance.

Placement (``placement``): by default the network shapes only the first
search direction of each Stokes solve (the first iteration of its first FP32
inner solve, whose right-hand side is the stage's own); the other iterations
are flexible CG with the spectral preconditioner.  It may work on the
residual restricted to a coarser grid (f x f cell means), its output
prolonged bilinearly.  ``calibrate_gain`` sets the network's output gain with
plain PCG as the judge, on held-out solves.

What it can gain is bounded by what the spectral preconditioner leaves: at
the workloads' shifts (k / h^2 of order 1e-3) one PCG iteration already
takes a smooth right-hand side to a relative residual near 2e-5, below the
inner solves' tolerance, and a correction only shortens a solve if its own
error (in the Schur norm) is below that, which a BF16 network with 8-bit
mantissas does not reach.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .grid import MACGrid
from .stokes import Plan, dptr, stream_handle

DEFAULT_CHANNELS = (16, 32, 64, 64)


def layer_shapes(channels=DEFAULT_CHANNELS) -> list[tuple[int, int, int]]:
    """(c_out, c_in, k) of the 12 layers in parameter order (csrc/unet.cu)."""
    c0, c1, c2, c3 = channels
    return [(c0, 1, 3), (c0, c0, 3), (c1, c0, 3), (c1, c1, 3), (c2, c1, 3), (c2, c2, 3), (c3, c2, 3), (c3, c3, 3),
            (c2, c3 + c2, 3), (c1, c2 + c1, 3), (c0, c1 + c0, 3), (1, c0, 1)]


class UNet:
    """Owns one ``macsav_unet`` (weights, Adam state, workspace) on the GPU."""

    def __init__(self, channels=DEFAULT_CHANNELS, seed: int = 0, output_gain: float = 1e-2) -> None:
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (the GB300 library has no CPU fallback)")
        self.lib = _lib.load()
        self.channels = tuple(int(c) for c in channels)
        handle = C.c_void_p()
        arr = (C.c_int * 4)(*self.channels)
        torch.cuda.init()
        code = self.lib.macsav_unet_create(C.byref(handle), arr)
        if code != _lib.OK:
            raise ValueError(self.lib.macsav_unet_error(None).decode())
        self.handle = handle
        self.tensor_cores = True  # the library default: 3x3 forward convolutions on tcgen05
        self.set_params(self.initial_params(seed, output_gain))

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.macsav_unet_destroy(h)
            self.handle = None

    def set_tensor_cores(self, enable: bool) -> None:
        """Forward 3x3 convolutions on the tcgen05 tensor cores (or the CUDA cores)."""
        self._check(self.lib.macsav_unet_set_tensor_cores(self.handle, 1 if enable else 0))
        self.tensor_cores = bool(enable)

    def _check(self, code: int) -> None:
        if code != _lib.OK:
            msg = self.lib.macsav_unet_error(self.handle).decode()
            if code in (_lib.ERR_VALUE, _lib.ERR_UNSUPPORTED):
                raise ValueError(msg)
            raise _lib.MacsavError(msg or f"macsav error code {code}")

    @property
    def num_params(self) -> int:
        return int(self.lib.macsav_unet_num_params(self.handle))

    def initial_params(self, seed: int, output_gain: float) -> np.ndarray:
        """He-normal weights; the output layer scaled by ``output_gain`` so an
        untrained network starts close to the plain preconditioner."""
        rng = np.random.default_rng(seed)
        parts = []
        shapes = layer_shapes(self.channels)
        for idx, (co, ci, k) in enumerate(shapes):
            w = rng.normal(0.0, np.sqrt(2.0 / (ci * k * k)), size=co * ci * k * k)
            if idx == len(shapes) - 1:
                w *= output_gain
            parts.append(w)
        return np.concatenate(parts).astype(np.float32)

    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        self._check(self.lib.macsav_unet_get_params(self.handle, out.ctypes.data_as(C.c_void_p)))
        return out

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        self._check(self.lib.macsav_unet_set_params(self.handle, p.ctypes.data_as(C.c_void_p)))

    @staticmethod
    def _dev(x) -> torch.Tensor:
        t = x if isinstance(x, torch.Tensor) else torch.from_numpy(np.asarray(x))
        return t.to(device="cuda", dtype=torch.float32).contiguous()

    def forward(self, x) -> torch.Tensor:
        """x: [batch, ny, nx] -> net(x), FP32 on the device."""
        x = self._dev(x)
        b, ny, nx = x.shape
        out = torch.empty_like(x)
        self._check(self.lib.macsav_unet_forward(self.handle, dptr(x), b, ny, nx, dptr(out), stream_handle()))
        return out

    def gradients(self, x, target) -> tuple[float, np.ndarray]:
        """Mean squared error against ``target`` and its parameter gradient."""
        x, t = self._dev(x), self._dev(target)
        b, ny, nx = x.shape
        grads = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.macsav_unet_gradients(self.handle, dptr(x), dptr(t), b, ny, nx, C.byref(loss),
                                                   grads.ctypes.data_as(C.c_void_p), stream_handle()))
        return float(loss.value), grads

    def train_step(self, x, target, lr: float) -> float:
        x, t = self._dev(x), self._dev(target)
        b, ny, nx = x.shape
        loss = C.c_double()
        self._check(self.lib.macsav_unet_train_step(self.handle, dptr(x), dptr(t), b, ny, nx, float(lr),
                                                    C.byref(loss), stream_handle()))
        return float(loss.value)


@dataclass
class Pairs:
    """Normalised training pairs on one grid: inputs r/rms(r) and targets
    (e - M r)/s(r), [n, ny, nx] FP32 on the device."""
    inputs: torch.Tensor
    targets: torch.Tensor
    iterations: list[int]


def collect_pairs(grid: MACGrid, rhs_columns, mass: float, viscosity: float, *, max_pairs: int = 64,
                  krylov_tolerance: float = 1e-12, min_relative_residual: float = 1e-7) -> Pairs:
    """Log plain FP64 Schur CG on each RHS and turn every iteration into a pair."""
    plan = Plan(grid, "fp64", 1e-9, krylov_tolerance, 100, 2)
    lib = plan.lib
    np_ = grid.np
    logs = [torch.empty((max_pairs + 1) * np_, dtype=torch.float64, device="cuda") for _ in range(3)]
    inputs, targets, iters = [], [], []
    for rhs in rhs_columns:
        f = torch.as_tensor(np.ascontiguousarray(rhs, dtype=np.float64), device="cuda")
        n = C.c_int()
        plan.check(lib.macsav_stokes_log(plan.handle, dptr(f), float(mass), float(viscosity), max_pairs,
                                         dptr(logs[0]), dptr(logs[1]), dptr(logs[2]), C.byref(n), stream_handle()))
        k = int(n.value)
        iters.append(k)
        r = logs[0][:k * np_].reshape(k, np_)
        z = logs[1][:k * np_].reshape(k, np_)
        x = logs[2][:(k + 1) * np_].reshape(k + 1, np_)
        e = x[k][None, :] - x[:k]
        t = e - z
        t = t - t.mean(dim=1, keepdim=True)
        rr = (r * r).sum(dim=1)
        keep = rr.sqrt() > min_relative_residual * rr[0].sqrt()
        rms = (rr / np_).sqrt()
        scale = rms * (r * z).sum(dim=1) / rr
        inputs.append((r / rms[:, None])[keep])
        targets.append((t / scale[:, None])[keep])
    shape = (-1, grid.ny, grid.nx)
    return Pairs(torch.cat(inputs).reshape(shape).float().contiguous(),
                 torch.cat(targets).reshape(shape).float().contiguous(), iters)


def train(net: UNet, pairs: Pairs, *, steps: int = 200, batch: int = 8, lr: float = 1e-3, seed: int = 0) -> list[float]:
    """Adam on random mini-batches of the pairs; returns the loss per step."""
    gen = torch.Generator().manual_seed(seed)
    n = pairs.inputs.shape[0]
    losses = []
    for _ in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), generator=gen).to("cuda")
        losses.append(net.train_step(pairs.inputs[idx].contiguous(), pairs.targets[idx].contiguous(), lr))
    return losses


def collect_first_direction_pairs(grid: MACGrid, rhs_columns, mass: float, viscosity: float, *,
                                  restriction: int = 1, krylov_tolerance: float = 1e-12) -> Pairs:
    """Pairs for the first-direction placement: for each right-hand side, the
    pressure right-hand side b of plain FP64 Schur CG (its first residual) and
    the error of the spectral preconditioner's first direction, p* - M b, in
    the units of ``collect_pairs``; both restricted by f x f cell means when
    ``restriction`` f > 1 (the network then works on the restricted grid)."""
    plan = Plan(grid, "fp64", 1e-9, krylov_tolerance, 100, 2)
    lib = plan.lib
    np_ = grid.np
    logs = [torch.empty(2 * np_, dtype=torch.float64, device="cuda") for _ in range(3)]
    inputs, targets, iters = [], [], []
    for rhs in rhs_columns:
        f = torch.as_tensor(np.ascontiguousarray(rhs, dtype=np.float64), device="cuda")
        n = C.c_int()
        # the log keeps one pair (k = 0) and the converged iterate (row 1 of x)
        plan.check(lib.macsav_stokes_log(plan.handle, dptr(f), float(mass), float(viscosity), 1,
                                         dptr(logs[0]), dptr(logs[1]), dptr(logs[2]), C.byref(n), stream_handle()))
        k = int(n.value)
        iters.append(k)
        if k < 1:
            continue
        b, mb, xs = logs[0][:np_], logs[1][:np_], logs[2][np_:2 * np_]
        rr = float((b * b).sum())
        rms = (rr / np_) ** 0.5
        scale = rms * float((b * mb).sum()) / rr
        t = xs - mb
        t = t - t.mean()
        inputs.append((b / rms).reshape(1, 1, grid.ny, grid.nx))
        targets.append((t / scale).reshape(1, 1, grid.ny, grid.nx))
    x, y = torch.cat(inputs), torch.cat(targets)
    if restriction > 1:
        x = torch.nn.functional.avg_pool2d(x, restriction)
        y = torch.nn.functional.avg_pool2d(y, restriction)
    return Pairs(x[:, 0].float().contiguous(), y[:, 0].float().contiguous(), iters)


def scale_output(net: UNet, gain: float) -> None:
    """Multiply the network's output by ``gain`` (the bias-free network is
    linear in its last layer's weights)."""
    p = net.params()
    co, ci, k = layer_shapes(net.channels)[-1]
    n_last = co * ci * k * k
    p[-n_last:] *= np.float32(gain)
    net.set_params(p)


def calibrate_gain(net: UNet, grid: MACGrid, rhs_columns, mass: float, viscosity: float, *,
                   gains=(0.0, 0.25, 0.5, 1.0), restriction: int = 1, krylov_tolerance: float = 1e-10,
                   max_columns: int = 2) -> dict:
    """Choose the output gain of the network with plain PCG as the judge: for
    every candidate gain, the FP32 Stokes solves of the held-out right-hand
    sides (two columns per solve) with the network in the first-direction
    placement, counting all inner CG iterations; the gain kept is the largest
    one that needs no more iterations than the smallest count (gain 0 is plain
    PCG's count).  The network's last layer is scaled by that gain; returns
    the counts per gain and the choice."""
    from .stokes import TensorStokes
    base = net.params()
    counts = {}
    for gain in gains:
        net.set_params(base)
        scale_output(net, gain)
        ts = TensorStokes(grid, precision="fp32", krylov_tolerance=krylov_tolerance, max_columns=max_columns)
        attach(ts, net)
        placement(ts, every_iteration=False, restriction=restriction)
        total = 0
        for cols in rhs_columns:
            ts.solve(cols, mass=mass, viscosity=viscosity)
            total += sum(cg_counters(ts, cols.shape[1])["iterations"])
        counts[float(gain)] = total
        attach(ts, None)
    best = min(counts.values())
    chosen = max(g for g, c in counts.items() if c == best)
    net.set_params(base)
    scale_output(net, chosen)
    return {"iterations_per_gain": counts, "gain": chosen}


def placement(backend, *, every_iteration: bool = False, restriction: int = 1) -> None:
    """Where the attached network runs: the first search direction of each
    Stokes solve (default) or every CG iteration; on the residual restricted
    by f x f cell means (``restriction`` 1, 2, 4 or 8)."""
    backend = getattr(backend, "backend", backend)
    plan = backend.plan
    plan.check(plan.lib.macsav_plan_set_learned_placement(plan.handle, 1 if every_iteration else 0,
                                                          int(restriction)))


def attach(backend, net: UNet | None, learned_max_iterations: int = 20) -> None:
    """Use ``net`` in the FP32 inner solves of an FP32 ``TensorStokes`` (or a
    model's backend); ``None`` detaches it."""
    backend = getattr(backend, "backend", backend)
    plan = backend.plan
    plan.check(plan.lib.macsav_plan_set_preconditioner(plan.handle, net.handle if net is not None else None,
                                                       int(learned_max_iterations)))
    backend.learned = net  # keeps the network alive while the plan points at it


def cg_counters(backend, columns: int = 1) -> dict[str, list[int]]:
    """Per-column CG iterations of the last solve: all inner iterations, those
    run with the network, and plain-PCG restarts."""
    backend = getattr(backend, "backend", backend)
    plan = backend.plan
    it, lt, fb = (C.c_int * columns)(), (C.c_int * columns)(), (C.c_int * columns)()
    plan.check(plan.lib.macsav_plan_cg_counters(plan.handle, columns, it, lt, fb))
    return {"iterations": list(it), "learned_iterations": list(lt), "fallbacks": list(fb)}
