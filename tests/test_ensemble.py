"""Ensembles of cavities: member draw and sharding (CPU, including a two-rank
gloo run), and the concurrent GPU step against lone steps of the same members."""
import os
import socket

import numpy as np
import pytest

from helpers import load_package


def _ens():
    from importlib import import_module
    return import_module(load_package().__name__ + ".ensemble")


def test_members_are_seeded_and_in_range():
    E = _ens()
    a, b = E.ensemble_members(256, seed=3), E.ensemble_members(256, seed=3)
    assert a == b and a != E.ensemble_members(256, seed=4)
    assert {m.nx for m in a} <= set(E.SIZES) and {m.ny for m in a} <= set(E.SIZES)
    assert len({m.nx for m in a}) == len(E.SIZES)          # every size drawn at this count
    assert any(m.nx != m.ny for m in a)                      # rectangles included
    nus = np.array([m.nu for m in a])
    assert nus.min() >= 1e-4 and nus.max() <= 1e-2
    assert len({m.seed for m in a}) == 256
    assert a[0].grid().lx == pytest.approx(a[0].nx / a[0].ny) and a[0].grid().ly == 1.0


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shards_are_disjoint_cover_and_balanced(world):
    E = _ens()
    members = E.ensemble_members(256, seed=1)
    shards = [E.shard_members(members, world, r) for r in range(world)]
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(256))
    loads = [sum(members[i].cells for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(m.cells for m in members)
    with pytest.raises(ValueError):
        E.shard_members(members, world, world)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    E = _ens()
    members = E.ensemble_members(64, seed=9)
    mine = E.shard_members(members, world, rank)
    # each rank reports per-member host results; rank 0 gathers them (no device data moves)
    gathered = [None] * world
    dist.all_gather_object(gathered, {i: members[i].cells for i in mine})
    if rank == 0:
        with open(out, "w") as f:
            f.write(repr(gathered))
    dist.destroy_process_group()


def test_two_rank_gloo_sharding(tmp_path):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "gathered.txt")
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    gathered = eval(open(out).read())
    keys = [set(g) for g in gathered]
    assert not keys[0] & keys[1] and keys[0] | keys[1] == set(range(64))
    E = _ens()
    members = E.ensemble_members(64, seed=9)
    assert all(g[i] == members[i].cells for g in gathered for i in g)


# ----------------------------------------------------------------- GPU ---

@pytest.mark.gpu
@pytest.mark.parametrize("batched", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ensemble_step_equals_lone_steps(precision, batched):
    import torch
    pkg = load_package()
    E = _ens()
    members = [E.Member(64, 96, 3e-3, 11), E.Member(96, 64, 2e-4, 12), E.Member(128, 128, 8e-3, 13),
               E.Member(64, 96, 9e-4, 14), E.Member(64, 96, 1e-2, 15)]
    ens = E.Ensemble(members, "sdirk2_mrsav", precision=precision, batched=batched)
    assert len(ens.units) == (3 if batched else 5)
    ens.seed_fields(modes=8)
    x0 = [ens.velocity(i).clone() for i in range(len(members))]
    for _ in range(3):
        ens.step(5e-4)
    scheme = pkg.make_scheme("sdirk2_mrsav")
    for i, m in enumerate(members):
        model = pkg.MACNavierStokes(m.grid(), m.nu, precision=precision, use_graph=True)
        state = model.state(0.0, x0[i], 1.0)
        for _ in range(3):
            state = scheme.step(model, state, 5e-4).state
        assert torch.equal(model.device_vector(state), ens.velocity(i))
        assert state.r == ens.r[i] and state.t == pytest.approx(ens.t[i])
    d = ens.diagnostics()
    assert all(np.isfinite(list(x.values())).all() and x["divergence_inf"] < 1e-8 for x in d)


@pytest.mark.gpu
def test_host_buffers_upload_download_round_trip():
    """All members' states in and out through the ensemble's pinned host
    block (one kernel each way): bitwise the per-member copies, at both slot
    parities, and a step from uploaded states equals one from set_state."""
    import torch
    E = _ens()
    members = [E.Member(64, 96, 3e-3, 11), E.Member(96, 64, 2e-4, 12), E.Member(64, 96, 9e-4, 14)]
    a = E.Ensemble(members, "sdirk2_mrsav", precision="fp64")
    b = E.Ensemble(members, "sdirk2_mrsav", precision="fp64")
    a.seed_fields(modes=6)
    bufs = a.host_buffers()
    assert [v.size for v in bufs] == [m.grid().size for m in members]
    assert a.host_buffers()[0] is bufs[0]                     # allocated once
    assert torch.from_numpy(bufs[0]).is_pinned()
    for parity in range(2):
        out = a.download()
        for i in range(len(members)):
            np.testing.assert_array_equal(out[i], a.velocity(i).cpu().numpy())
        rng = np.random.default_rng(parity)
        for v in bufs:
            v[:] = rng.standard_normal(v.size) * 1e-2
        a.upload(r=[1.0] * 3, t=[0.0] * 3)
        for i in range(len(members)):
            np.testing.assert_array_equal(a.velocity(i).cpu().numpy(), bufs[i])
            b.set_state(i, bufs[i].copy(), r=1.0, t=0.0)
        a.step(5e-4)
        b.step(5e-4)
        for i in range(len(members)):
            assert torch.equal(a.velocity(i), b.velocity(i))
    with pytest.raises(ValueError):
        a.upload(r=[1.0])


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["sdirk3_mrsav", "sdirk2"])
def test_batched_plan_matches_single_member_plans(scheme):
    """Members sharing a plan (one launch per kernel for all of them) give
    bitwise the results of one plan per member, eager and graph."""
    import torch
    E = _ens()
    members = [E.Member(96, 64, nu, 40 + k) for k, nu in enumerate((1e-4, 3e-4, 1e-3, 3e-3, 1e-2))]
    runs = []
    for batched, graph in ((True, False), (True, True), (False, True)):
        ens = E.Ensemble(members, scheme, precision="fp32", batched=batched, use_graph=graph)
        ens.seed_fields(modes=8)
        ens.run(2, 5e-4)
        runs.append((ens, [ens.velocity(i).clone() for i in range(len(members))]))
    for ens, xs in runs[1:]:
        for a, b in zip(runs[0][1], xs):
            assert torch.equal(a, b)
        np.testing.assert_array_equal(ens.r, runs[0][0].r)
    assert runs[0][0].launches() > 0


@pytest.mark.gpu
def test_ensemble_fp32_against_fp64_and_failure_names_member():
    import torch
    E = _ens()
    members = E.ensemble_members(6, seed=2)
    e64 = E.Ensemble(members, precision="fp64")
    e32 = E.Ensemble(members, precision="fp32")
    for e in (e64, e32):
        e.seed_fields(modes=8)
        e.run(4, 5e-4)
    for i in range(len(members)):
        a, b = e64.velocity(i), e32.velocity(i)
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(a)) < 1e-9
    bad = e32.velocity(3).clone()
    bad[7] = float("nan")
    e32.set_state(3, bad, r=e32.r[3], t=e32.t[3])
    before = [e32.velocity(i).clone() for i in range(len(members))]
    with pytest.raises(E.EnsembleError) as info:
        e32.step(5e-4)
    assert info.value.index == 3 and isinstance(info.value.__cause__, (ValueError, RuntimeError))
    assert all(torch.equal(before[i], e32.velocity(i)) for i in range(len(members)) if i != 3)
