"""Learned preconditioner: CUDA U-Net kernels against a PyTorch CPU oracle
(forward and gradients), training on pairs logged by plain Schur CG, and
flexible CG that keeps the plain solve's answer, falls back when the network
is bad, and reports what the trained network gains."""
import numpy as np
import pytest

from helpers import load_package
import unet_torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from importlib import import_module
    pkg = load_package()
    L = import_module(pkg.__name__ + ".learned")
    return pkg, L, torch


def test_param_count_and_layout(env):
    pkg, L, torch = env
    net = L.UNet()
    shapes = L.layer_shapes()
    assert net.num_params == sum(co * ci * k * k for co, ci, k in shapes)
    assert 1.5e5 < net.num_params < 3e5
    p = net.params()
    np.testing.assert_array_equal(p, net.initial_params(0, 1e-2))


def test_forward_matches_torch_oracle(env):
    pkg, L, torch = env
    net = L.UNet(seed=3, output_gain=1.0)
    x = torch.randn(2, 32, 48, generator=torch.Generator().manual_seed(1))
    got = net.forward(x).cpu()
    ref = unet_torch.forward(unet_torch.split_params(net.params(), L.layer_shapes()), x).detach()
    err = float((got - ref).norm() / ref.norm())
    print("forward relative error against the oracle: %.1e" % err)
    assert err < 1e-2, err
    # positive homogeneity of the bias-free ReLU network
    got2 = net.forward(4.0 * x).cpu()
    assert float((got2 - 4.0 * got).norm() / got.norm().mul(4)) < 2e-2


def test_gradients_match_torch_autograd(env):
    pkg, L, torch = env
    net = L.UNet(seed=5, output_gain=1.0)
    gen = torch.Generator().manual_seed(2)
    x = torch.randn(3, 16, 24, generator=gen)
    t = torch.randn(3, 16, 24, generator=gen)
    loss, grads = net.gradients(x, t)
    ws = [w.requires_grad_(True) for w in unet_torch.split_params(net.params(), L.layer_shapes())]
    ref_loss = ((unet_torch.forward(ws, x) - t) ** 2).mean()
    ref_loss.backward()
    ref = torch.cat([w.grad.reshape(-1) for w in ws]).numpy()
    assert loss == pytest.approx(float(ref_loss.detach()), rel=1e-2)
    rel = np.linalg.norm(grads - ref) / np.linalg.norm(ref)
    cos = float(grads @ ref / (np.linalg.norm(grads) * np.linalg.norm(ref)))
    # every layer's gradient: the oracle rounds the same activations to BF16,
    # so what is left is FP32 summation order and the odd activation that
    # rounds to the other BF16 neighbour
    off, per_layer = 0, []
    for co, ci, k in L.layer_shapes():
        n = co * ci * k * k
        g, r = grads[off:off + n], ref[off:off + n]
        per_layer.append(float(np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)))
        off += n
    print("gradient relative error per layer:", ["%.1e" % e for e in per_layer], "overall %.1e" % rel)
    assert rel < 1e-2 and cos > 0.9999, (rel, cos)
    assert max(per_layer) < 1e-2, per_layer


def _stage_rhs(pkg, grid, seeds, torch):
    """Stage-like Stokes right-hand sides: seeded curl fields and their convection."""
    out = []
    model = pkg.MACNavierStokes(grid, 1e-3)
    for s in seeds:
        x = pkg.fields.packed_curl_velocity(grid.nx, grid.ny, grid.lx, grid.ly, 8, s)
        out.append(x)
        out.append(model.nonlinear(x).cpu().numpy() * 1e-3)
    return out


def _trained(env, grid, steps=300):
    pkg, L, torch = env
    shift = (1.0, 1e-3 * 2.5e-4 * 0.4358665215)
    pairs = L.collect_pairs(grid, _stage_rhs(pkg, grid, range(6), torch), *shift)
    net = L.UNet(seed=0)
    losses = L.train(net, pairs, steps=steps, batch=8, lr=1e-3)
    return net, pairs, losses, shift


def test_pairs_and_training(env):
    pkg, L, torch = env
    grid = pkg.MACGrid(64, 64)
    net, pairs, losses, _ = _trained(env, grid)
    assert pairs.inputs.shape[1:] == (64, 64) and pairs.inputs.shape == pairs.targets.shape
    assert min(pairs.iterations) >= 2
    rms = pairs.inputs.pow(2).mean(dim=(1, 2)).sqrt()
    assert torch.allclose(rms, torch.ones_like(rms), rtol=1e-5)
    assert np.isfinite(losses).all()
    assert np.mean(losses[-20:]) < 0.7 * np.mean(losses[:5])


def test_flexible_cg_keeps_answer_and_falls_back(env):
    pkg, L, torch = env
    grid = pkg.MACGrid(64, 64)
    net, pairs, _, shift = _trained(env, grid, steps=150)
    rhs = np.column_stack(_stage_rhs(pkg, grid, [101], torch))
    plain = pkg.TensorStokes(grid, precision="fp32")
    base = plain.solve(rhs, mass=shift[0], viscosity=shift[1])
    learned = pkg.TensorStokes(grid, precision="fp32")
    L.attach(learned, net)
    res = learned.solve(rhs, mass=shift[0], viscosity=shift[1])
    cnt = L.cg_counters(learned, 2)
    assert sum(cnt["learned_iterations"]) > 0
    for a, b in ((res.velocity, base.velocity), (res.pressure, base.pressure)):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)
    assert res.residual <= 1e-9 and base.residual <= 1e-9
    # a deliberately bad network in every iteration: the learned attempt
    # fails, plain PCG restarts
    bad = L.UNet(seed=9, output_gain=1e4)
    L.attach(learned, bad, learned_max_iterations=2)
    L.placement(learned, every_iteration=True)
    res_bad = learned.solve(rhs, mass=shift[0], viscosity=shift[1])
    cnt_bad = L.cg_counters(learned, 2)
    assert sum(cnt_bad["fallbacks"]) > 0
    assert np.linalg.norm(res_bad.velocity - base.velocity) <= 1e-8 * np.linalg.norm(base.velocity)
    L.attach(learned, None)
    again = learned.solve(rhs, mass=shift[0], viscosity=shift[1])
    assert L.cg_counters(learned, 2)["learned_iterations"] == [0, 0]
    np.testing.assert_allclose(again.velocity, base.velocity, rtol=0, atol=1e-12 * np.abs(base.velocity).max())


def _first_direction_net(env, grid, shift, restriction):
    pkg, L, torch = env
    rhs = [c for c in _stage_rhs(pkg, grid, range(12), torch)]
    pairs = L.collect_first_direction_pairs(grid, rhs, *shift, restriction=restriction)
    assert pairs.inputs.shape == (len(rhs), grid.ny // restriction, grid.nx // restriction)
    net = L.UNet(seed=0)
    losses = L.train(net, pairs, steps=200, batch=8, lr=1e-3)
    assert np.isfinite(losses).all()
    return net


@pytest.mark.parametrize("restriction", [1, 2, 8])
def test_first_direction_placement_keeps_answer(env, restriction):
    """The network shaping only the first search direction of each Stokes
    solve (on the full, the 2x2- or the 8x8-restricted residual): the answer is the
    plain solve's to the defect-corrected tolerance, the gates hold, and the
    network ran in the first inner solve only."""
    pkg, L, torch = env
    grid = pkg.MACGrid(64, 64)
    shift = (1.0, 2.6e-3 * grid.hx * grid.hy)  # k / h^2 of the 1024^2 case (nu dt / 4 = 2.5e-9)
    net = _first_direction_net(env, grid, shift, restriction)
    rhs = np.column_stack(_stage_rhs(pkg, grid, [77], torch))
    base = pkg.TensorStokes(grid, precision="fp32").solve(rhs, mass=shift[0], viscosity=shift[1])
    ts = pkg.TensorStokes(grid, precision="fp32")
    L.attach(ts, net)
    L.placement(ts, every_iteration=False, restriction=restriction)
    res = ts.solve(rhs, mass=shift[0], viscosity=shift[1])
    cnt = L.cg_counters(ts, 2)
    assert all(0 < li <= it for li, it in zip(cnt["learned_iterations"], cnt["iterations"]))
    for a, b in ((res.velocity, base.velocity), (res.pressure, base.pressure)):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)
    assert res.residual <= 1e-9


def test_judge_never_lets_the_network_cost_iterations(env):
    """The output gain chosen with plain PCG as the judge (held-out solves, k /
    h^2 of the 1024^2 learned case): the chosen gain needs no more inner
    iterations than plain PCG (gain 0), and the counts per gain are printed.
    What the network can gain here is bounded by what the spectral
    preconditioner leaves, measured in tests/test_learned_headroom.py."""
    pkg, L, torch = env
    grid = pkg.MACGrid(128, 128)
    shift = (1.0, 2.6e-3 * grid.hx * grid.hy)
    net = _first_direction_net(env, grid, shift, 2)
    held = [np.column_stack(_stage_rhs(pkg, grid, [s], torch)) for s in (301, 302)]
    judge = L.calibrate_gain(net, grid, held, *shift, restriction=2, krylov_tolerance=1e-10)
    counts = judge["iterations_per_gain"]
    print("inner CG iterations per output gain:", counts, "chosen gain:", judge["gain"])
    assert counts[judge["gain"]] <= counts[0.0]
    assert judge["gain"] in counts


@pytest.mark.parametrize("shape", [(2, 32, 48), (1, 64, 64), (3, 24, 40)])
def test_tensor_core_forward_matches_cuda_core_forward(env, shape):
    """The tcgen05 implicit-GEMM convolutions give the CUDA-core result (same
    BF16 operands, FP32 sums in another order) and the oracle's."""
    import time
    pkg, L, torch = env
    net = L.UNet(seed=7, output_gain=1.0)
    x = torch.randn(*shape, generator=torch.Generator().manual_seed(3))
    net.set_tensor_cores(False)
    ref = net.forward(x).cpu()
    net.set_tensor_cores(True)
    got = net.forward(x).cpu()
    err = float((got - ref).norm() / ref.norm())
    assert err < 2e-2, err
    oracle = unet_torch.forward(unet_torch.split_params(net.params(), L.layer_shapes()), x).detach()
    assert float((got - oracle).norm() / oracle.norm()) < 3e-2
    # timing of both paths on a larger batch (printed, informational)
    xb = torch.randn(4, 256, 256, generator=torch.Generator().manual_seed(4)).cuda()
    for flag in (False, True):
        net.set_tensor_cores(flag)
        net.forward(xb)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            net.forward(xb)
        torch.cuda.synchronize()
        print(f"U-Net forward 4x256x256 tensor_cores={flag}: {(time.perf_counter() - t0) / 5 * 1e3:.2f} ms")
