"""The reconstruction step's loss as one differentiable call
(``step.render_advect_loss``) against the same composition of the separate
autograd operators, across calls with new inputs, an upstream gradient scale,
and two forwards before their backwards."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = a.detach().double(), b.detach().double()
    return float((a - b).norm() / b.norm())


def inputs(seed, dev):
    from ngt_gb300 import workloads
    w = workloads.render_step(grid=(24, 28, 20), views=2, image=(24, 20), depth=24, max_u=1.5, density_seed=seed)
    return w, [torch.as_tensor(a, device=dev) for a in (w.rho, w.ux, w.uy, w.uz)]


def composed(ts, w, tgt):
    from ngt_gb300 import advect, ops
    xs = [t.clone().requires_grad_() for t in ts]
    r2 = advect.warp(*xs, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
    img = ops.raymarch_grid_transform(r2[None], w.M, w.V, w.P, w.F, w.image_dhw,
                                      emission_scale=(w.depth_step, w.depth_step))
    loss = ops.image_l2_loss(img, tgt)
    loss.backward()
    return loss, [x.grad for x in xs]


def test_fused_loss_matches_operator_composition():
    from ngt_gb300.step import render_advect_loss
    dev = torch.device("cuda", 0)
    w, ts = inputs(0, dev)
    tgt = torch.zeros((1, 2, 24, 20, 1), device=dev) + 0.01
    for seed in (0, 3):  # a second call with new inputs reuses the kept buffers
        w2, ts = inputs(seed, dev)
        want_loss, want = composed(ts, w2, tgt)
        xs = [t.clone().requires_grad_() for t in ts]
        loss = render_advect_loss(*xs, w2.M, w2.V, w2.P, w2.F, tgt, w2.image_dhw)
        (2.5 * loss).backward()
        assert abs(float(loss) - float(want_loss)) <= 1e-5 * abs(float(want_loss))
        for x, g in zip(xs, want):
            assert rel(x.grad, 2.5 * g) < 1e-4


def test_two_forwards_before_backward():
    from ngt_gb300.step import render_advect_loss
    dev = torch.device("cuda", 0)
    w, ta = inputs(1, dev)
    _, tb = inputs(2, dev)
    tgt = torch.zeros((1, 2, 24, 20, 1), device=dev) + 0.01
    xa = [t.clone().requires_grad_() for t in ta]
    xb = [t.clone().requires_grad_() for t in tb]
    la = render_advect_loss(*xa, w.M, w.V, w.P, w.F, tgt, w.image_dhw)
    lb = render_advect_loss(*xb, w.M, w.V, w.P, w.F, tgt, w.image_dhw)
    (la + lb).backward()
    _, ga = composed(ta, w, tgt)
    _, gb = composed(tb, w, tgt)
    for x, g in zip(xa, ga):
        assert rel(x.grad, g) < 1e-4
    for x, g in zip(xb, gb):
        assert rel(x.grad, g) < 1e-4


def test_graph_replay_reads_current_data():
    """Calls at the same tensor addresses run directly, then as captured graphs:
    every call, with the tensors refilled in place, matches the composition."""
    from ngt_gb300.step import render_advect_loss
    dev = torch.device("cuda", 0)
    tgt = torch.zeros((1, 2, 24, 20, 1), device=dev) + 0.01
    w, ts0 = inputs(4, dev)
    _, ts1 = inputs(5, dev)
    xs = [t.clone().requires_grad_() for t in ts0]
    for it in range(5):
        src = ts0 if it % 2 == 0 else ts1
        with torch.no_grad():
            for x, t in zip(xs, src):
                x.copy_(t)
                x.grad = None
        loss = render_advect_loss(*xs, w.M, w.V, w.P, w.F, tgt, w.image_dhw)
        loss.backward()
        want_loss, want = composed(src, w, tgt)
        assert abs(float(loss) - float(want_loss)) <= 1e-5 * abs(float(want_loss)), it
        for x, g in zip(xs, want):
            assert rel(x.grad, g) < 1e-4, it


def test_cameras_changed_in_place_take_effect():
    """Camera matrices updated in place between calls (the same array objects)
    render with their new values: the loss is that of the operator composition
    with the moved cameras, not a step kept for the old ones."""
    from ngt_gb300.step import render_advect_loss
    dev = torch.device("cuda", 0)
    w, ts = inputs(4, dev)
    tgt = torch.zeros((1, 2, 24, 20, 1), device=dev) + 0.01
    M, V, P, F = (np.array(m, np.float32) for m in (w.M, w.V, w.P, w.F))
    first = float(render_advect_loss(*ts, M, V, P, F, tgt, w.image_dhw))
    V[:, 12:15] += np.float32(0.35)  # every camera shifted, in place
    second = float(render_advect_loss(*ts, M, V, P, F, tgt, w.image_dhw))
    w.M, w.V, w.P, w.F = M.copy(), V.copy(), P.copy(), F.copy()
    want, _ = composed(ts, w, tgt)
    assert abs(second - float(want)) <= 1e-5 * abs(float(want))
    assert abs(second - first) > 1e-3 * abs(first)


def test_deterministic_loss_repeats_bits():
    """With ops.set_deterministic(True) the one-node loss takes the fixed-point
    adjoints: the same gradient bits on every call, and the operator
    composition's gradients to the float tolerance."""
    from ngt_gb300 import ops
    from ngt_gb300.step import render_advect_loss
    dev = torch.device("cuda", 0)
    w, ts = inputs(6, dev)
    tgt = torch.zeros((1, 2, 24, 20, 1), device=dev) + 0.01
    _, want = composed(ts, w, tgt)
    runs = []
    ops.set_deterministic(True)
    try:
        for _ in range(2):
            xs = [t.clone().requires_grad_() for t in ts]
            render_advect_loss(*xs, w.M, w.V, w.P, w.F, tgt, w.image_dhw).backward()
            runs.append([x.grad for x in xs])
    finally:
        ops.set_deterministic(False)
    for a, b, g in zip(runs[0], runs[1], want):
        assert torch.equal(a, b)
        assert rel(a, g) < 1e-4
