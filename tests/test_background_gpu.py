"""The render composition's background composite (renderer.py:779-781,
804-806): the operator against the oracle and against FP64 central
differences, and the fused step with a background against the oracle's
composition."""
import numpy as np
import pytest
import torch

from oracle import ops as oops
from oracle import parallel

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("C", [2, 4])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_composite_matches_oracle(C, dtype):
    from ngt_gb300 import ops
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(31 + C)
    img = rng.uniform(0.0, 2.0, (2, 3, 9, 7, C)).astype(dtype)
    bkg = rng.uniform(0.0, 1.0, (3, 9, 7, C - 1)).astype(dtype)
    g = rng.standard_normal((2, 3, 9, 7, C - 1)).astype(dtype)
    ti = torch.as_tensor(img, device=dev).requires_grad_()
    tb = torch.as_tensor(bkg, device=dev).requires_grad_()
    out = ops.background_composite(ti, tb)
    tol = 1e-6 if dtype == np.float32 else 1e-13
    assert rel(out, oops.background_composite(img, bkg)) < tol
    out.backward(torch.as_tensor(g, device=dev))
    gi, gb = oops.background_composite_grad(img, bkg, g)
    assert rel(ti.grad, gi) < tol
    assert rel(tb.grad, gb) < tol


def test_composite_finite_differences():
    from ngt_gb300 import ops
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    img = torch.as_tensor(rng.uniform(0.0, 2.0, (1, 2, 4, 3, 2)), device=dev).requires_grad_()
    bkg = torch.as_tensor(rng.uniform(0.0, 1.0, (2, 4, 3, 1)), device=dev).requires_grad_()
    assert torch.autograd.gradcheck(ops.background_composite, (img, bkg), eps=1e-6, atol=1e-9, rtol=1e-6)


def test_step_with_background_matches_oracle():
    """The fused step with the background composited in its loss epilogue
    against the oracle's composition (warp, render, composite, L2, backward)."""
    from ngt_gb300 import workloads
    from ngt_gb300.step import RenderAdvectStep
    w = workloads.render_step(grid=(24, 28, 20), views=3, image=(32, 24), depth=28, max_u=1.5)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(8)
    bkg = rng.uniform(0.0, 0.3, (w.views, 32, 24, 1)).astype(np.float32)
    p, n = parallel.make_pool(4)
    try:
        img_t, _, _ = parallel.render_l2(p, n, w.rho_target, w.depth_step, w.M, w.V, w.P, w.F, w.image_dhw)
        tgt = np.ascontiguousarray(oops.background_composite(img_t, bkg))
        image, ref_loss, ref = parallel.render_advect_step(p, n, w.rho, w.ux, w.uy, w.uz, w.M, w.V, w.P, w.F, tgt,
                                                           w.image_dhw, w.depth_step, background=bkg)
    finally:
        p.close()
        p.join()
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    step = RenderAdvectStep(T(w.rho), T(w.ux), T(w.uy), T(w.uz), w.M, w.V, w.P, w.F, T(tgt), w.image_dhw,
                            background=T(bkg))
    loss = float(step.step().item())
    assert rel(step.image, image) < 1e-5
    assert abs(loss - ref_loss) <= 1e-5 * abs(ref_loss)
    for a, b in zip(step.gradients(), ref):
        assert rel(a, b) < 1e-4
    # the background changes the loss and the gradients
    plain = RenderAdvectStep(T(w.rho), T(w.ux), T(w.uy), T(w.uz), w.M, w.V, w.P, w.F, T(tgt), w.image_dhw)
    assert abs(float(plain.step().item()) - loss) > 1e-3 * loss
