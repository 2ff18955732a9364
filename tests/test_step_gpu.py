"""The fused differentiated step at the 128^3 x 5-view size: FP64 central finite
differences on the GPU, FP32 parity with the oracle, and the error of BF16 /
FP16 storage against the FP64 path."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def make_step(w, dtype, tgt=None, clamp="MC_SMOOTH", inputs=None):
    from ngt_gb300 import ops
    from ngt_gb300.step import RenderAdvectStep
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev).to(dtype)
    if tgt is None:
        with torch.no_grad():
            tgt = ops.raymarch_grid_transform(torch.as_tensor(w.rho_target, device=dev, dtype=torch.float64)[None],
                                              w.M, w.V, w.P, w.F, w.image_dhw,
                                              emission_scale=(w.depth_step, w.depth_step))[..., :1]
    rho, ux, uy, uz = inputs if inputs is not None else (w.rho, w.ux, w.uy, w.uz)
    return RenderAdvectStep(T(rho), T(ux), T(uy), T(uz), w.M, w.V, w.P, w.F, tgt, w.image_dhw, clamp=clamp), tgt


def _face_density(rho, shape, axis):
    """Mean density of the two cells either side of each face (clamped at the walls)."""
    r = rho[..., 0]
    n = r.shape[axis]
    lo = torch.clamp(torch.arange(shape[axis], device=r.device) - 1, 0, n - 1)
    hi = torch.clamp(torch.arange(shape[axis], device=r.device), 0, n - 1)
    return 0.5 * (r.index_select(axis, lo) + r.index_select(axis, hi))


def _fd_errors(step, eligible, n_per, eps, seed):
    grads = [g.clone() for g in step.gradients()]
    params = [step.rho, step.ux, step.uy, step.uz]
    rng = np.random.default_rng(seed)
    errs = []
    for p, g, ok in zip(params, grads, eligible):
        gf = g.reshape(-1)
        nz = torch.nonzero((gf.abs() > 1e-12 * gf.abs().max()) & ok.reshape(-1)).reshape(-1).cpu().numpy()
        idx = rng.choice(nz, n_per, replace=False)
        scale = float(gf.abs().max())
        pf = p.view(-1)
        for i in idx:
            v = float(pf[i])
            pf[i] = v + eps
            lp = float(step.loss_only().item())
            pf[i] = v - eps
            lm = float(step.loss_only().item())
            pf[i] = v
            fd = (lp - lm) / (2 * eps)
            errs.append(abs(fd - float(gf[i])) / scale)
    return np.asarray(errs)


def test_fp64_finite_differences_config2():
    """Central differences (eps = 1e-4) of the FP64 loss at 200 voxels drawn with
    seed 3 (50 of the density, 50 of each velocity component) against the FP64
    adjoint, MacCormack with the MC_SMOOTH limiter.  The limiter is piecewise: in
    the near-empty tails (density << eps) a perturbation of eps switches its
    revert mask and the loss is not differentiable there at that scale, so the
    voxels are drawn where the (face-averaged) density is at least 1 % of its
    maximum; the unclamped test below covers every voxel."""
    from ngt_gb300 import workloads
    w = workloads.config2()
    step, _ = make_step(w, torch.float64)
    step.step()
    rho = step.rho
    thr = 1e-2 * float(rho.max())
    eligible = [rho >= thr] + [_face_density(rho, u.shape, ax) >= thr
                               for u, ax in ((step.ux, 2), (step.uy, 1), (step.uz, 0))]
    errs = _fd_errors(step, eligible, 50, 1e-4, 3)
    assert np.median(errs) < 1e-6, np.sort(errs)[-10:]
    assert np.quantile(errs, 0.95) < 1e-4, np.sort(errs)[-10:]


def test_fp64_finite_differences_config2_unclamped():
    """The same check over every voxel with a non-zero gradient, MacCormack
    without the limiter (the step is then smooth in the density and piecewise
    smooth in the velocity only at trilinear cell crossings)."""
    from ngt_gb300 import workloads
    w = workloads.config2()
    step, _ = make_step(w, torch.float64, clamp="NONE")
    step.step()
    eligible = [torch.ones_like(t, dtype=torch.bool) for t in (step.rho, step.ux, step.uy, step.uz)]
    errs = _fd_errors(step, eligible, 50, 1e-4, 3)
    assert np.median(errs) < 1e-6, np.sort(errs)[-10:]
    assert np.quantile(errs, 0.95) < 1e-4, np.sort(errs)[-10:]


def test_step_matches_oracle_fp32():
    """FP32 step at 128^3 (one 64x64 view, 128 depth samples) against the FP32
    oracle on the same inputs: image 1e-5, gradients 1e-4 relative L2."""
    from ngt_gb300 import workloads
    from oracle import advect as oadvect
    from oracle import ops as oops
    w = workloads.render_step(grid=(128, 128, 128), views=1, image=(64, 64), depth=128)
    s = np.float32(w.depth_step)
    sc = np.asarray([s, s], np.float32)
    tgt = oops.raymarch_grid_transform((w.rho_target * sc)[None], w.M, w.V, w.P, w.F, w.image_dhw)[..., :1]
    dev = torch.device("cuda", 0)
    step, _ = make_step(w, torch.float32, torch.as_tensor(tgt, device=dev))
    step.step()
    rho2 = oadvect.density_maccormack(w.rho, w.ux, w.uy, w.uz)
    x = rho2[None] * sc
    img = oops.raymarch_grid_transform(x, w.M, w.V, w.P, w.F, w.image_dhw)
    diff = img[..., :1] - tgt
    gimg = np.concatenate([diff, np.zeros_like(diff)], -1)
    gx = oops.raymarch_grid_transform_grad(x, img, gimg, w.M, w.V, w.P, w.F, w.image_dhw)
    ref = oadvect.density_maccormack_grad(w.rho, w.ux, w.uy, w.uz, (gx[0] * sc).sum(-1, keepdims=True))

    def rl2(a, b):
        a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else a
        return float(np.linalg.norm((a - b.astype(np.float64)).ravel()) / np.linalg.norm(b.ravel()))

    assert rl2(step.image, img) < 1e-5
    for a, b in zip(step.gradients(), ref):
        assert rl2(a, b) < 1e-4


@pytest.mark.parametrize("storage", [torch.bfloat16, torch.float16])
def test_reduced_precision_storage(storage):
    """Density and velocity stored in 16 bits, arithmetic in FP32.

    Against the FP64 step on the same stored values (what the kernels add:
    FP32 arithmetic and the 16-bit advected density): image <= 1e-2 and every
    gradient <= 2e-2 relative L2.  Against the FP64 step on the unrounded
    inputs the rounding of the inputs themselves adds to that (the MacCormack
    limiter and the 5 % image residual amplify it); those totals are bounded
    loosely here and their measured values stated with the benchmark."""
    from ngt_gb300 import workloads
    w = workloads.config2()
    q = [torch.as_tensor(a).to(storage).double().numpy() for a in (w.rho, w.ux, w.uy, w.uz)]
    ref, tgt = make_step(w, torch.float64)
    ref.step()
    refq, _ = make_step(w, torch.float64, tgt, inputs=q)
    refq.step()
    lo, _ = make_step(w, storage, tgt)
    lo.step()
    f32, _ = make_step(w, torch.float32, tgt)
    f32.step()

    def rl2(a, b):
        a, b = a.double(), b.double()
        return float((a - b).norm() / b.norm())

    assert rl2(lo.image, refq.image) < 1e-2
    assert rl2(lo.image, ref.image) < 1e-2
    # FP32 against FP64: the residual image - target is ~5 % of the image, so the
    # image's 1e-5 relative rounding reaches the gradients as a few 1e-4
    assert rl2(f32.image, ref.image) < 2e-5
    for a, b, bq, c in zip(lo.gradients(), ref.gradients(), refq.gradients(), f32.gradients()):
        assert rl2(a, bq) < 2e-2
        assert rl2(a, b) < (5e-2 if storage == torch.bfloat16 else 1.5e-1)
        assert rl2(c, b) < 1e-3
