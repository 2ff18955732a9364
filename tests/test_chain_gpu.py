"""The checkpointed multi-frame chain: against the oracle's frame-by-frame
composition, independent of the checkpoint interval, and against FP64 central
differences."""
import numpy as np
import pytest
import torch

from oracle import advect as oadvect
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def small(frames=4, grid=(12, 16, 10), image=(16, 16), depth=12):
    from ngt_gb300 import workloads
    return workloads.plume_chain(grid=grid, frames=frames, image=image, depth=depth)


def oracle_chain(w, rho0, targets, clamp="MC_SMOOTH"):
    """Loss and gradients (rho0, ux, uy, uz) of the chain by the oracle."""
    s = np.float64(w.depth_step) if rho0.dtype == np.float64 else np.float32(w.depth_step)
    sc = np.asarray([s, s], rho0.dtype)
    u = [a.astype(rho0.dtype) for a in (w.ux, w.uy, w.uz)]
    src = w.source.astype(rho0.dtype)
    rhos = [rho0]
    for _ in range(w.frames):
        rhos.append(oadvect.density_maccormack(rhos[-1], *u, clamp=clamp) + src)
    loss = 0.0
    g = np.zeros_like(rho0)
    gu = [np.zeros_like(a) for a in u]
    for t in range(w.frames - 1, -1, -1):
        x = rhos[t + 1][None] * sc
        img = oops.raymarch_grid_transform(x, w.M, w.V, w.P, w.F, w.image_dhw)
        diff = img[..., :1] - targets[t]
        loss += 0.5 * float((diff.astype(np.float64) ** 2).sum())
        gimg = np.concatenate([diff, np.zeros_like(diff)], -1)
        gx = oops.raymarch_grid_transform_grad(x, img, gimg, w.M, w.V, w.P, w.F, w.image_dhw)
        g = g + (gx[0] * sc).sum(-1, keepdims=True)
        gr, gx_, gy_, gz_ = oadvect.density_maccormack_grad(rhos[t], *u, g, clamp=clamp)
        for a, b in zip(gu, (gx_, gy_, gz_)):
            a += b
        g = gr
    return loss, (g,) + tuple(gu)


def oracle_targets(w, rho0):
    s = np.float32(w.depth_step)
    sc = np.asarray([s, s], np.float32)
    rho, out = rho0, []
    for _ in range(w.frames):
        rho = oadvect.density_maccormack(rho, w.ux, w.uy, w.uz) + w.source
        out.append(oops.raymarch_grid_transform(rho[None] * sc, w.M, w.V, w.P, w.F, w.image_dhw)[..., :1])
    return np.stack(out)


def make_chain(w, dtype, targets, K, clamp="MC_SMOOTH", rho0=None):
    from ngt_gb300.chain import AdvectRenderChain
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev).to(dtype)
    return AdvectRenderChain(T(w.rho0 if rho0 is None else rho0), T(w.ux), T(w.uy), T(w.uz), T(w.source), w.M, w.V,
                             w.P, w.F, torch.as_tensor(targets, device=dev), w.image_dhw, w.frames,
                             checkpoint_every=K, clamp=clamp)


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def test_chain_matches_oracle():
    w = small(frames=4)
    tg = oracle_targets(w, w.rho0_target)
    ch = make_chain(w, torch.float32, tg, K=3)
    loss = float(ch.run().item())
    ref_loss, ref = oracle_chain(w, w.rho0, tg)
    assert abs(loss - ref_loss) <= 2e-5 * abs(ref_loss)
    for a, b in zip(ch.gradients(), ref):
        assert rel(a, b) < 1e-4


def test_chain_checkpoint_interval_invariance():
    """Same loss and gradients for K = 1, 4, T (recompute is bit-identical; only
    the order of the backward's atomic additions differs)."""
    w = small(frames=9, grid=(20, 28, 18), image=(24, 24), depth=20)
    tg = oracle_targets(w, w.rho0_target)
    runs = []
    for K in (1, 4, 9):
        ch = make_chain(w, torch.float32, tg, K=K)
        loss = float(ch.run().item())
        runs.append((loss, [g.clone() for g in ch.gradients()]))
    for loss, grads in runs[1:]:
        assert abs(loss - runs[0][0]) <= 1e-6 * abs(runs[0][0])
        for a, b in zip(grads, runs[0][1]):
            assert rel(a, b.double().cpu().numpy()) < 1e-5


def test_chain_graph_replay():
    w = small(frames=5)
    tg = oracle_targets(w, w.rho0_target)
    ch = make_chain(w, torch.float32, tg, K=2)
    l0 = float(ch.run().item())
    g0 = [g.clone() for g in ch.gradients()]
    ch.capture()
    for _ in range(2):
        l1 = float(ch.run().item())
        assert abs(l1 - l0) <= 1e-6 * abs(l0)
        for a, b in zip(ch.gradients(), g0):
            assert rel(a, b.double().cpu().numpy()) < 1e-5


def test_chain_fp64_finite_differences():
    """FP64 central differences through 6 frames (no limiter: the chain is then
    smooth in the density), at 16 voxels of rho0 and 8 faces of each velocity
    component drawn with seed 3 among entries with a non-zero gradient."""
    w = small(frames=6)
    tg = oracle_targets(w, w.rho0_target)
    ch = make_chain(w, torch.float64, tg, K=4, clamp="NONE")
    ch.run()
    grads = [g.clone() for g in ch.gradients()]
    params = [ch.rho0, ch.ux, ch.uy, ch.uz]
    rng = np.random.default_rng(3)
    errs = []
    for p, g, n in zip(params, grads, (16, 8, 8, 8)):
        gf = g.reshape(-1)
        nz = torch.nonzero(gf.abs() > 1e-10 * gf.abs().max()).reshape(-1).cpu().numpy()
        scale = float(gf.abs().max())
        pf = p.view(-1)
        for i in rng.choice(nz, n, replace=False):
            v = float(pf[i])
            pf[i] = v + 1e-5
            lp = float(ch.run().item())
            pf[i] = v - 1e-5
            lm = float(ch.run().item())
            pf[i] = v
            errs.append(abs((lp - lm) / 2e-5 - float(gf[i])) / scale)
    errs = np.asarray(errs)
    assert np.median(errs) < 1e-6, np.sort(errs)[-5:]
    assert np.quantile(errs, 0.9) < 1e-4, np.sort(errs)[-5:]
