"""Batched uneven scenes: the persistent batched raymarch and the batched
advection against one single-scene call per scene, against the oracle, with a
scene whose extinction can be negative, and through the autotuner and a CUDA
graph."""
import numpy as np
import pytest
import torch

from oracle import advect as oadvect
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def scenes(n=5, seed=7, signed=(), dtype=torch.float32):
    from ngt_gb300 import ops, workloads
    from ngt_gb300.batch import Scene
    dev = torch.device("cuda", 0)
    ws = workloads.batched_scenes(n=n, seed=seed, sizes=(12, 16, 20, 24), cameras=(1, 3), image_sides=(16, 32),
                                  depths=(12, 16, 20))
    out = []
    for k, w in enumerate(ws):
        rho = w.rho
        if k in signed:
            rho = rho - np.float32(0.1)
            w.rho = rho
        with torch.no_grad():
            tgt = ops.raymarch_grid_transform(torch.as_tensor(w.rho_target, device=dev)[None], w.M, w.V, w.P, w.F,
                                              w.image_dhw, emission_scale=(w.depth_step, w.depth_step))[..., :1]
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev).to(dtype)
        out.append(Scene(T(rho), T(w.ux), T(w.uy), T(w.uz), w.M, w.V, w.P, w.F, w.image_dhw, tgt))
    return ws, out


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = b.detach().double().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def run_both(sc, **kw):
    from ngt_gb300.batch import BatchedScenes
    b = BatchedScenes(sc, **kw)
    b.launch()
    torch.cuda.synchronize()
    got = (float(b.loss.item()), b.images.clone(), [[g.clone() for g in b.gradients(k)] for k in range(b.n)])
    b.per_scene()
    want = (float(b.loss.item()), b.images.clone(), [[g.clone() for g in b.gradients(k)] for k in range(b.n)])
    return b, got, want


def test_batched_matches_per_scene():
    _, sc = scenes()
    b, got, want = run_both(sc)
    assert torch.equal(got[1], want[1])  # same tile code, same samples
    assert abs(got[0] - want[0]) <= 1e-6 * abs(want[0])
    for gk, wk in zip(got[2], want[2]):
        for a, c in zip(gk, wk):
            assert rel(a, c) < 1e-5


def test_batched_maccormack_matches_per_scene():
    _, sc = scenes(n=3, seed=11)
    b, got, want = run_both(sc, order=2, clamp="MC_SMOOTH")
    assert torch.equal(got[1], want[1])
    for gk, wk in zip(got[2], want[2]):
        for a, c in zip(gk, wk):
            assert rel(a, c) < 1e-5


def test_batched_negative_extinction_scene():
    """Scene 1 has negative densities: its backward takes the checkpointed path
    inside the batch, the others the one-pass path."""
    _, sc = scenes(n=4, seed=9, signed=(1,))
    b, got, want = run_both(sc)
    assert torch.equal(got[1], want[1])
    for gk, wk in zip(got[2], want[2]):
        for a, c in zip(gk, wk):
            assert rel(a, c) < 1e-5


def test_batched_against_oracle():
    ws, sc = scenes(n=2, seed=5)
    from ngt_gb300.batch import BatchedScenes
    b = BatchedScenes(sc)
    b.launch()
    torch.cuda.synchronize()
    off = 0
    for k, w in enumerate(ws):
        s = np.float32(w.depth_step)
        scale = np.asarray([s, s], np.float32)
        rho2 = oadvect.density_maccormack(w.rho, w.ux, w.uy, w.uz, order=1, clamp="NONE")
        x = rho2[None] * scale
        img = oops.raymarch_grid_transform(x, w.M, w.V, w.P, w.F, w.image_dhw)
        npx = img.shape[1] * img.shape[2] * img.shape[3]
        got_img = b.images[off:off + npx].reshape(img.shape[1:])
        assert rel(got_img, img[0]) < 2e-5
        tgt = sc[k].targets.double().cpu().numpy().reshape(img.shape[:-1] + (1,)).astype(np.float32)
        diff = img[..., :1] - tgt
        gimg = np.concatenate([diff, np.zeros_like(diff)], -1)
        gx = oops.raymarch_grid_transform_grad(x, img, gimg, w.M, w.V, w.P, w.F, w.image_dhw)
        ref = oadvect.density_maccormack_grad(w.rho, w.ux, w.uy, w.uz, (gx[0] * scale).sum(-1, keepdims=True),
                                              order=1, clamp="NONE")
        for a, c in zip(b.gradients(k), ref):
            assert rel(a, c) < 1e-4
        off += npx


def test_autotune_and_graph():
    _, sc = scenes(n=4, seed=13)
    from ngt_gb300.batch import BatchedScenes
    b = BatchedScenes(sc)
    b.launch()
    torch.cuda.synchronize()
    loss0 = float(b.loss.item())
    g0 = [g.clone() for g in b.gradients(0)]
    best = b.autotune(candidates=(2, 8), repeats=2)
    assert all(c in (2, 8) for c, _ in best)
    b.capture()
    for _ in range(2):
        assert abs(float(b.step().item()) - loss0) <= 1e-6 * abs(loss0)
    torch.cuda.synchronize()
    for a, c in zip(b.gradients(0), g0):
        assert rel(a, c) < 1e-5


def test_backward_reuses_forward_quads():
    """The batched render backward that reuses the forward's quad layouts and
    sign words equals the one that builds its own, with a scene whose
    extinction can be negative among them."""
    import ctypes
    _, sc = scenes(n=4, seed=17, signed=(2,))
    from ngt_gb300.batch import BatchedScenes
    b = BatchedScenes(sc)
    b.launch()
    torch.cuda.synchronize()
    got = [[g.clone() for g in b.gradients(k)] for k in range(b.n)]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    b.render_bwd(s, after_fwd=False)
    b.advect_bwd(s)
    torch.cuda.synchronize()
    for k in range(b.n):
        for a, c in zip(got[k], b.gradients(k)):
            assert rel(a, c) < 1e-6


@pytest.mark.parametrize("signed", [(), (1,)])
def test_fused_render_launch_matches_three_calls(signed):
    """The step's one persistent render launch (forward, loss and backward of every
    scene, ngt_raymarch_fwd_l2_bwd_batch) equals the batched forward, the loss call
    and the batched backward; with a scene whose extinction can be negative (its
    items take the checkpointed adjoint)."""
    from ngt_gb300.batch import BatchedScenes
    _, sc = scenes(n=6, seed=21, signed=signed)
    b = BatchedScenes(sc)
    b.launch_passes()
    torch.cuda.synchronize()
    want = (float(b.loss.item()), b.images.clone(), b.g_images.clone(),
            [[g.clone() for g in b.gradients(k)] for k in range(b.n)])
    b.images.fill_(float("nan"))
    b.g_images.fill_(float("nan"))
    b.launch()
    torch.cuda.synchronize()
    assert torch.equal(b.images, want[1]) and torch.equal(b.g_images, want[2])
    assert abs(float(b.loss.item()) - want[0]) <= 1e-6 * abs(want[0])
    for k in range(b.n):
        for a, c in zip(b.gradients(k), want[3][k]):
            assert rel(a, c) < 1e-6
