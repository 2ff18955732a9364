"""ngt_raymarch_fwd_l2_bwd: a render's forward, image L2 loss and backward in one
call equal ngt_raymarch_fwd_l2 (or its background form) followed by
ngt_raymarch_bwd -- in one launch for the exact Beer-Lambert adjoint with emission
through the quad layout (with and without the sample cache, float and 16-bit
storage, with a background), and as the two passes for the settings it does not
fuse (reference gradient, deterministic mode)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

VOL = (12, 16, 20)
CAM = (14, 18, 22)  # depth samples, image height, width
YAWS = (10, -50, 95)


def setup(dtype, cache, seed=0, prepared=True, bm="BORDER"):
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops, scene
    rng = np.random.default_rng(seed)
    x = torch.as_tensor((rng.uniform(0, 1, (1,) + VOL + (1,)) * 0.3).astype(np.float32), device="cuda").to(dtype)
    vol = scene.volume_transform(list(VOL))
    cams = scene.orbit_cameras(list(CAM), list(YAWS))
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    mats = [ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6))]
    attrs = dict(interpolation="LINEAR", boundary=bm, blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=(0.6, 1.2))
    y = torch.empty((1, len(YAWS)) + CAM[1:] + (2,), device="cuda")
    r = ops._ray_args(x, *mats, list(CAM), y, attrs)
    lib, st = L.load(), ops._stream()
    rays = torch.empty(int(lib.ngt_raymarch_rays_bytes(ctypes.byref(r))), dtype=torch.uint8, device="cuda")
    assert lib.ngt_raymarch_rays(ctypes.byref(r), ops._ptr(rays), st) == L.NGT_OK
    r.rays = ops._ptr(rays)
    r.sample_cache = int(cache)
    quad = None
    if prepared:
        quad = torch.empty(int(lib.ngt_raymarch_quad_bytes(ctypes.byref(r))), dtype=torch.uint8, device="cuda")
        assert lib.ngt_raymarch_quad(ctypes.byref(r), ops._ptr(quad), st) == L.NGT_OK
        r.quad = ops._ptr(quad)
    else:
        # the separate forward builds its quad layout in its workspace, as the fused call does in its own
        quad = torch.empty(int(lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))), dtype=torch.uint8,
                           device="cuda")
        r.workspace, r.workspace_bytes = ops._ptr(quad), quad.numel()
    target = torch.as_tensor(rng.uniform(0, 0.5, (1, len(YAWS)) + CAM[1:] + (1,)).astype(np.float32), device="cuda")
    bkg = torch.as_tensor(rng.uniform(0, 0.4, (len(YAWS),) + CAM[1:] + (1,)).astype(np.float32), device="cuda")
    return dict(L=L, ops=ops, lib=lib, st=st, x=x, r=r, keep=(rays, quad, mats), target=target, bkg=bkg)


def grad_args(c, y, gy, gx, mode="exact", det=0):
    L, ops, lib = c["L"], c["ops"], c["lib"]
    g = L.RaymarchGradArgs()
    g.fwd = c["r"]
    g.output, g.output_grad, g.input_grad = ops._ptr(y), ops._ptr(gy), ops._ptr(gx)
    g.grad_mode, g.deterministic = L.GRAD[mode], det
    ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8, device="cuda")
    g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
    return g, ws


def separate(c, background, mode="exact", det=0):
    L, ops, lib = c["L"], c["ops"], c["lib"]
    y = torch.empty((1, len(YAWS)) + CAM[1:] + (2,), device="cuda")
    gy, loss = torch.empty_like(y), torch.zeros(1, device="cuda")
    r = c["r"]
    r.output = ops._ptr(y)
    if background:
        rc = lib.ngt_raymarch_fwd_l2_background(ctypes.byref(r), ops._ptr(c["bkg"]), ops._ptr(c["target"]), 1,
                                                ops._ptr(gy), ops._ptr(loss), c["st"])
    else:
        rc = lib.ngt_raymarch_fwd_l2(ctypes.byref(r), ops._ptr(c["target"]), 1, ops._ptr(gy), ops._ptr(loss), c["st"])
    assert rc == L.NGT_OK
    gx = torch.empty(c["x"].shape, device="cuda")
    g, ws = grad_args(c, y, gy, gx, mode, det)
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), c["st"]) == L.NGT_OK
    torch.cuda.synchronize()
    return y, gy, loss, gx


def fused(c, background, mode="exact", det=0):
    L, ops, lib = c["L"], c["ops"], c["lib"]
    y = torch.full((1, len(YAWS)) + CAM[1:] + (2,), float("nan"), device="cuda")
    gy, loss = torch.full_like(y, float("nan")), torch.zeros(1, device="cuda")
    gx = torch.empty(c["x"].shape, device="cuda")
    g, ws = grad_args(c, y, gy, gx, mode, det)
    bk = ops._ptr(c["bkg"]) if background else None
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), bk, ops._ptr(c["target"]), 1, ops._ptr(loss),
                                       c["st"]) == L.NGT_OK
    torch.cuda.synchronize()
    return y, gy, loss, gx


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("cache", [0, 1])
@pytest.mark.parametrize("background", [False, True])
def test_fused_equals_separate_calls(dtype, cache, background):
    c = setup(dtype, cache)
    y0, gy0, l0, g0 = separate(c, background)
    y1, gy1, l1, g1 = fused(c, background)
    assert torch.equal(y0, y1) and torch.equal(gy0, gy1)
    assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
    assert rel(g1, g0) < 1e-6


@pytest.mark.parametrize("mode,det", [("reference", 0), ("exact", 1)])
def test_unfused_settings_run_the_two_passes(mode, det):
    c = setup(torch.float32, 1, seed=4)
    y0, gy0, l0, g0 = separate(c, False, mode, det)
    y1, gy1, l1, g1 = fused(c, False, mode, det)
    assert torch.equal(y0, y1) and torch.equal(gy0, gy1)
    assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
    if det:
        assert torch.equal(g0, g1)  # the deterministic gradient: the same bits
    else:
        assert rel(g1, g0) < 1e-6


def test_fused_without_prepared_quad():
    """Without a prepared quad layout the fused call builds its own in the workspace
    (no sample cache) and still equals the separate calls."""
    c = setup(torch.float32, 0, seed=6, prepared=False)
    y0, gy0, l0, g0 = separate(c, False)
    y1, gy1, l1, g1 = fused(c, False)
    assert torch.equal(y0, y1) and torch.equal(gy0, gy1)
    assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
    assert rel(g1, g0) < 1e-6


@pytest.mark.parametrize("bm", ["CLAMP", "WRAP"])
def test_fused_other_boundaries(bm):
    """CLAMP and WRAP rays (never clipped: every ray takes the frustum's depth
    samples, the quad layout's padding maps the outside cells)."""
    c = setup(torch.float32, 1, seed=8, bm=bm)
    y0, gy0, l0, g0 = separate(c, False)
    y1, gy1, l1, g1 = fused(c, False)
    assert torch.equal(y0, y1) and torch.equal(gy0, gy1)
    assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
    assert rel(g1, g0) < 1e-6
