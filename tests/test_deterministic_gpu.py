"""Bit-reproducible gradients of the render and transform-resample adjoints:
two runs give identical bits, and the result is the exact adjoint (against the
oracle and against the float-atomic path).  The render uses fixed-point integer
accumulation, the transform resample the gather form."""
import numpy as np
import pytest
import torch

from oracle import ops as oops

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = b.detach().double().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def scene(grid=(14, 18, 16), image=(16, 20, 18), yaws=(17.0, -40.0, 65.0), batch=2):
    """Matrices of ``batch`` grids (one model matrix each) seen by the cameras at ``yaws``."""
    from ngt_gb300 import scene as sc
    cams = sc.orbit_cameras(list(image), list(yaws))
    V, P, F = sc.camera_params(cams)
    M = sc.model_params([sc.volume_transform(list(grid))] * batch)
    return M, V, P, F


# (channels in, emission channels, blend, boundary, negative extinction somewhere)
CASES = [(1, 2, "BEER_LAMBERT", "BORDER", False), (2, 0, "BEER_LAMBERT", "BORDER", False),
         (2, 0, "BEER_LAMBERT", "CLAMP", True), (4, 0, "ALPHA", "BORDER", False),
         (1, 0, "ADDITIVE", "WRAP", False), (1, 4, "BEER_LAMBERT", "BORDER", False)]


@pytest.mark.parametrize("cin,emission,blend,boundary,negative", CASES)
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_raymarch_deterministic(cin, emission, blend, boundary, negative, dtype):
    from ngt_gb300 import ops
    dev = torch.device("cuda", 0)
    grid, image = (14, 18, 16), (16, 20, 18)
    M, V, P, F = scene(grid, image)
    rng = np.random.default_rng(3 + cin + emission)
    x = rng.uniform(0.0, 0.5, (2,) + grid + (cin,))
    if negative:
        x[0, 3, 4, 5, -1] = -0.2  # a negative extinction sample: the checkpointed adjoint
    scale = None if not emission else tuple(float(v) for v in rng.uniform(0.5, 1.5, emission))
    xt = torch.as_tensor(x, device=dev, dtype=dtype)
    y = ops.raymarch_grid_transform(xt, M, V, P, F, image, blending_mode=blend, boundary=boundary,
                                    emission_scale=scale)
    gy = torch.as_tensor(rng.standard_normal(tuple(y.shape)), device=dev, dtype=y.dtype)
    kw = dict(blending_mode=blend, boundary=boundary, emission_scale=scale)
    runs = [ops.raymarch_grid_transform_grad(xt, y, gy, M, V, P, F, image, deterministic=True, **kw)
            for _ in range(3)]
    for r in runs[1:]:
        assert torch.equal(r, runs[0])
    atomic = ops.raymarch_grid_transform_grad(xt, y, gy, M, V, P, F, image, deterministic=False, **kw)
    tol = 1e-5 if dtype == torch.float32 else 1e-11
    assert rel(runs[0], atomic) < tol
    # the oracle on the expanded grid, reduced back to the input channels
    xn = x.astype(np.float64 if dtype == torch.float64 else np.float32)
    sc = np.asarray(scale, xn.dtype) if scale else None
    xo = xn * sc if scale else xn
    yo = y.detach().cpu().numpy()
    want = oops.raymarch_grid_transform_grad(xo, yo, gy.cpu().numpy(), M, V, P, F, image, blending_mode=blend,
                                             boundary=boundary)
    if scale:
        want = (want * sc).sum(-1, keepdims=True)
    # sample positions are float in every storage type (the reference's), so the
    # float64 run differs from the float64 oracle's positions by float rounding
    assert rel(runs[0], want) < 1e-4


@pytest.mark.parametrize("boundary", ["BORDER", "CLAMP"])
@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_transform_deterministic(boundary, C, dtype):
    from ngt_gb300 import ops
    dev = torch.device("cuda", 0)
    grid, out = (10, 12, 14), (9, 11, 13)
    M, V, P, F = scene(grid, out, (10.0, -70.0))
    rng = np.random.default_rng(40 + C)
    x = rng.uniform(0.0, 1.0, (2,) + grid + (C,))
    g = rng.standard_normal((2, 2) + out + (C,))
    xt = torch.as_tensor(x, device=dev, dtype=dtype)
    gt = torch.as_tensor(g, device=dev, dtype=dtype)
    runs = [ops.sample_grid_transform_grad(xt, gt, M, V, P, F, boundary=boundary, deterministic=True)
            for _ in range(3)]
    for r in runs[1:]:
        assert torch.equal(r, runs[0])
    atomic = ops.sample_grid_transform_grad(xt, gt, M, V, P, F, boundary=boundary, deterministic=False)
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    assert rel(runs[0], atomic) < tol
    xn = x.astype(np.float32) if dtype == torch.float32 else x
    want = oops.sample_grid_transform_grad(xn, g.astype(xn.dtype), M, V, P, F, boundary=boundary)
    assert rel(runs[0], want) < 1e-5  # float sample positions, as in the raymarch


def test_autograd_deterministic_flag():
    """ops.set_deterministic routes the autograd backward of both ops through
    the reproducible forms."""
    from ngt_gb300 import ops
    dev = torch.device("cuda", 0)
    grid, image = (12, 14, 10), (12, 10, 12)
    M, V, P, F = scene(grid, image, (5.0, 60.0), batch=1)
    rng = np.random.default_rng(9)
    x = torch.as_tensor(rng.uniform(0, 0.5, (1,) + grid + (1,)).astype(np.float32), device=dev)
    old = ops.get_deterministic()
    ops.set_deterministic(True)
    try:
        grads = []
        for _ in range(2):
            xr = x.clone().requires_grad_()
            y = ops.raymarch_grid_transform(xr, M, V, P, F, image, emission_scale=(0.7, 1.3))
            z = ops.sample_grid_transform(xr, M, V, P, F, image)
            (y[..., 0].square().sum() + z.square().sum()).backward()
            grads.append(xr.grad.clone())
        assert torch.equal(grads[0], grads[1])
    finally:
        ops.set_deterministic(old)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("boundary", ["BORDER", "CLAMP", "WRAP"])
def test_raymarch_deterministic_prepared_quad(dtype, boundary):
    """The deterministic render adjoint reads its samples through the caller's
    prepared quad layout when there is one: the same bits as with the direct
    gathers (the quad reads the same corner values and weights)."""
    import ctypes
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops, scene
    lib = L.load()
    vol, cam = (10, 13, 15), (12, 14, 16)
    rng = np.random.default_rng(7)
    x = torch.as_tensor(rng.uniform(0, 0.5, (1,) + vol + (1,)).astype(np.float32), device="cuda").to(dtype)
    cams = scene.orbit_cameras(list(cam), [25.0, -70.0])
    M = scene.model_params([scene.volume_transform(list(vol))])
    V, P, F = scene.camera_params(cams)
    mats = [ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6))]
    attrs = dict(interpolation="LINEAR", boundary=boundary, blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=(0.8, 1.3))
    y = torch.empty((1, 2) + cam[1:] + (2,), device="cuda")
    r = ops._ray_args(x, *mats, list(cam), y, attrs)
    st = ops._stream()
    assert lib.ngt_raymarch_fwd(ctypes.byref(r), st) == L.NGT_OK
    gy = torch.as_tensor(rng.standard_normal(tuple(y.shape)).astype(np.float32), device="cuda")
    quad = torch.empty(int(lib.ngt_raymarch_quad_bytes(ctypes.byref(r))), dtype=torch.uint8, device="cuda")
    out = []
    for prepared in (False, True):
        if prepared:
            assert lib.ngt_raymarch_quad(ctypes.byref(r), ops._ptr(quad), st) == L.NGT_OK
            r.quad = ops._ptr(quad)
        g = L.RaymarchGradArgs()
        g.fwd = r
        gx = torch.empty(x.shape, device="cuda")
        g.output, g.output_grad, g.input_grad = ops._ptr(y), ops._ptr(gy), ops._ptr(gx)
        g.grad_mode, g.deterministic = L.GRAD["exact"], 1
        ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                         device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_raymarch_bwd(ctypes.byref(g), st) == L.NGT_OK
        torch.cuda.synchronize()
        out.append(gx)
    assert float(out[0].abs().max()) > 0
    assert torch.equal(out[0], out[1])
