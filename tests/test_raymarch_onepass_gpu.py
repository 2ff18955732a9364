"""Exact one-pass Beer-Lambert render backward (one-channel density through the
quad layout, with emission channels, quad-gradient fold) against the oracle:
footprints of pixels smaller and much larger than cells (a 5x6 image of a 40^3
grid), the three boundary rules (the fold maps CLAMP and WRAP padding back onto
cells), batches with separate cameras, 16-bit storage, and accumulation into an
existing gradient."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import ops as oops

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(17)


def T(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(a).max(), 1e-30)


def mats(vol_dhw, cam_dhw, yaws, batch=1):
    from ngt_gb300 import scene
    vol = scene.volume_transform(list(vol_dhw))
    cams = scene.orbit_cameras(list(cam_dhw), list(yaws))
    M = scene.model_params([vol] * batch)
    V, P, F = scene.camera_params(cams)
    return M, V, P, F


# (grid D,H,W; image depth,H,W; camera yaws; batch): pixels smaller than cells,
# pixels much larger (one 16x8 tile spans the grid), and a batch of two grids
CASES = {
    "fine": ((20, 24, 28), (24, 40, 36), (10, -35, 60), 1),
    "coarse": ((40, 40, 40), (20, 6, 5), (0, 45), 1),
    "batch": ((12, 16, 20), (12, 20, 18), (5, -70, 100), 2),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("cb", [2, 4])
def test_onepass_backward_matches_oracle(case, bm, cb):
    from ngt_gb300 import ops
    vol, cam, yaws, batch = CASES[case]
    M, V, P, F = mats(vol, cam, yaws, batch)
    rho = (RNG.uniform(0, 1, (batch,) + vol + (1,)) * 0.3).astype(np.float32)
    scale = [0.7, 1.3] if cb == 2 else [0.2, 0.5, 0.9, 1.3]
    full = (rho * np.asarray(scale, np.float32)).astype(np.float32)
    rt = T(rho).requires_grad_()
    y = ops.raymarch_grid_transform(rt, M, V, P, F, list(cam), boundary=bm, emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, list(cam), boundary=bm)
    assert rel(ref, y.detach().cpu().numpy()) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    with ops.gradient_mode("exact"):
        y.backward(T(gy))
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, list(cam), boundary=bm, grad_mode="exact")
    want = (gfull * np.asarray(scale)).sum(-1, keepdims=True)
    assert rel(want, rt.grad.cpu().numpy()) < 1e-4


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
def test_onepass_backward_16bit_storage(dtype):
    """16-bit density (quad layout of 8-byte entries), FP32 adjoint: against the
    oracle on the stored values."""
    from ngt_gb300 import ops
    vol, cam, yaws, batch = CASES["fine"]
    M, V, P, F = mats(vol, cam, yaws)
    xt = T((RNG.uniform(0, 1, (1,) + vol + (1,)) * 0.3).astype(np.float32), dtype)
    rho = xt.float().cpu().numpy()
    scale = [0.7, 1.3]
    full = rho * np.asarray(scale, np.float32)
    y = ops.raymarch_grid_transform(xt, M, V, P, F, list(cam), emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, list(cam))
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    # the gradient op returns the FP32 gradient (an autograd leaf's would be rounded to its storage type)
    gx = ops.raymarch_grid_transform_grad(xt, y, T(gy), M, V, P, F, list(cam), emission_scale=scale,
                                          grad_mode="exact")
    assert gx.dtype == torch.float32
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, list(cam), grad_mode="exact")
    want = (gfull * np.asarray(scale)).sum(-1, keepdims=True)
    assert rel(want, gx.cpu().numpy()) < 1e-4


def test_onepass_backward_accumulates():
    """With ``accumulate`` the gradient is added to what the buffer holds."""
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops
    lib = L.load()
    vol, cam, yaws, batch = CASES["fine"]
    M, V, P, F = mats(vol, cam, yaws)
    xt = T((RNG.uniform(0, 1, (1,) + vol + (1,)) * 0.3).astype(np.float32))
    Md, Vd, Pd, Fd = (ops._floats(m, w, xt.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6)))
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=(0.6, 1.2))
    stream = ops._stream()
    y = torch.empty((1, 3) + cam[1:] + (2,), device="cuda")
    r = ops._ray_args(xt, Md, Vd, Pd, Fd, list(cam), y, attrs)
    ws = torch.empty(int(lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))) + 1, dtype=torch.uint8,
                     device="cuda")
    r.workspace, r.workspace_bytes = ops._ptr(ws), ws.numel()
    assert lib.ngt_raymarch_fwd(ctypes.byref(r), stream) == L.NGT_OK
    gy = T(RNG.standard_normal(tuple(y.shape)).astype(np.float32))

    def backward(start, accumulate):
        g = L.RaymarchGradArgs()
        g.fwd = r
        g.fwd.workspace, g.fwd.workspace_bytes = None, 0
        gx = start.clone()
        g.output, g.output_grad, g.input_grad, g.grad_mode = ops._ptr(y), ops._ptr(gy), ops._ptr(gx), L.GRAD["exact"]
        g.accumulate = accumulate
        gws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                          device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(gws), gws.numel()
        assert lib.ngt_raymarch_bwd(ctypes.byref(g), stream) == L.NGT_OK
        torch.cuda.synchronize()
        return gx

    base = torch.full((1,) + vol + (1,), 0.25, device="cuda")
    plain = backward(torch.full_like(base, 7.0), 0)  # written, not added
    added = backward(base, 1)
    assert torch.allclose(added - base, plain, rtol=1e-5, atol=1e-6)
