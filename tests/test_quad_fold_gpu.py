"""The fold of a BORDER quad gradient into the cell gradient: every cell gets,
bit for bit, the sum of its four quad components in the order (0,0) of entry
(x+1, y+1), (1,0) of (x, y+1), (0,1) of (x+1, y), (1,1) of (x, y) -- checked
against that sum formed in NumPy from the quad gradient the exact backward
leaves at the end of its workspace, at widths that are not a multiple of 32,
above 256 and of one cell."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def align256(n):
    return (n + 255) // 256 * 256


@pytest.mark.parametrize("vol", [(6, 9, 45), (3, 5, 300), (4, 7, 32), (2, 1, 1)])
def test_border_fold_bitexact(vol):
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops, scene
    lib = L.load()
    D, H, W = vol
    cam = (10, 12, 14)
    rng = np.random.default_rng(sum(vol))
    x = torch.as_tensor((rng.uniform(0, 1, (1,) + vol + (1,)) * 0.4).astype(np.float32), device="cuda")
    cams = scene.orbit_cameras(list(cam), [20.0, -35.0, 160.0])
    M = scene.model_params([scene.volume_transform(list(vol))])
    V, P, F = scene.camera_params(cams)
    mats = [ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6))]
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=(0.7, 1.1))
    y = torch.empty((1, 3) + cam[1:] + (2,), device="cuda")
    r = ops._ray_args(x, *mats, list(cam), y, attrs)
    st = ops._stream()
    assert lib.ngt_raymarch_fwd(ctypes.byref(r), st) == L.NGT_OK
    gy = torch.as_tensor(rng.standard_normal(tuple(y.shape)).astype(np.float32), device="cuda")
    g = L.RaymarchGradArgs()
    g.fwd = r
    gx = torch.empty(x.shape, device="cuda")
    g.output, g.output_grad, g.input_grad, g.grad_mode = ops._ptr(y), ops._ptr(gy), ops._ptr(gx), L.GRAD["exact"]
    ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8, device="cuda")
    g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), st) == L.NGT_OK
    torch.cuda.synchronize()
    # the quad gradient: (D + 2) planes of (H + 1) x (W + 1) float4 entries, last in the workspace
    n = (D + 2) * (H + 1) * (W + 1) * 16
    start = ws.numel() - align256(n)
    q = ws[start:start + n].cpu().numpy().view(np.float32).reshape(D + 2, H + 1, W + 1, 4)[1:D + 1]
    if min(H, W) > 1:
        assert np.any(q != 0)
    acc = np.zeros((D, H, W), np.float32)
    acc += q[:, 1:, 1:, 0]
    acc += q[:, 1:, :-1, 1]
    acc += q[:, :-1, 1:, 2]
    acc += q[:, :-1, :-1, 3]
    got = gx.cpu().numpy().reshape(D, H, W)
    assert np.array_equal(got.view(np.int32), acc.view(np.int32))
