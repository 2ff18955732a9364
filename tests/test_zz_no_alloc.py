"""ngt_raymarch_bwd_static -- the render backward for callers that cannot
allocate device memory (their host program's pool owns the device, or they may
not allocate once running), with its scratch in a static device array --
against ngt_raymarch_bwd with a caller workspace, through the C ABI, on two
calls in a row (the second finds the first call's leftovers in the array).

Collected last on purpose: it must pass both alone in a fresh process and after
every other test has used the library."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _grad_args(x, y, gy, gx, M, V, P, F, shape, scale):
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=scale)
    g = L.RaymarchGradArgs()
    g.fwd = ops._ray_args(x, M, V, P, F, shape, None, attrs)
    g.output, g.output_grad, g.input_grad = ops._ptr(y), ops._ptr(gy), ops._ptr(gx)
    g.grad_mode = L.GRAD["exact"]
    return g


def test_static_scratch_backward_matches_workspace_backward():
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops, scene
    lib = L.load()
    dev = torch.device("cuda", 0)
    vol = scene.volume_transform([12, 14, 16])
    cams = scene.orbit_cameras([12, 10, 8], [17.0, -40.0])
    M = ops._floats(scene.model_params([vol]), 16, dev)
    V, P, F = (ops._floats(m, w, dev) for m, w in zip(scene.camera_params(cams), (16, 16, 6)))
    rng = np.random.default_rng(11)
    x = torch.as_tensor(rng.uniform(0, 0.4, (1, 12, 14, 16, 1)).astype(np.float32), device=dev)
    scale = (0.6, 1.2)
    y = ops.raymarch_grid_transform(x, M, V, P, F, [12, 10, 8], emission_scale=scale)
    gy = torch.as_tensor(rng.standard_normal(tuple(y.shape)).astype(np.float32), device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # the existing entry point with a caller workspace
    want = torch.empty_like(x)
    g = _grad_args(x, y, gy, want, M, V, P, F, [12, 10, 8], scale)
    ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8, device=dev)
    g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), stream) == L.NGT_OK
    torch.cuda.synchronize()
    assert float(want.abs().max()) > 0

    # the static-scratch entry point, twice in a row (the second call sees the
    # first call's leftovers in the shared array)
    for _ in range(2):
        got = torch.full_like(x, float("nan"))
        gs = _grad_args(x, y, gy, got, M, V, P, F, [12, 10, 8], scale)
        rc = lib.ngt_raymarch_bwd_static(ctypes.byref(gs), stream)
        assert rc == L.NGT_OK, lib.ngt_last_error_message().decode()
        torch.cuda.synchronize()
        err = float((got - want).abs().max()) / float(want.abs().max())
        assert err < 1e-5, err


def test_static_scratch_rejects_oversized_calls():
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops, scene
    lib = L.load()
    dev = torch.device("cuda", 0)
    vol = scene.volume_transform([128, 128, 128])
    cams = scene.orbit_cameras([16, 16, 16], [0.0])
    M = ops._floats(scene.model_params([vol]), 16, dev)
    V, P, F = (ops._floats(m, w, dev) for m, w in zip(scene.camera_params(cams), (16, 16, 6)))
    x = torch.zeros((1, 128, 128, 128, 1), device=dev)
    y = torch.zeros((1, 1, 16, 16, 2), device=dev)
    g = _grad_args(x, y, torch.zeros_like(y), torch.empty_like(x), M, V, P, F, [16, 16, 16], (1.0, 1.0))
    assert lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g)) > (16 << 20)
    rc = lib.ngt_raymarch_bwd_static(ctypes.byref(g), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.NGT_ERR_WORKSPACE
    assert b"static scratch" in lib.ngt_last_error_message()
