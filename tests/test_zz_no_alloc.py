"""ngt_raymarch_bwd_static -- the render backward for callers that cannot
allocate device memory (their host program's pool owns the device, or they may
not allocate once running), with its scratch in a static device array --
against ngt_raymarch_bwd with a caller workspace, through the C ABI, on
calls in a row (each finds the previous call's leftovers in the array).

Collected last on purpose: it must pass both alone in a fresh process and after
every other test has used the library."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _grad_args(x, y, gy, gx, M, V, P, F, shape, scale, grad_mode):
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=scale)
    g = L.RaymarchGradArgs()
    g.fwd = ops._ray_args(x, M, V, P, F, shape, None, attrs)
    g.output, g.output_grad, g.input_grad = ops._ptr(y), ops._ptr(gy), ops._ptr(gx)
    g.grad_mode = L.GRAD[grad_mode]
    return g


def _case(grid, image, yaws, storage, seed):
    """A render of a seeded density: (x, y, gy, M, V, P, F, image shape, scale)."""
    from ngt_gb300 import ops, scene
    dev = torch.device("cuda", 0)
    vol = scene.volume_transform(list(grid))
    cams = scene.orbit_cameras(list(image), list(yaws))
    M = ops._floats(scene.model_params([vol]), 16, dev)
    V, P, F = (ops._floats(m, w, dev) for m, w in zip(scene.camera_params(cams), (16, 16, 6)))
    rng = np.random.default_rng(seed)
    x = torch.as_tensor(rng.uniform(0, 0.4, (1,) + tuple(grid) + (1,)).astype(np.float32), device=dev).to(storage)
    scale = (0.6, 1.2)
    y = ops.raymarch_grid_transform(x, M, V, P, F, list(image), emission_scale=scale)
    gy = torch.as_tensor(rng.standard_normal(tuple(y.shape)).astype(np.float32), device=dev)
    return x, y, gy, M, V, P, F, list(image), scale


# (storage, gradient semantics): the exact adjoint through the quad layout in float
# and 16-bit storage, and the reference mode, whose weight-sum buffers the call
# clears inside the shared array
CASES = [(torch.float32, "exact"), (torch.bfloat16, "exact"), (torch.float32, "reference")]


@pytest.mark.parametrize("storage,grad_mode", CASES, ids=["f32-exact", "bf16-exact", "f32-reference"])
def test_static_scratch_backward_matches_workspace_backward(storage, grad_mode):
    """Three static-scratch calls in a row -- a larger grid with three cameras,
    then a smaller grid twice, so the later calls find an earlier call's larger
    layout left in the shared array -- each against ngt_raymarch_bwd with a
    caller workspace (relative max difference 1e-5: float atomics in both)."""
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _lib as L
    from ngt_gb300 import ops
    lib = L.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    big = _case((20, 22, 24), (16, 12, 10), (17.0, -40.0, 65.0), storage, 11)
    small = _case((12, 14, 16), (12, 10, 8), (17.0, -40.0), storage, 12)
    for x, y, gy, M, V, P, F, shape, scale in (big, small, small):
        # the existing entry point with a caller workspace
        want = torch.empty(x.shape, dtype=torch.float32, device=x.device)
        g = _grad_args(x, y, gy, want, M, V, P, F, shape, scale, grad_mode)
        ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                         device=x.device)
        g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_raymarch_bwd(ctypes.byref(g), stream) == L.NGT_OK
        torch.cuda.synchronize()
        assert float(want.abs().max()) > 0
        # the static-scratch entry point on the same arguments
        got = torch.full_like(want, float("nan"))
        gs = _grad_args(x, y, gy, got, M, V, P, F, shape, scale, grad_mode)
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
    g = _grad_args(x, y, torch.zeros_like(y), torch.empty_like(x), M, V, P, F, [16, 16, 16], (1.0, 1.0), "exact")
    assert lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g)) > (16 << 20)
    rc = lib.ngt_raymarch_bwd_static(ctypes.byref(g), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.NGT_ERR_WORKSPACE
    assert b"static scratch" in lib.ngt_last_error_message()
