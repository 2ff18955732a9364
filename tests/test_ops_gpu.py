"""GPU parity: every operator against the oracle on seeded inputs.

Tolerances (float32, relative to the largest reference magnitude):
* LUT resample forward and the MacCormack forward use the same operation order
  as the oracle and must match bit for bit;
* transform resample and raymarch forward: 2e-5 (positions come from fp32
  matrix math on the GPU, fp64 in the oracle);
* gradients: 1e-4 (atomic accumulation order), reference-normalised raymarch
  gradient 5e-4 (division by summed sample weights).
"""
import numpy as np
import pytest
import torch

from oracle import advect as oadvect
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def ngt():
    import ngt_gb300.ops as ops
    return ops


def T(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def N(t):
    return t.detach().cpu().numpy()


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(a).max(), 1e-30)


def scene_mats(vol_dhw=(8, 10, 12), cam_dhw=(8, 8, 6), yaws=(13, -47, 71)):
    from ngt_gb300 import scene
    vol = scene.volume_transform(list(vol_dhw))
    cams = scene.orbit_cameras(list(cam_dhw), list(yaws))
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    return M, V, P, F


RNG = np.random.default_rng(7)

# ---------------------------------------------------------------- LUT
LUT_CASES = [(fm, bm, cn, sep, C) for fm in ("NEAREST", "LINEAR", "MIN", "MAX") for bm in ("BORDER", "CLAMP", "WRAP")
             for cn in ("rel", "abs", "nrm") for sep in (True, False) for C in (1, 2, 4)]


def lut_inputs(cn, C, seed=0):
    r = np.random.default_rng(seed)
    x = r.standard_normal((2, 5, 6, 7, C)).astype(np.float32)
    lut = r.uniform(-1.5, 1.5, (2, 4, 5, 6, 4)).astype(np.float32)
    lut[..., 3] = 0
    if cn == "abs":
        lut = lut + np.array([2, 2.5, 2, 0], np.float32)
    if cn == "nrm":
        lut = lut * np.float32(0.05)
    kw = dict(relative_coords=cn != "abs", normalized_coords=cn == "nrm", cell_center_offset=0.5 if cn == "nrm" else 0.0)
    return x, lut, kw


@pytest.mark.parametrize("fm,bm,cn,sep,C", LUT_CASES)
def test_lut_forward_bitexact(fm, bm, cn, sep, C):
    x, lut, kw = lut_inputs(cn, C)
    y = ngt().sample_grid_lut(T(x), T(lut), interpolation=fm, boundary=bm, separate_camera_batch=sep, **kw)
    ref = oops.sample_grid_lut(x, lut, fm, bm, separate_camera_batch=sep, **kw)
    assert y.shape == ref.shape
    assert np.array_equal(N(y), ref)


@pytest.mark.parametrize("mode", ["exact", "reference"])
@pytest.mark.parametrize("fm,bm,cn,sep,C", [c for c in LUT_CASES if c[4] != 4])
def test_lut_backward(fm, bm, cn, sep, C, mode):
    x, lut, kw = lut_inputs(cn, C, seed=1)
    gy = np.random.default_rng(2).standard_normal(oops.sample_grid_lut(x, lut, fm, bm, separate_camera_batch=sep,
                                                                        **kw).shape).astype(np.float32)
    gx, gl = ngt().sample_grid_lut_grad(T(x), T(gy), T(lut), interpolation=fm, boundary=bm,
                                        separate_camera_batch=sep, grad_mode=mode, **kw)
    rx, rl = oops.sample_grid_lut_grad(x, gy, lut, fm, bm, separate_camera_batch=sep, grad_mode=mode, **kw)
    assert rel(rx, N(gx)) < 1e-5
    if np.abs(rl).max() > 0:
        assert rel(rl, N(gl)) < 1e-5
    else:
        assert np.abs(N(gl)).max() == 0


@pytest.mark.parametrize("mipmode", ["NEAREST", "LINEAR"])
def test_lut_mipmapped(mipmode):
    x = RNG.standard_normal((1, 16, 12, 20, 2)).astype(np.float32)
    lut = RNG.uniform(-3, 3, (2, 5, 6, 7, 4)).astype(np.float32)
    lut[..., 3] = RNG.uniform(-0.5, 3.5, lut.shape[:-1])
    kw = dict(interpolation="LINEAR", boundary="CLAMP", mipmapping=mipmode, num_mipmaps=2, mip_bias=0.25,
              cell_center_offset=0.5)
    y = ngt().sample_grid_lut(T(x), T(lut), **kw)
    assert rel(oops.sample_grid_lut(x, lut, **kw), N(y)) < 1e-6


def test_mip_pyramid():
    from oracle import core
    x = RNG.standard_normal((2, 9, 12, 16, 2)).astype(np.float32)
    levels = ngt().mip_pyramid(T(x), 3)
    for b in range(2):
        ref = core.mip_pyramid(x[b], 3)
        for lv in range(3):
            assert np.array_equal(N(levels[lv][b]), ref[lv + 1])


def test_lut_autograd_matches_grad_op():
    x, lut, kw = lut_inputs("rel", 2, seed=3)
    xt, lt = T(x).requires_grad_(), T(lut).requires_grad_()
    y = ngt().sample_grid_lut(xt, lt, interpolation="LINEAR", boundary="CLAMP", **kw)
    g = torch.randn_like(y)
    y.backward(g)
    gx, gl = ngt().sample_grid_lut_grad(T(x), g, T(lut), interpolation="LINEAR", boundary="CLAMP",
                                        grad_mode="exact", **kw)
    assert torch.equal(xt.grad, gx) or rel(N(gx), N(xt.grad)) < 1e-6
    assert rel(N(gl), N(lt.grad)) < 1e-6


# ---------------------------------------------------------- transform resample
@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH", "TRANSFORM"])
@pytest.mark.parametrize("fm", ["LINEAR", "NEAREST", "QUADRATIC"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
def test_transform(cm, fm, bm):
    M, V, P, F = scene_mats()
    x = RNG.uniform(0, 1, (1, 8, 10, 12, 2)).astype(np.float32)
    y = ngt().sample_grid_transform(T(x), M, V, P, F, [8, 8, 6], fm, bm, coordinate_mode=cm)
    ref = oops.sample_grid_transform(x, M, V, P, F, [8, 8, 6], fm, bm, coordinate_mode=cm)
    if fm == "NEAREST":
        assert np.isclose(N(y), ref, atol=1e-6).mean() > 0.99
    else:
        assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    for mode in ("exact", "reference"):
        if fm == "QUADRATIC" and bm == "BORDER" and mode == "reference":
            continue
        gx = ngt().sample_grid_transform_grad(T(x), T(gy), M, V, P, F, fm, bm, coordinate_mode=cm, grad_mode=mode)
        rx = oops.sample_grid_transform_grad(x, gy, M, V, P, F, fm, bm, coordinate_mode=cm, grad_mode=mode)
        if np.abs(rx).max() == 0:
            assert np.abs(N(gx)).max() == 0
        elif fm == "NEAREST":
            assert np.isclose(N(gx), rx, atol=1e-4).mean() > 0.98
        else:
            assert rel(rx, N(gx)) < 1e-4


@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH_REVERSE", "TRANSFORM_REVERSE"])
def test_transform_reverse(cm):
    M, V, P, F = scene_mats()
    xf = RNG.uniform(0, 1, (1, 8, 8, 6, 1)).astype(np.float32)
    y = ngt().sample_grid_transform(T(xf), M, V[:1], P[:1], F[:1], [8, 10, 12], "LINEAR", "BORDER",
                                    coordinate_mode=cm)
    ref = oops.sample_grid_transform(xf, M, V[:1], P[:1], F[:1], [8, 10, 12], "LINEAR", "BORDER", coordinate_mode=cm)
    assert rel(ref, N(y)) < 2e-5


def test_transform_mipmapped():
    M, V, P, F = scene_mats(vol_dhw=(32, 32, 32), cam_dhw=(8, 8, 8))
    x = RNG.uniform(0, 1, (1, 32, 32, 32, 1)).astype(np.float32)
    kw = dict(interpolation="LINEAR", boundary="CLAMP", mipmapping="LINEAR", num_mipmaps=3)
    y = ngt().sample_grid_transform(T(x), M, V, P, F, [8, 8, 8], **kw)
    ref = oops.sample_grid_transform(x, M, V, P, F, [8, 8, 8], **kw)
    assert rel(ref, N(y)) < 1e-4


@pytest.mark.parametrize("lin", [True, False])
def test_lod_transform(lin):
    from ngt_gb300 import scene
    vol = scene.volume_transform([8, 10, 12])
    cams = scene.orbit_cameras([8, 8, 6], [13, -47])
    MV = np.stack([scene.colmajor(c.view_matrix() @ vol.get_transform_matrix()) for c in cams])
    _, P, F = scene.camera_params(cams)
    y = ngt().lod_transform([8, 10, 12], MV, P, F, [8, 8, 6], linearize_depth=lin)
    ref = oops.lod_transform([8, 10, 12], MV, P, F, [8, 8, 6], linearize_depth=lin)
    assert rel(ref, N(y)) < 1e-5


# -------------------------------------------------------------------- raymarch
BLENDS = ["BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"]


@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("blend", BLENDS)
def test_raymarch(C, bm, blend):
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    x = (RNG.uniform(0, 1, (1, 10, 12, 14, C)) * 0.3).astype(np.float32)
    y = ngt().raymarch_grid_transform(T(x), M, V, P, F, [10, 8, 6], "LINEAR", bm, blend)
    ref = oops.raymarch_grid_transform(x, M, V, P, F, [10, 8, 6], "LINEAR", bm, blend)
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    gx = ngt().raymarch_grid_transform_grad(T(x), y, T(gy), M, V, P, F, [10, 8, 6], "LINEAR", bm, blend,
                                            grad_mode="exact")
    rx = oops.raymarch_grid_transform_grad(x, ref, gy, M, V, P, F, [10, 8, 6], "LINEAR", bm, blend, grad_mode="exact")
    assert rel(rx, N(gx)) < 1e-4
    gx = ngt().raymarch_grid_transform_grad(T(x), y, T(gy), M, V, P, F, [10, 8, 6], "LINEAR", bm, blend,
                                            grad_mode="reference")
    rx = oops.raymarch_grid_transform_grad(x, ref, gy, M, V, P, F, [10, 8, 6], "LINEAR", bm, blend,
                                           grad_mode="reference")
    assert rel(rx, N(gx)) < 5e-4


@pytest.mark.parametrize("C", [2, 4])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
def test_raymarch_signed_extinction(C, bm):
    """Exact Beer-Lambert gradients when extinction samples can be negative (the
    max(d + sigma, 0) clamp can switch): the checkpointed backward, against the
    oracle; and a one-channel density under a negative extinction scale."""
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    x = RNG.uniform(-0.25, 0.3, (1, 10, 12, 14, C)).astype(np.float32)
    y = ngt().raymarch_grid_transform(T(x), M, V, P, F, [10, 8, 6], "LINEAR", bm, "BEER_LAMBERT")
    ref = oops.raymarch_grid_transform(x, M, V, P, F, [10, 8, 6], "LINEAR", bm, "BEER_LAMBERT")
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    gx = ngt().raymarch_grid_transform_grad(T(x), y, T(gy), M, V, P, F, [10, 8, 6], "LINEAR", bm, "BEER_LAMBERT",
                                            grad_mode="exact")
    rx = oops.raymarch_grid_transform_grad(x, ref, gy, M, V, P, F, [10, 8, 6], "LINEAR", bm, "BEER_LAMBERT",
                                           grad_mode="exact")
    assert rel(rx, N(gx)) < 1e-4
    rho = RNG.uniform(0, 0.3, (1, 10, 12, 14, 1)).astype(np.float32)
    scale = [0.7, -0.4]
    full = (rho * np.asarray(scale, np.float32)).astype(np.float32)
    rt = T(rho).requires_grad_()
    y = ngt().raymarch_grid_transform(rt, M, V, P, F, [10, 8, 6], boundary=bm, emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, [10, 8, 6], boundary=bm)
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    y.backward(T(gy))
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, [10, 8, 6], boundary=bm, grad_mode="exact")
    assert rel((gfull * np.asarray(scale)).sum(-1, keepdims=True), N(rt.grad)) < 1e-4


def _ray_direct_and_quad(x, M, V, P, F, shape, bm, blend):
    """Raymarch forward through the C ABI twice: without a workspace (each block
    forms its camera, direct gathers) and with one (cameras formed once, quad
    layout gathers)."""
    import ctypes
    from ngt_gb300 import _lib as L
    ops = ngt()
    attrs = dict(interpolation="LINEAR", boundary=bm, blending_mode=blend, keep_dims=False,
                 separate_camera_batch=True, emission_scale=None)
    dev = x.device
    Mt, Vt, Pt, Ft = (ops._floats(m, w, dev) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6)))
    outs = []
    for with_ws in (False, True):
        out = torch.empty(ops._ray_out_shape(x, Vt, shape, attrs), dtype=torch.float32, device=dev)
        r = ops._ray_args(x, Mt, Vt, Pt, Ft, shape, out, attrs)
        ws = None
        if with_ws:
            ws = torch.empty(int(L.load().ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))), dtype=torch.uint8,
                             device=dev)
            r.workspace, r.workspace_bytes = ops._ptr(ws), ws.numel()
        L.call("ngt_raymarch_fwd", ctypes.byref(r), ops._stream())
        torch.cuda.synchronize()
        outs.append(out)
    return outs


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("blend", BLENDS)
def test_raymarch_quad_layout(dtype, bm, blend):
    """One-channel input: the quad-layout gathers match the direct gathers (bit
    for bit except Beer-Lambert, whose quad loop contracts to FMAs and uses the
    fast exponential), and forward and exact gradient match the oracle on the
    stored values."""
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    x32 = (RNG.uniform(0, 1, (1, 10, 12, 14, 1)) * 0.3).astype(np.float32)
    xt = T(x32, dtype)
    xs = N(xt.float())
    direct, quad = _ray_direct_and_quad(xt, M, V, P, F, [10, 8, 6], bm, blend)
    # Beer-Lambert through the quad layout uses FMA lerps and the fast exponential
    assert rel(N(direct), N(quad)) < 2e-6
    ref = oops.raymarch_grid_transform(xs, M, V, P, F, [10, 8, 6], "LINEAR", bm, blend)
    assert rel(ref, N(quad)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    gx = ngt().raymarch_grid_transform_grad(xt, quad, T(gy), M, V, P, F, [10, 8, 6], "LINEAR", bm, blend,
                                            grad_mode="exact")
    rx = oops.raymarch_grid_transform_grad(xs, ref, gy, M, V, P, F, [10, 8, 6], "LINEAR", bm, blend,
                                           grad_mode="exact")
    assert rel(rx, N(gx)) < 1e-4


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("signed", [False, True])
def test_raymarch_prepared_quad(dtype, bm, signed):
    """A quad layout prepared once (ngt_raymarch_quad) and handed to the forward
    and the exact backward gives the forward bit for bit and the gradient of
    the calls that build their own; with negative densities its sign word sends
    the backward to the checkpointed adjoint, as the own build's does."""
    import ctypes
    from ngt_gb300 import _lib as L
    ops = ngt()
    lib = L.load()
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    x32 = (RNG.uniform(0, 1, (1, 10, 12, 14, 1)) * 0.3).astype(np.float32) - np.float32(0.1 if signed else 0.0)
    xt = T(x32, dtype)
    Md, Vd, Pd, Fd = (ops._floats(m, w, xt.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6)))
    attrs = dict(interpolation="LINEAR", boundary=bm, blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=(0.6, 1.2))
    stream = ops._stream()

    def run(prepared):
        y = torch.empty((1, 3, 8, 6, 2), device="cuda")
        r = ops._ray_args(xt, Md, Vd, Pd, Fd, [10, 8, 6], y, attrs)
        quad = None
        if prepared:
            quad = torch.empty(int(lib.ngt_raymarch_quad_bytes(ctypes.byref(r))), dtype=torch.uint8, device="cuda")
            assert lib.ngt_raymarch_quad(ctypes.byref(r), ops._ptr(quad), stream) == L.NGT_OK
            r.quad = ops._ptr(quad)
        ws = torch.empty(int(lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))) + 1, dtype=torch.uint8,
                         device="cuda")
        r.workspace, r.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_raymarch_fwd(ctypes.byref(r), stream) == L.NGT_OK
        g = L.RaymarchGradArgs()
        g.fwd = r
        g.fwd.workspace, g.fwd.workspace_bytes = None, 0
        gy = torch.as_tensor(np.random.default_rng(3).standard_normal((1, 3, 8, 6, 2)).astype(np.float32),
                             device="cuda")
        gx = torch.empty((1, 10, 12, 14, 1), device="cuda")
        g.output, g.output_grad, g.input_grad, g.grad_mode = ops._ptr(y), ops._ptr(gy), ops._ptr(gx), L.GRAD["exact"]
        gws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                          device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(gws), gws.numel()
        assert lib.ngt_raymarch_bwd(ctypes.byref(g), stream) == L.NGT_OK
        torch.cuda.synchronize()
        flag = int(quad[:4].view(torch.int32).item()) if prepared else None
        return y, gx, flag, ws.numel(), gws.numel()

    y0, g0, _, fw0, bw0 = run(False)
    y1, g1, flag, fw1, bw1 = run(True)
    assert torch.equal(y0, y1)
    assert rel(N(g0), N(g1)) < 1e-6
    assert (flag != 0) == signed
    assert fw1 < fw0 and bw1 < bw0  # the prepared layout is not sized again


@pytest.mark.parametrize("case", ["quad_f32", "emission_f64", "two_channel_f32"])
def test_raymarch_fwd_fused_l2(case):
    """ngt_raymarch_fwd_l2 against ngt_raymarch_fwd followed by
    ngt_image_l2_loss: the same image and image gradient bit for bit, the loss
    up to the order of its additions."""
    import ctypes
    from ngt_gb300 import _lib as L
    ops = ngt()
    lib = L.load()
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    dt = torch.float64 if case == "emission_f64" else torch.float32
    C = 2 if case == "two_channel_f32" else 1
    x = T((RNG.uniform(0, 1, (1, 10, 12, 14, C)) * 0.3).astype(np.float32), dt)
    Md, Vd, Pd, Fd = (ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6)))
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=None if C == 2 else (0.6, 1.2))
    tgt = torch.as_tensor(RNG.uniform(0, 0.2, (1, 3, 8, 6, 1)), device="cuda", dtype=dt)
    stream = ops._stream()

    def run(fused):
        y = torch.empty((1, 3, 8, 6, 2), device="cuda", dtype=dt)
        gy = torch.full_like(y, float("nan"))
        loss = torch.zeros((1,), device="cuda", dtype=dt)
        r = ops._ray_args(x, Md, Vd, Pd, Fd, [10, 8, 6], y, attrs)
        ws = torch.empty(max(int(lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))), 1), dtype=torch.uint8,
                         device="cuda")
        r.workspace, r.workspace_bytes = ops._ptr(ws), ws.numel()
        if fused:
            rc = lib.ngt_raymarch_fwd_l2(ctypes.byref(r), ops._ptr(tgt), 1, ops._ptr(gy), ops._ptr(loss), stream)
            assert rc == L.NGT_OK, lib.ngt_last_error_message()
        else:
            assert lib.ngt_raymarch_fwd(ctypes.byref(r), stream) == L.NGT_OK
            assert lib.ngt_image_l2_loss(ops._code(y), 3 * 8 * 6, 2, 1, ops._ptr(y), ops._ptr(tgt), ops._ptr(gy),
                                         ops._ptr(loss), stream) == L.NGT_OK
        torch.cuda.synchronize()
        return y, gy, float(loss.item())

    y0, g0, l0 = run(False)
    y1, g1, l1 = run(True)
    assert torch.equal(y0, y1) and torch.equal(g0, g1)
    assert abs(l1 - l0) <= 1e-6 * abs(l0) and l0 > 0
    want = 0.5 * float(((y0[..., :1] - tgt) ** 2).sum())
    assert abs(l1 - want) <= 1e-5 * want


@pytest.mark.parametrize("sep", [True, False])
def test_raymarch_prepared_quad_batches(sep):
    """Two grids in one call (per-batch quad layouts in one prepared buffer), with
    cameras per batch or shared, forward with the fused loss and exact backward:
    against the oracle."""
    import ctypes
    from ngt_gb300 import _lib as L
    ops = ngt()
    lib = L.load()
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6), yaws=(13, -47))
    M2 = np.concatenate([M, M])
    x = (RNG.uniform(0, 1, (2, 10, 12, 14, 1)) * 0.3).astype(np.float32)
    xt = T(x)
    Md, Vd, Pd, Fd = (ops._floats(m, w, xt.device) for m, w in ((M2, 16), (V, 16), (P, 16), (F, 6)))
    attrs = dict(interpolation="LINEAR", boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=sep, emission_scale=(0.6, 1.2))
    shape = ops._ray_out_shape(xt, Vd, [10, 8, 6], attrs)
    y = torch.empty(shape, device="cuda")
    r = ops._ray_args(xt, Md, Vd, Pd, Fd, [10, 8, 6], y, attrs)
    quad = torch.empty(int(lib.ngt_raymarch_quad_bytes(ctypes.byref(r))), dtype=torch.uint8, device="cuda")
    stream = ops._stream()
    assert lib.ngt_raymarch_quad(ctypes.byref(r), ops._ptr(quad), stream) == L.NGT_OK
    r.quad = ops._ptr(quad)
    tgt = T(RNG.uniform(0, 0.1, shape[:-1] + (1,)).astype(np.float32))
    gy = torch.empty_like(y)
    loss = torch.zeros((1,), device="cuda")
    assert lib.ngt_raymarch_fwd_l2(ctypes.byref(r), ops._ptr(tgt), 1, ops._ptr(gy), ops._ptr(loss), stream) == 0
    g = L.RaymarchGradArgs()
    g.fwd = r
    gx = torch.empty_like(xt)
    g.output, g.output_grad, g.input_grad, g.grad_mode = ops._ptr(y), ops._ptr(gy), ops._ptr(gx), L.GRAD["exact"]
    ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8, device="cuda")
    g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), stream) == L.NGT_OK
    torch.cuda.synchronize()
    full = (x * np.asarray([0.6, 1.2], np.float32)).astype(np.float32)
    ref = oops.raymarch_grid_transform(full, M2, V, P, F, [10, 8, 6], separate_camera_batch=sep)
    assert rel(ref, N(y)) < 2e-5
    gimg = np.concatenate([ref[..., :1] - N(tgt), np.zeros_like(ref[..., :1])], -1)
    assert rel(gimg, N(gy)) < 1e-4
    rx = oops.raymarch_grid_transform_grad(full, ref, gimg, M2, V, P, F, [10, 8, 6], separate_camera_batch=sep,
                                           grad_mode="exact")
    assert rel((rx * np.asarray([0.6, 1.2])).sum(-1, keepdims=True), N(gx)) < 1e-4


def test_raymarch_autograd_signed_extinction_emission():
    """Autograd over the emission-expanded one-channel raymarch keeps the
    forward's quad layout for the backward; with negative densities its sign
    word selects the checkpointed adjoint (against the oracle)."""
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    rho = (RNG.uniform(0, 1, (1, 10, 12, 14, 1)) * 0.3 - 0.08).astype(np.float32)
    scale = [0.7, 1.3]
    full = (rho * np.asarray(scale, np.float32)).astype(np.float32)
    rt = T(rho).requires_grad_()
    y = ngt().raymarch_grid_transform(rt, M, V, P, F, [10, 8, 6], emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, [10, 8, 6])
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    y.backward(T(gy))
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, [10, 8, 6], grad_mode="exact")
    assert rel((gfull * np.asarray(scale)).sum(-1, keepdims=True), N(rt.grad)) < 1e-4


def test_host_matrix_and_camera_caches():
    """Host matrices are uploaded once per content (a changed array uploads
    again), cameras and ray tables formed from cached uploads are reused, and
    results match the call given device matrices (cameras formed per call, rays
    set up per ray in float arithmetic instead of taken from the double-precision
    table: the same images to a few float roundings)."""
    ops = ngt()
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    dev = torch.device("cuda", 0)
    a = ops._floats(M, 16, dev)
    assert ops._floats(M.copy(), 16, dev) is a
    M2 = M.copy()
    M2[0, 12] += 0.25
    b = ops._floats(M2, 16, dev)
    assert b is not a and not torch.equal(a, b)
    x = T((RNG.uniform(0, 1, (1, 10, 12, 14, 1)) * 0.3).astype(np.float32)).requires_grad_()
    y1 = ops.raymarch_grid_transform(x, M, V, P, F, [10, 8, 6], emission_scale=(0.5, 1.0))
    n_cams, n_rays = len(ops._CAMERAS), len(ops._RAYS)
    y2 = ops.raymarch_grid_transform(x, M, V, P, F, [10, 8, 6], emission_scale=(0.5, 1.0))
    assert len(ops._CAMERAS) == n_cams and len(ops._RAYS) == n_rays and torch.equal(y1, y2)
    y3 = ops.raymarch_grid_transform(x, torch.as_tensor(M, device=dev), torch.as_tensor(V, device=dev),
                                     torch.as_tensor(P, device=dev), torch.as_tensor(F, device=dev), [10, 8, 6],
                                     emission_scale=(0.5, 1.0))
    assert rel(N(y3), N(y1)) < 1e-5
    g = T(RNG.standard_normal(tuple(y1.shape)).astype(np.float32))
    ga, = torch.autograd.grad(y1, x, g)
    gb, = torch.autograd.grad(y3, x, g)
    assert rel(N(gb), N(ga)) < 1e-5
    # moved to the new matrix content: a different image
    y4 = ops.raymarch_grid_transform(x, M2, V, P, F, [10, 8, 6], emission_scale=(0.5, 1.0))
    assert not torch.equal(y1, y4)
    # a call on another stream reuses the entries made on the default stream
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        y5 = ops.raymarch_grid_transform(x.detach(), M, V, P, F, [10, 8, 6], emission_scale=(0.5, 1.0))
    torch.cuda.current_stream(dev).wait_stream(side)
    assert len(ops._CAMERAS) >= n_cams and torch.equal(y1, y5)


@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("dhw", [(1, 5, 6), (7, 1, 4), (5, 6, 1)])
def test_raymarch_thin_grids(bm, dhw):
    """Grids one cell thick along an axis (the quad layout's padding then maps
    both padding coordinates onto the same cell under CLAMP and WRAP)."""
    M, V, P, F = scene_mats(vol_dhw=dhw, cam_dhw=(10, 8, 6))
    x = (RNG.uniform(0, 1, (1,) + dhw + (1,)) * 0.5).astype(np.float32)
    scale = [0.8, 1.1]
    full = (x * np.asarray(scale, np.float32)).astype(np.float32)
    xt = T(x).requires_grad_()
    y = ngt().raymarch_grid_transform(xt, M, V, P, F, [10, 8, 6], boundary=bm, emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, [10, 8, 6], boundary=bm)
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    y.backward(T(gy))
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, [10, 8, 6], boundary=bm, grad_mode="exact")
    assert rel((gfull * np.asarray(scale)).sum(-1, keepdims=True), N(xt.grad)) < 1e-4


def test_raymarch_nearest_and_batches():
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    M2 = np.concatenate([M, M])
    x = (RNG.uniform(0, 1, (2, 10, 12, 14, 2)) * 0.3).astype(np.float32)
    y = ngt().raymarch_grid_transform(T(x), M2, V, P, F, [10, 8, 6], "NEAREST", "BORDER", "BEER_LAMBERT")
    ref = oops.raymarch_grid_transform(x, M2, V, P, F, [10, 8, 6], "NEAREST", "BORDER", "BEER_LAMBERT")
    assert np.isclose(N(y), ref, rtol=1e-5, atol=1e-6).all(-1).mean() > 0.97
    y = ngt().raymarch_grid_transform(T(x), M2, V[:2], P[:2], F[:2], [10, 8, 6], "LINEAR", "BORDER", "BEER_LAMBERT",
                                      separate_camera_batch=False)
    ref = oops.raymarch_grid_transform(x, M2, V[:2], P[:2], F[:2], [10, 8, 6], "LINEAR", "BORDER", "BEER_LAMBERT",
                                       separate_camera_batch=False)
    assert rel(ref, N(y)) < 2e-5


@pytest.mark.parametrize("cb", [2, 4])
def test_raymarch_emission_expansion(cb):
    """A one-channel density with per-channel scales equals the materialised light grid."""
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    rho = (RNG.uniform(0, 1, (1, 10, 12, 14, 1)) * 0.3).astype(np.float32)
    scale = [0.7, 1.3] if cb == 2 else [0.2, 0.5, 0.9, 1.3]
    full = (rho * np.asarray(scale, np.float32)).astype(np.float32)
    rt = T(rho).requires_grad_()
    y = ngt().raymarch_grid_transform(rt, M, V, P, F, [10, 8, 6], emission_scale=scale)
    ref = oops.raymarch_grid_transform(full, M, V, P, F, [10, 8, 6])
    assert rel(ref, N(y)) < 2e-5
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    y.backward(T(gy))
    gfull = oops.raymarch_grid_transform_grad(full, ref, gy, M, V, P, F, [10, 8, 6], grad_mode="exact")
    assert rel((gfull * np.asarray(scale)).sum(-1, keepdims=True), N(rt.grad)) < 1e-4


# ---------------------------------------------------------------- reduce blend
@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("blend", BLENDS)
@pytest.mark.parametrize("kd", [False, True])
def test_reduce_blend(C, blend, kd):
    x = RNG.uniform(0, 0.3, (2, 9, 5, 6, C)).astype(np.float32)
    y = ngt().reduce_grid_blend(T(x), blend, kd)
    ref = oops.reduce_grid_blend(x, blend, kd)
    assert rel(ref, N(y)) < 1e-6
    gy = RNG.standard_normal(ref.shape).astype(np.float32)
    for mode in ("exact", "reference"):
        gx = ngt().reduce_grid_blend_grad(T(gy), y, T(x), blend, kd, grad_mode=mode)
        rx = oops.reduce_grid_blend_grad(gy, ref, x, blend, kd, grad_mode=mode)
        assert rel(rx, N(gx)) < 1e-5


# -------------------------------------------------------------------- advection
def advect_inputs(shape=(10, 12, 14), max_u=2.0, seed=11, dtype=np.float32):
    from ngt_gb300 import synthetic
    rho = synthetic.gaussian_blobs(shape, n=4, sigma=(2, 4), seed=seed, dtype=dtype)
    ux, uy, uz = synthetic.curl_noise_mac(shape, max_u=max_u, seed=seed + 1, smooth=2.0, dtype=dtype)
    return rho, ux, uy, uz


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (2, "NONE"), (1, "NONE"), (1, "NEGATIVE"), (2, "NEGATIVE")])
def test_advect_forward_bitexact(bm, order, clamp):
    from ngt_gb300 import advect
    rho, ux, uy, uz = advect_inputs()
    y = advect.warp(T(rho), T(ux), T(uy), T(uz), dt=1.0, order=order, clamp=clamp, boundary=bm)
    ref = oadvect.density_maccormack(rho, ux, uy, uz, 1.0, order, clamp, bm)
    assert np.array_equal(N(y), ref)


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER"])
@pytest.mark.parametrize("mode", ["exact", "reference"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NONE"), (2, "NEGATIVE")])
def test_advect_backward(bm, mode, order, clamp):
    from ngt_gb300 import advect, ops
    rho, ux, uy, uz = advect_inputs(seed=13)
    g = RNG.standard_normal(rho.shape).astype(np.float32)
    ts = [T(a).requires_grad_() for a in (rho, ux, uy, uz)]
    with ops.gradient_mode(mode):
        y = advect.warp(*ts, dt=1.0, order=order, clamp=clamp, boundary=bm)
        y.backward(T(g))
    ref = oadvect.density_maccormack_grad(rho, ux, uy, uz, g, 1.0, order, clamp, bm, grad_mode=mode)
    for t, r in zip(ts, ref):
        assert rel(r, N(t.grad)) < 1e-4


def test_advect_float64_matches_oracle():
    from ngt_gb300 import advect
    rho, ux, uy, uz = advect_inputs(dtype=np.float64)
    g = RNG.standard_normal(rho.shape)
    ts = [T(a, torch.float64).requires_grad_() for a in (rho, ux, uy, uz)]
    y = advect.warp(*ts)
    y.backward(T(g, torch.float64))
    assert rel(oadvect.density_maccormack(rho, ux, uy, uz), N(y)) < 1e-13
    ref = oadvect.density_maccormack_grad(rho, ux, uy, uz, g)
    for t, r in zip(ts, ref):
        assert rel(r, N(t.grad)) < 1e-11


# ------------------------------------------------------- velocity self-advection
@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NONE")])
def test_velocity_advect_forward_bitexact(bm, order, clamp):
    from ngt_gb300 import advect
    _, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=17)
    out = advect.warp_velocity(T(ux), T(uy), T(uz), dt=1.0, order=order, clamp=clamp, boundary=bm)
    ref = oadvect.velocity_maccormack(ux, uy, uz, 1.0, order, clamp, bm)
    for o, r in zip(out, ref):
        assert np.array_equal(N(o), r)


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NONE")])
def test_velocity_advect_backward_deterministic(bm, order, clamp):
    """Velocity self-advection with the deterministic adjoint (fixed-point trace
    adjoints per face component): the same bits on every run and the oracle's
    gradients."""
    from ngt_gb300 import advect, ops
    _, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=41)
    gs = [RNG.standard_normal(u.shape).astype(np.float32) for u in (ux, uy, uz)]
    runs = []
    for _ in range(2):
        ts = [T(u).requires_grad_() for u in (ux, uy, uz)]
        ops.set_deterministic(True)
        try:
            out = advect.warp_velocity(*ts, order=order, clamp=clamp, boundary=bm)
            torch.autograd.backward(out, [T(g) for g in gs])
        finally:
            ops.set_deterministic(False)
        runs.append([t.grad for t in ts])
    for a, b in zip(*runs):
        assert torch.equal(a, b)
    ref = oadvect.velocity_maccormack_grad(ux, uy, uz, gs, order=order, clamp=clamp, boundary=bm)
    for t, r in zip(runs[0], ref):
        assert rel(r, N(t)) < 1e-4


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("mode", ["exact", "reference"])
def test_velocity_advect_backward(bm, mode):
    from ngt_gb300 import advect, ops
    _, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=19)
    gs = [RNG.standard_normal(u.shape).astype(np.float32) for u in (ux, uy, uz)]
    ts = [T(u).requires_grad_() for u in (ux, uy, uz)]
    with ops.gradient_mode(mode):
        out = advect.warp_velocity(*ts, boundary=bm)
        torch.autograd.backward(out, [T(g) for g in gs])
    ref = oadvect.velocity_maccormack_grad(ux, uy, uz, gs, boundary=bm, grad_mode=mode)
    for t, r in zip(ts, ref):
        assert rel(r, N(t.grad)) < 1e-4


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("shape", [(1, 6, 7), (5, 1, 6), (4, 6, 1)])
def test_velocity_advect_backward_single_cell_axis(bm, shape):
    """Grids one cell thick along an axis: the lookup adjoint's clamped and wrapped
    corners of both edges land on the same faces."""
    from ngt_gb300 import advect
    _, ux, uy, uz = advect_inputs(shape=shape, seed=23, max_u=1.0)
    gs = [RNG.standard_normal(u.shape).astype(np.float32) for u in (ux, uy, uz)]
    ts = [T(u).requires_grad_() for u in (ux, uy, uz)]
    out = advect.warp_velocity(*ts, boundary=bm)
    torch.autograd.backward(out, [T(g) for g in gs])
    ref = oadvect.velocity_maccormack_grad(ux, uy, uz, gs, boundary=bm, grad_mode="exact")
    for t, r in zip(ts, ref):
        assert rel(r, N(t.grad)) < 1e-4


# ------------------------------------------------------------- deterministic mode
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("sep", [True, False])
def test_lut_backward_deterministic(bm, sep):
    x, lut, kw = lut_inputs("rel", 2, seed=5)
    lut = lut * np.float32(2.0)  # several samples per bucket
    gy = RNG.standard_normal(oops.sample_grid_lut(x, lut, "LINEAR", bm, separate_camera_batch=sep,
                                                  **kw).shape).astype(np.float32)
    runs = [ngt().sample_grid_lut_grad(T(x), T(gy), T(lut), interpolation="LINEAR", boundary=bm,
                                       separate_camera_batch=sep, grad_mode="exact", deterministic=True, **kw)
            for _ in range(2)]
    assert torch.equal(runs[0][0], runs[1][0]) and torch.equal(runs[0][1], runs[1][1])
    rx, rl = oops.sample_grid_lut_grad(x, gy, lut, "LINEAR", bm, separate_camera_batch=sep, grad_mode="exact", **kw)
    assert rel(rx, N(runs[0][0])) < 1e-5
    assert rel(rl, N(runs[0][1])) < 1e-5


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
def test_advect_backward_deterministic(bm):
    from ngt_gb300 import advect, ops
    rho, ux, uy, uz = advect_inputs(shape=(12, 14, 16), seed=23)
    g = RNG.standard_normal(rho.shape).astype(np.float32)
    grads = []
    for _ in range(2):
        ts = [T(a).requires_grad_() for a in (rho, ux, uy, uz)]
        ops.set_deterministic(True)
        try:
            y = advect.warp(*ts, boundary=bm)
            y.backward(T(g))
        finally:
            ops.set_deterministic(False)
        grads.append([t.grad for t in ts])
    for a, b in zip(*grads):
        assert torch.equal(a, b)
    ref = oadvect.density_maccormack_grad(rho, ux, uy, uz, g, boundary=bm)
    for t, r in zip(grads[0], ref):
        assert rel(r, N(t)) < 1e-4


@pytest.mark.parametrize("C,dtype,order,clamp", [(2, np.float32, 2, "MC_SMOOTH"), (4, np.float32, 2, "NONE"),
                                                  (1, np.float64, 2, "MC_SMOOTH"), (1, np.float32, 1, "NEGATIVE")])
def test_advect_backward_deterministic_channels(C, dtype, order, clamp):
    """The deterministic MacCormack adjoint (64-bit fixed-point sums of both trace
    adjoints) with several channels, double storage and first order: the same
    bits on every run, the oracle's gradients (f64 at 1e-10: each contribution is
    resolved to 2^(en - 62) of the largest), and a NaN in the upstream gradient
    reaching the gradients."""
    from ngt_gb300 import advect, ops
    rho, ux, uy, uz = advect_inputs(shape=(9, 11, 13), seed=31, dtype=dtype)
    rho = np.concatenate([rho * dtype(k + 1) for k in range(C)], -1)
    g = RNG.standard_normal(rho.shape).astype(dtype)
    td = torch.float64 if dtype == np.float64 else torch.float32

    def run(gup):
        ts = [T(a, td).requires_grad_() for a in (rho, ux, uy, uz)]
        ops.set_deterministic(True)
        try:
            y = advect.warp(*ts, order=order, clamp=clamp, boundary="CLAMP")
            y.backward(T(gup, td))
        finally:
            ops.set_deterministic(False)
        return [t.grad for t in ts]

    a, b = run(g), run(g)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    ref = oadvect.density_maccormack_grad(rho, ux, uy, uz, g, order=order, clamp=clamp, boundary="CLAMP")
    for t, r in zip(a, ref):
        assert rel(r, N(t)) < (1e-10 if dtype == np.float64 else 1e-4)
    gn = g.copy()
    gn[4, 5, 6, 0] = np.nan
    assert all(bool(torch.isnan(t).any()) for t in run(gn)[:1])


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("C", [1, 2, 4])
def test_advect_stored_extrema_bitexact(bm, C):
    """MacCormack forward with the corner extrema and the lookup handed from
    forward 1 to forward 2 against the forward forming them again: identical
    outputs, masks and forward fields."""
    import ctypes
    from ngt_gb300 import _lib as L
    from ngt_gb300 import advect
    ops = ngt()
    rho, ux, uy, uz = advect_inputs(shape=(9, 12, 14), seed=37)
    rho = np.concatenate([rho * (k + 1) for k in range(C)], -1) - np.float32(0.05)
    ts = [T(a) for a in (rho, ux, uy, uz)]
    res = []
    for with_ext in (False, True):
        out = torch.empty_like(ts[0])
        fwd = torch.empty_like(ts[0])
        mask = torch.empty(ts[0].shape, dtype=torch.uint8, device="cuda")
        ext = torch.empty(ts[0].shape[:3] + (2 * C,), device="cuda") if with_ext else None
        a = advect._args(*ts, out, fwd, 1.0, 2, "MC_SMOOTH", bm, mask, ext)
        if with_ext:  # with the stored lookup too
            lut = torch.empty(ts[0].shape[:3] + (3,), device="cuda")
            a.lookup = ops._ptr(lut)
        assert L.load().ngt_advect_maccormack_fwd(ctypes.byref(a), ops._stream()) == L.NGT_OK
        torch.cuda.synchronize()
        res.append((out, fwd, mask))
    for a, b in zip(*res):
        assert torch.equal(a, b)
    assert int(res[0][2].sum()) > 0


@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NEGATIVE"), (2, "NONE")])
def test_advect_backward_stored_lookup(order, clamp):
    """The MacCormack backward reading the lookup that forward 1 stored against
    the backward averaging the faces again."""
    import ctypes
    from ngt_gb300 import _lib as L
    from ngt_gb300 import advect
    ops = ngt()
    lib = L.load()
    rho, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=47)
    ts = [T(a) for a in (rho, ux, uy, uz)]
    gy = T(RNG.standard_normal(rho.shape).astype(np.float32))
    res = []
    for stored in (False, True):
        out, fwd = torch.empty_like(ts[0]), torch.empty_like(ts[0])
        a = advect._args(*ts, out, fwd, 1.0, order, clamp, "CLAMP")
        lut = torch.empty(ts[0].shape[:3] + (3,), device="cuda")
        if stored:
            a.lookup = ops._ptr(lut)
        assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), ops._stream()) == L.NGT_OK
        g = L.AdvectGradArgs()
        g.fwd = a
        grads = [torch.empty_like(t) for t in ts]
        g.output_grad = ops._ptr(gy)
        g.data_grad, g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (ops._ptr(t) for t in grads)
        g.grad_mode = L.GRAD["exact"]
        ws = torch.empty(int(lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                         device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_advect_maccormack_bwd(ctypes.byref(g), ops._stream()) == L.NGT_OK
        torch.cuda.synchronize()
        res.append((out, grads))
    assert torch.equal(res[0][0], res[1][0])
    for a_, b_ in zip(res[0][1], res[1][1]):
        assert rel(N(a_), N(b_)) < 1e-6


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
def test_advect_stored_mask_matches_recomputed(bm):
    """The backward reading the forward's stored MC_SMOOTH mask equals the
    backward recomputing it from the corner extrema."""
    from ngt_gb300 import advect
    rho, ux, uy, uz = advect_inputs(shape=(12, 14, 16), seed=29)
    ts = [T(a) for a in (rho, ux, uy, uz)]
    g = T(RNG.standard_normal(rho.shape).astype(np.float32))
    out, fwd, mask = advect.warp_forward(*ts, boundary=bm, keep_mask=True)
    out2, _, _ = advect.warp_forward(*ts, boundary=bm)
    assert torch.equal(out, out2)
    assert int(mask.sum()) > 0
    a = advect.warp_backward(*ts, fwd, g, boundary=bm, mask=mask)
    b = advect.warp_backward(*ts, fwd, g, boundary=bm)
    for x, y in zip(a, b):
        assert rel(N(y), N(x)) < 1e-6


@pytest.mark.parametrize("C,emission", [(1, (0.6, 1.2)), (2, None), (1, None)])
def test_raymarch_backward_accumulates(C, emission):
    """accumulate = 1 adds the exact input gradient to what input_grad holds
    (quad layout and direct paths)."""
    import ctypes
    from ngt_gb300 import _lib as L
    ops = ngt()
    lib = L.load()
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    x = T((RNG.uniform(0, 1, (1, 10, 12, 14, C)) * 0.3).astype(np.float32))
    Md, Vd, Pd, Fd = (ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6)))
    attrs = dict(interpolation="LINEAR", boundary="CLAMP", blending_mode="BEER_LAMBERT", keep_dims=False,
                 separate_camera_batch=True, emission_scale=emission)
    y, _ = ops._ray_forward(x, Md, Vd, Pd, Fd, [10, 8, 6], attrs)
    gy = T(RNG.standard_normal(tuple(y.shape)).astype(np.float32))
    want = ops._ray_backward(x, y, gy, Md, Vd, Pd, Fd, [10, 8, 6], attrs, "exact")
    base = T(RNG.standard_normal(tuple(want.shape)).astype(np.float32))
    got = base.clone()
    for _ in range(2):
        g = L.RaymarchGradArgs()
        g.fwd = ops._ray_args(x, Md, Vd, Pd, Fd, [10, 8, 6], None, attrs)
        g.output, g.output_grad, g.input_grad, g.grad_mode = ops._ptr(y), ops._ptr(gy), ops._ptr(got), L.GRAD["exact"]
        g.accumulate = 1
        ws = torch.empty(int(lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))) + 1, dtype=torch.uint8,
                         device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_raymarch_bwd(ctypes.byref(g), ops._stream()) == L.NGT_OK
    torch.cuda.synchronize()
    assert rel(N(base + 2 * want), N(got)) < 1e-5


@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NEGATIVE"), (2, "NONE")])
def test_advect_backward_accumulates(order, clamp):
    import ctypes
    from ngt_gb300 import _lib as L
    from ngt_gb300 import advect
    ops = ngt()
    lib = L.load()
    rho, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=41)
    ts = [T(a) for a in (rho, ux, uy, uz)]
    out, fwd, mask = advect.warp_forward(*ts, order=order, clamp=clamp, keep_mask=True)
    gy = T(RNG.standard_normal(tuple(out.shape)).astype(np.float32))
    want = advect.warp_backward(*ts, fwd, gy, order=order, clamp=clamp, mask=mask)
    base = [T(RNG.standard_normal(tuple(w.shape)).astype(np.float32)) for w in want]
    got = [b.clone() for b in base]
    g = L.AdvectGradArgs()
    g.fwd = advect._args(*ts, None, fwd, 1.0, order, clamp, "CLAMP", mask)
    g.output_grad = ops._ptr(gy)
    g.data_grad, g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (ops._ptr(t) for t in got)
    g.grad_mode, g.accumulate = L.GRAD["exact"], 1
    ws = torch.empty(int(lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                     device="cuda")
    g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
    assert lib.ngt_advect_maccormack_bwd(ctypes.byref(g), ops._stream()) == L.NGT_OK
    torch.cuda.synchronize()
    for b, w, a in zip(base, want, got):
        assert rel(N(b + w), N(a)) < 1e-5


@pytest.mark.parametrize("dt", [torch.float32, torch.float64])
def test_image_l2_loss_op(dt):
    ops = ngt()
    img = torch.as_tensor(RNG.uniform(0, 1, (1, 3, 8, 6, 2)), device="cuda", dtype=dt).requires_grad_()
    tgt = torch.as_tensor(RNG.uniform(0, 1, (1, 3, 8, 6, 1)), device="cuda", dtype=dt)
    loss = ops.image_l2_loss(img, tgt)
    want = 0.5 * ((img[..., :1] - tgt) ** 2).sum()
    assert abs(float(loss.detach()) - float(want.detach())) <= 1e-6 * float(want.detach())
    loss.backward(torch.tensor(2.0, device="cuda", dtype=dt))
    gw = torch.zeros_like(img)
    gw[..., :1] = 2.0 * (img[..., :1] - tgt)
    assert torch.allclose(img.grad, gw.detach(), rtol=1e-6, atol=1e-7)
    with pytest.raises(ValueError):
        ops.image_l2_loss(img, tgt.expand(1, 3, 8, 6, 2).contiguous(), loss_channels=1)


@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (2, "NONE"), (1, "NEGATIVE")])
@pytest.mark.parametrize("bm", ["CLAMP", "WRAP", "BORDER"])
def test_velocity_advection_stored_lookup(order, clamp, bm):
    """MAC self-advection with the per-component lookups (and MC_SMOOTH mask and
    extrema) kept from forward 1 against resampling them in every kernel: the
    same outputs bit for bit, the same gradients up to atomic order."""
    import ctypes
    from ngt_gb300 import _lib as L
    from ngt_gb300 import advect
    ops = ngt()
    lib = L.load()
    _, ux, uy, uz = advect_inputs(shape=(9, 10, 11), seed=43)
    u = [T(a) for a in (ux, uy, uz)]
    gin = [T(RNG.standard_normal(t.shape).astype(np.float32)) for t in u]
    res = []
    for stored in (False, True):
        outs = [torch.empty_like(t) for t in u]
        fwds = [torch.empty_like(t) for t in u]
        scratch = advect._vel_scratch(u, order, clamp) if stored else None
        a = advect._vel_args(*u, outs, fwds, 1.0, order, clamp, bm, scratch)
        assert lib.ngt_advect_velocity_fwd(ctypes.byref(a), ops._stream()) == L.NGT_OK
        g = L.AdvectVelocityGradArgs()
        g.fwd = a
        gu = [torch.empty_like(t) for t in u]
        g.grad_x, g.grad_y, g.grad_z = (ops._ptr(t) for t in gin)
        g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (ops._ptr(t) for t in gu)
        g.grad_mode = L.GRAD["exact"]
        ws = torch.empty(int(lib.ngt_advect_velocity_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                         device="cuda")
        g.workspace, g.workspace_bytes = ops._ptr(ws), ws.numel()
        assert lib.ngt_advect_velocity_bwd(ctypes.byref(g), ops._stream()) == L.NGT_OK
        torch.cuda.synchronize()
        res.append((outs, gu))
    for a, b in zip(res[0][0], res[1][0]):
        assert torch.equal(a, b)
    for a, b in zip(res[0][1], res[1][1]):
        assert rel(N(a), N(b)) < 1e-6


# ------------------------------------------------------------- unprojection
@pytest.mark.parametrize("mode", ["reference", "exact"])
def test_unproject_and_its_gradient(mode):
    """Images scattered into the volume by the ADDITIVE gradient op (renderer.py:372-398)
    match the oracle; its registered gradient w.r.t. the images is the forward
    raymarch of the volume gradient (ops_loader.py:98-118)."""
    M, V, P, F = scene_mats(vol_dhw=(10, 12, 14), cam_dhw=(10, 8, 6))
    img = RNG.uniform(0, 1, (1, 3, 8, 6, 2)).astype(np.float32)
    it = T(img).requires_grad_()
    vol = ngt().unproject(it, M, V, P, F, (10, 12, 14), 10, grad_mode=mode)
    dummy = np.zeros((1, 10, 12, 14, 2), np.float32)
    ref = oops.raymarch_grid_transform_grad(dummy, img, img, M, V, P, F, [10, 8, 6], "LINEAR", "BORDER", "ADDITIVE",
                                            grad_mode=mode)
    assert rel(ref, N(vol)) < (5e-4 if mode == "reference" else 1e-4)
    wv = RNG.standard_normal(ref.shape).astype(np.float32)
    (vol * T(wv)).sum().backward()
    want = oops.raymarch_grid_transform(wv, M, V, P, F, [10, 8, 6], "LINEAR", "BORDER", "ADDITIVE")
    assert rel(want, N(it.grad)) < 2e-5


def test_bf16_density_with_f16_faces():
    """FP16 faces with BF16 density: the warp and its gradients equal the BF16
    warp given the FP16 faces' values widened to FP32 lookups -- checked against
    the FP64 oracle on the stored values (the storage types only round the
    inputs; arithmetic is FP32)."""
    from ngt_gb300 import advect, workloads
    w = workloads.render_step(grid=(20, 24, 28), views=1, image=(8, 8), depth=8, max_u=2.0)
    rho = torch.as_tensor(w.rho, device="cuda").to(torch.bfloat16)
    u = [torch.as_tensor(a, device="cuda").to(torch.float16) for a in (w.ux, w.uy, w.uz)]
    ts = [rho.requires_grad_()] + [t.requires_grad_() for t in u]
    out = advect.warp(*ts, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
    assert out.dtype == torch.bfloat16
    g = torch.as_tensor(RNG.standard_normal(w.rho.shape).astype(np.float32), device="cuda")
    out.float().backward(g)
    r64 = [N(t.detach().double()) for t in ts]
    want = oadvect.density_maccormack(*r64)
    assert rel(want, N(out.float())) < 1e-2
    gw = oadvect.density_maccormack_grad(*r64, N(g).astype(np.float64))
    for t, b in zip(ts, gw):
        assert rel(b, N(t.grad.float())) < 2e-2
