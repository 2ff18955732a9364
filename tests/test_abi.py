"""The C-ABI library: it loads, exports every function ``include/ngt_ops.h``
declares, and its host-side validation rejects bad arguments with a status code
and message before any device work (so these run without a GPU)."""
import ctypes
import os
import re

import pytest

import __graft_entry__

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    __graft_entry__.load_package()
    from ngt_gb300 import _build, _lib
    _build.build_library()
    return _lib.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "ngt_ops.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ngt_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from ngt_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_version(lib):
    assert lib.ngt_version() >= 1


def _lut_args(L, C=1, shape=(1, 4, 4, 4), lut=(1, 2, 2, 2, 4)):
    a = L.SampleLutArgs()
    a.dtype = L.F32
    a.input_shape = L.I64x5(*shape, C)
    a.lookup_shape = L.I64x5(*lut)
    a.input = ctypes.c_void_p(0x1000)
    a.lookup = ctypes.c_void_p(0x2000)
    a.output = ctypes.c_void_p(0x3000)
    a.interpolation, a.boundary = 1, 0
    a.separate_camera_batch = 1
    return a


def test_rejects_three_channels(lib):
    from ngt_gb300 import _lib as L
    a = _lut_args(L, C=3)
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"Channel" in lib.ngt_last_error_message()


def test_rejects_bad_enums_and_shapes(lib):
    from ngt_gb300 import _lib as L
    a = _lut_args(L)
    a.boundary = 7
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    a = _lut_args(L, lut=(1, 2, 2, 2, 3))
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    a = _lut_args(L)
    a.input = None
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    a = _lut_args(L)
    a.normalized_coords, a.cell_center_offset = 1, 0.0
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT


def test_rejects_camera_batch_mismatch(lib):
    from ngt_gb300 import _lib as L
    a = _lut_args(L, shape=(2, 4, 4, 4), lut=(3, 2, 2, 2, 4))
    a.separate_camera_batch = 0
    assert lib.ngt_sample_lut_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"camera batch" in lib.ngt_last_error_message()


def test_raymarch_validation(lib):
    from ngt_gb300 import _lib as L
    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 4, 4, 4, 2)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ctypes.c_void_p(0x1000))
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    r.blending_mode = 1  # BEER_LAMBERT_EXCLUSIVE is not an op attribute value
    assert lib.ngt_raymarch_fwd(ctypes.byref(r), None) == L.NGT_ERR_INVALID_ARGUMENT
    r.blending_mode = 0
    r.emission_channels = 2  # needs a one-channel input
    assert lib.ngt_raymarch_fwd(ctypes.byref(r), None) == L.NGT_ERR_INVALID_ARGUMENT
    g = L.RaymarchGradArgs()
    g.fwd = r
    g.fwd.emission_channels = 0
    g.fwd.interpolation = 0  # gradients are LINEAR only
    g.output_grad = g.input_grad = ctypes.c_void_p(0x1000)
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), None) == L.NGT_ERR_UNSUPPORTED


def test_static_scratch_backward_validates_before_sizing(lib):
    """The static-scratch backward checks the arguments as ngt_raymarch_bwd does
    before it forms its scratch size from the shapes: a negative or absurd shape
    is an invalid argument, not a scratch-size failure."""
    from ngt_gb300 import _lib as L
    g = L.RaymarchGradArgs()
    r = g.fwd
    r.dtype = L.F32
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ctypes.c_void_p(0x1000))
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    g.output = g.output_grad = g.input_grad = ctypes.c_void_p(0x1000)
    for shape in ((1, -4, 4, 4, 1), (1, 1 << 40, 1 << 40, 4, 1), (1, 4, 4, 4, 3)):
        g.fwd.input_shape = L.I64x5(*shape)
        assert lib.ngt_raymarch_bwd_static(ctypes.byref(g), None) == L.NGT_ERR_INVALID_ARGUMENT, shape
    g.fwd.input_shape = L.I64x5(1, 4, 4, 4, 1)
    g.grad_mode = 9
    assert lib.ngt_raymarch_bwd_static(ctypes.byref(g), None) == L.NGT_ERR_INVALID_ARGUMENT


def test_advect_validation(lib):
    from ngt_gb300 import _lib as L
    a = L.AdvectArgs()
    a.dtype = L.F32
    a.grid_dhw = L.I64x3(4, 4, 4)
    a.channels = 1
    for f in ("data", "vel_x", "vel_y", "vel_z", "output"):
        setattr(a, f, ctypes.c_void_p(0x1000))
    a.order, a.clamp, a.boundary = 2, 1, 1
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT  # no fwd_field
    a.order, a.clamp = 3, 0
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    g = L.AdvectGradArgs()
    g.fwd = a
    g.fwd.order = 1
    g.output_grad = g.data_grad = ctypes.c_void_p(0x1000)
    assert lib.ngt_advect_maccormack_bwd(ctypes.byref(g), None) == L.NGT_ERR_WORKSPACE
    assert lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g)) == 4 * 4 * 4 * 4 * 4


def test_workspace_queries(lib):
    from ngt_gb300 import _lib as L
    g = L.SampleLutGradArgs()
    g.fwd = _lut_args(L, shape=(2, 4, 5, 6))
    g.grad_mode = 0
    assert lib.ngt_sample_lut_bwd_workspace_bytes(ctypes.byref(g)) == 0
    g.grad_mode = 1
    assert lib.ngt_sample_lut_bwd_workspace_bytes(ctypes.byref(g)) == 2 * 4 * 5 * 6 * 4
    shape = L.I64x5(1, 8, 8, 8, 2)
    assert lib.ngt_mip_bytes(L.F32, shape, 2) == 4 * 4 * 4 * 2 * 4 + 256  # 512 B level 1, 64 B -> 256 level 2


def test_prepared_quad_validation(lib):
    """The prepared quad layout: sized only for inputs it serves, rejected for
    the others, for misaligned buffers and by the batch entry points -- all
    before any device work."""
    from ngt_gb300 import _lib as L
    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 6, 5, 4, 1)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ctypes.c_void_p(0x1000))
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    # (W+1)(H+1)(D+2) entries of four floats after a 256-byte sign word
    n = 256 + ((5 * 6 * 8 * 16 + 255) // 256) * 256
    assert lib.ngt_raymarch_quad_bytes(ctypes.byref(r)) == n
    assert lib.ngt_raymarch_quad(ctypes.byref(r), ctypes.c_void_p(0x1010), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_raymarch_quad(ctypes.byref(r), None, None) == L.NGT_ERR_INVALID_ARGUMENT
    r.quad = ctypes.c_void_p(0x1000)
    assert lib.ngt_raymarch_fwd_batch(ctypes.byref(r), 1, 0, ctypes.c_void_p(0x1000), 1 << 20,
                                      None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"own quad" in lib.ngt_last_error_message()
    r.quad = None
    for field, value in (("input_shape", L.I64x5(1, 6, 5, 4, 2)), ("interpolation", 0), ("dtype", L.F64)):
        old = getattr(r, field)
        setattr(r, field, value)
        assert lib.ngt_raymarch_quad_bytes(ctypes.byref(r)) == 0
        assert lib.ngt_raymarch_quad(ctypes.byref(r), ctypes.c_void_p(0x1000), None) == L.NGT_ERR_UNSUPPORTED
        r.quad = ctypes.c_void_p(0x1000)  # a forward given one where it does not apply
        assert lib.ngt_raymarch_fwd(ctypes.byref(r), None) == L.NGT_ERR_INVALID_ARGUMENT
        assert b"prepared quad" in lib.ngt_last_error_message()
        r.quad = None
        setattr(r, field, old)


def test_fused_l2_forward_validation(lib):
    from ngt_gb300 import _lib as L
    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 4, 4, 4, 1)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ctypes.c_void_p(0x1000))
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    r.emission_channels = 2
    p = ctypes.c_void_p(0x2000)
    assert lib.ngt_raymarch_fwd_l2(ctypes.byref(r), p, 3, p, p, None) == L.NGT_ERR_INVALID_ARGUMENT  # > 2 channels
    assert lib.ngt_raymarch_fwd_l2(ctypes.byref(r), p, 0, p, p, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_raymarch_fwd_l2(ctypes.byref(r), None, 1, p, p, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_raymarch_fwd_l2(None, p, 1, p, p, None) == L.NGT_ERR_INVALID_ARGUMENT


def test_nvtx_ranges_wrap_calls(monkeypatch, lib):
    """With NVTX on, every library call sits inside one pushed / popped range,
    also when the call fails."""
    import torch
    from ngt_gb300 import _lib as L
    events = []
    monkeypatch.setattr(L, "NVTX", True)
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda n: events.append(("push", n)))
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda: events.append(("pop",)))
    with pytest.raises(L.NGTError):
        L.call("ngt_raymarch_fwd", None, None)
    with pytest.raises(L.NGTError):
        L.call("ngt_advect_maccormack_fwd", None, None)
    assert events == [("push", "ngt_raymarch_fwd"), ("pop",), ("push", "ngt_advect_maccormack_fwd"), ("pop",)]


def test_accumulate_validation(lib):
    from ngt_gb300 import _lib as L
    p = ctypes.c_void_p(0x1000)
    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 4, 4, 4, 1)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, p)
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    g = L.RaymarchGradArgs()
    g.fwd = r
    g.output = g.output_grad = g.input_grad = p
    g.grad_mode, g.accumulate = L.GRAD["reference"], 1
    assert lib.ngt_raymarch_bwd(ctypes.byref(g), None) == L.NGT_ERR_UNSUPPORTED
    g.grad_mode = L.GRAD["exact"]
    assert lib.ngt_raymarch_bwd_batch(ctypes.byref(g), 1, 0, p, 1 << 20, None) == L.NGT_ERR_UNSUPPORTED
    a = L.AdvectArgs()
    a.dtype = L.F32
    a.grid_dhw = L.I64x3(4, 4, 4)
    a.channels = 1
    for f in ("data", "vel_x", "vel_y", "vel_z", "output", "fwd_field"):
        setattr(a, f, p)
    a.order, a.clamp, a.boundary = 2, 1, 1
    ag = L.AdvectGradArgs()
    ag.fwd = a
    ag.output_grad = ag.data_grad = p
    ag.accumulate, ag.deterministic = 1, 1
    assert lib.ngt_advect_maccormack_bwd(ctypes.byref(ag), None) == L.NGT_ERR_UNSUPPORTED
    ag.deterministic = 0
    ag.vel_x_grad = ag.vel_y_grad = ag.vel_z_grad = p
    assert lib.ngt_advect_maccormack_bwd_batch(ctypes.byref(ag), 1, p, 1 << 20, None) == L.NGT_ERR_UNSUPPORTED


def test_struct_layouts_match_the_header(lib):
    """The ctypes mirrors of the argument structs have the library's sizes (a
    field added on one side only would shift every field after it)."""
    from ngt_gb300 import _lib as L
    mirrors = {"ngt_sample_lut_args": L.SampleLutArgs, "ngt_sample_lut_grad_args": L.SampleLutGradArgs,
               "ngt_sample_transform_args": L.SampleTransformArgs,
               "ngt_sample_transform_grad_args": L.SampleTransformGradArgs, "ngt_lod_args": L.LodArgs,
               "ngt_raymarch_args": L.RaymarchArgs, "ngt_raymarch_grad_args": L.RaymarchGradArgs,
               "ngt_reduce_blend_args": L.ReduceBlendArgs, "ngt_reduce_blend_grad_args": L.ReduceBlendGradArgs,
               "ngt_advect_args": L.AdvectArgs, "ngt_advect_grad_args": L.AdvectGradArgs,
               "ngt_advect_velocity_args": L.AdvectVelocityArgs,
               "ngt_advect_velocity_grad_args": L.AdvectVelocityGradArgs}
    text = open(os.path.join(ROOT, "include", "ngt_ops.h")).read()
    assert set(re.findall(r"} (ngt_\w+_args);", text)) == set(mirrors)
    for name, cls in mirrors.items():
        assert lib.ngt_struct_size(name.encode()) == ctypes.sizeof(cls), name
    assert lib.ngt_struct_size(b"ngt_no_such_args") == 0


def test_misaligned_buffers_rejected(lib):
    """A device buffer that does not start on a multiple of its element size (a
    workspace, camera block or prepared quad layout: of 16 / 256 bytes) is
    rejected with a status code naming it, before any device work."""
    from ngt_gb300 import _lib as L
    a = L.AdvectArgs()
    a.dtype, a.grid_dhw, a.channels = L.F32, L.I64x3(4, 4, 4), 1
    for f in ("data", "vel_x", "vel_y", "vel_z", "output", "fwd_field"):
        setattr(a, f, ctypes.c_void_p(0x1000))
    a.order, a.clamp, a.boundary = 2, 1, 1
    for f, addr in (("data", 0x1002), ("lookup", 0x1001), ("extrema", 0x1006)):
        old = getattr(a, f)
        setattr(a, f, ctypes.c_void_p(addr))
        assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
        assert f.encode() in lib.ngt_last_error_message() and b"aligned" in lib.ngt_last_error_message()
        setattr(a, f, old)
    a.dtype = L.BF16  # 16-bit storage: two-byte data, float scratch
    a.data = ctypes.c_void_p(0x1002)
    a.fwd_field = ctypes.c_void_p(0x1002)
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"fwd_field" in lib.ngt_last_error_message()
    a.dtype, a.data, a.fwd_field = L.F32, ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000)
    g = L.AdvectGradArgs()
    g.fwd = a
    g.output_grad = g.data_grad = ctypes.c_void_p(0x1000)
    g.workspace, g.workspace_bytes = ctypes.c_void_p(0x1008), 1 << 20
    assert lib.ngt_advect_maccormack_bwd(ctypes.byref(g), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"workspace" in lib.ngt_last_error_message()

    v = L.AdvectVelocityArgs()
    v.dtype, v.grid_dhw, v.order, v.clamp, v.boundary = L.F32, L.I64x3(4, 4, 4), 1, 0, 1
    for f in ("vel_x", "vel_y", "vel_z", "out_x", "out_y", "out_z"):
        setattr(v, f, ctypes.c_void_p(0x1000))
    v.lookup[1] = 0x1003
    assert lib.ngt_advect_velocity_fwd(ctypes.byref(v), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"lookup[1]" in lib.ngt_last_error_message()

    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 6, 5, 4, 1)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ctypes.c_void_p(0x1000))
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    for f, addr in (("input", 0x1001), ("matrix_v", 0x1002), ("cameras", 0x1004), ("quad", 0x1010),
                    ("workspace", 0x1008)):
        old = getattr(r, f)
        setattr(r, f, ctypes.c_void_p(addr))
        assert lib.ngt_raymarch_fwd(ctypes.byref(r), None) == L.NGT_ERR_INVALID_ARGUMENT
        assert f.encode() in lib.ngt_last_error_message()
        setattr(r, f, old)
    assert lib.ngt_raymarch_fwd_l2(ctypes.byref(r), ctypes.c_void_p(0x1000), 1, ctypes.c_void_p(0x1002),
                                   ctypes.c_void_p(0x1000), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"image_grad" in lib.ngt_last_error_message()
    rg = L.RaymarchGradArgs()
    rg.fwd = r
    rg.output, rg.output_grad, rg.input_grad = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1001)
    assert lib.ngt_raymarch_bwd(ctypes.byref(rg), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"input_grad" in lib.ngt_last_error_message()

    s = L.SampleLutArgs()
    s.dtype = L.F32
    s.input_shape, s.lookup_shape = L.I64x5(1, 4, 4, 4, 1), L.I64x5(1, 2, 2, 2, 4)
    s.input, s.lookup, s.output = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1002), ctypes.c_void_p(0x1000)
    s.interpolation, s.boundary, s.separate_camera_batch, s.relative_coords = 1, 0, 1, 1
    assert lib.ngt_sample_lut_fwd(ctypes.byref(s), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"lookup" in lib.ngt_last_error_message()
    assert lib.ngt_image_l2_loss(L.F32, 4, 2, 1, ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1001),
                                 ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"target" in lib.ngt_last_error_message()


def test_background_validation(lib):
    """The background composite and the fused loss with a background reject bad
    sizes, channel counts and pointers before any device work."""
    from ngt_gb300 import _lib as L
    ok = ctypes.c_void_p(0x1000)
    assert lib.ngt_background_composite(L.F32, 1, 16, 3, ok, ok, ok, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_background_composite(L.F32, 0, 16, 2, ok, ok, ok, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_background_composite(L.F32, 1, 16, 2, ok, None, ok, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_background_composite(L.BF16, 1, 16, 2, ok, ok, ok, None) == L.NGT_ERR_UNSUPPORTED
    assert lib.ngt_background_composite_bwd(L.F32, 1, 16, 2, ok, ok, ok, None, None, None) == \
        L.NGT_ERR_INVALID_ARGUMENT
    r = L.RaymarchArgs()
    r.dtype = L.F32
    r.input_shape = L.I64x5(1, 4, 4, 4, 1)
    r.output_dhw = L.I64x3(4, 4, 4)
    for f in ("input", "output", "matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(r, f, ok)
    r.num_cameras = 1
    r.interpolation, r.boundary, r.blending_mode, r.separate_camera_batch = 1, 0, 0, 1
    r.emission_channels = 2
    fn = lib.ngt_raymarch_fwd_l2_background
    assert fn(ctypes.byref(r), None, ok, 1, ok, ok, None) == L.NGT_ERR_INVALID_ARGUMENT  # no background
    assert fn(ctypes.byref(r), ok, ok, 2, ok, ok, None) == L.NGT_ERR_INVALID_ARGUMENT  # loss on the depth channel
    r.blending_mode = 4
    assert fn(ctypes.byref(r), ok, ok, 1, ok, ok, None) == L.NGT_ERR_UNSUPPORTED  # not Beer-Lambert
    r.blending_mode, r.emission_channels = 0, 0
    assert fn(ctypes.byref(r), ok, ok, 1, ok, ok, None) == L.NGT_ERR_INVALID_ARGUMENT  # one blend channel


def test_face_storage_validation(lib):
    """FP16 faces go with BF16 density only; other differing face types are refused."""
    from ngt_gb300 import _lib as L
    a = L.AdvectArgs()
    a.grid_dhw = L.I64x3(4, 4, 4)
    a.channels = 1
    for f in ("data", "vel_x", "vel_y", "vel_z", "output", "fwd_field"):
        setattr(a, f, ctypes.c_void_p(0x1000))
    a.order, a.clamp, a.boundary = 2, 1, 1
    a.dtype, a.velocity_dtype = L.F32, L.F16
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_UNSUPPORTED
    a.dtype, a.velocity_dtype = L.BF16, L.F64
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_UNSUPPORTED
    a.dtype, a.velocity_dtype = L.BF16, L.F16
    a.vel_x = ctypes.c_void_p(0x1001)  # misaligned for 2-byte faces
    assert lib.ngt_advect_maccormack_fwd(ctypes.byref(a), None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"vel_x" in lib.ngt_last_error_message()


def test_wait_poll_limit_setting(lib):
    """The bricked kernels' first-wait poll limit: the setter returns the
    previous value and a negative value restores the default (host only)."""
    default = lib.ngt_set_wait_polls(7)
    assert default == 1 << 22
    assert lib.ngt_set_wait_polls(0) == 7
    assert lib.ngt_set_wait_polls(-1) == 0
    assert lib.ngt_set_wait_polls(default) == default
    from ngt_gb300 import _lib as L
    assert lib.ngt_wait_timeouts(None, 0) == L.NGT_ERR_INVALID_ARGUMENT


def test_fused_render_loss_validation(lib):
    """ngt_raymarch_fwd_l2_bwd rejects null buffers, loss channels out of range and
    a background without an optical-depth channel before any launch."""
    from ngt_gb300 import _lib as L
    g = L.RaymarchGradArgs()
    a = g.fwd
    a.dtype = L.F32
    a.input_shape = L.I64x5(1, 4, 4, 4, 1)
    a.output_dhw = L.I64x3(4, 4, 4)
    a.input = ctypes.c_void_p(0x1000)
    for f in ("matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(a, f, ctypes.c_void_p(0x2000))
    a.num_cameras = 1
    a.interpolation, a.boundary, a.blending_mode = 1, 0, 0
    a.emission_channels = 2
    a.emission_scale[0], a.emission_scale[1] = 1.0, 1.0
    g.output, g.output_grad, g.input_grad = ctypes.c_void_p(0x3000), ctypes.c_void_p(0x4000), ctypes.c_void_p(0x5000)
    tgt, loss = ctypes.c_void_p(0x6000), ctypes.c_void_p(0x7000)
    assert lib.ngt_raymarch_fwd_l2_bwd(None, None, tgt, 1, loss, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), None, None, 1, loss, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), None, tgt, 3, loss, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"loss_channels" in lib.ngt_last_error_message()
    # with a background the light channels are 1..Cb-1
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), ctypes.c_void_p(0x8000), tgt, 2, loss,
                                       None) == L.NGT_ERR_INVALID_ARGUMENT
    a.emission_channels = 0
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), ctypes.c_void_p(0x8000), tgt, 1, loss,
                                       None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"optical depth" in lib.ngt_last_error_message()
    a.emission_channels = 2
    g.output_grad = ctypes.c_void_p(0x4002)  # misaligned image gradient
    assert lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), None, tgt, 1, loss, None) != L.NGT_OK


def test_fused_render_fallback_checks_backward_first(lib):
    """A call that runs as two passes (reference gradient here) rejects a short
    backward workspace before its forward launches anything."""
    from ngt_gb300 import _lib as L
    g = L.RaymarchGradArgs()
    a = g.fwd
    a.dtype = L.F32
    a.input_shape = L.I64x5(1, 4, 4, 4, 1)
    a.output_dhw = L.I64x3(4, 4, 4)
    a.input = ctypes.c_void_p(0x1000)
    for f in ("matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(a, f, ctypes.c_void_p(0x2000))
    a.num_cameras = 1
    a.interpolation, a.boundary, a.blending_mode = 1, 0, 0
    a.emission_channels = 2
    a.emission_scale[0], a.emission_scale[1] = 1.0, 1.0
    g.output, g.output_grad, g.input_grad = ctypes.c_void_p(0x3000), ctypes.c_void_p(0x4000), ctypes.c_void_p(0x5000)
    g.grad_mode = L.GRAD["reference"]
    g.workspace, g.workspace_bytes = ctypes.c_void_p(0x6000), 16
    rc = lib.ngt_raymarch_fwd_l2_bwd(ctypes.byref(g), None, ctypes.c_void_p(0x7000), 1, ctypes.c_void_p(0x8000), None)
    assert rc == L.NGT_ERR_WORKSPACE


def test_sample_cache_policy():
    """The render keeps its sample cache for float storage, and for 16-bit storage
    while the quad gradient fits in the L2 (host logic; without a GPU the L2 is
    taken as 128 MiB)."""
    import torch
    from ngt_gb300.ops import sample_cache_pays
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else torch.device("cpu")
    assert sample_cache_pays((256, 448, 256), 1, torch.float32, dev)
    assert sample_cache_pays((128, 128, 128), 1, torch.bfloat16, dev)    # 34 MB quad gradient
    assert not sample_cache_pays((256, 448, 256), 1, torch.float16, dev)  # 476 MB
    assert not sample_cache_pays((128, 128, 128), 8, torch.bfloat16, dev)  # 8 grids: 272 MB


def test_fused_batch_validation(lib):
    """ngt_raymarch_fwd_l2_bwd_batch rejects loss channels out of range, scenes
    without emission channels and null targets before any launch."""
    from ngt_gb300 import _lib as L
    g = (L.RaymarchGradArgs * 1)()
    a = g[0].fwd
    a.dtype = L.F32
    a.input_shape = L.I64x5(1, 4, 4, 4, 1)
    a.output_dhw = L.I64x3(4, 4, 4)
    a.input = ctypes.c_void_p(0x1000)
    for f in ("matrix_m", "matrix_v", "matrix_p", "frustum"):
        setattr(a, f, ctypes.c_void_p(0x2000))
    a.num_cameras = 1
    a.interpolation, a.boundary, a.blending_mode = 1, 0, 0
    a.emission_channels = 2
    a.emission_scale[0], a.emission_scale[1] = 1.0, 1.0
    g[0].output, g[0].output_grad, g[0].input_grad = (ctypes.c_void_p(0x3000), ctypes.c_void_p(0x4000),
                                                      ctypes.c_void_p(0x5000))
    targets = (ctypes.c_void_p * 1)(0x6000)
    loss = ctypes.c_void_p(0x7000)
    ws = ctypes.c_void_p(0x100000)
    assert lib.ngt_raymarch_fwd_l2_bwd_batch(g, targets, 1, 3, loss, 0, ws, 1 << 30, None) == L.NGT_ERR_INVALID_ARGUMENT
    assert b"loss_channels" in lib.ngt_last_error_message()
    nulls = (ctypes.c_void_p * 1)(None)
    assert lib.ngt_raymarch_fwd_l2_bwd_batch(g, nulls, 1, 1, loss, 0, ws, 1 << 30, None) == L.NGT_ERR_INVALID_ARGUMENT
    a.emission_channels = 0
    assert lib.ngt_raymarch_fwd_l2_bwd_batch(g, targets, 1, 1, loss, 0, ws, 1 << 30, None) == L.NGT_ERR_UNSUPPORTED


@pytest.mark.parametrize("C", [1, 2, 4])
def test_deterministic_advection_workspace_covers_fixed_point(lib, C):
    """The deterministic advection backward's workspace holds the fwd-field and
    lookup gradients, the back-trace gradient and the 64-bit fixed-point sums
    (one per cell and channel) after 16-byte alignment; the velocity one the
    same over its largest face lattice."""
    from ngt_gb300 import _lib as L
    D, H, W = 5, 7, 9
    n = D * H * W
    g = L.AdvectGradArgs()
    g.fwd.dtype, g.fwd.grid_dhw, g.fwd.channels = L.F32, L.I64x3(D, H, W), C
    g.grad_mode = L.GRAD["exact"]
    exact = int(lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g)))
    g.deterministic = 1
    det = int(lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g)))
    assert exact == n * (C + 3) * 4
    assert det >= exact + n * C * 4 + 15 + n * C * 8 + 4
    v = L.AdvectVelocityGradArgs()
    v.fwd.dtype, v.fwd.grid_dhw = L.F32, L.I64x3(D, H, W)
    v.grad_mode = L.GRAD["exact"]
    vexact = int(lib.ngt_advect_velocity_bwd_workspace_bytes(ctypes.byref(v)))
    v.deterministic = 1
    vdet = int(lib.ngt_advect_velocity_bwd_workspace_bytes(ctypes.byref(v)))
    nmax = max((W + 1) * H * D, W * (H + 1) * D, W * H * (D + 1))
    assert vdet >= vexact + nmax * 4 + 15 + nmax * 8 + 4
