"""ctypes binding of ``libngt_ops.so`` (declarations in ``include/ngt_ops.h``).

The library is built in-tree by ``_build.build_library``.  Loading fails loudly
when it is missing: there is no CPU or eager fallback for any operator.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libngt_ops.so")

NGT_OK, NGT_ERR_INVALID_ARGUMENT, NGT_ERR_UNSUPPORTED, NGT_ERR_CUDA, NGT_ERR_WORKSPACE = 0, 1, 2, 3, 4
F32, F64, BF16, F16 = 0, 1, 2, 3
INTERP = {"NEAREST": 0, "LINEAR": 1, "MIN": 2, "MAX": 3, "QUADRATIC": 4}
BOUNDARY = {"BORDER": 0, "CLAMP": 1, "WRAP": 2}
MIP = {"NONE": 0, "NEAREST": 1, "LINEAR": 2}
BLEND = {"BEER_LAMBERT": 0, "ALPHA": 2, "ALPHA_ADDITIVE": 3, "ADDITIVE": 4}
COORD = {"TRANSFORM_LINDEPTH": 0, "TRANSFORM_LINDEPTH_REVERSE": 1, "TRANSFORM": 3, "TRANSFORM_REVERSE": 4}
GRAD = {"exact": 0, "reference": 1}
CLAMP = {"NONE": 0, "MC_SMOOTH": 1, "NEGATIVE": 2}

c_i32, c_i64, c_f32, c_vp, c_sz = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p, ctypes.c_size_t
I64x5 = c_i64 * 5
I64x3 = c_i64 * 3


class SampleLutArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("input_shape", I64x5), ("lookup_shape", I64x5), ("input", c_vp), ("lookup", c_vp),
                ("output", c_vp), ("interpolation", c_i32), ("boundary", c_i32), ("mipmapping", c_i32),
                ("num_mipmaps", c_i32), ("mip_bias", c_f32), ("cell_center_offset", c_f32),
                ("separate_camera_batch", c_i32), ("relative_coords", c_i32), ("normalized_coords", c_i32),
                ("workspace", c_vp), ("workspace_bytes", c_sz)]


class SampleLutGradArgs(ctypes.Structure):
    _fields_ = [("fwd", SampleLutArgs), ("output_grad", c_vp), ("input_grad", c_vp), ("lookup_grad", c_vp),
                ("grad_mode", c_i32), ("deterministic", c_i32), ("workspace", c_vp), ("workspace_bytes", c_sz)]


class SampleTransformArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("input_shape", I64x5), ("output_dhw", I64x3), ("input", c_vp),
                ("matrix_m", c_vp), ("matrix_v", c_vp), ("matrix_p", c_vp), ("frustum", c_vp),
                ("num_cameras", c_i32), ("output", c_vp), ("interpolation", c_i32), ("boundary", c_i32),
                ("mipmapping", c_i32), ("num_mipmaps", c_i32), ("mip_bias", c_f32), ("cell_center_offset", c_f32),
                ("coordinate_mode", c_i32), ("separate_camera_batch", c_i32), ("workspace", c_vp),
                ("workspace_bytes", c_sz)]


class SampleTransformGradArgs(ctypes.Structure):
    _fields_ = [("fwd", SampleTransformArgs), ("output_grad", c_vp), ("input_grad", c_vp), ("grad_mode", c_i32),
                ("workspace", c_vp), ("workspace_bytes", c_sz), ("deterministic", c_i32)]


class LodArgs(ctypes.Structure):
    _fields_ = [("input_dhw", I64x3), ("output_dhw", I64x3), ("matrix_mv", c_vp), ("matrix_p", c_vp),
                ("frustum", c_vp), ("num_cameras", c_i32), ("inverse_transform", c_i32),
                ("linearize_depth", c_i32), ("relative_coords", c_i32), ("output", c_vp)]


class RaymarchArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("input_shape", I64x5), ("output_dhw", I64x3), ("input", c_vp),
                ("matrix_m", c_vp), ("matrix_v", c_vp), ("matrix_p", c_vp), ("frustum", c_vp),
                ("num_cameras", c_i32), ("output", c_vp), ("interpolation", c_i32), ("boundary", c_i32),
                ("blending_mode", c_i32), ("keep_dims", c_i32), ("separate_camera_batch", c_i32),
                ("emission_channels", c_i32), ("emission_scale", c_f32 * 4), ("workspace", c_vp),
                ("workspace_bytes", c_sz), ("cameras", c_vp), ("quad", c_vp), ("rays", c_vp),
                ("sample_cache", c_i32)]


class RaymarchGradArgs(ctypes.Structure):
    _fields_ = [("fwd", RaymarchArgs), ("output", c_vp), ("output_grad", c_vp), ("input_grad", c_vp),
                ("grad_mode", c_i32), ("workspace", c_vp), ("workspace_bytes", c_sz), ("accumulate", c_i32),
                ("deterministic", c_i32)]


class ReduceBlendArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("input_shape", I64x5), ("input", c_vp), ("output", c_vp),
                ("blending_mode", c_i32), ("keep_dims", c_i32)]


class ReduceBlendGradArgs(ctypes.Structure):
    _fields_ = [("fwd", ReduceBlendArgs), ("output", c_vp), ("output_grad", c_vp), ("input_grad", c_vp),
                ("grad_mode", c_i32)]


class AdvectArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("grid_dhw", I64x3), ("channels", c_i32), ("data", c_vp), ("vel_x", c_vp),
                ("vel_y", c_vp), ("vel_z", c_vp), ("dt", c_f32), ("order", c_i32), ("clamp", c_i32),
                ("boundary", c_i32), ("output", c_vp), ("fwd_field", c_vp), ("mask", c_vp), ("extrema", c_vp),
                ("lookup", c_vp), ("velocity_dtype", c_i32)]


class AdvectGradArgs(ctypes.Structure):
    _fields_ = [("fwd", AdvectArgs), ("output_grad", c_vp), ("data_grad", c_vp), ("vel_x_grad", c_vp),
                ("vel_y_grad", c_vp), ("vel_z_grad", c_vp), ("grad_mode", c_i32), ("deterministic", c_i32),
                ("workspace", c_vp), ("workspace_bytes", c_sz), ("accumulate", c_i32)]


class AdvectVelocityArgs(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("grid_dhw", I64x3), ("vel_x", c_vp), ("vel_y", c_vp), ("vel_z", c_vp),
                ("dt", c_f32), ("order", c_i32), ("clamp", c_i32), ("boundary", c_i32), ("out_x", c_vp),
                ("out_y", c_vp), ("out_z", c_vp), ("fwd_x", c_vp), ("fwd_y", c_vp), ("fwd_z", c_vp),
                ("lookup", c_vp * 3), ("mask", c_vp * 3), ("extrema", c_vp * 3)]


class AdvectVelocityGradArgs(ctypes.Structure):
    _fields_ = [("fwd", AdvectVelocityArgs), ("grad_x", c_vp), ("grad_y", c_vp), ("grad_z", c_vp),
                ("vel_x_grad", c_vp), ("vel_y_grad", c_vp), ("vel_z_grad", c_vp), ("grad_mode", c_i32),
                ("workspace", c_vp), ("workspace_bytes", c_sz), ("deterministic", c_i32)]


# name -> (argument types, result type)
SIGNATURES = {
    "ngt_sample_lut_fwd": ([ctypes.POINTER(SampleLutArgs), c_vp], c_i32),
    "ngt_sample_lut_fwd_workspace_bytes": ([ctypes.POINTER(SampleLutArgs)], c_sz),
    "ngt_sample_lut_bwd": ([ctypes.POINTER(SampleLutGradArgs), c_vp], c_i32),
    "ngt_sample_lut_bwd_workspace_bytes": ([ctypes.POINTER(SampleLutGradArgs)], c_sz),
    "ngt_sample_transform_fwd": ([ctypes.POINTER(SampleTransformArgs), c_vp], c_i32),
    "ngt_sample_transform_fwd_workspace_bytes": ([ctypes.POINTER(SampleTransformArgs)], c_sz),
    "ngt_sample_transform_bwd": ([ctypes.POINTER(SampleTransformGradArgs), c_vp], c_i32),
    "ngt_sample_transform_bwd_workspace_bytes": ([ctypes.POINTER(SampleTransformGradArgs)], c_sz),
    "ngt_mip_build": ([c_i32, ctypes.POINTER(c_i64), c_vp, c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_mip_bytes": ([c_i32, ctypes.POINTER(c_i64), c_i32], c_sz),
    "ngt_lod_transform": ([ctypes.POINTER(LodArgs), c_vp], c_i32),
    "ngt_raymarch_fwd_workspace_bytes": ([ctypes.POINTER(RaymarchArgs)], c_sz),
    "ngt_raymarch_cameras_bytes": ([ctypes.POINTER(RaymarchArgs)], c_sz),
    "ngt_raymarch_cameras": ([ctypes.POINTER(RaymarchArgs), c_vp, c_vp], c_i32),
    "ngt_raymarch_rays_bytes": ([ctypes.POINTER(RaymarchArgs)], c_sz),
    "ngt_raymarch_rays": ([ctypes.POINTER(RaymarchArgs), c_vp, c_vp], c_i32),
    "ngt_raymarch_quad_bytes": ([ctypes.POINTER(RaymarchArgs)], c_sz),
    "ngt_raymarch_quad": ([ctypes.POINTER(RaymarchArgs), c_vp, c_vp], c_i32),
    "ngt_raymarch_fwd_l2": ([ctypes.POINTER(RaymarchArgs), c_vp, c_i32, c_vp, c_vp, c_vp], c_i32),
    "ngt_raymarch_fwd_l2_background": ([ctypes.POINTER(RaymarchArgs), c_vp, c_vp, c_i32, c_vp, c_vp, c_vp], c_i32),
    "ngt_background_composite": ([c_i32, c_i64, c_i64, c_i32, c_vp, c_vp, c_vp, c_vp], c_i32),
    "ngt_background_composite_bwd": ([c_i32, c_i64, c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_i32),
    "ngt_raymarch_fwd": ([ctypes.POINTER(RaymarchArgs), c_vp], c_i32),
    "ngt_raymarch_bwd": ([ctypes.POINTER(RaymarchGradArgs), c_vp], c_i32),
    "ngt_raymarch_fwd_l2_bwd": ([ctypes.POINTER(RaymarchGradArgs), c_vp, c_vp, c_i32, c_vp, c_vp], c_i32),
    "ngt_raymarch_bwd_workspace_bytes": ([ctypes.POINTER(RaymarchGradArgs)], c_sz),
    "ngt_raymarch_bwd_static": ([ctypes.POINTER(RaymarchGradArgs), c_vp], c_i32),
    "ngt_raymarch_batch_workspace_bytes": ([ctypes.POINTER(RaymarchArgs), c_i32], c_sz),
    "ngt_raymarch_fwd_batch": ([ctypes.POINTER(RaymarchArgs), c_i32, c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_raymarch_bwd_batch": ([ctypes.POINTER(RaymarchGradArgs), c_i32, c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_raymarch_bwd_batch_after_fwd": ([ctypes.POINTER(RaymarchGradArgs), c_i32, c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_raymarch_fwd_l2_bwd_batch": ([ctypes.POINTER(RaymarchGradArgs), ctypes.POINTER(c_vp), c_i32, c_i32, c_vp,
                                       c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_advect_maccormack_fwd_batch": ([ctypes.POINTER(AdvectArgs), c_i32, c_vp], c_i32),
    "ngt_advect_maccormack_bwd_batch_workspace_bytes": ([ctypes.POINTER(AdvectGradArgs), c_i32], c_sz),
    "ngt_advect_maccormack_bwd_batch": ([ctypes.POINTER(AdvectGradArgs), c_i32, c_vp, c_sz, c_vp], c_i32),
    "ngt_reduce_blend_fwd": ([ctypes.POINTER(ReduceBlendArgs), c_vp], c_i32),
    "ngt_reduce_blend_bwd": ([ctypes.POINTER(ReduceBlendGradArgs), c_vp], c_i32),
    "ngt_advect_maccormack_fwd": ([ctypes.POINTER(AdvectArgs), c_vp], c_i32),
    "ngt_advect_maccormack_bwd": ([ctypes.POINTER(AdvectGradArgs), c_vp], c_i32),
    "ngt_advect_maccormack_bwd_workspace_bytes": ([ctypes.POINTER(AdvectGradArgs)], c_sz),
    "ngt_advect_velocity_fwd": ([ctypes.POINTER(AdvectVelocityArgs), c_vp], c_i32),
    "ngt_advect_velocity_bwd": ([ctypes.POINTER(AdvectVelocityGradArgs), c_vp], c_i32),
    "ngt_advect_velocity_bwd_workspace_bytes": ([ctypes.POINTER(AdvectVelocityGradArgs)], c_sz),
    "ngt_image_l2_loss": ([c_i32, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp], c_i32),
    "ngt_last_error_message": ([], ctypes.c_char_p),
    "ngt_version": ([], c_i32),
    "ngt_struct_size": ([ctypes.c_char_p], c_sz),
    "ngt_wait_timeouts": ([ctypes.POINTER(ctypes.c_uint64), c_i32], c_i32),
    "ngt_set_wait_polls": ([c_i32], c_i32),
}

_lib = None


class NGTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ngt error %d: %s" % (code, msg))
        self.code = code


def load():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libngt_ops.so is not built (run __graft_entry__.build()); "
                               "the grid operators have no fallback implementation")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (argtypes, restype) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = restype
        _lib = lib
    return _lib


# NVTX ranges around every library call, for timelines taken with a profiler
# (NGT_NVTX=1 in the environment; off by default, one flag test per call then).
NVTX = os.environ.get("NGT_NVTX", "0") not in ("", "0")


def call(name, *args):
    lib = load()
    if NVTX:
        import torch
        torch.cuda.nvtx.range_push(name)
        try:
            rc = getattr(lib, name)(*args)
        finally:
            torch.cuda.nvtx.range_pop()
    else:
        rc = getattr(lib, name)(*args)
    if rc != NGT_OK:
        raise NGTError(rc, lib.ngt_last_error_message().decode(errors="replace"))
    return rc
