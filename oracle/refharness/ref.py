"""ctypes binding of the host-compiled reference harness (``oracle/_ref/libref_*.so``).

Test infrastructure: used to generate the golden vectors in ``tests/golden`` and
to cross-check the NumPy oracle where the reference tree is available.
Enumerations follow the reference headers: blend modes
(blending_settings.hpp:6-12), v2 filter / boundary (sampling_settings_v2.hpp:10-11),
v1 filter / boundary / coordinate modes (sampling_settings.hpp:18-20, 60-69).
"""
import ctypes
import os

import numpy as np

_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_ref")

BLEND = {"BEER_LAMBERT": 0, "ALPHA": 2, "ALPHA_ADDITIVE": 3, "ADDITIVE": 4}
FILTER_V2 = {"NEAREST": 0, "LINEAR": 1, "MIN": 2, "MAX": 3}
FILTER_V1 = {"NEAREST": 0, "LINEAR": 1, "MIN": 2, "MAX": 3, "QUADRATIC": 4}
BOUNDARY = {"BORDER": 0, "CLAMP": 1, "WRAP": 2}
COORD = {"TRANSFORM_LINDEPTH": 0, "TRANSFORM_LINDEPTH_REVERSE": 1, "TRANSFORM": 3, "TRANSFORM_REVERSE": 4}

_libs = {}


def lib(unit):
    if unit not in _libs:
        path = os.path.join(_DIR, "libref_%s.so" % unit)
        if not os.path.exists(path):
            raise FileNotFoundError(path + " (build it with oracle/refharness/build.py)")
        _libs[unit] = ctypes.CDLL(path)
    return _libs[unit]


def available():
    return all(os.path.exists(os.path.join(_DIR, "libref_%s.so" % u)) for u in ("v1", "v2", "rb"))


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _shape(s):
    a = np.asarray(s, dtype=np.int64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))


def _check(rc, what):
    if rc != 0:
        raise ValueError("reference harness rejected %s" % what)


def raymarch_fwd(x, M, V, P, F, output_shape, interpolation="LINEAR", boundary="BORDER",
                 blending_mode="BEER_LAMBERT", separate_camera_batch=True):
    x, xp = _f(x)
    M, Mp = _f(M)
    V, Vp = _f(V)
    P, Pp = _f(P)
    F, Fp = _f(F)
    N, C = x.shape[0], x.shape[-1]
    nc = V.reshape(-1, 16).shape[0]
    nv = nc if separate_camera_batch else 1
    D, H, W = output_shape
    out = np.zeros((N, nv, H, W, C), np.float32)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape([N, nv, D, H, W, C])
    _, op = _f(out)
    rc = lib("v2").ref_raymarch_fwd(xp, insp, Mp, Vp, Pp, Fp, ctypes.c_int(nc), FILTER_V2[interpolation],
                                    BOUNDARY[boundary], BLEND[blending_mode], int(separate_camera_batch), op, outsp)
    _check(rc, "raymarch_fwd")
    return out


def raymarch_grad(x, y, gy, M, V, P, F, output_shape, boundary="BORDER", blending_mode="BEER_LAMBERT",
                  separate_camera_batch=True):
    x, xp = _f(x)
    y, yp = _f(y)
    gy, gyp = _f(gy)
    M, Mp = _f(M)
    V, Vp = _f(V)
    P, Pp = _f(P)
    F, Fp = _f(F)
    N, C = x.shape[0], x.shape[-1]
    nc = V.reshape(-1, 16).shape[0]
    nv = nc if separate_camera_batch else 1
    D, H, W = output_shape
    gx = np.zeros_like(x)
    _, gxp = _f(gx)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape([N, nv, D, H, W, C])
    rc = lib("v2").ref_raymarch_grad(xp, yp, gyp, insp, Mp, Vp, Pp, Fp, ctypes.c_int(nc), BOUNDARY[boundary],
                                     BLEND[blending_mode], int(separate_camera_batch), gxp, outsp)
    _check(rc, "raymarch_grad")
    return gx


def sample_v2(grid, pos, interpolation="LINEAR", boundary="BORDER"):
    g = np.asarray(grid, np.float32)
    if g.ndim == 4:
        g = g[None]
    g, gp = _f(g)
    pos, pp = _f(np.asarray(pos).reshape(-1, 3))
    s, sp = _shape(g.shape)
    out = np.zeros((pos.shape[0], g.shape[-1]), np.float32)
    _, op = _f(out)
    rc = lib("v2").ref_sample_v2(gp, sp, pp, ctypes.c_longlong(pos.shape[0]), FILTER_V2[interpolation],
                                 BOUNDARY[boundary], op)
    _check(rc, "sample_v2")
    return out


def blend(acc, cell, mode):
    acc, ap = _f(acc)
    cell, cp = _f(cell)
    C = acc.shape[-1]
    n = acc.size // C
    out = np.zeros_like(acc)
    _, op = _f(out)
    _check(lib("v2").ref_blend(C, BLEND[mode], ctypes.c_longlong(n), ap, cp, op), "blend")
    return out


def blend_grad(grads_out, cell, cell_out, mode):
    g, gp = _f(grads_out)
    c, cp = _f(cell)
    o, opp = _f(cell_out)
    C = g.shape[-1]
    n = g.size // C
    d, dp = _f(np.zeros_like(g))
    ng, ngp = _f(np.zeros_like(g))
    no, nop = _f(np.zeros_like(g))
    _check(lib("v2").ref_blend_grad(C, BLEND[mode], ctypes.c_longlong(n), gp, cp, opp, dp, ngp, nop), "blend_grad")
    return d, ng, no


# ------------------------------------------------------------------ resample (v1)

def lut_fwd(x, lut, interpolation="LINEAR", boundary="BORDER", cell_center_offset=0.0,
            separate_camera_batch=True, relative_coords=True, normalized_coords=False):
    x, xp = _f(x)
    lut, lp = _f(lut)
    N, C = x.shape[0], x.shape[-1]
    nc = lut.shape[0]
    nv = nc if separate_camera_batch else 1
    out = np.zeros((N, nv) + lut.shape[1:4] + (C,), np.float32)
    _, op = _f(out)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(out.shape)
    rc = lib("v1").ref_lut_fwd(xp, insp, ctypes.c_int(nc), lp, FILTER_V1[interpolation], BOUNDARY[boundary],
                               ctypes.c_float(cell_center_offset), int(separate_camera_batch), int(relative_coords),
                               int(normalized_coords), op, outsp)
    _check(rc, "lut_fwd")
    return out


def lut_grad(x, gy, lut, interpolation="LINEAR", boundary="BORDER", cell_center_offset=0.0,
             separate_camera_batch=True, relative_coords=True, normalized_coords=False):
    x, xp = _f(x)
    gy, gyp = _f(gy)
    lut, lp = _f(lut)
    nc = lut.shape[0]
    gx = np.zeros_like(x)
    _, gxp = _f(gx)
    gl = np.zeros_like(lut)
    _, glp = _f(gl)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(gy.shape)
    rc = lib("v1").ref_lut_grad(xp, insp, ctypes.c_int(nc), lp, FILTER_V1[interpolation], BOUNDARY[boundary],
                                ctypes.c_float(cell_center_offset), int(separate_camera_batch), int(relative_coords),
                                int(normalized_coords), gyp, outsp, gxp, glp)
    _check(rc, "lut_grad")
    return gx, gl


def transform_fwd(x, M, V, P, F, output_shape, interpolation="LINEAR", boundary="BORDER",
                  coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5, separate_camera_batch=True):
    x, xp = _f(x)
    M, Mp = _f(M)
    V, Vp = _f(V)
    P, Pp = _f(P)
    F, Fp = _f(F)
    N, C = x.shape[0], x.shape[-1]
    nc = V.reshape(-1, 16).shape[0]
    nv = nc if separate_camera_batch else 1
    out = np.zeros((N, nv) + tuple(output_shape) + (C,), np.float32)
    _, op = _f(out)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(out.shape)
    rc = lib("v1").ref_transform_fwd(xp, insp, Mp, Vp, Pp, Fp, ctypes.c_int(nc), COORD[coordinate_mode],
                                     FILTER_V1[interpolation], BOUNDARY[boundary], ctypes.c_float(cell_center_offset),
                                     int(separate_camera_batch), op, outsp)
    _check(rc, "transform_fwd")
    return out


def transform_grad(x, gy, M, V, P, F, interpolation="LINEAR", boundary="BORDER",
                   coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5, separate_camera_batch=True):
    x, xp = _f(x)
    gy, gyp = _f(gy)
    M, Mp = _f(M)
    V, Vp = _f(V)
    P, Pp = _f(P)
    F, Fp = _f(F)
    nc = V.reshape(-1, 16).shape[0]
    gx = np.zeros_like(x)
    _, gxp = _f(gx)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(gy.shape)
    rc = lib("v1").ref_transform_grad(xp, insp, Mp, Vp, Pp, Fp, ctypes.c_int(nc), COORD[coordinate_mode],
                                      FILTER_V1[interpolation], BOUNDARY[boundary], ctypes.c_float(cell_center_offset),
                                      int(separate_camera_batch), gyp, outsp, gxp)
    _check(rc, "transform_grad")
    return gx


def lod(input_shape_dhw, MV, P, F, output_shape_dhw, coordinate_mode="TRANSFORM_LINDEPTH", relative=False):
    MV, Mp = _f(MV)
    P, Pp = _f(P)
    F, Fp = _f(F)
    nv = MV.reshape(-1, 16).shape[0]
    out = np.zeros((nv,) + tuple(output_shape_dhw) + (4,), np.float32)
    _, op = _f(out)
    ins, insp = _shape([nv] + list(input_shape_dhw) + [1])
    outs, outsp = _shape(out.shape)
    rc = lib("v1").ref_lod(insp, Mp, Pp, Fp, COORD[coordinate_mode], int(relative), op, outsp)
    _check(rc, "lod")
    return out


def sample_v1(grid, pos, interpolation="LINEAR", boundary="BORDER", cell_center_offset=0.0):
    g = np.asarray(grid, np.float32)
    if g.ndim == 4:
        g = g[None]
    g, gp = _f(g)
    pos, pp = _f(np.asarray(pos).reshape(-1, 3))
    s, sp = _shape(g.shape)
    out = np.zeros((pos.shape[0], g.shape[-1]), np.float32)
    _, op = _f(out)
    rc = lib("v1").ref_sample_v1(gp, sp, pp, ctypes.c_longlong(pos.shape[0]), FILTER_V1[interpolation],
                                 BOUNDARY[boundary], ctypes.c_float(cell_center_offset), op)
    _check(rc, "sample_v1")
    return out


def data_grad_v1(grid, pos, boundary="BORDER"):
    g = np.asarray(grid, np.float32)
    if g.ndim == 4:
        g = g[None]
    g, gp = _f(g)
    pos, pp = _f(np.asarray(pos).reshape(-1, 3))
    s, sp = _shape(g.shape)
    out = np.zeros((pos.shape[0], 3, g.shape[-1]), np.float32)
    _, op = _f(out)
    rc = lib("v1").ref_data_grad_v1(gp, sp, pp, ctypes.c_longlong(pos.shape[0]), BOUNDARY[boundary], op)
    _check(rc, "data_grad_v1")
    return out


# ------------------------------------------------------------------ reduce blend

def reduce_blend(x, mode, keep_dims=False):
    x, xp = _f(x)
    N, D, H, W, C = x.shape
    out = np.zeros((N, D if keep_dims else 1, H, W, C), np.float32)
    _, op = _f(out)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(out.shape)
    _check(lib("rb").ref_reduce_blend(xp, insp, BLEND[mode], int(keep_dims), op, outsp), "reduce_blend")
    return out if keep_dims else out[:, 0]


def reduce_blend_grad(gy, y, x, mode, keep_dims=False):
    x, xp = _f(x)
    N, D, H, W, C = x.shape
    if not keep_dims:
        gy = np.asarray(gy)[:, None]
        y = np.asarray(y)[:, None]
    gy, gyp = _f(gy)
    y, yp = _f(y)
    gx = np.zeros_like(x)
    _, gxp = _f(gx)
    ins, insp = _shape(x.shape)
    outs, outsp = _shape(y.shape)
    _check(lib("rb").ref_reduce_blend_grad(xp, yp, gyp, insp, BLEND[mode], int(keep_dims), gxp, outsp),
           "reduce_blend_grad")
    return gx
