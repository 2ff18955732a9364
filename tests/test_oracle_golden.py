"""The oracle against golden vectors produced by the reference's own code.

``tests/golden/reference_vectors.npz`` was written by
``tests/golden/make_golden.py``, which runs the reference's samplers, blends,
transforms and kernel bodies compiled for the host.  Every oracle path that the
CUDA kernels are later checked against is pinned here, in float32.
"""
import os

import numpy as np
import pytest

from oracle import core, ops

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(a).max(), 1e-30)


@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR", "MIN", "MAX", "QUADRATIC"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_sampler_v1(fm, bm):
    if fm == "QUADRATIC" and bm == "WRAP":
        pytest.skip("the resample op restricts QUADRATIC to BORDER / CLAMP")
    out = core.read(G["s_grid"], G["s_pos"], fm, bm)
    assert rel(G["s1_%s_%s" % (fm, bm)], out) < 1e-6


@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_data_gradient(bm):
    assert rel(G["dg1_%s" % bm], core.data_gradient(G["s_grid"], G["s_pos"], bm)) < 1e-6


@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_sampler_v2(fm, bm):
    out = ops._v2_sample(G["s_grid"], G["s_pos"], fm, bm)
    assert rel(G["s2_%s_%s" % (fm, bm)], out) < 1e-6


@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("m", ["BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"])
def test_blend(C, m):
    acc, cell, g = G["b_acc_%d" % C], G["b_cell_%d" % C], G["b_g_%d" % C]
    assert rel(G["b_%s_%d" % (m, C)], core.blend(acc, cell, m)) < 1e-6
    dc, ng, no = core.blend_gradients_reference(g, cell, acc, m)
    assert rel(G["bg_%s_%d" % (m, C)], np.stack([dc, ng, no])) < 1e-6


LUT_COORDS = {"rel": (True, False, 0.0, np.zeros(4, np.float32), 1.0),
              "abs": (False, False, 0.0, np.array([1, 2, 1.5, 0], np.float32), 1.0),
              "nrm": (True, True, 0.5, np.zeros(4, np.float32), 0.05)}


@pytest.mark.parametrize("sep", [True, False])
@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR", "MIN", "MAX"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("cn", ["rel", "abs", "nrm"])
def test_lut(sep, fm, bm, cn):
    relc, nrm, cco, off, scale = LUT_COORDS[cn]
    x = G["l_x"]
    lut = G["l_lut"] * np.float32(scale) + off if cn != "abs" else G["l_lut"] + off
    k = "%d_%s_%s_%s" % (sep, fm, bm, cn)
    kw = dict(interpolation=fm, boundary=bm, cell_center_offset=cco, separate_camera_batch=sep,
              relative_coords=relc, normalized_coords=nrm)
    assert rel(G["lf_" + k], ops.sample_grid_lut(x, lut, **kw)) < 1e-6
    gx, gl = ops.sample_grid_lut_grad(x, G["lgy_" + k], lut, grad_mode="reference", **kw)
    assert rel(G["lgx_" + k], gx) < 1e-5
    assert rel(G["lgl_" + k], gl) < 1e-5 if np.abs(G["lgl_" + k]).max() > 0 else np.abs(gl).max() == 0


@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH", "TRANSFORM"])
@pytest.mark.parametrize("fm", ["LINEAR", "NEAREST", "QUADRATIC"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
def test_transform(cm, fm, bm):
    k = "%s_%s_%s" % (cm, fm, bm)
    args = (G["t_M"], G["t_V"], G["t_P"], G["t_F"])
    y = ops.sample_grid_transform(G["t_x"], *args, [8, 6, 4], fm, bm, coordinate_mode=cm)
    # positions are computed in float64 here and in fp32 by the reference
    assert rel(G["tf_" + k], y) < 2e-5
    if fm == "QUADRATIC" and bm == "BORDER":
        return
    gx = ops.sample_grid_transform_grad(G["t_x"], G["tgy_" + k], *args, fm, bm, coordinate_mode=cm,
                                        grad_mode="reference")
    assert rel(G["tgx_" + k], gx) < 2e-5


@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH_REVERSE", "TRANSFORM_REVERSE"])
def test_transform_reverse(cm):
    y = ops.sample_grid_transform(G["t_xf"], G["t_M"], G["t_V"][:1], G["t_P"][:1], G["t_F"][:1], [8, 10, 12],
                                  "LINEAR", "BORDER", coordinate_mode=cm)
    assert rel(G["tr_" + cm], y) < 2e-5


@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH", "TRANSFORM"])
def test_lod_transform(cm):
    y = ops.lod_transform([8, 10, 12], G["lod_MV"], G["t_P"], G["t_F"], [8, 6, 4],
                          linearize_depth=(cm == "TRANSFORM_LINDEPTH"))
    assert rel(G["lod_" + cm], y) < 1e-5


@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("m", ["BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"])
def test_raymarch(C, bm, m):
    x = G["r_x_%d" % C]
    args = (G["t_M"], G["r_V"], G["r_P"], G["r_F"], [8, 8, 6])
    for fm in ("LINEAR", "NEAREST"):
        y = ops.raymarch_grid_transform(x, *args, fm, bm, m)
        ref_y = G["rf_%d_%s_%s_%s" % (C, bm, m, fm)]
        if fm == "LINEAR":
            assert rel(ref_y, y) < 1e-5
        else:
            # nearest-cell choice flips where fp32 and fp64 positions straddle a cell edge
            close = np.isclose(ref_y, y, rtol=1e-5, atol=1e-6).all(-1)
            assert close.mean() > 0.97
    gx = ops.raymarch_grid_transform_grad(x, G["rf_%d_%s_%s_LINEAR" % (C, bm, m)], G["rgy_%d_%s_%s" % (C, bm, m)],
                                          *args, "LINEAR", bm, m, grad_mode="reference")
    # per-voxel division by summed sample weights amplifies fp32 position noise
    assert rel(G["rgx_%d_%s_%s" % (C, bm, m)], gx) < 5e-4


@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("m", ["BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"])
@pytest.mark.parametrize("kd", [False, True])
def test_reduce_blend(C, m, kd):
    x = G["rb_x_%d" % C]
    k = "%d_%s_%d" % (C, m, kd)
    assert rel(G["rbf_" + k], ops.reduce_grid_blend(x, m, kd)) < 1e-6
    gx = ops.reduce_grid_blend_grad(G["rbgy_" + k], G["rbf_" + k], x, m, kd, grad_mode="reference")
    assert rel(G["rbgx_" + k], gx) < 1e-5
