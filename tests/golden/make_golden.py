"""Generate the golden vectors that pin the oracle to the reference.

The reference's own device code (samplers, blends, transforms and the kernel
bodies of the LUT / transform resample, fused raymarch and reduce-blend ops) is
compiled for the host by ``oracle/refharness/build.py`` and run on seeded
inputs; inputs and outputs are stored in ``reference_vectors.npz`` next to this
script.  Requires the reference tree (development container only):

    python tests/golden/make_golden.py [--ref /path/to/reference]

Cases the reference cannot run are left out and documented:
* QUADRATIC + BORDER transform gradient: the reference writes out of bounds
  (centre taps unchecked, resample_grid.cu.cc:938-1076);
* raymarch MIN / MAX filters: the reference's extrema reader collapses its
  FLOAT_MAX start value through ``lerp`` (sampling_v2.hpp:150-160), so the
  result depends on argument evaluation order;
* frustum grids with an odd height or width: their centre row / column of rays
  is axis-parallel in exact arithmetic and the reference's fp32 slab test then
  divides rounding noise by rounding noise.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refharness import build as refbuild  # noqa: E402
from oracle.refharness import ref  # noqa: E402

OUT = os.path.join(HERE, "reference_vectors.npz")


def _scene():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_ngt_scene", os.path.join(ROOT, "neural-global-transport_gb300", "scene.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=refbuild.DEFAULT_REF)
    a = ap.parse_args()
    refbuild.build(a.ref)
    scene = _scene()
    rng = np.random.default_rng(2024)
    f32 = np.float32
    d = {}

    # ---- direct sampler probes
    g = rng.standard_normal((5, 6, 7, 2)).astype(f32)
    pos = rng.uniform(-2.0, 9.0, (400, 3)).astype(f32)
    d["s_grid"], d["s_pos"] = g, pos
    for fm in ("NEAREST", "LINEAR", "MIN", "MAX", "QUADRATIC"):
        for bm in ("BORDER", "CLAMP", "WRAP"):
            if fm == "QUADRATIC" and bm == "WRAP":
                continue
            d["s1_%s_%s" % (fm, bm)] = ref.sample_v1(g, pos, fm, bm, 0.0)
    for bm in ("BORDER", "CLAMP", "WRAP"):
        d["dg1_%s" % bm] = ref.data_grad_v1(g, pos, bm)
        for fm in ("NEAREST", "LINEAR"):
            d["s2_%s_%s" % (fm, bm)] = ref.sample_v2(g, pos, fm, bm)

    # ---- blend / blendGradients
    for C in (1, 2, 4):
        acc = rng.uniform(0, 0.8, (64, C)).astype(f32)
        cell = rng.uniform(0, 0.5, (64, C)).astype(f32)
        gout = rng.standard_normal((64, C)).astype(f32)
        d["b_acc_%d" % C], d["b_cell_%d" % C], d["b_g_%d" % C] = acc, cell, gout
        for m in ("BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"):
            d["b_%s_%d" % (m, C)] = ref.blend(acc, cell, m)
            dc, ng, no = ref.blend_grad(gout, cell, acc, m)
            d["bg_%s_%d" % (m, C)] = np.stack([dc, ng, no])

    # ---- LUT resample
    x = rng.standard_normal((2, 4, 5, 6, 2)).astype(f32)
    lut = rng.uniform(-1.5, 1.5, (2, 3, 4, 5, 4)).astype(f32)
    lut[..., 3] = 0
    d["l_x"], d["l_lut"] = x, lut
    coords = {"rel": (True, False, 0.0, lut), "abs": (False, False, 0.0, lut + np.array([1, 2, 1.5, 0], f32)),
              "nrm": (True, True, 0.5, lut * f32(0.05))}
    for sep in (True, False):
        for fm in ("NEAREST", "LINEAR", "MIN", "MAX"):
            for bm in ("BORDER", "CLAMP", "WRAP"):
                for cn, (rel, nrm, cco, l) in coords.items():
                    k = "%d_%s_%s_%s" % (sep, fm, bm, cn)
                    y = ref.lut_fwd(x, l, fm, bm, cco, sep, rel, nrm)
                    gy = rng.standard_normal(y.shape).astype(f32)
                    gx, gl = ref.lut_grad(x, gy, l, fm, bm, cco, sep, rel, nrm)
                    d["lf_" + k], d["lgy_" + k], d["lgx_" + k], d["lgl_" + k] = y, gy, gx, gl

    # ---- transform resample
    vol = scene.volume_transform([8, 10, 12])
    cams = scene.orbit_cameras([8, 6, 4], [13, -47])
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    d["t_M"], d["t_V"], d["t_P"], d["t_F"] = M, V, P, F
    xt = rng.uniform(0, 1, (1, 8, 10, 12, 2)).astype(f32)
    d["t_x"] = xt
    for cm in ("TRANSFORM_LINDEPTH", "TRANSFORM"):
        for fm in ("LINEAR", "NEAREST", "QUADRATIC"):
            for bm in ("BORDER", "CLAMP"):
                k = "%s_%s_%s" % (cm, fm, bm)
                y = ref.transform_fwd(xt, M, V, P, F, [8, 6, 4], fm, bm, cm)
                d["tf_" + k] = y
                if fm == "QUADRATIC" and bm == "BORDER":
                    continue
                gy = rng.standard_normal(y.shape).astype(f32)
                d["tgy_" + k] = gy
                d["tgx_" + k] = ref.transform_grad(xt, gy, M, V, P, F, fm, bm, cm)
    xf = rng.uniform(0, 1, (1, 8, 6, 4, 1)).astype(f32)
    d["t_xf"] = xf
    for cm in ("TRANSFORM_LINDEPTH_REVERSE", "TRANSFORM_REVERSE"):
        d["tr_" + cm] = ref.transform_fwd(xf, M, V[:1], P[:1], F[:1], [8, 10, 12], "LINEAR", "BORDER", cm)
    MV = np.stack([scene.colmajor(c.view_matrix() @ vol.get_transform_matrix()) for c in cams])
    d["lod_MV"] = MV
    for cm in ("TRANSFORM_LINDEPTH", "TRANSFORM"):
        d["lod_" + cm] = ref.lod([8, 10, 12], MV, P, F, [8, 6, 4], cm, False)

    # ---- fused raymarch
    cams = scene.orbit_cameras([8, 8, 6], [13, -47, 71])
    V, P, F = scene.camera_params(cams)
    d["r_V"], d["r_P"], d["r_F"] = V, P, F
    for C in (1, 2, 4):
        xr = (rng.uniform(0, 1, (1, 8, 10, 12, C)) * 0.3).astype(f32)
        d["r_x_%d" % C] = xr
        for bm in ("BORDER", "CLAMP", "WRAP"):
            for m in ("BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"):
                for fm in ("LINEAR", "NEAREST"):
                    d["rf_%d_%s_%s_%s" % (C, bm, m, fm)] = ref.raymarch_fwd(xr, M, V, P, F, [8, 8, 6], fm, bm, m)
                y = d["rf_%d_%s_%s_LINEAR" % (C, bm, m)]
                gy = rng.standard_normal(y.shape).astype(f32)
                d["rgy_%d_%s_%s" % (C, bm, m)] = gy
                d["rgx_%d_%s_%s" % (C, bm, m)] = ref.raymarch_grad(xr, y, gy, M, V, P, F, [8, 8, 6], bm, m)

    # ---- reduce blend
    for C in (1, 2, 4):
        xb = rng.uniform(0, 0.3, (2, 6, 4, 5, C)).astype(f32)
        d["rb_x_%d" % C] = xb
        for m in ("BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE"):
            for kd in (False, True):
                y = ref.reduce_blend(xb, m, kd)
                gy = rng.standard_normal(y.shape).astype(f32)
                k = "%d_%s_%d" % (C, m, kd)
                d["rbf_" + k], d["rbgy_" + k], d["rbgx_" + k] = y, gy, ref.reduce_blend_grad(gy, y, xb, m, kd)

    np.savez_compressed(OUT, **d)
    print("wrote", OUT, "with", len(d), "arrays,", os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
