"""Volume files, ScalarFlow captures and the camera calibration on the host:
archives in the reference's layouts read and written both ways, the ScalarFlow
conversions against hand-built arrays, calibrated cameras against their
geometric meaning, and the aligned-rescale matrices on the oracle."""
import numpy as np
import pytest

import __graft_entry__

__graft_entry__.load_package()

from ngt_gb300 import formats, scene  # noqa: E402
from oracle import ops as oops  # noqa: E402

FLIP = np.asarray([1.0, 1.0, -1.0])


def synthetic_calibration(n=5, seed=0, missing_fov=2):
    """A calibration with the ScalarFlow keys: ``n`` cameras on an arc about the
    focus, each looking at it, with right-handed (right, up, -look) bases in the
    z-flipped frame the renderer uses."""
    rng = np.random.default_rng(seed)
    focus = np.asarray([0.35, 0.55, -0.3])
    c = {"focus": focus.tolist(), "focus_error": 0.0, "fov_horizontal_average": 24.0, "fov_vertical_average": 40.5,
         "marker_width": 0.5, "scale_y": 1.77, "volume_offset": [0.1, -0.05, -0.6], "volume_size": [0.5, 0.885, 0.5],
         "volume_width": 0.5}
    fp = FLIP * focus
    for i in range(n):
        yaw = np.radians(-60 + 30 * i)
        pos = fp + rng.uniform(0.8, 1.0) * np.asarray([np.sin(yaw), 0.25, np.cos(yaw)])
        look = (fp - pos) / np.linalg.norm(fp - pos)
        z = -look
        up = np.asarray([0.0, 1.0, 0.0]) - z * z[1]
        up /= np.linalg.norm(up)
        right = np.cross(up, z)
        c[str(i)] = {"position": (FLIP * pos).tolist(), "forward": (FLIP * look).tolist(), "up": (FLIP * up).tolist(),
                     "right": (FLIP * right).tolist(), "rotation": [0.0, 0.0, 0.0], "position_error": 0.0,
                     "fov_horizontal": None if i == missing_fov else float(23 + rng.uniform()),
                     "fov_vertical": float(40 + rng.uniform())}
    return c


# --------------------------------------------------------------------------- archives

def test_density_archive_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    d = rng.uniform(0, 1, (1, 6, 7, 8, 1)).astype(np.float32)
    hull = (rng.uniform(0, 1, d.shape) > 0.3).astype(np.float32)
    inflow = rng.uniform(0, 1, (1, 2, 3, 4, 1)).astype(np.float32)
    mask = (rng.uniform(0, 1, inflow.shape) > 0.5).astype(np.float32)
    p = tmp_path / "density.npz"
    formats.save_density(p, d, hull=hull, inflow=inflow, inflow_mask=mask, inflow_offset=[1, 2, 3])
    with np.load(p) as f:
        assert sorted(f.keys()) == ["arr_0", "hull", "inflow", "inflow_mask", "inflow_offset"]
        assert np.array_equal(f["arr_0"], d)
    g = formats.load_density(p)
    assert np.array_equal(g.d, d) and np.array_equal(g.hull, hull)
    assert np.array_equal(g.inflow, inflow) and np.array_equal(g.inflow_mask, mask)
    assert g.inflow_offset == [1, 2, 3] and g.shape == [6, 7, 8]
    # inflow offset is (z, y, x), like the grid shape
    want = d * hull
    want[:, 1:3, 2:5, 3:7] += inflow * mask
    assert np.array_equal(g.with_inflow(), np.maximum(want, 0))


def test_density_archive_written_like_the_reference(tmp_path):
    """A file laid out as ``DensityGrid.save`` writes it (grid unnamed, optional
    entries by name) and one with the grid only."""
    d = np.arange(2 * 3 * 4, dtype=np.float32).reshape(1, 2, 3, 4, 1)
    p = tmp_path / "a.npz"
    np.savez_compressed(p, d, inflow=d[:, :1], inflow_offset=np.asarray([0, 0, 0]))
    g = formats.load_density(p)
    assert np.array_equal(g.d, d) and g.hull is None and g.inflow_mask is None
    assert np.array_equal(g.inflow, d[:, :1]) and g.inflow_offset == [0, 0, 0]
    # arrays given by the caller win over the stored ones
    own = np.zeros((1, 1, 3, 4, 1), np.float32)
    assert np.array_equal(formats.load_density(p, inflow=own).inflow, own)
    p2 = tmp_path / "b.npz"
    np.savez_compressed(p2, d)
    g2 = formats.load_density(p2)
    assert g2.inflow is None and np.array_equal(g2.with_inflow(), d)


def test_density_archive_missing_file_gives_none(tmp_path):
    assert formats.load_density(tmp_path / "missing.npz") is None


def test_velocity_archive_round_trip_and_legacy(tmp_path):
    rng = np.random.default_rng(1)
    D, H, W = 4, 5, 6
    xs, ys, zs = formats.velocity_component_shapes([D, H, W])
    x, y, z = (rng.standard_normal([1] + s + [1]).astype(np.float32) for s in (xs, ys, zs))
    p = tmp_path / "vel.npz"
    formats.save_velocity(p, x, y, z)
    with np.load(p) as f:
        assert sorted(f.keys()) == ["centered_shape", "vel_x", "vel_y", "vel_z"]
        assert f["centered_shape"].tolist() == [D, H, W]
    v = formats.load_velocity(p)
    assert v.centered_shape == [D, H, W]
    assert all(np.array_equal(a, b) for a, b in zip((v.x, v.y, v.z), (x, y, z)))
    # legacy archive without centered_shape, stored in float64
    p2 = tmp_path / "legacy.npz"
    np.savez_compressed(p2, vel_x=x.astype(np.float64), vel_y=y, vel_z=z)
    v2 = formats.load_velocity(p2)
    assert v2.centered_shape == [D, H, W] and v2.x.dtype == np.float32
    # components that disagree with the shape are refused
    p3 = tmp_path / "bad.npz"
    np.savez_compressed(p3, centered_shape=np.asarray([D, H, W]), vel_x=x, vel_y=x, vel_z=z)
    assert formats.load_velocity(p3) is None


def test_load_numpy_forms(tmp_path):
    a = np.arange(6.0).reshape(2, 3)
    np.save(tmp_path / "a.npy", a)
    assert np.array_equal(formats.load_numpy(tmp_path / "a.npy"), a)
    np.savez(tmp_path / "one.npz", data=a)
    assert np.array_equal(formats.load_numpy(tmp_path / "one.npz"), a)
    np.savez(tmp_path / "two.npz", data=a, other=a + 1)
    both = formats.load_numpy(tmp_path / "two.npz")
    assert sorted(both) == ["data", "other"] and np.array_equal(both["other"], a + 1)
    assert np.array_equal(formats.load_numpy(tmp_path / "two.npz", "other"), a + 1)
    with pytest.raises(KeyError):
        formats.load_numpy(tmp_path / "two.npz", "nope")


# --------------------------------------------------------------------------- ScalarFlow captures

def test_scalarflow_density_flip_and_inflow(tmp_path):
    rng = np.random.default_rng(2)
    raw = rng.uniform(0, 1, (20, 24, 10, 1)).astype(np.float32)  # D, H, W, 1 with z reversed
    np.savez_compressed(tmp_path / "sf.npz", data=raw)
    g = formats.load_scalarflow_density(tmp_path / "sf.npz")
    k = formats.SCALARFLOW_INFLOW_CELLS
    flipped = raw[::-1][None]
    assert g.d.shape == (1, 20, 24, 10, 1) and g.shape == [20, 24, 10]
    assert np.array_equal(g.inflow, flipped[:, :, :k])
    assert np.array_equal(g.inflow_mask, np.ones_like(g.inflow)) and g.inflow_offset == [0, 0, 0]
    assert np.all(g.d[:, :, :k] == 0) and np.array_equal(g.d[:, :, k:], flipped[:, :, k:])
    assert np.array_equal(g.with_inflow(), flipped)
    # the same shape asked for explicitly: no rescale, no device needed
    g2 = formats.load_scalarflow_density(tmp_path / "sf.npz", shape=[20, 24, 10])
    assert np.array_equal(g2.d, g.d)
    with pytest.raises(ValueError):
        formats.load_scalarflow_density(tmp_path / "sf.npz", shape=[10, 12, 5])


def test_scalarflow_velocity_components(tmp_path):
    rng = np.random.default_rng(3)
    raw = rng.standard_normal((5, 6, 7, 3)).astype(np.float32)
    np.savez_compressed(tmp_path / "sfv.npz", data=raw)
    v = formats.load_scalarflow_velocity(tmp_path / "sfv.npz")
    f = raw[::-1][None]
    assert v.centered_shape == [5, 6, 7]
    assert np.array_equal(v.x[..., :7, :], f[..., :, 0:1]) and np.array_equal(v.x[..., 7, :], f[..., 6, 0:1])
    assert np.array_equal(v.y[:, :, :6], f[:, :, :, :, 1:2]) and np.array_equal(v.y[:, :, 6], f[:, :, 5, :, 1:2])
    assert np.array_equal(v.z[:, 1:], -f[..., 2:3]) and np.array_equal(v.z[:, 0], -f[:, 0, ..., 2:3])


# --------------------------------------------------------------------------- calibration

def test_calibrated_cameras_look_at_the_focus():
    c = synthetic_calibration()
    res = [64, 96, 56]
    cams = formats.scalarflow_cameras(c, res)
    assert len(cams) == 5
    fp = FLIP * np.asarray(c["focus"])
    for cid, cam in zip(formats.SCALARFLOW_CAMERA_IDS, cams):
        cal = c[str(cid)]
        dist = np.linalg.norm(fp - FLIP * np.asarray(cal["position"]))
        # the focus sits on the optical axis (view -z) at its distance
        assert np.allclose(cam.view_matrix() @ np.append(fp, 1.0), [0, 0, -dist, 1], atol=1e-12)
        assert np.allclose(cam.clip, [dist - 0.5, dist + 0.5])
        fh = cal["fov_horizontal"] if cal["fov_horizontal"] is not None else c["fov_horizontal_average"]
        half_h = np.tan(np.radians(fh) / 2) * cam.near
        assert np.allclose(cam.trbl, [half_h * cal["fov_vertical"] / fh, half_h, -half_h * cal["fov_vertical"] / fh,
                                      -half_h])
        assert cam.transform.grid_size == res
        assert np.isclose(cam.depth_step, 1.0 / res[0])
    # synthetic data: the vertical fov follows the image aspect
    cams_s = formats.scalarflow_cameras(c, res, synthetic=True)
    for cam in cams_s:
        assert np.isclose(cam.trbl[1] / cam.trbl[0], res[2] / res[1])
    # the calibration passed in is left as it was
    assert c["2"]["fov_horizontal"] is None


def test_interpolated_cameras():
    c = synthetic_calibration()
    cams = formats.scalarflow_cameras(c, [32, 32, 32], ids=(0, 1, 2), interpolation_weights=(0.25, 0.5))
    assert len(cams) == 3 + 2 * 2
    a, b = c["0"], c["1"]
    for t in (0.0, 1.0):
        ci = formats.interpolate_camera_calibration(a, b, t, c)
        e = a if t == 0.0 else b
        for k in ("forward", "up", "right", "position"):
            assert np.allclose(ci[k], e[k], atol=1e-12)
    mid = formats.interpolate_camera_calibration(a, b, 0.5, c)
    assert np.isclose(np.linalg.norm(mid["forward"]), 1.0)
    ang = lambda u, v: np.arccos(np.clip(np.dot(u, v) / np.linalg.norm(u) / np.linalg.norm(v), -1, 1))
    assert np.isclose(ang(a["forward"], mid["forward"]), ang(mid["forward"], b["forward"]))
    # the interpolated camera still looks at the common focus
    fp = FLIP * np.asarray(c["focus"])
    for cam in cams:
        v = cam.view_matrix() @ np.append(fp, 1.0)
        assert np.allclose(v[:2], 0, atol=1e-9) and v[2] < 0


def test_simulation_grid_transform():
    c = synthetic_calibration()
    size = formats.scalarflow_density_size(64, c)
    assert size == [64, int(np.ceil(64 * 1.77)), 64]
    assert formats.scalarflow_density_size(64, c, y_scale=1.0) == [64, 64, 64]
    t = formats.scalarflow_sim_transform(size, c)
    m = t.get_transform_matrix()
    mw = c["marker_width"]
    # MIN-normalised and scaled by the marker width: one cell is mw / 64
    assert np.allclose(np.diag(m)[:3], mw / 64)
    world = t.grid_size_world()
    assert np.allclose(world, [mw, mw * size[1] / 64, mw])
    # x, z centred on the marker volume (z flipped), the grid's floor at y = 0.005
    centre = FLIP * (np.asarray(c["volume_offset"]) + np.asarray([mw, mw * c["scale_y"], mw]) / 2)
    assert np.allclose(m[[0, 2], 3] + world[[0, 2]] / 2, centre[[0, 2]])
    assert np.isclose(m[1, 3], 0.005)
    assert np.isclose(formats.scalarflow_sim_transform(size, c, render_targets=True).get_transform_matrix()[1, 3], 0.05)
    cap = formats.scalarflow_capture_transform(c)
    assert cap.grid_size == [100, 178, 100]
    assert np.allclose(cap.get_transform_matrix()[:3, 3], FLIP * (np.asarray(c["volume_offset"]) + [0, 0, mw]))


def test_calibration_json_round_trip(tmp_path):
    import json
    c = synthetic_calibration()
    (tmp_path / "cams.json").write_text(json.dumps(c))
    assert formats.load_calibration(tmp_path / "cams.json") == c


# --------------------------------------------------------------------------- aligned rescale matrices

def test_aligned_matrices_identity_and_linear_fields():
    """On the oracle's transform resample: BORDER alignment at the same shape is
    the identity, and every alignment carries a linear field to the positions
    its rule defines (trilinear interpolation reproduces linear fields)."""
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, (1, 6, 7, 8, 1)).astype(np.float32)
    M, V, P, F = formats.aligned_matrices((6, 7, 8), (6, 7, 8))
    y = oops.sample_grid_transform(x, M, V, P, F, (6, 7, 8), coordinate_mode="TRANSFORM")
    assert np.abs(y[:, 0] - x).max() < 1e-6
    D, H, W = 5, 6, 7
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    ramp = (0.3 * xx + 0.2 * yy + 0.1 * zz).astype(np.float32)[None, ..., None]
    out = (9, 11, 13)

    def centres(align, n_in, n_out):
        # input-cell coordinate of each output cell centre under the alignment
        i = np.arange(n_out) + 0.5
        if align == "CENTER":
            return (i - 0.5) * (n_in - 1) / (n_out - 1)
        if align == "STAGGER_INPUT":
            return i * (n_in - 1) / n_out
        if align == "STAGGER_OUTPUT":
            return i * (n_in + 1) / n_out - 1
        return i * n_in / n_out - 0.5

    for align in ("CENTER", "STAGGER_INPUT", "STAGGER_OUTPUT", "BORDER"):
        M, V, P, F = formats.aligned_matrices((D, H, W), out, align, align, align)
        y = oops.sample_grid_transform(ramp, M, V, P, F, out, coordinate_mode="TRANSFORM", boundary="CLAMP")[:, 0]
        tz, ty, tx = np.meshgrid(*(np.clip(centres(align, n, o), 0, n - 1) for n, o in zip((D, H, W), out)),
                                 indexing="ij")
        want = (0.3 * tx + 0.2 * ty + 0.1 * tz)[None, ..., None]
        assert np.abs(y - want).max() < 1e-5, align
    with pytest.raises(ValueError):
        formats.aligned_matrices((D, H, W), out, "MIDDLE")


def test_matrix_transform_basis():
    t = scene.MatrixTransform.from_fwd_up_right_pos([0, 0, 1], [0, 1, 0], [1, 0, 0], [1, 2, 3],
                                                    parent=scene.Transform(translation=[1, 0, 0]))
    assert np.allclose(t.get_transform_matrix()[:3, 3], [2, 2, 3])
    assert np.allclose(t.get_inverse_transform() @ t.get_transform_matrix(), np.eye(4))
