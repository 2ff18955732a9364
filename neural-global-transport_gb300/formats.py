"""On-disk volume formats and the ScalarFlow camera calibration.

What a user of the reference reads and writes around the operators, in the
reference's own layouts so that files move between the two unchanged:

* density files: ``np.savez_compressed`` archives holding the NDHWC float32 grid
  as the unnamed first array (``arr_0``) and, when present, ``hull``, ``inflow``,
  ``inflow_mask`` and ``inflow_offset`` (``DensityGrid.save`` /
  ``DensityGrid.from_file``, data_structures.py:465-485, 704-727);
* velocity files: archives with ``centered_shape`` (D, H, W) and the three MAC
  components ``vel_x`` (N, D, H, W+1, 1), ``vel_y`` (N, D, H+1, W, 1) and ``vel_z``
  (N, D+1, H, W, 1); older files without ``centered_shape`` take it from
  ``vel_x`` (``VelocityGrid.save`` / ``from_file``, data_structures.py:909-928,
  1197-1198);
* ScalarFlow captures: density DHW1 and combined-staggered velocity DHW3 with the
  z axis reversed and the upper faces missing (``from_scalarFlow_file``,
  data_structures.py:487-510, 930-962);
* the calibration json of the five ScalarFlow cameras (keys ``"0"``..``"4"`` with
  position / forward / up / right / fov per camera, plus ``focus``,
  ``fov_*_average``, ``marker_width``, ``scale_y``, ``volume_offset``) turned
  into cameras and the simulation-grid transform (reconstruct_sequence.py:47-121,
  759-777);
* the aligned grid rescale used when a loaded grid's shape differs from the
  requested one (``Renderer.resample_grid3D_aligned``, renderer.py:843-917, and
  ``VelocityGrid.scaled``, data_structures.py:975-997), run on this package's
  transform resample.

File I/O and the calibration arithmetic are host work (numpy); only the rescale
runs on the GPU.
"""
import copy
import json
import logging
import math

import numpy as np

from . import scene

LOG = logging.getLogger("ngt_gb300.formats")

#: lower cells of a ScalarFlow density split off as the inflow region
#: (data_structures.py:501-505)
SCALARFLOW_INFLOW_CELLS = 15

#: camera order of the reconstruction setup (reconstruct_sequence.py:70)
SCALARFLOW_CAMERA_IDS = (2, 1, 0, 4, 3)


# --------------------------------------------------------------------------- numpy archives

def load_numpy(path, name=None):
    """An array from ``.npy``, or from ``.npz``: the entry ``name``; the only entry
    when there is one; else a dict of all entries (util.py:461-490)."""
    data = np.load(path)
    if isinstance(data, np.ndarray):
        return data
    try:
        keys = list(data.keys())
        if name is None:
            return data[keys[0]] if len(keys) < 2 else {k: data[k] for k in keys}
        if name not in keys:
            raise KeyError("Key '{}' not in loaded dict. Available keys: {}".format(name, keys))
        return data[name]
    finally:
        data.close()


def _numpy(a):
    if a is None:
        return None
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a)


class DensityData:
    """A density grid and the optional arrays stored beside it."""

    def __init__(self, d, hull=None, inflow=None, inflow_mask=None, inflow_offset=None):
        self.d = d
        self.hull = hull
        self.inflow = inflow
        self.inflow_mask = inflow_mask
        self.inflow_offset = inflow_offset

    @property
    def shape(self):
        """(D, H, W) of the grid."""
        return list(self.d.shape[-4:-1])

    def with_hull(self):
        """The grid times its hull mask when it has one (data_structures.py:436-447)."""
        return self.d if self.hull is None else self.d * self.hull

    def with_inflow(self):
        """``max(d + inflow, 0)``, the grid hull-masked and the inflow masked and
        padded to the grid from its offset, given in (z, y, x) like the shape
        (``DensityGrid.inflow`` / ``with_inflow``, data_structures.py:419-462)."""
        d = self.with_hull()
        if self.inflow is None:
            return d
        inflow = self.inflow if self.inflow_mask is None else self.inflow * self.inflow_mask
        offset = [int(v) for v in (self.inflow_offset if self.inflow_offset is not None else (0, 0, 0))]
        pad = [(0, 0)] + [(o, s - o - i) for o, s, i in zip(offset, self.shape, inflow.shape[-4:-1])] + [(0, 0)]
        return np.maximum(d + np.pad(inflow, pad), 0)


def save_density(path, d, hull=None, inflow=None, inflow_mask=None, inflow_offset=None):
    """Write a density archive (data_structures.py:704-727): the grid unnamed, then
    ``hull``; ``inflow`` with ``inflow_mask`` and ``inflow_offset`` (default [0, 0, 0])."""
    extra = {}
    if hull is not None:
        extra["hull"] = _numpy(hull)
    if inflow is not None:
        extra["inflow"] = _numpy(inflow)
        if inflow_mask is not None:
            extra["inflow_mask"] = _numpy(inflow_mask)
        extra["inflow_offset"] = np.asarray([0, 0, 0] if inflow_offset is None else inflow_offset)
    np.savez_compressed(path, _numpy(d), **extra)


def load_density(path, hull=None, inflow=None, inflow_offset=None, inflow_mask=None):
    """Read a density archive (data_structures.py:465-485).  Arrays passed in win
    over the stored ones, as in the reference; ``inflow_mask`` and
    ``inflow_offset`` are read only with a stored inflow.  Returns None (with a
    warning) when the file cannot be read."""
    try:
        with np.load(path) as f:
            d = f["arr_0"]
            if hull is None and "hull" in f:
                hull = f["hull"]
            if inflow is None and "inflow" in f:
                inflow = f["inflow"]
                if inflow_mask is None and "inflow_mask" in f:
                    inflow_mask = f["inflow_mask"]
                if inflow_offset is None and "inflow_offset" in f:
                    inflow_offset = f["inflow_offset"].tolist()
    except Exception:
        LOG.warning("Failed to load density from '%s':", path, exc_info=True)
        return None
    return DensityData(d, hull=hull, inflow=inflow, inflow_mask=inflow_mask, inflow_offset=inflow_offset)


def velocity_component_shapes(centered_shape):
    """(D, H, W+1), (D, H+1, W), (D+1, H, W) of a MAC grid with ``centered_shape``
    (data_structures.py:764-773)."""
    D, H, W = (int(s) for s in centered_shape)
    return [D, H, W + 1], [D, H + 1, W], [D + 1, H, W]


class VelocityData:
    """A MAC velocity grid: ``centered_shape`` (D, H, W) and its three face
    components, NDHW1 float32."""

    def __init__(self, centered_shape, x, y, z):
        self.centered_shape = [int(s) for s in centered_shape]
        self.x, self.y, self.z = x, y, z
        for comp, shp, name in zip((x, y, z), velocity_component_shapes(self.centered_shape), "xyz"):
            got = list(comp.shape)
            if len(got) != 5 or got[-1] != 1 or got[-4:-1] != shp:
                raise ValueError("Invalid or incompatible shape of velocity {} component: is {}, required: NDHW1 "
                                 "with DHW={}".format(name, got, shp))


def save_velocity(path, x, y, z, centered_shape=None):
    """Write a velocity archive (data_structures.py:1197-1198)."""
    x, y, z = _numpy(x), _numpy(y), _numpy(z)
    if centered_shape is None:
        centered_shape = [x.shape[-4], x.shape[-3], x.shape[-2] - 1]
    np.savez_compressed(path, centered_shape=np.asarray(centered_shape), vel_x=x, vel_y=y, vel_z=z)


def load_velocity(path):
    """Read a velocity archive (data_structures.py:909-928); without
    ``centered_shape`` the shape is ``vel_x``'s with one x face less.  Returns None
    (with a warning) when the file cannot be read or its shapes disagree."""
    try:
        with np.load(path) as f:
            if "centered_shape" not in f:
                shape = list(f["vel_x"].shape)
                shape[-2] -= 1
                shape = shape[1:-1]
            else:
                shape = f["centered_shape"].tolist()
            vel = VelocityData(shape, f["vel_x"].astype(np.float32), f["vel_y"].astype(np.float32),
                               f["vel_z"].astype(np.float32))
    except Exception:
        LOG.warning("Failed to load velocity from '%s':", path, exc_info=True)
        return None
    return vel


# --------------------------------------------------------------------------- aligned rescale (GPU)

def _align_scale(align, in_size, out_size):
    """Object-space scale of the input grid so that its cells line up with the
    output's (renderer.py:867-878)."""
    a = align.upper()
    if a == "BORDER":
        return 2.0 / in_size
    if a == "CENTER":
        return 2.0 / out_size * (out_size - 1.0) / (in_size - 1.0)
    if a == "STAGGER_INPUT":
        return 2.0 / (in_size - 1.0)
    if a == "STAGGER_OUTPUT":
        return 2.0 / (in_size + 1.0)
    raise ValueError("unknown alignment {}".format(align))


def aligned_matrices(in_shape, target_shape, align_x="BORDER", align_y="BORDER", align_z="BORDER"):
    """M, V, P, F (column-major float32) that resample a grid of ``in_shape``
    (D, H, W) onto ``target_shape`` with the chosen alignment per axis.

    The input grid is centred and scaled into the output's [-1, 1] cube; the
    output's view is the inverse of its plain grid transform; projection
    identity and frustum [-1, 1, -1, 1, 1, -1] (renderer.py:222-235, 879-905)."""
    D, H, W = (int(s) for s in in_shape)
    tD, tH, tW = (int(s) for s in target_shape)
    scale = [_align_scale(align_x, W, tW), _align_scale(align_y, H, tH), _align_scale(align_z, D, tD)]
    src = scene.GridTransform([D, H, W], scale=scale, center=True)
    dst = scene.GridTransform([tD, tH, tW])
    M = scene.model_params([src])
    V = scene.colmajor(dst.get_inverse_transform())[None]
    P = scene.colmajor(np.eye(4))[None]
    F = np.asarray([[-1, 1, -1, 1, 1, -1]], np.float32)
    return M, V, P, F


def resample_aligned(data, target_shape, align_x="BORDER", align_y="BORDER", align_z="BORDER",
                     interpolation="LINEAR", boundary="BORDER", mipmapping="LINEAR", num_mipmaps=2, mip_bias=0.0):
    """Resample an NDHWC CUDA tensor (C in 1, 2, 4) onto ``target_shape`` (D, H, W)
    with outer borders (BORDER), outer cell centres (CENTER) or staggered cells
    aligned per axis (``resample_grid3D_aligned``, renderer.py:843-917; sampler
    defaults of the reference's ``Renderer``, renderer.py:65-68).  Differentiable
    through the transform resample's registered gradient."""
    from . import ops
    if data.dim() != 5:
        raise ValueError("input shape must be NDHWC, is : {}".format(list(data.shape)))
    if len(target_shape) != 3:
        raise ValueError("target_shape must be (D, H, W)")
    M, V, P, F = aligned_matrices(data.shape[1:4], target_shape, align_x, align_y, align_z)
    M = np.repeat(M, data.shape[0], 0)
    out = ops.sample_grid_transform(data, M, V, P, F, tuple(int(s) for s in target_shape),
                                    interpolation=interpolation, boundary=boundary, mipmapping=mipmapping,
                                    num_mipmaps=num_mipmaps, mip_bias=mip_bias, coordinate_mode="TRANSFORM")
    return out[:, 0]


def scale_velocity(x, y, z, centered_shape, new_centered_shape, scale_magnitude=True, **sampler):
    """The MAC components resampled onto ``new_centered_shape``, each with its
    staggered axis centre-aligned, and (``scale_magnitude``) multiplied by the
    size ratio of its axis (``VelocityGrid.scaled``, data_structures.py:975-997)."""
    new_centered_shape = [int(s) for s in new_centered_shape]
    if new_centered_shape == [int(s) for s in centered_shape]:
        return x.clone(), y.clone(), z.clone()
    xs, ys, zs = velocity_component_shapes(new_centered_shape)
    x2 = resample_aligned(x, xs, align_x="CENTER", **sampler)
    y2 = resample_aligned(y, ys, align_y="CENTER", **sampler)
    z2 = resample_aligned(z, zs, align_z="CENTER", **sampler)
    if scale_magnitude:
        sz, sy, sx = (o / i for i, o in zip(centered_shape, new_centered_shape))
        x2, y2, z2 = x2 * sx, y2 * sy, z2 * sz
    return x2, y2, z2


# --------------------------------------------------------------------------- ScalarFlow captures

def _ndhwc(a):
    a = np.asarray(a)
    if a.ndim == 4:
        a = a[None]
    if a.ndim != 5:
        raise ValueError("expected a DHWC or NDHWC grid, got shape {}".format(list(a.shape)))
    return a


def load_scalarflow_density(path, shape=None, device=None, **sampler):
    """A ScalarFlow density capture (DHW1, z reversed) as NDHWC float32
    (data_structures.py:487-510).

    With ``shape`` (D, H, W) different from the file's the grid is rescaled with
    outer borders aligned (on ``device``, a CUDA device) and carries no inflow.
    Otherwise its lower ``SCALARFLOW_INFLOW_CELLS`` rows (y) become the inflow
    (mask 1, offset 0) and are zeroed in the density."""
    d = np.ascontiguousarray(load_numpy(path).astype(np.float32)[::-1])
    d = d.reshape([1] + list(d.shape))
    d_shape = list(d.shape[1:4])
    if shape is not None and [int(s) for s in shape] != d_shape:
        if device is None:
            raise ValueError("No device provided to scale density.")
        import torch
        t = torch.as_tensor(d, device=device)
        return DensityData(resample_aligned(t, shape, **sampler).cpu().numpy())
    k = SCALARFLOW_INFLOW_CELLS
    inflow = d[:, :, :k].copy()
    d = np.concatenate([np.zeros_like(inflow), d[:, :, k:]], axis=2)
    return DensityData(d, inflow=inflow, inflow_mask=np.ones_like(inflow), inflow_offset=[0, 0, 0])


def scalarflow_velocity_components(v):
    """Split a ScalarFlow velocity (NDHW3 after the z flip, lower faces of each
    axis) into MAC components: the missing upper x and y faces repeat the last
    ones, z changes sign and its missing face (first, the axis being reversed)
    repeats the first one (data_structures.py:938-946)."""
    v = _ndhwc(v)
    vx, vy, vz = v[..., 0:1], v[..., 1:2], -v[..., 2:3]
    x = np.concatenate([vx, vx[:, :, :, -1:]], axis=3)
    y = np.concatenate([vy, vy[:, :, -1:]], axis=2)
    z = np.concatenate([vz[:, :1], vz], axis=1)
    return x, y, z


def load_scalarflow_velocity(path, shape=None, device=None, **sampler):
    """A ScalarFlow velocity capture as a MAC grid (data_structures.py:930-962).
    With ``shape`` different from the file's the components are rescaled and
    their magnitudes scaled (``scale_velocity``) on ``device``."""
    v = load_numpy(path).astype(np.float32)[::-1]
    x, y, z = scalarflow_velocity_components(np.ascontiguousarray(v))
    v_shape = list(_ndhwc(v).shape[1:4])
    if shape is not None and [int(s) for s in shape] != v_shape:
        if device is None:
            raise ValueError("No device provided to scale velocity.")
        import torch
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=device)
        x, y, z = (c.cpu().numpy() for c in scale_velocity(T(x), T(y), T(z), v_shape, shape, **sampler))
        v_shape = [int(s) for s in shape]
    return VelocityData(v_shape, x, y, z)


# --------------------------------------------------------------------------- calibration

def load_calibration(path):
    """The calibration json as a dict."""
    with open(path) as f:
        return json.load(f)


def _flip_z(v):
    return np.asarray(v, dtype=np.float64) * np.asarray([1.0, 1.0, -1.0])


def camera_from_calibration(position, forward, up, right, resolution, fov_horizontal, fov_vertical, focus,
                            focus_depth_clip=1.0, **_):
    """One calibrated camera (reconstruct_sequence.py:52-68): the calibration's
    right-handed z is flipped, the view looks along -forward, near / far sit
    ``focus_depth_clip / 2`` either side of the focus distance, the horizontal
    fov is the camera's and the aspect is ``fov_horizontal / fov_vertical``."""
    pos, fwd, up, right, cam_focus = (_flip_z(position), -_flip_z(forward), _flip_z(up), _flip_z(right),
                                      _flip_z(focus))
    aspect = fov_horizontal / fov_vertical
    half = focus_depth_clip * 0.5
    dist = float(np.linalg.norm(cam_focus - pos))
    t = scene.MatrixTransform.from_fwd_up_right_pos(fwd, up, right, pos)
    t.grid_size = [int(s) for s in resolution]
    return scene.Camera(t, near_far=[dist - half, dist + half], fov=fov_horizontal, aspect=aspect)


def slerp_vector(v1, v2, t, normalized=True):
    """Spherical linear interpolation (Shoemake 1985) of two 3-vectors.  With
    ``normalized`` the inputs are unit directions and so is the result; otherwise
    the direction is slerped and the length interpolated linearly.  The
    reference imports a helper of this name from a module its tree does not
    ship (reconstruct_sequence.py:103); this is the textbook form."""
    v1 = np.asarray(v1, dtype=np.float64)
    v2 = np.asarray(v2, dtype=np.float64)
    l1, l2 = np.linalg.norm(v1), np.linalg.norm(v2)
    a, b = v1 / l1, v2 / l2
    omega = math.acos(float(np.clip(np.dot(a, b), -1.0, 1.0)))
    if omega < 1e-7:
        d = a * (1 - t) + b * t
    else:
        s = math.sin(omega)
        d = (math.sin((1 - t) * omega) / s) * a + (math.sin(t * omega) / s) * b
    d = d / np.linalg.norm(d)
    return d if normalized else d * ((1 - t) * l1 + t * l2)


def interpolate_camera_calibration(cal1, cal2, t, calib_base):
    """A camera between two calibrated ones (reconstruct_sequence.py:105-121):
    orientation vectors slerped, the position slerped about the focus, the fovs
    interpolated linearly."""
    focus = np.asarray(calib_base["focus"], dtype=np.float64)
    out = {
        "forward": slerp_vector(cal1["forward"], cal2["forward"], t, normalized=True),
        "up": slerp_vector(cal1["up"], cal2["up"], t, normalized=True),
        "right": slerp_vector(cal1["right"], cal2["right"], t, normalized=True),
        "position": slerp_vector(np.subtract(cal1["position"], focus), np.subtract(cal2["position"], focus), t,
                                 normalized=False) + focus,
        "fov_horizontal": cal1["fov_horizontal"] + t * (cal2["fov_horizontal"] - cal1["fov_horizontal"]),
        "fov_vertical": cal1["fov_vertical"] + t * (cal2["fov_vertical"] - cal1["fov_vertical"]),
    }
    return out


def train_resolution(base_resolution, res_down):
    """(D, H, W) of the training cameras: the base image sides divided by
    ``res_down`` and truncated, depth kept (reconstruct_sequence.py:71-74)."""
    r = [int(s) for s in base_resolution]
    scale = 1.0 / res_down
    return [r[0], int(r[1] * scale), int(r[2] * scale)]


def scalarflow_cameras(calibration, resolution, ids=SCALARFLOW_CAMERA_IDS, focus_depth_clip=1.0, synthetic=False,
                       interpolation_weights=()):
    """The calibrated cameras, frustum grid ``resolution`` (D, H, W)
    (reconstruct_sequence.py:70-101).  A missing horizontal fov takes the
    average; the vertical fov is the horizontal one over the image aspect for
    synthetic data, else the camera's (or the average when missing).  With
    ``interpolation_weights`` cameras interpolated between neighbours follow
    each camera but the last."""
    calib = copy.deepcopy(calibration)
    aspect = resolution[2] / resolution[1]
    for cid in ids:
        c = calib[str(cid)]
        if c.get("fov_horizontal") is None:
            c["fov_horizontal"] = calib["fov_horizontal_average"]
        if synthetic:
            c["fov_vertical"] = c["fov_horizontal"] / aspect
        elif c.get("fov_vertical") is None:
            c["fov_vertical"] = calib["fov_vertical_average"]
    shared = {k: v for k, v in calib.items() if not k.isdigit()}
    cams = []
    for i, cid in enumerate(ids):
        c = calib[str(cid)]
        cams.append(camera_from_calibration(**{**shared, **c}, resolution=resolution,
                                            focus_depth_clip=focus_depth_clip))
        if interpolation_weights and i < len(ids) - 1:
            for w in interpolation_weights:
                ci = interpolate_camera_calibration(c, calib[str(ids[i + 1])], w, calib)
                cams.append(camera_from_calibration(**{**shared, **ci}, resolution=resolution,
                                                    focus_depth_clip=focus_depth_clip))
    return cams


def scalarflow_density_size(grid_size, calibration, y_scale="SF"):
    """(D, H, W) of the simulation grid: ``grid_size`` cells along x and z and
    ``ceil(grid_size * y_scale)`` along y, ``y_scale`` "SF" meaning the
    calibration's ``scale_y`` (reconstruct_sequence.py:761-764)."""
    if y_scale == "SF":
        y_scale = calibration["scale_y"]
    g = int(grid_size)
    return [g, int(math.ceil(g * y_scale)), g]


def scalarflow_sim_transform(density_size, calibration, render_targets=False):
    """Grid transform of the simulation grid ``density_size`` (D, H, W) in the
    calibrated world: a calibration transform (translation to the marker
    volume's centre, z flipped, uniform scale ``marker_width``), an identity
    randomisation transform and the centred, MIN-normalised grid; the domain's
    y centre is then raised to half the grid's world height plus 0.05
    (``render_targets``) or 0.005 (reconstruct_sequence.py:765-775)."""
    mw = float(calibration["marker_width"])
    volume_size = np.asarray([mw, mw * calibration["scale_y"], mw])
    center = _flip_z(np.asarray(calibration["volume_offset"]) + volume_size / 2.0)
    calibration_t = scene.Transform(translation=center, scale=[mw] * 3)
    randomization_t = scene.Transform(parent=calibration_t)
    grid = scene.GridTransform(density_size, center=True, normalize="MIN", parent=randomization_t)
    calibration_t.translation[1] = grid.grid_size_world()[1] / 2 + (0.05 if render_targets else 0.005)
    return grid


def scalarflow_capture_transform(calibration, capture_shape=(100, 178, 100)):
    """Grid transform of the ScalarFlow capture grid (D, H, W) = (100, 178, 100)
    by default: translation to the marker volume's corner, z flipped, uniform
    scale ``marker_width``, MIN-normalised (reconstruct_sequence.py:776-777)."""
    mw = float(calibration["marker_width"])
    shape = list(capture_shape)
    return scene.GridTransform(shape, translation=_flip_z(np.asarray(calibration["volume_offset"]) + [0, 0, mw]),
                               scale=[mw] * 3, normalize="MIN")
