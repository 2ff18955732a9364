"""Host-side camera and grid-transform matrices.

Mirrors the conventions of ``phitest/render/transform.py`` and
``phitest/render/camera.py`` so that callers build the same M / V / P / frustum
inputs as the reference renderer:

* ``Transform.get_local_transform`` = T @ R @ S (transform.py:247-251), Euler
  angles 'xyz' in degrees (transform.py:59-70, 184-190);
* ``GridTransform.get_local_transform`` = T @ R @ (N @ (S @ C)) with C the
  centring translation and N the size normalisation (transform.py:370-384);
* ``Camera.view_matrix`` = inverse of the camera's transform (camera.py:61-62),
  ``projection_matrix`` the OpenGL perspective matrix (camera.py:74-95),
  ``frustum`` = [near, far, left, right, top, bottom] (camera.py:64-65),
  ``depth_step`` = (far - near) / D (camera.py:98-100);
* matrices reach the operators as 16 floats read column-major, i.e. the
  transposed numpy matrix flattened (renderer.py:117-121).
"""
import math

import numpy as np


def translation_matrix(t):
    m = np.eye(4)
    m[:3, 3] = t
    return m


def scale_matrix(s):
    return np.diag([s[0], s[1], s[2], 1.0])


def rotation_matrix_xyz_deg(angles):
    """Extrinsic x, then y, then z rotation (scipy ``Rotation.from_euler('xyz')``)."""
    ax, ay, az = (math.radians(a) for a in angles)
    rx = np.array([[1, 0, 0], [0, math.cos(ax), -math.sin(ax)], [0, math.sin(ax), math.cos(ax)]])
    ry = np.array([[math.cos(ay), 0, math.sin(ay)], [0, 1, 0], [-math.sin(ay), 0, math.cos(ay)]])
    rz = np.array([[math.cos(az), -math.sin(az), 0], [math.sin(az), math.cos(az), 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = rz @ ry @ rx
    return m


class Transform:
    def __init__(self, translation=(0, 0, 0), rotation_deg=(0, 0, 0), scale=(1, 1, 1), parent=None):
        self.translation = np.asarray(translation, dtype=np.float64)
        self.rotation_deg = np.asarray(rotation_deg, dtype=np.float64)
        self.scale = np.asarray(scale, dtype=np.float64)
        self.parent = parent

    def get_local_transform(self):
        return translation_matrix(self.translation) @ (rotation_matrix_xyz_deg(self.rotation_deg) @ scale_matrix(self.scale))

    def get_transform_matrix(self):
        m = self.get_local_transform()
        if self.parent is not None:
            return self.parent.get_transform_matrix() @ m
        return m

    def get_inverse_transform(self):
        return np.linalg.inv(self.get_transform_matrix())


class MatrixTransform:
    """A transform given by its 4x4 matrix (``MatrixTransform``, transform.py:11-39);
    ``grid_size`` (D, H, W) is carried for cameras whose frustum grid it sets."""

    def __init__(self, matrix=None, parent=None, grid_size=None):
        self.matrix = np.eye(4) if matrix is None else np.asarray(matrix, dtype=np.float64)
        self.parent = parent
        self.grid_size = None if grid_size is None else [int(s) for s in grid_size]

    @classmethod
    def from_fwd_up_right_pos(cls, fwd, up, right, pos, parent=None):
        """Columns right, up, forward and the position (transform.py:32-39)."""
        m = np.eye(4)
        m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = right, up, fwd, pos
        return cls(m, parent)

    def get_local_transform(self):
        return self.matrix

    def get_transform_matrix(self):
        m = self.get_local_transform()
        if self.parent is not None:
            return self.parent.get_transform_matrix() @ m
        return m

    def get_inverse_transform(self):
        return np.linalg.inv(self.get_transform_matrix())


class GridTransform(Transform):
    """A grid of shape ``grid_size`` (D, H, W) placed in world space."""

    def __init__(self, grid_size, translation=(0, 0, 0), rotation_deg=(0, 0, 0), scale=(1, 1, 1),
                 center=False, normalize="NONE", parent=None):
        super().__init__(translation, rotation_deg, scale, parent)
        self.grid_size = [int(s) for s in grid_size]
        self.center = center
        self.normalize = normalize

    def get_local_transform(self):
        size = np.asarray(self.grid_size[::-1], dtype=np.float64)  # zyx -> xyz
        m = scale_matrix(self.scale)
        if self.center:
            m = m @ translation_matrix(-size / 2.0)
        if self.normalize == "ALL":
            m = scale_matrix(1.0 / size) @ m
        elif self.normalize == "MIN":
            m = scale_matrix([1.0 / size.min()] * 3) @ m
        elif self.normalize == "MAX":
            m = scale_matrix([1.0 / size.max()] * 3) @ m
        return translation_matrix(self.translation) @ (rotation_matrix_xyz_deg(self.rotation_deg) @ m)

    def grid_size_world(self):
        """World-space lengths of the grid's x, y and z edges (transform.py:390-395)."""
        m = self.get_transform_matrix()
        size = np.asarray(self.grid_size[::-1], dtype=np.float64)
        return np.linalg.norm(m[:3, :3] * size[None, :], axis=0)


class Camera:
    """Pinhole camera whose frustum grid is ``transform.grid_size`` (D, H, W)."""

    def __init__(self, transform, near_far=(1.0, 10.0), fov=None, aspect=1.0, trbl=(1, 1, -1, -1)):
        self.transform = transform
        self.clip = [float(near_far[0]), float(near_far[1])]
        self.trbl = list(trbl)
        if fov is not None:
            self.set_fov(fov, aspect)

    def set_fov(self, fov, aspect=1.0):
        half_h = math.tan(fov / 2.0 * math.pi / 180.0) * self.clip[0]
        half_v = half_h / aspect
        self.trbl = [half_v, half_h, -half_v, -half_h]

    @property
    def near(self):
        return self.clip[0]

    @property
    def far(self):
        return self.clip[1]

    def view_matrix(self):
        return self.transform.get_inverse_transform()

    def projection_matrix(self):
        t, r, b, l = self.trbl
        n, f = self.clip
        return np.asarray([[2 * n / (r - l), 0, 0, 0],
                           [0, 2 * n / (t - b), 0, 0],
                           [(r + l) / (r - l), (t + b) / (t - b), -(f + n) / (f - n), -1],
                           [0, 0, -2 * f * n / (f - n), 0]], dtype=np.float64).T

    def frustum(self):
        return np.asarray([self.clip[0], self.clip[1], self.trbl[3], self.trbl[1], self.trbl[0], self.trbl[2]],
                          dtype=np.float32)

    @property
    def depth_step(self):
        return (self.far - self.near) / self.transform.grid_size[0]


def colmajor(m):
    """16 floats of ``m`` in the operators' column-major order (``m.transpose()`` flattened)."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T).reshape(16).astype(np.float32)


def camera_params(cameras):
    """(V, P, F) arrays for a list of cameras: (n,16), (n,16), (n,6) float32
    (``Renderer._get_camera_params_batch``, renderer.py:117-121)."""
    V = np.stack([colmajor(c.view_matrix()) for c in cameras])
    P = np.stack([colmajor(c.projection_matrix()) for c in cameras])
    F = np.stack([c.frustum() for c in cameras]).astype(np.float32)
    return V, P, F


def model_params(transforms):
    return np.stack([colmajor(t.get_transform_matrix()) for t in transforms])


def volume_transform(grid_size_zyx):
    """Density grid placed as in the reconstruction setup: centred, normalised by the
    smallest side (reconstruct_sequence.py:767-772)."""
    return GridTransform(grid_size_zyx, center=True, normalize="MIN")


def orbit_cameras(frustum_dhw, yaws_deg, fov=40.0, distance=None, depth_half=None):
    """Cameras on a circle about +y looking at the origin (pattern of
    reconstruct_sequence.py:785, 1402).  Defaults: distance 1.3 x the unit-cube
    diagonal, near/far = distance -/+ half the diagonal."""
    diag = math.sqrt(3.0)
    distance = 1.3 * diag if distance is None else distance
    depth_half = diag / 2.0 if depth_half is None else depth_half
    cams = []
    for yaw in yaws_deg:
        t = GridTransform(frustum_dhw, translation=[0, 0, distance], parent=Transform(rotation_deg=[0, yaw, 0]))
        cams.append(Camera(t, near_far=[distance - depth_half, distance + depth_half], fov=fov, aspect=1.0))
    return cams
