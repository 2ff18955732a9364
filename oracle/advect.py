"""Advection oracle: semi-Lagrangian / MacCormack warps of density and of the
MAC-staggered velocity, restated from the TensorFlow composition in
``phitest/render/data_structures.py:1634-1737`` (density) and ``:1081-1164``
(velocity), which call the LUT resample op (``renderer.py:559-574``).

Grids here carry no batch axis: density ``(D, H, W, 1)``; MAC components
``ux (D, H, W+1)``, ``uy (D, H+1, W)``, ``uz (D+1, H, W)`` without channel
(``data_structures.py:764-773``).
"""
import numpy as np

from . import core, ops
from .core import LINEAR, MIN, MAX


def centered_velocity(ux, uy, uz):
    """``VelocityGrid.centered`` (data_structures.py:1634-1654): average of the two
    faces of each cell, ``(right + left) * 0.5``.  Returns (D, H, W, 3) xyz."""
    h = ux.dtype.type(0.5)
    cx = (ux[:, :, 1:] + ux[:, :, :-1]) * h
    cy = (uy[:, 1:] + uy[:, :-1]) * h
    cz = (uz[1:] + uz[:-1]) * h
    return np.stack([cx, cy, cz], -1)


def centered_velocity_adjoint(g_uc, shapes):
    """Adjoint of :func:`centered_velocity`; ``shapes`` are the three face-grid shapes."""
    h = g_uc.dtype.type(0.5)
    gx = np.zeros(shapes[0], g_uc.dtype)
    gy = np.zeros(shapes[1], g_uc.dtype)
    gz = np.zeros(shapes[2], g_uc.dtype)
    gx[:, :, 1:] += g_uc[..., 0] * h
    gx[:, :, :-1] += g_uc[..., 0] * h
    gy[:, 1:] += g_uc[..., 1] * h
    gy[:, :-1] += g_uc[..., 1] * h
    gz[1:] += g_uc[..., 2] * h
    gz[:-1] += g_uc[..., 2] * h
    return gx, gy, gz


def _idx(shape, dt, z0=0):
    d, h, w = shape
    z, y, x = np.meshgrid(np.arange(z0, z0 + d), np.arange(h), np.arange(w), indexing="ij")
    return np.stack([x, y, z], -1).astype(dt)


def _positions(lut, shape, dt, z0, sign):
    """Sample positions ``sign * lut + index`` of a lattice whose first plane is
    global plane ``z0``, returned relative to that plane: the global position
    is formed first (the arithmetic of the whole-grid warp) and ``z0`` then
    subtracted, which is exact, so a slab ``data[z0:z0+d]`` is sampled at the
    same fractions as the whole grid."""
    p = (lut if sign > 0 else -lut) + _idx(shape, dt, z0)
    if z0:
        p[..., 2] -= dt.type(z0)
    return p


def maccormack(data, lut, order=2, clamp="MC_SMOOTH", boundary="CLAMP", return_state=False, z0=0):
    """Warp ``data`` (D,H,W,C) by a relative lookup ``lut`` (D,H,W,3) on the same
    lattice (``VelocityGrid.warp`` data_structures.py:1690-1737 /
    ``_warp_vel_component`` :1081-1106).

    order 1: semi-Lagrangian ``fwd = S(data, idx+lut)``.
    order 2: ``back = S(fwd, idx-lut)``; ``corr = fwd + 0.5*(data-back)``; with
    MC_SMOOTH the voxels where ``corr`` leaves the [min, max] of the forward
    lookup's 8 corners revert to ``fwd``.  ``clamp='NEGATIVE'`` applies max(.,0).

    ``z0``: ``data`` and ``lut`` are planes z0.. of a larger grid (a slab cut with
    a halo by a caller that splits the warp over processes); positions are then
    formed with global indices as in the whole-grid warp.  The slab's own edge
    planes see the boundary rule, so only planes a trace cannot carry past the
    slab edge match the whole-grid result.
    """
    dt = data.dtype
    p1 = _positions(lut, data.shape[:3], dt, z0, 1)
    fwd = core.read_linear(data, p1, boundary)
    st = {"p1": p1, "fwd": fwd}
    out = fwd
    if order == 2:
        p2 = _positions(lut, data.shape[:3], dt, z0, -1)
        back = core.read_linear(fwd, p2, boundary)
        corr = fwd + dt.type(0.5) * (data - back)
        st.update(p2=p2, back=back, corr=corr)
        if clamp == "MC":
            raise NotImplementedError("MIM and MAX warp sampling have wrong gradients.")
        if clamp == "MC_SMOOTH":
            mn = core.read_extremum(data, p1, boundary, MIN)
            mx = core.read_extremum(data, p1, boundary, MAX)
            mask = (corr < mn) | (corr > mx)
            corr = np.where(mask, fwd, corr)
            st.update(mask=mask, mn=mn, mx=mx)
        out = corr
    elif order != 1:
        raise ValueError("Unsupported warp order '{}'".format(order))
    if clamp == "NEGATIVE":
        st["pre_neg"] = out
        out = np.maximum(out, 0)
    if return_state:
        return out, st
    return out


def _scatter(grid_like, p, g, boundary, mode):
    gx = np.zeros_like(grid_like)
    if mode == "exact":
        ops.scatter_linear_exact(gx, p, g, boundary)
    else:
        cnt = np.zeros(grid_like.shape[:3] + (1,), np.int64)
        ops.scatter_linear_reference(gx, cnt, p, g, boundary)
        ops._normalize_by_count(gx, cnt)
    return gx


def maccormack_grad(data, lut, grad_out, order=2, clamp="MC_SMOOTH", boundary="CLAMP", grad_mode="exact", z0=0):
    """Backward of :func:`maccormack`.  Returns (d_data, d_lut).

    ``exact``: adjoint of the composition (the MC_SMOOTH mask is piecewise constant,
    MIN/MAX lookups carry no gradient, as ``tf.less/tf.greater`` give none).
    ``reference``: the same TF composition but each LUT-resample adjoint is the
    reference's count-normalised scatter (``ops_loader.py:41-58``).
    ``z0``: slab origin as in :func:`maccormack`."""
    dt = data.dtype
    out, st = maccormack(data, lut, order, clamp, boundary, return_state=True, z0=z0)
    g = np.asarray(grad_out, dt)
    if clamp == "NEGATIVE":
        g = np.where(st["pre_neg"] >= 0, g, 0)
    half = dt.type(0.5)
    if order == 2:
        g_fwd = g.copy()
        g_corr = np.where(st["mask"], 0, g) if "mask" in st else g
        g_data = half * g_corr
        g_back = -(half * g_corr)
        g_fwd = g_fwd + _scatter(st["fwd"], st["p2"], g_back, boundary, grad_mode)
        d_lut2 = np.sum(core.data_gradient(st["fwd"], st["p2"], boundary) * g_back[..., None, :], -1)
    else:
        g_fwd = g
        g_data = np.zeros_like(data)
        d_lut2 = 0
    g_data = g_data + _scatter(data, st["p1"], g_fwd, boundary, grad_mode)
    d_lut1 = np.sum(core.data_gradient(data, st["p1"], boundary) * g_fwd[..., None, :], -1)
    return g_data, d_lut1 - d_lut2


def density_maccormack(rho, ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """``DensityGrid.warped`` -> ``VelocityGrid.warp`` (data_structures.py:614-617,1690):
    the lookup is ``centered(u) * (-dt)``."""
    lut = centered_velocity(ux, uy, uz) * rho.dtype.type(-dt)
    return maccormack(rho, lut, order, clamp, boundary)


def density_maccormack_grad(rho, ux, uy, uz, grad_out, dt=1.0, order=2, clamp="MC_SMOOTH",
                            boundary="CLAMP", grad_mode="exact"):
    """Gradient of :func:`density_maccormack` w.r.t. (rho, ux, uy, uz)."""
    lut = centered_velocity(ux, uy, uz) * rho.dtype.type(-dt)
    g_rho, g_lut = maccormack_grad(rho, lut, grad_out, order, clamp, boundary, grad_mode)
    g_uc = g_lut * rho.dtype.type(-dt)
    gx, gy, gz = centered_velocity_adjoint(g_uc, (ux.shape, uy.shape, uz.shape))
    return g_rho, gx, gy, gz


# ------------------------------------------------------------ MAC velocity warp

# Offsets used to resample one face component onto another component's lattice
# (``_sampled_to_component_shape``, data_structures.py:1655-1682): keys are
# (source, target), values xyz offsets added to the target index.
COMPONENT_OFFSETS = {
    ("x", "y"): (0.5, -0.5, 0.0), ("x", "z"): (0.5, 0.0, -0.5),
    ("y", "x"): (-0.5, 0.5, 0.0), ("y", "z"): (0.0, 0.5, -0.5),
    ("z", "x"): (-0.5, 0.0, 0.5), ("z", "y"): (0.0, -0.5, 0.5),
}


def resample_offset(src, target_shape, offset, boundary="CLAMP"):
    """``Renderer.resample_grid3D_offset`` (renderer.py:922-936): relative LUT sample of
    ``src`` (D,H,W) at ``target index + offset``."""
    dt = src.dtype
    p = _idx(target_shape, dt) + np.asarray(offset, dt)
    return core.read_linear(src[..., None], p, boundary)[..., 0]


def resample_offset_adjoint(g, src_shape, offset, boundary="CLAMP", grad_mode="exact"):
    """Adjoint of :func:`resample_offset`; ``reference`` divides by the per-voxel
    sample count as the LUT op's registered gradient does."""
    dt = g.dtype
    p = _idx(g.shape, dt) + np.asarray(offset, dt)
    out = np.zeros(tuple(src_shape) + (1,), dt)
    if grad_mode == "exact":
        ops.scatter_linear_exact(out, p, g[..., None], boundary)
    else:
        cnt = np.zeros(tuple(src_shape) + (1,), np.int64)
        ops.scatter_linear_reference(out, cnt, p, g[..., None], boundary)
        ops._normalize_by_count(out, cnt)
    return out[..., 0]


def component_lut(comps, target, dt_step, boundary="CLAMP"):
    """Lookup for warping face component ``target`` ('x','y','z'):
    ``-vel*dt`` of all three components sampled on the target lattice
    (data_structures.py:1119,1127,1136)."""
    names = ("x", "y", "z")
    shape = comps[names.index(target)].shape
    vel = []
    for n, c in zip(names, comps):
        v = c if n == target else resample_offset(c, shape, COMPONENT_OFFSETS[(n, target)], boundary)
        vel.append((-v) * c.dtype.type(dt_step))
    return np.stack(vel, -1)


def velocity_maccormack(ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """``VelocityGrid.warped`` with the grid's own velocity (data_structures.py:1108-1164)."""
    comps = (ux, uy, uz)
    out = []
    for n, c in zip(("x", "y", "z"), comps):
        lut = component_lut(comps, n, dt, boundary)
        out.append(maccormack(c[..., None], lut, order, clamp, boundary)[..., 0])
    return tuple(out)


def velocity_maccormack_grad(ux, uy, uz, grads, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP",
                             grad_mode="exact"):
    """Gradient of :func:`velocity_maccormack` w.r.t. (ux, uy, uz): the data path of each
    component plus the lookup paths through every component's resampled velocity."""
    comps = (ux, uy, uz)
    names = ("x", "y", "z")
    acc = [np.zeros_like(c) for c in comps]
    for ti, (n, c) in enumerate(zip(names, comps)):
        lut = component_lut(comps, n, dt, boundary)
        g_data, g_lut = maccormack_grad(c[..., None], lut, grads[ti][..., None], order, clamp, boundary, grad_mode)
        acc[ti] += g_data[..., 0]
        g_vel = -(g_lut * c.dtype.type(dt))
        for si, s in enumerate(names):
            if s == n:
                acc[si] += g_vel[..., si]
            else:
                acc[si] += resample_offset_adjoint(g_vel[..., si], comps[si].shape, COMPONENT_OFFSETS[(s, n)],
                                                   boundary, grad_mode)
    return tuple(acc)
