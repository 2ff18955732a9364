"""Op-level oracle: the reference's TF op surface restated in NumPy.

Signatures mirror ``phitest/render/cuda/ops_loader.py`` and the ``REGISTER_OP``
attributes in ``resample_grid.cc``, ``raymarch_grid.cc`` and ``reduce_blend.cc``.
Matrices are passed as the reference passes them: per matrix 16 floats read
column-major (``renderer.py:117-121`` passes ``matrix.transpose()``).
"""
import numpy as np

from . import core
from .core import BORDER, CLAMP, WRAP, LINEAR, NEAREST, MIN, MAX, QUADRATIC


def _mats(a, n=None):
    a = np.asarray(a, dtype=np.float64).reshape(-1, 16)
    return a


def _frusta(f):
    return np.asarray(f, dtype=np.float64).reshape(-1, 6)


def _camera_loop(batch, num_cameras, separate_camera_batch):
    """(batch, camera, output slot) triples of the launchers' host loops
    (resample_grid.cu.cc:456-460, raymarch_grid.cu.cc:403-407)."""
    for b in range(batch):
        if separate_camera_batch:
            for c in range(num_cameras):
                yield b, c, c
        else:
            yield b, b, 0


def _index_grid(out_dims_zyx, dtype):
    d, h, w = out_dims_zyx
    z, y, x = np.meshgrid(np.arange(d), np.arange(h), np.arange(w), indexing="ij")
    return np.stack([x, y, z], -1).astype(dtype)


# ------------------------------------------------------------------ LUT resample

def _lut_positions(lut, relative, normalized, dtype):
    """Sample positions of ``kSampleGrid3DLuT`` (resample_grid.cu.cc:604-623):
    normalized coordinates are scaled by the *output* grid size, relative ones get
    the output index added."""
    d, h, w = lut.shape[:3]
    pos = lut.astype(dtype).copy()
    if normalized:
        pos[..., :3] = pos[..., :3] * np.array([w, h, d], dtype=dtype)
    if relative:
        pos[..., :3] = pos[..., :3] + _index_grid((d, h, w), dtype)
    return pos


def sample_grid_lut(input, lookup, interpolation=LINEAR, boundary=BORDER, mipmapping="NONE",
                    num_mipmaps=0, mip_bias=0.0, cell_center_offset=0.0,
                    separate_camera_batch=True, relative_coords=True, normalized_coords=False):
    """Forward of ``SampleGridLut`` (resample_grid.cc:94-120, 789-891;
    resample_grid.cu.cc:604-801).  input NDHWC, lookup VDHW4 -> NVDHWC."""
    x = np.asarray(input)
    dt = x.dtype
    lut = np.asarray(lookup)
    N = x.shape[0]
    V = lut.shape[0]
    if not separate_camera_batch and V != N:
        raise ValueError("camera batch must match data batch when not using global sampling.")
    out = np.zeros((N, V if separate_camera_batch else 1) + lut.shape[1:4] + (x.shape[-1],), dt)
    for b, c, slot in _camera_loop(N, V, separate_camera_batch):
        mips = core.mip_pyramid(x[b], num_mipmaps) if mipmapping != "NONE" else [x[b]]
        pos = _lut_positions(lut[c], relative_coords, normalized_coords, dt)
        out[b, slot] = core.sample_mip(mips, pos, cell_center_offset, interpolation, boundary,
                                       mipmapping, mip_bias, num_mipmaps)
    return out


def scatter_linear_exact(grad, p, g, boundary):
    """Adjoint of ``core.read_linear`` at positions p (..., 3) with output grad g (..., C)."""
    dims = core.dims_xyz(grad)
    fi, ci, fv, cv, w, inside = core.corner_setup(p, dims, boundary)
    wts = core.trilinear_weights(w)
    for k, (sx, sy, sz) in enumerate(core.CORNERS):
        ix = np.stack([(ci if sx else fi)[..., 0], (ci if sy else fi)[..., 1], (ci if sz else fi)[..., 2]], -1)
        va = (cv if sx else fv)[..., 0] & (cv if sy else fv)[..., 1] & (cv if sz else fv)[..., 2] & inside
        core.scatter_add(grad, ix, g * wts[k][..., None], va)


def scatter_linear_reference(grad, count, p, g, boundary):
    """``scatterGradInterpolated`` (resample_grid.cu.cc:1080-1131): BORDER scatters when
    -1 < p < dims on every axis; each receiving corner's sample count is incremented
    regardless of its weight."""
    dims = core.dims_xyz(grad)
    f = np.floor(p)
    w = p - f
    fi = f.astype(np.int64)
    ci = np.ceil(p).astype(np.int64)
    if boundary == BORDER:
        gate = np.all((p > -1) & (p < dims), axis=-1)
    else:
        gate = np.ones(p.shape[:-1], bool)
        if boundary == CLAMP:
            fi, ci = np.clip(fi, 0, dims - 1), np.clip(ci, 0, dims - 1)
        else:
            fi, ci = np.mod(fi, dims), np.mod(ci, dims)
    wts = core.trilinear_weights(w)
    for k, (sx, sy, sz) in enumerate(core.CORNERS):
        ix = np.stack([(ci if sx else fi)[..., 0], (ci if sy else fi)[..., 1], (ci if sz else fi)[..., 2]], -1)
        va = gate.copy()
        if boundary == BORDER:
            va &= np.all((ix >= 0) & (ix < dims), axis=-1)
        core.scatter_add(grad, ix, g * wts[k][..., None], va)
        core.scatter_add(count, ix, np.ones(ix.shape[:-1] + (1,), count.dtype), va)


def scatter_nearest_exact(grad, p, g, boundary):
    dims = core.dims_xyz(grad)
    idx = core.nearest_index(p)
    if boundary == BORDER:
        valid = np.all((idx >= 0) & (idx < dims), axis=-1)
        core.scatter_add(grad, np.where(valid[..., None], idx, 0), g, valid)
        return
    idx = np.clip(idx, 0, dims - 1) if boundary == CLAMP else np.mod(idx, dims)
    core.scatter_add(grad, idx, g, np.ones(idx.shape[:-1], bool))


def scatter_extremum_exact(grad, x, p, g, boundary, mode):
    """Adjoint of MIN / MAX: the gradient goes to the corner that produced the value."""
    _, arg, idx, valid = core.read_extremum(x, p, boundary, mode, return_arg=True)
    C = x.shape[-1]
    for k, cnr in enumerate(core.CORNERS):
        for ch in range(C):
            sel = arg[..., ch] == k
            gg = np.zeros(g.shape, g.dtype)
            gg[..., ch] = np.where(sel, g[..., ch], 0)
            core.scatter_add(grad, idx[cnr], gg, sel)


def _normalize_by_count(grad, count):
    n = count[..., 0]
    nz = n > 0
    grad[nz] = grad[nz] * (grad.dtype.type(1) / n[nz].astype(grad.dtype))[..., None]


def sample_grid_lut_grad(input, output_grad, lookup, interpolation=LINEAR, boundary=BORDER,
                         mipmapping="NONE", num_mipmaps=0, mip_bias=0.0, cell_center_offset=0.0,
                         separate_camera_batch=True, relative_coords=True, normalized_coords=False,
                         grad_mode="exact"):
    """Gradient of ``SampleGridLut`` (resample_grid.cc:124-150, 966-1073;
    resample_grid.cu.cc:1420-1665).  Returns (input_grad, lookup_grad).

    ``reference``: input grad is always a trilinear scatter, normalised per batch by
    the number of corner hits; the lookup grad is the data gradient for LINEAR only
    and ignores the normalized-coordinate scale.  ``exact``: the adjoint of the
    forward for every filter (nearest / argmin / argmax corner), lookup grad
    including the normalized-coordinate scale."""
    if mipmapping != "NONE":
        raise NotImplementedError("gradients of mipmapped sampling are not supported")
    x = np.asarray(input)
    dt = x.dtype
    lut = np.asarray(lookup)
    gy = np.asarray(output_grad, dtype=dt)
    N, V = x.shape[0], lut.shape[0]
    gx = np.zeros_like(x)
    glut = np.zeros(lut.shape, dt)
    cco = dt.type(cell_center_offset)
    for b in range(N):
        count = np.zeros(x.shape[1:4] + (1,), np.int64)
        for bb, c, slot in _camera_loop(N, V, separate_camera_batch):
            if bb != b:
                continue
            pos = _lut_positions(lut[c], relative_coords, normalized_coords, dt)
            p = pos[..., :3] - cco
            g = gy[b, slot]
            if interpolation == LINEAR:
                dg = core.data_gradient(x[b], p, boundary)  # (...,3,C)
                lg = np.sum(dg * g[..., None, :], axis=-1)  # (...,3)
                if normalized_coords and grad_mode == "exact":
                    d, h, w = lut.shape[1:4]
                    lg = lg * np.array([w, h, d], dtype=dt)
                if grad_mode == "exact":
                    glut[c, ..., :3] += lg  # every batch reading this lookup contributes
                else:
                    glut[c, ..., :3] = lg   # the reference kernel overwrites per batch
            if grad_mode == "reference":
                scatter_linear_reference(gx[b], count, p, g, boundary)
            elif interpolation == LINEAR:
                scatter_linear_exact(gx[b], p, g, boundary)
            elif interpolation == NEAREST:
                scatter_nearest_exact(gx[b], p, g, boundary)
            else:
                scatter_extremum_exact(gx[b], x[b], p, g, boundary, interpolation)
        if grad_mode == "reference":
            _normalize_by_count(gx[b], count)
    return gx, glut


# -------------------------------------------------------------- transform resample

def _positions_transform(coordinate_mode, out_dims_zyx, in_dims_xyz, cam, lod=False):
    idx = _index_grid(out_dims_zyx, np.float64) + 0.5
    out_xyz = np.array(out_dims_zyx[::-1], dtype=np.int64)
    if lod:
        return core.lod_of_positions(coordinate_mode, out_xyz, in_dims_xyz, cam, idx)
    return core.transform_positions(coordinate_mode, out_xyz, in_dims_xyz, cam, idx), None


def sample_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                          interpolation=LINEAR, boundary=BORDER, mipmapping="NONE", num_mipmaps=0,
                          mip_bias=0.0, coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5,
                          separate_camera_batch=True):
    """Forward of ``SampleGridTransform`` (resample_grid.cc:23-65, 365-509;
    resample_grid.cu.cc:255-544).  input NDHWC -> NVDHWC with DHW = output_shape.
    Positions are computed in float64 and rounded to the grid dtype."""
    x = np.asarray(input)
    dt = x.dtype
    M, Vm, P, F = _mats(matrix_m), _mats(matrix_v), _mats(matrix_p), _frusta(frustum_params)
    N, V = x.shape[0], Vm.shape[0]
    out_dims = tuple(int(s) for s in output_shape)
    in_xyz = core.dims_xyz(x[0])
    out = np.zeros((N, V if separate_camera_batch else 1) + out_dims + (x.shape[-1],), dt)
    use_mip = mipmapping != "NONE"
    for b, c, slot in _camera_loop(N, V, separate_camera_batch):
        cam = core.CameraMatrices(M[b], Vm[c], P[c], F[c])
        pos, lod = _positions_transform(coordinate_mode, out_dims, in_xyz, cam, lod=use_mip)
        pos4 = np.concatenate([pos, (lod if use_mip else np.zeros(pos.shape[:-1]))[..., None]], -1).astype(dt)
        mips = core.mip_pyramid(x[b], num_mipmaps) if use_mip else [x[b]]
        out[b, slot] = core.sample_mip(mips, pos4, cell_center_offset, interpolation, boundary,
                                       mipmapping, mip_bias, num_mipmaps)
    return out


def scatter_quadratic_exact(grad, p, g, boundary):
    if boundary == BORDER:
        return
    dims = core.dims_xyz(grad)
    idx, wts = core.quadratic_taps(p, dims, boundary)
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                ix = np.stack([idx[kx][..., 0], idx[ky][..., 1], idx[kz][..., 2]], -1)
                wgt = wts[kx][..., 0] * wts[ky][..., 1] * wts[kz][..., 2]
                core.scatter_add(grad, ix, g * wgt[..., None], np.ones(ix.shape[:-1], bool))


def scatter_quadratic_reference(grad, count, p, g, boundary):
    """``scatterGradQuadratic`` (resample_grid.cu.cc:903-1078)."""
    dims = core.dims_xyz(grad)
    dt = p.dtype
    center = np.floor(p + dt.type(0.5)).astype(np.int64)
    raw = [center - 1, center, center + 1]
    wts = [core.bspline2_weight(np.abs(p.astype(np.float64) - i)).astype(dt) for i in raw]
    if boundary == BORDER:
        gate = np.all((p > -1.5) & (p < dims), axis=-1)
        idx = raw
    elif boundary == CLAMP:
        gate = np.ones(p.shape[:-1], bool)
        idx = [np.clip(i, 0, dims - 1) for i in raw]
    else:
        gate = np.ones(p.shape[:-1], bool)
        idx = [np.mod(i, dims) for i in raw]
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                ix = np.stack([idx[kx][..., 0], idx[ky][..., 1], idx[kz][..., 2]], -1)
                va = gate.copy()
                if boundary == BORDER:
                    # per-tap checks: prev must be >= 0, next < dims, centre unchecked
                    # (resample_grid.cu.cc:933-1076); the centre-centre-centre tap is skipped.
                    for a, k in zip(range(3), (kx, ky, kz)):
                        if k == 0:
                            va &= ix[..., a] >= 0
                        elif k == 2:
                            va &= ix[..., a] < dims[a]
                    if (kx, ky, kz) == (1, 1, 1):
                        va &= False
                    # the reference leaves centre taps unchecked and writes out of bounds
                    # for them; those contributions are dropped here
                    va &= np.all((ix >= 0) & (ix < dims), axis=-1)
                wgt = wts[kx][..., 0] * wts[ky][..., 1] * wts[kz][..., 2]
                core.scatter_add(grad, np.where(va[..., None], ix, 0), g * wgt[..., None], va)
                core.scatter_add(count, np.where(va[..., None], ix, 0), np.ones(ix.shape[:-1] + (1,), count.dtype), va)


def sample_grid_transform_grad(input, output_grad, matrix_m, matrix_v, matrix_p, frustum_params,
                               interpolation=LINEAR, boundary=BORDER, mipmapping="NONE", num_mipmaps=0,
                               mip_bias=0.0, coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5,
                               separate_camera_batch=True, grad_mode="exact"):
    """Gradient of ``SampleGridTransform`` (resample_grid.cc:68-92, 538-717;
    resample_grid.cu.cc:1160-1387).  ``reference`` is the count-normalised scatter
    (normalised per batch after all cameras); ``exact`` is the adjoint."""
    if mipmapping != "NONE":
        raise NotImplementedError("gradients of mipmapped sampling are not supported")
    x = np.asarray(input)
    dt = x.dtype
    gy = np.asarray(output_grad, dtype=dt)
    M, Vm, P, F = _mats(matrix_m), _mats(matrix_v), _mats(matrix_p), _frusta(frustum_params)
    N, V = x.shape[0], Vm.shape[0]
    out_dims = gy.shape[2:5]
    in_xyz = core.dims_xyz(x[0])
    gx = np.zeros_like(x)
    cco = dt.type(cell_center_offset)
    for b in range(N):
        count = np.zeros(x.shape[1:4] + (1,), np.int64)
        for bb, c, slot in _camera_loop(N, V, separate_camera_batch):
            if bb != b:
                continue
            cam = core.CameraMatrices(M[b], Vm[c], P[c], F[c])
            pos, _ = _positions_transform(coordinate_mode, out_dims, in_xyz, cam)
            p = pos.astype(dt) - cco
            g = gy[b, slot]
            if grad_mode == "reference":
                if interpolation == QUADRATIC:
                    scatter_quadratic_reference(gx[b], count, p, g, boundary)
                else:
                    scatter_linear_reference(gx[b], count, p, g, boundary)
            elif interpolation == LINEAR:
                scatter_linear_exact(gx[b], p, g, boundary)
            elif interpolation == NEAREST:
                scatter_nearest_exact(gx[b], p, g, boundary)
            elif interpolation == QUADRATIC:
                scatter_quadratic_exact(gx[b], p, g, boundary)
            else:
                raise ValueError(interpolation)
        if grad_mode == "reference":
            _normalize_by_count(gx[b], count)
    return gx


def lod_transform(input_shape, matrix_mv, matrix_p, frustum_params, output_shape,
                  inverse_transform=False, linearize_depth=True, relative_coords=False):
    """``LodTransform`` (resample_grid.cc:152-172, 1089-1178; resample_grid.cu.cc:1702-1786):
    per camera a lookup table (x, y, z, LoD) of sampling positions."""
    MV, P, F = _mats(matrix_mv), _mats(matrix_p), _frusta(frustum_params)
    V = MV.shape[0]
    out_dims = tuple(int(s) for s in output_shape)
    in_xyz = np.array(list(input_shape)[::-1], dtype=np.int64)
    if linearize_depth:
        mode = "TRANSFORM_LINDEPTH_REVERSE" if inverse_transform else "TRANSFORM_LINDEPTH"
    else:
        mode = "TRANSFORM_REVERSE" if inverse_transform else "TRANSFORM"
    out = np.zeros((V,) + out_dims + (4,), np.float64)
    for v in range(V):
        cam = core.CameraMatrices(None, MV[v], P[v], F[v])
        idx = _index_grid(out_dims, np.float64) + 0.5
        od = np.array(out_dims[::-1])
        pos = core.transform_positions(mode, od, in_xyz, cam, idx)
        lod = core.calc_lod(mode, od, in_xyz, cam, idx)
        if relative_coords:
            pos = pos - _index_grid(out_dims, np.float64)
        out[v] = np.concatenate([pos, lod[..., None]], -1)
    return out.astype(np.float32)


# ------------------------------------------------------------------------ raymarch

def ray_setup(cam, in_xyz, out_dims_zyx, boundary, rows=None):
    """Per-pixel ray start, step and step count (``getRaymarchStep``,
    raymarch_grid.cu.cc:109-200), in float64.  Returns start (H,W,3), step (H,W,3),
    steps (H,W) int, hit (H,W) bool and the far end used by the reference backward.
    ``rows = (y0, y1)`` restricts the rays to image rows y0..y1-1 of the full
    H x W image (the arrays then have y1 - y0 rows)."""
    D, H, W = out_dims_zyx
    dims = np.array([W, H, D], dtype=np.float64)
    zmax = float(max(D - 1, 1))
    y0, y1 = (0, H) if rows is None else (int(rows[0]), int(rows[1]))
    y, x = np.meshgrid(np.arange(y0, y1), np.arange(W), indexing="ij")
    i0 = np.stack([x + 0.5, y + 0.5, np.full(x.shape, 0.5)], -1)
    i1 = np.stack([x + 0.5, y + 0.5, np.full(x.shape, zmax + 0.5)], -1)
    start = core.idx_to_os(i0, dims, cam)
    end = core.idx_to_os(i1, dims, cam)
    step = (end - start) / zmax
    steps = np.full(x.shape, D, dtype=np.int64)
    hit = np.ones(x.shape, bool)
    if boundary == BORDER:
        d = end - start
        rd = d / np.linalg.norm(d, axis=-1, keepdims=True)
        bmax = in_xyz.astype(np.float64)
        half = bmax * 0.5 - 0.5
        co = start - bmax * 0.5
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / rd
            n = inv * co
            k = np.abs(inv) * half
            # fmaxf / fminf ignore NaN (an axis-parallel ray gives inf*0 in the slab test)
            tmin = np.fmax.reduce(-n - k, axis=-1)
            tmax = np.fmin.reduce(k - n, axis=-1)
        hit = ~((tmin > tmax) | (tmax < 0))
        end = start + rd * (tmax[..., None] + 1.0)
        start = start + rd * np.maximum(tmin - 1.0, 0.0)[..., None]
        ss = np.linalg.norm(step, axis=-1)
        rl = np.linalg.norm(start - end, axis=-1)
        start = np.where(hit[..., None], start, 0.0)
        end = np.where(hit[..., None], end, 0.0)
        with np.errstate(invalid="ignore"):
            steps = np.where(hit, np.where(hit, rl / ss, 0.0).astype(np.int64) + 2, 0)
    return start, step, steps, hit, end


def _ray_positions(start, step, steps, dt):
    """Sample positions ``start + step + step + ...`` accumulated in the grid dtype,
    as the kernel's ``samplePos += step`` (raymarch_grid.cu.cc:241-247)."""
    n = int(steps.max()) if steps.size else 0
    pos = np.empty((n,) + start.shape, dt)
    cur = start.astype(dt)
    st = step.astype(dt)
    for i in range(n):
        pos[i] = cur
        cur = cur + st
    return pos


def _v2_sample(grid, pos, interpolation, boundary):
    """``Sampling::sample3D`` of sampling_v2.hpp:358-372 (cell centre offset 0.5).
    MIN / MAX use the corner extrema with the resample sampler's semantics."""
    return core.read(grid, pos - grid.dtype.type(0.5), interpolation, boundary)


def raymarch_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                            interpolation=LINEAR, boundary=BORDER, blending_mode="BEER_LAMBERT",
                            keep_dims=False, separate_camera_batch=True, rows=None):
    """Forward of ``RaymarchGridTransform`` (raymarch_grid.cc:29-63, 208-313;
    raymarch_grid.cu.cc:202-252, 359-433).  input NDHWC -> NVHWC (NV1HWC with keep_dims).
    ``rows = (y0, y1)``: only image rows y0..y1-1 (output height y1 - y0)."""
    x = np.asarray(input)
    dt = x.dtype
    M, Vm, P, F = _mats(matrix_m), _mats(matrix_v), _mats(matrix_p), _frusta(frustum_params)
    N, V = x.shape[0], Vm.shape[0]
    D, H, W = (int(s) for s in output_shape)
    C = x.shape[-1]
    in_xyz = core.dims_xyz(x[0])
    Hr = H if rows is None else int(rows[1]) - int(rows[0])
    out = np.zeros((N, V if separate_camera_batch else 1, Hr, W, C), dt)
    for b, c, slot in _camera_loop(N, V, separate_camera_batch):
        cam = core.CameraMatrices(M[b], Vm[c], P[c], F[c])
        start, step, steps, hit, _ = ray_setup(cam, in_xyz, (D, H, W), boundary, rows)
        pos = _ray_positions(start, step, steps, dt)
        acc = np.zeros((Hr, W, C), dt)
        for i in range(pos.shape[0]):
            active = (i < steps) & hit
            s = _v2_sample(x[b], pos[i], interpolation, boundary)
            nxt = core.blend(acc, s, blending_mode)
            acc = np.where(active[..., None], nxt, acc)
        out[b, slot] = acc
    if keep_dims:
        out = out[:, :, None]
    return out


def raymarch_grid_transform_grad(input, output, output_grad, matrix_m, matrix_v, matrix_p,
                                 frustum_params, output_shape, interpolation=LINEAR, boundary=BORDER,
                                 blending_mode="BEER_LAMBERT", keep_dims=False,
                                 separate_camera_batch=True, grad_mode="exact", rows=None):
    """Gradient of ``RaymarchGridTransform`` (raymarch_grid.cc:67-92, 363-497;
    raymarch_grid.cu.cc:458-724).

    ``reference``: back-to-front from the far end with ``pos -= step`` (for BORDER a
    different lattice than the forward's), accumulator rebuilt by subtraction,
    scatter weighted and divided per voxel by the summed weights, per camera.
    ``exact``: the adjoint of the forward at the forward's own sample positions.
    ``rows = (y0, y1)``: the rays of image rows y0..y1-1 only (``output`` and
    ``output_grad`` hold those rows); the exact gradients of row bands add up to
    the full image's."""
    if interpolation != LINEAR:
        raise NotImplementedError("raymarch gradients support LINEAR interpolation only")
    x = np.asarray(input)
    dt = x.dtype
    y = np.asarray(output, dtype=dt)
    gy = np.asarray(output_grad, dtype=dt)
    if keep_dims:
        y, gy = y[:, :, 0], gy[:, :, 0]
    M, Vm, P, F = _mats(matrix_m), _mats(matrix_v), _mats(matrix_p), _frusta(frustum_params)
    N, V = x.shape[0], Vm.shape[0]
    D, H, W = (int(s) for s in output_shape)
    C = x.shape[-1]
    in_xyz = core.dims_xyz(x[0])
    gx = np.zeros_like(x)
    for b, c, slot in _camera_loop(N, V, separate_camera_batch):
        cam = core.CameraMatrices(M[b], Vm[c], P[c], F[c])
        start, step, steps, hit, end = ray_setup(cam, in_xyz, (D, H, W), boundary, rows)
        g = gy[b, slot]
        if grad_mode == "exact":
            pos = _ray_positions(start, step, steps, dt)
            n = pos.shape[0]
            if n == 0:  # every ray of this camera misses the clip box
                continue
            cells = np.stack([_v2_sample(x[b], pos[i], interpolation, boundary) for i in range(n)])
            active = (np.arange(n)[:, None, None] < steps[None]) & hit[None]
            cells = np.where(active[..., None], cells, 0)
            dcells = core.blend_sequence_exact_grad(cells, g, blending_mode)
            for i in range(n):
                scatter_linear_exact(gx[b], pos[i] - dt.type(0.5), np.where(active[i][..., None], dcells[i], 0), boundary)
        else:
            buf = np.zeros_like(x[b])
            wsum = np.zeros(x.shape[1:4] + (1,), dt)
            sp = end.astype(dt)
            st = step.astype(dt)
            acc = y[b, slot].copy()
            gout = g.copy()
            n = int(steps.max()) if steps.size else 0
            for k in range(n):
                i = n - 1 - k  # rays with fewer steps start later
                active = (i < steps) & hit
                s = _v2_sample(x[b], sp, interpolation, boundary)
                dcell, gnew, anew = core.blend_gradients_reference(gout, s, acc, blending_mode)
                _scatter_weighted(buf, wsum, sp - dt.type(0.5), np.where(active[..., None], dcell, 0),
                                  active, boundary)
                gout = np.where(active[..., None], gnew, gout)
                acc = np.where(active[..., None], anew, acc)
                sp = np.where(active[..., None], sp - st, sp)
            nz = wsum[..., 0] > 0
            gx[b][nz] += buf[nz] * (dt.type(1) / wsum[nz])
    if keep_dims:
        pass
    return gx


def _scatter_weighted(buf, wsum, p, g, active, boundary):
    """``scatterGrad3DInterpolated`` with per-voxel weight sums (sampling_v2.hpp:438-559)."""
    dims = core.dims_xyz(buf)
    f = np.floor(p)
    w = p - f
    fi = f.astype(np.int64)
    ci = np.ceil(p).astype(np.int64)
    if boundary == BORDER:
        gate = np.all((p > -1) & (p < dims), axis=-1) & active
    else:
        gate = active.copy()
        if boundary == CLAMP:
            fi, ci = np.clip(fi, 0, dims - 1), np.clip(ci, 0, dims - 1)
        else:
            fi, ci = np.mod(fi, dims), np.mod(ci, dims)
    wts = core.trilinear_weights(w)
    for k, (sx, sy, sz) in enumerate(core.CORNERS):
        ix = np.stack([(ci if sx else fi)[..., 0], (ci if sy else fi)[..., 1], (ci if sz else fi)[..., 2]], -1)
        va = gate.copy()
        if boundary == BORDER:
            va &= np.all((ix >= 0) & (ix < dims), axis=-1)
        ix = np.where(va[..., None], ix, 0)
        core.scatter_add(buf, ix, g * wts[k][..., None], va)
        core.scatter_add(wsum, ix, wts[k][..., None].astype(wsum.dtype), va)


# -------------------------------------------------------------------- reduce blend

def reduce_grid_blend(input, blending_mode="BEER_LAMBERT", keep_dims=False):
    """``ReduceGridBlend`` (reduce_blend.cc:24-35; reduce_blend.cu.cc:34-52):
    front-to-back blend along D.  NDHWC -> NHWC, or all prefixes NDHWC with keep_dims."""
    x = np.asarray(input)
    acc = np.zeros((x.shape[0],) + x.shape[2:], x.dtype)
    outs = []
    for i in range(x.shape[1]):
        acc = core.blend(acc, x[:, i], blending_mode)
        outs.append(acc)
    return np.stack(outs, 1) if keep_dims else acc


def reduce_grid_blend_grad(output_grad, output, input, blending_mode="BEER_LAMBERT", keep_dims=False,
                           grad_mode="reference"):
    """``ReduceGridBlendGrad`` (reduce_blend.cc:38-56; reduce_blend.cu.cc:55-80).
    ``reference`` rebuilds the accumulator from the stored output as the kernel does;
    ``exact`` recomputes it forward."""
    x = np.asarray(input)
    gy = np.asarray(output_grad, dtype=x.dtype)
    y = np.asarray(output, dtype=x.dtype)
    D = x.shape[1]
    if grad_mode == "exact":
        if keep_dims:
            # each prefix output contributes; accumulate the adjoint of every prefix
            gx = np.zeros_like(x)
            for j in range(D):
                cells = np.moveaxis(x[:, :j + 1], 1, 0)
                gx[:, :j + 1] += np.moveaxis(core.blend_sequence_exact_grad(cells, gy[:, j], blending_mode), 0, 1)
            return gx
        cells = np.moveaxis(x, 1, 0)
        return np.moveaxis(core.blend_sequence_exact_grad(cells, gy, blending_mode), 0, 1)
    gx = np.zeros_like(x)
    grads = np.zeros_like(x[:, 0])
    prev = np.zeros_like(x[:, 0])
    if not keep_dims:
        grads = gy.copy()
        prev = y.copy()
    for i in range(D - 1, -1, -1):
        if keep_dims:
            grads = grads + gy[:, i]
            prev = y[:, i].copy()
        d, grads, prev = core.blend_gradients_reference(grads, x[:, i], prev, blending_mode)
        gx[:, i] = d
    return gx


# ---------------------------------------------------------- background composite

def background_composite(image, background):
    """Background composite of ``Renderer.render_density`` (renderer.py:779-781,
    804-806): ``t = exp(-image[..., -1:])``, the alpha channel cut, and
    ``image[..., :-1] + background * t``; ``background`` broadcasts to the
    per-camera image (V, H, W, C - 1) and is shared by the batch."""
    x = np.asarray(image)
    t = np.exp(-x[..., -1:])
    return x[..., :-1] + np.asarray(background, x.dtype) * t


def background_composite_grad(image, background, output_grad):
    """Adjoint of :func:`background_composite`: (d image, d background), the latter
    summed over the batch."""
    x = np.asarray(image)
    g = np.asarray(output_grad, x.dtype)
    b = np.broadcast_to(np.asarray(background, x.dtype), x.shape[1:-1] + (x.shape[-1] - 1,))
    t = np.exp(-x[..., -1:])
    gi = np.concatenate([g, -t * (b * g).sum(-1, keepdims=True)], -1)
    gb = (t * g).sum(0)
    return gi, gb
