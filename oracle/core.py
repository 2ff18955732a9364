"""Sampler, blend and transform primitives of the oracle (NumPy).

Arrays follow the reference layout: a grid is ``(D, H, W, C)`` (NDHWC
without N, x fastest); positions are ``(..., 3)`` in **xyz** order, in cell
coordinates where cell centres sit at integer positions (the reference
subtracts ``cell_center_offset`` before interpolating).  Arithmetic is done
in the dtype of the grid, so a float32 grid reproduces the reference's fp32
operation order and a float64 grid gives the FP64 oracle.
"""
import numpy as np

BORDER, CLAMP, WRAP = "BORDER", "CLAMP", "WRAP"
NEAREST, LINEAR, MIN, MAX, QUADRATIC = "NEAREST", "LINEAR", "MIN", "MAX", "QUADRATIC"

# vectormath.hpp:13-19 (FLOAT_MAX is written as a double literal and narrowed)
FLOAT_MAX = 3.40282e38


def dims_xyz(grid):
    """(W, H, D) of a (D, H, W, C) grid, as the reference's ``dimensionsFromGridShape``
    (dimensions_v2.hpp:29-31)."""
    d, h, w = grid.shape[:3]
    return np.array([w, h, d], dtype=np.int64)


def lerp(a, b, t):
    """helper_math / vmath lerp ``a + t*(b-a)`` (vectormath_helper.hpp:246-248)."""
    return a + t * (b - a)


def _fetch(grid, idx, valid=None):
    """Read grid[z, y, x, :] for integer xyz indices; invalid entries read 0."""
    v = grid[idx[..., 2], idx[..., 1], idx[..., 0]]
    if valid is not None:
        v = np.where(valid[..., None], v, np.zeros((), grid.dtype))
    return v


def _wrap(idx, dims):
    # The reference's positivemod ``(v%m) + m*(v<0)`` (vectormath.hpp:263-268) maps
    # v == -m to m, an out-of-range read; a true modulo is used instead.
    return np.mod(idx, dims)


def corner_setup(p, dims, boundary):
    """Corner indices, validity and fractional weights of a trilinear lookup.

    Follows ``read3DInterpolated`` (sampling.hpp:371-465, sampling_v2.hpp:37-124):
    weights are ``fract(p)``; CLAMP clamps both corners to ``[0, dims-1]``; WRAP
    wraps them; BORDER keeps them and marks out-of-range corners invalid.
    Returns (floor_idx, ceil_idx, floor_valid, ceil_valid, w, inside) where
    ``inside`` is the BORDER domain test ``0 <= p+0.5 < dims``.
    """
    dt = p.dtype
    f = np.floor(p)
    w = p - f
    c = np.ceil(p)
    fi = f.astype(np.int64)
    ci = c.astype(np.int64)
    one = np.ones(p.shape, dtype=bool)
    if boundary == BORDER:
        q = p + dt.type(0.5)
        inside = np.all((q >= 0) & (q < dims), axis=-1)
        fv = (fi > -1) & (fi < dims)
        cv = (ci > -1) & (ci < dims)
        fi = np.where(fv, fi, 0)
        ci = np.where(cv, ci, 0)
        return fi, ci, fv, cv, w, inside
    if boundary == CLAMP:
        fi = np.clip(fi, 0, dims - 1)
        ci = np.clip(ci, 0, dims - 1)
    elif boundary == WRAP:
        fi = _wrap(fi, dims)
        ci = _wrap(ci, dims)
    else:
        raise ValueError(boundary)
    return fi, ci, one, one, w, np.ones(p.shape[:-1], dtype=bool)


CORNERS = [(sx, sy, sz) for sz in (0, 1) for sy in (0, 1) for sx in (0, 1)]


def corner_values(grid, p, boundary):
    """The 8 corner reads of a trilinear lookup as dict[(sx,sy,sz)] -> (..., C),
    plus weights, validity and domain mask."""
    dims = dims_xyz(grid)
    fi, ci, fv, cv, w, inside = corner_setup(p, dims, boundary)
    vals, valid, idx = {}, {}, {}
    for (sx, sy, sz) in CORNERS:
        ix = np.stack([(ci if sx else fi)[..., 0], (ci if sy else fi)[..., 1], (ci if sz else fi)[..., 2]], -1)
        va = (cv if sx else fv)[..., 0] & (cv if sy else fv)[..., 1] & (cv if sz else fv)[..., 2]
        vals[(sx, sy, sz)] = _fetch(grid, ix, va)
        valid[(sx, sy, sz)] = va
        idx[(sx, sy, sz)] = ix
    return vals, valid, idx, w, inside


def trilinear_from_corners(vals, w):
    """Lerp order of read3DInterpolated: x within each (y,z) pair, then y, then z
    (sampling.hpp:389-430)."""
    wx, wy, wz = w[..., 0:1], w[..., 1:2], w[..., 2:3]
    v00 = lerp(vals[(0, 0, 0)], vals[(1, 0, 0)], wx)
    v01 = lerp(vals[(0, 1, 0)], vals[(1, 1, 0)], wx)
    v0 = lerp(v00, v01, wy)
    v10 = lerp(vals[(0, 0, 1)], vals[(1, 0, 1)], wx)
    v11 = lerp(vals[(0, 1, 1)], vals[(1, 1, 1)], wx)
    v1 = lerp(v10, v11, wy)
    return lerp(v0, v1, wz)


def read_linear(grid, p, boundary):
    """Trilinear read, cell centres at integer positions (sampling.hpp:371-465)."""
    vals, valid, idx, w, inside = corner_values(grid, p, boundary)
    out = trilinear_from_corners(vals, w)
    if boundary == BORDER:
        out = np.where(inside[..., None], out, np.zeros((), grid.dtype))
    return out


def nearest_index(p):
    """``ivec3(position + 0.5)``: conversion truncates toward zero
    (sampling.hpp:571, sampling_v2.hpp:127)."""
    return np.trunc(p + p.dtype.type(0.5)).astype(np.int64)


def read_nearest(grid, p, boundary):
    """Nearest read (sampling.hpp:569-584)."""
    dims = dims_xyz(grid)
    idx = nearest_index(p)
    if boundary == BORDER:
        valid = np.all((idx >= 0) & (idx < dims), axis=-1)
        return _fetch(grid, np.where(valid[..., None], idx, 0), valid)
    if boundary == CLAMP:
        idx = np.clip(idx, 0, dims - 1)
    else:
        idx = _wrap(idx, dims)
    return _fetch(grid, idx)


def read_extremum(grid, p, boundary, mode, return_arg=False):
    """MIN / MAX of the 8 trilinear corners (sampling.hpp:585-704).

    BORDER: 0 outside the domain; if any corner is out of range the running
    extremum starts at 0 instead of +-FLOAT_MAX, and only in-range corners are
    compared.  Corners are visited in the reference order (x fastest, then y,
    then z).  With ``return_arg`` also returns, per sample and channel, the
    index of the corner that produced the value (-1 when it is the initial
    value) -- the corner the exact adjoint routes the gradient to.
    """
    dt = grid.dtype
    vals, valid, idx, w, inside = corner_values(grid, p, boundary)
    shape = p.shape[:-1] + (grid.shape[-1],)
    big = dt.type(FLOAT_MAX) if mode == MIN else -dt.type(FLOAT_MAX)
    acc = np.full(shape, big, dtype=dt)
    if boundary == BORDER:
        any_invalid = ~np.all(np.stack([valid[c] for c in CORNERS], -1), axis=-1)
        acc = np.where(any_invalid[..., None], np.zeros((), dt), acc)
    arg = np.full(shape, -1, dtype=np.int64)
    for k, c in enumerate(CORNERS):
        v = vals[c]
        better = (v < acc) if mode == MIN else (v > acc)
        better &= valid[c][..., None]
        acc = np.where(better, v, acc)
        arg = np.where(better, k, arg)
    if boundary == BORDER:
        acc = np.where(inside[..., None], acc, np.zeros((), dt))
        arg = np.where(inside[..., None], arg, -1)
    if return_arg:
        return acc, arg, idx, valid
    return acc


def bspline2_weight(dist):
    """Quadratic B-spline weight (sampling.hpp:247-256)."""
    dist = np.asarray(dist, dtype=np.float64)
    w = np.where(dist < 0.5, 0.75 - dist * dist,
                 np.where(dist < 1.5, 0.5 * (1.5 - dist) ** 2, 0.0))
    return w


def quadratic_taps(p, dims, boundary):
    """27-tap quadratic B-spline stencil (sampling.hpp:268-366): per axis the
    indices (prev, centre, next) around ``floor(p+0.5)`` and their weights."""
    dt = p.dtype
    center = np.floor(p + dt.type(0.5)).astype(np.int64)
    idx = [center - 1, center, center + 1]
    wts = [bspline2_weight(np.abs(p.astype(np.float64) - i)).astype(dt) for i in idx]
    if boundary == CLAMP:
        idx = [np.clip(i, 0, dims - 1) for i in idx]
    elif boundary == WRAP:
        idx = [_wrap(i, dims) for i in idx]
    return idx, wts


def read_quadratic(grid, p, boundary):
    """Quadratic B-spline read; BORDER returns 0 everywhere (sampling.hpp:284-287)."""
    if boundary == BORDER:
        return np.zeros(p.shape[:-1] + (grid.shape[-1],), grid.dtype)
    dims = dims_xyz(grid)
    idx, wts = quadratic_taps(p, dims, boundary)
    out_z = []
    for kz in range(3):
        out_y = []
        for ky in range(3):
            acc = None
            for kx in range(3):
                ix = np.stack([idx[kx][..., 0], idx[ky][..., 1], idx[kz][..., 2]], -1)
                term = wts[kx][..., 0:1] * _fetch(grid, ix)
                acc = term if acc is None else acc + term
            out_y.append(acc)
        v = wts[0][..., 1:2] * out_y[0] + wts[1][..., 1:2] * out_y[1] + wts[2][..., 1:2] * out_y[2]
        out_z.append(v)
    return wts[0][..., 2:3] * out_z[0] + wts[1][..., 2:3] * out_z[1] + wts[2][..., 2:3] * out_z[2]


def read(grid, p, filter_mode, boundary):
    """Dispatch of ``_internal_fetch3D`` (sampling.hpp:956-977)."""
    if filter_mode == LINEAR:
        return read_linear(grid, p, boundary)
    if filter_mode == NEAREST:
        return read_nearest(grid, p, boundary)
    if filter_mode in (MIN, MAX):
        return read_extremum(grid, p, boundary, filter_mode)
    if filter_mode == QUADRATIC:
        return read_quadratic(grid, p, boundary)
    raise ValueError(filter_mode)


def data_gradient(grid, p, boundary):
    """Spatial derivative of the trilinear read w.r.t. xyz position
    (``read3DGrad``, sampling.hpp:470-565).  Returns (..., 3, C)."""
    vals, valid, idx, w, inside = corner_values(grid, p, boundary)
    wx, wy, wz = w[..., 0:1], w[..., 1:2], w[..., 2:3]
    c = vals
    dx = lerp(lerp(c[(1, 0, 0)] - c[(0, 0, 0)], c[(1, 1, 0)] - c[(0, 1, 0)], wy),
              lerp(c[(1, 0, 1)] - c[(0, 0, 1)], c[(1, 1, 1)] - c[(0, 1, 1)], wy), wz)
    dy = lerp(lerp(c[(0, 1, 0)] - c[(0, 0, 0)], c[(1, 1, 0)] - c[(1, 0, 0)], wx),
              lerp(c[(0, 1, 1)] - c[(0, 0, 1)], c[(1, 1, 1)] - c[(1, 0, 1)], wx), wz)
    dz = lerp(lerp(c[(0, 0, 1)] - c[(0, 0, 0)], c[(1, 0, 1)] - c[(1, 0, 0)], wx),
              lerp(c[(0, 1, 1)] - c[(0, 1, 0)], c[(1, 1, 1)] - c[(1, 1, 0)], wx), wy)
    g = np.stack([dx, dy, dz], axis=-2)
    if boundary == BORDER:
        g = np.where(inside[..., None, None], g, np.zeros((), grid.dtype))
    return g


def trilinear_weights(w):
    """Per-corner weights (fw/cw products) in CORNERS order (resample_grid.cu.cc:1083-1129)."""
    cw = w
    fw = 1 - w
    out = []
    for (sx, sy, sz) in CORNERS:
        out.append((cw if sx else fw)[..., 0] * (cw if sy else fw)[..., 1] * (cw if sz else fw)[..., 2])
    return out


def scatter_add(target, idx, values, valid=None):
    """target[z,y,x,:] += values for integer xyz indices (unbuffered, duplicates add)."""
    if valid is not None:
        idx = idx[valid]
        values = values[valid]
    else:
        idx = idx.reshape(-1, 3)
        values = values.reshape(-1, values.shape[-1])
    np.add.at(target, (idx[..., 2], idx[..., 1], idx[..., 0]), values)


# ---------------------------------------------------------------- mip pyramid

def mip_level_down(grid):
    """One 2x2x2 box-filter level (``kGenerateMip3D``, resample_grid.cu.cc:58-84):
    pairs are averaged along z first, then y, then x; odd trailing layers are dropped."""
    d, h, w = (s // 2 for s in grid.shape[:3])
    g = grid[:2 * d, :2 * h, :2 * w]
    h5 = g.dtype.type(0.5)
    s = (g[0::2] + g[1::2]) * h5
    s = (s[:, 0::2] + s[:, 1::2]) * h5
    s = (s[:, :, 0::2] + s[:, :, 1::2]) * h5
    return s


def mip_pyramid(grid, levels):
    out = [grid]
    for _ in range(levels):
        out.append(mip_level_down(out[-1]))
    return out


def sample_mip(mips, pos4, cco, filter_mode, boundary, mip_mode, mip_bias, max_level):
    """``sample3D`` with mipmapping (sampling.hpp:991-1010).  ``pos4`` holds xyz and
    the level of detail in w; level m reads ``dims>>m`` at ``pos/2^m - cco``."""
    dt = mips[0].dtype
    xyz = pos4[..., :3]
    if mip_mode == "NONE":
        return read(mips[0], xyz - dt.type(cco), filter_mode, boundary)
    lod = np.clip(pos4[..., 3] + dt.type(mip_bias), 0, dt.type(max_level))

    def level_read(level):
        out = np.zeros(xyz.shape[:-1] + (mips[0].shape[-1],), dt)
        for m in np.unique(level):
            sel = level == m
            scale = dt.type(1 << int(m))
            out[sel] = read(mips[int(m)], xyz[sel] / scale - dt.type(cco), filter_mode, boundary)
        return out

    if mip_mode == "NEAREST":
        lf = np.minimum((lod + dt.type(0.5)).astype(np.int64), max_level)
        return level_read(lf)
    lf = np.minimum(lod.astype(np.int64), max_level)
    lc = np.minimum(np.ceil(lod).astype(np.int64), max_level)
    data = level_read(lf)
    hi = level_read(lc)
    t = (lod - np.floor(lod))[..., None]
    return np.where((lc > lf)[..., None], lerp(data, hi, t), data)


# ------------------------------------------------------------------- blending

BLEND_MODES = ("BEER_LAMBERT", "ALPHA", "ALPHA_ADDITIVE", "ADDITIVE")


def blend(acc, cell, mode):
    """One front-to-back blend step (blending.hpp:9-243).  The last channel is the
    density / alpha; with one channel every mode is additive (blending.hpp:9-19)."""
    if cell.shape[-1] == 1 or mode == "ADDITIVE":
        return acc + cell
    l_acc, a_acc = acc[..., :-1], acc[..., -1:]
    l, a = cell[..., :-1], cell[..., -1:]
    one = acc.dtype.type(1)
    if mode == "BEER_LAMBERT":
        d = np.maximum(a_acc + a, 0)
        t = np.exp(-d)
        return np.concatenate([l_acc + t * l, d], -1)
    if mode == "ALPHA":
        t = one - a_acc
        return np.concatenate([l_acc + t * l, a_acc + t * a], -1)
    if mode == "ALPHA_ADDITIVE":
        t = one - a
        return np.concatenate([l_acc + t * l, a_acc + a], -1)
    raise ValueError(mode)


def blend_gradients_reference(grads_out, cell, cell_out, mode):
    """The reference's back-to-front ``blendGradients`` (blending.hpp:40-54,64-78,
    124-139,160-175,184-199,208-223).  Returns (d_cell, new_grads_out, new_cell_out).
    The accumulator state is rebuilt by subtracting / dividing out the cell, as the
    reference does (not an exact inverse of the forward)."""
    if cell.shape[-1] == 1 or mode == "ADDITIVE":
        return grads_out, grads_out, cell_out
    one = cell.dtype.type(1)
    gl, gd = grads_out[..., :-1], grads_out[..., -1:]
    l, a = cell[..., :-1], cell[..., -1:]
    ol, oa = cell_out[..., :-1], cell_out[..., -1:]
    sum_lg = np.sum(l * gl, axis=-1, keepdims=True)
    if mode == "BEER_LAMBERT":
        e = np.exp(-oa)
        oa_new = np.maximum(oa - a, 0)
        d_dacc = gd - e * sum_lg
        d_cell = np.concatenate([e * gl, d_dacc], -1)
        new_g = np.concatenate([gl, d_dacc], -1)
        return d_cell, new_g, np.concatenate([ol, oa_new], -1)
    if mode == "ALPHA":
        oa_new = (one - oa) / (one - a)
        t = one - oa_new
        d_dacc = (one - a) * gd - sum_lg
        d_cell = np.concatenate([t * gl, t * gd], -1)
        new_g = np.concatenate([gl, d_dacc], -1)
        return d_cell, new_g, np.concatenate([ol, oa_new], -1)
    if mode == "ALPHA_ADDITIVE":
        oa_new = oa - a
        t = one - a
        d_cell = np.concatenate([t * gl, gd - sum_lg], -1)
        new_g = np.concatenate([gl, gd], -1)
        return d_cell, new_g, np.concatenate([ol, oa_new], -1)
    raise ValueError(mode)


def blend_sequence_exact_grad(cells, grad_out, mode):
    """Exact adjoint of a front-to-back blend over ``cells`` (n, ..., C) for an
    output gradient ``grad_out`` (..., C).  Accumulator states are recomputed
    forward, not rebuilt by subtraction.  max(., 0) in Beer-Lambert is
    differentiated as 1 where its argument is >= 0."""
    n = cells.shape[0]
    dt = cells.dtype
    C = cells.shape[-1]
    if C == 1 or mode == "ADDITIVE":
        return np.broadcast_to(grad_out, cells.shape).copy()
    accs = []
    acc = np.zeros_like(cells[0])
    for i in range(n):
        accs.append(acc)
        acc = blend(acc, cells[i], mode)
    one = dt.type(1)
    g = grad_out.copy()  # gradient w.r.t. the accumulator after cell i
    d_cells = np.zeros_like(cells)
    for i in range(n - 1, -1, -1):
        prev = accs[i]
        cell = cells[i]
        gl, ga = g[..., :-1], g[..., -1:]
        l, a = cell[..., :-1], cell[..., -1:]
        pa = prev[..., -1:]
        if mode == "BEER_LAMBERT":
            x = pa + a
            m = (x >= 0).astype(dt)
            d = np.maximum(x, 0)
            t = np.exp(-d)
            # L_new = L + t*l ; d_new = max(pa+a,0)
            dd = ga - t * np.sum(l * gl, -1, keepdims=True)   # total grad w.r.t. d_new
            d_cells[i] = np.concatenate([t * gl, m * dd], -1)
            g = np.concatenate([gl, m * dd], -1)
        elif mode == "ALPHA":
            t = one - pa
            # L_new = L + (1-pa) l ; a_new = pa + (1-pa) a
            d_cells[i] = np.concatenate([t * gl, t * ga], -1)
            g_pa = -np.sum(l * gl, -1, keepdims=True) + ga * (one - a)
            g = np.concatenate([gl, g_pa], -1)
        elif mode == "ALPHA_ADDITIVE":
            t = one - a
            d_cells[i] = np.concatenate([t * gl, ga - np.sum(l * gl, -1, keepdims=True)], -1)
            g = np.concatenate([gl, ga], -1)
        else:
            raise ValueError(mode)
    return d_cells


# ----------------------------------------------------------------- transforms

def mat_from_colmajor(arr16):
    """The reference reads 16 floats as a column-major 4x4 (transformations.hpp:42-47);
    return the corresponding (row, col) matrix."""
    return np.asarray(arr16, dtype=np.float64).reshape(4, 4).T


class CameraMatrices:
    """Per (batch, camera) transform set of ``setTransformations``
    (transformations.hpp:48-68): model, view, projection, model-view and inverses."""

    def __init__(self, M16, V16, P16, frustum):
        self.M = mat_from_colmajor(M16) if M16 is not None else np.eye(4)
        self.V = mat_from_colmajor(V16) if V16 is not None else np.eye(4)
        self.P = mat_from_colmajor(P16)
        self.MV = self.V @ self.M
        self.MV_inv = np.linalg.inv(self.MV)
        self.P_inv = np.linalg.inv(self.P)
        f = np.asarray(frustum, dtype=np.float64)
        self.near, self.far = f[0], f[1]


def _apply(m, v4):
    return np.einsum("ij,...j->...i", m, v4)


def idx_to_ndc(idx, dims):
    """IDXtoNDC (transformations.hpp:124-127)."""
    dims_inv = 1.0 / np.asarray(dims, dtype=np.float64)
    xyz = (idx * dims_inv) * 2.0 - 1.0
    return np.concatenate([xyz, np.ones(xyz.shape[:-1] + (1,))], -1)


def ndc_to_os(ndc, cam):
    """NDCtoVS then VStoOS (transformations.hpp:129-135)."""
    vs = _apply(cam.P_inv, ndc)
    vs = vs / vs[..., 3:4]
    return _apply(cam.MV_inv, vs)


def idx_to_os(idx, dims, cam):
    """IDXtoOS (transformations.hpp:136-138)."""
    return ndc_to_os(idx_to_ndc(idx, dims), cam)[..., :3]


def idx_to_os_lindepth(idx, dims, cam):
    """IDXtoOSlinearDepth (transformations.hpp:139-149): depth index maps linearly to
    view-space distance between near and far."""
    ndc = idx_to_ndc(idx, dims)
    t = idx[..., 2] / float(dims[2])
    z = -(cam.near + t * (cam.far - cam.near))
    ndc[..., 2] = -cam.P[2, 2] - cam.P[2, 3] / z
    return ndc_to_os(ndc, cam)[..., :3]


def os_to_idx(pos, dims, cam):
    """OStoIDX (transformations.hpp:106-109)."""
    p4 = np.concatenate([pos, np.ones(pos.shape[:-1] + (1,))], -1)
    ndc = _apply(cam.P, _apply(cam.MV, p4))
    ndc = ndc / ndc[..., 3:4]
    return (ndc[..., :3] * 0.5 + 0.5) * np.asarray(dims, dtype=np.float64), ndc


def os_to_idx_lindepth(pos, dims, cam):
    """OStoIDXlinearDepth (transformations.hpp:110-121)."""
    idx, ndc = os_to_idx(pos, dims, cam)
    z = -cam.P[2, 3] / (ndc[..., 2] + cam.P[2, 2])
    t = -(z + cam.near) / (cam.far - cam.near)
    idx[..., 2] = t * dims[2]
    return idx


def transform_positions(coordinate_mode, out_dims, in_dims, cam, idx):
    """``samplePos3D<CM,false>`` (sampling.hpp:154-228) for cell-centre index
    coordinates ``idx`` (already +0.5)."""
    if coordinate_mode == "TRANSFORM":
        return idx_to_os(idx, out_dims, cam)
    if coordinate_mode == "TRANSFORM_LINDEPTH":
        return idx_to_os_lindepth(idx, out_dims, cam)
    if coordinate_mode == "TRANSFORM_REVERSE":
        return os_to_idx(idx, in_dims, cam)[0]
    if coordinate_mode == "TRANSFORM_LINDEPTH_REVERSE":
        return os_to_idx_lindepth(idx, in_dims, cam)
    raise ValueError(coordinate_mode)


def lod_of_positions(coordinate_mode, out_dims, in_dims, cam, idx):
    """Level of detail of ``samplePos3D<CM,true>`` (sampling.hpp:159-228): log2 of the
    largest footprint of a one-cell step of the output grid, clamped at 0."""
    p0 = transform_positions(coordinate_mode, out_dims, in_dims, cam, idx)
    ds = []
    for a in range(3):
        e = np.zeros(3)
        e[a] = 1.0
        ds.append(p0 - transform_positions(coordinate_mode, out_dims, in_dims, cam, idx + e))
    dx, dy, dz = ds
    if coordinate_mode in ("TRANSFORM_REVERSE", "TRANSFORM_LINDEPTH_REVERSE"):
        px, py, pz = (np.linalg.norm(v, axis=-1) for v in (dx, dy, dz))
    else:
        px = np.linalg.norm(np.stack([dx[..., 0], dy[..., 0], dz[..., 0]], -1), axis=-1)
        py = np.linalg.norm(np.stack([dx[..., 1], dy[..., 1], dz[..., 1]], -1), axis=-1)
        pz = np.linalg.norm(np.stack([dx[..., 2], dy[..., 2], dz[..., 2]], -1), axis=-1)
    d = np.maximum(px, np.maximum(py, pz))
    with np.errstate(divide="ignore"):
        lod = np.maximum(0.0, np.log2(d))
    return p0, lod


def calc_lod(coordinate_mode, out_dims, in_dims, cam, idx):
    """``calcLoD<CM>`` (sampling.hpp:74-148), used by the LoD lookup op: central
    differences over +-1 output cell, footprint per axis taken across the three
    difference vectors, ``max(0, log2(max footprint))``."""
    ds = []
    for a in range(3):
        e = np.zeros(3)
        e[a] = 1.0
        ds.append((transform_positions(coordinate_mode, out_dims, in_dims, cam, idx - e)
                   - transform_positions(coordinate_mode, out_dims, in_dims, cam, idx + e)) * 0.5)
    dx, dy, dz = ds
    px = np.linalg.norm(np.stack([dx[..., 0], dy[..., 0], dz[..., 0]], -1), axis=-1)
    py = np.linalg.norm(np.stack([dx[..., 1], dy[..., 1], dz[..., 1]], -1), axis=-1)
    pz = np.linalg.norm(np.stack([dx[..., 2], dy[..., 2], dz[..., 2]], -1), axis=-1)
    d = np.maximum(px, np.maximum(py, pz))
    with np.errstate(divide="ignore"):
        return np.maximum(0.0, np.log2(d))
