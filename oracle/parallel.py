"""The oracle at the benchmark sizes, split over host processes.

Test and baseline infrastructure only (like the rest of ``oracle/``): the
parity tests at the benchmark configurations and the CPU legs of ``bench.py``
use it; the product never does.

One process of the NumPy oracle needs about a minute for one differentiated
step at 128^3 x 5 views of 256 x 256 x 128.  Here the work is split the way
the step's data allow, over a pool of spawned worker processes:

* the MacCormack warp and its adjoint (``advect.maccormack`` /
  ``maccormack_grad``, restating data_structures.py:1690-1737) run as slabs
  of z planes with a halo of planes on either side.  A trace moves at most
  ``R = ceil(max|lookup|) + 1`` planes (trilinear footprint included) and the
  back-trace of MacCormack reads the forward field, so the planes of a slab
  whose traces stay inside the halo (2 R + 1 planes) are those of the whole-
  grid warp; positions are formed with global plane indices (``z0``), so the
  slab result is the whole-grid result, and the adjoint of the slab's own
  output planes is added into the whole-grid gradients;
* the render (``ops.raymarch_grid_transform`` and its exact gradient,
  restating raymarch_grid.cu.cc:202-252 and 482-521) runs as bands of image
  rows of every camera; each ray is independent in the forward, and the exact
  input gradient is a sum over rays, so the bands' gradients add up to the
  whole image's.

Workers are started with ``spawn`` (the callers may already hold a CUDA
context) and receive their inputs by pickling.
"""
import multiprocessing as mp
import os

import numpy as np

from . import advect, ops

BAND_ROWS = 8  # image rows per render band


def make_pool(processes=None):
    """A pool of ``processes`` (default: every host CPU) spawned workers."""
    n = int(processes or os.cpu_count() or 1)
    return mp.get_context("spawn").Pool(n), n


# ---------------------------------------------------------------- advection
def trace_reach(lut):
    """Planes a trace (plus its trilinear footprint) can move: ceil(max|lut|) + 1."""
    m = float(np.abs(lut).max()) if lut.size else 0.0
    return int(np.ceil(m)) + 1


def slabs(depth, parts, halo):
    """(lo, hi, z_lo, z_hi) per slab: output planes lo..hi-1, input planes
    z_lo..z_hi-1 with ``halo`` planes either side (cut at the grid).  A slab
    whose halo would start within ``halo`` planes of the bottom starts at 0,
    so every slab origin is 0 or at least ``halo`` (which keeps the subtraction
    of the origin from a global position exact, see advect._positions)."""
    parts = max(1, min(int(parts), depth))
    edges = np.linspace(0, depth, parts + 1).round().astype(int)
    out = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        if hi <= lo:
            continue
        z_lo = lo - halo
        z_lo = z_lo if z_lo >= halo else 0
        out.append((int(lo), int(hi), int(z_lo), int(min(depth, hi + halo))))
    return out


def _advect_fwd_task(a):
    data, lut, z0, lo, hi, order, clamp, boundary = a
    out = advect.maccormack(data, lut, order, clamp, boundary, z0=z0)
    return lo, hi, out[lo - z0:hi - z0]


def _advect_bwd_task(a):
    data, lut, g, z0, lo, hi, order, clamp, boundary, grad_mode = a
    gs = np.zeros_like(data)
    gs[lo - z0:hi - z0] = g
    gd, gl = advect.maccormack_grad(data, lut, gs, order, clamp, boundary, grad_mode, z0=z0)
    return z0, gd, gl


def _halo(lut, order):
    r = trace_reach(lut)
    return (2 * r + 1) if order == 2 else r + 1


def advect_fwd(pool, nproc, data, lut, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """advect.maccormack of ``data`` (D,H,W,C) by the relative ``lut`` (D,H,W,3)."""
    D = data.shape[0]
    tasks = [(data[z_lo:z_hi], lut[z_lo:z_hi], z_lo, lo, hi, order, clamp, boundary)
             for lo, hi, z_lo, z_hi in slabs(D, nproc, _halo(lut, order))]
    out = np.empty_like(data)
    for lo, hi, part in pool.map(_advect_fwd_task, tasks):
        out[lo:hi] = part
    return out


def advect_bwd(pool, nproc, data, lut, grad_out, order=2, clamp="MC_SMOOTH", boundary="CLAMP", grad_mode="exact"):
    """advect.maccormack_grad: (d data, d lut).  With ``grad_mode='reference'``
    the count normalisation of each slab only sees that slab's samples, so only
    the exact mode is split; the reference mode runs in one process."""
    if grad_mode != "exact":
        return advect.maccormack_grad(data, lut, grad_out, order, clamp, boundary, grad_mode)
    D = data.shape[0]
    tasks = [(data[z_lo:z_hi], lut[z_lo:z_hi], grad_out[lo:hi], z_lo, lo, hi, order, clamp, boundary, grad_mode)
             for lo, hi, z_lo, z_hi in slabs(D, nproc, _halo(lut, order))]
    gd = np.zeros_like(data)
    gl = np.zeros_like(lut)
    for z0, a, b in pool.map(_advect_bwd_task, tasks):
        gd[z0:z0 + a.shape[0]] += a
        gl[z0:z0 + b.shape[0]] += b
    return gd, gl


def density_fwd(pool, nproc, rho, ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """advect.density_maccormack split over the pool."""
    lut = advect.centered_velocity(ux, uy, uz) * rho.dtype.type(-dt)
    return advect_fwd(pool, nproc, rho, lut, order, clamp, boundary)


def density_bwd(pool, nproc, rho, ux, uy, uz, grad_out, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """advect.density_maccormack_grad split over the pool: (d rho, d ux, d uy, d uz)."""
    lut = advect.centered_velocity(ux, uy, uz) * rho.dtype.type(-dt)
    g_rho, g_lut = advect_bwd(pool, nproc, rho, lut, grad_out, order, clamp, boundary)
    g_uc = g_lut * rho.dtype.type(-dt)
    gx, gy, gz = advect.centered_velocity_adjoint(g_uc, (ux.shape, uy.shape, uz.shape))
    return g_rho, gx, gy, gz


# ------------------------------------------------------------------- render
def _render_task(a):
    """Render bands of one-channel density ``rho`` as the [light*step, step]
    grid (emission ``scale``) with the image L2 on the light channel: the
    bands' images, their loss and the density gradient of their rays."""
    rho, scale, M, V, P, F, dhw, bands, targets, boundary, background = a
    x = rho[None] * scale
    loss = 0.0
    g_rho = np.zeros_like(rho)
    images = []
    for (v, y0, y1), tgt in zip(bands, targets):
        sl = slice(v, v + 1)
        img = ops.raymarch_grid_transform(x, M, V[sl], P[sl], F[sl], dhw, boundary=boundary, rows=(y0, y1))
        lit = img[..., :1]
        t = None
        if background is not None:
            t = np.exp(-img[..., 1:2])
            lit = lit + background[v][y0:y1][None, None] * t
        images.append((v, y0, y1, img))
        if tgt is None:
            continue
        diff = lit - tgt
        loss += 0.5 * float((diff.astype(np.float64) ** 2).sum())
        gd = np.zeros_like(diff) if t is None else -(background[v][y0:y1][None, None] * t) * diff
        gimg = np.concatenate([diff, gd], -1)
        gx = ops.raymarch_grid_transform_grad(x, img, gimg, M, V[sl], P[sl], F[sl], dhw, boundary=boundary,
                                              rows=(y0, y1))
        g_rho += (gx[0] * scale).sum(-1, keepdims=True)
    return images, loss, g_rho


def render_l2(pool, nproc, rho, depth_step, M, V, P, F, image_dhw, targets=None, boundary=ops.BORDER,
              light=1.0, background=None, band_rows=BAND_ROWS):
    """Render of the one-channel density ``rho`` (D,H,W,1) from every camera
    (emission [light*step, step]) and, with ``targets`` (1, V, H, W, 1), the
    image L2 loss on the light channel and its density gradient.  With
    ``background`` (V, H, W, 1) the light channel is composited over it as
    ``light + background * exp(-optical depth)`` before the loss.
    Returns (image (1, V, H, W, 2), loss, d rho)."""
    dt = rho.dtype
    s = dt.type(depth_step)
    scale = np.asarray([dt.type(light) * s, s], dt)
    M, V, P, F = (np.asarray(m, np.float32) for m in (M, V, P, F))
    V = V.reshape(-1, 16)
    P = P.reshape(-1, 16)
    F = F.reshape(-1, 6)
    nv = V.shape[0]
    D, H, W = (int(v) for v in image_dhw)
    bands = [(v, y0, min(H, y0 + band_rows)) for v in range(nv) for y0 in range(0, H, band_rows)]
    ntask = max(1, min(nproc, len(bands)))
    tasks = []
    bkg = None if background is None else np.asarray(background, dt).reshape(nv, H, W, 1)
    for k in range(ntask):
        mine = bands[k::ntask]
        tg = [None if targets is None else np.asarray(targets[0, v, y0:y1], dt)[None, None] for v, y0, y1 in mine]
        tasks.append((rho, scale, M, V, P, F, (D, H, W), mine, tg, boundary, bkg))
    image = np.zeros((1, nv, H, W, 2), dt)
    loss = 0.0
    g_rho = np.zeros_like(rho)
    for images, l, g in pool.map(_render_task, tasks):
        for v, y0, y1, img in images:
            image[0, v, y0:y1] = img[0, 0]
        loss += l
        g_rho += g
    return image, loss, g_rho


# --------------------------------------------------------------------- step
def render_advect_step(pool, nproc, rho, ux, uy, uz, M, V, P, F, targets, image_dhw, depth_step, dt=1.0,
                       order=2, clamp="MC_SMOOTH", advect_boundary="CLAMP", render_boundary=ops.BORDER,
                       light=1.0, background=None):
    """One differentiated reconstruction step (the composition of
    ``RenderAdvectStep``): MacCormack warp of rho by u, render of every camera,
    image L2 to ``targets``, backward to rho and the three face grids.
    Returns (image, loss, (d rho, d ux, d uy, d uz))."""
    lut = advect.centered_velocity(ux, uy, uz) * rho.dtype.type(-dt)
    rho2 = advect_fwd(pool, nproc, rho, lut, order, clamp, advect_boundary)
    image, loss, g_rho2 = render_l2(pool, nproc, rho2, depth_step, M, V, P, F, image_dhw, targets,
                                    render_boundary, light, background)
    g_rho, g_lut = advect_bwd(pool, nproc, rho, lut, g_rho2, order, clamp, advect_boundary)
    g_uc = g_lut * rho.dtype.type(-dt)
    gx, gy, gz = advect.centered_velocity_adjoint(g_uc, (ux.shape, uy.shape, uz.shape))
    return image, loss, (g_rho, gx, gy, gz)
