"""Semi-Lagrangian / MacCormack advection by a MAC-staggered velocity.

``warp`` is the fused replacement of ``VelocityGrid.warp``
(phitest/render/data_structures.py:1690-1737) -- which the reference composes
from four ``SampleGridLut`` calls and TensorFlow elementwise ops -- and is
differentiable w.r.t. the advected grid and all three face grids.
"""
import ctypes

import torch

from . import _lib as L
from .ops import _code, _cuda, _ptr, _stream, _workspace, compute_dtype, get_deterministic, get_gradient_mode


def _spatial(t, name):
    """Accept (D,H,W,C), (1,D,H,W,C), (D,H,W) or (1,D,H,W,1) layouts."""
    t = _cuda(t, name)
    if t.dim() == 5:
        if t.shape[0] != 1:
            raise ValueError("%s: batch must be 1" % name)
        t = t[0]
    return t.contiguous()


def _faces(t, name):
    t = _spatial(t, name)
    if t.dim() == 4:
        if t.shape[-1] != 1:
            raise ValueError("%s: a face grid has one channel" % name)
        t = t[..., 0]
    return t.contiguous()


def _args(data, vx, vy, vz, out, fwd, dt, order, clamp, boundary, mask=None, extrema=None, lookup=None):
    a = L.AdvectArgs()
    a.dtype = _code(data)
    D, H, W, C = data.shape
    a.grid_dhw = L.I64x3(D, H, W)
    a.channels = C
    a.data, a.vel_x, a.vel_y, a.vel_z = _ptr(data), _ptr(vx), _ptr(vy), _ptr(vz)
    a.dt = float(dt)
    a.order = int(order)
    a.clamp = L.CLAMP[clamp.upper()]
    a.boundary = L.BOUNDARY[boundary]
    a.output, a.fwd_field = _ptr(out), _ptr(fwd)
    a.mask = _ptr(mask)
    a.extrema = _ptr(extrema)
    a.lookup = _ptr(lookup)
    if vx.dtype != data.dtype:
        a.velocity_dtype = _code(vx)  # FP16 faces with BF16 data
    return a


def _face_dtype(data, v):
    """The faces' storage: the data's, except FP16 faces kept with BF16 data."""
    return v.dtype if (data.dtype == torch.bfloat16 and v.dtype == torch.float16) else data.dtype


def _check_faces(data, vx, vy, vz):
    D, H, W = data.shape[:3]
    if tuple(vx.shape) != (D, H, W + 1) or tuple(vy.shape) != (D, H + 1, W) or tuple(vz.shape) != (D + 1, H, W):
        raise ValueError("shapes of components do not fit: data %s, x %s, y %s, z %s"
                         % (tuple(data.shape), tuple(vx.shape), tuple(vy.shape), tuple(vz.shape)))


def warp_forward(data, vx, vy, vz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP", keep_mask=False,
                 lookup=None):
    """Forward only; returns (output, fwd_field, mask) with fwd_field and the
    MC_SMOOTH revert mask (when ``keep_mask``) kept for the backward.
    ``lookup``: optional (D, H, W, 3) compute-type buffer where forward 1 leaves
    the lookup (centred velocity times -dt) for forward 2 and the backward."""
    out = torch.empty_like(data)
    fwd = torch.empty(data.shape, dtype=compute_dtype(data), device=data.device) if order == 2 else None
    smooth = order == 2 and clamp.upper() == "MC_SMOOTH"
    mask = torch.empty(data.shape, dtype=torch.uint8, device=data.device) if keep_mask and smooth else None
    # the forward trace's corner extrema, passed from forward 1 to forward 2
    ext = torch.empty(data.shape[:3] + (2 * data.shape[3],), dtype=compute_dtype(data),
                      device=data.device) if smooth else None
    L.call("ngt_advect_maccormack_fwd",
           ctypes.byref(_args(data, vx, vy, vz, out, fwd, dt, order, clamp, boundary, mask, ext, lookup)), _stream())
    return out, fwd, mask


def warp_backward(data, vx, vy, vz, fwd, grad, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP",
                  grad_mode=None, velocity_grad=True, deterministic=None, mask=None, lookup=None):
    """``lookup``: the buffer the forward stored its lookup in, or None."""
    cd = compute_dtype(data)
    g = L.AdvectGradArgs()
    g.fwd = _args(data, vx, vy, vz, None, fwd, dt, order, clamp, boundary, mask, lookup=lookup)
    gd = torch.empty(data.shape, dtype=cd, device=data.device)
    gx = torch.empty(vx.shape, dtype=cd, device=data.device) if velocity_grad else None
    gy = torch.empty(vy.shape, dtype=cd, device=data.device) if velocity_grad else None
    gz = torch.empty(vz.shape, dtype=cd, device=data.device) if velocity_grad else None
    keep = grad.to(cd).contiguous()
    g.output_grad, g.data_grad = _ptr(keep), _ptr(gd)
    g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = _ptr(gx), _ptr(gy), _ptr(gz)
    g.grad_mode = L.GRAD[grad_mode or get_gradient_mode()]
    g.deterministic = int(get_deterministic() if deterministic is None else deterministic)
    ws = _workspace(L.load().ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g)), data.device)
    g.workspace, g.workspace_bytes = _ptr(ws), ws.numel()
    L.call("ngt_advect_maccormack_bwd", ctypes.byref(g), _stream())
    return gd, gx, gy, gz


class _Warp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, vx, vy, vz, dt, order, clamp, boundary):
        # MacCormack: forward 1 stores the lookup for forward 2 and the backward
        lut = torch.empty(data.shape[:3] + (3,), dtype=compute_dtype(data), device=data.device) \
            if order == 2 else None
        out, fwd, mask = warp_forward(data, vx, vy, vz, dt, order, clamp, boundary, keep_mask=True, lookup=lut)
        ctx.save_for_backward(data, vx, vy, vz, fwd, mask, lut)
        ctx.cfg = (dt, order, clamp, boundary, get_gradient_mode(), get_deterministic())
        return out

    @staticmethod
    def backward(ctx, grad):
        data, vx, vy, vz, fwd, mask, lut = ctx.saved_tensors
        dt, order, clamp, boundary, mode, det = ctx.cfg
        gd, gx, gy, gz = warp_backward(data, vx, vy, vz, fwd, grad.contiguous(), dt, order, clamp, boundary, mode,
                                       velocity_grad=any(ctx.needs_input_grad[1:4]), deterministic=det, mask=mask,
                                       lookup=lut)
        return gd, gx, gy, gz, None, None, None, None


def warp(data, vel_x, vel_y, vel_z, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """Advect ``data`` (D,H,W,C) -- or (1,D,H,W,C) -- by the MAC velocity
    (x: D,H,W+1; y: D,H+1,W; z: D+1,H,W).  order 1 is semi-Lagrangian, order 2
    MacCormack; clamp 'MC_SMOOTH' reverts to the semi-Lagrangian value where the
    correction leaves the range of the forward lookup's corners, 'NEGATIVE'
    clips at 0, 'NONE' does neither.  The faces are used in the data's storage
    type, except that FP16 faces are kept as they are with BF16 data."""
    lead = data.dim() == 5
    d = _spatial(data, "data")
    vx, vy, vz = _faces(vel_x, "vel_x"), _faces(vel_y, "vel_y"), _faces(vel_z, "vel_z")
    _check_faces(d, vx, vy, vz)
    if clamp.upper() == "MC":
        raise NotImplementedError("MIM and MAX warp sampling have wrong gradients.")
    fd = _face_dtype(d, vx)
    out = _Warp.apply(d, vx.to(fd), vy.to(fd), vz.to(fd), float(dt), int(order), clamp.upper(), boundary)
    return out[None] if lead else out


# --------------------------------------------------------- velocity self-advection
def _vel_args(vx, vy, vz, outs, fwds, dt, order, clamp, boundary, scratch=None):
    """``scratch``: per component (lookup, mask, extrema) tensors or Nones."""
    a = L.AdvectVelocityArgs()
    a.dtype = _code(vx)
    D, H, W1 = vx.shape
    a.grid_dhw = L.I64x3(D, H, W1 - 1)
    a.vel_x, a.vel_y, a.vel_z = _ptr(vx), _ptr(vy), _ptr(vz)
    a.dt, a.order, a.clamp, a.boundary = float(dt), int(order), L.CLAMP[clamp], L.BOUNDARY[boundary]
    a.out_x, a.out_y, a.out_z = (_ptr(t) for t in outs)
    a.fwd_x, a.fwd_y, a.fwd_z = (_ptr(t) for t in fwds)
    if scratch is not None:
        for c, (lut, mask, ext) in enumerate(scratch):
            a.lookup[c], a.mask[c], a.extrema[c] = _ptr(lut), _ptr(mask), _ptr(ext)
    return a


def _vel_scratch(comps, order, clamp):
    """Per face component: the stored lookup (3 values per face), and for
    MacCormack with MC_SMOOTH the revert mask and the corner extrema."""
    cd = compute_dtype(comps[0])
    smooth = order == 2 and clamp.upper() == "MC_SMOOTH"
    out = []
    for t in comps:
        lut = torch.empty(tuple(t.shape) + (3,), dtype=cd, device=t.device)
        mask = torch.empty(t.shape, dtype=torch.uint8, device=t.device) if smooth else None
        ext = torch.empty(tuple(t.shape) + (2,), dtype=cd, device=t.device) if smooth else None
        out.append((lut, mask, ext))
    return out


class _WarpVelocity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vx, vy, vz, dt, order, clamp, boundary):
        cd = compute_dtype(vx)
        outs = [torch.empty_like(t) for t in (vx, vy, vz)]
        fwds = [torch.empty(t.shape, dtype=cd, device=t.device) if order == 2 else None for t in (vx, vy, vz)]
        scratch = _vel_scratch((vx, vy, vz), order, clamp)
        L.call("ngt_advect_velocity_fwd",
               ctypes.byref(_vel_args(vx, vy, vz, outs, fwds, dt, order, clamp, boundary, scratch)), _stream())
        ctx.save_for_backward(vx, vy, vz, *[f for f in fwds if f is not None])
        ctx.scratch = scratch
        ctx.cfg = (dt, order, clamp, boundary, get_gradient_mode(), get_deterministic())
        return tuple(outs)

    @staticmethod
    def backward(ctx, gx, gy, gz):
        saved = ctx.saved_tensors
        vx, vy, vz = saved[:3]
        fwds = list(saved[3:]) if len(saved) > 3 else [None, None, None]
        dt, order, clamp, boundary, mode, det = ctx.cfg
        cd = compute_dtype(vx)
        gs = [(g if g is not None else torch.zeros(t.shape, device=t.device)).to(cd).contiguous()
              for g, t in zip((gx, gy, gz), (vx, vy, vz))]
        outs = [torch.empty(t.shape, dtype=cd, device=t.device) for t in (vx, vy, vz)]
        g = L.AdvectVelocityGradArgs()
        g.fwd = _vel_args(vx, vy, vz, (None, None, None), fwds, dt, order, clamp, boundary, ctx.scratch)
        g.grad_x, g.grad_y, g.grad_z = (_ptr(t) for t in gs)
        g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (_ptr(t) for t in outs)
        g.grad_mode = L.GRAD[mode]
        g.deterministic = int(bool(det) and mode == "exact")
        ws = _workspace(L.load().ngt_advect_velocity_bwd_workspace_bytes(ctypes.byref(g)), vx.device)
        g.workspace, g.workspace_bytes = _ptr(ws), ws.numel()
        L.call("ngt_advect_velocity_bwd", ctypes.byref(g), _stream())
        ctx.scratch = None
        return outs[0], outs[1], outs[2], None, None, None, None


def warp_velocity(vel_x, vel_y, vel_z, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP"):
    """Self-advection of a MAC velocity (``VelocityGrid.warped``): returns the
    three warped face grids; differentiable w.r.t. all three inputs."""
    lead = vel_x.dim() == 5
    vx, vy, vz = _faces(vel_x, "vel_x"), _faces(vel_y, "vel_y"), _faces(vel_z, "vel_z")
    D, H, W1 = vx.shape
    if tuple(vy.shape) != (D, H + 1, W1 - 1) or tuple(vz.shape) != (D + 1, H, W1 - 1):
        raise ValueError("shapes of components do not fit: x %s, y %s, z %s"
                         % (tuple(vx.shape), tuple(vy.shape), tuple(vz.shape)))
    if clamp.upper() == "MC":
        raise NotImplementedError("MIM and MAX warp sampling have wrong gradients.")
    out = _WarpVelocity.apply(vx, vy.to(vx.dtype), vz.to(vx.dtype), float(dt), int(order), clamp.upper(), boundary)
    return tuple(o[None, ..., None] for o in out) if lead else out
