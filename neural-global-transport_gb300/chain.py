"""Differentiated multi-frame advect + render chain with checkpoint-and-recompute.

The sequence reconstruction (reconstruct_sequence.py / optimization.py: density
advected frame to frame by ``VelocityGrid.warp`` with an inflow added, every
frame rendered and compared to its target images) as one differentiable chain:

    rho_{t+1} = MacCormack(rho_t, u) + source          t = 0 .. T-1
    image_t   = raymarch(rho_{t+1} as [light*step, step])
    loss      = sum_t 0.5 * ||image_t.light - target_t||^2

with gradients with respect to rho_0 and the frame-constant MAC velocity u.

Memory: the forward keeps only every K-th density (checkpoints); the backward
walks the segments last to first, recomputes the segment's densities and
MacCormack fields from its checkpoint, then runs render forward, loss, render
backward and advection backward frame by frame in reverse.  Peak memory is
ceil(T/K) + K + 1 densities plus K forward fields, instead of 2T.  The
recomputation is bit-identical to the forward (the advection and render
forwards are deterministic), so the gradient does not depend on K beyond the
order of the backward's atomic additions.

Every launch goes through the C ABI with argument structs built once; the
whole chain (forward and backward) can be recorded as one CUDA graph.
"""
import ctypes

import torch

from . import _lib as L
from .ops import _code, _ptr, sample_cache_pays


class AdvectRenderChain:
    def __init__(self, rho0, ux, uy, uz, source, M, V, P, F, targets, image_dhw, frames, checkpoint_every=10,
                 dt=1.0, light=1.0, clamp="MC_SMOOTH", advect_boundary="CLAMP", render_boundary="BORDER"):
        dev = rho0.device
        self.lib = L.load()
        st = rho0.dtype
        cd = torch.float64 if st == torch.float64 else torch.float32
        self.T, self.K = int(frames), max(1, int(checkpoint_every))
        T, K = self.T, self.K
        self.nseg = (T + K - 1) // K
        D, H, W = rho0.shape[:3]
        self.dhw = (D, H, W)
        self.rho0 = rho0.contiguous()
        self.ux, self.uy, self.uz = ux.contiguous(), uy.contiguous(), uz.contiguous()
        self.source = source.to(device=dev, dtype=st).contiguous()
        self.M = torch.as_tensor(M, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.V = torch.as_tensor(V, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.P = torch.as_tensor(P, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.F = torch.as_tensor(F, dtype=torch.float32, device=dev).reshape(-1, 6).contiguous()
        nv = self.V.shape[0]
        dd, hh, ww = image_dhw
        self.targets = targets.to(device=dev, dtype=cd).reshape(T, 1, nv, hh, ww, 1).contiguous()
        depth_step = float(self.F[0, 1] - self.F[0, 0]) / dd
        self.pixels = nv * hh * ww

        # densities: checkpoints, the two chain buffers, the segment under differentiation
        self.ckpt = torch.empty((self.nseg, D, H, W, 1), dtype=st, device=dev)
        self.cur = torch.empty((2, D, H, W, 1), dtype=st, device=dev)
        self.seg = torch.empty((K + 1, D, H, W, 1), dtype=st, device=dev)
        self.seg_fwd = torch.empty((K, D, H, W, 1), dtype=cd, device=dev)
        self.chain_fwd = torch.empty((D, H, W, 1), dtype=cd, device=dev)
        self.image = torch.empty((1, nv, hh, ww, 2), dtype=cd, device=dev)
        self.g_image = torch.empty_like(self.image)
        self.loss = torch.zeros((1,), dtype=cd, device=dev)
        # gradients: w.r.t. the current frame's density (ping-pong), the render's part,
        # the velocity (total and one frame's)
        self.g_rho = torch.empty((2, D, H, W, 1), dtype=cd, device=dev)
        self.g_u = [torch.empty(u.shape, dtype=cd, device=dev) for u in (ux, uy, uz)]

        # MC_SMOOTH revert masks of the segment's frames (forward writes, backward reads)
        self.seg_mask = torch.empty((K, D, H, W, 1), dtype=torch.uint8, device=dev)
        # forward 1 -> forward 2 corner extrema of every advection (stream-ordered, one buffer)
        self.adv_ext = torch.empty((D, H, W, 2), dtype=cd, device=dev)
        # the lookup (centred velocity times -dt): the velocity is the same for every
        # frame, so one buffer serves every frame's forward 2 and backward
        self.adv_lut = torch.empty((D, H, W, 3), dtype=cd, device=dev)

        def advect_args(data, out, fwd, mask=None):
            a = L.AdvectArgs()
            a.dtype = _code(rho0)
            a.grid_dhw = L.I64x3(D, H, W)
            a.channels = 1
            a.data, a.vel_x, a.vel_y, a.vel_z = _ptr(data), _ptr(self.ux), _ptr(self.uy), _ptr(self.uz)
            a.dt, a.order, a.clamp, a.boundary = float(dt), 2, L.CLAMP[clamp], L.BOUNDARY[advect_boundary]
            a.output, a.fwd_field = _ptr(out), _ptr(fwd)
            a.mask = _ptr(mask)
            a.extrema = _ptr(self.adv_ext)
            a.lookup = _ptr(self.adv_lut)
            return a

        # chain forward: cur[t % 2] -> cur[(t + 1) % 2]
        self.adv_chain = [advect_args(self.cur[k], self.cur[1 - k], self.chain_fwd) for k in range(2)]
        # segment recompute: seg[j] -> seg[j + 1], fwd field seg_fwd[j]
        self.adv_seg = [advect_args(self.seg[j], self.seg[j + 1], self.seg_fwd[j], self.seg_mask[j])
                        for j in range(K)]
        # advection backward of segment frame j with output gradient g_rho[k] -> g_rho[1 - k]
        self.adv_bwd = {}
        ws_bytes = 0
        for j in range(K):
            for k in range(2):
                g = L.AdvectGradArgs()
                g.fwd = self.adv_seg[j]
                g.output_grad, g.data_grad = _ptr(self.g_rho[k]), _ptr(self.g_rho[1 - k])
                # the frame's velocity gradient is added to the chain's
                g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (_ptr(t) for t in self.g_u)
                g.accumulate = 1
                g.grad_mode = L.GRAD["exact"]
                ws_bytes = max(ws_bytes, int(self.lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(g))))
                self.adv_bwd[(j, k)] = g
        self.adv_ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        for g in self.adv_bwd.values():
            g.workspace, g.workspace_bytes = _ptr(self.adv_ws), ws_bytes

        # render of segment density j + 1
        def ray_args(rho):
            r = L.RaymarchArgs()
            r.dtype = _code(rho0)
            r.input_shape = L.I64x5(1, D, H, W, 1)
            r.output_dhw = L.I64x3(dd, hh, ww)
            r.input, r.output = _ptr(rho), _ptr(self.image)
            r.matrix_m, r.matrix_v, r.matrix_p, r.frustum = _ptr(self.M), _ptr(self.V), _ptr(self.P), _ptr(self.F)
            r.num_cameras = nv
            r.interpolation, r.boundary = L.INTERP["LINEAR"], L.BOUNDARY[render_boundary]
            r.blending_mode, r.keep_dims, r.separate_camera_batch = L.BLEND["BEER_LAMBERT"], 0, 1
            r.emission_channels = 2
            r.emission_scale[0], r.emission_scale[1] = light * depth_step, depth_step
            # the render backward reads its forward's samples back where that pays
            r.sample_cache = int(sample_cache_pays((D, H, W), 1, rho0.dtype, dev))
            return r

        self.ray = [ray_args(self.seg[j + 1]) for j in range(K)]
        # each frame's density in the quad gather layout, prepared once for the
        # frame's render forward and backward (one buffer, frames run in order)
        nq = int(self.lib.ngt_raymarch_quad_bytes(ctypes.byref(self.ray[0])))
        self.ray_quad = torch.empty(nq, dtype=torch.uint8, device=dev) if nq else None
        if nq:
            for r in self.ray:
                r.quad = _ptr(self.ray_quad)
        fws = max(int(self.lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))) for r in self.ray)
        self.ray_fws = torch.empty(fws, dtype=torch.uint8, device=dev)
        self.cameras = torch.empty(int(self.lib.ngt_raymarch_cameras_bytes(ctypes.byref(self.ray[0]))),
                                   dtype=torch.uint8, device=dev)
        self._call("ngt_raymarch_cameras", ctypes.byref(self.ray[0]), _ptr(self.cameras), self._stream())
        # the rays of the fixed camera, set up once in double precision
        self.rays = torch.empty(int(self.lib.ngt_raymarch_rays_bytes(ctypes.byref(self.ray[0]))), dtype=torch.uint8,
                                device=dev)
        self._call("ngt_raymarch_rays", ctypes.byref(self.ray[0]), _ptr(self.rays), self._stream())
        # render backward of segment slot j, its density gradient added to g_rho[k]
        self.ray_g = {}
        bws = 0
        for r in self.ray:
            r.workspace, r.workspace_bytes = _ptr(self.ray_fws), fws
            r.cameras = _ptr(self.cameras)
            r.rays = _ptr(self.rays)
        for j, r in enumerate(self.ray):
            for k in range(2):
                g = L.RaymarchGradArgs()
                g.fwd = r
                g.output, g.output_grad, g.input_grad = _ptr(self.image), _ptr(self.g_image), _ptr(self.g_rho[k])
                g.grad_mode = L.GRAD["exact"]
                g.accumulate = 1
                bws = max(bws, int(self.lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))))
                self.ray_g[(j, k)] = g
        self.ray_bws = torch.empty(bws, dtype=torch.uint8, device=dev)
        for g in self.ray_g.values():
            g.workspace, g.workspace_bytes = _ptr(self.ray_bws), bws
        self.graph = None

    # ------------------------------------------------------------------ helpers
    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _call(self, name, *args):
        L.call(name, *args)

    # ------------------------------------------------------------------ the chain
    def launch(self):
        """Enqueue forward (checkpoints) and backward on the current stream."""
        s = self._stream()
        T, K = self.T, self.K
        self.loss.zero_()
        # forward: every K-th density up to the last segment's start
        self.cur[0].copy_(self.rho0)
        last = (self.nseg - 1) * K
        for t in range(last + 1):
            k = t % 2
            if t % K == 0:
                self.ckpt[t // K].copy_(self.cur[k])
            if t < last:
                self._call("ngt_advect_maccormack_fwd", ctypes.byref(self.adv_chain[k]), s)
                self.cur[1 - k].add_(self.source)
        # backward: segments last to first; g_rho[k] holds d loss / d rho_{t+1}
        for g in self.g_u:
            g.zero_()
        k = 0
        self.g_rho[k].zero_()
        for seg in range(self.nseg - 1, -1, -1):
            s0 = seg * K
            s1 = min(s0 + K, T)
            self.seg[0].copy_(self.ckpt[seg])
            for j in range(s1 - s0):
                self._call("ngt_advect_maccormack_fwd", ctypes.byref(self.adv_seg[j]), s)
                self.seg[j + 1].add_(self.source)
            for j in range(s1 - s0 - 1, -1, -1):
                t = s0 + j
                # frame t's render, image loss and render backward in one launch: g_rho[k] += render grad
                if self.ray_quad is not None:
                    self._call("ngt_raymarch_quad", ctypes.byref(self.ray[j]), _ptr(self.ray_quad), s)
                self._call("ngt_raymarch_fwd_l2_bwd", ctypes.byref(self.ray_g[(j, k)]), None, _ptr(self.targets[t]), 1,
                           _ptr(self.loss), s)
                self.g_rho[1 - k].zero_()
                self._call("ngt_advect_maccormack_bwd", ctypes.byref(self.adv_bwd[(j, k)]), s)  # and g_u +=
                k = 1 - k
        self.result = k  # g_rho[k] = d loss / d rho_0

    def capture(self):
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.launch()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.launch()
        return self.graph

    def run(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self.loss

    def gradients(self):
        """(d loss / d rho_0, d loss / d u_x, u_y, u_z)."""
        return (self.g_rho[self.result],) + tuple(self.g_u)


def chain_targets(rho0, ux, uy, uz, source, M, V, P, F, image_dhw, frames, dt=1.0, light=1.0,
                  clamp="MC_SMOOTH", advect_boundary="CLAMP", render_boundary="BORDER"):
    """Target images of a chain: the light channel of every frame's render,
    (frames, views, H, W, 1), through the operator API."""
    from . import advect, ops
    F32 = torch.as_tensor(F, dtype=torch.float32).reshape(-1, 6)
    step = float(F32[0, 1] - F32[0, 0]) / image_dhw[0]
    out = []
    rho = rho0
    with torch.no_grad():
        for _ in range(frames):
            rho = advect.warp(rho, ux, uy, uz, dt=dt, order=2, clamp=clamp, boundary=advect_boundary) + source
            img = ops.raymarch_grid_transform(rho[None], M, V, P, F, image_dhw, boundary=render_boundary,
                                              emission_scale=(light * step, step))
            out.append(img[0, ..., :1])
    return torch.stack(out)
