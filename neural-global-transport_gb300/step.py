"""One differentiated reconstruction step on device-resident tensors.

The step of the density / velocity optimisation (optimization.py:1018-1046 and
1263-1281 around State.render_density / VelocityGrid.warp):

    rho' = MacCormack(rho, u)                        (warp, MC_SMOOTH, CLAMP)
    image_v = raymarch(rho' as [light*step, step])    (Beer-Lambert, BORDER)
    (optional) light_v += background_v * exp(-d_v)     (renderer.py:779, 804-806)
    loss = 0.5 * sum_v ||image_v.light - target_v||^2
    backward to rho and to the three MAC face grids

The ambient light grid ``rho*c*i`` (lighting.py:26-34) and the step
premultiply (renderer.py:533-548) are linear in rho, so the raymarch reads the
one-channel rho' and forms both blend channels in registers; its gradient comes
back as one channel.  All launches go through the C ABI with argument structs
built once; ``capture()`` records the whole step as one CUDA graph.
"""
import collections
import ctypes

import numpy as np
import torch

from . import _lib as L
from .ops import _code, _ptr, get_deterministic, sample_cache_pays


class RenderAdvectStep:
    # kernels of one f32 exact Beer-Lambert step: advect fwd 2, the quad layout of
    # the advected density with its extinction-sign check 1, the render's forward,
    # image loss and backward in one launch 1 (each ray marched forward and back;
    # the checkpointed adjoint where the sign check fails), the quad-gradient fold
    # 1, advect bwd 2
    KERNELS_PER_STEP = 7

    def __init__(self, rho, ux, uy, uz, M, V, P, F, targets, image_dhw, dt=1.0, light=1.0, order=2,
                 clamp="MC_SMOOTH", advect_boundary="CLAMP", render_boundary="BORDER", grad_mode="exact",
                 background=None, deterministic=False):
        dev = rho.device
        self.lib = L.load()
        self.rho, self.ux, self.uy, self.uz = rho.contiguous(), ux.contiguous(), uy.contiguous(), uz.contiguous()
        self.M = torch.as_tensor(M, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.V = torch.as_tensor(V, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.P = torch.as_tensor(P, dtype=torch.float32, device=dev).reshape(-1, 16).contiguous()
        self.F = torch.as_tensor(F, dtype=torch.float32, device=dev).reshape(-1, 6).contiguous()
        self.targets = targets.to(device=dev, dtype=torch.float64 if rho.dtype == torch.float64
                                  else torch.float32).contiguous()
        D, H, W = rho.shape[:3]
        nv = self.V.shape[0]
        dd, hh, ww = image_dhw
        Fh = self.F.cpu()
        depth_step = float(Fh[0, 1] - Fh[0, 0]) / dd
        self.emission = (light * depth_step, depth_step)
        st = rho.dtype
        f32 = torch.float64 if st == torch.float64 else torch.float32  # compute / gradient precision
        self.rho_adv = torch.empty((D, H, W, 1), dtype=st, device=dev)
        self.fwd_field = torch.empty((D, H, W, 1), dtype=f32, device=dev)
        self.image = torch.empty((1, nv, hh, ww, 2), dtype=f32, device=dev)
        self.g_image = torch.empty_like(self.image)
        self.g_rho_adv = torch.empty((D, H, W, 1), dtype=f32, device=dev)
        self.g_rho = torch.empty((D, H, W, 1), dtype=f32, device=dev)
        self.g_ux = torch.empty(ux.shape, dtype=f32, device=dev)
        self.g_uy = torch.empty(uy.shape, dtype=f32, device=dev)
        self.g_uz = torch.empty(uz.shape, dtype=f32, device=dev)
        self.loss = torch.zeros((1,), dtype=f32, device=dev)
        self.pixels = nv * hh * ww
        # the cameras' backgrounds behind the volume (renderer.py:804-806), composited
        # into the light channel by the loss epilogue: (views, H, W, 1)
        self.background = None
        if background is not None:
            self.background = torch.as_tensor(background, device=dev).to(self.image.dtype).expand(
                nv, hh, ww, 1).contiguous()

        a = L.AdvectArgs()
        a.dtype = _code(rho)
        if self.ux.dtype != rho.dtype:  # FP16 faces with BF16 density
            a.velocity_dtype = _code(self.ux)
        a.grid_dhw = L.I64x3(D, H, W)
        a.channels = 1
        a.data, a.vel_x, a.vel_y, a.vel_z = _ptr(self.rho), _ptr(self.ux), _ptr(self.uy), _ptr(self.uz)
        a.dt, a.order, a.clamp, a.boundary = float(dt), int(order), L.CLAMP[clamp], L.BOUNDARY[advect_boundary]
        a.output, a.fwd_field = _ptr(self.rho_adv), _ptr(self.fwd_field)
        # the forward's MC_SMOOTH revert mask, read back by the backward
        self.mc_mask = torch.empty((D, H, W, 1), dtype=torch.uint8, device=dev)
        a.mask = _ptr(self.mc_mask)
        # forward 1 hands the forward trace's corner extrema to forward 2
        self.mc_ext = torch.empty((D, H, W, 2), dtype=f32, device=dev)
        a.extrema = _ptr(self.mc_ext)
        # ... and its lookup (centred velocity times -dt) to forward 2 and the backward
        self.mc_lut = torch.empty((D, H, W, 3), dtype=f32, device=dev)
        a.lookup = _ptr(self.mc_lut)
        self.adv = a
        ag = L.AdvectGradArgs()
        ag.fwd = a
        ag.output_grad, ag.data_grad = _ptr(self.g_rho_adv), _ptr(self.g_rho)
        ag.vel_x_grad, ag.vel_y_grad, ag.vel_z_grad = _ptr(self.g_ux), _ptr(self.g_uy), _ptr(self.g_uz)
        ag.grad_mode = L.GRAD[grad_mode]
        # the bit-reproducible (fixed-point) adjoints, exact mode only; set before the
        # workspaces are sized
        det = int(bool(deterministic) and grad_mode == "exact")
        ag.deterministic = det
        self.adv_ws = torch.empty(int(self.lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(ag))),
                                  dtype=torch.uint8, device=dev)
        ag.workspace, ag.workspace_bytes = _ptr(self.adv_ws), self.adv_ws.numel()
        self.adv_g = ag

        r = L.RaymarchArgs()
        r.dtype = _code(rho)
        r.input_shape = L.I64x5(1, D, H, W, 1)
        r.output_dhw = L.I64x3(dd, hh, ww)
        r.input, r.output = _ptr(self.rho_adv), _ptr(self.image)
        r.matrix_m, r.matrix_v, r.matrix_p, r.frustum = _ptr(self.M), _ptr(self.V), _ptr(self.P), _ptr(self.F)
        r.num_cameras = nv
        r.interpolation, r.boundary = L.INTERP["LINEAR"], L.BOUNDARY[render_boundary]
        r.blending_mode, r.keep_dims, r.separate_camera_batch = L.BLEND["BEER_LAMBERT"], 0, 1
        r.emission_channels = 2
        r.emission_scale[0], r.emission_scale[1] = self.emission
        # the advected density in the quad gather layout, prepared once per step for
        # the render's forward and backward; with the exact backward it also keeps
        # the forward's density samples, which the one-pass adjoint reads back
        # instead of gathering them again, where that pays (ops.sample_cache_pays)
        r.sample_cache = int(grad_mode == "exact" and not det and sample_cache_pays((D, H, W), 1, rho.dtype, dev))
        nq = int(self.lib.ngt_raymarch_quad_bytes(ctypes.byref(r)))
        self.ray_quad = torch.empty(nq, dtype=torch.uint8, device=dev) if nq else None
        if nq:
            r.quad = _ptr(self.ray_quad)
        self.ray_fws = torch.empty(int(self.lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))),
                                   dtype=torch.uint8, device=dev)
        r.workspace, r.workspace_bytes = _ptr(self.ray_fws), self.ray_fws.numel()
        # the cameras are fixed for the optimisation: their transforms are formed once
        self.cameras = torch.empty(int(self.lib.ngt_raymarch_cameras_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                   device=dev)
        self._call("ngt_raymarch_cameras", ctypes.byref(r), _ptr(self.cameras),
                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        r.cameras = _ptr(self.cameras)
        # ... and so are their rays, set up in double precision
        self.rays = torch.empty(int(self.lib.ngt_raymarch_rays_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                device=dev)
        self._call("ngt_raymarch_rays", ctypes.byref(r), _ptr(self.rays),
                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        r.rays = _ptr(self.rays)
        self.ray = r
        rg = L.RaymarchGradArgs()
        rg.fwd = r
        rg.output, rg.output_grad, rg.input_grad = _ptr(self.image), _ptr(self.g_image), _ptr(self.g_rho_adv)
        rg.grad_mode = L.GRAD[grad_mode]
        rg.deterministic = det
        self.ray_ws = None
        nb = int(self.lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(rg)))
        if nb:
            self.ray_ws = torch.empty(nb, dtype=torch.uint8, device=dev)
            rg.workspace, rg.workspace_bytes = _ptr(self.ray_ws), nb
        self.ray_g = rg
        self.graph = None

    def _call(self, name, *args):
        L.call(name, *args)

    def bind_inputs(self, rho, ux, uy, uz, targets=None):
        """Point the step at other input tensors of the same shapes and dtype
        (and other targets); the step's own buffers stay."""
        self.rho, self.ux, self.uy, self.uz = rho, ux, uy, uz
        for a in (self.adv, self.adv_g.fwd):
            a.data, a.vel_x, a.vel_y, a.vel_z = _ptr(rho), _ptr(ux), _ptr(uy), _ptr(uz)
        if targets is not None:
            self.targets = targets

    def bind_gradients(self, g_rho, g_ux, g_uy, g_uz):
        """Write the next backward's gradients into these tensors."""
        self.g_rho, self.g_ux, self.g_uy, self.g_uz = g_rho, g_ux, g_uy, g_uz
        ag = self.adv_g
        ag.data_grad, ag.vel_x_grad, ag.vel_y_grad, ag.vel_z_grad = _ptr(g_rho), _ptr(g_ux), _ptr(g_uy), _ptr(g_uz)

    def backward(self, stream=None, render=True):
        """The render and advection backward of the last forward (gradients into
        the bound gradient tensors); ``render`` False: the advection backward
        only, after a forward that ran the render's backward with it."""
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream if stream is None else stream)
        if render:
            self._call("ngt_raymarch_bwd", ctypes.byref(self.ray_g), s)
        self._call("ngt_advect_maccormack_bwd", ctypes.byref(self.adv_g), s)

    def forward(self, stream=None, render_backward=False):
        """Advect, render and the image loss (its gradient included), added to
        ``self.loss``; with ``render_backward`` the render's backward too (into the
        advected density's gradient), in the same launch as its forward."""
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream if stream is None else stream)
        self._call("ngt_advect_maccormack_fwd", ctypes.byref(self.adv), s)
        if self.ray_quad is not None:
            self._call("ngt_raymarch_quad", ctypes.byref(self.ray), _ptr(self.ray_quad), s)
        if render_backward:
            bkg = None if self.background is None else _ptr(self.background)
            self._call("ngt_raymarch_fwd_l2_bwd", ctypes.byref(self.ray_g), bkg, _ptr(self.targets), 1,
                       _ptr(self.loss), s)
        elif self.background is None:
            self._call("ngt_raymarch_fwd_l2", ctypes.byref(self.ray), _ptr(self.targets), 1, _ptr(self.g_image),
                       _ptr(self.loss), s)
        else:
            self._call("ngt_raymarch_fwd_l2_background", ctypes.byref(self.ray), _ptr(self.background),
                       _ptr(self.targets), 1, _ptr(self.g_image), _ptr(self.loss), s)

    def launch(self):
        """Enqueue forward + loss + backward on the current stream."""
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.loss.zero_()
        self.forward(s.value, render_backward=True)
        self.backward(s.value, render=False)

    def loss_only(self):
        """Forward and loss only (e.g. finite differences); returns the loss tensor."""
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.loss.zero_()
        self.forward(s.value)
        return self.loss

    def capture(self):
        """Record one step as a CUDA graph (warm-up launch on a side stream first)."""
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

    def step(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self.loss

    def gradients(self):
        return self.g_rho, self.g_ux, self.g_uy, self.g_uz


# ------------------------------------------------------ differentiable call
# Steps kept per (shapes, dtype, device, cameras, options): their intermediate
# buffers (advected density, MacCormack fields, quad layout, images, workspaces)
# are reused by every call with the same key.  A step is taken from forward to
# backward; a forward while all kept steps of a key wait for their backward
# makes another (up to _MAX_PLANS per key, after which the oldest is taken over
# and its pending backward refuses to run).
#
# Each step also keeps CUDA graphs of its forward and of its backward, keyed by
# the addresses of the tensors they read and write (inputs and targets; input
# gradients): PyTorch's caching allocator hands a training loop the same few
# addresses again and again, so from the second call with the same addresses the
# pass is one graph launch instead of a row of library calls.
_PLANS = {}
_MAX_PLANS = 4
_GRAPHS_PER_PASS = 4


def _matrix_key(M, V, P, F):
    """Content key of the camera matrices (their float32 bytes), formed on every
    call: matrices changed in place between calls key another step, so a step is
    never reused with cameras it was not built for (a few microseconds for the
    usual handful of cameras)."""
    return tuple(np.ascontiguousarray(np.asarray(m.detach().cpu() if isinstance(m, torch.Tensor) else m,
                                                 np.float32)).tobytes() for m in (M, V, P, F))


def _plan_key(rho, ux, uy, uz, M, V, P, F, image_dhw, options):
    return (tuple(rho.shape), tuple(ux.shape), tuple(uy.shape), tuple(uz.shape), rho.dtype, ux.dtype, str(rho.device),
            tuple(int(v) for v in image_dhw), _matrix_key(M, V, P, F), tuple(sorted(options.items())))


class _Pass:
    """Graphs of one pass of a step, by the addresses it binds."""

    def __init__(self):
        self.graphs = collections.OrderedDict()
        self.seen = collections.deque(maxlen=_GRAPHS_PER_PASS)

    def run(self, key, body):
        g = self.graphs.get(key)
        if g is not None:
            self.graphs.move_to_end(key)
            g.replay()
            return
        if key not in self.seen:  # first call at these addresses: run it directly
            self.seen.append(key)
            body()
            return
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            body()
        self.graphs[key] = g
        if len(self.graphs) > _GRAPHS_PER_PASS:
            self.graphs.popitem(last=False)
        g.replay()


class _Plan:
    def __init__(self, step):
        self.step = step
        self.busy = False
        self.generation = 0
        self.fwd = _Pass()
        self.bwd = _Pass()

    def forward(self, render_backward=False):
        st = self.step
        st.loss.zero_()
        st.forward(render_backward=render_backward)


def _take_plan(key, make):
    plans = _PLANS.setdefault(key, [])
    for pl in plans:
        if not pl.busy:
            return pl
    if len(plans) < _MAX_PLANS:
        plans.append(_Plan(make()))
        return plans[-1]
    pl = min(plans, key=lambda q: q.generation)  # the oldest pending forward loses its buffers
    pl.busy = False
    return pl


class _RenderAdvectLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, ux, uy, uz, targets, plan, needs_backward):
        st = plan.step
        st.bind_inputs(rho, ux, uy, uz, targets)
        ctx.fwd_key = tuple(t.data_ptr() for t in (rho, ux, uy, uz, targets))
        # a forward whose backward will follow runs the render's backward with it
        # (one launch); the advection backward waits for the upstream gradient
        nb = bool(needs_backward)
        plan.fwd.run(ctx.fwd_key + (nb,), lambda: plan.forward(render_backward=nb))
        plan.generation = max(pl.generation for pls in _PLANS.values() for pl in pls) + 1
        plan.busy = bool(needs_backward)
        ctx.plan, ctx.generation = plan, plan.generation
        ctx.shapes = (rho, ux, uy, uz)
        return st.loss[0].clone()

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        if plan.generation != ctx.generation or not plan.busy:
            raise RuntimeError("render_advect_loss: the buffers of this forward were taken by a later call "
                               "(more than %d forwards of the same step waiting for their backward)" % _MAX_PLANS)
        st = plan.step
        f = st.g_image.dtype
        grads = [torch.empty(t.shape, dtype=f, device=t.device) for t in ctx.shapes]
        st.bind_gradients(*grads)
        # the render's gradient (linear in the image gradient) takes the upstream scale
        st.g_rho_adv.mul_(g.to(f))
        # the advection backward also reads the forward's inputs
        plan.bwd.run(ctx.fwd_key + tuple(t.data_ptr() for t in grads), lambda: st.backward(render=False))
        plan.busy = False
        return grads[0], grads[1], grads[2], grads[3], None, None, None


def render_advect_loss(rho, ux, uy, uz, M, V, P, F, targets, image_dhw, dt=1.0, light=1.0, order=2,
                       clamp="MC_SMOOTH", advect_boundary="CLAMP", render_boundary="BORDER", background=None):
    """The reconstruction step's loss as one differentiable call: MacCormack warp
    of ``rho`` (D, H, W, 1) by the MAC faces ``ux, uy, uz``, render of every camera
    (Beer-Lambert, the [light*step, step] emission grid), optional background
    composite, and 0.5 * sum of squared differences of the light channel to
    ``targets`` (1, views, H, W, 1).  Returns the loss (a 0-d tensor);
    differentiable w.r.t. rho and the three face grids.

    The same work as ``advect.warp`` + ``ops.raymarch_grid_transform`` +
    ``ops.image_l2_loss`` with autograd between them (data_structures.py:1690-1737,
    renderer.py:718-827, optimization.py:478), as five library calls and one
    autograd node instead of three nodes and their intermediate tensors: the
    step's buffers are kept per shape and camera set and reused by later calls,
    and its passes are replayed as CUDA graphs once the same tensor addresses
    come back.  With ``ops.set_deterministic(True)`` the gradients come from
    the bit-reproducible adjoints (fixed-point sums), the same bits on every
    run."""
    dev = rho.device
    rho, ux, uy, uz = (t.contiguous() for t in (rho, ux, uy, uz))
    cd = torch.float64 if rho.dtype == torch.float64 else torch.float32
    targets = torch.as_tensor(targets, device=dev).to(cd).contiguous()
    options = dict(dt=float(dt), light=float(light), order=int(order), clamp=clamp, advect_boundary=advect_boundary,
                   render_boundary=render_boundary, background=background is not None,
                   deterministic=get_deterministic())
    key = _plan_key(rho, ux, uy, uz, M, V, P, F, image_dhw, options)

    def make():
        return RenderAdvectStep(rho, ux, uy, uz, M, V, P, F, targets, image_dhw, dt=dt, light=light, order=order,
                                clamp=clamp, advect_boundary=advect_boundary, render_boundary=render_boundary,
                                background=background, deterministic=options["deterministic"])

    plan = _take_plan(key, make)
    if background is not None:
        plan.step.background.copy_(torch.as_tensor(background, device=dev).to(cd).expand_as(plan.step.background))
    needs = torch.is_grad_enabled() and any(t.requires_grad for t in (rho, ux, uy, uz))
    return _RenderAdvectLoss.apply(rho, ux, uy, uz, targets, plan, needs)
