"""Many scenes of uneven size in one differentiated step: the batched library
calls (one persistent raymarch launch per pass, one advection launch per
phase), one loss call over all images, recorded as one CUDA graph, with the
persistent grid size chosen by a small autotuner.

Each scene: semi-Lagrangian (or MacCormack) advection of its density by its MAC
velocity, a render of each of its cameras (Beer-Lambert, emission expansion),
and the image L2 to its targets; the backward gives every scene's density and
velocity gradients.  ``per_scene()`` runs the same step with one library call
per scene and operator, the reference's calling pattern, for comparison.
"""
import ctypes

import torch

from . import _lib as L
from .ops import _code, _ptr


class Scene:
    """One scene's inputs: density (D,H,W,1), MAC faces, cameras (V, P, F arrays
    with one row per camera), model matrix M, frustum (depth, H, W), targets
    (1, cameras, H, W, 1)."""

    def __init__(self, rho, ux, uy, uz, M, V, P, F, image_dhw, targets):
        self.rho, self.ux, self.uy, self.uz = rho, ux, uy, uz
        self.M, self.V, self.P, self.F = M, V, P, F
        self.image_dhw = tuple(int(v) for v in image_dhw)
        self.targets = targets


class BatchedScenes:
    def __init__(self, scenes, dt=1.0, light=1.0, order=1, clamp="NONE", advect_boundary="CLAMP",
                 render_boundary="BORDER", blocks_per_sm=(0, 0)):
        assert 1 <= len(scenes) <= 32
        self.lib = L.load()
        self.n = n = len(scenes)
        dev = scenes[0].rho.device
        st = scenes[0].rho.dtype
        cd = torch.float64 if st == torch.float64 else torch.float32
        self.blocks_per_sm = list(blocks_per_sm)
        self.keep = []  # tensors referenced by the argument structs

        def keep(t):
            self.keep.append(t)
            return t

        f32 = lambda a, w: keep(torch.as_tensor(a, dtype=torch.float32, device=dev).reshape(-1, w).contiguous())
        # images and targets of all scenes back to back: one loss call
        sizes = [int(s.V.shape[0] if hasattr(s.V, "shape") else len(s.V)) * s.image_dhw[1] * s.image_dhw[2]
                 for s in scenes]
        self.pixels = sum(sizes)
        self.images = torch.empty((self.pixels, 2), dtype=cd, device=dev)
        self.g_images = torch.empty_like(self.images)
        self.targets = torch.cat([s.targets.to(device=dev, dtype=cd).reshape(-1) for s in scenes]).contiguous()
        self.loss = torch.zeros((1,), dtype=cd, device=dev)

        self.adv = (L.AdvectArgs * n)()
        self.adv_g = (L.AdvectGradArgs * n)()
        self.ray = (L.RaymarchArgs * n)()
        self.ray_g = (L.RaymarchGradArgs * n)()
        self.rho, self.u, self.grads = [], [], []
        off = 0
        for k, s in enumerate(scenes):
            D, H, W = s.rho.shape[:3]
            rho = keep(s.rho.contiguous())
            u = [keep(t.contiguous()) for t in (s.ux, s.uy, s.uz)]
            self.rho.append(rho)
            self.u.append(u)
            rho_adv = keep(torch.empty((D, H, W, 1), dtype=st, device=dev))
            fwd = keep(torch.empty((D, H, W, 1), dtype=cd, device=dev))
            g_rho_adv = keep(torch.empty((D, H, W, 1), dtype=cd, device=dev))
            g = [torch.empty((D, H, W, 1), dtype=cd, device=dev)] + [torch.empty(t.shape, dtype=cd, device=dev)
                                                                     for t in u]
            self.grads.append(g)
            a = self.adv[k]
            a.dtype = _code(rho)
            a.grid_dhw = L.I64x3(D, H, W)
            a.channels = 1
            a.data, a.vel_x, a.vel_y, a.vel_z = _ptr(rho), _ptr(u[0]), _ptr(u[1]), _ptr(u[2])
            a.dt, a.order, a.clamp, a.boundary = float(dt), int(order), L.CLAMP[clamp], L.BOUNDARY[advect_boundary]
            a.output, a.fwd_field = _ptr(rho_adv), _ptr(fwd)
            a.lookup = _ptr(keep(torch.empty((D, H, W, 3), dtype=cd, device=dev)))
            if int(order) == 2 and clamp.upper() == "MC_SMOOTH":
                # the revert mask (forward 2 -> backward 1) and the forward trace's
                # corner extrema (forward 1 -> forward 2)
                a.mask = _ptr(keep(torch.empty((D, H, W, 1), dtype=torch.uint8, device=dev)))
                a.extrema = _ptr(keep(torch.empty((D, H, W, 2), dtype=cd, device=dev)))
            ag = self.adv_g[k]
            ag.fwd = a
            ag.output_grad, ag.data_grad = _ptr(g_rho_adv), _ptr(g[0])
            ag.vel_x_grad, ag.vel_y_grad, ag.vel_z_grad = _ptr(g[1]), _ptr(g[2]), _ptr(g[3])
            ag.grad_mode = L.GRAD["exact"]

            V, P, F = f32(s.V, 16), f32(s.P, 16), f32(s.F, 6)
            M = f32(s.M, 16)
            nv = V.shape[0]
            dd, hh, ww = s.image_dhw
            step = float(F[0, 1] - F[0, 0]) / dd
            img = self.images[off:off + sizes[k]]
            gimg = self.g_images[off:off + sizes[k]]
            off += sizes[k]
            r = self.ray[k]
            r.dtype = _code(rho)
            r.input_shape = L.I64x5(1, D, H, W, 1)
            r.output_dhw = L.I64x3(dd, hh, ww)
            r.input, r.output = _ptr(rho_adv), _ptr(img)
            r.matrix_m, r.matrix_v, r.matrix_p, r.frustum = _ptr(M), _ptr(V), _ptr(P), _ptr(F)
            r.num_cameras = nv
            r.interpolation, r.boundary = L.INTERP["LINEAR"], L.BOUNDARY[render_boundary]
            r.blending_mode, r.keep_dims, r.separate_camera_batch = L.BLEND["BEER_LAMBERT"], 0, 1
            r.emission_channels = 2
            r.emission_scale[0], r.emission_scale[1] = light * step, step
            cams = keep(torch.empty(int(self.lib.ngt_raymarch_cameras_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                    device=dev))
            self._call("ngt_raymarch_cameras", ctypes.byref(r), _ptr(cams), self._stream())
            r.cameras = _ptr(cams)
            # the scene's rays, set up once in double precision
            rays = keep(torch.empty(int(self.lib.ngt_raymarch_rays_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                    device=dev))
            self._call("ngt_raymarch_rays", ctypes.byref(r), _ptr(rays), self._stream())
            r.rays = _ptr(rays)
            rg = self.ray_g[k]
            rg.fwd = r
            rg.output, rg.output_grad, rg.input_grad = _ptr(img), _ptr(gimg), _ptr(g_rho_adv)
            rg.grad_mode = L.GRAD["exact"]
        # every scene's targets within the one target array (the fused render's loss)
        tsz = self.targets.element_size()
        starts = [sum(sizes[:k]) for k in range(n)]
        self.target_ptrs = (ctypes.c_void_p * n)(*[self.targets.data_ptr() + o * tsz for o in starts])
        self.ray_ws = torch.empty(int(self.lib.ngt_raymarch_batch_workspace_bytes(self.ray, n)), dtype=torch.uint8,
                                  device=dev)
        self.adv_ws = torch.empty(int(self.lib.ngt_advect_maccormack_bwd_batch_workspace_bytes(self.adv_g, n)),
                                  dtype=torch.uint8, device=dev)
        self.graph = None

    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _call(self, name, *args):
        L.call(name, *args)

    # ---------------------------------------------------------------- passes
    def advect_fwd(self, s):
        self._call("ngt_advect_maccormack_fwd_batch", self.adv, self.n, s)

    def render_fwd(self, s):
        self._call("ngt_raymarch_fwd_batch", self.ray, self.n, self.blocks_per_sm[0], _ptr(self.ray_ws),
                   self.ray_ws.numel(), s)

    def render_bwd(self, s, after_fwd=True):
        """The batched render backward; ``after_fwd``: right after render_fwd on the
        same workspace, whose quad layouts and sign words it reuses."""
        name = "ngt_raymarch_bwd_batch_after_fwd" if after_fwd else "ngt_raymarch_bwd_batch"
        self._call(name, self.ray_g, self.n, self.blocks_per_sm[1], _ptr(self.ray_ws), self.ray_ws.numel(), s)

    def advect_bwd(self, s):
        self._call("ngt_advect_maccormack_bwd_batch", self.adv_g, self.n, _ptr(self.adv_ws), self.adv_ws.numel(), s)

    def render_fused(self, s):
        """Every scene's render forward, image loss and backward in one persistent
        launch (each (scene, camera, tile) item marched forward and back by the
        same threads), then the folds."""
        self._call("ngt_raymarch_fwd_l2_bwd_batch", self.ray_g, self.target_ptrs, self.n, 1, _ptr(self.loss),
                   self.blocks_per_sm[1], _ptr(self.ray_ws), self.ray_ws.numel(), s)

    def launch(self):
        s = self._stream()
        self.loss.zero_()
        self.advect_fwd(s)
        self.render_fused(s)
        self.advect_bwd(s)

    def launch_passes(self):
        """The same step with the render as three calls: batched forward, one loss
        call over all images, batched backward reusing the forward's quad layouts."""
        s = self._stream()
        self.loss.zero_()
        self.advect_fwd(s)
        self.render_fwd(s)
        self._call("ngt_image_l2_loss", _code(self.images), self.pixels, 2, 1, _ptr(self.images),
                   _ptr(self.targets), _ptr(self.g_images), _ptr(self.loss), s)
        self.render_bwd(s)
        self.advect_bwd(s)

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

    def step(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self.loss

    def gradients(self, k):
        """(d rho, d ux, d uy, d uz) of scene k."""
        return tuple(self.grads[k])

    # ------------------------------------------------------------ comparison
    def _per_scene_args(self):
        """Single-scene argument structs with their own workspaces (built once)."""
        if getattr(self, "_single", None) is not None:
            return self._single
        dev = self.images.device
        ray, ray_g, adv_g = [], [], []
        for k in range(self.n):
            r = L.RaymarchArgs.from_buffer_copy(self.ray[k])
            ws = self.keep_ws(int(self.lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r))), dev)
            r.workspace, r.workspace_bytes = _ptr(ws), ws.numel()
            ray.append(r)
            g = L.RaymarchGradArgs.from_buffer_copy(self.ray_g[k])
            ws = self.keep_ws(int(self.lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dev)
            g.workspace, g.workspace_bytes = _ptr(ws), ws.numel()
            ray_g.append(g)
            a = L.AdvectGradArgs.from_buffer_copy(self.adv_g[k])
            ws = self.keep_ws(int(self.lib.ngt_advect_maccormack_bwd_workspace_bytes(ctypes.byref(a))), dev)
            a.workspace, a.workspace_bytes = _ptr(ws), ws.numel()
            adv_g.append(a)
        self._single = (ray, ray_g, adv_g)
        return self._single

    def keep_ws(self, nbytes, dev):
        t = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
        self.keep.append(t)
        return t

    def per_scene_launch(self):
        """Enqueue the same step with one single-scene library call per scene and operator."""
        ray, ray_g, adv_g = self._per_scene_args()
        s = self._stream()
        self.loss.zero_()
        for k in range(self.n):
            self._call("ngt_advect_maccormack_fwd", ctypes.byref(self.adv[k]), s)
        for k in range(self.n):
            self._call("ngt_raymarch_fwd", ctypes.byref(ray[k]), s)
        self._call("ngt_image_l2_loss", _code(self.images), self.pixels, 2, 1, _ptr(self.images),
                   _ptr(self.targets), _ptr(self.g_images), _ptr(self.loss), s)
        for k in range(self.n):
            self._call("ngt_raymarch_bwd", ctypes.byref(ray_g[k]), s)
        for k in range(self.n):
            self._call("ngt_advect_maccormack_bwd", ctypes.byref(adv_g[k]), s)

    def per_scene(self):
        self.per_scene_launch()
        torch.cuda.current_stream().synchronize()
        return self.loss

    # -------------------------------------------------------------- autotune
    def autotune(self, candidates=(4, 6, 8, 10, 12, 16), repeats=5):
        """Time the step's persistent raymarch launch (forward, loss and backward)
        for each blocks-per-SM setting on these scenes and keep the fastest;
        returns [(blocks per SM, {setting: ms})]."""
        s = self._stream()
        self.launch()
        best = []
        for which, fn in ((1, self.render_fused),):
            times = {}
            for c in candidates:
                self.blocks_per_sm[which] = c
                fn(s)  # warm
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(repeats):
                    fn(s)
                b.record()
                torch.cuda.synchronize()
                times[c] = a.elapsed_time(b) / repeats
            c = min(times, key=times.get)
            self.blocks_per_sm[which] = c
            best.append((c, times))
        self.graph = None
        return best
