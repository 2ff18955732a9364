"""The render's sample cache (ngt_raymarch_args::sample_cache): a Beer-Lambert
forward through a prepared quad layout keeps every ray's first D density
samples, and the one-pass backward of the same rays reads them instead of
gathering again.  The image is the same bits and the gradient the same sums;
a cache that no longer matches -- the quad layout rebuilt for another density,
or a forward of another ray table in between -- is not used."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(29)
VOL = (14, 18, 22)
CAM = (16, 20, 24)  # depth samples, image height, width


def mats(yaws):
    from ngt_gb300 import scene
    vol = scene.volume_transform(list(VOL))
    cams = scene.orbit_cameras(list(CAM), list(yaws))
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    return M, V, P, F


class Render:
    """ABI-level forward and exact backward of one scene through a prepared quad
    layout and ray table."""

    def __init__(self, x, yaws, bm, sample_cache):
        from ngt_gb300 import _lib as L
        from ngt_gb300 import ops
        self.L, self.ops, self.lib = L, ops, L.load()
        self.x = x
        M, V, P, F = mats(yaws)
        self.mats = [ops._floats(m, w, x.device) for m, w in ((M, 16), (V, 16), (P, 16), (F, 6))]
        attrs = dict(interpolation="LINEAR", boundary=bm, blending_mode="BEER_LAMBERT", keep_dims=False,
                     separate_camera_batch=True, emission_scale=(0.6, 1.2))
        self.y = torch.empty((1, len(yaws)) + CAM[1:] + (2,), device="cuda")
        r = ops._ray_args(x, *self.mats, list(CAM), self.y, attrs)
        r.sample_cache = sample_cache
        self.stream = ops._stream()
        self.quad = torch.empty(int(self.lib.ngt_raymarch_quad_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                device="cuda")
        self.rays = torch.empty(int(self.lib.ngt_raymarch_rays_bytes(ctypes.byref(r))), dtype=torch.uint8,
                                device="cuda")
        assert self.lib.ngt_raymarch_rays(ctypes.byref(r), ops._ptr(self.rays), self.stream) == L.NGT_OK
        r.rays = ops._ptr(self.rays)
        self.r = r
        self.prepare()

    def prepare(self):
        self.r.input = self.ops._ptr(self.x)
        assert self.lib.ngt_raymarch_quad(ctypes.byref(self.r), self.ops._ptr(self.quad), self.stream) == self.L.NGT_OK
        self.r.quad = self.ops._ptr(self.quad)

    def forward(self):
        self.r.input = self.ops._ptr(self.x)
        assert self.lib.ngt_raymarch_fwd(ctypes.byref(self.r), self.stream) == self.L.NGT_OK
        return self.y.clone()

    def backward(self, y, gy):
        L = self.L
        g = L.RaymarchGradArgs()
        g.fwd = self.r
        g.fwd.input = self.ops._ptr(self.x)
        gx = torch.empty(self.x.shape, device="cuda")
        g.output, g.output_grad, g.input_grad, g.grad_mode = (self.ops._ptr(y), self.ops._ptr(gy), self.ops._ptr(gx),
                                                              L.GRAD["exact"])
        ws = torch.empty(int(self.lib.ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                         device="cuda")
        g.workspace, g.workspace_bytes = self.ops._ptr(ws), ws.numel()
        assert self.lib.ngt_raymarch_bwd(ctypes.byref(g), self.stream) == L.NGT_OK
        torch.cuda.synchronize()
        return gx


def density(dtype, seed):
    a = (np.random.default_rng(seed).uniform(0, 1, (1,) + VOL + (1,)) * 0.3).astype(np.float32)
    return torch.as_tensor(a, device="cuda").to(dtype)


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
def test_cached_samples_give_the_same_image_and_gradient(dtype, bm):
    x = density(dtype, 1)
    yaws = (10, -40, 75)
    plain, cached = Render(x, yaws, bm, 0), Render(x, yaws, bm, 1)
    assert cached.quad.numel() > plain.quad.numel()
    y0, y1 = plain.forward(), cached.forward()
    assert torch.equal(y0, y1)
    gy = torch.as_tensor(RNG.standard_normal(tuple(y0.shape)).astype(np.float32), device="cuda")
    g0, g1 = plain.backward(y0, gy), cached.backward(y1, gy)
    assert rel(g1, g0) < 1e-6
    # the forward tagged the cache (an odd word: its ray table and sizes mixed)
    tag = int(cached.quad[8:16].view(torch.int64).item())
    assert tag & 1


def test_cache_of_another_density_is_not_used():
    """Forward of density A keeps A's samples; the quad layout rebuilt for density B
    clears the tag, so B's backward gathers B (a stale cache would give A's)."""
    yaws = (20, -60)
    a, b = density(torch.float32, 2), density(torch.float32, 3)
    ref = Render(b, yaws, "BORDER", 0)
    yb = ref.forward()
    gy = torch.as_tensor(RNG.standard_normal(tuple(yb.shape)).astype(np.float32), device="cuda")
    want = ref.backward(yb, gy)
    r = Render(a, yaws, "BORDER", 1)
    r.forward()
    r.x = b
    r.prepare()
    assert int(r.quad[8:16].view(torch.int64).item()) == 0
    got = r.backward(yb, gy)
    assert rel(got, want) < 1e-6


def test_cache_of_other_rays_is_not_used():
    """A forward of another ray table through the same quad buffer re-tags the
    cache; a backward of the first rays then gathers."""
    x = density(torch.float32, 4)
    first = Render(x, (15, -25), "BORDER", 1)
    other = Render(x, (80, 140), "BORDER", 1)
    other.quad, other.r.quad = first.quad, first.r.quad  # one quad buffer, two ray tables
    y = first.forward()
    gy = torch.as_tensor(RNG.standard_normal(tuple(y.shape)).astype(np.float32), device="cuda")
    want = first.backward(y, gy)  # from the cache
    tag_first = int(first.quad[8:16].view(torch.int64).item())
    other.forward()
    assert int(first.quad[8:16].view(torch.int64).item()) not in (0, tag_first)
    got = first.backward(y, gy)  # the tag names the other rays: gathers
    assert rel(got, want) < 1e-6
