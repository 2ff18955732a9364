"""Spot-light shadow transmission (the shadow-map composition of the
reference's SpotLight) on the library's resample and depth-scan operators,
forward and gradient, against the oracle's composition."""
import numpy as np
import pytest
import torch

from oracle import ops as oops

pytestmark = pytest.mark.gpu


def light(vol_dhw=(10, 12, 14), shadow_dhw=(12, 10, 10)):
    from ngt_gb300 import scene
    vol = scene.volume_transform(list(vol_dhw))
    cams = scene.orbit_cameras(list(shadow_dhw), [23.0])
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    return M, V, P, F, cams[0].depth_step


def mask_np(h, w):
    y, x = np.meshgrid(np.linspace(-1, 1, h), np.linspace(-1, 1, w), indexing="ij")
    return (np.sqrt(y * y + x * x) <= 1).astype(np.float32)[..., None]


@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])  # the transform resample takes no WRAP
def test_shadow_transmission(bm):
    from ngt_gb300 import lighting
    M, V, P, F, step = light()
    rng = np.random.default_rng(17)
    rho = rng.uniform(0, 0.5, (1, 10, 12, 14, 1)).astype(np.float32)
    dev = torch.device("cuda", 0)
    rt = torch.as_tensor(rho, device=dev).requires_grad_()
    out = lighting.shadow_transmission(rt, M, V, P, F, (12, 10, 10), step, boundary=bm)
    g = rng.standard_normal(tuple(out.shape)).astype(np.float32)
    out.backward(torch.as_tensor(g, device=dev))

    # oracle composition
    x = (rho * np.float32(step)).astype(np.float32)
    sd = oops.sample_grid_transform(x, M, V, P, F, [12, 10, 10], "LINEAR", bm)[:, 0]
    cum = oops.reduce_grid_blend(sd, "BEER_LAMBERT", keep_dims=True)
    pad = {"BORDER": np.zeros_like(cum[:, :1]), "CLAMP": cum[:, :1]}[bm]
    sh = np.concatenate([pad, cum[:, :-1]], 1)
    m = mask_np(10, 10)
    tr = np.exp(-sh) * m
    ref = oops.sample_grid_transform(tr.astype(np.float32), M, V, P, F, [10, 12, 14], "LINEAR", bm,
                                     coordinate_mode="TRANSFORM_LINDEPTH_REVERSE")[:, 0]
    rel = lambda a, b: np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30)
    assert rel(out.detach().cpu().numpy(), ref) < 2e-5

    g_tr = oops.sample_grid_transform_grad(tr.astype(np.float32), g[:, None], M, V, P, F, "LINEAR", bm,
                                           coordinate_mode="TRANSFORM_LINDEPTH_REVERSE")
    g_sh = -(g_tr * m * np.exp(-sh))
    g_cum = np.zeros_like(cum)
    g_cum[:, :-1] += g_sh[:, 1:]
    if bm == "CLAMP":
        g_cum[:, :1] += g_sh[:, :1]
    g_sd = oops.reduce_grid_blend_grad(g_cum.astype(np.float32), cum, sd, "BEER_LAMBERT", keep_dims=True)
    g_x = oops.sample_grid_transform_grad(x, g_sd[:, None].astype(np.float32), M, V, P, F, "LINEAR", bm)
    assert rel(rt.grad.cpu().numpy(), g_x * np.float32(step)) < 1e-4
