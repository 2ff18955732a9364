"""The GPU side of the data formats: the aligned rescale of loaded grids against
the oracle's transform resample (all alignments, mip-mapped downscale,
gradients), the magnitude-scaled MAC velocity rescale, a ScalarFlow density
loaded at another resolution, and a density archive rendered through calibrated
cameras in the calibrated simulation grid against the oracle's raymarch."""
import numpy as np
import pytest
import torch

from oracle import ops as oops

from test_formats import synthetic_calibration

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda", 0)
RNG = np.random.default_rng(21)


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def rel(ref, got):
    got = got.detach().double().cpu().numpy() if isinstance(got, torch.Tensor) else np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.linalg.norm((got - ref).ravel()) / max(np.linalg.norm(ref.ravel()), 1e-300))


def oracle_aligned(x, shape, align=("BORDER",) * 3, **kw):
    from ngt_gb300 import formats
    M, V, P, F = formats.aligned_matrices(x.shape[1:4], shape, *align)
    M = np.repeat(M, x.shape[0], 0)
    return oops.sample_grid_transform(x, M, V, P, F, tuple(shape), coordinate_mode="TRANSFORM", **kw)[:, 0]


@pytest.mark.parametrize("C", [1, 2, 4])
@pytest.mark.parametrize("case", [
    ((24, 20, 16), (12, 10, 8), ("BORDER", "BORDER", "BORDER")),
    ((10, 12, 14), (17, 9, 21), ("CENTER", "STAGGER_INPUT", "STAGGER_OUTPUT")),
    ((9, 16, 11), (9, 16, 11), ("BORDER", "CENTER", "BORDER")),
])
def test_resample_aligned_matches_oracle(C, case):
    from ngt_gb300 import formats
    src, dst, align = case
    x = RNG.uniform(0, 1, (2, *src, C)).astype(np.float32)
    kw = dict(interpolation="LINEAR", boundary="BORDER", mipmapping="LINEAR", num_mipmaps=2, mip_bias=0.0)
    y = formats.resample_aligned(T(x), dst, *align)
    assert tuple(y.shape) == (2, *dst, C)
    ref = oracle_aligned(x, dst, align, **kw)
    assert rel(ref, y) < 1e-4


@pytest.mark.parametrize("boundary", ["BORDER", "CLAMP"])
def test_resample_aligned_gradient(boundary):
    """The rescale is differentiable through the transform resample's registered
    gradient (exact adjoint), without mips."""
    from ngt_gb300 import formats
    from ngt_gb300 import ops
    x = RNG.uniform(0, 1, (1, 12, 10, 8, 1)).astype(np.float32)
    xt = T(x).requires_grad_(True)
    y = formats.resample_aligned(xt, (7, 13, 9), "CENTER", "BORDER", "CENTER", boundary=boundary,
                                 mipmapping="NONE")
    gy = RNG.standard_normal(tuple(y.shape)).astype(np.float32)
    with ops.gradient_mode("exact"):
        y.backward(T(gy))
    M, V, P, F = formats.aligned_matrices((12, 10, 8), (7, 13, 9), "CENTER", "BORDER", "CENTER")
    ref = oops.sample_grid_transform_grad(x, gy[:, None], M, V, P, F, boundary=boundary, coordinate_mode="TRANSFORM",
                                          grad_mode="exact")
    assert rel(ref, xt.grad) < 1e-4


def test_scale_velocity_matches_oracle():
    from ngt_gb300 import formats
    old, new = [10, 12, 8], [15, 9, 12]
    comps = [RNG.standard_normal([1] + s + [1]).astype(np.float32) for s in formats.velocity_component_shapes(old)]
    got = formats.scale_velocity(*(T(c) for c in comps), old, new)
    ratio = [o / i for i, o in zip(old, new)]  # z, y, x
    aligns = (("CENTER", "BORDER", "BORDER"), ("BORDER", "CENTER", "BORDER"), ("BORDER", "BORDER", "CENTER"))
    kw = dict(interpolation="LINEAR", boundary="BORDER", mipmapping="LINEAR", num_mipmaps=2)
    for g, c, shp, al, s in zip(got, comps, formats.velocity_component_shapes(new), aligns, ratio[::-1]):
        assert list(g.shape[1:4]) == shp
        assert rel(oracle_aligned(c, shp, al, **kw) * np.float32(s), g) < 1e-4
    same = formats.scale_velocity(*(T(c) for c in comps), old, old)
    assert all(torch.equal(a, T(b)) for a, b in zip(same, comps))


def test_scalarflow_density_rescaled_on_load(tmp_path):
    from ngt_gb300 import formats
    raw = RNG.uniform(0, 1, (20, 36, 20, 1)).astype(np.float32)
    np.savez_compressed(tmp_path / "sf.npz", data=raw)
    g = formats.load_scalarflow_density(tmp_path / "sf.npz", shape=[10, 18, 10], device=DEV)
    assert g.inflow is None and g.d.shape == (1, 10, 18, 10, 1)
    kw = dict(interpolation="LINEAR", boundary="BORDER", mipmapping="LINEAR", num_mipmaps=2)
    ref = oracle_aligned(np.ascontiguousarray(raw[::-1])[None], (10, 18, 10), **kw)
    assert rel(ref, g.d) < 1e-4


def test_scalarflow_velocity_rescaled_on_load(tmp_path):
    from ngt_gb300 import formats
    raw = RNG.standard_normal((8, 14, 8, 3)).astype(np.float32)
    np.savez_compressed(tmp_path / "sfv.npz", data=raw)
    v = formats.load_scalarflow_velocity(tmp_path / "sfv.npz", shape=[12, 21, 12], device=DEV)
    full = formats.load_scalarflow_velocity(tmp_path / "sfv.npz")
    want = formats.scale_velocity(T(full.x), T(full.y), T(full.z), full.centered_shape, [12, 21, 12])
    assert v.centered_shape == [12, 21, 12]
    for a, b in zip((v.x, v.y, v.z), want):
        assert np.array_equal(a, b.cpu().numpy())


def test_archive_rendered_through_calibrated_cameras(tmp_path):
    """A density archive (with inflow) loaded, placed in the calibrated
    simulation grid and rendered by the five calibrated cameras: the GPU raymarch
    against the oracle's on the same matrices, image 2e-5 relative."""
    from ngt_gb300 import formats, ops, scene, synthetic
    c = synthetic_calibration()
    size = formats.scalarflow_density_size(24, c)  # D, H, W = 24, 43, 24
    d = synthetic.gaussian_blobs(size, n=4, center_lo=np.asarray([6, 8, 6]), center_hi=np.asarray([18, 34, 18]),
                                 seed=5)[None]
    inflow = np.full((1, 4, 3, 24, 1), 0.5, np.float32)
    formats.save_density(tmp_path / "d.npz", d, inflow=inflow, inflow_offset=[10, 0, 0])
    g = formats.load_density(tmp_path / "d.npz")
    dens = g.with_inflow().astype(np.float32)
    cams = formats.scalarflow_cameras(c, [32, 24, 20])
    grid = formats.scalarflow_sim_transform(size, c)
    M = scene.model_params([grid])
    V, P, F = scene.camera_params(cams)
    step = np.float32(cams[0].depth_step)
    x = np.concatenate([dens, dens], -1) * step
    img = ops.raymarch_grid_transform(T(x), M, V, P, F, [32, 24, 20])
    ref = oops.raymarch_grid_transform(x, M, V, P, F, [32, 24, 20])
    assert float(np.abs(ref).max()) > 0
    assert rel(ref, img) < 2e-5
