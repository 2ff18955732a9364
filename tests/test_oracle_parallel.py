"""The oracle split over host processes (z-slabs for the warp, row bands for the
render) against the same oracle run whole, on the CPU: the warp forward bit for
bit, the render bands and every gradient to float32 rounding."""
import numpy as np
import pytest

from oracle import advect, ops, parallel


@pytest.fixture(scope="module")
def pool():
    p, n = parallel.make_pool(3)
    yield p, n
    p.close()
    p.join()


def small():
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import workloads
    return workloads.render_step(grid=(26, 20, 22), views=2, image=(20, 18), depth=24, max_u=2.0)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def test_slabs_cover_the_grid_with_their_halo():
    for depth, parts, halo in ((128, 16, 7), (26, 3, 7), (5, 8, 3), (96, 16, 5)):
        s = parallel.slabs(depth, parts, halo)
        assert s[0][0] == 0 and s[-1][1] == depth
        for (lo, hi, z_lo, z_hi), nxt in zip(s, s[1:] + [None]):
            assert z_lo <= max(0, lo - halo) and z_hi == min(depth, hi + halo)
            assert z_lo == 0 or z_lo >= halo
            if nxt:
                assert nxt[0] == hi


@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NONE"), (2, "NONE")])
def test_slab_warp_matches_whole_grid(pool, order, clamp):
    w = small()
    p, n = pool
    want = advect.density_maccormack(w.rho, w.ux, w.uy, w.uz, order=order, clamp=clamp)
    got = parallel.density_fwd(p, n, w.rho, w.ux, w.uy, w.uz, order=order, clamp=clamp)
    assert np.array_equal(got, want)
    g = np.random.default_rng(4).standard_normal(w.rho.shape).astype(np.float32)
    want_g = advect.density_maccormack_grad(w.rho, w.ux, w.uy, w.uz, g, order=order, clamp=clamp)
    got_g = parallel.density_bwd(p, n, w.rho, w.ux, w.uy, w.uz, g, order=order, clamp=clamp)
    for a, b in zip(got_g, want_g):
        assert rel(a, b) < 1e-6


def test_band_render_and_step_match_whole_image(pool):
    w = small()
    p, n = pool
    s = np.float32(w.depth_step)
    sc = np.asarray([s, s], np.float32)
    tgt = ops.raymarch_grid_transform((w.rho_target * sc)[None], w.M, w.V, w.P, w.F, w.image_dhw)[..., :1]
    image, loss, grads = parallel.render_advect_step(p, n, w.rho, w.ux, w.uy, w.uz, w.M, w.V, w.P, w.F, tgt,
                                                     w.image_dhw, w.depth_step)
    rho2 = advect.density_maccormack(w.rho, w.ux, w.uy, w.uz)
    x = rho2[None] * sc
    img = ops.raymarch_grid_transform(x, w.M, w.V, w.P, w.F, w.image_dhw)
    assert np.array_equal(image, img)
    diff = img[..., :1] - tgt
    assert abs(loss - 0.5 * float((diff.astype(np.float64) ** 2).sum())) <= 1e-9 * loss
    gx = ops.raymarch_grid_transform_grad(x, img, np.concatenate([diff, np.zeros_like(diff)], -1), w.M, w.V, w.P,
                                          w.F, w.image_dhw)
    ref = advect.density_maccormack_grad(w.rho, w.ux, w.uy, w.uz, (gx[0] * sc).sum(-1, keepdims=True))
    for a, b in zip(grads, ref):
        assert rel(a, b) < 1e-6
