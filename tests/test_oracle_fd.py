"""The oracle's gradients of the compositions the reference forms with
TensorFlow ops -- the advection and the background composite -- against central
finite differences (CPU, float64).

The reference forms the MacCormack warp and its gradient through TensorFlow
(data_structures.py:1690-1737 for the density, 1081-1164 for the velocity),
which cannot run here, so the oracle's exact adjoints of those compositions are
pinned by differentiating its own forward: for a random upstream gradient g,
d<warp(x), g>/dx_k from two forward evaluations at x_k +- eps matches the
adjoint's entry k, for the density and every face of the velocity, with the
MC_SMOOTH revert switch and all three boundary rules.  Trilinear sampling is
piecewise linear in the position, so the differences are exact up to rounding
unless a perturbation crosses a cell boundary or a revert switch (probability
~eps per entry with random velocities)."""
import numpy as np
import pytest

import __graft_entry__

__graft_entry__.load_package()

from oracle import advect as oadvect  # noqa: E402

EPS = 1e-6
SHAPE = (5, 6, 7)
FACE_SHAPES = ((5, 6, 8), (5, 7, 7), (6, 6, 7))


def inputs(seed):
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.0, 1.0, SHAPE + (1,))
    u = [rng.uniform(-1.6, 1.6, s) for s in FACE_SHAPES]
    return rng, rho, u


def fd_entry(f, arrays, which, idx, g):
    """Central difference of <f(arrays), g> in arrays[which][idx]."""
    a = [x.copy() for x in arrays]
    a[which][idx] += EPS
    hi = f(*a)
    a[which][idx] -= 2 * EPS
    lo = f(*a)
    if isinstance(hi, tuple):
        return sum(float(np.sum((h - l) * gg)) for h, l, gg in zip(hi, lo, g)) / (2 * EPS)
    return float(np.sum((hi - lo) * g)) / (2 * EPS)


def check(analytic, f, arrays, g, rng, picks=12):
    """``picks`` random entries of every array: each difference matches the
    analytic entry to 1e-6 of the array's largest gradient; at most one entry
    per array may sit on a kink."""
    for which, (an, arr) in enumerate(zip(analytic, arrays)):
        scale = max(float(np.abs(an).max()), 1e-12)
        bad = 0
        for _ in range(picks):
            idx = tuple(int(rng.integers(0, n)) for n in arr.shape)
            d = fd_entry(f, arrays, which, idx, g)
            if abs(d - float(an[idx])) > 1e-6 * scale:
                bad += 1
        assert bad <= 1, (which, bad)


@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (2, "NONE"), (1, "NONE")])
def test_density_advection_gradient_matches_differences(bm, order, clamp):
    rng, rho, u = inputs(7)
    g = rng.standard_normal(SHAPE + (1,))

    def f(r, ux, uy, uz):
        return oadvect.density_maccormack(r, ux, uy, uz, 1.0, order, clamp, bm)

    grads = oadvect.density_maccormack_grad(rho, *u, g, 1.0, order, clamp, bm)
    check(grads, f, [rho] + u, g, rng)


@pytest.mark.parametrize("bm", ["CLAMP", "WRAP"])
@pytest.mark.parametrize("order,clamp", [(2, "MC_SMOOTH"), (1, "NONE")])
def test_velocity_advection_gradient_matches_differences(bm, order, clamp):
    rng, _, u = inputs(11)
    gs = [rng.standard_normal(s) for s in FACE_SHAPES]

    def f(ux, uy, uz):
        return tuple(oadvect.velocity_maccormack(ux, uy, uz, 1.0, order, clamp, bm))

    grads = oadvect.velocity_maccormack_grad(*u, gs, 1.0, order, clamp, bm)
    check(grads, f, u, gs, rng, picks=6)


def test_background_composite_gradient_matches_differences():
    """The background composite of the render composition (renderer.py:779-781,
    804-806: light + background * exp(-d), the depth channel cut), restated from
    TensorFlow ops: its adjoint to the image (light and depth channels) and to
    the background shared by the batch, against central differences."""
    from oracle import ops as oops
    rng = np.random.default_rng(5)
    image = rng.uniform(0.0, 2.0, (2, 3, 4, 5, 3))  # batch, views, H, W, [light x2, depth]
    bkg = rng.uniform(0.0, 1.0, (3, 4, 5, 2))
    g = rng.standard_normal((2, 3, 4, 5, 2))
    gi, gb = oops.background_composite_grad(image, bkg, g)
    for which, an in ((0, gi), (1, gb)):
        arr = (image, bkg)[which]
        for _ in range(20):
            idx = tuple(int(rng.integers(0, n)) for n in arr.shape)
            d = fd_entry(oops.background_composite, [image, bkg], which, idx, g)
            assert abs(d - float(an[idx])) <= 1e-8 * max(1.0, abs(float(an[idx])))
