"""Known answers and adjoint identities of the oracle (CPU, float64).

Known answers: an integer shift of the velocity moves the density by whole
cells (CLAMP repeats the edge, WRAP rolls), and a uniform integer ux carries
the velocity's other faces the same way; zero velocity is the identity; a
constant grid blends to the closed-form Beer-Lambert sums; rays that miss the
grid's box render 0 under BORDER; index -> object space -> index round trips.
Adjoint identities <A x, y> = <x, A^T y> hold for every operator that is linear
in its input, with the exact gradient as A^T."""
import numpy as np
import pytest

import __graft_entry__

__graft_entry__.load_package()

from ngt_gb300 import scene  # noqa: E402
from oracle import advect as oadvect  # noqa: E402
from oracle import core  # noqa: E402
from oracle import ops as oops  # noqa: E402

RNG = np.random.default_rng(101)


def mats(vol_dhw=(6, 7, 8), cam_dhw=(6, 5, 4), yaws=(17.0, -41.0), shift=None):
    vol = scene.volume_transform(list(vol_dhw))
    if shift is not None:
        vol = scene.GridTransform(list(vol_dhw), translation=shift, center=True, normalize="MIN")
    cams = scene.orbit_cameras(list(cam_dhw), list(yaws))
    M = scene.model_params([vol]).astype(np.float64)
    V, P, F = (a.astype(np.float64) for a in scene.camera_params(cams))
    return M, V, P, F


def faces(shape, ux=0.0, uy=0.0, uz=0.0):
    D, H, W = shape
    return (np.full((D, H, W + 1), ux), np.full((D, H + 1, W), uy), np.full((D + 1, H, W), uz))


def dot(a, b):
    return float(np.sum(np.asarray(a, np.float64) * np.asarray(b, np.float64)))


def assert_adjoint(ax, y, x, aty, tol=1e-12):
    lhs, rhs = dot(ax, y), dot(x, aty)
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs), 1e-300), (lhs, rhs)


# --------------------------------------------------------------------------- known answers

@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bm", ["CLAMP", "WRAP", "BORDER"])
@pytest.mark.parametrize("clamp", ["NONE", "MC_SMOOTH", "NEGATIVE"])
def test_zero_velocity_is_identity(order, bm, clamp):
    rho = RNG.uniform(0, 1, (5, 6, 7, 1))
    out = oadvect.density_maccormack(rho, *faces((5, 6, 7)), order=order, clamp=clamp, boundary=bm)
    assert np.array_equal(out, rho)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bm", ["CLAMP", "WRAP", "BORDER"])
def test_zero_velocity_negative_clamp_cuts_below_zero(order, bm):
    """The NEGATIVE clamp (tf.maximum(d, 0) after the warp, data_structures.py:
    1715-1735) on a density with negative cells and zero velocity: max(rho, 0);
    without a clamp the density itself."""
    rho = RNG.uniform(-1, 1, (5, 6, 7, 1))
    u = faces((5, 6, 7))
    out = oadvect.density_maccormack(rho, *u, order=order, clamp="NEGATIVE", boundary=bm)
    assert np.array_equal(out, np.maximum(rho, 0.0)) and np.any(rho < 0)
    assert np.array_equal(oadvect.density_maccormack(rho, *u, order=order, clamp="NONE", boundary=bm), rho)


@pytest.mark.parametrize("axis,comp", [(2, "ux"), (1, "uy"), (0, "uz")])
@pytest.mark.parametrize("shift", [1, 2, -1])
def test_integer_velocity_shifts_by_whole_cells(axis, comp, shift):
    """dt * u = an integer number of cells: semi-Lagrangian under WRAP rolls the
    grid, under CLAMP shifts it with the edge cells repeated; MacCormack under
    WRAP rolls it too (the back-trace lands on the cells themselves), under
    CLAMP adds half the back-trace's miss on the edge cells."""
    shape = (5, 6, 7)
    rho = RNG.uniform(0, 1, shape + (1,))
    u = faces(shape, **{comp: float(shift)})
    rolled = np.roll(rho, shift, axis=axis)
    assert np.array_equal(oadvect.density_maccormack(rho, *u, order=1, clamp="NONE", boundary="WRAP"), rolled)
    for clamp in ("NONE", "MC_SMOOTH"):
        assert np.allclose(oadvect.density_maccormack(rho, *u, order=2, clamp=clamp, boundary="WRAP"), rolled,
                           rtol=0, atol=1e-15)
    n = shape[axis]
    src = np.clip(np.arange(n) - shift, 0, n - 1)
    clamped = np.take(rho, src, axis=axis)
    assert np.array_equal(oadvect.density_maccormack(rho, *u, order=1, clamp="NONE", boundary="CLAMP"), clamped)
    # MacCormack under CLAMP: the back-trace of the shifted grid, clamped at the
    # edge, leaves the correction 0.5 * (rho - back) on the cells it cannot return to
    back = np.take(clamped, np.clip(np.arange(n) + shift, 0, n - 1), axis=axis)
    assert np.array_equal(oadvect.density_maccormack(rho, *u, order=2, clamp="NONE", boundary="CLAMP"),
                          clamped + 0.5 * (rho - back))


@pytest.mark.parametrize("shift", [1, 2, 3])
@pytest.mark.parametrize("order,clamp", [(1, "NONE"), (2, "MC_SMOOTH"), (2, "NONE")])
def test_velocity_self_advection_integer_transport(shift, order, clamp):
    """Self-advection (VelocityGrid.warped) under a uniform integer ux = c with
    uy = 0 and uz varying along x only: ux stays c, uy stays 0, and the z faces
    are carried c cells along x (their own z motion reads a field constant along
    z).  WRAP rolls them; CLAMP repeats the edge, and second-order MacCormack's
    back-trace from x + c, clamped at the last cell there, leaves the correction
    0.5 * (f(x) - f(W-1-c)) on the last c cells (MC_SMOOTH may revert it: only
    the other cells are fixed then)."""
    D, H, W = 4, 5, 9
    f = RNG.uniform(-0.4, 0.4, W)
    u = (np.full((D, H, W + 1), float(shift)), np.zeros((D, H + 1, W)), np.broadcast_to(f, (D + 1, H, W)).copy())
    ox, oy, oz = oadvect.velocity_maccormack(*u, 1.0, order, clamp, "WRAP")
    assert np.array_equal(oz, np.broadcast_to(np.roll(f, shift), oz.shape))
    assert np.all(ox == shift) and np.all(oy == 0)
    ox, oy, oz = oadvect.velocity_maccormack(*u, 1.0, order, clamp, "CLAMP")
    x = np.arange(W)
    fwd = f[np.clip(x - shift, 0, W - 1)]
    edge = x > W - 1 - shift if order == 2 else np.zeros(W, bool)
    assert np.array_equal(oz[..., ~edge], np.broadcast_to(fwd[~edge], oz[..., ~edge].shape))
    if order == 2 and clamp == "NONE":
        want = fwd[edge] + 0.5 * (f[edge] - f[W - 1 - shift])
        assert np.array_equal(oz[..., edge], np.broadcast_to(want, oz[..., edge].shape))
    assert np.all(ox == shift) and np.all(oy == 0)


@pytest.mark.parametrize("depth", [1, 5, 16])
def test_reduce_blend_constant_closed_form(depth):
    """A constant (emission l, extinction s) column: Beer-Lambert gives
    L = l * sum_{i=1..D} exp(-i s) and optical depth D s; ADDITIVE gives D l, D s."""
    l, s = 0.3, 0.2
    x = np.zeros((1, depth, 2, 3, 2))
    x[..., 0], x[..., 1] = l, s
    out = oops.reduce_grid_blend(x, "BEER_LAMBERT")
    want_l = l * np.exp(-s) * (1 - np.exp(-depth * s)) / (1 - np.exp(-s))
    assert np.allclose(out[..., 0], want_l, rtol=1e-13) and np.allclose(out[..., 1], depth * s, rtol=1e-13)
    add = oops.reduce_grid_blend(x, "ADDITIVE")
    assert np.allclose(add[..., 0], depth * l) and np.allclose(add[..., 1], depth * s)


def test_raymarch_constant_grid_clamp_closed_form():
    """Under CLAMP a constant grid reads its constant everywhere, so every ray
    blends D' equal samples: the image is the closed-form sum for every pixel."""
    M, V, P, F = mats()
    l, s = 0.25, 0.15
    x = np.zeros((1, 6, 7, 8, 2))
    x[..., 0], x[..., 1] = l, s
    img = oops.raymarch_grid_transform(x, M, V, P, F, [6, 5, 4], "LINEAR", "CLAMP", "BEER_LAMBERT")
    n = 6
    want_l = l * np.exp(-s) * (1 - np.exp(-n * s)) / (1 - np.exp(-s))
    assert np.allclose(img[..., 0], want_l, rtol=1e-12) and np.allclose(img[..., 1], n * s, rtol=1e-12)


@pytest.mark.parametrize("blend", ["BEER_LAMBERT", "ALPHA", "ADDITIVE"])
def test_raymarch_missing_rays_are_zero(blend):
    """A grid moved out of every camera's view: all rays miss its box (BORDER)."""
    M, V, P, F = mats(shift=[25.0, 0.0, 0.0])
    x = RNG.uniform(0.1, 1, (1, 6, 7, 8, 2))
    img = oops.raymarch_grid_transform(x, M, V, P, F, [6, 5, 4], "LINEAR", "BORDER", blend)
    assert np.array_equal(img, np.zeros_like(img))


@pytest.mark.parametrize("lin", [False, True])
def test_index_object_space_round_trip(lin):
    M, V, P, F = mats()
    cam = core.CameraMatrices(M[0], V[0], P[0], F[0])
    dims = np.asarray([4, 5, 6], np.float64)  # x, y, z of a frustum grid
    idx = RNG.uniform(0, 1, (50, 3)) * dims
    if lin:
        back = core.os_to_idx_lindepth(core.idx_to_os_lindepth(idx, dims, cam), dims, cam)
    else:
        back = core.os_to_idx(core.idx_to_os(idx, dims, cam), dims, cam)[0]
    assert np.abs(back - idx).max() < 1e-9


# --------------------------------------------------------------------------- adjoint identities

@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_adjoint_lut(fm, bm):
    x = RNG.standard_normal((2, 5, 6, 7, 2))
    lut = RNG.uniform(-1.5, 1.5, (3, 4, 5, 6, 4))
    lut[..., 3] = 0
    y = RNG.standard_normal((2, 3, 4, 5, 6, 2))
    ax = oops.sample_grid_lut(x, lut, fm, bm)
    aty, _ = oops.sample_grid_lut_grad(x, y, lut, fm, bm, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR", "QUADRATIC"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH", "TRANSFORM"])
def test_adjoint_transform(fm, bm, cm):
    M, V, P, F = mats()
    x = RNG.standard_normal((1, 6, 7, 8, 1))
    ax = oops.sample_grid_transform(x, M, V, P, F, [6, 5, 4], fm, bm, coordinate_mode=cm)
    y = RNG.standard_normal(ax.shape)
    aty = oops.sample_grid_transform_grad(x, y, M, V, P, F, fm, bm, coordinate_mode=cm, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_adjoint_raymarch_additive(bm):
    M, V, P, F = mats()
    x = RNG.standard_normal((1, 6, 7, 8, 2))
    ax = oops.raymarch_grid_transform(x, M, V, P, F, [6, 5, 4], "LINEAR", bm, "ADDITIVE")
    y = RNG.standard_normal(ax.shape)
    aty = oops.raymarch_grid_transform_grad(x, ax, y, M, V, P, F, [6, 5, 4], "LINEAR", bm, "ADDITIVE",
                                            grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("kd", [False, True])
def test_adjoint_reduce_blend_additive(kd):
    x = RNG.standard_normal((2, 5, 3, 4, 2))
    ax = oops.reduce_grid_blend(x, "ADDITIVE", kd)
    y = RNG.standard_normal(ax.shape)
    aty = oops.reduce_grid_blend_grad(y, ax, x, "ADDITIVE", kd, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_adjoint_advection_in_density(order, bm):
    """For fixed velocity, semi-Lagrangian and unclamped MacCormack are linear
    in the density."""
    shape = (5, 6, 7)
    u = [RNG.uniform(-1.5, 1.5, s) for s in ((5, 6, 8), (5, 7, 7), (6, 6, 7))]
    x = RNG.standard_normal(shape + (1,))
    ax = oadvect.density_maccormack(x, *u, order=order, clamp="NONE", boundary=bm)
    y = RNG.standard_normal(ax.shape)
    aty = oadvect.density_maccormack_grad(x, *u, y, order=order, clamp="NONE", boundary=bm)[0]
    assert_adjoint(ax, y, x, aty)
