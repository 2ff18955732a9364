"""Adjoint identities and known answers of the CUDA operators (float64).

<A x, y> = <x, A^T y> for every operator linear in its input, A the forward
kernel and A^T its exact gradient kernel (both on the GPU, float64 so that the
identity holds to rounding); and the known answers of the oracle's identity
tests: zero velocity, integer shifts, a constant grid under CLAMP, rays that
miss the box."""
import numpy as np
import pytest
import torch

from test_oracle_identities import faces, mats

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(202)
DEV = torch.device("cuda", 0)


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV, dtype=torch.float64)


def dot(a, b):
    return float((a.double() * b.double()).sum())


def assert_adjoint(ax, y, x, aty, tol=1e-12):
    lhs, rhs = dot(ax, y), dot(x, aty)
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs), 1e-300), (lhs, rhs)


@pytest.fixture(scope="module")
def ops():
    from ngt_gb300 import ops as o
    return o


@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
def test_adjoint_lut(ops, fm, bm):
    x = T(RNG.standard_normal((2, 5, 6, 7, 2)))
    lut = RNG.uniform(-1.5, 1.5, (3, 4, 5, 6, 4))
    lut[..., 3] = 0
    lut = T(lut)
    ax = ops.sample_grid_lut(x, lut, fm, bm)
    y = T(RNG.standard_normal(tuple(ax.shape)))
    aty, _ = ops.sample_grid_lut_grad(x, y, lut, fm, bm, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("fm", ["NEAREST", "LINEAR", "QUADRATIC"])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP"])
@pytest.mark.parametrize("cm", ["TRANSFORM_LINDEPTH", "TRANSFORM"])
def test_adjoint_transform(ops, fm, bm, cm):
    M, V, P, F = mats()
    x = T(RNG.standard_normal((1, 6, 7, 8, 1)))
    ax = ops.sample_grid_transform(x, M, V, P, F, [6, 5, 4], fm, bm, coordinate_mode=cm)
    y = T(RNG.standard_normal(tuple(ax.shape)))
    aty = ops.sample_grid_transform_grad(x, y, M, V, P, F, fm, bm, coordinate_mode=cm, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("C", [1, 2, 4])
def test_adjoint_raymarch_additive(ops, bm, C):
    M, V, P, F = mats()
    x = T(RNG.standard_normal((1, 6, 7, 8, C)))
    ax = ops.raymarch_grid_transform(x, M, V, P, F, [6, 5, 4], "LINEAR", bm, "ADDITIVE")
    y = T(RNG.standard_normal(tuple(ax.shape)))
    aty = ops.raymarch_grid_transform_grad(x, ax, y, M, V, P, F, [6, 5, 4], "LINEAR", bm, "ADDITIVE",
                                           grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("kd", [False, True])
def test_adjoint_reduce_blend_additive(ops, kd):
    x = T(RNG.standard_normal((2, 5, 3, 4, 2)))
    ax = ops.reduce_grid_blend(x, "ADDITIVE", kd)
    y = T(RNG.standard_normal(tuple(ax.shape)))
    aty = ops.reduce_grid_blend_grad(y, ax, x, "ADDITIVE", kd, grad_mode="exact")
    assert_adjoint(ax, y, x, aty)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bm", ["BORDER", "CLAMP", "WRAP"])
@pytest.mark.parametrize("det", [False, True])
def test_adjoint_advection_in_density(order, bm, det):
    from ngt_gb300 import advect
    shape = (5, 6, 7)
    u = [T(RNG.uniform(-1.5, 1.5, s)) for s in ((5, 6, 8), (5, 7, 7), (6, 6, 7))]
    x = T(RNG.standard_normal(shape + (1,)))
    out, fwd, _ = advect.warp_forward(x, *u, order=order, clamp="NONE", boundary=bm)
    y = T(RNG.standard_normal(tuple(out.shape)))
    aty = advect.warp_backward(x, *u, fwd, y, order=order, clamp="NONE", boundary=bm, grad_mode="exact",
                               deterministic=det)[0]
    assert_adjoint(out, y, x, aty)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bm", ["CLAMP", "WRAP", "BORDER"])
@pytest.mark.parametrize("clamp", ["NONE", "MC_SMOOTH", "NEGATIVE"])
def test_zero_velocity_is_identity(order, bm, clamp):
    from ngt_gb300 import advect
    rho = T(RNG.uniform(0, 1, (5, 6, 7, 1))).float()
    u = [T(a).float() for a in faces((5, 6, 7))]
    out = advect.warp(rho, *u, order=order, clamp=clamp, boundary=bm)
    assert torch.equal(out, rho)


@pytest.mark.parametrize("axis,comp", [(2, "ux"), (1, "uy"), (0, "uz")])
@pytest.mark.parametrize("shift", [1, -2])
def test_integer_velocity_shifts_by_whole_cells(axis, comp, shift):
    from ngt_gb300 import advect
    shape = (5, 6, 7)
    rho = T(RNG.uniform(0, 1, shape + (1,))).float()
    u = [T(a).float() for a in faces(shape, **{comp: float(shift)})]
    assert torch.equal(advect.warp(rho, *u, order=1, clamp="NONE", boundary="WRAP"),
                       torch.roll(rho, shift, dims=axis))
    n = shape[axis]
    src = torch.clamp(torch.arange(n, device=DEV) - shift, 0, n - 1)
    assert torch.equal(advect.warp(rho, *u, order=1, clamp="NONE", boundary="CLAMP"),
                       torch.index_select(rho, axis, src))


def test_raymarch_constant_grid_and_missing_rays(ops):
    M, V, P, F = mats()
    l, s = 0.25, 0.15
    x = torch.zeros((1, 6, 7, 8, 2), dtype=torch.float32, device=DEV)
    x[..., 0], x[..., 1] = l, s
    img = ops.raymarch_grid_transform(x, M, V, P, F, [6, 5, 4], "LINEAR", "CLAMP", "BEER_LAMBERT")
    n = 6
    want_l = l * np.exp(-s) * (1 - np.exp(-n * s)) / (1 - np.exp(-s))
    assert torch.allclose(img[..., 0].double(), torch.full_like(img[..., 0].double(), want_l), rtol=1e-6)
    assert torch.allclose(img[..., 1].double(), torch.full_like(img[..., 1].double(), n * s), rtol=1e-6)
    Mf, Vf, Pf, Ff = mats(shift=[25.0, 0.0, 0.0])
    away = ops.raymarch_grid_transform(T(RNG.uniform(0.1, 1, (1, 6, 7, 8, 2))).float(), Mf, Vf, Pf, Ff, [6, 5, 4])
    assert torch.count_nonzero(away) == 0
