"""MacCormack forward 2 through TMA-staged fwd-field bricks (one channel, x extent
a multiple of 4): bit-exact against the oracle at sizes with partial tiles, with
traces that leave the brick's halo and wrapped indices, and the bounded wait's
give-up path (every block reads global memory, the same bits, and is counted)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import advect as oadvect

pytestmark = pytest.mark.gpu

TILE = (32, 8, 4)  # cells per block along x, y, z


def T(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def inputs(shape, max_u, seed):
    from ngt_gb300 import synthetic
    rho = synthetic.gaussian_blobs(shape, n=5, sigma=(2, 5), seed=seed, dtype=np.float32)
    u = synthetic.curl_noise_mac(shape, max_u=max_u, seed=seed + 1, smooth=2.0, dtype=np.float32)
    return (rho,) + tuple(u)


def blocks(shape):
    d, h, w = shape
    return -(-w // TILE[0]) * -(-h // TILE[1]) * -(-d // TILE[2])


def timeouts(reset=True):
    from ngt_gb300 import _lib
    c = ctypes.c_uint64(0)
    _lib.call("ngt_wait_timeouts", ctypes.byref(c), 1 if reset else 0)
    return c.value


# (depth, height, width): one tile row; partial tiles in every axis
@pytest.mark.parametrize("shape", [(20, 24, 32), (9, 13, 68), (5, 3, 4)])
@pytest.mark.parametrize("bm", ["CLAMP", "BORDER", "WRAP"])
@pytest.mark.parametrize("clamp", ["MC_SMOOTH", "NONE"])
def test_bricked_forward_bitexact(shape, bm, clamp):
    from ngt_gb300 import advect
    # max |u| = 6 cells: many traces leave the 4-cell halo and read global memory
    rho, ux, uy, uz = inputs(shape, 6.0, seed=sum(shape))
    timeouts()
    y = advect.warp(T(rho), T(ux), T(uy), T(uz), dt=1.0, order=2, clamp=clamp, boundary=bm)
    ref = oadvect.density_maccormack(rho, ux, uy, uz, 1.0, 2, clamp, bm)
    assert np.array_equal(y.cpu().numpy(), ref)
    assert timeouts() == 0


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_brick_wait_give_up_path(dtype):
    """With a first-wait limit of 0 polls every block gives up at once, is
    counted, reads every corner from global memory and still waits for its copy
    before it leaves: the output is the same bits as with the bricks."""
    from ngt_gb300 import _lib, advect
    shape = (12, 20, 40)
    rho, ux, uy, uz = (T(a, dtype) for a in inputs(shape, 2.0, seed=5))
    timeouts()
    want = advect.warp(rho, ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
    assert timeouts() == 0
    lib = _lib.load()
    prev = lib.ngt_set_wait_polls(0)
    try:
        got = advect.warp(rho, ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
        torch.cuda.synchronize()
    finally:
        assert lib.ngt_set_wait_polls(prev) == 0
    assert timeouts() == blocks(shape)
    assert torch.equal(got, want)
    again = advect.warp(rho, ux, uy, uz, dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
    assert torch.equal(again, want)
    assert timeouts() == 0
