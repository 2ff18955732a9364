"""Seeded synthetic smoke inputs standing in for the ScalarFlow captures.

* density: sum of isotropic Gaussian blobs, clamped at 0;
* velocity: MAC-staggered, the discrete curl of a smoothed random vector
  potential stored on cell edges, hence exactly divergence-free on the grid;
  scaled so that the largest face value equals ``max_u`` cells per step.

All generators are deterministic functions of their seed.
"""
import numpy as np


def gaussian_blobs(shape_zyx, n=6, center_lo=None, center_hi=None, sigma=(4.0, 10.0), peak=(0.2, 1.0),
                   seed=0, amp_noise=0.0, noise_seed=None, dtype=np.float32):
    """(D, H, W, 1) density.  Centres uniform in [center_lo, center_hi]^3 (xyz, voxel
    units, defaults 3/16 .. 13/16 of each axis), sigma and peak uniform in the given
    ranges.  ``amp_noise`` scales each blob by (1 + amp_noise * N(0,1)) drawn from
    ``noise_seed`` (the perturbed target density)."""
    d, h, w = shape_zyx
    size = np.array([w, h, d], dtype=np.float64)
    lo = size * 3 / 16 if center_lo is None else np.broadcast_to(np.asarray(center_lo, np.float64), (3,))
    hi = size * 13 / 16 if center_hi is None else np.broadcast_to(np.asarray(center_hi, np.float64), (3,))
    rng = np.random.default_rng(seed)
    centers = rng.uniform(lo, hi, size=(n, 3))
    sigmas = rng.uniform(sigma[0], sigma[1], size=n)
    peaks = rng.uniform(peak[0], peak[1], size=n)
    if amp_noise:
        nrng = np.random.default_rng(noise_seed)
        peaks = peaks * (1.0 + amp_noise * nrng.standard_normal(n))
    z, y, x = np.meshgrid(np.arange(d) + 0.5, np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    rho = np.zeros((d, h, w), np.float64)
    for c, s, p in zip(centers, sigmas, peaks):
        r2 = (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2
        rho += p * np.exp(-r2 / (2.0 * s * s))
    return np.maximum(rho, 0.0)[..., None].astype(dtype)


def _smooth(a, sigma):
    """Periodic Gaussian smoothing via FFT (separable kernel in frequency space)."""
    f = np.fft.fftn(a)
    for ax, n in enumerate(a.shape):
        k = np.fft.fftfreq(n)
        g = np.exp(-2.0 * (np.pi * k * sigma) ** 2)
        shape = [1] * a.ndim
        shape[ax] = n
        f = f * g.reshape(shape)
    return np.real(np.fft.ifftn(f))


def curl_noise_mac(shape_zyx, max_u=1.0, seed=1, smooth=6.0, dtype=np.float32):
    """MAC velocity (ux (D,H,W+1), uy (D,H+1,W), uz (D+1,H,W)) from the discrete curl
    of an edge-centred vector potential."""
    d, h, w = shape_zyx
    rng = np.random.default_rng(seed)
    ax = _smooth(rng.standard_normal((d + 1, h + 1, w)), smooth)   # x-edges
    ay = _smooth(rng.standard_normal((d + 1, h, w + 1)), smooth)   # y-edges
    az = _smooth(rng.standard_normal((d, h + 1, w + 1)), smooth)   # z-edges
    ux = (az[:, 1:, :] - az[:, :-1, :]) - (ay[1:, :, :] - ay[:-1, :, :])
    uy = (ax[1:, :, :] - ax[:-1, :, :]) - (az[:, :, 1:] - az[:, :, :-1])
    uz = (ay[:, :, 1:] - ay[:, :, :-1]) - (ax[:, 1:, :] - ax[:, :-1, :])
    m = max(np.abs(ux).max(), np.abs(uy).max(), np.abs(uz).max())
    s = max_u / m if m > 0 else 0.0
    return (ux * s).astype(dtype), (uy * s).astype(dtype), (uz * s).astype(dtype)


def plume_velocity(shape_zyx, up=0.5, noise=0.3, seed=5, dtype=np.float32):
    """Buoyant plume velocity: constant upward (+y) flow plus curl noise."""
    ux, uy, uz = curl_noise_mac(shape_zyx, max_u=noise, seed=seed, dtype=np.float64)
    uy = uy + up
    return ux.astype(dtype), uy.astype(dtype), uz.astype(dtype)


def inflow_source(shape_zyx, sigma=6.0, amplitude=0.1, height=8.0, dtype=np.float32):
    """Gaussian inflow blob centred at the bottom of the domain (y = ``height``)."""
    d, h, w = shape_zyx
    z, y, x = np.meshgrid(np.arange(d) + 0.5, np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    r2 = (x - w / 2) ** 2 + (y - height) ** 2 + (z - d / 2) ** 2
    return (amplitude * np.exp(-r2 / (2 * sigma * sigma)))[..., None].astype(dtype)
