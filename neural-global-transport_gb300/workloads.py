"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Stand-ins for the ScalarFlow captures (not available offline): Gaussian-blob
densities, curl-noise MAC velocities and an orbit of cameras built with the
reference's camera / grid-transform conventions (``scene``).
"""
import numpy as np

from . import scene, synthetic


class Workload:
    """Arrays (float32, numpy) and camera parameters of one configuration."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def render_step(grid=(128, 128, 128), views=5, image=(256, 256), depth=128, max_u=2.0, yaw_span=120.0,
                density_seed=0, velocity_seed=1, target_seed=2, blobs=6, target_noise=0.05):
    """The differentiated single step (MacCormack advect, render, L2, backward):
    grid ``D,H,W``, ``views`` cameras on a ``yaw_span`` arc about +y, frustum
    ``depth x image``.  Blob centres span the middle 5/8 of each axis."""
    D, H, W = grid
    lo = np.array([W, H, D]) * 3 / 16
    hi = np.array([W, H, D]) * 13 / 16
    rho = synthetic.gaussian_blobs(grid, n=blobs, center_lo=lo, center_hi=hi, seed=density_seed)
    rho_target = synthetic.gaussian_blobs(grid, n=blobs, center_lo=lo, center_hi=hi, seed=density_seed,
                                          amp_noise=target_noise, noise_seed=target_seed)
    ux, uy, uz = synthetic.curl_noise_mac(grid, max_u=max_u, seed=velocity_seed)
    yaws = np.linspace(-yaw_span / 2, yaw_span / 2, views) if views > 1 else np.array([0.0])
    cams = scene.orbit_cameras([depth, image[0], image[1]], list(yaws))
    vol = scene.volume_transform(list(grid))
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    return Workload(rho=rho, rho_target=rho_target, ux=ux, uy=uy, uz=uz, M=M, V=V, P=P, F=F, cameras=cams,
                    image_dhw=(depth, image[0], image[1]), grid=tuple(grid), views=views,
                    depth_step=cams[0].depth_step)


def config2():
    """128^3, 5 views at 256x256x128, max|u| = 2 cells/step."""
    return render_step()


def config1_small():
    """64^3 grid, one camera 128x128x64, max|u| = 1 (the plain-forward case)."""
    return render_step(grid=(64, 64, 64), views=1, image=(128, 128), depth=64, max_u=1.0)


def plume_chain(grid=(96, 176, 96), frames=120, image=(192, 192), depth=96, up=0.5, noise=0.3, source_sigma=6.0,
                source_amp=0.1, density_seed=0, velocity_seed=5, target_seed=2, target_noise=0.05):
    """The long chain: a plume-aspect grid (D, H, W), inflow source near the bottom
    (y = 8) added every frame, velocity (0, +up, 0) cells/step plus curl noise of
    max ``noise``, one front camera.  The initial density is three blobs in the
    lower half; the targets come from the same chain started from the blobs with
    amplitudes perturbed by ``target_noise`` (rendered by the caller)."""
    D, H, W = grid
    lo = np.array([W * 0.3, H * 0.1, D * 0.3])
    hi = np.array([W * 0.7, H * 0.45, D * 0.7])
    sig = (min(grid) / 16.0, min(grid) / 8.0)
    rho0 = synthetic.gaussian_blobs(grid, n=3, center_lo=lo, center_hi=hi, sigma=sig, seed=density_seed)
    rho0_target = synthetic.gaussian_blobs(grid, n=3, center_lo=lo, center_hi=hi, sigma=sig, seed=density_seed,
                                           amp_noise=target_noise, noise_seed=target_seed)
    ux, uy, uz = synthetic.plume_velocity(grid, up=up, noise=noise, seed=velocity_seed)
    src = synthetic.inflow_source(grid, sigma=source_sigma, amplitude=source_amp, height=min(8.0, H / 4))
    cams = scene.orbit_cameras([depth, image[0], image[1]], [0.0])
    vol = scene.volume_transform(list(grid))
    M = scene.model_params([vol])
    V, P, F = scene.camera_params(cams)
    return Workload(rho0=rho0, rho0_target=rho0_target, ux=ux, uy=uy, uz=uz, source=src, M=M, V=V, P=P, F=F,
                    cameras=cams, image_dhw=(depth, image[0], image[1]), grid=tuple(grid), frames=frames,
                    depth_step=cams[0].depth_step)


def config3():
    """96 x 176 x 96 plume, 120 frames, one 192 x 192 x 96 camera."""
    return plume_chain()


def batched_scenes(n=32, seed=4, sizes=tuple(range(48, 161, 8)), cameras=(1, 8), image_sides=tuple(range(64, 257, 16)),
                   depths=tuple(range(32, 129, 8)), max_u=1.0):
    """Scenes of uneven size: each axis size drawn from ``sizes`` independently,
    1-8 cameras on random yaws, square images with the side from ``image_sides``
    and the depth from ``depths``.  Density blobs, curl-noise velocity and a
    perturbed target density per scene (targets rendered by the caller)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        D, H, W = (int(v) for v in rng.choice(sizes, 3))
        nv = int(rng.integers(cameras[0], cameras[1] + 1))
        side = int(rng.choice(image_sides))
        depth = int(rng.choice(depths))
        yaws = list(rng.uniform(-90.0, 90.0, nv))
        rho = synthetic.gaussian_blobs((D, H, W), n=4, seed=1000 + k)
        rho_t = synthetic.gaussian_blobs((D, H, W), n=4, seed=1000 + k, amp_noise=0.05, noise_seed=2000 + k)
        ux, uy, uz = synthetic.curl_noise_mac((D, H, W), max_u=max_u, seed=3000 + k)
        cams = scene.orbit_cameras([depth, side, side], yaws)
        V, P, F = scene.camera_params(cams)
        M = scene.model_params([scene.volume_transform([D, H, W])])
        out.append(Workload(rho=rho, rho_target=rho_t, ux=ux, uy=uy, uz=uz, M=M, V=V, P=P, F=F,
                            image_dhw=(depth, side, side), grid=(D, H, W), views=nv, depth_step=cams[0].depth_step))
    return out


def config4():
    """32 scenes, axis sizes 48-160, 1-8 cameras, images 64-256, depth 32-128."""
    return batched_scenes()


def algorithmic_bytes(grid, views, image, elem=4):
    """Compulsory HBM bytes of one differentiated step: every tensor that must
    cross HBM counted once at its storage size (density read / advected write /
    read by render forward and backward / its gradient written and read / density
    read and gradient written by the advection backward; velocity read forward
    and backward and its gradient written; images written, read back and the
    targets read).  Intermediates a fused implementation keeps on chip excluded."""
    D, H, W = grid
    n_rho = D * H * W
    n_u = (W + 1) * H * D + W * (H + 1) * D + W * H * (D + 1)
    px = views * image[0] * image[1]
    return elem * (8 * n_rho + 3 * n_u) + 4 * 5 * px
