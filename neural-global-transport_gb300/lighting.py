"""Spot-light shadow transmission of a density grid, differentiable.

The composition of ``SpotLight._render_shadow_map`` (lighting.py:134-177 of the
reference) on the operators of this package:

    shadow density  = resample of density * depth_step into the light's frustum
                      (``sample_camera``, TRANSFORM_LINDEPTH)
    optical depth   = reduce_grid_blend(shadow density, keep_dims=True)
                      (one channel: the cumulative sum along depth)
    shift           = one cell deeper, the new first cell from the boundary rule
                      (BORDER 0, CLAMP the first cell; the transform resample,
                      like the reference's, takes no WRAP)
    transmission    = exp(-depth) (BEER_LAMBERT) or 1 - clip(depth, 0, 1) (ALPHA),
                      times the light's circular cone mask
    light volume    = transmission resampled back onto the grid
                      (``sample_camera(inverse=True)``, TRANSFORM_LINDEPTH_REVERSE)

The resamples and the depth scan are the library's kernels (with their
gradients); the shift, exponential and mask are elementwise tensor glue.
"""
import torch

from . import ops


def cone_mask(height, width, device, dtype=torch.float32):
    """1 inside the unit circle of the light's image plane, 0 outside
    (``SpotLight._get_shadow_mask``): (H, W, 1)."""
    y = torch.linspace(-1.0, 1.0, height, device=device, dtype=dtype)
    x = torch.linspace(-1.0, 1.0, width, device=device, dtype=dtype)
    yy, xx = torch.meshgrid(y, x, indexing="ij")
    return ((yy * yy + xx * xx).sqrt() <= 1.0).to(dtype)[..., None]


def shadow_transmission(density, matrix_m, matrix_v, matrix_p, frustum_params, shadow_dhw, depth_step,
                        blend_mode="BEER_LAMBERT", boundary="BORDER", interpolation="LINEAR", mipmapping="NONE",
                        num_mipmaps=0, mip_bias=0.0, lin_depth=True, use_cone_mask=True):
    """Light transmission on the density grid: density (N, D, H, W, 1), one
    light camera (V, P, F of one row), its frustum grid ``shadow_dhw`` and depth
    step.  Returns (N, D, H, W, 1)."""
    if blend_mode not in ("BEER_LAMBERT", "ALPHA"):
        raise ValueError("Unknown blend_mode '%s'" % blend_mode)
    fwd_mode = "TRANSFORM_LINDEPTH" if lin_depth else "TRANSFORM"
    sd = ops.sample_grid_transform(density * float(depth_step), matrix_m, matrix_v, matrix_p, frustum_params,
                                   shadow_dhw, interpolation=interpolation, boundary=boundary, mipmapping=mipmapping,
                                   num_mipmaps=num_mipmaps, mip_bias=mip_bias, coordinate_mode=fwd_mode)[:, 0]
    sd = ops.reduce_grid_blend(sd.contiguous(), blend_mode, keep_dims=True)
    if boundary == "BORDER":
        pad = torch.zeros_like(sd[:, :1])
    elif boundary == "CLAMP":
        pad = sd[:, :1]
    elif boundary == "WRAP":
        pad = sd[:, -1:]
    else:
        raise ValueError("Unknow boundary_mode %s" % boundary)
    sd = torch.cat([pad, sd[:, :-1]], dim=1)
    if blend_mode == "BEER_LAMBERT":
        tr = torch.exp(-sd)
    else:
        tr = 1.0 - torch.clamp(sd, 0.0, 1.0)
    if use_cone_mask:
        tr = tr * cone_mask(tr.shape[2], tr.shape[3], tr.device, tr.dtype)
    D, H, W = density.shape[1:4]
    out = ops.sample_grid_transform(tr.contiguous(), matrix_m, matrix_v, matrix_p, frustum_params, (D, H, W),
                                    interpolation=interpolation, boundary=boundary, mipmapping="NONE",
                                    coordinate_mode=fwd_mode + "_REVERSE")
    return out[:, 0]
