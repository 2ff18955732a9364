/*
 * ngt_ops.h -- C ABI of the GB300 (sm_103a) differentiable grid operators.
 *
 * Drop-in boundary for the operator layer of Neural-Global-Transport's
 * reconstruction loop (phitest/render/cuda).  Each forward / backward pair
 * replaces one TensorFlow custom op and the gradient registered for it in
 * phitest/render/cuda/ops_loader.py; attribute names and meanings are kept
 * (enums below), shapes follow the ops' NDHWC conventions.
 *
 * Conventions
 *  - All data pointers are device pointers; the library allocates nothing.
 *    Outputs, gradients and any workspace are owned by the caller.  Every
 *    op that needs scratch memory reports its size through the matching
 *    *_workspace_bytes() query.
 *  - Every buffer starts on a multiple of its element size (the storage type
 *    for grids, float -- double for NGT_F64 -- for images, gradients and
 *    scratch fields, float for matrices); workspaces and camera blocks on 16
 *    bytes, prepared quad layouts on 256.  A misaligned pointer is rejected
 *    with NGT_ERR_INVALID_ARGUMENT naming it.  (Allocations from cudaMalloc
 *    or a PyTorch tensor of the element type always qualify.)
 *  - Matrices (model M per batch entry, view V / projection P per camera)
 *    are 16 floats read column-major, exactly the buffer the reference ops
 *    receive (renderer.py:117-121 passes matrix.transpose()); frusta are 6
 *    floats [near, far, left, right, top, bottom] (camera.py:64-65).  They
 *    are read on the device, so a call can be captured in a CUDA graph.
 *  - ``stream`` is a cudaStream_t passed as void*; all work is ordered on it
 *    and no call synchronises the host.
 *  - Return value: NGT_OK or an NGT_ERR_* code; ngt_last_error_message()
 *    describes the last failure of the calling thread.  No call exits or
 *    traps (the reference calls exit(10) on CUDA errors,
 *    kernel_setup.hpp:44-50).
 *  - Gradients come in two semantics: NGT_GRAD_EXACT is the true adjoint of
 *    the forward; NGT_GRAD_REFERENCE reproduces the reference's registered
 *    gradients (per-voxel division by sample counts / summed sample weights,
 *    resample_grid.cu.cc:1133-1151, raymarch_grid.cu.cc:458-480, and the
 *    raymarch backward's own sampling positions, raymarch_grid.cu.cc:508-518).
 */
#ifndef NGT_OPS_H
#define NGT_OPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define NGT_OK 0
#define NGT_ERR_INVALID_ARGUMENT 1 /* shape, channel count, enum or pointer rejected */
#define NGT_ERR_UNSUPPORTED 2      /* valid but unsupported combination */
#define NGT_ERR_CUDA 3             /* a CUDA launch or copy failed */
#define NGT_ERR_WORKSPACE 4        /* workspace missing or too small */

/* ------------------------------------------------------------------ enums */
/* storage type of grids / images; arithmetic is float32 (float64 for F64) */
enum { NGT_F32 = 0, NGT_F64 = 1, NGT_BF16 = 2, NGT_F16 = 3 };
/* attr interpolation (resample_grid.cc:32,100; raymarch_grid.cc:37) */
enum { NGT_NEAREST = 0, NGT_LINEAR = 1, NGT_MIN = 2, NGT_MAX = 3, NGT_QUADRATIC = 4 };
/* attr boundary (resample_grid.cc:33,101; raymarch_grid.cc:38) */
enum { NGT_BORDER = 0, NGT_CLAMP = 1, NGT_WRAP = 2 };
/* attr mipmapping (resample_grid.cc:34) */
enum { NGT_MIP_NONE = 0, NGT_MIP_NEAREST = 1, NGT_MIP_LINEAR = 2 };
/* attr blending_mode (raymarch_grid.cc:44, reduce_blend.cc:26) */
enum { NGT_BEER_LAMBERT = 0, NGT_ALPHA = 2, NGT_ALPHA_ADDITIVE = 3, NGT_ADDITIVE = 4 };
/* attr coordinate_mode (resample_grid.cc:40) */
enum { NGT_TRANSFORM_LINDEPTH = 0, NGT_TRANSFORM_LINDEPTH_REVERSE = 1, NGT_TRANSFORM = 3,
       NGT_TRANSFORM_REVERSE = 4 };
/* gradient semantics */
enum { NGT_GRAD_EXACT = 0, NGT_GRAD_REFERENCE = 1 };
/* advection clamp (data_structures.py:1715-1735); MC_SMOOTH, MacCormack's
 * limiter, has no effect with order 1 */
enum { NGT_CLAMP_NONE = 0, NGT_CLAMP_MC_SMOOTH = 1, NGT_CLAMP_NEGATIVE = 2 };

/* ------------------------------------------------------------ LUT resample */
/* Replaces op SampleGridLut (resample_grid.cc:94-120, 742-899) and its
 * gradient op SampleGridLutGrad (resample_grid.cc:124-150, 925-1081) as
 * registered in ops_loader.py:41-60. */
typedef struct {
  int32_t dtype;              /* NGT_F32 or NGT_F64 (lookup uses the same type) */
  int64_t input_shape[5];     /* N, D, H, W, C with C in {1, 2, 4} */
  int64_t lookup_shape[5];    /* V, D', H', W', 4 (x, y, z, LoD) */
  const void* input;          /* NDHWC */
  const void* lookup;         /* V D' H' W' 4 */
  void* output;               /* N, V (1 unless separate_camera_batch), D', H', W', C */
  int32_t interpolation;      /* NEAREST, LINEAR, MIN, MAX */
  int32_t boundary;           /* BORDER, CLAMP, WRAP */
  int32_t mipmapping;         /* NONE, NEAREST, LINEAR */
  int32_t num_mipmaps;
  float mip_bias;
  float cell_center_offset;   /* default 0.0; must be 0.5 with normalized coordinates */
  int32_t separate_camera_batch;
  int32_t relative_coords;
  int32_t normalized_coords;
  void* workspace;            /* mip pyramid when mipmapping != NONE */
  size_t workspace_bytes;
} ngt_sample_lut_args;

typedef struct {
  ngt_sample_lut_args fwd;    /* the forward call's arguments (fwd.output unused) */
  const void* output_grad;    /* shape of fwd.output */
  void* input_grad;           /* shape of fwd.input */
  void* lookup_grad;          /* shape of fwd.lookup; may be null */
  int32_t grad_mode;          /* NGT_GRAD_EXACT / NGT_GRAD_REFERENCE */
  int32_t deterministic;      /* exact LINEAR only: gather form, bit-reproducible input gradient */
  void* workspace;            /* sample counts (reference mode) / gather buckets (deterministic) */
  size_t workspace_bytes;
} ngt_sample_lut_grad_args;

int ngt_sample_lut_fwd(const ngt_sample_lut_args* args, void* stream);
size_t ngt_sample_lut_fwd_workspace_bytes(const ngt_sample_lut_args* args);
int ngt_sample_lut_bwd(const ngt_sample_lut_grad_args* args, void* stream);
size_t ngt_sample_lut_bwd_workspace_bytes(const ngt_sample_lut_grad_args* args);

/* ------------------------------------------------------ transform resample */
/* Replaces op SampleGridTransform (resample_grid.cc:23-65, 316-516) and
 * SampleGridTransformGrad (resample_grid.cc:68-92, 538-717) as registered in
 * ops_loader.py:19-39. */
typedef struct {
  int32_t dtype;              /* NGT_F32 or NGT_F64 */
  int64_t input_shape[5];     /* N, D, H, W, C with C in {1, 2, 4} */
  int64_t output_dhw[3];      /* D', H', W' of the sampled grid */
  const void* input;
  const float* matrix_m;      /* N x 16 */
  const float* matrix_v;      /* V x 16 */
  const float* matrix_p;      /* V x 16 */
  const float* frustum;       /* V x 6 */
  int32_t num_cameras;        /* V */
  void* output;               /* N, V (1 unless separate_camera_batch), D', H', W', C */
  int32_t interpolation;      /* NEAREST, LINEAR, QUADRATIC */
  int32_t boundary;           /* BORDER, CLAMP */
  int32_t mipmapping;
  int32_t num_mipmaps;
  float mip_bias;
  float cell_center_offset;   /* default 0.5 */
  int32_t coordinate_mode;
  int32_t separate_camera_batch;
  void* workspace;            /* mip pyramid when mipmapping != NONE */
  size_t workspace_bytes;
} ngt_sample_transform_args;

typedef struct {
  ngt_sample_transform_args fwd;
  const void* output_grad;
  void* input_grad;
  int32_t grad_mode;
  void* workspace;            /* per-voxel sample counts (reference mode) / cameras and
                                 gather buckets (deterministic) */
  size_t workspace_bytes;
  /* Exact LINEAR mode: nonzero computes the input gradient in gather form
   * (bit-reproducible): the frustum samples are bucketed by the cell of their
   * lower corner (counting sort) and every voxel sums the samples of its 8
   * neighbouring buckets in sample order, in place of the reference's float
   * atomics (resample_grid.cu.cc:1160-1190).  Fewer than 2^31 samples per
   * batch entry. */
  int32_t deterministic;
} ngt_sample_transform_grad_args;

int ngt_sample_transform_fwd(const ngt_sample_transform_args* args, void* stream);
size_t ngt_sample_transform_fwd_workspace_bytes(const ngt_sample_transform_args* args);
int ngt_sample_transform_bwd(const ngt_sample_transform_grad_args* args, void* stream);
size_t ngt_sample_transform_bwd_workspace_bytes(const ngt_sample_transform_grad_args* args);

/* Mip pyramid of a grid (MipAtlas3D, resample_grid.cu.cc:116-251): levels 1..L
 * written back to back into ``pyramid`` (each level (D>>l, H>>l, W>>l, C)). */
int ngt_mip_build(int32_t dtype, const int64_t input_shape[5], const void* input, int32_t levels, void* pyramid,
                  size_t pyramid_bytes, void* stream);
size_t ngt_mip_bytes(int32_t dtype, const int64_t input_shape[5], int32_t levels);

/* Replaces op LodTransform (resample_grid.cc:152-172, 1089-1178): per camera a
 * lookup table (x, y, z, LoD) of the sampling positions of a transform resample. */
typedef struct {
  int64_t input_dhw[3];       /* grid sampled from */
  int64_t output_dhw[3];      /* grid sampled to */
  const float* matrix_mv;     /* V x 16 model-view */
  const float* matrix_p;      /* V x 16 */
  const float* frustum;       /* V x 6 */
  int32_t num_cameras;
  int32_t inverse_transform;
  int32_t linearize_depth;
  int32_t relative_coords;
  float* output;              /* V, D', H', W', 4 (float32) */
} ngt_lod_args;
int ngt_lod_transform(const ngt_lod_args* args, void* stream);

/* ------------------------------------------------------------ fused raymarch */
/* Replaces op RaymarchGridTransform (raymarch_grid.cc:29-63, 186-320) and
 * RaymarchGridTransformGrad (raymarch_grid.cc:67-92, 342-504) as registered in
 * ops_loader.py:73-95. */
typedef struct {
  int32_t dtype;              /* NGT_F32, NGT_F64, NGT_BF16, NGT_F16 (storage of input) */
  int64_t input_shape[5];     /* N, D, H, W, C with C in {1, 2, 4} */
  int64_t output_dhw[3];      /* depth samples D', image H', W' */
  const void* input;
  const float* matrix_m;      /* N x 16 */
  const float* matrix_v;      /* V x 16 */
  const float* matrix_p;      /* V x 16 */
  const float* frustum;       /* V x 6 */
  int32_t num_cameras;
  void* output;               /* N, V (1 unless separate_camera_batch), H', W', Cb (float32/64) */
  int32_t interpolation;      /* NEAREST, LINEAR, MIN, MAX (gradient: LINEAR) */
  int32_t boundary;
  int32_t blending_mode;
  int32_t keep_dims;          /* output N, V, 1, H', W', Cb */
  int32_t separate_camera_batch;
  /* Emission expansion: with emission_channels = Cb > 0 the input has one
   * channel (density) and the blend sees Cb channels, channel c being
   * emission_scale[c] * sample.  This is the renderer's light grid
   * [rho*c*i*step, rho*step] (lighting.py:26-34, renderer.py:533-548,763)
   * formed on the fly instead of materialised. 0 = off (Cb = C). */
  int32_t emission_channels;
  float emission_scale[4];
  /* Forward scratch for the quad gather layout of a one-channel LINEAR input
   * (size from ngt_raymarch_fwd_workspace_bytes; null: direct gathers, same
   * results).  Unused by the backward, which takes its own workspace. */
  void* workspace;
  size_t workspace_bytes;
  /* Optional: the per-(batch, camera) transforms already formed by
   * ngt_raymarch_cameras for these matrices (static cameras across calls).
   * Null: formed on every call.  Used by forward and backward. */
  const void* cameras;
  /* Optional: this input in the quad gather layout, prepared by
   * ngt_raymarch_quad (one-channel LINEAR input in float or 16-bit storage)
   * and valid while the input is unchanged.  Forward and exact backward read it
   * instead of building their own.  Null: built per call.  The batch entry
   * points build their own and reject it. */
  const void* quad;
  /* Optional: every ray's start, step and sample count, prepared by
   * ngt_raymarch_rays for these matrices, frustum, image and grid sizes and
   * boundary (static cameras across calls).  Those are set up in double
   * precision and rounded once, so the march starts from the float nearest the
   * exact start; null: set up per ray in float arithmetic.  Used by the forward
   * and the exact backward.  With up to 4096 (camera, 16x8-pixel tile) items the
   * table also holds the items ordered by their rays' summed sample counts, and
   * the forward and the one-pass backward start the longest items first. */
  const void* rays;
  /* Optional, with a prepared quad layout and a ray table: nonzero reserves in
   * the quad buffer (ngt_raymarch_quad_bytes grows by (batch, camera) slots x
   * 16x8-pixel tiles x 128 rays x D' floats) room for every ray's first D'
   * density samples.  A Beer-Lambert forward with emission through that buffer
   * stores them (a warp's 32 rays interleaved: 128 contiguous bytes per step)
   * and tags the buffer with its ray table's address and its sizes; the
   * one-pass exact backward of the same quad buffer, ray table and sizes reads
   * them instead of gathering each sample's corners again.  ngt_raymarch_quad
   * clears the tag; the buffer must be sized (ngt_raymarch_quad_bytes) with the
   * args of the calls that use it, as for the quad layout itself.  The samples
   * are the forward's own values, so the gradient is unchanged.  0: the
   * backward gathers. */
  int32_t sample_cache;
} ngt_raymarch_args;

typedef struct {
  ngt_raymarch_args fwd;
  const void* output;         /* the forward's output */
  const void* output_grad;    /* same shape */
  void* input_grad;           /* shape of fwd.input (float32/64) */
  int32_t grad_mode;
  void* workspace;            /* reference mode: gradient buffer + sample-weight sums;
                                 exact mode: an extinction-sign flag (Beer-Lambert)
                                 and, for a one-channel float / 16-bit input, the
                                 quad layout and its gradient accumulator (size
                                 from ngt_raymarch_bwd_workspace_bytes; 256 bytes
                                 select direct gathers and scatters) */
  size_t workspace_bytes;
  /* Exact mode: nonzero adds the input gradient to input_grad instead of
   * writing it (a gradient summed over several renders of one grid, e.g. the
   * frames of a chain).  The reference's ops write their outputs. */
  int32_t accumulate;
  /* Exact mode: nonzero makes the input gradient bit-reproducible.  The
   * reference's scatter (raymarch_grid.cu.cc:482-521) adds float atomics in
   * an order that varies from run to run; here every sample's contribution is
   * rounded to a 64-bit fixed-point integer whose scale a first pass over the
   * rays chooses (the largest contribution times the ray-sample count stays
   * below 2^62, so no sum overflows and each contribution is resolved to
   * 2^-36 of the largest at 2^26 samples), the integers are summed with
   * integer atomics (associative: the same sums in every run) and converted
   * once.  Samples read through fwd.quad when one is prepared (the same
   * values), else gathered directly; two passes over the rays; the workspace
   * holds one 64-bit integer per input cell and channel. */
  int32_t deterministic;
} ngt_raymarch_grad_args;

size_t ngt_raymarch_fwd_workspace_bytes(const ngt_raymarch_args* args);
/* Forms the camera block of args' matrices into ``cameras`` (device memory of
 * ngt_raymarch_cameras_bytes bytes); no counterpart in the reference, whose
 * launchers upload and invert the matrices per call (raymarch_grid.cu.cc:411-415). */
size_t ngt_raymarch_cameras_bytes(const ngt_raymarch_args* args);
int ngt_raymarch_cameras(const ngt_raymarch_args* args, void* cameras, void* stream);
int ngt_raymarch_fwd(const ngt_raymarch_args* args, void* stream);
/* The quad gather layout of args' input (each cell's 2x2 (x, y) neighbours per z
 * slab, the boundary rule applied), prepared once for the forward and the
 * backward of the same input, which then skip their own builds; it holds the
 * extinction-sign word of the one-pass Beer-Lambert adjoint, taken with args'
 * emission scale.  ``quad``: device memory of ngt_raymarch_quad_bytes bytes,
 * 256-byte aligned.  ngt_raymarch_quad_bytes is 0 for inputs the layout does
 * not serve (several channels, NEAREST / MIN / MAX, F64), for which
 * ngt_raymarch_quad fails with NGT_ERR_UNSUPPORTED.  No counterpart in the
 * reference, whose kernels gather the eight corners per sample
 * (sampling_v2.hpp:37-124). */
/* The ray table of args (32 bytes per (batch, camera) slot and pixel, then the
 * item order; 16-byte aligned): the ray set-up of getRaymarchStep /
 * RayGridIntersectionDistances (raymarch_grid.cu.cc:109-200) in double
 * precision, rounded to the float start and step the march accumulates.  No
 * counterpart in the reference, which sets up every ray in float arithmetic in
 * each kernel. */
size_t ngt_raymarch_rays_bytes(const ngt_raymarch_args* args);
int ngt_raymarch_rays(const ngt_raymarch_args* args, void* rays, void* stream);
size_t ngt_raymarch_quad_bytes(const ngt_raymarch_args* args);
int ngt_raymarch_quad(const ngt_raymarch_args* args, void* quad, void* stream);
int ngt_raymarch_bwd(const ngt_raymarch_grad_args* args, void* stream);
size_t ngt_raymarch_bwd_workspace_bytes(const ngt_raymarch_grad_args* args);
/* A render's forward, its image L2 loss and its backward in one call:
 * ngt_raymarch_fwd_l2 (or ngt_raymarch_fwd_l2_background with a non-null
 * ``background``) writing the image to args->output and the loss gradient to
 * args->output_grad (both written here), then ngt_raymarch_bwd of that gradient
 * into args->input_grad.  For the exact float-atomic Beer-Lambert adjoint with
 * emission of a one-channel LINEAR input in float or 16-bit storage this is one
 * launch: the loss gradient of a pixel depends on that pixel alone, so each
 * thread marches its ray forward and back in turn, the image is not read back,
 * and the samples cached on the way (sample_cache) are read by the same
 * thread.  Other settings run the two passes (args->fwd.workspace then serves
 * the forward).  Workspace and other fields as ngt_raymarch_bwd.  No reference
 * counterpart: the renderer runs the op, the loss and the registered gradient
 * as three TF ops (renderer.py:718-827, optimization.py:478). */
int ngt_raymarch_fwd_l2_bwd(const ngt_raymarch_grad_args* args, const void* background, const void* target,
                            int32_t loss_channels, void* loss, void* stream);
/* ngt_raymarch_bwd for callers that cannot allocate device memory -- a host
 * program whose own pool owns the whole device, or a loop that may not allocate
 * once it runs.  No counterpart in the reference.  args->workspace is ignored:
 * the scratch is a 16 MiB static device array that every GPU using the library
 * holds until exit, shared by all calls and keeping the last call's contents
 * (each call clears what must start at zero).  Calls needing more (see
 * ngt_raymarch_bwd_workspace_bytes) fail with NGT_ERR_WORKSPACE.  Each call made
 * outside a stream capture looks up the array's device address in the current
 * context; a call under capture reuses the last address found on its device, so
 * the first call on a device (and the first after a device reset) must come
 * before any stream capture.  Calls whose GPU work overlaps race on the array. */
int ngt_raymarch_bwd_static(const ngt_raymarch_grad_args* args, void* stream);

/* ------------------------------------------------------------ reduce blend */
/* Replaces op ReduceGridBlend / ReduceGridBlendGrad (reduce_blend.cc:24-56,
 * 68-252) as registered in ops_loader.py:64-69. */
typedef struct {
  int32_t dtype;              /* NGT_F32 or NGT_F64 */
  int64_t input_shape[5];     /* N, D, H, W, C */
  const void* input;
  void* output;               /* N, H, W, C or N, D, H, W, C with keep_dims */
  int32_t blending_mode;
  int32_t keep_dims;
} ngt_reduce_blend_args;

typedef struct {
  ngt_reduce_blend_args fwd;
  const void* output;
  const void* output_grad;
  void* input_grad;
  int32_t grad_mode;
} ngt_reduce_blend_grad_args;

int ngt_reduce_blend_fwd(const ngt_reduce_blend_args* args, void* stream);
int ngt_reduce_blend_bwd(const ngt_reduce_blend_grad_args* args, void* stream);

/* ------------------------------------------------------ MacCormack advection */
/* Fused semi-Lagrangian / MacCormack warp of a cell-centred grid by a
 * MAC-staggered velocity.  Replaces the TensorFlow composition of
 * VelocityGrid.warp (data_structures.py:1690-1737: centred velocity, LUT
 * sample forward, LUT sample back, correction, MIN / MAX lookups, revert
 * clamp) -- four SampleGridLut calls and their registered gradients. */
typedef struct {
  int32_t dtype;              /* NGT_F32, NGT_F64, NGT_BF16, NGT_F16 (storage) */
  int64_t grid_dhw[3];        /* D, H, W of the advected grid */
  int32_t channels;           /* C in {1, 2, 4} */
  const void* data;           /* D, H, W, C */
  const void* vel_x;          /* D, H, W+1 */
  const void* vel_y;          /* D, H+1, W */
  const void* vel_z;          /* D+1, H, W */
  float dt;
  int32_t order;              /* 1 semi-Lagrangian, 2 MacCormack */
  int32_t clamp;              /* NGT_CLAMP_* */
  int32_t boundary;           /* BORDER, CLAMP, WRAP (configs: CLAMP) */
  void* output;               /* D, H, W, C */
  void* fwd_field;            /* D, H, W, C scratch written by the forward (order 2), read by the backward */
  /* Optional, MacCormack with MC_SMOOTH: one byte per cell and channel, the
   * forward's revert mask (1 where the correction left the corners' range);
   * the backward then reads it instead of re-gathering the corner extrema.
   * Null: recomputed.  No reference counterpart (TF keeps the tf.where mask). */
  void* mask;
  /* Optional, MacCormack with MC_SMOOTH: scratch of 2 x C compute-type values
   * per cell (float, double for F64) where forward 1 leaves the forward trace's
   * corner extrema, taken from the same corner fetch as its trilinear value;
   * forward 2 (and a backward without a stored mask) reads them instead of
   * gathering the eight corners again.  Null: gathered again.  No reference
   * counterpart. */
  void* extrema;
  /* Optional scratch of 3 compute-type values per cell, kept for the backward
   * like fwd_field: forward 1 stores the lookup (centred velocity times -dt)
   * there and forward 2 and the backward read it instead of averaging the
   * faces again.  Null: averaged in every kernel.  No reference counterpart. */
  void* lookup;
  /* Storage of the three face grids when it differs from dtype: NGT_F16 faces
   * with NGT_BF16 data (BF16's exponent range keeps the near-empty tails of a
   * density that the limiter compares, FP16's mantissa keeps four times finer
   * velocities and so trace positions).  NGT_F32 (0): the faces are stored as
   * dtype.  Single-grid calls only. */
  int32_t velocity_dtype;
} ngt_advect_args;

typedef struct {
  ngt_advect_args fwd;        /* fwd.output unused; fwd.fwd_field as written by the forward */
  const void* output_grad;
  void* data_grad;            /* D, H, W, C */
  void* vel_x_grad;           /* face grids, may all be null */
  void* vel_y_grad;
  void* vel_z_grad;
  int32_t grad_mode;
  int32_t deterministic;      /* exact mode: 64-bit fixed-point trace adjoints, bit-reproducible gradients */
  void* workspace;
  size_t workspace_bytes;
  /* Exact, non-deterministic mode: nonzero adds the data and velocity
   * gradients to data_grad and vel_*_grad instead of writing them. */
  int32_t accumulate;
} ngt_advect_grad_args;

int ngt_advect_maccormack_fwd(const ngt_advect_args* args, void* stream);
int ngt_advect_maccormack_bwd(const ngt_advect_grad_args* args, void* stream);
size_t ngt_advect_maccormack_bwd_workspace_bytes(const ngt_advect_grad_args* args);

/* Self-advection of the MAC velocity: every face component is warped on its own
 * staggered lattice by the velocity resampled onto that lattice (the other two
 * components read at +-1/2 cell offsets).  Replaces VelocityGrid.warped
 * (data_structures.py:1108-1164, with _sampled_to_component_shape :1655-1682 and
 * _warp_vel_component :1081-1106): per component two resample_grid3D_offset
 * calls (renderer.py:922-936) and four SampleGridLut calls.  The three warps all
 * read the incoming velocity. */
typedef struct {
  int32_t dtype;              /* NGT_F32, NGT_F64, NGT_BF16, NGT_F16 */
  int64_t grid_dhw[3];        /* cell grid D, H, W */
  const void* vel_x;          /* D, H, W+1 */
  const void* vel_y;          /* D, H+1, W */
  const void* vel_z;          /* D+1, H, W */
  float dt;
  int32_t order;
  int32_t clamp;
  int32_t boundary;
  void* out_x;                /* warped components, shapes as the inputs */
  void* out_y;
  void* out_z;
  void* fwd_x;                /* per-component fwd fields (compute type), kept for the backward */
  void* fwd_y;
  void* fwd_z;
  /* Optional scratch per face component (x, y, z), kept from the forward to the
   * backward like fwd_*: lookup (3 compute-type values per face: the velocity
   * resampled onto that component's lattice, times -dt), written by forward 1
   * and read by forward 2 and the backward instead of being resampled again;
   * mask (the MC_SMOOTH revert mask, 1 byte per face) and extrema (2
   * compute-type values per face) as in ngt_advect_args.  Null: recomputed.
   * No reference counterpart. */
  void* lookup[3];
  void* mask[3];
  void* extrema[3];
} ngt_advect_velocity_args;

typedef struct {
  ngt_advect_velocity_args fwd;
  const void* grad_x;         /* gradients of the warped components */
  const void* grad_y;
  const void* grad_z;
  void* vel_x_grad;           /* gradients w.r.t. the incoming components */
  void* vel_y_grad;
  void* vel_z_grad;
  int32_t grad_mode;
  void* workspace;
  size_t workspace_bytes;
  /* Exact mode: nonzero takes each component's trace adjoints as 64-bit
   * fixed-point sums (bit-reproducible gradients, as for the density). */
  int32_t deterministic;
} ngt_advect_velocity_grad_args;

int ngt_advect_velocity_fwd(const ngt_advect_velocity_args* args, void* stream);
int ngt_advect_velocity_bwd(const ngt_advect_velocity_grad_args* args, void* stream);
size_t ngt_advect_velocity_bwd_workspace_bytes(const ngt_advect_velocity_grad_args* args);

/* ------------------------------------------------------------------ batches */
/* Many scenes of different grid, image and depth sizes per call (no
 * counterpart in the reference, whose ops take one grid shape per call and are
 * called once per scene).  Each scene's arguments are those of the single-scene
 * call; up to 32 scenes, sharing dtype and channel layout.
 *
 * Raymarch: one persistent launch per pass; blocks take (scene, camera, 16x8
 * ray tile) work items from a counter, largest scenes first.  ``blocks_per_sm``
 * sets the persistent grid (0: default), the knob an autotuner sets.  Workspace
 * from ngt_raymarch_batch_workspace_bytes (work counters, per-scene flags, the
 * cameras of scenes without a prepared ``cameras`` block).  The backward takes
 * exact Beer-Lambert gradients of LINEAR sampling (one-pass for scenes with
 * non-negative extinction, checkpointed otherwise); input gradients are float. */
size_t ngt_raymarch_batch_workspace_bytes(const ngt_raymarch_args* scenes, int32_t count);
int ngt_raymarch_fwd_batch(const ngt_raymarch_args* scenes, int32_t count, int32_t blocks_per_sm, void* workspace,
                           size_t workspace_bytes, void* stream);
int ngt_raymarch_bwd_batch(const ngt_raymarch_grad_args* scenes, int32_t count, int32_t blocks_per_sm,
                           void* workspace, size_t workspace_bytes, void* stream);
/* ngt_raymarch_bwd_batch for the scenes whose ngt_raymarch_fwd_batch ran last on
 * this workspace (same arguments, inputs unchanged since): the quad layouts and
 * extinction-sign words that forward left in the workspace are used instead of
 * being built again.  No counterpart in the reference. */
int ngt_raymarch_bwd_batch_after_fwd(const ngt_raymarch_grad_args* scenes, int32_t count, int32_t blocks_per_sm,
                                     void* workspace, size_t workspace_bytes, void* stream);
/* The batched render's forward, image L2 loss and backward in one persistent
 * launch: every (scene, camera, tile) item is marched forward (image written to
 * the scene's output, loss gradient to its output_grad, 0.5 * the summed squared
 * difference of the first loss_channels channels to ``targets[i]`` (the scene's
 * H' x W' x loss_channels per camera) added to *loss) and back by the same
 * threads, since a pixel's loss gradient depends on that pixel alone; then the
 * folds.  Scenes as ngt_raymarch_bwd_batch, and one-channel LINEAR density with
 * emission channels in float or 16-bit storage (the quad layout); workspace of
 * ngt_raymarch_batch_workspace_bytes.  Replaces ngt_raymarch_fwd_batch +
 * ngt_image_l2_loss + ngt_raymarch_bwd_batch_after_fwd.  No reference
 * counterpart (the reference renders one scene per op call). */
int ngt_raymarch_fwd_l2_bwd_batch(const ngt_raymarch_grad_args* scenes, const void* const* targets, int32_t count,
                                  int32_t loss_channels, void* loss, int32_t blocks_per_sm, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* Density warps of many grids: one launch per phase over the concatenated z
 * planes.  The backward takes exact, non-deterministic gradients with all three
 * face gradients; workspace from ngt_advect_maccormack_bwd_batch_workspace_bytes
 * (args' own workspace fields are ignored). */
int ngt_advect_maccormack_fwd_batch(const ngt_advect_args* grids, int32_t count, void* stream);
size_t ngt_advect_maccormack_bwd_batch_workspace_bytes(const ngt_advect_grad_args* grids, int32_t count);
int ngt_advect_maccormack_bwd_batch(const ngt_advect_grad_args* grids, int32_t count, void* workspace,
                                    size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------ step helpers */
/* Image loss of the reconstruction step, 0.5 * sum over pixels of
 * (image[..., c] - target[..., c])^2 for the first ``loss_channels`` channels
 * (loss_dens_target, optimization.py:478, on the rendered light channel).
 * Writes the image gradient (zero in the remaining channels) and adds the loss
 * to *loss (device scalar of the image dtype, float or double; zero it first).
 * No reference counterpart as a single call: the reference forms this loss
 * with TensorFlow ops. */
int ngt_image_l2_loss(int32_t dtype, int64_t pixels, int32_t channels, int32_t loss_channels, const void* image,
                      const void* target, void* image_grad, void* loss, void* stream);
/* ngt_raymarch_fwd with ngt_image_l2_loss fused into its epilogue: each ray's
 * pixel, once blended, also writes its image gradient (target: loss_channels
 * per pixel; image_grad: the output's shape) and the loss is added to *loss per
 * block (zero it first).  One launch instead of two; the loss differs from the
 * separate call's only by the order of its additions.  No reference
 * counterpart (see ngt_image_l2_loss). */
int ngt_raymarch_fwd_l2(const ngt_raymarch_args* args, const void* target, int32_t loss_channels, void* image_grad,
                        void* loss, void* stream);

/* Background composite of the render composition, replacing the TensorFlow
 * ops of Renderer.render_density (renderer.py:779-781, 804-806): with t =
 * exp(-d) the transmittance of each ray (d the image's last, optical-depth
 * channel) the camera's background shows through behind the light channels,
 * output_c = image_c + background_c * t, and the depth channel is cut
 * (cut_alpha).  image: batch x pixels x C (C in {2, 4}; pixels = V * H * W);
 * background: pixels x (C - 1), shared by the batch entries; output: batch x
 * pixels x (C - 1).  F32 or F64.  The backward writes image_grad (the light
 * channels' gradient, and -t * sum_c background_c * g_c in the depth channel)
 * and, if background_grad is not null, the background's gradient (summed over
 * the batch). */
int ngt_background_composite(int32_t dtype, int64_t batch, int64_t pixels, int32_t channels, const void* image,
                             const void* background, void* output, void* stream);
int ngt_background_composite_bwd(int32_t dtype, int64_t batch, int64_t pixels, int32_t channels, const void* image,
                                 const void* background, const void* output_grad, void* image_grad,
                                 void* background_grad, void* stream);
/* ngt_raymarch_fwd_l2 with that composite in its epilogue: the loss compares
 * the composited light channels (background: cameras x H' x W' x (Cb - 1), per
 * camera, shared by the batch; Beer-Lambert blending) with the target, and
 * image_grad receives the gradient with respect to the raw output [light, d]
 * (what ngt_raymarch_bwd takes), the depth channel's being -t * sum_c
 * background_c * g_c.  The raw render stays in args->output.  loss_channels is
 * at most Cb - 1.  No reference counterpart as a single call (see
 * ngt_image_l2_loss). */
int ngt_raymarch_fwd_l2_background(const ngt_raymarch_args* args, const void* background, const void* target,
                                   int32_t loss_channels, void* image_grad, void* loss, void* stream);

/* ------------------------------------------------------------ diagnostics */
const char* ngt_last_error_message(void);
int ngt_version(void);
/* sizeof of the argument struct named ``name`` (e.g. "ngt_raymarch_args"), 0 for
 * an unknown name: lets a binding check its mirror of the layouts. */
size_t ngt_struct_size(const char* name);
/* Bounded waits.  A kernel that waits for an asynchronous copy (the MacCormack
 * forward's TMA-staged bricks of the fwd field) gives up after a bounded number
 * of polls, counts the event, finishes with plain global-memory reads (the same
 * results) and waits again, bounded, for its copy before it leaves.
 * ngt_wait_timeouts copies the count into *count (synchronising the device) and
 * clears it when reset is non-zero.  ngt_set_wait_polls sets the poll limit of
 * the first wait (default 4194304; 0 makes every first wait give up at once, a
 * way to exercise the path; negative restores the default) and returns the
 * previous limit.  No reference counterpart (its kernels do not wait). */
int ngt_wait_timeouts(uint64_t* count, int32_t reset);
int32_t ngt_set_wait_polls(int32_t polls);

#ifdef __cplusplus
}
#endif
#endif /* NGT_OPS_H */
