"""The grid operators with the reference's call signatures.

Mirrors ``sampling_ops``, ``raymarching_ops`` and ``blending_ops`` of
``phitest/render/cuda/ops_loader.py``: the same keyword names and attribute
strings, NDHWC tensors, matrices as 16 floats read column-major (callers pass
``matrix.transpose()`` exactly as ``renderer.py:117-121`` does).  Every forward
is a ``torch.autograd.Function`` whose backward is the matching gradient op, so
``torch.autograd`` plays the role of the gradients registered in ops_loader.py.

Gradient semantics: ``set_gradient_mode("exact")`` (default, the true adjoint)
or ``"reference"`` (the reference's count / weight normalised gradients).

All tensors must be contiguous CUDA tensors; there is no CPU path.
"""
import collections
import contextlib
import ctypes
import functools

import numpy as np
import torch

from . import _lib as L

_GRAD_MODE = ["exact"]
_DETERMINISTIC = [False]


def set_deterministic(flag):
    """Bit-reproducible input gradients in exact mode: the gather form for the
    LUT and transform resamples, fixed-point integer accumulation for the
    advection of density and velocity and for the raymarch."""
    _DETERMINISTIC[0] = bool(flag)


def get_deterministic():
    return _DETERMINISTIC[0]


def set_gradient_mode(mode):
    if mode not in L.GRAD:
        raise ValueError("gradient mode must be 'exact' or 'reference'")
    _GRAD_MODE[0] = mode


def get_gradient_mode():
    return _GRAD_MODE[0]


@contextlib.contextmanager
def gradient_mode(mode):
    old = get_gradient_mode()
    set_gradient_mode(mode)
    try:
        yield
    finally:
        set_gradient_mode(old)


# ------------------------------------------------------------------ helpers
_DTYPES = {torch.float32: L.F32, torch.float64: L.F64, torch.bfloat16: L.BF16, torch.float16: L.F16}


def _code(t):
    if t.dtype not in _DTYPES:
        raise TypeError("unsupported dtype %s" % t.dtype)
    return _DTYPES[t.dtype]


def compute_dtype(t):
    return torch.float64 if t.dtype == torch.float64 else torch.float32


def _cuda(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor (the operators have no CPU path)" % name)
    return t.contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


# the current stream's handle of a device; the raw accessor skips the argument
# parsing of torch.cuda.current_stream, a noticeable share of a call's host time
_RAW_STREAM = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def _stream_handle(index=None):
    if index is None:
        index = torch.cuda.current_device()
    if _RAW_STREAM is not None:
        return int(_RAW_STREAM(index))
    return torch.cuda.current_stream(index).cuda_stream


def _stream():
    return ctypes.c_void_p(_stream_handle())


def _enum(table, value, name):
    v = value.decode() if isinstance(value, bytes) else value
    if v not in table:
        raise ValueError("invalid %s '%s'" % (name, value))
    return table[v]


# Device copies of host matrices, by content, and camera blocks formed from them
# (cameras are usually the same from one call to the next).  Entries are made on
# the caller's stream; a call on another stream waits for that stream's event.
_CACHE_SIZE = 32
_HOST_MATS = collections.OrderedDict()  # (shape, bytes, width, device) -> (tensor, event, stream)
_CAMERAS = collections.OrderedDict()    # (ids of cached matrices, slots) -> (block, event, stream, matrices)
_RAYS = collections.OrderedDict()       # (ids of cached matrices, slots, sizes, boundary) -> (table, event, stream, ...)


def _cache_put(cache, key, value):
    cache[key] = value
    if len(cache) > _CACHE_SIZE:
        cache.popitem(last=False)


def _cache_get(cache, key):
    hit = cache.get(key)
    if hit is None:
        return None
    cache.move_to_end(key)
    index = hit[0].device.index
    if _stream_handle(index) != hit[2]:
        stream = torch.cuda.current_stream(index)
        stream.wait_event(hit[1])
        # an entry evicted while this stream still reads it must not be reused early
        hit[0].record_stream(stream)
    return hit[0]


def _recorded(t):
    ev = torch.cuda.Event()
    stream = torch.cuda.current_stream(t.device)
    ev.record(stream)
    return ev, stream.cuda_stream


def _floats(m, width, device):
    """Matrices / frusta as the contiguous float32 device buffer the kernels read:
    the C-order flattening of what the caller passed, ``width`` floats per entry.

    Host arrays are uploaded once per content and device (through pinned memory
    with a stream-ordered copy: a copy from pageable memory would first wait for
    all work queued on the stream) and the device copy is reused."""
    device = torch.device(device)
    if device.type == "cuda" and device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    if isinstance(m, torch.Tensor):
        return m.detach().to(device=device, dtype=torch.float32, non_blocking=True).reshape(-1, width).contiguous()
    a = np.ascontiguousarray(m, dtype=np.float32)
    key = (a.shape, a.tobytes(), width, device.type, device.index)
    t = _cache_get(_HOST_MATS, key)
    if t is None:
        t = torch.tensor(a).pin_memory().to(device=device, non_blocking=True).reshape(-1, width).contiguous()
        t._ngt_host_key = key
        _cache_put(_HOST_MATS, key, (t,) + _recorded(t))
    return t


def _cameras(r, M, V, P, F):
    """The camera block of raymarch args ``r`` (ngt_raymarch_cameras) when all four
    matrix buffers are cached host uploads, formed once per matrices and slot
    layout; None otherwise (the call then forms its cameras itself)."""
    if any(getattr(t, "_ngt_host_key", None) is None for t in (M, V, P, F)):
        return None
    key = (id(M), id(V), id(P), id(F), int(r.input_shape[0]), int(r.separate_camera_batch))
    cams = _cache_get(_CAMERAS, key)
    if cams is None:
        lib = L.load()
        cams = torch.empty(int(lib.ngt_raymarch_cameras_bytes(ctypes.byref(r))), dtype=torch.uint8, device=M.device)
        L.call("ngt_raymarch_cameras", ctypes.byref(r), _ptr(cams), _stream())
        # the entry holds the matrices, so their ids stay theirs while it lives
        _cache_put(_CAMERAS, key, (cams,) + _recorded(cams) + ((M, V, P, F),))
    return cams


def sample_cache_pays(grid_dhw, batch, dtype, device):
    """Whether the render's sample cache (``ngt_raymarch_args.sample_cache``) is
    worth its L2 footprint: always for float storage, and for 16-bit storage while
    the quad gradient (16 bytes per (x, y)-quad and plane) fits in the L2 -- beyond
    that, 16-bit storage's 8-byte quad gathers cost less than the cache (measured
    both ways at 128^3 and at 256x448x256)."""
    if dtype == torch.float32:
        return True
    D, H, W = (int(v) for v in grid_dhw)
    gquad = int(batch) * (W + 1) * (H + 1) * (D + 2) * 16
    return gquad <= _l2_bytes(torch.device(device).index if torch.device(device).type == "cuda" else -1)


@functools.lru_cache(maxsize=None)
def _l2_bytes(index):
    """L2 size of CUDA device ``index`` (128 MiB when it cannot be read)."""
    try:
        dev = torch.device("cuda", index if index is not None and index >= 0 else torch.cuda.current_device())
        return int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0)) or (128 << 20)
    except (RuntimeError, AssertionError):
        return 128 << 20


def _rays(r, M, V, P, F):
    """The ray table of raymarch args ``r`` (ngt_raymarch_rays: every ray set up in
    double precision) when all four matrix buffers are cached host uploads,
    formed once per matrices, slot layout, image and grid sizes and boundary;
    None otherwise (the kernels then set up each ray in float arithmetic)."""
    if any(getattr(t, "_ngt_host_key", None) is None for t in (M, V, P, F)):
        return None
    key = (id(M), id(V), id(P), id(F), int(r.input_shape[0]), int(r.separate_camera_batch),
           tuple(int(v) for v in r.output_dhw), tuple(int(v) for v in r.input_shape[1:4]), int(r.boundary))
    rays = _cache_get(_RAYS, key)
    if rays is None:
        lib = L.load()
        rays = torch.empty(int(lib.ngt_raymarch_rays_bytes(ctypes.byref(r))), dtype=torch.uint8, device=M.device)
        L.call("ngt_raymarch_rays", ctypes.byref(r), _ptr(rays), _stream())
        _cache_put(_RAYS, key, (rays,) + _recorded(rays) + ((M, V, P, F),))
    return rays


def _check_matrices(input, M, V, P, F):
    """The kernels read one model matrix per batch entry and one view, projection
    and frustum per camera through plain pointers: shorter buffers are refused
    here rather than read past."""
    if M.shape[0] < input.shape[0]:
        raise ValueError("matrix_m holds %d matrices for a batch of %d grids" % (M.shape[0], input.shape[0]))
    if P.shape[0] < V.shape[0] or F.shape[0] < V.shape[0]:
        raise ValueError("matrix_p / frustum_params hold fewer entries (%d / %d) than matrix_v (%d cameras)"
                         % (P.shape[0], F.shape[0], V.shape[0]))


def _workspace(nbytes, device):
    if nbytes == 0:
        return None
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def _shape5(t):
    return L.I64x5(*[int(s) for s in t.shape])


# ------------------------------------------------------------------ LUT resample
def _lut_args(input, lookup, output, a):
    args = L.SampleLutArgs()
    args.dtype = _code(input)
    args.input_shape = _shape5(input)
    args.lookup_shape = _shape5(lookup)
    args.input, args.lookup, args.output = _ptr(input), _ptr(lookup), _ptr(output)
    args.interpolation = _enum(L.INTERP, a["interpolation"], "interpolation")
    args.boundary = _enum(L.BOUNDARY, a["boundary"], "boundary")
    args.mipmapping = _enum(L.MIP, a["mipmapping"], "mipmapping")
    args.num_mipmaps = int(a["num_mipmaps"])
    args.mip_bias = float(a["mip_bias"])
    args.cell_center_offset = float(a["cell_center_offset"])
    args.separate_camera_batch = int(bool(a["separate_camera_batch"]))
    args.relative_coords = int(bool(a["relative_coords"]))
    args.normalized_coords = int(bool(a["normalized_coords"]))
    return args


def _lut_forward(input, lookup, a):
    N, C = input.shape[0], input.shape[-1]
    V = lookup.shape[0]
    out = torch.empty((N, V if a["separate_camera_batch"] else 1) + tuple(lookup.shape[1:4]) + (C,),
                      dtype=input.dtype, device=input.device)
    args = _lut_args(input, lookup, out, a)
    ws = _workspace(L.load().ngt_sample_lut_fwd_workspace_bytes(ctypes.byref(args)), input.device)
    args.workspace, args.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
    L.call("ngt_sample_lut_fwd", ctypes.byref(args), _stream())
    return out


def _lut_backward(input, output_grad, lookup, a, mode, deterministic=None):
    g = L.SampleLutGradArgs()
    g.fwd = _lut_args(input, lookup, None, a)
    input_grad = torch.empty_like(input)
    lookup_grad = torch.empty_like(lookup)
    g.output_grad, g.input_grad, g.lookup_grad = _ptr(output_grad), _ptr(input_grad), _ptr(lookup_grad)
    g.grad_mode = L.GRAD[mode]
    g.deterministic = int(get_deterministic() if deterministic is None else deterministic)
    ws = _workspace(L.load().ngt_sample_lut_bwd_workspace_bytes(ctypes.byref(g)), input.device)
    g.workspace, g.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
    L.call("ngt_sample_lut_bwd", ctypes.byref(g), _stream())
    return input_grad, lookup_grad


class _SampleGridLut(torch.autograd.Function):
    @staticmethod
    def forward(ctx, input, lookup, attrs):
        ctx.attrs = attrs
        ctx.mode = get_gradient_mode()
        ctx.det = get_deterministic()
        ctx.save_for_backward(input, lookup)
        return _lut_forward(input, lookup, attrs)

    @staticmethod
    def backward(ctx, grad):
        input, lookup = ctx.saved_tensors
        gi, gl = _lut_backward(input, grad.contiguous(), lookup, ctx.attrs, ctx.mode, ctx.det)
        return gi, gl, None


def sample_grid_lut(input, lookup, interpolation="LINEAR", boundary="BORDER", mipmapping="NONE", num_mipmaps=0,
                    mip_bias=0.0, coordinate_mode="LOOKUP", cell_center_offset=0.0, separate_camera_batch=True,
                    relative_coords=True, normalized_coords=False):
    """``SampleGridLut`` (resample_grid.cc:94-120): input NDHWC, lookup VDHW4 (x, y, z,
    LoD) -> NVDHWC.  Differentiable w.r.t. input and lookup."""
    if coordinate_mode != "LOOKUP":
        raise ValueError("Invalid coorindate_mode")
    input = _cuda(input, "input")
    lookup = _cuda(lookup, "lookup").to(input.dtype)
    attrs = dict(interpolation=interpolation, boundary=boundary, mipmapping=mipmapping, num_mipmaps=num_mipmaps,
                 mip_bias=mip_bias, cell_center_offset=cell_center_offset,
                 separate_camera_batch=separate_camera_batch, relative_coords=relative_coords,
                 normalized_coords=normalized_coords)
    return _SampleGridLut.apply(input, lookup, attrs)


def sample_grid_lut_grad(input, output_grad, lookup, interpolation="LINEAR", boundary="BORDER", mipmapping="NONE",
                         num_mipmaps=0, mip_bias=0.0, coordinate_mode="LOOKUP", cell_center_offset=0.0,
                         separate_camera_batch=True, relative_coords=True, normalized_coords=False, grad_mode=None,
                         deterministic=None):
    """``SampleGridLutGrad`` (resample_grid.cc:124-150): returns (input_grad, lookup_grad)."""
    input = _cuda(input, "input")
    attrs = dict(interpolation=interpolation, boundary=boundary, mipmapping=mipmapping, num_mipmaps=num_mipmaps,
                 mip_bias=mip_bias, cell_center_offset=cell_center_offset,
                 separate_camera_batch=separate_camera_batch, relative_coords=relative_coords,
                 normalized_coords=normalized_coords)
    return _lut_backward(input, _cuda(output_grad, "output_grad").to(input.dtype),
                         _cuda(lookup, "lookup").to(input.dtype), attrs, grad_mode or get_gradient_mode(),
                         deterministic)


# ------------------------------------------------------------ transform resample
def _xf_args(input, M, V, P, F, out_dhw, output, a):
    args = L.SampleTransformArgs()
    args.dtype = _code(input)
    args.input_shape = _shape5(input)
    args.output_dhw = L.I64x3(*[int(s) for s in out_dhw])
    args.input, args.output = _ptr(input), _ptr(output)
    args.matrix_m, args.matrix_v, args.matrix_p, args.frustum = _ptr(M), _ptr(V), _ptr(P), _ptr(F)
    args.num_cameras = V.shape[0]
    args.interpolation = _enum(L.INTERP, a["interpolation"], "interpolation")
    args.boundary = _enum(L.BOUNDARY, a["boundary"], "boundary")
    args.mipmapping = _enum(L.MIP, a["mipmapping"], "mipmapping")
    args.num_mipmaps = int(a["num_mipmaps"])
    args.mip_bias = float(a["mip_bias"])
    args.cell_center_offset = float(a["cell_center_offset"])
    args.coordinate_mode = _enum(L.COORD, a["coordinate_mode"], "coordinate_mode")
    args.separate_camera_batch = int(bool(a["separate_camera_batch"]))
    return args


class _SampleGridTransform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, input, M, V, P, F, out_dhw, attrs):
        N, C = input.shape[0], input.shape[-1]
        out = torch.empty((N, V.shape[0] if attrs["separate_camera_batch"] else 1) + tuple(out_dhw) + (C,),
                          dtype=input.dtype, device=input.device)
        args = _xf_args(input, M, V, P, F, out_dhw, out, attrs)
        ws = _workspace(L.load().ngt_sample_transform_fwd_workspace_bytes(ctypes.byref(args)), input.device)
        args.workspace, args.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
        L.call("ngt_sample_transform_fwd", ctypes.byref(args), _stream())
        ctx.save_for_backward(input, M, V, P, F)
        ctx.attrs, ctx.out_dhw, ctx.mode, ctx.det = attrs, out_dhw, get_gradient_mode(), get_deterministic()
        return out

    @staticmethod
    def backward(ctx, grad):
        input, M, V, P, F = ctx.saved_tensors
        gi = _xf_backward(input, grad.contiguous(), M, V, P, F, ctx.out_dhw, ctx.attrs, ctx.mode, ctx.det)
        return gi, None, None, None, None, None, None


def _xf_backward(input, output_grad, M, V, P, F, out_dhw, a, mode, deterministic=None):
    g = L.SampleTransformGradArgs()
    g.fwd = _xf_args(input, M, V, P, F, out_dhw, None, a)
    gi = torch.empty_like(input)
    g.output_grad, g.input_grad, g.grad_mode = _ptr(output_grad), _ptr(gi), L.GRAD[mode]
    det = get_deterministic() if deterministic is None else deterministic
    g.deterministic = int(bool(det) and mode == "exact" and a["interpolation"] == "LINEAR")
    ws = _workspace(L.load().ngt_sample_transform_bwd_workspace_bytes(ctypes.byref(g)), input.device)
    g.workspace, g.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
    L.call("ngt_sample_transform_bwd", ctypes.byref(g), _stream())
    return gi


def _xf_prepare(input, matrix_m, matrix_v, matrix_p, frustum_params):
    input = _cuda(input, "input")
    dev = input.device
    M, V, P, F = (_floats(matrix_m, 16, dev), _floats(matrix_v, 16, dev), _floats(matrix_p, 16, dev),
                  _floats(frustum_params, 6, dev))
    _check_matrices(input, M, V, P, F)
    return input, M, V, P, F


def sample_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape, interpolation="LINEAR",
                          boundary="BORDER", mipmapping="NONE", num_mipmaps=0, mip_bias=0.0,
                          coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5, separate_camera_batch=True):
    """``SampleGridTransform`` (resample_grid.cc:23-65): input NDHWC -> NVDHWC with
    DHW = output_shape, sampled through model / view / projection / frustum."""
    input, M, V, P, F = _xf_prepare(input, matrix_m, matrix_v, matrix_p, frustum_params)
    attrs = dict(interpolation=interpolation, boundary=boundary, mipmapping=mipmapping, num_mipmaps=num_mipmaps,
                 mip_bias=mip_bias, coordinate_mode=coordinate_mode, cell_center_offset=cell_center_offset,
                 separate_camera_batch=separate_camera_batch)
    out_dhw = tuple(int(s) for s in list(output_shape)[:3])
    return _SampleGridTransform.apply(input, M, V, P, F, out_dhw, attrs)


def sample_grid_transform_grad(input, output_grad, matrix_m, matrix_v, matrix_p, frustum_params,
                               interpolation="LINEAR", boundary="BORDER", mipmapping="NONE", num_mipmaps=0,
                               mip_bias=0.0, coordinate_mode="TRANSFORM_LINDEPTH", cell_center_offset=0.5,
                               separate_camera_batch=True, grad_mode=None, deterministic=None):
    """``SampleGridTransformGrad`` (resample_grid.cc:68-92).  ``deterministic``
    (default: ``get_deterministic()``): the bit-reproducible gather form of the
    exact LINEAR gradient."""
    input, M, V, P, F = _xf_prepare(input, matrix_m, matrix_v, matrix_p, frustum_params)
    output_grad = _cuda(output_grad, "output_grad").to(input.dtype)
    attrs = dict(interpolation=interpolation, boundary=boundary, mipmapping=mipmapping, num_mipmaps=num_mipmaps,
                 mip_bias=mip_bias, coordinate_mode=coordinate_mode, cell_center_offset=cell_center_offset,
                 separate_camera_batch=separate_camera_batch)
    return _xf_backward(input, output_grad, M, V, P, F, tuple(output_grad.shape[2:5]), attrs,
                        grad_mode or get_gradient_mode(), deterministic)


def lod_transform(input_shape, matrix_mv, matrix_p, frustum_params, output_shape, inverse_transform=False,
                  linearize_depth=True, relative_coords=False, device="cuda"):
    """``LodTransform`` (resample_grid.cc:152-172): per camera a (V, D', H', W', 4)
    float32 lookup table of sampling positions and level of detail."""
    MV, P, F = _floats(matrix_mv, 16, device), _floats(matrix_p, 16, device), _floats(frustum_params, 6, device)
    out_dhw = [int(s) for s in list(output_shape)[:3]]
    out = torch.empty([MV.shape[0]] + out_dhw + [4], dtype=torch.float32, device=device)
    a = L.LodArgs()
    a.input_dhw = L.I64x3(*[int(s) for s in list(input_shape)[:3]])
    a.output_dhw = L.I64x3(*out_dhw)
    a.matrix_mv, a.matrix_p, a.frustum = _ptr(MV), _ptr(P), _ptr(F)
    a.num_cameras = MV.shape[0]
    a.inverse_transform, a.linearize_depth, a.relative_coords = int(inverse_transform), int(linearize_depth), \
        int(relative_coords)
    a.output = _ptr(out)
    L.call("ngt_lod_transform", ctypes.byref(a), _stream())
    return out


def mip_pyramid(input, levels):
    """Mip levels 1..levels of an NDHWC grid (box filter, as the resample op's
    mip atlas), returned as a list of tensors."""
    input = _cuda(input, "input")
    shape = L.I64x5(*[int(s) for s in input.shape])
    nbytes = L.load().ngt_mip_bytes(_code(input), shape, int(levels))
    ws = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=input.device)
    L.call("ngt_mip_build", _code(input), shape, _ptr(input), int(levels), _ptr(ws), ctypes.c_size_t(nbytes),
           _stream())
    out, off = [], 0
    es = input.element_size()
    for lv in range(1, int(levels) + 1):
        s = [input.shape[0], input.shape[1] >> lv, input.shape[2] >> lv, input.shape[3] >> lv, input.shape[4]]
        n = int(np.prod(s))
        out.append(ws[off:off + n * es].view(input.dtype).view(s).clone())
        off += (n * es + 255) // 256 * 256
    return out


# ------------------------------------------------------------------ raymarch
def _ray_args(input, M, V, P, F, out_dhw, output, a):
    r = L.RaymarchArgs()
    r.dtype = _code(input)
    r.input_shape = _shape5(input)
    r.output_dhw = L.I64x3(*[int(s) for s in out_dhw])
    r.input, r.output = _ptr(input), _ptr(output)
    r.matrix_m, r.matrix_v, r.matrix_p, r.frustum = _ptr(M), _ptr(V), _ptr(P), _ptr(F)
    r.num_cameras = V.shape[0]
    r.interpolation = _enum(L.INTERP, a["interpolation"], "interpolation")
    r.boundary = _enum(L.BOUNDARY, a["boundary"], "boundary")
    r.blending_mode = _enum(L.BLEND, a["blending_mode"], "blending_mode")
    r.keep_dims = int(bool(a["keep_dims"]))
    r.separate_camera_batch = int(bool(a["separate_camera_batch"]))
    es = a.get("emission_scale")
    if es is not None:
        r.emission_channels = len(es)
        for i, v in enumerate(es):
            r.emission_scale[i] = float(v)
    return r


def _ray_out_shape(input, V, out_dhw, a):
    N = input.shape[0]
    nv = V.shape[0] if a["separate_camera_batch"] else 1
    cb = len(a["emission_scale"]) if a.get("emission_scale") is not None else input.shape[-1]
    shape = (N, nv, int(out_dhw[1]), int(out_dhw[2]), cb)
    return shape if not a["keep_dims"] else (N, nv, 1) + shape[2:]


def _ray_forward(input, M, V, P, F, out_dhw, a, keep_quad=False):
    """The forward raymarch: (output, quad).  With ``keep_quad`` an input the
    quad gather layout serves is prepared into a buffer of its own, returned as
    ``quad`` = (buffer, sample_cache) for the backward to reuse instead of
    building it again; with a ray table the buffer also keeps the forward's
    density samples (``sample_cache`` 1) for the one-pass adjoint.  Otherwise
    ``quad`` is None."""
    out = torch.empty(_ray_out_shape(input, V, out_dhw, a), dtype=compute_dtype(input), device=input.device)
    r = _ray_args(input, M, V, P, F, out_dhw, out, a)
    cams = _cameras(r, M, V, P, F)
    if cams is not None:
        r.cameras = _ptr(cams)
    rays = _rays(r, M, V, P, F)
    if rays is not None:
        r.rays = _ptr(rays)
    lib = L.load()
    quad = None
    if keep_quad:
        r.sample_cache = int(rays is not None and sample_cache_pays(input.shape[1:4], input.shape[0], input.dtype,
                                                                     input.device))
        nq = int(lib.ngt_raymarch_quad_bytes(ctypes.byref(r)))
        if nq:
            buf = torch.empty(nq, dtype=torch.uint8, device=input.device)
            L.call("ngt_raymarch_quad", ctypes.byref(r), _ptr(buf), _stream())
            r.quad = _ptr(buf)
            quad = (buf, r.sample_cache)
    ws = _workspace(lib.ngt_raymarch_fwd_workspace_bytes(ctypes.byref(r)), input.device)
    r.workspace, r.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
    L.call("ngt_raymarch_fwd", ctypes.byref(r), _stream())
    return out, quad


def _ray_backward(input, output, output_grad, M, V, P, F, out_dhw, a, mode, quad=None, deterministic=None):
    g = L.RaymarchGradArgs()
    g.fwd = _ray_args(input, M, V, P, F, out_dhw, None, a)
    cams = _cameras(g.fwd, M, V, P, F)
    if cams is not None:
        g.fwd.cameras = _ptr(cams)
    rays = _rays(g.fwd, M, V, P, F)
    if rays is not None:
        g.fwd.rays = _ptr(rays)
    det = bool(get_deterministic() if deterministic is None else deterministic) and mode == "exact"
    if quad is not None and mode == "exact" and not det:
        g.fwd.quad, g.fwd.sample_cache = _ptr(quad[0]), quad[1]
    gi = torch.empty(input.shape, dtype=compute_dtype(input), device=input.device)
    g.output, g.output_grad, g.input_grad, g.grad_mode = _ptr(output), _ptr(output_grad), _ptr(gi), L.GRAD[mode]
    g.deterministic = int(det)
    ws = _workspace(L.load().ngt_raymarch_bwd_workspace_bytes(ctypes.byref(g)), input.device)
    g.workspace, g.workspace_bytes = _ptr(ws), 0 if ws is None else ws.numel()
    L.call("ngt_raymarch_bwd", ctypes.byref(g), _stream())
    return gi


class _RaymarchGridTransform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, input, M, V, P, F, out_dhw, attrs):
        mode = get_gradient_mode()
        # the quad layout built for the forward is kept for an exact backward
        det = get_deterministic()
        out, quad = _ray_forward(input, M, V, P, F, out_dhw, attrs,
                                 keep_quad=ctx.needs_input_grad[0] and mode == "exact" and not det)
        ctx.save_for_backward(input, M, V, P, F, out)
        ctx.attrs, ctx.out_dhw, ctx.mode, ctx.quad, ctx.det = attrs, out_dhw, mode, quad, det
        return out

    @staticmethod
    def backward(ctx, grad):
        input, M, V, P, F, out = ctx.saved_tensors
        gi = _ray_backward(input, out, grad.contiguous().to(out.dtype), M, V, P, F, ctx.out_dhw, ctx.attrs, ctx.mode,
                           quad=ctx.quad, deterministic=ctx.det)
        ctx.quad = None
        return gi, None, None, None, None, None, None


def raymarch_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape, interpolation="LINEAR",
                            boundary="BORDER", blending_mode="BEER_LAMBERT", keep_dims=False,
                            separate_camera_batch=True, emission_scale=None):
    """``RaymarchGridTransform`` (raymarch_grid.cc:29-63): input NDHWC -> NVHWC
    (NV1HWC with keep_dims); output_shape = (depth samples, H, W).

    ``emission_scale`` (2 or 4 floats) is an extension for a 1-channel density
    input: the blend then sees channel c = emission_scale[c] * density, the
    renderer's ``[light*step, density*step]`` grid (renderer.py:533-548,763)
    formed inside the kernel instead of materialised."""
    input = _cuda(input, "input")
    dev = input.device
    M, V, P, F = (_floats(matrix_m, 16, dev), _floats(matrix_v, 16, dev), _floats(matrix_p, 16, dev),
                  _floats(frustum_params, 6, dev))
    _check_matrices(input, M, V, P, F)
    attrs = dict(interpolation=interpolation, boundary=boundary, blending_mode=blending_mode, keep_dims=keep_dims,
                 separate_camera_batch=separate_camera_batch,
                 emission_scale=None if emission_scale is None else tuple(float(v) for v in emission_scale))
    out_dhw = tuple(int(s) for s in list(output_shape)[:3])
    return _RaymarchGridTransform.apply(input, M, V, P, F, out_dhw, attrs)


class _RaymarchGridTransformGrad(torch.autograd.Function):
    """The gradient op used as a forward op (the renderer's unprojection of images
    into the volume), differentiable w.r.t. ``output_grad`` as registered in
    ops_loader.py:98-118: for ADDITIVE blending its gradient is the forward
    raymarch of the incoming volume gradient; input and output get none."""

    @staticmethod
    def forward(ctx, input, output, output_grad, M, V, P, F, out_dhw, attrs, mode, deterministic):
        ctx.geom = (M, V, P, F, out_dhw, attrs, output_grad.shape)
        return _ray_backward(input, output, output_grad, M, V, P, F, out_dhw, attrs, mode,
                             deterministic=deterministic)

    @staticmethod
    def backward(ctx, grad):
        M, V, P, F, out_dhw, attrs, shape = ctx.geom
        blend = attrs["blending_mode"]
        blend = blend.decode() if isinstance(blend, bytes) else blend
        if blend != "ADDITIVE":
            raise NotImplementedError("Gradient of raymach op gradient only available for ADDITIVE blending, is %s"
                                      % blend)
        gg, _ = _ray_forward(grad.contiguous(), M, V, P, F, out_dhw, dict(attrs, emission_scale=None))
        return None, None, gg.reshape(shape), None, None, None, None, None, None, None, None


def raymarch_grid_transform_grad(input, output, output_grad, matrix_m, matrix_v, matrix_p, frustum_params,
                                 output_shape, interpolation="LINEAR", boundary="BORDER",
                                 blending_mode="BEER_LAMBERT", keep_dims=False, separate_camera_batch=True,
                                 grad_mode=None, emission_scale=None, deterministic=None):
    """``RaymarchGridTransformGrad`` (raymarch_grid.cc:67-92): the input gradient.
    Differentiable w.r.t. ``output_grad`` for ADDITIVE blending (ops_loader.py:98-118).
    ``deterministic`` (default: ``get_deterministic()``): bit-reproducible exact
    gradient (fixed-point integer accumulation)."""
    input = _cuda(input, "input")
    dev = input.device
    M, V, P, F = (_floats(matrix_m, 16, dev), _floats(matrix_v, 16, dev), _floats(matrix_p, 16, dev),
                  _floats(frustum_params, 6, dev))
    _check_matrices(input, M, V, P, F)
    attrs = dict(interpolation=interpolation, boundary=boundary, blending_mode=blending_mode, keep_dims=keep_dims,
                 separate_camera_batch=separate_camera_batch,
                 emission_scale=None if emission_scale is None else tuple(float(v) for v in emission_scale))
    cd = compute_dtype(input)
    return _RaymarchGridTransformGrad.apply(input, _cuda(output, "output").to(cd),
                                            _cuda(output_grad, "output_grad").to(cd), M, V, P, F,
                                            tuple(int(s) for s in list(output_shape)[:3]), attrs,
                                            grad_mode or get_gradient_mode(),
                                            get_deterministic() if deterministic is None else bool(deterministic))


def unproject(images, matrix_m, matrix_v, matrix_p, frustum_params, grid_dhw, depth, interpolation="LINEAR",
              boundary="BORDER", separate_camera_batch=True, grad_mode="reference"):
    """Scatter images back into the volume along the camera rays, as
    ``Renderer._raymarch_camera_transform(inverse=True)`` does (renderer.py:372-398):
    the ADDITIVE raymarch gradient op with the images as output gradient and a zero
    volume, ``depth`` samples per ray.  ``images``: N, V, H, W, C.  The reference op
    normalises each camera's scatter by its summed sample weights
    (``grad_mode='reference'``); ``'exact'`` gives the plain adjoint.
    Differentiable w.r.t. the images (the forward raymarch)."""
    images = _cuda(images, "images")
    N, H, W, C = images.shape[0], images.shape[2], images.shape[3], images.shape[4]
    D0, H0, W0 = (int(v) for v in grid_dhw)
    dummy = torch.zeros((N, D0, H0, W0, C), dtype=images.dtype, device=images.device)
    return raymarch_grid_transform_grad(dummy, images, images, matrix_m, matrix_v, matrix_p, frustum_params,
                                        (int(depth), H, W), interpolation=interpolation, boundary=boundary,
                                        blending_mode="ADDITIVE", separate_camera_batch=separate_camera_batch,
                                        grad_mode=grad_mode)


# -------------------------------------------------------------- reduce blend
def _rb_args(input, output, blending_mode, keep_dims):
    a = L.ReduceBlendArgs()
    a.dtype = _code(input)
    a.input_shape = _shape5(input)
    a.input, a.output = _ptr(input), _ptr(output)
    a.blending_mode = _enum(L.BLEND, blending_mode, "blending_mode")
    a.keep_dims = int(bool(keep_dims))
    return a


def _rb_backward(output_grad, output, input, blending_mode, keep_dims, mode):
    g = L.ReduceBlendGradArgs()
    g.fwd = _rb_args(input, None, blending_mode, keep_dims)
    gi = torch.empty_like(input)
    g.output, g.output_grad, g.input_grad, g.grad_mode = _ptr(output), _ptr(output_grad), _ptr(gi), L.GRAD[mode]
    L.call("ngt_reduce_blend_bwd", ctypes.byref(g), _stream())
    return gi


class _ReduceGridBlend(torch.autograd.Function):
    @staticmethod
    def forward(ctx, input, blending_mode, keep_dims):
        N, D, H, W, C = input.shape
        out = torch.empty((N, D, H, W, C) if keep_dims else (N, H, W, C), dtype=input.dtype, device=input.device)
        L.call("ngt_reduce_blend_fwd", ctypes.byref(_rb_args(input, out, blending_mode, keep_dims)), _stream())
        ctx.save_for_backward(input, out)
        ctx.blend, ctx.keep, ctx.mode = blending_mode, keep_dims, get_gradient_mode()
        return out

    @staticmethod
    def backward(ctx, grad):
        input, out = ctx.saved_tensors
        return _rb_backward(grad.contiguous(), out, input, ctx.blend, ctx.keep, ctx.mode), None, None


def reduce_grid_blend(input, blending_mode="BEER_LAMBERT", keep_dims=False):
    """``ReduceGridBlend`` (reduce_blend.cc:24-35): front-to-back blend along D."""
    return _ReduceGridBlend.apply(_cuda(input, "input"), blending_mode, keep_dims)


def reduce_grid_blend_grad(output_grad, output, input, blending_mode="BEER_LAMBERT", keep_dims=False,
                           grad_mode=None):
    """``ReduceGridBlendGrad`` (reduce_blend.cc:38-56)."""
    input = _cuda(input, "input")
    return _rb_backward(_cuda(output_grad, "output_grad").to(input.dtype), _cuda(output, "output").to(input.dtype),
                        input, blending_mode, keep_dims, grad_mode or get_gradient_mode())


# ------------------------------------------------------------------ image loss
class _ImageL2Loss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, target, loss_channels):
        grad = torch.empty_like(image)
        loss = torch.zeros((1,), dtype=image.dtype, device=image.device)
        C = image.shape[-1]
        L.call("ngt_image_l2_loss", _code(image), image.numel() // C, C, int(loss_channels), _ptr(image),
               _ptr(target), _ptr(grad), _ptr(loss), _stream())
        ctx.save_for_backward(grad)
        return loss[0]

    @staticmethod
    def backward(ctx, g):
        grad, = ctx.saved_tensors
        return grad * g, None, None


def image_l2_loss(image, target, loss_channels=1):
    """0.5 * sum over pixels of (image[..., c] - target[..., c])^2 for the first
    ``loss_channels`` channels of ``image`` (loss_dens_target on the rendered
    light channel, optimization.py:478), one kernel that also forms the image
    gradient; differentiable w.r.t. ``image``.  ``target`` holds
    ``loss_channels`` channels per pixel.  Float32 or float64 images."""
    image = _cuda(image, "image")
    if image.dtype not in (torch.float32, torch.float64):
        raise TypeError("image_l2_loss: images are float32 or float64")
    target = _cuda(target, "target").to(image.dtype)
    C = image.shape[-1]
    if not 0 < int(loss_channels) <= C or target.numel() != image.numel() // C * int(loss_channels):
        raise ValueError("image_l2_loss: target must hold loss_channels (1..%d) values per pixel" % C)
    return _ImageL2Loss.apply(image, target, int(loss_channels))


# ------------------------------------------------------- background composite
class _BackgroundComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, background):
        N, V, H, W, C = image.shape
        out = torch.empty((N, V, H, W, C - 1), dtype=image.dtype, device=image.device)
        L.call("ngt_background_composite", _code(image), N, V * H * W, C, _ptr(image), _ptr(background), _ptr(out),
               _stream())
        ctx.save_for_backward(image, background)
        return out

    @staticmethod
    def backward(ctx, g):
        image, background = ctx.saved_tensors
        N, V, H, W, C = image.shape
        gi = torch.empty_like(image)
        gb = torch.empty_like(background) if ctx.needs_input_grad[1] else None
        L.call("ngt_background_composite_bwd", _code(image), N, V * H * W, C, _ptr(image), _ptr(background),
               _ptr(g.contiguous()), _ptr(gi), _ptr(gb), _stream())
        return gi, gb


def background_composite(image, background):
    """The render composition's background composite (Renderer.render_density,
    renderer.py:779-781, 804-806): ``image`` (N, V, H, W, C) from a Beer-Lambert
    raymarch, C in {2, 4} with the optical depth d last; ``background`` the
    cameras' images behind the volume, broadcast to (V, H, W, C - 1) (one per
    camera, shared by the batch).  Returns the light channels with the background
    attenuated by the transmittance, ``image[..., :-1] + background * exp(-d)``
    (N, V, H, W, C - 1).  Differentiable w.r.t. both."""
    image = _cuda(image, "image")
    if image.dtype not in (torch.float32, torch.float64):
        raise TypeError("background_composite: images are float32 or float64")
    if image.dim() != 5 or image.shape[-1] not in (2, 4):
        raise ValueError("background_composite: image is (N, V, H, W, C) with C = 2 or 4")
    N, V, H, W, C = image.shape
    background = torch.as_tensor(background, device=image.device).to(image.dtype)
    background = background.expand(V, H, W, C - 1).contiguous()
    return _BackgroundComposite.apply(image, background)
