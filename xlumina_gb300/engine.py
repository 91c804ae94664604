"""Host side of the propagation path: geometry planning, caches, and the calls
into libxlgb.

Everything here either prepares small float64 host data (offset grids, chirp
vectors, separable mask factors), manages device buffers owned by torch, or
launches a libxlgb entry point on the current torch stream.  No field data is
computed on the host.
"""
from __future__ import annotations

import collections
import ctypes
import math
import threading

import numpy as np
import torch

from . import _lib

_LOCK = threading.Lock()


# ----------------------------------------------------------------- device --

def lib():
    return _lib.load()


_cuda_checked = False
_devices: dict = {}


def device() -> torch.device:
    """The current CUDA device (checked once; no CPU path)."""
    global _cuda_checked
    if not _cuda_checked:
        if not torch.cuda.is_available():
            raise RuntimeError("xlumina_gb300 needs a CUDA device (sm_103a); there is no CPU path")
        _cuda_checked = True
    i = torch.cuda.current_device()
    d = _devices.get(i)
    if d is None:
        d = _devices[i] = torch.device("cuda", i)
    return d


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def _is_broadcast_batch(t: torch.Tensor) -> bool:
    """One contiguous plane repeated along a leading batch dimension (stride 0)."""
    return t.dim() == 3 and t.shape[0] > 1 and t.stride(0) == 0 and t[0].is_contiguous()


def as_field(a, dev=None) -> torch.Tensor:
    """complex64 on the CUDA device, contiguous; a batch that is one plane
    broadcast along the batch (an ``expand``-ed view) stays a view, since
    every launch takes it without copying (batch stride 0)."""
    if isinstance(a, torch.Tensor) and a.is_cuda and a.dtype == torch.complex64 and dev is None:
        return a if (a.is_contiguous() or _is_broadcast_batch(a)) else a.contiguous()
    dev = dev or device()
    if isinstance(a, torch.Tensor):
        t = a.to(device=dev)
        if t.dtype != torch.complex64:
            t = t.to(torch.complex64)
        if _is_broadcast_batch(t):
            return t
        return t.contiguous()
    return torch.as_tensor(np.asarray(a), device=dev).to(torch.complex64).contiguous()


def batch_planes(comps, ny, nx):
    """Component planes for a launch: (tensors, batch, batch stride in elements).

    A batch of fields that is one plane broadcast along the batch (an
    ``expand``-ed view, stride 0) is passed without copying, with batch stride 0.
    """
    comps = [c if isinstance(c, torch.Tensor) else as_field(c) for c in comps]
    lead = comps[0].shape[:-2]
    B = int(np.prod(lead)) if len(lead) else 1
    if B > 1 and all(c.dim() == 3 and c.stride(0) == 0 and c.dtype == torch.complex64 and c.is_cuda and
                     c[0].is_contiguous() for c in comps):
        return [c[0] for c in comps], B, 0
    return [as_field(c).contiguous() for c in comps], B, ny * nx


def as_real_param(a, dev=None):
    """A mask parameter: python float for scalars, else a float32 contiguous CUDA tensor."""
    if isinstance(a, (int, float, np.floating, np.integer)):
        return float(a)
    if isinstance(a, torch.Tensor):
        if a.dim() == 0 and not a.requires_grad:
            return float(a.item())
        return a.to(device=dev or device(), dtype=torch.float32).contiguous()
    arr = np.asarray(a)
    if arr.ndim == 0:
        return float(arr)
    return torch.as_tensor(arr, device=dev or device()).to(torch.float32).contiguous()


_bytes_keys: "collections.OrderedDict" = collections.OrderedDict()


def array_key(a: np.ndarray) -> bytes:
    """The bytes of a host grid array, as a cache key; remembered per array
    object (a light's grid is shared by every light derived from it), so a
    repeated call does not copy and hash the array again."""
    k = id(a)
    hit = _bytes_keys.get(k)
    if hit is not None and hit[0] is a:
        return hit[1]
    b = a.tobytes()
    with _LOCK:
        _bytes_keys[k] = (a, b)       # the reference keeps the id valid
        while len(_bytes_keys) > 256:
            _bytes_keys.popitem(last=False)
    return b


def as_grid(a) -> np.ndarray:
    """A grid axis as a read-only float64 host array (as the reference's
    immutable jax arrays); an array that already is one is returned as it is."""
    if isinstance(a, np.ndarray) and a.dtype == np.float64 and not a.flags.writeable:
        return a
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    arr = np.array(a, dtype=np.float64)
    arr.setflags(write=False)
    return arr


_grid_cache: "collections.OrderedDict" = collections.OrderedDict()


def device_grid(a: np.ndarray) -> torch.Tensor:
    """float64 copy of a coordinate array on the device (cached by value)."""
    key = (array_key(a), torch.cuda.current_device())
    with _LOCK:
        t = _grid_cache.get(key)
        if t is not None:
            _grid_cache.move_to_end(key)
            return keep_for_capture(t)
    t = torch.tensor(a, dtype=torch.float64, device=device())
    with _LOCK:
        _grid_cache[key] = t
        while len(_grid_cache) > 64:
            _grid_cache.popitem(last=False)
    return keep_for_capture(t)


# Buffers handed out by the host caches while a CUDA graph is being captured
# (see plans.py): the plan holds them for the graph's lifetime, since a cache
# eviction must not free memory a replay will read.
_capture_keep = threading.local()


def keep_for_capture(t):
    keep = getattr(_capture_keep, "items", None)
    if keep is not None and t is not None:
        keep.append(t)
    return t


_array_cache: "collections.OrderedDict" = collections.OrderedDict()


def device_array(a, dtype) -> torch.Tensor:
    """A small constant array (distances, indices, pointers) on the device,
    cached by value: repeated calls reuse it, and a call replayed from a
    captured CUDA graph finds it already on the device."""
    arr = np.ascontiguousarray(np.asarray(a))
    key = (arr.tobytes(), arr.dtype.str, str(dtype), torch.cuda.current_device())
    with _LOCK:
        t = _array_cache.get(key)
        if t is not None:
            _array_cache.move_to_end(key)
            return keep_for_capture(t)
    t = torch.tensor(arr, device=device()).to(dtype)
    with _LOCK:
        _array_cache[key] = t
        while len(_array_cache) > 256:
            _array_cache.popitem(last=False)
    return keep_for_capture(t)


class _Built:
    """A cached device buffer and the event recorded after the launch that
    filled it.  A user on another stream waits for the event (only while it
    is pending) and marks the buffer as used by its stream, so the caching
    allocator cannot recycle it under that stream's pending work."""

    __slots__ = ("t", "ev", "stream")

    def __init__(self, t):
        self.t = t
        self.stream = torch.cuda.current_stream()
        self.ev = torch.cuda.Event()
        self.ev.record(self.stream)

    def use(self) -> torch.Tensor:
        if torch.cuda.is_current_stream_capturing():
            # the plan's warm-up run built it; the plan keeps it alive
            return keep_for_capture(self.t)
        cur = torch.cuda.current_stream()
        if cur != self.stream:
            if not self.ev.query():
                cur.wait_event(self.ev)
            self.t.record_stream(cur)
        return self.t


# ------------------------------------------------------------- geometry --

def rs_logq(ny: int, nx: int) -> int:
    """Q = 2^logq is the half transform length: the smallest power of two >= the
    field side, at least 32 (the kernels' smallest CTA shapes need P >= 64)."""
    n = max(ny, nx)
    return max(5, int(math.ceil(math.log2(n))))


def rs_offset_axis(x: np.ndarray) -> np.ndarray:
    """The reference's 2N-1 impulse-response offsets (wave_optics.py:265-279):
    ``x[0] - x[N-1-j]`` for j < N, then ``x[m] - x[0]``."""
    return np.concatenate([x[0] - x[::-1], x[1:] - x[0]])


def rs_wrapped_offsets(x: np.ndarray, P: int) -> np.ndarray:
    """Offsets in wrapped order for a P-point circular convolution: entry d mod P
    holds the offset of index distance d, |d| <= N-1; other entries are NaN."""
    n = len(x)
    ext = rs_offset_axis(x)
    out = np.full(P, np.nan)
    d = np.arange(-(n - 1), n)
    out[d % P] = ext[d + n - 1]
    return out


def quality_factor(x, y, wavelength, z):
    """wave_optics.py:187-191 / vectorized_optics.py:264-270 (a tensor distance
    gives a device tensor, computed without a host read)."""
    dx = x[1] - x[0]
    dy = y[1] - y[0]
    dr_real = np.sqrt(dx ** 2 + dy ** 2)
    rmax = np.sqrt((x ** 2).max() + (y ** 2).max())
    if isinstance(z, torch.Tensor):
        z = z.detach().to(torch.float64)
        return (torch.sqrt(wavelength ** 2 + rmax ** 2 + 2 * wavelength * torch.sqrt(rmax ** 2 + z ** 2)) -
                rmax) / dr_real
    z = np.asarray(z, dtype=np.float64)
    dr_ideal = np.sqrt(wavelength ** 2 + rmax ** 2 + 2 * wavelength * np.sqrt(rmax ** 2 + z ** 2)) - rmax
    return dr_ideal / dr_real


# --------------------------------------------------------- Jones program --

class JonesOp:
    """One per-pixel operation of a fused program (see XL_OP_* in xlgb.h)."""

    __slots__ = ("kind", "params", "ptrs", "sval", "dval", "keep", "planes")

    def __init__(self, kind, params=(), ptrs=(), sval=(), dval=(), keep=()):
        self.kind = kind
        self.params = list(params)   # floats or float32 tensors, parameter slots 0..3
        self.ptrs = list(ptrs)       # raw device tensors for pointer slots (SEPMASK / CMUL / HIGHNA)
        self.sval = list(sval)
        self.dval = list(dval)
        self.keep = list(keep)
        self.planes = {}             # slot -> plane a one-element tensor parameter was expanded to

    @staticmethod
    def is_scalar_tensor(p) -> bool:
        """A tensor parameter of one value, or of one value per batch entry (a
        trainable global setting, e.g. an LCD's retardance, or one per noisy
        table): it is expanded to planes for the launch and its gradient is
        the planes' sums."""
        return isinstance(p, torch.Tensor) and p.dim() < 2

    @staticmethod
    def plane_shape(p, ny, nx):
        return (ny, nx) if p.numel() == 1 else (p.numel(), ny, nx)

    def fill(self, op: _lib.XlOp, ny: int, nx: int) -> None:
        op.kind = self.kind
        pmask = 0
        pbstride = 0
        for i, p in enumerate(self.params):
            if self.is_scalar_tensor(p):
                shape = self.plane_shape(p, ny, nx)
                plane = self.planes.get(i)
                if plane is None or tuple(plane.shape) != shape:
                    plane = p.detach().to(torch.float32).reshape((-1, 1, 1)[-len(shape):]).expand(shape)
                    plane = plane.contiguous()
                    self.planes[i] = plane
                p = keep_for_capture(plane)
            if isinstance(p, torch.Tensor):
                if p.shape[-2:] != (ny, nx):
                    raise ValueError(f"mask parameter has shape {tuple(p.shape)}, field is {(ny, nx)}")
                pmask |= 1 << i
                op.ptr[i] = p.data_ptr()
                if p.dim() == 3 and p.shape[0] > 1:
                    pbstride = ny * nx
            else:
                op.sval[i] = float(p)
        for i, t in enumerate(self.ptrs):
            op.ptr[i] = 0 if t is None else t.data_ptr()
            if t is not None and t.dim() == 3 and t.shape[0] > 1:
                pbstride = ny * nx
        for i, s in enumerate(self.sval):
            op.sval[i] = float(s)
        for i, d in enumerate(self.dval):
            op.dval[i] = float(d)
        op.pmask = pmask
        op.pbstride = pbstride


def fill_prog(prog: _lib.XlProg, ops, ny, nx) -> None:
    ops = list(ops or ())
    if len(ops) > _lib.XL_MAX_OPS:
        raise ValueError(f"at most {_lib.XL_MAX_OPS} fused operations per pass")
    prog.nops = len(ops)
    for i, o in enumerate(ops):
        o.fill(prog.ops[i], ny, nx)


def op_phase(phase):
    return JonesOp(_lib.OP_PHASE, [as_real_param(phase)])


def op_sslm(alpha, phi):
    return JonesOp(_lib.OP_SSLM, [as_real_param(alpha), as_real_param(phi)])


def op_sslm_amp(alpha, phi, a1, a2):
    return JonesOp(_lib.OP_SSLM_AMP, [as_real_param(alpha), as_real_param(phi), as_real_param(a1),
                                      as_real_param(a2)])


def op_lcd(eta, theta):
    e, t = as_real_param(eta), as_real_param(theta)
    dv = [0.0, 0.0, 0.0, 0.0]
    if not isinstance(e, torch.Tensor):
        dv[0], dv[1] = math.cos(0.5 * e), math.sin(0.5 * e)
    if not isinstance(t, torch.Tensor):
        dv[2], dv[3] = math.cos(t), math.sin(t)
    return JonesOp(_lib.OP_LCD, [e, t], dval=dv)


def op_lp(alpha):
    a = as_real_param(alpha)
    sv = [] if isinstance(a, torch.Tensor) else [a, 0.0, math.cos(a), math.sin(a)]
    op = JonesOp(_lib.OP_LP, [a], sval=sv)
    return op


def lens_factors(x, y, wavelength, radius, focal):
    """Separable factors of optical_elements.py:678-703 (float64 on the host):
    colfac = exp(-ik x^2/2fx), rowfac = exp(-ik y^2/2fy), pupil terms x^2/rx^2, y^2/ry^2."""
    k = 2 * np.pi / wavelength
    fx, fy = focal
    rx, ry = radius
    colfac = np.exp(-1j * k * (x ** 2 / (2 * fx)))
    rowfac = np.exp(-1j * k * (y ** 2 / (2 * fy)))
    return colfac, rowfac, x ** 2 / rx ** 2, y ** 2 / ry ** 2


def op_lens(x, y, wavelength, radius, focal, vector):
    colfac, rowfac, tc, tr = lens_factors(x, y, wavelength, radius, focal)
    c = device_array(colfac.astype(np.complex64), torch.complex64)
    r = device_array(rowfac.astype(np.complex64), torch.complex64)
    tct = device_array(np.asarray(tc, dtype=np.float64), torch.float64)
    trt = device_array(np.asarray(tr, dtype=np.float64), torch.float64)
    return JonesOp(_lib.OP_SEPMASK, ptrs=[c, r, tct, trt], sval=[1.0 if vector else 0.0])


_highna_cache: "collections.OrderedDict" = collections.OrderedDict()


def highna_coefficients(x, y, radius, f):
    """The lens's 6 per-pixel coefficient planes, cached by geometry (computed by libxlgb)."""
    key = (array_key(x), array_key(y), float(radius), float(f), torch.cuda.current_device())
    with _LOCK:
        e = _highna_cache.get(key)
        if e is not None:
            _highna_cache.move_to_end(key)
    if e is not None:
        return e.use()
    t = torch.empty((6, len(y), len(x)), dtype=torch.float32, device=device())
    _lib.check(lib().xl_highna_coefficients(stream_handle(), len(y), len(x), device_grid(x).data_ptr(),
                                            device_grid(y).data_ptr(), float(radius), float(f), t.data_ptr()),
               "xl_highna_coefficients")
    e = _Built(t)
    with _LOCK:
        _highna_cache[key] = e
        while len(_highna_cache) > 8:
            _highna_cache.popitem(last=False)
    return t


def op_high_na(x, y, radius, f, ez_only=False):
    """optical_elements.py:515-594 as one per-pixel op (returns the op and
    sin(theta_max)); ``ez_only``: the lens's Ez row alone (one output
    component), for a focus whose Ex and Ey nothing reads."""
    s_max = radius / np.sqrt(radius ** 2 + f ** 2)
    coef = highna_coefficients(x, y, radius, f)
    op = JonesOp(_lib.OP_HIGHNA_EZ if ez_only else _lib.OP_HIGHNA, ptrs=[device_grid(x), device_grid(y), coef],
                 dval=[radius, f, s_max, 1.0 / (radius * radius)])
    return op, s_max


def op_cmul(mask: torch.Tensor):
    return JonesOp(_lib.OP_CMUL, ptrs=[as_field(mask).contiguous()])


def apply_ops(comps, ops, ny, nx):
    """Materialise a Jones program on 1..3 component planes; returns new tensors."""
    L = lib()
    lead = comps[0].shape[:-2]
    comps, B, ibs = batch_planes(comps, ny, nx)
    outs = [torch.empty(tuple(lead) + (ny, nx), dtype=torch.complex64, device=comps[0].device) for _ in comps]
    prog = _lib.XlProg()
    fill_prog(prog, ops, ny, nx)
    inp = (ctypes.c_void_p * 3)(*[c.data_ptr() for c in comps] + [0] * (3 - len(comps)))
    out = (ctypes.c_void_p * 3)(*[o.data_ptr() for o in outs] + [0] * (3 - len(outs)))
    _lib.check(L.xl_apply_ops(stream_handle(), B, len(comps), ny, nx, inp, ibs, out, ny * nx,
                              ctypes.byref(prog)), "xl_apply_ops")
    return outs


def ops_backward(base, gout, ops, ny, nx, want_input=True):
    """Backward of a Jones program.  ``base``: the program's input planes (None
    for a plane that is zero); ``gout``: gradients of its output planes (None
    after the first for a plane whose gradient is zero: it is not read).
    Returns (input gradients, {(op, slot): parameter gradient})."""
    L = lib()
    C = len(gout)
    ref = next(t for t in gout if t is not None)
    lead = ref.shape[:-2]
    B = int(np.prod(lead)) if len(lead) else 1
    dev = ref.device
    present = [b for b in base if b is not None]
    planes, _, ibs = batch_planes(present, ny, nx) if present else ([], B, ny * nx)
    it = iter(planes)
    base = [next(it) if b is not None else None for b in base]
    gin = [torch.empty_like(ref) if (want_input and i < len(base) and base[i] is not None) else None
           for i in range(C)]
    pgrad = (ctypes.c_void_p * (_lib.XL_MAX_OPS * 4))()
    grads = {}
    scalars = []
    for k, o in enumerate(ops):
        for q, p in enumerate(o.params):
            if isinstance(p, torch.Tensor):
                if not p.requires_grad:
                    continue
                if JonesOp.is_scalar_tensor(p):
                    t = torch.empty(JonesOp.plane_shape(p, ny, nx), dtype=torch.float32, device=dev)
                    scalars.append((k, q, p.shape))
                else:
                    t = torch.empty(p.shape, dtype=torch.float32, device=dev)
            else:
                continue
            grads[(k, q)] = t
            pgrad[k * 4 + q] = t.data_ptr()
    prog = _lib.XlProg()
    fill_prog(prog, ops, ny, nx)
    inp = (ctypes.c_void_p * 3)(*[(b.data_ptr() if b is not None else 0) for b in base] + [0] * (3 - len(base)))
    go = (ctypes.c_void_p * 3)(*[(g.data_ptr() if g is not None else 0) for g in gout] + [0] * (3 - C))
    gi = (ctypes.c_void_p * 3)(*[(g.data_ptr() if g is not None else 0) for g in gin] + [0] * (3 - C))
    _lib.check(L.xl_ops_backward(stream_handle(), B, C, ny, nx, inp, ibs, go, ny * nx, gi, ny * nx,
                                 ctypes.byref(prog), pgrad), "xl_ops_backward")
    for k, q, shape in scalars:
        grads[(k, q)] = grads[(k, q)].sum(dim=(-2, -1)).reshape(shape)
    return gin, grads


# ------------------------------------------------------ RS transfer spectra --

class SpectrumCache:
    """Transfer spectra keyed by (grid, z, wavelength); LRU, bounded in bytes.

    A spectrum depends only on the geometry, never on field data; the
    reference recomputes it on every call (wave_optics.py:285-288)."""

    def __init__(self, max_bytes=8 << 30):
        self.max_bytes = max_bytes
        self._d: "collections.OrderedDict" = collections.OrderedDict()
        self._bytes = 0
        self.builds = 0

    @staticmethod
    def key(x, y, z, wavelength, dz=False):
        return (array_key(x), array_key(y), float(z), float(wavelength), bool(dz), torch.cuda.current_device())

    def get(self, x, y, z, wavelength, dz=False):
        """The transfer spectrum, or with ``dz`` the spectrum of its z-derivative."""
        k = self.key(x, y, z, wavelength, dz)
        with _LOCK:
            e = self._d.get(k)
            if e is not None:
                self._d.move_to_end(k)
        if e is not None:
            return e.use()
        s = build_rs_spectrum(x, y, z, wavelength, dz)
        nb = s.numel() * 8
        with _LOCK:
            self._d[k] = _Built(s)
            self._bytes += nb
            self.builds += 1
            while self._bytes > self.max_bytes and len(self._d) > 1:
                _, old = self._d.popitem(last=False)
                self._bytes -= old.t.numel() * 8
        return s

    def clear(self):
        with _LOCK:
            self._d.clear()
            self._bytes = 0


SPECTRA = SpectrumCache()


def build_rs_spectrum(x, y, z, wavelength, dz=False) -> torch.Tensor:
    L = lib()
    ny, nx = len(y), len(x)
    lq = rs_logq(ny, nx)
    P = 2 << lq
    dev = device()
    offx = device_array(rs_wrapped_offsets(x, P), torch.float64)
    offy = device_array(rs_wrapped_offsets(y, P), torch.float64)
    spec = torch.empty(P * P, dtype=torch.complex64, device=dev)
    work = torch.empty(P * P, dtype=torch.complex64, device=dev)
    dx = x[1] - x[0]
    dy = y[1] - y[0]
    scale = dx * dy / float(P * P)
    fn = L.xl_rs_transfer_spectrum_dz if dz else L.xl_rs_transfer_spectrum
    _lib.check(fn(stream_handle(), ny, nx, offx.data_ptr(), offy.data_ptr(), float(z), float(wavelength), scale,
                  spec.data_ptr(), work.data_ptr()), "xl_rs_transfer_spectrum")
    return spec


def device_z(z, B) -> torch.Tensor:
    """A distance tensor as a contiguous float64 device array of 1 or B values
    (never read back to the host)."""
    zd = z.detach().to(device=device(), dtype=torch.float64).reshape(-1).contiguous()
    if zd.numel() not in (1, B):
        raise ValueError(f"{zd.numel()} distances for a batch of {B} fields")
    return zd


_offsets_cache: dict = {}


def device_offsets(a: np.ndarray, P: int) -> torch.Tensor:
    """The wrapped impulse-response offsets of a grid axis on the device (cached)."""
    key = (array_key(a), P, torch.cuda.current_device())
    t = _offsets_cache.get(key)
    if t is None:
        t = device_array(rs_wrapped_offsets(a, P), torch.float64)
        with _LOCK:
            if len(_offsets_cache) > 64:
                _offsets_cache.clear()
            _offsets_cache[key] = t
    return keep_for_capture(t)


def build_rs_spectra_device(x, y, zd: torch.Tensor, wavelength, dz=False) -> torch.Tensor:
    """Transfer spectra (or dH/dz spectra) for the distances of a device array,
    one per entry, stacked: shape (len(zd), P*P).  No host synchronisation."""
    L = lib()
    ny, nx = len(y), len(x)
    P = 2 << rs_logq(ny, nx)
    dev = zd.device
    offx = device_offsets(x, P)
    offy = device_offsets(y, P)
    n = zd.numel()
    spec = torch.empty((n, P * P), dtype=torch.complex64, device=dev)
    work = torch.empty(P * P, dtype=torch.complex64, device=dev)
    scale = (x[1] - x[0]) * (y[1] - y[0]) / float(P * P)
    _lib.check(L.xl_rs_transfer_spectra_device_z(stream_handle(), ny, nx, offx.data_ptr(), offy.data_ptr(),
                                                 zd.data_ptr(), n, float(wavelength), scale, 1 if dz else 0,
                                                 spec.data_ptr(), P * P, work.data_ptr()),
               "xl_rs_transfer_spectra_device_z")
    return spec


def out_pointer(t, shape):
    """Address the kernels write an output plane to: a CUDA tensor's data, or
    page-locked host memory (a pinned CPU tensor) reached over the host link,
    which saves the device-to-host copy of a result wanted on the host."""
    if t.dtype != torch.complex64 or tuple(t.shape) != tuple(shape) or not t.is_contiguous():
        raise ValueError(f"output must be a contiguous complex64 tensor of shape {tuple(shape)}, "
                         f"got {t.dtype} {tuple(t.shape)}")
    if t.is_cuda:
        return t.data_ptr()
    if t.device.type != "cpu" or not t.is_pinned():
        raise ValueError("an output on the host must be pinned (page-locked) memory")
    dev = ctypes.c_void_p()
    _lib.check(lib().xl_host_mapped(ctypes.c_void_p(t.data_ptr()), ctypes.byref(dev)), "xl_host_mapped")
    return dev.value


class RsCall:
    """One prepared RS / VRS launch: arguments, outputs and the buffers they point at.

    ``comps`` are complex64 CUDA tensors of shape (ny, nx) or (B, ny, nx);
    ``z`` is a float or a sequence of B floats (one transfer spectrum per
    distinct value, from the cache).  ``outs``: the output planes to write,
    CUDA tensors or pinned host tensors (see ``out_pointer``)."""

    def __init__(self, comps, x, y, wavelength, z, vector: bool, pre=(), post=(), outs=None, work=None,
                 adjoint=False, dz=False, want_ez=False, spectra=None):
        """``dz``: propagate with the spectrum of dH/dz (the output's z-derivative);
        ``want_ez``: a VRS adjoint also returns the propagated Ez gradient before
        it is folded into Ex, Ey (third output); ``spectra``: for a device
        distance, the stacked spectra an earlier call built for the same
        distances (``self.device_spectra``), reused instead of rebuilt."""
        L = lib()
        x = as_grid(x)
        y = as_grid(y)
        ny, nx = len(y), len(x)
        if comps[0].shape[-2:] != (ny, nx):
            raise ValueError(f"field shape {tuple(comps[0].shape)} does not match the grid ({ny}, {nx})")
        if len(comps) != (1 if not vector else (3 if adjoint else 2)):
            raise ValueError("RS takes one field, VRS takes (Ex, Ey) (adjoint: three gradients)")
        lead = comps[0].shape[:-2]
        comps, B, ibs = batch_planes(comps, ny, nx)
        dev = comps[0].device
        spec_ptrs = spec_index = None
        if isinstance(z, torch.Tensor):
            # distances on the device (e.g. being optimised): spectra built
            # from them in this call, stacked one per distance
            zd = device_z(z, B)
            spec = spectra if spectra is not None else build_rs_spectra_device(x, y, zd, wavelength, dz)
            specs = [spec]
            if zd.numel() > 1:
                spec_index = device_array(np.arange(B, dtype=np.int32), torch.int32)
            zt = (zd if zd.numel() == B else zd.expand(B).contiguous()) if vector else None
        else:
            zs = [float(v) for v in np.broadcast_to(np.asarray(z, dtype=np.float64), (B,))]
            uniq = sorted(set(zs))
            specs = [SPECTRA.get(x, y, zz, wavelength, dz) for zz in uniq]
            if len(specs) == 1:
                spec = specs[0]
            else:   # one spectrum pointer per batch entry, no stacked copy
                spec = None
                spec_ptrs = device_array([specs[uniq.index(v)].data_ptr() for v in zs], torch.int64)
            zt = device_array(np.asarray(zs, dtype=np.float64), torch.float64) if vector else None
        cout = 3 if vector else 1
        if work is None:
            work = torch.empty(L.xl_rs_work_bytes(B, cout, ny, nx) // 8, dtype=torch.complex64, device=dev)
        if outs is None:
            nout = (3 if want_ez else 2) if (adjoint and vector) else cout
            outs = [torch.empty(tuple(lead) + (ny, nx), dtype=torch.complex64, device=dev) for _ in range(nout)]
        a = _lib.XlRsArgs()
        a.batch = B
        a.comps_in = len(comps)
        a.comps_out = cout
        a.ny, a.nx = ny, nx
        for i, c in enumerate(comps):
            a.inp[i] = c.data_ptr()
        for i, o in enumerate(outs):
            a.out[i] = out_pointer(o, tuple(lead) + (ny, nx))
        a.in_bstride = ibs
        a.out_bstride = ny * nx
        if vector:
            a.x = device_grid(x).data_ptr()
            a.y = device_grid(y).data_ptr()
            a.z = zt.data_ptr()
        a.spectrum = _ptr(spec)
        a.spectrum_stride = spec.shape[-1] if spec_index is not None else 0
        a.spectrum_index = _ptr(spec_index)
        a.spectra = _ptr(spec_ptrs)
        a.work = work.data_ptr()
        fill_prog(a.pre, pre, ny, nx)
        fill_prog(a.post, post, ny, nx)
        a.adjoint = 1 if adjoint else 0
        self.args = a
        self.outs = outs
        self.device_spectra = spec if isinstance(z, torch.Tensor) else None
        self.batch, self.ny, self.nx, self.comps = B, ny, nx, cout
        self._keep = (comps, specs, spec_ptrs, spec_index, work, zt, list(pre or ()), list(post or ()))

    def run(self):
        _lib.check_device_status()     # an earlier launch's wait that ran out is reported here
        _lib.check(lib().xl_rs_propagate(stream_handle(), ctypes.byref(self.args)), "xl_rs_propagate")
        return self.outs

    def stage(self, s: int):
        if s == 0:
            _lib.check_device_status()
        _lib.check(lib().xl_rs_stage(stream_handle(), ctypes.byref(self.args), int(s)), "xl_rs_stage")


def rs_propagate(comps, x, y, wavelength, z, vector: bool, pre=(), post=(), outs=None):
    """Scalar RS (comps = [field]) or VRS (comps = [Ex, Ey]); returns 1 or 3 tensors
    (``outs``, if given: CUDA or pinned host tensors written in place)."""
    return RsCall(comps, x, y, wavelength, z, vector, pre, post, outs=outs).run()


# ---------------------------------------------------------------- sources --

def _mesh64(x, y):
    dev = device()
    return torch.meshgrid(torch.tensor(x, device=dev), torch.tensor(y, device=dev), indexing="xy")


def gaussian_field(x, y, wavelength, w0, E0=1.0, center=(0, 0), z_w0=(0, 0), alpha=0.0):
    """wave_optics.py:468-523 evaluated on the device in float64, returned as complex64.
    (The reference tests z_w0x for both radii of curvature, :503-510; kept.)"""
    k = 2 * np.pi / wavelength
    w0x, w0y = w0
    x0, y0 = center
    zx, zy = z_w0
    Rlx = k * w0x ** 2 / 2
    Rly = k * w0y ** 2 / 2
    gx = np.arctan2(zx, Rlx)
    gy = np.arctan2(zy, Rly)
    wx = w0x * np.sqrt(1 + (zx / Rlx) ** 2)
    wy = w0y * np.sqrt(1 + (zy / Rly) ** 2)
    Rx = 1e12 if zx == 0 else zx * (1 + (Rlx / zx) ** 2)
    Ry = 1e12 if zx == 0 else zy * (1 + (Rly / zy) ** 2)
    X, Y = _mesh64(x, y)
    xr = X * np.cos(alpha) + Y * np.sin(alpha)
    yr = -X * np.sin(alpha) + Y * np.cos(alpha)
    ph = -((k * zx + k * X ** 2 / (2 * Rx) - gx) + (k * zy + k * Y ** 2 / (2 * Ry) - gy))
    amp = E0 * (w0x / wx) * (w0y / wy) * torch.exp(-(xr - x0) ** 2 / wx ** 2 - (yr - y0) ** 2 / wy ** 2)
    return torch.polar(amp, ph).to(torch.complex64)


def plane_wave_field(x, y, wavelength, A=1.0, theta=0.0, phi=0.0, z0=0.0):
    """wave_optics.py:525-542 on the device (float64, returned as complex64)."""
    k = 2 * np.pi / wavelength
    X, Y = _mesh64(x, y)
    ph = k * (X * np.sin(theta) * np.cos(phi) + Y * np.sin(theta) * np.sin(phi) + z0 * np.cos(theta))
    return torch.polar(torch.full_like(ph, float(A)), ph).to(torch.complex64)


# -------------------------------------------------------------------- CZT --

def czt_grid(z, wavelength, xin, yin, xout, yout):
    """wave_optics.py:299-331: Dm = lambda z / dx and the frequency limits."""
    dx = xin[1] - xin[0]
    dy = yin[1] - yin[0]
    Dm = wavelength * z / dx
    return dict(nx=len(xout), ny=len(yout), dx=dx, dy=dy, Dm=Dm,
                fy1=yout[0] + Dm / 2, fy2=yout[-1] + Dm / 2,
                fx1=xout[0] + Dm / 2, fx2=xout[-1] + Dm / 2)


def bluestein_length(m, M):
    """The transform length of an m-point chirp-z onto M outputs: the
    reference's np2 = next power of two >= m + M - 1 (wave_optics.py:373-383,
    438), at least 32 here."""
    if M < 2:
        raise ValueError("chirp-z needs at least 2 output samples per axis")
    mp = m + M - 1
    L = int(2 ** int(np.ceil(np.log2(mp))))
    if L == mp:
        raise ValueError(f"m + M - 1 = {mp} is a power of two: the reference's Bluestein output slice "
                         "(wave_optics.py:446) is one sample short for this size")
    return max(L, 32)


def entry_chirps(z, wavelength, x, y, xout, yout, adjoint=False):
    """Chirp vectors and constant factors of a chirp-z at one distance per
    batch entry, built on the device (float64, stored complex64) from the
    device float64 distances ``z`` (B,): the per-entry form of
    ``device_chirps`` for build_CZT_grid's Dm = lambda z / dx
    (wave_optics.py:299-331).  Returns (Lx, Ly, pre_x, g_x, post_x, pre_y,
    g_y, post_y, cte), packed entry after entry as XlCztArgs.z_batch reads
    them; the vectors of ``adjoint`` calls are the adjoint set."""
    L = lib()
    B = int(z.numel())
    nx, ny, mx, my = len(x), len(y), len(xout), len(yout)
    Lx, Ly = bluestein_length(nx, mx), bluestein_length(ny, my)
    ix, ox = (mx, nx) if adjoint else (nx, mx)
    iy, oy = (my, ny) if adjoint else (ny, my)
    sizes = [ix, Lx, ox, iy, Ly, oy, 1]
    buf = torch.empty(B * sum(sizes), dtype=torch.complex64, device=z.device)
    views, o = [], 0
    for n in sizes:
        views.append(buf[o:o + B * n])
        o += B * n
    a = _lib.XlCztChirpArgs()
    a.batch, a.ny, a.nx, a.my, a.mx = B, ny, nx, my, mx
    a.log2_lx, a.log2_ly = Lx.bit_length() - 1, Ly.bit_length() - 1
    a.adjoint = 1 if adjoint else 0
    a.z = z.data_ptr()
    a.wavelength, a.dx, a.dy = float(wavelength), float(x[1] - x[0]), float(y[1] - y[0])
    a.xout0, a.xout1, a.yout0, a.yout1 = float(xout[0]), float(xout[-1]), float(yout[0]), float(yout[-1])
    (a.pre_x, a.g_x, a.post_x, a.pre_y, a.g_y, a.post_y, a.cte) = (v.data_ptr() for v in views)
    _lib.check(L.xl_czt_chirps(stream_handle(), ctypes.byref(a)), "xl_czt_chirps")
    return (Lx, Ly) + tuple(views)


def _per_entry(z):
    """True when ``z`` holds one distance per batch entry (a sequence or a 1-D tensor)."""
    if isinstance(z, torch.Tensor):
        return z.dim() >= 1
    return isinstance(z, (list, tuple, np.ndarray)) and np.ndim(z) >= 1


def bluestein_plan(m, f1, f2, Dm, M):
    """Chirp data of wave_optics.py:385-460 for an m-point input and M outputs, float64.

    Returns (L, pre, g, post): L the transform length; pre[n] = A^-n
    h[m-1+n]; g = fft(1/h[:m+M], L) in natural order;
    post[l] = h[m-1+l] exp(-i 2 pi l_f (1/2 - m/2) / Dm) / L, where
    h[q] = W^((q-m+1)^2/2) with the complex power's principal branch.
    """
    Lk = bluestein_length(m, M)
    D1 = f1 + (M * Dm + f2 - f1) / (2 * M)
    D2 = f2 + (M * Dm + f2 - f1) / (2 * M)
    mp = m + M - 1
    A = np.exp(1j * 2 * np.pi * D1 / Dm)
    W = np.exp(-1j * 2 * np.pi * (D2 - D1) / (M * Dm))
    q = np.arange(-m + 1, max(M - 1, m - 1) + 1)
    h = W ** (q ** 2 / 2)
    g = np.fft.fft(1 / h[:mp + 1], Lk)
    pre = A ** (-np.arange(m)) * h[m - 1:2 * m - 1]
    lf = np.linspace(0, M - 1, M) / M * (D2 - D1) + D1
    post = h[m - 1:mp] * np.exp(-1j * 2 * np.pi * lf * (-m / 2 + 0.5) / Dm) / Lk
    return Lk, pre, g, post


_chirp_cache: "collections.OrderedDict" = collections.OrderedDict()


def device_chirps(m, f1, f2, Dm, M, adjoint=False):
    """Chirp vectors on the device; the adjoint set is (conj(post) L, conj(g), conj(pre) / L)."""
    key = (int(m), float(f1), float(f2), float(Dm), int(M), bool(adjoint), torch.cuda.current_device())
    with _LOCK:
        v = _chirp_cache.get(key)
        if v is not None:
            _chirp_cache.move_to_end(key)
            for t in v[1:]:
                keep_for_capture(t)
            return v
    L, pre, g, post = bluestein_plan(m, f1, f2, Dm, M)
    if adjoint:
        pre, g, post = np.conj(post) * L, np.conj(g), np.conj(pre) / L
    dev = device()
    v = (L,) + tuple(torch.as_tensor(a, device=dev).to(torch.complex64) for a in (pre, g, post))
    with _LOCK:
        _chirp_cache[key] = v
        while len(_chirp_cache) > 64:
            _chirp_cache.popitem(last=False)
    return v


class TransferPlaneCache:
    """The chirp-z transfer function F = H(z, X, Y) (wave_optics.py:339-341)
    on whole grids, keyed by (grid, z, wavelength); LRU, bounded in bytes.

    A geometry is evaluated per pixel inside the kernels the first time it is
    seen and gets a plane the second time, so a table propagated every step
    reads F from memory while a distance used once (a serving request) costs
    no extra pass.  Planes are never built during graph capture."""

    def __init__(self, max_bytes=2 << 30):
        self.max_bytes = max_bytes
        self._d: "collections.OrderedDict" = collections.OrderedDict()
        self._seen: "collections.OrderedDict" = collections.OrderedDict()
        self._bytes = 0
        self.builds = 0

    @staticmethod
    def _key(x, y, z, wavelength):
        return (array_key(x), array_key(y), float(z), float(wavelength), torch.cuda.current_device())

    def pair(self, x, y, xout, yout, z, wavelength):
        """(F on the input grid, F0 on the output grid), or (None, None) while the
        geometry has not been seen before (or during graph capture, unless built)."""
        kin, kout = self._key(x, y, z, wavelength), self._key(xout, yout, z, wavelength)
        with _LOCK:
            built = kin in self._d and kout in self._d
            seen = all(k in self._d or k in self._seen for k in (kin, kout))
            if not built and (not seen or torch.cuda.is_current_stream_capturing()):
                for k in (kin, kout):
                    self._seen[k] = True
                while len(self._seen) > 4096:
                    self._seen.popitem(last=False)
                return None, None
        return self._plane(kin, x, y, z, wavelength), self._plane(kout, xout, yout, z, wavelength)

    def _plane(self, k, x, y, z, wavelength):
        with _LOCK:
            e = self._d.get(k)
            if e is not None:
                self._d.move_to_end(k)
        if e is not None:
            return e.use()
        ny, nx = len(y), len(x)
        t = torch.empty((ny, nx), dtype=torch.complex64, device=device())
        _lib.check(lib().xl_czt_transfer_plane(stream_handle(), ny, nx, device_grid(x).data_ptr(),
                                               device_grid(y).data_ptr(), float(z), float(wavelength),
                                               t.data_ptr()), "xl_czt_transfer_plane")
        with _LOCK:
            self._d[k] = _Built(t)
            self._bytes += t.numel() * 8
            self.builds += 1
            while self._bytes > self.max_bytes and len(self._d) > 2:
                _, old = self._d.popitem(last=False)
                self._bytes -= old.t.numel() * 8
        return t

    def clear(self):
        with _LOCK:
            self._d.clear()
            self._seen.clear()
            self._bytes = 0


TRANSFER_PLANES = TransferPlaneCache()


class CztCall:
    """One prepared chirp-z launch (scalar CZT, VCZT, or the high-NA focus).

    mode "scalar": wave_optics.py:233-263; "vczt": vectorized_optics.py:321-361;
    "high_na": optical_elements.py:600-638 (the lens op must be in ``pre``,
    ``lens`` = (radius, f, sin_theta_max)); "high_na_ez": the same focus of the
    Ez component alone (``pre`` ends with the lens's Ez-row op, one output).  ``z``: one distance, or one per
    batch entry (a sequence or a 1-D tensor, kept on the device; the chirps
    are then built there by ``entry_chirps``)."""

    def __init__(self, comps, x, y, wavelength, z, xout, yout, mode, pre=(), lens=None, outs=None,
                 adjoint=False):
        L = lib()
        x, y, xout, yout = (as_grid(a) for a in (x, y, xout, yout))
        ny, nx, my, mx = len(y), len(x), len(yout), len(xout)
        if comps[0].shape[-2:] != ((my, mx) if adjoint else (ny, nx)):
            raise ValueError(f"field shape {tuple(comps[0].shape)} does not match the grid")
        lead = comps[0].shape[:-2]
        comps, B, ibs = batch_planes(comps, *comps[0].shape[-2:])
        dev = comps[0].device
        zb = None
        if mode not in ("high_na", "high_na_ez") and _per_entry(z):
            zb = (z.detach() if isinstance(z, torch.Tensor) else torch.tensor(np.asarray(z, dtype=np.float64)))
            zb = zb.to(device=dev, dtype=torch.float64).reshape(-1).contiguous()
            if zb.numel() != B:
                raise ValueError(f"{zb.numel()} distances for a batch of {B} fields")
        if mode in ("high_na", "high_na_ez"):
            r, f, s_max = lens
            Dm = f * wavelength * (nx - 1) / (2 * r)
            if mode == "high_na":
                cmode, cin, cout = _lib.XL_CZT_PLAIN, (3 if adjoint else len(comps)), 3
            else:
                cmode, cin, cout = _lib.XL_CZT_PLAIN, (1 if adjoint else len(comps)), 1
            cte = -(1j * s_max ** 2 / (f * wavelength))
            zz = 0.0
        else:
            cmode = _lib.XL_CZT_SCALAR if mode == "scalar" else _lib.XL_CZT_VECTOR
            cin, cout = (1, 1) if mode == "scalar" else ((3 if adjoint else 2), 3)
            if zb is None:
                Dm = wavelength * z / (x[1] - x[0])
                cte = z * (x[1] - x[0]) * (y[1] - y[0]) * wavelength
                zz = float(z)
        cteb = None
        if zb is not None:
            Lx, Ly, prex, gx, postx, prey, gy, posty, cteb = entry_chirps(zb, wavelength, x, y, xout, yout, adjoint)
            cte, zz = 0.0, 0.0
        else:
            Lx, prex, gx, postx = device_chirps(nx, xout[0] + Dm / 2, xout[-1] + Dm / 2, Dm, mx, adjoint)
            Ly, prey, gy, posty = device_chirps(ny, yout[0] + Dm / 2, yout[-1] + Dm / 2, Dm, my, adjoint)
        if adjoint:   # the call reads the forward's output plane and writes its input plane
            x, y, xout, yout = xout, yout, x, y
            ny, nx, my, mx = my, mx, ny, nx
        work = torch.empty(L.xl_czt_work_bytes(B, cout, ny, mx) // 8, dtype=torch.complex64, device=dev)
        if outs is None:
            nout = 2 if (adjoint and cmode == _lib.XL_CZT_VECTOR) else cout
            outs = [torch.empty(tuple(lead) + (my, mx), dtype=torch.complex64, device=dev) for _ in range(nout)]
        a = _lib.XlCztArgs()
        a.batch, a.comps_in, a.comps_out, a.mode = B, cin, cout, cmode
        a.ny, a.nx, a.my, a.mx = ny, nx, my, mx
        a.adjoint = 1 if adjoint else 0
        a.log2_lx, a.log2_ly = int(Lx).bit_length() - 1, int(Ly).bit_length() - 1
        for i, c in enumerate(comps):
            a.inp[i] = c.data_ptr()
        for i, o in enumerate(outs):
            a.out[i] = o.data_ptr()
        a.in_bstride, a.out_bstride = (ibs if ibs == 0 else ny * nx), my * mx
        gx_, gy_, gxo, gyo = (device_grid(v) for v in (x, y, xout, yout))
        a.x, a.y, a.xout, a.yout = gx_.data_ptr(), gy_.data_ptr(), gxo.data_ptr(), gyo.data_ptr()
        a.z, a.wavelength = zz, float(wavelength)
        a.cte_re, a.cte_im = complex(cte).real, complex(cte).imag
        a.pre_x, a.g_x, a.post_x = prex.data_ptr(), gx.data_ptr(), postx.data_ptr()
        a.pre_y, a.g_y, a.post_y = prey.data_ptr(), gy.data_ptr(), posty.data_ptr()
        a.work = work.data_ptr()
        fin = fout = None
        if zb is not None:
            a.z_batch, a.cte_batch = zb.data_ptr(), cteb.data_ptr()
        elif cmode != _lib.XL_CZT_PLAIN:
            # F on the call's input plane and F0 on its output plane (for the
            # adjoint the grids are already swapped)
            fin, fout = TRANSFER_PLANES.pair(x, y, xout, yout, zz, wavelength)
            if fin is not None:
                a.f_in, a.f_out = fin.data_ptr(), fout.data_ptr()
        fill_prog(a.pre, pre, ny, nx)
        self.args = a
        self.outs = outs
        self._keep = (comps, work, prex, gx, postx, prey, gy, posty, gx_, gy_, gxo, gyo, list(pre or ()), zb, cteb,
                      fin, fout)

    def run(self):
        _lib.check_device_status()     # an earlier launch's wait that ran out is reported here
        _lib.check(lib().xl_czt(stream_handle(), ctypes.byref(self.args)), "xl_czt")
        return self.outs

    def stage(self, s: int):
        if s == 0:
            _lib.check_device_status()
        _lib.check(lib().xl_czt_stage(stream_handle(), ctypes.byref(self.args), int(s)), "xl_czt_stage")


def czt_plain(comps, mx, my, Dm, fy1, fy2, fx1, fx2, cte=1.0):
    """The two Bluestein transforms alone (CZT_for_high_NA_jit,
    wave_optics.py:359-371): each (ny, nx) plane onto my x mx outputs over the
    frequency ranges given; ``comps`` are 1 to 3 components, each of shape
    (ny, nx) or (B, ny, nx).  Returns the output planes."""
    L = lib()
    ny, nx = comps[0].shape[-2:]
    lead = comps[0].shape[:-2]
    planes, B, ibs = batch_planes(comps, ny, nx)
    dev = planes[0].device
    Lx, prex, gx, postx = device_chirps(nx, float(fx1), float(fx2), float(Dm), int(mx))
    Ly, prey, gy, posty = device_chirps(ny, float(fy1), float(fy2), float(Dm), int(my))
    C = len(planes)
    work = torch.empty(L.xl_czt_work_bytes(B, C, ny, mx) // 8, dtype=torch.complex64, device=dev)
    outs = [torch.empty(tuple(lead) + (my, mx), dtype=torch.complex64, device=dev) for _ in range(C)]
    a = _lib.XlCztArgs()
    a.batch, a.comps_in, a.comps_out, a.mode = B, C, C, _lib.XL_CZT_PLAIN
    a.ny, a.nx, a.my, a.mx = ny, nx, int(my), int(mx)
    a.log2_lx, a.log2_ly = int(Lx).bit_length() - 1, int(Ly).bit_length() - 1
    for i, c in enumerate(planes):
        a.inp[i] = c.data_ptr()
    for i, o in enumerate(outs):
        a.out[i] = o.data_ptr()
    a.in_bstride, a.out_bstride = ibs, int(my) * int(mx)
    a.cte_re, a.cte_im = complex(cte).real, complex(cte).imag
    a.pre_x, a.g_x, a.post_x = prex.data_ptr(), gx.data_ptr(), postx.data_ptr()
    a.pre_y, a.g_y, a.post_y = prey.data_ptr(), gy.data_ptr(), posty.data_ptr()
    a.work = work.data_ptr()
    fill_prog(a.pre, [], ny, nx)
    keep = (planes, work, prex, gx, postx, prey, gy, posty)
    _lib.check(L.xl_czt(stream_handle(), ctypes.byref(a)), "xl_czt")
    del keep
    return outs


def czt_propagate(comps, x, y, wavelength, z, xout, yout, mode, pre=(), lens=None):
    """Scalar CZT, VCZT or the high-NA focus; returns 1 or 3 output tensors."""
    return CztCall(comps, x, y, wavelength, z, xout, yout, mode, pre, lens).run()


# ------------------------------------------------------------------ losses --

def _planes(t: torch.Tensor):
    """(contiguous view, number of planes, plane stride) of a (..., ny, nx) complex64 tensor;
    a single plane repeated by an expand-ed view keeps plane stride 0."""
    ny, nx = t.shape[-2:]
    if t.dim() == 3 and t.shape[0] > 1 and t.stride(0) == 0 and t[0].is_contiguous():
        return t[0], t.shape[0], 0
    t = t.contiguous()
    n = t.numel() // (ny * nx)
    return t, n, ny * nx


MSE_KINDS = {"intensity": 0, "amplitude": 1, "phase": 2}


def mse_intensity(a: torch.Tensor, b: torch.Tensor, kind: str = "intensity") -> torch.Tensor:
    """sum((|a|^2 - |b|^2)^2) / npix over the last two dims (libxlgb, fixed-order
    sums); ``kind`` "amplitude": (|a| - |b|)^2, "phase": (arg a - arg b)^2."""
    a = as_field(a)
    b = as_field(b)
    ny, nx = a.shape[-2:]
    if b.shape[-2:] != (ny, nx):
        raise ValueError(f"input {tuple(a.shape)} and target {tuple(b.shape)} planes differ")
    av, na, aps = _planes(a)
    if b.shape[:-2] == a.shape[:-2]:
        bv, nb, bps = _planes(b)
    elif b.dim() == 2 or b.numel() == ny * nx:
        bv, nb, bps = b.reshape(ny, nx).contiguous(), 1, 0
    else:
        raise ValueError(f"target of shape {tuple(b.shape)} does not broadcast over input {tuple(a.shape)}")
    npix = ny * nx
    L = lib()
    work = torch.empty(max(1, L.xl_mse_intensity_work_bytes(na, npix) // 8), dtype=torch.float64, device=a.device)
    out = torch.empty(na, dtype=torch.float32, device=a.device)
    _lib.check(L.xl_plane_mse(stream_handle(), MSE_KINDS[kind], na, npix, av.data_ptr(), aps, bv.data_ptr(), bps,
                              work.data_ptr(), out.data_ptr()), "xl_plane_mse")
    return out.reshape(a.shape[:-2])


def mse_intensity_grad(a, b, g, want_a=True, want_b=False, kind: str = "intensity"):
    """Gradients of ``mse_intensity`` for the upstream gradient ``g`` (shape a.shape[:-2])."""
    a = as_field(a)
    b = as_field(b)
    ny, nx = a.shape[-2:]
    av, na, aps = _planes(a)
    if b.shape[:-2] == a.shape[:-2]:
        bv, nb, bps = _planes(b)
    else:
        bv, bps = b.reshape(ny, nx).contiguous(), 0
    g = g.to(device=a.device, dtype=torch.float32).reshape(-1).contiguous()
    ga = torch.empty(a.shape, dtype=torch.complex64, device=a.device) if want_a else None
    gb = torch.empty(a.shape, dtype=torch.complex64, device=a.device) if want_b else None
    _lib.check(lib().xl_plane_mse_grad(stream_handle(), MSE_KINDS[kind], na, ny * nx, av.data_ptr(), aps,
                                       bv.data_ptr(), bps, g.data_ptr(), _ptr(ga), _ptr(gb)), "xl_plane_mse_grad")
    return ga, gb


def z_values(z):
    """(the distance as the propagators take it, the tensor that needs its
    gradient or None).  A tensor distance stays on the device: its transfer
    spectra are built there from its values, with no host read."""
    if isinstance(z, torch.Tensor):
        return z.detach(), (z if z.requires_grad else None)
    return z, None


def re_inner(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """sum over the last two dims of Re(conj(a) b), one value per plane (fixed-order sums)."""
    a = as_field(a)
    b = as_field(b)
    ny, nx = a.shape[-2:]
    av, na, aps = _planes(a)
    bv, nb, bps = _planes(b)
    if nb != na:
        raise ValueError("re_inner: plane counts differ")
    L = lib()
    work = torch.empty(max(1, L.xl_mse_intensity_work_bytes(na, ny * nx) // 8), dtype=torch.float64,
                       device=a.device)
    out = torch.empty(na, dtype=torch.float32, device=a.device)
    _lib.check(L.xl_re_inner(stream_handle(), na, ny * nx, av.data_ptr(), aps, bv.data_ptr(), bps, work.data_ptr(),
                             out.data_ptr()), "xl_re_inner")
    return out.reshape(a.shape[:-2])


def vrs_dz_ez(ex, ey, gez, x, y, zs) -> torch.Tensor:
    """Per batch entry: sum Re(conj(gez) dEz/dz) for the VRS Ez derivation (libxlgb)."""
    ex, ey, gez = as_field(ex), as_field(ey), as_field(gez)
    ny, nx = gez.shape[-2:]
    B = gez.numel() // (ny * nx)
    (exv, eyv), _, ebs = batch_planes([ex, ey], ny, nx)
    gv = gez.contiguous()
    x, y = as_grid(x), as_grid(y)
    if isinstance(zs, torch.Tensor):
        zd = device_z(zs, B)
        zt = zd if zd.numel() == B else zd.expand(B).contiguous()
    else:
        zt = device_array(np.broadcast_to(np.asarray(zs, dtype=np.float64), (B,)).copy(), torch.float64)
    L = lib()
    work = torch.empty(max(1, L.xl_mse_intensity_work_bytes(B, ny * nx) // 8), dtype=torch.float64, device=gv.device)
    out = torch.empty(B, dtype=torch.float32, device=gv.device)
    _lib.check(L.xl_vrs_dz_ez(stream_handle(), B, ny, nx, exv.data_ptr(), eyv.data_ptr(), ebs, gv.data_ptr(),
                              ny * nx, device_grid(x).data_ptr(), device_grid(y).data_ptr(), zt.data_ptr(),
                              work.data_ptr(), out.data_ptr()), "xl_vrs_dz_ez")
    return out


def rs_z_gradient(gouts, douts, x, y, z, ex=None, ey=None, gez=None) -> torch.Tensor:
    """dL/dz of one RS / VRS call per batch entry (libxlgb, one pass): the
    output gradients ``gouts`` against the dH/dz propagation ``douts``, plus
    for VRS the Ez term of the Jones-program output (ex, ey) against the
    adjoint's unfolded Ez gradient ``gez``."""
    ny, nx = gouts[0].shape[-2:]
    B = gouts[0].numel() // (ny * nx)
    gs = [as_field(g).contiguous() for g in gouts]
    ds = [as_field(d).contiguous() for d in douts]
    dev = gs[0].device
    L = lib()
    work = torch.empty(max(1, L.xl_mse_intensity_work_bytes(B, ny * nx) // 8), dtype=torch.float64, device=dev)
    out = torch.empty(B, dtype=torch.float32, device=dev)
    keep = []
    exp = eyp = gp = xp = yp = zp = 0
    ebs = 0
    if ex is not None:
        (exv, eyv), _, ebs = batch_planes([ex, ey], ny, nx)
        gv = as_field(gez).contiguous()
        x, y = as_grid(x), as_grid(y)
        if isinstance(z, torch.Tensor):
            zd = device_z(z, B)
            zt = zd if zd.numel() == B else zd.expand(B).contiguous()
        else:
            zt = device_array(np.broadcast_to(np.asarray(z, dtype=np.float64), (B,)).copy(), torch.float64)
        keep = [exv, eyv, gv, zt]
        exp, eyp, gp = exv.data_ptr(), eyv.data_ptr(), gv.data_ptr()
        xp, yp, zp = device_grid(x).data_ptr(), device_grid(y).data_ptr(), zt.data_ptr()
    gpp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in gs] + [0] * (3 - len(gs)))
    dpp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in ds] + [0] * (3 - len(ds)))
    _lib.check(L.xl_rs_z_gradient(stream_handle(), B, ny, nx, len(gs), gpp, dpp, ny * nx, exp, eyp, ebs, gp, xp, yp,
                                  zp, work.data_ptr(), out.data_ptr()), "xl_rs_z_gradient")
    del keep
    return out.reshape(gouts[0].shape[:-2])


# ---------------------------------------------------------- beam splitters --

def _bs_port(comps, B, ny, nx):
    """(Ex, Ey) planes of one port for a launch of batch B: (planes, batch stride)."""
    if comps is None:
        return [None, None], 0
    comps = [as_field(c) for c in comps]
    lead = comps[0].shape[:-2]
    nb = int(np.prod(lead)) if len(lead) else 1
    if nb == 1:
        return [c.reshape(ny, nx).contiguous() for c in comps], 0
    if nb != B:
        raise ValueError(f"beam splitter ports hold {nb} and {B} fields")
    planes, _, bs = batch_planes(comps, ny, nx)
    return planes, bs


def _bs_batch(a, b, m):
    leads = [c.shape[:-2] for c in list(a) + list(b or [])]
    sizes = [int(np.prod(s)) if len(s) else 1 for s in leads]
    if m.dim() == 3:
        sizes.append(m.shape[0])
    B = max(sizes)
    lead = next((s for s, n in zip(leads, sizes) if n == B), (B,))
    return B, tuple(lead) if B > 1 else ()


def _bs_args(a, b, m, ny, nx, kind=0):
    """``m``: the complex (2, 2) / (B, 2, 2) matrix (kind XL_BS_MATRIX), or the
    splitting angle(s) as a float64 device tensor of 1 or B values."""
    if kind == _lib.XL_BS_MATRIX:
        B, lead = _bs_batch(a, b, m)
    else:
        B, lead = _bs_batch(a, b, m.reshape(-1, 1, 1) if m.numel() > 1 else m.reshape(1, 1))
    pa, sa = _bs_port(a, B, ny, nx)
    pb, sb = _bs_port(b, B, ny, nx)
    args = _lib.XlBsArgs()
    args.batch, args.ny, args.nx, args.kind = B, ny, nx, int(kind)
    if kind == _lib.XL_BS_MATRIX:
        if m.dim() == 3 and m.shape[0] == 1:
            m = m[0]
        if m.dim() == 3 and m.shape[0] != B:
            raise ValueError(f"{m.shape[0]} splitter matrices for a batch of {B}")
        m = m.to(torch.complex64).contiguous()
        args.m = m.data_ptr()
        args.m_bstride = 4 if m.dim() == 3 else 0
    else:
        m = m.detach().to(device=device(), dtype=torch.float64).reshape(-1).contiguous()
        if m.numel() not in (1, B):
            raise ValueError(f"{m.numel()} splitter angles for a batch of {B}")
        args.theta = m.data_ptr()
        args.theta_bstride = 1 if m.numel() > 1 else 0
    for j, port in enumerate((pa, pb)):
        for c in range(2):
            args.inp[j][c] = _ptr(port[c])
    args.in_bstride[0], args.in_bstride[1] = sa, sb
    return args, B, lead, (pa, pb, m)


def beam_splitter(a, b, m, kind=0):
    """[c.Ex, c.Ey, d.Ex, d.Ey] = M [a; b] on the (Ex, Ey) planes (libxlgb).
    ``a``, ``b``: [Ex, Ey] tensors of shape (ny, nx) or (B, ny, nx) (``b`` may be
    None); ``m``: complex device tensor (2, 2) or (B, 2, 2), or for the angle
    kinds (XL_BS_SYMMETRIC, XL_BS_SINGLE_PORT0/1) the splitting angle(s)."""
    ny, nx = a[0].shape[-2:]
    args, B, lead, keep = _bs_args(a, b, m, ny, nx, kind)
    dev = keep[0][0].device
    outs = [torch.empty(lead + (ny, nx), dtype=torch.complex64, device=dev) for _ in range(4)]
    for i in range(2):
        for c in range(2):
            args.out[i][c] = outs[2 * i + c].data_ptr()
    args.out_bstride = ny * nx
    _lib.check(lib().xl_beam_splitter(stream_handle(), ctypes.byref(args)), "xl_beam_splitter")
    return outs


def beam_splitter_backward(a, b, m, gouts, want_a=True, want_b=True, want_m=True, kind=0):
    """Gradients of ``beam_splitter``: (ga [Ex, Ey] or None, gb or None, the
    matrix's S (B, 2, 2) complex64 with S_ij = sum conj(g_i) in_j, or for the
    angle kinds dL/dtheta (B,) float64; None when not wanted)."""
    ny, nx = a[0].shape[-2:]
    args, B, lead, keep = _bs_args(a, b, m, ny, nx, kind)
    dev = keep[0][0].device
    gs = [None if g is None else as_field(g).reshape((B, ny, nx) if B > 1 else (ny, nx)).contiguous()
          for g in gouts]
    gin = [None] * 4
    if want_a:
        gin[0:2] = [torch.empty(lead + (ny, nx), dtype=torch.complex64, device=dev) for _ in range(2)]
    if want_b and b is not None:
        gin[2:4] = [torch.empty(lead + (ny, nx), dtype=torch.complex64, device=dev) for _ in range(2)]
    s = work = None
    if want_m:
        s = torch.empty((B, 2, 2), dtype=torch.complex64, device=dev)
        work = torch.empty(max(1, lib().xl_beam_splitter_work_bytes(B, ny, nx) // 8), dtype=torch.float64,
                           device=dev)
    dth = torch.empty(B, dtype=torch.float64, device=dev) if (want_m and kind != _lib.XL_BS_MATRIX) else None
    gp = (ctypes.c_void_p * 4)(*[_ptr(g) for g in gs])
    ip = (ctypes.c_void_p * 4)(*[_ptr(g) for g in gin])
    _lib.check(lib().xl_beam_splitter_backward(stream_handle(), ctypes.byref(args), gp, ny * nx, ip, ny * nx,
                                               _ptr(s), _ptr(work), _ptr(dth)), "xl_beam_splitter_backward")
    ga = gin[0:2] if want_a else None
    gb = gin[2:4] if (want_b and b is not None) else None
    return ga, gb, (dth if kind != _lib.XL_BS_MATRIX else s)


# ------------------------------------------------------ fused loss epilogues --

def _loss_planes(t: torch.Tensor):
    """(contiguous planes, count, plane stride, complex?) of a (..., ny, nx)
    complex64 field or float32 intensity."""
    cplx = t.is_complex()
    t = (t.to(torch.complex64) if cplx else t.to(torch.float32)).contiguous()
    ny, nx = t.shape[-2:]
    return t, t.numel() // (ny * nx), ny * nx, cplx


def area_loss(x: torch.Tensor):
    """small_area_hybrid per plane (loss_functions.py:24-40) of intensities
    or, for a complex field, of its intensity |x|^2, in two fused passes.
    Returns (losses of shape x.shape[:-2], the work buffer its gradient needs)."""
    t, n, ps, cplx = _loss_planes(x)
    L = lib()
    work = torch.empty(max(1, L.xl_loss_work_bytes(n, ps) // 8), dtype=torch.float64, device=t.device)
    out = torch.empty(n, dtype=torch.float32, device=t.device)
    _lib.check(L.xl_area_loss(stream_handle(), n, ps, int(cplx), t.data_ptr(), ps, work.data_ptr(), out.data_ptr()),
               "xl_area_loss")
    return out.reshape(x.shape[:-2]), work


def area_loss_grad(x: torch.Tensor, work: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    t, n, ps, cplx = _loss_planes(x)
    g = g.to(device=t.device, dtype=torch.float32).reshape(-1).contiguous()
    gin = torch.empty(t.shape, dtype=t.dtype, device=t.device)
    _lib.check(lib().xl_area_loss_grad(stream_handle(), n, ps, int(cplx), t.data_ptr(), ps, work.data_ptr(),
                                       g.data_ptr(), gin.data_ptr()), "xl_area_loss_grad")
    return gin


def _target_planes(target: torch.Tensor, ny, nx, n):
    tg = target.to(torch.float32)
    if tg.numel() == ny * nx:
        return tg.reshape(ny, nx).contiguous(), 0
    if tg.numel() != n * ny * nx:
        raise ValueError(f"target of shape {tuple(target.shape)} does not match {n} planes of {ny}x{nx}")
    return tg.contiguous(), ny * nx


def norm_intensity_mse(x: torch.Tensor, target: torch.Tensor):
    """The 4f tables' normalised intensity MSE per plane
    (experiments/four_f_optical_table.py:129-141): In = I / sum I,
    sum((In - T)^2) / npix.  Returns (losses, work buffer)."""
    t, n, ps, cplx = _loss_planes(x)
    ny, nx = t.shape[-2:]
    tg, tps = _target_planes(target, ny, nx, n)
    L = lib()
    work = torch.empty(max(1, L.xl_loss_work_bytes(n, ps) // 8), dtype=torch.float64, device=t.device)
    out = torch.empty(n, dtype=torch.float32, device=t.device)
    _lib.check(L.xl_norm_intensity_mse(stream_handle(), n, ps, int(cplx), t.data_ptr(), ps, tg.data_ptr(), tps,
                                       work.data_ptr(), out.data_ptr()), "xl_norm_intensity_mse")
    return out.reshape(x.shape[:-2]), work


def norm_intensity_mse_grad(x, target, work, g):
    t, n, ps, cplx = _loss_planes(x)
    ny, nx = t.shape[-2:]
    tg, tps = _target_planes(target, ny, nx, n)
    g = g.to(device=t.device, dtype=torch.float32).reshape(-1).contiguous()
    gin = torch.empty(t.shape, dtype=t.dtype, device=t.device)
    _lib.check(lib().xl_norm_intensity_mse_grad(stream_handle(), n, ps, int(cplx), t.data_ptr(), ps, tg.data_ptr(),
                                                tps, work.data_ptr(), g.data_ptr(), gin.data_ptr()),
               "xl_norm_intensity_mse_grad")
    return gin
