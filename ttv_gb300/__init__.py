"""GB300-native mode-q tensor-times-vector engine (host mirror of tlib's API).

The compute lives in ``libttvgpu.so`` (hand-written sm_103a kernels behind the
C ABI of ``include/tlibg.h``); this module binds it with ctypes and mirrors
the reference library's interfaces on device memory:

* :func:`ttv` -- the low-level call ``tlib::ttv::ttv(ep, sp, fp, q, p, a, na,
  wa, pia, b, nb, c, nc, wc, pic)`` (reference ``include/tlib/ttv.h:54-92``)
  on device pointers; raises :class:`TTVError` with the reference's message
  for every invalid call.
* :func:`ttv_array` / :func:`ttvs` -- ``ttvpy.ttv(q, A, b)`` and
  ``ttvpy.ttvs(q, A, bs, order)`` (reference ``ttvpy/src/wrapped_ttv.cpp:
  20-78, 85-199``) on torch CUDA tensors, with the same last-order
  (row-major) layout convention.
* metadata helpers ``output_shape``, ``output_layout``, ``strides``,
  ``k_order_layout`` (reference ``detail/shape.h``, ``layout.h``,
  ``strides.h``).

There is no CPU fallback: without the built library or a CUDA device every
compute call raises.
"""
from __future__ import annotations

import ctypes as C
import os

__all__ = [
    "TTVError", "UnsupportedError", "ttv", "ttv_ex", "ttv_host", "ttv_array", "ttvs", "plan",
    "output_shape", "output_layout", "strides", "k_order_layout", "inverse_mode",
    "library", "library_path", "launch_count", "device_error", "device_alloc_count",
    "plan_hint", "clear_plan_hint", "F32", "F64", "BF16A",
    "ACC_COMPENSATED", "ACC_PLAIN", "ACC_DOUBLE_FLOAT", "KIND_ROW", "KIND_COL", "KIND_STREAM",
    "KIND_COL_REALIGN", "KIND_COL_THIN", "KIND_ROW_TILE", "KIND_COL_BULK", "KIND_ROW_PANEL",
    "KIND_ROW_SHIFT", "ttv_strided", "ttv_view",
]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libttvgpu.so")

F32, F64, BF16A = 0, 1, 2
ACC_COMPENSATED, ACC_PLAIN, ACC_DOUBLE_FLOAT = 0, 1, 2
KIND_ROW, KIND_COL, KIND_STREAM, KIND_COL_REALIGN, KIND_COL_THIN, KIND_ROW_TILE, KIND_COL_BULK, \
    KIND_ROW_PANEL, KIND_ROW_SHIFT = 0, 1, 2, 3, 4, 5, 6, 7, 8
OK, ERR_ARGUMENT, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT = range(6)


class TTVError(RuntimeError):
    """An invalid call: same text as the reference's std::runtime_error."""


class UnsupportedError(TTVError):
    """Valid for the reference but outside this engine (e.g. non-dense strides)."""


class DeviceError(RuntimeError):
    """CUDA failure, missing device, out of memory or an expired device wait."""


class Options(C.Structure):
    _fields_ = [("accumulate", C.c_int), ("kind", C.c_int), ("group", C.c_int),
                ("vec", C.c_int), ("split", C.c_int), ("sync", C.c_int)]


class PlanInfo(C.Structure):
    _fields_ = [("P", C.c_uint64), ("nq", C.c_uint64), ("S", C.c_uint64), ("kind", C.c_int),
                ("group", C.c_int), ("vec", C.c_int), ("split", C.c_int),
                ("accumulate", C.c_int), ("grid", C.c_int), ("block", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_sz = C.c_size_t
_psz = C.POINTER(C.c_size_t)
_vp = C.c_void_p
_lib = None


def library_path() -> str:
    return LIB_PATH


def library() -> C.CDLL:
    """The engine's shared library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m ttv_gb300.build` "
                "(the engine has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        sig = [_sz, _sz, _vp, _psz, _psz, _psz, _vp, _psz, _vp, _psz, _psz, _psz]
        for name in ("tlibg_ttv_f32", "tlibg_ttv_f64", "tlibg_ttv_bf16a_f32"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = sig + [_vp]
        L.tlibg_ttv_ex.restype = C.c_int
        L.tlibg_ttv_ex.argtypes = [C.c_int] + sig + [C.POINTER(Options), _vp]
        L.tlibg_ttv_host.restype = C.c_int
        L.tlibg_ttv_host.argtypes = [C.c_int] + sig + [C.POINTER(Options)]
        L.tlibg_validate.restype = C.c_int
        L.tlibg_validate.argtypes = [_sz, _sz, _psz, _psz, _psz, _psz, _psz, _psz, _psz]
        L.tlibg_plan.restype = C.c_int
        L.tlibg_plan.argtypes = [C.c_int, _sz, _sz, _psz, _psz, C.POINTER(Options),
                                 C.POINTER(PlanInfo)]
        L.tlibg_output_shape.argtypes = [_psz, _sz, _sz, _psz]
        L.tlibg_output_layout.argtypes = [_psz, _sz, _sz, _psz]
        L.tlibg_strides.argtypes = [_psz, _psz, _sz, _psz]
        L.tlibg_k_order_layout.argtypes = [_sz, _sz, _psz]
        L.tlibg_inverse_mode.restype = _sz
        L.tlibg_inverse_mode.argtypes = [_psz, _sz, _sz]
        L.tlibg_last_error.restype = _sz
        L.tlibg_last_error.argtypes = [C.c_char_p, _sz]
        L.tlibg_device_error.restype = C.c_int
        L.tlibg_launch_count.restype = C.c_uint64
        L.tlibg_ttvs.restype = C.c_int
        L.tlibg_ttvs.argtypes = [C.c_int, _sz, _sz, _vp, _psz, _psz, _psz, C.POINTER(_vp), _psz,
                                 _vp, _vp]
        L.tlibg_ttv_strided.restype = C.c_int
        L.tlibg_ttv_strided.argtypes = [C.c_int, _sz, _sz, _vp, _psz, _psz, _psz, _vp, _psz, _sz, _vp,
                                        _psz, _psz, _psz, _vp]
        L.tlibg_device_alloc_count.restype = C.c_uint64
        L.tlibg_plan_hint.restype = C.c_int
        L.tlibg_plan_hint.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64,
                                      C.POINTER(Options)]
        L.tlibg_version.restype = C.c_char_p
        _lib = L
    return _lib


def _last_error() -> str:
    buf = C.create_string_buffer(1024)
    library().tlibg_last_error(buf, 1024)
    return buf.value.decode()


def _raise(status: int):
    if status == OK:
        return
    msg = _last_error()
    if status == ERR_ARGUMENT:
        raise TTVError(msg)
    if status == ERR_UNSUPPORTED:
        raise UnsupportedError(msg)
    raise DeviceError(f"status {status}: {msg}")


def _sizes(v):
    if v is None:
        return None
    n = len(v)
    return (C.c_size_t * max(n, 1))(*[int(x) for x in v])


def _p(arr):
    return None if arr is None else C.cast(arr, _psz)


def _ptr(x):
    """Device pointer of a torch tensor (or an int address, or None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream_handle(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _options(accumulate=ACC_COMPENSATED, kind=-1, group=0, vec=0, split=0, sync=False):
    return Options(int(accumulate), int(kind), int(group), int(vec), int(split), int(bool(sync)))


# --------------------------------------------------------------------------
# low-level call (reference ttv.h:54-92)
# --------------------------------------------------------------------------
def ttv(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, *, dtype=None, stream=None, **opts):
    """C = A x_q b on device memory, the reference's low-level argument list.

    ``a``, ``b``, ``c`` are torch CUDA tensors (or device addresses); ``na``,
    ``wa``, ``pia``, ``nb``, ``nc``, ``wc``, ``pic`` host sequences of sizes
    (one-based modes and layouts, as tlib).  ``dtype`` defaults to the tensor
    dtype (float32 / float64; bfloat16 A with float32 b and c selects the
    bf16-stored path).  Keyword options: accumulate, kind, group, vec, split,
    sync.  Work is enqueued on ``stream`` (default: torch's current stream).
    """
    if dtype is None:
        dtype = _dtype_of(a)
    keep = [_sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    _check_buffers(dtype, q, p, keep, a, b, c)
    o = _options(**opts)
    st = library().tlibg_ttv_ex(dtype, q, p, _ptr(a), _p(keep[0]), _p(keep[1]), _p(keep[2]),
                                _ptr(b), _p(keep[3]), _ptr(c), _p(keep[4]), _p(keep[5]),
                                _p(keep[6]), C.byref(o), _stream_handle(stream))
    _raise(st)
    return c


ttv_ex = ttv

_ELEM_BYTES = {F32: (4, 4, 4), F64: (8, 8, 8), BF16A: (2, 4, 4)}


def _addressed(n, w):
    """Elements a dense tensor with extents n and strides w spans (0 if empty)."""
    if any(int(x) == 0 for x in n):
        return 0
    return 1 + sum((int(x) - 1) * int(s) for x, s in zip(n, w))


def _check_buffers(dtype, q, p, keep, a, b, c):
    """Refuse tensors smaller than the memory their layout addresses, before
    any launch: the kernels trust the metadata as the reference does.  Runs
    after the reference's own checks (same messages, same order) and only for
    sized buffers (torch tensors); raw addresses are the caller's contract."""
    bufs = [(name, t) for name, t in (("a", a), ("b", b), ("c", c)) if hasattr(t, "numel")]
    if not bufs or dtype not in _ELEM_BYTES:
        return
    na, wa, pia, nb, nc, wc, pic = keep
    if len(na) < p or len(wa) < p or len(nb) < 1 or (p > 1 and (len(nc) < p - 1 or len(wc) < p - 1)):
        return   # malformed metadata: the C ABI reports it
    _raise(library().tlibg_validate(q, p, _p(na), _p(wa), _p(pia), _p(nb), _p(nc), _p(wc), _p(pic)))
    need = {"a": _addressed(na[:p], wa[:p]), "b": int(nb[0]),
            "c": _addressed(nc[:p - 1], wc[:p - 1])}
    esz = dict(zip("abc", _ELEM_BYTES[dtype]))
    for name, t in bufs:
        have = t.numel() * t.element_size()
        if have < need[name] * esz[name]:
            raise TTVError(f"tlibg: buffer {name} holds {have} bytes, its layout addresses "
                           f"{need[name] * esz[name]}")


def ttv_strided(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, *, wb=1, dtype=None, stream=None):
    """Extension: C = A x_q b on device memory with the natural meaning of every
    stride (tlibg_ttv_strided): A's element (i_1..i_p) at a[sum i_r wa[r]], b's
    i-th at b[i wb], C's at c[sum j_r wc[r]] (zero-based, in elements), for
    sliced, padded or transposed views.  Same checks and messages as ``ttv``
    for shapes, layouts and monotonic strides; refused when two outputs would
    share an element of C.  Tensors must hold every element their strides
    address."""
    if dtype is None:
        dtype = _dtype_of(a)
    keep = [_sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    need = {"a": _addressed(keep[0][:p], keep[1][:p]),
            "b": (int(keep[3][0]) - 1) * int(wb) + 1 if len(keep[3]) and int(keep[3][0]) else 0,
            "c": _addressed(keep[4][:p - 1], keep[5][:p - 1]) if p > 1 else 0}
    for name, t in (("a", a), ("b", b), ("c", c)):
        if hasattr(t, "untyped_storage"):
            # elements from the tensor's first element to the end of its storage (views too)
            have = t.untyped_storage().nbytes() // t.element_size() - t.storage_offset()
            if have < need[name]:
                raise TTVError(f"tlibg: buffer {name} holds {have} elements, its strides address "
                               f"{need[name]}")
    st = library().tlibg_ttv_strided(dtype, q, p, _ptr(a), _p(keep[0]), _p(keep[1]), _p(keep[2]),
                                     _ptr(b), _p(keep[3]), int(wb), _ptr(c), _p(keep[4]), _p(keep[5]),
                                     _p(keep[6]), _stream_handle(stream))
    _raise(st)
    return c


def ttv_view(q, A, b, out=None, *, stream=None):
    """``ttv_array`` for any strided torch view (slices, transposes, padding)
    without a copy: A's own strides go to tlibg_ttv_strided; b may be strided
    too.  Returns C (the modes of A without q, in order), contiguous, or fills
    ``out`` (any strides that give every output its own element)."""
    torch = _torch()
    p = A.dim()
    if not 1 <= q <= p:
        raise TTVError("Error in tlib::tensor_times_vector: contraction mode should be greater zero or "
                       "less than or equal to p.")
    na = list(A.shape)
    wa = list(A.stride())
    shape_c = [n for m, n in enumerate(na) if m != q - 1]
    if out is None:
        out = torch.empty(shape_c, dtype=A.dtype, device=A.device)
    wc = list(out.stride())
    # layouts that pass the reference's monotonic-stride check: modes by increasing stride
    pia = [m + 1 for m in sorted(range(p), key=lambda m: (wa[m], m))]
    pic = [m + 1 for m in sorted(range(p - 1), key=lambda m: (wc[m], m))] or [1]
    return ttv_strided(q, p, A, na, wa, pia, b, [int(b.shape[0])], out, shape_c or [1], wc or [1], pic,
                       wb=int(b.stride(0)), stream=stream)


def ttv_host(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, *, dtype=None, **opts):
    """The low-level call on HOST buffers (numpy arrays or pinned torch CPU
    tensors): copies in, computes on the GPU, copies C back, returns when done."""
    if dtype is None:
        dtype = _dtype_of(a)
    keep = [_sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    o = _options(**opts)
    st = library().tlibg_ttv_host(dtype, q, p, _host_ptr(a), _p(keep[0]), _p(keep[1]),
                                  _p(keep[2]), _host_ptr(b), _p(keep[3]), _host_ptr(c),
                                  _p(keep[4]), _p(keep[5]), _p(keep[6]), C.byref(o))
    _raise(st)
    return c


def _host_ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    return x.data_ptr()


def _dtype_of(a):
    name = str(getattr(a, "dtype", "float32"))
    if "float64" in name or name.endswith("double"):
        return F64
    if "bfloat16" in name or "uint16" in name:
        return BF16A
    return F32


def plan(q, na, pia, dtype=F32, **opts):
    """The kernel configuration the engine picks for a dense problem."""
    info = PlanInfo()
    o = _options(**opts)
    st = library().tlibg_plan(dtype, q, len(na), _p(_sizes(na)), _p(_sizes(pia)), C.byref(o),
                              C.byref(info))
    _raise(st)
    return info.as_dict()


# --------------------------------------------------------------------------
# metadata helpers (reference detail/shape.h, layout.h, strides.h)
# --------------------------------------------------------------------------
def output_shape(na, q):
    p = len(na)
    out = (C.c_size_t * max(p - 1, 1))()
    _raise(library().tlibg_output_shape(_p(_sizes(na)), p, q, out))
    return [out[i] for i in range(p - 1)]


def output_layout(pia, q):
    p = len(pia)
    out = (C.c_size_t * max(p - 1, 1))()
    _raise(library().tlibg_output_layout(_p(_sizes(pia)), p, q, out))
    return [out[i] for i in range(p - 1)]


def strides(n, pi):
    p = len(n)
    out = (C.c_size_t * max(p, 1))()
    _raise(library().tlibg_strides(_p(_sizes(n)), _p(_sizes(pi)), p, out))
    return [out[i] for i in range(p)]


def k_order_layout(p, k):
    out = (C.c_size_t * max(p, 1))()
    _raise(library().tlibg_k_order_layout(p, k, out))
    return [out[i] for i in range(p)]


def inverse_mode(pi, mode):
    r = library().tlibg_inverse_mode(_p(_sizes(pi)), len(pi), mode)
    if r == 0:
        raise TTVError(_last_error())
    return r


def device_alloc_count() -> int:
    """Device allocations (cudaMalloc) the engine made since load."""
    return int(library().tlibg_device_alloc_count())


def plan_hint(dtype, P, nq, S, **options):
    """Install autotuned options for the canonical problem (dtype, P, n_q, S):
    later calls that leave every choice to the planner use them."""
    o = _options(**options)
    _raise(library().tlibg_plan_hint(dtype, P, nq, S, C.byref(o)))


def clear_plan_hint(dtype=0, P=0, nq=0, S=0):
    """Remove one plan hint, or all of them (the default)."""
    _raise(library().tlibg_plan_hint(dtype, P, nq, S, None))


def launch_count() -> int:
    return int(library().tlibg_launch_count())


def device_error() -> int:
    return int(library().tlibg_device_error())


# --------------------------------------------------------------------------
# array-level API (reference ttvpy: wrapped_ttv.cpp)
# --------------------------------------------------------------------------
def _torch():
    import torch
    return torch


def ttv_array(q, A, b, *, out=None, stream=None, **opts):
    """``ttvpy.ttv(q, A, b)`` on a torch CUDA tensor A (row-major, i.e. the
    last-order layout pia = (p, ..., 1)) and vector b; returns C with A's
    shape minus mode q (wrapped_ttv.cpp:20-78)."""
    torch = _torch()
    p = A.dim()
    if p == 0:
        raise ValueError("Error calling ttvpy::ttv: input tensor order should be greater than zero.")
    if q == 0 or q > p:
        raise ValueError("Error calling ttvpy::ttv: contraction mode should be greater than zero "
                         "or less than or equal to p.")
    if not A.is_contiguous():
        A = A.contiguous()
    na = list(A.shape)
    pia = list(range(p, 0, -1))
    wa = [s for s in A.stride()]
    nc = output_shape(na, q)
    pic = output_layout(pia, q)
    wc = strides(nc, pic)
    cdt = torch.float32 if A.dtype == torch.bfloat16 else A.dtype
    if out is None:
        out = torch.empty(nc, dtype=cdt, device=A.device)
    dt = BF16A if A.dtype == torch.bfloat16 else (F64 if A.dtype == torch.float64 else F32)
    a_ptr = A.view(torch.int16) if dt == BF16A else A
    ttv(q, p, a_ptr, na, wa, pia, b, [b.shape[0]], out, nc, wc, pic, dtype=dt, stream=stream,
        **opts)
    return out


def ttvs(q, A, bs, order="optimal", *, stream=None, fused=True, **opts):
    """``ttvpy.ttvs(q, A, bs, order)``: contract every mode except q with the
    vectors bs (one per mode r != q, in mode order), in "forward",
    "backward" or "optimal" (largest vector first) order
    (wrapped_ttv.cpp:85-199).  Returns a vector of length A.shape[q-1].

    By default the chain runs fused in the engine (``tlibg_ttvs``): A is read
    once whatever the order, which then only names the reference's rounding
    sequence.  ``fused=False`` (or any kernel option) runs the reference's
    step-by-step chain, one engine TTV per vector in the given order."""
    if order not in ("optimal", "backward", "forward"):
        raise ValueError("Error calling ttvpy::ttvs: multiplication order should be either "
                         "'optimal', 'backward' or 'forward'.")
    p = A.dim()
    if p == 0:
        raise ValueError("Error calling ttvpy::ttvs: input tensor order should be greater than zero.")
    if len(bs) != p - 1:
        raise ValueError("Error calling ttvpy::ttvs: number of input vectors is not equal to the "
                         "tensor order - 1.")
    if q == 0 or q > p:
        raise ValueError("Error calling ttvpy::ttvs: contraction mode should be greater than zero "
                         "or less than or equal to p.")
    if any(bj.dim() != 1 for bj in bs):
        raise ValueError("Error calling ttvpy::ttvs: some of the input vectors is not a vector.")
    na = list(A.shape)
    nb = [int(bj.shape[0]) for bj in bs]
    if nb[:q - 1] != na[:q - 1] or nb[q - 1:] != na[q:]:
        raise ValueError("Error calling ttvpy::ttvs: vector dimension is not compatible with the "
                         "dimension of a tensor mode.")
    if fused and not opts and p > 1:
        return _ttvs_fused(q, A, bs, stream)
    # modes contracted, as (one-based mode of A, vector)
    pairs = [(r, bs[r - 1]) for r in range(1, q)] + [(r, bs[r - 2]) for r in range(q + 1, p + 1)]
    if order == "backward":
        seq = sorted(pairs, key=lambda t: -t[0])
    elif order == "forward":
        seq = sorted(pairs, key=lambda t: t[0])
    else:
        # largest vector first (stable among equals by descending mode, as the
        # reference walks its ascending sort from the back)
        seq = sorted(pairs, key=lambda t: (int(t[1].shape[0]), t[0]), reverse=True)
    C_ = A
    remaining = [r for r, _ in pairs]
    for r, bj in seq:
        cur = 1 + sum(1 for m in remaining if m < r) + (1 if q < r else 0)
        C_ = ttv_array(cur, C_, bj, stream=stream, **opts)
        remaining.remove(r)
    return C_


def _ttvs_fused(q, A, bs, stream):
    torch = _torch()
    p = A.dim()
    if not A.is_contiguous():
        A = A.contiguous()
    dt = BF16A if A.dtype == torch.bfloat16 else (F64 if A.dtype == torch.float64 else F32)
    vdt = torch.float64 if dt == F64 else torch.float32
    vecs = [bj.to(device=A.device, dtype=vdt).contiguous() for bj in bs]
    na = list(A.shape)
    pia = list(range(p, 0, -1))
    wa = list(A.stride())
    out = torch.empty(na[q - 1], dtype=vdt, device=A.device)
    keep = [_sizes(v) for v in (na, wa, pia, [int(v.shape[0]) for v in vecs])]
    ptrs = (_vp * len(vecs))(*[v.data_ptr() for v in vecs])
    a_ptr = A.view(torch.int16) if dt == BF16A else A
    st = library().tlibg_ttvs(dt, q, p, _ptr(a_ptr), _p(keep[0]), _p(keep[1]), _p(keep[2]), ptrs,
                              _p(keep[3]), out.data_ptr(), _stream_handle(stream))
    _raise(st)
    return out
