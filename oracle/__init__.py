"""CPU oracle for the mode-q tensor-times-vector path (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference arm import this package.  It is the checker, never the product:
the GPU engine in ``ttv_gb300`` neither imports nor links it.

Three libraries sit behind this module:

* ``liboracle.so`` -- ``ttv_oracle.c``, a plain-C restatement of the reference
  algorithm (bassoy/ttv ``include/tlib``), built on every host;
* ``_ref/libttvref.so`` -- the reference itself compiled from its own headers
  through ``ref_shim.cpp`` without BLAS (its plain loops); pins the
  restatement bit for bit;
* ``_ref/libttvref_blas.so`` -- the same headers with ``-DUSE_OPENBLAS``
  against the OpenBLAS that NumPy's wheel ships (``cblas_shim/cblas.h`` maps
  the standard CBLAS names onto its renamed symbols): the reference's
  configured BLAS path, timed as the CPU baseline.

The reference headers are compiled from ``baseline/_ref/include`` (git-ignored;
``make -C oracle stage-ref`` copies them there from a reference checkout, and
the copy travels with the repository to hosts without one), or from the
directory named by ``TTV_REFERENCE_INCLUDE``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libttvref.so")
REF_BLAS_PATH = os.path.join(HERE, "_ref", "libttvref_blas.so")
REF_BLAS_CFG = os.path.join(HERE, "_ref", "blas.cfg")
REF_INCLUDE = os.environ.get("TTV_REFERENCE_INCLUDE",
                             os.path.join(os.path.dirname(HERE), "baseline", "_ref", "include"))

_sz = C.c_size_t
_psz = C.POINTER(C.c_size_t)
_u64 = C.c_uint64
_vp = C.c_void_p

POLICIES = {
    "seq/subtensor/none": 0,
    "par_loop/subtensor/all": 1,
    "par_loop/slice/all": 2,
}

_lib = None
_ref = None


def find_blas():
    """OpenBLAS to build the reference's BLAS path against: (library path, symbol
    prefix, symbol suffix, ILP64) of the copy NumPy's wheel bundles, or None."""
    import ctypes.util
    import glob
    try:
        import numpy
        libdir = os.path.join(os.path.dirname(os.path.dirname(numpy.__file__)), "numpy.libs")
        cands = sorted(glob.glob(os.path.join(libdir, "lib*openblas*.so*")))
    except ImportError:
        cands = []
    sysblas = ctypes.util.find_library("openblas")
    if sysblas:
        cands.append(sysblas)
    for path in cands:
        try:
            L = C.CDLL(path)
        except OSError:
            continue
        for prefix, suffix, ilp64 in (("scipy_", "64_", True), ("", "64_", True), ("scipy_", "", False),
                                      ("", "", False)):
            names = [f"{prefix}{n}{suffix}" for n in ("cblas_sgemv", "cblas_dgemv",
                                                      "openblas_set_num_threads",
                                                      "openblas_get_num_threads")]
            if all(hasattr(L, n) for n in names):
                if not os.path.isabs(path):
                    continue   # a bare soname cannot be linked by path; skip it
                return path, prefix, suffix, ilp64
    return None


def blas_info():
    """What libttvref_blas.so was linked against (the text of _ref/blas.cfg), or None."""
    try:
        with open(REF_BLAS_CFG) as f:
            return f.read().strip() or None
    except OSError:
        return None


def build(with_ref: bool | None = None) -> None:
    """Compile liboracle.so and, where the reference headers are available (a
    reference checkout, or the staged copy in baseline/_ref/include), the two
    builds of the reference: _ref/libttvref.so and _ref/libttvref_blas.so."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref is False:
        return
    # refresh the staged headers where a reference checkout exists (no-op elsewhere)
    subprocess.run(["make", "-s", "-C", HERE, "stage-ref"], capture_output=True)
    if not os.path.isdir(os.path.join(REF_INCLUDE, "tlib")):
        if with_ref:
            raise FileNotFoundError(f"reference headers not found in {REF_INCLUDE}")
        return
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_INCLUDE={REF_INCLUDE}"], check=True)
    blas = find_blas()
    os.makedirs(os.path.dirname(REF_BLAS_CFG), exist_ok=True)
    cfg = "" if blas is None else f"{blas[0]} prefix={blas[1]} suffix={blas[2]} ilp64={int(blas[3])}"
    if blas_info() != (cfg or None):
        with open(REF_BLAS_CFG, "w") as f:
            f.write(cfg + "\n")
    if blas is None:
        if os.path.exists(REF_BLAS_PATH):
            os.remove(REF_BLAS_PATH)
        return
    subprocess.run(["make", "-s", "-C", HERE, "ref-blas", f"REF_INCLUDE={REF_INCLUDE}",
                    f"BLAS_LIB={blas[0]}", f"BLAS_PREFIX={blas[1]}", f"BLAS_SUFFIX={blas[2]}",
                    f"BLAS_ILP64={int(blas[3])}"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = C.CDLL(LIB_PATH)
        L.orc_check.restype = C.c_int
        L.orc_check.argtypes = [_sz, _sz, C.c_int, _psz, _psz, _psz, C.c_int, _psz, C.c_int,
                                _psz, _psz, _psz]
        L.orc_check_message.restype = C.c_char_p
        L.orc_check_message.argtypes = [C.c_int]
        for name in ("orc_ttv_f32", "orc_ttv_f64"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [C.c_int, _sz, _sz, _vp, _psz, _psz, _psz, _vp, _psz, _vp, _psz, _psz, _psz]
        for name in ("orc_canon_f32", "orc_canon_f64"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_u64, _u64, _u64, _vp, _vp, _vp]
        for name in ("orc_truth_f32", "orc_truth_f64", "orc_truth_bf16a"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_u64, _u64, _u64, _vp, _vp, _vp, _vp]
        for name in ("orc_truth_ttvs_f32", "orc_truth_ttvs_f64", "orc_truth_ttvs_bf16a"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_u64, _u64, _u64, _vp, _vp, _vp, _vp, _vp]
        L.orc_is_valid_shape.argtypes = [_psz, _sz]
        L.orc_is_valid_layout.argtypes = [_psz, _sz]
        L.orc_is_valid_strides.argtypes = [_psz, _sz, _psz]
        L.orc_output_shape.argtypes = [_psz, _sz, _sz, _psz]
        L.orc_output_layout.argtypes = [_psz, _sz, _sz, _psz]
        L.orc_strides.argtypes = [_psz, _psz, _sz, _psz]
        L.orc_k_order_layout.argtypes = [_sz, _sz, _psz]
        L.orc_inverse_mode.restype = _sz
        L.orc_inverse_mode.argtypes = [_psz, _sz, _sz]
        L.orc_case.argtypes = [_sz, _sz, _psz]
        L.orc_check_pic.argtypes = [_psz, _psz, _sz, _sz]
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_blas_available() -> bool:
    return os.path.exists(REF_BLAS_PATH)


def _bind_ref(path):
    L = C.CDLL(path)
    for name in ("ref_ttv_f32", "ref_ttv_f64"):
        f = getattr(L, name)
        f.restype = C.c_int
        f.argtypes = [C.c_int, _sz, _sz, _vp, _psz, _psz, _psz, _vp, _psz, _vp, _psz, _psz,
                      _psz, C.c_char_p, _sz]
    L.ref_output_shape.argtypes = [_psz, _sz, _sz, _psz]
    L.ref_output_layout.argtypes = [_psz, _sz, _sz, _psz]
    L.ref_strides.argtypes = [_psz, _psz, _sz, _psz]
    L.ref_k_order_layout.argtypes = [_sz, _sz, _psz]
    L.ref_is_valid_shape.argtypes = [_psz, _sz]
    L.ref_is_valid_layout.argtypes = [_psz, _sz]
    L.ref_is_valid_strides.argtypes = [_psz, _sz, _psz]
    L.ref_inverse_mode.restype = _sz
    L.ref_inverse_mode.argtypes = [_psz, _sz, _sz]
    return L


def ref() -> C.CDLL:
    """The reference compiled from source without BLAS (only where it could be built)."""
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("oracle/_ref/libttvref.so not built (reference headers absent)")
        _ref = _bind_ref(REF_PATH)
    return _ref


_ref_blas = None


def ref_blas() -> C.CDLL:
    """The reference compiled from source with -DUSE_OPENBLAS (its configured BLAS path)."""
    global _ref_blas
    if _ref_blas is None:
        if not ref_blas_available():
            raise FileNotFoundError("oracle/_ref/libttvref_blas.so not built (no OpenBLAS found)")
        _ref_blas = _bind_ref(REF_BLAS_PATH)
    return _ref_blas


# --------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------
def sizes(v):
    """A size_t array (kept alive by the caller) from a sequence, or None."""
    if v is None:
        return None
    arr = (C.c_size_t * max(len(v), 1))(*[int(x) for x in v])
    return arr


def _ptr(x):
    if x is None:
        return None
    return C.cast(x, _psz)


def _data(a):
    return None if a is None else a.ctypes.data_as(_vp)


def output_shape(na, q):
    nc = (C.c_size_t * max(len(na) - 1, 1))()
    if lib().orc_output_shape(_ptr(sizes(na)), len(na), q, nc) != 0:
        raise ValueError("invalid shape or mode")
    return [nc[i] for i in range(len(na) - 1)]


def output_layout(pia, q):
    pic = (C.c_size_t * max(len(pia) - 1, 1))()
    if lib().orc_output_layout(_ptr(sizes(pia)), len(pia), q, pic) != 0:
        raise ValueError("invalid layout or mode")
    return [pic[i] for i in range(len(pia) - 1)]


def strides(n, pi):
    w = (C.c_size_t * max(len(n), 1))()
    if lib().orc_strides(_ptr(sizes(n)), _ptr(sizes(pi)), len(n), w) != 0:
        raise ValueError("invalid shape or layout")
    return [w[i] for i in range(len(n))]


def k_order_layout(p, k):
    pi = (C.c_size_t * max(p, 1))()
    lib().orc_k_order_layout(p, k, pi)
    return [pi[i] for i in range(p)]


def inverse_mode(pi, mode):
    return lib().orc_inverse_mode(_ptr(sizes(pi)), len(pi), mode)


def case(p, q, pi):
    return lib().orc_case(p, q, _ptr(sizes(pi)))


def canonical(na, pia, q):
    """(P, nq, S): prefix before q in the layout, contracted extent, suffix."""
    k = list(pia).index(q)
    P = int(np.prod([na[m - 1] for m in pia[:k]], dtype=np.uint64)) if k else 1
    S = int(np.prod([na[m - 1] for m in pia[k + 1:]], dtype=np.uint64)) if k + 1 < len(pia) else 1
    return P, int(na[q - 1]), S


def check(q, p, a_ok, na, wa, pia, b_ok, nb, c_ok, nc, wc, pic):
    """Index of the first failing argument check of the low-level call (0 = ok)."""
    keep = [sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    return lib().orc_check(q, p, int(a_ok), *[_ptr(k) for k in keep[:3]], int(b_ok),
                           _ptr(keep[3]), int(c_ok), *[_ptr(k) for k in keep[4:]])


def check_message(code):
    return lib().orc_check_message(code).decode()


def ttv(policy, q, a, na, wa, pia, b, nb, nc, wc, pic, c=None):
    """Run the restated reference path; returns (status, c)."""
    a = np.ascontiguousarray(a)
    dt = a.dtype
    if c is None:
        c = np.zeros(int(np.prod(nc)) if nc else 1, dtype=dt)
    f = lib().orc_ttv_f32 if dt == np.float32 else lib().orc_ttv_f64
    keep = [sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    pol = POLICIES.get(policy, policy)
    st = f(pol, q, len(na), _data(a), *[_ptr(k) for k in keep[:3]], _data(b), _ptr(keep[3]),
           _data(c), *[_ptr(k) for k in keep[4:]])
    return st, c


def ref_ttv(policy, q, a, na, wa, pia, b, nb, nc, wc, pic, c=None, blas=False):
    """Run the reference compiled from source (blas=True: its OpenBLAS build);
    returns (status, message, c)."""
    a = np.ascontiguousarray(a)
    dt = a.dtype
    if c is None:
        c = np.zeros(int(np.prod(nc)) if nc else 1, dtype=dt)
    R = ref_blas() if blas else ref()
    f = R.ref_ttv_f32 if dt == np.float32 else R.ref_ttv_f64
    keep = [sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    msg = C.create_string_buffer(512)
    pol = POLICIES.get(policy, policy)
    st = f(pol, q, len(na), _data(a), *[_ptr(k) for k in keep[:3]], _data(b), _ptr(keep[3]),
           _data(c), *[_ptr(k) for k in keep[4:]], msg, 512)
    return st, msg.value.decode(), c


def canon(S, nq, P, a, b):
    """Canonical (S, nq, P) products with the reference's accumulation order."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    c = np.empty(int(S * P), dtype=a.dtype)
    f = lib().orc_canon_f32 if a.dtype == np.float32 else lib().orc_canon_f64
    f(S, nq, P, _data(a), _data(b), _data(c))
    return c


def truth(S, nq, P, a, b, kind=None):
    """FP64 (double-double accumulated) truth and the sum |a*b| per output."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    ref_ = np.empty(int(S * P), dtype=np.float64)
    absn = np.empty(int(S * P), dtype=np.float64)
    if kind == "bf16a" or a.dtype == np.uint16:
        lib().orc_truth_bf16a(S, nq, P, _data(a), _data(b.astype(np.float32)), _data(ref_),
                              _data(absn))
    elif a.dtype == np.float32:
        lib().orc_truth_f32(S, nq, P, _data(a), _data(b), _data(ref_), _data(absn))
    else:
        lib().orc_truth_f64(S, nq, P, _data(a), _data(b.astype(np.float64)), _data(ref_),
                            _data(absn))
    return ref_, absn


def kron_weights(na, pia, q, bs):
    """Kronecker weights (wS, wP) in double of the suffix and prefix modes of
    the canonical view w.r.t. q; bs in mode order without mode q."""
    vec = {}
    r = 0
    for m in range(1, len(na) + 1):
        if m == q:
            continue
        vec[m] = np.asarray(bs[r], dtype=np.float64)
        r += 1
    k = list(pia).index(q)
    wP = np.ones(1)
    for m in pia[:k]:           # prefix modes, fastest first: each new mode is slower
        wP = np.kron(vec[m], wP)
    wS = np.ones(1)
    for m in pia[k + 1:]:
        wS = np.kron(vec[m], wS)
    return wS, wP


def ttvs_truth(q, a, na, pia, bs, kind=None):
    """Double-double truth of the chain ttvs(q, A, bs) (every mode but q
    contracted) and sum |a w| per output, for A dense in layout pia."""
    P, nq, S = canonical(na, pia, q)
    wS, wP = kron_weights(na, pia, q, bs)
    a = np.ascontiguousarray(a)
    ref_ = np.empty(nq, dtype=np.float64)
    absn = np.empty(nq, dtype=np.float64)
    f = (lib().orc_truth_ttvs_bf16a if (kind == "bf16a" or a.dtype == np.uint16) else
         lib().orc_truth_ttvs_f32 if a.dtype == np.float32 else lib().orc_truth_ttvs_f64)
    f(S, nq, P, _data(a), _data(wS), _data(wP), _data(ref_), _data(absn))
    return ref_, absn


def rel_error(c, ref_, absn):
    """max_i |c_i - ref_i| / sum_k |a_ik b_k|  (component-wise, condition-normalised)."""
    c = np.asarray(c, dtype=np.float64)
    d = np.abs(c - ref_)
    den = np.where(absn > 0, absn, 1.0)
    return float(np.max(d / den)) if d.size else 0.0


def num_threads() -> int:
    return lib().orc_num_threads()
