"""Batched TTVs and the learned cost model (host side, ctypes over the C ABI).

    from ttv_gb300 import batch as B
    probs = [B.Problem(q, na, pia, A, b, c), ...]       # torch CUDA tensors
    bt = B.Batch(probs, select=B.SELECT_LEARNED)          # descriptors + CUDA graph
    bt.launch()                                           # one persistent launch
    bt.variants()                                         # what each problem ran with

The cost model (``set_cost_model``, ``mlp_*``) is the engine's MLP: its
forward, backward and Adam steps are hand-written CUDA kernels in the library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import F32, _check_buffers, _last_error, _options, _p, _raise, _sizes, library, \
    output_layout, output_shape, strides

SELECT_HEURISTIC, SELECT_LEARNED, SELECT_FIXED, SELECT_GIVEN = 0, 1, 2, 3
NVARIANT = 9
VARIANT_STAGED = 8   # q-fastest rows of at most 64 elements through shared memory
MLP_FEATURES, MLP_IN, MLP_HIDDEN, MLP_PARAMS = 8, 17, 64, 9537
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
MODEL_PATH = os.path.join(DATA, "cost_model.npz")

_vp = C.c_void_p
_psz = C.POINTER(C.c_size_t)


class _Problem(C.Structure):
    _fields_ = [("q", C.c_size_t), ("p", C.c_size_t), ("a", _vp), ("na", _psz), ("wa", _psz),
                ("pia", _psz), ("b", _vp), ("nb", _psz), ("c", _vp), ("nc", _psz), ("wc", _psz),
                ("pic", _psz)]


class _BatchOptions(C.Structure):
    _fields_ = [("select", C.c_int), ("variant", C.c_int), ("accumulate", C.c_int),
                ("no_graph", C.c_int), ("variants", C.POINTER(C.c_int)),
                ("record_costs", C.c_int)]


_bound = False


def _lib():
    global _bound
    L = library()
    if not _bound:
        P = C.POINTER(_Problem)
        L.tlibg_batch_create.restype = C.c_int
        L.tlibg_batch_create.argtypes = [C.c_int, P, C.c_size_t, C.POINTER(_BatchOptions), _vp,
                                         C.POINTER(_vp)]
        L.tlibg_batch_launch.argtypes = [_vp, _vp]
        L.tlibg_batch_variants.argtypes = [_vp, C.POINTER(C.c_int), _vp]
        L.tlibg_batch_set_variant.argtypes = [_vp, C.c_int]
        L.tlibg_batch_costs.argtypes = [_vp, C.POINTER(C.c_uint64), _vp]
        L.tlibg_batch_destroy.argtypes = [_vp]
        L.tlibg_ttv_batch.argtypes = [C.c_int, P, C.c_size_t, C.POINTER(_BatchOptions), _vp]
        L.tlibg_ttv_percall.argtypes = [C.c_int, P, C.c_size_t, _vp]
        L.tlibg_ttv_batch_f32.argtypes = [P, C.c_int, _vp]
        L.tlibg_batch_features.argtypes = [P, C.c_size_t, C.POINTER(C.c_float),
                                           C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.tlibg_batch_device_error.restype = C.c_uint
        fp = C.POINTER(C.c_float)
        L.tlibg_mlp_loss_grad.argtypes = [_vp, _vp, _vp, C.c_size_t, _vp, _vp, _vp]
        L.tlibg_mlp_adam.argtypes = [_vp, _vp, _vp, _vp, C.c_uint64, C.c_float, C.c_float,
                                     C.c_float, C.c_float, _vp]
        L.tlibg_mlp_predict.argtypes = [_vp, _vp, C.c_size_t, _vp, _vp]
        L.tlibg_mlp_train.argtypes = [_vp, _vp, _vp, _vp, _vp, C.c_size_t, C.c_int, C.c_int,
                                      C.c_float, C.c_uint64, fp, _vp]
        L.tlibg_set_cost_model.argtypes = [fp, C.c_size_t, C.c_float]
        _bound = True
    return L


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream if isinstance(stream, int) else stream.cuda_stream


class Problem:
    """One TTV of a batch: A, b, c device tensors (fp32), dense layout pia."""

    def __init__(self, q, na, pia, a, b, c):
        self.q, self.na, self.pia = int(q), [int(x) for x in na], [int(x) for x in pia]
        self.a, self.b, self.c = a, b, c
        wa = strides(self.na, self.pia)
        nc, pic = output_shape(self.na, self.q), output_layout(self.pia, self.q)
        wc = strides(nc, pic)
        self._keep = [_sizes(v) for v in (self.na, wa, self.pia, [self.na[self.q - 1]], nc, wc,
                                          pic)]
        _check_buffers(F32, self.q, len(self.na), self._keep, a, b, c)

    def _struct(self):
        k = self._keep
        ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
        return _Problem(self.q, len(self.na), ptr(self.a), _p(k[0]), _p(k[1]), _p(k[2]),
                        ptr(self.b), _p(k[3]), ptr(self.c), _p(k[4]), _p(k[5]), _p(k[6]))


def _array(problems):
    arr = (_Problem * len(problems))(*[pr._struct() for pr in problems])
    return arr


def _opts(select, variant, accumulate, no_graph, variants, record=False):
    keep = None
    o = _BatchOptions(select, variant, accumulate, int(bool(no_graph)), None, int(bool(record)))
    if variants is not None:
        keep = (C.c_int * len(variants))(*[int(v) for v in variants])
        o.variants = C.cast(keep, C.POINTER(C.c_int))
    return o, keep


class Batch:
    """Descriptors of many problems plus the CUDA graph of one launch."""

    def __init__(self, problems, select=SELECT_HEURISTIC, variant=0, accumulate=0,
                 no_graph=False, variants=None, stream=None, record_costs=False):
        self.problems = list(problems)
        self._arr = _array(self.problems)
        self._opt, self._vkeep = _opts(select, variant, accumulate, no_graph, variants,
                                       record_costs)
        h = _vp()
        st = _lib().tlibg_batch_create(0, self._arr, len(self.problems), C.byref(self._opt),
                                       _stream(stream), C.byref(h))
        _raise(st)
        self._h = h

    def launch(self, stream=None):
        _raise(_lib().tlibg_batch_launch(self._h, _stream(stream)))

    def set_variant(self, v):
        """Change the forced variant of a SELECT_FIXED batch built with no_graph."""
        _raise(_lib().tlibg_batch_set_variant(self._h, int(v)))

    def costs(self, stream=None):
        """SM cycles of each problem in the last launch (record_costs batches): its
        units' clock cycles over the CTAs (staged rows: warps) resident per SM."""
        out = np.zeros(len(self.problems), np.uint64)
        _raise(_lib().tlibg_batch_costs(self._h, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                        _stream(stream)))
        return out

    def variants(self, stream=None):
        out = (C.c_int * len(self.problems))()
        _raise(_lib().tlibg_batch_variants(self._h, out, _stream(stream)))
        return np.array(out[:], dtype=np.int32)

    def close(self):
        if getattr(self, "_h", None):
            _lib().tlibg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def ttv_batch(problems, select=SELECT_HEURISTIC, variant=0, variants=None, stream=None):
    arr = _array(problems)
    o, keep = _opts(select, variant, 0, True, variants)
    _raise(_lib().tlibg_ttv_batch(0, arr, len(problems), C.byref(o), _stream(stream)))


def ttv_batch_f32(problems, stream=None):
    """tlibg_ttv_batch_f32: one synchronous call, learned selection (fixed rule
    when no cost model is installed)."""
    arr = _array(problems)
    _raise(_lib().tlibg_ttv_batch_f32(arr, len(problems), _stream(stream)))


def ttv_percall(problems, stream=None):
    """The plain alternative: one tlibg_ttv_ex launch per problem."""
    arr = _array(problems)
    _raise(_lib().tlibg_ttv_percall(0, arr, len(problems), _stream(stream)))


def features(problems):
    """(features [n, 8], kernel family [n], fixed-rule variant [n])."""
    n = len(problems)
    arr = _array(problems)
    f = np.zeros((n, MLP_FEATURES), np.float32)
    kind = np.zeros(n, np.int32)
    heur = np.zeros(n, np.int32)
    _raise(_lib().tlibg_batch_features(arr, n, f.ctypes.data_as(C.POINTER(C.c_float)),
                                       kind.ctypes.data_as(C.POINTER(C.c_int)),
                                       heur.ctypes.data_as(C.POINTER(C.c_int))))
    return f, kind, heur


def batch_device_error() -> int:
    return int(_lib().tlibg_batch_device_error())


# --------------------------------------------------------------------------
# cost model
# --------------------------------------------------------------------------
def set_cost_model(params, margin=0.0):
    """Install (numpy float32 [9537]) or clear (None) the model SELECT_LEARNED uses;
    a problem leaves the fixed rule only for a predicted gain beyond ``margin``."""
    if params is None:
        _raise(_lib().tlibg_set_cost_model(None, 0, 0.0))
        return
    p = np.ascontiguousarray(params, dtype=np.float32)
    _raise(_lib().tlibg_set_cost_model(p.ctypes.data_as(C.POINTER(C.c_float)), p.size,
                                       float(margin)))


def load_cost_model(path=MODEL_PATH, install=True):
    """The committed trained weights (None if absent); installs them by default."""
    if not os.path.exists(path):
        return None
    d = np.load(path)
    params = d["params"].astype(np.float32)
    if params.size != MLP_PARAMS:   # trained for another variant set: not usable
        return None
    margin = float(d["margin"]) if "margin" in d else 0.0
    if install:
        set_cost_model(params, margin)
    return params


def init_params(seed=0):
    """He-initialised parameters (host, float32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((MLP_IN, MLP_HIDDEN), (MLP_HIDDEN, MLP_HIDDEN),
                            (MLP_HIDDEN, MLP_HIDDEN)):
        parts.append(rng.standard_normal((fan_in, fan_out)) * np.sqrt(2.0 / fan_in))
        parts.append(np.zeros(fan_out))
    parts.append(rng.standard_normal(MLP_HIDDEN) * np.sqrt(1.0 / MLP_HIDDEN))
    parts.append(np.zeros(1))
    out = np.concatenate([p.ravel() for p in parts]).astype(np.float32)
    assert out.size == MLP_PARAMS
    return out


def mlp_loss_grad(params, x, y, stream=None):
    """(loss, grad) of the mean squared error on device tensors."""
    import torch
    grad = torch.empty(MLP_PARAMS, device=params.device, dtype=torch.float32)
    loss = torch.empty(1, device=params.device, dtype=torch.float32)
    _raise(_lib().tlibg_mlp_loss_grad(params.data_ptr(), x.data_ptr(), y.data_ptr(), x.shape[0],
                                      grad.data_ptr(), loss.data_ptr(), _stream(stream)))
    return loss, grad


def mlp_adam(params, grad, m, v, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
    _raise(_lib().tlibg_mlp_adam(params.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(),
                                 step, lr, beta1, beta2, eps, _stream(stream)))


def mlp_predict(params, x, stream=None):
    import torch
    y = torch.empty(x.shape[0], device=x.device, dtype=torch.float32)
    _raise(_lib().tlibg_mlp_predict(params.data_ptr(), x.data_ptr(), x.shape[0], y.data_ptr(),
                                    _stream(stream)))
    return y


def mlp_train(params, x, y, epochs=30, batch=512, lr=1e-3, seed=0, stream=None):
    """Train in place (device tensors); returns the per-epoch mean loss."""
    import torch
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    losses = np.zeros(epochs, np.float32)
    _raise(_lib().tlibg_mlp_train(params.data_ptr(), m.data_ptr(), v.data_ptr(), x.data_ptr(),
                                  y.data_ptr(), x.shape[0], epochs, batch, lr, seed,
                                  losses.ctypes.data_as(C.POINTER(C.c_float)), _stream(stream)))
    return losses


def mlp_inputs(feat, nvariant=NVARIANT):
    """Rows (features, one-hot variant) for every (problem, variant)."""
    n = feat.shape[0]
    x = np.zeros((n * nvariant, MLP_IN), np.float32)
    x[:, :MLP_FEATURES] = np.repeat(feat, nvariant, axis=0)
    x[np.arange(n * nvariant), MLP_FEATURES + np.tile(np.arange(nvariant), n)] = 1.0
    return x
