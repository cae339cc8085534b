"""Parity at full size: every TTV of the symmetric and asymmetric sweeps that
the benchmark times, through the C ABI's drop-in entry points
(tlibg_ttv_f32 / tlibg_ttv_f64), against the oracle's double-double truth on
the same seeded inputs.

* symmetric sweep: p = 2..7, n = floor(2^(28/p)) in integers (16384, 645,
  128, 48, 25, 16), every q, first-order and last-order layouts, fp32 and
  fp64 (108 TTVs of about 2^28 elements);
* asymmetric sweep: p = 2..10, n_1 = 2^(28 - 2(p-1)), n_k = 4, every q,
  first-order, fp32 (54 TTVs of 2^28 elements).

Inputs: A and b uniform[-1, 1] from a fixed seed (one array per dtype, each
case reads its leading N elements).  Error metric: max_i |c_i - ref_i| /
sum_k |a_ik b_k|, bars 1e-5 (fp32) and 1e-13 (fp64).  C is filled with NaN
before every call, so an output the kernels never write fails the check.
Every case runs (about 0.1-0.3 s of oracle time each); failures are listed
together at the end.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f64": 1e-13}


def int_root(p, bits=28):
    """Largest n with n**p <= 2**bits."""
    n = int(round(2 ** (bits / p)))
    while n ** p > 2 ** bits:
        n -= 1
    while (n + 1) ** p <= 2 ** bits:
        n += 1
    return n


def sym_cases(dtype):
    out = []
    for p in range(2, 8):
        n = int_root(p)
        for pia in (list(range(1, p + 1)), list(range(p, 0, -1))):
            for q in range(1, p + 1):
                out.append(([n] * p, pia, q))
    return out


def asym_cases():
    out = []
    for p in range(2, 11):
        na = [2 ** (28 - 2 * (p - 1))] + [4] * (p - 1)
        for q in range(1, p + 1):
            out.append((na, list(range(1, p + 1)), q))
    return out


@pytest.fixture(scope="module")
def inputs(cuda):
    """Host and device copies of A and b per dtype (2^28 elements of A)."""
    import torch
    rng = np.random.default_rng(20261204)
    data = {}
    # b and C sized for the longest contraction (2^26, asymmetric p = 2) and the
    # most outputs (2^26 fp32, asymmetric p = 2 q = 2; 2^24 fp64, symmetric p = 7)
    for dt, npdt, tdt, nb, ncm in (("f32", np.float32, torch.float32, 1 << 26, 1 << 26),
                                   ("f64", np.float64, torch.float64, 1 << 14, 1 << 24)):
        a = rng.random(1 << 28, dtype=npdt)
        a *= 2
        a -= 1
        b = (rng.random(nb, dtype=npdt) * 2 - 1).astype(npdt)
        da = torch.from_numpy(a).to(cuda)
        db = torch.from_numpy(b).to(cuda)
        dc = torch.empty(ncm, dtype=tdt, device=cuda)
        data[dt] = (a, b, da, db, dc)
    yield data
    data.clear()
    torch.cuda.empty_cache()


def run_sweep(engine, orc, inputs, cases, dt):
    import torch
    T = engine
    lib = T.library()
    fn = lib.tlibg_ttv_f32 if dt == "f32" else lib.tlibg_ttv_f64
    a, b, da, db, dc = inputs[dt]
    stream = torch.cuda.current_stream().cuda_stream
    failures, worst = [], 0.0
    for na, pia, q in cases:
        p = len(na)
        wa = T.strides(na, pia)
        nc, pic = T.output_shape(na, q), T.output_layout(pia, q)
        wc = T.strides(nc, pic)
        keep = [T._sizes(v) for v in (na, wa, pia, [na[q - 1]], nc, wc, pic)]
        P, nq, S = orc.canonical(na, pia, q)
        dc[:P * S].fill_(float("nan"))
        st = fn(q, p, da.data_ptr(), *[T._p(k) for k in keep[:3]], db.data_ptr(), T._p(keep[3]),
                dc.data_ptr(), *[T._p(k) for k in keep[4:]], stream)
        assert st == 0, f"na={na} pia={pia} q={q}: {T._last_error()}"
        torch.cuda.synchronize()
        c = dc[:P * S].cpu().numpy()
        ref, absn = orc.truth(S, nq, P, a[:P * nq * S], b[:nq])
        err = orc.rel_error(c, ref, absn)
        if not np.isfinite(c).all():
            err = float("inf")
        worst = max(worst, err)
        if not err <= TOL[dt]:
            failures.append(f"na={na} pia={pia} q={q} {dt}: err {err:.3e} "
                            f"plan={T.plan(q, na, pia, dtype=T.F32 if dt == 'f32' else T.F64)}")
    assert T.device_error() == 0
    assert not failures, "\n".join(failures)
    return worst


def test_symmetric_sweep_fp32(engine, orc, inputs):
    worst = run_sweep(engine, orc, inputs, sym_cases("f32"), "f32")
    assert worst <= TOL["f32"]


def test_symmetric_sweep_fp64(engine, orc, inputs):
    worst = run_sweep(engine, orc, inputs, sym_cases("f64"), "f64")
    assert worst <= TOL["f64"]


def test_asymmetric_sweep_fp32(engine, orc, inputs):
    worst = run_sweep(engine, orc, inputs, asym_cases(), "f32")
    assert worst <= TOL["f32"]
