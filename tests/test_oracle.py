"""The CPU oracle, pinned against the reference (CPU only).

* the reference's known-answer test (test/src/gtest_tlib_ttv.cpp:28-140,
  gtest_aux.h:29-79), restated: ranks 2-4, extents {2, 4, 8}, every layout
  and every q, on all three restated policies;
* the golden fixtures in tests/golden (outputs and exception texts of the
  reference compiled from source, made by tests/golden/make_golden.py);
* when the reference shim is built here (oracle/_ref), a direct bit-for-bit
  comparison on random shapes.
"""
import itertools
import json
import os
import platform

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


def shapes(rank):
    return [list(s) for s in itertools.product([2, 4, 8], repeat=rank)]


def kat_input(orc, q, na, wa, pia, dtype):
    """A numbered 1, 2, 3, ... along mode q, the layout's other modes outside it
    (gtest_tlib_ttv.cpp:28-66)."""
    p = len(na)
    a = np.zeros(int(np.prod(na)), dtype=dtype)
    q1 = pia.index(q)
    order = [pia[r] - 1 for r in range(p - 1, -1, -1) if r != q1] + [q - 1]
    k = 0
    for idx in itertools.product(*[range(na[m]) for m in order]):
        off = sum(i * wa[m] for i, m in zip(idx, order))
        k += 1
        a[off] = k
    return a


def kat_expect(nq, count):
    i = np.arange(1, count + 1, dtype=np.float64)
    return (nq * nq * (2 * i - 1) + nq) / 2


@pytest.mark.parametrize("rank", [2, 3, 4])
@pytest.mark.parametrize("policy", ["seq/subtensor/none", "par_loop/subtensor/all",
                                    "par_loop/slice/all"])
def test_kat(orc, rank, policy):
    for na in shapes(rank)[:: (3 if rank == 4 else 1)]:
        for pia in itertools.permutations(range(1, rank + 1)):
            pia = list(pia)
            wa = orc.strides(na, pia)
            for q in range(1, rank + 1):
                nc, pic = orc.output_shape(na, q), orc.output_layout(pia, q)
                wc = orc.strides(nc, pic)
                for dt in (np.float64, np.float32):
                    a = kat_input(orc, q, na, wa, pia, dt)
                    b = np.ones(na[q - 1], dt)
                    st, c = orc.ttv(policy, q, a, na, wa, pia, b, [na[q - 1]], nc, wc, pic)
                    assert st == 0
                    # C in its own layout order holds outputs 1, 2, 3, ... (dense C: offset order)
                    np.testing.assert_array_equal(c.astype(np.float64),
                                                  kat_expect(na[q - 1], c.size))


def test_golden_random(orc):
    data = np.load(os.path.join(GOLDEN, "ttv_random.npz"))
    index = json.loads(bytes(data["index"]).decode())
    assert len(index) >= 100
    for n, case in enumerate(index):
        a, b, want = data[f"a{n}"], data[f"b{n}"], data[f"c{n}"]
        for policy in ("par_loop/subtensor/all", "seq/subtensor/none"):
            st, c = orc.ttv(policy, case["q"], a, case["na"], case["wa"], case["pia"], b,
                            [case["na"][case["q"] - 1]], case["nc"], case["wc"], case["pic"])
            assert st == 0
            if EXACT_HOST:
                np.testing.assert_array_equal(c, want, err_msg=str(case))
            else:
                np.testing.assert_allclose(c, want, rtol=1e-5, atol=1e-6, err_msg=str(case))
        # the canonical form used as CPU baseline gives the same numbers
        P, nq, S = orc.canonical(case["na"], case["pia"], case["q"])
        cc = orc.canon(S, nq, P, a, b)
        np.testing.assert_allclose(cc, want, rtol=1e-5 if a.dtype == np.float32 else 1e-12,
                                   atol=1e-6)


def test_golden_errors(orc):
    with open(os.path.join(GOLDEN, "errors.json")) as f:
        cases = json.load(f)
    for case in cases:
        x = case["args"]
        if x["p"] == 1:
            code = orc.check(1, 1, 1, [3], [1], [1], 1, [3], 1, [1] * 0 or [0], [1], [1])
            # C has no modes: the order-1 call always fails on C's shape
            assert orc.check_message(15) == case["message"]
            continue
        code = orc.check(x["q"], x["p"], 1, x["na"], x["wa"], x["pia"], 1, x["nb"], 1, x["nc"],
                         x["wc"], x["pic"])
        if code == 0 and 1 <= x["q"] <= x["p"] and orc.case(x["p"], x["q"], x["pia"]) == 8:
            perr = orc.lib().orc_check_pic(orc.sizes(x["pia"]), orc.sizes(x["pic"]), x["p"],
                                           x["q"])
            code = 19 + perr if perr else 0
        msg = orc.check_message(code) if code else ""
        assert msg == case["message"], (x, msg, case["message"])


def test_golden_metadata(orc):
    with open(os.path.join(GOLDEN, "metadata.json")) as f:
        meta = json.load(f)
    for na, q, nc in meta["output_shape"]:
        assert orc.output_shape(na, q) == nc
    for pia, q, pic in meta["output_layout"]:
        assert orc.output_layout(pia, q) == pic
    for n, pi, w in meta["strides"]:
        assert orc.strides(n, pi) == w
    for p, k, pi in meta["k_order"]:
        assert orc.k_order_layout(p, k) == pi


def test_slice_path_refuses_unit_extents(orc):
    """The reference's par_loop/slice/all addresses outside A and C when a
    fused mode has extent 1 (generate_strides gives vector-like shapes unit
    strides); the oracle refuses instead of reproducing it."""
    na, pia, q = [1, 6, 7, 5, 1], [3, 2, 1, 4, 5], 4
    wa = orc.strides(na, pia)
    nc, pic = orc.output_shape(na, q), orc.output_layout(pia, q)
    wc = orc.strides(nc, pic)
    a = np.ones(int(np.prod(na)), np.float32)
    st, _ = orc.ttv("par_loop/slice/all", q, a, na, wa, pia, np.ones(5, np.float32), [5], nc, wc,
                    pic)
    assert st == 22


@pytest.mark.skipif(not __import__("oracle").ref_available(),
                    reason="reference shim not built (reference sources absent)")
def test_against_reference_build(orc):
    rng = np.random.default_rng(11)
    for t in range(400):
        p = int(rng.integers(2, 7))
        na = [int(x) for x in rng.integers(1, 9, p)]
        pia = [int(x) + 1 for x in rng.permutation(p)]
        q = int(rng.integers(1, p + 1))
        wa = orc.strides(na, pia)
        nc, pic = orc.output_shape(na, q), orc.output_layout(pia, q)
        wc = orc.strides(nc, pic)
        dt = np.float32 if t % 2 else np.float64
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
        b = rng.uniform(-1, 1, na[q - 1]).astype(dt)
        for policy in (0, 1, 2):
            st, c = orc.ttv(policy, q, a, na, wa, pia, b, [na[q - 1]], nc, wc, pic)
            if st == 22:
                continue
            st2, msg, c2 = orc.ref_ttv(policy, q, a, na, wa, pia, b, [na[q - 1]], nc, wc, pic)
            assert st == st2 == 0, msg
            np.testing.assert_array_equal(c, c2)


def test_truth_and_error_metric(orc):
    rng = np.random.default_rng(3)
    S, nq, P = 5, 3000, 7
    a = rng.uniform(-1, 1, S * nq * P).astype(np.float32)
    b = rng.uniform(-1, 1, nq).astype(np.float32)
    ref, absn = orc.truth(S, nq, P, a, b)
    exact = np.einsum("sip,i->sp", a.reshape(S, nq, P).astype(np.float64),
                      b.astype(np.float64)).ravel()
    assert np.max(np.abs(ref - exact) / absn) < 1e-13
    np.testing.assert_allclose(absn, np.einsum("sip,i->sp", np.abs(a.reshape(S, nq, P)).astype(
        np.float64), np.abs(b).astype(np.float64)).ravel(), rtol=1e-12)
    # the fp32 restated reference sits well inside 1e-5 under this metric
    c = orc.canon(S, nq, P, a, b)
    assert orc.rel_error(c, ref, absn) < 1e-5
