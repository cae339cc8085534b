"""Generate the golden fixtures of the TTV path from the reference itself.

Run in a checkout where the reference sources exist (its headers are compiled
into oracle/_ref/libttvref.so by ``oracle.build(with_ref=True)``):

    python tests/golden/make_golden.py

Writes, next to this script:
  ttv_random.npz   seeded random small problems (fp32 and fp64), their inputs
                   and the reference's outputs of par_loop/subtensor/all (the
                   path the reference's ``A(q) * b`` operator takes)
  errors.json      invalid calls and the exception text the reference throws
  metadata.json    output shapes, output layouts, strides and k-order layouts
                   computed by the reference's detail helpers
"""
from __future__ import annotations

import itertools
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def random_cases(rng, count):
    cases = []
    while len(cases) < count:
        p = int(rng.integers(2, 8))
        na = [int(x) for x in rng.integers(1, 10, p)]
        if np.prod(na) > 1536:
            continue
        pia = [int(x) + 1 for x in rng.permutation(p)]
        q = int(rng.integers(1, p + 1))
        dt = np.float32 if len(cases) % 2 == 0 else np.float64
        cases.append((na, pia, q, dt))
    return cases


def main():
    O.build(with_ref=True)
    rng = np.random.default_rng(20261203)
    arrays = {}
    index = []
    for n, (na, pia, q, dt) in enumerate(random_cases(rng, 160)):
        wa = O.strides(na, pia)
        nc = O.output_shape(na, q)
        pic = O.output_layout(pia, q)
        wc = O.strides(nc, pic)
        a = rng.uniform(-1.0, 1.0, int(np.prod(na))).astype(dt)
        b = rng.uniform(-1.0, 1.0, na[q - 1]).astype(dt)
        st, msg, c = O.ref_ttv("par_loop/subtensor/all", q, a, na, wa, pia, b, [na[q - 1]], nc,
                               wc, pic)
        assert st == 0, msg
        arrays[f"a{n}"] = a
        arrays[f"b{n}"] = b
        arrays[f"c{n}"] = c
        index.append({"na": na, "pia": pia, "q": q, "wa": wa, "nc": nc, "wc": wc, "pic": pic,
                      "dtype": np.dtype(dt).name})
    arrays["index"] = np.frombuffer(json.dumps(index).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "ttv_random.npz"), **arrays)

    # invalid calls: the reference's exception text for each
    na, pia = [2, 3, 4], [1, 2, 3]
    base = dict(q=2, p=3, na=na, wa=O.strides(na, pia), pia=pia, nb=[3], nc=[2, 4], wc=[1, 2],
                pic=[1, 2])
    variants = [
        {}, {"q": 0}, {"q": 4}, {"nb": [5]}, {"na": [2, 3, 0]}, {"nc": [2, 0]},
        {"pia": [1, 1, 3]}, {"pia": [0, 1, 2]}, {"pic": [2, 2]}, {"pic": [1, 3]},
        {"wa": [1, 8, 2]}, {"wc": [4, 1]}, {"pic": [2, 1], "wc": [4, 1]},
        {"q": 2, "pia": [3, 2, 1], "wa": [12, 4, 1], "pic": [1, 2], "wc": [1, 2]},
        {"q": 2, "pia": [1, 3, 2], "wa": [1, 8, 2], "pic": [2, 1], "wc": [4, 1]},
        {"q": 2, "pia": [1, 3, 2], "wa": [1, 8, 2], "pic": [1, 2], "wc": [1, 2]},
        {"p": 1, "q": 1, "na": [3], "wa": [1], "pia": [1], "nc": [], "wc": [], "pic": []},
        {"p": 2, "q": 1, "na": [3, 8], "wa": [1, 3], "pia": [1, 2], "nc": [8], "wc": [1],
         "pic": [1]},
    ]
    errors = []
    for v in variants:
        args = dict(base)
        args.update(v)
        nb0 = args["nb"][0]
        a = np.zeros(max(int(np.prod(args["na"])), 1), np.float64)
        b = np.zeros(max(nb0, 1), np.float64)
        nc = args["nc"] if args["nc"] else [1]
        st, msg, _ = O.ref_ttv("par_loop/subtensor/all", args["q"], a, args["na"], args["wa"],
                               args["pia"], b, args["nb"], nc, args["wc"] or [1],
                               args["pic"] or [1]) if args["p"] != 1 else _order1(args)
        errors.append({"args": args, "status": st, "message": msg})
    with open(os.path.join(HERE, "errors.json"), "w") as f:
        json.dump(errors, f, indent=1)

    # metadata helpers
    R = O.ref()
    meta = {"output_shape": [], "output_layout": [], "strides": [], "k_order": []}
    for p in range(1, 5):
        for na in itertools.product([1, 2, 3], repeat=p):
            for pia in itertools.permutations(range(1, p + 1)):
                w = O.sizes([0] * p)
                R.ref_strides(O.sizes(na), O.sizes(pia), p, w)
                meta["strides"].append([list(na), list(pia), [w[i] for i in range(p)]])
                if p >= 2:
                    for q in range(1, p + 1):
                        nc = O.sizes([0] * (p - 1))
                        R.ref_output_shape(O.sizes(na), p, q, nc)
                        pic = O.sizes([0] * (p - 1))
                        R.ref_output_layout(O.sizes(pia), p, q, pic)
                        meta["output_shape"].append([list(na), q, [nc[i] for i in range(p - 1)]])
                        meta["output_layout"].append([list(pia), q,
                                                      [pic[i] for i in range(p - 1)]])
    for p in range(1, 11):
        for k in range(0, p + 2):
            pi = O.sizes([0] * p)
            R.ref_k_order_layout(p, k, pi)
            meta["k_order"].append([p, k, [pi[i] for i in range(p)]])
    # thin the (large, redundant) lists deterministically
    meta["output_shape"] = meta["output_shape"][::7]
    meta["output_layout"] = meta["output_layout"][::5]
    meta["strides"] = meta["strides"][::3]
    with open(os.path.join(HERE, "metadata.json"), "w") as f:
        json.dump(meta, f)
    print("golden fixtures written to", HERE)


def _order1(args):
    """p = 1: C has no modes, so the reference rejects C's (empty) shape."""
    a = np.zeros(3, np.float64)
    b = np.zeros(3, np.float64)
    import ctypes as C
    msg = C.create_string_buffer(512)
    one = O.sizes([1])
    st = O.ref().ref_ttv_f64(1, 1, 1, a.ctypes.data_as(C.c_void_p), C.cast(O.sizes([3]), O._psz),
                             C.cast(O.sizes([1]), O._psz), C.cast(O.sizes([1]), O._psz),
                             b.ctypes.data_as(C.c_void_p), C.cast(O.sizes([3]), O._psz),
                             np.zeros(1).ctypes.data_as(C.c_void_p), C.cast(one, O._psz),
                             C.cast(one, O._psz), C.cast(one, O._psz), msg, 512)
    return st, msg.value.decode(), None


if __name__ == "__main__":
    main()
