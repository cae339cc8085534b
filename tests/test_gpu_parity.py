"""Parity of the CUDA engine with the oracle (GPU; calls go through the C ABI).

Bars (component-wise error normalised by sum_k |a_ik b_k|, against the
oracle's double-double truth):
  fp32 (compensated and plain, n_q <= 2^16)   1e-5
  fp64                                        1e-13
  bf16-stored A vs its own bf16 values        1e-5
  bf16-stored A vs the fp32 A it came from    2e-3 for n_q >= 64 (2^-8 + 1e-5 always:
                                              bf16 rounds each element by up to 2^-8)
Integer-valued inputs (the reference's known-answer test, one-hot b) must
match bit for bit.
"""
import itertools
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
TOL = {np.float32: 1e-5, np.float64: 1e-13}


def meta(T, na, pia, q):
    wa = T.strides(na, pia)
    nc, pic = T.output_shape(na, q), T.output_layout(pia, q)
    return wa, nc, T.strides(nc, pic), pic


def run(T, torch, dev, q, na, pia, a, b, **opts):
    wa, nc, wc, pic = meta(T, na, pia, q)
    da = torch.from_numpy(a).to(dev)
    db = torch.from_numpy(b).to(dev)
    cdt = torch.float64 if a.dtype == np.float64 else torch.float32
    dc = torch.full((max(int(np.prod(nc)), 1),), float("nan"), dtype=cdt, device=dev)
    T.ttv(q, len(na), da, na, wa, pia, db, [na[q - 1]], dc, nc, wc, pic, sync=True, **opts)
    return dc.cpu().numpy()


def check(orc, T, torch, dev, q, na, pia, a, b, tol=None, truth=None, **opts):
    c = run(T, torch, dev, q, na, pia, a, b, **opts)
    P, nq, S = orc.canonical(na, pia, q)
    ref, absn = truth if truth is not None else orc.truth(S, nq, P, a, b)
    err = orc.rel_error(c, ref, absn)
    bar = tol if tol is not None else TOL[a.dtype.type]
    assert err <= bar, f"na={na} pia={pia} q={q} {a.dtype} opts={opts}: err {err:.3e} > {bar}"
    return c, err


@pytest.fixture(scope="module")
def torch_dev(cuda):
    import torch
    return torch, cuda


def kat_input(na, wa, pia, q, dtype):
    p = len(na)
    a = np.zeros(int(np.prod(na)), dtype=dtype)
    q1 = pia.index(q)
    order = [pia[r] - 1 for r in range(p - 1, -1, -1) if r != q1] + [q - 1]
    offs = np.zeros(1, dtype=np.int64)
    for m in order:
        offs = (offs[:, None] + np.arange(na[m]) * wa[m]).ravel()
    a[offs] = np.arange(1, a.size + 1, dtype=dtype)
    return a


@pytest.mark.parametrize("rank", [2, 3, 4])
def test_kat_grid(engine, torch_dev, rank):
    """The reference's known-answer test, every shape / layout / q, exact."""
    torch, dev = torch_dev
    T = engine
    for na in itertools.product([2, 4, 8], repeat=rank):
        na = list(na)
        for pia in itertools.permutations(range(1, rank + 1)):
            pia = list(pia)
            wa = T.strides(na, pia)
            for q in range(1, rank + 1):
                nq = na[q - 1]
                for dt in (np.float32, np.float64):
                    a = kat_input(na, wa, pia, q, dt)
                    b = np.ones(nq, dt)
                    c = run(T, torch, dev, q, na, pia, a, b)
                    i = np.arange(1, c.size + 1, dtype=np.float64)
                    np.testing.assert_array_equal(c.astype(np.float64),
                                                  (nq * nq * (2 * i - 1) + nq) / 2,
                                                  err_msg=f"{na} {pia} q={q} {dt}")


@pytest.mark.parametrize("standalone", [False, True], ids=["reference_headers", "standalone"])
def test_cpp_kat_through_policy(engine, cuda, tmp_path, standalone):
    """The same KAT through the C++ `execution_policy::gpu` drop-in, every
    (slicing, fusion) pair of the reference's tests.  With the reference
    headers (staged in baseline/_ref/include) the call goes through the
    reference's own tlib::ttv::ttv (ttv.h:54-92: its checks, then its dispatch
    to detail::ttv at ttv.h:91), which resolves to the gpu overloads."""
    from test_abi import _compile_cpp
    import subprocess
    exe = _compile_cpp(tmp_path, standalone=standalone)
    r = subprocess.run([exe, "kat"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "PASSED" in r.stdout, r.stdout + r.stderr
    assert ("reference headers" if not standalone else "standalone") in r.stdout


@pytest.mark.parametrize("standalone", [False, True], ids=["reference_headers", "standalone"])
def test_cpp_device_tensor_interface(engine, cuda, tmp_path, standalone):
    """tlib/ttv_gpu_tensor.h: A(q) * b and ttv(q, A, b) on device tensors, the gpu
    policy on host pointers (the engine's host path) and, with the reference
    headers, the reference's own tensor<T> through the gpu policy."""
    from test_abi import _compile_cpp
    import subprocess
    exe = _compile_cpp(tmp_path, standalone=standalone)
    r = subprocess.run([exe, "tensor"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "PASSED" in r.stdout, r.stdout + r.stderr


def test_golden_fixtures(engine, orc, torch_dev):
    """Outputs of the reference itself (fixtures made from it) on random inputs."""
    torch, dev = torch_dev
    data = np.load(os.path.join(GOLDEN, "ttv_random.npz"))
    index = json.loads(bytes(data["index"]).decode())
    for n, case in enumerate(index):
        a, b, want = data[f"a{n}"], data[f"b{n}"], data[f"c{n}"]
        c, err = check(orc, engine, torch, dev, case["q"], case["na"], case["pia"], a, b)
        # and close to the reference's own rounding of the same sums
        P, nq, S = orc.canonical(case["na"], case["pia"], case["q"])
        _, absn = orc.truth(S, nq, P, a, b)
        assert np.max(np.abs(c.astype(np.float64) - want) / np.maximum(absn, 1e-300)) <= \
            2 * TOL[a.dtype.type]


def random_case(rng, max_elems=1 << 18, max_p=8):
    while True:
        p = int(rng.integers(2, max_p + 1))
        na = [int(x) for x in rng.integers(1, 40, p)]
        if np.prod(na) <= max_elems:
            break
    pia = [int(x) + 1 for x in rng.permutation(p)]
    q = int(rng.integers(1, p + 1))
    return na, pia, q


def test_random_shapes(engine, orc, torch_dev):
    torch, dev = torch_dev
    rng = np.random.default_rng(2026)
    for t in range(300):
        na, pia, q = random_case(rng)
        dt = (np.float32, np.float64)[t % 2]
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
        b = rng.uniform(-1, 1, na[q - 1]).astype(dt)
        check(orc, engine, torch, dev, q, na, pia, a, b)
        if dt == np.float32 and t % 5 == 0:
            check(orc, engine, torch, dev, q, na, pia, a, b, accumulate=engine.ACC_PLAIN)


SHAPES = [
    ([256, 256, 256], [1, 2, 3], 2),
    ([256, 256, 256], [1, 2, 3], 1),
    ([256, 256, 256], [1, 2, 3], 3),
    ([645, 64, 7], [1, 2, 3], 2),
    ([25, 25, 25, 25], [4, 3, 2, 1], 3),
    ([48, 48, 48], [3, 1, 2], 1),
    ([1024, 4, 4, 4], [1, 2, 3, 4], 3),
    ([16, 16, 16, 16, 16], [1, 2, 3, 4, 5], 5),
    ([3, 50000], [1, 2], 2),
    ([50000, 3], [1, 2], 1),
    ([1, 1, 4096, 1], [1, 2, 3, 4], 3),
    ([7, 1, 33], [2, 1, 3], 2),
]


@pytest.mark.parametrize("na,pia,q", SHAPES)
def test_variant_sweep(engine, orc, torch_dev, na, pia, q):
    """Every kernel instantiation the planner may pick gives the same answer."""
    torch, dev = torch_dev
    rng = np.random.default_rng(sum(na) + q)
    P, nq, S = orc.canonical(na, pia, q)
    for dt in (np.float32, np.float64):
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
        b = rng.uniform(-1, 1, nq).astype(dt)
        truth = orc.truth(S, nq, P, a, b)
        vmax = 16 // np.dtype(dt).itemsize
        groups = [1, 2, 4, 8, 16, 32] if P == 1 else [1, 2, 4, 8]
        vecs = [v for v in (1, 2, 4, 8) if v <= vmax and (nq if P == 1 else P) % v == 0]
        kind = engine.KIND_ROW if P == 1 else engine.KIND_COL
        for g in groups:
            for v in vecs:
                bmax = 16384 // np.dtype(dt).itemsize   # b elements staged per segment
                for split in (0, 1, 3, 17):
                    if P > 1 and 0 < split < -(-nq // bmax):
                        continue
                    if split > nq:
                        continue
                    check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth, kind=kind,
                          group=g, vec=v, split=split)
        # the row-tile kernel, for short q-fastest rows
        if P == 1 and nq <= 64:
            accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN) if dt == np.float32 else \
                (engine.ACC_COMPENSATED, engine.ACC_PLAIN, engine.ACC_DOUBLE_FLOAT)
            for acc in accs:
                check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth,
                      kind=engine.KIND_ROW_TILE, accumulate=acc)
        # the TMA-streamed kernel, where whole rows fit a stage
        L = nq if P == 1 else P
        if L * np.dtype(dt).itemsize <= 16384 and (P == 1 or -(-P // 256) <= 8):
            for g in ([1, 2, 4, 8, 16, 32] if P == 1 else [0]):
                for split in ((0,) if P == 1 else (0, 1, 3, 17)):
                    if split > nq:
                        continue
                    check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth,
                          kind=engine.KIND_STREAM, group=g, split=split)


def test_bf16_stored_a(engine, orc, torch_dev):
    torch, dev = torch_dev
    rng = np.random.default_rng(5)
    for na, pia, q in SHAPES[:8]:
        a32 = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
        abf = torch.from_numpy(a32).to(torch.bfloat16)
        bits = abf.view(torch.int16).numpy().view(np.uint16).copy()
        wa, nc, wc, pic = meta(engine, na, pia, q)
        dc = torch.empty(int(np.prod(nc)), dtype=torch.float32, device=dev)
        engine.ttv(q, len(na), abf.to(dev).view(torch.int16), na, wa, pia,
                   torch.from_numpy(b).to(dev), [na[q - 1]], dc, nc, wc, pic,
                   dtype=engine.BF16A, sync=True)
        c = dc.cpu().numpy()
        P, nq, S = orc.canonical(na, pia, q)
        ref32, absn32 = orc.truth(S, nq, P, a32, b)
        err32 = orc.rel_error(c, ref32, absn32)
        # bf16 keeps 8 significant bits: each stored element is within 2^-8 of
        # the fp32 one, so the storage alone can cost up to 2^-8 of sum|a*b|;
        # over longer contractions the roundings average out below 2e-3
        assert err32 <= 2.0 ** -8 + 1e-5
        if nq >= 64:
            assert err32 <= 2e-3
        refb, absnb = orc.truth(S, nq, P, bits, b, kind="bf16a")
        assert orc.rel_error(c, refb, absnb) <= 1e-5


def test_misaligned_pointers(engine, orc, torch_dev):
    """Views that start 1-3 elements into an allocation: narrower loads, same answer."""
    torch, dev = torch_dev
    rng = np.random.default_rng(9)
    for na, pia, q in ([64, 64, 64], [1, 2, 3], 2), ([64, 64, 64], [1, 2, 3], 1), \
            ([100, 300], [1, 2], 2):
        wa, nc, wc, pic = meta(engine, na, pia, q)
        N, M = int(np.prod(na)), int(np.prod(nc))
        a = rng.uniform(-1, 1, N + 3).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1] + 3).astype(np.float32)
        da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        dc = torch.zeros(M + 3, dtype=torch.float32, device=dev)
        P, nq, S = orc.canonical(na, pia, q)
        for oa, ob, oc in ((1, 0, 0), (0, 1, 0), (0, 0, 1), (3, 2, 1)):
            engine.ttv(q, len(na), da[oa:oa + N], na, wa, pia, db[ob:ob + nq], [nq],
                       dc[oc:oc + M], nc, wc, pic, sync=True)
            ref, absn = orc.truth(S, nq, P, a[oa:oa + N], b[ob:ob + nq])
            assert orc.rel_error(dc[oc:oc + M].cpu().numpy(), ref, absn) <= 1e-5


def test_unit_extents_and_degenerate(engine, orc, torch_dev):
    torch, dev = torch_dev
    rng = np.random.default_rng(1)
    cases = [([1, 5], [1, 2], 1), ([5, 1], [1, 2], 2), ([1, 1], [1, 2], 1), ([1, 1, 1], [3, 2, 1], 2),
             ([1, 300000], [1, 2], 2), ([300000, 1], [2, 1], 1), ([2, 1, 2], [1, 2, 3], 2),
             ([1, 7, 1, 3], [2, 4, 1, 3], 4), ([9, 1, 11, 1, 2], [5, 1, 3, 2, 4], 1)]
    for na, pia, q in cases:
        for dt in (np.float32, np.float64):
            a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
            b = rng.uniform(-1, 1, na[q - 1]).astype(dt)
            check(orc, engine, torch, dev, q, na, pia, a, b)


def test_long_contraction_precision(engine, orc, torch_dev):
    """Precision configuration: 64 x 2^22 and 16 x 2^20 x 16, contraction over
    the long mode, A = N(0,1) * 10^U(-3,3), b = U[-1,1]."""
    torch, dev = torch_dev
    rng = np.random.default_rng(77)
    for na, pia, q in (([64, 1 << 22], [1, 2], 2), ([16, 1 << 20, 16], [1, 2, 3], 2)):
        N = int(np.prod(na))
        a = (rng.standard_normal(N) * 10.0 ** rng.uniform(-3, 3, N)).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
        P, nq, S = orc.canonical(na, pia, q)
        truth = orc.truth(S, nq, P, a, b)
        c, err = check(orc, engine, torch, dev, q, na, pia, a, b, tol=1e-5, truth=truth)
        cp, errp = check(orc, engine, torch, dev, q, na, pia, a, b, tol=1e-3, truth=truth,
                         accumulate=engine.ACC_PLAIN)
        assert err <= errp * 1.01 + 1e-9   # compensation never worse than plain


def test_full_size_properties(engine, torch_dev):
    """Symmetric sweep sizes (2^28 elements): size-independent properties.
    b = e_k picks one slice exactly; linearity in b; checksum of checksums."""
    torch, dev = torch_dev
    g = torch.Generator(device=dev)
    g.manual_seed(123)
    for p in (2, 3, 4):
        n = int(np.floor(2 ** (28 / p) + 1e-9))
        na = [n] * p
        A = torch.rand(n ** p, generator=g, device=dev, dtype=torch.float32) * 2 - 1
        for pia in (list(range(1, p + 1)), list(range(p, 0, -1))):
            for q in (1, (p + 1) // 2, p):
                wa, nc, wc, pic = meta(engine, na, pia, q)
                M = n ** (p - 1)
                C = torch.empty(M, dtype=torch.float32, device=dev)
                # one-hot b: C is the slice k of A along q, bit for bit
                k = n // 3
                b = torch.zeros(n, dtype=torch.float32, device=dev)
                b[k] = 1.0
                engine.ttv(q, p, A, na, wa, pia, b, [n], C, nc, wc, pic, sync=True)
                # the slice, addressed through A's layout: view A with mode strides
                At = torch.as_strided(A, na, wa)
                slice_ = At.select(q - 1, k)
                # C's dense layout pic over the remaining modes
                Ct = torch.as_strided(C, nc, wc)
                assert torch.equal(Ct, slice_), (p, pia, q)
                # linearity
                b1 = torch.rand(n, generator=g, device=dev) * 2 - 1
                b2 = torch.rand(n, generator=g, device=dev) * 2 - 1
                C1, C2, C12 = (torch.empty_like(C) for _ in range(3))
                for bb, cc in ((b1, C1), (b2, C2), (b1 + b2, C12)):
                    engine.ttv(q, p, A, na, wa, pia, bb, [n], cc, nc, wc, pic, sync=True)
                # each result is within 1e-5 * sum|a b| <= 1e-5 * 2n of exact
                assert float((C12.double() - C1.double() - C2.double()).abs().max()) <= 4e-5 * n
                # checksum of checksums: sum_j C = sum_i b_i * (sum of slice i)
                slice_sums = At.double().sum(dim=[d for d in range(p) if d != q - 1])
                want = float((slice_sums * b1.double()).sum())
                got = float(C1.double().sum())
                assert abs(got - want) <= 1e-5 * float(At.double().abs().sum()), (got, want)
        del A
        torch.cuda.empty_cache()


def test_host_buffers(engine, orc, torch_dev):
    """The host-pointer entry point (the reference's own calling convention): pinned A
    is read in place by the column kernels with 16-byte loads, other plans and
    pageable A are staged through device memory in chunks; pinned C is written in
    place, pageable C copied back."""
    torch, dev = torch_dev
    rng = np.random.default_rng(4)
    # column forms with 16-byte loads read pinned A in place; row forms (rows of 25,
    # rows of 645 over two staged chunks) and odd prefixes are staged; n_q <= 16
    # column outputs go to pinned C in place (read in place and staged)
    for na, pia, q in (([200, 300, 50], [1, 2, 3], 2), ([128, 64, 300], [3, 1, 2], 3),
                       ([4096, 4096], [1, 2], 2), ([25, 4000], [1, 2], 1), ([7, 999, 5], [1, 2, 3], 2),
                       ([645, 60000], [1, 2], 1), ([512, 4, 1024], [1, 2, 3], 2),
                       ([645, 4, 301], [1, 2, 3], 2)):
        wa, nc, wc, pic = meta(engine, na, pia, q)
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
        P, nq, S = orc.canonical(na, pia, q)
        ref, absn = orc.truth(S, nq, P, a, b)
        # pageable numpy buffers
        c = np.zeros(int(np.prod(nc)), np.float32)
        engine.ttv_host(q, len(na), a, na, wa, pia, b, [nq], c, nc, wc, pic)
        assert orc.rel_error(c, ref, absn) <= 1e-5
        # pinned torch buffers
        ta = torch.from_numpy(a).pin_memory()
        tb = torch.from_numpy(b).pin_memory()
        tc = torch.zeros(int(np.prod(nc)), dtype=torch.float32).pin_memory()
        engine.ttv_host(q, len(na), ta, na, wa, pia, tb, [nq], tc, nc, wc, pic)
        assert orc.rel_error(tc.numpy(), ref, absn) <= 1e-5
        # pinned A (read in place) with pageable C (copied back) and vice versa
        c2 = np.zeros(int(np.prod(nc)), np.float32)
        engine.ttv_host(q, len(na), ta, na, wa, pia, b, [nq], c2, nc, wc, pic)
        assert orc.rel_error(c2, ref, absn) <= 1e-5
        tc.zero_()
        engine.ttv_host(q, len(na), a, na, wa, pia, b, [nq], tc, nc, wc, pic)
        assert orc.rel_error(tc.numpy(), ref, absn) <= 1e-5
        # pinned A one element off the 16-byte grid: staged chunks start mid-block
        ta1 = torch.from_numpy(np.concatenate([np.zeros(1, np.float32), a])).pin_memory()[1:]
        tc.zero_()
        engine.ttv_host(q, len(na), ta1, na, wa, pia, tb, [nq], tc, nc, wc, pic)
        assert orc.rel_error(tc.numpy(), ref, absn) <= 1e-5
    # fp64, pinned, every path: in place (column tiles), staged (rows, odd prefix)
    for na, pia, q in (([64, 300, 50], [1, 2, 3], 2), ([645, 3000], [1, 2], 1), ([25, 999, 7], [1, 2, 3], 2)):
        wa, nc, wc, pic = meta(engine, na, pia, q)
        a = rng.uniform(-1, 1, int(np.prod(na)))
        b = rng.uniform(-1, 1, na[q - 1])
        P, nq, S = orc.canonical(na, pia, q)
        ref, absn = orc.truth(S, nq, P, a, b)
        ta = torch.from_numpy(a).pin_memory()
        tc = torch.zeros(int(np.prod(nc)), dtype=torch.float64).pin_memory()
        engine.ttv_host(q, len(na), ta, na, wa, pia, torch.from_numpy(b).pin_memory(), [nq], tc, nc, wc, pic)
        assert orc.rel_error(tc.numpy(), ref, absn) <= 1e-13


def test_array_api_matches_einsum(engine, torch_dev):
    """ttvpy's tests (ttvpy/tests/test.py), restated on device tensors."""
    torch, dev = torch_dev
    A = torch.arange(3 * 2 * 4, dtype=torch.float64).reshape(3, 2, 4)
    for q, spec in ((1, "ijk,i->jk"), (2, "ijk,j->ik"), (3, "ijk,k->ij")):
        b = torch.arange(A.shape[q - 1], dtype=torch.float64)
        D = torch.einsum(spec, A, b)
        C_ = engine.ttv_array(q, A.to(dev), b.to(dev))
        assert torch.equal(C_.cpu(), D)
    for shape in ((3, 2, 4, 5), (5, 5, 5, 5)):
        A = torch.arange(int(np.prod(shape)), dtype=torch.float64).reshape(*shape)
        for q in range(1, 5):
            dims = [d for d in range(4) if d != q - 1]
            B = [torch.arange(A.shape[d], dtype=torch.float64) for d in dims]
            D = A
            for d, bj in sorted(zip(dims, B), key=lambda t: -t[0]):
                D = torch.tensordot(D, bj, dims=([d], [0]))
            for order in ("forward", "backward", "optimal"):
                C_ = engine.ttvs(q, A.to(dev), [bj.to(dev) for bj in B], order)
                assert torch.equal(C_.cpu(), D), (shape, q, order)


def test_determinism_and_streams(engine, torch_dev):
    torch, dev = torch_dev
    na, pia, q = [64, 1 << 20], [1, 2], 2
    wa, nc, wc, pic = meta(engine, na, pia, q)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    A = torch.rand(int(np.prod(na)), generator=g, device=dev)
    b = torch.rand(na[q - 1], generator=g, device=dev)
    outs = []
    s = torch.cuda.Stream()
    for i in range(3):
        c = torch.empty(64, device=dev)
        with torch.cuda.stream(s):
            engine.ttv(q, 2, A, na, wa, pia, b, [na[1]], c, nc, wc, pic)
        s.synchronize()
        outs.append(c.cpu())
    assert all(torch.equal(outs[0], o) for o in outs[1:])
    assert engine.device_error() == 0


def test_launch_counter(engine, torch_dev):
    torch, dev = torch_dev
    before = engine.launch_count()
    na, pia, q = [32, 32], [1, 2], 2
    wa, nc, wc, pic = meta(engine, na, pia, q)
    engine.ttv(q, 2, torch.ones(1024, device=dev), na, wa, pia, torch.ones(32, device=dev), [32],
               torch.empty(32, device=dev), nc, wc, pic, sync=True)
    assert engine.launch_count() > before


def test_fp64_emulation_window_and_fallback(engine, orc, torch_dev):
    """fp64 with ACC_DOUBLE_FLOAT accumulates in double-float on the FP32/INT32 pipes
    when every exponent is inside [2^-60, 2^61) and falls back to native DFMA outside:
    wide-range values, zeros and subnormals, every kernel family, against the
    oracle (1e-13) and against the native-DFMA mode."""
    torch, dev = torch_dev
    rng = np.random.default_rng(64)
    for na, pia, q in (([300, 200, 50], [1, 2, 3], 2), ([64, 48, 300], [1, 2, 3], 1),
                       ([2000, 400], [2, 1], 2), ([16, 4096, 8], [1, 2, 3], 2),
                       ([4096, 3], [1, 2], 2)):
        N = int(np.prod(na))
        a = rng.uniform(-1, 1, N) * 10.0 ** rng.uniform(-40, 40, N)
        a[rng.integers(0, N, N // 50)] = 0.0
        a[rng.integers(0, N, N // 100)] = 5e-310                      # subnormal
        b = rng.uniform(-1, 1, na[q - 1]) * 10.0 ** rng.uniform(-5, 5, na[q - 1])
        if na == [4096, 3]:
            b[1] = 1e-70   # b outside the window: the kernels' pre-split of b is off
        P, nq, S = orc.canonical(na, pia, q)
        truth = orc.truth(S, nq, P, a, b)
        kinds = (-1, engine.KIND_ROW) if P == 1 else \
            (-1, engine.KIND_COL, engine.KIND_COL_REALIGN, engine.KIND_COL_BULK)
        if P == 1 and nq <= 64:
            kinds += (engine.KIND_ROW_TILE,)
        for kind in kinds:
            check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth, kind=kind,
                  accumulate=engine.ACC_DOUBLE_FLOAT)
            check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth, kind=kind)
        # in-window data: the emulation stays within the fp64 bar
        a2 = rng.uniform(-1, 1, N)
        truth2 = orc.truth(S, nq, P, a2, b)
        _, e_emu = check(orc, engine, torch, dev, q, na, pia, a2, b, truth=truth2,
                         accumulate=engine.ACC_DOUBLE_FLOAT)
        assert e_emu <= 1e-13


REALIGN_SHAPES = [
    ([645, 33, 7], [1, 2, 3], 2),        # P = 645: windows straddle rows and slabs
    ([1001, 9, 5], [1, 2, 3], 2),        # odd P, short contraction
    ([2, 3, 1023, 5], [1, 2, 3, 4], 4),  # P = 6138 = 2 (mod 4)
    ([25, 25, 25, 25], [1, 2, 3, 4], 3),  # P = 625, S = 25
    ([7, 50, 3], [1, 2, 3], 2),          # P < one window: scalar path only
    ([129, 5000, 2], [1, 2, 3], 2),      # long contraction: split b stages
    ([1000, 17, 3], [1, 2, 3], 2),       # aligned P: misalignment 0 throughout
    ([5, 3, 700], [3, 1, 2], 2),         # layout permuted: P = 700 * 5, n_q = 3
]


@pytest.mark.parametrize("na,pia,q", REALIGN_SHAPES)
def test_realigned_column_kernel(engine, orc, torch_dev, na, pia, q):
    """The column kernel with aligned 16-byte loads into shifted per-lane
    accumulators: every warp-row count and split, A at element offsets 0-3 (every
    row misalignment), fp32 (compensated and plain) and fp64 (native and
    double-float)."""
    torch, dev = torch_dev
    rng = np.random.default_rng(sum(na) * 7 + q)
    P, nq, S = orc.canonical(na, pia, q)
    wa, nc, wc, pic = meta(engine, na, pia, q)
    N, M = int(np.prod(na)), int(np.prod(nc))
    for dt in (np.float32, np.float64):
        tdt = torch.float32 if dt == np.float32 else torch.float64
        a = rng.uniform(-1, 1, N + 3).astype(dt)
        b = rng.uniform(-1, 1, nq).astype(dt)
        da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        dc = torch.empty(M, dtype=tdt, device=dev)
        bmax = 16384 // np.dtype(dt).itemsize
        accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN) if dt == np.float32 else \
            (engine.ACC_PLAIN, engine.ACC_DOUBLE_FLOAT)
        for oa in (0, 1, 2, 3):
            truth = orc.truth(S, nq, P, a[oa:oa + N], b)
            for g, split, acc in itertools.product((1, 2, 4, 8), (0, 1, 3, 17), accs):
                if (0 < split < -(-nq // bmax)) or split > nq:
                    continue
                dc.fill_(float("nan"))
                engine.ttv(q, len(na), da[oa:oa + N], na, wa, pia, db, [nq], dc, nc, wc, pic,
                           kind=engine.KIND_COL_REALIGN, group=g, split=split, accumulate=acc,
                           sync=True)
                err = orc.rel_error(dc.cpu().numpy(), *truth)
                assert err <= TOL[dt], (na, pia, q, dt, oa, g, split, acc, err)


def test_short_rows(engine, orc, torch_dev):
    """q-fastest rows of a few vectors: several rows per lane group in flight
    (one or two vectors per lane), groups wider than the row, row counts that
    leave the last iteration partial; fp32 compensated and plain, fp64 both modes."""
    torch, dev = torch_dev
    rng = np.random.default_rng(77)
    for dt in (np.float32, np.float64):
        vmax = 16 // np.dtype(dt).itemsize
        accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN)
        for nq in (2, 4, 6, 8, 12, 16, 24, 32, 48, 64):
            S = 1237 + nq
            na, pia, q = [nq, S], [1, 2], 1
            a = rng.uniform(-1, 1, nq * S).astype(dt)
            b = rng.uniform(-1, 1, nq).astype(dt)
            truth = orc.truth(S, nq, 1, a, b)
            for v in (1, 2, 4):
                if v > vmax or nq % v:
                    continue
                for g in (1, 2, 4, 8, 16, 32):
                    for acc in accs:
                        check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth,
                              kind=engine.KIND_ROW, group=g, vec=v, accumulate=acc)


def test_row_tile_kernel(engine, orc, torch_dev):
    """Short q-fastest rows through the row-tile kernel: every n_q up to 64 (odd
    and even, so both column walks), row counts below, at and around one
    32-row tile and across many tiles, A at element offsets 0-3 (ragged bulk
    copies), fp32 (compensated and plain), fp64 (mix, native, double-float)
    and bf16-stored A; fp64 rows of at most 32 elements take it by default."""
    torch, dev = torch_dev
    rng = np.random.default_rng(55)
    for nq in (1, 2, 3, 5, 8, 15, 16, 17, 24, 25, 31, 32, 33, 48, 63, 64):
        for S in (1, 31, 32, 33, 1000 + nq, 4099):
            na, pia, q = [nq, S], [1, 2], 1
            N = nq * S
            for dt in (np.float32, np.float64):
                tdt = torch.float32 if dt == np.float32 else torch.float64
                a = rng.uniform(-1, 1, N + 3).astype(dt)
                b = rng.uniform(-1, 1, nq).astype(dt)
                da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
                dc = torch.empty(S, dtype=tdt, device=dev)
                accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN) if dt == np.float32 else \
                    (engine.ACC_COMPENSATED, engine.ACC_PLAIN, engine.ACC_DOUBLE_FLOAT)
                for oa in ((0, 1, 2, 3) if S >= 1000 else (0, 3)):
                    truth = orc.truth(S, nq, 1, a[oa:oa + N], b)
                    for acc in accs:
                        dc.fill_(float("nan"))
                        engine.ttv(q, 2, da[oa:oa + N], na, [1, nq], pia, db, [nq], dc, [S], [1], [1],
                                   kind=engine.KIND_ROW_TILE, accumulate=acc, sync=True)
                        err = orc.rel_error(dc.cpu().numpy(), *truth)
                        assert err <= TOL[dt], (nq, S, dt, oa, acc, err)
        pl = engine.plan(1, [nq, 4099], [1, 2], dtype=engine.F64)
        assert pl["kind"] == (engine.KIND_ROW_TILE if nq <= 32 else engine.KIND_ROW), pl
    # bf16-stored A
    for nq, S in ((25, 3001), (16, 64), (64, 33)):
        a32 = rng.uniform(-1, 1, nq * S).astype(np.float32)
        b = rng.uniform(-1, 1, nq).astype(np.float32)
        abf = torch.from_numpy(a32).to(torch.bfloat16)
        bits = abf.view(torch.int16).numpy().view(np.uint16).copy()
        dc = torch.empty(S, dtype=torch.float32, device=dev)
        engine.ttv(1, 2, abf.to(dev).view(torch.int16), [nq, S], [1, nq], [1, 2],
                   torch.from_numpy(b).to(dev), [nq], dc, [S], [1], [1],
                   dtype=engine.BF16A, kind=engine.KIND_ROW_TILE, sync=True)
        refb, absnb = orc.truth(S, nq, 1, bits, b, kind="bf16a")
        assert orc.rel_error(dc.cpu().numpy(), refb, absnb) <= 1e-5
    # refused where it does not apply
    with pytest.raises(engine.TTVError):
        engine.ttv(1, 2, torch.zeros(65 * 4, device=dev), [65, 4], [1, 65], [1, 2],
                   torch.zeros(65, device=dev), [65], torch.zeros(4, device=dev), [4], [1], [1],
                   kind=engine.KIND_ROW_TILE)


def test_row_panel_kernel(engine, orc, torch_dev):
    """Long q-fastest rows through the row-panel kernel (b's segment held in
    registers across a block of rows): n_q a few segments long, not a multiple
    of the segment, S from 1 to past the row-block split, rows in flight 1 and
    2, fp32 (compensated and plain), fp64 (mix, native), bf16-stored A; on
    request only (the planner keeps the row kernel); refused for rows without
    16-byte vectors."""
    torch, dev = torch_dev
    rng = np.random.default_rng(77)
    cases = [(4096 * 3 + 4, 1), (4096 * 5, 7), (4096 * 2 + 36, 64), (1 << 16, 513), (70000, 3)]
    for nq, S in cases:
        na, pia, q = [nq, S], [1, 2], 1
        N = nq * S
        for dt in (np.float32, np.float64):
            if nq % (16 // np.dtype(dt).itemsize):
                continue
            tdt = torch.float32 if dt == np.float32 else torch.float64
            a = rng.uniform(-1, 1, N).astype(dt)
            b = rng.uniform(-1, 1, nq).astype(dt)
            da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
            dc = torch.empty(S, dtype=tdt, device=dev)
            truth = orc.truth(S, nq, 1, a, b)
            seg = 4096 if dt == np.float32 else 2048
            if nq <= seg:
                continue
            for acc in (engine.ACC_COMPENSATED, engine.ACC_PLAIN):
                for rr in (1, 2):
                    dc.fill_(float("nan"))
                    engine.ttv(q, 2, da, na, [1, nq], pia, db, [nq], dc, [S], [1], [1],
                               kind=engine.KIND_ROW_PANEL, group=rr, accumulate=acc, sync=True)
                    err = orc.rel_error(dc.cpu().numpy(), *truth)
                    assert err <= TOL[dt], (nq, S, dt, acc, rr, err)
    # bf16-stored A (segments of 8192 elements)
    for nq, S in ((8192 * 2 + 8, 5), (1 << 15, 40)):
        a32 = rng.uniform(-1, 1, nq * S).astype(np.float32)
        b = rng.uniform(-1, 1, nq).astype(np.float32)
        abf = torch.from_numpy(a32).to(torch.bfloat16)
        bits = abf.view(torch.int16).numpy().view(np.uint16).copy()
        dc = torch.empty(S, dtype=torch.float32, device=dev)
        engine.ttv(1, 2, abf.to(dev).view(torch.int16), [nq, S], [1, nq], [1, 2],
                   torch.from_numpy(b).to(dev), [nq], dc, [S], [1], [1],
                   dtype=engine.BF16A, kind=engine.KIND_ROW_PANEL, sync=True)
        refb, absnb = orc.truth(S, nq, 1, bits, b, kind="bf16a")
        assert orc.rel_error(dc.cpu().numpy(), refb, absnb) <= 1e-5
    # on request only: the planner keeps the row kernel for long rows
    assert engine.plan(1, [1 << 24, 4, 4], [1, 2, 3])["kind"] == engine.KIND_ROW
    na = [1 << 22, 6]
    a = rng.uniform(-1, 1, (1 << 22) * 6).astype(np.float32)
    b = rng.uniform(-1, 1, 1 << 22).astype(np.float32)
    c, err = check(orc, engine, torch, dev, 1, na, [1, 2], a, b, kind=engine.KIND_ROW_PANEL)
    # refused where it does not apply
    with pytest.raises(engine.TTVError):
        engine.ttv(1, 2, torch.zeros(8190 * 4, device=dev), [8190, 4], [1, 8190], [1, 2],
                   torch.zeros(8190, device=dev), [8190], torch.zeros(4, device=dev), [4], [1], [1],
                   kind=engine.KIND_ROW_PANEL)


def test_row_shift_kernel(engine, orc, torch_dev):
    """Rows that are not whole 16-byte vectors through the row-shift kernel
    (aligned vector bodies against shifted copies of b in shared memory, head
    and tail elements scalar): odd and even unaligned n_q from 1 to the shared-
    memory limit, A at every element offset of the 16-byte grid, S from 1 to
    many rounds, lanes per row 1..32, fp32 (compensated and plain), fp64 (mix
    and native); default for rows of 645 elements; refused for bf16-stored A
    and for rows whose shifted copies exceed 48 KB."""
    torch, dev = torch_dev
    rng = np.random.default_rng(91)
    for dt in (np.float32, np.float64):
        V = 16 // np.dtype(dt).itemsize
        tdt = torch.float32 if dt == np.float32 else torch.float64
        nmax = 3068 if dt == np.float32 else 1534
        for nq, S in ((1, 5), (3, 7), (V + 1, 33), (63, 100), (645, 2000), (625, 3001), (1001, 17),
                      (nmax, 40), (nmax - 1, 3)):
            if nq % V == 0:
                continue
            N = nq * S
            for off in range(V):
                a = rng.uniform(-1, 1, N + V).astype(dt)
                b = rng.uniform(-1, 1, nq).astype(dt)
                da_full, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
                da = da_full[off:off + N]
                truth = orc.truth(S, nq, 1, a[off:off + N], b)
                dc = torch.empty(S, dtype=tdt, device=dev)
                for acc in (engine.ACC_COMPENSATED, engine.ACC_PLAIN):
                    for G in ((1, 8, 32) if off == 0 else (4,)):
                        dc.fill_(float("nan"))
                        engine.ttv(1, 2, da, [nq, S], [1, nq], [1, 2], db, [nq], dc, [S], [1], [1],
                                   kind=engine.KIND_ROW_SHIFT, group=G, accumulate=acc, sync=True)
                        err = orc.rel_error(dc.cpu().numpy(), *truth)
                        assert err <= TOL[dt], (nq, S, off, dt, acc, G, err)
    # the planner's default for the sweep's rows of 645 (and the chain's rows of 625)
    for dt, code in ((np.float32, engine.F32), (np.float64, engine.F64)):
        assert engine.plan(1, [645, 645, 645], [1, 2, 3], dtype=code)["kind"] == engine.KIND_ROW_SHIFT
        assert engine.plan(1, [625, 625, 625], [1, 2, 3], dtype=code)["kind"] == engine.KIND_ROW_SHIFT
    na = [645, 645, 645]
    a = rng.uniform(-1, 1, 645 ** 3).astype(np.float64)
    b = rng.uniform(-1, 1, 645).astype(np.float64)
    check(orc, engine, torch, dev, 1, na, [1, 2, 3], a, b)
    # refused where it does not apply
    with pytest.raises(engine.TTVError):
        engine.ttv(1, 2, torch.zeros(4000 * 4, device=dev), [4000, 4], [1, 4000], [1, 2],
                   torch.zeros(4000, device=dev), [4000], torch.zeros(4, device=dev), [4], [1], [1],
                   kind=engine.KIND_ROW_SHIFT)
    with pytest.raises(engine.TTVError):
        engine.ttv(1, 2, torch.zeros(645 * 4, device=dev, dtype=torch.bfloat16).view(torch.int16),
                   [645, 4], [1, 645], [1, 2], torch.zeros(645, device=dev), [645],
                   torch.zeros(4, device=dev), [4], [1], [1], dtype=engine.BF16A, kind=engine.KIND_ROW_SHIFT)


def test_short_contraction_column_kernel(engine, orc, torch_dev):
    """Column form with n_q <= 4 and vector loads: two tiles per thread, every row
    loaded before any product; odd and even tile counts, one slice and many,
    fp32 (compensated and plain) and fp64 (mix and native)."""
    torch, dev = torch_dev
    rng = np.random.default_rng(404)
    for na, pia, q in (([64, 3, 1000], [1, 2, 3], 2), ([4096, 4], [1, 2], 2), ([8, 2, 33], [1, 2, 3], 2),
                       ([1024, 4, 4, 4], [1, 2, 3, 4], 3), ([16, 1, 4100], [1, 2, 3], 2),
                       ([2, 4, 4, 3, 5], [1, 2, 3, 4, 5], 4), ([100, 4, 7], [3, 2, 1], 1)):
        P, nq, S = orc.canonical(na, pia, q)
        for dt in (np.float32, np.float64):
            a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
            b = rng.uniform(-1, 1, nq).astype(dt)
            truth = orc.truth(S, nq, P, a, b)
            accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN)
            for acc in accs:
                check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth, accumulate=acc)
                check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth, accumulate=acc,
                      kind=engine.KIND_COL, group=1, split=1)


BULK_SHAPES = [
    ([1024, 33, 7], [1, 2, 3], 2),       # P = 1024: one full tile per slice (fp32)
    ([1001, 9, 5], [1, 2, 3], 2),        # odd P, partial tile, short contraction
    ([2, 3, 1023, 5], [1, 2, 3, 4], 4),  # P = 6138 = 2 (mod 4): partial last tile
    ([645, 33, 7], [1, 2, 3], 2),        # P = 645: one partial tile per slice
    ([129, 5000, 2], [1, 2, 3], 2),      # long contraction: several b segments
    ([5, 3, 700], [3, 1, 2], 2),         # layout permuted: P = 3500, n_q = 3
    ([4097, 6], [1, 2], 2),              # S = 1, P one past a multiple of the tile
]


@pytest.mark.parametrize("na,pia,q", BULK_SHAPES)
def test_bulk_column_kernel(engine, orc, torch_dev, na, pia, q):
    """The TMA-staged column kernel: rows of the prefix at every misalignment
    (A at element offsets 0-3), full and partial tiles, splits of q, fp32
    (compensated and plain), fp64 (mix and native) and bf16-stored A."""
    torch, dev = torch_dev
    rng = np.random.default_rng(sum(na) * 11 + q)
    P, nq, S = orc.canonical(na, pia, q)
    wa, nc, wc, pic = meta(engine, na, pia, q)
    N, M = int(np.prod(na)), int(np.prod(nc))
    for dt in (np.float32, np.float64):
        tdt = torch.float32 if dt == np.float32 else torch.float64
        a = rng.uniform(-1, 1, N + 3).astype(dt)
        b = rng.uniform(-1, 1, nq).astype(dt)
        da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        dc = torch.empty(M, dtype=tdt, device=dev)
        bmax = 16384 // np.dtype(dt).itemsize
        accs = (engine.ACC_COMPENSATED, engine.ACC_PLAIN)
        for oa in (0, 1, 2, 3):
            truth = orc.truth(S, nq, P, a[oa:oa + N], b)
            for split, acc in itertools.product((0, 1, 3, 17), accs):
                if (0 < split < -(-nq // bmax)) or split > nq:
                    continue
                dc.fill_(float("nan"))
                engine.ttv(q, len(na), da[oa:oa + N], na, wa, pia, db, [nq], dc, nc, wc, pic,
                           kind=engine.KIND_COL_BULK, split=split, accumulate=acc, sync=True)
                err = orc.rel_error(dc.cpu().numpy(), *truth)
                assert err <= TOL[dt], (na, pia, q, dt, oa, split, acc, err)
    a32 = rng.uniform(-1, 1, N).astype(np.float32)
    b = rng.uniform(-1, 1, nq).astype(np.float32)
    abf = torch.from_numpy(a32).to(torch.bfloat16)
    bits = abf.view(torch.int16).numpy().view(np.uint16).copy()
    dc = torch.empty(M, dtype=torch.float32, device=dev)
    engine.ttv(q, len(na), abf.to(dev).view(torch.int16), na, wa, pia, torch.from_numpy(b).to(dev), [nq],
               dc, nc, wc, pic, dtype=engine.BF16A, kind=engine.KIND_COL_BULK, sync=True)
    refb, absnb = orc.truth(S, nq, P, bits, b, kind="bf16a")
    assert orc.rel_error(dc.cpu().numpy(), refb, absnb) <= 1e-5


THIN_SHAPES = [
    ([64, 50000], [1, 2], 2),
    ([16, 30000, 3], [1, 2, 3], 2),
    ([4, 70000], [1, 2], 2),
    ([2, 9000, 5], [1, 2, 3], 2),
    ([128, 5000], [1, 2], 2),
    ([8, 4, 20000], [1, 2, 3], 3),
]


@pytest.mark.parametrize("na,pia,q", THIN_SHAPES)
def test_thin_prefix_column_kernel(engine, orc, torch_dev, na, pia, q):
    """Thin prefixes (P / V divides 32), few outputs, long contraction: several
    rows per warp step, every vector width and split, fp32 and fp64 both
    accumulation modes."""
    torch, dev = torch_dev
    rng = np.random.default_rng(sum(na) + 3 * q)
    P, nq, S = orc.canonical(na, pia, q)
    for dt in (np.float32, np.float64):
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
        b = rng.uniform(-1, 1, nq).astype(dt)
        truth = orc.truth(S, nq, P, a, b)
        vmax = 16 // np.dtype(dt).itemsize
        bmax = 16384 // np.dtype(dt).itemsize
        for v in (1, 2, 4):
            if v > vmax or P % v or 32 % (P // v):
                continue
            for split in (0, 1, 3, 17):
                if 0 < split < -(-nq // bmax):
                    continue
                for acc in (engine.ACC_COMPENSATED, engine.ACC_PLAIN):
                    check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth,
                          kind=engine.KIND_COL_THIN, vec=v, split=split, accumulate=acc)
        check(orc, engine, torch, dev, q, na, pia, a, b, truth=truth)   # the planner's choice


def test_pageable_host_pointers_refused(engine, torch_dev):
    """Pageable host memory never reaches a kernel: the C ABI refuses it (the
    host path, tlibg_ttv_host, is the way for host buffers)."""
    torch, dev = torch_dev
    na, pia, q = [8, 16, 4], [1, 2, 3], 2
    wa, nc, wc, pic = meta(engine, na, pia, q)
    a_h, b_h, c_h = torch.rand(512), torch.rand(16), torch.zeros(32)
    a_d, b_d, c_d = a_h.to(dev), b_h.to(dev), c_h.to(dev)
    for a, b, c in ((a_h, b_d, c_d), (a_d, b_h, c_d), (a_d, b_d, c_h)):
        with pytest.raises(engine.TTVError, match="device-accessible"):
            engine.ttv(q, 3, a, na, wa, pia, b, [16], c, nc, wc, pic, sync=True)
    engine.ttv(q, 3, a_d, na, wa, pia, b_d, [16], c_d, nc, wc, pic, sync=True)   # still usable
    assert engine.device_error() == 0


def test_bounded_wait_expiry_reports_timeout(engine, orc, torch_dev):
    """An mbarrier wait that nothing completes gives up after its poll limit:
    the call returns TLIBG_ERR_TIMEOUT with the engine's message, nothing
    traps or hangs, and the next TTV on the same context is correct."""
    import ctypes
    torch, dev = torch_dev
    L = engine.library()
    L.tlibg_selftest_bounded_wait.argtypes = [ctypes.c_void_p]
    st = L.tlibg_selftest_bounded_wait(torch.cuda.current_stream().cuda_stream)
    assert st == engine.ERR_TIMEOUT, st
    assert "bounded device wait expired" in engine._last_error()
    assert engine.device_error() == 0   # read and cleared by the call
    na, pia, q = [64, 48, 32], [1, 2, 3], 2
    rng = np.random.default_rng(1)
    a = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
    b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
    check(orc, engine, torch, dev, q, na, pia, a, b)
