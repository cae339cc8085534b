"""Batched TTVs in one persistent launch (GPU; through the C ABI).

Every problem of a random uneven batch (orders 3-5, extents 8..512 log-uniform,
random q and layout; smaller elements cap than the benchmark's 2^22 so the
oracle stays fast) must match the oracle within 1e-5 for every selection mode,
through the CUDA graph (replayed) and the direct launch, and the per-call path
must agree with it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(torch, dev, n, seed, max_elems=1 << 16):
    from ttv_gb300 import batch as B
    from ttv_gb300 import costmodel as CM
    shapes = CM.random_shapes(n, seed, max_elems=max_elems)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    probs, host = [], []
    for na, pia, q in shapes:
        N = int(np.prod(na))
        a = torch.rand(N, generator=g, device=dev) * 2 - 1
        b = torch.rand(na[q - 1], generator=g, device=dev) * 2 - 1
        c = torch.full((N // na[q - 1],), float("nan"), device=dev)
        probs.append(B.Problem(q, na, pia, a, b, c))
        host.append((na, pia, q))
    return probs, host


def check_all(orc, probs, host, tol=1e-5):
    worst = 0.0
    for pr, (na, pia, q) in zip(probs, host):
        P, nq, S = orc.canonical(na, pia, q)
        ref, absn = orc.truth(S, nq, P, pr.a.cpu().numpy(), pr.b.cpu().numpy())
        err = orc.rel_error(pr.c.cpu().numpy(), ref, absn)
        worst = max(worst, err)
        assert err <= tol, (na, pia, q, err)
    return worst


def reset(probs):
    for pr in probs:
        pr.c.fill_(float("nan"))


def test_batch_every_mode(engine, orc, cuda):
    import torch
    from ttv_gb300 import batch as B
    probs, host = make_batch(torch, cuda, 150, seed=11)
    # fixed rule, through the CUDA graph, replayed twice
    with B.Batch(probs) as bt:
        for _ in range(2):
            reset(probs)
            bt.launch()
            torch.cuda.synchronize()
            check_all(orc, probs, host)
        v = bt.variants()
        assert v.shape == (150,) and v.min() >= 0 and v.max() < B.NVARIANT
    # every forced variant (direct launches); the staged rows only where they apply
    _, kind, heur = B.features(probs)
    short_rows = np.array([k == engine.KIND_ROW and na[q - 1] <= 64 for k, (na, _p, q) in zip(kind, host)])
    assert short_rows.sum() >= 5
    for var in range(B.NVARIANT):
        reset(probs)
        with B.Batch(probs, select=B.SELECT_FIXED, variant=var, no_graph=True) as bt:
            bt.launch()
            torch.cuda.synchronize()
            check_all(orc, probs, host)
            got = bt.variants()
            if var == B.VARIANT_STAGED:
                assert np.array_equal(got, np.where(short_rows, var, heur))
            else:
                assert set(got) == {var}
    # per-problem given variants (staged rows given to column problems run the fixed rule)
    rng = np.random.default_rng(1)
    given = rng.integers(0, B.NVARIANT, len(probs))
    given[short_rows] = B.VARIANT_STAGED
    reset(probs)
    with B.Batch(probs, select=B.SELECT_GIVEN, variants=given) as bt:
        bt.launch()
        torch.cuda.synchronize()
        check_all(orc, probs, host)
        ran = bt.variants()
        ok = (given != B.VARIANT_STAGED) | short_rows
        assert np.array_equal(ran[ok], given[ok]) and np.array_equal(ran[~ok], heur[~ok])
    # learned selection with an (untrained) installed model: any choice is correct
    B.set_cost_model(B.init_params(3))
    try:
        reset(probs)
        with B.Batch(probs, select=B.SELECT_LEARNED) as bt:
            bt.launch()
            torch.cuda.synchronize()
            check_all(orc, probs, host)
    finally:
        B.set_cost_model(None)
    # plain accumulation and the per-call path
    reset(probs)
    with B.Batch(probs, accumulate=1) as bt:
        bt.launch()
        torch.cuda.synchronize()
        check_all(orc, probs, host)
    reset(probs)
    B.ttv_percall(probs)
    torch.cuda.synchronize()
    check_all(orc, probs, host)
    assert B.batch_device_error() == 0


def test_learned_without_model_falls_back(engine, orc, cuda):
    import torch
    from ttv_gb300 import batch as B
    probs, host = make_batch(torch, cuda, 40, seed=12)
    B.set_cost_model(None)
    _, _, heur = B.features(probs)
    with B.Batch(probs, select=B.SELECT_LEARNED) as bt:
        bt.launch()
        torch.cuda.synchronize()
        assert np.array_equal(bt.variants(), heur)
    check_all(orc, probs, host)
    given = np.full(len(probs), 5)
    reset(probs)
    with B.Batch(probs, select=B.SELECT_LEARNED, variants=given) as bt:
        bt.launch()
        torch.cuda.synchronize()
        assert np.array_equal(bt.variants(), given)   # tuned variants are the fallback
    check_all(orc, probs, host)


def test_batch_large_problems_split(engine, orc, cuda):
    """Problems big enough to split across CTAs (two-phase combine in the
    persistent kernel, last CTA of each problem)."""
    import torch
    from ttv_gb300 import batch as B
    shapes = [([64, 4096, 3], [1, 2, 3], 2), ([3, 64, 4096], [3, 2, 1], 3), ([2, 3, 8192], [1, 2, 3], 3),
              ([500, 500, 7], [2, 1, 3], 2), ([5, 5000, 9], [3, 1, 2], 2)]
    probs, host = [], []
    for na, pia, q in shapes:
        N = int(np.prod(na))
        a = torch.rand(N, device=cuda) * 2 - 1
        b = torch.rand(na[q - 1], device=cuda) * 2 - 1
        c = torch.full((N // na[q - 1],), float("nan"), device=cuda)
        probs.append(B.Problem(q, na, pia, a, b, c))
        host.append((na, pia, q))
    for var in range(B.NVARIANT):
        reset(probs)
        with B.Batch(probs, select=B.SELECT_FIXED, variant=var) as bt:
            bt.launch()
            bt.launch()   # replay: counters reset by the plan kernel
            torch.cuda.synchronize()
        check_all(orc, probs, host)


def test_one_shot_and_errors(engine, orc, cuda):
    import torch
    from ttv_gb300 import batch as B
    probs, host = make_batch(torch, cuda, 20, seed=13)
    B.ttv_batch(probs)
    torch.cuda.synchronize()
    check_all(orc, probs, host)
    reset(probs)
    B.ttv_batch_f32(probs)   # learned selection through the short entry point
    check_all(orc, probs, host)
    bad = B.Problem(2, [4, 5, 6], [1, 2, 3], probs[0].a, probs[0].b, probs[0].c)
    bad._keep[3][0] = 7   # nb != na[q-1]
    with pytest.raises(engine.TTVError, match="contraction dimension of A and B are not equal"):
        B.Batch([probs[1], bad])
    with pytest.raises(engine.TTVError, match="variant must be in 0..8"):
        B.Batch(probs, select=B.SELECT_FIXED, variant=9)


def test_recorded_costs(engine, orc, cuda):
    """A recording batch returns every problem's SM cycles and the same results."""
    import torch
    from ttv_gb300 import batch as B
    probs, host = make_batch(torch, cuda, 64, seed=14)
    with B.Batch(probs, select=B.SELECT_FIXED, variant=0, no_graph=True,
                 record_costs=True) as bt:
        bt.launch()
        torch.cuda.synchronize()
        c1 = bt.costs()
        check_all(orc, probs, host)
        reset(probs)
        bt.set_variant(2)
        bt.launch()
        torch.cuda.synchronize()
        c2 = bt.costs()
        check_all(orc, probs, host)
        reset(probs)
        bt.set_variant(B.VARIANT_STAGED)   # short rows staged, the rest their fixed rule
        bt.launch()
        torch.cuda.synchronize()
        c3 = bt.costs()
        check_all(orc, probs, host)
    assert (c1 > 0).all() and (c2 > 0).all() and (c3 > 0).all()
    with B.Batch(probs) as bt:   # not recording: costs stay zero
        bt.launch()
        assert (bt.costs() == 0).all()
