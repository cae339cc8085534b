"""The general-stride extension, tlibg_ttv_strided (no reference counterpart:
the drop-in calls keep the reference's dense-only rule).  Natural meaning of
every stride: A's element (i_1..i_p) at a[sum i_r wa[r]], b's i-th at b[i wb],
C's element at c[sum j_r wc[r]].  Truth: numpy fp64 over the same strided
views (as_strided), error max |c - ref| / sum |a b| against the bars 1e-5
(fp32) and 1e-13 (fp64); C's untouched elements (padding) must stay as they
were.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.float32: 1e-5, np.float64: 1e-13}


def view(buf, shape, strides):
    return np.lib.stride_tricks.as_strided(buf, shape=shape, strides=[s * buf.itemsize for s in strides])


def padded_strides(na, pia, rng, pad_max=3):
    """Strides of a padded dense tensor in layout pia (each mode's stride at least
    the span of the faster ones)."""
    w = [0] * len(na)
    span = 1
    for m in pia:
        w[m - 1] = span
        span *= na[m - 1] + int(rng.integers(0, pad_max + 1))
    return w


def case(rng, dt, p, max_elems=1 << 18):
    while True:
        na = [int(x) for x in rng.integers(1, 24, p)]
        if np.prod(na) <= max_elems:
            break
    pia = [int(x) + 1 for x in rng.permutation(p)]
    q = int(rng.integers(1, p + 1))
    wa = padded_strides(na, pia, rng)
    nc = [n for m, n in enumerate(na) if m != q - 1]
    pic = [int(x) + 1 for x in rng.permutation(p - 1)]
    wc = padded_strides(nc, pic, rng)
    wb = int(rng.integers(1, 4))
    return na, pia, q, wa, nc, pic, wc, wb


def run_case(engine, torch, dev, rng, dt, na, pia, q, wa, nc, pic, wc, wb):
    p = len(na)
    size_a = 1 + sum((n - 1) * w for n, w in zip(na, wa))
    size_c = 1 + sum((n - 1) * w for n, w in zip(nc, wc))
    nq = na[q - 1]
    abuf = rng.uniform(-1, 1, size_a).astype(dt)
    bbuf = rng.uniform(-1, 1, (nq - 1) * wb + 1).astype(dt)
    cbuf = np.full(size_c, 7.0, dt)
    Av, bv = view(abuf, na, wa).astype(np.float64), view(bbuf, [nq], [wb]).astype(np.float64)
    ref = np.tensordot(Av, bv, axes=([q - 1], [0]))
    absn = np.tensordot(np.abs(Av), np.abs(bv), axes=([q - 1], [0]))
    da, db, dc = (torch.from_numpy(x).to(dev) for x in (abuf, bbuf, cbuf))
    engine.ttv_strided(q, p, da, na, wa, pia, db, [nq], dc, nc, wc, pic, wb=wb)
    torch.cuda.synchronize()
    out = dc.cpu().numpy()
    got = view(out, nc, wc).astype(np.float64)
    err = np.max(np.abs(got - ref) / np.maximum(absn, 1e-300)) if ref.size else 0.0
    # every element C's strides do not address keeps its value
    mask = np.ones(size_c, bool)
    idx = np.zeros(1, np.int64)
    for n, w in zip(nc, wc):
        idx = (idx[:, None] + np.arange(n) * w).ravel()
    mask[idx] = False
    assert (out[mask] == 7.0).all()
    return err


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["fp32", "fp64"])
def test_random_padded_views(engine, cuda, dt):
    import torch
    rng = np.random.default_rng(5150 if dt == np.float32 else 5151)
    worst = 0.0
    for t in range(60):
        na, pia, q, wa, nc, pic, wc, wb = case(rng, dt, int(rng.integers(2, 6)))
        err = run_case(engine, torch, cuda, rng, dt, na, pia, q, wa, nc, pic, wc, wb)
        assert err <= TOL[dt], (na, pia, q, wa, nc, pic, wc, wb, err)
        worst = max(worst, err)


def test_long_rows_and_columns(engine, cuda):
    """Row form (q fastest, warp per output) and column form with long contractions."""
    import torch
    rng = np.random.default_rng(77)
    for dt in (np.float32, np.float64):
        for na, pia, q in (([3000, 40], [1, 2], 1), ([40, 3000], [1, 2], 2), ([17, 999, 13], [2, 1, 3], 2),
                           ([1, 5000, 1], [1, 2, 3], 2), ([300, 1, 200], [3, 1, 2], 1)):
            wa = padded_strides(na, pia, rng)
            nc = [n for m, n in enumerate(na) if m != q - 1]
            pic = list(range(1, len(nc) + 1))
            wc = padded_strides(nc, pic, rng)
            err = run_case(engine, torch, cuda, rng, dt, na, pia, q, wa, nc, pic, wc, 2)
            assert err <= TOL[dt], (na, pia, q, dt, err)


def test_dense_strides_match_the_dense_call(engine, orc, cuda):
    import torch
    rng = np.random.default_rng(9)
    for na, pia, q in (([64, 48, 80], [1, 2, 3], 2), ([25, 25, 25, 25], [4, 3, 2, 1], 3), ([7, 300], [2, 1], 2)):
        p = len(na)
        wa = engine.strides(na, pia)
        nc, pic = engine.output_shape(na, q), engine.output_layout(pia, q)
        wc = engine.strides(nc, pic)
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
        da, db = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
        c1 = torch.empty(int(np.prod(nc)), device=cuda)
        c2 = torch.empty_like(c1)
        engine.ttv(q, p, da, na, wa, pia, db, [na[q - 1]], c1, nc, wc, pic, sync=True)
        engine.ttv_strided(q, p, da, na, wa, pia, db, [na[q - 1]], c2, nc, wc, pic)
        P, nq, S = orc.canonical(na, pia, q)
        ref, absn = orc.truth(S, nq, P, a, b)
        assert orc.rel_error(c2.cpu().numpy(), ref, absn) <= 1e-5
        assert orc.rel_error(c1.cpu().numpy(), ref, absn) <= 1e-5


def test_torch_views(engine, cuda):
    """ttv_view: slices, transposes and a strided b, no copy, against torch in fp64."""
    import torch
    g = torch.Generator(device=cuda)
    g.manual_seed(3)
    base = torch.rand(64, 90, 70, generator=g, device=cuda, dtype=torch.float64) * 2 - 1
    bb = torch.rand(300, generator=g, device=cuda, dtype=torch.float64) * 2 - 1
    for A in (base[:, ::2, 5:60], base.transpose(0, 2), base[::3].permute(1, 2, 0), base[10:20, :, ::7]):
        for q in range(1, 4):
            n = A.shape[q - 1]
            b = bb[: 2 * n : 2]
            c = engine.ttv_view(q, A, b)
            ref = torch.tensordot(A, b, dims=([q - 1], [0]))
            absn = torch.tensordot(A.abs(), b.abs(), dims=([q - 1], [0]))
            torch.cuda.synchronize()
            assert c.shape == ref.shape
            assert ((c - ref).abs() / absn.clamp_min(1e-300)).max().item() <= 1e-13


def test_vector_forms(engine, cuda):
    """Views on the 16-byte grid take the 16-byte forms: padded rows contracted
    along the row (row form) and across rows (column form, which takes them when
    the outputs fill the GPU: the 4 x 800 x 800 view), fp32 and fp64, with rows
    long and short, against torch in fp64."""
    import torch
    g = torch.Generator(device=cuda)
    g.manual_seed(11)
    for dt, V in ((torch.float32, 4), (torch.float64, 2)):
        for shape, pad in (((48, 30, 64), 4), ((7, 5, 1000), 8), ((3, 200, 8), 2 * V), ((4, 800, 800), 8)):
            base = torch.rand(shape[0], shape[1], shape[2] + pad, generator=g, device=cuda, dtype=dt) * 2 - 1
            A = base[:, :, :shape[2]]
            for q in (1, 2, 3):
                b = torch.rand(A.shape[q - 1], generator=g, device=cuda, dtype=dt) * 2 - 1
                c = engine.ttv_view(q, A, b)
                ref = torch.tensordot(A.double(), b.double(), dims=([q - 1], [0]))
                absn = torch.tensordot(A.double().abs(), b.double().abs(), dims=([q - 1], [0]))
                bar = 1e-5 if dt == torch.float32 else 1e-13
                assert ((c.double() - ref).abs() / absn.clamp_min(1e-300)).max().item() <= bar, (dt, shape, q)
