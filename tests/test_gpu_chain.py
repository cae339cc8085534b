"""The fused multi-vector chain (ttvpy.ttvs, reference ttvpy/src/wrapped_ttv.cpp:
85-199) on the GPU, through tlibg_ttvs, against the oracle's double-double
truth of the full contraction (every mode but q, Kronecker weights in fp64).

* an order-4 tensor of more than 2^26 elements, every q, all three orders
  ("forward", "backward", "optimal"), fp32 and fp64, last-order layout (the
  ttvpy convention) -- bars 1e-5 / 1e-13 of sum |a w| per output;
* first-order and mixed layouts through the C ABI directly;
* bf16-stored A;
* the fused chain and the reference's step-by-step chain agree;
* no device allocation after the first call on a stream, and one kernel per
  stage (prefix rows, suffix columns, plus their split combines; a weight
  launch only for stages over several modes).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.float32: 1e-5, np.float64: 1e-13}
BIG = [96, 90, 88, 94]   # 71,464,960 elements (> 2^26)


@pytest.fixture(scope="module")
def big(cuda):
    import torch
    rng = np.random.default_rng(2604)
    a = rng.uniform(-1, 1, int(np.prod(BIG)))
    out = {}
    for dt in (np.float32, np.float64):
        h = a.astype(dt)
        out[dt] = (h, torch.from_numpy(h).to(cuda).view(*BIG))
    return out


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["fp32", "fp64"])
def test_fused_chain_full_size_all_orders(engine, orc, cuda, big, dt):
    import torch
    h, A = big[dt]
    rng = np.random.default_rng(7)
    pia = [4, 3, 2, 1]   # torch / NumPy row-major = the reference's last-order layout
    for q in range(1, 5):
        bs_h = [rng.uniform(-1, 1, BIG[m]).astype(dt) for m in range(4) if m != q - 1]
        bs = [torch.from_numpy(b).to(cuda) for b in bs_h]
        ref, absn = orc.ttvs_truth(q, h, BIG, pia, bs_h)
        for order in ("forward", "backward", "optimal"):
            c = engine.ttvs(q, A, bs, order)
            torch.cuda.synchronize()
            assert c.shape == (BIG[q - 1],)
            err = orc.rel_error(c.cpu().numpy(), ref, absn)
            assert err <= TOL[dt], (q, order, err)
    assert engine.device_error() == 0


def test_fused_chain_layouts_through_c_abi(engine, orc, cuda):
    """Any dense layout of A through the C entry point (vectors in mode order)."""
    import ctypes as C
    import torch
    lib = engine.library()
    rng = np.random.default_rng(9)
    for na, pia in (([40, 33, 27, 5], [1, 2, 3, 4]), ([40, 33, 27, 5], [2, 4, 1, 3]),
                    ([7, 600, 9], [3, 1, 2]), ([1000, 3], [1, 2]), ([3, 1000], [1, 2]),
                    ([4, 1, 5, 1, 6], [5, 4, 3, 2, 1])):
        p = len(na)
        wa = engine.strides(na, pia)
        for dt, code in ((np.float32, engine.F32), (np.float64, engine.F64)):
            a = rng.uniform(-1, 1, int(np.prod(na))).astype(dt)
            da = torch.from_numpy(a).to(cuda)
            for q in range(1, p + 1):
                bs_h = [rng.uniform(-1, 1, na[m]).astype(dt) for m in range(p) if m != q - 1]
                bs = [torch.from_numpy(b).to(cuda) for b in bs_h]
                c = torch.full((na[q - 1],), float("nan"), dtype=da.dtype, device=cuda)
                keep = [engine._sizes(v) for v in (na, wa, pia, [len(b) for b in bs_h])]
                ptrs = (C.c_void_p * (p - 1))(*[b.data_ptr() for b in bs])
                st = lib.tlibg_ttvs(code, q, p, da.data_ptr(), engine._p(keep[0]), engine._p(keep[1]),
                                    engine._p(keep[2]), ptrs, engine._p(keep[3]), c.data_ptr(), None)
                assert st == 0, engine._last_error()
                torch.cuda.synchronize()
                ref, absn = orc.ttvs_truth(q, a, na, pia, bs_h)
                err = orc.rel_error(c.cpu().numpy(), ref, absn)
                assert err <= TOL[dt], (na, pia, q, dt, err)


def test_fused_chain_bf16_and_step_by_step(engine, orc, cuda):
    import torch
    rng = np.random.default_rng(10)
    na = [30, 70, 50]
    a32 = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
    Abf = torch.from_numpy(a32).to(torch.bfloat16).view(*na).to(cuda)
    bits = Abf.cpu().view(torch.int16).numpy().view(np.uint16).ravel().copy()
    for q in (1, 2, 3):
        bs_h = [rng.uniform(-1, 1, na[m]).astype(np.float32) for m in range(3) if m != q - 1]
        bs = [torch.from_numpy(b).to(cuda) for b in bs_h]
        c = engine.ttvs(q, Abf, bs)
        ref, absn = orc.ttvs_truth(q, bits, na, [3, 2, 1], bs_h, kind="bf16a")
        assert orc.rel_error(c.cpu().numpy(), ref, absn) <= 1e-5
        # fp32: fused and the reference's step-by-step order agree within the bar
        A = torch.from_numpy(a32).view(*na).to(cuda)
        ref32, absn32 = orc.ttvs_truth(q, a32, na, [3, 2, 1], bs_h)
        for order in ("forward", "backward", "optimal"):
            f = engine.ttvs(q, A, bs, order).cpu().numpy()
            s = engine.ttvs(q, A, bs, order, fused=False).cpu().numpy()
            assert orc.rel_error(f, ref32, absn32) <= 1e-5
            assert orc.rel_error(s, ref32, absn32) <= 1e-5


def test_fused_chain_no_allocation_after_first_call(engine, cuda):
    import torch
    A = torch.rand(64, 48, 80, device=cuda)
    bs = [torch.rand(64, device=cuda), torch.rand(80, device=cuda)]
    engine.ttvs(2, A, bs)
    torch.cuda.synchronize()
    allocs, launches = engine.device_alloc_count(), engine.launch_count()
    for _ in range(3):
        engine.ttvs(2, A, bs)
    torch.cuda.synchronize()
    assert engine.device_alloc_count() == allocs
    # prefix rows + suffix columns (single modes: their vectors are the weights, no weight
    # launch), plus a combine where a stage splits its contraction: 2 to 4 per call
    assert 3 * 2 <= engine.launch_count() - launches <= 3 * 4


def test_fused_chain_unaligned_vectors(engine, orc, cuda):
    """Vectors at odd element offsets (a stage over one mode reads its vector in place)."""
    import torch
    rng = np.random.default_rng(12)
    for na in ([40, 33, 27, 5], [7, 600, 9], [3000, 2, 5]):
        p = len(na)
        a = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
        A = torch.from_numpy(a).view(*na).to(cuda)
        for q in range(1, p + 1):
            bs_h = [rng.uniform(-1, 1, na[m]).astype(np.float32) for m in range(p) if m != q - 1]
            bs = []
            for b in bs_h:
                buf = torch.empty(len(b) + 1, device=cuda)
                buf[1:] = torch.from_numpy(b).to(cuda)
                bs.append(buf[1:])
            c = engine.ttvs(q, A, bs)
            ref, absn = orc.ttvs_truth(q, a, na, list(range(p, 0, -1)), bs_h)
            assert orc.rel_error(c.cpu().numpy(), ref, absn) <= 1e-5, (na, q)
