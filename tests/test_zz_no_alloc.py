"""The allocation-free entry point, tlibg_ttv_f32_noalloc (GPU, through the C ABI).

Some callers cannot let this library allocate device memory: frameworks whose
caching allocator owns and accounts for every device byte, memory-budgeted or
multi-tenant processes, and latency-critical loops that cannot absorb the
implicit device synchronisation of cudaMalloc/cudaFree.  For them the split
reduction's partial sums live in one fixed array compiled into the library
(TLIBG_NOALLOC_SCRATCH_BYTES).  Here its results are checked against the
oracle's double-double truth and against the regular tlibg_ttv_f32 on the same
inputs, on two calls in a row with different data (stale partial sums of the
first call would show in the second); a call on a shape and stream the process
has not used before must leave the library's device-allocation count where it
was; a plan whose split needs more scratch than the array (an installed plan
hint) is planned again with fewer segments; and a problem that fits no plan
must be refused.

The file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 8 << 20   # TLIBG_NOALLOC_SCRATCH_BYTES in include/tlibg.h


def bind(engine):
    lib = engine.library()
    f = lib.tlibg_ttv_f32_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_size_t, C.c_size_t, C.c_void_p, engine._psz, engine._psz, engine._psz,
                  C.c_void_p, engine._psz, C.c_void_p, engine._psz, engine._psz, engine._psz,
                  C.c_void_p]
    return lib


def call(engine, fn, q, na, pia, A, b, c, stream):
    wa = engine.strides(na, pia)
    nc, pic = engine.output_shape(na, q), engine.output_layout(pia, q)
    wc = engine.strides(nc, pic)
    keep = [engine._sizes(v) for v in (na, wa, pia, [na[q - 1]], nc, wc, pic)]
    p = [engine._p(k) for k in keep]
    return fn(q, len(na), A.data_ptr(), p[0], p[1], p[2], b.data_ptr(), p[3], c.data_ptr(),
              p[4], p[5], p[6], stream)


def split_scratch_bytes(engine, q, na, pia):
    pl = engine.plan(q, na, pia)
    return pl["split"] * pl["S"] * pl["P"] * 8 if pl["split"] > 1 else 0


CASES = [
    ([64, 1 << 20], [1, 2], 2),           # thin prefix, long contraction: heavy split
    ([256, 256, 256], [1, 2, 3], 2),      # the plain CPU configuration's shape
    ([6, 1 << 20], [2, 1], 2),            # row kernel: q is the fastest mode
    ([33, 4099, 7], [1, 2, 3], 2),        # odd extents, scalar loads
]


def oracle_error(orc, engine, q, na, pia, A, b, c):
    """max |c - truth| / sum_k |a_ik b_k| against the oracle's fp64 truth."""
    P, nq, S = orc.canonical(na, pia, q)
    ref, absn = orc.truth(S, nq, P, A.cpu().numpy(), b.cpu().numpy())
    return orc.rel_error(c.cpu().numpy(), ref, absn)


@pytest.mark.parametrize("na,pia,q", CASES)
def test_noalloc_matches_regular_entry_point(engine, orc, cuda, na, pia, q):
    import torch
    lib = bind(engine)
    assert split_scratch_bytes(engine, q, na, pia) <= LIMIT
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device=cuda)
    g.manual_seed(sum(na) + q)
    N = int(np.prod(na))
    M = N // na[q - 1]
    for round_ in range(2):   # two calls in a row, different inputs each time
        A = torch.rand(N, generator=g, device=cuda) * 2 - 1
        b = torch.rand(na[q - 1], generator=g, device=cuda) * 2 - 1
        c_ref = torch.full((M,), float("nan"), device=cuda)
        c_new = torch.full((M,), float("nan"), device=cuda)
        assert call(engine, lib.tlibg_ttv_f32, q, na, pia, A, b, c_ref, stream) == 0
        st = call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c_new, stream)
        assert st == 0, engine._last_error()
        torch.cuda.synchronize()
        # the tolerance of the parity tests: 1e-5 of sum_k |a_ik b_k| per output
        pl = engine.plan(q, na, pia)
        P, nq, S = pl["P"], pl["nq"], pl["S"]
        absn = torch.einsum("sip,i->sp", A.view(S, nq, P).abs().double(), b.abs().double())
        err = ((c_new.double() - c_ref.double()).abs().view(S, P) / absn.clamp_min(1e-300)).max()
        assert not torch.isnan(c_new).any(), f"round {round_}: unwritten outputs"
        assert float(err) <= 1e-5, f"round {round_}: {float(err):.3e}"
        e_orc = oracle_error(orc, engine, q, na, pia, A, b, c_new)
        assert e_orc <= 1e-5, f"round {round_}: {e_orc:.3e} against the oracle"
    assert engine.device_error() == 0


def test_noalloc_allocates_nothing(engine, orc, cuda):
    """A shape and a stream this process has not used: the regular entry point
    allocates split scratch for the new stream, the allocation-free one does not."""
    import torch
    lib = bind(engine)
    na, pia, q = [96, 3 << 17], [1, 2], 2          # split reduction (thin prefix, long q)
    assert split_scratch_bytes(engine, q, na, pia) > 0
    g = torch.Generator(device=cuda)
    g.manual_seed(11)
    A = torch.rand(int(np.prod(na)), generator=g, device=cuda) * 2 - 1
    b = torch.rand(na[1], generator=g, device=cuda) * 2 - 1
    c = torch.full((na[0],), float("nan"), device=cuda)
    fresh = torch.cuda.Stream()
    torch.cuda.synchronize()
    before = engine.device_alloc_count()
    for _ in range(2):
        assert call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c, fresh.cuda_stream) == 0
    fresh.synchronize()
    assert engine.device_alloc_count() == before
    assert oracle_error(orc, engine, q, na, pia, A, b, c) <= 1e-5
    # the regular entry point on the same fresh stream does allocate its scratch
    c2 = torch.full((na[0],), float("nan"), device=cuda)
    assert call(engine, lib.tlibg_ttv_f32, q, na, pia, A, b, c2, fresh.cuda_stream) == 0
    fresh.synchronize()
    assert engine.device_alloc_count() > before
    assert engine.device_error() == 0


def test_noalloc_caps_an_oversize_split(engine, orc, cuda):
    """An installed plan hint asks for more segments than the array holds: the
    call plans again with the most segments that fit and still matches the
    oracle; the regular entry point keeps the hint."""
    import torch
    lib = bind(engine)
    na, pia, q = [1 << 14, 1 << 13], [1, 2], 2
    engine.plan_hint(engine.F32, 1 << 14, 1 << 13, 1, kind=engine.KIND_COL, split=128)
    try:
        assert engine.plan(q, na, pia)["split"] == 128
        assert split_scratch_bytes(engine, q, na, pia) > LIMIT
        g = torch.Generator(device=cuda)
        g.manual_seed(12)
        A = torch.rand(int(np.prod(na)), generator=g, device=cuda) * 2 - 1
        b = torch.rand(na[1], generator=g, device=cuda) * 2 - 1
        c = torch.full((na[0],), float("nan"), device=cuda)
        st = call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c,
                  torch.cuda.current_stream().cuda_stream)
        assert st == 0, engine._last_error()
        torch.cuda.synchronize()
        assert oracle_error(orc, engine, q, na, pia, A, b, c) <= 1e-5
    finally:
        engine.clear_plan_hint(engine.F32, 1 << 14, 1 << 13, 1)
    assert engine.plan(q, na, pia)["split"] != 128


def test_noalloc_refuses_oversize_scratch(engine, cuda):
    import torch
    lib = bind(engine)
    # a problem whose split reduction needs more than the fixed array
    pick = None
    for P in (1 << 18, 1 << 19, 1 << 20):
        for nq in (1 << 13, 1 << 14):
            na, pia, q = [P, nq], [1, 2], 2
            if split_scratch_bytes(engine, q, na, pia) > LIMIT:
                pick = (na, pia, q)
                break
        if pick:
            break
    assert pick is not None
    na, pia, q = pick
    A = torch.empty(int(np.prod(na)), device=cuda)   # never read: the call is refused first
    b = torch.empty(na[1], device=cuda)
    c = torch.empty(na[0], device=cuda)
    st = call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c,
              torch.cuda.current_stream().cuda_stream)
    assert st == engine.ERR_UNSUPPORTED
    msg = engine._last_error()
    assert "tlibg_ttv_f32_noalloc" in msg and str(LIMIT) in msg
    # invalid calls get the reference's text, as on the regular entry point
    keep = [engine._sizes(v) for v in ([4, 5], [1, 4], [1, 2], [7], [4], [1], [1])]
    p = [engine._p(k) for k in keep]
    st = lib.tlibg_ttv_f32_noalloc(2, 2, A.data_ptr(), p[0], p[1], p[2], b.data_ptr(), p[3],
                                   c.data_ptr(), p[4], p[5], p[6], None)
    assert st == engine.ERR_ARGUMENT
    assert engine._last_error() == ("Error in tlib::tensor_times_vector: contraction dimension "
                                    "of A and B are not equal.")


def test_noalloc_and_chain_captured_in_a_cuda_graph(engine, orc, cuda):
    """The allocation-free call (main kernel + its dependent combine) and the fused
    chain (dependent stages) captured into one CUDA graph and replayed on new data."""
    import torch
    lib = bind(engine)
    na, pia, q = [64, 1 << 20], [1, 2], 2          # heavy split: main kernel + combine
    cna = [48, 40, 56, 36]                           # chain: four stages' worth of modes
    s = torch.cuda.Stream(device=cuda)
    g = torch.Generator(device=cuda)
    g.manual_seed(77)
    A = torch.empty(int(np.prod(na)), device=cuda)
    b = torch.empty(na[q - 1], device=cuda)
    c = torch.empty(int(np.prod(na)) // na[q - 1], device=cuda)
    T4 = torch.empty(*cna, device=cuda)
    bs = [torch.empty(cna[m], device=cuda) for m in (0, 2, 3)]   # chain over every mode but 2

    def fill():
        A.uniform_(-1, 1, generator=g)
        b.uniform_(-1, 1, generator=g)
        T4.uniform_(-1, 1, generator=g)
        for v in bs:
            v.uniform_(-1, 1, generator=g)

    fill()
    with torch.cuda.stream(s):   # warm-up on the capture stream: scratch, symbol address, plans
        assert call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c, s.cuda_stream) == 0
        engine.ttvs(2, T4, bs, stream=s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        st = call(engine, lib.tlibg_ttv_f32_noalloc, q, na, pia, A, b, c, s.cuda_stream)
        out = engine.ttvs(2, T4, bs, stream=s)
    assert st == 0, engine._last_error()
    for _ in range(2):
        fill()
        c.fill_(float("nan"))
        out.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        assert oracle_error(orc, engine, q, na, pia, A, b, c) <= 1e-5
        ref, absn = orc.ttvs_truth(2, T4.view(-1).cpu().numpy(), cna, [4, 3, 2, 1],
                                   [v.cpu().numpy() for v in bs])
        assert orc.rel_error(out.cpu().numpy(), ref, absn) <= 1e-5
    assert engine.device_error() == 0
