"""The C ABI and the host-side logic, without a GPU.

* libttvgpu.so loads and exports every entry point include/tlibg.h declares;
* invalid calls fail with the reference's exception text, in the reference's
  order of checks (golden errors.json), before any device work;
* valid calls without a device fail loudly (no CPU fallback);
* the metadata helpers reproduce the reference's (golden metadata.json);
* the planner picks the kernel family the layout calls for;
* the C++ drop-in header compiles against the reference's own dispatch and in
  standalone mode, and maps errors to std::runtime_error with the same text;
* ttvs' contraction order bookkeeping (forward / backward / optimal).
"""
import ctypes as C
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
HEADER = os.path.join(ROOT, "include", "tlibg.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tlibg_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(engine):
    lib = engine.library()
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in tlibg.h but not exported"


def _call(engine, dtype, q, p, na, wa, pia, nb, nc, wc, pic, a=16, b=32, c=48):
    sizes = engine._sizes
    keep = [sizes(v) for v in (na, wa, pia, nb, nc, wc, pic)]
    o = engine._options()
    return engine.library().tlibg_ttv_ex(dtype, q, p, a, *[engine._p(k) for k in keep[:3]], b,
                                         engine._p(keep[3]), c,
                                         *[engine._p(k) for k in keep[4:]], C.byref(o), None)


def test_invalid_calls_match_reference_messages(engine):
    with open(os.path.join(GOLDEN, "errors.json")) as f:
        cases = json.load(f)
    for case in cases:
        x = case["args"]
        nc = x["nc"] if x["nc"] else []
        for dt in (engine.F32, engine.F64):
            st = _call(engine, dt, x["q"], x["p"], x["na"], x["wa"], x["pia"], x["nb"], nc or [0],
                       x["wc"] or [0], x["pic"] or [0]) if x["p"] != 1 else _order1(engine, dt)
            if case["status"] == 0:
                # valid for the reference: past validation, the engine refuses the stand-in
                # pointers loudly (no device; with a device they are not device memory)
                msg = engine._last_error()
                assert st in (engine.ERR_CUDA, engine.OK) or (
                    st == engine.ERR_ARGUMENT and "device-accessible" in msg), msg
            else:
                assert st == engine.ERR_ARGUMENT
                assert engine._last_error() == case["message"]


def _order1(engine, dt):
    sizes = engine._sizes
    keep = [sizes([3]), sizes([1]), sizes([1]), sizes([3])]
    o = engine._options()
    # C of an order-1 tensor has no modes: nc is an empty range
    return engine.library().tlibg_ttv_ex(dt, 1, 1, 16, *[engine._p(k) for k in keep[:3]], 32,
                                         engine._p(keep[3]), 48, engine._p(sizes([1])),
                                         engine._p(sizes([1])), engine._p(sizes([1])), C.byref(o),
                                         None)


def test_null_pointer_checks(engine):
    na, wa, pia = [2, 3, 4], [1, 2, 6], [1, 2, 3]
    E = "Error in tlib::tensor_times_vector: "
    st = _call(engine, engine.F32, 2, 3, na, wa, pia, [3], [2, 4], [1, 2], [1, 2], a=None)
    assert st == engine.ERR_ARGUMENT
    assert engine._last_error() == E + "pointer to input tensor A should not be zero."
    st = _call(engine, engine.F32, 2, 3, na, wa, pia, [3], [2, 4], [1, 2], [1, 2], c=None)
    assert engine._last_error() == E + "pointer to output tensor C should not be zero."
    lib, o = engine.library(), engine._options()
    st = lib.tlibg_ttv_ex(0, 2, 3, 16, None, engine._p(engine._sizes(wa)),
                          engine._p(engine._sizes(pia)), 32, engine._p(engine._sizes([3])), 48,
                          engine._p(engine._sizes([2, 4])), engine._p(engine._sizes([1, 2])),
                          engine._p(engine._sizes([1, 2])), C.byref(o), None)
    assert st == engine.ERR_ARGUMENT
    assert engine._last_error() == E + "pointer to input tensor shape vector na should not be zero."


def test_non_dense_strides_are_refused(engine):
    # valid (monotone) for the reference, but not dense: outside this engine
    st = _call(engine, engine.F32, 2, 3, [2, 3, 4], [1, 3, 9], [1, 2, 3], [3], [2, 4], [1, 2],
               [1, 2])
    assert st == engine.ERR_UNSUPPORTED
    assert "dense" in engine._last_error()


def test_valid_call_without_device_fails_loudly(engine):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    st = _call(engine, engine.F32, 2, 3, [2, 3, 4], [1, 2, 6], [1, 2, 3], [3], [2, 4], [1, 2],
               [1, 2])
    assert st == engine.ERR_CUDA
    with pytest.raises(engine.DeviceError):
        engine.ttv(2, 3, torch.zeros(24), [2, 3, 4], [1, 2, 6], [1, 2, 3], torch.zeros(3), [3],
                   torch.zeros(8), [2, 4], [1, 2], [1, 2])


def test_metadata_helpers_match_reference(engine):
    with open(os.path.join(GOLDEN, "metadata.json")) as f:
        meta = json.load(f)
    for na, q, nc in meta["output_shape"]:
        assert engine.output_shape(na, q) == nc
    for pia, q, pic in meta["output_layout"]:
        assert engine.output_layout(pia, q) == pic
    for n, pi, w in meta["strides"]:
        assert engine.strides(n, pi) == w
    for p, k, pi in meta["k_order"]:
        assert engine.k_order_layout(p, k) == pi
    for pi in ([1, 2, 3], [3, 1, 2], [2, 4, 1, 3]):
        for m in range(1, len(pi) + 1):
            assert pi[engine.inverse_mode(pi, m) - 1] == m
    with pytest.raises(engine.TTVError, match="input shape is not valid"):
        engine.output_shape([2, 0, 3], 1)
    with pytest.raises(engine.TTVError, match="input layout is not valid"):
        engine.output_layout([1, 1, 3], 1)
    with pytest.raises(engine.TTVError, match="compute_strides"):
        engine.strides([2, 3], [1, 3])


def test_planner_kernel_family(engine):
    # q-fastest rows: aligned -> register row kernel; unaligned rows of 64 or more
    # elements, many of them -> the row-shift kernel (fp32 and fp64), few -> row kernel
    assert engine.plan(1, [64, 32, 16], [1, 2, 3])["kind"] == engine.KIND_ROW
    assert engine.plan(3, [645, 645, 645], [3, 2, 1])["kind"] == engine.KIND_ROW_SHIFT
    assert engine.plan(3, [645, 645, 645], [3, 2, 1], dtype=engine.F64)["kind"] == engine.KIND_ROW_SHIFT
    assert engine.plan(1, [645, 99], [1, 2])["kind"] == engine.KIND_ROW
    assert engine.plan(3, [645, 645, 645], [3, 2, 1], vec=1)["kind"] == engine.KIND_ROW
    assert engine.plan(1, [4001, 9999], [1, 2])["kind"] == engine.KIND_ROW   # copies of b over 48 KB
    # rows that fill few rounds of lane groups are split in two (16384 rows of 16384 over the
    # lane groups of 152 SMs without a device); rows that fill many rounds are not
    assert engine.plan(1, [16384, 16384], [1, 2])["split"] == 2
    assert engine.plan(1, [16384, 16384], [1, 2], dtype=engine.F64)["split"] == 2
    assert engine.plan(1, [4096, 65536], [1, 2])["split"] == 1
    # unaligned fp32 rows under 64 elements: the row-tile kernel; aligned ones the row kernel
    assert engine.plan(3, [25, 25, 25], [3, 2, 1])["kind"] == engine.KIND_ROW_TILE
    assert engine.plan(1, [63, 99], [1, 2])["kind"] == engine.KIND_ROW_TILE
    assert engine.plan(1, [16, 99], [1, 2])["kind"] == engine.KIND_ROW
    assert engine.plan(1, [65, 99], [1, 2])["kind"] == engine.KIND_ROW
    assert engine.plan(3, [25, 25, 25], [3, 2, 1], kind=engine.KIND_STREAM)["kind"] == engine.KIND_STREAM
    # fp64 rows of at most 64 elements: the row-tile kernel (native-DFMA mode keeps the row kernel)
    assert engine.plan(1, [25, 25, 25], [1, 2, 3], dtype=engine.F64)["kind"] == engine.KIND_ROW_TILE
    assert engine.plan(1, [25, 25, 25], [1, 2, 3], dtype=engine.F64)["block"] == 128
    assert engine.plan(1, [32, 9], [1, 2], dtype=engine.F64)["kind"] == engine.KIND_ROW_TILE
    assert engine.plan(1, [33, 9], [1, 2], dtype=engine.F64)["kind"] == engine.KIND_ROW
    # fp64 rows under 8 elements: native DFMA in the row-tile kernel unless the mix is asked for
    pl = engine.plan(1, [5, 999], [1, 2], dtype=engine.F64)
    assert pl["kind"] == engine.KIND_ROW_TILE and pl["accumulate"] == engine.ACC_PLAIN
    assert engine.plan(1, [5, 999], [1, 2], dtype=engine.F64,
                       accumulate=engine.ACC_DOUBLE_FLOAT)["accumulate"] == engine.ACC_COMPENSATED
    assert engine.plan(1, [25, 25, 25], [1, 2, 3], dtype=engine.F64,
                       accumulate=engine.ACC_PLAIN)["kind"] == engine.KIND_ROW
    assert engine.plan(1, [16, 4096], [1, 2], kind=engine.KIND_ROW_TILE)["kind"] == engine.KIND_ROW_TILE
    with pytest.raises(engine.TTVError):
        engine.plan(1, [65, 9], [1, 2], kind=engine.KIND_ROW_TILE)
    with pytest.raises(engine.TTVError):
        engine.plan(2, [16, 9], [1, 2], kind=engine.KIND_ROW_TILE)
    # the TMA-staged column kernel: on request for any prefix P > 1, 288 threads
    pl = engine.plan(2, [645, 33, 7], [1, 2, 3], kind=engine.KIND_COL_BULK)
    assert pl["kind"] == engine.KIND_COL_BULK and pl["block"] == 288 and pl["vec"] == 4
    assert engine.plan(2, [645, 33, 7], [1, 2, 3], dtype=engine.F64, kind=engine.KIND_COL_BULK)["vec"] == 2
    assert engine.plan(2, [645, 33, 7], [1, 2, 3])["kind"] == engine.KIND_COL
    with pytest.raises(engine.TTVError):
        engine.plan(1, [16, 9], [1, 2], kind=engine.KIND_COL_BULK)
    assert engine.plan(1, [645, 645, 645], [1, 2, 3], dtype=engine.F64)["kind"] == engine.KIND_ROW_SHIFT
    # fp64 column kernel: the DFMA / double-float mix by default
    assert engine.plan(2, [64, 32, 16], [1, 2, 3], dtype=engine.F64)["accumulate"] == \
        engine.ACC_COMPENSATED
    assert engine.plan(2, [256, 32, 64], [1, 2, 3])["kind"] == engine.KIND_COL
    # its column form on request
    assert engine.plan(2, [645, 645, 645], [1, 2, 3], kind=engine.KIND_STREAM)["kind"] == \
        engine.KIND_STREAM
    # long rows: the register kernels (q fastest -> row kernel, else column kernel)
    assert engine.plan(1, [16384, 16384], [1, 2])["kind"] == engine.KIND_ROW
    assert engine.plan(2, [16384, 16384], [1, 2])["kind"] == engine.KIND_COL
    # prefix rows not 16-byte aligned: scalar loads (two outputs per thread); the
    # realigning kernel on request
    assert engine.plan(3, [645, 645, 645], [1, 2, 3])["kind"] == engine.KIND_COL
    assert engine.plan(3, [645, 645, 645], [1, 2, 3])["vec"] == 1
    assert engine.plan(3, [645, 645, 645], [1, 2, 3], dtype=engine.F64)["kind"] == engine.KIND_COL
    assert engine.plan(3, [645, 645, 645], [1, 2, 3], kind=engine.KIND_COL_REALIGN)["vec"] == 4
    assert engine.plan(2, [25, 25, 25], [1, 2, 3])["kind"] == engine.KIND_COL
    assert engine.plan(3, [645, 645, 645], [1, 2, 3], dtype=engine.BF16A)["kind"] == engine.KIND_COL
    assert engine.plan(2, [25, 25, 25], [1, 2, 3], kind=engine.KIND_COL_REALIGN)["kind"] == \
        engine.KIND_COL_REALIGN
    with pytest.raises(engine.TTVError, match="realigning column kernel"):
        engine.plan(1, [25, 25, 25], [1, 2, 3], kind=engine.KIND_COL_REALIGN)
    # thin prefix, few outputs, long contraction: several rows per warp step
    assert engine.plan(2, [64, 1 << 22], [1, 2])["kind"] == engine.KIND_COL_THIN
    assert engine.plan(2, [16, 1 << 20, 16], [1, 2, 3])["kind"] == engine.KIND_COL_THIN
    assert engine.plan(2, [64, 1 << 22], [1, 2], dtype=engine.F64)["kind"] == engine.KIND_COL_THIN
    assert engine.plan(2, [16, 16, 1 << 20], [1, 2, 3])["kind"] == engine.KIND_COL   # many outputs
    with pytest.raises(engine.TTVError, match="thin-prefix column kernel"):
        engine.plan(2, [24, 1000], [1, 2], kind=engine.KIND_COL_THIN)
    # forced register kernels
    R, Cn = engine.KIND_ROW, engine.KIND_COL
    assert engine.plan(1, [64, 32, 16], [1, 2, 3], kind=R)["kind"] == R
    assert engine.plan(3, [64, 32, 16], [3, 2, 1], kind=R)["kind"] == R
    pl = engine.plan(2, [256, 256, 256], [1, 2, 3], kind=Cn)
    assert (pl["P"], pl["nq"], pl["S"]) == (256, 256, 256)
    assert pl["vec"] == 4 and pl["accumulate"] == engine.ACC_COMPENSATED
    # odd prefix: scalar loads; fp64: 2 per 16-byte load; bf16: 8
    assert engine.plan(2, [25, 25, 25], [1, 2, 3], kind=Cn)["vec"] == 1
    assert engine.plan(2, [256, 256, 256], [1, 2, 3], dtype=engine.F64, kind=Cn)["vec"] == 2
    assert engine.plan(2, [256, 256, 256], [1, 2, 3], dtype=engine.BF16A, kind=Cn)["vec"] == 8
    with pytest.raises(engine.TTVError, match="streamed kernel"):
        engine.plan(1, [16384, 16384], [1, 2], kind=engine.KIND_STREAM)
    # long contraction with a thin prefix is split, and segments fit the staged b
    pl = engine.plan(2, [64, 1 << 22], [1, 2], kind=Cn)
    assert pl["kind"] == Cn and pl["split"] >= (1 << 22) // 4096
    assert engine.plan(2, [64, 1 << 22], [1, 2], kind=engine.KIND_STREAM)["split"] > 1
    # forced options are honoured or refused
    assert engine.plan(2, [256, 256, 256], [1, 2, 3], kind=Cn, group=2, split=3)["group"] == 2
    with pytest.raises(engine.TTVError):
        engine.plan(1, [256, 256, 256], [1, 2, 3], kind=engine.KIND_COL)


def _compile_cpp(tmp_path, standalone):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ missing")
    import oracle
    ref_inc = oracle.REF_INCLUDE   # the staged reference headers (or TTV_REFERENCE_INCLUDE)
    if not standalone and not os.path.isdir(os.path.join(ref_inc, "tlib")):
        pytest.skip("reference headers absent")
    exe = str(tmp_path / ("kat_sa" if standalone else "kat_ref"))
    cuda_inc = "/usr/local/cuda/include"
    cmd = [gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "ttv_gpu_kat.cpp"), "-o", exe,
           "-L", os.path.join(ROOT, "ttv_gb300"), "-lttvgpu", "-L/usr/local/cuda/lib64",
           "-lcudart", "-Wl,-rpath," + os.path.join(ROOT, "ttv_gb300")]
    if standalone:
        cmd.insert(2, "-DTLIBG_STANDALONE")
    else:
        cmd[3:3] = ["-I", ref_inc, "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("standalone", [False, True])
def test_cpp_header_dispatch_and_messages(engine, tmp_path, standalone):
    exe = _compile_cpp(tmp_path, standalone)
    r = subprocess.run([exe, "validate"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout


def test_ttvs_contraction_order(engine, monkeypatch):
    """ttvs' mode bookkeeping against the reference's Python tests
    (ttvpy/tests/test.py), with the per-step TTV done by einsum on the CPU."""
    import torch

    def cpu_ttv(q, A, b, **kw):
        return torch.tensordot(A, b, dims=([q - 1], [0]))

    monkeypatch.setattr(engine, "ttv_array", cpu_ttv)
    A = torch.arange(3 * 2 * 4 * 5, dtype=torch.float64).reshape(3, 2, 4, 5)
    for q in range(1, 5):
        dims = [d for d in range(4) if d != q - 1]
        B = [torch.arange(A.shape[d], dtype=torch.float64) for d in dims]
        D = A
        for d, bj in sorted(zip(dims, B), key=lambda t: -t[0]):
            D = torch.tensordot(D, bj, dims=([d], [0]))
        for order in ("forward", "backward", "optimal"):
            Cq = engine.ttvs(q, A, B, order, fused=False)
            assert torch.equal(Cq, D), (q, order)
    with pytest.raises(ValueError, match="multiplication order"):
        engine.ttvs(1, A, B, "sideways")
    with pytest.raises(ValueError, match="number of input vectors"):
        engine.ttvs(1, A, B[:2])


def test_ttvs_entry_point_checks(engine):
    """tlibg_ttvs refuses bad calls with ttvpy's messages before touching memory."""
    import ctypes as C
    lib = engine.library()
    buf = (C.c_float * 64)()
    vec = (C.c_void_p * 3)(C.addressof(buf), C.addressof(buf), C.addressof(buf))

    def call(q, p, na, nbs, pia=None):
        pia = pia or list(range(1, p + 1))
        wa = engine.strides(na, pia) if p else [1]
        keep = [engine._sizes(v) for v in (na or [1], wa, pia or [1], nbs or [1])]
        st = lib.tlibg_ttvs(engine.F32, q, p, C.addressof(buf), engine._p(keep[0]), engine._p(keep[1]),
                            engine._p(keep[2]), vec, engine._p(keep[3]), C.addressof(buf), None)
        return st, engine._last_error()

    assert call(1, 0, [], []) == (engine.ERR_ARGUMENT, "Error calling ttvpy::ttvs: input tensor "
                                  "order should be greater than zero.")
    st, msg = call(5, 4, [2, 3, 4, 5], [2, 3, 4])
    assert st == engine.ERR_ARGUMENT and "contraction mode should be greater than zero" in msg
    st, msg = call(2, 4, [2, 3, 4, 5], [2, 4, 4])
    assert st == engine.ERR_ARGUMENT and msg == ("Error calling ttvpy::ttvs: vector dimension is not "
                                                 "compatible with the dimension of a tensor mode.")
    st, msg = call(1, 1, [7], [])
    assert st == engine.ERR_ARGUMENT and "order 1" in msg
    # a valid call gets as far as the device (none here)
    import torch
    if not torch.cuda.is_available():
        st, msg = call(2, 4, [2, 3, 4, 5], [2, 4, 5])
        assert st in (engine.ERR_CUDA, engine.ERR_ARGUMENT), msg


def test_ttvs_truth_matches_einsum(orc):
    """The oracle's chain truth (Kronecker weights, double-double sum) against
    float64 tensordot chains, for first- and last-order layouts."""
    rng = np.random.default_rng(8)
    na = [5, 3, 4, 6]
    A = rng.uniform(-1, 1, int(np.prod(na)))
    for pia in ([1, 2, 3, 4], [4, 3, 2, 1], [2, 4, 1, 3]):
        # the tensor with layout pia: element (i1..i4) at sum i_r w_r
        wa = orc.strides(na, pia)
        T = np.zeros(na)
        for idx in np.ndindex(*na):
            T[idx] = A[sum(i * w for i, w in zip(idx, wa))]
        for q in range(1, 5):
            bs = [rng.uniform(-1, 1, na[m]) for m in range(4) if m != q - 1]
            D = T
            for d, bj in sorted(zip([m for m in range(4) if m != q - 1], bs), key=lambda t: -t[0]):
                D = np.tensordot(D, bj, axes=([d], [0]))
            ref, absn = orc.ttvs_truth(q, A, na, pia, bs)
            assert np.allclose(ref, D, rtol=0, atol=1e-13), (pia, q)


def test_validate_only_entry_point(engine):
    """tlibg_validate runs the reference's checks on metadata alone."""
    L, sz = engine.library(), engine._sizes
    ok = [sz(v) for v in ([4, 5, 6], [1, 4, 20], [1, 2, 3], [5], [4, 6], [1, 4], [1, 2])]
    assert L.tlibg_validate(2, 3, *[engine._p(k) for k in ok]) == 0
    bad = list(ok)
    bad[3] = sz([7])
    assert L.tlibg_validate(2, 3, *[engine._p(k) for k in bad]) == 1
    assert "contraction dimension of A and B are not equal" in engine._last_error()


def test_undersized_tensors_are_refused_before_launch(engine):
    """Tensors smaller than their layout addresses never reach a kernel; the
    reference's own messages still come first."""
    torch = pytest.importorskip("torch")
    na, pia, q = [4, 5, 6], [1, 2, 3], 2
    wa = engine.strides(na, pia)
    nc, pic = engine.output_shape(na, q), engine.output_layout(pia, q)
    wc = engine.strides(nc, pic)
    a, b, c = torch.zeros(120), torch.zeros(5), torch.zeros(24)
    for small in ("a", "b", "c"):
        args = {"a": a, "b": b, "c": c}
        args[small] = args[small][:-1]
        with pytest.raises(engine.TTVError, match=f"buffer {small} holds"):
            engine.ttv(q, 3, args["a"], na, wa, pia, args["b"], [5], args["c"], nc, wc, pic)
    with pytest.raises(engine.TTVError, match="contraction dimension of A and B are not equal"):
        engine.ttv(q, 3, a[:1], na, wa, pia, b, [4], c, nc, wc, pic)


def test_element_misaligned_pointers_refused(engine):
    """Pointers not aligned to their element type never reach a kernel."""
    sz = engine._sizes
    meta = [sz(v) for v in ([4, 5, 6], [1, 4, 20], [1, 2, 3], [5], [4, 6], [1, 4], [1, 2])]
    L = engine.library()
    o = engine._options()
    for dt, a, b, c in ((engine.F32, 18, 32, 64), (engine.F64, 20, 32, 64), (engine.F64, 64, 36, 64),
                        (engine.F32, 64, 32, 66)):
        st = L.tlibg_ttv_ex(dt, 2, 3, a, *[engine._p(k) for k in meta[:3]], b, engine._p(meta[3]), c,
                            *[engine._p(k) for k in meta[4:]], C.byref(o), None)
        assert st == engine.ERR_UNSUPPORTED, (dt, a, b, c, st)
        assert "aligned to their element sizes" in engine._last_error()


def test_pointer_location_without_device(engine):
    """No device in this process: every pointer is a host pointer; null is unknown."""
    import ctypes
    L = engine.library()
    L.tlibg_pointer_location.argtypes = [ctypes.c_void_p]
    buf = ctypes.create_string_buffer(64)
    assert L.tlibg_pointer_location(None) == -1
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:
        assert L.tlibg_pointer_location(ctypes.addressof(buf)) == 0


def test_strided_extension_checks(engine):
    """tlibg_ttv_strided's host checks (no device needed): the reference's messages
    for shapes, layouts and monotonic strides; C strides that make two outputs
    share an element, b's zero stride and bf16 storage refused."""
    lib = engine.library()
    def call(na, wa, pia, q, nc, wc, pic, wb=1, dtype=engine.F32):
        keep = [engine._sizes(v) for v in (na, wa, pia, [na[q - 1]], nc, wc, pic)]
        st = lib.tlibg_ttv_strided(dtype, q, len(na), 16, engine._p(keep[0]), engine._p(keep[1]),
                                   engine._p(keep[2]), 32, engine._p(keep[3]), wb, 48, engine._p(keep[4]),
                                   engine._p(keep[5]), engine._p(keep[6]), None)
        return st, engine._last_error()
    # C's strides overlap (both modes stride 1)
    st, msg = call([4, 5, 6], [1, 4, 20], [1, 2, 3], 2, [4, 6], [1, 1], [1, 2])
    assert st == engine.ERR_UNSUPPORTED and "share an element" in msg
    # A's strides not monotonic along its layout: the reference's message
    st, msg = call([4, 5, 6], [20, 4, 1], [1, 2, 3], 2, [4, 6], [1, 4], [1, 2])
    assert st == engine.ERR_ARGUMENT and "stride" in msg
    # b's stride zero
    st, msg = call([4, 5, 6], [1, 4, 20], [1, 2, 3], 2, [4, 6], [1, 4], [1, 2], wb=0)
    assert st == engine.ERR_ARGUMENT and "b's stride" in msg
    # bf16-stored A is not taken here
    st, msg = call([4, 5, 6], [1, 4, 20], [1, 2, 3], 2, [4, 6], [1, 4], [1, 2], dtype=engine.BF16A)
    assert st == engine.ERR_UNSUPPORTED
    # valid padded metadata passes the host checks (then needs a device)
    st, msg = call([4, 5, 6], [1, 5, 40], [1, 2, 3], 2, [4, 6], [1, 7], [1, 2])
    assert st in (engine.ERR_CUDA, engine.ERR_ARGUMENT, engine.OK)
    if st == engine.ERR_ARGUMENT:
        assert "device-accessible" in msg
