"""Benchmark of the GB300 TTV engine (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sym|asym]

Workload (default ``sym``): the symmetric sweep -- orders p = 2..7, every
extent n = floor(2^(28/p)) (integer arithmetic: 16384, 645, 128, 48, 25, 16),
every contraction mode q, first-order and last-order layouts, fp32 and fp64:
108 TTVs of about 2^28 elements (1 GiB fp32 / 2 GiB fp64 each).  One step is
one pass over the 108 TTVs.  ``asym``: orders 2..10, n_1 = 2^(28-2(p-1)),
other extents 4, every q, first-order, fp32 (54 TTVs).

Inputs are seeded synthetic data (uniform[-1, 1]); A is larger than the
129 MB L2, so no flush is needed between steps.  value = algorithmic bytes
(bytes(A) + bytes(C) per TTV) / device time, summed over all ranks' work.

Arms:
  ours       the engine, device-resident inputs (value) and end to end
             through the host-pointer entry point with pinned host buffers
             (e2e); roofline of the dominant kernel; the CPU oracle port
             timed on a bounded sample (cpu_baseline)
  reference  the reference's algorithm for this path (par_loop / subtensor /
             all) restated in C with OpenMP (oracle port), on all host cores
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TTV HBM GB/s (% of roofline); batched TTVs/s learned vs plain @ rel err<=1e-5"
L2_BYTES = 129 * 1024 * 1024


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
def int_root(p, bits=28):
    """Largest n with n**p <= 2**bits (floor(2^(bits/p)) in integers)."""
    n = int(round(2 ** (bits / p)))
    while n ** p > 2 ** bits:
        n -= 1
    while (n + 1) ** p <= 2 ** bits:
        n += 1
    return n


def sym_cases():
    cases = []
    for dt in ("f32", "f64"):
        for p in range(2, 8):
            n = int_root(p)
            for pia in (list(range(1, p + 1)), list(range(p, 0, -1))):
                for q in range(1, p + 1):
                    cases.append({"dtype": dt, "na": [n] * p, "pia": pia, "q": q})
    return cases


def asym_cases():
    cases = []
    for p in range(2, 11):
        na = [2 ** (28 - 2 * (p - 1))] + [4] * (p - 1)
        for q in range(1, p + 1):
            cases.append({"dtype": "f32", "na": na, "pia": list(range(1, p + 1)), "q": q})
    return cases


def precision_cases():
    return [{"dtype": "f32", "na": [64, 1 << 22], "pia": [1, 2], "q": 2},
            {"dtype": "f32", "na": [16, 1 << 20, 16], "pia": [1, 2, 3], "q": 2}]


WORKLOADS = {
    "sym": (sym_cases, "symmetric sweep: p=2..7, n=floor(2^(28/p)), every q, first- and "
                       "last-order layouts, fp32+fp64 (108 TTVs of ~2^28 elements)"),
    "asym": (asym_cases, "asymmetric sweep: p=2..10, n1=2^(28-2(p-1)), n_k=4, every q, "
                         "first-order, fp32 (54 TTVs of 2^28 elements)"),
    "precision": (precision_cases, "precision and long contraction: 64x2^22 and 16x2^20x16, "
                                   "q=2, fp32"),
}


def esize(dt):
    return 8 if dt == "f64" else 4


def case_bytes(c):
    N = int(np.prod(c["na"]))
    M = N // c["na"][c["q"] - 1]
    return esize(c["dtype"]) * (N + M)


def canonical(c):
    na, pia, q = c["na"], c["pia"], c["q"]
    k = pia.index(q)
    P = int(np.prod([na[m - 1] for m in pia[:k]])) if k else 1
    S = int(np.prod([na[m - 1] for m in pia[k + 1:]])) if k + 1 < len(pia) else 1
    return P, na[q - 1], S


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_element(kernel):
    """DRAM bytes per A element of a kernel from a committed ncu summary, or None.
    profiles/dram_traffic.txt lines: kernel=<label> elements=<N> dram_bytes=<B>"""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        for ln in open(path):
            kv = dict(x.split("=", 1) for x in ln.split() if "=" in x)
            if kv.get("kernel") == kernel:
                return float(kv["dram_bytes"]) / float(kv["elements"])
    except (OSError, ValueError, KeyError):
        pass
    return None


def aggregate(ms_total, bytes_step, steps, world, dist=None, device=None):
    """Max of the timed region over ranks, and the whole-job throughput: every
    rank processed bytes_step per step (replicas, no data-path collective)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(ms_total)], dtype=torch.float64,
                         device=device if device is not None else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    return ms_total, world * bytes_step * steps / (ms_total / 1e3) / 1e9


# --------------------------------------------------------------------------
# the engine arm
# --------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch
    import ttv_gb300 as T

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    cases = WORKLOADS[args.workload][0]()
    dtypes = sorted({c["dtype"] for c in cases})
    maxN = max(int(np.prod(c["na"])) for c in cases)
    maxM = max(int(np.prod(c["na"])) // c["na"][c["q"] - 1] for c in cases)
    maxB = max(max(c["na"]) for c in cases)
    tdt = {"f32": torch.float32, "f64": torch.float64}
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    A, Bv, Cv = {}, {}, {}
    for dt in dtypes:
        A[dt] = (torch.rand(maxN, generator=g, device=dev, dtype=tdt[dt]) * 2 - 1)
        Bv[dt] = (torch.rand(maxB, generator=g, device=dev, dtype=tdt[dt]) * 2 - 1)
        Cv[dt] = torch.empty(maxM, device=dev, dtype=tdt[dt])
    lib = T.library()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    # per-case argument blocks, built once
    prepared = []
    for c in cases:
        na, pia, q = c["na"], c["pia"], c["q"]
        wa = T.strides(na, pia)
        nc, pic = T.output_shape(na, q), T.output_layout(pia, q)
        wc = T.strides(nc, pic)
        keep = [T._sizes(v) for v in (na, wa, pia, [na[q - 1]], nc, wc, pic)]
        dt = c["dtype"]
        fn = lib.tlibg_ttv_f32 if dt == "f32" else lib.tlibg_ttv_f64
        argv = (q, len(na), A[dt].data_ptr(), *[T._p(k) for k in keep[:3]], Bv[dt].data_ptr(),
                T._p(keep[3]), Cv[dt].data_ptr(), *[T._p(k) for k in keep[4:]], sh)
        pl = T.plan(q, na, pia, dtype=T.F32 if dt == "f32" else T.F64)
        fam = {T.KIND_ROW: "row_kernel", T.KIND_COL: "col_kernel",
               T.KIND_STREAM: "stream_kernel", T.KIND_COL_REALIGN: "col_realign_kernel",
               T.KIND_COL_THIN: "col_thin_kernel", T.KIND_ROW_TILE: "row_tile_kernel",
               T.KIND_COL_BULK: "col_bulk_kernel"}[pl["kind"]]
        if pl["kind"] == T.KIND_COL and pl["vec"] == 1:
            fam = "col_strided_kernel"   # scalar loads, two outputs per thread
        kname = fam + f"<{dt}" + ("" if pl["kind"] in (T.KIND_STREAM, T.KIND_ROW_TILE, T.KIND_COL_BULK) else f",V{pl['vec']}") + \
            (",kahan" if pl["accumulate"] == T.ACC_COMPENSATED and dt != "f64" else "") + ">"
        prepared.append((fn, argv, keep, case_bytes(c), kname, c))

    def one_pass(evs=None):
        for i, (fn, argv, _keep, _b, _k, _c) in enumerate(prepared):
            if evs is not None:
                evs[i][0].record(stream)
            st = fn(*argv)
            if st:
                raise RuntimeError(f"ttv failed: {T._last_error()}")
            if evs is not None:
                evs[i][1].record(stream)

    dist = None
    if world > 1:
        import torch.distributed as dist

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        one_pass()
    torch.cuda.synchronize()
    if T.device_error() != 0:
        raise RuntimeError("device error word set during warm-up")

    K = args.steps
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in prepared] for _ in range(K)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = T.launch_count()
    with ClockSampler(local_rank) as clk:
        barrier()
        torch.cuda.synchronize()
        t0.record(stream)
        for k in range(K):
            one_pass(evs[k])
        t1.record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = T.launch_count() - launches0
    bytes_step = sum(p[3] for p in prepared)
    ms_total, value = aggregate(t0.elapsed_time(t1), bytes_step, K, world, dist, dev)
    ms_step = ms_total / K

    # per-kernel breakdown from the per-case events (same timed region)
    per_kernel = {}
    per_case_ms = [0.0] * len(prepared)
    for k in range(K):
        for i, (e0, e1) in enumerate(evs[k]):
            per_case_ms[i] += e0.elapsed_time(e1) / K
    for i, (_fn, _a, _kp, nb, kname, c) in enumerate(prepared):
        d = per_kernel.setdefault(kname, {"ms": 0.0, "bytes": 0, "launches": 0, "elements": 0})
        d["ms"] += per_case_ms[i]
        d["bytes"] += nb
        d["launches"] += 1
        d["elements"] += int(np.prod(c["na"]))
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms"])
    dk = per_kernel[dom]
    peak, peak_kind = measured_peak()
    achieved = dk["bytes"] / dk["launches"] / (dk["ms"] / dk["launches"] / 1e3) / 1e9
    tpe = traffic_per_element(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s", "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": (round(tpe * dk["elements"] / dk["launches"])
                            if tpe is not None else None),
                "algorithmic_bytes_per_launch": round(dk["bytes"] / dk["launches"])}
    breakdown = {k: {"GB/s": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1),
                     "frac": round(v["bytes"] / (v["ms"] / 1e3) / 1e9 / peak, 3),
                     "share": round(v["ms"] / sum(x["ms"] for x in per_kernel.values()), 3),
                     "cases": v["launches"]} for k, v in per_kernel.items()}
    per_dtype = {}
    for i, (_fn, _a, _kp, nb, _kn, c) in enumerate(prepared):
        d = per_dtype.setdefault(c["dtype"], [0, 0.0])
        d[0] += nb
        d[1] += per_case_ms[i]
    per_dtype = {k: round(v[0] / (v[1] / 1e3) / 1e9, 1) for k, v in per_dtype.items()}
    worst = sorted(((nb / (per_case_ms[i] / 1e3) / 1e9, c) for i, (_f, _a, _k, nb, _n, c)
                    in enumerate(prepared)), key=lambda t: t[0])[:3]

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if len(dtypes) > 1 else dtypes[0], "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload][1], "ttvs_per_step": len(prepared),
                   "bytes_per_step": bytes_step, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{world} (no collective)",
                   "per_dtype_GBps": per_dtype},
        "roofline": roofline,
        "kernels": breakdown,
        "slowest_cases": [{"GB/s": round(v, 1), "na": c["na"], "pia": c["pia"], "q": c["q"],
                           "dtype": c["dtype"]} for v, c in worst],
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }

    if rank == 0 and args.detail:
        with open(args.detail, "w") as f:
            json.dump([{"na": c["na"], "pia": c["pia"], "q": c["q"], "dtype": c["dtype"],
                        "kernel": kn, "ms": per_case_ms[i],
                        "GB/s": nb / (per_case_ms[i] / 1e3) / 1e9,
                        "plan": T.plan(c["q"], c["na"], c["pia"],
                                       dtype=T.F32 if c["dtype"] == "f32" else T.F64)}
                       for i, (_f, _a, _k, nb, kn, c) in enumerate(prepared)], f, indent=0)
    if rank == 0:
        out["accuracy"] = accuracy_sample(T, torch, dev, A, Bv, Cv, prepared)
        if not args.no_e2e:
            out["e2e"] = run_e2e(T, torch, prepared, A, Bv, dtypes, args)
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = run_cpu_baseline(prepared, args)
        if not args.no_batch and args.workload != "case":
            A.clear()
            Bv.clear()
            Cv.clear()
            torch.cuda.empty_cache()
            out["batched"] = run_batched(T, torch, dev, args, n=args.batch_problems)
    return out


def run_batched(T, torch, dev, args, n=4096, seed=4096):
    """Batched configuration: 4096 uneven fp32 TTVs (orders 3-5, extents log-uniform in
    [8, 512], <= 2^22 elements each, random q and layout) per launch.  Learned-selected
    persistent CUDA-graph launch vs the fixed rule vs one plain kernel launch per problem."""
    from ttv_gb300 import batch as B
    from ttv_gb300 import costmodel as CM
    shapes = CM.random_shapes(n, seed)
    sizes = [int(np.prod(na)) for na, _, _ in shapes]
    outs = [s // na[q - 1] for s, (na, _, q) in zip(sizes, shapes)]
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    A = torch.rand(sum((s + 63) // 64 * 64 for s in sizes), generator=g, device=dev) * 2 - 1
    bvec = torch.rand(512, generator=g, device=dev) * 2 - 1
    C = torch.empty(sum((m + 63) // 64 * 64 for m in outs), device=dev)
    probs = CM.problems_from_arena([(sh, 1) for sh in shapes], A, bvec, C)
    nbytes = sum(4 * (s + m) for s, m in zip(sizes, outs))
    model = B.load_cost_model()   # committed trained weights (installs them), or None
    res = {"problems": n, "bytes_per_launch": nbytes, "model": "trained" if model is not None
           else "absent (learned mode falls back to the fixed rule)"}
    K = max(3, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(K):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K

    for name, sel in (("learned", B.SELECT_LEARNED), ("fixed_rule", B.SELECT_HEURISTIC)):
        with B.Batch(probs, select=sel) as bt:
            l0 = T.launch_count()
            ms = timed(bt.launch)
            res[name] = {"ms": round(ms, 3), "TTVs/s": round(n / ms * 1e3, 1),
                         "GB/s": round(nbytes / ms / 1e6, 1),
                         "gpu_launches_per_batch": (T.launch_count() - l0) // (K + 3)}
    ms = timed(lambda: B.ttv_percall(probs))
    res["plain_per_call"] = {"ms": round(ms, 3), "TTVs/s": round(n / ms * 1e3, 1),
                             "GB/s": round(nbytes / ms / 1e6, 1)}
    res["speedup_learned_vs_plain"] = round(res["plain_per_call"]["ms"] / res["learned"]["ms"], 3)
    res["speedup_learned_vs_fixed_rule"] = round(res["fixed_rule"]["ms"] / res["learned"]["ms"], 3)
    # accuracy of the learned launch on a sample of problems
    import oracle
    errs = []
    for pr, (na, pia, q) in list(zip(probs, shapes))[:: max(1, n // 64)]:
        P, nq, S = canonical({"na": na, "pia": pia, "q": q})
        ref, absn = oracle.truth(S, nq, P, pr.a_view.cpu().numpy(), pr.b.cpu().numpy())
        errs.append(oracle.rel_error(pr.c_view.cpu().numpy(), ref, absn))
    res["max_rel_err_fp32"] = float(max(errs))
    return res


def run_precision(args):
    """Precision and long contraction: 64 x 2^22 and 16 x 2^20 x 16 fp32, contraction over
    the long mode, A = N(0,1) * 10^U(-3,3), b = U[-1,1]; fp32 compensated (default),
    fp32 plain accumulation, bf16-stored A; error vs the oracle's fp64 truth and GB/s."""
    import torch
    import oracle
    import ttv_gb300 as T
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(5)
    problems = [([64, 1 << 22], [1, 2], 2), ([16, 1 << 20, 16], [1, 2, 3], 2)]
    res = {}
    tot = {"compensated": [0, 0.0], "plain": [0, 0.0], "bf16a": [0, 0.0]}
    K = max(3, args.steps)
    for na, pia, q in problems:
        N = int(np.prod(na))
        a = (rng.standard_normal(N) * 10.0 ** rng.uniform(-3, 3, N)).astype(np.float32)
        b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
        P, nq, S = canonical({"na": na, "pia": pia, "q": q})
        ref, absn = oracle.truth(S, nq, P, a, b)
        wa = T.strides(na, pia)
        nc, pic = T.output_shape(na, q), T.output_layout(pia, q)
        wc = T.strides(nc, pic)
        da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        dab = torch.from_numpy(a).to(torch.bfloat16).to(dev).view(torch.int16)
        dc = torch.empty(int(np.prod(nc)), device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        key = "x".join(str(n) for n in na)
        res[key] = {}
        for name, A_, dt, acc, nbytes in (("compensated", da, T.F32, T.ACC_COMPENSATED, 4 * N),
                                          ("plain", da, T.F32, T.ACC_PLAIN, 4 * N),
                                          ("bf16a", dab, T.BF16A, T.ACC_COMPENSATED, 2 * N)):
            def call():
                T.ttv(q, len(na), A_, na, wa, pia, db, [nq], dc, nc, wc, pic, dtype=dt,
                      accumulate=acc)
            for _ in range(3):
                call()
            torch.cuda.synchronize()
            e0.record()
            for _ in range(K):
                call()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / K
            algo = nbytes + 4 * int(np.prod(nc))
            err = oracle.rel_error(dc.cpu().numpy(), ref, absn)
            res[key][name] = {"max_rel_err": err, "GB/s": round(algo / ms / 1e6, 1),
                              "ms": round(ms, 4)}
            tot[name][0] += algo
            tot[name][1] += ms
    gbs = {k: round(v[0] / v[1] / 1e6, 1) for k, v in tot.items()}
    peak, _ = measured_peak()
    return {"metric": METRIC, "value": gbs["compensated"], "unit": "GB/s", "n_gpus": 1,
            "steps": K, "warmup": 3, "ms_per_step": round(tot["compensated"][1], 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "precision and long contraction: 64x2^22 (q=2) and "
                                   "16x2^20x16 (q=2), A = N(0,1)*10^U(-3,3), b = U[-1,1]",
                       "l2": "inputs larger than L2 (no flush)"},
            "roofline": {"bound": "hbm", "achieved": gbs["compensated"], "peak": peak,
                         "unit": "GB/s", "frac": round(gbs["compensated"] / peak, 4)},
            "variants_GBps": gbs, "precision": res,
            "bars": {"fp32": 1e-5, "bf16a": "2e-3 vs the fp32 A (rounding of A: 2^-8 per element)"}}


def accuracy_sample(T, torch, dev, A, Bv, Cv, prepared):
    """max rel error vs the oracle's fp64 truth on one case per order (fp32)."""
    import oracle
    errs = []
    seen = set()
    for fn, argv, keep, nb, kname, c in prepared:
        key = (len(c["na"]), c["dtype"])
        if c["dtype"] != "f32" or key in seen:
            continue
        seen.add(key)
        st = fn(*argv)
        assert st == 0
        torch.cuda.synchronize()
        P, nq, S = canonical(c)
        N = P * nq * S
        a = A["f32"][:N].cpu().numpy()
        b = Bv["f32"][:nq].cpu().numpy()
        ref, absn = oracle.truth(S, nq, P, a, b)
        errs.append(oracle.rel_error(Cv["f32"][:S * P].cpu().numpy(), ref, absn))
    return {"max_rel_err_fp32": float(max(errs)) if errs else None,
            "cases": len(errs), "metric": "max|c-ref|/sum|a*b| vs fp64 oracle"}


def run_e2e(T, torch, prepared, A, Bv, dtypes, args):
    """Same sweep through the host-pointer C ABI entry point, pinned buffers."""
    lib = T.library()
    host = {}
    for dt in dtypes:
        host[dt] = (A[dt].cpu().pin_memory(), Bv[dt].cpu().pin_memory(),
                    torch.empty(max(int(np.prod(c["na"])) // c["na"][c["q"] - 1]
                                    for *_x, c in prepared), dtype=A[dt].dtype).pin_memory())
    o = T._options()
    steps = max(1, args.e2e_steps)

    def one(fn_argv):
        _fn, argv, keep, nb, kname, c = fn_argv
        ha, hb, hc = host[c["dtype"]]
        dtc = T.F32 if c["dtype"] == "f32" else T.F64
        q, p = argv[0], argv[1]
        st = lib.tlibg_ttv_host(dtc, q, p, ha.data_ptr(), T._p(keep[0]), T._p(keep[1]),
                                T._p(keep[2]), hb.data_ptr(), T._p(keep[3]), hc.data_ptr(),
                                T._p(keep[4]), T._p(keep[5]), T._p(keep[6]), T.C.byref(o))
        if st:
            raise RuntimeError(f"ttv_host failed: {T._last_error()}")

    for x in prepared[:3]:
        one(x)
    t = time.perf_counter()
    for _ in range(steps):
        for x in prepared:
            one(x)
    dt_s = time.perf_counter() - t
    nbytes = sum(x[3] for x in prepared)
    h2d = sum(esize(c["dtype"]) * (int(np.prod(c["na"])) + c["na"][c["q"] - 1])
              for *_x, c in prepared)
    d2h = sum(esize(c["dtype"]) * (int(np.prod(c["na"])) // c["na"][c["q"] - 1])
              for *_x, c in prepared)
    return {"value": round(nbytes * steps / dt_s / 1e9, 1), "unit": "GB/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps,
            "api": "tlibg_ttv_host (host pointers, pinned)"}


def cpu_inputs(cases, seed=99):
    rng = np.random.default_rng(seed)
    maxN = max(int(np.prod(c["na"])) for c in cases)
    maxB = max(max(c["na"]) for c in cases)
    data = {}
    for dt in sorted({c["dtype"] for c in cases}):
        npdt = np.float32 if dt == "f32" else np.float64
        a = rng.random(maxN, dtype=npdt)
        a *= 2
        a -= 1
        data[dt] = (a, (rng.random(maxB, dtype=npdt) * 2 - 1).astype(npdt))
    return data


def run_cpu_sweep(cases, data, passes):
    import oracle
    t = time.perf_counter()
    nbytes = 0
    for _ in range(passes):
        for c in cases:
            P, nq, S = canonical(c)
            a, b = data[c["dtype"]]
            oracle.canon(S, nq, P, a[:P * nq * S], b[:nq])
            nbytes += case_bytes(c)
    return nbytes / (time.perf_counter() - t) / 1e9


def run_cpu_baseline(prepared, args):
    """The oracle port (reference algorithm, OpenMP) on a bounded sample."""
    import oracle
    cases = [x[5] for x in prepared]
    sample = cases[::max(1, len(cases) // 36)]
    data = cpu_inputs(sample)
    v = run_cpu_sweep(sample, data, 1)
    return {"value": round(v, 2), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{len(sample)} of the {len(cases)} TTVs of the sweep (every "
                      f"{max(1, len(cases) // 36)}th), one pass, oracle/ttv_oracle.c "
                      "orc_canon (reference par_loop/subtensor/all loops, OpenMP)"}


# --------------------------------------------------------------------------
# the reference arm
# --------------------------------------------------------------------------
def run_reference(args):
    import oracle
    oracle.build(with_ref=False) if not os.path.exists(oracle.LIB_PATH) else None
    cases = WORKLOADS[args.workload][0]()
    # bounded per-step sample of the workload: every 3rd TTV of the sweep
    sample = cases[::3] if len(cases) > 6 else cases
    data = cpu_inputs(sample)
    for _ in range(args.warmup):
        run_cpu_sweep(sample[:2], data, 1)
    # the reference itself (compiled from its own headers by oracle/Makefile) where it
    # exists on this host, else the C restatement of its algorithm
    use_ref = False
    try:
        use_ref = oracle.ref_available() and oracle.ref() is not None
    except OSError:
        use_ref = False
    calls = []
    for c in sample:
        P, nq, S = canonical(c)
        a, b = data[c["dtype"]]
        na, pia, q = c["na"], c["pia"], c["q"]
        nc, pic = oracle.output_shape(na, q), oracle.output_layout(pia, q)
        meta = (q, a[:P * nq * S], na, oracle.strides(na, pia), pia, b[:nq], [nq], nc,
                oracle.strides(nc, pic), pic, np.zeros(P * S, dtype=a.dtype))
        calls.append((c, P, nq, S, a, b, meta))
    t = time.perf_counter()
    nbytes = 0
    for _ in range(args.steps):
        for c, P, nq, S, a, b, meta in calls:
            if use_ref:
                q, av, na, wa, pia, bv, nb, nc, wc, pic, cv = meta
                st, msg, _ = oracle.ref_ttv("par_loop/subtensor/all", q, av, na, wa, pia, bv, nb, nc,
                                            wc, pic, c=cv)
                if st:
                    raise RuntimeError(msg)
            else:
                oracle.canon(S, nq, P, a[:P * nq * S], b[:nq])
            nbytes += case_bytes(c)
    el = time.perf_counter() - t
    v = nbytes / el / 1e9
    cores = oracle.num_threads()
    if use_ref:
        kind, what = "reference", ("the reference's own par_loop/subtensor/all (its headers compiled "
                                   "by oracle/Makefile into oracle/_ref), OpenMP on all host cores")
    else:
        kind, what = "port", ("the reference's par_loop/subtensor/all algorithm restated in C "
                              "(oracle/ttv_oracle.c orc_canon), OpenMP on all host cores; the "
                              "reference itself is not built on this host (its sources are absent)")
    return {"metric": METRIC, "value": round(v, 2), "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(el / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.workload == "sym" else "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload][1],
                       "sample_per_step": f"{len(sample)} of {len(cases)} TTVs (every 3rd)"},
            "cpu_baseline": {"value": round(v, 2), "unit": "GB/s", "cores": cores,
                             "kind": kind, "sample": f"{len(sample)} TTVs per step: {what}"},
            "e2e": {"value": round(v, 2), "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def parse_case(spec):
    """'na=645,645,128 pia=1,2,3 q=2 dtype=f32' -> a one-TTV workload."""
    kv = dict(x.split("=", 1) for x in spec.split())
    c = {"na": [int(x) for x in kv["na"].split(",")], "q": int(kv["q"]),
         "dtype": kv.get("dtype", "f32")}
    c["pia"] = [int(x) for x in kv["pia"].split(",")] if "pia" in kv else \
        list(range(1, len(c["na"]) + 1))
    return c


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch"], default="sym")
    ap.add_argument("--batch-problems", type=int, default=4096,
                    help="problems per launch of the batched configuration")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--detail", default=None, help="write per-TTV timings and plans (JSON)")
    ap.add_argument("--case", default=None,
                    help="one TTV instead of a sweep, e.g. 'na=645,645,128 pia=1,2,3 q=2 "
                         "dtype=f32' (profiling)")
    args = ap.parse_args()
    if args.case:
        case = parse_case(args.case)
        WORKLOADS["case"] = (lambda: [case], f"single TTV {args.case}")
        args.workload = "case"
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return

    if args.workload == "precision":
        if rank == 0:
            print(json.dumps(run_precision(args)), flush=True)
        return
    if args.workload == "batch":
        # the batched configuration alone (profiling; --batch-problems sets its size)
        if rank == 0:
            import torch
            import ttv_gb300 as T
            dev = torch.device("cuda", 0)
            print(json.dumps(run_batched(T, torch, dev, args, n=args.batch_problems)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    out = run_ours(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
