"""Benchmark of the GB300 TTV engine (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sym|asym|precision|batch]

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
             (e2e); roofline of the dominant kernel; accuracy against the
             oracle's fp64 truth (fp32 and fp64); the asymmetric sweep,
             the precision configuration and the batched configuration as
             sub-objects; the reference on the host cores (cpu_baseline)
  reference  the reference's own par_loop / subtensor / all path on the
             host cores, compiled from its headers with OpenBLAS
             (oracle/_ref/libttvref_blas.so), on the same TTVs
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
def kernel_label(T, c):
    """Kernel family and template of the plan a case runs (for the breakdown)."""
    dt = c["dtype"]
    pl = T.plan(c["q"], c["na"], c["pia"], dtype=T.F32 if dt == "f32" else T.F64)
    fam = {T.KIND_ROW: "row_kernel", T.KIND_COL: "col_kernel",
           T.KIND_STREAM: "stream_kernel", T.KIND_COL_REALIGN: "col_realign_kernel",
           T.KIND_COL_THIN: "col_thin_kernel", T.KIND_ROW_TILE: "row_tile_kernel",
           T.KIND_COL_BULK: "col_bulk_kernel", T.KIND_ROW_PANEL: "row_panel_kernel",
           T.KIND_ROW_SHIFT: "row_shift_kernel"}[pl["kind"]]
    if pl["kind"] == T.KIND_COL and pl["vec"] == 1:
        fam = "col_strided_kernel"   # scalar loads, two outputs per thread
    templ = "" if pl["kind"] in (T.KIND_STREAM, T.KIND_ROW_TILE, T.KIND_COL_BULK) else f",V{pl['vec']}"
    if pl["kind"] == T.KIND_ROW_PANEL:
        templ += f",R{pl['group']}"
    acc = ",kahan" if pl["accumulate"] == T.ACC_COMPENSATED and dt != "f64" else ""
    return f"{fam}<{dt}{templ}{acc}>" + ("+combine" if pl["split"] > 1 else "")


def prepare_sweep(T, torch, dev, cases, seed):
    """Device inputs (one A, b and C per dtype, sized for the largest case) and
    the C-ABI argument block of every case, built once."""
    dtypes = sorted({c["dtype"] for c in cases})
    maxN = max(int(np.prod(c["na"])) for c in cases)
    maxM = max(int(np.prod(c["na"])) // c["na"][c["q"] - 1] for c in cases)
    maxB = max(max(c["na"]) for c in cases)
    tdt = {"f32": torch.float32, "f64": torch.float64}
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    A, Bv, Cv = {}, {}, {}
    for dt in dtypes:
        A[dt] = (torch.rand(maxN, generator=g, device=dev, dtype=tdt[dt]) * 2 - 1)
        Bv[dt] = (torch.rand(maxB, generator=g, device=dev, dtype=tdt[dt]) * 2 - 1)
        Cv[dt] = torch.empty(maxM, device=dev, dtype=tdt[dt])
    lib = T.library()
    sh = torch.cuda.current_stream(dev).cuda_stream
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
        prepared.append((fn, argv, keep, case_bytes(c), kernel_label(T, c), c))
    return {"A": A, "B": Bv, "C": Cv, "prepared": prepared, "dtypes": dtypes}


def one_pass(T, prepared, stream, evs=None):
    for i, (fn, argv, _keep, _b, _k, _c) in enumerate(prepared):
        if evs is not None:
            evs[i][0].record(stream)
        st = fn(*argv)
        if st:
            raise RuntimeError(f"ttv failed: {T._last_error()}")
        if evs is not None:
            evs[i][1].record(stream)


def kernel_breakdown(prepared, per_case_ms, peak):
    per_kernel = {}
    for i, (_fn, _a, _kp, nb, kname, c) in enumerate(prepared):
        d = per_kernel.setdefault(kname, {"ms": 0.0, "bytes": 0, "launches": 0, "elements": 0})
        d["ms"] += per_case_ms[i]
        d["bytes"] += nb
        d["launches"] += 1
        d["elements"] += int(np.prod(c["na"]))
    tot = sum(x["ms"] for x in per_kernel.values())
    breakdown = {k: {"GB/s": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1),
                     "frac": round(v["bytes"] / (v["ms"] / 1e3) / 1e9 / peak, 3),
                     "share": round(v["ms"] / tot, 3), "cases": v["launches"]}
                 for k, v in per_kernel.items()}
    return per_kernel, breakdown


def run_ours(args, rank, world, local_rank):
    import torch
    import ttv_gb300 as T

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    cases = WORKLOADS[args.workload][0]()
    sw = prepare_sweep(T, torch, dev, cases, 1234 + rank)
    A, Bv, Cv, prepared, dtypes = sw["A"], sw["B"], sw["C"], sw["prepared"], sw["dtypes"]
    stream = torch.cuda.current_stream(dev)

    dist = None
    if world > 1:
        import torch.distributed as dist

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        one_pass(T, prepared, stream)
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
            one_pass(T, prepared, stream, evs[k])
        t1.record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = T.launch_count() - launches0
    bytes_step = sum(p[3] for p in prepared)
    ms_total, value = aggregate(t0.elapsed_time(t1), bytes_step, K, world, dist, dev)
    ms_step = ms_total / K

    # per-kernel breakdown from the per-case events (same timed region)
    per_case_ms = [0.0] * len(prepared)
    for k in range(K):
        for i, (e0, e1) in enumerate(evs[k]):
            per_case_ms[i] += e0.elapsed_time(e1) / K
    peak, peak_kind = measured_peak()
    per_kernel, breakdown = kernel_breakdown(prepared, per_case_ms, peak)
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms"])
    dk = per_kernel[dom]
    achieved = dk["bytes"] / dk["launches"] / (dk["ms"] / dk["launches"] / 1e3) / 1e9
    tr = traffic_per_launch(dom, dk["elements"] / dk["launches"])
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s", "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": tr[0] if tr else None,
                "traffic_source": tr[1] if tr else None,
                "algorithmic_bytes_per_launch": round(dk["bytes"] / dk["launches"])}
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
        out["accuracy"] = accuracy_sample(T, torch, sw)
        if not args.no_e2e:
            out["e2e"] = run_e2e(T, torch, sw, args)
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = run_cpu_baseline(cases, args)
        A.clear()
        Bv.clear()
        Cv.clear()
        sw.clear()
        torch.cuda.empty_cache()
        if args.workload == "sym" and not args.no_sub:
            out["asym"] = run_sweep_sub(T, torch, dev, "asym", args)
            torch.cuda.empty_cache()
            out["precision"] = run_precision_sub(T, torch, dev, args)
            torch.cuda.empty_cache()
            out["ttvs"] = run_ttvs_sub(T, torch, dev, args)
            torch.cuda.empty_cache()
        if not args.no_batch and args.workload != "case":
            out["batched"] = run_batched(T, torch, dev, args, n=args.batch_problems)
    return out


def run_sweep_sub(T, torch, dev, workload, args):
    """Another sweep as a sub-object of the line: GB/s over the sweep, the
    fraction of the measured peak, per-kernel shares and the oracle error on
    one case per order."""
    cases = WORKLOADS[workload][0]()
    sw = prepare_sweep(T, torch, dev, cases, 4321)
    prepared = sw["prepared"]
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        one_pass(T, prepared, stream)
    torch.cuda.synchronize()
    K = max(3, min(args.steps, 10))
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in prepared] for _ in range(K)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(K):
        one_pass(T, prepared, stream, evs[k])
    t1.record(stream)
    torch.cuda.synchronize()
    if T.device_error() != 0:
        raise RuntimeError(f"device error word set during the {workload} sweep")
    bytes_step = sum(p[3] for p in prepared)
    ms = t0.elapsed_time(t1) / K
    per_case_ms = [sum(evs[k][i][0].elapsed_time(evs[k][i][1]) for k in range(K)) / K
                   for i in range(len(prepared))]
    peak, _ = measured_peak()
    _per_kernel, breakdown = kernel_breakdown(prepared, per_case_ms, peak)
    gbs = bytes_step / (ms / 1e3) / 1e9
    worst = sorted(((nb / (per_case_ms[i] / 1e3) / 1e9, c) for i, (_f, _a, _k, nb, _n, c)
                    in enumerate(prepared)), key=lambda t: t[0])[:3]
    q1 = {}
    for i, (_f, _a, _k, nb, _n, c) in enumerate(prepared):
        if c["q"] == 1 and len(c["na"]) <= 4:
            q1["x".join(str(n) for n in c["na"])] = round(nb / (per_case_ms[i] / 1e3) / 1e9, 1)
    acc = accuracy_sample(T, torch, sw, per_order=True)
    res = {"workload": WORKLOADS[workload][1], "ttvs": len(prepared), "bytes_per_pass": bytes_step,
           "ms_per_pass": round(ms, 3), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4),
           "passes": K, "kernels": breakdown, "q1_long_rows_GBps": q1,
           "slowest_cases": [{"GB/s": round(v, 1), "na": c["na"], "q": c["q"]} for v, c in worst],
           "accuracy": acc}
    sw.clear()
    return res


def run_precision_sub(T, torch, dev, args):
    """The precision configuration as a sub-object (see run_precision)."""
    full = run_precision(args)
    return {"workload": full["config"]["workload"], "variants_GBps": full["variants_GBps"],
            "frac_compensated": full["roofline"]["frac"], "errors": full["precision"],
            "bars": full["bars"]}


def run_ttvs_sub(T, torch, dev, args, na=(128, 128, 128, 128)):
    """The multi-vector chain (ttvpy.ttvs) on an order-4 fp32 tensor of 2^28
    elements, every q: the fused chain (A read once) against the first TTV of
    the reference's optimal order alone (the largest vector's mode, which
    reads A once too) and the step-by-step chain; error vs the oracle."""
    import oracle
    na = list(na)
    g = torch.Generator(device=dev)
    g.manual_seed(28)
    A = (torch.rand(int(np.prod(na)), generator=g, device=dev) * 2 - 1).view(*na)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    K = max(3, min(args.steps, 10))

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

    res, tot = {}, {"fused": 0.0, "first_ttv": 0.0, "step_by_step": 0.0}
    nbytes = 0
    for q in range(1, 5):
        bs = [torch.rand(na[m], generator=g, device=dev) * 2 - 1 for m in range(4) if m != q - 1]
        first_mode = max((m for m in range(1, 5) if m != q), key=lambda m: (na[m - 1], m))
        bfirst = bs[first_mode - 1 if first_mode < q else first_mode - 2]
        c1 = torch.empty([n for i, n in enumerate(na) if i != first_mode - 1], device=dev)
        ms_f = timed(lambda: T.ttvs(q, A, bs))
        ms_1 = timed(lambda: T.ttv_array(first_mode, A, bfirst, out=c1))
        ms_s = timed(lambda: T.ttvs(q, A, bs, fused=False))
        c = T.ttvs(q, A, bs).cpu().numpy()
        ref, absn = oracle.ttvs_truth(q, A.view(-1).cpu().numpy(), na, [4, 3, 2, 1],
                                      [b.cpu().numpy() for b in bs])
        b_chain = 4 * (A.numel() + na[q - 1])
        b_first = 4 * (A.numel() + c1.numel())
        res[f"q{q}"] = {"fused_GBps": round(b_chain / ms_f / 1e6, 1),
                        "first_ttv_GBps": round(b_first / ms_1 / 1e6, 1),
                        "fused_ms": round(ms_f, 4), "first_ttv_ms": round(ms_1, 4),
                        "step_by_step_ms": round(ms_s, 4),
                        "max_rel_err": oracle.rel_error(c, ref, absn)}
        tot["fused"] += ms_f
        tot["first_ttv"] += ms_1
        tot["step_by_step"] += ms_s
        nbytes += b_chain
    return {"workload": "ttvs (every mode but q) on a 128^4 fp32 tensor (2^28 elements), "
                        "q = 1..4, last-order layout",
            "fused_GBps": round(nbytes / tot["fused"] / 1e6, 1),
            "fused_over_first_ttv_time": round(tot["fused"] / tot["first_ttv"], 4),
            "step_by_step_over_fused_time": round(tot["step_by_step"] / tot["fused"], 3),
            "per_q": res, "bar": 1e-5}


def traffic_per_launch(kernel, elements):
    """DRAM bytes of one launch of a kernel from a committed ncu summary, or None.
    profiles/dram_traffic.txt lines: kernel=<label> elements=<N> dram_bytes=<B>
    [note=...]; a capture of the exact case (same element count) is taken as is,
    another case is scaled by the elements of A."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    best = None
    try:
        for ln in open(path):
            kv = dict(x.split("=", 1) for x in ln.split() if "=" in x)
            if kv.get("kernel") != kernel.split("+")[0]:
                continue
            n, byts = float(kv["elements"]), float(kv["dram_bytes"])
            if abs(n - elements) < 0.5:
                return round(byts), f"ncu capture of a sweep launch ({int(n)} elements)"
            best = (round(byts / n * elements),
                    f"ncu capture of {int(n)} elements scaled to {int(elements)}")
    except (OSError, ValueError, KeyError):
        pass
    return best
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
    peak, _ = measured_peak()

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
                         "frac": round(nbytes / ms / 1e6 / peak, 4),
                         "gpu_launches_per_batch": (T.launch_count() - l0) // (K + 3)}
            if name == "learned":
                res[name]["variants_used"] = {str(k): v for k, v in sorted(
                    __import__("collections").Counter(bt.variants()).items())}
    ms = timed(lambda: B.ttv_percall(probs))
    res["plain_per_call"] = {"ms": round(ms, 3), "TTVs/s": round(n / ms * 1e3, 1),
                             "GB/s": round(nbytes / ms / 1e6, 1)}
    res["speedup_learned_vs_plain"] = round(res["plain_per_call"]["ms"] / res["learned"]["ms"], 3)
    res["speedup_learned_vs_fixed_rule"] = round(res["fixed_rule"]["ms"] / res["learned"]["ms"], 3)
    l2x = nbytes / (129 << 20)
    res["l2"] = (f"{nbytes / 1e9:.2f} GB of A and C per launch, {l2x:.0f}x L2: consecutive launches "
                 "find no problem resident (no flush)" if l2x >= 4 else
                 f"{nbytes / 1e9:.2f} GB per launch, {l2x:.1f}x L2: part of the previous launch may "
                 "still be resident (no flush; a profiling-size case)")
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
    dev = torch.device("cuda", torch.cuda.current_device())
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


def accuracy_cases(prepared, per_order=False):
    """Indices of the cases checked against the oracle: one per (order, dtype,
    layout), q rotating with the order so every kernel family is visited
    (per_order: one per order)."""
    picked, seen = [], set()
    for i, (_fn, _argv, _keep, _nb, _kname, c) in enumerate(prepared):
        p = len(c["na"])
        lay = 0 if c["pia"][0] == 1 else 1
        key = (p,) if per_order else (p, c["dtype"], lay)
        if per_order:   # even orders: q = 1 (the long rows), odd: the middle mode
            want_q = 1 if p % 2 == 0 else p // 2 + 1
        else:           # first, last and middle modes over the orders and layouts
            want_q = (2 * (p - 2) + lay) % p + 1
        if key in seen or c["q"] != want_q:
            continue
        seen.add(key)
        picked.append(i)
    return picked


def accuracy_sample(T, torch, sw, per_order=False):
    """max rel error vs the oracle's fp64 truth (fp32 and fp64 separately)."""
    import oracle
    prepared, A, Bv, Cv = sw["prepared"], sw["A"], sw["B"], sw["C"]
    errs = {}
    idx = accuracy_cases(prepared, per_order)
    host = {dt: A[dt].cpu().numpy() for dt in A}
    hostb = {dt: Bv[dt].cpu().numpy() for dt in Bv}
    for i in idx:
        fn, argv, keep, nb, kname, c = prepared[i]
        Cv[c["dtype"]].fill_(float("nan"))
        st = fn(*argv)
        assert st == 0, T._last_error()
        torch.cuda.synchronize()
        P, nq, S = canonical(c)
        N = P * nq * S
        ref, absn = oracle.truth(S, nq, P, host[c["dtype"]][:N], hostb[c["dtype"]][:nq])
        err = oracle.rel_error(Cv[c["dtype"]][:S * P].cpu().numpy(), ref, absn)
        errs.setdefault(c["dtype"], []).append(err)
    out = {f"max_rel_err_fp{dt[1:]}": float(max(v)) for dt, v in errs.items()}
    out.update({"cases": len(idx), "cases_per_dtype": {dt: len(v) for dt, v in errs.items()},
                "bars": {"fp32": 1e-5, "fp64": 1e-13},
                "metric": "max|c-ref|/sum|a*b| vs the oracle's double-double truth"})
    return out


def link_peak(torch, nbytes=1 << 30):
    """Pinned host <-> device copy bandwidth of this machine (GB/s), one copy engine
    per direction, best of 3."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h", lambda: h.copy_(d, non_blocking=True))):
        best = None
        for _ in range(3):
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = round(nbytes / best / 1e6, 1)
    del h, d
    return out


def run_e2e(T, torch, sw, args):
    """Same sweep through the host-pointer C ABI entry point, pinned buffers,
    timed over --e2e-steps passes; the host link's own copy bandwidth beside it."""
    lib = T.library()
    prepared, A, Bv = sw["prepared"], sw["A"], sw["B"]
    host = {}
    for dt in sw["dtypes"]:
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

    for x in prepared:   # one untimed pass: the host path's staging buffers reach their size
        one(x)
    per_case = [0.0] * len(prepared)
    t = time.perf_counter()
    for _ in range(steps):
        for i, x in enumerate(prepared):
            t0 = time.perf_counter()
            one(x)   # synchronous: returns after the kernels and C are done
            per_case[i] += time.perf_counter() - t0
    dt_s = time.perf_counter() - t
    by_kernel = {}
    for i, (_f, _a, _k, nb, kname, _c) in enumerate(prepared):
        d = by_kernel.setdefault(kname, [0, 0.0])
        d[0] += nb * steps
        d[1] += per_case[i]
    worst = sorted(((x[3] * steps / per_case[i] / 1e9, x[5]) for i, x in enumerate(prepared)),
                   key=lambda t_: t_[0])[:3]
    nbytes = sum(x[3] for x in prepared)
    h2d = sum(esize(c["dtype"]) * (int(np.prod(c["na"])) + c["na"][c["q"] - 1])
              for *_x, c in prepared)
    d2h = sum(esize(c["dtype"]) * (int(np.prod(c["na"])) // c["na"][c["q"] - 1])
              for *_x, c in prepared)
    host.clear()
    link = link_peak(torch)
    v = nbytes * steps / dt_s / 1e9
    return {"value": round(v, 1), "unit": "GB/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps,
            "api": "tlibg_ttv_host (host pointers, pinned)",
            "link_GBps": link, "frac_of_link_h2d": round(v / link["h2d"], 3),
            "by_kernel_GBps": {k: round(d[0] / d[1] / 1e9, 1) for k, d in by_kernel.items()},
            "slowest_cases": [{"GB/s": round(g, 1), "na": c["na"], "pia": c["pia"], "q": c["q"],
                               "dtype": c["dtype"]} for g, c in worst]}


# --------------------------------------------------------------------------
# the reference on the host cores (cpu_baseline and the reference arm)
# --------------------------------------------------------------------------
def cpu_inputs(cases, seed=99):
    rng = np.random.default_rng(seed)
    maxN = max(int(np.prod(c["na"])) for c in cases)
    maxB = max(max(c["na"]) for c in cases)
    maxM = max(int(np.prod(c["na"])) // c["na"][c["q"] - 1] for c in cases)
    data = {}
    for dt in sorted({c["dtype"] for c in cases}):
        npdt = np.float32 if dt == "f32" else np.float64
        a = rng.random(maxN, dtype=npdt)
        a *= 2
        a -= 1
        data[dt] = (a, (rng.random(maxB, dtype=npdt) * 2 - 1).astype(npdt),
                    np.zeros(maxM, dtype=npdt))
    return data


def host_info():
    info = {"nproc": os.cpu_count(), "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "CPU part", "CPU implementer"):
            for ln in txt.splitlines():
                if ln.startswith(key):
                    info[key.replace(" ", "_")] = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            k = ln.split(":", 1)[0].strip()
            if k in ("Model name", "Socket(s)", "Core(s) per socket", "Thread(s) per core"):
                info[k] = ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


class CpuReference:
    """The reference's par_loop / subtensor / all call on the host cores: its
    OpenBLAS build (the configured path) where one was linked, else its plain
    build, else the oracle's C restatement (only if neither exists)."""

    def __init__(self):
        import oracle
        self.O = oracle
        if not os.path.exists(oracle.LIB_PATH) or not (oracle.ref_available() or
                                                       oracle.ref_blas_available()):
            try:
                oracle.build()
            except (OSError, subprocess.CalledProcessError):
                oracle.build(with_ref=False)
        if oracle.ref_blas_available():
            self.kind, self.blas = "reference", True
            self.what = ("the reference's own par_loop/subtensor/all (its headers compiled by "
                         "oracle/Makefile with -DUSE_OPENBLAS into oracle/_ref/libttvref_blas.so, "
                         f"BLAS {oracle.blas_info()}), OpenMP + OpenBLAS threads on all host cores")
        elif oracle.ref_available():
            self.kind, self.blas = "reference", False
            self.what = ("the reference's own par_loop/subtensor/all without BLAS (no OpenBLAS on "
                         "this host: its cases 2-7 run its serial gemv loops), OpenMP on all host "
                         "cores")
        else:
            self.kind, self.blas = "port", None
            self.what = ("the reference's par_loop/subtensor/all algorithm restated in C "
                         "(oracle/ttv_oracle.c orc_canon, a restructured port), OpenMP on all host "
                         "cores; the reference headers are absent on this host")
        self.cores = oracle.num_threads()

    def calls(self, cases, data):
        O = self.O
        out = []
        for c in cases:
            P, nq, S = canonical(c)
            a, b, cbuf = data[c["dtype"]]
            na, pia, q = c["na"], c["pia"], c["q"]
            nc, pic = O.output_shape(na, q), O.output_layout(pia, q)
            out.append((c, P, nq, S, (q, a[:P * nq * S], na, O.strides(na, pia), pia, b[:nq], [nq],
                                      nc, O.strides(nc, pic), pic, cbuf[:P * S])))
        return out

    def run(self, call):
        c, P, nq, S, meta = call
        q, av, na, wa, pia, bv, nb, nc, wc, pic, cv = meta
        if self.blas is None:
            cv[:] = self.O.canon(S, nq, P, av, bv)
            return
        st, msg, _ = self.O.ref_ttv("par_loop/subtensor/all", q, av, na, wa, pia, bv, nb, nc, wc,
                                    pic, c=cv, blas=self.blas)
        if st:
            raise RuntimeError(msg)

    def check(self, call):
        """Error of one result against the oracle's truth (the timed build is correct)."""
        c, P, nq, S, meta = call
        self.run(call)
        ref, absn = self.O.truth(S, nq, P, meta[1], meta[5])
        return self.O.rel_error(meta[10], ref, absn)


def run_cpu_pass(ref, calls):
    t = time.perf_counter()
    nbytes = 0
    for call in calls:
        ref.run(call)
        nbytes += case_bytes(call[0])
    return nbytes, time.perf_counter() - t


def run_cpu_baseline(cases, args):
    """The reference on the host cores, one pass over the same TTVs as the GPU step."""
    ref = CpuReference()
    data = cpu_inputs(cases)
    calls = ref.calls(cases, data)
    err = ref.check(calls[len(calls) // 2])
    nbytes, el = run_cpu_pass(ref, calls)
    return {"value": round(nbytes / el / 1e9, 2), "unit": "GB/s", "cores": ref.cores,
            "kind": ref.kind, "sample": f"all {len(cases)} TTVs of the step, one pass: {ref.what}",
            "s_per_pass": round(el, 3), "max_rel_err_checked_case": err, "host": host_info()}


# --------------------------------------------------------------------------
# the reference arm
# --------------------------------------------------------------------------
def run_reference(args):
    cases = WORKLOADS[args.workload][0]()
    ref = CpuReference()
    data = cpu_inputs(cases)
    calls = ref.calls(cases, data)
    err = ref.check(calls[len(calls) // 2])
    # warm-up passes; a pass that would make the run take more than a few minutes
    # is cut to a regular sample of the TTVs (every k-th), and the line says so
    sample = calls
    for w in range(max(1, args.warmup)):
        nb, el = run_cpu_pass(ref, sample)
        if w == 0 and el * (args.steps + args.warmup) > 240 and len(sample) > 6:
            k = int(np.ceil(el * (args.steps + args.warmup) / 240))
            sample = calls[::k]
    t = time.perf_counter()
    nbytes = 0
    for _ in range(args.steps):
        nb, _el = run_cpu_pass(ref, sample)
        nbytes += nb
    el = time.perf_counter() - t
    v = nbytes / el / 1e9
    same = len(sample) == len(calls)
    return {"metric": METRIC, "value": round(v, 2), "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(el / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.workload == "sym" else "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload][1],
                       "sample_per_step": (f"all {len(cases)} TTVs" if same else
                                           f"{len(sample)} of {len(cases)} TTVs (regular sample)"),
                       "same_ttvs_as_gpu_step": same},
            "cpu_baseline": {"value": round(v, 2), "unit": "GB/s", "cores": ref.cores,
                             "kind": ref.kind, "sample": f"{len(sample)} TTVs per step: {ref.what}",
                             "max_rel_err_checked_case": err, "host": host_info()},
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
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the asymmetric and precision sub-objects of the default line")
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
