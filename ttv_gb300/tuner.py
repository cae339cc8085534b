"""Autotuner for single TTVs: times candidate plans and keeps the fastest.

    python -m ttv_gb300.tuner --workload sym --out tuned.json        (on a GPU)

For one problem (element type, extents, layout, q) the candidates are the
kernel families that can run it (row / column register kernels, the
TMA-streamed kernel), their lane-group or warp-stacking parameter, the split
of the contracted mode and, for fp64, native DFMA or the DFMA / double-float
mix.  Each candidate is CUDA-event timed on device-resident random data
(inputs larger than L2 or flushed before every launch), best of several
launches after warm-up.  Results can be installed as plan hints
(``install``): later calls with the same (type, P, n_q, S) use the tuned
options instead of the planner's rules.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

from . import F32, F64, KIND_COL, KIND_COL_BULK, KIND_COL_REALIGN, KIND_ROW, KIND_ROW_PANEL, KIND_ROW_SHIFT, \
    KIND_ROW_TILE, KIND_STREAM, \
    ACC_DOUBLE_FLOAT, \
    clear_plan_hint, output_layout, output_shape, plan, plan_hint, strides, ttv

L2_FLUSH_BYTES = 256 << 20


def candidates(dtype, P, nq, S):
    """Option dicts worth timing for a canonical problem."""
    out = [{}]   # the planner's own choice
    es = 8 if dtype == F64 else 4
    accs = (0, ACC_DOUBLE_FLOAT) if dtype == F64 else (0,)
    if P == 1:
        for g in (1, 2, 4, 8, 16, 32):
            for acc in accs:
                out.append({"kind": KIND_ROW, "group": g, "accumulate": acc})
        if nq * es <= 16384:
            for g in (0, 2, 4, 8, 16, 32):
                out.append({"kind": KIND_STREAM, "group": g})
        if nq <= 64:
            for acc in accs:
                out.append({"kind": KIND_ROW_TILE, "accumulate": acc})
        if nq % (16 // es) == 0 and nq > 1024 * (16 // es):   # longer than one segment of b
            for rr in (1, 2):
                out.append({"kind": KIND_ROW_PANEL, "group": rr})
        # rows that are not whole 16-byte vectors, b's shifted copies within 48 KB
        w = (nq + 2 * (16 // es) - 1) // (16 // es) * (16 // es)
        if nq % (16 // es) and (16 // es) * w * (es + (8 if dtype == F64 else 0)) <= 48 * 1024:
            for g in (4, 8, 16, 32):
                out.append({"kind": KIND_ROW_SHIFT, "group": g})
    else:
        min_split = -(-nq // (16384 // es))
        kinds = (KIND_COL, KIND_COL_REALIGN) if P % (16 // es) else (KIND_COL,)
        for kind in kinds:
            for wi in (1, 2, 4, 8):
                for split in (0, 1, 2, 4, 16):
                    if split and (split > nq or split < min_split):
                        continue
                    for acc in accs:
                        out.append({"kind": kind, "group": wi, "split": split, "accumulate": acc})
        if P * es <= 16384 and -(-P // 256) <= 8:
            out.append({"kind": KIND_STREAM})
        if P * es >= 2048:
            for split in (0, 1):
                if split and split < min_split:
                    continue
                for acc in accs:
                    out.append({"kind": KIND_COL_BULK, "split": split, "accumulate": acc})
    return out


def time_options(q, na, pia, A, b, c, opts, reps=5, flush=None):
    import torch
    wa = strides(na, pia)
    nc, pic = output_shape(na, q), output_layout(pia, q)
    wc = strides(nc, pic)
    p = len(na)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dt = F64 if A.dtype == torch.float64 else F32

    def call():
        ttv(q, p, A, na, wa, pia, b, [na[q - 1]], c, nc, wc, pic, dtype=dt, **opts)

    for _ in range(2):
        call()
    best = float("inf")
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
        e0.record()
        call()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune_problem(dtype, na, pia, q, A, b, c, reps=5, flush=None):
    """(best options, best ms, default ms, table) for one problem."""
    pl = plan(q, na, pia, dtype=dtype)
    table = []
    for opts in candidates(dtype, pl["P"], pl["nq"], pl["S"]):
        try:
            ms = time_options(q, na, pia, A, b, c, opts, reps, flush)
        except Exception as exc:   # refused combination
            table.append((opts, None, str(exc)[:80]))
            continue
        table.append((opts, ms, ""))
    timed = [(o, ms) for o, ms, _ in table if ms is not None]
    best_opts, best_ms = min(timed, key=lambda t: t[1])
    return best_opts, best_ms, table[0][1], table


def install(entries):
    """Install tuned options as plan hints: [{'dtype', 'P', 'nq', 'S', 'options'}]."""
    for e in entries:
        plan_hint(e["dtype"], e["P"], e["nq"], e["S"], **e["options"])


def clear_hints():
    clear_plan_hint()


def main():
    import torch
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sym", choices=["sym", "asym"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    cases = bench.WORKLOADS[args.workload][0]()
    dev = torch.device("cuda")
    tdt = {"f32": torch.float32, "f64": torch.float64}
    maxN = max(int(np.prod(c["na"])) for c in cases)
    maxM = max(int(np.prod(c["na"])) // c["na"][c["q"] - 1] for c in cases)
    maxQ = max(c["na"][c["q"] - 1] for c in cases)
    bufs = {}
    results = []
    tot_def = tot_best = 0.0
    for cs in cases:
        dt = cs["dtype"]
        if dt not in bufs:
            bufs[dt] = (torch.rand(maxN, device=dev, dtype=tdt[dt]) * 2 - 1,
                        torch.rand(maxQ, device=dev, dtype=tdt[dt]) * 2 - 1,
                        torch.empty(maxM, device=dev, dtype=tdt[dt]))
        A, b, c = bufs[dt]
        code = F64 if dt == "f64" else F32
        best, best_ms, def_ms, table = tune_problem(code, cs["na"], cs["pia"], cs["q"], A, b, c,
                                                    args.reps)
        pl = plan(cs["q"], cs["na"], cs["pia"], dtype=code)
        nbytes = bench.case_bytes(cs)
        results.append({"dtype": code, "na": cs["na"], "pia": cs["pia"], "q": cs["q"],
                        "P": pl["P"], "nq": pl["nq"], "S": pl["S"], "options": best,
                        "best_GBps": nbytes / best_ms / 1e6, "default_GBps": nbytes / def_ms / 1e6,
                        "table": [(o, ms) for o, ms, _ in table]})
        tot_def += def_ms
        tot_best += best_ms
        print(f"{dt} {cs['na'][0]}^{len(cs['na'])} pia={cs['pia'][0]} q={cs['q']} "
              f"P={pl['P']} nq={pl['nq']} S={pl['S']}: default {nbytes / def_ms / 1e6:7.0f} "
              f"best {nbytes / best_ms / 1e6:7.0f} GB/s with {best}", flush=True)
    print(json.dumps({"workload": args.workload, "default_ms": tot_def, "tuned_ms": tot_best,
                      "gain": tot_def / tot_best}))
    if args.out:
        with open(args.out, "w") as f:
            json.dump(results, f)


if __name__ == "__main__":
    main()
