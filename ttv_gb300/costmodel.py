"""Autotuner, training and evaluation of the learned variant selector.

    python -m ttv_gb300.costmodel --train 20000 --test 2000      (on a GPU)

1. ``random_shapes`` draws batched-TTV problems: order p uniform in {3,4,5},
   every extent log-uniform in [8, 512] (rounded), re-drawn until the problem
   has at most 2^22 elements, a random contraction mode and a random layout.
2. ``tune_mixed`` times every kernel variant of each shape exhaustively inside
   mixed batches (random sizes 64..4096): each batch runs once per forced
   variant, L2 flushed before each recorded launch, and the persistent
   executor sums every problem's SM clock cycles; cost = microseconds per
   problem.  (``tune``: the older K-copies method, launch time / K.)
3. ``train`` fits the MLP (features + one-hot variant -> log2 cost) with the
   engine's own CUDA forward/backward/Adam kernels.
4. ``evaluate`` measures regret against exhaustive tuning on held-out shapes,
   for the learned choice and for the engine's fixed rule.

Results go to ttv_gb300/data/: tuning_db.npz (features, times, fixed-rule
variant, split) and cost_model.npz (parameters, loss curve, regret).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import batch as B

DATA = B.DATA
DB_PATH = os.path.join(DATA, "tuning_db.npz")


def random_shapes(n, seed, max_elems=1 << 22, lo=8, hi=512, orders=(3, 4, 5)):
    """Shapes of the batched configuration (rejection-resampled to <= max_elems)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        p = int(rng.choice(orders))
        na = [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(p)]
        if int(np.prod(na)) > max_elems:
            continue
        q = int(rng.integers(1, p + 1))
        pia = [int(x) + 1 for x in rng.permutation(p)]
        out.append((na, pia, q))
    return out


def problems_from_arena(shapes_counts, A, b, C):
    """Problems laid out back to back in device arenas A (inputs) and C (outputs);
    every problem shares the vector arena b.  Offsets are 64-element aligned."""
    import copy
    probs = []
    oa = oc = 0
    a0, c0 = A.data_ptr(), C.data_ptr()
    for (na, pia, q), k in shapes_counts:
        N = int(np.prod(na))
        M = N // na[q - 1]
        first = B.Problem(q, na, pia, a0 + 4 * oa, b[:na[q - 1]], c0 + 4 * oc)
        for j in range(k):
            pr = first if j == 0 else copy.copy(first)   # metadata shared, buffers differ
            pr.a, pr.c = a0 + 4 * oa, c0 + 4 * oc
            pr.a_view, pr.c_view = A[oa:oa + N], C[oc:oc + M]
            probs.append(pr)
            oa += (N + 63) // 64 * 64
            oc += (M + 63) // 64 * 64
    assert oa <= A.numel() and oc <= C.numel()
    return probs


def copies_for(na, target_bytes=256 << 20, lo=32, hi=4096):
    nbytes = 4 * int(np.prod(na))
    return int(min(hi, max(lo, -(-target_bytes // nbytes))))


def tune(shapes, reps=2, log_every=500, flush_bytes=256 << 20):
    """Exhaustive timing of every variant of every shape: (features [n, 8], times [n, 8] us
    per problem, fixed-rule variant [n])."""
    import torch
    dev = torch.device("cuda")
    A = torch.rand(int(1.2 * (1 << 28)) // 4 * 4 + (1 << 22), device=dev) * 2 - 1
    b = torch.rand(1024, device=dev) * 2 - 1
    C = torch.empty(64 << 20, device=dev)
    flush = torch.empty(flush_bytes // 4, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    feats = np.zeros((len(shapes), B.MLP_FEATURES), np.float32)
    times = np.zeros((len(shapes), B.NVARIANT), np.float32)
    heur = np.zeros(len(shapes), np.int32)
    t0 = time.time()
    for si, (na, pia, q) in enumerate(shapes):
        k = copies_for(na)
        probs = problems_from_arena([((na, pia, q), k)], A, b, C)
        f, _kind, h = B.features(probs)
        feats[si] = f[0]
        heur[si] = h[0]
        with B.Batch(probs, select=B.SELECT_FIXED, variant=0, no_graph=True) as bt:
            for v in range(B.NVARIANT):
                bt.set_variant(v)
                best = float("inf")
                for r in range(reps + 1):
                    flush.zero_()
                    e0.record()
                    bt.launch()
                    e1.record()
                    e1.synchronize()
                    if r:
                        best = min(best, e0.elapsed_time(e1))
                times[si, v] = best * 1e3 / k
        if log_every and (si + 1) % log_every == 0:
            print(f"tuned {si + 1}/{len(shapes)} shapes in {time.time() - t0:.0f} s", flush=True)
    return feats, times, heur


def tune_mixed(shapes, seed=0, reps=2, lo=64, hi=4096, log_every=5000,
               flush_bytes=256 << 20, arena_elems=3 << 30):
    """Exhaustive timing of every variant of every shape inside mixed batches.

    Shapes are taken in consecutive batches whose sizes are drawn log-uniformly in
    [lo, hi]; each batch runs once per variant with that variant forced on every
    problem, L2 flushed before each recorded launch, and the executor sums each
    problem's SM clock cycles (``Batch.costs``).  Cost = min over reps, in
    microseconds at the 2070 MHz maximum SM clock.  The batch-size feature is the
    size of the batch the problem was timed in."""
    import torch
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed)
    A = torch.empty(arena_elems, device=dev)
    A.uniform_(-1, 1)
    b = torch.rand(1024, device=dev) * 2 - 1
    C = torch.empty(arena_elems // 8, device=dev)
    flush = torch.empty(flush_bytes // 4, device=dev)
    feats = np.zeros((len(shapes), B.MLP_FEATURES), np.float32)
    times = np.zeros((len(shapes), B.NVARIANT), np.float32)
    heur = np.zeros(len(shapes), np.int32)
    batch_of = np.zeros(len(shapes), np.int32)
    valid = variant_mask(shapes)
    t0 = time.time()
    i = nb = 0
    while i < len(shapes):
        want = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        chunk, tot_a, tot_c = [], 0, 0
        for sh in shapes[i:i + want]:
            N = int(np.prod(sh[0]))
            na_a = (N + 63) // 64 * 64
            na_c = (N // sh[0][sh[2] - 1] + 63) // 64 * 64
            if tot_a + na_a > A.numel() or tot_c + na_c > C.numel():
                break
            chunk.append(sh)
            tot_a += na_a
            tot_c += na_c
        idx = np.arange(i, i + len(chunk))
        probs = problems_from_arena([(sh, 1) for sh in chunk], A, b, C)
        f, _kind, h = B.features(probs)
        feats[idx], heur[idx], batch_of[idx] = f, h, nb
        with B.Batch(probs, select=B.SELECT_FIXED, variant=0, no_graph=True,
                     record_costs=True) as bt:
            for v in range(B.NVARIANT):
                bt.set_variant(v)
                bt.launch()
                best = None
                for _ in range(reps):
                    flush.zero_()
                    bt.launch()
                    c = bt.costs().astype(np.float64)
                    best = c if best is None else np.minimum(best, c)
                times[idx, v] = np.where(valid[idx, v], best / 2070.0, np.inf)
        i += len(chunk)
        nb += 1
        if log_every and i // log_every != (i - len(chunk)) // log_every:
            print(f"tuned {i}/{len(shapes)} shapes in {nb} mixed batches, {time.time() - t0:.0f} s",
                  flush=True)
    return feats, times, heur


def variant_mask(shapes):
    """Variants each shape can run: all but the staged rows, which need q to be the
    fastest layout mode (prefix P == 1) and n_q <= 64."""
    valid = np.ones((len(shapes), B.NVARIANT), bool)
    for i, (na, pia, q) in enumerate(shapes):
        valid[i, B.VARIANT_STAGED] = pia[0] == q and na[q - 1] <= 64
    return valid


def training_set(feats, times):
    """(inputs, log2 cost) of every runnable (problem, variant) pair."""
    x = B.mlp_inputs(feats)
    t = times.ravel()
    ok = np.isfinite(t)
    y = np.log2(np.maximum(t[ok], 1e-3)).astype(np.float32)
    return x[ok], y


def rule_class(feats):
    """(kernel family, widest load, short row) of each shape: the classes the fixed
    rule distinguishes (short: q-fastest rows of at most 64 elements, the ones the
    staged variant can take)."""
    kind = np.where(feats[:, 2] > 0, 1, 0)          # log2 P > 0: column form
    vec = np.rint(feats[:, 7] * 4).astype(int)
    nq = np.rint(2.0 ** (feats[:, 3].astype(np.float64) * 24))
    short = ((kind == 0) & (nq <= 64)).astype(int)
    return kind, vec, short


def derive_fixed_rule(feats, times):
    """The best single variant of each (kernel family, widest load, short row) class
    over tuned shapes: the variant with the least total time in the class."""
    kind, vec, short = rule_class(feats)
    rule = {}
    for k in (0, 1):
        for v in (1, 2, 4):
            for sh in (0, 1):
                m = (kind == k) & (vec == v) & (short == sh)
                if m.any():
                    tot = np.where(np.isfinite(times[m]), times[m], np.inf).sum(axis=0)
                    rule[(k, v, sh)] = int(np.argmin(tot))
    return rule


def apply_fixed_rule(rule, feats):
    kind, vec, short = rule_class(feats)
    return np.array([rule.get((k, v, sh), 0) for k, v, sh in zip(kind, vec, short)], np.int32)


def train(feats, times, epochs=60, batch=512, lr=2e-3, seed=0):
    import torch
    x, y = training_set(feats, times)
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y).cuda()
    params = torch.from_numpy(B.init_params(seed)).cuda()
    losses = B.mlp_train(params, dx, dy, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return params.cpu().numpy(), losses


def predict_scores(params, feats, valid=None):
    """Predicted log2 cost of every variant of every shape (the engine's inference
    kernel); variants a shape cannot run score +inf."""
    import torch
    x = torch.from_numpy(B.mlp_inputs(feats)).cuda()
    pred = B.mlp_predict(torch.from_numpy(np.asarray(params, np.float32)).cuda(), x)
    scores = pred.cpu().numpy().reshape(len(feats), B.NVARIANT)
    if valid is not None:
        scores = np.where(valid, scores, np.inf)
    return scores


def choose(scores, heuristic, margin):
    """The batch selection rule: argmin of the predicted cost, unless it does not beat
    the fixed rule's variant by the relative margin."""
    best = scores.argmin(axis=1)
    idx = np.arange(len(scores))
    keep = ~(scores[idx, best] < scores[idx, heuristic] + np.log2(1.0 - margin))
    return np.where(keep, heuristic, best)


def predict_variants(params, feats, heuristic=None, margin=0.0, valid=None):
    scores = predict_scores(params, feats, valid)
    if heuristic is None:
        return scores.argmin(axis=1)
    return choose(scores, heuristic, margin)


def regret(times, chosen):
    """Aggregate time of the chosen variants over exhaustive tuning's best, minus one;
    and the mean per-shape ratio minus one."""
    idx = np.arange(len(times))
    t_sel = times[idx, chosen].astype(np.float64)
    t_best = times.min(axis=1).astype(np.float64)
    return float(t_sel.sum() / t_best.sum() - 1.0), float(np.mean(t_sel / t_best) - 1.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--out", default=DATA)
    ap.add_argument("--reuse-db", action="store_true", help="train on an existing tuning_db.npz")
    ap.add_argument("--mode", choices=["mixed", "copies"], default="mixed",
                    help="mixed: per-problem cycles inside mixed batches (default); copies: K "
                         "copies of each shape, launch time / K")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    db_path = os.path.join(args.out, "tuning_db.npz")
    if args.reuse_db and os.path.exists(db_path):
        d = np.load(db_path)
        feats, times, heur, split = d["features"], d["times"], d["heuristic"], d["is_test"]
        valid = d["valid"] if "valid" in d else np.isfinite(times)
    else:
        shapes = random_shapes(args.train + args.test, args.seed)
        t0 = time.time()
        if args.mode == "mixed":
            feats, times, heur = tune_mixed(shapes, seed=args.seed)
        else:
            feats, times, heur = tune(shapes)
        valid = variant_mask(shapes)
        print(f"tuning: {time.time() - t0:.1f} s for {len(shapes)} shapes x {B.NVARIANT} variants")
        split = np.zeros(len(shapes), bool)
        split[args.train:] = True
        np.savez_compressed(db_path, features=feats, times=times, heuristic=heur, is_test=split,
                            valid=valid, shapes=np.frombuffer(json.dumps(shapes).encode(), np.uint8))
    tr, te = ~split, split
    # the fixed rule, re-derived from the training shapes: the best single variant of
    # each (kernel family, widest load) class
    rule = derive_fixed_rule(feats[tr], times[tr])
    fixed = apply_fixed_rule(rule, feats)
    if not args.reuse_db:   # the engine's rule is set to this one (the db records it)
        np.savez_compressed(db_path, features=feats, times=times, heuristic=fixed, is_test=split,
                            valid=valid, shapes=np.frombuffer(json.dumps(shapes).encode(), np.uint8))
    # the last tenth of the training shapes picks the selection margin
    tr_idx = np.where(tr)[0]
    fit, val = tr_idx[: len(tr_idx) * 9 // 10], tr_idx[len(tr_idx) * 9 // 10:]
    t0 = time.time()
    params, losses = train(feats[fit], times[fit], epochs=args.epochs, seed=args.seed)
    t_train = time.time() - t0
    val_scores = predict_scores(params, feats[val], valid[val])
    margins = [0.0, 0.02, 0.05, 0.1, 0.15, 0.2, 0.3, 0.5]
    val_regret = {m: regret(times[val], choose(val_scores, fixed[val], m))[0] for m in margins}
    margin = min(margins, key=lambda m: val_regret[m])
    learned = predict_variants(params, feats[te], fixed[te], margin, valid[te])
    r_learn = regret(times[te], learned)
    r_argmin = regret(times[te], predict_variants(params, feats[te], valid=valid[te]))
    r_fixed_rule = regret(times[te], fixed[te])
    r_engine_rule = regret(times[te], heur[te])
    r_single = {v: regret(times[te], np.where(valid[te][:, v], v, fixed[te]))[0] for v in range(B.NVARIANT)}
    best = np.where(valid[te], times[te], np.inf).argmin(axis=1)
    summary = {"train_shapes": int(len(fit)), "validation_shapes": int(len(val)),
               "test_shapes": int(te.sum()),
               "train_seconds": round(t_train, 2), "final_loss": float(losses[-1]),
               "fixed_rule": {f"{'col' if k else 'row'}_vec{v}{'_short' if sh else ''}": r
                              for (k, v, sh), r in sorted(rule.items())},
               "margin": margin, "validation_regret_by_margin": val_regret,
               "regret_learned": r_learn, "regret_learned_plain_argmin": r_argmin,
               "regret_fixed_rule": r_fixed_rule, "regret_engine_rule": r_engine_rule,
               "regret_single_variant": r_single,
               "learned_picks_best": float(np.mean(learned == best)),
               "learned_leaves_fixed_rule": float(np.mean(learned != fixed[te]))}
    np.savez_compressed(os.path.join(args.out, "cost_model.npz"), params=params, losses=losses,
                        margin=np.float32(margin),
                        summary=np.frombuffer(json.dumps(summary).encode(), np.uint8))
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
