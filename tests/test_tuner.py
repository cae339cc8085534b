"""The single-call autotuner (ttv_gb300/tuner.py) and the plan hints it
installs (tlibg_plan_hint, looked up by the planner through tlibg_plan).

CPU: candidate enumeration per kernel family; hint install, lookup,
precedence over the planner's rules, fallback when a hint no longer applies,
removal.  GPU: a problem run under a hinted plan matches the oracle, and the
tuner's own timing loop picks a candidate that is at least as fast as the
planner's choice on its own measurements.
"""
import numpy as np
import pytest

from ttv_gb300 import tuner as TU


@pytest.fixture()
def T(engine):
    engine.clear_plan_hint()
    yield engine
    engine.clear_plan_hint()


def test_candidates_row_form(T):
    cands = TU.candidates(T.F32, 1, 48, 1 << 20)
    assert cands[0] == {}   # the planner's own choice comes first
    kinds = {c.get("kind") for c in cands[1:]}
    assert kinds == {T.KIND_ROW, T.KIND_STREAM, T.KIND_ROW_TILE}
    assert sorted({c["group"] for c in cands if c.get("kind") == T.KIND_ROW}) == [1, 2, 4, 8, 16, 32]
    # long rows: no streamed or row-tile candidates (a row must fit a 16 KB stage / 64 elements)
    long_ = TU.candidates(T.F32, 1, 1 << 16, 64)
    assert {c.get("kind") for c in long_[1:]} == {T.KIND_ROW, T.KIND_ROW_PANEL}
    # the row-panel kernel needs rows of whole 16-byte vectors longer than one segment
    assert T.KIND_ROW_PANEL not in {c.get("kind") for c in TU.candidates(T.F32, 1, (1 << 16) + 1, 64)}
    assert T.KIND_ROW_PANEL not in {c.get("kind") for c in TU.candidates(T.F32, 1, 4096, 64)}
    # fp64 adds the double-float accumulation to every row candidate
    f64 = TU.candidates(T.F64, 1, 48, 1 << 20)
    assert {c.get("accumulate") for c in f64 if c.get("kind") == T.KIND_ROW} == {0, T.ACC_DOUBLE_FLOAT}
    # rows that are not whole 16-byte vectors: row-shift candidates while b's shifted copies fit 48 KB
    odd = TU.candidates(T.F32, 1, 645, 1 << 16)
    assert sorted(c["group"] for c in odd if c.get("kind") == T.KIND_ROW_SHIFT) == [4, 8, 16, 32]
    assert T.KIND_ROW_SHIFT not in {c.get("kind") for c in TU.candidates(T.F32, 1, 644, 1 << 16)}
    assert T.KIND_ROW_SHIFT not in {c.get("kind") for c in TU.candidates(T.F32, 1, 4001, 1 << 16)}
    assert T.KIND_ROW_SHIFT in {c.get("kind") for c in TU.candidates(T.F64, 1, 1533, 1 << 16)}
    assert T.KIND_ROW_SHIFT not in {c.get("kind") for c in TU.candidates(T.F64, 1, 1535, 1 << 16)}


def test_candidates_column_form(T):
    aligned = TU.candidates(T.F32, 256, 256, 256)
    assert {c.get("kind") for c in aligned[1:]} == {T.KIND_COL, T.KIND_STREAM}
    odd = TU.candidates(T.F32, 645, 645, 645)
    assert T.KIND_COL_REALIGN in {c.get("kind") for c in odd}
    assert T.KIND_COL_BULK in {c.get("kind") for c in odd}
    # splits below the staged-b minimum (n_q / 4096 floats) are never proposed
    long_q = TU.candidates(T.F32, 64, 1 << 14, 1)
    splits = {c["split"] for c in long_q if c.get("kind") == T.KIND_COL}
    assert 0 in splits and 16 in splits and not (splits & {1, 2})


def test_hint_install_lookup_and_precedence(T):
    na, pia, q = [645, 645, 645], [1, 2, 3], 2
    base = T.plan(q, na, pia)
    base64 = T.plan(q, na, pia, dtype=T.F64)
    other = T.plan(2, [644, 645, 645], [1, 2, 3])
    P, nq, S = base["P"], base["nq"], base["S"]
    want = {"kind": T.KIND_COL, "group": 4, "split": 3}
    assert (base["group"], base["split"]) != (4, 3)
    TU.install([{"dtype": T.F32, "P": P, "nq": nq, "S": S, "options": want}])
    got = T.plan(q, na, pia)
    assert (got["kind"], got["group"], got["split"]) == (T.KIND_COL, 4, 3)
    # the hint is keyed on the canonical problem: another layout with the same
    # (P, n_q, S) takes it, another dtype or shape does not
    same = T.plan(2, [645, 645, 645], [1, 2, 3])
    assert same["group"] == 4
    assert T.plan(q, na, pia, dtype=T.F64) == base64
    assert T.plan(2, [644, 645, 645], [1, 2, 3]) == other
    # explicit options win over the hint
    forced = T.plan(q, na, pia, kind=T.KIND_COL, group=2, split=1)
    assert (forced["group"], forced["split"]) == (2, 1)
    # removal restores the rules
    T.clear_plan_hint(T.F32, P, nq, S)
    again = T.plan(q, na, pia)
    assert (again["group"], again["split"]) == (base["group"], base["split"])


def test_hint_that_no_longer_applies_falls_back(T):
    # a row-kernel hint stored for a column problem cannot be planned: the rules apply
    na, pia, q = [256, 256, 256], [1, 2, 3], 2
    base = T.plan(q, na, pia)
    T.plan_hint(T.F32, base["P"], base["nq"], base["S"], kind=T.KIND_ROW, group=4)
    got = T.plan(q, na, pia)
    assert (got["kind"], got["group"], got["split"]) == (base["kind"], base["group"], base["split"])


def test_clear_all_hints(T):
    for P in (16, 32, 64):
        T.plan_hint(T.F32, P, 4096, 1, kind=T.KIND_COL, split=7)
    assert T.plan(2, [32, 4096], [1, 2])["split"] == 7
    TU.clear_hints()
    assert T.plan(2, [32, 4096], [1, 2])["split"] != 7


@pytest.mark.gpu
def test_hinted_plan_matches_oracle_and_tuner_picks_fastest(T, orc, cuda):
    import torch
    na, pia, q = [645, 645, 645], [1, 2, 3], 2
    rng = np.random.default_rng(3)
    a = rng.uniform(-1, 1, int(np.prod(na))).astype(np.float32)
    b = rng.uniform(-1, 1, na[q - 1]).astype(np.float32)
    A, B = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    C = torch.empty(645 * 645, device=cuda)
    base = T.plan(q, na, pia)
    ref, absn = orc.truth(645, 645, 645, a, b)
    for opts in ({"kind": T.KIND_COL, "group": 4, "split": 3},
                 {"kind": T.KIND_COL_BULK, "split": 0},
                 {"kind": T.KIND_COL_REALIGN, "group": 2, "split": 2}):
        T.plan_hint(T.F32, base["P"], base["nq"], base["S"], **opts)
        assert T.plan(q, na, pia)["kind"] == opts["kind"]
        C.fill_(float("nan"))
        wa = T.strides(na, pia)
        nc, pic = T.output_shape(na, q), T.output_layout(pia, q)
        T.ttv(q, 3, A, na, wa, pia, B, [645], C, nc, T.strides(nc, pic), pic, sync=True)
        err = orc.rel_error(C.cpu().numpy(), ref, absn)
        assert err <= 1e-5, (opts, err)
        T.clear_plan_hint()
    best, best_ms, def_ms, table = TU.tune_problem(T.F32, na, pia, q, A, B, C, reps=3)
    timed = [ms for _o, ms, _e in table if ms is not None]
    assert best_ms == min(timed) and best_ms <= def_ms
    assert table[0][0] == {} and table[0][1] == def_ms
