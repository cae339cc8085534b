"""Learned cost model: the numpy oracle (CPU), the engine's CUDA forward /
backward / Adam kernels against it (GPU), the problem features, and what the
trained network gains over the fixed rule (GPU, committed tuning data)."""
import os

import numpy as np
import pytest

import oracle.mlp as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def rand_params(seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(M.NPARAMS) * 0.3).astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rand_params(1).astype(np.float64)
    x = rng.standard_normal((7, M.IN))
    y = rng.standard_normal(7)
    L, g = M.loss_grad(p, x, y)
    assert abs(L - M.loss(p, x, y)) < 1e-12
    idx = rng.choice(M.NPARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (M.loss(p + e, x, y) - M.loss(p - e, x, y)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_layout_constants(engine):
    from ttv_gb300 import batch as B
    assert M.NPARAMS == B.MLP_PARAMS == 9537
    hdr = open(os.path.join(ROOT, "include", "tlibg.h")).read()
    assert "#define TLIBG_MLP_PARAMS 9537" in hdr
    assert B.init_params(0).size == M.NPARAMS


def test_features_and_fixed_rule_on_cpu(engine):
    """Features come from host-side validation only: no device is needed."""
    from ttv_gb300 import batch as B
    probs = [B.Problem(2, [16, 32, 64], [1, 2, 3], 256, 512, 1024),
             B.Problem(1, [100, 7, 9, 11], [1, 2, 3, 4], 256, 512, 1024),
             B.Problem(3, [8, 512, 40], [3, 2, 1], 256, 512, 1024)]
    f, kind, heur = B.features(probs)
    assert f.shape == (3, 8)
    # problem 0: P = 16, nq = 32, S = 64, q at layout position 1 of 0..2
    # (fake pointers 256/512/1024 are 16-byte aligned and P % 4 == 0: loads of 4)
    np.testing.assert_allclose(f[0], [3 / 8, 0.5, 4 / 24, 5 / 24, 6 / 24, 0, np.log2(3) / 16, 1],
                               rtol=1e-6)
    assert list(kind) == [1, 0, 0]   # column, row (q first), row (q first in layout 3,2,1)
    assert all(0 <= h < B.NVARIANT for h in heur)


def test_mlp_inputs_rows():
    from ttv_gb300 import batch as B
    f = np.arange(16, dtype=np.float32).reshape(2, 8)
    x = B.mlp_inputs(f)
    nv = B.NVARIANT
    assert x.shape == (2 * nv, 8 + nv)
    assert np.all(x[3, :8] == f[0]) and x[3, 8 + 3] == 1 and x[3, 8:].sum() == 1
    assert np.all(x[nv + 1, :8] == f[1]) and x[nv + 1, 8 + 1] == 1


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_gpu_loss_grad_matches_oracle(engine, cuda):
    import torch
    from ttv_gb300 import batch as B
    rng = np.random.default_rng(3)
    for n in (1, 5, 257):
        p = rand_params(n)
        x = rng.standard_normal((n, M.IN)).astype(np.float32)
        y = rng.standard_normal(n).astype(np.float32)
        loss, grad = B.mlp_loss_grad(torch.from_numpy(p).cuda(), torch.from_numpy(x).cuda(),
                                     torch.from_numpy(y).cuda())
        L, g = M.loss_grad(p, x, y)
        assert abs(float(loss) - L) <= 1e-4 * max(1, abs(L))
        gg = grad.cpu().numpy().astype(np.float64)
        scale = np.max(np.abs(g)) + 1e-12
        assert np.max(np.abs(gg - g)) <= 2e-4 * scale, (n, np.max(np.abs(gg - g)), scale)


@pytest.mark.gpu
def test_gpu_adam_and_predict_match_oracle(engine, cuda):
    import torch
    from ttv_gb300 import batch as B
    rng = np.random.default_rng(4)
    p = rand_params(7)
    g = rng.standard_normal(M.NPARAMS).astype(np.float32)
    m = rng.standard_normal(M.NPARAMS).astype(np.float32) * 0.1
    v = np.abs(rng.standard_normal(M.NPARAMS)).astype(np.float32) * 0.1
    dp, dm, dv = (torch.from_numpy(t.copy()).cuda() for t in (p, m, v))
    B.mlp_adam(dp, torch.from_numpy(g).cuda(), dm, dv, step=3, lr=1e-2)
    ep, em, ev = M.adam(p.astype(np.float64), g, m, v, 3, lr=1e-2)
    np.testing.assert_allclose(dp.cpu().numpy(), ep, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(dm.cpu().numpy(), em, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(dv.cpu().numpy(), ev, rtol=1e-5, atol=1e-7)
    x = rng.standard_normal((300, M.IN)).astype(np.float32)
    y = B.mlp_predict(torch.from_numpy(p).cuda(), torch.from_numpy(x).cuda()).cpu().numpy()
    ref, _ = M.forward(p, x)
    np.testing.assert_allclose(y, ref, rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_gpu_training_fits_a_known_function(engine, cuda):
    """Training with the engine's kernels drives the loss down on y = f(x)."""
    import torch
    from ttv_gb300 import batch as B
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (4096, M.IN)).astype(np.float32)
    y = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3]).astype(np.float32)
    params = torch.from_numpy(B.init_params(1)).cuda()
    losses = B.mlp_train(params, torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda(),
                         epochs=40, batch=256, lr=3e-3, seed=1)
    assert losses[-1] < 0.1 * losses[0], losses
    final = M.loss(params.cpu().numpy(), x, y)
    assert final < 0.02, final


@pytest.mark.gpu
def test_learned_selection_beats_fixed_rule(engine, cuda):
    """On held-out shapes timed by exhaustive autotuning, the trained network's
    choices cost less than the fixed rule (regret vs the tuned best).  The fixed
    rule is re-derived from the same tuning data (the best single variant of each
    kernel family and load width on the training shapes), and it is the rule the
    engine applies without a model."""
    from ttv_gb300 import batch as B
    from ttv_gb300 import costmodel as CM
    if not (os.path.exists(CM.DB_PATH) and os.path.exists(B.MODEL_PATH)):
        pytest.skip("no committed tuning database / trained model")
    d = np.load(CM.DB_PATH)
    if d["times"].shape[1] != B.NVARIANT or np.load(B.MODEL_PATH)["params"].size != B.MLP_PARAMS:
        pytest.skip("tuning database / model made for another variant set")
    te = d["is_test"]
    valid = d["valid"] if "valid" in d else np.isfinite(d["times"])
    rule = CM.derive_fixed_rule(d["features"][~te], d["times"][~te])
    feats, times = d["features"][te], d["times"][te]
    fixed = CM.apply_fixed_rule(rule, feats)
    assert np.array_equal(fixed, d["heuristic"][te])   # the engine's own rule is this one
    m = np.load(B.MODEL_PATH)
    params, margin = m["params"], (float(m["margin"]) if "margin" in m else 0.0)
    learned = CM.predict_variants(params, feats, fixed, margin, valid[te])   # the engine's inference kernel
    assert valid[te][np.arange(te.sum()), learned].all()
    r_learn, _ = CM.regret(times, learned)
    r_fixed, _ = CM.regret(times, fixed)
    assert r_learn < r_fixed, (r_learn, r_fixed)
    assert r_learn < 0.10, r_learn
