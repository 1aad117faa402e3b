"""The learned fusion cost model.

CPU: the FP64 MLP oracle's gradient against central differences; the feature
layout constants.  GPU: the engine's hand-written training kernels against the
FP64 oracle; training on engine-measured timings; and what the trained model
gains over the method without it (greedy fixed-k fusion) in measured wall time:
in FP64 (where dense blocks are FP64-bound and the model turns fusion down) and
in FP32 (where it scores the fuser's candidate blocks).
"""
import os
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import mlp_oracle  # noqa: E402
from quant_iron_gb300 import costmodel, workloads  # noqa: E402


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(scale=0.2, size=costmodel.num_params())
    X = rng.uniform(0, 1, size=(20, 20))
    y = rng.normal(size=20)
    _, g = mlp_oracle.loss_and_gradient(p, X, y)
    for j in rng.choice(p.size, 40, replace=False):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[j] += e
        pm[j] -= e
        fd = (mlp_oracle.loss_and_gradient(pp, X, y)[0] - mlp_oracle.loss_and_gradient(pm, X, y)[0]) / (2 * e)
        assert abs(fd - g[j]) < 1e-6 * max(1.0, abs(fd))


def test_param_count_matches_oracle_layout():
    assert costmodel.num_params() == sum(i * o + o for i, o in mlp_oracle.SIZES)


@pytest.mark.gpu
def test_gpu_gradient_matches_fp64_oracle():
    rng = np.random.default_rng(1)
    X = rng.uniform(0, 1, size=(300, 20)).astype(np.float32)
    y = rng.normal(size=300).astype(np.float32)
    costmodel.init(seed=3)
    p, _ = costmodel.params()
    loss, g = costmodel.loss_and_gradient(X, y)
    loss_ref, g_ref = mlp_oracle.loss_and_gradient(p, X, y)
    assert abs(loss - loss_ref) < 1e-5 * max(1.0, loss_ref)
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-5


@pytest.mark.gpu
def test_train_on_engine_timings_and_learned_gain():
    n = 24   # 256 MB FP64 state: above the 129 MB L2, so op times are HBM-bound and stable
    X, y = costmodel.collect(n, 1200, seed=5)
    idx = np.random.default_rng(0).permutation(len(y))
    tr, te = idx[:1000], idx[1000:]
    hist = costmodel.train(X[tr], y[tr], epochs=1500, lr=3e-3, seed=1)
    assert hist[-1] < 0.25 * hist[0]
    pred = costmodel.predict(X[te])
    corr = np.corrcoef(pred, y[te])[0, 1]
    assert corr > 0.8, corr

    import quant_iron_gb300 as qi
    gates = workloads.random_circuit(n, layers=20, seed=9)

    def wall(prec, **kw):
        plan = qi.Plan(n, prec, gates, **kw)
        with qi.DeviceState(n, prec) as st:
            st.set_plus()
            plan.execute(st)
            st.synchronize()
            t0 = time.perf_counter()
            for _ in range(3):
                plan.execute(st)
            st.synchronize()
            return (time.perf_counter() - t0) / 3, plan.stats()

    # FP64: dense fused blocks are FP64-compute-bound on GB300, so greedy
    # fixed-k (the method without the model) loses to one kernel per gate
    t_greedy64, _ = wall(qi.F64, fusion=qi.FUSION_GREEDY, max_block_qubits=5)
    t_learned64, st64 = wall(qi.F64, fusion=qi.FUSION_LEARNED, max_block_qubits=5)
    t_none64, _ = wall(qi.F64, fusion=qi.FUSION_NONE)
    assert st64["predicted_us"] > 0
    assert t_learned64 < 0.8 * t_greedy64, (t_learned64, t_greedy64)
    assert t_learned64 < 1.5 * min(t_none64, t_greedy64), (t_learned64, t_none64, t_greedy64)
    # FP32: the model-scored plan (block by block, or a whole-plan preset, whichever it predicts
    # faster) is no slower than the greedy fixed-k fuser it falls back to (5% for timing noise)
    t_greedy32, _ = wall(qi.F32, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
    t_learned32, st32 = wall(qi.F32, fusion=qi.FUSION_LEARNED, max_block_qubits=6)
    assert st32["predicted_us"] > 0
    print("FP32 greedy %.3f ms, learned %.3f ms (%d kernels), gain %.1f%%" %
          (t_greedy32 * 1e3, t_learned32 * 1e3, st32["n_kernels"], 100 * (1 - t_learned32 / t_greedy32)))
    assert t_learned32 <= 1.05 * t_greedy32, (t_learned32, t_greedy32)
