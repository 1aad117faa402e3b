"""Fused k-qubit blocks on the tensor cores (tcgen05, 3xTF32) vs numpy FP64 (GPU).

Tolerance: the 3xTF32 products keep ~22 significant bits, so one block on a
normalised random state stays within 2e-6 per amplitude of the FP64 result
and its infidelity below 1e-10."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def haar(k, seed):
    rng = np.random.default_rng(seed)
    z = (rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def apply_np(state, n, targets, U):
    k = len(targets)
    psi = state.reshape([2] * n)
    axes = [n - 1 - t for t in targets[::-1]]
    rest = [a for a in range(n) if a not in axes]
    perm = axes + rest
    t = np.transpose(psi, perm).reshape(1 << k, -1)
    out = (U @ t).reshape([2] * n)
    return np.transpose(out, np.argsort(perm)).reshape(-1)


def rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


TARGET_SETS = {
    6: [[0, 1, 2, 3, 4, 5], [7, 8, 9, 10, 11, 12], [0, 2, 5, 8, 11, 12], [1, 3, 4, 6, 9, 10], [0, 6, 7, 8, 9, 12]],
    5: [[0, 1, 2, 3, 4], [8, 9, 10, 11, 12], [0, 3, 7, 10, 12], [2, 4, 5, 6, 11]],
}


@pytest.mark.parametrize("k", [5, 6])
@pytest.mark.parametrize("n", [13, 14, 16])
def test_tensor_core_block_vs_numpy(qi, k, n):
    for i, targets in enumerate(TARGET_SETS[k]):
        targets = [t if t < n else t - (13 - n) for t in targets]
        U = haar(k, 10 * k + i)
        init = rand_state(n, i)
        want = apply_np(init, n, targets, U)
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            qi.apply_matrix(st, targets, U, use_tensor_cores=1)
            got = st.download()
        err = np.max(np.abs(got - want))
        infid = 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real
        assert err < 2e-6 and infid < 1e-10, (k, n, targets, err, infid)


@pytest.mark.parametrize("k", [5, 6])
def test_tensor_core_many_tiles_per_sm(qi, k):
    """n = 23: 1024 (k = 6) or 2048 (k = 5) tiles, several per persistent CTA,
    so every shared buffer, A stage and accumulator is reused and every
    barrier goes through both phases."""
    n = 23
    # k = 6: [10..15] and [8, 10, ..., 18] take the tile-pair ring (all targets above qubit 7),
    # k = 5: [8, 11, 14, 18, 22] and [9..13];
    # [0..5], [0, 1, 2, 3, 9, 17] read row pairs in lane-rotated order (columns >= 128 B apart)
    # and store four rows at once; [0, 1, 4, 5, 12, 20] stores four rows without the rotation
    sets = {6: [[0, 1, 2, 3, 4, 5], [0, 6, 9, 17, 21, 22], [2, 3, 10, 15, 20, 22],
                [10, 11, 12, 13, 14, 15], [7, 9, 11, 15, 19, 22], [0, 9, 13, 16, 20, 22],
                [0, 1, 2, 3, 9, 17], [0, 1, 4, 5, 12, 20], [8, 10, 12, 14, 16, 18]],
            5: [[0, 1, 2, 3, 4], [0, 7, 16, 21, 22], [1, 5, 12, 19, 22], [0, 1, 2, 3, 11],
                [8, 11, 14, 18, 22], [9, 10, 11, 12, 13]]}[k]
    init = rand_state(n, 5)
    for i, targets in enumerate(sets):
        U = haar(k, 100 + i)
        want = apply_np(init, n, targets, U)
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            qi.apply_matrix(st, targets, U, use_tensor_cores=1)
            got = st.download()
        err = np.max(np.abs(got - want))
        infid = 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real
        assert err < 1e-6 and infid < 1e-10, (k, targets, err, infid)


@pytest.mark.parametrize("k", [5, 6])
def test_tensor_core_matches_cuda_core_path(qi, k):
    n = 15
    targets = [1, 4, 5, 9, 12, 14][:k]
    U = haar(k, 3)
    init = rand_state(n, 9)
    outs = []
    for tc in (1, 2):
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            qi.apply_matrix(st, targets, U, use_tensor_cores=tc)
            outs.append(st.download())
    assert np.max(np.abs(outs[0] - outs[1])) < 3e-6


def test_unsorted_targets_and_small_states(qi):
    # targets given out of order; n too small for the tensor-core tile falls back to CUDA cores
    for n in (6, 9, 13):
        targets = [3, 0, 5, 1, 4, 2] if n > 6 else [5, 0, 3, 1, 4, 2]
        U = haar(6, n)
        init = rand_state(n, n)
        want = apply_np(init, n, targets, U)
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            qi.apply_matrix(st, targets, U)
            assert np.max(np.abs(st.download() - want)) < 2e-6


def test_circuit_fused_tensor_cores_vs_oracle(qi, orc):
    from quant_iron_gb300 import workloads
    n = 16
    gates = workloads.random_circuit(n, layers=6, seed=21)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    for k in (5, 6):
        plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=k, use_tensor_cores=1)
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            plan.execute(st)
            got = st.download()
        # renormalised at the end of the plan: both the raw overlap and the
        # normalised infidelity are within the headline bound
        assert abs(np.vdot(got, got).real - 1.0) < 1e-6
        assert np.max(np.abs(got - want)) < 5e-6
        assert 1 - abs(np.vdot(want, got)) ** 2 < 1e-6


def test_tensor_core_norm_drift_and_renormalisation(qi):
    """The tensor cores accumulate FP32 with rounding toward zero, so repeated
    blocks shrink the norm slightly; the plan's FP64 renormalisation removes it."""
    from quant_iron_gb300.workloads import GateList
    n = 14
    gl = GateList()
    rng = np.random.default_rng(4)
    for layer in range(30):
        for q in range(6):
            gl.add("RY", [q], [], [rng.uniform(0, 6.28)])
            gl.add("RZ", [q], [], [rng.uniform(0, 6.28)])
        for q in range(5):
            gl.add("CNOT", [q + 1], [q])
    gates = gl.array()
    norms = {}
    for renorm in (-1, 0, 5):
        plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6, use_tensor_cores=1,
                       renorm_every=renorm)
        with qi.DeviceState(n, qi.F32) as st:
            st.set_plus()
            plan.execute(st)
            norms[renorm] = st.norm_sqr()
    assert abs(norms[0] - 1.0) < 1e-6 and abs(norms[5] - 1.0) < 1e-6
    assert abs(norms[-1] - 1.0) < 1e-3   # drift without renormalisation stays small


def test_tf32_rate_probe(qi):
    """The tensor roof probe runs, reports a rate in the range of a GB300's dense TF32
    (nominal 1.1 PFLOP/s) and leaves the device usable."""
    tf, ms = qi.tf32_rate_probe(iters=4096, reps=2)
    assert 100.0 < tf < 3000.0, tf
    assert ms > 0.0
    with qi.DeviceState(14, qi.F32) as st:
        st.set_plus()
        assert abs(st.norm_sqr() - 1.0) < 1e-6


def test_small_dense_blocks_padded_to_five_qubits(qi, orc):
    """A 3- or 4-qubit dense block of an FP32 plan runs as a 5-qubit tensor-core block with the
    identity on the lowest free qubits; the result matches the oracle."""
    from quant_iron_gb300.workloads import GateList
    n = 14
    for qubits in ([5, 9, 12], [1, 2, 7, 13], [0, 1, 2]):
        gl = GateList()
        rng = np.random.default_rng(len(qubits))
        for _ in range(3):
            for q in qubits:
                gl.add("RY", [q], [], [rng.uniform(0, 6.28)])
                gl.add("RZ", [q], [], [rng.uniform(0, 6.28)])
            for a, b in zip(qubits[:-1], qubits[1:]):
                gl.add("CNOT", [b], [a])
        gates = gl.array()
        init = rand_state(n, 3)
        want = orc.execute(init, n, gates)
        plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6, use_tensor_cores=1)
        dense = [o for o in plan.ops() if o["kind"] == 4]
        assert len(dense) == 1 and dense[0]["k"] == 5 and dense[0].get("tensor_cores"), plan.ops()
        assert set(qubits) <= set(dense[0]["targets"])
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            plan.execute(st)
            got = st.download()
        assert np.max(np.abs(got - want)) < 2e-6
        assert 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real < 1e-10
