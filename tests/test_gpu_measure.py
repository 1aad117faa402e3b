"""State::measure / measure_n on the GPU vs the oracle (state.rs:525-784).

The outcome is integer work: given the same uniform draw r the engine and the
oracle must pick the same outcome bit for bit; probabilities and the collapsed
state agree to FP64 rounding (1e-12)."""
import numpy as np
import pytest

from tests.golden import known_answers as ka

pytestmark = pytest.mark.gpu


def rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("qubits", [[3, 0, 7], [5], [], [1, 2, 3, 4, 5, 6]])
def test_computational_measure_matches_oracle(qi, orc, qubits):
    n = 9
    for seed in range(6):
        init = rand_state(n, 10 + seed)
        r = qi.splitmix_uniform(seed)
        want_o, want_state, want_p = orc.measure(init, n, qubits, r)
        with qi.DeviceState(n, 0) as st:
            st.upload(init)
            o, p = qi.measure(st, qubits, seed=seed, return_probs=True)
            got_state = st.download()
        assert o == want_o
        assert np.max(np.abs(p - want_p)) < 1e-12
        assert np.max(np.abs(got_state - want_state)) < 1e-12


def test_known_answer_collapse(qi):
    # measurement_tests.rs:119-151: |+>|1> measured on qubit 1 collapses to |o>|1>
    st_vec = ka.kron(ka.plus(1), ka.basis(1, 1))
    seen = set()
    for seed in range(12):
        with qi.DeviceState(2, 0) as st:
            st.upload(st_vec)
            o, p = qi.measure(st, [1], seed=seed, return_probs=True)
            assert np.allclose(p, [0.5, 0.5])
            assert np.allclose(st.download(), ka.basis(2, 1 | (o << 1)))
            seen.add(o)
    assert seen == {0, 1}


@pytest.mark.parametrize("basis", ["X", "Y", "Custom"])
def test_basis_measurement_matches_oracle_emulation(qi, orc, basis):
    from quant_iron_gb300.workloads import GateList
    n = 7
    qubits = [2, 5]
    u = ka.haar if hasattr(ka, "haar") else None
    th = 0.7
    U = np.array([[np.cos(th), -np.sin(th) * np.exp(0.3j)], [np.sin(th), np.cos(th) * np.exp(0.3j)]])
    Ud = U.conj().T

    def gates(kind_list, mat=None):
        gl = GateList()
        for kind in kind_list:
            for q in qubits:
                if kind == "U2":
                    gl.add("U2", [q], [], [mat[0, 0].real, mat[0, 0].imag, mat[0, 1].real, mat[0, 1].imag,
                                           mat[1, 0].real, mat[1, 0].imag, mat[1, 1].real, mat[1, 1].imag])
                else:
                    gl.add(kind, [q])
        return gl.array()
    before = {"X": gates(["H"]), "Y": gates(["SDAG", "H"]), "Custom": gates(["U2"], U)}[basis]
    after = {"X": gates(["H"]), "Y": gates(["H", "S"]), "Custom": gates(["U2"], Ud)}[basis]
    for seed in range(4):
        init = rand_state(n, seed)
        r = qi.splitmix_uniform(seed)
        o_ref, post, _ = orc.measure(orc.execute(init, n, before), n, qubits, r)
        want = orc.execute(post, n, after)
        with qi.DeviceState(n, 0) as st:
            st.upload(init)
            o = qi.measure(st, qubits, basis=basis, custom=U if basis == "Custom" else None, seed=seed)
            got = st.download()
        assert o == o_ref
        assert np.max(np.abs(got - want)) < 1e-12


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_measure_n_leaves_state_and_matches_cdf(qi, orc, prec):
    n = 10
    qubits = [0, 4, 9]
    init = rand_state(n, 3)
    _, _, p_ref = orc.measure(init, n, qubits, 0.5)
    cdf = np.cumsum(p_ref)
    shots = 2000
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        before = st.download()
        outs = qi.measure_n(st, shots, qubits, seed=77)
        after = st.download()
    assert np.max(np.abs(after - before)) < (1e-12 if prec == 0 else 2e-6)
    want = np.array([min(np.searchsorted(cdf, qi.splitmix_uniform(77 + j), side="right"), len(cdf) - 1)
                     for j in range(shots)])
    if prec == 0:
        assert np.array_equal(outs.astype(np.int64), want)
    else:
        assert np.mean(outs.astype(np.int64) == want) > 0.99
    # chi-square style check of the histogram against the probabilities
    hist = np.bincount(outs.astype(np.int64), minlength=8) / shots
    assert np.max(np.abs(hist - p_ref)) < 0.05


def test_measure_errors(qi):
    with qi.DeviceState(3, 0) as st:
        st.set_plus()
        with pytest.raises(qi.QuantIronError) as ei:
            qi.measure(st, [3])
        assert ei.value.variant == "InvalidQubitIndex" and (ei.value.a, ei.value.b) == (3, 3)
        with pytest.raises(qi.QuantIronError) as ei:
            qi.measure(st, [0, 1, 2, 0])
        assert ei.value.variant == "InvalidNumberOfQubits"
        with pytest.raises(qi.QuantIronError) as ei:
            qi.measure_n(st, 0, [0])
        assert ei.value.variant == "InvalidNumberOfMeasurements"


def test_duplicate_qubits_give_zero_probability(qi):
    with qi.DeviceState(4, 0) as st:
        st.set_plus()
        o, p = qi.measure(st, [2, 2], seed=1, return_probs=True)
        assert p[1] == 0.0 and p[2] == 0.0 and abs(p[0] + p[3] - 1.0) < 1e-12
        assert o in (0, 3)


def test_measure_24q_fp32_probabilities(qi):
    n = 24
    qubits = list(range(0, 24, 2))
    with qi.DeviceState(n, 1) as s32, qi.DeviceState(n, 0) as s64:
        s32.set_plus()
        s64.set_plus()
        from quant_iron_gb300 import workloads
        g = workloads.random_circuit(n, 3, seed=4, with_qft=False)
        qi.circuit_execute(s32, g, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
        qi.circuit_execute(s64, g)
        o32, p32 = qi.measure(s32, qubits, seed=5, return_probs=True)
        o64, p64 = qi.measure(s64, qubits, seed=5, return_probs=True)
    assert abs(p32.sum() - 1.0) < 1e-9
    assert np.max(np.abs(p32 - p64)) < 1e-6


def test_mirror_state_measure(qi, orc):
    """quant_iron.State.measure / measure_n: the crate's call shapes, outcomes equal the
    oracle's for the same draw, and the measured State itself is unchanged."""
    from quant_iron_gb300 import quant_iron as q
    n, qubits = 8, [6, 1, 3]
    init = rand_state(n, 41)
    st = q.State.new(init)
    for seed in range(4):
        res = st.measure(q.MeasurementBasis.Computational, qubits, seed=seed)
        want_o, want_state, _ = orc.measure(init, n, qubits, qi.splitmix_uniform(seed))
        assert res.indices == qubits and res.basis == "Computational"
        assert res.outcomes == [(want_o >> k) & 1 for k in range(3)]
        assert np.max(np.abs(res.new_state.state_vector - want_state)) < 1e-12
    assert np.array_equal(st.state_vector, init)
    every = st.measure(q.MeasurementBasis.Computational, [], seed=3)
    assert every.indices == list(range(n)) and len(every.outcomes) == n
    shots = st.measure_n(q.MeasurementBasis.X, [2, 5], 6, seed=9)
    for j, r in enumerate(shots):
        one = st.measure(q.MeasurementBasis.X, [2, 5], seed=9 + j)
        assert r.outcomes == one.outcomes and r.new_state == one.new_state
    custom = q.MeasurementBasis.Custom([[0, 1], [1, 0]])
    assert len(st.measure_n(custom, [0], 2)) == 2
    with pytest.raises(qi.QuantIronError) as ei:
        st.measure_n(q.MeasurementBasis.Computational, [0], 0)
    assert ei.value.variant == "InvalidNumberOfMeasurements"
    with pytest.raises(qi.QuantIronError) as ei:
        st.measure(q.MeasurementBasis.Computational, [n])
    assert ei.value.variant == "InvalidQubitIndex"
