"""The CPU oracle against the reference test-suite's known answers (no GPU)."""
import numpy as np
import pytest

from tests.golden import known_answers as ka


@pytest.mark.parametrize("case", ka.GATE_CASES, ids=[c[0] for c in ka.GATE_CASES])
def test_gate_known_answer(orc, case):
    name, cite, n, init, gates, expected = case
    s = orc.execute(init, n, np.stack(gates))
    assert np.all(np.abs(s.real - expected.real) < ka.F32_EPS), (name, cite)
    assert np.all(np.abs(s.imag - expected.imag) < ka.F32_EPS), (name, cite)


@pytest.mark.parametrize("case", ka.ERROR_CASES, ids=[c[0] for c in ka.ERROR_CASES])
def test_gate_error_variant(orc, case):
    from quant_iron_gb300._abi import STATUS_NAMES
    name, cite, n, row, variant, (a, b) = case
    with pytest.raises(orc.OracleError) as ei:
        orc.apply_gate(ka.zero(n), n, row)
    assert STATUS_NAMES[ei.value.code] == variant, (name, cite)
    assert ei.value.a == a, (name, cite)
    if b != -1:
        assert ei.value.b == b, (name, cite)


@pytest.mark.parametrize("case", ka.PAULI_CASES, ids=[c[0] for c in ka.PAULI_CASES])
def test_pauli_known_answer(orc, case):
    name, cite, n, init, op, payload, expected = case
    if op == "expectation":
        got = orc.sumop_expectation(init, n, payload)
        assert abs(got - expected) < 1e-12, (name, cite)
        return
    if op == "sumop_apply":
        got = orc.sumop_apply(init, n, payload)
    elif op == "apply":
        got = orc.pauli_apply(init, n, payload)
    elif op == "exp":
        got = orc.pauli_apply_exp_factor(init, n, payload, 1.0)
    elif op == "exp_factor":
        got = orc.pauli_apply_exp_factor(init, n, payload[0], payload[1])
    elif op == "exp_neg_i_dt":
        t, dt = payload
        got = orc.pauli_apply_exp_factor(init, n, t, complex(0.0, -dt))
    else:
        raise AssertionError(op)
    assert np.max(np.abs(got - expected)) < ka.F32_EPS, (name, cite)


def test_pauli_time_evolution_gate(orc):
    # Gate::PauliTimeEvolution on |00> equals the exp_neg_i_dt vector (gate_tests.rs:124-186)
    got = orc.execute(ka.zero(2), 2, np.stack([ka.TE_GATE]))
    want = ka.R2 * ka.basis(2, 0) - 1j * ka.R2 * ka.basis(2, 2)
    assert np.max(np.abs(got - want)) < ka.F32_EPS


def test_trotter_first_order_composition(orc):
    # time_evolution_tests.rs:14-41: one first-order step equals the manual chain of
    # apply_exp_factor(-i dt) over the terms in order.
    from quant_iron_gb300.workloads import term, terms_array
    terms = terms_array([term(0.7, [(0, "X"), (1, "X")]), term(-0.4, [(1, "Z")]), term(0.2, [(0, "Y")])])
    init = ka.plus(2)
    step = orc.trotter(init, 2, terms, 0.1, 1, 1)
    manual = init.copy()
    for t in terms:
        manual = orc.pauli_apply_exp_factor(manual, 2, t, -0.1j)
    assert np.max(np.abs(step - manual)) == 0.0


def test_trotter_second_order_composition(orc):
    # time_evolution_tests.rs:80-108: forward half steps then reversed half steps.
    from quant_iron_gb300.workloads import term, terms_array
    terms = terms_array([term(0.7, [(0, "X"), (1, "X")]), term(-0.4, [(1, "Z")]), term(0.2, [(0, "Y")])])
    init = ka.plus(2)
    step = orc.trotter(init, 2, terms, 0.1, 1, 2)
    manual = init.copy()
    for t in list(terms) + list(terms[::-1]):
        manual = orc.pauli_apply_exp_factor(manual, 2, t, -0.05j)
    assert np.max(np.abs(step - manual)) == 0.0


def test_trotter_empty_hamiltonian_error(orc):
    # time_evolution_tests.rs:43-58 -> InvalidNumberOfQubits(0)
    from quant_iron_gb300.workloads import terms_array
    with pytest.raises(orc.OracleError) as ei:
        orc.trotter(ka.plus(2), 2, terms_array([]), 0.1, 1, 1)
    assert ei.value.code == -3 and ei.value.a == 0


def test_fidelity_and_distance(orc):
    # state_tests.rs:225-296: fs_dist(|0>,|+>) = pi/4, fs_fidelity(|0>,|+>) = 0.5
    ip = orc.inner_product(ka.zero(1), ka.plus(1), 1)
    assert abs(np.arccos(abs(ip)) - np.pi / 4) < 1e-12
    assert abs(abs(ip) ** 2 - 0.5) < 1e-12


def test_tensor_product_and_normalise(orc):
    # state_tests.rs:149-212
    tp = orc.tensor_product(ka.plus(1), 1, ka.basis(1, 1), 1)
    assert np.allclose(tp, np.kron(ka.plus(1), ka.basis(1, 1)))
    v = np.array([3.0, 4.0j])
    assert np.allclose(orc.normalise(v, 1), v / 5.0)
    with pytest.raises(orc.OracleError) as ei:
        orc.normalise(np.zeros(2, dtype=complex), 1)
    assert ei.value.code == -14   # ZeroNorm


def test_unitary2_check(orc):
    assert orc.unitary2_check([0, 0, 1, 0, 1, 0, 0, 0]) == 0
    assert orc.unitary2_check([1, 0, 1, 0, 0, 0, 1, 0]) == -6   # NonUnitaryMatrix


def test_measurement_collapse(orc):
    # measurement_tests.rs:119-151: the collapsed state matches the drawn outcome.
    st = ka.kron(ka.plus(1), ka.basis(1, 1))
    for r in (0.1, 0.9):
        out, post, probs = orc.measure(st, 2, [1], r)
        assert np.allclose(probs, [0.5, 0.5])
        assert out == (0 if r < 0.5 else 1)
        assert np.allclose(post, ka.basis(2, 1 | (out << 1)))


def test_random_circuit_norm(orc):
    from quant_iron_gb300 import workloads
    n = 10
    s = orc.execute(workloads.plus_state(n), n, workloads.random_circuit(n, layers=8, seed=3))
    assert abs(np.vdot(s, s).real - 1.0) < 1e-12
