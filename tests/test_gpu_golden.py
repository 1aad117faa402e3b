"""The reference test-suite's known answers through the engine's C ABI (GPU)."""
import numpy as np
import pytest

from tests.golden import known_answers as ka

pytestmark = pytest.mark.gpu


def run_gates(qi, n, prec, init, rows):
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        for r in rows:
            st.apply_gate(r)
        return st.download()


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("case", ka.GATE_CASES, ids=[c[0] for c in ka.GATE_CASES])
def test_gate_known_answer(qi, case, prec):
    name, cite, n, init, gates, expected = case
    got = run_gates(qi, n, prec, init, gates)
    # PartialEq for State: per-component |diff| < f32::EPSILON (state.rs:2348-2372)
    assert np.all(np.abs(got.real - expected.real) < ka.F32_EPS), (name, cite)
    assert np.all(np.abs(got.imag - expected.imag) < ka.F32_EPS), (name, cite)


@pytest.mark.parametrize("case", ka.ERROR_CASES, ids=[c[0] for c in ka.ERROR_CASES])
def test_gate_error_variant(qi, case):
    name, cite, n, row, variant, (a, b) = case
    with qi.DeviceState(n, qi.F64) as st:
        st.set_zero()
        with pytest.raises(qi.QuantIronError) as ei:
            st.apply_gate(row)
        assert ei.value.variant == variant, (name, cite)
        assert ei.value.a == a, (name, cite)
        if b != -1:
            assert ei.value.b == b, (name, cite)
        # an invalid gate leaves the state untouched
        assert np.array_equal(st.download(), ka.zero(n))


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("case", ka.PAULI_CASES, ids=[c[0] for c in ka.PAULI_CASES])
def test_pauli_known_answer(qi, case, prec):
    name, cite, n, init, op, payload, expected = case
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        if op == "expectation":
            got = qi.sumop_expectation(st, payload)
            assert abs(got - expected) < 1e-6, (name, cite)
            return
        if op == "sumop_apply":
            with qi.DeviceState(n, prec) as out:
                qi.sumop_apply(out, st, payload)
                got = out.download()
        elif op == "apply":
            with qi.DeviceState(n, prec) as out:
                qi.pauli_apply(out, st, payload)
                got = out.download()
        elif op == "exp":
            qi.pauli_apply_exp(st, payload)
            got = st.download()
        elif op == "exp_factor":
            qi.pauli_apply_exp_factor(st, payload[0], payload[1])
            got = st.download()
        elif op == "exp_neg_i_dt":
            qi.pauli_apply_exp_neg_i_dt(st, payload[0], payload[1])
            got = st.download()
        else:
            raise AssertionError(op)
    assert np.max(np.abs(got - expected)) < ka.F32_EPS, (name, cite)


def test_pauli_time_evolution_gate(qi):
    with qi.DeviceState(2, qi.F64) as st:
        st.set_zero()
        qi.circuit_execute(st, np.stack([ka.TE_GATE]))
        got = st.download()
    want = ka.R2 * ka.basis(2, 0) - 1j * ka.R2 * ka.basis(2, 2)
    assert np.max(np.abs(got - want)) < ka.F32_EPS


def test_pauli_evolution_rejects_complex_coefficient(qi):
    # pauli_string.rs:282-284 -> InvalidPauliStringCoefficient
    from quant_iron_gb300.workloads import GateList
    row = GateList().add("PAULI_EVOLUTION", [], [], [1.0, 0.5, 0.1], xmask=1, zmask=0).array()
    with qi.DeviceState(1, qi.F64) as st:
        st.set_zero()
        with pytest.raises(qi.QuantIronError) as ei:
            qi.circuit_execute(st, row)
        assert ei.value.variant == "InvalidPauliStringCoefficient"
        assert ei.value.coeff == complex(1.0, 0.5)
