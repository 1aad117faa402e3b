"""Circuits holding Gate::Measurement (gate.rs:19, :104-106) run through the engine's plan on
the GPU, against the oracle's gate loop with the same seeds: the collapsed state (and so the
drawn outcome) must agree, per gate in FP64 and fused in FP32, in every basis."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads
from tests.test_measure_gate import circuit_with_measurements

pytestmark = pytest.mark.gpu

U = np.array([[np.cos(0.3), -np.sin(0.3) * np.exp(-0.4j)], [np.sin(0.3), np.cos(0.3) * np.exp(-0.4j)]])


@pytest.mark.parametrize("basis", [0, 1, 2, 3], ids=["computational", "x", "y", "custom"])
@pytest.mark.parametrize("prec,fusion,tol", [(0, 0, 1e-12), (1, 1, 2e-6)], ids=["f64_per_gate", "f32_fused"])
def test_mid_circuit_measurement_matches_oracle(qi, orc, basis, prec, fusion, tol):
    n = 12
    for seed in range(3):
        _, _, gates = circuit_with_measurements(n, seed=seed, basis=basis, custom=U if basis == 3 else None)
        init = workloads.plus_state(n)
        want = orc.execute(init, n, gates)
        with qi.DeviceState(n, prec) as st:
            st.upload(init)
            qi.circuit_execute(st, gates, fusion=fusion, max_block_qubits=6)
            got = st.download()
        assert np.max(np.abs(got - want)) < tol, (basis, seed)


def test_mirror_gate_measurement(qi, orc):
    from quant_iron_gb300 import quant_iron as q
    n = 6
    st = q.State.new_plus(n)
    c = q.Circuit([q.Gate.operator(q.Hadamard(), [0]), q.Gate.new_measurement([0, 2], q.MeasurementBasis.X, seed=5),
                   q.Gate.operator(q.RotateY(0.7), [2])], n)
    got = c.execute(st).state_vector
    want = orc.execute(workloads.plus_state(n), n, c.gate_array())
    assert np.max(np.abs(got - want)) < 1e-12
