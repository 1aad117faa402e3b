"""Gate::Measurement inside a circuit (gate.rs:19, :104-106), checked without a GPU: the
oracle's gate loop against its own measure call, and the plan's placement of the
measurement as a barrier (a fused plan's blocks never straddle it)."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads
from tests.test_planner import replay



def circuit_with_measurements(n, seed, basis=0, custom=None):
    """Random layers, a measurement of three qubits, more random layers, a second one."""
    head = workloads.random_circuit(n, layers=3, seed=seed, with_qft=False)
    tail = workloads.random_circuit(n, layers=3, seed=seed + 1, with_qft=True)
    gl = workloads.GateList()
    gl._rows = list(head)
    gl.measure([3, n - 1, 1], basis=basis, custom=custom, seed=seed + 100)
    gl._rows += list(tail)
    gl.measure([0, 2], basis=0, seed=seed + 200)
    return head, tail, gl.array()


def test_oracle_gate_loop_matches_measure_call(qi, orc):
    n = 8
    head, tail, gates = circuit_with_measurements(n, seed=4)
    init = workloads.plus_state(n)
    got = orc.execute(init, n, gates)
    s = orc.execute(init, n, head)
    _, s, _ = orc.measure(s, n, [3, n - 1, 1], qi.splitmix_uniform(104))
    s = orc.execute(s, n, tail)
    _, s, _ = orc.measure(s, n, [0, 2], qi.splitmix_uniform(204))
    assert np.array_equal(got, s)


@pytest.mark.parametrize("fusion", [0, 1])
def test_plan_keeps_measurement_as_barrier(qi, orc, fusion):
    n = 10
    _, _, gates = circuit_with_measurements(n, seed=9)
    plan = qi.Plan(n, qi.F32, gates, fusion=fusion, max_block_qubits=5)
    ops = plan.ops()
    kinds = [op["kind"] for op in ops]
    assert kinds.count(12) == 2
    m0 = kinds.index(12)
    assert ops[m0]["targets"][:3] == [3, n - 1, 1] and ops[m0]["k"] == 3
    # the ops before the first measurement reproduce exactly the gates before it
    head_len = 3 * n + sum(1 for layer in range(3) for j in range(n) if 2 * j + 1 + layer % 2 < n)
    init = workloads.plus_state(n)
    before = replay(ops[:m0], n, init)
    want = orc.execute(init, n, gates[:head_len])
    assert np.max(np.abs(before / np.linalg.norm(before) - want)) < 1e-12


def test_measurement_gate_validation(qi):
    n = 4
    bad = workloads.GateList().measure([5], seed=1).array()
    with pytest.raises(qi.QuantIronError) as ei:
        qi.Plan(n, qi.F64, bad)
    assert ei.value.variant == "InvalidQubitIndex"
    bad = workloads.GateList().measure([0, 1, 2, 3, 0], seed=1).array()
    with pytest.raises(qi.QuantIronError) as ei:
        qi.Plan(n, qi.F64, bad)
    assert ei.value.variant == "InvalidNumberOfQubits"
    bad = workloads.GateList().measure([0], basis=7).array()
    with pytest.raises(qi.QuantIronError) as ei:
        qi.Plan(n, qi.F64, bad)
    assert ei.value.variant == "InvalidInputValue"


def test_adjoint_rejects_measurement(qi):
    gates, theta = workloads.hea_ansatz(4, 1, seed=1)
    gl = workloads.GateList()
    gl._rows = list(gates)
    gl.measure([0], seed=3)
    with pytest.raises(qi.QuantIronError) as ei:
        qi.adjoint_sweep_plan(4, qi.F32, gl.array(), theta)
    assert ei.value.variant == "Unsupported"
