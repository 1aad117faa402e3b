"""The FP32 restatement of the reference's OpenCL kernels (oracle/opencl_f32.py), on the CPU:
pinned to the reference test-suite's known answers (the 15-qubit cases run the GPU path
in the reference), and checked against the FP64 CPU restatement kernel by kernel."""
import math

import numpy as np
import pytest

from oracle import opencl_f32 as ocl
from quant_iron_gb300 import workloads
from tests.golden import known_answers as ka

F32_EPS = float(np.finfo(np.float32).eps)


@pytest.mark.parametrize("case", ka.GATE_CASES, ids=[c[0] for c in ka.GATE_CASES])
def test_known_answers(case):
    name, cite, n, init, gates, expected = case
    got = ocl.execute(init, n, gates)
    # PartialEq for State: per-component |diff| < f32::EPSILON (state.rs:2348-2372)
    assert np.all(np.abs(got.real - expected.real) < F32_EPS) and np.all(np.abs(got.imag - expected.imag) < F32_EPS), \
        (name, cite)


def _rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


KERNEL_GATES = [("H", [3], [], []), ("H", [14], [2, 9], []), ("X", [0], [], []), ("Y", [7], [1], []),
                ("Z", [5], [], []), ("S", [2], [], []), ("SDAG", [11], [4], []), ("T", [6], [], []),
                ("TDAG", [13], [], []), ("P", [9], [0], [0.731]), ("RX", [4], [], [1.234]),
                ("RY", [12], [3], [-2.2]), ("RZ", [1], [], [0.4]), ("CNOT", [8], [2], []),
                ("TOFFOLI", [10], [0, 14], []), ("SWAP", [3, 12], [], []), ("SWAP", [0, 1], [6], []),
                ("MATCHGATE", [5], [], [1.1, 0.7, 0.7]), ("U2", [2], [], [0.6, 0.0, 0.8, 0.0, -0.8, 0.0, 0.6, 0.0]),
                ("IDENTITY", [9], [], [])]


@pytest.mark.parametrize("kind,targets,controls,params", KERNEL_GATES,
                         ids=["%s%s%s" % (k, t, c) for k, t, c, _ in KERNEL_GATES])
def test_kernels_agree_with_fp64_branch(orc, kind, targets, controls, params):
    """At 15 qubits every kernel equals the FP64 CPU branch to FP32 rounding (matchgate
    with phi1 == phi2, where its kernel and the CPU branch coincide)."""
    n = 15
    v = _rand_state(n, 7)
    gate = workloads.GateList().add(kind, targets, controls, params).array()[0]
    want = orc.apply_gate(v, n, gate)
    got = ocl.apply_gate(v, n, gate)
    assert np.max(np.abs(got - want)) < 4 * F32_EPS * np.max(np.abs(v))


def test_matchgate_kernel_uses_phi2_where_the_cpu_branch_uses_phi1(orc):
    """match_gate.cl multiplies the a10 term of new_a10 by e^{i phi2}; operator.rs:962-963
    uses e^{i phi1}.  With phi1 != phi2 the two paths differ in the a10 amplitudes; at
    theta = pi (cos = 0, as in operator_tests.rs) the difference vanishes."""
    n = 15
    v = _rand_state(n, 8)
    q = 4
    g = workloads.GateList().add("MATCHGATE", [q], [], [1.1, 0.3, 1.9]).array()[0]
    cpu, gpu = orc.apply_gate(v, n, g), ocl.apply_gate(v, n, g)
    idx = np.arange(1 << n)
    i10 = idx[((idx >> q) & 1 == 0) & ((idx >> (q + 1)) & 1 == 1)]
    others = np.setdiff1d(idx, i10)
    assert np.max(np.abs(gpu[i10] - cpu[i10])) > 1e-3
    assert np.max(np.abs(gpu[others] - cpu[others])) < 4 * F32_EPS
    c, s = math.cos(1.1 / 2), math.sin(1.1 / 2)
    want10 = s * v[i10 ^ (1 << q) ^ (1 << (q + 1))] + np.exp(1j * 1.9) * c * v[i10]
    assert np.max(np.abs(gpu[i10] - want10)) < 4 * F32_EPS
    g_pi = workloads.GateList().add("MATCHGATE", [q], [], [math.pi, 0.3, 1.9]).array()[0]
    assert np.max(np.abs(ocl.apply_gate(v, n, g_pi) - orc.apply_gate(v, n, g_pi))) < 4 * F32_EPS


def test_below_threshold_runs_the_fp64_branch(orc):
    n = 14
    v = _rand_state(n, 9)
    gates = workloads.random_circuit(n, layers=2, seed=3, with_qft=False)
    assert np.array_equal(ocl.execute(v, n, gates), orc.execute(v, n, gates))
