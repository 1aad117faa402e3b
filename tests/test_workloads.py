"""Shapes of the benchmark workloads (no GPU)."""
import numpy as np

from quant_iron_gb300 import workloads


def test_random_circuit_gate_counts():
    assert len(workloads.random_circuit(20, 40, seed=0)) == 1400   # 800 1q + 380 CNOT + 220 QFT
    assert len(workloads.random_circuit(30, 40, seed=0)) == 2260   # 1200 1q + 580 CNOT + 480 QFT


def test_random_circuit_is_seeded():
    a = workloads.random_circuit(12, 5, seed=7)
    b = workloads.random_circuit(12, 5, seed=7)
    c = workloads.random_circuit(12, 5, seed=8)
    assert a.tobytes() == b.tobytes()
    assert a.tobytes() != c.tobytes()


def test_hamiltonian_term_counts():
    assert len(workloads.heisenberg_open_chain(20, seed=0)) == 77
    assert len(workloads.lattice_xyz(5, 6, seed=0)) == 177
    assert len(workloads.lattice_tfim(5, 6, seed=0)) == 79
    assert len(workloads.xxz_periodic(26, seed=1)) == 104


def test_ansatz_shape():
    gates, theta = workloads.hea_ansatz(26, 12, seed=1)
    assert len(gates) == 12 * (26 * 2 + 25) == 924
    assert theta.size == 624
    assert np.all(np.abs(theta) <= np.pi)
    ids = gates["param_ids"][:, 0]
    assert sorted(ids[ids >= 0].tolist()) == list(range(624))
