"""Runs of diagonal blocks applied as one phase polynomial (FP32 plans) vs the
oracle and vs the per-block diagonal kernel of an FP64 plan (GPU).

Tolerance: the kernel's phases are exp(2 pi i f) with f in 2^-32 turns and a
1024-entry FP32 table times a short Taylor polynomial, so every amplitude is
rotated to within ~1e-7 relative; FP32 amplitudes of a normalised state stay
within 2e-6 of the FP64 result."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads
from tests.test_planner import diag_mix

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,kmax", [(4, 2), (9, 4), (14, 4), (20, 4)])
def test_phase_poly_plan_vs_oracle(qi, orc, n, kmax):
    gates = diag_mix(n, seed=n, layers=2)
    init = orc.execute(workloads.plus_state(n), n, workloads.random_circuit(n, 2, seed=n, with_qft=False))
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax)
    assert any(op["kind"] == 9 for op in plan.ops())
    with qi.DeviceState(n, qi.F32) as st:
        st.upload(init)
        plan.execute(st)
        got = st.download()
    assert np.max(np.abs(got - want)) < 2e-6
    # normalised infidelity: FP32 rounding of the other kernels also moves the norm by ~1e-8
    assert 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real < 1e-9


@pytest.mark.parametrize("tensor_cores", [2, 1], ids=["standalone", "in_tc_epilogue"])
@pytest.mark.parametrize("n", [23, 27])
def test_phase_poly_many_iterations_vs_per_gate(qi, n, tensor_cores):
    """n = 23 and 27: 2^5 and 2^9 iterations per thread (the iteration-bit tables
    and per-thread cross terms are exercised); compared with the per-gate FP32
    execution of the same QFT.  With CUDA-core blocks the polynomials run as their own
    pass (k_phase_poly); after a tensor-core block they ride on its epilogue."""
    gates = workloads.qft(workloads.GateList(), list(range(n))).array()
    init_gates = workloads.random_circuit(n, 1, seed=2, with_qft=False)
    fused = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6, use_tensor_cores=tensor_cores)
    ops = fused.ops()
    if tensor_cores == 2:
        assert sum(op["kind"] == 9 for op in ops) >= 2
    else:
        assert sum(op["kind"] == 4 and "poly" in op for op in ops) >= 2
    with qi.DeviceState(n, qi.F32) as a, qi.DeviceState(n, qi.F32) as b:
        for s in (a, b):
            s.set_plus()
            qi.circuit_execute(s, init_gates)
        fused.execute(a)
        qi.circuit_execute(b, gates)
        ov = a.inner_product(b)
        na, nb = a.norm_sqr(), b.norm_sqr()
    assert abs(na - 1.0) < 1e-5 and abs(nb - 1.0) < 1e-5
    assert 1 - abs(ov) ** 2 / (na * nb) < 1e-8
