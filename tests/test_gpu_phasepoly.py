"""Runs of diagonal blocks applied as one phase polynomial (FP32 plans) vs the
oracle and vs the per-block diagonal kernel of an FP64 plan (GPU).

Tolerance: the kernel's phases are exp(2 pi i f) with f in 2^-32 turns and a
1024-entry FP32 table times a short Taylor polynomial, so every amplitude is
rotated to within ~1e-7 relative; FP32 amplitudes of a normalised state stay
within 2e-6 of the FP64 result.  A polynomial carried by a tensor-core block's epilogue
uses the SFU's sin / cos (absolute error about 2^-21)."""
import math

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
    # CUDA-core blocks: the polynomials run as their own passes; default: a polynomial after a
    # tensor-core block (3- and 4-qubit blocks are widened to 5 qubits from 12 qubits up) rides on
    # its epilogue
    for tc in (2, 0):
        plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax, use_tensor_cores=tc)
        if tc == 2:
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


def _rev(v, n):
    return int(format(v, "0%db" % n)[::-1], 2)


def test_qft_convention_matches_oracle(orc):
    """The reference QFT (H, controlled phases, swaps) maps |x> to
    exp(2 pi i rev(x) rev(y) / 2^n) / 2^(n/2) (rev: bit reversal); pinned on the oracle."""
    n = 8
    for x in (0b10110011, 1, 6):
        out = orc.execute(workloads.basis_state(n, x), n, workloads.qft(workloads.GateList(), list(range(n))).array())
        y = np.arange(1 << n)
        want = np.exp(2j * np.pi * _rev(x, n) * np.array([_rev(int(v), n) for v in y]) / (1 << n)) / np.sqrt(1 << n)
        assert np.max(np.abs(out - want)) < 1e-12


@pytest.mark.parametrize("n", [33, 34])
def test_qft_largest_states_vs_analytic(qi, n):
    """2^33 and 2^34 FP32 amplitudes (64 / 128 GiB): at 33 qubits (2^20 tiles) the phase
    polynomials ride on the tensor-core epilogues (phase tables); at 34 they run as their
    own passes.  Sampled amplitudes of QFT|x> against the closed form; the norm stays 1."""
    gates = workloads.qft(workloads.GateList(), list(range(n))).array()
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
    ops = plan.ops()
    if n == 33:
        assert sum(op["kind"] == 4 and "poly" in op for op in ops) >= 2
    else:
        assert sum(op["kind"] == 9 for op in ops) >= 2
    x = 0x1D2C3B4A5 & ((1 << n) - 1)
    rng = np.random.default_rng(n)
    ys = [int(v) for v in rng.integers(0, 1 << n, size=24)] + [0, (1 << n) - 1]
    with qi.DeviceState(n, qi.F32) as st:
        st.set_basis(x)
        plan.execute(st)
        assert abs(st.norm_sqr() - 1.0) < 1e-5
        got = np.array([st.amplitude(y) for y in ys]) * math.sqrt(1 << n)
    rx = _rev(x, n)
    want = np.array([np.exp(2j * np.pi * ((rx * _rev(y, n)) % (1 << n)) / (1 << n)) for y in ys])
    assert np.max(np.abs(got - want)) < 2e-4
