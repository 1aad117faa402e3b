"""Seeded random circuits through the fused FP32 plans (window partition, tensor-core
blocks in every mode, phase polynomials standalone and on the tensor-core epilogues)
and the FP64 grouped exponentials, against the FP64 oracle."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu

KINDS_1Q = ["H", "X", "Y", "Z", "S", "T", "SDAG", "TDAG", "RX", "RY", "RZ", "P"]


def random_gates(n, count, rng):
    gl = workloads.GateList()
    for _ in range(count):
        r = rng.random()
        if r < 0.55:
            k = KINDS_1Q[int(rng.integers(0, len(KINDS_1Q)))]
            q = int(rng.integers(0, n))
            params = [float(rng.uniform(-3, 3))] if k in ("RX", "RY", "RZ", "P") else []
            gl.add(k, [q], [], params)
        elif r < 0.75:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gl.add("CNOT", [b], [a])
        elif r < 0.85:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gl.add("P", [b], [a], [float(rng.uniform(-3, 3))])   # controlled phase (diagonal)
        elif r < 0.92:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gl.add("SWAP", [a, b])
        else:
            a = int(rng.integers(0, n - 1))
            gl.add("MATCHGATE", [a], [], [float(rng.uniform(-3, 3)), 0.4, 0.4])
    return gl


@pytest.mark.parametrize("seed", range(10))
def test_fused_fp32_random_circuits(qi, orc, seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(13, 19))
    gl = random_gates(n, int(rng.integers(60, 220)), rng)
    lo = int(rng.integers(0, n - 6))
    workloads.qft(gl, list(range(lo, lo + int(rng.integers(4, n - lo + 1)))))   # diagonal ladders
    gates = gl.array()
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init = v / np.linalg.norm(v)
    want = orc.execute(init, n, gates)
    for tc in (1, 2):
        plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6, use_tensor_cores=tc)
        with qi.DeviceState(n, qi.F32) as st:
            st.upload(init)
            plan.execute(st)
            got = st.download()
        infid = 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real
        assert np.max(np.abs(got - want)) < 3e-5 and infid < 1e-8, (seed, n, tc, infid)


@pytest.mark.parametrize("seed", range(4))
def test_fp64_grouped_random_trotter(qi, orc, seed):
    rng = np.random.default_rng(2000 + seed)
    n = int(rng.integers(9, 14))
    out = []
    for _ in range(int(rng.integers(20, 60))):
        w = int(rng.integers(1, 4))
        qs = rng.choice(n, w, replace=False)
        out.append(workloads.term(float(rng.normal()), [(int(q), "XYZ"[int(rng.integers(0, 3))]) for q in qs]))
    terms = workloads.terms_array(out)
    init = workloads.plus_state(n)
    for order in (1, 2):
        want = orc.trotter(init, n, terms, 0.07, 3, order)
        with qi.DeviceState(n, qi.F64) as st:
            st.upload(init)
            qi.trotter_evolve(st, terms, 0.07, 3, order=order)
            got = st.download()
        assert np.max(np.abs(got - want)) < 1e-11, (seed, n, order)
