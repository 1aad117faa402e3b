"""Qubit permutations on the GPU: SWAP / X runs lowered to one tiled permutation pass
(k_bitperm) and its in-place fallback, against the oracle."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu


def swap_runs_circuit(n, seed):
    rng = np.random.default_rng(seed)
    gl = workloads.GateList()
    for _ in range(3):
        for q in range(n):
            gl.add("RY", [q], [], [float(rng.uniform(0, 6.28))])
            gl.add("RZ", [q], [], [float(rng.uniform(0, 6.28))])
        for q in range(0, n - 1, 2):
            gl.add("CNOT", [q + 1], [q])
        for _ in range(int(rng.integers(3, 9))):
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            gl.add("SWAP", [a, b])
            if rng.random() < 0.3:
                gl.add("X", [int(rng.integers(0, n))])
    return gl.array()


@pytest.mark.parametrize("n", [7, 12, 18])
@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_swap_runs_plan_vs_oracle(qi, orc, n, prec):
    gates = swap_runs_circuit(n, n)
    init = workloads.plus_state(n) * np.exp(1j * np.arange(1 << n) * 0.13)
    init /= np.linalg.norm(init)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, prec, gates, fusion=qi.FUSION_GREEDY)
    assert any(op["kind"] == 11 for op in plan.ops())
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        plan.execute(st)
        got = st.download()
    assert np.max(np.abs(got - want)) < (1e-12 if prec == 0 else 2e-5)


def test_state_buffer_stays_put(qi):
    """An odd number of permutations leaves the amplitudes in the state's own buffer
    (the device pointer a caller may hold is unchanged)."""
    n = 14
    gl = workloads.GateList()
    for q in range(n):
        gl.add("H", [q])
    workloads.qft(gl, list(range(n)))
    plan = qi.Plan(n, 1, gl.array(), fusion=qi.FUSION_GREEDY)
    with qi.DeviceState(n, 1) as st:
        st.set_zero()
        p0 = st.device_ptr()
        plan.execute(st)
        assert st.device_ptr() == p0
        plan.execute(st)
        assert st.device_ptr() == p0


def test_in_place_fallback_matches(qi):
    """With no device memory left for the second buffer, the permutation runs in place as
    SWAP / X kernels: the amplitudes equal the out-of-place result exactly (pure moves)."""
    torch = pytest.importorskip("torch")
    n = 24
    gl = workloads.GateList()
    for q in range(n):
        gl.add("RY", [q], [], [0.1 + 0.05 * q])
    for q in range(n // 2):
        gl.add("SWAP", [q, n - 1 - q])
    gl.add("X", [3])
    plan = qi.Plan(n, 1, gl.array(), fusion=qi.FUSION_GREEDY)
    assert [op["kind"] for op in plan.ops()].count(11) == 1
    with qi.DeviceState(n, 1) as a:
        a.set_plus()
        plan.execute(a)
        want = a.download()
    with qi.DeviceState(n, 1) as b:
        b.set_plus()
        free, _ = torch.cuda.mem_get_info()
        state_bytes = (1 << n) * 8
        hog = None
        if free > state_bytes // 2:
            hog = torch.empty(free - state_bytes // 2, dtype=torch.uint8, device="cuda")
        try:
            plan.execute(b)
            b.synchronize()
        finally:
            del hog
            torch.cuda.empty_cache()
        got = b.download()   # host transfers stage through device memory: after the release
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n", [16, 21])
def test_renormalisation_after_a_permutation_uses_its_norm(qi, orc, n):
    """Tensor-core blocks, then a SWAP network lowered to one permutation, then the plan's closing
    renormalisation: the permutation sums the norm as it writes and the renormalisation scales with
    it (no read pass of its own). The result matches the oracle and has unit norm."""
    rng = np.random.default_rng(n)
    gl = workloads.GateList()
    for _ in range(4):
        for q in range(n):
            gl.add("RY", [q], [], [float(rng.uniform(0, 6.28))])
            gl.add("RZ", [q], [], [float(rng.uniform(0, 6.28))])
        for q in range(n - 1):
            gl.add("CNOT", [q + 1], [q])
    for q in range(n // 2):
        gl.add("SWAP", [q, n - 1 - q])
    gates = gl.array()
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
    kinds = [op["kind"] for op in plan.ops()]
    assert kinds[-2:] == [11, 8] and any(op["kind"] == 4 and op.get("tensor_cores") for op in plan.ops())
    with qi.DeviceState(n, qi.F32) as st:
        st.upload(init)
        p0 = st.device_ptr()
        plan.execute(st)
        got = st.download()
        assert st.device_ptr() == p0
        assert abs(st.norm_sqr() - 1.0) < 1e-6
    assert np.max(np.abs(got - want)) < 2e-6
    assert 1 - abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real < 1e-10
