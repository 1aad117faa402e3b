"""CUDA engine vs the CPU oracle on seeded inputs (GPU).

Tolerances: FP64 kernels agree with the FP64 oracle to 1e-12 per amplitude
(FMA contraction is the only difference).  FP32 kernels: max |amplitude error|
<= 2e-6 after <= 300 gates and infidelity 1 - |<ref|psi>|^2 <= 1e-6 (the
headline bound)."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 2e-6


def infidelity(a, b):
    return 1.0 - abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)


def random_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def run(qi, n, prec, init, gates, fusion=0, k=0, theta=None):
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        qi.circuit_execute(st, gates, theta=theta, fusion=fusion, max_block_qubits=k)
        return st.download()


ALL_1Q = ["H", "X", "Y", "Z", "S", "T", "SDAG", "TDAG", "P", "RX", "RY", "RZ", "U2", "RYPHASE", "RYPHASE_DAG",
          "IDENTITY"]


def one_gate(kind, rng, n, ncontrols):
    qs = rng.permutation(n)
    t, cs = int(qs[0]), [int(c) for c in qs[1:1 + ncontrols]]
    gl = workloads.GateList()
    if kind == "U2":
        th, a, b, c = rng.uniform(0, 6.28, 4)
        u = np.exp(1j * a) * np.array([[np.exp(1j * b) * np.cos(th), np.exp(1j * c) * np.sin(th)],
                                       [-np.exp(-1j * c) * np.sin(th), np.exp(-1j * b) * np.cos(th)]])
        p = [u[0, 0].real, u[0, 0].imag, u[0, 1].real, u[0, 1].imag, u[1, 0].real, u[1, 0].imag, u[1, 1].real,
             u[1, 1].imag]
        gl.add(kind, [t], cs, p)
    else:
        gl.add(kind, [t], cs, list(rng.uniform(0, 6.28, 2)))
    return gl.array()


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("kind", ALL_1Q)
def test_single_qubit_gates_random_targets(qi, orc, kind, prec):
    rng = np.random.default_rng(hash(kind) % 1000)
    for n in (1, 2, 5, 9):
        init = random_state(n, n)
        for ncont in range(0, min(3, n)):
            g = one_gate(kind, rng, n, ncont)
            want = orc.execute(init, n, g)
            got = run(qi, n, prec, init, g)
            tol = F64_TOL if prec == 0 else F32_TOL
            assert np.max(np.abs(got - want)) < tol, (kind, n, ncont, g["targets"][0], g["controls"][0][:ncont])


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_two_qubit_gates_random(qi, orc, prec):
    rng = np.random.default_rng(17)
    n = 8
    init = random_state(n, 3)
    gl = workloads.GateList()
    for _ in range(40):
        a, b, c, d = [int(x) for x in rng.permutation(n)[:4]]
        gl.add("SWAP", [a, b], [c] if rng.random() < 0.5 else [])
        q = int(rng.integers(0, n - 1))
        ctrl = [x for x in [c, d] if x not in (q,)][:int(rng.integers(0, 2))]
        gl.add("MATCHGATE", [q], ctrl, list(rng.uniform(0, 6.28, 3)))
        gl.add("CNOT", [a], [b])
        gl.add("TOFFOLI", [a], [b, c])
    gates = gl.array()
    want = orc.execute(init, n, gates)
    got = run(qi, n, prec, init, gates)
    tol = F64_TOL * 10 if prec == 0 else 1e-5
    assert np.max(np.abs(got - want)) < tol


@pytest.mark.parametrize("n", [3, 7, 12, 16])
def test_random_circuit_per_gate_f64(qi, orc, n):
    gates = workloads.random_circuit(n, layers=6, seed=n)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    got = run(qi, n, 0, init, gates)
    assert np.max(np.abs(got - want)) < 1e-11


@pytest.mark.parametrize("n", [3, 7, 12, 16])
def test_random_circuit_per_gate_f32(qi, orc, n):
    gates = workloads.random_circuit(n, layers=6, seed=n)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    got = run(qi, n, 1, init, gates)
    assert np.max(np.abs(got - want)) < 1e-5
    assert infidelity(got, want) < 1e-6


@pytest.mark.parametrize("k", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("n", [6, 11, 14])
def test_random_circuit_fused(qi, orc, n, prec, k):
    if prec == 0 and k == 6:
        pytest.skip("FP64 fused blocks are limited to k <= 5")
    gates = workloads.random_circuit(n, layers=5, seed=100 + n)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    got = run(qi, n, prec, init, gates, fusion=qi.FUSION_GREEDY, k=k)
    if prec == 0:
        assert np.max(np.abs(got - want)) < 1e-11
    else:
        assert np.max(np.abs(got - want)) < 1e-5
        assert infidelity(got, want) < 1e-6


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_small_states_fused(qi, orc, n, prec):
    """Tiles smaller than a warp (2^n < 32 amplitudes): the CUDA-core block
    kernel's barriers are reached by every thread of the CTA."""
    gates = workloads.random_circuit(n, layers=4, seed=200 + n)
    init = orc.execute(workloads.plus_state(n), n, workloads.random_circuit(n, 1, seed=n, with_qft=False))
    want = orc.execute(init, n, gates)
    for k in range(1, min(n, 5) + 1):
        got = run(qi, n, prec, init, gates, fusion=qi.FUSION_GREEDY, k=k)
        assert np.max(np.abs(got - want)) < (1e-12 if prec == 0 else 2e-6), (n, k)


def test_config0_20q_full(qi, orc):
    """Config 0: 20 qubits, |+>^20, 40 layers + QFT (1400 gates), <H> of the open-chain Heisenberg."""
    n = 20
    gates = workloads.random_circuit(n, layers=40, seed=0)
    terms = workloads.heisenberg_open_chain(n, seed=0)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    e_want = orc.sumop_expectation(want, n, terms)
    for prec, fusion, tol_amp, tol_e in ((0, 0, 1e-11, 1e-10), (1, 0, 5e-6, 1e-4), (1, 1, 5e-6, 1e-4)):
        with qi.DeviceState(n, prec) as st:
            st.upload(init)
            qi.circuit_execute(st, gates, fusion=fusion, max_block_qubits=6 if prec else 5)
            e = qi.sumop_expectation(st, terms)
            got = st.download()
        assert np.max(np.abs(got - want)) < tol_amp, (prec, fusion)
        assert abs(e - e_want) < tol_e, (prec, fusion, e, e_want)
        if prec == 1:
            assert infidelity(got, want) < 1e-6


def test_parametric_theta_binding(qi, orc):
    n = 6
    gates, theta = workloads.hea_ansatz(n, layers=3, seed=4)
    init = workloads.zero_state(n)
    want = orc.execute(init, n, gates, theta=theta)
    theta2 = theta * 0.5
    want2 = orc.execute(init, n, gates, theta=theta2)
    assert np.max(np.abs(run(qi, n, 0, init, gates, theta=theta) - want)) < 1e-12
    assert np.max(np.abs(run(qi, n, 0, init, gates, theta=theta2) - want2)) < 1e-12


def test_large_state_fused_vs_per_gate(qi):
    """26 qubits: fused FP32 (k=6) against per-gate FP64 on the GPU (size-independent check)."""
    n = 26
    gates = workloads.random_circuit(n, layers=4, seed=9)
    with qi.DeviceState(n, 0) as ref, qi.DeviceState(n, 1) as f32, qi.DeviceState(n, 1) as tmp:
        ref.set_plus()
        qi.circuit_execute(ref, gates)
        f32.set_plus()
        qi.circuit_execute(f32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
        assert abs(f32.norm_sqr() - 1.0) < 1e-5
        tmp.copy_from(ref)   # FP64 -> FP32 conversion on the device
        ov = tmp.inner_product(f32)
        assert 1.0 - abs(ov) ** 2 < 1e-6
