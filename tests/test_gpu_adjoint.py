"""Adjoint gradient vs FP64 central finite differences and parameter shift (GPU).

Norm-wise relative error ||g - g_ref|| / ||g_ref|| <= 1e-6 (the benchmark spec's bound)
with an FP64 and with an FP32 state; finite differences use eps = 1e-4 in FP64 (the
oracle, or the engine's plain FP64 per-gate path at 20 and more qubits)."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu


def as_stored(v, prec):
    """`v` as an FP32 (prec 1) or FP64 (prec 0) device state holds it."""
    return v.astype(np.complex64).astype(np.complex128) if prec == 1 else v


def energy_oracle(orc, n, gates, theta, terms, init):
    return orc.sumop_expectation(orc.execute(init, n, gates, theta=theta), n, terms).real


def fd_grad(orc, n, gates, theta, terms, init, ids, eps=1e-4):
    g = np.zeros(len(ids))
    for i, j in enumerate(ids):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += eps
        tm[j] -= eps
        g[i] = (energy_oracle(orc, n, gates, tp, terms, init) - energy_oracle(orc, n, gates, tm, terms, init)) / (2 * eps)
    return g


@pytest.mark.parametrize("prec,tol", [(0, 1e-6), (1, 1e-6)], ids=["f64", "f32"])
def test_hea_gradient_vs_finite_differences(qi, orc, prec, tol):
    n = 8
    gates, theta = workloads.hea_ansatz(n, layers=3, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    init = workloads.zero_state(n)
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        e, g = qi.adjoint_gradient(st, gates, theta, terms)
        back = st.download()
    e_ref = energy_oracle(orc, n, gates, theta, terms, init)
    assert abs(e - e_ref) < (1e-12 if prec == 0 else 1e-5)
    ids = list(range(theta.size))
    g_ref = fd_grad(orc, n, gates, theta, terms, init, ids)
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel < tol, rel
    # the caller's state is untouched (the sweep runs on a copy)
    assert np.array_equal(back, as_stored(init, prec))


def test_parameter_shift_rotations(qi, orc):
    """RY/RZ: dE/dtheta = (E(theta + pi/2) - E(theta - pi/2)) / 2 exactly."""
    n = 7
    gates, theta = workloads.hea_ansatz(n, layers=2, seed=3)
    terms = workloads.heisenberg_open_chain(n, seed=2)
    init = workloads.zero_state(n)
    with qi.DeviceState(n, 0) as st:
        st.upload(init)
        _, g = qi.adjoint_gradient(st, gates, theta, terms)
    rng = np.random.default_rng(0)
    for j in rng.choice(theta.size, 8, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += np.pi / 2
        tm[j] -= np.pi / 2
        ps = (energy_oracle(orc, n, gates, tp, terms, init) - energy_oracle(orc, n, gates, tm, terms, init)) / 2
        assert abs(g[j] - ps) < 1e-10


def test_controlled_and_two_parameter_gates(qi, orc):
    n = 6
    gl = workloads.GateList()
    rng = np.random.default_rng(7)
    theta = rng.uniform(-3, 3, size=10)
    gl.add("H", [0]).add("H", [3])
    gl.add("RX", [1], [0], [0.0], [0])
    gl.add("RYPHASE", [2], [], [0.0, 0.0], [1, 2])
    gl.add("CNOT", [3], [2])
    gl.add("P", [4], [3, 1], [0.0], [3])
    gl.add("MATCHGATE", [4], [], [0.0, 0.0, 0.0], [4, 5, 6])
    gl.add("RYPHASE_DAG", [0], [5], [0.0, 0.0], [7, 8])
    gl.add("RZ", [5], [], [0.0], [9])
    gl.add("RX", [2], [], [0.0], [0])   # parameter 0 used twice
    gates = gl.array()
    terms = workloads.heisenberg_open_chain(n, seed=4)
    init = workloads.plus_state(n)
    with qi.DeviceState(n, 0) as st:
        st.upload(init)
        _, g = qi.adjoint_gradient(st, gates, theta, terms)
    g_ref = fd_grad(orc, n, gates, theta, terms, init, list(range(theta.size)))
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-7


def test_adjoint_rejects_non_differentiable(qi):
    gl = workloads.GateList().add("H", [0], [], [], [0])
    with qi.DeviceState(2, 0) as st:
        st.set_zero()
        with pytest.raises(qi.QuantIronError) as ei:
            qi.adjoint_gradient(st, gl.array(), np.zeros(1), workloads.heisenberg_open_chain(2))
        assert ei.value.variant == "Unsupported"


def test_adjoint_26q_fp32_vs_fp64_gpu(qi):
    """Config-3 shape (26 qubits, 12 layers, 624 parameters): FP32 adjoint vs FP64 adjoint
    on the GPU (norm-wise relative difference), and a finite-difference spot check in FP64."""
    n = 26
    gates, theta = workloads.hea_ansatz(n, layers=12, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    grads = {}
    for prec in (0, 1):
        with qi.DeviceState(n, prec) as st:
            st.set_zero()
            e, g = qi.adjoint_gradient(st, gates, theta, terms)
            grads[prec] = (e, g)
    rel = np.linalg.norm(grads[1][1] - grads[0][1]) / np.linalg.norm(grads[0][1])
    assert rel < 1e-6, rel
    assert abs(grads[1][0] - grads[0][0]) < 1e-6


def gpu_fd_grad(qi, n, gates, theta, terms, eps=1e-4):
    """FP64 central differences of E on every parameter with the plain FP64 per-gate path."""
    g = np.zeros(theta.size)
    with qi.DeviceState(n, 0) as st:
        for j in range(theta.size):
            e = []
            for sgn in (1.0, -1.0):
                th = theta.copy()
                th[j] += sgn * eps
                st.set_zero()
                qi.Plan(n, 0, gates, theta=th, fusion=qi.FUSION_NONE).execute(st)
                e.append(qi.sumop_expectation(st, terms).real)
            g[j] = (e[0] - e[1]) / (2 * eps)
    return g


def test_hea20_fp32_adjoint_within_1e6_of_finite_differences(qi):
    """20 qubits, 12 layers (480 parameters), periodic XXZ: the FP32-state adjoint gradient
    within 1e-6 (norm-wise) of FP64 central differences on all parameters, and the
    FP64-state adjoint within 1e-8; calling twice on the same state gives the same result."""
    n = 20
    gates, theta = workloads.hea_ansatz(n, layers=12, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    g_fd = gpu_fd_grad(qi, n, gates, theta, terms)
    out = {}
    for prec in (0, 1):
        with qi.DeviceState(n, prec) as st:
            st.set_zero()
            out[prec] = qi.adjoint_gradient(st, gates, theta, terms)[1]
            again = qi.adjoint_gradient(st, gates, theta, terms)[1]
            assert np.array_equal(again, out[prec])
    rel64 = np.linalg.norm(out[0] - g_fd) / np.linalg.norm(g_fd)
    rel32 = np.linalg.norm(out[1] - g_fd) / np.linalg.norm(g_fd)
    assert rel64 < 1e-8, rel64
    assert rel32 < 1e-6, rel32


def grouped_sweep_circuit(n, n_runs, seed):
    """Alternating runs for the reverse sweep's three paths: single-qubit runs (parametric
    and fixed gates, one to three gates on the same qubit in a row, so groups split on a
    fifth qubit and on a third gate per qubit), fixed runs (CNOT, SWAP, Toffoli, H, Pauli
    evolutions) un-applied as one fused plan, and lone controlled or two-parameter gates
    on the per-gate path.  Parameter ids are shared now and then."""
    rng = np.random.default_rng(seed)
    gl = workloads.GateList()
    npar = 0
    for _ in range(n_runs):
        for _ in range(int(rng.integers(3, 12))):
            q = int(rng.integers(0, n))
            for _ in range(int(rng.integers(1, 4))):
                kind = str(rng.choice(["RX", "RY", "RZ", "P", "H", "T", "SDAG"]))
                if kind in workloads.PARAMETRIC:
                    pid = npar if rng.random() < 0.85 or npar == 0 else int(rng.integers(0, npar))
                    npar = max(npar, pid + 1)
                    gl.add(kind, [q], [], [0.0], [pid])
                else:
                    gl.add(kind, [q])
        for _ in range(int(rng.integers(2, 8))):
            r = rng.random()
            a, b, c = (int(x) for x in rng.choice(n, 3, replace=False))
            if r < 0.4:
                gl.add("CNOT", [b], [a])
            elif r < 0.55:
                gl.add("SWAP", [a, b])
            elif r < 0.65:
                gl.add("TOFFOLI", [c], [a, b])
            elif r < 0.8:
                gl.add("H", [a])
            else:
                gl.add("PAULI_EVOLUTION", [], [], [rng.uniform(-1, 1), 0.0, 0.3], xmask=(1 << a) | (1 << b),
                       zmask=(1 << b) | (1 << c))
        if rng.random() < 0.5:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            gl.add("RY", [a], [b], [0.0], [npar])
            npar += 1
        else:
            gl.add("RYPHASE", [int(rng.integers(0, n))], [], [0.0, 0.0], [npar, npar + 1])
            npar += 2
    theta = rng.uniform(-np.pi, np.pi, size=npar)
    return gl.array(), theta


@pytest.mark.parametrize("n", [9, 12])
def test_grouped_reverse_sweep_vs_per_gate_and_fd(qi, orc, n):
    """Single-qubit groups and fused fixed runs in the reverse sweep: FP64 gradients equal
    the per-gate sweep (fusion off) to 1e-10, match FP64 finite differences of the oracle
    to 1e-6 on a seeded subset, FP32 stays within 1e-5 of FP64 (these circuits carry controlled
    and fixed gates whose FP32 rounding the sweep does not divide out), and the caller's
    state is left as it was."""
    gates, theta = grouped_sweep_circuit(n, 6, seed=n)
    terms = workloads.xxz_periodic(n, seed=2)
    init = workloads.plus_state(n)
    res = {}
    for prec, fusion in ((0, qi.FUSION_NONE), (0, qi.FUSION_GREEDY), (1, qi.FUSION_GREEDY)):
        with qi.DeviceState(n, prec) as st:
            st.upload(init)
            e, g = qi.adjoint_gradient(st, gates, theta, terms, fusion=fusion)
            back = st.download()
        assert np.array_equal(back, as_stored(init, prec))
        res[(prec, fusion)] = (e, g)
    g_none, g64 = res[(0, qi.FUSION_NONE)][1], res[(0, qi.FUSION_GREEDY)][1]
    assert np.linalg.norm(g64 - g_none) / np.linalg.norm(g_none) < 1e-10
    g32 = res[(1, qi.FUSION_GREEDY)][1]
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-5
    rng = np.random.default_rng(5)
    ids = sorted(int(x) for x in rng.choice(theta.size, min(12, theta.size), replace=False))
    g_ref = fd_grad(orc, n, gates, theta, terms, init, ids)
    assert np.linalg.norm(g64[ids] - g_ref) / np.linalg.norm(g_ref) < 1e-6


@pytest.mark.parametrize("layers", [1, 2, 3])
@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_permutation_runs_in_reverse_sweep(qi, orc, layers, prec):
    """Runs of X / CNOT / SWAP / singly-controlled X between rotation layers are un-applied
    as one index permutation per state (psi and lambda move between three buffers; an odd
    number of runs leaves psi in another buffer): gradients equal the per-gate sweep and the
    caller's state is left as it was."""
    n = 11
    rng = np.random.default_rng(layers)
    gl = workloads.GateList()
    npar = 0
    for _ in range(layers):
        for q in range(n):
            gl.add("RY", [q], [], [0.0], [npar])
            gl.add("RZ", [q], [], [0.0], [npar + 1])
            npar += 2
        for q in range(n - 1):
            gl.add("CNOT", [q + 1], [q])
        gl.add("SWAP", [0, n - 1])
        gl.add("X", [3])
        gl.add("X", [5], [2])
        gl.add("CNOT", [0], [n - 1])
    theta = rng.uniform(-np.pi, np.pi, size=npar)
    terms = workloads.xxz_periodic(n, seed=4)
    init = workloads.plus_state(n)
    res = {}
    for fusion in (qi.FUSION_NONE, qi.FUSION_GREEDY):
        with qi.DeviceState(n, prec) as st:
            st.upload(init)
            e, g = qi.adjoint_gradient(st, gates=gl.array(), theta=theta, terms=terms, fusion=fusion)
            back = st.download()
        assert np.array_equal(back, as_stored(init, prec))
        res[fusion] = (e, g)
    (e0, g0), (e1, g1) = res[qi.FUSION_NONE], res[qi.FUSION_GREEDY]
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < (1e-10 if prec == 0 else 1e-5)
    if prec == 0:
        e_ref = energy_oracle(orc, n, gl.array(), theta, terms, init)
        assert abs(e1 - e_ref) < 1e-12
        ids = list(range(0, npar, 7))
        g_ref = fd_grad(orc, n, gl.array(), theta, terms, init, ids)
        assert np.linalg.norm(g1[ids] - g_ref) / np.linalg.norm(g_ref) < 1e-6


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_pauli_exponential_inside_a_cnot_swap_run(qi, orc, prec):
    """A fixed run of CNOT / SWAP gates with a Pauli exponential inside is un-applied as a
    fused plan (an index permutation would drop the exponential): gradients equal the
    per-gate sweep and FP64 finite differences."""
    n = 8
    gl = workloads.GateList()
    npar = 0
    for rep in range(2):
        for q in range(n):
            gl.add("RY", [q], [], [0.0], [npar])
            npar += 1
        gl.add("CNOT", [1], [0]).add("SWAP", [2, 6])
        gl.add("PAULI_EVOLUTION", [], [], [0.7, 0.0, 0.3 + rep], xmask=0b1010, zmask=0b0110)
        gl.add("CNOT", [5], [4]).add("SWAP", [3, 7])
    gates = gl.array()
    theta = np.linspace(-1.2, 1.4, npar)
    assert any(k == qi.SWEEP_PLAN for k, _, _ in qi.adjoint_sweep_plan(n, prec, gates, theta))
    terms = workloads.xxz_periodic(n, seed=5)
    init = workloads.plus_state(n)
    res = {}
    for fusion in (qi.FUSION_NONE, qi.FUSION_GREEDY):
        with qi.DeviceState(n, prec) as st:
            st.upload(init)
            res[fusion] = qi.adjoint_gradient(st, gates, theta, terms, fusion=fusion)[1]
    g0, g1 = res[qi.FUSION_NONE], res[qi.FUSION_GREEDY]
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < (1e-10 if prec == 0 else 1e-5)
    if prec == 0:
        ids = list(range(npar))
        g_ref = fd_grad(orc, n, gates, theta, terms, init, ids)
        assert np.linalg.norm(g1 - g_ref) / np.linalg.norm(g_ref) < 1e-6
