"""The fusion pass, checked on the CPU: a plan's device operations, replayed in
numpy, reproduce the oracle's gate-by-gate result (no GPU needed)."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads


def _apply_local(state, n, targets, mat, cmask=0):
    """Apply a dense matrix on sorted `targets` (local bit j <-> targets[j]) with controls."""
    k = len(targets)
    psi = state.reshape([2] * n)   # axis a <-> qubit n-1-a
    axes = [n - 1 - t for t in targets[::-1]]   # most significant local bit first
    rest = [a for a in range(n) if a not in axes]
    perm = axes + rest
    t = np.transpose(psi, perm).reshape(1 << k, -1)
    out = (mat.reshape(1 << k, 1 << k) @ t)
    # controls: keep columns where control bits are not all set
    if cmask:
        cols = np.arange(1 << (n - k))
        # column index bits <-> `rest` axes, most significant first
        idx_full = np.zeros_like(cols)
        for pos, a in enumerate(rest):
            q = n - 1 - a
            bit = (cols >> (len(rest) - 1 - pos)) & 1
            idx_full |= bit << q
        on = (idx_full & cmask) == cmask
        out[:, ~on] = t[:, ~on]
    res = out.reshape([2] * n)
    inv = np.argsort(perm)
    return np.transpose(res, inv).reshape(-1)


def poly_phases(poly, n):
    """exp(2 pi i f(x) / 2^64) for every index x (uint64 arithmetic wraps like the engine's)."""
    c0, a, b = poly
    x = np.arange(1 << n, dtype=np.uint64)
    bits = [((x >> np.uint64(q)) & np.uint64(1)) for q in range(n)]
    f = np.full(1 << n, c0, dtype=np.uint64)
    with np.errstate(over="ignore"):
        for q in range(n):
            f += bits[q] * a[q]
            for r in range(q + 1, n):
                if b[q, r]:
                    f += (bits[q] & bits[r]) * b[q, r]
    turns = f.astype(np.float64) / 2.0 ** 64
    return np.exp(2j * np.pi * turns)


def replay(ops, n, init):
    s = init.astype(np.complex128).copy()
    for op in ops:
        kind = op["kind"]
        if kind == 1:
            s = _apply_local(s, n, op["targets"][:1], op["matrix"], op["control_mask"])
        elif kind == 2:
            sw = np.zeros(16, dtype=complex)
            sw[0], sw[1 * 4 + 2], sw[2 * 4 + 1], sw[15] = 1, 1, 1, 1
            s = _apply_local(s, n, sorted(op["targets"][:2]), sw, op["control_mask"])
        elif kind == 3:
            s = _apply_local(s, n, op["targets"][:2], op["matrix"], op["control_mask"])
        elif kind == 4:
            s = _apply_local(s, n, op["targets"], op["matrix"], 0)
            if "poly" in op:   # a phase polynomial applied after the block in the same pass
                s = s * poly_phases(op["poly"], n)
        elif kind == 7:
            s = _apply_local(s, n, op["targets"], np.diag(op["matrix"]).reshape(-1), 0)
        elif kind == 9:
            s = s * poly_phases(op["poly"], n)
        elif kind == 8:
            s = s / np.linalg.norm(s)
        elif kind == 5:
            x, z = op["xmask"], op["zmask"]
            ch, sh = op["matrix"][0], op["matrix"][1]
            idx = np.arange(1 << n)
            ny = bin(x & z).count("1")
            ph = (-1j) ** ny * np.where(np.array([bin(i & z).count("1") % 2 for i in idx]) == 1, -1, 1)
            s = ch * s + sh * ph * s[idx ^ x]
        elif kind == 10:
            s = _replay_pauli_group(s, n, op)
        elif kind == 11:   # qubit permutation: out[j] = in[flip ^ sum_k bit_k(j) << source_bit[k]]
            idx = np.arange(1 << n, dtype=np.int64)
            src = np.full(1 << n, op["flip"], dtype=np.int64)
            for k in range(n):
                src ^= ((idx >> k) & 1) << int(op["source_bit"][k])
            s = s[src]
        else:
            raise AssertionError("unexpected op kind %d" % kind)
    return s


def _parities(basis, idx):
    """Table index of every entry of `idx`: bit j = popcount(idx & basis[j]) & 1."""
    out = np.zeros(idx.size, dtype=np.int64)
    for j, w in enumerate(basis):
        out |= (np.bitwise_count(idx & np.uint64(w)).astype(np.int64) & 1) << j
    return out


def _replay_pauli_group(s, n, op):
    idx = np.arange(1 << n, dtype=np.uint64)
    x = int(op["xmask"])
    if x == 0:
        f = np.ones(1 << n, dtype=complex)
        for basis, tab in op["group"]:
            f *= tab[_parities(basis, idx)]
        return s * f
    hb = np.uint64(1 << (x.bit_length() - 1))
    i0 = idx[(idx & hb) == 0]
    i1 = i0 ^ np.uint64(x)
    (basis, tab), = op["group"]
    m = tab[_parities(basis, i0)]
    a0, a1 = s[i0], s[i1]
    out = s.copy()
    out[i0] = m[:, 0, 0] * a0 + m[:, 0, 1] * a1
    out[i1] = m[:, 1, 0] * a0 + m[:, 1, 1] * a1
    return out


@pytest.mark.parametrize("kmax", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_greedy_fusion_replay_matches_oracle(qi, orc, kmax, seed):
    n = 8
    gates = workloads.random_circuit(n, layers=5, seed=seed)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax)
    ops = plan.ops()
    assert all(op["k"] <= kmax for op in ops if op["kind"] != 11)
    got = replay(ops, n, init)
    assert np.max(np.abs(got - want)) < 1e-12
    st = plan.stats()
    assert st["n_kernels"] == len(ops) < len(gates)


def test_per_gate_plan_replay_matches_oracle(qi, orc):
    n = 7
    gates = workloads.random_circuit(n, layers=4, seed=11)
    init = workloads.plus_state(n)
    plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_NONE)
    assert plan.stats()["n_kernels"] == len(gates)
    assert np.max(np.abs(replay(plan.ops(), n, init) - orc.execute(init, n, gates))) < 1e-12


def test_fusion_with_controls_matchgate_toffoli(qi, orc):
    from quant_iron_gb300.workloads import GateList
    n = 6
    gl = GateList()
    rng = np.random.default_rng(5)
    for _ in range(30):
        q = int(rng.integers(0, n - 1))
        gl.add("MATCHGATE", [q], [int((q + 2) % n)] if q + 2 < n else [], [rng.uniform(0, 6), rng.uniform(0, 6),
                                                                           rng.uniform(0, 6)])
        gl.add("TOFFOLI", [int(rng.integers(0, 2))], [2, 3])
        gl.add("RX", [int(rng.integers(0, n))], [], [rng.uniform(0, 6)])
        gl.add("SWAP", [1, 4], [0])
        # control on q2 of the matchgate (the (01,10) rotation is then disabled)
        gl.add("MATCHGATE", [2], [3], [1.1, 0.3, 0.7])
    gates = gl.array()
    init = orc.execute(workloads.plus_state(n), n, workloads.random_circuit(n, 2, seed=1, with_qft=False))
    want = orc.execute(init, n, gates)
    for kmax in (3, 4, 6):
        plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax)
        assert np.max(np.abs(replay(plan.ops(), n, init) - want)) < 1e-12


def test_pauli_evolution_gates_fuse(qi, orc):
    from quant_iron_gb300.workloads import GateList
    n = 6
    gl = GateList()
    rng = np.random.default_rng(2)
    for _ in range(20):
        a, b = rng.choice(n, 2, replace=False)
        x = (1 << int(a)) if rng.random() < 0.5 else 0
        z = (1 << int(b)) | (1 << int(a) if rng.random() < 0.5 else 0)
        gl.add("PAULI_EVOLUTION", [], [], [rng.uniform(-1, 1), 0.0, 0.07], xmask=x, zmask=z)
        gl.add("H", [int(rng.integers(0, n))])
    gates = gl.array()
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=4)
    assert np.max(np.abs(replay(plan.ops(), n, init) - want)) < 1e-12


def test_qft_diagonal_runs_fuse(qi):
    n = 20
    gates = workloads.qft(workloads.GateList(), list(range(n))).array()
    st = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6).stats()
    assert st["n_kernels"] < len(gates) / 3


def diag_mix(n, seed, layers=3):
    """QFT ladders plus random diagonal gates (RZ, S, T, P, CZ, controlled phases) between H layers."""
    from quant_iron_gb300.workloads import GateList
    rng = np.random.default_rng(seed)
    gl = GateList()
    for _ in range(layers):
        for q in range(n):
            gl.add("H", [q])
        for _ in range(4 * n):
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            kind = rng.integers(0, 6)
            if kind == 0:
                gl.add("RZ", [a], [], [rng.uniform(-3, 3)])
            elif kind == 1:
                gl.add("S", [a])
            elif kind == 2:
                gl.add("T", [a], [b])
            elif kind == 3:
                gl.add("P", [a], [b], [rng.uniform(-3, 3)])
            elif kind == 4:
                gl.add("Z", [a], [b])
            else:
                gl.add("RZ", [a], [b], [rng.uniform(-3, 3)])
    workloads.qft(gl, list(range(n)))
    return gl.array()


@pytest.mark.parametrize("seed", [0, 1])
def test_fp32_diagonal_runs_become_phase_polynomials(qi, orc, seed):
    n = 9
    gates = diag_mix(n, seed)
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=4)
    ops = plan.ops()
    polys = [op for op in ops if op["kind"] == 9]
    # a run of two or more diagonal blocks, or a single block on three or more qubits
    assert polys and all(op["k"] >= 2 or len(op["targets"]) >= 3 for op in polys)
    got = replay(ops, n, init)
    assert np.max(np.abs(got - want)) < 1e-12
    # FP64 plans keep one diagonal kernel per block
    assert all(op["kind"] != 9 for op in qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_GREEDY,
                                                  max_block_qubits=4).ops())


def test_phase_polynomial_rejects_degree_three(qi, orc):
    """A doubly controlled phase has an x_a x_b x_c term: its block stays a diagonal table."""
    from quant_iron_gb300.workloads import GateList
    n = 8
    gl = GateList()
    gl.add("P", [0], [1], [0.7])
    gl.add("RZ", [5], [6], [0.3])
    gl.add("P", [2], [3, 4], [1.1])   # degree 3
    gl.add("S", [3], [2])
    gl.add("Z", [7], [0])
    gl.add("P", [6], [7], [0.4])
    gates = gl.array()
    init = orc.execute(workloads.plus_state(n), n, workloads.random_circuit(n, 2, seed=3, with_qft=False))
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=3)
    ops = plan.ops()
    # the degree-2 gates commute into one polynomial; the {2, 3, 4} block stays a table
    assert [op["kind"] for op in ops] == [9, 7]
    assert ops[1]["targets"] == [2, 3, 4]
    got = replay(ops, n, init)
    assert np.max(np.abs(got - orc.execute(init, n, gates))) < 1e-12


def _evolution_gates(terms, t):
    gl = workloads.GateList()
    for r in terms:
        gl.add("PAULI_EVOLUTION", [], [], [r["re"], r["im"], t], xmask=int(r["xmask"]), zmask=int(r["zmask"]))
    return gl.array()


@pytest.mark.parametrize("lattice", ["xyz", "tfim", "xxz"])
def test_grouped_exponentials_replay_matches_oracle(qi, orc, lattice):
    """QI_FUSION_PAULI_GROUPS: each run of exponentials with X-masks in {0, X} is one
    table-driven op; replayed in numpy it equals the oracle's term-by-term result."""
    if lattice == "xyz":
        n, terms = 9, workloads.lattice_xyz(3, 3, seed=3)
    elif lattice == "tfim":
        n, terms = 9, workloads.lattice_tfim(3, 3, seed=3)
    else:
        n, terms = 8, workloads.xxz_periodic(8, seed=3)
    gates = _evolution_gates(terms, 0.07)
    init = workloads.basis_state(n, 0b10110101 & ((1 << n) - 1)).astype(complex)
    init = orc.execute(init, n, workloads.random_circuit(n, layers=2, seed=4))
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_PAULI_GROUPS)
    ops = plan.ops()
    assert len(ops) < len(gates)
    assert {op["kind"] for op in ops} <= {5, 10}
    got = replay(ops, n, init)
    assert np.max(np.abs(got - want)) < 1e-12
    assert sum(op["k"] if op["kind"] == 10 else 1 for op in ops) == len(gates)
    if lattice == "xyz":
        # 12 bonds (XX, YY, ZZ: one pair op each, one parity bit); the last bond's op
        # also takes Z fields until its table would need more than 2^6 entries; the rest:
        # one diagonal op
        kinds = [op["kind"] for op in ops]
        assert kinds == [10] * 13 and ops[-1]["xmask"] == 0
        assert all(op["k"] == 3 and len(op["group"][0][0]) == 1 for op in ops[:11])
        assert ops[11]["k"] > 3 and ops[11]["k"] + ops[12]["k"] == 3 + 9
        assert len(ops[11]["group"][0][0]) == 6


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_grouped_exponentials_random_runs(qi, orc, seed):
    """Random runs: X-masks drawn from {0, X1, X2}, random Z-masks and coefficients,
    long diagonal runs that overflow one table and the four-table limit, a term whose
    Z-mask is 0.  (Gate::PauliTimeEvolution takes real coefficients; complex ones, whose
    factors are not unitary, are covered through the Trotter entry point on the GPU.)"""
    n = 10
    rng = np.random.default_rng(seed)
    xs = [0, int(rng.integers(1, 1 << n)), int(rng.integers(1, 1 << n))]
    rows = []
    for k in range(140):
        x = 0 if 40 <= k < 110 else xs[int(rng.integers(0, 3))]
        z = int(rng.integers(0, 1 << n)) if k != 5 else 0
        r = np.zeros((), dtype=qi.TERM_DTYPE)
        r["re"], r["xmask"], r["zmask"] = rng.normal(), x, z
        rows.append(r)
    terms = np.array(rows, dtype=qi.TERM_DTYPE)
    gates = _evolution_gates(terms, 0.09)
    init = workloads.plus_state(n).astype(complex)
    want = orc.execute(init, n, gates)
    ops = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_PAULI_GROUPS).ops()
    assert any(op["kind"] == 10 and op["xmask"] == 0 and len(op["group"]) == 4 for op in ops)
    got = replay(ops, n, init)
    assert np.max(np.abs(got - want)) < 1e-12


def test_window_partition_pass_counts(qi):
    """The fuser's window candidates grow light-cone diamonds on brickwork circuits: the
    30-qubit, 40-layer benchmark circuit (2260 gates) needs 76 dense blocks, 8 phase
    polynomials and one qubit permutation (the QFT's 15 closing SWAPs, which filled 4 dense
    blocks before), where the first gate's light-cone block alone needed 141 dense blocks; a
    bare QFT takes 6 dense blocks and the permutation."""
    n = 30
    plan = qi.Plan(n, qi.F32, workloads.random_circuit(n, 40, seed=0), fusion=qi.FUSION_GREEDY, max_block_qubits=6)
    ops = plan.ops()
    kinds = [op["kind"] for op in ops]
    # each phase polynomial right after a tensor-core block rides on that block's pass
    assert kinds.count(4) == 76 and kinds.count(9) + sum("poly" in op for op in ops) == 8
    assert kinds.count(11) == 1 and kinds[-2:] == [11, 8]
    assert len(kinds) == 78 + kinds.count(9)
    qft = qi.Plan(n, qi.F32, workloads.qft(workloads.GateList(), list(range(n))).array(), fusion=qi.FUSION_GREEDY,
                  max_block_qubits=6)
    assert [op["kind"] for op in qft.ops()] == [4] * 6 + [11, 8]


@pytest.mark.parametrize("kmax", [3, 4, 6])
@pytest.mark.parametrize("n", [7, 10, 12])
def test_qft_swap_network_becomes_one_permutation(qi, orc, n, kmax):
    """The QFT's closing SWAP network (n // 2 swaps across the register) is one qubit
    permutation op after the fused blocks; replaying the plan matches the oracle."""
    gl = workloads.GateList()
    for q in range(n):
        gl.add("H", [q])
    workloads.qft(gl, list(range(n)))
    gates = gl.array()
    init = workloads.plus_state(n) * np.exp(1j * np.arange(1 << n) * 0.37)
    init /= np.linalg.norm(init)
    want = orc.execute(init, n, gates)
    for prec in (qi.F64, qi.F32):
        plan = qi.Plan(n, prec, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax)
        ops = plan.ops()
        perms = [op for op in ops if op["kind"] == 11]
        keff = min(kmax, 5) if prec == qi.F64 else kmax   # FP64 blocks stop at 5 qubits
        assert len(perms) == (1 if n // 2 >= 3 and 2 * (n // 2) > keff else 0)   # the swaps' qubits vs the block size
        if perms:
            assert perms[0]["k"] == n // 2 and perms[0]["flip"] == 0
            assert list(perms[0]["source_bit"]) == list(range(n))[::-1]
        got = replay(ops, n, init)
        assert np.max(np.abs(got - want)) < 1e-10


@pytest.mark.parametrize("seed", range(6))
def test_swap_x_runs_replay(qi, orc, seed):
    """Random circuits with runs of long-range SWAPs and X gates between dense layers: runs
    of three or more SWAPs spanning more than kmax qubits become permutation ops (with the X
    flips folded in), shorter or narrower runs stay in the fused blocks."""
    n, kmax = 9, 4
    rng = np.random.default_rng(seed)
    gl = workloads.GateList()
    expect = 0
    for _ in range(4):
        for q in range(n):
            gl.add("RY", [q], [], [float(rng.uniform(0, 6.28))])
        gl.add("CNOT", [int(rng.integers(1, n))], [0])
        nsw = int(rng.integers(1, 6))
        support = set()
        for _ in range(nsw):
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            gl.add("SWAP", [a, b])
            support |= {a, b}
            if rng.random() < 0.4:
                t = int(rng.integers(0, n))
                gl.add("X", [t])
                support.add(t)
        expect += nsw >= 3 and len(support) > kmax
    gates = gl.array()
    init = workloads.plus_state(n) * np.exp(1j * np.arange(1 << n) * 0.21)
    init /= np.linalg.norm(init)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=kmax)
    ops = plan.ops()
    assert sum(op["kind"] == 11 for op in ops) == expect
    assert np.max(np.abs(replay(ops, n, init) - want)) < 1e-12


@pytest.mark.parametrize("qubits", [[5, 9, 12], [1, 2, 7, 13], [0, 1, 2]])
def test_small_dense_blocks_widened_to_five_qubits(qi, orc, qubits):
    """FP32 plans of 12 qubits and more widen a 3- or 4-qubit dense block to a 5-qubit tensor-core
    block (identity on the lowest free qubits); the widened matrix replays to the oracle's result.
    FP64 plans, plans without tensor cores and smaller states keep the block as it is."""
    rng = np.random.default_rng(len(qubits))
    gl = workloads.GateList()
    for _ in range(3):
        for q in qubits:
            gl.add("RY", [q], [], [rng.uniform(0, 6.28)])
            gl.add("RZ", [q], [], [rng.uniform(0, 6.28)])
        for a, b in zip(qubits[:-1], qubits[1:]):
            gl.add("CNOT", [b], [a])
    gates = gl.array()
    n = 14
    init = workloads.plus_state(n)
    want = orc.execute(init, n, gates)
    ops = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6).ops()
    dense = [op for op in ops if op["kind"] == 4]
    assert len(dense) == 1 and dense[0]["k"] == 5 and dense[0].get("tensor_cores")
    free = [q for q in range(n) if q not in qubits][:5 - len(qubits)]
    assert sorted(dense[0]["targets"]) == sorted(qubits + free)
    assert np.max(np.abs(replay(ops, n, init) - want)) < 1e-12
    for prec, nq, tc in ((qi.F64, 14, 0), (qi.F32, 14, 2), (qi.F32, 11, 0)):
        g2 = gates if nq == 14 else np.array([g for g in gates if max(g["targets"][:1]) < nq], dtype=gates.dtype)
        if nq != 14 and max(qubits) >= nq:
            continue
        ops2 = qi.Plan(nq, prec, g2, fusion=qi.FUSION_GREEDY, max_block_qubits=6, use_tensor_cores=tc).ops()
        assert [op["k"] for op in ops2 if op["kind"] == 4] == [len(qubits)]
