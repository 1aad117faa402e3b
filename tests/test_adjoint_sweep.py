"""The adjoint gradient's reverse-sweep plan (host logic, no GPU): which gates share a pass.

qi_adjoint_sweep_plan lists the passes qi_adjoint_gradient runs; these tests check that the
passes cover the gate list once in reverse order, that every pass obeys its kind's rules,
that groups are maximal, and the pass structure of the 26-qubit hardware-efficient ansatz."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

def kinds_of(qi):
    from quant_iron_gb300 import _abi
    return _abi.GATE_KINDS


def gate_info(qi, g):
    kinds = kinds_of(qi)
    name = {v: k for k, v in kinds.items()}[int(g["kind"])]
    nparams = int(np.sum(g["param_ids"] >= 0))
    nt, nc = int(g["n_targets"]), int(g["n_controls"])
    return name, nparams, nt, nc


def groupable(qi, g):
    name, nparams, nt, nc = gate_info(qi, g)
    return name not in ("PAULI_EVOLUTION", "PAULI_STRING", "IDENTITY", "SWAP", "MATCHGATE") and nt == 1 and nc == 0 \
        and nparams <= 1


def affine(qi, g):
    name, nparams, nt, nc = gate_info(qi, g)
    return (name in ("X", "CNOT", "TOFFOLI") and nc <= 1) or (name == "SWAP" and nc == 0)


def check_sweep(qi, gates, steps, f32, fusion_on):
    n = len(gates)
    expect_hi = n - 1
    max_q = 4 if f32 else 3
    for kind, hi, lo in steps:
        assert hi == expect_hi and lo < hi
        run = [gates[k] for k in range(hi, lo, -1)]   # sweep order
        expect_hi = lo
        if kind == qi.SWEEP_GATE:
            assert hi - lo == 1
            continue
        assert hi - lo >= 2
        if kind == qi.SWEEP_GROUP:
            assert all(groupable(qi, g) for g in run)
            qs = [int(g["targets"][0]) for g in run]
            assert len(set(qs)) <= max_q and max(qs.count(q) for q in qs) <= 2
            if lo >= 0 and groupable(qi, gates[lo]):   # maximal: the next gate would break a limit
                q = int(gates[lo]["targets"][0])
                assert (q not in qs and len(set(qs)) == max_q) or qs.count(q) == 2
            continue
        assert fusion_on
        assert all(gate_info(qi, g)[1] == 0 for g in run)
        moves = [g for g in run if gate_info(qi, g)[0] != "IDENTITY"]
        if kind == qi.SWEEP_AFFINE:
            assert len(moves) >= 2 and all(affine(qi, g) for g in moves)
        elif kind == qi.SWEEP_PLAN:
            assert moves and (len(moves) == 1 or not all(affine(qi, g) for g in moves))
        else:
            assert kind == qi.SWEEP_SKIP and not moves
    assert expect_hi == -1


def random_sweep_circuit(n, seed):
    rng = np.random.default_rng(seed)
    gl = workloads.GateList()
    npar = 0
    for _ in range(40):
        r = rng.random()
        a, b, c = (int(x) for x in rng.choice(n, 3, replace=False))
        if r < 0.45:
            kind = str(rng.choice(["RX", "RY", "RZ", "P", "H", "T"]))
            if kind in workloads.PARAMETRIC:
                gl.add(kind, [a], [], [0.0], [npar])
                npar += 1
            else:
                gl.add(kind, [a])
        elif r < 0.6:
            gl.add("CNOT", [b], [a])
        elif r < 0.68:
            gl.add("SWAP", [a, b])
        elif r < 0.74:
            gl.add("X", [a])
        elif r < 0.78:
            gl.add("X", [b], [a])
        elif r < 0.82:
            gl.add("TOFFOLI", [c], [a, b])
        elif r < 0.86:
            gl.add("IDENTITY", [a])
        elif r < 0.9:
            gl.add("PAULI_EVOLUTION", [], [], [0.4, 0.0, 0.2], xmask=(1 << a) | (1 << b), zmask=1 << c)
        elif r < 0.95:
            gl.add("RY", [a], [b], [0.0], [npar])
            npar += 1
        else:
            gl.add("RYPHASE", [a], [], [0.0, 0.0], [npar, npar + 1])
            npar += 2
    return gl.array(), np.linspace(-1, 1, max(1, npar))


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_random_sweeps_obey_the_rules(qi, seed, prec):
    gates, theta = random_sweep_circuit(7, seed)
    for fusion in (qi.FUSION_NONE, qi.FUSION_GREEDY):
        steps = qi.adjoint_sweep_plan(7, prec, gates, theta, fusion=fusion)
        check_sweep(qi, gates, steps, prec == 1, fusion != qi.FUSION_NONE)
        if fusion == qi.FUSION_NONE:
            assert all(k in (qi.SWEEP_GATE, qi.SWEEP_GROUP) for k, _, _ in steps)


def test_hea_26_sweep_structure(qi):
    """12 layers of RY.RZ on 26 qubits + a CNOT ladder: per layer one permutation for the
    ladder and 7 group passes (6 x 4 qubits x 2 gates + 1 x 2 qubits) in FP32, 9 in FP64
    (3 qubits per group); no per-gate passes."""
    n, layers = 26, 12
    gates, theta = workloads.hea_ansatz(n, layers, seed=1)
    for prec, per_layer in ((1, [8] * 6 + [4]), (0, [6] * 8 + [4])):   # gates per group pass
        steps = qi.adjoint_sweep_plan(n, prec, gates, theta)
        check_sweep(qi, gates, steps, prec == 1, True)
        assert len(steps) == layers * (1 + len(per_layer))
        for layer in range(layers):
            chunk = steps[layer * (1 + len(per_layer)):(layer + 1) * (1 + len(per_layer))]
            assert chunk[0][0] == qi.SWEEP_AFFINE and chunk[0][1] - chunk[0][2] == n - 1
            assert [k for k, _, _ in chunk[1:]] == [qi.SWEEP_GROUP] * len(per_layer)
            assert [hi - lo for _, hi, lo in chunk[1:]] == per_layer


def test_pauli_exponential_breaks_a_permutation_run(qi):
    """A Pauli exponential inside a run of CNOTs and SWAPs is not an index permutation: the
    run is un-applied as a fused plan."""
    gl = workloads.GateList()
    gl.add("RY", [0], [], [0.0], [0])
    gl.add("CNOT", [1], [0]).add("SWAP", [2, 5])
    gl.add("PAULI_EVOLUTION", [], [], [0.3, 0.0, 0.1], xmask=0b110, zmask=0b001)
    gl.add("CNOT", [4], [3]).add("IDENTITY", [1])
    gates = gl.array()
    steps = qi.adjoint_sweep_plan(6, 1, gates, np.array([0.2]))
    assert steps == [(qi.SWEEP_PLAN, 5, 0), (qi.SWEEP_GATE, 0, -1)]
    gl2 = workloads.GateList()
    gl2.add("RY", [0], [], [0.0], [0]).add("CNOT", [1], [0]).add("SWAP", [2, 5]).add("X", [3], [1])
    gl2.add("IDENTITY", [2]).add("IDENTITY", [4]).add("IDENTITY", [3])
    steps2 = qi.adjoint_sweep_plan(6, 1, gl2.array(), np.array([0.2]))
    assert steps2[0][0] == qi.SWEEP_AFFINE and steps2[0][1:] == (6, 0)


def test_sweep_plan_errors(qi):
    """The introspection validates like qi_adjoint_gradient: parameter ids past theta, a
    non-differentiable parametric kind, a normalising Pauli string, bad qubit counts."""
    gl = workloads.GateList().add("RY", [0], [], [0.0], [3])
    with pytest.raises(qi.QuantIronError) as ei:
        qi.adjoint_sweep_plan(2, 1, gl.array(), np.zeros(2))
    assert ei.value.variant == "MismatchedNumberOfParameters"
    gl = workloads.GateList().add("H", [0], [], [], [0])
    with pytest.raises(qi.QuantIronError) as ei:
        qi.adjoint_sweep_plan(2, 1, gl.array(), np.zeros(1))
    assert ei.value.variant == "Unsupported"
    gl = workloads.GateList().add("PAULI_STRING", [], [], [1.0, 0.0], xmask=1, zmask=0)
    with pytest.raises(qi.QuantIronError) as ei:
        qi.adjoint_sweep_plan(2, 1, gl.array(), np.zeros(1))
    assert ei.value.variant == "Unsupported"
    for nq in (0, 41):
        with pytest.raises(qi.QuantIronError) as ei:
            qi.adjoint_sweep_plan(nq, 1, workloads.GateList().array(), np.zeros(1))
        assert ei.value.variant == "InvalidNumberOfQubits"
    assert qi.adjoint_sweep_plan(3, 0, workloads.GateList().array(), np.zeros(1)) == []
