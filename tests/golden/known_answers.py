"""Known-answer vectors of quant-iron's own test-suite, restated as data.

The reference crate is Rust and cannot be built here, so its tests cannot be
run; their asserted input/output pairs are analytical and are restated below,
each citing the test (file:line within the quant-iron crate) it comes from.
The same cases pin the CPU oracle (tests/test_oracle_golden.py) and the GPU
engine through the C ABI (tests/test_gpu_golden.py).  Equality is the
reference's `PartialEq for State`: |diff| < f32::EPSILON per component
(src/components/state.rs:2348-2372).

A gate case is (name, cite, n, init, [gate rows], expected).
"""
import math

import numpy as np

from quant_iron_gb300.workloads import GateList, term, terms_array

PI = math.pi
R2 = 1.0 / math.sqrt(2.0)
I = 1j
F32_EPS = float(np.finfo(np.float32).eps)


def basis(n, i):
    v = np.zeros(1 << n, dtype=np.complex128)
    v[i] = 1.0
    return v


def zero(n):
    return basis(n, 0)


def plus(n):
    return np.full(1 << n, 1.0 / math.sqrt(1 << n), dtype=np.complex128)


def minus(n):
    v = plus(n)
    for i in range(1 << n):
        if bin(i).count("1") % 2:
            v[i] = -v[i]
    return v


def kron(a, b):
    """State::tensor_product: self is the high qubits (state.rs:801-836)."""
    return np.kron(a, b)


def g(kind, targets, controls=(), params=()):
    return GateList().add(kind, list(targets), list(controls), list(params)).array()[0]


def multi(kind, qubits, controls=(), params=()):
    return [g(kind, [q], controls, params) for q in qubits]


GATE_CASES = []


def case(name, cite, n, init, gates, expected):
    if not isinstance(gates, list):
        gates = [gates]
    GATE_CASES.append((name, cite, n, np.asarray(init, dtype=np.complex128), gates,
                       np.asarray(expected, dtype=np.complex128)))


def one_qubit_family(kind, cite, params, on_zero, on_one, on_plus, on_minus):
    z, o, p, m = zero(1), basis(1, 1), plus(1), minus(1)
    case(kind + "|0>", cite, 1, z, g(kind, [0], (), params), on_zero)
    case(kind + "|1>", cite, 1, o, g(kind, [0], (), params), on_one)
    case(kind + "|+>", cite, 1, p, g(kind, [0], (), params), on_plus)
    case(kind + "|->", cite, 1, m, g(kind, [0], (), params), on_minus)


# --- Hadamard: operator_tests.rs:17-121
one_qubit_family("H", "operator_tests.rs:17-31", (), plus(1), minus(1), zero(1), basis(1, 1))
case("H multi |00>", "operator_tests.rs:34-38", 2, zero(2), multi("H", [0, 1]), plus(2))
case("CH(c0,t1)|+1>", "operator_tests.rs:40-44", 2, kron(plus(1), basis(1, 1)), g("H", [1], [0]), basis(2, 1))
case("CH(c1,t0)|00+>", "operator_tests.rs:46-50", 3, kron(basis(2, 0), plus(1)), g("H", [0], [1]),
     kron(basis(2, 0), plus(1)))
for nq, cite in ((11, "operator_tests.rs:52-80"), (15, "operator_tests.rs:83-115")):
    case("H all |0..0> %dq" % nq, cite, nq, zero(nq), multi("H", range(nq)), plus(nq))
    case("CH c=0 %dq" % nq, cite, nq, zero(nq), g("H", [0], [nq - 1]), zero(nq))
    e = np.zeros(1 << nq, dtype=np.complex128)
    e[1 << (nq - 1)] = R2
    e[(1 << (nq - 1)) | 1] = R2
    case("CH c=1 %dq" % nq, cite, nq, basis(nq, 1 << (nq - 1)), g("H", [0], [nq - 1]), e)

# --- Pauli X: operator_tests.rs:124-237
one_qubit_family("X", "operator_tests.rs:124-136", (), basis(1, 1), zero(1), plus(1), -minus(1))
case("X multi |00>", "operator_tests.rs:138-142", 2, zero(2), multi("X", [0, 1]), basis(2, 3))
case("XX|0>", "operator_tests.rs:144-146", 1, zero(1), multi("X", [0, 0]), zero(1))
case("CX(c0,t1)|11>", "operator_tests.rs:148-152", 2, basis(2, 3), g("X", [1], [0]), basis(2, 1))
case("CCX(c0,c1,t2)|011>", "operator_tests.rs:154-158", 3, basis(3, 3), g("X", [2], [0, 1]), basis(3, 7))
case("CX(c0,t1)|10>", "operator_tests.rs:160-164", 2, basis(2, 2), g("X", [1], [0]), basis(2, 2))
for nq, cite in ((11, "operator_tests.rs:168-199"), (15, "operator_tests.rs:200-235")):
    case("X all %dq" % nq, cite, nq, zero(nq), multi("X", range(nq)), basis(nq, (1 << nq) - 1))
    case("CX c=1 %dq" % nq, cite, nq, basis(nq, 1 << (nq - 1)), g("X", [0], [nq - 1]),
         basis(nq, (1 << (nq - 1)) | 1))

# --- Pauli Y: operator_tests.rs:240-356
one_qubit_family("Y", "operator_tests.rs:240-259", (), I * basis(1, 1), -I * zero(1), -I * minus(1), I * plus(1))
case("Y multi |00>", "operator_tests.rs:261-265", 2, zero(2), multi("Y", [0, 1]), -basis(2, 3))
case("YY|0>", "operator_tests.rs:267-269", 1, zero(1), multi("Y", [0, 0]), zero(1))
case("CY(c0,t1)|11>", "operator_tests.rs:271-275", 2, basis(2, 3), g("Y", [1], [0]), kron(-I * zero(1), basis(1, 1)))
case("CY(c0,t1)|10>", "operator_tests.rs:277-281", 2, basis(2, 2), g("Y", [1], [0]), basis(2, 2))
for nq, cite in ((11, "operator_tests.rs:284-318"), (15, "operator_tests.rs:319-354")):
    case("CY c=1 %dq" % nq, cite, nq, basis(nq, 1 << (nq - 1)), g("Y", [0], [nq - 1]),
         I * basis(nq, (1 << (nq - 1)) | 1))

# --- Pauli Z: operator_tests.rs:359-485
one_qubit_family("Z", "operator_tests.rs:359-372", (), zero(1), -basis(1, 1), minus(1), plus(1))
case("Z multi |00>", "operator_tests.rs:374-378", 2, zero(2), multi("Z", [0, 1]), zero(2))
case("CZ(c0,t1)|11>", "operator_tests.rs:384-388", 2, basis(2, 3), g("Z", [1], [0]), -basis(2, 3))
case("CZ(c0,t1)|10>", "operator_tests.rs:390-394", 2, basis(2, 2), g("Z", [1], [0]), basis(2, 2))
for nq, cite in ((11, "operator_tests.rs:397-442"), (15, "operator_tests.rs:444-483")):
    idx = (1 << (nq - 1)) | 1
    case("CZ c=1 t=1 %dq" % nq, cite, nq, basis(nq, idx), g("Z", [0], [nq - 1]), -basis(nq, idx))
    case("CZ c=0 t=1 %dq" % nq, cite, nq, basis(nq, 1), g("Z", [0], [nq - 1]), basis(nq, 1))

# --- Identity: operator_tests.rs:537-579
one_qubit_family("IDENTITY", "operator_tests.rs:537-552", (), zero(1), basis(1, 1), plus(1), minus(1))

# --- S, T, S-dagger, T-dagger: operator_tests.rs:582-1105
EIPI4 = np.exp(1j * PI / 4)
for kind, ph, cite in (("S", 1j, "operator_tests.rs:582-717"), ("T", EIPI4, "operator_tests.rs:720-855"),
                       ("SDAG", -1j, "operator_tests.rs:858-983"), ("TDAG", np.conj(EIPI4), "operator_tests.rs:986-1105")):
    one_qubit_family(kind, cite, (), zero(1), ph * basis(1, 1), R2 * (zero(1) + ph * basis(1, 1)),
                     R2 * (zero(1) - ph * basis(1, 1)))
    case("C%s(c0,t1)|+1>" % kind, cite, 2, kron(plus(1), basis(1, 1)), g(kind, [1], [0]),
         kron(R2 * (zero(1) + ph * basis(1, 1)), basis(1, 1)))
    case("C%s(c1,t0)|00+>" % kind, cite, 3, kron(basis(2, 0), plus(1)), g(kind, [0], [1]), kron(basis(2, 0), plus(1)))
    for nq in (11, 15):
        idx = (1 << (nq - 1)) | 1
        case("C%s c=1 t=1 %dq" % (kind, nq), cite, nq, basis(nq, idx), g(kind, [0], [nq - 1]), ph * basis(nq, idx))

# --- PhaseShift: operator_tests.rs:1108-1247
TH = PI / 2.5
ET = np.exp(1j * TH)
one_qubit_family("P", "operator_tests.rs:1108-1125", (TH,), zero(1), ET * basis(1, 1), R2 * (zero(1) + ET * basis(1, 1)),
                 R2 * (zero(1) - ET * basis(1, 1)))
case("P(pi/2)|+> = S|+>", "operator_tests.rs:1127-1129", 1, plus(1), g("P", [0], (), (PI / 2,)),
     R2 * (zero(1) + 1j * basis(1, 1)))
case("CP(c0,t1,pi/2)|+1>", "operator_tests.rs:1143-1148", 2, kron(plus(1), basis(1, 1)), g("P", [1], [0], (PI / 2,)),
     kron(R2 * (zero(1) + np.exp(1j * PI / 2) * basis(1, 1)), basis(1, 1)))
for nq in (11, 15):
    idx = (1 << (nq - 1)) | 1
    case("CP c=1 t=1 %dq" % nq, "operator_tests.rs:1163-1245", nq, basis(nq, idx), g("P", [0], [nq - 1], (PI / 5,)),
         np.exp(1j * PI / 5) * basis(nq, idx))

# --- RotateX / RotateY / RotateZ: operator_tests.rs:1250-1749
C, S = math.cos(TH / 2), math.sin(TH / 2)
one_qubit_family("RX", "operator_tests.rs:1250-1275", (TH,), C * zero(1) - 1j * S * basis(1, 1),
                 -1j * S * zero(1) + C * basis(1, 1), np.exp(-1j * TH / 2) * plus(1), np.exp(1j * TH / 2) * minus(1))
case("RX multi |00>", "operator_tests.rs:1277-1284", 2, zero(2), multi("RX", [0, 1], (), (TH,)),
     C * C * basis(2, 0) - 1j * C * S * basis(2, 1) - 1j * C * S * basis(2, 2) - S * S * basis(2, 3))
case("CRX(c0,t1,pi)|11>", "operator_tests.rs:1286-1290", 2, basis(2, 3), g("RX", [1], [0], (PI,)),
     kron(-1j * zero(1), basis(1, 1)))
one_qubit_family("RY", "operator_tests.rs:1428-1455", (TH,), C * zero(1) + S * basis(1, 1),
                 -S * zero(1) + C * basis(1, 1), R2 * ((C - S) * zero(1) + (C + S) * basis(1, 1)),
                 R2 * ((C + S) * zero(1) - (C - S) * basis(1, 1)))
case("RY multi |00>", "operator_tests.rs:1457-1464", 2, zero(2), multi("RY", [0, 1], (), (TH,)),
     C * C * basis(2, 0) + S * C * basis(2, 1) + S * C * basis(2, 2) + S * S * basis(2, 3))
case("CRY(c0,t1,pi)|11>", "operator_tests.rs:1466-1470", 2, basis(2, 3), g("RY", [1], [0], (PI,)),
     kron(-zero(1), basis(1, 1)))
EM, EP = np.exp(-1j * TH / 2), np.exp(1j * TH / 2)
one_qubit_family("RZ", "operator_tests.rs:1602-1622", (TH,), EM * zero(1), EP * basis(1, 1),
                 R2 * (EM * zero(1) + EP * basis(1, 1)), R2 * (EM * zero(1) - EP * basis(1, 1)))
case("RZ multi |00>", "operator_tests.rs:1624-1627", 2, zero(2), multi("RZ", [0, 1], (), (TH,)), EM * EM * zero(2))
case("CRZ(c0,t1,pi)|11>", "operator_tests.rs:1629-1633", 2, basis(2, 3), g("RZ", [1], [0], (PI,)),
     kron(1j * basis(1, 1), basis(1, 1)))
for kind, ang, cite in (("RX", PI / 2.2, "operator_tests.rs:1318-1350"), ("RY", PI / 2.8, "operator_tests.rs:1496-1530"),
                        ("RZ", PI / 3.3, "operator_tests.rs:1660-1695")):
    for nq in (11, 15):
        c, s = math.cos(ang / 2), math.sin(ang / 2)
        col = {"RX": (c, -1j * s), "RY": (c, s), "RZ": (np.exp(-1j * ang / 2), 0.0)}[kind]
        e = np.zeros(1 << nq, dtype=np.complex128)
        e[1 << (nq - 1)] = col[0]
        e[(1 << (nq - 1)) | 1] = col[1]
        case("C%s c=1 %dq" % (kind, nq), cite, nq, basis(nq, 1 << (nq - 1)), g(kind, [0], [nq - 1], (ang,)), e)

# --- Unitary2 (X as a matrix): operator_tests.rs:1752-1844
UX = (0, 0, 1, 0, 1, 0, 0, 0)
one_qubit_family("U2", "operator_tests.rs:1752-1775", UX, basis(1, 1), zero(1), plus(1), -minus(1))
case("CU2(c0,t1)|11>", "operator_tests.rs:1782-1786", 2, basis(2, 3), g("U2", [1], [0], UX), basis(2, 1))

# --- ry_phase / ry_phase_dag: operator_tests.rs:1847-1983
PH = PI / 4.0
RYP = np.array([[C, -np.exp(1j * PH) * S], [S, np.exp(1j * PH) * C]])
case("RyPhase|0>", "operator_tests.rs:1847-1870", 1, zero(1), g("RYPHASE", [0], (), (TH, PH)), RYP[:, 0])
case("RyPhase|1>", "operator_tests.rs:1847-1870", 1, basis(1, 1), g("RYPHASE", [0], (), (TH, PH)), RYP[:, 1])
case("RyPhase then dagger", "operator_tests.rs:1957-1983", 1, plus(1),
     [g("RYPHASE", [0], (), (TH, PH)), g("RYPHASE_DAG", [0], (), (TH, PH))], plus(1))
case("U(pi/2,pi) = H", "operator_tests.rs:2128-2129 (doc)", 1, zero(1), g("RYPHASE", [0], (), (PI / 2, PI)), plus(1))

# --- CNOT: operator_tests.rs:1986-2067 (State::cnot(control, target))
case("CNOT(c0,t1)|01>", "operator_tests.rs:1986-2000", 2, basis(2, 1), g("CNOT", [1], [0]), basis(2, 3))
case("CNOT(c0,t1)|00>", "operator_tests.rs:1986-2000", 2, basis(2, 0), g("CNOT", [1], [0]), basis(2, 0))
case("CNOT(c0,t1)|11>", "operator_tests.rs:1986-2000", 2, basis(2, 3), g("CNOT", [1], [0]), basis(2, 1))
case("CNOT(c1,t0)|10>", "operator_tests.rs:2002-2010", 2, basis(2, 2), g("CNOT", [0], [1]), basis(2, 3))

# --- SWAP: operator_tests.rs:2070-2211
case("SWAP |01>", "operator_tests.rs:2070-2080", 2, basis(2, 1), g("SWAP", [0, 1]), basis(2, 2))
case("SWAP |+0>", "operator_tests.rs:2082-2090", 2, kron(plus(1), zero(1)), g("SWAP", [0, 1]), kron(zero(1), plus(1)))
case("CSWAP c=1 |101>", "operator_tests.rs:2092-2110", 3, basis(3, 5), g("SWAP", [0, 1], [2]), basis(3, 6))
case("CSWAP c=0 |001>", "operator_tests.rs:2092-2110", 3, basis(3, 1), g("SWAP", [0, 1], [2]), basis(3, 1))
for nq in (11, 15):
    case("SWAP(0,%d) %dq" % (nq - 1, nq), "operator_tests.rs:2112-2209", nq, basis(nq, 1), g("SWAP", [0, nq - 1]),
         basis(nq, 1 << (nq - 1)))

# --- Matchgate: operator_tests.rs:2214-2388
case("Matchgate(1; pi,pi,0)|101>", "operator_tests.rs:2217-2221", 3, basis(3, 5), g("MATCHGATE", [1], (), (PI, PI, 0.0)),
     basis(3, 3))
case("Matchgate twice", "operator_tests.rs:2223-2228", 3, basis(3, 5),
     [g("MATCHGATE", [1], (), (PI, PI, 0.0))] * 2, basis(3, 5))
MG = (PI, PI / 2, PI / 3)
case("M|00>", "operator_tests.rs:2240-2244", 2, basis(2, 0), g("MATCHGATE", [0], (), MG), basis(2, 0))
case("M|01>", "operator_tests.rs:2246-2249", 2, basis(2, 1), g("MATCHGATE", [0], (), MG), basis(2, 2))
case("M|10>", "operator_tests.rs:2251-2254", 2, basis(2, 2), g("MATCHGATE", [0], (), MG), -1j * basis(2, 1))
case("M|11>", "operator_tests.rs:2256-2259", 2, basis(2, 3), g("MATCHGATE", [0], (), MG),
     np.exp(1j * PI / 3) * basis(2, 3))
case("CM c0=1 |011>", "operator_tests.rs:2265-2269", 3, basis(3, 3), g("MATCHGATE", [1], [0], MG), basis(3, 5))
case("CM c0=0 |100>", "operator_tests.rs:2271-2275", 3, basis(3, 4), g("MATCHGATE", [1], [0], MG), basis(3, 4))
case("M(0,1) 11q |..01>", "operator_tests.rs:2283-2287", 11, basis(11, 1), g("MATCHGATE", [0], (), MG), basis(11, 2))
case("M(0,1) 11q |..10>", "operator_tests.rs:2289-2292", 11, basis(11, 2), g("MATCHGATE", [0], (), MG), -1j * basis(11, 1))

# --- Toffoli: operator_tests.rs:2391-2490
case("Toffoli |011>", "operator_tests.rs:2391-2400", 3, basis(3, 3), g("TOFFOLI", [2], [0, 1]), basis(3, 7))
case("Toffoli |001>", "operator_tests.rs:2391-2400", 3, basis(3, 1), g("TOFFOLI", [2], [0, 1]), basis(3, 1))
case("Toffoli |111>", "operator_tests.rs:2402-2410", 3, basis(3, 7), g("TOFFOLI", [2], [0, 1]), basis(3, 3))

# --- error cases.  (name, cite, n, gate row, error variant, (a, b))
# test_single_qubit_gate_errors (operator_tests.rs:2513-2566): every single-qubit
# gate at index 2 of a 2-qubit state -> InvalidQubitIndex(2, 2).
ERROR_CASES = []
for _k, _p in (("H", ()), ("X", ()), ("Y", ()), ("Z", ()), ("S", ()), ("T", ()), ("SDAG", ()), ("TDAG", ()),
               ("IDENTITY", ()), ("P", (PI / 4,)), ("RX", (PI / 4,)), ("RY", (PI / 4,)), ("RZ", (PI / 4,))):
    ERROR_CASES.append(("%s index 2 of 2" % _k, "operator_tests.rs:2513-2566", 2, g(_k, [2], (), _p),
                        "InvalidQubitIndex", (2, 2)))
# test_multi_qubit_gate_errors (operator_tests.rs:2569-2703): index 3 of a 3-qubit state.
ERROR_CASES += [
    ("CNOT invalid control", "operator_tests.rs:2575-2585", 3, g("CNOT", [0], [3]), "InvalidQubitIndex", (3, 3)),
    ("CNOT invalid target", "operator_tests.rs:2587-2597", 3, g("CNOT", [3], [0]), "InvalidQubitIndex", (3, 3)),
    ("SWAP invalid q1", "operator_tests.rs:2599-2609", 3, g("SWAP", [3, 1]), "InvalidQubitIndex", (3, 3)),
    ("SWAP invalid q2", "operator_tests.rs:2611-2621", 3, g("SWAP", [0, 3]), "InvalidQubitIndex", (3, 3)),
    ("Toffoli invalid c1", "operator_tests.rs:2623-2660", 3, g("TOFFOLI", [2], [3, 1]), "InvalidQubitIndex", (3, 3)),
    ("Toffoli invalid target", "operator_tests.rs:2623-2660", 3, g("TOFFOLI", [3], [0, 1]), "InvalidQubitIndex",
     (3, 3)),
]
# validate_qubits / per-gate checks in operator.rs (no dedicated reference test):
ERROR_CASES += [
    ("H wrong #targets", "operator.rs:220-223", 2, g("H", [0, 1]), "InvalidNumberOfQubits", (2, -1)),
    ("H control == target", "operator.rs:235-244", 2, g("H", [0], [0]), "OverlappingControlAndTargetQubits", (0, 0)),
    ("SWAP duplicate targets", "operator.rs:249-270", 2, g("SWAP", [0, 0]), "InvalidQubitIndex", (0, 2)),
    ("CNOT no control", "operator.rs:675-678", 2, g("CNOT", [0]), "InvalidNumberOfQubits", (0, -1)),
    ("CNOT two controls", "operator.rs:675-678", 3, g("CNOT", [0], [1, 2]), "InvalidNumberOfQubits", (2, -1)),
    ("Toffoli one control", "operator.rs:1063-1066", 3, g("TOFFOLI", [0], [1]), "InvalidNumberOfQubits", (1, -1)),
    ("Toffoli same controls", "operator.rs:1068-1071", 3, g("TOFFOLI", [0], [1, 1]), "InvalidNumberOfQubits", (2, -1)),
    ("Matchgate on last qubit", "operator.rs:907-910", 3, g("MATCHGATE", [2], (), (1.0, 0.0, 0.0)),
     "InvalidQubitIndex", (2, 3)),
]

# --- Pauli strings and sums: pauli_string_tests.rs
PAULI_CASES = []   # (name, cite, n, init, op, payload, expected)


def pcase(name, cite, n, init, op, payload, expected):
    PAULI_CASES.append((name, cite, n, np.asarray(init, dtype=np.complex128), op, payload,
                        np.asarray(expected, dtype=np.complex128) if not np.isscalar(expected) else expected))


T_XY = terms_array([term(2.0, [(0, "X")]), term(3.0, [(1, "Y")]), term(4.0, [(1, "Z")])])
pcase("<2X0+3Y1+4Z1> on |11> = -4", "pauli_string_tests.rs:348-365", 2, basis(2, 3), "expectation", T_XY, -4.0 + 0j)
pcase("SumOp empty apply = 0 * state", "pauli_string_tests.rs:330-340", 2, basis(2, 3), "sumop_apply",
      terms_array([]), 0.0 * basis(2, 3))
pcase("exp(-i 0.5 (pi/2) Z0 X1)|00>", "pauli_string_tests.rs:408-439", 2, zero(2), "exp_neg_i_dt",
      (terms_array([term(0.5 * PI, [(0, "Z"), (1, "X")])])[0], 0.5), R2 * basis(2, 0) - 1j * R2 * basis(2, 2))
pcase("exp_neg_i_dt with dt = 0 is identity", "pauli_string_tests.rs:433-438", 2, zero(2), "exp_neg_i_dt",
      (terms_array([term(0.5 * PI, [(0, "Z"), (1, "X")])])[0], 0.0), zero(2))
# apply: X0 on |0> = |1>, Y on |0> = i|1>, Z on |1> = -|1>  (operator_tests.rs:488-534, Pauli::to_pauli_string)
pcase("PauliString X0 apply |0>", "operator_tests.rs:505-509", 1, zero(1), "apply", terms_array([term(1.0, [(0, "X")])])[0],
      basis(1, 1))
pcase("PauliString Y0 apply |0>", "operator_tests.rs:511-515", 1, zero(1), "apply", terms_array([term(1.0, [(0, "Y")])])[0],
      1j * basis(1, 1))
pcase("PauliString Z0 apply |1>", "operator_tests.rs:517-521", 1, basis(1, 1), "apply",
      terms_array([term(1.0, [(0, "Z")])])[0], -basis(1, 1))
# exp(alpha P) = cosh(alpha) + sinh(alpha) P  (pauli_string_tests.rs:161-252)
AL = 0.3 + 0.2j
pcase("exp((0.3+0.2i) X0)|0>", "pauli_string_tests.rs:161-200", 1, zero(1), "exp",
      terms_array([term(AL, [(0, "X")])])[0], np.cosh(AL) * zero(1) + np.sinh(AL) * basis(1, 1))
pcase("exp_factor(0.5 Z0, -i)|+>", "pauli_string_tests.rs:214-252", 1, plus(1), "exp_factor",
      (terms_array([term(0.5, [(0, "Z")])])[0], -1j),
      np.cosh(-0.5j) * plus(1) + np.sinh(-0.5j) * minus(1))

# --- Gate::PauliTimeEvolution vector: gate_tests.rs:124-186 (same physics as :408-439)
TE_GATE = GateList().add("PAULI_EVOLUTION", [], [], [0.5 * PI, 0.0, 0.5], xmask=0b10, zmask=0b01).array()[0]
