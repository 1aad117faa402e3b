"""Mirror of quant-iron's public API (src/lib.rs:59-70) over the GB300 engine.

Same names, argument meaning and error behaviour as the Rust crate, so that
code written against `quant_iron` reads the same here:

  State (state.rs)              `state_vector` like the Rust pub field; gate
                                methods return new States; measure / measure_n
  MeasurementBasis, MeasurementResult (measurement.rs)
  Hadamard, Pauli, CNOT, ... (operator.rs)   Operator.apply(state, targets, controls)
  PauliString, SumOp (pauli_string.rs)
  Gate, Circuit (gate.rs, circuit.rs)
  first/second_order_trotter_step, trotter_evolve_state (time_evolution.rs)

Every operation runs on the GPU.  A State lives on the device once it has been
used there: an operation copies it device to device, runs its kernels and
returns a new State that owns the result, so chains (`st.h(0).cnot(0, 1)...`,
`*_multi`, Circuit.execute, Trotter steps) never round-trip through the host.
`state_vector` is downloaded on first read (and cached); assigning it replaces
the device copy.  Errors raise QuantIronError whose `.variant` is the name of
the Rust Error variant.
"""
import math

import numpy as np

from . import _abi
from . import DeviceState, Plan, sumop_expectation as _expect, sumop_apply as _sumop_apply
from . import pauli_apply as _pauli_apply, pauli_apply_normalised as _pauli_norm
from . import pauli_apply_exp_factor as _pauli_exp_factor, trotter_evolve as _trotter
from . import measure as _measure, measure_n as _measure_n
from ._abi import F32, F64, FUSION_GREEDY, FUSION_NONE, GATE_DTYPE, TERM_DTYPE, QuantIronError, check, lib
from .workloads import GateList, qft as _qft

PRECISION = F64          # precision of device states created by this module
FUSION = FUSION_NONE     # fusion used by Circuit.execute
F32_EPS = float(np.finfo(np.float32).eps)
F64_EPS = float(np.finfo(np.float64).eps)


def _err(variant_code, a=-1, b=-1):
    return QuantIronError(variant_code, a, b)


# --------------------------------------------------------------------- State
class State:
    """`State { state_vector, num_qubits }` (state.rs:74-81).  Holds a host copy, a
    device copy, or both; `state_vector` reads download once and cache."""

    def __init__(self, state_vector, num_qubits, _dev=None):
        self.num_qubits = int(num_qubits)
        self._host = None if state_vector is None else np.ascontiguousarray(state_vector, dtype=np.complex128)
        self._dev = _dev

    @property
    def state_vector(self):
        if self._host is None:
            self._host = self._dev.download()
        return self._host

    @state_vector.setter
    def state_vector(self, v):
        self._host = np.ascontiguousarray(v, dtype=np.complex128)
        self._dev = None

    @staticmethod
    def _take(d, n):
        """A State owning the device state `d` (no download)."""
        return State(None, n, _dev=d.release())

    def _resident(self):
        """The device copy (uploaded on first use); read-only for callers."""
        if self._dev is None:
            d = DeviceState(self.num_qubits, PRECISION)
            d.upload(self._host)
            self._dev = d
        return self._dev

    # constructors (state.rs:99-373)
    @staticmethod
    def new(state_vector):
        v = np.ascontiguousarray(state_vector, dtype=np.complex128)
        ln = v.size
        if ln == 0:
            raise _err(-3, 0)
        if ln & (ln - 1):
            raise _err(-3, int(math.floor(math.log2(ln))))
        n = ln.bit_length() - 1
        st = State(v, n)
        st._resident().check_normalised()
        return st

    @staticmethod
    def _made(n, fill):
        if n == 0:
            raise _err(-3, 0)
        with DeviceState(n, PRECISION) as d:
            fill(d)
            return State._take(d, n)

    @staticmethod
    def new_zero(n):
        return State._made(n, lambda d: d.set_zero())

    @staticmethod
    def new_basis_n(n, idx):
        if idx >= (1 << n):
            raise _err(-4, idx, n)
        return State._made(n, lambda d: d.set_basis(idx))

    @staticmethod
    def new_plus(n):
        return State._made(n, lambda d: d.set_plus())

    @staticmethod
    def new_minus(n):
        return State._made(n, lambda d: d.set_minus())

    @staticmethod
    def new_ghz(n):
        return State._made(n, lambda d: d.set_ghz())

    def num_qubits_(self):
        return self.num_qubits

    def _device(self):
        """A scratch device copy the caller may modify (device to device)."""
        d = DeviceState(self.num_qubits, PRECISION)
        d.copy_from(self._resident())
        return d

    def clone(self):
        if self._dev is None:
            return State(self._host.copy(), self.num_qubits)
        with self._device() as d:
            return State._take(d, self.num_qubits)

    # PartialEq: per-component |diff| < f32::EPSILON (state.rs:2348-2372)
    def __eq__(self, other):
        if not isinstance(other, State) or self.num_qubits != other.num_qubits:
            return False
        a, b = self.state_vector, other.state_vector
        return bool(np.all(np.abs(a.real - b.real) < F32_EPS) and np.all(np.abs(a.imag - b.imag) < F32_EPS))

    def __repr__(self):
        return "State(num_qubits=%d)" % self.num_qubits

    def equals_without_phase(self, other):
        return self.num_qubits == other.num_qubits and abs(abs(self.inner_product(other)) - 1.0) < F32_EPS

    def probability(self, n):
        return abs(self.amplitude(n)) ** 2

    def amplitude(self, n):
        if n >= (1 << self.num_qubits):
            raise _err(-4, n, self.num_qubits)
        if self._host is not None:
            return self._host[n]
        return self._dev.amplitude(n)   # one device read, no download

    def inner_product(self, other):   # state.rs:890-917
        if self.num_qubits == 0 or other.num_qubits == 0:
            raise _err(-3, 0)
        if self.num_qubits != other.num_qubits:
            raise _err(-3, self.num_qubits)
        return self._resident().inner_product(other._resident())

    def normalise(self):   # state.rs:924-945
        with self._device() as d:
            d.normalise()
            return State._take(d, self.num_qubits)

    def fs_fidelity(self, other):
        return abs(self.normalise().inner_product(other.normalise())) ** 2

    def fs_dist(self, other):
        return math.acos(min(1.0, abs(self.normalise().inner_product(other.normalise()))))

    def tensor_product(self, other):   # state.rs:801-836
        if self.num_qubits == 0 or other.num_qubits == 0:
            raise _err(-3, 0)
        from . import tensor_product as _tp
        n = self.num_qubits + other.num_qubits
        with DeviceState(n, PRECISION) as o:
            _tp(o, self._resident(), other._resident())
            out = State._take(o, n)
        out._resident().check_normalised()   # State::new's check
        return out

    # arithmetic (state.rs:2687-2862)
    def __mul__(self, c):
        with self._device() as d:
            d.scale(complex(c))
            return State._take(d, self.num_qubits)

    __rmul__ = __mul__

    def __add__(self, other):
        with self._device() as y:
            y.axpy(1.0, other._resident())
            return State._take(y, self.num_qubits)

    def __sub__(self, other):
        with self._device() as y:
            y.axpy(-1.0, other._resident())
            return State._take(y, self.num_qubits)

    # operate (state.rs:970-1002)
    def operate(self, op, target_qubits, control_qubits=()):
        nt, nc = len(target_qubits), len(control_qubits)
        if op.base_qubits() != nt + nc:
            raise _err(-3, op.base_qubits())
        if nt > self.num_qubits:
            raise _err(-3, self.num_qubits)
        for q in list(target_qubits) + list(control_qubits):
            if q >= self.num_qubits:
                raise _err(-4, q, self.num_qubits)
        return op.apply(self, target_qubits, control_qubits)

    # gate methods (state.rs:1019-2346)
    def _multi(self, op, qubits, controls=()):
        st = self
        for q in qubits:
            st = op.apply(st, [q], list(controls))
        return st

    def h(self, i): return Hadamard().apply(self, [i], [])
    def h_multi(self, qs): return self._multi(Hadamard(), qs)
    def ch_multi(self, ts, cs): return self._multi(Hadamard(), ts, cs)
    def x(self, i): return Pauli.X.apply(self, [i], [])
    def x_multi(self, qs): return self._multi(Pauli.X, qs)
    def cx_multi(self, ts, cs): return self._multi(Pauli.X, ts, cs)
    def y(self, i): return Pauli.Y.apply(self, [i], [])
    def y_multi(self, qs): return self._multi(Pauli.Y, qs)
    def cy_multi(self, ts, cs): return self._multi(Pauli.Y, ts, cs)
    def z(self, i): return Pauli.Z.apply(self, [i], [])
    def z_multi(self, qs): return self._multi(Pauli.Z, qs)
    def cz_multi(self, ts, cs): return self._multi(Pauli.Z, ts, cs)
    def i(self, q): return Identity().apply(self, [q], [])
    def s(self, i): return PhaseS().apply(self, [i], [])
    def s_multi(self, qs): return self._multi(PhaseS(), qs)
    def cs_multi(self, ts, cs): return self._multi(PhaseS(), ts, cs)
    def t(self, i): return PhaseT().apply(self, [i], [])
    def t_multi(self, qs): return self._multi(PhaseT(), qs)
    def ct_multi(self, ts, cs): return self._multi(PhaseT(), ts, cs)
    def s_dag(self, i): return PhaseSdag().apply(self, [i], [])
    def s_dag_multi(self, qs): return self._multi(PhaseSdag(), qs)
    def t_dag(self, i): return PhaseTdag().apply(self, [i], [])
    def t_dag_multi(self, qs): return self._multi(PhaseTdag(), qs)
    def p(self, i, a): return PhaseShift(a).apply(self, [i], [])
    def p_multi(self, qs, a): return self._multi(PhaseShift(a), qs)
    def cp_multi(self, ts, cs, a): return self._multi(PhaseShift(a), ts, cs)
    def rx(self, i, a): return RotateX(a).apply(self, [i], [])
    def rx_multi(self, qs, a): return self._multi(RotateX(a), qs)
    def crx_multi(self, ts, cs, a): return self._multi(RotateX(a), ts, cs)
    def ry(self, i, a): return RotateY(a).apply(self, [i], [])
    def ry_multi(self, qs, a): return self._multi(RotateY(a), qs)
    def cry_multi(self, ts, cs, a): return self._multi(RotateY(a), ts, cs)
    def rz(self, i, a): return RotateZ(a).apply(self, [i], [])
    def rz_multi(self, qs, a): return self._multi(RotateZ(a), qs)
    def crz_multi(self, ts, cs, a): return self._multi(RotateZ(a), ts, cs)
    def unitary(self, i, m): return Unitary2.new(m).apply(self, [i], [])
    def unitary_multi(self, qs, m): return self._multi(Unitary2.new(m), qs)
    def cunitary_multi(self, ts, cs, m): return self._multi(Unitary2.new(m), ts, cs)
    def ry_phase(self, i, th, ph): return Unitary2.from_ry_phase(th, ph).apply(self, [i], [])
    def ry_phase_dag(self, i, th, ph): return Unitary2.from_ry_phase_dagger(th, ph).apply(self, [i], [])
    # measurement (state.rs:525-784)
    def measure(self, basis=None, measured_qubits=(), seed=0):
        """One draw (splitmix64(seed)) in `basis`; an empty `measured_qubits` measures all
        qubits.  The State itself is unchanged; `new_state` of the result is collapsed."""
        b, u = _basis_args(basis)
        qs = [int(q) for q in measured_qubits] or list(range(self.num_qubits))
        with self._device() as d:
            o = _measure(d, qs, basis=b, custom=u, seed=seed)
            new = State._take(d, self.num_qubits)
        return MeasurementResult(basis or MeasurementBasis.Computational, qs, _bits(o, len(qs)), new)

    def measure_n(self, basis, measured_qubits, n, seed=0):
        """`n` draws (shot j uses splitmix64(seed + j)) from the same distribution.  Each
        result's `new_state` is collapsed on first read: measuring a copy with seed + j
        draws the same outcome."""
        if n == 0:
            raise _err(-1, 0)
        b, u = _basis_args(basis)
        qs = [int(q) for q in measured_qubits] or list(range(self.num_qubits))
        if b == "Computational":
            outs = _measure_n(self._resident(), n, qs, seed=seed)
        else:   # the basis change and its undo round the amplitudes: use a scratch copy
            with self._device() as d:
                outs = _measure_n(d, n, qs, basis=b, custom=u, seed=seed)
        label = basis or MeasurementBasis.Computational
        return [MeasurementResult(label, qs, _bits(int(o), len(qs)),
                                  _collapse=lambda j=j: self.measure(basis, qs, seed + j).new_state)
                for j, o in enumerate(outs)]

    def cnot(self, control, target): return CNOT().apply(self, [target], [control])   # state.rs:2230-2232
    def swap(self, q1, q2): return SWAP().apply(self, [q1, q2], [])
    def cswap(self, t1, t2, cs): return SWAP().apply(self, [t1, t2], list(cs))
    def toffoli(self, c1, c2, t): return Toffoli().apply(self, [t], [c1, c2])
    def matchgate(self, t, th, p1, p2): return Matchgate(th, p1, p2).apply(self, [t], [])
    def cmatchgate(self, t, th, p1, p2, cs): return Matchgate(th, p1, p2).apply(self, [t], list(cs))


# --------------------------------------------------------------- measurement
class MeasurementBasis:
    """`enum MeasurementBasis` (measurement.rs:76-86): Computational, X, Y, or
    Custom(U) for a 2x2 unitary U."""
    Computational = "Computational"
    X = "X"
    Y = "Y"

    @staticmethod
    def Custom(u):
        return ("Custom", np.asarray(u, dtype=np.complex128).reshape(2, 2))


def _basis_args(basis):
    if basis is None:
        return "Computational", None
    if isinstance(basis, tuple):
        return basis[0], basis[1]
    return basis, None


def _bits(o, m):
    return [(o >> k) & 1 for k in range(m)]


class MeasurementResult:
    """`MeasurementResult { basis, indices, outcomes, new_state }` (measurement.rs:13-25);
    outcomes[k] is the bit drawn for qubit indices[k]."""

    def __init__(self, basis, indices, outcomes, new_state=None, _collapse=None):
        self.basis, self.indices, self.outcomes = basis, list(indices), list(outcomes)
        self._new, self._collapse = new_state, _collapse

    @property
    def new_state(self):
        if self._new is None:
            self._new = self._collapse()
        return self._new

    def get_basis(self):
        return self.basis

    def get_indices(self):
        return self.indices

    def get_outcomes(self):
        return self.outcomes

    def get_new_state(self):
        return self.new_state


# ----------------------------------------------------------------- operators
class Operator:
    """`trait Operator` (operator.rs:151-190): apply(state, targets, controls) -> State."""
    KIND = None
    BASE = 1

    def params(self):
        return ()

    def base_qubits(self):
        return self.BASE

    def gate_row(self, targets, controls):
        gl = GateList()
        gl.add(self.KIND, list(targets), list(controls), list(self.params()))
        return gl.array()[0]

    def apply(self, state, target_qubits, control_qubits=()):
        row = self.gate_row(target_qubits, control_qubits)
        with state._device() as d:
            d.apply_gate(row)
            return State._take(d, state.num_qubits)


def _op(name, kind, base=1):
    return type(name, (Operator,), {"KIND": kind, "BASE": base})


Hadamard = _op("Hadamard", "H")
CNOT = _op("CNOT", "CNOT", 2)
SWAP = _op("SWAP", "SWAP", 2)
Toffoli = _op("Toffoli", "TOFFOLI", 3)
Identity = _op("Identity", "IDENTITY")
PhaseS = _op("PhaseS", "S")
PhaseT = _op("PhaseT", "T")
PhaseSdag = _op("PhaseSdag", "SDAG")
PhaseTdag = _op("PhaseTdag", "TDAG")


class _PauliOp(Operator):
    def __init__(self, kind):
        self.KIND = kind

    def __repr__(self):
        return self.KIND

    def to_pauli_string(self, q):
        return PauliString(1.0, {q: self})


class Pauli:
    X = _PauliOp("X")
    Y = _PauliOp("Y")
    Z = _PauliOp("Z")


class _Angle(Operator):
    def __init__(self, angle):
        self.angle = float(angle)

    def params(self):
        return (self.angle,)


PhaseShift = type("PhaseShift", (_Angle,), {"KIND": "P"})
RotateX = type("RotateX", (_Angle,), {"KIND": "RX"})
RotateY = type("RotateY", (_Angle,), {"KIND": "RY"})
RotateZ = type("RotateZ", (_Angle,), {"KIND": "RZ"})


class Matchgate(Operator):
    KIND = "MATCHGATE"
    BASE = 2

    def __init__(self, theta, phi1, phi2):
        self.theta, self.phi1, self.phi2 = float(theta), float(phi1), float(phi2)

    def params(self):
        return (self.theta, self.phi1, self.phi2)


class Unitary2(Operator):
    KIND = "U2"

    def __init__(self, matrix):
        m = np.asarray(matrix, dtype=np.complex128).reshape(2, 2)
        self.matrix = m

    @staticmethod
    def new(matrix):   # operator.rs:2092-2125
        u = Unitary2(matrix)
        flat = np.array([u.matrix[0, 0].real, u.matrix[0, 0].imag, u.matrix[0, 1].real, u.matrix[0, 1].imag,
                         u.matrix[1, 0].real, u.matrix[1, 0].imag, u.matrix[1, 1].real, u.matrix[1, 1].imag])
        check(lib.qi_unitary2_check(flat.ctypes.data_as(_abi._pd)))
        return u

    @staticmethod
    def from_ry_phase(theta, phi):
        u = Unitary2(np.eye(2))
        u.KIND, u._p = "RYPHASE", (float(theta), float(phi))
        return u

    @staticmethod
    def from_ry_phase_dagger(theta, phi):
        u = Unitary2(np.eye(2))
        u.KIND, u._p = "RYPHASE_DAG", (float(theta), float(phi))
        return u

    def params(self):
        if self.KIND != "U2":
            return self._p
        m = self.matrix
        return (m[0, 0].real, m[0, 0].imag, m[0, 1].real, m[0, 1].imag, m[1, 0].real, m[1, 0].imag, m[1, 1].real,
                m[1, 1].imag)


# ------------------------------------------------------------- Pauli strings
class PauliString:
    """`PauliString { ops: HashMap<usize, Pauli>, coefficient }` (pauli_string.rs:13-18)."""

    def __init__(self, coefficient, ops=None):
        self.coefficient = complex(coefficient)
        self.ops = dict(ops or {})

    def with_op(self, qubit, op):
        if qubit in self.ops:
            raise ValueError("Duplicate Pauli string operator for qubit: %d" % qubit)
        self.ops[qubit] = op
        return self

    def masks(self):
        x = z = 0
        for q, op in self.ops.items():
            k = op.KIND
            if k in ("X", "Y"):
                x |= 1 << q
            if k in ("Z", "Y"):
                z |= 1 << q
        return x, z

    def row(self):
        x, z = self.masks()
        a = np.zeros((), dtype=TERM_DTYPE)
        a["re"], a["im"], a["xmask"], a["zmask"] = self.coefficient.real, self.coefficient.imag, x, z
        return a

    def get_targets(self):
        return sorted(self.ops)

    def apply(self, state):
        with DeviceState(state.num_qubits, PRECISION) as o:
            _pauli_apply(o, state._resident(), self.row())
            return State._take(o, state.num_qubits)

    def apply_normalised(self, state):
        with state._device() as d:
            _pauli_norm(d, self.row())
            return State._take(d, state.num_qubits)

    def apply_exp_factor(self, state, factor):
        with state._device() as d:
            _pauli_exp_factor(d, self.row(), factor)
            return State._take(d, state.num_qubits)

    def apply_exp(self, state):
        return self.apply_exp_factor(state, 1.0)

    def apply_exp_neg_i_dt(self, state, dt):
        if self.coefficient.imag != 0.0:
            raise QuantIronError(-15, re=self.coefficient.real, im=self.coefficient.imag)
        return self.apply_exp_factor(state, complex(0.0, -dt))

    def hermitian_conjugate(self):
        return PauliString(self.coefficient.conjugate(), dict(self.ops))

    def __add__(self, other):
        return SumOp([self, other])

    def __mul__(self, c):
        return PauliString(self.coefficient * complex(c), dict(self.ops))

    __rmul__ = __mul__


class SumOp:
    """`SumOp { terms: Vec<PauliString> }` (pauli_string.rs:390-393)."""

    def __init__(self, terms=None):
        self.terms = list(terms or [])

    def num_terms(self):
        return len(self.terms)

    def with_term(self, t):
        self.terms.append(t)
        return self

    def rows(self):
        a = np.zeros(len(self.terms), dtype=TERM_DTYPE)
        for i, t in enumerate(self.terms):
            a[i] = t.row()
        return a

    def apply(self, state):
        with DeviceState(state.num_qubits, PRECISION) as o:
            _sumop_apply(o, state._resident(), self.rows())
            return State._take(o, state.num_qubits)

    def expectation_value(self, state):
        return _expect(state._resident(), self.rows())


# -------------------------------------------------------------- gates/circuit
class Gate:
    """`enum Gate` (gate.rs:13-52) as a gate-list row."""

    def __init__(self, row):
        self.row = row

    @staticmethod
    def operator(op, targets, controls=()):
        return Gate(op.gate_row(targets, controls))

    @staticmethod
    def new_measurement(qubit_indices, basis=None, seed=0):
        """Gate::new_measurement (gate.rs:63-65): State::measure in `basis` on the qubits (all
        of them when empty), keeping the collapsed state; `seed` seeds the outcome draw (the
        reference's draw is unseeded)."""
        name, u = _basis_args(basis)
        code = {"Computational": 0, "X": 1, "Y": 2, "Custom": 3}[name]
        return Gate(GateList().measure(list(qubit_indices), code, u, seed).array()[0])

    measurement = new_measurement

    @staticmethod
    def pauli_string(ps):
        x, z = ps.masks()
        gl = GateList().add("PAULI_STRING", [], [], [ps.coefficient.real, ps.coefficient.imag], xmask=x, zmask=z)
        return Gate(gl.array()[0])

    @staticmethod
    def pauli_time_evolution(ps, t):
        x, z = ps.masks()
        gl = GateList().add("PAULI_EVOLUTION", [], [], [ps.coefficient.real, ps.coefficient.imag, float(t)],
                            xmask=x, zmask=z)
        return Gate(gl.array()[0])

    def apply(self, state):
        return Circuit([self], state.num_qubits).execute(state)


class Circuit:
    """`Circuit { gates, num_qubits }` (circuit.rs:34-39)."""

    def __init__(self, gates, num_qubits):
        self.gates = list(gates)
        self.num_qubits = int(num_qubits)

    def gate_array(self):
        if not self.gates:
            return np.zeros(0, dtype=GATE_DTYPE)
        return np.stack([g.row if isinstance(g, Gate) else g for g in self.gates]).astype(GATE_DTYPE)

    def execute(self, initial_state):   # circuit.rs:160-172
        if initial_state.num_qubits != self.num_qubits:
            raise _err(-3, initial_state.num_qubits)
        plan = Plan(self.num_qubits, PRECISION, self.gate_array(), fusion=FUSION)
        with initial_state._device() as d:
            plan.execute(d)
            return State._take(d, self.num_qubits)

    def trace_execution(self, initial_state):   # circuit.rs:188-202
        if initial_state.num_qubits != self.num_qubits:
            raise _err(-3, initial_state.num_qubits)
        states = [initial_state.clone()]
        cur = initial_state
        for g in self.gates:
            cur = Circuit([g], self.num_qubits).execute(cur)
            states.append(cur)
        return states


def qft_circuit(qubits, num_qubits):
    """Subroutine::qft (subroutine.rs:90-112) as a Circuit."""
    gl = _qft(GateList(), list(qubits))
    return Circuit(list(gl.array()), num_qubits)


# -------------------------------------------------------------------- Trotter
def _trotter_call(hamiltonian, state, dt, steps, order):
    if hamiltonian.num_terms() == 0:
        raise _err(-3, 0)
    with state._device() as d:
        _trotter(d, hamiltonian.rows(), dt, steps, order)
        return State._take(d, state.num_qubits)


def first_order_trotter_step(hamiltonian, state, dt):
    return _trotter_call(hamiltonian, state, dt, 1, 1)


def second_order_trotter_step(hamiltonian, state, dt):
    return _trotter_call(hamiltonian, state, dt, 1, 2)


def trotter_evolve_state(hamiltonian, state, dt, num_steps, order="First"):
    return _trotter_call(hamiltonian, state, dt, num_steps, 1 if order in ("First", 1) else 2)
