"""Seeded synthetic workloads with the shapes of the benchmark configurations.

All randomness comes from numpy.random.Generator(PCG64(seed)); the draw order
is documented per function so that the same lists can be rebuilt anywhere.

random_circuit     random single-qubit layers + CNOT brickwork + QFT
                   (20 qubits: 1400 gates; 30 qubits: 2260 gates)
heisenberg_open_chain   1D open-chain Heisenberg SumOp with Z fields
lattice_xyz / lattice_tfim   5x6 open-lattice anisotropic Heisenberg and TFIM
xxz_periodic       1D periodic XXZ SumOp with Z fields
hea_ansatz         RY/RZ layers + linear CNOT ladder, all angles parametric
"""
import math

import numpy as np

from ._types import GATE_DTYPE, GATE_KINDS, TERM_DTYPE

ONE_QUBIT_SET = ["H", "X", "Y", "Z", "S", "T", "RX", "RY", "RZ", "P"]
PARAMETRIC = {"RX", "RY", "RZ", "P"}


class GateList:
    """Append-only builder of a qi_gate array (the C struct layout)."""

    def __init__(self):
        self._rows = []

    def add(self, kind, targets, controls=(), params=(), param_ids=(), xmask=0, zmask=0):
        g = np.zeros((), dtype=GATE_DTYPE)
        g["kind"] = GATE_KINDS[kind] if isinstance(kind, str) else int(kind)
        g["n_targets"] = len(targets)
        g["targets"][:len(targets)] = targets
        g["n_controls"] = len(controls)
        g["controls"][:len(controls)] = controls
        g["params"][:len(params)] = params
        g["param_ids"][:] = -1
        g["param_ids"][:len(param_ids)] = param_ids
        g["xmask"] = xmask
        g["zmask"] = zmask
        self._rows.append(g)
        return self

    def measure(self, qubits, basis=0, custom=None, seed=0):
        """Gate::Measurement(basis, qubits): basis 0 computational, 1 X, 2 Y, 3 custom (2x2
        complex matrix `custom`); `seed` seeds the outcome draw."""
        g = np.zeros((), dtype=GATE_DTYPE)
        g["kind"] = GATE_KINDS["MEASUREMENT"]
        g["n_targets"] = 0
        g["targets"][0] = int(basis)
        g["n_controls"] = len(qubits)
        g["controls"][:len(qubits)] = qubits
        g["param_ids"][:] = -1
        if custom is not None:
            u = np.asarray(custom, dtype=np.complex128).reshape(4)
            g["params"][0::2] = u.real
            g["params"][1::2] = u.imag
        g["xmask"] = np.uint64(seed)
        self._rows.append(g)
        return self

    def array(self):
        if not self._rows:
            return np.zeros(0, dtype=GATE_DTYPE)
        return np.stack(self._rows).astype(GATE_DTYPE)

    def __len__(self):
        return len(self._rows)


def qft(gl, qubits):
    """Subroutine::qft gate order (src/subroutine.rs:90-112): for each i, H(q_i)
    then CP(pi/2^k) with target q_i and control q_{i+k}; then swaps."""
    n = len(qubits)
    for i in range(n):
        gl.add("H", [qubits[i]])
        denom = 2.0
        for k in range(1, n - i):
            gl.add("P", [qubits[i]], [qubits[i + k]], [math.pi / denom])
            denom *= 2.0
    for i in range(n // 2):
        gl.add("SWAP", [qubits[i], qubits[n - 1 - i]])
    return gl


def random_circuit(n, layers=40, seed=0, with_qft=True):
    """Random-circuit family of the benchmark: `layers` layers, each one gate per
    qubit q = 0..n-1 drawn uniformly from {H,X,Y,Z,S,T,RX,RY,RZ,P} (draw:
    integers(0, 10); then, for RX/RY/RZ/P, uniform(0, 2*pi)), then CNOTs on the
    brickwork pairs (control 2j+o, target 2j+1+o) with o = layer % 2; then the
    QFT on all qubits.  Returns a qi_gate array."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gl = GateList()
    for layer in range(layers):
        for q in range(n):
            name = ONE_QUBIT_SET[int(rng.integers(0, 10))]
            if name in PARAMETRIC:
                gl.add(name, [q], [], [float(rng.uniform(0.0, 2.0 * math.pi))])
            else:
                gl.add(name, [q])
        off = layer % 2
        j = 0
        while 2 * j + 1 + off < n:
            gl.add("CNOT", [2 * j + 1 + off], [2 * j + off])
            j += 1
    if with_qft:
        qft(gl, list(range(n)))
    return gl.array()


def plus_state(n):
    """State::new_plus (state.rs:225-237) as interleaved complex128."""
    return np.full(1 << n, 1.0 / math.sqrt(1 << n), dtype=np.complex128)


def zero_state(n):
    v = np.zeros(1 << n, dtype=np.complex128)
    v[0] = 1.0
    return v


def basis_state(n, idx):
    v = np.zeros(1 << n, dtype=np.complex128)
    v[idx] = 1.0
    return v


def term(coeff, ops):
    """One Pauli term; ops: list of (qubit, 'X'|'Y'|'Z')."""
    x = z = 0
    for q, p in ops:
        if p in ("X", "Y"):
            x |= 1 << q
        if p in ("Z", "Y"):
            z |= 1 << q
    c = complex(coeff)
    return (c.real, c.imag, x, z)


def terms_array(terms):
    a = np.zeros(len(terms), dtype=TERM_DTYPE)
    for i, (re, im, x, z) in enumerate(terms):
        a[i] = (re, im, x, z)
    return a


def heisenberg_open_chain(n, seed=0, j=(1.0, 1.0, 1.0)):
    """sum_{i<n-1} (Jx X_iX_{i+1} + Jy Y_iY_{i+1} + Jz Z_iZ_{i+1}) + sum_i h_i Z_i,
    h_i ~ U(-1, 1) from PCG64(seed) (n draws, i ascending).  Terms: bonds in
    order (XX, YY, ZZ per bond), then fields."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = rng.uniform(-1.0, 1.0, size=n)
    out = []
    for i in range(n - 1):
        out.append(term(j[0], [(i, "X"), (i + 1, "X")]))
        out.append(term(j[1], [(i, "Y"), (i + 1, "Y")]))
        out.append(term(j[2], [(i, "Z"), (i + 1, "Z")]))
    for i in range(n):
        out.append(term(h[i], [(i, "Z")]))
    return terms_array(out)


def lattice_bonds(rows=5, cols=6):
    """Open rows x cols lattice, site r*cols + c: horizontal bonds then vertical."""
    bonds = []
    for r in range(rows):
        for c in range(cols - 1):
            bonds.append((r * cols + c, r * cols + c + 1))
    for r in range(rows - 1):
        for c in range(cols):
            bonds.append((r * cols + c, (r + 1) * cols + c))
    return bonds


def lattice_xyz(rows=5, cols=6, seed=0, j=(1.0, 0.8, 0.5)):
    """Anisotropic Heisenberg on the open lattice: per bond Jx XX + Jy YY + Jz ZZ,
    then h_i Z_i with h ~ U(-1, 1) from PCG64(seed).  5x6: 49 bonds, 177 terms."""
    n = rows * cols
    rng = np.random.Generator(np.random.PCG64(seed))
    h = rng.uniform(-1.0, 1.0, size=n)
    out = []
    for a, b in lattice_bonds(rows, cols):
        out.append(term(j[0], [(a, "X"), (b, "X")]))
        out.append(term(j[1], [(a, "Y"), (b, "Y")]))
        out.append(term(j[2], [(a, "Z"), (b, "Z")]))
    for i in range(n):
        out.append(term(h[i], [(i, "Z")]))
    return terms_array(out)


def lattice_tfim(rows=5, cols=6, seed=0, g=1.0):
    """Transverse-field Ising H = -sum J_ij Z_iZ_j - g sum X_i on the open lattice,
    J_ij ~ U(0.5, 1.5) from PCG64(seed) (one draw per bond, bond order).  5x6: 79 terms."""
    n = rows * cols
    rng = np.random.Generator(np.random.PCG64(seed))
    bonds = lattice_bonds(rows, cols)
    jv = rng.uniform(0.5, 1.5, size=len(bonds))
    out = [term(-jv[k], [(a, "Z"), (b, "Z")]) for k, (a, b) in enumerate(bonds)]
    out += [term(-g, [(i, "X")]) for i in range(n)]
    return terms_array(out)


def xxz_periodic(n, seed=1, jz=0.5):
    """Periodic XXZ: sum_i (X_iX_{i+1} + Y_iY_{i+1} + jz Z_iZ_{i+1}) (i+1 mod n)
    + sum_i h_i Z_i, h ~ U(-1, 1) from PCG64(seed).  n = 26: 104 terms."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = rng.uniform(-1.0, 1.0, size=n)
    out = []
    for i in range(n):
        k = (i + 1) % n
        out.append(term(1.0, [(i, "X"), (k, "X")]))
        out.append(term(1.0, [(i, "Y"), (k, "Y")]))
        out.append(term(jz, [(i, "Z"), (k, "Z")]))
    for i in range(n):
        out.append(term(h[i], [(i, "Z")]))
    return terms_array(out)


def hea_ansatz(n, layers=12, seed=1):
    """Hardware-efficient ansatz: per layer RY(theta) then RZ(phi) on every qubit
    (qubit order), then CNOT(control q, target q+1) for q = 0..n-2.  Every angle
    is a parameter: param id = 2*(layer*n + q) for RY, +1 for RZ.  Initial
    values theta, phi ~ U(-pi, pi) from PCG64(seed), drawn in param-id order.
    Returns (gate array, theta vector)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    npar = 2 * layers * n
    theta = rng.uniform(-math.pi, math.pi, size=npar)
    gl = GateList()
    for layer in range(layers):
        for q in range(n):
            pid = 2 * (layer * n + q)
            gl.add("RY", [q], [], [theta[pid]], [pid])
            gl.add("RZ", [q], [], [theta[pid + 1]], [pid + 1])
        for q in range(n - 1):
            gl.add("CNOT", [q + 1], [q])
    return gl.array(), theta
