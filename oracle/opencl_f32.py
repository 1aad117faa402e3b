"""FP32 restatement of the reference crate's OpenCL gate kernels (its GPU path).

TEST INFRASTRUCTURE ONLY — a second checker beside the FP64 CPU restatement in
qi_oracle.cpp; never called by the engine.

With the `gpu` feature the crate runs a gate on the device when the state has
at least 15 qubits (OPENCL_THRESHOLD_NUM_QUBITS, src/components/operator.rs:21):
`execute_on_gpu` (operator.rs:24-148) rounds the FP64 state to `float2`, runs
one kernel from src/components/kernels/*.cl and widens the result back to FP64.
Gates without a kernel (Unitary2 and its ry_phase forms, Identity) stay on the
FP64 CPU branch.  Each function below restates one kernel's per-element
arithmetic in numpy float32 (one rounding per operation, no fused multiply-add,
so agreement with an OpenCL device is to FP32 rounding, not bit for bit):

  hadamard.cl       (a0 + a1) * 0.70710678118f, (a0 - a1) * 0.70710678118f
  pauli_x.cl        swap; pauli_y.cl (Im a1, -Re a1), (-Im a0, Re a0); pauli_z.cl negate
  phase_s_sdag.cl   (-sign Im a, sign Re a)
  phase_shift.cl    a * (cos, sin) for P(angle), T (pi/4), T-dagger (-pi/4)
  rotate_x.cl, rotate_y.cl, rotate_z.cl   with cos / sin of the half angle
  swap.cl           swap the pair with bit q_low = 1, bit q_high = 0
  match_gate.cl     new_a10 = s a01 + e^{i phi2} c a10  (the CPU branch,
                    operator.rs:962-963, uses e^{i phi1}: the documented
                    discrepancy of the reference GPU path), new_a11 = a11 e^{i phi2}

Controls are tested on the pair's |..0..> index (i00 for the matchgate), which
equals the CPU branch's test because validation keeps controls off the targets.
"""
import math

import numpy as np

from . import oracle as _cpu

GPU_THRESHOLD_QUBITS = 15          # operator.rs:21
_K = dict(H=0, X=1, Y=2, Z=3, S=4, T=5, SDAG=6, TDAG=7, P=8, RX=9, RY=10, RZ=11, U2=12, RYPHASE=13,
          RYPHASE_DAG=14, CNOT=15, SWAP=16, MATCHGATE=17, TOFFOLI=18, IDENTITY=19)
_F = np.float32


def _ctrl_ok(idx, controls):
    ok = np.ones(idx.shape, dtype=bool)
    for c in controls:
        ok &= ((idx >> np.uint64(c)) & np.uint64(1)).astype(bool)
    return ok


def _pairs(n, t, controls):
    idx = np.arange(1 << n, dtype=np.uint64)
    i0 = idx[(idx >> np.uint64(t)) & np.uint64(1) == 0]
    i0 = i0[_ctrl_ok(i0, controls)]
    return i0, i0 | np.uint64(1 << t)


def _ones(n, t, controls):
    idx = np.arange(1 << n, dtype=np.uint64)
    sel = idx[(idx >> np.uint64(t)) & np.uint64(1) == 1]
    return sel[_ctrl_ok(sel, controls)]


def hadamard(re, im, n, t, controls):            # hadamard.cl:1-53
    i0, i1 = _pairs(n, t, controls)
    k = _F(0.70710678118)
    r0, m0, r1, m1 = re[i0], im[i0], re[i1], im[i1]
    re[i0], im[i0] = k * (r0 + r1), k * (m0 + m1)
    re[i1], im[i1] = k * (r0 - r1), k * (m0 - m1)


def pauli_x(re, im, n, t, controls):             # pauli_x.cl:1-32
    i0, i1 = _pairs(n, t, controls)
    re[i0], re[i1] = re[i1].copy(), re[i0].copy()
    im[i0], im[i1] = im[i1].copy(), im[i0].copy()


def pauli_y(re, im, n, t, controls):             # pauli_y.cl:1-31
    i0, i1 = _pairs(n, t, controls)
    r0, m0, r1, m1 = re[i0], im[i0], re[i1], im[i1]
    re[i0], im[i0] = m1, -r1
    re[i1], im[i1] = -m0, r0


def pauli_z(re, im, n, t, controls):             # pauli_z.cl:1-31
    s = _ones(n, t, controls)
    re[s], im[s] = -re[s], -im[s]


def phase_s_sdag(re, im, n, t, controls, sign):  # phase_s_sdag.cl:1-38
    s = _ones(n, t, controls)
    sg = _F(sign)
    r, m = re[s], im[s]
    re[s], im[s] = -sg * m, sg * r


def phase_shift(re, im, n, t, controls, angle):  # phase_shift.cl:1-37
    s = _ones(n, t, controls)
    c, sn = _F(math.cos(angle)), _F(math.sin(angle))
    r, m = re[s], im[s]
    re[s], im[s] = r * c - m * sn, r * sn + m * c


def rotate_x(re, im, n, t, controls, angle):     # rotate_x.cl:1-54
    i0, i1 = _pairs(n, t, controls)
    c, s = _F(math.cos(angle / 2.0)), _F(math.sin(angle / 2.0))
    r0, m0, r1, m1 = re[i0], im[i0], re[i1], im[i1]
    re[i0], im[i0] = c * r0 + s * m1, c * m0 - s * r1
    re[i1], im[i1] = s * m0 + c * r1, -s * r0 + c * m1


def rotate_y(re, im, n, t, controls, angle):     # rotate_y.cl:1-43
    i0, i1 = _pairs(n, t, controls)
    c, s = _F(math.cos(angle / 2.0)), _F(math.sin(angle / 2.0))
    r0, m0, r1, m1 = re[i0], im[i0], re[i1], im[i1]
    re[i0], im[i0] = c * r0 - s * r1, c * m0 - s * m1
    re[i1], im[i1] = s * r0 + c * r1, s * m0 + c * m1


def rotate_z(re, im, n, t, controls, angle):     # rotate_z.cl:1-44
    idx = np.arange(1 << n, dtype=np.uint64)
    sel = idx[_ctrl_ok(idx, controls)]
    c, s = _F(math.cos(angle / 2.0)), _F(math.sin(angle / 2.0))
    one = ((sel >> np.uint64(t)) & np.uint64(1)).astype(bool)
    pi = np.where(one, s, -s).astype(_F)
    r, m = re[sel], im[sel]
    re[sel], im[sel] = r * c - m * pi, r * pi + m * c


def swap(re, im, n, q1, q2, controls):           # swap.cl:1-84
    lo, hi = min(q1, q2), max(q1, q2)
    idx = np.arange(1 << n, dtype=np.uint64)
    i = idx[(((idx >> np.uint64(lo)) & np.uint64(1)) == 1) & (((idx >> np.uint64(hi)) & np.uint64(1)) == 0)]
    i = i[_ctrl_ok(i, controls)]
    j = i ^ np.uint64((1 << lo) | (1 << hi))
    re[i], re[j] = re[j].copy(), re[i].copy()
    im[i], im[j] = im[j].copy(), im[i].copy()


def _cmul(ar, ai, br, bi):                       # match_gate.cl:2-4
    return ar * br - ai * bi, ar * bi + ai * br


def match_gate(re, im, n, q1, controls, theta, phi1, phi2):   # match_gate.cl:21-92
    q2 = q1 + 1
    idx = np.arange(1 << n, dtype=np.uint64)
    base = idx[(((idx >> np.uint64(q1)) & np.uint64(1)) == 0) & (((idx >> np.uint64(q2)) & np.uint64(1)) == 0)]
    base = base[_ctrl_ok(base, controls)]
    i01, i10 = base | np.uint64(1 << q1), base | np.uint64(1 << q2)
    i11 = i01 | i10
    c, s = _F(math.cos(theta / 2.0)), _F(math.sin(theta / 2.0))
    e1r, e1i = _F(math.cos(phi1)), _F(math.sin(phi1))
    e2r, e2i = _F(math.cos(phi2)), _F(math.sin(phi2))
    r01, m01, r10, m10, r11, m11 = re[i01], im[i01], re[i10], im[i10], re[i11], im[i11]
    t2r, t2i = _cmul(e1r, e1i, s * r10, s * m10)
    n01r, n01i = c * r01 - t2r, c * m01 - t2i
    t4r, t4i = _cmul(e2r, e2i, c * r10, c * m10)
    n10r, n10i = s * r01 + t4r, s * m01 + t4i
    n11r, n11i = _cmul(r11, m11, e2r, e2i)
    re[i01], im[i01] = n01r, n01i
    re[i10], im[i10] = n10r, n10i
    re[i11], im[i11] = n11r, n11i


def apply_gate(state, n, gate):
    """One operator gate as the reference runs it with the `gpu` feature: the OpenCL
    kernel's FP32 arithmetic at n >= 15 qubits when the gate has a kernel, else the
    FP64 CPU branch (the FP64 oracle)."""
    g = np.asarray(gate).reshape(())
    kind = int(g["kind"])
    if n < GPU_THRESHOLD_QUBITS or kind in (_K["U2"], _K["RYPHASE"], _K["RYPHASE_DAG"], _K["IDENTITY"]):
        return _cpu.apply_gate(state, n, g)
    if kind not in _K.values():
        raise NotImplementedError("gate kind %d has no restated kernel" % kind)
    v = np.ascontiguousarray(state, dtype=np.complex128)
    re, im = v.real.astype(_F), v.imag.astype(_F)   # execute_on_gpu: c.re as f32, c.im as f32
    t = int(g["targets"][0])
    ctl = [int(c) for c in g["controls"][:int(g["n_controls"])]]
    a = float(g["params"][0])
    if kind == _K["H"]:
        hadamard(re, im, n, t, ctl)
    elif kind in (_K["X"], _K["CNOT"], _K["TOFFOLI"]):   # CNOT and Toffoli delegate to Pauli X
        pauli_x(re, im, n, t, ctl)
    elif kind == _K["Y"]:
        pauli_y(re, im, n, t, ctl)
    elif kind == _K["Z"]:
        pauli_z(re, im, n, t, ctl)
    elif kind in (_K["S"], _K["SDAG"]):
        phase_s_sdag(re, im, n, t, ctl, 1.0 if kind == _K["S"] else -1.0)
    elif kind in (_K["T"], _K["TDAG"], _K["P"]):
        phase_shift(re, im, n, t, ctl, math.pi / 4.0 if kind == _K["T"] else -math.pi / 4.0 if kind == _K["TDAG"] else a)
    elif kind == _K["RX"]:
        rotate_x(re, im, n, t, ctl, a)
    elif kind == _K["RY"]:
        rotate_y(re, im, n, t, ctl, a)
    elif kind == _K["RZ"]:
        rotate_z(re, im, n, t, ctl, a)
    elif kind == _K["SWAP"]:
        swap(re, im, n, t, int(g["targets"][1]), ctl)
    elif kind == _K["MATCHGATE"]:
        match_gate(re, im, n, t, ctl, a, float(g["params"][1]), float(g["params"][2]))
    return re.astype(np.float64) + 1j * im.astype(np.float64)


def execute(state, n, gates):
    """Circuit::execute (circuit.rs:160-172) gate by gate through apply_gate."""
    s = np.ascontiguousarray(state, dtype=np.complex128)
    for g in np.asarray(gates):
        s = apply_gate(s, n, g)
    return s
