"""quant-iron GB300 state-vector engine — Python binding of the C ABI.

The engine itself is `lib/libqi_gb300.so` (CUDA, sm_103a).  This package is a
thin ctypes layer over include/qi_engine.h:

  DeviceState        a device-resident state handle (qi_state_*)
  Plan               a compiled circuit (qi_plan_*), fused or per-gate
  circuit_execute    Circuit::execute on a resident state
  sumop_expectation / sumop_apply / pauli_* / trotter_evolve

`quant_iron` (the submodule) mirrors the reference crate's public API —
State, the Operator types, PauliString, SumOp, Circuit — on top of it.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import (F32, F64, FUSION_GREEDY, FUSION_LEARNED, FUSION_NONE, FUSION_PAULI_GROUPS, GATE_DTYPE, TERM_DTYPE,
                   QuantIronError, check, lib)

__all__ = ["DeviceState", "Plan", "circuit_execute", "sumop_expectation", "sumop_apply", "trotter_evolve",
           "launch_count", "F32", "F64", "FUSION_NONE", "FUSION_GREEDY", "FUSION_LEARNED",
           "FUSION_PAULI_GROUPS", "QuantIronError"]


def launch_count():
    """Kernels launched by the engine since it was loaded."""
    return int(lib.qi_launch_count())


def version():
    return lib.qi_version().decode()


def _as_c128(v):
    v = np.ascontiguousarray(v, dtype=np.complex128)
    return v


class DeviceState:
    """A 2^n-amplitude state resident in GPU memory (complex FP64 or FP32)."""

    def __init__(self, num_qubits, precision=F64):
        self.h = ctypes.c_void_p()
        check(lib.qi_state_create(int(num_qubits), int(precision), ctypes.byref(self.h)))
        self.n = int(num_qubits)
        self.precision = int(precision)

    @property
    def dim(self):
        return 1 << self.n

    def close(self):
        if self.h:
            lib.qi_state_destroy(self.h)
            self.h = ctypes.c_void_p()

    def release(self):
        """Hand the handle to a new owner: returns a DeviceState owning it and leaves this
        object empty (so a `with` block ending afterwards frees nothing)."""
        other = DeviceState.__new__(DeviceState)
        other.h, other.n, other.precision = self.h, self.n, self.precision
        self.h = ctypes.c_void_p()
        return other

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle):
        check(lib.qi_state_set_stream(self.h, ctypes.c_void_p(int(stream_handle) if stream_handle else 0)))

    def stream(self):
        s = ctypes.c_void_p()
        check(lib.qi_state_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def device_ptr(self):
        p = ctypes.c_void_p()
        check(lib.qi_state_device_ptr(self.h, ctypes.byref(p)))
        return p.value

    def wait_for(self, other):
        """Order this state's subsequent work behind the work issued so far on `other`."""
        check(lib.qi_state_wait(self.h, other.h))

    def synchronize(self):
        check(lib.qi_state_synchronize(self.h))

    def upload(self, amps):
        a = _as_c128(amps)
        if a.size != self.dim:
            raise ValueError("expected %d amplitudes, got %d" % (self.dim, a.size))
        check(lib.qi_state_upload(self.h, a.ctypes.data, a.size))

    def upload_ptr(self, host_ptr, num_amps):
        """Upload from a raw host pointer (e.g. pinned memory) of interleaved f64 pairs."""
        check(lib.qi_state_upload(self.h, ctypes.c_void_p(host_ptr), int(num_amps)))

    def download(self, out=None):
        if out is None:
            out = np.empty(self.dim, dtype=np.complex128)
        check(lib.qi_state_download(self.h, out.ctypes.data, out.size))
        return out

    def download_ptr(self, host_ptr, num_amps):
        check(lib.qi_state_download(self.h, ctypes.c_void_p(host_ptr), int(num_amps)))

    def upload_async(self, host_ptr, num_amps):
        """Upload from a page-locked host buffer on the copy engine, in this state's stream
        order; the buffer must stay untouched until synchronize()."""
        check(lib.qi_state_upload_async(self.h, ctypes.c_void_p(host_ptr), int(num_amps)))

    def download_async(self, host_ptr, num_amps):
        """Download into a page-locked host buffer on the copy engine; complete after
        synchronize()."""
        check(lib.qi_state_download_async(self.h, ctypes.c_void_p(host_ptr), int(num_amps)))

    def set_zero(self):
        check(lib.qi_state_set_zero(self.h))

    def set_basis(self, n):
        check(lib.qi_state_set_basis(self.h, int(n)))

    def set_plus(self):
        check(lib.qi_state_set_plus(self.h))

    def set_minus(self):
        check(lib.qi_state_set_minus(self.h))

    def set_ghz(self):
        check(lib.qi_state_set_ghz(self.h))

    def check_normalised(self):
        check(lib.qi_state_check_normalised(self.h))

    def copy_from(self, other):
        check(lib.qi_state_copy(self.h, other.h))

    def scale(self, c):
        c = complex(c)
        check(lib.qi_state_scale(self.h, c.real, c.imag))

    def axpy(self, a, x):
        a = complex(a)
        check(lib.qi_state_axpy(self.h, a.real, a.imag, x.h))

    def inner_product(self, other):
        out = (ctypes.c_double * 2)()
        check(lib.qi_state_inner_product(self.h, other.h, out))
        return complex(out[0], out[1])

    def compare(self, reference):
        """Errors of this state against `reference` (same size, any precisions; FP64 on the
        device): max amplitude error, squared distance, overlap <reference|self>, infidelity."""
        out = (ctypes.c_double * 4)()
        check(lib.qi_state_compare(self.h, reference.h, out))
        ov = complex(out[2], out[3])
        na, nb = self.norm_sqr(), reference.norm_sqr()
        return {"max_abs_err": out[0], "dist_sqr": out[1], "overlap": ov,
                "infidelity": 1.0 - abs(ov) ** 2 / (na * nb)}

    def norm_sqr(self):
        out = ctypes.c_double()
        check(lib.qi_state_norm_sqr(self.h, ctypes.byref(out)))
        return out.value

    def normalise(self):
        check(lib.qi_state_normalise(self.h))

    def amplitude(self, idx):
        out = (ctypes.c_double * 2)()
        check(lib.qi_state_amplitude(self.h, int(idx), out))
        return complex(out[0], out[1])

    def apply_gate(self, gate_row):
        g = np.ascontiguousarray(gate_row, dtype=GATE_DTYPE).reshape(())
        check(lib.qi_apply_gate(self.h, g.ctypes.data))


def tensor_product(out, a, b):
    check(lib.qi_state_tensor_product(out.h, a.h, b.h))


def _options(fusion, max_block_qubits=0, use_tensor_cores=0, renorm_every=0):
    return _abi.ExecOptions(int(fusion), int(max_block_qubits), int(use_tensor_cores), int(renorm_every))


def _theta_arg(theta):
    if theta is None:
        return None, 0, None
    t = np.ascontiguousarray(theta, dtype=np.float64)
    return t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), t.size, t


class Plan:
    """A validated, compiled gate list for one qubit count and precision."""

    def __init__(self, num_qubits, precision, gates, theta=None, fusion=FUSION_NONE, max_block_qubits=0,
                 use_tensor_cores=0, renorm_every=0):
        gates = np.ascontiguousarray(gates, dtype=GATE_DTYPE)
        self.num_qubits = int(num_qubits)
        self.h = ctypes.c_void_p()
        opts = _options(fusion, max_block_qubits, use_tensor_cores, renorm_every)
        tp, tn, self._keep = _theta_arg(theta)
        check(lib.qi_plan_create(int(num_qubits), int(precision), gates.ctypes.data if gates.size else None,
                                 gates.size, tp, tn, ctypes.byref(opts), ctypes.byref(self.h)))

    def execute(self, state):
        check(lib.qi_plan_execute(self.h, state.h))

    def stats(self):
        s = _abi.PlanStats()
        check(lib.qi_plan_stats_get(self.h, ctypes.byref(s)))
        return {"n_gates": s.n_gates, "n_kernels": s.n_kernels, "n_blocks_by_k": list(s.n_blocks_by_k),
                "predicted_us": s.predicted_us}

    def ops(self):
        """The plan's device operations: list of dicts (kind, k, targets, control_mask,
        xmask, zmask, matrix as complex numpy array)."""
        n = ctypes.c_int64()
        check(lib.qi_plan_num_ops(self.h, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            info = _abi.PlanOpInfo()
            check(lib.qi_plan_op_get(self.h, i, ctypes.byref(info), None, 0))
            buf = np.zeros(2 * max(1, info.n_matrix), dtype=np.float64)
            check(lib.qi_plan_op_get(self.h, i, ctypes.byref(info), buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     info.n_matrix))
            mat = buf[0::2][:info.n_matrix] + 1j * buf[1::2][:info.n_matrix]
            op = {"kind": info.kind, "k": info.k, "targets": list(info.targets)[:max(info.k, 0)],
                  "tensor_cores": info.tensor_cores,
                  "control_mask": info.control_mask, "xmask": info.xmask, "zmask": info.zmask,
                  "matrix": mat}
            if info.kind == 9 or (info.kind == 4 and info.phase_poly):   # 2^-64 turns; kind 4: after the block
                nq = self.num_qubits
                c0 = ctypes.c_uint64()
                a = np.zeros(nq, dtype=np.uint64)
                b = np.zeros(nq * nq, dtype=np.uint64)
                check(lib.qi_plan_op_phase_poly(self.h, i, ctypes.byref(c0), a.ctypes.data, b.ctypes.data))
                if info.kind == 9:
                    op["targets"] = [q for q in range(nq) if (info.zmask >> q) & 1]
                op["poly"] = (np.uint64(c0.value), a, b.reshape(nq, nq))
            if info.kind == 10:   # grouped Pauli exponentials: parity bases and their tables
                nt = ctypes.c_int32()
                rank = np.zeros(4, dtype=np.int32)
                basis = np.zeros(32, dtype=np.uint64)
                check(lib.qi_plan_op_pauli_group(self.h, i, ctypes.byref(nt), rank.ctypes.data, basis.ctypes.data))
                per = 4 if info.xmask else 1
                tables, off = [], 0
                for t in range(nt.value):
                    cnt = per << int(rank[t])
                    tab = mat[off:off + cnt]
                    tables.append((basis[8 * t:8 * t + rank[t]].copy(), tab.reshape(-1, 2, 2) if per == 4 else tab))
                    off += cnt
                op["group"] = tables
            if info.kind == 11:   # qubit permutation: out[j] = in[flip ^ sum_k bit_k(j) << source_bit[k]]
                src = np.zeros(self.num_qubits, dtype=np.int32)
                flip = ctypes.c_uint64()
                check(lib.qi_plan_op_bitperm(self.h, i, src.ctypes.data, ctypes.byref(flip)))
                op["source_bit"] = src
                op["flip"] = int(flip.value)
                op["targets"] = []
            out.append(op)
        return out

    def close(self):
        if self.h:
            lib.qi_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def circuit_execute(state, gates, theta=None, fusion=FUSION_NONE, max_block_qubits=0, use_tensor_cores=0,
                    renorm_every=0):
    """Circuit::execute (src/circuit.rs:160-172) on a resident state (in place)."""
    gates = np.ascontiguousarray(gates, dtype=GATE_DTYPE)
    opts = _options(fusion, max_block_qubits, use_tensor_cores, renorm_every)
    tp, tn, _keep = _theta_arg(theta)
    check(lib.qi_circuit_execute(state.h, gates.ctypes.data if gates.size else None, gates.size, tp, tn,
                                 ctypes.byref(opts)))


def _terms(terms):
    return np.ascontiguousarray(terms, dtype=TERM_DTYPE)


def sumop_expectation(state, terms):
    t = _terms(terms)
    out = (ctypes.c_double * 2)()
    check(lib.qi_sumop_expectation(state.h, t.ctypes.data if t.size else None, t.size, out))
    return complex(out[0], out[1])


def sumop_apply(out_state, in_state, terms):
    t = _terms(terms)
    check(lib.qi_sumop_apply(out_state.h, in_state.h, t.ctypes.data if t.size else None, t.size))


def pauli_apply(out_state, in_state, term_row):
    t = _terms(term_row).reshape(())
    check(lib.qi_pauli_apply(out_state.h, in_state.h, t.ctypes.data))


def pauli_apply_normalised(state, term_row):
    t = _terms(term_row).reshape(())
    check(lib.qi_pauli_apply_normalised(state.h, t.ctypes.data))


def pauli_apply_exp(state, term_row):
    t = _terms(term_row).reshape(())
    check(lib.qi_pauli_apply_exp(state.h, t.ctypes.data))


def pauli_apply_exp_factor(state, term_row, factor):
    t = _terms(term_row).reshape(())
    f = complex(factor)
    check(lib.qi_pauli_apply_exp_factor(state.h, t.ctypes.data, f.real, f.imag))


def pauli_apply_exp_neg_i_dt(state, term_row, dt):
    t = _terms(term_row).reshape(())
    check(lib.qi_pauli_apply_exp_neg_i_dt(state.h, t.ctypes.data, float(dt)))


def trotter_evolve(state, terms, dt, num_steps, order=1, observable=None, observe_every=0):
    """trotter_evolve_state (src/algorithms/time_evolution.rs:140-166); returns the
    list of <observable> values taken every `observe_every` steps."""
    t = _terms(terms)
    nobs = 0
    obs_ptr = None
    energies = None
    if observable is not None and observe_every > 0:
        o = _terms(observable)
        obs_ptr = o.ctypes.data
        nobs = o.size
        energies = np.zeros(2 * max(1, num_steps // observe_every), dtype=np.float64)
    check(lib.qi_trotter_evolve(state.h, t.ctypes.data if t.size else None, t.size, float(dt), int(num_steps),
                                int(order), obs_ptr, nobs, int(observe_every),
                                energies.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if energies is not None
                                else None))
    if energies is None:
        return []
    return [complex(energies[2 * k], energies[2 * k + 1]) for k in range(num_steps // observe_every)]


# op kind -> the kernels one op launches (8, the renormalisation: k_norm_partial first, unless a
# qubit permutation just before it summed the norm as it wrote)
KERNEL_OF_OP_KIND = {1: "k_mat1", 2: "k_swap", 3: "k_mat2", 4: "k_fused", 5: "k_pauli_exp", 6: "k_pauli_exp+normalise",
                     7: "k_diagk", 8: "k_finalize+k_normalise_apply|to", 9: "k_phase_poly",
                     10: "k_pauli_group_diag|k_pauli_group_pair", 11: "k_bitperm"}


def plan_profile(plan, state):
    """Run `plan` once on `state` with CUDA events around every op (on the state's
    stream); returns (ops, per-op milliseconds)."""
    ops = plan.ops()
    ms = (ctypes.c_float * max(1, len(ops)))()
    check(lib.qi_plan_profile(plan.h, state.h, ms))
    return ops, [float(ms[i]) for i in range(len(ops))]


def apply_matrix(state, targets, matrix, use_tensor_cores=0):
    """Dense 2^k x 2^k matrix on `targets` (local bit j <-> targets[j]), one HBM pass."""
    t = np.ascontiguousarray(targets, dtype=np.int32)
    m = np.ascontiguousarray(matrix, dtype=np.complex128).reshape(-1).view(np.float64)
    check(lib.qi_apply_matrix(state.h, t.ctypes.data, t.size, m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              int(use_tensor_cores)))


def _basis_args(basis, custom):
    b = _abi.BASIS[basis] if isinstance(basis, str) else int(basis)
    u = None
    if custom is not None:
        m = np.asarray(custom, dtype=np.complex128).reshape(2, 2)
        u = np.array([m[0, 0].real, m[0, 0].imag, m[0, 1].real, m[0, 1].imag, m[1, 0].real, m[1, 0].imag,
                      m[1, 1].real, m[1, 1].imag])
    return b, u


def tf32_rate_probe(iters=16384, reps=5):
    """Dense tcgen05 kind::tf32 rate of the current GPU: (TFLOP/s, ms of the best launch)."""
    tf = ctypes.c_double()
    ms = ctypes.c_double()
    check(lib.qi_tf32_rate_probe(int(iters), int(reps), ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value, ms.value


def splitmix_uniform(seed):
    """The uniform draw qi_measure uses for `seed`: (splitmix64(seed) >> 11) * 2^-53."""
    m = (1 << 64) - 1
    x = (seed + 0x9E3779B97F4A7C15) & m
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
    x ^= x >> 31
    return (x >> 11) * 2.0 ** -53


def measure(state, qubits=(), basis="Computational", custom=None, seed=0, return_probs=False):
    """State::measure on the device (state collapses in place); returns the outcome integer
    (bit k = qubit qubits[k]) and optionally the normalised probabilities."""
    b, u = _basis_args(basis, custom)
    q = np.ascontiguousarray(qubits, dtype=np.int32)
    m = q.size if q.size else state.n
    out = ctypes.c_uint64()
    probs = np.zeros(1 << m, dtype=np.float64) if return_probs else None
    pd = ctypes.POINTER(ctypes.c_double)
    check(lib.qi_measure(state.h, b, u.ctypes.data_as(pd) if u is not None else None, q.ctypes.data if q.size else None,
                         q.size, int(seed), ctypes.byref(out), probs.ctypes.data_as(pd) if probs is not None else None))
    return (out.value, probs) if return_probs else out.value


def measure_n(state, n_shots, qubits=(), basis="Computational", custom=None, seed=0):
    """State::measure_n: n_shots outcomes of the same distribution; the state is unchanged."""
    b, u = _basis_args(basis, custom)
    q = np.ascontiguousarray(qubits, dtype=np.int32)
    out = np.zeros(max(int(n_shots), 1), dtype=np.uint64)
    pd = ctypes.POINTER(ctypes.c_double)
    check(lib.qi_measure_n(state.h, b, u.ctypes.data_as(pd) if u is not None else None, q.ctypes.data if q.size else None,
                           q.size, int(n_shots), int(seed), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out[:n_shots]


SWEEP_GATE, SWEEP_GROUP, SWEEP_AFFINE, SWEEP_PLAN, SWEEP_SKIP = 0, 1, 2, 3, 4


def adjoint_sweep_plan(num_qubits, precision, gates, theta, fusion=FUSION_GREEDY):
    """The reverse sweep's passes for this gate list (host only): list of (kind, hi, lo), each
    pass covering gates hi, hi - 1, ..., lo + 1; kinds SWEEP_GATE / GROUP / AFFINE / PLAN / SKIP."""
    gates = np.ascontiguousarray(gates, dtype=GATE_DTYPE)
    t = np.ascontiguousarray(theta, dtype=np.float64)
    opts = _options(fusion, 0, 0)
    pd = ctypes.POINTER(ctypes.c_double)
    count = ctypes.c_int64()
    args = (num_qubits, precision, gates.ctypes.data if gates.size else None, gates.size, t.ctypes.data_as(pd), t.size,
            ctypes.byref(opts))
    check(lib.qi_adjoint_sweep_plan(*args, None, None, None, 0, ctypes.byref(count)))
    kinds = np.zeros(max(1, count.value), dtype=np.int32)
    hi = np.zeros(max(1, count.value), dtype=np.int64)
    lo = np.zeros(max(1, count.value), dtype=np.int64)
    check(lib.qi_adjoint_sweep_plan(*args, kinds.ctypes.data, hi.ctypes.data, lo.ctypes.data, count.value,
                                    ctypes.byref(count)))
    return [(int(kinds[i]), int(hi[i]), int(lo[i])) for i in range(count.value)]


def adjoint_gradient(state, gates, theta, terms, fusion=FUSION_GREEDY, max_block_qubits=0, use_tensor_cores=0,
                     renorm_every=0):
    """dE/dtheta of E = <psi(theta)|H|psi(theta)> by one forward and one reverse sweep.
    `state` holds |psi0> before and after the call.  Returns (E, grads)."""
    gates = np.ascontiguousarray(gates, dtype=GATE_DTYPE)
    t = np.ascontiguousarray(theta, dtype=np.float64)
    h = _terms(terms)
    grads = np.zeros(t.size, dtype=np.float64)
    energy = ctypes.c_double()
    opts = _options(fusion, max_block_qubits, use_tensor_cores, renorm_every)
    pd = ctypes.POINTER(ctypes.c_double)
    check(lib.qi_adjoint_gradient(state.h, gates.ctypes.data if gates.size else None, gates.size, t.ctypes.data_as(pd),
                                  t.size, h.ctypes.data if h.size else None, h.size, ctypes.byref(opts),
                                  ctypes.byref(energy), grads.ctypes.data_as(pd)))
    return energy.value, grads
