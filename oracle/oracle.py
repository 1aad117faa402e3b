"""ctypes wrapper of oracle/_build/libqi_oracle.so (built from oracle/qi_oracle.cpp).

TEST INFRASTRUCTURE ONLY — the checker for the CUDA engine, never the thing
measured or shipped.  Each function restates the reference crate's sequential
CPU semantics; see qi_oracle.cpp for the file:line each one follows.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libqi_oracle.so")


def _load():
    if not os.path.exists(LIB_PATH):
        import sys
        sys.path.insert(0, os.path.dirname(_HERE))
        import __graft_entry__
        __graft_entry__.build_oracle()
    return ctypes.CDLL(LIB_PATH)


lib = _load()
_vp, _i32, _i64, _d = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_pd = ctypes.POINTER(ctypes.c_double)
_sig = {
    "oracle_last_error": (None, [ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "oracle_apply_gate": (_i32, [_vp, _i32, _vp]),
    "oracle_execute": (_i32, [_vp, _i32, _vp, _i64, _vp, ctypes.POINTER(_i64)]),
    "oracle_pauli_apply": (_i32, [_vp, _vp, _i32, _vp]),
    "oracle_pauli_apply_normalised": (_i32, [_vp, _i32, _vp]),
    "oracle_pauli_apply_exp_factor": (_i32, [_vp, _i32, _vp, _d, _d]),
    "oracle_sumop_apply": (_i32, [_vp, _vp, _i32, _vp, _i64]),
    "oracle_sumop_expectation": (_i32, [_vp, _i32, _vp, _i64, _pd]),
    "oracle_inner_product": (None, [_vp, _vp, _i32, _pd]),
    "oracle_normalise": (_i32, [_vp, _i32]),
    "oracle_tensor_product": (None, [_vp, _vp, _i32, _vp, _i32]),
    "oracle_trotter": (_i32, [_vp, _i32, _vp, _i64, _d, _i64, _i32]),
    "oracle_measure": (_i32, [_vp, _i32, _vp, _i32, _d, ctypes.POINTER(_i64), _vp]),
    "oracle_unitary2_check": (_i32, [_pd]),
    "oracle_port_execute": (_d, [_vp, _i32, _vp, _i64, _i32]),
    "oracle_port_execute_timed": (_d, [_vp, _i32, _vp, _i64, _i32, _pd]),
}
for _n, (_r, _a) in _sig.items():
    f = getattr(lib, _n)
    f.restype = _r
    f.argtypes = _a


class OracleError(Exception):
    def __init__(self, code, a, b):
        self.code, self.a, self.b = code, a, b
        super().__init__("oracle status %d (%d, %d)" % (code, a, b))


def _check(st):
    if st != 0:
        a, b = _i64(), _i64()
        lib.oracle_last_error(ctypes.byref(a), ctypes.byref(b))
        raise OracleError(st, a.value, b.value)


def _vec(v):
    return np.array(v, dtype=np.complex128, copy=True, order="C")


def _gates(gates):
    from numpy.lib import recfunctions  # noqa: F401  (keeps numpy structured arrays importable)
    g = np.ascontiguousarray(gates)
    return g


def apply_gate(state, n, gate):
    s = _vec(state)
    g = np.ascontiguousarray(gate).reshape(())
    _check(lib.oracle_apply_gate(s.ctypes.data, n, g.ctypes.data))
    return s


def execute(state, n, gates, theta=None):
    s = _vec(state)
    g = np.ascontiguousarray(gates)
    t = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    failed = _i64(-1)
    _check(lib.oracle_execute(s.ctypes.data, n, g.ctypes.data if g.size else None, g.size,
                              t.ctypes.data if t is not None else None, ctypes.byref(failed)))
    return s


def pauli_apply(state, n, term_row):
    s = np.ascontiguousarray(state, dtype=np.complex128)
    out = np.empty_like(s)
    t = np.ascontiguousarray(term_row).reshape(())
    _check(lib.oracle_pauli_apply(out.ctypes.data, s.ctypes.data, n, t.ctypes.data))
    return out


def pauli_apply_normalised(state, n, term_row):
    s = _vec(state)
    t = np.ascontiguousarray(term_row).reshape(())
    _check(lib.oracle_pauli_apply_normalised(s.ctypes.data, n, t.ctypes.data))
    return s


def pauli_apply_exp_factor(state, n, term_row, factor):
    s = _vec(state)
    t = np.ascontiguousarray(term_row).reshape(())
    f = complex(factor)
    _check(lib.oracle_pauli_apply_exp_factor(s.ctypes.data, n, t.ctypes.data, f.real, f.imag))
    return s


def sumop_apply(state, n, terms):
    s = np.ascontiguousarray(state, dtype=np.complex128)
    out = np.empty_like(s)
    t = np.ascontiguousarray(terms)
    _check(lib.oracle_sumop_apply(out.ctypes.data, s.ctypes.data, n, t.ctypes.data if t.size else None, t.size))
    return out


def sumop_expectation(state, n, terms):
    s = np.ascontiguousarray(state, dtype=np.complex128)
    t = np.ascontiguousarray(terms)
    out = (ctypes.c_double * 2)()
    _check(lib.oracle_sumop_expectation(s.ctypes.data, n, t.ctypes.data if t.size else None, t.size, out))
    return complex(out[0], out[1])


def inner_product(a, b, n):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    out = (ctypes.c_double * 2)()
    lib.oracle_inner_product(a.ctypes.data, b.ctypes.data, n, out)
    return complex(out[0], out[1])


def normalise(state, n):
    s = _vec(state)
    _check(lib.oracle_normalise(s.ctypes.data, n))
    return s


def tensor_product(a, na, b, nb):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    out = np.empty(1 << (na + nb), dtype=np.complex128)
    lib.oracle_tensor_product(out.ctypes.data, a.ctypes.data, na, b.ctypes.data, nb)
    return out


def trotter(state, n, terms, dt, steps, order=1):
    s = _vec(state)
    t = np.ascontiguousarray(terms)
    _check(lib.oracle_trotter(s.ctypes.data, n, t.ctypes.data if t.size else None, t.size, dt, steps, order))
    return s


def measure(state, n, qubits, r):
    s = _vec(state)
    q = np.ascontiguousarray(qubits, dtype=np.int32)
    nq = q.size
    probs = np.zeros(1 << (nq if nq else n), dtype=np.float64)
    out = _i64()
    _check(lib.oracle_measure(s.ctypes.data, n, q.ctypes.data if nq else None, nq, float(r), ctypes.byref(out),
                              probs.ctypes.data))
    return int(out.value), s, probs


def unitary2_check(m):
    a = np.ascontiguousarray(m, dtype=np.float64)
    return lib.oracle_unitary2_check(a.ctypes.data_as(_pd))


def port_execute(state, n, gates, threads):
    """Timing port of the reference's rayon data flow; returns (state, seconds)."""
    s = _vec(state)
    g = np.ascontiguousarray(gates)
    secs = lib.oracle_port_execute(s.ctypes.data, n, g.ctypes.data, g.size, int(threads))
    return s, secs


def port_execute_timed(state, n, gates, threads):
    """port_execute with one wall time per gate; returns (state, seconds per gate).
    A C-contiguous complex128 `state` is updated in place (no copy)."""
    s = np.ascontiguousarray(state, dtype=np.complex128)
    g = np.ascontiguousarray(gates)
    secs = np.zeros(g.size, dtype=np.float64)
    lib.oracle_port_execute_timed(s.ctypes.data, n, g.ctypes.data, g.size, int(threads),
                                  secs.ctypes.data_as(_pd))
    return s, secs
