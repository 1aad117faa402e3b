"""qi_sumop_expectation_noalloc: the energy reduction for callers that cannot
allocate device memory (their GPU memory belongs to their own pool, or they
must not add an allocation's device-wide synchronisation).  It keeps its
temporaries in one fixed static device array, so it is checked here against
the allocating entry point qi_sumop_expectation on two calls in a row (the
second call sees the previous call's leftovers in the shared array).  The file
name makes pytest collect it last."""
import ctypes

import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu


def noalloc_expectation(qi, st, terms):
    lib = qi._abi.lib
    t = np.ascontiguousarray(terms, dtype=qi.TERM_DTYPE)
    out = (ctypes.c_double * 2)()
    qi._abi.check(lib.qi_sumop_expectation_noalloc(ctypes.c_void_p(st.device_ptr()), st.n, st.precision,
                                                   t.ctypes.data if t.size else None, t.size,
                                                   ctypes.c_void_p(st.stream()), out))
    return complex(out[0], out[1])


def rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 2e-5)], ids=["f64", "f32"])
def test_noalloc_matches_allocating_entry_point(qi, prec, tol):
    for n, terms in ((12, workloads.heisenberg_open_chain(12, seed=3)), (16, workloads.xxz_periodic(16, seed=5))):
        with qi.DeviceState(n, prec) as st:
            st.upload(rand_state(n, n))
            want = qi.sumop_expectation(st, terms)
            first = noalloc_expectation(qi, st, terms)
            second = noalloc_expectation(qi, st, terms)   # same array, previous contents left behind
            assert abs(first - want) < tol, (n, first, want)
            assert abs(second - want) < tol, (n, second, want)
            assert first == second


def test_noalloc_rejects_oversized_input(qi):
    terms = workloads.terms_array([workloads.term(1.0, [(0, "Z")])] * 4097)
    with qi.DeviceState(4, 0) as st:
        st.set_plus()
        with pytest.raises(qi.QuantIronError) as ei:
            noalloc_expectation(qi, st, terms)
        assert ei.value.variant == "InvalidInputValue"
