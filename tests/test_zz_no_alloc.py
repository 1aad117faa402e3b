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


def one_xmask_group(count, seed):
    """`count` terms that all share the X mask on qubits 0 and 1 (distinct Z masks)."""
    rng = np.random.default_rng(seed)
    t = np.zeros(count, dtype=workloads.TERM_DTYPE)
    t["re"] = rng.uniform(-1.0, 1.0, size=count)
    t["im"] = 0.0
    t["xmask"] = 0b11
    t["zmask"] = np.arange(count, dtype=np.uint64)
    return t


@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 2e-4)], ids=["f64", "f32"])
def test_noalloc_largest_group(qi, prec, tol):
    """A group of exactly the largest accepted size (2048 terms on one X mask) runs and
    agrees with the allocating entry point; one more term is rejected."""
    n = 12
    terms = one_xmask_group(2048, seed=7)
    with qi.DeviceState(n, prec) as st:
        st.upload(rand_state(n, 11))
        want = qi.sumop_expectation(st, terms)
        got = noalloc_expectation(qi, st, terms)
        assert abs(got - want) < tol * max(1.0, abs(want)), (got, want)
        with pytest.raises(qi.QuantIronError) as ei:
            noalloc_expectation(qi, st, one_xmask_group(2049, seed=7))
        assert ei.value.variant == "InvalidInputValue"


def test_noalloc_rejects_host_pointer(qi):
    terms = workloads.heisenberg_open_chain(4, seed=1)
    host = np.zeros(16, dtype=np.complex128)
    out = (ctypes.c_double * 2)()
    t = np.ascontiguousarray(terms, dtype=qi.TERM_DTYPE)
    rc = qi._abi.lib.qi_sumop_expectation_noalloc(ctypes.c_void_p(host.ctypes.data), 4, 0, t.ctypes.data, t.size,
                                                  None, out)
    with pytest.raises(qi.QuantIronError) as ei:
        qi._abi.check(rc)
    assert ei.value.variant == "InvalidInputValue"
