"""State storage, constructors, arithmetic and reductions on the GPU vs numpy/oracle."""
import math

import numpy as np
import pytest

from tests.golden import known_answers as ka

pytestmark = pytest.mark.gpu


def rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_upload_download_roundtrip(qi, prec):
    for n in (1, 2, 5, 13, 23):
        v = rand_state(n, n)
        with qi.DeviceState(n, prec) as st:
            st.upload(v)
            back = st.download()
        if prec == 0:
            assert np.array_equal(back, v)
        else:
            assert np.array_equal(back, v.astype(np.complex64).astype(np.complex128))


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_pinned_host_buffers_roundtrip(qi, prec):
    """Page-locked host buffers take the direct path (the GPU reads / writes the host
    memory in one conversion pass); results equal the pageable path's bit for bit."""
    torch = pytest.importorskip("torch")
    for n in (1, 4, 13, 22):
        v = rand_state(n, 100 + n)
        host = torch.empty(2 << n, dtype=torch.float64, pin_memory=True)
        host.numpy()[:] = v.view(np.float64)
        out = torch.zeros(2 << n, dtype=torch.float64, pin_memory=True)
        with qi.DeviceState(n, prec) as st:
            st.upload_ptr(host.data_ptr(), 1 << n)
            st.download_ptr(out.data_ptr(), 1 << n)
            back_pageable = st.download()
        back = out.numpy().view(np.complex128)
        want = v if prec == 0 else v.astype(np.complex64).astype(np.complex128)
        assert np.array_equal(back, want) and np.array_equal(back_pageable, want)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_constructors(qi, prec):
    for n in (1, 3, 10):
        with qi.DeviceState(n, prec) as st:
            st.set_zero()
            assert np.allclose(st.download(), ka.zero(n))
            st.set_basis((1 << n) - 1)
            assert np.allclose(st.download(), ka.basis(n, (1 << n) - 1))
            st.set_plus()
            assert np.allclose(st.download(), ka.plus(n))
            st.set_minus()
            assert np.allclose(st.download(), ka.minus(n))
            st.set_ghz()
            g = np.zeros(1 << n, dtype=complex)
            g[0] = g[-1] = ka.R2
            assert np.allclose(st.download(), g)
            with pytest.raises(qi.QuantIronError) as ei:
                st.set_basis(1 << n)
            assert ei.value.variant == "InvalidQubitIndex"


def test_create_zero_qubits_error(qi):
    with pytest.raises(qi.QuantIronError) as ei:
        qi.DeviceState(0, 0)
    assert ei.value.variant == "InvalidNumberOfQubits" and ei.value.a == 0


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_reductions(qi, orc, prec):
    tol = 1e-12 if prec == 0 else 1e-6
    for n in (1, 4, 12, 20):
        a, b = rand_state(n, 1), rand_state(n, 2)
        with qi.DeviceState(n, prec) as da, qi.DeviceState(n, prec) as db:
            da.upload(a)
            db.upload(b)
            assert abs(da.inner_product(db) - orc.inner_product(a, b, n)) < tol
            assert abs(da.norm_sqr() - 1.0) < tol
            da.scale(3.0 - 4.0j)
            assert abs(da.norm_sqr() - 25.0) < 25 * tol
            da.normalise()
            assert abs(da.norm_sqr() - 1.0) < tol
            da.upload(a)
            da.axpy(0.5j, db)
            assert np.max(np.abs(da.download() - (a + 0.5j * b))) < tol * 10


def test_normalise_zero_norm(qi):
    with qi.DeviceState(3, 0) as st:
        st.upload(np.zeros(8, dtype=complex))
        with pytest.raises(qi.QuantIronError) as ei:
            st.normalise()
        assert ei.value.variant == "ZeroNorm"


def test_check_normalised(qi):
    with qi.DeviceState(4, 0) as st:
        st.set_plus()
        st.check_normalised()
        st.scale(1.01)
        with pytest.raises(qi.QuantIronError) as ei:
            st.check_normalised()
        assert ei.value.variant == "StateVectorNotNormalised"


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_tensor_product(qi, orc, prec):
    a, b = rand_state(3, 5), rand_state(4, 6)
    with qi.DeviceState(3, prec) as da, qi.DeviceState(4, prec) as db, qi.DeviceState(7, prec) as o:
        da.upload(a)
        db.upload(b)
        from quant_iron_gb300 import tensor_product
        tensor_product(o, da, db)
        got = o.download()
    assert np.max(np.abs(got - orc.tensor_product(a, 3, b, 4))) < (1e-14 if prec == 0 else 1e-6)


def test_amplitude(qi):
    v = rand_state(6, 3)
    with qi.DeviceState(6, 0) as st:
        st.upload(v)
        for i in (0, 17, 63):
            assert st.amplitude(i) == v[i]
        with pytest.raises(qi.QuantIronError):
            st.amplitude(64)


def test_mirror_api_reads_like_reference(qi):
    """The quant_iron mirror: State methods and operators as the crate's tests use them."""
    from quant_iron_gb300 import quant_iron as q
    zero, plus = q.State.new_zero(1), q.State.new_plus(1)
    assert zero.h(0) == plus
    assert q.State.new_basis_n(2, 1).cnot(0, 1) == q.State.new_basis_n(2, 3)
    st = q.State.new_zero(3).h(0).cnot(0, 1).cnot(1, 2)
    assert st == q.State.new_ghz(3)
    assert abs(zero.fs_fidelity(plus) - 0.5) < 1e-12
    assert abs(zero.fs_dist(plus) - math.pi / 4) < 1e-7
    h = q.SumOp([q.PauliString(2.0, {0: q.Pauli.X}), q.PauliString(3.0, {1: q.Pauli.Y}),
                 q.PauliString(4.0, {1: q.Pauli.Z})])
    assert abs(h.expectation_value(q.State.new_basis_n(2, 3)) - (-4.0)) < 1e-12
    with pytest.raises(qi.QuantIronError) as ei:
        q.State.new_zero(2).h(2)
    assert ei.value.variant == "InvalidQubitIndex"
    circ = q.qft_circuit([0, 1, 2], 3)
    out = circ.execute(q.State.new_zero(3))
    assert out == q.State.new_plus(3)


def test_mirror_chain_stays_on_device(qi):
    """A gate chain in the mirror downloads nothing until `state_vector` is read."""
    from quant_iron_gb300 import quant_iron as q
    st = q.State.new_zero(12).h_multi(range(12)).cnot(0, 5).rz(3, 0.4).swap(2, 9)
    assert st._host is None and st._dev is not None
    assert abs(st.probability(0) - 1.0 / 4096) < 1e-12 and st._host is None
    v = st.state_vector
    assert st._host is not None and abs(np.vdot(v, v) - 1.0) < 1e-12
    st.state_vector = ka.zero(12)
    assert st._dev is None and st.h(0).x(0).probability(1) == pytest.approx(0.5)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_async_transfers_roundtrip_and_overlap(qi, prec):
    """upload_async / download_async (copy engine, page-locked buffers) match the synchronous
    path bit for bit; two states keep their own stream order while both are in flight; a
    pageable buffer is refused."""
    torch = pytest.importorskip("torch")
    n = 20
    v = rand_state(n, 7)
    w = rand_state(n, 8)
    host_v = torch.empty(2 << n, dtype=torch.float64, pin_memory=True)
    host_w = torch.empty(2 << n, dtype=torch.float64, pin_memory=True)
    host_v.numpy()[:] = v.view(np.float64)
    host_w.numpy()[:] = w.view(np.float64)
    out_a = torch.zeros(2 << n, dtype=torch.float64, pin_memory=True)
    out_b = torch.zeros(2 << n, dtype=torch.float64, pin_memory=True)
    with qi.DeviceState(n, prec) as a, qi.DeviceState(n, prec) as b:
        a.upload_async(host_v.data_ptr(), 1 << n)
        b.upload_async(host_w.data_ptr(), 1 << n)
        a.apply_gate(qi_gate_row(qi, "H", [3]))
        b.apply_gate(qi_gate_row(qi, "X", [19]))
        a.download_async(out_a.data_ptr(), 1 << n)
        b.download_async(out_b.data_ptr(), 1 << n)
        a.synchronize()
        b.synchronize()
        sync_a = a.download()
        sync_b = b.download()
        with pytest.raises(qi.QuantIronError) as ei:
            a.upload_async(np.zeros(2 << n).ctypes.data, 1 << n)
        assert ei.value.variant == "InvalidInputValue"
    assert np.array_equal(out_a.numpy().view(np.complex128), sync_a)
    assert np.array_equal(out_b.numpy().view(np.complex128), sync_b)
    tol = 0 if prec == 0 else 1e-6
    ref_b = w.reshape(2, -1)[::-1].reshape(-1)   # X on the top qubit swaps the halves
    assert np.max(np.abs(sync_b - ref_b)) <= tol + 1e-15


def qi_gate_row(qi, kind, targets):
    from quant_iron_gb300 import workloads
    return workloads.GateList().add(kind, targets).array()[0]
