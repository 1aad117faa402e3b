"""Pauli kernels, SumOp and Trotter evolution on the GPU vs the oracle."""
import numpy as np
import pytest

from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu


def rand_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def rand_terms(n, count, seed, max_weight=3):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        w = int(rng.integers(1, min(max_weight, n) + 1))
        qs = rng.choice(n, w, replace=False)
        ops = [(int(q), "XYZ"[int(rng.integers(0, 3))]) for q in qs]
        out.append(workloads.term(complex(rng.uniform(-1, 1), rng.uniform(-1, 1) * (rng.random() < 0.3)), ops))
    return workloads.terms_array(out)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_pauli_apply_and_exp(qi, orc, prec):
    tol = 1e-12 if prec == 0 else 2e-6
    for n in (1, 3, 8, 13):
        init = rand_state(n, n)
        for t in rand_terms(n, 12, n, max_weight=min(n, 4)):
            with qi.DeviceState(n, prec) as st, qi.DeviceState(n, prec) as out:
                st.upload(init)
                qi.pauli_apply(out, st, t)
                assert np.max(np.abs(out.download() - orc.pauli_apply(init, n, t))) < tol
                qi.pauli_apply_exp_factor(st, t, complex(0.1, -0.37))
                want = orc.pauli_apply_exp_factor(init, n, t, complex(0.1, -0.37))
                assert np.max(np.abs(st.download() - want)) < tol * 4


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_sumop_apply_and_expectation(qi, orc, prec):
    for n in (2, 6, 12):
        init = rand_state(n, 7 + n)
        terms = rand_terms(n, 25, n)
        with qi.DeviceState(n, prec) as st, qi.DeviceState(n, prec) as out:
            st.upload(init)
            qi.sumop_apply(out, st, terms)
            want = orc.sumop_apply(init, n, terms)
            tol = 1e-11 if prec == 0 else 2e-5
            assert np.max(np.abs(out.download() - want)) < tol
            e = qi.sumop_expectation(st, terms)
            e_want = orc.sumop_expectation(init, n, terms)
            assert abs(e - e_want) < (1e-11 if prec == 0 else 2e-5)


def diagonal_heavy_terms(n, seed):
    """Many Z-only terms (so one x-mask group gets byte tables): random Z masks within one
    byte and across bytes, an identity term, complex coefficients; plus a few X/Y terms."""
    rng = np.random.default_rng(seed)
    out = [workloads.term(complex(0.3, -0.2), [])]
    for _ in range(30):
        w = int(rng.integers(1, min(4, n) + 1))
        qs = rng.choice(n, w, replace=False)
        out.append(workloads.term(complex(rng.uniform(-1, 1), rng.uniform(-0.5, 0.5)), [(int(q), "Z") for q in qs]))
    for _ in range(8):
        qs = rng.choice(n, 2, replace=False)
        out.append(workloads.term(complex(rng.uniform(-1, 1), 0.0), [(int(qs[0]), "X"), (int(qs[1]), "Y")]))
    return workloads.terms_array(out)


@pytest.mark.parametrize("case", ["xxz20", "diag13", "diag18", "lattice16"])
def test_sumop_apply_f32_tabled_group(qi, orc, case):
    """FP32 SumOp::apply with the largest x-mask group evaluated from byte tables (ZZ / Z
    terms, straddling bonds such as (7, 8) and the periodic (0, n-1)) against the oracle."""
    if case == "xxz20":
        n, terms = 20, workloads.xxz_periodic(20, seed=3)
    elif case == "lattice16":
        n, terms = 16, workloads.lattice_xyz(4, 4, seed=1)
    else:
        n = int(case[4:])
        terms = diagonal_heavy_terms(n, n)
    init = rand_state(n, 11 + n)
    want = orc.sumop_apply(init, n, terms)
    with qi.DeviceState(n, 1) as st, qi.DeviceState(n, 1) as out:
        st.upload(init)
        qi.sumop_apply(out, st, terms)
        got = out.download()
    scale = float(np.sum(np.abs(terms["re"]) + np.abs(terms["im"])))
    assert np.max(np.abs(got - want)) < 2e-6 * scale


@pytest.mark.parametrize("n", [11, 12, 17, 22])
def test_sumop_apply_f32_streamed_tiles(qi, orc, n):
    """FP32 SumOp::apply from states of 2^12 amplitudes up streams input tiles through shared
    memory, one step per distinct X-mask offset above the tile: random terms of weight up to 4
    on every qubit give dozens of steps (the copy ring wraps many times), n = 22 gives several
    tiles per block; n = 11 takes the per-element gather kernel."""
    init = rand_state(n, 40 + n)
    terms = rand_terms(n, 60, 70 + n, max_weight=4)
    want = orc.sumop_apply(init, n, terms)
    with qi.DeviceState(n, 1) as st, qi.DeviceState(n, 1) as out:
        st.upload(init)
        qi.sumop_apply(out, st, terms)
        got = out.download()
        assert np.max(np.abs(st.download() - init)) < 1e-6   # the input is left as it was
    scale = float(np.sum(np.abs(terms["re"]) + np.abs(terms["im"])))
    assert np.max(np.abs(got - want)) < 2e-6 * scale


def test_heisenberg_expectation_20q(qi, orc):
    n = 20
    init = rand_state(n, 1)
    terms = workloads.heisenberg_open_chain(n, seed=0)
    e_want = orc.sumop_expectation(init, n, terms)
    with qi.DeviceState(n, 0) as st:
        st.upload(init)
        assert abs(qi.sumop_expectation(st, terms) - e_want) < 1e-11


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_trotter_vs_oracle(qi, orc, prec, order):
    n = 9
    terms = workloads.lattice_xyz(3, 3, seed=2)
    init = workloads.basis_state(n, 0b101100101)
    want = orc.trotter(init, n, terms, 0.05, 6, order)
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        energies = qi.trotter_evolve(st, terms, 0.05, 6, order=order, observable=terms, observe_every=3)
        got = st.download()
    assert np.max(np.abs(got - want)) < (1e-11 if prec == 0 else 1e-5)
    assert len(energies) == 2
    assert abs(energies[-1] - orc.sumop_expectation(want, n, terms)) < (1e-10 if prec == 0 else 1e-4)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_trotter_fused_14q_vs_oracle(qi, orc, prec):
    """2 x 7 lattice: the fused step has 5- and 6-qubit blocks (tensor cores for FP32,
    renormalised per step) and phase polynomials for the Z-type exponentials."""
    n = 14
    terms = workloads.lattice_xyz(2, 7, seed=5)
    init = workloads.basis_state(n, 0b10110010110101)
    want = orc.trotter(init, n, terms, 0.05, 5, 1)
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        qi.trotter_evolve(st, terms, 0.05, 5, order=1)
        got = st.download()
    assert np.max(np.abs(got - want)) < (1e-11 if prec == 0 else 2e-5)


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
def test_trotter_complex_coefficients_keep_the_norm_change(qi, orc, prec):
    """Complex coefficients make the step non-unitary (exp(-i c dt P) with Im c != 0):
    no renormalisation, the norm changes exactly as in the oracle."""
    n = 13
    terms = workloads.lattice_xyz(1, 13, seed=7)
    terms["im"][::5] = 0.3
    init = workloads.plus_state(n)
    want = orc.trotter(init, n, terms, 0.05, 4, 1)
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        qi.trotter_evolve(st, terms, 0.05, 4, order=1)
        got = st.download()
    assert abs(np.vdot(want, want).real - 1.0) > 1e-3   # the reference step changes the norm
    assert np.max(np.abs(got - want)) < (1e-11 if prec == 0 else 2e-5)


def test_trotter_errors(qi):
    with qi.DeviceState(3, 0) as st:
        st.set_zero()
        with pytest.raises(qi.QuantIronError) as ei:
            qi.trotter_evolve(st, workloads.terms_array([]), 0.1, 1)
        assert ei.value.variant == "InvalidNumberOfQubits" and ei.value.a == 0
        with pytest.raises(qi.QuantIronError) as ei:
            qi.trotter_evolve(st, workloads.terms_array([workloads.term(1.0, [(5, "X")])]), 0.1, 1)
        assert ei.value.variant == "InvalidQubitIndex" and (ei.value.a, ei.value.b) == (5, 3)


def test_pauli_normalised_gate(qi, orc):
    n = 5
    init = rand_state(n, 4)
    t = rand_terms(n, 1, 9)[0]
    with qi.DeviceState(n, 0) as st:
        st.upload(init)
        qi.pauli_apply_normalised(st, t)
        assert np.max(np.abs(st.download() - orc.pauli_apply_normalised(init, n, t))) < 1e-12


def _evolution_gates(terms, t):
    gl = workloads.GateList()
    for r in terms:
        gl.add("PAULI_EVOLUTION", [], [], [r["re"], r["im"], t], xmask=int(r["xmask"]), zmask=int(r["zmask"]))
    return gl.array()


def _random_runs(n, count, seed):
    """Exponentials with X-masks drawn from {0, X1, X2} and a long diagonal stretch."""
    rng = np.random.default_rng(seed)
    xs = [0, int(rng.integers(1, 1 << n)), int(rng.integers(1, 1 << n))]
    t = np.zeros(count, dtype=workloads.TERM_DTYPE)
    for k in range(count):
        t[k]["re"] = rng.normal()
        t[k]["xmask"] = 0 if count // 4 <= k < count // 2 else xs[int(rng.integers(0, 3))]
        t[k]["zmask"] = int(rng.integers(0, 1 << n))
    return t


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("n", [3, 11, 18])
def test_grouped_exponentials_on_device(qi, orc, prec, n):
    """QI_FUSION_PAULI_GROUPS plans (table-driven diagonal and pair passes) vs the
    oracle's term-by-term exponentials; also the 5x6-shaped lattices' run structure."""
    terms = _random_runs(n, 90, seed=n)
    gates = _evolution_gates(terms, 0.11)
    init = rand_state(n, 3)
    want = orc.execute(init, n, gates)
    plan = qi.Plan(n, prec, gates, fusion=qi.FUSION_PAULI_GROUPS)
    assert any(op["kind"] == 10 for op in plan.ops())
    with qi.DeviceState(n, prec) as st:
        st.upload(init)
        plan.execute(st)
        got = st.download()
    assert np.max(np.abs(got - want)) < (1e-12 if prec == 0 else 2e-5)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("lattice", ["tfim", "xxz"])
def test_trotter_fp64_grouped_vs_oracle(qi, orc, lattice, order):
    """FP64 Trotter steps run as grouped exponentials (one pass per bond / field run)."""
    if lattice == "tfim":
        n, terms = 12, workloads.lattice_tfim(3, 4, seed=1)
    else:
        n, terms = 12, workloads.xxz_periodic(12, seed=2)
    init = workloads.basis_state(n, 0b101101001101)
    want = orc.trotter(init, n, terms, 0.04, 5, order)
    with qi.DeviceState(n, 0) as st:
        st.upload(init)
        qi.trotter_evolve(st, terms, 0.04, 5, order=order)
        got = st.download()
    assert np.max(np.abs(got - want)) < 1e-11


def test_grouped_exponentials_32_qubits_round_trip(qi):
    """2^32 amplitudes (64-bit index arithmetic in the grouped kernels): the run
    followed by its inverse (reversed order, -t) returns |+...+> (FP32, 32 GiB each)."""
    n = 32
    terms = _random_runs(n, 24, seed=9)
    fwd = qi.Plan(n, qi.F32, _evolution_gates(terms, 0.13), fusion=qi.FUSION_PAULI_GROUPS)
    back = qi.Plan(n, qi.F32, _evolution_gates(terms[::-1].copy(), -0.13), fusion=qi.FUSION_PAULI_GROUPS)
    assert sum(op["kind"] == 10 for op in fwd.ops()) >= 2
    with qi.DeviceState(n, qi.F32) as st, qi.DeviceState(n, qi.F32) as ref:
        st.set_plus()
        ref.set_plus()
        fwd.execute(st)
        assert abs(st.inner_product(ref)) < 0.999   # the run moved the state
        back.execute(st)
        assert abs(st.inner_product(ref) - 1.0) < 1e-4


@pytest.mark.parametrize("model", ["heisenberg", "tfim"])
def test_fp32_trotter_energy_error_20q_20_steps(qi, orc, model):
    """The FP32 fused Trotter method on a 4x5 lattice (20 qubits), 20 first-order steps of
    dt = 0.05 from a seeded basis state, against the oracle's FP64 steps
    (time_evolution.rs:45-66): <H> after 10 and 20 steps within 2e-6 relative to the
    Hamiltonian's coefficient scale (sum |c_k|), state infidelity within 1e-8.  The error
    comes from the tensor-core blocks' FP32 accumulation (round toward zero) and grows
    about linearly with the number of steps."""
    rows, cols, n = 4, 5, 20
    terms = workloads.lattice_xyz(rows, cols, seed=3) if model == "heisenberg" else \
        workloads.lattice_tfim(rows, cols, seed=3)
    basis = int(np.random.default_rng(3).integers(0, 1 << n))
    init = workloads.basis_state(n, basis)
    scale = float(np.sum(np.abs(terms["re"])))
    want10 = orc.trotter(init, n, terms, 0.05, 10, 1)
    want20 = orc.trotter(want10, n, terms, 0.05, 10, 1)
    e_want = [orc.sumop_expectation(w, n, terms).real for w in (want10, want20)]
    with qi.DeviceState(n, qi.F32) as st:
        st.set_basis(basis)
        e_got = [complex(x).real for x in qi.trotter_evolve(st, terms, 0.05, 20, observable=terms, observe_every=10)]
        got = st.download()
    for a, b in zip(e_got, e_want):
        assert abs(a - b) < 2e-6 * scale, (a, b, scale)
    infid = 1.0 - abs(np.vdot(want20, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want20, want20).real)
    assert infid < 1e-8, infid
