// qi_oracle.cpp — CPU FP64 restatement of quant-iron's state-vector semantics.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the engine's CUDA
// path is checked against; it is never linked into, loaded by, or called from
// the engine library.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load it.
//
// Every function restates the reference's *sequential* CPU branch (the
// branch the reference itself takes below 10 qubits) with the same formulas,
// the same operation order inside each complex expression and FP contraction
// disabled (-ffp-contract=off), so that results follow num_complex::Complex<f64>
// arithmetic (num-complex 0.4.6, Cargo.lock:326-327): (a+bi)(c+di) =
// (ac-bd) + (ad+bc)i, f64*(a+bi) = (fa)+(fb)i.
//
// Pinning: tests/test_oracle_golden.py checks this oracle against the
// known-answer vectors of the reference's own test-suite
// (src/tests/operator_tests.rs, pauli_string_tests.rs,
// time_evolution_tests.rs, circuit_tests.rs, state_tests.rs, gate_tests.rs).
// The reference crate (Rust) cannot be built in this environment, so no
// outputs of the reference binary itself exist; its test vectors are the pin.
//
// A second entry point, oracle_port_execute(), restates the data flow of the
// reference's rayon branch (clone, per-pair update list, serial scatter;
// e.g. operator.rs:338-360) on std::thread workers.  It is used only to time a
// CPU baseline of the reference implementation.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <thread>
#include <chrono>
#include <algorithm>
#include <unordered_set>

#include "../include/qi_engine.h"

namespace {

struct C {
    double re, im;
};
static inline C cadd(C a, C b) { return {a.re + b.re, a.im + b.im}; }
static inline C csub(C a, C b) { return {a.re - b.re, a.im - b.im}; }
static inline C cmul(C a, C b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline C rmul(double s, C a) { return {s * a.re, s * a.im}; }
static inline C cneg(C a) { return {-a.re, -a.im}; }
static inline C cconj(C a) { return {a.re, -a.im}; }
static inline double cnorm_sqr(C a) { return a.re * a.re + a.im * a.im; }
// num_complex: exp(a+bi) = e^a (cos b + i sin b)
static inline C cexp(C a) { double e = std::exp(a.re); return {e * std::cos(a.im), e * std::sin(a.im)}; }
// num_complex: cosh(a+bi) = cosh a cos b + i sinh a sin b; sinh = sinh a cos b + i cosh a sin b
static inline C ccosh(C a) { return {std::cosh(a.re) * std::cos(a.im), std::sinh(a.re) * std::sin(a.im)}; }
static inline C csinh(C a) { return {std::sinh(a.re) * std::cos(a.im), std::cosh(a.re) * std::sin(a.im)}; }

static inline C *amp(double *sv) { return reinterpret_cast<C *>(sv); }
static inline const C *amp(const double *sv) { return reinterpret_cast<const C *>(sv); }

// check_controls (operator.rs:195-199)
static inline bool check_controls(uint64_t i, const int32_t *controls, int nc) {
    for (int k = 0; k < nc; ++k)
        if (((i >> controls[k]) & 1ull) != 1ull) return false;
    return true;
}

struct Err { int code; int64_t a, b; };
static Err ok() { return {QI_OK, -1, -1}; }

// validate_qubits (operator.rs:214-273): target count, target range, control
// range + overlap (controls outer loop, targets inner), duplicate targets.
static Err validate_qubits(int n, const int32_t *t, int nt, const int32_t *c, int nc, int expected) {
    if (nt != expected) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, nt, -1};
    for (int k = 0; k < nt; ++k)
        if (t[k] < 0 || t[k] >= n) return {QI_ERR_INVALID_QUBIT_INDEX, t[k], n};
    for (int k = 0; k < nc; ++k) {
        if (c[k] < 0 || c[k] >= n) return {QI_ERR_INVALID_QUBIT_INDEX, c[k], n};
        for (int j = 0; j < nt; ++j)
            if (c[k] == t[j]) return {QI_ERR_OVERLAPPING_CONTROL_AND_TARGET, c[k], t[j]};
    }
    if (expected > 1) {
        for (int i = 0; i < nt; ++i)
            for (int j = i + 1; j < nt; ++j)
                if (t[i] == t[j]) return {QI_ERR_INVALID_QUBIT_INDEX, t[i], n};
    }
    return ok();
}

// Generic controlled 2x2 update on pairs (i, i|1<<t), i with target bit 0 and
// controls satisfied on i: the sequential loop of Hadamard/RX/RY/Unitary2.
template <class F>
static void pair_loop(C *s, int n, int t, const int32_t *c, int nc, F f) {
    const uint64_t dim = 1ull << n;
    for (uint64_t i = 0; i < dim; ++i) {
        if (((i >> t) & 1ull) == 0) {
            uint64_t j = i | (1ull << t);
            if (check_controls(i, c, nc)) {
                C ai = s[i], aj = s[j];
                f(ai, aj, s[i], s[j]);
            }
        }
    }
}

// Diagonal phase on target bit 1 (PhaseS/T/Sdag/Tdag/PhaseShift sequential loops).
static void phase_on_one(C *s, int n, int t, const int32_t *c, int nc, C ph) {
    const uint64_t dim = 1ull << n;
    for (uint64_t i = 0; i < dim; ++i)
        if (((i >> t) & 1ull) == 1ull && check_controls(i, c, nc)) s[i] = cmul(s[i], ph);
}

struct Unitary { C m[2][2]; };

static Unitary ry_phase(double theta, double phi) {   // operator.rs:2136-2156
    double ch = std::cos(theta / 2.0), sh = std::sin(theta / 2.0);
    C e = cexp({0.0, phi});
    Unitary u;
    u.m[0][0] = {ch, 0.0};
    u.m[0][1] = rmul(sh, cneg(e));                 // -expi_phi * sin_half_theta
    u.m[1][0] = {sh, 0.0};
    u.m[1][1] = rmul(ch, e);                       // expi_phi * cos_half_theta
    // num_complex: Complex * f64 multiplies both parts; same as f64 * Complex.
    return u;
}
static Unitary ry_phase_dag(double theta, double phi) {   // operator.rs:2172-2192
    double ch = std::cos(theta / 2.0), sh = std::sin(theta / 2.0);
    C e = cexp({0.0, -phi});
    Unitary u;
    u.m[0][0] = {ch, 0.0};
    u.m[0][1] = {sh, 0.0};
    u.m[1][0] = rmul(sh, cneg(e));
    u.m[1][1] = rmul(ch, e);
    return u;
}

static void apply_unitary2(C *s, int n, int t, const int32_t *c, int nc, const Unitary &u) {
    pair_loop(s, n, t, c, nc, [&](C ai, C aj, C &oi, C &oj) {
        oi = cadd(cmul(u.m[0][0], ai), cmul(u.m[0][1], aj));
        oj = cadd(cmul(u.m[1][0], ai), cmul(u.m[1][1], aj));
    });
}

static Err apply_gate(C *s, int n, const qi_gate &g) {
    const int32_t *t = g.targets;
    const int32_t *c = g.controls;
    const int nt = g.n_targets, nc = g.n_controls;
    const double *p = g.params;
    const C I = {0.0, 1.0};
    Err e;
    switch (g.kind) {
    case QI_GATE_H: {   // operator.rs:303-424 (sequential branch :384-412)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const double r = 1.0 / std::sqrt(2.0);
        pair_loop(s, n, t[0], c, nc, [&](C a0, C a1, C &o0, C &o1) {
            o0 = rmul(r, cadd(a0, a1));
            o1 = rmul(r, csub(a0, a1));
        });
        return ok();
    }
    case QI_GATE_X:
    case QI_GATE_Y:
    case QI_GATE_Z: {   // operator.rs:474-606 (sequential branch :569-599)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const int tq = t[0];
        const uint64_t dim = 1ull << n;
        for (uint64_t i = 0; i < dim; ++i) {
            if (!check_controls(i, c, nc)) continue;
            if (g.kind == QI_GATE_Z) {
                if ((i >> tq) & 1ull) s[i] = cneg(s[i]);
            } else if (((i >> tq) & 1ull) == 0) {
                uint64_t j = i | (1ull << tq);
                C ai = s[i], aj = s[j];
                if (g.kind == QI_GATE_X) { s[i] = aj; s[j] = ai; }
                else { s[i] = cmul(cneg(I), aj); s[j] = cmul(I, ai); }
            }
        }
        return ok();
    }
    case QI_GATE_S:     // operator.rs:1160-1216
    case QI_GATE_SDAG:  // operator.rs:1352-1408
    case QI_GATE_T:     // operator.rs:1253-1315
    case QI_GATE_TDAG:  // operator.rs:1445-1507
    case QI_GATE_P: {   // operator.rs:1565-1624
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const double r = 1.0 / std::sqrt(2.0);
        C ph;
        if (g.kind == QI_GATE_S) ph = {0.0, 1.0};
        else if (g.kind == QI_GATE_SDAG) ph = {0.0, -1.0};
        else if (g.kind == QI_GATE_T) ph = {r, r};
        else if (g.kind == QI_GATE_TDAG) ph = {r, -r};
        else ph = {std::cos(p[0]), std::sin(p[0])};
        phase_on_one(s, n, t[0], c, nc, ph);
        return ok();
    }
    case QI_GATE_RX: {  // operator.rs:1674-1767 (sequential :1740-1760)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const double h = p[0] / 2.0, ch = std::cos(h), sh = std::sin(h);
        pair_loop(s, n, t[0], c, nc, [&](C ai, C aj, C &oi, C &oj) {
            // cos_half * amp_i - i_complex * sin_half * amp_j
            oi = csub(rmul(ch, ai), cmul(rmul(sh, I), aj));
            // -i_complex * sin_half * amp_i + cos_half * amp_j
            oj = cadd(cmul(rmul(sh, cneg(I)), ai), rmul(ch, aj));
        });
        return ok();
    }
    case QI_GATE_RY: {  // operator.rs:1817-1908 (sequential :1883-1902)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const double h = p[0] / 2.0, ch = std::cos(h), sh = std::sin(h);
        pair_loop(s, n, t[0], c, nc, [&](C ai, C aj, C &oi, C &oj) {
            oi = csub(rmul(ch, ai), rmul(sh, aj));
            oj = cadd(rmul(sh, ai), rmul(ch, aj));
        });
        return ok();
    }
    case QI_GATE_RZ: {  // operator.rs:1958-2035 (sequential :2016-2028)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const double h = p[0] / 2.0;
        const C p0 = {std::cos(h), -std::sin(h)}, p1 = {std::cos(h), std::sin(h)};
        const uint64_t dim = 1ull << n;
        for (uint64_t i = 0; i < dim; ++i)
            if (check_controls(i, c, nc)) s[i] = cmul(s[i], ((i >> t[0]) & 1ull) ? p1 : p0);
        return ok();
    }
    case QI_GATE_U2:
    case QI_GATE_RYPHASE:
    case QI_GATE_RYPHASE_DAG: {   // operator.rs:2206-2266
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        Unitary u;
        if (g.kind == QI_GATE_U2) {
            u.m[0][0] = {p[0], p[1]}; u.m[0][1] = {p[2], p[3]};
            u.m[1][0] = {p[4], p[5]}; u.m[1][1] = {p[6], p[7]};
        } else if (g.kind == QI_GATE_RYPHASE) u = ry_phase(p[0], p[1]);
        else u = ry_phase_dag(p[0], p[1]);
        apply_unitary2(s, n, t[0], c, nc, u);
        return ok();
    }
    case QI_GATE_CNOT: {   // operator.rs:667-685
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        if (nc != 1) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, nc, -1};
        qi_gate x = g; x.kind = QI_GATE_X;
        return apply_gate(s, n, x);
    }
    case QI_GATE_TOFFOLI: {   // operator.rs:1055-1075
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        if (nc != 2) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, nc, -1};
        if (c[0] == c[1]) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, nc, -1};
        qi_gate x = g; x.kind = QI_GATE_X;
        return apply_gate(s, n, x);
    }
    case QI_GATE_SWAP: {   // operator.rs:731-820 (sequential :802-815)
        if ((e = validate_qubits(n, t, nt, c, nc, 2)).code) return e;
        const int t1 = t[0], t2 = t[1];
        const uint64_t dim = 1ull << n;
        for (uint64_t i = 0; i < dim; ++i) {
            uint64_t b1 = (i >> t1) & 1ull, b2 = (i >> t2) & 1ull;
            if (b1 != b2) {
                uint64_t j = i ^ (1ull << t1) ^ (1ull << t2);
                if (i < j && check_controls(i, c, nc)) { C ai = s[i]; s[i] = s[j]; s[j] = ai; }
            }
        }
        return ok();
    }
    case QI_GATE_MATCHGATE: {   // operator.rs:893-1014 (sequential :987-1007)
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        const int q1 = t[0];
        if (q1 == n - 1) return {QI_ERR_INVALID_QUBIT_INDEX, q1, n};
        const int q2 = q1 + 1;
        const double ch = std::cos(p[0] / 2.0), sh = std::sin(p[0] / 2.0);
        const C e1 = cexp({0.0, p[1]}), e2 = cexp({0.0, p[2]});
        const uint64_t quads = 1ull << (n - 2);
        for (uint64_t i = 0; i < quads; ++i) {
            uint64_t k = ((i >> q1) << (q1 + 1)) | (i & ((1ull << q1) - 1));
            uint64_t l = ((k >> (q2 - 1)) << q2) | (k & ((1ull << (q2 - 1)) - 1));
            uint64_t i01 = l | (1ull << q1), i10 = l | (1ull << q2), i11 = l | (1ull << q1) | (1ull << q2);
            if (check_controls(i01, c, nc)) {
                C a01 = s[i01], a10 = s[i10];
                // cos_theta_half * amp01 - exp_i_phi1 * sin_theta_half * amp10
                s[i01] = csub(rmul(ch, a01), cmul(rmul(sh, e1), a10));
                // sin_theta_half * amp01 + exp_i_phi1 * cos_theta_half * amp10
                s[i10] = cadd(rmul(sh, a01), cmul(rmul(ch, e1), a10));
            }
            if (check_controls(i11, c, nc)) s[i11] = cmul(s[i11], e2);
        }
        return ok();
    }
    case QI_GATE_IDENTITY: {   // operator.rs:1112-1123
        if ((e = validate_qubits(n, t, nt, c, nc, 1)).code) return e;
        return ok();
    }
    default:
        return {QI_ERR_INVALID_INPUT_VALUE, g.kind, -1};
    }
}

// ---- Pauli strings (pauli_string.rs) ------------------------------------

// Validation of a PauliString against a state: every op qubit goes through
// Pauli::apply -> validate_qubits (operator.rs:488), so the first qubit >= n
// yields InvalidQubitIndex(q, n).  The reference visits ops in HashMap order;
// the oracle reports the lowest such qubit.
static Err validate_term(int n, const qi_pauli_term &t) {
    uint64_t m = t.xmask | t.zmask;
    if (n < 64 && (m >> n)) {
        int q = n;
        while (!((m >> q) & 1ull)) ++q;
        return {QI_ERR_INVALID_QUBIT_INDEX, q, n};
    }
    return ok();
}

// P |in> without the coefficient (apply_operators, pauli_string.rs:172-184):
// the product of single-qubit Paulis, each applied with Pauli::apply's
// sequential formulas (operator.rs:569-599).  Ops on distinct qubits commute
// and every factor is exact (+-1, +-i, swap), so the HashMap visiting order
// does not change the result.
static void apply_operators(C *s, int n, const qi_pauli_term &t) {
    const C I = {0.0, 1.0};
    const uint64_t dim = 1ull << n;
    for (int q = 0; q < n; ++q) {
        bool x = (t.xmask >> q) & 1ull, z = (t.zmask >> q) & 1ull;
        if (!x && !z) continue;
        for (uint64_t i = 0; i < dim; ++i) {
            if (x && !z) {
                if (((i >> q) & 1ull) == 0) { uint64_t j = i | (1ull << q); C a = s[i]; s[i] = s[j]; s[j] = a; }
            } else if (x && z) {
                if (((i >> q) & 1ull) == 0) {
                    uint64_t j = i | (1ull << q);
                    C ai = s[i], aj = s[j];
                    s[i] = cmul(cneg(I), aj);
                    s[j] = cmul(I, ai);
                }
            } else {
                if ((i >> q) & 1ull) s[i] = cneg(s[i]);
            }
        }
    }
}

static void scale(C *s, uint64_t dim, C a) { for (uint64_t i = 0; i < dim; ++i) s[i] = cmul(s[i], a); }

static C inner_product(const C *a, const C *b, uint64_t dim) {   // state.rs:890-917
    C acc = {0.0, 0.0};
    for (uint64_t i = 0; i < dim; ++i) acc = cadd(acc, cmul(cconj(a[i]), b[i]));
    return acc;
}

static Err normalise(C *s, uint64_t dim) {   // state.rs:924-945
    double ss = 0.0;
    for (uint64_t i = 0; i < dim; ++i) ss += cnorm_sqr(s[i]);
    double norm = std::sqrt(ss);
    if (norm == 0.0) return {QI_ERR_ZERO_NORM, -1, -1};
    if (norm == 1.0) return ok();
    for (uint64_t i = 0; i < dim; ++i) s[i] = {s[i].re / norm, s[i].im / norm};
    return ok();
}

// exp(alpha P)|s> = cosh(alpha)|s> + sinh(alpha) P|s>  (pauli_string.rs:237-262)
static Err apply_exp_alpha(C *s, int n, const qi_pauli_term &t, C alpha) {
    Err e = validate_term(n, t);
    if (e.code) return e;
    const uint64_t dim = 1ull << n;
    if ((t.xmask | t.zmask) == 0) { scale(s, dim, cexp(alpha)); return ok(); }
    std::vector<C> ps(s, s + dim);
    apply_operators(ps.data(), n, t);
    C ch = ccosh(alpha), sh = csinh(alpha);
    for (uint64_t i = 0; i < dim; ++i) s[i] = cadd(cmul(s[i], ch), cmul(ps[i], sh));
    return ok();
}

static thread_local Err g_last;
static int ret(Err e, int64_t *ea = nullptr, int64_t *eb = nullptr) {
    g_last = e;
    if (ea) *ea = e.a;
    if (eb) *eb = e.b;
    return e.code;
}

}  // namespace

extern "C" {

void oracle_last_error(int64_t *a, int64_t *b) { *a = g_last.a; *b = g_last.b; }

int oracle_apply_gate(double *sv, int n, const qi_gate *g) {
    return ret(apply_gate(amp(sv), n, *g));
}

// Resolve parametric gates (param_ids) against theta, as Parameter::get +
// to_concrete_gates do (parametric_gate.rs:30-211).
static qi_gate resolve(const qi_gate &g, const double *theta) {
    qi_gate r = g;
    for (int k = 0; k < 3; ++k)
        if (g.param_ids[k] >= 0 && theta) r.params[k] = theta[g.param_ids[k]];
    return r;
}

int oracle_measure(double *sv, int n, const int32_t *qubits, int nq, double r, int64_t *outcome,
                   double *probs_out);

// SplitMix64 (Steele, Lea, Flood 2014), the seeded stand-in for the reference's unseeded
// rand::rng() in State::measure (state.rs:601): r = top 53 bits / 2^53.
static double uniform01(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * 0x1.0p-53;
}

// Gate::Measurement (gate.rs:104-106) -> State::measure (state.rs:525-730), keeping the new
// state: basis change on every measured qubit (X: H; Y: S-dagger then H; Custom: U), the
// computational measurement with r drawn from the gate's seed (xmask), then the change back
// (X: H; Y: H then S; Custom: U-dagger, calculate_adjoint state.rs:17-22).
static Err apply_measurement(C *s, int n, const qi_gate &g) {
    const int basis = g.targets[0];
    if (g.n_targets != 0) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, g.n_targets, -1};
    if (basis < QI_BASIS_COMPUTATIONAL || basis > QI_BASIS_CUSTOM) return {QI_ERR_INVALID_INPUT_VALUE, basis, -1};
    std::vector<int32_t> q(g.controls, g.controls + g.n_controls);
    if (q.empty()) for (int k = 0; k < n; ++k) q.push_back(k);
    if ((int)q.size() > n) return {QI_ERR_INVALID_NUMBER_OF_QUBITS, n, -1};
    for (int32_t x : q)
        if (x < 0 || x >= n) return {QI_ERR_INVALID_QUBIT_INDEX, x, n};
    auto each = [&](int kind, const double *m8) {
        for (int32_t x : q) {
            qi_gate h;
            std::memset(&h, 0, sizeof(h));
            h.kind = kind;
            h.n_targets = 1;
            h.targets[0] = x;
            h.param_ids[0] = h.param_ids[1] = h.param_ids[2] = -1;
            if (m8) std::memcpy(h.params, m8, 8 * sizeof(double));
            Err e = apply_gate(s, n, h);
            if (e.code) return e;
        }
        return ok();
    };
    const double *u = g.params;
    const double ud[8] = {u[0], -u[1], u[4], -u[5], u[2], -u[3], u[6], -u[7]};
    Err e = ok();
    if (basis == QI_BASIS_X) e = each(QI_GATE_H, nullptr);
    else if (basis == QI_BASIS_Y) {
        e = each(QI_GATE_SDAG, nullptr);
        if (!e.code) e = each(QI_GATE_H, nullptr);
    } else if (basis == QI_BASIS_CUSTOM) e = each(QI_GATE_U2, u);
    if (e.code) return e;
    int64_t outcome = 0;
    if (oracle_measure(reinterpret_cast<double *>(s), n, q.data(), (int)q.size(), uniform01(g.xmask), &outcome,
                       nullptr))
        return g_last;
    if (basis == QI_BASIS_X) e = each(QI_GATE_H, nullptr);
    else if (basis == QI_BASIS_Y) {
        e = each(QI_GATE_H, nullptr);
        if (!e.code) e = each(QI_GATE_S, nullptr);
    } else if (basis == QI_BASIS_CUSTOM) e = each(QI_GATE_U2, ud);
    return e;
}

static Err apply_any(C *s, int n, const qi_gate &g) {
    if (g.kind == QI_GATE_MEASUREMENT) return apply_measurement(s, n, g);
    if (g.kind == QI_GATE_PAULI_STRING) {       // gate.rs:115-117 -> apply_normalised
        qi_pauli_term t = {g.params[0], g.params[1], g.xmask, g.zmask};
        Err e = validate_term(n, t);
        if (e.code) return e;
        apply_operators(s, n, t);
        return normalise(s, 1ull << n);
    }
    if (g.kind == QI_GATE_PAULI_EVOLUTION) {    // gate.rs:118-120 -> apply_exp_neg_i_dt
        qi_pauli_term t = {g.params[0], g.params[1], g.xmask, g.zmask};
        if (t.coeff_im != 0.0) return {QI_ERR_INVALID_PAULI_COEFFICIENT, -1, -1};
        C alpha = cmul({t.coeff_re, t.coeff_im}, {0.0, -g.params[2]});
        return apply_exp_alpha(s, n, t, alpha);
    }
    return apply_gate(s, n, g);
}

// Circuit::execute (circuit.rs:160-172): gates in order; stops at the first error.
int oracle_execute(double *sv, int n, const qi_gate *gates, int64_t n_gates, const double *theta,
                   int64_t *failed_gate) {
    for (int64_t k = 0; k < n_gates; ++k) {
        Err e = apply_any(amp(sv), n, resolve(gates[k], theta));
        if (e.code) { if (failed_gate) *failed_gate = k; return ret(e); }
    }
    return ret(ok());
}

// PauliString::apply (pauli_string.rs:139-151): out = coefficient * P|in>
int oracle_pauli_apply(double *out, const double *in, int n, const qi_pauli_term *t) {
    Err e = validate_term(n, *t);
    if (e.code) return ret(e);
    const uint64_t dim = 1ull << n;
    std::memcpy(out, in, dim * sizeof(C));
    apply_operators(amp(out), n, *t);
    scale(amp(out), dim, {t->coeff_re, t->coeff_im});
    return ret(ok());
}

int oracle_pauli_apply_normalised(double *sv, int n, const qi_pauli_term *t) {
    Err e = validate_term(n, *t);
    if (e.code) return ret(e);
    apply_operators(amp(sv), n, *t);
    return ret(normalise(amp(sv), 1ull << n));
}

int oracle_pauli_apply_exp_factor(double *sv, int n, const qi_pauli_term *t, double fre, double fim) {
    C alpha = cmul({t->coeff_re, t->coeff_im}, {fre, fim});
    return ret(apply_exp_alpha(amp(sv), n, *t, alpha));
}

// SumOp::apply (pauli_string.rs:453-466): sum over terms, summed in term order.
int oracle_sumop_apply(double *out, const double *in, int n, const qi_pauli_term *terms, int64_t nt) {
    const uint64_t dim = 1ull << n;
    std::vector<C> acc(dim, C{0.0, 0.0}), tmp(dim);
    if (nt == 0) {   // state * 0.0
        for (uint64_t i = 0; i < dim; ++i) acc[i] = rmul(0.0, amp(in)[i]);
    }
    for (int64_t k = 0; k < nt; ++k) {
        int st = oracle_pauli_apply(reinterpret_cast<double *>(tmp.data()), in, n, &terms[k]);
        if (st) return st;
        if (k == 0) acc = tmp;
        else for (uint64_t i = 0; i < dim; ++i) acc[i] = cadd(acc[i], tmp[i]);
    }
    std::memcpy(out, acc.data(), dim * sizeof(C));
    return ret(ok());
}

// SumOp::expectation_value (pauli_string.rs:485-507)
int oracle_sumop_expectation(const double *sv, int n, const qi_pauli_term *terms, int64_t nt, double out[2]) {
    const uint64_t dim = 1ull << n;
    std::vector<C> tmp(dim);
    C total = {0.0, 0.0};
    for (int64_t k = 0; k < nt; ++k) {
        int st = oracle_pauli_apply(reinterpret_cast<double *>(tmp.data()), sv, n, &terms[k]);
        if (st) return st;
        total = cadd(total, inner_product(amp(sv), tmp.data(), dim));
    }
    out[0] = total.re; out[1] = total.im;
    return ret(ok());
}

void oracle_inner_product(const double *a, const double *b, int n, double out[2]) {
    C r = inner_product(amp(a), amp(b), 1ull << n);
    out[0] = r.re; out[1] = r.im;
}

int oracle_normalise(double *sv, int n) { return ret(normalise(amp(sv), 1ull << n)); }

void oracle_tensor_product(double *out, const double *a, int na, const double *b, int nb) {   // state.rs:801-836
    const uint64_t db = 1ull << nb, dim = 1ull << (na + nb);
    for (uint64_t k = 0; k < dim; ++k) amp(out)[k] = cmul(amp(a)[k >> nb], amp(b)[k & (db - 1)]);
}

// first/second_order_trotter_step and trotter_evolve_state (time_evolution.rs:45-166)
int oracle_trotter(double *sv, int n, const qi_pauli_term *terms, int64_t nt, double dt, int64_t steps, int order) {
    if (nt == 0) return ret({QI_ERR_INVALID_NUMBER_OF_QUBITS, 0, -1});
    for (int64_t s = 0; s < steps; ++s) {
        if (order == 1) {
            for (int64_t k = 0; k < nt; ++k) {
                int st = oracle_pauli_apply_exp_factor(sv, n, &terms[k], 0.0, -dt);
                if (st) return st;
            }
        } else {
            for (int64_t k = 0; k < nt; ++k) {
                int st = oracle_pauli_apply_exp_factor(sv, n, &terms[k], 0.0, -dt / 2.0);
                if (st) return st;
            }
            for (int64_t k = nt - 1; k >= 0; --k) {
                int st = oracle_pauli_apply_exp_factor(sv, n, &terms[k], 0.0, -dt / 2.0);
                if (st) return st;
            }
        }
    }
    return ret(ok());
}

// Computational-basis measurement (state.rs:555-669) with the uniform draw
// `r` supplied by the caller instead of rand::rng(): probabilities per outcome
// (bit k of the outcome = qubit qubits[k]), normalised, CDF scan with
// `r < cumulative`, collapse, renormalise.  Writes the outcome integer.
int oracle_measure(double *sv, int n, const int32_t *qubits, int nq, double r, int64_t *outcome,
                   double *probs_out) {
    const uint64_t dim = 1ull << n;
    std::vector<int32_t> all;
    if (nq == 0) { for (int q = 0; q < n; ++q) all.push_back(q); qubits = all.data(); nq = n; }
    if (nq > n) return ret({QI_ERR_INVALID_NUMBER_OF_QUBITS, n, -1});
    for (int k = 0; k < nq; ++k)
        if (qubits[k] < 0 || qubits[k] >= n) return ret({QI_ERR_INVALID_QUBIT_INDEX, qubits[k], n});
    const uint64_t no = 1ull << nq;
    std::vector<double> pr(no, 0.0);
    auto outcome_of = [&](uint64_t i) {
        uint64_t o = 0;
        for (int k = 0; k < nq; ++k) if ((i >> qubits[k]) & 1ull) o |= 1ull << k;
        return o;
    };
    for (uint64_t i = 0; i < dim; ++i) pr[outcome_of(i)] += cnorm_sqr(amp(sv)[i]);
    double total = 0.0;
    for (double x : pr) total += x;
    if (total < 2.220446049250313e-16) return ret({QI_ERR_UNKNOWN, -1, -1});
    for (auto &x : pr) x = x / total;
    if (probs_out) std::memcpy(probs_out, pr.data(), no * sizeof(double));
    double cum = 0.0;
    uint64_t out = 0;
    for (uint64_t i = 0; i < no; ++i) {
        cum += pr[i];
        if (r < cum) { out = i; break; }
    }
    if (r >= cum) out = no - 1;
    double nrm = 0.0;
    for (uint64_t i = 0; i < dim; ++i) {
        if (outcome_of(i) == out) nrm += cnorm_sqr(amp(sv)[i]);
        else amp(sv)[i] = {0.0, 0.0};
    }
    if (nrm > 2.220446049250313e-16) {
        double f = std::sqrt(nrm);
        for (uint64_t i = 0; i < dim; ++i) amp(sv)[i] = {amp(sv)[i].re / f, amp(sv)[i].im / f};
    }
    *outcome = (int64_t)out;
    return ret(ok());
}

int oracle_unitary2_check(const double m[8]) {   // Unitary2::new (operator.rs:2092-2125)
    const double tol = 2.220446049250313e-16 * 2.0;
    C a = {m[0], m[1]}, b = {m[2], m[3]}, c = {m[4], m[5]}, d = {m[6], m[7]};
    if (std::fabs((cnorm_sqr(a) + cnorm_sqr(b)) - 1.0) > tol) return QI_ERR_NON_UNITARY_MATRIX;
    if (std::fabs((cnorm_sqr(c) + cnorm_sqr(d)) - 1.0) > tol) return QI_ERR_NON_UNITARY_MATRIX;
    if (cnorm_sqr(cadd(cmul(a, cconj(c)), cmul(b, cconj(d)))) > tol * tol) return QI_ERR_NON_UNITARY_MATRIX;
    return QI_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Timing port of the reference's rayon branch (operator.rs thresholds :17-21,
// rayon branches e.g. Hadamard :338-382, Pauli :515-568, phase :1187-1199,
// SWAP :775-800).  Each gate: clone the state, build the update list
// (index, value) in parallel with one heap vector per pair, then scatter it
// serially; diagonal gates mutate the clone in parallel.  Threads stand in
// for rayon's pool.  Returns wall seconds.  Gate kinds other than the ones the
// random-circuit workload uses fall back to the sequential restatement.
// ---------------------------------------------------------------------------
namespace {
struct Upd { uint64_t idx; C val; };

template <class F>
static void par_for(uint64_t n, int threads, F f) {
    std::vector<std::thread> th;
    uint64_t chunk = (n + threads - 1) / threads;
    for (int w = 0; w < threads; ++w) {
        uint64_t lo = w * chunk, hi = std::min<uint64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=, &f] { f(w, lo, hi); });
    }
    for (auto &t : th) t.join();
}

static void port_gate(std::vector<C> &state, int n, const qi_gate &g, int threads) {
    const uint64_t dim = 1ull << n;
    std::vector<C> nsv = state;   // `state.state_vector.clone()`
    const int32_t *c = g.controls;
    const int nc = g.n_controls;
    const C I = {0.0, 1.0};
    auto pair_gate = [&](auto fn) {
        const int t = g.targets[0];
        std::vector<std::vector<Upd>> parts(threads);
        par_for(dim, threads, [&](int w, uint64_t lo, uint64_t hi) {
            auto &out = parts[w];
            for (uint64_t i = lo; i < hi; ++i) {
                if (((i >> t) & 1ull) == 0 && check_controls(i, c, nc)) {
                    uint64_t j = i | (1ull << t);
                    C a = state[i], b = state[j], oa, ob;
                    fn(a, b, oa, ob);
                    std::vector<Upd> pv{{i, oa}, {j, ob}};   // per-pair `vec![...]`
                    out.insert(out.end(), pv.begin(), pv.end());
                }
            }
        });
        for (auto &p : parts) for (auto &u : p) nsv[u.idx] = u.val;   // serial scatter
    };
    auto diag_gate = [&](C p0, C p1, bool touch0) {
        const int t = g.targets[0];
        par_for(dim, threads, [&](int, uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                if (!check_controls(i, c, nc)) continue;
                if ((i >> t) & 1ull) nsv[i] = cmul(state[i], p1);
                else if (touch0) nsv[i] = cmul(state[i], p0);
            }
        });
    };
    const double *p = g.params;
    const double r2 = 1.0 / std::sqrt(2.0);
    switch (g.kind) {
    case QI_GATE_H:
        pair_gate([&](C a, C b, C &oa, C &ob) { oa = rmul(r2, cadd(a, b)); ob = rmul(r2, csub(a, b)); });
        break;
    case QI_GATE_X: case QI_GATE_CNOT: case QI_GATE_TOFFOLI:
        pair_gate([&](C a, C b, C &oa, C &ob) { oa = b; ob = a; });
        break;
    case QI_GATE_Y:
        pair_gate([&](C a, C b, C &oa, C &ob) { oa = cmul(cneg(I), b); ob = cmul(I, a); });
        break;
    case QI_GATE_RX: {
        const double ch = std::cos(p[0] / 2), sh = std::sin(p[0] / 2);
        pair_gate([&](C a, C b, C &oa, C &ob) {
            oa = csub(rmul(ch, a), cmul(rmul(sh, I), b));
            ob = cadd(cmul(rmul(sh, cneg(I)), a), rmul(ch, b));
        });
        break;
    }
    case QI_GATE_RY: {
        const double ch = std::cos(p[0] / 2), sh = std::sin(p[0] / 2);
        pair_gate([&](C a, C b, C &oa, C &ob) { oa = csub(rmul(ch, a), rmul(sh, b)); ob = cadd(rmul(sh, a), rmul(ch, b)); });
        break;
    }
    case QI_GATE_Z: diag_gate({1, 0}, {-1, 0}, false); break;
    case QI_GATE_S: diag_gate({1, 0}, {0, 1}, false); break;
    case QI_GATE_SDAG: diag_gate({1, 0}, {0, -1}, false); break;
    case QI_GATE_T: diag_gate({1, 0}, {r2, r2}, false); break;
    case QI_GATE_TDAG: diag_gate({1, 0}, {r2, -r2}, false); break;
    case QI_GATE_P: diag_gate({1, 0}, {std::cos(p[0]), std::sin(p[0])}, false); break;
    case QI_GATE_RZ: {
        const double h = p[0] / 2;
        diag_gate({std::cos(h), -std::sin(h)}, {std::cos(h), std::sin(h)}, true);
        break;
    }
    case QI_GATE_SWAP: {
        const int t1 = g.targets[0], t2 = g.targets[1];
        std::vector<std::vector<Upd>> parts(threads);
        par_for(dim, threads, [&](int w, uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                if (((i >> t1) & 1ull) != ((i >> t2) & 1ull)) {
                    uint64_t j = i ^ (1ull << t1) ^ (1ull << t2);
                    if (i < j && check_controls(i, c, nc)) {
                        std::vector<Upd> pv{{i, state[j]}, {j, state[i]}};
                        parts[w].insert(parts[w].end(), pv.begin(), pv.end());
                    }
                }
            }
        });
        for (auto &pp : parts) for (auto &u : pp) nsv[u.idx] = u.val;
        break;
    }
    default:
        apply_gate(nsv.data(), n, g);
        break;
    }
    state.swap(nsv);
}
}  // namespace

extern "C" {

// Runs gates [0, n_gates) of the list on `sv` (in place) with the rayon-style
// data flow; returns the wall time in seconds.
double oracle_port_execute(double *sv, int n, const qi_gate *gates, int64_t n_gates, int threads) {
    const uint64_t dim = 1ull << n;
    std::vector<C> st(amp(sv), amp(sv) + dim);
    auto t0 = std::chrono::steady_clock::now();
    for (int64_t k = 0; k < n_gates; ++k) port_gate(st, n, gates[k], threads);
    auto t1 = std::chrono::steady_clock::now();
    std::memcpy(sv, st.data(), dim * sizeof(C));
    return std::chrono::duration<double>(t1 - t0).count();
}

// As oracle_port_execute, with the wall time of each gate written to secs_out[k].
double oracle_port_execute_timed(double *sv, int n, const qi_gate *gates, int64_t n_gates, int threads,
                                 double *secs_out) {
    const uint64_t dim = 1ull << n;
    std::vector<C> st(amp(sv), amp(sv) + dim);
    double total = 0.0;
    for (int64_t k = 0; k < n_gates; ++k) {
        auto t0 = std::chrono::steady_clock::now();
        port_gate(st, n, gates[k], threads);
        auto t1 = std::chrono::steady_clock::now();
        secs_out[k] = std::chrono::duration<double>(t1 - t0).count();
        total += secs_out[k];
    }
    std::memcpy(sv, st.data(), dim * sizeof(C));
    return total;
}

}  // extern "C"
