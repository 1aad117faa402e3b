// qi_gates.cu — gate validation, gate -> matrix lowering and the per-gate
// streaming kernels (one HBM pass per gate).
//
// Reference: src/components/operator.rs — validate_qubits (:214-273),
// check_controls (:195-199) and the 16 Operator::apply implementations
// (:279-2285).  Semantics follow the reference's sequential CPU branch.
// Each kernel enumerates only the amplitudes the gate can change: the index
// space of the qubits that are neither target nor control, with the control
// bits forced to 1, so a gate with c controls touches 2^(n-c) amplitudes.
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <algorithm>
#include <cmath>

namespace qi {

// --------------------------------------------------------------- validation
// validate_qubits (operator.rs:214-273): target count, target range, control
// range and control/target overlap (controls outer, targets inner), then
// duplicate targets.
static Status validate_qubits(int n, const int32_t *t, int nt, const int32_t *c, int nc, int expected) {
    if (nt != expected) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, nt);
    for (int k = 0; k < nt; ++k)
        if (t[k] < 0 || t[k] >= n) return err(QI_ERR_INVALID_QUBIT_INDEX, t[k], n);
    for (int k = 0; k < nc; ++k) {
        if (c[k] < 0 || c[k] >= n) return err(QI_ERR_INVALID_QUBIT_INDEX, c[k], n);
        for (int j = 0; j < nt; ++j)
            if (c[k] == t[j]) return err(QI_ERR_OVERLAPPING_CONTROL_AND_TARGET, c[k], t[j]);
    }
    if (expected > 1)
        for (int i = 0; i < nt; ++i)
            for (int j = i + 1; j < nt; ++j)
                if (t[i] == t[j]) return err(QI_ERR_INVALID_QUBIT_INDEX, t[i], n);
    return ok_status();
}

Status validate_pauli(int n, const qi_pauli_term &t) {
    const uint64_t m = t.xmask | t.zmask;
    if (n < 64 && (m >> n)) {
        int q = n;
        while (!((m >> q) & 1ull)) ++q;
        return err(QI_ERR_INVALID_QUBIT_INDEX, q, n);
    }
    return ok_status();
}

Status validate_gate(int n, const qi_gate &g) {
    if (g.n_controls < 0 || g.n_controls > QI_MAX_CONTROLS) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, g.n_controls);
    if (g.n_targets < 0 || g.n_targets > 2) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, g.n_targets);
    const int32_t *t = g.targets, *c = g.controls;
    const int nt = g.n_targets, nc = g.n_controls;
    Status st;
    switch (g.kind) {
    case QI_GATE_H: case QI_GATE_X: case QI_GATE_Y: case QI_GATE_Z: case QI_GATE_S: case QI_GATE_T:
    case QI_GATE_SDAG: case QI_GATE_TDAG: case QI_GATE_P: case QI_GATE_RX: case QI_GATE_RY: case QI_GATE_RZ:
    case QI_GATE_U2: case QI_GATE_RYPHASE: case QI_GATE_RYPHASE_DAG: case QI_GATE_IDENTITY:
        return validate_qubits(n, t, nt, c, nc, 1);
    case QI_GATE_CNOT:   // operator.rs:667-685
        st = validate_qubits(n, t, nt, c, nc, 1);
        if (!st.ok()) return st;
        if (nc != 1) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, nc);
        return ok_status();
    case QI_GATE_TOFFOLI:   // operator.rs:1055-1075
        st = validate_qubits(n, t, nt, c, nc, 1);
        if (!st.ok()) return st;
        if (nc != 2) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, nc);
        if (c[0] == c[1]) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, nc);
        return ok_status();
    case QI_GATE_SWAP:
        return validate_qubits(n, t, nt, c, nc, 2);
    case QI_GATE_MATCHGATE:   // operator.rs:893-914
        st = validate_qubits(n, t, nt, c, nc, 1);
        if (!st.ok()) return st;
        if (t[0] == n - 1) return err(QI_ERR_INVALID_QUBIT_INDEX, t[0], n);
        return ok_status();
    case QI_GATE_PAULI_STRING: {
        qi_pauli_term pt = {g.params[0], g.params[1], g.xmask, g.zmask};
        return validate_pauli(n, pt);
    }
    case QI_GATE_PAULI_EVOLUTION: {   // pauli_string.rs:281-287
        qi_pauli_term pt = {g.params[0], g.params[1], g.xmask, g.zmask};
        if (g.params[1] != 0.0) {
            Status e = err(QI_ERR_INVALID_PAULI_COEFFICIENT);
            e.re = g.params[0];
            e.im = g.params[1];
            return e;
        }
        return validate_pauli(n, pt);
    }
    case QI_GATE_MEASUREMENT: {   // state.rs:543-552
        if (nt != 0) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, nt);
        if (t[0] < QI_BASIS_COMPUTATIONAL || t[0] > QI_BASIS_CUSTOM)
            return err(QI_ERR_INVALID_INPUT_VALUE, t[0], -1, "measurement basis");
        if (nc > n) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, n);
        for (int k = 0; k < nc; ++k)
            if (c[k] < 0 || c[k] >= n) return err(QI_ERR_INVALID_QUBIT_INDEX, c[k], n);
        if ((nc == 0 ? n : nc) > 24) return err(QI_ERR_UNSUPPORTED, nc == 0 ? n : nc, 24, "measuring more than 24 qubits");
        return ok_status();
    }
    default:
        return err(QI_ERR_INVALID_INPUT_VALUE, g.kind, -1, "unknown gate kind");
    }
}

// ----------------------------------------------------------------- matrices
static inline void setc(double *m, int idx, double re, double im) { m[2 * idx] = re; m[2 * idx + 1] = im; }

static void dedup_controls(const qi_gate &g, std::vector<int32_t> &out) {
    out.clear();
    for (int k = 0; k < g.n_controls; ++k)
        if (std::find(out.begin(), out.end(), g.controls[k]) == out.end()) out.push_back(g.controls[k]);
}

Status gate_to_matrix(int n, const qi_gate &g, GateMatrix *gm) {
    Status st = validate_gate(n, g);
    if (!st.ok()) return st;
    GateMatrix &o = *gm;
    o = GateMatrix();
    o.kind = g.kind;
    dedup_controls(g, o.controls);
    std::fill(o.m, o.m + 32, 0.0);
    const double *p = g.params;
    const double r = 1.0 / std::sqrt(2.0);
    o.nt = 1;
    o.t[0] = g.targets[0];
    auto m2 = [&](double a, double b, double c, double d, double e, double f, double gg, double h) {
        setc(o.m, 0, a, b); setc(o.m, 1, c, d); setc(o.m, 2, e, f); setc(o.m, 3, gg, h);
    };
    switch (g.kind) {
    case QI_GATE_H: m2(r, 0, r, 0, r, 0, -r, 0); break;
    case QI_GATE_X: case QI_GATE_CNOT: case QI_GATE_TOFFOLI: m2(0, 0, 1, 0, 1, 0, 0, 0); break;
    case QI_GATE_Y: m2(0, 0, 0, -1, 0, 1, 0, 0); break;
    case QI_GATE_Z: m2(1, 0, 0, 0, 0, 0, -1, 0); break;
    case QI_GATE_S: m2(1, 0, 0, 0, 0, 0, 0, 1); break;
    case QI_GATE_SDAG: m2(1, 0, 0, 0, 0, 0, 0, -1); break;
    case QI_GATE_T: m2(1, 0, 0, 0, 0, 0, r, r); break;
    case QI_GATE_TDAG: m2(1, 0, 0, 0, 0, 0, r, -r); break;
    case QI_GATE_P: m2(1, 0, 0, 0, 0, 0, std::cos(p[0]), std::sin(p[0])); break;
    case QI_GATE_RX: {
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        m2(c, 0, 0, -s, 0, -s, c, 0);
        break;
    }
    case QI_GATE_RY: {
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        m2(c, 0, -s, 0, s, 0, c, 0);
        break;
    }
    case QI_GATE_RZ: {
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        m2(c, -s, 0, 0, 0, 0, c, s);
        break;
    }
    case QI_GATE_U2: m2(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7]); break;
    case QI_GATE_RYPHASE: {   // operator.rs:2140-2156
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        const double er = std::cos(p[1]), ei = std::sin(p[1]);
        m2(c, 0, -er * s, -ei * s, s, 0, er * c, ei * c);
        break;
    }
    case QI_GATE_RYPHASE_DAG: {   // operator.rs:2172-2192
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        const double er = std::cos(-p[1]), ei = std::sin(-p[1]);
        m2(c, 0, s, 0, -er * s, -ei * s, er * c, ei * c);
        break;
    }
    case QI_GATE_IDENTITY: o.nt = 0; break;
    case QI_GATE_SWAP: {
        o.nt = 2;
        o.t[0] = std::min(g.targets[0], g.targets[1]);
        o.t[1] = std::max(g.targets[0], g.targets[1]);
        // basis |b1 b0> with b0 = t[0], b1 = t[1]
        setc(o.m, 0 * 4 + 0, 1, 0);
        setc(o.m, 1 * 4 + 2, 1, 0);
        setc(o.m, 2 * 4 + 1, 1, 0);
        setc(o.m, 3 * 4 + 3, 1, 0);
        break;
    }
    case QI_GATE_MATCHGATE: {   // operator.rs:893-1014, on (q1, q1 + 1)
        o.nt = 2;
        const int q1 = g.targets[0], q2 = q1 + 1;
        o.t[0] = q1;
        o.t[1] = q2;
        const double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
        const double e1r = std::cos(p[1]), e1i = std::sin(p[1]);
        const double e2r = std::cos(p[2]), e2i = std::sin(p[2]);
        // local index bit 0 = q1, bit 1 = q2: i01 -> 1, i10 -> 2, i11 -> 3.
        // The (i01, i10) rotation needs the controls on i01 (q2 = 0); a
        // control on q2 therefore disables it and leaves only the i11 phase.
        const bool q2_ctrl = std::find(o.controls.begin(), o.controls.end(), q2) != o.controls.end();
        setc(o.m, 0, 1, 0);
        if (q2_ctrl) {
            setc(o.m, 1 * 4 + 1, 1, 0);
            setc(o.m, 2 * 4 + 2, 1, 0);
            o.controls.erase(std::remove(o.controls.begin(), o.controls.end(), q2), o.controls.end());
        } else {
            setc(o.m, 1 * 4 + 1, c, 0);
            setc(o.m, 1 * 4 + 2, -e1r * s, -e1i * s);
            setc(o.m, 2 * 4 + 1, s, 0);
            setc(o.m, 2 * 4 + 2, e1r * c, e1i * c);
        }
        setc(o.m, 3 * 4 + 3, e2r, e2i);
        break;
    }
    case QI_GATE_PAULI_STRING:
    case QI_GATE_PAULI_EVOLUTION: {
        o.nt = 0;
        o.pauli = true;
        o.xmask = g.xmask;
        o.zmask = g.zmask;
        if (g.kind == QI_GATE_PAULI_STRING) {
            o.normalise_after = true;
        } else {
            // alpha = coefficient * (-i dt)   (pauli_string.rs:281-287)
            const double cr = g.params[0], ci = g.params[1], dt = g.params[2];
            o.alpha_re = ci * dt;
            o.alpha_im = -cr * dt;
        }
        break;
    }
    case QI_GATE_MEASUREMENT: {
        o.nt = 0;
        o.measure = true;
        o.controls.clear();
        o.basis = g.targets[0];
        o.seed = g.xmask;
        for (int k = 0; k < g.n_controls; ++k) o.measured.push_back(g.controls[k]);
        if (o.measured.empty())
            for (int q = 0; q < n; ++q) o.measured.push_back(q);
        std::copy(g.params, g.params + 8, o.m);
        break;
    }
    default: return err(QI_ERR_INVALID_INPUT_VALUE, g.kind);
    }
    // diagonal?
    if (o.nt == 1) o.diagonal = o.m[2] == 0 && o.m[3] == 0 && o.m[4] == 0 && o.m[5] == 0;
    else if (o.nt == 2) {
        bool d = true;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                if (i != j && (o.m[2 * (i * 4 + j)] != 0 || o.m[2 * (i * 4 + j) + 1] != 0)) d = false;
        o.diagonal = d;
    }
    return ok_status();
}

Op lower_gate(int n, const GateMatrix &gm) {
    (void)n;
    Op op;
    uint64_t cm = 0;
    for (int32_t c : gm.controls) cm |= 1ull << c;
    op.cmask = cm;
    if (gm.pauli) {
        op.kind = gm.normalise_after ? OP_PAULI_NORM : OP_PAULI_EXP;
        op.xmask = gm.xmask;
        op.zmask = gm.zmask;
        op.alpha_re = gm.alpha_re;
        op.alpha_im = gm.alpha_im;
        return op;
    }
    if (gm.measure) {
        op.kind = OP_MEASURE;
        op.mode = gm.basis;
        op.k = (int32_t)gm.measured.size();
        for (size_t k = 0; k < gm.measured.size(); ++k) op.perm[k] = (int8_t)gm.measured[k];
        op.xmask = gm.seed;
        std::copy(gm.m, gm.m + 8, op.m);
        return op;
    }
    if (gm.nt == 0) { op.kind = OP_NOP; return op; }
    if (gm.nt == 1) {
        op.kind = OP_MAT1;
        op.k = 1;
        op.targets[0] = gm.t[0];
        std::copy(gm.m, gm.m + 8, op.m);
        const double *m = gm.m;
        const bool off_zero = m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0;
        const bool diag_zero = m[0] == 0 && m[1] == 0 && m[6] == 0 && m[7] == 0;
        if (off_zero && m[0] == 1 && m[1] == 0) op.mode = M1_PHASE1;
        else if (off_zero) op.mode = M1_DIAG;
        else if (diag_zero) op.mode = M1_ANTIDIAG;
        else if (m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0) op.mode = M1_REAL;
        else op.mode = M1_GENERAL;
        return op;
    }
    if (gm.kind == QI_GATE_SWAP) {
        op.kind = OP_SWAP;
        op.k = 2;
        op.targets[0] = gm.t[0];
        op.targets[1] = gm.t[1];
        return op;
    }
    op.kind = OP_MAT2;
    op.k = 2;
    op.targets[0] = gm.t[0];
    op.targets[1] = gm.t[1];
    std::copy(gm.m, gm.m + 32, op.m);
    return op;
}

// ------------------------------------------------------------------ kernels
struct GateParams {
    uint64_t nwork;    // work items (each: one amplitude pair / quad, or two with VEC)
    uint64_t cmask;    // control bits, set to 1
    uint64_t b0, b1;   // target bit masks (b1 for SWAP / MAT2)
    int32_t np;        // number of zero-insert positions
    int8_t pos[44];    // ascending positions of targets and controls
    double m[32];      // complex matrix entries (row-major)
};

// Phase-1 fast paths (multiplication by -1, +i, -i is exact and needs no FMA).
enum PhaseKind : int { PH_GENERAL = 0, PH_NEG = 1, PH_I = 2, PH_NEG_I = 3 };

template <typename T>
struct Mat1Coef {
    typename Cx<T>::V2 m00, m01, m10, m11;
    __device__ Mat1Coef(const double *m)
        : m00(Cx<T>::make((T)m[0], (T)m[1])), m01(Cx<T>::make((T)m[2], (T)m[3])),
          m10(Cx<T>::make((T)m[4], (T)m[5])), m11(Cx<T>::make((T)m[6], (T)m[7])) {}
};

template <typename T, int MODE, int PH>
__device__ __forceinline__ void mat1_update(typename Cx<T>::V2 &a0, typename Cx<T>::V2 &a1, const Mat1Coef<T> &c) {
    using X = Cx<T>;
    if constexpr (MODE == M1_GENERAL) {
        typename X::V2 o0 = X::fma(c.m01, a1, X::mul(c.m00, a0));
        typename X::V2 o1 = X::fma(c.m11, a1, X::mul(c.m10, a0));
        a0 = o0; a1 = o1;
    } else if constexpr (MODE == M1_REAL) {
        const T r00 = c.m00.x, r01 = c.m01.x, r10 = c.m10.x, r11 = c.m11.x;
        typename X::V2 o0 = X::make(r00 * a0.x + r01 * a1.x, r00 * a0.y + r01 * a1.y);
        typename X::V2 o1 = X::make(r10 * a0.x + r11 * a1.x, r10 * a0.y + r11 * a1.y);
        a0 = o0; a1 = o1;
    } else if constexpr (MODE == M1_DIAG) {
        a0 = X::mul(c.m00, a0);
        a1 = X::mul(c.m11, a1);
    } else if constexpr (MODE == M1_ANTIDIAG) {
        typename X::V2 o0, o1;
        if constexpr (PH == PH_NEG) {   // Pauli X: plain swap
            o0 = a1; o1 = a0;
        } else if constexpr (PH == PH_I) {   // Pauli Y: o0 = -i a1, o1 = i a0
            o0 = X::make(a1.y, -a1.x);
            o1 = X::make(-a0.y, a0.x);
        } else {
            o0 = X::mul(c.m01, a1);
            o1 = X::mul(c.m10, a0);
        }
        a0 = o0; a1 = o1;
    } else {   // M1_PHASE1: only a1 changes
        if constexpr (PH == PH_NEG) a1 = X::make(-a1.x, -a1.y);
        else if constexpr (PH == PH_I) a1 = X::make(-a1.y, a1.x);
        else if constexpr (PH == PH_NEG_I) a1 = X::make(a1.y, -a1.x);
        else a1 = X::mul(c.m11, a1);
    }
}

// One target, controlled.  VEC (FP32 only, all special qubits >= 1): a work
// item covers two consecutive base indices, loaded as one float4 per side.
template <typename T, int MODE, int PH, bool VEC>
__global__ void __launch_bounds__(256) k_mat1(typename Cx<T>::V2 *a, GateParams p) {
    using V2 = typename Cx<T>::V2;
    const Mat1Coef<T> c(p.m);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += stride) {
        const uint64_t i0 = insert_zeros(VEC ? (w << 1) : w, p.pos, p.np) | p.cmask;
        const uint64_t i1 = i0 | p.b0;
        if constexpr (VEC) {
            float4 *a4 = reinterpret_cast<float4 *>(a);
            if constexpr (MODE == M1_PHASE1) {
                float4 v = a4[i1 >> 1];
                float2 x = make_float2(v.x, v.y), y = make_float2(v.z, v.w), d0 = make_float2(0.f, 0.f);
                mat1_update<float, MODE, PH>(d0, x, c);
                mat1_update<float, MODE, PH>(d0, y, c);
                a4[i1 >> 1] = make_float4(x.x, x.y, y.x, y.y);
            } else {
                float4 u = a4[i0 >> 1], v = a4[i1 >> 1];
                float2 u0 = make_float2(u.x, u.y), u1 = make_float2(u.z, u.w);
                float2 v0 = make_float2(v.x, v.y), v1 = make_float2(v.z, v.w);
                mat1_update<float, MODE, PH>(u0, v0, c);
                mat1_update<float, MODE, PH>(u1, v1, c);
                a4[i0 >> 1] = make_float4(u0.x, u0.y, u1.x, u1.y);
                a4[i1 >> 1] = make_float4(v0.x, v0.y, v1.x, v1.y);
            }
        } else {
            if constexpr (MODE == M1_PHASE1) {
                V2 y = a[i1], d0 = Cx<T>::make(T(0), T(0));
                mat1_update<T, MODE, PH>(d0, y, c);
                a[i1] = y;
            } else {
                V2 x = a[i0], y = a[i1];
                mat1_update<T, MODE, PH>(x, y, c);
                a[i0] = x;
                a[i1] = y;
            }
        }
    }
}

// One target on qubit 0 (FP32): a pair (i0, i0 + 1) is one 16-byte load and store, so a
// warp moves 512 contiguous bytes per instruction (the generic path's two 8-byte accesses
// per pair sit 8 bytes apart).  Two pairs per thread are in flight.
template <int MODE, int PH>
__global__ void __launch_bounds__(256) k_mat1_q0(float2 *a, GateParams p) {
    const Mat1Coef<float> c(p.m);
    float4 *a4 = reinterpret_cast<float4 *>(a);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += 2 * stride) {
        const bool two = w + stride < p.nwork;
        const uint64_t j0 = (insert_zeros(w, p.pos, p.np) | p.cmask) >> 1;
        const uint64_t j1 = two ? (insert_zeros(w + stride, p.pos, p.np) | p.cmask) >> 1 : j0;
        float4 u = a4[j0], v = two ? a4[j1] : u;
        float2 x0 = make_float2(u.x, u.y), y0 = make_float2(u.z, u.w);
        float2 x1 = make_float2(v.x, v.y), y1 = make_float2(v.z, v.w);
        mat1_update<float, MODE, PH>(x0, y0, c);
        mat1_update<float, MODE, PH>(x1, y1, c);
        a4[j0] = make_float4(x0.x, x0.y, y0.x, y0.y);
        if (two) a4[j1] = make_float4(x1.x, x1.y, y1.x, y1.y);
    }
}

template <typename T, bool VEC>
__global__ void __launch_bounds__(256) k_swap(typename Cx<T>::V2 *a, GateParams p) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += stride) {
        const uint64_t base = insert_zeros(VEC ? (w << 1) : w, p.pos, p.np) | p.cmask;
        const uint64_t i01 = base | p.b0, i10 = base | p.b1;
        if constexpr (VEC) {
            float4 *a4 = reinterpret_cast<float4 *>(a);
            float4 x = a4[i01 >> 1], y = a4[i10 >> 1];
            a4[i01 >> 1] = y;
            a4[i10 >> 1] = x;
        } else {
            typename Cx<T>::V2 x = a[i01], y = a[i10];
            a[i01] = y;
            a[i10] = x;
        }
    }
}

template <typename T>
__device__ __forceinline__ void mat2_update(typename Cx<T>::V2 v[4], const typename Cx<T>::V2 m[16]) {
    using X = Cx<T>;
    typename X::V2 o[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        typename X::V2 acc = X::mul(m[r * 4], v[0]);
#pragma unroll
        for (int c = 1; c < 4; ++c) acc = X::fma(m[r * 4 + c], v[c], acc);
        o[r] = acc;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) v[r] = o[r];
}

template <typename T, bool VEC>
__global__ void __launch_bounds__(256) k_mat2(typename Cx<T>::V2 *a, GateParams p) {
    using V2 = typename Cx<T>::V2;
    V2 m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = Cx<T>::make((T)p.m[2 * i], (T)p.m[2 * i + 1]);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += stride) {
        const uint64_t base = insert_zeros(VEC ? (w << 1) : w, p.pos, p.np) | p.cmask;
        const uint64_t idx[4] = {base, base | p.b0, base | p.b1, base | p.b0 | p.b1};
        if constexpr (VEC) {
            float4 *a4 = reinterpret_cast<float4 *>(a);
            float4 q[4];
            float2 lo[4], hi[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) q[j] = a4[idx[j] >> 1];
#pragma unroll
            for (int j = 0; j < 4; ++j) { lo[j] = make_float2(q[j].x, q[j].y); hi[j] = make_float2(q[j].z, q[j].w); }
            mat2_update<float>(lo, reinterpret_cast<const float2 *>(m));
            mat2_update<float>(hi, reinterpret_cast<const float2 *>(m));
#pragma unroll
            for (int j = 0; j < 4; ++j) a4[idx[j] >> 1] = make_float4(lo[j].x, lo[j].y, hi[j].x, hi[j].y);
        } else {
            V2 v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = a[idx[j]];
            mat2_update<T>(v, m);
#pragma unroll
            for (int j = 0; j < 4; ++j) a[idx[j]] = v[j];
        }
    }
}

// ------------------------------------------------------------------ launch
static unsigned gate_grid(uint64_t work) {
    uint64_t g = (work + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152 * 8) g = 152 * 8;
    return (unsigned)g;
}

static void fill_positions(GateParams &p, const int32_t *targets, int k, uint64_t cmask) {
    int8_t tmp[64];
    int np = 0;
    uint64_t all = cmask;
    for (int j = 0; j < k; ++j) all |= 1ull << targets[j];
    for (int q = 0; q < 64; ++q)
        if ((all >> q) & 1ull) tmp[np++] = (int8_t)q;
    p.np = np;
    for (int j = 0; j < np; ++j) p.pos[j] = tmp[j];
}

static int phase_kind(const Op &op) {
    if (op.mode == M1_ANTIDIAG) {
        const double *m = op.m;
        if (m[2] == 1 && m[3] == 0 && m[4] == 1 && m[5] == 0) return PH_NEG;    // X: marker "swap"
        if (m[2] == 0 && m[3] == -1 && m[4] == 0 && m[5] == 1) return PH_I;     // Y
        return PH_GENERAL;
    }
    if (op.mode == M1_PHASE1) {
        const double *m = op.m;
        if (m[6] == -1 && m[7] == 0) return PH_NEG;
        if (m[6] == 0 && m[7] == 1) return PH_I;
        if (m[6] == 0 && m[7] == -1) return PH_NEG_I;
    }
    return PH_GENERAL;
}

static void launch_mat1_q0(float2 *a, const GateParams &p, int mode, int ph, unsigned g, cudaStream_t st) {
#define QI_M1(MODE, PH) k_mat1_q0<MODE, PH><<<g, 256, 0, st>>>(a, p)
    switch (mode) {
    case M1_GENERAL: QI_M1(M1_GENERAL, PH_GENERAL); break;
    case M1_REAL: QI_M1(M1_REAL, PH_GENERAL); break;
    case M1_DIAG: QI_M1(M1_DIAG, PH_GENERAL); break;
    case M1_ANTIDIAG:
        if (ph == PH_NEG) QI_M1(M1_ANTIDIAG, PH_NEG);
        else if (ph == PH_I) QI_M1(M1_ANTIDIAG, PH_I);
        else QI_M1(M1_ANTIDIAG, PH_GENERAL);
        break;
    default:
        if (ph == PH_NEG) QI_M1(M1_PHASE1, PH_NEG);
        else if (ph == PH_I) QI_M1(M1_PHASE1, PH_I);
        else if (ph == PH_NEG_I) QI_M1(M1_PHASE1, PH_NEG_I);
        else QI_M1(M1_PHASE1, PH_GENERAL);
        break;
    }
#undef QI_M1
}

template <typename T, bool VEC>
static void launch_mat1_t(typename Cx<T>::V2 *a, const GateParams &p, int mode, int ph, unsigned g, cudaStream_t st) {
#define QI_M1(MODE, PH) k_mat1<T, MODE, PH, VEC><<<g, 256, 0, st>>>(a, p)
    switch (mode) {
    case M1_GENERAL: QI_M1(M1_GENERAL, PH_GENERAL); break;
    case M1_REAL: QI_M1(M1_REAL, PH_GENERAL); break;
    case M1_DIAG: QI_M1(M1_DIAG, PH_GENERAL); break;
    case M1_ANTIDIAG:
        if (ph == PH_NEG) QI_M1(M1_ANTIDIAG, PH_NEG);
        else if (ph == PH_I) QI_M1(M1_ANTIDIAG, PH_I);
        else QI_M1(M1_ANTIDIAG, PH_GENERAL);
        break;
    default:
        if (ph == PH_NEG) QI_M1(M1_PHASE1, PH_NEG);
        else if (ph == PH_I) QI_M1(M1_PHASE1, PH_I);
        else if (ph == PH_NEG_I) QI_M1(M1_PHASE1, PH_NEG_I);
        else QI_M1(M1_PHASE1, PH_GENERAL);
        break;
    }
#undef QI_M1
}

Status launch_op(qi_state *s, const Op &op, const void *d_mats, const void *d_tc) {
    const int n = s->n;
    const bool f32 = s->prec == QI_F32;
    GateParams p;
    std::memset(&p, 0, sizeof(p));
    p.cmask = op.cmask;
    const int nc = __builtin_popcountll(op.cmask);
    switch (op.kind) {
    case OP_NOP: return ok_status();
    case OP_MAT1: {
        fill_positions(p, op.targets, 1, op.cmask);
        p.b0 = 1ull << op.targets[0];
        std::copy(op.m, op.m + 8, p.m);
        const int free_bits = n - 1 - nc;
        const bool vec = f32 && p.pos[0] >= 1 && free_bits >= 1;
        p.nwork = 1ull << (free_bits - (vec ? 1 : 0));
        const unsigned g = gate_grid(p.nwork);
        const int ph = phase_kind(op);
        if (f32 && op.targets[0] == 0) {   // pairs are adjacent: one 16-byte access each
            launch_mat1_q0((float2 *)s->amps, p, op.mode, ph, gate_grid((p.nwork + 1) / 2), s->stream);
        } else if (f32) {
            if (vec) launch_mat1_t<float, true>((float2 *)s->amps, p, op.mode, ph, g, s->stream);
            else launch_mat1_t<float, false>((float2 *)s->amps, p, op.mode, ph, g, s->stream);
        } else {
            launch_mat1_t<double, false>((double2 *)s->amps, p, op.mode, ph, g, s->stream);
        }
        count_launch();
        return check_launch("k_mat1");
    }
    case OP_SWAP:
    case OP_MAT2: {
        fill_positions(p, op.targets, 2, op.cmask);
        p.b0 = 1ull << op.targets[0];
        p.b1 = 1ull << op.targets[1];
        std::copy(op.m, op.m + 32, p.m);
        const int free_bits = n - 2 - nc;
        const bool vec = f32 && p.pos[0] >= 1 && free_bits >= 1;
        p.nwork = 1ull << (free_bits - (vec ? 1 : 0));
        const unsigned g = gate_grid(p.nwork);
        if (op.kind == OP_SWAP) {
            if (f32) {
                if (vec) k_swap<float, true><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
                else k_swap<float, false><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
            } else {
                k_swap<double, false><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p);
            }
        } else {
            if (f32) {
                if (vec) k_mat2<float, true><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
                else k_mat2<float, false><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
            } else {
                k_mat2<double, false><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p);
            }
        }
        count_launch();
        return check_launch(op.kind == OP_SWAP ? "k_swap" : "k_mat2");
    }
    case OP_PAULI_EXP:
        return launch_pauli_exp(s, op.xmask, op.zmask, op.cre, op.cim, op.sre, op.sim);
    case OP_PAULI_GROUP:
        return launch_pauli_group(s, op, d_mats);
    case OP_PAULI_NORM: {
        Status st = launch_pauli_exp(s, op.xmask, op.zmask, 0.0, 0.0, 1.0, 0.0);   // P psi
        if (!st.ok()) return st;
        return state_normalise_device_async(s);
    }
    case OP_FUSED: {
        const size_t esz = f32 ? sizeof(float2) : sizeof(double2);
        const char *mp = (const char *)d_mats + (size_t)op.mat_offset * esz;
        const void *tp = (d_tc && op.tc_offset >= 0) ? (const void *)((const float *)d_tc + op.tc_offset) : nullptr;
        const void *pp = (d_tc && op.poly_tc >= 0) ? (const void *)((const float *)d_tc + op.poly_tc) : nullptr;
        return launch_fused(s, op.k, op.targets, mp, tp, op.mode, pp);
    }
    case OP_NORMALISE:
        return state_normalise_device_async(s);
    case OP_DIAGK: {
        const size_t esz = f32 ? sizeof(float2) : sizeof(double2);
        const char *mp = (const char *)d_mats + (size_t)op.mat_offset * esz;
        return launch_diagk(s, op.k, op.targets, mp);
    }
    case OP_PHASE_POLY: {
        if (!d_tc || op.tc_offset < 0) return err(QI_ERR_UNKNOWN, op.kind, -1, "phase polynomial without its block");
        return launch_phase_poly(s, (const float *)d_tc + op.tc_offset);
    }
    case OP_MEASURE: {   // Gate::Measurement keeps the collapsed state (gate.rs:104-106)
        int32_t q[64];
        for (int k = 0; k < op.k; ++k) q[k] = op.perm[k];
        uint64_t outcome = 0;
        return measure_state(s, op.mode, op.m, q, op.k, op.xmask, &outcome, nullptr);
    }
    default:
        return err(QI_ERR_UNKNOWN, op.kind, -1, "unknown op");
    }
}

}  // namespace qi

using namespace qi;

extern "C" {

qi_status qi_apply_gate(qi_state *s, const qi_gate *g) {
    if (!s || !g) return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    if (g->kind == QI_GATE_PAULI_STRING || g->kind == QI_GATE_PAULI_EVOLUTION) {
        GateMatrix gm;
        Status st = gate_to_matrix(s->n, *g, &gm);
        if (!st.ok()) return publish(st);
        Op op = lower_gate(s->n, gm);
        if (op.kind == OP_PAULI_EXP) {
            // cosh/sinh of alpha (num_complex formulas) computed in FP64 on the host
            const double ar = op.alpha_re, ai = op.alpha_im;
            op.cre = std::cosh(ar) * std::cos(ai);
            op.cim = std::sinh(ar) * std::sin(ai);
            op.sre = std::sinh(ar) * std::cos(ai);
            op.sim = std::cosh(ar) * std::sin(ai);
        }
        st = launch_op(s, op, nullptr);
        if (!st.ok()) return publish(st);
        if (op.kind == OP_PAULI_NORM) {
            int flag = 0;
            st = state_read_flag(s, &flag);
            if (!st.ok()) return publish(st);
            if (flag) return publish(err(QI_ERR_ZERO_NORM));
        }
        return publish(ok_status());
    }
    GateMatrix gm;
    Status st = gate_to_matrix(s->n, *g, &gm);
    if (!st.ok()) return publish(st);
    Op op = lower_gate(s->n, gm);
    return publish(launch_op(s, op, nullptr));
}

qi_status qi_unitary2_check(const double m[8]) {   // operator.rs:2092-2125
    if (!m) return publish(err(QI_ERR_NULL_ARGUMENT));
    const double tol = 2.220446049250313e-16 * 2.0;
    auto ns = [](double r, double i) { return r * r + i * i; };
    const double ar = m[0], ai = m[1], br = m[2], bi = m[3], cr = m[4], ci = m[5], dr = m[6], di = m[7];
    if (std::fabs((ns(ar, ai) + ns(br, bi)) - 1.0) > tol) return publish(err(QI_ERR_NON_UNITARY_MATRIX));
    if (std::fabs((ns(cr, ci) + ns(dr, di)) - 1.0) > tol) return publish(err(QI_ERR_NON_UNITARY_MATRIX));
    // a*conj(c) + b*conj(d)
    const double xr = (ar * cr - ai * -ci) + (br * dr - bi * -di);
    const double xi = (ar * -ci + ai * cr) + (br * -di + bi * dr);
    if (ns(xr, xi) > tol * tol) return publish(err(QI_ERR_NON_UNITARY_MATRIX));
    return publish(ok_status());
}

}  // extern "C"
