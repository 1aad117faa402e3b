// qi_adjoint.cu — adjoint (reverse-mode) gradient of <psi(theta)|H|psi(theta)>.
//
// No reference counterpart: quant-iron has parametric gates
// (src/components/parametric/parametric_gate.rs:30-211) but no gradient.
// Method: psi_N = U_N ... U_1 psi_0 (forward, fused plan); E = <psi_N|H|psi_N>;
// lambda_N = H psi_N; then for j = N .. 1:
//   psi_{j-1} = U_j^dagger psi_j
//   dE/dtheta += 2 Re <lambda_j| dU_j/dtheta |psi_{j-1}>      (FP64 accumulation)
//   lambda_{j-1} = U_j^dagger lambda_j
// The three steps of a parametric gate are one kernel: each work item loads
// its pair (or quad) of psi and lambda, writes both back un-applied and adds
// the derivative products to per-block FP64 partial sums.
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_plan.hpp"

#include <algorithm>
#include <cmath>
#include <complex>

namespace qi {

Status sumop_apply(qi_state *o, qi_state *in, const qi_pauli_term *terms, int64_t nt);
Status sumop_expectation(qi_state *s, const qi_pauli_term *terms, int64_t nt, double out[2]);

struct AdjParams {
    uint64_t nwork;
    uint64_t cmask;
    uint64_t b0, b1;
    int32_t np, nd;        // zero-insert positions, number of derivative matrices (<= 3)
    int8_t pos[44];
    double uinv[32];       // U^dagger, (2^NT)^2 complex, row-major
    double d[3][32];       // dU/dtheta_k
};

template <typename T, int NT>
__global__ void __launch_bounds__(256) k_adjoint(typename Cx<T>::V2 *psi, typename Cx<T>::V2 *lam, AdjParams p,
                                                 double *partials) {
    using X = Cx<T>;
    using V2 = typename X::V2;
    constexpr int D = 1 << NT;
    V2 u[D * D];
#pragma unroll
    for (int i = 0; i < D * D; ++i) u[i] = X::make((T)p.uinv[2 * i], (T)p.uinv[2 * i + 1]);
    // dU/dtheta_k in the state's precision, converted once per block (conversions of the
    // FP64 parameters inside the element loop would run on the FP64 pipe)
    __shared__ V2 sd[3 * D * D];
    for (int i = threadIdx.x; i < p.nd * D * D; i += blockDim.x)
        sd[i] = X::make((T)p.d[i / (D * D)][2 * (i % (D * D))], (T)p.d[i / (D * D)][2 * (i % (D * D)) + 1]);
    __syncthreads();
    double acc[3] = {0.0, 0.0, 0.0};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // per-thread sums in T over kAdjBatch elements, folded into FP64 once per outer step
    constexpr int kAdjBatch = 8;
    for (uint64_t wb = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wb < p.nwork; wb += stride * kAdjBatch) {
      T part0 = 0, part1 = 0, part2 = 0;
#pragma unroll 1
      for (int bs = 0; bs < kAdjBatch; ++bs) {
        const uint64_t w = wb + (uint64_t)bs * stride;
        if (w >= p.nwork) break;
        const uint64_t base = insert_zeros(w, p.pos, p.np) | p.cmask;
        uint64_t idx[D];
        idx[0] = base;
        idx[1] = base | p.b0;
        if constexpr (NT == 2) {
            idx[2] = base | p.b1;
            idx[3] = base | p.b0 | p.b1;
        }
        V2 x[D], l[D], xn[D], ln[D];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            x[r] = psi[idx[r]];
            l[r] = lam[idx[r]];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            V2 a = X::make(0, 0), b = X::make(0, 0);
#pragma unroll
            for (int c = 0; c < D; ++c) {
                a = X::fma(u[r * D + c], x[c], a);
                b = X::fma(u[r * D + c], l[c], b);
            }
            xn[r] = a;
            ln[r] = b;
        }
        for (int k = 0; k < p.nd; ++k) {
            T re = 0;
#pragma unroll
            for (int r = 0; r < D; ++r) {
                V2 dx = X::make(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) dx = X::fma(sd[k * D * D + r * D + c], xn[c], dx);
                re += l[r].x * dx.x + l[r].y * dx.y;   // Re(conj(lambda_r) * dx)
            }
            // three named sums (a dynamically indexed array would live in local memory)
            if (k == 0) part0 += re;
            else if (k == 1) part1 += re;
            else part2 += re;
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            psi[idx[r]] = xn[r];
            lam[idx[r]] = ln[r];
        }
      }
      acc[0] += (double)part0;
      acc[1] += (double)part1;
      acc[2] += (double)part2;
    }
    for (int k = 0; k < 3; ++k) {
        double v = block_sum(acc[k]);
        if (threadIdx.x == 0) partials[blockIdx.x * 4 + k] = v;
    }
}

// Fixed-order sum of the partial slots, written to out[0..ncomp).
__global__ void k_finalize_to(const double *partials, int nb, int ncomp, double *out) {
    for (int c = 0; c < ncomp; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i * 4 + c];
        double r = block_sum(acc);
        if (threadIdx.x == 0) out[c] = r;
        __syncthreads();
    }
}

static void inverse_matrix(const GateMatrix &g, double *out) {
    const int d = 1 << g.nt;
    for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) {
            out[2 * (r * d + c)] = g.m[2 * (c * d + r)];
            out[2 * (r * d + c) + 1] = -g.m[2 * (c * d + r) + 1];
        }
}

static bool differentiable(int kind) {
    switch (kind) {
    case QI_GATE_RX: case QI_GATE_RY: case QI_GATE_RZ: case QI_GATE_P: case QI_GATE_RYPHASE:
    case QI_GATE_RYPHASE_DAG: case QI_GATE_MATCHGATE:
        return true;
    default:
        return false;
    }
}

// dU/dp_k by Richardson-extrapolated central differences of the FP64 gate
// matrix (truncation O(h^4) = 1e-12, rounding ~1e-13 for h = 1e-3).
static Status derivative_matrix(int n, const qi_gate &g, int k, double *out) {
    const double h = 1e-3;
    GateMatrix mp1, mm1, mp2, mm2;
    qi_gate q = g;
    q.params[k] = g.params[k] + h;
    Status st = gate_to_matrix(n, q, &mp1);
    if (!st.ok()) return st;
    q.params[k] = g.params[k] - h;
    gate_to_matrix(n, q, &mm1);
    q.params[k] = g.params[k] + 2 * h;
    gate_to_matrix(n, q, &mp2);
    q.params[k] = g.params[k] - 2 * h;
    gate_to_matrix(n, q, &mm2);
    const int cnt = 2 * (1 << (2 * mp1.nt));
    for (int i = 0; i < cnt; ++i)
        out[i] = (8.0 * (mp1.m[i] - mm1.m[i]) - (mp2.m[i] - mm2.m[i])) / (12.0 * h);
    return ok_status();
}

static void fill_adj_positions(AdjParams &p, const GateMatrix &gm, uint64_t cmask) {
    uint64_t all = cmask;
    for (int j = 0; j < gm.nt; ++j) all |= 1ull << gm.t[j];
    int np = 0;
    for (int q = 0; q < 64; ++q)
        if ((all >> q) & 1ull) p.pos[np++] = (int8_t)q;
    p.np = np;
}

}  // namespace qi

using namespace qi;

extern "C" qi_status qi_adjoint_gradient(qi_state *s, const qi_gate *gates, int64_t n_gates, const double *theta,
                                         int64_t n_theta, const qi_pauli_term *terms, int64_t n_terms,
                                         const qi_exec_options *forward_opts, double *energy_out, double *grads_out) {
    if (!s || (!gates && n_gates > 0) || (!terms && n_terms > 0) || (!grads_out && n_theta > 0))
        return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    const int n = s->n;
    for (int64_t k = 0; k < n_terms; ++k) {
        Status st = validate_pauli(n, terms[k]);
        if (!st.ok()) return publish(st);
    }
    // resolve parameters + validate (whole list first)
    std::vector<qi_gate> resolved((size_t)n_gates);
    std::vector<GateMatrix> mats((size_t)n_gates);
    for (int64_t j = 0; j < n_gates; ++j) {
        qi_gate g = gates[j];
        for (int k = 0; k < 3; ++k) {
            if (g.param_ids[k] >= 0) {
                if (!theta || g.param_ids[k] >= n_theta)
                    return publish(err(QI_ERR_MISMATCHED_NUMBER_OF_PARAMETERS, g.param_ids[k] + 1, n_theta));
                if (!differentiable(g.kind))
                    return publish(err(QI_ERR_UNSUPPORTED, g.kind, j, "gate kind has no parameter derivative"));
                g.params[k] = theta[g.param_ids[k]];
            }
        }
        if (g.kind == QI_GATE_PAULI_STRING)
            return publish(err(QI_ERR_UNSUPPORTED, j, -1, "a normalising Pauli-string gate has no inverse"));
        Status st = gate_to_matrix(n, g, &mats[(size_t)j]);
        if (!st.ok()) return publish(st);
        resolved[(size_t)j] = g;
    }
    // forward sweep
    {
        qi_plan plan;
        plan.n = n;
        plan.prec = s->prec;
        if (forward_opts) plan.opts = *forward_opts;
        else plan.opts.fusion = QI_FUSION_GREEDY;
        std::vector<Elem> elems;
        Status st = plan_elems_from_gates(n, gates, n_gates, theta, n_theta, elems);
        if (st.ok()) st = build_plan(&plan, elems);
        if (st.ok()) st = upload_plan(&plan);
        if (st.ok()) st = plan_execute(&plan, s);
        if (plan.d_mats) cudaFree(plan.d_mats);
        if (plan.d_tc) cudaFree(plan.d_tc);
        if (!st.ok()) return publish(st);
    }
    double ev[2] = {0, 0};
    if (n_terms > 0) {
        Status st = sumop_expectation(s, terms, n_terms, ev);
        if (!st.ok()) return publish(st);
    }
    if (energy_out) *energy_out = ev[0];
    // lambda = H psi
    qi_state *lam = nullptr;
    qi_status cs = qi_state_create(n, s->prec, &lam);
    if (cs != QI_OK) return cs;
    qi_state_set_stream(lam, s->stream);
    Status st = ok_status();
    if (n_terms > 0) st = sumop_apply(lam, s, terms, n_terms);
    else e = cudaMemsetAsync(lam->amps, 0, lam->bytes(), s->stream);
    // derivative slots
    int64_t nslots = 0;
    for (int64_t j = 0; j < n_gates; ++j)
        for (int k = 0; k < 3; ++k)
            if (gates[j].param_ids[k] >= 0) ++nslots;
    double *d_gres = nullptr;
    if (st.ok() && nslots > 0) {
        e = cudaMalloc(&d_gres, (size_t)nslots * sizeof(double));
        if (e != cudaSuccess) st = cuda_status(e, "cudaMalloc(gradient slots)");
    }
    std::vector<std::pair<int64_t, int32_t>> slot_param;   // slot -> parameter id
    int64_t slot = nslots;
    const bool f32 = s->prec == QI_F32;
    for (int64_t j = n_gates - 1; j >= 0 && st.ok(); --j) {
        const GateMatrix &gm = mats[(size_t)j];
        const qi_gate &g = resolved[(size_t)j];
        int ids[3], nd = 0;
        for (int k = 0; k < 3; ++k)
            if (g.param_ids[k] >= 0) ids[nd++] = k;
        if (gm.pauli) {   // Pauli exponential: inverse exp(-alpha P), never parametric
            const double ar = -gm.alpha_re, ai = -gm.alpha_im;
            const double cre = std::cosh(ar) * std::cos(ai), cim = std::sinh(ar) * std::sin(ai);
            const double sre = std::sinh(ar) * std::cos(ai), sim = std::cosh(ar) * std::sin(ai);
            st = launch_pauli_exp(s, gm.xmask, gm.zmask, cre, cim, sre, sim);
            if (st.ok()) st = launch_pauli_exp(lam, gm.xmask, gm.zmask, cre, cim, sre, sim);
            continue;
        }
        if (gm.nt == 0) continue;   // identity
        if (nd == 0) {   // un-apply U^dagger on psi and lambda
            GateMatrix inv = gm;
            inverse_matrix(gm, inv.m);
            Op op = lower_gate(n, inv);
            st = launch_op(s, op, nullptr);
            if (st.ok()) st = launch_op(lam, op, nullptr);
            continue;
        }
        AdjParams p;
        std::memset(&p, 0, sizeof(p));
        uint64_t cm = 0;
        for (int32_t c : gm.controls) cm |= 1ull << c;
        p.cmask = cm;
        fill_adj_positions(p, gm, cm);
        p.b0 = 1ull << gm.t[0];
        p.b1 = gm.nt == 2 ? (1ull << gm.t[1]) : 0;
        inverse_matrix(gm, p.uinv);
        p.nd = nd;
        for (int q = 0; q < nd && st.ok(); ++q) st = derivative_matrix(n, g, ids[q], p.d[q]);
        if (!st.ok()) break;
        const int nc = __builtin_popcountll(cm);
        p.nwork = 1ull << (n - gm.nt - nc);
        uint64_t nb64 = (p.nwork + 255) / 256;
        const unsigned nb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nb64, kReduceBlocks));
        if (gm.nt == 1) {
            if (f32) k_adjoint<float, 1><<<nb, 256, 0, s->stream>>>((float2 *)s->amps, (float2 *)lam->amps, p, s->d_partials);
            else k_adjoint<double, 1><<<nb, 256, 0, s->stream>>>((double2 *)s->amps, (double2 *)lam->amps, p, s->d_partials);
        } else {
            if (f32) k_adjoint<float, 2><<<nb, 256, 0, s->stream>>>((float2 *)s->amps, (float2 *)lam->amps, p, s->d_partials);
            else k_adjoint<double, 2><<<nb, 256, 0, s->stream>>>((double2 *)s->amps, (double2 *)lam->amps, p, s->d_partials);
        }
        slot -= nd;
        k_finalize_to<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, nd, d_gres + slot);
        count_launch(2);
        st = check_launch("k_adjoint");
        for (int q = 0; q < nd; ++q) slot_param.push_back({slot + q, g.param_ids[ids[q]]});
    }
    if (st.ok()) {
        for (int64_t k = 0; k < n_theta; ++k) grads_out[k] = 0.0;
        std::vector<double> h((size_t)nslots, 0.0);
        if (nslots > 0) e = cudaMemcpyAsync(h.data(), d_gres, (size_t)nslots * sizeof(double), cudaMemcpyDeviceToHost,
                                            s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) st = cuda_status(e, "adjoint");
        for (auto &sp : slot_param) grads_out[sp.second] += 2.0 * h[(size_t)sp.first];
    }
    if (d_gres) cudaFree(d_gres);
    cudaStreamSynchronize(s->stream);
    qi_state_destroy(lam);
    return publish(st);
}
