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
// the derivative products to per-block FP64 partial sums.  Runs of single-qubit
// gates share one such pass (k_adjoint_multi), and runs of fixed gates are
// un-applied on both states by one fused plan of their inverses.
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_plan.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <memory>

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

// A group of single-qubit gates, consecutive in the reverse sweep, on at most kMultiQubits
// distinct qubits with at most kMultiStages gates per qubit.  Gates on distinct qubits
// commute (and commute with one another's derivatives), so the group is processed qubit by
// qubit in ascending order, each qubit's gates in sweep order: a work item holds the 2^M
// amplitudes of psi and lambda its qubits span and, gate after gate, un-applies U on psi,
// accumulates Re(conj(lambda) dU psi) and un-applies U on lambda, all in registers.
constexpr int kMultiQubits = 4, kMultiStages = 2, kMultiComps = kMultiQubits * kMultiStages;
struct MultiParams {
    uint64_t nwork;
    int8_t pos[kMultiQubits];                     // the group's qubits, ascending (combo bit i <-> pos[i])
    double uinv[kMultiQubits][kMultiStages][8];   // qubit i, stage s: U^dagger, 2x2 complex row-major
    double d[kMultiQubits][kMultiStages][8];      // dU/dtheta (zero for a fixed gate or an unused stage)
};

// Shared-memory read the compiler may not hoist out of the work loop: the group's
// matrices are re-read (broadcast) per work item instead of pinning 16 registers per gate.
__device__ __forceinline__ float2 lds_fresh(const float2 *p) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ double2 lds_fresh(const double2 *p) {
    double2 v;
    asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}

template <typename T, int M, int S>
__global__ void __launch_bounds__(256, (1 << M) * sizeof(T) >= 64 ? 1 : 2) k_adjoint_multi(typename Cx<T>::V2 *psi, typename Cx<T>::V2 *lam,
                                                          const __grid_constant__ MultiParams p, double *partials) {
    using X = Cx<T>;
    using V2 = typename X::V2;
    constexpr int D = 1 << M;
    __shared__ V2 s_u[M][S][4], s_d[M][S][4];   // uniform across the block: broadcast reads
    if (threadIdx.x < 4 * M * S) {
        const int g = threadIdx.x / (4 * S), st = (threadIdx.x >> 2) % S, i = threadIdx.x & 3;
        s_u[g][st][i] = X::make((T)p.uinv[g][st][2 * i], (T)p.uinv[g][st][2 * i + 1]);
        s_d[g][st][i] = X::make((T)p.d[g][st][2 * i], (T)p.d[g][st][2 * i + 1]);
    }
    __syncthreads();
    uint64_t bitm[M];
#pragma unroll
    for (int i = 0; i < M; ++i) bitm[i] = 1ull << p.pos[i];
    double acc[M * S];
#pragma unroll
    for (int g = 0; g < M * S; ++g) acc[g] = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += stride) {
        const uint64_t base = insert_zeros(w, p.pos, M);
        V2 x[D], l[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            uint64_t o = base;
#pragma unroll
            for (int i = 0; i < M; ++i)
                if ((c >> i) & 1) o |= bitm[i];
            x[c] = psi[o];
            l[c] = lam[o];
        }
#pragma unroll
        for (int g = 0; g < M; ++g) {   // qubit pos[g] is combo bit g: compile-time pair indices
#pragma unroll
            for (int st = 0; st < S; ++st) {
                const V2 u0 = lds_fresh(&s_u[g][st][0]), u1 = lds_fresh(&s_u[g][st][1]);
                const V2 u2 = lds_fresh(&s_u[g][st][2]), u3 = lds_fresh(&s_u[g][st][3]);
                const V2 e0 = lds_fresh(&s_d[g][st][0]), e1 = lds_fresh(&s_d[g][st][1]);
                const V2 e2 = lds_fresh(&s_d[g][st][2]), e3 = lds_fresh(&s_d[g][st][3]);
                T part = 0;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    if ((c >> g) & 1) continue;
                    const int c1 = c | (1 << g);
                    const V2 x0 = x[c], x1 = x[c1], l0 = l[c], l1 = l[c1];
                    const V2 xn0 = X::fma(u1, x1, X::mul(u0, x0)), xn1 = X::fma(u3, x1, X::mul(u2, x0));
                    const V2 d0 = X::fma(e1, xn1, X::mul(e0, xn0));
                    const V2 d1 = X::fma(e3, xn1, X::mul(e2, xn0));
                    part += l0.x * d0.x + l0.y * d0.y + l1.x * d1.x + l1.y * d1.y;   // Re(conj(lambda) dU psi')
                    x[c] = xn0;
                    x[c1] = xn1;
                    l[c] = X::fma(u1, l1, X::mul(u0, l0));
                    l[c1] = X::fma(u3, l1, X::mul(u2, l0));
                }
                acc[g * S + st] += (double)part;
            }
        }
#pragma unroll
        for (int c = 0; c < D; ++c) {
            uint64_t o = base;
#pragma unroll
            for (int i = 0; i < M; ++i)
                if ((c >> i) & 1) o |= bitm[i];
            psi[o] = x[c];
            lam[o] = l[c];
        }
    }
#pragma unroll
    for (int g = 0; g < M * S; ++g) {
        const double v = block_sum(acc[g]);
        if (threadIdx.x == 0) partials[blockIdx.x * kMultiComps + g] = v;
    }
}

// Fixed-order sum of the partial slots (block i, component c at partials[i * stride + c]),
// written to out[0..ncomp).
__global__ void k_finalize_to(const double *partials, int nb, int ncomp, int stride, double *out) {
    for (int c = 0; c < ncomp; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i * stride + c];
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
    // forward sweep; the reverse sweep's fixed-gate segments use the same options
    qi_exec_options plan_opts = {QI_FUSION_GREEDY, 0, 0, 0};
    if (forward_opts) plan_opts = *forward_opts;
    {
        qi_plan plan;
        plan.n = n;
        plan.prec = s->prec;
        plan.opts = plan_opts;
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
    // derivative slots (one per parameter of a gate; a gate group uses one per member)
    const int64_t nslots = 3 * n_gates + kMultiComps;
    double *d_gres = nullptr;
    if (st.ok() && nslots > 0) {
        e = cudaMalloc(&d_gres, (size_t)nslots * sizeof(double));
        if (e != cudaSuccess) st = cuda_status(e, "cudaMalloc(gradient slots)");
    }
    std::vector<std::pair<int64_t, int32_t>> slot_param;   // slot -> parameter id
    int64_t slot = nslots;
    const bool f32 = s->prec == QI_F32;
    auto n_params = [&](int64_t jj) {
        int c = 0;
        for (int k = 0; k < 3; ++k) c += resolved[(size_t)jj].param_ids[k] >= 0;
        return c;
    };
    // a single-qubit, uncontrolled gate with at most one parameter can join a gate group
    auto groupable = [&](int64_t jj) {
        const GateMatrix &m = mats[(size_t)jj];
        return !m.pauli && m.nt == 1 && m.controls.empty() && n_params(jj) <= 1;
    };
    std::vector<std::unique_ptr<qi_plan>> seg_plans;   // kept until the sweep has run
    for (int64_t j = n_gates - 1; j >= 0 && st.ok();) {
        // single-qubit gates, consecutive in reverse, on at most kMultiQubits qubits with at
        // most kMultiStages gates each: one pass for the group
        int qcount[64] = {0};
        uint64_t qmask = 0;
        int64_t jj = j;
        const int max_q = f32 ? kMultiQubits : kMultiQubits - 1;   // FP64 x 16 amplitudes spills
        for (; jj >= 0 && groupable(jj); --jj) {
            const int q = mats[(size_t)jj].t[0];
            if (!((qmask >> q) & 1ull) && __builtin_popcountll(qmask) == max_q) break;
            if (qcount[q] == kMultiStages) break;
            qmask |= 1ull << q;
            ++qcount[q];
        }
        const int64_t gsize = j - jj;
        if (gsize >= 2) {
            MultiParams mp;
            std::memset(&mp, 0, sizeof(mp));
            const int M = __builtin_popcountll(qmask);
            int S = 1, b_of[64];
            for (int q = 0, i = 0; q < 64; ++q)
                if ((qmask >> q) & 1ull) {
                    mp.pos[i] = (int8_t)q;
                    b_of[q] = i++;
                    S = std::max(S, qcount[q]);
                }
            for (int i = 0; i < M; ++i)
                for (int t = 0; t < kMultiStages; ++t) mp.uinv[i][t][0] = mp.uinv[i][t][6] = 1.0;   // identity
            int used[64] = {0};
            std::vector<std::pair<int, int32_t>> comp_param;   // component -> parameter id
            for (int64_t k = j; k > jj && st.ok(); --k) {
                const GateMatrix &gm = mats[(size_t)k];
                const qi_gate &g = resolved[(size_t)k];
                const int b = b_of[gm.t[0]], t = used[gm.t[0]]++;
                inverse_matrix(gm, mp.uinv[b][t]);
                for (int q = 0; q < 3; ++q)
                    if (g.param_ids[q] >= 0) {
                        st = derivative_matrix(n, g, q, mp.d[b][t]);
                        comp_param.push_back({b * S + t, g.param_ids[q]});
                    }
            }
            if (!st.ok()) break;
            mp.nwork = 1ull << (n - M);
            const uint64_t nb64 = (mp.nwork + 255) / 256;
            const unsigned nb = (unsigned)std::max<uint64_t>(
                1, std::min<uint64_t>(nb64, (uint64_t)kReduceBlocks * 4 / kMultiComps));
#define QI_AM(T, MM, SS) k_adjoint_multi<T, MM, SS><<<nb, 256, 0, s->stream>>>( \
                (Cx<T>::V2 *)s->amps, (Cx<T>::V2 *)lam->amps, mp, s->d_partials)
#define QI_AM_S(T, MM) { if (S == 1) QI_AM(T, MM, 1); else QI_AM(T, MM, 2); }
            if (f32) {
                if (M == 1) QI_AM_S(float, 1) else if (M == 2) QI_AM_S(float, 2)
                else if (M == 3) QI_AM_S(float, 3) else QI_AM_S(float, 4)
            } else {
                if (M == 1) QI_AM_S(double, 1) else if (M == 2) QI_AM_S(double, 2) else QI_AM_S(double, 3)
            }
#undef QI_AM_S
#undef QI_AM
            slot -= M * S;
            k_finalize_to<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, M * S, kMultiComps, d_gres + slot);
            count_launch(2);
            st = check_launch("k_adjoint_multi");
            for (auto &cp : comp_param) slot_param.push_back({slot + cp.first, cp.second});
            j = jj;
            continue;
        }
        // fixed gates, consecutive in reverse: their inverses as one fused plan on psi and lambda
        for (jj = j; jj >= 0 && n_params(jj) == 0; --jj) {}
        if (j - jj >= 2 && plan_opts.fusion != QI_FUSION_NONE) {
            std::vector<Elem> inv;
            for (int64_t k = j; k > jj; --k) {
                GateMatrix gi = mats[(size_t)k];
                if (gi.pauli) {
                    gi.alpha_re = -gi.alpha_re;
                    gi.alpha_im = -gi.alpha_im;
                    gi.normalise_after = false;
                } else {
                    if (gi.nt == 0) continue;
                    inverse_matrix(mats[(size_t)k], gi.m);
                }
                inv.push_back(make_elem_from_gate(gi, (int)inv.size()));
            }
            if (inv.empty()) {   // identities only
                j = jj;
                continue;
            }
            std::unique_ptr<qi_plan> seg(new qi_plan());
            seg->n = n;
            seg->prec = s->prec;
            seg->opts = plan_opts;
            seg->opts.renorm_every = -1;   // lambda = H psi is not a unit vector
            st = build_plan(seg.get(), inv);
            if (st.ok()) st = upload_plan(seg.get());
            if (st.ok()) st = plan_execute(seg.get(), s);
            if (st.ok()) st = plan_execute(seg.get(), lam);
            seg_plans.push_back(std::move(seg));
            j = jj;
            continue;
        }
        const GateMatrix &gm = mats[(size_t)j];
        const qi_gate &g = resolved[(size_t)j];
        --j;
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
        k_finalize_to<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, nd, 4, d_gres + slot);
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
    cudaStreamSynchronize(s->stream);
    for (auto &sp : seg_plans) {
        if (sp->d_mats) cudaFree(sp->d_mats);
        if (sp->d_tc) cudaFree(sp->d_tc);
    }
    if (d_gres) cudaFree(d_gres);
    qi_state_destroy(lam);
    return publish(st);
}
