// qi_measure.cu — State::measure / measure_n on the device.
//
// Reference: src/components/state.rs:525-784.  Probabilities of the measured
// qubits are summed in FP64 on the device in a fixed order (FP32 states: FP32
// sums of 8 |a|^2, each folded into the FP64 sum; one block per
// (outcome, chunk), then one ordered sum per outcome), copied to the host,
// normalised and sampled exactly as the reference does (sequential CDF in
// outcome order, `r < cumulative`, last outcome on fall-through).  The
// reference draws r from an unseeded rand::rng() (state.rs:601); here r comes
// from splitmix64 of a caller seed, so outcomes are reproducible and
// bit-identical to the oracle for the same r.  The outcome index arithmetic
// (bit k of the outcome = qubit qubits[k]) is integer and exact.
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace qi {

// Distinct measured qubits, sorted (duplicates in the caller's list must agree).
struct MeasGeom {
    int32_t nd;              // distinct measured qubits
    int8_t pos[64];          // ascending
    uint64_t dmask;
};

// P[d] partials: block b covers outcome d = b / chunks, chunk b % chunks of the
// 2^(n - nd) amplitudes that share those measured bits.
template <typename T>
__global__ void __launch_bounds__(256) k_meas_partial(const typename Cx<T>::V2 *a, MeasGeom g, uint64_t rest_count,
                                                      uint64_t chunk, uint64_t chunks, double *partials) {
    const uint64_t b = blockIdx.x + (uint64_t)blockIdx.y * gridDim.x;
    const uint64_t d = b / chunks, c = b % chunks;
    // deposit d into the measured positions
    uint64_t fixed = 0;
    for (int k = 0; k < g.nd; ++k) fixed |= ((d >> k) & 1ull) << g.pos[k];
    double acc = 0.0;
    const uint64_t lo = c * chunk, hi = min(rest_count, lo + chunk);
    if constexpr (sizeof(T) == 4) {
        // FP32 |a|^2 summed over 8 amplitudes, folded into FP64 once per outer step
        // (per-element FP64 arithmetic would bound this kernel on this part)
        for (uint64_t w0 = lo + threadIdx.x; w0 < hi; w0 += 8 * (uint64_t)blockDim.x) {
            float part = 0.0f;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint64_t w = w0 + (uint64_t)u * blockDim.x;
                if (w < hi) {
                    const float2 v = a[insert_zeros(w, g.pos, g.nd) | fixed];
                    part += fmaf(v.x, v.x, v.y * v.y);
                }
            }
            acc += (double)part;
        }
    } else {
        for (uint64_t w = lo + threadIdx.x; w < hi; w += blockDim.x) {
            const uint64_t i = insert_zeros(w, g.pos, g.nd) | fixed;
            const typename Cx<T>::V2 v = a[i];
            acc += v.x * v.x + v.y * v.y;
        }
    }
    const double r = block_sum(acc);
    if (threadIdx.x == 0) partials[b] = r;
}

__global__ void k_meas_reduce(const double *partials, uint64_t chunks, uint64_t outcomes, double *P) {
    const uint64_t d = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (d >= outcomes) return;
    double acc = 0.0;
    for (uint64_t c = 0; c < chunks; ++c) acc += partials[d * chunks + c];
    P[d] = acc;
}

// Zero every amplitude whose measured bits differ from `want` (state.rs:622-654).
template <typename T>
__global__ void __launch_bounds__(256) k_collapse(typename Cx<T>::V2 *a, uint64_t dim, uint64_t dmask, uint64_t want) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x)
        if ((i & dmask) != want) a[i] = Cx<T>::make(0, 0);
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static double uniform01(uint64_t seed) { return (double)(splitmix64(seed) >> 11) * 0x1.0p-53; }

static Status apply_named(qi_state *s, int kind, int q, const double *m8) {
    qi_gate g;
    std::memset(&g, 0, sizeof(g));
    g.kind = kind;
    g.n_targets = 1;
    g.targets[0] = q;
    g.param_ids[0] = g.param_ids[1] = g.param_ids[2] = -1;
    if (m8) for (int j = 0; j < 8; ++j) g.params[j] = m8[j];
    GateMatrix gm;
    Status st = gate_to_matrix(s->n, g, &gm);
    if (!st.ok()) return st;
    return launch_op(s, lower_gate(s->n, gm), nullptr);
}

// Basis change before (dir = 0) or after (dir = 1) the computational measurement.
static Status basis_change(qi_state *s, int basis, const double *u, const int32_t *q, int m, int dir) {
    Status st = ok_status();
    double ud[8];
    if (basis == QI_BASIS_CUSTOM) {   // calculate_adjoint (state.rs:17-22)
        ud[0] = u[0]; ud[1] = -u[1]; ud[2] = u[4]; ud[3] = -u[5];
        ud[4] = u[2]; ud[5] = -u[3]; ud[6] = u[6]; ud[7] = -u[7];
    }
    auto each = [&](int kind, const double *mm) {
        for (int k = 0; k < m && st.ok(); ++k) st = apply_named(s, kind, q[k], mm);
    };
    if (basis == QI_BASIS_X) each(QI_GATE_H, nullptr);
    else if (basis == QI_BASIS_Y) {
        if (dir == 0) { each(QI_GATE_SDAG, nullptr); each(QI_GATE_H, nullptr); }
        else { each(QI_GATE_H, nullptr); each(QI_GATE_S, nullptr); }
    } else if (basis == QI_BASIS_CUSTOM) {
        each(QI_GATE_U2, dir == 0 ? u : ud);
    }
    return st;
}

// Normalised outcome probabilities (host, outcome order) for the caller's qubit list.
static Status outcome_probs(qi_state *s, const int32_t *q, int m, std::vector<double> &prob, double *total_out) {
    const int n = s->n;
    MeasGeom g;
    std::memset(&g, 0, sizeof(g));
    uint64_t dmask = 0;
    for (int k = 0; k < m; ++k) dmask |= 1ull << q[k];
    for (int b = 0; b < 64; ++b)
        if ((dmask >> b) & 1ull) g.pos[g.nd++] = (int8_t)b;
    g.dmask = dmask;
    const uint64_t outcomes = 1ull << g.nd, rest = 1ull << (n - g.nd);
    const uint64_t chunk = std::min<uint64_t>(rest, 8192);
    const uint64_t chunks = (rest + chunk - 1) / chunk;
    const uint64_t nblocks = outcomes * chunks;
    double *d_part = nullptr, *d_P = nullptr;
    QI_CUDA(cudaMallocAsync((void **)&d_part, nblocks * sizeof(double), s->stream));
    QI_CUDA(cudaMallocAsync((void **)&d_P, outcomes * sizeof(double), s->stream));
    const unsigned gx = (unsigned)std::min<uint64_t>(nblocks, 65535);
    const unsigned gy = (unsigned)((nblocks + gx - 1) / gx);
    // grid is gx * gy >= nblocks; surplus blocks map past the last outcome, so size the grid exactly
    if ((uint64_t)gx * gy != nblocks) {
        // nblocks is a product of powers of two, so gx = 65535 only when nblocks > 65535: use 32768 columns
        const unsigned gx2 = 32768, gy2 = (unsigned)(nblocks / gx2);
        if ((uint64_t)gx2 * gy2 != nblocks) return err(QI_ERR_UNKNOWN, (int64_t)nblocks, -1, "measure grid");
        if (s->prec == QI_F32)
            k_meas_partial<float><<<dim3(gx2, gy2), 256, 0, s->stream>>>((const float2 *)s->amps, g, rest, chunk, chunks, d_part);
        else
            k_meas_partial<double><<<dim3(gx2, gy2), 256, 0, s->stream>>>((const double2 *)s->amps, g, rest, chunk, chunks, d_part);
    } else {
        if (s->prec == QI_F32)
            k_meas_partial<float><<<dim3(gx, gy), 256, 0, s->stream>>>((const float2 *)s->amps, g, rest, chunk, chunks, d_part);
        else
            k_meas_partial<double><<<dim3(gx, gy), 256, 0, s->stream>>>((const double2 *)s->amps, g, rest, chunk, chunks, d_part);
    }
    k_meas_reduce<<<(unsigned)((outcomes + 255) / 256), 256, 0, s->stream>>>(d_part, chunks, outcomes, d_P);
    count_launch(2);
    Status st = check_launch("k_meas_partial");
    if (!st.ok()) return st;
    std::vector<double> P(outcomes);
    QI_CUDA(cudaMemcpyAsync(P.data(), d_P, outcomes * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    QI_CUDA(cudaFreeAsync(d_part, s->stream));
    QI_CUDA(cudaFreeAsync(d_P, s->stream));
    QI_CUDA(cudaStreamSynchronize(s->stream));
    // map to the caller's outcome integers (bit k = qubit q[k]); duplicated qubits must agree
    const uint64_t no = 1ull << m;
    prob.assign(no, 0.0);
    for (uint64_t o = 0; o < no; ++o) {
        uint64_t d = 0;
        bool ok = true;
        uint64_t seen = 0, val = 0;
        for (int k = 0; k < m; ++k) {
            const uint64_t bit = (o >> k) & 1ull, qb = 1ull << q[k];
            if (seen & qb) { if (((val & qb) != 0) != (bit != 0)) { ok = false; break; } }
            seen |= qb;
            if (bit) val |= qb;
        }
        if (!ok) continue;
        for (int k = 0; k < g.nd; ++k) if ((val >> g.pos[k]) & 1ull) d |= 1ull << k;
        prob[o] = P[d];
    }
    double total = 0.0;
    for (double x : prob) total += x;   // probabilities.iter().sum()
    *total_out = total;
    return ok_status();
}

static Status check_measured(int n, const int32_t *q, int m) {
    if (m > n) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, n);
    for (int k = 0; k < m; ++k)
        if (q[k] < 0 || q[k] >= n) return err(QI_ERR_INVALID_QUBIT_INDEX, q[k], n);
    if (m > 24) return err(QI_ERR_UNSUPPORTED, m, 24, "measuring more than 24 qubits");
    return ok_status();
}

static uint64_t sample(const std::vector<double> &prob, double r) {   // state.rs:604-619
    double cum = 0.0;
    for (size_t i = 0; i < prob.size(); ++i) {
        cum += prob[i];
        if (r < cum) return i;
    }
    return prob.size() - 1;
}

Status measure_state(qi_state *s, int basis, const double *custom_u, const int32_t *qubits, int n_qubits,
                     uint64_t seed, uint64_t *outcome_out, double *probs_out) {
    std::vector<int32_t> all;
    if (n_qubits == 0) { for (int q = 0; q < s->n; ++q) all.push_back(q); qubits = all.data(); n_qubits = s->n; }
    Status st = check_measured(s->n, qubits, n_qubits);
    if (!st.ok()) return st;
    st = basis_change(s, basis, custom_u, qubits, n_qubits, 0);
    std::vector<double> prob;
    double total = 0.0;
    if (st.ok()) st = outcome_probs(s, qubits, n_qubits, prob, &total);
    if (st.ok() && total < 2.220446049250313e-16) st = err(QI_ERR_UNKNOWN, -1, -1, "total probability below f64::EPSILON");
    if (!st.ok()) {
        basis_change(s, basis, custom_u, qubits, n_qubits, 1);   // leave the state as it was
        return st;
    }
    for (double &x : prob) x = x / total;
    const uint64_t o = sample(prob, uniform01(seed));
    if (prob[o] * total <= 2.220446049250313e-16) {   // the collapsed state would not be normalisable
        basis_change(s, basis, custom_u, qubits, n_qubits, 1);
        return err(QI_ERR_STATE_NOT_NORMALISED);
    }
    // required measured bits for outcome o
    uint64_t dmask = 0, want = 0;
    for (int k = 0; k < n_qubits; ++k) {
        dmask |= 1ull << qubits[k];
        if ((o >> k) & 1ull) want |= 1ull << qubits[k];
    }
    uint64_t gsz = std::min<uint64_t>((s->dim() + 255) / 256, 152 * 8);
    if (s->prec == QI_F32) k_collapse<float><<<(unsigned)gsz, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), dmask, want);
    else k_collapse<double><<<(unsigned)gsz, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), dmask, want);
    count_launch();
    st = check_launch("k_collapse");
    if (st.ok()) st = state_normalise_device_async(s);
    if (st.ok()) st = basis_change(s, basis, custom_u, qubits, n_qubits, 1);
    if (st.ok()) {
        int flag = 0;
        st = state_read_flag(s, &flag);
    }
    if (!st.ok()) return st;
    *outcome_out = o;
    if (probs_out) std::copy(prob.begin(), prob.end(), probs_out);
    return ok_status();
}

}  // namespace qi

using namespace qi;

extern "C" {

qi_status qi_measure(qi_state *s, int32_t basis, const double *custom_u, const int32_t *qubits, int32_t n_qubits,
                     uint64_t seed, uint64_t *outcome_out, double *probs_out) {
    if (!s || !outcome_out || (n_qubits > 0 && !qubits)) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (basis < 0 || basis > 3 || (basis == QI_BASIS_CUSTOM && !custom_u))
        return publish(err(QI_ERR_INVALID_INPUT_VALUE, basis));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    return publish(measure_state(s, basis, custom_u, qubits, n_qubits, seed, outcome_out, probs_out));
}

qi_status qi_measure_n(qi_state *s, int32_t basis, const double *custom_u, const int32_t *qubits, int32_t n_qubits,
                       int64_t n_shots, uint64_t seed, uint64_t *outcomes_out) {
    if (!s || (n_shots > 0 && !outcomes_out) || (n_qubits > 0 && !qubits)) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (n_shots <= 0) return publish(err(QI_ERR_INVALID_NUMBER_OF_MEASUREMENTS, 0));   // state.rs:756-758
    if (basis < 0 || basis > 3 || (basis == QI_BASIS_CUSTOM && !custom_u))
        return publish(err(QI_ERR_INVALID_INPUT_VALUE, basis));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    std::vector<int32_t> all;
    if (n_qubits == 0) { for (int q = 0; q < s->n; ++q) all.push_back(q); qubits = all.data(); n_qubits = s->n; }
    Status st = check_measured(s->n, qubits, n_qubits);
    if (!st.ok()) return publish(st);
    st = basis_change(s, basis, custom_u, qubits, n_qubits, 0);
    std::vector<double> prob;
    double total = 0.0;
    if (st.ok()) st = outcome_probs(s, qubits, n_qubits, prob, &total);
    // undo the basis change: the state is left as it was
    Status st2 = basis_change(s, basis, custom_u, qubits, n_qubits, 1);
    if (!st.ok()) return publish(st);
    if (!st2.ok()) return publish(st2);
    if (total < 2.220446049250313e-16) return publish(err(QI_ERR_UNKNOWN, -1, -1, "total probability below f64::EPSILON"));
    for (double &x : prob) x = x / total;
    // CDF once, binary search per shot (same result as the sequential scan)
    std::vector<double> cdf(prob.size());
    double cum = 0.0;
    for (size_t i = 0; i < prob.size(); ++i) { cum += prob[i]; cdf[i] = cum; }
    for (int64_t j = 0; j < n_shots; ++j) {
        const double r = uniform01(seed + (uint64_t)j);
        const size_t i = (size_t)(std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin());
        outcomes_out[j] = i < cdf.size() ? i : cdf.size() - 1;
    }
    return publish(ok_status());
}

}  // extern "C"
