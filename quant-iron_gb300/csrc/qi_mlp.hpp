// qi_mlp.hpp — the cost model's network and its op features.
#pragma once
#include "qi_internal.hpp"

#include <mutex>
#include <vector>

namespace qi {

constexpr int kFeat = 20;   // features per device op (see op_features)
constexpr int kH = 64;      // hidden width (3 hidden layers)
constexpr int kParams = (kFeat * kH + kH) + 2 * (kH * kH + kH) + (kH + 1);
constexpr int kActBufs = 12;

inline int layer_in(int l) { return l == 0 ? kFeat : kH; }
inline int layer_out(int l) { return l == 3 ? 1 : kH; }

struct Mlp {
    std::mutex mu;
    std::vector<float> host;   // flat parameters (host copy)
    bool trained = false;
    float *d_params = nullptr, *d_grads = nullptr, *d_m = nullptr, *d_v = nullptr, *d_loss = nullptr;
    double *d_partials = nullptr;
    float *act[kActBufs] = {nullptr};
    int cap = 0;

    void init_params(uint64_t seed);
    Status ensure_device(int N);
    Status upload_params(cudaStream_t st);
    Status run(int N, bool with_grad, cudaStream_t st);
    Status predict(const float *X, int N, float *out, cudaStream_t st);
};

Mlp &global_mlp();

// Op classes the model distinguishes.
enum CostClass : int { CC_DENSE_TC = 0, CC_DENSE_SIMT = 1, CC_DIAG = 2, CC_PER_GATE = 3 };

// Arithmetic shape of an op (per-gate kernel mode, or block kind).
enum CostShape : int { CS_GENERAL = 0, CS_REAL = 1, CS_DIAGONAL = 2, CS_PERMUTATION = 3 };

// Feature vector of one device op (normalised to O(1)):
//  0 k/6 | 1..6 sorted targets/34 (0 past k) | 7 min target/34 | 8 #targets below qubit 5 / 6
//  9 n/34 | 10 FP32 | 11..14 one-hot class (TC, SIMT, diagonal, per-gate) | 15 controls/8
//  16..19 one-hot shape (general, real, diagonal, permutation) | (touched fraction folded into 15)
inline void op_features(int n, bool f32, int cls, int k, const int *targets, int ncontrols, int shape, float *f) {
    for (int i = 0; i < kFeat; ++i) f[i] = 0.0f;
    f[0] = k / 6.0f;
    int mn = 64, low = 0;
    for (int j = 0; j < k && j < 6; ++j) {
        f[1 + j] = targets[j] / 34.0f;
        mn = targets[j] < mn ? targets[j] : mn;
        low += targets[j] < 5;
    }
    f[7] = (k > 0 ? mn : 0) / 34.0f;
    f[8] = low / 6.0f;
    f[9] = n / 34.0f;
    f[10] = f32 ? 1.0f : 0.0f;
    f[11 + cls] = 1.0f;
    f[15] = ncontrols / 8.0f;
    f[16 + shape] = 1.0f;
}

// Shape of a per-gate op from its kind and 2x2 mode.
inline int per_gate_shape(int op_kind, int mode) {
    if (op_kind == OP_SWAP) return CS_PERMUTATION;
    if (op_kind == OP_MAT1) {
        if (mode == M1_DIAG || mode == M1_PHASE1) return CS_DIAGONAL;
        if (mode == M1_ANTIDIAG) return CS_PERMUTATION;
        if (mode == M1_REAL) return CS_REAL;
    }
    return CS_GENERAL;
}

// Model output y = log(ms per 2^28 amplitudes): ms = exp(y) * 2^(n - 28).
inline double ms_from_y(float y, int n) { return std::exp((double)y) * std::ldexp(1.0, n - 28); }
inline float y_from_ms(double ms, int n) { return (float)std::log(ms / std::ldexp(1.0, n - 28)); }

}  // namespace qi
