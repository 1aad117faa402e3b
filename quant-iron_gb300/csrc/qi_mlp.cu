// qi_mlp.cu — the learned fusion cost model: a small MLP trained on the GPU.
//
// Network: kFeat inputs -> 64 -> 64 -> 64 -> 1, ReLU on the hidden layers,
// mean-squared error on y = log(device time per 2^28 amplitudes, ms).  All
// parameters are one flat FP32 vector (per layer: W [out][in] row-major, then
// b [out]).  Training is full-batch Adam; every kernel sums in a fixed order,
// so a gradient is reproducible bit for bit and can be compared with an FP64
// CPU implementation.
//
// Kernels (hand-written, one thread per output element):
//   k_dense_fwd   Z = X W^T + b, A = relu(Z) (or identity on the last layer)
//   k_mse         dY = 2 (P - Y) / N, per-block loss partials
//   k_dense_bwd_x dX = (dZ) W, then masked by relu'(Z_prev) in k_relu_mask
//   k_dense_bwd_w dW[o][i] = sum_n dZ[n][o] X[n][i], db[o] = sum_n dZ[n][o]
//   k_adam        Adam update of the flat parameter vector
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_mlp.hpp"

#include <cmath>
#include <random>

namespace qi {

__global__ void k_dense_fwd(const float *X, const float *W, const float *b, float *Z, float *A, int N, int in, int out,
                            int relu) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * out) return;
    const int n = idx / out, o = idx % out;
    float acc = b[o];
    const float *x = X + (size_t)n * in;
    const float *w = W + (size_t)o * in;
    for (int i = 0; i < in; ++i) acc = fmaf(w[i], x[i], acc);
    Z[idx] = acc;
    A[idx] = relu ? fmaxf(acc, 0.0f) : acc;
}

__global__ void k_mse(const float *P, const float *Y, float *dP, double *partials, int N) {
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const float d = P[n] - Y[n];
        dP[n] = 2.0f * d / (float)N;
        local += (double)d * (double)d;
    }
    double r = block_sum(local);
    if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

__global__ void k_loss_final(const double *partials, int nb, int N, float *loss) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i];
    double r = block_sum(acc);
    if (threadIdx.x == 0) *loss = (float)(r / N);
}

// dX[n][i] = sum_o dZ[n][o] W[o][i]
__global__ void k_dense_bwd_x(const float *dZ, const float *W, float *dX, int N, int in, int out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * in) return;
    const int n = idx / in, i = idx % in;
    float acc = 0.0f;
    for (int o = 0; o < out; ++o) acc = fmaf(dZ[(size_t)n * out + o], W[(size_t)o * in + i], acc);
    dX[idx] = acc;
}

// dA -> dZ through the ReLU of the previous layer (Z > 0)
__global__ void k_relu_mask(float *d, const float *Z, int count) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < count && Z[idx] <= 0.0f) d[idx] = 0.0f;
}

// dW[o][i] = sum_n dZ[n][o] X[n][i] (i < in), db[o] = sum_n dZ[n][o] (i == in)
__global__ void k_dense_bwd_w(const float *dZ, const float *X, float *dW, float *db, int N, int in, int out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= out * (in + 1)) return;
    const int o = idx / (in + 1), i = idx % (in + 1);
    float acc = 0.0f;
    if (i < in) {
        for (int n = 0; n < N; ++n) acc = fmaf(dZ[(size_t)n * out + o], X[(size_t)n * in + i], acc);
        dW[(size_t)o * in + i] = acc;
    } else {
        for (int n = 0; n < N; ++n) acc += dZ[(size_t)n * out + o];
        db[o] = acc;
    }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int count, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    const float gi = g[idx];
    const float mi = b1 * m[idx] + (1.0f - b1) * gi;
    const float vi = b2 * v[idx] + (1.0f - b2) * gi * gi;
    m[idx] = mi;
    v[idx] = vi;
    p[idx] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ------------------------------------------------------------------ host
static unsigned blocks_for(int count) { return (unsigned)((count + 255) / 256); }

Mlp &global_mlp() {
    static Mlp m;
    return m;
}

Status Mlp::ensure_device(int N) {
    if (!d_params) {
        QI_CUDA(cudaMalloc(&d_params, kParams * sizeof(float)));
        QI_CUDA(cudaMalloc(&d_grads, kParams * sizeof(float)));
        QI_CUDA(cudaMalloc(&d_m, kParams * sizeof(float)));
        QI_CUDA(cudaMalloc(&d_v, kParams * sizeof(float)));
        QI_CUDA(cudaMalloc(&d_loss, sizeof(float)));
        QI_CUDA(cudaMalloc(&d_partials, 1024 * sizeof(double)));
    }
    if (N > cap) {
        for (float *&p : act) if (p) { cudaFree(p); p = nullptr; }
        // buffers: X, Y, P, dP, Z1, A1, Z2, A2, Z3, A3, Z4(P), dA (N x 64) x 2
        const size_t sizes[kActBufs] = {(size_t)N * kFeat, (size_t)N, (size_t)N, (size_t)N,
                                        (size_t)N * kH, (size_t)N * kH, (size_t)N * kH, (size_t)N * kH,
                                        (size_t)N * kH, (size_t)N * kH, (size_t)N * kH, (size_t)N * kH};
        for (int i = 0; i < kActBufs; ++i) QI_CUDA(cudaMalloc(&act[i], sizes[i] * sizeof(float)));
        cap = N;
    }
    return ok_status();
}

void Mlp::init_params(uint64_t seed) {
    std::mt19937_64 rng(seed);
    host.assign(kParams, 0.0f);
    int off = 0;
    for (int l = 0; l < 4; ++l) {
        const int in = layer_in(l), out = layer_out(l);
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / in));   // He initialisation
        for (int i = 0; i < in * out; ++i) host[off + i] = (float)nd(rng);
        off += in * out + out;   // biases start at 0
    }
    trained = false;
}

// Forward (+ loss and backward if Y != nullptr) for N samples already in act[X]/act[Y].
Status Mlp::run(int N, bool with_grad, cudaStream_t st) {
    float *X = act[0], *Y = act[1], *P = act[2], *dP = act[3];
    float *Z[3] = {act[4], act[6], act[8]}, *A[3] = {act[5], act[7], act[9]};
    float *dA = act[10], *dZ = act[11];
    const float *prm = d_params;
    // offsets of each layer's W and b
    int off[4], o = 0;
    for (int l = 0; l < 4; ++l) { off[l] = o; o += layer_in(l) * layer_out(l) + layer_out(l); }
    const float *in_act = X;
    for (int l = 0; l < 3; ++l) {
        const int in = layer_in(l);
        k_dense_fwd<<<blocks_for(N * kH), 256, 0, st>>>(in_act, prm + off[l], prm + off[l] + in * kH, Z[l], A[l], N,
                                                       in, kH, 1);
        in_act = A[l];
    }
    k_dense_fwd<<<blocks_for(N), 256, 0, st>>>(A[2], prm + off[3], prm + off[3] + kH, P, P, N, kH, 1, 0);
    count_launch(4);
    if (!with_grad) return check_launch("mlp forward");
    const unsigned nb = std::min(1024u, blocks_for(N));
    k_mse<<<nb, 256, 0, st>>>(P, Y, dP, d_partials, N);
    k_loss_final<<<1, 256, 0, st>>>(d_partials, (int)nb, N, d_loss);
    count_launch(2);
    // layer 4 (linear): dZ4 = dP
    float *g = d_grads;
    k_dense_bwd_w<<<blocks_for(1 * (kH + 1)), 256, 0, st>>>(dP, A[2], g + off[3], g + off[3] + kH, N, kH, 1);
    k_dense_bwd_x<<<blocks_for(N * kH), 256, 0, st>>>(dP, prm + off[3], dA, N, kH, 1);
    count_launch(2);
    for (int l = 2; l >= 0; --l) {
        const int in = layer_in(l);
        // dZ_l = dA_l * relu'(Z_l)
        cudaMemcpyAsync(dZ, dA, (size_t)N * kH * sizeof(float), cudaMemcpyDeviceToDevice, st);
        k_relu_mask<<<blocks_for(N * kH), 256, 0, st>>>(dZ, Z[l], N * kH);
        const float *xin = l == 0 ? X : A[l - 1];
        k_dense_bwd_w<<<blocks_for(kH * (in + 1)), 256, 0, st>>>(dZ, xin, g + off[l], g + off[l] + in * kH, N, in, kH);
        count_launch(2);
        if (l > 0) {
            k_dense_bwd_x<<<blocks_for(N * in), 256, 0, st>>>(dZ, prm + off[l], dA, N, in, kH);
            count_launch();
        }
    }
    return check_launch("mlp backward");
}

Status Mlp::upload_params(cudaStream_t st) {
    QI_CUDA(cudaMemcpyAsync(d_params, host.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, st));
    return ok_status();
}

Status Mlp::predict(const float *X, int N, float *out, cudaStream_t st) {
    Status s = ensure_device(N);
    if (!s.ok()) return s;
    QI_CUDA(cudaMemcpyAsync(act[0], X, (size_t)N * kFeat * sizeof(float), cudaMemcpyHostToDevice, st));
    s = run(N, false, st);
    if (!s.ok()) return s;
    QI_CUDA(cudaMemcpyAsync(out, act[2], (size_t)N * sizeof(float), cudaMemcpyDeviceToHost, st));
    QI_CUDA(cudaStreamSynchronize(st));
    return ok_status();
}

}  // namespace qi

using namespace qi;

extern "C" {

qi_status qi_costmodel_init(uint64_t seed) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    m.init_params(seed);
    return publish(ok_status());
}

qi_status qi_costmodel_num_params(int64_t *out) {
    if (!out) return publish(err(QI_ERR_NULL_ARGUMENT));
    *out = kParams;
    return publish(ok_status());
}

qi_status qi_costmodel_get_params(float *out, int64_t capacity, int32_t *trained) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!out || capacity < kParams) return publish(err(QI_ERR_INVALID_INPUT_VALUE, capacity, kParams));
    if (m.host.empty()) m.init_params(0);
    std::copy(m.host.begin(), m.host.end(), out);
    if (trained) *trained = m.trained ? 1 : 0;
    return publish(ok_status());
}

qi_status qi_costmodel_set_params(const float *in, int64_t count, int32_t trained) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!in || count != kParams) return publish(err(QI_ERR_INVALID_INPUT_VALUE, count, kParams));
    m.host.assign(in, in + kParams);
    m.trained = trained != 0;
    return publish(ok_status());
}

qi_status qi_costmodel_loss_and_gradient(const float *X, const float *Y, int64_t n, float *loss_out, float *grad_out) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!X || !Y || !loss_out || !grad_out || n <= 0) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (m.host.empty()) m.init_params(0);
    cudaStream_t st = nullptr;
    Status s = m.ensure_device((int)n);
    if (s.ok()) s = m.upload_params(st);
    if (!s.ok()) return publish(s);
    cudaError_t e = cudaMemcpyAsync(m.act[0], X, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m.act[1], Y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return publish(cuda_status(e, "costmodel"));
    s = m.run((int)n, true, st);
    if (!s.ok()) return publish(s);
    e = cudaMemcpyAsync(loss_out, m.d_loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad_out, m.d_grads, kParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return publish(cuda_status(e, "costmodel"));
    return publish(ok_status());
}

qi_status qi_costmodel_train(const float *X, const float *Y, int64_t n, int32_t epochs, float lr, uint64_t seed,
                             float *loss_history) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!X || !Y || n <= 0 || epochs <= 0) return publish(err(QI_ERR_NULL_ARGUMENT));
    m.init_params(seed);
    cudaStream_t st = nullptr;
    Status s = m.ensure_device((int)n);
    if (s.ok()) s = m.upload_params(st);
    if (!s.ok()) return publish(s);
    cudaError_t e = cudaMemcpyAsync(m.act[0], X, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m.act[1], Y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(m.d_m, 0, kParams * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(m.d_v, 0, kParams * sizeof(float), st);
    if (e != cudaSuccess) return publish(cuda_status(e, "costmodel train"));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        s = m.run((int)n, true, st);
        if (!s.ok()) return publish(s);
        const float c1 = 1.0f - std::pow(b1, (float)(ep + 1)), c2 = 1.0f - std::pow(b2, (float)(ep + 1));
        k_adam<<<blocks_for(kParams), 256, 0, st>>>(m.d_params, m.d_grads, m.d_m, m.d_v, kParams, lr, b1, b2, eps, c1, c2);
        count_launch();
        if (loss_history) {
            e = cudaMemcpyAsync(loss_history + ep, m.d_loss, sizeof(float), cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) return publish(cuda_status(e, "costmodel train"));
        }
    }
    e = cudaMemcpyAsync(m.host.data(), m.d_params, kParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return publish(cuda_status(e, "costmodel train"));
    m.trained = true;
    return publish(ok_status());
}

qi_status qi_costmodel_predict(const float *X, int64_t n, float *y_out) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!X || !y_out || n <= 0) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (m.host.empty()) m.init_params(0);
    Status s = m.ensure_device((int)n);
    if (s.ok()) s = m.upload_params(nullptr);
    if (s.ok()) s = m.predict(X, (int)n, y_out, nullptr);
    return publish(s);
}

}  // extern "C"
