// qi_core.cu — state handles, host<->device transfer, constructors, state
// arithmetic and FP64-accumulated reductions.
//
// Reference: src/components/state.rs (State, constructors :99-373,
// inner_product :890-917, normalise :924-945, tensor_product :801-836,
// arithmetic :2687-2862) and the device round trip of execute_on_gpu
// (src/components/operator.rs:24-148), which this file replaces with a
// resident device state.
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <cmath>
#include <cstdio>

namespace qi {

std::atomic<uint64_t> g_launches{0};
static thread_local qi_error_info t_last = {QI_OK, 0, -1, -1, 0.0, 0.0, {0}};
static int g_device = 0;

qi_status publish(const Status &s) {
    t_last.code = s.code;
    t_last.a = s.a;
    t_last.b = s.b;
    t_last.re = s.re;
    t_last.im = s.im;
    std::snprintf(t_last.message, sizeof(t_last.message), "%s", s.msg.c_str());
    return s.code;
}

Status cuda_status(cudaError_t e, const char *what) {
    qi_status code = (e == cudaErrorMemoryAllocation) ? QI_ERR_OUT_OF_MEMORY : QI_ERR_DEVICE;
    char buf[200];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return err(code, (int64_t)e, -1, buf);
}

Status check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, what);
    return ok_status();
}

// ---------------------------------------------------------------- kernels --
template <typename T>
__global__ void k_fill_const(typename Cx<T>::V2 *a, uint64_t dim, T re, T im) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = Cx<T>::make(re, im);
}

// State::new_minus (state.rs:252-290): +amp for even popcount, -amp for odd.
template <typename T>
__global__ void k_fill_minus(typename Cx<T>::V2 *a, uint64_t dim, T amp) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = Cx<T>::make((__popcll(i) & 1) ? -amp : amp, T(0));
}

template <typename TO, typename TI>
__global__ void k_convert(typename Cx<TO>::V2 *o, const typename Cx<TI>::V2 *in, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        typename Cx<TI>::V2 v = in[i];
        o[i] = Cx<TO>::make((TO)v.x, (TO)v.y);
    }
}

// The same conversion for a buffer on the other side of the CPU-GPU link (mapped,
// page-locked host memory): four independent 16-byte accesses in flight per
// thread to cover the link's latency.  At most 32 registers a thread, so a block
// fits on an SM beside a tensor-core block (448 threads x 128 registers).
template <typename TO, typename TI>
__global__ void __launch_bounds__(256, 8) k_convert_link(typename Cx<TO>::V2 *o, const typename Cx<TI>::V2 *in,
                                                         uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        typename Cx<TI>::V2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i0 + u * stride < n) v[u] = in[i0 + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i0 + u * stride < n) o[i0 + u * stride] = Cx<TO>::make((TO)v[u].x, (TO)v[u].y);
    }
}

template <typename T>
__global__ void k_scale(typename Cx<T>::V2 *a, uint64_t dim, T re, T im) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        typename Cx<T>::V2 v = a[i];
        a[i] = Cx<T>::mul(v, Cx<T>::make(re, im));
    }
}

template <typename T>
__global__ void k_axpy(typename Cx<T>::V2 *y, const typename Cx<T>::V2 *x, uint64_t dim, T re, T im) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        typename Cx<T>::V2 yv = y[i], xv = x[i];
        y[i] = Cx<T>::add(yv, Cx<T>::mul(Cx<T>::make(re, im), xv));
    }
}

// State::tensor_product (state.rs:801-836): out[k] = a[k >> nb] * b[k & (2^nb - 1)].
template <typename T>
__global__ void k_tensor(typename Cx<T>::V2 *o, const typename Cx<T>::V2 *a, const typename Cx<T>::V2 *b,
                         uint64_t dim, int nb) {
    const uint64_t mb = (1ull << nb) - 1;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < dim; k += (uint64_t)gridDim.x * blockDim.x)
        o[k] = Cx<T>::mul(a[k >> nb], b[k & mb]);
}

// --- reductions: per-thread FP64 accumulators, fixed-order two-pass sum ----
// Sum of |a|^2.  FP32 states: |a|^2 of two amplitudes is summed in FP32 (four
// products, relative error <= 2^-22) and accumulated in FP64.
template <typename T>
__global__ void k_norm_partial(const typename Cx<T>::V2 *a, uint64_t dim, double *partials) {
    double acc = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if constexpr (sizeof(T) == 4) {
        const float4 *a4 = reinterpret_cast<const float4 *>(a);
        const uint64_t n4 = dim >> 1;
        // FP32 sums of 8 float4 (16 amplitudes) folded into FP64 once per outer step: a
        // conversion and an FP64 add per float4 (or a fold the compiler if-converts into
        // every iteration) make this kernel FP64-bound on this part
        for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n4; i0 += 8 * stride) {
            float4 v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                v[u] = i0 + u * stride < n4 ? ldg_stream(a4 + i0 + u * stride) : make_float4(0.f, 0.f, 0.f, 0.f);
            float part = 0.0f;
#pragma unroll
            for (int u = 0; u < 8; ++u) part += fmaf(v[u].x, v[u].x, fmaf(v[u].y, v[u].y, fmaf(v[u].z, v[u].z, v[u].w * v[u].w)));
            acc += (double)part;
        }
        if ((dim & 1) && blockIdx.x == 0 && threadIdx.x == 0) {   // dim == 1 only when n == 0
            float2 v = reinterpret_cast<const float2 *>(a)[dim - 1];
            acc += (double)v.x * v.x + (double)v.y * v.y;
        }
    } else {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
            double2 v = ldg_stream(reinterpret_cast<const double2 *>(a) + i);
            acc += v.x * v.x + v.y * v.y;
        }
    }
    double r = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x * 4] = r;
}

// <a|b> = sum conj(a_i) b_i (state.rs:890-917).
template <typename T>
__global__ void k_inner_partial(const typename Cx<T>::V2 *a, const typename Cx<T>::V2 *b, uint64_t dim,
                                double *partials) {
    double re = 0.0, im = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if constexpr (sizeof(T) == 4) {
        const float4 *a4 = reinterpret_cast<const float4 *>(a);
        const float4 *b4 = reinterpret_cast<const float4 *>(b);
        const uint64_t n4 = dim >> 1;
        // FP32 sums of 4 float4 pairs (8 amplitudes) folded into FP64 once per outer step
        for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n4; i0 += 4 * stride) {
            float4 x[4], y[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool in = i0 + u * stride < n4;
                x[u] = in ? ldg_stream(a4 + i0 + u * stride) : make_float4(0.f, 0.f, 0.f, 0.f);
                y[u] = in ? ldg_stream(b4 + i0 + u * stride) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            float r = 0.0f, m = 0.0f;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                r += fmaf(x[u].x, y[u].x, fmaf(x[u].y, y[u].y, fmaf(x[u].z, y[u].z, x[u].w * y[u].w)));
                m += fmaf(x[u].x, y[u].y, fmaf(-x[u].y, y[u].x, fmaf(x[u].z, y[u].w, -x[u].w * y[u].z)));
            }
            re += (double)r;
            im += (double)m;
        }
    } else {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
            double2 x = ldg_stream(reinterpret_cast<const double2 *>(a) + i);
            double2 y = ldg_stream(reinterpret_cast<const double2 *>(b) + i);
            re += x.x * y.x + x.y * y.y;
            im += x.x * y.y - x.y * y.x;
        }
    }
    double r0 = block_sum(re);
    double r1 = block_sum(im);
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = r0;
        partials[blockIdx.x * 4 + 1] = r1;
    }
}

// Comparison of two states of any precisions (a verification tool, FP64 throughout): per
// block [max |a_i - b_i|^2, sum |a_i - b_i|^2, Re <b|a>, Im <b|a>].
template <typename TA, typename TB>
__global__ void k_compare_partial(const typename Cx<TA>::V2 *a, const typename Cx<TB>::V2 *b, uint64_t dim,
                                  double *partials) {
    double mx = 0.0, d2 = 0.0, re = 0.0, im = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        const typename Cx<TA>::V2 x = ldg_stream(a + i);
        const typename Cx<TB>::V2 y = ldg_stream(b + i);
        const double xr = (double)x.x, xi = (double)x.y, yr = (double)y.x, yi = (double)y.y;
        const double dr = xr - yr, di = xi - yi, m = dr * dr + di * di;
        mx = fmax(mx, m);
        d2 += m;
        re += yr * xr + yi * xi;
        im += yr * xi - yi * xr;
    }
    __shared__ double wmax[32];
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < ((blockDim.x + 31) >> 5) ? wmax[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    const double s0 = block_sum(d2), s1 = block_sum(re), s2 = block_sum(im);
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = mx;
        partials[blockIdx.x * 4 + 1] = s0;
        partials[blockIdx.x * 4 + 2] = s1;
        partials[blockIdx.x * 4 + 3] = s2;
    }
}

// Final reduction of k_compare_partial's slots: component 0 by maximum, 1..3 by fixed-order sums.
__global__ void k_compare_finalize(const double *partials, int nb, double *result) {
    __shared__ double wmax[32];
    double mx = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) mx = fmax(mx, partials[i * 4]);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < ((blockDim.x + 31) >> 5) ? wmax[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        if (threadIdx.x == 0) result[0] = mx;
    }
    for (int c = 1; c < 4; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i * 4 + c];
        const double r = block_sum(acc);
        if (threadIdx.x == 0) result[c] = r;
        __syncthreads();
    }
}

// Fixed-order final sum of `nb` partial slots (ncomp components each).
__global__ void k_finalize(const double *partials, int nb, int ncomp, double *result) {
    for (int c = 0; c < ncomp; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partials[i * 4 + c];
        double r = block_sum(acc);
        if (threadIdx.x == 0) result[c] = r;
        __syncthreads();
    }
}

// normalise on device (state.rs:924-945): result[0] holds sum |a|^2.
// norm == 0 -> flag ZeroNorm (state untouched); norm == 1 -> untouched.
template <typename T>
__global__ void k_normalise_apply(typename Cx<T>::V2 *a, uint64_t dim, const double *result, int *flag) {
    // one thread per block takes the FP64 square root and reciprocal (tens of FP64
    // operations; FP64 is the GB300's slowest pipe)
    __shared__ T s_inv;
    __shared__ int s_scale;
    if (threadIdx.x == 0) {
        const double norm = sqrt(result[0]);
        if (norm == 0.0 && blockIdx.x == 0) *flag = 1;
        s_scale = norm != 0.0 && norm != 1.0;
        s_inv = (T)(1.0 / norm);
    }
    __syncthreads();
    if (!s_scale) return;
    const T inv = s_inv;
    constexpr int U = 4;
    const uint64_t step = blockDim.x, stride = (uint64_t)gridDim.x * blockDim.x * U;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x * U + threadIdx.x; base < dim; base += stride) {
        typename Cx<T>::V2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < dim) v[u] = a[base + u * step];
        // multiply by the reciprocal (within 1 ulp of x / norm)
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < dim) a[base + u * step] = Cx<T>::make(v[u].x * inv, v[u].y * inv);
    }
}

// out = in / norm for a permuted copy moving back to the state's own buffer: always writes
// (a norm of 0 or 1 copies unchanged; 0 also flags ZeroNorm).
template <typename T>
__global__ void k_normalise_to(typename Cx<T>::V2 *__restrict__ out, const typename Cx<T>::V2 *__restrict__ in,
                               uint64_t dim, const double *result, int *flag) {
    __shared__ T s_inv;
    if (threadIdx.x == 0) {
        const double norm = sqrt(result[0]);
        if (norm == 0.0 && blockIdx.x == 0) *flag = 1;
        s_inv = (T)(norm != 0.0 && norm != 1.0 ? 1.0 / norm : 1.0);
    }
    __syncthreads();
    const T inv = s_inv;
    constexpr int U = 4;
    const uint64_t step = blockDim.x, stride = (uint64_t)gridDim.x * blockDim.x * U;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x * U + threadIdx.x; base < dim; base += stride) {
        typename Cx<T>::V2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < dim) v[u] = in[base + u * step];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < dim) out[base + u * step] = Cx<T>::make(v[u].x * inv, v[u].y * inv);
    }
}

// ---------------------------------------------------------------- helpers --
static unsigned grid_for(uint64_t work, unsigned threads = 256, unsigned cap = 152 * 16) {
    uint64_t g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

static Status ensure_device(const qi_state *s) {
    QI_CUDA(cudaSetDevice(s->device));
    return ok_status();
}

static unsigned reduce_grid(uint64_t work) {
    uint64_t g = (work + kReduceThreads - 1) / kReduceThreads;
    if (g < 1) g = 1;
    if (g > (uint64_t)kReduceBlocks) g = kReduceBlocks;
    return (unsigned)g;
}

static Status finish_reduce(qi_state *s, unsigned nb, int ncomp, double *out) {
    k_finalize<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, ncomp, s->d_result);
    count_launch();
    Status st = check_launch("k_finalize");
    if (!st.ok()) return st;
    QI_CUDA(cudaMemcpyAsync(s->h_result, s->d_result, ncomp * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    QI_CUDA(cudaStreamSynchronize(s->stream));
    for (int c = 0; c < ncomp; ++c) out[c] = s->h_result[c];
    return ok_status();
}

// Norm^2 reduction into d_result[0] (asynchronous).
static Status norm_async(qi_state *s, unsigned *nb_out) {
    const uint64_t work = s->prec == QI_F32 ? (s->dim() >> 1) : s->dim();
    unsigned nb = reduce_grid(work);
    if (s->prec == QI_F32)
        k_norm_partial<float><<<nb, kReduceThreads, 0, s->stream>>>((const float2 *)s->amps, s->dim(), s->d_partials);
    else
        k_norm_partial<double><<<nb, kReduceThreads, 0, s->stream>>>((const double2 *)s->amps, s->dim(), s->d_partials);
    count_launch();
    *nb_out = nb;
    return check_launch("k_norm_partial");
}

Status state_reduce_norm_sqr(qi_state *s, double *out) {
    unsigned nb;
    Status st = norm_async(s, &nb);
    if (!st.ok()) return st;
    return finish_reduce(s, nb, 1, out);
}

Status state_inner(qi_state *a, qi_state *b, double out[2]) {
    const uint64_t work = a->prec == QI_F32 ? (a->dim() >> 1) : a->dim();
    unsigned nb = reduce_grid(work);
    if (b->stream != a->stream) {
        // order b's pending work before the reduction on a's stream
        cudaEvent_t ev;
        QI_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        QI_CUDA(cudaEventRecord(ev, b->stream));
        QI_CUDA(cudaStreamWaitEvent(a->stream, ev, 0));
        QI_CUDA(cudaEventDestroy(ev));
    }
    if (a->prec == QI_F32)
        k_inner_partial<float><<<nb, kReduceThreads, 0, a->stream>>>((const float2 *)a->amps, (const float2 *)b->amps,
                                                                    a->dim(), a->d_partials);
    else
        k_inner_partial<double><<<nb, kReduceThreads, 0, a->stream>>>((const double2 *)a->amps, (const double2 *)b->amps,
                                                                     a->dim(), a->d_partials);
    count_launch();
    Status st = check_launch("k_inner_partial");
    if (!st.ok()) return st;
    return finish_reduce(a, nb, 2, out);
}

Status state_scale_async(qi_state *s, double re, double im) {
    unsigned g = grid_for(s->dim());
    if (s->prec == QI_F32) k_scale<float><<<g, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), (float)re, (float)im);
    else k_scale<double><<<g, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), re, im);
    count_launch();
    return check_launch("k_scale");
}

Status state_normalise_device_async(qi_state *s) {
    unsigned nb;
    Status st = norm_async(s, &nb);
    if (!st.ok()) return st;
    k_finalize<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, 1, s->d_result);
    count_launch();
    unsigned g = grid_for(s->dim());
    if (s->prec == QI_F32)
        k_normalise_apply<float><<<g, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), s->d_result, s->d_flag);
    else
        k_normalise_apply<double><<<g, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), s->d_result, s->d_flag);
    count_launch();
    return check_launch("k_normalise_apply");
}

Status state_normalise_device_to_async(qi_state *s, void *out, const void *in) {
    unsigned nb;
    void *const home = s->amps;
    s->amps = const_cast<void *>(in);   // the norm of `in`
    Status st = norm_async(s, &nb);
    s->amps = home;
    if (!st.ok()) return st;
    return state_normalise_to_from_partials_async(s, out, in, nb);
}

Status state_normalise_to_from_partials_async(qi_state *s, void *out, const void *in, unsigned nb) {
    k_finalize<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, 1, s->d_result);
    count_launch();
    unsigned g = grid_for(s->dim());
    if (s->prec == QI_F32)
        k_normalise_to<float><<<g, 256, 0, s->stream>>>((float2 *)out, (const float2 *)in, s->dim(), s->d_result, s->d_flag);
    else
        k_normalise_to<double><<<g, 256, 0, s->stream>>>((double2 *)out, (const double2 *)in, s->dim(), s->d_result,
                                                         s->d_flag);
    count_launch();
    return check_launch("k_normalise_to");
}

Status state_scratch(qi_state *s, void **out) {
    if (!s->d_scratch) {
        cudaError_t e = cudaMalloc(&s->d_scratch, s->bytes());
        if (e != cudaSuccess) {
            s->d_scratch = nullptr;
            cudaGetLastError();   // clear the allocation error: the caller falls back
            return cuda_status(e, "cudaMalloc(second state buffer)");
        }
    }
    *out = s->d_scratch;
    return ok_status();
}

Status state_read_flag(qi_state *s, int *flag) {
    int h = 0;
    QI_CUDA(cudaMemcpyAsync(&h, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    QI_CUDA(cudaStreamSynchronize(s->stream));
    if (h) QI_CUDA(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream));
    *flag = h;
    return ok_status();
}

Status state_copy_async(qi_state *dst, const qi_state *src) {
    if (dst->n != src->n) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, src->n, -1);
    if (src->stream != dst->stream) QI_CUDA(cudaStreamSynchronize(src->stream));
    if (dst->prec == src->prec) {
        QI_CUDA(cudaMemcpyAsync(dst->amps, src->amps, src->bytes(), cudaMemcpyDeviceToDevice, dst->stream));
        return ok_status();
    }
    unsigned g = grid_for(src->dim());
    if (dst->prec == QI_F32)
        k_convert<float, double><<<g, 256, 0, dst->stream>>>((float2 *)dst->amps, (const double2 *)src->amps, src->dim());
    else
        k_convert<double, float><<<g, 256, 0, dst->stream>>>((double2 *)dst->amps, (const float2 *)src->amps, src->dim());
    count_launch();
    return check_launch("k_convert");
}

static Status ensure_staging(qi_state *s, size_t bytes) {
    if (s->staging_bytes >= bytes) return ok_status();
    if (s->d_staging) { cudaFree(s->d_staging); s->d_staging = nullptr; s->staging_bytes = 0; }
    QI_CUDA(cudaMalloc(&s->d_staging, bytes));
    s->staging_bytes = bytes;
    return ok_status();
}

}  // namespace qi

using namespace qi;

#define QI_GUARD(s)                                                   \
    if (!(s)) return publish(err(QI_ERR_NULL_ARGUMENT, -1, -1, "null state")); \
    std::lock_guard<std::recursive_mutex> qi_lock_((s)->mu);          \
    {                                                                 \
        Status qi_dev_ = ensure_device(s);                            \
        if (!qi_dev_.ok()) return publish(qi_dev_);                   \
    }

// Transfers the GPU itself makes over the CPU-GPU link (page-locked, mapped host buffers) run on
// the handle's lowest-priority link stream, ordered after and before the handle's stream by events,
// in short blocks (1024 amplitudes each, four 16-byte accesses in flight per thread): a circuit on a
// higher-priority stream of another handle gets each SM back as soon as the blocks on it finish, and
// the transfer fills what the circuit leaves free.
static unsigned link_blocks(uint64_t num_amps) { return (unsigned)((num_amps + 1023) / 1024); }

template <typename Launch>
static Status on_link_stream(qi_state *s, Launch launch) {
    cudaError_t e = cudaSuccess;
    if (!s->link_stream) {
        int least = 0, greatest = 0;
        e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->link_stream, cudaStreamNonBlocking, least);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&s->link_ev[i], cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_status(e, "link stream");
    }
    e = cudaEventRecord(s->link_ev[0], s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->link_stream, s->link_ev[0], 0);
    if (e != cudaSuccess) return cuda_status(e, "link stream order");
    launch(s->link_stream);
    count_launch();
    Status st = check_launch("k_convert_link");
    if (!st.ok()) return st;
    e = cudaEventRecord(s->link_ev[1], s->link_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->link_ev[1], 0);
    if (e != cudaSuccess) return cuda_status(e, "link stream order");
    return ok_status();
}

extern "C" {

qi_status qi_last_error(qi_error_info *out) {
    if (!out) return QI_ERR_NULL_ARGUMENT;
    *out = t_last;
    return QI_OK;
}

const char *qi_version(void) { return "quant-iron-gb300 0.1 (sm_103a)"; }

uint64_t qi_launch_count(void) { return g_launches.load(); }

qi_status qi_set_device(int32_t device) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaGetDeviceCount"));
    if (device < 0 || device >= count) return publish(err(QI_ERR_INVALID_INPUT_VALUE, device, count, "no such device"));
    g_device = device;
    return publish(ok_status());
}

qi_status qi_state_create(int32_t num_qubits, int32_t precision, qi_state **out) {
    if (!out) return publish(err(QI_ERR_NULL_ARGUMENT));
    *out = nullptr;
    if (num_qubits <= 0) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, num_qubits < 0 ? 0 : num_qubits));
    if (num_qubits > 40) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, num_qubits));
    if (precision != QI_F32 && precision != QI_F64) return publish(err(QI_ERR_INVALID_INPUT_VALUE, precision));
    qi_state *s = new qi_state();
    s->n = num_qubits;
    s->prec = precision;
    s->device = g_device;
    auto fail = [&](Status st) {
        if (s->amps) cudaFree(s->amps);
        if (s->d_partials) cudaFree(s->d_partials);
        if (s->d_result) cudaFree(s->d_result);
        if (s->h_result) cudaFreeHost(s->h_result);
        if (s->d_flag) cudaFree(s->d_flag);
        if (s->own_stream) cudaStreamDestroy(s->own_stream);
        delete s;
        return publish(st);
    };
    cudaError_t e;
    if ((e = cudaSetDevice(s->device)) != cudaSuccess) return fail(cuda_status(e, "cudaSetDevice"));
    if ((e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(cuda_status(e, "cudaStreamCreate"));
    s->stream = s->own_stream;
    if ((e = cudaMalloc(&s->amps, s->bytes())) != cudaSuccess) return fail(cuda_status(e, "cudaMalloc(state)"));
    if ((e = cudaMalloc(&s->d_partials, kReduceBlocks * 4 * sizeof(double))) != cudaSuccess)
        return fail(cuda_status(e, "cudaMalloc(partials)"));
    if ((e = cudaMalloc(&s->d_result, 8 * sizeof(double))) != cudaSuccess) return fail(cuda_status(e, "cudaMalloc"));
    if ((e = cudaMallocHost(&s->h_result, 8 * sizeof(double))) != cudaSuccess) return fail(cuda_status(e, "cudaMallocHost"));
    if ((e = cudaMalloc(&s->d_flag, sizeof(int))) != cudaSuccess) return fail(cuda_status(e, "cudaMalloc"));
    if ((e = cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream)) != cudaSuccess) return fail(cuda_status(e, "memset"));
    *out = s;
    return publish(ok_status());
}

qi_status qi_state_destroy(qi_state *s) {
    if (!s) return QI_OK;
    {
        std::lock_guard<std::recursive_mutex> lk(s->mu);
        cudaSetDevice(s->device);
        cudaStreamSynchronize(s->stream);
        if (s->amps) cudaFree(s->amps);
        if (s->d_partials) cudaFree(s->d_partials);
        if (s->d_result) cudaFree(s->d_result);
        if (s->h_result) cudaFreeHost(s->h_result);
        if (s->d_flag) cudaFree(s->d_flag);
        if (s->d_staging) cudaFree(s->d_staging);
        if (s->d_scratch) cudaFree(s->d_scratch);
        if (s->link_stream) {
            cudaStreamSynchronize(s->link_stream);
            cudaStreamDestroy(s->link_stream);
        }
        for (cudaEvent_t ev : s->link_ev)
            if (ev) cudaEventDestroy(ev);
        if (s->own_stream) cudaStreamDestroy(s->own_stream);
    }
    delete s;
    return QI_OK;
}

qi_status qi_state_info(const qi_state *s, int32_t *num_qubits, int32_t *precision) {
    if (!s) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_qubits) *num_qubits = s->n;
    if (precision) *precision = s->prec;
    return QI_OK;
}

qi_status qi_state_set_stream(qi_state *s, void *cuda_stream) {
    QI_GUARD(s);
    s->stream = cuda_stream ? (cudaStream_t)cuda_stream : s->own_stream;
    return publish(ok_status());
}

qi_status qi_state_get_stream(qi_state *s, void **cuda_stream) {
    QI_GUARD(s);
    if (cuda_stream) *cuda_stream = (void *)s->stream;
    return publish(ok_status());
}

qi_status qi_state_device_ptr(qi_state *s, void **dev_ptr) {
    QI_GUARD(s);
    if (dev_ptr) *dev_ptr = s->amps;
    return publish(ok_status());
}

qi_status qi_state_wait(qi_state *s, qi_state *other) {
    if (!other) return publish(err(QI_ERR_NULL_ARGUMENT, -1, -1, "null state"));
    cudaStream_t theirs;
    {
        std::lock_guard<std::recursive_mutex> lk(other->mu);
        theirs = other->stream;
    }
    QI_GUARD(s);
    if (theirs == s->stream) return publish(ok_status());
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaEventCreate"));
    e = cudaEventRecord(ev, theirs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, ev, 0);
    cudaEventDestroy(ev);   // released once the wait has been satisfied
    if (e != cudaSuccess) return publish(cuda_status(e, "qi_state_wait"));
    return publish(ok_status());
}

qi_status qi_state_synchronize(qi_state *s) {
    QI_GUARD(s);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaStreamSynchronize"));
    return publish(ok_status());
}

// Chunked transfer through a device staging buffer with on-device conversion.
static constexpr uint64_t kChunkAmps = 1ull << 22;   // 4 Mi amplitudes = 64 MiB of f64 pairs

// Device-side address of a page-locked, mapped, 16-byte aligned host buffer (the GPU
// reads and writes it directly over the CPU-GPU link), or nullptr otherwise.
static void *mapped_host_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || ((uintptr_t)at.devicePointer & 15) != 0) return nullptr;
    return at.devicePointer;
}

qi_status qi_state_upload(qi_state *s, const double *amps, uint64_t num_amps) {
    QI_GUARD(s);
    if (!amps) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_amps != s->dim()) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n));
    if (s->prec == QI_F64) {
        cudaError_t e = cudaMemcpyAsync(s->amps, amps, s->bytes(), cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "upload"));
        return publish(ok_status());
    }
    if (const void *dp = mapped_host_ptr(amps)) {   // pinned: one pass reads the host buffer and converts
        const Status st = on_link_stream(s, [&](cudaStream_t ls) {
            k_convert_link<float, double><<<link_blocks(num_amps), 256, 0, ls>>>((float2 *)s->amps,
                                                                               (const double2 *)dp, num_amps);
        });
        return publish(st);
    }
    const uint64_t chunk = num_amps < kChunkAmps ? num_amps : kChunkAmps;
    Status st = ensure_staging(s, 2 * chunk * 16);
    if (!st.ok()) return publish(st);
    for (uint64_t off = 0, it = 0; off < num_amps; off += chunk, ++it) {
        uint64_t cnt = (num_amps - off) < chunk ? (num_amps - off) : chunk;
        double2 *stg = (double2 *)s->d_staging + (it & 1) * chunk;
        cudaError_t e = cudaMemcpyAsync(stg, amps + 2 * off, cnt * 16, cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "upload chunk"));
        k_convert<float, double><<<grid_for(cnt), 256, 0, s->stream>>>((float2 *)s->amps + off, stg, cnt);
        count_launch();
    }
    return publish(check_launch("k_convert"));
}

qi_status qi_state_upload_async(qi_state *s, const double *amps, uint64_t num_amps) {
    QI_GUARD(s);
    if (!amps) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_amps != s->dim()) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n));
    if (!mapped_host_ptr(amps)) return publish(err(QI_ERR_INVALID_INPUT_VALUE, -1, -1, "host buffer not page-locked"));
    if (s->prec == QI_F64) {
        cudaError_t e = cudaMemcpyAsync(s->amps, amps, s->bytes(), cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "upload_async"));
        return publish(ok_status());
    }
    Status st = ensure_staging(s, num_amps * 16);
    if (!st.ok()) return publish(st);
    cudaError_t e = cudaMemcpyAsync(s->d_staging, amps, num_amps * 16, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "upload_async"));
    k_convert<float, double><<<grid_for(num_amps), 256, 0, s->stream>>>((float2 *)s->amps,
                                                                        (const double2 *)s->d_staging, num_amps);
    count_launch();
    return publish(check_launch("k_convert"));
}

qi_status qi_state_download_async(qi_state *s, double *amps, uint64_t num_amps) {
    QI_GUARD(s);
    if (!amps) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_amps != s->dim()) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n));
    if (!mapped_host_ptr(amps)) return publish(err(QI_ERR_INVALID_INPUT_VALUE, -1, -1, "host buffer not page-locked"));
    if (s->prec == QI_F64) {
        cudaError_t e = cudaMemcpyAsync(amps, s->amps, s->bytes(), cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "download_async"));
        return publish(ok_status());
    }
    Status st = ensure_staging(s, num_amps * 16);
    if (!st.ok()) return publish(st);
    k_convert<double, float><<<grid_for(num_amps), 256, 0, s->stream>>>((double2 *)s->d_staging,
                                                                        (const float2 *)s->amps, num_amps);
    count_launch();
    st = check_launch("k_convert");
    if (!st.ok()) return publish(st);
    cudaError_t e = cudaMemcpyAsync(amps, s->d_staging, num_amps * 16, cudaMemcpyDeviceToHost, s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "download_async"));
    return publish(ok_status());
}

qi_status qi_state_download(qi_state *s, double *amps, uint64_t num_amps) {
    QI_GUARD(s);
    if (!amps) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_amps != s->dim()) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n));
    if (s->prec == QI_F64) {
        cudaError_t e = cudaMemcpyAsync(amps, s->amps, s->bytes(), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "download"));
        return publish(ok_status());
    }
    if (void *dp = mapped_host_ptr(amps)) {   // pinned: one pass converts and writes the host buffer
        Status st = on_link_stream(s, [&](cudaStream_t ls) {
            k_convert_link<double, float><<<link_blocks(num_amps), 256, 0, ls>>>((double2 *)dp,
                                                                               (const float2 *)s->amps, num_amps);
        });
        if (!st.ok()) return publish(st);
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "download"));
        return publish(ok_status());
    }
    const uint64_t chunk = num_amps < kChunkAmps ? num_amps : kChunkAmps;
    Status st = ensure_staging(s, 2 * chunk * 16);
    if (!st.ok()) return publish(st);
    for (uint64_t off = 0, it = 0; off < num_amps; off += chunk, ++it) {
        uint64_t cnt = (num_amps - off) < chunk ? (num_amps - off) : chunk;
        double2 *stg = (double2 *)s->d_staging + (it & 1) * chunk;
        k_convert<double, float><<<grid_for(cnt), 256, 0, s->stream>>>(stg, (const float2 *)s->amps + off, cnt);
        count_launch();
        cudaError_t e = cudaMemcpyAsync(amps + 2 * off, stg, cnt * 16, cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "download chunk"));
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "download"));
    return publish(ok_status());
}

static qi_status fill_const(qi_state *s, double re, double im) {
    unsigned g = grid_for(s->dim());
    if (s->prec == QI_F32) k_fill_const<float><<<g, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), (float)re, (float)im);
    else k_fill_const<double><<<g, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), re, im);
    count_launch();
    return publish(check_launch("k_fill_const"));
}

static qi_status set_one(qi_state *s, uint64_t idx, double re) {
    cudaError_t e = cudaMemsetAsync(s->amps, 0, s->bytes(), s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "memset"));
    if (s->prec == QI_F32) {
        static const float2 one = {1.0f, 0.0f};
        float2 v = one; v.x = (float)re;
        // value copied from a stack temporary: synchronise before it goes out of scope
        e = cudaMemcpyAsync((float2 *)s->amps + idx, &v, sizeof(v), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    } else {
        double2 v = {re, 0.0};
        e = cudaMemcpyAsync((double2 *)s->amps + idx, &v, sizeof(v), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    if (e != cudaSuccess) return publish(cuda_status(e, "set amplitude"));
    return publish(ok_status());
}

qi_status qi_state_set_zero(qi_state *s) { QI_GUARD(s); return set_one(s, 0, 1.0); }

qi_status qi_state_set_basis(qi_state *s, uint64_t n) {
    QI_GUARD(s);
    if (n >= s->dim()) return publish(err(QI_ERR_INVALID_QUBIT_INDEX, (int64_t)n, s->n));   // state.rs:196-198
    return set_one(s, n, 1.0);
}

qi_status qi_state_set_plus(qi_state *s) {   // state.rs:225-237
    QI_GUARD(s);
    return fill_const(s, 1.0 / std::sqrt((double)s->dim()), 0.0);
}

qi_status qi_state_set_minus(qi_state *s) {
    QI_GUARD(s);
    double a = 1.0 / std::sqrt((double)s->dim());
    unsigned g = grid_for(s->dim());
    if (s->prec == QI_F32) k_fill_minus<float><<<g, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), (float)a);
    else k_fill_minus<double><<<g, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), a);
    count_launch();
    return publish(check_launch("k_fill_minus"));
}

qi_status qi_state_set_ghz(qi_state *s) {   // state.rs:305-325
    QI_GUARD(s);
    const double r = 0.70710678118654752440;   // FRAC_1_SQRT_2
    qi_status st = set_one(s, 0, r);
    if (st != QI_OK) return st;
    if (s->prec == QI_F32) {
        float2 v = {(float)r, 0.0f};
        cudaError_t e = cudaMemcpy((float2 *)s->amps + (s->dim() - 1), &v, sizeof(v), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return publish(cuda_status(e, "ghz"));
    } else {
        double2 v = {r, 0.0};
        cudaError_t e = cudaMemcpy((double2 *)s->amps + (s->dim() - 1), &v, sizeof(v), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return publish(cuda_status(e, "ghz"));
    }
    return publish(ok_status());
}

qi_status qi_state_check_normalised(qi_state *s) {   // state.rs:118-123
    QI_GUARD(s);
    double nrm;
    Status st = state_reduce_norm_sqr(s, &nrm);
    if (!st.ok()) return publish(st);
    const double tol = 2.220446049250313e-16 * (double)s->dim();
    if (std::fabs(nrm - 1.0) > tol) return publish(err(QI_ERR_STATE_NOT_NORMALISED));
    return publish(ok_status());
}

qi_status qi_state_copy(qi_state *dst, const qi_state *src) {
    QI_GUARD(dst);
    if (!src) return publish(err(QI_ERR_NULL_ARGUMENT));
    return publish(state_copy_async(dst, src));
}

qi_status qi_state_scale(qi_state *s, double re, double im) {
    QI_GUARD(s);
    return publish(state_scale_async(s, re, im));
}

qi_status qi_state_axpy(qi_state *y, double re, double im, const qi_state *x) {
    QI_GUARD(y);
    if (!x) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (x->n != y->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, x->n));
    if (x->prec != y->prec) return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "axpy needs equal precisions"));
    if (x->stream != y->stream) {
        cudaError_t e = cudaStreamSynchronize(x->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "sync"));
    }
    unsigned g = grid_for(y->dim());
    if (y->prec == QI_F32)
        k_axpy<float><<<g, 256, 0, y->stream>>>((float2 *)y->amps, (const float2 *)x->amps, y->dim(), (float)re, (float)im);
    else
        k_axpy<double><<<g, 256, 0, y->stream>>>((double2 *)y->amps, (const double2 *)x->amps, y->dim(), re, im);
    count_launch();
    return publish(check_launch("k_axpy"));
}

qi_status qi_state_inner_product(qi_state *a, qi_state *b, double out[2]) {
    QI_GUARD(a);
    if (!b || !out) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (a->n != b->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, a->n));   // state.rs:895-897
    if (a->prec != b->prec) return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "inner product needs equal precisions"));
    return publish(state_inner(a, b, out));
}

qi_status qi_state_compare(qi_state *a, qi_state *b, double out[4]) {
    QI_GUARD(a);
    if (!b || !out) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (a->n != b->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, b->n));
    if (b->stream != a->stream) {   // order b's pending work before the comparison on a's stream
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ev, b->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(a->stream, ev, 0);
        if (e == cudaSuccess) e = cudaEventDestroy(ev);
        if (e != cudaSuccess) return publish(cuda_status(e, "qi_state_compare"));
    }
    const unsigned nb = reduce_grid(a->dim());
    const bool fa = a->prec == QI_F32, fb = b->prec == QI_F32;
    if (fa && fb)
        k_compare_partial<float, float><<<nb, kReduceThreads, 0, a->stream>>>((const float2 *)a->amps,
                                                                             (const float2 *)b->amps, a->dim(), a->d_partials);
    else if (fa)
        k_compare_partial<float, double><<<nb, kReduceThreads, 0, a->stream>>>((const float2 *)a->amps,
                                                                              (const double2 *)b->amps, a->dim(), a->d_partials);
    else if (fb)
        k_compare_partial<double, float><<<nb, kReduceThreads, 0, a->stream>>>((const double2 *)a->amps,
                                                                              (const float2 *)b->amps, a->dim(), a->d_partials);
    else
        k_compare_partial<double, double><<<nb, kReduceThreads, 0, a->stream>>>((const double2 *)a->amps,
                                                                               (const double2 *)b->amps, a->dim(), a->d_partials);
    k_compare_finalize<<<1, 256, 0, a->stream>>>(a->d_partials, (int)nb, a->d_result);
    count_launch(2);
    Status st = check_launch("k_compare_partial");
    if (!st.ok()) return publish(st);
    cudaError_t e = cudaMemcpyAsync(a->h_result, a->d_result, 4 * sizeof(double), cudaMemcpyDeviceToHost, a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "qi_state_compare"));
    out[0] = std::sqrt(a->h_result[0]);
    for (int c = 1; c < 4; ++c) out[c] = a->h_result[c];
    return publish(ok_status());
}

qi_status qi_state_norm_sqr(qi_state *s, double *out) {
    QI_GUARD(s);
    if (!out) return publish(err(QI_ERR_NULL_ARGUMENT));
    return publish(state_reduce_norm_sqr(s, out));
}

qi_status qi_state_normalise(qi_state *s) {   // state.rs:924-945
    QI_GUARD(s);
    Status st = state_normalise_device_async(s);
    if (!st.ok()) return publish(st);
    int flag = 0;
    st = state_read_flag(s, &flag);
    if (!st.ok()) return publish(st);
    if (flag) return publish(err(QI_ERR_ZERO_NORM));
    return publish(ok_status());
}

qi_status qi_state_tensor_product(qi_state *out, qi_state *a, qi_state *b) {
    QI_GUARD(out);
    if (!a || !b) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (out->n != a->n + b->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, out->n));
    if (a->prec != out->prec || b->prec != out->prec)
        return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "tensor product needs equal precisions"));
    cudaError_t e = cudaStreamSynchronize(a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "sync"));
    unsigned g = grid_for(out->dim());
    if (out->prec == QI_F32)
        k_tensor<float><<<g, 256, 0, out->stream>>>((float2 *)out->amps, (const float2 *)a->amps, (const float2 *)b->amps,
                                                   out->dim(), b->n);
    else
        k_tensor<double><<<g, 256, 0, out->stream>>>((double2 *)out->amps, (const double2 *)a->amps,
                                                    (const double2 *)b->amps, out->dim(), b->n);
    count_launch();
    return publish(check_launch("k_tensor"));
}

qi_status qi_state_amplitude(qi_state *s, uint64_t n, double out[2]) {
    QI_GUARD(s);
    if (!out) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (n >= s->dim()) return publish(err(QI_ERR_INVALID_QUBIT_INDEX, (int64_t)n, s->n));   // state.rs:449-451
    cudaError_t e;
    if (s->prec == QI_F32) {
        float2 v;
        e = cudaMemcpyAsync(&v, (const float2 *)s->amps + n, sizeof(v), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        out[0] = v.x; out[1] = v.y;
    } else {
        double2 v;
        e = cudaMemcpyAsync(&v, (const double2 *)s->amps + n, sizeof(v), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        out[0] = v.x; out[1] = v.y;
    }
    if (e != cudaSuccess) return publish(cuda_status(e, "amplitude"));
    return publish(ok_status());
}

}  // extern "C"
