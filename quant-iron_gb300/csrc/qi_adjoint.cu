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
#include "qi_tile.cuh"

#include <algorithm>
#include <atomic>
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
// amplitudes of psi and lambda its qubits span and, gate after gate, adds
// Re(conj(lambda) D psi) with D = dU U^dagger (the derivative taken before un-applying),
// then un-applies U^dagger on psi and on lambda, all in registers.
constexpr int kMultiQubits = 4, kMultiStages = 2, kMultiComps = kMultiQubits * kMultiStages;
// Stage kinds: matrix structure of U^dagger and D together (host-classified, exact zeros).
enum : int8_t { kStageGeneral = 0, kStageDiag = 1, kStageReal = 2, kStageNoDeriv = 4 };
struct MultiParams {
    uint64_t nwork;
    int8_t pos[kMultiQubits];                     // the group's qubits, ascending (combo bit i <-> pos[i])
    int8_t kind[kMultiQubits][kMultiStages];      // kStage* (| kStageNoDeriv when D = 0)
    double uinv[kMultiQubits][kMultiStages][8];   // qubit i, stage s: U^dagger, 2x2 complex row-major
    double d[kMultiQubits][kMultiStages][8];      // D = dU/dtheta U^dagger (zero for a fixed gate / unused stage)
};

// Launch shape per precision: threads per block and cp.async buffers (the copies of the
// next kPipe - 1 work items are in flight while one is computed).  Both fill ~192 KB of
// shared memory with one block per SM.
template <typename T> struct MultiShape;
template <> struct MultiShape<float> { static constexpr int kThreads = 384, kPipe = 2; using Amp = uint64_t; };
template <> struct MultiShape<double> { static constexpr int kThreads = 256, kPipe = 3; using Amp = double2; };

// ---- FP32: an amplitude is one 64-bit register pair (re, im), arithmetic in packed f32x2.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 upk2(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t swap2(uint64_t v) {
    const float2 f = upk2(v);
    return pk2(f.y, f.x);
}
// Stage table: entry k of a 2x2 complex matrix (a + ib) as A = (a, a) and B = (-b, b), so
// that (a + ib) x = A * x + B * swap(x) lane-wise; T[0..7] = U^dagger, T[8..15] = D.
__device__ __forceinline__ void build_stage_table(uint64_t *T, const double *u, const double *d) {
    for (int k = 0; k < 4; ++k) {
        T[2 * k] = pk2((float)u[2 * k], (float)u[2 * k]);
        T[2 * k + 1] = pk2((float)-u[2 * k + 1], (float)u[2 * k + 1]);
        T[8 + 2 * k] = pk2((float)d[2 * k], (float)d[2 * k]);
        T[8 + 2 * k + 1] = pk2((float)-d[2 * k + 1], (float)d[2 * k + 1]);
    }
}

// One stage (gate) on combo bit G: derivative term Re(conj(lambda) D psi), then un-apply.
template <int D, int G>
__device__ __forceinline__ float multi_stage_f32(uint64_t *x, uint64_t *l, int kind, const uint64_t *T) {
    uint64_t acc = 0;   // lane-wise partial sums (+0.0f, +0.0f)
    const bool deriv = !(kind & kStageNoDeriv);
    kind &= 3;
    if (kind == kStageDiag) {
        const uint64_t A0 = T[0], B0 = T[1], A3 = T[6], B3 = T[7], P0 = T[8], Q0 = T[9], P3 = T[14], Q3 = T[15];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if ((c >> G) & 1) continue;
            const int c1 = c | (1 << G);
            const uint64_t x0 = x[c], x1 = x[c1], l0 = l[c], l1 = l[c1];
            const uint64_t x0s = swap2(x0), x1s = swap2(x1);
            if (deriv) {   // Re(delta conj(l) x) = (l * (dr, dr)) . x + (l * (-di, di)) . swap(x)
                acc = fma2(mul2(l0, P0), x0, acc);
                acc = fma2(mul2(l0, Q0), x0s, acc);
                acc = fma2(mul2(l1, P3), x1, acc);
                acc = fma2(mul2(l1, Q3), x1s, acc);
            }
            x[c] = fma2(B0, x0s, mul2(A0, x0));
            x[c1] = fma2(B3, x1s, mul2(A3, x1));
            l[c] = fma2(B0, swap2(l0), mul2(A0, l0));
            l[c1] = fma2(B3, swap2(l1), mul2(A3, l1));
        }
    } else if (kind == kStageReal) {
        const uint64_t R0 = T[0], R1 = T[2], R2 = T[4], R3 = T[6], Q0 = T[8], Q1 = T[10], Q2 = T[12], Q3 = T[14];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if ((c >> G) & 1) continue;
            const int c1 = c | (1 << G);
            const uint64_t x0 = x[c], x1 = x[c1], l0 = l[c], l1 = l[c1];
            if (deriv) {
                acc = fma2(l0, fma2(Q1, x1, mul2(Q0, x0)), acc);
                acc = fma2(l1, fma2(Q3, x1, mul2(Q2, x0)), acc);
            }
            x[c] = fma2(R1, x1, mul2(R0, x0));
            x[c1] = fma2(R3, x1, mul2(R2, x0));
            l[c] = fma2(R1, l1, mul2(R0, l0));
            l[c1] = fma2(R3, l1, mul2(R2, l0));
        }
    } else {
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if ((c >> G) & 1) continue;
            const int c1 = c | (1 << G);
            const uint64_t x0 = x[c], x1 = x[c1], l0 = l[c], l1 = l[c1];
            const uint64_t x0s = swap2(x0), x1s = swap2(x1), l0s = swap2(l0), l1s = swap2(l1);
            if (deriv) {
                const uint64_t d0 = fma2(T[11], x1s, fma2(T[10], x1, fma2(T[9], x0s, mul2(T[8], x0))));
                const uint64_t d1 = fma2(T[15], x1s, fma2(T[14], x1, fma2(T[13], x0s, mul2(T[12], x0))));
                acc = fma2(l0, d0, acc);
                acc = fma2(l1, d1, acc);
            }
            x[c] = fma2(T[3], x1s, fma2(T[2], x1, fma2(T[1], x0s, mul2(T[0], x0))));
            x[c1] = fma2(T[7], x1s, fma2(T[6], x1, fma2(T[5], x0s, mul2(T[4], x0))));
            l[c] = fma2(T[3], l1s, fma2(T[2], l1, fma2(T[1], l0s, mul2(T[0], l0))));
            l[c1] = fma2(T[7], l1s, fma2(T[6], l1, fma2(T[5], l0s, mul2(T[4], l0))));
        }
    }
    const float2 a = upk2(acc);
    return a.x + a.y;
}

// ---- FP64: double2 amplitudes, plain complex arithmetic.
template <int D, int G>
__device__ __forceinline__ double multi_stage_f64(double2 *x, double2 *l, int kind, const double2 *u,
                                                  const double2 *e) {
    using X = Cx<double>;
    double part = 0;
    const bool deriv = !(kind & kStageNoDeriv);
    kind &= 3;
    if (kind == kStageDiag) {
        const double2 u0 = u[0], u3 = u[3], e0 = e[0], e3 = e[3];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if ((c >> G) & 1) continue;
            const int c1 = c | (1 << G);
            if (deriv) {
                const double2 d0 = X::mul(e0, x[c]), d1 = X::mul(e3, x[c1]);
                part += l[c].x * d0.x + l[c].y * d0.y + l[c1].x * d1.x + l[c1].y * d1.y;
            }
            x[c] = X::mul(u0, x[c]);
            x[c1] = X::mul(u3, x[c1]);
            l[c] = X::mul(u0, l[c]);
            l[c1] = X::mul(u3, l[c1]);
        }
    } else {   // real matrices take the general form: FP64 states are bound by the FP64 pipe either way
        const double2 u0 = u[0], u1 = u[1], u2 = u[2], u3 = u[3];
        const double2 e0 = e[0], e1 = e[1], e2 = e[2], e3 = e[3];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            if ((c >> G) & 1) continue;
            const int c1 = c | (1 << G);
            const double2 x0 = x[c], x1 = x[c1], l0 = l[c], l1 = l[c1];
            if (deriv) {
                const double2 d0 = X::fma(e1, x1, X::mul(e0, x0)), d1 = X::fma(e3, x1, X::mul(e2, x0));
                part += l0.x * d0.x + l0.y * d0.y + l1.x * d1.x + l1.y * d1.y;
            }
            x[c] = X::fma(u1, x1, X::mul(u0, x0));
            x[c1] = X::fma(u3, x1, X::mul(u2, x0));
            l[c] = X::fma(u1, l1, X::mul(u0, l0));
            l[c1] = X::fma(u3, l1, X::mul(u2, l0));
        }
    }
    return part;
}

// Per-block stage data in shared memory.
template <typename T, int M, int S> struct MultiStageSmem;
template <int M, int S> struct MultiStageSmem<float, M, S> {
    uint64_t tab[M][S][16];
    int8_t kind[M][S];
    __device__ void load(const MultiParams &p) {
        if (threadIdx.x < M * S) {
            const int g = threadIdx.x / S, st = threadIdx.x % S;
            build_stage_table(tab[g][st], p.uinv[g][st], p.d[g][st]);
            kind[g][st] = p.kind[g][st];
        }
    }
    template <int G> __device__ __forceinline__ float run(uint64_t *x, uint64_t *l, int st) const {
        return multi_stage_f32<1 << M, G>(x, l, kind[G][st], tab[G][st]);
    }
};
template <int M, int S> struct MultiStageSmem<double, M, S> {
    double2 u[M][S][4], e[M][S][4];
    int8_t kind[M][S];
    __device__ void load(const MultiParams &p) {
        if (threadIdx.x < 4 * M * S) {
            const int g = threadIdx.x / (4 * S), st = (threadIdx.x >> 2) % S, i = threadIdx.x & 3;
            u[g][st][i] = make_double2(p.uinv[g][st][2 * i], p.uinv[g][st][2 * i + 1]);
            e[g][st][i] = make_double2(p.d[g][st][2 * i], p.d[g][st][2 * i + 1]);
            if (i == 0) kind[g][st] = p.kind[g][st];
        }
    }
    template <int G> __device__ __forceinline__ double run(double2 *x, double2 *l, int st) const {
        return multi_stage_f64<1 << M, G>(x, l, kind[G][st], u[G][st], e[G][st]);
    }
};

template <typename T, int M, int S, int G, typename Amp, typename Acc>
__device__ __forceinline__ void multi_qubits(Amp *x, Amp *l, const MultiStageSmem<T, M, S> &sm, Acc *acc) {
    if constexpr (G < M) {
#pragma unroll
        for (int st = 0; st < S; ++st) acc[G * S + st] += sm.template run<G>(x, l, st);
        multi_qubits<T, M, S, G + 1>(x, l, sm, acc);
    }
}

// Work items stream through shared memory: each thread copies its item's 2^M amplitudes of
// psi and lambda with cp.async kPipe - 1 items ahead (the copies hold no registers while in
// flight), then reads them back, runs the stages and stores to global memory.  Thread t owns
// column t of every buffer, so no block barrier is needed in the loop.  FP32 derivative
// terms are summed in FP32 over batches of 16 items per thread and folded into FP64 per batch (an
// FP64 add per item and stage would load the scarce FP64 pipe).
// P0 (FP32, qubit 0 in the group): combos c and c | 1 are adjacent amplitudes, so each pair moves
// as one 16-byte copy, read and stored as one 16-byte access (the group's items are 2^M
// consecutive amplitudes; 8-byte copies would request every 32-byte sector four times).
template <typename T, int M, int S, bool P0 = false>
__global__ void __launch_bounds__(MultiShape<T>::kThreads, 1)
    k_adjoint_multi(typename MultiShape<T>::Amp *psi, typename MultiShape<T>::Amp *lam,
                    const __grid_constant__ MultiParams p, double *partials) {
    using Amp = typename MultiShape<T>::Amp;
    constexpr int TH = MultiShape<T>::kThreads, PIPE = MultiShape<T>::kPipe, D = 1 << M;
    constexpr int BATCH = sizeof(T) == 4 ? 16 : 1;
    extern __shared__ __align__(16) unsigned char multi_smem[];
    Amp *buf = reinterpret_cast<Amp *>(multi_smem);   // [PIPE][2][D][TH]
    __shared__ MultiStageSmem<T, M, S> sm;
    sm.load(p);
    __syncthreads();
    uint64_t bitm[M];
#pragma unroll
    for (int i = 0; i < M; ++i) bitm[i] = 1ull << p.pos[i];
    const int t = threadIdx.x;
    auto slot = [&](int stage, int which, int c) -> Amp * {
        return buf + (((size_t)stage * 2 + which) * D + c) * TH + t;
    };
    // P0: pair cp (combos 2cp, 2cp + 1) of thread t, 16 bytes
    auto slot2 = [&](int stage, int which, int cp) -> Amp * {
        return buf + ((((size_t)stage * 2 + which) * (D / 2) + cp) * TH + t) * 2;
    };
    auto issue = [&](uint64_t w, int stage) {
        if (w < p.nwork) {
            const uint64_t base = insert_zeros(w, p.pos, M);
#pragma unroll
            for (int c = 0; c < D; c += (P0 ? 2 : 1)) {
                uint64_t o = base;
#pragma unroll
                for (int i = 0; i < M; ++i)
                    if ((c >> i) & 1) o |= bitm[i];
                if constexpr (P0) {
                    cp_async_16(slot2(stage, 0, c >> 1), psi + o);
                    cp_async_16(slot2(stage, 1, c >> 1), lam + o);
                } else if constexpr (sizeof(Amp) == 8) {
                    cp_async_8(slot(stage, 0, c), psi + o);
                    cp_async_8(slot(stage, 1, c), lam + o);
                } else {
                    cp_async_16(slot(stage, 0, c), psi + o);
                    cp_async_16(slot(stage, 1, c), lam + o);
                }
            }
        }
        cp_async_commit();   // an empty group past the end keeps the group count uniform
    };
    double acc[M * S];
    T accb[M * S];
#pragma unroll
    for (int g = 0; g < M * S; ++g) acc[g] = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * TH;
    const uint64_t w0 = blockIdx.x * (uint64_t)TH + t;
#pragma unroll
    for (int k = 0; k < PIPE - 1; ++k) issue(w0 + k * stride, k);
    int stage = 0;
    for (uint64_t wb = w0; wb < p.nwork; wb += BATCH * stride) {
        const uint64_t wend = min(p.nwork, wb + BATCH * stride);
#pragma unroll
        for (int g = 0; g < M * S; ++g) accb[g] = 0;
#pragma unroll 1
        for (uint64_t w = wb; w < wend; w += stride) {
            cp_async_wait<PIPE - 2>();   // this item's group has landed
            Amp x[D], l[D];
            if constexpr (P0) {
#pragma unroll
                for (int c = 0; c < D; c += 2) {
                    const ulonglong2 u = *reinterpret_cast<const ulonglong2 *>(slot2(stage, 0, c >> 1));
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(slot2(stage, 1, c >> 1));
                    x[c] = u.x;
                    x[c + 1] = u.y;
                    l[c] = v.x;
                    l[c + 1] = v.y;
                }
            } else {
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    x[c] = *slot(stage, 0, c);
                    l[c] = *slot(stage, 1, c);
                }
            }
            // refill the buffer read one iteration ago (only this thread uses its column)
            issue(w + (PIPE - 1) * stride, stage == 0 ? PIPE - 1 : stage - 1);
            multi_qubits<T, M, S, 0>(x, l, sm, accb);
            const uint64_t base = insert_zeros(w, p.pos, M);
#pragma unroll
            for (int c = 0; c < D; c += (P0 ? 2 : 1)) {
                uint64_t o = base;
#pragma unroll
                for (int i = 0; i < M; ++i)
                    if ((c >> i) & 1) o |= bitm[i];
                if constexpr (P0) {
                    *reinterpret_cast<ulonglong2 *>(psi + o) = make_ulonglong2(x[c], x[c + 1]);
                    *reinterpret_cast<ulonglong2 *>(lam + o) = make_ulonglong2(l[c], l[c + 1]);
                } else {
                    psi[o] = x[c];
                    lam[o] = l[c];
                }
            }
            stage = stage == PIPE - 1 ? 0 : stage + 1;
        }
#pragma unroll
        for (int g = 0; g < M * S; ++g) acc[g] += (double)accb[g];
    }
    cp_async_wait<0>();
#pragma unroll
    for (int g = 0; g < M * S; ++g) {
        const double v = block_sum(acc[g]);
        if (threadIdx.x == 0) partials[blockIdx.x * kMultiComps + g] = v;
    }
}

// One block per SM slot the shared-memory pipeline leaves (grid-stride over the work items);
// *nb_out = blocks launched (= partial-sum rows).
template <typename T, int M, int S, bool P0 = false>
static Status launch_adjoint_multi(qi_state *s, qi_state *lam, const MultiParams &mp, unsigned *nb_out) {
    using Amp = typename MultiShape<T>::Amp;
    constexpr int TH = MultiShape<T>::kThreads;
    const size_t smem = (size_t)MultiShape<T>::kPipe * 2 * (1 << M) * TH * sizeof(Amp);
    auto kern = k_adjoint_multi<T, M, S, P0>;
    static std::atomic<int> per_sm_of[64];   // per instantiation and device: blocks per SM, 0 = not set up
    static std::atomic<int> sms_of[64];
    int dev = 0;
    QI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return err(QI_ERR_UNSUPPORTED, dev, 64, "device ordinal");
    if (per_sm_of[dev].load() == 0) {
        QI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0, sms = 0;
        QI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TH, smem));
        QI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        sms_of[dev].store(std::max(sms, 1));
        per_sm_of[dev].store(std::max(per_sm, 1));
    }
    const uint64_t want = (mp.nwork + TH - 1) / TH;
    const uint64_t cap = std::min<uint64_t>((uint64_t)sms_of[dev].load() * per_sm_of[dev].load(),
                                            (uint64_t)kReduceBlocks * 4 / kMultiComps);
    const unsigned nb = (unsigned)std::max<uint64_t>(1, std::min(want, cap));
    kern<<<nb, TH, smem, s->stream>>>((Amp *)s->amps, (Amp *)lam->amps, mp, s->d_partials);
    *nb_out = nb;
    return check_launch("k_adjoint_multi");
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

// FP32 sweeps: the 2x2 matrix u (row-major complex, FP64) a stage un-applies, replaced by the
// FP32 values the kernel will use, chosen so that they form an exact multiple r of a unitary;
// returns r^2.  Entry-wise rounding keeps that form for the real, diagonal and reflection
// matrices of the gate set; otherwise u is first brought to SU(2) by a global phase (which
// cancels in <lambda|D|psi>, psi and lambda carrying the same phase) and a, b of
// [[a, -conj(b)], [b, conj(a)]] are rounded.  Un-applying then scales psi and lambda by
// exactly r, a deterministic drift of up to ~1e-7 per stage that the host divides out of
// the gradient instead of letting it accumulate over the sweep.
static double fp32_stage_matrix(double *u, std::complex<double> *phase = nullptr) {
    if (phase) *phase = 1.0;
    double f[8];
    for (int i = 0; i < 8; ++i) f[i] = (double)(float)u[i];
    auto dot = [&](int a, int b, double &re, double &im) {   // conj(col a) . col b
        re = f[2 * a] * f[2 * b] + f[2 * a + 1] * f[2 * b + 1] + f[2 * (a + 2)] * f[2 * (b + 2)] +
             f[2 * (a + 2) + 1] * f[2 * (b + 2) + 1];
        im = f[2 * a] * f[2 * b + 1] - f[2 * a + 1] * f[2 * b] + f[2 * (a + 2)] * f[2 * (b + 2) + 1] -
             f[2 * (a + 2) + 1] * f[2 * (b + 2)];
    };
    double c00, i00, c11, i11, c01r, c01i;
    dot(0, 0, c00, i00);
    dot(1, 1, c11, i11);
    dot(0, 1, c01r, c01i);
    if (c01r == 0.0 && c01i == 0.0 && std::fabs(c00 - c11) <= 1e-15 * c00) {
        std::copy(f, f + 8, u);
        return c00;
    }
    // det u = e^{i phi}; u e^{-i phi / 2} = [[a, -conj(b)], [b, conj(a)]]
    const std::complex<double> u00(u[0], u[1]), u01(u[2], u[3]), u10(u[4], u[5]), u11(u[6], u[7]);
    const std::complex<double> ph = std::exp(std::complex<double>(0.0, -0.5 * std::arg(u00 * u11 - u01 * u10)));
    const std::complex<double> a = u00 * ph, b = u10 * ph;
    if (phase) *phase = ph;
    const double ar = (float)a.real(), ai = (float)a.imag(), br = (float)b.real(), bi = (float)b.imag();
    u[0] = ar; u[1] = ai; u[2] = -br; u[3] = bi;
    u[4] = br; u[5] = bi; u[6] = ar; u[7] = -ai;
    return ar * ar + ai * ai + br * br + bi * bi;
}

}  // namespace qi

using namespace qi;

// Resolve parameters and build every gate's matrix (whole list first, as the entry point reports
// the first invalid gate before touching the state).
static Status resolve_adjoint_gates(int n, const qi_gate *gates, int64_t n_gates, const double *theta, int64_t n_theta,
                                    std::vector<qi_gate> &resolved, std::vector<GateMatrix> &mats) {
    resolved.assign((size_t)n_gates, qi_gate());
    mats.assign((size_t)n_gates, GateMatrix());
    for (int64_t j = 0; j < n_gates; ++j) {
        qi_gate g = gates[j];
        for (int k = 0; k < 3; ++k) {
            if (g.param_ids[k] >= 0) {
                if (!theta || g.param_ids[k] >= n_theta)
                    return err(QI_ERR_MISMATCHED_NUMBER_OF_PARAMETERS, g.param_ids[k] + 1, n_theta);
                if (!differentiable(g.kind)) return err(QI_ERR_UNSUPPORTED, g.kind, j, "gate kind has no parameter derivative");
                g.params[k] = theta[g.param_ids[k]];
            }
        }
        if (g.kind == QI_GATE_PAULI_STRING)
            return err(QI_ERR_UNSUPPORTED, j, -1, "a normalising Pauli-string gate has no inverse");
        if (g.kind == QI_GATE_MEASUREMENT)
            return err(QI_ERR_UNSUPPORTED, j, -1, "a measurement has no inverse");
        Status st = gate_to_matrix(n, g, &mats[(size_t)j]);
        if (!st.ok()) return st;
        resolved[(size_t)j] = g;
    }
    return ok_status();
}

// The reverse sweep as a list of passes, each over gates hi, hi - 1, ..., lo + 1:
//   kSweepGroup  single-qubit gates with at most one parameter, on at most kMultiQubits qubits
//                (kMultiQubits - 1 for FP64 states) with at most kMultiStages gates per qubit
//                (at least two gates): one k_adjoint_multi pass;
//   kSweepAffine fixed X / CNOT / SWAP gates (at least two that are not identities): one
//                k_affine_gather per state;
//   kSweepPlan   other fixed gates (at least two): one fused plan of their inverses per state;
//   kSweepSkip   fixed identities only;
//   kSweepGate   one gate on its own (k_adjoint, a per-gate un-apply or a Pauli exponential).
// Runs of fixed gates become plans or gathers only when fusion is on.
enum SweepKind : int32_t { kSweepGate = 0, kSweepGroup = 1, kSweepAffine = 2, kSweepPlan = 3, kSweepSkip = 4 };
struct SweepStep {
    int32_t kind;
    int64_t hi, lo;
};

static std::vector<SweepStep> plan_reverse_sweep(const std::vector<GateMatrix> &mats, const std::vector<qi_gate> &resolved,
                                                 bool f32, int fusion) {
    const int64_t n_gates = (int64_t)mats.size();
    auto n_params = [&](int64_t jj) {
        int c = 0;
        for (int k = 0; k < 3; ++k) c += resolved[(size_t)jj].param_ids[k] >= 0;
        return c;
    };
    auto groupable = [&](int64_t jj) {
        const GateMatrix &m = mats[(size_t)jj];
        return !m.pauli && m.nt == 1 && m.controls.empty() && n_params(jj) <= 1;
    };
    const int max_q = f32 ? kMultiQubits : kMultiQubits - 1;   // FP64 x 16 amplitudes spills
    // One group from gate j down, at most max_q qubits; returns the gate below it.
    auto take_group = [&](int64_t j) {
        int qcount[64] = {0};
        uint64_t qmask = 0;
        int64_t jj = j;
        for (; jj >= 0 && groupable(jj); --jj) {
            const int q = mats[(size_t)jj].t[0];
            if (!((qmask >> q) & 1ull) && __builtin_popcountll(qmask) == max_q) break;
            if (qcount[q] == kMultiStages) break;
            qmask |= 1ull << q;
            ++qcount[q];
        }
        return jj;
    };
    std::vector<SweepStep> steps;
    for (int64_t j = n_gates - 1; j >= 0;) {
        // (Putting a run's short group first, on the high qubits, so that the low qubits share a
        // full group, measured slower: a group on qubits 0-3 took 1.15 ms at 26 qubits against
        // 0.55 ms for qubits 0-1 and 0.42 ms for 2-5.)
        int64_t jj = take_group(j);
        if (j - jj >= 2) {
            steps.push_back({kSweepGroup, j, jj});
            j = jj;
            continue;
        }
        for (jj = j; jj >= 0 && n_params(jj) == 0; --jj) {}
        if (j - jj >= 2 && fusion != QI_FUSION_NONE) {
            int moves = 0;
            bool affine = true;
            for (int64_t k = j; k > jj; --k) {
                if (mats[(size_t)k].nt == 0 && !mats[(size_t)k].pauli) continue;
                affine = affine && affine_gate(mats[(size_t)k]);
                ++moves;
            }
            steps.push_back({moves == 0 ? kSweepSkip : (affine && moves >= 2) ? kSweepAffine : kSweepPlan, j, jj});
            j = jj;
            continue;
        }
        steps.push_back({kSweepGate, j, j - 1});
        --j;
    }
    return steps;
}

extern "C" qi_status qi_adjoint_sweep_plan(int32_t num_qubits, int32_t precision, const qi_gate *gates, int64_t n_gates,
                                           const double *theta, int64_t n_theta, const qi_exec_options *opts,
                                           int32_t *kinds, int64_t *hi, int64_t *lo, int64_t capacity,
                                           int64_t *n_steps) {
    if ((!gates && n_gates > 0) || !n_steps) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_qubits <= 0 || num_qubits > 40) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, num_qubits));
    if (precision != QI_F32 && precision != QI_F64) return publish(err(QI_ERR_INVALID_INPUT_VALUE, precision));
    std::vector<qi_gate> resolved;
    std::vector<GateMatrix> mats;
    Status st = resolve_adjoint_gates(num_qubits, gates, n_gates, theta, n_theta, resolved, mats);
    if (!st.ok()) return publish(st);
    const int fusion = opts ? opts->fusion : QI_FUSION_GREEDY;
    const std::vector<SweepStep> steps = plan_reverse_sweep(mats, resolved, precision == QI_F32, fusion);
    *n_steps = (int64_t)steps.size();
    if (kinds && hi && lo) {
        if (capacity < (int64_t)steps.size())
            return publish(err(QI_ERR_INVALID_INPUT_VALUE, capacity, (int64_t)steps.size()));
        for (size_t i = 0; i < steps.size(); ++i) {
            kinds[i] = steps[i].kind;
            hi[i] = steps[i].hi;
            lo[i] = steps[i].lo;
        }
    }
    return publish(ok_status());
}

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
    std::vector<qi_gate> resolved;
    std::vector<GateMatrix> mats;
    {
        Status st = resolve_adjoint_gates(n, gates, n_gates, theta, n_theta, resolved, mats);
        if (!st.ok()) return publish(st);
    }
    // forward sweep; the reverse sweep's fixed-gate segments use the same options.  FP32 states
    // fuse at most 5 qubits per block unless the caller chose: a 6-qubit tensor-core block sums
    // 48 truncating FP32 steps per amplitude (a 5-qubit one 24), and at 26 qubits that drift
    // alone took the gradient from 7e-7 to 1.3e-6 of the FP64 result.
    qi_exec_options plan_opts = {QI_FUSION_GREEDY, 0, 0, 0};
    if (forward_opts) plan_opts = *forward_opts;
    if (s->prec == QI_F32 && plan_opts.max_block_qubits <= 0) plan_opts.max_block_qubits = 5;
    // psi_0 stays untouched in the caller's buffer: the sweep runs on a copy (un-applying psi in
    // FP32 would hand back psi_0 with the sweep's rounding in it); without room for the copy it
    // runs in place and psi_0 is restored by the sweep itself.
    void *const psi_home = s->amps;
    void *work = nullptr;
    if (cudaMalloc(&work, s->bytes()) == cudaSuccess) {
        e = cudaMemcpyAsync(work, psi_home, s->bytes(), cudaMemcpyDeviceToDevice, s->stream);
        if (e != cudaSuccess) {
            cudaFree(work);
            return publish(cuda_status(e, "copy psi_0"));
        }
        s->amps = work;
    } else {
        work = nullptr;
        cudaGetLastError();
    }
    auto bail = [&](Status st) {   // before lambda exists: psi is in `work` (or in place)
        if (work) {
            cudaStreamSynchronize(s->stream);
            cudaFree(s->amps);
            s->amps = psi_home;
        }
        return publish(st);
    };
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
        if (!st.ok()) return bail(st);
    }
    // lambda = H psi, and E = <psi|lambda> (one read pass of two states with FP64 sums, in place of
    // one pass per X-mask group of H)
    qi_state *lam = nullptr;
    qi_status cs = qi_state_create(n, s->prec, &lam);
    if (cs != QI_OK) return bail(err(cs, -1, -1, "lambda state"));
    qi_state_set_stream(lam, s->stream);
    Status st = ok_status();
    double ev[2] = {0, 0};
    if (n_terms > 0) {
        st = sumop_apply(lam, s, terms, n_terms);
        if (st.ok()) st = state_inner(s, lam, ev);
        int flag = 0;
        if (st.ok()) st = state_read_flag(lam, &flag);
        if (st.ok() && flag == 2) st = err(QI_ERR_TIMEOUT, -1, -1, "SumOp::apply: a device wait timed out");
    } else {
        e = cudaMemsetAsync(lam->amps, 0, lam->bytes(), s->stream);
    }
    if (energy_out) *energy_out = ev[0];
    // derivative slots (one per parameter of a gate; a gate group uses one per member)
    const int64_t nslots = 3 * n_gates + kMultiComps;
    double *d_gres = nullptr;
    if (st.ok() && nslots > 0) {
        e = cudaMalloc(&d_gres, (size_t)nslots * sizeof(double));
        if (e != cudaSuccess) st = cuda_status(e, "cudaMalloc(gradient slots)");
    }
    struct SlotParam {
        int64_t slot;
        int32_t param;
        double factor;   // divides out the norm drift psi and lambda carried when the term was taken
    };
    std::vector<SlotParam> slot_param;
    int64_t slot = nslots;
    const bool f32 = s->prec == QI_F32;
    std::vector<std::unique_ptr<qi_plan>> seg_plans;   // kept until the sweep has run
    void *scratch = nullptr;          // third state buffer for affine gathers (rotates with psi, lambda)
    // Norm^2 of psi and lambda relative to where the sweep started (FP32 sweeps): exact stage
    // scales (fp32_stage_matrix) multiply in; after a tensor-core plan segment (which rounds
    // toward zero) both are measured.  A derivative term is divided by sqrt(cpsi * clam).
    double cpsi = 1.0, clam = 1.0, npsi0 = 1.0, nlam0 = 1.0;
    // (the exact-scale matrices may carry a global phase into psi: only when psi_0 is not the
    // state the sweep hands back)
    const bool scale_fix = f32 && work != nullptr;
    if (st.ok() && f32) st = state_reduce_norm_sqr(s, &npsi0);
    if (st.ok() && f32 && n_terms > 0) st = state_reduce_norm_sqr(lam, &nlam0);
    if (!(npsi0 > 0.0)) npsi0 = 1.0;
    if (!(nlam0 > 0.0)) nlam0 = 1.0;
    const std::vector<SweepStep> steps = plan_reverse_sweep(mats, resolved, f32, plan_opts.fusion);
    for (size_t si = 0; si < steps.size() && st.ok(); ++si) {
        const int64_t j = steps[si].hi, jj = steps[si].lo;
        const int32_t kind = steps[si].kind;
        if (kind == kSweepSkip) continue;
        if (kind == kSweepGroup) {   // gates j .. jj + 1: one k_adjoint_multi pass
            int qcount[64] = {0};
            uint64_t qmask = 0;
            for (int64_t k = j; k > jj; --k) {
                const int q = mats[(size_t)k].t[0];
                qmask |= 1ull << q;
                ++qcount[q];
            }
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
                for (int t = 0; t < kMultiStages; ++t) {
                    mp.uinv[i][t][0] = mp.uinv[i][t][6] = 1.0;   // identity, no derivative
                    mp.kind[i][t] = kStageDiag | kStageNoDeriv;
                }
            int used[64] = {0};
            std::vector<std::pair<int, int32_t>> comp_param;   // component -> parameter id
            double r2[kMultiQubits][kMultiStages];
            for (int i = 0; i < kMultiQubits; ++i)
                for (int t = 0; t < kMultiStages; ++t) r2[i][t] = 1.0;
            for (int64_t k = j; k > jj && st.ok(); --k) {
                const GateMatrix &gm = mats[(size_t)k];
                const qi_gate &g = resolved[(size_t)k];
                const int b = b_of[gm.t[0]], t = used[gm.t[0]]++;
                double *ui = mp.uinv[b][t], *dd = mp.d[b][t];
                inverse_matrix(gm, ui);
                double dU[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                bool has_d = false;
                for (int q = 0; q < 3; ++q)
                    if (g.param_ids[q] >= 0) {
                        st = derivative_matrix(n, g, q, dU);
                        comp_param.push_back({b * S + t, g.param_ids[q]});
                        has_d = true;
                    }
                // D = dU U^dagger: the derivative term on psi before it is un-applied
                for (int r = 0; r < 2; ++r)
                    for (int c = 0; c < 2; ++c) {
                        double re = 0, im = 0;
                        for (int m = 0; m < 2; ++m) {
                            const double ar = dU[2 * (2 * r + m)], ai = dU[2 * (2 * r + m) + 1];
                            const double br = ui[2 * (2 * m + c)], bi = ui[2 * (2 * m + c) + 1];
                            re += ar * br - ai * bi;
                            im += ar * bi + ai * br;
                        }
                        dd[2 * (2 * r + c)] = re;
                        dd[2 * (2 * r + c) + 1] = im;
                    }
                if (scale_fix) r2[b][t] = fp32_stage_matrix(ui);
                bool diag = true, real = true;
                for (int e = 0; e < 8; ++e) {
                    const bool off = e == 2 || e == 3 || e == 4 || e == 5;
                    if (off && (ui[e] != 0.0 || dd[e] != 0.0)) diag = false;
                    if ((e & 1) && (ui[e] != 0.0 || dd[e] != 0.0)) real = false;
                }
                mp.kind[b][t] = (int8_t)((diag ? kStageDiag : real ? kStageReal : kStageGeneral) |
                                         (has_d ? 0 : kStageNoDeriv));
            }
            if (!st.ok()) break;
            mp.nwork = 1ull << (n - M);
            unsigned nb = 1;
#define QI_AM(T, MM, SS)                                                                         \
    st = (sizeof(T) == 4 && mp.pos[0] == 0) ? launch_adjoint_multi<T, MM, SS, sizeof(T) == 4>(s, lam, mp, &nb) \
                                            : launch_adjoint_multi<T, MM, SS>(s, lam, mp, &nb)
#define QI_AM_S(T, MM) { if (S == 1) QI_AM(T, MM, 1); else QI_AM(T, MM, 2); }
            if (f32) {
                if (M == 1) QI_AM_S(float, 1) else if (M == 2) QI_AM_S(float, 2)
                else if (M == 3) QI_AM_S(float, 3) else QI_AM_S(float, 4)
            } else {
                if (M == 1) QI_AM_S(double, 1) else if (M == 2) QI_AM_S(double, 2) else QI_AM_S(double, 3)
            }
#undef QI_AM_S
#undef QI_AM
            if (!st.ok()) break;
            slot -= M * S;
            k_finalize_to<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, M * S, kMultiComps, d_gres + slot);
            count_launch(2);
            st = check_launch("k_finalize_to");
            // the kernel runs qubit by qubit (mp.pos order), each qubit's stages in order: a
            // stage's term sees every scale applied before it in that order
            double fac[kMultiComps];
            for (int i = 0; i < M; ++i)
                for (int t = 0; t < S; ++t) {
                    fac[i * S + t] = 1.0 / std::sqrt(cpsi * clam);
                    cpsi *= r2[i][t];
                    clam *= r2[i][t];
                }
            for (auto &cp : comp_param) slot_param.push_back({slot + cp.first, cp.second, fac[cp.first]});
            continue;
        }
        bool as_plan = kind == kSweepPlan;
        if (kind == kSweepAffine) {
            // X / CNOT / SWAP only: one index permutation per state, out[x] = in[f(x)] with f the
            // run's forward map (gathering through f un-applies the run)
            if (!scratch && cudaMalloc(&scratch, s->bytes()) != cudaSuccess) {
                scratch = nullptr;
                cudaGetLastError();   // no room for a third state buffer: un-apply the run as a plan
                as_plan = true;
            } else {
                AffineMap am;
                affine_identity(am);
                for (int64_t k = jj + 1; k <= j; ++k)
                    if (mats[(size_t)k].nt != 0) affine_compose(am, mats[(size_t)k]);
                for (qi_state *q : {s, lam}) {
                    st = affine_gather_async(s, scratch, q->amps, am);
                    if (!st.ok()) break;
                    std::swap(q->amps, scratch);
                }
                continue;
            }
        }
        if (as_plan) {   // fixed gates: their inverses as one fused plan on psi and lambda
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
            if (inv.empty()) continue;   // identities only (planned as kSweepSkip)
            std::unique_ptr<qi_plan> seg(new qi_plan());
            seg->n = n;
            seg->prec = s->prec;
            seg->opts = plan_opts;
            seg->opts.renorm_every = -1;   // lambda = H psi is not a unit vector
            st = build_plan(seg.get(), inv);
            if (st.ok()) st = upload_plan(seg.get());
            if (st.ok()) st = plan_execute(seg.get(), s);
            if (st.ok()) st = plan_execute(seg.get(), lam);
            if (st.ok() && f32 && !seg->tc.empty()) {   // tensor-core blocks: measure the drift
                double a = 0.0, b = 0.0;
                st = state_reduce_norm_sqr(s, &a);
                if (st.ok()) st = state_reduce_norm_sqr(lam, &b);
                if (st.ok()) {
                    cpsi = a / npsi0;
                    if (n_terms > 0) clam = b / nlam0;
                }
            }
            seg_plans.push_back(std::move(seg));
            continue;
        }
        // kSweepGate: gate j on its own
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
        // an uncontrolled single-qubit stage scales both states by exactly r (FP32); the term
        // uses psi after the un-apply and lambda before it, so a global phase ph taken into
        // U^dagger is taken out of dU (conj(ph) dU U^dagger ph = dU U^dagger)
        double r2g = 1.0;
        if (scale_fix && gm.nt == 1 && cm == 0) {
            std::complex<double> ph;
            r2g = fp32_stage_matrix(p.uinv, &ph);
            for (int q = 0; q < nd; ++q)
                for (int e2 = 0; e2 < 4; ++e2) {
                    const std::complex<double> v = std::complex<double>(p.d[q][2 * e2], p.d[q][2 * e2 + 1]) * std::conj(ph);
                    p.d[q][2 * e2] = v.real();
                    p.d[q][2 * e2 + 1] = v.imag();
                }
        }
        const double facg = 1.0 / std::sqrt(cpsi * r2g * clam);
        cpsi *= r2g;
        clam *= r2g;
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
        for (int q = 0; q < nd; ++q) slot_param.push_back({slot + q, g.param_ids[ids[q]], facg});
    }
    if (st.ok()) {
        for (int64_t k = 0; k < n_theta; ++k) grads_out[k] = 0.0;
        std::vector<double> h((size_t)nslots, 0.0);
        if (nslots > 0) e = cudaMemcpyAsync(h.data(), d_gres, (size_t)nslots * sizeof(double), cudaMemcpyDeviceToHost,
                                            s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) st = cuda_status(e, "adjoint");
        for (auto &sp : slot_param) grads_out[sp.param] += 2.0 * h[(size_t)sp.slot] * sp.factor;
    }
    cudaStreamSynchronize(s->stream);
    if (work) {   // psi_0 never left the caller's buffer; psi ends in one of the sweep's buffers
        cudaFree(s->amps);
        s->amps = psi_home;
    } else if (s->amps != psi_home) {   // psi_home is lambda's or the scratch buffer now
        e = cudaMemcpyAsync(psi_home, s->amps, s->bytes(), cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess && st.ok()) st = cuda_status(e, "restore psi buffer");
        if (lam->amps == psi_home) lam->amps = s->amps;
        else scratch = s->amps;
        s->amps = psi_home;
    }
    if (scratch) cudaFree(scratch);
    for (auto &sp : seg_plans) {
        if (sp->d_mats) cudaFree(sp->d_mats);
        if (sp->d_tc) cudaFree(sp->d_tc);
    }
    if (d_gres) cudaFree(d_gres);
    qi_state_destroy(lam);
    return publish(st);
}
