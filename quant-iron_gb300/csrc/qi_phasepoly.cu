// qi_phasepoly.cu — a run of diagonal blocks applied as one phase polynomial.
//
// Every diagonal gate of the gate set whose phases are a polynomial of degree
// <= 2 in the index bits (Z, S, T, P, RZ and their adjoints, CZ / controlled
// phase with one control, identity) multiplies amplitude x by exp(2 pi i f(x)),
//   f(x) = c0 + sum_q a[q] x_q + sum_{q<r} b[q][r] x_q x_r      (turns),
// and a product of such gates adds their polynomials.  The planner folds a run
// of consecutive diagonal blocks (for example the controlled-phase ladders of
// a quantum Fourier transform, which split into many 6-qubit tables) into one
// polynomial and applies it in a single pass over the state, whatever the
// number of qubits the run touches.
//
// Coefficients are fixed-point turns: 2^64 units (host) or 2^32 units (the
// FP32 kernel) per turn, so sums wrap modulo 2 pi exactly.  A table's
// polynomial comes from the Moebius transform over subsets of its qubits of
// the entries' angles: the coefficient of a subset S is
// sum_{T subset S} (-1)^{|S|-|T|} angle(T); the table is accepted if every
// coefficient of degree >= 3 vanishes (to 2^-50 turns) and |entry| = 1.
//
// Kernel (FP32 states): the 2^(n-1) amplitude pairs are split as
// pair = it * 2^m + tid with 2^m threads and 2^h iterations per thread.  Per
// thread, the terms of f that involve only its own index bits (and the
// cross terms with each iteration bit, gam[k]) are summed once; per
// iteration, f = F + G0[it] + sum_k it_k gam[k], where the host table G0
// holds c0 plus the terms among iteration bits, and the odd amplitude of the
// pair adds P0 + G1[it] (the terms of qubit 0).  exp(2 pi i f) = T1[f >> 22]
// * exp(i x) with x the remaining 22 bits as an angle (< 2 pi / 1024), from
// T1 = exp(2 pi i j / 1024) (1024 entries, rounded from FP64 on the host) and
// the Taylor polynomials of sin and cos to x^5 and x^4 (remainder < 1e-16).
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <cmath>

namespace qi {

constexpr int kPolyThreads = 256, kPolyMaxH = 12, kPolyUnroll = 8;

static uint64_t turns64(double angle_rad) {
    double t = angle_rad / (2.0 * M_PI);          // (-0.5, 0.5]
    double sc = t * 18446744073709551616.0;       // 2^64
    if (sc >= 9223372036854775808.0) sc -= 18446744073709551616.0;
    if (sc < -9223372036854775808.0) sc += 18446744073709551616.0;
    sc = std::nearbyint(sc);
    if (sc >= 9223372036854775808.0) return 1ull << 63;
    return (uint64_t)(int64_t)sc;
}

static uint32_t round32(uint64_t v) { return (uint32_t)((v + 0x80000000ull) >> 32); }

bool phase_poly_add_table(PhasePoly &pp, int k, const int32_t *qubits, const std::complex<double> *phases) {
    if (k < 0 || k > 16) return false;
    const int dim = 1 << k;
    std::vector<uint64_t> c((size_t)dim);
    for (int x = 0; x < dim; ++x) {
        const std::complex<double> d = phases[x];
        if (std::fabs(std::abs(d) - 1.0) > 1e-9) return false;
        c[(size_t)x] = turns64(std::atan2(d.imag(), d.real()));
    }
    for (int j = 0; j < k; ++j)   // Moebius transform over subsets (wrapping arithmetic)
        for (int x = 0; x < dim; ++x)
            if ((x >> j) & 1) c[(size_t)x] -= c[(size_t)(x ^ (1 << j))];
    for (int x = 0; x < dim; ++x) {
        if (__builtin_popcount((unsigned)x) < 3) continue;
        const int64_t v = (int64_t)c[(size_t)x];
        if (v > (1ll << 14) || v < -(1ll << 14)) return false;
    }
    for (int j = 0; j < k; ++j)
        if (qubits[j] < 0 || qubits[j] >= pp.n) return false;
    pp.c0 += c[0];
    for (int j = 0; j < k; ++j) {
        pp.a[(size_t)qubits[j]] += c[(size_t)1 << j];
        for (int l = j + 1; l < k; ++l) {
            const int q = std::min(qubits[j], qubits[l]), r = std::max(qubits[j], qubits[l]);
            pp.b[(size_t)q * pp.n + r] += c[((size_t)1 << j) | ((size_t)1 << l)];
        }
    }
    return true;
}

// Threads 2^m and iterations 2^h with m + h = n - 1 (amplitude pairs).
int phase_poly_iter_bits(int n) {
    const int pairs = n - 1;
    int m = std::min(pairs, 19);
    int h = pairs - m;
    if (h > kPolyMaxH) h = kPolyMaxH;
    return h;
}

void phase_poly_device_block(const PhasePoly &pp, std::vector<float> &out) {
    const int n = pp.n, h = phase_poly_iter_bits(n), m = n - 1 - h;
    const size_t words = (size_t)kPolyG0 + 2 * ((size_t)1 << h);
    std::vector<uint32_t> w(words, 0);
    for (int q = 0; q < n; ++q) w[kPolyA + q] = round32(pp.a[(size_t)q]);
    for (int q = 0; q < n; ++q)
        for (int r = q + 1; r < n; ++r) {
            const uint32_t v = round32(pp.b[(size_t)q * n + r]);
            w[kPolyB + q * 64 + r] = v;
            w[kPolyB + r * 64 + q] = v;
        }
    for (int j = 0; j < 1024; ++j) {
        const float cr = (float)std::cos(2.0 * M_PI * j / 1024.0), ci = (float)std::sin(2.0 * M_PI * j / 1024.0);
        std::memcpy(&w[kPolyT1 + 2 * j], &cr, 4);
        std::memcpy(&w[kPolyT1 + 2 * j + 1], &ci, 4);
    }
    // G0[it] = c0 + terms among the iteration qubits m+1+k; G1[it] = terms of qubit 0 with them
    const uint32_t iters = 1u << h;
    std::vector<uint64_t> g0(iters), g1(iters);
    g0[0] = pp.c0;
    g1[0] = 0;
    for (uint32_t it = 1; it < iters; ++it) {
        const int top = 31 - __builtin_clz(it);
        const uint32_t rest = it & ~(1u << top);
        const int qt = m + 1 + top;
        uint64_t v = g0[rest] + pp.a[(size_t)qt];
        for (int k = 0; k < top; ++k)
            if ((rest >> k) & 1u) v += pp.b[(size_t)(m + 1 + k) * n + qt];
        g0[it] = v;
        g1[it] = g1[rest] + (n > 1 ? pp.b[(size_t)0 * n + qt] : 0);
    }
    for (uint32_t it = 0; it < iters; ++it) {
        w[kPolyG0 + it] = round32(g0[it]);
        w[kPolyG0 + iters + it] = round32(g1[it]);
    }
    const size_t base = out.size();
    const size_t padded = (words + 3) & ~(size_t)3;
    out.resize(base + padded, 0.0f);
    std::memcpy(out.data() + base, w.data(), words * 4);
}

__global__ void __launch_bounds__(kPolyThreads) k_phase_poly(float4 *v, const uint32_t *blk, int m, int h) {
    __shared__ float2 T1[1024];
    {
        const float2 *g = reinterpret_cast<const float2 *>(blk + kPolyT1);
        for (int i = threadIdx.x; i < 1024; i += blockDim.x) T1[i] = g[i];
    }
    __syncthreads();
    const uint32_t *a = blk + kPolyA, *b = blk + kPolyB, *G0 = blk + kPolyG0, *G1 = G0 + (1u << h);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;   // amplitude bits 1..m
    uint32_t F = 0, P0 = a[0], gam[kPolyMaxH];
#pragma unroll
    for (int k = 0; k < kPolyMaxH; ++k) gam[k] = 0;
    for (int j = 1; j <= m; ++j) {
        if (!((tid >> (j - 1)) & 1u)) continue;
        F += a[j];
        P0 += b[j];   // b[0][j]
        for (int l = j + 1; l <= m; ++l)
            if ((tid >> (l - 1)) & 1u) F += b[j * 64 + l];
#pragma unroll
        for (int k = 0; k < kPolyMaxH; ++k)
            if (k < h) gam[k] += b[j * 64 + m + 1 + k];
    }
    // cross terms of the low log2(kPolyUnroll) iteration bits, one value per unrolled slot
    uint32_t low[kPolyUnroll];
#pragma unroll
    for (int u = 0; u < kPolyUnroll; ++u) {
        low[u] = 0;
#pragma unroll
        for (int k = 0; (1 << k) < kPolyUnroll; ++k)
            if (k < h && ((u >> k) & 1)) low[u] += gam[k];
    }
    const uint32_t iters = 1u << h;
    for (uint32_t it0 = 0; it0 < iters; it0 += kPolyUnroll) {
        float4 x[kPolyUnroll];
#pragma unroll
        for (int u = 0; u < kPolyUnroll; ++u)
            if (it0 + u < iters) x[u] = __ldcs(v + (((uint64_t)(it0 + u) << m) | tid));
        // cross terms of the remaining iteration bits, once per group of kPolyUnroll
        uint32_t base = F;
#pragma unroll
        for (int k = 0; k < kPolyMaxH; ++k)
            if ((1 << k) >= kPolyUnroll && k < h && ((it0 >> k) & 1u)) base += gam[k];
#pragma unroll
        for (int u = 0; u < kPolyUnroll; ++u) {
            const uint32_t it = it0 + u;
            if (it >= iters) break;
            const uint32_t f = base + low[u] + __ldg(G0 + it);
            const uint32_t f1 = f + P0 + __ldg(G1 + it);
            const float2 p0 = turn_phase(f, T1), p1 = turn_phase(f1, T1);
            float4 y;
            y.x = x[u].x * p0.x - x[u].y * p0.y;
            y.y = x[u].x * p0.y + x[u].y * p0.x;
            y.z = x[u].z * p1.x - x[u].w * p1.y;
            y.w = x[u].z * p1.y + x[u].w * p1.x;
            __stcs(v + (((uint64_t)it << m) | tid), y);
        }
    }
}

Status launch_phase_poly(qi_state *s, const void *d_block) {
    if (s->prec != QI_F32) return err(QI_ERR_UNSUPPORTED, s->prec, -1, "phase polynomial kernel is FP32");
    if (!d_block || ((uintptr_t)d_block & 15) != 0) return err(QI_ERR_UNKNOWN, -1, -1, "phase polynomial block");
    const int n = s->n;
    if (n < 1 || n > 63) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, n);
    const int h = phase_poly_iter_bits(n), m = n - 1 - h;
    const uint64_t threads = 1ull << m;
    const unsigned tpb = (unsigned)std::min<uint64_t>(threads, kPolyThreads);
    const uint64_t blocks = threads / tpb;
    k_phase_poly<<<(unsigned)blocks, tpb, 0, s->stream>>>((float4 *)s->amps, (const uint32_t *)d_block, m, h);
    count_launch();
    return check_launch("k_phase_poly");
}

}  // namespace qi
