// qi_pauli.cu — Pauli-string kernels: exp(alpha P) in one pass, P|psi>,
// SumOp apply and SumOp expectation grouped by X-mask, Trotter evolution.
//
// Reference: src/components/pauli_string.rs (apply :139-151, apply_exp_factor
// :237-262, SumOp::apply :453-466, expectation_value :485-507) and
// src/algorithms/time_evolution.rs:45-166.
//
// For a Pauli string with X-or-Y qubits xmask, Z-or-Y qubits zmask and ny Y
// factors, (P psi)_i = (-i)^ny (-1)^popcount(i & zmask) psi_{i ^ xmask}.
// The reference applies each single-qubit Pauli as a full pass and builds
// cosh(a) psi + sinh(a) P psi from three state vectors; here one pass reads
// the pair (i, i ^ xmask) and writes both outputs.
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_async.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <type_traits>
#include <vector>

namespace qi {

// (-i)^ny as (re, im)
static inline void minus_i_pow(int ny, double &re, double &im) {
    switch (ny & 3) {
    case 0: re = 1; im = 0; break;
    case 1: re = 0; im = -1; break;
    case 2: re = -1; im = 0; break;
    default: re = 0; im = 1; break;
    }
}

struct ExpParams {
    uint64_t nwork;
    uint64_t xmask, zmask;
    uint64_t hbit;     // highest bit of xmask (pair enumeration), 0 if xmask == 0
    int32_t hpos;
    int32_t swap_halves;   // VEC: xmask bit 0 set -> partner float4 halves are swapped
    double cre, cim;   // cosh(alpha)
    double sre, sim;   // sinh(alpha) * (-i)^ny
};

// Amplitudes (or pairs) a thread keeps in flight per loop step: one load per
// step leaves too few bytes in flight to cover HBM latency at full occupancy.
template <typename T> struct Unroll { static constexpr int kDiag = 8, kPair = 2; };
template <> struct Unroll<double> { static constexpr int kDiag = 4, kPair = 2; };

// Diagonal case (xmask == 0): psi_i *= cosh + sinh * (-1)^popc(i & z).  The two
// factors arrive in the state's precision: computed in the kernel from the FP64
// coefficients, the compiler may move the FP64 add and conversion into the
// per-amplitude select, which makes the FP32 kernel FP64-bound on this part.
template <typename T>
__global__ void __launch_bounds__(256) k_pauli_exp_diag(typename Cx<T>::V2 *a, uint64_t nwork, uint64_t zmask,
                                                        typename Cx<T>::V2 plus, typename Cx<T>::V2 minus) {
    using X = Cx<T>;
    constexpr int U = Unroll<T>::kDiag;
    const uint64_t step = (uint64_t)blockDim.x, stride = (uint64_t)gridDim.x * blockDim.x * U;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x * U + threadIdx.x; base < nwork; base += stride) {
        typename X::V2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < nwork) v[u] = a[base + u * step];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = base + u * step;
            if (i < nwork) a[i] = X::mul((__popcll(i & zmask) & 1) ? minus : plus, v[u]);
        }
    }
}

// FP64 pair case for exp(-i theta P) with a real coefficient: c = cos(theta) is
// real and s is real (SIMAG = false) or imaginary (SIMAG = true), so each output
// costs 4 FP64 operations instead of 8 (FP64 arithmetic bounds this kernel here).
template <bool SIMAG>
__global__ void __launch_bounds__(256) k_pauli_exp_pair_real64(double2 *a, ExpParams p) {
    constexpr int U = Unroll<double>::kPair;
    const double c = p.cre, s = SIMAG ? p.sim : p.sre;
    const uint64_t step = (uint64_t)blockDim.x, stride = (uint64_t)gridDim.x * blockDim.x * U;
    const uint64_t lo_mask = p.hbit - 1;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x * U + threadIdx.x; base < p.nwork; base += stride) {
        double2 x[U], y[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t w = base + u * step;
            if (w < p.nwork) {
                const uint64_t i = ((w & ~lo_mask) << 1) | (w & lo_mask);
                x[u] = a[i];
                y[u] = a[i ^ p.xmask];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t w = base + u * step;
            if (w >= p.nwork) continue;
            const uint64_t i = ((w & ~lo_mask) << 1) | (w & lo_mask), j = i ^ p.xmask;
            const double si = (__popcll(i & p.zmask) & 1) ? -s : s, sj = (__popcll(j & p.zmask) & 1) ? -s : s;
            if (SIMAG) {   // c x + i s y
                a[i] = make_double2(::fma(-si, y[u].y, c * x[u].x), ::fma(si, y[u].x, c * x[u].y));
                a[j] = make_double2(::fma(-sj, x[u].y, c * y[u].x), ::fma(sj, x[u].x, c * y[u].y));
            } else {       // c x + s y
                a[i] = make_double2(::fma(si, y[u].x, c * x[u].x), ::fma(si, y[u].y, c * x[u].y));
                a[j] = make_double2(::fma(sj, x[u].x, c * y[u].x), ::fma(sj, x[u].y, c * y[u].y));
            }
        }
    }
}

// Pair case: i with bit hpos clear, j = i ^ xmask.
//   new_i = c psi_i + s (-1)^popc(i&z) psi_j,  new_j = c psi_j + s (-1)^popc(j&z) psi_i
template <typename T, bool VEC>
__global__ void __launch_bounds__(256) k_pauli_exp_pair(typename Cx<T>::V2 *a, ExpParams p) {
    using X = Cx<T>;
    const typename X::V2 c = X::make((T)p.cre, (T)p.cim);
    const typename X::V2 s = X::make((T)p.sre, (T)p.sim);
    const typename X::V2 sn = X::make((T)-p.sre, (T)-p.sim);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t lo_mask = p.hbit - 1;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < p.nwork; w += stride) {
        const uint64_t ww = VEC ? (w << 1) : w;
        const uint64_t i = ((ww & ~lo_mask) << 1) | (ww & lo_mask);
        const uint64_t j = i ^ p.xmask;
        if constexpr (VEC) {
            // i even; the partner pair (j, j^1) lives in float4 j >> 1
            float4 *a4 = reinterpret_cast<float4 *>(a);
            float4 u = a4[i >> 1], v = a4[j >> 1];
            float2 i0 = make_float2(u.x, u.y), i1 = make_float2(u.z, u.w);
            float2 j0 = make_float2(v.x, v.y), j1 = make_float2(v.z, v.w);
            if (p.swap_halves) { float2 t = j0; j0 = j1; j1 = t; }   // j0 = psi_{i ^ x}, j1 = psi_{(i+1) ^ x}
            const uint64_t ja = j, jb = j ^ 1ull;   // partners of i and i+1
            float2 ni0 = X::fma((__popcll(i & p.zmask) & 1) ? sn : s, j0, X::mul(c, i0));
            float2 ni1 = X::fma((__popcll((i + 1) & p.zmask) & 1) ? sn : s, j1, X::mul(c, i1));
            float2 nj0 = X::fma((__popcll(ja & p.zmask) & 1) ? sn : s, i0, X::mul(c, j0));
            float2 nj1 = X::fma((__popcll(jb & p.zmask) & 1) ? sn : s, i1, X::mul(c, j1));
            if (p.swap_halves) { float2 t = nj0; nj0 = nj1; nj1 = t; }
            a4[i >> 1] = make_float4(ni0.x, ni0.y, ni1.x, ni1.y);
            a4[j >> 1] = make_float4(nj0.x, nj0.y, nj1.x, nj1.y);
        } else {
            typename X::V2 x = a[i], y = a[j];
            a[i] = X::fma((__popcll(i & p.zmask) & 1) ? sn : s, y, X::mul(c, x));
            a[j] = X::fma((__popcll(j & p.zmask) & 1) ? sn : s, x, X::mul(c, y));
        }
    }
}

// out_i = coeff * (-i)^ny (-1)^popc(i&z) in_{i ^ x}   (PauliString::apply, out of place)
template <typename T>
__global__ void __launch_bounds__(256) k_pauli_gather(typename Cx<T>::V2 *o, const typename Cx<T>::V2 *in, uint64_t dim,
                                                      uint64_t xmask, uint64_t zmask, double fre, double fim) {
    using X = Cx<T>;
    const typename X::V2 f = X::make((T)fre, (T)fim), fn = X::make((T)-fre, (T)-fim);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride)
        o[i] = X::mul((__popcll(i & zmask) & 1) ? fn : f, in[i ^ xmask]);
}

// ------------------------------------------------------------------------
// Grouped exponentials (OP_PAULI_GROUP).  A run of exponentials whose X-masks
// all lie in {0, X} maps each pair (i0, i1 = i0 ^ X) (each amplitude, X = 0)
// to itself, and every factor depends on i0 only through the parities
// popc(i0 & z_k) & 1.  Those parities are XORs of r basis parities
// beta_j = popc(i0 & w_j) & 1, so the whole run is one 2x2 matrix (one
// factor) per beta in [0, 2^r): a table built on the host, applied in one
// pass.  Diagonal runs split into up to kGroupChunks tables (factors commute).
struct GroupParams {
    uint64_t nwork;            // amplitudes (diagonal) or pairs
    uint64_t xmask, lo_mask;   // pair groups: partner mask; bits below its highest bit
    int32_t nchunk, ntab;      // tables and their total entries (complex)
    int32_t nbytes;            // index bytes (ceil(n / 8))
    int32_t rank[kGroupChunks];
    int32_t off[kGroupChunks];
    uint64_t basis[kGroupChunks * kGroupRank];
};

// Parities are a GF(2)-linear map of the index, so they are gathered per index
// byte: ptab[b][v] packs, at bit 8c + j, the parity of (v << 8b) & basis[c][j];
// the parities of i are the XOR of ptab[b][byte b of i] over its bytes.
constexpr int kParityBytes = 5;   // indices up to 40 bits

__device__ __forceinline__ void build_parity_bytes(uint32_t *ptab, const GroupParams &p) {
    for (int e = threadIdx.x; e < p.nbytes * 256; e += blockDim.x) {
        const uint64_t v = (uint64_t)(e & 255) << (8 * (e >> 8));
        uint32_t word = 0;
        for (int c = 0; c < p.nchunk; ++c)
            for (int j = 0; j < p.rank[c]; ++j)
                word |= (uint32_t)(__popcll(v & p.basis[c * kGroupRank + j]) & 1) << (8 * c + j);
        ptab[e] = word;
    }
}

template <typename IDX>
__device__ __forceinline__ uint32_t parity_word(IDX i, const uint32_t *ptab, int nbytes) {
    uint32_t word = ptab[(uint32_t)i & 255u];
#pragma unroll
    for (int b = 1; b < kParityBytes; ++b)
        if (b < nbytes) word ^= ptab[b * 256 + (uint32_t)(((uint64_t)i >> (8 * b)) & 255u)];
    return word;
}

template <typename T, typename IDX>
__global__ void __launch_bounds__(256) k_pauli_group_diag(typename Cx<T>::V2 *a, const __grid_constant__ GroupParams p,
                                                          const typename Cx<T>::V2 *tab) {
    using X = Cx<T>;
    constexpr int U = Unroll<T>::kDiag;
    __shared__ typename X::V2 st[kGroupChunks << kGroupRank];
    __shared__ uint32_t ptab[kParityBytes * 256];
    for (int k = threadIdx.x; k < p.ntab; k += blockDim.x) st[k] = tab[k];
    build_parity_bytes(ptab, p);
    __syncthreads();
    const IDX nwork = (IDX)p.nwork, step = (IDX)blockDim.x, stride = (IDX)gridDim.x * blockDim.x * U;
    for (IDX base = (IDX)blockIdx.x * blockDim.x * U + threadIdx.x; base < nwork; base += stride) {
        typename X::V2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (base + u * step < nwork) v[u] = a[base + u * step];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const IDX i = base + u * step;
            if (i >= nwork) continue;
            const uint32_t word = parity_word(i, ptab, p.nbytes);
            typename X::V2 f = st[word & 255u];
            for (int c = 1; c < p.nchunk; ++c) f = X::mul(f, st[p.off[c] + ((word >> (8 * c)) & 255u)]);
            a[i] = X::mul(f, v[u]);
        }
    }
}

// Pair groups: table entry beta holds (m00, m01, m10, m11); new (psi_i0, psi_i1) = M (psi_i0, psi_i1).
template <typename T, typename IDX>
__global__ void __launch_bounds__(256) k_pauli_group_pair(typename Cx<T>::V2 *a, const __grid_constant__ GroupParams p,
                                                          const typename Cx<T>::V2 *tab) {
    using X = Cx<T>;
    constexpr int U = Unroll<T>::kPair;
    __shared__ typename X::V2 st[4 << kPairRank];
    __shared__ uint32_t ptab[kParityBytes * 256];
    for (int k = threadIdx.x; k < p.ntab; k += blockDim.x) st[k] = tab[k];
    build_parity_bytes(ptab, p);
    __syncthreads();
    const IDX nwork = (IDX)p.nwork, step = (IDX)blockDim.x, stride = (IDX)gridDim.x * blockDim.x * U;
    const IDX lo = (IDX)p.lo_mask, xm = (IDX)p.xmask;
    for (IDX base = (IDX)blockIdx.x * blockDim.x * U + threadIdx.x; base < nwork; base += stride) {
        typename X::V2 x[U], y[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const IDX w = base + u * step;
            if (w < nwork) {
                const IDX i = ((w & ~lo) << 1) | (w & lo);
                x[u] = a[i];
                y[u] = a[i ^ xm];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const IDX w = base + u * step;
            if (w >= nwork) continue;
            const IDX i = ((w & ~lo) << 1) | (w & lo);
            const typename X::V2 *m = st + 4 * parity_word(i, ptab, p.nbytes);
            a[i] = X::fma(m[1], y[u], X::mul(m[0], x[u]));
            a[i ^ xm] = X::fma(m[3], y[u], X::mul(m[2], x[u]));
        }
    }
}

static unsigned pgrid(uint64_t work) {
    uint64_t g = (work + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152 * 8) g = 152 * 8;
    return (unsigned)g;
}

Status launch_pauli_exp(qi_state *s, uint64_t xmask, uint64_t zmask, double cre, double cim, double sre, double sim) {
    ExpParams p;
    std::memset(&p, 0, sizeof(p));
    p.xmask = xmask;
    p.zmask = zmask;
    double pr, pi;
    minus_i_pow(__builtin_popcountll(xmask & zmask), pr, pi);
    p.cre = cre; p.cim = cim;
    p.sre = sre * pr - sim * pi;
    p.sim = sre * pi + sim * pr;
    const bool f32 = s->prec == QI_F32;
    if (xmask == 0) {
        p.nwork = s->dim();
        unsigned g = pgrid(p.nwork);
        const double pr = p.cre + p.sre, pi = p.cim + p.sim, mr = p.cre - p.sre, mi = p.cim - p.sim;
        if (f32)
            k_pauli_exp_diag<float><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p.nwork, zmask,
                                                              make_float2((float)pr, (float)pi),
                                                              make_float2((float)mr, (float)mi));
        else
            k_pauli_exp_diag<double><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p.nwork, zmask,
                                                               make_double2(pr, pi), make_double2(mr, mi));
        count_launch();
        return check_launch("k_pauli_exp_diag");
    }
    int h = 63 - __builtin_clzll(xmask);
    p.hpos = h;
    p.hbit = 1ull << h;
    const bool vec = f32 && h >= 1 && s->n >= 2;
    p.swap_halves = (xmask & 1ull) ? 1 : 0;
    p.nwork = s->dim() >> (vec ? 2 : 1);
    unsigned g = pgrid(p.nwork);
    if (f32) {
        if (vec) k_pauli_exp_pair<float, true><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
        else k_pauli_exp_pair<float, false><<<g, 256, 0, s->stream>>>((float2 *)s->amps, p);
    } else if (p.cim == 0.0 && p.sre == 0.0) {
        k_pauli_exp_pair_real64<true><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p);
    } else if (p.cim == 0.0 && p.sim == 0.0) {
        k_pauli_exp_pair_real64<false><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p);
    } else {
        k_pauli_exp_pair<double, false><<<g, 256, 0, s->stream>>>((double2 *)s->amps, p);
    }
    count_launch();
    return check_launch("k_pauli_exp_pair");
}

// GF(2) basis of parity masks: each placed mask is the XOR of a subset of the
// basis masks w[j] (kept with a row-echelon copy for the reduction).
struct ParityBasis {
    int r = 0;
    uint64_t w[kGroupRank] = {0}, ech[kGroupRank] = {0};
    uint32_t comb[kGroupRank] = {0};
    int piv[kGroupRank] = {0};
    // subset of w whose XOR is z; adds z as a basis mask when independent and r < cap
    bool place(uint64_t z, int cap, uint32_t *subset) {
        uint32_t c = 0;
        uint64_t v = z;
        for (int j = 0; j < r; ++j)
            if ((v >> piv[j]) & 1ull) { v ^= ech[j]; c ^= comb[j]; }
        if (v == 0) { *subset = c; return true; }
        if (r >= cap) return false;
        piv[r] = 63 - __builtin_clzll(v);
        ech[r] = v;
        comb[r] = c ^ (1u << r);
        w[r] = z;
        *subset = 1u << r;
        ++r;
        return true;
    }
};

using cd = std::complex<double>;

// cosh(alpha) and sinh(alpha) * (-i)^ny of exp(alpha P) (the factors launch_pauli_exp uses)
static void exp_factors(const GateMatrix &g, cd *ch, cd *sh) {
    const double ar = g.alpha_re, ai = g.alpha_im;
    *ch = cd(std::cosh(ar) * std::cos(ai), std::sinh(ar) * std::sin(ai));
    double pr, pi;
    minus_i_pow(__builtin_popcountll(g.xmask & g.zmask), pr, pi);
    *sh = cd(std::sinh(ar) * std::cos(ai), std::cosh(ar) * std::sin(ai)) * cd(pr, pi);
}

size_t pauli_group_op(const std::vector<const GateMatrix *> &run, size_t start, Op &op, std::vector<cd> &mats) {
    const GateMatrix &g0 = *run[start];
    std::vector<std::pair<size_t, uint32_t>> members;   // (term, subset of basis parities), application order
    if (g0.xmask == 0) {
        // diagonal run: factors commute, so each term joins any table that can index it
        ParityBasis chunk[kGroupChunks];
        std::vector<int> which;
        int nchunk = 0;
        size_t k = start;
        for (; k < run.size() && run[k]->xmask == 0; ++k) {
            uint32_t sub = 0;
            int c = 0;
            for (; c < nchunk; ++c)   // a table that indexes the term without a new basis mask
                if (chunk[c].place(run[k]->zmask, chunk[c].r, &sub)) break;
            if (c == nchunk) {        // else the first table with room for one
                for (c = 0; c < nchunk; ++c)
                    if (chunk[c].place(run[k]->zmask, kGroupRank, &sub)) break;
                if (c == nchunk) {
                    if (nchunk == kGroupChunks) break;   // the run continues in the next group
                    chunk[nchunk++].place(run[k]->zmask, kGroupRank, &sub);
                }
            }
            members.emplace_back(k, sub);
            which.push_back(c);
        }
        const size_t count = k - start;
        if (count < 2) return 1;
        op = Op();
        op.kind = OP_PAULI_GROUP;
        op.k = (int32_t)count;
        op.nchunk = nchunk;
        op.mat_offset = (int64_t)mats.size();
        for (int c = 0; c < nchunk; ++c) {
            op.rank[c] = chunk[c].r;
            for (int j = 0; j < chunk[c].r; ++j) {
                op.basis[c * kGroupRank + j] = chunk[c].w[j];
                op.zmask |= chunk[c].w[j];
            }
            std::vector<cd> tab((size_t)1 << chunk[c].r, cd(1.0, 0.0));
            for (size_t m = 0; m < members.size(); ++m) {
                if (which[m] != c) continue;
                cd ch, sh;
                exp_factors(*run[members[m].first], &ch, &sh);
                for (size_t b = 0; b < tab.size(); ++b)
                    tab[b] *= (__builtin_popcount((uint32_t)b & members[m].second) & 1) ? ch - sh : ch + sh;
            }
            mats.insert(mats.end(), tab.begin(), tab.end());
        }
        return count;
    }
    // pair run: every X-mask is 0 or X; parities are taken on i0 (highest bit of X clear)
    const uint64_t X = g0.xmask, hb = 1ull << (63 - __builtin_clzll(X));
    ParityBasis basis;
    size_t k = start;
    for (; k < run.size() && (run[k]->xmask == 0 || run[k]->xmask == X); ++k) {
        uint32_t sub = 0;
        if (!basis.place(run[k]->zmask & ~hb, kPairRank, &sub)) break;
        members.emplace_back(k, sub);
    }
    const size_t count = k - start;
    if (count < 2) return 1;
    op = Op();
    op.kind = OP_PAULI_GROUP;
    op.k = (int32_t)count;
    op.nchunk = 1;
    op.rank[0] = basis.r;
    op.xmask = X;
    for (int j = 0; j < basis.r; ++j) {
        op.basis[j] = basis.w[j];
        op.zmask |= basis.w[j];
    }
    op.mat_offset = (int64_t)mats.size();
    for (uint32_t b = 0; b < (1u << basis.r); ++b) {
        cd m[4] = {1.0, 0.0, 0.0, 1.0};
        for (const auto &mem : members) {
            const GateMatrix &g = *run[mem.first];
            cd ch, sh;
            exp_factors(g, &ch, &sh);
            const int p0 = __builtin_popcount(b & mem.second) & 1;
            const int p1 = p0 ^ (__builtin_popcountll(X & g.zmask) & 1);
            const cd s0 = p0 ? -sh : sh, s1 = p1 ? -sh : sh;
            cd t[4];
            if (g.xmask == 0) { t[0] = ch + s0; t[1] = 0.0; t[2] = 0.0; t[3] = ch + s1; }
            else { t[0] = ch; t[1] = s0; t[2] = s1; t[3] = ch; }
            const cd r0 = t[0] * m[0] + t[1] * m[2], r1 = t[0] * m[1] + t[1] * m[3];
            const cd r2 = t[2] * m[0] + t[3] * m[2], r3 = t[2] * m[1] + t[3] * m[3];
            m[0] = r0; m[1] = r1; m[2] = r2; m[3] = r3;
        }
        mats.insert(mats.end(), m, m + 4);
    }
    return count;
}

Status launch_pauli_group(qi_state *s, const Op &op, const void *d_mats) {
    GroupParams p;
    std::memset(&p, 0, sizeof(p));
    p.xmask = op.xmask;
    p.nchunk = op.nchunk;
    int32_t ntab = 0;
    for (int c = 0; c < op.nchunk; ++c) {
        p.rank[c] = op.rank[c];
        p.off[c] = ntab;
        ntab += (op.xmask ? 4 : 1) << op.rank[c];
        for (int j = 0; j < op.rank[c]; ++j) p.basis[c * kGroupRank + j] = op.basis[c * kGroupRank + j];
    }
    p.ntab = ntab;
    p.nbytes = (s->n + 7) / 8;
    const bool f32 = s->prec == QI_F32;
    const size_t esz = f32 ? sizeof(float2) : sizeof(double2);
    const void *tab = (const char *)d_mats + (size_t)op.mat_offset * esz;
    const bool narrow = s->dim() <= (1ull << 31);   // 32-bit indices
    if (op.xmask == 0) {
        p.nwork = s->dim();
        const unsigned g = pgrid(p.nwork);
#define QI_GD(T, I) k_pauli_group_diag<T, I><<<g, 256, 0, s->stream>>>((Cx<T>::V2 *)s->amps, p, (const Cx<T>::V2 *)tab)
        if (f32) { if (narrow) QI_GD(float, uint32_t); else QI_GD(float, uint64_t); }
        else { if (narrow) QI_GD(double, uint32_t); else QI_GD(double, uint64_t); }
#undef QI_GD
        count_launch();
        return check_launch("k_pauli_group_diag");
    }
    const uint64_t hb = 1ull << (63 - __builtin_clzll(op.xmask));
    p.lo_mask = hb - 1;
    p.nwork = s->dim() >> 1;
    const unsigned g = pgrid(p.nwork);
#define QI_GP(T, I) k_pauli_group_pair<T, I><<<g, 256, 0, s->stream>>>((Cx<T>::V2 *)s->amps, p, (const Cx<T>::V2 *)tab)
    if (f32) { if (narrow) QI_GP(float, uint32_t); else QI_GP(float, uint64_t); }
    else { if (narrow) QI_GP(double, uint32_t); else QI_GP(double, uint64_t); }
#undef QI_GP
    count_launch();
    return check_launch("k_pauli_group_pair");
}

Status launch_pauli_apply(qi_state *out, qi_state *in, uint64_t xmask, uint64_t zmask, double cre, double cim) {
    double pr, pi;
    minus_i_pow(__builtin_popcountll(xmask & zmask), pr, pi);
    const double fre = cre * pr - cim * pi, fim = cre * pi + cim * pr;
    unsigned g = pgrid(out->dim());
    if (out->prec == QI_F32)
        k_pauli_gather<float><<<g, 256, 0, out->stream>>>((float2 *)out->amps, (const float2 *)in->amps, out->dim(),
                                                          xmask, zmask, fre, fim);
    else
        k_pauli_gather<double><<<g, 256, 0, out->stream>>>((double2 *)out->amps, (const double2 *)in->amps, out->dim(),
                                                           xmask, zmask, fre, fim);
    count_launch();
    return check_launch("k_pauli_gather");
}

// ------------------------------------------------- grouped SumOp kernels --
// Terms are grouped by xmask.  For group g with xmask x:
//   f_g(i) = sum_{k in g} c_k (-i)^{ny_k} (-1)^popc(i & z_k)
//   (H psi)_i = sum_g f_g(i) psi_{i ^ x_g}
//   <psi|H|psi> = sum_g sum_i conj(psi_i) f_g(i) psi_{i ^ x_g}
struct GroupTerm {
    uint64_t zmask;
    double re, im;   // c_k (-i)^{ny_k}
};
struct GroupHdr {
    uint64_t xmask;
    int32_t first, count;   // into the term array
};

struct SumOpDev {
    GroupHdr *groups = nullptr;
    GroupTerm *terms = nullptr;
    int ngroups = 0;
    int nterms = 0;
    size_t cap_groups = 0, cap_terms = 0;
};

template <typename T>
__device__ __forceinline__ typename Cx<T>::V2 group_factor(const GroupTerm *t, int cnt, uint64_t i) {
    T re = 0, im = 0;
    for (int k = 0; k < cnt; ++k) {
        const GroupTerm g = t[k];
        const T sgn = (__popcll(i & g.zmask) & 1) ? T(-1) : T(1);
        re += sgn * (T)g.re;
        im += sgn * (T)g.im;
    }
    return Cx<T>::make(re, im);
}

// Expectation contribution of one group, FP64 block partials.
template <typename T>
__global__ void __launch_bounds__(256) k_group_expect(const typename Cx<T>::V2 *a, uint64_t dim, GroupHdr hdr,
                                                       const GroupTerm *terms, double *partials) {
    using X = Cx<T>;
    extern __shared__ GroupTerm sterm[];
    for (int k = threadIdx.x; k < hdr.count; k += blockDim.x) sterm[k] = terms[hdr.first + k];
    __syncthreads();
    double re = 0.0, im = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (hdr.xmask == 0) {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
            typename X::V2 v = ldg_stream(a + i);
            const T p = v.x * v.x + v.y * v.y;
            typename X::V2 f = group_factor<T>(sterm, hdr.count, i);
            re += (double)(p * f.x);
            im += (double)(p * f.y);
        }
    } else {
        const int h = 63 - __clzll(hdr.xmask);
        const uint64_t lo_mask = (1ull << h) - 1;
        const uint64_t npairs = dim >> 1;
        for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < npairs; w += stride) {
            const uint64_t i = ((w & ~lo_mask) << 1) | (w & lo_mask);
            const uint64_t j = i ^ hdr.xmask;
            typename X::V2 x = a[i], y = a[j];
            typename X::V2 fi = group_factor<T>(sterm, hdr.count, i);
            typename X::V2 fj = group_factor<T>(sterm, hdr.count, j);
            // conj(x) * fi * y + conj(y) * fj * x
            typename X::V2 cxy = X::make(x.x * y.x + x.y * y.y, x.x * y.y - x.y * y.x);   // conj(x) y
            typename X::V2 t0 = X::mul(fi, cxy);
            typename X::V2 t1 = X::mul(fj, X::make(cxy.x, -cxy.y));                        // conj(y) x
            re += (double)(t0.x + t1.x);
            im += (double)(t0.y + t1.y);
        }
    }
    double r0 = block_sum(re);
    double r1 = block_sum(im);
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = r0;
        partials[blockIdx.x * 4 + 1] = r1;
    }
}

// A group's terms live in dynamic shared memory (24 bytes each).  Above the default 48 KB
// window (less the kernel's 256 bytes of static block-sum space) the launch needs the
// opt-in attribute; every caller raises it to the same fixed cap, so concurrent callers
// never lower it under one another.
constexpr size_t kGroupExpectSmemCap = 200 * 1024;
static Status group_expect_smem(bool f32, size_t sm) {
    if (sm > kGroupExpectSmemCap)
        return err(QI_ERR_UNSUPPORTED, (int64_t)(sm / sizeof(GroupTerm)), (int64_t)(kGroupExpectSmemCap / sizeof(GroupTerm)),
                   "too many Pauli terms sharing one X mask for one pass");
    if (sm + 1024 > 48 * 1024) {
        if (f32) QI_CUDA(cudaFuncSetAttribute(k_group_expect<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)kGroupExpectSmemCap));
        else QI_CUDA(cudaFuncSetAttribute(k_group_expect<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kGroupExpectSmemCap));
    }
    return ok_status();
}

// ---- FP32 states: products and per-thread sums in FP32, folded into FP64
// every kExpBatch elements, so a pass is bound by memory rather than by the
// FP64 pipe (FP64 arithmetic runs at a small fraction of the FP32 rate here).
constexpr int kExpBatch = 32, kExpUnroll = 4;
constexpr int kExpLog2Threads = 18;   // diagonal group: 2^18 threads (1024 blocks of 256)

struct TermF {   // a GroupTerm with its coefficient rounded to FP32 once per block
    uint64_t zmask;
    float re, im;
};
__device__ __forceinline__ TermF term_f32(const GroupTerm &g) { return TermF{g.zmask, (float)g.re, (float)g.im}; }

template <int N>
__device__ __forceinline__ float2 factor_f32(const TermF *t, uint64_t i) {
    float re = 0.0f, im = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float sgn = (__popcll(i & t[k].zmask) & 1) ? -1.0f : 1.0f;
        re = fmaf(sgn, t[k].re, re);
        im = fmaf(sgn, t[k].im, im);
    }
    return make_float2(re, im);
}
__device__ __forceinline__ float2 factor_f32_n(const TermF *t, int n, uint64_t i) {
    float re = 0.0f, im = 0.0f;
    for (int k = 0; k < n; ++k) {
        const float sgn = (__popcll(i & t[k].zmask) & 1) ? -1.0f : 1.0f;
        re = fmaf(sgn, t[k].re, re);
        im = fmaf(sgn, t[k].im, im);
    }
    return make_float2(re, im);
}

// Diagonal group (xmask = 0): sum_i |psi_i|^2 f(i).  With i = it * 2^s + tid,
// f(i) = F(tid) [terms whose Z bits lie below s] + G[it] [terms above s, a
// host table] + the straddling terms, evaluated per element.
// NM = number of straddling terms held in registers (-1: runtime count nmix, read from shared memory).
template <int NM>
__global__ void __launch_bounds__(256) k_diag_expect_f32(const float2 *a, int s, int h, const float2 *G,
                                                         const GroupTerm *terms, int nlo, int nmix, double *partials) {
    constexpr int NR = NM > 0 ? NM : 1;
    extern __shared__ TermF st_terms[];
    for (int k = threadIdx.x; k < nlo + nmix; k += blockDim.x) st_terms[k] = term_f32(terms[k]);
    __syncthreads();
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const float2 F = factor_f32_n(st_terms, nlo, tid);
    const TermF *mix = st_terms + nlo;
    // straddling terms: sign = (low part of the sign, fixed per thread) x (high part, per iteration)
    uint32_t zh[NR];
    float mr[NR], mi[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        if (NM > 0) {
            const bool sl = __popcll((uint64_t)tid & mix[k].zmask) & 1;
            zh[k] = (uint32_t)(mix[k].zmask >> s);
            mr[k] = sl ? -mix[k].re : mix[k].re;
            mi[k] = sl ? -mix[k].im : mix[k].im;
        }
    }
    const uint32_t iters = 1u << h;
    double dr = 0.0, di = 0.0;
    constexpr int U = 2 * kExpUnroll;
    // FP32 sums of kExpBatch elements, folded into FP64 once per outer step (a fold
    // inside the element loop may be if-converted into every iteration)
    for (uint32_t b0 = 0; b0 < iters; b0 += kExpBatch) {
      float br = 0.0f, bi = 0.0f;
      const uint32_t bend = min(b0 + (uint32_t)kExpBatch, iters);
#pragma unroll 1
      for (uint32_t it0 = b0; it0 < bend; it0 += U) {
        float2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (it0 + u < iters) v[u] = ldg_stream(a + ((((uint64_t)(it0 + u)) << s) | tid));
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t it = it0 + u;
            if (it >= iters) break;
            const float2 g = __ldg(G + it);
            float fr = F.x + g.x, fi = F.y + g.y;
            if (NM > 0) {
#pragma unroll
                for (int k = 0; k < NR; ++k) {
                    const bool sh = __popc(it & zh[k]) & 1;
                    fr += sh ? -mr[k] : mr[k];
                    fi += sh ? -mi[k] : mi[k];
                }
            } else if (nmix > 0) {
                const float2 f = factor_f32_n(mix, nmix, ((uint64_t)it << s) | tid);
                fr += f.x;
                fi += f.y;
            }
            const float p = fmaf(v[u].x, v[u].x, v[u].y * v[u].y);
            br = fmaf(p, fr, br);
            bi = fmaf(p, fi, bi);
        }
      }
      dr += br;
      di += bi;
    }
    const double r0 = block_sum(dr), r1 = block_sum(di);
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = r0;
        partials[blockIdx.x * 4 + 1] = r1;
    }
}

// Group with xmask != 0: pairs (i, i ^ x), i with bit h (the top bit of x) clear:
// conj(psi_i) f(i) psi_j + conj(psi_j) f(j) psi_i.  Terms with Z mask 0 are the
// constant c0; the other N terms (N = 0: runtime count cnt) are held in
// registers, and the sign of a term at j = i ^ x is its sign at i times
// (-1)^popc(x & z).  IDX is the index type (uint32_t for n <= 32).
template <int N, typename IDX>
__global__ void __launch_bounds__(256) k_xgroup_expect_f32(const float2 *a, uint64_t npairs, uint64_t xmask, float c0r,
                                                           float c0i, const GroupTerm *terms, int cnt,
                                                           double *partials) {
    constexpr int NR = N > 0 ? N : 1;
    extern __shared__ TermF st_terms[];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) st_terms[k] = term_f32(terms[k]);
    __syncthreads();
    IDX z[NR];
    float cr_[NR], ci_[NR];
    bool px[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        if (N > 0) {
            z[k] = (IDX)st_terms[k].zmask;
            cr_[k] = st_terms[k].re;
            ci_[k] = st_terms[k].im;
            px[k] = (__popcll(xmask & st_terms[k].zmask) & 1) != 0;
        }
    }
    const int h = 63 - __clzll(xmask);
    const IDX lo_mask = (IDX)((1ull << h) - 1), xm = (IDX)xmask;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    double dr = 0.0, di = 0.0;
    // FP32 sums of kExpBatch pairs, folded into FP64 once per outer step (a fold inside
    // the pair loop may be if-converted into every iteration)
    for (uint64_t wb = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wb < npairs; wb += stride * kExpBatch) {
      float br = 0.0f, bi = 0.0f;
#pragma unroll 1
      for (int bstep = 0; bstep < kExpBatch / kExpUnroll; ++bstep) {
        const uint64_t w0 = wb + (uint64_t)bstep * stride * kExpUnroll;
        if (w0 >= npairs) break;
        float2 x[kExpUnroll], y[kExpUnroll];
        IDX iv[kExpUnroll];
#pragma unroll
        for (int u = 0; u < kExpUnroll; ++u) {
            const uint64_t w = w0 + u * stride;
            const IDX ww = (IDX)w;
            iv[u] = ((ww & ~lo_mask) << 1) | (ww & lo_mask);
            if (w < npairs) {
                x[u] = ldg_stream(a + iv[u]);
                y[u] = ldg_stream(a + (iv[u] ^ xm));
            }
        }
#pragma unroll
        for (int u = 0; u < kExpUnroll; ++u) {
            if (w0 + u * stride >= npairs) break;
            const IDX i = iv[u];
            float fir = c0r, fii = c0i, fjr = c0r, fji = c0i;
            if (N > 0) {
#pragma unroll
                for (int k = 0; k < NR; ++k) {
                    const bool si = (sizeof(IDX) == 4 ? __popc((uint32_t)(i & z[k])) : __popcll((uint64_t)(i & z[k]))) & 1;
                    const bool sj = si != px[k];
                    fir += si ? -cr_[k] : cr_[k];
                    fii += si ? -ci_[k] : ci_[k];
                    fjr += sj ? -cr_[k] : cr_[k];
                    fji += sj ? -ci_[k] : ci_[k];
                }
            } else {
                const float2 fi = factor_f32_n(st_terms, cnt, i), fj = factor_f32_n(st_terms, cnt, i ^ xm);
                fir += fi.x;
                fii += fi.y;
                fjr += fj.x;
                fji += fj.y;
            }
            // c = conj(x) y;  fi c + fj conj(c)
            const float cr = fmaf(x[u].x, y[u].x, x[u].y * y[u].y), ci = fmaf(x[u].x, y[u].y, -x[u].y * y[u].x);
            br += (fir * cr - fii * ci) + (fjr * cr + fji * ci);
            bi += (fir * ci + fii * cr) + (fji * cr - fjr * ci);
        }
      }
      dr += br;
      di += bi;
    }
    const double r0 = block_sum(dr), r1 = block_sum(di);
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = r0;
        partials[blockIdx.x * 4 + 1] = r1;
    }
}

// acc[0..1] += fixed-order sum of the partials (one thread block).
__global__ void k_accumulate(const double *partials, int nb, double *acc) {
    for (int c = 0; c < 2; ++c) {
        double v = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) v += partials[i * 4 + c];
        double r = block_sum(v);
        if (threadIdx.x == 0) acc[c] += r;
        __syncthreads();
    }
}

// (H psi)_i = sum_g f_g(i) psi_{i ^ x_g}   (SumOp::apply)
template <typename T>
__global__ void __launch_bounds__(256) k_sumop_apply(typename Cx<T>::V2 *o, const typename Cx<T>::V2 *in, uint64_t dim,
                                                     const GroupHdr *groups, int ngroups, const GroupTerm *terms,
                                                     int nterms) {
    using X = Cx<T>;
    // FP32 states keep the coefficients in shared memory already rounded to FP32
    // (converting FP64 per element would run on the scarce FP64 pipe)
    using Term = typename std::conditional<sizeof(T) == 4, TermF, GroupTerm>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Term *sterm = reinterpret_cast<Term *>(smem_raw);
    GroupHdr *shdr = reinterpret_cast<GroupHdr *>(sterm + nterms);
    for (int k = threadIdx.x; k < nterms; k += blockDim.x) {
        if constexpr (sizeof(T) == 4) sterm[k] = term_f32(terms[k]);
        else sterm[k] = terms[k];
    }
    for (int k = threadIdx.x; k < ngroups; k += blockDim.x) shdr[k] = groups[k];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
        typename X::V2 acc = X::make(0, 0);
        for (int g = 0; g < ngroups; ++g) {
            const GroupHdr h = shdr[g];
            typename X::V2 f;
            if constexpr (sizeof(T) == 4) f = factor_f32_n(sterm + h.first, h.count, i);
            else f = group_factor<T>(sterm + h.first, h.count, i);
            acc = X::fma(f, in[i ^ h.xmask], acc);
        }
        o[i] = acc;
    }
}

// FP32 SumOp::apply.  Per element the gathers of all groups are issued four at a time
// (independent loads in flight), and the largest group's factor — typically the diagonal
// ZZ / Z terms — comes from byte tables: T_b[v] sums the terms whose Z bits lie in byte b
// of the index, evaluated at byte value v, so f(i) = sum_b T_b[(i >> 8b) & 255] plus the
// few terms that straddle bytes.  IDX = uint32_t below 2^32 amplitudes (one POPC per term).
template <typename IDX> struct ApplyTerm {
    IDX zmask;
    float re, im;
};
template <typename IDX> struct ApplyHdr {
    IDX xmask;
    int32_t first, count;   // direct terms
};
constexpr int kApplyTableMin = 6;   // terms in a group before it gets byte tables
constexpr int kApplyBatch = 4;      // gathers in flight per element (16 measured slower: 4.5 against 3.6 ms)

template <typename IDX>
__device__ __forceinline__ float2 apply_factor(const ApplyTerm<IDX> *t, int n, IDX i) {
    float re = 0.0f, im = 0.0f;
    for (int k = 0; k < n; ++k) {
        const int par = (sizeof(IDX) == 4 ? __popc((uint32_t)(i & t[k].zmask)) : __popcll((uint64_t)(i & t[k].zmask))) & 1;
        const float sgn = par ? -1.0f : 1.0f;
        re = fmaf(sgn, t[k].re, re);
        im = fmaf(sgn, t[k].im, im);
    }
    return make_float2(re, im);
}

template <typename IDX>
__global__ void __launch_bounds__(256) k_sumop_apply_f32(float2 *o, const float2 *in, uint64_t dim,
                                                         const ApplyHdr<IDX> *hdrs, int ngroups,
                                                         const ApplyTerm<IDX> *terms, int nterms,
                                                         const float2 *tables, int ntables) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *stab = reinterpret_cast<float2 *>(smem_raw);                       // [ntables][256], group 0
    ApplyHdr<IDX> *shdr = reinterpret_cast<ApplyHdr<IDX> *>(stab + ntables * 256);
    ApplyTerm<IDX> *sterm = reinterpret_cast<ApplyTerm<IDX> *>(shdr + ngroups);
    for (int k = threadIdx.x; k < ntables * 256; k += blockDim.x) stab[k] = tables[k];
    for (int k = threadIdx.x; k < ngroups; k += blockDim.x) shdr[k] = hdrs[k];
    for (int k = threadIdx.x; k < nterms; k += blockDim.x) sterm[k] = terms[k];
    __syncthreads();
    using X = Cx<float>;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i64 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i64 < dim; i64 += stride) {
        const IDX i = (IDX)i64;
        float2 acc = make_float2(0.0f, 0.0f);
        int g0 = 0;
        if (ntables > 0) {   // group 0: byte tables + straddling terms
            const float2 v = in[i ^ shdr[0].xmask];
            float2 f = apply_factor(sterm + shdr[0].first, shdr[0].count, i);
            for (int b = 0; b < ntables; ++b) {
                const float2 t = stab[b * 256 + (int)((i >> (8 * b)) & 255)];
                f.x += t.x;
                f.y += t.y;
            }
            acc = X::fma(f, v, acc);
            g0 = 1;
        }
        for (int g = g0; g < ngroups; g += kApplyBatch) {
            float2 v[kApplyBatch];
#pragma unroll
            for (int j = 0; j < kApplyBatch; ++j)
                if (g + j < ngroups) v[j] = in[i ^ shdr[g + j].xmask];
#pragma unroll
            for (int j = 0; j < kApplyBatch; ++j)
                if (g + j < ngroups) acc = X::fma(apply_factor(sterm + shdr[g + j].first, shdr[g + j].count, i), v[j], acc);
        }
        o[i64] = acc;
    }
}

// Streamed FP32 SumOp::apply for states of 2^kApplyTileBits amplitudes and more.  The output is
// taken in tiles of 2^kApplyTileBits consecutive amplitudes; a group with X mask x reads, for
// output tile T, the input tile T ^ (x >> kApplyTileBits) at local offsets l ^ (x & tile mask).
// The groups are ordered by that tile offset (one step per distinct offset, offset 0 first), so
// each step is one contiguous 32 KB bulk copy into a ring of shared-memory buffers and every
// gather becomes a shared-memory read.  Roles: 16 compute warps, and one copy warp whose lane 0
// issues the copies as soon as the compute warps release a buffer (full / empty mbarriers per
// buffer; no block-wide barrier in the loop, every wait bounded).
// Factors: compute thread t owns the amplitudes l_j = t + 512 j (j = 0..7) of a tile, whose
// indices differ only in bits 9-11.  A term with Z mask z contributes c (-1)^popc(i_j & z) =
// c (-1)^popc(b & z) (-1)^popc(j & m), b = tile bits | t, m = bits 9-11 of z; so the thread sums
// each group's terms once per tile into A[m] (terms are sorted by m on the host) and an 8-point
// Walsh-Hadamard transform of A gives the factors of all eight amplitudes (one term evaluation per
// eight amplitudes instead of one per amplitude).
constexpr int kApplyTileBits = 12, kApplyTileAmps = 1 << kApplyTileBits;
constexpr int kApplyTileThreads = 512, kApplyTileBufs = 6;
constexpr int kApplyComputeWarps = kApplyTileThreads / 32;
constexpr int kApplyBlockThreads = kApplyTileThreads + 32;             // + the copy warp
constexpr int kApplyTilePer = kApplyTileAmps / kApplyTileThreads;   // 8 amplitudes per thread
static_assert(kApplyTileThreads == 512 && kApplyTilePer == 8, "bits 9-11 of a tile index select the amplitude");
struct ApplyStep {
    uint64_t tile_xor;        // input tile = output tile ^ tile_xor
    int32_t g_first, g_count;  // its groups
};
struct TileGroup {
    uint32_t xl;       // X mask bits below the tile size
    int32_t m[9];      // terms with bits 9-11 of the Z mask = m: [m[m], m[m + 1])
    int32_t flat;      // 1: every term has m = 0 (one factor for all eight amplitudes, no transform)
};
template <typename IDX> struct alignas(16) TileTerm {   // one 16-byte shared-memory load
    IDX z;
    float re, im;
};

template <typename IDX>
__global__ void __launch_bounds__(kApplyBlockThreads, 1)
    k_sumop_apply_tiles_f32(float2 *o, const float2 *in, uint64_t ntiles, const ApplyStep *steps, int nsteps,
                            const TileGroup *groups, int ngroups, const TileTerm<IDX> *terms, int nterms,
                            int *err_flag) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *buf = reinterpret_cast<float2 *>(smem_raw);                          // [kApplyTileBufs][tile]
    ApplyStep *sstep = reinterpret_cast<ApplyStep *>(buf + (size_t)kApplyTileBufs * kApplyTileAmps);
    TileTerm<IDX> *sterm = reinterpret_cast<TileTerm<IDX> *>(sstep + nsteps);
    TileGroup *sgrp = reinterpret_cast<TileGroup *>(sterm + nterms);
    __shared__ __align__(8) uint64_t full[kApplyTileBufs], empty[kApplyTileBufs];
    __shared__ int abort_flag;
    volatile int *abort_v = &abort_flag;
    const int tid = threadIdx.x;
    for (int k = tid; k < nsteps; k += blockDim.x) sstep[k] = steps[k];
    for (int k = tid; k < nterms; k += blockDim.x) sterm[k] = terms[k];
    for (int k = tid; k < ngroups; k += blockDim.x) sgrp[k] = groups[k];
    if (tid == 0) {
        for (int b = 0; b < kApplyTileBufs; ++b) {
            mbar_init(full + b, 1);
            mbar_init(empty + b, kApplyComputeWarps);
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    constexpr uint32_t kBytes = kApplyTileAmps * sizeof(float2);
    const uint64_t mine = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint64_t total = mine * (uint64_t)nsteps;   // (tile, step) pairs of this block, in order
    if (tid >= kApplyTileThreads) {
        // ------------------------------------------------ copy warp (lane 0)
        if (tid == kApplyTileThreads) {
            uint64_t issued = 0, tile = blockIdx.x;
            int st = 0, b = 0;
            uint32_t phase = 0;   // of empty[b]: the compute warps' release of the buffer's previous fill
            for (; issued < total; ++issued) {
                if (issued >= (uint64_t)kApplyTileBufs && !wait_or_abort(empty + b, phase, abort_v, err_flag)) break;
                const uint64_t src = tile ^ sstep[st].tile_xor;
                mbar_arrive_expect_tx(full + b, kBytes);
                bulk_load(buf + (size_t)b * kApplyTileAmps, in + (src << kApplyTileBits), kBytes, full + b);
                if (++b == kApplyTileBufs) {
                    b = 0;
                    if (issued >= (uint64_t)kApplyTileBufs) phase ^= 1u;
                }
                if (++st == nsteps) {
                    st = 0;
                    tile += gridDim.x;
                }
            }
            // the last copies land before the block exits (after an abort, unread ones too)
            for (uint64_t k = issued > (uint64_t)kApplyTileBufs ? issued - kApplyTileBufs : 0; k < issued; ++k)
                if (!mbar_wait_bounded(full + (k % kApplyTileBufs), (uint32_t)(k / kApplyTileBufs) & 1u))
                    atomicExch(err_flag, 2);
        }
        return;
    }
    // ---------------------------------------------------- compute warps
    const int lane = tid & 31;
    float2 acc[kApplyTilePer];
    // (tile, step, buffer, phase) advance by counting: no divisions in the loop
    uint64_t tile = blockIdx.x;
    int st = 0, b = 0;
    uint32_t phase = 0;
    for (uint64_t q = 0; q < total; ++q) {
        if (st == 0) {
#pragma unroll
            for (int j = 0; j < kApplyTilePer; ++j) acc[j] = make_float2(0.0f, 0.0f);
        }
        const bool ok = wait_or_abort(full + b, phase, abort_v, err_flag);
        if (!__all_sync(0xffffffffu, ok)) break;
        const float2 *P = buf + (size_t)b * kApplyTileAmps;
        const ApplyStep stp = sstep[st];
        const IDX base = (IDX)((tile << kApplyTileBits) | (uint64_t)tid);   // bits 9-11 clear
        for (int g = stp.g_first; g < stp.g_first + stp.g_count; ++g) {
            const TileGroup &G = sgrp[g];
            if (G.flat) {
                float re = 0.0f, im = 0.0f;
                for (int k = G.m[0]; k < G.m[8]; ++k) {
                    const TileTerm<IDX> t = sterm[k];
                    const uint32_t par = (uint32_t)(sizeof(IDX) == 4 ? __popc((uint32_t)(base & t.z))
                                                                    : __popcll((uint64_t)(base & t.z)));
                    const uint32_t sb = par << 31;
                    re += __uint_as_float(__float_as_uint(t.re) ^ sb);
                    im += __uint_as_float(__float_as_uint(t.im) ^ sb);
                }
                const float2 f = make_float2(re, im);
#pragma unroll
                for (int j = 0; j < kApplyTilePer; ++j)
                    acc[j] = Cx<float>::fma(f, P[(uint32_t)(tid + j * kApplyTileThreads) ^ G.xl], acc[j]);
                continue;
            }
            float2 A[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                float re = 0.0f, im = 0.0f;
                for (int k = G.m[m]; k < G.m[m + 1]; ++k) {
                    const TileTerm<IDX> t = sterm[k];
                    const uint32_t par = (uint32_t)(sizeof(IDX) == 4 ? __popc((uint32_t)(base & t.z))
                                                                    : __popcll((uint64_t)(base & t.z)));
                    const uint32_t sb = par << 31;   // the parity's sign, as an FP32 sign bit
                    re += __uint_as_float(__float_as_uint(t.re) ^ sb);
                    im += __uint_as_float(__float_as_uint(t.im) ^ sb);
                }
                A[m] = make_float2(re, im);
            }
#pragma unroll
            for (int h = 1; h < 8; h <<= 1)   // f[j] = sum_m A[m] (-1)^popc(j & m)
#pragma unroll
                for (int m = 0; m < 8; ++m)
                    if (!(m & h)) {
                        const float2 u = A[m], v = A[m | h];
                        A[m] = make_float2(u.x + v.x, u.y + v.y);
                        A[m | h] = make_float2(u.x - v.x, u.y - v.y);
                    }
#pragma unroll
            for (int j = 0; j < kApplyTilePer; ++j)
                acc[j] = Cx<float>::fma(A[j], P[(uint32_t)(tid + j * kApplyTileThreads) ^ G.xl], acc[j]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + b);   // this warp is done with buffer b
        if (++b == kApplyTileBufs) {
            b = 0;
            phase ^= 1u;
        }
        if (++st == nsteps) {
#pragma unroll
            for (int j = 0; j < kApplyTilePer; ++j)
                o[(tile << kApplyTileBits) | (uint64_t)(tid + j * kApplyTileThreads)] = acc[j];
            st = 0;
            tile += gridDim.x;
        }
    }
}

// Host side of k_sumop_apply_f32: term records, the byte tables of the largest group (moved
// to index 0) and the shared-memory size.
template <typename IDX>
struct ApplyPlan {
    std::vector<ApplyHdr<IDX>> hdrs;
    std::vector<ApplyTerm<IDX>> terms;
    std::vector<float2> tables;
    int ntables = 0;
    size_t smem() const {
        return tables.size() * sizeof(float2) + hdrs.size() * sizeof(ApplyHdr<IDX>) + terms.size() * sizeof(ApplyTerm<IDX>);
    }
};

template <typename IDX>
static void build_apply_plan(int n, const std::vector<GroupHdr> &hdrs, const std::vector<GroupTerm> &gts,
                             ApplyPlan<IDX> &ap) {
    int big = -1;
    for (size_t g = 0; g < hdrs.size(); ++g)
        if (hdrs[g].count >= kApplyTableMin && (big < 0 || hdrs[g].count > hdrs[(size_t)big].count)) big = (int)g;
    std::vector<size_t> order;
    if (big >= 0) order.push_back((size_t)big);
    for (size_t g = 0; g < hdrs.size(); ++g)
        if ((int)g != big) order.push_back(g);
    const int nbytes = (n + 7) / 8;
    std::vector<std::complex<double>> tab;
    for (size_t g : order) {
        const GroupHdr &h = hdrs[g];
        ApplyHdr<IDX> ah;
        ah.xmask = (IDX)h.xmask;
        ah.first = (int32_t)ap.terms.size();
        const bool tabled = (int)g == big;
        if (tabled) tab.assign((size_t)nbytes * 256, std::complex<double>(0, 0));
        for (int k = 0; k < h.count; ++k) {
            const GroupTerm &t = gts[(size_t)(h.first + k)];
            int byte = -1;
            if (tabled) {
                if (t.zmask == 0) byte = 0;
                for (int b = 0; b < nbytes && byte < 0; ++b)
                    if ((t.zmask & ~(0xffull << (8 * b))) == 0) byte = b;
            }
            if (byte >= 0) {
                const uint64_t zb = (t.zmask >> (8 * byte)) & 0xff;
                for (int v = 0; v < 256; ++v) {
                    const double sgn = (__builtin_popcountll((uint64_t)v & zb) & 1) ? -1.0 : 1.0;
                    tab[(size_t)byte * 256 + (size_t)v] += std::complex<double>(sgn * t.re, sgn * t.im);
                }
            } else {
                ap.terms.push_back(ApplyTerm<IDX>{(IDX)t.zmask, (float)t.re, (float)t.im});
            }
        }
        ah.count = (int32_t)ap.terms.size() - ah.first;
        ap.hdrs.push_back(ah);
        if (tabled) {
            ap.ntables = nbytes;
            for (auto &c : tab) ap.tables.push_back(make_float2((float)c.real(), (float)c.imag()));
        }
    }
}

// The streamed form: groups ordered by input-tile offset (offset 0 first), one step per offset,
// each group's terms sorted by bits 9-11 of their Z masks.  *done = false (nothing launched) when
// the state is smaller than a tile or the records do not fit beside the ring.
template <typename IDX>
static Status launch_sumop_apply_tiles_f32(qi_state *o, qi_state *in, const std::vector<GroupHdr> &hdrs,
                                           const std::vector<GroupTerm> &gts, bool *done) {
    *done = false;
    if (o->n < kApplyTileBits) return ok_status();
    std::map<uint64_t, std::vector<size_t>> by_off;
    for (size_t g = 0; g < hdrs.size(); ++g) by_off[hdrs[g].xmask >> kApplyTileBits].push_back(g);
    std::vector<ApplyStep> steps;
    std::vector<TileGroup> groups;
    std::vector<TileTerm<IDX>> terms;
    for (auto &kv : by_off) {
        ApplyStep stp;
        stp.tile_xor = kv.first;
        stp.g_first = (int32_t)groups.size();
        stp.g_count = (int32_t)kv.second.size();
        for (size_t g : kv.second) {
            const GroupHdr &h = hdrs[g];
            TileGroup tg;
            tg.xl = (uint32_t)(h.xmask & (uint64_t)(kApplyTileAmps - 1));
            for (int m = 0; m < 8; ++m) {
                tg.m[m] = (int32_t)terms.size();
                for (int k = 0; k < h.count; ++k) {
                    const GroupTerm &t = gts[(size_t)(h.first + k)];
                    if ((int)((t.zmask >> 9) & 7) == m)
                        terms.push_back(TileTerm<IDX>{(IDX)t.zmask, (float)t.re, (float)t.im});
                }
            }
            tg.m[8] = (int32_t)terms.size();
            tg.flat = tg.m[1] == tg.m[8] ? 1 : 0;
            groups.push_back(tg);
        }
        steps.push_back(stp);
    }
    const size_t ring = (size_t)kApplyTileBufs * kApplyTileAmps * sizeof(float2);
    const size_t meta = steps.size() * sizeof(ApplyStep) + terms.size() * sizeof(TileTerm<IDX>) +
                        groups.size() * sizeof(TileGroup);
    const size_t sm = ring + meta;
    if (sm > 220 * 1024) return ok_status();
    int dev = 0, sms = 0;
    QI_CUDA(cudaGetDevice(&dev));
    QI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // one device block for the records, each array starting on a 16-byte boundary
    auto up16 = [](size_t v) { return (v + 15) & ~(size_t)15; };
    const size_t off_term = up16(steps.size() * sizeof(ApplyStep));
    const size_t off_grp = off_term + up16(std::max<size_t>(1, terms.size()) * sizeof(TileTerm<IDX>));
    const size_t bytes = off_grp + up16(groups.size() * sizeof(TileGroup));
    unsigned char *d = nullptr;
    QI_CUDA(cudaMallocAsync((void **)&d, bytes, o->stream));
    ApplyStep *d_steps = reinterpret_cast<ApplyStep *>(d);
    TileTerm<IDX> *d_term = reinterpret_cast<TileTerm<IDX> *>(d + off_term);
    TileGroup *d_grp = reinterpret_cast<TileGroup *>(d + off_grp);
    QI_CUDA(cudaMemcpyAsync(d_steps, steps.data(), steps.size() * sizeof(ApplyStep), cudaMemcpyHostToDevice, o->stream));
    if (!terms.empty())
        QI_CUDA(cudaMemcpyAsync(d_term, terms.data(), terms.size() * sizeof(TileTerm<IDX>), cudaMemcpyHostToDevice,
                                o->stream));
    QI_CUDA(cudaMemcpyAsync(d_grp, groups.data(), groups.size() * sizeof(TileGroup), cudaMemcpyHostToDevice, o->stream));
    auto kern = k_sumop_apply_tiles_f32<IDX>;
    QI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const uint64_t ntiles = o->dim() >> kApplyTileBits;
    const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)std::max(sms, 1));
    kern<<<grid, kApplyBlockThreads, sm, o->stream>>>((float2 *)o->amps, (const float2 *)in->amps, ntiles, d_steps,
                                                     (int)steps.size(), d_grp, (int)groups.size(), d_term,
                                                     (int)terms.size(), o->d_flag);
    count_launch();
    Status st = check_launch("k_sumop_apply_tiles_f32");
    QI_CUDA(cudaFreeAsync(d, o->stream));
    *done = st.ok();
    return st;
}

template <typename IDX>
static Status launch_sumop_apply_f32(qi_state *o, qi_state *in, const std::vector<GroupHdr> &hdrs,
                                     const std::vector<GroupTerm> &gts, bool *done) {
    Status tst = launch_sumop_apply_tiles_f32<IDX>(o, in, hdrs, gts, done);
    if (!tst.ok() || *done) return tst;
    ApplyPlan<IDX> ap;
    build_apply_plan<IDX>(o->n, hdrs, gts, ap);
    const size_t sm = ap.smem();
    if (sm > 200 * 1024) return ok_status();   // the caller takes the generic kernel
    ApplyHdr<IDX> *d_hdr = nullptr;
    ApplyTerm<IDX> *d_term = nullptr;
    float2 *d_tab = nullptr;
    QI_CUDA(cudaMallocAsync((void **)&d_hdr, std::max<size_t>(1, ap.hdrs.size()) * sizeof(ApplyHdr<IDX>), o->stream));
    QI_CUDA(cudaMallocAsync((void **)&d_term, std::max<size_t>(1, ap.terms.size()) * sizeof(ApplyTerm<IDX>), o->stream));
    QI_CUDA(cudaMallocAsync((void **)&d_tab, std::max<size_t>(1, ap.tables.size()) * sizeof(float2), o->stream));
    QI_CUDA(cudaMemcpyAsync(d_hdr, ap.hdrs.data(), ap.hdrs.size() * sizeof(ApplyHdr<IDX>), cudaMemcpyHostToDevice, o->stream));
    QI_CUDA(cudaMemcpyAsync(d_term, ap.terms.data(), ap.terms.size() * sizeof(ApplyTerm<IDX>), cudaMemcpyHostToDevice,
                            o->stream));
    QI_CUDA(cudaMemcpyAsync(d_tab, ap.tables.data(), ap.tables.size() * sizeof(float2), cudaMemcpyHostToDevice, o->stream));
    auto kern = k_sumop_apply_f32<IDX>;
    if (sm + 1024 > 48 * 1024) QI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    kern<<<pgrid(o->dim()), 256, sm, o->stream>>>((float2 *)o->amps, (const float2 *)in->amps, o->dim(), d_hdr,
                                                 (int)ap.hdrs.size(), d_term, (int)ap.terms.size(), d_tab, ap.ntables);
    count_launch();
    Status st = check_launch("k_sumop_apply_f32");
    QI_CUDA(cudaFreeAsync(d_hdr, o->stream));
    QI_CUDA(cudaFreeAsync(d_term, o->stream));
    QI_CUDA(cudaFreeAsync(d_tab, o->stream));
    *done = st.ok();
    return st;
}

// Build the grouped representation of a term list (host).
static void group_terms(const qi_pauli_term *terms, int64_t nt, std::vector<GroupHdr> &hdrs,
                        std::vector<GroupTerm> &out) {
    std::map<uint64_t, std::vector<GroupTerm>> by_x;
    std::vector<uint64_t> order;
    for (int64_t k = 0; k < nt; ++k) {
        const qi_pauli_term &t = terms[k];
        double pr, pi;
        minus_i_pow(__builtin_popcountll(t.xmask & t.zmask), pr, pi);
        GroupTerm g;
        g.zmask = t.zmask;
        g.re = t.coeff_re * pr - t.coeff_im * pi;
        g.im = t.coeff_re * pi + t.coeff_im * pr;
        if (!by_x.count(t.xmask)) order.push_back(t.xmask);
        by_x[t.xmask].push_back(g);
    }
    hdrs.clear();
    out.clear();
    for (uint64_t x : order) {
        GroupHdr h;
        h.xmask = x;
        h.first = (int32_t)out.size();
        h.count = (int32_t)by_x[x].size();
        for (auto &g : by_x[x]) out.push_back(g);
        hdrs.push_back(h);
    }
}

static Status upload_groups(qi_state *s, const std::vector<GroupHdr> &hdrs, const std::vector<GroupTerm> &terms,
                            GroupHdr **d_hdr, GroupTerm **d_terms) {
    QI_CUDA(cudaMallocAsync((void **)d_hdr, std::max<size_t>(1, hdrs.size()) * sizeof(GroupHdr), s->stream));
    QI_CUDA(cudaMallocAsync((void **)d_terms, std::max<size_t>(1, terms.size()) * sizeof(GroupTerm), s->stream));
    QI_CUDA(cudaMemcpyAsync(*d_hdr, hdrs.data(), hdrs.size() * sizeof(GroupHdr), cudaMemcpyHostToDevice, s->stream));
    QI_CUDA(cudaMemcpyAsync(*d_terms, terms.data(), terms.size() * sizeof(GroupTerm), cudaMemcpyHostToDevice, s->stream));
    // host vectors are pageable: the copies complete before cudaMemcpyAsync returns
    return ok_status();
}

// <psi|H|psi> into out[2]; synchronises.
Status sumop_expectation(qi_state *s, const qi_pauli_term *terms, int64_t nt, double out[2]) {
    std::vector<GroupHdr> hdrs;
    std::vector<GroupTerm> gts;
    group_terms(terms, nt, hdrs, gts);
    GroupHdr *d_hdr = nullptr;
    GroupTerm *d_terms = nullptr;
    Status st = upload_groups(s, hdrs, gts, &d_hdr, &d_terms);
    if (!st.ok()) return st;
    QI_CUDA(cudaMemsetAsync(s->d_result, 0, 2 * sizeof(double), s->stream));
    const bool f32 = s->prec == QI_F32;
    std::vector<void *> scratch;   // per-call device tables, freed (stream-ordered) at the end
    for (const GroupHdr &h : hdrs) {
        // FP32 kernels keep a group's terms in the default 48 KB shared-memory window (less their
        // static block-sum space); larger groups take k_group_expect below
        if (f32 && (size_t)h.count * sizeof(GroupTerm) + 1024 <= 48 * 1024) {
            const GroupTerm *gt = gts.data() + h.first;
            unsigned nb = 1;
            if (h.xmask == 0) {
                // split the Z terms at the thread bits: below sb, above sb, straddling
                const int n = s->n, sb = std::min(n, kExpLog2Threads), hb = n - sb;
                const uint64_t lo = (sb >= 64) ? ~0ull : ((1ull << sb) - 1);
                std::vector<GroupTerm> lm;
                std::vector<const GroupTerm *> hi;
                int nlo = 0;
                for (int k = 0; k < h.count; ++k)
                    if ((gt[k].zmask & ~lo) == 0) { lm.insert(lm.begin() + nlo, gt[k]); ++nlo; }
                for (int k = 0; k < h.count; ++k)
                    if ((gt[k].zmask & lo) == 0 && (gt[k].zmask & ~lo) != 0) hi.push_back(&gt[k]);
                    else if ((gt[k].zmask & lo) != 0 && (gt[k].zmask & ~lo) != 0) lm.push_back(gt[k]);
                const int nmix = (int)lm.size() - nlo;
                std::vector<float2> G((size_t)1 << hb);
                for (uint64_t it = 0; it < G.size(); ++it) {
                    double re = 0.0, im = 0.0;
                    for (const GroupTerm *t : hi) {
                        const double sgn = (__builtin_popcountll((it << sb) & t->zmask) & 1) ? -1.0 : 1.0;
                        re += sgn * t->re;
                        im += sgn * t->im;
                    }
                    G[it] = make_float2((float)re, (float)im);
                }
                void *dG = nullptr, *dT = nullptr;
                QI_CUDA(cudaMallocAsync(&dG, G.size() * sizeof(float2), s->stream));
                QI_CUDA(cudaMallocAsync(&dT, std::max<size_t>(1, lm.size()) * sizeof(GroupTerm), s->stream));
                scratch.push_back(dG);
                scratch.push_back(dT);
                QI_CUDA(cudaMemcpyAsync(dG, G.data(), G.size() * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
                if (!lm.empty())
                    QI_CUDA(cudaMemcpyAsync(dT, lm.data(), lm.size() * sizeof(GroupTerm), cudaMemcpyHostToDevice, s->stream));
                const uint64_t threads = 1ull << sb;
                const unsigned tpb = (unsigned)std::min<uint64_t>(threads, 256);
                nb = (unsigned)(threads / tpb);
                const size_t smd = std::max<size_t>(1, lm.size()) * sizeof(GroupTerm);
                const float2 *amp = (const float2 *)s->amps;
                const GroupTerm *dtt = (const GroupTerm *)dT;
                switch (nmix) {
                case 0: k_diag_expect_f32<0><<<nb, tpb, smd, s->stream>>>(amp, sb, hb, (const float2 *)dG, dtt, nlo, nmix, s->d_partials); break;
                case 1: k_diag_expect_f32<1><<<nb, tpb, smd, s->stream>>>(amp, sb, hb, (const float2 *)dG, dtt, nlo, nmix, s->d_partials); break;
                case 2: k_diag_expect_f32<2><<<nb, tpb, smd, s->stream>>>(amp, sb, hb, (const float2 *)dG, dtt, nlo, nmix, s->d_partials); break;
                case 3: k_diag_expect_f32<3><<<nb, tpb, smd, s->stream>>>(amp, sb, hb, (const float2 *)dG, dtt, nlo, nmix, s->d_partials); break;
                default: k_diag_expect_f32<-1><<<nb, tpb, smd, s->stream>>>(amp, sb, hb, (const float2 *)dG, dtt, nlo, nmix, s->d_partials);
                }
            } else {
                // constant part (Z mask 0) on the host; the other terms packed for the kernel
                double c0r = 0.0, c0i = 0.0;
                std::vector<GroupTerm> nz;
                for (int k = 0; k < h.count; ++k) {
                    if (gt[k].zmask == 0) { c0r += gt[k].re; c0i += gt[k].im; }
                    else nz.push_back(gt[k]);
                }
                void *dT = nullptr;
                QI_CUDA(cudaMallocAsync(&dT, std::max<size_t>(1, nz.size()) * sizeof(GroupTerm), s->stream));
                scratch.push_back(dT);
                if (!nz.empty())
                    QI_CUDA(cudaMemcpyAsync(dT, nz.data(), nz.size() * sizeof(GroupTerm), cudaMemcpyHostToDevice, s->stream));
                const uint64_t npairs = s->dim() >> 1;
                nb = (unsigned)std::min<uint64_t>(std::max<uint64_t>((npairs + 256 * kExpUnroll - 1) / (256 * kExpUnroll), 1),
                                                  kReduceBlocks);
                const size_t sm = std::max<size_t>(1, nz.size()) * sizeof(GroupTerm);
                const GroupTerm *dt = (const GroupTerm *)dT;
                const float2 *amp = (const float2 *)s->amps;
                const int cnt = (int)nz.size();
                const float fr = (float)c0r, fi = (float)c0i;
#define QI_XG(NN, IDX)                                                                                               \
    k_xgroup_expect_f32<NN, IDX><<<nb, 256, sm, s->stream>>>(amp, npairs, h.xmask, fr, fi, dt, cnt, s->d_partials)
                const bool narrow = s->n <= 32;
                switch (cnt) {
                case 0: if (narrow) QI_XG(0, uint32_t); else QI_XG(0, uint64_t); break;
                case 1: if (narrow) QI_XG(1, uint32_t); else QI_XG(1, uint64_t); break;
                case 2: if (narrow) QI_XG(2, uint32_t); else QI_XG(2, uint64_t); break;
                case 3: if (narrow) QI_XG(3, uint32_t); else QI_XG(3, uint64_t); break;
                default: if (narrow) QI_XG(0, uint32_t); else QI_XG(0, uint64_t);
                }
#undef QI_XG
            }
            k_accumulate<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, s->d_result);
            count_launch(2);
            st = check_launch(h.xmask ? "k_xgroup_expect_f32" : "k_diag_expect_f32");
            if (!st.ok()) return st;
            continue;
        }
        const uint64_t work = h.xmask ? (s->dim() >> 1) : s->dim();
        uint64_t nb64 = (work + kReduceThreads - 1) / kReduceThreads;
        const unsigned nb = (unsigned)std::min<uint64_t>(std::max<uint64_t>(nb64, 1), kReduceBlocks);
        const size_t sm = (size_t)h.count * sizeof(GroupTerm);
        st = group_expect_smem(f32, sm);
        if (!st.ok()) return st;
        if (f32)
            k_group_expect<float><<<nb, kReduceThreads, sm, s->stream>>>((const float2 *)s->amps, s->dim(), h, d_terms,
                                                                         s->d_partials);
        else
            k_group_expect<double><<<nb, kReduceThreads, sm, s->stream>>>((const double2 *)s->amps, s->dim(), h, d_terms,
                                                                          s->d_partials);
        k_accumulate<<<1, 256, 0, s->stream>>>(s->d_partials, (int)nb, s->d_result);
        count_launch(2);
        st = check_launch("k_group_expect");
        if (!st.ok()) return st;
    }
    QI_CUDA(cudaMemcpyAsync(s->h_result, s->d_result, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    for (void *p : scratch) QI_CUDA(cudaFreeAsync(p, s->stream));
    QI_CUDA(cudaFreeAsync(d_hdr, s->stream));
    QI_CUDA(cudaFreeAsync(d_terms, s->stream));
    QI_CUDA(cudaStreamSynchronize(s->stream));
    out[0] = s->h_result[0];
    out[1] = s->h_result[1];
    return ok_status();
}

Status sumop_apply(qi_state *o, qi_state *in, const qi_pauli_term *terms, int64_t nt) {
    std::vector<GroupHdr> hdrs;
    std::vector<GroupTerm> gts;
    group_terms(terms, nt, hdrs, gts);
    if (o->prec == QI_F32) {
        bool done = false;
        Status st = o->n <= 32 ? launch_sumop_apply_f32<uint32_t>(o, in, hdrs, gts, &done)
                               : launch_sumop_apply_f32<uint64_t>(o, in, hdrs, gts, &done);
        if (!st.ok() || done) return st;
    }
    GroupHdr *d_hdr = nullptr;
    GroupTerm *d_terms = nullptr;
    Status st = upload_groups(o, hdrs, gts, &d_hdr, &d_terms);
    if (!st.ok()) return st;
    const size_t sm = gts.size() * sizeof(GroupTerm) + hdrs.size() * sizeof(GroupHdr);
    if (sm > 200 * 1024) return err(QI_ERR_UNSUPPORTED, (int64_t)nt, -1, "too many Pauli terms for one pass");
    unsigned g = pgrid(o->dim());
    if (o->prec == QI_F32) {
        if (sm + 1024 > 48 * 1024) QI_CUDA(cudaFuncSetAttribute(k_sumop_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        k_sumop_apply<float><<<g, 256, sm, o->stream>>>((float2 *)o->amps, (const float2 *)in->amps, o->dim(), d_hdr,
                                                       (int)hdrs.size(), d_terms, (int)gts.size());
    } else {
        if (sm + 1024 > 48 * 1024) QI_CUDA(cudaFuncSetAttribute(k_sumop_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        k_sumop_apply<double><<<g, 256, sm, o->stream>>>((double2 *)o->amps, (const double2 *)in->amps, o->dim(), d_hdr,
                                                        (int)hdrs.size(), d_terms, (int)gts.size());
    }
    count_launch();
    st = check_launch("k_sumop_apply");
    if (!st.ok()) return st;
    QI_CUDA(cudaFreeAsync(d_hdr, o->stream));
    QI_CUDA(cudaFreeAsync(d_terms, o->stream));
    return ok_status();
}

// cosh / sinh of a complex alpha with num_complex's formulas.
void exp_coeffs(double ar, double ai, double &cre, double &cim, double &sre, double &sim) {
    cre = std::cosh(ar) * std::cos(ai);
    cim = std::sinh(ar) * std::sin(ai);
    sre = std::sinh(ar) * std::cos(ai);
    sim = std::cosh(ar) * std::sin(ai);
}

}  // namespace qi

using namespace qi;

#define QI_LOCK(s)                                                        \
    if (!(s)) return publish(err(QI_ERR_NULL_ARGUMENT));                  \
    std::lock_guard<std::recursive_mutex> qi_lk_((s)->mu);                \
    {                                                                     \
        cudaError_t qi_e_ = cudaSetDevice((s)->device);                   \
        if (qi_e_ != cudaSuccess) return publish(cuda_status(qi_e_, "cudaSetDevice")); \
    }

extern "C" {

qi_status qi_pauli_apply(qi_state *out, qi_state *in, const qi_pauli_term *t) {
    QI_LOCK(out);
    if (!in || !t) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (in->n != out->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, in->n));
    if (in->prec != out->prec) return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "equal precisions required"));
    Status st = validate_pauli(in->n, *t);
    if (!st.ok()) return publish(st);
    if (in == out) {
        // in place: pair update with cosh = 0, sinh = coefficient
        return publish(launch_pauli_exp(out, t->xmask, t->zmask, 0.0, 0.0, t->coeff_re, t->coeff_im));
    }
    if (in->stream != out->stream) {
        cudaError_t e = cudaStreamSynchronize(in->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "sync"));
    }
    return publish(launch_pauli_apply(out, in, t->xmask, t->zmask, t->coeff_re, t->coeff_im));
}

qi_status qi_pauli_apply_normalised(qi_state *s, const qi_pauli_term *t) {
    QI_LOCK(s);
    if (!t) return publish(err(QI_ERR_NULL_ARGUMENT));
    Status st = validate_pauli(s->n, *t);
    if (!st.ok()) return publish(st);
    st = launch_pauli_exp(s, t->xmask, t->zmask, 0.0, 0.0, 1.0, 0.0);
    if (!st.ok()) return publish(st);
    st = state_normalise_device_async(s);
    if (!st.ok()) return publish(st);
    int flag = 0;
    st = state_read_flag(s, &flag);
    if (!st.ok()) return publish(st);
    if (flag) return publish(err(QI_ERR_ZERO_NORM));
    return publish(ok_status());
}

qi_status qi_pauli_apply_exp_factor(qi_state *s, const qi_pauli_term *t, double fre, double fim) {
    QI_LOCK(s);
    if (!t) return publish(err(QI_ERR_NULL_ARGUMENT));
    Status st = validate_pauli(s->n, *t);
    if (!st.ok()) return publish(st);
    const double ar = t->coeff_re * fre - t->coeff_im * fim;   // alpha = coefficient * factor
    const double ai = t->coeff_re * fim + t->coeff_im * fre;
    if ((t->xmask | t->zmask) == 0) {   // identity string: state * exp(alpha)
        const double e = std::exp(ar);
        return publish(state_scale_async(s, e * std::cos(ai), e * std::sin(ai)));
    }
    double cre, cim, sre, sim;
    exp_coeffs(ar, ai, cre, cim, sre, sim);
    return publish(launch_pauli_exp(s, t->xmask, t->zmask, cre, cim, sre, sim));
}

qi_status qi_pauli_apply_exp(qi_state *s, const qi_pauli_term *t) {
    return qi_pauli_apply_exp_factor(s, t, 1.0, 0.0);
}

qi_status qi_pauli_apply_exp_neg_i_dt(qi_state *s, const qi_pauli_term *t, double dt) {
    if (!t) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (t->coeff_im != 0.0) {   // pauli_string.rs:282-284
        Status e = err(QI_ERR_INVALID_PAULI_COEFFICIENT);
        e.re = t->coeff_re;
        e.im = t->coeff_im;
        return publish(e);
    }
    return qi_pauli_apply_exp_factor(s, t, 0.0, -dt);
}

qi_status qi_sumop_apply(qi_state *out, qi_state *in, const qi_pauli_term *terms, int64_t n_terms) {
    QI_LOCK(out);
    if (!in || (!terms && n_terms > 0)) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (in->n != out->n) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, in->n));
    if (in->prec != out->prec) return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "equal precisions required"));
    if (in == out) return publish(err(QI_ERR_UNSUPPORTED, -1, -1, "SumOp::apply needs distinct input and output"));
    for (int64_t k = 0; k < n_terms; ++k) {
        Status st = validate_pauli(in->n, terms[k]);
        if (!st.ok()) return publish(st);
    }
    if (in->stream != out->stream) {
        cudaError_t e = cudaStreamSynchronize(in->stream);
        if (e != cudaSuccess) return publish(cuda_status(e, "sync"));
    }
    if (n_terms == 0) {   // empty SumOp: state * 0.0 (pauli_string.rs:454-457)
        Status st = state_copy_async(out, in);
        if (!st.ok()) return publish(st);
        return publish(state_scale_async(out, 0.0, 0.0));
    }
    Status st = sumop_apply(out, in, terms, n_terms);
    if (!st.ok()) return publish(st);
    int flag = 0;
    st = state_read_flag(out, &flag);
    if (st.ok() && flag == 2) st = err(QI_ERR_TIMEOUT, -1, -1, "SumOp::apply: a device wait timed out");
    return publish(st);
}

qi_status qi_sumop_expectation(qi_state *s, const qi_pauli_term *terms, int64_t n_terms, double out[2]) {
    QI_LOCK(s);
    if (!out || (!terms && n_terms > 0)) return publish(err(QI_ERR_NULL_ARGUMENT));
    out[0] = out[1] = 0.0;
    if (n_terms == 0) return publish(ok_status());   // pauli_string.rs:486-489
    for (int64_t k = 0; k < n_terms; ++k) {
        Status st = validate_pauli(s->n, terms[k]);
        if (!st.ok()) return publish(st);
    }
    return publish(sumop_expectation(s, terms, n_terms, out));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// SumOp expectation without device allocation.
//
// For callers that cannot allocate GPU memory at the point of the call — a
// host application that has handed the whole device to its own memory pool,
// or a solver loop that must not insert the device-wide synchronisation that
// cudaMalloc/cudaFree imply — this entry point reads the caller's amplitude
// buffer and keeps all of its temporaries (per-block partial sums, the
// accumulated result and the grouped term table) in one fixed, statically
// allocated device array, kNoAllocScratchBytes bytes per GPU that loads the
// library, held until process exit.  Limits: at most kNoAllocMaxTerms terms,
// and at most kNoAllocMaxGroupTerms terms sharing one X mask.
// Every call reuses the same array: two calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it.
// ---------------------------------------------------------------------------
namespace qi {

constexpr int kNoAllocMaxTerms = 4096;
constexpr int kNoAllocMaxGroupTerms = 2048;   // 48 KB of dynamic shared memory per group kernel
constexpr size_t kNoAllocPartialsOff = 0;
constexpr size_t kNoAllocResultOff = (size_t)kReduceBlocks * 4 * sizeof(double);        // 38912, 256-aligned
constexpr size_t kNoAllocTermsOff = kNoAllocResultOff + 256;
constexpr size_t kNoAllocScratchBytes = kNoAllocTermsOff + (size_t)kNoAllocMaxTerms * sizeof(GroupTerm);   // 137472

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64] = {nullptr};   // device address of g_noalloc_scratch, per device ordinal

// Device address of the scratch array on the current device.  Set-up on the first call per
// device, with that device current: cudaGetSymbolAddress, and the shared-memory opt-in of the
// group kernels (a group of kNoAllocMaxGroupTerms terms needs 48 KB of dynamic shared memory
// plus the kernel's static block-sum space, just above the default window).  The address is
// cached for the life of the process; a cudaDeviceReset between calls is not supported.
static Status noalloc_scratch(int dev, void **out) {
    if (dev < 0 || dev >= 64) return err(QI_ERR_UNSUPPORTED, dev, -1, "device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        QI_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        Status st = group_expect_smem(true, (size_t)kNoAllocMaxGroupTerms * sizeof(GroupTerm));
        if (st.ok()) st = group_expect_smem(false, (size_t)kNoAllocMaxGroupTerms * sizeof(GroupTerm));
        if (!st.ok()) return st;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return ok_status();
}

// The caller's buffer and stream must belong to the current device (the scratch address
// is the current device's).
static Status noalloc_check_device(int dev, const void *amps, cudaStream_t stream) {
    cudaPointerAttributes pa;
    cudaError_t e = cudaPointerGetAttributes(&pa, amps);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return err(QI_ERR_INVALID_INPUT_VALUE, -1, dev, "qi_sumop_expectation_noalloc: amps is not a device pointer");
    }
    if ((pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) || pa.device != dev)
        return err(QI_ERR_INVALID_INPUT_VALUE, pa.device, dev,
                   "qi_sumop_expectation_noalloc: amps must be device memory of the current device");
    if (stream) {
        int sdev = -1;
        e = cudaStreamGetDevice(stream, &sdev);
        if (e != cudaSuccess) return cuda_status(e, "qi_sumop_expectation_noalloc: cudaStreamGetDevice");
        if (sdev != dev)
            return err(QI_ERR_INVALID_INPUT_VALUE, sdev, dev,
                       "qi_sumop_expectation_noalloc: cuda_stream belongs to another device");
    }
    return ok_status();
}

}  // namespace qi

extern "C" qi_status qi_sumop_expectation_noalloc(const void *amps, int32_t num_qubits, int32_t precision,
                                                  const qi_pauli_term *terms, int64_t n_terms, void *cuda_stream,
                                                  double out[2]) {
    if (!amps || !out || (!terms && n_terms > 0)) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (num_qubits <= 0 || num_qubits > 40) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, num_qubits));
    if (precision != QI_F32 && precision != QI_F64) return publish(err(QI_ERR_INVALID_INPUT_VALUE, precision));
    if (n_terms < 0 || n_terms > kNoAllocMaxTerms)
        return publish(err(QI_ERR_INVALID_INPUT_VALUE, n_terms, kNoAllocMaxTerms,
                           "qi_sumop_expectation_noalloc: at most 4096 terms (fixed scratch array)"));
    out[0] = out[1] = 0.0;
    if (n_terms == 0) return publish(ok_status());   // pauli_string.rs:486-489
    for (int64_t k = 0; k < n_terms; ++k) {
        Status st = validate_pauli(num_qubits, terms[k]);
        if (!st.ok()) return publish(st);
    }
    // group by X mask into fixed host arrays (no heap)
    static thread_local uint64_t gx[kNoAllocMaxTerms];
    static thread_local int32_t gcount[kNoAllocMaxTerms], gfirst[kNoAllocMaxTerms], term_group[kNoAllocMaxTerms];
    static thread_local GroupTerm packed[kNoAllocMaxTerms];
    int ng = 0;
    for (int64_t k = 0; k < n_terms; ++k) {
        int gi = 0;
        while (gi < ng && gx[gi] != terms[k].xmask) ++gi;
        if (gi == ng) { gx[ng] = terms[k].xmask; gcount[ng] = 0; ++ng; }
        term_group[k] = gi;
        ++gcount[gi];
    }
    for (int gi = 0, off = 0; gi < ng; ++gi) {
        if (gcount[gi] > kNoAllocMaxGroupTerms)
            return publish(err(QI_ERR_INVALID_INPUT_VALUE, gcount[gi], kNoAllocMaxGroupTerms,
                               "qi_sumop_expectation_noalloc: at most 2048 terms per X mask"));
        gfirst[gi] = off;
        off += gcount[gi];
        gcount[gi] = 0;
    }
    for (int64_t k = 0; k < n_terms; ++k) {
        const int gi = term_group[k];
        double pr, pi;
        minus_i_pow(__builtin_popcountll(terms[k].xmask & terms[k].zmask), pr, pi);
        GroupTerm t;
        t.zmask = terms[k].zmask;
        t.re = terms[k].coeff_re * pr - terms[k].coeff_im * pi;
        t.im = terms[k].coeff_re * pi + terms[k].coeff_im * pr;
        packed[gfirst[gi] + gcount[gi]++] = t;
    }
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    int dev = 0;
    cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess) return publish(cuda_status(de, "cudaGetDevice"));
    Status st = noalloc_check_device(dev, amps, stream);
    if (!st.ok()) return publish(st);
    void *scratch = nullptr;
    st = noalloc_scratch(dev, &scratch);
    if (!st.ok()) return publish(st);
    double *partials = (double *)((char *)scratch + kNoAllocPartialsOff);
    double *result = (double *)((char *)scratch + kNoAllocResultOff);
    GroupTerm *d_terms = (GroupTerm *)((char *)scratch + kNoAllocTermsOff);
    cudaError_t e = cudaMemcpyAsync(d_terms, packed, (size_t)n_terms * sizeof(GroupTerm), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(result, 0, 2 * sizeof(double), stream);   // the accumulator starts at zero
    if (e != cudaSuccess) return publish(cuda_status(e, "qi_sumop_expectation_noalloc"));
    const uint64_t dim = 1ull << num_qubits;
    for (int gi = 0; gi < ng; ++gi) {
        GroupHdr h;
        h.xmask = gx[gi];
        h.first = gfirst[gi];
        h.count = gcount[gi];
        const uint64_t work = h.xmask ? (dim >> 1) : dim;
        const unsigned nb = (unsigned)std::min<uint64_t>(std::max<uint64_t>((work + kReduceThreads - 1) / kReduceThreads, 1),
                                                         kReduceBlocks);
        const size_t sm = (size_t)h.count * sizeof(GroupTerm);
        if (precision == QI_F32)
            k_group_expect<float><<<nb, kReduceThreads, sm, stream>>>((const float2 *)amps, dim, h, d_terms, partials);
        else
            k_group_expect<double><<<nb, kReduceThreads, sm, stream>>>((const double2 *)amps, dim, h, d_terms, partials);
        k_accumulate<<<1, 256, 0, stream>>>(partials, (int)nb, result);
        count_launch(2);
        st = check_launch("qi_sumop_expectation_noalloc");
        if (!st.ok()) return publish(st);
    }
    double host_res[2] = {0.0, 0.0};
    e = cudaMemcpyAsync(host_res, result, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "qi_sumop_expectation_noalloc"));
    out[0] = host_res[0];
    out[1] = host_res[1];
    return publish(ok_status());
}
