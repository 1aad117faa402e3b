// qi_fused.cu — fused k-qubit blocks on CUDA cores, and k-qubit diagonal blocks.
//
// A fused block is a dense 2^k x 2^k complex matrix U on sorted target qubits
// t_0 < ... < t_{k-1} (local bit j <-> qubit t_j).  Applying it is one HBM
// pass: out[r'][c] = sum_r U[r'][r] in[r][c], where r is the target-bit
// pattern of an amplitude index and c the pattern of the other qubits.
//
// Tiling: a CTA tile holds all 2^k target patterns for 2^nb "columns", the
// columns being the nb lowest non-target qubits.  Every qubit below the
// highest of those is in the tile, so the tile is 2^h contiguous runs of
// global memory (h = targets above that point): the load and store are
// coalesced 16-byte accesses.  In shared memory the tile is stored
// transposed as [2^k rows][2^nb + 1 columns] (one padding element per row):
// the scatter from address order and the per-column reads of the compute
// phase are both free of bank conflicts.
// Compute: thread j owns column j, holds its 2^k amplitudes in registers and
// forms the matrix-vector product with U read from shared memory (broadcast).
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <algorithm>

namespace qi {

struct FusedParams {
    uint64_t ntiles;
    int32_t k, nb, L;        // targets, column bits, width of the contiguous low run
    int32_t nlow_t;          // targets below L
    int32_t nhigh;           // targets at or above L
    int8_t low_t[8];         // target positions below L (ascending)
    int8_t high_t[8];        // target positions >= L (ascending)
    int8_t free_pos[64];     // qubits outside the tile (ascending): tile index -> base address
    int32_t nfree;
};

template <typename T>
__device__ __forceinline__ void tile_coords(const FusedParams &p, uint32_t x, uint32_t &r, uint32_t &c, uint64_t &goff) {
    // x: tile-local index in address order = (xh << L) | xl
    const uint32_t xl = x & ((1u << p.L) - 1), xh = x >> p.L;
    // r_lo = pext(xl, low targets); c = xl with low-target bits removed
    uint32_t rl = 0, cc = xl;
    for (int j = p.nlow_t - 1; j >= 0; --j) {
        const int q = p.low_t[j];
        rl = (rl << 1) | ((xl >> q) & 1u);
        cc = ((cc >> (q + 1)) << q) | (cc & ((1u << q) - 1));
    }
    r = rl | (xh << p.nlow_t);
    c = cc;
    uint64_t g = xl;
    for (int j = 0; j < p.nhigh; ++j) g |= (uint64_t)((xh >> j) & 1u) << p.high_t[j];
    goff = g;
}

template <typename T, int K, int B>
__global__ void __launch_bounds__(1 << B) k_fused_simt(typename Cx<T>::V2 *a, const typename Cx<T>::V2 *mat,
                                                       FusedParams p) {
    using V2 = typename Cx<T>::V2;
    constexpr int R = 1 << K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V2 *sm_mat = reinterpret_cast<V2 *>(smem_raw);
    V2 *tile = sm_mat + R * R;
    const int ncol = 1 << p.nb;
    const int ld = ncol + 1;
    const uint32_t tile_amps = (uint32_t)R << p.nb;

    for (int i = threadIdx.x; i < R * R; i += blockDim.x) sm_mat[i] = mat[i];

    for (uint64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        // base address of this tile: deposit t into the non-tile qubits
        uint64_t base = 0;
        for (int j = 0; j < p.nfree; ++j) base |= ((t >> j) & 1ull) << p.free_pos[j];
        __syncthreads();   // previous tile fully stored / matrix loaded
        // load (qubit 0 is always in the tile, so pairs (x, x+1) are adjacent)
        if constexpr (sizeof(T) == 4) {
            const float4 *a4 = reinterpret_cast<const float4 *>(a);
            for (uint32_t v = threadIdx.x; v < tile_amps / 2; v += blockDim.x) {
                uint32_t r0, c0, r1, c1;
                uint64_t g0, g1;
                tile_coords<T>(p, 2 * v, r0, c0, g0);
                tile_coords<T>(p, 2 * v + 1, r1, c1, g1);
                float4 q = __ldcs(a4 + ((base | g0) >> 1));
                tile[r0 * ld + c0] = make_float2(q.x, q.y);
                tile[r1 * ld + c1] = make_float2(q.z, q.w);
            }
        } else {
            for (uint32_t x = threadIdx.x; x < tile_amps; x += blockDim.x) {
                uint32_t r, c;
                uint64_t g;
                tile_coords<T>(p, x, r, c, g);
                tile[r * ld + c] = __ldcs(a + (base | g));
            }
        }
        __syncthreads();
        // compute: column j
        for (int j = threadIdx.x; j < ncol; j += blockDim.x) {
            V2 in[R];
#pragma unroll
            for (int r = 0; r < R; ++r) in[r] = tile[r * ld + j];
#pragma unroll 1
            for (int ro = 0; ro < R; ++ro) {
                const V2 *mrow = sm_mat + ro * R;
                T accx = 0, accy = 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const V2 m = mrow[r];
                    accx = ::fma(m.x, in[r].x, accx);
                    accx = ::fma(-m.y, in[r].y, accx);
                    accy = ::fma(m.x, in[r].y, accy);
                    accy = ::fma(m.y, in[r].x, accy);
                }
                tile[ro * ld + j] = Cx<T>::make(accx, accy);
            }
        }
        __syncthreads();
        // store
        if constexpr (sizeof(T) == 4) {
            float4 *a4 = reinterpret_cast<float4 *>(a);
            for (uint32_t v = threadIdx.x; v < tile_amps / 2; v += blockDim.x) {
                uint32_t r0, c0, r1, c1;
                uint64_t g0, g1;
                tile_coords<T>(p, 2 * v, r0, c0, g0);
                tile_coords<T>(p, 2 * v + 1, r1, c1, g1);
                const float2 u = tile[r0 * ld + c0], w = tile[r1 * ld + c1];
                __stcs(a4 + ((base | g0) >> 1), make_float4(u.x, u.y, w.x, w.y));
            }
        } else {
            for (uint32_t x = threadIdx.x; x < tile_amps; x += blockDim.x) {
                uint32_t r, c;
                uint64_t g;
                tile_coords<T>(p, x, r, c, g);
                __stcs(a + (base | g), tile[r * ld + c]);
            }
        }
    }
}

// Diagonal block: a[i] *= phase[pext(i, targets)].
template <typename T>
__global__ void __launch_bounds__(256) k_diagk(typename Cx<T>::V2 *a, uint64_t dim, const typename Cx<T>::V2 *ph,
                                               int k, uint64_t tmask) {
    using V2 = typename Cx<T>::V2;
    __shared__ V2 sph[1 << 10];
    const int R = 1 << k;
    for (int i = threadIdx.x; i < R; i += blockDim.x) sph[i] = ph[i];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
        // pext(i, tmask)
        uint32_t r = 0;
        uint64_t m = tmask;
        int b = 0;
        while (m) {
            const int q = __ffsll((long long)m) - 1;
            r |= (uint32_t)((i >> q) & 1ull) << b;
            ++b;
            m &= m - 1;
        }
        V2 v = a[i];
        a[i] = Cx<T>::mul(sph[r], v);
    }
}

static int column_bits(int prec, int k) {
    if (prec == QI_F32) return k <= 5 ? 8 : 7;
    return k <= 4 ? 8 : (k == 5 ? 7 : 6);
}

template <typename T, int K, int B>
static Status launch_simt_t(qi_state *s, const FusedParams &p, const void *d_mat) {
    constexpr int R = 1 << K;
    const size_t smem = (size_t)R * R * sizeof(typename Cx<T>::V2) +
                        (size_t)R * ((1 << p.nb) + 1) * sizeof(typename Cx<T>::V2);
    auto kern = k_fused_simt<T, K, B>;
    static bool attr_set = false;   // per instantiation
    if (!attr_set) {
        QI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set = true;
    }
    int dev_sms = 152;
    uint64_t grid = p.ntiles;
    const uint64_t cap = (uint64_t)dev_sms * (smem <= 70 * 1024 ? 3 : (smem <= 110 * 1024 ? 2 : 1)) * 4;
    if (grid > cap) grid = cap;
    kern<<<(unsigned)grid, 1 << B, smem, s->stream>>>((typename Cx<T>::V2 *)s->amps,
                                                     (const typename Cx<T>::V2 *)d_mat, p);
    count_launch();
    return check_launch("k_fused_simt");
}

Status launch_fused(qi_state *s, int k, const int32_t *targets, const void *d_mat, int use_tc) {
    (void)use_tc;
    const int n = s->n;
    if (k < 1 || k > 6 || k > n) return err(QI_ERR_INVALID_INPUT_VALUE, k, n, "fused block width");
    if (s->prec == QI_F64 && k > 5) return err(QI_ERR_UNSUPPORTED, k, -1, "FP64 fused blocks are limited to k <= 5");
    FusedParams p;
    std::memset(&p, 0, sizeof(p));
    p.k = k;
    uint64_t tmask = 0;
    for (int j = 0; j < k; ++j) tmask |= 1ull << targets[j];
    const int bmax = column_bits(s->prec, k);
    p.nb = std::min(bmax, n - k);
    // columns: the nb lowest non-target qubits; L = one past the highest of them
    int got = 0, q = 0;
    while (got < p.nb) {
        if (!((tmask >> q) & 1ull)) ++got;
        ++q;
    }
    // if nb == 0 every qubit is a target: L = number of low targets contiguous from 0
    if (p.nb == 0) q = 0;
    // extend L over targets directly above the columns (still contiguous)
    while (q < n && ((tmask >> q) & 1ull)) ++q;
    p.L = q;
    p.nlow_t = 0;
    p.nhigh = 0;
    for (int j = 0; j < k; ++j) {
        if (targets[j] < p.L) p.low_t[p.nlow_t++] = (int8_t)targets[j];
        else p.high_t[p.nhigh++] = (int8_t)targets[j];
    }
    p.nfree = 0;
    for (int qq = 0; qq < n; ++qq)
        if (qq >= p.L && !((tmask >> qq) & 1ull)) p.free_pos[p.nfree++] = (int8_t)qq;
    p.ntiles = 1ull << p.nfree;
    if (p.nfree != n - k - p.nb) return err(QI_ERR_UNKNOWN, p.nfree, n - k - p.nb, "tile decomposition");
    if (s->prec == QI_F32) {
        switch (k) {
        case 1: return launch_simt_t<float, 1, 8>(s, p, d_mat);
        case 2: return launch_simt_t<float, 2, 8>(s, p, d_mat);
        case 3: return launch_simt_t<float, 3, 8>(s, p, d_mat);
        case 4: return launch_simt_t<float, 4, 8>(s, p, d_mat);
        case 5: return launch_simt_t<float, 5, 8>(s, p, d_mat);
        default: return launch_simt_t<float, 6, 7>(s, p, d_mat);
        }
    }
    switch (k) {
    case 1: return launch_simt_t<double, 1, 8>(s, p, d_mat);
    case 2: return launch_simt_t<double, 2, 8>(s, p, d_mat);
    case 3: return launch_simt_t<double, 3, 8>(s, p, d_mat);
    case 4: return launch_simt_t<double, 4, 8>(s, p, d_mat);
    default: return launch_simt_t<double, 5, 7>(s, p, d_mat);
    }
}

Status launch_diagk(qi_state *s, int k, const int32_t *targets, const void *d_phases) {
    if (k < 1 || k > 10) return err(QI_ERR_INVALID_INPUT_VALUE, k, -1, "diagonal block width");
    uint64_t tmask = 0;
    for (int j = 0; j < k; ++j) tmask |= 1ull << targets[j];
    uint64_t g = (s->dim() + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    if (s->prec == QI_F32)
        k_diagk<float><<<(unsigned)g, 256, 0, s->stream>>>((float2 *)s->amps, s->dim(), (const float2 *)d_phases, k, tmask);
    else
        k_diagk<double><<<(unsigned)g, 256, 0, s->stream>>>((double2 *)s->amps, s->dim(), (const double2 *)d_phases, k,
                                                           tmask);
    count_launch();
    return check_launch("k_diagk");
}

}  // namespace qi
