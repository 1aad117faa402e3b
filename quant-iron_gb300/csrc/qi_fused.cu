// qi_fused.cu — fused k-qubit blocks on CUDA cores, and k-qubit diagonal blocks.
//
// A fused block is a dense 2^k x 2^k complex matrix U on sorted target qubits
// t_0 < ... < t_{k-1} (local bit j <-> qubit t_j).  Applying it is one HBM
// pass: out[r'][c] = sum_r U[r'][r] in[r][c], where r is the target-bit
// pattern of an amplitude index and c the pattern of the other qubits.
//
// Tiles and their shared-memory layout are described in qi_tile.cuh.  This
// file holds the CUDA-core kernel (any k <= 6, FP32 or FP64) and the
// diagonal-block kernel; the tensor-core kernel is in qi_fused_tc.cu.
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_tile.cuh"

#include <algorithm>
#include <atomic>

namespace qi {

constexpr int kSimtThreads = 256;

// Rows [r0, r1) of U times the column `in`, written to column j of the tile.
template <typename T, int R>
__device__ __forceinline__ void column_rows(const typename Cx<T>::V2 *sm_mat, const typename Cx<T>::V2 (&in)[R], int r0,
                                            int r1, typename Cx<T>::V2 *S, const TileGeom &g, int j) {
    using V2 = typename Cx<T>::V2;
#pragma unroll 1
    for (int ro = r0; ro < r1; ++ro) {
        const V2 *mrow = sm_mat + ro * R;
        T ax = 0, ay = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const V2 m = mrow[r];
            ax = ::fma(m.x, in[r].x, ax);
            ax = ::fma(-m.y, in[r].y, ax);
            ay = ::fma(m.x, in[r].y, ay);
            ay = ::fma(m.y, in[r].x, ay);
        }
        S[tile_sidx(g, ro, j)] = Cx<T>::make(ax, ay);
    }
}

// Fused block on CUDA cores.  Persistent CTAs walk the tiles; tile t + 2*grid
// is prefetched with cp.async into the buffer tile t just released, so loads
// overlap the matrix-vector work of the other buffer.  Each column's 2^K
// amplitudes are read into registers, multiplied by U (read from shared
// memory as a broadcast) and written back in place; when several threads
// share a column (few columns per tile) each computes a slice of the rows,
// after all of them have read the inputs.
template <typename T, int K>
__global__ void __launch_bounds__(kSimtThreads) k_fused_simt(typename Cx<T>::V2 *a, const typename Cx<T>::V2 *mat,
                                                             TileGeom g) {
    using V2 = typename Cx<T>::V2;
    constexpr int R = 1 << K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V2 *sm_mat = reinterpret_cast<V2 *>(smem_raw);
    TileIterTab *tab = reinterpret_cast<TileIterTab *>(sm_mat + R * R);
    V2 *S0 = reinterpret_cast<V2 *>(tab + 32);
    const uint32_t tile_amps = 1u << (K + g.nb);
    V2 *S1 = S0 + tile_amps;
    const int tid = threadIdx.x;
    const int ncol = 1 << g.nb;

    for (int i = tid; i < R * R; i += kSimtThreads) sm_mat[i] = mat[i];
    const TileWalk w = tile_walk_init(g, tid, kSimtThreads);
    if (tid < w.iters) tile_iter_fill(g, kSimtThreads, tid, tab);
    __syncthreads();

    // column / row-slice assignment
    const int split = ncol >= kSimtThreads ? 1 : min(R, kSimtThreads / ncol);
    const int rows_per = R / split;
    const int col0 = tid % (ncol >= kSimtThreads ? kSimtThreads : ncol);
    const int part = ncol >= kSimtThreads ? 0 : tid / ncol;
    const bool computes = part < split;

    uint64_t t = blockIdx.x;
    if (t < g.ntiles) tile_load_async(g, w, tab, a, tile_base(g, t), S0);
    cp_async_commit();
    if (t + gridDim.x < g.ntiles) tile_load_async(g, w, tab, a, tile_base(g, t + gridDim.x), S1);
    cp_async_commit();
    for (int it = 0; t < g.ntiles; ++it, t += gridDim.x) {
        V2 *S = (it & 1) ? S1 : S0;
        cp_async_wait<1>();
        __syncthreads();
        // Every thread runs the same number of column steps and reaches every
        // barrier: the computing threads can share a warp with idle ones when a
        // tile has fewer than 32 amplitudes.
        for (int j0 = 0; j0 < ncol; j0 += kSimtThreads) {
            const int j = j0 + col0;
            const bool act = computes && j < ncol;
            V2 in[R];
            if (act) {
#pragma unroll
                for (int r = 0; r < R; ++r) in[r] = S[tile_sidx(g, r, j)];
            }
            if (split > 1) __syncthreads();   // every row slice has read the column
            if (act) column_rows<T, R>(sm_mat, in, part * rows_per, (part + 1) * rows_per, S, g, j);
        }
        __syncthreads();
        tile_store(g, w, tab, a, tile_base(g, t), S);
        __syncthreads();
        const uint64_t nt = t + 2ull * gridDim.x;
        if (nt < g.ntiles) tile_load_async(g, w, tab, a, tile_base(g, nt), S);
        cp_async_commit();
    }
    cp_async_wait<0>();
}

// Diagonal block: a[i] *= phase[pext(i, targets)].  Each thread handles
// kDiagUnroll independent 16-byte vectors per iteration (2 FP32 or 1 FP64
// amplitude each) so that enough bytes are in flight to saturate HBM.
constexpr int kDiagUnroll = 4;

struct DiagParams {
    uint64_t nvec;       // number of 16-byte vectors
    int32_t k;
    int8_t pos[10];      // target positions, ascending
};

__device__ __forceinline__ uint32_t pext_pos(uint64_t i, const DiagParams &p) {
    uint32_t r = 0;
#pragma unroll
    for (int b = 0; b < 10; ++b)
        if (b < p.k) r |= (uint32_t)((i >> p.pos[b]) & 1ull) << b;
    return r;
}

template <typename T>
__global__ void __launch_bounds__(256) k_diagk(typename Cx<T>::V2 *a, const typename Cx<T>::V2 *ph, DiagParams p) {
    using V2 = typename Cx<T>::V2;
    __shared__ V2 sph[1 << 10];
    const int R = 1 << p.k;
    for (int i = threadIdx.x; i < R; i += blockDim.x) sph[i] = ph[i];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; base < p.nvec; base += stride * kDiagUnroll) {
        if constexpr (sizeof(T) == 4) {
            float4 *a4 = reinterpret_cast<float4 *>(a);
            float4 v[kDiagUnroll];
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u) {
                const uint64_t j = base + u * stride;
                if (j < p.nvec) v[u] = __ldcs(a4 + j);
            }
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u) {
                const uint64_t j = base + u * stride;
                if (j < p.nvec) {
                    const float2 x = Cx<float>::mul(sph[pext_pos(2 * j, p)], make_float2(v[u].x, v[u].y));
                    const float2 y = Cx<float>::mul(sph[pext_pos(2 * j + 1, p)], make_float2(v[u].z, v[u].w));
                    __stcs(a4 + j, make_float4(x.x, x.y, y.x, y.y));
                }
            }
        } else {
            double2 v[kDiagUnroll];
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u) {
                const uint64_t j = base + u * stride;
                if (j < p.nvec) v[u] = __ldcs(reinterpret_cast<const double2 *>(a) + j);
            }
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u) {
                const uint64_t j = base + u * stride;
                if (j < p.nvec) __stcs(reinterpret_cast<double2 *>(a) + j, Cx<double>::mul(sph[pext_pos(j, p)], v[u]));
            }
        }
    }
}

// Column bits per tile: 2^(K + nb) amplitudes = 32 KB per buffer.
static int column_bits(int prec, int k) { return (prec == QI_F32 ? 12 : 11) - k; }

template <typename T, int K>
static Status launch_simt_t(qi_state *s, const TileGeom &g, const void *d_mat) {
    constexpr int R = 1 << K;
    using V2 = typename Cx<T>::V2;
    const size_t smem = (size_t)R * R * sizeof(V2) + 32 * sizeof(TileIterTab) + 2 * ((size_t)R << g.nb) * sizeof(V2);
    auto kern = k_fused_simt<T, K>;
    static std::atomic<bool> attr_set[64];   // per instantiation and device
    int dev = 0;
    QI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return err(QI_ERR_UNSUPPORTED, dev, 64, "device ordinal");
    if (!attr_set[dev].load()) {
        QI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set[dev].store(true);
    }
    int per_sm = 0;
    QI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSimtThreads, smem));
    if (per_sm < 1) per_sm = 1;
    uint64_t grid = g.ntiles;
    const uint64_t cap = (uint64_t)152 * per_sm;
    if (grid > cap) grid = cap;
    kern<<<(unsigned)grid, kSimtThreads, smem, s->stream>>>((V2 *)s->amps, (const V2 *)d_mat, g);
    count_launch();
    return check_launch("k_fused_simt");
}

Status launch_fused_simt(qi_state *s, int k, const int32_t *targets, const void *d_mat) {
    const int n = s->n;
    const int nb = std::min(column_bits(s->prec, k), n - k);
    const TileGeom g = make_tile_geom(n, k, targets, nb);
    if (g.nfree != n - k - nb) return err(QI_ERR_UNKNOWN, g.nfree, n - k - nb, "tile decomposition");
    if (s->prec == QI_F32) {
        switch (k) {
        case 1: return launch_simt_t<float, 1>(s, g, d_mat);
        case 2: return launch_simt_t<float, 2>(s, g, d_mat);
        case 3: return launch_simt_t<float, 3>(s, g, d_mat);
        case 4: return launch_simt_t<float, 4>(s, g, d_mat);
        case 5: return launch_simt_t<float, 5>(s, g, d_mat);
        default: return launch_simt_t<float, 6>(s, g, d_mat);
        }
    }
    switch (k) {
    case 1: return launch_simt_t<double, 1>(s, g, d_mat);
    case 2: return launch_simt_t<double, 2>(s, g, d_mat);
    case 3: return launch_simt_t<double, 3>(s, g, d_mat);
    case 4: return launch_simt_t<double, 4>(s, g, d_mat);
    default: return launch_simt_t<double, 5>(s, g, d_mat);
    }
}

Status launch_fused(qi_state *s, int k, const int32_t *targets, const void *d_mat, const void *d_tc, int use_tc,
                    const void *poly) {
    const int n = s->n;
    if (k < 1 || k > 6 || k > n) return err(QI_ERR_INVALID_INPUT_VALUE, k, n, "fused block width");
    if (s->prec == QI_F64 && k > 5) return err(QI_ERR_UNSUPPORTED, k, -1, "FP64 fused blocks are limited to k <= 5");
    if (use_tc && d_tc && s->prec == QI_F32 && k >= 5 && n >= k + 7) return launch_fused_tc(s, k, targets, d_tc, poly);
    if (poly) return err(QI_ERR_UNKNOWN, k, n, "a phase polynomial rides only on a tensor-core block");
    return launch_fused_simt(s, k, targets, d_mat);
}

Status launch_diagk(qi_state *s, int k, const int32_t *targets, const void *d_phases) {
    if (k < 1 || k > 10) return err(QI_ERR_INVALID_INPUT_VALUE, k, -1, "diagonal block width");
    DiagParams p;
    std::memset(&p, 0, sizeof(p));
    p.k = k;
    for (int j = 0; j < k; ++j) p.pos[j] = (int8_t)targets[j];
    const bool f32 = s->prec == QI_F32;
    p.nvec = f32 ? (s->dim() >> 1) : s->dim();
    if (f32 && s->n < 1) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n);
    uint64_t g = (p.nvec + 256ull * kDiagUnroll - 1) / (256ull * kDiagUnroll);
    if (g < 1) g = 1;
    if (g > 152 * 8) g = 152 * 8;
    if (f32) k_diagk<float><<<(unsigned)g, 256, 0, s->stream>>>((float2 *)s->amps, (const float2 *)d_phases, p);
    else k_diagk<double><<<(unsigned)g, 256, 0, s->stream>>>((double2 *)s->amps, (const double2 *)d_phases, p);
    count_launch();
    return check_launch("k_diagk");
}

}  // namespace qi
