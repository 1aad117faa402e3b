// qi_fused_tc.cu — fused k-qubit blocks (k = 5, 6) on the 5th-generation
// tensor cores: tcgen05.mma kind::tf32, 3xTF32 split products, FP32
// accumulation in tensor memory.
//
// For a tile of 128 columns (the 7 lowest non-target qubits, plus the tile's
// fixed high bits) the block computes OUT[n][m] = sum_r U[n][r] X[r][m] with
// R = 2^k rows.  As a real GEMM with M = 128 (tile columns) and K = 2R:
//   A[m][k]   = Re X[k][m] (k < R), Im X[k-R][m] (k >= R)      — tensor memory
//   D_re[m][n] = sum_{k<R} A[m][k] Re U[n][k] + A[m][R+k] (-Im U[n][k])
//   D_im[m][n] = sum_{k<R} A[m][k] Im U[n][k] + A[m][R+k] ( Re U[n][k])
// so the B operands are the R x R blocks Re U, Im U and -Im U (K-major,
// shared memory), each N = R wide.  Every operand is split as x = hi + lo
// with hi = tf32(x) (round to nearest) and lo = tf32(x - hi); the products
// A_hi B_hi + A_hi B_lo + A_lo B_hi are accumulated in FP32, which keeps
// about 22 significant bits (the dropped A_lo B_lo term is ~2^-22 relative).
//
// Per tile (one CTA of 16 warps per SM, persistent):
//   16 warps read the tile (qi_tile.cuh, [row][column] layout), split hi/lo
//   and tcgen05.st A_hi / A_lo to TMEM (warp w: lanes 32*(w%4).., rows slice w/4)
//   one thread issues the 6 * 2R/8 MMAs (M128 x N=R x K8) and commits to an
//   mbarrier; every wait on it is bounded and a timeout sets the error flag
//   while the MMAs run: store tile t-1's output, cp.async-prefetch tile t+1
//   16 warps tcgen05.ld D and write OUT into the tile buffer.
// Tensor-memory columns: A_hi [0, 2R), A_lo [2R, 4R), D_re [4R, 5R), D_im [5R, 6R).
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_tile.cuh"

#include <algorithm>
#include <cmath>

namespace qi {

constexpr int kTcThreads = 512;   // 16 warps: 4 lane quarters x 4 row slices
constexpr uint32_t kWaitLimit = 1u << 22;   // bounded mbarrier wait (iterations of try_wait)

// ---------------------------------------------------------- PTX wrappers --
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false if the phase did not complete within kWaitLimit tries.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle (core matrices of
// 8 rows x 16 bytes), LBO = byte distance between core matrices along K,
// SBO = byte distance between 8-row groups along N; version field = 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    return d;
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tf32_idesc(uint32_t M, uint32_t N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return r;
}

// 32x32b tensor-memory stores / loads of N consecutive 32-bit columns.
template <int N>
__device__ __forceinline__ void tmem_st(uint32_t taddr, const uint32_t (&v)[N]);
template <>
__device__ __forceinline__ void tmem_st<8>(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
template <>
__device__ __forceinline__ void tmem_st<16>(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};\n" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
template <>
__device__ __forceinline__ void tmem_st<32>(uint32_t taddr, const uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};\n" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]),
        "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]),
        "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}
template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&v)[N]);
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t (&v)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr)
                 : "memory");
}
template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
template <>
__device__ __forceinline__ void tmem_ld<32>(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// ------------------------------------------------------------------ kernel
template <int K>
struct TcCfg {
    static constexpr int R = 1 << K;            // rows (target patterns)
    static constexpr int KR = 2 * R;            // real K of the GEMM
    static constexpr int H = R / 4;             // rows per warp slice
    static constexpr int BLK = R * R;           // floats per operand block
    static constexpr uint32_t LBO = 128;        // next core matrix along K
    static constexpr uint32_t SBO = (R / 4) * 128;   // next 8-row group along N
    static constexpr uint32_t TMEM_COLS = K == 6 ? 512 : 256;
    static constexpr uint32_t COL_AHI = 0, COL_ALO = KR, COL_D = 2 * KR;
    static constexpr size_t SMEM_B = 6 * BLK * sizeof(float);
    static constexpr size_t SMEM_TILE = (size_t)R * 128 * sizeof(float2);
    static constexpr size_t SMEM = SMEM_B + 2 * SMEM_TILE + 32 * sizeof(TileIterTab) + 64;
};

template <int K>
__global__ void __launch_bounds__(kTcThreads, 1) k_fused_tc(float2 *a, const float *blocks, TileGeom g, int *err_flag) {
    using C = TcCfg<K>;
    constexpr int R = C::R, H = C::H;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float *sB = reinterpret_cast<float *>(smem_raw);                      // 6 operand blocks
    float2 *S0 = reinterpret_cast<float2 *>(smem_raw + C::SMEM_B);
    float2 *S1 = S0 + R * 128;
    TileIterTab *tab = reinterpret_cast<TileIterTab *>(S1 + R * 128);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(tab + 32);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;   // lane quarter, row slice (0..3)

    // operand blocks -> shared memory (16-byte vectors), visible to the async proxy
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(blocks);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        for (int i = tid; i < (int)(C::SMEM_B / 16); i += kTcThreads) dst[i] = src[i];
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    const TileWalk w = tile_walk_init(g, tid, kTcThreads);
    if (tid < w.iters) tile_iter_fill(g, kTcThreads, tid, tab);
    if (tid == 0) {
        mbar_init(mbar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tmem_slot, C::TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int m = quarter * 32 + lane;   // this thread's tile column / TMEM lane

    // Descriptor of block 0 at K offset 0; every MMA adds a constant byte offset
    // (>> 4 into the start-address field, which cannot carry: blocks stay below 256 KB).
    const uint64_t desc0 = smem_desc(smem_u32(sB), C::LBO, C::SBO);
    const uint32_t idesc = tf32_idesc(128, R);

    // Software pipeline over this CTA's tiles (buffers alternate):
    //   wait tile t -> convert(t) -> issue MMA(t) -> store output of tile t-1 and
    //   prefetch tile t+1 into its buffer while the MMAs run -> wait -> epilogue(t)
    uint64_t t = blockIdx.x;
    if (t < g.ntiles) tile_load_async(g, w, tab, a, tile_base(g, t), S0);
    cp_async_commit();

    uint64_t prev_t = 0;
    int it = 0;
    for (; t < g.ntiles; ++it, t += gridDim.x) {
        float2 *S = (it & 1) ? S1 : S0;
        float2 *Sprev = (it & 1) ? S0 : S1;
        cp_async_wait<0>();
        __syncthreads();
        if (*abort_flag) break;

        // ---- convert: rows [half*H, half*H + H) of column m -> A_hi / A_lo
        {
            const int r0 = half * H;
            uint32_t hi_re[H], hi_im[H];
            float lo_re[H], lo_im[H];
#pragma unroll
            for (int i = 0; i < H; ++i) {
                const float2 x = S[tile_sidx(g, r0 + i, m)];
                hi_re[i] = tf32_rna(x.x);
                hi_im[i] = tf32_rna(x.y);
                lo_re[i] = x.x - __uint_as_float(hi_re[i]);
                lo_im[i] = x.y - __uint_as_float(hi_im[i]);
            }
            tmem_st<H>(tmem + lane_base + C::COL_AHI + r0, hi_re);
            tmem_st<H>(tmem + lane_base + C::COL_AHI + R + r0, hi_im);
            uint32_t lr[H], li[H];
#pragma unroll
            for (int i = 0; i < H; ++i) {
                lr[i] = tf32_rna(lo_re[i]);
                li[i] = tf32_rna(lo_im[i]);
            }
            tmem_st<H>(tmem + lane_base + C::COL_ALO + r0, lr);
            tmem_st<H>(tmem + lane_base + C::COL_ALO + R + r0, li);
            tmem_wait_st();
        }
        tc_fence_before();
        __syncthreads();

        // ---- MMA: one thread issues all products, commits to the mbarrier
        if (tid == 0) {
            tc_fence_after();
            // block order in shared memory: 0 Re hi, 1 Im hi, 2 -Im hi, 3 Re lo, 4 Im lo, 5 -Im lo
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const uint32_t d = tmem + C::COL_D + part * R;
#pragma unroll
                for (int prod = 0; prod < 3; ++prod) {
                    const uint32_t acol = (prod == 2) ? C::COL_ALO : C::COL_AHI;   // A_hi, A_hi, A_lo
                    const int bset = (prod == 1) ? 3 : 0;                          // B_hi, B_lo, B_hi
#pragma unroll
                    for (int j = 0; j < C::KR / 8; ++j) {
                        const int kk = 8 * j;
                        const bool first_half = kk < R;
                        const int blk = part == 0 ? (first_half ? 0 : 2) : (first_half ? 1 : 0);
                        const int koff = first_half ? kk : kk - R;
                        const uint32_t boff = (uint32_t)((bset + blk) * C::BLK * 4) + (uint32_t)(koff / 4) * C::LBO;
                        mma_tf32_ts(d, tmem + acol + kk, desc0 + (uint64_t)(boff >> 4), idesc,
                                    (prod == 0 && j == 0) ? 0u : 1u);
                    }
                }
            }
            mma_commit(mbar);
        }
        // ---- while the tensor cores run: store tile t-1's output, prefetch tile t+1
        if (it > 0) tile_store(g, w, tab, a, tile_base(g, prev_t), Sprev);
        __syncthreads();
        const uint64_t nt = t + gridDim.x;
        if (nt < g.ntiles) tile_load_async(g, w, tab, a, tile_base(g, nt), Sprev);
        cp_async_commit();
        // ---- wait for the products (bounded)
        if (!mbar_wait_bounded(mbar, (uint32_t)(it & 1))) {
            *abort_flag = 1;
            atomicExch(err_flag, 2);   // 2 = a bounded device wait ran out (1 is ZeroNorm)
        }
        tc_fence_after();
        __syncthreads();
        if (*abort_flag) break;

        // ---- epilogue: D rows [half*H, +H) of column m -> tile buffer
        {
            const int n0 = half * H;
            uint32_t dr[H], di[H];
            tmem_ld<H>(tmem + lane_base + C::COL_D + n0, dr);
            tmem_ld<H>(tmem + lane_base + C::COL_D + R + n0, di);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < H; ++i)
                S[tile_sidx(g, n0 + i, m)] = make_float2(__uint_as_float(dr[i]), __uint_as_float(di[i]));
        }
        tc_fence_before();
        prev_t = t;
    }
    cp_async_wait<0>();
    __syncthreads();
    // output of the last tile (skipped if the loop stopped on a timeout)
    if (it > 0 && !*abort_flag) tile_store(g, w, tab, a, tile_base(g, prev_t), ((it - 1) & 1) ? S1 : S0);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, C::TMEM_COLS);
    }
}

// ------------------------------------------------------------------- host
static inline float tf32_round_host(double x) {
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {   // finite: round to nearest (ties away), keep 10 mantissa bits
        u += 0x1000u;
        u &= 0xffffe000u;
    }
    std::memcpy(&f, &u, 4);
    return f;
}

void tc_blocks(int k, const double *U, std::vector<float> &out) {
    const int R = 1 << k;
    const uint32_t sbo = (uint32_t)(R / 4) * 128;
    const size_t base = out.size();
    out.resize(base + 6 * (size_t)R * R, 0.0f);
    for (int n = 0; n < R; ++n) {
        for (int kk = 0; kk < R; ++kk) {
            const double re = U[2 * ((size_t)n * R + kk)], im = U[2 * ((size_t)n * R + kk) + 1];
            const double vals[3] = {re, im, -im};
            const size_t off = ((size_t)(n / 8) * sbo + (size_t)(kk / 4) * 128 + (size_t)(n % 8) * 16 + (kk % 4) * 4) / 4;
            for (int b = 0; b < 3; ++b) {
                const float hi = tf32_round_host(vals[b]);
                const float lo = tf32_round_host(vals[b] - (double)hi);
                out[base + (size_t)b * R * R + off] = hi;
                out[base + (size_t)(3 + b) * R * R + off] = lo;
            }
        }
    }
}

template <int K>
static Status launch_tc_t(qi_state *s, const TileGeom &g, const void *d_tc) {
    using C = TcCfg<K>;
    static bool attr_set = false;
    if (!attr_set) {
        QI_CUDA(cudaFuncSetAttribute(k_fused_tc<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM));
        attr_set = true;
    }
    uint64_t grid = g.ntiles;
    if (grid > 152) grid = 152;
    k_fused_tc<K><<<(unsigned)grid, kTcThreads, C::SMEM, s->stream>>>((float2 *)s->amps, (const float *)d_tc, g,
                                                                      s->d_flag);
    count_launch();
    return check_launch("k_fused_tc");
}

Status launch_fused_tc(qi_state *s, int k, const int32_t *targets, const void *d_tc) {
    const int n = s->n;
    if (s->prec != QI_F32 || (k != 5 && k != 6) || n < k + 7)
        return err(QI_ERR_UNSUPPORTED, k, n, "tensor-core blocks need FP32, k in {5, 6}, n >= k + 7");
    const TileGeom g = make_tile_geom(n, k, targets, 7);
    if (g.nfree != n - k - 7) return err(QI_ERR_UNKNOWN, g.nfree, n - k - 7, "tile decomposition");
    if (((uintptr_t)d_tc & 15) != 0) return err(QI_ERR_UNKNOWN, -1, -1, "operand blocks must be 16-byte aligned");
    return k == 6 ? launch_tc_t<6>(s, g, d_tc) : launch_tc_t<5>(s, g, d_tc);
}

}  // namespace qi
