// qi_fused_tc.cu — fused k-qubit blocks (k = 5, 6) on the 5th-generation
// tensor cores: tcgen05.mma kind::tf32, 3xTF32 split products, FP32
// accumulation in tensor memory.
//
// For a tile of 128 columns (the 7 lowest non-target qubits, plus the tile's
// fixed high bits) the block computes OUT[n][m] = sum_r U[n][r] X[r][m] with
// R = 2^k rows.  As a real GEMM with M = 128 (tile columns), N = 2R and the
// K dimension split into a real half and an imaginary half of R each:
//   [D_re | D_im][m] += Re X[.][m] . [ Re U ; Im U ]^T     (real half)
//   [D_re | D_im][m] += Im X[.][m] . [-Im U ; Re U ]^T     (imaginary half)
// The B operands are the R x R blocks -Im U, Re U, Im U stored one after the
// other along N (K-major, shared memory), so [Re U ; Im U] starts at block 1
// and [-Im U ; Re U] at block 0.  Pair mode with k = 6 (below), short of shared memory,
// keeps only Re U, Im U and splits the imaginary half into two N = R products,
//   D_re -= Im X . Im U^T (negate-B)   and   D_im += Im X . Re U^T.
// Every operand is split as x = hi + lo with
// hi = tf32(x) (round to nearest) and lo = tf32(x - hi); the products
// A_hi B_hi + A_hi B_lo + A_lo B_hi are accumulated in FP32, which keeps
// about 22 significant bits (the dropped A_lo B_lo term is ~2^-22 relative).
//
// One persistent CTA per SM, warp-specialised, synchronised by mbarriers:
//   producer (1 thread): cp.async.bulk copies of each tile (2^nhigh runs of
//     2^L contiguous amplitudes) into one of NBUF shared buffers, in address
//     order; completion by transaction count on raw_full[b]
//   converters (8 warps; warp w owns TMEM lanes 32*(w%4).. = tile columns and
//     rows slice w/4): once A stage 0 is free, read the tile in 16-row chunks,
//     splitting the real parts into A_hi/A_lo of stage 0 (tcgen05.st) and
//     keeping the imaginary parts in registers; release the buffer
//     (raw_empty[b]); split the imaginary parts into stage 1 once it is free;
//     each stage is signalled on a_full[h]
//   MMA issuer (1 thread): per half 3 products x R/8 MMAs (M128 x N2R x K8;
//     pair mode's imaginary half: two M128 x NR x K8 per step) into
//     accumulator buffer it%2; tcgen05.commit frees the A stage
//     (a_empty[h]) and publishes the accumulator (d_full[d])
//   epilogue (4 warps): tcgen05.ld the accumulator, release it (d_empty[d]),
//     store the amplitudes straight to global memory (rows r, r+1 as one
//     16-byte store when qubit 0 is a target; adjacent lanes are adjacent
//     amplitudes when it is a column)
// Every wait is bounded; a timeout sets the state's error flag (2) and a
// shared abort flag that every other wait polls, so all roles leave their
// loops; the MMA thread then waits for its own products and the producer for
// its copies before the tensor memory is freed.
// Tensor-memory columns: A stage h at h*2R (A_hi [0,R), A_lo [R,2R)),
// accumulator d at 4R + d*2R (D_re [0,R), D_im [R,2R)): 8R columns in all.
#include "qi_internal.hpp"
#include "qi_device.cuh"
#include "qi_async.cuh"
#include "qi_tile.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>

namespace qi {

constexpr int kConvWarps = 8, kEpiWarps = 4;
constexpr int kProducerWarp = kConvWarps + kEpiWarps, kMmaWarp = kProducerWarp + 1;
constexpr int kTcThreads = (kMmaWarp + 1) * 32;   // 448

// ---------------------------------------------------------- PTX wrappers --
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
// negate B at bit 14, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tf32_idesc(uint32_t M, uint32_t N, bool negate_b = false) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((negate_b ? 1u : 0u) << 14) | ((N >> 3) << 17) | ((M >> 4) << 24);
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

// Warp-uniform form: every lane waits, the warp proceeds only if all saw the phase.
__device__ __forceinline__ bool warp_wait_or_abort(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                                   int *err_flag) {
    const bool ok = wait_or_abort(bar, parity, abort_flag, err_flag);
    return __all_sync(0xffffffffu, ok);
}

// Phase table of a tensor-core block that carries a phase polynomial (32-bit words, 2^-32 turns):
// [0, 64) the terms among each row's bits; [kPhaseLane, +128 x 8) per column index m: the terms
// among its column bits, then its cross terms with each row bit j; [kPhaseTile, +16 per tile):
// c0 + the terms among the tile's bits, its cross terms with column bit b (1 + b) and with row
// bit j (8 + j).
constexpr int kPhaseLane = 64, kPhaseTile = 64 + 128 * 8;

// ------------------------------------------------------------------ kernel
template <int K, bool PAIR = false>
struct TcCfg {
    static constexpr int R = 1 << K;                   // rows (target patterns)
    static constexpr int BLK = R * R;                  // floats per operand block
    static constexpr uint32_t LBO = 128;               // next core matrix along K
    static constexpr uint32_t SBO = (R / 4) * 128;     // next 8-row group along N
    // shared buffers: whole tiles, or (pair mode) a ring of units of 16 rows x 2 KB runs
    static constexpr int NBUF = PAIR ? (K == 6 ? 10 : 12) : (K == 6 ? 2 : 6);
    static constexpr uint32_t STAGE = 2 * R;           // TMEM columns of one A stage or one accumulator
    static constexpr uint32_t COL_A = 0, COL_D = 2 * STAGE;
    static constexpr uint32_t TMEM_COLS = 4 * STAGE;   // 512 for k = 6, 256 for k = 5
    static constexpr int CONV_ROWS = R / 2;            // rows per converter thread (2 row slices)
    static constexpr int CHUNK = PAIR ? 8 : 16;        // rows converted per step (register footprint)
    static constexpr uint32_t TILE_BYTES = (uint32_t)R * 128 * sizeof(float2);
    static constexpr int UNIT_ROWS = 8;                // pair mode: rows per ring unit (one chunk)
    static constexpr int UNITS_PER_PAIR = 2 * CONV_ROWS / UNIT_ROWS;   // pair mode: 8
    static constexpr uint32_t BUF_BYTES = PAIR ? (uint32_t)UNIT_ROWS * 2 * 128 * sizeof(float2) : TILE_BYTES;
    // operand blocks in shared memory: -Im U, Re U, Im U (hi, then lo); pair mode with k = 6,
    // short of shared memory, Re U, Im U (the imaginary half as two N = R products)
    static constexpr bool SPLIT_IM = PAIR && K == 6;
    static constexpr int NBLK = SPLIT_IM ? 4 : 6;
    static constexpr size_t OFF_TILES = (size_t)NBLK * BLK * sizeof(float);
    static constexpr size_t OFF_ROWX = OFF_TILES + (size_t)NBUF * BUF_BYTES;
    static constexpr size_t OFF_GROW = OFF_ROWX + 64 * sizeof(uint32_t);
    static constexpr size_t OFF_BAR = OFF_GROW + 64 * sizeof(uint64_t);
    static constexpr int NBARS = 2 * NBUF + 9;
    static constexpr size_t OFF_MISC = OFF_BAR + NBARS * sizeof(uint64_t);
    static constexpr size_t OFF_FR = OFF_MISC + 16;    // phase polynomial: terms among each row's bits
    static constexpr size_t SMEM = OFF_FR + 64 * sizeof(uint32_t);
};

// Tile-local position of column m: its bits deposited, in order, on the bits
// below L that are not targets.
__device__ __forceinline__ uint32_t tile_colx(const TileGeom &g, uint32_t m) {
    uint32_t x = 0;
    int j = 0;
    for (int q = 0; q < g.L; ++q) {
        bool tgt = false;
        for (int u = 0; u < g.nlow_t; ++u) tgt |= (g.low_t[u] == q);
        if (!tgt) {
            x |= ((m >> j) & 1u) << q;
            ++j;
        }
    }
    return x;
}

// x = hi + lo split of N rows of one column into A_hi / A_lo tensor-memory columns.
// x is left holding x - hi.
template <int N>
__device__ __forceinline__ void split_store(uint32_t taddr_hi, uint32_t taddr_lo, float (&x)[N]) {
    uint32_t v[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        v[i] = tf32_rna(x[i]);
        x[i] -= __uint_as_float(v[i]);
    }
    tmem_st<N>(taddr_hi, v);
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = tf32_rna(x[i]);
    tmem_st<N>(taddr_lo, v);
}

// out[p] = a[(p - s) mod 8]: undoes a per-lane rotation of 8 values (s in 0..7),
// three select stages with compile-time indices.
__device__ __forceinline__ void unrotate8(float (&a)[8], int s) {
#pragma unroll
    for (int st = 0; st < 3; ++st) {
        const int k = 1 << st;
        const bool on = (s >> st) & 1;
        float t[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) t[p] = on ? a[(p - k) & 7] : a[p];
#pragma unroll
        for (int p = 0; p < 8; ++p) a[p] = t[p];
    }
}

// 32-byte streaming store of four consecutive amplitudes (address 32-byte aligned).
__device__ __forceinline__ void st_cs_v8(float2 *p, float a0, float a1, float a2, float a3, float a4, float a5,
                                         float a6, float a7) {
    asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n" ::"l"(p), "f"(a0), "f"(a1),
                 "f"(a2), "f"(a3), "f"(a4), "f"(a5), "f"(a6), "f"(a7)
                 : "memory");
}

// PAIR: a CTA takes tiles in pairs (2p, 2p+1), which differ in qubit L = 7, so the row
// runs of the two tiles are adjacent in memory; one bulk copy of 2 x 2^L amplitudes per
// row run loads both.  The pair's rows go through a ring of NBUF units of 8 rows
// (unit u = 2c + s: chunk c of converter slice s); a unit is released after the pair's
// second tile has read it, so the next pair's first units load while the second tile
// is converted.  Used when the runs are 1 KB (all targets above qubit 7), where the
// copy granularity bounds the load rate.
// ROT: qubits 0-3 are all targets, so the tile's columns are 128 bytes or more apart and the
// 8 lanes of a quarter warp would read the same banks for one row pair; each lane then reads the
// chunk's row pairs starting at its own (lane mod 8), undone in registers.
// PHASE: a diagonal phase polynomial exp(2 pi i f(x)) that follows the block in the plan is
// applied by the epilogue before the store (its phase table at `poly`, tc_phase_table).
template <int K, bool PAIR, bool ROT, bool PHASE>
__global__ void __launch_bounds__(kTcThreads, 1) k_fused_tc(float2 *a, const float *blocks, TileGeom g, int *err_flag,
                                                            const uint32_t *__restrict__ poly) {
    using C = TcCfg<K, PAIR>;
    constexpr int R = C::R, NB = C::NBUF;
    static_assert(!PAIR || ((K == 5 || K == 6) && C::UNIT_ROWS == C::CHUNK), "pair mode: K = 5 or 6, one ring unit per chunk");
    static_assert(!(PAIR && ROT), "pair-mode tiles have qubit 0 as a column");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float *sB = reinterpret_cast<float *>(smem_raw);   // operand blocks (C::NBLK)
    unsigned char *tiles = smem_raw + C::OFF_TILES;
    uint32_t *rowx = reinterpret_cast<uint32_t *>(smem_raw + C::OFF_ROWX);
    uint64_t *grow = reinterpret_cast<uint64_t *>(smem_raw + C::OFF_GROW);
    uint64_t *raw_full = reinterpret_cast<uint64_t *>(smem_raw + C::OFF_BAR);
    uint64_t *raw_empty = raw_full + NB, *a_full = raw_empty + NB, *a_empty = a_full + 2;
    uint64_t *d_full = a_empty + 2, *d_empty = d_full + 2, *mma_done = d_empty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem_raw + C::OFF_MISC);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // operand blocks -> shared memory (16-byte vectors), visible to the async proxy;
    // pair mode with k = 6 takes blocks 1, 2, 4, 5 (Re U, Im U; hi then lo) of the six
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(blocks);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        constexpr int per_blk = C::BLK * (int)sizeof(float) / 16;
        for (int i = tid; i < C::NBLK * per_blk; i += kTcThreads) {
            const int blk = i / per_blk;
            const int from = C::NBLK == 4 ? (blk < 2 ? blk + 1 : blk + 2) : blk;
            dst[i] = src[from * per_blk + i % per_blk];
        }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    // row r (bit j <-> target j) -> tile-local position and global offset
    if (tid < R) {
        uint32_t x = 0;
        uint64_t go = 0;
        for (int j = 0; j < g.nlow_t; ++j) {
            const uint32_t bit = ((uint32_t)tid >> j) & 1u;
            x |= bit << g.low_t[j];
            go |= (uint64_t)bit << g.low_t[j];
        }
        for (int j = 0; j < g.nhigh; ++j) {
            const uint32_t bit = ((uint32_t)tid >> (g.nlow_t + j)) & 1u;
            // pair mode: the top row bits select the ring unit (slice, chunk); the others index
            // its runs of 2 x 2^L
            if (!PAIR) x |= bit << (g.L + j);
            else if ((1 << j) < C::UNIT_ROWS) x |= bit << (g.L + 1 + j);
            go |= (uint64_t)bit << g.high_t[j];
        }
        rowx[tid] = x;
        grow[tid] = go;
    }
    if (tid == 0) {
        for (int i = 0; i < NB; ++i) {
            mbar_init(raw_full + i, 1);
            mbar_init(raw_empty + i, PAIR ? kConvWarps / 2 : kConvWarps);   // pair mode: one slice per unit
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(a_full + i, kConvWarps);
            mbar_init(a_empty + i, 1);
            mbar_init(d_full + i, 1);
            mbar_init(d_empty + i, kEpiWarps);
        }
        mbar_init(mma_done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tmem_slot, C::TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // tile counts stay below 2^32 (2^(n-13) tiles for n <= 44)
    const uint32_t ntiles = (uint32_t)g.ntiles;
    // iteration -> tile; pair mode takes 2p and 2p + 1 in consecutive iterations
    auto tile_of = [&](int it) -> uint32_t {
        return PAIR ? 2u * (blockIdx.x + (uint32_t)(it >> 1) * gridDim.x) + (uint32_t)(it & 1)
                    : blockIdx.x + (uint32_t)it * gridDim.x;
    };
    const bool pair_rows = !g.q0_is_col;   // qubit 0 is target 0: rows r, r+1 are adjacent amplitudes
    // qubits 0 and 1 both targets: rows r..r+3 are four adjacent amplitudes (one 32-byte store)
    const bool quad_rows = pair_rows && g.nlow_t >= 2 && g.low_t[1] == 1;

    if (warp < kConvWarps) {
        // ------------------------------------------------ converters
        const int quarter = warp & 3, slice = warp >> 2;
        const uint32_t cx = tile_colx(g, (uint32_t)(quarter * 32 + lane));
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        const int r0 = slice * C::CONV_ROWS;
        for (int it = 0; tile_of(it) < ntiles; ++it) {
            const int b = it % NB;   // whole-tile buffer (pair mode: units, below)
            if (!PAIR && !warp_wait_or_abort(raw_full + b, (uint32_t)(it / NB) & 1u, abort_flag, err_flag)) break;
            // real half -> A stage 0, once the products of the previous tile have read it;
            // the imaginary parts stay in registers for stage 1
            if (it > 0 && !warp_wait_or_abort(a_empty + 0, (uint32_t)(it - 1) & 1u, abort_flag, err_flag)) break;
            tc_fence_after();
            bool ok = true;
            float im[C::CONV_ROWS];
#pragma unroll
            for (int c0 = 0; c0 < C::CONV_ROWS; c0 += C::CHUNK) {
                const float2 *S;
                uint32_t unit = 0;
                if constexpr (PAIR) {
                    const uint32_t k = (uint32_t)C::UNITS_PER_PAIR * (uint32_t)(it >> 1) +
                                       2u * (uint32_t)(c0 / C::CHUNK) + (uint32_t)slice;
                    unit = k % NB;
                    if (!(it & 1) && !warp_wait_or_abort(raw_full + unit, (k / NB) & 1u, abort_flag, err_flag)) {
                        ok = false;
                        break;
                    }
                    S = reinterpret_cast<const float2 *>(tiles + (size_t)unit * C::BUF_BYTES) + ((uint32_t)(it & 1) << g.L);
                } else {
                    S = reinterpret_cast<const float2 *>(tiles + (size_t)b * C::BUF_BYTES);
                }
                float re[C::CHUNK];
                if constexpr (ROT) {
                    static_assert(C::CHUNK == 16, "8 row pairs per chunk");
                    // lane reads row pair (j + lane) mod 8 at step j: 8 lanes, 8 bank groups
                    const int sft = lane & 7;
                    float r0v[8], i0v[8], r1v[8], i1v[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int pr = (j + sft) & 7;
                        const float4 v = *reinterpret_cast<const float4 *>(S + (rowx[r0 + c0 + 2 * pr] | cx));
                        r0v[j] = v.x;
                        i0v[j] = v.y;
                        r1v[j] = v.z;
                        i1v[j] = v.w;
                    }
                    unrotate8(r0v, sft);
                    unrotate8(i0v, sft);
                    unrotate8(r1v, sft);
                    unrotate8(i1v, sft);
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        re[2 * j] = r0v[j];
                        im[c0 + 2 * j] = i0v[j];
                        re[2 * j + 1] = r1v[j];
                        im[c0 + 2 * j + 1] = i1v[j];
                    }
                } else if (pair_rows) {
#pragma unroll
                    for (int i = 0; i < C::CHUNK; i += 2) {
                        const float4 v = *reinterpret_cast<const float4 *>(S + (rowx[r0 + c0 + i] | cx));
                        re[i] = v.x;
                        im[c0 + i] = v.y;
                        re[i + 1] = v.z;
                        im[c0 + i + 1] = v.w;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < C::CHUNK; ++i) {
                        const float2 v = S[rowx[r0 + c0 + i] | cx];
                        re[i] = v.x;
                        im[c0 + i] = v.y;
                    }
                }
                split_store<C::CHUNK>(tmem + lane_base + C::COL_A + r0 + c0, tmem + lane_base + C::COL_A + R + r0 + c0,
                                      re);
                if constexpr (PAIR) {   // the pair's second tile was the unit's last reader
                    __syncwarp();
                    if (lane == 0 && (it & 1)) mbar_arrive(raw_empty + unit);
                }
            }
            if (!ok) break;
            if (!PAIR) {
                __syncwarp();
                if (lane == 0) mbar_arrive(raw_empty + b);   // the buffer may take the next tile
            }
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(a_full + 0);
            // imaginary half -> A stage 1
            if (it > 0 && !warp_wait_or_abort(a_empty + 1, (uint32_t)(it - 1) & 1u, abort_flag, err_flag)) break;
            tc_fence_after();
#pragma unroll
            for (int c0 = 0; c0 < C::CONV_ROWS; c0 += C::CHUNK)
                split_store<C::CHUNK>(tmem + lane_base + C::COL_A + C::STAGE + r0 + c0,
                                      tmem + lane_base + C::COL_A + C::STAGE + R + r0 + c0,
                                      *reinterpret_cast<float(*)[C::CHUNK]>(im + c0));
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(a_full + 1);
        }
    } else if (warp < kConvWarps + kEpiWarps) {
        // ------------------------------------------------ epilogue
        const int quarter = warp & 3;
        const uint32_t m = (uint32_t)(quarter * 32 + lane);
        const uint64_t cx = tile_colx(g, m);
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        // Phase polynomial f(i) = c0 + sum_q a_q i_q + sum_{q<r} b_qr i_q i_r (2^-32 turns, wrapping)
        // over i = tile bits | column bits | row bits, from the host table (tc_phase_table): the
        // terms among a row's bits (FR), among this lane's column bits (p_lane) and the column-row
        // cross terms (wz[j] per row bit j) once; the tile terms once per tile.
        uint32_t p_lane = 0, wz[K], *FR = reinterpret_cast<uint32_t *>(smem_raw + C::OFF_FR);
        if constexpr (PHASE) {
#pragma unroll
            for (int j = 0; j < K; ++j) wz[j] = __ldg(poly + kPhaseLane + m * 8 + 1 + j);
            p_lane = __ldg(poly + kPhaseLane + m * 8);
            const int e = (warp - kConvWarps) * 32 + lane;
            if (e < R) FR[e] = __ldg(poly + e);
            asm volatile("bar.sync 1, %0;\n" ::"r"(kEpiWarps * 32) : "memory");   // the epilogue warps only
        }
        for (int it = 0; tile_of(it) < ntiles; ++it) {
            const uint32_t t = tile_of(it);
            const int d = it & 1;
            uint32_t pbase = 0, z[K];
            if constexpr (PHASE) {   // c0 + the tile's own terms, its cross terms with columns / rows
                const uint32_t *tt = poly + kPhaseTile + (size_t)t * 16;
                pbase = p_lane + __ldg(tt);
#pragma unroll
                for (int b = 0; b < 7; ++b)
                    if ((m >> b) & 1u) pbase += __ldg(tt + 1 + b);
#pragma unroll
                for (int j = 0; j < K; ++j) z[j] = wz[j] + __ldg(tt + 8 + j);
            }
            if (!warp_wait_or_abort(d_full + d, (uint32_t)(it >> 1) & 1u, abort_flag, err_flag)) break;
            tc_fence_after();
            float2 *out = a + (tile_base(g, t) | cx);   // column base; rows add disjoint bits
            const uint32_t dcol = tmem + lane_base + C::COL_D + d * C::STAGE;
            auto chunk = [&](int c) {   // rows 16c .. 16c + 15
                uint32_t vr[16], vi[16];
                tmem_ld<16>(dcol + 16 * c, vr);
                tmem_ld<16>(dcol + R + 16 * c, vi);
                tmem_wait_ld();
                if (c == R / 16 - 1) {   // accumulator read out: the next tile but one may use it
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(d_empty + d);
                }
                if constexpr (PHASE) {
                    uint32_t fc = pbase;   // the chunk's row bits 4.. (bits of c)
#pragma unroll
                    for (int j = 4; j < K; ++j)
                        if ((c >> (j - 4)) & 1) fc += z[j];
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        uint32_t f = fc + FR[16 * c + i];
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            if ((i >> j) & 1) f += z[j];
                        // the angle as a signed fraction of a turn, in [-pi, pi): the SFU's sin / cos
                        // (absolute error about 2^-21, the order of the FP32 state's own rounding)
                        float sn, cs;
                        __sincosf((float)(int32_t)f * 1.46291807926715968e-9f, &sn, &cs);   // 2 pi / 2^32
                        const float2 ph = make_float2(cs, sn);
                        const float xr = __uint_as_float(vr[i]), xi = __uint_as_float(vi[i]);
                        vr[i] = __float_as_uint(ph.x * xr - ph.y * xi);
                        vi[i] = __float_as_uint(ph.x * xi + ph.y * xr);
                    }
                }
                if (quad_rows) {
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        st_cs_v8(out + grow[16 * c + i], __uint_as_float(vr[i]), __uint_as_float(vi[i]),
                                 __uint_as_float(vr[i + 1]), __uint_as_float(vi[i + 1]), __uint_as_float(vr[i + 2]),
                                 __uint_as_float(vi[i + 2]), __uint_as_float(vr[i + 3]), __uint_as_float(vi[i + 3]));
                } else if (pair_rows) {
#pragma unroll
                    for (int i = 0; i < 16; i += 2)
                        __stcs(reinterpret_cast<float4 *>(out + grow[16 * c + i]),
                               make_float4(__uint_as_float(vr[i]), __uint_as_float(vi[i]), __uint_as_float(vr[i + 1]),
                                           __uint_as_float(vi[i + 1])));
                } else {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        __stcs(out + grow[16 * c + i], make_float2(__uint_as_float(vr[i]), __uint_as_float(vi[i])));
                }
            };
            // Not unrolled: the kernel's four roles run different code, and with the epilogue unrolled
            // over its chunks the warps waited on instruction fetch ("no instruction" stalls 3.2-4.7
            // per issue). Rolled, 30-qubit launches took 3.09 against 3.44 ms (pairs), 2.67 against
            // 2.80 ms (single tiles) and, carrying a phase polynomial, 2.83 against 3.81 ms.
#pragma unroll 1
            for (int c = 0; c < R / 16; ++c) chunk(c);
        }
    } else if (warp == kProducerWarp) {
        // ------------------------------------------------ producer (one thread)
        if (lane == 0) {
            const uint32_t run_bytes = (uint32_t)sizeof(float2) << g.L;
            if (!PAIR) {
                const int nruns = 1 << g.nhigh;
                int issued = 0;
                for (int it = 0; tile_of(it) < ntiles; ++it) {
                    const int b = it % NB;
                    if (it >= NB && !wait_or_abort(raw_empty + b, (uint32_t)(it / NB - 1) & 1u, abort_flag, err_flag))
                        break;
                    mbar_arrive_expect_tx(raw_full + b, C::TILE_BYTES);
                    const uint64_t base = tile_base(g, tile_of(it));
                    unsigned char *dst = tiles + (size_t)b * C::TILE_BYTES;
                    for (int h = 0; h < nruns; ++h)
                        bulk_load(dst + (size_t)h * run_bytes, a + (base | grow[h << g.nlow_t]), run_bytes, raw_full + b);
                    issued = it + 1;
                }
                // copies still in flight (only after an abort) land before the CTA exits
                for (int j = issued > NB ? issued - NB : 0; j < issued; ++j)
                    if (!mbar_wait_bounded(raw_full + (j % NB), (uint32_t)(j / NB) & 1u)) atomicExch(err_flag, 2);
            } else {
                // ring unit k (pair k / 4, u = k % 4 = 2c + s) <- rows 32 s + 16 c .. + 15 of the
                // pair: runs of 2 x 2^L amplitudes (both tiles), in the order the converters use them
                int issued = 0;
                bool ok = true;
                for (uint32_t lp = 0; ok && tile_of(2 * (int)lp) < ntiles; ++lp) {
                    const uint64_t base = tile_base(g, tile_of(2 * (int)lp));
                    for (uint32_t u = 0; u < (uint32_t)C::UNITS_PER_PAIR; ++u) {
                        const uint32_t k = (uint32_t)C::UNITS_PER_PAIR * lp + u, unit = k % NB;
                        if (k >= (uint32_t)NB &&
                            !wait_or_abort(raw_empty + unit, (k / NB - 1) & 1u, abort_flag, err_flag)) {
                            ok = false;
                            break;
                        }
                        mbar_arrive_expect_tx(raw_full + unit, C::BUF_BYTES);
                        unsigned char *dst = tiles + (size_t)unit * C::BUF_BYTES;
                        const int row0 = C::CONV_ROWS * (int)(u & 1u) + C::UNIT_ROWS * (int)(u >> 1);
                        for (int i = 0; i < C::UNIT_ROWS; ++i)
                            bulk_load(dst + (size_t)i * 2 * run_bytes, a + (base | grow[row0 + i]), 2 * run_bytes,
                                      raw_full + unit);
                        issued = (int)k + 1;
                    }
                }
                // copies still in flight (only after an abort) land before the CTA exits
                for (int j = issued > NB ? issued - NB : 0; j < issued; ++j)
                    if (!mbar_wait_bounded(raw_full + (j % NB), (uint32_t)(j / NB) & 1u)) atomicExch(err_flag, 2);
            }
        }
        __syncwarp();
    } else {
        // ------------------------------------------------ MMA issuer (one thread)
        if (lane == 0) {
            // Descriptor of block 0 at K offset 0; every MMA adds a constant byte offset
            // (>> 4 into the start-address field, which cannot carry: blocks stay below 256 KB).
            const uint64_t desc0 = smem_desc(smem_u32(sB), C::LBO, C::SBO);
            constexpr uint32_t idesc = tf32_idesc(128, 2 * R), idesc_r = tf32_idesc(128, R),
                               idesc_rneg = tf32_idesc(128, R, true);
            bool ok = true;
            for (int it = 0; ok && tile_of(it) < ntiles; ++it) {
                const int d = it & 1;
                if (it >= 2 && !wait_or_abort(d_empty + d, (uint32_t)((it >> 1) - 1) & 1u, abort_flag, err_flag))
                    break;
                tc_fence_after();
                const uint32_t dcol = tmem + C::COL_D + d * C::STAGE;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (!wait_or_abort(a_full + h, (uint32_t)it & 1u, abort_flag, err_flag)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t acol = tmem + C::COL_A + h * C::STAGE;
#pragma unroll
                    for (int p = 0; p < 3; ++p) {   // (A_hi, B_hi), (A_hi, B_lo), (A_lo, B_hi)
#pragma unroll
                        for (int j = 0; j < R / 8; ++j) {
                            const uint32_t kstep = (uint32_t)(2 * j) * C::LBO;
                            const uint32_t a_col = acol + (p == 2 ? R : 0) + 8 * j;
                            if constexpr (!C::SPLIT_IM) {   // window [Re U ; Im U] (block 1) or [-Im U ; Re U] (block 0)
                                const int blk = (p == 1 ? 3 : 0) + (h == 0 ? 1 : 0);
                                const uint32_t boff = (uint32_t)(blk * C::BLK * 4) + kstep;
                                mma_tf32_ts(dcol, a_col, desc0 + (uint64_t)(boff >> 4), idesc, (h | p | j) ? 1u : 0u);
                            } else {
                                const int blk = p == 1 ? 2 : 0;   // Re U of the hi or lo pair, Im U next to it
                                const uint32_t b_re = (uint32_t)(blk * C::BLK * 4) + kstep, b_im = b_re + C::BLK * 4;
                                if (h == 0) {   // [D_re | D_im] += Re X . [Re U ; Im U]^T
                                    mma_tf32_ts(dcol, a_col, desc0 + (uint64_t)(b_re >> 4), idesc, (p | j) ? 1u : 0u);
                                } else {        // D_re -= Im X . Im U^T;  D_im += Im X . Re U^T
                                    mma_tf32_ts(dcol, a_col, desc0 + (uint64_t)(b_im >> 4), idesc_rneg, 1u);
                                    mma_tf32_ts(dcol + R, a_col, desc0 + (uint64_t)(b_re >> 4), idesc_r, 1u);
                                }
                            }
                        }
                    }
                    mma_commit(a_empty + h);
                }
                if (ok) mma_commit(d_full + d);
            }
            // every product issued here has completed before the tensor memory is freed
            mma_commit(mma_done);
            if (!mbar_wait_bounded(mma_done, 0)) atomicExch(err_flag, 2);
        }
        __syncwarp();
    }
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
            const double vals[3] = {-im, re, im};   // block order along N: -Im U, Re U, Im U
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

// Host: the phase table of a block on `targets` that carries the phase polynomial pp (layout
// at kPhaseLane / kPhaseTile).  Coefficients are rounded to 2^-32 turns one by one and summed
// with wrapping, as the standalone phase-polynomial kernel does.  Tiles are visited in Gray-code
// order, so each tile's terms follow from the previous tile's by one qubit.  False (nothing
// appended) beyond 2^20 tiles (16 words each).
bool tc_phase_table(const PhasePoly &pp, int k, const int32_t *targets, std::vector<float> &out) {
    const int n = pp.n;
    const TileGeom g = make_tile_geom(n, k, targets, 7);
    if (g.nfree > 20 || k > 6) return false;
    auto r32 = [](uint64_t v) { return (uint32_t)((v + 0x80000000ull) >> 32); };
    auto A = [&](int q) { return r32(pp.a[(size_t)q]); };
    auto B = [&](int q, int r) -> uint32_t {
        if (q == r) return 0u;
        if (q > r) std::swap(q, r);
        return r32(pp.b[(size_t)q * n + r]);
    };
    int tq[6] = {0, 0, 0, 0, 0, 0}, colq[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < k; ++j) tq[j] = j < g.nlow_t ? g.low_t[j] : g.high_t[j - g.nlow_t];
    for (int q = 0, b = 0; q < g.L && b < 7; ++q) {   // the 7 lowest non-target qubits, in order
        bool tgt = false;
        for (int u = 0; u < g.nlow_t; ++u) tgt |= g.low_t[u] == q;
        if (!tgt) colq[b++] = q;
    }
    auto host_tile_base = [&](uint64_t t) {
        uint64_t base = 0;
        for (int j = 0; j < g.nruns; ++j) base |= ((t >> g.run_src[j]) & g.run_mask[j]) << g.run_dst[j];
        return base;
    };
    int fq[64];
    for (int j = 0; j < g.nfree; ++j) fq[j] = __builtin_ctzll(host_tile_base(1ull << j));
    const size_t ntiles = (size_t)g.ntiles;
    std::vector<uint32_t> w((size_t)kPhaseTile + 16 * ntiles, 0);
    for (int r = 0; r < (1 << k); ++r) {   // terms among a row's bits
        uint32_t v = 0;
        for (int j = 0; j < k; ++j) {
            if (!((r >> j) & 1)) continue;
            v += A(tq[j]);
            for (int j2 = 0; j2 < j; ++j2)
                if ((r >> j2) & 1) v += B(tq[j], tq[j2]);
        }
        w[(size_t)r] = v;
    }
    for (int m = 0; m < 128; ++m) {   // per column index: its own terms, cross terms with each row bit
        uint32_t pl = 0;
        for (int b = 0; b < 7; ++b) {
            if (!((m >> b) & 1)) continue;
            pl += A(colq[b]);
            for (int b2 = 0; b2 < b; ++b2)
                if ((m >> b2) & 1) pl += B(colq[b], colq[b2]);
        }
        w[(size_t)kPhaseLane + (size_t)m * 8] = pl;
        for (int j = 0; j < k; ++j) {
            uint32_t v = 0;
            for (int b = 0; b < 7; ++b)
                if ((m >> b) & 1) v += B(colq[b], tq[j]);
            w[(size_t)kPhaseLane + (size_t)m * 8 + 1 + (size_t)j] = v;
        }
    }
    uint32_t pt = r32(pp.c0), U[7] = {0, 0, 0, 0, 0, 0, 0}, V[6] = {0, 0, 0, 0, 0, 0};
    uint64_t cur = 0;   // tile bits of the current tile
    auto store = [&](uint64_t t) {
        uint32_t *o = w.data() + kPhaseTile + (size_t)t * 16;
        o[0] = pt;
        for (int b = 0; b < 7; ++b) o[1 + b] = U[b];
        for (int j = 0; j < k; ++j) o[8 + j] = V[j];
    };
    store(0);
    for (uint64_t i = 1; i < (uint64_t)ntiles; ++i) {   // Gray code: tile i ^ (i >> 1) flips bit ctz(i)
        const int j = __builtin_ctzll(i), q = fq[j];
        const bool on = !((cur >> j) & 1ull);
        uint32_t delta = A(q);
        for (uint64_t rest = cur & ~(1ull << j); rest; rest &= rest - 1) delta += B(q, fq[__builtin_ctzll(rest)]);
        pt += on ? delta : (uint32_t)(0u - delta);
        for (int b = 0; b < 7; ++b) U[b] += on ? B(q, colq[b]) : (uint32_t)(0u - B(q, colq[b]));
        for (int jj = 0; jj < k; ++jj) V[jj] += on ? B(q, tq[jj]) : (uint32_t)(0u - B(q, tq[jj]));
        cur ^= 1ull << j;
        store(cur);
    }
    const size_t base = out.size();
    out.resize(base + w.size(), 0.0f);
    std::memcpy(out.data() + base, w.data(), w.size() * 4);
    return true;
}

template <int K, bool PAIR, bool ROT, bool PHASE>
static Status launch_tc_t(qi_state *s, const TileGeom &g, const void *d_tc, const void *poly) {
    using C = TcCfg<K, PAIR>;
    static_assert(C::SMEM <= 232448, "shared memory per CTA");
    // the shared-memory opt-in and the SM count are per device (state handles may live on several)
    static std::atomic<int> num_sms_of[64];
    int dev = 0;
    QI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return err(QI_ERR_UNSUPPORTED, dev, 64, "device ordinal");
    int num_sms = num_sms_of[dev].load();
    if (num_sms == 0) {
        QI_CUDA(cudaFuncSetAttribute(k_fused_tc<K, PAIR, ROT, PHASE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)C::SMEM));
        QI_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
        num_sms_of[dev].store(num_sms);
    }
    uint64_t grid = PAIR ? g.ntiles / 2 : g.ntiles;   // one persistent CTA per SM
    if (grid > (uint64_t)num_sms) grid = (uint64_t)num_sms;
    k_fused_tc<K, PAIR, ROT, PHASE><<<(unsigned)grid, kTcThreads, C::SMEM, s->stream>>>(
        (float2 *)s->amps, (const float *)d_tc, g, s->d_flag, (const uint32_t *)poly);
    count_launch();
    return check_launch("k_fused_tc");
}

Status launch_fused_tc(qi_state *s, int k, const int32_t *targets, const void *d_tc, const void *poly) {
    const int n = s->n;
    if (s->prec != QI_F32 || (k != 5 && k != 6) || n < k + 7)
        return err(QI_ERR_UNSUPPORTED, k, n, "tensor-core blocks need FP32, k in {5, 6}, n >= k + 7");
    const TileGeom g = make_tile_geom(n, k, targets, 7);
    if (g.nfree != n - k - 7) return err(QI_ERR_UNKNOWN, g.nfree, n - k - 7, "tile decomposition");
    if (((uintptr_t)d_tc & 15) != 0) return err(QI_ERR_UNKNOWN, -1, -1, "operand blocks must be 16-byte aligned");
    // Tile pairs when a tile's rows are 1 KB runs (all targets above qubit 7): tiles 2p, 2p + 1
    // differ in qubit L = 7, so each pair of runs is one 2 KB copy.  (Measured at 30 qubits: 3.28 ms
    // per launch against 4.4 ms for single tiles of 1 KB runs; a 4-unit ring with the N = 2R
    // imaginary half took 3.83 ms, so the ring depth matters more than the extra MMAs.)
    const bool pair = g.nlow_t == 0 && g.nhigh == k && g.nfree >= 1 && g.L == 7 && g.L < n;
    // qubits 0-3 all targets: lane-rotated row reads (k_fused_tc's ROT)
    bool rot = true;
    for (int q = 0; q < 4; ++q) rot = rot && std::find(targets, targets + k, q) != targets + k;
    if (poly && ((uintptr_t)poly & 15) != 0) return err(QI_ERR_UNKNOWN, -1, -1, "phase block must be 16-byte aligned");
#define QI_TC(KK, PA, RO)                                                                    \
    (poly ? launch_tc_t<KK, PA, RO, true>(s, g, d_tc, poly) : launch_tc_t<KK, PA, RO, false>(s, g, d_tc, nullptr))
    if (k == 5) return pair ? QI_TC(5, true, false) : rot ? QI_TC(5, false, true) : QI_TC(5, false, false);
    if (pair) return QI_TC(6, true, false);
    return rot ? QI_TC(6, false, true) : QI_TC(6, false, false);
#undef QI_TC
}

// ------------------------------------------------------------ rate probe --
// Dense kind::tf32 rate of this GPU, the tensor roof the fused blocks are reported against:
// one CTA per SM (the dynamic shared-memory request keeps it alone on its SM), one thread
// issues `iters` tcgen05.mma M128 x N256 x K8 from the same tensor-memory A operand and
// shared-memory B block into one accumulator (the pattern of k_fused_tc's product chains),
// commits and waits.  Operands are zeros; no global memory is touched.
constexpr int kProbeN = 256, kProbeThreads = 128;
__global__ void __launch_bounds__(kProbeThreads, 1) k_tf32_rate_probe(int iters, int *err_flag) {
    __shared__ __align__(1024) float sB[kProbeN * 8];   // N x K = 256 x 8 tf32 (8 KB)
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tslot;
    const int warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kProbeN * 8; i += blockDim.x) sB[i] = 0.0f;
    if (threadIdx.x == 0) {
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&tslot, 512);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");   // sB visible to the tensor core
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    {   // A: columns 0..7 of every lane, zeros (warp w writes lanes 32w .. 32w + 31)
        uint32_t z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        tmem_st<8>(tbase + ((uint32_t)(warp * 32) << 16), z);
        tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        // K-major, no swizzle: core matrices (8 rows x 16 B) at 128 B along K, 256 B along N
        const uint64_t desc = smem_desc(smem_u32(sB), 128, 256);
        constexpr uint32_t idesc = tf32_idesc(128, kProbeN);
        const uint32_t d_col = tbase + 256;
        for (int i = 0; i < iters; ++i) mma_tf32_ts(d_col, tbase, desc, idesc, i > 0 ? 1u : 0u);
        mma_commit(&done);
        if (!mbar_wait_bounded(&done, 0)) {
            atomicExch(err_flag, 2);
            mbar_wait_bounded(&done, 0);   // once more before the tensor memory is freed
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tbase, 512);
}

}  // namespace qi

using namespace qi;

extern "C" qi_status qi_tf32_rate_probe(int32_t iters, int32_t reps, double *tflops_out, double *ms_out) {
    if (!tflops_out) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (iters < 1 || iters > (1 << 20) || reps < 1 || reps > 1000)
        return publish(err(QI_ERR_INVALID_INPUT_VALUE, iters, reps, "1 <= iters <= 2^20, 1 <= reps <= 1000"));
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // 120 KB of dynamic shared memory: one probe CTA per SM, so every CTA gets its 512 columns
    const int dyn = 120 * 1024;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tf32_rate_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    int *d_flag = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&d_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d_flag, 0, sizeof(int));
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    float best = 0.0f;
    if (e == cudaSuccess) {
        k_tf32_rate_probe<<<(unsigned)sms, kProbeThreads, dyn>>>(iters, d_flag);   // warm-up
        count_launch();
        for (int r = 0; r < reps && e == cudaSuccess; ++r) {
            e = cudaEventRecord(ev0);
            k_tf32_rate_probe<<<(unsigned)sms, kProbeThreads, dyn>>>(iters, d_flag);
            count_launch();
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(ev1);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
            if (e == cudaSuccess && (best == 0.0f || ms < best)) best = ms;
        }
    }
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (d_flag) cudaFree(d_flag);
    if (e != cudaSuccess) return publish(cuda_status(e, "qi_tf32_rate_probe"));
    if (flag) return publish(err(QI_ERR_TIMEOUT, -1, -1, "tf32 rate probe: mbarrier wait timed out"));
    const double flop = 2.0 * 128.0 * kProbeN * 8.0 * (double)iters * (double)sms;
    *tflops_out = flop / (best * 1e-3) / 1e12;
    if (ms_out) *ms_out = best;
    return publish(ok_status());
}

