// qi_tile.cuh — tiles of a fused k-qubit block: geometry, cp.async loads into
// a swizzled [row][column] shared-memory layout, and coalesced stores.
//
// A fused block acts on sorted targets t_0 < ... < t_{k-1}.  For an amplitude
// index, its "row" r is the pattern of the target bits (local bit j <-> t_j)
// and its "column" c the pattern of the other bits.  A tile holds all 2^k
// rows of 2^nb columns, the columns being the nb lowest non-target qubits.
// Every qubit below L (one past the highest column qubit, extended over
// targets directly above it) belongs to the tile, so a tile is 2^nhigh
// contiguous runs of 2^L amplitudes of global memory; qubit 0 is always in
// the tile.
//
// Shared memory holds the tile as S[r][c ^ swz(r)] (row length 2^nb, no
// padding).  swz(r) = ((r ^ (r >> 1)) * step) mod 2^nb with step = 2 when
// qubit 0 is a column (pairs of adjacent amplitudes then stay adjacent, so
// FP32 pairs move as 16-byte chunks) and step = 1 otherwise.  Reading or
// writing one row across 32 consecutive columns, and the address-order copy
// of 32 consecutive chunks, are both free of bank conflicts up to the
// 2-wavefront minimum of 8-byte accesses.
//
// Address-order work distribution: thread `tid` of `nthr` handles the chunks
// x = x0 + i * (2 * nthr) with x0 = 2 * tid; the bits of x above bit
// log2(2*nthr) come only from i, so r, c and the global offset split into a
// per-thread part and a per-iteration part (tables in shared memory).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>

namespace qi {

struct TileGeom {
    uint64_t ntiles;
    int32_t k, nb, L;
    int32_t nlow_t, nhigh, nfree;
    int32_t step;            // swizzle step
    int32_t q0_is_col;       // 1 if qubit 0 is a column bit
    int32_t nruns;           // runs of consecutive free qubits (between high targets)
    int8_t low_t[8];         // tile-local positions of targets below L (== qubit indices)
    int8_t high_t[8];        // qubit indices of targets >= L
    int8_t free_pos[64];     // qubits outside the tile (ascending)
    // tile index t -> base address: sum over runs j of ((t >> src[j]) & mask[j]) << dst[j]
    uint8_t run_src[8], run_dst[8];
    uint64_t run_mask[8];
};

// Host: geometry for targets[k] (sorted) with nb column bits.
inline TileGeom make_tile_geom(int n, int k, const int32_t *targets, int nb) {
    TileGeom g;
    std::memset(&g, 0, sizeof(g));
    g.k = k;
    uint64_t tmask = 0;
    for (int j = 0; j < k; ++j) tmask |= 1ull << targets[j];
    g.nb = nb;
    int got = 0, q = 0;
    while (got < nb) {
        if (!((tmask >> q) & 1ull)) ++got;
        ++q;
    }
    while (q < n && ((tmask >> q) & 1ull)) ++q;
    g.L = q;
    for (int j = 0; j < k; ++j) {
        if (targets[j] < g.L) g.low_t[g.nlow_t++] = (int8_t)targets[j];
        else g.high_t[g.nhigh++] = (int8_t)targets[j];
    }
    for (int qq = 0; qq < n; ++qq)
        if (qq >= g.L && !((tmask >> qq) & 1ull)) g.free_pos[g.nfree++] = (int8_t)qq;
    g.ntiles = 1ull << g.nfree;
    // free qubits grouped into runs of consecutive qubit indices (at most nhigh + 1 runs)
    g.nruns = 0;
    for (int j = 0; j < g.nfree;) {
        int e = j;
        while (e + 1 < g.nfree && g.free_pos[e + 1] == g.free_pos[e] + 1) ++e;
        g.run_src[g.nruns] = (uint8_t)j;
        g.run_dst[g.nruns] = (uint8_t)g.free_pos[j];
        g.run_mask[g.nruns] = (e - j + 1) >= 64 ? ~0ull : ((1ull << (e - j + 1)) - 1);
        ++g.nruns;
        j = e + 1;
    }
    g.q0_is_col = (tmask & 1ull) ? 0 : 1;
    g.step = g.q0_is_col ? 2 : 1;
    return g;
}

// Device: (row, column, global offset within the tile) of tile-local index x.
__device__ __forceinline__ void tile_decompose(const TileGeom &g, uint32_t x, uint32_t &r, uint32_t &c, uint64_t &off) {
    const uint32_t xl = x & ((1u << g.L) - 1), xh = x >> g.L;
    uint32_t rl = 0, cc = xl;
    for (int j = g.nlow_t - 1; j >= 0; --j) {
        const int qb = g.low_t[j];
        rl = (rl << 1) | ((xl >> qb) & 1u);
        cc = ((cc >> (qb + 1)) << qb) | (cc & ((1u << qb) - 1));
    }
    r = rl | (xh << g.nlow_t);
    c = cc;
    uint64_t o = xl;
    for (int j = 0; j < g.nhigh; ++j) o |= (uint64_t)((xh >> j) & 1u) << g.high_t[j];
    off = o;
}

__device__ __forceinline__ uint64_t tile_base(const TileGeom &g, uint64_t t) {
    uint64_t base = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < g.nruns) base |= ((t >> g.run_src[j]) & g.run_mask[j]) << g.run_dst[j];
    return base;
}

__device__ __forceinline__ uint32_t tile_swz(const TileGeom &g, uint32_t r) {
    return ((r ^ (r >> 1)) * (uint32_t)g.step) & ((1u << g.nb) - 1);
}

// Shared-memory element index of (r, c).
__device__ __forceinline__ uint32_t tile_sidx(const TileGeom &g, uint32_t r, uint32_t c) {
    return (r << g.nb) | (c ^ tile_swz(g, r));
}

// Per-thread and per-iteration parts of the address-order walk.
struct TileWalk {
    uint32_t r0, c0;        // this thread's chunk x0 = 2 * tid
    uint64_t off0;
    int iters;              // chunks per thread per tile
    bool active;            // x0 lies inside the tile
};

struct TileIterTab {        // one entry per iteration i (x = x0 + i * 2 * nthr)
    uint32_t r, c;
    uint64_t off;
};

__device__ __forceinline__ TileWalk tile_walk_init(const TileGeom &g, int tid, int nthr) {
    TileWalk w;
    const uint32_t tile_amps = 1u << (g.k + g.nb);
    const uint32_t x0 = 2u * (uint32_t)tid;
    w.active = x0 < tile_amps;
    w.iters = (int)((tile_amps + 2u * nthr - 1) / (2u * nthr));
    if (w.active) tile_decompose(g, x0, w.r0, w.c0, w.off0);
    else { w.r0 = w.c0 = 0; w.off0 = 0; }
    return w;
}

// Fill tab[i] for i < iters (call from threads 0..iters-1, then __syncthreads).
__device__ __forceinline__ void tile_iter_fill(const TileGeom &g, int nthr, int i, TileIterTab *tab) {
    uint32_t r, c;
    uint64_t off;
    tile_decompose(g, (uint32_t)i * 2u * (uint32_t)nthr, r, c, off);
    tab[i].r = r;
    tab[i].c = c;
    tab[i].off = off;
}

// ---------------------------------------------------------------- cp.async
__device__ __forceinline__ void cp_async_16(void *smem, const void *gmem) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_8(void *smem, const void *gmem) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Issue the asynchronous copy of tile `base` into S (element type V2: float2 or double2).
template <typename V2>
__device__ __forceinline__ void tile_load_async(const TileGeom &g, const TileWalk &w, const TileIterTab *tab,
                                                const V2 *gsrc, uint64_t base, V2 *S) {
    if (!w.active) return;
    for (int i = 0; i < w.iters; ++i) {
        const uint32_t r = w.r0 | tab[i].r, c = w.c0 | tab[i].c;
        const uint64_t gi = base | w.off0 | tab[i].off;   // amplitude index of the chunk's first element
        if constexpr (sizeof(V2) == 8) {
            if (g.q0_is_col) {
                cp_async_16(S + tile_sidx(g, r, c), gsrc + gi);
            } else {   // the pair is rows r, r + 1 of column c
                cp_async_8(S + tile_sidx(g, r, c), gsrc + gi);
                cp_async_8(S + tile_sidx(g, r + 1, c), gsrc + gi + 1);
            }
        } else {
            const uint32_t r1 = g.q0_is_col ? r : r + 1, c1 = g.q0_is_col ? c + 1 : c;
            cp_async_16(S + tile_sidx(g, r, c), gsrc + gi);
            cp_async_16(S + tile_sidx(g, r1, c1), gsrc + gi + 1);
        }
    }
}

// Store tile S back to global memory in address order (coalesced, streaming).
template <typename V2>
__device__ __forceinline__ void tile_store(const TileGeom &g, const TileWalk &w, const TileIterTab *tab, V2 *gdst,
                                           uint64_t base, const V2 *S) {
    if (!w.active) return;
    for (int i = 0; i < w.iters; ++i) {
        const uint32_t r = w.r0 | tab[i].r, c = w.c0 | tab[i].c;
        const uint64_t gi = base | w.off0 | tab[i].off;
        const uint32_t r1 = g.q0_is_col ? r : r + 1, c1 = g.q0_is_col ? c + 1 : c;
        const V2 a = S[tile_sidx(g, r, c)], b = S[tile_sidx(g, r1, c1)];
        if constexpr (sizeof(V2) == 8) {
            __stcs(reinterpret_cast<float4 *>(gdst + gi), make_float4(a.x, a.y, b.x, b.y));
        } else {
            __stcs(gdst + gi, a);
            __stcs(gdst + gi + 1, b);
        }
    }
}

}  // namespace qi
