// qi_permute.cu — a run of X / CNOT / SWAP gates as one GF(2)-affine index permutation.
//
// Each of these gates maps basis index j to an index whose bits are XORs of j's bits plus a
// constant (X: flip, CNOT: target ^= control, SWAP: exchange), so a whole run is one map
// f(j) = A j ^ b over GF(2).  The engine stores A by columns in byte tables
// (T_t[v] = XOR of the columns of the set bits of v << 8t), so f(j) costs one shared-memory
// lookup per index byte.  Un-applying the run is the gather out[j] = in[f(j)]: one read and
// one write of the state instead of a fused block per window of the run.
#include "qi_internal.hpp"
#include "qi_device.cuh"

#include <algorithm>
#include <cstring>
#include <utility>

namespace qi {

bool affine_gate(const GateMatrix &gm) {
    if (gm.pauli) return false;
    if (gm.kind == QI_GATE_X || gm.kind == QI_GATE_CNOT || gm.kind == QI_GATE_TOFFOLI) return gm.controls.size() <= 1;
    return gm.kind == QI_GATE_SWAP && gm.controls.empty();
}

void affine_identity(AffineMap &m) {
    for (int k = 0; k < 64; ++k) m.row[k] = 1ull << k;
    m.b = 0;
}

// m := gate o m (the gate acts after the gates already in m).
void affine_compose(AffineMap &m, const GateMatrix &gm) {
    if (gm.kind == QI_GATE_SWAP) {
        const int a = gm.t[0], c = gm.t[1];
        std::swap(m.row[a], m.row[c]);
        const uint64_t ba = (m.b >> a) & 1ull, bc = (m.b >> c) & 1ull;
        if (ba != bc) m.b ^= (1ull << a) | (1ull << c);
        return;
    }
    const int t = gm.t[0];
    if (gm.controls.empty()) {
        m.b ^= 1ull << t;
    } else {
        const int c = gm.controls[0];
        m.row[t] ^= m.row[c];
        m.b ^= ((m.b >> c) & 1ull) << t;
    }
}

template <typename IDX> struct AffineTables {
    IDX tab[kAffineMaxBytes][256];
    IDX b;
    int32_t ntab;
};

// out[j] = in[f(j)], four independent gathers in flight per thread.
template <typename V2, typename IDX>
__global__ void __launch_bounds__(256) k_affine_gather(V2 *__restrict__ out, const V2 *__restrict__ in, uint64_t dim,
                                                       const __grid_constant__ AffineTables<IDX> p) {
    __shared__ IDX stab[kAffineMaxBytes * 256];
    for (int k = threadIdx.x; k < p.ntab * 256; k += blockDim.x) stab[k] = p.tab[k >> 8][k & 255];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    constexpr int U = 4;
    for (uint64_t j0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j0 < dim; j0 += U * stride) {
        V2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t j = j0 + u * stride;
            if (j < dim) {
                IDX src = p.b;
                for (int t = 0; t < p.ntab; ++t) src ^= stab[t * 256 + (int)((j >> (8 * t)) & 255)];
                v[u] = in[src];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t j = j0 + u * stride;
            if (j < dim) out[j] = v[u];
        }
    }
}

template <typename IDX>
static void build_tables(int n, const AffineMap &m, AffineTables<IDX> &p) {
    uint64_t col[64] = {0};
    for (int k = 0; k < n; ++k)
        for (int c = 0; c < n; ++c)
            if ((m.row[k] >> c) & 1ull) col[c] |= 1ull << k;
    p.ntab = (n + 7) / 8;
    p.b = (IDX)m.b;
    for (int t = 0; t < p.ntab; ++t)
        for (int v = 0; v < 256; ++v) {
            uint64_t acc = 0;
            for (int e = 0; e < 8; ++e)
                if (((v >> e) & 1) && 8 * t + e < n) acc ^= col[8 * t + e];
            p.tab[t][v] = (IDX)acc;
        }
}

Status affine_gather_async(qi_state *s, void *out, const void *in, const AffineMap &m) {
    if (s->n > 8 * kAffineMaxBytes) return err(QI_ERR_UNSUPPORTED, s->n, 8 * kAffineMaxBytes, "affine permutation width");
    uint64_t g = (s->dim() + 1023) / 1024;
    g = std::max<uint64_t>(1, std::min<uint64_t>(g, 152 * 8));
    if (s->n <= 32) {
        AffineTables<uint32_t> p;
        build_tables(s->n, m, p);
        if (s->prec == QI_F32) k_affine_gather<float2, uint32_t><<<(unsigned)g, 256, 0, s->stream>>>((float2 *)out, (const float2 *)in, s->dim(), p);
        else k_affine_gather<double2, uint32_t><<<(unsigned)g, 256, 0, s->stream>>>((double2 *)out, (const double2 *)in, s->dim(), p);
    } else {
        AffineTables<uint64_t> p;
        build_tables(s->n, m, p);
        if (s->prec == QI_F32) k_affine_gather<float2, uint64_t><<<(unsigned)g, 256, 0, s->stream>>>((float2 *)out, (const float2 *)in, s->dim(), p);
        else k_affine_gather<double2, uint64_t><<<(unsigned)g, 256, 0, s->stream>>>((double2 *)out, (const double2 *)in, s->dim(), p);
    }
    count_launch();
    return check_launch("k_affine_gather");
}

// ---------------------------------------------------------------- qubit permutations
// out[j] = in[s(j)], s(j) = flip ^ sum_k bit k of j << perm[k].  A tile is every index that
// varies only in the tile bits T = {k : k < L or perm[k] < L} (the output's L lowest bits and
// the outputs whose sources are the source's L lowest bits), so the reads run over 2^L
// consecutive source amplitudes and the writes over 2^L consecutive output amplitudes; the
// tile (up to 2^2L amplitudes) passes through shared memory, one pad slot per 2^L entries
// against bank conflicts.  Per-element offsets come from two tables of 2^L entries (the
// tile index's low and high L bits).  L = 6 for FP32 (512-byte runs), 5 for FP64.
constexpr int kPermTileBits = 12;
struct BitPermParams {
    uint64_t flip;
    uint64_t ntiles;
    int32_t nt, no;                  // tile bits, outer bits
    int8_t tbits[kPermTileBits];     // tile bits (output side), ascending
    int8_t sbits[kPermTileBits];     // their sources, ascending
    int8_t sdst[kPermTileBits];      // source tile bit i comes from tile bit sdst[i]
    int8_t obits[64];                // outer bits (output side), ascending
    int8_t perm[64];
};

template <int L> struct PermRun;
template <> struct PermRun<5> { static constexpr int kTile = 1 << 10; };
template <> struct PermRun<6> { static constexpr int kTile = 1 << 12; };

// With `partials`, the block also sums |amplitude|^2 of what it writes (FP32 per tile and thread for
// FP32 states, folded into FP64) into partials[blockIdx.x * 4]: the norm of the permuted state for
// a renormalisation that follows, without a read pass of its own.
template <typename V2, int L>
__global__ void __launch_bounds__(256) k_bitperm(V2 *__restrict__ out, const V2 *__restrict__ in,
                                                 const __grid_constant__ BitPermParams p, double *partials) {
    constexpr int TMAX = PermRun<L>::kTile, H = 1 << L, U = 4;
    __shared__ V2 tile[TMAX + TMAX / H];
    __shared__ uint64_t rd_lo[H], rd_hi[H], wr_lo[H], wr_hi[H];
    __shared__ uint16_t dst_lo[H], dst_hi[H];
    __shared__ uint64_t dep_j[2 * kAffineMaxBytes][16], dep_s[2 * kAffineMaxBytes][16];   // per 4-bit nibble
    const int nlo = min(p.nt, L), nhi = p.nt - nlo;
    for (int v = threadIdx.x; v < H; v += blockDim.x) {
        uint64_t rl = 0, rh = 0, wl = 0, wh = 0;
        uint32_t dl = 0, dh = 0;
        for (int i = 0; i < L; ++i) {
            if (!((v >> i) & 1)) continue;
            if (i < nlo) {
                rl |= 1ull << p.sbits[i];
                wl |= 1ull << p.tbits[i];
                dl |= 1u << p.sdst[i];
            }
            if (i < nhi) {
                rh |= 1ull << p.sbits[nlo + i];
                wh |= 1ull << p.tbits[nlo + i];
                dh |= 1u << p.sdst[nlo + i];
            }
        }
        rd_lo[v] = rl;
        rd_hi[v] = rh;
        wr_lo[v] = wl;
        wr_hi[v] = wh;
        dst_lo[v] = (uint16_t)dl;
        dst_hi[v] = (uint16_t)dh;
    }
    // outer index t -> (output base, source base) by one table lookup per nibble of t
    const int nnib = (p.no + 3) / 4;
    for (int k = threadIdx.x; k < nnib * 16; k += blockDim.x) {
        const int b = k >> 4, v = k & 15;
        uint64_t dj = 0, ds = 0;
        for (int e = 0; e < 4; ++e) {
            const int i = 4 * b + e;
            if (i < p.no && ((v >> e) & 1)) {
                dj |= 1ull << p.obits[i];
                ds |= 1ull << p.perm[p.obits[i]];
            }
        }
        dep_j[b][v] = dj;
        dep_s[b][v] = ds;
    }
    __syncthreads();
    const int te = 1 << p.nt, lmask = (1 << nlo) - 1;
    const int step = blockDim.x;
    double acc = 0.0;
    for (uint64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        uint64_t bj = 0, bs = p.flip;
        for (int b = 0; b < nnib; ++b) {
            const int v = (int)((t >> (4 * b)) & 15);
            bj |= dep_j[b][v];
            bs ^= dep_s[b][v];
        }
        for (int e0 = threadIdx.x; e0 < te; e0 += U * step) {   // U gathers in flight per thread
            V2 v[U];
            uint32_t d[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + u * step;
                if (e < te) {
                    const int el = e & lmask, eh = e >> nlo;
                    d[u] = (uint32_t)dst_lo[el] | dst_hi[eh];
                    v[u] = in[bs ^ rd_lo[el] ^ rd_hi[eh]];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (e0 + u * step < te) tile[d[u] + (d[u] >> L)] = v[u];
        }
        __syncthreads();
        decltype(V2::x) tsum = 0;
        for (int e = threadIdx.x; e < te; e += step) {
            const int el = e & lmask, eh = e >> nlo;
            const V2 w = tile[e + (e >> L)];
            out[bj | wr_lo[el] | wr_hi[eh]] = w;
            tsum += w.x * w.x + w.y * w.y;
        }
        acc += (double)tsum;
        __syncthreads();
    }
    if (partials) {   // uniform over the grid
        const double v = block_sum(acc);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * 4] = v;
    }
}

Status bitperm_async(qi_state *s, void *out, const void *in, const int8_t *perm, uint64_t flip, unsigned *norm_nb) {
    const int n = s->n;
    if (n > 8 * kAffineMaxBytes) return err(QI_ERR_UNSUPPORTED, n, 8 * kAffineMaxBytes, "qubit permutation width");
    BitPermParams p;
    std::memset(&p, 0, sizeof(p));
    int src_of[64];   // source bit -> output bit
    for (int k = 0; k < n; ++k) {
        p.perm[k] = perm[k];
        src_of[perm[k]] = k;
    }
    const int L = s->prec == QI_F32 ? 6 : 5;   // run bits: 512-byte (FP32) / 512-byte (FP64) runs
    bool in_tile[64] = {false};
    for (int k = 0; k < n; ++k)
        if (k < L || perm[k] < L) in_tile[k] = true;
    int tpos[64];
    for (int k = 0; k < n; ++k)
        if (in_tile[k]) {
            tpos[k] = p.nt;
            p.tbits[p.nt++] = (int8_t)k;
        } else {
            p.obits[p.no++] = (int8_t)k;
        }
    // sources of the tile bits, ascending, each with its tile bit
    int ns = 0;
    for (int q = 0; q < n; ++q)
        if (in_tile[src_of[q]]) {
            p.sbits[ns] = (int8_t)q;
            p.sdst[ns] = (int8_t)tpos[src_of[q]];
            ++ns;
        }
    p.flip = flip;
    p.ntiles = 1ull << p.no;
    const uint64_t g = std::max<uint64_t>(1, std::min<uint64_t>(p.ntiles, 152 * 4));   // <= kReduceBlocks
    double *partials = norm_nb ? s->d_partials : nullptr;
    if (s->prec == QI_F32)
        k_bitperm<float2, 6><<<(unsigned)g, 256, 0, s->stream>>>((float2 *)out, (const float2 *)in, p, partials);
    else
        k_bitperm<double2, 5><<<(unsigned)g, 256, 0, s->stream>>>((double2 *)out, (const double2 *)in, p, partials);
    if (norm_nb) *norm_nb = (unsigned)g;
    count_launch();
    return check_launch("k_bitperm");
}

Status bitperm_in_place_async(qi_state *s, const int8_t *perm, uint64_t flip) {
    // out[j] = in[s(j)] moves the amplitude at source bit perm[k] to output bit k.  Realise the
    // bit permutation by transpositions: walk output positions k = 0.., swapping the qubit that
    // currently sits where bit k's source is into place.  cur[q] = the source bit held at q.
    const int n = s->n;
    int cur[64], where[64];
    for (int q = 0; q < n; ++q) cur[q] = where[q] = q;
    // flips act on the source index: apply them first (X on source bit q)
    for (int q = 0; q < n; ++q)
        if ((flip >> q) & 1ull) {
            qi_gate g;
            std::memset(&g, 0, sizeof(g));
            g.kind = QI_GATE_X;
            g.n_targets = 1;
            g.targets[0] = q;
            for (int k = 0; k < 3; ++k) g.param_ids[k] = -1;
            GateMatrix gm;
            Status st = gate_to_matrix(n, g, &gm);
            if (st.ok()) st = launch_op(s, lower_gate(n, gm), nullptr);
            if (!st.ok()) return st;
        }
    for (int k = 0; k < n; ++k) {
        const int want = perm[k];            // source bit that must end at position k
        const int at = where[want];
        if (at == k) continue;
        qi_gate g;
        std::memset(&g, 0, sizeof(g));
        g.kind = QI_GATE_SWAP;
        g.n_targets = 2;
        g.targets[0] = k;
        g.targets[1] = at;
        for (int j = 0; j < 3; ++j) g.param_ids[j] = -1;
        GateMatrix gm;
        Status st = gate_to_matrix(n, g, &gm);
        if (st.ok()) st = launch_op(s, lower_gate(n, gm), nullptr);
        if (!st.ok()) return st;
        const int other = cur[k];
        cur[k] = want;
        cur[at] = other;
        where[want] = k;
        where[other] = at;
    }
    return ok_status();
}

}  // namespace qi
