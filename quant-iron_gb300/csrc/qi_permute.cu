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

}  // namespace qi
