// qi_plan.cu — circuit plans: validation, the gate-fusion pass and execution.
//
// Reference: Circuit::execute (src/circuit.rs:160-172) applies gates one by
// one, each a full copy of the state (Gate::apply, src/components/gate.rs:99-122).
// A plan validates the whole gate list first (so an invalid gate leaves the
// state untouched, as the reference's functional execute does), then lowers
// it to device operations:
//   QI_FUSION_NONE   one streaming kernel per gate (the plain per-gate method);
//   QI_FUSION_GREEDY the greedy fuser below with block width k;
//   QI_FUSION_LEARNED candidate partitions scored by the learned cost model
//                    (qi_costmodel.cu), greedy as the fallback;
//   QI_FUSION_PAULI_GROUPS per gate, but runs of Pauli exponentials with X-masks
//                    in {0, X} become one grouped pass each (qi_pauli.cu).
//
// Greedy fuser ("light-cone" absorption).  A block starts empty; the
// remaining gates are scanned in order.  A gate joins the block when its
// qubits fit (|Q u S| <= k) and it does not depend on a gate that was passed
// over: passed-over gates block their qubits, except that diagonal gates
// commute with each other, so a diagonal gate may pass over a diagonal gate.
// Every absorbed gate therefore commutes with every passed-over gate it
// overtakes, and the block can run before all of them.
//
// The partition takes, at each step, the best of several such blocks: the
// light-cone block of the first remaining gate, and for every window of k
// consecutive qubits the block of all remaining gates inside the window that
// the same rule admits (window_partition).  The first remaining gate's block
// when it is all-diagonal is kept as is (consecutive diagonal blocks become one
// phase-polynomial pass); otherwise the candidate with the most gates wins.  On
// brickwork circuits the windows grow light-cone diamonds instead of the first
// gate's triangles: the 30-qubit 40-layer benchmark circuit needs 80 dense
// blocks and 8 diagonal runs instead of 142 and 9.
#include "qi_internal.hpp"
#include "qi_plan.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <thread>

namespace qi {

using cd = std::complex<double>;

// ------------------------------------------------------------ elements ---
Elem make_elem_from_gate(const GateMatrix &gm, int src) {
    Elem e;
    e.src = src;
    e.gm = gm;
    if (gm.measure) {   // a barrier: nothing is fused or reordered across a measurement
        e.mask = ~0ull;
        e.diagonal = false;
        e.fusable = false;
        return e;
    }
    if (gm.pauli) {
        const uint64_t sup = gm.xmask | gm.zmask;
        e.mask = gm.normalise_after ? ~0ull : sup;
        e.diagonal = gm.xmask == 0 && !gm.normalise_after;
        e.fusable = false;   // decided later (dense only if narrow enough)
        e.pauli = true;
        return e;
    }
    uint64_t m = 0;
    for (int j = 0; j < gm.nt; ++j) m |= 1ull << gm.t[j];
    for (int32_t c : gm.controls) m |= 1ull << c;
    e.mask = m;
    e.diagonal = gm.diagonal;
    e.fusable = gm.nt > 0;
    return e;
}

// Dense matrix of an element on its support (sorted qubits of e.mask).
static void dense_of(const Elem &e, std::vector<int> &sup, std::vector<cd> &D) {
    sup.clear();
    for (int q = 0; q < 64; ++q)
        if ((e.mask >> q) & 1ull) sup.push_back(q);
    const int s = (int)sup.size();
    const int dim = 1 << s;
    D.assign((size_t)dim * dim, cd(0, 0));
    auto local = [&](int q) { return (int)(std::find(sup.begin(), sup.end(), q) - sup.begin()); };
    if (e.pauli) {
        // cosh(a) I + sinh(a) P on the support
        uint32_t lx = 0, lz = 0;
        for (int j = 0; j < s; ++j) {
            if ((e.gm.xmask >> sup[j]) & 1ull) lx |= 1u << j;
            if ((e.gm.zmask >> sup[j]) & 1ull) lz |= 1u << j;
        }
        const int ny = __builtin_popcount(lx & lz);
        const cd mi_pow[4] = {cd(1, 0), cd(0, -1), cd(-1, 0), cd(0, 1)};
        const double ar = e.gm.alpha_re, ai = e.gm.alpha_im;
        const cd ch(std::cosh(ar) * std::cos(ai), std::sinh(ar) * std::sin(ai));
        const cd sh(std::sinh(ar) * std::cos(ai), std::cosh(ar) * std::sin(ai));
        for (int o = 0; o < dim; ++o) {
            D[(size_t)o * dim + o] += ch;
            const double sg = (__builtin_popcount(o & lz) & 1) ? -1.0 : 1.0;
            D[(size_t)o * dim + (o ^ lx)] += sh * mi_pow[ny & 3] * sg;
        }
        return;
    }
    const GateMatrix &g = e.gm;
    uint32_t cmask = 0;
    for (int32_t c : g.controls) cmask |= 1u << local(c);
    int tl[2] = {0, 0};
    for (int j = 0; j < g.nt; ++j) tl[j] = local(g.t[j]);
    const int td = 1 << g.nt;
    for (int col = 0; col < dim; ++col) {
        if ((col & cmask) != cmask) { D[(size_t)col * dim + col] = cd(1, 0); continue; }
        int tin = 0;
        for (int j = 0; j < g.nt; ++j) tin |= ((col >> tl[j]) & 1) << j;
        int rest = col;
        for (int j = 0; j < g.nt; ++j) rest &= ~(1 << tl[j]);
        for (int tout = 0; tout < td; ++tout) {
            int row = rest;
            for (int j = 0; j < g.nt; ++j) row |= ((tout >> j) & 1) << tl[j];
            D[(size_t)row * dim + col] = cd(g.m[2 * (tout * td + tin)], g.m[2 * (tout * td + tin) + 1]);
        }
    }
}

// B <- G_embedded * B, B row-major 2^nq x 2^nq, G dense on local positions pos[].
static void left_multiply(std::vector<cd> &B, int nq, const std::vector<int> &pos, const std::vector<cd> &G) {
    const int dim = 1 << nq, s = (int)pos.size(), gd = 1 << s;
    uint32_t smask = 0;
    for (int p : pos) smask |= 1u << p;
    std::vector<int> offs(gd);
    for (int r = 0; r < gd; ++r) {
        int o = 0;
        for (int j = 0; j < s; ++j) o |= ((r >> j) & 1) << pos[j];
        offs[r] = o;
    }
    std::vector<cd> in(gd), out(gd);
    for (int base = 0; base < dim; ++base) {
        if (base & (int)smask) continue;
        for (int col = 0; col < dim; ++col) {
            for (int r = 0; r < gd; ++r) in[r] = B[(size_t)(base | offs[r]) * dim + col];
            for (int r = 0; r < gd; ++r) {
                cd acc(0, 0);
                for (int c = 0; c < gd; ++c) acc += G[(size_t)r * gd + c] * in[c];
                out[r] = acc;
            }
            for (int r = 0; r < gd; ++r) B[(size_t)(base | offs[r]) * dim + col] = out[r];
        }
    }
}

// ---------------------------------------------------------------- fuser ---
// The light-cone block of the first remaining element: scan the remaining
// elements in order, absorbing every one that fits (|Q u S| <= k) and depends
// on no passed-over element.
Block light_cone_block(const std::vector<Elem> &elems, const std::vector<int> &remaining, int n, int kmax) {
    Block b;
    const uint64_t all = n >= 64 ? ~0ull : ((1ull << n) - 1);
    const Elem &first = elems[remaining[0]];
    if (!first.fusable || __builtin_popcountll(first.mask) > kmax) {
        b.members.push_back(remaining[0]);
        b.mask = first.mask;
        b.single = true;
        return b;
    }
    uint64_t Q = 0, blocked_any = 0, blocked_diag = 0;
    for (int idx : remaining) {
        const Elem &e = elems[idx];
        const uint64_t S = e.mask;
        bool can = e.fusable && __builtin_popcountll(S) <= kmax;
        if (can) {
            if (S & blocked_any) can = false;
            else if (!e.diagonal && (S & blocked_diag)) can = false;
            else if (__builtin_popcountll(Q | S) > kmax) can = false;
        }
        if (can) {
            Q |= S;
            b.members.push_back(idx);
        } else {
            if (e.diagonal && e.fusable) blocked_diag |= S;
            else blocked_any |= S;
            if ((blocked_any & all) == all) break;
        }
    }
    b.mask = Q;
    b.single = b.members.size() == 1;
    return b;
}

// Everything the window W can absorb: the remaining elements on qubits inside W
// that depend on no passed-over element (same blocking rule as above).
Block window_block(const std::vector<Elem> &elems, const std::vector<int> &remaining, uint64_t W) {
    Block b;
    uint64_t blocked_any = 0, blocked_diag = 0;
    for (int idx : remaining) {
        const Elem &e = elems[idx];
        const uint64_t S = e.mask;
        bool can = e.fusable && S != 0 && (S & ~W) == 0;
        if (can) {
            if (S & blocked_any) can = false;
            else if (!e.diagonal && (S & blocked_diag)) can = false;
        }
        if (can) {
            b.mask |= S;
            b.members.push_back(idx);
        } else {
            if (e.diagonal && e.fusable) blocked_diag |= S;
            else blocked_any |= S;
            if ((blocked_any & W) == W) break;   // nothing further can enter the window
        }
    }
    b.single = b.members.size() == 1;
    return b;
}

template <typename Pick>
static std::vector<Block> partition_with(const std::vector<Elem> &elems, int n, int kmax, Pick pick) {
    std::vector<Block> blocks;
    std::vector<int> remaining(elems.size());
    for (size_t i = 0; i < elems.size(); ++i) remaining[i] = (int)i;
    std::vector<char> taken(elems.size(), 0);
    while (!remaining.empty()) {
        Block b = pick(remaining);
        for (int idx : b.members) taken[idx] = 1;
        std::vector<int> rest;
        rest.reserve(remaining.size());
        for (int idx : remaining)
            if (!taken[idx]) rest.push_back(idx);
        remaining.swap(rest);
        blocks.push_back(std::move(b));
    }
    return blocks;
}

std::vector<Block> greedy_partition(const std::vector<Elem> &elems, int n, int kmax) {
    return partition_with(elems, n, kmax,
                          [&](const std::vector<int> &rem) { return light_cone_block(elems, rem, n, kmax); });
}

std::vector<Block> window_partition(const std::vector<Elem> &elems, int n, int kmax) {
    return partition_with(elems, n, kmax, [&](const std::vector<int> &rem) {
        Block best = light_cone_block(elems, rem, n, kmax);
        if (best.single) return best;
        bool diag = true;
        for (int idx : best.members) diag = diag && elems[idx].diagonal;
        if (diag) return best;   // joins (or starts) a run of diagonal blocks: one phase-polynomial pass
        const uint64_t win = (1ull << kmax) - 1;
        for (int a = 0; a + kmax <= n; ++a) {
            Block w = window_block(elems, rem, win << a);
            if (w.members.size() > best.members.size()) best = std::move(w);
        }
        return best;
    });
}

// Dense (or diagonal) matrix of a block on its sorted qubits.
void compose_block(const std::vector<Elem> &elems, const Block &b, std::vector<int> &qubits, std::vector<cd> &B) {
    qubits.clear();
    for (int q = 0; q < 64; ++q)
        if ((b.mask >> q) & 1ull) qubits.push_back(q);
    const int nq = (int)qubits.size();
    const int dim = 1 << nq;
    B.assign((size_t)dim * dim, cd(0, 0));
    for (int i = 0; i < dim; ++i) B[(size_t)i * dim + i] = cd(1, 0);
    std::vector<int> sup, pos;
    std::vector<cd> D;
    for (int idx : b.members) {
        dense_of(elems[idx], sup, D);
        pos.clear();
        for (int q : sup) pos.push_back((int)(std::find(qubits.begin(), qubits.end(), q) - qubits.begin()));
        left_multiply(B, nq, pos, D);
    }
}

// ------------------------------------------------------------------ plan ---
// Runs of at least kPermMinSwaps uncontrolled SWAPs (X gates may sit between them) whose
// qubits do not fit one fused block: one qubit permutation (a tiled transpose, one pass)
// instead of the blocks a partition would spend on pure data movement (the SWAP network
// at the end of a QFT on n qubits fills n / 6 blocks).
constexpr int kPermMinSwaps = 3;

static bool perm_elem(const Elem &e) {
    const GateMatrix &g = e.gm;
    if (e.pauli || !g.controls.empty()) return false;
    return g.kind == QI_GATE_SWAP || (g.kind == QI_GATE_X && g.nt == 1);
}

static std::vector<Block> partition_with_permutations(qi_plan *p, const std::vector<Elem> &elems, int kmax) {
    std::vector<Block> out;
    size_t seg = 0;   // first element not yet partitioned
    auto take_segment = [&](size_t end) {
        if (end <= seg) return;
        std::vector<Elem> sub(elems.begin() + (long)seg, elems.begin() + (long)end);
        std::vector<Block> bs = choose_partition(p, sub, kmax);
        for (Block &b : bs) {
            for (int &m : b.members) m += (int)seg;
            out.push_back(std::move(b));
        }
    };
    for (size_t i = 0; i < elems.size();) {
        if (!perm_elem(elems[i])) {
            ++i;
            continue;
        }
        size_t j = i;
        int swaps = 0;
        uint64_t support = 0;
        for (; j < elems.size() && perm_elem(elems[j]); ++j) {
            swaps += elems[j].gm.kind == QI_GATE_SWAP;
            support |= elems[j].mask;
        }
        if (swaps >= kPermMinSwaps && __builtin_popcountll(support) > kmax) {
            take_segment(i);
            Block b;
            b.perm = true;
            b.mask = support;
            for (size_t k = i; k < j; ++k) b.members.push_back((int)k);
            out.push_back(std::move(b));
            seg = j;
        }
        i = j;
    }
    take_segment(elems.size());
    return out;
}

// The run's gather: applying gates G_1..G_m is out[j] = in[s(j)] with s the inverse of their
// index map, i.e. the gates' own (self-inverse) maps composed in reverse order.
static Op bitperm_op(const std::vector<Elem> &elems, const Block &b) {
    AffineMap g;
    affine_identity(g);
    for (auto it = b.members.rbegin(); it != b.members.rend(); ++it) affine_compose(g, elems[(size_t)*it].gm);
    Op op;
    op.kind = OP_BITPERM;
    op.k = (int32_t)b.members.size();
    op.xmask = g.b;
    for (int m = 0; m < 64; ++m)   // row m of g is the single bit j_k: source bit m <- output bit k
        if (g.row[m]) op.perm[__builtin_ctzll(g.row[m])] = (int8_t)m;
    return op;
}

// Widen a dense k-qubit block (k < 5; local bit j <-> op.targets[j], ascending) to 5 qubits: the
// lowest qubits outside it join as identity factors.  op.targets / op.k and the matrix M are
// rewritten in place (local bits again ascending by qubit).
static void pad_block_to_5(int n, Op &op, std::vector<cd> &M) {
    const int k = op.k;
    uint64_t mask = 0;
    for (int j = 0; j < k; ++j) mask |= 1ull << op.targets[j];
    uint64_t sel = mask;
    for (int q = 0, need = 5 - k; q < n && need > 0; ++q)
        if (!((mask >> q) & 1ull)) {
            sel |= 1ull << q;
            --need;
        }
    int qs[5], nq = 0;
    for (int q = 0; q < 64 && nq < 5; ++q)
        if ((sel >> q) & 1ull) qs[nq++] = q;
    int src[5];   // new local bit -> old local bit, or -1 for a padding qubit
    for (int j = 0; j < 5; ++j) {
        src[j] = -1;
        for (int i = 0; i < k; ++i)
            if (op.targets[i] == qs[j]) src[j] = i;
    }
    const int od = 1 << k;
    std::vector<cd> W((size_t)32 * 32, cd(0, 0));
    for (int r = 0; r < 32; ++r)
        for (int c = 0; c < 32; ++c) {
            int ro = 0, co = 0;
            bool same = true;
            for (int j = 0; j < 5; ++j) {
                const int rb = (r >> j) & 1, cb = (c >> j) & 1;
                if (src[j] < 0) same = same && rb == cb;
                else {
                    ro |= rb << src[j];
                    co |= cb << src[j];
                }
            }
            if (same) W[(size_t)r * 32 + c] = M[(size_t)ro * od + co];
        }
    M.swap(W);
    op.k = 5;
    for (int j = 0; j < 5; ++j) op.targets[j] = qs[j];
}

Status build_plan(qi_plan *p, std::vector<Elem> &elems) {
    const int n = p->n;
    int fusion = p->opts.fusion;
    int kmax = p->opts.max_block_qubits > 0 ? p->opts.max_block_qubits : 6;
    kmax = std::min(kmax, std::min(6, n));
    if (p->prec == QI_F64) kmax = std::min(kmax, 5);
    int use_tc = p->opts.use_tensor_cores != 2;
    p->ops.clear();
    p->mats.clear();
    p->tc.clear();
    p->polys.clear();
    int tc_blocks_since = 0, tc_total = 0;
    std::fill(std::begin(p->stats.n_blocks_by_k), std::end(p->stats.n_blocks_by_k), 0);
    p->stats.n_gates = (int64_t)elems.size();
    p->stats.predicted_us = 0.0;
    if (fusion == QI_FUSION_LEARNED && p->partition_override.empty()) {
        // the cost model picks per-gate vs greedy k (and tensor cores); greedy k = kmax without a model
        int kbest = kmax, tcbest = use_tc;
        double ms = 0.0;
        if (learned_choice(p, elems, kmax, &kbest, &tcbest, &ms)) {
            p->stats.predicted_us = ms * 1e3;
            if (kbest <= 1) fusion = QI_FUSION_NONE;
            kmax = std::max(2, kbest);
            use_tc = tcbest;
        }
    }
    // Pauli exponentials narrow enough become dense elements when fusing.
    for (Elem &e : elems) {
        if (e.pauli && !e.gm.normalise_after && fusion != QI_FUSION_NONE && __builtin_popcountll(e.mask) <= kmax)
            e.fusable = true;
    }
    auto lower_single = [&](const Elem &e) {
        Op op = lower_gate(n, e.gm);
        if (op.kind == OP_PAULI_EXP) {
            const double ar = op.alpha_re, ai = op.alpha_im;
            op.cre = std::cosh(ar) * std::cos(ai);
            op.cim = std::sinh(ar) * std::sin(ai);
            op.sre = std::sinh(ar) * std::cos(ai);
            op.sim = std::cosh(ar) * std::sin(ai);
        }
        if (op.kind != OP_NOP) {
            p->ops.push_back(op);
            p->stats.n_blocks_by_k[0]++;
        }
    };
    if (fusion == QI_FUSION_NONE || fusion == QI_FUSION_PAULI_GROUPS) {
        auto groupable = [&](const Elem &e) {
            return fusion == QI_FUSION_PAULI_GROUPS && e.pauli && !e.gm.normalise_after;
        };
        for (size_t i = 0; i < elems.size();) {
            if (!groupable(elems[i])) {
                lower_single(elems[i++]);
                continue;
            }
            std::vector<const GateMatrix *> run;
            size_t j = i;
            for (; j < elems.size() && groupable(elems[j]); ++j) run.push_back(&elems[j].gm);
            for (size_t used = 0; used < run.size();) {
                Op op;
                const size_t took = pauli_group_op(run, used, op, p->mats);
                if (took == 1) {
                    lower_single(elems[i + used]);
                } else {
                    p->ops.push_back(op);
                    p->stats.n_blocks_by_k[0]++;
                }
                used += took;
            }
            i = j;
        }
    } else {
        std::vector<Block> blocks = p->partition_override.empty() ? partition_with_permutations(p, elems, kmax)
                                                                  : p->partition_override;
        // compose block matrices in parallel (independent)
        std::vector<std::vector<int>> qb(blocks.size());
        std::vector<std::vector<cd>> mb(blocks.size());
        const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (unsigned w = 0; w < nth; ++w) {
            th.emplace_back([&, w] {
                for (size_t bi = w; bi < blocks.size(); bi += nth)
                    if (!blocks[bi].single && !blocks[bi].perm) compose_block(elems, blocks[bi], qb[bi], mb[bi]);
            });
        }
        for (auto &t : th) t.join();
        // FP32 plans: a run of consecutive diagonal blocks whose phases are
        // polynomials of degree <= 2 is applied as one phase polynomial (one pass;
        // also a run of one block of three or more qubits, where the polynomial pass
        // is faster than the table kernel: 2.6 vs 3.0 ms at 30 qubits).
        const bool poly_ok = p->prec == QI_F32;
        PhasePoly pending;
        std::vector<Op> pending_ops;
        if (poly_ok) pending.init(n);
        auto flush = [&]() {
            if (pending_ops.size() >= 2 || (pending_ops.size() == 1 && pending_ops[0].k >= 3)) {
                Op op;
                op.kind = OP_PHASE_POLY;
                op.k = (int32_t)pending_ops.size();
                for (const Op &d : pending_ops)
                    for (int j = 0; j < d.k; ++j) op.zmask |= 1ull << d.targets[j];
                op.mat_offset = (int64_t)p->polys.size();
                op.tc_offset = (int64_t)p->tc.size();
                p->polys.push_back(pending);
                Op *prev = p->ops.empty() ? nullptr : &p->ops.back();
                if (prev && prev->kind == OP_FUSED && prev->tc_offset >= 0 && prev->poly_tc < 0 &&
                    tc_phase_table(pending, prev->k, prev->targets, p->tc)) {
                    // right after a tensor-core block: its epilogue applies the phases (no extra pass)
                    prev->poly_tc = op.tc_offset;
                    prev->poly_idx = op.mat_offset;
                } else {
                    phase_poly_device_block(pending, p->tc);
                    p->ops.push_back(op);
                }
            } else if (pending_ops.size() == 1) {
                p->ops.push_back(pending_ops[0]);
            }
            pending_ops.clear();
            if (poly_ok) pending.init(n);
        };
        for (size_t bi = 0; bi < blocks.size(); ++bi) {
            const Block &b = blocks[bi];
            if (b.single) {
                flush();
                lower_single(elems[b.members[0]]);
                continue;
            }
            if (b.perm) {
                flush();
                p->ops.push_back(bitperm_op(elems, b));
                p->stats.n_blocks_by_k[0]++;
                continue;
            }
            bool diag = true;
            for (int idx : b.members) diag = diag && elems[idx].diagonal;
            const int k = (int)qb[bi].size();
            Op op;
            op.k = k;
            for (int j = 0; j < k; ++j) op.targets[j] = qb[bi][j];
            op.mat_offset = (int64_t)p->mats.size();
            const int dim = 1 << k;
            if (diag) {
                op.kind = OP_DIAGK;
                std::vector<cd> table((size_t)dim);
                for (int r = 0; r < dim; ++r) table[(size_t)r] = mb[bi][(size_t)r * dim + r];
                p->mats.insert(p->mats.end(), table.begin(), table.end());
                if (poly_ok && phase_poly_add_table(pending, k, op.targets, table.data())) {
                    pending_ops.push_back(op);
                    p->stats.n_blocks_by_k[k]++;
                    continue;
                }
                flush();
            } else {
                flush();
                op.kind = OP_FUSED;
                op.mode = use_tc;
                if (op.mode && p->prec == QI_F32 && (k == 3 || k == 4) && n >= 12) {
                    // a 3- or 4-qubit block runs faster on the tensor cores as a 5-qubit block with the
                    // identity on the lowest free qubits (30 qubits: 3.5 ms on the CUDA cores, 2.6-2.9 ms
                    // padded; low padding qubits give the tile long row runs)
                    pad_block_to_5(n, op, mb[bi]);
                }
                const int kk = op.k, dd = 1 << kk;
                for (size_t i = 0; i < (size_t)dd * dd; ++i) p->mats.push_back(mb[bi][i]);
                if (op.mode && p->prec == QI_F32 && kk >= 5 && n >= kk + 7) {
                    op.tc_offset = (int64_t)p->tc.size();
                    tc_blocks(kk, reinterpret_cast<const double *>(mb[bi].data()), p->tc);
                }
            }
            p->ops.push_back(op);
            p->stats.n_blocks_by_k[op.k]++;
            if (op.tc_offset >= 0) {
                ++tc_blocks_since;
                ++tc_total;
                if (p->opts.renorm_every > 0 && tc_blocks_since >= p->opts.renorm_every) {
                    Op nrm;
                    nrm.kind = OP_NORMALISE;
                    p->ops.push_back(nrm);
                    tc_blocks_since = 0;
                }
            }
        }
        flush();
    }
    // Tensor-core accumulation rounds toward zero: renormalise once at the end
    // (unless disabled, or the last op already did).
    if (tc_total > 0 && p->opts.renorm_every >= 0 && (p->ops.empty() || p->ops.back().kind != OP_NORMALISE)) {
        Op nrm;
        nrm.kind = OP_NORMALISE;
        p->ops.push_back(nrm);
    }
    p->stats.n_kernels = (int64_t)p->ops.size();
    return ok_status();
}

Status upload_plan(qi_plan *p) {
    if (p->d_mats) { cudaFree(p->d_mats); p->d_mats = nullptr; }
    if (p->d_tc) { cudaFree(p->d_tc); p->d_tc = nullptr; }
    if (!p->tc.empty()) {
        QI_CUDA(cudaMalloc(&p->d_tc, p->tc.size() * sizeof(float)));
        QI_CUDA(cudaMemcpy(p->d_tc, p->tc.data(), p->tc.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (p->mats.empty()) return ok_status();
    const size_t cnt = p->mats.size();
    if (p->prec == QI_F32) {
        std::vector<float2> h(cnt);
        for (size_t i = 0; i < cnt; ++i) h[i] = make_float2((float)p->mats[i].real(), (float)p->mats[i].imag());
        QI_CUDA(cudaMalloc(&p->d_mats, cnt * sizeof(float2)));
        QI_CUDA(cudaMemcpy(p->d_mats, h.data(), cnt * sizeof(float2), cudaMemcpyHostToDevice));
    } else {
        std::vector<double2> h(cnt);
        for (size_t i = 0; i < cnt; ++i) h[i] = make_double2(p->mats[i].real(), p->mats[i].imag());
        QI_CUDA(cudaMalloc(&p->d_mats, cnt * sizeof(double2)));
        QI_CUDA(cudaMemcpy(p->d_mats, h.data(), cnt * sizeof(double2), cudaMemcpyHostToDevice));
    }
    return ok_status();
}

Status plan_elems_from_gates(int n, const qi_gate *gates, int64_t ng, const double *theta, int64_t ntheta,
                             std::vector<Elem> &elems) {
    elems.clear();
    elems.reserve((size_t)ng);
    for (int64_t k = 0; k < ng; ++k) {
        qi_gate g = gates[k];
        for (int j = 0; j < 3; ++j) {
            if (g.param_ids[j] >= 0) {
                if (!theta || g.param_ids[j] >= ntheta)
                    return err(QI_ERR_MISMATCHED_NUMBER_OF_PARAMETERS, g.param_ids[j] + 1, ntheta);
                g.params[j] = theta[g.param_ids[j]];
            }
        }
        GateMatrix gm;
        Status st = gate_to_matrix(n, g, &gm);
        if (!st.ok()) {
            st.msg = "gate " + std::to_string(k) + (st.msg.empty() ? "" : ": " + st.msg);
            return st;
        }
        elems.push_back(make_elem_from_gate(gm, (int)k));
    }
    return ok_status();
}

// Launches a plan's ops on a state.  OP_BITPERM writes out of place: the amplitudes move to
// the state's second buffer and back (the next renormalisation writes into the state's own
// buffer; otherwise one copy at the end), so the state's device pointer never changes.
struct PlanRunner {
    qi_plan *p;
    qi_state *s;
    void *home;
    unsigned norm_nb = 0;   // norm partials of the current amplitudes are in s->d_partials (rows)
    PlanRunner(qi_plan *p_, qi_state *s_) : p(p_), s(s_), home(s_->amps) {}
    Status op(const Op &o, int next_kind) {
        const unsigned have_norm = norm_nb;   // left by the op before this one
        norm_nb = 0;
        if (o.kind == OP_BITPERM) {
            void *scratch = nullptr;
            if (s->amps == home && !state_scratch(s, &scratch).ok())
                return bitperm_in_place_async(s, o.perm, o.xmask);   // no room for a second buffer
            void *dst = s->amps == home ? scratch : home;
            // a renormalisation next: the permutation sums the norm as it writes
            unsigned nb = 0;
            Status st = bitperm_async(s, dst, s->amps, o.perm, o.xmask, next_kind == OP_NORMALISE ? &nb : nullptr);
            if (st.ok()) {
                s->amps = dst;
                norm_nb = nb;
            }
            return st;
        }
        if (o.kind == OP_MEASURE && s->amps != home) {   // measure the amplitudes in the state's own buffer
            Status st = finish(ok_status());
            if (!st.ok()) return st;
        }
        if (o.kind == OP_NORMALISE && s->amps != home) {
            Status st = have_norm ? state_normalise_to_from_partials_async(s, home, s->amps, have_norm)
                                  : state_normalise_device_to_async(s, home, s->amps);
            if (st.ok()) s->amps = home;
            return st;
        }
        return launch_op(s, o, p->d_mats, p->d_tc);
    }
    Status finish(Status st) {   // the amplitudes back in the state's own buffer
        if (s->amps != home) {
            if (st.ok()) {
                cudaError_t e = cudaMemcpyAsync(home, s->amps, s->bytes(), cudaMemcpyDeviceToDevice, s->stream);
                if (e != cudaSuccess) st = cuda_status(e, "copy back after qubit permutation");
            }
            s->amps = home;
        }
        return st;
    }
};

Status plan_execute(qi_plan *p, qi_state *s) {
    if (s->n != p->n) return err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n);   // circuit.rs:161-163
    if (s->prec != p->prec) return err(QI_ERR_UNSUPPORTED, -1, -1, "plan precision differs from state");
    if ((!p->d_mats && !p->mats.empty()) || (!p->d_tc && !p->tc.empty())) {   // matrices go to the device on first use
        Status up = upload_plan(p);
        if (!up.ok()) return up;
    }
    bool has_norm = false;
    PlanRunner run(p, s);
    for (size_t i = 0; i < p->ops.size(); ++i) {
        const Op &op = p->ops[i];
        Status st = run.op(op, i + 1 < p->ops.size() ? p->ops[i + 1].kind : -1);
        if (!st.ok()) return run.finish(st);
        has_norm = has_norm || op.kind == OP_PAULI_NORM;
    }
    {
        Status st = run.finish(ok_status());
        if (!st.ok()) return st;
    }
    if (has_norm) {
        int flag = 0;
        Status st = state_read_flag(s, &flag);
        if (!st.ok()) return st;
        if (flag) return err(QI_ERR_ZERO_NORM);
    }
    return ok_status();
}

Elem pauli_exp_elem(const qi_pauli_term &t, double far, double fai, int src) {
    GateMatrix gm;
    gm.kind = QI_GATE_PAULI_EVOLUTION;
    gm.pauli = true;
    gm.xmask = t.xmask;
    gm.zmask = t.zmask;
    gm.alpha_re = t.coeff_re * far - t.coeff_im * fai;
    gm.alpha_im = t.coeff_re * fai + t.coeff_im * far;
    return make_elem_from_gate(gm, src);
}

Status sumop_expectation(qi_state *s, const qi_pauli_term *terms, int64_t nt, double out[2]);

}  // namespace qi

using namespace qi;

extern "C" {

qi_status qi_plan_create(int32_t num_qubits, int32_t precision, const qi_gate *gates, int64_t n_gates,
                         const double *theta, int64_t n_theta, const qi_exec_options *opts, qi_plan **out) {
    if (!out || (!gates && n_gates > 0)) return publish(err(QI_ERR_NULL_ARGUMENT));
    *out = nullptr;
    if (num_qubits <= 0 || num_qubits > 40) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, num_qubits));
    if (precision != QI_F32 && precision != QI_F64) return publish(err(QI_ERR_INVALID_INPUT_VALUE, precision));
    qi_plan *p = new qi_plan();
    p->n = num_qubits;
    p->prec = precision;
    if (opts) p->opts = *opts;
    std::vector<Elem> elems;
    Status st = plan_elems_from_gates(num_qubits, gates, n_gates, theta, n_theta, elems);
    if (st.ok()) st = build_plan(p, elems);
    if (!st.ok()) { delete p; return publish(st); }
    *out = p;
    return publish(ok_status());
}

qi_status qi_plan_execute(qi_plan *p, qi_state *s) {
    if (!p || !s) return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    return publish(plan_execute(p, s));
}

qi_status qi_plan_stats_get(const qi_plan *p, qi_plan_stats *out) {
    if (!p || !out) return publish(err(QI_ERR_NULL_ARGUMENT));
    *out = p->stats;
    return publish(ok_status());
}

qi_status qi_plan_profile(qi_plan *p, qi_state *s, float *ms_out) {
    if (!p || !s || !ms_out) return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    if (s->n != p->n || s->prec != p->prec) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, s->n));
    if ((!p->d_mats && !p->mats.empty()) || (!p->d_tc && !p->tc.empty())) {
        Status up = upload_plan(p);
        if (!up.ok()) return publish(up);
    }
    const size_t nops = p->ops.size();
    std::vector<cudaEvent_t> ev(nops + 1);
    for (auto &x : ev) {
        e = cudaEventCreate(&x);
        if (e != cudaSuccess) return publish(cuda_status(e, "cudaEventCreate"));
    }
    Status st = ok_status();
    PlanRunner run(p, s);
    cudaEventRecord(ev[0], s->stream);
    for (size_t i = 0; i < nops && st.ok(); ++i) {
        st = run.op(p->ops[i], i + 1 < nops ? p->ops[i + 1].kind : -1);
        cudaEventRecord(ev[i + 1], s->stream);
    }
    st = run.finish(st);
    e = cudaStreamSynchronize(s->stream);
    if (st.ok() && e != cudaSuccess) st = cuda_status(e, "profile");
    for (size_t i = 0; i < nops && st.ok(); ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        ms_out[i] = ms;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    return publish(st);
}

qi_status qi_apply_matrix(qi_state *s, const int32_t *targets, int32_t k, const double *matrix,
                          int32_t use_tensor_cores) {
    if (!s || !targets || !matrix) return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    if (k < 1 || k > 6) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, k));
    const int n = s->n;
    for (int j = 0; j < k; ++j) {
        if (targets[j] < 0 || targets[j] >= n) return publish(err(QI_ERR_INVALID_QUBIT_INDEX, targets[j], n));
        for (int i = 0; i < j; ++i)
            if (targets[i] == targets[j]) return publish(err(QI_ERR_INVALID_QUBIT_INDEX, targets[j], n));
    }
    // sort targets and permute the matrix to the sorted local order
    std::vector<int> order(k);
    for (int j = 0; j < k; ++j) order[j] = j;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return targets[x] < targets[y]; });
    const int dim = 1 << k;
    auto remap = [&](int idx) {   // sorted-local index -> caller-local index
        int o = 0;
        for (int j = 0; j < k; ++j) o |= ((idx >> j) & 1) << order[j];
        return o;
    };
    std::vector<cd> U((size_t)dim * dim);
    for (int r = 0; r < dim; ++r)
        for (int c = 0; c < dim; ++c) {
            const size_t src = (size_t)remap(r) * dim + remap(c);
            U[(size_t)r * dim + c] = cd(matrix[2 * src], matrix[2 * src + 1]);
        }
    qi_plan plan;
    plan.n = n;
    plan.prec = s->prec;
    Op op;
    op.kind = OP_FUSED;
    op.k = k;
    for (int j = 0; j < k; ++j) op.targets[j] = targets[order[j]];
    op.mat_offset = 0;
    op.mode = use_tensor_cores != 2;
    plan.mats = U;
    if (op.mode && s->prec == QI_F32 && k >= 5 && n >= k + 7) {
        op.tc_offset = 0;
        tc_blocks(k, reinterpret_cast<const double *>(U.data()), plan.tc);
    }
    if (s->prec == QI_F64 && k > 5) return publish(err(QI_ERR_UNSUPPORTED, k, -1, "FP64 blocks are limited to k <= 5"));
    plan.ops.push_back(op);
    Status st = upload_plan(&plan);
    if (st.ok()) st = plan_execute(&plan, s);
    if (st.ok()) {
        e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) st = cuda_status(e, "apply_matrix");
    }
    if (st.ok()) {
        int flag = 0;
        st = state_read_flag(s, &flag);
        if (st.ok() && flag == 2) st = err(QI_ERR_TIMEOUT, -1, -1, "tensor-core kernel wait timed out");
    }
    if (plan.d_mats) cudaFree(plan.d_mats);
    if (plan.d_tc) cudaFree(plan.d_tc);
    plan.d_mats = plan.d_tc = nullptr;
    return publish(st);
}

qi_status qi_plan_num_ops(const qi_plan *p, int64_t *out) {
    if (!p || !out) return publish(err(QI_ERR_NULL_ARGUMENT));
    *out = (int64_t)p->ops.size();
    return publish(ok_status());
}

qi_status qi_plan_op_phase_poly(const qi_plan *p, int64_t i, uint64_t *c0, uint64_t *a, uint64_t *b) {
    if (!p || !c0 || !a || !b) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (i < 0 || i >= (int64_t)p->ops.size()) return publish(err(QI_ERR_INVALID_INPUT_VALUE, i));
    const Op &op = p->ops[(size_t)i];
    const int64_t idx = op.kind == OP_PHASE_POLY ? op.mat_offset : op.kind == OP_FUSED ? op.poly_idx : -1;
    if (idx < 0 || idx >= (int64_t)p->polys.size())
        return publish(err(QI_ERR_INVALID_INPUT_VALUE, i, op.kind, "no phase polynomial on this op"));
    const PhasePoly &pp = p->polys[(size_t)idx];
    *c0 = pp.c0;
    std::copy(pp.a.begin(), pp.a.end(), a);
    std::copy(pp.b.begin(), pp.b.end(), b);
    return publish(ok_status());
}

qi_status qi_plan_op_pauli_group(const qi_plan *p, int64_t i, int32_t *n_tables, int32_t *rank, uint64_t *basis) {
    if (!p || !n_tables || !rank || !basis) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (i < 0 || i >= (int64_t)p->ops.size()) return publish(err(QI_ERR_INVALID_INPUT_VALUE, i));
    const Op &op = p->ops[(size_t)i];
    if (op.kind != OP_PAULI_GROUP) return publish(err(QI_ERR_INVALID_INPUT_VALUE, i, op.kind, "not a Pauli-group op"));
    *n_tables = op.nchunk;
    std::copy(op.rank, op.rank + kGroupChunks, rank);
    std::copy(op.basis, op.basis + kGroupChunks * kGroupRank, basis);
    return publish(ok_status());
}

qi_status qi_plan_op_bitperm(const qi_plan *p, int64_t i, int32_t *source_bit, uint64_t *flip) {
    if (!p || !source_bit || !flip) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (i < 0 || i >= (int64_t)p->ops.size()) return publish(err(QI_ERR_INVALID_INPUT_VALUE, i));
    const Op &op = p->ops[(size_t)i];
    if (op.kind != OP_BITPERM) return publish(err(QI_ERR_INVALID_INPUT_VALUE, op.kind, OP_BITPERM));
    for (int k = 0; k < p->n; ++k) source_bit[k] = op.perm[k];
    *flip = op.xmask;
    return publish(ok_status());
}

qi_status qi_plan_op_get(const qi_plan *p, int64_t i, qi_plan_op_info *info, double *matrix_out, int64_t capacity) {
    if (!p || !info) return publish(err(QI_ERR_NULL_ARGUMENT));
    if (i < 0 || i >= (int64_t)p->ops.size()) return publish(err(QI_ERR_INVALID_INPUT_VALUE, i));
    const Op &op = p->ops[(size_t)i];
    std::memset(info, 0, sizeof(*info));
    info->kind = op.kind;
    info->k = op.k;
    for (int j = 0; j < 6; ++j) info->targets[j] = op.targets[j];
    info->tensor_cores = (op.kind == OP_FUSED && op.tc_offset >= 0) ? 1 : 0;
    info->phase_poly = (op.kind == OP_FUSED && op.poly_idx >= 0) ? 1 : 0;
    info->control_mask = op.cmask;
    info->xmask = op.xmask;
    info->zmask = op.zmask;
    std::vector<double> m;
    switch (op.kind) {
    case OP_MAT1: m.assign(op.m, op.m + 8); break;
    case OP_MAT2: m.assign(op.m, op.m + 32); break;
    case OP_FUSED:
    case OP_DIAGK: {
        const size_t cnt = op.kind == OP_FUSED ? ((size_t)1 << (2 * op.k)) : ((size_t)1 << op.k);
        for (size_t j = 0; j < cnt; ++j) {
            m.push_back(p->mats[(size_t)op.mat_offset + j].real());
            m.push_back(p->mats[(size_t)op.mat_offset + j].imag());
        }
        break;
    }
    case OP_PAULI_EXP: m = {op.cre, op.cim, op.sre, op.sim}; break;
    case OP_MEASURE:   // k measured qubits (the first six in targets), basis in zmask, seed in xmask
        for (int j = 0; j < 6; ++j) info->targets[j] = j < op.k ? op.perm[j] : 0;
        info->zmask = (uint64_t)op.mode;
        if (op.mode == QI_BASIS_CUSTOM) m.assign(op.m, op.m + 8);
        break;
    case OP_PAULI_GROUP: {
        size_t cnt = 0;
        for (int c = 0; c < op.nchunk; ++c) cnt += (size_t)(op.xmask ? 4 : 1) << op.rank[c];
        for (size_t j = 0; j < cnt; ++j) {
            m.push_back(p->mats[(size_t)op.mat_offset + j].real());
            m.push_back(p->mats[(size_t)op.mat_offset + j].imag());
        }
        break;
    }
    default: break;
    }
    info->n_matrix = (int64_t)(m.size() / 2);
    if (matrix_out) {
        if (capacity < info->n_matrix) return publish(err(QI_ERR_INVALID_INPUT_VALUE, capacity, info->n_matrix));
        std::copy(m.begin(), m.end(), matrix_out);
    }
    return publish(ok_status());
}

qi_status qi_plan_destroy(qi_plan *p) {
    if (!p) return QI_OK;
    if (p->d_mats) cudaFree(p->d_mats);
    if (p->d_tc) cudaFree(p->d_tc);
    delete p;
    return QI_OK;
}

qi_status qi_circuit_execute(qi_state *s, const qi_gate *gates, int64_t n_gates, const double *theta, int64_t n_theta,
                             const qi_exec_options *opts) {
    if (!s) return publish(err(QI_ERR_NULL_ARGUMENT));
    qi_plan *p = nullptr;
    qi_status st = qi_plan_create(s->n, s->prec, gates, n_gates, theta, n_theta, opts, &p);
    if (st != QI_OK) return st;
    st = qi_plan_execute(p, s);
    if (st == QI_OK) {
        std::lock_guard<std::recursive_mutex> lk(s->mu);
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            st = publish(cuda_status(e, "execute"));
        } else {
            int flag = 0;
            Status fs = state_read_flag(s, &flag);
            if (!fs.ok()) st = publish(fs);
            else if (flag == 2) st = publish(err(QI_ERR_TIMEOUT, -1, -1, "tensor-core kernel wait timed out"));
        }
    }
    qi_plan_destroy(p);
    return st;
}

qi_status qi_trotter_evolve(qi_state *s, const qi_pauli_term *terms, int64_t n_terms, double dt, int64_t num_steps,
                            int32_t order, const qi_pauli_term *observable, int64_t n_obs, int64_t observe_every,
                            double *energies_out) {
    if (!s || (!terms && n_terms > 0)) return publish(err(QI_ERR_NULL_ARGUMENT));
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return publish(cuda_status(e, "cudaSetDevice"));
    if (n_terms == 0) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, 0));   // time_evolution.rs:51-53
    if (order != 1 && order != 2) return publish(err(QI_ERR_INVALID_INPUT_VALUE, order));
    for (int64_t k = 0; k < n_terms; ++k) {
        Status st = validate_pauli(s->n, terms[k]);
        if (!st.ok()) return publish(st);
    }
    if (observable && observe_every > 0 && !energies_out) return publish(err(QI_ERR_NULL_ARGUMENT));
    // One step as an ordered list of exponentials (time_evolution.rs:45-115).
    std::vector<Elem> elems;
    if (order == 1) {
        for (int64_t k = 0; k < n_terms; ++k) elems.push_back(pauli_exp_elem(terms[k], 0.0, -dt, (int)k));
    } else {
        for (int64_t k = 0; k < n_terms; ++k) elems.push_back(pauli_exp_elem(terms[k], 0.0, -dt / 2.0, (int)k));
        for (int64_t k = n_terms - 1; k >= 0; --k) elems.push_back(pauli_exp_elem(terms[k], 0.0, -dt / 2.0, (int)k));
    }
    // FP32: the step is one fused plan: narrow exponentials compose into dense
    // blocks (FP64 composition) and runs of Z-type exponentials into phase
    // polynomials.  With real coefficients every exponential is unitary, so the
    // plan may use the tensor-core blocks and renormalise once per step; complex
    // coefficients (a non-unitary step) keep the CUDA-core blocks and the norm.
    // FP64: FP64 arithmetic is scarce on this part (dense FP64 blocks would be
    // compute-bound), so each run of exponentials whose X-masks lie in {0, X}
    // (e.g. the XX, YY, ZZ terms of one bond, or a run of Z fields) is one pass
    // with a parity-indexed table; other terms are one pass each.
    bool unitary = true;
    for (int64_t k = 0; k < n_terms; ++k) unitary = unitary && terms[k].coeff_im == 0.0;
    qi_plan plan;
    plan.n = s->n;
    plan.prec = s->prec;
    plan.opts.fusion = s->prec == QI_F32 ? QI_FUSION_GREEDY : QI_FUSION_PAULI_GROUPS;
    plan.opts.use_tensor_cores = unitary ? 1 : 2;
    plan.opts.renorm_every = unitary ? 0 : -1;
    plan.opts.max_block_qubits = 0;
    Status st = build_plan(&plan, elems);
    if (st.ok()) st = upload_plan(&plan);
    if (!st.ok()) return publish(st);
    int64_t obs_k = 0;
    for (int64_t step = 0; step < num_steps; ++step) {
        st = plan_execute(&plan, s);
        if (!st.ok()) break;
        if (observable && observe_every > 0 && ((step + 1) % observe_every) == 0) {
            double ev[2];
            st = sumop_expectation(s, observable, n_obs, ev);
            if (!st.ok()) break;
            energies_out[2 * obs_k] = ev[0];
            energies_out[2 * obs_k + 1] = ev[1];
            ++obs_k;
        }
    }
    if (plan.d_mats) cudaFree(plan.d_mats);
    if (plan.d_tc) cudaFree(plan.d_tc);
    plan.d_tc = nullptr;
    plan.d_mats = nullptr;
    if (!st.ok()) return publish(st);
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return publish(cuda_status(e, "trotter"));
    return publish(ok_status());
}

}  // extern "C"
