// qi_costmodel.cu — partition choice for the fusion pass, and the engine's
// own timing collection that trains the learned cost model (qi_mlp.cu).
//
// QI_FUSION_GREEDY uses the greedy fixed-k fuser (window_partition, qi_plan.cu).
// QI_FUSION_LEARNED scores partitions with the trained MLP in two ways and keeps the plan with the
// smallest predicted device time: (1) whole-plan candidates {one kernel per gate} and {greedy k,
// tensor cores on/off} for k = 2..kmax; (2) a partition built block by block, where each step
// scores the greedy fuser's own candidate blocks — the first remaining gate's light-cone block and
// everything each window of w consecutive qubits can absorb, for every w = 2..kmax — and takes the
// block that saves the most predicted time against running its gates one kernel each (which
// gates merge, and at what k).  Without a trained model it falls back to greedy.
#include "qi_plan.hpp"
#include "qi_mlp.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <random>

namespace qi {

// Features of the device op a block lowers to (per-gate kernel, diagonal table, dense block on
// the tensor or the CUDA cores), as build_plan lowers it.
static void block_features(int n, bool f32, bool tc, const std::vector<Elem> &elems, const Block &b, float *f) {
    if (b.single) {
        const Elem &e = elems[b.members[0]];
        int t[6] = {0, 0, 0, 0, 0, 0}, kk = 0, nc = 0, shape = CS_GENERAL;
        if (e.pauli) {
            const uint64_t m = e.gm.xmask | e.gm.zmask;
            for (int q = 0; q < 64 && kk < 6; ++q)
                if ((m >> q) & 1ull) t[kk++] = q;
            shape = e.gm.xmask ? CS_GENERAL : CS_DIAGONAL;
        } else if (e.gm.nt > 0) {
            for (int j = 0; j < e.gm.nt; ++j) t[kk++] = e.gm.t[j];
            nc = (int)e.gm.controls.size();
            const Op op = lower_gate(n, e.gm);
            shape = per_gate_shape(op.kind, op.mode);
        }
        op_features(n, f32, CC_PER_GATE, kk, t, nc, shape, f);
        return;
    }
    bool diag = true;
    for (int idx : b.members) diag = diag && elems[idx].diagonal;
    int t[6] = {0, 0, 0, 0, 0, 0}, kk = 0;
    for (int q = 0; q < 64 && kk < 6; ++q)
        if ((b.mask >> q) & 1ull) t[kk++] = q;
    int cls = CC_DENSE_SIMT;
    if (diag) cls = CC_DIAG;
    else if (tc && f32 && kk >= 5 && n >= kk + 7) cls = CC_DENSE_TC;
    op_features(n, f32, cls, kk, t, 0, diag ? CS_DIAGONAL : CS_GENERAL, f);
}

// Predicted ms of each feature row (caller holds the model's mutex).
static bool predict_ms(Mlp &m, int n, const std::vector<float> &F, std::vector<double> &ms) {
    const int rows = (int)(F.size() / kFeat);
    ms.assign((size_t)rows, 0.0);
    if (rows == 0) return true;
    std::vector<float> y((size_t)rows);
    Status s = m.ensure_device(rows);
    if (s.ok()) s = m.upload_params(nullptr);
    if (s.ok()) s = m.predict(F.data(), rows, y.data(), nullptr);
    if (!s.ok()) return false;
    for (int i = 0; i < rows; ++i) ms[(size_t)i] = ms_from_y(y[(size_t)i], n);
    return true;
}

// The model-scored partition (see the file comment); empty on failure.  Caller holds m.mu.
static std::vector<Block> learned_partition_locked(Mlp &m, int n, bool f32, bool tc, const std::vector<Elem> &elems,
                                                   int kmax, double *pred_ms) {
    std::vector<Block> blocks;
    // every gate as its own kernel: the baseline a block's saving is measured against
    std::vector<float> F((size_t)elems.size() * kFeat);
    for (size_t i = 0; i < elems.size(); ++i) {
        Block one;
        one.members.push_back((int)i);
        one.mask = elems[i].mask;
        one.single = true;
        block_features(n, f32, tc, elems, one, F.data() + i * kFeat);
    }
    std::vector<double> t_gate;
    if (!predict_ms(m, n, F, t_gate)) return {};
    std::vector<int> remaining(elems.size());
    for (size_t i = 0; i < elems.size(); ++i) remaining[i] = (int)i;
    std::vector<char> taken(elems.size(), 0);
    double total = 0.0;
    std::vector<Block> cands;
    std::vector<double> t_cand;
    while (!remaining.empty()) {
        cands.clear();
        Block lc = light_cone_block(elems, remaining, n, kmax);
        bool diag = !lc.single;
        for (int idx : lc.members) diag = diag && elems[idx].diagonal;
        const bool alone = lc.single || diag;   // a lone gate, or a diagonal block for a phase-polynomial run
        cands.push_back(std::move(lc));
        if (!alone) {
            for (int w = 2; w <= kmax; ++w) {
                const uint64_t win = (1ull << w) - 1;
                for (int a = 0; a + w <= n; ++a) {
                    Block b = window_block(elems, remaining, win << a);
                    if (b.members.size() >= 2) cands.push_back(std::move(b));
                }
            }
        }
        size_t best = 0;
        if (cands.size() > 1) {
            F.assign(cands.size() * kFeat, 0.0f);
            for (size_t c = 0; c < cands.size(); ++c) block_features(n, f32, tc, elems, cands[c], F.data() + c * kFeat);
            if (!predict_ms(m, n, F, t_cand)) return {};
            double best_save = -1e300;
            for (size_t c = 0; c < cands.size(); ++c) {
                double per_gate = 0.0;
                for (int idx : cands[c].members) per_gate += t_gate[(size_t)idx];
                const double save = per_gate - t_cand[c];
                if (save > best_save || (save == best_save && cands[c].members.size() > cands[best].members.size())) {
                    best_save = save;
                    best = c;
                }
            }
            total += t_cand[best];
        } else {
            double per_gate = 0.0;
            for (int idx : cands[0].members) per_gate += t_gate[(size_t)idx];
            total += cands[0].single ? per_gate : per_gate * 0.25;   // diagonal runs share one pass
        }
        Block b = std::move(cands[best]);
        for (int idx : b.members) taken[(size_t)idx] = 1;
        std::vector<int> rest;
        rest.reserve(remaining.size());
        for (int idx : remaining)
            if (!taken[(size_t)idx]) rest.push_back(idx);
        remaining.swap(rest);
        blocks.push_back(std::move(b));
    }
    if (pred_ms) *pred_ms = total;
    return blocks;
}

std::vector<Block> choose_partition(qi_plan *p, const std::vector<Elem> &elems, int kmax) {
    if (p->learned_blocks) {
        Mlp &m = global_mlp();
        std::lock_guard<std::mutex> lk(m.mu);
        if (m.trained) {
            std::vector<Block> b = learned_partition_locked(m, p->n, p->prec == QI_F32,
                                                            p->opts.use_tensor_cores != 2, elems, kmax, nullptr);
            if (!b.empty() || elems.empty()) return b;
        }
    }
    return window_partition(elems, p->n, kmax);
}

// Features of the device ops one candidate produces.
static void candidate_features(int n, bool f32, const std::vector<Elem> &elems, int k, bool tc, std::vector<float> &F,
                               int *n_norm) {
    float f[kFeat];
    auto add_single = [&](const Elem &e) {
        int t[6] = {0, 0, 0, 0, 0, 0}, kk = 0, nc = 0, shape = CS_GENERAL;
        if (e.pauli) {
            const uint64_t m = e.gm.xmask | e.gm.zmask;
            for (int q = 0; q < 64 && kk < 6; ++q)
                if ((m >> q) & 1ull) t[kk++] = q;
            shape = e.gm.xmask ? CS_GENERAL : CS_DIAGONAL;
        } else {
            if (e.gm.nt == 0) return;   // identity: no kernel
            for (int j = 0; j < e.gm.nt; ++j) t[kk++] = e.gm.t[j];
            nc = (int)e.gm.controls.size();
            const Op op = lower_gate(n, e.gm);
            shape = per_gate_shape(op.kind, op.mode);
        }
        op_features(n, f32, CC_PER_GATE, kk, t, nc, shape, f);
        F.insert(F.end(), f, f + kFeat);
    };
    *n_norm = 0;
    if (k <= 1) {
        for (const Elem &e : elems) add_single(e);
        return;
    }
    std::vector<Block> blocks = window_partition(elems, n, k);
    bool used_tc = false;
    for (const Block &b : blocks) {
        if (b.single) { add_single(elems[b.members[0]]); continue; }
        bool diag = true;
        for (int idx : b.members) diag = diag && elems[idx].diagonal;
        int t[6] = {0, 0, 0, 0, 0, 0}, kk = 0;
        for (int q = 0; q < 64 && kk < 6; ++q)
            if ((b.mask >> q) & 1ull) t[kk++] = q;
        int cls = CC_DENSE_SIMT;
        if (diag) cls = CC_DIAG;
        else if (tc && f32 && kk >= 5 && n >= kk + 7) { cls = CC_DENSE_TC; used_tc = true; }
        op_features(n, f32, cls, kk, t, 0, diag ? CS_DIAGONAL : CS_GENERAL, f);
        F.insert(F.end(), f, f + kFeat);
    }
    if (used_tc) *n_norm = 1;
}

// Kernels a block list lowers to (the rules of build_plan, qi_plan.cu): one per single, permutation
// and dense block; a run of diagonal blocks is one phase-polynomial pass (two or more blocks, or one
// of three or more qubits; otherwise the block's own pass), none when it follows a tensor-core block
// of an FP32 plan, whose epilogue applies it (dense blocks of 3 or 4 qubits are widened to 5-qubit
// tensor-core blocks from 12 qubits up).
static int64_t lowered_kernels(const std::vector<Block> &blocks, const std::vector<Elem> &elems, int n, bool f32,
                               bool tc) {
    int64_t kern = 0;
    bool prev_tc = false;
    int run = 0, run_k = 0;
    auto end_run = [&]() {
        if (run >= 2 || (run == 1 && run_k >= 3)) kern += (f32 && prev_tc) ? 0 : 1;
        else if (run == 1) kern += 1;
        run = run_k = 0;
    };
    for (const Block &b : blocks) {
        bool diag = !b.single && !b.perm;
        for (int idx : b.members) diag = diag && elems[(size_t)idx].diagonal;
        const int k = __builtin_popcountll(b.mask);
        if (diag && f32) {
            ++run;
            run_k = std::max(run_k, k);
            continue;
        }
        end_run();
        ++kern;
        const int kt = (k == 3 || k == 4) && n >= 12 ? 5 : k;   // the width it runs at
        prev_tc = !b.single && !b.perm && !diag && tc && f32 && kt >= 5 && n >= kt + 7;
    }
    end_run();
    return kern;
}

bool learned_choice(qi_plan *p, const std::vector<Elem> &elems, int kmax, int *k_out, int *tc_out, double *ms_out) {
    Mlp &m = global_mlp();
    std::lock_guard<std::mutex> lk(m.mu);
    if (!m.trained || elems.empty()) return false;
    const int n = p->n;
    const bool f32 = p->prec == QI_F32;
    struct Cand { int k, tc, first, count, nnorm; };
    std::vector<Cand> cands;
    std::vector<float> F;
    for (int k = 1; k <= kmax; ++k) {
        for (int tc = 0; tc <= ((f32 && k >= 5) ? 1 : 0); ++tc) {
            Cand c;
            c.k = k;
            c.tc = tc;
            c.first = (int)(F.size() / kFeat);
            candidate_features(n, f32, elems, k, tc != 0, F, &c.nnorm);
            c.count = (int)(F.size() / kFeat) - c.first;
            cands.push_back(c);
        }
    }
    // one extra row: a diagonal k=1 op stands in for a pass of the renormalisation
    float f[kFeat];
    const int t0[6] = {0, 0, 0, 0, 0, 0};
    op_features(n, f32, CC_DIAG, 1, t0, 0, CS_DIAGONAL, f);
    const int norm_row = (int)(F.size() / kFeat);
    F.insert(F.end(), f, f + kFeat);
    const int rows = (int)(F.size() / kFeat);
    std::vector<float> y((size_t)rows);
    Status s = m.ensure_device(rows);
    if (s.ok()) s = m.upload_params(nullptr);
    if (s.ok()) s = m.predict(F.data(), rows, y.data(), nullptr);
    if (!s.ok()) return false;
    double best = 1e300;
    int bk = kmax, btc = 1;
    for (const Cand &c : cands) {
        double ms = 0.0;
        for (int i = 0; i < c.count; ++i) ms += ms_from_y(y[(size_t)(c.first + i)], n);
        ms += c.nnorm * 1.5 * ms_from_y(y[(size_t)norm_row], n);
        if (ms < best) { best = ms; bk = c.k; btc = c.tc; }
    }
    // the block-by-block partition at kmax, tensor cores as the caller allows
    p->learned_blocks = false;
    const bool tc_ok = p->opts.use_tensor_cores != 2;
    double lp_ms = 0.0;
    const std::vector<Block> lp = learned_partition_locked(m, n, f32, tc_ok, elems, kmax, &lp_ms);
    // Every kernel is one pass over the state, so a partition that lowers to more kernels than the
    // greedy one at the same k is not taken on the model's word alone: over 21 seeded circuits of
    // 28-34 qubits, each learned plan with more kernels than greedy's ran 2-5 % slower.
    if (!lp.empty() &&
        lowered_kernels(lp, elems, n, f32, tc_ok) <= lowered_kernels(window_partition(elems, n, kmax), elems, n, f32, tc_ok)) {
        bool any_tc = false;
        for (const Block &b : lp) {
            if (b.single) continue;
            bool diag = true;
            for (int idx : b.members) diag = diag && elems[idx].diagonal;
            const int w = __builtin_popcountll(b.mask);
            any_tc = any_tc || (!diag && tc_ok && f32 && w >= 5 && n >= w + 7);
        }
        lp_ms += (any_tc ? 1.5 : 0.0) * ms_from_y(y[(size_t)norm_row], n);
        if (lp_ms < best) {
            best = lp_ms;
            bk = kmax;
            btc = tc_ok ? 1 : 0;
            p->learned_blocks = true;
        }
    }
    *k_out = bk;
    *tc_out = btc;
    *ms_out = best;
    return true;
}

}  // namespace qi

using namespace qi;

// Time `count` random device ops on n-qubit states with CUDA events, as the
// training data of the cost model.  Op mix: dense blocks (CUDA cores, k 1..6;
// tensor cores, k 5..6, FP32), diagonal blocks (k 1..6) and per-gate kernels
// (2x2 in every mode with 0..2 controls, SWAP, 4x4), FP32 and FP64 states.
extern "C" qi_status qi_costmodel_collect(int32_t num_qubits, int64_t count, uint64_t seed, float *features_out,
                                          float *log_ms_out) {
    if (!features_out || !log_ms_out || count <= 0) return publish(err(QI_ERR_NULL_ARGUMENT));
    const int n = num_qubits;
    if (n < 14 || n > 34) return publish(err(QI_ERR_INVALID_NUMBER_OF_QUBITS, n));
    qi_state *s32 = nullptr, *s64 = nullptr;
    qi_status cs = qi_state_create(n, QI_F32, &s32);
    if (cs != QI_OK) return cs;
    cs = qi_state_create(n, QI_F64, &s64);
    if (cs != QI_OK) { qi_state_destroy(s32); return cs; }
    qi_state_set_plus(s32);
    qi_state_set_plus(s64);
    void *d_mat = nullptr, *d_tc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Status st = ok_status();
    cudaError_t ce = cudaMalloc(&d_mat, 64 * 64 * sizeof(double2));
    if (ce == cudaSuccess) ce = cudaMalloc(&d_tc, 6 * 64 * 64 * sizeof(float));
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) st = cuda_status(ce, "costmodel collect");
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    const int warm = 24;
    for (int64_t i = -warm; i < count && st.ok(); ++i) {
        const bool f32 = (rng() % 4) != 0;
        qi_state *s = f32 ? s32 : s64;
        int cls = (int)(rng() % 4);
        if (cls == CC_DENSE_TC && !f32) cls = CC_DENSE_SIMT;
        int k;
        if (cls == CC_DENSE_TC) k = 5 + (int)(rng() % 2);
        else if (cls == CC_PER_GATE) k = 1 + (int)(rng() % 2);
        else k = 1 + (int)(rng() % (f32 ? 6 : 5));
        // random distinct sorted targets
        int t[6];
        {
            std::vector<int> pool(n);
            for (int q = 0; q < n; ++q) pool[q] = q;
            std::shuffle(pool.begin(), pool.end(), rng);
            std::sort(pool.begin(), pool.begin() + k);
            for (int j = 0; j < k; ++j) t[j] = pool[j];
        }
        Op op;
        op.k = k;
        for (int j = 0; j < k; ++j) op.targets[j] = t[j];
        int ncontrols = 0;
        const int dim = 1 << k;
        std::vector<double> M((size_t)2 * dim * dim);
        for (auto &x : M) x = U(rng) / dim;
        if (cls == CC_PER_GATE) {
            // controls outside the targets
            ncontrols = (int)(rng() % 3);
            uint64_t cm = 0;
            int placed = 0;
            while (placed < ncontrols) {
                const int q = (int)(rng() % n);
                bool clash = false;
                for (int j = 0; j < k; ++j) clash = clash || t[j] == q;
                if (clash || ((cm >> q) & 1ull)) continue;
                cm |= 1ull << q;
                ++placed;
            }
            op.cmask = cm;
            if (k == 1) {
                op.kind = OP_MAT1;
                op.mode = (int)(rng() % 5);
                for (int j = 0; j < 8; ++j) op.m[j] = M[j];
                if (op.mode == M1_PHASE1) { op.m[0] = 1; op.m[1] = 0; op.m[2] = op.m[3] = op.m[4] = op.m[5] = 0; }
                if (op.mode == M1_DIAG) { op.m[2] = op.m[3] = op.m[4] = op.m[5] = 0; }
                if (op.mode == M1_ANTIDIAG) { op.m[0] = op.m[1] = op.m[6] = op.m[7] = 0; }
                if (op.mode == M1_REAL) { op.m[1] = op.m[3] = op.m[5] = op.m[7] = 0; }
            } else {
                op.kind = (rng() % 2) ? OP_SWAP : OP_MAT2;
                for (int j = 0; j < 32; ++j) op.m[j] = M[j];
            }
        } else if (cls == CC_DIAG) {
            op.kind = OP_DIAGK;
            op.mat_offset = 0;
            std::vector<double> ph((size_t)2 * dim);
            for (auto &x : ph) x = U(rng);
            if (f32) {
                std::vector<float2> hf((size_t)dim);
                for (int r = 0; r < dim; ++r) hf[r] = make_float2((float)ph[2 * r], (float)ph[2 * r + 1]);
                ce = cudaMemcpy(d_mat, hf.data(), dim * sizeof(float2), cudaMemcpyHostToDevice);
            } else {
                ce = cudaMemcpy(d_mat, ph.data(), dim * sizeof(double2), cudaMemcpyHostToDevice);
            }
        } else {
            op.kind = OP_FUSED;
            op.mat_offset = 0;
            op.mode = cls == CC_DENSE_TC ? 1 : 0;
            if (f32) {
                std::vector<float2> hf((size_t)dim * dim);
                for (size_t r = 0; r < hf.size(); ++r) hf[r] = make_float2((float)M[2 * r], (float)M[2 * r + 1]);
                ce = cudaMemcpy(d_mat, hf.data(), hf.size() * sizeof(float2), cudaMemcpyHostToDevice);
            } else {
                ce = cudaMemcpy(d_mat, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice);
            }
            if (cls == CC_DENSE_TC && ce == cudaSuccess) {
                if (n < k + 7) { op.mode = 0; cls = CC_DENSE_SIMT; }
                else {
                    std::vector<float> blocks;
                    tc_blocks(k, M.data(), blocks);
                    ce = cudaMemcpy(d_tc, blocks.data(), blocks.size() * sizeof(float), cudaMemcpyHostToDevice);
                    op.tc_offset = 0;
                }
            }
        }
        if (ce != cudaSuccess) { st = cuda_status(ce, "costmodel collect"); break; }
        cudaEventRecord(e0, s->stream);
        st = launch_op(s, op, d_mat, op.tc_offset >= 0 ? d_tc : nullptr);
        cudaEventRecord(e1, s->stream);
        if (!st.ok()) break;
        ce = cudaEventSynchronize(e1);
        if (ce != cudaSuccess) { st = cuda_status(ce, "costmodel collect"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (i >= 0) {
            const int shape = cls == CC_PER_GATE ? per_gate_shape(op.kind, op.mode)
                                                 : (cls == CC_DIAG ? CS_DIAGONAL : CS_GENERAL);
            op_features(n, f32, cls, k, t, ncontrols, shape, features_out + (size_t)i * kFeat);
            log_ms_out[i] = y_from_ms((double)ms, n);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (d_mat) cudaFree(d_mat);
    if (d_tc) cudaFree(d_tc);
    qi_state_destroy(s32);
    qi_state_destroy(s64);
    return publish(st);
}
