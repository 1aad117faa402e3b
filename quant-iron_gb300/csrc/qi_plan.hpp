// qi_plan.hpp — plan structures shared by the planner, the cost model and
// the adjoint-gradient driver.
#pragma once
#include "qi_internal.hpp"

#include <complex>
#include <vector>

namespace qi {

// A validated gate (or Pauli exponential) as the fuser sees it.
struct Elem {
    GateMatrix gm;
    uint64_t mask = 0;      // support: targets and controls
    bool diagonal = false;
    bool fusable = false;   // may join a dense block
    bool pauli = false;
    int src = -1;           // index in the caller's gate list
};

struct Block {
    std::vector<int> members;   // element indices, in application order
    uint64_t mask = 0;          // qubits of the block
    bool single = false;        // lowered as one per-gate op
    bool perm = false;          // a run of SWAP / X gates lowered as one qubit permutation
};

std::vector<Block> greedy_partition(const std::vector<Elem> &elems, int n, int kmax);
// Greedy over candidate blocks: the light-cone block of the first remaining element
// (taken as is when it is all-diagonal), and everything each window of kmax
// consecutive qubits can absorb; the candidate with the most elements wins.
std::vector<Block> window_partition(const std::vector<Elem> &elems, int n, int kmax);
// The light-cone block of the first remaining element (at most kmax qubits), and everything the
// qubit window W can absorb from the remaining elements (order and commutation respected).
Block light_cone_block(const std::vector<Elem> &elems, const std::vector<int> &remaining, int n, int kmax);
Block window_block(const std::vector<Elem> &elems, const std::vector<int> &remaining, uint64_t W);
void compose_block(const std::vector<Elem> &elems, const Block &b, std::vector<int> &qubits,
                   std::vector<std::complex<double>> &B);

}  // namespace qi

struct qi_plan {
    int32_t n = 0;
    int32_t prec = QI_F32;
    qi_exec_options opts = {QI_FUSION_NONE, 0, 0, 0};
    std::vector<qi::Op> ops;
    std::vector<std::complex<double>> mats;   // block matrices / phase tables (host copy, FP64)
    void *d_mats = nullptr;                   // same, in the plan's precision
    std::vector<float> tc;                    // FP32 device blocks: tensor-core operands (fused ops, k >= 5)
                                              // and phase-polynomial blocks, as raw 32-bit words
    void *d_tc = nullptr;
    std::vector<qi::PhasePoly> polys;         // host copy of each OP_PHASE_POLY op (op.mat_offset indexes it)
    qi_plan_stats stats = {};
    std::vector<qi::Block> partition_override;   // set by callers that chose the partition
    bool learned_blocks = false;                 // QI_FUSION_LEARNED chose the model-scored partition
};

namespace qi {
Status build_plan(qi_plan *p, std::vector<Elem> &elems);
Status upload_plan(qi_plan *p);
Status plan_execute(qi_plan *p, qi_state *s);
Status plan_elems_from_gates(int n, const qi_gate *gates, int64_t ng, const double *theta, int64_t ntheta,
                             std::vector<Elem> &elems);
// Partition choice for QI_FUSION_GREEDY / QI_FUSION_LEARNED (qi_costmodel.cu).
std::vector<Block> choose_partition(qi_plan *p, const std::vector<Elem> &elems, int kmax);
// QI_FUSION_LEARNED: best (k, tensor cores) by the trained cost model (k = 1: one kernel per gate);
// false when no trained model is loaded.  *ms_out = predicted device time of the chosen plan.
bool learned_choice(qi_plan *p, const std::vector<Elem> &elems, int kmax, int *k_out, int *tc_out, double *ms_out);
Elem pauli_exp_elem(const qi_pauli_term &t, double far, double fai, int src);
// Plan element of one gate matrix (support, diagonal and fusable flags).
Elem make_elem_from_gate(const GateMatrix &gm, int src);
}  // namespace qi
