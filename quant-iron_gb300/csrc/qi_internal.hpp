// qi_internal.hpp — declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <complex>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qi_engine.h"

namespace qi {

// ---------------------------------------------------------------- errors --
struct Status {
    qi_status code = QI_OK;
    int64_t a = -1, b = -1;
    double re = 0.0, im = 0.0;
    std::string msg;
    bool ok() const { return code == QI_OK; }
};
inline Status ok_status() { return Status{}; }
inline Status err(qi_status c, int64_t a = -1, int64_t b = -1, std::string m = std::string()) {
    Status s;
    s.code = c; s.a = a; s.b = b; s.msg = std::move(m);
    return s;
}
// Record `s` as the calling thread's last error and return its code.
qi_status publish(const Status &s);
Status cuda_status(cudaError_t e, const char *what);

#define QI_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t qi_e_ = (call);                                     \
        if (qi_e_ != cudaSuccess) return ::qi::cuda_status(qi_e_, #call); \
    } while (0)

// Counts every kernel launch made by the engine (reported by the benchmark).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }
Status check_launch(const char *what);

// ----------------------------------------------------------------- state --
constexpr int kReduceBlocks = 1216;  // 152 SMs x 8: partial-sum slots per reduction
constexpr int kReduceThreads = 256;

}  // namespace qi

// Device-resident state vector handle (the opaque qi_state of the C ABI).
struct qi_state {
    int32_t n = 0;
    int32_t prec = QI_F64;
    int32_t device = 0;
    void *amps = nullptr;             // 2^n complex amplitudes (double2 or float2)
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;    // stream all work of this handle is issued on
    std::recursive_mutex mu;          // serialises calls on this handle
    double *d_partials = nullptr;     // reduction scratch: kReduceBlocks x 4 doubles
    double *d_result = nullptr;       // finalised reduction results (8 doubles)
    double *h_result = nullptr;       // pinned mirror of d_result
    void *d_staging = nullptr;        // host<->device conversion staging (lazy)
    size_t staging_bytes = 0;
    int *d_flag = nullptr;            // device-side error flag (ZeroNorm inside async sequences)
    void *d_scratch = nullptr;        // second state buffer for out-of-place permutations (lazy)
    cudaStream_t link_stream = nullptr;   // lowest-priority stream of uploads the GPU reads over the link (lazy)
    cudaEvent_t link_ev[2] = {nullptr, nullptr};   // orders it after, and before, this handle's stream

    uint64_t dim() const { return 1ull << n; }
    size_t amp_bytes() const { return prec == QI_F64 ? 16 : 8; }
    size_t bytes() const { return dim() * amp_bytes(); }
};

namespace qi {

// --------------------------------------------------------- state helpers --
Status state_reduce_norm_sqr(qi_state *s, double *out);                       // sync
Status state_inner(qi_state *a, qi_state *b, double out[2]);                  // sync
Status state_scale_async(qi_state *s, double re, double im);
Status state_normalise_device_async(qi_state *s);   // norm on device, divides if != 0 and != 1; flags ZeroNorm
Status state_read_flag(qi_state *s, int *flag);      // sync; resets the flag
Status state_copy_async(qi_state *dst, const qi_state *src);

// ----------------------------------------------------------------- gates --
// A gate lowered to one primitive device operation.
enum OpKind : int32_t {
    OP_NOP = 0,
    OP_MAT1 = 1,    // 2x2 on one target, controlled
    OP_SWAP = 2,    // swap |..1..0..> <-> |..0..1..> on (t0, t1), controlled
    OP_MAT2 = 3,    // 4x4 on (t0 < t1), controlled
    OP_FUSED = 4,   // dense 2^k x 2^k on k targets (fused block)
    OP_PAULI_EXP = 5,     // cosh(a) psi + sinh(a) P psi
    OP_PAULI_NORM = 6,    // P psi then normalise (Gate::PauliString)
    OP_DIAGK = 7,         // diagonal on k targets (2^k phases), controlled by nothing
    OP_NORMALISE = 8,     // FP64 norm on the device, divide (periodic renormalisation)
    OP_PHASE_POLY = 9,    // run of diagonal blocks as one quadratic phase polynomial over all qubits (FP32)
    OP_PAULI_GROUP = 10,  // run of Pauli exponentials with X-masks in {0, X}: parity-indexed table, one pass
    OP_BITPERM = 11,      // run of SWAP / X gates as one qubit permutation: out[j] = in[s(j)] (tiled transpose)
    OP_MEASURE = 12,      // Gate::Measurement: outcome probabilities, seeded draw, collapse (host-synchronising)
};
// OP_PAULI_GROUP limits: diagonal runs use up to kGroupChunks tables of up to
// 2^kGroupRank factors; pair runs one table of up to 2^kPairRank 2x2 matrices.
constexpr int kGroupChunks = 4, kGroupRank = 8, kPairRank = 6;
enum Mat1Mode : int32_t { M1_GENERAL = 0, M1_DIAG = 1, M1_ANTIDIAG = 2, M1_PHASE1 = 3, M1_REAL = 4 };

struct Op {
    int32_t kind = OP_NOP;
    int32_t mode = 0;
    int32_t k = 0;                 // number of targets
    int32_t targets[6] = {0, 0, 0, 0, 0, 0};
    uint64_t cmask = 0;            // control mask (controls must be 1)
    double m[32] = {0};            // MAT1: 4 complex; MAT2: 16 complex (row-major re, im)
    int64_t mat_offset = -1;       // OP_FUSED / OP_DIAGK: offset (complex entries) into the plan's matrix buffer
    int64_t tc_offset = -1;        // OP_FUSED: offset (floats) of the tensor-core operand blocks, -1 if none
    uint64_t xmask = 0, zmask = 0; // Pauli ops
    double alpha_re = 0, alpha_im = 0;   // Pauli exp: cosh/sinh coefficients are derived from this
    double cre = 0, cim = 0, sre = 0, sim = 0;
    // OP_FUSED on the tensor cores: a phase polynomial applied after the block in the same pass
    // (its device block at tc offset poly_tc, its host copy plan->polys[poly_idx]), or -1
    int64_t poly_tc = -1, poly_idx = -1;
    // OP_PAULI_GROUP: table c is indexed by the parities popc(i & basis[c * kGroupRank + j]) & 1,
    // j < rank[c] (pair groups: i = the partner with the highest bit of xmask clear)
    int32_t nchunk = 0;
    int32_t rank[kGroupChunks] = {0, 0, 0, 0};
    uint64_t basis[kGroupChunks * kGroupRank] = {0};
    // OP_BITPERM: s(j) = xmask ^ sum_k bit k of j << perm[k] (the source of output index j)
    int8_t perm[64] = {0};
};

// Host-side description of a gate after validation: 2x2 / 4x4 matrix on its
// targets plus controls.  Used by both the per-gate lowering and the fuser.
struct GateMatrix {
    int32_t kind = -1;             // qi_gate_kind
    int32_t nt = 0;                // 0 = identity (no-op), 1 or 2 targets
    int32_t t[2] = {0, 0};         // targets (for nt == 2: t[0] < t[1] after normalisation)
    std::vector<int32_t> controls; // deduplicated
    double m[32];                  // row-major complex (re, im) 2^nt x 2^nt
    bool diagonal = false;
    bool pauli = false;            // Gate::PauliString / PauliTimeEvolution (not fusable as a matrix)
    bool normalise_after = false;
    uint64_t xmask = 0, zmask = 0;
    double alpha_re = 0, alpha_im = 0;
    // Gate::Measurement: basis (QI_BASIS_*), measured qubits in outcome-bit order, seed of the
    // draw (xmask of the gate); m[0..7] = the custom basis matrix
    bool measure = false;
    int32_t basis = 0;
    uint64_t seed = 0;
    std::vector<int32_t> measured;
};

// GF(2)-affine index map of a run of X / CNOT / SWAP gates (qi_permute.cu):
// bit k of f(j) = parity(row[k] & j) ^ bit k of b.
constexpr int kAffineMaxBytes = 5;   // index bytes (states up to 40 qubits)
struct AffineMap {
    uint64_t row[64];
    uint64_t b;
};
bool affine_gate(const GateMatrix &gm);   // X / CNOT with at most one control, or uncontrolled SWAP
void affine_identity(AffineMap &m);
void affine_compose(AffineMap &m, const GateMatrix &gm);   // m := gate o m
// out[j] = in[f(j)] for every amplitude j of s's size and precision (out != in), on s's stream.
Status affine_gather_async(qi_state *s, void *out, const void *in, const AffineMap &m);
// Qubit permutation (tiled through shared memory, coalesced on both sides):
// out[j] = in[flip ^ sum_k bit k of j << perm[k]], out != in.
// norm_nb != nullptr: also the norm partials of the permuted state in s->d_partials (*norm_nb rows)
Status bitperm_async(qi_state *s, void *out, const void *in, const int8_t *perm, uint64_t flip,
                     unsigned *norm_nb = nullptr);
// The same permutation in place, as one SWAP per transposition of perm's cycles and one X per
// flipped bit (used when no second state buffer can be allocated).
Status bitperm_in_place_async(qi_state *s, const int8_t *perm, uint64_t flip);
// The state's second buffer (allocated on first use, freed with the state).
Status state_scratch(qi_state *s, void **out);
// Divide in by its FP64 norm into out (out != in; a norm of 0 or 1 copies unchanged, 0 flags ZeroNorm).
Status state_normalise_device_to_async(qi_state *s, void *out, const void *in);
// the same with the norm partials of `in` already in s->d_partials (nb rows)
Status state_normalise_to_from_partials_async(qi_state *s, void *out, const void *in, unsigned nb);

Status validate_gate(int n, const qi_gate &g);
// State::measure (state.rs:525-730) on s (caller holds s's mutex): basis change, FP64 outcome
// probabilities, draw r = uniform01(seed), collapse + renormalise, basis change back.
Status measure_state(qi_state *s, int basis, const double *custom_u, const int32_t *qubits, int m, uint64_t seed,
                     uint64_t *outcome_out, double *probs_out);
// Validate + build the matrix of a (resolved) gate.
Status gate_to_matrix(int n, const qi_gate &g, GateMatrix *out);
// Lower a GateMatrix to a single primitive op.
Op lower_gate(int n, const GateMatrix &gm);
// Launch one primitive op on the state's stream (no synchronisation).
Status launch_op(qi_state *s, const Op &op, const void *d_mats, const void *d_tc = nullptr);

// ------------------------------------------------------------------ pauli --
Status launch_pauli_exp(qi_state *s, uint64_t xmask, uint64_t zmask, double cre, double cim, double sre, double sim);
Status launch_pauli_apply(qi_state *out, qi_state *in, uint64_t xmask, uint64_t zmask, double cre, double cim);
Status validate_pauli(int n, const qi_pauli_term &t);
// Group the Pauli exponentials run[start..] (exp(alpha P) each) into one
// OP_PAULI_GROUP op, its tables appended to `mats`.  Returns how many terms
// the op covers; 1 means no group formed (op untouched; lower the term alone).
size_t pauli_group_op(const std::vector<const GateMatrix *> &run, size_t start, Op &op,
                      std::vector<std::complex<double>> &mats);
Status launch_pauli_group(qi_state *s, const Op &op, const void *d_mats);

// ------------------------------------------------------------------ fused --
// Apply a dense 2^k x 2^k complex matrix (device pointer, row-major, element
// type matches the state's precision) on sorted targets.
Status launch_fused(qi_state *s, int k, const int32_t *targets, const void *d_mat, const void *d_tc, int use_tc,
                    const void *poly = nullptr);
// 3xTF32 tcgen05 kernel (FP32 states, k = 5 or 6, n >= k + 7); d_tc holds the
// six operand blocks prepared by tc_blocks().
// poly: device block of a phase polynomial applied after the block in the same pass (or null)
Status launch_fused_tc(qi_state *s, int k, const int32_t *targets, const void *d_tc, const void *poly = nullptr);
// Host: the six K-major operand blocks {-Im U, Re U, Im U} x {tf32 hi, lo}
// (each 2^k x 2^k floats in the no-swizzle core-matrix layout) of a fused
// matrix U (row-major complex, FP64).  Appends 6 * 4^k floats to `out`.
void tc_blocks(int k, const double *U, std::vector<float> &out);
Status launch_diagk(qi_state *s, int k, const int32_t *targets, const void *d_phases);

// ------------------------------------------------------------ phase poly --
// A diagonal operator exp(2 pi i f(x)) with f a polynomial of degree <= 2 in
// the amplitude-index bits x_q: f = c0 + sum_q a[q] x_q + sum_{q<r} b[q][r] x_q x_r.
// Coefficients are fixed-point turns (2^64 = one turn), so sums wrap mod 2 pi exactly.
struct PhasePoly {
    int n = 0;
    uint64_t c0 = 0;
    std::vector<uint64_t> a;   // n
    std::vector<uint64_t> b;   // n * n, b[q * n + r] for q < r
    void init(int nq) {
        n = nq;
        c0 = 0;
        a.assign((size_t)nq, 0);
        b.assign((size_t)nq * nq, 0);
    }
};
// Add the phase polynomial of a diagonal table over `qubits` (phases[x], bit j
// of x <-> qubits[j]) to pp.  False (pp unchanged) if an entry is not of unit
// modulus or the table has terms of degree > 2.
bool phase_poly_add_table(PhasePoly &pp, int k, const int32_t *qubits, const std::complex<double> *phases);
// Iteration bits h of the phase-polynomial kernel for n qubits (FP32 states).
int phase_poly_iter_bits(int n);
// Device block of pp (32-bit words) appended to `out`, padded to 16 bytes.
// Device block of a phase polynomial (32-bit words): a[q] at kPolyA, b[q][r] (symmetric,
// 64 x 64) at kPolyB, the exp table T1 (1024 x float2) at kPolyT1, c0 + iteration tables at kPolyG0.
constexpr int kPolyA = 0, kPolyB = 64, kPolyT1 = 64 + 64 * 64, kPolyG0 = kPolyT1 + 2 * 1024;
void phase_poly_device_block(const PhasePoly &pp, std::vector<float> &out);
// The phase table a tensor-core block on `targets` (sorted) uses to apply pp after the block in
// its epilogue (qi_fused_tc.cu); false (nothing appended) when the state has too many tiles.
bool tc_phase_table(const PhasePoly &pp, int k, const int32_t *targets, std::vector<float> &out);
Status launch_phase_poly(qi_state *s, const void *d_block);

}  // namespace qi
