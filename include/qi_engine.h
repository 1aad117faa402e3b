/*
 * qi_engine.h — C ABI of the GB300 state-vector engine for quant-iron.
 *
 * This is the drop-in boundary.  Every entry point takes plain pointers and
 * sizes and returns a qi_status.  The Rust side of quant-iron binds these in an
 * `extern "C"` block next to its build.rs; each function names the reference
 * item it replaces as `file:line` within the quant-iron crate (src/...).
 *
 * Conventions shared by all calls
 *  - Amplitude index bit q is qubit q (little-endian), as in
 *    src/components/operator.rs:347-349.
 *  - Host amplitude buffers are interleaved (re, im) f64 pairs, the memory
 *    layout of `Vec<Complex<f64>>` (src/components/state.rs:77).
 *  - Device states are resident in HBM in complex FP64 (double2) or complex
 *    FP32 (float2), chosen at creation.
 *  - Errors: 0 is success; negative codes map 1:1 onto the variants of
 *    `quant_iron::errors::Error` (src/errors.rs:4-97).  The offending values
 *    (the tuple fields of the variant) are kept per thread and read back with
 *    qi_last_error().
 *  - Calls on one state handle are serialised by a mutex held in the handle
 *    (replacing the global GPU_CONTEXT mutex, src/components/gpu_context.rs:166-168);
 *    calls on different handles may run from different threads.
 */
#ifndef QI_ENGINE_H
#define QI_ENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes (src/errors.rs:4-97)                                          */
/* ------------------------------------------------------------------------ */
typedef int32_t qi_status;

#define QI_OK                                   0
#define QI_ERR_INVALID_NUMBER_OF_MEASUREMENTS  (-1)  /* Error::InvalidNumberOfMeasurements(a)        errors.rs:11 */
#define QI_ERR_OVERLAPPING_CONTROL_AND_TARGET  (-2)  /* Error::OverlappingControlAndTargetQubits(a,b) errors.rs:21 */
#define QI_ERR_INVALID_NUMBER_OF_QUBITS        (-3)  /* Error::InvalidNumberOfQubits(a)               errors.rs:29 */
#define QI_ERR_INVALID_QUBIT_INDEX             (-4)  /* Error::InvalidQubitIndex(a,b)                 errors.rs:38 */
#define QI_ERR_STATE_NOT_NORMALISED            (-5)  /* Error::StateVectorNotNormalised               errors.rs:42 */
#define QI_ERR_NON_UNITARY_MATRIX              (-6)  /* Error::NonUnitaryMatrix                       errors.rs:46 */
#define QI_ERR_INVALID_NUMBER_OF_INPUTS        (-7)  /* Error::InvalidNumberOfInputs(a,b)             errors.rs:56 */
#define QI_ERR_MISMATCHED_NUMBER_OF_PARAMETERS (-8)  /* Error::MismatchedNumberOfParameters{a,b}      errors.rs:66 */
#define QI_ERR_UNKNOWN                         (-9)  /* Error::UnknownError                           errors.rs:70 */
#define QI_ERR_DEVICE                          (-10) /* Error::OpenCLError(String): CUDA runtime error errors.rs:78 */
#define QI_ERR_CONTEXT_LOCK                    (-11) /* Error::GpuContextLockError                    errors.rs:82 */
#define QI_ERR_CIRCUIT_MACRO                   (-12) /* Error::CircuitMacroError(String)              errors.rs:86 */
#define QI_ERR_INVALID_INPUT_VALUE             (-13) /* Error::InvalidInputValue(a)                   errors.rs:90 */
#define QI_ERR_ZERO_NORM                       (-14) /* Error::ZeroNorm                               errors.rs:94 */
#define QI_ERR_INVALID_PAULI_COEFFICIENT       (-15) /* Error::InvalidPauliStringCoefficient(re,im)   errors.rs:97 */
/* Codes without a reference variant (the Rust shim maps them onto OpenCLError(String)). */
#define QI_ERR_OUT_OF_MEMORY                   (-16) /* device allocation failed */
#define QI_ERR_TIMEOUT                         (-17) /* a bounded device-side wait ran out */
#define QI_ERR_NULL_ARGUMENT                   (-18) /* a required pointer was NULL */
#define QI_ERR_UNSUPPORTED                     (-19) /* valid request outside what this build implements */

typedef struct qi_error_info {
    qi_status code;
    int32_t   reserved;
    int64_t   a;            /* first tuple field of the Error variant (or -1) */
    int64_t   b;            /* second tuple field (or -1) */
    double    re, im;       /* InvalidPauliStringCoefficient payload */
    char      message[256]; /* human-readable text, e.g. the CUDA error string */
} qi_error_info;

/* Last error recorded on the calling thread.  Replaces the payload of the
 * `Err(Error)` value the reference returns (src/errors.rs:4-97). */
qi_status qi_last_error(qi_error_info *out);

/* ------------------------------------------------------------------------ */
/* Engine                                                                    */
/* ------------------------------------------------------------------------ */
#define QI_F64 0   /* complex FP64 amplitudes (double2, 16 B/amp) */
#define QI_F32 1   /* complex FP32 amplitudes (float2,   8 B/amp) */

/* Version / build identification; no reference counterpart. */
const char *qi_version(void);
/* Number of engine kernels launched since load (all threads).  Used by the
 * benchmark to report its own launches; no reference counterpart. */
uint64_t qi_launch_count(void);
/* Select the CUDA device used for new handles (default 0). */
qi_status qi_set_device(int32_t device);

/* ------------------------------------------------------------------------ */
/* State (src/components/state.rs)                                            */
/* ------------------------------------------------------------------------ */
typedef struct qi_state qi_state;

/* Allocate a device-resident state of 2^num_qubits amplitudes, contents
 * undefined.  Storage of `State { state_vector, num_qubits }` (state.rs:74-81).
 * Errors: InvalidNumberOfQubits(0) for num_qubits == 0 (state.rs:166-168). */
qi_status qi_state_create(int32_t num_qubits, int32_t precision, qi_state **out);
qi_status qi_state_destroy(qi_state *s);
qi_status qi_state_info(const qi_state *s, int32_t *num_qubits, int32_t *precision);
/* Run this handle's work on an external CUDA stream (a cudaStream_t passed as
 * void*); NULL restores the handle's own stream. */
qi_status qi_state_set_stream(qi_state *s, void *cuda_stream);
qi_status qi_state_get_stream(qi_state *s, void **cuda_stream);
qi_status qi_state_device_ptr(qi_state *s, void **dev_ptr);
qi_status qi_state_synchronize(qi_state *s);

/* Copy host amplitudes (interleaved f64 pairs) into the device state,
 * converting to the state's precision on the device.  The host buffer stays
 * caller-owned.  num_amps must equal 2^num_qubits (else InvalidNumberOfQubits).
 * A page-locked buffer is read in the state's stream order after the call
 * returns (into an FP32 state by the GPU itself, over the link, converting as it
 * reads), so it must stay unchanged until qi_state_synchronize; pageable buffers
 * are staged before the call returns.
 * Replaces the host->device half of execute_on_gpu (operator.rs:48-58). */
qi_status qi_state_upload(qi_state *s, const double *amps, uint64_t num_amps);
/* Copy the device state back as interleaved f64 pairs (operator.rs:137-147). */
qi_status qi_state_download(qi_state *s, double *amps, uint64_t num_amps);
/* Asynchronous forms for page-locked host buffers: the transfer runs on the copy
 * engine (no SM time) through a device staging buffer of the FP64 size, converted
 * by one device pass, in the handle's stream order; the call returns at once and
 * the host buffer must stay untouched (upload) or is complete (download) only after
 * qi_state_synchronize.  Lets a caller keep two states in flight, one transferring
 * while the other computes.  A pageable host buffer returns InvalidInputValue. */
qi_status qi_state_upload_async(qi_state *s, const double *amps, uint64_t num_amps);
qi_status qi_state_download_async(qi_state *s, double *amps, uint64_t num_amps);
/* Order the work issued on s after this call behind the work issued so far on
 * other's stream (a CUDA event; no host synchronisation).  With two states in
 * flight, a caller puts each state's circuit behind the other's: the circuits
 * then run one after the other at full device rate while the idle state's
 * transfers proceed on the copy engines, instead of both circuits sharing the
 * SMs and finishing together with every transfer left to wait. */
qi_status qi_state_wait(qi_state *s, qi_state *other);

/* Device-side constructors: State::new_zero / new_basis_n / new_plus /
 * new_minus / new_ghz (state.rs:165-325), filled in place. */
qi_status qi_state_set_zero(qi_state *s);
qi_status qi_state_set_basis(qi_state *s, uint64_t n);
qi_status qi_state_set_plus(qi_state *s);
qi_status qi_state_set_minus(qi_state *s);
qi_status qi_state_set_ghz(qi_state *s);

/* `State::new` normalisation check (state.rs:118-123): |sum|a|^2 - 1| <= eps*len,
 * else StateVectorNotNormalised.  Sum in FP64 on the device. */
qi_status qi_state_check_normalised(qi_state *s);
/* Clone with precision conversion (the per-gate `state.clone()`, operator.rs:315). */
qi_status qi_state_copy(qi_state *dst, const qi_state *src);

/* Scalar and vector arithmetic: `State * Complex` (state.rs:2687-2704),
 * `State + State` / `State - State` (state.rs:2773-2862) as y += a*x. */
qi_status qi_state_scale(qi_state *s, double re, double im);
qi_status qi_state_axpy(qi_state *y, double re, double im, const qi_state *x);
/* Comparison of two states of the same size and any precisions (FP64
 * arithmetic): out[0] = max_i |a_i - b_i|, out[1] = sum_i |a_i - b_i|^2,
 * out[2..3] = <b|a>.  No counterpart in the reference; it measures the
 * max-amplitude error and infidelity of an FP32 state against an FP64 one. */
qi_status qi_state_compare(qi_state *a, qi_state *b, double out[4]);
/* Reductions, accumulated in FP64 on the device:
 * inner_product <a|b> = sum conj(a_i) b_i (state.rs:890-917); norm^2. */
qi_status qi_state_inner_product(qi_state *a, qi_state *b, double out[2]);
qi_status qi_state_norm_sqr(qi_state *s, double *out);
/* `State::normalise` (state.rs:924-945): ZeroNorm if the norm is 0. */
qi_status qi_state_normalise(qi_state *s);
/* `State::tensor_product` (state.rs:801-836): out[i*dim_b + j] = a[i]*b[j].
 * out must have num_qubits(a)+num_qubits(b) qubits. */
qi_status qi_state_tensor_product(qi_state *out, qi_state *a, qi_state *b);
/* Read one amplitude: `State::amplitude` (state.rs:448-453). */
qi_status qi_state_amplitude(qi_state *s, uint64_t n, double out[2]);

/* ------------------------------------------------------------------------ */
/* Gates (src/components/operator.rs)                                         */
/* ------------------------------------------------------------------------ */
enum qi_gate_kind {
    QI_GATE_H          = 0,   /* Hadamard            operator.rs:279-433   params: -            */
    QI_GATE_X          = 1,   /* Pauli::X            operator.rs:443-615                        */
    QI_GATE_Y          = 2,   /* Pauli::Y                                                       */
    QI_GATE_Z          = 3,   /* Pauli::Z                                                       */
    QI_GATE_S          = 4,   /* PhaseS              operator.rs:1144-1225                      */
    QI_GATE_T          = 5,   /* PhaseT              operator.rs:1237-1324                      */
    QI_GATE_SDAG       = 6,   /* PhaseSdag           operator.rs:1336-1417                      */
    QI_GATE_TDAG       = 7,   /* PhaseTdag           operator.rs:1429-1516                      */
    QI_GATE_P          = 8,   /* PhaseShift          operator.rs:1528-1633 params: angle        */
    QI_GATE_RX         = 9,   /* RotateX             operator.rs:1645-1776 params: angle        */
    QI_GATE_RY         = 10,  /* RotateY             operator.rs:1788-1917 params: angle        */
    QI_GATE_RZ         = 11,  /* RotateZ             operator.rs:1929-2044 params: angle        */
    QI_GATE_U2         = 12,  /* Unitary2            operator.rs:2058-2285 params: m00re,m00im,m01re,m01im,m10re,m10im,m11re,m11im */
    QI_GATE_RYPHASE    = 13,  /* Unitary2::from_ry_phase          params: theta, phi     */
    QI_GATE_RYPHASE_DAG= 14,  /* Unitary2::from_ry_phase_dagger   params: theta, phi     */
    QI_GATE_CNOT       = 15,  /* CNOT                operator.rs:643-694  (exactly 1 control)   */
    QI_GATE_SWAP       = 16,  /* SWAP                operator.rs:706-829  (2 targets)           */
    QI_GATE_MATCHGATE  = 17,  /* Matchgate           operator.rs:852-1019 params: theta, phi1, phi2; acts on (t, t+1) */
    QI_GATE_TOFFOLI    = 18,  /* Toffoli             operator.rs:1031-1084 (exactly 2 controls) */
    QI_GATE_IDENTITY   = 19,  /* Identity            operator.rs:1096-1132                      */
    /* Circuit-only gate variants (src/components/gate.rs:13-52). */
    QI_GATE_PAULI_STRING    = 20, /* Gate::PauliString -> apply_normalised (gate.rs:115-117) */
    QI_GATE_PAULI_EVOLUTION = 21, /* Gate::PauliTimeEvolution -> apply_exp_neg_i_dt (gate.rs:118-120); params[2] = dt */
    /* Gate::Measurement(basis, indices) -> State::measure, keeping the collapsed state
     * (gate.rs:19, :104-106; state.rs:525-730).  n_targets = 0; targets[0] = basis
     * (QI_BASIS_*); the measured qubits, in outcome-bit order, in controls[0 .. n_controls)
     * (n_controls = 0: every qubit, as State::measure with no indices); params[0..7] = the
     * custom basis matrix for QI_BASIS_CUSTOM; xmask = seed of the outcome draw (the
     * reference draws from the unseeded rand::rng(), state.rs:601).  At most 24 measured
     * qubits.  A plan runs it between its fused segments (nothing is fused across it). */
    QI_GATE_MEASUREMENT     = 22,
    QI_GATE_KIND_COUNT      = 23
};

#define QI_MAX_CONTROLS 32

/* One gate as plain old data: the `Gate::Operator(op, targets, controls)` and
 * `Gate::Parametric(..)` variants (gate.rs:13-52) flattened.  Parametric gates
 * (src/components/parametric/parametric_gate.rs) set param_ids[k] >= 0: at
 * execution params[k] is replaced by theta[param_ids[k]] of the parameter
 * vector passed to the call (Parameter::get, parameter.rs:40-50). */
typedef struct qi_gate {
    int32_t  kind;                      /* enum qi_gate_kind */
    int32_t  n_targets;                 /* 1, or 2 for SWAP */
    int32_t  n_controls;                /* <= QI_MAX_CONTROLS */
    int32_t  param_ids[3];              /* -1 = fixed parameter */
    int32_t  targets[2];
    int32_t  controls[QI_MAX_CONTROLS];
    double   params[8];                 /* kind-specific, see enum; Pauli gates: params[0..1] = coefficient */
    uint64_t xmask, zmask;              /* Pauli gates only: X|Y qubits, Z|Y qubits */
} qi_gate;

/* Apply one operator in place: `Operator::apply(state, targets, controls)`
 * (operator.rs:151-190), validation identical to validate_qubits
 * (operator.rs:214-273) plus the per-gate checks (CNOT control count,
 * Toffoli controls, Matchgate last qubit). */
qi_status qi_apply_gate(qi_state *s, const qi_gate *g);
/* Apply a dense 2^k x 2^k complex matrix (row-major interleaved f64 pairs,
 * local bit j <-> targets[j]) to k distinct qubits, k <= 6; one HBM pass.
 * Generalises Unitary2::apply (operator.rs:2206-2266) to k qubits; no
 * unitarity check.  use_tensor_cores as in qi_exec_options. */
qi_status qi_apply_matrix(qi_state *s, const int32_t *targets, int32_t k, const double *matrix,
                          int32_t use_tensor_cores);
/* `Unitary2::new` unitarity check (operator.rs:2092-2125), tol 2*eps. */
qi_status qi_unitary2_check(const double m[8]);

/* ------------------------------------------------------------------------ */
/* Pauli strings and sums (src/components/pauli_string.rs)                    */
/* ------------------------------------------------------------------------ */
/* A PauliString as masks: qubit q carries X if bit q of xmask only, Z if bit q
 * of zmask only, Y if both (pauli_string.rs:13-18). */
typedef struct qi_pauli_term {
    double   coeff_re, coeff_im;
    uint64_t xmask, zmask;
} qi_pauli_term;

/* out = coefficient * P |in>           PauliString::apply            pauli_string.rs:139-151 */
qi_status qi_pauli_apply(qi_state *out, qi_state *in, const qi_pauli_term *t);
/* s = normalise(P |s>)                 PauliString::apply_normalised  pauli_string.rs:165-168 */
qi_status qi_pauli_apply_normalised(qi_state *s, const qi_pauli_term *t);
/* s = exp(coefficient * P) |s>         PauliString::apply_exp         pauli_string.rs:199-223 */
qi_status qi_pauli_apply_exp(qi_state *s, const qi_pauli_term *t);
/* s = exp(coefficient*factor * P) |s>  PauliString::apply_exp_factor  pauli_string.rs:237-262 */
qi_status qi_pauli_apply_exp_factor(qi_state *s, const qi_pauli_term *t, double factor_re, double factor_im);
/* s = exp(-i dt coefficient P) |s>     PauliString::apply_exp_neg_i_dt pauli_string.rs:281-287 */
qi_status qi_pauli_apply_exp_neg_i_dt(qi_state *s, const qi_pauli_term *t, double dt);
/* out = sum_k c_k P_k |in>             SumOp::apply                   pauli_string.rs:453-466
 * Returns after the result is complete (it reads the output's device flag):
 * QI_ERR_TIMEOUT if a bounded device-side wait of the streamed FP32 kernel ran out. */
qi_status qi_sumop_apply(qi_state *out, qi_state *in, const qi_pauli_term *terms, int64_t n_terms);
/* out = sum_k <s|c_k P_k|s>            SumOp::expectation_value       pauli_string.rs:485-507 */
qi_status qi_sumop_expectation(qi_state *s, const qi_pauli_term *terms, int64_t n_terms, double out[2]);

/* <s|H|s> for H = sum of `terms`, on caller-owned device amplitudes
 * (2^num_qubits float2 or double2 at `amps`), allocating no device memory.
 * It has no counterpart in the reference.  It exists for callers that cannot
 * call cudaMalloc where they evaluate energies — a host application whose GPU
 * memory is owned by its own pool, or a tight solver loop that must not add
 * the device-wide synchronisation of an allocation.  All temporaries live in
 * one static device array of 137,472 bytes that every GPU loading this
 * library holds until exit.  Limits: n_terms <= 4096, and at most 2048 terms
 * sharing one X mask (else InvalidInputValue).  `amps` and `cuda_stream`
 * must belong to the current device (else InvalidInputValue).  The first call
 * on a device looks up that array's device address (cudaGetSymbolAddress) and
 * sets the group kernels' shared-memory limit, with the device current; make
 * that first call before any stream capture.  The address is kept for the
 * life of the process, so a cudaDeviceReset between calls is not supported.
 * All calls share the array: calls whose work overlaps on the GPU (other
 * streams, other host threads) race.  Work is issued on `cuda_stream` (NULL =
 * legacy default stream) and the call returns after it completes. */
qi_status qi_sumop_expectation_noalloc(const void *amps, int32_t num_qubits, int32_t precision,
                                       const qi_pauli_term *terms, int64_t n_terms, void *cuda_stream,
                                       double out[2]);

/* Trotter evolution (src/algorithms/time_evolution.rs:45-166).  order 1 =
 * first_order_trotter_step, 2 = second_order_trotter_step.  If observable !=
 * NULL and observe_every > 0, <observable> is evaluated (FP64 reduction)
 * after every observe_every steps and written to energies_out[2*k..2*k+1]
 * (k = 0 .. num_steps/observe_every - 1). */
qi_status qi_trotter_evolve(qi_state *s, const qi_pauli_term *terms, int64_t n_terms,
                            double dt, int64_t num_steps, int32_t order,
                            const qi_pauli_term *observable, int64_t n_obs,
                            int64_t observe_every, double *energies_out);

/* ------------------------------------------------------------------------ */
/* Circuits (src/circuit.rs:160-202) and the fusion pass                      */
/* ------------------------------------------------------------------------ */
#define QI_FUSION_NONE    0  /* one kernel per gate (the plain per-gate method) */
#define QI_FUSION_GREEDY  1  /* greedy fixed-k fuser, k = max_block_qubits */
#define QI_FUSION_LEARNED 2  /* partitions scored by the learned cost model (greedy fallback) */
#define QI_FUSION_PAULI_GROUPS 3  /* one kernel per gate, except that each run of Pauli exponentials
                                     (Gate::PauliTimeEvolution) whose X-masks lie in {0, X} is one
                                     pass (FP64 Trotter steps use this) */

typedef struct qi_exec_options {
    int32_t fusion;            /* QI_FUSION_* */
    int32_t max_block_qubits;  /* k <= 6; 0 = default (6) */
    int32_t use_tensor_cores;  /* 0 or 1: 3xTF32 tcgen05 kernel for FP32 blocks of k >= 5 (default); 2: CUDA cores only */
    int32_t renorm_every;      /* FP64 renormalisation on the device: 0 = once at the end when tensor-core
                                  blocks ran (their FP32 accumulation rounds toward zero, so the norm drifts
                                  down by ~1e-6 per block); N > 0 = also after every N tensor-core blocks;
                                  -1 = never */
} qi_exec_options;

typedef struct qi_plan_stats {
    int64_t n_gates;          /* gates in the source list */
    int64_t n_kernels;        /* kernel launches per execution */
    int64_t n_blocks_by_k[7]; /* fused blocks by width k (index 0 = per-gate ops) */
    double  predicted_us;     /* cost-model prediction of one execution (0 if none) */
} qi_plan_stats;

typedef struct qi_plan qi_plan;

/* Validate and compile a gate list for one qubit count and precision.
 * Validation runs over the whole list before anything executes, so an invalid
 * gate leaves the state untouched, as the reference's functional
 * Circuit::execute does. `theta` holds the parametric values (may be NULL if
 * no gate has param_ids >= 0). */
qi_status qi_plan_create(int32_t num_qubits, int32_t precision, const qi_gate *gates, int64_t n_gates,
                         const double *theta, int64_t n_theta, const qi_exec_options *opts, qi_plan **out);
qi_status qi_plan_execute(qi_plan *p, qi_state *s);
qi_status qi_plan_stats_get(const qi_plan *p, qi_plan_stats *out);
qi_status qi_plan_destroy(qi_plan *p);
/* Adjoint (reverse-mode) gradient of E(theta) = <psi(theta)|H|psi(theta)> with
 * psi(theta) = U_N(theta) ... U_1(theta) |psi0> and H = sum of `terms` (a
 * SumOp, pauli_string.rs:390-507).  No reference counterpart: it sits beside
 * Circuit::execute (circuit.rs:160-172) and differentiates through the
 * parametric gates (parametric_gate.rs:30-211, Parameter::get parameter.rs:52-57).
 * One forward sweep (fused plan), lambda = H psi, then one reverse sweep in
 * which gates are un-applied to psi and lambda while 2 Re<lambda|dU/dtheta|psi>
 * accumulates in FP64: runs of single-qubit gates share one pass, runs of fixed
 * X / CNOT / SWAP gates are one index permutation, other fixed runs one fused
 * plan of their inverses, the rest one pass per gate (qi_adjoint_sweep_plan
 * lists the passes).  Differentiable kinds: RX, RY, RZ, P, RYPHASE,
 * RYPHASE_DAG, MATCHGATE (any controls).
 * On entry `s` holds |psi0>; on return it holds |psi0> again (restored by the
 * reverse sweep up to rounding).  energy_out (may be NULL) receives E;
 * grads_out[j] = dE/dtheta_j for j < n_theta (parameters that no gate uses get 0). */
qi_status qi_adjoint_gradient(qi_state *s, const qi_gate *gates, int64_t n_gates, const double *theta,
                              int64_t n_theta, const qi_pauli_term *terms, int64_t n_terms,
                              const qi_exec_options *forward_opts, double *energy_out, double *grads_out);
/* The passes of qi_adjoint_gradient's reverse sweep for this gate list (host
 * only, no device work): pass i covers gates hi[i], hi[i] - 1, ..., lo[i] + 1
 * and is one of 0 one gate (k_adjoint, a per-gate un-apply or a Pauli
 * exponential), 1 a group of single-qubit gates (k_adjoint_multi), 2 an index
 * permutation (X / CNOT / SWAP run, k_affine_gather per state), 3 a fused plan
 * of fixed gates' inverses, 4 identities only.  *n_steps receives the count;
 * kinds / hi / lo (capacity entries, may all be NULL) receive the passes. */
qi_status qi_adjoint_sweep_plan(int32_t num_qubits, int32_t precision, const qi_gate *gates, int64_t n_gates,
                                const double *theta, int64_t n_theta, const qi_exec_options *opts,
                                int32_t *kinds, int64_t *hi, int64_t *lo, int64_t capacity, int64_t *n_steps);

/* ------------------------------------------------------------------------ */
/* Measurement (src/components/state.rs:525-784, measurement.rs:15-101)       */
/* ------------------------------------------------------------------------ */
#define QI_BASIS_COMPUTATIONAL 0   /* MeasurementBasis::Computational */
#define QI_BASIS_X             1   /* H before and after (state.rs:671-690) */
#define QI_BASIS_Y             2   /* S-dagger then H before, H then S after (state.rs:691-712) */
#define QI_BASIS_CUSTOM        3   /* U before, U-dagger after (state.rs:713-729) */
/* `State::measure`: outcome probabilities of the measured qubits (bit k of the
 * outcome integer = qubit qubits[k]; n_qubits == 0 measures all qubits in
 * order) summed in FP64 on the device, normalised, one uniform draw
 * r = (splitmix64(seed) >> 11) * 2^-53 (the reference draws from an unseeded
 * rand::rng(), state.rs:601), CDF scan `r < cumulative` in outcome order,
 * collapse and renormalisation in place.  custom_u (8 doubles, Unitary2
 * layout) only for QI_BASIS_CUSTOM.  probs_out (2^m doubles, may be NULL)
 * receives the normalised probabilities.  Errors: InvalidNumberOfQubits when
 * more qubits than the state has, InvalidQubitIndex(q, n), UnknownError when
 * the total probability is below f64::EPSILON (state.rs:593-595).
 * Measuring more than 24 qubits returns Unsupported. */
qi_status qi_measure(qi_state *s, int32_t basis, const double *custom_u, const int32_t *qubits, int32_t n_qubits,
                     uint64_t seed, uint64_t *outcome_out, double *probs_out);
/* `State::measure_n` (state.rs:750-784): n_shots outcomes drawn from the same
 * pre-measurement distribution (shot j uses splitmix64(seed + j)); the state
 * is left unchanged (the basis change is undone).  InvalidNumberOfMeasurements(0)
 * for n_shots == 0. */
qi_status qi_measure_n(qi_state *s, int32_t basis, const double *custom_u, const int32_t *qubits, int32_t n_qubits,
                       int64_t n_shots, uint64_t seed, uint64_t *outcomes_out);

/* Dense tcgen05.mma kind::tf32 rate of the current GPU (no reference
 * counterpart): one CTA per SM issues `iters` M128 x N256 x K8 products from
 * tensor-memory and shared-memory operands into one accumulator, no global
 * memory traffic; best of `reps` timed launches (CUDA events) after one
 * warm-up.  The tensor roof the 3xTF32 fused blocks are measured against. */
qi_status qi_tf32_rate_probe(int32_t iters, int32_t reps, double *tflops_out, double *ms_out);

/* ------------------------------------------------------------------------ */
/* Learned fusion cost model (no reference counterpart)                      */
/* ------------------------------------------------------------------------ */
/* An MLP (20 features -> 3 x 64 ReLU -> 1) predicting y = log(device ms per
 * 2^28 amplitudes) of one device op (dense block on tensor or CUDA cores,
 * diagonal block, per-gate kernel; features in quant-iron_gb300/csrc/qi_mlp.hpp).
 * Trained on the GPU by the engine's own kernels; QI_FUSION_LEARNED plans use
 * it to choose between one kernel per gate and greedy k (tensor cores on/off). */
#define QI_COSTMODEL_FEATURES 20
/* Time `count` seeded random device ops on num_qubits-qubit FP32 and FP64
 * states with CUDA events: features_out[count][20], log_ms_out[count]. */
qi_status qi_costmodel_collect(int32_t num_qubits, int64_t count, uint64_t seed, float *features_out,
                               float *log_ms_out);
/* Full-batch Adam on (X[n][16], Y[n]) from a seeded He initialisation; the
 * trained model becomes the process-wide model.  loss_history[epochs] may be NULL. */
qi_status qi_costmodel_train(const float *X, const float *Y, int64_t n, int32_t epochs, float lr, uint64_t seed,
                             float *loss_history);
qi_status qi_costmodel_predict(const float *X, int64_t n, float *y_out);
/* MSE loss and its gradient w.r.t. the flat parameter vector, for the current parameters. */
qi_status qi_costmodel_loss_and_gradient(const float *X, const float *Y, int64_t n, float *loss_out,
                                         float *grad_out);
qi_status qi_costmodel_init(uint64_t seed);
qi_status qi_costmodel_num_params(int64_t *out);
qi_status qi_costmodel_get_params(float *out, int64_t capacity, int32_t *trained);
qi_status qi_costmodel_set_params(const float *in, int64_t count, int32_t trained);

/* Inspect the i-th device operation of a plan (host only; no device work).
 * Lets tests check the fusion pass without a GPU. */
typedef struct qi_plan_op_info {
    int32_t  kind;          /* 1 one-target gate, 2 SWAP, 3 two-target gate, 4 fused dense block,
                               5 Pauli exponential, 6 Pauli string + normalise, 7 diagonal block,
                               8 renormalisation, 9 phase polynomial (a run of diagonal blocks),
                               10 grouped Pauli exponentials (a run with X-masks in {0, X}),
                               11 qubit permutation (a run of SWAP / X gates; qi_plan_op_bitperm),
                               12 measurement (basis in zmask, seed in xmask) */
    int32_t  k;             /* number of targets (kind 9: number of diagonal blocks in the run;
                               kind 10: number of exponentials in the run; kind 11: gates in the run;
                               kind 12: measured qubits, the first six in targets) */
    int32_t  targets[6];    /* sorted ascending for kinds 3, 4, 7 */
    int32_t  tensor_cores;  /* kind 4: 1 if the block runs on the tcgen05 tensor-core kernel */
    int32_t  phase_poly;    /* kind 4: 1 if a phase polynomial (qi_plan_op_phase_poly) follows the block
                               in the same pass */
    uint64_t control_mask;
    uint64_t xmask, zmask;  /* kinds 5 and 6; kind 9: zmask = the qubits the run touches;
                               kind 10: xmask = X, zmask = OR of the parity basis masks */
    int64_t  n_matrix;      /* complex entries of the op's matrix: 4 (kind 1), 16 (kind 3), 4^k (kind 4),
                               2^k (kind 7: the diagonal), 2 (kind 5: cosh(alpha), sinh(alpha)),
                               kind 10: the tables (see qi_plan_op_pauli_group), else 0 */
} qi_plan_op_info;
qi_status qi_plan_num_ops(const qi_plan *p, int64_t *out);
/* Kind 11 ops: the state after the op is out[j] = in[s(j)] with
 * s(j) = flip ^ sum_k ((j >> k) & 1) << source_bit[k]  (source_bit: num_qubits entries).
 * No reference counterpart: the reference applies each SWAP / X on its own
 * (operator.rs SWAP and Pauli-X apply). */
qi_status qi_plan_op_bitperm(const qi_plan *p, int64_t i, int32_t *source_bit, uint64_t *flip);
qi_status qi_plan_op_get(const qi_plan *p, int64_t i, qi_plan_op_info *info, double *matrix_out, int64_t capacity);
/* Kind 9 ops, and kind 4 ops with phase_poly = 1 (applied after the block): the phase
 * polynomial f(x) = c0 + sum_q a[q] x_q + sum_{q<r} b[q*n+r] x_q x_r applied as
 * exp(2 pi i f / 2^64) (coefficients in units of 2^-64 turns; a: n entries, b: n*n entries,
 * zero for q >= r).  Introspection aid; no reference counterpart. */
qi_status qi_plan_op_phase_poly(const qi_plan *p, int64_t i, uint64_t *c0, uint64_t *a, uint64_t *b);
/* Kind 10 ops: *n_tables tables (<= 4); table t is indexed by the parities
 * beta_j = popcount(i & basis[8 t + j]) & 1, j < rank[t] (index bit j = beta_j),
 * where i is the amplitude index (xmask == 0; the op multiplies amplitude i by the
 * product of its tables' entries) or the pair member with the highest bit of
 * xmask clear (one table of 2^rank[0] row-major 2x2 matrices acting on
 * (psi_i, psi_{i ^ xmask})).  rank: 4 entries, basis: 32.  Introspection aid. */
qi_status qi_plan_op_pauli_group(const qi_plan *p, int64_t i, int32_t *n_tables, int32_t *rank, uint64_t *basis);
/* Execute the plan once with a CUDA event pair around every operation, on the
 * state's stream, and write each operation's device time in milliseconds to
 * ms_out (qi_plan_num_ops entries).  Measurement aid; no reference counterpart. */
qi_status qi_plan_profile(qi_plan *p, qi_state *s, float *ms_out);
/* `Circuit::execute` (circuit.rs:160-172) on a resident state: plan + run. */
qi_status qi_circuit_execute(qi_state *s, const qi_gate *gates, int64_t n_gates,
                             const double *theta, int64_t n_theta, const qi_exec_options *opts);

#ifdef __cplusplus
}
#endif
#endif /* QI_ENGINE_H */
