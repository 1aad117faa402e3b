"""ctypes binding of the engine's C ABI (include/qi_engine.h).

Loads quant-iron_gb300/lib/libqi_gb300.so.  There is no fallback: if the
library is missing the import fails with an error that says how to build it.
"""
import ctypes
import os

from ._types import (F32, F64, FUSION_GREEDY, FUSION_LEARNED, FUSION_NONE, FUSION_PAULI_GROUPS,  # noqa: F401
                     GATE_DTYPE, GATE_KINDS, MAX_CONTROLS, OK, STATUS_NAMES, TERM_DTYPE)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libqi_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError("quant-iron GB300 engine library not found at %s; build it with "
                      "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
lib = ctypes.CDLL(LIB_PATH)


class ErrorInfo(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("reserved", ctypes.c_int32), ("a", ctypes.c_int64),
                ("b", ctypes.c_int64), ("re", ctypes.c_double), ("im", ctypes.c_double),
                ("message", ctypes.c_char * 256)]


class ExecOptions(ctypes.Structure):
    _fields_ = [("fusion", ctypes.c_int32), ("max_block_qubits", ctypes.c_int32),
                ("use_tensor_cores", ctypes.c_int32), ("renorm_every", ctypes.c_int32)]


class PlanStats(ctypes.Structure):
    _fields_ = [("n_gates", ctypes.c_int64), ("n_kernels", ctypes.c_int64), ("n_blocks_by_k", ctypes.c_int64 * 7),
                ("predicted_us", ctypes.c_double)]


class PlanOpInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("k", ctypes.c_int32), ("targets", ctypes.c_int32 * 6),
                ("tensor_cores", ctypes.c_int32), ("phase_poly", ctypes.c_int32),
                ("control_mask", ctypes.c_uint64), ("xmask", ctypes.c_uint64), ("zmask", ctypes.c_uint64),
                ("n_matrix", ctypes.c_int64)]


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_d = ctypes.c_double
_pd = ctypes.POINTER(ctypes.c_double)

SIGNATURES = {
    "qi_last_error": (_i32, [ctypes.POINTER(ErrorInfo)]),
    "qi_version": (ctypes.c_char_p, []),
    "qi_launch_count": (_u64, []),
    "qi_set_device": (_i32, [_i32]),
    "qi_state_create": (_i32, [_i32, _i32, ctypes.POINTER(_vp)]),
    "qi_state_destroy": (_i32, [_vp]),
    "qi_state_info": (_i32, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "qi_state_set_stream": (_i32, [_vp, _vp]),
    "qi_state_get_stream": (_i32, [_vp, ctypes.POINTER(_vp)]),
    "qi_state_device_ptr": (_i32, [_vp, ctypes.POINTER(_vp)]),
    "qi_state_synchronize": (_i32, [_vp]),
    "qi_state_wait": (_i32, [_vp, _vp]),
    "qi_state_upload": (_i32, [_vp, _vp, _u64]),
    "qi_state_download": (_i32, [_vp, _vp, _u64]),
    "qi_state_upload_async": (_i32, [_vp, _vp, _u64]),
    "qi_state_download_async": (_i32, [_vp, _vp, _u64]),
    "qi_state_set_zero": (_i32, [_vp]),
    "qi_state_set_basis": (_i32, [_vp, _u64]),
    "qi_state_set_plus": (_i32, [_vp]),
    "qi_state_set_minus": (_i32, [_vp]),
    "qi_state_set_ghz": (_i32, [_vp]),
    "qi_state_check_normalised": (_i32, [_vp]),
    "qi_state_copy": (_i32, [_vp, _vp]),
    "qi_state_scale": (_i32, [_vp, _d, _d]),
    "qi_state_axpy": (_i32, [_vp, _d, _d, _vp]),
    "qi_state_inner_product": (_i32, [_vp, _vp, _pd]),
    "qi_state_compare": (_i32, [_vp, _vp, _pd]),
    "qi_tf32_rate_probe": (_i32, [_i32, _i32, _pd, _pd]),
    "qi_state_norm_sqr": (_i32, [_vp, _pd]),
    "qi_state_normalise": (_i32, [_vp]),
    "qi_state_tensor_product": (_i32, [_vp, _vp, _vp]),
    "qi_state_amplitude": (_i32, [_vp, _u64, _pd]),
    "qi_apply_gate": (_i32, [_vp, _vp]),
    "qi_unitary2_check": (_i32, [_pd]),
    "qi_pauli_apply": (_i32, [_vp, _vp, _vp]),
    "qi_pauli_apply_normalised": (_i32, [_vp, _vp]),
    "qi_pauli_apply_exp": (_i32, [_vp, _vp]),
    "qi_pauli_apply_exp_factor": (_i32, [_vp, _vp, _d, _d]),
    "qi_pauli_apply_exp_neg_i_dt": (_i32, [_vp, _vp, _d]),
    "qi_sumop_apply": (_i32, [_vp, _vp, _vp, _i64]),
    "qi_sumop_expectation": (_i32, [_vp, _vp, _i64, _pd]),
    "qi_trotter_evolve": (_i32, [_vp, _vp, _i64, _d, _i64, _i32, _vp, _i64, _i64, _pd]),
    "qi_plan_create": (_i32, [_i32, _i32, _vp, _i64, _pd, _i64, ctypes.POINTER(ExecOptions), ctypes.POINTER(_vp)]),
    "qi_plan_execute": (_i32, [_vp, _vp]),
    "qi_plan_stats_get": (_i32, [_vp, ctypes.POINTER(PlanStats)]),
    "qi_plan_destroy": (_i32, [_vp]),
    "qi_plan_num_ops": (_i32, [_vp, ctypes.POINTER(_i64)]),
    "qi_plan_op_get": (_i32, [_vp, _i64, ctypes.POINTER(PlanOpInfo), _pd, _i64]),
    "qi_circuit_execute": (_i32, [_vp, _vp, _i64, _pd, _i64, ctypes.POINTER(ExecOptions)]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


class QuantIronError(Exception):
    """A failed engine call: `variant` names the quant_iron::errors::Error variant,
    `args_` holds its tuple fields."""

    def __init__(self, code, a=-1, b=-1, message="", re=0.0, im=0.0):
        self.code = code
        self.variant = STATUS_NAMES.get(code, "Unknown(%d)" % code)
        self.a, self.b = a, b
        self.coeff = complex(re, im)
        self.message = message
        super().__init__("%s(%s)%s" % (self.variant, ", ".join(str(x) for x in (a, b) if x != -1),
                                       (": " + message) if message else ""))


def last_error():
    info = ErrorInfo()
    lib.qi_last_error(ctypes.byref(info))
    return info


def check(status):
    if status != OK:
        info = last_error()
        raise QuantIronError(status, info.a, info.b, info.message.decode(errors="replace"), info.re, info.im)
    return status


lib.qi_plan_profile.restype = _i32
lib.qi_plan_profile.argtypes = [_vp, _vp, ctypes.POINTER(ctypes.c_float)]
lib.qi_apply_matrix.restype = _i32
lib.qi_apply_matrix.argtypes = [_vp, _vp, _i32, _pd, _i32]
_pf = ctypes.POINTER(ctypes.c_float)
for _name, _args in {
    "qi_costmodel_collect": [_i32, _i64, _u64, _pf, _pf],
    "qi_costmodel_train": [_pf, _pf, _i64, _i32, ctypes.c_float, _u64, _pf],
    "qi_costmodel_predict": [_pf, _i64, _pf],
    "qi_costmodel_loss_and_gradient": [_pf, _pf, _i64, _pf, _pf],
    "qi_costmodel_init": [_u64],
    "qi_costmodel_num_params": [ctypes.POINTER(_i64)],
    "qi_costmodel_get_params": [_pf, _i64, ctypes.POINTER(_i32)],
    "qi_costmodel_set_params": [_pf, _i64, _i32],
}.items():
    getattr(lib, _name).restype = _i32
    getattr(lib, _name).argtypes = _args
COSTMODEL_FEATURES = 20
lib.qi_measure.restype = _i32
lib.qi_measure.argtypes = [_vp, _i32, _pd, _vp, _i32, _u64, ctypes.POINTER(_u64), _pd]
lib.qi_measure_n.restype = _i32
lib.qi_measure_n.argtypes = [_vp, _i32, _pd, _vp, _i32, _i64, _u64, ctypes.POINTER(_u64)]
BASIS = {"Computational": 0, "X": 1, "Y": 2, "Custom": 3}
lib.qi_sumop_expectation_noalloc.restype = _i32
lib.qi_sumop_expectation_noalloc.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _pd]
lib.qi_plan_op_phase_poly.restype = _i32
lib.qi_plan_op_phase_poly.argtypes = [_vp, _i64, ctypes.POINTER(_u64), _vp, _vp]
lib.qi_plan_op_pauli_group.restype = _i32
lib.qi_plan_op_pauli_group.argtypes = [_vp, _i64, ctypes.POINTER(_i32), _vp, _vp]
lib.qi_plan_op_bitperm.restype = _i32
lib.qi_plan_op_bitperm.argtypes = [_vp, _i64, _vp, ctypes.POINTER(ctypes.c_uint64)]
lib.qi_adjoint_gradient.restype = _i32
lib.qi_adjoint_gradient.argtypes = [_vp, _vp, _i64, _pd, _i64, _vp, _i64, ctypes.POINTER(ExecOptions), _pd, _pd]
lib.qi_adjoint_sweep_plan.restype = _i32
lib.qi_adjoint_sweep_plan.argtypes = [_i32, _i32, _vp, _i64, _pd, _i64, ctypes.POINTER(ExecOptions), _vp, _vp, _vp, _i64,
                                      ctypes.POINTER(_i64)]
