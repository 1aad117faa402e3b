"""Constants and C struct layouts of the engine's C ABI (include/qi_engine.h).

Plain data only: importing this module does not load the engine library, so
workload generators can build gate and term arrays without it.
"""
import numpy as np

OK = 0
F64 = 0
F32 = 1
FUSION_NONE = 0
FUSION_GREEDY = 1
FUSION_LEARNED = 2
FUSION_PAULI_GROUPS = 3
MAX_CONTROLS = 32

# qi_status -> name of the quant_iron::errors::Error variant (src/errors.rs:4-97)
STATUS_NAMES = {
    -1: "InvalidNumberOfMeasurements",
    -2: "OverlappingControlAndTargetQubits",
    -3: "InvalidNumberOfQubits",
    -4: "InvalidQubitIndex",
    -5: "StateVectorNotNormalised",
    -6: "NonUnitaryMatrix",
    -7: "InvalidNumberOfInputs",
    -8: "MismatchedNumberOfParameters",
    -9: "UnknownError",
    -10: "OpenCLError",
    -11: "GpuContextLockError",
    -12: "CircuitMacroError",
    -13: "InvalidInputValue",
    -14: "ZeroNorm",
    -15: "InvalidPauliStringCoefficient",
    -16: "OutOfMemory",
    -17: "Timeout",
    -18: "NullArgument",
    -19: "Unsupported",
}

GATE_KINDS = dict(H=0, X=1, Y=2, Z=3, S=4, T=5, SDAG=6, TDAG=7, P=8, RX=9, RY=10, RZ=11, U2=12, RYPHASE=13,
                  RYPHASE_DAG=14, CNOT=15, SWAP=16, MATCHGATE=17, TOFFOLI=18, IDENTITY=19, PAULI_STRING=20,
                  PAULI_EVOLUTION=21, MEASUREMENT=22)

# qi_gate as a numpy structured dtype (same layout as the C struct)
GATE_DTYPE = np.dtype([
    ("kind", "<i4"), ("n_targets", "<i4"), ("n_controls", "<i4"), ("param_ids", "<i4", (3,)),
    ("targets", "<i4", (2,)), ("controls", "<i4", (MAX_CONTROLS,)), ("params", "<f8", (8,)),
    ("xmask", "<u8"), ("zmask", "<u8"),
], align=True)
assert GATE_DTYPE.itemsize == 240, GATE_DTYPE.itemsize

TERM_DTYPE = np.dtype([("re", "<f8"), ("im", "<f8"), ("xmask", "<u8"), ("zmask", "<u8")])
