"""The engine's FP32 per-gate path against the FP32 restatement of the reference's own
GPU path (oracle/opencl_f32.py): same arithmetic precision, so they agree to FP32
rounding, gate by gate and over a whole benchmark-family circuit."""
import numpy as np
import pytest

from oracle import opencl_f32 as ocl
from quant_iron_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_fp32_per_gate_matches_reference_gpu_path(qi, orc):
    n = 16
    gates = workloads.random_circuit(n, layers=8, seed=21)
    init = workloads.plus_state(n)
    want_gpu = ocl.execute(init, n, gates)      # the reference with its `gpu` feature
    want_cpu = orc.execute(init, n, gates)      # the reference's FP64 CPU branch
    with qi.DeviceState(n, qi.F32) as st:
        st.upload(init)
        qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_NONE).execute(st)
        got = st.download()
    scale = np.max(np.abs(want_cpu))
    d_gpu = np.max(np.abs(got - want_gpu))
    assert d_gpu < 2e-5 * scale, d_gpu
    # the engine is no further from the FP64 branch than the reference's own GPU path, within rounding
    assert np.max(np.abs(got - want_cpu)) < 2.0 * np.max(np.abs(want_gpu - want_cpu)) + 1e-6 * scale


@pytest.mark.parametrize("kind,targets,controls,params", [
    ("H", [15], [3], []), ("Y", [0], [], []), ("S", [8], [2], []), ("T", [4], [], []), ("P", [12], [1], [2.5]),
    ("RX", [9], [], [0.3]), ("RY", [2], [11], [1.7]), ("RZ", [13], [], [-0.9]), ("SWAP", [5, 14], [], []),
    ("TOFFOLI", [6], [0, 10], []), ("MATCHGATE", [7], [], [0.8, 1.2, 1.2])])
def test_fp32_gates_match_reference_kernels(qi, kind, targets, controls, params):
    n = 16
    rng = np.random.default_rng(5)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v = (v / np.linalg.norm(v)).astype(np.complex64).astype(np.complex128)
    gate = workloads.GateList().add(kind, targets, controls, params).array()[0]
    want = ocl.apply_gate(v, n, gate)
    with qi.DeviceState(n, qi.F32) as st:
        st.upload(v)
        st.apply_gate(gate)
        got = st.download()
    assert np.max(np.abs(got - want)) < 4 * float(np.finfo(np.float32).eps) * np.max(np.abs(v))
