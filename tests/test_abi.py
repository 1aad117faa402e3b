"""The C-ABI library loads and exports every entry point include/qi_engine.h declares (no GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "qi_engine.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qi_[a-z0-9_]+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(qi):
    lib = qi._abi.lib
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts(qi):
    assert qi._abi.GATE_DTYPE.itemsize == 240
    assert qi._abi.TERM_DTYPE.itemsize == 32
    assert ctypes.sizeof(qi._abi.ErrorInfo) == 296


def test_status_codes_match_header(qi):
    txt = open(os.path.join(ROOT, "include", "qi_engine.h")).read()
    codes = {int(v): k for k, v in re.findall(r"#define (QI_ERR_[A-Z_]+)\s+\((-\d+)\)", txt)}
    assert len(codes) == len(qi._abi.STATUS_NAMES)
    for code in codes:
        assert code in qi._abi.STATUS_NAMES


def test_unitary2_check_host_only(qi):
    from quant_iron_gb300 import quant_iron as q
    q.Unitary2.new([[0, 1], [1, 0]])
    with pytest.raises(qi.QuantIronError) as ei:
        q.Unitary2.new([[1, 1], [0, 1]])
    assert ei.value.variant == "NonUnitaryMatrix"


def test_plan_validation_runs_without_gpu(qi):
    """qi_plan_create validates the whole list on the host, before any device work."""
    from quant_iron_gb300.workloads import GateList
    gl = GateList().add("H", [0]).add("CNOT", [1], [0]).add("H", [5])
    with pytest.raises(qi.QuantIronError) as ei:
        qi.Plan(3, qi.F64, gl.array())
    assert ei.value.variant == "InvalidQubitIndex" and (ei.value.a, ei.value.b) == (5, 3)
    assert "gate 2" in ei.value.message


def test_parametric_gate_needs_theta(qi):
    from quant_iron_gb300.workloads import GateList
    gl = GateList().add("RY", [0], [], [0.0], [4])
    with pytest.raises(qi.QuantIronError) as ei:
        qi.Plan(2, qi.F32, gl.array(), theta=np.zeros(2))
    assert ei.value.variant == "MismatchedNumberOfParameters"
