"""Generated sources of pass-specialised kernels compile for sm_103a (NVRTC,
no GPU needed) and passes without a specialised form are refused."""

import ctypes

import numpy as np
import pytest

from cirq_gb300 import _lib, workloads
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements

import cirq


def _plan(n, depth):
    c = workloads.random_layer_circuit(n, depth, 1)
    body, _ = split_measurements(c)
    cc = CompiledCircuit(body, sorted(c.all_qubits()), dm=False, planner=Planner(budget=25.0),
                         resolvers=[cirq.ParamResolver({})])
    return cc.nbits_dev, cc.plan


def _source(lib, nbits, plan, q, dual=0):
    passes = np.ascontiguousarray(plan.passes)
    ops = np.ascontiguousarray(plan.ops)
    need = ctypes.c_size_t(0)
    rc = lib.gbq_jit_source(nbits, passes[q:q + 1].ctypes.data, ops.ctypes.data, len(ops), dual, None, 0,
                            ctypes.byref(need))
    if rc:
        return rc, None
    buf = ctypes.create_string_buffer(need.value)
    rc = lib.gbq_jit_source(nbits, passes[q:q + 1].ctypes.data, ops.ctypes.data, len(ops), dual, buf, need.value,
                            ctypes.byref(need))
    return rc, buf.value


def test_generated_pass_compiles():
    lib = _lib.load()
    nbits, plan = _plan(18, 8)
    rc, src = _source(lib, nbits, plan, 0)
    assert rc == 0
    assert b"k_jit" in src and b"rdense<" in src
    size = ctypes.c_size_t(0)
    rc = lib.gbq_jit_compile_check(src, ctypes.byref(size))
    if rc == _lib.ERR_UNSUPPORTED and b"not found" in lib.gbq_last_error():
        pytest.skip("NVRTC is not installed")
    assert rc == 0, lib.gbq_last_error().decode()[:2000]
    assert size.value > 1000


def test_pass_without_specialised_form_is_refused():
    lib = _lib.load()
    # a shared-memory dense op (width 3) has no specialised form
    passes = np.zeros(1, dtype=_lib.PASS_DTYPE)
    passes[0]["L"], passes[0]["m"], passes[0]["op_begin"], passes[0]["op_count"] = 12, 5, 0, 1
    passes[0]["hi"][:7] = np.arange(5, 12)
    ops = np.zeros(1, dtype=_lib.OP_DTYPE)
    ops[0]["kind"], ops[0]["k"] = _lib.OP_DENSE, 3
    ops[0]["bits"][:3] = [0, 1, 2]
    need = ctypes.c_size_t(0)
    rc = lib.gbq_jit_source(12, passes.ctypes.data, ops.ctypes.data, 1, 0, None, 0, ctypes.byref(need))
    assert rc == _lib.ERR_UNSUPPORTED


def test_generated_two_state_pass_compiles():
    # a reverse (two-state) pass of an adjoint program: probes and both states
    from cirq_gb300 import adjoint

    lib = _lib.load()
    circuit, symbols, _ = workloads.hea_circuit(14, 2, seed=0)
    ham = workloads.random_pauli_hamiltonian(14, 10, seed=1)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    plan = prog.reverse
    for q in range(len(plan.passes)):
        rc, src = _source(lib, prog.nbits, plan, q, dual=1)
        if rc == 0 and b"rprobe<" in src:
            break
    else:
        pytest.fail("no two-state pass with a probe has a specialised form")
    assert b"probe_flush" in src and b"a.partial" in src
    size = ctypes.c_size_t(0)
    rc = lib.gbq_jit_compile_check(src, ctypes.byref(size))
    if rc == _lib.ERR_UNSUPPORTED and b"not found" in lib.gbq_last_error():
        pytest.skip("NVRTC is not installed")
    assert rc == 0, lib.gbq_last_error().decode()[:2000]


def test_all_diagonal_passes_get_a_register_phase_and_a_specialised_form():
    # rz layers and CZ ladders only: every pass is diagonal, and each must be
    # one register phase (LAYOUT then register diagonals) with a generated source
    q = cirq.LineQubit.range(16)
    import sympy

    syms = sympy.symbols("z0:16")
    c = cirq.Circuit([cirq.rz(s).on(qq) for s, qq in zip(syms, q)],
                     [cirq.CZ(q[i], q[i + 1]) for i in range(15)],
                     [cirq.ZZ(q[i], q[(i + 5) % 16]) ** 0.3 for i in range(16)])
    r = cirq.ParamResolver({s: 0.1 * (i + 1) for i, s in enumerate(syms)})
    cc = CompiledCircuit(list(c.all_operations()), q, dm=False, planner=Planner(budget=25.0), resolvers=[r])
    plan = cc.plan
    lib = _lib.load()
    for p in range(len(plan.passes)):
        rec = plan.passes[p]
        kinds = plan.ops["kind"][rec["op_begin"]: rec["op_begin"] + rec["op_count"]]
        assert kinds[0] == _lib.OP_LAYOUT
        assert set(kinds[1:].tolist()) <= {_lib.OP_RDIAG}
        rc, src = _source(lib, cc.nbits_dev, plan, p)
        assert rc == 0 and b"tab[base" in src  # tables staged in shared memory


def test_two_state_diagonal_passes_have_specialised_forms():
    from cirq_gb300 import adjoint

    circuit, symbols, _ = workloads.hea_circuit(14, 2, seed=0)
    ham = workloads.random_pauli_hamiltonian(14, 10, seed=1)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    plan = prog.reverse
    lib = _lib.load()
    diag_only = 0
    for p in range(len(plan.passes)):
        rec = plan.passes[p]
        kinds = set(plan.ops["kind"][rec["op_begin"] + 1: rec["op_begin"] + rec["op_count"]].tolist())
        if kinds <= {_lib.OP_RDIAG, _lib.OP_RPROBE_DIAG}:
            diag_only += 1
        rc, _ = _source(lib, prog.nbits, plan, p, dual=1)
        assert rc == 0, p
    assert diag_only > 0
