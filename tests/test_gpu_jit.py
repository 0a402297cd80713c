"""Pass-specialised kernels (gbq_jit.cu) against the tile-pass interpreter.

A specialised kernel folds a pass's op records into straight-line code but
keeps the interpreter's arithmetic and its order, so the final states must be
bit-identical; the 20-qubit depth-20 state is also checked against the
reference's complex128 amplitudes (golden/golden_large.npz).
"""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import workloads

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_jit.py", "golden/golden_large.npz"))


def _final(sim, circuit, jit):
    sim.engine.set_jit(jit)
    try:
        return sim.simulate(circuit).final_state_vector.copy()
    finally:
        sim.engine.set_jit(False)


def test_specialised_passes_bit_identical_and_pinned():
    c = workloads.random_layer_circuit(20, 20, 0)
    sim = cirq_gb300.Simulator()
    plain = _final(sim, c, False)
    before = sim.engine.jit_launches()
    spec = _final(sim, c, True)
    assert sim.engine.jit_launches() > before, "no specialised kernel ran"
    assert np.array_equal(spec, plain)
    key = "layers_n20_d20_s0_c128"
    idx = GOLD[f"{key}_idx"]
    assert np.max(np.abs(spec[idx] - GOLD[f"{key}_amps"])) < 1e-5


def test_specialised_passes_cached_and_reused():
    c = workloads.random_layer_circuit(16, 12, 3)
    sim = cirq_gb300.Simulator()
    first = _final(sim, c, True)
    n = sim.engine.jit_compiles()
    again = _final(sim, c, True)
    assert sim.engine.jit_compiles() == n, "a cached pass was compiled again"
    assert np.array_equal(first, again)
    assert np.array_equal(first, _final(sim, c, False))


def test_specialised_passes_parameter_sweep():
    # one structure, new matrix pools per point: the kernels are reused and
    # each point matches the interpreter
    q = cirq.LineQubit.range(14)
    import sympy

    t = sympy.Symbol("t")
    c = cirq.Circuit(
        [cirq.H(x) for x in q],
        [cirq.CZ(q[i], q[i + 1]) for i in range(0, 13, 2)],
        [cirq.rx(t * (i + 1)).on(x) for i, x in enumerate(q)],
        [cirq.CZ(q[i], q[i + 1]) for i in range(1, 13, 2)],
        [cirq.ry(0.3 * t).on(x) for x in q],
    )
    sim = cirq_gb300.Simulator()
    sweep = cirq.Linspace("t", 0.1, 1.3, 4)
    sim.engine.set_jit(True)
    try:
        spec = [r.final_state_vector.copy() for r in sim.simulate_sweep(c, sweep)]
    finally:
        sim.engine.set_jit(False)
    plain = [r.final_state_vector.copy() for r in sim.simulate_sweep(c, sweep)]
    for a, b in zip(spec, plain):
        assert np.array_equal(a, b)


def test_background_compilation_switches_kernels_without_changing_results():
    # mode 2: the first run queues the kernels and runs the interpreter;
    # once they are built the same program runs them -- identical bits
    c = workloads.random_layer_circuit(20, 12, 5)
    sim = cirq_gb300.Simulator()
    plain = _final(sim, c, 0)
    sim.engine.set_jit(2)
    try:
        first = sim.simulate(c).final_state_vector.copy()
        assert sim.engine.jit_wait(300.0)
        before = sim.engine.jit_launches()
        second = sim.simulate(c).final_state_vector.copy()
        assert sim.engine.jit_launches() > before
    finally:
        sim.engine.set_jit(0)
    assert np.array_equal(first, plain)
    assert np.array_equal(second, plain)


def test_specialised_two_state_passes_match_interpreter():
    # adjoint gradient: forward passes (one state) and reverse passes (two
    # states with probes) on the generated kernels against the interpreter;
    # probe sums are reduced with atomics, so they agree to rounding
    from cirq_gb300 import adjoint

    circuit, symbols, values = workloads.hea_circuit(20, 4, seed=2)
    ham = workloads.random_pauli_hamiltonian(20, 40, seed=3)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    eng = prog.engine
    eng.set_jit(0)
    e0, g0 = prog.value_and_grad(values)
    before = eng.jit_launches()
    eng.set_jit(1)
    try:
        e1, g1 = prog.value_and_grad(values)
    finally:
        eng.set_jit(0)
    assert eng.jit_launches() - before > prog.reverse.npasses // 2
    # the forward state is bit-identical; <psi|H|psi> is reduced with atomics
    assert abs(e1 - e0) < 1e-12 * max(1.0, abs(e0))
    assert np.allclose(g1, g0, rtol=1e-5, atol=1e-6), np.max(np.abs(g1 - g0))
