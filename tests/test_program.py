"""Host-side compilation: planner encoding checked with the CPU emulator
against the reference's golden states (no GPU needed)."""

import numpy as np
import pytest
import sympy

import cirq
from cirq_gb300 import workloads
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements
from emulator import run_program
from oracle.circuits import simulate_state_vector

GOLD = np.load(__file__.replace("test_program.py", "golden/golden.npz"))

PLANNERS = [
    Planner(tile_bits=10, kmax=3, budget=20),
    Planner(tile_bits=12, kmax=4),
    Planner(tile_bits=10, kmax=2, budget=8),
    Planner(tile_bits=11, kmax=5, budget=100),
    Planner(tile_bits=13, kmax=1, budget=6),
]


def _emulate(compiled, resolver=None, initial=0):
    from cirq_gb300 import _lib

    _lib.validate_program(compiled.plan)  # the engine's own pre-launch checks
    nb = compiled.nbits_dev
    psi = np.zeros(2**nb, complex)
    psi[initial] = 1
    pool = compiled.pool([resolver or cirq.ParamResolver({})])[0].astype(np.complex128)
    return run_program(psi, nb, compiled.plan.passes, compiled.plan.ops, pool)


@pytest.mark.parametrize("planner", PLANNERS, ids=lambda p: f"L{p.tile_bits}k{p.kmax}b{p.budget}")
@pytest.mark.parametrize("n,d,s", [(10, 20, 1), (12, 8, 2), (5, 6, 3)])
def test_layers_plan_vs_golden(planner, n, d, s):
    c = workloads.random_layer_circuit(n, d, s)
    body, _ = split_measurements(c)
    cc = CompiledCircuit(body, sorted(c.all_qubits()), dm=False, planner=planner, resolvers=[cirq.ParamResolver({})])
    out = _emulate(cc)
    np.testing.assert_allclose(out[: 2**n], GOLD[f"layers_n{n}_d{d}_s{s}_c128"], atol=1e-6)
    assert np.abs(out[2**n :]).max(initial=0) == 0


def test_gate_zoo_plan_vs_golden():
    import make_zoo

    zoo = make_zoo.gate_zoo()
    body, _ = split_measurements(zoo)
    for planner in PLANNERS:
        cc = CompiledCircuit(body, sorted(zoo.all_qubits()), dm=False, planner=planner, resolvers=[cirq.ParamResolver({})])
        np.testing.assert_allclose(_emulate(cc)[:32], GOLD["zoo_c128"], atol=1e-6)


def test_density_plan_vs_golden():
    c = workloads.noisy_layer_circuit(4, 4, seed=2, p=0.05, gamma=0.1)
    body, _ = split_measurements(c)
    for planner in PLANNERS:
        cc = CompiledCircuit(body, sorted(c.all_qubits()), dm=True, planner=planner, resolvers=[cirq.ParamResolver({})])
        out = _emulate(cc)[: 4**4].reshape(16, 16)
        np.testing.assert_allclose(out, GOLD["dm_noisy_n4_d4"], atol=1e-6)


def test_sweep_replay_matches_per_point_planning():
    """Pools replayed from one plan equal the states of per-point simulation,
    including points where a parameterised gate degenerates (X**0 = I)."""
    t, u = sympy.symbols("t u")
    q = cirq.LineQubit.range(11)
    c = cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.X(q[0]) ** t,
        cirq.ZZPowGate(exponent=u).on(q[1], q[9]),
        cirq.CZ(q[0], q[10]) ** t,
        cirq.rx(u).on(q[5]),
        cirq.CNOT(q[5], q[3]),
    )
    pts = [{t: 0.0, u: 0.0}, {t: 1.0, u: 0.5}, {t: 0.3, u: -1.7}]
    res = [cirq.ParamResolver(p) for p in pts]
    cc = CompiledCircuit(split_measurements(c)[0], q, dm=False, planner=Planner(tile_bits=10), resolvers=res[:1])
    for r in res:
        want = simulate_state_vector(c, r)
        np.testing.assert_allclose(_emulate(cc, r)[: 2**11], want, atol=1e-6)


def test_unsupported_operations_raise():
    q = cirq.LineQubit.range(6)
    with pytest.raises(NotImplementedError):
        CompiledCircuit([cirq.MatrixGate(cirq.testing.random_unitary(64)).on(*q)], q, dm=False,
                        planner=Planner(), resolvers=[cirq.ParamResolver({})])
    with pytest.raises(NotImplementedError):
        CompiledCircuit([cirq.depolarize(0.1).on(q[0])], q, dm=False, planner=Planner(),
                        resolvers=[cirq.ParamResolver({})])
    qt = cirq.LineQid.range(2, dimension=3)
    with pytest.raises(NotImplementedError):
        CompiledCircuit([cirq.MatrixGate(np.eye(3), qid_shape=(3,)).on(qt[0])], qt, dm=False,
                        planner=Planner(), resolvers=[cirq.ParamResolver({})])


def test_register_layouts_are_complete():
    """Every LAYOUT op names exactly L - 8 distinct register bits, none of which
    is a selector of a register op in its phase (the engine rejects others)."""
    from cirq_gb300 import adjoint

    circuit, symbols, values = workloads.hea_circuit(12, 3, seed=12)
    ham = workloads.random_pauli_hamiltonian(12, 30, seed=13)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    c2 = workloads.random_layer_circuit(16, 12, seed=1)
    cc = CompiledCircuit(split_measurements(c2)[0], sorted(c2.all_qubits()), dm=False,
                         planner=Planner(tile_bits=12), resolvers=[cirq.ParamResolver({})])
    from cirq_gb300 import _lib

    _lib.validate_program(prog.reverse, dual=True)
    for plan in (prog.forward.plan, prog.reverse, cc.plan):
        _lib.validate_program(plan, dual=plan is prog.reverse)
        for p in plan.passes:
            L = int(p["L"])
            regs = None
            for o in plan.ops[p["op_begin"] : p["op_begin"] + p["op_count"]]:
                if o["kind"] == 4:
                    regs = [int(b) for b in o["bits"][: int(o["k"])]]
                    assert len(regs) == L - 8 and len(set(regs)) == L - 8
                elif o["kind"] in (5, 7):
                    pos = [regs.index(int(b)) for b in o["bits"][: int(o["k"])]]
                    assert pos == sorted(pos)
                    for c in o["sel"][: int(o["nsel"])]:
                        assert int(c) not in regs
                elif o["kind"] in (0, 1, 2, 3):
                    regs = None


def test_wide_unitaries_are_decomposed_exactly():
    """A 7-qubit multi-controlled gate (beyond the 5-qubit op limit) goes
    through the reference's own decomposition; the plan still matches the
    oracle's direct application of the 7-qubit unitary."""
    from cirq_gb300.ir import flatten_ops

    q = cirq.LineQubit.range(8)
    c = cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.X(q[6]).controlled_by(*q[:6]),
        cirq.rz(0.3).on(q[7]).controlled_by(*q[1:6]),
        cirq.CZ(q[0], q[7]),
    )
    ops = flatten_ops(c)
    assert max(len(o.qubits) for o in ops) <= 5
    compiled = CompiledCircuit(ops, q, dm=False, planner=Planner(tile_bits=10, kmax=4),
                               resolvers=[cirq.ParamResolver({})])
    got = _emulate(compiled)[: 2**8]
    want = simulate_state_vector(c, qubit_order=q)
    assert np.max(np.abs(got - want)) < 1e-6
