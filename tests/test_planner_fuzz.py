"""Planner fuzz: seeded random circuits of mixed gate families and widths,
planned under random planner settings, executed by the numpy emulator of the
ABI's pass/op arrays (with the engine's own pre-launch validation), against
the oracle.  Parameterized circuits are planned once and replayed for
several points, as sweeps are.  CPU only."""

import numpy as np
import pytest
import sympy

import cirq
from cirq_gb300.ir import flatten_ops
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit
from emulator import run_program
from oracle.circuits import simulate_density_matrix, simulate_state_vector

SYMS = sympy.symbols("a b c")


def _random_op(rng, q, allow_params: bool):
    n = len(q)
    kind = rng.integers(0, 14)
    pick = lambda k: [q[i] for i in rng.choice(n, size=k, replace=False)]  # noqa: E731
    sym = SYMS[rng.integers(0, 3)] if allow_params and rng.random() < 0.3 else None
    val = sym if sym is not None else float(rng.uniform(-1, 1))
    if kind == 0:
        return cirq.PhasedXZGate(x_exponent=rng.uniform(-1, 1), z_exponent=rng.uniform(-1, 1),
                                 axis_phase_exponent=rng.uniform(-1, 1)).on(*pick(1))
    if kind == 1:
        return cirq.rx(val * np.pi if sym is None else val).on(*pick(1))
    if kind == 2:
        return (cirq.Z ** val).on(*pick(1))
    if kind == 3:
        return cirq.H.on(*pick(1))
    if kind == 4 and n >= 2:
        return (cirq.CZ ** val).on(*pick(2))
    if kind == 5 and n >= 2:
        return cirq.CNOT.on(*pick(2))
    if kind == 6 and n >= 2:
        return cirq.ZZPowGate(exponent=val).on(*pick(2))
    if kind == 7 and n >= 2:
        return cirq.ISWAP.on(*pick(2)) ** float(rng.uniform(-1, 1))
    if kind == 8 and n >= 3:
        return cirq.CCZ.on(*pick(3))
    if kind == 9 and n >= 3:
        return cirq.MatrixGate(cirq.testing.random_unitary(8, random_state=int(rng.integers(1 << 30)))).on(*pick(3))
    if kind == 10 and n >= 2:
        d = np.exp(1j * rng.uniform(-np.pi, np.pi, size=4))
        return cirq.DiagonalGate(list(np.angle(d))).on(*pick(2))
    if kind == 11 and n >= 4:
        return cirq.MatrixGate(cirq.testing.random_unitary(16, random_state=int(rng.integers(1 << 30)))).on(*pick(4))
    if kind == 12 and n >= 3:
        return cirq.ControlledGate(cirq.Y ** float(rng.uniform(-1, 1)), num_controls=2).on(*pick(3))
    if kind == 13 and n >= 2:
        return cirq.SWAP.on(*pick(2))
    return cirq.X.on(*pick(1))


def _random_circuit(seed: int, n: int, nops: int, allow_params: bool):
    rng = np.random.default_rng(seed)
    q = cirq.LineQubit.range(n)
    return cirq.Circuit(_random_op(rng, q, allow_params) for _ in range(nops)), q


def _random_planner(rng):
    return Planner(
        tile_bits=int(rng.integers(10, 14)),
        kmax=int(rng.integers(1, 6)),
        budget=float(rng.choice([4.0, 10.0, 25.0, 60.0])),
    )


def _emulate(compiled, resolver):
    from cirq_gb300 import _lib

    _lib.validate_program(compiled.plan)
    nb = compiled.nbits_dev
    psi = np.zeros(2**nb, complex)
    psi[0] = 1
    pool = compiled.pool([resolver])[0].astype(np.complex128)
    return run_program(psi, nb, compiled.plan.passes, compiled.plan.ops, pool)


@pytest.mark.parametrize("seed", range(120))
def test_state_vector_plans_match_the_oracle(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(3, 12))
    allow_params = seed % 2 == 1
    c, q = _random_circuit(seed, n, int(rng.integers(5, 60)), allow_params)
    points = [cirq.ParamResolver({s: float(rng.uniform(-2, 2)) for s in SYMS}) for _ in range(2)]
    if allow_params:
        points.append(cirq.ParamResolver({s: float(v) for s, v in zip(SYMS, (0.0, 1.0, 2.0))}))
    planner = _random_planner(rng)
    cc = CompiledCircuit(flatten_ops(c), q, dm=False, planner=planner, resolvers=points[:1])
    for r in points:
        want = simulate_state_vector(c, r, qubit_order=q)
        got = _emulate(cc, r)
        assert np.max(np.abs(got[: 2**n] - want)) < 1e-6, (seed, planner.tile_bits, planner.kmax)
        assert np.abs(got[2**n :]).max(initial=0) == 0


@pytest.mark.parametrize("seed", range(40))
def test_density_matrix_plans_match_the_oracle(seed):
    rng = np.random.default_rng(2000 + seed)
    n = int(rng.integers(2, 6))
    c, q = _random_circuit(seed + 500, n, int(rng.integers(4, 25)), allow_params=False)
    # interleave channels on one and two qubits
    ops = list(c.all_operations())
    chans = [cirq.depolarize(0.05), cirq.amplitude_damp(0.1), cirq.phase_damp(0.2), cirq.bit_flip(0.1)]
    for i in range(0, len(ops), 3):
        ops.insert(i, chans[int(rng.integers(0, 4))].on(q[int(rng.integers(0, n))]))
    if n >= 2:
        ops.append(cirq.depolarize(0.03, n_qubits=2).on(q[0], q[1]))
    c = cirq.Circuit(ops)
    cc = CompiledCircuit(flatten_ops(c), q, dm=True, planner=_random_planner(rng),
                         resolvers=[cirq.ParamResolver({})])
    got = _emulate(cc, cirq.ParamResolver({}))[: 4**n].reshape(2**n, 2**n)
    want = simulate_density_matrix(c, qubit_order=q)
    assert np.max(np.abs(got - want)) < 1e-6, seed


@pytest.mark.parametrize("seed", range(40))
def test_wide_plans_with_out_of_tile_bits(seed):
    """Wider than a tile: passes over many tiles, selector bits outside the
    tile, layout changes between passes."""
    rng = np.random.default_rng(3000 + seed)
    n = int(rng.integers(11, 15))
    c, q = _random_circuit(seed + 900, n, int(rng.integers(20, 80)), allow_params=seed % 3 == 0)
    planner = Planner(tile_bits=int(rng.integers(10, 12)), kmax=int(rng.integers(2, 6)),
                      budget=float(rng.choice([10.0, 25.0, 40.0])))
    r = cirq.ParamResolver({s: float(rng.uniform(-2, 2)) for s in SYMS})
    cc = CompiledCircuit(flatten_ops(c), q, dm=False, planner=planner, resolvers=[r])
    want = simulate_state_vector(c, r, qubit_order=q)
    got = _emulate(cc, r)
    assert cc.plan.npasses >= 1
    assert np.max(np.abs(got[: 2**n] - want)) < 1e-6, (seed, planner.tile_bits, planner.kmax)
