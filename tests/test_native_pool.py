"""gbq_pool_build (csrc/gbq_pool.cu) against the planner's numpy replay of
the fusion recipes, for one parameter point: fused dense ops with selectors
and permutations, diagonal ops, two-state probe programs, tensor-core
blocks and density-matrix superoperators.  No GPU needed."""

import numpy as np
import pytest
import cirq
from cirq_gb300 import planner as P
from cirq_gb300 import adjoint, workloads
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements


def _both(plan, gates):
    native = plan._native_pool(gates)
    assert native is not None
    P.NATIVE_POOLS = False
    try:
        ref = plan.pool_for(gates, 1)
    finally:
        P.NATIVE_POOLS = True
    return native, ref


def _check(plan, gates):
    native, ref = _both(plan, gates)
    assert native.shape == ref.shape and native.dtype == np.complex64
    # complex128 sums in a different order: at most one float32 ulp apart
    assert np.allclose(native, ref, rtol=2e-7, atol=1e-7), np.max(np.abs(native - ref))


def _compiled(circuit, planner, dm=False, resolvers=None):
    body, _ = split_measurements(circuit)
    return CompiledCircuit(body, sorted(circuit.all_qubits()), dm=dm, planner=planner,
                           resolvers=resolvers or [cirq.ParamResolver({})])


@pytest.mark.parametrize("kw", [dict(budget=25.0), dict(budget=40.0, kmax=4), dict(kmax=2, budget=10.0),
                                dict(tile_bits=10, kmax=5, budget=60.0), dict(tensor=True, budget=4)])
def test_random_layers(kw):
    c = workloads.random_layer_circuit(16, 12, 4)
    cc = _compiled(c, Planner(**kw))
    gates = cc.gate_batch([cirq.ParamResolver({})])
    _check(cc.plan, {i: gates[j] for i, j in enumerate(cc.kept)})


def test_parameterised_qaoa_point():
    c = workloads.qaoa_circuit(14, 3, seed=2)[0]
    r = cirq.ParamResolver({s: 0.37 * (i + 1) for i, s in enumerate(sorted(cirq.parameter_symbols(c), key=str))})
    cc = _compiled(c, Planner(budget=25.0), resolvers=[r])
    gates = cc.gate_batch([r])
    _check(cc.plan, {i: gates[j] for i, j in enumerate(cc.kept)})


def test_density_matrix_superoperators():
    c = workloads.noisy_layer_circuit(6, 6, 1)
    cc = _compiled(c, Planner(budget=25.0), dm=True)
    gates = cc.gate_batch([cirq.ParamResolver({})])
    _check(cc.plan, {i: gates[j] for i, j in enumerate(cc.kept)})


def test_adjoint_reverse_program_with_probes():
    circuit, symbols, values = workloads.hea_circuit(12, 3, seed=0)
    ham = workloads.random_pauli_hamiltonian(12, 20, seed=1)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    r = cirq.ParamResolver(dict(zip(prog.symbols, [float(v) for v in values])))
    gates = prog.forward.gate_batch([r])
    batch = prog._reverse_batch(r, gates)
    _check(prog.reverse, batch)


def test_points_match_one_point_builds_and_the_numpy_batch_replay():
    # gbq_pool_build_points on host threads: every point's pool equals the
    # one-point build bit for bit, and the numpy replay of the whole batch
    # to float32 rounding
    c, gammas, betas, _, _ = workloads.qaoa_circuit(14, 3, seed=5)
    rng = np.random.default_rng(3)
    res = [cirq.ParamResolver({**{g: float(rng.uniform(-1, 1)) for g in gammas},
                               **{b: np.float64(rng.uniform(-1, 1)) for b in betas}}) for _ in range(37)]
    cc = _compiled(c, Planner(budget=25.0), resolvers=res[:1])
    gates = cc.gate_batch(res)
    g = {i: gates[j] for i, j in enumerate(cc.kept)}
    plan = cc.plan
    many = plan._native_pool(g, len(res))
    for p in range(len(res)):
        one = plan._native_pool({k: v[p : p + 1] for k, v in g.items()}, 1)
        assert np.array_equal(many[p : p + 1].view(np.uint32), one.view(np.uint32)), p
    P.NATIVE_POOLS = False
    try:
        ref = plan.pool_for(g, len(res))
    finally:
        P.NATIVE_POOLS = True
    assert np.allclose(many, ref, rtol=2e-7, atol=1e-7)
    assert np.array_equal(plan.pool_for(g, len(res)), many)  # pool_for takes the native route
