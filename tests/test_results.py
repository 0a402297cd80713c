"""Result assembly on the host: genuine cirq trial results around downloaded
arrays, without the reference's host-side copies (no GPU involved)."""

import numpy as np

import cirq
from cirq_gb300.simulator import _density_matrix_result, _state_vector_result


def test_state_vector_result_wraps_the_downloaded_vector():
    q = cirq.LineQubit.range(3)
    vec = np.zeros(8, dtype=np.complex64)
    vec[5] = 1
    res = _state_vector_result(cirq.ParamResolver({}), {"m": np.array([1], np.uint8)}, q, vec)
    assert isinstance(res, cirq.StateVectorTrialResult)
    assert res.final_state_vector is vec
    assert res.qubit_map == {q[0]: 0, q[1]: 1, q[2]: 2}
    np.testing.assert_array_equal(res.measurements["m"], [1])
    assert res.dirac_notation() == "|101⟩"


def test_density_matrix_result_hands_over_the_downloaded_matrix():
    q = cirq.LineQubit.range(2)
    rho = np.zeros((4, 4), dtype=np.complex64)
    rho[0, 0] = rho[3, 3] = 0.5
    res = _density_matrix_result(cirq.ParamResolver({}), {}, q, rho)
    assert isinstance(res, cirq.DensityMatrixTrialResult)
    got = res.final_density_matrix
    assert got.shape == (4, 4)
    assert np.shares_memory(got, rho)  # no host copy
    np.testing.assert_array_equal(got, rho)
    assert res.qubit_map == {q[0]: 0, q[1]: 1}
    # the reference's merged-state accessor still sees the same tensor
    np.testing.assert_allclose(res._get_merged_sim_state().target_tensor.reshape(4, 4), rho)
    assert "final density matrix" in str(res).lower()


def test_cache_eviction_releases_graph_runners():
    """With CUDA graphs, a compiled circuit's runner (its state and pool
    buffers and graph) is released when the LRU cache evicts the circuit."""
    import cirq_gb300
    from cirq_gb300 import simulator as S

    class FakeBuffer:
        def __init__(self):
            self.freed = False

        def free(self):
            self.freed = True

    sim = cirq_gb300.Simulator(use_cuda_graphs=True)
    q = cirq.LineQubit.range(3)
    first = sim._compile([cirq.H(q[0])], q, [cirq.ParamResolver({})])
    bufs = (FakeBuffer(), FakeBuffer())
    sim._runners[id(first)] = (first, bufs[0], bufs[1], object())
    for i in range(S._MAX_CACHE):
        sim._compile([cirq.rx(0.1 * (i + 1)).on(q[i % 3])] * (i + 2), q, [cirq.ParamResolver({})])
    assert id(first) not in sim._runners
    assert all(b.freed for b in bufs)
    assert len(sim._cache) == S._MAX_CACHE


def test_simulation_state_initial_states_are_unwrapped():
    """A cirq SimulationState initial state -> its tensor and its own qubit
    order (the reference simulates such a state as is)."""
    import cirq_gb300

    q = cirq.LineQubit.range(3)
    order = [q[2], q[0], q[1]]
    sv = cirq.StateVectorSimulationState(qubits=order, initial_state=5, dtype=np.complex64)
    sim = cirq_gb300.Simulator()
    raw, qo = sim._unwrap_initial_state(sv, cirq.QubitOrder.DEFAULT)
    assert raw.shape == (8,) and raw[5] == 1
    assert tuple(qo.order_for(q)) == tuple(order)
    # a product state (the reference's default split_untangled_states) is merged
    prod = cirq.Simulator(split_untangled_states=True)._create_simulation_state(6, q)
    raw, qo = sim._unwrap_initial_state(prod, cirq.QubitOrder.DEFAULT)
    assert raw.shape == (8,) and abs(raw[6] - 1) < 1e-7
    # density-matrix states: accepted by the density-matrix simulator only
    dm = cirq.DensityMatrixSimulationState(qubits=q, initial_state=2, dtype=np.complex64)
    raw, _ = cirq_gb300.DensityMatrixSimulator()._unwrap_initial_state(dm, cirq.QubitOrder.DEFAULT)
    assert raw.shape == (8, 8) and raw[2, 2] == 1
    try:
        sim._unwrap_initial_state(dm, cirq.QubitOrder.DEFAULT)
    except ValueError:
        pass
    else:
        raise AssertionError("expected ValueError")
    # raw states pass through
    assert sim._unwrap_initial_state(3, "x") == (3, "x")


def _noise_ops(c):
    return [op for op in c.all_operations() if cirq.VirtualTag() in op.tags]


def test_noise_placement_follows_the_reference_run_rule():
    """DensityMatrixSimulator.run: noise on the prefix's qubits after each
    prefix moment, then the terminal measurements' moment, whose noise is
    kept unless it acts on a qubit tuple already measured."""
    import cirq_gb300

    q = cirq.LineQubit.range(2)
    body = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]))
    sim = cirq_gb300.DensityMatrixSimulator(noise=cirq.depolarize(0.1))
    # one two-qubit measurement: the noise after it acts on (q0,) and (q1,)
    c = sim._reference_noisy_circuit(body + cirq.measure(*q, key="m"), "run")
    assert len(_noise_ops(c)) == 3 * 2
    assert isinstance(list(c.all_operations())[-1].gate, cirq.MeasurementGate)
    # one measurement per qubit: the noise after them is skipped
    c = sim._reference_noisy_circuit(body + cirq.Moment([cirq.measure(q[0]), cirq.measure(q[1])]), "run")
    assert len(_noise_ops(c)) == 2 * 2
    # state vector: no prefix; noise after every moment on the circuit's qubits
    sv = cirq_gb300.Simulator(noise=cirq.depolarize(0.1))
    c = sv._reference_noisy_circuit(body + cirq.measure(*q, key="m"), "simulate")
    assert len(_noise_ops(c)) == 3 * 2


def test_noise_placement_follows_the_reference_simulate_split():
    """simulate(): parameterized ops and what follows them on their qubits
    form the suffix; each part is noised on its own qubits, so a moment
    split between the parts gets two noise layers."""
    import sympy

    import cirq_gb300

    q = cirq.LineQubit.range(3)
    t = sympy.Symbol("t")
    c = cirq.Circuit(
        cirq.Moment([cirq.H(q[2]), cirq.rx(t).on(q[0])]),
        cirq.Moment([cirq.CZ(q[0], q[1])]),
    )
    sim = cirq_gb300.DensityMatrixSimulator(noise=cirq.depolarize(0.1))
    noisy = sim._reference_noisy_circuit(c, "simulate")
    # prefix [H(q2)] on {q2}: 1 noise op; suffix [rx(q0)], [CZ(q0,q1)] on {q0, q1}: 2 x 2
    assert len(_noise_ops(noisy)) == 1 + 4
    on_q2 = [op for op in _noise_ops(noisy) if op.qubits == (q[2],)]
    assert len(on_q2) == 1
