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
