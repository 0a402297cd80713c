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
