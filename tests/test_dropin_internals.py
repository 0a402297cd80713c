"""The reference internals the drop-in's result construction relies on, the
public-constructor route it falls back to, and the vectorised confusion-map
draw against the reference's own per-repetition draw."""

import functools
import inspect

import numpy as np
import pytest
import scipy.stats

import cirq
from cirq_gb300 import simulator as sim_mod


def test_reference_internals_used_for_results_exist():
    """cirq_gb300.simulator builds genuine result objects around downloaded
    arrays without the reference's copies and validation; these are the
    names and shapes that route depends on.  A Cirq release that changes one
    of them fails here rather than silently taking the slow public route."""
    from cirq.sim.density_matrix_simulation_state import _BufferedDensityMatrix
    from cirq.sim.state_vector_simulation_state import _BufferedStateVector

    assert list(inspect.signature(_BufferedStateVector.__init__).parameters)[1:3] == ["state_vector", "buffer"]
    assert list(inspect.signature(_BufferedDensityMatrix.__init__).parameters)[1:3] == ["density_matrix", "buffer"]
    params = inspect.signature(cirq.SimulationState.__init__).parameters
    assert {"state", "prng", "qubits", "classical_data"} <= set(params)
    prop = cirq.StateVectorTrialResult.__dict__["final_state_vector"]
    assert isinstance(prop, functools.cached_property) and prop.attrname == "final_state_vector"
    q = cirq.LineQubit.range(1)
    st = cirq.DensityMatrixSimulationState(qubits=q, initial_state=0, dtype=np.complex64)
    res = cirq.DensityMatrixTrialResult(params=cirq.ParamResolver({}), measurements={}, final_simulator_state=st)
    assert hasattr(res, "_final_density_matrix")


def test_results_through_the_private_route():
    q = cirq.LineQubit.range(2)
    vec = np.array([0.6, 0, 0, 0.8j], dtype=np.complex64)
    r = sim_mod._state_vector_result(cirq.ParamResolver({}), {}, q, vec)
    assert isinstance(r, cirq.StateVectorTrialResult)
    assert r.final_state_vector is vec
    np.testing.assert_array_equal(r._final_simulator_state.target_tensor.reshape(-1), vec)
    rho = np.outer(vec, vec.conj()).astype(np.complex64)
    d = sim_mod._density_matrix_result(cirq.ParamResolver({}), {}, q, rho)
    assert isinstance(d, cirq.DensityMatrixTrialResult)
    np.testing.assert_array_equal(d.final_density_matrix, rho)


def test_results_through_the_public_constructor_fallback(monkeypatch):
    """If the private buffers are gone, results are built with the public
    constructors (which copy and validate) and hold the same values."""
    def gone(*args, **kwargs):
        raise ImportError("cannot import name '_BufferedStateVector'")

    monkeypatch.setattr(sim_mod, "_state_vector_state_private", gone)
    monkeypatch.setattr(sim_mod, "_density_matrix_state_private", gone)
    q = cirq.LineQubit.range(2)
    vec = np.array([0.6, 0, 0, 0.8j], dtype=np.complex64)
    r = sim_mod._state_vector_result(cirq.ParamResolver({}), {}, q, vec)
    np.testing.assert_allclose(r.final_state_vector, vec)
    np.testing.assert_allclose(r._final_simulator_state.target_tensor.reshape(-1), vec)
    rho = np.outer(vec, vec.conj()).astype(np.complex64)
    d = sim_mod._density_matrix_result(cirq.ParamResolver({}), {}, q, rho)
    np.testing.assert_allclose(d.final_density_matrix, rho, atol=1e-7)


def _reference_confuse(bits, qubits, cmap, seed):
    cirq.StepResult._confuse_results(None, bits, qubits, cmap, seed)


@pytest.mark.parametrize(
    "cmap",
    [
        {(0, 1): np.array([[0.7, 0.1, 0.1, 0.1], [0.0, 0.9, 0.1, 0.0], [0.2, 0.2, 0.5, 0.1], [0.25, 0.25, 0.25, 0.25]])},
        # overlapping entries: the second reads the digit the first wrote
        {(0,): np.array([[0.8, 0.2], [0.3, 0.7]]), (0, 2): np.array([[0.5, 0.5, 0, 0], [0, 0.5, 0.5, 0],
                                                                       [0, 0, 0.5, 0.5], [0.5, 0, 0, 0.5]])},
    ],
)
def test_vectorised_confusion_matches_the_reference_distribution(cmap):
    q = cirq.LineQubit.range(3)
    reps = 20000
    rs = np.random.RandomState(3)
    start = rs.randint(0, 2, size=(reps, 3)).astype(np.int8)
    ours = start.copy()
    sim_mod._confuse(ours, q, cmap, np.random.RandomState(11))
    ref = start.copy()
    _reference_confuse(ref, q, cmap, 12)
    key_o = ours.astype(int) @ np.array([4, 2, 1]) + 8 * (start.astype(int) @ np.array([4, 2, 1]))
    key_r = ref.astype(int) @ np.array([4, 2, 1]) + 8 * (start.astype(int) @ np.array([4, 2, 1]))
    co = np.bincount(key_o, minlength=64)
    cr = np.bincount(key_r, minlength=64)
    keep = (co + cr) > 0
    _, p, _, _ = scipy.stats.chi2_contingency(np.stack([co[keep], cr[keep]]))
    assert p > 1e-4
