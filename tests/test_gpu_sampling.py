"""run() / measurement semantics on the GPU, checked statistically (chi^2)
against the exact distribution, as the reference's sampling cannot be
reproduced draw by draw (it uses RandomState.choice)."""

import numpy as np
import pytest
import scipy.stats

import cirq
import cirq_gb300
from cirq_gb300 import workloads
from oracle.circuits import simulate_state_vector
from oracle.statevector import probabilities_by_indices

pytestmark = pytest.mark.gpu


def _chi2_pvalue(counts, probs, reps):
    keep = probs * reps >= 5
    obs = np.concatenate([counts[keep], [counts[~keep].sum()]])
    exp = np.concatenate([probs[keep], [probs[~keep].sum()]]) * reps
    if exp[-1] == 0:
        obs, exp = obs[:-1], exp[:-1]
    return scipy.stats.chisquare(obs, exp).pvalue


def test_run_all_qubits_chi2():
    c = workloads.random_layer_circuit(8, 6, seed=11)
    q = sorted(c.all_qubits())
    psi = simulate_state_vector(c)
    probs = np.abs(psi) ** 2
    reps = 20000
    res = cirq_gb300.Simulator(seed=1).run(c + cirq.measure(*q, key="m"), repetitions=reps)
    bits = res.measurements["m"]
    assert bits.shape == (reps, 8)
    idx = bits.dot(1 << np.arange(7, -1, -1))
    counts = np.bincount(idx, minlength=256)
    assert _chi2_pvalue(counts, probs, reps) > 1e-4


def test_run_subset_invert_mask_and_keys():
    c = workloads.random_layer_circuit(6, 5, seed=12)
    q = sorted(c.all_qubits())
    psi = simulate_state_vector(c)
    reps = 20000
    circ = c + cirq.Moment(
        cirq.measure(q[4], q[1], key="a", invert_mask=(True, False)), cirq.measure(q[2], key="b")
    )
    res = cirq_gb300.Simulator(seed=2).run(circ, repetitions=reps)
    a = res.measurements["a"]
    b = res.measurements["b"]
    assert a.shape == (reps, 2) and b.shape == (reps, 1)
    joint = np.stack([1 - a[:, 0], a[:, 1], b[:, 0]], axis=1)
    idx = joint.dot([4, 2, 1])
    counts = np.bincount(idx, minlength=8)
    probs = probabilities_by_indices(np.abs(psi) ** 2, [4, 1, 2], 6)
    assert _chi2_pvalue(counts, probs, reps) > 1e-4


def test_run_records_shape_and_sweep():
    q0, q1 = cirq.LineQubit.range(2)
    import sympy

    t = sympy.Symbol("t")
    c = cirq.Circuit(cirq.X(q0) ** t, cirq.measure(q0, q1, key="m"))
    results = cirq_gb300.Simulator().run_sweep(c, cirq.Points("t", [0, 1]), repetitions=7)
    assert results[0].records["m"].shape == (7, 1, 2)
    np.testing.assert_array_equal(results[0].measurements["m"], np.zeros((7, 2)))
    np.testing.assert_array_equal(results[1].measurements["m"], np.tile([1, 0], (7, 1)))


def test_run_no_measurements_raises():
    q0 = cirq.LineQubit(0)
    with pytest.raises(ValueError, match="no measurements"):
        cirq_gb300.Simulator().run(cirq.Circuit(cirq.X(q0)))


def test_simulate_with_terminal_measurement_collapses():
    q0, q1 = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q0), cirq.CNOT(q0, q1), cirq.measure(q0, q1, key="m"))
    for seed in range(4):
        r = cirq_gb300.Simulator(seed=seed).simulate(c)
        m = r.measurements["m"]
        assert m[0] == m[1]
        want = np.zeros(4, complex)
        want[3 * m[0]] = 1
        np.testing.assert_allclose(r.final_state_vector, want, atol=1e-6)


def test_mid_circuit_measurement_runs_per_repetition():
    q0 = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.measure(q0, key="a"), cirq.X(q0), cirq.measure(q0, key="b"))
    res = cirq_gb300.Simulator().run(c, repetitions=3)
    assert res.records["a"].tolist() == [[[0]]] * 3 and res.records["b"].tolist() == [[[1]]] * 3


def test_large_state_sampling_chi2_marginal():
    """20 qubits (the run() workload size), marginal of 4 qubits."""
    c = workloads.random_layer_circuit(20, 6, seed=13)
    q = sorted(c.all_qubits())
    psi = simulate_state_vector(c)
    reps = 10000
    res = cirq_gb300.Simulator(seed=3).run(c + cirq.measure(*q, key="m"), repetitions=reps)
    bits = res.measurements["m"]
    assert bits.shape == (reps, 20)
    sub = [0, 7, 13, 19]
    idx = bits[:, sub].dot([8, 4, 2, 1])
    counts = np.bincount(idx, minlength=16)
    probs = probabilities_by_indices(np.abs(psi) ** 2, sub, 20)
    assert _chi2_pvalue(counts, probs, reps) > 1e-4
