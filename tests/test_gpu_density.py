"""Density-matrix simulation on the GPU vs the reference's DensityMatrixSimulator."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import workloads
from oracle.circuits import simulate_density_matrix

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_density.py", "golden/golden.npz"))
TOL = 1e-5


def _check_rho(rho):
    assert abs(np.trace(rho) - 1) < 1e-5
    np.testing.assert_allclose(rho, rho.conj().T, atol=1e-6)


def test_noisy_layers_vs_golden():
    c = workloads.noisy_layer_circuit(4, 4, seed=2, p=0.05, gamma=0.1)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisy_n4_d4"], atol=TOL)
    _check_rho(rho)


def test_noise_model_vs_golden():
    c = workloads.random_layer_circuit(3, 3, seed=5)
    rho = cirq_gb300.DensityMatrixSimulator(noise=cirq.depolarize(0.02)).simulate(c).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisemodel_n3"], atol=TOL)


def test_channel_zoo_vs_golden():
    qd = cirq.LineQubit.range(3)
    cg = cirq.Circuit(
        cirq.H(qd[0]),
        cirq.CNOT(qd[0], qd[1]),
        cirq.generalized_amplitude_damp(0.3, 0.2).on(qd[1]),
        cirq.phase_damp(0.25).on(qd[0]),
        cirq.bit_flip(0.1).on(qd[2]),
        cirq.asymmetric_depolarize(0.05, 0.1, 0.15).on(qd[2]),
        cirq.CZ(qd[1], qd[2]) ** 0.3,
        cirq.depolarize(0.1, n_qubits=2).on(qd[0], qd[2]),
        cirq.reset(qd[1]),
    )
    rho = cirq_gb300.DensityMatrixSimulator().simulate(cg).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_channels_n3"], atol=TOL)


def test_known_noisy_expectations():
    """density_matrix_simulator_test.py:894-905 known answers."""
    q0 = cirq.LineQubit(0)
    psums = [cirq.Z(q0), cirq.X(q0)]
    sim = cirq_gb300.DensityMatrixSimulator()
    r = sim.simulate_expectation_values(cirq.Circuit(cirq.X(q0), cirq.amplitude_damp(gamma=0.1).on(q0)), psums)
    np.testing.assert_allclose(np.real(r), GOLD["known_dm_ad"], atol=1e-6)
    r = sim.simulate_expectation_values(cirq.Circuit(cirq.H(q0), cirq.depolarize(p=0.3).on(q0)), psums)
    np.testing.assert_allclose(np.real(r), GOLD["known_dm_dep"], atol=1e-6)


@pytest.mark.parametrize("n", [7, 9])
def test_noisy_layers_vs_oracle(n):
    c = workloads.noisy_layer_circuit(n, 6, seed=n, p=1e-2, gamma=2e-2)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    want = simulate_density_matrix(c)
    assert np.max(np.abs(rho - want)) < TOL
    _check_rho(rho)


def test_dm_sampling_chi2():
    import scipy.stats

    c = workloads.noisy_layer_circuit(5, 4, seed=3, p=0.05, gamma=0.1)
    q = sorted(c.all_qubits())
    want = np.real(np.diag(simulate_density_matrix(c)))
    reps = 20000
    res = cirq_gb300.DensityMatrixSimulator(seed=5).run(c + cirq.measure(*q, key="m"), repetitions=reps)
    idx = res.measurements["m"].dot(1 << np.arange(4, -1, -1))
    counts = np.bincount(idx, minlength=32)
    keep = want * reps >= 5
    obs = np.concatenate([counts[keep], [counts[~keep].sum()]])
    exp = np.concatenate([want[keep], [want[~keep].sum()]]) * reps
    if exp[-1] == 0:
        obs, exp = obs[:-1], exp[:-1]
    assert scipy.stats.chisquare(obs, exp).pvalue > 1e-4


def test_bench_size_noisy_density_matrix_properties():
    """The 13-qubit noisy-layers workload (rho = 2^26 amplitudes): trace one,
    Hermitian, positive diagonal, and the same result on a rerun."""
    c = workloads.noisy_layer_circuit(13, 16, seed=0, p=1e-3, gamma=5e-3)
    sim = cirq_gb300.DensityMatrixSimulator()
    rho = sim.simulate(c).final_density_matrix
    assert abs(np.trace(rho) - 1) < 1e-5
    assert np.max(np.abs(rho - rho.conj().T)) < 1e-6
    assert np.real(np.diag(rho)).min() > -1e-6
    rho2 = sim.simulate(c).final_density_matrix
    assert np.array_equal(rho, rho2)


def test_noise_placement_matches_the_reference():
    """Noise model on a parameterized circuit (prefix / suffix noised apart,
    as the reference's density-matrix simulator does) against the reference's
    own result, and run() with a terminal two-qubit measurement (noise after
    the measurement moment acts before sampling) against the exact
    distribution of the same placement."""
    import sympy
    import scipy.stats

    import make_zoo

    pc, r = make_zoo.golden_module()._noisy_param_circuit(cirq, sympy)
    rho = cirq_gb300.DensityMatrixSimulator(noise=cirq.amplitude_damp(0.2)).simulate(pc, r).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisy_param_split"], atol=TOL)

    q = cirq.LineQubit.range(2)
    cm = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(*q), cirq.ry(0.4).on(q[1]), cirq.measure(*q, key="m"))
    sim = cirq_gb300.DensityMatrixSimulator(noise=cirq.amplitude_damp(0.3), seed=6)
    placed = sim._reference_noisy_circuit(cm, "run")
    body = cirq.Circuit(op for op in placed.all_operations() if not cirq.is_measurement(op))
    from oracle.circuits import simulate_density_matrix as oracle_dm

    p = np.real(np.diag(oracle_dm(body, qubit_order=q)))
    reps = 20000
    bits = sim.run(cm, repetitions=reps).measurements["m"]
    counts = np.bincount(bits[:, 0].astype(int) * 2 + bits[:, 1], minlength=4)
    assert scipy.stats.chisquare(counts, p / p.sum() * reps).pvalue > 1e-3
