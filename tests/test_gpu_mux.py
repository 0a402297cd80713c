"""Module-level entry points (``cirq_gb300.sample`` / ``sample_sweep`` /
``final_state_vector`` / ``final_density_matrix``) on the GPU, against the
oracle, analytic results and the exact sample distribution."""

import numpy as np
import pytest
import scipy.stats
import sympy

import cirq
import cirq_gb300
from cirq_gb300 import mux, workloads
from oracle.circuits import simulate_density_matrix, simulate_state_vector

pytestmark = pytest.mark.gpu


def test_final_state_vector_vs_oracle():
    c = workloads.random_layer_circuit(10, 8, seed=4)
    got = cirq_gb300.final_state_vector(c)
    want = simulate_state_vector(c)
    assert got.dtype == np.complex64
    assert np.max(np.abs(got - want)) < 2e-6


def test_final_state_vector_options():
    q = cirq.LineQubit.range(3)
    t = sympy.Symbol("t")
    c = cirq.Circuit(cirq.rx(t).on(q[0]), cirq.CNOT(q[0], q[1]), cirq.H(q[2]), cirq.measure(*q, key="m"))
    order = [q[2], q[0], q[1]]
    got = cirq_gb300.final_state_vector(
        c, param_resolver={"t": 0.7}, qubit_order=order, initial_state=1, ignore_terminal_measurements=True
    )
    want = simulate_state_vector(c, {"t": 0.7}, qubit_order=order, initial_state=1)
    assert np.max(np.abs(got - want)) < 2e-6
    # a gate is accepted as a program
    np.testing.assert_allclose(cirq_gb300.final_state_vector(cirq.H), [2**-0.5, 2**-0.5], atol=1e-6)


def test_final_density_matrix_pure_noisy_and_measured():
    q = cirq.LineQubit.range(4)
    c = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(0.4).on(q[2]), cirq.CZ(q[2], q[3]))
    # pure: state-vector path and an outer product
    psi = simulate_state_vector(c)
    got = cirq_gb300.final_density_matrix(c)
    assert np.max(np.abs(got - np.outer(psi, psi.conj()))) < 2e-6
    # noisy: the density-matrix simulator
    noise = cirq.depolarize(0.05)
    got = cirq_gb300.final_density_matrix(c, noise=noise)
    want = simulate_density_matrix(c, noise=noise)
    assert np.max(np.abs(got - want)) < 2e-6
    # terminal measurements dephase the measured qubits (the oracle skips
    # keyed channels, so it gets the unkeyed form; tests/test_mux.py checks
    # that form against cirq.dephase_measurements channel by channel)
    cm = c + cirq.measure(q[0], q[2], key="m")
    got = cirq_gb300.final_density_matrix(cm)
    want = simulate_density_matrix(mux._dephase(cm))
    assert np.max(np.abs(got - want)) < 2e-6


def test_final_density_matrix_classical_control_is_deferred_and_traced_out():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0], key="a"), cirq.X(q[1]).with_classical_controls("a"))
    got = cirq_gb300.final_density_matrix(c)
    want = np.zeros((4, 4))
    want[0, 0] = want[3, 3] = 0.5
    assert got.shape == (4, 4)
    assert np.max(np.abs(got - want)) < 2e-6


def test_final_density_matrix_conditioned_on_sampled_results():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0], key="a"), cirq.CNOT(q[0], q[1]))
    rho = cirq_gb300.final_density_matrix(c, ignore_measurement_results=False, seed=3)
    # collapsed: |00><00| or |11><11|
    diag = np.real(np.diag(rho))
    assert abs(np.trace(rho) - 1) < 1e-5
    assert (abs(diag[0] - 1) < 1e-5) or (abs(diag[3] - 1) < 1e-5)


def _chi2_p(bits: np.ndarray, probs: np.ndarray) -> float:
    n = bits.shape[1]
    idx = bits.astype(np.int64) @ (1 << np.arange(n - 1, -1, -1))
    counts = np.bincount(idx, minlength=len(probs))
    keep = probs > 0
    exp = probs[keep] * len(idx)
    return scipy.stats.chisquare(counts[keep], exp * counts[keep].sum() / exp.sum()).pvalue


@pytest.mark.parametrize("noisy", [False, True])
def test_sample_distribution(noisy):
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(1.1).on(q[2]), cirq.measure(*q, key="m"))
    noise = cirq.amplitude_damp(0.2) if noisy else None
    res = cirq_gb300.sample(c, noise=noise, repetitions=4000, seed=11)
    # cirq.sample runs the density-matrix simulator: with noise, the noise
    # after the terminal three-qubit measurement acts before sampling
    placed = cirq_gb300.DensityMatrixSimulator(noise=noise)._reference_noisy_circuit(c, "run") if noisy else c
    body = cirq.Circuit(op for op in placed.all_operations() if not cirq.is_measurement(op))
    rho = simulate_density_matrix(body, qubit_order=q)
    probs = np.clip(np.real(np.diag(rho)), 0, None)
    assert res.measurements["m"].shape == (4000, 3)
    assert _chi2_p(res.measurements["m"], probs / probs.sum()) > 1e-3


def test_sample_sweep_one_result_per_point():
    q = cirq.LineQubit(0)
    t = sympy.Symbol("t")
    c = cirq.Circuit(cirq.rx(t).on(q), cirq.measure(q, key="m"))
    res = cirq_gb300.sample_sweep(c, cirq.Linspace("t", 0, np.pi, 3), repetitions=500, seed=2)
    assert len(res) == 3
    means = [float(r.measurements["m"].mean()) for r in res]
    assert means[0] == 0.0 and means[2] == 1.0 and 0.35 < means[1] < 0.65


GOLD = np.load(__file__.replace("test_gpu_mux.py", "golden/golden.npz"))


def test_module_helpers_vs_reference_fixtures():
    """cirq.final_density_matrix / final_state_vector results computed by the
    reference itself (tests/golden/make_golden.py)."""
    import make_zoo

    cc = make_zoo.fixture_circuit("_classical_control_circuit")
    got = cirq_gb300.final_density_matrix(cc)
    assert np.max(np.abs(got - GOLD["mux_fdm_classical_control"])) < 2e-6
    meas = make_zoo.fixture_circuit("_measured_circuit")
    got = cirq_gb300.final_density_matrix(meas)
    assert np.max(np.abs(got - GOLD["mux_fdm_dephased"])) < 2e-6
    got = cirq_gb300.final_density_matrix(meas, noise=cirq.amplitude_damp(0.1))
    assert np.max(np.abs(got - GOLD["mux_fdm_dephased_noisy"])) < 2e-6
    q = sorted(meas.all_qubits())
    got = cirq_gb300.final_state_vector(meas, ignore_terminal_measurements=True, qubit_order=q[::-1])
    assert np.max(np.abs(got - GOLD["mux_fsv_ignore_terminal"])) < 2e-6
    wide = make_zoo.fixture_circuit("_wide_controlled_circuit")
    got = cirq_gb300.Simulator().simulate(wide).final_state_vector
    assert np.max(np.abs(got - GOLD["wide_controlled_c128"])) < 2e-6
