"""Expectation values on the GPU vs the reference's golden values and the oracle."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import workloads
from oracle.circuits import expectation_state_vector, simulate_state_vector

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_expectation.py", "golden/golden.npz"))
TOL = 1e-4


def test_pauli_terms_on_golden_state():
    """Per-term and summed <psi|P|psi> on the reference's random state
    (values produced by PauliString/PauliSum.expectation_from_state_vector)."""
    n = 6
    psi = GOLD["pauli_n6_state"].astype(np.complex64)
    ham = workloads.random_pauli_hamiltonian(n, 20, seed=12, min_w=1, max_w=4)
    qs = cirq.LineQubit.range(n)
    sim = cirq_gb300.Simulator()
    vals = sim.simulate_expectation_values(cirq.Circuit(cirq.I.on_each(*qs)), list(ham), initial_state=psi)
    np.testing.assert_allclose(vals, GOLD["pauli_n6_terms_expect"], atol=TOL)
    tot = sim.simulate_expectation_values(cirq.Circuit(cirq.I.on_each(*qs)), ham, initial_state=psi)
    np.testing.assert_allclose(tot[0], GOLD["pauli_n6_sum_expect"], atol=TOL)


def test_qaoa_sweep_vs_golden():
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(8, 4, seed=7)
    pts = GOLD["qaoa_n8_p4_points"]
    res = [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]
    vals = cirq_gb300.Simulator().simulate_expectation_values_sweep(circuit, obs, res)
    np.testing.assert_allclose([v[0] for v in vals], GOLD["qaoa_n8_p4_expect"], atol=TOL)


def test_hamiltonian_on_random_circuit_vs_oracle():
    c = workloads.random_layer_circuit(16, 8, seed=21)
    q = sorted(c.all_qubits())
    ham = workloads.random_pauli_hamiltonian(16, 40, seed=22)
    got = cirq_gb300.Simulator().simulate_expectation_values(c, ham)[0]
    psi = simulate_state_vector(c)
    want = expectation_state_vector(psi, ham, {x: i for i, x in enumerate(q)})
    assert abs(got - want) < TOL


def test_terminal_measurement_guard():
    q0 = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.X(q0), cirq.measure(q0))
    with pytest.raises(ValueError, match="terminal measurements"):
        cirq_gb300.Simulator().simulate_expectation_values(c, cirq.Z(q0))
    v = cirq_gb300.Simulator().simulate_expectation_values(c, cirq.Z(q0), permit_terminal_measurements=True)
    assert abs(v[0] + 1) < 1e-6


def test_compute_amplitudes():
    c = workloads.random_layer_circuit(10, 20, seed=1)
    amps = cirq_gb300.Simulator().compute_amplitudes(c, [0, 5, 1023])
    want = GOLD["layers_n10_d20_s1_c128"][[0, 5, 1023]]
    np.testing.assert_allclose(amps, want, atol=1e-5)
