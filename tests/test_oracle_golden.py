"""Pins the CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py runs quantumlib/Cirq's simulators)."""

import numpy as np
import pytest

import cirq
from cirq_gb300 import workloads
from oracle import circuits as oc
from oracle.statevector import probabilities_by_indices, renormalize_like_cirq, sample_from_probs

GOLD = np.load(__file__.replace("test_oracle_golden.py", "golden/golden.npz"))


@pytest.mark.parametrize("n,d,s", [(10, 20, 1), (12, 8, 2), (5, 6, 3)])
def test_state_vectors(n, d, s):
    c = workloads.random_layer_circuit(n, d, s)
    np.testing.assert_allclose(oc.simulate_state_vector(c), GOLD[f"layers_n{n}_d{d}_s{s}_c128"], atol=1e-12)


def test_qubit_order_and_initial_state():
    c = workloads.random_layer_circuit(6, 5, 4)
    q = sorted(c.all_qubits())
    got = oc.simulate_state_vector(c, qubit_order=q[::-1], initial_state=5)
    np.testing.assert_allclose(got, GOLD["layers_n6_d5_s4_reversed_init5"], atol=1e-12)


def test_gate_zoo():
    import make_zoo

    np.testing.assert_allclose(oc.simulate_state_vector(make_zoo.gate_zoo()), GOLD["zoo_c128"], atol=1e-12)


def test_density_matrices():
    c = workloads.noisy_layer_circuit(4, 4, seed=2, p=0.05, gamma=0.1)
    np.testing.assert_allclose(oc.simulate_density_matrix(c), GOLD["dm_noisy_n4_d4"], atol=1e-12)
    c = workloads.random_layer_circuit(3, 3, seed=5)
    np.testing.assert_allclose(
        oc.simulate_density_matrix(c, noise=cirq.depolarize(0.02)), GOLD["dm_noisemodel_n3"], atol=1e-12
    )


def test_qaoa_expectations():
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(8, 4, seed=7)
    pts = GOLD["qaoa_n8_p4_points"]
    for p, want in zip(pts, GOLD["qaoa_n8_p4_expect"]):
        r = {**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}
        assert abs(oc.expectation_of_circuit(circuit, obs, r) - want) < 1e-10


def test_hea_energy_and_gradients():
    circuit, symbols, _ = workloads.hea_circuit(5, 2, seed=9)
    ham = workloads.random_pauli_hamiltonian(5, 12, seed=10)
    values = GOLD["hea_n5_l2_values"]
    e = oc.expectation_of_circuit(circuit, ham, dict(zip(symbols, values))).real
    assert abs(e - float(GOLD["hea_n5_l2_energy"])) < 1e-10
    fd = oc.finite_difference_gradient(circuit, ham, symbols, values, h=1e-4)
    np.testing.assert_allclose(fd, GOLD["hea_n5_l2_grad_fd"], atol=1e-7)
    # parameter shift is exact for rx/rz; it agrees with central differences
    np.testing.assert_allclose(GOLD["hea_n5_l2_grad_ps"], GOLD["hea_n5_l2_grad_fd"], atol=1e-6)


def test_pauli_expectations():
    psi = GOLD["pauli_n6_state"]
    ham = workloads.random_pauli_hamiltonian(6, 20, seed=12, min_w=1, max_w=4)
    qmap = {q: i for i, q in enumerate(cirq.LineQubit.range(6))}
    terms = [oc.expectation_state_vector(psi, ps, qmap) for ps in ham]
    np.testing.assert_allclose(terms, GOLD["pauli_n6_terms_expect"], atol=1e-12)
    assert abs(oc.expectation_state_vector(psi, ham, qmap) - GOLD["pauli_n6_sum_expect"]) < 1e-12


@pytest.mark.parametrize("idx", [[0, 1, 2, 3, 4, 5], [2], [4, 1], [5, 0, 3]])
def test_marginal_probabilities(idx):
    probs = np.abs(GOLD["pauli_n6_state"]) ** 2
    got = probabilities_by_indices(probs, idx, 6)
    np.testing.assert_allclose(got, GOLD["probs_n6_" + "_".join(map(str, idx))], atol=1e-14)


def test_inverse_cdf_sampling_is_unbiased():
    p = np.array([0.1, 0.0, 0.6, 0.3])
    u = np.random.RandomState(0).random_sample(200000)
    counts = np.bincount(sample_from_probs(p, u), minlength=4) / len(u)
    np.testing.assert_allclose(counts, p, atol=5e-3)
    assert counts[1] == 0


def test_renormalization_rule_matches_reference_c64():
    """The reference's complex64 final states went through the same rule."""
    for n, d, s in [(10, 20, 1), (12, 8, 2)]:
        v64 = GOLD[f"layers_n{n}_d{d}_s{s}_c64"]
        np.testing.assert_allclose(np.linalg.norm(renormalize_like_cirq(v64)), 1.0, atol=1e-6)


def test_final_density_matrix_fixtures():
    """cirq.final_density_matrix / final_state_vector fixtures: the oracle's
    arithmetic on circuits prepared by the package's host-side transforms
    (dephasing with the reference's transformer, noise placed where the
    reference's density-matrix simulator places it, keys dropped)."""
    import make_zoo
    from cirq_gb300 import DensityMatrixSimulator
    from cirq_gb300.mux import _dephase, _unkey

    meas = make_zoo.fixture_circuit("_measured_circuit")
    np.testing.assert_allclose(oc.simulate_density_matrix(_dephase(meas)), GOLD["mux_fdm_dephased"], atol=1e-12)
    sim = DensityMatrixSimulator(noise=cirq.amplitude_damp(0.1))
    noisy = sim._reference_noisy_circuit(cirq.dephase_measurements(meas), "simulate")
    np.testing.assert_allclose(oc.simulate_density_matrix(_unkey(noisy)), GOLD["mux_fdm_dephased_noisy"], atol=1e-12)
    q = sorted(meas.all_qubits())
    np.testing.assert_allclose(
        oc.simulate_state_vector(meas, qubit_order=q[::-1]), GOLD["mux_fsv_ignore_terminal"], atol=1e-12
    )
    # classical control: deferred to ancillas, dephased, ancillas traced out
    cc = make_zoo.fixture_circuit("_classical_control_circuit")
    deferred = _dephase(cirq.defer_measurements(cc))
    rho = oc.simulate_density_matrix(deferred)
    n = len(cc.all_qubits())
    m = len(deferred.all_qubits())
    reduced = cirq.partial_trace(rho.reshape((2,) * (2 * m)), list(range(n))).reshape(2**n, 2**n)
    np.testing.assert_allclose(reduced, GOLD["mux_fdm_classical_control"], atol=1e-12)


def test_wide_controlled_gates():
    import make_zoo

    c = make_zoo.fixture_circuit("_wide_controlled_circuit")
    np.testing.assert_allclose(oc.simulate_state_vector(c), GOLD["wide_controlled_c128"], atol=1e-12)


def test_qudit_circuits():
    """Qids of dimensions 2..5: mixed-radix states and qudit channels."""
    import make_zoo

    mg = make_zoo.golden_module()
    c, order = mg._qudit_circuit(cirq)
    got = oc.simulate_state_vector(c, qubit_order=order, initial_state=17)
    np.testing.assert_allclose(got, GOLD["qudit_sv_c128"], atol=1e-12)
    rho = oc.simulate_density_matrix(mg._qudit_noisy_circuit(cirq))
    np.testing.assert_allclose(rho, GOLD["qudit_dm_c128"], atol=1e-12)


def test_noise_placement_of_the_density_matrix_simulator():
    """Noise placed by the package's host-side rule (prefix / suffix split of
    the reference's density-matrix simulator) + the oracle's arithmetic
    reproduce the reference: simulate() of a parameterized noisy circuit
    (golden), and run()'s sample distribution with a terminal two-qubit
    measurement (the reference's own samples, chi-squared)."""
    import sympy
    import scipy.stats

    import make_zoo
    from cirq_gb300 import DensityMatrixSimulator

    make_golden = make_zoo.golden_module()

    pc, r = make_golden._noisy_param_circuit(cirq, sympy)
    sim = DensityMatrixSimulator(noise=cirq.amplitude_damp(0.2))
    got = oc.simulate_density_matrix(sim._reference_noisy_circuit(pc, "simulate"), r)
    np.testing.assert_allclose(got, GOLD["dm_noisy_param_split"], atol=1e-12)

    q = cirq.LineQubit.range(2)
    cm = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(*q), cirq.ry(0.4).on(q[1]), cirq.measure(*q, key="m"))
    noise = cirq.amplitude_damp(0.3)
    ours = DensityMatrixSimulator(noise=noise)._reference_noisy_circuit(cm, "run")
    body = cirq.Circuit(op for op in ours.all_operations() if not cirq.is_measurement(op))
    p = np.real(np.diag(oc.simulate_density_matrix(body, qubit_order=q)))
    reps = 40000
    res = cirq.DensityMatrixSimulator(noise=noise, seed=5).run(cm, repetitions=reps)
    bits = res.measurements["m"]
    counts = np.bincount(bits[:, 0] * 2 + bits[:, 1], minlength=4)
    assert scipy.stats.chisquare(counts, p / p.sum() * reps).pvalue > 1e-3

