"""Qudits (qids of dimension > 2) on the GPU: the reference's golden states
for a circuit over qids of dimensions 2..5 (state vector, custom qubit order
and initial state) and a noisy qutrit/ququart circuit (density matrix), and
run() samples of qudit levels against the golden (density matrix) and the
oracle's (state vector) probabilities."""

import numpy as np
import pytest

import cirq
import cirq_gb300
import make_zoo
from oracle.circuits import simulate_state_vector

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_qudits.py", "golden/golden.npz"))
MG = make_zoo.golden_module()


def test_state_vector_vs_reference_golden():
    c, order = MG._qudit_circuit(cirq)
    res = cirq_gb300.Simulator().simulate(c, qubit_order=order, initial_state=17)
    np.testing.assert_allclose(res.final_state_vector, GOLD["qudit_sv_c128"], atol=1e-5)
    assert cirq.qid_shape(res) == tuple(q.dimension for q in order)


def test_density_matrix_vs_reference_golden():
    rho = cirq_gb300.DensityMatrixSimulator().simulate(MG._qudit_noisy_circuit(cirq)).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["qudit_dm_c128"], atol=1e-5)


@pytest.mark.parametrize("dm", [False, True])
def test_level_samples_vs_golden_probabilities(dm):
    if dm:
        c = MG._qudit_noisy_circuit(cirq)
        probs = np.real(np.diagonal(GOLD["qudit_dm_c128"]))
    else:
        c, _ = MG._qudit_circuit(cirq)
        probs = np.abs(simulate_state_vector(c)) ** 2
    qids = sorted(c.all_qubits())
    dims = [q.dimension for q in qids]
    c = c + cirq.measure(*qids, key="z")
    sim = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=7)
    reps = 20000
    rec = sim.run(c, repetitions=reps).records["z"][:, 0, :].astype(np.int64)
    assert rec.shape == (reps, len(qids))
    assert all(rec[:, j].max() < d for j, d in enumerate(dims))
    codes = np.ravel_multi_index(rec.T, dims)
    hist = np.bincount(codes, minlength=len(probs)) / reps
    assert 0.5 * np.abs(hist - probs / probs.sum()).sum() < 0.03
