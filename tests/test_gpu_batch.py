"""Batched sweeps (points evolved together; one persistent launch over mixed
widths) vs the reference and the oracle."""

import numpy as np
import pytest

import cirq
from cirq_gb300 import batch, workloads
from oracle.circuits import expectation_of_circuit

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_batch.py", "golden/golden.npz"))
TOL = 1e-4


def _resolvers(gammas, betas, pts):
    return [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_qaoa_vs_golden(persistent):
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(8, 4, seed=7)
    pts = GOLD["qaoa_n8_p4_points"]
    (vals,) = batch.simulate_expectation_values_batch([(circuit, obs, _resolvers(gammas, betas, pts))],
                                                      persistent=persistent)
    np.testing.assert_allclose(vals[:, 0], GOLD["qaoa_n8_p4_expect"], atol=TOL)


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_mixed_widths_vs_oracle(persistent):
    jobs, want = [], []
    for n, npts in [(12, 6), (14, 5), (16, 4), (10, 3)]:
        circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(n, 4, seed=n)
        pts = workloads.qaoa_points(4, npts, seed=100 + n)
        res = _resolvers(gammas, betas, pts)
        jobs.append((circuit, [obs, cirq.X(cirq.LineQubit(0)) * cirq.Y(cirq.LineQubit(1))], res))
        want.append(
            [
                [expectation_of_circuit(circuit, o, r) for o in (obs, cirq.X(cirq.LineQubit(0)) * cirq.Y(cirq.LineQubit(1)))]
                for r in res[:2]
            ]
        )
    got = batch.simulate_expectation_values_batch(jobs, persistent=persistent)
    for g, w, (_, _, res) in zip(got, want, jobs):
        assert g.shape == (len(res), 2)
        np.testing.assert_allclose(g[:2], np.array(w), atol=TOL)


def test_batch_matches_sweep_api():
    import cirq_gb300

    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(14, 2, seed=3)
    pts = np.random.RandomState(0).uniform(0, 1, size=(8, 4))
    res = [cirq.ParamResolver({**dict(zip(gammas[:2], p[:2])), **dict(zip(betas[:2], p[2:]))}) for p in pts]
    (vals,) = batch.simulate_expectation_values_batch([(circuit, obs, res)])
    ref = cirq_gb300.Simulator().simulate_expectation_values_sweep(circuit, obs, res)
    np.testing.assert_allclose(vals[:, 0], [r[0] for r in ref], atol=TOL)


def test_points_path_agrees_with_persistent_kernel_at_scale():
    """1000 points of 20 qubits (chunks of points evolved together) against
    the persistent kernel: two independent execution paths, same numbers."""
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(20, 4, seed=20)
    res = _resolvers(gammas, betas, workloads.qaoa_points(4, 1000, seed=5))
    job = batch.BatchJob(circuit, [obs, cirq.X(cirq.LineQubit(3)) * cirq.Z(cirq.LineQubit(9))], res)
    (a,) = batch.simulate_expectation_values_batch([job])
    (b,) = batch.simulate_expectation_values_batch([job], persistent=True)
    assert a.shape == (1000, 2)
    np.testing.assert_allclose(a, b, atol=1e-5)
