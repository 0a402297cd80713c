"""Batched sweeps driven by the package's host logic (job pools, point
chunks, term grouping, the persistent launch's point/pass/term tables) on
the CPU emulation of the engine, against the reference's own sweep values
(golden) and the oracle.  CPU only; the GPU tests run the same host logic on
the kernels."""

import numpy as np
import pytest

import cirq
from cirq_gb300 import batch, workloads
from cpu_engine import EmuEngine
from oracle.circuits import expectation_of_circuit

GOLD = np.load(__file__.replace("test_batch_emulated.py", "golden/golden.npz"))
TOL = 1e-6


def _resolvers(gammas, betas, pts):
    p = len(gammas)
    return [cirq.ParamResolver({**dict(zip(gammas, x[:p])), **dict(zip(betas, x[p:]))}) for x in pts]


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_qaoa_vs_reference_sweep(persistent):
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(8, 4, seed=7)
    pts = GOLD["qaoa_n8_p4_points"]
    (vals,) = batch.simulate_expectation_values_batch(
        [(circuit, obs, _resolvers(gammas, betas, pts))], engine=EmuEngine(), persistent=persistent
    )
    np.testing.assert_allclose(vals[:, 0], GOLD["qaoa_n8_p4_expect"], atol=1e-5)


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_mixed_widths_vs_oracle(persistent):
    q = cirq.LineQubit.range(2)
    extra = cirq.X(q[0]) * cirq.Y(q[1])
    jobs, want = [], []
    for n, npts in [(8, 3), (12, 2), (6, 3)]:
        circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(n, 2, seed=n)
        pts = workloads.qaoa_points(2, npts, seed=100 + n)
        res = _resolvers(gammas, betas, pts)
        jobs.append((circuit, [obs, extra], res))
        want.append([[expectation_of_circuit(circuit, o, r) for o in (obs, extra)] for r in res])
    got = batch.simulate_expectation_values_batch(jobs, engine=EmuEngine(), persistent=persistent)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, np.array(w), atol=TOL)


def test_empty_jobs():
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(6, 1, seed=1)
    for persistent in (False, True):
        (vals,) = batch.simulate_expectation_values_batch([(circuit, obs, [])], engine=EmuEngine(),
                                                          persistent=persistent)
        assert vals.shape == (0, 1)


@pytest.mark.parametrize("persistent", [False, True])
def test_empty_and_nonempty_jobs_together(persistent):
    c1, g1, b1, obs1, _ = workloads.qaoa_circuit(6, 1, seed=1)
    c2, g2, b2, obs2, _ = workloads.qaoa_circuit(8, 1, seed=2)
    res2 = _resolvers(g2, b2, workloads.qaoa_points(1, 2, seed=3))
    got = batch.simulate_expectation_values_batch([(c1, [obs1, obs1], []), (c2, obs2, res2)],
                                                  engine=EmuEngine(), persistent=persistent)
    assert got[0].shape == (0, 2)
    want = [expectation_of_circuit(c2, obs2, r) for r in res2]
    np.testing.assert_allclose(got[1][:, 0], want, atol=TOL)
