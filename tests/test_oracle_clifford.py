"""The stabilizer-tableau oracle (oracle/clifford.py) against the reference's
own tableau simulation and samplers (golden/golden_clifford.npz, made by
golden/make_golden_clifford.py)."""

import collections

import numpy as np
import pytest
import scipy.stats

import cirq
from cirq_gb300 import workloads
from oracle import clifford as oc

GOLD = np.load(__file__.replace("test_oracle_clifford.py", "golden/golden_clifford.npz"))
TAB_CASES = [(4, 6, 0), (6, 10, 1), (9, 12, 2)]
MEAS_CASES = [(5, 10, 3), (7, 12, 4)]
DIST_CASES = [(5, 6, 5), (4, 8, 6)]


@pytest.mark.parametrize("i", range(len(TAB_CASES)))
def test_tableau_matches_reference(i):
    n, depth, seed = TAB_CASES[i]
    c = workloads.random_clifford_circuit(n, depth, seed, final_measure=False)
    q = cirq.LineQubit.range(n)
    ops, nrec, _ = oc.program_from_circuit(cirq, c, q)
    _, t = oc.run_shot(ops, n, nrec, prng=None, choose=lambda r: 0)
    # the reference's public arrays leave out the scratch row 2n
    assert np.array_equal(t.xs[: 2 * n], GOLD[f"tab_{i}_xs"])
    assert np.array_equal(t.zs[: 2 * n], GOLD[f"tab_{i}_zs"])
    assert np.array_equal(t.rs[: 2 * n], GOLD[f"tab_{i}_rs"])


@pytest.mark.parametrize("i", range(len(MEAS_CASES)))
def test_measurements_replay_reference(i):
    # the reference's random outcomes fed back: every outcome and the final
    # tableau must agree (rowsum, g and the measurement procedure)
    n, depth, seed = MEAS_CASES[i]
    c = workloads.random_clifford_circuit(n, depth, seed, mid_measure=0.6, feedback=True)
    q = cirq.LineQubit.range(n)
    ops, nrec, _ = oc.program_from_circuit(cirq, c, q)
    want = GOLD[f"meas_{i}_outcomes"]
    rec, t = oc.run_shot(ops, n, nrec, prng=None, choose=lambda r: int(want[r]))
    assert np.array_equal(rec, want)
    # the reference's public arrays leave out the scratch row 2n
    assert np.array_equal(t.xs[: 2 * n], GOLD[f"meas_{i}_xs"])
    assert np.array_equal(t.zs[: 2 * n], GOLD[f"meas_{i}_zs"])
    assert np.array_equal(t.rs[: 2 * n], GOLD[f"meas_{i}_rs"])


def _joint(records: dict, keys, reps):
    rows = np.concatenate([records[k].reshape(reps, -1) for k in keys], axis=1)
    return collections.Counter(map(bytes, rows))


def two_sample_pvalue(ca: collections.Counter, cb: collections.Counter) -> float:
    cats = sorted(set(ca) | set(cb))
    table = np.array([[ca.get(c, 0) for c in cats], [cb.get(c, 0) for c in cats]], dtype=float)
    keep = table.sum(axis=0) >= 10
    rest = table[:, ~keep].sum(axis=1, keepdims=True)
    table = np.concatenate([table[:, keep], rest], axis=1)
    table = table[:, table.sum(axis=0) > 0]
    if table.shape[1] < 2:
        return 1.0
    return scipy.stats.chi2_contingency(table)[1]


@pytest.mark.parametrize("i", range(len(DIST_CASES)))
def test_noisy_distribution_matches_reference_samplers(i):
    n, depth, seed = DIST_CASES[i]
    c = workloads.random_clifford_circuit(n, depth, seed, mid_measure=0.7, resets=True, feedback=True, p=0.02)
    q = cirq.LineQubit.range(n)
    ops, nrec, keys = oc.program_from_circuit(cirq, c, q)
    reps = 2000
    prng = np.random.RandomState(7 + i)
    mine = {k: [] for k in keys}
    for _ in range(reps):
        rec, _ = oc.run_shot(ops, n, nrec, prng=prng)
        for k, inst in keys.items():
            mine[k].append(rec[inst[-1]])
    mine = {k: np.array(v, np.uint8) for k, v in mine.items()}
    names = sorted(keys)
    ours = _joint(mine, names, reps)
    for sampler in ("stab", "cliff"):
        ref = {k: GOLD[f"dist_{i}_{sampler}_{k}"] for k in names}
        assert two_sample_pvalue(ours, _joint(ref, names, reps)) > 1e-4, sampler
