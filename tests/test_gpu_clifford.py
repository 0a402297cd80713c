"""Clifford sampling on the GPU (gbq_cliff_reference / gbq_cliff_sample)
against the tableau oracle (oracle/clifford.py, pinned to the reference) and
against the reference's own samplers (golden/golden_clifford.npz).

* The GPU reference run takes outcome 0 for every random measurement; the
  oracle run with the same rule must give the same records exactly.
* Frame samples must follow the circuit's distribution: a two-sample
  chi-square test of the joint records against the oracle's samples and
  against the reference samplers' records (p > 1e-4).
* Properties at sizes the oracle cannot reach: GHZ states of 1000 and 5000
  qubits, deterministic circuits, noise rates (binomial bounds), seeds.
"""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import clifford as C
from cirq_gb300 import workloads
from cirq_gb300.engine import Engine
from oracle import clifford as oc
from tests.test_oracle_clifford import DIST_CASES, GOLD, _joint, two_sample_pvalue

pytestmark = pytest.mark.gpu


def _eng():
    return Engine.get(0)


@pytest.mark.parametrize(
    "n,depth,seed,kw",
    [
        (5, 10, 0, dict(mid_measure=0.7, feedback=True)),
        (17, 12, 1, dict(mid_measure=0.8, resets=True, feedback=True)),
        (70, 8, 2, dict(mid_measure=1.0, resets=True, feedback=True, p=0.01)),
        (130, 6, 3, dict(mid_measure=1.0, resets=True, feedback=True)),
    ],
)
def test_reference_run_matches_oracle(n, depth, seed, kw):
    c = workloads.random_clifford_circuit(n, depth, seed, **kw)
    q = cirq.LineQubit.range(n)
    prog = C.CliffordProgram(c, q)
    ref = prog.reference(_eng())
    ops, nrec, _ = oc.program_from_circuit(cirq, c, q)
    want, _ = oc.run_shot(ops, n, nrec, prng=None, choose=lambda r: 0)
    assert np.array_equal(ref, want)


def _gpu_records(c, reps, seed, keys):
    q = sorted(c.all_qubits())
    prog = C.CliffordProgram(c, q)
    recs = prog.records(_eng(), reps, seed)
    return {k: recs[k][:, -1, :] for k in keys}


@pytest.mark.parametrize("i", range(len(DIST_CASES)))
def test_frames_match_reference_samplers_and_oracle(i):
    n, depth, seed = DIST_CASES[i]
    c = workloads.random_clifford_circuit(n, depth, seed, mid_measure=0.7, resets=True, feedback=True, p=0.02)
    names = sorted(c.all_measurement_key_names())
    reps = 2000
    gpu = _joint(_gpu_records(c, reps, 11 + i, names), names, reps)
    for sampler in ("stab", "cliff"):
        ref = {k: GOLD[f"dist_{i}_{sampler}_{k}"] for k in names}
        assert two_sample_pvalue(gpu, _joint(ref, names, reps)) > 1e-4, sampler
    q = cirq.LineQubit.range(n)
    ops, nrec, keys = oc.program_from_circuit(cirq, c, q)
    prng = np.random.RandomState(3 + i)
    mine = {k: [] for k in keys}
    for _ in range(reps):
        rec, _ = oc.run_shot(ops, n, nrec, prng=prng)
        for k, inst in keys.items():
            mine[k].append(rec[inst[-1]])
    mine = {k: np.array(v, np.uint8) for k, v in mine.items()}
    assert two_sample_pvalue(gpu, _joint(mine, names, reps)) > 1e-4


@pytest.mark.parametrize("n", [1000, 5000])
def test_ghz_properties(n):
    q = cirq.LineQubit.range(n)
    c = cirq.Circuit(cirq.H(q[0]), [cirq.CNOT(q[i], q[i + 1]) for i in range(n - 1)], cirq.measure(*q, key="m"))
    reps = 4096
    m = _gpu_records(c, reps, 5, ["m"])["m"]
    assert m.shape == (reps, n)
    assert np.all(m == m[:, :1])  # all qubits agree in every shot
    ones = int(m[:, 0].sum())
    assert abs(ones - reps / 2) < 5 * np.sqrt(reps / 4)


def test_deterministic_circuit_exact():
    q = cirq.LineQubit.range(40)
    c = cirq.Circuit(
        [cirq.X(q[i]) for i in range(0, 40, 3)],
        [cirq.CNOT(q[i], q[i + 1]) for i in range(0, 39, 2)],
        cirq.H(q[5]), cirq.S(q[5]), cirq.S(q[5]), cirq.H(q[5]),  # = X on q5
        cirq.measure(*q, key="m", invert_mask=(True,) * 3),
    )
    state = np.zeros(40, np.uint8)
    for i in range(0, 40, 3):
        state[i] ^= 1
    for i in range(0, 39, 2):
        state[i + 1] ^= state[i]
    state[5] ^= 1
    state[:3] ^= 1
    m = _gpu_records(c, 1000, 9, ["m"])["m"]
    assert np.all(m == state[None, :])


def test_noise_rates():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.bit_flip(0.1).on(q[0]),
        cirq.H(q[1]), cirq.phase_flip(0.3).on(q[1]), cirq.H(q[1]),
        cirq.depolarize(0.3).on(q[2]),
        cirq.measure(*q, key="m"),
    )
    reps = 200_000
    m = _gpu_records(c, reps, 21, ["m"])["m"]
    for col, p in ((0, 0.1), (1, 0.3), (2, 0.2)):  # depolarize(p): X or Y flip with 2p/3
        k = int(m[:, col].sum())
        assert abs(k - p * reps) < 5 * np.sqrt(reps * p * (1 - p)), (col, k)


def test_reset_and_feedback_semantics():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(
        cirq.H(q[0]), cirq.measure(q[0], key="a"),
        cirq.X(q[0]).with_classical_controls("a"),  # active reset of q0
        cirq.H(q[1]), cirq.CNOT(q[1], q[0]), cirq.reset(q[1]),
        cirq.measure(q[0], key="b"), cirq.measure(q[1], key="c"),
    )
    reps = 20_000
    r = _gpu_records(c, reps, 4, ["a", "b", "c"])
    assert np.all(r["c"] == 0)
    for k in ("a", "b"):
        assert abs(int(r[k].sum()) - reps / 2) < 5 * np.sqrt(reps / 4)


def test_seeds_repeat_and_differ():
    c = workloads.random_clifford_circuit(12, 8, 2, mid_measure=0.5)
    q = sorted(c.all_qubits())
    prog = C.CliffordProgram(c, q)
    a = prog.sample_records(_eng(), 5000, 42)
    b = prog.sample_records(_eng(), 5000, 42)
    d = prog.sample_records(_eng(), 5000, 43)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, d)


def test_drop_in_samplers_match_reference_shapes():
    c = workloads.random_clifford_circuit(6, 6, 7, mid_measure=1.0, resets=True, feedback=True)
    reps = 300
    ours = C.StabilizerSampler(seed=1).run(c, repetitions=reps)
    ref = cirq.StabilizerSampler(seed=1).run(c, repetitions=reps)
    assert ours.measurements.keys() == ref.measurements.keys()
    for k in ref.measurements:
        assert ours.measurements[k].shape == ref.measurements[k].shape
        assert ours.measurements[k].dtype == ref.measurements[k].dtype
    ours = C.CliffordSimulator(seed=1).run(c, repetitions=reps)
    ref = cirq.CliffordSimulator(seed=1).run(c, repetitions=reps)
    for k in ref.records:
        assert ours.records[k].shape == ref.records[k].shape


def test_sample_routes_wide_clifford_circuits():
    # 200 qubits: no state vector fits; cirq.sample would use its tableau
    c = workloads.random_clifford_circuit(200, 4, 8, mid_measure=0.5)
    r = cirq_gb300.sample(c, repetitions=64, seed=3)
    assert r.measurements["m"].shape == (64, 200)


def test_sweep_and_non_frameable_fallback():
    q = cirq.LineQubit.range(3)
    import sympy

    t = sympy.Symbol("t")
    c = cirq.Circuit(cirq.X(q[0]) ** t, cirq.CNOT(q[0], q[1]), cirq.measure(*q, key="m"))
    res = C.CliffordSimulator(seed=2).run_sweep(c, cirq.Points("t", [0, 1]), repetitions=50)
    assert np.all(res[0].measurements["m"] == 0)
    assert np.all(res[1].measurements["m"] == [1, 1, 0])
    # a T gate is not Clifford: the sampler runs it on the state-vector path
    c2 = cirq.Circuit(cirq.H(q[0]), cirq.T(q[0]), cirq.H(q[0]), cirq.measure(q[0], key="m"))
    r = C.StabilizerSampler(seed=3).run(c2, repetitions=2000)
    p1 = abs((1 - np.exp(1j * np.pi / 4)) / 2) ** 2
    assert abs(r.measurements["m"].mean() - p1) < 5 * np.sqrt(p1 * (1 - p1) / 2000)


def test_word_and_byte_outputs_agree():
    c = workloads.random_clifford_circuit(40, 6, 9, mid_measure=1.0, resets=True, p=0.01)
    prog = C.CliffordProgram(c, sorted(c.all_qubits()))
    reps = 3000  # not a multiple of 32
    words = prog.sample_words(_eng(), reps, 77)
    bits = np.unpackbits(words.view(np.uint8), axis=1, bitorder="little")[:, :reps].T
    assert np.array_equal(bits, prog.sample_records(_eng(), reps, 77))


def test_small_noise_rate_and_lane_uniformity():
    # rare errors are placed by geometric skipping: the rate and the spread
    # over the 32 shot positions of a word must match independent draws
    q = cirq.LineQubit.range(2)
    p = 2e-3
    c = cirq.Circuit(cirq.bit_flip(p).on(q[0]), cirq.H(q[1]), cirq.phase_flip(0.05).on(q[1]), cirq.H(q[1]),
                     cirq.measure(*q, key="m"))
    reps = 1 << 22
    m = _gpu_records(c, reps, 31, ["m"])["m"]
    for col, pr in ((0, p), (1, 0.05)):
        k = int(m[:, col].sum())
        assert abs(k - pr * reps) < 5 * np.sqrt(reps * pr * (1 - pr)), (col, k)
    lanes = np.bincount(np.nonzero(m[:, 0])[0] % 32, minlength=32)
    expect = lanes.sum() / 32
    chi2 = float(((lanes - expect) ** 2 / expect).sum())
    from scipy.stats import chi2 as chi2_dist

    assert chi2_dist.sf(chi2, 31) > 1e-4
