"""Batched density-matrix trajectories (trajectories.run_batched_dm) on the
emulated engine: run() of density-matrix circuits with mid-circuit
measurements evolves every repetition's density matrix together, and its
records match the reference DensityMatrixSimulator's in distribution."""

import numpy as np
import pytest
import scipy.stats

import cirq
import cirq_gb300
import cirq_gb300.simulator as sim_mod
from cirq_gb300 import trajectories as traj
from cpu_engine import EmuEngine


@pytest.fixture
def emu(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    return eng


def _circuit():
    q = cirq.LineQubit.range(4)
    return cirq.Circuit(
        cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(0.8).on(q[2]),
        cirq.amplitude_damp(0.3).on(q[1]), cirq.depolarize(0.1).on(q[2]),
        cirq.measure(q[1], key="a"),
        cirq.CNOT(q[1], q[3]), cirq.H(q[2]), cirq.CZ(q[2], q[3]),
        cirq.measure(q[2], q[3], key="b", invert_mask=(True, False)),
        cirq.X(q[0]) ** 0.3, cirq.phase_damp(0.2).on(q[0]),
        cirq.measure(*q, key="all"),
    ), q


def _keys(rec):
    bits = [rec[k][:, 0, :] for k in ("a", "b", "all")]
    flat = np.concatenate(bits, axis=1).astype(np.int64)
    return flat @ (1 << np.arange(flat.shape[1] - 1, -1, -1))


def test_batched_dm_runner_is_used_and_matches_the_reference(emu, monkeypatch):
    c, q = _circuit()
    reps = 3000
    calls = []
    orig = traj.run_batched_dm

    def spy(*a, **k):
        out = orig(*a, **k)
        calls.append(out is not None)
        return out

    monkeypatch.setattr(traj, "run_batched_dm", spy)
    ours = cirq_gb300.DensityMatrixSimulator(seed=3).run(c, repetitions=reps)
    assert calls == [True]
    ref = cirq.DensityMatrixSimulator(seed=4).run(c, repetitions=reps)
    for k in ("a", "b", "all"):
        assert ours.records[k].shape == ref.records[k].shape
        assert ours.records[k].dtype == ref.records[k].dtype
    h1 = np.bincount(_keys(ours.records), minlength=1 << 7)
    h2 = np.bincount(_keys(ref.records), minlength=1 << 7)
    keep = (h1 + h2) > 0
    assert scipy.stats.chi2_contingency(np.stack([h1[keep], h2[keep]]))[1] > 1e-4


def test_batched_dm_terminal_measurement_of_many_qubits(emu):
    """More than 5 terminally measured qubits: one draw per repetition from
    its own density matrix's diagonal."""
    q = cirq.LineQubit.range(7)
    c = cirq.Circuit(
        [cirq.H(x) for x in q[:3]], cirq.measure(q[0], key="m0"), cirq.CNOT(q[0], q[4]),
        cirq.amplitude_damp(0.4).on(q[4]), [cirq.CNOT(q[i], q[i + 3]) for i in range(1, 3)],
        cirq.measure(*q, key="z"),
    )
    reps = 2000
    ours = cirq_gb300.DensityMatrixSimulator(seed=5).run(c, repetitions=reps).records
    ref = cirq.DensityMatrixSimulator(seed=6).run(c, repetitions=reps).records
    a = ours["z"][:, 0, :].astype(int) @ (1 << np.arange(6, -1, -1))
    b = ref["z"][:, 0, :].astype(int) @ (1 << np.arange(6, -1, -1))
    h1, h2 = np.bincount(a, minlength=128), np.bincount(b, minlength=128)
    keep = (h1 + h2) > 0
    assert scipy.stats.chi2_contingency(np.stack([h1[keep], h2[keep]]))[1] > 1e-4
    # the mid-circuit record agrees with the final one on qubit 0 (no later gate on it)
    np.testing.assert_array_equal(ours["m0"][:, 0, 0], ours["z"][:, 0, 0])
