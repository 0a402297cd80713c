"""Mid-circuit measurement and state-vector noise as GPU trajectories,
checked statistically against exact distributions from the oracle."""

import itertools

import numpy as np
import pytest
import scipy.stats

import cirq
import cirq_gb300
from cirq_gb300.ir import flatten_ops
from oracle.circuits import simulate_density_matrix
from oracle.statevector import apply_matrix

pytestmark = pytest.mark.gpu


def _pvalue(counts: dict, probs: dict, reps: int) -> float:
    keys = sorted(set(probs) | set(counts))
    obs = np.array([counts.get(k, 0) for k in keys], dtype=float)
    exp = np.array([probs.get(k, 0.0) for k in keys]) * reps
    assert obs[exp == 0].sum() == 0, "outcome with probability 0 was sampled"
    keep = exp > 0
    return scipy.stats.chisquare(obs[keep], exp[keep]).pvalue


def _record_distribution(circuit, qubits):
    """Exact joint distribution of every measurement record, by enumerating
    the branches of each measurement on the oracle's state vector."""
    n = len(qubits)
    index = {q: i for i, q in enumerate(qubits)}
    ops = flatten_ops(circuit)
    out: dict = {}

    def rec(i, psi, p, bits):
        if p < 1e-14:
            return
        if i == len(ops):
            out[tuple(bits)] = out.get(tuple(bits), 0.0) + p
            return
        op = ops[i]
        axes = [index[q] for q in op.qubits]
        if cirq.is_measurement(op):
            inv = op.gate.full_invert_mask()
            for outcome in itertools.product([0, 1], repeat=len(axes)):
                sl = [slice(None)] * n
                for a, b in zip(axes, outcome):
                    sl[a] = b
                proj = np.zeros_like(psi)
                proj[tuple(sl)] = psi[tuple(sl)]
                pr = float(np.sum(np.abs(proj) ** 2))
                if pr > 1e-14:
                    rb = [b ^ int(v) for b, v in zip(outcome, inv)]
                    rec(i + 1, proj / np.sqrt(pr), p * pr, bits + rb)
        else:
            rec(i + 1, apply_matrix(psi, axes, cirq.unitary(op)), p, bits)

    psi0 = np.zeros((2,) * n, dtype=np.complex128)
    psi0[(0,) * n] = 1
    rec(0, psi0, 1.0, [])
    return out


def _counts(result, keys):
    recs = [result.records[k] for k in keys]  # (R, instances, bits)
    counts: dict = {}
    for r in range(recs[0].shape[0]):
        key = tuple(int(b) for rr in recs for b in rr[r].reshape(-1))
        counts[key] = counts.get(key, 0) + 1
    return counts


def test_mid_circuit_measurements_chi2():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.H(q[0]),
        cirq.CNOT(q[0], q[1]),
        cirq.ry(0.7).on(q[2]),
        cirq.measure(q[0], key="a"),
        cirq.H(q[1]),
        cirq.CZ(q[1], q[2]),
        cirq.measure(q[1], q[2], key="b", invert_mask=(True,)),
        cirq.rx(1.1).on(q[0]),
        cirq.measure(q[0], key="c"),
        strategy=cirq.InsertStrategy.NEW,
    )
    probs = _record_distribution(c, q)
    reps = 4000
    res = cirq_gb300.Simulator(seed=5).run(c, repetitions=reps)
    assert res.records["b"].shape == (reps, 1, 2)
    assert _pvalue(_counts(res, ["a", "b", "c"]), probs, reps) > 1e-3


def test_repeated_key_and_deterministic_outcomes():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(
        cirq.X(q[0]),
        cirq.measure(q[0], key="m"),
        cirq.CNOT(q[0], q[1]),
        cirq.measure(q[1], key="m"),
        cirq.X(q[0]),
        cirq.measure(q[0], key="z"),
        strategy=cirq.InsertStrategy.NEW,
    )
    res = cirq_gb300.Simulator(seed=1).run(c, repetitions=50)
    assert res.records["m"].shape == (50, 2, 1)
    assert np.all(res.records["m"] == 1) and np.all(res.records["z"] == 0)


def test_noisy_state_vector_matches_density_matrix_distribution():
    q = cirq.LineQubit.range(3)
    body = cirq.Circuit(
        cirq.H(q[0]),
        cirq.depolarize(0.15).on(q[0]),
        cirq.CNOT(q[0], q[1]),
        cirq.bit_flip(0.1).on(q[1]),
        cirq.ry(0.9).on(q[2]),
        cirq.amplitude_damp(0.3).on(q[2]),
        cirq.CZ(q[1], q[2]),
        cirq.phase_damp(0.4).on(q[1]),
        cirq.H(q[1]),
        strategy=cirq.InsertStrategy.NEW,
    )
    rho = simulate_density_matrix(body, qubit_order=q)
    p = np.clip(np.real(np.diag(rho)), 0, None)
    probs = {tuple((i >> (2 - j)) & 1 for j in range(3)): p[i] for i in range(8)}
    reps = 5000
    res = cirq_gb300.Simulator(seed=7).run(body + cirq.measure(*q, key="m"), repetitions=reps)
    assert _pvalue(_counts(res, ["m"]), probs, reps) > 1e-3


def test_noise_model_trajectories_match_density_matrix():
    q = cirq.LineQubit.range(2)
    body = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.rx(0.6).on(q[1]))
    noise = cirq.ConstantQubitNoiseModel(cirq.amplitude_damp(0.2))
    rho = simulate_density_matrix(body, qubit_order=q, noise=noise)
    p = np.clip(np.real(np.diag(rho)), 0, None)
    probs = {((i >> 1) & 1, i & 1): p[i] for i in range(4)}
    reps = 4000
    res = cirq_gb300.Simulator(noise=noise, seed=3).run(body + cirq.measure(*q, key="m"), repetitions=reps)
    assert _pvalue(_counts(res, ["m"]), probs, reps) > 1e-3


def test_amplitude_damping_decay_rate():
    q = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.X(q), cirq.amplitude_damp(0.3).on(q), cirq.measure(q, key="m"))
    reps = 4000
    ones = int(cirq_gb300.Simulator(seed=11).run(c, repetitions=reps).records["m"].sum())
    assert scipy.stats.binomtest(ones, reps, 0.7).pvalue > 1e-3


def test_simulate_returns_one_normalised_trajectory():
    q = cirq.LineQubit.range(4)
    c = cirq.Circuit([cirq.H.on_each(*q), cirq.amplitude_damp(0.5).on_each(*q), cirq.CNOT(q[0], q[3])])
    res = cirq_gb300.Simulator(seed=2).simulate(c, qubit_order=q)
    assert abs(np.linalg.norm(res.final_state_vector) - 1) < 1e-5


def test_density_matrix_mid_circuit_measurement():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(
        cirq.H(q[0]),
        cirq.measure(q[0], key="a"),
        cirq.CNOT(q[0], q[1]),
        cirq.measure(q[1], key="b"),
        strategy=cirq.InsertStrategy.NEW,
    )
    sim = cirq_gb300.DensityMatrixSimulator(seed=4)
    res = sim.run(c, repetitions=400)
    a, b = res.records["a"][:, 0, 0], res.records["b"][:, 0, 0]
    assert np.array_equal(a, b) and 100 < a.sum() < 300
    out = sim.simulate(c, qubit_order=q)
    rho = out.final_density_matrix
    bit = int(out.measurements["a"][0])
    expect = np.zeros((4, 4))
    expect[3 * bit, 3 * bit] = 1
    assert np.allclose(rho, expect, atol=1e-6)


def test_expectation_with_terminal_measurement_uses_the_collapsed_state():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.measure(q[0], key="m"))
    obs = [cirq.Z(q[1]), cirq.X(q[0])]
    for sim in (cirq_gb300.Simulator(seed=9), cirq_gb300.DensityMatrixSimulator(seed=9)):
        vals = sim.simulate_expectation_values(c, obs, permit_terminal_measurements=True)
        assert abs(abs(vals[0]) - 1) < 1e-5 and abs(vals[1]) < 1e-5


def test_moment_steps_match_the_oracle_after_every_moment():
    from oracle.circuits import simulate_state_vector
    from cirq_gb300 import workloads

    c = workloads.random_layer_circuit(6, 4, seed=21)
    q = sorted(c.all_qubits())
    sim = cirq_gb300.Simulator(seed=1)
    steps = list(sim.simulate_moment_steps(c, qubit_order=q))
    assert len(steps) == len(c)
    for i, _ in enumerate(c):
        pass
    for i, step in enumerate(sim.simulate_moment_steps(c, qubit_order=q)):
        want = simulate_state_vector(c[: i + 1], qubit_order=q)
        assert np.abs(step.state_vector(copy=True) - want).max() < 1e-5
        if i == len(c) - 1:
            samples = step.sample(q[:2], repetitions=2000, seed=3)
            assert samples.shape == (2000, 2) and samples.dtype == np.uint8
            p = np.abs(want.reshape(4, -1)) ** 2
            probs = {(a >> 1 & 1, a & 1): float(p[a].sum()) for a in range(4)}
            counts: dict = {}
            for row in samples:
                counts[tuple(int(x) for x in row)] = counts.get(tuple(int(x) for x in row), 0) + 1
            assert _pvalue(counts, probs, 2000) > 1e-3


def test_moment_steps_with_measurements_and_density_matrix():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.X(q[0]), cirq.measure(q[0], key="a"), cirq.CNOT(q[0], q[1]), cirq.measure(q[1], key="b"))
    steps = list(cirq_gb300.Simulator(seed=1).simulate_moment_steps(c))
    assert [dict(s.measurements) for s in steps][1]["a"].tolist() == [1]
    dm_steps = cirq_gb300.DensityMatrixSimulator(seed=1, noise=cirq.amplitude_damp(0.25)).simulate_moment_steps(
        cirq.Circuit(cirq.X(q[0]), cirq.X(q[1]))
    )
    last = None
    for s in dm_steps:
        last = s.density_matrix()
    assert abs(np.trace(last) - 1) < 1e-5
    assert abs(np.real(last[3, 3]) - 0.75**2) < 1e-5


def test_mixture_noise_runs_as_batched_trajectories():
    """Mixture-only noise with terminal measurements: the repetitions are
    evolved together (far fewer launches than repetitions) and sample the
    density matrix's distribution."""
    q = cirq.LineQubit.range(4)
    body = cirq.Circuit(
        cirq.H(q[0]),
        cirq.depolarize(0.2).on(q[0]),
        cirq.CNOT(q[0], q[1]),
        cirq.bit_flip(0.15).on(q[1]),
        cirq.ry(0.7).on(q[2]),
        cirq.phase_flip(0.3).on(q[2]),
        cirq.CZ(q[1], q[2]),
        cirq.H(q[2]),
        cirq.depolarize(0.1).on_each(*q),
        cirq.CNOT(q[2], q[3]),
        strategy=cirq.InsertStrategy.NEW,
    )
    rho = simulate_density_matrix(body, qubit_order=q)
    p = np.clip(np.real(np.diag(rho)), 0, None)
    probs = {tuple((i >> (3 - j)) & 1 for j in range(4)): p[i] for i in range(16)}
    reps = 5000
    sim = cirq_gb300.Simulator(seed=13)
    l0 = sim.engine.launches()
    res = sim.run(body + cirq.measure(*q, key="m"), repetitions=reps)
    assert sim.engine.launches() - l0 < reps
    assert res.records["m"].shape == (reps, 1, 4)
    assert _pvalue(_counts(res, ["m"]), probs, reps) > 1e-3


@pytest.mark.parametrize("bits", [[3], [0], [10], [7, 2], [2, 7], [10, 0]])
def test_points_rdm_matches_partial_trace(bits):
    """Batched reduced density matrices of one or two index bits against a
    numpy partial trace, for several points at once."""
    rng = np.random.default_rng(len(bits) * 31 + bits[0])
    n, npts = 11, 3
    psi = rng.normal(size=(npts, 1 << n)) + 1j * rng.normal(size=(npts, 1 << n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    eng = cirq_gb300.Simulator().engine
    states = eng.upload(psi.astype(np.complex64).reshape(-1))
    got = eng.points_rdm(states, n, npts, bits)
    k = len(bits)
    for p in range(npts):
        # axes of the reshaped state: axis a <-> global bit n - 1 - a
        t = psi[p].reshape((2,) * n)
        keep = [n - 1 - b for b in bits]
        rest = [a for a in range(n) if a not in keep]
        m = np.transpose(t, keep + rest).reshape(1 << k, -1)
        want = m @ m.conj().T
        assert np.max(np.abs(got[p] - want)) < 2e-6


def _kraus_channel(ops):
    return cirq.KrausChannel([np.asarray(k, dtype=np.complex128) for k in ops])


@pytest.mark.parametrize("width", [2, 3])
def test_general_kraus_channels_match_density_matrix(width):
    """Non-mixture channels on two qubits (batched reduced density matrix)
    and three qubits (Pauli-basis weights) sample the density matrix's
    distribution."""
    g = 0.35
    ad = [np.array([[1, 0], [0, np.sqrt(1 - g)]]), np.array([[0, np.sqrt(g)], [0, 0]])]
    ops = ad
    for _ in range(width - 1):
        ops = [np.kron(a, b) for a in ops for b in ad]
    q = cirq.LineQubit.range(4)
    body = cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.CNOT(q[0], q[1]),
        cirq.ry(0.4).on(q[3]),
        _kraus_channel(ops).on(*q[1 : 1 + width]),
        cirq.CZ(q[1], q[2]),
        cirq.H(q[2]),
        strategy=cirq.InsertStrategy.NEW,
    )
    rho = simulate_density_matrix(body, qubit_order=q)
    p = np.clip(np.real(np.diag(rho)), 0, None)
    probs = {tuple((i >> (3 - j)) & 1 for j in range(4)): p[i] for i in range(16)}
    reps = 3000
    sim = cirq_gb300.Simulator(seed=5 + width)
    res = sim.run(body + cirq.measure(*q, key="m"), repetitions=reps)
    assert res.records["m"].shape == (reps, 1, 4)
    assert _pvalue(_counts(res, ["m"]), probs, reps) > 1e-3


def _teleport_like():
    q = cirq.LineQubit.range(3)
    return q, cirq.Circuit(
        cirq.H(q[0]),
        cirq.measure(q[0], key="a"),
        cirq.X(q[1]).with_classical_controls("a"),
        cirq.ry(0.9).on(q[2]),
        cirq.measure(q[2], key="c"),
        cirq.CNOT(q[1], q[2]).with_classical_controls("c"),
        cirq.measure(q[1], q[2], key="m"),
        strategy=cirq.InsertStrategy.NEW,
    )


@pytest.mark.parametrize("dm", [False, True])
def test_classical_control_in_run(dm):
    """Records follow the controls exactly: m[0] = a, m[1] = c xor (c and a)
    (the controlled CNOT flips q2 when c and q1 = a are both 1)."""
    q, c = _teleport_like()
    sim = cirq_gb300.DensityMatrixSimulator(seed=4) if dm else cirq_gb300.Simulator(seed=4)
    reps = 400 if dm else 3000
    res = sim.run(c, repetitions=reps)
    a = res.records["a"][:, 0, 0]
    cc = res.records["c"][:, 0, 0]
    m = res.records["m"][:, 0, :]
    np.testing.assert_array_equal(m[:, 0], a)
    np.testing.assert_array_equal(m[:, 1], cc ^ (cc & a))
    assert 0.4 < a.mean() < 0.6
    assert abs(cc.mean() - np.sin(0.45) ** 2) < (0.08 if dm else 0.04)


def test_classical_control_in_simulate_and_moment_steps():
    q, c = _teleport_like()
    body = c[:-1]
    for seed in range(6):
        r = cirq_gb300.Simulator(seed=seed).simulate(body)
        a = int(r.measurements["a"][0])
        cc = int(r.measurements["c"][0])
        want = np.zeros(8)
        want[(a << 2) | (a << 1) | (cc ^ (cc & a))] = 1  # q0 collapsed to a
        got = np.abs(r.final_state_vector) ** 2
        np.testing.assert_allclose(got, want, atol=1e-5)
        steps = list(cirq_gb300.Simulator(seed=seed).simulate_moment_steps(body))
        last = steps[-1]
        a2 = int(last.measurements["a"][0])
        c2 = int(last.measurements["c"][0])
        want2 = np.zeros(8)
        want2[(a2 << 2) | (a2 << 1) | (c2 ^ (c2 & a2))] = 1
        np.testing.assert_allclose(np.abs(last.state_vector()) ** 2, want2, atol=1e-5)


@pytest.mark.parametrize("dm", [False, True])
def test_keyed_and_classically_controlled_channels(dm):
    """Amplitude damping (gamma 0.4) of |1>, keyed: the state-vector record
    is 1 exactly when the decay operator acted (then q0 reads 0); the
    density-matrix simulator records nothing.  A damping channel controlled
    by a fair coin `a` acts only where a == 1."""
    q0, q1, q2 = cirq.LineQubit.range(3)
    kc = cirq.KrausChannel(cirq.kraus(cirq.amplitude_damp(0.4)), key="k")
    c = cirq.Circuit(
        [cirq.X(q0), cirq.X(q1), cirq.H(q2), kc.on(q0), cirq.measure(q2, key="a"),
         cirq.amplitude_damp(0.4).on(q1).with_classical_controls("a"), cirq.measure(q0, q1, key="m")],
        strategy=cirq.InsertStrategy.NEW,
    )
    sim = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=5)
    res = sim.run(c, repetitions=6000)
    m = res.records["m"][:, 0, :].astype(int)
    a = res.records["a"][:, 0, 0].astype(int)
    assert abs(1 - m[:, 0].mean() - 0.4) < 0.03
    assert abs(1 - m[a == 1, 1].mean() - 0.4) < 0.04
    assert np.all(m[a == 0, 1] == 1)
    if dm:
        assert "k" not in res.records
    else:
        k = res.records["k"][:, 0, 0].astype(int)
        np.testing.assert_array_equal(k, 1 - m[:, 0])


@pytest.mark.parametrize("dm", [False, True])
def test_repeat_until_loops_and_pauli_measurements(dm):
    """A loop of H + measure until the outcome is 1 runs a geometric number
    of times (mean 2); Pauli measurements of eigenstates are deterministic
    (ZZ of |11> -> +1, X of |+> -> +1) and XZ of a Bell state is a fair coin."""
    q0, q1, q2 = cirq.LineQubit.range(3)
    loop = cirq.CircuitOperation(cirq.FrozenCircuit(cirq.H(q2), cirq.measure(q2, key="m")),
                                 repeat_until=cirq.KeyCondition(cirq.MeasurementKey("m")), use_repetition_ids=False)
    sim = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=9)
    rec = sim.run(cirq.Circuit(loop), repetitions=3000).records["m"][:, :, 0]
    iters = np.argmax(rec == 1, axis=1) + 1
    assert abs(iters.mean() - 2.0) < 0.12 and iters.min() == 1
    pm = lambda obs, *qs: cirq.PauliMeasurementGate(cirq.DensePauliString(obs), key=obs).on(*qs)
    c = cirq.Circuit(cirq.X(q0), cirq.X(q1), pm("ZZ", q0, q1), cirq.H(q2), pm("X", q2))
    res = sim.run(c, repetitions=500)
    assert not res.records["ZZ"].any() and not res.records["X"].any()
    bell = cirq.Circuit(cirq.H(q0), cirq.CNOT(q0, q1), pm("XZ", q0, q1))
    p = sim.run(bell, repetitions=4000).records["XZ"].mean()
    assert abs(p - 0.5) < 0.03


def test_batched_density_matrix_trajectories_vs_reference_samples():
    """run() of a density-matrix circuit with mid-circuit measurements: every
    repetition's density matrix evolves as a batched point
    (trajectories.run_batched_dm); records match the reference's in
    distribution."""
    import scipy.stats

    from cirq_gb300 import trajectories as traj

    q = cirq.LineQubit.range(5)
    c = cirq.Circuit(
        cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(0.8).on(q[2]),
        cirq.amplitude_damp(0.3).on(q[1]), cirq.depolarize(0.1).on(q[2]),
        cirq.measure(q[1], key="a"),
        cirq.CNOT(q[1], q[3]), cirq.H(q[2]), cirq.CZ(q[2], q[3]), cirq.CNOT(q[3], q[4]),
        cirq.measure(q[2], q[3], key="b", invert_mask=(True, False)),
        cirq.X(q[0]) ** 0.3, cirq.phase_damp(0.2).on(q[0]),
        cirq.measure(*q, key="all"),
    )
    reps = 4000
    sim = cirq_gb300.DensityMatrixSimulator(seed=3)
    ops = traj.circuit_ops(sim, c, tuple(sorted(c.all_qubits())), cirq.ParamResolver({}))
    assert traj.run_batched_dm(sim, ops, tuple(sorted(c.all_qubits())), cirq.ParamResolver({}), 4) is not None
    ours = sim.run(c, repetitions=reps).records
    ref = cirq.DensityMatrixSimulator(seed=4).run(c, repetitions=reps).records

    def keys(rec):
        flat = np.concatenate([rec[k][:, 0, :] for k in ("a", "b", "all")], axis=1).astype(np.int64)
        return flat @ (1 << np.arange(flat.shape[1] - 1, -1, -1))

    h1 = np.bincount(keys(ours), minlength=1 << 8)
    h2 = np.bincount(keys(ref), minlength=1 << 8)
    keep = (h1 + h2) > 0
    assert scipy.stats.chi2_contingency(np.stack([h1[keep], h2[keep]]))[1] > 1e-4
