"""Random circuits through the public API on the CPU emulation of the engine,
compared with the reference simulators themselves (complex128), run here on
the same inputs: noiseless parameterized state vectors under random qubit
orders and initial states, and noisy parameterized density matrices with
explicit channels and noise models (whose placement follows the reference's
simulators).  CPU only."""

import numpy as np
import pytest
import sympy

import cirq
import cirq_gb300
from cirq_gb300 import simulator as sim_mod
from cpu_engine import EmuEngine

SYMS = sympy.symbols("a b")


@pytest.fixture
def emu(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    return eng


def _random_circuit(rng, q, channels: bool):
    n = len(q)
    moments = []
    for _ in range(int(rng.integers(3, 9))):
        ops, used = [], set()
        for _ in range(int(rng.integers(1, n + 1))):
            kind = int(rng.integers(0, 9 if channels else 6))
            k = 2 if kind in (3, 4) else 1
            free = [x for x in q if x not in used]
            if len(free) < k:
                break
            qs = [free[i] for i in rng.choice(len(free), size=k, replace=False)]
            used.update(qs)
            s = SYMS[int(rng.integers(0, 2))] if rng.random() < 0.4 else float(rng.uniform(-1, 1))
            op = [
                lambda: cirq.rx(s).on(*qs),
                lambda: (cirq.Z ** s).on(*qs),
                lambda: cirq.PhasedXZGate(x_exponent=0.3, z_exponent=-0.2, axis_phase_exponent=0.7).on(*qs),
                lambda: (cirq.CZ ** s).on(*qs),
                lambda: cirq.ZZPowGate(exponent=s).on(*qs),
                lambda: cirq.H(*qs),
                lambda: cirq.amplitude_damp(0.15).on(*qs),
                lambda: cirq.depolarize(0.1).on(*qs),
                lambda: cirq.phase_damp(0.3).on(*qs),
            ][kind]()
            ops.append(op)
        if ops:
            moments.append(cirq.Moment(ops))
    return cirq.Circuit(moments)


@pytest.mark.parametrize("seed", range(60))
def test_state_vectors_match_the_reference(emu, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 7))
    q = cirq.LineQubit.range(n)
    c = _random_circuit(rng, q, channels=False)
    r = cirq.ParamResolver({s: float(rng.uniform(-2, 2)) for s in SYMS})
    order = [q[i] for i in rng.permutation(n)]
    init = int(rng.integers(0, 2**n))
    want = cirq.Simulator(dtype=np.complex128).simulate(c, r, qubit_order=order, initial_state=init)
    got = cirq_gb300.Simulator().simulate(c, r, qubit_order=order, initial_state=init)
    np.testing.assert_allclose(got.final_state_vector, want.final_state_vector, atol=1e-5)


@pytest.mark.parametrize("seed", range(60))
def test_noisy_density_matrices_match_the_reference(emu, seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 5))
    q = cirq.LineQubit.range(n)
    c = _random_circuit(rng, q, channels=True)
    r = cirq.ParamResolver({s: float(rng.uniform(-2, 2)) for s in SYMS})
    noise = [None, cirq.depolarize(0.05), cirq.amplitude_damp(0.1)][seed % 3]
    want = cirq.DensityMatrixSimulator(dtype=np.complex128, noise=noise).simulate(c, r).final_density_matrix
    got = cirq_gb300.DensityMatrixSimulator(noise=noise).simulate(c, r).final_density_matrix
    np.testing.assert_allclose(got, want, atol=1e-5)


def _two_sample_p(a: np.ndarray, b: np.ndarray) -> float:
    """Chi-squared homogeneity test of two samples of outcome indices."""
    import scipy.stats

    keys = np.union1d(a, b)
    table = np.array([[np.sum(a == k) for k in keys], [np.sum(b == k) for k in keys]])
    table = table[:, table.sum(axis=0) > 0]
    if table.shape[1] < 2:
        return 1.0
    return scipy.stats.chi2_contingency(table)[1]


@pytest.mark.parametrize("seed", range(8))
def test_run_distributions_match_the_reference(emu, seed):
    """run() of random measured circuits (terminal and mid-circuit
    measurements, noise models on either simulator) sampled by the reference
    and by the package: the two samples agree (chi-squared homogeneity)."""
    rng = np.random.default_rng(500 + seed)
    n = int(rng.integers(2, 4))
    q = cirq.LineQubit.range(n)
    body = _random_circuit(rng, q, channels=seed % 2 == 1)
    r = cirq.ParamResolver({s: float(rng.uniform(-2, 2)) for s in SYMS})
    mid = seed % 3 == 0
    c = cirq.Circuit(body[: len(body) // 2])
    if mid:
        c.append(cirq.measure(q[0], key="mid"))
    c += body[len(body) // 2 :]
    c.append(cirq.measure(*q, key="m"))
    noise = [None, cirq.depolarize(0.08), cirq.amplitude_damp(0.2)][seed % 3]
    dm = seed % 4 < 2
    reps = 1500
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    want = ref_cls(noise=noise, seed=seed).run(c, r, repetitions=reps)
    got = ours_cls(noise=noise, seed=seed + 1).run(c, r, repetitions=reps)
    weights = 1 << np.arange(n - 1, -1, -1)
    a = want.records["m"][:, -1, :].astype(int) @ weights
    b = got.records["m"][:, -1, :].astype(int) @ weights
    if mid:
        a = a * 2 + want.records["mid"][:, 0, 0]
        b = b * 2 + got.records["mid"][:, 0, 0]
    assert _two_sample_p(a, b) > 1e-3, (seed, dm, str(noise))


def _random_pauli_sum(rng, q):
    terms = []
    for _ in range(int(rng.integers(1, 5))):
        k = int(rng.integers(1, len(q) + 1))
        qs = [q[i] for i in rng.choice(len(q), size=k, replace=False)]
        ps = cirq.PauliString({x: [cirq.X, cirq.Y, cirq.Z][int(rng.integers(0, 3))] for x in qs})
        terms.append(float(rng.normal()) * ps)
    return sum(terms[1:], terms[0])


@pytest.mark.parametrize("seed", range(30))
def test_expectations_amplitudes_and_sweeps_match_the_reference(emu, seed):
    rng = np.random.default_rng(900 + seed)
    n = int(rng.integers(2, 5))
    q = cirq.LineQubit.range(n)
    dm = seed % 2 == 1
    c = _random_circuit(rng, q, channels=dm)
    obs = [_random_pauli_sum(rng, q) for _ in range(2)]
    sweep = cirq.Zip(cirq.Linspace("a", -1.0, 1.0, 3), cirq.Linspace("b", 0.5, 2.0, 3))
    if dm:
        noise = [None, cirq.depolarize(0.05)][seed % 4 // 2]
        ref = cirq.DensityMatrixSimulator(dtype=np.complex128, noise=noise)
        ours = cirq_gb300.DensityMatrixSimulator(noise=noise)
    else:
        ref, ours = cirq.Simulator(dtype=np.complex128), cirq_gb300.Simulator()
    want = ref.simulate_expectation_values_sweep(c, obs, sweep)
    got = ours.simulate_expectation_values_sweep(c, obs, sweep)
    np.testing.assert_allclose(np.array(got), np.array(want), atol=1e-5)
    wres = ref.simulate_sweep(c, sweep)
    gres = ours.simulate_sweep(c, sweep)
    for w, g in zip(wres, gres):
        if dm:
            np.testing.assert_allclose(g.final_density_matrix, w.final_density_matrix, atol=1e-5)
        else:
            np.testing.assert_allclose(g.final_state_vector, w.final_state_vector, atol=1e-5)
    if not dm:
        bits = [int(b) for b in rng.integers(0, 2**n, size=4)]
        r = cirq.ParamResolver({"a": 0.3, "b": -0.4})
        np.testing.assert_allclose(ours.compute_amplitudes(c, bits, r), ref.compute_amplitudes(c, bits, r),
                                   atol=1e-5)


def _measurement_circuit(rng, q):
    """Random circuit exercising measurement semantics: mid-circuit
    measurements (repeated keys included), classical controls on earlier
    keys, invert masks, and a terminal measurement with a confusion map."""
    n = len(q)
    ops = []
    keys = []
    for step in range(int(rng.integers(3, 7))):
        a = q[int(rng.integers(0, n))]
        b = q[int(rng.integers(0, n))]
        ops.append(cirq.ry(float(rng.uniform(0.3, 2.8))).on(a))
        if a != b:
            ops.append(cirq.CNOT(a, b))
        r = rng.random()
        if r < 0.35:
            key = f"k{int(rng.integers(0, 3))}"
            inv = (bool(rng.integers(0, 2)),)
            ops.append(cirq.measure(a, key=key, invert_mask=inv))
            keys.append(key)
        elif r < 0.55 and keys:
            ops.append(cirq.X(b).with_classical_controls(keys[int(rng.integers(0, len(keys)))]))
    confusion = np.array([[0.9, 0.1], [0.2, 0.8]])
    ops.append(cirq.measure(q[0], key="t", confusion_map={(0,): confusion}))
    ops.append(cirq.measure(*q, key="all"))
    return cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)


def _outcome_codes(result, key):
    """One integer per repetition from all instances and bits of a key."""
    rec = np.asarray(result.records[key]).astype(np.int64)
    flat = rec.reshape(rec.shape[0], -1)
    return flat @ (1 << np.arange(flat.shape[1] - 1, -1, -1))


@pytest.mark.parametrize("seed", range(6))
def test_measurement_semantics_match_the_reference(emu, seed):
    rng = np.random.default_rng(4000 + seed)
    q = cirq.LineQubit.range(3)
    c = _measurement_circuit(rng, q)
    noise = [None, cirq.depolarize(0.05)][seed % 2]
    dm = seed % 4 >= 2
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    reps = 500
    want = ref_cls(noise=noise, seed=seed).run(c, repetitions=reps)
    got = ours_cls(noise=noise, seed=seed + 7).run(c, repetitions=reps)
    assert set(got.records) == set(want.records)
    for key in want.records:
        assert got.records[key].shape == want.records[key].shape, key
        assert _two_sample_p(_outcome_codes(want, key), _outcome_codes(got, key)) > 1e-3, (seed, key)


_CONFUSION = np.array([[0.9, 0.1], [0.2, 0.8]])


def _confused_circuit(terminal: bool, mid_then_control: bool):
    """One qubit in |0>, measured with an invert mask and a confusion map:
    the reference records 1 with p 0.9 where it measures in place (confuse,
    then invert: simulation_state.py:94-95) and 0.8 where it samples terminal
    measurements at the end of run() (invert, then confuse:
    simulator.py:803-808)."""
    q0, q1 = cirq.LineQubit.range(2)
    m = cirq.measure(q0, key="a", invert_mask=(True,), confusion_map={(0,): _CONFUSION})
    ops = [cirq.I(q0), cirq.I(q1), m]
    if not terminal:
        ops.append(cirq.X(q1).with_classical_controls("a") if mid_then_control else cirq.H(q0))
    ops.append(cirq.measure(q1, key="b"))
    return cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("terminal,control", [(True, False), (False, False), (False, True)])
def test_invert_mask_and_confusion_map_orders_match_the_reference(emu, dm, terminal, control):
    c = _confused_circuit(terminal, control)
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    reps = 2000
    want = ref_cls(seed=3).run(c, repetitions=reps)
    got = ours_cls(seed=4).run(c, repetitions=reps)
    for key in ("a", "b"):
        assert _two_sample_p(_outcome_codes(want, key), _outcome_codes(got, key)) > 1e-3, key
    p1 = float(np.mean(got.records["a"][:, 0, 0]))
    assert abs(p1 - (0.8 if terminal else 0.9)) < 0.04
    if control:
        # the condition reads the recorded (confused, inverted) value
        np.testing.assert_array_equal(got.records["b"][:, 0, 0], got.records["a"][:, 0, 0])


@pytest.mark.parametrize("dm", [False, True])
def test_simulate_applies_confusion_maps_as_the_reference(emu, dm):
    """simulate() measures in place: confusion, then the invert mask."""
    q = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.measure(q, key="a", invert_mask=(True,), confusion_map={(0,): _CONFUSION}))
    ours = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=5)
    got = np.array([int(ours.simulate(c).measurements["a"][0]) for _ in range(600)])
    ref = (cirq.DensityMatrixSimulator if dm else cirq.Simulator)(seed=6)
    want = np.array([int(ref.simulate(c).measurements["a"][0]) for _ in range(600)])
    assert _two_sample_p(want, got) > 1e-3
    assert abs(got.mean() - 0.9) < 0.05


def test_complex128_array_initial_states_are_cast_as_the_reference(emu):
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(*q), cirq.amplitude_damp(0.2).on(q[1]))
    rho = cirq.testing.random_density_matrix(4, random_state=4)
    assert rho.dtype == np.complex128
    want = cirq.DensityMatrixSimulator().simulate(c, initial_state=rho).final_density_matrix
    got = cirq_gb300.DensityMatrixSimulator().simulate(c, initial_state=rho).final_density_matrix
    np.testing.assert_allclose(got, want, atol=1e-5)
    vec = cirq.testing.random_superposition(4, random_state=5)
    u = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(*q))
    np.testing.assert_allclose(cirq_gb300.Simulator().simulate(u, initial_state=vec).final_state_vector,
                               cirq.Simulator().simulate(u, initial_state=vec).final_state_vector, atol=1e-5)


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("inner", ["damp", "depolarize", "reset", "reset_then_use"])
def test_classical_control_of_non_unitary_operations(emu, dm, inner):
    """Channels, mixtures and resets under classical control: applied in a
    repetition only when the condition holds there."""
    q0, q1, q2 = cirq.LineQubit.range(3)
    body = {
        "damp": cirq.amplitude_damp(0.6).on(q1),
        "depolarize": cirq.depolarize(0.5).on(q1),
        "reset": cirq.reset(q1),
        "reset_then_use": cirq.reset(q1),
    }[inner]
    ops = [cirq.H(q0), cirq.X(q1), cirq.ry(0.7).on(q2), cirq.measure(q0, key="a"),
           body.with_classical_controls("a"), cirq.H(q2)]
    if inner == "reset_then_use":
        ops += [cirq.measure(q1, key="c"), cirq.X(q2).with_classical_controls("c"), cirq.measure(q2, key="d")]
    ops.append(cirq.measure(q1, q2, key="m"))
    c = cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    reps = 1500
    want = ref_cls(seed=1).run(c, repetitions=reps)
    got = ours_cls(seed=2).run(c, repetitions=reps)
    assert set(got.records) == set(want.records)
    for key in want.records:
        assert got.records[key].shape == want.records[key].shape, key
        assert _two_sample_p(_outcome_codes(want, key), _outcome_codes(got, key)) > 1e-3, key
    joint_w = _outcome_codes(want, "a") * 4 + _outcome_codes(want, "m")
    joint_g = _outcome_codes(got, "a") * 4 + _outcome_codes(got, "m")
    assert _two_sample_p(joint_w, joint_g) > 1e-3


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("case", ["kraus", "mixture", "control", "two_qubit"])
def test_keyed_channels_match_the_reference(emu, dm, case):
    """Channels with a measurement key: the state-vector simulator records
    the index of the operator that acted (and conditions may read it); the
    density-matrix simulator applies the channel and records nothing."""
    q0, q1 = cirq.LineQubit.range(2)
    kc = cirq.KrausChannel(cirq.kraus(cirq.amplitude_damp(0.4)), key="k")
    mc = cirq.MixedUnitaryChannel([(0.3, np.eye(2)), (0.7, cirq.unitary(cirq.X))], key="k")
    ops = [cirq.X(q0), cirq.H(q1)]
    if case == "kraus":
        ops.append(kc.on(q0))
    elif case == "mixture":
        ops.append(mc.on(q0))
    elif case == "control":
        ops += [kc.on(q0), cirq.X(q1).with_classical_controls("k")]
    else:
        mix = cirq.mixture(cirq.asymmetric_depolarize(error_probabilities={"XZ": 0.3, "YY": 0.2}))
        ops.append(cirq.MixedUnitaryChannel(mix, key="k").on(q0, q1))
    ops.append(cirq.measure(q0, q1, key="m"))
    c = cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    if dm and case == "control":
        with pytest.raises(ValueError, match="missing"):
            ref_cls().run(c, repetitions=5)
        with pytest.raises(ValueError, match="missing"):
            ours_cls().run(c, repetitions=5)
        return
    reps = 1500
    want = ref_cls(seed=1).run(c, repetitions=reps)
    got = ours_cls(seed=2).run(c, repetitions=reps)
    assert set(got.records) == set(want.records)
    for key in want.records:
        assert got.records[key].shape == want.records[key].shape, key
        assert _two_sample_p(_outcome_codes(want, key), _outcome_codes(got, key)) > 1e-3, key
    if not dm:
        joint_w = _outcome_codes(want, "k") * 4 + _outcome_codes(want, "m")
        joint_g = _outcome_codes(got, "k") * 4 + _outcome_codes(got, "m")
        assert _two_sample_p(joint_w, joint_g) > 1e-3
        assert set(cirq_gb300.Simulator(seed=3).simulate(c).measurements) == {"k", "m"}


def _iterations(result, key):
    """Loop iterations per repetition: instances up to the first 1 of `key`
    (the loop stops there; later instances are the reference's padding)."""
    rec = np.asarray(result.records[key])[:, :, 0]
    return np.argmax(rec == 1, axis=1) + 1


@pytest.mark.parametrize("dm", [False, True])
def test_repeat_until_loops_match_the_reference(emu, dm):
    """CircuitOperation(repeat_until=...): the body repeats per repetition
    until its condition holds (a geometric number of iterations here)."""
    q0, q1 = cirq.LineQubit.range(2)
    body = cirq.Circuit(cirq.ry(1.2).on(q0), cirq.measure(q0, key="m"), cirq.X(q1).with_classical_controls("m"))
    loop = cirq.CircuitOperation(body.freeze(), repeat_until=cirq.KeyCondition(cirq.MeasurementKey("m")),
                                 use_repetition_ids=False)
    c = cirq.Circuit(cirq.X(q1), loop, cirq.measure(q1, key="z"))
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    want = ref_cls(seed=1).run(c, repetitions=800)
    got = ours_cls(seed=2).run(c, repetitions=800)
    assert _two_sample_p(_iterations(want, "m"), _iterations(got, "m")) > 1e-3
    # the controlled X fires once (in the last iteration): z = 0 always
    assert not got.records["z"].any() and not want.records["z"].any()


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("obs", ["X", "XZ", "YY", "ZXZ"])
def test_pauli_measurement_gates_match_the_reference(emu, dm, obs):
    """PauliMeasurementGate acts through its decomposition.  The reference's
    density-matrix simulator leaves a non-Hermitian matrix after a
    multi-qubit Pauli measurement, so both simulators here are compared with
    the reference's state-vector samples."""
    q = cirq.LineQubit.range(len(obs))
    pm = cirq.PauliMeasurementGate(cirq.DensePauliString(obs), key="p").on(*q)
    c = cirq.Circuit(cirq.H(q[0]), *[cirq.CNOT(q[0], x) for x in q[1:]], cirq.ry(0.6).on(q[-1]), pm,
                     cirq.rx(0.4).on(q[0]), cirq.measure(*q, key="f"))
    want = cirq.Simulator(seed=1).run(c, repetitions=2000)
    got = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=2).run(c, repetitions=2000)
    for key in ("p", "f"):
        assert got.records[key].shape == want.records[key].shape
        assert _two_sample_p(_outcome_codes(want, key), _outcome_codes(got, key)) > 1e-3, key


@pytest.mark.parametrize("dm", [False, True])
def test_symbolic_repetitions_and_nested_loops_match_the_reference(emu, dm):
    q0, q1 = cirq.LineQubit.range(2)
    rep = cirq.CircuitOperation(cirq.FrozenCircuit(cirq.rx(0.3).on(q0), cirq.CNOT(q0, q1))) ** sympy.Symbol("a")
    c = cirq.Circuit(cirq.H(q1), rep)
    sweep = cirq.Points("a", [0, 1, 3, 4])
    ref = (cirq.DensityMatrixSimulator if dm else cirq.Simulator)(dtype=np.complex128)
    ours = cirq_gb300.DensityMatrixSimulator() if dm else cirq_gb300.Simulator()
    for w, g in zip(ref.simulate_sweep(c, sweep), ours.simulate_sweep(c, sweep)):
        assert g.params == w.params
        if dm:
            np.testing.assert_allclose(g.final_density_matrix, w.final_density_matrix, atol=1e-5)
        else:
            np.testing.assert_allclose(g.final_state_vector, w.final_state_vector, atol=1e-5)
    obs = [cirq.Z(q0) * cirq.X(q1)]
    np.testing.assert_allclose(ours.simulate_expectation_values_sweep(c, obs, sweep),
                               ref.simulate_expectation_values_sweep(c, obs, sweep), atol=1e-5)
    # a repeat-until loop inside a repeated CircuitOperation (repetition ids)
    inner = cirq.CircuitOperation(
        cirq.FrozenCircuit(cirq.H(q0), cirq.measure(q0, key="inner")),
        repeat_until=cirq.SympyCondition(sympy.Eq(sympy.Symbol("inner"), 0)),
    )
    outer = cirq.CircuitOperation(cirq.FrozenCircuit(inner, cirq.X(q0), cirq.measure(q0, key="outer")),
                                  repetitions=2, use_repetition_ids=True)
    circuit = cirq.Circuit(outer)
    sim = cirq_gb300.DensityMatrixSimulator(seed=3) if dm else cirq_gb300.Simulator(seed=3)
    got = sim.run(circuit, repetitions=200)
    want = (cirq.DensityMatrixSimulator if dm else cirq.Simulator)(seed=4).run(circuit, repetitions=200)
    assert set(got.records) == set(want.records) == {"0:inner", "1:inner", "0:outer", "1:outer"}
    for key in ("0:outer", "1:outer"):
        assert got.records[key].all() and want.records[key].all()
