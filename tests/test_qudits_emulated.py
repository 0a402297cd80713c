"""Qudits (qids of dimension > 2) through the public API on the CPU emulation
of the engine, against the reference simulators (complex128) run here on
the same inputs: random circuits over qids of dimensions 2..5 with random
unitaries, parameterized qudit gates, qudit channels, mixtures and resets;
measurements of qudits with invert masks, confusion maps and classical
control; expectation values, amplitudes, initial states and moment steps.
CPU only."""

import numpy as np
import pytest
import scipy.stats
import sympy

import cirq
import cirq_gb300
from cirq_gb300 import qudits
from cirq_gb300 import simulator as sim_mod
from cpu_engine import EmuEngine

T = sympy.Symbol("t")


@pytest.fixture
def emu(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    return eng


class _Unitary(cirq.Gate):
    def __init__(self, shape, seed):
        self._shape = tuple(shape)
        self._u = scipy.stats.unitary_group.rvs(int(np.prod(shape)), random_state=seed)

    def _qid_shape_(self):
        return self._shape

    def _unitary_(self):
        return self._u


class _Phase(cirq.Gate):
    """diag(exp(i t v)) on one qudit: a parameterized qudit gate."""

    def __init__(self, d, t):
        self._d, self._t = d, t

    def _qid_shape_(self):
        return (self._d,)

    def _has_unitary_(self):
        return not cirq.is_parameterized(self._t)

    def _unitary_(self):
        if cirq.is_parameterized(self._t):
            return NotImplemented
        return np.diag(np.exp(1j * float(self._t) * np.arange(self._d)))

    def _is_parameterized_(self):
        return cirq.is_parameterized(self._t)

    def _parameter_names_(self):
        return cirq.parameter_names(self._t)

    def _resolve_parameters_(self, resolver, recursive):
        return _Phase(self._d, cirq.resolve_parameters(self._t, resolver, recursive))


class _Decay(cirq.Gate):
    """Amplitude damping of a qutrit: |2> -> |1> -> |0> with rate g."""

    def __init__(self, g):
        self._g = g

    def _qid_shape_(self):
        return (3,)

    def _kraus_(self):
        g = self._g
        k0 = np.diag([1.0, np.sqrt(1 - g), np.sqrt(1 - g)])
        k1 = np.zeros((3, 3))
        k1[0, 1] = np.sqrt(g)
        k2 = np.zeros((3, 3))
        k2[1, 2] = np.sqrt(g)
        return [k0, k1, k2]


class _Shift(cirq.Gate):
    """A mixture of level shifts of a qutrit."""

    def _qid_shape_(self):
        return (3,)

    def _mixture_(self):
        x = np.roll(np.eye(3), 1, axis=0)
        return [(0.6, np.eye(3)), (0.3, x), (0.1, x @ x)]


def _qids(rng):
    dims = [int(d) for d in rng.choice([2, 3, 4, 5], size=int(rng.integers(2, 4)))]
    if all(d == 2 for d in dims):
        dims[0] = 3
    return [cirq.LineQid(i, dimension=d) for i, d in enumerate(dims)]


def _random_circuit(rng, qids, channels=False):
    width = {q: qudits.bits_for(q.dimension) if q.dimension > 2 else 1 for q in qids}
    moments = []
    for _ in range(int(rng.integers(3, 7))):
        ops, used = [], set()
        for _ in range(3):
            free = [q for q in qids if q not in used]
            if not free:
                break
            kind = int(rng.integers(0, 6 if channels else 4))
            a = free[int(rng.integers(0, len(free)))]
            if kind == 0:
                op = _Unitary((a.dimension,), int(rng.integers(0, 1 << 30))).on(a)
            elif kind == 1 and len(free) > 1:
                b = [q for q in free if q != a][0]
                if width[a] + width[b] > 5:
                    continue
                op = _Unitary((a.dimension, b.dimension), int(rng.integers(0, 1 << 30))).on(a, b)
            elif kind == 2:
                op = _Phase(a.dimension, T if rng.random() < 0.5 else float(rng.uniform(-2, 2))).on(a)
            elif kind == 3 and a.dimension == 2:
                op = cirq.rx(T).on(a)
            elif kind == 4 and a.dimension == 3:
                op = _Decay(0.2).on(a)
            elif kind == 5 and a.dimension == 3:
                op = _Shift().on(a)
            else:
                op = _Unitary((a.dimension,), int(rng.integers(0, 1 << 30))).on(a)
            ops.append(op)
            used.update(op.qubits)
        moments.append(cirq.Moment(ops))
    return cirq.Circuit(moments)


def test_embedding_index_and_bits():
    q = [cirq.LineQid(0, dimension=3), cirq.LineQubit(1), cirq.LineQid(2, dimension=5)]
    emb = qudits.Embedding(q)
    assert len(emb.qubits) == 2 + 1 + 3 and emb.size == 30
    # index (a, b, c) of the reference's state -> bits a(2) b(1) c(3)
    idx = emb.index
    for a in range(3):
        for b in range(2):
            for c in range(5):
                assert idx[(a * 2 + b) * 5 + c] == (a << 4) | (b << 3) | c
    assert emb.qubits[2] is q[1]
    assert sorted(emb.qubits[3:]) == list(emb.qubits[3:])


@pytest.mark.parametrize("seed", range(40))
def test_state_vectors_match_the_reference(emu, seed):
    rng = np.random.default_rng(seed)
    q = _qids(rng)
    c = _random_circuit(rng, q)
    r = cirq.ParamResolver({T: float(rng.uniform(-2, 2))})
    order = [q[i] for i in rng.permutation(len(q))]
    size = int(np.prod([x.dimension for x in q]))
    init = int(rng.integers(0, size)) if seed % 2 else cirq.testing.random_superposition(size, random_state=seed)
    want = cirq.Simulator(dtype=np.complex128).simulate(c, r, qubit_order=order, initial_state=init)
    got = cirq_gb300.Simulator().simulate(c, r, qubit_order=order, initial_state=init)
    np.testing.assert_allclose(got.final_state_vector, want.final_state_vector, atol=1e-5)
    assert got.qubit_map == want.qubit_map
    assert cirq.qid_shape(got) == cirq.qid_shape(want)


@pytest.mark.parametrize("seed", range(30))
def test_density_matrices_match_the_reference(emu, seed):
    rng = np.random.default_rng(300 + seed)
    q = _qids(rng)
    c = _random_circuit(rng, q, channels=True)
    r = cirq.ParamResolver({T: float(rng.uniform(-2, 2))})
    want = cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(c, r).final_density_matrix
    got = cirq_gb300.DensityMatrixSimulator().simulate(c, r).final_density_matrix
    np.testing.assert_allclose(got, want, atol=1e-5)


def test_sweeps_with_and_without_parameterized_qudit_gates(emu):
    q3, q2 = cirq.LineQid(0, dimension=3), cirq.LineQubit(1)
    u = _Unitary((3, 2), 7).on(q3, q2)
    sweep = cirq.Linspace(T, -1.0, 1.5, 4)
    for c in (cirq.Circuit(u, cirq.rx(T).on(q2)), cirq.Circuit(u, _Phase(3, T).on(q3), cirq.ry(T).on(q2))):
        want = cirq.Simulator(dtype=np.complex128).simulate_sweep(c, sweep)
        got = cirq_gb300.Simulator().simulate_sweep(c, sweep)
        for w, g in zip(want, got):
            assert g.params == w.params
            np.testing.assert_allclose(g.final_state_vector, w.final_state_vector, atol=1e-5)
    with pytest.raises(ValueError, match="not specified"):
        cirq_gb300.Simulator().simulate(cirq.Circuit(_Phase(3, T).on(q3)))


def _pauli_expectation(vec, qids, observable) -> complex:
    """<psi| observable |psi> over qids of any dimension (Paulis on qubits)."""
    dims = [x.dimension for x in qids]
    psi = vec.reshape(dims)
    total = 0j
    for term in cirq.PauliSum.wrap(observable):
        phi = psi
        for x, p in term.items():
            ax = qids.index(x)
            phi = np.moveaxis(np.tensordot(cirq.unitary(p), phi, axes=([1], [ax])), 0, ax)
        total += complex(term.coefficient) * np.vdot(psi, phi)
    return total


def test_expectation_values_and_amplitudes(emu):
    rng = np.random.default_rng(5)
    q = [cirq.LineQid(0, dimension=3), cirq.LineQubit(1), cirq.LineQubit(2), cirq.LineQid(3, dimension=4)]
    c = _random_circuit(rng, q) + cirq.Circuit(cirq.CNOT(q[1], q[2]), cirq.H(q[1]))
    obs = [cirq.Z(q[1]) * cirq.X(q[2]) + 0.5 * cirq.Y(q[2]), 0.3 * cirq.Z(q[2])]
    sweep = cirq.Linspace(T, 0.0, 1.0, 3)
    # the reference's PauliSum expectations assume 2^n states, so the values
    # are contracted here from the reference's own final states
    states = cirq.Simulator(dtype=np.complex128).simulate_sweep(c, sweep)
    want = [[_pauli_expectation(s.final_state_vector, q, o) for o in obs] for s in states]
    got = cirq_gb300.Simulator().simulate_expectation_values_sweep(c, obs, sweep)
    np.testing.assert_allclose(np.array(got), np.array(want), atol=1e-5)
    dgot = cirq_gb300.DensityMatrixSimulator().simulate_expectation_values_sweep(c, obs, sweep)
    np.testing.assert_allclose(np.array(dgot), np.array(want), atol=1e-5)
    bits = [0, 5, 17, 47]
    r = cirq.ParamResolver({T: 0.4})
    np.testing.assert_allclose(cirq_gb300.Simulator().compute_amplitudes(c, bits, r),
                               cirq.Simulator(dtype=np.complex128).compute_amplitudes(c, bits, r), atol=1e-5)


def test_simulation_state_and_density_matrix_initial_states(emu):
    q = [cirq.LineQid(0, dimension=3), cirq.LineQubit(1)]
    c = cirq.Circuit(_Unitary((3, 2), 3).on(*q))
    vec = cirq.testing.random_superposition(6, random_state=2)
    st = cirq.StateVectorSimulationState(qubits=q, initial_state=vec.reshape(3, 2).astype(np.complex64))
    want = cirq.Simulator(dtype=np.complex128).simulate(c, initial_state=vec.reshape(3, 2), qubit_order=q)
    got = cirq_gb300.Simulator().simulate(c, initial_state=st)
    np.testing.assert_allclose(got.final_state_vector, want.final_state_vector, atol=1e-5)
    rho = cirq.testing.random_density_matrix(6, random_state=4)
    dwant = cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(c, initial_state=rho, qubit_order=q)
    dgot = cirq_gb300.DensityMatrixSimulator().simulate(c, initial_state=rho, qubit_order=q)
    np.testing.assert_allclose(dgot.final_density_matrix, dwant.final_density_matrix, atol=1e-5)
    with pytest.raises(ValueError):
        cirq_gb300.Simulator().simulate(c, initial_state=6, qubit_order=q)


def _two_sample_p(a, b) -> float:
    keys = np.union1d(a, b)
    table = np.array([[np.sum(a == k) for k in keys], [np.sum(b == k) for k in keys]])
    if table.shape[1] < 2:
        return 1.0
    return scipy.stats.chi2_contingency(table)[1]


def _codes(result, key, dims):
    rec = np.asarray(result.records[key]).astype(np.int64)
    flat = rec.reshape(rec.shape[0], -1)
    base = [d for _ in range(rec.shape[1]) for d in dims]
    out = np.zeros(flat.shape[0], dtype=np.int64)
    for j, d in enumerate(base):
        out = out * d + flat[:, j]
    return out


_CONF3 = np.array([[0.8, 0.1, 0.1], [0.05, 0.9, 0.05], [0.2, 0.2, 0.6]])


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("case", ["terminal", "mid", "control", "sympy", "reset"])
def test_run_distributions_match_the_reference(emu, dm, case):
    q3, q2, q4 = cirq.LineQid(0, dimension=3), cirq.LineQubit(1), cirq.LineQid(2, dimension=4)
    ops = [_Unitary((3,), 1).on(q3), cirq.H(q2), _Unitary((4,), 2).on(q4), _Unitary((3, 2), 3).on(q3, q2)]
    m = cirq.measure(q3, q2, key="a", invert_mask=(True, False), confusion_map={(0,): _CONF3})
    ops.append(m)
    if case == "mid":
        ops += [_Unitary((3,), 4).on(q3), _Shift().on(q3) if not dm else _Decay(0.3).on(q3)]
    elif case == "control":
        ops.append(_Unitary((4,), 5).on(q4).with_classical_controls("a"))
    elif case == "sympy":
        cond = cirq.SympyCondition(sympy.Eq(sympy.Symbol("a"), 3))
        ops.append(cirq.X(q2).with_classical_controls(cond))
    elif case == "reset":
        ops += [cirq.ResetChannel(dimension=3).on(q3), _Unitary((3,), 6).on(q3)]
    ops.append(cirq.measure(q3, q4, key="b"))
    ops.append(cirq.measure(q2, key="c"))
    c = cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)
    ref_cls = cirq.DensityMatrixSimulator if dm else cirq.Simulator
    ours_cls = cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator
    reps = 1500
    want = ref_cls(seed=1).run(c, repetitions=reps)
    got = ours_cls(seed=2).run(c, repetitions=reps)
    assert set(got.records) == set(want.records)
    dims = {"a": (3, 2), "b": (3, 4), "c": (2,)}
    for key in want.records:
        assert got.records[key].shape == want.records[key].shape, key
        assert got.records[key].max() < max(dims[key])
        assert _two_sample_p(_codes(want, key, dims[key]), _codes(got, key, dims[key])) > 1e-3, key


@pytest.mark.parametrize("dm", [False, True])
def test_simulate_measurements_and_moment_steps(emu, dm):
    q3, q2 = cirq.LineQid(0, dimension=3), cirq.LineQubit(1)
    c = cirq.Circuit(_Unitary((3, 2), 11).on(q3, q2), cirq.measure(q3, key="m"), _Unitary((3,), 12).on(q3))
    ours = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=3)
    ref = (cirq.DensityMatrixSimulator if dm else cirq.Simulator)(seed=4)
    got = np.array([int(ours.simulate(c).measurements["m"][0]) for _ in range(300)])
    want = np.array([int(ref.simulate(c).measurements["m"][0]) for _ in range(300)])
    assert set(got) <= {0, 1, 2}
    assert _two_sample_p(want, got) > 1e-3
    u = cirq.Circuit(_Unitary((3, 2), 13).on(q3, q2), _Phase(3, 0.7).on(q3), _Unitary((3,), 14).on(q3))
    # step results are live views of the state: compare them in lockstep
    ref_steps = (cirq.DensityMatrixSimulator if dm else cirq.Simulator)(dtype=np.complex128).simulate_moment_steps(u)
    n = 0
    for step, w in zip(ours.simulate_moment_steps(u), ref_steps):
        if dm:
            np.testing.assert_allclose(step.density_matrix(), w.density_matrix(), atol=1e-5)
        else:
            np.testing.assert_allclose(step.state_vector(), w.state_vector(), atol=1e-5)
            assert cirq.qid_shape(step) == (3, 2)
        s = step.sample([q3], repetitions=50)
        assert s.shape == (50, 1) and s.max() <= 2
        n += 1
    assert n == 3


def test_wide_qudit_unitary_without_decomposition_raises(emu):
    q = cirq.LineQid.range(3, dimension=3)
    c = cirq.Circuit(_Unitary((3, 3, 3), 1).on(*q))
    with pytest.raises(NotImplementedError, match="index bits"):
        cirq_gb300.Simulator().simulate(c)


def test_qudit_module_functions(emu):
    q3, q2 = cirq.LineQid(0, dimension=3), cirq.LineQubit(1)
    c = cirq.Circuit(_Unitary((3, 2), 21).on(q3, q2))
    np.testing.assert_allclose(cirq_gb300.final_state_vector(c), cirq.final_state_vector(c, dtype=np.complex128),
                               atol=1e-5)
    np.testing.assert_allclose(cirq_gb300.final_density_matrix(c),
                               cirq.final_density_matrix(c, dtype=np.complex128), atol=1e-5)
    s = cirq_gb300.sample(c + cirq.measure(q3, q2, key="z"), repetitions=200, seed=1)
    assert s.records["z"].shape == (200, 1, 2) and s.records["z"][:, 0, 0].max() <= 2


GOLD = np.load(__file__.replace("test_qudits_emulated.py", "golden/golden.npz"))


def test_qudit_fixtures_vs_reference_golden(emu):
    import make_zoo

    mg = make_zoo.golden_module()
    c, order = mg._qudit_circuit(cirq)
    got = cirq_gb300.Simulator().simulate(c, qubit_order=order, initial_state=17).final_state_vector
    np.testing.assert_allclose(got, GOLD["qudit_sv_c128"], atol=1e-5)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(mg._qudit_noisy_circuit(cirq)).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["qudit_dm_c128"], atol=1e-5)


def test_noisy_qudit_sample_counts_state_bits(emu):
    """cirq.sample of a noisy circuit picks the density-matrix simulator by
    state bits: 8 qutrits are 16 bits, beyond its 14, so they run as
    trajectories (a density matrix would need 32 bits)."""
    from cirq_gb300 import mux

    q = cirq.LineQid.range(8, dimension=3)
    assert mux._state_bits(q) == 16 and mux._state_bits(cirq.LineQubit.range(5)) == 5
    c = cirq.Circuit(_Shift().on(x) for x in q) + cirq.measure(*q, key="z")
    s = cirq_gb300.sample(c, repetitions=300, seed=2, noise=cirq.NO_NOISE)
    assert s.records["z"].shape == (300, 1, 8) and s.records["z"].max() <= 2
    shifted = (s.records["z"][:, 0, :] > 0).mean()
    assert abs(shifted - 0.4) < 0.05
