"""The public API (simulators, module helpers, trajectories, noise
placement) driven end to end on the CPU emulation of the engine, against the
reference's own results (golden) and the oracle.  This checks the package's
host logic without a GPU; the GPU tests run the same paths on the kernels.
CPU only: the emulated engine is test infrastructure."""

import numpy as np
import pytest
import scipy.stats
import sympy

import cirq
import cirq_gb300
from cirq_gb300 import simulator as sim_mod
from cirq_gb300 import workloads
from cpu_engine import EmuEngine
from oracle.circuits import simulate_density_matrix, simulate_state_vector

GOLD = np.load(__file__.replace("test_simulators_emulated.py", "golden/golden.npz"))


@pytest.fixture
def emu(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    return eng


def _chi2_p(counts, probs):
    keep = probs > 1e-12
    exp = probs[keep] / probs[keep].sum() * counts[keep].sum()
    return scipy.stats.chisquare(counts[keep], exp).pvalue


def test_state_vectors_vs_golden(emu):
    for n, d, s in [(10, 20, 1), (5, 6, 3)]:
        c = workloads.random_layer_circuit(n, d, s)
        got = cirq_gb300.Simulator().simulate(c).final_state_vector
        np.testing.assert_allclose(got, GOLD[f"layers_n{n}_d{d}_s{s}_c128"], atol=1e-5)
    c = workloads.random_layer_circuit(6, 5, 4)
    q = sorted(c.all_qubits())
    got = cirq_gb300.Simulator().simulate(c, qubit_order=q[::-1], initial_state=5).final_state_vector
    np.testing.assert_allclose(got, GOLD["layers_n6_d5_s4_reversed_init5"], atol=1e-5)
    assert emu.launches() > 0


def test_density_matrices_vs_golden(emu):
    c = workloads.noisy_layer_circuit(4, 4, seed=2, p=0.05, gamma=0.1)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisy_n4_d4"], atol=1e-5)
    c = workloads.random_layer_circuit(3, 3, seed=5)
    rho = cirq_gb300.DensityMatrixSimulator(noise=cirq.depolarize(0.02)).simulate(c).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisemodel_n3"], atol=1e-5)
    import make_zoo

    pc, r = make_zoo.golden_module()._noisy_param_circuit(cirq, sympy)
    rho = cirq_gb300.DensityMatrixSimulator(noise=cirq.amplitude_damp(0.2)).simulate(pc, r).final_density_matrix
    np.testing.assert_allclose(rho, GOLD["dm_noisy_param_split"], atol=1e-5)


def test_module_helpers_vs_golden(emu):
    import make_zoo

    cc = make_zoo.fixture_circuit("_classical_control_circuit")
    np.testing.assert_allclose(cirq_gb300.final_density_matrix(cc), GOLD["mux_fdm_classical_control"], atol=1e-5)
    meas = make_zoo.fixture_circuit("_measured_circuit")
    np.testing.assert_allclose(cirq_gb300.final_density_matrix(meas), GOLD["mux_fdm_dephased"], atol=1e-5)
    np.testing.assert_allclose(
        cirq_gb300.final_density_matrix(meas, noise=cirq.amplitude_damp(0.1)), GOLD["mux_fdm_dephased_noisy"],
        atol=1e-5,
    )
    q = sorted(meas.all_qubits())
    got = cirq_gb300.final_state_vector(meas, ignore_terminal_measurements=True, qubit_order=q[::-1])
    np.testing.assert_allclose(got, GOLD["mux_fsv_ignore_terminal"], atol=1e-5)
    wide = make_zoo.fixture_circuit("_wide_controlled_circuit")
    np.testing.assert_allclose(cirq_gb300.Simulator().simulate(wide).final_state_vector,
                               GOLD["wide_controlled_c128"], atol=1e-5)


def test_expectation_values_vs_reference_known_answers(emu):
    # the reference's own known answers (sparse_simulator_test.py:630-651)
    q0, q1 = cirq.LineQubit.range(2)
    psum1 = cirq.Z(q0) + 3.2 * cirq.Z(q1)
    psum2 = -1 * cirq.X(q0) + 2 * cirq.X(q1)
    c1 = cirq.Circuit(cirq.I(q0), cirq.X(q1))
    got = cirq_gb300.Simulator().simulate_expectation_values(c1, [psum1, psum2])
    np.testing.assert_allclose(got, GOLD["known_expect_c1"], atol=1e-5)
    c2 = cirq.Circuit(cirq.H(q0), cirq.H(q1))
    got = cirq_gb300.Simulator().simulate_expectation_values(c2, [psum1, psum2])
    np.testing.assert_allclose(got, GOLD["known_expect_c2"], atol=1e-5)


def test_run_samples_terminal_and_noisy(emu):
    q = cirq.LineQubit.range(3)
    body = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(1.1).on(q[2]))
    c = body + cirq.measure(*q, key="m")
    reps = 4000
    for sim, placed in [
        (cirq_gb300.Simulator(seed=1), body),
        (cirq_gb300.DensityMatrixSimulator(seed=2), body),
    ]:
        bits = sim.run(c, repetitions=reps).records["m"][:, 0, :]
        p = np.real(np.diag(simulate_density_matrix(placed, qubit_order=q)))
        idx = bits.astype(int) @ np.array([4, 2, 1])
        assert _chi2_p(np.bincount(idx, minlength=8), p) > 1e-3
    # noise model: the density-matrix run's placement (noise after the
    # three-qubit terminal measurement acts before sampling)
    noise = cirq.amplitude_damp(0.25)
    dm = cirq_gb300.DensityMatrixSimulator(noise=noise, seed=3)
    placed = dm._reference_noisy_circuit(c, "run")
    pbody = cirq.Circuit(op for op in placed.all_operations() if not cirq.is_measurement(op))
    p = np.real(np.diag(simulate_density_matrix(pbody, qubit_order=q)))
    bits = dm.run(c, repetitions=reps).records["m"][:, 0, :]
    assert _chi2_p(np.bincount(bits.astype(int) @ np.array([4, 2, 1]), minlength=8), p) > 1e-3


def test_batched_state_vector_trajectories(emu):
    """Noise on the state vector: all repetitions evolve together (batched
    points, reduced density matrices for the Kraus weights, batched terminal
    sampling); the records follow the density matrix's distribution."""
    q = cirq.LineQubit.range(3)
    body = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.ry(0.8).on(q[2]), cirq.CZ(q[1], q[2]))
    noise = cirq.ConstantQubitNoiseModel(cirq.amplitude_damp(0.2))
    rho = simulate_density_matrix(body, qubit_order=q, noise=noise)
    reps = 3000
    sim = cirq_gb300.Simulator(noise=noise, seed=4)
    bits = sim.run(body + cirq.measure(*q, key="m"), repetitions=reps).records["m"][:, 0, :]
    p = np.real(np.diag(rho))
    assert _chi2_p(np.bincount(bits.astype(int) @ np.array([4, 2, 1]), minlength=8), p) > 1e-3
    # batched: far fewer "launches" than repetitions
    assert emu.launches() < reps


def test_mid_circuit_measurement_and_classical_control(emu):
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.H(q[0]),
        cirq.measure(q[0], key="a"),
        cirq.X(q[1]).with_classical_controls("a"),
        cirq.ry(0.9).on(q[2]),
        cirq.measure(q[2], key="c"),
        cirq.CNOT(q[1], q[2]).with_classical_controls("c"),
        cirq.measure(q[1], q[2], key="m"),
        strategy=cirq.InsertStrategy.NEW,
    )
    for sim in (cirq_gb300.Simulator(seed=5), cirq_gb300.DensityMatrixSimulator(seed=6)):
        res = sim.run(c, repetitions=300)
        a = res.records["a"][:, 0, 0]
        cc = res.records["c"][:, 0, 0]
        m = res.records["m"][:, 0, :]
        np.testing.assert_array_equal(m[:, 0], a)
        np.testing.assert_array_equal(m[:, 1], cc ^ (cc & a))
    r = cirq_gb300.Simulator(seed=7).simulate(c[:-1])
    a, cc = int(r.measurements["a"][0]), int(r.measurements["c"][0])
    want = np.zeros(8)
    want[(a << 2) | (a << 1) | (cc ^ (cc & a))] = 1
    np.testing.assert_allclose(np.abs(r.final_state_vector) ** 2, want, atol=1e-5)


def test_moment_steps(emu):
    c = workloads.random_layer_circuit(4, 3, seed=2)
    q = sorted(c.all_qubits())
    # a step's state is a view of the live simulation, valid until the next
    # step (as in the reference), so it is read inside the loop
    count = 0
    for i, st in enumerate(cirq_gb300.Simulator().simulate_moment_steps(c)):
        want = simulate_state_vector(c[: i + 1], qubit_order=q)
        np.testing.assert_allclose(st.state_vector(), want, atol=1e-5)
        count += 1
    assert count == len(c)


def test_overlapping_final_measurements(emu):
    """Measurements of the same qubits at the end commute: all read one
    sampled basis state (the reference's test_overlapping_measurements_at_end)."""
    a, b = cirq.LineQubit.range(2)
    c = cirq.Circuit(
        cirq.H(a),
        cirq.CNOT(a, b),
        cirq.measure(a, key="a"),
        cirq.measure(a, key="not a", invert_mask=(True,)),
        cirq.measure(b, key="b"),
        cirq.measure(a, b, key="ab"),
    )
    for sim in (cirq_gb300.Simulator(seed=1), cirq_gb300.DensityMatrixSimulator(seed=2)):
        m = sim.run(c, repetitions=200).measurements
        np.testing.assert_array_equal(m["a"][:, 0], m["not a"][:, 0] ^ 1)
        np.testing.assert_array_equal(m["a"][:, 0] * 2 + m["b"][:, 0], m["ab"][:, 0] * 2 + m["ab"][:, 1])
        assert 20 <= int(m["b"].sum()) <= 180


def _blocks_circuit(nblocks, seed):
    """Independent 3-qubit blocks (H, CNOT chain, a rotation): a GHZ-like
    pair per block and one rotated qubit."""
    rng = np.random.default_rng(seed)
    q = cirq.LineQubit.range(3 * nblocks)
    ops = []
    thetas = rng.uniform(0.3, 2.5, size=nblocks)
    for b in range(nblocks):
        a, c, d = q[3 * b], q[3 * b + 1], q[3 * b + 2]
        ops += [cirq.H(a), cirq.CNOT(a, c), cirq.ry(float(thetas[b])).on(d), cirq.CZ(c, d)]
    return q, cirq.Circuit(ops), thetas


def test_run_of_untangled_circuits_beyond_the_device_state(emu):
    """36 qubits in 12 independent blocks (a 2^36 state would not fit):
    run() simulates the blocks one at a time and reassembles the records."""
    q, body, thetas = _blocks_circuit(12, seed=3)
    c = body + cirq.measure(*q, key="all") + cirq.measure(q[0], q[4], key="pair")
    reps = 400
    res = cirq_gb300.Simulator(seed=9).run(c, repetitions=reps)
    ref = cirq.Simulator(seed=9).run(c, repetitions=5)
    assert res.records["all"].shape == (reps,) + ref.records["all"].shape[1:] == (reps, 1, 36)
    assert res.records["pair"].shape == (reps, 1, 2)
    bits = res.records["all"][:, 0, :]
    # within every block the first two qubits agree (H + CNOT)
    np.testing.assert_array_equal(bits[:, 0::3], bits[:, 1::3])
    # the rotated qubit of each block: P(1) = sin^2(theta / 2)
    for b in range(12):
        p1 = np.sin(thetas[b] / 2) ** 2
        n1 = int(bits[:, 3 * b + 2].sum())
        assert scipy.stats.binomtest(n1, reps, p1).pvalue > 1e-4
    # the split measurement reads the same sampled state
    np.testing.assert_array_equal(res.records["pair"][:, 0, 0], bits[:, 0])
    np.testing.assert_array_equal(res.records["pair"][:, 0, 1], bits[:, 4])


def test_unmeasured_components_are_not_simulated(emu):
    q = cirq.LineQubit.range(40)
    big = cirq.Circuit(cirq.H(q[0]), *[cirq.CNOT(q[i], q[i + 1]) for i in range(33)])  # 34 entangled qubits
    small = cirq.Circuit(cirq.X(q[36]), cirq.H(q[38]))
    c = big + small + cirq.measure(q[36], q[38], key="m")
    res = cirq_gb300.Simulator(seed=1).run(c, repetitions=200)
    m = res.records["m"][:, 0, :]
    assert (m[:, 0] == 1).all() and 0.3 < m[:, 1].mean() < 0.7


def test_noisy_density_matrix_run_of_untangled_blocks(emu):
    """18 qubits on the density-matrix simulator (2n = 36 bits): noise placed
    on the whole circuit first, then the blocks run one by one."""
    q, body, thetas = _blocks_circuit(6, seed=4)
    c = body + cirq.measure(*q, key="m")
    noise = cirq.amplitude_damp(0.2)
    dm = cirq_gb300.DensityMatrixSimulator(noise=noise, seed=2)
    reps = 600
    bits = dm.run(c, repetitions=reps).records["m"][:, 0, :]
    placed = dm._reference_noisy_circuit(c, "run")
    for b in range(6):
        qs = q[3 * b : 3 * b + 3]
        block = cirq.Circuit(op for op in placed.all_operations()
                             if set(op.qubits) <= set(qs) and not cirq.is_measurement(op))
        p = np.real(np.diag(simulate_density_matrix(block, qubit_order=qs)))
        idx = bits[:, 3 * b : 3 * b + 3].astype(int) @ np.array([4, 2, 1])
        assert _chi2_p(np.bincount(idx, minlength=8), p) > 1e-4


def test_simulate_of_untangled_circuits_beyond_the_device_state(emu):
    """simulate() of 36 untangled qubits: a product state of the blocks
    (the reference's SimulationProductState, merged only on demand)."""
    q, body, thetas = _blocks_circuit(12, seed=5)
    c = body + cirq.measure(q[0], q[3], key="m")
    res = cirq_gb300.Simulator(seed=3).simulate(c)
    st = res._final_simulator_state
    assert isinstance(st, cirq.SimulationProductState)
    assert set(st.qubits) == set(q)
    m = res.measurements["m"]
    assert m.shape == (2,)
    # an unmeasured block's state equals the oracle's
    blk = st.sim_states[q[6]]
    want = simulate_state_vector(cirq.Circuit(op for op in body.all_operations() if set(op.qubits) <= set(q[6:9])),
                                 qubit_order=q[6:9])
    np.testing.assert_allclose(blk.target_tensor.reshape(-1), want, atol=1e-5)
    # a measured block collapsed to its record: q[0] and q[1] agree with m[0]
    b0 = st.sim_states[q[0]].target_tensor.reshape(-1)
    probs = np.abs(b0) ** 2
    i = int(np.argmax(probs))
    assert ((i >> 2) & 1) == m[0] and ((i >> 1) & 1) == m[0]


def test_unnormalized_array_initial_state_is_taken_as_given(emu):
    """An ndarray initial state is not validated (the reference's
    _BufferedStateVector.create takes it as given); the final state keeps its
    norm and simulate() warns, as the reference does, that it skips
    renormalising."""
    q = cirq.LineQubit.range(11)
    c = workloads.random_layer_circuit(11, 3, seed=5)
    init = np.zeros(2**11, dtype=np.complex64)
    init[0] = 1.01
    with pytest.warns(UserWarning, match="skipping renormalization"):
        ref = cirq.Simulator(dtype=np.complex64).simulate(c, qubit_order=q, initial_state=init).final_state_vector
    with pytest.warns(UserWarning, match="skipping renormalization"):
        got = cirq_gb300.Simulator().simulate(c, qubit_order=q, initial_state=init).final_state_vector
    np.testing.assert_allclose(got, ref, atol=1e-5)
