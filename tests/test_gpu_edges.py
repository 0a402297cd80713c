"""Edge cases of the drop-in API on the GPU: empty and degenerate circuits,
zero repetitions, unresolved parameters, sweep objects, initial states,
amplitudes and non-line qubits.  Values are checked against the oracle;
shapes and dtypes of results against the reference simulator itself."""

import numpy as np
import pytest
import sympy

import cirq
import cirq_gb300
from cirq_gb300 import workloads
from oracle.circuits import simulate_density_matrix, simulate_state_vector

pytestmark = pytest.mark.gpu


def test_empty_circuit_and_idle_qubits():
    r = cirq_gb300.Simulator().simulate(cirq.Circuit())
    assert r.final_state_vector.shape == (1,) and abs(r.final_state_vector[0] - 1) < 1e-7
    q = cirq.LineQubit.range(3)
    r = cirq_gb300.Simulator().simulate(cirq.Circuit(), qubit_order=q, initial_state=6)
    want = np.zeros(8)
    want[6] = 1
    np.testing.assert_allclose(r.final_state_vector, want, atol=1e-7)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(cirq.Circuit(), qubit_order=q).final_density_matrix
    assert rho.shape == (8, 8) and abs(rho[0, 0] - 1) < 1e-7


def test_global_phase_only_and_single_qubit():
    c = cirq.Circuit(cirq.global_phase_operation(1j))
    r = cirq_gb300.Simulator().simulate(c)
    np.testing.assert_allclose(r.final_state_vector, [1j], atol=1e-7)
    q = cirq.LineQubit(0)
    c1 = cirq.Circuit(cirq.rx(0.3).on(q), cirq.global_phase_operation(-1), cirq.rz(1.1).on(q))
    np.testing.assert_allclose(
        cirq_gb300.Simulator().simulate(c1).final_state_vector, simulate_state_vector(c1), atol=1e-6
    )


def test_zero_repetitions_shapes_match_reference():
    q = cirq.LineQubit.range(3)
    for c in (
        cirq.Circuit(cirq.H(q[0]), cirq.measure(*q, key="m")),
        cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0], key="a"), cirq.X(q[1]), cirq.measure(q[1], key="b")),
    ):
        ours = cirq_gb300.Simulator().run(c, repetitions=0)
        ref = cirq.Simulator().run(c, repetitions=0)
        assert set(ours.records) == set(ref.records)
        for k in ref.records:
            assert ours.records[k].shape == ref.records[k].shape


def test_run_result_types_match_reference():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(cirq.H.on_each(*q), cirq.measure(q[0], q[2], key="m"))
    ours = cirq_gb300.Simulator(seed=1).run(c, repetitions=7)
    ref = cirq.Simulator(seed=1).run(c, repetitions=7)
    assert ours.measurements["m"].shape == ref.measurements["m"].shape
    assert ours.measurements["m"].dtype == ref.measurements["m"].dtype


def test_unresolved_symbols_raise_like_the_reference():
    q = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.rx(sympy.Symbol("t")).on(q), cirq.measure(q, key="m"))
    with pytest.raises(ValueError):
        cirq_gb300.Simulator().run(c)
    with pytest.raises(ValueError):
        cirq_gb300.Simulator().simulate(c)
    with pytest.raises(ValueError):
        cirq_gb300.DensityMatrixSimulator().simulate(c)


def test_complex128_is_rejected():
    with pytest.raises(ValueError):
        cirq_gb300.Simulator(dtype=np.complex128)


def test_sweep_objects_and_amplitudes():
    c, syms = workloads.random_layer_circuit(5, 4, seed=9), None
    t = sympy.Symbol("t")
    q = sorted(c.all_qubits())
    cp = c + cirq.Circuit(cirq.rx(t).on(q[0]), cirq.CZ(q[0], q[1]) ** t)
    sweep = cirq.Linspace(t, 0, 1, 5) * cirq.Points("u", [0.0])
    results = cirq_gb300.Simulator().simulate_sweep(cp, sweep)
    assert len(results) == 5
    for r in results:
        want = simulate_state_vector(cp, r.params)
        np.testing.assert_allclose(r.final_state_vector, want, atol=1e-5)
    amps = cirq_gb300.Simulator().compute_amplitudes(cp, [0, 5, 31], param_resolver={"t": 0.25})
    want = simulate_state_vector(cp, cirq.ParamResolver({"t": 0.25}))
    np.testing.assert_allclose(amps, want[[0, 5, 31]], atol=1e-5)


def test_state_vector_initial_states_both_simulators():
    q = cirq.LineQubit.range(4)
    c = workloads.random_layer_circuit(4, 3, seed=2)
    rs = np.random.RandomState(3)
    psi = rs.normal(size=16) + 1j * rs.normal(size=16)
    psi /= np.linalg.norm(psi)
    got = cirq_gb300.Simulator().simulate(c, qubit_order=q, initial_state=psi.astype(np.complex64))
    u = cirq.unitary(cirq.Circuit(c.all_operations()).transform_qubits(lambda x: x))
    np.testing.assert_allclose(got.final_state_vector, cirq.final_state_vector(c, qubit_order=q, initial_state=psi.astype(np.complex64)), atol=1e-5)
    rho0 = np.outer(psi, psi.conj())
    dm = cirq_gb300.DensityMatrixSimulator().simulate(c, qubit_order=q, initial_state=rho0.astype(np.complex64))
    want = u @ rho0 @ u.conj().T
    np.testing.assert_allclose(dm.final_density_matrix, want, atol=1e-5)


def test_grid_and_named_qubits_keep_the_reference_order():
    qs = [cirq.GridQubit(1, 0), cirq.GridQubit(0, 1), cirq.NamedQubit("z"), cirq.NamedQubit("a")]
    c = cirq.Circuit(cirq.H(qs[0]), cirq.CNOT(qs[0], qs[2]), cirq.ry(0.4).on(qs[3]), cirq.CZ(qs[1], qs[3]))
    ours = cirq_gb300.Simulator().simulate(c)
    ref = cirq.Simulator().simulate(c)
    assert ours.qubit_map == ref.qubit_map
    np.testing.assert_allclose(ours.final_state_vector, ref.final_state_vector, atol=1e-6)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    np.testing.assert_allclose(rho, simulate_density_matrix(c), atol=1e-6)


def test_multi_controlled_gates_beyond_five_qubits():
    q = cirq.LineQubit.range(8)
    c = cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.X(q[6]).controlled_by(*q[:6]),
        cirq.rz(0.3).on(q[7]).controlled_by(*q[1:6]),
        cirq.CZ(q[0], q[7]),
    )
    got = cirq_gb300.Simulator().simulate(c).final_state_vector
    want = simulate_state_vector(c)
    assert np.max(np.abs(got - want)) < 2e-6
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    assert np.max(np.abs(rho - np.outer(want, want.conj()))) < 2e-6


def test_simulation_state_initial_states():
    c = workloads.random_layer_circuit(4, 3, seed=8)
    qs = sorted(c.all_qubits())
    order = [qs[3], qs[1], qs[0], qs[2]]
    st = cirq.StateVectorSimulationState(qubits=order, initial_state=9, dtype=np.complex64)
    r = cirq_gb300.Simulator().simulate(c, initial_state=st)
    want = simulate_state_vector(c, qubit_order=order, initial_state=9)
    assert np.max(np.abs(r.final_state_vector - want)) < 2e-6
    assert r.qubit_map == {qq: i for i, qq in enumerate(order)}
    # a product state from the reference's own simulator, and the density matrix
    prod = cirq.Simulator()._create_simulation_state(5, qs)
    r = cirq_gb300.Simulator().simulate(c, initial_state=prod)
    assert np.max(np.abs(r.final_state_vector - simulate_state_vector(c, initial_state=5))) < 2e-6
    dst = cirq.DensityMatrixSimulationState(qubits=qs, initial_state=5, dtype=np.complex64)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c, initial_state=dst).final_density_matrix
    assert np.max(np.abs(rho - simulate_density_matrix(c, initial_state=5))) < 2e-6


_CONFUSION = np.array([[0.9, 0.1], [0.2, 0.8]])


@pytest.mark.parametrize("dm", [False, True])
@pytest.mark.parametrize("where", ["terminal", "mid", "control"])
def test_invert_mask_and_confusion_map_orders(dm, where):
    """A qubit in |0>, measured with an invert mask and a confusion map: the
    record is 1 with p 0.9 where the measurement is performed in place
    (confusion, then invert) and 0.8 where run() samples terminal
    measurements at the end (invert, then confusion); a classical control
    reads the recorded value."""
    q0, q1 = cirq.LineQubit.range(2)
    ops = [cirq.I(q0), cirq.I(q1),
           cirq.measure(q0, key="a", invert_mask=(True,), confusion_map={(0,): _CONFUSION})]
    if where == "mid":
        ops.append(cirq.H(q0))
    elif where == "control":
        ops.append(cirq.X(q1).with_classical_controls("a"))
    ops.append(cirq.measure(q1, key="b"))
    c = cirq.Circuit(ops, strategy=cirq.InsertStrategy.NEW)
    sim = (cirq_gb300.DensityMatrixSimulator if dm else cirq_gb300.Simulator)(seed=11)
    res = sim.run(c, repetitions=4000)
    p1 = float(np.mean(res.records["a"][:, 0, 0]))
    assert abs(p1 - (0.8 if where == "terminal" else 0.9)) < 0.03
    if where == "control":
        np.testing.assert_array_equal(res.records["b"][:, 0, 0], res.records["a"][:, 0, 0])
    got = [int(sim.simulate(cirq.Circuit(ops[2])).measurements["a"][0]) for _ in range(300)]
    assert abs(np.mean(got) - 0.9) < 0.07


@pytest.mark.parametrize("delta,renormalized", [(3e-3, False), (5e-4, False), (2e-4, True), (1e-5, True)])
def test_device_final_renormalization_rule(delta, renormalized):
    """gbq_sv_final_renormalize on states whose norm is 1 + delta, on both
    sides of the reference's sqrt(eps) threshold
    (cirq-core/cirq/sim/state_vector_simulator.py:131-146): beyond it the
    state is returned unchanged (the reference warns and skips), within it
    the state is divided by its norm because that reduces the round-off of
    the total probability."""
    import ctypes

    from cirq_gb300 import _lib
    from oracle.statevector import renormalize_like_cirq

    n = 14
    psi = simulate_state_vector(workloads.random_layer_circuit(n, 6, seed=77)).astype(np.complex64)
    psi = (psi * np.float32(1 + delta)).astype(np.complex64)
    eng = cirq_gb300.Simulator().engine
    state = eng.upload(psi)
    applied = ctypes.c_int(-1)
    norm = ctypes.c_double()
    _lib.check(eng.lib.gbq_sv_final_renormalize(eng.ctx, state.ptr, n, ctypes.byref(applied), ctypes.byref(norm)),
               "renormalize")
    assert abs(norm.value - np.linalg.norm(psi.astype(np.complex128))) < 1e-6
    got = np.zeros_like(psi)
    state.download(got)
    want = renormalize_like_cirq(psi)
    assert applied.value == int(renormalized)
    assert np.array_equal(want, psi) == (not renormalized)  # the oracle takes the same branch
    if renormalized:
        np.testing.assert_allclose(got, psi / np.linalg.norm(psi.astype(np.complex128)), atol=1e-7)
        assert abs(np.linalg.norm(got.astype(np.complex128)) - 1) < 1e-6
    else:
        np.testing.assert_array_equal(got, psi)


def test_final_state_vector_of_an_unnormalized_initial_state():
    """The public path: an initial state off by more than sqrt(eps) comes
    back as simulated (no renormalisation), as in the reference."""
    q = cirq.LineQubit.range(12)
    c = workloads.random_layer_circuit(12, 3, seed=5)
    init = np.zeros(2**12, dtype=np.complex64)
    init[0] = 1.01
    with pytest.warns(UserWarning, match="skipping renormalization"):
        ref = cirq.Simulator(dtype=np.complex64).simulate(c, qubit_order=q, initial_state=init).final_state_vector
    with pytest.warns(UserWarning, match="skipping renormalization"):
        got = cirq_gb300.Simulator().simulate(c, qubit_order=q, initial_state=init).final_state_vector
    np.testing.assert_allclose(got, ref, atol=1e-5)
    assert abs(np.linalg.norm(got) - 1.01) < 1e-5


def _two_halves(n_half, depth):
    """Two independent random-layer registers of n_half qubits each."""
    a = workloads.random_layer_circuit(n_half, depth, seed=81)
    b = workloads.random_layer_circuit(n_half, depth, seed=82)
    qb = {cirq.LineQubit(i): cirq.LineQubit(n_half + i) for i in range(n_half)}
    return a, b.transform_qubits(lambda x: qb[x]), a + b.transform_qubits(lambda x: qb[x])


def test_untangled_36_qubit_simulate_per_component_vs_oracle():
    """simulate() of 36 qubits in two untangled 18-qubit halves (a 2^36 state
    does not fit one GPU): each half is simulated alone and held in the
    reference's product state (cirq-core/cirq/sim/simulation_product_state.py:31-181)."""
    a, b, c = _two_halves(18, 6)
    res = cirq_gb300.Simulator().simulate(c)
    st = res._final_simulator_state
    assert isinstance(st, cirq.SimulationProductState)
    for half in (a, b):
        q = sorted(half.all_qubits())
        comp = st.sim_states[q[0]]
        assert set(comp.qubits) == set(q)
        got = comp.target_tensor.reshape(-1)
        want = simulate_state_vector(half, qubit_order=list(comp.qubits))
        assert np.max(np.abs(got - want)) < 1e-5


def test_untangled_36_qubit_run_per_component_vs_oracle():
    a, b, c = _two_halves(18, 6)
    q = sorted(c.all_qubits())
    reps = 4000
    bits = cirq_gb300.Simulator(seed=4).run(c + cirq.measure(*q, key="m"), repetitions=reps).measurements["m"]
    assert bits.shape == (reps, 36)
    import scipy.stats

    for off, half in ((0, a), (18, b)):
        psi = simulate_state_vector(half, qubit_order=sorted(half.all_qubits()))
        p = (np.abs(psi) ** 2).reshape((8, -1)).sum(axis=1)  # first three qubits of the half
        idx = bits[:, off : off + 3].astype(int) @ np.array([4, 2, 1])
        counts = np.bincount(idx, minlength=8)
        keep = p * reps >= 5
        assert scipy.stats.chisquare(counts[keep], p[keep] * counts[keep].sum() / p[keep].sum()).pvalue > 1e-4
