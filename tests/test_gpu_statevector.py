"""State-vector parity on the GPU: cirq_gb300.Simulator vs the reference's
golden states and the complex128 CPU oracle."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import workloads
from oracle.circuits import simulate_state_vector

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_statevector.py", "golden/golden.npz"))
TOL = 1e-5  # max amplitude error for complex64


@pytest.mark.parametrize("n,d,s", [(10, 20, 1), (12, 8, 2), (5, 6, 3)])
@pytest.mark.parametrize(
    "cfg",
    [
        dict(),
        dict(tile_bits=10, fusion_max_qubits=3, pass_budget=20),
        dict(tile_bits=10, fusion_max_qubits=2, pass_budget=8),
        dict(tile_bits=11, fusion_max_qubits=5, pass_budget=200),
        dict(tile_bits=13, fusion_max_qubits=1, pass_budget=10),
    ],
)
def test_layers_vs_golden(n, d, s, cfg):
    c = workloads.random_layer_circuit(n, d, s)
    got = cirq_gb300.Simulator(**cfg).simulate(c).final_state_vector
    assert got.dtype == np.complex64
    np.testing.assert_allclose(got, GOLD[f"layers_n{n}_d{d}_s{s}_c128"], atol=TOL)
    np.testing.assert_allclose(got, GOLD[f"layers_n{n}_d{d}_s{s}_c64"], atol=TOL)


def test_reversed_order_and_initial_state():
    c = workloads.random_layer_circuit(6, 5, 4)
    q = sorted(c.all_qubits())
    got = cirq_gb300.Simulator().simulate(c, qubit_order=q[::-1], initial_state=5).final_state_vector
    np.testing.assert_allclose(got, GOLD["layers_n6_d5_s4_reversed_init5"], atol=TOL)


def test_gate_zoo():
    import make_zoo

    zoo = make_zoo.gate_zoo()
    got = cirq_gb300.Simulator().simulate(zoo).final_state_vector
    np.testing.assert_allclose(got, GOLD["zoo_c128"], atol=TOL)


@pytest.mark.parametrize("n", [16, 18, 20])
def test_larger_vs_oracle(n):
    c = workloads.random_layer_circuit(n, 10, seed=n)
    got = cirq_gb300.Simulator().simulate(c).final_state_vector
    want = simulate_state_vector(c)
    assert np.max(np.abs(got - want)) < TOL


def test_known_expectations():
    """Known answers of the reference's own test (sparse_simulator_test.py:630-651)."""
    q0, q1 = cirq.LineQubit.range(2)
    psum1 = cirq.Z(q0) + 3.2 * cirq.Z(q1)
    psum2 = -1 * cirq.X(q0) + 2 * cirq.X(q1)
    sim = cirq_gb300.Simulator()
    r = sim.simulate_expectation_values(cirq.Circuit(cirq.I(q0), cirq.X(q1)), [psum1, psum2])
    np.testing.assert_allclose(np.real(r), GOLD["known_expect_c1"], atol=1e-6)
    r = sim.simulate_expectation_values(cirq.Circuit(cirq.H(q0), cirq.H(q1)), [psum1, psum2])
    np.testing.assert_allclose(np.real(r), GOLD["known_expect_c2"], atol=1e-6)
    r = sim.simulate_expectation_values(cirq.Circuit(cirq.I(q0), cirq.H(q1)), cirq.Z(q0) + cirq.X(q1))
    np.testing.assert_allclose(np.real(r), GOLD["known_expect_c3"], atol=1e-6)


def test_cuda_graph_sweep_matches_plain_path():
    """Graph capture + replay over a sweep gives the same states as plain launches."""
    import sympy

    t = sympy.Symbol("t")
    q = cirq.LineQubit.range(12)
    c = workloads.random_layer_circuit(12, 6, seed=9) + cirq.Circuit(cirq.rx(t).on_each(*q))
    pts = cirq.Points("t", [0.0, 0.3, -1.2, 2.5])
    plain = cirq_gb300.Simulator().simulate_sweep(c, pts)
    graph_sim = cirq_gb300.Simulator(use_cuda_graphs=True)
    graphed = graph_sim.simulate_sweep(c, pts)
    again = graph_sim.simulate_sweep(c, pts)  # replays the captured graph
    for a, b, d in zip(plain, graphed, again):
        np.testing.assert_allclose(a.final_state_vector, b.final_state_vector, atol=1e-6)
        np.testing.assert_allclose(a.final_state_vector, d.final_state_vector, atol=1e-6)
    # and against the complex128 oracle, point by point
    for r, b in zip(cirq.to_resolvers(pts), again):
        assert np.max(np.abs(b.final_state_vector - simulate_state_vector(c, r))) < TOL


def test_cuda_graph_sweep_vs_reference_golden():
    """Graph replay over the reference's QAOA sweep (golden expectation values)."""
    circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(8, 4, seed=7)
    pts = GOLD["qaoa_n8_p4_points"]
    res = [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]
    sim = cirq_gb300.Simulator(use_cuda_graphs=True)
    for _ in range(2):  # capture, then replay
        vals = sim.simulate_expectation_values_sweep(circuit, obs, res)
        np.testing.assert_allclose(np.array([v[0] for v in vals]), GOLD["qaoa_n8_p4_expect"], atol=1e-4)
    for r, tr in zip(res[:4], sim.simulate_sweep(circuit, res[:4])):
        assert np.max(np.abs(tr.final_state_vector - simulate_state_vector(circuit, r))) < TOL


def test_autotuned_simulator_matches_oracle(tmp_path, monkeypatch):
    monkeypatch.setenv("CIRQ_GB300_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    c = workloads.random_layer_circuit(18, 8, seed=44)
    got = cirq_gb300.Simulator(autotune=True).simulate(c).final_state_vector
    want = simulate_state_vector(c)
    assert np.max(np.abs(got - want)) < TOL
    assert (tmp_path / "tune.json").exists()


def _final_device_norm_and_state(sim, circuit):
    """Runs the plan on the device and returns (norm^2 before any host-side
    renormalisation, final state)."""
    eng = sim.engine
    qubits, resolvers, compiled, _ = sim._prepare(circuit, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))
    state = sim._evolve(compiled, compiled.pool([cirq.ParamResolver({})])[0], 0)
    try:
        return eng.norm2(state, compiled.n), eng.download_state(state, compiled.n, pinned=False)
    finally:
        state.free()


def test_full_size_properties_26_qubits():
    """Bench-like size (the oracle is too slow here): norm preservation over
    a 26-qubit, depth-40 run with thousands of tiles per launch, bit-identical
    reruns (the kernels are deterministic), and agreement with a plan of
    13-bit tiles that runs on a different kernel."""
    c = workloads.random_layer_circuit(26, 40, seed=0)
    sim = cirq_gb300.Simulator()
    n1, v1 = _final_device_norm_and_state(sim, c)
    assert abs(n1 - 1) < 1e-5
    n2, v2 = _final_device_norm_and_state(sim, c)
    assert np.array_equal(v1, v2)
    n3, v3 = _final_device_norm_and_state(cirq_gb300.Simulator(tile_bits=13), c)
    assert abs(n3 - 1) < 1e-5
    assert np.abs(v1 - v3).max() < 1e-5


def test_33_qubit_properties():
    """The largest configured width (33 qubits, a 64 GiB state): device-side
    norm after a depth-8 random-layer circuit, bit-identical reruns, and
    agreement with a plan of 13-bit tiles on sampled amplitudes."""
    import cirq_gb300.engine as engine_mod

    eng = engine_mod.default_engine()
    _, free, _ = eng.device_info()
    if free < (72 << 30):
        pytest.skip("needs 72 GiB of free device memory")
    c = workloads.random_layer_circuit(33, 8, seed=4)
    idx = np.random.RandomState(0).randint(0, 2**33, size=4096)

    def run(sim):
        qubits, resolvers, compiled, _ = sim._prepare(c, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))
        state = sim._evolve(compiled, compiled.pool(resolvers)[0], 0)
        try:
            norm = eng.norm2(state, compiled.n)
            # sampled amplitudes: one small device-to-host copy per index
            vals = np.empty(len(idx), np.complex64)
            one = np.empty(1, np.complex64)
            for j, i in enumerate(idx):
                eng.lib.gbq_d2h(eng.ctx, one.ctypes.data, state.ptr + 8 * int(i), 8)
                vals[j] = one[0]
            return norm, vals
        finally:
            state.free()

    n1, a1 = run(cirq_gb300.Simulator())
    assert abs(n1 - 1) < 1e-5
    n2, a2 = run(cirq_gb300.Simulator())
    assert np.array_equal(a1, a2)
    n3, a3 = run(cirq_gb300.Simulator(tile_bits=13))
    assert abs(n3 - 1) < 1e-5
    assert np.abs(a1 - a3).max() < 1e-6
