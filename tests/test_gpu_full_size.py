"""Parity at the benchmarked sizes.

The reference's own simulators produced ``golden/golden_large.npz``
(``golden/make_golden_large.py``, complex128): the 20-qubit depth-20 and
24-qubit depth-40 random-layer states (seeded amplitude samples, norm,
every <Z_i>, a 4-qubit marginal), the 11-qubit depth-16 noisy density
matrix, QAOA expectation values at 16-22 qubits and the 16-qubit,
320-parameter hardware-efficient-ansatz gradient by parameter shift through
``cirq.Simulator.simulate_expectation_values``.  The 30-qubit depth-40 state
is checked against a complex128 run on the GPU that shares no code with the
tile passes (``gbq_sv64_*``: one plain double-precision pass per gate).

Tolerances: 1e-5 max amplitude error for complex64 states, 1e-4 absolute on
expectation values and gradients, chi^2 p-value > 1e-4 for samples.
"""

import numpy as np
import pytest
import scipy.stats

import cirq
import cirq_gb300
from cirq_gb300 import _lib, adjoint, batch, workloads

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_full_size.py", "golden/golden_large.npz"))
AMP_TOL = 1e-5
EXP_TOL = 1e-4


def _chi2_pvalue(counts, probs, reps):
    keep = probs * reps >= 5
    obs = np.concatenate([counts[keep], [counts[~keep].sum()]])
    exp = np.concatenate([probs[keep], [probs[~keep].sum()]]) * reps
    if exp[-1] == 0:
        obs, exp = obs[:-1], exp[:-1]
    return scipy.stats.chisquare(obs, exp * obs.sum() / exp.sum()).pvalue


def _z_values(psi, n):
    p = (np.abs(psi.astype(np.complex128)) ** 2).reshape((2,) * n)
    z = np.empty(n)
    for i in range(n):
        m = p.sum(axis=tuple(j for j in range(n) if j != i))
        z[i] = m[0] - m[1]
    return z


@pytest.mark.parametrize("n,depth", [(20, 20), (24, 40)])
def test_random_layers_vs_reference(n, depth):
    key = f"layers_n{n}_d{depth}_s0_c128"
    c = workloads.random_layer_circuit(n, depth, 0)
    psi = cirq_gb300.Simulator().simulate(c).final_state_vector
    idx = GOLD[f"{key}_idx"]
    err = np.max(np.abs(psi[idx] - GOLD[f"{key}_amps"]))
    assert err < AMP_TOL, err
    if f"layers_n{n}_d{depth}_s0_c64_amps" in GOLD:
        assert np.max(np.abs(psi[idx] - GOLD[f"layers_n{n}_d{depth}_s0_c64_amps"])) < AMP_TOL
    assert abs(np.linalg.norm(psi.astype(np.complex128)) - GOLD[f"{key}_norm"]) < 1e-5
    np.testing.assert_allclose(_z_values(psi, n), GOLD[f"{key}_z"], atol=EXP_TOL)


def test_run_20_qubits_10k_repetitions_vs_reference():
    n, reps = 20, 10_000
    key = "layers_n20_d20_s0_c128"
    c = workloads.random_layer_circuit(n, 20, 0)
    q = sorted(c.all_qubits())
    res = cirq_gb300.Simulator(seed=5).run(c + cirq.measure(*q, key="m"), repetitions=reps)
    bits = res.measurements["m"]
    assert bits.shape == (reps, n)
    idx4 = bits[:, :4].astype(int) @ np.array([8, 4, 2, 1])
    assert _chi2_pvalue(np.bincount(idx4, minlength=16), GOLD[f"{key}_marg4"], reps) > 1e-4
    # every qubit's frequency of 1 against the reference's (1 - <Z_i>) / 2
    p1 = (1 - GOLD[f"{key}_z"]) / 2
    for i in range(n):
        assert scipy.stats.binomtest(int(bits[:, i].sum()), reps, p1[i]).pvalue > 1e-5


def test_noisy_density_matrix_11_qubits_vs_reference():
    n, depth = 11, 16
    key = f"noisy_n{n}_d{depth}"
    c = workloads.noisy_layer_circuit(n, depth, seed=0, p=1e-3, gamma=5e-3)
    rho = cirq_gb300.DensityMatrixSimulator().simulate(c).final_density_matrix
    assert np.max(np.abs(np.real(np.diagonal(rho)) - GOLD[f"{key}_diag"])) < AMP_TOL
    got = rho[GOLD[f"{key}_rows"], GOLD[f"{key}_cols"]]
    assert np.max(np.abs(got - GOLD[f"{key}_entries"])) < AMP_TOL
    assert abs(np.trace(rho) - GOLD[f"{key}_trace"]) < EXP_TOL
    assert np.max(np.abs(rho - rho.conj().T)) < 1e-6


def test_noisy_density_matrix_11_qubits_100k_samples():
    n, depth, reps = 11, 16, 100_000
    c = workloads.noisy_layer_circuit(n, depth, seed=0, p=1e-3, gamma=5e-3)
    q = sorted(c.all_qubits())
    res = cirq_gb300.DensityMatrixSimulator(seed=7).run(c + cirq.measure(*q, key="m"), repetitions=reps)
    idx = res.measurements["m"].astype(int) @ (1 << np.arange(n - 1, -1, -1))
    probs = np.clip(GOLD[f"noisy_n{n}_d{depth}_diag"], 0, None)
    assert _chi2_pvalue(np.bincount(idx, minlength=2**n), probs / probs.sum(), reps) > 1e-4


@pytest.mark.parametrize("persistent", [False, True])
def test_qaoa_points_16_to_22_qubits_vs_reference(persistent):
    jobs, want = [], []
    for n in (16, 18, 20, 22):
        circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(n, 4, seed=n)
        pts = GOLD[f"qaoa_n{n}_points"]
        res = [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]
        jobs.append(batch.BatchJob(circuit, obs, res))
        want.append(GOLD[f"qaoa_n{n}_expect"])
    got = batch.simulate_expectation_values_batch(jobs, persistent=persistent)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g[:, 0], w, atol=EXP_TOL)


def test_hea_16_qubit_gradient_vs_reference_parameter_shift():
    circuit, symbols, values = workloads.hea_circuit(16, 10, seed=0)
    np.testing.assert_array_equal(values, GOLD["hea_n16_l10_values"])
    ham = workloads.random_pauli_hamiltonian(16, 300, seed=1)
    E, g = adjoint.AdjointProgram(circuit, ham, symbols).value_and_grad(values)
    assert abs(E - float(GOLD["hea_n16_l10_energy"])) < EXP_TOL
    assert g.shape == (320,)
    np.testing.assert_allclose(g, GOLD["hea_n16_l10_grad_ps"], atol=EXP_TOL)


def _complex128_gpu_run(eng, circuit, n):
    """The circuit's state at complex128 on the device, one gbq_sv64 pass per gate."""
    q = sorted(circuit.all_qubits())
    index = {x: i for i, x in enumerate(q)}
    state = eng.alloc(16 << n)
    _lib.check(eng.lib.gbq_sv64_set_basis(eng.ctx, state.ptr, n, 0), "gbq_sv64_set_basis")
    for op in circuit.all_operations():
        bits = np.array([n - 1 - index[x] for x in reversed(op.qubits)], dtype=np.int32)
        m = np.ascontiguousarray(cirq.unitary(op), dtype=np.complex128)
        _lib.check(
            eng.lib.gbq_sv64_apply(eng.ctx, state.ptr, n, len(bits), bits.ctypes.data, m.ctypes.data),
            "gbq_sv64_apply",
        )
    return state


def _compare(eng, s64, s32, n):
    out = np.zeros(3)
    _lib.check(eng.lib.gbq_sv64_compare(eng.ctx, s64.ptr, s32.ptr, n, out.ctypes.data), "gbq_sv64_compare")
    return out


def test_complex128_gpu_path_matches_the_oracle():
    """The double-precision check path itself, pinned at 12 qubits."""
    from oracle.circuits import simulate_state_vector

    n = 12
    c = workloads.random_layer_circuit(n, 10, seed=41)
    sim = cirq_gb300.Simulator()
    eng = sim.engine
    s64 = _complex128_gpu_run(eng, c, n)
    host = np.zeros(2**n, dtype=np.complex128)
    s64.download(host)
    assert np.max(np.abs(host - simulate_state_vector(c))) < 1e-12
    s64.free()


def test_30_qubit_depth_40_vs_complex128_gpu_run():
    """BASELINE config 2's check: the benchmarked 30-qubit state (complex64
    tile passes, the bench's planner settings) against a complex128 run of
    the same circuit on the GPU."""
    n = 30
    eng = cirq_gb300.Simulator().engine
    _, free, _ = eng.device_info()
    if free < (26 << 30):
        pytest.skip(f"needs 26 GiB of free device memory, {free >> 30} GiB free")
    c = workloads.random_layer_circuit(n, 40, 0)
    sim = cirq_gb300.Simulator(tile_bits=12, fusion_max_qubits=4, pass_budget=25)
    _, _, compiled, _ = sim._prepare(c, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))
    s32 = sim._evolve(compiled, compiled.pool([cirq.ParamResolver({})])[0], 0)
    s64 = _complex128_gpu_run(sim.engine, c, n)
    err, n64, n32 = _compare(sim.engine, s64, s32, n)
    print(f"30q depth 40: max |psi64 - psi128| = {err:.3e}, norms^2 {n64:.12f} {n32:.9f}")
    assert abs(n64 - 1) < 1e-10
    assert abs(n32 - 1) < 1e-5
    assert err < AMP_TOL
    s64.free()
