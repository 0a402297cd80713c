"""The pipelined tensor-core pass (12-bit tiles, 4-bit MMA blocks, csrc/gbq_tc.cu)
against the CPU emulator of the same program, the complex128 oracle, the
reference's golden states, and the complex128 GPU run."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import _lib, workloads
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements
from emulator import run_program
from oracle.circuits import simulate_density_matrix, simulate_state_vector

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_tc.py", "golden/golden.npz"))
GOLD_LARGE = np.load(__file__.replace("test_gpu_tc.py", "golden/golden_large.npz"))
TOL = 1e-5


def _compile(circuit, budget):
    body, _ = split_measurements(circuit)
    return CompiledCircuit(body, sorted(circuit.all_qubits()), dm=False, planner=Planner(tensor=True, budget=budget),
                           resolvers=[cirq.ParamResolver({})])


@pytest.mark.parametrize("n,depth,budget", [(12, 6, 2), (14, 10, 4), (18, 12, 4), (22, 16, 6)])
def test_tc_program_matches_emulator_and_oracle(n, depth, budget):
    c = workloads.random_layer_circuit(n, depth, seed=200 + n)
    plan = _compile(c, budget).plan
    mma_passes = sum(
        1 for p in plan.passes if any(plan.ops[p["op_begin"] + i]["kind"] == _lib.OP_MMA for i in range(p["op_count"]))
    )
    assert mma_passes >= plan.npasses - 1  # the tensor-core form carries (almost) every pass
    sim = cirq_gb300.Simulator()
    eng = sim.engine
    st = eng.new_state(n, basis=0)
    pool = eng.upload(plan.pool)
    l0 = eng.launches()
    _lib.check(eng.lib.gbq_run(eng.ctx, st.ptr, n, plan.passes.ctypes.data, len(plan.passes), plan.ops.ctypes.data,
                               len(plan.ops), pool.ptr), "gbq_run")
    eng.sync()
    assert eng.launches() - l0 == plan.npasses
    got = eng.download_state(st, n)
    psi0 = np.zeros(2**n, complex)
    psi0[0] = 1
    emu = run_program(psi0, n, plan.passes, plan.ops, plan.pool.astype(np.complex128))
    assert np.max(np.abs(got - emu)) < 1e-6
    assert np.max(np.abs(got - simulate_state_vector(c))) < TOL


def test_tc_simulator_vs_reference_golden():
    c = workloads.random_layer_circuit(12, 8, 2)
    got = cirq_gb300.Simulator(tensor_cores=True).simulate(c).final_state_vector
    np.testing.assert_allclose(got, GOLD["layers_n12_d8_s2_c128"], atol=TOL)


@pytest.mark.parametrize("n,depth", [(20, 20), (24, 40)])
def test_tc_simulator_vs_reference_at_bench_sizes(n, depth):
    key = f"layers_n{n}_d{depth}_s0_c128"
    psi = cirq_gb300.Simulator(tensor_cores=True).simulate(workloads.random_layer_circuit(n, depth, 0)).final_state_vector
    idx = GOLD_LARGE[f"{key}_idx"]
    assert np.max(np.abs(psi[idx] - GOLD_LARGE[f"{key}_amps"])) < TOL
    assert abs(np.linalg.norm(psi.astype(np.complex128)) - 1) < 1e-5


def test_tc_sweep_parameters_replay():
    """Parameterised circuits: the MMA blocks' matrices are rebuilt per point."""
    circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(14, 4, seed=14)
    pts = workloads.qaoa_points(4, 3, seed=5)
    res = [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]
    sim = cirq_gb300.Simulator(tensor_cores=True)
    for r, tr in zip(res, sim.simulate_sweep(circuit, res)):
        want = simulate_state_vector(circuit, r)
        assert np.max(np.abs(tr.final_state_vector - want)) < TOL


def test_tc_density_matrix_noisy_layers():
    c = workloads.noisy_layer_circuit(7, 5, seed=3, p=0.02, gamma=0.05)
    rho = cirq_gb300.DensityMatrixSimulator(tensor_cores=True).simulate(c).final_density_matrix
    assert np.max(np.abs(rho - simulate_density_matrix(c))) < TOL


def test_tc_26_qubits_vs_complex128_gpu_run():
    n = 26
    c = workloads.random_layer_circuit(n, 40, 1)
    sim = cirq_gb300.Simulator(tensor_cores=True)
    _, _, compiled, _ = sim._prepare(c, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))
    s32 = sim._evolve(compiled, compiled.pool([cirq.ParamResolver({})])[0], 0)
    eng = sim.engine
    q = sorted(c.all_qubits())
    index = {x: i for i, x in enumerate(q)}
    s64 = eng.alloc(16 << n)
    _lib.check(eng.lib.gbq_sv64_set_basis(eng.ctx, s64.ptr, n, 0), "gbq_sv64_set_basis")
    for op in c.all_operations():
        bits = np.array([n - 1 - index[x] for x in reversed(op.qubits)], dtype=np.int32)
        m = np.ascontiguousarray(cirq.unitary(op), dtype=np.complex128)
        _lib.check(eng.lib.gbq_sv64_apply(eng.ctx, s64.ptr, n, len(bits), bits.ctypes.data, m.ctypes.data), "apply")
    out = np.zeros(3)
    _lib.check(eng.lib.gbq_sv64_compare(eng.ctx, s64.ptr, s32.ptr, n, out.ctypes.data), "gbq_sv64_compare")
    print(f"tensor-core 26q depth 40: max |psi_tc - psi128| = {out[0]:.3e}, norm^2 {out[2]:.9f}")
    assert out[0] < TOL
    # the tensor cores' fp32 accumulation rounds toward zero: over ~200 MMA
    # ops per amplitude the norm shrinks by ~1e-4 (measured 8.5e-5 here),
    # inside the reference's renormalisation threshold sqrt(eps) = 3.5e-4
    assert abs(out[2] - 1) < 5e-4
