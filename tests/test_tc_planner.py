"""Tensor-core planning (Planner(tensor=True)) on the CPU: the engine's own
pre-launch checks accept the programs (gbq_validate_program runs the
tensor-core argument builder), the emulated programs match the oracle, and
the simulators with tensor_cores=True run on the emulated engine."""

import numpy as np
import pytest

import cirq
import cirq_gb300
import cirq_gb300.simulator as sim_mod
from cirq_gb300 import _lib, workloads
from cirq_gb300.planner import TC_MAX_MATS, Planner
from cirq_gb300.program import CompiledCircuit, split_measurements
from cpu_engine import EmuEngine
from emulator import run_program
from oracle.circuits import simulate_density_matrix, simulate_state_vector


@pytest.fixture
def emu(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    return eng


def _plan(circuit, budget, dm=False):
    body, _ = split_measurements(circuit)
    return CompiledCircuit(body, sorted(circuit.all_qubits()), dm=dm, planner=Planner(tensor=True, budget=budget),
                           resolvers=[cirq.ParamResolver({})]).plan


def _mma_passes(plan):
    return [p for p in plan.passes
            if any(plan.ops[p["op_begin"] + i]["kind"] == _lib.OP_MMA for i in range(p["op_count"]))]


@pytest.mark.parametrize("n,depth,budget,seed", [(12, 6, 2, 1), (14, 10, 4, 2), (16, 12, 3, 3), (17, 9, 6, 4)])
def test_tc_plans_validate_and_match_the_oracle(n, depth, budget, seed):
    c = workloads.random_layer_circuit(n, depth, seed)
    plan = _plan(c, budget)
    _lib.validate_program(plan)
    tc = _mma_passes(plan)
    assert len(tc) >= plan.npasses - 1
    for p in tc:
        ops = plan.ops[p["op_begin"] : p["op_begin"] + p["op_count"]]
        mma = ops[ops["kind"] == _lib.OP_MMA]
        assert p["L"] == 12 and p["m"] == 5 and ops[0]["kind"] == _lib.OP_MMA
        assert set(ops["kind"]) <= {_lib.OP_MMA, _lib.OP_DIAG}
        assert len(mma) <= budget and (mma["k"] == 4).all()
        assert (mma["sel"][:, :3][np.arange(3)[None, :] < mma["nsel"][:, None]] < 0).all()  # global selectors
        assert int((2 ** mma["nsel"].astype(int)).sum()) <= TC_MAX_MATS
    psi0 = np.zeros(2**n, complex)
    psi0[0] = 1
    got = run_program(psi0, n, plan.passes, plan.ops, plan.pool.astype(np.complex128))
    assert np.max(np.abs(got - simulate_state_vector(c))) < 1e-6


def test_tc_pass_count_for_the_30_qubit_workload():
    """The tensor-core form needs fewer passes than the CUDA-core plan (101)."""
    plan = _plan(workloads.random_layer_circuit(30, 40, 0), 4)
    assert len(_mma_passes(plan)) == plan.npasses <= 70
    _lib.validate_program(plan)


def test_tc_simulators_on_the_emulated_engine(emu):
    c = workloads.random_layer_circuit(13, 7, seed=8)
    got = cirq_gb300.Simulator(tensor_cores=True).simulate(c).final_state_vector
    assert np.max(np.abs(got - simulate_state_vector(c))) < 1e-5
    circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(12, 4, seed=12)
    pts = workloads.qaoa_points(4, 3, seed=5)
    res = [cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts]
    sim = cirq_gb300.Simulator(tensor_cores=True)
    for r, tr in zip(res, sim.simulate_sweep(circuit, res)):
        assert np.max(np.abs(tr.final_state_vector - simulate_state_vector(circuit, r))) < 1e-5
    noisy = workloads.noisy_layer_circuit(7, 4, seed=3, p=0.02, gamma=0.05)
    rho = cirq_gb300.DensityMatrixSimulator(tensor_cores=True).simulate(noisy).final_density_matrix
    assert np.max(np.abs(rho - simulate_density_matrix(noisy))) < 1e-5
