"""The contract cirq-google's virtual engine relies on, exercised without
cirq-google (its dependencies tunits, google-api-core and proto-plus are
absent here).

``create_noisy_virtual_engine_from_processor_id``
(cirq-google/cirq_google/engine/virtual_engine_factory.py:456-470) builds
``simulator_class(noise=noise_model, **kwargs)`` and hands the simulator to
``SimulatedLocalProcessor`` as its ``cirq.Sampler``, which then calls
``run_sweep`` / ``run_batch`` (cirq-core/cirq/work/sampler.py:219-283).  These
tests construct the simulators exactly that way and drive them through the
Sampler entry points, comparing the sampled distributions with the
reference simulator's (chi^2 homogeneity)."""

import numpy as np
import pytest
import scipy.stats
import sympy

import cirq
import cirq_gb300
import cirq_gb300.simulator as sim_mod
from cpu_engine import EmuEngine


def _programs():
    q = cirq.LineQubit.range(3)
    t = sympy.Symbol("t")
    a = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.rx(t).on(q[2]), cirq.measure(*q, key="m"))
    b = cirq.Circuit(cirq.X(q[0]), cirq.ry(0.7).on(q[1]), cirq.CZ(q[0], q[1]), cirq.measure(q[0], q[1], key="m"))
    return [a, b], [cirq.Points("t", [0.3, 1.9]), None]


def _hist(result):
    bits = result.measurements["m"]
    return np.bincount(bits.astype(int) @ (1 << np.arange(bits.shape[1] - 1, -1, -1)), minlength=2 ** bits.shape[1])


def _same_distribution(h1, h2):
    keep = (h1 + h2) > 0
    if keep.sum() < 2:
        return np.array_equal(h1, h2)
    return scipy.stats.chi2_contingency(np.stack([h1[keep], h2[keep]]))[1] > 1e-4


def _check_contract(simulator_class, reference_class):
    """reference_class: the reference simulator the drop-in replaces (the two
    reference simulators place a noise model differently, so each drop-in is
    compared with its own counterpart)."""
    noise = cirq.ConstantQubitNoiseModel(cirq.depolarize(0.05))
    kwargs = {"seed": 17}
    sim = simulator_class(noise=noise, **kwargs)  # the factory's call
    assert isinstance(sim, cirq.Sampler)
    ref = reference_class(noise=noise, seed=18)
    programs, params = _programs()
    reps = 3000
    got = sim.run_batch(programs, params_list=params, repetitions=reps)
    want = ref.run_batch(programs, params_list=params, repetitions=reps)
    assert [len(x) for x in got] == [len(x) for x in want] == [2, 1]
    for g_list, w_list in zip(got, want):
        for g, w in zip(g_list, w_list):
            assert isinstance(g, cirq.Result)
            assert g.params == w.params
            assert g.measurements["m"].shape == w.measurements["m"].shape
            assert g.measurements["m"].dtype == w.measurements["m"].dtype
            assert _same_distribution(_hist(g), _hist(w))
    # run_sweep, as SimulatedLocalProcessor calls it for one program
    sweep = sim.run_sweep(programs[0], params[0], repetitions=reps)
    assert [r.params for r in sweep] == [r.params for r in ref.run_sweep(programs[0], params[0], repetitions=1)]
    # the noise model is applied: the depolarised GHZ pair disagrees sometimes
    bits = sweep[0].measurements["m"]
    assert 0 < np.mean(bits[:, 0] != bits[:, 1]) < 0.2


def test_engine_contract_on_the_emulated_engine(monkeypatch):
    eng = EmuEngine()
    monkeypatch.setattr(sim_mod, "default_engine", lambda device=None: eng)
    _check_contract(cirq_gb300.Simulator, cirq.Simulator)
    _check_contract(cirq_gb300.DensityMatrixSimulator, cirq.DensityMatrixSimulator)


@pytest.mark.gpu
def test_engine_contract_on_the_gpu():
    _check_contract(cirq_gb300.Simulator, cirq.Simulator)
    _check_contract(cirq_gb300.DensityMatrixSimulator, cirq.DensityMatrixSimulator)
