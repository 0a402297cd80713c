"""Moment-by-moment simulation (``simulate_moment_steps``) on the GPU.

Mirrors ``SimulatesIntermediateState.simulate_moment_steps``
(``cirq-core/cirq/sim/simulator.py:607-640``) and the step loop of
``SimulatorBase._core_iterator`` (``cirq-core/cirq/sim/simulator_base.py:169-214``):
the noise model is expanded into moments, every (noisy) moment is applied to
the one device state -- its unitary operations as a fused GPU program, its
measurements and general channels as trajectory events -- and a step result
is yielded after it.

A step result refers to the live device state, as the reference's step
results refer to the live simulation state: ``sample`` draws from the state
as it is when called (on the GPU, without collapsing it) and
``state_vector`` / ``density_matrix`` download it on first use.  Consume a
step before advancing the iterator.
"""

from __future__ import annotations

from typing import Any, Iterator

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.ir import flatten_ops

cirq = ensure_cirq()


class _GpuStep(cirq.StepResult):
    """Common part of the GPU step results (measurements, sampling)."""

    def __init__(self, sim, state, qubits, measurements):
        self._sim = sim
        self._state = state
        self._qubits = tuple(qubits)
        self._measurements = measurements
        self._host = None

    def _qid_shape_(self):
        return (2,) * len(self._qubits)

    def sample(self, qubits, repetitions: int = 1, seed: Any = None) -> np.ndarray:
        """Draws from |psi|^2 (or diag rho) on the device; no collapse
        (``cirq-core/cirq/sim/state_vector.py:170-232``)."""
        index = {q: i for i, q in enumerate(self._qubits)}
        for q in qubits:
            if q not in index:
                raise ValueError(f"qubit {q} is not simulated")
        if repetitions == 0 or not qubits:
            return np.zeros((repetitions, len(qubits)), dtype=np.uint8)
        prng = self._sim._prng if seed is None else cirq.value.parse_random_state(seed)
        n = len(self._qubits)
        idx = self._sim.engine.sample(self._state, n, prng.random_sample(repetitions), dm=self._sim._dm)
        idx = idx.astype(np.int64)
        out = np.empty((repetitions, len(qubits)), dtype=np.uint8)
        for j, q in enumerate(qubits):
            out[:, j] = (idx >> (n - 1 - index[q])) & 1
        return out

    def _download(self, nbits: int) -> np.ndarray:
        if self._host is None:
            self._host = np.array(self._sim.engine.download_state(self._state, nbits), copy=True)
        return self._host


class GpuStateVectorStep(cirq.StateVectorMixin, _GpuStep):
    """Step result of ``cirq_gb300.Simulator.simulate_moment_steps``."""

    def __init__(self, sim, state, qubits, measurements):
        # StateVectorMixin passes the remaining arguments on to _GpuStep
        super().__init__({q: i for i, q in enumerate(qubits)}, sim, state, qubits, measurements)

    def state_vector(self, copy: bool = False) -> np.ndarray:
        vec = self._download(len(self._qubits))
        return vec.copy() if copy else vec

    def _simulator_state(self):
        return cirq.StateVectorSimulationState(
            qubits=self._qubits, initial_state=self.state_vector(copy=True), dtype=np.complex64
        )


class GpuDensityMatrixStep(_GpuStep):
    """Step result of ``cirq_gb300.DensityMatrixSimulator.simulate_moment_steps``."""

    def density_matrix(self, copy: bool = True) -> np.ndarray:
        n = len(self._qubits)
        rho = self._download(2 * n).reshape(2**n, 2**n)
        return rho.copy() if copy else rho

    def _simulator_state(self):
        return cirq.DensityMatrixSimulationState(
            qubits=self._qubits, initial_state=self.density_matrix(), dtype=np.complex64
        )


def moment_steps(sim, circuit, param_resolver, qubit_order, initial_state) -> Iterator[Any]:
    from cirq_gb300 import trajectories as tj

    resolver = cirq.ParamResolver(param_resolver)
    resolved = cirq.resolve_parameters(circuit, resolver)
    unresolved = cirq.parameter_symbols(resolved)
    if unresolved:
        raise ValueError(f"Circuit contains unresolved parameters: {sorted(map(str, unresolved))}")
    qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(circuit.all_qubits()))
    step_cls = GpuDensityMatrixStep if sim._dm else GpuStateVectorStep
    if not qubits:
        # no amplitudes to evolve: the reference's own step results around a
        # 0-qubit state (the global phase so far), one per moment, or one
        # for an empty circuit (simulator_base.py:192-194)
        phase = 1.0 + 0j
        steps_needed = max(len(resolved), 1)
        for i in range(steps_needed):
            if i < len(resolved):
                for op in resolved[i].operations:
                    phase *= complex(np.asarray(cirq.unitary(op)).reshape(-1)[0])
            if sim._dm:
                st = cirq.DensityMatrixSimulationState(qubits=(), initial_state=np.full((1, 1), abs(phase) ** 2),
                                                       dtype=np.complex64)
                yield cirq.DensityMatrixStepResult(sim_state=st, dtype=np.complex64)
            else:
                st = cirq.StateVectorSimulationState(qubits=(), initial_state=np.array([phase], dtype=np.complex64),
                                                     dtype=np.complex64)
                yield cirq.SparseSimulatorStep(sim_state=st, dtype=np.complex64)
        return
    moments = list(sim.noise.noisy_moments(resolved, sorted(resolved.all_qubits())))
    initial = 0 if initial_state is None else initial_state
    empty = sim._compile([], qubits, [cirq.ParamResolver({})])
    # the steps keep the device state alive; it is freed with the last of them
    state = sim._initial_device_state(empty, initial)
    if not moments:
        yield step_cls(sim, state, qubits, {})
        return
    log: dict = {}  # the measurement log so far, as the reference's step results carry it
    records: dict = {}  # every measurement so far (classical control reads it)
    measured: dict = {}
    for moment in moments:
        ops = flatten_ops(cirq.Circuit(cirq.flatten_to_ops_or_moments([moment])))
        runner = tj.TrajectoryRunner(sim, ops, qubits, resolver)
        try:
            picks, pools = runner.prepare(1)
            runner.apply(state, picks[0], pools, 0, records, measured)
        finally:
            runner.close()
        log.update({k: np.array(v[-1], dtype=np.uint8) for k, v in records.items()})
        yield step_cls(sim, state, qubits, dict(log))
