"""Module-level entry points of ``cirq.sim.mux`` on the GPU simulators.

``cirq.sample``, ``cirq.sample_sweep``, ``cirq.final_state_vector`` and
``cirq.final_density_matrix`` (cirq-core/cirq/sim/mux.py:53-333) build a
fresh ``cirq.Simulator`` / ``cirq.DensityMatrixSimulator`` per call; the
functions here keep their signatures, argument checks and error messages and
run on :class:`cirq_gb300.Simulator` / :class:`cirq_gb300.DensityMatrixSimulator`
instead.  Choices of simulator:

* ``sample``: a noiseless Clifford circuit samples by Pauli frames on the GPU
  (:class:`cirq_gb300.clifford.CliffordSimulator`), as the reference sends it
  to its tableau simulator; another noiseless circuit runs on the
  state-vector simulator (mid-circuit measurements as trajectories) where the
  reference uses the density-matrix simulator.  The sample distribution is
  the same.
  A noisy circuit runs on the density-matrix simulator up to
  ``DM_MAX_QUBITS`` qubits, as in the reference, and above that (where a
  density matrix does not fit) as state-vector trajectories of the circuit
  with its noise placed where the density-matrix simulator places it.
* ``final_density_matrix``: unitary, unmeasured and noiseless -> the
  state-vector simulator and an outer product on the host (mux.py:285-293);
  otherwise the density-matrix simulator with measurements dephased
  (mux.py:294-333) by the reference's own ``cirq.dephase_measurements``
  (cirq-core/cirq/transformers/measurement_transformers.py:217-256), whose
  keyed ``phase_damp(1)`` channels lose their key (it only records the
  Kraus index).

Only ``dtype=np.complex64`` is accepted, as by the simulators.
"""

from __future__ import annotations

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq

cirq = ensure_cirq()

DM_MAX_QUBITS = 14


def _state_bits(qids) -> int:
    """Index bits of a state over `qids` (a qid of dimension d > 2 takes
    ceil(log2 d))."""
    from cirq_gb300.qudits import bits_for

    return sum(1 if q.dimension == 2 else bits_for(q.dimension) for q in qids)


def _sv_sim(dtype, seed, noise=None):
    from cirq_gb300.simulator import Simulator

    return Simulator(dtype=dtype, seed=seed, noise=noise)


def _dm_sim(dtype, seed, noise=None):
    from cirq_gb300.simulator import DensityMatrixSimulator

    return DensityMatrixSimulator(dtype=dtype, seed=seed, noise=noise)


def _is_clifford_circuit(program) -> bool:
    """mux.py:336-339: every non-measurement operation has a stabilizer effect."""
    return all(cirq.has_stabilizer_effect(op) for op in program.all_operations() if not cirq.is_measurement(op))


def _to_circuit(program) -> cirq.Circuit:
    """Circuit, gate or OP_TREE -> Circuit (mux.py:97-106)."""
    if isinstance(program, cirq.Circuit):
        return program
    if isinstance(program, cirq.Gate):
        return cirq.Circuit(program.on(*cirq.LineQid.for_gate(program)))
    return cirq.Circuit(program)


def sample(
    program: cirq.Circuit,
    *,
    noise: cirq.NOISE_MODEL_LIKE = None,
    param_resolver: cirq.ParamResolver | None = None,
    repetitions: int = 1,
    dtype: type[np.complexfloating] = np.complex64,
    seed: cirq.RANDOM_STATE_OR_SEED_LIKE = None,
) -> cirq.Result:
    """Samples the circuit's measurements (``cirq.sample``, mux.py:53-94)."""
    noise_model = cirq.NoiseModel.from_noise_model_like(noise)
    if noise_model == cirq.NO_NOISE:
        if _is_clifford_circuit(program):
            # as the reference (mux.py:81-86): Clifford circuits sample on the
            # stabilizer path, here Pauli frames on the GPU
            from cirq_gb300.clifford import CliffordSimulator

            return CliffordSimulator(seed=seed).run(program, param_resolver=param_resolver, repetitions=repetitions)
        return _sv_sim(dtype, seed).run(program, param_resolver=param_resolver, repetitions=repetitions)
    dm = _dm_sim(dtype, seed, noise_model)
    if _state_bits(program.all_qubits()) <= DM_MAX_QUBITS:
        return dm.run(program, param_resolver=param_resolver, repetitions=repetitions)
    # too wide for a density matrix: trajectories of the circuit with the
    # noise placed as the density-matrix simulator places it for run()
    placed = dm._reference_noisy_circuit(program, "run")
    return _sv_sim(dtype, seed).run(placed, param_resolver=param_resolver, repetitions=repetitions)


def sample_sweep(
    program: cirq.Circuit,
    params: cirq.Sweepable,
    *,
    noise: cirq.NOISE_MODEL_LIKE = None,
    repetitions: int = 1,
    dtype: type[np.complexfloating] = np.complex64,
    seed: cirq.RANDOM_STATE_OR_SEED_LIKE = None,
) -> list[cirq.Result]:
    """One ``sample`` per resolver with a shared random state (mux.py:180-222)."""
    prng = cirq.value.parse_random_state(seed)
    return [
        sample(program, noise=noise, param_resolver=r, repetitions=repetitions, dtype=dtype, seed=prng)
        for r in cirq.to_resolvers(params)
    ]


def final_state_vector(
    program: cirq.CIRCUIT_LIKE,
    *,
    initial_state: cirq.STATE_VECTOR_LIKE = 0,
    param_resolver: cirq.ParamResolverOrSimilarType = None,
    qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
    ignore_terminal_measurements: bool = False,
    dtype: type[np.complexfloating] = np.complex64,
    seed: cirq.RANDOM_STATE_OR_SEED_LIKE = None,
) -> np.ndarray:
    """Final state of a unitary program (``cirq.final_state_vector``,
    mux.py:109-177).

    Raises:
        ValueError: the circuit contains a measurement (unless
            ``ignore_terminal_measurements`` and they are terminal) or is not
            unitary.
    """
    circuit_like = _to_circuit(program)
    if not ignore_terminal_measurements:
        if any(cirq.is_measurement(op) for op in circuit_like.all_operations()):
            raise ValueError('Circuit contains a measurement.')
    else:
        circuit_like = cirq.drop_terminal_measurements(circuit_like)
    if not cirq.has_unitary(cirq.resolve_parameters(circuit_like, param_resolver)):
        raise ValueError(
            "Program doesn't have a single well defined final state vector "
            "because it is not unitary. "
            "Maybe you wanted `cirq.final_density_matrix`?\n"
            "\n"
            f"Program: {circuit_like!r}"
        )
    result = _sv_sim(dtype, seed).simulate(
        program=circuit_like,
        initial_state=initial_state,
        qubit_order=qubit_order,
        param_resolver=param_resolver,
    )
    return result.state_vector()


_DEPHASE_SUPEROP = None


def _is_dephasing_record(op) -> bool:
    """A keyed one-qubit KrausChannel equal to phase_damp(1): what
    cirq.dephase_measurements puts in place of a measured qubit."""
    global _DEPHASE_SUPEROP
    if not isinstance(op.gate, cirq.KrausChannel) or len(op.qubits) != 1:
        return False
    if _DEPHASE_SUPEROP is None:
        _DEPHASE_SUPEROP = cirq.kraus_to_superoperator(cirq.kraus(cirq.phase_damp(1)))
    return np.allclose(cirq.kraus_to_superoperator(cirq.kraus(op)), _DEPHASE_SUPEROP, atol=1e-12)


def _unkey(circuit: cirq.AbstractCircuit) -> cirq.Circuit:
    """Drops the measurement key of every dephasing channel that
    ``cirq.dephase_measurements`` inserted: the key only records the Kraus
    index, which the final density matrix ignores.  Op for op, so the moment
    structure stays the reference's."""

    def unkey(op, _):
        if cirq.is_measurement(op) and _is_dephasing_record(op):
            return cirq.phase_damp(1).on(*op.qubits)
        return op

    return cirq.map_operations(circuit, unkey, deep=True).unfreeze()


def _dephase(circuit: cirq.AbstractCircuit) -> cirq.Circuit:
    """The reference's own ``cirq.dephase_measurements`` (which raises for
    classical control) with the keys dropped (``_unkey``)."""
    return _unkey(cirq.dephase_measurements(circuit))


def final_density_matrix(
    program: cirq.CIRCUIT_LIKE,
    *,
    noise: cirq.NOISE_MODEL_LIKE = None,
    initial_state: cirq.STATE_VECTOR_LIKE = 0,
    param_resolver: cirq.ParamResolverOrSimilarType = None,
    qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
    dtype: type[np.complexfloating] = np.complex64,
    seed: int | np.random.RandomState | None = None,
    ignore_measurement_results: bool = True,
) -> np.ndarray:
    """Final density matrix (``cirq.final_density_matrix``, mux.py:225-333):
    measurements dephase unless ``ignore_measurement_results`` is False, in
    which case they collapse with sampled outcomes."""
    noise_model = cirq.NoiseModel.from_noise_model_like(noise)
    circuit_like = _to_circuit(program)
    can_do_unitary_simulation = cirq.has_unitary(circuit_like)
    if isinstance(circuit_like, cirq.Circuit) and circuit_like.has_measurements():
        can_do_unitary_simulation = False
    if noise_model != cirq.NO_NOISE:
        can_do_unitary_simulation = False

    if can_do_unitary_simulation:
        result = _sv_sim(dtype, seed).simulate(
            program=circuit_like,
            initial_state=initial_state,
            qubit_order=qubit_order,
            param_resolver=param_resolver,
        )
        return result.density_matrix_of()

    has_classical_control = circuit_like != cirq.defer_measurements(circuit_like)
    handling_classical_control = ignore_measurement_results and has_classical_control
    sim = _dm_sim(dtype, seed, None if handling_classical_control else noise)
    if handling_classical_control:
        noise_applied = circuit_like.with_noise(noise) if noise is not None else circuit_like
        dephased = cirq.dephase_measurements(cirq.defer_measurements(noise_applied))
        prog = dephased
    elif ignore_measurement_results:
        prog = cirq.dephase_measurements(circuit_like)
    else:
        prog = circuit_like
    if sim.noise is not cirq.NO_NOISE:
        # noise goes where the reference's simulator puts it, which depends on
        # the dephasing channels' keys; the keys are dropped afterwards
        prog = sim._reference_noisy_circuit(prog, "simulate")
        sim = sim._noiseless()
    result = sim.simulate(
        _unkey(prog),
        initial_state=initial_state,
        qubit_order=qubit_order,
        param_resolver=param_resolver,
    )
    rho = result.final_density_matrix
    if handling_classical_control:
        # the deferral's ancillas come after the circuit's own qubits
        keep = list(range(cirq.num_qubits(circuit_like)))
        shape = cirq.qid_shape(dephased)
        reduced = cirq.partial_trace(np.reshape(rho, shape + shape), keep)
        width = int(np.prod(cirq.qid_shape(circuit_like)))
        rho = np.reshape(reduced, (width, width))
    return rho
