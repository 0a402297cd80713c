"""Drop-in GPU simulators with the ``cirq.Simulator`` / ``cirq.DensityMatrixSimulator`` API.

``Simulator`` implements the reference's simulator interfaces
(``cirq-core/cirq/sim/simulator.py``): ``SimulatesSamples._run`` (:97-117),
``SimulatesFinalState.simulate_sweep_iter`` (:510-538),
``SimulatesExpectationValues.simulate_expectation_values_sweep_iter``
(:398-441) and ``SimulatesAmplitudes.compute_amplitudes_sweep_iter``
(:188-216); ``run``, ``simulate``, ``simulate_sweep``,
``simulate_expectation_values(_sweep)``, ``compute_amplitudes`` and
``Sampler.run_batch`` come from the reference's base classes.  Results are the
reference's own result types (``cirq.StateVectorTrialResult``,
``cirq.DensityMatrixTrialResult``, ``cirq.ResultDict``).

All amplitude arithmetic runs on the GPU through the C ABI; there is no CPU
fallback.  Differences from the reference, by design:

* arithmetic is complex64 only (``dtype=np.complex64``, the reference's
  default); other dtypes raise ``ValueError``;
* mid-circuit measurement and state-vector noise run as per-repetition
  trajectories (``cirq_gb300/trajectories.py``), as the reference's ``_run``
  does; samples are statistically, not bit-for-bit, equal to the reference's;
* ``split_untangled_states`` is accepted and ignored: the reference's
  product-state factoring (``cirq-core/cirq/sim/simulation_product_state.py``)
  changes no result, only its CPU cost.
"""

from __future__ import annotations

import collections
import math
import threading
import warnings
from typing import Any, Iterator, Sequence

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.engine import Engine, default_engine
from cirq_gb300.ir import pauli_terms
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements, structure_key
from cirq_gb300 import qudits as _qudits
from cirq_gb300 import trajectories as _traj

cirq = ensure_cirq()

_MAX_CACHE = 64  # compiled circuits kept per simulator (trajectory segments count too)
_MAX_STATE_BITS = 34  # widest device state run() simulates in one piece (2^34 amplitudes: 128 GiB)
_PART = "\x00"  # separator of the internal measurement keys of untangled parts


def _check_dtype(dtype):
    if np.dtype(dtype).kind != "c":
        raise ValueError(f"dtype must be a complex type but was {dtype}")
    if np.dtype(dtype) != np.complex64:
        raise ValueError(
            f"cirq_gb300 simulates in complex64 only (got {np.dtype(dtype)}); "
            "use dtype=np.complex64"
        )


_MEMO_LOCK = threading.Lock()
_SPLIT_MEMO: collections.OrderedDict = collections.OrderedDict()


def _memo(store: collections.OrderedDict, program, name, fn):
    """fn(program), remembered per circuit object for as long as it holds
    the same moment objects.  Moments are immutable, so the same moments are
    the same operations.  The entry keeps the moments alive, so a reused
    id() cannot match another circuit."""
    moments = getattr(program, "moments", None)
    if moments is None:
        return fn(program)
    moments = tuple(moments)
    key = (id(program), name)
    with _MEMO_LOCK:
        hit = store.get(key)
        if hit is not None and len(hit[0]) == len(moments) and all(a is b for a, b in zip(hit[0], moments)):
            store.move_to_end(key)
            return hit[1]
    val = fn(program)
    with _MEMO_LOCK:
        store[key] = (moments, val)
        while len(store) > 128:
            store.popitem(last=False)
    return val


def _split_terminal(program):
    """split_measurements(program) as tuples, remembered per circuit."""
    return _memo(_SPLIT_MEMO, program, "split",
                 lambda p: tuple(tuple(part) for part in split_measurements(p)))


def _check_all_resolved(program, resolver) -> None:
    """Restates check_all_resolved (cirq-core/cirq/sim/simulator.py:942-949)."""
    syms = cirq.parameter_symbols(program)
    if not syms:
        return
    unresolved = [s for s in syms if cirq.is_parameterized(resolver.value_of(s))]
    if unresolved:
        ops = [
            op
            for op in cirq.resolve_parameters(program, resolver, recursive=False).all_operations()
            if cirq.is_parameterized(op)
        ]
        raise ValueError(
            "Circuit contains ops whose symbols were not specified in "
            f"parameter sweep. Ops: {ops}"
        )


def _symbolic_repetitions(program) -> bool:
    """Does a CircuitOperation of `program` repeat a symbolic number of
    times?  Its structure is then known only per sweep point.  (Remembered
    per circuit.)"""
    return _memo(_SPLIT_MEMO, program, "symbolic_repetitions", _symbolic_repetitions_of)


def _symbolic_repetitions_of(program) -> bool:
    gate_op = cirq.GateOperation
    for op in program.all_operations():
        if type(op) is gate_op:
            continue
        u = op.untagged
        if isinstance(u, cirq.ClassicallyControlledOperation):
            u = u.without_classical_controls().untagged
        if isinstance(u, cirq.CircuitOperation):
            if cirq.is_parameterized(u.repetitions) or _symbolic_repetitions_of(u.circuit):
                return True
    return False


def _per_point(program, params):
    """(resolver, resolved program) per sweep point."""
    for r in cirq.to_resolvers(params):
        _check_all_resolved(program, r)
        yield r, cirq.resolve_parameters(program, r)


class _GpuSimulatorBase:
    """Shared machinery of the state-vector and density-matrix drop-ins."""

    _dm = False

    def __init__(
        self,
        *,
        dtype: type[np.complexfloating] = np.complex64,
        noise: cirq.NOISE_MODEL_LIKE = None,
        seed: cirq.RANDOM_STATE_OR_SEED_LIKE = None,
        split_untangled_states: bool = True,
        device: int | None = None,
        fusion_max_qubits: int = 4,
        tile_bits: int = 12,
        pass_budget: float = 25.0,
        use_cuda_graphs: bool = False,
        autotune: bool = False,
        tensor_cores: bool = False,
        mma_ops_per_pass: int = 4,
    ):
        _check_dtype(dtype)
        self._use_graphs = use_cuda_graphs
        self._autotune = autotune
        self._runners: dict = {}
        self._dtype = np.complex64
        self.noise = cirq.NoiseModel.from_noise_model_like(noise)
        self._prng = cirq.value.parse_random_state(seed)
        self._split_untangled_states = split_untangled_states
        self._device = device
        if tensor_cores:
            # 12-bit tiles, 4-bit blocks on the tensor cores (tcgen05, TF32
            # three-term split); passes it cannot express run on the CUDA cores
            self.planner = Planner(tensor=True, budget=mma_ops_per_pass)
        else:
            self.planner = Planner(tile_bits=tile_bits, kmax=fusion_max_qubits, budget=pass_budget)
        self._cache: collections.OrderedDict = collections.OrderedDict()
        self._slot_programs: dict = {}  # one-op trajectory programs (trajectories.slot_program)
        self._engine: Engine | None = None

    # ---- plumbing --------------------------------------------------------
    @property
    def engine(self) -> Engine:
        if self._engine is None:
            self._engine = default_engine(self._device)
        return self._engine

    def _noisy_ops(self, program, qubits):
        """Noise is placed before compiling, by the entry points
        (_reference_noisy_circuit, then a noise-free clone): a program that
        reaches the compiler with a noise model still attached is a bug."""
        if self.noise is cirq.NO_NOISE:
            return None
        raise RuntimeError("internal: a noise model reached the compiler unplaced")

    def _noiseless(self):
        """This simulator without its noise model (engine, caches and random
        state shared), for a program whose noise is already inserted."""
        import copy

        inner = copy.copy(self)
        inner.noise = cirq.NO_NOISE
        return inner

    def _reference_noisy_circuit(self, program, mode: str):
        """`program` with the noise model inserted where the reference's
        simulators insert it (cirq-core/cirq/sim/simulator_base.py:216-320).

        The density-matrix simulator puts a noise model that touches no
        measurement key into a prefix: split_into_matching_protocol_then_general
        (cirq-core/cirq/sim/simulator.py:952-983) splits the program into the
        ops that qualify for the prefix and the rest, and each part gets the
        model's noise on its own qubits.  For simulate() (mode "simulate")
        prefix ops touch no measurement key and have no parameters; for run()
        (mode "run") they touch no measurement key, and when the rest is
        measurements only, those are sampled at the end from the state after
        the rest's noise, skipping noise on a tuple of qubits already measured
        (the all_measurements_are_terminal rule of _core_iterator,
        simulator_base.py:196-213).  The state-vector simulator's noise never
        qualifies (it has no unitary): noise on the circuit's qubits after
        every moment."""
        noise = self.noise

        def noisy(c):
            if not len(c):
                return cirq.Circuit()
            return cirq.Circuit(noise.noisy_moments(c, sorted(c.all_qubits())))

        split = cirq.sim.simulator.split_into_matching_protocol_then_general
        if not self._dm or cirq.measurement_keys_touched(noise):
            prefix, suffix = cirq.Circuit(), program
        elif mode == "simulate":
            prefix, suffix = split(
                program, lambda op: not cirq.measurement_keys_touched(op) and not cirq.is_parameterized(op)
            )
        else:
            prefix, suffix = split(program, lambda op: not cirq.measurement_keys_touched(op))
        if mode == "simulate":
            return noisy(prefix) + noisy(suffix)
        suffix_ops = list(suffix.all_operations())
        if not all(isinstance(op.gate, cirq.MeasurementGate) for op in suffix_ops):
            return noisy(prefix) + noisy(suffix)
        measured: set = set()
        kept = []
        for moment in noisy(suffix):
            part = []
            for op in moment.operations:
                if op.qubits in measured:
                    continue
                if isinstance(op.gate, cirq.MeasurementGate):
                    measured.add(op.qubits)
                    continue
                part.append(op)
            if part:
                kept.append(cirq.Moment(part))
        return noisy(prefix) + cirq.Circuit(kept) + cirq.Circuit(suffix_ops)

    def _compile(self, body_ops, qubits, resolvers) -> CompiledCircuit:
        # the key of a remembered (identical) body tuple is computed once
        keys = self.__dict__.setdefault("_key_memo", {})
        mk = (id(body_ops), tuple(qubits))
        hit = keys.get(mk)
        if hit is not None and hit[0] is body_ops:
            key = hit[1]
        else:
            key = structure_key(body_ops, qubits, self._dm, self.planner)
            if isinstance(body_ops, tuple):
                if len(keys) > 128:
                    keys.clear()
                keys[mk] = (body_ops, key)
        c = self._cache.get(key)
        if c is not None:
            self._cache.move_to_end(key)
            return c
        planner = self.planner
        if self._autotune and qubits:
            from cirq_gb300 import autotune

            planner = autotune.tune(body_ops, qubits, self._dm, resolvers[:1], self.engine)
        c = CompiledCircuit(body_ops, qubits, dm=self._dm, planner=planner, resolvers=resolvers[:1])
        self._cache[key] = c
        if len(self._cache) > _MAX_CACHE:
            _, old = self._cache.popitem(last=False)
            # its CUDA-graph runner (state and pool buffers, graph) goes with it
            runner = self._runners.pop(id(old), None)
            if runner is not None and runner[0] is old:
                runner[1].free()
                runner[2].free()
        return c

    def _prepare(self, program, qubit_order, params):
        qubit_order = cirq.QubitOrder.as_qubit_order(qubit_order)
        qubits = tuple(qubit_order.order_for(program.all_qubits()))
        resolvers = list(cirq.to_resolvers(params))
        # unresolved symbols are the caller's error (ValueError, as the
        # reference), checked before anything is compiled
        for r in resolvers or [cirq.ParamResolver({})]:
            _check_all_resolved(program, r)
        body, meas = _split_terminal(program)
        self._noisy_ops(None, qubits)  # noise is placed by the entry points
        compiled = self._compile(body, qubits, resolvers or [cirq.ParamResolver({})])
        return qubits, resolvers, compiled, meas

    def _evolve(self, compiled: CompiledCircuit, pool_row: np.ndarray, initial_state):
        """Allocates the initial state on the device and runs the program.

        With use_cuda_graphs, one state and one matrix-pool buffer are kept per
        compiled circuit and the pass sequence is captured once into a CUDA
        graph; later points upload new matrices into the same buffer and
        replay the graph.  The returned state is then that shared buffer: it
        stays valid until the next simulation of the same circuit."""
        eng = self.engine
        if not self._use_graphs or not compiled.plan.npasses:
            state = self._initial_device_state(compiled, initial_state)
            if compiled.plan.npasses:
                pool_dev = eng.upload(np.ascontiguousarray(pool_row))
                eng.run(state, compiled.nbits_dev, compiled.plan, pool_dev)
            return state
        runner = self._runners.get(id(compiled))
        if runner is None or runner[0] is not compiled:
            state = eng.alloc(8 << compiled.nbits_dev)
            pool_dev = eng.alloc(8 * max(len(compiled.plan.pool), 2))
            graph = eng.graph(state, compiled.nbits_dev, compiled.plan, pool_dev)
            runner = (compiled, state, pool_dev, graph)
            self._runners[id(compiled)] = runner
        _, state, pool_dev, graph = runner
        self._initial_device_state(compiled, initial_state, into=state)
        pool_dev.upload(np.ascontiguousarray(pool_row, dtype=np.complex64))
        graph.launch()
        return _Borrowed(state)

    def _measure_terminal(self, state, compiled, meas_ops) -> dict[str, np.ndarray]:
        """One shot of every terminal measurement, then collapse (the reference
        measures inside simulate(): cirq-core/cirq/sim/state_vector.py:235-322)."""
        if not meas_ops:
            return {}
        eng = self.engine
        n = compiled.n
        index = {q: i for i, q in enumerate(compiled.qubits)}
        u = self._prng.random_sample(1)
        idx = int(eng.sample(state, n, u, dm=self._dm)[0])
        measured = []
        for op in meas_ops:
            for q in op.qubits:
                if q not in measured:
                    measured.append(q)
        mask = 0
        for q in measured:
            mask |= 1 << (n - 1 - index[q])
        value = idx & mask
        records: dict[str, list] = {}
        for op in meas_ops:
            gate = op.gate
            bits = np.array([[(idx >> (n - 1 - index[q])) & 1 for q in op.qubits]], dtype=np.int8)
            records.setdefault(gate.key, []).append(_recorded_in_place(bits, op, self._prng)[0])
        # collapse: keep the sampled outcome, renormalise
        if self._dm:
            full_mask = mask | (mask << n)
            full_value = value | (value << n)
            eng.project(state, compiled.nbits, full_mask, full_value, 1.0)
            p = float(eng.probabilities(state, n, dm=True).astype(np.float64).sum())
            if p > 0:
                eng.scale(state, compiled.nbits, 1.0 / p)
        else:
            eng.project(state, n, mask, value, 1.0)
            p = eng.norm2(state, n)
            if p > 0:
                eng.scale(state, n, 1.0 / math.sqrt(p))
        out = {}
        for key, v in records.items():
            arr = np.array(v[-1], dtype=np.uint8)
            out[key] = arr
        return out

    def _measure_op(self, state, compiled, op) -> list:
        """One shot of one measurement with collapse (a mid-circuit measurement,
        cirq-core/cirq/sim/state_vector.py:235-322 and
        cirq-core/cirq/sim/density_matrix_utils.py:97-183); returns the
        recorded bits (invert mask and confusion map applied)."""
        eng = self.engine
        n = compiled.n
        index = {q: i for i, q in enumerate(compiled.qubits)}
        idx = int(eng.sample(state, n, self._prng.random_sample(1), dm=self._dm)[0])
        mask = 0
        for q in op.qubits:
            mask |= 1 << (n - 1 - index[q])
        value = idx & mask
        if self._dm:
            eng.project(state, compiled.nbits, mask | (mask << n), value | (value << n), 1.0)
            p = float(eng.probabilities(state, n, dm=True).astype(np.float64).sum())
            if p > 0:
                eng.scale(state, compiled.nbits, 1.0 / p)
        else:
            eng.project(state, n, mask, value, 1.0)
            p = eng.norm2(state, n)
            if p > 0:
                eng.scale(state, n, 1.0 / math.sqrt(p))
        bits = np.array([[(idx >> (n - 1 - index[q])) & 1 for q in op.qubits]], dtype=np.int8)
        return [int(b) for b in _recorded_in_place(bits, op, self._prng)[0]]

    def _traj_needed(self, program) -> bool:
        """Does this circuit need per-repetition trajectories?  (Remembered
        per circuit: the answer depends only on its operations and on this
        simulator's kind and noise.)"""
        from cirq_gb300.ir import flatten_ops

        if not program.all_qubits():
            return False
        if not self._dm and self.noise is not cirq.NO_NOISE:
            return True
        store = self.__dict__.setdefault("_traj_memo", collections.OrderedDict())
        return _memo(store, program, "traj", lambda p: _traj.needs_trajectories(flatten_ops(p), self._dm))

    def _traj_states(self, program, qubits, resolver, initial_state, reps, records_only=False):
        """Yields (runner, device state, records) for `reps` trajectories; the
        state is the runner's buffer, valid until the next trajectory.  With
        records_only, ops after the last measurement are skipped."""
        ops = _traj.circuit_ops(self, program, qubits, resolver)
        if records_only:
            ops = _traj.records_relevant(ops)
        runner = _traj.TrajectoryRunner(self, ops, qubits, resolver)
        try:
            picks, pools = runner.prepare(reps)
            for r in range(reps):
                state, records = runner.run(initial_state, picks[r], pools, r)
                yield runner, _Borrowed(state), records
        finally:
            runner.close()

    def _unwrap_initial_state(self, initial_state, qubit_order):
        """A ``cirq.SimulationStateBase`` initial state -> (its raw tensor,
        its own qubit order).  As in the reference
        (``SimulatorBase._create_simulation_state``,
        cirq-core/cirq/sim/simulator_base.py:322-352, which uses such a state
        as is), the state's qubits and their order define the simulation;
        product states are merged first.  Other initial states pass through."""
        if not isinstance(initial_state, cirq.SimulationStateBase):
            return initial_state, qubit_order
        merged = initial_state.create_merged_state()
        qubits = tuple(merged.qubits)
        size = int(np.prod([q.dimension for q in qubits], dtype=np.int64))
        tensor = np.asarray(merged.target_tensor)
        if isinstance(merged, cirq.DensityMatrixSimulationState):
            if not self._dm:
                raise ValueError("a density-matrix initial state needs cirq_gb300.DensityMatrixSimulator")
            raw = tensor.reshape(size, size)
        elif isinstance(merged, cirq.StateVectorSimulationState):
            raw = tensor.reshape(-1)
        else:
            raise NotImplementedError(f"initial states of type {type(merged).__name__} are not supported")
        return raw, cirq.QubitOrder.explicit(qubits)

    # ---- SimulatesIntermediateState ------------------------------------------
    def simulate_moment_steps(
        self,
        circuit: cirq.AbstractCircuit,
        param_resolver: cirq.ParamResolverOrSimilarType = None,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
        initial_state: Any = None,
    ):
        """One step result per (noisy) moment, as
        ``SimulatesIntermediateState.simulate_moment_steps``
        (cirq-core/cirq/sim/simulator.py:607-640); see cirq_gb300/steps.py."""
        from cirq_gb300.steps import moment_steps

        initial_state, qubit_order = self._unwrap_initial_state(initial_state, qubit_order)
        if _qudits.has_qudits(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(circuit.all_qubits())):
            return _qudits.moment_steps(self, circuit, param_resolver, qubit_order, initial_state)
        return moment_steps(self, circuit, param_resolver, qubit_order, initial_state)

    def _traj_expectations(self, program, pslist, params, qubit_order, initial_state):
        qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
        index = {q: i for i, q in enumerate(qubits)}
        for ps in pslist:
            for q in ps.qubits:
                if q not in index:
                    raise ValueError(f"Qubit {q} of the observable is not in the qubit order")
        terms = [pauli_terms(ps, index, len(qubits)) for ps in pslist]
        eng = self.engine
        for r in cirq.to_resolvers(params):
            _check_all_resolved(program, r)
            for runner, state, _rec in self._traj_states(program, qubits, r, initial_state, 1):
                out = [complex(np.sum(eng.expect_paulis(state, runner.n, t, dm=self._dm))) for t in terms]
                state.free()
                yield out

    def _sample_records(self, state, compiled, meas_ops, repetitions) -> dict[str, np.ndarray]:
        """Terminal-measurement sampling, mirroring StepResult.sample_measurement_ops
        (cirq-core/cirq/sim/simulator.py:733-820) with _allow_repeated=True."""
        u = self._prng.random_sample(repetitions)
        samples = self.engine.sample(state, compiled.n, u, dm=self._dm).astype(np.int64)
        return self._records_from_samples(samples, compiled, meas_ops)

    def _records_from_samples(self, samples, compiled, meas_ops) -> dict[str, np.ndarray]:
        """run() records (repetitions, instances, bits) from sampled basis
        indices: invert masks and confusion maps applied per measurement."""
        n = compiled.n
        repetitions = len(samples)
        index = {q: i for i, q in enumerate(compiled.qubits)}
        results: dict[str, list] = {}
        for op in meas_ops:
            out = np.zeros((repetitions, len(op.qubits)), dtype=np.int8)
            for i, q in enumerate(op.qubits):
                out[:, i] = (samples >> (n - 1 - index[q])) & 1
            out, gate, qids = _qudits.recorded_view(op, out)
            inv = gate.full_invert_mask()
            for i in range(out.shape[1]):
                if inv[i]:
                    out[:, i] ^= out[:, i] < 2
            if gate.confusion_map:
                _confuse(out, qids, gate.confusion_map, self._prng)
            results.setdefault(gate.key, []).append(out)
        return {k: np.array(v).swapaxes(0, 1) for k, v in results.items()}

    # ---- SimulatesSamples ---------------------------------------------------
    def _split_untangled(self, ops, extra_qubits=()):
        """(parts, per-part op lists, measured flags, assembly, phase ops) of
        a flattened op list whose qubits fall into components no operation
        joins, or None (see _untangled_parts).  A measurement across
        components becomes one measurement per component under internal
        keys; assembly[key] lists, per instance, the (internal key, bit
        positions) pieces and the width.  `extra_qubits` (idle qubits of a
        qubit order) become components of their own."""
        from cirq_gb300.ir import is_keyed_channel, is_measurement_op

        if not self._dm and any(is_keyed_channel(op) for op in ops):
            return None  # channel records stay with the whole state
        parts = _untangled_parts(ops)
        if parts is None:
            return None
        seen = {q for part in parts for q in part}
        parts = parts + [[q] for q in extra_qubits if q not in seen]
        if len(parts) < 2:
            return None
        where = {q: i for i, part in enumerate(parts) for q in part}
        sub_ops: list = [[] for _ in parts]
        measured = [False] * len(parts)
        assembly: dict = {}
        phases = []
        for op in ops:
            if not op.qubits:
                phases.append(op)
                continue
            gate = getattr(op, "gate", None)
            if not is_measurement_op(op):
                sub_ops[where[op.qubits[0]]].append(op)
                continue
            if not isinstance(gate, cirq.MeasurementGate):
                return None
            key = cirq.measurement_key_name(op)
            t = len(assembly.setdefault(key, []))
            inv = gate.full_invert_mask()
            groups: dict = {}
            for pos, q in enumerate(op.qubits):
                groups.setdefault(where[q], []).append(pos)
            pieces = []
            for c, positions in groups.items():
                sub_key = f"{_PART}{key}{_PART}{t}{_PART}{c}"
                kwargs = {"key": sub_key, "invert_mask": tuple(inv[p] for p in positions)}
                if gate.confusion_map:  # within one component (checked by _untangled_parts)
                    kwargs["confusion_map"] = gate.confusion_map
                sub_ops[c].append(cirq.measure(*[op.qubits[p] for p in positions], **kwargs))
                measured[c] = True
                pieces.append((sub_key, positions))
            assembly[key].append((pieces, len(op.qubits)))
        return parts, sub_ops, measured, assembly, phases

    def _run_untangled(self, circuit, param_resolver, repetitions):
        """run() of a circuit whose qubits fall into components that no
        operation joins, one component at a time.  The components are
        independent, so the joint distribution of the records is the product
        of theirs, which is what the reference samples from its product
        state (cirq-core/cirq/sim/simulation_product_state.py).  Measurement
        bits split across components are reassembled in the original order,
        repetition by repetition; components without a measurement are not
        simulated.  Returns None when the circuit does not split."""
        from cirq_gb300.ir import flatten_ops

        split = self._split_untangled(flatten_ops(circuit))
        if split is None:
            return None
        parts, sub_ops, measured, assembly, _ = split
        records: dict = {}
        for c, ops_c in enumerate(sub_ops):
            if measured[c]:
                records.update(self._run(cirq.Circuit(ops_c), param_resolver, repetitions))
        out = {}
        for key, instances in assembly.items():
            width = max(w for _, w in instances)
            dtype = next(iter(records.values())).dtype if records else np.uint8
            arr = np.zeros((repetitions, len(instances), width), dtype=dtype)
            for t, (pieces, _) in enumerate(instances):
                for sub_key, positions in pieces:
                    arr[:, t, positions] = records[sub_key][:, 0, :]
            out[key] = arr
        return out

    def _simulate_untangled(self, program, params, qubit_order, initial_state):
        """simulate() of a circuit wider than one device state whose qubits
        fall into untangled components: each component is simulated alone
        and the results are held as the reference's own product state
        (cirq.SimulationProductState of per-component states, merged only on
        demand, as the reference's split_untangled_states does).  Yields
        trial results, or returns None when the circuit does not split or
        the initial state is not a basis index."""
        from cirq_gb300.ir import flatten_ops

        if initial_state is not None and not isinstance(initial_state, (int, np.integer)):
            return None
        qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
        split = self._split_untangled(flatten_ops(program), extra_qubits=qubits)
        if split is None:
            return None
        parts, sub_ops, _, assembly, phase_ops = split
        index = {q: i for i, q in enumerate(qubits)}
        basis = int(initial_state or 0)
        n = len(qubits)

        def results():
            for r in cirq.to_resolvers(params):
                _check_all_resolved(program, r)
                states: dict = {}
                meas_parts: dict = {}
                for c, part in enumerate(parts):
                    order = sorted(part, key=lambda q: index[q])
                    sub_basis = 0
                    for q in order:
                        sub_basis = (sub_basis << 1) | ((basis >> (n - 1 - index[q])) & 1)
                    res = self.simulate(cirq.Circuit(sub_ops[c]), r, qubit_order=order, initial_state=sub_basis)
                    st = res._final_simulator_state
                    for q in order:
                        states[q] = st
                    meas_parts.update(res.measurements)
                phase = 1.0 + 0j
                for op in cirq.resolve_parameters(phase_ops, r):
                    phase *= complex(np.asarray(cirq.unitary(op)).reshape(-1)[0])
                if self._dm:
                    states[None] = cirq.DensityMatrixSimulationState(
                        qubits=(), initial_state=np.ones((1, 1)), dtype=np.complex64)
                else:
                    states[None] = cirq.StateVectorSimulationState(
                        qubits=(), initial_state=np.array([phase], dtype=np.complex64), dtype=np.complex64)
                product = cirq.SimulationProductState(states, qubits, split_untangled_states=True)
                meas = {}
                for key, instances in assembly.items():
                    pieces, width = instances[-1]  # simulate() reports a key's last instance
                    bits = np.zeros(width, dtype=np.uint8)
                    for sub_key, positions in pieces:
                        bits[positions] = meas_parts[sub_key]
                    meas[key] = bits
                cls = cirq.DensityMatrixTrialResult if self._dm else cirq.StateVectorTrialResult
                yield cls(params=r, measurements=meas, final_simulator_state=product)

        return results()

    def _run(self, circuit, param_resolver, repetitions) -> dict[str, np.ndarray]:
        param_resolver = param_resolver or cirq.ParamResolver({})
        _check_all_resolved(circuit, param_resolver)
        if _symbolic_repetitions(circuit):
            circuit = cirq.resolve_parameters(circuit, param_resolver)
        if self.noise is not cirq.NO_NOISE:
            return self._noiseless()._run(self._reference_noisy_circuit(circuit, "run"), param_resolver, repetitions)
        qubits = tuple(sorted(circuit.all_qubits()))
        if _qudits.has_qudits(qubits):
            return _qudits.run(self, circuit, param_resolver, repetitions)
        if self._split_untangled_states and len(qubits) * (2 if self._dm else 1) > _MAX_STATE_BITS:
            rec = self._run_untangled(circuit, param_resolver, repetitions)
            if rec is not None:
                return rec
        if self._traj_needed(circuit):
            ops = _traj.circuit_ops(self, circuit, qubits, param_resolver)
            if self._dm:
                rec = _traj.run_batched_dm(self, ops, qubits, param_resolver, repetitions)
            else:
                rec = _traj.run_batched(self, ops, qubits, param_resolver, repetitions)
            if rec is not None:
                return rec
            per_rep = []
            for _, state, rec in self._traj_states(circuit, qubits, param_resolver, 0, repetitions,
                                                   records_only=True):
                state.free()
                per_rep.append(rec)
            return _traj.pad_records(per_rep)
        _, resolvers, compiled, meas = self._prepare(circuit, qubits, param_resolver)
        if compiled.n == 0:
            return {op.gate.key: np.zeros((repetitions, 1, 0), dtype=np.int8) for op in meas}
        pool = compiled.pool([param_resolver])[0]
        state = self._evolve(compiled, pool, 0)
        return self._sample_records(state, compiled, meas, repetitions)


def _untangled_parts(ops) -> list[list] | None:
    """Qubit components of a flattened op list that no operation joins
    (union-find over the qubits of multi-qubit non-measurement operations;
    measurements do not entangle), or None when the split is not valid:
    classical control, or a confusion map across components."""
    from cirq_gb300 import trajectories as tj
    from cirq_gb300.ir import is_measurement_op

    parent: dict = {}

    def find(x):
        while parent.setdefault(x, x) != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for op in ops:
        for q in op.qubits:
            find(q)
        if tj.is_classically_controlled(op):
            return None
        if len(op.qubits) > 1 and not is_measurement_op(op):
            r = find(op.qubits[0])
            for q in op.qubits[1:]:
                parent[find(q)] = r
    comps: dict = {}
    for q in sorted(parent):
        comps.setdefault(find(q), []).append(q)
    parts = list(comps.values())
    where = {q: i for i, part in enumerate(parts) for q in part}
    for op in ops:
        gate = getattr(op, "gate", None)
        if isinstance(gate, cirq.MeasurementGate) and gate.confusion_map:
            if len({where[q] for q in op.qubits}) > 1:
                return None
    return parts


class _Borrowed:
    """A non-owning view of a device buffer kept by the simulator (free() is a no-op)."""

    def __init__(self, buf):
        self._buf = buf
        self.ptr = buf.ptr
        self.nbytes = buf.nbytes
        self.engine = buf.engine

    def free(self) -> None:
        pass

    def upload(self, host):
        self._buf.upload(host)

    def download(self, host):
        return self._buf.download(host)


def _recorded_in_place(bits: np.ndarray, op, prng) -> np.ndarray:
    """The record of a measurement performed in place (simulate(), and
    run() with measurements that are not all terminal): its confusion map
    first, then its invert mask, as SimulationState.measure does
    (cirq-core/cirq/sim/simulation_state.py:70-98).  `bits` is
    (repetitions, qubits); a qudit measurement's record is its levels.
    Terminal sampling in run() applies them the other way round
    (_records_from_samples)."""
    bits, gate, qids = _qudits.recorded_view(op, bits)
    if gate.confusion_map:
        _confuse(bits, qids, gate.confusion_map, prng)
    inv = gate.full_invert_mask()
    for i in range(bits.shape[1]):
        if inv[i]:
            bits[:, i] ^= bits[:, i] < 2
    return bits


def _confuse(bits, qubits, confusion_map, prng) -> None:
    """Applies measurement confusion matrices to every repetition (rows of
    `bits`, in place), with the distribution of
    StepResult._confuse_results (cirq-core/cirq/sim/simulator.py:822-844):
    for each map entry in order, the entry's digits (big-endian, mixed
    radix) pick a row of its confusion matrix and the new digits are drawn
    from that row.  All repetitions are drawn at once per entry (one
    inverse-CDF lookup per repetition) instead of one prng.choice per
    repetition and entry; entries still apply in order, so overlapping
    entries see the digits the earlier ones wrote."""
    dims = [q.dimension for q in qubits]
    nrep = bits.shape[0]
    if nrep == 0:
        return
    for indices, confuser in confusion_map.items():
        mat_dims = [dims[k] for k in indices]
        conf = np.asarray(confuser, dtype=np.float64)
        row = np.zeros(nrep, dtype=np.int64)
        for k, d in zip(indices, mat_dims):
            row = row * d + bits[:, k].astype(np.int64)
        cdf = np.cumsum(conf, axis=1)
        u = prng.random_sample(nrep) * cdf[:, -1][row]
        new_val = np.minimum((u[:, None] >= cdf[row]).sum(axis=1), conf.shape[1] - 1)
        for k, d in reversed(list(zip(indices, mat_dims))):
            bits[:, k] = (new_val % d).astype(bits.dtype)
            new_val //= d


def _final_renormalize(eng, state, n: int) -> None:
    """Applies StateVectorTrialResult.final_state_vector's renormalisation rule
    (cirq-core/cirq/sim/state_vector_simulator.py:131-146) on the device, with
    the reference's warning when the norm is too far from 1 to renormalise."""
    _, norm = eng.final_renormalize(state, n)
    tol = float(np.sqrt(np.finfo(np.float32).eps))
    if abs(norm - 1) > tol:
        warnings.warn(
            f"final state vector's norm={np.float32(norm)!r} is too far from 1,"
            f" {abs(norm - 1)} > {tol}."
            "skipping renormalization"
        )


def _state_vector_state_private(qubits, vec: np.ndarray, shape):
    """A cirq.StateVectorSimulationState around `vec` (no copy), built from the
    reference's _BufferedStateVector and SimulationState.__init__."""
    from cirq.sim.state_vector_simulation_state import _BufferedStateVector

    st = cirq.StateVectorSimulationState.__new__(cirq.StateVectorSimulationState)
    buffered = _BufferedStateVector(vec.reshape(shape), np.empty(0, dtype=np.complex64))
    cirq.SimulationState.__init__(st, state=buffered, prng=None, qubits=tuple(qubits), classical_data=None)
    return st


def _state_vector_result(params, measurements, qubits, vec: np.ndarray):
    """Builds a genuine cirq.StateVectorTrialResult around `vec` without copying
    it; if the reference's internals have changed, through its public
    constructor instead (which copies and validates)."""
    shape = tuple(q.dimension for q in qubits)
    try:
        st = _state_vector_state_private(qubits, vec, shape)
    except Exception:
        st = cirq.StateVectorSimulationState(
            qubits=tuple(qubits), initial_state=vec.reshape(shape), dtype=np.complex64
        )
    res = cirq.StateVectorTrialResult(
        params=params, measurements=measurements, final_simulator_state=st
    )
    # the renormalisation rule was applied on the device
    res.__dict__["final_state_vector"] = vec
    return res


def _density_matrix_state_private(qubits, rho: np.ndarray, shape):
    """A cirq.DensityMatrixSimulationState around `rho` (no copy, no
    validation), built from the reference's _BufferedDensityMatrix and
    SimulationState.__init__."""
    from cirq.sim.density_matrix_simulation_state import _BufferedDensityMatrix

    st = cirq.DensityMatrixSimulationState.__new__(cirq.DensityMatrixSimulationState)
    empty = np.empty(0, dtype=np.complex64)
    buffered = _BufferedDensityMatrix(rho.reshape(shape + shape), [empty, empty, empty])
    cirq.SimulationState.__init__(st, state=buffered, prng=None, qubits=tuple(qubits), classical_data=None)
    return st


def _density_matrix_result(params, measurements, qubits, rho: np.ndarray):
    """Builds a genuine cirq.DensityMatrixTrialResult around `rho` without the
    reference's re-validation (an eigen-decomposition of the 2^n x 2^n matrix
    on the host, seconds at 13 qubits); rho comes from trace-preserving
    channels applied on the device."""
    shape = tuple(q.dimension for q in qubits)
    size = int(np.prod(shape, dtype=np.int64))
    try:
        st = _density_matrix_state_private(qubits, rho, shape)
    except Exception:  # the public constructor validates and copies
        st = cirq.DensityMatrixSimulationState(
            qubits=tuple(qubits), initial_state=rho.reshape(shape + shape), dtype=np.complex64
        )
    res = cirq.DensityMatrixTrialResult(params=params, measurements=measurements, final_simulator_state=st)
    # the reference fills final_density_matrix lazily with a host copy of the
    # state tensor (density_matrix_simulator.py:369-374: 44 ms at 13 qubits);
    # the downloaded matrix is already a fresh array, so it is handed over
    if hasattr(res, "_final_density_matrix"):
        res._final_density_matrix = rho.reshape(size, size)
    return res


class Simulator(
    _GpuSimulatorBase,
    cirq.SimulatesSamples,
    cirq.SimulatesExpectationValues,
    cirq.SimulatesFinalState,
    cirq.SimulatesAmplitudes,
):
    """GPU state-vector simulator with the API of ``cirq.Simulator``
    (``cirq-core/cirq/sim/sparse_simulator.py:31-218``)."""

    def _initial_device_state(self, compiled, initial_state, into=None):
        eng = self.engine
        n = compiled.n
        if initial_state is None:
            initial_state = 0
        if isinstance(initial_state, (int, np.integer)):
            if not 0 <= int(initial_state) < 2**n:
                raise ValueError(f"initial_state {initial_state} out of range for {n} qubits")
            return eng.new_state(n, basis=int(initial_state), nbits_dev=compiled.nbits_dev, into=into)
        if isinstance(initial_state, cirq.SimulationStateBase):
            raise NotImplementedError("unwrap SimulationState initial states first")
        if isinstance(initial_state, np.ndarray):
            # taken as given, without the normalisation check, as the
            # reference's _BufferedStateVector.create does
            # (cirq-core/cirq/sim/state_vector_simulation_state.py:76-90)
            vec = initial_state.reshape(-1).astype(np.complex64, copy=False)
            if vec.size != 2**n:
                raise ValueError(f"initial state has {vec.size} amplitudes, expected {2**n}")
        else:
            vec = cirq.to_valid_state_vector(initial_state, n, qid_shape=(2,) * n, dtype=np.complex64)
        return eng.new_state(n, initial=vec, nbits_dev=compiled.nbits_dev, into=into)

    def simulate_sweep_iter(
        self,
        program: cirq.AbstractCircuit,
        params: cirq.Sweepable,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
        initial_state: Any = None,
    ) -> Iterator[cirq.StateVectorTrialResult]:
        if _symbolic_repetitions(program):
            for r, resolved in _per_point(program, params):
                yield from self.simulate_sweep_iter(resolved, r, qubit_order, initial_state)
            return
        initial_state, qubit_order = self._unwrap_initial_state(initial_state, qubit_order)
        if self.noise is not cirq.NO_NOISE:
            yield from self._noiseless().simulate_sweep_iter(
                self._reference_noisy_circuit(program, "simulate"), params, qubit_order, initial_state
            )
            return
        if _qudits.has_qudits(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits())):
            yield from _qudits.simulate_sweep(self, program, params, qubit_order, initial_state)
            return
        if self._split_untangled_states:
            width = len(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
            if width * (2 if self._dm else 1) > _MAX_STATE_BITS:
                parts = self._simulate_untangled(program, params, qubit_order, initial_state)
                if parts is not None:
                    yield from parts
                    return
        if self._traj_needed(program):
            qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
            eng = self.engine
            for r in cirq.to_resolvers(params):
                _check_all_resolved(program, r)
                for runner, state, rec in self._traj_states(program, qubits, r, initial_state, 1):
                    _final_renormalize(eng, state, runner.n)
                    vec = eng.download_state(state, runner.n)
                    state.free()
                    meas = {k: np.array(v[-1], dtype=np.uint8) for k, v in rec.items()}
                    yield _state_vector_result(r, meas, qubits, vec)
            return
        qubits, resolvers, compiled, meas = self._prepare(program, qubit_order, params)
        if compiled.n == 0:
            for r in resolvers:
                vec = np.array([compiled.global_phase(r)], dtype=np.complex64)
                yield _state_vector_result(r, {}, qubits, vec)
            return
        pools = compiled.pool(resolvers)
        eng = self.engine
        for p, r in enumerate(resolvers):
            state = self._evolve(compiled, pools[p], initial_state)
            measurements = self._measure_terminal(state, compiled, meas)
            _final_renormalize(eng, state, compiled.n)
            vec = eng.download_state(state, compiled.n)
            state.free()
            yield _state_vector_result(r, measurements, qubits, vec)

    def simulate_expectation_values_sweep_iter(
        self,
        program: cirq.AbstractCircuit,
        observables: cirq.PauliSumLike | list[cirq.PauliSumLike],
        params: cirq.Sweepable,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
        initial_state: Any = None,
        permit_terminal_measurements: bool = False,
    ) -> Iterator[list[float]]:
        """Mirrors Simulator.simulate_expectation_values_sweep_iter
        (cirq-core/cirq/sim/sparse_simulator.py:193-218): expectation values are
        evaluated on the device from the final state, which never leaves HBM."""
        if _symbolic_repetitions(program):
            for r, resolved in _per_point(program, params):
                yield from self.simulate_expectation_values_sweep_iter(
                    resolved, observables, r, qubit_order, initial_state, permit_terminal_measurements
                )
            return
        initial_state, qubit_order = self._unwrap_initial_state(initial_state, qubit_order)
        if not permit_terminal_measurements and program.are_any_measurements_terminal():
            raise ValueError(
                "Provided circuit has terminal measurements, which may "
                "skew expectation values. If this is intentional, set "
                "permit_terminal_measurements=True."
            )
        if not isinstance(observables, list):
            observables = [observables]
        pslist = [cirq.PauliSum.wrap(o) for o in observables]
        for ps in pslist:
            if any(abs(p.coefficient.imag) > 0.0001 for p in ps):
                raise NotImplementedError(
                    "Cannot compute expectation value of a non-Hermitian "
                    f"PauliString <{ps}>. Coefficient must be real."
                )
        if self.noise is not cirq.NO_NOISE:
            yield from self._noiseless().simulate_expectation_values_sweep_iter(
                self._reference_noisy_circuit(program, "simulate"), pslist, params, qubit_order,
                initial_state, permit_terminal_measurements=True,
            )
            return
        if _qudits.has_qudits(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits())):
            yield from _qudits.expectation_values(self, program, pslist, params, qubit_order, initial_state)
            return
        if self._traj_needed(program) or program.has_measurements():
            # the reference evaluates the final state of simulate(), which
            # collapses measurements: one trajectory per point
            yield from self._traj_expectations(program, pslist, params, qubit_order, initial_state)
            return
        body_prog = cirq.Circuit(op for op in program.all_operations() if not cirq.is_measurement(op))
        qubits, resolvers, compiled, _ = self._prepare(body_prog, qubit_order, params)
        index = {q: i for i, q in enumerate(qubits)}
        for ps in pslist:
            for q in ps.qubits:
                if q not in index:
                    raise ValueError(f"Qubit {q} of the observable is not in the qubit order")
        terms = [pauli_terms(ps, index, compiled.n) for ps in pslist]
        pools = compiled.pool(resolvers)
        eng = self.engine
        for p, r in enumerate(resolvers):
            state = self._evolve(compiled, pools[p], initial_state)
            out = []
            for t in terms:
                vals = eng.expect_paulis(state, compiled.n, t)
                out.append(complex(np.sum(vals)))
            state.free()
            yield out

    def compute_amplitudes_sweep_iter(
        self,
        program: cirq.AbstractCircuit,
        bitstrings: Sequence[int],
        params: cirq.Sweepable,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
    ) -> Iterator[Sequence[complex]]:
        """Amplitudes of the final state (cirq-core/cirq/sim/state_vector_simulator.py:74-98)."""
        if isinstance(bitstrings, np.ndarray) and len(bitstrings.shape) > 1:
            raise ValueError(
                "The list of bitstrings must be input as a 1-dimensional array of ints. "
                f"Got an array with shape {bitstrings.shape}."
            )
        if isinstance(bitstrings, tuple):
            bitstrings = list(bitstrings)
        for result in self.simulate_sweep_iter(program, params, qubit_order):
            yield result.final_state_vector[bitstrings].tolist()


class DensityMatrixSimulator(
    _GpuSimulatorBase,
    cirq.SimulatesSamples,
    cirq.SimulatesExpectationValues,
    cirq.SimulatesFinalState,
):
    """GPU density-matrix simulator with the API of ``cirq.DensityMatrixSimulator``
    (``cirq-core/cirq/sim/density_matrix_simulator.py:32-236``).

    rho (2^n x 2^n complex64) lives in HBM as a 2n-bit vector; unitaries act
    as U on the row bits and conj(U) on the column bits, channels as fused
    superoperators sum_i conj(K_i) (x) K_i."""

    _dm = True

    def _initial_device_state(self, compiled, initial_state, into=None):
        eng = self.engine
        n = compiled.n
        if initial_state is None:
            initial_state = 0
        if isinstance(initial_state, (int, np.integer)):
            if not 0 <= int(initial_state) < 2**n:
                raise ValueError(f"initial_state {initial_state} out of range for {n} qubits")
            i = int(initial_state)
            return eng.new_state(2 * n, basis=(i << n) | i, nbits_dev=compiled.nbits_dev, into=into)
        if isinstance(initial_state, cirq.SimulationStateBase):
            raise NotImplementedError("unwrap SimulationState initial states first")
        if isinstance(initial_state, np.ndarray) and initial_state.dtype != np.complex64:
            # the reference casts an array to the simulator's dtype first
            # (cirq-core/cirq/sim/density_matrix_simulation_state.py:84-89)
            initial_state = initial_state.astype(np.complex64)
        rho = cirq.to_valid_density_matrix(initial_state, n, qid_shape=(2,) * n, dtype=np.complex64)
        return eng.new_state(2 * n, initial=rho.reshape(-1), nbits_dev=compiled.nbits_dev, into=into)

    def simulate_sweep_iter(
        self,
        program: cirq.AbstractCircuit,
        params: cirq.Sweepable,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
        initial_state: Any = None,
    ) -> Iterator[cirq.DensityMatrixTrialResult]:
        if _symbolic_repetitions(program):
            for r, resolved in _per_point(program, params):
                yield from self.simulate_sweep_iter(resolved, r, qubit_order, initial_state)
            return
        initial_state, qubit_order = self._unwrap_initial_state(initial_state, qubit_order)
        if self.noise is not cirq.NO_NOISE:
            yield from self._noiseless().simulate_sweep_iter(
                self._reference_noisy_circuit(program, "simulate"), params, qubit_order, initial_state
            )
            return
        if _qudits.has_qudits(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits())):
            yield from _qudits.simulate_sweep(self, program, params, qubit_order, initial_state)
            return
        if self._split_untangled_states:
            width = len(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
            if width * (2 if self._dm else 1) > _MAX_STATE_BITS:
                parts = self._simulate_untangled(program, params, qubit_order, initial_state)
                if parts is not None:
                    yield from parts
                    return
        if self._traj_needed(program):
            qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))
            eng = self.engine
            for r in cirq.to_resolvers(params):
                _check_all_resolved(program, r)
                for runner, state, rec in self._traj_states(program, qubits, r, initial_state, 1):
                    n = runner.n
                    rho = eng.download_state(state, 2 * n).reshape(2**n, 2**n)
                    state.free()
                    meas = {k: np.array(v[-1], dtype=np.uint8) for k, v in rec.items()}
                    yield _density_matrix_result(r, meas, qubits, rho)
            return
        qubits, resolvers, compiled, meas = self._prepare(program, qubit_order, params)
        n = compiled.n
        if n == 0:
            for r in resolvers:
                st = cirq.DensityMatrixSimulationState(qubits=(), initial_state=np.ones((1, 1)), dtype=np.complex64)
                yield cirq.DensityMatrixTrialResult(params=r, measurements={}, final_simulator_state=st)
            return
        pools = compiled.pool(resolvers)
        eng = self.engine
        for p, r in enumerate(resolvers):
            state = self._evolve(compiled, pools[p], initial_state)
            measurements = self._measure_terminal(state, compiled, meas)
            rho = eng.download_state(state, 2 * n).reshape(2**n, 2**n)
            state.free()
            yield _density_matrix_result(r, measurements, qubits, rho)

    def simulate_expectation_values_sweep_iter(
        self,
        program: cirq.AbstractCircuit,
        observables: cirq.PauliSumLike | list[cirq.PauliSumLike],
        params: cirq.Sweepable,
        qubit_order: cirq.QubitOrderOrList = cirq.QubitOrder.DEFAULT,
        initial_state: Any = None,
        permit_terminal_measurements: bool = False,
    ) -> Iterator[list[float]]:
        """Mirrors DensityMatrixSimulator.simulate_expectation_values_sweep_iter
        (cirq-core/cirq/sim/density_matrix_simulator.py:204-236): Tr(P rho)
        is evaluated on the device."""
        if _symbolic_repetitions(program):
            for r, resolved in _per_point(program, params):
                yield from self.simulate_expectation_values_sweep_iter(
                    resolved, observables, r, qubit_order, initial_state, permit_terminal_measurements
                )
            return
        initial_state, qubit_order = self._unwrap_initial_state(initial_state, qubit_order)
        if not permit_terminal_measurements and program.are_any_measurements_terminal():
            raise ValueError(
                "Provided circuit has terminal measurements, which may "
                "skew expectation values. If this is intentional, set "
                "permit_terminal_measurements=True."
            )
        if not isinstance(observables, list):
            observables = [observables]
        pslist = [cirq.PauliSum.wrap(o) for o in observables]
        if self.noise is not cirq.NO_NOISE:
            yield from self._noiseless().simulate_expectation_values_sweep_iter(
                self._reference_noisy_circuit(program, "simulate"), pslist, params, qubit_order,
                initial_state, permit_terminal_measurements=True,
            )
            return
        if _qudits.has_qudits(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits())):
            yield from _qudits.expectation_values(self, program, pslist, params, qubit_order, initial_state)
            return
        if self._traj_needed(program) or program.has_measurements():
            yield from self._traj_expectations(program, pslist, params, qubit_order, initial_state)
            return
        body_prog = cirq.Circuit(op for op in program.all_operations() if not cirq.is_measurement(op))
        qubits, resolvers, compiled, _ = self._prepare(body_prog, qubit_order, params)
        index = {q: i for i, q in enumerate(qubits)}
        terms = [pauli_terms(ps, index, compiled.n) for ps in pslist]
        pools = compiled.pool(resolvers)
        eng = self.engine
        for p, r in enumerate(resolvers):
            state = self._evolve(compiled, pools[p], initial_state)
            out = []
            for t in terms:
                vals = eng.expect_paulis(state, compiled.n, t, dm=True)
                out.append(complex(np.sum(vals)))
            state.free()
            yield out
