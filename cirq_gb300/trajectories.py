"""Per-repetition trajectories: mid-circuit measurement and state-vector noise.

Follows the reference's ``SimulatorBase._run``
(``cirq-core/cirq/sim/simulator_base.py:216-273``): when a circuit has
measurements that are not terminal, or (for a state vector) noise, every
repetition simulates the circuit again,

* collapsing the state at every measurement -- one outcome drawn from the
  Born distribution of the measured qubits, then projection and
  renormalisation (``cirq-core/cirq/sim/state_vector.py:235-322``,
  ``cirq-core/cirq/sim/density_matrix_utils.py:97-183``);
* applying one operator of every channel: a mixture's unitary drawn with the
  mixture's fixed probabilities
  (``cirq-core/cirq/sim/state_vector_simulation_state.py:183-204``), a
  general channel's Kraus operator K_i drawn with weight ||K_i psi||^2 and
  applied as K_i / ||K_i psi|| (:206-257, same fallback to the heaviest
  operator when round-off leaves the draw unassigned).

On the GPU a circuit becomes a list of items: fused unitary segments (one
plan each, compiled once), measurement events and general-channel events.
Mixture operations stay inside the fused segments as :class:`Slot`s whose
matrix is each trajectory's draw, so a noisy circuit keeps its fused passes;
the draws of all repetitions are made up front and their matrix pools built
in one vectorised call per segment.  A general channel on k <= 5 qubits
reads the reduced density matrix of its qubits (one batched state read for
k <= 2; the 4^k - 1 Pauli expectations, rho_Q = 2^-k sum_P <P> P, for wider
channels), computes the weights Tr(K_i^dagger K_i rho_Q) on the host, and
applies the drawn operator as a one-slot segment.  The density-matrix simulator needs trajectories only for
mid-circuit measurement (its channels are exact superoperators).
"""

from __future__ import annotations

import dataclasses
import math
from typing import Any

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.ir import UnsupportedOperation, flatten_ops, is_keyed_channel, is_loop
from cirq_gb300.program import Slot, TrajectoryPoint
from cirq_gb300.qudits import record_qids

cirq = ensure_cirq()

_PAULI = {
    0: np.eye(2, dtype=np.complex128),
    1: np.array([[0, 1], [1, 0]], dtype=np.complex128),
    2: np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    3: np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


@dataclasses.dataclass
class Segment:
    ops: list  # unitary ops and mixture Slots
    slots: list  # (slot id, op) of the mixture slots in this segment


@dataclasses.dataclass
class Measure:
    op: Any


@dataclasses.dataclass
class Channel:
    op: Any
    slot: int
    key: str | None = None  # a keyed channel records the index of its drawn operator


@dataclasses.dataclass
class Loop:
    """A CircuitOperation with ``repeat_until``: in each trajectory its body
    runs, then its condition is resolved on that trajectory's records, until
    it holds (``CircuitOperation._act_on_``,
    cirq-core/cirq/circuits/circuit_operation.py)."""

    op: Any  # the CircuitOperation (untagged)

    def body(self):
        return self.op.replace(repeat_until=None).mapped_circuit(deep=False)

    def condition(self):
        # the condition with the operation's key mapping and path applied
        mapped = getattr(self.op, "_mapped_repeat_until", None)
        return mapped if mapped is not None else self.op.repeat_until


@dataclasses.dataclass
class Conditional:
    """A classically controlled operation: applied in a trajectory when all
    of its conditions hold on that trajectory's records so far
    (``ClassicallyControlledOperation._act_on_``,
    cirq-core/cirq/ops/classically_controlled_operation.py)."""

    op: Any  # the ClassicallyControlledOperation (untagged)
    inner: Any  # the controlled operation
    # "program": a compiled program (a unitary; on the density-matrix
    # simulator also a channel, as its superoperator); "channel": a Kraus
    # draw in slot `slot` (state-vector simulator).  The reference forbids
    # classical control of operations with measurement keys.
    kind: str = "program"
    slot: int = -1


def is_classically_controlled(op) -> bool:
    return isinstance(op.untagged, cirq.ClassicallyControlledOperation)


def _store(records: dict, measured: dict):
    """A ClassicalDataDictionaryStore of one trajectory's records."""
    channel = {k for k, v in measured.items() if v and v[0] is None}  # keyed channels' records
    keyed = {cirq.MeasurementKey.parse_serialized(k): [tuple(int(b) for b in bits) for bits in v]
             for k, v in records.items() if k not in channel}
    chans = {cirq.MeasurementKey.parse_serialized(k): [int(v[0]) for v in records[k]] for k in channel}
    qubits = {cirq.MeasurementKey.parse_serialized(k): [tuple(q) for q in v] for k, v in measured.items()
              if k not in channel}
    return cirq.ClassicalDataDictionaryStore(_records=keyed, _measured_qubits=qubits, _channel_records=chans)


def conditions_hold(op, records: dict, measured: dict) -> bool:
    """Evaluates a ClassicallyControlledOperation's conditions with the
    reference's own Condition.resolve (cirq-core/cirq/value/condition.py)
    on the trajectory's records: records[key] = [bits, ...] (as recorded,
    invert masks applied), measured[key] = [qubits, ...] of each instance
    (None for a keyed channel's record, [operator index]).
    A condition on a key not measured yet raises ValueError, as the
    reference does."""
    store = _store(records, measured)
    return all(c.resolve(store) for c in op.classical_controls)


def needs_trajectories(ops, dm: bool) -> bool:
    """True when a flattened op list cannot be simulated once and sampled."""
    from cirq_gb300.ir import is_measurement_op

    unitary_families = (cirq.EigenGate, cirq.PhasedXZGate, cirq.MatrixGate, cirq.PhasedXPowGate)
    gate_op, meas = cirq.GateOperation, cirq.MeasurementGate
    seen_measure = False
    for op in ops:
        if type(op) is gate_op:
            gate = op.gate
            if isinstance(gate, meas):
                seen_measure = True
                continue
            if isinstance(gate, unitary_families):
                if seen_measure:
                    return True  # an operation after a measurement
                continue
        if is_classically_controlled(op) or is_loop(op):
            return True
        if is_measurement_op(op):
            seen_measure = True
            continue
        if seen_measure and op.qubits:
            return True  # an operation after a measurement
        if isinstance(getattr(op, "gate", None), unitary_families):
            continue
        if not dm and not cirq.is_parameterized(op) and not cirq.has_unitary(op):
            return True
    return False


def build_items(ops, dm: bool) -> tuple[list, int]:
    """Splits a flattened op list into segments and events; returns (items,
    number of slots)."""
    items: list = []
    cur: list = []
    cur_slots: list = []
    nslot = 0

    def flush():
        nonlocal cur, cur_slots
        if cur:
            items.append(Segment(cur, cur_slots))
        cur, cur_slots = [], []

    for op in ops:
        if is_loop(op):
            flush()
            items.append(Loop(op.untagged))
            continue
        if is_classically_controlled(op):
            cc = op.untagged
            inner = cc.without_classical_controls()
            if cirq.is_parameterized(inner):
                raise UnsupportedOperation(f"classical control of a parameterized operation: {op!r}")
            flush()
            if dm or cirq.has_unitary(inner):
                items.append(Conditional(cc, inner, "program"))
            elif cirq.has_kraus(inner):
                if len(inner.qubits) > 5:
                    raise UnsupportedOperation(f"channels on more than 5 qubits are not supported: {op!r}")
                items.append(Conditional(cc, inner, "channel", nslot))
                nslot += 1
            else:
                raise TypeError(
                    "Can't simulate operations that don't implement SupportsUnitary, "
                    f"SupportsConsistentApplyUnitary, SupportsMixture or is a measurement: {op!r}"
                )
            continue
        if is_keyed_channel(op):
            if dm:
                cur.append(op)  # a channel; the density-matrix simulator records nothing
                continue
            if len(op.qubits) > 5:
                raise UnsupportedOperation(f"channels on more than 5 qubits are not supported: {op!r}")
            flush()
            items.append(Channel(op, nslot, cirq.measurement_key_name(op)))
            nslot += 1
            continue
        if cirq.is_measurement(op):
            if not isinstance(getattr(op, "gate", None), cirq.MeasurementGate):
                raise NotImplementedError(f"unsupported measurement {op!r}")
            flush()
            items.append(Measure(op))
            continue
        if dm or not op.qubits or cirq.is_parameterized(op) or cirq.has_unitary(op):
            cur.append(op)
            continue
        if cirq.has_mixture(op):
            cur.append(Slot(op, nslot))
            cur_slots.append((nslot, op))
            nslot += 1
            continue
        if cirq.has_kraus(op):
            if len(op.qubits) > 5:
                raise UnsupportedOperation(f"channels on more than 5 qubits are not supported: {op!r}")
            flush()
            items.append(Channel(op, nslot))
            nslot += 1
            continue
        # the reference's error for an operation it cannot act on
        # (cirq-core/cirq/sim/state_vector_simulation_state.py:395-399)
        raise TypeError(
            "Can't simulate operations that don't implement SupportsUnitary, "
            f"SupportsConsistentApplyUnitary, SupportsMixture or is a measurement: {op!r}"
        )
    flush()
    return items, nslot


def records_relevant(ops):
    """The ops that can influence run() records: everything after the last
    measurement (for instance noise a model inserts after the final
    measurement moment) changes no recorded outcome."""
    last = max((i for i, op in enumerate(ops) if cirq.is_measurement(op)), default=-1)
    return list(ops[: last + 1]) if last >= 0 else list(ops)


def circuit_ops(sim, program, qubits, resolver):
    """The resolved operations of a circuit whose noise is already placed
    (measurements included)."""
    if sim.noise is not cirq.NO_NOISE:
        # the entry points place noise first (_reference_noisy_circuit)
        raise RuntimeError("internal: a noise model reached the trajectory runner unplaced")
    return flatten_ops(cirq.resolve_parameters(program, resolver))


_MAX_SLOT_PROGRAMS = 256  # one-op programs kept per simulator


def slot_program(sim, op_qubits, qubits):
    """A compiled one-op program whose matrix each trajectory supplies as
    pick 0 (a Kraus operator or a projector), cached per simulator by the
    op's qubits: every channel or measurement on the same qubits shares it."""
    cache = sim.__dict__.setdefault("_slot_programs", {})
    key = (tuple(op_qubits), tuple(qubits))
    c = cache.get(key)
    if c is None:
        if len(cache) >= _MAX_SLOT_PROGRAMS:
            cache.clear()
        from cirq_gb300.program import CompiledCircuit

        op = cirq.IdentityGate(len(op_qubits)).on(*op_qubits)
        c = CompiledCircuit([Slot(op, 0)], qubits, dm=False, planner=sim.planner,
                            resolvers=[cirq.ParamResolver({})])
        cache[key] = c
    return c


class TrajectoryRunner:
    """Runs trajectories of one resolved circuit on a simulator's engine."""

    def __init__(self, sim, ops, qubits, resolver):
        self.sim = sim
        self.qubits = tuple(qubits)
        self.index = {q: i for i, q in enumerate(self.qubits)}
        self.n = len(self.qubits)
        self.dm = sim._dm
        self.resolver = resolver
        self.items, self.nslot = build_items(ops, self.dm)
        base = [cirq.ParamResolver({})]
        self.compiled = [
            sim._compile(it.ops, self.qubits, base) if isinstance(it, Segment)
            else sim._compile([it.inner], self.qubits, base)
            if isinstance(it, Conditional) and it.kind == "program"
            else None
            for it in self.items
        ]
        self.empty = sim._compile([], self.qubits, base)  # geometry of the state buffer
        # Kraus channels (drawn per trajectory), plain or classically controlled
        channels = [it if isinstance(it, Channel) else Channel(it.inner, it.slot) for it in self.items
                    if isinstance(it, Channel) or (isinstance(it, Conditional) and it.kind == "channel")]
        self.kraus_seg = {c.slot: slot_program(sim, c.op.qubits, self.qubits) for c in channels}
        self._kraus = {c.slot: [np.asarray(k, dtype=np.complex128) for k in cirq.kraus(c.op)] for c in channels}
        # the bodies of repeat-until loops, each with a runner of its own
        self._loops = {j: TrajectoryRunner(sim, flatten_ops(it.body()), self.qubits, resolver)
                       for j, it in enumerate(self.items) if isinstance(it, Loop)}
        # device buffers reused by every trajectory: the state and one
        # matrix pool per segment / channel
        self._state = None
        self._pools: dict = {}

    def _pool_dev(self, key, pool: np.ndarray):
        eng = self.sim.engine
        pool = np.ascontiguousarray(pool, dtype=np.complex64)
        buf = self._pools.get(key)
        if buf is None or buf.nbytes < max(pool.nbytes, 16):
            buf = eng.alloc(max(pool.nbytes, 16))
            self._pools[key] = buf
        buf.upload(pool)
        return buf

    def close(self) -> None:
        for sub in self._loops.values():
            sub.close()
        for buf in self._pools.values():
            buf.free()
        self._pools.clear()
        if self._state is not None:
            self._state.free()
            self._state = None

    def channel_bits(self, op) -> list:
        """Global index bits of a channel's qubits (first qubit first)."""
        return [self.n - 1 - self.index[q] for q in op.qubits]

    def channel_rdm(self, states, nbits: int, npoints: int, op) -> np.ndarray:
        """(npoints, d, d) reduced density matrices of a channel's qubits:
        one state read per point for 1-2 qubits, the 4^k - 1 Pauli
        expectations of the wider channels otherwise."""
        eng = self.sim.engine
        k = len(op.qubits)
        if k <= 2:
            return eng.points_rdm(states, nbits, npoints, self.channel_bits(op))
        from cirq_gb300.engine import Engine

        recs, mats = self._pauli_basis(op)
        vals = np.real(eng.points_expect(states, nbits, npoints, Engine.pauli_records(recs)))
        d = 2**k
        rho = np.eye(d, dtype=np.complex128)[None] + np.einsum("pt,tij->pij", vals, np.array(mats))
        return rho / d

    def _pauli_basis(self, op):
        """Pauli strings on the channel's qubits: (records, matrices)."""
        k = len(op.qubits)
        recs, mats = [], []
        for code in range(1, 4**k):
            x = zy = ny = 0
            m = np.eye(1, dtype=np.complex128)
            for j, q in enumerate(op.qubits):
                p = (code >> (2 * (k - 1 - j))) & 3
                b = 1 << (self.n - 1 - self.index[q])
                if p in (1, 2):
                    x |= b
                if p in (2, 3):
                    zy |= b
                if p == 2:
                    ny += 1
                m = np.kron(m, _PAULI[p])
            recs.append((x, zy, ny, 1.0))
            mats.append(m)
        return recs, mats

    # ---- host-side draws ---------------------------------------------------
    def _draw_mixtures(self, reps: int) -> dict:
        """slot -> (its unitaries (n, d, d), each trajectory's choice (reps,)),
        drawn with the mixture's probabilities (the reference's mixture
        sampling, cirq-core/cirq/sim/state_vector_simulation_state.py:183-205)."""
        prng = self.sim._prng
        draws = {}
        mixtures: dict = {}  # a mixture depends on the gate only, not on its qubits
        for it in self.items:
            if not isinstance(it, Segment):
                continue
            for sid, op in it.slots:
                key = getattr(op, "gate", None)
                try:
                    hash(key)
                except TypeError:  # an unhashable gate: no caching
                    key = None
                if key is None or key not in mixtures:
                    probs, unitaries = zip(*cirq.mixture(op))
                    entry = (np.asarray(probs, dtype=np.float64),
                             np.array([np.asarray(u, dtype=np.complex128) for u in unitaries]))
                    if key is not None:
                        mixtures[key] = entry
                else:
                    entry = mixtures[key]
                p, U = entry
                choice = prng.choice(len(U), size=reps, p=p / p.sum())
                draws[sid] = (U, choice)
        return draws

    # ---- one trajectory ------------------------------------------------------
    def run(self, initial_state, picks: dict, pools: list, rep: int):
        """One trajectory; returns (device state, records {key: [bits, ...]}).
        The state buffer belongs to the runner and is reused by the next
        trajectory."""
        sim = self.sim
        if self._state is None:
            self._state = sim._initial_device_state(self.empty, initial_state)
        else:
            sim._initial_device_state(self.empty, initial_state, into=self._state)
        return self._state, self.apply(self._state, picks, pools, rep)

    def apply(self, state, picks: dict, pools: list, rep: int, records: dict | None = None,
              measured: dict | None = None) -> dict:
        """Applies the items to a device state in place; returns the records.
        `records` / `measured` (key -> bits / qubits of each instance) carry
        earlier measurements of the same trajectory, for classical control;
        they are extended in place."""
        sim = self.sim
        eng = sim.engine
        records = {} if records is None else records
        measured = {} if measured is None else measured
        for j, it in enumerate(self.items):
            if isinstance(it, Segment):
                c = self.compiled[j]
                if c.plan.npasses:
                    pool = pools[j][rep] if pools[j] is not None else c.plan.pool
                    eng.run(state, c.nbits_dev, c.plan, self._pool_dev(("seg", j), pool))
            elif isinstance(it, Measure):
                self._measure(state, it.op, records, measured)
            elif isinstance(it, Loop):
                sub = self._loops[j]
                cond = it.condition()
                while True:
                    sub_picks, sub_pools = sub.prepare(1)
                    sub.apply(state, sub_picks[0], sub_pools, 0, records, measured)
                    if cond.resolve(_store(records, measured)):
                        break
            elif isinstance(it, Conditional):
                if not conditions_hold(it.op, records, measured):
                    continue
                if it.kind == "channel":
                    self._apply_kraus(state, Channel(it.inner, it.slot), picks)
                else:
                    c = self.compiled[j]
                    if c.plan.npasses:
                        eng.run(state, c.nbits_dev, c.plan, self._pool_dev(("seg", j), c.plan.pool))
            else:
                index = self._apply_kraus(state, it, picks)
                if it.key is not None:
                    records.setdefault(it.key, []).append([index])
                    measured.setdefault(it.key, []).append(None)
        return records

    def _measure(self, state, op, records: dict, measured: dict) -> None:
        bits = self.sim._measure_op(state, self.empty, op)
        key = cirq.measurement_key_name(op)
        records.setdefault(key, []).append(bits)
        measured.setdefault(key, []).append(record_qids(op))

    def _apply_kraus(self, state, it: Channel, picks: dict) -> None:
        eng = self.sim.engine
        ks = self._kraus[it.slot]
        rho = self.channel_rdm(state, self.empty.nbits_dev, 1, it.op)[0]
        weights = [max(float(np.real(np.trace(K.conj().T @ K @ rho))), 0.0) for K in ks]
        p = self.sim._prng.random()
        fallback = int(np.argmax(weights))
        index = None
        for i, w in enumerate(weights):
            p -= w
            if p < 0:
                index = i
                break
        if index is None or weights[index] == 0:
            index = fallback
        w = weights[index]
        picks[it.slot] = ks[index] / math.sqrt(w)
        c = self.kraus_seg[it.slot]
        pool = c.pool([TrajectoryPoint(self.resolver, {0: picks[it.slot]})])[0]
        eng.run(state, c.nbits_dev, c.plan, self._pool_dev(("kraus", it.slot), pool))
        return index

    def prepare(self, reps: int):
        """Draws the mixtures of `reps` trajectories; returns (picks, pools):
        per-trajectory dicts for the channel draws made later, and each
        segment's (reps, pool_len) matrix pools (None without slots)."""
        draws = self._draw_mixtures(reps)
        picks = [dict() for _ in range(reps)]
        pools = []
        for j, it in enumerate(self.items):
            c = self.compiled[j]
            if isinstance(it, Segment) and c.plan.npasses and it.slots:
                batch, codes = self._segment_batch(c, draws, reps)
                pools.append(c.pool_from_batch(batch, reps, codes))
            else:
                pools.append(None)
        return picks, pools

    def _segment_batch(self, c, draws: dict, reps: int):
        """A segment's gate matrices for `reps` trajectories: slots from the
        draws (with their choice indices as codes, so fused ops are built once
        per distinct combination), everything else once at the base point."""
        values: dict = {}
        base = [self.resolver]
        batch, codes = {}, {}
        for i, src in enumerate(c.sources):
            if src.slot is not None:
                U, choice = draws[src.slot]
                batch[i] = U[choice]
                codes[i] = choice
            else:
                m = src.matrices(base, values)
                batch[i] = np.broadcast_to(m[0], (reps,) + m.shape[1:])
        return batch, codes


def pad_records(per_rep: list[dict]) -> dict[str, np.ndarray]:
    """Repetition records -> {key: (repetitions, instances, bits) uint8}, padded
    like the reference's ``pad_evenly`` (simulator_base.py:265-271)."""
    keys: list = []
    for rec in per_rep:
        for k in rec:
            if k not in keys:
                keys.append(k)
    out = {}
    for k in keys:
        rows = [rec.get(k, []) for rec in per_rep]
        width = max(len(r[0]) for r in rows if r)
        largest = max(len(r) for r in rows)
        xs = np.zeros((len(rows), largest, width), dtype=np.uint8)
        for i, r in enumerate(rows):
            for j, bits in enumerate(r):
                xs[i, j, : len(bits)] = bits
        out[k] = xs
    return out


def _z_subset_records(runner, qubits_m):
    """Unit Z-string records for every nonempty subset S of the measured
    qubits (bit j of S <-> qubits_m[j]) and the subset masks."""
    m = len(qubits_m)
    recs, masks = [], []
    for S in range(1, 1 << m):
        zy = 0
        for j, q in enumerate(qubits_m):
            if (S >> j) & 1:
                zy |= 1 << (runner.n - 1 - runner.index[q])
        recs.append((0, zy, 0, 1.0))
        masks.append(S)
    return recs, np.array(masks, dtype=np.int64)


def run_batched(sim, ops, qubits, resolver, reps: int):
    """All repetitions of a state-vector circuit with noise and/or
    mid-circuit measurements evolved together (see the module doc):
    segments as batched passes with each trajectory's mixture draws,
    general channels and mid-circuit measurements as batched Pauli
    expectations -> per-trajectory draws on the host -> one batched
    one-slot pass (K_i / sqrt(w_i), or the projector / sqrt(p)), terminal
    measurements as one batched draw.  Returns run() records, or None when a
    mid-circuit measurement covers more than 5 qubits (the caller then runs
    trajectories one by one)."""
    from cirq_gb300.engine import Engine
    from cirq_gb300.simulator import _recorded_in_place

    if reps < 1 or getattr(sim.planner, "tensor", False):
        return None  # batched points run on the CUDA-core passes only
    ops = records_relevant(ops)
    items, _ = build_items(ops, dm=False)
    last_unitary = max((i for i, it in enumerate(items) if not isinstance(it, Measure)), default=-1)
    for i, it in enumerate(items):
        if isinstance(it, Measure) and i < last_unitary and len(it.op.qubits) > 5:
            return None
        if isinstance(it, Loop):
            return None  # a data-dependent number of iterations per trajectory
    terminal = [it.op for it in items[last_unitary + 1 :]]
    body = items[: last_unitary + 1]
    runner = TrajectoryRunner(sim, ops, qubits, resolver)
    eng = sim.engine
    prng = sim._prng
    try:
        picks, pools = runner.prepare(reps)
        n = runner.empty.nbits_dev
        _, free, _ = eng.device_info()
        budget = max(1 << 28, min(int(free) // 2, 32 << 30))
        chunk = max(1, min(reps, 65535, budget // (8 << n), (1 << 24) >> max(n - 10, 0)))
        # one-slot programs of the mid-circuit measurements (projector slots)
        proj = {}
        for i, it in enumerate(body):
            if isinstance(it, Measure):
                proj[i] = slot_program(sim, it.op.qubits, runner.qubits)
        # one-slot programs of the classically controlled unitaries
        for i, it in enumerate(body):
            if isinstance(it, Conditional) and it.kind == "program":
                proj[i] = slot_program(sim, it.inner.qubits, runner.qubits)
        states = eng.alloc((8 << n) * chunk)
        records: list = [dict() for _ in range(reps)]
        samples = np.empty(reps, dtype=np.int64)

        def run_slot(compiled, mats, k, start):
            """One-slot program with a per-trajectory matrix (mats: (k, d, d))."""
            pool = np.ascontiguousarray(compiled.pool_from_batch({0: np.asarray(mats)}, k), dtype=np.complex64)
            plen = pool.shape[1]
            if plen & 1:
                pool = np.concatenate([pool, np.zeros((k, 1), np.complex64)], axis=1)
                plen += 1
            pool_dev = eng.upload(pool.reshape(-1))
            eng.run_points(states, n, k, compiled.plan, pool_dev, plen)
            eng.sync()
            pool_dev.free()

        try:
            for start in range(0, reps, chunk):
                k = min(chunk, reps - start)
                eng.points_set_zero(states, n, k)
                measured: dict = {}  # key -> qubits of each instance (same for every trajectory)
                for j, it in enumerate(body):
                    if isinstance(it, Segment):
                        c = runner.compiled[j]
                        if not c.plan.npasses:
                            continue
                        pool = pools[j] if pools[j] is not None else np.broadcast_to(c.plan.pool, (reps, len(c.plan.pool)))
                        pool = np.ascontiguousarray(pool[start : start + k], dtype=np.complex64)
                        plen = pool.shape[1]
                        if plen & 1:
                            pool = np.concatenate([pool, np.zeros((k, 1), np.complex64)], axis=1)
                            plen += 1
                        pool_dev = eng.upload(pool.reshape(-1))
                        eng.run_points(states, n, k, c.plan, pool_dev, plen)
                        eng.sync()
                        pool_dev.free()
                    elif isinstance(it, Conditional) and it.kind == "program":
                        u = cirq.unitary(it.inner)
                        eye = np.eye(u.shape[0], dtype=np.complex128)
                        hold = [conditions_hold(it.op, records[start + r], measured) for r in range(k)]
                        if any(hold):
                            run_slot(proj[j], np.array([u if h else eye for h in hold]), k, start)
                    elif isinstance(it, (Channel, Conditional)):
                        # a Kraus draw per trajectory; a classically controlled
                        # channel draws only where its conditions hold
                        hold = None
                        if isinstance(it, Conditional):
                            hold = np.array([conditions_hold(it.op, records[start + r], measured) for r in range(k)])
                            if not hold.any():
                                continue
                            it = Channel(it.inner, it.slot)
                        ks = runner._kraus[it.slot]
                        rho = runner.channel_rdm(states, n, k, it.op)  # (k, d, d)
                        kk = np.array([K.conj().T @ K for K in ks])  # (nK, d, d)
                        w = np.clip(np.real(np.einsum("kij,pji->pk", kk, rho)), 0.0, None)  # (k, nK)
                        u = prng.random_sample(k)
                        cum = np.cumsum(w, axis=1)
                        idx = (cum <= u[:, None]).sum(axis=1)
                        bad = (idx >= len(ks))
                        idx = np.where(bad, np.argmax(w, axis=1), idx)
                        bad |= w[np.arange(k), idx] <= 0
                        idx = np.where(bad, np.argmax(w, axis=1), idx)
                        wsel = w[np.arange(k), idx]
                        mats_k = np.array([ks[a] / np.sqrt(b) for a, b in zip(idx, wsel)])
                        if hold is not None:
                            mats_k[~hold] = np.eye(mats_k.shape[1])
                        run_slot(runner.kraus_seg[it.slot], mats_k, k, start)
                        if it.key is not None:
                            measured.setdefault(it.key, []).append(None)
                            for r in range(k):
                                records[start + r].setdefault(it.key, []).append([int(idx[r])])
                    else:  # mid-circuit measurement
                        op = it.op
                        qm = list(op.qubits)
                        m = len(qm)
                        drawn = eng.points_sample(states, n, k, prng.random_sample(k)).astype(np.int64)
                        outcome = np.zeros(k, dtype=np.int64)  # bit j <-> qm[j]
                        for jq, q in enumerate(qm):
                            outcome |= ((drawn >> (runner.n - 1 - runner.index[q])) & 1) << jq
                        recs_z, masks = _z_subset_records(runner, qm)
                        zv = np.real(eng.points_expect(states, n, k, Engine.pauli_records(recs_z)))  # (k, 2^m - 1)
                        par = np.array([[bin(o & S).count("1") & 1 for S in masks] for o in range(1 << m)])
                        sign = 1.0 - 2.0 * par  # (2^m, 2^m - 1)
                        prob = (1.0 + np.einsum("pt,pt->p", zv, sign[outcome])) / (1 << m)
                        prob = np.maximum(prob, 1e-30)
                        # projector / sqrt(p) in the op's matrix order (qubit 0 most significant)
                        d = 1 << m
                        mats_k = np.zeros((k, d, d), dtype=np.complex128)
                        for r in range(k):
                            row = 0
                            for jq in range(m):
                                row |= ((int(outcome[r]) >> jq) & 1) << (m - 1 - jq)
                            mats_k[r, row, row] = 1.0 / np.sqrt(prob[r])
                        run_slot(proj[j], mats_k, k, start)
                        key = cirq.measurement_key_name(op)
                        measured.setdefault(key, []).append(record_qids(op))
                        raw = ((outcome[:, None] >> np.arange(m)[None, :]) & 1).astype(np.int8)
                        rec = _recorded_in_place(raw, op, prng)
                        for r in range(k):
                            records[start + r].setdefault(key, []).append([int(b) for b in rec[r]])
                if terminal:
                    samples[start : start + k] = eng.points_sample(states, n, k, prng.random_sample(k))
        finally:
            states.free()
        out = pad_records(records) if any(records) else {}
        if terminal:
            term = sim._records_from_samples(samples, runner.empty, terminal)
            for key, v in term.items():
                v8 = v.astype(np.uint8)
                # a key measured mid-circuit and again at the end: more instances
                out[key] = np.concatenate([out[key], v8], axis=1) if key in out else v8
        return out
    finally:
        runner.close()


def _dm_projector_program(sim, op_qubits, qubits):
    """A one-slot program on the 2n-bit vector of a density matrix whose
    matrix each trajectory supplies: it acts on the row bits and the column
    bits of `op_qubits` (virtual qubit p <-> row bit of qubit p, virtual
    qubit n + p <-> its column bit, so that position p owns index bit
    2n-1-p).  Cached per simulator like slot_program."""
    cache = sim.__dict__.setdefault("_slot_programs", {})
    key = ("dm", tuple(op_qubits), tuple(qubits))
    c = cache.get(key)
    if c is None:
        if len(cache) >= _MAX_SLOT_PROGRAMS:
            cache.clear()
        from cirq_gb300.planner import Planner
        from cirq_gb300.program import CompiledCircuit

        n = len(qubits)
        vq = [cirq.NamedQubit(f"__dm_index_{i:04d}") for i in range(2 * n)]
        pos = {q: i for i, q in enumerate(qubits)}
        targets = [vq[pos[q]] for q in op_qubits] + [vq[n + pos[q]] for q in op_qubits]
        op = cirq.IdentityGate(len(targets)).on(*targets)
        c = CompiledCircuit([Slot(op, 0)], vq, dm=False, planner=Planner(tile_bits=12, kmax=4, budget=25.0),
                            resolvers=[cirq.ParamResolver({})])
        cache[key] = c
    return c


def run_batched_dm(sim, ops, qubits, resolver, reps: int):
    """run() of a density-matrix circuit with mid-circuit measurements, all
    repetitions at once: the repetitions' density matrices lie back to back as
    batched points, each segment of channels and unitaries is one launch per
    pass over all of them (gbq_run_points, the same matrices for every
    point), and each mid-circuit measurement reads every point's outcome
    distribution from the diagonal (gbq_points_dm_marginal), draws an outcome
    per repetition on the host and applies P rho P / p as a one-slot pass with
    per-repetition projectors -- the procedure of the reference's
    measure_density_matrix (cirq-core/cirq/sim/density_matrix_utils.py:97-183)
    in each trajectory of SimulatorBase._run
    (cirq-core/cirq/sim/simulator_base.py:248-264).  Returns run() records, or
    None when the circuit needs the one-at-a-time runner (classical control,
    loops, a mid-circuit measurement of more than 2 qubits, tensor-core
    plans)."""
    from cirq_gb300.simulator import _recorded_in_place

    if reps < 1 or getattr(sim.planner, "tensor", False):
        return None
    ops = records_relevant(ops)
    items, _ = build_items(ops, dm=True)
    last_unitary = max((i for i, it in enumerate(items) if not isinstance(it, Measure)), default=-1)
    body = items[: last_unitary + 1]
    terminal = [it.op for it in items[last_unitary + 1 :]]
    for it in body:
        if not isinstance(it, (Segment, Measure)):
            return None
        if isinstance(it, Measure) and (len(it.op.qubits) > 2 or any(q.dimension != 2 for q in it.op.qubits)):
            return None
    if not any(isinstance(it, Measure) for it in body):
        return None  # nothing mid-circuit: the caller samples one final state
    runner = TrajectoryRunner(sim, ops, qubits, resolver)
    eng = sim.engine
    prng = sim._prng
    try:
        n = runner.n
        nb = runner.empty.nbits_dev  # bits of one density-matrix slot (2n, padded to >= 10)
        _, free, _ = eng.device_info()
        budget = max(1 << 28, min(int(free) // 2, 32 << 30))
        chunk = max(1, min(reps, 65535, budget // (8 << nb), (1 << 24) >> max(nb - 10, 0)))
        proj = {i: _dm_projector_program(sim, it.op.qubits, runner.qubits)
                for i, it in enumerate(body) if isinstance(it, Measure)}
        states = eng.alloc((8 << nb) * chunk)
        records: list = [dict() for _ in range(reps)]
        samples = np.zeros(reps, dtype=np.int64)
        term_qubits = []
        for op in terminal:
            for q in op.qubits:
                if q not in term_qubits:
                    term_qubits.append(q)
        try:
            for start in range(0, reps, chunk):
                k = min(chunk, reps - start)
                eng.points_set_zero(states, nb, k)
                for j, it in enumerate(body):
                    if isinstance(it, Segment):
                        c = runner.compiled[j]
                        if not c.plan.npasses:
                            continue
                        pool_dev = eng.upload(np.ascontiguousarray(c.plan.pool, dtype=np.complex64))
                        eng.run_points(states, nb, k, c.plan, pool_dev, 0)  # one pool for every point
                        eng.sync()
                        pool_dev.free()
                        continue
                    op = it.op
                    qm = list(op.qubits)
                    m = len(qm)
                    bits = [n - 1 - runner.index[q] for q in qm]  # outcome bit j <-> qm[j]
                    probs = np.clip(eng.points_dm_marginal(states, nb, n, k, bits), 0.0, None)
                    cum = np.cumsum(probs, axis=1)
                    u = prng.random_sample(k) * cum[:, -1]
                    outcome = np.minimum((u[:, None] >= cum).sum(axis=1), (1 << m) - 1)
                    p = np.maximum(probs[np.arange(k), outcome], 1e-30)
                    d = 1 << m
                    mats = np.zeros((k, d * d, d * d), dtype=np.complex128)
                    for r in range(k):
                        be = 0  # the outcome with qm[0] most significant, as the slot's matrix order
                        for jq in range(m):
                            be |= ((int(outcome[r]) >> jq) & 1) << (m - 1 - jq)
                        mats[r, be * d + be, be * d + be] = 1.0 / p[r]
                    c = proj[j]
                    pool = np.ascontiguousarray(c.pool_from_batch({0: mats}, k), dtype=np.complex64)
                    plen = pool.shape[1]
                    if plen & 1:
                        pool = np.concatenate([pool, np.zeros((k, 1), np.complex64)], axis=1)
                        plen += 1
                    pool_dev = eng.upload(pool.reshape(-1))
                    eng.run_points(states, nb, k, c.plan, pool_dev, plen)
                    eng.sync()
                    pool_dev.free()
                    key = cirq.measurement_key_name(op)
                    raw = ((outcome[:, None] >> np.arange(m)[None, :]) & 1).astype(np.int8)
                    rec = _recorded_in_place(raw, op, prng)
                    for r in range(k):
                        records[start + r].setdefault(key, []).append([int(b) for b in rec[r]])
                if term_qubits:
                    if len(term_qubits) <= 5:
                        tb = [n - 1 - runner.index[q] for q in term_qubits]
                        probs = np.clip(eng.points_dm_marginal(states, nb, n, k, tb), 0.0, None)
                        cum = np.cumsum(probs, axis=1)
                        u = prng.random_sample(k) * cum[:, -1]
                        o = np.minimum((u[:, None] >= cum).sum(axis=1), (1 << len(tb)) - 1)
                        idx = np.zeros(k, dtype=np.int64)
                        for jq, b in enumerate(tb):
                            idx |= ((o >> jq) & 1) << b
                        samples[start : start + k] = idx
                    else:
                        for r in range(k):
                            samples[start + r] = int(eng.sample_point(states, nb, r, n, prng.random_sample(1),
                                                                      dm=True)[0])
        finally:
            states.free()
        out = pad_records(records) if any(records) else {}
        if terminal:
            term = sim._records_from_samples(samples, runner.empty, terminal)
            for key, v in term.items():
                v8 = v.astype(np.uint8)
                out[key] = np.concatenate([out[key], v8], axis=1) if key in out else v8
        return out
    finally:
        runner.close()
