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
in one vectorised call per segment.  A general channel on k <= 2 qubits
reads the reduced density matrix of its qubits from the 4^k - 1 Pauli
expectations of the state (rho_Q = 2^-k sum_P <P> P), computes the weights
Tr(K_i^dagger K_i rho_Q) on the host, and applies the drawn operator as a
one-slot segment.  The density-matrix simulator needs trajectories only for
mid-circuit measurement (its channels are exact superoperators).
"""

from __future__ import annotations

import dataclasses
import math
from typing import Any

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.ir import UnsupportedOperation, flatten_ops
from cirq_gb300.program import Slot, TrajectoryPoint

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


def needs_trajectories(ops, dm: bool) -> bool:
    """True when a flattened op list cannot be simulated once and sampled."""
    seen_measure = False
    for op in ops:
        if cirq.is_measurement(op):
            seen_measure = True
            continue
        if seen_measure and op.qubits:
            return True  # an operation after a measurement
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
            if len(op.qubits) > 2:
                raise UnsupportedOperation(f"channels on more than 2 qubits are not supported: {op!r}")
            flush()
            items.append(Channel(op, nslot))
            nslot += 1
            continue
        raise UnsupportedOperation(f"operation {op!r} has neither a unitary, a mixture nor Kraus operators")
    flush()
    return items, nslot


def circuit_ops(sim, program, qubits, resolver):
    """The resolved, noise-inserted operations of a circuit (measurements
    included: noise after a mid-circuit measurement acts on later ops)."""
    resolved = cirq.resolve_parameters(program, resolver)
    if sim.noise is not cirq.NO_NOISE:
        moments = sim.noise.noisy_moments(resolved, sorted(qubits))
        resolved = cirq.Circuit(cirq.flatten_to_ops_or_moments(moments))
    return flatten_ops(resolved)


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
            sim._compile(it.ops, self.qubits, base) if isinstance(it, Segment) else None for it in self.items
        ]
        self.empty = sim._compile([], self.qubits, base)  # geometry of the state buffer
        self.kraus_seg = {}
        for it in self.items:
            if isinstance(it, Channel):
                self.kraus_seg[it.slot] = sim._compile([Slot(it.op, it.slot)], self.qubits, base)
        self._kraus = {it.slot: [np.asarray(k, dtype=np.complex128) for k in cirq.kraus(it.op)]
                       for it in self.items if isinstance(it, Channel)}
        self._pauli = {it.slot: self._pauli_basis(it.op) for it in self.items if isinstance(it, Channel)}
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
        for buf in self._pools.values():
            buf.free()
        self._pools.clear()
        if self._state is not None:
            self._state.free()
            self._state = None

    # ---- host-side draws ---------------------------------------------------
    def _draw_mixtures(self, reps: int) -> list[dict]:
        prng = self.sim._prng
        picks = [dict() for _ in range(reps)]
        for it in self.items:
            if not isinstance(it, Segment):
                continue
            for sid, op in it.slots:
                probs, unitaries = zip(*cirq.mixture(op))
                p = np.asarray(probs, dtype=np.float64)
                choice = prng.choice(len(unitaries), size=reps, p=p / p.sum())
                for r in range(reps):
                    picks[r][sid] = unitaries[choice[r]]
        return picks

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

    def apply(self, state, picks: dict, pools: list, rep: int) -> dict:
        """Applies the items to a device state in place; returns the records."""
        sim = self.sim
        eng = sim.engine
        records: dict = {}
        for j, it in enumerate(self.items):
            if isinstance(it, Segment):
                c = self.compiled[j]
                if c.plan.npasses:
                    pool = pools[j][rep] if pools[j] is not None else c.plan.pool
                    eng.run(state, c.nbits_dev, c.plan, self._pool_dev(("seg", j), pool))
            elif isinstance(it, Measure):
                bits = sim._measure_op(state, self.empty, it.op)
                records.setdefault(cirq.measurement_key_name(it.op), []).append(bits)
            else:
                self._apply_kraus(state, it, picks)
        return records

    def _apply_kraus(self, state, it: Channel, picks: dict) -> None:
        eng = self.sim.engine
        ks = self._kraus[it.slot]
        recs, mats = self._pauli[it.slot]
        vals = np.real(eng.expect_paulis(state, self.n, recs))
        k = len(it.op.qubits)
        rho = np.eye(2**k, dtype=np.complex128)
        for v, m in zip(vals, mats):
            rho = rho + v * m
        rho /= 2**k
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
        pool = c.pool([TrajectoryPoint(self.resolver, picks)])[0]
        eng.run(state, c.nbits_dev, c.plan, self._pool_dev(("kraus", it.slot), pool))

    def prepare(self, reps: int):
        """Draws the mixtures of `reps` trajectories; returns (picks, pools)."""
        picks = self._draw_mixtures(reps)
        pools = []
        for j, it in enumerate(self.items):
            c = self.compiled[j]
            if isinstance(it, Segment) and c.plan.npasses and it.slots:
                pools.append(c.pool([TrajectoryPoint(self.resolver, p) for p in picks]))
            elif isinstance(it, Segment) and c.plan.npasses:
                pools.append(None)
            else:
                pools.append(None)
        return picks, pools


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
