"""Qudits (qids of dimension d > 2) on the qubit engine.

The reference simulates any qid shape natively: its state tensor has one
axis of length d per qid (``cirq-core/cirq/sim/state_vector_simulation_state.py``,
``cirq-core/cirq/linalg/transformations.py:105-172`` with qid shapes) and its
measurement records hold levels 0..d-1
(``cirq-core/cirq/sim/simulation_state.py:70-128``,
``cirq-core/cirq/sim/simulator.py:780-844``).

Here a qid of dimension d > 2 occupies b = ceil(log2 d) index bits of the
device state (:class:`QuditBit`), level v stored as the b-bit binary of v,
most significant bit first in the qubit order; qubits keep their own bit.
Indices with a level >= d are never populated: every operation on a qudit is
embedded as the original on the valid levels and the identity on the others
(a unitary or each unitary of a mixture), or, for Kraus operators, zero there
except the first operator, which carries the identity so the embedded channel
stays trace preserving.  Operations on qubits only pass through unchanged, so
their parameters still sweep on the batched paths.

A measurement of qudits becomes a :class:`QuditMeasurementGate` on their
bits: the simulators turn its bits into levels where they record it and then
apply the original gate's confusion map (mixed radix over the measured qids'
dimensions) and invert mask (``v ^ (v < 2)``) in the order of the path that
records it, and keep the qids as the measured qubits, so conditions on qudit
keys resolve as in the reference.  States are gathered back at the valid
indices in the reference's mixed-radix big-endian order.
"""

from __future__ import annotations

import copy
import functools
from typing import Any, Iterator, Sequence

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.ir import MAX_OP_QUBITS

cirq = ensure_cirq()


def has_qudits(qids) -> bool:
    return any(q.dimension != 2 for q in qids)


def bits_for(d: int) -> int:
    """Index bits of a qid of dimension d."""
    if d < 2:
        raise NotImplementedError(f"qids of dimension {d} are not supported")
    return (d - 1).bit_length()


class QuditBit(cirq.Qid):
    """Index bit `j` (0 = most significant) of the embedded qudit `qid`."""

    def __init__(self, qid: cirq.Qid, j: int):
        self._qid = qid
        self._j = j

    @property
    def qid(self) -> cirq.Qid:
        return self._qid

    @property
    def j(self) -> int:
        return self._j

    @property
    def dimension(self) -> int:
        return 2

    def _comparison_key(self):
        return (self._qid, self._j)

    def __repr__(self) -> str:
        return f"cirq_gb300.qudits.QuditBit({self._qid!r}, {self._j})"

    def __str__(self) -> str:
        return f"{self._qid}.b{self._j}"


def index_map(dims: Sequence[int], widths: Sequence[int]) -> np.ndarray:
    """Embedded index of every mixed-radix (big-endian) index over `dims`:
    the concatenated `widths`-bit binaries of the digits."""
    idx = np.zeros(1, dtype=np.int64)
    for d, w in zip(dims, widths):
        idx = ((idx << w)[:, None] | np.arange(d, dtype=np.int64)[None, :]).reshape(-1)
    return idx


class QuditMeasurementGate(cirq.MeasurementGate):
    """Measurement of the bits of embedded qids; the record holds their
    levels, with `original`'s invert mask and confusion map."""

    def __init__(self, original: cirq.MeasurementGate, qids: Sequence[cirq.Qid]):
        self.original = original
        self.qids = tuple(qids)
        self.widths = tuple(bits_for(q.dimension) if q.dimension != 2 else 1 for q in self.qids)
        super().__init__(num_qubits=sum(self.widths), key=original.mkey)

    def levels(self, bits: np.ndarray) -> np.ndarray:
        """(repetitions, bits) -> (repetitions, qids) levels."""
        out = np.zeros((bits.shape[0], len(self.qids)), dtype=np.int8)
        off = 0
        for j, w in enumerate(self.widths):
            v = np.zeros(bits.shape[0], dtype=np.int64)
            for t in range(w):
                v = (v << 1) | bits[:, off + t]
            out[:, j] = v
            off += w
        return out

    def _value_equality_values_(self):
        return (super()._value_equality_values_(), self.original, self.qids)

    def __repr__(self) -> str:
        return f"cirq_gb300.qudits.QuditMeasurementGate({self.original!r}, {self.qids!r})"


def recorded_view(op, bits: np.ndarray):
    """(record, gate, qids) of a measurement's sampled bits: levels and the
    original gate for a qudit measurement, else the bits and the gate."""
    gate = op.gate
    if isinstance(gate, QuditMeasurementGate):
        return gate.levels(bits), gate.original, gate.qids
    return bits, gate, op.qubits


def record_qids(op) -> tuple:
    """The qids a measurement's record refers to."""
    gate = getattr(op, "gate", None)
    return gate.qids if isinstance(gate, QuditMeasurementGate) else tuple(op.qubits)


def _key_of(op):
    keys = cirq.measurement_key_objs(op)
    return next(iter(keys)) if len(keys) == 1 else None


class Embedding:
    """The qubit form of a problem over `qids` (its qubit order)."""

    def __init__(self, qids: Sequence[cirq.Qid]):
        self.qids = tuple(qids)
        self.dims = tuple(q.dimension for q in self.qids)
        self._bits = {}
        for q in self.qids:
            self._bits[q] = (q,) if q.dimension == 2 else tuple(QuditBit(q, j) for j in range(bits_for(q.dimension)))
        self.qubits = tuple(b for q in self.qids for b in self._bits[q])
        self.size = int(np.prod(self.dims, dtype=np.int64)) if self.qids else 1

    def bits(self, qids) -> tuple:
        out = []
        for q in qids:
            if q not in self._bits:
                raise ValueError(f"qubit {q} is not simulated")
            out.extend(self._bits[q])
        return tuple(out)

    @functools.cached_property
    def index(self) -> np.ndarray:
        """Embedded index of every index of the reference's state."""
        return index_map(self.dims, [len(self._bits[q]) for q in self.qids])

    # ---- operations ------------------------------------------------------
    def _embed(self, m: np.ndarray, qids, rest_identity: bool) -> np.ndarray:
        idx = index_map([q.dimension for q in qids], [len(self._bits[q]) for q in qids])
        size = 1 << sum(len(self._bits[q]) for q in qids)
        out = np.eye(size, dtype=np.complex128) if rest_identity else np.zeros((size, size), np.complex128)
        out[np.ix_(idx, idx)] = m
        return out

    def _rest(self, qids) -> np.ndarray:
        idx = index_map([q.dimension for q in qids], [len(self._bits[q]) for q in qids])
        size = 1 << sum(len(self._bits[q]) for q in qids)
        p = np.eye(size, dtype=np.complex128)
        p[idx, idx] = 0
        return p

    def op(self, op) -> list:
        """The embedded operations of one operation."""
        if not has_qudits(op.qubits):
            return [op]
        untagged = op.untagged
        if isinstance(untagged, cirq.ClassicallyControlledOperation):
            conds = untagged.classical_controls
            return [e.with_classical_controls(*conds) for e in self.op(untagged.without_classical_controls())]
        if isinstance(untagged, cirq.CircuitOperation):
            if untagged.repeat_until is not None:
                raise NotImplementedError(f"repeat-until loops over qudits are not supported: {op!r}")
            return [e for sub in untagged.mapped_circuit(deep=False).all_operations() for e in self.op(sub)]
        gate = getattr(op, "gate", None)
        bits = self.bits(op.qubits)
        if isinstance(gate, cirq.MeasurementGate):
            return [QuditMeasurementGate(gate, op.qubits).on(*bits)]
        if cirq.is_parameterized(op):
            raise ValueError("internal: a parameterized qudit operation reached the embedding unresolved")
        if len(bits) > MAX_OP_QUBITS:
            sub = cirq.decompose_once(op, default=None)
            if sub is not None:
                return [e for s in sub for e in self.op(s)]
            raise NotImplementedError(
                f"{op!r} spans {len(bits)} index bits (more than {MAX_OP_QUBITS}) and has no decomposition"
            )
        u = cirq.unitary(op, default=None)
        if u is not None:
            return [cirq.MatrixGate(self._embed(u, op.qubits, True), unitary_check=False).on(*bits)]
        key = _key_of(op)
        mix = cirq.mixture(op, default=None)
        if mix is not None:
            emb = [(p, self._embed(m, op.qubits, True)) for p, m in mix]
            return [cirq.MixedUnitaryChannel(emb, key=key).on(*bits)]
        kraus = cirq.kraus(op, default=None)
        if kraus is not None:
            emb = [self._embed(k, op.qubits, False) for k in kraus]
            emb[0] = emb[0] + self._rest(op.qubits)
            return [cirq.KrausChannel(emb, key=key).on(*bits)]
        sub = cirq.decompose_once(op, default=None)
        if sub is not None:
            return [e for s in sub for e in self.op(s)]
        raise TypeError(f"cannot simulate {op!r}: it has no unitary, mixture, Kraus operators or decomposition")

    def circuit(self, program) -> cirq.Circuit:
        """The embedded circuit, moment for moment (an operation that
        expands to several is kept in its moment as a CircuitOperation)."""
        moments = []
        for moment in program:
            ops = []
            for op in moment:
                emb = self.op(op)
                if len(emb) == 1:
                    ops.append(emb[0])
                elif emb:
                    ops.append(cirq.CircuitOperation(cirq.FrozenCircuit(emb)))
            moments.append(cirq.Moment(ops))
        return cirq.Circuit(moments)

    # ---- states ----------------------------------------------------------
    def initial_state(self, initial_state: Any, dm: bool):
        """The embedded form of a reference initial state (an index of the
        reference's state, a state vector / tensor, or a density matrix)."""
        if initial_state is None:
            initial_state = 0
        if isinstance(initial_state, (int, np.integer)):
            i = int(initial_state)
            if not 0 <= i < self.size:
                raise ValueError(f"initial_state {i} out of range for qid shape {self.dims}")
            e = 0
            for q, digit in zip(self.qids, cirq.big_endian_int_to_digits(i, base=self.dims)):
                e = (e << len(self._bits[q])) | digit
            return e
        n = 1 << len(self.qubits)
        if isinstance(initial_state, np.ndarray) and initial_state.dtype != np.complex64:
            initial_state = initial_state.astype(np.complex64)
        if dm:
            rho = cirq.to_valid_density_matrix(initial_state, len(self.qids), qid_shape=self.dims, dtype=np.complex64)
            out = np.zeros((n, n), dtype=np.complex64)
            out[np.ix_(self.index, self.index)] = rho
            return out
        vec = cirq.to_valid_state_vector(initial_state, len(self.qids), qid_shape=self.dims, dtype=np.complex64)
        out = np.zeros(n, dtype=np.complex64)
        out[self.index] = vec
        return out

    def state_vector(self, vec: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(vec).reshape(-1)[self.index])

    def density_matrix(self, rho: np.ndarray) -> np.ndarray:
        n = 1 << len(self.qubits)
        return np.ascontiguousarray(np.asarray(rho).reshape(n, n)[np.ix_(self.index, self.index)])

    def levels(self, bits: np.ndarray, qids) -> np.ndarray:
        """(repetitions, bits of `qids`) -> (repetitions, qids) levels."""
        out = np.zeros((bits.shape[0], len(qids)), dtype=np.uint8)
        off = 0
        for j, q in enumerate(qids):
            w = len(self._bits[q])
            v = np.zeros(bits.shape[0], dtype=np.int64)
            for t in range(w):
                v = (v << 1) | bits[:, off + t].astype(np.int64)
            out[:, j] = v
            off += w
        return out


# ---- simulator entry points ------------------------------------------------
def _inner(sim):
    """`sim` for an embedded program: noise already placed, no product-state
    splitting (its components would be over index bits)."""
    inner = copy.copy(sim)
    inner.noise = cirq.NO_NOISE
    inner._split_untangled_states = False
    return inner


def _qudit_ops_parameterized(program) -> bool:
    return any(has_qudits(op.qubits) and cirq.is_parameterized(op) for op in program.all_operations())


def _sweeps(program, params, emb: Embedding) -> Iterator[tuple[list, cirq.Circuit]]:
    """(resolvers, embedded circuit) chunks: one for the whole sweep, or one
    per resolver when a qudit operation has parameters."""
    from cirq_gb300.simulator import _check_all_resolved

    resolvers = list(cirq.to_resolvers(params))
    if not _qudit_ops_parameterized(program):
        yield resolvers, emb.circuit(program)
        return
    for r in resolvers:
        _check_all_resolved(program, r)
        yield [r], emb.circuit(cirq.resolve_parameters(program, r))


def _order(program, qubit_order) -> tuple:
    return tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(program.all_qubits()))


def run(sim, circuit, param_resolver, repetitions: int) -> dict:
    """SimulatesSamples._run of a circuit with qudits."""
    emb = Embedding(sorted(circuit.all_qubits()))
    (resolvers, embedded), = _sweeps(circuit, [param_resolver], emb)
    return _inner(sim)._run(embedded, resolvers[0], repetitions)


def simulate_sweep(sim, program, params, qubit_order, initial_state) -> Iterator[Any]:
    from cirq_gb300.simulator import _density_matrix_result, _state_vector_result

    emb = Embedding(_order(program, qubit_order))
    inner = _inner(sim)
    order = cirq.QubitOrder.explicit(emb.qubits)
    init = emb.initial_state(initial_state, sim._dm)
    for resolvers, embedded in _sweeps(program, params, emb):
        for res in inner.simulate_sweep_iter(embedded, resolvers, order, init):
            if sim._dm:
                rho = emb.density_matrix(res.final_density_matrix)
                yield _density_matrix_result(res.params, res.measurements, emb.qids, rho)
            else:
                vec = emb.state_vector(res.final_state_vector)
                yield _state_vector_result(res.params, res.measurements, emb.qids, vec)


def expectation_values(sim, program, pslist, params, qubit_order, initial_state) -> Iterator[list]:
    emb = Embedding(_order(program, qubit_order))
    inner = _inner(sim)
    order = cirq.QubitOrder.explicit(emb.qubits)
    init = emb.initial_state(initial_state, sim._dm)
    for resolvers, embedded in _sweeps(program, params, emb):
        yield from inner.simulate_expectation_values_sweep_iter(
            embedded, pslist, resolvers, order, init, permit_terminal_measurements=True
        )


class _QuditStep(cirq.StepResult):
    def __init__(self, step, emb: Embedding):
        self._step = step
        self._emb = emb
        self._measurements = step.measurements

    def sample(self, qubits, repetitions: int = 1, seed: Any = None) -> np.ndarray:
        bits = self._step.sample(self._emb.bits(qubits), repetitions, seed)
        return self._emb.levels(np.asarray(bits), qubits)


class QuditStateVectorStep(cirq.StateVectorMixin, _QuditStep):
    """A state-vector step result over qids of any dimension."""

    def __init__(self, step, emb: Embedding):
        super().__init__({q: i for i, q in enumerate(emb.qids)}, step, emb)

    def state_vector(self, copy: bool = False) -> np.ndarray:
        return self._emb.state_vector(self._step.state_vector())

    def _simulator_state(self):
        return cirq.StateVectorSimulationState(
            qubits=self._emb.qids, initial_state=self.state_vector().reshape(self._emb.dims), dtype=np.complex64
        )


class QuditDensityMatrixStep(_QuditStep):
    """A density-matrix step result over qids of any dimension."""

    def _qid_shape_(self):
        return self._emb.dims

    def density_matrix(self, copy: bool = True) -> np.ndarray:
        return self._emb.density_matrix(self._step.density_matrix(copy=False))

    def _simulator_state(self):
        return cirq.DensityMatrixSimulationState(
            qubits=self._emb.qids, initial_state=self.density_matrix(), dtype=np.complex64
        )


def moment_steps(sim, circuit, param_resolver, qubit_order, initial_state) -> Iterator[Any]:
    """simulate_moment_steps of a circuit with qudits: the noise model's
    moments over the qids, embedded moment for moment."""
    from cirq_gb300.steps import moment_steps as qubit_steps

    resolver = cirq.ParamResolver(param_resolver)
    resolved = cirq.resolve_parameters(circuit, resolver)
    unresolved = cirq.parameter_symbols(resolved)
    if unresolved:
        raise ValueError(f"Circuit contains unresolved parameters: {sorted(map(str, unresolved))}")
    emb = Embedding(_order(circuit, qubit_order))
    noisy = cirq.Circuit(sim.noise.noisy_moments(resolved, sorted(resolved.all_qubits())))
    init = emb.initial_state(initial_state, sim._dm)
    step_cls = QuditDensityMatrixStep if sim._dm else QuditStateVectorStep
    for step in qubit_steps(_inner(sim), emb.circuit(noisy), resolver, cirq.QubitOrder.explicit(emb.qubits), init):
        yield step_cls(step, emb)
