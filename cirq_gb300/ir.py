"""Translates resolved ``cirq.Circuit`` operations into index-bit gates.

A :class:`BitGate` acts on index bits of the simulated vector: ``bits[j]`` is
the index bit carried by matrix-index bit ``j`` (little-endian), so a Cirq
matrix on qubits ``(q_0 .. q_{k-1})`` -- ``q_0`` most significant, the
convention of ``cirq.unitary`` -- is used unchanged with
``bits = (bit(q_{k-1}), ..., bit(q_0))``.

State vectors: qubit at position ``p`` of the qubit order owns index bit
``n-1-p`` (big-endian, ``cirq-core/cirq/sim/state_vector.py:81-112``).

Density matrices: the 2n-bit vector index is ``row * 2^n + col``
(``cirq-core/cirq/sim/density_matrix_simulation_state.py:178``); qubit ``p``
owns row bit ``2n-1-p`` and column bit ``n-1-p``.  A unitary U becomes U on
the row bits and conj(U) on the column bits (the left/right application of
``apply_channel_protocol._apply_unitary``, :274-295); a channel with Kraus
operators K_i becomes the superoperator sum_i conj(K_i) (x) K_i on
(row bits, column bits) (``_apply_kraus``, :297-356).
"""

from __future__ import annotations

import dataclasses
from typing import Any, Sequence

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq


@dataclasses.dataclass
class BitGate:
    bits: tuple[int, ...]
    matrix: np.ndarray  # complex128, (2^k, 2^k)
    diagonal: bool
    # bookkeeping: index of the source gate in the translated list
    tag: Any = None
    # probe slot: >= 0 marks a gradient probe Re<lam|matrix|psi> (two-state
    # programs only); probes are never fused with other gates
    probe: int = -1

    @property
    def k(self) -> int:
        return len(self.bits)


def is_diagonal(m: np.ndarray) -> bool:
    off = m - np.diag(np.diagonal(m))
    return not np.any(off)


_CIRQ = None


def _cirq():
    global _CIRQ
    if _CIRQ is None:
        _CIRQ = ensure_cirq()
    return _CIRQ


_PLAIN_GATES = None


def _plain_gates():
    """Gate families that are a unitary (or a measurement) by construction:
    a plain GateOperation of one of them needs no flattening checks."""
    global _PLAIN_GATES
    if _PLAIN_GATES is None:
        cirq = _cirq()
        _PLAIN_GATES = (cirq.EigenGate, cirq.PhasedXZGate, cirq.MatrixGate, cirq.PhasedXPowGate)
    return _PLAIN_GATES


_CHANNEL_GATES = None


def _channel_gates():
    """The reference's channel gate families: each defines its own Kraus
    operators or mixture (cirq-core/cirq/ops/common_channels.py,
    kraus_channel.py, mixed_unitary_channel.py), so none needs the
    decomposition fallback, and answering that from the type avoids building
    their operators twice per simulation."""
    global _CHANNEL_GATES
    if _CHANNEL_GATES is None:
        cirq = _cirq()
        _CHANNEL_GATES = (
            cirq.DepolarizingChannel, cirq.AsymmetricDepolarizingChannel, cirq.AmplitudeDampingChannel,
            cirq.GeneralizedAmplitudeDampingChannel, cirq.PhaseDampingChannel, cirq.PhaseFlipChannel,
            cirq.BitFlipChannel, cirq.ResetChannel, cirq.KrausChannel, cirq.MixedUnitaryChannel,
        )
    return _CHANNEL_GATES


def _is_measurement(op) -> bool:
    return _cirq().is_measurement(op)


class UnsupportedOperation(NotImplementedError):
    pass


def qubit_positions(qubits: Sequence[Any]) -> dict:
    return {q: i for i, q in enumerate(qubits)}


MAX_OP_QUBITS = 5


def _wide_unitary(op) -> bool:
    cirq = _cirq()
    return (
        len(op.qubits) > MAX_OP_QUBITS
        and not cirq.is_measurement(op)
        and not isinstance(op.untagged, cirq.ClassicallyControlledOperation)
        and cirq.has_unitary(op)
    )


def flatten_ops(circuit) -> list:
    """All operations of a resolved circuit in moment order (CircuitOperations
    unrolled).  A unitary on more than 5 qubits (a multi-controlled gate, a
    wide MatrixGate with a decomposition) is replaced by the reference's own
    exact decomposition (``cirq.decompose``, which keeps global phases) into
    operations of at most 5 qubits; one without a decomposition is kept and
    rejected by the compiler."""
    cirq = _cirq()
    plain, gate_op, meas = _plain_gates(), cirq.GateOperation, cirq.MeasurementGate
    chans = _channel_gates()
    ops = []
    for moment in circuit:
        for op in moment:
            if type(op) is gate_op:
                gate = op.gate
                if isinstance(gate, meas) or (isinstance(gate, plain) and len(op.qubits) <= MAX_OP_QUBITS):
                    ops.append(op)
                    continue
                if isinstance(gate, chans) and len(op.qubits) <= MAX_OP_QUBITS:
                    ops.append(op)  # a channel with operators of its own
                    continue
            if is_loop(op):
                ops.append(op)  # repeats a data-dependent number of times: a trajectory event
            elif isinstance(op.untagged, cirq.CircuitOperation):
                # one level at a time, so loops nested inside stay whole
                ops.extend(flatten_ops(op.untagged.mapped_circuit(deep=False)))
            elif _decomposed_measurement(op):
                # e.g. PauliMeasurementGate: the reference acts on its
                # decomposition (basis change, parity, a plain measurement,
                # and back)
                sub = cirq.decompose_once(op, default=None)
                if sub is None:
                    ops.append(op)
                else:
                    ops.extend(flatten_ops(cirq.Circuit(sub)))
            elif _wide_unitary(op):
                ops.extend(
                    cirq.decompose(op, keep=lambda o: len(o.qubits) <= MAX_OP_QUBITS, on_stuck_raise=None)
                )
            elif _needs_decomposition(op):
                # no unitary, mixture or Kraus operators of its own: the
                # reference acts on its decomposition (act_on's fallback)
                sub = cirq.decompose_once(op, default=None)
                if sub is None:
                    ops.append(op)
                else:
                    ops.extend(flatten_ops(cirq.Circuit(sub)))
            else:
                ops.append(op)
    return ops


def is_measurement_op(op) -> bool:
    """cirq.is_measurement, answered without the protocol for the common
    gate families (unitary by construction) and for measurement gates.  A
    channel with a measurement key is a channel here (is_keyed_channel)."""
    cirq = _cirq()
    gate = getattr(op, "gate", None)
    if gate is not None:
        if isinstance(gate, cirq.MeasurementGate):
            return True
        if isinstance(gate, (cirq.EigenGate, cirq.PhasedXZGate, cirq.MatrixGate, cirq.PhasedXPowGate)):
            return False
        if isinstance(gate, _channel_gates()) and not isinstance(gate, (cirq.KrausChannel, cirq.MixedUnitaryChannel)):
            return False  # channels without a measurement key
    return cirq.is_measurement(op) and not is_keyed_channel(op)


def is_loop(op) -> bool:
    """A CircuitOperation with ``repeat_until``: its body runs until the
    condition holds on the measurement results
    (cirq-core/cirq/circuits/circuit_operation.py ``_act_on_``)."""
    cirq = _cirq()
    u = op.untagged
    return isinstance(u, cirq.CircuitOperation) and u.repeat_until is not None


def _decomposed_measurement(op) -> bool:
    """A measurement other than a MeasurementGate or a keyed channel."""
    cirq = _cirq()
    gate = getattr(op, "gate", None)
    if gate is not None and isinstance(gate, (cirq.MeasurementGate, cirq.EigenGate, cirq.PhasedXZGate,
                                               cirq.MatrixGate, cirq.PhasedXPowGate)):
        return False
    if isinstance(op.untagged, (cirq.ClassicallyControlledOperation, cirq.CircuitOperation)):
        return False
    return cirq.is_measurement(op) and not is_keyed_channel(op)


def is_keyed_channel(op) -> bool:
    """A mixture or Kraus channel with a measurement key: the state-vector
    simulator records the index of the operator that acted
    (cirq-core/cirq/sim/state_vector_simulation_state.py:183-257,
    ``record_channel_measurement``); the density-matrix simulator applies the
    channel and records nothing."""
    cirq = _cirq()
    if isinstance(getattr(op, "gate", None), cirq.MeasurementGate):
        return False
    if isinstance(op.untagged, (cirq.ClassicallyControlledOperation, cirq.CircuitOperation)):
        return False
    if not cirq.is_measurement(op):
        return False
    # operators of its own (has_kraus would also answer through a
    # decomposition, as for PauliMeasurementGate)
    return cirq.mixture(op, default=None) is not None or cirq.kraus(op, default=None) is not None


def _needs_decomposition(op) -> bool:
    cirq = _cirq()
    gate = getattr(op, "gate", None)
    if gate is not None and isinstance(gate, (cirq.EigenGate, cirq.PhasedXZGate, cirq.MatrixGate,
                                               cirq.MeasurementGate, cirq.PhasedXPowGate)):
        return False  # the common gate families: unitary (or a measurement) by construction
    if gate is not None and isinstance(gate, _channel_gates()):
        return False  # operators of their own
    if not op.qubits or cirq.is_parameterized(op) or cirq.is_measurement(op):
        return False
    if isinstance(op.untagged, cirq.ClassicallyControlledOperation):
        return False
    if cirq.has_unitary(op):
        return False
    # has_kraus / has_mixture may answer through a decomposition that
    # cirq.kraus / cirq.mixture do not follow: ask for the operators
    return cirq.mixture(op, default=None) is None and cirq.kraus(op, default=None) is None


def pauli_terms(observable, index: dict, n: int):
    """PauliSum-like -> (gbq_pauli records, coefficients are complex).

    Returns a list of (x_mask, zy_mask, n_y, coefficient) with masks over the
    n index bits of a state vector.
    """
    cirq = _cirq()
    out = []
    for ps in cirq.PauliSum.wrap(observable):
        x = zy = 0
        ny = 0
        for q, p in ps.items():
            b = 1 << (n - 1 - index[q])
            if p == cirq.X:
                x |= b
            elif p == cirq.Y:
                x |= b
                zy |= b
                ny += 1
            elif p == cirq.Z:
                zy |= b
        out.append((x, zy, ny, complex(ps.coefficient)))
    return out
