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


def _cirq():
    return ensure_cirq()


def _is_measurement(op) -> bool:
    return _cirq().is_measurement(op)


class UnsupportedOperation(NotImplementedError):
    pass


def qubit_positions(qubits: Sequence[Any]) -> dict:
    return {q: i for i, q in enumerate(qubits)}


def flatten_ops(circuit) -> list:
    """All operations of a resolved circuit in moment order (CircuitOperations unrolled)."""
    cirq = _cirq()
    ops = []
    for moment in circuit:
        for op in moment:
            if isinstance(op.untagged, cirq.CircuitOperation):
                ops.extend(flatten_ops(op.untagged.mapped_circuit(deep=True)))
            else:
                ops.append(op)
    return ops


def unitary_gates(ops, index: dict, n: int, *, dm: bool = False) -> tuple[list[BitGate], complex]:
    """Unitary ops -> BitGates (state vector: n bits; dm=True: 2n bits).

    Returns (gates, global_phase).  Measurements must already be removed.
    """
    cirq = _cirq()
    gates: list[BitGate] = []
    phase = 1.0 + 0j
    for op in ops:
        if not op.qubits:
            if cirq.has_unitary(op):
                phase *= complex(cirq.unitary(op).reshape(-1)[0])
                continue
            raise UnsupportedOperation(f"operation without qubits and without a unitary: {op!r}")
        if any(q.dimension != 2 for q in op.qubits):
            raise UnsupportedOperation(f"only qubits are supported, got {op!r}")
        if not cirq.has_unitary(op):
            raise UnsupportedOperation(f"operation without a unitary: {op!r}")
        u = np.asarray(cirq.unitary(op), dtype=np.complex128)
        gates.extend(_unitary_to_bitgates(op, u, index, n, dm))
    return gates, phase


def _unitary_to_bitgates(op, u, index, n, dm):
    pos = [index[q] for q in op.qubits]
    k = len(pos)
    if np.allclose(u, np.eye(2**k), atol=0, rtol=0):
        return []
    diag = is_diagonal(u)
    if not dm:
        bits = tuple(n - 1 - p for p in reversed(pos))
        return [BitGate(bits, u, diag)]
    rows = tuple(2 * n - 1 - p for p in reversed(pos))
    cols = tuple(n - 1 - p for p in reversed(pos))
    return [BitGate(rows, u, diag), BitGate(cols, np.conjugate(u), diag)]


def channel_gates(ops, index: dict, n: int) -> list[BitGate]:
    """Any ops (unitaries or channels) -> BitGates on the 2n-bit density vector."""
    cirq = _cirq()
    gates: list[BitGate] = []
    for op in ops:
        if not op.qubits:
            if cirq.has_unitary(op):  # global phase cancels in rho
                continue
            raise UnsupportedOperation(f"operation without qubits: {op!r}")
        if any(q.dimension != 2 for q in op.qubits):
            raise UnsupportedOperation(f"only qubits are supported, got {op!r}")
        if cirq.has_unitary(op):
            u = np.asarray(cirq.unitary(op), dtype=np.complex128)
            gates.extend(_unitary_to_bitgates(op, u, index, n, True))
            continue
        if not cirq.has_kraus(op):
            raise UnsupportedOperation(f"operation without Kraus operators: {op!r}")
        kraus = [np.asarray(k, dtype=np.complex128) for k in cirq.kraus(op)]
        pos = [index[q] for q in op.qubits]
        k = len(pos)
        if 2 * k > 5:
            raise UnsupportedOperation(
                f"channels on more than 2 qubits are not supported on the GPU path: {op!r}"
            )
        s = sum(np.kron(np.conjugate(kk), kk) for kk in kraus)
        rows = tuple(2 * n - 1 - p for p in reversed(pos))
        cols = tuple(n - 1 - p for p in reversed(pos))
        gates.append(BitGate(rows + cols, s, is_diagonal(s)))
    return gates


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
