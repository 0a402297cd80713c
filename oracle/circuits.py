"""Circuit-level oracle: walks a ``cirq.Circuit`` op by op at complex128.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates the moment loop of ``SimulatorBase._core_iterator``
(``cirq-core/cirq/sim/simulator_base.py:169-214``): every operation is
applied in circuit order to one dense tensor (the reference's
``split_untangled_states`` product-state factoring changes nothing numerically
and is not restated).  Matrices come from the reference's own protocols
(``cirq.unitary`` / ``cirq.kraus``), so this module needs ``cirq`` importable.
"""

from __future__ import annotations

from typing import Any, Sequence

import numpy as np

from oracle.statevector import (
    apply_kraus_dm,
    apply_matrix,
    apply_unitary_dm,
    pauli_expectation,
)


def _cirq():
    import cirq

    return cirq


def _ordered_qubits(circuit, qubit_order):
    cirq = _cirq()
    return list(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(circuit.all_qubits()))


def _ops(circuit, param_resolver):
    cirq = _cirq()
    resolved = cirq.resolve_parameters(circuit, param_resolver or cirq.ParamResolver({}))
    for moment in resolved:
        for op in moment:
            yield op


def simulate_state_vector(
    circuit,
    param_resolver=None,
    qubit_order=None,
    initial_state: int | np.ndarray = 0,
) -> np.ndarray:
    """Final state vector (complex128, flattened big-endian) of a unitary
    circuit over qids of any dimension (mixed radix, as the reference).

    Measurements are skipped (they are terminal in every caller); any other
    non-unitary operation raises ``TypeError`` as the reference does for ops
    it cannot act on (``simulator_base.py:211-212``).
    """
    cirq = _cirq()
    qubit_order = cirq.QubitOrder.DEFAULT if qubit_order is None else qubit_order
    qubits = _ordered_qubits(circuit, qubit_order)
    n = len(qubits)
    dims = tuple(q.dimension for q in qubits)
    size = int(np.prod(dims, dtype=np.int64))
    index = {q: i for i, q in enumerate(qubits)}
    if isinstance(initial_state, (int, np.integer)):
        psi = np.zeros(size, dtype=np.complex128)
        psi[int(initial_state)] = 1
    else:
        psi = np.asarray(initial_state, dtype=np.complex128).reshape(-1).copy()
    t = psi.reshape(dims) if n else psi
    for op in _ops(circuit, param_resolver):
        if cirq.is_measurement(op):
            continue
        if not cirq.has_unitary(op):
            raise TypeError(f"oracle: operation without a unitary: {op!r}")
        u = cirq.unitary(op)
        t = apply_matrix(t, [index[q] for q in op.qubits], u)
    return np.asarray(t).reshape(-1)


def simulate_density_matrix(
    circuit,
    param_resolver=None,
    qubit_order=None,
    noise=None,
    initial_state: int = 0,
) -> np.ndarray:
    """Final density matrix (complex128, D x D for D the product of the qid
    dimensions) of a possibly noisy circuit.

    Unitary ops use ``apply_unitary_dm`` and channels ``apply_kraus_dm``,
    restating the strategy order of ``protocols.apply_channel``
    (``cirq-core/cirq/protocols/apply_channel_protocol.py:168-272``).  A
    ``noise`` model is expanded with the reference's own
    ``NoiseModel.noisy_moments`` (``cirq-core/cirq/devices/noise_model.py:118-131``).
    """
    cirq = _cirq()
    qubit_order = cirq.QubitOrder.DEFAULT if qubit_order is None else qubit_order
    qubits = _ordered_qubits(circuit, qubit_order)
    n = len(qubits)
    dims = tuple(q.dimension for q in qubits)
    size = int(np.prod(dims, dtype=np.int64))
    index = {q: i for i, q in enumerate(qubits)}
    rho = np.zeros((size, size), dtype=np.complex128)
    rho[initial_state, initial_state] = 1
    t = rho.reshape(dims + dims)
    resolved = cirq.resolve_parameters(circuit, param_resolver or cirq.ParamResolver({}))
    if noise is not None:
        model = cirq.NoiseModel.from_noise_model_like(noise)
        moments = model.noisy_moments(resolved, sorted(qubits))
        resolved = cirq.Circuit(cirq.flatten_to_ops_or_moments(moments))
    for moment in resolved:
        for op in moment:
            if cirq.is_measurement(op):
                continue
            axes = [index[q] for q in op.qubits]
            if cirq.has_unitary(op):
                t = apply_unitary_dm(t, n, axes, cirq.unitary(op))
            else:
                t = apply_kraus_dm(t, n, axes, cirq.kraus(op))
    return np.asarray(t).reshape(size, size)


def pauli_sum_terms(observable, qubit_index) -> list[tuple[complex, dict[int, str]]]:
    """Splits a PauliSum-like into (coefficient, {axis: 'X'|'Y'|'Z'}) terms."""
    cirq = _cirq()
    out = []
    for ps in cirq.PauliSum.wrap(observable):
        paulis = {}
        for q, p in ps.items():
            paulis[qubit_index[q]] = {cirq.X: "X", cirq.Y: "Y", cirq.Z: "Z"}[p]
        out.append((complex(ps.coefficient), paulis))
    return out


def expectation_state_vector(psi: np.ndarray, observable, qubit_index) -> complex:
    """Sum of coefficient * <psi|P|psi> (``cirq-core/cirq/ops/linear_combinations.py:716-718``)."""
    n = int(np.log2(psi.size))
    return sum(pauli_expectation(psi, n, p, c) for c, p in pauli_sum_terms(observable, qubit_index))


def expectation_density_matrix(rho: np.ndarray, observable, qubit_index) -> complex:
    """Sum of coefficient * Tr(P rho)."""
    n = int(np.log2(rho.shape[0]))
    total = 0j
    t = rho.reshape((2,) * (2 * n))
    from oracle.statevector import _PAULI

    for c, paulis in pauli_sum_terms(observable, qubit_index):
        m = t
        for axis, p in paulis.items():
            m = apply_matrix(m, [axis], _PAULI[p])
        total += c * np.trace(np.asarray(m).reshape(2**n, 2**n))
    return total


def expectation_of_circuit(circuit, observable, resolver, qubit_order=None) -> complex:
    cirq = _cirq()
    qubit_order = cirq.QubitOrder.DEFAULT if qubit_order is None else qubit_order
    qubits = _ordered_qubits(circuit, qubit_order)
    psi = simulate_state_vector(circuit, resolver, qubit_order)
    return expectation_state_vector(psi, observable, {q: i for i, q in enumerate(qubits)})


def finite_difference_gradient(
    circuit, observable, symbols: Sequence[Any], values: Sequence[float], h: float = 1e-3, indices=None
) -> np.ndarray:
    """Central differences (E(theta+h e_i) - E(theta-h e_i)) / 2h at complex128,
    for the parameters in `indices` (all by default)."""
    idx = list(range(len(symbols))) if indices is None else list(indices)
    grad = np.zeros(len(idx))
    base = dict(zip(symbols, [float(v) for v in values]))
    for k, i in enumerate(idx):
        s = symbols[i]
        plus = dict(base)
        minus = dict(base)
        plus[s] = base[s] + h
        minus[s] = base[s] - h
        ep = expectation_of_circuit(circuit, observable, plus).real
        em = expectation_of_circuit(circuit, observable, minus).real
        grad[k] = (ep - em) / (2 * h)
    return grad
