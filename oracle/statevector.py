"""Numpy restatement of the reference's state-vector / density-matrix numerics.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Layout conventions are the reference's: a state of ``n`` qubits is a tensor of
shape ``(2,)*n`` (flattened big-endian: axis 0 is the most significant index
bit), and a density matrix is a tensor of shape ``(2,)*2n`` whose first ``n``
axes are the row (ket) axes and last ``n`` the column (bra) axes
(``cirq-core/cirq/sim/density_matrix_simulation_state.py:178``).
"""

from __future__ import annotations

from typing import Mapping, Sequence

import numpy as np

_PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def apply_matrix(tensor: np.ndarray, axes: Sequence[int], matrix: np.ndarray) -> np.ndarray:
    """Left-multiplies ``matrix`` onto ``axes`` of ``tensor``; returns a new tensor.

    Restates ``targeted_left_multiply`` (``cirq-core/cirq/linalg/transformations.py:105-172``):
    the matrix over the target axes (dimension d_j each: 2 for qubits) is
    viewed as a (d_0..d_{k-1}, d_0..d_{k-1}) tensor whose first k axes are
    output axes and last k input axes, ``axes[0]`` being the most significant
    matrix-index digit; the contraction replaces each target axis by the
    corresponding output axis.
    """
    k = len(axes)
    d = tensor.ndim
    dims = tuple(tensor.shape[a] for a in axes)
    m = np.asarray(matrix).reshape(dims + dims)
    work = list(range(k))
    data = list(range(k, k + d))
    inp = work + [data[a] for a in axes]
    out = list(data)
    for w, a in zip(work, axes):
        out[a] = w
    return np.einsum(m, inp, tensor, data, out)


def apply_unitary_dm(rho: np.ndarray, n: int, axes: Sequence[int], u: np.ndarray) -> np.ndarray:
    """rho -> U rho U^dagger on a (2,)*2n density tensor.

    Restates ``apply_channel_protocol._apply_unitary``
    (``cirq-core/cirq/protocols/apply_channel_protocol.py:274-295``): apply U to
    the left axes, conjugate, apply U to the right axes, conjugate.
    """
    left = apply_matrix(rho, axes, u)
    right = apply_matrix(np.conjugate(left), [a + n for a in axes], u)
    return np.conjugate(right)


def apply_kraus_dm(
    rho: np.ndarray, n: int, axes: Sequence[int], kraus: Sequence[np.ndarray]
) -> np.ndarray:
    """rho -> sum_i K_i rho K_i^dagger.

    Restates ``_apply_kraus_multi_qubit``
    (``cirq-core/cirq/protocols/apply_channel_protocol.py:336-356``): each
    Kraus operator is applied to the left axes and its conjugate to the right
    axes, and the results are summed.
    """
    out = np.zeros_like(rho)
    for k in kraus:
        t = apply_matrix(rho, axes, k)
        out += apply_matrix(t, [a + n for a in axes], np.conjugate(k))
    return out


def apply_superop(rho: np.ndarray, n: int, axes: Sequence[int], superop: np.ndarray) -> np.ndarray:
    """Applies a superoperator given as sum_i conj(K_i) (x) K_i acting on
    (column axes, row axes): matrix index = col_index * 2^k + row_index.

    Used to check fused channel blocks; equivalent to ``apply_kraus_dm`` for
    ``superop = sum_i kron(conj(K_i), K_i)``.
    """
    k = len(axes)
    # Matrix index bit order (most significant first): col axes then row axes.
    all_axes = [a + n for a in axes] + list(axes)
    return apply_matrix(rho, all_axes, superop.reshape(4**k, 4**k))


def probabilities_by_indices(probs: np.ndarray, indices: Sequence[int], n: int) -> np.ndarray:
    """Marginal probabilities of the measured ``indices`` (big-endian order).

    Restates ``state_probabilities_by_indices``
    (``cirq-core/cirq/sim/simulation_utils.py:24-65``): transpose measured axes
    to the front, sum out the rest, clip at 0, renormalise.
    """
    p = np.asarray(probs, dtype=np.float64).reshape((2,) * n)
    rest = [i for i in range(n) if i not in indices]
    p = np.transpose(p, list(indices) + rest).reshape(-1)
    if rest:
        p = p.reshape((2 ** len(indices), -1)).sum(axis=-1)
    p = np.clip(p, 0, None)
    return p / p.sum()


def sample_from_probs(probs: np.ndarray, uniforms: np.ndarray) -> np.ndarray:
    """Inverse-CDF sampling: index i with cdf[i-1] <= u*total < cdf[i].

    The reference draws with ``RandomState.choice(len(p), size, p=p)``
    (``cirq-core/cirq/sim/state_vector.py:226``), which is inverse-CDF
    sampling on the cumulative sum; this restatement takes the uniforms
    explicitly so a device implementation can be compared draw by draw.
    """
    cdf = np.cumsum(np.asarray(probs, dtype=np.float64))
    target = np.asarray(uniforms, dtype=np.float64) * cdf[-1]
    idx = np.searchsorted(cdf, target, side="right")
    return np.minimum(idx, len(cdf) - 1)


def pauli_apply(state: np.ndarray, n: int, paulis: Mapping[int, str]) -> np.ndarray:
    """Returns P|psi> for a Pauli string given as {axis: 'X'|'Y'|'Z'}.

    Restates the per-qubit ``apply_unitary`` loop of
    ``PauliString._expectation_from_state_vector_no_validation``
    (``cirq-core/cirq/ops/pauli_string.py:625-655``).
    """
    ket = np.asarray(state).reshape((2,) * n)
    for axis, p in paulis.items():
        ket = apply_matrix(ket, [axis], _PAULI[p])
    return ket.reshape(-1)


def pauli_expectation(
    state: np.ndarray, n: int, paulis: Mapping[int, str], coefficient: complex = 1.0
) -> complex:
    """coefficient * <psi|P|psi> (``pauli_string.py:651-655``: tensordot of psi* and P psi)."""
    ket = pauli_apply(state, n, paulis)
    return coefficient * np.vdot(np.asarray(state).reshape(-1), ket)


def renormalize_like_cirq(vec: np.ndarray) -> np.ndarray:
    """Final-state renormalisation rule of ``StateVectorTrialResult.final_state_vector``
    (``cirq-core/cirq/sim/state_vector_simulator.py:131-146``): divide by the
    norm only when that reduces the round-off of the total probability, and
    not at all when the norm is further than sqrt(eps) from 1."""
    ret = vec.reshape(-1)
    norm = np.linalg.norm(ret)
    if abs(norm - 1) > np.sqrt(np.finfo(ret.dtype).eps):
        return ret
    ret_norm = ret / norm
    change = abs(np.vdot(ret_norm, ret_norm) - 1) - abs(np.vdot(ret, ret) - 1)
    return ret_norm if change < 0 else ret
