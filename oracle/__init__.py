"""CPU oracle for the Cirq simulation hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy at complex128, the numeric algorithm
that quantumlib/Cirq's ``cirq.Simulator`` and ``cirq.DensityMatrixSimulator``
run (``cirq-core/cirq/linalg/transformations.py``,
``cirq-core/cirq/protocols/apply_channel_protocol.py``,
``cirq-core/cirq/sim/state_vector.py``, ``cirq-core/cirq/sim/simulation_utils.py``,
``cirq-core/cirq/ops/pauli_string.py``).  Each function cites the reference
lines it follows.

It is the checker, never the thing measured or shipped: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product package ``cirq_gb300`` never imports it.

Pinning: ``tests/test_oracle_golden.py`` checks this restatement against
golden vectors produced by the reference itself (``tests/golden/make_golden.py``
imports quantumlib/Cirq from source and runs its simulators).
"""

from oracle.statevector import (  # noqa: F401
    apply_matrix,
    apply_superop,
    apply_kraus_dm,
    apply_unitary_dm,
    probabilities_by_indices,
    sample_from_probs,
    pauli_expectation,
    pauli_apply,
    renormalize_like_cirq,
)
