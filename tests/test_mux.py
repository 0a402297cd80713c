"""Host-side behaviour of the module-level entry points (cirq_gb300.mux):
argument checks and error messages of ``cirq.final_state_vector`` and the
measurement dephasing of ``cirq.final_density_matrix``
(cirq-core/cirq/sim/mux.py:109-177, 225-333).  No GPU is touched: every
case here fails or transforms before a simulator is built."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import mux


def test_exports():
    for name in ("sample", "sample_sweep", "final_state_vector", "final_density_matrix"):
        assert getattr(cirq_gb300, name) is getattr(mux, name)


def test_final_state_vector_rejects_measurements_like_the_reference():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0]))
    with pytest.raises(ValueError, match="Circuit contains a measurement."):
        cirq_gb300.final_state_vector(c)
    with pytest.raises(ValueError, match="Circuit contains a measurement."):
        cirq.final_state_vector(c)


def test_final_state_vector_rejects_non_unitary_like_the_reference():
    q = cirq.LineQubit(0)
    c = cirq.Circuit(cirq.amplitude_damp(0.1).on(q))
    with pytest.raises(ValueError, match="not unitary"):
        cirq_gb300.final_state_vector(c)
    with pytest.raises(ValueError, match="not unitary"):
        cirq.final_state_vector(c)


def test_to_circuit_accepts_gates_and_op_trees():
    c = mux._to_circuit(cirq.CZ)
    assert len(c.all_qubits()) == 2
    q = cirq.LineQubit.range(2)
    assert mux._to_circuit([cirq.H(q[0]), cirq.CNOT(*q)]) == cirq.Circuit([cirq.H(q[0]), cirq.CNOT(*q)])


def test_dephase_matches_the_reference_transformer_channel_by_channel():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0], q[2], key="m"), cirq.CNOT(q[0], q[1]))
    ours = mux._dephase(c)
    ref = cirq.dephase_measurements(c)
    # same moments (a noise model inserts noise per moment)
    assert [sorted(map(str, m.qubits)) for m in ours] == [sorted(map(str, m.qubits)) for m in ref]
    ours_ops = list(ours.all_operations())
    ref_ops = list(ref.all_operations())
    assert [o.qubits for o in ours_ops] == [o.qubits for o in ref_ops]
    for a, b in zip(ours_ops, ref_ops):
        if cirq.has_unitary(a):
            np.testing.assert_allclose(cirq.unitary(a), cirq.unitary(b))
        else:
            # same channel, without the measurement key
            sa = cirq.kraus_to_superoperator(cirq.kraus(a))
            sb = cirq.kraus_to_superoperator(cirq.kraus(b))
            np.testing.assert_allclose(sa, sb, atol=1e-12)
            assert not cirq.is_measurement(a)


def test_dephase_requires_deferred_classical_control():
    q = cirq.LineQubit.range(2)
    c = cirq.Circuit(cirq.measure(q[0], key="a"), cirq.X(q[1]).with_classical_controls("a"))
    with pytest.raises(ValueError, match="defer_measurements"):
        mux._dephase(c)
