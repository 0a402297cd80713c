"""Compilation of Clifford circuits into Pauli-frame programs (no GPU):
conjugation tables against the oracle's tableau, frame maps, the ops that
frames cannot take, and the C-ABI validator."""

import ctypes

import numpy as np
import pytest

import cirq
from cirq_gb300 import _lib, clifford as C, workloads
from oracle import clifford as oc

TWO_QUBIT = [cirq.CNOT, cirq.CZ, cirq.SWAP, cirq.ISWAP, cirq.CNOT ** -1, cirq.ISWAP ** -1]


def _oracle_image(u, k, idx):
    """(x', z', sign) of U P U^dagger for the Pauli with bits idx, by the
    oracle's tableau: a k-qubit tableau whose row 0 is set to P."""
    t = oc.Tableau(k)
    t.xs[:] = False
    t.zs[:] = False
    t.rs[:] = False
    for j in range(k):
        t.xs[0, j] = (idx >> j) & 1
        t.zs[0, j] = (idx >> (k + j)) & 1
    t.apply_unitary(u, list(range(k)))
    x = sum(int(t.xs[0, j]) << j for j in range(k))
    z = sum(int(t.zs[0, j]) << j for j in range(k))
    return x | (z << k) | (int(t.rs[0]) << (2 * k))


@pytest.mark.parametrize("gi", range(24))
def test_single_qubit_clifford_tables(gi):
    g = cirq.SingleQubitCliffordGate.all_single_qubit_cliffords[gi]
    u = cirq.unitary(g)
    table, lin = C.conjugation_table(u, 1)
    for idx in range(4):
        assert table[idx] == _oracle_image(u, 1, idx)


@pytest.mark.parametrize("gate", TWO_QUBIT, ids=str)
def test_two_qubit_tables_and_frame_maps(gate):
    u = cirq.unitary(gate)
    table, lin = C.conjugation_table(u, 2)
    rs = np.random.RandomState(0)
    for idx in range(16):
        assert table[idx] == _oracle_image(u, 2, idx)
    for _ in range(20):
        bits = int(rs.randint(16))
        out = 0
        for o in range(4):
            if bin(lin[o] & bits).count("1") & 1:
                out |= 1 << o
        assert out == table[bits] & 15


def test_three_qubit_clifford_and_global_phase():
    q = cirq.LineQubit.range(3)
    sub = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.CZ(q[1], q[2]), cirq.S(q[2]))
    op = cirq.CircuitOperation(sub.freeze())
    prog = C.CliffordProgram(cirq.Circuit(op, cirq.global_phase_operation(1j), cirq.measure(*q, key="m")))
    assert prog.nrec == 3 and prog.keys == {"m": [[0, 1, 2]]}
    u = cirq.unitary(cirq.MatrixGate(cirq.unitary(sub)))
    table, _ = C.conjugation_table(u, 3)
    for idx in (1, 8, 63, 37):
        assert table[idx] == _oracle_image(u, 3, idx)


@pytest.mark.parametrize(
    "make",
    [
        lambda q: cirq.Circuit(cirq.T(q[0]), cirq.measure(q[0])),
        lambda q: cirq.Circuit(cirq.measure(q[0], key="a", confusion_map={(0,): np.array([[0.9, 0.1], [0.1, 0.9]])})),
        lambda q: cirq.Circuit(cirq.amplitude_damp(0.1).on(q[0]), cirq.measure(q[0])),
        lambda q: cirq.Circuit(cirq.depolarize(0.1, n_qubits=2).on(q[0], q[1]), cirq.measure(q[0])),
        lambda q: cirq.Circuit(cirq.measure(q[0], key="a"), cirq.H(q[1]).with_classical_controls("a")),
    ],
    ids=["T", "confusion", "amplitude_damp", "depolarize2", "conditioned_H"],
)
def test_not_frameable(make):
    with pytest.raises(C.NotFrameable):
        C.CliffordProgram(make(cirq.LineQubit.range(2)))


def test_records_and_instances():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.Moment(cirq.measure(q[0], q[1], key="a", invert_mask=(True,))),
        cirq.Moment(cirq.X(q[2]).with_classical_controls("a")),
        cirq.Moment(cirq.measure(q[2], key="a")),
        cirq.Moment(cirq.reset(q[0])),
        cirq.Moment(cirq.bit_flip(0.25).on(q[1])),
    )
    prog = C.CliffordProgram(c)
    assert prog.keys == {"a": [[0, 1], [2]]}
    # layers of ops on disjoint qubits: the condition waits for its records,
    # the reset and the noise move up next to it
    kinds = list(prog.ops["kind"])
    assert kinds == [_lib.CLIFF_MEASURE, _lib.CLIFF_MEASURE, _lib.CLIFF_COND_PAULI, _lib.CLIFF_RESET,
                     _lib.CLIFF_NOISE, _lib.CLIFF_MEASURE]
    assert list(prog.layers) == [0, 2, 5, 6]
    assert prog.ops[0]["lin"][0] == 1 and prog.ops[1]["lin"][0] == 0
    assert list(prog.conds[:2]) == [0, 1]
    assert np.allclose(prog.ops[4]["p"], [0.25, 0, 0])


def test_validator_rejects_bad_programs():
    lib = _lib.load()
    c = workloads.random_clifford_circuit(4, 3, 0, mid_measure=1.0, feedback=True)
    prog = C.CliffordProgram(c)
    prog.validate(lib)

    def bad(mutate):
        ops = prog.ops.copy()
        mutate(ops)
        return lib.gbq_cliff_validate(4, ops.ctypes.data, len(ops), len(prog.tables), prog.nconds, prog.nrec)

    u = int(np.nonzero(prog.ops["kind"] == _lib.CLIFF_UNITARY)[0][0])
    m = int(np.nonzero(prog.ops["kind"] == _lib.CLIFF_MEASURE)[0][0])
    assert bad(lambda o: o[u].__setitem__("q", [7, 0, 0])) == _lib.ERR_ARG
    assert bad(lambda o: o[u].__setitem__("tab", len(prog.tables))) == _lib.ERR_ARG
    assert bad(lambda o: o[m].__setitem__("rec", prog.nrec)) == _lib.ERR_ARG
    assert bad(lambda o: o[u].__setitem__("k", 4)) == _lib.ERR_ARG
    two = int(np.nonzero((prog.ops["kind"] == _lib.CLIFF_UNITARY) & (prog.ops["k"] == 2))[0][0])
    assert bad(lambda o: o[two].__setitem__("q", [1, 1, 0])) == _lib.ERR_ARG
    noise = np.zeros(1, dtype=_lib.CLIFF_OP_DTYPE)
    noise[0]["kind"], noise[0]["k"] = _lib.CLIFF_NOISE, 1
    noise[0]["p"] = [0.6, 0.3, 0.3]
    assert lib.gbq_cliff_validate(2, noise.ctypes.data, 1, 0, 0, 0) == _lib.ERR_ARG
    assert _lib.CLIFF_OP_DTYPE.itemsize == 48
