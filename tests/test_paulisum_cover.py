"""Host planning of the tiled H psi passes (gbq_paulisum_cover; no GPU)."""

import ctypes
import time

import numpy as np

from cirq_gb300 import _lib
from cirq_gb300.engine import Engine


def _cover(nbits, terms):
    rec = Engine.pauli_records(terms)
    np_, nw = ctypes.c_int(0), ctypes.c_int(0)
    rc = _lib.load().gbq_paulisum_cover(rec.ctypes.data, len(rec), nbits, ctypes.byref(np_), ctypes.byref(nw), None, 0)
    assert rc == 0
    return np_.value, nw.value


def test_small_states_are_one_pass():
    assert _cover(10, [(0b1111111111, 0, 0, 1.0), (1, 2, 0, 0.5)]) == (1, 0)
    assert _cover(13, [(1 << 12, 0, 0, 1.0)]) == (1, 0)
    assert _cover(20, []) == (0, 0)


def test_wide_terms_are_counted():
    n = 24
    full = (1 << n) - 1
    # nine high X bits fit a tile with bits 0..3; ten do not
    nine = sum(1 << q for q in range(4, 13))
    ten = sum(1 << q for q in range(4, 14))
    assert _cover(n, [(full, 0, 0, 1.0)]) == (0, 1)
    assert _cover(n, [(nine, 0, 0, 1.0)]) == (1, 0)
    assert _cover(n, [(ten, 0, 0, 1.0), (nine | 0xF, 0, 0, 1.0)]) == (1, 1)


def test_bench_hamiltonian_needs_few_passes():
    from cirq_gb300 import workloads
    from cirq_gb300.adjoint import AdjointProgram

    circuit, symbols, _ = workloads.hea_circuit(24, 1, seed=0)
    ham = workloads.random_pauli_hamiltonian(24, 300, seed=1)
    prog = AdjointProgram(circuit, ham, symbols)
    t = time.perf_counter()
    npasses, nwide = _cover(prog.n, prog.terms)
    first = time.perf_counter() - t
    xgroups = len({x for x, *_ in prog.terms})
    assert nwide == 0
    assert npasses * 3 < xgroups  # fewer state transfers than one read per X mask
    t = time.perf_counter()
    assert _cover(prog.n, prog.terms) == (npasses, nwide)
    assert time.perf_counter() - t < max(first, 0.01)  # memoised


def test_single_qubit_x_terms_all_covered():
    # sum_j X_j on 30 qubits: 26 masks above bit 3, nine per pass
    n = 30
    npasses, nwide = _cover(n, [(1 << q, 0, 0, 1.0) for q in range(n)])
    assert nwide == 0 and npasses == 3
