"""The allocation-free expectation entry point, checked against the regular one.

gbq_sv_expect_paulis_noalloc serves callers that cannot allocate device
memory (services whose device memory belongs to a host framework's pool,
loops that cannot pay cudaMalloc's device synchronisation).  Its scratch is
a fixed array in the library's device image that every call shares, so the
test makes two calls in a row with different term lists -- the second must
not see anything left over from the first -- passes the terms' own
coefficients through the call, and makes one call on a freshly created
non-default stream.  This file is collected last, so a failure here does not
stop the other GPU tests.
"""

import numpy as np
import pytest

import cirq
from cirq_gb300 import _lib, workloads
from cirq_gb300.engine import Engine
from cirq_gb300.ir import pauli_terms

pytestmark = pytest.mark.gpu

TOL = 1e-4  # absolute, as for every expectation value in these tests


def _noalloc(eng, state, n, terms, stream=None):
    rec = Engine.pauli_records(terms)
    out = np.zeros(2 * len(rec), dtype=np.float64)
    _lib.check(
        eng.lib.gbq_sv_expect_paulis_noalloc(stream, state.ptr, n, rec.ctypes.data, len(rec), out.ctypes.data),
        "gbq_sv_expect_paulis_noalloc",
    )
    return out[0::2] + 1j * out[1::2]


def _state(n, seed):
    import cirq_gb300

    circuit = workloads.random_layer_circuit(n, 8, seed=seed)
    sim = cirq_gb300.Simulator()
    compiled = sim._prepare(circuit, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))[2]
    state = sim._evolve(compiled, compiled.pool([cirq.ParamResolver({})])[0], 0)
    index = {x: i for i, x in enumerate(sorted(circuit.all_qubits()))}
    return sim.engine, state, index


def test_noalloc_matches_regular_entry_point_twice():
    n = 18
    eng, state, index = _state(n, 31)
    ham1 = workloads.random_pauli_hamiltonian(n, 120, seed=32, min_w=1, max_w=4)
    ham2 = workloads.random_pauli_hamiltonian(n, 17, seed=33, min_w=2, max_w=3)
    for ham in (ham1, ham2):  # two calls in a row, different sizes
        terms = pauli_terms(ham, index, n)
        assert any(abs(c - 1.0) > 1e-3 for *_, c in terms)  # the coefficients are applied by the call
        want = eng.expect_paulis(state, n, terms)
        got = _noalloc(eng, state, n, terms)
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) < TOL


def test_noalloc_on_a_non_default_stream():
    torch = pytest.importorskip("torch")
    n = 16
    eng, state, index = _state(n, 34)
    eng.sync()  # the state was written on the engine's stream
    terms = pauli_terms(workloads.random_pauli_hamiltonian(n, 40, seed=35), index, n)
    want = eng.expect_paulis(state, n, terms)
    stream = torch.cuda.Stream(device=0)
    got = _noalloc(eng, state, n, terms, stream=stream.cuda_stream)
    assert np.max(np.abs(got - want)) < TOL


def test_noalloc_rejects_oversized_term_lists():
    eng = Engine.get(0)
    n = 16
    state = eng.new_state(n, basis=0)
    rs = np.random.RandomState(0)
    terms = [(int(rs.randint(1 << n)), int(rs.randint(1 << n)), 0, 1.0) for _ in range(5000)]
    rec = Engine.pauli_records(terms)
    out = np.zeros(2 * len(rec))
    rc = eng.lib.gbq_sv_expect_paulis_noalloc(None, state.ptr, n, rec.ctypes.data, len(rec), out.ctypes.data)
    assert rc == _lib.ERR_ARG
    msg = eng.lib.gbq_last_error().decode()
    assert "scratch" in msg
    # the limit it names fits
    fit = int(msg.split("at most ")[1].split(" ")[0])
    assert 0 < fit < 5000
    rc = eng.lib.gbq_sv_expect_paulis_noalloc(None, state.ptr, n, rec.ctypes.data, fit, out.ctypes.data)
    assert rc == 0
