"""lam = H psi on the GPU (gbq_sv_apply_paulisum: tiled passes over a cover
of the X masks, per-amplitude kernel for wide terms) against a complex128
numpy restatement of P = i^ny X^x Z^zy acting on a state
(cirq-core/cirq/ops/pauli_string.py:625-655 conventions).

Float32 amplitudes: the tolerance is 2e-6 of the largest output amplitude
per unit of sum |coef|."""

import ctypes

import numpy as np
import pytest

from cirq_gb300 import _lib
from cirq_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def _ref(psi, nbits, terms):
    idx = np.arange(1 << nbits, dtype=np.uint64)
    out = np.zeros(1 << nbits, np.complex128)
    for x, zy, ny, coef in terms:
        j = idx ^ np.uint64(x)
        sign = 1.0 - 2.0 * (np.bitwise_count(j & np.uint64(zy)) & 1)
        out += coef * (1j ** ny) * sign * psi[j.astype(np.int64)]
    return out


def _random_terms(rng, nbits, nterms, wmin=1, wmax=4):
    terms = []
    for _ in range(nterms):
        w = int(rng.integers(wmin, min(wmax, nbits) + 1))
        qs = rng.choice(nbits, size=w, replace=False)
        x = zy = ny = 0
        for q in qs:
            p = int(rng.integers(3))  # X, Y, Z
            if p in (0, 1):
                x |= 1 << int(q)
            if p in (1, 2):
                zy |= 1 << int(q)
            ny += p == 1
        terms.append((x, zy, ny, float(rng.normal())))
    return terms


def _gpu(nbits, psi, terms):
    eng = Engine.get(0)
    d_psi = eng.upload(psi.astype(np.complex64))
    d_out = eng.alloc(8 << nbits)
    eng.apply_paulisum(d_psi, nbits, terms, d_out)
    return d_out.download(np.empty(1 << nbits, np.complex64)).astype(np.complex128)


def _check(nbits, terms, seed=0):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=1 << nbits) + 1j * rng.normal(size=1 << nbits)
    psi /= np.linalg.norm(psi)
    psi = psi.astype(np.complex64).astype(np.complex128)
    got = _gpu(nbits, psi, terms)
    want = _ref(psi, nbits, terms)
    scale = max(1e-30, np.abs(want).max()) * max(1.0, sum(abs(t[3]) for t in terms))
    assert np.abs(got - want).max() <= 2e-6 * scale


def _cover(nbits, terms):
    rec = Engine.pauli_records(terms)
    np_, nw = ctypes.c_int(0), ctypes.c_int(0)
    assert _lib.load().gbq_paulisum_cover(rec.ctypes.data, len(rec), nbits, ctypes.byref(np_), ctypes.byref(nw), None, 0) == 0
    return np_.value, nw.value


@pytest.mark.parametrize("nbits", [1, 3, 5, 10, 11, 12, 13, 14, 16, 20])
def test_random_local_terms(nbits):
    rng = np.random.default_rng(nbits)
    _check(nbits, _random_terms(rng, nbits, 60), seed=nbits)


def test_many_terms_split_launches():
    # one pass (the whole state is one tile) holding more terms than a launch takes
    rng = np.random.default_rng(7)
    _check(12, _random_terms(rng, 12, 2500, 1, 6))


def test_wide_terms_mixed_with_tiled_ones():
    rng = np.random.default_rng(3)
    n = 18
    wide = [((1 << n) - 1, 0, 0, 0.7), ((1 << n) - 1 - 5, (1 << n) - 1, 3, -0.4), (0x3FF00, 0x3FF00, 10, 0.25)]
    terms = _random_terms(rng, n, 40) + wide
    npasses, nwide = _cover(n, terms)
    assert nwide == 3 and npasses >= 1
    _check(n, terms, seed=3)


def test_only_wide_terms_and_only_diagonal_terms():
    n = 16
    _check(n, [((1 << n) - 1, 0, 0, 1.0)])
    _check(n, [(0, 0b1011, 0, 0.5), (0, 0, 0, -1.25)])


def test_no_terms_gives_zeros():
    n = 15
    psi = np.ones(1 << n, np.complex128) / np.sqrt(1 << n)
    assert np.all(_gpu(n, psi, []) == 0)


def test_hamiltonian_of_the_gradient_bench():
    # 300 Pauli strings of weight 2..4 on 24 qubits are covered by few passes
    from cirq_gb300 import workloads
    from cirq_gb300.adjoint import AdjointProgram

    circuit, symbols, _ = workloads.hea_circuit(20, 1, seed=0)
    ham = workloads.random_pauli_hamiltonian(20, 300, seed=1)
    prog = AdjointProgram(circuit, ham, symbols)
    npasses, nwide = _cover(prog.n, prog.terms)
    assert nwide == 0 and npasses < 60
    _check(prog.n, prog.terms, seed=5)


def test_energy_at_bench_size_matches_per_term_expectations():
    # 24 qubits, the gradient bench's 300-term H: <psi|H psi> through the
    # tiled passes against the sum of the per-term expectation kernel's values
    from cirq_gb300 import workloads
    from cirq_gb300.adjoint import AdjointProgram

    circuit, symbols, values = workloads.hea_circuit(24, 2, seed=0)
    ham = workloads.random_pauli_hamiltonian(24, 300, seed=1)
    prog = AdjointProgram(circuit, ham, symbols)
    eng = prog.engine
    psi, lam, e_tiled, _ = prog.forward_state(values)
    per_term = eng.expect_paulis(psi, prog.n, prog.terms)
    e_terms = float(np.sum(per_term).real)
    scale = sum(abs(t[3]) for t in prog.terms)
    assert abs(e_tiled - e_terms) <= 2e-6 * scale
    psi.free()
    lam.free()
