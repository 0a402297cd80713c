"""Adjoint gradients computed by the package's host logic (forward and
reverse programs, probe slots, symbol bookkeeping) on the CPU emulation of
the engine, against the reference's own gradients (golden) and the oracle's
finite differences.  CPU only; the GPU tests run the same programs on the
kernels."""

import numpy as np
import pytest
import sympy

import cirq
from cirq_gb300 import adjoint, workloads
from cpu_engine import EmuEngine
from oracle.circuits import expectation_of_circuit, finite_difference_gradient

GOLD = np.load(__file__.replace("test_adjoint_emulated.py", "golden/golden.npz"))
TOL = 1e-6


def test_hea_vs_reference_gradients():
    circuit, symbols, _ = workloads.hea_circuit(5, 2, seed=9)
    ham = workloads.random_pauli_hamiltonian(5, 12, seed=10)
    values = GOLD["hea_n5_l2_values"]
    eng = EmuEngine()
    prog = adjoint.AdjointProgram(circuit, ham, symbols, engine=eng)
    E, g = prog.value_and_grad(values)
    assert abs(E - float(GOLD["hea_n5_l2_energy"])) < TOL
    np.testing.assert_allclose(g, GOLD["hea_n5_l2_grad_ps"], atol=1e-5)
    assert eng.launches() > 0


def _param_circuit(seed, n):
    rng = np.random.default_rng(seed)
    q = cirq.LineQubit.range(n)
    syms = sympy.symbols(f"t0:{6}")
    ops = []
    for _ in range(4 * n):
        s = syms[rng.integers(0, len(syms))]
        kind = rng.integers(0, 8)
        a, b = [q[i] for i in rng.choice(n, size=2, replace=False)]
        if kind == 0:
            ops.append(cirq.rx(s).on(a))
        elif kind == 1:
            ops.append(cirq.ry(2 * s).on(a))
        elif kind == 2:
            ops.append(cirq.rz(s).on(a))
        elif kind == 3:
            ops.append(cirq.ZZPowGate(exponent=s).on(a, b))
        elif kind == 4:
            ops.append((cirq.X ** s).on(a))
        elif kind == 5:
            ops.append((cirq.CZ ** s).on(a, b))
        elif kind == 6:
            ops.append(cirq.CNOT(a, b))
        else:
            ops.append(cirq.H(a))
    return cirq.Circuit(ops), list(syms)


@pytest.mark.parametrize("seed,n,tile,rtile", [(1, 6, 12, 11), (2, 11, 10, 10), (3, 12, 10, 11), (4, 9, 11, 10)])
def test_random_parameterized_circuits_vs_oracle_fd(seed, n, tile, rtile):
    circuit, symbols = _param_circuit(seed, n)
    symbols = [s for s in symbols if s in cirq.parameter_symbols(circuit)]
    ham = workloads.random_pauli_hamiltonian(n, 10, seed=seed + 50)
    values = np.random.default_rng(seed + 7).uniform(-1.5, 1.5, len(symbols))
    prog = adjoint.AdjointProgram(circuit, ham, symbols, engine=EmuEngine(), tile_bits=tile,
                                  reverse_tile_bits=rtile)
    E, g = prog.value_and_grad(values)
    r = dict(zip(symbols, values))
    assert abs(E - expectation_of_circuit(circuit, ham, r).real) < TOL
    fd = finite_difference_gradient(circuit, ham, symbols, values, h=1e-4)
    np.testing.assert_allclose(g, fd, atol=1e-5)


def test_repeated_calls_reuse_buffers_and_match_fresh_ones():
    circuit, symbols, _ = workloads.hea_circuit(5, 2, seed=3)
    ham = workloads.random_pauli_hamiltonian(5, 9, seed=4)
    eng = EmuEngine()
    prog = adjoint.AdjointProgram(circuit, ham, symbols, engine=eng)
    rng = np.random.default_rng(0)
    points = [rng.uniform(-2, 2, len(symbols)) for _ in range(3)]
    first = [prog.value_and_grad(v) for v in points]
    kept = {k: b.ptr for k, b in prog._buffers.items()}
    again = [prog.value_and_grad(v) for v in points]
    assert {k: b.ptr for k, b in prog._buffers.items()} == kept  # no new buffers
    for (e1, g1), (e2, g2) in zip(first, again):
        assert e1 == e2 and np.array_equal(g1, g2)
    for v, (e1, g1) in zip(points, first):
        # the allocating path (as the torch autograd function uses it)
        psi, lam, e, r = prog.forward_state(v)
        g = prog.gradient_from(psi, lam, r)
        assert e == e1 and np.array_equal(g, g1)
    prog.release()
    assert not getattr(prog, "_buffers", {})
