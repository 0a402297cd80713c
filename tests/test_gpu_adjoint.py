"""Adjoint gradients vs the reference's finite-difference / parameter-shift
gradients (golden), the complex128 oracle, and torch autograd."""

import numpy as np
import pytest

import cirq
import cirq_gb300
from cirq_gb300 import adjoint, workloads
from oracle.circuits import expectation_of_circuit, finite_difference_gradient

pytestmark = pytest.mark.gpu

GOLD = np.load(__file__.replace("test_gpu_adjoint.py", "golden/golden.npz"))
TOL = 1e-4  # absolute, on expectations and gradients


def test_hea_vs_reference_gradients():
    circuit, symbols, _ = workloads.hea_circuit(5, 2, seed=9)
    ham = workloads.random_pauli_hamiltonian(5, 12, seed=10)
    values = GOLD["hea_n5_l2_values"]
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    E, g = prog.value_and_grad(values)
    assert abs(E - float(GOLD["hea_n5_l2_energy"])) < TOL
    np.testing.assert_allclose(g, GOLD["hea_n5_l2_grad_ps"], atol=TOL)
    np.testing.assert_allclose(g, GOLD["hea_n5_l2_grad_fd"], atol=TOL)


@pytest.mark.parametrize("n,layers", [(12, 3), (14, 2)])
def test_hea_vs_oracle_fd(n, layers):
    circuit, symbols, values = workloads.hea_circuit(n, layers, seed=n)
    ham = workloads.random_pauli_hamiltonian(n, 30, seed=n + 1)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    E, g = prog.value_and_grad(values)
    r = dict(zip(symbols, values))
    assert abs(E - expectation_of_circuit(circuit, ham, r).real) < TOL
    idx = [0, 1, n, 2 * n - 1, len(symbols) - 1]
    fd = finite_difference_gradient(circuit, ham, symbols, values, h=1e-3, indices=idx)
    np.testing.assert_allclose(g[idx], fd, atol=TOL)


def test_general_parameterised_gates():
    """Shared symbols, expressions and non-rotation gates (chain rule)."""
    import sympy

    a, b = sympy.symbols("a b")
    q = cirq.LineQubit.range(11)
    circuit = cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.XPowGate(exponent=a).on(q[0]),
        cirq.ZZPowGate(exponent=2 * a + b).on(q[1], q[5]),
        cirq.CZPowGate(exponent=b).on(q[2], q[10]),
        cirq.ry(a * b).on(q[3]),
        cirq.PhasedXPowGate(phase_exponent=b, exponent=0.3).on(q[4]),
        cirq.ISwapPowGate(exponent=a).on(q[6], q[7]),
        cirq.CNOT(q[0], q[8]),
    )
    ham = workloads.random_pauli_hamiltonian(11, 25, seed=3)
    prog = adjoint.AdjointProgram(circuit, ham, [a, b])
    vals = [0.41, -0.77]
    E, g = prog.value_and_grad(vals)
    fd = finite_difference_gradient(circuit, ham, [a, b], vals, h=1e-4)
    np.testing.assert_allclose(g, fd, atol=TOL)


def test_torch_autograd():
    torch = pytest.importorskip("torch")
    circuit, symbols, values = workloads.hea_circuit(6, 2, seed=4)
    ham = workloads.random_pauli_hamiltonian(6, 15, seed=5)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    theta = torch.tensor(values, dtype=torch.float64, requires_grad=True)
    e = adjoint.expectation(theta, prog)
    (3.0 * e).backward()
    E, g = prog.value_and_grad(values)
    assert abs(e.item() - E) < 1e-9
    np.testing.assert_allclose(theta.grad.numpy(), 3.0 * g, atol=1e-9)


def test_parameter_shift_through_plain_simulator_matches():
    circuit, symbols, values = workloads.hea_circuit(10, 2, seed=6)
    ham = workloads.random_pauli_hamiltonian(10, 20, seed=7)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    _, g = prog.value_and_grad(values)
    ps = adjoint.parameter_shift_gradient(cirq_gb300.Simulator(), circuit, ham, symbols, values, indices=range(8))
    np.testing.assert_allclose(g[:8], ps[:8], atol=TOL)


def test_one_call_adjoint_entry_point_matches():
    """gbq_adjoint (the whole gradient in one C-ABI call) against the
    reference's parameter-shift gradient and the orchestrated path."""
    circuit, symbols, _ = workloads.hea_circuit(5, 2, seed=9)
    ham = workloads.random_pauli_hamiltonian(5, 12, seed=10)
    values = GOLD["hea_n5_l2_values"]
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    E, g = prog.value_and_grad_native(values)
    assert abs(E - float(GOLD["hea_n5_l2_energy"])) < TOL
    np.testing.assert_allclose(g, GOLD["hea_n5_l2_grad_ps"], atol=TOL)
    circuit, symbols, values = workloads.hea_circuit(14, 3, seed=14)
    ham = workloads.random_pauli_hamiltonian(14, 40, seed=15)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    E1, g1 = prog.value_and_grad(values)
    E2, g2 = prog.value_and_grad_native(values)
    assert abs(E1 - E2) < 1e-6
    np.testing.assert_allclose(g1, g2, atol=1e-6)
