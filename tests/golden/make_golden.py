"""Generates the golden fixtures in this directory by running quantumlib/Cirq itself.

Run from the repository root in a checkout that has the reference source:

    python tests/golden/make_golden.py /path/to/Cirq/cirq-core

(or set ``CIRQ_REFERENCE_PATH`` to that directory instead of passing it).

The reference's own simulators (``cirq.Simulator``,
``cirq.DensityMatrixSimulator``) and protocols produce every array stored
here; nothing in this script re-implements them.  The fixtures are small
(a few hundred KB in total) so the test suite can pin both the CPU oracle and
the CUDA path against the reference on machines where the reference source is
absent.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _import_reference(path: str):
    sys.path.insert(0, path)
    sys.path.insert(0, ROOT)
    from cirq_gb300._cirq_env import ensure_cirq

    cirq = ensure_cirq()
    assert os.path.abspath(cirq.__file__).startswith(os.path.abspath(path)), cirq.__file__
    return cirq


def main(ref_path: str) -> None:
    cirq = _import_reference(ref_path)
    import sympy

    from cirq_gb300 import workloads

    out = {}

    # 1. random PhasedXZ + CZ layers, final states at complex128 and complex64.
    for n, d, seed in [(10, 20, 1), (12, 8, 2), (5, 6, 3)]:
        c = workloads.random_layer_circuit(n, d, seed)
        s128 = cirq.Simulator(dtype=np.complex128).simulate(c).final_state_vector
        s64 = cirq.Simulator(dtype=np.complex64).simulate(c).final_state_vector
        out[f"layers_n{n}_d{d}_s{seed}_c128"] = s128
        out[f"layers_n{n}_d{d}_s{seed}_c64"] = s64
    # custom qubit order (reversed) and a basis-state initial state
    c = workloads.random_layer_circuit(6, 5, 4)
    q = sorted(c.all_qubits())
    out["layers_n6_d5_s4_reversed_init5"] = (
        cirq.Simulator(dtype=np.complex128)
        .simulate(c, qubit_order=q[::-1], initial_state=5)
        .final_state_vector
    )

    # 2. mixed gate zoo (every gate family the translator handles).
    zoo = _gate_zoo(cirq)
    out["zoo_c128"] = cirq.Simulator(dtype=np.complex128).simulate(zoo).final_state_vector

    # 3. noisy density matrices.
    c = workloads.noisy_layer_circuit(4, 4, seed=2, p=0.05, gamma=0.1)
    out["dm_noisy_n4_d4"] = (
        cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(c).final_density_matrix
    )
    c = workloads.random_layer_circuit(3, 3, seed=5)
    out["dm_noisemodel_n3"] = (
        cirq.DensityMatrixSimulator(dtype=np.complex128, noise=cirq.depolarize(0.02))
        .simulate(c)
        .final_density_matrix
    )
    qd = cirq.LineQubit.range(3)
    cg = cirq.Circuit(
        cirq.H(qd[0]),
        cirq.CNOT(qd[0], qd[1]),
        cirq.generalized_amplitude_damp(0.3, 0.2).on(qd[1]),
        cirq.phase_damp(0.25).on(qd[0]),
        cirq.bit_flip(0.1).on(qd[2]),
        cirq.asymmetric_depolarize(0.05, 0.1, 0.15).on(qd[2]),
        cirq.CZ(qd[1], qd[2]) ** 0.3,
        cirq.depolarize(0.1, n_qubits=2).on(qd[0], qd[2]),
        cirq.reset(qd[1]),
    )
    out["dm_channels_n3"] = (
        cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(cg).final_density_matrix
    )

    # 4. QAOA expectation values over a sweep.
    circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(8, 4, seed=7)
    pts = workloads.qaoa_points(4, 16, seed=8)
    resolvers = [
        cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))}) for p in pts
    ]
    vals = cirq.Simulator(dtype=np.complex128).simulate_expectation_values_sweep(
        circuit, obs, resolvers
    )
    out["qaoa_n8_p4_points"] = pts
    out["qaoa_n8_p4_expect"] = np.array([v[0] for v in vals])

    # 5. HEA energy, central finite differences and parameter-shift gradients
    #    evaluated with the reference's simulate_expectation_values.
    circuit, symbols, values = workloads.hea_circuit(5, 2, seed=9)
    ham = workloads.random_pauli_hamiltonian(5, 12, seed=10)
    sim = cirq.Simulator(dtype=np.complex128)

    def energy(v):
        return sim.simulate_expectation_values(
            circuit, ham, param_resolver=dict(zip(symbols, v))
        )[0].real

    e0 = energy(values)
    fd = np.zeros(len(symbols))
    ps = np.zeros(len(symbols))
    for i in range(len(symbols)):
        vp = values.copy()
        vm = values.copy()
        vp[i] += 1e-4
        vm[i] -= 1e-4
        fd[i] = (energy(vp) - energy(vm)) / 2e-4
        vp = values.copy()
        vm = values.copy()
        vp[i] += np.pi / 2
        vm[i] -= np.pi / 2
        ps[i] = (energy(vp) - energy(vm)) / 2
    out["hea_n5_l2_values"] = values
    out["hea_n5_l2_energy"] = np.array(e0)
    out["hea_n5_l2_grad_fd"] = fd
    out["hea_n5_l2_grad_ps"] = ps

    # 6. Pauli-sum expectations on a random state.
    rs = np.random.RandomState(11)
    n = 6
    psi = rs.normal(size=2**n) + 1j * rs.normal(size=2**n)
    psi /= np.linalg.norm(psi)
    qs = cirq.LineQubit.range(n)
    ham = workloads.random_pauli_hamiltonian(n, 20, seed=12, min_w=1, max_w=4)
    qmap = {x: i for i, x in enumerate(qs)}
    out["pauli_n6_state"] = psi
    out["pauli_n6_terms_expect"] = np.array(
        [ps_.expectation_from_state_vector(psi, qmap) for ps_ in ham]
    )
    out["pauli_n6_sum_expect"] = np.array(ham.expectation_from_state_vector(psi, qmap))

    # 7. marginal probabilities used for sampling.
    probs = np.abs(psi) ** 2
    for idx in ([0, 1, 2, 3, 4, 5], [2], [4, 1], [5, 0, 3]):
        key = "probs_n6_" + "_".join(map(str, idx))
        out[key] = cirq.sim.simulation_utils.state_probabilities_by_indices(probs, idx, (2,) * n)

    # 8. known answers copied from the reference's own tests, kept as data.
    out["known_expect_c1"] = np.array([-2.2, 0.0])  # sparse_simulator_test.py:638-640
    out["known_expect_c2"] = np.array([0.0, 1.0])  # :643-645
    out["known_expect_c3"] = np.array([2.0])  # :650
    out["known_dm_ad"] = np.array([-0.8, 0.0])  # density_matrix_simulator_test.py:899-900
    out["known_dm_dep"] = np.array([0.0, 0.6])  # :904-905

    # 9. module-level helpers (cirq-core/cirq/sim/mux.py) and wide gates
    cc = _classical_control_circuit(cirq)
    out["mux_fdm_classical_control"] = cirq.final_density_matrix(cc, dtype=np.complex128)
    meas = _measured_circuit(cirq)
    out["mux_fdm_dephased"] = cirq.final_density_matrix(meas, dtype=np.complex128)
    out["mux_fdm_dephased_noisy"] = cirq.final_density_matrix(
        meas, noise=cirq.amplitude_damp(0.1), dtype=np.complex128
    )
    qm = sorted(meas.all_qubits())
    out["mux_fsv_ignore_terminal"] = cirq.final_state_vector(
        meas, ignore_terminal_measurements=True, qubit_order=qm[::-1], dtype=np.complex128
    )
    pc, presolver = _noisy_param_circuit(cirq, sympy)
    out["dm_noisy_param_split"] = (
        cirq.DensityMatrixSimulator(dtype=np.complex128, noise=cirq.amplitude_damp(0.2))
        .simulate(pc, presolver)
        .final_density_matrix
    )
    out["wide_controlled_c128"] = (
        cirq.Simulator(dtype=np.complex128).simulate(_wide_controlled_circuit(cirq)).final_state_vector
    )

    qc, qorder = _qudit_circuit(cirq)
    out["qudit_sv_c128"] = (
        cirq.Simulator(dtype=np.complex128).simulate(qc, qubit_order=qorder, initial_state=17).final_state_vector
    )
    out["qudit_dm_c128"] = (
        cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(_qudit_noisy_circuit(cirq)).final_density_matrix
    )

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    with open(os.path.join(HERE, "golden_meta.txt"), "w") as f:
        f.write(f"generated by tests/golden/make_golden.py with cirq {cirq.__version__}\n")
        for k in sorted(out):
            f.write(f"{k}: shape={np.shape(out[k])} dtype={np.asarray(out[k]).dtype}\n")
    print("wrote", len(out), "arrays")


def _gate_zoo(cirq):
    """A circuit that touches every gate family the GPU translator handles."""
    q = cirq.LineQubit.range(5)
    return cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.X(q[0]) ** 0.3,
        cirq.Y(q[1]) ** 0.7,
        cirq.Z(q[2]) ** 0.11,
        cirq.rx(0.4).on(q[3]),
        cirq.ry(-1.1).on(q[4]),
        cirq.rz(2.3).on(q[0]),
        cirq.S(q[1]),
        cirq.T(q[2]),
        cirq.CNOT(q[0], q[3]),
        cirq.CZ(q[1], q[4]) ** 0.37,
        cirq.SWAP(q[2], q[0]),
        cirq.ISWAP(q[3], q[4]) ** 0.5,
        cirq.ZZ(q[0], q[4]) ** 0.21,
        cirq.XX(q[1], q[2]) ** 0.4,
        cirq.YY(q[3], q[0]) ** -0.6,
        cirq.CCZ(q[0], q[1], q[2]),
        cirq.CCX(q[2], q[3], q[4]),
        cirq.CSWAP(q[4], q[0], q[1]),
        cirq.FSimGate(0.3, 0.9).on(q[1], q[3]),
        cirq.PhasedXPowGate(phase_exponent=0.25, exponent=0.5).on(q[2]),
        cirq.PhasedXZGate(x_exponent=0.3, z_exponent=-0.2, axis_phase_exponent=0.6).on(q[4]),
        cirq.MatrixGate(cirq.testing.random_unitary(4, random_state=3)).on(q[4], q[1]),
        cirq.DiagonalGate([0.1, 0.5, -0.7, 1.3]).on(q[3], q[2]),
        cirq.ControlledGate(cirq.Y ** 0.25).on(q[0], q[4]),
        cirq.global_phase_operation(np.exp(0.3j)),
        cirq.I(q[2]),
        cirq.MatrixGate(cirq.testing.random_unitary(8, random_state=4)).on(q[0], q[2], q[4]),
    )


def _classical_control_circuit(cirq):
    """Mid-circuit measurements feeding classically controlled gates."""
    q = cirq.LineQubit.range(3)
    return cirq.Circuit(
        cirq.H(q[0]),
        cirq.ry(0.7).on(q[2]),
        cirq.measure(q[0], key="a"),
        cirq.X(q[1]).with_classical_controls("a"),
        cirq.measure(q[2], key="b"),
        cirq.CZ(q[0], q[1]).with_classical_controls("b"),
        cirq.H(q[1]),
    )


def _measured_circuit(cirq):
    """Unitary layers ending in a measurement of two of four qubits."""
    q = cirq.LineQubit.range(4)
    return cirq.Circuit(
        cirq.H(q[0]),
        cirq.CNOT(q[0], q[1]),
        cirq.rx(0.4).on(q[2]),
        cirq.CZ(q[2], q[3]),
        cirq.ry(1.1).on(q[3]),
        cirq.measure(q[1], q[3], key="m"),
    )


def _noisy_param_circuit(cirq, sympy):
    """Moments mixing unparameterized and parameterized ops: the reference's
    density-matrix simulator noises its prefix and suffix separately."""
    q = cirq.LineQubit.range(3)
    t = sympy.Symbol("t")
    c = cirq.Circuit(
        cirq.Moment([cirq.H(q[2]), cirq.rx(t).on(q[0])]),
        cirq.Moment([cirq.CZ(q[0], q[1])]),
        cirq.Moment([cirq.ry(0.3).on(q[1]), cirq.X(q[2])]),
    )
    return c, cirq.ParamResolver({"t": 0.7})


def _wide_controlled_circuit(cirq):
    """Gates on 6 and 7 qubits (more than one fused block holds)."""
    q = cirq.LineQubit.range(8)
    return cirq.Circuit(
        cirq.H.on_each(*q),
        cirq.X(q[6]).controlled_by(*q[:6]),
        cirq.rz(0.3).on(q[7]).controlled_by(*q[1:6]),
        cirq.CZ(q[0], q[7]),
        cirq.Y(q[2]).controlled_by(q[0], q[1], q[3], q[4], q[5], q[7], control_values=[1, 0, 1, 1, 0, 1]),
    )


def _givens(d: int, i: int, j: int, theta: float, phi: float) -> np.ndarray:
    """A rotation by theta (with phase phi) in the (i, j) plane of d levels."""
    g = np.eye(d, dtype=np.complex128)
    c, s = np.cos(theta), np.sin(theta)
    g[i, i], g[j, j] = c, c
    g[i, j], g[j, i] = -s * np.exp(-1j * phi), s * np.exp(1j * phi)
    return g


def _qudit_unitary(d: int, seed: int) -> np.ndarray:
    """A dense d-level unitary from closed-form factors (Givens rotations
    and phases), identical on every machine."""
    u = np.diag(np.exp(1j * (0.3 + 0.17 * seed) * np.arange(d) ** 2))
    for k in range(2 * d):
        i, j = k % d, (k * (seed + 2) + 1) % d
        if i != j:
            u = _givens(d, i, j, 0.4 + 0.11 * k + 0.07 * seed, 0.2 * k - 0.3 * seed) @ u
    return u


def _qudit_circuit(cirq):
    """Qids of dimensions 3, 2, 4 and 5 (8 index bits) with one- and two-qid
    unitaries; simulated with a custom qubit order."""
    q3, q2, q4, q5 = cirq.LineQid(0, 3), cirq.LineQubit(1), cirq.LineQid(2, 4), cirq.LineQid(3, 5)
    dft4 = np.exp(2j * np.pi * np.outer(np.arange(4), np.arange(4)) / 4) / 2
    c = cirq.Circuit(
        cirq.MatrixGate(_qudit_unitary(3, 1), qid_shape=(3,)).on(q3),
        cirq.H(q2),
        cirq.MatrixGate(dft4, qid_shape=(4,)).on(q4),
        cirq.MatrixGate(_qudit_unitary(5, 2), qid_shape=(5,)).on(q5),
        cirq.MatrixGate(_qudit_unitary(6, 3), qid_shape=(3, 2)).on(q3, q2),
        cirq.MatrixGate(_qudit_unitary(20, 4), qid_shape=(4, 5)).on(q4, q5),
        cirq.rz(0.4).on(q2),
        cirq.MatrixGate(_qudit_unitary(12, 5), qid_shape=(3, 4)).on(q3, q4),
    )
    return c, [q5, q2, q3, q4]


def _qudit_noisy_circuit(cirq):
    """Qutrit and ququart channels (damping, a mixture, a reset) between
    unitaries, for the density-matrix simulator."""
    q3, q2, q4 = cirq.LineQid(0, 3), cirq.LineQubit(1), cirq.LineQid(2, 4)
    g = 0.25
    k0 = np.diag([1.0, np.sqrt(1 - g), np.sqrt(1 - g)]).astype(np.complex128)
    k1 = np.zeros((3, 3), dtype=np.complex128)
    k1[0, 1] = np.sqrt(g)
    k2 = np.zeros((3, 3), dtype=np.complex128)
    k2[1, 2] = np.sqrt(g)
    shift = np.roll(np.eye(4), 1, axis=0)

    class QutritDamping(cirq.Gate):
        def _qid_shape_(self):
            return (3,)

        def _kraus_(self):
            return [k0, k1, k2]

    class QuartShift(cirq.Gate):
        def _qid_shape_(self):
            return (4,)

        def _mixture_(self):
            return [(0.7, np.eye(4)), (0.3, shift)]

    return cirq.Circuit(
        cirq.MatrixGate(_qudit_unitary(3, 6), qid_shape=(3,)).on(q3),
        cirq.H(q2),
        cirq.MatrixGate(_qudit_unitary(4, 7), qid_shape=(4,)).on(q4),
        cirq.MatrixGate(_qudit_unitary(6, 8), qid_shape=(3, 2)).on(q3, q2),
        QutritDamping().on(q3),
        QuartShift().on(q4),
        cirq.MatrixGate(_qudit_unitary(8, 9), qid_shape=(2, 4)).on(q2, q4),
        cirq.ResetChannel(dimension=3).on(q3),
        cirq.MatrixGate(_qudit_unitary(3, 10), qid_shape=(3,)).on(q3),
    )


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CIRQ_REFERENCE_PATH")
    if not ref:
        sys.exit("usage: make_golden.py <path to the reference's cirq-core> (or set CIRQ_REFERENCE_PATH)")
    main(ref)
