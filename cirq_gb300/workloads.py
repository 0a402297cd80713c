"""Seeded synthetic circuits for the simulation workloads this package is measured on.

All generators are deterministic in ``seed`` (``numpy.random.RandomState``).

* ``random_layer_circuit`` -- n qubits on a line, depth d: each layer puts a
  ``cirq.PhasedXZGate(x, z, a)`` (x, z, a ~ U(-1, 1)) on every qubit, then
  ``CZ(i, i+1)`` for every i with i = layer (mod 2).
* ``noisy_layer_circuit`` -- the same layers, each gate followed by
  ``depolarize(p)`` on each of its qubits and each layer by
  ``amplitude_damp(gamma)`` on every qubit.
* ``qaoa_circuit`` -- QAOA on a seeded random 3-regular graph: H on all
  qubits, then p layers of ``ZZPowGate(exponent=gamma_l)`` on every edge and
  ``XPowGate(exponent=beta_l)`` on every qubit; observable sum of Z_i Z_j
  over edges.
* ``hea_circuit`` -- hardware-efficient ansatz: per layer ``rx(theta)``,
  ``rz(theta)`` on every qubit then a CZ ladder; Hamiltonian of random Pauli
  strings of weight 2..4 with N(0, 1) coefficients.
* ``random_clifford_circuit`` -- n qubits, depth d: each layer a random
  single-qubit Clifford (one of the 24, as a ``SingleQubitCliffordGate``) on
  every qubit, then two-qubit Cliffords (CNOT, CZ, SWAP or ISWAP, chosen at
  random) on a brickwork of neighbouring pairs; optionally measurements of
  random qubits into fresh keys after some layers (``mid_measure``),
  resets, a Pauli X conditioned on the previous key (``feedback``),
  ``depolarize(p)`` on every qubit after each layer, and a final measurement
  of every qubit into key "m".
"""

from __future__ import annotations

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq


def _cirq():
    return ensure_cirq()


def random_layer_circuit(n: int, depth: int, seed: int = 0):
    cirq = _cirq()
    rs = np.random.RandomState(seed)
    q = cirq.LineQubit.range(n)
    moments = []
    for d in range(depth):
        layer = []
        for i in range(n):
            x, z, a = rs.uniform(-1, 1, size=3)
            layer.append(
                cirq.PhasedXZGate(x_exponent=x, z_exponent=z, axis_phase_exponent=a).on(q[i])
            )
        moments.append(cirq.Moment(layer))
        cz = [cirq.CZ(q[i], q[i + 1]) for i in range(d % 2, n - 1, 2)]
        if cz:
            moments.append(cirq.Moment(cz))
    return cirq.Circuit(moments)


def noisy_layer_circuit(n: int, depth: int, seed: int = 0, p: float = 1e-3, gamma: float = 5e-3):
    cirq = _cirq()
    base = random_layer_circuit(n, depth, seed)
    q = sorted(base.all_qubits())
    out = []
    layer_moments = list(base)
    for mi, moment in enumerate(layer_moments):
        out.append(moment)
        noise = [cirq.depolarize(p).on(qq) for op in moment for qq in op.qubits]
        out.append(cirq.Moment(noise))
        # a layer ends after its CZ moment (or after the 1q moment when it has no CZs)
        ends_layer = mi + 1 == len(layer_moments) or all(
            len(op.qubits) == 1 for op in layer_moments[mi + 1]
        )
        if ends_layer:
            out.append(cirq.Moment(cirq.amplitude_damp(gamma).on(qq) for qq in q))
    return cirq.Circuit(out)


def random_regular_graph_edges(n: int, seed: int, degree: int = 3) -> list[tuple[int, int]]:
    import networkx as nx

    g = nx.random_regular_graph(degree, n, seed=seed)
    return sorted(tuple(sorted(e)) for e in g.edges())


def qaoa_circuit(n: int, p: int = 4, seed: int = 0):
    """Returns (circuit, gamma symbols, beta symbols, observable, edges)."""
    cirq = _cirq()
    import sympy

    edges = random_regular_graph_edges(n, seed)
    q = cirq.LineQubit.range(n)
    gammas = [sympy.Symbol(f"gamma_{l}") for l in range(p)]
    betas = [sympy.Symbol(f"beta_{l}") for l in range(p)]
    moments = [cirq.Moment(cirq.H(x) for x in q)]
    for l in range(p):
        moments.append(cirq.Circuit(cirq.ZZPowGate(exponent=gammas[l]).on(q[i], q[j]) for i, j in edges))
        moments.append(cirq.Moment(cirq.XPowGate(exponent=betas[l]).on(x) for x in q))
    circuit = cirq.Circuit()
    for m in moments:
        circuit += m
    obs = sum(cirq.Z(q[i]) * cirq.Z(q[j]) for i, j in edges)
    return circuit, gammas, betas, obs, edges


def qaoa_points(p: int, count: int, seed: int = 0):
    """``count`` parameter points with gamma, beta ~ U(0, 1)."""
    rs = np.random.RandomState(seed)
    return rs.uniform(0, 1, size=(count, 2 * p))


def hea_circuit(n: int, layers: int, seed: int = 0):
    """Returns (circuit, symbols, values) for the rx/rz + CZ-ladder ansatz."""
    cirq = _cirq()
    import sympy

    rs = np.random.RandomState(seed)
    q = cirq.LineQubit.range(n)
    symbols = []
    moments = []
    for l in range(layers):
        rx_s = [sympy.Symbol(f"tx_{l}_{i}") for i in range(n)]
        rz_s = [sympy.Symbol(f"tz_{l}_{i}") for i in range(n)]
        symbols += rx_s + rz_s
        moments.append(cirq.Moment(cirq.rx(rx_s[i]).on(q[i]) for i in range(n)))
        moments.append(cirq.Moment(cirq.rz(rz_s[i]).on(q[i]) for i in range(n)))
        for i in range(n - 1):
            moments.append(cirq.Moment([cirq.CZ(q[i], q[i + 1])]))
    values = rs.uniform(-np.pi, np.pi, size=len(symbols))
    return cirq.Circuit(moments), symbols, values


def random_pauli_hamiltonian(n: int, terms: int, seed: int = 0, min_w: int = 2, max_w: int = 4):
    cirq = _cirq()
    rs = np.random.RandomState(seed)
    q = cirq.LineQubit.range(n)
    paulis = [cirq.X, cirq.Y, cirq.Z]
    total = cirq.PauliSum()
    for _ in range(terms):
        w = rs.randint(min_w, max_w + 1)
        qs = rs.choice(n, size=w, replace=False)
        ps = cirq.PauliString({q[int(i)]: paulis[rs.randint(3)] for i in qs}, coefficient=rs.normal())
        total += ps
    return total


def random_clifford_circuit(n: int, depth: int, seed: int = 0, *, mid_measure: float = 0.0,
                            resets: bool = False, feedback: bool = False, p: float = 0.0,
                            final_measure: bool = True):
    cirq = _cirq()
    rs = np.random.RandomState(seed)
    q = cirq.LineQubit.range(n)
    cliffords = cirq.SingleQubitCliffordGate.all_single_qubit_cliffords
    two = [cirq.CNOT, cirq.CZ, cirq.SWAP, cirq.ISWAP]
    moments = []
    nkeys = 0
    for d in range(depth):
        moments.append(cirq.Moment(cliffords[rs.randint(24)].on(x) for x in q))
        pairs = [two[rs.randint(len(two))].on(q[i], q[i + 1]) for i in range(d % 2, n - 1, 2)]
        if pairs:
            moments.append(cirq.Moment(pairs))
        if p > 0:
            moments.append(cirq.Moment(cirq.depolarize(p).on(x) for x in q))
        if mid_measure and rs.uniform() < mid_measure:
            a = int(rs.randint(n))
            key = f"k{nkeys}"
            moments.append(cirq.Moment(cirq.measure(q[a], key=key)))
            if feedback and nkeys > 0:
                b = int(rs.randint(n))
                moments.append(cirq.Moment(cirq.X(q[b]).with_classical_controls(f"k{nkeys - 1}")))
            if resets:
                moments.append(cirq.Moment(cirq.reset(q[a])))
            nkeys += 1
    if final_measure:
        moments.append(cirq.Moment(cirq.measure(*q, key="m")))
    return cirq.Circuit(moments)
