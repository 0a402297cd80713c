"""Stabilizer-tableau oracle for Clifford circuits -- TEST INFRASTRUCTURE ONLY.

Restates, in plain numpy, the Aaronson-Gottesman tableau that the reference
runs (cirq-core/cirq/qis/clifford_tableau.py):

* rows 0..n-1 destabilizers, n..2n-1 stabilizers, row 2n scratch
  (clifford_tableau.py:147-168);
* ``rowsum`` with the phase function g (clifford_tableau.py:457-481);
* ``measure`` (clifford_tableau.py:522-559);
* a gate acts on every row by conjugation.  Here the images of the single-
  qubit generators X_j and Z_j are taken from the gate's unitary and a row's
  image is their product, with the phases of the product tracked by g.  The
  reference applies its gates by hand-written updates
  (clifford_tableau.py:561-656); conjugation of a row is unique, so both give
  the same tableau.

``run_shot`` runs one repetition as ``StabilizerSampler._run`` does
(cirq-core/cirq/sim/clifford/stabilizer_sampler.py:52-70): the random
outcomes and noise come from a ``np.random.RandomState``.  ``choose`` lets a
test force the random outcomes (0 for the GPU reference run, or the
reference's recorded outcomes for pinning).

It is the checker, never the thing measured or shipped.
"""

from __future__ import annotations

import numpy as np

_P = {
    (0, 0): np.eye(2, dtype=np.complex128),
    (1, 0): np.array([[0, 1], [1, 0]], dtype=np.complex128),
    (1, 1): np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    (0, 1): np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def g(x1, z1, x2, z2):
    """Exponent of i in P(x1, z1) * P(x2, z2) (clifford_tableau.py:462-470)."""
    if not x1 and not z1:
        return 0
    if x1 and z1:
        return int(z2) - int(x2)
    if x1 and not z1:
        return int(z2) * (2 * int(x2) - 1)
    return int(x2) * (1 - 2 * int(z2))


def _local_pauli(xs, zs):
    m = np.eye(1, dtype=np.complex128)
    for x, z in zip(xs, zs):
        m = np.kron(m, _P[(int(x), int(z))])
    return m


_IMAGES: dict = {}


def _images(u: np.ndarray, k: int):
    """For each generator X_j (j < k) then Z_j: (x bits, z bits, exponent of i)
    of U g U^dagger (cached per matrix)."""
    key = (u.tobytes(), k)
    hit = _IMAGES.get(key)
    if hit is not None:
        return hit
    out = []
    basis = []
    for c in range(4 ** k):
        xs = [(c >> j) & 1 for j in range(k)]
        zs = [(c >> (k + j)) & 1 for j in range(k)]
        basis.append((xs, zs, _local_pauli(xs, zs)))
    ud = u.conj().T
    for kind in ("x", "z"):
        for j in range(k):
            xs = [1 if (kind == "x" and i == j) else 0 for i in range(k)]
            zs = [1 if (kind == "z" and i == j) else 0 for i in range(k)]
            q = u @ _local_pauli(xs, zs) @ ud
            for bx, bz, pm in basis:
                t = np.vdot(pm, q) / (2 ** k)
                if abs(abs(t) - 1) < 1e-9 and np.allclose(q, t * pm, atol=1e-9):
                    e = 0 if abs(t - 1) < 1e-9 else 2
                    out.append((np.array(bx, bool), np.array(bz, bool), e))
                    break
            else:
                raise ValueError("not a Clifford unitary")
    _IMAGES[key] = out
    return out


class Tableau:
    def __init__(self, n: int):
        self.n = n
        self.xs = np.zeros((2 * n + 1, n), dtype=bool)
        self.zs = np.zeros((2 * n + 1, n), dtype=bool)
        self.rs = np.zeros(2 * n + 1, dtype=bool)
        for i in range(n):
            self.xs[i, i] = True
            self.zs[n + i, i] = True

    def copy(self) -> "Tableau":
        t = Tableau.__new__(Tableau)
        t.n, t.xs, t.zs, t.rs = self.n, self.xs.copy(), self.zs.copy(), self.rs.copy()
        return t

    def rowsum(self, h: int, i: int) -> None:
        """Row h <- row i * row h (clifford_tableau.py:457-481)."""
        r = 2 * int(self.rs[h]) + 2 * int(self.rs[i])
        for j in range(self.n):
            r += g(self.xs[i, j], self.zs[i, j], self.xs[h, j], self.zs[h, j])
        r %= 4
        self.rs[h] = bool(r)
        self.xs[h, :] ^= self.xs[i, :]
        self.zs[h, :] ^= self.zs[i, :]

    def measure(self, q: int, choose) -> int:
        """clifford_tableau.py:522-559; choose() gives a random outcome."""
        n = self.n
        p = next((i for i in range(n, 2 * n) if self.xs[i, q]), None)
        if p is None:
            self.xs[2 * n, :] = False
            self.zs[2 * n, :] = False
            self.rs[2 * n] = False
            for i in range(n):
                if self.xs[i, q]:
                    self.rowsum(2 * n, n + i)
            return int(self.rs[2 * n])
        for i in range(2 * n):
            if i != p and self.xs[i, q]:
                self.rowsum(i, p)
        self.xs[p - n, :] = self.xs[p, :]
        self.zs[p - n, :] = self.zs[p, :]
        self.rs[p - n] = self.rs[p]
        self.xs[p, :] = False
        self.zs[p, :] = False
        self.zs[p, q] = True
        self.rs[p] = bool(choose())
        return int(self.rs[p])

    def apply_unitary(self, u: np.ndarray, qs) -> None:
        """Conjugates every row by u acting on qubits qs (qs[0] most significant)."""
        k = len(qs)
        imgs = _images(np.asarray(u, dtype=np.complex128), k)
        for row in range(2 * self.n):
            lx = [bool(self.xs[row, q]) for q in qs]
            lz = [bool(self.zs[row, q]) for q in qs]
            # P(lx, lz) = prod_j i^{x_j z_j} X_j^{x_j} Z_j^{z_j}; image = product of images
            e = 2 * int(self.rs[row])
            ax = np.zeros(k, bool)
            az = np.zeros(k, bool)
            for j in range(k):
                if lx[j] and lz[j]:
                    e += 1
                for on, (bx, bz, be) in ((lx[j], imgs[j]), (lz[j], imgs[k + j])):
                    if not on:
                        continue
                    e += be
                    for t in range(k):
                        e += g(ax[t], az[t], bx[t], bz[t])
                    ax ^= bx
                    az ^= bz
            e %= 4
            assert e in (0, 2), "image of a Hermitian Pauli must have a real sign"
            self.rs[row] = e == 2
            for t, q in enumerate(qs):
                self.xs[row, q] = ax[t]
                self.zs[row, q] = az[t]

    def apply_pauli(self, xs, zs, qs) -> None:
        """Pauli P on qubits qs: rows anticommuting with P change sign."""
        for row in range(2 * self.n):
            anti = 0
            for t, q in enumerate(qs):
                anti ^= (bool(xs[t]) and bool(self.zs[row, q])) ^ (bool(zs[t]) and bool(self.xs[row, q]))
            if anti:
                self.rs[row] = not self.rs[row]


def run_shot(ops, n: int, nrec: int, prng: np.random.RandomState | None = None, choose=None):
    """One repetition of a program given as a list of plain tuples:
    ("u", unitary, qubits) | ("m", qubit, record, invert) | ("r", qubit) |
    ("noise", qubit, (px, py, pz)) | ("cp", xs, zs, qubits, records).
    Returns the records (uint8).  Random outcomes: choose(record) if given,
    else prng; noise is drawn from prng (skipped when prng is None)."""
    t = Tableau(n)
    rec = np.zeros(nrec, np.uint8)
    for op in ops:
        kind = op[0]
        if kind == "u":
            t.apply_unitary(op[1], op[2])
        elif kind == "m":
            _, q, r, inv = op
            pick = (lambda: choose(r)) if choose is not None else (lambda: prng.randint(2))
            rec[r] = t.measure(q, pick) ^ int(inv)
        elif kind == "r":
            q = op[1]
            pick = (lambda: 0) if choose is not None else (lambda: prng.randint(2))
            if t.measure(q, pick):
                t.apply_pauli([1], [0], [q])
        elif kind == "noise":
            if prng is None:
                continue
            q, (px, py, pz) = op[1], op[2]
            u = prng.random_sample()
            if u < px:
                t.apply_pauli([1], [0], [q])
            elif u < px + py:
                t.apply_pauli([1], [1], [q])
            elif u < px + py + pz:
                t.apply_pauli([0], [1], [q])
        elif kind == "cp":
            _, xs, zs, qs, recs = op
            if any(rec[r] for r in recs):
                t.apply_pauli(xs, zs, qs)
        else:
            raise ValueError(kind)
    return rec, t


def program_from_circuit(cirq, circuit, qubits):
    """(ops, nrec, keys) for run_shot from a circuit (the oracle's own
    translation of the operations the reference's stabilizer simulation
    accepts: unitaries by matrix, measurements, resets, one-qubit Pauli
    mixtures and Paulis conditioned on a measurement key)."""
    index = {q: i for i, q in enumerate(qubits)}
    ops, keys, nrec = [], {}, 0
    for op in circuit.all_operations():
        if isinstance(op, cirq.ClassicallyControlledOperation):
            (cond,) = op.classical_controls
            sub = op.without_classical_controls()
            u = np.asarray(cirq.unitary(sub), dtype=np.complex128)
            k = len(sub.qubits)
            for c in range(4 ** k):
                xs = [(c >> j) & 1 for j in range(k)]
                zs = [(c >> (k + j)) & 1 for j in range(k)]
                pm = _local_pauli(xs, zs)
                t = np.vdot(pm, u) / (2 ** k)
                if abs(abs(t) - 1) < 1e-9 and np.allclose(u, t * pm, atol=1e-9):
                    break
            else:
                raise ValueError("conditioned operation is not a Pauli")
            ops.append(("cp", xs, zs, [index[q] for q in sub.qubits], keys[str(cond.key)][-1]))
            continue
        gate = getattr(op, "gate", None)
        if isinstance(gate, cirq.MeasurementGate):
            inv = gate.full_invert_mask()
            recs = []
            for j, q in enumerate(op.qubits):
                ops.append(("m", index[q], nrec, bool(inv[j])))
                recs.append(nrec)
                nrec += 1
            keys.setdefault(cirq.measurement_key_name(op), []).append(recs)
            continue
        if isinstance(gate, cirq.ResetChannel):
            ops.extend(("r", index[q]) for q in op.qubits)
            continue
        if cirq.has_unitary(op):
            if op.qubits:
                ops.append(("u", np.asarray(cirq.unitary(op), dtype=np.complex128), [index[q] for q in op.qubits]))
            continue
        probs = {(1, 0): 0.0, (1, 1): 0.0, (0, 1): 0.0}
        for p, m in cirq.mixture(op):
            for key, pm in _P.items():
                t = np.vdot(pm, m) / 2
                if abs(abs(t) - 1) < 1e-9 and np.allclose(m, t * pm, atol=1e-9):
                    if key != (0, 0):
                        probs[key] += p
                    break
            else:
                raise ValueError("noise is not a Pauli mixture")
        ops.append(("noise", index[op.qubits[0]], (probs[(1, 0)], probs[(1, 1)], probs[(0, 1)])))
    return ops, nrec, keys
