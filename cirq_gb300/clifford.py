"""Clifford circuits on the GPU: one tableau run and Pauli-frame shots.

Drop-ins for the reference's stabilizer samplers:

* :class:`StabilizerSampler` for ``cirq.StabilizerSampler``
  (cirq-core/cirq/sim/clifford/stabilizer_sampler.py:24-70), which re-runs the
  circuit on a ``CliffordTableau`` once per repetition;
* :class:`CliffordSimulator` for ``cirq.CliffordSimulator``
  (cirq-core/cirq/sim/clifford/clifford_simulator.py:46-117): ``run`` /
  ``run_sweep`` sample on the GPU; ``simulate`` and the step API keep the
  reference class's own CH-form state (this class inherits them).

A circuit is compiled once per structure (:class:`CliffordProgram`) into
``gbq_cliff_op`` records (include/cirq_gb300.h):

* a unitary on up to 3 qubits becomes its Pauli-conjugation table, taken from
  its matrix (``U P U^dagger`` for every Pauli ``P`` on its qubits), and the
  GF(2) frame map of that table;
* a measurement becomes one record per measured qubit (inversions kept);
* a reset stays a reset;
* a mixture of Pauli unitaries on one qubit (``depolarize``, ``bit_flip``,
  ``phase_flip``, ``asymmetric_depolarize``) becomes Pauli noise;
* a Pauli conditioned on a measurement key is kept as a conditioned Pauli.

``gbq_cliff_reference`` runs the program once on a GPU tableau (random
outcomes take 0, noise is skipped), and ``gbq_cliff_sample`` propagates one
Pauli frame per shot against that run, 32 shots per thread.  Records come
back bit-packed and are unpacked here into the reference's result shapes.

A circuit that does not fit these forms (a non-Clifford gate, a confusion
map, a condition other than a measurement key, noise that is not a Pauli
mixture on one qubit) raises :class:`NotFrameable`; the drop-ins then run it
on :class:`cirq_gb300.Simulator` when its qubits fit a state vector.
"""

from __future__ import annotations

import ctypes
import functools
import itertools
from collections.abc import Sequence
from typing import Any

import numpy as np

from cirq_gb300 import _lib
from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300._lib import check

cirq = ensure_cirq()
from cirq.sim.simulator import check_all_resolved  # noqa: E402  (the reference's own check)

#: widest circuit that a non-frameable circuit may still run on the
#: state-vector simulator
STATE_VECTOR_MAX_QUBITS = 30


class NotFrameable(ValueError):
    """The circuit has an operation that Pauli-frame sampling cannot take."""


_PAULI = {
    (0, 0): np.eye(2, dtype=np.complex128),
    (1, 0): np.array([[0, 1], [1, 0]], dtype=np.complex128),
    (1, 1): np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    (0, 1): np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def _pauli_string(xbits: int, zbits: int, k: int) -> np.ndarray:
    """Hermitian Pauli string on k qubits (qubit 0 most significant, as in
    ``cirq.unitary`` of an operation), Y where x = z = 1."""
    m = np.eye(1, dtype=np.complex128)
    for j in range(k):
        m = np.kron(m, _PAULI[((xbits >> j) & 1, (zbits >> j) & 1)])
    return m


@functools.lru_cache(maxsize=None)
def _pauli_basis(k: int) -> tuple:
    return tuple(_pauli_string(i & ((1 << k) - 1), i >> k, k) for i in range(1 << (2 * k)))


def conjugation_table(u: np.ndarray, k: int) -> tuple[list[int], list[int]]:
    """(table, lin) of a k-qubit unitary: table[x | z << k] = x' | z' << k |
    sign << 2k with U P(x, z) U^dagger = (-1)^sign P(x', z'), and lin[o] the
    input bits whose XOR is output bit o of the frame map.  Raises
    NotFrameable if U is not a Clifford."""
    basis = _pauli_basis(k)
    d = 1 << k
    table = []
    ud = u.conj().T
    for idx, p in enumerate(basis):
        q = u @ p @ ud
        found = None
        if idx == 0:
            found = (0, 0)
        else:
            # candidates by the support of q's entries (one nonzero per row)
            for c, pc in enumerate(basis):
                t = np.vdot(pc, q).real / d
                if abs(abs(t) - 1.0) < 1e-6 and np.allclose(q, np.sign(t) * pc, atol=1e-6):
                    found = (c, 1 if t < 0 else 0)
                    break
        if found is None:
            raise NotFrameable("not a Clifford operation")
        c, s = found
        table.append(c | (s << (2 * k)))
    lin = [0] * (2 * k)
    for b in range(2 * k):
        img = table[1 << b] & ((1 << (2 * k)) - 1)
        for o in range(2 * k):
            if (img >> o) & 1:
                lin[o] |= 1 << b
    # linearity of the frame map (guards against a bad table)
    for idx in range(1 << (2 * k)):
        want = 0
        for b in range(2 * k):
            if (idx >> b) & 1:
                want ^= table[1 << b] & ((1 << (2 * k)) - 1)
        if want != table[idx] & ((1 << (2 * k)) - 1):
            raise NotFrameable("not a Clifford operation")
    return table, lin


@functools.lru_cache(maxsize=4096)
def _table_cached(key: bytes, k: int) -> tuple[tuple[int, ...], tuple[int, ...]]:
    u = np.frombuffer(key, dtype=np.complex128).reshape(1 << k, 1 << k)
    t, lin = conjugation_table(u, k)
    return tuple(t), tuple(lin)


def _unitary_table(u: np.ndarray, k: int):
    u = np.asarray(u, dtype=np.complex128)
    # a global phase does not change the conjugation: normalise it so that
    # equal gates share one cache entry
    flat = u.reshape(-1)
    j = int(np.argmax(np.abs(flat) > 1e-9))
    u = u * (abs(flat[j]) / flat[j])
    return _table_cached(np.round(u, 12).astype(np.complex128).tobytes(), k)


def _pauli_noise(op) -> tuple[float, float, float] | None:
    """(px, py, pz) of a one-qubit mixture of Pauli unitaries, else None."""
    if len(op.qubits) != 1 or cirq.has_unitary(op):
        return None
    mix = cirq.mixture(op, None)
    if mix is None:
        return None
    probs = {"x": 0.0, "y": 0.0, "z": 0.0, "i": 0.0}
    for p, m in mix:
        m = np.asarray(m, dtype=np.complex128)
        for name, (x, z) in (("i", (0, 0)), ("x", (1, 0)), ("y", (1, 1)), ("z", (0, 1))):
            pm = _PAULI[(x, z)]
            t = np.vdot(pm, m) / 2
            if abs(abs(t) - 1) < 1e-9 and np.allclose(m, t * pm, atol=1e-9):
                probs[name] += float(p)
                break
        else:
            return None
    return probs["x"], probs["y"], probs["z"]


class CliffordProgram:
    """A circuit compiled into ``gbq_cliff_op`` records (see module doc).

    ``keys`` maps each measurement key to the record indices of its
    measurements, one list per instance, in circuit order."""

    def __init__(self, circuit: cirq.AbstractCircuit, qubits: Sequence[Any] | None = None):
        self.qubits = tuple(qubits) if qubits is not None else tuple(sorted(circuit.all_qubits()))
        self.index = {q: i for i, q in enumerate(self.qubits)}
        if any(q.dimension != 2 for q in self.qubits):
            raise NotFrameable("only qubits can be sampled by Pauli frames")
        self._ops: list[tuple] = []
        self._tables: list[int] = []
        self._table_at: dict = {}
        self._conds: list[int] = []
        self._gates: dict = {}  # gate -> ("u", table offset, lin, k) | ("id",) | ("noise", p)
        self.keys: dict[str, list[list[int]]] = {}
        self.nrec = 0
        for op in circuit.all_operations():
            self._add(op, depth=0)
        self._build()
        self._ref: np.ndarray | None = None

    def _emit(self, kind, qs, tab=0, rec=0, lin=(), cond=(0, 0), p=()) -> None:
        self._ops.append((kind, len(qs), tuple(qs), tab, rec, tuple(lin), cond, tuple(p)))

    def _build(self) -> None:
        """Op records in layers of ops on disjoint qubits (an op's layer is
        one past the last layer of its qubits and of the records it reads);
        circuit order within a layer."""
        nq = len(self.qubits)
        qlayer = [-1] * nq
        rlayer = [-1] * max(self.nrec, 1)
        layer_of = []
        for kind, k, qs, tab, rec, lin, cond, p in self._ops:
            L = max(qlayer[q] for q in qs) + 1
            if kind == _lib.CLIFF_COND_PAULI:
                for r in self._conds[cond[0]: cond[0] + cond[1]]:
                    L = max(L, rlayer[r] + 1)
            for q in qs:
                qlayer[q] = L
            if kind == _lib.CLIFF_MEASURE:
                rlayer[rec] = L
            layer_of.append(L)
        order = sorted(range(len(self._ops)), key=lambda i: layer_of[i])
        n = len(self._ops)
        ops = np.zeros(max(n, 1), dtype=_lib.CLIFF_OP_DTYPE)[:n]
        if n:
            src = [self._ops[i] for i in order]
            ops["kind"] = [t[0] for t in src]
            ops["k"] = [t[1] for t in src]
            ops["q"] = [t[2] + (0,) * (3 - len(t[2])) for t in src]
            ops["tab"] = [t[3] for t in src]
            ops["rec"] = [t[4] for t in src]
            ops["lin"] = [t[5] + (0,) * (6 - len(t[5])) for t in src]
            ops["cond_begin"] = [t[6][0] for t in src]
            ops["cond_count"] = [t[6][1] for t in src]
            ops["p"] = [t[7] + (0.0,) * (3 - len(t[7])) for t in src]
        self.ops = ops
        counts = np.bincount(np.asarray(layer_of, dtype=np.int64), minlength=1) if n else np.zeros(0, np.int64)
        self.layers = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        self.nlayers = len(self.layers) - 1
        self.tables = np.asarray(self._tables or [0], dtype=np.uint32)
        self.conds = np.asarray(self._conds or [0], dtype=np.int32)
        self.nconds = len(self._conds)

    # ---- compilation ----------------------------------------------------
    def _table(self, table, k) -> int:
        key = (tuple(table), k)
        at = self._table_at.get(key)
        if at is None:
            at = len(self._tables)
            self._tables.extend(table)
            self._table_at[key] = at
        return at

    def _qidx(self, op) -> list[int]:
        return [self.index[q] for q in op.qubits]

    def _add(self, op, depth: int) -> None:
        if depth > 8:
            raise NotFrameable(f"cannot decompose {op!r} into frameable operations")
        if isinstance(op, cirq.ClassicallyControlledOperation):
            self._add_conditioned(op)
            return
        gate = getattr(op, "gate", None)
        if isinstance(gate, cirq.MeasurementGate):
            if gate.confusion_map:
                raise NotFrameable("measurement confusion maps are not sampled by Pauli frames")
            inv = gate.full_invert_mask()
            recs = []
            for j, q in enumerate(self._qidx(op)):
                rec = self.nrec
                self.nrec += 1
                recs.append(rec)
                self._emit(_lib.CLIFF_MEASURE, (q,), rec=rec, lin=(int(bool(inv[j])),))
            self.keys.setdefault(cirq.measurement_key_name(op), []).append(recs)
            return
        if isinstance(gate, cirq.ResetChannel):
            for q in self._qidx(op):
                self._emit(_lib.CLIFF_RESET, (q,))
            return
        if not op.qubits:
            if cirq.has_unitary(op):
                return  # a global phase changes no sample
            raise NotFrameable(f"operation without qubits: {op!r}")
        hit = self._gates.get(gate) if gate is not None and len(op.qubits) <= 3 else None
        if hit is None and gate is not None and len(op.qubits) <= 3:
            hit = self._classify(op)
            if hit is not None:
                try:
                    self._gates[gate] = hit
                except TypeError:  # an unhashable gate
                    pass
        if hit is not None:
            if hit[0] == "u":
                self._emit(_lib.CLIFF_UNITARY, self._qidx(op), tab=hit[1], lin=hit[2])
            elif hit[0] == "noise":
                self._emit(_lib.CLIFF_NOISE, self._qidx(op), p=hit[1])
            return
        if cirq.has_unitary(op):
            k = len(op.qubits)
            if k <= 3:
                u = cirq.unitary(op)
                if np.allclose(u, u[0, 0] * np.eye(u.shape[0]), atol=1e-12):
                    return
                table, lin = _unitary_table(u, k)
                self._emit(_lib.CLIFF_UNITARY, self._qidx(op), tab=self._table(table, k), lin=lin)
                return
        else:
            noise = _pauli_noise(op)
            if noise is not None:
                if sum(noise) > 0:
                    self._emit(_lib.CLIFF_NOISE, self._qidx(op), p=noise)
                return
            if cirq.is_measurement(op):
                raise NotFrameable(f"measurement-like operation {op!r} is not sampled by Pauli frames")
        sub = cirq.decompose_once(op, None)
        if sub is None:
            raise NotFrameable(f"{op!r} is not a Clifford operation on at most 3 qubits")
        for s in sub:
            self._add(s, depth + 1)

    def _classify(self, op):
        """("u", table offset, lin) / ("id",) / ("noise", p) for a gate
        operation on at most 3 qubits that frames take directly, else None."""
        k = len(op.qubits)
        if cirq.has_unitary(op):
            u = cirq.unitary(op)
            if np.allclose(u, u[0, 0] * np.eye(u.shape[0]), atol=1e-12):
                return ("id",)
            try:
                table, lin = _unitary_table(u, k)
            except NotFrameable:
                return None
            return ("u", self._table(table, k), lin)
        noise = _pauli_noise(op)
        if noise is None:
            return None
        return ("noise", noise) if sum(noise) > 0 else ("id",)

    def _add_conditioned(self, op) -> None:
        conds = op.classical_controls
        sub = op.without_classical_controls()
        if len(conds) != 1 or not isinstance(next(iter(conds)), cirq.KeyCondition):
            raise NotFrameable("only single measurement-key conditions are sampled by Pauli frames")
        cond = next(iter(conds))
        key = str(cond.key)
        if key not in self.keys:
            raise NotFrameable(f"condition on key {key!r} before its measurement")
        k = len(sub.qubits)
        if k > 3 or not cirq.has_unitary(sub):
            raise NotFrameable("only Pauli operations can be conditioned")
        u = np.asarray(cirq.unitary(sub), dtype=np.complex128)
        xb = zb = None
        for xs, zs in itertools.product(range(1 << k), repeat=2):
            p = _pauli_string(xs, zs, k)
            t = np.vdot(p, u) / (1 << k)
            if abs(abs(t) - 1) < 1e-9 and np.allclose(u, t * p, atol=1e-9):
                xb, zb = xs, zs
                break
        if xb is None:
            raise NotFrameable("only Pauli operations can be conditioned")
        table, _ = _unitary_table(u, k)
        recs = self.keys[key][-1]
        begin = len(self._conds)
        self._conds.extend(recs)
        lin = [((xb >> j) & 1) | (((zb >> j) & 1) << 1) for j in range(k)]
        self._emit(_lib.CLIFF_COND_PAULI, self._qidx(sub), tab=self._table(table, k), lin=lin,
                   cond=(begin, len(recs)))

    # ---- device -----------------------------------------------------------
    def validate(self, lib) -> None:
        check(lib.gbq_cliff_validate(len(self.qubits), self.ops.ctypes.data, len(self.ops), len(self.tables),
                                     self.nconds, self.nrec), "gbq_cliff_validate")

    def reference(self, eng) -> np.ndarray:
        """Records of the program's reference run (random outcomes 0)."""
        if self._ref is None:
            ref = np.zeros(max(self.nrec, 1), dtype=np.uint8)
            check(eng.lib.gbq_cliff_reference(
                eng.ctx, len(self.qubits), self.ops.ctypes.data, len(self.ops), self.tables.ctypes.data,
                len(self.tables), self.conds.ctypes.data, self.nconds, self.nrec, ref.ctypes.data),
                "gbq_cliff_reference")
            self._ref = ref[: self.nrec]
        return self._ref

    def _sample(self, eng, repetitions: int, seed: int, out_bytes: bool) -> np.ndarray:
        ref = self.reference(eng)
        nw = (repetitions + 31) // 32
        if out_bytes:
            out = np.zeros((repetitions, max(self.nrec, 1)), dtype=np.uint8)
        else:
            out = np.zeros((max(self.nrec, 1), nw), dtype=np.uint32)
        refbuf = np.ascontiguousarray(ref if self.nrec else np.zeros(1, np.uint8))
        check(eng.lib.gbq_cliff_sample(
            eng.ctx, len(self.qubits), self.ops.ctypes.data, len(self.ops), self.tables.ctypes.data,
            len(self.tables), self.conds.ctypes.data, self.nconds, refbuf.ctypes.data, self.nrec,
            ctypes.c_int64(repetitions), ctypes.c_uint64(seed & ((1 << 64) - 1)), out.ctypes.data,
            self.layers.ctypes.data, self.nlayers, int(out_bytes)),
            "gbq_cliff_sample")
        return out

    def sample_words(self, eng, repetitions: int, seed: int) -> np.ndarray:
        """(nrec, ceil(repetitions / 32)) uint32: record r's bit of shot j is
        bit j % 32 of word j // 32."""
        return self._sample(eng, repetitions, seed, False)[: self.nrec]

    def sample_records(self, eng, repetitions: int, seed: int) -> np.ndarray:
        """(repetitions, nrec) uint8 outcomes (transposed on the device)."""
        return self._sample(eng, repetitions, seed, True)[:, : self.nrec]

    def records(self, eng, repetitions: int, seed: int) -> dict[str, np.ndarray]:
        """{key: (repetitions, instances, bits)} as ``SimulatorBase._run`` returns;
        a key measured once with consecutive records is a view of the samples."""
        rec = self.sample_records(eng, repetitions, seed)
        out = {}
        for key, insts in self.keys.items():
            if len(insts) == 1 and insts[0] == list(range(insts[0][0], insts[0][0] + len(insts[0]))):
                lo = insts[0][0]
                out[key] = rec[:, None, lo: lo + len(insts[0])]
                continue
            width = max(len(r) for r in insts)
            arr = np.zeros((repetitions, len(insts), width), dtype=np.uint8)
            for i, r in enumerate(insts):
                arr[:, i, : len(r)] = rec[:, r]
            out[key] = arr
        return out


def _seed_from(prng: np.random.RandomState) -> int:
    return int(prng.randint(0, 2**62, dtype=np.int64))


_PROGRAMS: dict = {}


def compile_program(circuit: cirq.AbstractCircuit, qubits=None) -> CliffordProgram:
    """CliffordProgram of a resolved circuit, cached per circuit and qubit order."""
    frozen = circuit if isinstance(circuit, cirq.FrozenCircuit) else cirq.FrozenCircuit(circuit)
    key = (frozen, tuple(qubits) if qubits is not None else None)
    prog = _PROGRAMS.get(key)
    if prog is None:
        prog = CliffordProgram(circuit, qubits)
        if len(_PROGRAMS) > 256:
            _PROGRAMS.clear()
        _PROGRAMS[key] = prog
    return prog


def _engine():
    from cirq_gb300.engine import Engine

    return Engine.get(0)


class StabilizerSampler(cirq.Sampler):
    """``cirq.StabilizerSampler`` with the repetitions as Pauli frames on the
    GPU (module doc).  Results keep the reference's shapes: each key's last
    measurement, (repetitions, bits) uint8."""

    def __init__(self, *, seed: cirq.RANDOM_STATE_OR_SEED_LIKE = None):
        self._prng = cirq.value.parse_random_state(seed)

    def run_sweep(self, program: cirq.AbstractCircuit, params: cirq.Sweepable,
                  repetitions: int = 1) -> Sequence[cirq.Result]:
        results = []
        for resolver in cirq.to_resolvers(params):
            circuit = cirq.resolve_parameters(program, resolver)
            results.append(cirq.ResultDict(params=resolver, measurements=self._run(circuit, repetitions)))
        return results

    def _run(self, circuit: cirq.AbstractCircuit, repetitions: int) -> dict[str, np.ndarray]:
        keys = cirq.measurement_key_names(circuit)
        qubits = list(circuit.all_qubits())
        try:
            prog = compile_program(circuit, qubits)
        except NotFrameable:
            if len(qubits) > STATE_VECTOR_MAX_QUBITS:
                raise
            return _state_vector_last(circuit, repetitions, self._prng, keys)
        eng = _engine()
        recs = prog.records(eng, repetitions, _seed_from(self._prng))
        return {k: (recs[k][:, -1, :] if k in recs else np.zeros((repetitions, 0), np.uint8)) for k in keys}


def _state_vector_last(circuit, repetitions, prng, keys) -> dict[str, np.ndarray]:
    """Each key's last measurement from the GPU state-vector simulator."""
    import cirq_gb300

    res = cirq_gb300.Simulator(seed=prng).run(circuit, repetitions=repetitions)
    return {k: np.asarray(res.records[k][:, -1, :], dtype=np.uint8) for k in keys}


class CliffordSimulator(cirq.CliffordSimulator):
    """``cirq.CliffordSimulator`` whose ``run`` / ``run_sweep`` sample all
    repetitions as Pauli frames on the GPU (module doc); ``simulate`` and the
    step API are the reference class's own (CH-form states)."""

    def _run(self, circuit: cirq.AbstractCircuit, param_resolver: cirq.ParamResolver,
             repetitions: int) -> dict[str, np.ndarray]:
        param_resolver = param_resolver or cirq.ParamResolver({})
        resolved = cirq.resolve_parameters(circuit, param_resolver)
        check_all_resolved(resolved)
        qubits = cirq.QubitOrder.DEFAULT.order_for(resolved.all_qubits())
        try:
            prog = compile_program(resolved, qubits)
        except NotFrameable:
            if len(qubits) > STATE_VECTOR_MAX_QUBITS:
                raise
            import cirq_gb300

            res = cirq_gb300.Simulator(seed=self._prng).run(resolved, repetitions=repetitions)
            return {k: np.asarray(v, dtype=np.uint8) for k, v in res.records.items()}
        return prog.records(_engine(), repetitions, _seed_from(self._prng))


def is_clifford_circuit(program: cirq.AbstractCircuit) -> bool:
    """The reference's routing test (cirq-core/cirq/sim/mux.py:336-339): every
    non-measurement operation has a stabilizer effect."""
    return all(cirq.has_stabilizer_effect(op) for op in program.all_operations() if not cirq.is_measurement(op))
