"""Circuits compiled once, evaluated for many parameter points.

A :class:`CompiledCircuit` holds the structure of a (possibly parameterised)
circuit over a fixed qubit order: its BitGates, the plan of passes/ops, and
for every BitGate an evaluator that produces its matrices for a batch of
``cirq.ParamResolver`` points.  Evaluating a sweep therefore costs one plan
plus vectorised numpy per point, instead of the reference's per-point
``resolve_parameters`` + per-operation dispatch
(``cirq-core/cirq/sim/simulator.py:558-640``,
``cirq-core/cirq/protocols/resolve_parameters.py:137-199``).

EigenGates with a symbolic exponent (XPow/YPow/ZPow/CZPow/ZZPow/Rx/Ry/Rz,
...) are evaluated from their eigen-decomposition, U(t) = sum_k
exp(i pi t (h_k + s)) P_k, which is the formula of ``EigenGate._unitary_``
(``cirq-core/cirq/ops/eigen_gate.py:295-305``); any other parameterised
operation falls back to resolving it and calling ``cirq.unitary``/``cirq.kraus``
per point.
"""

from __future__ import annotations

import dataclasses
from typing import Any, Sequence

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.ir import BitGate, UnsupportedOperation, is_diagonal
from cirq_gb300.planner import MIN_TILE_BITS, Plan, Planner


def _cirq():
    return ensure_cirq()


@dataclasses.dataclass(frozen=True)
class Slot:
    """An operation whose matrix each trajectory chooses (a sampled mixture
    unitary or a rescaled Kraus operator).  Its matrix comes from the
    ``picks`` of a :class:`TrajectoryPoint`; it is planned as a dense op."""

    op: Any
    slot: int

    @property
    def qubits(self):
        return self.op.qubits


class TrajectoryPoint:
    """A ParamResolver plus the matrices one trajectory picked for its slots."""

    def __init__(self, base, picks: dict):
        self.base = base
        self.picks = picks

    def value_of(self, value, recursive: bool = True):
        return self.base.value_of(value, recursive)

    @property
    def param_dict(self):
        return self.base.param_dict


def _generic_unitary(d: int) -> np.ndarray:
    """A fixed dense unitary (plans a slot as a dense op)."""
    rs = np.random.RandomState(4321 + d)
    q, _ = np.linalg.qr(rs.normal(size=(d, d)) + 1j * rs.normal(size=(d, d)))
    return q


_EXPR_FORMS: dict = {}  # sympy expression -> how to evaluate it (see _expr_form)


def _expr_form(expr):
    """("sym", s) | ("lin", c, s) for c * s | ("const", v) | ("fn", f, symbols)
    with f a ``sympy.lambdify`` function, cached per expression."""
    form = _EXPR_FORMS.get(expr)
    if form is not None:
        return form
    import sympy

    if isinstance(expr, sympy.Symbol):
        form = ("sym", expr)
    elif not getattr(expr, "free_symbols", None):
        form = ("const", float(expr))
    else:
        coeff, rest = expr.as_coeff_Mul()
        num, den = sympy.fraction(expr)
        ncoeff, nrest = num.as_coeff_Mul()
        if isinstance(rest, sympy.Symbol) and coeff.is_number:
            form = ("lin", float(coeff), rest)
        elif den.is_number and den != 1 and isinstance(nrest, sympy.Symbol) and ncoeff.is_number:
            # c * s / d (rx(t) gives t / pi): evaluated as (c * s) / d, kept
            # only where that gives the lambdified expression's bits
            form = ("div", float(ncoeff), float(den), nrest)
            fn = sympy.lambdify((nrest,), expr, "numpy")
            probe = np.random.RandomState(77).normal(size=16) * 4.0
            want = np.array([float(fn(float(v))) for v in probe])
            got = (form[1] * probe if form[1] != 1.0 else probe) / form[2]
            if not np.array_equal(got.view(np.int64), want.view(np.int64)):
                form = ("fn", fn, (nrest,))
        else:
            syms = tuple(sorted(expr.free_symbols, key=str))
            form = ("fn", sympy.lambdify(syms, expr, "numpy"), syms)
    if len(_EXPR_FORMS) > 4096:
        _EXPR_FORMS.clear()
    _EXPR_FORMS[expr] = form
    return form


def _expr_values(expr, resolvers, values: dict | None) -> np.ndarray:
    """Per-resolver float values of an exponent expression.

    Free symbols are resolved by each resolver (value_of, so symbol-to-symbol
    mappings resolve as in the reference) once per batch; the expression is
    then evaluated from those values (a constant times a symbol directly,
    anything else by a cached ``sympy.lambdify`` function) rather than by
    sympy substitution per resolver.  `values` caches results across the
    sources of one batch."""
    if values is not None:
        v = values.get(expr)
        if v is not None:
            return v
    form = _expr_form(expr)
    if form[0] == "sym":
        v = np.array([float(r.value_of(expr)) for r in resolvers])
    elif form[0] == "const":
        v = np.full(len(resolvers), form[1])
    elif form[0] == "lin":
        v = form[1] * _expr_values(form[2], resolvers, values)
    elif form[0] == "div":
        v = _expr_values(form[3], resolvers, values)
        v = (v if form[1] == 1.0 else form[1] * v) / form[2]
    else:
        args = [_expr_values(x, resolvers, values) for x in form[2]]
        v = np.broadcast_to(np.asarray(form[1](*args), dtype=np.float64), (len(resolvers),)).copy()
    if values is not None:
        values[expr] = v
    return v


def _linear_exponents(exprs):
    """(symbols, index, coef, div, const) when every expression is a
    constant, a symbol, or a constant times a symbol over a constant (index
    -1 for constants), else None."""
    forms = [_expr_form(e) for e in exprs]
    if not all(f[0] in ("sym", "lin", "div", "const") for f in forms):
        return None
    syms: list = []
    pos: dict = {}
    index = np.full(len(forms), -1, dtype=np.int64)
    coef = np.ones(len(forms))
    div = np.ones(len(forms))
    const = np.zeros(len(forms))
    for j, f in enumerate(forms):
        if f[0] == "const":
            const[j] = f[1]
            continue
        sym = f[1] if f[0] == "sym" else f[2] if f[0] == "lin" else f[3]
        if f[0] in ("lin", "div"):
            coef[j] = f[1]
        if f[0] == "div":
            div[j] = f[2]
        if sym not in pos:
            pos[sym] = len(syms)
            syms.append(sym)
        index[j] = pos[sym]
    return syms, index, coef, div, const


# values that ParamResolver.value_of returns as the same number
_PLAIN_NUMBERS = frozenset({float, int, np.float64, np.float32, np.int64, np.int32})


def _symbol_values(syms, resolvers) -> np.ndarray:
    """(len(syms), P) values of plain symbols.  A symbol whose name maps to a
    float or int (Python or numpy) in the resolver's dictionary takes that
    number (what ParamResolver.value_of returns for it); anything else goes
    through value_of."""
    import sympy

    out = np.empty((len(syms), len(resolvers)))
    for p, r in enumerate(resolvers):
        byname = {(k.name if isinstance(k, sympy.Symbol) else k): v for k, v in r.param_dict.items()}
        for j, sym in enumerate(syms):
            v = byname.get(sym.name)
            if type(v) in _PLAIN_NUMBERS:
                out[j, p] = v
            else:
                out[j, p] = float(r.value_of(sym))
    return out


@dataclasses.dataclass
class OpSource:
    """How to produce one BitGate's matrix for a batch of resolvers."""

    op: Any
    transform: str  # 'u' (unitary), 'conj' (conjugate unitary), 'superop'
    const: np.ndarray | None  # constant matrix (unparameterised ops)
    eigen: tuple | None  # (components [(h, P)], shift, exponent expr) for EigenGates
    slot: int | None = None  # trajectory slot: the matrix is the resolver's pick

    def matrices(self, resolvers: Sequence[Any], values: dict | None = None) -> np.ndarray:
        """(P, d, d) matrices; `values` caches expression -> per-resolver
        values across the sources of one batch (gates sharing a symbol)."""
        P = len(resolvers)
        if self.const is not None:
            return self.const[None] if P == 1 else np.broadcast_to(self.const, (P,) + self.const.shape)
        if self.slot is not None:
            d = 2 ** len(self.op.qubits)
            mats = []
            for r in resolvers:
                m = getattr(r, "picks", {}).get(self.slot)
                mats.append(_generic_unitary(d) if m is None else np.asarray(m, dtype=np.complex128))
            return np.array(mats)
        cirq = _cirq()
        resolvers = [getattr(r, "base", r) for r in resolvers]
        if self.eigen is not None:
            comps, shift, expr = self.eigen
            t = _expr_values(expr, resolvers, values)
            out = 0
            for h, proj in comps:
                out = out + np.exp(1j * np.pi * t * (h + shift))[:, None, None] * proj[None]
            return self._finish(np.asarray(out, dtype=np.complex128))
        mats = []
        for r in resolvers:
            op = cirq.resolve_parameters(self.op, r)
            if self.transform == "superop":
                ks = cirq.kraus(op)
                mats.append(sum(np.kron(np.conjugate(k), k) for k in ks))
            else:
                mats.append(np.asarray(cirq.unitary(op), dtype=np.complex128))
        return self._finish(np.array(mats))

    def _finish(self, m: np.ndarray) -> np.ndarray:
        if self.transform == "conj":
            return np.conjugate(m)
        if self.transform == "phase":  # (P, 1, 1) scalar -> scalar * I_2
            return m.reshape(-1, 1, 1) * np.eye(2)[None]
        return m

    def derivatives(self, resolvers: Sequence[Any], symbol, values: dict | None = None) -> np.ndarray | None:
        """dU/d(symbol) for every resolver (P, d, d), or None if U does not depend
        on it.  `values` caches expression -> per-resolver values across calls."""
        cirq = _cirq()
        if self.const is not None:
            return None
        if self.eigen is not None:
            comps, shift, expr = self.eigen
            cache = self.__dict__.setdefault("_dexpr", {})
            dexpr = cache.get(symbol)
            if dexpr is None:
                import sympy

                dexpr = cache[symbol] = sympy.diff(expr, symbol)
            if dexpr == 0:
                return None

            t = _expr_values(expr, [getattr(r, "base", r) for r in resolvers], values)
            dt = _expr_values(dexpr, [getattr(r, "base", r) for r in resolvers], values)
            out = 0
            for h, proj in comps:
                f = 1j * np.pi * (h + shift) * np.exp(1j * np.pi * t * (h + shift)) * dt
                out = out + f[:, None, None] * proj[None]
            return self._finish(np.asarray(out, dtype=np.complex128))
        if symbol not in cirq.parameter_symbols(self.op):
            return None
        h = 1e-6
        mats = []
        for r in resolvers:
            base = dict(r.param_dict)
            plus = dict(base)
            minus = dict(base)
            v = float(r.value_of(symbol))
            plus[symbol] = v + h
            minus[symbol] = v - h
            up = np.asarray(cirq.unitary(cirq.resolve_parameters(self.op, plus)), dtype=np.complex128)
            um = np.asarray(cirq.unitary(cirq.resolve_parameters(self.op, minus)), dtype=np.complex128)
            mats.append((up - um) / (2 * h))
        return self._finish(np.array(mats))


def _eigen_info(op):
    """(components, shift, exponent expression) for a GateOperation of an EigenGate
    whose only parameter is its exponent; None otherwise."""
    cirq = _cirq()
    gate = getattr(op, "gate", None)
    if not isinstance(gate, cirq.EigenGate):
        return None
    if type(op) is not cirq.GateOperation:
        return None
    expr = gate.exponent
    if not cirq.is_parameterized(expr):
        return None
    if cirq.is_parameterized(gate.global_shift):
        return None
    try:
        comps = [(float(h), np.asarray(p, dtype=np.complex128)) for h, p in gate._eigen_components()]
    except Exception:
        return None
    return comps, float(gate.global_shift), expr


def split_measurements(circuit):
    """(unitary part ops, terminal measurement ops).

    Raises NotImplementedError for measurements that are not terminal."""
    cirq = _cirq()
    from cirq_gb300.ir import flatten_ops

    from cirq_gb300.ir import is_measurement_op

    ops = flatten_ops(circuit)
    flags = [is_measurement_op(op) for op in ops]
    if not any(flags):
        return ops, []
    # terminal: no operation other than a measurement acts on a measured
    # qubit afterwards (measurements commute with one another, so repeated or
    # overlapping final measurements all read one sampled basis state)
    measured: set = set()
    for op, is_meas in zip(ops, flags):
        if is_meas:
            measured.update(op.qubits)
        elif measured.intersection(op.qubits):
            raise NotImplementedError(
                "cirq_gb300 simulates measurements only at the end of the circuit "
                "(mid-circuit measurement needs per-repetition trajectories)"
            )
    body = [op for op, m in zip(ops, flags) if not m]
    meas = [op for op, m in zip(ops, flags) if m]
    for op in meas:
        if not isinstance(op.gate, cirq.MeasurementGate):
            raise NotImplementedError(f"unsupported measurement {op!r}")
    return body, meas


MAX_STATE_BITS = 40  # widest state the engine's ABI accepts (gbq_run and friends)


class CompiledCircuit:
    """Structure + plan of a circuit over a fixed qubit order (see module doc)."""

    def __init__(
        self,
        ops: Sequence[Any],
        qubits: Sequence[Any],
        *,
        dm: bool,
        planner: Planner,
        resolvers: Sequence[Any],
    ):
        cirq = _cirq()
        self.qubits = tuple(qubits)
        self.n = len(qubits)
        self.dm = dm
        self.nbits = 2 * self.n if dm else self.n
        if self.nbits > MAX_STATE_BITS:
            # the reference's numpy allocation fails the same way
            raise MemoryError(
                f"Unable to allocate a state of {self.nbits} bits (2^{self.nbits} complex64 amplitudes): "
                f"at most {MAX_STATE_BITS} bits fit a device state"
            )
        # device width: narrow registers run padded with |0> high bits
        self.nbits_dev = max(self.nbits, MIN_TILE_BITS)
        index = {q: i for i, q in enumerate(self.qubits)}
        n = self.n
        self.sources: list[OpSource] = []
        self.gates: list[BitGate] = []
        self._phase_ops = [op for op in ops if not op.qubits]
        for op in ops:
            if isinstance(op, Slot):
                if dm:
                    raise UnsupportedOperation("trajectory slots are state-vector only")
                pos = [index[q] for q in op.qubits]
                if len(pos) > 5:
                    raise UnsupportedOperation(f"operations on more than 5 qubits are not supported: {op.op!r}")
                src = OpSource(op, "u", None, None, slot=op.slot)
                self.sources.append(src)
                self.gates.append(
                    BitGate(bits=tuple(n - 1 - p for p in reversed(pos)), matrix=None, diagonal=False,
                            tag=len(self.sources) - 1)
                )
                continue
            if not op.qubits:
                if dm:
                    continue  # a global phase cancels in rho
                if not cirq.has_unitary(op) and not cirq.is_parameterized(op):
                    raise UnsupportedOperation(f"operation without qubits: {op!r}")
                if self.n == 0:
                    continue
                # a global phase is a diagonal gate on index bit 0 (absorbed for free)
                const = None
                if not cirq.is_parameterized(op):
                    const = complex(np.asarray(cirq.unitary(op)).reshape(-1)[0]) * np.eye(2)
                self._add(op, "phase", const, None, (0,))
                continue
            if any(q.dimension != 2 for q in op.qubits):
                raise UnsupportedOperation(f"only qubits are supported, got {op!r}")
            pos = [index[q] for q in op.qubits]
            k = len(pos)
            param = cirq.is_parameterized(op)
            unitary = cirq.has_unitary(op) if not param else _param_has_unitary(op, resolvers[0])
            if not unitary and not dm:
                raise UnsupportedOperation(
                    f"noisy operation {op!r}: the state-vector simulator only handles unitary "
                    "operations (use DensityMatrixSimulator for channels)"
                )
            eig = _eigen_info(op) if param else None
            if unitary:
                if k > 5:
                    raise UnsupportedOperation(f"gates on more than 5 qubits are not supported: {op!r}")
                const = None if param else np.asarray(cirq.unitary(op), dtype=np.complex128)
                if not dm:
                    self._add(op, "u", const, eig, tuple(n - 1 - p for p in reversed(pos)))
                else:
                    self._add(op, "u", const, eig, tuple(2 * n - 1 - p for p in reversed(pos)))
                    self._add(
                        op, "conj", None if const is None else np.conjugate(const), eig,
                        tuple(n - 1 - p for p in reversed(pos)),
                    )
            else:
                if 2 * k > 5:
                    raise UnsupportedOperation(
                        f"channels on more than 2 qubits are not supported: {op!r}"
                    )
                const = None
                if not param:
                    ks = cirq.kraus(op)
                    const = sum(np.kron(np.conjugate(np.asarray(kk)), np.asarray(kk)) for kk in ks)
                    const = np.asarray(const, dtype=np.complex128)
                rows = tuple(2 * n - 1 - p for p in reversed(pos))
                cols = tuple(n - 1 - p for p in reversed(pos))
                self._add(op, "superop", const, None, rows + cols)
        self.planner = planner
        self.plan: Plan | None = None
        self._plan_resolvers(resolvers)

    def _add(self, op, transform, const, eig, bits):
        src = OpSource(op, transform, const, eig)
        self.sources.append(src)
        self.gates.append(BitGate(bits=bits, matrix=None, diagonal=False, tag=len(self.sources) - 1))

    def _eigen_groups(self) -> list:
        """Parameterised EigenGate sources grouped by (matrix size, number of
        eigencomponents): (source indices, exponent expressions, (S, K)
        half-turns h + shift, (S, K, d, d) projectors, (S,) conjugate flags)."""
        groups = self.__dict__.get("_eigen_group_cache")
        if groups is None:
            by_key: dict = {}
            for i, src in enumerate(self.sources):
                if src.const is not None or src.slot is not None or src.eigen is None:
                    continue
                if src.transform not in ("u", "conj"):
                    continue
                comps, shift, expr = src.eigen
                d = comps[0][1].shape[0]
                by_key.setdefault((d, len(comps)), []).append((i, src, comps, shift, expr))
            groups = []
            for items in by_key.values():
                idx = [it[0] for it in items]
                exprs = [it[4] for it in items]
                H = np.array([[h + it[3] for h, _ in it[2]] for it in items], dtype=np.float64)
                Pm = np.array([[np.asarray(p, dtype=np.complex128) for _, p in it[2]] for it in items])
                conj = np.array([it[1].transform == "conj" for it in items])
                groups.append((idx, exprs, H, Pm, conj))
            self.__dict__["_eigen_group_cache"] = groups
        return groups

    def gate_batch(self, resolvers) -> dict:
        """Every source's (P, d, d) matrices for the resolvers.  Parameterised
        EigenGates are evaluated together per group (one einsum of the
        phases exp(i pi t (h + shift)) with the projectors), the rest one by
        one (OpSource.matrices)."""
        values: dict = {}
        out: dict = {}
        plain = [r.base if hasattr(r, "base") else r for r in resolvers]
        lin_cache = self.__dict__.setdefault("_linear_exponent_cache", {})
        for g, (idx, exprs, H, Pm, conj) in enumerate(self._eigen_groups()):
            if g not in lin_cache:
                lin_cache[g] = _linear_exponents(exprs)
            lin = lin_cache[g]
            if lin is None:
                T = np.stack([_expr_values(e, plain, values) for e in exprs])  # (S, P)
            else:
                # constants, symbols and constant multiples of symbols: each
                # symbol resolved once, the exponents by one gather
                syms, index, coef, div, const = lin
                sv = _symbol_values(syms, plain)
                T = np.empty((len(exprs), len(plain)))
                has = index >= 0
                # (c * s) / d as _expr_values computes it (c = 1 and d = 1 exact)
                T[has] = (coef[has, None] * sv[index[has]]) / div[has, None]
                T[~has] = const[~has, None]
                for sym, row in zip(syms, sv):
                    values[sym] = row
            phase = np.exp(1j * np.pi * T[:, :, None] * H[:, None, :])  # (S, P, K)
            S_, K_, d_ = Pm.shape[0], Pm.shape[1], Pm.shape[-1]
            # sum_k phase_k P_k as one batched product (S, P, K) @ (S, K, d*d)
            M = np.matmul(phase, Pm.reshape(S_, K_, d_ * d_)).reshape(S_, phase.shape[1], d_, d_)
            if conj.any():
                M[conj] = np.conjugate(M[conj])
            for j, i in enumerate(idx):
                out[i] = M[j]
        for i, s in enumerate(self.sources):
            if i not in out:
                out[i] = s.matrices(resolvers, values)
        return out

    def _plan_resolvers(self, resolvers):
        batch = self.gate_batch(resolvers)
        # a parameterised gate is planned as diagonal only if it is diagonal at
        # generic parameter values too, not just at the given points (X**t is
        # the identity at t = 0); a dense op handles any matrix
        cirq = _cirq()
        rs = np.random.RandomState(1234)
        syms = sorted(
            {
                s
                for src in self.sources
                if src.const is None and src.slot is None
                for s in cirq.parameter_symbols(src.op)
            },
            key=str,
        )
        generic = [cirq.ParamResolver({s: float(rs.uniform(0.1, 0.9)) for s in syms}) for _ in range(2)]
        keep = []
        for i, g in enumerate(self.gates):
            m = np.asarray(batch[i])
            d = m.shape[-1]
            g.matrix = m[0]
            mats = [m[p] for p in range(m.shape[0])]
            if self.sources[i].const is None:
                mats += list(self.sources[i].matrices(generic))
            g.diagonal = bool(all(is_diagonal(x) for x in mats))
            ident = self.sources[i].const is not None and np.array_equal(m[0], np.eye(d))
            if not ident:
                keep.append(i)
        self.kept = keep
        gates = [self.gates[i] for i in keep]
        sub = {j: batch[i][:1] for j, i in enumerate(keep)}
        self.plan = self.planner.plan(gates, self.nbits_dev, batch=sub)

    @property
    def parameterized(self) -> bool:
        # fixed once the plan's gates are chosen (kept); remembered for them
        hit = self.__dict__.get("_parameterized")
        if hit is None or hit[0] is not self.kept:
            hit = (self.kept, any(self.sources[i].const is None for i in self.kept))
            self.__dict__["_parameterized"] = hit
        return hit[1]

    def pool(self, resolvers) -> np.ndarray:
        """complex64 (P, pool_len) matrix pools for the resolvers."""
        if not self.parameterized:
            return np.broadcast_to(self.plan.pool, (len(resolvers), len(self.plan.pool)))
        return self.pool_from_batch(self.gate_batch(resolvers), len(resolvers))

    def pool_from_batch(self, batch: dict, npoints: int, codes: dict | None = None) -> np.ndarray:
        """Matrix pools from already evaluated gate matrices (gate_batch).
        `codes[source index]` (optional): (P,) ints equal where that source's
        matrices are equal (see Plan.pool_for)."""
        if not self.parameterized:
            return np.broadcast_to(self.plan.pool, (npoints, len(self.plan.pool)))
        sub = {j: np.asarray(batch[i]) for j, i in enumerate(self.kept)}
        sub_codes = None
        if codes:
            sub_codes = {j: codes[i] for j, i in enumerate(self.kept) if i in codes}
        return self.plan.pool_for(sub, npoints, sub_codes)

    def global_phase(self, resolver) -> complex:
        """Product of the global-phase operations (used for 0-qubit circuits)."""
        cirq = _cirq()
        ph = 1.0 + 0j
        for op in self._phase_ops:
            ph *= complex(np.asarray(cirq.unitary(cirq.resolve_parameters(op, resolver))).reshape(-1)[0])
        return ph


def _param_has_unitary(op, resolver) -> bool:
    cirq = _cirq()
    return cirq.has_unitary(cirq.resolve_parameters(op, resolver))


class _ByIdentity:
    """Cache-key stand-in for an operation that has neither a hash nor
    operators to key on: equal only to itself (the cache entry holds it,
    so its id stays unique)."""

    __slots__ = ("op",)

    def __init__(self, op):
        self.op = op

    def __hash__(self):
        return id(self.op)

    def __eq__(self, other):
        return isinstance(other, _ByIdentity) and other.op is self.op


def _op_key(op) -> Any:
    """An operation as part of a cache key.  Unhashable operations (user
    KrausChannel / MixedUnitaryChannel / MatrixGate-like gates with array
    fields, PauliString operations) are keyed on the exact bytes of their
    operators, with their type, qubits and measurement keys."""
    try:
        hash(op)
        return op
    except TypeError:
        pass
    if isinstance(op, Slot):
        return ("slot", _op_key(op.op), op.slot)
    cirq = ensure_cirq()
    if cirq.is_parameterized(op) or isinstance(op.untagged, cirq.ClassicallyControlledOperation):
        return _ByIdentity(op)
    head = (type(op.untagged).__name__, tuple(op.qubits), tuple(sorted(map(str, cirq.measurement_key_objs(op)))))
    u = cirq.unitary(op, default=None)
    if u is not None:
        return head + ("u", np.asarray(u, dtype=np.complex128).tobytes())
    mix = cirq.mixture(op, default=None)
    if mix is not None:
        return head + ("m",) + tuple((float(p), np.asarray(m, dtype=np.complex128).tobytes()) for p, m in mix)
    kraus = cirq.kraus(op, default=None)
    if kraus is not None:
        return head + ("k",) + tuple(np.asarray(k, dtype=np.complex128).tobytes() for k in kraus)
    return _ByIdentity(op)


def structure_key(ops, qubits, dm, planner: Planner, noise_repr: str = "") -> Any:
    """A cache key for the compiled structure of an op list (parameter values of
    unparameterised gates are part of the structure)."""
    return (tuple(_op_key(op) for op in ops), tuple(qubits), dm, planner.tile_bits, planner.kmax, planner.budget,
            getattr(planner, "tensor", False), noise_repr)
