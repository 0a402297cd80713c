"""Adjoint differentiation of <psi(theta)|H|psi(theta)> on the GPU.

The reference has no gradient code; this module adds one behind
``torch.autograd.Function``.  For a circuit U_N ... U_1 and Hamiltonian H
(a PauliSum with real coefficients):

1. forward:   psi = U_N ... U_1 |0>  (the fused tile-pass program);
2.            lam = H psi  (``gbq_sv_apply_paulisum``),  E = Re<psi|lam>;
3. reverse:   for j = N .. 1, with psi and lam both "after gate j":
                  dE/dtheta += 2 Re <lam| (dU_j/dtheta) U_j^dagger |psi>
              then psi <- U_j^dagger psi, lam <- U_j^dagger lam.

Step 3 runs as one two-state program (``gbq_run_dual``): un-applications are
fused exactly like a forward circuit, and every parameterised gate adds a
probe op that reduces Re<lam|D|psi> over each tile into a per-slot partial
(D = dU/dtheta U^dagger, diagonal probes for Rz-like gates).  Cost is ~3
state sweeps instead of the 2P circuit evaluations of parameter shift.

Symbols may appear in several gates and inside expressions: derivatives
follow the chain rule through ``sympy`` (EigenGates) or central differences of
the gate matrix (any other parameterised gate).
"""

from __future__ import annotations

import threading

from typing import Any, Sequence

import numpy as np

from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.engine import Engine, default_engine
from cirq_gb300.ir import BitGate, is_diagonal, pauli_terms
from cirq_gb300.planner import MIN_TILE_BITS, Planner
from cirq_gb300.program import _expr_values, CompiledCircuit, split_measurements

cirq = ensure_cirq()


class AdjointProgram:
    """Forward and reverse programs of a parameterised circuit (compiled once).

    `pass_budget` bounds the work the planner puts in one pass of the forward
    program; `reverse_pass_budget` (default: the same) does so for the
    two-state reverse sweep, whose passes read and write two states."""

    def __init__(
        self,
        circuit,
        observable,
        symbols: Sequence[Any],
        *,
        qubit_order=None,
        engine: Engine | None = None,
        tile_bits: int = 12,
        reverse_tile_bits: int = 11,
        fusion_max_qubits: int = 4,
        pass_budget: float = 60.0,
        reverse_pass_budget: float | None = None,
    ):
        self._engine = engine
        qubit_order = cirq.QubitOrder.DEFAULT if qubit_order is None else qubit_order
        self.qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(circuit.all_qubits()))
        body, meas = split_measurements(circuit)
        if meas:
            raise ValueError("adjoint differentiation needs a circuit without measurements")
        self.symbols = list(symbols)
        self.n = len(self.qubits)
        index = {q: i for i, q in enumerate(self.qubits)}
        self.terms = pauli_terms(observable, index, self.n)
        if any(abs(np.imag(c)) > 1e-12 for *_, c in self.terms):
            raise ValueError("the observable must have real coefficients (Hermitian)")
        # a representative point (all symbols at 0.37) fixes the structure
        rep = cirq.ParamResolver({s: 0.37 for s in self.symbols})
        rep2 = cirq.ParamResolver({s: -1.13 for s in self.symbols})
        self.forward = CompiledCircuit(
            body, self.qubits, dm=False, resolvers=[rep],
            planner=Planner(tile_bits=tile_bits, kmax=fusion_max_qubits, budget=pass_budget),
        )
        self.nbits = self.forward.nbits_dev
        fwd = self.forward
        # reverse structure: gate j^dagger preceded by its probes, j = N..1
        rev: list[BitGate] = []
        self._rev_src: list[tuple] = []  # (kind, source index, symbol index)
        self.slot_symbol: list[int] = []
        sym_index = {s: i for i, s in enumerate(self.symbols)}
        for i in reversed(fwd.kept):
            src = fwd.sources[i]
            g = fwd.gates[i]
            used = sorted(sym_index[s] for s in cirq.parameter_symbols(src.op) if s in sym_index)
            for si in used:
                sym = self.symbols[si]
                d1 = src.derivatives([rep], sym)
                if d1 is None:
                    continue
                d2 = src.derivatives([rep2], sym)
                u1 = src.matrices([rep])[0]
                u2 = src.matrices([rep2])[0]
                D1 = d1[0] @ u1.conj().T
                D2 = d2[0] @ u2.conj().T if d2 is not None else D1
                diag = is_diagonal(np.round(D1, 14)) and is_diagonal(np.round(D2, 14))
                slot = len(self.slot_symbol)
                self.slot_symbol.append(si)
                rev.append(BitGate(bits=g.bits, matrix=D1, diagonal=diag, probe=slot))
                self._rev_src.append(("probe", i, si))
            rev.append(BitGate(bits=g.bits, matrix=g.matrix.conj().T, diagonal=g.diagonal))
            self._rev_src.append(("dagger", i, -1))
        rtb = max(MIN_TILE_BITS, min(reverse_tile_bits, self.nbits))
        rbudget = pass_budget if reverse_pass_budget is None else reverse_pass_budget
        self.reverse_planner = Planner(tile_bits=rtb, kmax=2, budget=rbudget)
        for g in rev:
            if g.probe >= 0 and not g.diagonal and len(g.bits) > 3:
                raise NotImplementedError("gradient of a gate on more than 3 qubits")
        self.reverse = self.reverse_planner.plan(rev, self.nbits)
        self.nslots = len(self.slot_symbol)
        self.reverse_tiles = 1 << (self.nbits - rtb)
        self._pauli = Engine.pauli_records(self.terms)

    @property
    def engine(self) -> Engine:
        if self._engine is None:
            self._engine = default_engine()
        return self._engine

    # ------------------------------------------------------------------
    def _reverse_layout(self) -> dict:
        """How each reverse-program entry is produced (computed once):
        eigen-gate probes as a fixed generator times the exponent's
        derivative, daggers of forward gates, and the rest one by one."""
        lay = self.__dict__.get("_rev_layout")
        if lay is not None:
            return lay
        import sympy

        fwd = self.forward
        gen_groups: dict = {}  # d -> (js, gens list, derivative exprs)
        dag_groups: dict = {}  # d -> (js, forward source indices)
        other: list = []
        for j, (kind, i, si) in enumerate(self._rev_src):
            src = fwd.sources[i]
            if kind != "dagger" and src.eigen is not None and src.transform == "u":
                # U = sum_k exp(i pi t (h_k + s)) P_k with orthogonal projectors, so
                # dU/dtheta U^dagger = i pi (dt/dtheta) sum_k (h_k + s) P_k: a fixed
                # generator times the exponent's derivative at this point
                comps, shift, expr = src.eigen
                gen = 1j * np.pi * sum((h + shift) * np.asarray(p, dtype=np.complex128) for h, p in comps)
                g = gen_groups.setdefault(gen.shape[-1], ([], [], []))
                g[0].append(j)
                g[1].append(gen)
                g[2].append(sympy.diff(expr, self.symbols[si]))
            elif kind == "dagger":
                d = fwd.gates[i].matrix.shape[-1]
                g = dag_groups.setdefault(d, ([], []))
                g[0].append(j)
                g[1].append(i)
            else:
                other.append((j, kind, i, si))
        lay = {
            "gen": [(js, np.stack(gens), exprs) for js, gens, exprs in gen_groups.values()],
            "dag": list(dag_groups.values()),
            "other": other,
        }
        self.__dict__["_rev_layout"] = lay
        return lay

    def _reverse_batch(self, resolver, gates: dict | None = None) -> dict:
        """Reverse-program matrices at one point; `gates` are the forward
        program's evaluated gate matrices at that point, when available."""
        fwd = self.forward
        lay = self._reverse_layout()
        values: dict = {}  # expression -> value at this point, shared by all gates
        out: dict = {}
        for js, gens, exprs in lay["gen"]:
            dt = np.array([_expr_values(e, [resolver], values)[0] for e in exprs])
            mats = dt[:, None, None] * gens
            for k, j in enumerate(js):
                out[j] = mats[k : k + 1]
        cache_u: dict = {}

        def forward_u(i):
            if i not in cache_u:
                cache_u[i] = gates[i][:1] if gates is not None else fwd.sources[i].matrices([resolver], values)[:1]
            return cache_u[i]

        for js, srcs in lay["dag"]:
            daggers = np.concatenate([forward_u(i) for i in srcs]).conj().transpose(0, 2, 1)
            for k, j in enumerate(js):
                out[j] = daggers[k : k + 1]
        for j, kind, i, si in lay["other"]:
            u = forward_u(i)[0]
            du = fwd.sources[i].derivatives([resolver], self.symbols[si], values)
            out[j] = (du[0] @ u.conj().T)[None]
        return out

    def forward_state(self, values, overlap=None, reuse: bool = False):
        """Runs the forward program; returns (psi, lam, E, resolver).

        `overlap(resolver, gates)` (optional) runs on the host while the
        forward passes execute on the GPU; its result is stored in
        self._overlap_result.  With `reuse`, psi, lam and the pool live in
        the program's own buffers (valid until the next reuse call);
        otherwise they are new buffers that the caller frees."""
        eng = self.engine
        r = cirq.ParamResolver(dict(zip(self.symbols, [float(v) for v in values])))
        fwd = self.forward
        gates = fwd.gate_batch([r])
        sbytes = 8 << self.nbits
        psi = eng.new_state(self.n, basis=0, nbits_dev=self.nbits,
                            into=self._buffer("psi", sbytes) if reuse else None)
        pool = None
        if fwd.plan.npasses:
            host_pool = np.ascontiguousarray(fwd.pool_from_batch(gates, 1)[0])
            pool = self._upload("forward_pool", host_pool) if reuse else eng.upload(host_pool)
            eng.run(psi, self.nbits, fwd.plan, pool, sync=False)
        # host work on a helper thread: the calls below wait for the GPU inside
        # the C library (ctypes releases the GIL), so it runs alongside them
        worker = None
        self._overlap_result = None
        if overlap is not None:
            def job():
                self._overlap_result = overlap(r, gates)

            worker = threading.Thread(target=job)
            worker.start()
        if self.nbits > self.n:
            # padding amplitudes of lam stay zero; apply_paulisum writes the first 2^n
            lam = eng.new_state(self.nbits, basis=0, into=self._buffer("lam", sbytes) if reuse else None)
        else:
            lam = self._buffer("lam", sbytes) if reuse else eng.alloc(sbytes)
        try:
            eng.apply_paulisum(psi, self.n, self.terms, lam)  # synchronises: the forward pool is free
            if pool is not None and not reuse:
                pool.free()
            E = eng.inner(psi, lam, self.n).real
        finally:
            if worker is not None:
                worker.join()
        return psi, lam, E, r

    def _reverse_pool(self, resolver, gates=None) -> np.ndarray:
        return self.reverse.pool_for(self._reverse_batch(resolver, gates), 1)[0]

    def gradient_from(self, psi, lam, resolver, reverse_pool=None, reuse: bool = False) -> np.ndarray:
        """Reverse sweep from (psi, lam) after the forward pass (consumes
        both; with `reuse`, the pool and partials use the program's buffers)."""
        eng = self.engine
        grad = np.zeros(len(self.symbols))
        if self.nslots == 0:
            return grad
        pool = reverse_pool if reverse_pool is not None else self._reverse_pool(resolver)
        if reuse:
            pool_dev = self._upload("reverse_pool", pool)
            partial = self._buffer("partial", 8 * self.nslots * self.reverse_tiles)
            slots = self._buffer("slots", 8 * self.nslots)
        else:
            pool_dev = eng.upload(np.ascontiguousarray(pool))
            partial = eng.alloc(8 * self.nslots * self.reverse_tiles)
            slots = eng.alloc(8 * self.nslots)
        eng.run_dual(psi, lam, self.nbits, self.reverse, pool_dev, partial)
        eng.reduce_slots(partial, self.nslots, self.reverse_tiles, slots)
        vals = np.empty(self.nslots, dtype=np.float64)
        slots.download(vals)
        np.add.at(grad, np.array(self.slot_symbol), 2.0 * vals)
        return grad

    def _buffer(self, name: str, nbytes: int):
        """A device buffer kept by the program for value_and_grad (reused
        across calls: no cudaMalloc / cudaFree, which synchronises, per
        gradient)."""
        bufs = self.__dict__.setdefault("_buffers", {})
        buf = bufs.get(name)
        if buf is None or buf.nbytes < nbytes:
            if buf is not None:
                buf.free()
            buf = bufs[name] = self.engine.alloc(max(nbytes, 16))
        return buf

    def release(self) -> None:
        """Frees the device buffers value_and_grad keeps between calls."""
        for buf in self.__dict__.pop("_buffers", {}).values():
            buf.free()

    def _upload(self, name: str, host: np.ndarray):
        host = np.ascontiguousarray(host)
        buf = self._buffer(name, host.nbytes)
        buf.upload(host)
        return buf

    def value_and_grad(self, values) -> tuple[float, np.ndarray]:
        # the reverse program's matrices are built on the host while the
        # forward passes run on the GPU; states, pools and partials live in
        # buffers the program keeps between calls
        overlap = self._reverse_pool if self.nslots else None
        psi, lam, E, r = self.forward_state(values, overlap=overlap, reuse=True)
        g = self.gradient_from(psi, lam, r, reverse_pool=self._overlap_result, reuse=True)
        return E, g

    def value_and_grad_native(self, values) -> tuple[float, np.ndarray]:
        """The same (E, gradient) through one C-ABI call (gbq_adjoint): the
        matrix pools of the forward and reverse programs are built here and
        the engine runs the forward passes, lam = H psi, <psi|lam>, the
        reverse sweep and the slot sums on its own."""
        import ctypes

        from cirq_gb300 import _lib

        eng = self.engine
        r = cirq.ParamResolver(dict(zip(self.symbols, [float(v) for v in values])))
        fwd = self.forward
        gates = fwd.gate_batch([r])
        fpool = eng.upload(np.ascontiguousarray(fwd.pool_from_batch(gates, 1)[0]))
        rpool = eng.upload(np.ascontiguousarray(self._reverse_pool(r, gates)))
        slots = np.zeros(max(self.nslots, 1), dtype=np.float64)
        value = ctypes.c_double()
        fp, rp = fwd.plan, self.reverse
        try:
            _lib.check(
                eng.lib.gbq_adjoint(
                    eng.ctx, self.n, self.nbits, fp.passes.ctypes.data, len(fp.passes), fp.ops.ctypes.data,
                    len(fp.ops), fpool.ptr, self._pauli.ctypes.data, len(self._pauli), rp.passes.ctypes.data,
                    len(rp.passes), rp.ops.ctypes.data, len(rp.ops), rpool.ptr, self.nslots, ctypes.byref(value),
                    slots.ctypes.data,
                ),
                "gbq_adjoint",
            )
        finally:
            fpool.free()
            rpool.free()
        grad = np.zeros(len(self.symbols))
        if self.nslots:
            np.add.at(grad, np.array(self.slot_symbol), 2.0 * slots[: self.nslots])
        return value.value, grad

    def value(self, values) -> float:
        psi, lam, E, _ = self.forward_state(values)
        psi.free()
        lam.free()
        return E


def _torch():
    import torch

    return torch


class _AdjointExpectation:
    """Holder for the torch.autograd.Function (built lazily so that importing
    this module does not import torch)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _torch()

            class AdjointExpectationFn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, theta, program):
                    vals = theta.detach().to("cpu", torch.float64).numpy()
                    psi, lam, E, r = program.forward_state(vals)
                    ctx.program = program
                    ctx.saved_device = (psi, lam, r)
                    ctx.theta_meta = (theta.dtype, theta.device)
                    return torch.tensor(E, dtype=theta.dtype, device=theta.device)

                @staticmethod
                def backward(ctx, grad_out):
                    psi, lam, r = ctx.saved_device
                    g = ctx.program.gradient_from(psi, lam, r)
                    psi.free()
                    lam.free()
                    ctx.saved_device = None
                    dtype, device = ctx.theta_meta
                    gt = torch.as_tensor(g, dtype=dtype, device=device)
                    return grad_out * gt, None

            cls.fn = AdjointExpectationFn
        return cls.fn


def expectation(theta, program: AdjointProgram):
    """Differentiable <H>(theta) (torch scalar); backward runs the adjoint sweep."""
    return _AdjointExpectation.get().apply(theta, program)


def parameter_shift_gradient(simulator, circuit, observable, symbols, values, indices=None) -> np.ndarray:
    """Parameter-shift gradient through the plain GPU simulator
    (``simulate_expectation_values_sweep`` with two resolvers per parameter):
    dE/dtheta_i = (E(theta + pi/2 e_i) - E(theta - pi/2 e_i)) / 2, exact for
    symbols that each enter one rotation exp(-i theta P / 2) (rx/ry/rz).
    `indices` restricts the evaluation to some parameters."""
    values = np.asarray(values, dtype=np.float64)
    idx = list(range(len(values))) if indices is None else list(indices)
    resolvers = []
    for i in idx:
        for sgn in (1.0, -1.0):
            v = values.copy()
            v[i] += sgn * np.pi / 2
            resolvers.append(cirq.ParamResolver(dict(zip(symbols, v))))
    vals = simulator.simulate_expectation_values_sweep(circuit, observable, resolvers)
    g = np.zeros(len(values))
    for k, i in enumerate(idx):
        g[i] = 0.5 * (np.real(vals[2 * k][0]) - np.real(vals[2 * k + 1][0]))
    return g
