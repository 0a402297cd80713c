"""Batched expectation-value sweeps: many circuits x many parameter points in one launch.

``simulate_expectation_values_batch(jobs)`` evaluates, for every job
``(circuit, observables, params)``, the expectation values that
``cirq.Simulator.simulate_expectation_values_sweep(circuit, observables, params)``
returns (``cirq-core/cirq/sim/simulator.py:349-371`` /
``cirq-core/cirq/sim/sparse_simulator.py:193-218``), for all jobs and all
points at once: each circuit is planned once, the matrices of all points are
produced by vectorised recipe replay, and a single persistent kernel
(``gbq_batch_expect``) lets every CTA claim points from a shared counter and
simulate each one alone in its own scratch slot.  Jobs may have different
widths (the "mixed-width" case); there is no synchronisation between CTAs.
"""

from __future__ import annotations

from typing import Any, Sequence

import numpy as np

from cirq_gb300 import _lib
from cirq_gb300._cirq_env import ensure_cirq
from cirq_gb300.engine import Engine, default_engine
from cirq_gb300.ir import pauli_terms
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, split_measurements

cirq = ensure_cirq()

BATCH_TILE_BITS = 12  # the batch kernel's tile width
MAX_BATCH_QUBITS = 24


class BatchJob:
    """One circuit with its observables and parameter points, compiled."""

    def __init__(self, circuit, observables, params, qubit_order=None, planner: Planner | None = None):
        qubit_order = cirq.QubitOrder.DEFAULT if qubit_order is None else qubit_order
        self.qubits = tuple(cirq.QubitOrder.as_qubit_order(qubit_order).order_for(circuit.all_qubits()))
        self.n = len(self.qubits)
        if self.n > MAX_BATCH_QUBITS:
            raise ValueError(f"batched sweeps support up to {MAX_BATCH_QUBITS} qubits")
        body, meas = split_measurements(circuit)
        if meas:
            raise ValueError("batched expectation sweeps need circuits without measurements")
        if not isinstance(observables, list):
            observables = [observables]
        self.observables = [cirq.PauliSum.wrap(o) for o in observables]
        self.resolvers = list(cirq.to_resolvers(params))
        planner = planner or Planner(tile_bits=BATCH_TILE_BITS, kmax=4, budget=40.0)
        if planner.tile_bits != BATCH_TILE_BITS:
            raise ValueError("batched sweeps use 12-bit tiles")
        self.compiled = CompiledCircuit(body, self.qubits, dm=False, planner=planner,
                                        resolvers=self.resolvers[:1] or [cirq.ParamResolver({})])
        # the batch kernel needs at least one full 12-bit tile
        if self.compiled.nbits_dev < BATCH_TILE_BITS:
            self.compiled.nbits_dev = BATCH_TILE_BITS
            self.compiled.plan = planner.plan(
                [self.compiled.gates[i] for i in self.compiled.kept], BATCH_TILE_BITS,
                batch={j: self.compiled.gates[i].matrix[None] for j, i in enumerate(self.compiled.kept)},
            )
        index = {q: i for i, q in enumerate(self.qubits)}
        self.terms = [pauli_terms(o, index, self.n) for o in self.observables]


def simulate_expectation_values_batch(
    jobs: Sequence[Any], engine: Engine | None = None
) -> list[np.ndarray]:
    """Returns, per job, a complex array (points, observables).

    `jobs` holds BatchJob objects or (circuit, observables, params) tuples."""
    eng = engine or default_engine()
    jobs = [j if isinstance(j, BatchJob) else BatchJob(*j) for j in jobs]
    passes_l, ops_l, pools_l, terms_l, points_l = [], [], [], [], []
    npass = nop = 0
    mat_off = 0
    term_off = 0
    layout = []  # per job: (first point index, npoints, term slices per observable)
    total_points = 0
    for job in jobs:
        plan = job.compiled.plan
        p = plan.passes.copy()
        p["op_begin"] += nop
        passes_l.append(p)
        ops_l.append(plan.ops)
        pool = np.ascontiguousarray(job.compiled.pool(job.resolvers))  # (P, pool_len)
        P, plen = pool.shape
        if plen & 1:
            pool = np.concatenate([pool, np.zeros((P, 1), np.complex64)], axis=1)
            plen += 1
        pools_l.append(pool.reshape(-1))
        # terms of one observable with equal X masks sit next to each other,
        # so the kernel evaluates them with one read of the state
        flat_terms = [t for obs in job.terms for t in sorted(obs, key=lambda term: term[0])]
        slices = []
        k = 0
        for obs in job.terms:
            slices.append((k, k + len(obs)))
            k += len(obs)
        recs = Engine.pauli_records([(x, zy, ny, 1.0) for x, zy, ny, _ in flat_terms])
        coefs = np.array([c for *_, c in flat_terms], dtype=np.complex128)
        pts = np.zeros(P, dtype=_lib.POINT_DTYPE)
        pts["nbits"] = job.compiled.nbits_dev
        pts["pass_begin"] = npass
        pts["pass_count"] = len(plan.passes)
        pts["term_count"] = len(flat_terms)
        for i in range(P):
            pts[i]["term_begin"] = term_off
            pts[i]["mat_base"] = mat_off + i * plen
            terms_l.append(recs)
            term_off += len(flat_terms)
        points_l.append(pts)
        layout.append((total_points, P, slices, coefs))
        total_points += P
        mat_off += P * plen
        npass += len(plan.passes)
        nop += len(plan.ops)
    if total_points == 0:
        return [np.zeros((0, len(j.observables)), dtype=np.complex128) for j in jobs]
    passes = np.concatenate(passes_l)
    ops = np.concatenate(ops_l) if nop else np.zeros(1, _lib.OP_DTYPE)
    pool_dev = eng.upload(np.concatenate(pools_l))
    terms = np.concatenate(terms_l) if term_off else np.zeros(0, _lib.PAULI_DTYPE)
    points = np.concatenate(points_l)
    # CTAs claim points in array order: widest first, so the tail of the
    # launch is filled with short points (each point keeps its term block)
    order = np.argsort(-points["nbits"], kind="stable")
    run_points = np.ascontiguousarray(points[order])
    max_nbits = max(int(points["nbits"].max()), BATCH_TILE_BITS)
    out = eng.batch_expect(run_points, passes, ops, pool_dev, terms, max_nbits)[:term_off]
    results = []
    for (first, P, slices, coefs), job in zip(layout, jobs):
        nt = len(coefs)
        vals = np.zeros((P, len(slices)), dtype=np.complex128)
        for i in range(P):
            tb = int(points[first + i]["term_begin"])
            tv = out[tb : tb + nt] * coefs
            for o, (a, b) in enumerate(slices):
                vals[i, o] = tv[a:b].sum()
        results.append(vals)
    return results
