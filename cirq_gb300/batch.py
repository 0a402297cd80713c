"""Batched expectation-value sweeps: many circuits x many parameter points.

``simulate_expectation_values_batch(jobs)`` evaluates, for every job
``(circuit, observables, params)``, the expectation values that
``cirq.Simulator.simulate_expectation_values_sweep(circuit, observables, params)``
returns (``cirq-core/cirq/sim/simulator.py:349-371`` /
``cirq-core/cirq/sim/sparse_simulator.py:193-218``), for all jobs and all
points at once: each circuit is planned once and the matrices of all points
are produced by vectorised recipe replay.  Two execution modes:

* default: the states of a job's points lie back to back in HBM and every
  pass runs over all of them in one launch of the ordinary tile pass
  (``gbq_run_points``), each tile reading its point's matrices; the Pauli
  terms of every point are then summed in one launch
  (``gbq_points_expect``).  A sweep streams through HBM like one large state.
* ``persistent=True``: all jobs and points in a single persistent launch
  (``gbq_batch_expect``): every CTA claims points from a shared counter and
  simulates each one alone in its own scratch slot; jobs may have different
  widths and no CTA ever waits for another.
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
        # the structure comes from the first point, or from a generic one when
        # the sweep is empty (every symbol at 0.37, as for adjoint programs)
        rep = self.resolvers[:1] or [cirq.ParamResolver({s: 0.37 for s in cirq.parameter_symbols(circuit)})]
        self.compiled = CompiledCircuit(body, self.qubits, dm=False, planner=planner, resolvers=rep)
        # the batch kernel needs at least one full 12-bit tile
        if self.compiled.nbits_dev < BATCH_TILE_BITS:
            self.compiled.nbits_dev = BATCH_TILE_BITS
            self.compiled.plan = planner.plan(
                [self.compiled.gates[i] for i in self.compiled.kept], BATCH_TILE_BITS,
                batch={j: self.compiled.gates[i].matrix[None] for j, i in enumerate(self.compiled.kept)},
            )
        index = {q: i for i, q in enumerate(self.qubits)}
        self.terms = [pauli_terms(o, index, self.n) for o in self.observables]


def _job_terms(job):
    """Unit-coefficient Pauli records of a job (terms of one observable with
    equal X masks adjacent), their coefficients and per-observable slices."""
    flat_terms = [t for obs in job.terms for t in sorted(obs, key=lambda term: term[0])]
    slices = []
    k = 0
    for obs in job.terms:
        slices.append((k, k + len(obs)))
        k += len(obs)
    recs = Engine.pauli_records([(x, zy, ny, 1.0) for x, zy, ny, _ in flat_terms])
    coefs = np.array([c for *_, c in flat_terms], dtype=np.complex128)
    return recs, coefs, slices


def _job_pool(job) -> tuple[np.ndarray, int]:
    """(P, even pool length) complex64 matrix pools of a job's points."""
    pool = np.ascontiguousarray(job.compiled.pool(job.resolvers), dtype=np.complex64)
    P, plen = pool.shape
    if plen & 1:
        pool = np.concatenate([pool, np.zeros((P, 1), np.complex64)], axis=1)
        plen += 1
    return pool, plen


class _PointsRun:
    """One chunk of a job's points on the device: launched asynchronously,
    collected later (so the host can build the next job's pools meanwhile)."""

    def __init__(self, eng: Engine, job, pool, plen, start, count, states):
        c = job.compiled
        self.eng, self.job, self.start, self.count, self.states = eng, job, start, count, states
        self.n = c.nbits_dev
        eng.points_set_zero(states, self.n, count)
        self.pool_dev = eng.upload(pool[start : start + count].reshape(-1))
        eng.run_points(states, self.n, count, c.plan, self.pool_dev, plen)

    def collect(self, vals, recs, coefs, slices) -> None:
        tv = self.eng.points_expect(self.states, self.n, self.count, recs) * coefs[None, :]
        self.pool_dev.free()
        for o, (a, b) in enumerate(slices):
            vals[self.start : self.start + self.count, o] = tv[:, a:b].sum(axis=1)


def _points_jobs(eng: Engine, jobs, budget_bytes: int) -> list[np.ndarray]:
    """Default mode: each job's points evolved together, chunked to fit
    `budget_bytes`; the host builds job k+1's pools while job k runs."""
    results = []
    nxt = _job_pool(jobs[0]) if jobs and jobs[0].resolvers else None
    for j, job in enumerate(jobs):
        c = job.compiled
        n = c.nbits_dev
        P = len(job.resolvers)
        recs, coefs, slices = _job_terms(job)
        vals = np.zeros((P, len(slices)), dtype=np.complex128)
        results.append(vals)
        if P == 0:
            nxt = _job_pool(jobs[j + 1]) if j + 1 < len(jobs) and jobs[j + 1].resolvers else None
            continue
        pool, plen = nxt
        L = int(c.plan.passes["L"].min()) if c.plan.npasses else n
        chunk = max(1, min(P, budget_bytes // (8 << n), (1 << 24) >> max(n - L, 0)))
        states = eng.alloc((8 << n) * chunk)
        try:
            for start in range(0, P, chunk):
                run = _PointsRun(eng, job, pool, plen, start, min(chunk, P - start), states)
                if start + chunk >= P:  # last chunk: overlap the next job's host work
                    nxt = _job_pool(jobs[j + 1]) if j + 1 < len(jobs) and jobs[j + 1].resolvers else None
                run.collect(vals, recs, coefs, slices)
        finally:
            states.free()
    return results


def simulate_expectation_values_batch(
    jobs: Sequence[Any], engine: Engine | None = None, persistent: bool = False
) -> list[np.ndarray]:
    """Returns, per job, a complex array (points, observables).

    `jobs` holds BatchJob objects or (circuit, observables, params) tuples;
    `persistent` selects the single-launch mode (see the module doc)."""
    eng = engine or default_engine()
    jobs = [j if isinstance(j, BatchJob) else BatchJob(*j) for j in jobs]
    if not persistent:
        _, free, _ = eng.device_info()
        budget = max(1 << 28, min(int(free) // 2, 64 << 30))
        return _points_jobs(eng, jobs, budget)
    passes_l, ops_l, pools_l, terms_l, points_l = [], [], [], [], []
    npass = nop = 0
    mat_off = 0
    term_off = 0
    layout = []  # per job: (first point index, npoints, term slices per observable)
    total_points = 0
    for job in jobs:
        if not job.resolvers:  # an empty sweep: no points, no passes
            layout.append((total_points, 0, [(0, 0)] * len(job.observables), np.zeros(0, np.complex128)))
            continue
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
