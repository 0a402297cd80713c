"""Autotuner: picks tile width, fusion width and pass budget by timing them.

The best planner settings depend on the circuit (how gates spread over the
qubits), its width and the GPU.  ``tune(circuit)`` compiles the circuit with
each candidate ``(tile_bits, fusion_max_qubits, pass_budget)``, times a few
runs of every plan on the device (CUDA events on the engine's stream, state
resident in HBM) and returns the fastest; results are cached in a JSON file
keyed by the circuit's structural signature and the GPU name, so a
``Simulator(autotune=True)`` pays the tuning cost once per circuit family.

Cache path: ``$CIRQ_GB300_AUTOTUNE_CACHE`` or
``~/.cache/cirq_gb300/autotune.json``.
"""

from __future__ import annotations

import hashlib
import json
import os
import threading
from typing import Callable, Sequence

from cirq_gb300.planner import Planner

DEFAULT_GRID: tuple = (
    (12, 4, 25.0),
    (12, 2, 25.0),
    (12, 4, 15.0),
    (12, 4, 40.0),
    (11, 4, 25.0),
    (13, 4, 25.0),
)

_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("CIRQ_GB300_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "cirq_gb300", "autotune.json")


def signature(ops, n: int, dm: bool) -> str:
    """Structural key of an op list: width, mode and the sequence of
    (arity, diagonality class, gate type) -- parameter values do not matter."""
    h = hashlib.sha256()
    h.update(f"{n}:{int(dm)}".encode())
    for op in ops:
        h.update(f"{len(op.qubits)}:{type(getattr(op, 'gate', op)).__name__};".encode())
    return h.hexdigest()[:24]


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, data: dict) -> None:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(key: str, device_name: str) -> Planner | None:
    entry = _load(cache_path()).get(f"{device_name}/{key}")
    if not entry:
        return None
    return Planner(tile_bits=entry["tile_bits"], kmax=entry["kmax"], budget=entry["budget"])


def choose(
    key: str,
    device_name: str,
    timer: Callable[[Planner], float],
    grid: Sequence[tuple] = DEFAULT_GRID,
    max_tile_bits: int = 13,
) -> tuple[Planner, list]:
    """Times every candidate with `timer(planner) -> seconds`, stores and
    returns the fastest planner and the (config, seconds) list."""
    results = []
    for tb, k, b in grid:
        tb = min(tb, max_tile_bits)
        planner = Planner(tile_bits=max(tb, 10), kmax=k, budget=b)
        results.append(((planner.tile_bits, k, b), timer(planner)))
    (tb, k, b), best = min(results, key=lambda r: r[1])
    with _lock:
        data = _load(cache_path())
        data[f"{device_name}/{key}"] = {"tile_bits": tb, "kmax": k, "budget": b, "seconds": best}
        _store(cache_path(), data)
    return Planner(tile_bits=tb, kmax=k, budget=b), results


def device_timer(engine, ops, qubits, dm: bool, resolvers, reps: int = 2) -> Callable[[Planner], float]:
    """A timer that compiles `ops` with a planner and times `reps` runs of the
    plan from |0> on the device (after one warm-up run)."""
    from cirq_gb300.program import CompiledCircuit

    def timer(planner: Planner) -> float:
        c = CompiledCircuit(ops, qubits, dm=dm, planner=planner, resolvers=resolvers)
        if not c.plan.npasses:
            return 0.0
        state = engine.alloc(8 << c.nbits_dev)
        pool = engine.upload(c.pool(resolvers[:1])[0])
        try:
            engine.new_state(c.nbits_dev, basis=0, into=state)
            engine.run(state, c.nbits_dev, c.plan, pool)
            engine.event(2)
            for _ in range(reps):
                engine.run(state, c.nbits_dev, c.plan, pool)
            engine.event(3)
            return engine.elapsed_ms(2, 3) / 1e3 / reps
        finally:
            state.free()
            pool.free()

    return timer


def tune(ops, qubits, dm: bool, resolvers, engine, grid: Sequence[tuple] = DEFAULT_GRID) -> Planner:
    """Cached planner for this op list on this GPU (tuning it on a miss)."""
    key = signature(ops, len(qubits), dm)
    name = engine.device_name()
    hit = lookup(key, name)
    if hit is not None:
        return hit
    planner, _ = choose(key, name, device_timer(engine, ops, qubits, dm, resolvers), grid)
    return planner
