"""Autotuner cache logic (CPU, with an injected timer)."""

import json

from cirq_gb300 import autotune, workloads
from cirq_gb300.planner import Planner
from cirq_gb300.program import split_measurements


def test_choose_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("CIRQ_GB300_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    times = {(12, 4, 25.0): 3.0, (12, 2, 25.0): 1.0, (11, 4, 25.0): 2.0}

    def timer(p: Planner) -> float:
        return times.get((p.tile_bits, p.kmax, p.budget), 9.0)

    best, res = autotune.choose("k1", "GPU X", timer)
    assert (best.tile_bits, best.kmax, best.budget) == (12, 2, 25.0)
    assert len(res) == len(autotune.DEFAULT_GRID)
    hit = autotune.lookup("k1", "GPU X")
    assert (hit.tile_bits, hit.kmax, hit.budget) == (12, 2, 25.0)
    assert autotune.lookup("k1", "GPU Y") is None
    data = json.loads((tmp_path / "tune.json").read_text())
    assert data["GPU X/k1"]["seconds"] == 1.0


def test_signature_ignores_parameter_values():
    a = workloads.random_layer_circuit(6, 4, seed=1)
    b = workloads.random_layer_circuit(6, 4, seed=2)
    c = workloads.random_layer_circuit(6, 5, seed=1)
    sa = autotune.signature(split_measurements(a)[0], 6, False)
    assert sa == autotune.signature(split_measurements(b)[0], 6, False)
    assert sa != autotune.signature(split_measurements(c)[0], 6, False)
    assert sa != autotune.signature(split_measurements(a)[0], 6, True)
