"""Generates ``golden_clifford.npz``: the reference's stabilizer simulations.

quantumlib/Cirq's own tableau simulation (``cirq.CliffordTableauSimulationState``
driven by ``cirq.act_on``, cirq-core/cirq/sim/clifford/) and samplers
(``cirq.StabilizerSampler``, ``cirq.CliffordSimulator``) are run on seeded
circuits from ``cirq_gb300.workloads.random_clifford_circuit``:

* ``tab_<i>_{xs,zs,rs}``: the final tableau of a circuit without
  measurements (4, 6 and 9 qubits);
* ``meas_<i>_{outcomes,xs,zs,rs}``: a circuit with mid-circuit measurements
  and feedback, run once with a seeded random state: every measured bit in
  circuit order and the final tableau;
* ``dist_<i>_<sampler>_<key>``: (repetitions, bits) records of noisy circuits
  with resets, feedback and mid-circuit measurements from
  ``cirq.StabilizerSampler`` and ``cirq.CliffordSimulator``.

Usage (from the repository root; the argument or ``CIRQ_REFERENCE_PATH``
names the reference's ``cirq-core`` directory):

    python tests/golden/make_golden_clifford.py /path/to/Cirq/cirq-core
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "golden_clifford.npz")

TAB_CASES = [(4, 6, 0), (6, 10, 1), (9, 12, 2)]
MEAS_CASES = [(5, 10, 3), (7, 12, 4)]
DIST_CASES = [(5, 6, 5), (4, 8, 6)]
DIST_REPS = 2000


def _reference(path: str):
    if path not in sys.path:
        sys.path.insert(0, path)
    if ROOT not in sys.path:
        sys.path.insert(1, ROOT)
    from cirq_gb300._cirq_env import ensure_cirq

    cirq = ensure_cirq()
    assert os.path.abspath(cirq.__file__).startswith(os.path.abspath(path)), cirq.__file__
    return cirq


def main() -> int:
    path = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CIRQ_REFERENCE_PATH")
    if not path:
        print(__doc__)
        return 2
    cirq = _reference(path)
    from cirq_gb300 import workloads

    out = {}

    def run_state(circuit, n, seed):
        q = cirq.LineQubit.range(n)
        state = cirq.CliffordTableauSimulationState(
            cirq.CliffordTableau(num_qubits=n), qubits=q, prng=np.random.RandomState(seed)
        )
        bits = []
        for op in circuit.all_operations():
            cirq.act_on(op, state)
            if cirq.is_measurement(op):
                bits.extend(state.log_of_measurement_results[cirq.measurement_key_name(op)])
        t = state.tableau
        return np.array(bits, np.uint8), t.xs.copy(), t.zs.copy(), t.rs.copy()

    for i, (n, depth, seed) in enumerate(TAB_CASES):
        c = workloads.random_clifford_circuit(n, depth, seed, final_measure=False)
        _, xs, zs, rs = run_state(c, n, seed)
        out[f"tab_{i}_xs"], out[f"tab_{i}_zs"], out[f"tab_{i}_rs"] = xs, zs, rs
    for i, (n, depth, seed) in enumerate(MEAS_CASES):
        c = workloads.random_clifford_circuit(n, depth, seed, mid_measure=0.6, feedback=True)
        bits, xs, zs, rs = run_state(c, n, 100 + seed)
        out[f"meas_{i}_outcomes"] = bits
        out[f"meas_{i}_xs"], out[f"meas_{i}_zs"], out[f"meas_{i}_rs"] = xs, zs, rs
    for i, (n, depth, seed) in enumerate(DIST_CASES):
        c = workloads.random_clifford_circuit(n, depth, seed, mid_measure=0.7, resets=True, feedback=True, p=0.02)
        r1 = cirq.StabilizerSampler(seed=200 + i).run(c, repetitions=DIST_REPS)
        r2 = cirq.CliffordSimulator(seed=300 + i).run(c, repetitions=DIST_REPS)
        for key in sorted(c.all_measurement_key_names()):
            out[f"dist_{i}_stab_{key}"] = np.asarray(r1.measurements[key], np.uint8)
            out[f"dist_{i}_cliff_{key}"] = np.asarray(r2.measurements[key], np.uint8)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")
    return 0


if __name__ == "__main__":
    sys.exit(main())
