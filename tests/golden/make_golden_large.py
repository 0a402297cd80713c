"""Generates ``golden_large.npz``: reference results at the benchmarked sizes.

The benchmark workloads (20-qubit and 24-qubit random layers, the 11-qubit
noisy density matrix, QAOA points at 16-22 qubits, the 16-qubit
hardware-efficient-ansatz gradient) are run through quantumlib/Cirq's own
simulators here, at complex128, and stored compactly so that the GPU tests
can pin the CUDA path at those sizes on a machine without the reference:

* state vectors: 4096 seeded amplitude indices and their values, the norm,
  every single-qubit <Z_i>, and the marginal distribution of qubits 0..3;
* the density matrix: its diagonal, 4096 seeded off-diagonal entries and
  the trace;
* QAOA: <sum Z_i Z_j> of 16 seeded parameter points per width;
* HEA: the energy and the parameter-shift gradient of all 320 parameters,
  every shifted energy taken from ``cirq.Simulator.simulate_expectation_values``.

Usage (from the repository root; the argument or ``CIRQ_REFERENCE_PATH``
names the reference's ``cirq-core`` directory):

    python tests/golden/make_golden_large.py /path/to/Cirq/cirq-core

Independent units run in a process pool (spawned); the whole run takes a few
minutes on 8 cores.  Nothing here re-implements the reference's numerics:
every stored number is the reference's output or a plain numpy reduction of
its output state.
"""

from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

# one BLAS thread per worker process (the pool supplies the parallelism)
for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "golden_large.npz")

SAMPLE_SEED = 1234
NSAMPLE = 4096
QAOA_WIDTHS = (16, 18, 20, 22)
QAOA_POINTS = 16
HEA_N, HEA_LAYERS, HEA_TERMS = 16, 10, 300


def _reference(path: str):
    if path not in sys.path:
        sys.path.insert(0, path)
    if ROOT not in sys.path:
        sys.path.insert(1, ROOT)
    from cirq_gb300._cirq_env import ensure_cirq

    cirq = ensure_cirq()
    assert os.path.abspath(cirq.__file__).startswith(os.path.abspath(path)), cirq.__file__
    return cirq


def state_sample_index(n: int) -> np.ndarray:
    """The amplitude indices stored for an n-qubit state (sorted, distinct)."""
    rs = np.random.RandomState(SAMPLE_SEED + n)
    return np.sort(rs.choice(2**n, size=min(NSAMPLE, 2**n), replace=False))


def state_summary(psi: np.ndarray, n: int) -> dict:
    """Seeded amplitudes, norm, <Z_i> and the qubit-0..3 marginal of a state."""
    idx = state_sample_index(n)
    p = np.abs(psi.astype(np.complex128)) ** 2
    pt = p.reshape((2,) * n)
    z = np.empty(n)
    for i in range(n):
        m = pt.sum(axis=tuple(j for j in range(n) if j != i))
        z[i] = m[0] - m[1]
    marg = pt.sum(axis=tuple(range(4, n))).reshape(-1)
    return {"idx": idx, "amps": psi[idx], "norm": np.sqrt(p.sum()), "z": z, "marg4": marg}


def job_layers(args):
    path, n, depth, seed, with_c64 = args
    cirq = _reference(path)
    from cirq_gb300 import workloads

    c = workloads.random_layer_circuit(n, depth, seed)
    t = time.time()
    out = {}
    s = state_summary(cirq.Simulator(dtype=np.complex128).simulate(c).final_state_vector, n)
    for k, v in s.items():
        out[f"layers_n{n}_d{depth}_s{seed}_c128_{k}"] = v
    if with_c64:
        s64 = cirq.Simulator(dtype=np.complex64).simulate(c).final_state_vector
        out[f"layers_n{n}_d{depth}_s{seed}_c64_amps"] = s64[s["idx"]]
    return out, f"layers n={n} d={depth}: {time.time() - t:.1f} s"


def dm_sample_index(n: int) -> tuple[np.ndarray, np.ndarray]:
    rs = np.random.RandomState(SAMPLE_SEED + 100 + n)
    r = rs.randint(0, 2**n, size=NSAMPLE)
    c = rs.randint(0, 2**n, size=NSAMPLE)
    return r, c


def job_density(args):
    path, n, depth = args
    cirq = _reference(path)
    from cirq_gb300 import workloads

    c = workloads.noisy_layer_circuit(n, depth, seed=0, p=1e-3, gamma=5e-3)
    t = time.time()
    rho = cirq.DensityMatrixSimulator(dtype=np.complex128).simulate(c).final_density_matrix
    r, cc = dm_sample_index(n)
    key = f"noisy_n{n}_d{depth}"
    out = {
        f"{key}_diag": np.real(np.diagonal(rho)).copy(),
        f"{key}_rows": r,
        f"{key}_cols": cc,
        f"{key}_entries": rho[r, cc],
        f"{key}_trace": np.trace(rho),
    }
    return out, f"density n={n} d={depth}: {time.time() - t:.1f} s"


def job_qaoa(args):
    path, n = args
    cirq = _reference(path)
    from cirq_gb300 import workloads

    circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(n, 4, seed=n)
    pts = workloads.qaoa_points(4, QAOA_POINTS, seed=100 + n)
    res = [cirq.ParamResolver({**dict(zip(gammas, q[:4])), **dict(zip(betas, q[4:]))}) for q in pts]
    t = time.time()
    vals = cirq.Simulator(dtype=np.complex128).simulate_expectation_values_sweep(circuit, [obs], res)
    out = {f"qaoa_n{n}_points": pts, f"qaoa_n{n}_expect": np.array([v[0] for v in vals])}
    return out, f"qaoa n={n}: {time.time() - t:.1f} s"


def hea_problem(cirq):
    from cirq_gb300 import workloads

    circuit, symbols, values = workloads.hea_circuit(HEA_N, HEA_LAYERS, seed=0)
    ham = workloads.random_pauli_hamiltonian(HEA_N, HEA_TERMS, seed=1)
    return circuit, symbols, values, ham


def job_hea(args):
    """Energies at the given shifted parameter vectors (rows of `vals`)."""
    path, rows = args
    cirq = _reference(path)
    circuit, symbols, values, ham = hea_problem(cirq)
    t = time.time()
    res = [cirq.ParamResolver(dict(zip(symbols, v))) for v in rows]
    e = cirq.Simulator(dtype=np.complex128).simulate_expectation_values_sweep(circuit, [ham], res)
    return np.array([np.real(x[0]) for x in e]), f"hea {len(rows)} points: {time.time() - t:.1f} s"


def main(path: str) -> None:
    cirq = _reference(path)
    circuit, symbols, values, ham = hea_problem(cirq)
    P = len(symbols)
    # energy, then +pi/2 and -pi/2 shifts of every parameter (rx(t), rz(t): exact
    # two-term shift rule dE/dt = (E(t + pi/2) - E(t - pi/2)) / 2)
    rows = [values.copy()]
    for i in range(P):
        for s in (+1, -1):
            v = values.copy()
            v[i] += s * np.pi / 2
            rows.append(v)
    rows = np.array(rows)
    chunks = np.array_split(np.arange(len(rows)), 24)

    jobs = [(job_layers, (path, 24, 40, 0, False)), (job_layers, (path, 20, 20, 0, True)),
            (job_density, (path, 11, 16))]
    jobs += [(job_qaoa, (path, n)) for n in QAOA_WIDTHS]
    jobs += [(job_hea, (path, rows[ch])) for ch in chunks]
    out: dict = {}
    hea_e = [None] * len(chunks)
    t0 = time.time()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, os.cpu_count() or 1)) as pool:
        handles = [pool.apply_async(fn, (a,)) for fn, a in jobs]
        for j, h in enumerate(handles):
            res, msg = h.get()
            print(msg, flush=True)
            if jobs[j][0] is job_hea:
                hea_e[j - (len(jobs) - len(chunks))] = res
            else:
                out.update(res)
    e = np.concatenate(hea_e)
    out["hea_n16_l10_values"] = values
    out["hea_n16_l10_energy"] = np.float64(e[0])
    out["hea_n16_l10_grad_ps"] = (e[1::2] - e[2::2]) / 2
    np.savez_compressed(OUT, **out)
    with open(OUT.replace(".npz", "_meta.txt"), "w") as f:
        f.write(f"generated by tests/golden/make_golden_large.py with cirq {cirq.__version__}\n")
        for k in sorted(out):
            a = np.asarray(out[k])
            f.write(f"{k}: shape={a.shape} dtype={a.dtype}\n")
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.0f} KB) in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CIRQ_REFERENCE_PATH")
    if not ref:
        sys.exit("usage: make_golden_large.py <path to the reference's cirq-core> (or set CIRQ_REFERENCE_PATH)")
    main(ref)
