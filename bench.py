"""Benchmark: 30-qubit random-layer circuit, gate-updates/s and HBM roofline.

Workload (one "step"): simulate the 30-qubit, depth-40 random-layer circuit
(PhasedXZ(x, z, a ~ U(-1,1)) on every qubit, then CZ on alternating pairs;
1780 gates) from |0...0> on one GB300: prepare the basis state and run every
fused tile pass of the plan.  The 8 GiB state is larger than L2, so no L2
flush is needed between steps.

Printed JSON line (rank 0):
  value      gate-updates/s = gates / device time per step (state resident in HBM)
  e2e        the same metric through cirq_gb300.Simulator.simulate() -- circuit
             in, final state vector out in host memory (H2D of the matrix pool
             and D2H of the 8 GiB state inside the timed region)
  roofline   dominant kernel (k_jit, the pass-specialised tile kernels; k_tile_ws
             where none is built): algorithmic bytes per launch (16 B x 2^30:
             one read + one write of the state) / mean launch time
  cpu_baseline  the reference's numpy cirq.Simulator on a bounded gate sample
  fusion_sweep  gate-updates/s for fusion width k = 1..5

`--extra-only NAME` runs one secondary workload (adjoint, density_matrix,
clifford_sampling, ...) and prints its JSON (with --no-cpu, the Clifford
line skips timing the reference's sampler).

`--impl reference` times the reference (cirq.Simulator, complex64) on the
host cores instead and prints the reference line.  Under torchrun with N > 1
every rank simulates its own replica (replicas only: the workload is one
state per GPU, with no exchange step); value = N x gates / max time over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "30q gate-updates/s & % HBM peak; 24q adjoint grads/s vs plain param-shift"
UNIT = "gate-updates/s"


def _cirq():
    from cirq_gb300._cirq_env import ensure_cirq

    return ensure_cirq((os.path.join(ROOT, "baseline", "_ref"),))


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks/throttle reasons while the timed region runs."""

    Q = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        return {
            "sm_mhz": statistics.median(sm),
            "sm_max_mhz": mx,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def build_workload(n: int, depth: int, seed: int):
    from cirq_gb300 import workloads

    circuit = workloads.random_layer_circuit(n, depth, seed)
    return circuit, len(list(circuit.all_operations()))


def compile_plan(circuit, planner):
    cirq = _cirq()
    from cirq_gb300.program import CompiledCircuit, split_measurements

    body, _ = split_measurements(circuit)
    qubits = sorted(circuit.all_qubits())
    return CompiledCircuit(body, qubits, dm=False, planner=planner, resolvers=[cirq.ParamResolver({})])


def device_steps(eng, compiled, steps: int, warmup: int, pass_timing: bool):
    """Times `steps` simulations with the state resident in HBM.

    Returns (ms per step, mean tile-pass launch ms, tile-pass launches per step,
    kernel launches per step)."""
    nbits = compiled.nbits_dev
    state = eng.alloc(8 << nbits)
    pool = eng.upload(compiled.plan.pool)
    plan = compiled.plan

    from cirq_gb300._lib import check

    def one():
        check(eng.lib.gbq_sv_set_basis(eng.ctx, state.ptr, nbits, 0), "gbq_sv_set_basis")
        check(
            eng.lib.gbq_run(
                eng.ctx, state.ptr, nbits, plan.passes.ctypes.data, len(plan.passes),
                plan.ops.ctypes.data, len(plan.ops), pool.ptr,
            ),
            "gbq_run",
        )

    for _ in range(warmup):
        one()
    eng.sync()
    # steady state: the pass-specialised kernels queued by the first run are built
    eng.jit_wait()
    one()
    eng.sync()
    if pass_timing:
        eng.set_pass_timing(True)
    l0 = eng.launches()
    j0 = eng.jit_launches()
    eng.event(0)
    for _ in range(steps):
        one()
    eng.event(1)
    ms = eng.elapsed_ms(0, 1)
    launches = (eng.launches() - l0) / steps
    device_steps.jit_launches_per_step = (eng.jit_launches() - j0) / steps
    pass_ms, pass_n = (0.0, 0)
    if pass_timing:
        pass_ms, pass_n = eng.pass_timing()
        eng.set_pass_timing(False)
    state.free()
    pool.free()
    mean_pass = pass_ms / pass_n if pass_n else None
    return ms / steps, mean_pass, (pass_n / steps if pass_n else plan.npasses), launches


def e2e_steps(circuit, planner_kwargs, steps: int, warmup: int):
    """Times Simulator.simulate() end to end: returns (s per step, h2d bytes, d2h bytes)."""
    import cirq_gb300

    sim = cirq_gb300.Simulator(**planner_kwargs)
    a0 = sim.engine.pinned.allocations
    for _ in range(warmup):
        r = sim.simulate(circuit)
        vec = r.final_state_vector
        # drop the result so that its pinned host buffer returns to the pool
        # (a user's loop that keeps no result reuses one buffer per call)
        del r, vec
    sim.engine.jit_wait()
    times = []
    vec_bytes = 0
    for _ in range(steps):
        t = time.perf_counter()
        r = sim.simulate(circuit)
        vec = r.final_state_vector
        times.append(time.perf_counter() - t)
        vec_bytes = vec.nbytes
        del r, vec
    compiled = next(iter(sim._cache.values()))
    e2e_steps.pinned_allocations = sim.engine.pinned.allocations - a0
    return float(np.mean(times)), int(compiled.plan.pool.nbytes), int(vec_bytes)


def e2e_phases(circuit, planner_kwargs, repeats: int = 2):
    """Where the time of one Simulator.simulate() goes, step by step, with a
    device synchronisation after each step (so the steps do not overlap):
    compile (translation + planning; only on the first call, later calls hit
    the compile cache), pool (the fused matrices of the point), passes (pool
    upload, basis state and every tile pass), renormalise (the final-state
    rule: a norm pass, and a scale pass when it applies), d2h (the state into
    pinned host memory; d2h_gc and d2h_pin are the parts of it spent in a
    garbage collection that returned a buffer and in pinning a new one) and
    assemble (the cirq result object).  Returns
    {"first": {...}, "cached": {...}, "specialised_kernels_ready_s": T} in
    seconds: the first call runs the interpreter while the pass-specialised
    kernels of the circuit compile in the background (T after its start they
    are all built); the cached calls run them."""
    cirq = _cirq()
    import cirq_gb300
    from cirq_gb300 import simulator as sim_mod

    sim = cirq_gb300.Simulator(**planner_kwargs)
    eng = sim.engine
    out = {}
    t_first = time.perf_counter()
    for rep in range(repeats + 1):
        ph = {}
        t = time.perf_counter()
        qubits, resolvers, compiled, meas = sim._prepare(circuit, cirq.QubitOrder.DEFAULT, cirq.ParamResolver({}))
        ph["compile"] = time.perf_counter() - t
        t = time.perf_counter()
        pool = compiled.pool(resolvers or [cirq.ParamResolver({})])
        ph["pool"] = time.perf_counter() - t
        t = time.perf_counter()
        state = sim._evolve(compiled, pool[0], None)
        eng.sync()
        ph["passes"] = time.perf_counter() - t
        t = time.perf_counter()
        sim_mod._final_renormalize(eng, state, compiled.n)
        eng.sync()
        ph["renormalise"] = time.perf_counter() - t
        g0, p0 = eng.pinned.gc_seconds, eng.pinned.pin_seconds
        t = time.perf_counter()
        vec = eng.download_state(state, compiled.n)
        ph["d2h"] = time.perf_counter() - t
        ph["d2h_gc"] = eng.pinned.gc_seconds - g0
        ph["d2h_pin"] = eng.pinned.pin_seconds - p0
        state.free()
        t = time.perf_counter()
        res = sim_mod._state_vector_result(cirq.ParamResolver({}), {}, qubits, vec)
        ph["assemble"] = time.perf_counter() - t
        ph["total"] = sum(v for k, v in ph.items() if k not in ("d2h_gc", "d2h_pin"))
        ph["pinned_allocations_so_far"] = eng.pinned.allocations
        del res, vec
        if rep == 0:
            out["first"] = ph
            eng.jit_wait()
            ready = time.perf_counter() - t_first
        else:
            prev = out.get("cached")
            out["cached"] = ph if prev is None or ph["total"] < prev["total"] else prev
    res = {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()} for k, v in out.items()}
    res["specialised_kernels_ready_s"] = round(ready, 3)
    return res


def max_over_ranks(ms: float, dist=None, device: str = "cpu") -> float:
    """The slowest rank's time (every rank gets it); identity without torch.distributed."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_replica: float, ms_step: float, world: int) -> float:
    """Whole-job throughput of `world` independent replicas timed by the slowest."""
    return world * units_per_replica / (ms_step / 1e3)


# ---------------------------------------------------------------------------
# reference (numpy cirq.Simulator) timing on a bounded gate sample
def reference_gate_rates(n: int, circuit, sample_1q: int = 2, sample_2q: int = 1, repeat: int = 1):
    """Seconds per PhasedXZ and per CZ of the reference cirq.Simulator(complex64)
    on a dense n-qubit state (split_untangled_states=False, so no product-state
    shortcut).  Returns (s_per_1q, s_per_2q, sample description)."""
    cirq = _cirq()
    qubits = sorted(circuit.all_qubits())
    ops = list(circuit.all_operations())
    ones = [op for op in ops if len(op.qubits) == 1][:sample_1q]
    twos = [op for op in ops if len(op.qubits) == 2][:sample_2q]
    sim = cirq.Simulator(dtype=np.complex64, split_untangled_states=False)
    init = np.full(2**n, 2.0 ** (-n / 2), dtype=np.complex64)

    def timed(opl):
        c = cirq.Circuit(opl)
        best = None
        for _ in range(repeat):
            t = time.perf_counter()
            sim.simulate(c, qubit_order=qubits, initial_state=init)
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        return best

    t_empty = timed([cirq.I(qubits[0])])  # state setup + result assembly
    t1 = max(timed(ones) - t_empty, 1e-9) / max(len(ones), 1)
    t2 = max(timed(twos) - t_empty, 1e-9) / max(len(twos), 1)
    desc = (
        f"{len(ones)} PhasedXZ + {len(twos)} CZ of the workload on a dense {n}-qubit complex64 "
        f"state, setup subtracted; rate extrapolated to the workload's gate mix"
    )
    return t1, t2, desc


def component_sizes(circuit):
    """Per moment of `circuit`, the size of every operation's untangled
    component when the reference's default simulator (split_untangled_states
    on, cirq-core/cirq/sim/simulation_product_state.py) applies it: qubits
    join a component when an operation acts on them together."""
    parent = {q: q for q in circuit.all_qubits()}
    size = {q: 1 for q in parent}

    def find(q):
        while parent[q] != q:
            parent[q] = parent[parent[q]]
            q = parent[q]
        return q

    out = []
    for moment in circuit:
        sizes = []
        for op in moment:
            roots = list({find(q) for q in op.qubits})
            for r in roots[1:]:
                parent[r] = roots[0]
                size[roots[0]] += size[r]
            sizes.append(size[find(op.qubits[0])])
        out.append(sizes)
    return out


def reference_rate(n, circuit, max_component: int = 22):
    """Gate-updates/s of the reference's default cirq.Simulator(complex64)
    (product states on) on the workload: the moments whose components stay
    within `max_component` qubits are simulated in full by the reference
    itself; every later gate is charged the measured dense per-gate rate on
    an n-qubit state (reference_gate_rates) scaled by 2^(component size - n),
    the size of the tensor it acts on.  Returns (rate, seconds, description)."""
    cirq = _cirq()
    ops = list(circuit.all_operations())
    sizes = component_sizes(circuit)
    k = 0
    while k < len(sizes) and max(sizes[k], default=0) <= max_component:
        k += 1
    moments = list(circuit)
    prefix = cirq.Circuit(moments[:k])
    qubits = sorted(circuit.all_qubits())
    sim = cirq.Simulator(dtype=np.complex64)  # the default configuration
    t = time.perf_counter()
    sim.simulate(prefix, qubit_order=qubits)
    t_prefix = time.perf_counter() - t
    t1, t2, desc = reference_gate_rates(n, circuit)
    rest = 0.0
    nrest = 0
    for moment, sz in zip(moments[k:], sizes[k:]):
        for op, s in zip(moment, sz):
            rest += (t1 if len(op.qubits) == 1 else t2) * 2.0 ** (s - n)
            nrest += 1
    secs = t_prefix + rest
    nprefix = len(list(prefix.all_operations()))
    desc = (
        f"default cirq.Simulator (product states on): the first {k} moments ({nprefix} gates, components "
        f"<= {max_component} qubits) simulated in full in {t_prefix:.2f} s; the other {nrest} gates charged "
        f"the dense per-gate rate on the component they act on ({desc})"
    )
    return len(ops) / secs, secs, desc


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    _cirq()  # the reference install under baseline/_ref
    circuit, ngates = build_workload(args.n, args.depth, args.seed)
    vals = []
    desc = ""
    for i in range(args.warmup + args.steps):
        v, secs, desc = reference_rate(args.n, circuit)
        if i >= args.warmup:
            vals.append(v)
    v = float(np.mean(vals))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * ngates / v,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64",
        "data": "synthetic",
        "config": {"workload": f"random-layer circuit {args.n}q depth {args.depth} ({ngates} gates), seed {args.seed}"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "reference",
                         "sample": desc + " (numpy path is single-threaded)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# secondary workloads (reported beside the headline number)
def adjoint_bench(n: int = 24, layers: int = 10, terms: int = 300, reps: int = 3, ps_params: int = 16):
    """Gradient of <H> for the hardware-efficient ansatz (rx/rz layers + CZ
    ladder, 480 parameters at 24 qubits, H = 300 random Pauli strings of
    weight 2..4): adjoint gradients per second through AdjointProgram, and
    parameter shift through the plain GPU simulator (simulate_expectation_values_sweep,
    2 evaluations per parameter) timed on `ps_params` parameters and
    extrapolated to all of them."""
    import cirq_gb300
    from cirq_gb300 import adjoint, workloads

    circuit, symbols, values = workloads.hea_circuit(n, layers, seed=0)
    ham = workloads.random_pauli_hamiltonian(n, terms, seed=1)
    prog = adjoint.AdjointProgram(circuit, ham, symbols)
    prog.value_and_grad(values)  # warm-up
    prog.engine.jit_wait()  # steady state: the specialised kernels are built
    t = time.perf_counter()
    for _ in range(reps):
        e, g = prog.value_and_grad(values)
    t_adj = (time.perf_counter() - t) / reps
    sim = cirq_gb300.Simulator()
    idx = list(range(ps_params))
    adjoint.parameter_shift_gradient(sim, circuit, ham, symbols, values, indices=idx[:1])  # warm-up
    t = time.perf_counter()
    ps = adjoint.parameter_shift_gradient(sim, circuit, ham, symbols, values, indices=idx)
    t_ps = (time.perf_counter() - t) * len(symbols) / len(idx)
    # algorithmic HBM bytes of one gradient: forward passes (one read + one
    # write of psi), lam = H psi (per tiled pass: a read of psi and a write
    # of lam, plus a read of lam after the first; per group of wide terms
    # with the same X mask: a read of psi, a read and a write of lam),
    # <lam|psi> (two reads) and the reverse two-state passes (read + write
    # of psi and lam)
    amp = 8 * (1 << prog.nbits)
    xgroups = len({t[0] for t in prog.terms})
    hp_passes, hp_wide = prog.engine.paulisum_cover(prog.n, prog.terms)
    # wide terms: more than nine X/Y factors on qubits 4 and up
    wide_groups = len({t[0] for t in prog.terms if bin(t[0] >> 4).count("1") > 9}) if hp_wide else 0
    hpsi = max(0, 3 * hp_passes - 1) + (wide_groups + 2 if hp_wide else 0)
    alg_bytes = (2 * prog.forward.plan.npasses + hpsi + 2 + 4 * prog.reverse.npasses) * amp
    peak, peak_kind = peaks()
    return {
        "workload": f"HEA {n}q x {layers} layers ({len(symbols)} params), H = {terms} Pauli strings",
        "grads_per_s": 1.0 / t_adj,
        "hbm_bytes_per_grad": alg_bytes,
        "passes": {"forward": int(prog.forward.plan.npasses), "reverse_two_state": int(prog.reverse.npasses),
                   "h_psi_x_groups": xgroups, "h_psi_tiled_passes": hp_passes, "h_psi_wide_terms": hp_wide},
        "hbm_frac_of_wall_time": alg_bytes / t_adj / 1e9 / peak,
        "hbm_frac_note": f"algorithmic bytes / wall time per gradient (host work included) / {peak_kind} hbm_gbs",
        "s_per_grad": t_adj,
        "param_shift_s_per_grad": t_ps,
        "param_shift_sample": f"{len(idx)} of {len(symbols)} parameters timed, extrapolated",
        "speedup_vs_param_shift": t_ps / t_adj,
        "max_abs_diff_vs_param_shift": float(np.max(np.abs(g[idx] - ps[idx]))),
        "energy": e,
    }


def density_bench(n: int = 13, depth: int = 16):
    """Noisy density matrix: random layers, depolarize(1e-3) after every gate
    on each of its qubits, amplitude_damp(5e-3) on all qubits per layer;
    rho = 2^26 complex64 (512 MiB)."""
    import cirq_gb300
    from cirq_gb300 import workloads

    c = workloads.noisy_layer_circuit(n, depth, seed=0, p=1e-3, gamma=5e-3)
    nops = len(list(c.all_operations()))
    sim = cirq_gb300.DensityMatrixSimulator()
    r = sim.simulate(c)
    rho = r.final_density_matrix
    del r, rho  # its pinned host buffer returns to the pool for the timed call
    sim.engine.jit_wait()  # steady state: the passes' specialised kernels are built
    times = []
    for _ in range(3):
        t = time.perf_counter()
        r = sim.simulate(c)
        rho = r.final_density_matrix
        times.append(time.perf_counter() - t)
        if len(times) < 3:
            del r, rho
    dt = min(times)
    compiled = next(iter(sim._cache.values()))
    # the same passes with rho resident in HBM (the C3 roofline figure)
    ms, pass_ms, npass, _ = device_steps(sim.engine, compiled, 3, 2, True)
    peak, _ = peaks()
    pass_bytes = 16 * (1 << compiled.nbits)
    return {
        "workload": f"noisy layers {n}q depth {depth} ({nops} ops incl. channels)",
        "s_per_simulate": dt,
        "ops_per_s": nops / dt,
        "device_ms_per_simulate": ms,
        "mean_pass_ms": pass_ms,
        "hbm_frac_per_pass": (pass_bytes / (pass_ms / 1e3) / 1e9 / peak) if pass_ms else None,
        "passes": int(compiled.plan.npasses),
        "trace": float(np.real(np.trace(rho))),
        "hermiticity_err": float(np.max(np.abs(rho - rho.conj().T))),
    }


def batch_bench(points: int = 4096, widths=(16, 18, 20, 22), p: int = 4):
    """QAOA p=4 on seeded random 3-regular graphs, <sum Z_i Z_j> for `points`
    parameter points split evenly over the widths, one persistent launch."""
    import cirq

    from cirq_gb300 import batch, workloads

    jobs = []
    per = points // len(widths)
    for w in widths:
        circuit, gammas, betas, obs, edges = workloads.qaoa_circuit(w, p, seed=w)
        pts = workloads.qaoa_points(p, per, seed=100 + w)
        res = [cirq.ParamResolver({**dict(zip(gammas, q[:p])), **dict(zip(betas, q[p:]))}) for q in pts]
        jobs.append(batch.BatchJob(circuit, obs, res))
    batch.simulate_expectation_values_batch(jobs[:1])  # warm-up
    batch.simulate_expectation_values_batch(jobs[:1], persistent=True)
    t = time.perf_counter()
    vals = batch.simulate_expectation_values_batch(jobs)
    dt = time.perf_counter() - t
    t = time.perf_counter()
    vals_p = batch.simulate_expectation_values_batch(jobs, persistent=True)
    dt_p = time.perf_counter() - t
    # algorithmic HBM bytes: per point, every pass reads and writes its state,
    # then one read of the state per group of terms with the same X mask
    alg_bytes = 0
    for job in jobs:
        amp = 8 * (1 << job.compiled.nbits_dev)
        xg = len({t[0] for obs in job.terms for t in obs})
        alg_bytes += len(job.resolvers) * (2 * job.compiled.plan.npasses + xg) * amp
    peak, peak_kind = peaks()
    return {
        "workload": f"QAOA p={p}, {points} points over widths {list(widths)}",
        "points_per_s": points / dt,
        "hbm_bytes_total": alg_bytes,
        "passes_per_point": {str(j.n): int(j.compiled.plan.npasses) for j in jobs},
        "hbm_frac_of_wall_time": alg_bytes / dt / 1e9 / peak,
        "hbm_frac_note": f"algorithmic bytes / wall time (host pool building included) / {peak_kind} hbm_gbs",
        "s_total": dt,
        "mode": "points of a job evolved together (one tile-pass launch per pass)",
        "persistent_single_launch_s_total": dt_p,
        "max_abs_diff_between_modes": float(max(np.abs(a - b).max() for a, b in zip(vals, vals_p))),
        "mean_expectation": float(np.mean([np.real(v).mean() for v in vals])),
    }


def clifford_bench(n: int = 500, depth: int = 100, shots: int = 1_000_000, ref_shots: int = 1):
    """Clifford sampling: a random Clifford circuit of n qubits and depth
    layers with a mid-circuit measurement and reset every layer, depolarizing
    noise and a final measurement of every qubit, sampled `shots` times by
    Pauli frames on the GPU; the reference's cirq.StabilizerSampler (one
    tableau run per repetition) is timed on `ref_shots` repetitions (0:
    not timed).
    Frame-kernel bytes: per op and 32 shots, the frame and record words it
    reads and writes (4 B each)."""
    cirq = _cirq()
    from cirq_gb300 import clifford as C, workloads
    from cirq_gb300.engine import Engine
    from cirq_gb300 import _lib as L

    eng = Engine.get(0)
    c = workloads.random_clifford_circuit(n, depth, 0, mid_measure=1.0, resets=True, p=1e-3)
    q = sorted(c.all_qubits())
    t = time.perf_counter()
    prog = C.CliffordProgram(c, q)
    compile_s = time.perf_counter() - t
    t = time.perf_counter()
    prog.reference(eng)
    reference_s = time.perf_counter() - t
    nw = (shots + 31) // 32
    words = 2 * n  # frame initialisation
    for op in prog.ops:
        kind, k = int(op["kind"]), int(op["k"])
        words += {L.CLIFF_UNITARY: 4 * k, L.CLIFF_MEASURE: 4, L.CLIFF_RESET: 2, L.CLIFF_NOISE: 4,
                  L.CLIFF_COND_PAULI: 2 * k + int(op["cond_count"])}[kind]
    alg_bytes = words * 4 * nw
    prog.sample_records(eng, 4096, 1)  # warm-up
    dev = []
    wall = []
    for rep in range(3):
        eng.set_pass_timing(True)
        t = time.perf_counter()
        prog.sample_records(eng, shots, 100 + rep)
        wall.append(time.perf_counter() - t)
        ms, nlaunch = eng.pass_timing()
        eng.set_pass_timing(False)
        dev.append(ms)
    t = time.perf_counter()
    res = C.StabilizerSampler(seed=5).run(c, repetitions=shots)
    api_s = time.perf_counter() - t
    ref_s = None
    if ref_shots:
        t = time.perf_counter()
        cirq.StabilizerSampler(seed=5).run(c, repetitions=ref_shots)
        ref_s = (time.perf_counter() - t) / ref_shots
    peak, _ = peaks()
    dev_s = min(dev) / 1e3
    return {
        "workload": f"random Clifford circuit {n}q depth {depth}, a measurement + reset per layer, "
                    f"depolarize(1e-3), {prog.nrec} records, {len(prog.ops)} ops",
        "shots": shots,
        "shots_per_s_device": shots / dev_s,
        "shots_per_s_api": shots / api_s,
        "api_s": api_s,
        "device_ms": min(dev),
        "device_ms_note": "the frame kernel alone (CUDA events around its launch)",
        "wall_s_sample_records": min(wall),
        "wall_note": "one gbq_cliff_sample call: uploads, reference records, frame kernel, on-device transpose "
                     "to shot-major bytes and their download",
        "compile_s": compile_s,
        "reference_run_s": reference_s,
        "frame_bytes": alg_bytes,
        "frame_gbs_of_device_time": alg_bytes / dev_s / 1e9,
        "frame_hbm_frac": alg_bytes / dev_s / 1e9 / peak,
        "frame_note": "frames + records are 2*n*nw + nrec*nw words; at these sizes much of the traffic stays in L2",
        "reference_shots_per_s": 1.0 / ref_s if ref_s else None,
        "reference_sample": f"cirq.StabilizerSampler, {ref_shots} repetitions",
        "speedup_api_vs_reference": (shots / api_s) * ref_s if ref_s else None,
        "result_shape": list(res.measurements["m"].shape),
    }


def c1_bench(n: int = 20, depth: int = 20, reps: int = 10_000, calls: int = 5):
    """The CPU-runnable configuration: 20 qubits, depth 20 (590 gates).
    simulate() latency (first call, with planning, and cached) and
    run(repetitions=10^4) measuring every qubit, through the public API,
    beside the reference's cirq.Simulator(dtype=complex64) on the same
    circuits in the same process (one host core: numpy's path is
    single-threaded).  The 8 MiB state fits in L2, so there is no HBM
    roofline here: the figures are latencies."""
    cirq = _cirq()
    import cirq_gb300

    circuit, ngates = build_workload(n, depth, 0)
    q = sorted(circuit.all_qubits())
    measured = circuit + cirq.measure(*q, key="m")

    def timed(fn, k):
        best = None
        for _ in range(k):
            t = time.perf_counter()
            fn()
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        return best

    sim = cirq_gb300.Simulator()
    t = time.perf_counter()
    sim.simulate(circuit).final_state_vector
    first = time.perf_counter() - t
    sim.engine.jit_wait()  # steady state: the specialised kernels are built
    ours_sim = timed(lambda: sim.simulate(circuit).final_state_vector, calls)
    sim.run(measured, repetitions=reps)
    sim.engine.jit_wait()
    ours_run = timed(lambda: sim.run(measured, repetitions=reps), calls)
    ref = cirq.Simulator(dtype=np.complex64)
    ref_sim = timed(lambda: ref.simulate(circuit).final_state_vector, 1)
    ref_run = timed(lambda: ref.run(measured, repetitions=reps), 1)
    return {
        "workload": f"random-layer circuit {n}q depth {depth} ({ngates} gates), seed 0",
        "simulate_s_first_call": first,
        "simulate_s": ours_sim,
        "run_10k_s": ours_run,
        "reference_simulate_s": ref_sim,
        "reference_run_10k_s": ref_run,
        "speedup_simulate": ref_sim / ours_sim,
        "speedup_run": ref_run / ours_run,
        "gate_updates_per_s": ngates / ours_sim,
        "reference_cores": 1,
        "note": "state (8 MiB) is L2-resident: latency figures, no HBM roofline",
    }


def width33_bench(depth: int = 40, steps: int = 2):
    """The 33-qubit form of the headline workload (64 GiB state, same
    construction): gate-updates/s and the HBM fraction of the tile passes."""
    from cirq_gb300.engine import Engine
    from cirq_gb300.planner import Planner

    eng = Engine.get(0)
    _, free, _ = eng.device_info()
    if free < (70 << 30):
        return {"skipped": f"needs 70 GiB free device memory, {free >> 30} GiB free"}
    circuit, ngates = build_workload(33, depth, 0)
    compiled = compile_plan(circuit, Planner(tile_bits=12, kmax=4, budget=25.0))
    ms, pass_ms, passes, _ = device_steps(eng, compiled, steps, 1, pass_timing=True)
    peak, _ = peaks()
    return {
        "workload": f"random-layer circuit 33q depth {depth} ({ngates} gates), seed 0",
        "gate_updates_per_s": ngates / (ms / 1e3),
        "ms_per_step": ms,
        "passes": passes,
        "hbm_frac": 16 * (1 << 33) / (pass_ms / 1e3) / 1e9 / peak if pass_ms else None,
    }


def tc_bench(n: int = 30, depth: int = 40, budgets=(3, 4, 6), steps: int = 2):
    """The pipelined tensor-core pass (k_tc_pass: 12-bit tiles, 4-qubit blocks
    as tcgen05 TF32 three-term MMAs) on the headline workload, against the
    CUDA-core plan of the headline line: ms per step and per pass, passes,
    and the HBM fraction per pass, for a few MMA-op budgets per pass."""
    from cirq_gb300.engine import Engine
    from cirq_gb300.planner import Planner

    eng = Engine.get(0)
    circuit, ngates = build_workload(n, depth, 0)
    peak, _ = peaks()
    out = {"workload": f"random-layer circuit {n}q depth {depth} ({ngates} gates), seed 0"}
    for b in budgets:
        ck = compile_plan(circuit, Planner(tensor=True, budget=b))
        ms, pms, npass, _ = device_steps(eng, ck, steps, 1, pass_timing=True)
        mma = int((ck.plan.ops["kind"] == 9).sum())
        out[f"mma_ops_per_pass_{b}"] = {
            "gate_updates_per_s": ngates / (ms / 1e3),
            "ms_per_step": ms,
            "passes": int(ck.plan.npasses),
            "mma_ops": mma,
            "mean_pass_ms": pms,
            "hbm_frac": 16 * (1 << ck.nbits) / (pms / 1e3) / 1e9 / peak if pms else None,
        }
    return out


def mma_bench(n: int = 30, reps: int = 3):
    """Tensor-core evaluation: one 11-bit-tile pass applying 1, 2 or 4
    random 4-qubit matrices with tcgen05 MMAs (GBQ_OP_MMA, TF32 three-term
    split) against the same program on the FP32 CUDA-core path (plain dense
    ops), ms per pass on a 2^n state resident in HBM."""
    from cirq_gb300 import _lib
    from cirq_gb300.engine import Engine

    eng = Engine.get(0)
    rs = np.random.RandomState(0)
    state = eng.alloc(8 << n)
    check = _lib.check
    out = {"workload": f"{n}q state, one pass, 4-qubit matrices on tile bits (3o + j) mod 11"}
    try:
        check(eng.lib.gbq_sv_set_basis(eng.ctx, state.ptr, n, 0))
        for nm in (1, 2, 4):
            ops = np.zeros(nm, dtype=_lib.OP_DTYPE)
            pool = []
            for o in range(nm):
                ops[o]["kind"] = _lib.OP_MMA
                ops[o]["k"] = 4
                ops[o]["bits"][:4] = [(3 * o + j) % 11 for j in range(4)]
                ops[o]["mat"] = 256 * o
                a = rs.normal(size=(16, 16)) + 1j * rs.normal(size=(16, 16))
                pool.append(np.linalg.qr(a)[0].astype(np.complex64).reshape(-1))
            passes = np.zeros(1, dtype=_lib.PASS_DTYPE)
            passes[0]["L"], passes[0]["m"], passes[0]["op_count"] = 11, 5, nm
            passes[0]["hi"][:6] = list(range(5, 11))
            pool_dev = eng.upload(np.concatenate(pool))
            row = {}
            for label, kind in (("mma_ms", _lib.OP_MMA), ("fp32_ms", _lib.OP_DENSE)):
                ops["kind"] = kind

                def one():
                    check(eng.lib.gbq_run(eng.ctx, state.ptr, n, passes.ctypes.data, 1, ops.ctypes.data, nm,
                                          pool_dev.ptr), "gbq_run")

                one()
                eng.event(0)
                for _ in range(reps):
                    one()
                eng.event(1)
                row[label] = eng.elapsed_ms(0, 1) / reps
            eng.sync()
            pool_dev.free()
            out[f"{nm}_ops"] = row
    finally:
        state.free()
    return out


# ---------------------------------------------------------------------------
def extra_benches() -> dict:
    """The secondary workloads reported under "extra" (name -> function)."""
    return {"c1_20q": c1_bench, "adjoint": adjoint_bench, "density_matrix": density_bench,
            "batch_sweep": batch_bench, "clifford_sampling": clifford_bench, "width_33": width33_bench,
            "tensor_core_pipelined": tc_bench, "tensor_core_pass_11bit": mma_bench}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=30)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tile-bits", type=int, default=12)
    ap.add_argument("--kmax", type=int, default=4)
    ap.add_argument("--budget", type=float, default=25.0)
    ap.add_argument("--tensor-cores", type=int, default=0, help="plan tensor-core passes with this many MMA ops per pass")
    ap.add_argument("--jit", type=int, default=None, help="pass-specialised kernels: 1 on, 0 off (default: library default)")
    ap.add_argument("--no-sweep", action="store_true", help="skip the fusion-width sweep")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the adjoint / density / batch lines")
    ap.add_argument("--extra-only", default=None, help="run only this secondary workload and print its JSON")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    if args.impl == "reference":
        return run_reference(args)
    if args.extra_only:
        _cirq()
        benches = extra_benches()
        if args.extra_only not in benches:
            ap.error(f"--extra-only: one of {', '.join(benches)}")
        fn = benches[args.extra_only]
        if args.no_cpu and args.extra_only == "clifford_sampling":
            result = fn(ref_shots=0)  # the reference sampler takes about a minute per shot
        else:
            result = fn()
        print(json.dumps({args.extra_only: result}))
        return 0

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    _cirq()
    from cirq_gb300.engine import Engine
    from cirq_gb300.planner import Planner

    eng = Engine.get(local)
    if args.jit is not None:
        eng.set_jit(bool(args.jit))
    circuit, ngates = build_workload(args.n, args.depth, args.seed)
    if args.tensor_cores:
        planner = Planner(tensor=True, budget=args.tensor_cores)
    else:
        planner = Planner(tile_bits=args.tile_bits, kmax=args.kmax, budget=args.budget)
    t0 = time.perf_counter()
    compiled = compile_plan(circuit, planner)
    plan_s = time.perf_counter() - t0

    def barrier():
        if dist is not None:
            dist.barrier()

    kw = dict(tile_bits=args.tile_bits, fusion_max_qubits=args.kmax, pass_budget=args.budget)
    if args.tensor_cores:
        kw = dict(tensor_cores=True, mma_ops_per_pass=args.tensor_cores)
    # first: the per-phase breakdown, whose first call is the process's first
    # sight of this circuit structure (no specialised kernel cached yet)
    phases = e2e_phases(circuit, kw) if not args.no_e2e and rank == 0 else None

    barrier()
    with ClockSampler(local) as clocks:
        ms_step, pass_ms, passes_per_step, launches = device_steps(
            eng, compiled, args.steps, args.warmup, pass_timing=True
        )
    barrier()
    ms_step = max_over_ranks(ms_step, dist, device=f"cuda:{local}")
    value = replica_value(ngates, ms_step, world)

    peak, peak_kind = peaks()
    alg_bytes = 16 * (1 << compiled.nbits)
    achieved = alg_bytes / (pass_ms / 1e3) / 1e9 if pass_ms else None
    traffic = None
    jit_per_step = getattr(device_steps, "jit_launches_per_step", 0)
    kernel = "k_jit (pass-specialised k_tile_ws)" if jit_per_step >= 0.5 * passes_per_step else "k_tile_ws"
    tpath = os.path.join(ROOT, "profiles", "jit_pass_traffic.json" if kernel.startswith("k_jit") else "tile_ws_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if tj.get("nbits") and tj.get("dram_bytes_per_launch"):
            traffic = tj["dram_bytes_per_launch"] * (1 << compiled.nbits) / (1 << tj["nbits"])

    e2e = None
    if not args.no_e2e and rank == 0:
        e2e_s, h2d, d2h = e2e_steps(circuit, kw, steps=min(args.steps, 3), warmup=1)
        e2e = {"value": ngates / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "s_per_step": e2e_s, "pinned_host_allocations": getattr(e2e_steps, "pinned_allocations", None),
               "phases_s": phases}

    sweep = None
    if not args.no_sweep and rank == 0:
        sweep = {}
        for k in range(1, 6):
            pk = Planner(tile_bits=args.tile_bits, kmax=k, budget=args.budget)
            ck = compile_plan(circuit, pk)
            msk, pmk, ppk, _ = device_steps(eng, ck, 2, 1, pass_timing=True)
            sweep[str(k)] = {
                "gate_updates_per_s": ngates / (msk / 1e3),
                "passes": int(ck.plan.npasses),
                "ms_per_step": msk,
                "hbm_frac": (16 * (1 << ck.nbits) / (pmk / 1e3) / 1e9) / peak if pmk else None,
            }

    cpu = None
    if not args.no_cpu and rank == 0:
        try:
            v, secs, desc = reference_rate(args.n, circuit)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "reference",
                   "sample": desc + " (numpy path is single-threaded)"}
        except MemoryError as e:  # pragma: no cover
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "reference", "sample": f"failed: {e}"}

    extra = {}
    if not args.no_extra and rank == 0:
        for name, fn in extra_benches().items():
            try:
                extra[name] = fn()
            except Exception as e:  # reported, not hidden
                extra[name] = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "c64",
            "data": "synthetic",
            "config": {
                "workload": f"random-layer circuit {args.n}q depth {args.depth} ({ngates} gates), seed {args.seed}",
                "state_bytes": 8 << compiled.nbits,
                "l2": "state (8 GiB) larger than L2; no flush needed",
                "tile_bits": args.tile_bits,
                "fusion_max_qubits": args.kmax,
                "pass_budget": args.budget,
                "passes_per_step": int(compiled.plan.npasses),
                "fused_ops": int(len(compiled.plan.ops)),
                "plan_seconds": round(plan_s, 3),
                "parallelism": f"replicas x{world}",
            },
            "hbm_frac": (achieved / peak) if achieved else None,
            "roofline": {
                "kernel": kernel,
                "bound": "hbm",
                "achieved": achieved,
                "peak": peak,
                "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": traffic,
                "algorithmic_bytes_per_launch": alg_bytes,
                "mean_launch_ms": pass_ms,
                "launches_per_step": passes_per_step,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            },
            "gpu_launches": int(round(launches * args.steps)),
            "specialised_passes": {"launches_per_step": jit_per_step, "kernels_compiled": eng.jit_compiles(),
                                   "mode": 0 if args.jit == 0 else (args.jit or 2)},
            "clocks": clocks.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "fusion_sweep": sweep,
            **extra,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
