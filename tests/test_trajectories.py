"""Trajectory planning (mid-circuit measurement, state-vector noise): host
logic only, no GPU."""

import numpy as np

import cirq
from cirq_gb300 import trajectories as tj
from cirq_gb300.ir import flatten_ops
from cirq_gb300.planner import Planner
from cirq_gb300.program import CompiledCircuit, Slot, TrajectoryPoint
from emulator import run_program


def _ops(c):
    return flatten_ops(c)


def test_needs_trajectories():
    q = cirq.LineQubit.range(2)
    terminal = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(*q), cirq.measure(*q, key="m"))
    mid = cirq.Circuit(cirq.H(q[0]), cirq.measure(q[0], key="a"), cirq.H(q[0]), cirq.measure(q[0], key="b"))
    noisy = cirq.Circuit(cirq.X(q[0]), cirq.amplitude_damp(0.1)(q[0]), cirq.measure(q[0], key="m"))
    assert not tj.needs_trajectories(_ops(terminal), dm=False)
    assert tj.needs_trajectories(_ops(mid), dm=False)
    assert tj.needs_trajectories(_ops(mid), dm=True)
    assert tj.needs_trajectories(_ops(noisy), dm=False)
    assert not tj.needs_trajectories(_ops(noisy), dm=True)


def test_build_items_splits_at_events_and_keeps_mixtures_fused():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.H(q[0]),
        cirq.depolarize(0.1)(q[0]),  # mixture: a slot inside the segment
        cirq.CNOT(q[0], q[1]),
        cirq.measure(q[1], key="a"),
        cirq.amplitude_damp(0.2)(q[2]),  # general channel: an event
        cirq.X(q[2]),
        cirq.measure(q[2], key="b"),
        strategy=cirq.InsertStrategy.NEW,
    )
    items, nslot = tj.build_items(_ops(c), dm=False)
    kinds = [type(it).__name__ for it in items]
    assert kinds == ["Segment", "Measure", "Channel", "Segment", "Measure"]
    assert nslot == 2
    seg = items[0]
    assert any(isinstance(op, Slot) for op in seg.ops) and len(seg.slots) == 1
    # density matrices keep every channel in the segments
    items_dm, nslot_dm = tj.build_items(_ops(c), dm=True)
    assert [type(it).__name__ for it in items_dm] == ["Segment", "Measure", "Segment", "Measure"]
    assert nslot_dm == 0


def test_slot_pool_follows_the_picks():
    """A slot is planned as a dense op and takes each point's picked matrix."""
    q = cirq.LineQubit.range(3)
    dep = cirq.depolarize(0.3)(q[1])
    ops = [cirq.H(q[0]), Slot(dep, 0), cirq.CNOT(q[0], q[2])]
    cc = CompiledCircuit(ops, q, dm=False, planner=Planner(tile_bits=10), resolvers=[cirq.ParamResolver({})])
    probs, unitaries = zip(*cirq.mixture(dep))
    n = cc.nbits_dev
    for i, u in enumerate(unitaries):
        pool = cc.pool([TrajectoryPoint(cirq.ParamResolver({}), {0: u})])[0]
        psi0 = np.zeros(2**n, complex)
        psi0[0] = 1
        out = run_program(psi0, n, cc.plan.passes, cc.plan.ops, pool.astype(np.complex128))[:8]
        ref = cirq.final_state_vector(cirq.Circuit(cirq.H(q[0]), cirq.MatrixGate(u)(q[1]), cirq.CNOT(q[0], q[2])),
                                      qubit_order=q)
        assert np.allclose(out, ref, atol=1e-6), i


def test_pad_records_matches_reference_layout():
    recs = [{"a": [[1, 0]], "b": [[1]]}, {"a": [[0, 1], [1, 1]]}]
    out = tj.pad_records(recs)
    assert out["a"].shape == (2, 2, 2) and out["a"].dtype == np.uint8
    assert out["a"][0, 0].tolist() == [1, 0] and out["a"][0, 1].tolist() == [0, 0]
    assert out["b"].shape == (2, 1, 1) and out["b"][1, 0, 0] == 0


def test_classical_control_becomes_a_conditional_item():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(
        cirq.H(q[0]),
        cirq.measure(q[0], key="a"),
        cirq.X(q[1]).with_classical_controls("a"),
        cirq.CNOT(q[1], q[2]),
    )
    ops = flatten_ops(c)
    assert tj.needs_trajectories(ops, dm=False) and tj.needs_trajectories(ops, dm=True)
    items, _ = tj.build_items(ops, dm=False)
    kinds = [type(it).__name__ for it in items]
    assert kinds == ["Segment", "Measure", "Conditional", "Segment"]
    assert items[2].inner == cirq.X(q[1])
    assert items[2].kind == "program"
    # a controlled channel: a Kraus draw in its own slot on the state-vector
    # simulator, a compiled superoperator on the density-matrix simulator
    noisy = flatten_ops(cirq.Circuit(cirq.measure(q[0], key="a"),
                                     cirq.amplitude_damp(0.1).on(q[1]).with_classical_controls("a")))
    items, nslot = tj.build_items(noisy, dm=False)
    assert [(type(it).__name__, getattr(it, "kind", None)) for it in items] == [
        ("Measure", None), ("Conditional", "channel")]
    assert nslot == 1 and items[1].slot == 0
    items, _ = tj.build_items(noisy, dm=True)
    assert items[1].kind == "program"


def test_conditions_resolve_like_the_reference():
    q = cirq.LineQubit.range(3)
    op = cirq.X(q[2]).with_classical_controls("a")
    measured = {"a": [(q[0], q[1])]}
    assert not tj.conditions_hold(op, {"a": [[0, 0]]}, measured)
    assert tj.conditions_hold(op, {"a": [[0, 1]]}, measured)
    # the latest instance of a repeated key decides
    assert not tj.conditions_hold(op, {"a": [[1, 0], [0, 0]]}, {"a": measured["a"] * 2})
    # several conditions must all hold; sympy conditions read the integer value
    op2 = cirq.X(q[2]).with_classical_controls("a", "b")
    rec = {"a": [[1, 0]], "b": [[0]]}
    mq = {"a": [(q[0], q[1])], "b": [(q[2],)]}
    assert not tj.conditions_hold(op2, rec, mq)
    rec["b"] = [[1]]
    assert tj.conditions_hold(op2, rec, mq)
    import sympy

    op3 = cirq.X(q[2]).with_classical_controls(sympy.Eq(sympy.Symbol("a"), 2))
    assert tj.conditions_hold(op3, {"a": [[1, 0]]}, measured)
    assert not tj.conditions_hold(op3, {"a": [[1, 1]]}, measured)
    # a key that was never measured: the reference's ValueError
    try:
        tj.conditions_hold(cirq.X(q[2]).with_classical_controls("zz"), {"a": [[1, 0]]}, measured)
    except ValueError:
        pass
    else:
        raise AssertionError("expected ValueError")


def test_grouped_pool_replay_matches_point_by_point():
    """Trajectory pools built once per distinct combination of drawn
    unitaries (choice codes, broadcast gates) equal the point-by-point
    replay."""
    q = cirq.LineQubit.range(4)
    ops = flatten_ops(cirq.Circuit(
        cirq.H.on_each(*q), cirq.depolarize(0.3).on(q[0]), cirq.CNOT(q[0], q[1]),
        cirq.bit_flip(0.2).on(q[2]), cirq.CZ(q[1], q[2]), cirq.ry(0.4).on(q[3]),
        cirq.phase_flip(0.25).on(q[3]), cirq.CNOT(q[3], q[0]),
    ))
    items, _ = tj.build_items(ops, dm=False)
    seg = items[0]
    c = CompiledCircuit(seg.ops, q, dm=False, planner=Planner(tile_bits=10, kmax=3),
                        resolvers=[cirq.ParamResolver({})])
    rng = np.random.default_rng(0)
    reps = 40
    batch, codes = {}, {}
    for i, src in enumerate(c.sources):
        if src.slot is not None:
            probs, us = zip(*cirq.mixture(src.op.op if hasattr(src.op, "op") else src.op))
            U = np.array([np.asarray(u, dtype=complex) for u in us])
            choice = rng.integers(0, len(U), size=reps)
            batch[i], codes[i] = U[choice], choice
        else:
            m = src.matrices([cirq.ParamResolver({})])
            batch[i] = np.broadcast_to(m[0], (reps,) + m.shape[1:])
    grouped = c.pool_from_batch(batch, reps, codes)
    sub = {j: np.ascontiguousarray(batch[i]) for j, i in enumerate(c.kept)}
    plain = c.plan._pool_for_reference(sub, reps)
    np.testing.assert_allclose(grouped, plain, atol=1e-6)
