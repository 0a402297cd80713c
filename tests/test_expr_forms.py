"""Exponent evaluation on the host: the c * s / d form and the per-group
gather in gate_batch give the same bits as the lambdified expressions and
the per-expression path."""

import numpy as np
import pytest

from cirq_gb300._cirq_env import ensure_cirq

cirq = ensure_cirq()
import sympy  # noqa: E402

from cirq_gb300 import program  # noqa: E402


@pytest.mark.parametrize(
    "make",
    [
        lambda t: t / sympy.pi,
        lambda t: 2 * t / sympy.pi,
        lambda t: -t / sympy.pi,
        lambda t: t / (2 * sympy.pi),
        lambda t: sympy.Rational(3, 7) * t / sympy.pi,
        lambda t: t / 3,
        lambda t: 0.5 * t,
    ],
)
def test_forms_match_lambdify_bits(make):
    t = sympy.Symbol("t")
    e = make(t)
    vals = np.random.default_rng(0).normal(size=500) * 3
    got = program._expr_values(e, [cirq.ParamResolver({t: float(v)}) for v in vals], None)
    fn = sympy.lambdify((t,), e, "numpy")
    want = np.array([float(fn(float(v))) for v in vals])
    assert np.array_equal(got.view(np.int64), want.view(np.int64))


def test_gate_batch_gather_matches_per_expression_path():
    q = cirq.LineQubit.range(3)
    a, b, c = sympy.symbols("a b c")
    circuit = cirq.Circuit(
        cirq.rx(a).on(q[0]), cirq.rz(2 * b).on(q[1]), cirq.ry(c).on(q[2]),
        cirq.XPowGate(exponent=a).on(q[1]), cirq.ZPowGate(exponent=0.25).on(q[0]),
        cirq.rx(b).on(q[2]), cirq.CZ(q[0], q[1]) ** c,
    )
    from cirq_gb300.planner import Planner

    rs = [cirq.ParamResolver({"a": 0.3, b: -1.7, "c": 2}), cirq.ParamResolver({a: 1e-3, "b": 5.0, c: 0.75})]
    cc = program.CompiledCircuit(list(circuit.all_operations()), q, dm=False, planner=Planner(), resolvers=rs)
    fast = cc.gate_batch(rs)
    for i, src in enumerate(cc.sources):
        slow = src.matrices(rs, None)
        assert np.array_equal(np.asarray(fast[i]), np.asarray(slow)), i


def test_symbol_values_follow_value_of():
    a, b = sympy.symbols("a b")
    r = cirq.ParamResolver({"a": 0.5, b: "a", "c": sympy.Symbol("a") * 2})
    got = program._symbol_values([a, b, sympy.Symbol("c")], [r])[:, 0]
    assert got.tolist() == [0.5, 0.5, 1.0]
