"""Per-circuit memo of the simulators' circuit analysis (no GPU): results are
reused while a circuit holds the same moment objects and recomputed after
any change."""

import cirq

from cirq_gb300 import simulator as S


def test_split_is_reused_and_follows_mutation():
    q = cirq.LineQubit.range(3)
    c = cirq.Circuit(cirq.H(q[0]), cirq.CNOT(q[0], q[1]), cirq.measure(*q[:2], key="m"))
    a = S._split_terminal(c)
    assert S._split_terminal(c) is a  # same moments: remembered
    body, meas = a
    assert len(body) == 2 and len(meas) == 1
    c.insert(0, cirq.X(q[2]))  # a new moment in front
    body2, meas2 = S._split_terminal(c)
    assert len(body2) == 3 and len(meas2) == 1
    c.append(cirq.measure(q[2], key="z"))
    assert len(S._split_terminal(c)[1]) == 2
    # an equal but distinct circuit is a separate entry with the same answer
    d = cirq.Circuit(c.moments)
    assert S._split_terminal(d) == S._split_terminal(c)


def test_memo_entries_keep_moments_alive():
    store = {}
    import collections

    store = collections.OrderedDict()
    calls = []

    def fn(p):
        calls.append(p)
        return len(p)

    q = cirq.LineQubit(0)
    for _ in range(3):
        c = cirq.Circuit([cirq.X(q)] * 4)
        assert S._memo(store, c, "n", fn) == 4
    # three distinct circuits (ids may repeat once freed): each was computed,
    # because the stored moments never match another circuit's moments
    assert len(calls) == 3
    c = cirq.Circuit([cirq.X(q)] * 4)
    S._memo(store, c, "n", fn)
    S._memo(store, c, "n", fn)
    assert len(calls) == 4
