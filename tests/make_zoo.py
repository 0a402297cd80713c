"""The gate-zoo circuit of tests/golden/make_golden.py (kept in sync by test_golden_zoo_matches)."""

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def gate_zoo():
    import cirq
    import make_golden

    return make_golden._gate_zoo(cirq)


def fixture_circuit(name: str):
    """One of the other fixture circuits of make_golden (by builder name)."""
    import cirq
    import make_golden

    return getattr(make_golden, name)(cirq)


def golden_module():
    """The fixture generator module itself (its circuit builders)."""
    import make_golden

    return make_golden
