"""Tensor-core (MMA) pass programs: validation rules, checked without a GPU."""

import numpy as np
import pytest

from cirq_gb300 import _lib
from mma_programs import random_mma_program
from emulator import run_program


def _validate(n, passes, ops, dual=0):
    lib = _lib.load()
    rc = lib.gbq_validate_program(n, passes.ctypes.data, len(passes), ops.ctypes.data, len(ops), dual)
    return rc, lib.gbq_last_error().decode()


@pytest.mark.parametrize("n,npasses,sel", [(11, 1, False), (14, 3, False), (18, 5, True)])
def test_random_mma_programs_validate(n, npasses, sel):
    rs = np.random.RandomState(n)
    passes, ops, pool = random_mma_program(rs, n, npasses, with_sel=sel)
    assert _validate(n, passes, ops)[0] == 0
    # single-state only
    rc, msg = _validate(n, passes, ops, dual=1)
    assert rc == -1 and "one state" in msg


def _one_pass(bits=(0, 3, 7, 9), L=11, first_kind=_lib.OP_MMA, k=4, sel=()):
    ops = np.zeros(2, dtype=_lib.OP_DTYPE)
    ops[0]["kind"] = first_kind
    ops[0]["k"] = k
    ops[0]["bits"][: len(bits)] = bits
    ops[0]["nsel"] = len(sel)
    ops[0]["sel"][: len(sel)] = sel
    ops[1]["kind"] = _lib.OP_MMA
    ops[1]["k"] = 4
    ops[1]["bits"][:4] = (1, 2, 4, 5)
    passes = np.zeros(1, dtype=_lib.PASS_DTYPE)
    passes[0]["L"] = L
    passes[0]["m"] = 5
    passes[0]["op_count"] = 2
    passes[0]["hi"][: L - 5] = list(range(5, L))
    return passes, ops


@pytest.mark.parametrize(
    "kwargs,needle",
    [
        (dict(L=13), "11-bit tiles"),
        (dict(first_kind=_lib.OP_DIAG, k=2, bits=(0, 1)), "first op"),
        (dict(k=3, bits=(0, 3, 7)), "exactly 4"),
        (dict(bits=(0, 3, 3, 9)), "distinct"),
        (dict(sel=(2,)), "global bits outside the tile"),
    ],
)
def test_invalid_mma_passes_are_rejected(kwargs, needle):
    passes, ops = _one_pass(**kwargs)
    rc, msg = _validate(16, passes, ops)
    assert rc == -1 and needle in msg, msg


def test_mma_matrix_budget():
    passes, ops = _one_pass(sel=(-12, -13, -14))  # 8 matrices > 6
    rc, msg = _validate(16, passes, ops)
    assert rc == -1 and "per pass" in msg


def test_emulator_treats_mma_as_dense():
    rs = np.random.RandomState(3)
    passes, ops, pool = random_mma_program(rs, 13, 2, with_sel=True)
    psi = rs.normal(size=2**13) + 1j * rs.normal(size=2**13)
    from mma_programs import as_plain

    a = run_program(psi, 13, passes, ops, pool.astype(np.complex128))
    b = run_program(psi, 13, passes, as_plain(ops), pool.astype(np.complex128))
    assert np.array_equal(a, b)
    assert np.isclose(np.linalg.norm(a), np.linalg.norm(psi))
