"""CPU emulation of the engine's program semantics -- TEST INFRASTRUCTURE ONLY.

Executes the gbq_pass / gbq_op arrays of a Plan on a numpy vector exactly as
the ABI documents them (include/cirq_gb300.h): ops run in order, a dense op
applies matrix number sum(sel_j << j) to its target bits, a diagonal op
multiplies by its table.  Tiles do not change the result, so the whole vector
is processed at once.  This lets CPU tests check the planner's encoding
(tile-bit mapping, selector codes, pool offsets) before any kernel runs.
"""

import numpy as np


def _global_bit(code, tile_of_inv):
    return tile_of_inv[code] if code >= 0 else -code - 1


def _dense(psi, idx, op, tile_to_global, pool):
    k = int(op["k"])
    base = int(op["mat"])
    tg = [tile_to_global[int(b)] for b in op["bits"][:k]]
    nsel = int(op["nsel"])
    sg = [_global_bit(int(c), tile_to_global) for c in op["sel"][:nsel]]
    d = 2**k
    mats = pool[base : base + (2**nsel) * d * d].reshape(2**nsel, d, d)
    sub = np.zeros_like(idx)
    clear = idx.copy()
    for j, b in enumerate(tg):
        sub |= ((idx >> b) & 1) << j
        clear &= ~(1 << b)
    sel = np.zeros_like(idx)
    for j, b in enumerate(sg):
        sel |= ((idx >> b) & 1) << j
    out = np.zeros_like(psi)
    for c in range(d):
        off = 0
        for j, b in enumerate(tg):
            if (c >> j) & 1:
                off |= 1 << b
        out += mats[sel, sub, c] * psi[clear | off]
    return out


def _diag(psi, idx, op, tile_to_global, pool):
    k = int(op["k"])
    base = int(op["mat"])
    bits = [_global_bit(int(c), tile_to_global) for c in op["bits"][:k]]
    tab = pool[base : base + 2**k]
    sub = np.zeros_like(idx)
    for j, b in enumerate(bits):
        sub |= ((idx >> b) & 1) << j
    return psi * tab[sub]


# register ops and tensor-core (MMA) ops compute what plain ops do
_PLAIN = {5: 0, 6: 1, 9: 0, 7: 2, 8: 3}


def run_dual_program(psi, lam, nbits, passes, ops, pool):
    """Two-state passes (gbq_run_dual): every non-probe op acts on both
    states; a probe op adds Re<lam|D|psi> (dense D, or a diagonal table) to
    its slot.  Returns (psi, lam, {slot: total})."""
    psi = np.array(psi, dtype=np.complex128).reshape(-1)
    lam = np.array(lam, dtype=np.complex128).reshape(-1)
    idx = np.arange(2**nbits, dtype=np.int64)
    slots: dict = {}
    for p in passes:
        L, m = int(p["L"]), int(p["m"])
        tile_to_global = list(range(m)) + [int(b) for b in p["hi"][: L - m]]
        for o in range(int(p["op_begin"]), int(p["op_begin"]) + int(p["op_count"])):
            op = ops[o]
            kind = int(op["kind"])
            if kind == 4:
                continue
            kind = _PLAIN.get(kind, kind)
            if kind == 0:
                psi = _dense(psi, idx, op, tile_to_global, pool)
                lam = _dense(lam, idx, op, tile_to_global, pool)
            elif kind == 1:
                psi = _diag(psi, idx, op, tile_to_global, pool)
                lam = _diag(lam, idx, op, tile_to_global, pool)
            elif kind in (2, 3):
                f = _dense if kind == 2 else _diag
                v = float(np.real(np.vdot(lam, f(psi, idx, op, tile_to_global, pool))))
                slots[int(op["slot"])] = slots.get(int(op["slot"]), 0.0) + v
            else:
                raise ValueError(f"op kind {kind} is not emulated")
    return psi, lam, slots


def run_program(state, nbits, passes, ops, pool):
    psi = np.array(state, dtype=np.complex128).reshape(-1)
    idx = np.arange(2**nbits, dtype=np.int64)
    for p in passes:
        L, m = int(p["L"]), int(p["m"])
        tile_to_global = list(range(m)) + [int(b) for b in p["hi"][: L - m]]
        for o in range(int(p["op_begin"]), int(p["op_begin"]) + int(p["op_count"])):
            op = ops[o]
            kind = int(op["kind"])
            if kind == 4:  # layout: changes where amplitudes live, not their values
                continue
            kind = _PLAIN.get(kind, kind)
            if kind == 0:
                psi = _dense(psi, idx, op, tile_to_global, pool)
            elif kind == 1:
                psi = _diag(psi, idx, op, tile_to_global, pool)
            else:
                raise ValueError("probe ops are not emulated")
    return psi
