"""Random tensor-core (MMA) programs for the parity tests -- TEST INFRASTRUCTURE.

Each pass is an 11-bit-tile pass whose ops are MMA ops (a 16 x 16 matrix on
4 tile bits, optionally selected by out-of-tile bits) followed by diagonal
ops on tile or global bits, as include/cirq_gb300.h documents for
GBQ_OP_MMA.
"""

import numpy as np

from cirq_gb300 import _lib


def _unitary(rs, k):
    a = rs.normal(size=(2**k, 2**k)) + 1j * rs.normal(size=(2**k, 2**k))
    q, _ = np.linalg.qr(a)
    return q


def random_mma_program(rs, n, npasses, with_diag=True, with_sel=False, max_mma=4):
    ops, passes, pool = [], [], []
    off = 0
    for _ in range(npasses):
        hi = sorted(rs.choice(np.arange(5, n), size=6, replace=False).tolist())
        outside = [b for b in range(5, n) if b not in hi]
        begin = len(ops)
        nm = int(rs.randint(1, max_mma + 1))
        slots = 0
        for o in range(nm):
            r = np.zeros(1, dtype=_lib.OP_DTYPE)[0]
            r["kind"] = _lib.OP_MMA
            r["k"] = 4
            r["bits"][:4] = rs.choice(_lib.MMA_TILE_BITS, size=4, replace=False)
            nsel = int(rs.randint(0, 2)) if (with_sel and outside) else 0
            if slots + 2**nsel + (nm - o - 1) > _lib.MAX_MMA_MATS:
                nsel = 0
            slots += 2**nsel
            r["nsel"] = nsel
            for s in range(nsel):
                r["sel"][s] = -int(outside[s]) - 1
            r["mat"] = off
            for _s in range(2**nsel):
                m = _unitary(rs, 4).astype(np.complex64).reshape(-1)
                pool.append(m)
                off += m.size
            ops.append(r)
            if with_diag and rs.rand() < 0.7:
                codes = []
                for _j in range(int(rs.randint(1, 4))):
                    if outside and rs.rand() < 0.3:
                        codes.append(-int(rs.choice(outside)) - 1)
                    else:
                        codes.append(int(rs.randint(0, _lib.MMA_TILE_BITS)))
                codes = list(dict.fromkeys(codes))
                d = np.zeros(1, dtype=_lib.OP_DTYPE)[0]
                d["kind"] = _lib.OP_DIAG
                d["k"] = len(codes)
                d["bits"][: len(codes)] = codes
                d["mat"] = off
                tab = np.exp(1j * rs.uniform(0, 6, 2 ** len(codes))).astype(np.complex64)
                pool.append(tab)
                off += tab.size
                ops.append(d)
        p = np.zeros(1, dtype=_lib.PASS_DTYPE)[0]
        p["L"] = _lib.MMA_TILE_BITS
        p["m"] = 5
        p["op_begin"] = begin
        p["op_count"] = len(ops) - begin
        p["hi"][:6] = hi
        passes.append(p)
    return (
        np.array(passes, dtype=_lib.PASS_DTYPE),
        np.array(ops, dtype=_lib.OP_DTYPE),
        np.concatenate(pool).astype(np.complex64),
    )


def as_plain(ops):
    """The same program with every MMA op turned into a plain dense op."""
    out = ops.copy()
    out["kind"][out["kind"] == _lib.OP_MMA] = _lib.OP_DENSE
    return out
