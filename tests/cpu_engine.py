"""A CPU stand-in for cirq_gb300.engine.Engine -- TEST INFRASTRUCTURE ONLY.

Implements the calls that cirq_gb300.adjoint.AdjointProgram makes (states,
uploads, program runs, two-state runs with probes, Pauli sums, inner
products, slot reductions) with the numpy emulator of the ABI's pass/op
arrays (emulator.py) and the Pauli convention of include/cirq_gb300.h
(P = coef i^ny X^x Z^zy).  It lets CPU tests drive the package's host logic
end to end; the product never uses it.
"""

import numpy as np

from emulator import run_dual_program, run_program


class EmuBuffer:
    def __init__(self, nbytes: int, arr=None):
        self.nbytes = int(nbytes)
        self.arr = arr  # complex128 state, float64 partials, or the uploaded array
        self.freed = False

    def free(self) -> None:
        self.freed = True

    def upload(self, host) -> None:
        self.arr = np.array(host).reshape(-1).copy()

    def download(self, host):
        host[...] = np.asarray(self.arr).reshape(host.shape).astype(host.dtype)
        return host


class EmuEngine:
    def __init__(self):
        self.launches = 0

    def alloc(self, nbytes: int) -> EmuBuffer:
        return EmuBuffer(nbytes)

    def upload(self, host) -> EmuBuffer:
        host = np.ascontiguousarray(host)
        return EmuBuffer(host.nbytes, np.array(host).reshape(-1).astype(np.complex128))

    def new_state(self, nbits, basis=0, initial=None, nbits_dev=None, into=None) -> EmuBuffer:
        nbits_dev = max(nbits, nbits_dev or nbits)
        psi = np.zeros(2**nbits_dev, dtype=np.complex128)
        if initial is not None:
            psi[: 2**nbits] = np.asarray(initial).reshape(-1)
        else:
            psi[int(basis)] = 1
        buf = into if into is not None else EmuBuffer(16 << nbits_dev)
        buf.arr = psi
        return buf

    def run(self, state, nbits, plan, pool_dev=None, sync=True) -> None:
        if plan.npasses:
            state.arr = run_program(state.arr, nbits, plan.passes, plan.ops, pool_dev.arr)
            self.launches += plan.npasses

    def run_dual(self, psi, lam, nbits, plan, pool_dev, partial) -> None:
        if plan.npasses == 0:
            return
        psi.arr, lam.arr, slots = run_dual_program(psi.arr, lam.arr, nbits, plan.passes, plan.ops, pool_dev.arr)
        self.launches += plan.npasses
        partial.arr = slots  # slot -> total (the tiles' sum)

    def reduce_slots(self, partial, nslots, ntiles, out) -> None:
        out.arr = np.array([partial.arr.get(s, 0.0) for s in range(nslots)], dtype=np.float64)

    def apply_paulisum(self, psi, nbits, terms, out) -> None:
        n = 2**nbits
        src = psi.arr[:n]
        j = np.arange(n, dtype=np.int64)
        acc = np.zeros(n, dtype=np.complex128)
        for x, zy, ny, coef in terms:
            sign = 1.0 - 2.0 * (np.bitwise_count((j ^ x) & zy) & 1)  # Z^zy first, then X^x
            acc += coef * (1j**ny) * sign * src[j ^ x]
        dst = np.zeros_like(psi.arr) if out.arr is None or len(out.arr) != len(psi.arr) else out.arr
        dst[:] = 0
        dst[:n] = acc
        out.arr = dst

    def inner(self, a, b, nbits) -> complex:
        n = 2**nbits
        return complex(np.vdot(a.arr[:n], b.arr[:n]))

    def sync(self) -> None:
        pass
