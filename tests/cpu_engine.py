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

    # ---- batched points (cirq_gb300.batch) ----------------------------------
    def device_info(self):
        return 152, 8 << 30, 16 << 30

    @staticmethod
    def _pauli_values(psi, nbits, recs) -> np.ndarray:
        """<psi| i^ny X^x Z^zy |psi> * coef for each gbq_pauli record."""
        n = 2**nbits
        src = psi[:n]
        j = np.arange(n, dtype=np.int64)
        out = np.zeros(len(recs), dtype=np.complex128)
        for t, r in enumerate(recs):
            x, zy, ny, coef = int(r["x"]), int(r["zy"]), int(r["ny"]), float(r["coef"])
            sign = 1.0 - 2.0 * (np.bitwise_count((j ^ x) & zy) & 1)
            out[t] = coef * (1j**ny) * np.vdot(src, sign * src[j ^ x])
        return out

    def points_set_zero(self, states, nbits, npoints) -> None:
        arr = np.zeros(npoints << nbits, dtype=np.complex128)
        arr[:: 1 << nbits] = 1
        states.arr = arr

    def run_points(self, states, nbits, npoints, plan, pool_dev, pool_stride) -> None:
        size = 1 << nbits
        for p in range(npoints):
            pool = pool_dev.arr[p * pool_stride : (p + 1) * pool_stride]
            states.arr[p * size : (p + 1) * size] = run_program(
                states.arr[p * size : (p + 1) * size], nbits, plan.passes, plan.ops, pool
            )
        self.launches += plan.npasses

    def points_expect(self, states, nbits, npoints, recs) -> np.ndarray:
        size = 1 << nbits
        unit = recs.copy()
        unit["coef"] = 1.0
        return np.array([self._pauli_values(states.arr[p * size : (p + 1) * size], nbits, unit)
                         for p in range(npoints)]).reshape(npoints, len(recs))

    def batch_expect(self, points, passes, ops, pool_dev, terms, max_nbits) -> np.ndarray:
        """Every point runs its pass range on its own state with the pool at
        its mat_base, then evaluates its term block (gbq_batch_expect)."""
        out = np.zeros(max(len(terms), 1), dtype=np.complex128)
        for pt in points:
            nbits = int(pt["nbits"])
            psi = np.zeros(1 << nbits, dtype=np.complex128)
            psi[0] = 1
            pb, pc = int(pt["pass_begin"]), int(pt["pass_count"])
            if pc:
                psi = run_program(psi, nbits, passes[pb : pb + pc], ops, pool_dev.arr[int(pt["mat_base"]):])
            tb, tc = int(pt["term_begin"]), int(pt["term_count"])
            out[tb : tb + tc] = self._pauli_values(psi, nbits, terms[tb : tb + tc])
        self.launches += 1
        return out
