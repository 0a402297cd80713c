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


def _buf(x):
    """The emulated buffer behind a buffer or a simulator's non-owning view."""
    return getattr(x, "_buf", x)


class EmuBuffer:
    def __init__(self, nbytes: int, arr=None):
        self.nbytes = int(nbytes)
        self.arr = arr  # complex128 state, float64 partials, or the uploaded array
        self.freed = False
        self.ptr = id(self)
        self.engine = None

    def free(self) -> None:
        self.freed = True

    def upload(self, host) -> None:
        self.arr = np.array(host).reshape(-1).copy()

    def download(self, host):
        host[...] = np.asarray(self.arr).reshape(host.shape).astype(host.dtype)
        return host


class EmuEngine:
    def __init__(self):
        self._launches = 0

    def launches(self) -> int:
        return self._launches

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
            _buf(state).arr = run_program(_buf(state).arr, nbits, plan.passes, plan.ops, _buf(pool_dev).arr)
            self._launches += plan.npasses

    def run_dual(self, psi, lam, nbits, plan, pool_dev, partial) -> None:
        if plan.npasses == 0:
            return
        _buf(psi).arr, _buf(lam).arr, slots = run_dual_program(_buf(psi).arr, _buf(lam).arr, nbits, plan.passes, plan.ops, _buf(pool_dev).arr)
        self._launches += plan.npasses
        _buf(partial).arr = slots  # slot -> total (the tiles' sum)

    def reduce_slots(self, partial, nslots, ntiles, out) -> None:
        _buf(out).arr = np.array([_buf(partial).arr.get(s, 0.0) for s in range(nslots)], dtype=np.float64)

    def apply_paulisum(self, psi, nbits, terms, out) -> None:
        n = 2**nbits
        src = _buf(psi).arr[:n]
        j = np.arange(n, dtype=np.int64)
        acc = np.zeros(n, dtype=np.complex128)
        for x, zy, ny, coef in terms:
            sign = 1.0 - 2.0 * (np.bitwise_count((j ^ x) & zy) & 1)  # Z^zy first, then X^x
            acc += coef * (1j**ny) * sign * src[j ^ x]
        dst = np.zeros_like(_buf(psi).arr) if _buf(out).arr is None or len(_buf(out).arr) != len(_buf(psi).arr) else _buf(out).arr
        dst[:] = 0
        dst[:n] = acc
        _buf(out).arr = dst

    def inner(self, a, b, nbits) -> complex:
        n = 2**nbits
        return complex(np.vdot(_buf(a).arr[:n], _buf(b).arr[:n]))

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
        _buf(states).arr = arr

    def run_points(self, states, nbits, npoints, plan, pool_dev, pool_stride) -> None:
        size = 1 << nbits
        for p in range(npoints):
            if pool_stride == 0:  # one pool for every point
                pool = _buf(pool_dev).arr
            else:
                pool = _buf(pool_dev).arr[p * pool_stride : (p + 1) * pool_stride]
            _buf(states).arr[p * size : (p + 1) * size] = run_program(
                _buf(states).arr[p * size : (p + 1) * size], nbits, plan.passes, plan.ops, pool
            )
        self._launches += plan.npasses

    def points_expect(self, states, nbits, npoints, recs) -> np.ndarray:
        size = 1 << nbits
        unit = recs.copy()
        unit["coef"] = 1.0
        return np.array([self._pauli_values(_buf(states).arr[p * size : (p + 1) * size], nbits, unit)
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
                psi = run_program(psi, nbits, passes[pb : pb + pc], ops, _buf(pool_dev).arr[int(pt["mat_base"]):])
            tb, tc = int(pt["term_begin"]), int(pt["term_count"])
            out[tb : tb + tc] = self._pauli_values(psi, nbits, terms[tb : tb + tc])
        self._launches += 1
        return out

    # ---- simulators (cirq_gb300.simulator / trajectories / steps) ------------
    def download_state(self, state, nbits, pinned=True) -> np.ndarray:
        return np.asarray(_buf(state).arr[: 1 << nbits]).astype(np.complex64)

    def final_renormalize(self, state, nbits) -> tuple[bool, float]:
        """gbq_sv_final_renormalize: the rule of state_vector_simulator.py:131-146
        at complex64; returns (applied, norm before)."""
        v = _buf(state).arr[: 1 << nbits].astype(np.complex64)
        norm = float(np.linalg.norm(v.astype(np.complex128)))
        if abs(norm - 1) > np.sqrt(np.finfo(np.float32).eps):
            return False, norm
        vn = (v / np.float32(norm)).astype(np.complex64)
        if abs(np.vdot(vn, vn) - 1) - abs(np.vdot(v, v) - 1) < 0:
            _buf(state).arr[: 1 << nbits] = vn
            return True, norm
        return False, norm

    def norm2(self, state, nbits) -> float:
        return float(np.sum(np.abs(_buf(state).arr[: 1 << nbits]) ** 2))

    def scale(self, state, nbits, factor) -> None:
        _buf(state).arr[: 1 << nbits] *= np.float32(factor)

    def project(self, state, nbits, mask, value, scale) -> None:
        j = np.arange(1 << nbits, dtype=np.int64)
        keep = (j & int(mask)) == int(value)
        a = _buf(state).arr[: 1 << nbits]
        _buf(state).arr[: 1 << nbits] = np.where(keep, a * np.float32(scale), 0)

    def _probs(self, state, nbits, dm) -> np.ndarray:
        if dm:
            d = 1 << nbits
            return np.real(np.diagonal(_buf(state).arr[: d * d].reshape(d, d)))
        return np.abs(_buf(state).arr[: 1 << nbits]) ** 2

    def probabilities(self, state, nbits, dm=False) -> np.ndarray:
        return self._probs(state, nbits, dm).astype(np.float32)

    def sample(self, state, nbits, uniforms, dm=False) -> np.ndarray:
        from oracle.statevector import sample_from_probs

        self._launches += 1
        return sample_from_probs(self._probs(state, nbits, dm), uniforms).astype(np.uint64)

    def expect_paulis(self, state, nbits, terms, dm=False) -> np.ndarray:
        if not terms:
            return np.zeros(0, dtype=np.complex128)
        coefs = np.array([c for *_, c in terms], dtype=np.complex128)
        if not dm:
            recs = np.zeros(len(terms), dtype=[("x", "u8"), ("zy", "u8"), ("ny", "i4"), ("coef", "f8")])
            for i, (x, zy, ny, _) in enumerate(terms):
                recs[i] = (x, zy, ny, 1.0)
            return self._pauli_values(_buf(state).arr, nbits, recs) * coefs
        d = 1 << nbits
        rho = _buf(state).arr[: d * d].reshape(d, d)
        m = np.arange(d, dtype=np.int64)
        out = np.zeros(len(terms), dtype=np.complex128)
        for t, (x, zy, ny, _) in enumerate(terms):
            sign = 1.0 - 2.0 * (np.bitwise_count(m & zy) & 1)
            out[t] = (1j**ny) * np.sum(sign * rho[m, m ^ x])  # Tr(P rho), P|m> = i^ny (-1)^{m.zy} |m^x>
        return out * coefs

    def points_dm_marginal(self, states, nbits, nq, npoints, bits) -> np.ndarray:
        """gbq_points_dm_marginal: outcome probabilities of the index bits
        `bits` from the diagonals of npoints density matrices."""
        size = 1 << nbits
        i = np.arange(1 << nq, dtype=np.int64)
        o = np.zeros_like(i)
        for j, b in enumerate(bits):
            o |= ((i >> b) & 1) << j
        out = np.zeros((npoints, 1 << len(bits)))
        for p in range(npoints):
            diag = np.real(_buf(states).arr[p * size : (p + 1) * size][i * ((1 << nq) + 1)])
            np.add.at(out[p], o, diag)
        self._launches += 1
        return out

    def sample_point(self, states, slot_bits, point, nbits, uniforms, dm=False) -> np.ndarray:
        size = 1 << slot_bits
        view = EmuBuffer(8 * size, _buf(states).arr[point * size : (point + 1) * size])
        return self.sample(view, nbits, uniforms, dm)

    def points_sample(self, states, nbits, npoints, uniforms) -> np.ndarray:
        from oracle.statevector import sample_from_probs

        size = 1 << nbits
        u = np.asarray(uniforms, dtype=np.float64)
        return np.array([sample_from_probs(np.abs(_buf(states).arr[p * size : (p + 1) * size]) ** 2, u[p : p + 1])[0]
                         for p in range(npoints)], dtype=np.uint64)

    def points_rdm(self, states, nbits, npoints, bits) -> np.ndarray:
        size = 1 << nbits
        k = len(bits)
        d = 1 << k
        j = np.arange(size, dtype=np.int64)
        sub = np.zeros(size, dtype=np.int64)
        rest = j.copy()
        for q, b in enumerate(bits):  # bits[0] is the most significant matrix index bit
            sub |= ((j >> b) & 1) << (k - 1 - q)
            rest &= ~(1 << b)
        out = np.zeros((npoints, d, d), dtype=np.complex128)
        for p in range(npoints):
            psi = _buf(states).arr[p * size : (p + 1) * size]
            for a in range(d):
                for c in range(d):
                    ia = np.nonzero(sub == a)[0]
                    ic = np.nonzero(sub == c)[0]
                    # pair entries with equal remaining bits
                    out[p, a, c] = np.sum(psi[ia[np.argsort(rest[ia])]] * np.conj(psi[ic[np.argsort(rest[ic])]]))
        return out
