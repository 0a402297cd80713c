"""Host planner: groups gates into tile passes and fuses them into k-qubit blocks.

Input: a list of :class:`cirq_gb300.ir.BitGate` over an ``nbits``-bit vector.
Output: a :class:`Plan` -- the ``gbq_pass`` / ``gbq_op`` arrays of the C ABI
plus a pool of complex64 matrices.

One pass = one read + one write of the state.  A pass owns a set S of L
"tile" index bits (always including the low ``m`` bits, so loads stay
contiguous).  Walking the gates in circuit order, a gate joins the pass when
every earlier gate it does not commute with has joined too, and, if it is not
diagonal, its bits fit in S.  Diagonal gates never need their bits in S: a
bit outside S is constant over a tile, so its value just selects which of
2^nsel precomputed matrices a dense op uses (``gbq_op.sel``).

Inside a pass gates are fused greedily (qsim-style) into dense ops on at most
``kmax`` bits or diagonal tables on at most 8 bits.  A pass stops growing when
its estimated arithmetic (sum of 2^k complex multiply-adds per amplitude plus
a per-op overhead) reaches ``budget``: beyond that the pass would be
compute-bound rather than HBM-bound.

Every fused op records a *recipe* (the sequence of embed/multiply steps), so
the matrices of a plan can be recomputed for a batch of parameter points with
vectorised numpy, without re-planning (``Plan.pool_for``).

The reference's own fusion (``merge_k_qubit_unitaries``,
``cirq-core/cirq/transformers/merge_k_qubit_gates.py:71-140``) only merges
nested qubit sets; this planner grows genuine k-bit blocks instead.
"""

from __future__ import annotations

import dataclasses
import functools
from typing import Sequence

import numpy as np

from cirq_gb300 import _lib
from cirq_gb300.ir import BitGate

MAX_OPS = 32  # fused ops per pass; register layouts at most double the engine's count (<= 64)
MAX_DIAG_BITS = 8
MAX_SEL = 3
MIN_TILE_BITS = 10  # the engine's narrowest tile; narrower registers are padded
TC_TILE_BITS = 12  # tensor-core passes: 12-bit tiles, 4-bit MMA blocks
TC_K = 4
TC_MAX_MMA_OPS = 8  # GBQ_MAX_MMA_OPS
TC_MAX_MATS = 10  # GBQ_TC_MAX_MATS


# ---------------------------------------------------------------- fused ops
@dataclasses.dataclass
class _Dense:
    tg: list  # global bits, matrix bit j <-> tg[j]
    sl: list  # global bits, selector bit j <-> sl[j]
    M: np.ndarray  # (P, 2^nsel, 2^k, 2^k)
    recipe: list

    kind = "dense"

    def touches(self):
        return set(self.tg) | set(self.sl)

    def cost(self, ovh):
        return 2 ** len(self.tg) + ovh


@dataclasses.dataclass
class _Diag:
    bits: list  # global bits, table bit j <-> bits[j]
    d: np.ndarray  # (P, 2^b)
    recipe: list

    kind = "diag"

    def touches(self):
        return set(self.bits)

    def cost(self, ovh):
        return 1 + ovh


@dataclasses.dataclass
class _Probe:
    bits: list  # global bits, matrix bit j <-> bits[j]
    M: np.ndarray  # (P, 2^k, 2^k) probe matrix D
    diagonal: bool
    slot: int
    recipe: list

    kind = "probe"

    def touches(self):
        return set(self.bits)

    def cost(self, ovh):
        return (1 if self.diagonal else 2 ** len(self.bits)) + ovh


# The index tables below depend only on a step's static shape; they are
# cached (read-only arrays) because recipes are replayed for every sweep point.


def _frozen(*arrays):
    for a in arrays:
        a.flags.writeable = False
    return arrays if len(arrays) > 1 else arrays[0]


@functools.lru_cache(maxsize=8192)
def _sub_index_cached(size_bits: int, pos: tuple) -> tuple[np.ndarray, np.ndarray]:
    idx = np.arange(2**size_bits)
    sub = np.zeros_like(idx)
    mask = 0
    for i, p in enumerate(pos):
        sub |= ((idx >> p) & 1) << i
        mask |= 1 << p
    return _frozen(sub, idx & ~mask)


def _sub_index(size_bits: int, pos: Sequence[int]) -> tuple[np.ndarray, np.ndarray]:
    return _sub_index_cached(int(size_bits), tuple(int(p) for p in pos))


@functools.lru_cache(maxsize=8192)
def _expand_index(k: int, pos: tuple):
    sub, rest = _sub_index_cached(k, pos)
    return _frozen(sub[:, None].copy(), sub[None, :].copy(), rest[:, None] == rest[None, :])


def _expand(G: np.ndarray, pos: Sequence[int], k: int) -> np.ndarray:
    """(P, 2^kg, 2^kg) gate on target positions `pos` -> (P, 2^k, 2^k)."""
    rows, cols, same = _expand_index(int(k), tuple(int(p) for p in pos))
    return G[:, rows, cols] * same


@functools.lru_cache(maxsize=8192)
def _diag_index_cached(nsel: int, k: int, tpos: tuple, spos: tuple) -> np.ndarray:
    s = np.arange(2**nsel)[:, None]
    t = np.arange(2**k)[None, :]
    sub = np.zeros((2**nsel, 2**k), dtype=np.int64)
    for j, (tp, sp) in enumerate(zip(tpos, spos)):
        if tp is not None:
            sub = sub | (((t >> tp) & 1) << j)
        else:
            sub = sub | (((s >> sp) & 1) << j)
    return _frozen(sub)


def _diag_index(nsel: int, k: int, tpos, spos) -> np.ndarray:
    """Gate sub-index for every (selector value, target index): shape (2^nsel, 2^k)."""
    norm = lambda xs: tuple(None if x is None else int(x) for x in xs)  # noqa: E731
    return _diag_index_cached(int(nsel), int(k), norm(tpos), norm(spos))


@functools.lru_cache(maxsize=4096)
def _s2t_index(ns: int, i: int) -> tuple[np.ndarray, np.ndarray]:
    sidx = np.arange(ns)
    keep = sidx[((sidx >> i) & 1) == 0]
    lo = ((keep & ((1 << i) - 1)) | ((keep >> (i + 1)) << i))
    keep = keep[np.argsort(lo)]
    return _frozen(keep, keep | (1 << i))


class _Replayer:
    """Applies recipe steps to batched matrices (shared by planning and replay)."""

    @staticmethod
    def dense_step(M: np.ndarray, step, gates: dict) -> np.ndarray:
        kind = step[0]
        P, ns, d, _ = M.shape
        if kind == "tx":  # add `n` identity target bits (new highest bits)
            n = step[1]
            eye = np.eye(2**n, dtype=M.dtype)
            return np.einsum("ab,psij->psaibj", eye, M).reshape(P, ns, d * 2**n, d * 2**n)
        if kind == "sx":  # add `n` selector bits (new highest selector bits)
            n = step[1]
            return np.concatenate([M] * (2**n), axis=1)
        if kind == "s2t":  # selector i becomes the new highest target bit
            keep, keep_hi = _s2t_index(ns, int(step[1]))
            out = np.zeros((P, ns // 2, 2 * d, 2 * d), dtype=M.dtype)
            out[:, :, :d, :d] = M[:, keep]
            out[:, :, d:, d:] = M[:, keep_hi]
            return out
        if kind == "mul":  # left-multiply a non-diagonal gate on target positions
            _, gi, pos = step
            k = int(np.log2(d))
            F = _expand(gates[gi], pos, k)  # (P, d, d)
            return np.matmul(F[:, None], M)  # batched over points and selector values
        if kind == "dmul":  # row-scale by a diagonal gate over (targets, selectors)
            _, gi, tpos, spos = step
            k = int(np.log2(d))
            nsel = int(np.log2(ns))
            dg = np.diagonal(gates[gi], axis1=1, axis2=2)  # (P, 2^kg)
            sub = _diag_index(nsel, k, tpos, spos)  # (ns, d)
            return dg[:, sub][..., None] * M
        raise ValueError(step)

    @staticmethod
    def diag_step(D: np.ndarray, step, gates: dict) -> np.ndarray:
        kind = step[0]
        if kind == "dx":
            n = step[1]
            return np.concatenate([D] * (2**n), axis=1)
        if kind == "dd":
            _, gi, pos = step
            b = int(np.log2(D.shape[1]))
            dg = np.diagonal(gates[gi], axis1=1, axis2=2)
            sub, _ = _sub_index(b, pos)
            return D * dg[:, sub]
        raise ValueError(step)


@dataclasses.dataclass
class PassPlan:
    L: int
    m: int
    hi: list
    ops: list  # _Dense / _Diag


_F32_1E12 = int(np.array(1e-12, dtype=np.float32).view(np.int32))

# recipe step kinds that read a gate matrix (gate index at step[1]) and the
# kinds that only reshape; anything else disables point grouping for an op
_GATE_STEPS = ("mul", "dmul", "dd", "init_diag", "init_dense", "probe")
#: pools of one point are built by gbq_pool_build (the numpy replay stays
#: for batches of points and as the checked reference of the native one)
NATIVE_POOLS = True
_GATE_FREE_STEPS = ("tx", "sx", "s2t", "dx")


def _snap(pool: np.ndarray) -> np.ndarray:
    """Matrix entries as stored in the complex64 pool: real and
    imaginary parts below 1e-12 become exact zeros, so that a gate at an
    integer or half-integer exponent (X**1 from its eigen-decomposition, whose
    phases carry ~1e-16 residues) is the exact permutation / phase matrix the
    reference's specialised code applies.  complex64 cannot resolve such
    parts next to O(1) entries in any case."""
    if pool.dtype == np.complex64:
        # in place: |x| < 1e-12 on the float32 bit pattern (sign bit cleared),
        # without the temporaries of abs()
        bits = pool.view(np.int32)
        np.copyto(bits, 0, where=(bits & 0x7FFFFFFF) < _F32_1E12)
        return pool
    # a (P, entries) block of one op, possibly a view of the caller's gates:
    # a new array
    re = np.where(np.abs(pool.real) < 1e-12, 0.0, pool.real)
    im = np.where(np.abs(pool.imag) < 1e-12, 0.0, pool.imag)
    return re + 1j * im


@dataclasses.dataclass
class Plan:
    """A planned program: passes, ops and the matrix pool (complex64)."""

    nbits: int
    passes: np.ndarray
    ops: np.ndarray
    pool: np.ndarray  # complex64 (pool_len,) for the planning point
    pass_plans: list
    ngates: int
    # op index -> (kind, recipe, pool offset, shape) for replay
    layout: list
    pool_len: int

    @property
    def npasses(self) -> int:
        return len(self.passes)

    def cost(self) -> float:
        """Estimated complex MACs per amplitude summed over all passes."""
        tot = 0.0
        for pp in self.pass_plans:
            for op in pp.ops:
                tot += op.cost(0.0)
        return tot

    def _native_program(self) -> np.ndarray:
        """The layout's recipes as the int32 program of gbq_pool_build
        (csrc/gbq_pool.cu), built once per plan."""
        prog = self.__dict__.get("_native_prog")
        if prog is not None:
            return prog
        words: list[int] = []

        def dense_steps(recipe):
            for st in recipe:
                k = st[0]
                if k == "init_dense":
                    words.extend((1, st[1]))
                elif k == "tx":
                    words.extend((2, st[1]))
                elif k == "sx":
                    words.extend((3, st[1]))
                elif k == "s2t":
                    words.extend((4, st[1]))
                elif k == "mul":
                    words.extend((5, st[1], len(st[2]), *st[2]))
                elif k == "dmul":
                    _, gi, tpos, spos = st
                    words.extend((6, gi, len(tpos)))
                    words.extend(-1 if t is None else int(t) for t in tpos)
                    words.extend(-1 if x is None else int(x) for x in spos)
                elif k == "diag_as_dense":
                    _, sub, bits, tg, sl = st
                    words.extend((7, len(sub)))
                    diag_steps(sub)
                    words.extend((len(bits), *bits, len(tg), *tg, len(sl), *sl))
                else:
                    raise ValueError(k)

        def diag_steps(recipe):
            for st in recipe:
                k = st[0]
                if k == "init_diag":
                    words.extend((8, st[1]))
                elif k == "dx":
                    words.extend((9, st[1]))
                elif k == "dd":
                    words.extend((10, st[1], len(st[2]), *st[2]))
                else:
                    raise ValueError(k)

        for kind, recipe, off, shape, perm in self.layout:
            code = {"dense": 0, "diag": 1, "probe": 2, "probe_diag": 3}[kind]
            words.extend((code, off & 0xFFFFFFFF, off >> 32))
            if kind == "dense":
                ns, d = shape
                words.extend((ns, d, int(perm is not None)))
                if perm is not None:
                    words.extend(int(x) for x in perm)
                words.append(len(recipe))
                dense_steps(recipe)
            elif kind == "diag":
                words.append(len(recipe))
                diag_steps(recipe)
            elif kind == "probe":
                d = 1 << shape[0]
                words.extend((recipe[0][1], d, int(perm is not None)))
                if perm is not None:
                    words.extend(int(x) for x in perm)
            else:
                words.append(recipe[0][1])
        prog = np.asarray(words, dtype=np.int64).astype(np.int32)
        self.__dict__["_native_prog"] = prog
        return prog

    def _native_pool(self, gates: dict, npoints: int = 1) -> np.ndarray | None:
        """The pools of `npoints` points through gbq_pool_build (one point)
        or gbq_pool_build_points (host threads over the points); None if the
        library cannot be loaded."""
        try:
            lib = _lib.load()
        except Exception:  # noqa: BLE001  (no engine: the numpy replay runs)
            return None
        prog = self._native_program()
        # one block per matrix size; the grouping depends only on the gate
        # indices and sizes, which a program's batches share
        key = tuple(gates)
        groups_cache = self.__dict__.setdefault("_native_groups", {})
        grp = groups_cache.get(key)
        if grp is None:
            ng = (max(gates) + 1) if gates else 0
            dims = np.zeros(max(ng, 1), dtype=np.int32)
            offs = np.zeros(max(ng, 1), dtype=np.int64)
            by_dim: dict = {}
            for gi, g in gates.items():
                by_dim.setdefault(g.shape[-1], []).append(gi)
            at = 0
            for d, gis in by_dim.items():
                idx = np.asarray(gis)
                dims[idx] = d
                offs[idx] = at + np.arange(len(gis), dtype=np.int64) * (d * d)
                at += len(gis) * d * d
            grp = (list(by_dim.items()), dims, offs, ng)
            if len(groups_cache) >= 8:
                groups_cache.clear()
            groups_cache[key] = grp
        order, dims, offs, ng = grp
        if npoints == 1:
            blocks = [np.concatenate([gates[gi][:1] for gi in gis]).astype(np.complex128, copy=False).reshape(-1)
                      for _, gis in order]
            flat = np.ascontiguousarray(np.concatenate(blocks)) if blocks else np.zeros(1, np.complex128)
            out = np.zeros((1, self.pool_len), dtype=np.complex64)
            rc = lib.gbq_pool_build(prog.ctypes.data, len(prog), flat.ctypes.data, offs.ctypes.data, dims.ctypes.data,
                                    ng, out.ctypes.data, self.pool_len)
        else:
            # (points, gate elements): each size group's (P, d, d) matrices side
            # by side, in the order of the one-point layout
            blocks = [np.stack([np.broadcast_to(gates[gi], (npoints, d, d)) for gi in gis], axis=1)
                      .reshape(npoints, -1) for d, gis in order]
            if blocks:
                flat = np.ascontiguousarray(np.concatenate(blocks, axis=1), dtype=np.complex128)
            else:
                flat = np.zeros((npoints, 1), np.complex128)
            out = np.zeros((npoints, self.pool_len), dtype=np.complex64)
            rc = lib.gbq_pool_build_points(prog.ctypes.data, len(prog), flat.ctypes.data, flat.shape[1],
                                           offs.ctypes.data, dims.ctypes.data, ng, npoints, out.ctypes.data,
                                           self.pool_len, 0)
        if rc != 0:
            raise ValueError("gbq_pool_build rejected the plan's recipes")
        return out  # snapped by the builder

    def pool_for(self, gates: dict, npoints: int, codes: dict | None = None) -> np.ndarray:
        """Recomputes the matrix pool for a batch: gates[gi] is (P, d, d).

        `codes` (optional) gives, for some gates, a (P,) integer array that
        is equal for points whose matrices are equal (trajectories: the index
        of the drawn unitary); gates broadcast over the points (zero stride)
        count as equal everywhere.  Each op is then built once per distinct
        combination of its gates and gathered to the points.

        Returns complex64 (P, pool_len).  Without `codes` the points run
        natively (gbq_pool_build / gbq_pool_build_points, the same steps as
        plain loops, host threads over the points).
        """
        if NATIVE_POOLS and (npoints == 1 or codes is None):
            # trajectory batches (codes) keep the replay below, which builds
            # each op once per distinct combination of drawn unitaries
            pool = self._native_pool(gates, npoints)
            if pool is not None:
                return pool
        out = np.zeros((npoints, self.pool_len), dtype=np.complex64)
        dedupe = npoints > 1 and (codes is not None or any(
            np.asarray(g).ndim and np.asarray(g).strides[0] == 0 for g in gates.values()))
        regions = []  # (offset, width) written point by point, snapped in place below
        for li, (kind, recipe, off, shape, perm) in enumerate(self.layout):
            if dedupe:
                gis, rep, inverse = self._point_groups(recipe, gates, npoints, codes or {})
                if rep is not None and gis:
                    sub = {gi: np.asarray(gates[gi])[rep] for gi in gis}
                    block = _snap(self._pool_entry(kind, recipe, shape, perm, sub, len(rep)))
                    out[:, off : off + block.shape[1]] = block[inverse]
                    continue
            block = self._pool_entry(kind, recipe, shape, perm, gates, npoints)
            out[:, off : off + block.shape[1]] = block
            regions.append((off, block.shape[1]))
        if not dedupe:
            return _snap(out)
        for off, width in regions:
            _snap(out[:, off : off + width])
        return out

    @staticmethod
    def _recipe_gates(recipe):
        """Sorted gate indices a recipe reads, or None if it has a step kind
        this scan does not know (the op is then built point by point)."""
        out: set = set()
        for step in recipe:
            kind = step[0]
            if kind in _GATE_STEPS:
                out.add(step[1])
            elif kind == "diag_as_dense":
                nested = Plan._recipe_gates(step[1])
                if nested is None:
                    return None
                out.update(nested)
            elif kind not in _GATE_FREE_STEPS:
                return None
        return sorted(out)

    def _point_groups(self, recipe, gates, npoints, codes):
        """(gate indices, representative points, inverse map) of the distinct
        gate combinations of one op; rep is None when the points differ."""
        gis = self._recipe_gates(recipe)
        if not gis:
            return gis, None, None
        cols = []
        for gi in gis:
            g = np.asarray(gates[gi])
            if gi in codes:
                cols.append(np.asarray(codes[gi]))
            elif g.strides[0] != 0:
                return gis, None, None
        if not cols:
            return gis, np.zeros(1, dtype=np.int64), np.zeros(npoints, dtype=np.int64)
        key = np.stack(cols, axis=1)
        _, rep, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
        if len(rep) * 2 > npoints:
            return gis, None, None  # too few repeats to pay for the gather
        return gis, rep, inverse.reshape(-1)

    def _pool_entry(self, kind, recipe, shape, perm, gates, npoints) -> np.ndarray:
        """One op's matrices / table for the points: (P, entries)."""
        if kind == "dense":
            ns, d = shape
            M = np.broadcast_to(np.eye(1, dtype=np.complex128), (npoints, 1, 1, 1)).copy()
            for step in recipe:
                M = _Replayer.dense_step(M, step, gates)
            if perm is not None:
                M = M[:, :, perm[:, None], perm[None, :]]
            return M.reshape(npoints, -1)
        if kind in ("probe", "probe_diag"):
            G = np.asarray(gates[recipe[0][1]])
            if kind == "probe_diag":
                return np.diagonal(G, axis1=1, axis2=2)
            if perm is not None:
                G = G[:, perm[:, None], perm[None, :]]
            return G.reshape(npoints, -1)
        D = np.ones((npoints, 1), dtype=np.complex128)
        for step in recipe:
            D = _Replayer.diag_step(D, step, gates)
        return D

    def _pool_for_reference(self, gates: dict, npoints: int) -> np.ndarray:
        """pool_for without grouping (kept for tests of the grouping)."""
        out = np.zeros((npoints, self.pool_len), dtype=np.complex64)
        for kind, recipe, off, shape, perm in self.layout:
            if kind == "dense":
                ns, d = shape
                M = np.broadcast_to(np.eye(1, dtype=np.complex128), (npoints, 1, 1, 1)).copy()
                for step in recipe:
                    M = _Replayer.dense_step(M, step, gates)
                if perm is not None:
                    M = M[:, :, perm[:, None], perm[None, :]]
                out[:, off : off + ns * d * d] = M.reshape(npoints, -1)
            elif kind in ("probe", "probe_diag"):
                (b,) = shape
                G = np.asarray(gates[recipe[0][1]])
                if kind == "probe_diag":
                    out[:, off : off + 2**b] = np.diagonal(G, axis1=1, axis2=2)
                else:
                    if perm is not None:
                        G = G[:, perm[:, None], perm[None, :]]
                    out[:, off : off + 4**b] = G.reshape(npoints, -1)
            else:
                (b,) = shape
                D = np.ones((npoints, 1), dtype=np.complex128)
                for step in recipe:
                    D = _Replayer.diag_step(D, step, gates)
                out[:, off : off + 2**b] = D
        return _snap(out)


class Planner:
    """Greedy pass/fusion planner (see module docstring)."""

    def __init__(
        self,
        tile_bits: int = 12,
        low_bits: int = 5,
        kmax: int = 4,
        budget: float = 40.0,
        op_overhead: float = 2.0,
        use_registers: bool = True,
        tensor: bool = False,
    ):
        """``tensor=True`` plans tensor-core passes: 12-bit tiles whose fused
        blocks are 4-bit MMA ops (tcgen05, three-term TF32 split) and whose
        diagonal ops run in the MMA read-back; ``budget`` is then the number
        of MMA ops a pass may hold (their cost does not depend on how many
        gates a block absorbs).  A pass the tensor-core form cannot express
        is emitted for the CUDA-core kernels instead."""
        if not 1 <= kmax <= 5:
            raise ValueError("fusion width kmax must be in 1..5")
        if not MIN_TILE_BITS <= tile_bits <= 13:
            raise ValueError(f"tile_bits must be in {MIN_TILE_BITS}..13")
        if tensor:
            tile_bits, kmax, low_bits = TC_TILE_BITS, TC_K, 5
            budget = float(min(max(int(budget), 1), TC_MAX_MMA_OPS))
        self.tile_bits = tile_bits
        self.low_bits = low_bits
        self.kmax = kmax
        self.budget = budget
        self.ovh = op_overhead
        self.use_registers = use_registers
        self.tensor = tensor

    # ------------------------------------------------------------------
    def plan(self, gates: Sequence[BitGate], nbits: int, batch: dict | None = None) -> Plan:
        """Plans `gates`; `batch` optionally gives (P, d, d) matrices per gate index
        (default: each gate's own matrix, P = 1).  nbits >= 10 (pad narrower
        registers with unused high bits)."""
        if nbits < MIN_TILE_BITS:
            raise ValueError(f"plan width must be >= {MIN_TILE_BITS} bits (pad narrower registers)")
        if batch is None:
            batch = {i: g.matrix[None] for i, g in enumerate(gates)}
        L = min(self.tile_bits, nbits)
        m = min(self.low_bits, L)
        # tensor-core passes take MMA selectors only when enough global bits
        # stay outside the tile; otherwise a selector soon blocks a gate that
        # needs its bit in the tile, and diagonal ops in the read-back are
        # cheaper
        self._tc_selectors = nbits - L >= 6
        remaining = list(range(len(gates)))
        pass_plans: list[PassPlan] = []
        while remaining:
            pp, remaining = self._one_pass(gates, remaining, nbits, L, m, batch)
            pass_plans.append(pp)
        return self._emit(pass_plans, nbits, len(gates))

    def _one_pass(self, gates, remaining, nbits, L, m, batch):
        S = set(range(m))
        ops: list = []
        last: dict = {}  # global bit -> index of latest op touching it
        blocked_nd: set = set()
        blocked_d: set = set()
        cost = 0.0
        taken: list = []
        left: list = []
        budget = self.budget if nbits > L else float("inf")
        if self.tensor:
            budget += 0.5  # room for read-back diagonals beside the MMA ops
        for gi in remaining:
            g = gates[gi]
            bits = g.bits
            ok = all(b not in blocked_nd for b in bits) and (
                g.diagonal or all(b not in blocked_d for b in bits)
            )
            if ok and len(ops) >= MAX_OPS:
                ok = False
            if ok and not g.diagonal:
                need = [b for b in bits if b not in S]
                if len(S) + len(need) > L:
                    ok = False
                elif self.tensor and need and any(
                        b in op.sl for op in ops if op.kind == "dense" for b in need):
                    # a selector of an MMA op must stay outside the tile
                    ok = False
            if ok:
                plan = self._fusion_choice(g, gi, ops, last, S if g.diagonal else S | set(bits))
                delta = plan[0]
                if taken and cost + delta > budget:
                    ok = False
            if not ok:
                (blocked_d if g.diagonal else blocked_nd).update(bits)
                left.append(gi)
                continue
            if not g.diagonal:
                S.update(bits)
            self._apply_fusion(plan, g, gi, ops, last, batch)
            cost += delta
            taken.append(gi)
        # fill the tile to exactly L bits (an MMA op's selectors stay outside)
        sels = {s for op in ops if op.kind == "dense" for s in op.sl} if self.tensor else set()
        for b in range(nbits):
            if len(S) >= L:
                break
            if b not in S and b not in sels:
                S.add(b)
        b = 0
        while len(S) < L:  # (the pass then runs on the CUDA cores)
            S.add(b)
            b += 1
        hi = sorted(x for x in S if x >= m)
        # selectors/diag bits that ended up inside S are fine: codes are resolved at emit
        return PassPlan(L=L, m=m, hi=hi, ops=ops), left

    # ---- fusion decisions ------------------------------------------------
    def _fusion_choice(self, g: BitGate, gi: int, ops, last, S):
        """Returns (delta_cost, action...) for adding gate g to the pass."""
        bits = list(g.bits)
        if g.probe >= 0:
            return ((1 if g.diagonal else 2 ** len(bits)) + self.ovh, "new_probe")
        if self.tensor:
            return self._fusion_choice_tc(g, ops, last, S)
        c = max((last.get(b, -1) for b in bits), default=-1)
        new_cost = (2 ** len(bits) if not g.diagonal else 1) + self.ovh
        if not g.diagonal:
            # g commutes with every op after c (none of them touches its
            # bits), so any later dense op may absorb it; take the cheapest
            best = None
            for d in range(max(c, 0), len(ops)):
                op = ops[d]
                if op.kind != "dense":
                    continue
                tg = list(op.tg)
                for b in bits:
                    if b not in tg:
                        tg.append(b)
                if len(tg) > self.kmax:
                    continue
                delta = 2 ** len(tg) - 2 ** len(op.tg)
                if best is None or delta < best[0] or (delta == best[0] and d > best[2]):
                    best = (delta, "merge_dense", d)
            if best is not None and best[0] < new_cost:
                return best
            if c >= 0 and ops[c].kind != "probe":
                op = ops[c]
                if op.kind == "diag":
                    loc = [b for b in op.bits if b in S]
                    glob = [b for b in op.bits if b not in S]
                    tg = list(loc)
                    for b in bits:
                        if b not in tg:
                            tg.append(b)
                    if len(tg) <= self.kmax and len(glob) <= MAX_SEL:
                        delta = 2 ** len(tg) - op.cost(0)
                        if delta < new_cost:
                            return (delta, "diag_to_dense", c, loc, glob)
            return (new_cost, "new_dense")
        # diagonal gate: absorb into a dense op (targets/selectors) or a diag table
        lo = max(c, 0)
        best = None
        for d in range(len(ops) - 1, lo - 1, -1):
            op = ops[d]
            if op.kind == "probe":
                continue
            if op.kind == "dense":
                tg = list(op.tg)
                sl = list(op.sl)
                grow_t = []
                grow_s = []
                for b in bits:
                    if b in tg or b in sl:
                        continue
                    if len(sl) + len(grow_s) < MAX_SEL:
                        grow_s.append(b)
                    elif b in S and len(tg) + len(grow_t) < self.kmax:
                        grow_t.append(b)
                    else:
                        grow_s = None
                        break
                if grow_s is None:
                    continue
                delta = 2 ** (len(tg) + len(grow_t)) - 2 ** len(tg)
                cand = (delta, "absorb_dense", d, grow_t, grow_s)
            else:
                ub = list(op.bits) + [b for b in bits if b not in op.bits]
                if len(ub) > MAX_DIAG_BITS:
                    continue
                cand = (0.0, "absorb_diag", d)
            if best is None or cand[0] < best[0]:
                best = cand
            if best[0] == 0:
                break
        if best is not None and best[0] < new_cost:
            return best
        return (new_cost, "new_diag")

    def _fusion_choice_tc(self, g: BitGate, ops, last, S):
        """Tensor-core pass costs: an MMA op costs 1 whatever it absorbs (it
        is padded to 4 bits), a diagonal op in the read-back a little; MMA
        selectors are global bits outside the tile only (a bit inside the
        tile becomes a target)."""
        bits = list(g.bits)
        c = max((last.get(b, -1) for b in bits), default=-1)
        # B operands in shared memory: 2^nsel matrices per MMA op, at most
        # TC_MAX_MATS per pass
        nmats = sum(2 ** len(op.sl) for op in ops if op.kind == "dense")
        if not g.diagonal:
            best = None
            for d in range(max(c, 0), len(ops)):
                op = ops[d]
                if op.kind != "dense":
                    continue
                tg = set(op.tg) | set(bits)
                if len(tg) > TC_K:
                    continue
                best = (0.0, "merge_dense", d)  # the latest op that fits
            if best is not None:
                return best
            if c >= 0 and ops[c].kind == "diag":
                op = ops[c]
                loc = [b for b in op.bits if b in S]
                glob = [b for b in op.bits if b not in S]
                tg = set(loc) | set(bits)
                sel_ok = not glob or getattr(self, "_tc_selectors", True)
                if len(tg) <= TC_K and len(glob) <= MAX_SEL and nmats + 2 ** len(glob) <= TC_MAX_MATS and sel_ok:
                    return (1.0 - 0.02, "diag_to_dense", c, loc, glob)
            if nmats + 1 > TC_MAX_MATS:
                return (float("inf"), "new_dense")
            return (1.0, "new_dense")
        lo = max(c, 0)
        best = None
        for d in range(len(ops) - 1, lo - 1, -1):
            op = ops[d]
            if op.kind == "probe":
                continue
            if op.kind == "dense":
                grow_t, grow_s = [], []
                for b in bits:
                    if b in op.tg or b in op.sl:
                        continue
                    if b in S:
                        grow_t.append(b)
                    else:
                        grow_s.append(b)
                if len(op.tg) + len(grow_t) > TC_K or len(op.sl) + len(grow_s) > MAX_SEL:
                    continue
                if grow_s and not getattr(self, "_tc_selectors", True):
                    continue
                if grow_s and nmats + 2 ** len(op.sl) * (2 ** len(grow_s) - 1) > TC_MAX_MATS:
                    continue
                cand = (0.0, "absorb_dense", d, grow_t, grow_s)
            else:
                ub = list(op.bits) + [b for b in bits if b not in op.bits]
                if len(ub) > MAX_DIAG_BITS:
                    continue
                cand = (0.0, "absorb_diag", d)
            if best is None or (cand[1] == "absorb_dense" and best[1] != "absorb_dense"):
                best = cand
            if best[1] == "absorb_dense":
                break
        if best is not None:
            return best
        return (0.02, "new_diag")

    def _apply_fusion(self, plan, g: BitGate, gi: int, ops, last, batch):
        action = plan[1]
        G = batch[gi]
        bits = list(g.bits)
        if action == "new_probe":
            op = _Probe(bits=bits, M=G.copy(), diagonal=g.diagonal, slot=g.probe, recipe=[("probe", gi)])
            ops.append(op)
            idx = len(ops) - 1
        elif action == "new_dense":
            op = _Dense(tg=bits, sl=[], M=G[:, None].copy(), recipe=[("init_dense", gi, len(bits))])
            ops.append(op)
            idx = len(ops) - 1
        elif action == "new_diag":
            op = _Diag(bits=bits, d=np.diagonal(G, axis1=1, axis2=2).copy(), recipe=[("init_diag", gi, len(bits))])
            ops.append(op)
            idx = len(ops) - 1
        elif action in ("merge_dense", "diag_to_dense"):
            idx = plan[2]
            op = ops[idx]
            if action == "diag_to_dense":
                op = self._diag_to_dense(op, ops, idx, plan[3], plan[4])
            newb = [b for b in bits if b not in op.tg and b not in op.sl]
            # selectors hit by a non-diagonal gate become targets
            for b in bits:
                if b in op.sl:
                    i = op.sl.index(b)
                    step = ("s2t", i)
                    op.M = _Replayer.dense_step(op.M, step, batch)
                    op.recipe.append(step)
                    op.sl.pop(i)
                    op.tg.append(b)
            if newb:
                step = ("tx", len(newb))
                op.M = _Replayer.dense_step(op.M, step, batch)
                op.recipe.append(step)
                op.tg.extend(newb)
            pos = tuple(op.tg.index(b) for b in bits)
            step = ("mul", gi, pos)
            op.M = _Replayer.dense_step(op.M, step, batch)
            op.recipe.append(step)
        elif action == "absorb_dense":
            _, _, idx, grow_t, grow_s = plan
            op = ops[idx]
            if grow_t:
                step = ("tx", len(grow_t))
                op.M = _Replayer.dense_step(op.M, step, batch)
                op.recipe.append(step)
                op.tg.extend(grow_t)
            if grow_s:
                step = ("sx", len(grow_s))
                op.M = _Replayer.dense_step(op.M, step, batch)
                op.recipe.append(step)
                op.sl.extend(grow_s)
            tpos = tuple(op.tg.index(b) if b in op.tg else None for b in bits)
            spos = tuple(op.sl.index(b) if b in op.sl else None for b in bits)
            step = ("dmul", gi, tpos, spos)
            op.M = _Replayer.dense_step(op.M, step, batch)
            op.recipe.append(step)
        elif action == "absorb_diag":
            idx = plan[2]
            op = ops[idx]
            newb = [b for b in bits if b not in op.bits]
            if newb:
                step = ("dx", len(newb))
                op.d = _Replayer.diag_step(op.d, step, batch)
                op.recipe.append(step)
                op.bits.extend(newb)
            pos = tuple(op.bits.index(b) for b in bits)
            step = ("dd", gi, pos)
            op.d = _Replayer.diag_step(op.d, step, batch)
            op.recipe.append(step)
        else:
            raise AssertionError(action)
        for b in ops[idx].touches():
            last[b] = max(last.get(b, -1), idx)

    def _diag_to_dense(self, dop: _Diag, ops, idx, loc, glob):
        """Turns a diagonal table into a dense op: its tile bits become targets and
        its out-of-tile bits selectors (the caller checked both limits)."""
        tg = list(loc)
        sl = list(glob)
        recipe = [("diag_as_dense", list(dop.recipe), list(dop.bits), list(tg), list(sl))]
        M = _diag_to_dense_matrix(dop.d, dop.bits, tg, sl)
        op = _Dense(tg=tg, sl=sl, M=M, recipe=recipe)
        ops[idx] = op
        return op

    # ---- register phases ---------------------------------------------------------
    def _phases(self, pp: PassPlan) -> list:
        """Orders a pass's ops into register phases.

        Returns items ("layout", [register bits]) or ("op", op, on_registers).
        Ops that commute may be reordered: an op is *ready* when no earlier,
        not yet emitted op conflicts with it (one of the two acts
        non-diagonally on a bit the other touches).  A phase repeatedly takes
        every ready op whose targets fit R = L - 8 register bits (growing the
        set as needed) and whose selector bits stay out of it; diagonal ops
        fit any phase.  Ops that cannot run on registers run from shared
        memory between phases."""
        R = pp.L - 8 if (self.use_registers and pp.L <= 12) else 0
        tile = set(range(pp.m)) | set(pp.hi)
        ops = list(pp.ops)

        def writes(op):
            if op.kind == "dense":
                return set(op.tg)
            if op.kind == "probe" and not op.diagonal:
                return set(op.bits)
            return set()

        def touches(op):
            return set(op.touches())

        def targets(op):
            if op.kind == "dense":
                return list(op.tg)
            if op.kind == "probe" and not op.diagonal:
                return list(op.bits)
            return []

        def reg_ok(op):
            if op.kind == "dense":
                return len(op.tg) <= min(R, 4)
            if op.kind == "probe" and not op.diagonal:
                return len(op.bits) <= min(R, 3)
            return R > 0

        def local_sels(op):
            return {b for b in getattr(op, "sl", []) if b in tile}

        def conflicts(a, b):
            return bool(writes(a) & touches(b)) or bool(writes(b) & touches(a))

        items: list = []
        remaining = list(range(len(ops)))

        def ready(i, done_set):
            for j in remaining:
                if j >= i:
                    break
                if j not in done_set and conflicts(ops[j], ops[i]):
                    return False
            return True

        if R and ops and all(not targets(op) and reg_ok(op) for op in ops):
            # diagonals only: one register phase on the top tile bits (every
            # op of the pass then has a register form)
            items.append(("layout", sorted(tile, reverse=True)[:R]))
            items.extend(("op", op, True) for op in ops)
            return items
        while remaining:
            first = remaining[0]
            if not R or not reg_ok(ops[first]) or (not targets(ops[first]) and not any(
                    targets(ops[j]) for j in remaining)):
                # shared-memory op (or a phase would hold no dense op)
                items.append(("op", ops[first], False))
                remaining.pop(0)
                continue
            rb: list = []
            sels: set = set()
            phase: list = []
            taken: set = set()
            progress = True
            while progress:
                progress = False
                for i in list(remaining):
                    if i in taken or not reg_ok(ops[i]) or not ready(i, taken):
                        continue
                    need = [b for b in targets(ops[i]) if b not in rb]
                    nsel = sels | local_sels(ops[i])
                    if len(rb) + len(need) > R or any(b in nsel for b in rb + need):
                        continue
                    if len(tile - nsel - set(rb) - set(need)) < R - len(rb) - len(need):
                        continue
                    rb += need
                    sels = nsel
                    phase.append(i)
                    taken.add(i)
                    progress = True
            if not phase or not any(targets(ops[i]) for i in phase):
                # nothing dense fits a fresh phase: run the first op from shared memory
                if phase and not any(targets(ops[i]) for i in phase):
                    pass
                items.append(("op", ops[first], False))
                remaining.pop(0)
                continue
            free = [b for b in sorted(tile, reverse=True) if b not in rb and b not in sels]
            rb += free[: R - len(rb)]
            items.append(("layout", rb))
            for i in sorted(phase):
                items.append(("op", ops[i], True))
            remaining = [i for i in remaining if i not in taken]
        return items

    # ---- emission -----------------------------------------------------------
    def _tc_items(self, pp: PassPlan):
        """The items of a tensor-core pass (("mma", op) and diagonal ("op",
        op, False) in execution order; each diagonal runs in the read-back of
        the MMA op before it), or None when the pass cannot take that form:
        no dense op, probes, a matrix budget overrun, or a leading diagonal
        on a bit the first MMA op targets (it must act before that op).
        Dense ops are padded to 4 targets with identity bits."""
        if pp.L != TC_TILE_BITS or pp.m < 5:
            return None
        tile = set(range(pp.m)) | set(pp.hi)
        ops = list(pp.ops)
        if any(op.kind == "probe" for op in ops):
            return None
        dense = [i for i, op in enumerate(ops) if op.kind == "dense"]
        if not dense or len(dense) > TC_MAX_MMA_OPS:
            return None
        first = dense[0]
        for d in ops[:first]:  # diagonals commute with an op that does not target their bits
            if set(d.bits) & set(ops[first].tg):
                return None
        order = [ops[first]] + ops[:first] + ops[first + 1:]
        nmats = 0
        for op in order:
            if op.kind == "dense":
                if len(op.tg) > TC_K or any(b in tile for b in op.sl):
                    return None
                nmats += 2 ** len(op.sl)
        if nmats > TC_MAX_MATS:
            return None
        items = []
        for op in order:
            if op.kind != "dense":
                items.append(("op", op, False))
                continue
            if len(op.tg) < TC_K:
                pad = [b for b in sorted(tile, reverse=True) if b not in op.tg][: TC_K - len(op.tg)]
                step = ("tx", len(pad))
                op.M = _Replayer.dense_step(op.M, step, {})
                op.recipe.append(step)
                op.tg.extend(pad)
            items.append(("mma", op))
        return items

    def _emit(self, pass_plans, nbits, ngates) -> Plan:
        phased = []
        for pp in pass_plans:
            items = self._tc_items(pp) if self.tensor else None
            phased.append(items if items is not None else self._phases(pp))
        passes = np.zeros(len(pass_plans), dtype=_lib.PASS_DTYPE)
        nops = sum(len(items) for items in phased)
        ops = np.zeros(nops, dtype=_lib.OP_DTYPE)
        layout = []
        chunks = []
        off = 0
        oi = 0
        for q, (pp, items) in enumerate(zip(pass_plans, phased)):
            tile_of = {b: b for b in range(pp.m)}
            for j, b in enumerate(pp.hi):
                tile_of[b] = pp.m + j
            rec = passes[q]
            rec["L"] = pp.L
            rec["m"] = pp.m
            rec["op_begin"] = oi
            rec["op_count"] = len(items)
            rec["hi"][: len(pp.hi)] = pp.hi

            def code(b):
                return tile_of[b] if b in tile_of else -(b + 1)

            rb_cur: list = []
            for item in items:
                r = ops[oi]
                oi += 1
                if item[0] == "layout":
                    rb_cur = item[1]
                    r["kind"] = _lib.OP_LAYOUT
                    r["k"] = len(rb_cur)
                    r["bits"][: len(rb_cur)] = [tile_of[b] for b in rb_cur]
                    continue
                if item[0] == "mma":
                    op = item[1]
                    r["kind"] = _lib.OP_MMA
                    r["k"] = TC_K
                    r["nsel"] = len(op.sl)
                    r["bits"][:TC_K] = [tile_of[b] for b in op.tg]
                    r["sel"][: len(op.sl)] = [code(b) for b in op.sl]
                    data = op.M[0].reshape(-1)
                    layout.append(("dense", op.recipe, off, (op.M.shape[1], op.M.shape[2]), None))
                    r["mat"] = off
                    chunks.append(np.asarray(data).astype(np.complex64))
                    off += len(data)
                    continue
                _, op, reg = item
                perm = None
                if op.kind == "dense":
                    tg = list(op.tg)
                    if reg:
                        order = sorted(range(len(tg)), key=lambda j: rb_cur.index(tg[j]))
                        if order != list(range(len(tg))):
                            perm = _bit_perm_index(order)
                        tg = [tg[o] for o in order]
                    k = len(tg)
                    r["kind"] = _lib.OP_RDENSE if reg else _lib.OP_DENSE
                    r["k"] = k
                    r["nsel"] = len(op.sl)
                    r["bits"][:k] = [tile_of[b] for b in tg]
                    r["sel"][: len(op.sl)] = [code(b) for b in op.sl]
                    data = op.M[0]
                    if perm is not None:
                        data = data[:, perm[:, None], perm[None, :]]
                    data = data.reshape(-1)
                    layout.append(("dense", op.recipe, off, (op.M.shape[1], op.M.shape[2]), perm))
                elif op.kind == "probe":
                    r["slot"] = op.slot
                    r["k"] = len(op.bits)
                    if op.diagonal:
                        r["kind"] = _lib.OP_RPROBE_DIAG if reg else _lib.OP_PROBE_DIAG
                        r["bits"][: len(op.bits)] = [code(b) for b in op.bits]
                        data = np.diagonal(op.M[0]).copy()
                        layout.append(("probe_diag", op.recipe, off, (len(op.bits),), None))
                    else:
                        bits = list(op.bits)
                        M0 = op.M[0]
                        if reg:
                            order = sorted(range(len(bits)), key=lambda j: rb_cur.index(bits[j]))
                            if order != list(range(len(bits))):
                                perm = _bit_perm_index(order)
                                M0 = M0[perm[:, None], perm[None, :]]
                            bits = [bits[o] for o in order]
                        r["kind"] = _lib.OP_RPROBE if reg else _lib.OP_PROBE
                        r["bits"][: len(bits)] = [tile_of[b] for b in bits]
                        data = M0.reshape(-1)
                        layout.append(("probe", op.recipe, off, (len(op.bits),), perm))
                else:
                    r["kind"] = _lib.OP_RDIAG if reg else _lib.OP_DIAG
                    r["k"] = len(op.bits)
                    r["bits"][: len(op.bits)] = [code(b) for b in op.bits]
                    data = op.d[0]
                    layout.append(("diag", op.recipe, off, (len(op.bits),), None))
                r["mat"] = off
                chunks.append(np.asarray(data).astype(np.complex64))
                off += len(data)
                if off & 1:
                    chunks.append(np.zeros(1, np.complex64))
                    off += 1
        pool = _snap(np.concatenate(chunks)) if chunks else np.zeros(2, np.complex64)
        return Plan(
            nbits=nbits,
            passes=passes,
            ops=ops,
            pool=pool,
            pass_plans=pass_plans,
            ngates=ngates,
            layout=layout,
            pool_len=max(off, 2),
        )


def _bit_perm_index(order) -> np.ndarray:
    """Index map for reordering matrix-index bits: new bit q = old bit order[q]."""
    k = len(order)
    idx = np.zeros(2**k, dtype=np.int64)
    for i2 in range(2**k):
        i = 0
        for q in range(k):
            if (i2 >> q) & 1:
                i |= 1 << order[q]
        idx[i2] = i
    return idx


def _diag_to_dense_matrix(d: np.ndarray, bits, tg, sl) -> np.ndarray:
    """(P, 2^b) diagonal table over `bits` -> (P, 2^|sl|, 2^|tg|, 2^|tg|) diagonal matrices."""
    P = d.shape[0]
    ns, dt = 2 ** len(sl), 2 ** len(tg)
    s = np.arange(ns)[:, None]
    t = np.arange(dt)[None, :]
    sub = np.zeros((ns, dt), dtype=np.int64)
    for j, b in enumerate(bits):
        if b in tg:
            sub = sub | (((t >> tg.index(b)) & 1) << j)
        else:
            sub = sub | (((s >> sl.index(b)) & 1) << j)
    vals = d[:, sub]  # (P, ns, dt)
    M = np.zeros((P, ns, dt, dt), dtype=d.dtype)
    ar = np.arange(dt)
    M[:, :, ar, ar] = vals
    return M


# recipe steps that need access to nested recipes are handled here
_orig_dense_step = _Replayer.dense_step


def _dense_step(M, step, gates):
    kind = step[0]
    if kind == "init_dense":
        _, gi, k = step
        return np.asarray(gates[gi])[:, None].astype(np.complex128, copy=True)
    if kind == "diag_as_dense":
        _, sub_recipe, bits, tg, sl = step
        P = np.asarray(next(iter(gates.values()))).shape[0]
        D = np.ones((P, 1), dtype=np.complex128)
        for st in sub_recipe:
            D = _Replayer.diag_step(D, st, gates)
        return _diag_to_dense_matrix(D, bits, tg, sl)
    return _orig_dense_step(M, step, gates)


_orig_diag_step = _Replayer.diag_step


def _diag_step(D, step, gates):
    if step[0] == "init_diag":
        _, gi, k = step
        return np.diagonal(np.asarray(gates[gi]), axis1=1, axis2=2).astype(np.complex128, copy=True)
    return _orig_diag_step(D, step, gates)


_Replayer.dense_step = staticmethod(_dense_step)
_Replayer.diag_step = staticmethod(_diag_step)
