"""Python handle on the CUDA engine: contexts, device buffers and program runs.

Everything here calls the C ABI of ``libcirq_gb300.so`` (include/cirq_gb300.h)
through ctypes.  Device memory belongs to an :class:`Engine`; host arrays are
numpy arrays owned by the caller.
"""

from __future__ import annotations

import ctypes
import gc
import os
import threading
import time
import weakref

import numpy as np

from cirq_gb300 import _lib
from cirq_gb300._lib import check


class DeviceBuffer:
    """A device allocation owned by an Engine (freed when garbage-collected)."""

    def __init__(self, engine: "Engine", nbytes: int):
        self.engine = engine
        self.nbytes = int(nbytes)
        ptr = engine._take_spare(self.nbytes)
        if ptr is None:
            p = ctypes.c_void_p()
            check(engine.lib.gbq_alloc(engine.ctx, self.nbytes, ctypes.byref(p)), "gbq_alloc")
            ptr = p.value
        self.ptr = ptr
        self._fin = weakref.finalize(self, engine._release, self.nbytes, self.ptr)

    def free(self) -> None:
        self._fin()

    def upload(self, host: np.ndarray) -> None:
        host = np.ascontiguousarray(host)
        if host.nbytes > self.nbytes:
            raise ValueError("upload larger than the device buffer")
        check(self.engine.lib.gbq_h2d(self.engine.ctx, self.ptr, host.ctypes.data, host.nbytes), "gbq_h2d")

    def download(self, host: np.ndarray) -> np.ndarray:
        if not host.flags.c_contiguous or host.nbytes > self.nbytes:
            raise ValueError("bad host buffer")
        check(self.engine.lib.gbq_d2h(self.engine.ctx, host.ctypes.data, self.ptr, host.nbytes), "gbq_d2h")
        return host


class PinnedArrayPool:
    """Reusable pinned host buffers handed out as numpy arrays.

    Device->host copies of large states run at full link speed only into
    page-locked memory; pinning is slow, so buffers are recycled when the
    numpy array that owns one is garbage-collected."""

    def __init__(self, lib):
        self.lib = lib
        self.free: dict[int, list[int]] = {}
        self.lock = threading.Lock()
        self.allocations = 0  # buffers pinned so far (each reuse avoids one)
        self.gc_seconds = 0.0  # spent in collections that returned a buffer
        self.pin_seconds = 0.0  # spent pinning new buffers

    # pinning a large buffer costs far more than a garbage collection (0.5 s
    # for 8 GiB on a GB300 host, against tens of ms)
    GC_BYTES = 64 << 20

    def _take(self, nbytes):
        with self.lock:
            lst = self.free.get(nbytes)
            return lst.pop() if lst else None

    def array(self, shape, dtype) -> np.ndarray:
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        p = self._take(nbytes)
        if p is None and nbytes >= self.GC_BYTES:
            # results that the caller dropped but that still sit in reference
            # cycles (cirq result objects) return their buffers here
            t = time.perf_counter()
            gc.collect()
            self.gc_seconds += time.perf_counter() - t
            p = self._take(nbytes)
        if p is None:
            t = time.perf_counter()
            hp = ctypes.c_void_p()
            check(self.lib.gbq_host_alloc(nbytes, ctypes.byref(hp)), "gbq_host_alloc")
            p = hp.value
            self.allocations += 1
            self.pin_seconds += time.perf_counter() - t
        raw = (ctypes.c_char * nbytes).from_address(p)
        arr = np.frombuffer(raw, dtype=dtype).reshape(shape)
        pool = self

        class _Owner:
            pass

        owner = _Owner()
        weakref.finalize(owner, pool._release, nbytes, p)
        # keep the owner alive as long as the array (and its views) live
        arr = _OwnedArray(arr, owner)
        return arr

    def _release(self, nbytes, p):
        with self.lock:
            self.free.setdefault(nbytes, []).append(p)


class _OwnedArray(np.ndarray):
    def __new__(cls, arr, owner):
        obj = arr.view(cls)
        obj._owner = owner
        return obj

    def __array_finalize__(self, obj):
        if obj is not None:
            self._owner = getattr(obj, "_owner", None)


class Engine:
    """One CUDA context (device + stream) of the engine."""

    _instances: dict[int, "Engine"] = {}
    _lock = threading.Lock()

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        ctx = ctypes.c_void_p()
        check(self.lib.gbq_ctx_create(int(device), ctypes.byref(ctx)), "gbq_ctx_create")
        self.ctx = ctx.value
        self.device = device
        sm = ctypes.c_int()
        free = ctypes.c_size_t()
        total = ctypes.c_size_t()
        check(self.lib.gbq_device_info(self.ctx, ctypes.byref(sm), ctypes.byref(free), ctypes.byref(total)))
        self.sm_count = sm.value
        self.total_bytes = total.value
        self.pinned = PinnedArrayPool(self.lib)
        self._pool_cache: dict = {}
        self._spare: dict[int, list[int]] = {}
        self._spare_bytes = 0
        self._spare_lock = threading.Lock()

    @classmethod
    def get(cls, device: int = 0) -> "Engine":
        with cls._lock:
            eng = cls._instances.get(device)
            if eng is None:
                eng = cls(device)
                cls._instances[device] = eng
            return eng

    @staticmethod
    def _free(lib, ctx, ptr):
        try:
            lib.gbq_free(ctx, ptr)
        except Exception:
            pass

    # Freed buffers of up to SPARE_MAX bytes are kept (SPARE_TOTAL in all)
    # and handed out again for the same size: a small simulate() then needs
    # no cudaMalloc and no synchronising cudaFree.  Reuse is safe because all
    # of the engine's work is ordered on its one stream.
    SPARE_MAX = 64 << 20
    SPARE_TOTAL = 256 << 20

    def _take_spare(self, nbytes: int):
        with self._spare_lock:
            lst = self._spare.get(nbytes)
            if not lst:
                return None
            self._spare_bytes -= nbytes
            return lst.pop()

    def _release(self, nbytes: int, ptr: int) -> None:
        with self._spare_lock:
            if nbytes <= self.SPARE_MAX and self._spare_bytes + nbytes <= self.SPARE_TOTAL:
                self._spare.setdefault(nbytes, []).append(ptr)
                self._spare_bytes += nbytes
                return
        Engine._free(self.lib, self.ctx, ptr)

    def release_spare(self) -> None:
        """Frees the kept buffers."""
        with self._spare_lock:
            spare, self._spare, self._spare_bytes = self._spare, {}, 0
        for ptrs in spare.values():
            for ptr in ptrs:
                Engine._free(self.lib, self.ctx, ptr)

    # ---- buffers -------------------------------------------------------
    def alloc(self, nbytes: int) -> DeviceBuffer:
        return DeviceBuffer(self, nbytes)

    def upload(self, host: np.ndarray) -> DeviceBuffer:
        host = np.ascontiguousarray(host)
        buf = self.alloc(max(host.nbytes, 16))
        buf.upload(host)
        return buf

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        check(self.lib.gbq_device_name(self.ctx, buf, 256), "gbq_device_name")
        return buf.value.decode(errors="replace")

    def sync(self) -> None:
        check(self.lib.gbq_ctx_sync(self.ctx), "gbq_ctx_sync")

    def launches(self) -> int:
        v = ctypes.c_int64()
        check(self.lib.gbq_launch_count(self.ctx, ctypes.byref(v)))
        return v.value

    # ---- timing ----------------------------------------------------------
    def event(self, slot: int) -> None:
        check(self.lib.gbq_event_record(self.ctx, slot), "gbq_event_record")

    def elapsed_ms(self, a: int, b: int) -> float:
        v = ctypes.c_float()
        check(self.lib.gbq_event_elapsed(self.ctx, a, b, ctypes.byref(v)), "gbq_event_elapsed")
        return v.value

    def set_jit(self, mode: int | bool) -> None:
        """Pass-specialised kernels for this engine's passes: 0 (or False)
        off, 1 (or True) compiled before a program's first launch, 2 compiled
        in the background while the interpreter runs."""
        check(self.lib.gbq_set_jit(self.ctx, int(mode)), "gbq_set_jit")

    def jit_compiles(self) -> int:
        """Specialised kernels compiled by this process so far."""
        v = ctypes.c_int64()
        check(self.lib.gbq_jit_stats(ctypes.byref(v), None, None), "gbq_jit_stats")
        return v.value

    def jit_launches(self) -> int:
        """Launches of specialised kernels by this process so far."""
        v, n = ctypes.c_int64(), ctypes.c_int64()
        check(self.lib.gbq_jit_stats(ctypes.byref(v), None, ctypes.byref(n)), "gbq_jit_stats")
        return n.value

    def jit_pending(self) -> int:
        """Specialised kernels queued or being compiled now."""
        v, p = ctypes.c_int64(), ctypes.c_int64()
        check(self.lib.gbq_jit_stats(ctypes.byref(v), ctypes.byref(p), None), "gbq_jit_stats")
        return p.value

    def jit_wait(self, timeout_s: float = 300.0) -> bool:
        """Waits until no specialised kernel is being compiled; False on timeout."""
        import time

        end = time.monotonic() + timeout_s
        while self.jit_pending():
            if time.monotonic() > end:
                return False
            time.sleep(0.01)
        return True

    def set_pass_timing(self, enable: bool) -> None:
        check(self.lib.gbq_set_pass_timing(self.ctx, int(enable)), "gbq_set_pass_timing")

    def pass_timing(self) -> tuple[float, int]:
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        check(self.lib.gbq_pass_timing(self.ctx, ctypes.byref(ms), ctypes.byref(n)), "gbq_pass_timing")
        return ms.value, n.value

    # ---- state vectors -------------------------------------------------
    def new_state(
        self,
        nbits: int,
        basis: int = 0,
        initial: np.ndarray | None = None,
        nbits_dev: int | None = None,
        into: DeviceBuffer | None = None,
    ) -> DeviceBuffer:
        """A 2^nbits_dev buffer holding |basis> or `initial` (2^nbits amplitudes)
        in its first 2^nbits entries and zeros above (written into `into` when given)."""
        nbits_dev = max(nbits, nbits_dev or nbits)
        if into is not None:
            if into.nbytes < 8 * (1 << nbits_dev):
                raise ValueError("state buffer too small")
            buf = into
        else:
            buf = self.alloc(8 * (1 << nbits_dev))
        if initial is not None:
            arr = np.ascontiguousarray(np.asarray(initial, dtype=np.complex64).reshape(-1))
            if arr.size != 1 << nbits:
                raise ValueError(f"initial state has {arr.size} amplitudes, expected {1 << nbits}")
            if nbits_dev > nbits:
                check(self.lib.gbq_sv_set_basis(self.ctx, buf.ptr, nbits_dev, 0), "gbq_sv_set_basis")
            buf.upload(arr)
        else:
            check(self.lib.gbq_sv_set_basis(self.ctx, buf.ptr, nbits_dev, int(basis)), "gbq_sv_set_basis")
        return buf

    def run(self, state: DeviceBuffer, nbits: int, plan, pool_dev: DeviceBuffer | None = None,
            sync: bool = True) -> None:
        """Runs a program; with sync=False it returns once the passes are
        queued and the caller keeps `pool_dev` alive until a later sync."""
        if plan.npasses == 0:
            return
        if pool_dev is None:
            pool_dev = self.upload(plan.pool)
        check(
            self.lib.gbq_run(
                self.ctx,
                state.ptr,
                nbits,
                plan.passes.ctypes.data,
                len(plan.passes),
                plan.ops.ctypes.data,
                len(plan.ops),
                pool_dev.ptr,
            ),
            "gbq_run",
        )
        # keep the pool alive until the stream has consumed it
        if sync:
            self.sync()

    def graph(self, state: DeviceBuffer, nbits: int, plan, pool_dev: DeviceBuffer) -> "Graph":
        """Captures the program's launches on (state, pool_dev) into a CUDA graph."""
        g = ctypes.c_void_p()
        check(
            self.lib.gbq_graph_create(
                self.ctx, state.ptr, nbits, plan.passes.ctypes.data, len(plan.passes),
                plan.ops.ctypes.data, len(plan.ops), pool_dev.ptr, ctypes.byref(g),
            ),
            "gbq_graph_create",
        )
        return Graph(self, g.value, (state, pool_dev))

    def run_dual(self, psi, lam, nbits, plan, pool_dev, partial) -> None:
        if plan.npasses == 0:
            return
        check(
            self.lib.gbq_run_dual(
                self.ctx,
                psi.ptr,
                lam.ptr,
                nbits,
                plan.passes.ctypes.data,
                len(plan.passes),
                plan.ops.ctypes.data,
                len(plan.ops),
                pool_dev.ptr,
                partial.ptr if partial is not None else None,
            ),
            "gbq_run_dual",
        )

    def norm2(self, state: DeviceBuffer, nbits: int) -> float:
        v = ctypes.c_double()
        check(self.lib.gbq_sv_norm2(self.ctx, state.ptr, nbits, ctypes.byref(v)), "gbq_sv_norm2")
        return v.value

    def final_renormalize(self, state: DeviceBuffer, nbits: int) -> tuple[bool, float]:
        """The final-state renormalisation rule on the device: (applied, norm before)."""
        v = ctypes.c_int()
        nrm = ctypes.c_double()
        check(self.lib.gbq_sv_final_renormalize(self.ctx, state.ptr, nbits, ctypes.byref(v), ctypes.byref(nrm)))
        return bool(v.value), nrm.value

    def scale(self, state: DeviceBuffer, nbits: int, factor: float) -> None:
        check(self.lib.gbq_sv_scale(self.ctx, state.ptr, nbits, ctypes.c_float(factor)))

    def project(self, state, nbits, mask, value, scale) -> None:
        check(self.lib.gbq_sv_project(self.ctx, state.ptr, nbits, int(mask), int(value), ctypes.c_float(scale)))

    def download_state(self, state: DeviceBuffer, nbits: int, pinned: bool = True) -> np.ndarray:
        n = 1 << nbits
        if pinned and n >= (1 << 16):
            out = self.pinned.array((n,), np.complex64)
        else:
            out = np.empty(n, dtype=np.complex64)
        check(self.lib.gbq_d2h(self.ctx, out.ctypes.data, state.ptr, out.nbytes), "gbq_d2h")
        return out

    def sample(self, state: DeviceBuffer, nbits: int, uniforms: np.ndarray, dm: bool = False) -> np.ndarray:
        return self._sample_at(state.ptr, nbits, uniforms, dm)

    def sample_point(self, states: DeviceBuffer, slot_bits: int, point: int, nbits: int, uniforms: np.ndarray,
                     dm: bool = False) -> np.ndarray:
        """sample() of point `point` of a batch of states in slots of
        2^slot_bits amplitudes."""
        return self._sample_at(states.ptr + point * (8 << slot_bits), nbits, uniforms, dm)

    def _sample_at(self, ptr: int, nbits: int, uniforms: np.ndarray, dm: bool) -> np.ndarray:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        out = np.empty(u.size, dtype=np.uint64)
        check(
            self.lib.gbq_sample(self.ctx, ptr, nbits, int(dm), u.ctypes.data, u.size, out.ctypes.data),
            "gbq_sample",
        )
        return out

    def probabilities(self, state: DeviceBuffer, nbits: int, dm: bool = False) -> np.ndarray:
        buf = self.alloc(4 * (1 << nbits))
        check(self.lib.gbq_probabilities(self.ctx, state.ptr, nbits, int(dm), buf.ptr), "gbq_probabilities")
        out = np.empty(1 << nbits, dtype=np.float32)
        return buf.download(out)

    @staticmethod
    def pauli_records(terms) -> np.ndarray:
        rec = np.zeros(len(terms), dtype=_lib.PAULI_DTYPE)
        for i, (x, zy, ny, coef) in enumerate(terms):
            rec[i]["x"] = x
            rec[i]["zy"] = zy
            rec[i]["ny"] = ny
            rec[i]["coef"] = float(np.real(coef))
        return rec

    def expect_paulis(self, state, nbits, terms, dm: bool = False) -> np.ndarray:
        """Per-term complex values coef * <P> (terms from ir.pauli_terms).

        Complex coefficients are handled by evaluating the unit string and
        multiplying on the host."""
        if not terms:
            return np.zeros(0, dtype=np.complex128)
        unit = [(x, zy, ny, 1.0) for x, zy, ny, _ in terms]
        rec = self.pauli_records(unit)
        out = np.zeros(2 * len(terms), dtype=np.float64)
        fn = self.lib.gbq_dm_expect_paulis if dm else self.lib.gbq_sv_expect_paulis
        check(fn(self.ctx, state.ptr, nbits, rec.ctypes.data, len(rec), out.ctypes.data), "expect_paulis")
        vals = out[0::2] + 1j * out[1::2]
        return vals * np.array([c for *_, c in terms], dtype=np.complex128)

    def apply_paulisum(self, psi, nbits, terms, out) -> None:
        rec = self.pauli_records(terms)
        for t in terms:
            if abs(np.imag(t[3])) > 0:
                raise NotImplementedError("apply_paulisum needs real coefficients")
        check(
            self.lib.gbq_sv_apply_paulisum(self.ctx, psi.ptr, nbits, rec.ctypes.data, len(rec), out.ptr),
            "gbq_sv_apply_paulisum",
        )

    def paulisum_cover(self, nbits, terms, per_pass: bool = False) -> tuple:
        """(tiled passes, terms left to the per-amplitude kernel) that
        apply_paulisum uses for these terms; with per_pass, also the number
        of terms of each pass."""
        rec = self.pauli_records(terms)
        npasses, nwide = ctypes.c_int(0), ctypes.c_int(0)
        counts = np.zeros(max(1, len(rec)), dtype=np.int32)
        check(
            self.lib.gbq_paulisum_cover(rec.ctypes.data, len(rec), nbits, ctypes.byref(npasses), ctypes.byref(nwide),
                                        counts.ctypes.data, len(counts)),
            "gbq_paulisum_cover",
        )
        if per_pass:
            return npasses.value, nwide.value, counts[: npasses.value].tolist()
        return npasses.value, nwide.value

    def inner(self, a, b, nbits) -> complex:
        out = np.zeros(2, dtype=np.float64)
        check(self.lib.gbq_sv_inner(self.ctx, a.ptr, b.ptr, nbits, out.ctypes.data), "gbq_sv_inner")
        return complex(out[0], out[1])

    def reduce_slots(self, partial, nslots, ntiles, out) -> None:
        check(self.lib.gbq_reduce_slots(self.ctx, partial.ptr, nslots, int(ntiles), out.ptr), "gbq_reduce_slots")

    def batch_expect(self, points, passes, ops, pool_dev, terms, max_nbits) -> np.ndarray:
        """Per-term complex values coef_j <P_j> of every point's term block."""
        out = np.zeros(2 * max(len(terms), 1), dtype=np.float64)
        check(
            self.lib.gbq_batch_expect(
                self.ctx,
                points.ctypes.data,
                len(points),
                passes.ctypes.data,
                len(passes),
                ops.ctypes.data,
                len(ops),
                pool_dev.ptr,
                terms.ctypes.data,
                len(terms),
                int(max_nbits),
                out.ctypes.data,
            ),
            "gbq_batch_expect",
        )
        return out[0::2] + 1j * out[1::2]


    def device_info(self) -> tuple[int, int, int]:
        """(SM count, free bytes, total bytes) of the engine's GPU."""
        sm = ctypes.c_int()
        free = ctypes.c_size_t()
        total = ctypes.c_size_t()
        check(self.lib.gbq_device_info(self.ctx, ctypes.byref(sm), ctypes.byref(free), ctypes.byref(total)),
              "gbq_device_info")
        return sm.value, free.value, total.value

    # ---- batched points (states of many points back to back) ---------------
    def points_set_zero(self, states: DeviceBuffer, nbits: int, npoints: int) -> None:
        check(self.lib.gbq_points_set_zero(self.ctx, states.ptr, nbits, npoints), "gbq_points_set_zero")

    def run_points(self, states: DeviceBuffer, nbits: int, npoints: int, plan, pool_dev: DeviceBuffer,
                   pool_stride: int) -> None:
        if plan.npasses == 0:
            return
        check(
            self.lib.gbq_run_points(
                self.ctx, states.ptr, nbits, npoints, plan.passes.ctypes.data, len(plan.passes),
                plan.ops.ctypes.data, len(plan.ops), pool_dev.ptr, int(pool_stride),
            ),
            "gbq_run_points",
        )

    def points_rdm(self, states, nbits: int, npoints: int, bits) -> np.ndarray:
        """(npoints, D, D) complex reduced density matrices of the global
        index bits `bits` (bits[0] = most significant matrix index bit)."""
        k = len(bits)
        b = np.ascontiguousarray(bits, dtype=np.int32)
        out = np.zeros(npoints * (1 << (2 * k)) * 2, dtype=np.float64)
        check(self.lib.gbq_points_rdm(self.ctx, states.ptr, nbits, npoints, k, b.ctypes.data, out.ctypes.data),
              "gbq_points_rdm")
        d = 1 << k
        return (out[0::2] + 1j * out[1::2]).reshape(npoints, d, d)

    def points_dm_marginal(self, states, nbits: int, nq: int, npoints: int, bits) -> np.ndarray:
        """(npoints, 2^m) outcome probabilities of the measured index bits
        `bits` (bit j of the outcome <-> bits[j]) from the diagonals of npoints
        density matrices of nq qubits (slots of 2^nbits amplitudes)."""
        m = len(bits)
        b = np.ascontiguousarray(bits, dtype=np.int32)
        out = np.zeros(npoints << m, dtype=np.float64)
        check(self.lib.gbq_points_dm_marginal(self.ctx, states.ptr, nbits, nq, npoints, m, b.ctypes.data,
                                              out.ctypes.data), "gbq_points_dm_marginal")
        return out.reshape(npoints, 1 << m)

    def points_sample(self, states: DeviceBuffer, nbits: int, npoints: int, uniforms: np.ndarray) -> np.ndarray:
        """One basis index per point, drawn from |psi_p|^2."""
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        out = np.empty(npoints, dtype=np.uint64)
        check(self.lib.gbq_points_sample(self.ctx, states.ptr, nbits, npoints, u.ctypes.data, out.ctypes.data),
              "gbq_points_sample")
        return out

    def points_expect(self, states: DeviceBuffer, nbits: int, npoints: int, records: np.ndarray) -> np.ndarray:
        """(npoints, nterms) complex <psi_p|P_t|psi_p> for unit-coefficient records."""
        out = np.zeros(2 * npoints * max(len(records), 1), dtype=np.float64)
        if len(records):
            check(
                self.lib.gbq_points_expect(self.ctx, states.ptr, nbits, npoints, records.ctypes.data, len(records),
                                           out.ctypes.data),
                "gbq_points_expect",
            )
        vals = out[0::2] + 1j * out[1::2]
        return vals[: npoints * len(records)].reshape(npoints, len(records))


class Graph:
    """A captured program; launch() replays it on the engine's stream.  Holds
    references to the device buffers whose addresses are baked in."""

    def __init__(self, engine: Engine, handle: int, buffers):
        self.engine = engine
        self.handle = handle
        self._buffers = buffers
        self._fin = weakref.finalize(self, engine.lib.gbq_graph_destroy, handle)

    def launch(self) -> None:
        check(self.engine.lib.gbq_graph_launch(self.engine.ctx, self.handle), "gbq_graph_launch")


def default_engine(device: int | None = None) -> Engine:
    if device is None:
        device = int(os.environ.get("CIRQ_GB300_DEVICE", "0"))
    return Engine.get(device)
