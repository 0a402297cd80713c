"""Builds and loads the CUDA engine ``libcirq_gb300.so`` and binds its C ABI.

The shared library is compiled in-tree (``cirq_gb300/lib/``) from
``cirq_gb300/csrc/*.cu`` with ``nvcc -gencode arch=compute_103a,code=sm_103a``
(GB300).  There is no CPU fallback: every simulation entry point of this
package goes through this library, and loading fails loudly when it cannot be
built or has no usable GPU.
"""

from __future__ import annotations

import concurrent.futures
import ctypes
import hashlib
import os
import shutil
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libcirq_gb300.so"
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

# numpy mirrors of the C structs (include/cirq_gb300.h); sizes are checked
# against gbq_struct_sizes() when the library is loaded.
OP_DTYPE = np.dtype(
    [
        ("kind", "i1"),
        ("k", "i1"),
        ("nsel", "i1"),
        ("pad0", "i1"),
        ("bits", "i1", (8,)),
        ("sel", "i1", (4,)),
        ("slot", "i4"),
        ("pad1", "i4"),
        ("mat", "i8"),
    ],
    align=True,
)
PASS_DTYPE = np.dtype(
    [("L", "i4"), ("m", "i4"), ("op_begin", "i4"), ("op_count", "i4"), ("hi", "i1", (16,))],
    align=True,
)
CLIFF_OP_DTYPE = np.dtype(
    [
        ("kind", "i1"),
        ("k", "i1"),
        ("lin", "i1", (6,)),
        ("q", "i4", (3,)),
        ("tab", "i4"),
        ("rec", "i4"),
        ("cond_begin", "i4"),
        ("cond_count", "i4"),
        ("p", "f4", (3,)),
    ],
    align=True,
)
CLIFF_UNITARY, CLIFF_MEASURE, CLIFF_RESET, CLIFF_NOISE, CLIFF_COND_PAULI = 0, 1, 2, 3, 4
PAULI_DTYPE = np.dtype(
    [("x", "u8"), ("zy", "u8"), ("ny", "i4"), ("pad", "i4"), ("coef", "f8")], align=True
)
POINT_DTYPE = np.dtype(
    [
        ("nbits", "i4"),
        ("pass_begin", "i4"),
        ("pass_count", "i4"),
        ("term_begin", "i4"),
        ("term_count", "i4"),
        ("pad", "i4"),
        ("mat_base", "i8"),
    ],
    align=True,
)

OP_DENSE, OP_DIAG, OP_PROBE, OP_PROBE_DIAG = 0, 1, 2, 3
OP_LAYOUT, OP_RDENSE, OP_RDIAG, OP_RPROBE, OP_RPROBE_DIAG = 4, 5, 6, 7, 8
OP_MMA = 9
MMA_TILE_BITS, MAX_MMA_OPS, MAX_MMA_MATS = 11, 8, 6

ERR_ARG, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED = -1, -2, -3, -4


class GpuError(RuntimeError):
    """A CUDA-side failure reported by the engine."""


def sources() -> list[str]:
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu")
    )


def _source_hash() -> str:
    h = hashlib.sha256()
    for path in sources() + [
        os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cuh", ".h"))
    ] + [os.path.join(INCLUDE, "cirq_gb300.h")]:
        with open(path, "rb") as f:
            h.update(os.path.basename(path).encode())
            h.update(f.read())
    h.update(" ".join(ARCH_FLAGS + NVCC_FLAGS).encode())
    return h.hexdigest()[:16]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the cirq_gb300 CUDA engine cannot be built")


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the engine for sm_103a into cirq_gb300/lib/; returns the .so path.

    Translation units compile in parallel; the build is skipped when the
    sources are unchanged since the last build.
    """
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, LIBNAME)
    stamp = os.path.join(LIBDIR, "build.stamp")
    digest = _source_hash()
    if not force and os.path.exists(out) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return out
    nvcc = nvcc_path()
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)

    def compile_one(src: str) -> str:
        obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(sources())) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = out + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, "-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(digest)
    return out


_lib = None
_lock = threading.Lock()

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_SZ = ctypes.c_size_t
_D = ctypes.c_double
_F = ctypes.c_float

# name -> argtypes (restype is int unless listed in _RESTYPES)
SIGNATURES = {
    "gbq_last_error": [],
    "gbq_version": [],
    "gbq_struct_sizes": [_P, _P, _P, _P],
    "gbq_ctx_create": [_I, _P],
    "gbq_ctx_destroy": [_P],
    "gbq_ctx_sync": [_P],
    "gbq_device_info": [_P, _P, _P, _P],
    "gbq_set_graphs": [_P, _I],
    "gbq_set_jit": [_P, _I],
    "gbq_pool_build": [_P, _I64, _P, _P, _P, _I, _P, _I64],
    "gbq_pool_build_points": [_P, _I64, _P, _I64, _P, _P, _I, _I, _P, _I64, _I],
    "gbq_cliff_validate": [_I, _P, _I, _I, _I, _I],
    "gbq_cliff_reference": [_P, _I, _P, _I, _P, _I, _P, _I, _I, _P],
    "gbq_cliff_sample": [_P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _I64, _U64, _P, _P, _I, _I],
    "gbq_jit_stats": [_P, _P, _P],
    "gbq_jit_source": [_I, _P, _P, _I, _I, _P, _SZ, _P],
    "gbq_jit_compile_check": [ctypes.c_char_p, _P],
    "gbq_jit_shutdown": [_D],
    "gbq_device_name": [_P, _P, _I],
    "gbq_launch_count": [_P, _P],
    "gbq_event_record": [_P, _I],
    "gbq_event_elapsed": [_P, _I, _I, _P],
    "gbq_set_pass_timing": [_P, _I],
    "gbq_pass_timing": [_P, _P, _P],
    "gbq_alloc": [_P, _SZ, _P],
    "gbq_free": [_P, _P],
    "gbq_host_alloc": [_SZ, _P],
    "gbq_host_free": [_P],
    "gbq_h2d": [_P, _P, _P, _SZ],
    "gbq_d2h": [_P, _P, _P, _SZ],
    "gbq_sv_set_basis": [_P, _P, _I, _U64],
    "gbq_validate_program": [_I, _P, _I, _P, _I, _I],
    "gbq_graph_create": [_P, _P, _I, _P, _I, _P, _I, _P, _P],
    "gbq_graph_launch": [_P, _P],
    "gbq_graph_destroy": [_P],
    "gbq_run": [_P, _P, _I, _P, _I, _P, _I, _P],
    "gbq_run_dual": [_P, _P, _P, _I, _P, _I, _P, _I, _P, _P],
    "gbq_reduce_slots": [_P, _P, _I, _I64, _P],
    "gbq_adjoint": [_P, _I, _I, _P, _I, _P, _I, _P, _P, _I, _P, _I, _P, _I, _P, _I, _P, _P],
    "gbq_sv_norm2": [_P, _P, _I, _P],
    "gbq_sv_scale": [_P, _P, _I, _F],
    "gbq_sv_final_renormalize": [_P, _P, _I, _P, _P],
    "gbq_sample": [_P, _P, _I, _I, _P, _I64, _P],
    "gbq_probabilities": [_P, _P, _I, _I, _P],
    "gbq_sv_expect_paulis": [_P, _P, _I, _P, _I, _P],
    "gbq_dm_expect_paulis": [_P, _P, _I, _P, _I, _P],
    "gbq_sv_expect_paulis_noalloc": [_P, _P, _I, _P, _I, _P],
    "gbq_sv_apply_paulisum": [_P, _P, _I, _P, _I, _P],
    "gbq_paulisum_cover": [_P, _I, _I, _P, _P, _P, _I],
    "gbq_sv_inner": [_P, _P, _P, _I, _P],
    "gbq_batch_expect": [_P, _P, _I, _P, _I, _P, _I, _P, _P, _I, _I, _P],
    "gbq_sv_project": [_P, _P, _I, _U64, _U64, _F],
    "gbq_points_set_zero": [_P, _P, _I, _I],
    "gbq_run_points": [_P, _P, _I, _I, _P, _I, _P, _I, _P, _I64],
    "gbq_points_expect": [_P, _P, _I, _I, _P, _I, _P],
    "gbq_points_sample": [_P, _P, _I, _I, _P, _P],
    "gbq_points_rdm": [_P, _P, _I, _I, _I, _P, _P],
    "gbq_points_dm_marginal": [_P, _P, _I, _I, _I, _I, _P, _P],
    "gbq_sv64_set_basis": [_P, _P, _I, _U64],
    "gbq_sv64_apply": [_P, _P, _I, _I, _P, _P],
    "gbq_sv64_compare": [_P, _P, _P, _I, _P],
}
_RESTYPES = {"gbq_last_error": ctypes.c_char_p}


def declared_symbols() -> list[str]:
    """Function names declared in include/cirq_gb300.h."""
    import re

    with open(os.path.join(INCLUDE, "cirq_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gbq_\w+)\s*\(", text, re.M)))


def load(path: str | None = None, build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads (building first if needed) and binds the engine library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if path is None:
            path = os.path.join(LIBDIR, LIBNAME)
            if build_if_missing:
                path = build()
        if not os.path.exists(path):
            raise RuntimeError(f"cirq_gb300 engine library not found at {path}")
        lib = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        sizes = (ctypes.c_int * 4)()
        lib.gbq_struct_sizes(
            ctypes.byref(sizes, 0), ctypes.byref(sizes, 4), ctypes.byref(sizes, 8), ctypes.byref(sizes, 12)
        )
        want = (OP_DTYPE.itemsize, PASS_DTYPE.itemsize, PAULI_DTYPE.itemsize, POINT_DTYPE.itemsize)
        if tuple(sizes) != want:
            raise RuntimeError(f"C struct sizes {tuple(sizes)} != numpy mirrors {want}")
        _lib = lib
        _register_shutdown(lib)
        return lib


class _Sentinel:
    pass


_SENTINEL = _Sentinel()


def _register_shutdown(lib) -> None:
    """At interpreter exit, stop the background compilation of specialised
    kernels before anything is torn down: Python runs atexit handlers in
    reverse order of registration, so this one (registered after the
    weakref module's own exit hook, which the dummy finalizer below forces)
    runs before the finalizers that free device buffers and graphs, and all
    of them run before the C runtime's exit handlers."""
    import atexit
    import weakref

    weakref.finalize(_SENTINEL, int)

    def _stop():
        try:
            lib.gbq_jit_shutdown(30.0)
        except Exception:  # noqa: BLE001  (exit path: never raise)
            pass

    atexit.register(_stop)


def check(rc: int, what: str = "") -> None:
    if rc == 0:
        return
    msg = _lib.gbq_last_error().decode(errors="replace") if _lib is not None else "?"
    if rc == ERR_ARG:
        raise ValueError(f"{what}: {msg}" if what else msg)
    if rc == ERR_OOM:
        raise MemoryError(f"{what}: {msg}" if what else msg)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(f"{what}: {msg}" if what else msg)
    raise GpuError(f"{what}: {msg}" if what else msg)


def validate_program(plan, dual: bool = False) -> None:
    """Runs the engine's host-side program checks (no GPU needed); raises on error."""
    lib = load()
    check(
        lib.gbq_validate_program(
            plan.nbits, plan.passes.ctypes.data, len(plan.passes), plan.ops.ctypes.data, len(plan.ops), int(dual)
        ),
        "gbq_validate_program",
    )


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    return a.ctypes.data
