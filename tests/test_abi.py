"""The C-ABI library builds, loads and exports every declared symbol (no GPU needed)."""

import ctypes


from cirq_gb300 import _lib


def test_library_exports_every_declared_symbol():
    path = _lib.build()
    raw = ctypes.CDLL(path)
    declared = _lib.declared_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(raw, s)]
    assert not missing, missing
    # every declared symbol has a ctypes binding and vice versa
    assert sorted(_lib.SIGNATURES) == declared


def test_struct_layouts_match_numpy_mirrors():
    lib = _lib.load()
    sizes = (ctypes.c_int * 4)()
    lib.gbq_struct_sizes(ctypes.byref(sizes, 0), ctypes.byref(sizes, 4), ctypes.byref(sizes, 8), ctypes.byref(sizes, 12))
    assert tuple(sizes) == (
        _lib.OP_DTYPE.itemsize,
        _lib.PASS_DTYPE.itemsize,
        _lib.PAULI_DTYPE.itemsize,
        _lib.POINT_DTYPE.itemsize,
    )
    assert _lib.OP_DTYPE.fields["mat"][1] == 24
    assert lib.gbq_version() == 1


def test_context_creation_fails_cleanly_without_gpu():
    """Without a usable device the ABI returns an error code and a message."""
    lib = _lib.load()
    ctx = ctypes.c_void_p()
    rc = lib.gbq_ctx_create(0, ctypes.byref(ctx))
    if rc == 0:  # a GPU is present: just release it
        lib.gbq_ctx_destroy(ctx)
        return
    assert rc < 0
    assert lib.gbq_last_error()
    rc = lib.gbq_ctx_create(10_000, ctypes.byref(ctx))
    assert rc < 0
