"""Tensor-core (tcgen05, TF32 three-term split) passes vs the CPU emulator."""

import numpy as np
import pytest

from cirq_gb300 import _lib
from emulator import run_program
from mma_programs import as_plain, random_mma_program

pytestmark = pytest.mark.gpu


def _run(eng, n, passes, ops, pool, psi0):
    st = eng.upload(psi0.astype(np.complex64))
    pd = eng.upload(pool)
    try:
        _lib.check(
            eng.lib.gbq_run(eng.ctx, st.ptr, n, passes.ctypes.data, len(passes), ops.ctypes.data, len(ops), pd.ptr),
            "gbq_run",
        )
        eng.sync()
        out = np.empty(2**n, np.complex64)
        _lib.check(eng.lib.gbq_d2h(eng.ctx, out.ctypes.data, st.ptr, out.nbytes), "gbq_d2h")
        eng.sync()
        return out
    finally:
        st.free()
        pd.free()


@pytest.mark.parametrize("n,npasses,sel", [(11, 1, False), (14, 3, False), (20, 6, True), (22, 4, True)])
def test_mma_passes_match_emulator(n, npasses, sel):
    from cirq_gb300.engine import Engine

    eng = Engine.get(0)
    rs = np.random.RandomState(100 + n)
    passes, ops, pool = random_mma_program(rs, n, npasses, with_sel=sel)
    psi0 = rs.normal(size=2**n) + 1j * rs.normal(size=2**n)
    psi0 /= np.linalg.norm(psi0)
    ref = run_program(psi0, n, passes, ops, pool.astype(np.complex128))
    launches0 = eng.launches()
    out = _run(eng, n, passes, ops, pool, psi0)
    assert eng.launches() - launches0 == npasses
    # TF32 three-term split: about 10x the fp32 rounding error, far below
    # the 1e-5 amplitude tolerance
    assert np.abs(out - ref).max() < 1e-6
    # the same program on the fp32 CUDA-core path agrees too
    out32 = _run(eng, n, passes, as_plain(ops), pool, psi0)
    assert np.abs(out32 - ref).max() < 1e-6
