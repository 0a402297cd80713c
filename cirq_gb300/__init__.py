"""GB300 (sm_103a) drop-in for Cirq's circuit-simulation path.

``cirq_gb300.Simulator`` and ``cirq_gb300.DensityMatrixSimulator`` keep the
API of ``cirq.Simulator`` / ``cirq.DensityMatrixSimulator`` (simulate,
simulate_sweep, run, simulate_expectation_values, compute_amplitudes) at
``dtype=np.complex64``.  The host side (this package) translates circuits,
plans fused tile passes and calls hand-written CUDA kernels through the C ABI
declared in ``include/cirq_gb300.h``.  Additions the reference lacks:
adjoint gradients behind ``torch.autograd.Function`` (``cirq_gb300.adjoint``)
and batched multi-point / mixed-width sweeps in one persistent launch
(``cirq_gb300.batch``).  Clifford circuits sample as Pauli frames on the GPU
(``cirq_gb300.StabilizerSampler``, ``cirq_gb300.CliffordSimulator.run``).

cirq is imported lazily, when a simulator is first requested, so the engine
library can be built without it.
"""

__version__ = "0.1.0"
__all__ = [
    "Simulator",
    "DensityMatrixSimulator",
    "CliffordSimulator",
    "StabilizerSampler",
    "sample",
    "sample_sweep",
    "final_state_vector",
    "final_density_matrix",
]


def __getattr__(name):
    if name in ("Simulator", "DensityMatrixSimulator"):
        from cirq_gb300 import simulator

        return getattr(simulator, name)
    if name in ("CliffordSimulator", "StabilizerSampler"):
        from cirq_gb300 import clifford

        return getattr(clifford, name)
    if name in ("sample", "sample_sweep", "final_state_vector", "final_density_matrix"):
        from cirq_gb300 import mux

        return getattr(mux, name)
    raise AttributeError(f"module 'cirq_gb300' has no attribute {name!r}")
