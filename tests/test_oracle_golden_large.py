"""The CPU oracle against the reference's results at the benchmarked sizes
(golden/golden_large.npz, made by golden/make_golden_large.py), on the parts
that the oracle finishes in seconds: the 20-qubit depth-20 state, the
16-qubit QAOA points and four parameters of the 16-qubit HEA gradient."""

import numpy as np

import cirq
from cirq_gb300 import workloads
from oracle.circuits import expectation_of_circuit, simulate_state_vector

GOLD = np.load(__file__.replace("test_oracle_golden_large.py", "golden/golden_large.npz"))


def test_oracle_20_qubit_layers_vs_reference():
    key = "layers_n20_d20_s0_c128"
    psi = simulate_state_vector(workloads.random_layer_circuit(20, 20, 0))
    idx = GOLD[f"{key}_idx"]
    assert len(idx) == 4096 and len(np.unique(idx)) == 4096
    assert np.max(np.abs(psi[idx] - GOLD[f"{key}_amps"])) < 1e-10
    assert abs(np.linalg.norm(psi) - GOLD[f"{key}_norm"]) < 1e-10
    p = (np.abs(psi) ** 2).reshape((2,) * 20)
    z0 = p[0].sum() - p[1].sum()
    assert abs(z0 - GOLD[f"{key}_z"][0]) < 1e-10
    np.testing.assert_allclose(p.sum(axis=tuple(range(4, 20))).reshape(-1), GOLD[f"{key}_marg4"], atol=1e-10)
    # the complex64 reference run agrees within complex64 round-off
    assert np.max(np.abs(psi[idx] - GOLD["layers_n20_d20_s0_c64_amps"])) < 1e-5


def test_oracle_qaoa_16_qubits_vs_reference():
    circuit, gammas, betas, obs, _ = workloads.qaoa_circuit(16, 4, seed=16)
    pts = GOLD["qaoa_n16_points"]
    for p, want in zip(pts[:4], GOLD["qaoa_n16_expect"][:4]):
        r = cirq.ParamResolver({**dict(zip(gammas, p[:4])), **dict(zip(betas, p[4:]))})
        assert abs(expectation_of_circuit(circuit, obs, r) - want) < 1e-9


def test_oracle_hea_16_qubit_shift_gradient_vs_reference():
    circuit, symbols, values = workloads.hea_circuit(16, 10, seed=0)
    ham = workloads.random_pauli_hamiltonian(16, 300, seed=1)
    np.testing.assert_array_equal(values, GOLD["hea_n16_l10_values"])
    for i in (0, 17, 160, 319):
        e = []
        for s in (+1, -1):
            v = values.copy()
            v[i] += s * np.pi / 2
            e.append(expectation_of_circuit(circuit, ham, cirq.ParamResolver(dict(zip(symbols, v)))).real)
        assert abs((e[0] - e[1]) / 2 - GOLD["hea_n16_l10_grad_ps"][i]) < 1e-9
