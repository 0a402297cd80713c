"""Test configuration: the `gpu` marker and import paths.

cirq itself comes from the environment; when it is not installed, the copy
of the reference installed under baseline/_ref (pure Python) is used, with
placeholders for its unused plotting/dataframe extras.
"""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

from cirq_gb300._cirq_env import ensure_cirq  # noqa: E402

ensure_cirq((os.path.join(ROOT, "baseline", "_ref"),))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
