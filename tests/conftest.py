"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs the oracle, golden-vector and host-logic tests on CPU;
`-m gpu` runs the CUDA parity tests through the C ABI.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.lib()


@pytest.fixture(scope="session")
def gbf():
    """libgbfusion built for sm_103a and loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    from libfusion_gb300 import build as B
    B.build()
    import libfusion_gb300 as L
    L.lib()
    return L
