"""pytest configuration: the `gpu` marker, import paths and native builds."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def built():
    """Native libraries of the package (built in-tree if missing)."""
    from gen import build as gen_build
    from simcoflow_gb300 import build
    gen_build.build()
    if not (ROOT / "simcoflow_gb300" / "_lib" / "libscf_proj.so").exists():
        build.build_proj()
    return True


@pytest.fixture(scope="session")
def cuda(built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("test marked gpu but no CUDA device is visible")
    from simcoflow_gb300 import projection
    projection.load()
    return torch.device("cuda:0")
