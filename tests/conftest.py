import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the native libraries once per session (incremental: only stale units recompile)."""
    from se2dr_fork_gb300 import build as B
    from oracle import oracle as O
    B.build_host()
    O.build()
    return True


@pytest.fixture(scope="session")
def gpu_lib():
    from se2dr_fork_gb300 import build as B
    B.build_gpu()
    from se2dr_fork_gb300 import gpu
    return gpu.lib()


@pytest.fixture(scope="session")
def nn_lib():
    from se2dr_fork_gb300 import build as B
    B.build_nn()
    from se2dr_fork_gb300 import nn
    return nn.lib()
