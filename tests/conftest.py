import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "q-pso_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def gpu_ctx():
    import qpso
    import build as pkg_build

    pkg_build.build()
    ctx = qpso.Context(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def c1():
    import scene

    return scene.workload_c1()
