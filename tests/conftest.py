"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need an sm_103 device and the built library; everything
else runs on the CPU. The oracle under oracle/ is the checker, never the
thing under test.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "sptc-smat_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) GPU")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(ref=True)  # the reference part only where its sources are present
    return oracle


@pytest.fixture(scope="session")
def smat_mod():
    import smat
    smat.lib()
    return smat
