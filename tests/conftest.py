import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "xpbd-tissue-sim_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, built in-tree if needed (build() also runs on CPU)."""
    import build as pkg_build
    import xpbd_gb300

    pkg_build.build()
    return xpbd_gb300.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


def reference_dir():
    """The reference checkout, when this machine has one: XPBD_REFERENCE_DIR,
    else the checkout the oracle's reference recipe (oracle/ref/Makefile)
    builds from. None when absent (the GPU machine has none)."""
    d = os.environ.get("XPBD_REFERENCE_DIR")
    if not d:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "print-ref"],
                           capture_output=True, text=True)
        d = r.stdout.strip()
    return d if d and os.path.isdir(d) else None
