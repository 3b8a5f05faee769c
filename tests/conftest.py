import gzip
import os
import shutil
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the product kernels)")


@pytest.fixture(scope="session")
def lib():
    from mfa_brush_gb300 import build, abi
    build.build()
    return abi.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def try_dir(tmp_path_factory):
    """The reference's try/ deck (Filled_Channel flags), with conf_old unpacked."""
    d = tmp_path_factory.mktemp("try")
    src = os.path.join(GOLDEN, "try")
    for f in ("system_input", "mfa_input", "control_simulation.h", "kat.json"):
        shutil.copyfile(os.path.join(src, f), os.path.join(d, f))
    with gzip.open(os.path.join(src, "conf_old.gz"), "rb") as g, open(os.path.join(d, "conf_old"), "wb") as f:
        f.write(g.read())
    return str(d)


@pytest.fixture(scope="session")
def try_deck(lib, try_dir):
    from mfa_brush_gb300 import md
    return md.read_deck(try_dir)


@pytest.fixture(scope="session")
def gpu(lib):
    from mfa_brush_gb300 import md
    if md.device_count() < 1:
        pytest.fail("no CUDA device visible: GPU tests need a GB300")
    return True


def rel_force_err(f, ref, floor=None):
    """max_i |f_i - ref_i| / max(|ref_i|, floor); floor defaults to 1e-3 x the RMS force."""
    nr = np.linalg.norm(ref, axis=1)
    if floor is None:
        floor = 1e-3 * np.sqrt(np.mean(nr ** 2)) + 1e-300
    return float(np.max(np.linalg.norm(f - ref, axis=1) / np.maximum(nr, floor)))
