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


def mixed_force_err(f, ref):
    """The mixed-precision force metric: (max_i |dF_i| / F_rms, 99th percentile over particles of
    |dF_i| / max(|F_i|, 1e-3 F_rms)).  Both must stay <= 1e-5.  Single particles whose total force
    nearly cancels can show larger ratios; they are bounded by the first number."""
    nr = np.linalg.norm(ref, axis=1)
    rms = np.sqrt(np.mean(nr ** 2)) + 1e-300
    de = np.linalg.norm(f - ref, axis=1)
    return float(de.max() / rms), float(np.percentile(de / np.maximum(nr, 1e-3 * rms), 99))


def assert_force_parity(f, ref, precision):
    if precision == "fp64":
        assert rel_force_err(f, ref) < 1e-9
    else:
        a, b = mixed_force_err(f, ref)
        assert a < 1e-5 and b < 1e-5, (a, b)
