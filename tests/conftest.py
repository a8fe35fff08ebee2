import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def boids_lib():
    """The product library, built in-tree if needed (fails loudly otherwise)."""
    import boidssimulatormpi_gb300 as B
    from boidssimulatormpi_gb300 import build as bld
    bld.build()
    B.lib()
    return B


def make_params(oracle, n, field, prm):
    return oracle.params(n, field, prm["sep"], prm["ali"], prm["coh"], prm["vmax"], prm["vmin"])


def make_sim(B, engine, n, field, prm, record_forces=True):
    """engine: "grid", "allpairs" (which runs the grid kernels where they
    fit) or "pairs" (the all-pairs engine on its own N^2 kernels)."""
    if engine == "pairs":
        s = B.BoidSimulation("allpairs", record_forces=record_forces, allpairs_kernels=True)
    else:
        s = B.BoidSimulation(engine, record_forces=record_forces)
    s.setup(n, field, *prm["sep"], *prm["ali"], *prm["coh"], prm["vmax"], prm["vmin"])
    return s


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_bits_equal(a, b, what=""):
    """Bit-for-bit equality of float32 arrays (NaNs compare equal to NaNs)."""
    a = np.ascontiguousarray(a, np.float32).reshape(-1)
    b = np.ascontiguousarray(b, np.float32).reshape(-1)
    assert a.shape == b.shape, what
    nan = np.isnan(a) & np.isnan(b)
    diff = (bits(a) != bits(b)) & ~nan
    if diff.any():
        idx = np.nonzero(diff)[0]
        raise AssertionError("%s: %d of %d values differ; first at %d: %r vs %r"
                             % (what, idx.size, a.size, idx[0], a[idx[0]], b[idx[0]]))


@pytest.fixture(scope="session")
def cli(boids_lib):
    """Paths of the boidsim / boidsim_grid executables (built with the library)."""
    from boidssimulatormpi_gb300 import build as bld
    paths = {name: os.path.join(bld.BIN, name) for name in ("boidsim", "boidsim_grid")}
    for p in paths.values():
        assert os.access(p, os.X_OK), p
    return paths


DATA = os.path.join(ROOT, "tests", "data")


@pytest.fixture(scope="session")
def capi_caller(boids_lib, tmp_path_factory):
    """tests/native/capi_caller.c, a plain C99 caller of the C ABI, compiled
    with warnings as errors against include/boids.h and linked against the
    in-tree library."""
    import subprocess
    from boidssimulatormpi_gb300 import build as bld
    exe = str(tmp_path_factory.mktemp("capi") / "capi_caller")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O2", "-I", bld.INCLUDE,
                    os.path.join(ROOT, "tests", "native", "capi_caller.c"), "-L", bld.PKG, "-lboids_gb300",
                    "-Wl,-rpath," + bld.PKG, "-o", exe], check=True)
    return exe
