"""The C++ adapter include/boids_compat (class BoidSimulation with the shape
of src/boid_simulation.h:15-71 over the C ABI), without a GPU: the driver the
oracle uses to run the reference engine (oracle/ref_driver.cpp) compiles and
links against it unchanged -- against the adapter's own stand-in headers with
warnings as errors, and, where the reference's sources are here, against the
reference's own headers in place of src/boid_simulation_grid.cpp, the way a
reference build would take it.  tests/test_gpu_compat.py runs it."""
import os
import subprocess

import pytest

from conftest import ROOT

INC = os.path.join(ROOT, "include")
COMPAT = os.path.join(INC, "boids_compat")
DRIVER = os.path.join(ROOT, "oracle", "ref_driver.cpp")


def build_adapter_driver(B, out, std="c++11", ref_src=None, workdir=None):
    """libref_gb300.so: ref_driver.cpp + the adapter, linked to the library.
    With ref_src, the reference's headers declare the class and one source
    file includes the adapter's member definitions after them."""
    from boidssimulatormpi_gb300 import build as bld
    common = ["g++", "-std=" + std, "-O2", "-fPIC", "-shared", "-DREF_GRID", "-Wl,--no-undefined"]
    libs = ["-L", bld.PKG, "-lboids_gb300", "-Wl,-rpath," + bld.PKG]
    if ref_src is None:
        cmd = common + ["-Wall", "-Wextra", "-Werror", "-I", COMPAT, "-I", INC, DRIVER, "-o", out] + libs
    else:
        engine = os.path.join(workdir, "engine_gb300.cpp")
        with open(engine, "w") as f:
            f.write('#include "boid_simulation.h"\n#define BOIDS_COMPAT_INLINE\n'
                    '#include "boid_simulation_gb300.hpp"\n')
        cmd = common + ["-w", "-I", ref_src, "-I", COMPAT, "-I", INC, DRIVER, engine,
                        os.path.join(ref_src, "boid.cpp"), os.path.join(ref_src, "vector3D.cpp"),
                        "-o", out] + libs
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


REF_SYMBOLS = ("ref_create", "ref_init", "ref_set_state", "ref_update", "ref_get_state", "ref_get_force",
               "ref_grid_num", "ref_destroy")


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], check=True, capture_output=True,
                         text=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


@pytest.mark.parametrize("std", ["c++11", "c++17"])
def test_reference_driver_builds_against_the_adapter(boids_lib, tmp_path, std):
    lib = build_adapter_driver(boids_lib, str(tmp_path / "libref_gb300.so"), std)
    assert set(REF_SYMBOLS) <= _exports(lib)


def test_adapter_links_in_place_of_the_reference_engine(boids_lib, tmp_path):
    import oracle
    root = oracle.ref_root()
    src = os.path.join(root, "src") if root else None
    if not src or not os.path.exists(os.path.join(src, "boid_simulation.h")):
        pytest.skip("reference sources not here")
    lib = build_adapter_driver(boids_lib, str(tmp_path / "libref_gb300.so"), ref_src=src, workdir=str(tmp_path))
    assert set(REF_SYMBOLS) <= _exports(lib)
