"""The C ABI without a GPU: the library loads, exports every function that
include/boids.h declares, and rejects bad configurations before touching the
device, with the reference's error conditions."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "boids.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z0-9_ ]+?\s*\**\s*(boids_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_api():
    fns = header_functions()
    for f in ("boids_create", "boids_step", "boids_get_state", "boids_get_forces", "boids_get_cells",
              "boids_destroy", "boids_last_error", "boids_step_noalloc"):
        assert f in fns


def test_library_exports_every_declared_symbol(boids_lib):
    L = boids_lib.lib()
    for f in header_functions():
        assert hasattr(L, f), f
    assert set(header_functions()) == set(boids_lib.SIGNATURES)


def test_version_and_last_error(boids_lib):
    L = boids_lib.lib()
    assert b"sm_103a" in L.boids_version()
    assert isinstance(L.boids_last_error(), bytes)


def _params(B, **kw):
    from oracle import MARUN2019 as m
    d = dict(n=1000, field=1.0, engine=B.ENGINE_GRID)
    d.update(kw)
    return B.Params(d["n"], d["field"], *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"],
                    d["engine"], 0, 0, 0)


@pytest.mark.parametrize("kw,needle", [
    (dict(field=0.0), "field_size"),
    (dict(field=float("inf")), "field_size"),
    (dict(field=0.09), "Invalid GRID_NUM"),   # int(F/2R) == 0
    (dict(field=0.20000000298023224), "Invalid GRID_NUM"),  # GRID_NUM 2, 2R >= GRID_SIZE: aborts
    (dict(field=0.15), "GRID_NUM == 1"),      # the reference double-lists boids
    (dict(n=(1 << 29) + 1), "2^29"),
    (dict(engine=7), "engine"),
])
def test_create_rejects_like_the_reference(boids_lib, kw, needle):
    B = boids_lib
    L = B.lib()
    p = _params(B, **kw)
    h = C.c_void_p()
    rc = L.boids_create(C.byref(p), C.byref(h))
    assert rc == -1 and not h.value
    assert needle in L.boids_last_error().decode()


def test_allpairs_engine_has_no_grid_check(boids_lib):
    # the all-pairs reference engine has no grid check (src/boid_simulation.cpp:46-77):
    # a field the grid engine refuses passes validation and only meets the device
    B = boids_lib
    L = B.lib()
    p = _params(B, field=0.09, engine=B.ENGINE_ALLPAIRS)
    h = C.c_void_p()
    rc = L.boids_create(C.byref(p), C.byref(h))
    assert rc in (0, -3), L.boids_last_error().decode()  # -3: no GPU in this process
    if rc == 0:
        L.boids_destroy(h)


def test_null_arguments(boids_lib):
    L = boids_lib.lib()
    assert L.boids_create(None, None) == -1
    assert L.boids_step(None, 1) == -1
    assert L.boids_get_state(None, None, None) == -1
    assert L.boids_set_state(None, None, None) == -1
    assert L.boids_set_population(None, 0, None, None) == -1
    assert b"null handle" in L.boids_last_error()
    assert L.boids_step_noalloc(None, None, None, None, None, None) == -1


def test_noalloc_rejects_before_device_work(boids_lib):
    B = boids_lib
    L = B.lib()
    p = _params(B, engine=B.ENGINE_ALLPAIRS)
    dummy = C.c_void_p(16)
    assert L.boids_step_noalloc(C.byref(p), dummy, dummy, dummy, dummy, None) == -1
    assert "grid engine" in L.boids_last_error().decode()


def test_c_caller_builds_and_reports_errors(capi_caller, tmp_path):
    """A C99 program using only include/boids.h compiles with -Wall -Wextra
    -Werror -pedantic and links against the library.  Its usage error needs
    no device; without a GPU the library's first device call returns a
    status and a message instead of aborting the caller."""
    import subprocess
    r = subprocess.run([capi_caller], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([capi_caller, "64", "1.0", "2", str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=120)
    if r.returncode != 0:  # no usable GPU here
        assert r.returncode == 3, r.stderr
        assert "boids_create failed (%d)" % -3 in r.stderr, r.stderr


def test_missing_library_fails_loudly(boids_lib, monkeypatch):
    """Without the built library the binding raises; there is no fallback."""
    monkeypatch.setattr(boids_lib, "_lib", None)
    monkeypatch.setattr(boids_lib, "LIB_PATH", os.path.join(ROOT, "no-such-dir", "libboids_gb300.so"))
    with pytest.raises(RuntimeError, match="not built"):
        boids_lib.lib()


def test_product_never_uses_the_oracle():
    """The oracle is test infrastructure: no module or source file of the
    package imports, includes or loads it."""
    import ast
    pkg = os.path.join(ROOT, "boidssimulatormpi_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            path = os.path.join(dirpath, f)
            if f.endswith(".py"):
                tree = ast.parse(open(path).read(), path)
                for node in ast.walk(tree):
                    if isinstance(node, ast.Import):
                        names = [a.name for a in node.names]
                    elif isinstance(node, ast.ImportFrom):
                        names = [node.module or ""]
                    else:
                        continue
                    assert not any(n.split(".")[0] == "oracle" for n in names), path
            elif f.endswith((".cu", ".cpp", ".h")):
                assert "oracle" not in open(path).read(), path


def test_header_from_cxx(boids_lib, tmp_path):
    """include/boids.h compiles as C++11 with -Wall -Wextra -Werror -pedantic
    and its functions link as extern "C"; a bad configuration is refused
    before any device work."""
    import subprocess
    from boidssimulatormpi_gb300 import build as bld
    exe = str(tmp_path / "capi_cxx_check")
    subprocess.run(["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", bld.INCLUDE,
                    os.path.join(ROOT, "tests", "native", "capi_cxx_check.cpp"), "-L", bld.PKG, "-lboids_gb300",
                    "-Wl,-rpath," + bld.PKG, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("-1 ") and "field_size" in r.stdout
