"""boidsim / boidsim_grid on the GPU: the .ptcl files, resume from an
initialization file, and the reference's error exits.

* Byte identity with the reference: the files of the golden runs hash to
  the digests taken from the reference engine driven by the frame loop of
  src/main.cpp (tests/golden/ptcl_digests.json).  test_cli.py shows that
  tools/swarm_util.py load_data_legacy reads files with these digests.
* test/compare_split.sh: a run split in two through --velocity-output, an
  initialization file made from the last frame of the first half (the layout
  of tools/generate_initialization_file.py) and -i, merged, equals the
  unsplit run byte for byte.  The reference's grid engine never bins boids
  read from a file (src/boid_simulation_grid.cpp:137-160 skips
  update_list_grid); this one does, so the split works for boidsim_grid too.
* test/compare_grid.sh: boidsim and boidsim_grid write identical files
  from the same initial state.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import DATA, GOLDEN
import ptcl_io

pytestmark = pytest.mark.gpu

DIGESTS = json.load(open(os.path.join(GOLDEN, "ptcl_digests.json")))
INI = {"TEST_INI": os.path.join(DATA, "test.ini"), "MARUN2019": os.path.join(DATA, "marun2019.ini")}


def run(exe, *args):
    r = subprocess.run([exe, "-q", *map(str, args)], capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout + r.stderr


def run_ok(exe, *args):
    rc, out = run(exe, *args)
    assert rc == 0, out
    return out


@pytest.mark.parametrize("name", sorted(DIGESTS))
def test_ptcl_bytes_equal_the_reference(cli, tmp_path, name):
    c = DIGESTS[name]
    exe = cli["boidsim_grid" if c["engine"] == "grid" else "boidsim"]
    f, fv = tmp_path / "pos.ptcl", tmp_path / "vel.ptcl"
    args = ["-s", INI[c["settings"]], "-N", c["n"], "-T", c["steps"], "-F", repr(c["field"]),
            "-i", c["init"], "--random-seed", c["seed"], "-o", f, "--velocity-output", fv]
    if c["force"]:
        args.append("--force-data-output")
    run_ok(exe, *args)
    h, _ = ptcl_io.read(str(f), 12 if c["force"] else 3)
    assert h[:8] == (b"PTCL", 0, 2, 50, c["n"], c["steps"], 0, 30)
    assert f.stat().st_size == c["pos_bytes"] and ptcl_io.sha256(str(f)) == c["pos_sha256"]
    assert fv.stat().st_size == c["vel_bytes"] and ptcl_io.sha256(str(fv)) == c["vel_sha256"]


@pytest.mark.parametrize("exe_name", ["boidsim", "boidsim_grid"])
def test_split_run_resumes_bit_exact(cli, tmp_path, exe_name):
    """test/compare_split.sh with N=1000, T=30 on settings/test.ini values."""
    exe = cli[exe_name]
    N, T = 1000, 30
    t_first = T // 2
    t_last = T - t_first + 1
    full, a, av, b, init = (tmp_path / x for x in ("full", "a", "av", "b", "init"))
    common = ["-s", INI["TEST_INI"], "-N", N]
    run_ok(exe, *common, "-T", T, "-o", full)
    run_ok(exe, *common, "-T", t_first, "-o", a, "--velocity-output", av)
    _, pa = ptcl_io.read(str(a))
    _, va = ptcl_io.read(str(av))
    init.write_bytes(ptcl_io.init_file_bytes(pa[t_first - 1], va[t_first - 1]))
    run_ok(exe, *common, "-T", t_last, "-o", b, "--initialization", init)
    _, pb = ptcl_io.read(str(b))
    assert np.array_equal(pb[0].view(np.uint32), pa[t_first - 1].view(np.uint32))
    merged = ptcl_io.header(N, T, 1.0) + pa.tobytes() + pb[1:].tobytes()
    assert merged == full.read_bytes()


def test_grid_and_all_pairs_write_the_same_file(cli, tmp_path):
    """test/compare_grid.sh (N=100, T=30), from one initialization file: the
    two reference engines seed drand48 differently, so their own inits differ."""
    N, T = 100, 30
    src, vsrc, init = tmp_path / "src", tmp_path / "vsrc", tmp_path / "init"
    run_ok(cli["boidsim_grid"], "-s", INI["TEST_INI"], "-N", N, "-T", 1, "-o", src, "--velocity-output", vsrc)
    _, p0 = ptcl_io.read(str(src))
    _, v0 = ptcl_io.read(str(vsrc))
    init.write_bytes(ptcl_io.init_file_bytes(p0[0], v0[0]))
    outs = []
    for exe in ("boidsim", "boidsim_grid"):
        o = tmp_path / (exe + ".ptcl")
        run_ok(cli[exe], "-s", INI["TEST_INI"], "-N", N, "-T", T, "-i", init, "-o", o, "--force-data-output")
        outs.append(o.read_bytes())
    assert outs[0] == outs[1]


def test_output_interval_decimates_frames(cli, tmp_path):
    full, dec = tmp_path / "full", tmp_path / "dec"
    args = ["-s", INI["MARUN2019"], "-N", 4096, "-F", "0.63", "-T", 23]
    run_ok(cli["boidsim_grid"], *args, "-o", full)
    run_ok(cli["boidsim_grid"], *args, "-o", dec, "--output-interval", 4)
    hf, ff = ptcl_io.read(str(full))
    hd, fd = ptcl_io.read(str(dec))
    assert hf[5] == 23 and hd[5] == 6 and fd.shape[0] == 6
    assert np.array_equal(fd.view(np.uint32), ff[::4].view(np.uint32))


def test_large_flock_frames(cli, tmp_path, boids_lib):
    """2^18 boids with forces: frame 0 is the library's own init state with
    zero forces, and later frames carry the per-rule forces."""
    n = 1 << 18
    f = tmp_path / "big.ptcl"
    run_ok(cli["boidsim_grid"], "-s", INI["MARUN2019"], "-N", n, "-F", "2.52", "-T", 3, "-o", f,
           "--force-data-output")
    h, fr = ptcl_io.read(str(f), 12)
    assert h[4] == n and fr.shape == (3, n, 12)
    from oracle import MARUN2019 as m
    sim = boids_lib.BoidSimulation("grid")
    sim.setup(n, 2.52, *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"])
    sim.init()
    pos, _ = sim.state()
    sim.close()
    assert np.array_equal(fr[0, :, :3].reshape(-1).view(np.uint32), pos.reshape(-1).view(np.uint32))
    assert not fr[0, :, 3:].any() and fr[2, :, 3:].any()


@pytest.mark.parametrize("args,needle", [
    (["-i", "/nonexistent/init.bin", "-o", "{tmp}/x"], "Invalid initial placement type or file name"),
    (["-o", "/nonexistent/dir/out.ptcl"], "Couldn't open: /nonexistent/dir/out.ptcl"),
    (["-F", "0.15", "-o", "{tmp}/x"], "Invalid GRID_NUM"),
])
def test_error_exits(cli, tmp_path, args, needle):
    args = [a.replace("{tmp}", str(tmp_path)) for a in args]
    rc, out = run(cli["boidsim_grid"], "-s", INI["TEST_INI"], "-N", 100, "-T", 2, *args)
    assert rc == 255 and needle in out, out


def test_short_initialization_file_is_refused(cli, tmp_path):
    init = tmp_path / "short.bin"
    init.write_bytes(np.zeros(6 * 10, np.float32).tobytes())
    rc, out = run(cli["boidsim"], "-s", INI["TEST_INI"], "-N", 100, "-T", 2, "-i", init, "-o", tmp_path / "x")
    assert rc == 255 and "fewer than" in out, out
