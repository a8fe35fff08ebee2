"""The boidsim / boidsim_grid command line without a GPU.

* option parsing and .ini reading against the rules of the reference's
  Args::Args (src/args.cpp:17-154: Boost program_options + property_tree),
  checked through --print-config, which resolves the parameters and exits
  before any device work;
* the .ptcl frames the oracle writes for the golden runs hash to the digests
  taken from the reference engine (tests/golden/ptcl_digests.json), and the
  reference's own reader, tools/swarm_util.py load_data_legacy, reads them
  (where the reference's tools are present).  The GPU tests show that the
  executables write these same bytes.
"""
import importlib.util
import json
import os
import subprocess
import sys
import types

import numpy as np
import pytest

from conftest import DATA, GOLDEN, make_params
import ptcl_io


def _ref_dir(sub):
    """A directory of the reference checkout (oracle.ref_root()), or None."""
    import oracle
    root = oracle.ref_root()
    return os.path.join(root, sub) if root and os.path.isdir(os.path.join(root, sub)) else None


REF_TOOLS = _ref_dir("tools")
REF_SETTINGS = _ref_dir("settings")


def run(exe, *args, cwd=None):
    r = subprocess.run([exe, *args], capture_output=True, text=True, cwd=cwd, timeout=60)
    return r.returncode, r.stdout + r.stderr


def config(exe, *args):
    rc, out = run(exe, "--print-config", *args)
    assert rc == 0, out
    d = {}
    for line in out.splitlines():
        k, _, v = line.partition("=")
        d[k] = v
    return d


def test_ini_values_and_command_line_precedence(cli):
    c = config(cli["boidsim"], "-s", os.path.join(DATA, "test.ini"))
    assert c["population"] == "1000" and c["time_step"] == "30" and c["field_size"] == "1"
    assert float(c["separation_sight_angle"]) == 0.9 and float(c["cohesion_force_coefficient"]) == 0.1
    assert c["initialization"] == "test" and c["random_seed"] == "12345"
    assert float(c["velocity_max"]) == 0.003 and float(c["velocity_min"]) == 0.001
    # src/args.cpp:130-153: the command line wins over the file
    c = config(cli["boidsim_grid"], "-s", os.path.join(DATA, "test.ini"), "-N", "100", "-T5",
               "--field-size=2.5", "--vmin", "0.0005", "--vmax=0.004", "--random-seed", "-7",
               "-i", "random_uniform", "-o", "x.ptcl", "--velocity-output", "v.ptcl",
               "--force-data-output")
    assert c["population"] == "100" and c["time_step"] == "5" and c["field_size"] == "2.5"
    assert float(c["velocity_min"]) == 0.0005 and float(c["velocity_max"]) == 0.004
    assert c["random_seed"] == "-7" and c["initialization"] == "random_uniform"
    assert c["output"] == "x.ptcl" and c["velocity_output"] == "v.ptcl" and c["force_data_output"] == "1"
    # doubles are read exactly (strtod rounding)
    c = config(cli["boidsim"], "-s", os.path.join(DATA, "marun2019.ini"))
    assert float(c["alignment_sight_angle"]).hex() == (0.3333333333333333).hex()
    assert c["time_step"] == "unset"  # marun2019.ini has no TIME_STEP


def test_option_guessing_and_switches(cli):
    c = config(cli["boidsim"], "--pop", "64", "--time", "3", "--force", "-qp")
    assert c["population"] == "64" and c["time_step"] == "3" and c["force_data_output"] == "1"


@pytest.mark.parametrize("args,needle", [
    (["--bogus"], "unrecognised option '--bogus'"),
    (["-Z"], "unrecognised option '-Z'"),
    (["--v", "1"], "is ambiguous"),
    (["-N", "5", "--population", "6"], "cannot be specified more than once"),
    (["-N", "abc"], "the argument ('abc') for option '--population' is invalid"),
    (["-F", "1.0x"], "for option '--field-size' is invalid"),
    (["--random-seed", "99999999999"], "for option '--random-seed' is invalid"),
    (["stray"], "too many positional options"),
    (["-T"], "the required argument for option '--time-step' is missing"),
    (["--help=1"], "does not take any arguments"),
    (["-s", "/nonexistent/settings.ini"], "cannot open file"),
])
def test_command_line_errors_exit_like_the_reference(cli, args, needle):
    rc, out = run(cli["boidsim"], *args)
    assert rc == 255, out       # exit(-1)
    assert needle in out, out


def test_help_exits_zero(cli):
    rc, out = run(cli["boidsim_grid"], "-h", "-N", "5")
    assert rc == 0 and "--population" in out and "--velocity-output" in out


INI_CASES = [
    # text, expected (key -> value or None for unset), error needle
    ("[Global]\nPOPULATION=7\n", {"population": "7"}, None),
    ("  ; comment\n# comment\n[ Global ]\n\tPOPULATION   =   8   \n\n", {"population": "8"}, None),
    ("[Global]\nFIELD_SIZE = 0.5 # inline\n", {"field_size": "unset"}, None),  # does not convert
    ("[Global]\nPOPULATION = 1.5\n", {"population": "unset"}, None),
    ("[Global]\nPOPULATION = -1\n", {"population": "4294967295"}, None),       # wraps like num_get
    ("[Global]\nPOPULATION = 0x10\n", {"population": "unset"}, None),
    ("[Global]\nFIELD_SIZE = 1e-1\nINIT = my file.bin\n", {"field_size": "0.10000000000000001",
                                                          "initialization": "my file.bin"}, None),
    ("[Global]\nFIELD_SIZE = .5\n", {"field_size": "0.5"}, None),
    ("[Global]\nFIELD_SIZE = inf\n", {"field_size": "unset"}, None),
    ("[global]\nPOPULATION = 9\n", {"population": "unset"}, None),            # case-sensitive
    ("POPULATION = 9\n[Global]\n", {"population": "unset"}, None),            # outside a section
    ("[Velocity]\nMIN = 0.002\nMAX = 0.004\n", {"velocity_min": "0.002", "velocity_max": "0.0040000000000000001"}, None),
    ("[Global]\nPOPULATION = 1\nPOPULATION = 2\n", None, "(3): duplicate key name"),
    ("[Global]\n[Global]\n", None, "(2): duplicate section name"),
    ("[Global\n", None, "(1): unmatched '['"),
    ("[Global]\nPOPULATION\n", None, "(2): '=' character not found in line"),
    ("[Global]\n= 5\n", None, "(2): key expected"),
]


@pytest.mark.parametrize("text,expect,err", INI_CASES, ids=range(len(INI_CASES)))
def test_ini_reader(cli, tmp_path, text, expect, err):
    f = tmp_path / "s.ini"
    f.write_text(text)
    if err:
        rc, out = run(cli["boidsim"], "--print-config", "-s", str(f))
        assert rc == 255 and err in out and str(f) in out, out
        return
    c = config(cli["boidsim"], "-s", str(f))
    for k, v in expect.items():
        assert c[k] == v, (k, c[k])


def _py_read_ini(path):
    """property_tree read_ini's tree, for the comparison below."""
    tree, cur = {}, None
    for raw in open(path):
        line = raw.strip()
        if not line or line[0] in ";#":
            continue
        if line[0] == "[":
            cur = tree.setdefault(line[1:line.index("]")].strip(), {})
            continue
        k, _, v = line.partition("=")
        (cur if cur is not None else tree.setdefault("", {}))[k.strip()] = v.strip()
    return tree


@pytest.mark.skipif(REF_SETTINGS is None, reason="reference settings not here")
def test_every_reference_settings_file_reads_the_same(cli):
    import glob
    files = sorted(glob.glob(os.path.join(REF_SETTINGS, "**", "*.ini"), recursive=True))
    assert files
    keys = {"separation_sight_distance": ("Separation", "SIGHT_DISTANCE"),
            "alignment_sight_angle": ("Alignment", "SIGHT_ANGLE"),
            "cohesion_force_coefficient": ("Cohesion", "FORCE_COEFFICIENT"),
            "velocity_max": ("Velocity", "MAX"), "velocity_min": ("Velocity", "MIN"),
            "field_size": ("Global", "FIELD_SIZE")}
    for path in files:
        c = config(cli["boidsim"], "-s", path)
        t = _py_read_ini(path)
        for k, (sec, key) in keys.items():
            v = t.get(sec, {}).get(key)
            if v is None:
                assert c[k] == "unset", (path, k)
            else:
                assert float(c[k]) == float(v), (path, k)


# ------------------------------------------------------------------ .ptcl bytes

DIGESTS = json.load(open(os.path.join(GOLDEN, "ptcl_digests.json")))


def oracle_ptcl(O, case):
    """The golden run's files, with the oracle as the engine."""
    prm = getattr(O, case["settings"])
    n, field, steps = case["n"], case["field"], case["steps"]
    p = make_params(O, n, field, prm)
    grid = case["engine"] == "grid"
    pos, vel = O.init_state(p, case["init"], seeded=grid, seed=case["seed"])
    port = O.GridPort(p, pos) if grid else None
    last = {}

    def step():
        if grid:
            last["f"] = port.step(pos, vel, 1, forces=True)
        else:
            last["f"] = O.step_allpairs(p, pos, vel, 1, forces=True)

    return ptcl_io.run_frames(n, field, steps, lambda: (pos, vel), step, case["force"], lambda: last["f"])


@pytest.mark.parametrize("name", sorted(DIGESTS))
def test_oracle_frames_match_reference_digests(oracle_mod, name):
    case = DIGESTS[name]
    pb, vb = oracle_ptcl(oracle_mod, case)
    assert len(pb) == case["pos_bytes"] and ptcl_io.sha256(pb) == case["pos_sha256"]
    assert len(vb) == case["vel_bytes"] and ptcl_io.sha256(vb) == case["vel_sha256"]


def _import_swarm_util():
    """tools/swarm_util.py with its plotting imports stubbed (matplotlib,
    pandas and mpl_toolkits are not installed and not used by the readers)."""
    path = os.path.join(REF_TOOLS, "swarm_util.py") if REF_TOOLS else ""
    if not os.path.exists(path):
        pytest.skip("reference tools not present")
    class Anything(types.ModuleType):
        def __getattr__(self, attr):  # plt.cm.prism and the like, as default arguments
            return Anything(attr)

        def __call__(self, *a, **k):
            return self

    for name in ("matplotlib", "matplotlib.pyplot", "pandas", "mpl_toolkits", "mpl_toolkits.mplot3d",
                 "mpl_toolkits.mplot3d.axes3d"):
        sys.modules.setdefault(name, Anything(name))
    spec = importlib.util.spec_from_file_location("ref_swarm_util", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_load_data_legacy_reads_our_frames(oracle_mod, tmp_path):
    su = _import_swarm_util()
    case = DIGESTS["boidsim_grid_marun2019_n2048_t40"]
    pb, vb = oracle_ptcl(oracle_mod, case)
    assert ptcl_io.sha256(pb) == case["pos_sha256"]  # the bytes boidsim_grid writes
    f, fv = tmp_path / "pos.ptcl", tmp_path / "vel.ptcl"
    f.write_bytes(pb)
    fv.write_bytes(vb)
    n, steps, field = case["n"], case["steps"], case["field"]
    meta = su.load_metadata(str(f))
    assert meta["N"] == n and meta["steps"] == steps and meta["x_max"] == np.float32(field)
    sdm = su.SwarmDataManager(str(f))
    assert sdm.check_metadata() and sdm.valid_steps == steps and sdm.fps == 30 and sdm.t_0 == 0
    _, frames = ptcl_io.read(str(f))
    _, vframes = ptcl_io.read(str(fv))
    for t in (0, 17, steps - 2):
        x, v = su.load_data_legacy(str(f), t)
        assert np.array_equal(x, frames[t])
        # finite-difference velocity with the wrap-around offset: the next
        # frame's velocity up to the rounding of x + v and of the wrap
        assert np.allclose(v, vframes[t + 1], atol=2e-7, rtol=0)
    X, V = su.load_data_legacy(str(f), 3, end_time=9, time_interval=2)
    assert X.shape == (3, n, 3) and np.array_equal(X[1], frames[5])


def test_swarm_util_reads_force_frames(oracle_mod, tmp_path):
    su = _import_swarm_util()
    case = DIGESTS["boidsim_grid_test_ini_n100_t30_force"]
    pb, _ = oracle_ptcl(oracle_mod, case)
    f = tmp_path / "force.ptcl"
    f.write_bytes(pb)
    sdm = su.SwarmDataManager(str(f), force=True)
    assert sdm.check_metadata()
    d = sdm.read_all()
    assert d.shape == (case["steps"], case["n"], 12)
    assert not d[0, :, 3:].any() and d[5, :, 3:].any()  # no forces before the first update


def test_generate_initialization_file_layout(oracle_mod, tmp_path):
    """tools/generate_initialization_file.py (run with the stubs) interleaves
    a position and a velocity frame into the -i file that ptcl_io restates."""
    su = _import_swarm_util()
    case = DIGESTS["boidsim_test_ini_n100_t30"]
    pb, vb = oracle_ptcl(oracle_mod, case)
    f, fv, out = tmp_path / "p.ptcl", tmp_path / "v.ptcl", tmp_path / "init.bin"
    f.write_bytes(pb)
    fv.write_bytes(vb)
    script = os.path.join(REF_TOOLS, "generate_initialization_file.py")
    argv, sys.argv = sys.argv, [script, str(f), str(fv), "14", str(out)]
    sys.modules["swarm_util"] = su
    try:
        src = open(script).read()
        exec(compile(src, script, "exec"), {"__name__": "__main__"})
    finally:
        sys.argv = argv
        sys.modules.pop("swarm_util", None)
    _, frames = ptcl_io.read(str(f))
    _, vframes = ptcl_io.read(str(fv))
    assert out.read_bytes() == ptcl_io.init_file_bytes(frames[14], vframes[14])
