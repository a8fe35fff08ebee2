#!/usr/bin/env python3
"""Generates tests/golden/*.npz from the reference engine itself.

Runs BoidSimulation::setup/init/update/get/get_force of the reference, built
from its own sources by oracle/build_ref.sh into oracle/_ref (this needs the
reference sources; the committed .npz files are what the tests read).  Cases
are the sizes of the reference's test scripts (test/compare_grid.sh: N=100,
T=30; test/compare_legacy.sh: N=1000, T=30, both with settings/test.ini and
INIT=test) and two marun2019.ini flocks.

It also writes ptcl_digests.json: SHA-256 digests of the .ptcl files the
reference's command line would write for a few runs (src/main.cpp:60-74,
187-291 driving the reference engine, frame before update), which the
boidsim / boidsim_grid executables must reproduce byte for byte.

usage: python tests/golden/make_golden.py [REFERENCE_SRC_DIR]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
import ptcl_io  # noqa: E402

CASES = [
    # name, engine, n, field, settings, init, steps
    ("grid_test_ini_n100", "grid", 100, 1.0, "TEST_INI", "test", 30),
    ("allpairs_test_ini_n100", "allpairs", 100, 1.0, "TEST_INI", "test", 30),
    ("grid_test_ini_n1000", "grid", 1000, 1.0, "TEST_INI", "test", 30),
    ("allpairs_test_ini_n1000", "allpairs", 1000, 1.0, "TEST_INI", "test", 30),
    ("grid_marun2019_n2048", "grid", 2048, 0.5, "MARUN2019", "random_uniform", 50),
]

# name, engine, n, field, settings, init, steps, --force-data-output
PTCL_CASES = [
    ("boidsim_test_ini_n100_t30", "allpairs", 100, 1.0, "TEST_INI", "test", 30, False),
    ("boidsim_grid_test_ini_n100_t30_force", "grid", 100, 1.0, "TEST_INI", "test", 30, True),
    ("boidsim_test_ini_n1000_t30_force", "allpairs", 1000, 1.0, "TEST_INI", "test", 30, True),
    ("boidsim_grid_marun2019_n2048_t40", "grid", 2048, 0.5, "MARUN2019", "random_uniform", 40, False),
]


def ptcl_digests():
    out = {}
    for name, engine, n, field, sname, init, steps, force in PTCL_CASES:
        prm = getattr(O, sname)
        p = O.params(n, field, prm["sep"], prm["ali"], prm["coh"], prm["vmax"], prm["vmin"])
        eng = O.RefEngine(engine, p, init, 12345)
        eng.init(fresh_drand48=True)
        pb, vb = ptcl_io.run_frames(n, field, steps, eng.state, lambda: eng.update(1), force, eng.forces)
        eng.close()
        out[name] = dict(engine=engine, n=n, field=field, settings=sname, init=init, seed=12345,
                         steps=steps, force=force, pos_sha256=ptcl_io.sha256(pb), pos_bytes=len(pb),
                         vel_sha256=ptcl_io.sha256(vb), vel_bytes=len(vb))
        print("digest", name)
    return out


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else None
    if not O.build_ref(src):
        sys.exit("reference sources not found; cannot generate golden vectors")
    for name, engine, n, field, sname, init, steps in CASES:
        prm = getattr(O, sname)
        p = O.params(n, field, prm["sep"], prm["ali"], prm["coh"], prm["vmax"], prm["vmin"])
        eng = O.RefEngine(engine, p, init, 12345)
        eng.init(fresh_drand48=True)
        pos0, vel0 = eng.state()
        eng.update(steps)
        pos, vel = eng.state()
        out = dict(n=n, field=field, steps=steps, engine=engine, init=init, settings=sname,
                   seed=12345, pos0=pos0, vel0=vel0, pos=pos, vel=vel, force=eng.forces())
        if engine == "grid":
            out["grid_index"] = eng.grid_index()
        eng.close()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)
    with open(os.path.join(HERE, "ptcl_digests.json"), "w") as f:
        json.dump(ptcl_digests(), f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
