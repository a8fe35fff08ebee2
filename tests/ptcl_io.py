"""The .ptcl v0.2 data file, restated for the tests.

Layout (src/dtype.h:19-35, written by src/main.cpp:60-74 and read by
tools/swarm_util.py:6,83-113): a packed 50-byte little-endian header
``<4sBBIIIIIffffff`` = ("PTCL", 0, 2, header_length=50, N, step, t_0, fps=30,
x_min, x_max, y_min, y_max, z_min, z_max), then one frame per time step, the
state BEFORE that step's update (src/main.cpp:187-291): float32 x,y,z per boid
in id order, followed per boid by get_force's nine floats when
--force-data-output is on; a --velocity-output file holds vx,vy,vz frames
under the same header.  The initialization file read by -i is headerless:
x,y,z,vx,vy,vz float32 per boid (src/boid_simulation.cpp:113-136), the file
tools/generate_initialization_file.py builds from a frame of each.
"""
import hashlib
import struct

import numpy as np

HEADER_FORMAT = "<4sBBIIIIIffffff"
HEADER_SIZE = struct.calcsize(HEADER_FORMAT)
assert HEADER_SIZE == 50


def header(n, steps, field, t0=0, fps=30):
    f = np.float32(field)
    return struct.pack(HEADER_FORMAT, b"PTCL", 0, 2, HEADER_SIZE, n, steps, t0, fps,
                       0.0, f, 0.0, f, 0.0, f)


def read(path, dim=3):
    """(header tuple, frames[steps_in_file, N, dim]) of a .ptcl file."""
    raw = open(path, "rb").read()
    h = struct.unpack(HEADER_FORMAT, raw[:HEADER_SIZE])
    n = h[4]
    body = np.frombuffer(raw[HEADER_SIZE:], np.float32)
    assert body.size % (n * dim) == 0, "ragged frame data"
    return h, body.reshape(-1, n, dim)


def sha256(path_or_bytes):
    if isinstance(path_or_bytes, (bytes, bytearray)):
        return hashlib.sha256(path_or_bytes).hexdigest()
    return hashlib.sha256(open(path_or_bytes, "rb").read()).hexdigest()


def init_file_bytes(pos, vel):
    """Headerless x,y,z,vx,vy,vz float32 per boid."""
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    vel = np.asarray(vel, np.float32).reshape(-1, 3)
    return np.concatenate([pos, vel], axis=1).astype(np.float32).tobytes()


def run_frames(n, field, steps, frame_fn, step_fn, with_forces=False, force_fn=None):
    """Frames of the src/main.cpp loop: for t < steps, write the state, then update.

    frame_fn() -> (pos3n, vel3n); force_fn() -> 9n floats of the last update
    (zeros before the first); step_fn() advances one update.  Returns the
    bytes of the position file and of the velocity file."""
    p_out = [header(n, steps, field)]
    v_out = [header(n, steps, field)]
    forces = np.zeros((n, 9), np.float32)
    for t in range(steps):
        pos, vel = frame_fn()
        pos = np.asarray(pos, np.float32).reshape(n, 3)
        if with_forces:
            if t > 0:
                forces = np.asarray(force_fn(), np.float32).reshape(n, 9)
            p_out.append(np.concatenate([pos, forces], axis=1).tobytes())
        else:
            p_out.append(pos.tobytes())
        v_out.append(np.asarray(vel, np.float32).reshape(n, 3).tobytes())
        step_fn()
    return b"".join(p_out), b"".join(v_out)
