"""The candidate filters' view-cone pre-test, checked on the CPU.

The rule kernels drop a candidate before its exact tests when its
approximate v . r (fused products over the filter's relative vector, the
candidate shifted by the segment's periodic offset) is below -|v| * dot_eps,
which is safe only if that implies an exact v . r < 0 (the reference's
float products over the minimum image, src/boid.cpp:33 with
src/boid_simulation_grid.cpp:200-214).  dot_eps = 64 ulp(max(F, 1)) +
1e-5 rf (boids_capi.cpp, make_constants).  This restates both dot
products in numpy on pairs built at right angles to the velocity, within a
few ulps, across periodic faces, and checks the implication and the margin.
"""
import numpy as np

f32 = np.float32


def _fma(a, b, c):
    # exact float32 product in float64, one rounding of the sum
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def test_dot_eps_bounds_the_filter_dot_product():
    rng = np.random.default_rng(1)
    for F in (0.6, 1.0, 4.0, 40.0):
        Ff = f32(F)
        ulpF = float(np.spacing(f32(max(Ff, 1.0))))
        rf = 0.05 * (1 + 1e-4) + 8 * ulpF
        dot_eps = f32(64 * ulpF + 1e-5 * rf)
        N = 100000
        pi = (rng.random((N, 3)) * F).astype(f32)
        d = rng.standard_normal((N, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        d *= rng.uniform(0, rf, (N, 1))
        v = rng.standard_normal((N, 3))
        v *= rng.uniform(1e-4, 0.006, (N, 1)) / np.linalg.norm(v, axis=1)[:, None]
        v = v.astype(f32)
        vh = v / np.linalg.norm(v, axis=1)[:, None]
        h = N // 2  # half the pairs at right angles, give or take
        d[:h] -= np.sum(d[:h] * vh[:h], axis=1)[:, None] * vh[:h]
        d[:h] += rng.choice([0, 1e-9, -1e-9, 1e-7, -1e-7], (h, 1)) * vh[:h]
        raw = pi.astype(np.float64) + d
        sh = np.where(raw < 0, F, np.where(raw >= F, -F, 0.0))
        pj = (raw + sh).astype(f32)
        pj[pj >= Ff] = 0
        sigma = -sh  # the candidate's image is pj + sigma
        assert (sigma != 0).any()
        # the filter: q = pi - shift, dx = pj - q, dv = fma(vz, dz, fma(vy, dy, vx * dx))
        q = np.where(sigma < 0, pi.astype(np.float64) + np.float64(Ff),
                     np.where(sigma > 0, pi.astype(np.float64) - np.float64(Ff), pi)).astype(f32)
        dx = (pj - q).astype(f32)
        dv = _fma(v[:, 2], dx[:, 2], _fma(v[:, 1], dx[:, 1], (v[:, 0] * dx[:, 0]).astype(f32)))
        # the reference: t = (float)((double)pj + shift), r = t - pi, ((vx rx + vy ry) + vz rz)
        t = (pj.astype(np.float64) + sigma).astype(f32)
        r = (t - pi).astype(f32)
        pr = (v * r).astype(f32)
        dot = ((pr[:, 0] + pr[:, 1]).astype(f32) + pr[:, 2]).astype(f32)
        vv = (v * v).astype(f32)
        nv = np.sqrt(((vv[:, 0] + vv[:, 1]).astype(f32) + vv[:, 2]).astype(f32)).astype(f32)
        dropped = dv < -(nv * dot_eps)
        assert not (dropped & (dot >= 0)).any(), F
        gap = np.abs(dv.astype(np.float64) - dot.astype(np.float64)) / nv
        assert gap.max() < 0.1 * float(dot_eps), (F, gap.max(), dot_eps)
        assert dropped.sum() > N // 8  # the pre-test does drop the pairs behind
