"""The dense kernel's half-precision candidate filter, checked on the CPU.

k_grid_dense filters candidates two at a time in half precision: the
coordinates relative to the cell centre are scaled by hsc (a power of two
putting them within +-0.5) and rounded to half; velocities are scaled by
hvsc.  A pair is kept when the half |d|^2 < hfilt and the half v . d >=
-(hdot0 + hdot1 |v| hvsc).  That is exact-safe only if every pair within
the filter radius passes the first test and every pair the second test
drops has a negative reference v . r, so that all view cones reject it
(boids_capi.cpp, make_constants, holds the error budget).  This restates
the half arithmetic with numpy float16 (each operation rounded once, the
fused steps from exact float64) on pairs at the radius and at right angles
to the velocity, for cells from the smallest to the largest scale.
"""
import numpy as np

f16, f32 = np.float16, np.float32


def _fma16(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f16)


def _constants(side, rf, vmax):
    hsc = 2.0 ** np.floor(np.log2(0.5 / (1.5 * side)))
    hvsc = 2.0 ** np.floor(np.log2(0.5 / vmax))
    e = 3.0 * 2.0 ** -12
    r = rf * hsc + np.sqrt(3.0) * e
    hfilt = np.nextafter(f32(r * r * (1 + 2.0 ** -11) ** 3 + 1e-7), f32(np.inf))
    return hsc, hvsc, hfilt, f32(1.1e-3), f32(4.4e-3)


def _f16_up(x):
    h = f16(x)
    return h if float(h) >= float(x) else np.nextafter(h, f16(np.inf))


def _f16_down(x):
    h = f16(x)
    return h if float(h) <= float(x) else np.nextafter(h, f16(-np.inf))


def test_half_filter_keeps_every_pair_in_reach_and_drops_only_pairs_behind():
    rng = np.random.default_rng(5)
    for rf, side_factor, vmax in [(0.0500088, 1.012, 0.005), (0.05, 1.5, 0.005), (0.1, 1.01, 0.003),
                                  (2.0, 3.0, 0.3), (1e-3, 1.01, 1e-5), (0.05, 10.0, 0.005)]:
        side = rf * side_factor
        hsc, hvsc, hfilt, hd0, hd1 = _constants(side, rf, vmax)
        N = 60000
        cen = rng.uniform(0, 50 * side, 3).astype(f32)
        pi = (cen + rng.uniform(-0.5, 0.5, (N, 3)) * side).astype(f32)
        d = rng.standard_normal((N, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        v = rng.standard_normal((N, 3))
        v *= rng.uniform(0.02, 1.0, (N, 1)) * vmax / np.linalg.norm(v, axis=1)[:, None]
        v = v.astype(f32)
        vh = v / np.linalg.norm(v, axis=1)[:, None]
        h = N // 2  # half of them at right angles to the velocity, give or take
        d[:h] -= np.sum(d[:h] * vh[:h], axis=1)[:, None] * vh[:h]
        d[:h] /= np.linalg.norm(d[:h], axis=1)[:, None]
        d[:h] += rng.choice([0, 1e-4, -1e-4, 1e-3, -1e-3], (h, 1)) * vh[:h]
        d *= rng.uniform(0.0, 1.0, (N, 1)) ** 0.2 * rf * 0.99999  # most near the radius
        pj = (pi + d).astype(f32)
        # the kernel's half values
        hp = ((pj - cen) * f32(hsc)).astype(f16)
        hb = ((pi - cen) * f32(hsc)).astype(f16)
        dx = (hp.astype(f32) - hb.astype(f32)).astype(f16)
        d2 = _fma16(dx[:, 2], dx[:, 2], _fma16(dx[:, 1], dx[:, 1], (dx[:, 0].astype(f32) ** 2).astype(f16)))
        hv = (v * f32(hvsc)).astype(f16)
        dv = _fma16(hv[:, 2], dx[:, 2], _fma16(hv[:, 1], dx[:, 1],
                                                (hv[:, 0].astype(f32) * dx[:, 0].astype(f32)).astype(f16)))
        vv = (v * v).astype(f32)
        nv = np.sqrt(((vv[:, 0] + vv[:, 1]).astype(f32) + vv[:, 2]).astype(f32)).astype(f32)
        vt = nv * f32(hvsc)
        thr = np.array([_f16_down(-(hd0 + hd1 * x)) for x in vt], f16)
        keep_r = d2 < _f16_up(hfilt)
        keep_v = dv >= thr
        # the reference's float relative vector and dot product
        r = (pj - pi).astype(f32)
        true_d = np.sqrt((r.astype(np.float64) ** 2).sum(1))
        pr = (v * r).astype(f32)
        dot = ((pr[:, 0] + pr[:, 1]).astype(f32) + pr[:, 2]).astype(f32)
        inside = true_d < rf
        assert inside.sum() > N // 2
        assert keep_r[inside].all(), (rf, side_factor)
        assert (dot[~keep_v] < 0).all(), (rf, side_factor)
        # and the pre-test is not vacuous where cells are about the radius (the
        # usual grid; far larger cells, when the grid is capped, keep more)
        behind = (dot < 0) & inside & (np.abs(dot) > 0.1 * nv * true_d)
        if side_factor <= 1.5:
            assert (~keep_v[behind]).mean() > 0.8, (rf, side_factor, (~keep_v[behind]).mean())
