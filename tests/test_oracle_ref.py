"""The oracle against the reference's own sources compiled on the host
(Sources/Shaders/lib/Light.frag, the Light*.frag ray setups and
Sources/World/Systems/ShadowVoxSystem.cpp): bit-for-bit agreement.
Skipped where the reference tree is absent (the committed golden vectors in
tests/golden/ carry the same checks there)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests import cases
from tests.refbind import bind, march, raycast


@pytest.fixture(scope="module")
def R(ref_lib, oracle_lib):
    return bind(ref_lib, oracle_lib)


def _bits(a):
    return np.asarray(a, np.float32).view(np.int32)


def test_dda_matches_reference(R):
    g = cases.noise_grid(64)
    rays = np.concatenate([cases.edge_rays(64), cases.random_rays(64, 6000, seed=11)])
    for q in rays:
        o, d, maxt = q[:3], q[3:6], float(q[6])
        r, h, n, f = raycast(R, g, o, d, maxt)
        hh, hp, nn, nf = oracle.dda_literal(g, o, d, maxt)
        hs, rec = oracle.dda(g, o, d, maxt)
        assert r == hh == hs, (q, r, hh, hs)
        assert f == nf, (q, f, nf)
        if r:
            assert np.array_equal(_bits(h), _bits(hp)) and np.array_equal(n, nn), (q, h, hp, n, nn)
            assert rec["steps"] == f
            # hit = origin + dir * best_t ; normal = -sign(dir) * select
            assert np.array_equal(_bits(o + d * rec["t"]), _bits(h)), q
            sel = np.array([rec["flags"] & 2, rec["flags"] & 4, rec["flags"] & 8]) != 0
            assert np.array_equal(-np.sign(d) * sel, n), q
        else:
            # a miss by step count / maxt repeats the identical pass four times (Light.frag:79)
            assert f in (rec["steps"], 4 * rec["steps"]), (q, f, rec)


def test_marchers_match_reference(R):
    g = cases.noise_grid(64)
    rays = np.concatenate([cases.edge_rays(64), cases.random_rays(64, 4000, seed=12)])
    for q in rays:
        o, d, dist = q[:3], q[3:6], float(q[6])
        for ss in (False, True):
            t, f = march(R, g, o, d, dist, ss)
            t2, rec = oracle.march(g, o, d, dist, super_sparse=ss)
            assert _bits(t) == _bits(t2) and f == rec["steps"], (q, ss, t, t2, f, rec)


def test_get_volume_at_matches_reference(R):
    g = cases.noise_grid(32, seed=5)
    rng = np.random.default_rng(1)
    for x, y, z in rng.integers(-3, 36, (3000, 3)):
        for mip in (0, 1):
            sz, sy, sx = g.shape
            a = R.ref_get_volume_at(g.ctypes.data_as(C.POINTER(C.c_uint8)), sx, sy, sz, int(x), int(y), int(z), mip)
            b = oracle.get_volume_at(g, int(x), int(y), int(z), mip)
            assert a == b


def test_cosine_sample_matches_reference(R):
    rng = np.random.default_rng(2)
    out = np.zeros(3, np.float32)
    worst = 0.0
    for u1, u2 in rng.random((3000, 2)).astype(np.float32):
        R.ref_cosine_sample(C.c_float(u1), C.c_float(u2), 1, out.ctypes.data_as(C.POINTER(C.c_float)))
        assert np.array_equal(out, oracle.cosine_sample(u1, u2))
        R.ref_cosine_sample(C.c_float(u1), C.c_float(u2), 0, out.ctypes.data_as(C.POINTER(C.c_float)))
        worst = max(worst, float(np.abs(out - oracle.cosine_sample(u1, u2)).max()))
    # the libm sin/cos differ from this library's own by about one ulp
    assert worst < 1e-6


def _inv_view(rng):
    a = rng.normal(size=(3, 3))
    q, _ = np.linalg.qr(a)
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = q
    m[:3, 3] = rng.uniform(2, 6, 3)
    return m.astype(np.float32)


def test_light_passes_match_reference(R):
    g = cases.noise_grid(64, seed=9)
    sz, sy, sx = g.shape
    gp = g.ctypes.data_as(C.POINTER(C.c_uint8))
    rng = np.random.default_rng(4)
    n = 1500
    f = lambda a: np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    pos = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
    nrm = axes[rng.integers(0, 6, n)]
    depth = rng.uniform(0, 0.3, n).astype(np.float32)
    noise = rng.random((n, 4)).astype(np.float32)
    rough = rng.uniform(0.05, 1, n).astype(np.float32)
    Rv = rng.normal(size=(n, 3)).astype(np.float32)
    wcp = np.zeros((n, 3), np.float32)
    viewr = np.zeros((n, 3), np.float32)
    sh_ref = np.zeros(n, np.float32)
    irr_ref = np.zeros(n, np.float32)
    t_ref = np.zeros(n, np.float32)
    iv = _inv_view(rng)
    ivc = np.ascontiguousarray(iv.T)  # column-major
    for i in range(n):
        w = np.zeros(3, np.float32)
        s = np.zeros(1, np.float32)
        ir = np.zeros(1, np.float32)
        R.ref_ambient(gp, sx, sy, sz, f(pos[i]), f(ivc), f(nrm[i]), C.c_float(depth[i]), f(noise[i]), 1, f(w), f(s),
                      f(ir))
        wcp[i], sh_ref[i], irr_ref[i] = w, s[0], ir[0]
        w2 = np.zeros(3, np.float32)
        vr = np.zeros(3, np.float32)
        t_ref[i] = R.ref_reflection(gp, sx, sy, sz, f(pos[i]), f(ivc), f(Rv[i]), f(nrm[i]), C.c_float(rough[i]),
                                    f(noise[i]), f(w2), f(vr))
        viewr[i] = vr
        assert np.array_equal(w, w2)
    sh, irr, _ = oracle.light_ambient(g, wcp, nrm, depth, noise, threads=2)
    assert np.array_equal(sh, sh_ref) and np.array_equal(_bits(irr), _bits(irr_ref))
    t, _ = oracle.light_reflection(g, wcp, nrm, viewr, rough, noise, threads=2)
    assert np.array_equal(_bits(t), _bits(t_ref))
    # point / spot: world positions in world units, light inside the grid
    wpos = rng.uniform(0.5, 5.5, (n, 3)).astype(np.float32)
    for spot in (0, 1):
        lp = np.array([3.2, 4.1, 2.7], np.float32)
        rng_ = 2.5
        ref = np.full(n, -7.0, np.float32)
        for i in range(n):
            disc = C.c_int()
            v = R.ref_point(gp, sx, sy, sz, f(wpos[i]), f(lp), f(nrm[i]), C.c_float(rng_), f(noise[i]), spot,
                            C.byref(disc))
            if not disc.value:
                ref[i] = v
        got, _ = oracle.light_point(g, wpos, nrm, noise, lp, rng_, spot=bool(spot), threads=2)
        assert np.array_equal(got, ref), spot
        assert (ref == -7.0).any() and (ref != -7.0).any()


def test_sun_dir_matches_reference(R):
    out = np.zeros(3, np.float32)
    R.ref_sun_dir(out.ctypes.data_as(C.POINTER(C.c_float)))
    v = np.array([0.3, 0.4, 0.5], np.float32)
    d = np.float32(v[0] * v[0] + v[1] * v[1]) + np.float32(v[2] * v[2])
    r = np.float32(1.0) / np.sqrt(np.float32(d))
    assert np.array_equal(out, (v * r).astype(np.float32))
