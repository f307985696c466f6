"""Oracle pin for primary visibility: the oracle's restatement of
clipToAABB / intersectVolume (Sources/Shaders/GeometryVoxel.frag:50-125)
and of VoxAsset::Upload's mips (Sources/Asset/VoxAsset.cpp:3-63) against the
reference's own code compiled on the host (oracle/_ref), bit for bit: hit
flag, hit-position and normal bits, material and the number of texel
fetches, over random volumes, rays, cameras (near and far, so both branches
of the LOD test run), UVs and frames (glass voxels dithered by frame)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.gpu_util import same_bits

fp = C.POINTER(C.c_float)
u8 = C.POINTER(C.c_uint8)


def _bind(R):
    R.ref_clip_intersect.argtypes = [u8, u8, u8, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.c_float, C.c_float,
                                     C.c_float, C.c_float, C.c_int, C.c_int, fp, fp, C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_int)]
    R.ref_mip_down.argtypes = [u8, C.c_int, C.c_int, C.c_int, u8]
    return R


def _u8(a):
    return a.ctypes.data_as(u8)


def _f(a):
    return a.ctypes.data_as(fp)


def _ref_mips(R, vol):
    d = oracle.mip_dims(vol.shape[::-1])
    m1 = np.zeros(d[1][::-1], np.uint8)
    m2 = np.zeros(d[2][::-1], np.uint8)
    R.ref_mip_down(_u8(vol), d[0][0], d[0][1], d[0][2], _u8(m1))
    R.ref_mip_down(_u8(m1), d[1][0], d[1][1], d[1][2], _u8(m2))
    return m1, m2


def _volume(rng, shape, fill, glass=0.2):
    v = (rng.random(shape) < fill).astype(np.uint8) * rng.integers(16, 256, shape).astype(np.uint8)
    g = rng.random(shape) < fill * glass
    v[g] = rng.integers(1, 16, int(g.sum())).astype(np.uint8)
    return np.ascontiguousarray(v)


def test_volume_mips_match_reference(ref_lib):
    R = _bind(ref_lib)
    rng = np.random.default_rng(1)
    for _ in range(40):
        shape = tuple(int(4 * rng.integers(1, 13)) for _ in range(3))
        vol = _volume(rng, shape, float(rng.uniform(0.01, 0.6)))
        want = _ref_mips(R, vol)
        got = oracle.volume_mips(vol)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def _rays(rng, dims, n):
    dims = np.asarray(dims, np.float32)
    out = []
    for i in range(n):
        kind = i % 5
        target = rng.uniform(0, 1, 3) * dims
        if kind == 4:  # origin inside the volume: clipToAABB returns it unchanged
            o = rng.uniform(0, 1, 3) * dims
        else:
            o = target + rng.normal(size=3) * (dims.max() * rng.uniform(1.0, 3.0))
        d = target - o
        if kind == 1:  # axis-aligned component(s)
            d[rng.integers(0, 3)] = 0.0
        if kind == 2:  # exact diagonal
            d = np.sign(rng.normal(size=3)) * 1.0
        nrm = np.linalg.norm(d)
        d = d / nrm if nrm > 0 else np.array([1.0, 0.0, 0.0])
        lc = o if rng.random() < 0.5 else o - d * rng.uniform(1000.0, 6000.0)  # far camera: LOD accepts coarse hits
        uv = rng.uniform(-1, 1, 2)
        out.append((o.astype(np.float32), d.astype(np.float32), lc.astype(np.float32), uv.astype(np.float32),
                    int(rng.integers(0, 4))))
    return out


@pytest.mark.parametrize("fill", [0.02, 0.15, 0.5])
def test_clip_intersect_matches_reference(ref_lib, fill):
    R = _bind(ref_lib)
    rng = np.random.default_rng(int(fill * 1000))
    hits = 0
    lod_or_glass = 0
    for _ in range(12):
        shape = tuple(int(4 * rng.integers(2, 12)) for _ in range(3))
        vol = _volume(rng, shape, fill)
        m1, m2 = _ref_mips(R, vol)
        sz, sy, sx = vol.shape
        for o, d, lc, uv, frame in _rays(rng, (sx, sy, sz), 120):
            res = np.array([1920.0, 1080.0], np.float32)
            h = np.zeros(3, np.float32)
            nn = np.zeros(3, np.float32)
            mat = C.c_uint32()
            fe = C.c_int()
            r = R.ref_clip_intersect(_u8(vol), _u8(m1), _u8(m2), sx, sy, sz, _f(o), _f(d), _f(lc), uv[0], uv[1],
                                     res[0], res[1], frame, 1, _f(h), _f(nn), C.byref(mat), C.byref(fe))
            got = oracle.clip_intersect((vol, m1, m2), o, d, lc, uv=uv, res=res, frame=frame)
            assert got[0] == r
            assert got[4] == fe.value
            if r:
                hits += 1
                assert same_bits(got[1], h).all() and same_bits(got[2], nn).all()
                assert got[3] == mat.value
                if mat.value < 16 or np.linalg.norm(lc - o) > 500:
                    lod_or_glass += 1
    assert hits > 100 and lod_or_glass > 10
