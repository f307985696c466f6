"""RayVoxCast (Sources/World/Systems/PhysicsSystem.cpp:98-145), the engine's
own CPU DDA for picking one placed model.

Three checks of the oracle's restatement (oracle.ray_vox_cast):
* against the reference's function, compiled unmodified from its source by
  oracle/ref/build_ref.py: hit flags and t bits;
* against the golden vectors that same build produced
  (tests/golden/rayvox.npz), where the reference tree is absent;
* against the oracle's Light.frag DDA, whose stepping it shares. From an
  empty origin cell inside the model both visit the same cells; RayVoxCast
  tests them after stepping and Light.frag before. So they hit the same cell,
  with one fetch fewer for RayVoxCast. Its t is the entry time of that cell,
  Light.frag's the exit time."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from oracle.ref import build_ref
from tests import vox_cases

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _models(rng):
    shapes = [(8, 8, 8), (12, 20, 16), (32, 16, 24), (40, 8, 12), (16, 36, 28), (24, 24, 24)]
    return [vox_cases.random_model(rng, sx, sy, sz, fill=f) for (sz, sy, sx), f in
            zip(shapes, (0.4, 0.15, 0.05, 0.3, 0.02, 0.6))]


def _ref():
    if not build_ref.available():
        pytest.skip("reference sources not present on this machine")
    from tests.refbind import bind

    return bind(C.CDLL(build_ref.build()), oracle)


def _f(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))


def _ref_inverse(R, obb):
    inv = np.zeros(16, np.float32)
    R.ref_glm_inverse(_f(obb), _f(inv))
    return inv


def test_ray_vox_cast_matches_reference():
    R = _ref()
    rng = np.random.default_rng(21)
    models = _models(rng) + vox_cases.farmhouse_models(limit=4)
    cases = vox_cases.rayvox_cases(rng, [m.shape for m in models], n_per_model=300)
    hits = nudged = 0
    for mi, obb, p, d in cases:
        m = np.ascontiguousarray(models[mi])
        sz, sy, sx = m.shape
        t_ref = np.zeros(1, np.float32)
        h_ref = R.ref_ray_vox_cast(_f(obb), m.ctypes.data_as(C.POINTER(C.c_uint8)), sx, sy, sz, _f(p), _f(d),
                                   _f(t_ref))
        h, t, _, _ = oracle.ray_vox_cast(m, _ref_inverse(R, obb), p, d)
        assert h == bool(h_ref), (mi, p, d)
        if h:
            hits += 1
            assert np.float32(t).view(np.int32) == t_ref.view(np.int32)[0], (mi, p, d, t, t_ref[0])
        nudged += int((d == 0).any())
    assert 0.2 * len(cases) < hits < len(cases) and nudged > 0


def test_ray_vox_cast_golden():
    """The oracle against outputs of the reference's RayVoxCast stored by
    tests/golden/make_golden.py (glm's inverse stored beside each case)."""
    z = np.load(os.path.join(G, "rayvox.npz"))
    models, off = [], 0
    for shp in z["model_shapes"]:
        n = int(np.prod(shp))
        models.append(z["models"][off:off + n].reshape(shp))
        off += n
    for i in range(len(z["model_of"])):
        h, t, _, _ = oracle.ray_vox_cast(models[z["model_of"][i]], z["inv"][i], z["pos"][i], z["dir"][i])
        assert h == bool(z["hit"][i]), i
        if h:
            assert np.float32(t).view(np.int32) == z["t"][i:i + 1].view(np.int32)[0], i
    assert 0 < z["hit"].sum() < len(z["hit"])


def test_ray_vox_cast_cross_checks_light_dda():
    rng = np.random.default_rng(5)
    eye = np.eye(4, dtype=np.float32).reshape(16)
    checked = hits = 0
    for m in _models(rng):
        sz, sy, sx = m.shape
        fine = m != 0
        g = oracle.fine_to_r8(fine)
        for _ in range(600):
            c = np.array([rng.integers(0, sx), rng.integers(0, sy), rng.integers(0, sz)])
            p = ((c + rng.uniform(0.02, 0.98, 3)) * 0.1).astype(np.float32)
            d = rng.normal(size=3)
            d = (d / np.linalg.norm(d)).astype(np.float32)
            h, t, cell, iters = oracle.ray_vox_cast(m, eye, p, d)
            o = p * np.float32(10.0)  # RayVoxCast's local position under an identity placement
            gg = g
            if fine[tuple(np.floor(o).astype(int)[::-1])]:
                # RayVoxCast never tests the origin cell: compare with it cleared
                f2 = fine.copy()
                f2[tuple(np.floor(o).astype(int)[::-1])] = False
                gg = oracle.fine_to_r8(f2)
            hl, rec = oracle.dda(gg, o, d, 1e30)
            assert bool(hl) == h, (p, d)
            checked += 1
            if h:
                hits += 1
                assert [rec["vx"], rec["vy"], rec["vz"]] == cell.tolist()
                assert rec["steps"] == iters + 1
                assert t * 10.0 < rec["t"] * (1.0 + 1e-6)
    assert checked == 3600 and 0.2 * checked < hits < checked
