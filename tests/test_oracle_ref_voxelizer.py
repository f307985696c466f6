"""The oracle's voxelizer against the reference's ShadowVoxSystem.cpp compiled
unmodified on the host (OnUpdate, SetVolumeAt, OnVoxDestroyed): identical
ShadowVox bytes and dirty regions, on the shipped FarmHouse models and on
random models with random rigid transforms. Skipped without the reference tree."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests import vox_cases
from tests.refbind import bind

u8 = C.POINTER(C.c_uint8)
fp = C.POINTER(C.c_float)


@pytest.fixture(scope="module")
def R(ref_lib, oracle_lib):
    return bind(ref_lib, oracle_lib)


def _ref_buffer(R):
    d = np.zeros(3, np.int32)
    R.ref_vox_dims(d.ctypes.data_as(C.POINTER(C.c_int)))
    sx, sy, sz = d
    p = R.ref_vox_buffer()
    return np.ctypeslib.as_array(C.cast(p, u8), shape=(sz * sy * sx,)).reshape(sz, sy, sx).copy()


def _f(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(fp)


def test_shadowvox_update_matches_reference(R):
    rng = np.random.default_rng(7)
    models = vox_cases.farmhouse_models(limit=10)
    models += [vox_cases.random_model(rng, *rng.integers(4, 40, 3)) for _ in range(6)]
    R.ref_vox_reset()
    for m in models:
        msz, msy, msx = m.shape
        R.ref_vox_add_model(np.ascontiguousarray(m).ctypes.data_as(u8), msx, msy, msz)
    ents = []
    for e in range(24):
        mi = int(rng.integers(0, len(models)))
        prev = vox_cases.world_matrix(rng, 0, 90, rotate=e % 3 != 0)
        cur = vox_cases.world_matrix(rng, -3, 95, rotate=e % 4 != 0)  # some placements poke outside the grid
        if e % 5 == 0:
            cur = prev.copy()
            cur[12] += 0.35  # small move: old and new poses overlap
        piv = rng.uniform(-2, 2, 3).astype(np.float32)
        ents.append((mi, prev, cur, piv))
        R.ref_vox_add_entity(mi, _f(prev), _f(cur), _f(piv))
    out = np.zeros((64, 6), np.int32)
    nreg = R.ref_vox_update(out.ctypes.data_as(C.POINTER(C.c_int)), 64)
    ref = _ref_buffer(R)
    g = np.zeros_like(ref)
    regions = oracle.shadowvox_update(g, [models[e[0]] for e in ents], np.stack([e[1] for e in ents]),
                                      np.stack([e[2] for e in ents]), np.stack([e[3] for e in ents]))
    assert np.array_equal(g, ref)
    assert g.any()
    # the reference uploads one region per entity whose aabbmax moved (:181-190),
    # after the constructor's full-volume region
    want = [list(r) for r in regions if r[0] >= 0]
    got = [list(r) for r in out[:nreg]]
    assert got[0] == [0, 0, 0, 524, 188, 524]
    assert got[1:] == want

    # a second frame: only some entities changed, poses move on
    for k, (mi, prev, cur, piv) in enumerate(ents):
        R.ref_vox_set_changed(k, 0)
    moved = []
    for k in range(0, len(ents), 2):
        mi, _, cur, piv = ents[k]
        nxt = vox_cases.world_matrix(rng, 0, 90)
        R.ref_vox_set_changed(k, 1)
        # shim entity matrices are updated through a fresh add (same model, prev = old cur)
        moved.append((mi, cur, nxt, piv))
    R2 = R  # same library; re-run from the current state with new entities
    for mi, prev, cur, piv in moved:
        R2.ref_vox_add_entity(mi, _f(prev), _f(cur), _f(piv))
    for k in range(0, len(ents), 2):
        R.ref_vox_set_changed(k, 0)
    nreg = R.ref_vox_update(out.ctypes.data_as(C.POINTER(C.c_int)), 64)
    ref2 = _ref_buffer(R)
    regions2 = oracle.shadowvox_update(g, [models[e[0]] for e in moved], np.stack([e[1] for e in moved]),
                                       np.stack([e[2] for e in moved]), np.stack([e[3] for e in moved]))
    assert np.array_equal(g, ref2)
    assert [list(r) for r in out[:nreg]] == [list(r) for r in regions2 if r[0] >= 0]

    # OnVoxDestroyed on the first moved entity (no -Pivot, :22-25)
    first_new = len(ents)
    mi, prev, cur, piv = moved[0]
    R.ref_vox_destroy(first_new)
    nreg = R.ref_vox_flush(out.ctypes.data_as(C.POINTER(C.c_int)), 64)
    ref3 = _ref_buffer(R)
    reg = oracle.vox_destroyed(g, models[mi], cur)
    assert np.array_equal(g, ref3)
    if reg[0] >= 0:
        assert list(out[0]) == list(reg)
