"""Scene assets (host side): vxl_transform_matrix against the reference's own
TransformSystem::RealculateMatrix (compiled with its vendored glm), asset
GUIDs, the .p reader, and vxl_prefab_load on the shipped FarmHouse and
ModernHouse prefabs (the latter nests a rotated, scaled player_ik instance)
against an independent reading of PrefabAsset::Spawn."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from tests import prefab_walk, vox_cases

fp = C.POINTER(C.c_float)
from oracle.ref.build_ref import reference_dir

MODS = os.path.join(reference_dir(), "Assets", "Mods")


@pytest.fixture(scope="module")
def V():
    import voxelengine_gb300 as V

    V.build()
    return V


def _ref_transform(R):
    R.ref_transform.argtypes = [fp, fp, fp, fp, fp]

    def call(pos, rot, scale, parent=None):
        out = np.zeros(16, np.float32)
        p = [np.ascontiguousarray(a, np.float32) for a in (pos, rot, scale)]
        par = None if parent is None else np.ascontiguousarray(parent, np.float32).reshape(16)
        R.ref_transform(*[a.ctypes.data_as(fp) for a in p], None if par is None else par.ctypes.data_as(fp),
                        out.ctypes.data_as(fp))
        return out

    return call


def test_transform_matrix_matches_reference(V, ref_lib):
    ref = _ref_transform(ref_lib)
    rng = np.random.default_rng(3)
    for i in range(400):
        pos = rng.normal(size=3) * 30
        rot = rng.uniform(-np.pi, np.pi, 3) if i % 4 else np.zeros(3)
        scale = rng.uniform(0.2, 3.0, 3) if i % 3 else np.ones(3)
        parent = None if i % 2 else ref(rng.normal(size=3), rng.uniform(-3, 3, 3), rng.uniform(0.5, 2, 3))
        want = ref(pos, rot, scale, parent)
        got = V.transform_matrix(pos, rot, scale, parent)
        assert np.array_equal(got.view(np.int32), want.view(np.int32)), i


def test_asset_guid_is_fnv1a64(V):
    for s in ["", "default/FarmHouse/0.v", "default/player_ik.pf", "mod/ünïcode/path.v"]:
        assert V.asset_guid(s) == oracle.fnv1a64(s) == prefab_walk.fnv1a64(s)


def test_read_palette(V, tmp_path):
    raw = np.random.default_rng(1).integers(0, 256, 1792).astype(np.uint8)
    p = tmp_path / "x.p"
    p.write_bytes(raw.tobytes())
    assert np.array_equal(V.read_palette(str(p)).reshape(-1), raw)
    (tmp_path / "short.p").write_bytes(raw[:100].tobytes())
    with pytest.raises(V.VxlError):
        V.read_palette(str(tmp_path / "short.p"))


@pytest.mark.parametrize("prefab,n_expected", [("default/FarmHouse.pf", 67), ("default/ModernHouse.pf", 17)])
def test_prefab_load_matches_spawn(V, ref_lib, prefab, n_expected):
    if not os.path.isdir(MODS):
        pytest.skip("reference assets not present")
    ref = _ref_transform(ref_lib)
    want = prefab_walk.spawn(MODS, prefab, ref)
    got = V.load_prefab(MODS, prefab)
    assert len(got["renderers"]) == len(want) == n_expected
    for (gw, gp, gv, gpal, _), (ww, wp, wv, wpal, idx) in zip(got["renderers"], want):
        assert np.array_equal(gw.view(np.int32), ww.view(np.int32))
        assert np.array_equal(gp, wp)
        assert got["volume_guids"][gv] == wv and got["palette_guids"][gpal] == wpal
        assert np.array_equal(got["volumes"][gv], vox_cases.read_v(idx[wv]))
        assert np.array_equal(got["palettes"][gpal].reshape(-1),
                              np.frombuffer(open(idx[wpal], "rb").read(), np.uint8))
    if prefab.endswith("ModernHouse.pf"):
        rots = [w for w, *_ in want if abs(w[1]) > 1e-3]  # some world matrices carry a rotation
        assert rots


def test_prefab_errors(V, tmp_path):
    mods = tmp_path / "Mods"
    (mods / "m").mkdir(parents=True)
    with pytest.raises(V.VxlError):
        V.load_prefab(str(mods), "m/missing.pf")
    (mods / "m" / "bad.pf").write_text("[{\"Id\": 0, ")
    with pytest.raises(V.VxlError):
        V.load_prefab(str(mods), "m/bad.pf")
    (mods / "m" / "unresolved.pf").write_text(
        '[{"Id": 0, "Transform": {"Position": "0 0 0", "Rotation": "0 0 0", "Scale": "1 1 1"},'
        ' "VoxRenderer": {"Pallete": "1234", "Vox": "ABCD"}}]')
    with pytest.raises(V.VxlError):
        V.load_prefab(str(mods), "m/unresolved.pf")
    # a null Vox GUID draws nothing and is not an error
    (mods / "m" / "null.pf").write_text(
        '[{"Id": 0, "Transform": {"Position": "1 2 3", "Rotation": "0 0 0", "Scale": "1 1 1"},'
        ' "VoxRenderer": {"Pallete": "0", "Vox": "0"}}]')
    assert V.load_prefab(str(mods), "m/null.pf")["renderers"] == []
