"""Known answers worked out by hand from the reference's shader text (no
reference build, no fixture): the oracle's traversal against expected cells,
fetch counts and t values derived on paper. All inputs are exact binary
fractions, so every face-crossing time is exact.

* raycastShadowVolume (Light.frag:29-81): a diagonal path, a three-axis tie
  (t is the sum of the tied t_max components, dot(t_max, select)), and the
  inclusive +1 over-bound exit.
* raycastShadowVolumeSparse (Light.frag:131-173): the fine bit is chosen by
  mod(pos, 0.5) > 0.25, not by the cell the sample lies in.
* getVolumeAt (Light.frag:14-27): integer division truncates toward zero.
* ShadowVoxSystem::OnUpdate / SetVolumeAt (ShadowVoxSystem.cpp:82-94,
  :145-149): the index >= 16 test, the truncating conversion that folds
  (-1, 0) into cell 0, and the 2*Size bound."""
import numpy as np

import oracle


def _grid(n, cells):
    f = np.zeros((n, n, n), bool)
    for x, y, z in cells:
        f[z, y, x] = True
    return oracle.fine_to_r8(f)


def test_dda_diagonal_path():
    # d = (1, 0.5, 0.25) from (0.5, 2.5, 3.5): x faces at t = 0.5 + k, y at 1 + 2k, z at 2 + 4k.
    # Cells tested: (0,2,3) (1,2,3) (1,3,3) (2,3,3) (2,3,4) (3,3,4) (3,4,4).
    g = _grid(16, [(3, 4, 4)])
    h, r = oracle.dda(g, (0.5, 2.5, 3.5), (1.0, 0.5, 0.25), 100.0)
    assert h == 1
    assert (r["vx"], r["vy"], r["vz"]) == (3, 4, 4)
    assert r["steps"] == 7
    # at the hit t_max = (3.5, 5, 6): x is selected, best_t = 3.5
    assert r["t"] == 3.5 and r["flags"] & 2 and not r["flags"] & (4 | 8)
    # one cell earlier on the path: (3,3,4) at fetch 6, t_max (3.5, 3, 6) selects y
    h, r = oracle.dda(_grid(16, [(3, 3, 4)]), (0.5, 2.5, 3.5), (1.0, 0.5, 0.25), 100.0)
    assert h == 1 and r["steps"] == 6 and r["t"] == 3.0 and r["flags"] & 4


def test_dda_three_axis_tie_sums_t():
    # d = (1,1,1) from (0.5,0.5,0.5): every iteration steps all three axes;
    # dot(t_max, select) adds the three equal components.
    g = _grid(16, [(2, 2, 2)])
    h, r = oracle.dda(g, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 100.0)
    assert h == 1 and (r["vx"], r["vy"], r["vz"]) == (2, 2, 2) and r["steps"] == 3
    assert r["t"] == 7.5  # 3 x 2.5
    assert r["flags"] & (2 | 4 | 8) == (2 | 4 | 8)
    # maxt compares that sum: with maxt = 4.5 the loop ends after (1,1,1) (totalt 4.5)
    h, r = oracle.dda(g, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 4.5)
    assert h == 0 and r["steps"] == 2 and r["t"] == 4.5 and r["flags"] & 64


def test_dda_leaves_through_the_plus_one_bound():
    # 8^3 fine grid = 4^3 bytes: the bound is dims/mipSize*2 + 1 = 9, inclusive, so
    # cells 8 and 9 are tested (read empty) and cell 10 exits.
    # d = (1, 0.125, 0.0625) from (6.5, 0.5, 0.5): x faces at 0.5 + k, y at 4, z at 8.
    g = _grid(8, [])
    h, r = oracle.dda(g, (6.5, 0.5, 0.5), (1.0, 0.125, 0.0625), 100.0)
    assert h == 0 and r["flags"] & 16
    assert (r["vx"], r["vy"], r["vz"]) == (10, 0, 0) and r["steps"] == 4 and r["t"] == 3.5


def test_sparse_marcher_bit_quirk():
    # only fine voxel (1,0,0): byte (0,0,0), bit 1 (x)
    g = _grid(8, [(1, 0, 0)])
    # first sample at the origin (d = 0.5): pos.x = 0.3 lies in cell 0, but
    # mod(0.3, 0.5) = 0.3 > 0.25 selects the x bit, i.e. cell 1: a hit
    t, r = oracle.march(g, (0.3, 0.1, 0.1), (0.0, 0.0, 1.0), 128.0)
    assert t == 0.5 and r["flags"] & 1 and r["steps"] == 1 and (r["vx"], r["vy"], r["vz"]) == (1, 0, 0)
    # with only cell (0,0,0) set the same ray never reads bit 0: 31 fine samples
    # (d = 0.5 .. 15.5), then 112 coarse ones (d = 16 .. 127), and dist comes back
    t, r = oracle.march(_grid(8, [(0, 0, 0)]), (0.3, 0.1, 0.1), (0.0, 0.0, 1.0), 128.0)
    assert t == 128.0 and not r["flags"] & 1 and r["steps"] == 31 + 112


def test_get_volume_at_truncates_toward_zero():
    # byte (0,0,0) holds fine cell (1,0,0) in bit 1; pos/2 truncates, so cell
    # -1 reads byte 0 and its bit (-1 & 1) = 1, i.e. cell (1,0,0)
    g = _grid(8, [(1, 0, 0)])
    assert oracle.get_volume_at(g, 1, 0, 0, 0) == 1
    assert oracle.get_volume_at(g, -1, 0, 0, 0) == 1
    assert oracle.get_volume_at(g, 0, 0, 0, 0) == 0
    # odd mip: any voxel of the 2^3 block
    assert oracle.get_volume_at(g, 0, 1, 1, 1) == 1


def _translation(tx, ty, tz):
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (tx, ty, tz)
    return np.ascontiguousarray(m.T).reshape(16)  # column-major


def test_voxelizer_known_answers():
    """ShadowVoxSystem::OnUpdate's mapping (ShadowVoxSystem.cpp:145-149):
    voxel (x,y,z) of index >= 16 goes to ivec3((o + x*dx + y*dy + z*dz) * 10),
    dx = M[0] * 0.1 (fp32, truncating conversion), then SetVolumeAt
    (:82-94: 0 <= x < 2*SizeX, bit (x&1)|(y&1)<<1|(z&1)<<2 of byte (x/2, y/2, z/2))."""
    model = np.zeros((4, 4, 4), np.uint8)  # [z][y][x]
    model[3, 2, 1] = 20   # -> fine (1,2,3): 0.1f*3*10 rounds to exactly 3
    model[0, 0, 0] = 5    # index < 16 (glass): not a shadow caster
    g = np.zeros((4, 4, 4), np.uint8)  # 8^3 fine voxels
    oracle.voxelize_model(g, model, _translation(0, 0, 0), 1)
    want = np.zeros_like(g)
    want[1, 1, 0] = 1 << 5  # byte (0,1,1), bit 1 | 0 | 4
    assert np.array_equal(g, want)

    # truncation toward zero folds (-1, 0) into cell 0: x = 0 maps to (int)(-0.5) = 0
    # and x = 1 to (int)(0.5) = 0, so both source voxels land in one cell
    m2 = np.zeros((4, 4, 4), np.uint8)
    m2[0, 0, 0] = 20
    m2[0, 0, 1] = 20
    g = np.zeros((4, 4, 4), np.uint8)
    oracle.voxelize_model(g, m2, _translation(-0.05, 0, 0), 1)
    want = np.zeros_like(g)
    want[0, 0, 0] = 1
    assert np.array_equal(g, want)

    # SetVolumeAt's bound: x = 7 is set, x = 8 (= 2 * SizeX) is dropped
    m3 = np.zeros((4, 4, 4), np.uint8)
    m3[0, 0, 0] = 20
    g = np.zeros((4, 4, 4), np.uint8)
    oracle.voxelize_model(g, m3, _translation(0.7, 0, 0), 1)
    want = np.zeros_like(g)
    want[0, 0, 3] = 1 << 1
    assert np.array_equal(g, want)
    g = np.zeros((4, 4, 4), np.uint8)
    oracle.voxelize_model(g, m3, _translation(0.8, 0, 0), 1)
    assert not g.any()
