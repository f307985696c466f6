"""The oracle against golden vectors produced by the reference's own sources
(tests/golden/make_golden.py): traversal of Light.frag, the LightAmbient pass
and ShadowVoxSystem::OnUpdate. Runs without the reference tree."""
import os

import numpy as np

import oracle

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bits_equal(a, b):
    """Bit-for-bit equality where both are numbers; NaN where either is NaN must be
    NaN in both. The sign of the default NaN that arithmetic produces is the
    machine's (set on x86-64 SSE, clear on AArch64), and these fixtures were made
    on x86-64, so a NaN's bits are not compared."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.int32), b[~nb].view(np.int32))


def test_traversal_golden():
    d = np.load(os.path.join(G, "traversal_64.npz"))
    g, rays = d["grid"], d["rays"]
    recs = oracle.trace_rays(g, rays, oracle.MODE_DDA)
    hit = (recs["flags"] & 1).astype(np.int32)
    assert np.array_equal(hit, d["hit"])
    h = hit == 1
    # hit = origin + dir * best_t ; normal = -sign(dir) * select (Light.frag:61-62)
    hp = (rays[h, :3] + rays[h, 3:6] * recs["t"][h, None]).astype(np.float32)
    assert _bits_equal(hp, d["hitpos"][h])
    sel = np.stack([(recs["flags"] & 2) != 0, (recs["flags"] & 4) != 0, (recs["flags"] & 8) != 0], axis=1)
    assert np.array_equal((-np.sign(rays[:, 3:6]) * sel)[h], d["normal"][h])
    assert np.array_equal(recs["steps"][h], d["fetches"][h])
    miss_by_loop = ~h & ((recs["flags"] & (32 | 64)) != 0)
    assert np.array_equal(4 * recs["steps"][miss_by_loop], d["fetches"][miss_by_loop])  # four identical passes
    for mode, tk, fk in ((oracle.MODE_SPARSE, "t_sparse", "fetches_sparse"),
                         (oracle.MODE_SUPERSPARSE, "t_supersparse", "fetches_supersparse")):
        r = oracle.trace_rays(g, rays, mode)
        assert _bits_equal(r["t"], d[tk]) and np.array_equal(r["steps"], d[fk]), mode
    assert 0 < hit.sum() < len(hit)


def test_ambient_golden():
    d = np.load(os.path.join(G, "ambient_64.npz"))
    g = np.load(os.path.join(G, "traversal_64.npz"))["grid"]
    sh, irr, _ = oracle.light_ambient(g, d["wcp"], d["nrm"], d["depth"], d["noise"], threads=2)
    assert np.array_equal(sh, d["shadow"]) and _bits_equal(irr, d["irradiance"])


def test_shadowvox_update_golden():
    d = np.load(os.path.join(G, "shadowvox_update.npz"))
    sx, sy, sz = (int(v) for v in d["dims"])
    models, off = [], 0
    for shp in d["model_shapes"]:
        n = int(np.prod(shp))
        models.append(d["models"][off:off + n].reshape(shp))
        off += n
    g = np.zeros((sz, sy, sx), np.uint8)
    regions = oracle.shadowvox_update(g, [models[i] for i in d["ent_model"]], d["prev"], d["cur"], d["pivot"])
    flat = g.reshape(-1)
    nz = np.nonzero(flat)[0]
    assert np.array_equal(nz, d["nz_index"]) and np.array_equal(flat[nz], d["nz_value"])
    want = d["regions"]
    assert want[0].tolist() == [0, 0, 0, sx, sy, sz]  # the constructor's full-volume upload
    assert [list(r) for r in regions if r[0] >= 0] == [list(r) for r in want[1:]]
