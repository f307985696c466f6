"""Generate tests/golden/*.npz from the reference's own sources compiled on
this machine (oracle/ref/build_ref.py -> oracle/_ref/libvxl_ref.so).

Run: python tests/golden/make_golden.py   (needs the VoxelEngine tree at
$VXL_REFERENCE_DIR, or named `reference` beside this checkout);
`python tests/golden/make_golden.py
rayvox` writes only rayvox.npz. The fixtures let the oracle be checked
against the reference where the reference tree is absent.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle.ref import build_ref  # noqa: E402
from tests import cases, vox_cases  # noqa: E402
from tests.refbind import bind  # noqa: E402

fp = C.POINTER(C.c_float)
u8 = C.POINTER(C.c_uint8)


def f(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(fp)


def main():
    so = build_ref.build()
    if so is None:
        raise SystemExit("reference sources not found")
    R = bind(C.CDLL(so), oracle)
    # ---- traversal on a 64^3 noise grid
    g = cases.noise_grid(64, seed=3)
    sz, sy, sx = g.shape
    rays = np.concatenate([cases.edge_rays(64), cases.random_rays(64, 3000, seed=99)])
    n = len(rays)
    hit = np.zeros(n, np.int32)
    hitpos = np.zeros((n, 3), np.float32)
    normal = np.zeros((n, 3), np.float32)
    fetches = np.zeros(n, np.int64)
    t_sp = np.zeros(n, np.float32)
    f_sp = np.zeros(n, np.int64)
    t_ss = np.zeros(n, np.float32)
    f_ss = np.zeros(n, np.int64)
    lt = np.zeros(3, np.int32)
    for i, q in enumerate(rays):
        h = np.zeros(3, np.float32)
        nr = np.zeros(3, np.float32)
        fc = C.c_longlong()
        hit[i] = R.ref_raycast(g.ctypes.data_as(u8), sx, sy, sz, f(q[:3]), f(q[3:6]), C.c_float(q[6]),
                               h.ctypes.data_as(fp), nr.ctypes.data_as(fp), C.byref(fc),
                               lt.ctypes.data_as(C.POINTER(C.c_int)))
        hitpos[i], normal[i], fetches[i] = h, nr, fc.value
        t_sp[i] = R.ref_march(g.ctypes.data_as(u8), sx, sy, sz, f(q[:3]), f(q[3:6]), C.c_float(q[6]), 0,
                              C.byref(fc), lt.ctypes.data_as(C.POINTER(C.c_int)))
        f_sp[i] = fc.value
        t_ss[i] = R.ref_march(g.ctypes.data_as(u8), sx, sy, sz, f(q[:3]), f(q[3:6]), C.c_float(q[6]), 1,
                              C.byref(fc), lt.ctypes.data_as(C.POINTER(C.c_int)))
        f_ss[i] = fc.value
    np.savez_compressed(os.path.join(HERE, "traversal_64.npz"), grid=g, rays=rays, hit=hit, hitpos=hitpos,
                        normal=normal, fetches=fetches, t_sparse=t_sp, fetches_sparse=f_sp, t_supersparse=t_ss,
                        fetches_supersparse=f_ss)

    # ---- ambient pass per pixel (own sin/cos variant)
    rng = np.random.default_rng(4)
    m = 600
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    pos = rng.uniform(-2, 2, (m, 3)).astype(np.float32)
    nrm = axes[rng.integers(0, 6, m)]
    depth = rng.uniform(0, 0.3, m).astype(np.float32)
    noise = rng.random((m, 4)).astype(np.float32)
    iv = np.eye(4, dtype=np.float32)
    iv[:3, 3] = [3.1, 3.3, 2.9]
    ivc = np.ascontiguousarray(iv.T)
    wcp = np.zeros((m, 3), np.float32)
    sh = np.zeros(m, np.float32)
    irr = np.zeros(m, np.float32)
    for i in range(m):
        w = np.zeros(3, np.float32)
        s = np.zeros(1, np.float32)
        ir = np.zeros(1, np.float32)
        R.ref_ambient(g.ctypes.data_as(u8), sx, sy, sz, f(pos[i]), f(ivc), f(nrm[i]), C.c_float(depth[i]),
                      f(noise[i]), 1, w.ctypes.data_as(fp), s.ctypes.data_as(fp), ir.ctypes.data_as(fp))
        wcp[i], sh[i], irr[i] = w, s[0], ir[0]
    np.savez_compressed(os.path.join(HERE, "ambient_64.npz"), wcp=wcp, nrm=nrm, depth=depth, noise=noise,
                        shadow=sh, irradiance=irr)

    # ---- voxelizer: FarmHouse models (if shipped) + random models, one OnUpdate
    models = vox_cases.farmhouse_models(build_ref.reference_dir(), limit=4)
    models += [vox_cases.random_model(rng, *rng.integers(4, 24, 3)) for _ in range(3)]
    R.ref_vox_reset()
    for mdl in models:
        msz, msy, msx = mdl.shape
        R.ref_vox_add_model(np.ascontiguousarray(mdl).ctypes.data_as(u8), msx, msy, msz)
    ents = []
    for e in range(10):
        mi = int(rng.integers(0, len(models)))
        prev = vox_cases.world_matrix(rng, 0, 60)
        cur = vox_cases.world_matrix(rng, -2, 62)
        piv = rng.uniform(-2, 2, 3).astype(np.float32)
        ents.append((mi, prev, cur, piv))
        R.ref_vox_add_entity(mi, f(prev), f(cur), f(piv))
    out = np.zeros((32, 6), np.int32)
    nreg = R.ref_vox_update(out.ctypes.data_as(C.POINTER(C.c_int)), 32)
    d = np.zeros(3, np.int32)
    R.ref_vox_dims(d.ctypes.data_as(C.POINTER(C.c_int)))
    buf = np.ctypeslib.as_array(C.cast(R.ref_vox_buffer(), u8), shape=(int(d[2] * d[1] * d[0]),)).copy()
    nz = np.nonzero(buf)[0].astype(np.int64)
    mflat = np.concatenate([mm.reshape(-1) for mm in models])
    mshapes = np.array([mm.shape for mm in models], np.int32)
    np.savez_compressed(os.path.join(HERE, "shadowvox_update.npz"), dims=d, models=mflat, model_shapes=mshapes,
                        ent_model=np.array([e[0] for e in ents], np.int32), prev=np.stack([e[1] for e in ents]),
                        cur=np.stack([e[2] for e in ents]), pivot=np.stack([e[3] for e in ents]),
                        regions=out[:nreg], nz_index=nz, nz_value=buf[nz])
    # ---- the shipped FarmHouse prefab as world-space placements (PrefabAsset::Spawn
    # + TransformSystem::RealculateMatrix of the reference, then World * translate(-Pivot))
    mods = os.path.join(build_ref.reference_dir(), "Assets", "Mods")
    if os.path.isdir(mods):
        from tests import prefab_walk

        R.ref_transform.argtypes = [fp, fp, fp, fp, fp]

        def realculate(pos, rot, scale, parent=None):
            o = np.zeros(16, np.float32)
            par = None if parent is None else np.ascontiguousarray(parent, np.float32)
            R.ref_transform(f(pos), f(rot), f(scale), None if par is None else f(par), o.ctypes.data_as(fp))
            return o

        rens = prefab_walk.spawn(mods, "default/FarmHouse.pf", realculate)
        guids = []
        for _, _, vg, _, _ in rens:
            if vg not in guids:
                guids.append(vg)
        idx = rens[0][4]
        vols = [vox_cases.read_v(idx[g]) for g in guids]
        worlds = np.stack([r[0] for r in rens])
        pivots = np.stack([r[1] for r in rens])
        mats = np.stack([oracle.translate(w, -p) for w, p in zip(worlds, pivots)])
        pal = np.frombuffer(open(idx[rens[0][3]], "rb").read(), np.uint8)
        np.savez_compressed(os.path.join(HERE, "farmhouse_scene.npz"),
                            volumes=np.concatenate([v.reshape(-1) for v in vols]),
                            volume_shapes=np.array([v.shape for v in vols], np.int32),
                            vol_of=np.array([guids.index(r[2]) for r in rens], np.int32), world=worlds,
                            pivot=pivots, matrix=mats, palette=pal)
    make_rayvox(R)
    print("golden fixtures written to", HERE)


def make_rayvox(R):
    """RayVoxCast (PhysicsSystem.cpp:98-145) on seeded models, placements and
    picking rays, with glm's inverse of each placement beside it."""
    rng = np.random.default_rng(31)
    models = [vox_cases.random_model(rng, *rng.integers(2, 9, 3) * 4, fill=f) for f in (0.3, 0.08, 0.5, 0.02)]
    cases = vox_cases.rayvox_cases(rng, [m.shape for m in models], n_per_model=150)
    n = len(cases)
    inv = np.zeros((n, 16), np.float32)
    hit = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    for i, (mi, obb, p, d) in enumerate(cases):
        m = np.ascontiguousarray(models[mi])
        sz, sy, sx = m.shape
        R.ref_glm_inverse(f(obb), inv[i].ctypes.data_as(fp))
        tt = np.zeros(1, np.float32)
        hit[i] = R.ref_ray_vox_cast(f(obb), m.ctypes.data_as(u8), sx, sy, sz, f(p), f(d), tt.ctypes.data_as(fp))
        t[i] = tt[0]
    np.savez_compressed(os.path.join(HERE, "rayvox.npz"), models=np.concatenate([m.reshape(-1) for m in models]),
                        model_shapes=np.array([m.shape for m in models], np.int32),
                        model_of=np.array([c[0] for c in cases], np.int32), obb=np.stack([c[1] for c in cases]),
                        pos=np.stack([c[2] for c in cases]), dir=np.stack([c[3] for c in cases]), inv=inv, hit=hit,
                        t=t)


if __name__ == "__main__":
    if sys.argv[1:] == ["rayvox"]:
        make_rayvox(bind(C.CDLL(build_ref.build()), oracle))
    else:
        main()
