"""CPU oracle for the voxel-lighting path (TEST INFRASTRUCTURE ONLY).

This package is the parity checker for the CUDA path in ``voxelengine_gb300``.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
legs of ``bench.py`` import it; the product never does.

It wraps ``vxl_oracle.cpp`` (a restatement of the reference's shader and
voxelizer maths, each function citing the reference lines it follows), built
with ``g++ -O2 -ffp-contract=off`` into ``oracle/_build/``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libvxl_oracle.so")
_lock = threading.Lock()
_lib = None

REC_DTYPE = np.dtype(
    [("vx", "<i4"), ("vy", "<i4"), ("vz", "<i4"), ("t", "<f4"), ("steps", "<i4"), ("flags", "<i4")]
)
F_HIT, F_SELX, F_SELY, F_SELZ = 1, 2, 4, 8
F_EXIT_BOUNDS, F_EXIT_STEPS, F_EXIT_MAXT, F_COARSE = 16, 32, 64, 128
MODE_DDA, MODE_SPARSE, MODE_SUPERSPARSE = 0, 1, 2


class Params(C.Structure):
    """Same layout as ``vxl_trace_params`` (include/vxl.h)."""

    _fields_ = [
        ("light_dir", C.c_float * 3),
        ("cam_pos", C.c_float * 3),
        ("bias", C.c_float),
        ("shadow_len", C.c_float),
        ("ao_len", C.c_float),
        ("spec_len", C.c_float),
        ("default_rough", C.c_float),
        ("n_shadow", C.c_int32),
        ("n_ao", C.c_int32),
        ("n_spec", C.c_int32),
        ("seed", C.c_uint32),
        ("mode", C.c_int32),
    ]


class SoftParams(C.Structure):
    """Same layout as ``vxl_soft_params`` (include/vxl.h)."""

    _fields_ = [
        ("light_dir", C.c_float * 3),
        ("bias", C.c_float),
        ("len", C.c_float),
        ("k_sun", C.c_float),
        ("k_amb", C.c_float),
        ("n_shadow", C.c_int32),
        ("n_ao", C.c_int32),
        ("seed", C.c_uint32),
    ]


def build(force: bool = False, opt: str = "-O2") -> str:
    """Compile the oracle shared library into oracle/_build/ (idempotent)."""
    src = os.path.join(_HERE, "vxl_oracle.cpp")
    hdr = os.path.join(_HERE, "vxl_oracle.h")
    os.makedirs(_BUILD, exist_ok=True)
    if (
        not force
        and os.path.exists(_SO)
        and os.path.getmtime(_SO) >= max(os.path.getmtime(src), os.path.getmtime(hdr))
    ):
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    cmd = [
        "g++", opt, "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
        "-pthread", "-o", tmp, src,
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            fp = C.POINTER(C.c_float)
            u8p = C.POINTER(C.c_uint8)
            ip = C.POINTER(C.c_int)
            vp = C.c_void_p
            L.vo_sincos.argtypes = [C.c_float, fp, fp]
            L.vo_pcg.restype = C.c_uint32
            L.vo_pcg.argtypes = [C.c_uint32]
            L.vo_rand01.restype = C.c_float
            L.vo_rand01.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
            L.vo_get_volume_at.argtypes = [u8p] + [C.c_int] * 7
            L.vo_dda.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, vp]
            L.vo_dda_literal.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, fp, fp, ip]
            for fn in (L.vo_sparse, L.vo_supersparse):
                fn.restype = C.c_float
                fn.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, vp]
            L.vo_cosine_sample.argtypes = [C.c_float, C.c_float, fp]
            L.vo_trace_rays.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, C.c_int, C.c_int, vp, C.c_int]
            L.vo_occlusion.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, vp, C.c_int, C.POINTER(Params),
                                       vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]
            L.vo_light_ambient.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, C.c_int, fp, fp, vp,
                                           C.c_int]
            L.vo_light_reflection.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, fp, C.c_int, fp,
                                              vp, C.c_int]
            L.vo_light_point.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.c_int, fp, C.c_float,
                                         C.c_int, fp, vp, C.c_int]
            L.vo_scene_noise.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_float, C.c_float,
                                         C.c_int, C.c_int]
            L.vo_value_noise3.restype = C.c_float
            L.vo_value_noise3.argtypes = [C.c_float, C.c_float, C.c_float, C.c_uint32]
            L.vo_noise_octaves.restype = C.c_float
            L.vo_noise_octaves.argtypes = [C.c_float, C.c_float, C.c_float, C.c_uint32, C.c_float, C.c_int]
            L.vo_scene_terrain.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_float, C.c_float,
                                           C.c_float, C.c_int, vp, C.c_int]
            L.vo_scene_boxes.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int, C.c_int, C.c_int]
            L.vo_box_params.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, ip]
            L.vo_gbuffer.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, C.c_int, C.c_int,
                                     C.c_uint32, fp, fp, fp, C.c_int]
            L.vo_set_volume_at.argtypes = [u8p] + [C.c_int] * 7
            L.vo_voxelize_model.argtypes = [u8p, C.c_int, C.c_int, C.c_int, u8p, C.c_int, C.c_int, C.c_int, fp,
                                            C.c_int, ip]
            L.vo_translate.argtypes = [fp, fp, fp]
            L.vo_shadowvox_update.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(u8p), ip, fp,
                                              fp, fp, ip]
            L.vo_vox_destroyed.argtypes = [u8p, C.c_int, C.c_int, C.c_int, u8p, C.c_int, C.c_int, C.c_int, fp,
                                           ip]
            L.vo_fnv1a64.restype = C.c_uint64
            L.vo_fnv1a64.argtypes = [C.c_char_p]
            L.vo_volume_mips.argtypes = [u8p, C.c_int, C.c_int, C.c_int, u8p, u8p]
            L.vo_clip_intersect.argtypes = [u8p, u8p, u8p, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.c_float,
                                            C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, fp, fp,
                                            C.POINTER(C.c_uint32), ip]
            L.vo_affine_inverse.argtypes = [fp, fp, fp]
            L.vo_rebuild_from_depth.argtypes = [fp, fp, C.c_int, C.c_int, fp, fp, fp, fp]
            L.vo_ray_vox_cast.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp,
                                          C.POINTER(C.c_int), C.POINTER(C.c_int)]
            L.vo_ray_vox_cast.restype = C.c_int
            L.vo_primary.argtypes = [vp, vp, vp, ip, fp, ip, C.c_int, fp, fp, C.c_float, C.c_int, C.c_int, C.c_int,
                                     fp, fp, fp, ip, ip, C.c_int]
            L.vo_taa.argtypes = [fp, fp, fp, fp, fp, fp, fp, fp, C.c_int, C.c_int, fp, C.c_int]
            L.vo_soft_render.argtypes = [fp, C.c_int, C.c_int, C.c_int, fp, fp, C.c_int, C.POINTER(SoftParams),
                                         vp, C.c_int64, C.c_double, vp, vp, C.c_int]
            _lib = L
    return _lib


# ---------------------------------------------------------------- helpers
def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _vp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _grid(g):
    g = np.ascontiguousarray(g, dtype=np.uint8)
    sz, sy, sx = g.shape
    return g, sx, sy, sz


def threads_default() -> int:
    return max(1, os.cpu_count() or 1)


def sincos(x: float):
    s, c = C.c_float(), C.c_float()
    lib().vo_sincos(C.c_float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def rand01(seed, pixel, sample) -> float:
    return lib().vo_rand01(seed, pixel, sample)


def get_volume_at(g, x, y, z, mip=0) -> int:
    g, sx, sy, sz = _grid(g)
    return lib().vo_get_volume_at(_u8(g), sx, sy, sz, x, y, z, mip)


def dda(g, o, d, maxt):
    g, sx, sy, sz = _grid(g)
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    r = np.zeros(1, REC_DTYPE)
    h = lib().vo_dda(_u8(g), sx, sy, sz, _f(o), _f(d), C.c_float(maxt), _vp(r))
    return h, r[0]


def dda_literal(g, o, d, maxt):
    g, sx, sy, sz = _grid(g)
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    hit = np.zeros(3, np.float32)
    nrm = np.zeros(3, np.float32)
    nf = C.c_int(0)
    h = lib().vo_dda_literal(_u8(g), sx, sy, sz, _f(o), _f(d), C.c_float(maxt), _f(hit), _f(nrm), C.byref(nf))
    return h, hit, nrm, nf.value


def march(g, o, d, dist, super_sparse=False):
    g, sx, sy, sz = _grid(g)
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    r = np.zeros(1, REC_DTYPE)
    fn = lib().vo_supersparse if super_sparse else lib().vo_sparse
    t = fn(_u8(g), sx, sy, sz, _f(o), _f(d), C.c_float(dist), _vp(r))
    return t, r[0]


def cosine_sample(u1, u2):
    out = np.zeros(3, np.float32)
    lib().vo_cosine_sample(C.c_float(u1), C.c_float(u2), _f(out))
    return out


def trace_rays(g, rays, mode=MODE_DDA, threads=None):
    """rays: float32 [n,7] = origin(3), dir(3), maxt. Returns REC_DTYPE[n]."""
    g, sx, sy, sz = _grid(g)
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    recs = np.zeros(n, REC_DTYPE)
    lib().vo_trace_rays(_u8(g), sx, sy, sz, _f(rays), n, mode, _vp(recs), threads or threads_default())
    return recs


def make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=(0, 0, 0), bias=0.5, shadow_len=100.0, ao_len=16.0,
                spec_len=256.0, default_rough=0.5, n_shadow=1, n_ao=4, n_spec=0, seed=1, mode=MODE_DDA):
    p = Params()
    ld = np.asarray(light_dir, np.float64)
    ld = (ld / np.linalg.norm(ld)).astype(np.float32)
    p.light_dir[:] = [float(v) for v in ld]
    p.cam_pos[:] = [float(v) for v in np.asarray(cam_pos, np.float32)]
    p.bias, p.shadow_len, p.ao_len, p.spec_len, p.default_rough = bias, shadow_len, ao_len, spec_len, default_rough
    p.n_shadow, p.n_ao, p.n_spec, p.seed, p.mode = n_shadow, n_ao, n_spec, seed, mode
    return p


def occlusion(g, pos, nrm, rough, params: Params, with_recs=False, p0=0, p1=-1, threads=None):
    g, sx, sy, sz = _grid(g)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    npix = pos.shape[0]
    rough = None if rough is None else np.ascontiguousarray(rough, np.float32).reshape(-1)
    out = {k: np.zeros(npix, np.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    R = params.n_shadow + params.n_ao + params.n_spec
    recs = np.zeros(npix * R, REC_DTYPE) if with_recs else None
    lib().vo_occlusion(_u8(g), sx, sy, sz, _f(pos), _f(nrm), _vp(rough), npix, C.byref(params),
                       _vp(out["shadow"]), _vp(out["ao"]), _vp(out["ao_vis"]), _vp(out["spec"]),
                       _vp(out["spec_t"]), _vp(recs), p0, p1, threads or threads_default())
    if with_recs:
        out["recs"] = recs
    return out


def occlusion_range(g, pos, nrm, rough, params: Params, p0, p1, threads=None):
    """occlusion() for pixels [p0, p1) only, with records; outputs and records
    are returned for that range alone (the pixel index, which seeds the ray
    generator, stays the global one)."""
    g, sx, sy, sz = _grid(g)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    rough = None if rough is None else np.ascontiguousarray(rough, np.float32).reshape(-1)
    m = p1 - p0
    R = params.n_shadow + params.n_ao + params.n_spec
    out = {k: np.zeros(m, np.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    recs = np.zeros(m * R, REC_DTYPE)

    def shifted(a, per):  # address of element -p0*per, so that index p0 lands on a[0]
        return C.c_void_p(a.ctypes.data - p0 * per * a.itemsize)

    lib().vo_occlusion(_u8(g), sx, sy, sz, _f(pos), _f(nrm), _vp(rough), pos.shape[0], C.byref(params),
                       shifted(out["shadow"], 1), shifted(out["ao"], 1), shifted(out["ao_vis"], 1),
                       shifted(out["spec"], 1), shifted(out["spec_t"], 1), shifted(recs, R), p0, p1,
                       threads or threads_default())
    out["recs"] = recs
    return out


def light_ambient(g, wcp, nrm, depth, noise, threads=None):
    g, sx, sy, sz = _grid(g)
    wcp = np.ascontiguousarray(wcp, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    depth = np.ascontiguousarray(depth, np.float32).reshape(-1)
    noise = np.ascontiguousarray(noise, np.float32).reshape(-1, 4)
    n = wcp.shape[0]
    sh = np.zeros(n, np.float32)
    irr = np.zeros(n, np.float32)
    recs = np.zeros(2 * n, REC_DTYPE)
    lib().vo_light_ambient(_u8(g), sx, sy, sz, _f(wcp), _f(nrm), _f(depth), _f(noise), n, _f(sh), _f(irr),
                           _vp(recs), threads or threads_default())
    return sh, irr, recs


def light_reflection(g, wcp, nrm, view_r, rough, noise, threads=None):
    g, sx, sy, sz = _grid(g)
    wcp = np.ascontiguousarray(wcp, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    view_r = np.ascontiguousarray(view_r, np.float32).reshape(-1, 3)
    rough = np.ascontiguousarray(rough, np.float32).reshape(-1)
    noise = np.ascontiguousarray(noise, np.float32).reshape(-1, 4)
    n = wcp.shape[0]
    t = np.zeros(n, np.float32)
    recs = np.zeros(n, REC_DTYPE)
    lib().vo_light_reflection(_u8(g), sx, sy, sz, _f(wcp), _f(nrm), _f(view_r), _f(rough), _f(noise), n, _f(t),
                              _vp(recs), threads or threads_default())
    return t, recs


def light_point(g, wpos, nrm, noise, light_pos, light_range, spot=False, init=None, threads=None):
    g, sx, sy, sz = _grid(g)
    wpos = np.ascontiguousarray(wpos, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    noise = np.ascontiguousarray(noise, np.float32).reshape(-1, 4)
    n = wpos.shape[0]
    sh = np.full(n, -7.0, np.float32) if init is None else np.array(init, np.float32)
    recs = np.zeros(n, REC_DTYPE)
    lp = np.asarray(light_pos, np.float32)
    lib().vo_light_point(_u8(g), sx, sy, sz, _f(wpos), _f(nrm), _f(noise), n, _f(lp), C.c_float(light_range),
                         1 if spot else 0, _f(sh), _vp(recs), threads or threads_default())
    return sh, recs


def scene_noise(nx, ny, nz, seed, thresh=0.55, freq=1.0 / 32.0, ground_y=8, threads=None):
    """Seeded value-noise scene in the reference R8 2x2x2 layout: uint8[nz/2, ny/2, nx/2]."""
    sx, sy, sz = nx // 2, ny // 2, nz // 2
    g = np.zeros((sz, sy, sx), np.uint8)
    lib().vo_scene_noise(_u8(g), sx, sy, sz, seed, C.c_float(thresh), C.c_float(freq), ground_y,
                         threads or threads_default())
    return g


def scene_terrain(g, seed, base, amplitude, freq, octaves=5, threads=None):
    """OR the heightfield terrain into an R8 grid (uint8[nz/2, ny/2, nx/2]);
    returns the column heights float32[nz, nx]."""
    sz, sy, sx = g.shape
    assert g.flags.c_contiguous and g.dtype == np.uint8
    h = np.zeros((2 * sz, 2 * sx), np.float32)
    lib().vo_scene_terrain(_u8(g), sx, sy, sz, seed, C.c_float(base), C.c_float(amplitude), C.c_float(freq), octaves,
                           _vp(h), threads or threads_default())
    return h


def scene_boxes(g, seed, nboxes, smin=4, smax=48):
    sz, sy, sx = g.shape
    assert g.flags.c_contiguous and g.dtype == np.uint8
    lib().vo_scene_boxes(_u8(g), sx, sy, sz, seed, nboxes, smin, smax)
    return g


def box_params(seed, i, nx, ny, nz, smin=4, smax=48):
    out = np.zeros(6, np.int32)
    lib().vo_box_params(seed, i, nx, ny, nz, smin, smax, _i(out))
    return out


def gbuffer(g, cam, target, W, H, seed, tan_half_fov=0.57735026, threads=None):
    g, sx, sy, sz = _grid(g)
    cam = np.asarray(cam, np.float32)
    target = np.asarray(target, np.float32)
    pos = np.zeros((H * W, 3), np.float32)
    nrm = np.zeros((H * W, 3), np.float32)
    rough = np.zeros(H * W, np.float32)
    lib().vo_gbuffer(_u8(g), sx, sy, sz, _f(cam), _f(target), C.c_float(tan_half_fov), W, H, seed, _f(pos),
                     _f(nrm), _f(rough), threads or threads_default())
    return pos, nrm, rough


def translate(m, v):
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    v = np.asarray(v, np.float32)
    out = np.zeros(16, np.float32)
    lib().vo_translate(_f(m), _f(v), _f(out))
    return out


def voxelize_model(g, model, M, value, aabb=None):
    sz, sy, sx = g.shape
    model = np.ascontiguousarray(model, np.uint8)
    msz, msy, msx = model.shape
    M = np.ascontiguousarray(M, np.float32).reshape(16)
    if aabb is None:
        aabb = np.array([sx - 1, sy - 1, sz - 1, 0, 0, 0], np.int32)
    lib().vo_voxelize_model(_u8(g), sx, sy, sz, _u8(model), msx, msy, msz, _f(M), value, _i(aabb))
    return aabb


def shadowvox_update(g, models, prev, cur, pivot):
    """Entities in order; returns per-entity dirty regions int32[n,6]."""
    sz, sy, sx = g.shape
    n = len(models)
    ms = [np.ascontiguousarray(m, np.uint8) for m in models]
    ptrs = (C.POINTER(C.c_uint8) * max(n, 1))(*[_u8(m) for m in ms])
    dims = np.array([[m.shape[2], m.shape[1], m.shape[0]] for m in ms], np.int32).reshape(-1)
    prev = np.ascontiguousarray(prev, np.float32).reshape(-1)
    cur = np.ascontiguousarray(cur, np.float32).reshape(-1)
    pivot = np.ascontiguousarray(pivot, np.float32).reshape(-1)
    regions = np.zeros((n, 6), np.int32)
    lib().vo_shadowvox_update(_u8(g), sx, sy, sz, n, ptrs, _i(dims), _f(prev), _f(cur), _f(pivot), _i(regions))
    return regions


def vox_destroyed(g, model, world):
    sz, sy, sx = g.shape
    model = np.ascontiguousarray(model, np.uint8)
    msz, msy, msx = model.shape
    world = np.ascontiguousarray(world, np.float32).reshape(16)
    region = np.zeros(6, np.int32)
    lib().vo_vox_destroyed(_u8(g), sx, sy, sz, _u8(model), msx, msy, msz, _f(world), _i(region))
    return region


def fnv1a64(s: str) -> int:
    return lib().vo_fnv1a64(s.encode())


# ------------------------------------------------------ primary visibility
def mip_dims(s):
    """mip sizes of VoxAsset::Upload: p > 1 ? p / 2 : 1, per axis; s = (sx, sy, sz)"""
    d = [tuple(s)]
    for _ in range(2):
        d.append(tuple(v // 2 if v > 1 else 1 for v in d[-1]))
    return d


def volume_mips(vol):
    """vol uint8[sz, sy, sx] -> (mip1, mip2) as arrays [z, y, x] (VoxAsset::Upload)."""
    vol = np.ascontiguousarray(vol, np.uint8)
    sz, sy, sx = vol.shape
    d = mip_dims((sx, sy, sz))
    m1 = np.zeros(d[1][::-1], np.uint8)
    m2 = np.zeros(d[2][::-1], np.uint8)
    lib().vo_volume_mips(_u8(vol), sx, sy, sz, _u8(m1), _u8(m2))
    return m1, m2


def clip_intersect(mips, origin, direction, lcam, uv=(0.0, 0.0), res=(1.0, 1.0), frame=0, clip=True):
    """intersectVolume (after clipToAABB when clip) on a volume given as its 3 mips [z, y, x];
    returns (hit, hitpos[3], normal[3], material, fetches)."""
    m0, m1, m2 = (np.ascontiguousarray(m, np.uint8) for m in mips)
    sz, sy, sx = m0.shape
    h = np.zeros(3, np.float32)
    nrm = np.zeros(3, np.float32)
    mat = C.c_uint32()
    fe = C.c_int()
    o = np.asarray(origin, np.float32)
    d = np.asarray(direction, np.float32)
    lc = np.asarray(lcam, np.float32)
    r = lib().vo_clip_intersect(_u8(m0), _u8(m1), _u8(m2), sx, sy, sz, _f(o), _f(d), _f(lc), uv[0], uv[1], res[0],
                                res[1], frame, 1 if clip else 0, _f(h), _f(nrm), C.byref(mat), C.byref(fe))
    return r, h, nrm, mat.value, fe.value


def affine_inverse(m16):
    m = np.ascontiguousarray(m16, np.float32).reshape(16)
    ri = np.zeros(9, np.float32)
    ti = np.zeros(3, np.float32)
    lib().vo_affine_inverse(_f(m), _f(ri), _f(ti))
    return ri, ti


def rebuild_from_depth(depth, nrm, W, H, inv_view, inv_proj):
    """Fine-unit surface positions and sky-masked normals from a linear-depth
    G-buffer, as LightAmbient places a pixel (vo_rebuild_from_depth)."""
    depth = np.ascontiguousarray(depth, np.float32).reshape(-1)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    iv = np.ascontiguousarray(inv_view, np.float32).reshape(16)
    ip = np.ascontiguousarray(inv_proj, np.float32).reshape(16)
    assert depth.shape[0] == W * H and nrm.shape[0] == W * H
    wcp = np.zeros((W * H, 3), np.float32)
    n2 = np.zeros((W * H, 3), np.float32)
    lib().vo_rebuild_from_depth(_f(depth), _f(nrm), W, H, _f(iv), _f(ip), _f(wcp), _f(n2))
    return wcp, n2


def ray_vox_cast(model, inv_obb, ray_pos, ray_dir):
    """The engine's picking DDA (vo_ray_vox_cast) against one model, a
    uint8[sz, sy, sx] array. inv_obb: the inverse of the model's world matrix,
    float32[16] column-major. Returns (hit, t, cell[3], iterations)."""
    model = np.ascontiguousarray(model, np.uint8)
    msz, msy, msx = model.shape
    inv = np.ascontiguousarray(inv_obb, np.float32).reshape(16)
    p = np.ascontiguousarray(ray_pos, np.float32).reshape(3)
    d = np.ascontiguousarray(ray_dir, np.float32).reshape(3)
    t = np.zeros(1, np.float32)
    cell = np.zeros(3, np.int32)
    it = np.zeros(1, np.int32)
    ip = C.POINTER(C.c_int)
    hit = lib().vo_ray_vox_cast(model.ctypes.data_as(C.POINTER(C.c_uint8)), msx, msy, msz, _f(inv), _f(p), _f(d),
                                _f(t), cell.ctypes.data_as(ip), it.ctypes.data_as(ip))
    return bool(hit), float(t[0]), cell, int(it[0])


def primary(volumes, worlds, vol_of, cam, target, W, H, frame=0, tan_half_fov=0.57735026, threads=None):
    """Per-pixel primary visibility. volumes: list of uint8[sz, sy, sx] (mip 0);
    worlds: float32[n, 16] column-major; vol_of: int[n]. Camera in world units.
    Returns dict pos[npix,3] (fine units), nrm, depth, material, instance."""
    vols = [np.ascontiguousarray(v, np.uint8) for v in volumes]
    mips = [volume_mips(v) for v in vols]
    keep = vols + [m for mm in mips for m in mm]
    p0 = (C.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    p1 = (C.c_void_p * len(vols))(*[m[0].ctypes.data for m in mips])
    p2 = (C.c_void_p * len(vols))(*[m[1].ctypes.data for m in mips])
    dims = np.array([v.shape[::-1] for v in vols], np.int32).reshape(-1)
    worlds = np.ascontiguousarray(worlds, np.float32).reshape(-1, 16)
    vol_of = np.ascontiguousarray(vol_of, np.int32)
    n = W * H
    out = dict(pos=np.zeros((n, 3), np.float32), nrm=np.zeros((n, 3), np.float32), depth=np.zeros(n, np.float32),
               material=np.zeros(n, np.int32), instance=np.zeros(n, np.int32))
    c = np.asarray(cam, np.float32)
    t = np.asarray(target, np.float32)
    lib().vo_primary(C.cast(p0, C.c_void_p), C.cast(p1, C.c_void_p), C.cast(p2, C.c_void_p), _i(dims), _f(worlds),
                     _i(vol_of), worlds.shape[0], _f(c), _f(t), C.c_float(tan_half_fov), W, H, frame,
                     _f(out["pos"]), _f(out["nrm"]), _f(out["depth"]), _i(out["material"]), _i(out["instance"]),
                     threads or threads_default())
    del keep
    return out


def taa(light, last, color, normal, material, depth, motion, noise, threads=None):
    """LightTAA.frag main over [H, W, c] fp32 images; returns out [H, W, 4]."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (light, last, color, normal, material, depth, motion, noise)]
    H, W = arrs[0].shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    lib().vo_taa(*[_f(a) for a in arrs], W, H, _f(out), threads or threads_default())
    return out


def make_soft_params(light_dir=(0.3, 0.8, 0.5), bias=0.5, length=24.0, k_sun=0.7, k_amb=0.5, n_shadow=1,
                     n_ao=4, seed=7) -> SoftParams:
    p = SoftParams()
    p.light_dir[:] = list(light_dir)
    p.bias, p.len, p.k_sun, p.k_amb = bias, length, k_sun, k_amb
    p.n_shadow, p.n_ao, p.seed = n_shadow, n_ao, seed
    return p


def soft_render(vox, pos, nrm, params: SoftParams, grad_image=None, perturb_voxel=-1, perturb_delta=0.0,
                threads=None):
    """FP64 soft-opacity render of a float4 grid vox[nz,ny,nx,4] (opacity, albedo rgb).

    Returns image[npix,3] (float64), or (image, grad_vox[nz,ny,nx,4]) when
    grad_image (float32 [npix,3]) is given."""
    vox = np.ascontiguousarray(vox, np.float32)
    nz, ny, nx, _ = vox.shape
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    img = np.zeros((n, 3), np.float64)
    gv = None
    gi = None
    if grad_image is not None:
        gi = np.ascontiguousarray(grad_image, np.float32).reshape(n, 3)
        gv = np.zeros(vox.shape, np.float64)
    lib().vo_soft_render(_f(vox), nx, ny, nz, _f(pos), _f(nrm), n, C.byref(params), _vp(gi), int(perturb_voxel),
                         float(perturb_delta), _vp(img), _vp(gv), threads or threads_default())
    return img if gv is None else (img, gv)


# ------------------------------------------------- layout conversions (numpy)
def r8_to_fine(g):
    """Reference R8 2x2x2 bytes [sz,sy,sx] -> bool occupancy [2sz,2sy,2sx] (z,y,x)."""
    g = np.asarray(g, np.uint8)
    sz, sy, sx = g.shape
    out = np.zeros((2 * sz, 2 * sy, 2 * sx), bool)
    for bz in range(2):
        for by in range(2):
            for bx in range(2):
                bit = bx | (by << 1) | (bz << 2)
                out[bz::2, by::2, bx::2] = (g >> bit) & 1
    return out


def fine_to_r8(f):
    f = np.asarray(f, bool)
    nz, ny, nx = f.shape
    g = np.zeros((nz // 2, ny // 2, nx // 2), np.uint8)
    for bz in range(2):
        for by in range(2):
            for bx in range(2):
                bit = bx | (by << 1) | (bz << 2)
                g |= (f[bz::2, by::2, bx::2].astype(np.uint8) << bit)
    return g
