"""ctypes signatures of oracle/_ref/libvxl_ref.so (the reference's own sources
compiled on the host by oracle/ref/build_ref.py). Test infrastructure."""
import ctypes as C

import numpy as np

fp = C.POINTER(C.c_float)
u8 = C.POINTER(C.c_uint8)
ip = C.POINTER(C.c_int)


def bind(R, oracle_lib):
    R.ref_get_volume_at.argtypes = [u8] + [C.c_int] * 7
    R.ref_raycast.argtypes = [u8, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, fp, fp, C.POINTER(C.c_longlong), ip]
    R.ref_march.restype = C.c_float
    R.ref_march.argtypes = [u8, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, C.c_int, C.POINTER(C.c_longlong), ip]
    R.ref_cosine_sample.argtypes = [C.c_float, C.c_float, C.c_int, fp]
    R.ref_sun_dir.argtypes = [fp]
    R.ref_ambient.argtypes = [u8, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.c_float, fp, C.c_int, fp, fp, fp]
    R.ref_reflection.restype = C.c_float
    R.ref_reflection.argtypes = [u8, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, C.c_float, fp, fp, fp]
    R.ref_point.restype = C.c_float
    R.ref_point.argtypes = [u8, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.c_float, fp, C.c_int, ip]
    R.ref_vox_reset.argtypes = []
    R.ref_vox_dims.argtypes = [ip]
    R.ref_vox_buffer.restype = C.c_void_p
    R.ref_vox_add_model.argtypes = [u8, C.c_int, C.c_int, C.c_int]
    R.ref_vox_add_entity.argtypes = [C.c_int, fp, fp, fp]
    R.ref_vox_set_changed.argtypes = [C.c_int, C.c_int]
    R.ref_vox_update.argtypes = [ip, C.c_int]
    R.ref_vox_destroy.argtypes = [C.c_int]
    R.ref_vox_flush.argtypes = [ip, C.c_int]
    R.ref_ray_vox_cast.restype = C.c_int
    R.ref_ray_vox_cast.argtypes = [fp, u8, C.c_int, C.c_int, C.c_int, fp, fp, fp]
    R.ref_glm_inverse.argtypes = [fp, fp]
    R.ref_set_sincos.argtypes = [C.c_void_p]
    R.ref_set_sincos(C.cast(oracle_lib.lib().vo_sincos, C.c_void_p))
    return R


def F(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(fp)


def raycast(R, g, o, d, maxt):
    sz, sy, sx = g.shape
    h = np.zeros(3, np.float32)
    n = np.zeros(3, np.float32)
    f = C.c_longlong()
    lt = np.zeros(3, np.int32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    r = R.ref_raycast(g.ctypes.data_as(u8), sx, sy, sz, o.ctypes.data_as(fp), d.ctypes.data_as(fp), C.c_float(maxt),
                      h.ctypes.data_as(fp), n.ctypes.data_as(fp), C.byref(f), lt.ctypes.data_as(ip))
    return r, h, n, f.value


def march(R, g, o, d, dist, super_sparse):
    sz, sy, sx = g.shape
    f = C.c_longlong()
    lt = np.zeros(3, np.int32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    t = R.ref_march(g.ctypes.data_as(u8), sx, sy, sz, o.ctypes.data_as(fp), d.ctypes.data_as(fp), C.c_float(dist),
                    1 if super_sparse else 0, C.byref(f), lt.ctypes.data_as(ip))
    return t, f.value
