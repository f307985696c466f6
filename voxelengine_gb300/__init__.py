"""voxelengine_gb300 — Python binding of libvxl, the GB300 voxel-lighting path.

libvxl (include/vxl.h) is a C-ABI library of hand-written sm_103a CUDA kernels:
the ShadowVox voxelizer and the voxel ray traversal behind shadows, ambient
occlusion and specular occlusion of VoxelEngine (Sources/Shaders/lib/Light.frag,
Sources/World/Systems/ShadowVoxSystem.cpp). This module loads it with ctypes
and mirrors its entry points; device buffers are torch CUDA tensors (used only
as device memory and streams). There is no CPU fallback: every call raises if
the library cannot be loaded or returns an error.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvxl.so")

VXL_OK = 0
VXL_ERR_INVALID_ARG, VXL_ERR_OOM, VXL_ERR_CUDA, VXL_ERR_TIMEOUT = 1, 2, 3, 4
VXL_ERR_OUT_OF_RANGE, VXL_ERR_IO, VXL_ERR_NOT_SUPPORTED = 5, 6, 7
MODE_DDA, MODE_SPARSE, MODE_SUPERSPARSE = 0, 1, 2
OP_CLEAR, OP_SET = 0, 1
RF_HIT, RF_SELX, RF_SELY, RF_SELZ = 1, 2, 4, 8
RF_EXIT_BOUNDS, RF_EXIT_STEPS, RF_EXIT_MAXT, RF_COARSE = 16, 32, 64, 128
REC_DTYPE = np.dtype(
    [("vx", "<i4"), ("vy", "<i4"), ("vz", "<i4"), ("t", "<f4"), ("steps", "<i4"), ("flags", "<i4")]
)
REC_BYTES = 24

# every symbol include/vxl.h declares
EXPORTED = [
    "vxl_abi_version", "vxl_last_error_string", "vxl_status_string", "vxl_ctx_create", "vxl_ctx_destroy",
    "vxl_ctx_launch_count", "vxl_ctx_set_tuning", "vxl_ctx_get_tuning", "vxl_grid_create", "vxl_grid_destroy", "vxl_grid_describe", "vxl_grid_clear",
    "vxl_grid_build_bricks", "vxl_grid_import_r8", "vxl_grid_export_r8", "vxl_grid_import_palette",
    "vxl_grid_palette_alloc", "vxl_grid_export_palette", "vxl_scene_palette",
    "vxl_grid_count", "vxl_trace_rays", "vxl_trace_occlusion", "vxl_trace_occlusion_host",
    "vxl_trace_occlusion_from_depth", "vxl_batch_create",
    "vxl_batch_run", "vxl_batch_destroy", "vxl_batch_info", "vxl_light_ambient",
    "vxl_light_reflection", "vxl_light_point", "vxl_light_points", "vxl_light_taa", "vxl_voxelize", "vxl_voxelize_noalloc", "vxl_shadowvox_update",
    "vxl_vox_destroyed",
    "vxl_trace_soft_fwd", "vxl_trace_soft_bwd", "vxl_volume_build_mips", "vxl_trace_primary",
    "vxl_asset_guid", "vxl_read_palette", "vxl_transform_matrix", "vxl_prefab_load", "vxl_prefab_info",
    "vxl_prefab_renderer_at", "vxl_prefab_volume_at", "vxl_prefab_palette_at", "vxl_prefab_destroy",
    "vxl_vox_load", "vxl_vox_info", "vxl_vox_model_at", "vxl_vox_palette", "vxl_vox_destroy",
    "vxl_read_v", "vxl_scene_soft", "vxl_scene_terrain", "vxl_scene_noise", "vxl_scene_boxes", "vxl_scene_gbuffer",
    "vxl_diag_l2_read_gbs",
]


class VxlError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("vxl status %d: %s" % (status, msg))
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("bx", C.c_int32), ("by", C.c_int32),
                ("bz", C.c_int32), ("tx", C.c_int32), ("ty", C.c_int32), ("tz", C.c_int32), ("words", C.c_void_p),
                ("words_bytes", C.c_size_t), ("tile_mask", C.c_void_p), ("tile_mask_bytes", C.c_size_t),
                ("trace_words", C.c_void_p), ("trace_words_bytes", C.c_size_t), ("trace_lbx", C.c_int32),
                ("trace_lby", C.c_int32), ("trace_bz", C.c_int32), ("trace_wide", C.c_int32)]


class GBuffer(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("nrm", C.c_void_p), ("rough", C.c_void_p), ("npix", C.c_int64),
                ("width", C.c_int32), ("height", C.c_int32)]


class TraceParams(C.Structure):
    _fields_ = [("light_dir", C.c_float * 3), ("cam_pos", C.c_float * 3), ("bias", C.c_float),
                ("shadow_len", C.c_float), ("ao_len", C.c_float), ("spec_len", C.c_float),
                ("default_rough", C.c_float), ("n_shadow", C.c_int32), ("n_ao", C.c_int32), ("n_spec", C.c_int32),
                ("seed", C.c_uint32), ("mode", C.c_int32)]


class Outputs(C.Structure):
    _fields_ = [("shadow", C.c_void_p), ("ao", C.c_void_p), ("ao_vis", C.c_void_p), ("spec", C.c_void_p),
                ("spec_t", C.c_void_p), ("records", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("tile_px", C.c_int32), ("kstep", C.c_int32), ("leap", C.c_int32), ("order", C.c_int32),
                ("tile_w", C.c_int32), ("grab", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchItem(C.Structure):
    _fields_ = [("grid", C.c_void_p), ("gbuf", GBuffer), ("params", TraceParams), ("out", Outputs)]


class SoftParams(C.Structure):
    _fields_ = [("light_dir", C.c_float * 3), ("bias", C.c_float), ("len", C.c_float), ("k_sun", C.c_float),
                ("k_amb", C.c_float), ("n_shadow", C.c_int32), ("n_ao", C.c_int32), ("seed", C.c_uint32)]


class Volume(C.Structure):
    _fields_ = [("mip", C.c_void_p * 3), ("sx", C.c_int32), ("sy", C.c_int32), ("sz", C.c_int32),
                ("pad", C.c_int32)]


class VoxCmd(C.Structure):
    _fields_ = [("world", C.c_float * 16), ("volume", C.c_int32), ("palette", C.c_int32)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("target", C.c_float * 3), ("tan_half_fov", C.c_float), ("width", C.c_int32),
                ("height", C.c_int32), ("frame", C.c_int32)]


class PrimaryOut(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("nrm", C.c_void_p), ("depth", C.c_void_p), ("material", C.c_void_p),
                ("instance", C.c_void_p)]


class TaaFrame(C.Structure):
    _fields_ = [("light", C.c_void_p), ("last_light", C.c_void_p), ("color", C.c_void_p), ("normal", C.c_void_p),
                ("material", C.c_void_p), ("depth", C.c_void_p), ("motion", C.c_void_p), ("noise", C.c_void_p),
                ("width", C.c_int32), ("height", C.c_int32)]


class View(C.Structure):
    _fields_ = [("inverse_view", C.c_float * 16), ("inverse_projection", C.c_float * 16)]


class Light(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("range", C.c_float), ("spot", C.c_int32), ("pad", C.c_int32 * 3)]


class PrefabRenderer(C.Structure):
    _fields_ = [("world", C.c_float * 16), ("pivot", C.c_float * 3), ("volume", C.c_int32), ("palette", C.c_int32),
                ("entity", C.c_int32)]


class Model(C.Structure):
    _fields_ = [("data", C.c_void_p), ("sx", C.c_int32), ("sy", C.c_int32), ("sz", C.c_int32)]


class Instance(C.Structure):
    _fields_ = [("matrix", C.c_float * 16), ("model", C.c_int32), ("op", C.c_int32)]


class Entity(C.Structure):
    _fields_ = [("prev_world", C.c_float * 16), ("world", C.c_float * 16), ("pivot", C.c_float * 3),
                ("model", C.c_int32)]


_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    from . import buildlib as _b

    return _b.build(force=force)


def lib():
    """Load libvxl.so (raises if it is missing: there is no fallback path)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError("libvxl.so not built: run voxelengine_gb300.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp, i64, f = C.c_void_p, C.c_int64, C.c_float
        L.vxl_abi_version.restype = C.c_int
        L.vxl_last_error_string.restype = C.c_char_p
        L.vxl_status_string.restype = C.c_char_p
        L.vxl_status_string.argtypes = [C.c_int]
        L.vxl_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.vxl_ctx_destroy.argtypes = [vp]
        L.vxl_ctx_launch_count.argtypes = [vp, C.POINTER(C.c_uint64)]
        L.vxl_ctx_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.vxl_ctx_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.vxl_grid_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]
        L.vxl_grid_destroy.argtypes = [vp]
        L.vxl_grid_describe.argtypes = [vp, C.POINTER(GridDesc)]
        L.vxl_grid_clear.argtypes = [vp, vp]
        L.vxl_grid_build_bricks.argtypes = [vp, vp]
        L.vxl_grid_import_r8.argtypes = [vp, vp, vp]
        L.vxl_grid_export_r8.argtypes = [vp, vp, vp]
        L.vxl_grid_import_palette.argtypes = [vp, vp, C.c_int, vp]
        L.vxl_grid_palette_alloc.argtypes = [vp]
        L.vxl_grid_export_palette.argtypes = [vp, vp, vp]
        L.vxl_scene_palette.argtypes = [vp, vp, C.c_uint32, vp]
        L.vxl_grid_count.argtypes = [vp, C.POINTER(C.c_uint64), vp]
        L.vxl_trace_rays.argtypes = [vp, vp, vp, i64, C.c_int, vp, vp]
        L.vxl_trace_occlusion.argtypes = [vp, vp, C.POINTER(GBuffer), C.POINTER(TraceParams), C.POINTER(Outputs), vp]
        L.vxl_trace_occlusion_host.argtypes = [vp, vp, vp, vp, vp, i64, C.POINTER(TraceParams), vp, vp, vp, vp, vp, vp]
        L.vxl_trace_occlusion_from_depth.argtypes = [vp, vp, vp, vp, vp, C.c_int32, C.c_int32, C.POINTER(View),
                                                     C.POINTER(TraceParams), C.POINTER(Outputs), vp]
        L.vxl_batch_create.argtypes = [vp, C.POINTER(BatchItem), C.c_int, C.c_int, C.POINTER(vp)]
        L.vxl_batch_run.argtypes = [vp, vp]
        L.vxl_batch_destroy.argtypes = [vp]
        L.vxl_batch_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.vxl_light_ambient.argtypes = [vp, vp, vp, vp, vp, vp, i64, vp, vp, vp, vp]
        L.vxl_light_reflection.argtypes = [vp, vp, vp, vp, vp, vp, vp, i64, vp, vp, vp]
        L.vxl_light_point.argtypes = [vp, vp, vp, vp, vp, i64, C.POINTER(f * 3), f, C.c_int, vp, vp, vp]
        L.vxl_light_taa.argtypes = [vp, C.POINTER(TaaFrame), vp, vp]
        L.vxl_light_points.argtypes = [vp, vp, vp, vp, vp, i64, C.POINTER(Light), C.c_int, vp, vp, vp]
        L.vxl_voxelize.argtypes = [vp, vp, C.POINTER(Model), C.c_int, C.POINTER(Instance), C.c_int, vp, vp]
        L.vxl_diag_l2_read_gbs.argtypes = [vp, C.c_size_t, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.vxl_voxelize_noalloc.argtypes = [C.POINTER(GridDesc), C.POINTER(Model), C.c_int, C.POINTER(Instance),
                                           C.c_int, vp, vp]
        L.vxl_shadowvox_update.argtypes = [vp, vp, C.POINTER(Model), C.c_int, C.POINTER(Entity), C.c_int, vp, vp]
        L.vxl_vox_destroyed.argtypes = [vp, vp, C.POINTER(Model), C.POINTER(f * 16), vp, vp]
        L.vxl_read_v.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), vp,
                                 C.c_size_t]
        L.vxl_asset_guid.restype = C.c_uint64
        L.vxl_asset_guid.argtypes = [C.c_char_p]
        L.vxl_read_palette.argtypes = [C.c_char_p, vp]
        L.vxl_transform_matrix.argtypes = [vp, vp, vp, vp, vp]
        L.vxl_prefab_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
        L.vxl_prefab_info.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.vxl_prefab_renderer_at.argtypes = [vp, C.c_int, C.POINTER(PrefabRenderer)]
        L.vxl_vox_load.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.vxl_vox_info.argtypes = [vp, C.POINTER(C.c_int32)]
        L.vxl_vox_model_at.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32, C.POINTER(C.c_int32),
                                       C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_float)]
        L.vxl_vox_palette.argtypes = [vp, C.POINTER(C.c_uint8)]
        L.vxl_vox_destroy.argtypes = [vp]
        L.vxl_prefab_volume_at.argtypes = [vp, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.POINTER(C.c_int32), C.POINTER(C.POINTER(C.c_uint8)),
                                           C.POINTER(C.c_uint64)]
        L.vxl_prefab_palette_at.argtypes = [vp, C.c_int, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_uint64)]
        L.vxl_prefab_destroy.argtypes = [vp]
        L.vxl_volume_build_mips.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.vxl_trace_primary.argtypes = [vp, C.POINTER(Volume), C.c_int, C.POINTER(VoxCmd), C.c_int, C.POINTER(Camera),
                                        C.POINTER(PrimaryOut), vp]
        L.vxl_trace_soft_fwd.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(GBuffer), C.POINTER(SoftParams),
                                         vp, vp, vp]
        L.vxl_trace_soft_bwd.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(GBuffer), C.POINTER(SoftParams),
                                         vp, vp, vp, vp]
        L.vxl_scene_soft.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_uint32, f, f, f, C.c_int, C.c_uint32, vp]
        L.vxl_scene_noise.argtypes = [vp, vp, C.c_uint32, f, f, C.c_int, vp]
        L.vxl_scene_terrain.argtypes = [vp, vp, C.c_uint32, f, f, f, C.c_int, vp, vp]
        L.vxl_scene_boxes.argtypes = [vp, vp, C.c_uint32, C.c_int, C.c_int, C.c_int, vp]
        L.vxl_scene_gbuffer.argtypes = [vp, vp, C.POINTER(f * 3), C.POINTER(f * 3), f, C.c_int, C.c_int, C.c_uint32,
                                        vp, vp, vp, vp]
        for name in EXPORTED:
            if name not in ("vxl_abi_version", "vxl_last_error_string", "vxl_status_string", "vxl_asset_guid"):
                getattr(L, name).restype = C.c_int
        _lib = L
        return L


def check(status: int) -> None:
    if status != VXL_OK:
        msg = lib().vxl_last_error_string().decode(errors="replace")
        raise VxlError(status, msg)


def _ptr(t) -> int | None:
    """Device (or host) address of a torch tensor / numpy array / int / None."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class Context:
    """vxl_ctx on one CUDA device."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().vxl_ctx_create(device, C.byref(self._h)))
        self.device = device

    @property
    def handle(self):
        return self._h

    def launch_count(self) -> int:
        n = C.c_uint64()
        check(lib().vxl_ctx_launch_count(self._h, C.byref(n)))
        return n.value

    def set_tuning(self, tile_px=0, kstep=0, leap=0, order=0, tile_w=0, grab=0):
        t = Tuning(tile_px, kstep, leap, order, tile_w, grab)
        check(lib().vxl_ctx_set_tuning(self._h, C.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning()
        check(lib().vxl_ctx_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def close(self):
        if self._h:
            lib().vxl_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Grid:
    """Bit-packed ShadowVox grid of fine dimensions (nx, ny, nz)."""

    def __init__(self, ctx: Context, nx: int, ny: int, nz: int):
        self.ctx = ctx
        self._h = C.c_void_p()
        check(lib().vxl_grid_create(ctx.handle, nx, ny, nz, C.byref(self._h)))
        self.nx, self.ny, self.nz = nx, ny, nz

    @property
    def handle(self):
        return self._h

    def describe(self) -> GridDesc:
        d = GridDesc()
        check(lib().vxl_grid_describe(self._h, C.byref(d)))
        return d

    def clear(self, stream=None):
        check(lib().vxl_grid_clear(self._h, _stream(stream)))

    def build_bricks(self, stream=None):
        check(lib().vxl_grid_build_bricks(self._h, _stream(stream)))

    def import_r8(self, d_bytes, stream=None):
        check(lib().vxl_grid_import_r8(self._h, _ptr(d_bytes), _stream(stream)))

    def export_r8(self, d_bytes, stream=None):
        check(lib().vxl_grid_export_r8(self._h, _ptr(d_bytes), _stream(stream)))

    def import_palette(self, d_pal, opaque_min=16, stream=None):
        check(lib().vxl_grid_import_palette(self._h, _ptr(d_pal), opaque_min, _stream(stream)))

    def palette_alloc(self):
        """Give the grid its 4-bit palette plane (zeroed; no-op if present)."""
        check(lib().vxl_grid_palette_alloc(self._h))

    def export_palette(self, d_out, stream=None):
        """The palette plane as a dense device uint8 volume [nz][ny][nx]."""
        check(lib().vxl_grid_export_palette(self._h, _ptr(d_out), _stream(stream)))

    def scene_palette(self, seed, stream=None):
        check(lib().vxl_scene_palette(self.ctx.handle, self._h, seed, _stream(stream)))

    def count(self, stream=None) -> int:
        n = C.c_uint64()
        check(lib().vxl_grid_count(self._h, C.byref(n), _stream(stream)))
        return n.value

    def scene_noise(self, seed, thresh=0.55, freq=1.0 / 32.0, ground_y=8, stream=None):
        check(lib().vxl_scene_noise(self.ctx.handle, self._h, seed, thresh, freq, ground_y, _stream(stream)))

    def scene_terrain(self, seed, base, amplitude, freq, octaves=5, d_height=None, stream=None):
        check(lib().vxl_scene_terrain(self.ctx.handle, self._h, seed, base, amplitude, freq, octaves, _ptr(d_height),
                                      _stream(stream)))

    def scene_boxes(self, seed, nboxes, smin=4, smax=48, stream=None):
        check(lib().vxl_scene_boxes(self.ctx.handle, self._h, seed, nboxes, smin, smax, _stream(stream)))

    def close(self):
        if self._h:
            lib().vxl_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=(0, 0, 0), bias=0.5, shadow_len=100.0, ao_len=16.0,
                spec_len=256.0, default_rough=0.5, n_shadow=1, n_ao=4, n_spec=0, seed=1, mode=MODE_DDA):
    p = TraceParams()
    ld = np.asarray(light_dir, np.float64)
    ld = (ld / np.linalg.norm(ld)).astype(np.float32)
    p.light_dir[:] = [float(v) for v in ld]
    p.cam_pos[:] = [float(v) for v in np.asarray(cam_pos, np.float32)]
    p.bias, p.shadow_len, p.ao_len, p.spec_len, p.default_rough = bias, shadow_len, ao_len, spec_len, default_rough
    p.n_shadow, p.n_ao, p.n_spec, p.seed, p.mode = n_shadow, n_ao, n_spec, seed, mode
    return p


def trace_rays(ctx: Context, grid: Grid, d_rays, n: int, mode: int, d_records, stream=None):
    check(lib().vxl_trace_rays(ctx.handle, grid.handle, _ptr(d_rays), n, mode, _ptr(d_records), _stream(stream)))


def trace_occlusion(ctx: Context, grid: Grid, pos, nrm, rough, npix: int, params: TraceParams, shadow=None,
                    ao=None, ao_vis=None, spec=None, spec_t=None, records=None, stream=None, width=0, height=0):
    """width/height (optional, width*height == npix) let the kernel use
    image-block tiles (vxl_tuning.tile_w)."""
    gb = GBuffer(_ptr(pos), _ptr(nrm), _ptr(rough), npix, width, height)
    out = Outputs(_ptr(shadow), _ptr(ao), _ptr(ao_vis), _ptr(spec), _ptr(spec_t), _ptr(records))
    check(lib().vxl_trace_occlusion(ctx.handle, grid.handle, C.byref(gb), C.byref(params), C.byref(out),
                                    _stream(stream)))


def trace_occlusion_from_depth(ctx: Context, grid: Grid, depth, nrm, rough, W: int, H: int, inv_view, inv_proj,
                               params: TraceParams, shadow=None, ao=None, ao_vis=None, spec=None, spec_t=None,
                               records=None, stream=None):
    """vxl_trace_occlusion_from_depth: positions rebuilt from a linear-depth
    G-buffer as LightAmbient places a pixel; inv_view / inv_proj are the view
    buffer's InverseViewMatrix / InverseProjectionMatrix (column-major 16 floats)."""
    v = View()
    v.inverse_view[:] = [float(x) for x in np.asarray(inv_view, np.float32).reshape(16)]
    v.inverse_projection[:] = [float(x) for x in np.asarray(inv_proj, np.float32).reshape(16)]
    out = Outputs(_ptr(shadow), _ptr(ao), _ptr(ao_vis), _ptr(spec), _ptr(spec_t), _ptr(records))
    check(lib().vxl_trace_occlusion_from_depth(ctx.handle, grid.handle, _ptr(depth), _ptr(nrm), _ptr(rough), W, H,
                                               C.byref(v), C.byref(params), C.byref(out), _stream(stream)))


def trace_occlusion_host(ctx: Context, grid: Grid, h_pos, h_nrm, h_rough, npix: int, params: TraceParams,
                         h_shadow=None, h_ao=None, h_ao_vis=None, h_spec=None, h_spec_t=None, stream=None):
    check(lib().vxl_trace_occlusion_host(ctx.handle, grid.handle, _ptr(h_pos), _ptr(h_nrm), _ptr(h_rough), npix,
                                         C.byref(params), _ptr(h_shadow), _ptr(h_ao), _ptr(h_ao_vis), _ptr(h_spec),
                                         _ptr(h_spec_t), _stream(stream)))


class Batch:
    """vxl_batch: many scenes traced by one persistent launch (CUDA-graph replay).

    items: list of dicts with keys grid, pos, nrm, rough, npix, width, height,
    params, and output tensors shadow/ao/ao_vis/spec/spec_t (any may be None).
    The tensors must stay alive while the batch exists (kept referenced here)."""

    def __init__(self, ctx: Context, items, use_graph=True):
        self.ctx = ctx
        self._keep = items
        arr = (BatchItem * len(items))()
        for i, it in enumerate(items):
            arr[i].grid = it["grid"].handle.value
            arr[i].gbuf = GBuffer(_ptr(it["pos"]), _ptr(it["nrm"]), _ptr(it.get("rough")), it["npix"],
                                  it.get("width", 0), it.get("height", 0))
            arr[i].params = it["params"]
            arr[i].out = Outputs(_ptr(it.get("shadow")), _ptr(it.get("ao")), _ptr(it.get("ao_vis")),
                                 _ptr(it.get("spec")), _ptr(it.get("spec_t")), None)
        self._h = C.c_void_p()
        check(lib().vxl_batch_create(ctx.handle, arr, len(items), 1 if use_graph else 0, C.byref(self._h)))

    def run(self, stream=None):
        check(lib().vxl_batch_run(self._h, _stream(stream)))

    def info(self):
        t, r = C.c_int64(), C.c_int64()
        check(lib().vxl_batch_info(self._h, C.byref(t), C.byref(r)))
        return t.value, r.value

    def close(self):
        if self._h:
            lib().vxl_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def light_ambient(ctx, grid, wcp, nrm, depth, noise, npix, shadow, irradiance, records=None, stream=None):
    check(lib().vxl_light_ambient(ctx.handle, grid.handle, _ptr(wcp), _ptr(nrm), _ptr(depth), _ptr(noise), npix,
                                  _ptr(shadow), _ptr(irradiance), _ptr(records), _stream(stream)))


def light_reflection(ctx, grid, wcp, nrm, view_r, rough, noise, npix, t_out, records=None, stream=None):
    check(lib().vxl_light_reflection(ctx.handle, grid.handle, _ptr(wcp), _ptr(nrm), _ptr(view_r), _ptr(rough),
                                     _ptr(noise), npix, _ptr(t_out), _ptr(records), _stream(stream)))


def light_point(ctx, grid, wpos, nrm, noise, npix, light_pos, light_range, spot, shadow, records=None, stream=None):
    check(lib().vxl_light_point(ctx.handle, grid.handle, _ptr(wpos), _ptr(nrm), _ptr(noise), npix,
                                C.byref(_f3(light_pos)), float(light_range), 1 if spot else 0, _ptr(shadow),
                                _ptr(records), _stream(stream)))


def light_taa(ctx, light, last_light, color, normal, material, depth, motion, noise, W, H, out, stream=None):
    f = TaaFrame(_ptr(light), _ptr(last_light), _ptr(color), _ptr(normal), _ptr(material), _ptr(depth), _ptr(motion),
                 _ptr(noise), W, H)
    check(lib().vxl_light_taa(ctx.handle, C.byref(f), _ptr(out), _stream(stream)))


def light_points(ctx, grid, wpos, nrm, noise, npix, lights, lit, in_range=None, stream=None):
    """lights: list of (pos3, range, spot)."""
    arr = (Light * max(1, len(lights)))()
    for i, (p, r, sp) in enumerate(lights):
        arr[i].pos[:] = [float(x) for x in p]
        arr[i].range = float(r)
        arr[i].spot = 1 if sp else 0
    check(lib().vxl_light_points(ctx.handle, grid.handle, _ptr(wpos), _ptr(nrm), _ptr(noise), npix, arr, len(lights),
                                 _ptr(lit), _ptr(in_range), _stream(stream)))


def scene_gbuffer(ctx, grid, cam, target, W, H, seed, d_pos, d_nrm, d_rough, tan_half_fov=0.57735026, stream=None):
    check(lib().vxl_scene_gbuffer(ctx.handle, grid.handle, C.byref(_f3(cam)), C.byref(_f3(target)),
                                  float(tan_half_fov), W, H, seed, _ptr(d_pos), _ptr(d_nrm), _ptr(d_rough),
                                  _stream(stream)))


def make_soft_params(light_dir=(0.3, 0.8, 0.5), bias=0.5, length=24.0, k_sun=0.7, k_amb=0.5, n_shadow=1, n_ao=16,
                     seed=7) -> SoftParams:
    p = SoftParams()
    p.light_dir[:] = [float(x) for x in light_dir]
    p.bias, p.len, p.k_sun, p.k_amb = bias, length, k_sun, k_amb
    p.n_shadow, p.n_ao, p.seed = n_shadow, n_ao, seed
    return p


def _soft_dims(soft):
    nz, ny, nx, four = soft.shape
    assert four == 4, "soft grid is [nz, ny, nx, 4]"
    return nx, ny, nz


def trace_soft_fwd(ctx, soft, pos, nrm, npix: int, params: SoftParams, image, light=None, stream=None):
    """Soft-opacity forward (vxl_trace_soft_fwd); soft is a float32 [nz, ny, nx, 4] device tensor."""
    nx, ny, nz = _soft_dims(soft)
    gb = GBuffer(_ptr(pos), _ptr(nrm), None, npix, 0, 0)
    check(lib().vxl_trace_soft_fwd(ctx.handle, _ptr(soft), nx, ny, nz, C.byref(gb), C.byref(params), _ptr(image),
                                   _ptr(light), _stream(stream)))


def trace_soft_bwd(ctx, soft, pos, nrm, npix: int, params: SoftParams, grad_image, light, grad_soft, stream=None):
    """Adjoint (vxl_trace_soft_bwd): accumulates into grad_soft (same shape as soft)."""
    nx, ny, nz = _soft_dims(soft)
    gb = GBuffer(_ptr(pos), _ptr(nrm), None, npix, 0, 0)
    check(lib().vxl_trace_soft_bwd(ctx.handle, _ptr(soft), nx, ny, nz, C.byref(gb), C.byref(params),
                                   _ptr(grad_image), _ptr(light), _ptr(grad_soft), _stream(stream)))


def scene_soft(ctx, soft, seed, thresh=0.55, sharpness=8.0, freq=1.0 / 32.0, ground_y=8, albedo_seed=1, stream=None):
    nx, ny, nz = _soft_dims(soft)
    check(lib().vxl_scene_soft(ctx.handle, _ptr(soft), nx, ny, nz, seed, thresh, sharpness, freq, ground_y,
                               albedo_seed, _stream(stream)))


def volume_build_mips(ctx, d_mip0, sx, sy, sz, d_mip1, d_mip2, stream=None):
    check(lib().vxl_volume_build_mips(ctx.handle, _ptr(d_mip0), sx, sy, sz, _ptr(d_mip1), _ptr(d_mip2),
                                      _stream(stream)))


class VolumeSet:
    """Device copies of VoxAsset volumes (uint8 [sz, sy, sx] each) with their mips."""

    def __init__(self, ctx, volumes):
        import torch

        self.mips = []
        for v in volumes:
            v = np.ascontiguousarray(v, np.uint8)
            sz, sy, sx = v.shape
            d0 = torch.from_numpy(v).cuda()
            dims = [(sx, sy, sz)]
            for _ in range(2):
                dims.append(tuple(a // 2 if a > 1 else 1 for a in dims[-1]))
            d1 = torch.empty(int(np.prod(dims[1])), dtype=torch.uint8, device="cuda")
            d2 = torch.empty(int(np.prod(dims[2])), dtype=torch.uint8, device="cuda")
            volume_build_mips(ctx, d0, sx, sy, sz, d1, d2)
            self.mips.append((d0, d1, d2, (sx, sy, sz)))
        self.table = (Volume * max(1, len(self.mips)))()
        for i, (d0, d1, d2, (sx, sy, sz)) in enumerate(self.mips):
            self.table[i].mip[:] = [d0.data_ptr(), d1.data_ptr(), d2.data_ptr()]
            self.table[i].sx, self.table[i].sy, self.table[i].sz = sx, sy, sz

    def __len__(self):
        return len(self.mips)


VOXCMD_DTYPE = np.dtype([("world", "<f4", (16,)), ("volume", "<i4"), ("palette", "<i4")])


def voxcmds(worlds, vol_of, palette=None) -> np.ndarray:
    """The command table of vxl_trace_primary as a numpy record array (layout of vxl_voxcmd)."""
    worlds = np.ascontiguousarray(worlds, np.float32).reshape(-1, 16)
    rec = np.zeros(worlds.shape[0], dtype=VOXCMD_DTYPE)
    rec["world"] = worlds
    rec["volume"] = np.asarray(vol_of, np.int32)
    if palette is not None:
        rec["palette"] = np.asarray(palette, np.int32)
    return rec


def trace_primary(ctx, volset: VolumeSet, worlds, vol_of, cam, target, W, H, pos, nrm, depth=None, material=None,
                  instance=None, frame=0, tan_half_fov=0.57735026, stream=None, cmds=None):
    """vxl_trace_primary; worlds float[n, 16] column-major, vol_of int[n] (or a prebuilt
    `cmds` table from voxcmds()); camera in world units."""
    rec = cmds if cmds is not None else voxcmds(worlds, vol_of)
    n = rec.shape[0]
    if n == 0:
        rec = np.zeros(1, dtype=VOXCMD_DTYPE)
    cmds = rec.ctypes.data_as(C.POINTER(VoxCmd))
    c = Camera()
    c.pos[:] = [float(x) for x in cam]
    c.target[:] = [float(x) for x in target]
    c.tan_half_fov, c.width, c.height, c.frame = tan_half_fov, W, H, frame
    out = PrimaryOut(_ptr(pos), _ptr(nrm), _ptr(depth), _ptr(material), _ptr(instance))
    check(lib().vxl_trace_primary(ctx.handle, volset.table, len(volset), cmds, n, C.byref(c), C.byref(out),
                                  _stream(stream)))
    del rec


def _models(models):
    arr = (Model * max(1, len(models)))()
    for i, (ptr, sx, sy, sz) in enumerate(models):
        arr[i] = Model(ptr, sx, sy, sz)
    return arr


def voxelize(ctx, grid, models, instances, d_aabb=None, stream=None):
    """models: list of (device ptr, sx, sy, sz); instances: list of (matrix16, model, op)."""
    ms = _models(models)
    arr = (Instance * max(1, len(instances)))()
    for i, (m, mi, op) in enumerate(instances):
        arr[i].matrix[:] = [float(x) for x in np.asarray(m, np.float32).reshape(16)]
        arr[i].model, arr[i].op = mi, op
    check(lib().vxl_voxelize(ctx.handle, grid.handle, ms, len(models), arr, len(instances), _ptr(d_aabb),
                             _stream(stream)))


def voxelize_noalloc(grid_desc, models, instances, d_aabb=None, stream=None):
    """vxl_voxelize_noalloc: like voxelize(), for callers that cannot allocate:
    takes a GridDesc (no context, no grid handle) and uses the library's fixed
    static device table as its only scratch."""
    ms = _models(models)
    arr = (Instance * max(1, len(instances)))()
    for i, (m, mi, op) in enumerate(instances):
        arr[i].matrix[:] = [float(x) for x in np.asarray(m, np.float32).reshape(16)]
        arr[i].model, arr[i].op = mi, op
    check(lib().vxl_voxelize_noalloc(C.byref(grid_desc), ms, len(models), arr, len(instances), _ptr(d_aabb),
                                     _stream(stream)))


def shadowvox_update(ctx, grid, models, entities, stream=None):
    """entities: list of (prev16, world16, pivot3, model). Returns int32[n,6] dirty regions."""
    ms = _models(models)
    arr = (Entity * max(1, len(entities)))()
    for i, (pw, w, pv, mi) in enumerate(entities):
        arr[i].prev_world[:] = [float(x) for x in np.asarray(pw, np.float32).reshape(16)]
        arr[i].world[:] = [float(x) for x in np.asarray(w, np.float32).reshape(16)]
        arr[i].pivot[:] = [float(x) for x in np.asarray(pv, np.float32).reshape(3)]
        arr[i].model = mi
    regions = np.zeros((len(entities), 6), np.int32)
    check(lib().vxl_shadowvox_update(ctx.handle, grid.handle, ms, len(models), arr, len(entities), _ptr(regions),
                                     _stream(stream)))
    return regions


def vox_destroyed(ctx, grid, model, world, stream=None):
    ms = _models([model])
    w = (C.c_float * 16)(*[float(x) for x in np.asarray(world, np.float32).reshape(16)])
    region = np.zeros(6, np.int32)
    check(lib().vxl_vox_destroyed(ctx.handle, grid.handle, ms, C.byref(w), _ptr(region), _stream(stream)))
    return region


def asset_guid(mod_path: str) -> int:
    return lib().vxl_asset_guid(mod_path.encode())


def read_palette(path: str) -> np.ndarray:
    out = np.zeros((256, 7), np.uint8)
    check(lib().vxl_read_palette(path.encode(), out.ctypes.data))
    return out


def transform_matrix(pos, rot, scale, parent=None) -> np.ndarray:
    p = np.asarray(pos, np.float32)
    r = np.asarray(rot, np.float32)
    s_ = np.asarray(scale, np.float32)
    par = None if parent is None else np.ascontiguousarray(parent, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    check(lib().vxl_transform_matrix(p.ctypes.data, r.ctypes.data, s_.ctypes.data,
                                     None if par is None else par.ctypes.data, out.ctypes.data))
    return out


def load_vox(path: str) -> dict:
    """vxl_vox_load: a MagicaVoxel .vox file imported as the engine's importer
    does: dict(models=[dict(name, volume=uint8 [sz, sy, sx], position=float32[3])],
    palette=uint8 [256, 7])."""
    h = C.c_void_p()
    check(lib().vxl_vox_load(path.encode(), C.byref(h)))
    try:
        n = C.c_int32()
        check(lib().vxl_vox_info(h, C.byref(n)))
        models = []
        for i in range(n.value):
            name = C.create_string_buffer(256)
            size = (C.c_int32 * 3)()
            ptr = C.POINTER(C.c_uint8)()
            pos = (C.c_float * 3)()
            check(lib().vxl_vox_model_at(h, i, name, 256, size, C.byref(ptr), pos))
            sx, sy, sz = size
            vol = np.ctypeslib.as_array(ptr, (sx * sy * sz,)).copy().reshape(sz, sy, sx)
            models.append(dict(name=name.value.decode(), volume=vol, position=np.array(pos, np.float32)))
        pal = np.zeros(256 * 7, np.uint8)
        check(lib().vxl_vox_palette(h, pal.ctypes.data_as(C.POINTER(C.c_uint8))))
        return dict(models=models, palette=pal.reshape(256, 7))
    finally:
        lib().vxl_vox_destroy(h)


def load_prefab(mods_dir: str, mod_path: str) -> dict:
    """vxl_prefab_load: returns dict(renderers=[(world16, pivot3, volume, palette, entity)],
    volumes=[uint8 [sz, sy, sx]], palettes=[uint8 [256, 7]], volume_guids, palette_guids)."""
    h = C.c_void_p()
    check(lib().vxl_prefab_load(mods_dir.encode(), mod_path.encode(), C.byref(h)))
    try:
        nr, nv, npal = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().vxl_prefab_info(h, C.byref(nr), C.byref(nv), C.byref(npal)))
        rens = []
        for i in range(nr.value):
            r = PrefabRenderer()
            check(lib().vxl_prefab_renderer_at(h, i, C.byref(r)))
            rens.append((np.array(r.world, np.float32), np.array(r.pivot, np.float32), r.volume, r.palette, r.entity))
        vols, vg = [], []
        for i in range(nv.value):
            sx, sy, sz = C.c_int32(), C.c_int32(), C.c_int32()
            ptr = C.POINTER(C.c_uint8)()
            g = C.c_uint64()
            check(lib().vxl_prefab_volume_at(h, i, C.byref(sx), C.byref(sy), C.byref(sz), C.byref(ptr), C.byref(g)))
            n = sx.value * sy.value * sz.value
            vols.append(np.ctypeslib.as_array(ptr, (n,)).copy().reshape(sz.value, sy.value, sx.value))
            vg.append(g.value)
        pals, pg = [], []
        for i in range(npal.value):
            ptr = C.POINTER(C.c_uint8)()
            g = C.c_uint64()
            check(lib().vxl_prefab_palette_at(h, i, C.byref(ptr), C.byref(g)))
            pals.append(np.ctypeslib.as_array(ptr, (256 * 7,)).copy().reshape(256, 7))
            pg.append(g.value)
        return dict(renderers=rens, volumes=vols, palettes=pals, volume_guids=vg, palette_guids=pg)
    finally:
        lib().vxl_prefab_destroy(h)


def read_v(path: str) -> np.ndarray:
    """Read a .v asset (u32 sx, sy, sz then bytes) -> uint8[sz, sy, sx]."""
    sx, sy, sz = C.c_int32(), C.c_int32(), C.c_int32()
    check(lib().vxl_read_v(path.encode(), C.byref(sx), C.byref(sy), C.byref(sz), None, 0))
    out = np.zeros((sz.value, sy.value, sx.value), np.uint8)
    check(lib().vxl_read_v(path.encode(), C.byref(sx), C.byref(sy), C.byref(sz), _ptr(out), out.nbytes))
    return out


def l2_read_gbs(ctx: Context, nbytes: int = 64 << 20, reps: int = 50):
    """Best L2 read bandwidth (GB/s, ms) of a kernel streaming an
    L2-resident buffer of nbytes (vxl_diag_l2_read_gbs)."""
    g, ms = C.c_double(), C.c_double()
    check(lib().vxl_diag_l2_read_gbs(ctx.handle, nbytes, reps, C.byref(g), C.byref(ms)))
    return g.value, ms.value
