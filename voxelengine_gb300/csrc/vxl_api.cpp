// vxl_api.cpp — host side of libvxl: the C ABI declared in include/vxl.h.
// Validates arguments, owns contexts and grids, plans voxelizer runs, and
// dispatches to the kernel launchers. Compiled without FMA contraction so the
// host-side matrix arithmetic (glm::translate) matches the reference bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "vxl_internal.h"

namespace vxl {

static thread_local std::string g_last_error;

vxl_status fail(vxl_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

vxl_status cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? VXL_ERR_OOM : VXL_ERR_CUDA, "%s: %s (%s)", what,
                cudaGetErrorString(e), cudaGetErrorName(e));
}

vxl_status ctx_grow(void** p, size_t* have, size_t need) {
    if (*have >= need) return VXL_OK;
    size_t n = *have ? *have : (size_t)1 << 20;
    while (n < need) n *= 2;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
    *have = n;
    return VXL_OK;
}

vxl_status ctx_scratch(vxl_ctx* ctx, size_t bytes, void** out) {
    VXL_TRY(ctx_grow(&ctx->d_scratch, &ctx->d_scratch_bytes, bytes));
    *out = ctx->d_scratch;
    return VXL_OK;
}
vxl_status ctx_stage(vxl_ctx* ctx, size_t bytes, void** out) {
    VXL_TRY(ctx_grow(&ctx->d_stage, &ctx->d_stage_bytes, bytes));
    *out = ctx->d_stage;
    return VXL_OK;
}

// Device address of host memory the device can reach (pinned, mapped into the
// unified address space of this context's device); false for anything else,
// which then goes through explicit copies.
static bool device_view(const vxl_ctx* ctx, const void* h, void** d) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();  // clear the error of an unknown pointer
        return false;
    }
    // pinned under this device's context (memory pinned for another device is
    // not assumed to be mapped here)
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr || a.device != ctx->device) return false;
    int mapped = 0;
    if (cudaDeviceGetAttribute(&mapped, cudaDevAttrCanMapHostMemory, ctx->device) != cudaSuccess || !mapped)
        return false;
    *d = a.devicePointer;
    return true;
}

vxl_status ctx_take_counter(vxl_ctx* ctx, cudaStream_t s, unsigned long long** out) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    VXL_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
        *out = ctx->d_counters + (ctx->counter_next++ % kCounterRing);
        return VXL_OK;
    }
    // a captured launch replays with this counter for as long as its graph
    // lives: give it a slot that no other launch of this context ever gets
    if (ctx->capture_next >= kCaptureCounters)
        return fail(VXL_ERR_NOT_SUPPORTED, "trace_occlusion: more than %u captured occlusion calls on one context",
                    kCaptureCounters);
    *out = ctx->d_counters + kCounterRing + ctx->capture_next++;
    return VXL_OK;
}

// glm::translate(m, v): Result[3] = m[0]*v[0] + m[1]*v[1] + m[2]*v[2] + m[3]
static void translate(const float* m, const float* v, float* out) {
    std::memcpy(out, m, 16 * sizeof(float));
    for (int r = 0; r < 4; r++) {
        float a = m[0 + r] * v[0] + m[4 + r] * v[1];
        a = a + m[8 + r] * v[2];
        out[12 + r] = a + m[12 + r];
    }
}

static vxl_status set_device(const vxl_ctx* ctx) {
    VXL_TRY_CUDA(cudaSetDevice(ctx->device));
    return VXL_OK;
}

static bool grid_ok(const vxl_grid* g) { return g && g->ctx && g->words; }

// Plan a voxelizer run: upload instances/models/chunk table, launch.
static vxl_status voxelize_runs(vxl_ctx* ctx, vxl_grid* g, const vxl_model* models, int nmodels,
                                const std::vector<DevInstance>& inst, int32_t* d_aabb, cudaStream_t s) {
    const int n = (int)inst.size();
    if (n == 0) return VXL_OK;
    std::vector<DevModel> dm((size_t)nmodels);
    for (int i = 0; i < nmodels; i++) dm[i] = DevModel{models[i].data, models[i].sx, models[i].sy, models[i].sz, 0};
    // chunk tables per run of equal ops, concatenated
    std::vector<int2> chunks;
    std::vector<std::pair<size_t, size_t>> runs;  // [begin, end) into chunks
    std::vector<int> run_value;
    for (int i = 0; i < n;) {
        int j = i;
        size_t b = chunks.size();
        while (j < n && inst[j].op == inst[i].op) {
            const DevModel& m = dm[inst[j].model];
            long long cnt = (long long)m.sx * m.sy * m.sz;
            for (long long v = 0; v < cnt; v += kVoxChunk) chunks.push_back(make_int2(j, (int)v));
            j++;
        }
        runs.push_back({b, chunks.size()});
        run_value.push_back(inst[i].op == VXL_OP_SET ? 1 : 0);
        i = j;
    }
    size_t b_inst = inst.size() * sizeof(DevInstance);
    size_t b_mod = dm.size() * sizeof(DevModel);
    size_t b_ch = chunks.size() * sizeof(int2);
    size_t off_mod = (b_inst + 255) & ~(size_t)255, off_ch = (off_mod + b_mod + 255) & ~(size_t)255;
    void* scratch;
    VXL_TRY(ctx_scratch(ctx, off_ch + b_ch + 256, &scratch));
    char* base = (char*)scratch;
    VXL_TRY_CUDA(cudaMemcpyAsync(base, inst.data(), b_inst, cudaMemcpyHostToDevice, s));
    VXL_TRY_CUDA(cudaMemcpyAsync(base + off_mod, dm.data(), b_mod, cudaMemcpyHostToDevice, s));
    if (b_ch) VXL_TRY_CUDA(cudaMemcpyAsync(base + off_ch, chunks.data(), b_ch, cudaMemcpyHostToDevice, s));
    const DevInstance* d_inst = (const DevInstance*)base;
    const DevModel* d_mod = (const DevModel*)(base + off_mod);
    const int2* d_ch = (const int2*)(base + off_ch);
    for (size_t r = 0; r < runs.size(); r++) {
        int nch = (int)(runs[r].second - runs[r].first);
        VXL_TRY(launch_voxelize_run(g, d_inst, d_mod, d_ch + runs[r].first, nch, run_value[r], d_aabb, s));
    }
    // the host vectors must outlive the async copies
    VXL_TRY_CUDA(cudaStreamSynchronize(s));
    return launch_build_tile_mask(g, s);
}

static vxl_status check_models(const vxl_model* models, int nmodels) {
    if (nmodels < 0 || (nmodels > 0 && !models)) return fail(VXL_ERR_INVALID_ARG, "models: bad pointer/count");
    for (int i = 0; i < nmodels; i++) {
        const vxl_model& m = models[i];
        if (!m.data || m.sx <= 0 || m.sy <= 0 || m.sz <= 0)
            return fail(VXL_ERR_INVALID_ARG, "model %d: null data or non-positive size", i);
        if ((long long)m.sx * m.sy * m.sz > (1ll << 30))
            return fail(VXL_ERR_OUT_OF_RANGE, "model %d: more than 2^30 voxels", i);
    }
    return VXL_OK;
}

// dirty-region tail of OnUpdate (ShadowVoxSystem.cpp:180-190)
static void region_from_aabb(const int* aabb, int sx, int sy, int sz, int32_t* region) {
    if (aabb[3] != 0 || aabb[4] != 0 || aabb[5] != 0) {
        int mn[3] = {aabb[0] / 2, aabb[1] / 2, aabb[2] / 2};
        int mx[3] = {aabb[3] / 2, aabb[4] / 2, aabb[5] / 2};
        int lim[3] = {sx - 1, sy - 1, sz - 1};
        for (int a = 0; a < 3; a++) {
            if (mn[a] < 0) mn[a] = 0;
            if (mx[a] > lim[a]) mx[a] = lim[a];
            region[a] = mn[a];
            region[3 + a] = mx[a] - mn[a] + 1;
        }
    } else {
        for (int a = 0; a < 6; a++) region[a] = -1;
    }
}

static vxl_status check_params(const vxl_trace_params* p) {
    if (!p) return fail(VXL_ERR_INVALID_ARG, "params is NULL");
    if (p->mode != VXL_MODE_DDA) return fail(VXL_ERR_NOT_SUPPORTED, "trace_occlusion: mode must be VXL_MODE_DDA");
    if (p->n_shadow < 0 || p->n_shadow > 1) return fail(VXL_ERR_INVALID_ARG, "n_shadow must be 0 or 1");
    if (p->n_ao < 0 || p->n_ao > 64) return fail(VXL_ERR_INVALID_ARG, "n_ao must be in [0,64]");
    if (p->n_spec < 0 || p->n_spec > 8) return fail(VXL_ERR_INVALID_ARG, "n_spec must be in [0,8]");
    if (p->n_ao > 0 && !(p->ao_len > 0.0f)) return fail(VXL_ERR_INVALID_ARG, "ao_len must be > 0");
    return VXL_OK;
}

}  // namespace vxl

using namespace vxl;

extern "C" {

int vxl_abi_version(void) { return VXL_ABI_VERSION; }
const char* vxl_last_error_string(void) { return g_last_error.c_str(); }
const char* vxl_status_string(vxl_status s) {
    switch (s) {
        case VXL_OK: return "VXL_OK";
        case VXL_ERR_INVALID_ARG: return "VXL_ERR_INVALID_ARG";
        case VXL_ERR_OOM: return "VXL_ERR_OOM";
        case VXL_ERR_CUDA: return "VXL_ERR_CUDA";
        case VXL_ERR_TIMEOUT: return "VXL_ERR_TIMEOUT";
        case VXL_ERR_OUT_OF_RANGE: return "VXL_ERR_OUT_OF_RANGE";
        case VXL_ERR_IO: return "VXL_ERR_IO";
        case VXL_ERR_NOT_SUPPORTED: return "VXL_ERR_NOT_SUPPORTED";
    }
    return "VXL_ERR_?";
}

vxl_status vxl_ctx_create(int device, vxl_ctx** out) {
    if (!out) return fail(VXL_ERR_INVALID_ARG, "ctx_create: out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(VXL_ERR_INVALID_ARG, "ctx_create: device %d of %d", device, n);
    VXL_TRY_CUDA(cudaSetDevice(device));
    vxl_ctx* c = new (std::nothrow) vxl_ctx();
    if (!c) return fail(VXL_ERR_OOM, "ctx_create: host allocation");
    c->device = device;
    e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    const size_t counter_bytes = (size_t)(kCounterRing + kCaptureCounters) * sizeof(unsigned long long);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_counters, counter_bytes);
    if (e == cudaSuccess) e = cudaMemset(c->d_counters, 0, counter_bytes);
    if (e != cudaSuccess) {
        if (c->d_counters) cudaFree(c->d_counters);
        delete c;
        return cuda_fail(e, "ctx_create");
    }
    c->tune = vxl_tuning{16, 8, 2, 1, 16, 1};  // best on GB300 for the 512^3 / 1080p workload
    *out = c;
    return VXL_OK;
}

vxl_status vxl_ctx_destroy(vxl_ctx* ctx) {
    if (!ctx) return VXL_OK;
    cudaSetDevice(ctx->device);
    if (ctx->d_scratch) cudaFree(ctx->d_scratch);
    if (ctx->d_stage) cudaFree(ctx->d_stage);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->pipe_ready) {
        for (int k = 0; k < 2; k++) cudaStreamDestroy(ctx->pipe[k]);
        cudaEventDestroy(ctx->pipe_start);
    }
    if (ctx->pev) {
        cudaEventSynchronize(ctx->pev);
        cudaEventDestroy(ctx->pev);
    }
    if (ctx->d_plist) cudaFree(ctx->d_plist);
    if (ctx->h_ptotal) cudaFreeHost(ctx->h_ptotal);
    if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
    if (ctx->d_taa) cudaFree(ctx->d_taa);
    if (ctx->d_fd) cudaFree(ctx->d_fd);
    if (ctx->d_lpairs) cudaFree(ctx->d_lpairs);
    delete ctx;
    return VXL_OK;
}

vxl_status vxl_ctx_launch_count(const vxl_ctx* ctx, uint64_t* out) {
    if (!ctx || !out) return fail(VXL_ERR_INVALID_ARG, "ctx_launch_count: NULL argument");
    *out = ctx->launches;
    return VXL_OK;
}

vxl_status vxl_ctx_set_tuning(vxl_ctx* ctx, const vxl_tuning* t) {
    if (!ctx || !t) return fail(VXL_ERR_INVALID_ARG, "ctx_set_tuning: NULL argument");
    vxl_tuning n = ctx->tune;
    if (t->tile_px) {
        if (t->tile_px != 8 && t->tile_px != 16 && t->tile_px != 32)
            return fail(VXL_ERR_INVALID_ARG, "tile_px must be 8, 16 or 32");
        n.tile_px = t->tile_px;
    }
    if (t->kstep) {
        if (t->kstep != 1 && t->kstep != 2 && t->kstep != 4 && t->kstep != 8 && t->kstep != 16)
            return fail(VXL_ERR_INVALID_ARG, "kstep must be 1, 2, 4, 8 or 16");
        n.kstep = t->kstep;
    }
    if (t->leap) {
        if (t->leap != 1 && t->leap != 2 && t->leap != 3) return fail(VXL_ERR_INVALID_ARG, "leap must be 1, 2 or 3");
        n.leap = t->leap;
    }
    if (t->order) {
        if (t->order != 1 && t->order != 2) return fail(VXL_ERR_INVALID_ARG, "order must be 1 or 2");
        n.order = t->order;
    }
    if (t->grab) {
        if (t->grab != 1 && t->grab != 2 && t->grab != 4) return fail(VXL_ERR_INVALID_ARG, "grab must be 1, 2 or 4");
        n.grab = t->grab;
    }
    if (t->tile_w) n.tile_w = t->tile_w;
    if (n.tile_w > n.tile_px || n.tile_px % n.tile_w != 0 ||
        (n.tile_w != n.tile_px && n.tile_w != 4 && n.tile_w != 8))
        n.tile_w = n.tile_px;  // shapes that do not divide the tile fall back to pixel runs
    ctx->tune = n;
    return VXL_OK;
}

vxl_status vxl_ctx_get_tuning(const vxl_ctx* ctx, vxl_tuning* out) {
    if (!ctx || !out) return fail(VXL_ERR_INVALID_ARG, "ctx_get_tuning: NULL argument");
    *out = ctx->tune;
    return VXL_OK;
}

vxl_status vxl_grid_create(vxl_ctx* ctx, int nx, int ny, int nz, vxl_grid** out) {
    if (!ctx || !out) return fail(VXL_ERR_INVALID_ARG, "grid_create: NULL argument");
    *out = nullptr;
    if (nx < 2 || ny < 2 || nz < 2 || (nx & 1) || (ny & 1) || (nz & 1) || nx > 32768 || ny > 32768 || nz > 32768)
        return fail(VXL_ERR_INVALID_ARG, "grid_create: dims %dx%dx%d must be even and in [2, 32768]", nx, ny, nz);
    // bricks cover cells [0, n+1] (the DDA's inclusive bound): ceil(n/4) + 1 per axis
    int bx = (nx + 3) / 4 + 1, by = (ny + 3) / 4 + 1, bz = (nz + 3) / 4 + 1;
    int tx = (bx + 1) / 2, ty = (by + 1) / 2, tz = (bz + 1) / 2;
    unsigned long long nbricks = (unsigned long long)bx * by * bz;
    unsigned long long ntiles = (unsigned long long)tx * ty * tz;
    if (nbricks >= (1ull << 32))
        return fail(VXL_ERR_OUT_OF_RANGE, "grid_create: %dx%dx%d needs more than 2^32 brick words", nx, ny, nz);
    VXL_TRY(set_device(ctx));
    vxl_grid* g = new (std::nothrow) vxl_grid();
    if (!g) return fail(VXL_ERR_OOM, "grid_create: host allocation");
    g->ctx = ctx;
    g->device = ctx->device;
    g->nx = nx;
    g->ny = ny;
    g->nz = nz;
    g->bx = bx;
    g->by = by;
    g->bz = bz;
    g->tx = tx;
    g->ty = ty;
    g->tz = tz;
    g->nwords = (size_t)nbricks;
    g->nmask = (size_t)((ntiles + 31) / 32);
    trace_layout_dims(g);
    g->sx2 = (tx + 7) / 8;
    g->sy2 = (ty + 7) / 8;
    g->sz2 = (tz + 7) / 8;
    g->nclear2 = ((size_t)g->sx2 * g->sy2 * g->sz2 + 31) / 32;
    cudaError_t e = cudaMalloc(&g->words, g->nwords * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&g->tmask, g->nmask * sizeof(uint32_t));
    const bool maps = !g->tl_nwords || g->tl_wide;  // the exact-step kernel's two-level map of empty space
    if (e == cudaSuccess && maps) e = cudaMalloc(&g->clear1, g->nmask * sizeof(uint32_t));
    if (e == cudaSuccess && maps) e = cudaMalloc(&g->clear2, g->nclear2 * sizeof(uint32_t));
    if (e == cudaSuccess && g->tl_nwords) {
        e = cudaMalloc(&g->tl_words, g->tl_nwords * sizeof(uint64_t));
        if (e == cudaErrorMemoryAllocation && g->tl_wide) {
            // the wide layout is 4x the grid's own words (4.3 GB at 2048^3): without room for it the grid is
            // traced on its own words by the exact-step kernel, whose maps are allocated above
            (void)cudaGetLastError();
            g->tl_words = nullptr;
            g->tl_nwords = 0;
            g->tl_wide = 0;
            e = cudaSuccess;
        }
    }
    if (e == cudaSuccess) e = cudaMemset(g->words, 0, g->nwords * sizeof(uint64_t));
    if (e == cudaSuccess && g->tl_nwords) e = cudaMemset(g->tl_words, 0, g->tl_nwords * sizeof(uint64_t));
    if (e != cudaSuccess) {
        if (g->words) cudaFree(g->words);
        if (g->tmask) cudaFree(g->tmask);
        if (g->tl_words) cudaFree(g->tl_words);
        if (g->clear1) cudaFree(g->clear1);
        if (g->clear2) cudaFree(g->clear2);
        delete g;
        return cuda_fail(e, "grid_create: device allocation");
    }
    vxl_status st = launch_build_tile_mask(g, 0);
    if (st == VXL_OK) {
        e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) st = cuda_fail(e, "grid_create: build");
    }
    if (st != VXL_OK) {
        cudaFree(g->words);
        cudaFree(g->tmask);
        if (g->tl_words) cudaFree(g->tl_words);
        if (g->clear1) cudaFree(g->clear1);
        if (g->clear2) cudaFree(g->clear2);
        delete g;
        return st;
    }
    *out = g;
    return VXL_OK;
}

vxl_status vxl_grid_destroy(vxl_grid* g) {
    if (!g) return VXL_OK;
    cudaSetDevice(g->device);  // the context may already be gone
    cudaFree(g->words);
    cudaFree(g->tmask);
    if (g->tl_words) cudaFree(g->tl_words);
    if (g->clear1) cudaFree(g->clear1);
    if (g->clear2) cudaFree(g->clear2);
    if (g->pal4) cudaFree(g->pal4);
    delete g;
    return VXL_OK;
}

vxl_status vxl_grid_describe(const vxl_grid* g, vxl_grid_desc* out) {
    if (!grid_ok(g) || !out) return fail(VXL_ERR_INVALID_ARG, "grid_describe: NULL argument");
    out->nx = g->nx;
    out->ny = g->ny;
    out->nz = g->nz;
    out->bx = g->bx;
    out->by = g->by;
    out->bz = g->bz;
    out->tx = g->tx;
    out->ty = g->ty;
    out->tz = g->tz;
    out->words = g->words;
    out->words_bytes = g->nwords * sizeof(uint64_t);
    out->tile_mask = g->tmask;
    out->tile_mask_bytes = g->nmask * sizeof(uint32_t);
    out->trace_words = g->tl_words;
    out->trace_words_bytes = g->tl_nwords * sizeof(uint64_t);
    out->trace_lbx = g->tl_lbx;
    out->trace_lby = g->tl_lby;
    out->trace_bz = g->tl_bz;
    out->trace_wide = g->tl_wide;
    return VXL_OK;
}

vxl_status vxl_grid_clear(vxl_grid* g, void* stream) {
    if (!grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "grid_clear: bad grid");
    VXL_TRY(set_device(g->ctx));
    VXL_TRY_CUDA(cudaMemsetAsync(g->words, 0, g->nwords * sizeof(uint64_t), (cudaStream_t)stream));
    if (g->pal4) VXL_TRY_CUDA(cudaMemsetAsync(g->pal4, 0, 4 * g->nwords * sizeof(uint64_t), (cudaStream_t)stream));
    return launch_build_tile_mask(g, (cudaStream_t)stream);
}

vxl_status vxl_grid_build_bricks(vxl_grid* g, void* stream) {
    if (!grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "grid_build_bricks: bad grid");
    VXL_TRY(set_device(g->ctx));
    return launch_build_tile_mask(g, (cudaStream_t)stream);
}

vxl_status vxl_grid_import_r8(vxl_grid* g, const uint8_t* d_bytes, void* stream) {
    if (!grid_ok(g) || !d_bytes) return fail(VXL_ERR_INVALID_ARG, "grid_import_r8: NULL argument");
    VXL_TRY(set_device(g->ctx));
    return launch_grid_import_r8(g, d_bytes, (cudaStream_t)stream);
}

vxl_status vxl_grid_export_r8(const vxl_grid* g, uint8_t* d_bytes, void* stream) {
    if (!grid_ok(g) || !d_bytes) return fail(VXL_ERR_INVALID_ARG, "grid_export_r8: NULL argument");
    VXL_TRY(set_device(g->ctx));
    return launch_grid_export_r8(g, d_bytes, (cudaStream_t)stream);
}

vxl_status vxl_grid_import_palette(vxl_grid* g, const uint8_t* d_palette, int opaque_min, void* stream) {
    if (!grid_ok(g) || !d_palette) return fail(VXL_ERR_INVALID_ARG, "grid_import_palette: NULL argument");
    if (opaque_min < 0 || opaque_min > 256) return fail(VXL_ERR_INVALID_ARG, "opaque_min out of [0,256]");
    VXL_TRY(set_device(g->ctx));
    return launch_grid_import_palette(g, d_palette, opaque_min, (cudaStream_t)stream);
}

vxl_status vxl_grid_palette_alloc(vxl_grid* g) {
    if (!grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "grid_palette_alloc: bad grid");
    if (g->pal4) return VXL_OK;
    VXL_TRY(set_device(g->ctx));
    const size_t bytes = 4 * g->nwords * sizeof(uint64_t);
    uint64_t* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) e = cudaMemset(p, 0, bytes);
    if (e != cudaSuccess) {
        if (p) cudaFree(p);
        return cuda_fail(e, "grid_palette_alloc: device allocation");
    }
    g->pal4 = p;
    return VXL_OK;
}

vxl_status vxl_grid_export_palette(const vxl_grid* g, uint8_t* d_out, void* stream) {
    if (!grid_ok(g) || !d_out) return fail(VXL_ERR_INVALID_ARG, "grid_export_palette: NULL argument");
    if (!g->pal4) return fail(VXL_ERR_NOT_SUPPORTED, "grid_export_palette: the grid has no palette plane");
    VXL_TRY(set_device(g->ctx));
    return launch_grid_export_palette(g, d_out, (cudaStream_t)stream);
}

vxl_status vxl_grid_count(const vxl_grid* g, uint64_t* out, void* stream) {
    if (!grid_ok(g) || !out) return fail(VXL_ERR_INVALID_ARG, "grid_count: NULL argument");
    VXL_TRY(set_device(g->ctx));
    cudaStream_t s = (cudaStream_t)stream;
    void* scratch;
    VXL_TRY(ctx_scratch(g->ctx, 256, &scratch));
    VXL_TRY_CUDA(cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), s));
    VXL_TRY(launch_grid_count(g, (unsigned long long*)scratch, s));
    unsigned long long h = 0;
    VXL_TRY_CUDA(cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, s));
    VXL_TRY_CUDA(cudaStreamSynchronize(s));
    *out = h;
    return VXL_OK;
}

vxl_status vxl_trace_rays(vxl_ctx* ctx, const vxl_grid* g, const float* d_rays, int64_t n, vxl_mode mode,
                          vxl_ray_record* d_records, void* stream) {
    if (!ctx || !grid_ok(g) || (n > 0 && (!d_rays || !d_records)))
        return fail(VXL_ERR_INVALID_ARG, "trace_rays: NULL argument");
    if (n < 0) return fail(VXL_ERR_INVALID_ARG, "trace_rays: n < 0");
    if (mode != VXL_MODE_DDA && mode != VXL_MODE_SPARSE && mode != VXL_MODE_SUPERSPARSE)
        return fail(VXL_ERR_INVALID_ARG, "trace_rays: unknown mode %d", (int)mode);
    VXL_TRY(set_device(ctx));
    return launch_trace_rays(ctx, g, d_rays, n, (int)mode, d_records, (cudaStream_t)stream);
}

vxl_status vxl_trace_occlusion(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p,
                               const vxl_outputs* out, void* stream) {
    if (!ctx || !grid_ok(g) || !gb || !out) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion: NULL argument");
    VXL_TRY(check_params(p));
    if (gb->npix < 0) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion: npix < 0");
    if (gb->npix > 0 && (!gb->pos || !gb->nrm)) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion: NULL G-buffer");
    VXL_TRY(set_device(ctx));
    return launch_trace_occlusion(ctx, g, gb, p, out, (cudaStream_t)stream);
}

vxl_status vxl_trace_occlusion_from_depth(vxl_ctx* ctx, const vxl_grid* g, const float* d_depth, const float* d_nrm,
                                          const float* d_rough, int32_t width, int32_t height, const vxl_view* view,
                                          const vxl_trace_params* p, const vxl_outputs* out, void* stream) {
    if (!ctx || !grid_ok(g) || !view || !out) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion_from_depth: NULL argument");
    VXL_TRY(check_params(p));
    if (width < 0 || height < 0) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion_from_depth: bad image size");
    const int64_t npix = (int64_t)width * height;
    if (npix == 0) return VXL_OK;
    if (!d_depth || !d_nrm) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion_from_depth: NULL G-buffer");
    VXL_TRY(set_device(ctx));
    cudaStream_t s = (cudaStream_t)stream;
    VXL_TRY(ctx_grow(&ctx->d_fd, &ctx->fd_bytes, (size_t)npix * 6 * sizeof(float)));
    float* wcp = (float*)ctx->d_fd;
    float* nrm = wcp + 3 * npix;
    VXL_TRY(launch_rebuild_from_depth(ctx, d_depth, d_nrm, width, height, view, wcp, nrm, s));
    const vxl_gbuffer gb{wcp, nrm, d_rough, npix, width, height};
    return launch_trace_occlusion(ctx, g, &gb, p, out, s);
}

vxl_status vxl_trace_occlusion_host(vxl_ctx* ctx, const vxl_grid* g, const float* h_pos, const float* h_nrm,
                                    const float* h_rough, int64_t npix, const vxl_trace_params* p, float* h_shadow,
                                    float* h_ao, float* h_ao_vis, float* h_spec, float* h_spec_t, void* stream) {
    if (!ctx || !grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion_host: NULL argument");
    VXL_TRY(check_params(p));
    if (npix < 0 || (npix > 0 && (!h_pos || !h_nrm))) return fail(VXL_ERR_INVALID_ARG, "trace_occlusion_host: bad G-buffer");
    if (npix == 0) return VXL_OK;
    VXL_TRY(set_device(ctx));
    cudaStream_t s = (cudaStream_t)stream;
    // Pinned host memory is mapped into the device's address space; over the
    // coherent CPU-GPU link the kernel then reads the G-buffer and writes the
    // outputs in place, with no copy stages. Any other buffer (pageable memory)
    // takes the staged copy pipeline below.
    {
        const float* in[3] = {h_pos, h_nrm, h_rough};
        float* out[5] = {h_shadow, h_ao, h_ao_vis, h_spec, h_spec_t};
        const float* din[3] = {nullptr, nullptr, nullptr};
        float* dout[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        bool mapped = true;
        for (int k = 0; k < 3 && mapped; k++)
            if (in[k]) mapped = device_view(ctx, in[k], (void**)&din[k]);
        for (int k = 0; k < 5 && mapped; k++)
            if (out[k]) mapped = device_view(ctx, out[k], (void**)&dout[k]);
        if (mapped && occl_pool_supported(g, p)) {
            vxl_gbuffer gb{din[0], din[1], din[2], npix, 0, 0};
            vxl_outputs o{dout[0], dout[1], dout[2], dout[3], dout[4], nullptr};
            VXL_TRY(launch_trace_occlusion(ctx, g, &gb, p, &o, s));
            VXL_TRY_CUDA(cudaStreamSynchronize(s));
            return VXL_OK;
        }
    }
    const size_t b3 = (size_t)npix * 3 * sizeof(float), b1 = (size_t)npix * sizeof(float);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t need = 2 * al(b3) + 6 * al(b1);
    void* st;
    VXL_TRY(ctx_stage(ctx, need, &st));
    char* base = (char*)st;
    float* d_pos = (float*)base;
    float* d_nrm = (float*)(base + al(b3));
    float* d_rough = (float*)(base + 2 * al(b3));
    float* outs[5];
    for (int k = 0; k < 5; k++) outs[k] = (float*)(base + 2 * al(b3) + (k + 1) * al(b1));
    float* hs[5] = {h_shadow, h_ao, h_ao_vis, h_spec, h_spec_t};
    // Large frames run as a pipeline of pixel chunks on two streams, so the
    // copies of one chunk overlap the tracing of its neighbours. A pixel's
    // outputs depend only on its own rays, and the ray generator is seeded with
    // the global pixel index (pix_base), so the result equals the one-launch form.
    const int64_t kChunkMin = 1 << 18;
    if (!occl_pool_supported(g, p) || npix < 2 * kChunkMin || npix > (int64_t)UINT32_MAX) {
        VXL_TRY_CUDA(cudaMemcpyAsync(d_pos, h_pos, b3, cudaMemcpyHostToDevice, s));
        VXL_TRY_CUDA(cudaMemcpyAsync(d_nrm, h_nrm, b3, cudaMemcpyHostToDevice, s));
        if (h_rough) VXL_TRY_CUDA(cudaMemcpyAsync(d_rough, h_rough, b1, cudaMemcpyHostToDevice, s));
        vxl_gbuffer gb{d_pos, d_nrm, h_rough ? d_rough : nullptr, npix, 0, 0};
        vxl_outputs o{hs[0] ? outs[0] : nullptr, hs[1] ? outs[1] : nullptr, hs[2] ? outs[2] : nullptr,
                      hs[3] ? outs[3] : nullptr, hs[4] ? outs[4] : nullptr, nullptr};
        VXL_TRY(launch_trace_occlusion(ctx, g, &gb, p, &o, s));
        for (int k = 0; k < 5; k++)
            if (hs[k]) VXL_TRY_CUDA(cudaMemcpyAsync(hs[k], outs[k], b1, cudaMemcpyDeviceToHost, s));
        VXL_TRY_CUDA(cudaStreamSynchronize(s));
        return VXL_OK;
    }
    if (!ctx->pipe_ready) {
        for (int k = 0; k < 2; k++) VXL_TRY_CUDA(cudaStreamCreateWithFlags(&ctx->pipe[k], cudaStreamNonBlocking));
        VXL_TRY_CUDA(cudaEventCreateWithFlags(&ctx->pipe_start, cudaEventDisableTiming));
        ctx->pipe_ready = true;
    }
    // the chunks start after the work already queued on the caller's stream
    VXL_TRY_CUDA(cudaEventRecord(ctx->pipe_start, s));
    for (int k = 0; k < 2; k++) VXL_TRY_CUDA(cudaStreamWaitEvent(ctx->pipe[k], ctx->pipe_start, 0));
    // chunk sizes ramp up and down: the first chunk's copy and the last
    // chunk's read-back are the parts no tracing overlaps
    static const int kRamp[] = {1, 5, 8, 5, 1};
    constexpr int kRampN = (int)(sizeof(kRamp) / sizeof(kRamp[0]));
    int64_t wsum = 0;
    for (int k = 0; k < kRampN; k++) wsum += kRamp[k];
    int64_t bounds[kRampN + 1];
    bounds[0] = 0;
    for (int k = 0, acc = 0; k < kRampN; k++) {
        acc += kRamp[k];
        const int64_t b = k == kRampN - 1 ? npix : (((npix * acc / wsum) + 1023) & ~(int64_t)1023);
        bounds[k + 1] = std::min(std::max(b, bounds[k]), npix);
    }
    for (int ci = 0; ci < kRampN; ci++) {
        const int64_t p0 = bounds[ci], n = bounds[ci + 1] - bounds[ci];
        if (n <= 0) continue;
        cudaStream_t cs = ctx->pipe[ci & 1];
        VXL_TRY_CUDA(cudaMemcpyAsync(d_pos + 3 * p0, h_pos + 3 * p0, (size_t)n * 12, cudaMemcpyHostToDevice, cs));
        VXL_TRY_CUDA(cudaMemcpyAsync(d_nrm + 3 * p0, h_nrm + 3 * p0, (size_t)n * 12, cudaMemcpyHostToDevice, cs));
        if (h_rough)
            VXL_TRY_CUDA(cudaMemcpyAsync(d_rough + p0, h_rough + p0, (size_t)n * 4, cudaMemcpyHostToDevice, cs));
        vxl_gbuffer gb{d_pos + 3 * p0, d_nrm + 3 * p0, h_rough ? d_rough + p0 : nullptr, n, 0, 0};
        vxl_outputs o{hs[0] ? outs[0] + p0 : nullptr, hs[1] ? outs[1] + p0 : nullptr, hs[2] ? outs[2] + p0 : nullptr,
                      hs[3] ? outs[3] + p0 : nullptr, hs[4] ? outs[4] + p0 : nullptr, nullptr};
        unsigned long long* counter = nullptr;
        VXL_TRY(ctx_take_counter(ctx, cs, &counter));
        VXL_TRY(launch_trace_occlusion_pool(ctx, g, &gb, p, &o, counter, ctx->tune, cs,
                                            (uint32_t)p0));
        for (int k = 0; k < 5; k++)
            if (hs[k])
                VXL_TRY_CUDA(cudaMemcpyAsync(hs[k] + p0, outs[k] + p0, (size_t)n * 4, cudaMemcpyDeviceToHost, cs));
    }
    for (int k = 0; k < 2; k++) VXL_TRY_CUDA(cudaStreamSynchronize(ctx->pipe[k]));
    return VXL_OK;
}

}  // extern "C"

struct vxl_batch {
    vxl_ctx* ctx;
    void* d_table;
    unsigned long long* d_counter;
    int n, max_r;
    int64_t tiles, rays;
    size_t max_grid_bytes;
    vxl_tuning tune;
    bool lean;  // traced on the grids' trace layouts (k_occl_lean_batch)
    std::vector<unsigned char> h_table;  // host copy of the scene table
    cudaStream_t cap_stream;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

extern "C" {

vxl_status vxl_batch_create(vxl_ctx* ctx, const vxl_batch_item* items, int n, int use_graph, vxl_batch** out) {
    if (!ctx || !out || n <= 0 || !items) return fail(VXL_ERR_INVALID_ARG, "batch_create: bad argument");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        const vxl_batch_item& it = items[i];
        if (!grid_ok(it.grid)) return fail(VXL_ERR_INVALID_ARG, "batch item %d: bad grid", i);
        if (it.grid->ctx != ctx) return fail(VXL_ERR_INVALID_ARG, "batch item %d: grid of another context", i);
        VXL_TRY(check_params(&it.params));
        if (it.gbuf.npix < 0 || (it.gbuf.npix > 0 && (!it.gbuf.pos || !it.gbuf.nrm)))
            return fail(VXL_ERR_INVALID_ARG, "batch item %d: bad G-buffer", i);
        if (it.out.records) return fail(VXL_ERR_INVALID_ARG, "batch item %d: records are not supported in a batch", i);
        if (!occl_pool_supported(it.grid, &it.params))
            return fail(VXL_ERR_NOT_SUPPORTED, "batch item %d: more than 31 rays per pixel or grid above 32760", i);
    }
    VXL_TRY(set_device(ctx));
    vxl_batch* b = new (std::nothrow) vxl_batch();
    if (!b) return fail(VXL_ERR_OOM, "batch_create: host allocation");
    b->ctx = ctx;
    b->n = n;
    b->tune = ctx->tune;
    b->lean = lean_batch_supported(items, n, b->tune);
    std::vector<unsigned char> table;
    if (b->lean) {
        b->tune = lean_batch_tuning(ctx, items, n, b->tune);
        table.resize((size_t)n * lean_batch_desc_bytes());
        lean_batch_build_table(items, n, b->tune, table.data(), &b->max_r, &b->tiles, &b->rays);
    } else {
        table.resize((size_t)n * batch_desc_bytes());
        batch_build_table(items, n, b->tune, table.data(), &b->max_r, &b->tiles, &b->rays, &b->max_grid_bytes);
    }
    auto cleanup = [b]() {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
        if (b->d_table) cudaFree(b->d_table);
        if (b->d_counter) cudaFree(b->d_counter);
        delete b;
    };
    cudaError_t e = cudaMalloc(&b->d_table, table.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_table, table.data(), table.size(), cudaMemcpyHostToDevice);
    b->h_table = table;
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "batch_create: device table");
    }
    if (use_graph) {
        e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_fail(e, "batch_create: begin capture");
        }
        vxl_status st = b->lean ? launch_lean_batch(ctx, b->d_table, b->h_table.data(), n, b->max_r, b->tiles, b->tune,
                                                    b->d_counter, b->cap_stream)
                                : launch_batch(ctx, b->d_table, n, b->max_r, b->tiles, b->tune, b->d_counter,
                                               b->max_grid_bytes, b->cap_stream);
        ctx->launches--;  // captured, not run
        e = cudaStreamEndCapture(b->cap_stream, &b->graph);
        if (st != VXL_OK || e != cudaSuccess) {
            cleanup();
            return st != VXL_OK ? st : cuda_fail(e, "batch_create: end capture");
        }
        e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_fail(e, "batch_create: graph instantiate");
        }
    }
    *out = b;
    return VXL_OK;
}

vxl_status vxl_batch_run(vxl_batch* b, void* stream) {
    if (!b) return fail(VXL_ERR_INVALID_ARG, "batch_run: NULL batch");
    VXL_TRY(set_device(b->ctx));
    cudaStream_t s = (cudaStream_t)stream;
    if (b->exec) {
        VXL_TRY_CUDA(cudaGraphLaunch(b->exec, s));
        b->ctx->launches++;
        return VXL_OK;
    }
    if (b->lean)
        return launch_lean_batch(b->ctx, b->d_table, b->h_table.data(), b->n, b->max_r, b->tiles, b->tune, b->d_counter,
                                 s);
    return launch_batch(b->ctx, b->d_table, b->n, b->max_r, b->tiles, b->tune, b->d_counter, b->max_grid_bytes, s);
}

vxl_status vxl_batch_destroy(vxl_batch* b) {
    if (!b) return VXL_OK;
    cudaSetDevice(b->ctx->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    cudaFree(b->d_table);
    cudaFree(b->d_counter);
    delete b;
    return VXL_OK;
}

vxl_status vxl_batch_info(const vxl_batch* b, int64_t* tiles, int64_t* rays) {
    if (!b) return fail(VXL_ERR_INVALID_ARG, "batch_info: NULL batch");
    if (tiles) *tiles = b->tiles;
    if (rays) *rays = b->rays;
    return VXL_OK;
}

vxl_status vxl_light_ambient(vxl_ctx* ctx, const vxl_grid* g, const float* d_wcp, const float* d_nrm,
                             const float* d_depth, const float* d_noise, int64_t npix, float* d_shadow,
                             float* d_irradiance, vxl_ray_record* d_records, void* stream) {
    if (!ctx || !grid_ok(g) || npix < 0) return fail(VXL_ERR_INVALID_ARG, "light_ambient: bad argument");
    if (npix > 0 && (!d_wcp || !d_nrm || !d_depth || !d_noise || !d_shadow || !d_irradiance))
        return fail(VXL_ERR_INVALID_ARG, "light_ambient: NULL buffer");
    VXL_TRY(set_device(ctx));
    return launch_light_ambient(ctx, g, d_wcp, d_nrm, d_depth, d_noise, npix, d_shadow, d_irradiance, d_records,
                                (cudaStream_t)stream);
}

vxl_status vxl_light_reflection(vxl_ctx* ctx, const vxl_grid* g, const float* d_wcp, const float* d_nrm,
                                const float* d_view_r, const float* d_rough, const float* d_noise, int64_t npix,
                                float* d_t, vxl_ray_record* d_records, void* stream) {
    if (!ctx || !grid_ok(g) || npix < 0) return fail(VXL_ERR_INVALID_ARG, "light_reflection: bad argument");
    if (npix > 0 && (!d_wcp || !d_nrm || !d_view_r || !d_rough || !d_noise || !d_t))
        return fail(VXL_ERR_INVALID_ARG, "light_reflection: NULL buffer");
    VXL_TRY(set_device(ctx));
    return launch_light_reflection(ctx, g, d_wcp, d_nrm, d_view_r, d_rough, d_noise, npix, d_t, d_records,
                                   (cudaStream_t)stream);
}

vxl_status vxl_light_point(vxl_ctx* ctx, const vxl_grid* g, const float* d_wpos, const float* d_nrm,
                           const float* d_noise, int64_t npix, const float light_pos[3], float range, int spot,
                           float* d_shadow, vxl_ray_record* d_records, void* stream) {
    if (!ctx || !grid_ok(g) || npix < 0 || !light_pos) return fail(VXL_ERR_INVALID_ARG, "light_point: bad argument");
    if (npix > 0 && (!d_wpos || !d_nrm || !d_noise || !d_shadow))
        return fail(VXL_ERR_INVALID_ARG, "light_point: NULL buffer");
    VXL_TRY(set_device(ctx));
    return launch_light_point(ctx, g, d_wpos, d_nrm, d_noise, npix, light_pos, range, spot ? 1 : 0, d_shadow,
                              d_records, (cudaStream_t)stream);
}

vxl_status vxl_light_taa(vxl_ctx* ctx, const vxl_taa_frame* f, float* d_out, void* stream) {
    if (!ctx || !f || !d_out) return fail(VXL_ERR_INVALID_ARG, "light_taa: NULL argument");
    if (!f->light || !f->last_light || !f->color || !f->normal || !f->material || !f->depth || !f->motion ||
        !f->noise)
        return fail(VXL_ERR_INVALID_ARG, "light_taa: NULL image");
    if (f->width < 1 || f->height < 1 || (int64_t)f->width * f->height > (int64_t)INT32_MAX / 4)
        return fail(VXL_ERR_INVALID_ARG, "light_taa: bad image size");
    if (((uintptr_t)f->light | (uintptr_t)f->last_light | (uintptr_t)f->material) & 15u ||
        ((uintptr_t)f->motion & 7u))
        return fail(VXL_ERR_INVALID_ARG, "light_taa: 4-channel images must be 16-byte and motion 8-byte aligned");
    VXL_TRY(set_device(ctx));
    return launch_light_taa(ctx, f, d_out, (cudaStream_t)stream);
}

vxl_status vxl_light_points(vxl_ctx* ctx, const vxl_grid* g, const float* d_wpos, const float* d_nrm,
                            const float* d_noise, int64_t npix, const vxl_light* lights, int nlights,
                            uint64_t* d_lit, uint64_t* d_in_range, void* stream) {
    if (!ctx || !grid_ok(g) || npix < 0 || nlights < 0 || nlights > 64 || (nlights > 0 && !lights))
        return fail(VXL_ERR_INVALID_ARG, "light_points: bad argument (at most 64 lights)");
    if (npix > 0 && (!d_wpos || !d_nrm || !d_noise || !d_lit))
        return fail(VXL_ERR_INVALID_ARG, "light_points: NULL buffer");
    for (int l = 0; l < nlights; l++)
        if (!std::isfinite(lights[l].range) || !std::isfinite(lights[l].pos[0]) || !std::isfinite(lights[l].pos[1]) ||
            !std::isfinite(lights[l].pos[2]))
            return fail(VXL_ERR_INVALID_ARG, "light_points: light %d is not finite", l);
    VXL_TRY(set_device(ctx));
    return launch_light_points(ctx, g, d_wpos, d_nrm, d_noise, npix, lights, nlights,
                               reinterpret_cast<unsigned long long*>(d_lit),
                               reinterpret_cast<unsigned long long*>(d_in_range), (cudaStream_t)stream);
}

vxl_status vxl_voxelize(vxl_ctx* ctx, vxl_grid* g, const vxl_model* models, int nmodels,
                        const vxl_instance* instances, int n, int32_t* d_aabb, void* stream) {
    if (!ctx || !grid_ok(g) || n < 0 || (n > 0 && !instances)) return fail(VXL_ERR_INVALID_ARG, "voxelize: bad argument");
    VXL_TRY(check_models(models, nmodels));
    std::vector<DevInstance> inst((size_t)n);
    for (int i = 0; i < n; i++) {
        const vxl_instance& a = instances[i];
        if (a.model < 0 || a.model >= nmodels) return fail(VXL_ERR_INVALID_ARG, "instance %d: model %d of %d", i, a.model, nmodels);
        if (a.op != VXL_OP_SET && a.op != VXL_OP_CLEAR) return fail(VXL_ERR_INVALID_ARG, "instance %d: bad op", i);
        std::memcpy(inst[i].m, a.matrix, sizeof inst[i].m);
        inst[i].model = a.model;
        inst[i].op = a.op;
    }
    VXL_TRY(set_device(ctx));
    return voxelize_runs(ctx, g, models, nmodels, inst, d_aabb, (cudaStream_t)stream);
}

vxl_status vxl_shadowvox_update(vxl_ctx* ctx, vxl_grid* g, const vxl_model* models, int nmodels,
                                const vxl_entity* ents, int n, int32_t* h_regions, void* stream) {
    if (!ctx || !grid_ok(g) || n < 0 || (n > 0 && !ents)) return fail(VXL_ERR_INVALID_ARG, "shadowvox_update: bad argument");
    VXL_TRY(check_models(models, nmodels));
    if (n == 0) return VXL_OK;
    std::vector<DevInstance> inst((size_t)2 * n);
    for (int e = 0; e < n; e++) {
        const vxl_entity& E = ents[e];
        if (E.model < 0 || E.model >= nmodels) return fail(VXL_ERR_INVALID_ARG, "entity %d: model %d of %d", e, E.model, nmodels);
        float np[3] = {-E.pivot[0], -E.pivot[1], -E.pivot[2]};
        translate(E.prev_world, np, inst[2 * e].m);
        inst[2 * e].model = E.model;
        inst[2 * e].op = VXL_OP_CLEAR;
        translate(E.world, np, inst[2 * e + 1].m);
        inst[2 * e + 1].model = E.model;
        inst[2 * e + 1].op = VXL_OP_SET;
    }
    VXL_TRY(set_device(ctx));
    cudaStream_t s = (cudaStream_t)stream;
    const int sx = g->nx / 2, sy = g->ny / 2, sz = g->nz / 2;
    // per-instance aabb, started at (S-1,S-1,S-1)/(0,0,0) (ShadowVoxSystem.cpp:128-132);
    // the two instances of an entity are folded together on the host
    std::vector<int32_t> h_aabb((size_t)12 * n);
    for (int k = 0; k < 2 * n; k++) {
        int32_t* a = &h_aabb[(size_t)6 * k];
        a[0] = sx - 1;
        a[1] = sy - 1;
        a[2] = sz - 1;
        a[3] = a[4] = a[5] = 0;
    }
    void* st;
    VXL_TRY(ctx_stage(ctx, h_aabb.size() * sizeof(int32_t), &st));
    VXL_TRY_CUDA(cudaMemcpyAsync(st, h_aabb.data(), h_aabb.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    VXL_TRY(voxelize_runs(ctx, g, models, nmodels, inst, (int32_t*)st, s));
    VXL_TRY_CUDA(cudaMemcpyAsync(h_aabb.data(), st, h_aabb.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    VXL_TRY_CUDA(cudaStreamSynchronize(s));
    if (h_regions) {
        for (int e = 0; e < n; e++) {
            const int32_t* a = &h_aabb[(size_t)12 * e];
            const int32_t* b = a + 6;
            int m[6];
            for (int c = 0; c < 3; c++) {
                m[c] = a[c] < b[c] ? a[c] : b[c];
                m[3 + c] = a[3 + c] > b[3 + c] ? a[3 + c] : b[3 + c];
            }
            region_from_aabb(m, sx, sy, sz, h_regions + 6 * (size_t)e);
        }
    }
    return VXL_OK;
}

vxl_status vxl_vox_destroyed(vxl_ctx* ctx, vxl_grid* g, const vxl_model* model, const float world[16],
                             int32_t* h_region, void* stream) {
    if (!ctx || !grid_ok(g) || !model || !world) return fail(VXL_ERR_INVALID_ARG, "vox_destroyed: NULL argument");
    VXL_TRY(check_models(model, 1));
    VXL_TRY(set_device(ctx));
    cudaStream_t s = (cudaStream_t)stream;
    const int sx = g->nx / 2, sy = g->ny / 2, sz = g->nz / 2;
    std::vector<DevInstance> inst(1);
    std::memcpy(inst[0].m, world, sizeof inst[0].m);
    inst[0].model = 0;
    inst[0].op = VXL_OP_CLEAR;
    int32_t h_aabb[6] = {sx - 1, sy - 1, sz - 1, 0, 0, 0};
    void* st;
    VXL_TRY(ctx_stage(ctx, sizeof h_aabb, &st));
    VXL_TRY_CUDA(cudaMemcpyAsync(st, h_aabb, sizeof h_aabb, cudaMemcpyHostToDevice, s));
    VXL_TRY(voxelize_runs(ctx, g, model, 1, inst, (int32_t*)st, s));
    VXL_TRY_CUDA(cudaMemcpyAsync(h_aabb, st, sizeof h_aabb, cudaMemcpyDeviceToHost, s));
    VXL_TRY_CUDA(cudaStreamSynchronize(s));
    if (h_region) region_from_aabb(h_aabb, sx, sy, sz, h_region);
    return VXL_OK;
}

vxl_status vxl_read_v(const char* path, int32_t* sx, int32_t* sy, int32_t* sz, uint8_t* h_data, size_t capacity) {
    if (!path || !sx || !sy || !sz) return fail(VXL_ERR_INVALID_ARG, "read_v: NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(VXL_ERR_IO, "read_v: cannot open %s", path);
    uint32_t d[3];
    if (std::fread(d, sizeof(uint32_t), 3, f) != 3) {
        std::fclose(f);
        return fail(VXL_ERR_IO, "read_v: %s: truncated header", path);
    }
    if (d[0] == 0 || d[1] == 0 || d[2] == 0 || (unsigned long long)d[0] * d[1] * d[2] > (1ull << 30)) {
        std::fclose(f);
        return fail(VXL_ERR_IO, "read_v: %s: implausible size %ux%ux%u", path, d[0], d[1], d[2]);
    }
    *sx = (int32_t)d[0];
    *sy = (int32_t)d[1];
    *sz = (int32_t)d[2];
    size_t n = (size_t)d[0] * d[1] * d[2];
    if (!h_data) {
        std::fclose(f);
        return VXL_OK;
    }
    if (capacity < n) {
        std::fclose(f);
        return fail(VXL_ERR_INVALID_ARG, "read_v: capacity %zu < %zu", capacity, n);
    }
    size_t got = std::fread(h_data, 1, n, f);
    std::fclose(f);
    if (got != n) return fail(VXL_ERR_IO, "read_v: %s: truncated body (%zu of %zu bytes)", path, got, n);
    return VXL_OK;
}

vxl_status vxl_scene_noise(vxl_ctx* ctx, vxl_grid* g, uint32_t seed, float thresh, float freq, int ground_y,
                           void* stream) {
    if (!ctx || !grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "scene_noise: bad argument");
    VXL_TRY(set_device(ctx));
    return launch_scene_noise(g, seed, thresh, freq, ground_y, (cudaStream_t)stream);
}

// soft grid dims: even (the walk's upper bound is dims + 1, as for the bit
// grid), voxel indices fit an int32
static vxl_status check_soft_grid(const float* soft, int nx, int ny, int nz, const char* who) {
    if (!soft) return fail(VXL_ERR_INVALID_ARG, "%s: NULL soft grid", who);
    if (((uintptr_t)soft & 15u) != 0) return fail(VXL_ERR_INVALID_ARG, "%s: soft grid not 16-byte aligned", who);
    if (nx < 2 || ny < 2 || nz < 2 || (nx & 1) || (ny & 1) || (nz & 1))
        return fail(VXL_ERR_INVALID_ARG, "%s: dims must be even and >= 2", who);
    if ((int64_t)nx * ny * nz > (int64_t)INT32_MAX || nx > 32760 || ny > 32760 || nz > 32760)
        return fail(VXL_ERR_OUT_OF_RANGE, "%s: soft grid too large", who);
    return VXL_OK;
}

static vxl_status check_soft_call(const vxl_gbuffer* gb, const vxl_soft_params* p, const char* who) {
    if (!gb || !p) return fail(VXL_ERR_INVALID_ARG, "%s: NULL argument", who);
    if (gb->npix < 0 || gb->npix > (int64_t)INT32_MAX - 32) return fail(VXL_ERR_INVALID_ARG, "%s: bad npix", who);
    if (gb->npix > 0 && (!gb->pos || !gb->nrm)) return fail(VXL_ERR_INVALID_ARG, "%s: NULL G-buffer", who);
    if (p->n_shadow < 0 || p->n_shadow > 1 || p->n_ao < 0 || p->n_shadow + p->n_ao < 1 ||
        p->n_shadow + p->n_ao > 32)
        return fail(VXL_ERR_INVALID_ARG, "%s: need n_shadow in {0,1} and 1 <= n_shadow + n_ao <= 32", who);
    if (!(p->len >= 0.0f) || !std::isfinite(p->len) || !std::isfinite(p->bias))
        return fail(VXL_ERR_INVALID_ARG, "%s: len and bias must be finite, len >= 0", who);
    return VXL_OK;
}

vxl_status vxl_trace_soft_fwd(vxl_ctx* ctx, const float* d_soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                              const vxl_soft_params* p, float* d_image, float* d_light, void* stream) {
    if (!ctx) return fail(VXL_ERR_INVALID_ARG, "trace_soft_fwd: NULL context");
    VXL_TRY(check_soft_grid(d_soft, nx, ny, nz, "trace_soft_fwd"));
    VXL_TRY(check_soft_call(gb, p, "trace_soft_fwd"));
    if (gb->npix > 0 && !d_image) return fail(VXL_ERR_INVALID_ARG, "trace_soft_fwd: NULL image");
    VXL_TRY(set_device(ctx));
    return launch_soft_fwd(ctx, d_soft, nx, ny, nz, gb, p, d_image, d_light, (cudaStream_t)stream);
}

vxl_status vxl_trace_soft_bwd(vxl_ctx* ctx, const float* d_soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                              const vxl_soft_params* p, const float* d_grad_image, const float* d_light,
                              float* d_grad_soft, void* stream) {
    if (!ctx) return fail(VXL_ERR_INVALID_ARG, "trace_soft_bwd: NULL context");
    VXL_TRY(check_soft_grid(d_soft, nx, ny, nz, "trace_soft_bwd"));
    VXL_TRY(check_soft_call(gb, p, "trace_soft_bwd"));
    if (gb->npix > 0 && (!d_grad_image || !d_light || !d_grad_soft))
        return fail(VXL_ERR_INVALID_ARG, "trace_soft_bwd: NULL grad_image, light or grad_soft");
    if (((uintptr_t)d_grad_soft & 15u) != 0)
        return fail(VXL_ERR_INVALID_ARG, "trace_soft_bwd: grad_soft not 16-byte aligned");
    VXL_TRY(set_device(ctx));
    return launch_soft_bwd(ctx, d_soft, nx, ny, nz, gb, p, d_grad_image, d_light, d_grad_soft,
                           (cudaStream_t)stream);
}

vxl_status vxl_volume_build_mips(vxl_ctx* ctx, const uint8_t* d_mip0, int sx, int sy, int sz, uint8_t* d_mip1,
                                 uint8_t* d_mip2, void* stream) {
    if (!ctx || !d_mip0 || !d_mip1 || !d_mip2) return fail(VXL_ERR_INVALID_ARG, "volume_build_mips: NULL argument");
    if (sx < 4 || sy < 4 || sz < 4 || (int64_t)sx * sy * sz > (int64_t)INT32_MAX)
        return fail(VXL_ERR_INVALID_ARG, "volume_build_mips: sizes must be >= 4");
    VXL_TRY(set_device(ctx));
    return launch_volume_mips(ctx, d_mip0, sx, sy, sz, d_mip1, d_mip2, (cudaStream_t)stream);
}

vxl_status vxl_trace_primary(vxl_ctx* ctx, const vxl_volume* volumes, int nvolumes, const vxl_voxcmd* cmds, int ncmds,
                             const vxl_camera* cam, const vxl_primary_out* out, void* stream) {
    if (!ctx || !cam || !out) return fail(VXL_ERR_INVALID_ARG, "trace_primary: NULL argument");
    if (nvolumes < 0 || ncmds < 0 || (nvolumes > 0 && !volumes) || (ncmds > 0 && !cmds))
        return fail(VXL_ERR_INVALID_ARG, "trace_primary: bad volume or command table");
    if (cam->width < 1 || cam->height < 1 || (int64_t)cam->width * cam->height > (int64_t)INT32_MAX / 4)
        return fail(VXL_ERR_INVALID_ARG, "trace_primary: bad image size");
    if (!out->pos || !out->nrm) return fail(VXL_ERR_INVALID_ARG, "trace_primary: pos and nrm are required");
    {  // the screen-tile lists hold at most ncmds x tiles entries, counted in 32 bits
        const int64_t tiles = (int64_t)((cam->width + 15) / 16) * ((cam->height + 15) / 16);
        if ((int64_t)ncmds * tiles > (int64_t)INT32_MAX)
            return fail(VXL_ERR_INVALID_ARG, "trace_primary: %d commands x %lld screen tiles exceed 2^31 list entries",
                        ncmds, (long long)tiles);
    }
    for (int v = 0; v < nvolumes; v++) {
        const vxl_volume& V = volumes[v];
        if (!V.mip[0] || !V.mip[1] || !V.mip[2] || V.sx < 4 || V.sy < 4 || V.sz < 4 || V.sx > 32768 ||
            V.sy > 32768 || V.sz > 32768)
            return fail(VXL_ERR_INVALID_ARG, "trace_primary: volume %d: NULL mip or size < 4", v);
    }
    for (int k = 0; k < ncmds; k++)
        if (cmds[k].volume < 0 || cmds[k].volume >= nvolumes)
            return fail(VXL_ERR_OUT_OF_RANGE, "trace_primary: command %d names volume %d", k, cmds[k].volume);
    VXL_TRY(set_device(ctx));
    return launch_trace_primary(ctx, volumes, nvolumes, cmds, ncmds, cam, out, (cudaStream_t)stream);
}

vxl_status vxl_scene_soft(vxl_ctx* ctx, float* d_soft, int nx, int ny, int nz, uint32_t seed, float thresh,
                          float sharpness, float freq, int ground_y, uint32_t albedo_seed, void* stream) {
    if (!ctx) return fail(VXL_ERR_INVALID_ARG, "scene_soft: NULL context");
    VXL_TRY(check_soft_grid(d_soft, nx, ny, nz, "scene_soft"));
    VXL_TRY(set_device(ctx));
    return launch_scene_soft(ctx, d_soft, nx, ny, nz, seed, thresh, sharpness, freq, ground_y, albedo_seed,
                             (cudaStream_t)stream);
}

vxl_status vxl_scene_terrain(vxl_ctx* ctx, vxl_grid* g, uint32_t seed, float base, float amplitude, float freq,
                             int octaves, float* d_height, void* stream) {
    if (!ctx || !grid_ok(g) || octaves < 1 || octaves > 16 || !std::isfinite(base) || !std::isfinite(amplitude) ||
        !std::isfinite(freq))
        return fail(VXL_ERR_INVALID_ARG, "scene_terrain: bad argument");
    VXL_TRY(set_device(ctx));
    return launch_scene_terrain(g, seed, base, amplitude, freq, octaves, d_height, (cudaStream_t)stream);
}

vxl_status vxl_scene_palette(vxl_ctx* ctx, vxl_grid* g, uint32_t seed, void* stream) {
    if (!ctx || !grid_ok(g)) return fail(VXL_ERR_INVALID_ARG, "scene_palette: bad argument");
    if (!g->pal4) return fail(VXL_ERR_NOT_SUPPORTED, "scene_palette: the grid has no palette plane");
    VXL_TRY(set_device(ctx));
    return launch_scene_palette(g, seed, (cudaStream_t)stream);
}

vxl_status vxl_scene_boxes(vxl_ctx* ctx, vxl_grid* g, uint32_t seed, int nboxes, int smin, int smax, void* stream) {
    if (!ctx || !grid_ok(g) || nboxes < 0 || smin < 1 || smax < smin)
        return fail(VXL_ERR_INVALID_ARG, "scene_boxes: bad argument");
    VXL_TRY(set_device(ctx));
    return launch_scene_boxes(g, seed, nboxes, smin, smax, (cudaStream_t)stream);
}

vxl_status vxl_scene_gbuffer(vxl_ctx* ctx, const vxl_grid* g, const float cam[3], const float target[3],
                             float tan_half_fov, int W, int H, uint32_t seed, float* d_pos, float* d_nrm,
                             float* d_rough, void* stream) {
    if (!ctx || !grid_ok(g) || !cam || !target || W <= 0 || H <= 0 || !d_pos || !d_nrm || !d_rough)
        return fail(VXL_ERR_INVALID_ARG, "scene_gbuffer: bad argument");
    VXL_TRY(set_device(ctx));
    return launch_scene_gbuffer(g, cam, target, tan_half_fov, W, H, seed, d_pos, d_nrm, d_rough, (cudaStream_t)stream);
}

}  // extern "C"
