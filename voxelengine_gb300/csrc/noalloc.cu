// noalloc.cu — vxl_voxelize_noalloc: the ShadowVox voxelizer for callers that
// must not allocate device memory (a render or simulation loop that has
// committed its memory budget up front, code running inside a pool-managed
// engine, or work issued between frames where a cudaMalloc would stall the
// device). It needs no vxl_ctx and no vxl_grid handle: the caller passes the
// grid's descriptor and its own input and output buffers.
//
// Its only scratch, the instance and model tables the kernel reads, lives in
// the file-scope device array below: a fixed 1.2 MiB that every GPU which loads
// this library holds until the process exits. Host code cannot use the array's
// name as a device address, so the first call on each device looks the address
// up with cudaGetSymbolAddress (with that device current) and keeps it.
#include <climits>
#include <mutex>

#include "vxl_device.cuh"

namespace vxl {

constexpr size_t kNaInstBytes = (size_t)VXL_NOALLOC_MAX_INSTANCES * sizeof(DevInstance);
constexpr size_t kNaModelBytes = (size_t)VXL_NOALLOC_MAX_MODELS * sizeof(DevModel);
static __device__ __align__(256) unsigned char g_noalloc_tables[kNaInstBytes + kNaModelBytes];

static_assert(sizeof(vxl_instance) == sizeof(DevInstance), "vxl_instance and DevInstance must match");
static_assert(sizeof(vxl_model) == sizeof(DevModel), "vxl_model and DevModel must match");
static_assert(kNaInstBytes % 256 == 0, "model table alignment");

constexpr int kNaMaxDevices = 64;
static std::mutex g_na_mu;
static unsigned char* g_na_ptr[kNaMaxDevices];

// Device address of g_noalloc_tables on the current device (set up once per device).
static vxl_status noalloc_tables(unsigned char** out) {
    int dev = 0;
    VXL_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) return fail(VXL_ERR_NOT_SUPPORTED, "voxelize_noalloc: device %d", dev);
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_tables);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_tables)");
        g_na_ptr[dev] = (unsigned char*)p;
    }
    *out = g_na_ptr[dev];
    return VXL_OK;
}

// Same mapping as k_voxelize (ShadowVoxSystem.cpp:137-177: fine voxel
// ivec3((o + x*dx + y*dy + z*dz) * 10) for every model voxel with index >= 16,
// SetVolumeAt bounds :83), launched without a chunk table:
// blockIdx.y = instance first + y of a run with equal ops, blockIdx.x = chunk
// of kVoxChunk source voxels (blocks past the model's last chunk return at once).
__global__ void __launch_bounds__(256) k_voxelize_na(GridView g, unsigned long long* words,
                                                     const DevInstance* __restrict__ inst,
                                                     const DevModel* __restrict__ models, int first, int value,
                                                     int32_t* aabb) {
    const int ii = first + (int)blockIdx.y;
    const DevInstance& I = inst[ii];
    const DevModel M = models[I.model];
    const int sxy = M.sx * M.sy;
    const int count = sxy * M.sz;
    const int start = (int)blockIdx.x * kVoxChunk;
    if (start >= count) return;  // uniform per block: no warp-level call below is skipped by part of a warp
    const f3 o = mk(I.m[12], I.m[13], I.m[14]);
    const f3 dx = mk(I.m[0] * 0.1f, I.m[1] * 0.1f, I.m[2] * 0.1f);
    const f3 dy = mk(I.m[4] * 0.1f, I.m[5] * 0.1f, I.m[6] * 0.1f);
    const f3 dz = mk(I.m[8] * 0.1f, I.m[9] * 0.1f, I.m[10] * 0.1f);
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int k = threadIdx.x; k < kVoxChunk; k += blockDim.x) {
        const int v = start + k;
        if (v >= count || M.data[v] < 16) continue;
        const int z = v / sxy, r = v - z * sxy;
        const int y = r / M.sx, x = r - y * M.sx;
        const f3 wp = add(add(add(o, mul(dx, (float)x)), mul(dy, (float)y)), mul(dz, (float)z));
        const int fx = (int)(wp.x * 10.0f), fy = (int)(wp.y * 10.0f), fz = (int)(wp.z * 10.0f);
        mn[0] = min(mn[0], fx);
        mn[1] = min(mn[1], fy);
        mn[2] = min(mn[2], fz);
        mx[0] = max(mx[0], fx);
        mx[1] = max(mx[1], fy);
        mx[2] = max(mx[2], fz);
        if ((unsigned)fx < (unsigned)g.nx && (unsigned)fy < (unsigned)g.ny && (unsigned)fz < (unsigned)g.nz) {
            const unsigned long long bit = 1ull << bit_index(fx, fy, fz);
            if (value)
                atomicOr(words + word_index(g, fx, fy, fz), bit);
            else
                atomicAnd(words + word_index(g, fx, fy, fz), ~bit);
        }
    }
    if (aabb) {
        for (int a = 0; a < 3; a++) {
            const int lo = __reduce_min_sync(0xffffffffu, mn[a]);
            const int hi = __reduce_max_sync(0xffffffffu, mx[a]);
            if ((threadIdx.x & 31) == 0 && lo != INT_MAX) {
                atomicMin(aabb + 6 * ii + a, lo);
                atomicMax(aabb + 6 * ii + 3 + a, hi);
            }
        }
    }
}

cudaError_t launch_tile_mask_view(const GridView& v, uint32_t* mask, int by, int bz, int tx, int ty, int tz,
                                  cudaStream_t s);
cudaError_t launch_trace_layout_view(const GridView& v, const TraceLayout& t, cudaStream_t s);

}  // namespace vxl

using namespace vxl;

extern "C" vxl_status vxl_voxelize_noalloc(const vxl_grid_desc* gd, const vxl_model* models, int nmodels,
                                           const vxl_instance* instances, int n, int32_t* d_aabb, void* stream) {
    if (!gd || !gd->words || !gd->tile_mask) return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: NULL grid descriptor");
    if (gd->nx < 2 || gd->ny < 2 || gd->nz < 2 || (gd->nx & 1) || (gd->ny & 1) || (gd->nz & 1) ||
        gd->bx != (gd->nx + 3) / 4 + 1 || gd->by != (gd->ny + 3) / 4 + 1 || gd->bz != (gd->nz + 3) / 4 + 1 ||
        gd->tx != (gd->bx + 1) / 2 || gd->ty != (gd->by + 1) / 2 || gd->tz != (gd->bz + 1) / 2)
        return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: grid descriptor does not describe a vxl grid layout");
    if (gd->trace_words) {
        vxl_grid d{};
        d.nx = gd->nx;
        d.ny = gd->ny;
        d.nz = gd->nz;
        trace_layout_dims(&d);
        if (!d.tl_nwords || gd->trace_lbx != d.tl_lbx || gd->trace_lby != d.tl_lby || gd->trace_bz != d.tl_bz ||
            gd->trace_words_bytes < d.tl_nwords * sizeof(uint64_t))
            return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: grid descriptor's trace layout does not match its dims");
    }
    if (n < 0 || (n > 0 && !instances)) return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: bad instances");
    if (nmodels < 0 || (nmodels > 0 && !models)) return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: bad models");
    if (n > VXL_NOALLOC_MAX_INSTANCES)
        return fail(VXL_ERR_OUT_OF_RANGE, "voxelize_noalloc: %d instances exceed the fixed table of %d", n,
                    VXL_NOALLOC_MAX_INSTANCES);
    if (nmodels > VXL_NOALLOC_MAX_MODELS)
        return fail(VXL_ERR_OUT_OF_RANGE, "voxelize_noalloc: %d models exceed the fixed table of %d", nmodels,
                    VXL_NOALLOC_MAX_MODELS);
    for (int i = 0; i < nmodels; i++) {
        const vxl_model& m = models[i];
        if (!m.data || m.sx <= 0 || m.sy <= 0 || m.sz <= 0 || (long long)m.sx * m.sy * m.sz > (1ll << 30))
            return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: model %d: null data or bad size", i);
    }
    for (int i = 0; i < n; i++) {
        if (instances[i].model < 0 || instances[i].model >= nmodels)
            return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: instance %d: model %d of %d", i, instances[i].model,
                        nmodels);
        if (instances[i].op != VXL_OP_SET && instances[i].op != VXL_OP_CLEAR)
            return fail(VXL_ERR_INVALID_ARG, "voxelize_noalloc: instance %d: bad op", i);
    }
    if (n == 0) return VXL_OK;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* tables = nullptr;
    VXL_TRY(noalloc_tables(&tables));
    // The tables are overwritten in full for the entries this call reads; no
    // stale contents from an earlier call are used.
    VXL_TRY_CUDA(cudaMemcpyAsync(tables, instances, (size_t)n * sizeof(vxl_instance), cudaMemcpyHostToDevice, s));
    VXL_TRY_CUDA(cudaMemcpyAsync(tables + kNaInstBytes, models, (size_t)nmodels * sizeof(vxl_model),
                                 cudaMemcpyHostToDevice, s));
    GridView v;
    v.words = gd->words;
    v.tmask = gd->tile_mask;
    v.nx = gd->nx;
    v.ny = gd->ny;
    v.nz = gd->nz;
    v.bx = gd->bx;
    v.bxy = (uint32_t)gd->bx * (uint32_t)gd->by;
    v.tx = gd->tx;
    v.txy = (uint32_t)gd->tx * (uint32_t)gd->ty;
    v.ux = (uint32_t)gd->nx + 1u;
    v.uy = (uint32_t)gd->ny + 1u;
    v.uz = (uint32_t)gd->nz + 1u;
    const DevInstance* d_inst = (const DevInstance*)tables;
    const DevModel* d_models = (const DevModel*)(tables + kNaInstBytes);
    // runs of equal ops, applied in array order (same result as one by one)
    for (int i = 0; i < n;) {
        int j = i, maxchunks = 1;
        while (j < n && instances[j].op == instances[i].op) {
            const vxl_model& m = models[instances[j].model];
            long long c = ((long long)m.sx * m.sy * m.sz + kVoxChunk - 1) / kVoxChunk;
            if (c > maxchunks) maxchunks = (int)c;
            j++;
        }
        k_voxelize_na<<<dim3((unsigned)maxchunks, (unsigned)(j - i)), 256, 0, s>>>(
            v, (unsigned long long*)gd->words, d_inst, d_models, i, instances[i].op == VXL_OP_SET ? 1 : 0, d_aabb);
        VXL_TRY_CUDA(cudaGetLastError());
        i = j;
    }
    VXL_TRY_CUDA(launch_tile_mask_view(v, gd->tile_mask, gd->by, gd->bz, gd->tx, gd->ty, gd->tz, s));
    if (gd->trace_words) {
        const TraceLayout t{gd->trace_words, gd->trace_lbx, gd->trace_lby, gd->trace_bz, gd->nx, gd->ny, gd->nz};
        VXL_TRY_CUDA(launch_trace_layout_view(v, t, s));
    }
    // the copies read the caller's host arrays: finish before returning them
    VXL_TRY_CUDA(cudaStreamSynchronize(s));
    return VXL_OK;
}
