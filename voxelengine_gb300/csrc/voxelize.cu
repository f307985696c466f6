// voxelize.cu — GPU ShadowVox voxelizer (ShadowVoxSystem::OnUpdate inner
// loops, Sources/World/Systems/ShadowVoxSystem.cpp:137-177, SetVolumeAt :82-94).
//
// One launch applies a run of instances that all carry the same op: their
// writes commute (every write of a run stores the same bit value), so bits are
// combined with atomicOr / atomicAnd on the 64-bit brick words,
// one atomic per source voxel.
#include "vxl_device.cuh"

namespace vxl {

// One block per chunk (instance, first source voxel) of kVoxChunk voxels.
__global__ void __launch_bounds__(256) k_voxelize(GridView g, unsigned long long* words,
                                                  const DevInstance* __restrict__ inst,
                                                  const DevModel* __restrict__ models,
                                                  const int2* __restrict__ chunks, int value, int32_t* aabb) {
    const int2 ch = chunks[blockIdx.x];
    const DevInstance& I = inst[ch.x];
    const DevModel M = models[I.model];
    // o = M[3], dx,dy,dz = M[0..2] * 0.1f (ShadowVoxSystem.cpp:137-140)
    const f3 o = mk(I.m[12], I.m[13], I.m[14]);
    const f3 dx = mk(I.m[0] * 0.1f, I.m[1] * 0.1f, I.m[2] * 0.1f);
    const f3 dy = mk(I.m[4] * 0.1f, I.m[5] * 0.1f, I.m[6] * 0.1f);
    const f3 dz = mk(I.m[8] * 0.1f, I.m[9] * 0.1f, I.m[10] * 0.1f);
    const int sxy = M.sx * M.sy;
    const int count = sxy * M.sz;
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < kVoxChunk; k += blockDim.x) {
        int v = ch.y + k;
        bool act = false;
        uint32_t wi = 0;
        unsigned long long bit = 0;
        if (v < count) {
            uint8_t pal = M.data[v];
            if (pal >= 16) {
                int z = v / sxy, r = v - z * sxy;
                int y = r / M.sx, x = r - y * M.sx;
                // wp = o + x*dx + y*dy + z*dz ; fwp = ivec3(wp * 10) (:146-147)
                f3 wp = add(add(add(o, mul(dx, (float)x)), mul(dy, (float)y)), mul(dz, (float)z));
                int fx = (int)(wp.x * 10.0f), fy = (int)(wp.y * 10.0f), fz = (int)(wp.z * 10.0f);
                mn[0] = min(mn[0], fx);
                mn[1] = min(mn[1], fy);
                mn[2] = min(mn[2], fz);
                mx[0] = max(mx[0], fx);
                mx[1] = max(mx[1], fy);
                mx[2] = max(mx[2], fz);
                // SetVolumeAt bounds: 0 <= x < 2*SizeX (:83)
                if ((unsigned)fx < (unsigned)g.nx && (unsigned)fy < (unsigned)g.ny && (unsigned)fz < (unsigned)g.nz) {
                    act = true;
                    wi = word_index(g, fx, fy, fz);
                    bit = 1ull << bit_index(fx, fy, fz);
                }
            }
        }
        if (act) {
            if (value)
                atomicOr(words + wi, bit);
            else
                atomicAnd(words + wi, ~bit);
        }
    }
    if (aabb) {
        for (int a = 0; a < 3; a++) {
            int lo = __reduce_min_sync(0xffffffffu, mn[a]);
            int hi = __reduce_max_sync(0xffffffffu, mx[a]);
            if (lane == 0 && lo != INT_MAX) {
                atomicMin(aabb + 6 * ch.x + a, lo);
                atomicMax(aabb + 6 * ch.x + 3 + a, hi);
            }
        }
    }
}

vxl_status launch_voxelize_run(vxl_grid* g, const DevInstance* d_inst, const DevModel* d_models, const int2* d_chunks,
                               int nchunks, int value, int32_t* d_aabb, cudaStream_t s) {
    if (nchunks <= 0) return VXL_OK;
    GridView v = view_of(g);
    k_voxelize<<<nchunks, 256, 0, s>>>(v, (unsigned long long*)g->words, d_inst, d_models, d_chunks, value, d_aabb);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
