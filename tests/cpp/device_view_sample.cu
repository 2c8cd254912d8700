// A user kernel written against the reference's device-side view (VDBInfo,
// cuda_gvdb_nodes.cuh:42-67) through include/gbvdb_device.cuh: it walks the node
// pools from top_lev exactly as the reference's getNodeAtPoint does for a leaf
// (cuda_gvdb_nodes.cuh:199-241) and reads voxels at the reference's atlas
// coordinates (getAtlasPos, gvdb_allocator.cpp:705-715) instead of surf3Dread.
//
//   dv_read_bricks: for each slot, the 18^3 padded brick as atlas voxels
//                   getAtlasPos(slot) - 1 + (x, y, z), [slot][z][y][x], FP32
//   dv_find_leaves: for each slot, the leaf found by walking the tree at the
//                   slot's atlas-map position (-1 when not found), and whether that
//                   leaf's mValue equals getAtlasPos(slot)
#include <cuda_runtime.h>

#include <cstdint>

#include "gbvdb_device.cuh"

namespace {

struct VNode {  // VDBNode (cuda_gvdb_nodes.cuh:24-35)
    unsigned char mLev, mFlags, mPriority, pad;
    int3 mPos, mValue;
    float3 mVRange;
    unsigned long long mParent, mChildList, mMask;
};

__device__ const VNode* node_at(const gbvdb_vdb_info* v, int lev, unsigned long long i) {
    return reinterpret_cast<const VNode*>(v->nodelist[lev] + i * v->nodewid[lev]);
}

__global__ void k_read(const gbvdb_vdb_info* v, int used, float* out) {
    const int s = blockIdx.x;
    if (s >= used) return;
    const int ax = v->atlas_cnt.x, ay = v->atlas_cnt.y;
    const int px = (s % ax) * v->brick_res, py = ((s / ax) % ay) * v->brick_res, pz = (s / (ax * ay)) * v->brick_res;
    for (int i = threadIdx.x; i < 5832; i += blockDim.x) {
        const int x = i % 18, y = (i / 18) % 18, z = i / 324;
        out[(size_t)s * 5832 + i] = gbvdb_atlas_read<float>(v, 0, px + x, py + y, pz + z);
    }
}

__global__ void k_leaves(const gbvdb_vdb_info* v, int used, int* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= used) return;
    const int3 p = v->atlas_map[s].mPos;
    int lev = v->top_lev;
    const VNode* nd = node_at(v, lev, 0);
    long long idx = 0;
    while (lev > 0) {
        const int rg = v->noderange[lev].x, r = v->res[lev];
        const int3 o = make_int3(p.x - nd->mPos.x, p.y - nd->mPos.y, p.z - nd->mPos.z);
        if (o.x < 0 || o.y < 0 || o.z < 0 || o.x >= rg || o.y >= rg || o.z >= rg) { idx = -1; break; }
        const int cr = rg / r;
        const int b = ((o.z / cr) * r + o.y / cr) * r + o.x / cr;
        const unsigned long long* cl = reinterpret_cast<const unsigned long long*>(
            v->childlist[lev] + (nd->mChildList >> 16) * v->childwid[lev]);
        const unsigned long long c = cl[b];
        if (c == 0xFFFFFFFFFFFFFFFFull) { idx = -1; break; }
        lev--;
        idx = (long long)(c >> 16);
        nd = node_at(v, lev, (unsigned long long)idx);
    }
    int ok = 0;
    if (idx >= 0) {
        const int ax = v->atlas_cnt.x, ay = v->atlas_cnt.y;
        const int3 ap = make_int3((s % ax) * 18 + 1, ((s / ax) % ay) * 18 + 1, (s / (ax * ay)) * 18 + 1);
        ok = nd->mValue.x == ap.x && nd->mValue.y == ap.y && nd->mValue.z == ap.z &&
             nd->mPos.x == p.x && nd->mPos.y == p.y && nd->mPos.z == p.z;
    }
    out[2 * s] = (int)idx;
    out[2 * s + 1] = ok;
}

int run(const void* host_info, int used, void* host_out, size_t out_bytes, bool leaves) {
    gbvdb_vdb_info* dv = nullptr;
    void* dout = nullptr;
    if (cudaMalloc(&dv, sizeof(gbvdb_vdb_info)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, out_bytes) != cudaSuccess) { cudaFree(dv); return 1; }
    cudaMemcpy(dv, host_info, sizeof(gbvdb_vdb_info), cudaMemcpyHostToDevice);
    if (used > 0) {
        if (leaves) k_leaves<<<(used + 127) / 128, 128>>>(dv, used, (int*)dout);
        else k_read<<<used, 256>>>(dv, used, (float*)dout);
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(host_out, dout, out_bytes, cudaMemcpyDeviceToHost);
    cudaFree(dv);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 2;
}

}  // namespace

extern "C" int dv_read_bricks(const void* host_info, int used, float* host_out) {
    return run(host_info, used, host_out, (size_t)used * 5832 * 4 + 4, false);
}
extern "C" int dv_find_leaves(const void* host_info, int used, int* host_out) {
    return run(host_info, used, host_out, (size_t)used * 8 + 8, true);
}
