/*
 * gbvdb_device.cuh -- device-side view of a libgbvdb grid for user kernels.
 *
 * The reference hands its user kernels a VDBInfo* (cuda_gvdb_nodes.cuh:42-67)
 * and surface objects volOut[chan] over an atlas addressed by getAtlasPos
 * (gvdb_allocator.cpp:705-715): slot id -> (id % ax, (id / ax) % ay, id / (ax*ay))
 * * 18 + 1, voxel (x, y, z) of the padded 18^3 brick at that corner - 1.
 *
 * gbvdb_vdb_info has VDBInfo's byte layout field for field, so code that walks the
 * node pools through it (nodelist, childlist, nodewid, childwid, noderange, res,
 * top_lev, atlas_map, atlas_cnt, brick_res) reads this library's pools unchanged:
 * node records and child lists are the reference's.  The atlas is not a CUDA
 * array here; it is stored brick-major and split into the 16^3 interiors and the
 * apron records of each slot.  The 64-bit slots that hold the reference's texture
 * and surface objects hold instead, per channel c:
 *   volIn[c]  = device address of the interiors  (slot * 4096 + (z*16 + y)*16 + x)
 *   volOut[c] = device address of the apron records (slot * GBVDB_APRON_STRIDE + k)
 * and apron_table[c] (unused by the reference) holds channel c's bytes per voxel
 * (0: no channel).  A kernel that did
 *   surf3Dread<T>(gvdb->volOut[c], x * sizeof(T), y, z)      (atlas voxel x, y, z)
 * does
 *   gbvdb_atlas_read<T>(gvdb, c, x, y, z)
 * here, and surf3Dwrite likewise with gbvdb_atlas_write.  Obtain the struct with
 * gbvdb_get_vdb_info (include/gbvdb.h).
 */
#ifndef GBVDB_DEVICE_CUH
#define GBVDB_DEVICE_CUH

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#define GBVDB_MAX_CHANNEL 32
#define GBVDB_APRON_VOXELS 1736 /* 18^3 - 16^3 */
#define GBVDB_APRON_STRIDE 1744 /* apron record stride per slot (voxels) */

/* VDBAtlasNode (cuda_gvdb_nodes.cuh:38-41) */
struct __align__(16) gbvdb_atlas_node {
    int3 mPos;
    int mLeafID;
};

/* VDBInfo (cuda_gvdb_nodes.cuh:42-67), same field order, types and offsets */
struct __align__(16) gbvdb_vdb_info {
    int dim[10];
    int res[10];
    float3 vdel[10];
    int3 noderange[10];
    int nodecnt[10];
    int nodewid[10];
    int childwid[10];
    char* nodelist[10];
    char* childlist[10];
    gbvdb_atlas_node* atlas_map;
    int3 atlas_cnt;
    int3 atlas_res;
    int atlas_apron;
    int brick_res;
    int apron_table[8]; /* here: bytes per voxel of channels 0..7 */
    int top_lev;
    int max_iter;
    float epsilon;
    bool update;
    unsigned char clr_chan;
    float3 bmin;
    float3 bmax;
    unsigned long long volIn[GBVDB_MAX_CHANNEL];  /* here: interior base of each channel */
    unsigned long long volOut[GBVDB_MAX_CHANNEL]; /* here: apron-record base of each channel */
};
#ifdef __cplusplus
static_assert(offsetof(gbvdb_vdb_info, nodelist) == 440, "VDBInfo layout");
static_assert(offsetof(gbvdb_vdb_info, atlas_map) == 600, "VDBInfo layout");
static_assert(offsetof(gbvdb_vdb_info, bmin) == 688, "VDBInfo layout");
static_assert(offsetof(gbvdb_vdb_info, volIn) == 712, "VDBInfo layout");
static_assert(offsetof(gbvdb_vdb_info, volOut) == 968, "VDBInfo layout");
#endif

/* Apron record of a slot (GBVDB_APRON_VOXELS voxels, grouped by the neighbour each
 * voxel copies):
 *   faces   [f*256, +256)   f = 0:-x 1:+x 2:-y 3:+y 4:-z 5:+z, each in the order of the
 *                           neighbour's interior plane (x faces [z][y], y faces [z][x],
 *                           z faces [y][x]);
 *   edges   [1536 + e*16, +16) e = 0..3 along x ((y, z) in {0, 17}), 4..7 along y
 *                           ((x, z)), 8..11 along z ((x, y)); bit 0 / 1 = first / second
 *                           coordinate is 17;
 *   corners [1728 + c)      c = (z == 17)*4 + (y == 17)*2 + (x == 17).
 * Padded-brick coordinate (x, y, z in [0, 18)) on the apron shell -> record index. */
__host__ __device__ inline int gbvdb_apron_index(int x, int y, int z) {
    const bool bx = x == 0 || x == 17, by = y == 0 || y == 17, bz = z == 0 || z == 17;
    const int hx = x == 17, hy = y == 17, hz = z == 17;
    const int nb = (int)bx + (int)by + (int)bz;
    if (nb == 1) {
        if (bx) return (0 + hx) * 256 + (z - 1) * 16 + (y - 1);
        if (by) return (2 + hy) * 256 + (z - 1) * 16 + (x - 1);
        return (4 + hz) * 256 + (y - 1) * 16 + (x - 1);
    }
    if (nb == 2) {
        if (!bx) return 1536 + (hz * 2 + hy) * 16 + (x - 1);
        if (!by) return 1536 + (4 + hz * 2 + hx) * 16 + (y - 1);
        return 1536 + (8 + hy * 2 + hx) * 16 + (z - 1);
    }
    return 1728 + hz * 4 + hy * 2 + hx;
}

/* address of atlas voxel (x, y, z) of channel c, or NULL outside the atlas */
template <typename T>
__host__ __device__ inline T* gbvdb_atlas_ptr(const gbvdb_vdb_info* v, int c, int x, int y, int z) {
    const int br = v->brick_res;
    if (x < 0 || y < 0 || z < 0 || x >= v->atlas_res.x || y >= v->atlas_res.y || z >= v->atlas_res.z) return 0;
    const int bx = x / br, by = y / br, bz = z / br;
    const int lx = x - bx * br, ly = y - by * br, lz = z - bz * br;
    const long long slot = ((long long)bz * v->atlas_cnt.y + by) * v->atlas_cnt.x + bx;
    if (lx >= 1 && lx <= 16 && ly >= 1 && ly <= 16 && lz >= 1 && lz <= 16)
        return reinterpret_cast<T*>(v->volIn[c]) + slot * 4096 + ((lz - 1) * 16 + (ly - 1)) * 16 + (lx - 1);
    return reinterpret_cast<T*>(v->volOut[c]) + slot * GBVDB_APRON_STRIDE + gbvdb_apron_index(lx, ly, lz);
}
template <typename T>
__device__ inline T gbvdb_atlas_read(const gbvdb_vdb_info* v, int c, int x, int y, int z) {
    return *gbvdb_atlas_ptr<T>(v, c, x, y, z);
}
template <typename T>
__device__ inline void gbvdb_atlas_write(const gbvdb_vdb_info* v, int c, int x, int y, int z, T val) {
    *gbvdb_atlas_ptr<T>(v, c, x, y, z) = val;
}

#endif /* GBVDB_DEVICE_CUH */
