// common.cuh -- device-side types and helpers shared by the libgbvdb kernels.
//
// Node / pool layouts follow the reference byte for byte:
//   Node            gvdb_node.h:27-40, cuda_gvdb_nodes.cuh:24-35 (64 bytes)
//   Elem(grp,lev,n) gvdb_allocator.h:59-62
//   child lists     res^3 u64 entries per node, 0xFF..FF = empty (VG.cpp:979-985)
// The tree traversals restate getPosParent / getParent / getPosLeafParent /
// getNode (cuda_gvdb_nodes.cuh:199-397) with one addition: a position outside
// the node being descended is rejected instead of aliasing into a wrong child
// slot (the reference has no bounds check there, ND.cuh:317-322).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gbvdb_device.cuh"

namespace gbvdb {

constexpr int kMaxLev = 10;
constexpr unsigned long long kUndef64 = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kUndefL = 0xFFFFFFFFull;
constexpr float kNoHit = 1.0e10f;
constexpr int kBrick = 16;     // leaf resolution (log2dim[0] == 4)
constexpr int kPad = 18;       // brick with a 1-voxel apron
constexpr int kApronVox = 1736;  // 18^3 - 16^3
constexpr int kApronStride = 1744;  // apron record length (multiple of 16 elements)

struct __align__(16) Node {
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    unsigned long long parent;
    unsigned long long childlist;
    unsigned long long mask;
};
static_assert(sizeof(Node) == 64, "node record is 64 bytes");

struct __align__(16) AtlasNode {
    int32_t pos[3];
    int32_t leaf;
};

// Read-only view of the tree passed to kernels by value.
struct TreeView {
    int levs;
    int top_lev;
    int res[kMaxLev];
    int lgres[kMaxLev];
    int lgrange[kMaxLev];          // log2(range[l])
    long long ncnt[kMaxLev];
    Node* nodes[kMaxLev];
    unsigned long long* clist[kMaxLev];
};

__host__ __device__ inline unsigned long long elem(int grp, int lev, unsigned long long ndx) {
    return (unsigned long long)grp | ((unsigned long long)lev << 8) | (ndx << 16);
}

// ---- child-slot helpers -------------------------------------------------

// slot of integer position p inside node (at level l, corner npos); -1 if outside
__device__ __forceinline__ int child_slot(const TreeView& t, int l, const int32_t* npos, int px, int py, int pz) {
    long long dx = (long long)px - npos[0], dy = (long long)py - npos[1], dz = (long long)pz - npos[2];
    long long rg = 1ll << t.lgrange[l];
    if (dx < 0 || dy < 0 || dz < 0 || dx >= rg || dy >= rg || dz >= rg) return -1;
    int sh = t.lgrange[l] - t.lgres[l];  // log2 of the child range
    int cx = (int)(dx >> sh), cy = (int)(dy >> sh), cz = (int)(dz >> sh);
    return (cz << (2 * t.lgres[l])) | (cy << t.lgres[l]) | cx;
}

// getChild (ND.cuh:115-124): child index, -1 when empty
__device__ __forceinline__ long long get_child(const TreeView& t, const Node* nd, int b) {
    unsigned long long listid = nd->childlist;
    if (listid == kUndefL) return -1;
    int clev = (int)((listid >> 8) & 0xFF);
    unsigned long long cndx = listid >> 16;
    unsigned long long e = t.clist[clev][(cndx << (3 * t.lgres[clev])) + (unsigned)b];
    if (e == kUndef64) return -1;
    return (long long)(e >> 16);
}

// getPosParent (ND.cuh:303-348)
__device__ inline long long get_pos_parent(const TreeView& t, int px, int py, int pz, int stop_lev) {
    if (t.ncnt[t.top_lev] == 0) return -1;
    const Node* nd = t.nodes[t.top_lev];
    int l = nd->lev;
    if (l == 0) return 0;
    while (l > 0) {
        int b = child_slot(t, l, nd->pos, px, py, pz);
        if (b < 0) return -1;
        long long c = get_child(t, nd, b);
        l--;
        if (c < 0) return -1;
        if (l == stop_lev) return c;
        nd = t.nodes[l] + c;
    }
    return -1;
}

// getParent (ND.cuh:350-397)
__device__ inline long long get_parent(const TreeView& t, int stop_lev, int px, int py, int pz) {
    const Node* nd = t.nodes[t.top_lev];
    if (!nd->flags) return 0;
    int l = nd->lev;
    if (l == stop_lev) return 0;
    while (l > stop_lev) {
        int b = child_slot(t, l, nd->pos, px, py, pz);
        if (b < 0) return -1;
        l--;
        long long c = get_child(t, nd, b);
        if (c < 0) return -1;
        if (l == stop_lev) return c;
        nd = t.nodes[l] + c;
    }
    return -1;
}

// getPosLeafParent (ND.cuh:255-288); single-leaf trees check containment
__device__ inline long long get_pos_leaf(const TreeView& t, int px, int py, int pz) {
    if (t.ncnt[t.top_lev] == 0) return -1;
    const Node* nd = t.nodes[t.top_lev];
    int l = nd->lev;
    if (l == 0) {
        long long dx = (long long)px - nd->pos[0], dy = (long long)py - nd->pos[1], dz = (long long)pz - nd->pos[2];
        long long rg = 1ll << t.lgrange[0];
        if (dx < 0 || dy < 0 || dz < 0 || dx >= rg || dy >= rg || dz >= rg) return -1;
        return 0;
    }
    while (true) {
        int b = child_slot(t, l, nd->pos, px, py, pz);
        if (b < 0) return -1;
        long long c = get_child(t, nd, b);
        if (c < 0) return -1;
        l--;
        if (l == 0) return c;
        nd = t.nodes[l] + c;
    }
}

// getNode(float pos) as used by UpdateApron (ND.cuh:199-253) for integer voxel w
__device__ inline long long get_leaf_at_voxel(const TreeView& t, int wx, int wy, int wz) {
    if (t.ncnt[t.top_lev] == 0) return -1;
    int lev = t.top_lev;
    const Node* nd = t.nodes[lev];
    long long id = 0;
    while (lev > 0) {
        int b = child_slot(t, lev, nd->pos, wx, wy, wz);
        if (b < 0) return -1;
        lev--;
        long long c = get_child(t, nd, b);
        if (c < 0) return -1;
        id = c;
        nd = t.nodes[lev] + c;
    }
    long long dx = (long long)wx - nd->pos[0], dy = (long long)wy - nd->pos[1], dz = (long long)wz - nd->pos[2];
    long long rg = 1ll << t.lgrange[0];
    if (dx < 0 || dy < 0 || dz < 0 || dx >= rg || dy >= rg || dz >= rg) return -1;
    return id;
}

// Dense lookup of the leaf reachable at a brick position: cells[(bx*dy + by)*dz + bz]
// over the brick box [lo, lo+dim) = leaf index or -1.  Built by traversal, so it
// answers exactly what get_pos_leaf answers (for trees whose top level is >= 1);
// cells == nullptr means "not built": fall back to the traversal.
struct LeafGrid {
    const int* cells;
    int lo[3];
    int dim[3];
    int lgrange0;
};

__device__ __forceinline__ long long lookup_leaf(const LeafGrid& g, const TreeView& t, int px, int py, int pz) {
    if (g.cells) {
        int bx = (px >> g.lgrange0) - g.lo[0], by = (py >> g.lgrange0) - g.lo[1], bz = (pz >> g.lgrange0) - g.lo[2];
        if ((unsigned)bx >= (unsigned)g.dim[0] || (unsigned)by >= (unsigned)g.dim[1] || (unsigned)bz >= (unsigned)g.dim[2])
            return -1;
        return __ldg(g.cells + ((long long)bx * g.dim[1] + by) * g.dim[2] + bz);
    }
    return get_pos_leaf(t, px, py, pz);
}

// atlas slot from mValue (inverse of getAtlasPos, gvdb_allocator.cpp:705-715)
__device__ __forceinline__ int slot_of_value(const int32_t* v, int ax, int ay) {
    if (v[0] < 0) return -1;
    return ((v[2] / kPad) * ay + v[1] / kPad) * ax + v[0] / kPad;
}

// ---- exact float helpers (no contraction) ------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// GetCoveringNode float version (PT.cuh:88-100) as a node coordinate
__device__ __forceinline__ int cover_coord(float w, int lgrange) {
    float fr = (float)(1 << lgrange);
    // w / 2^lg as w * 2^-lg: a power-of-two scaling, exact (the same float as the division)
    float np = __fmul_rn(ceilf(__fmul_rn(w, __int_as_float((127 - lgrange) << 23))), fr);
    int ni = (int)np;
    if (w < (float)ni) ni -= (1 << lgrange);
    return ni >> lgrange;  // ni >= 0 for w >= 0
}

// ordered-int encoding of floats for atomicMin/Max
__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__host__ __device__ inline float o2f(int i) {
#ifdef __CUDA_ARCH__
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
#else
    int j = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    memcpy(&f, &j, 4);
    return f;
#endif
}

__device__ __forceinline__ void load_pos(const char* base, long long i, int stride, int off, float& x, float& y, float& z) {
    const float* q = reinterpret_cast<const float*>(base + i * (long long)stride + off);
    x = __ldg(q);
    y = __ldg(q + 1);
    z = __ldg(q + 2);
}

// Apron record layout (1,736 voxels per slot, grouped by the neighbour they copy):
//   faces  [f*256, +256)  f = 0:-x 1:+x 2:-y 3:+y 4:-z 5:+z; a face holds the 16x16
//          voxels that match one interior plane of the face neighbour, in that
//          plane's own order (x faces [z][y], y faces [z][x], z faces [y][x]);
//   edges  [1536 + e*16, +16) e = 0..3 along x (y,z in {0,17}), 4..7 along y
//          (x,z), 8..11 along z (x,y); bit order (high coordinate == 17);
//   corners [1728 + c) c = (z==17)*4 + (y==17)*2 + (x==17).
// padded-brick coordinate (x,y,z in [0,18)) on the apron shell -> record index; the
// layout is the public one of include/gbvdb_device.cuh, which consumer kernels use
__host__ __device__ inline int apron_index(int x, int y, int z) { return gbvdb_apron_index(x, y, z); }
static_assert(kApronStride == GBVDB_APRON_STRIDE, "apron record stride");

// inverse of apron_index: record index k in [0, 1736) -> padded-brick coordinate
// on the apron shell.  The voxel comes from the neighbour at direction
// d = (x==0 ? -1 : x==17 ? 1 : 0, ...), whose local voxel is (x-1-16*dx, ...).
__host__ __device__ constexpr void apron_shell_pos(int k, int& x, int& y, int& z) {
    if (k < 1536) {
        const int f = k >> 8, r = ((k >> 4) & 15) + 1, c = (k & 15) + 1, h = (f & 1) ? 17 : 0;
        if (f < 2) { x = h; z = r; y = c; }
        else if (f < 4) { y = h; z = r; x = c; }
        else { z = h; y = r; x = c; }
    } else if (k < 1728) {
        const int e = (k - 1536) >> 4, i = ((k - 1536) & 15) + 1;
        const int lo = (e & 1) ? 17 : 0, hi = ((e >> 1) & 1) ? 17 : 0;
        if (e < 4) { x = i; y = lo; z = hi; }
        else if (e < 8) { y = i; x = lo; z = hi; }
        else { z = i; x = lo; y = hi; }
    } else {
        const int c = k - 1728;
        x = (c & 1) ? 17 : 0;
        y = (c & 2) ? 17 : 0;
        z = (c & 4) ? 17 : 0;
    }
}

// Edges and corners of the apron record (records [1536, 1736)): for record
// 1536 + j, the voxel of the source brick (interior index (z << 8) | (y << 4) | x)
// and the direction index (dx+1) + 3 (dy+1) + 9 (dz+1) of the brick that receives
// it, seen from the source; the source, seen from the receiver, is 26 - that.
struct ApronEdgeTable {
    uint32_t e[200];  // record 1536 + j: tile index | receiver direction << 12
};
constexpr ApronEdgeTable make_apron_edge_table() {
    ApronEdgeTable t{};
    for (int j = 0; j < 200; j++) {
        int x = 0, y = 0, z = 0;
        apron_shell_pos(1536 + j, x, y, z);
        const int dx = x == 0 ? -1 : (x == 17 ? 1 : 0);
        const int dy = y == 0 ? -1 : (y == 17 ? 1 : 0);
        const int dz = z == 0 ? -1 : (z == 17 ? 1 : 0);
        const int tile_idx = ((z - 1 - 16 * dz) << 8) | ((y - 1 - 16 * dy) << 4) | (x - 1 - 16 * dx);
        const int recv = (1 - dz) * 9 + (1 - dy) * 3 + (1 - dx);
        t.e[j] = (uint32_t)tile_idx | ((uint32_t)recv << 12);
    }
    return t;
}
static __device__ const ApronEdgeTable kApronEdges = make_apron_edge_table();

}  // namespace gbvdb
