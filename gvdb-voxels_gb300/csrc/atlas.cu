// atlas.cu -- atlas slot assignment, apron update, atlas export and reductions.
//
// Replaces (reference file:line):
//   UpdateAtlas: AtlasAlloc/getAtlasPos loop + ClearMapping/AssignMapping
//       VG.cpp:2630-2704, 2557-2590; gvdb_allocator.cpp:692-715
//   UpdateApron<T> / gvdbUpdateApronF   cuda_gvdb_operators.cuh:72-131, VG.cpp:4418-4457
//
// Atlas storage is brick-major and split in two arrays per channel:
//   interior[slot][z][y][x]  16^3 voxels, the voxels gathers write
//   apron[slot][k]           1736 apron voxels (record stride 1744), k = apron_index(x,y,z)
// so that a gather writes whole 32-byte sectors and the apron pass writes its own
// records.  The logical atlas coordinate of padded voxel (x,y,z) of slot s is the
// reference's getAtlasPos(s) + (x,y,z) (gvdb_allocator.cpp:705-715).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>

#include "kernels.h"

namespace gbvdb {

namespace {

// flagged leaves in pool order get consecutive slot ids (VG.cpp:2655-2662)
__global__ void k_assign_slots(Node* leaves, long long n, const uint32_t* scan, int ax, int ay, AtlasNode* amap) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Node* nd = leaves + i;
    if (!nd->flags) return;
    unsigned id = scan[i];
    unsigned a2 = (unsigned)ax * (unsigned)ay;
    int pz = (int)(id / a2);
    unsigned rem = id - (unsigned)pz * a2;
    int py = (int)(rem / (unsigned)ax);
    int px = (int)(rem - (unsigned)py * ax);
    nd->value[0] = px * kPad + 1;
    nd->value[1] = py * kPad + 1;
    nd->value[2] = pz * kPad + 1;
    AtlasNode an;
    an.pos[0] = nd->pos[0];
    an.pos[1] = nd->pos[1];
    an.pos[2] = nd->pos[2];
    an.leaf = (int32_t)i;
    amap[id] = an;
}

__global__ void k_fill_u32(uint32_t* p, long long n, uint32_t v) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

// One block per assigned slot.  The 26 neighbour slots are looked up once per
// brick (the reference traverses the tree once per apron voxel); then the apron
// record is filled by copies grouped by neighbour: the four y/z faces are rows
// of the neighbour's boundary planes (16-byte vector loads and stores), the two
// x faces are strided columns, edges and corners single lines and voxels.  A
// missing neighbour gives the boundary value.
template <typename T>
__global__ void __launch_bounds__(256) k_apron(TreeView t, LeafGrid lg, const AtlasNode* __restrict__ amap, int ax, int ay,
                                               const T* __restrict__ interior, T* __restrict__ apron, T boundval) {
    __shared__ int nslot[27];
    const int s = blockIdx.x;
    const AtlasNode an = amap[s];
    if (an.leaf < 0) return;
    if (threadIdx.x < 27) {
        int dx = (int)threadIdx.x % 3 - 1, dy = ((int)threadIdx.x / 3) % 3 - 1, dz = (int)threadIdx.x / 9 - 1;
        int ns = -1;
        if (dx | dy | dz) {
            int px = an.pos[0] + 16 * dx, py = an.pos[1] + 16 * dy, pz = an.pos[2] + 16 * dz;
            long long nl = lg.cells ? ((px < 0 || py < 0 || pz < 0) ? -1 : lookup_leaf(lg, t, px, py, pz))
                                    : get_leaf_at_voxel(t, px, py, pz);
            if (nl >= 0) ns = slot_of_value(t.nodes[0][nl].value, ax, ay);
        }
        nslot[threadIdx.x] = ns;
    }
    __syncthreads();
    T* out = apron + (size_t)s * kApronStride;
    constexpr int V = 16 / sizeof(T);  // elements per 16-byte vector
    // y and z faces: 4 faces x 256 elements as 16-byte vectors
    for (int k = threadIdx.x; k < 4 * 256 / V; k += blockDim.x) {
        const int f = 2 + k / (256 / V);            // 2..5
        const int e0 = (k % (256 / V)) * V;        // first element within the face
        const int row = e0 >> 4, col = e0 & 15;    // face [row][col]
        int dir, src;
        if (f < 4) {  // y faces: neighbour plane y = 15 (f=2) or 0 (f=3); face [z][x]
            dir = f == 2 ? (1 * 9 + 0 * 3 + 1) : (1 * 9 + 2 * 3 + 1);
            src = (row << 8) + ((f == 2 ? 15 : 0) << 4) + col;
        } else {      // z faces: neighbour plane z = 15 (f=4) or 0 (f=5); face [y][x]
            dir = f == 4 ? (0 * 9 + 1 * 3 + 1) : (2 * 9 + 1 * 3 + 1);
            src = ((f == 4 ? 15 : 0) << 8) + (row << 4) + col;
        }
        const int ns = nslot[dir];
        uint4 v;
        if (ns >= 0) {
            v = *reinterpret_cast<const uint4*>(interior + (size_t)ns * 4096 + src);
        } else {
            T b[V];
#pragma unroll
            for (int q = 0; q < V; q++) b[q] = boundval;
            v = *reinterpret_cast<const uint4*>(b);
        }
        *reinterpret_cast<uint4*>(out + f * 256 + e0) = v;
    }
    // x faces: columns x = 15 (f=0) and x = 0 (f=1) of the x neighbours; face [z][y]
    for (int k = threadIdx.x; k < 512; k += blockDim.x) {
        const int f = k >> 8, e = k & 255, z = e >> 4, y = e & 15;
        const int ns = nslot[1 * 9 + 1 * 3 + (f == 0 ? 0 : 2)];
        out[f * 256 + e] = ns >= 0 ? interior[(size_t)ns * 4096 + (z << 8) + (y << 4) + (f == 0 ? 15 : 0)] : boundval;
    }
    // edges (12 x 16) and corners (8)
    for (int k = threadIdx.x; k < 200; k += blockDim.x) {
        int lx, ly, lz, dir;
        if (k < 192) {
            const int e = k >> 4, i = k & 15;
            const int a = e >> 2, h0 = e & 1, h1 = (e >> 1) & 1;
            if (a == 0) {         // along x: (y, z) = (h0, h1)
                lx = i; ly = h0 ? 0 : 15; lz = h1 ? 0 : 15;
                dir = (h1 ? 2 : 0) * 9 + (h0 ? 2 : 0) * 3 + 1;
            } else if (a == 1) {  // along y: (x, z) = (h0, h1)
                ly = i; lx = h0 ? 0 : 15; lz = h1 ? 0 : 15;
                dir = (h1 ? 2 : 0) * 9 + 1 * 3 + (h0 ? 2 : 0);
            } else {              // along z: (x, y) = (h0, h1)
                lz = i; lx = h0 ? 0 : 15; ly = h1 ? 0 : 15;
                dir = 1 * 9 + (h1 ? 2 : 0) * 3 + (h0 ? 2 : 0);
            }
        } else {
            const int c = k - 192, hx = c & 1, hy = (c >> 1) & 1, hz = c >> 2;
            lx = hx ? 0 : 15; ly = hy ? 0 : 15; lz = hz ? 0 : 15;
            dir = (hz ? 2 : 0) * 9 + (hy ? 2 : 0) * 3 + (hx ? 2 : 0);
        }
        const int ns = nslot[dir];
        out[1536 + k] = ns >= 0 ? interior[(size_t)ns * 4096 + (lz << 8) + (ly << 4) + lx] : boundval;
    }
}

// UpdateApron after a fused-apron gather (k_gather's push_apron): every brick has
// already copied its boundary voxels into its neighbours' apron records, so only
// the voxels of missing neighbours are left (the boundary value).  One warp per
// slot.  The push was made only when the grid passed that gather's push check
// (k_push_check: linked == flagged == found by the lookup, slot == linked rank),
// and then every neighbour the lookup finds here pushed into this slot.  If the
// check failed (*bad) this is the full pass.
template <typename T>
__global__ void __launch_bounds__(256) k_apron_fill(TreeView t, LeafGrid lg, const AtlasNode* __restrict__ amap, int used,
                                                    int ax, int ay, const T* __restrict__ interior,
                                                    T* __restrict__ apron, T boundval, const int* __restrict__ bad) {
    __shared__ int nsl[8][27];  // >= 0: copy from that slot; -1: boundary value; -2: written by the gather
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = blockIdx.x * 8 + w;
    if (s >= used) return;
    const bool pushed = __ldg(bad) == 0;
    const AtlasNode an = amap[s];
    if (an.leaf < 0) return;
    const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
    int ns = -1;
    if (lane < 27 && (dx | dy | dz)) {
        const int px = an.pos[0] + 16 * dx, py = an.pos[1] + 16 * dy, pz = an.pos[2] + 16 * dz;
        const long long nl = (px < 0 || py < 0 || pz < 0) ? -1 : lookup_leaf(lg, t, px, py, pz);
        if (pushed) ns = nl >= 0 ? -2 : -1;
        else if (nl >= 0) ns = slot_of_value(t.nodes[0][nl].value, ax, ay);
    }
    if (lane >= 27 || lane == 13) ns = -2;
    T* out = apron + (size_t)s * kApronStride;
    if (pushed) {
        // only the boundary value is left to write, where a neighbour is missing:
        // whole faces as 16-byte vectors, then the edge and corner voxels
        const unsigned miss = __ballot_sync(0xFFFFFFFFu, ns == -1);
        if (!miss) return;
        uint32_t bb;
        if constexpr (sizeof(T) == 4) bb = __float_as_uint(*reinterpret_cast<const float*>(&boundval));
        else bb = (uint32_t)(*reinterpret_cast<const uint16_t*>(&boundval)) * 0x10001u;
        const uint4 b4 = make_uint4(bb, bb, bb, bb);
        constexpr int kFaceDir[6] = {12, 14, 10, 16, 4, 22};  // source direction of faces -x +x -y +y -z +z
        constexpr int kVec = 256 * (int)sizeof(T) / 16;        // 16-byte vectors per face
#pragma unroll
        for (int f = 0; f < 6; f++) {
            if (!((miss >> kFaceDir[f]) & 1u)) continue;
            uint4* fo = reinterpret_cast<uint4*>(out + f * 256);
            for (int q = lane; q < kVec; q += 32) fo[q] = b4;
        }
        for (int j = lane; j < 200; j += 32)
            if ((miss >> (26 - (int)(__ldg(kApronEdges.e + j) >> 12))) & 1u) out[1536 + j] = boundval;
        return;
    }
    if (lane < 27) nsl[w][lane] = ns;
    if (!__ballot_sync(0xFFFFFFFFu, ns != -2)) return;
    __syncwarp();
    for (int k = lane; k < 1736; k += 32) {
        int x, y, z;
        apron_shell_pos(k, x, y, z);
        const int ex = x == 0 ? -1 : (x == 17 ? 1 : 0);
        const int ey = y == 0 ? -1 : (y == 17 ? 1 : 0);
        const int ez = z == 0 ? -1 : (z == 17 ? 1 : 0);
        const int n2 = nsl[w][(ez + 1) * 9 + (ey + 1) * 3 + (ex + 1)];
        if (n2 == -2) continue;
        out[k] = n2 >= 0 ? interior[(size_t)n2 * 4096 + (((z - 1 - 16 * ez) << 8) | ((y - 1 - 16 * ey) << 4) |
                                                         (x - 1 - 16 * ex))]
                         : boundval;
    }
}

template <typename T>
__global__ void k_export_bricks(const T* __restrict__ interior, const T* __restrict__ apron, int used, T* out) {
    long long total = (long long)used * 5832;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int s = (int)(i / 5832);
        int r = (int)(i - (long long)s * 5832);
        int z = r / 324, y = (r / 18) % 18, x = r % 18;
        T v;
        if (x > 0 && x < 17 && y > 0 && y < 17 && z > 0 && z < 17)
            v = interior[(size_t)s * 4096 + ((z - 1) << 8) + ((y - 1) << 4) + (x - 1)];
        else
            v = apron[(size_t)s * kApronStride + apron_index(x, y, z)];
        out[i] = v;
    }
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename T>
__device__ __forceinline__ T from_f32(float v);
template <>
__device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

template <typename T>
__global__ void k_fill_interior(const AtlasNode* __restrict__ amap, int used, T* interior, float value) {
    long long total = (long long)used * 4096;
    T v = from_f32<T>(value);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        if (amap[i >> 12].leaf < 0) continue;
        interior[i] = v;
    }
}

// ---- allocation-free checksum ------------------------------------------
// Scratch of gbvdb_checksum_noalloc: one FP64 partial sum per atlas slot, in a
// file-scope device array (every GPU that loads the library holds it until the
// process exits).  Host code must not pass `g_slot_partials` to a kernel: on the
// host that name is only a stand-in; its device address comes from
// cudaGetSymbolAddress, taken once per device (checksum_noalloc below).
constexpr int kNoAllocMaxSlots = 65536;
static __device__ __align__(256) double g_slot_partials[kNoAllocMaxSlots];

// Compensated FP32 accumulation (Knuth's TwoSum: s + e == a + b exactly in
// round-to-nearest): a running pair (hi, lo) whose value hi + lo carries about
// 48 significant bits, so a brick's 4096 values are summed to near-FP64 accuracy
// with FP32 arithmetic (GB300's FP64 rate is a small fraction of its FP32 rate).
// Non-finite sums keep hi (inf / nan) and drop the error term.
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    if (isfinite(s)) lo = __fadd_rn(lo, e);
}
__device__ __forceinline__ void df_merge(float& hi, float& lo, float h2, float l2) {
    df_add(hi, lo, h2);
    lo = __fadd_rn(lo, l2);
}

// one block per slot (grid-stride over slots): fixed-order sum of the 4096 interior
// voxels (compensated FP32 per thread and across the warp, FP64 across the warps),
// so the result is deterministic.  Launched with 256 threads per block.
template <typename T>
__global__ void k_slot_sums(const AtlasNode* __restrict__ amap, int used, const T* __restrict__ interior,
                            double* __restrict__ partials) {
    __shared__ double red[32];
    constexpr int V = 16 / sizeof(T);  // elements per 16-byte load
    // highest slots first: a gather writes the bricks roughly in slot order, so the
    // last-written ones may still be in L2 (the partials are summed in slot order
    // afterwards, so the visiting order does not change the result)
    for (int j = blockIdx.x; j < used; j += gridDim.x) {
        const int s = used - 1 - j;
        float hi = 0.0f, lo = 0.0f;
        if (amap == nullptr || amap[s].leaf >= 0) {  // null: every slot below used is assigned
            // all of this thread's 16-byte loads of the brick in flight together
            const uint4* src = reinterpret_cast<const uint4*>(interior + (size_t)s * 4096);
            constexpr int kLoads = 4096 / V / 256;
            uint4 w[kLoads];
#pragma unroll
            for (int k = 0; k < kLoads; k++) w[k] = __ldcs(src + threadIdx.x + 256 * k);
#pragma unroll
            for (int k = 0; k < kLoads; k++) {
                const T* e = reinterpret_cast<const T*>(&w[k]);
#pragma unroll
                for (int q = 0; q < V; q++) df_add(hi, lo, to_f32(e[q]));
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float h2 = __shfl_down_sync(0xFFFFFFFFu, hi, o), l2 = __shfl_down_sync(0xFFFFFFFFu, lo, o);
            df_merge(hi, lo, h2, l2);
        }
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)hi + (double)lo;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w8 = 0; w8 < (int)(blockDim.x >> 5); w8++) t += red[w8];
            partials[s] = t;
        }
        __syncthreads();
    }
}

// single block: fixed-order sum of the per-slot partials
__global__ void k_sum_partials(const double* __restrict__ partials, int used, double* __restrict__ out) {
    __shared__ double red[32];
    // four running sums per thread so that four loads are in flight at a time;
    // a fixed order, so the result is deterministic
    const int bd = (int)blockDim.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int s = threadIdx.x;
    for (; s + 3 * bd < used; s += 4 * bd) {
        a0 += partials[s];
        a1 += partials[s + bd];
        a2 += partials[s + 2 * bd];
        a3 += partials[s + 3 * bd];
    }
    for (; s < used; s += bd) a0 += partials[s];
    double acc = (a0 + a1) + (a2 + a3);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
        if (threadIdx.x == 0) *out = t;
    }
}

// One brick layer of the atlas in the reference's atlas layout (a 3D volume of
// ax*18 x ay*18 x az*18 voxels, x fastest, padded 18^3 bricks at getAtlasPos):
// slab[zz][y][x] for zz in [0, 18), the layer of slots bz*ax*ay .. +ax*ay.  Slots
// at or beyond `valid` are written as zero.
template <typename T>
__global__ void k_slab_pack(const T* __restrict__ interior, const T* __restrict__ apron, int ax, int ay, int bz,
                            long long valid, T* __restrict__ slab) {
    const long long W = (long long)ax * 18, H = (long long)ay * 18, n = W * H * 18;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % W), y = (int)((i / W) % H), zz = (int)(i / (W * H));
        const int bx = x / 18, by = y / 18, px = x - 18 * bx, py = y - 18 * by;
        const long long slot = ((long long)bz * ay + by) * ax + bx;
        T v = T(0.0f);
        if (slot < valid) {
            const bool in = px >= 1 && px <= 16 && py >= 1 && py <= 16 && zz >= 1 && zz <= 16;
            v = in ? interior[slot * 4096 + ((zz - 1) << 8) + ((py - 1) << 4) + (px - 1)]
                   : apron[slot * kApronStride + apron_index(px, py, zz)];
        }
        slab[i] = v;
    }
}
template <typename T>
__global__ void k_slab_unpack(const T* __restrict__ slab, int ax, int ay, int bz, T* __restrict__ interior,
                              T* __restrict__ apron) {
    const long long W = (long long)ax * 18, H = (long long)ay * 18, n = W * H * 18;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % W), y = (int)((i / W) % H), zz = (int)(i / (W * H));
        const int bx = x / 18, by = y / 18, px = x - 18 * bx, py = y - 18 * by;
        const long long slot = ((long long)bz * ay + by) * ax + bx;
        const bool in = px >= 1 && px <= 16 && py >= 1 && py <= 16 && zz >= 1 && zz <= 16;
        if (in)
            interior[slot * 4096 + ((zz - 1) << 8) + ((py - 1) << 4) + (px - 1)] = slab[i];
        else
            apron[slot * kApronStride + apron_index(px, py, zz)] = slab[i];
    }
}

// UpdateNeighbors (VG.cpp:2527-2556): per leaf, the leaf at its centre -/+ one brick
// along x, y, z (order -x, -y, -z, +x, +y, +z), -1 where there is none
__global__ void k_neighbors(TreeView t, LeafGrid lg, long long n, int d, int* __restrict__ table) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Node nd = t.nodes[0][i];
    const int dir[6][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const int px = nd.pos[0] + d / 2 + dir[k][0] * d, py = nd.pos[1] + d / 2 + dir[k][1] * d,
                  pz = nd.pos[2] + d / 2 + dir[k][2] * d;
        long long nl = -1;
        if (px >= 0 && py >= 0 && pz >= 0) nl = lg.cells ? lookup_leaf(lg, t, px, py, pz) : get_leaf_at_voxel(t, px, py, pz);
        table[i * 6 + k] = (int)nl;
    }
}

// UpdateApronFaces (VG.cpp:4461-4496, gvdbUpdateApronFacesF OP.cuh:27-61): one block
// per assigned slot; for each of its -x, -y, -z neighbours that owns a slot, the
// slot's first interior plane goes to the neighbour's far apron face and the
// neighbour's last interior plane to the slot's near face.  Each face record has one
// writer (the slot on its far side), so no two blocks write the same voxel.
template <typename T>
__global__ void k_apron_faces(const Node* __restrict__ leaves, const AtlasNode* __restrict__ amap, int used, int ax,
                              int ay, const int* __restrict__ table, T* __restrict__ interior, T* __restrict__ apron) {
    const int s = blockIdx.x;
    const int L = amap[s].leaf;
    if (L < 0) return;
    for (int side = 0; side < 3; side++) {
        const int nb = table[(size_t)L * 6 + side];
        if (nb < 0) continue;
        const int ns = slot_of_value(leaves[nb].value, ax, ay);
        if (ns < 0 || ns >= used || amap[ns].leaf != nb) continue;
        const T* si = interior + (size_t)s * 4096;
        const T* ni = interior + (size_t)ns * 4096;
        T* sa = apron + (size_t)s * kApronStride + (2 * side) * 256;       // near face of the slot
        T* na = apron + (size_t)ns * kApronStride + (2 * side + 1) * 256;  // far face of the neighbour
        for (int e = threadIdx.x; e < 256; e += blockDim.x) {
            const int hi = e >> 4, lo = e & 15;  // face element order: x faces [z][y], y faces [z][x], z faces [y][x]
            int first, last;
            if (side == 0) { first = (hi << 8) + (lo << 4); last = first + 15; }
            else if (side == 1) { first = (hi << 8) + lo; last = first + (15 << 4); }
            else { first = (hi << 4) + lo; last = first + (15 << 8); }
            sa[e] = ni[last];
            na[e] = si[first];
        }
    }
}

// Compute(FUNC_SMOOTH) one pass (gvdbOpSmooth, OP.cuh:383-400), one block per assigned
// slot: the padded brick (interior + the six apron faces: the stencil never reads
// edges or corners) is staged in shared memory, so the slot's interior is rewritten
// from the values before the pass.  v = p1*c + x-1 + x+1 + y-1 + y+1 + z-1 + z+1 in
// FP32 (this order, no contraction), then v / (p1 + 6.0) + p2 in double as the
// source's double literal makes it, rounded to float.
__global__ void __launch_bounds__(256) k_smooth(const AtlasNode* __restrict__ amap, float* __restrict__ interior,
                                                const float* __restrict__ apron, float p1, float p2) {
    __shared__ float sm[18 * 18 * 18];
    const int s = blockIdx.x;
    if (amap[s].leaf < 0) return;
    const float* in = interior + (size_t)s * 4096;
    const float* ap = apron + (size_t)s * kApronStride;
    for (int v = threadIdx.x; v < 4096; v += blockDim.x) {
        const int x = v & 15, y = (v >> 4) & 15, z = v >> 8;
        sm[((z + 1) * 18 + (y + 1)) * 18 + (x + 1)] = in[v];
    }
    for (int k = threadIdx.x; k < 1536; k += blockDim.x) {
        const int f = k >> 8, hi = (k >> 4) & 15, lo = k & 15, far = f & 1 ? 17 : 0;
        int x, y, z;
        if (f < 2) { x = far; y = lo + 1; z = hi + 1; }
        else if (f < 4) { y = far; x = lo + 1; z = hi + 1; }
        else { z = far; x = lo + 1; y = hi + 1; }
        sm[(z * 18 + y) * 18 + x] = ap[k];
    }
    __syncthreads();
    const double den = __dadd_rn((double)p1, 6.0);
    float* out = interior + (size_t)s * 4096;
    for (int v = threadIdx.x; v < 4096; v += blockDim.x) {
        const int x = (v & 15) + 1, y = ((v >> 4) & 15) + 1, z = (v >> 8) + 1;
        const int i = (z * 18 + y) * 18 + x;
        float a = __fmul_rn(p1, sm[i]);
        a = __fadd_rn(a, sm[i - 1]);
        a = __fadd_rn(a, sm[i + 1]);
        a = __fadd_rn(a, sm[i - 18]);
        a = __fadd_rn(a, sm[i + 18]);
        a = __fadd_rn(a, sm[i - 324]);
        a = __fadd_rn(a, sm[i + 324]);
        out[v] = __double2float_rn(__dadd_rn(__ddiv_rn((double)a, den), (double)p2));
    }
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }
inline unsigned gs_blocks(long long n, int t) {
    long long b = (n + t - 1) / t;
    long long cap = 152LL * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}
}  // namespace

void launch_assign_slots(Node* leaves, long long n, const uint32_t* scan, int ax, int ay, AtlasNode* amap,
                         cudaStream_t s) {
    if (n <= 0) return;
    k_assign_slots<<<counted(blocks_for(n, 256)), 256, 0, s>>>(leaves, n, scan, ax, ay, amap);
}
void launch_fill_u32(uint32_t* p, long long n, uint32_t v, cudaStream_t s) {
    if (n <= 0) return;
    k_fill_u32<<<counted(gs_blocks(n, 256)), 256, 0, s>>>(p, n, v);
}
void launch_apron(const TreeView& t, const LeafGrid& lg, const AtlasNode* amap, int used, int ax, int ay, int esize,
                  const void* interior, void* apron, uint32_t boundbits, const int* fill_only_bad, cudaStream_t s) {
    const bool fill_only = fill_only_bad != nullptr;
    if (used <= 0) return;
    if (esize == 4) {
        float b;
        memcpy(&b, &boundbits, 4);
        if (fill_only && lg.cells)
            k_apron_fill<float><<<counted((used + 7) / 8), 256, 0, s>>>(t, lg, amap, used, ax, ay, (const float*)interior,
                                                               (float*)apron, b, fill_only_bad);
        else
            k_apron<float><<<counted(used), 256, 0, s>>>(t, lg, amap, ax, ay, (const float*)interior, (float*)apron, b);
    } else {
        uint16_t b16 = (uint16_t)boundbits;
        __half_raw hr;
        hr.x = b16;
        if (fill_only && lg.cells)
            k_apron_fill<__half><<<counted((used + 7) / 8), 256, 0, s>>>(t, lg, amap, used, ax, ay, (const __half*)interior,
                                                                (__half*)apron, __half(hr), fill_only_bad);
        else
            k_apron<__half><<<counted(used), 256, 0, s>>>(t, lg, amap, ax, ay, (const __half*)interior, (__half*)apron,
                                                 __half(hr));
    }
}
void launch_export_bricks(const void* interior, const void* apron, int used, int esize, void* out, cudaStream_t s) {
    if (used <= 0) return;
    long long total = (long long)used * 5832;
    if (esize == 4)
        k_export_bricks<float><<<counted(gs_blocks(total, 256)), 256, 0, s>>>((const float*)interior, (const float*)apron, used,
                                                                     (float*)out);
    else
        k_export_bricks<__half><<<counted(gs_blocks(total, 256)), 256, 0, s>>>((const __half*)interior, (const __half*)apron,
                                                                       used, (__half*)out);
}
void launch_checksum_slots(const AtlasNode* amap, int used, int dtype, const void* interior, double* partials,
                           double* out, cudaStream_t s, int blocks_per_sm) {
    if (used > 0) {
        unsigned blocks = (unsigned)std::min(used, 152 * std::max(blocks_per_sm, 1));
        if (dtype == 3)
            k_slot_sums<float><<<counted(blocks), 256, 0, s>>>(amap, used, (const float*)interior, partials);
        else if (dtype == 100)
            k_slot_sums<__half><<<counted(blocks), 256, 0, s>>>(amap, used, (const __half*)interior, partials);
        else
            k_slot_sums<__nv_bfloat16><<<counted(blocks), 256, 0, s>>>(amap, used, (const __nv_bfloat16*)interior, partials);
    }
    k_sum_partials<<<counted(1), 1024, 0, s>>>(partials, used, out);
}
void launch_slab_pack(const void* interior, const void* apron, int esize, int ax, int ay, int bz, long long valid,
                      void* slab, cudaStream_t s) {
    long long n = (long long)ax * 18 * ay * 18 * 18;
    if (esize == 4)
        k_slab_pack<float><<<counted(gs_blocks(n, 256)), 256, 0, s>>>((const float*)interior, (const float*)apron, ax, ay, bz,
                                                             valid, (float*)slab);
    else
        k_slab_pack<__half><<<counted(gs_blocks(n, 256)), 256, 0, s>>>((const __half*)interior, (const __half*)apron, ax, ay,
                                                              bz, valid, (__half*)slab);
}
void launch_slab_unpack(const void* slab, int esize, int ax, int ay, int bz, void* interior, void* apron,
                        cudaStream_t s) {
    long long n = (long long)ax * 18 * ay * 18 * 18;
    if (esize == 4)
        k_slab_unpack<float><<<counted(gs_blocks(n, 256)), 256, 0, s>>>((const float*)slab, ax, ay, bz, (float*)interior,
                                                               (float*)apron);
    else
        k_slab_unpack<__half><<<counted(gs_blocks(n, 256)), 256, 0, s>>>((const __half*)slab, ax, ay, bz, (__half*)interior,
                                                                (__half*)apron);
}
void launch_neighbors(const TreeView& t, const LeafGrid& lg, long long n, int d, int* table, cudaStream_t s) {
    if (n <= 0) return;
    k_neighbors<<<counted(blocks_for(n, 128)), 128, 0, s>>>(t, lg, n, d, table);
}
void launch_apron_faces(const Node* leaves, const AtlasNode* amap, int used, int ax, int ay, const int* table,
                        int esize, void* interior, void* apron, cudaStream_t s) {
    if (used <= 0) return;
    if (esize == 4)
        k_apron_faces<float><<<counted(used), 128, 0, s>>>(leaves, amap, used, ax, ay, table, (float*)interior, (float*)apron);
    else
        k_apron_faces<__half><<<counted(used), 128, 0, s>>>(leaves, amap, used, ax, ay, table, (__half*)interior,
                                                   (__half*)apron);
}
void launch_smooth(const AtlasNode* amap, int used, float* interior, const float* apron, float p1, float p2,
                   cudaStream_t s) {
    if (used <= 0) return;
    k_smooth<<<counted(used), 256, 0, s>>>(amap, interior, apron, p1, p2);
}
void launch_fill_interior(const AtlasNode* amap, int used, int dtype, void* interior, float value, cudaStream_t s) {
    if (used <= 0) return;
    long long total = (long long)used * 4096;
    if (dtype == 3)
        k_fill_interior<float><<<counted(gs_blocks(total, 256)), 256, 0, s>>>(amap, used, (float*)interior, value);
    else if (dtype == 100)
        k_fill_interior<__half><<<counted(gs_blocks(total, 256)), 256, 0, s>>>(amap, used, (__half*)interior, value);
    else
        k_fill_interior<__nv_bfloat16><<<counted(gs_blocks(total, 256)), 256, 0, s>>>(amap, used, (__nv_bfloat16*)interior,
                                                                            value);
}

int noalloc_max_slots() { return kNoAllocMaxSlots; }

cudaError_t checksum_noalloc(const AtlasNode* amap, int used, int dtype, const void* interior, double* dev_out,
                             cudaStream_t s) {
    // device address of the static scratch, taken once per device with that device current
    static std::mutex mu;
    static double* addr[128] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
    double* partials = nullptr;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_slot_partials);
            if (e != cudaSuccess) return e;
            addr[dev] = static_cast<double*>(p);
        }
        partials = addr[dev];
    }
    if (used < 0 || used > kNoAllocMaxSlots) return cudaErrorInvalidValue;
    // the same launches as gbvdb_checksum, so both give the same bits; launch errors
    // are checked by the caller like every other launch of the grid
    launch_checksum_slots(amap, used, dtype, interior, partials, dev_out, s);
    return cudaSuccess;
}

}  // namespace gbvdb
