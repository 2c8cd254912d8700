// topology.cu -- bounding box, per-level node keys, node allocation, linking.
//
// Replaces (reference file:line):
//   GetBoundingBox + gvdbSplitPos + 6 Thrust min/max   VG.cpp:5404-5467, ND.cuh:507-517
//   gvdbCalcBrickId + Thrust sort + FindUnique/Compact  PT.cuh:352-382, 336-350, 934-943
//   gvdbCalcExtraBrickId                                PT.cuh:467-512
//   gvdbCalcIncreExtraBrickId (+ node markers)          PT.cuh:420-465
//   host node-allocation loop                           VG.cpp:1288-1332, 958-989, 1087-1112
//   gvdbLinkBricks / gvdbDelinkLeafBricks / gvdbDelinkBricks  ND.cuh:401-505
//
// Keys are deduplicated in per-level bitmaps over the key domain instead of a
// 64-bit sort: bit i of a level's bitmap is node coordinate (x,y,z) with
// i = ((x-lo)*ny + (y-lo))*nz + (z-lo), so ascending bit order equals the
// reference's ascending u64 key order {lev, x, y, z} and a popcount prefix sum
// gives each unique key its pool slot directly.
#include <algorithm>

#include "kernels.h"

namespace gbvdb {

namespace {

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

__global__ void k_bbox(PointSrc p, float3 orig, int* out6) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    const float o[3] = {orig.x, orig.y, orig.z};
    long long first = 0;
    if (p.stride == 12 && p.off == 0 && ((uintptr_t)p.base & 15) == 0) {
        // packed float3 on a 16-byte boundary: four points per three 16-byte loads
        const float4* v = reinterpret_cast<const float4*>(p.base);
        const long long groups = p.n >> 2;
        const long long gstride = (long long)gridDim.x * blockDim.x;
        // two groups per thread per step: six 16-byte loads in flight
        for (long long g0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; g0 < groups; g0 += 2 * gstride) {
            float4 q[6];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const long long gi = g0 + u * gstride;
                const bool in = gi < groups;
#pragma unroll
                for (int k = 0; k < 3; k++)
                    q[3 * u + k] = in ? __ldg(v + 3 * gi + k) : make_float4(INFINITY, INFINITY, INFINITY, INFINITY);
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const bool in = g0 + u * gstride < groups;
                const float e[12] = {q[3 * u].x,     q[3 * u].y,     q[3 * u].z,     q[3 * u].w,
                                     q[3 * u + 1].x, q[3 * u + 1].y, q[3 * u + 1].z, q[3 * u + 1].w,
                                     q[3 * u + 2].x, q[3 * u + 2].y, q[3 * u + 2].z, q[3 * u + 2].w};
                if (!in) continue;
#pragma unroll
                for (int k = 0; k < 12; k++) {
                    const float w = fadd(e[k], o[k % 3]);
                    mn[k % 3] = fminf(mn[k % 3], w);
                    mx[k % 3] = fmaxf(mx[k % 3], w);
                }
            }
        }
        first = groups << 2;
    }
    for (long long i = first + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n;
         i += (long long)gridDim.x * blockDim.x) {
        float x, y, z;
        load_pos(p.base, i, p.stride, p.off, x, y, z);
        float w[3] = {fadd(x, orig.x), fadd(y, orig.y), fadd(z, orig.z)};
#pragma unroll
        for (int a = 0; a < 3; a++) { mn[a] = fminf(mn[a], w[a]); mx[a] = fmaxf(mx[a], w[a]); }
    }
    __shared__ float red[6][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; a++) { mn[a] = warp_min(mn[a]); mx[a] = warp_max(mx[a]); }
    if (lane == 0)
        for (int a = 0; a < 3; a++) { red[a][warp] = mn[a]; red[3 + a][warp] = mx[a]; }
    __syncthreads();
    if (warp == 0) {
        for (int a = 0; a < 3; a++) {
            float v0 = lane < nw ? red[a][lane] : INFINITY;
            float v1 = lane < nw ? red[3 + a][lane] : -INFINITY;
            v0 = warp_min(v0);
            v1 = warp_max(v1);
            if (lane == 0) {
                atomicMin(out6 + a, f2o(v0));
                atomicMax(out6 + 3 + a, f2o(v1));
            }
        }
    }
}

// set bit `idx` of the bitmap, skipping the atomic when the bit is already visible
__device__ __forceinline__ void set_bit(uint32_t* bm, long long idx) {
    uint32_t* w = bm + (idx >> 5);
    uint32_t bit = 1u << (idx & 31);
    if ((__ldcg(w) & bit) == 0) atomicOr(w, bit);
}

__device__ __forceinline__ long long key_bit(const KeyDomain& d, int x, int y, int z) {
    int rx = x - d.lo[0], ry = y - d.lo[1], rz = z - d.lo[2];
    if (rx < 0 || ry < 0 || rz < 0 || rx >= d.dim[0] || ry >= d.dim[1] || rz >= d.dim[2]) return -1;
    return d.bitbase + ((long long)rx * d.dim[1] + ry) * d.dim[2] + rz;
}

// ---- sparse key sets (KeyHash): linear probing over a power-of-two table; a key is
// inserted once (compare-and-swap into a free slot).  A probe run longer than
// kKeyProbes (the table too full) sets err bit 4 and the host grows the table and runs
// the pass again.
constexpr int kKeyProbes = 512;

// splitmix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", 2014): spreads the x-major bit indices of a box over the table
__device__ __forceinline__ unsigned long long key_mix(unsigned long long x) {
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ void hash_insert(const KeyHash& h, unsigned long long key, int* err) {
    unsigned long long s = key_mix(key) & h.mask;
    for (int probe = 0; probe < kKeyProbes; probe++) {
        unsigned long long cur = __ldcg(h.tab + s);
        if (cur == key) return;
        if (cur == kKeyEmpty) {
            cur = atomicCAS(h.tab + s, kKeyEmpty, key);
            if (cur == kKeyEmpty || cur == key) return;
        }
        s = (s + 1) & h.mask;
    }
    atomicOr(err, 4);
}

// node coordinates (relative to the domain) of the level's local bit index li
__device__ __forceinline__ void key_coords(const KeyDomain& d, long long li, int& rx, int& ry, int& rz) {
    rz = (int)(li % d.dim[2]);
    const long long q = li / d.dim[2];
    ry = (int)(q % d.dim[1]);
    rx = (int)(q / d.dim[1]);
}

// gvdbCalcBrickId (PT.cuh:352-382): key of every level below the root for every
// point whose coordinates are all >= 0.  Bits are collected per block in shared memory
// for the words [sw0, nwords) of the bitmap when those fit (8,192 words at most): the whole
// bitmap (sw0 = 0), or, when the leaf level is too large, the levels above it (sw0 = their
// first word), whose few words every point of the cloud would otherwise test in L2.
__global__ void k_keys_pass1(PointSrc p, float3 orig, int depth, KeyDomains dom, TreeView tv, uint32_t* bm,
                             long long nwords, long long sw0, KeyHash kh, int* err) {
    extern __shared__ uint32_t sbm[];
    const bool use_smem = kh.tab == nullptr && nwords - sw0 <= 8192;
    if (use_smem) {
        for (long long k = threadIdx.x; k < nwords - sw0; k += blockDim.x) sbm[k] = 0;
        __syncthreads();
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (long long)gridDim.x * blockDim.x) {
        float x, y, z;
        load_pos(p.base, i, p.stride, p.off, x, y, z);
        float w0 = fadd(x, orig.x), w1 = fadd(y, orig.y), w2 = fadd(z, orig.z);
        if (w0 < 0 || w1 < 0 || w2 < 0) continue;
        for (int lev = 0; lev < depth; lev++) {
            int lg = tv.lgrange[lev];
            long long b = key_bit(dom.d[lev], cover_coord(w0, lg), cover_coord(w1, lg), cover_coord(w2, lg));
            if (b < 0) { atomicOr(err, 1); continue; }
            if (kh.tab) {
                hash_insert(kh, (unsigned long long)b, err);
            } else if (use_smem && (b >> 5) >= sw0) {
                uint32_t bit = 1u << (b & 31);
                if (!(sbm[(b >> 5) - sw0] & bit)) atomicOr(&sbm[(b >> 5) - sw0], bit);
            } else {
                set_bit(bm, b);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (long long k = threadIdx.x; k < nwords - sw0; k += blockDim.x) {
            uint32_t v = sbm[k];
            if (v && (__ldcg(bm + sw0 + k) & v) != v) atomicOr(bm + sw0 + k, v);
        }
    }
}

// gvdbCalcExtraBrickId (hi_mul = 2, PT.cuh:467-512) and gvdbCalcIncreExtraBrickId
// (hi_mul = 1, PT.cuh:420-465) in two steps.  The reference tests every node
// position of every point's box against the tree.  Here (1) each point sets the
// bits of the node positions its box covers in a per-level "touched" bitmap, and
// (2) each touched position is resolved once: not reachable from the root -> a
// key; a reachable leaf -> its marker.  Same sets, far fewer tree lookups.
// Bits go to a per-block copy of the bitmap in shared memory when the whole
// bitmap fits (kTouchSmemWords), then one atomicOr per non-zero word: a dense
// region maps its many points onto a few words, which would otherwise be one hot
// L2 line.  Larger (sparser) bitmaps are set in global memory directly.
constexpr int kTouchSmemWords = 8192;

__device__ __forceinline__ void touch_bit(uint32_t* sbm, bool use_smem, uint32_t* touched, long long b) {
    if (use_smem) {
        uint32_t bit = 1u << (b & 31);
        if (!(sbm[b >> 5] & bit)) atomicOr(&sbm[b >> 5], bit);
    } else {
        set_bit(touched, b);
    }
}

// Work is flattened across the warp: each lane computes its point's per-axis
// ranges of node positions at a level, a warp prefix sum over the lanes' counts
// lays all (point, position) items out in one list, and the lanes then take
// consecutive items, so that boxes of 1 to 8 positions do not leave lanes idle.
// x / 2^lg * 2^lg with C truncation toward zero
__device__ __forceinline__ int trunc_mult(int x, int lg) {
    const long long v = x;
    return (int)(v >= 0 ? (v >> lg) << lg : -(((-v) >> lg) << lg));
}

__global__ void k_touch_box(TreeView t, PointSrc p, float3 orig, float radius, int hi_mul, int depth, int3 rlo,
                            int3 rhi, KeyDomains dom, uint32_t* touched, long long nwords, KeyHash th, int* err) {
    extern __shared__ uint32_t sbm[];
    const bool use_smem = th.tab == nullptr && nwords <= kTouchSmemWords;
    if (use_smem) {
        for (long long k = threadIdx.x; k < nwords; k += blockDim.x) sbm[k] = 0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long gwarp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const float hr = hi_mul == 2 ? __fmul_rn(2.0f, radius) : radius;
    for (long long base = gwarp * 32; base < p.n; base += nwarps * 32) {
        const long long i = base + lane;
        bool valid = i < p.n;
        int bmin[3] = {0, 0, 0}, bmax[3] = {-1, -1, -1};
        if (valid) {
            float x, y, z;
            load_pos(p.base, i, p.stride, p.off, x, y, z);
            float w[3] = {fadd(x, orig.x), fadd(y, orig.y), fadd(z, orig.z)};
            valid = !(w[0] < 0 || w[1] < 0 || w[2] < 0);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float fi = (float)(int)w[a];
                bmin[a] = (int)fsub(fi, radius);
                bmax[a] = (int)fadd(fi, hr);
            }
        }
        // level 0 only: the box positions of every upper level are the parents of the
        // level-0 ones (k_touch_up), since the ranges nest
        for (int lev = 0; lev < 1; lev++) {
            const int lg = t.lgrange[lev];
            const int rr = 1 << lg;
            int lo[3], cnt[3];
            const int rl[3] = {rlo.x, rlo.y, rlo.z}, rh[3] = {rhi.x - 1, rhi.y - 1, rhi.z - 1};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                lo[a] = trunc_mult(bmin[a], lg);  // x / rr * rr with C truncation, as the reference
                int hi = trunc_mult(bmax[a], lg);
                // positions outside the root are skipped: clip the range to it
                if (lo[a] < rl[a]) lo[a] += ((rl[a] - lo[a] + rr - 1) >> lg) << lg;
                if (hi > rh[a]) hi -= ((hi - rh[a] + rr - 1) >> lg) << lg;
                cnt[a] = valid && hi >= lo[a] ? ((hi - lo[a]) >> lg) + 1 : 0;
            }
            long long mine64 = (long long)cnt[0] * cnt[1] * cnt[2];
            if (mine64 > (1ll << 26)) {  // keeps the warp's item count within int
                atomicOr(err, 2);
                mine64 = 0;
            }
            const int mine = (int)mine64;
            int incl = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            for (int k0 = 0; k0 < total; k0 += 32) {
                const int k = k0 + lane;
                // owner lane: the first lane whose inclusive prefix exceeds k
                int owner = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    int cand = owner + step - 1;
                    int pv = __shfl_sync(0xFFFFFFFFu, incl, cand);
                    if (pv <= k) owner += step;
                }
                const int excl = __shfl_sync(0xFFFFFFFFu, incl - mine, owner);
                const int ocx = __shfl_sync(0xFFFFFFFFu, cnt[0], owner);
                const int ocy = __shfl_sync(0xFFFFFFFFu, cnt[1], owner);
                const int olx = __shfl_sync(0xFFFFFFFFu, lo[0], owner);
                const int oly = __shfl_sync(0xFFFFFFFFu, lo[1], owner);
                const int olz = __shfl_sync(0xFFFFFFFFu, lo[2], owner);
                const bool small = __all_sync(0xFFFFFFFFu, ocx <= 2 && ocy <= 2);
                if (k >= total) continue;
                const int li = k - excl;
                int ix, iy, iz;
                if (small) {  // 1 or 2 positions along x and y (nearly every box): shifts
                    const int sx = ocx - 1, sy = ocy - 1, t2 = li >> sx;
                    ix = li & sx;
                    iy = t2 & sy;
                    iz = t2 >> sy;
                } else {
                    ix = li % ocx;
                    iy = (li / ocx) % ocy;
                    iz = li / (ocx * ocy);
                }
                const int nx = olx + ix * rr, ny = oly + iy * rr, nz = olz + iz * rr;
                // guard: positions outside the root (the reference aliases them)
                if (nx < rlo.x || ny < rlo.y || nz < rlo.z || nx >= rhi.x || ny >= rhi.y || nz >= rhi.z) continue;
                long long b = key_bit(dom.d[lev], nx >> lg, ny >> lg, nz >> lg);
                if (b < 0) { atomicOr(err, 1); continue; }
                if (th.tab) hash_insert(th, (unsigned long long)b, err);
                else touch_bit(sbm, use_smem, touched, b);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (long long k = threadIdx.x; k < nwords; k += blockDim.x) {
            uint32_t v = sbm[k];
            if (v && (__ldcg(touched + k) & v) != v) atomicOr(touched + k, v);
        }
    }
}

// Level-0 box positions in two steps when every box reaches at most one node past
// the point's own (home) node on each side, i.e. radius and the box's upper reach
// are both at most the node range: (1) each point ORs into its home node's entry
// the 27-bit set of neighbour directions d = (dx, dy, dz) in {-1, 0, 1}^3 that its
// box covers (bit (dz+1)*9 + (dy+1)*3 + (dx+1)), after the same truncation and
// root clipping as the per-point walk; (2) a node position of the key domain is
// touched iff the entry of the node at -d has bit d.  The same set as the walk over
// every box position, for one load (and on a new combination an atomic) per point.
// The entries cover the level-0 key domain widened by one node on each side.
struct DirDomain {
    int lo[3];
    int dim[3];
};

// Four consecutive points per thread per step (load_pos4): their position loads, then
// their entry loads, are issued together (the pass is bound by the latency of that
// two-load chain).
// kIntR: radius and the upper reach hr are whole numbers (below 2^20), so for a point
// coordinate below 2^23 the box bounds int(float(ip) -/+ r) are ip -/+ r exactly, in
// integer arithmetic (the float form's conversions are what bound this pass's issue)
template <int kU, bool kIntR>
__global__ void k_touch_dirs(PointSrc p, float3 orig, float radius, float hr, int lg, int3 rlo, int3 rhi,
                             DirDomain dd, uint32_t* __restrict__ dirs, int* err) {
    static_assert(kU == 4, "four consecutive points per thread");
    const int ir = (int)radius, ihr = (int)hr;
    const int rr = 1 << lg;
    const int rl[3] = {rlo.x, rlo.y, rlo.z}, rh[3] = {rhi.x - 1, rhi.y - 1, rhi.z - 1};
    const long long ngroups = (p.n + 3) >> 2;
    for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups;
         gi += (long long)gridDim.x * blockDim.x) {
        const long long i0 = gi << 2;
        float w[kU][3];
        bool ok[kU];
        load_pos4(p, i0, w);
#pragma unroll
        for (int u = 0; u < kU; u++) {
            ok[u] = i0 + u < p.n;
            if (ok[u]) {
                w[u][0] = fadd(w[u][0], orig.x);
                w[u][1] = fadd(w[u][1], orig.y);
                w[u][2] = fadd(w[u][2], orig.z);
            }
        }
        uint32_t m27[kU];
        int ent[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            m27[u] = 0;
            ent[u] = -1;
            if (!ok[u] || w[u][0] < 0 || w[u][1] < 0 || w[u][2] < 0) continue;
            int m[3], hb[3];
            bool any = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const int ip = (int)w[u][a];
                int bl, bh;
                if (kIntR && ip < (1 << 23)) {
                    bl = ip - ir;
                    bh = ip + ihr;
                } else {
                    const float fi = (float)ip;
                    bl = (int)fsub(fi, radius);
                    bh = (int)fadd(fi, hr);
                }
                // x / rr * rr with C truncation (bl >= -(r + 1) and bh >= 0 stay far from
                // INT_MIN, so 32-bit negation is safe)
                int lo = bl >= 0 ? (bl >> lg) << lg : -(((-bl) >> lg) << lg);
                int hi = bh >= 0 ? (bh >> lg) << lg : -(((-bh) >> lg) << lg);
                if (lo < rl[a]) lo += ((rl[a] - lo + rr - 1) >> lg) << lg;
                if (hi > rh[a]) hi -= ((hi - rh[a] + rr - 1) >> lg) << lg;
                hb[a] = ip >> lg;
                const int l = (lo >> lg) - hb[a], h = (hi >> lg) - hb[a];
                any &= hi >= lo;
                m[a] = hi >= lo ? (((1 << (h - l + 1)) - 1) << (l + 1)) & 7 : 0;
            }
            if (!any) continue;
            // the product of the three 3-bit masks: bit (dz*9 + dy*3 + dx) for every
            // (dx, dy, dz) they hold; the shifted copies of a mask never overlap, so
            // multiplying by a sum of powers of two places them without carries
            const uint32_t ym = (uint32_t)m[0] * (uint32_t)((m[1] & 1) | ((m[1] & 2) << 2) | ((m[1] & 4) << 4));
            m27[u] = ym * (uint32_t)((m[2] & 1) | ((m[2] & 2) << 8) | ((m[2] & 4) << 16));
            const int rx = hb[0] - dd.lo[0], ry = hb[1] - dd.lo[1], rz = hb[2] - dd.lo[2];
            if ((unsigned)rx >= (unsigned)dd.dim[0] || (unsigned)ry >= (unsigned)dd.dim[1] ||
                (unsigned)rz >= (unsigned)dd.dim[2]) {
                atomicOr(err, 1);
                m27[u] = 0;
                continue;
            }
            ent[u] = (rx * dd.dim[1] + ry) * dd.dim[2] + rz;  // the table has < 2^28 entries
        }
        // the entries of a dense region are few and hot: read them through L1 (a copy from
        // before another point's atomic only makes this point repeat a bit: the OR is
        // idempotent, so the table ends the same)
        uint32_t cur[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) cur[u] = ent[u] >= 0 ? __ldca(dirs + ent[u]) : 0xFFFFFFFFu;
#pragma unroll
        for (int u = 0; u < kU; u++)
            if (ent[u] >= 0 && (cur[u] & m27[u]) != m27[u]) atomicOr(dirs + ent[u], m27[u]);
    }
}

// a lane per level-0 bit (position of the key domain), a warp per bitmap word
__global__ void k_touch_from_dirs(KeyDomain d, DirDomain dd, const uint32_t* __restrict__ dirs, uint32_t* touched) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long w = g >> 5, nw = (d.nbits + 31) >> 5;
    if (w >= nw) return;  // whole warps leave together (blockDim is a multiple of 32)
    const int b = (int)(g & 31);
    const long long li = w * 32 + b;
    bool hit = false;
    if (li < d.nbits) {
        const int rz = (int)(li % d.dim[2]);
        const long long q = li / d.dim[2];
        const int ry = (int)(q % d.dim[1]);
        const int rx = (int)(q / d.dim[1]);
        // entry of the home node at -dir, in the widened domain (offset 1 per axis)
        for (int dz = -1; dz <= 1 && !hit; dz++)
            for (int dy = -1; dy <= 1 && !hit; dy++)
                for (int dx = -1; dx <= 1 && !hit; dx++) {
                    const long long e = ((long long)(rx + 1 - dx) * dd.dim[1] + (ry + 1 - dy)) * dd.dim[2] + (rz + 1 - dz);
                    hit = (__ldg(dirs + e) >> ((dz + 1) * 9 + (dy + 1) * 3 + (dx + 1))) & 1u;
                }
    }
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
    if (b == 0) touched[(d.bitbase >> 5) + w] = mask;
}

// The same bits from the other side, for key domains much larger than the set of home
// positions (sparse clouds): a thread per entry of the direction table (a coalesced
// read); a non-zero entry sets, for each direction in its mask, the bit of the position
// at that direction (atomicOr into the touched words, cleared before the pass).  The gather
// form above visits 27 entries for every position of the domain, most of them empty there.
__global__ void k_touch_dirs_scatter(KeyDomain d, DirDomain dd, const uint32_t* __restrict__ dirs, long long nent,
                                     uint32_t* touched) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nent; e += stride) {
        uint32_t m = __ldg(dirs + e);
        if (!m) continue;
        const int hz = (int)(e % dd.dim[2]);
        const long long q = e / dd.dim[2];
        const int hy = (int)(q % dd.dim[1]), hx = (int)(q / dd.dim[1]);
        while (m) {  // the entry's home position, domain coordinates h - 1, plus each direction
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const int px = hx - 1 + (k % 3 - 1), py = hy - 1 + ((k / 3) % 3 - 1), pz = hz - 1 + (k / 9 - 1);
            if ((unsigned)px >= (unsigned)d.dim[0] || (unsigned)py >= (unsigned)d.dim[1] || (unsigned)pz >= (unsigned)d.dim[2])
                continue;
            const long long li = ((long long)px * d.dim[1] + py) * d.dim[2] + pz;
            atomicOr(touched + (d.bitbase >> 5) + (li >> 5), 1u << (li & 31));
        }
    }
}

// Box positions of level lev from those of lev-1: every touched position's parent.  For
// one box, trunc(b / R_lev) * R_lev .. trunc(e / R_lev) * R_lev is the set of parents
// of trunc(b / R_lev-1) * R_lev-1 .. trunc(e / R_lev-1) * R_lev-1 once both are clipped
// to the root (coordinates >= 0, where truncation is floor and the ranges nest).
// The parent level's bitmap is small (a parent covers 8^3 or more children), so many
// children of one warp and block share its words: the bits are ORed per block in
// shared memory when the parent bitmap fits (kTouchSmemWords), then one atomicOr per
// non-zero word; a same-word atomic per child would serialise on a few L2 lines.
__global__ void k_touch_up(KeyDomain child, KeyDomain parent, int lgres, uint32_t* touched, int* err) {
    extern __shared__ uint32_t sbm[];
    const long long pw0 = parent.bitbase >> 5, pnw = (parent.nbits + 31) >> 5;
    const bool use_smem = pnw <= kTouchSmemWords;
    if (use_smem) {
        for (long long k = threadIdx.x; k < pnw; k += blockDim.x) sbm[k] = 0;
        __syncthreads();
    }
    // a lane per bit of the child level, warps striding over its bitmap words (the grid
    // is capped, so that few blocks clear and flush the parent copy in shared memory)
    const long long w0 = child.bitbase >> 5, nw = (child.nbits + 31) >> 5;
    const int b = (int)(threadIdx.x & 31);
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += wstride) {
        if (!((touched[w0 + w] >> b) & 1u)) continue;
        const long long li = w * 32 + b;
        const int rz = (int)(li % child.dim[2]);
        const long long q = li / child.dim[2];
        const int ry = (int)(q % child.dim[1]);
        const int rx = (int)(q / child.dim[1]);
        const long long pb = key_bit(parent, (child.lo[0] + rx) >> lgres, (child.lo[1] + ry) >> lgres,
                                     (child.lo[2] + rz) >> lgres);
        if (pb < 0) {
            atomicOr(err, 1);
        } else if (use_smem) {
            const long long lb = pb - parent.bitbase;
            atomicOr(&sbm[lb >> 5], 1u << (lb & 31));
        } else {
            set_bit(touched, pb);
        }
    }
    if (use_smem) {
        __syncthreads();
        for (long long k = threadIdx.x; k < pnw; k += blockDim.x) {
            const uint32_t v = sbm[k];
            if (v && (__ldcg(touched + pw0 + k) & v) != v) atomicOr(touched + pw0 + k, v);
        }
    }
}

// a warp per touched-bitmap word of levels [0, depth) (their words follow each other:
// each level's bitbase is word aligned; warps stride over the nw_all words, the grid
// capped, so that the empty words of a sparse domain cost a load each), a lane per bit:
// getPosParent(pos, lev) for every touched position; missing -> key bit, reachable
// leaf -> marker
__global__ void k_resolve_touched(TreeView t, LeafGrid lg, int depth, KeyDomains dom, long long nw_all,
                                  const uint32_t* __restrict__ touched, uint32_t* keys, int* markers) {
    const int b = (int)(threadIdx.x & 31);
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wg < nw_all; wg += wstride) {
        const uint32_t bits = touched[wg];
        if (!bits) continue;  // (the whole warp: one word per warp)
        int lev = -1;
        for (int l = 0; l < depth; l++)
            if (wg >= (dom.d[l].bitbase >> 5) && wg < (dom.d[l].bitbase >> 5) + ((dom.d[l].nbits + 31) >> 5)) lev = l;
        if (lev < 0) continue;
        const KeyDomain& d = dom.d[lev];
        const long long w0 = d.bitbase >> 5, w = wg - w0;
        bool miss = false;
        if ((bits >> b) & 1u) {
            const int lgr = t.lgrange[lev];
            const long long li = w * 32 + b;
            const int rz = (int)(li % d.dim[2]);
            const long long q = li / d.dim[2];
            const int ry = (int)(q % d.dim[1]);
            const int rx = (int)(q / d.dim[1]);
            const int px = (d.lo[0] + rx) << lgr, py = (d.lo[1] + ry) << lgr, pz = (d.lo[2] + rz) << lgr;
            const long long pid = (lev == 0) ? lookup_leaf(lg, t, px, py, pz) : get_pos_parent(t, px, py, pz, lev);
            if (pid < 0) miss = true;
            else if (lev == 0 && markers) markers[pid] = 1;
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, miss);
        if (b == 0 && m) keys[w0 + w] = m;  // each word has one owner warp
    }
}

// k_touch_up over the sparse form: a thread per table slot; the level-(lev-1)
// entries insert their parents (entries this launch adds are of level lev and skipped)
__global__ void k_touch_up_hashed(KeyHash th, KeyDomain child, KeyDomain parent, int lgres, int* err) {
    const unsigned long long cap = th.mask + 1;
    const unsigned long long lo = (unsigned long long)child.bitbase, hi = lo + (unsigned long long)child.nbits;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < cap;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long e = __ldcg(th.tab + s);
        if (e == kKeyEmpty || e < lo || e >= hi) continue;
        int rx, ry, rz;
        key_coords(child, (long long)(e - lo), rx, ry, rz);
        const long long pb = key_bit(parent, (child.lo[0] + rx) >> lgres, (child.lo[1] + ry) >> lgres,
                                     (child.lo[2] + rz) >> lgres);
        if (pb < 0) atomicOr(err, 1);
        else hash_insert(th, (unsigned long long)pb, err);
    }
}

// k_resolve_touched over the sparse form, all levels in one launch: a thread per
// touched-table slot; missing -> key, reachable leaf -> marker
__global__ void k_resolve_hashed(TreeView t, LeafGrid lg, int depth, KeyDomains dom, KeyHash th, KeyHash kh,
                                 int* markers, int* err) {
    const unsigned long long cap = th.mask + 1;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < cap;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long e = th.tab[s];
        if (e == kKeyEmpty) continue;
        int lev = -1;
        for (int l = 0; l < depth; l++)
            if (e >= (unsigned long long)dom.d[l].bitbase &&
                e < (unsigned long long)(dom.d[l].bitbase + dom.d[l].nbits))
                lev = l;
        if (lev < 0) continue;
        const KeyDomain& d = dom.d[lev];
        int rx, ry, rz;
        key_coords(d, (long long)e - d.bitbase, rx, ry, rz);
        const int lgr = t.lgrange[lev];
        const int px = (d.lo[0] + rx) << lgr, py = (d.lo[1] + ry) << lgr, pz = (d.lo[2] + rz) << lgr;
        const long long pid = (lev == 0) ? lookup_leaf(lg, t, px, py, pz) : get_pos_parent(t, px, py, pz, lev);
        if (pid < 0) hash_insert(kh, e, err);
        else if (lev == 0 && markers) markers[pid] = 1;
    }
}

// occupied slots -> out (warp-aggregated append; the table's capacity is a multiple of 32)
__global__ void k_hash_compact(KeyHash h, unsigned long long* __restrict__ out, unsigned int* count) {
    const unsigned long long cap = h.mask + 1;
    const int lane = threadIdx.x & 31;
    const unsigned long long nw = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long w = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w * 32 < cap;
         w += nw) {
        const unsigned long long e = h.tab[w * 32 + lane];
        const bool occ = e != kKeyEmpty;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, occ);
        if (!m) continue;
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(count, (unsigned)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (occ) out[base + __popc(m & ((1u << lane) - 1u))] = e;
    }
}

__global__ void k_key_bounds(const unsigned long long* __restrict__ sorted, const unsigned int* n, KeyDomains dom,
                             int depth, unsigned int* at) {
    const int l = threadIdx.x;
    if (l > depth) return;
    const unsigned int cnt = *n;
    if (l == depth) {
        at[l] = cnt;
        return;
    }
    const unsigned long long key = (unsigned long long)dom.d[l].bitbase;
    unsigned int lo = 0, hi = cnt;  // first index with sorted[i] >= key
    while (lo < hi) {
        const unsigned int mid = lo + ((hi - lo) >> 1);
        if (sorted[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    at[l] = lo;
}

// the node record of local key li of level lev (SetupNode, VG.cpp:2512-2524) at pool index idx
__device__ __forceinline__ Node key_node(int lev, int lgrange, const KeyDomain& d, long long li, long long idx) {
    int rx, ry, rz;
    key_coords(d, li, rx, ry, rz);
    Node n;
    n.lev = (uint8_t)lev;
    n.flags = 1;
    n.prio = 0;
    n.pad = 0;
    n.pos[0] = (d.lo[0] + rx) << lgrange;
    n.pos[1] = (d.lo[1] + ry) << lgrange;
    n.pos[2] = (d.lo[2] + rz) << lgrange;
    n.value[0] = n.value[1] = n.value[2] = -1;
    n.vrange[0] = n.vrange[1] = n.vrange[2] = 0.f;
    n.parent = kUndefL;
    n.childlist = lev > 0 ? elem(1, lev, (unsigned long long)idx) : kUndefL;
    n.mask = 0;
    return n;
}

// one thread per bitmap word of one level; every set bit becomes a node record
// (SetupNode, VG.cpp:2512-2524) at pool index base + rank
__global__ void k_alloc_nodes(const uint32_t* __restrict__ bm, const uint32_t* __restrict__ prefix, long long word0,
                              long long nwords, int lev, int lgrange, KeyDomain d, long long base, Node* nodes) {
    // a lane per bit, warps striding over the words (the grid is capped: a sparse level's
    // empty words cost a load each): rank = the word's prefix + the set bits below this one
    const int b = (int)(threadIdx.x & 31);
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwords; w += wstride) {
        const uint32_t bits = bm[word0 + w];
        if (!((bits >> b) & 1u)) continue;
        const long long rank = (long long)prefix[word0 + w] - (long long)prefix[word0] + __popc(bits & ((1u << b) - 1u));
        const long long li = (word0 + w) * 32 + b - d.bitbase;  // bitbase is word aligned
        nodes[base + rank] = key_node(lev, lgrange, d, li, base + rank);
    }
}

// the sparse form's allocation: a thread per sorted key of the level
__global__ void k_alloc_nodes_sorted(const unsigned long long* __restrict__ sorted, long long first, long long count,
                                     int lev, int lgrange, KeyDomain d, long long base, Node* nodes) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const long long li = (long long)sorted[first + i] - d.bitbase;
    nodes[base + i] = key_node(lev, lgrange, d, li, base + i);
}

__global__ void k_write_node(Node* dst, Node v) { *dst = v; }

// gvdbLinkBricks (ND.cuh:470-505), in two launches.  When two flagged nodes of
// one level map to the same child slot (duplicates the reference creates after
// its top-level quirk), the reference's single kernel races on that slot; here
// the highest pool index wins, which is what a sequential pass over the nodes
// leaves behind.  claim: set mParent, record the slot, atomicMax the index.
__global__ void k_link_claim(TreeView t, int lev, long long count, int* tag, long long* slot_of) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    slot_of[i] = -1;
    Node* node = t.nodes[lev] + i;
    if (!node->flags) return;
    long long pid = get_parent(t, lev + 1, node->pos[0], node->pos[1], node->pos[2]);
    if (pid < 0) return;
    const Node* pn = t.nodes[lev + 1] + pid;
    int sh = t.lgrange[lev + 1] - t.lgres[lev + 1];
    int r = t.res[lev + 1];
    long long px = ((long long)node->pos[0] - pn->pos[0]) >> sh;
    long long py = ((long long)node->pos[1] - pn->pos[1]) >> sh;
    long long pz = ((long long)node->pos[2] - pn->pos[2]) >> sh;
    if (px > r || px < 0 || py > r || py < 0 || pz > r || pz < 0) return;
    int b = (int)((pz * r + py) * r + px);
    node->parent = ((unsigned long long)pid << 16) | ((unsigned long long)(lev + 1) << 8);
    unsigned long long cndx = pn->childlist >> 16;
    if ((long long)cndx >= t.ncnt[lev + 1]) return;
    long long slot = (long long)(cndx << (3 * t.lgres[lev + 1])) + b;
    slot_of[i] = slot;
    atomicMax(tag + slot, (int)i);
}

__global__ void k_link_write(TreeView t, int lev, long long count, const int* tag, const long long* slot_of) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    long long slot = slot_of[i];
    if (slot < 0 || tag[slot] != (int)i) return;
    t.clist[lev + 1][slot] = ((unsigned long long)i << 16) | ((unsigned long long)lev << 8);
}

// one thread per leaf: the leaf reachable at its own position is entered in the grid
__global__ void k_build_leaf_grid(TreeView t, long long n, int* cells, int3 lo, int3 dim, int lgrange0) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Node* nd = t.nodes[0] + i;
    long long r = get_pos_leaf(t, nd->pos[0], nd->pos[1], nd->pos[2]);
    if (r != i) return;
    int bx = (nd->pos[0] >> lgrange0) - lo.x, by = (nd->pos[1] >> lgrange0) - lo.y, bz = (nd->pos[2] >> lgrange0) - lo.z;
    if ((unsigned)bx >= (unsigned)dim.x || (unsigned)by >= (unsigned)dim.y || (unsigned)bz >= (unsigned)dim.z) return;
    cells[((long long)bx * dim.y + by) * dim.z + bz] = (int)i;
}

// the setup of an incremental pass in one launch: the leaf markers (InitMarkers:
// 0, or the old flags when accumulating), the key pass's error flag and kept-leaf
// counter cleared, and (bbox6 set) the bounds' initial values (min +inf, max -inf as
// ordered ints)
__global__ void k_incr_setup(const Node* leaves, long long n, int* markers, int accum, int* err,
                             unsigned long long* kept, int* bbox6) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) markers[i] = accum ? (int)leaves[i].flags : 0;
    if (i == 0) {
        *err = 0;
        *kept = 0ull;
        if (bbox6) {
            for (int a = 0; a < 3; a++) {
                bbox6[a] = 0x7F800000;
                bbox6[3 + a] = (int)(0xFF800000u ^ 0x7FFFFFFFu);
            }
        }
    }
}

__global__ void k_apply_markers(Node* leaves, long long n, const int* markers) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) leaves[i].flags = (uint8_t)markers[i];
}

// gvdbDelinkLeafBricks (ND.cuh:401-429)
__global__ void k_delink_leaf(TreeView t, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Node* node = t.nodes[0] + i;
    if (node->flags) return;
    if (node->parent == kUndef64) return;
    long long pid = get_parent(t, 1, node->pos[0], node->pos[1], node->pos[2]);
    if (pid < 0) { node->parent = kUndef64; return; }
    const Node* pn = t.nodes[1] + pid;
    int sh = t.lgrange[1] - t.lgres[1];
    int r = t.res[1];
    long long px = ((long long)node->pos[0] - pn->pos[0]) >> sh;
    long long py = ((long long)node->pos[1] - pn->pos[1]) >> sh;
    long long pz = ((long long)node->pos[2] - pn->pos[2]) >> sh;
    int b = (int)((pz * r + py) * r + px);
    node->parent = kUndef64;
    unsigned long long cndx = pn->childlist >> 16;
    t.clist[1][(cndx << (3 * t.lgres[1])) + b] = kUndef64;
}

// gvdbDelinkBricks (ND.cuh:431-467)
__global__ void k_delink_upper(TreeView t, int lev, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Node* node = t.nodes[lev] + i;
    if (node->parent == kUndef64) { node->flags = 0; return; }
    const unsigned long long* cl = t.clist[lev] + ((unsigned long long)i << (3 * t.lgres[lev]));
    const int len = 1 << (3 * t.lgres[lev]);
    for (int k = 0; k < len; k++)
        if (cl[k] != kUndef64) { node->flags = 1; return; }
    node->flags = 0;
    long long pid = get_parent(t, lev + 1, node->pos[0], node->pos[1], node->pos[2]);
    if (pid < 0) { node->parent = kUndef64; return; }
    const Node* pn = t.nodes[lev + 1] + pid;
    int sh = t.lgrange[lev + 1] - t.lgres[lev + 1];
    int r = t.res[lev + 1];
    long long px = ((long long)node->pos[0] - pn->pos[0]) >> sh;
    long long py = ((long long)node->pos[1] - pn->pos[1]) >> sh;
    long long pz = ((long long)node->pos[2] - pn->pos[2]) >> sh;
    int b = (int)((pz * r + py) * r + px);
    node->parent = kUndef64;
    unsigned long long cndx = pn->childlist >> 16;
    t.clist[lev + 1][(cndx << (3 * t.lgres[lev + 1])) + b] = kUndef64;
}

__global__ void k_count_flags(const Node* nodes, long long n, unsigned long long* out) {
    unsigned c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c += nodes[i].flags ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

// The key-count readback in one copy: out[l] = the prefix at level l's first word
// (l <= nlev; the last entry is the total), out[16] = the pass's error flag, out[18..19]
// = the kept-leaf count (u64), out[20..25] = the point bounds (when given)
__global__ void k_stage_counts(const uint32_t* __restrict__ pscan, CountStage st, uint32_t* __restrict__ out) {
    const int t = threadIdx.x;
    if (t <= st.nlev) out[t] = pscan[st.words[t]];
    if (t == 16) out[16] = (uint32_t)*st.err;
    if (t == 17 && st.kept) *reinterpret_cast<unsigned long long*>(out + 18) = *st.kept;
    if (t >= 20 && t < 26 && st.bbox) out[t] = (uint32_t)st.bbox[t - 20];
}

// leaves an incremental pass keeps flagged: the non-zero markers
__global__ void k_count_markers(const int* markers, long long n, unsigned long long* out) {
    unsigned c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c += markers[i] ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

// ComputeBounds (VG.cpp:1792-1816): both corners start at the position of leaf 0 of
// the pool (flagged or not); every flagged leaf widens them by [pos, pos + range0).
// One block; out6 = {min xyz, max xyz}, written whole (no initialisation needed).
__global__ void __launch_bounds__(1024) k_leaf_bounds(const Node* leaves, long long n, int lgrange0, int* out6) {
    __shared__ int red[6][32];
    int v[6];
    for (int a = 0; a < 3; a++) v[a] = v[3 + a] = leaves[0].pos[a];
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const Node& nd = leaves[i];
        if (!nd.flags) continue;
        for (int a = 0; a < 3; a++) {
            v[a] = min(v[a], nd.pos[a]);
            v[3 + a] = max(v[3 + a], nd.pos[a] + (1 << lgrange0));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 6; k++) {
        const int r = k < 3 ? __reduce_min_sync(0xFFFFFFFFu, v[k]) : __reduce_max_sync(0xFFFFFFFFu, v[k]);
        if (lane == 0) red[k][warp] = r;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x, nw = (blockDim.x + 31) >> 5;
        int r = red[k][0];
        for (int w = 1; w < nw; w++) r = k < 3 ? min(r, red[k][w]) : max(r, red[k][w]);
        out6[k] = r;
    }
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }
inline unsigned grid_stride_blocks(long long n, int t) {
    long long b = (n + t - 1) / t;
    long long cap = 152LL * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}
}  // namespace

void launch_bbox(PointSrc p, float3 orig, int* out6, cudaStream_t s) {
    // at most 4 blocks per SM: each block ends with six same-address atomics
    const unsigned b = std::min<unsigned>(grid_stride_blocks(p.n, 512), 152u * 4u);
    k_bbox<<<counted(b), 512, 0, s>>>(p, orig, out6);
}
void launch_keys_pass1(const TreeView& t, PointSrc p, float3 orig, int depth, const KeyDomains& dom,
                       uint32_t* bitmap, const KeySets& ks, int* err, cudaStream_t s) {
    long long nwords = 0;
    for (int lev = 0; lev < depth; lev++) nwords = std::max(nwords, (dom.d[lev].bitbase + dom.d[lev].nbits + 31) >> 5);
    // the words staged in shared memory: all, else those of the levels above the leaves
    // (level bit bases are multiples of 32)
    long long w0 = 0;
    if (nwords > 8192 && depth > 1) w0 = dom.d[1].bitbase >> 5;
    size_t smem = !ks.keys.tab && nwords - w0 <= 8192 ? (size_t)(nwords - w0) * 4 : 0;
    unsigned blocks = smem ? std::min<unsigned>(grid_stride_blocks(p.n, 256), 152u * 4u) : grid_stride_blocks(p.n, 256);
    k_keys_pass1<<<counted(blocks), 256, smem, s>>>(p, orig, depth, dom, t, bitmap, nwords, w0, ks.keys, err);
}
long long touch_dirs_words(const KeyDomains& dom) {
    return (long long)(dom.d[0].dim[0] + 2) * (dom.d[0].dim[1] + 2) * (dom.d[0].dim[2] + 2);
}

void launch_keys_box(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 orig, float radius, int hi_mul,
                     int depth, int root_lo[3], int root_hi[3], const KeyDomains& dom, uint32_t* touched,
                     uint32_t* bitmap, int* markers, int* err, uint32_t* dirs, const KeySets& ks,
                     long long home_hint, cudaStream_t s) {
    int3 rlo = make_int3(root_lo[0], root_lo[1], root_lo[2]);
    int3 rhi = make_int3(root_hi[0], root_hi[1], root_hi[2]);
    const float hr = hi_mul == 2 ? 2.0f * radius : radius;
    const float rr = (float)(1 << t.lgrange[0]);
    if (ks.touched.tab) {
        // sparse form: the per-point walk into the touched table, parents level by level,
        // then every touched position resolved in one pass
        k_touch_box<<<counted(grid_stride_blocks(p.n, 256)), 256, 0, s>>>(t, p, orig, radius, hi_mul, depth, rlo, rhi, dom,
                                                                 nullptr, 0, ks.touched, err);
        const unsigned long long cap = ks.touched.mask + 1;
        for (int lev = 1; lev < depth; lev++)
            k_touch_up_hashed<<<counted(grid_stride_blocks((long long)cap, 256)), 256, 0, s>>>(ks.touched, dom.d[lev - 1],
                                                                                      dom.d[lev], t.lgres[lev], err);
        k_resolve_hashed<<<counted(grid_stride_blocks((long long)cap, 256)), 256, 0, s>>>(t, lg, depth, dom, ks.touched, ks.keys,
                                                                                 markers, err);
        return;
    }
    if (dirs && radius <= rr && hr <= rr) {
        // boxes within one node of the home node: direction sets per home node
        DirDomain dd;
        for (int a = 0; a < 3; a++) {
            dd.lo[a] = dom.d[0].lo[a] - 1;
            dd.dim[a] = dom.d[0].dim[a] + 2;
        }
        cudaMemsetAsync(dirs, 0, (size_t)touch_dirs_words(dom) * 4, s);
        if (p.n > 0) {
            // every 64th point first: it fills most entries while few points contend for
            // them, so that in the full pass nearly every point finds its bits set and
            // issues no atomic (when all points start on empty entries, the atomics of a
            // dense region pile up on its few entries)
            // (64-thread blocks: the sample's 16,384 threads per 4 M points then spread over
            // every SM instead of 64 of them)
            const bool int_r = radius >= 0.0f && radius == floorf(radius) && hr == floorf(hr) && hr <= 1048576.0f;
            auto touch = int_r ? k_touch_dirs<4, true> : k_touch_dirs<4, false>;
            if (p.n >= 64 * 1024) {
                PointSrc q = p;
                q.stride = p.stride * 64;
                q.n = (p.n + 63) / 64;
                touch<<<counted(grid_stride_blocks((q.n + 3) / 4, 64)), 64, 0, s>>>(q, orig, radius, hr, t.lgrange[0], rlo, rhi, dd,
                                                                            dirs, err);
            }
            touch<<<counted(grid_stride_blocks((p.n + 3) / 4, 256)), 256, 0, s>>>(p, orig, radius, hr, t.lgrange[0], rlo, rhi, dd,
                                                                          dirs, err);
        }
        if (dom.d[0].nbits > 8 * std::max(home_hint, 1ll)) {  // sparse domain: from the non-zero entries
            const long long nent = touch_dirs_words(dom);
            k_touch_dirs_scatter<<<counted(grid_stride_blocks(nent, 256)), 256, 0, s>>>(dom.d[0], dd, dirs, nent, touched);
        } else {
            const long long nw = (dom.d[0].nbits + 31) >> 5;
            k_touch_from_dirs<<<counted(blocks_for(nw * 32, 128)), 128, 0, s>>>(dom.d[0], dd, dirs, touched);
        }
    } else {
        // the points touch level 0 (its bits start at bit 0); the upper levels follow from it
        long long nwords = (dom.d[0].bitbase + dom.d[0].nbits + 31) >> 5;
        size_t smem = nwords <= kTouchSmemWords ? (size_t)nwords * 4 : 0;
        // fewer, fuller blocks when each one flushes a shared bitmap
        unsigned blocks = smem ? std::min<unsigned>(grid_stride_blocks(p.n, 256), 152u * 4u) : grid_stride_blocks(p.n, 256);
        k_touch_box<<<counted(blocks), 256, smem, s>>>(t, p, orig, radius, hi_mul, depth, rlo, rhi, dom, touched, nwords,
                                              KeyHash{nullptr, 0}, err);
    }
    for (int lev = 1; lev < depth; lev++) {
        long long nw = (dom.d[lev - 1].nbits + 31) >> 5;
        const long long pnw = (dom.d[lev].nbits + 31) >> 5;
        const size_t smem = pnw <= kTouchSmemWords ? (size_t)pnw * 4 : 0;
        // 1024 threads per block: fewer blocks flushing the parent words
        const unsigned blocks = std::min<unsigned>(blocks_for(nw * 32, 1024), 152u * 2u);
        k_touch_up<<<counted(blocks), 1024, smem, s>>>(dom.d[lev - 1], dom.d[lev], t.lgres[lev], touched, err);
    }
    const long long nw_all = (dom.d[depth - 1].bitbase + dom.d[depth - 1].nbits + 31) >> 5;
    k_resolve_touched<<<counted(std::min<unsigned>(blocks_for(nw_all * 32, 128), 152u * 16u)), 128, 0, s>>>(
        t, lg, depth, dom, nw_all, touched, bitmap, markers);
}
void launch_build_leaf_grid(const TreeView& t, long long n, int* cells, const int lo[3], const int dim[3],
                            int lgrange0, cudaStream_t s) {
    if (n <= 0) return;
    k_build_leaf_grid<<<counted(blocks_for(n, 256)), 256, 0, s>>>(t, n, cells, make_int3(lo[0], lo[1], lo[2]),
                                                         make_int3(dim[0], dim[1], dim[2]), lgrange0);
}
void launch_alloc_nodes(const uint32_t* bm, const uint32_t* prefix, long long word0, long long nwords,
                        int lev, int lgrange, const KeyDomain& d, long long base, Node* nodes, cudaStream_t s) {
    if (nwords <= 0) return;
    k_alloc_nodes<<<counted(std::min<unsigned>(blocks_for(nwords * 32, 256), 152u * 8u)), 256, 0, s>>>(
        bm, prefix, word0, nwords, lev, lgrange, d, base, nodes);
}
void launch_hash_compact(const KeyHash& h, unsigned long long* out, unsigned int* count, cudaStream_t s) {
    k_hash_compact<<<counted(grid_stride_blocks((long long)(h.mask + 1), 256)), 256, 0, s>>>(h, out, count);
}
void launch_key_bounds(const unsigned long long* sorted, const unsigned int* n, const KeyDomains& dom, int depth,
                       unsigned int* at, cudaStream_t s) {
    k_key_bounds<<<counted(1), 32, 0, s>>>(sorted, n, dom, depth, at);
}
void launch_alloc_nodes_sorted(const unsigned long long* sorted, long long first, long long count, int lev,
                               int lgrange, const KeyDomain& d, long long base, Node* nodes, cudaStream_t s) {
    if (count <= 0) return;
    k_alloc_nodes_sorted<<<counted(blocks_for(count, 256)), 256, 0, s>>>(sorted, first, count, lev, lgrange, d, base, nodes);
}
void launch_write_node(Node* dst, const Node& v, cudaStream_t s) { k_write_node<<<counted(1), 1, 0, s>>>(dst, v); }
void launch_link(const TreeView& t, int lev, long long count, int* tag, long long* slot_of, cudaStream_t s) {
    if (count <= 0) return;
    long long nslots = t.ncnt[lev + 1] << (3 * t.lgres[lev + 1]);
    cudaMemsetAsync(tag, 0xFF, (size_t)nslots * sizeof(int), s);
    k_link_claim<<<counted(blocks_for(count, 256)), 256, 0, s>>>(t, lev, count, tag, slot_of);
    k_link_write<<<counted(blocks_for(count, 256)), 256, 0, s>>>(t, lev, count, tag, slot_of);
}
void launch_apply_markers(Node* leaves, long long n, const int* markers, cudaStream_t s) {
    if (n <= 0) return;
    k_apply_markers<<<counted(blocks_for(n, 256)), 256, 0, s>>>(leaves, n, markers);
}
void launch_delink_leaf(const TreeView& t, long long n, cudaStream_t s) {
    if (n <= 0) return;
    k_delink_leaf<<<counted(blocks_for(n, 256)), 256, 0, s>>>(t, n);
}
void launch_delink_upper(const TreeView& t, int lev, long long n, cudaStream_t s) {
    if (n <= 0) return;
    k_delink_upper<<<counted(blocks_for(n, 128)), 128, 0, s>>>(t, lev, n);
}
void launch_stage_counts(const uint32_t* pscan, const CountStage& st, uint32_t* out, cudaStream_t s) {
    k_stage_counts<<<counted(1), 32, 0, s>>>(pscan, st, out);
}
void launch_incr_setup(const Node* leaves, long long n, int* markers, int accum, int* err, unsigned long long* kept,
                       int* bbox6, cudaStream_t s) {
    k_incr_setup<<<counted(blocks_for(std::max(n, 1ll), 256)), 256, 0, s>>>(leaves, n, markers, accum, err, kept, bbox6);
}
void launch_count_markers(const int* markers, long long n, unsigned long long* out, cudaStream_t s) {
    if (n <= 0) return;
    k_count_markers<<<counted(grid_stride_blocks(n, 256)), 256, 0, s>>>(markers, n, out);
}
void launch_count_flags(const Node* nodes, long long n, unsigned long long* out, cudaStream_t s) {
    if (n <= 0) return;
    k_count_flags<<<counted(grid_stride_blocks(n, 256)), 256, 0, s>>>(nodes, n, out);
}
void launch_leaf_bounds(const Node* leaves, long long n, int lgrange0, int* out6, cudaStream_t s) {
    if (n <= 0) return;
    k_leaf_bounds<<<counted(1), 1024, 0, s>>>(leaves, n, lgrange0, out6);
}

}  // namespace gbvdb
