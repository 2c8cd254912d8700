// points.cu -- InsertPointsSubcell binning and the GatherDensity / GatherLevelSet kernels.
//
// Replaces (reference file:line):
//   gvdbSetFlagSubcell + PrefixSum (sc_mapping)       PT.cuh:109-118, VG.cpp:4988-4996
//   gvdbCountSubcell / gvdbInsertSubcell              PT.cuh:218-315
//   gvdbCalcSubcellPos                                PT.cuh:677-694
//   gvdbGatherDensity / gvdbGatherLevelSet            PT.cuh:696-773
//
// Subcell membership is the reference's rule: point w (after +trans, all
// coordinates >= 0, z != NOHIT) belongs to subcell S of a linked leaf iff on every
// axis  int(w - R)/4*4 <= S <= int(w + 1 + R)/4*4  (C truncation, FP32).
// The reference copies each point into every member subcell's list (~34 copies
// at R = 4) and then re-reads those lists.  Here each point is binned once, by
// its home subcell (the subcell containing floor(w)), with a counting sort; the
// gather of a brick pulls the home bins of its 3x3x3 brick neighbourhood and
// applies the membership rule per (point, subcell).  The value of a voxel is a
// max / min over its subcell's members, so it does not depend on visiting order:
//   density   max(0, max_j (rho - |p_j - v|)) = max(0, rho - sqrt(min_j d_j^2))
//   level set min(3, min_j (|p_j - v| - rho)) = min(3, sqrt(min_j d_j^2) - rho)
// (with a correctly rounded sqrt both forms round identically, sqrt and the
// subtraction being monotonic).  The kernels reduce min d^2 per voxel and take its
// square root with sqrt.approx.f32, as the reference's kernels do (they are built
// with --use_fast_math): within one unit in the last place of the rounded root.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kernels.h"

namespace gbvdb {

namespace {

constexpr int kSc = 4;  // subcell size (voxels)

__device__ __forceinline__ void sc_range(float w, float R, int& lo, int& hi) {
    lo = ((int)fsub(w, R)) / kSc * kSc;
    hi = ((int)fadd(fadd(w, 1.0f), R)) / kSc * kSc;
}

__device__ __forceinline__ bool load_valid(PointSrc p, long long i, float3 trans, float& x, float& y, float& z) {
    load_pos(p.base, i, p.stride, p.off, x, y, z);
    if (z == kNoHit) return false;  // PT.cuh:282, tested before +trans
    x = fadd(x, trans.x);
    y = fadd(y, trans.y);
    z = fadd(z, trans.z);
    return !(x < 0 || y < 0 || z < 0);
}

// the stored (and gathered) position of a point: w itself, or its 16-bit quantised
// and dequantised form, one rounding per FP32 operation
__device__ __forceinline__ float quant16(float w, float mn, float rg) {
    if (!(rg > 0.0f)) return mn;
    const float t = __fmul_rn(__fdiv_rn(fsub(w, mn), rg), 65535.0f);
    const unsigned q = t <= 0.0f ? 0u : (t >= 65535.0f ? 65535u : (unsigned)t);
    return fadd(__fmul_rn(__fdiv_rn((float)q, 65535.0f), rg), mn);
}
__device__ __forceinline__ void stored_pos(const Quant& q, const float* w, float* out) {
    if (q.on) {
        out[0] = quant16(w[0], q.mn.x, q.rg.x);
        out[1] = quant16(w[1], q.mn.y, q.rg.y);
        out[2] = quant16(w[2], q.mn.z, q.rg.z);
    } else {
        out[0] = w[0];
        out[1] = w[1];
        out[2] = w[2];
    }
}

__global__ void k_linked_list(const Node* leaves, long long n, const uint32_t* scmap, int* linked) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (leaves[i].parent != kUndef64) linked[scmap[i]] = (int)i;
}

// the linked leaf at an index-space position.  A leaf is reachable from the root
// only through a child-list entry, which the link pass writes after setting the
// leaf's mParent, and delinking clears both; so every reachable leaf is linked and
// the dense grid (built by traversal) answers directly.
__device__ __forceinline__ long long linked_leaf(const LeafGrid& lg, const TreeView& t, int x, int y, int z) {
    if (lg.cells) return lookup_leaf(lg, t, x, y, z);
    long long l = get_pos_leaf(t, x, y, z);
    if (l < 0 || t.nodes[0][l].parent == kUndef64) return -1;
    return l;
}

// Home-subcell counting pass + total subcell-list length (the reference's
// pSCPntsLength) + orphans (valid points whose home leaf is not linked).
// Which of the 27 bricks around each linked leaf (itself included) are linked
// leaves: bit (dz+1)*9 + (dy+1)*3 + (dx+1); positions with a negative coordinate
// count as not linked, as in the list-length count.  One warp per leaf, a lane
// per direction.
// Also clears the binning counters it runs before (bin_cnt: 64 per leaf, every leaf;
// totals: 2) when they are given.
__global__ void k_nb_mask(TreeView t, LeafGrid lg, long long n, uint32_t* __restrict__ nbmask,
                          uint32_t* __restrict__ bin_cnt, unsigned long long* totals) {
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int d = threadIdx.x & 31;
    if (totals && i == 0 && d < 2) totals[d] = 0ull;
    if (i >= n) return;
    if (bin_cnt) {
        bin_cnt[i * 64 + d] = 0u;
        bin_cnt[i * 64 + 32 + d] = 0u;
    }
    const Node& nd = t.nodes[0][i];
    if (nd.parent == kUndef64) return;
    bool on = false;
    if (d < 27) {
        const int px = nd.pos[0] + 16 * (d % 3 - 1), py = nd.pos[1] + 16 * ((d / 3) % 3 - 1), pz = nd.pos[2] + 16 * (d / 9 - 1);
        on = px >= 0 && py >= 0 && pz >= 0 && linked_leaf(lg, t, px, py, pz) >= 0;
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, on);
    if (d == 0) nbmask[i] = m;
}

// subcells of the member range [lo, hi] (multiples of 4) inside the brick at origin o
__device__ __forceinline__ int range_in_brick(int lo, int hi, int o) {
    const int a = max(lo, o), b = min(hi, o + 12);
    return b >= a ? ((b - a) >> 2) + 1 : 0;
}

// kU points per thread per step: the position loads, the home-leaf lookups, the rank
// loads and the counting atomics of the kU points are each issued together (the pass
// is bound by the latency of that dependent chain).  kU comes from the tuning table
// (1, 2 or 4); measured on the fluid frame: kU = 1 or 2 (54 / 63 registers) beat 3 and
// 4 (72 / 80 registers, fewer resident warps) by about 10 us.  kU = 1 is held to 42
// registers (6 blocks of 256 per SM, no spills): the InsertPointsSubcell stage 0.233 ->
// 0.216 ms in a timing run of that stage alone; 8 blocks spill and lose.
template <int kU>
__global__ void __launch_bounds__(256, kU == 1 ? 6 : (kU == 2 ? 4 : 1))
    k_bin_count(TreeView t, LeafGrid lg, PointSrc p, float3 trans, float R, Quant qz,
                const uint32_t* __restrict__ scmap, const uint32_t* __restrict__ nbmask, uint32_t* bin_cnt,
                int* bin_of, uint32_t* rank_of, unsigned long long* totals) {
    // kU = 4: four consecutive points per thread, their positions in three 16-byte loads
    // (load_pos4); kU = 1, 2: points kU grid strides apart
    constexpr bool kConsec = kU == 4;
    unsigned long long members = 0, orphans = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = kConsec ? 4ll * ((long long)blockIdx.x * blockDim.x + threadIdx.x)
                                    : (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long step = kConsec ? 4 * stride : kU * stride;
    for (long long i0 = first; i0 < p.n; i0 += step) {
        auto idx = [&](int u) { return kConsec ? i0 + u : i0 + u * stride; };
        float w[kU][3];
        bool ok[kU];
        if constexpr (kConsec) {
            float raw[4][3];
            load_pos4(p, i0, raw);
#pragma unroll
            for (int u = 0; u < kU; u++) {
                ok[u] = false;
                if (i0 + u >= p.n || raw[u][2] == kNoHit) continue;  // PT.cuh:282, tested before +trans
                w[u][0] = fadd(raw[u][0], trans.x);
                w[u][1] = fadd(raw[u][1], trans.y);
                w[u][2] = fadd(raw[u][2], trans.z);
                ok[u] = !(w[u][0] < 0 || w[u][1] < 0 || w[u][2] < 0);
            }
        } else {
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const long long i = idx(u);
                ok[u] = i < p.n && load_valid(p, i, trans, w[u][0], w[u][1], w[u][2]);
            }
        }
        long long leaf[kU];
        unsigned loc[kU];
        int hb[kU][3];  // origin of the home brick
#pragma unroll
        for (int u = 0; u < kU; u++) {
            leaf[u] = -1;
            loc[u] = 0;
            if (!ok[u]) continue;
            float ps[3];
            stored_pos(qz, w[u], ps);
            int h[3];  // home subcell of the stored position
#pragma unroll
            for (int a = 0; a < 3; a++) {
                h[a] = ((int)ps[a]) & ~(kSc - 1);
                hb[u][a] = h[a] & ~15;
            }
            leaf[u] = linked_leaf(lg, t, h[0], h[1], h[2]);
            // subcell within the 16^3 leaf that contains h (leaf origin = h rounded down to 16)
            loc[u] = (unsigned)((((h[2] >> 2) & 3) << 4) | (((h[1] >> 2) & 3) << 2) | ((h[0] >> 2) & 3));
        }
        unsigned bin[kU];
        uint32_t nbm[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            bin[u] = leaf[u] >= 0 ? __ldg(scmap + leaf[u]) * 64u + loc[u] : 0u;
            nbm[u] = (nbmask && leaf[u] >= 0) ? __ldg(nbmask + leaf[u]) : 0u;
        }
        uint32_t rk[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) rk[u] = leaf[u] >= 0 ? atomicAdd(bin_cnt + bin[u], 1u) : 0u;
        int bo[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            bo[u] = !ok[u] ? -1 : (leaf[u] < 0 ? -2 : (int)bin[u]);
            if (ok[u] && leaf[u] < 0) orphans++;
        }
        if (kConsec && i0 + 4 <= p.n) {  // 16-byte stores of the four consecutive entries
            *reinterpret_cast<int4*>(bin_of + i0) = make_int4(bo[0], bo[kU > 1 ? 1 : 0], bo[kU > 2 ? 2 : 0],
                                                              bo[kU > 3 ? 3 : 0]);
            *reinterpret_cast<uint4*>(rank_of + i0) = make_uint4(rk[0], rk[kU > 1 ? 1 : 0], rk[kU > 2 ? 2 : 0],
                                                                 rk[kU > 3 ? 3 : 0]);
        } else {
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const long long i = idx(u);
                if (i >= p.n) continue;
                bin_of[i] = bo[u];
                if (bo[u] >= 0) rank_of[i] = rk[u];
            }
        }
        // number of (subcell, point) list entries each point creates
#pragma unroll
        for (int u = 0; u < kU; u++) {
            if (!ok[u]) continue;
            int lo[3], hi[3];
            bool any = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                sc_range(w[u][a], R, lo[a], hi[a]);
                if (lo[a] < 0) lo[a] = 0;  // guard: negative subcells are skipped
                if (hi[a] < lo[a]) any = false;
            }
            if (!any) continue;
            if (nbmask && leaf[u] >= 0) {
                // R <= 11: the member range reaches only the 27 bricks around the home
                // brick; their linked flags are nbm (k_nb_mask).  All 27 linked: every
                // member subcell counts
                if (nbm[u] == 0x7FFFFFFu) {
                    members += (unsigned long long)(((hi[0] - lo[0]) >> 2) + 1) * (unsigned)(((hi[1] - lo[1]) >> 2) + 1) *
                               (unsigned)(((hi[2] - lo[2]) >> 2) + 1);
                } else {
                    int c[3][3];
#pragma unroll
                    for (int a = 0; a < 3; a++)
#pragma unroll
                        for (int d = 0; d < 3; d++) c[a][d] = range_in_brick(lo[a], hi[a], hb[u][a] + 16 * (d - 1));
                    unsigned long long m = 0;
#pragma unroll
                    for (int dz = 0; dz < 3; dz++)
#pragma unroll
                        for (int dy = 0; dy < 3; dy++) {
                            const int row = (nbm[u] >> (dz * 9 + dy * 3)) & 7;
                            const int sx = ((row & 1) ? c[0][0] : 0) + ((row & 2) ? c[0][1] : 0) + ((row & 4) ? c[0][2] : 0);
                            m += (unsigned long long)(sx * c[1][dy] * c[2][dz]);
                        }
                    members += m;
                }
                continue;
            }
            for (int bx = lo[0] >> 4; bx <= hi[0] >> 4; bx++) {
                int x0 = max(lo[0], bx << 4), x1 = min(hi[0], (bx << 4) + 12);
                for (int by = lo[1] >> 4; by <= hi[1] >> 4; by++) {
                    int y0 = max(lo[1], by << 4), y1 = min(hi[1], (by << 4) + 12);
                    for (int bz = lo[2] >> 4; bz <= hi[2] >> 4; bz++) {
                        int z0 = max(lo[2], bz << 4), z1 = min(hi[2], (bz << 4) + 12);
                        if (linked_leaf(lg, t, bx << 4, by << 4, bz << 4) < 0) continue;
                        members += (unsigned long long)(((x1 - x0) >> 2) + 1) * (((y1 - y0) >> 2) + 1) * (((z1 - z0) >> 2) + 1);
                    }
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        members += __shfl_down_sync(0xFFFFFFFFu, members, o);
        orphans += __shfl_down_sync(0xFFFFFFFFu, orphans, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (members) atomicAdd(totals, members);
        if (orphans) atomicAdd(totals + 1, orphans);
    }
}

// Binned record of one point: position (after +trans) and, in .w, its subcell
// membership relative to its home subcell H = floor(w/4) as three 9-bit masks
// (axis a at bit 9a): bit d+4 is set iff subcell H+d is a member on that axis,
// i.e. lo <= d <= hi with lo = int(w-R)/4 - H and hi = int(w+1+R)/4 - H.  For
// R <= 11 (the range the brick-tiled gather serves) lo >= -4 and hi <= 3, so the
// masks are exact; outside that range they are clipped and not used.
__device__ __forceinline__ int pack_ranges(const float* w, const float* home, float R) {
    int packed = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int lo, hi;
        sc_range(w[a], R, lo, hi);
        int h = ((int)home[a]) >> 2;
        int l = max((lo >> 2) - h, -4), u = min((hi >> 2) - h, 4);  // lo, hi are multiples of 4
        if (l <= u) packed |= (int)((((1u << (u - l + 1)) - 1u) << (l + 4)) << (9 * a));
    }
    return packed;
}
// member range [l, u] on axis a (relative to the home subcell); false when empty
__device__ __forceinline__ bool mask_range(int packed, int a, int& l, int& u) {
    const unsigned f = ((unsigned)packed >> (9 * a)) & 0x1FFu;
    l = __ffs(f) - 5;
    u = 27 - __clz(f);
    return f != 0;
}
// bits an offset o = H - S must find set for S to be a member (d = S - H = -o)
__device__ __forceinline__ int member_bits(int ox, int oy, int oz) {
    return (1 << (4 - ox)) | (1 << (13 - oy)) | (1 << (22 - oz));
}

// kU points per thread per step (2, 4 or 8 from the tuning table), their loads issued
// together (the pass is bound by the latency of the dependent bin_of -> bin_off loads)
template <int kU>
__global__ void k_bin_scatter(PointSrc p, float3 trans, float R, Quant qz, const int* __restrict__ bin_of,
                              const uint32_t* __restrict__ rank_of, const uint32_t* __restrict__ bin_off,
                              float4* __restrict__ sorted, ClrSrc clr, uint32_t* __restrict__ sorted_clr) {
    // kU = 4: four consecutive points per thread (16-byte loads of their bins, ranks and
    // positions); kU = 2, 8: points grid strides apart
    constexpr bool kConsec = kU == 4;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = kConsec ? 4ll * ((long long)blockIdx.x * blockDim.x + threadIdx.x)
                                    : (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long step = kConsec ? 4 * stride : kU * stride;
    for (long long i0 = first; i0 < p.n; i0 += step) {
        auto idx = [&](int u) { return kConsec ? i0 + u : i0 + u * stride; };
        int b[kU];
        uint32_t rk[kU], off[kU];
        float x[kU], y[kU], z[kU];
        if (kConsec && i0 + 4 <= p.n) {
            const int4 bv = *reinterpret_cast<const int4*>(bin_of + i0);
            const int bb[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int u = 0; u < kU; u++) b[u] = bb[u < 4 ? u : 0];
        } else {
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const long long i = idx(u);
                b[u] = i < p.n ? bin_of[i] : -1;
            }
        }
        if constexpr (kConsec) {
            const bool any = (b[0] >= 0) | (b[kU > 1 ? 1 : 0] >= 0) | (b[kU > 2 ? 2 : 0] >= 0) | (b[kU > 3 ? 3 : 0] >= 0);
            if (any) {
                float raw[4][3];
                load_pos4(p, i0, raw);
                uint4 rv = make_uint4(0, 0, 0, 0);
                if (i0 + 4 <= p.n) rv = *reinterpret_cast<const uint4*>(rank_of + i0);
                const uint32_t rr[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
                for (int u = 0; u < kU; u++) {
                    if (b[u] < 0) continue;
                    rk[u] = i0 + 4 <= p.n ? rr[u < 4 ? u : 0] : rank_of[i0 + u];
                    off[u] = bin_off[b[u]];
                    x[u] = raw[u < 4 ? u : 0][0];
                    y[u] = raw[u < 4 ? u : 0][1];
                    z[u] = raw[u < 4 ? u : 0][2];
                }
            }
        } else {
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const long long i = idx(u);
                if (b[u] >= 0) {
                    rk[u] = rank_of[i];
                    off[u] = bin_off[b[u]];
                    load_pos(p.base, i, p.stride, p.off, x[u], y[u], z[u]);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
            if (b[u] < 0) continue;
            float w[3] = {fadd(x[u], trans.x), fadd(y[u], trans.y), fadd(z[u], trans.z)};
            float ps[3];
            stored_pos(qz, w, ps);
            sorted[off[u] + rk[u]] = make_float4(ps[0], ps[1], ps[2], __int_as_float(pack_ranges(w, ps, R)));
            if (sorted_clr) {
                const long long i = idx(u);
                sorted_clr[off[u] + rk[u]] = __ldg(reinterpret_cast<const uint32_t*>(clr.base + i * (long long)clr.stride + clr.off));
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ float ld_f32(const T* p);
template <>
__device__ __forceinline__ float ld_f32<float>(const float* p) { return *p; }
template <>
__device__ __forceinline__ float ld_f32<__half>(const __half* p) { return __half2float(*p); }
template <>
__device__ __forceinline__ float ld_f32<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }
template <typename T>
__device__ __forceinline__ T cvt_out(float v);
template <>
__device__ __forceinline__ float cvt_out<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half cvt_out<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt_out<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// final voxel value from min squared distance m, with c = sqrt(m) given
__device__ __forceinline__ float finish_c(const GatherParams& gp, float c, float old) {
    if (gp.mode == 0) return fmaxf(gp.accum ? old : 0.0f, fsub(gp.rho, c));
    return fminf(gp.accum ? old : 3.0f, fsub(c, gp.rho));
}

// Fused apron.  After the tile write, the tile holds the final values' storage
// bits and each brick copies its boundary voxels into the apron records of the
// neighbours that hold them (pslot[d]: slot of the neighbour at direction d =
// (dx+1) + 3 (dy+1) + 9 (dz+1), -1 for none).  Apron voxel k of a brick comes
// from the neighbour at direction d(k) (apron_shell_pos), so this brick writes
// voxel k of the brick at -d(k).  Every apron voxel of the atlas has one source
// brick: no two blocks write the same element.  Face records are in the order of
// the source plane (x faces [z][y], y faces [z][x], z faces [y][x]) and go as
// 4-voxel vectors; edges and corners take kApronEdges (tile index, receiver).

template <typename T>
__device__ __forceinline__ void push_apron(const uint32_t* tile, const int* pslot, T* apron) {
    const int tid = threadIdx.x;
    // faces: 6 x 64 vectors, iteration a = axis (x, y, z); the first 64 threads take
    // the minus face of the receiver (source plane 15, receiver at +axis), the
    // others the plus face (source plane 0, receiver at -axis)
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int plus = (tid >> 6) & 1, f = 2 * a + plus;
        const int e0 = (tid & 63) << 2, row = e0 >> 4, col = e0 & 15, h = plus ? 0 : 15;
        const int step = a == 0 ? 1 : (a == 1 ? 3 : 9);
        const int tgt = pslot[13 + (plus ? -step : step)];
        if (tgt < 0) continue;
        uint4 b;
        if (a == 0) {  // x face [z][y]: 4 voxels down a column of the source plane
            const uint32_t* c = tile + ((row << 8) | (col << 4) | h);
            b = make_uint4(c[0], c[16], c[32], c[48]);
        } else if (a == 1) {  // y face [z][x]
            b = *reinterpret_cast<const uint4*>(tile + ((row << 8) | (h << 4) | col));
        } else {  // z face [y][x]
            b = *reinterpret_cast<const uint4*>(tile + ((h << 8) | (row << 4) | col));
        }
        const size_t e = (size_t)tgt * kApronStride + (size_t)f * 256 + e0;
        if constexpr (sizeof(T) == 4)
            *reinterpret_cast<uint4*>(reinterpret_cast<uint32_t*>(apron) + e) = b;
        else
            *reinterpret_cast<uint2*>(reinterpret_cast<uint16_t*>(apron) + e) = make_uint2(b.x | (b.y << 16), b.z | (b.w << 16));
    }
    for (int j = tid; j < 200; j += blockDim.x) {  // edges and corners
        const uint32_t te = __ldg(kApronEdges.e + j);
        const int tgt = pslot[te >> 12];
        if (tgt < 0) continue;
        const uint32_t b = tile[te & 4095u];
        const size_t e = (size_t)tgt * kApronStride + 1536 + j;
        if constexpr (sizeof(T) == 4) reinterpret_cast<uint32_t*>(apron)[e] = b;
        else reinterpret_cast<uint16_t*>(apron)[e] = (uint16_t)b;
    }
}

// PTX sqrt.approx.f32 (the reference's kernels are built with --use_fast_math, so their
// sqrtf is this instruction too)
__device__ __forceinline__ float sqrt_approx(float a) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// Final values from the tile of minima, one coalesced write of the brick.  keep:
// the final values' storage bits replace the minima in the tile (fused apron).
template <typename T>
__device__ void write_tile(const GatherParams& gp, uint32_t* tile, T* out, bool keep) {
    // voxels no point reached hold the cutoff: their sqrt is one per thread
    const float sqrtT = __fsqrt_rn(__uint_as_float(gp.tbits));
    for (int v4 = threadIdx.x; v4 < 1024; v4 += blockDim.x) {
        float r[4];
        const uint4 m4 = reinterpret_cast<const uint4*>(tile)[v4];
        const uint32_t mv[4] = {m4.x, m4.y, m4.z, m4.w};
        const bool any = (m4.x != gp.tbits) | (m4.y != gp.tbits) | (m4.z != gp.tbits) | (m4.w != gp.tbits);
        float c[4] = {sqrtT, sqrtT, sqrtT, sqrtT};
        if (__any_sync(__activemask(), any)) {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (mv[k] != gp.tbits) c[k] = sqrt_approx(__uint_as_float(mv[k]));
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int v = v4 * 4 + k;
            float old = gp.accum ? ld_f32<T>(out + v) : 0.f;
            r[k] = finish_c(gp, c[k], old);
        }
        if constexpr (sizeof(T) == 4) {
            reinterpret_cast<float4*>(out)[v4] = make_float4(r[0], r[1], r[2], r[3]);
            if (keep)
                reinterpret_cast<uint4*>(tile)[v4] = make_uint4(__float_as_uint(r[0]), __float_as_uint(r[1]),
                                                                __float_as_uint(r[2]), __float_as_uint(r[3]));
        } else {
            T h[4];
#pragma unroll
            for (int k = 0; k < 4; k++) h[k] = cvt_out<T>(r[k]);
            uint2 pk;
            pk.x = (uint32_t)(*reinterpret_cast<uint16_t*>(&h[0])) | ((uint32_t)(*reinterpret_cast<uint16_t*>(&h[1])) << 16);
            pk.y = (uint32_t)(*reinterpret_cast<uint16_t*>(&h[2])) | ((uint32_t)(*reinterpret_cast<uint16_t*>(&h[3])) << 16);
            reinterpret_cast<uint2*>(out)[v4] = pk;
            if (keep)
                reinterpret_cast<uint4*>(tile)[v4] = make_uint4(pk.x & 0xFFFFu, pk.x >> 16, pk.y & 0xFFFFu, pk.y >> 16);
        }
    }
}

constexpr int kGatherThreads = 128;
// 1 / n for n = 1 .. 16 (entry 0 unused): the sparse walk's row-major column split
__constant__ float kRcp16[17] = {0.0f,       1.0f,       0.5f,       1.0f / 3,  0.25f,     0.2f,
                                 1.0f / 6,   1.0f / 7,   0.125f,     1.0f / 9,  0.1f,      1.0f / 11,
                                 1.0f / 12,  1.0f / 13,  1.0f / 14,  1.0f / 15, 0.0625f};
constexpr int kQueue = 64;  // per-warp point queue of the gather form (SoA x, y, z)
// scatter form: reaches of cutoffs below this radius (boxes of at most 4 voxels a side)
// are walked with the entries' columns packed across the warp
constexpr float kPackedReach = 2.0f;
constexpr int kLive = 256;  // live points per batch of the scatter form
constexpr int kScratch = kLive * 16 > (kGatherThreads / 32) * 3 * kQueue * 4 ? kLive * 16
                                                                              : (kGatherThreads / 32) * 3 * kQueue * 4;
static_assert(kGatherThreads == 128, "push_apron maps 128 threads onto the two faces of an axis");

// packed FP32 pairs (f32x2 arithmetic, round-to-nearest, no contraction)
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2pack(float lo, float hi) {
    return (f32x2)__float_as_uint(lo) | ((f32x2)__float_as_uint(hi) << 32);
}
__device__ __forceinline__ float f2lo(f32x2 v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float f2hi(f32x2 v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f32x2 f2sub(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2add(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2mul(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Unit-box pass of the gather form.  Every point within one voxel (per axis) of
// the brick lowers the voxels floor(p) and floor(p) + 1 on each axis (the only
// voxels it can be nearer than 1 to, on every axis) with shared atomicMin,
// member subcells only.  A voxel whose minimum is then below 1 is exact: every
// member point left out is at least 1 away on some axis, so its d^2 >= 1.  The
// points are the brick's own (its 64 bins, one range) and the bins of the
// subcell layer next to the brick in its 7 lower neighbours (61 ranges): a point
// homed above the brick is at least 1 from its last voxel.
// Range k of the 64 (62 used): neighbour index into nrank and bin in that brick.
__device__ __forceinline__ void unit_range(int k, int& nb, int& bin) {
    if (k == 0) { nb = 13; bin = 0; }                                              // own, all 64 bins
    else if (k <= 16) { const int j = k - 1; nb = 12; bin = (j >> 2) * 16 + (j & 3) * 4 + 3; }   // -x: lx = 3
    else if (k <= 32) { const int j = k - 17; nb = 10; bin = (j >> 2) * 16 + 12 + (j & 3); }     // -y: ly = 3
    else if (k <= 48) { nb = 4; bin = 48 + (k - 33); }                               // -z: lz = 3
    else if (k <= 52) { nb = 9; bin = (k - 49) * 16 + 15; }                          // -x-y
    else if (k <= 56) { nb = 3; bin = 48 + (k - 53) * 4 + 3; }                       // -x-z
    else if (k <= 60) { nb = 1; bin = 60 + (k - 57); }                               // -y-z
    else { nb = 0; bin = 63; }                                                       // -x-y-z
}

__device__ __forceinline__ void unit_box_pass(uint32_t* tile, const int* nrank, const uint32_t* __restrict__ bin_off,
                                              const float4* __restrict__ pts, int ox, int oy, int oz,
                                              uint32_t* rbeg, uint32_t* rpre) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        uint32_t beg[2] = {0, 0}, cnt[2] = {0, 0};
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int k = lane + 32 * h;
            if (k < 62) {
                int nb, bin;
                unit_range(k, nb, bin);
                const int r = nrank[nb];
                if (r >= 0) {
                    const size_t b0 = (size_t)r * 64 + bin;
                    beg[h] = __ldg(bin_off + b0);
                    cnt[h] = __ldg(bin_off + b0 + (k == 0 ? 64 : 1)) - beg[h];
                }
            }
        }
        uint32_t i0 = cnt[0], i1 = cnt[1];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, i0, o), b = __shfl_up_sync(0xFFFFFFFFu, i1, o);
            if (lane >= o) { i0 += a; i1 += b; }
        }
        const uint32_t t0 = __shfl_sync(0xFFFFFFFFu, i0, 31);
        rbeg[lane] = beg[0];
        rbeg[lane + 32] = beg[1];
        rpre[lane] = i0 - cnt[0];
        rpre[lane + 32] = t0 + i1 - cnt[1];
        if (lane == 31) rpre[64] = t0 + i1;
    }
    __syncthreads();
    const uint32_t total = rpre[64];
    const int org[3] = {ox, oy, oz};
    // two points per thread per round, both loads in flight together
    for (uint32_t i0 = threadIdx.x; i0 < total; i0 += 2 * blockDim.x) {
        float4 qq[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const uint32_t idx = i0 + u * blockDim.x;
            qq[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // w = 0: no member subcell, nothing written
            if (idx < total) {
                int k = 0;  // last range with rpre[k] <= idx (a non-empty one)
#pragma unroll
                for (int step = 32; step > 0; step >>= 1)
                    if (rpre[k + step] <= idx) k += step;
                qq[u] = pts[rbeg[k] + (idx - rpre[k])];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
        const float4 q = qq[u];
        const int pk = __float_as_int(q.w);
        const float pw[3] = {q.x, q.y, q.z};
        int vl[3];
        bool ok[3][2];
        float dd[3][2];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int fl = (int)pw[a];  // floor: stored positions are >= 0
            const int hs = fl >> 2;     // home subcell
            vl[a] = fl - org[a];
            ok[a][0] = (unsigned)vl[a] < 16u && ((pk >> (9 * a + 4)) & 1);
            ok[a][1] = (unsigned)(vl[a] + 1) < 16u && ((pk >> (9 * a + 4 + (((fl + 1) >> 2) - hs))) & 1);
            dd[a][0] = fsub(pw[a], (float)fl);
            dd[a][1] = fsub(pw[a], (float)(fl + 1));
        }
#pragma unroll
        for (int i = 0; i < 2; i++) {
            if (!ok[0][i]) continue;
            const float xx = __fmul_rn(dd[0][i], dd[0][i]);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                if (!ok[1][j]) continue;
                const float xy = __fmaf_rn(dd[1][j], dd[1][j], xx);
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    if (!ok[2][kk]) continue;
                    const uint32_t d = __float_as_uint(__fmaf_rn(dd[2][kk], dd[2][kk], xy));
                    const int v = ((vl[2] + kk) << 8) | ((vl[1] + j) << 4) | (vl[0] + i);
                    if (d < tile[v]) atomicMin(tile + v, d);
                }
            }
        }
        }
    }
    __syncthreads();
}

// Fused-apron check, one thread per leaf.  The gather's push and the apron fill
// assume that the grid is in the state every frame of the path leaves it in:
// a leaf is linked (mParent defined) exactly when it is flagged and exactly when
// the dense lookup finds it at its own position, its atlas slot is its rank among
// the linked leaves (so scmap gives neighbours' slots) and the slot maps back to
// it, and the linked count equals the assigned slots.  Any leaf that breaks this
// sets *bad, and both the push and the fill are then skipped for the whole grid.
__global__ void k_push_check(TreeView t, LeafGrid lg, const uint32_t* __restrict__ scmap,
                             const AtlasNode* __restrict__ amap, int used, int ax, int ay, long long n, int* bad) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && (long long)scmap[n] != (long long)used) *bad = 1;
    if (i >= n) return;
    const Node nd = t.nodes[0][i];
    const bool lk = nd.parent != kUndef64;
    const bool fl = nd.flags != 0;
    const bool fd = lg.cells && nd.pos[0] >= 0 && nd.pos[1] >= 0 && nd.pos[2] >= 0 &&
                    lookup_leaf(lg, t, nd.pos[0], nd.pos[1], nd.pos[2]) == i;
    bool ok = lk == fl && lk == fd;
    if (ok && lk) {
        const int s = slot_of_value(nd.value, ax, ay);
        ok = s >= 0 && s < used && (uint32_t)s == scmap[i] && amap[s].leaf == (int)i;
    }
    if (!ok) *bad = 1;
}

// Per-brick setup of the gather, one warp per linked leaf (lane = direction d =
// (dx+1) + 3 (dy+1) + 9 (dz+1)): the linked rank of the neighbour brick at d and
// the range of its 64 home bins in the binned points; entry 27 holds the brick's
// origin and atlas slot.  Done here with every warp's loads in flight at once,
// so that a gather block starts from one coalesced 512-byte read instead of a
// chain of dependent lookups.
//
// Launch order (long_min >= 0): the records of the bricks with more than long_min
// points homed around them (the gather form's bricks and the scatter form's
// fullest, whose blocks run longest) fill the table from the front, the others
// from the back, so that the gather starts its long blocks first and the short
// ones fill in behind them; a long block launched late is the kernel's tail.
// ctr[0], ctr[1] (zero on entry) count the two kinds.  The order within each kind
// varies from run to run; the result does not (every brick writes only its own
// slot and the apron voxels it is the one source of).  long_min < 0: linked order.
constexpr int kPrepThreads = 256;
__global__ void __launch_bounds__(kPrepThreads) k_gather_prep(TreeView t, LeafGrid lg, const int* __restrict__ linked,
                                                              long long nbricks, const uint32_t* __restrict__ scmap,
                                                              const uint32_t* __restrict__ bin_off, int ax, int ay,
                                                              int long_min, unsigned* ctr, int4* __restrict__ gtab) {
    __shared__ int kind[kPrepThreads / 32];  // 1 long, 0 short, -1 no brick
    __shared__ unsigned base[2];
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool have = b < nbricks;
    int4 e = make_int4(-1, 0, 0, 0);
    if (have) {
        const int leaf = linked[b];
        const Node& nd = t.nodes[0][leaf];
        const int ox = nd.pos[0], oy = nd.pos[1], oz = nd.pos[2];
        if (lane < 27) {
            const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
            int r = -1;
            if ((dx | dy | dz) == 0) {
                r = (int)scmap[leaf];
            } else {
                const int px = ox + 16 * dx, py = oy + 16 * dy, pz = oz + 16 * dz;
                if (px >= 0 && py >= 0 && pz >= 0) {
                    const long long l = linked_leaf(lg, t, px, py, pz);
                    if (l >= 0) r = (int)scmap[l];
                }
            }
            if (r >= 0) {
                const uint32_t beg = __ldg(bin_off + (size_t)r * 64);
                e = make_int4(r, (int)beg, (int)(__ldg(bin_off + (size_t)r * 64 + 64) - beg), 0);
            }
        } else if (lane == 27) {
            e = make_int4(ox, oy, oz, slot_of_value(nd.value, ax, ay));
        }
    }
    if (long_min < 0) {
        if (have && lane < 28) gtab[b * 32 + lane] = e;
        return;
    }
    // the neighbourhood's points (the gather's candidate count)
    const unsigned ncand = __reduce_add_sync(0xFFFFFFFFu, lane < 27 ? (unsigned)e.z : 0u);
    const int k = have ? (ncand > (unsigned)long_min ? 1 : 0) : -1;
    if (lane == 0) kind[warp] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned n[2] = {0, 0};
        for (int w = 0; w < kPrepThreads / 32; w++)
            if (kind[w] >= 0) n[kind[w]]++;
        base[1] = n[1] ? atomicAdd(ctr, n[1]) : 0u;
        base[0] = n[0] ? atomicAdd(ctr + 1, n[0]) : 0u;
    }
    __syncthreads();
    if (!have) return;
    unsigned rank = base[k];
    for (int w = 0; w < warp; w++) rank += kind[w] == k ? 1u : 0u;
    const long long pos = k ? (long long)rank : nbricks - 1 - (long long)rank;
    if (lane < 28) gtab[pos * 32 + lane] = e;
}

// Runs of home bins that can hold a point near enough to a brick to matter for
// cutoffs T <= 16 and T <= 25 (scatter form): the brick's own 64 bins, and of each of
// the 26 neighbours the layers of subcells next to the brick (local coordinate 0
// toward a neighbour on the + side; 3, or 2 and 3, toward one on the - side; all four
// along an axis where it is level with the brick), cut into runs of consecutive bin
// indices (bin = z*16 + y*4 + x).  A point homed farther out is at least 5 voxels from
// every voxel of the brick on some axis toward the + side (the brick's last voxel is at
// 15, the second layer starts at 20), and more than 4 (one layer) or 8 (two layers)
// toward the - side, so its d^2 >= 25 (> 16 with one layer) >= T.  Entry: direction
// (dx+1) + 3 (dy+1) + 9 (dz+1) | first bin << 8 | bins << 16.  One layer: 87 runs,
// 216 bins; two: 115 runs, 343 bins (of the neighbourhood's 1,728).
constexpr int kLayerRunsMax = 115;
struct LayerRunTable {
    uint32_t e[kLayerRunsMax];
    int n;
};
constexpr LayerRunTable make_layer_run_table(int minus_layers) {
    LayerRunTable t{};
    int n = 0;
    for (int d = 0; d < 27; d++) {
        const int dd[3] = {d % 3 - 1, (d / 3) % 3 - 1, d / 9 - 1};
        int run0 = -1, prev = -2;
        for (int b = 0; b <= 64; b++) {
            bool in = b < 64;
            for (int a = 0; a < 3 && in; a++) {
                const int c = (b >> (2 * a)) & 3;
                in = dd[a] == 0 || (dd[a] > 0 ? c == 0 : c >= 4 - minus_layers);
            }
            if (in && b == prev + 1) {
                prev = b;
                continue;
            }
            if (run0 >= 0) t.e[n++] = (uint32_t)d | ((uint32_t)run0 << 8) | ((uint32_t)(prev - run0 + 1) << 16);
            run0 = in ? b : -1;
            prev = in ? b : -2;
        }
    }
    t.n = n;
    return t;
}
static __device__ const LayerRunTable kLayerRuns16 = make_layer_run_table(1);
static __device__ const LayerRunTable kLayerRuns25 = make_layer_run_table(2);
static_assert(make_layer_run_table(1).n == 87 && make_layer_run_table(2).n == 115, "layer run counts");

// One block per linked leaf.  Setup: the brick's record from k_gather_prep (the
// ranks of the 3x3x3 neighbour bricks and their point ranges in the home-binned
// array, a brick's 64 bins being contiguous; the origin and the atlas slot).
// Then one of two forms, chosen per brick by the number of points homed in the
// neighbourhood (either form is exact; the choice only affects speed):
//
// scatter (sparse bricks): every thread loads one neighbourhood point at a time
//   (with a cutoff T <= 25 only the points homed in the neighbours' subcell layers
//   next to the brick, kLayerRuns16/25; all loads in flight together) and derives
//   its reach in this brick (member
//   subcells cut to the cutoff box); each warp then walks its live points: the
//   reach's voxel columns 32 at a time, each lane one column, z two at a time
//   over the part of the cutoff sphere above the group's nearest column, min d^2
//   reduced into the shared tile with shared atomics.
// gather (dense bricks): each warp owns whole subcells in turn.  It visits
//   candidate home bins in ascending order of their lower-bound distance lb^2 to
//   the subcell (host table) and stops at the first bin with lb^2 >= wmax, the
//   largest current minimum of its 64 voxels; a point is queued only if it is a
//   member and its own lower bound to the subcell's voxel box is below wmax.
//   Skipped points cannot lower any voxel's minimum, so the result is exact.
//
// One coalesced write of the brick from the tile at the end.
// kMinB blocks per SM, from the tuning table (10 or 8).  10 (48 registers; the 21.4 KiB
// of shared memory per block allows 10): measured 0.774 ms on the fluid frame against
// 0.787 at 9 and 0.798 at 8.  kPackedWalk: the scatter form's walk for cutoff radii
// below kPackedReach (columns of 32 entries packed across the warp), a kernel of its
// own so that the walk for larger reaches keeps its code.
template <typename T, int kMinB, bool kPackedWalk>
__global__ void __launch_bounds__(kGatherThreads, kMinB) k_gather(const int4* __restrict__ gtab,
                                                           const uint32_t* __restrict__ bin_off,
                                                           const float4* __restrict__ pts,
                                                           const int4* __restrict__ offs, int noffs,
                                                           GatherParams gp, T* __restrict__ interior) {
    __shared__ __align__(16) uint32_t tile[4096];
    __shared__ int nrank[27];
    __shared__ uint32_t nb_beg[27];
    __shared__ uint32_t nb_pre[28];  // exclusive prefix of the neighbours' point counts
    // scatter form: the live-point list; gather form: per-warp point queues
    __shared__ __align__(16) unsigned char scratch[kScratch];
    __shared__ int nlive;
    __shared__ int next_sc;  // gather form: next subcell to search
    __shared__ int pslot[27];  // fused apron: slot of the neighbour at each direction, -1: none / no push
    // scatter form with T <= 25: the layer runs' first points and exclusive prefix (kLayerRuns16/25)
    __shared__ uint32_t lr_beg[kLayerRunsMax];
    __shared__ uint32_t lr_pre[128];

    const int4* rec = gtab + (size_t)blockIdx.x * 32;  // this brick's setup (k_gather_prep)
    const int4 head = __ldg(rec + 27);
    const int slot = head.w;
    if (slot < 0) return;
    const int ox = head.x, oy = head.y, oz = head.z;
    const int sx0 = ox >> 2, sy0 = oy >> 2, sz0 = oz >> 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int v = threadIdx.x; v < 1024; v += blockDim.x)
        reinterpret_cast<uint4*>(tile)[v] = make_uint4(gp.tbits, gp.tbits, gp.tbits, gp.tbits);
    if (warp == 0) {
        int r = -1;
        uint32_t beg = 0, cnt = 0;
        // fused apron: the grid passed the push check (k_push_check), so a linked
        // leaf's rank is its atlas slot
        const bool push_ok = gp.apron != nullptr && __ldg(gp.apron_bad) == 0;
        if (lane < 27) {
            const int4 e = __ldg(rec + lane);
            r = e.x;
            beg = (uint32_t)e.y;
            cnt = (uint32_t)e.z;
            nrank[lane] = r;
            nb_beg[lane] = beg;
            pslot[lane] = (push_ok && lane != 13) ? r : -1;
        }
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane < 28) nb_pre[lane] = incl - cnt;
    }
    __syncthreads();
    const uint32_t ncand = nb_pre[27];
    const float Tf = __uint_as_float(gp.tbits);

    if (ncand <= (unsigned)gp.dense_min) {
        // ------------------------------------------------------ scatter form
        // A point's reach inside this brick: its member subcells, cut to the
        // voxels within rcut of it on every axis (brick-local voxel box).  The
        // live points of a batch of candidates go to a shared list; then the warps
        // take the list's entries in turn, each covering its entry's whole reach
        // (its columns row-major, 32 per group, a lane per column; z walked two at
        // a time over the group's reach) with shared atomicMin.
        float4* live_pts = reinterpret_cast<float4*>(scratch);
        // cutoff T <= 25: the candidates are the points of the layer runs (kLayerRuns16/25)
        // instead of all 27 neighbours' points
        const bool layered = gp.tbits <= 0x41C80000u;  // 25.0f
        const LayerRunTable& runs = gp.tbits <= 0x41800000u ? kLayerRuns16 : kLayerRuns25;  // 16.0f
        const int nruns = runs.n;
        uint32_t nsc = ncand;
        if (layered) {
            if (threadIdx.x < nruns) {
                const uint32_t e = runs.e[threadIdx.x];
                const int r = nrank[e & 0xFF];
                uint32_t b = 0, c = 0;
                if (r >= 0) {
                    const size_t b0 = (size_t)r * 64 + ((e >> 8) & 0xFF);
                    b = __ldg(bin_off + b0);
                    c = __ldg(bin_off + b0 + (e >> 16)) - b;
                }
                lr_beg[threadIdx.x] = b;
                lr_pre[threadIdx.x] = c;  // the count, replaced by the prefix below
            }
            __syncthreads();
            if (warp == 0) {  // exclusive prefix of the runs' counts, four per lane
                uint32_t c[4];
#pragma unroll
                for (int i = 0; i < 4; i++) c[i] = 4 * lane + i < nruns ? lr_pre[4 * lane + i] : 0u;
                const uint32_t sum = c[0] + c[1] + c[2] + c[3];
                uint32_t incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= o) incl += v;
                }
                __syncwarp();
                const uint32_t ex = incl - sum;
                lr_pre[4 * lane] = ex;
                lr_pre[4 * lane + 1] = ex + c[0];
                lr_pre[4 * lane + 2] = ex + c[0] + c[1];
                lr_pre[4 * lane + 3] = ex + c[0] + c[1] + c[2];
            }
            __syncthreads();
            nsc = lr_pre[nruns];
        }
        for (uint32_t cbase = 0; cbase < nsc; cbase += kLive) {
            if (threadIdx.x == 0) nlive = 0;
            __syncthreads();
            const uint32_t cend = min(nsc, cbase + (uint32_t)kLive);
            for (uint32_t idx = cbase + threadIdx.x; idx < cend; idx += blockDim.x) {
                uint32_t src;
                if (layered) {
                    int k = 0;  // run holding candidate idx: last k with lr_pre[k] <= idx
#pragma unroll
                    for (int step = 64; step > 0; step >>= 1)
                        if (k + step < nruns && lr_pre[k + step] <= idx) k += step;
                    src = lr_beg[k] + (idx - lr_pre[k]);
                } else {
                    int nb = 0;  // neighbour holding point idx: last nb with nb_pre[nb] <= idx
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (nb + step < 27 && nb_pre[nb + step] <= idx) nb += step;
                    src = nb_beg[nb] + (idx - nb_pre[nb]);
                }
                const float4 q = pts[src];
                const int pk = __float_as_int(q.w);
                const float pw[3] = {q.x, q.y, q.z};
                const int org[3] = {ox, oy, oz};
                int packed = 0;
                bool ok = true;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    int rl, ru;
                    ok &= mask_range(pk, a, rl, ru);
                    const int dh = (((int)pw[a]) >> 2) - (org[a] >> 2);  // home subcell, brick-relative
                    const float lp = fsub(pw[a], (float)org[a]);
                    int v0 = max(4 * (dh + rl), (int)ceilf(fsub(lp, gp.rcut)));
                    int v1 = min(4 * (dh + ru) + 3, (int)floorf(fadd(lp, gp.rcut)));
                    v0 = max(v0, 0);
                    v1 = min(v1, 15);
                    ok &= v0 <= v1;
                    packed |= (v0 | (v1 << 4)) << (8 * a);
                }
                if (ok) live_pts[atomicAdd(&nlive, 1)] = make_float4(q.x, q.y, q.z, __int_as_float(packed));
            }
            __syncthreads();
            const int nl = nlive;
            const float rc2 = __fmul_rn(gp.rcut, gp.rcut);
            if constexpr (kPackedWalk) {
                // small reaches (a few columns each): a warp takes 32 entries at a time and
                // lays their columns out in one list, a lane per (entry, column) item, so that
                // lanes are not left idle by entries of fewer than 32 columns; each lane walks
                // z over its own column's cut of the cutoff sphere
                for (int e0 = warp * 32; e0 < nl; e0 += kGatherThreads) {
                    const int e = e0 + lane;
                    float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    int ncol = 0, nx = 1;
                    if (e < nl) {
                        L = live_pts[e];
                        const int bx = __float_as_int(L.w);
                        nx = ((bx >> 4) & 15) - (bx & 15) + 1;
                        ncol = nx * (((bx >> 12) & 15) - ((bx >> 8) & 15) + 1);
                    }
                    const float rnx = __frcp_rn((float)nx);  // rounded 1 / nx, as kRcp16
                    int incl = ncol;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= o) incl += v;
                    }
                    const int pre = incl - ncol, total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                    for (int t0 = 0; t0 < total; t0 += 32) {
                        const int t = t0 + lane;
                        int j = 0;  // entry of item t: the last lane with pre <= t
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            const int pj = __shfl_sync(0xFFFFFFFFu, pre, j + step);
                            if (pj <= t) j += step;
                        }
                        const float jx = __shfl_sync(0xFFFFFFFFu, L.x, j), jy = __shfl_sync(0xFFFFFFFFu, L.y, j);
                        const float jz = __shfl_sync(0xFFFFFFFFu, L.z, j);
                        const int bx = __shfl_sync(0xFFFFFFFFu, __float_as_int(L.w), j);
                        const int jnx = __shfl_sync(0xFFFFFFFFu, nx, j);
                        const float jr = __shfl_sync(0xFFFFFFFFu, rnx, j);
                        const int k = t - __shfl_sync(0xFFFFFFFFu, pre, j);
                        const int ry = (int)__fmul_rn((float)k + 0.5f, jr);  // k / nx, as in the walk below
                        const int x = (bx & 15) + (k - ry * jnx), y = ((bx >> 8) & 15) + ry;
                        const float dx = fsub(jx, (float)(ox + x)), dy = fsub(jy, (float)(oy + y));
                        const float dxy = __fmaf_rn(dy, dy, __fmul_rn(dx, dx));
                        if (!(t < total && __float_as_uint(dxy) < gp.tbits)) continue;
                        const float zr = sqrt_approx(fsub(rc2, dxy));  // rcut's margin covers its error
                        const float lz = fsub(jz, (float)oz);
                        const int za = max((bx >> 16) & 15, (int)ceilf(lz - zr)), zb = min((bx >> 20) & 15, (int)floorf(lz + zr));
                        uint32_t* col = tile + (za << 8) + (y << 4) + x;
                        float fz = (float)(oz + za);  // integer-valued: steps of 1 are exact
                        for (int z = za; z <= zb; z++, col += 256, fz += 1.0f) {
                            const float dz = fsub(jz, fz);
                            atomicMin(col, __float_as_uint(__fmaf_rn(dz, dz, dxy)));
                        }
                    }
                }
            } else
            // warps take the live entries in turn; a warp covers all of its entry's
            // reach (rows in groups of 4), so an entry is decoded once, not once per
            // warp, and warps may update the same voxel: shared atomicMin
            for (int e = warp; e < nl; e += kGatherThreads / 32) {
                const float4 L = live_pts[e];
                const int bx = __float_as_int(L.w);
                const int x0 = bx & 15, x1 = (bx >> 4) & 15;
                const int Y0 = (bx >> 8) & 15, Y1 = (bx >> 12) & 15;
                const int z0 = (bx >> 16) & 15, z1 = (bx >> 20) & 15;
                const int nx = x1 - x0 + 1, ncol = nx * (Y1 - Y0 + 1);
                const float rnx = kRcp16[nx];
                const float lz = fsub(L.z, (float)oz);  // brick-local z
                const f32x2 pzz = f2pack(L.z, L.z);
                const f32x2 two = f2pack(2.0f, 2.0f);
                // the reach's columns, row-major over its rectangle, 32 per group
                for (int kb = 0; kb < ncol; kb += 32) {
                    const int k = kb + lane;
                    // k / nx: (k + 0.5) / nx is at least 1/32 away from an integer and the
                    // product's error is below 1e-4 for k < 512, so truncation is exact
                    const int ry = (int)__fmul_rn((float)k + 0.5f, rnx);
                    const int x = x0 + (k - ry * nx), y = Y0 + ry;
                    const float dx = fsub(L.x, (float)(ox + x)), dy = fsub(L.y, (float)(oy + y));
                    const float dxy = __fmaf_rn(dy, dy, __fmul_rn(dx, dx));
                    const bool in = k < ncol && __float_as_uint(dxy) < gp.tbits;
                    // z reach of the group: the sphere of radius rcut cut at its column
                    // nearest the point (a superset of every voxel with d^2 < T); no column
                    // in: mn = inf, zr2 < 0
                    const uint32_t mn = __reduce_min_sync(0xFFFFFFFFu, in ? __float_as_uint(dxy) : 0x7F800000u);
                    const float zr2 = fsub(rc2, __uint_as_float(mn));
                    if (!(zr2 >= 0.0f)) continue;
                    const float zr = sqrt_approx(zr2);  // rcut's margin (>= 0.01) covers its error
                    const int za = max(z0, (int)ceilf(lz - zr)), zb = min(z1, (int)floorf(lz + zr));
                    if (!in || za > zb) continue;
                    uint32_t* col = tile + (za << 8) + (y << 4) + x;
                    const float fz = (float)(oz + za);  // integer-valued: steps of 1 and 2 are exact
                    const f32x2 dxy2 = f2pack(dxy, dxy);
                    f32x2 fzz = f2pack(fz, fz + 1.0f);
                    int z = za;
#pragma unroll 2
                    for (; z < zb; z += 2, col += 512) {  // two z per step, packed FP32
                        const f32x2 dz = f2sub(pzz, fzz);
                        const f32x2 d = f2fma(dz, dz, dxy2);
                        fzz = f2add(fzz, two);
                        atomicMin(col, __float_as_uint(f2lo(d)));
                        atomicMin(col + 256, __float_as_uint(f2hi(d)));
                    }
                    if (z == zb) {
                        const float dz = fsub(L.z, f2lo(fzz));
                        atomicMin(col, __float_as_uint(__fmaf_rn(dz, dz, dxy)));
                    }
                }
            }
            __syncthreads();  // the list is refilled by the next batch
        }
    } else {
        // ------------------------------------------------------- gather form
        // Lane layout: half hf = lane >> 4 takes every other pair of queued points,
        // column (cx, cy) = lane & 15 holds the 4 voxels z = 0..3 of that column, so
        // one pass over the queue evaluates 4 points per warp step.  The two halves
        // keep partial minima of the same voxels and merge them after every bin.
        float* qx = reinterpret_cast<float*>(scratch) + warp * (3 * kQueue);
        float* qy = qx + kQueue;
        float* qz = qy + kQueue;
        if (threadIdx.x == 0) next_sc = blockDim.x >> 5;  // published by the pass's barriers
        unit_box_pass(tile, nrank, bin_off, pts, ox, oy, oz, reinterpret_cast<uint32_t*>(scratch),
                      reinterpret_cast<uint32_t*>(scratch) + 64);
        const int hf = lane >> 4, cx = lane & 3, cy = (lane >> 2) & 3;
        const unsigned lt = (1u << lane) - 1u;
        constexpr uint32_t kOne = 0x3F800000u;  // 1.0f: minima below it are exact after the unit-box pass
        // subcells are taken in turn from a shared counter (the searches' costs differ widely)
        auto next_subcell = [&]() {
            int n = 0;
            if (lane == 0) n = atomicAdd(&next_sc, 1);
            return __shfl_sync(0xFFFFFFFFu, n, 0);
        };
        for (int sc = warp; sc < 64; sc = next_subcell()) {
            const int lx = sc & 3, ly = (sc >> 2) & 3, lz = sc >> 4;
            const int tv = ((4 * lz) << 8) | ((4 * ly + cy) << 4) | (4 * lx + cx);
            float m0 = __uint_as_float(tile[tv]), m1 = __uint_as_float(tile[tv + 256]);
            float m2 = __uint_as_float(tile[tv + 512]), m3 = __uint_as_float(tile[tv + 768]);
            // needy voxels (minimum >= 1): the search runs for them alone, over the
            // points that can come nearer to their bounding box than wmax, the
            // largest needy minimum
            // (with a cutoff T <= 1 the unit-box pass alone is exact: d^2 < T needs every axis below 1)
            const uint32_t nb1 = gp.tbits > kOne ? kOne : 0xFFFFFFFFu;
            const bool n0 = __float_as_uint(m0) >= nb1, n1 = __float_as_uint(m1) >= nb1;
            const bool n2 = __float_as_uint(m2) >= nb1, n3 = __float_as_uint(m3) >= nb1;
            const bool anyn = n0 | n1 | n2 | n3;
            if (!__any_sync(0xFFFFFFFFu, anyn)) continue;
            const int Sx = sx0 + lx, Sy = sy0 + ly, Sz = sz0 + lz;
            const int vx = ox + 4 * lx + cx, vy = oy + 4 * ly + cy, vz = oz + 4 * lz;
            const float fx = (float)vx, fy = (float)vy;
            const float fz = (float)vz;
            const f32x2 fxx = f2pack(fx, fx), fyy = f2pack(fy, fy);
            const f32x2 z0 = f2pack(fz, fz), z1 = f2pack(fz + 1.0f, fz + 1.0f);
            const f32x2 z2 = f2pack(fz + 2.0f, fz + 2.0f), z3 = f2pack(fz + 3.0f, fz + 3.0f);
            const int zlo = n0 ? 0 : (n1 ? 1 : (n2 ? 2 : 3)), zhi = n3 ? 3 : (n2 ? 2 : (n1 ? 1 : 0));
            const int nlx = __reduce_min_sync(0xFFFFFFFFu, anyn ? vx : INT_MAX);
            const int nhx = __reduce_max_sync(0xFFFFFFFFu, anyn ? vx : INT_MIN);
            const int nly = __reduce_min_sync(0xFFFFFFFFu, anyn ? vy : INT_MAX);
            const int nhy = __reduce_max_sync(0xFFFFFFFFu, anyn ? vy : INT_MIN);
            const int nlz = __reduce_min_sync(0xFFFFFFFFu, anyn ? vz + zlo : INT_MAX);
            const int nhz = __reduce_max_sync(0xFFFFFFFFu, anyn ? vz + zhi : INT_MIN);
            const float blx = (float)nlx, bhx = (float)nhx;
            const float bly = (float)nly, bhy = (float)nhy;
            const float blz = (float)nlz, bhz = (float)nhz;
            auto needy_max = [&]() {
                const float a = fmaxf(n0 ? m0 : 0.0f, n1 ? m1 : 0.0f), b = fmaxf(n2 ? m2 : 0.0f, n3 ? m3 : 0.0f);
                return __uint_as_float(__reduce_max_sync(0xFFFFFFFFu, __float_as_uint(fmaxf(a, b))));
            };
            float wmax = needy_max();
            int nq = 0;
            bool drained = false;  // a drain since wmax was last taken
            // evaluate the queued points [0, nq) against the column's 4 voxels
            auto drain = [&]() {
                drained = true;
                const int n4 = (nq + 3) & ~3;
                if (lane < n4 - nq) {  // pad with points at infinity (d^2 = inf)
                    qx[nq + lane] = __int_as_float(0x7F800000);
                    qy[nq + lane] = __int_as_float(0x7F800000);
                    qz[nq + lane] = __int_as_float(0x7F800000);
                }
                __syncwarp();
                for (int i = 2 * hf; i < n4; i += 4) {
                    const f32x2 px = *reinterpret_cast<const f32x2*>(qx + i);
                    const f32x2 py = *reinterpret_cast<const f32x2*>(qy + i);
                    const f32x2 pz = *reinterpret_cast<const f32x2*>(qz + i);
                    const f32x2 dx = f2sub(px, fxx), dy = f2sub(py, fyy);
                    const f32x2 dxy = f2fma(dy, dy, f2mul(dx, dx));
                    f32x2 dz = f2sub(pz, z0), r = f2fma(dz, dz, dxy);
                    m0 = fmin3(m0, f2lo(r), f2hi(r));
                    dz = f2sub(pz, z1); r = f2fma(dz, dz, dxy);
                    m1 = fmin3(m1, f2lo(r), f2hi(r));
                    dz = f2sub(pz, z2); r = f2fma(dz, dz, dxy);
                    m2 = fmin3(m2, f2lo(r), f2hi(r));
                    dz = f2sub(pz, z3); r = f2fma(dz, dz, dxy);
                    m3 = fmin3(m3, f2lo(r), f2hi(r));
                }
                __syncwarp();
                nq = 0;
            };
            // offsets in groups of 32: each lane resolves one offset's bin range up
            // front (one memory round trip per group instead of one per bin)
            for (int g0 = 0; g0 < noffs; g0 += 32) {
                // sorted by lb^2: a group starting at or beyond wmax ends the subcell (tested
                // before the group's bin ranges are loaded)
                if ((float)__ldg(&offs[g0].w) >= wmax) break;
                const int e = g0 + lane;
                uint32_t gbeg = 0, gcnt = 0;
                int gneed = 0, gbnd = 0;
                if (e < noffs) {
                    const int4 o = offs[e];
                    gneed = member_bits(o.x, o.y, o.z);
                    const int hx = Sx + o.x, hy = Sy + o.y, hz = Sz + o.z;
                    // bound for the bin's points [4h, 4h + 4) against the needy box
                    const int gx = max(0, max(4 * hx - nhx, nlx - 4 * hx - 4));
                    const int gy = max(0, max(4 * hy - nhy, nly - 4 * hy - 4));
                    const int gz = max(0, max(4 * hz - nhz, nlz - 4 * hz - 4));
                    gbnd = gx * gx + gy * gy + gz * gz;  // at most 3 * 48^2: 13 bits
                    if (hx >= 0 && hy >= 0 && hz >= 0 && (float)gbnd < wmax) {
                        const int bx = (hx >> 2) - (sx0 >> 2), by = (hy >> 2) - (sy0 >> 2), bz = (hz >> 2) - (sz0 >> 2);
                        const int r = nrank[(bz + 1) * 9 + (by + 1) * 3 + (bx + 1)];
                        if (r >= 0) {
                            const unsigned bin = (unsigned)r * 64u + (unsigned)(((hz & 3) << 4) | ((hy & 3) << 2) | (hx & 3));
                            gbeg = __ldg(bin_off + bin);
                            gcnt = __ldg(bin_off + bin + 1) - gbeg;
                        }
                    }
                }
                unsigned nonempty = __ballot_sync(0xFFFFFFFFu, gcnt > 0);
                while (nonempty) {
                    // the group's bins nearest the needy box first (ties: lowest lane), so that
                    // wmax falls early; a bin whose bound is at or beyond wmax ends the group,
                    // as every bin left is at least as far (later groups: the test above)
                    const uint32_t kmin = __reduce_min_sync(
                        0xFFFFFFFFu, ((nonempty >> lane) & 1u) ? ((uint32_t)gbnd << 5) | (uint32_t)lane : 0xFFFFFFFFu);
                    const int l = (int)(kmin & 31u);
                    nonempty &= ~(1u << l);
                    if ((float)(kmin >> 5) >= wmax) break;
                    const uint32_t beg = __shfl_sync(0xFFFFFFFFu, gbeg, l);
                    const uint32_t end = beg + __shfl_sync(0xFFFFFFFFu, gcnt, l);
                    const int need = __shfl_sync(0xFFFFFFFFu, gneed, l);
                    // 64 points per round: both loads in flight before either is filtered
                    for (uint32_t base = beg; base < end; base += 64) {
                        float4 q[2];
                        bool ok[2];
#pragma unroll
                        for (int u = 0; u < 2; u++) {
                            const uint32_t j = base + 32 * u + lane;
                            ok[u] = j < end;
                            q[u] = ok[u] ? pts[j] : make_float4(0, 0, 0, 0);
                        }
#pragma unroll
                        for (int u = 0; u < 2; u++) {
                            if (ok[u]) {
                                ok[u] = false;
                                if ((__float_as_int(q[u].w) & need) == need) {
                                    const float gx = fmaxf(0.0f, fmaxf(fsub(blx, q[u].x), fsub(q[u].x, bhx)));
                                    const float gy = fmaxf(0.0f, fmaxf(fsub(bly, q[u].y), fsub(q[u].y, bhy)));
                                    const float gz = fmaxf(0.0f, fmaxf(fsub(blz, q[u].z), fsub(q[u].z, bhz)));
                                    const float lb = __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, __fmul_rn(gx, gx)));
                                    ok[u] = lb < wmax;
                                }
                            }
                            const unsigned live = __ballot_sync(0xFFFFFFFFu, ok[u]);
                            if (ok[u]) {
                                const int k = nq + __popc(live & lt);
                                qx[k] = q[u].x;
                                qy[k] = q[u].y;
                                qz[k] = q[u].z;
                            }
                            nq += __popc(live);
                            if (nq >= 32) drain();
                        }
                    }
                    // wmax after a drain: the largest needy minimum over both halves'
                    // partial minima, an upper bound of the merged one (so the bins and
                    // points it skips still cannot lower any needy voxel)
                    if (drained) {
                        wmax = needy_max();
                        drained = false;
                    }
                }
            }
            if (nq) drain();
            // merge the halves' minima
            m0 = fminf(m0, __shfl_xor_sync(0xFFFFFFFFu, m0, 16));
            m1 = fminf(m1, __shfl_xor_sync(0xFFFFFFFFu, m1, 16));
            m2 = fminf(m2, __shfl_xor_sync(0xFFFFFFFFu, m2, 16));
            m3 = fminf(m3, __shfl_xor_sync(0xFFFFFFFFu, m3, 16));
            if (hf == 0) {
                tile[tv] = __float_as_uint(m0);
                tile[tv + 256] = __float_as_uint(m1);
                tile[tv + 512] = __float_as_uint(m2);
                tile[tv + 768] = __float_as_uint(m3);
            }
        }
    }
    __syncthreads();
    const bool push = gp.apron != nullptr;
    write_tile<T>(gp, tile, interior + (size_t)slot * 4096, push);
    if (push) {
        __syncthreads();
        push_apron<T>(tile, pslot, reinterpret_cast<T*>(gp.apron));
    }
}

// ---- materialized subcell lists (reference-shaped; export + fallback) ----

template <bool kFill>
__device__ void list_points(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant qz,
                            const uint32_t* scmap, uint32_t* cnt, const uint32_t* off, float* out3, ClrSrc clr = {},
                            uint32_t* out_clr = nullptr) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (long long)gridDim.x * blockDim.x) {
        float w[3];
        if (!load_valid(p, i, trans, w[0], w[1], w[2])) continue;
        int lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; a++) sc_range(w[a], R, lo[a], hi[a]);
        for (int sx = lo[0]; sx <= hi[0]; sx += kSc)
            for (int sy = lo[1]; sy <= hi[1]; sy += kSc)
                for (int sz = lo[2]; sz <= hi[2]; sz += kSc) {
                    if (sx < 0 || sy < 0 || sz < 0) continue;
                    long long leaf = linked_leaf(lg, t, sx, sy, sz);
                    if (leaf < 0) continue;
                    const Node& nd = t.nodes[0][leaf];
                    int loc = (((sz - nd.pos[2]) >> 2) << 4) | (((sy - nd.pos[1]) >> 2) << 2) | ((sx - nd.pos[0]) >> 2);
                    unsigned idx = scmap[leaf] * 64u + (unsigned)loc;
                    unsigned k = atomicAdd(cnt + idx, 1u);
                    if (kFill) {
                        float ps[3];
                        stored_pos(qz, w, ps);
                        float* o = out3 + 3ull * (off[idx] + k);
                        o[0] = ps[0];
                        o[1] = ps[1];
                        o[2] = ps[2];
                        if (out_clr)
                            out_clr[off[idx] + k] =
                                __ldg(reinterpret_cast<const uint32_t*>(clr.base + i * (long long)clr.stride + clr.off));
                    }
                }
    }
}
__global__ void k_list_count(TreeView t, LeafGrid lg, PointSrc p, float3 trans, float R, Quant qz, const uint32_t* scmap,
                             uint32_t* cnt) {
    list_points<false>(t, lg, p, trans, R, qz, scmap, cnt, nullptr, nullptr);
}
__global__ void k_list_fill(TreeView t, LeafGrid lg, PointSrc p, float3 trans, float R, Quant qz, const uint32_t* scmap,
                            const uint32_t* off, uint32_t* cursor, float* out3, ClrSrc clr, uint32_t* out_clr) {
    list_points<true>(t, lg, p, trans, R, qz, scmap, cursor, off, out3, clr, out_clr);
}

// reference-shaped gather over materialized lists: one block per linked leaf,
// thread per voxel (16 voxels per thread), each voxel scans its subcell's list
template <typename T>
__global__ void k_gather_lists(TreeView t, const int* __restrict__ linked, const uint32_t* __restrict__ off,
                               const float* __restrict__ pts3, GatherParams gp, T* __restrict__ interior) {
    __shared__ uint32_t tile[4096];
    const int leaf = linked[blockIdx.x];
    const Node nd = t.nodes[0][leaf];
    const int slot = slot_of_value(nd.value, gp.ax, gp.ay);
    if (slot < 0) return;
    for (int v = threadIdx.x; v < 4096; v += blockDim.x) {
        int x = v & 15, y = (v >> 4) & 15, z = v >> 8;
        int s = ((z >> 2) << 4) | ((y >> 2) << 2) | (x >> 2);
        unsigned idx = blockIdx.x * 64u + (unsigned)s;
        float fx = (float)(nd.pos[0] + x), fy = (float)(nd.pos[1] + y), fz = (float)(nd.pos[2] + z);
        uint32_t m = gp.tbits;
        for (uint32_t j = off[idx]; j < off[idx + 1]; j++) {
            float dx = fsub(pts3[3ull * j], fx), dy = fsub(pts3[3ull * j + 1], fy), dz = fsub(pts3[3ull * j + 2], fz);
            float d = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
            m = min(m, __float_as_uint(d));
        }
        tile[v] = m;
    }
    __syncthreads();
    write_tile<T>(gp, tile, interior + (size_t)slot * 4096, false);
}

// ---- colour averages (GatherDensity / GatherLevelSet with a colour channel) ----
//
// The reference (PT.cuh:717-731, 757-771) gives every voxel of a subcell
//   CLR2CHAR((accum ? CHAR2CLR(old) : (0,0,0,1)) + sum_j CHAR2CLR(c_j)) / (n + accum))
// over the n entries of the subcell's list, adding the FP32 terms c/255 in the
// arbitrary order of its atomically filled list.  Here the sum is exact: the bytes
// are added as integers (with the old colour's bytes, or 255 for the alpha of the
// non-accumulating start), divided by 255 once, then the reference's remaining
// FP32 steps follow.  CLR2CHAR's uchar(x) conversion is the reference kernels' (pinned
// by golden fixtures of them): truncation to a 32-bit unsigned integer (NaN and negative
// values to 0, 2^32 and above to 0xFFFFFFFF), keeping the low byte, so a component
// above 255 wraps.

__device__ __forceinline__ uint32_t clr_byte(float x) {
    if (!(x == x) || x <= 0.0f) return 0u;
    if (x >= 4294967296.0f) return 255u;
    return (uint32_t)x & 0xFFu;
}
__device__ __forceinline__ uint32_t clr_average(const uint32_t sum[4], uint32_t n, uint32_t old, int accum) {
    uint32_t out = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t t = sum[k] + (accum ? ((old >> (8 * k)) & 0xFFu) : (k == 3 ? 255u : 0u));
        float c = __fdiv_rn(__uint2float_rn(t), 255.0f);
        c = __fdiv_rn(c, __uint2float_rn(n + (accum ? 1u : 0u)));
        out |= clr_byte(__fmul_rn(c, 255.0f)) << (8 * k);
    }
    return out;
}

// One block of 128 threads per linked brick; warp w takes subcells w, w+4, ...  For
// its subcell S the warp visits the home bins H = S + o, o in [olo, ohi]^3 (every
// offset at which a member can be homed), a lane per offset to resolve the bin
// ranges, then the lanes stride over each bin's points and keep those whose
// membership masks include S.  Integer sums, so the result is deterministic.
__global__ void __launch_bounds__(128) k_gather_colour(const int4* __restrict__ gtab, const uint32_t* __restrict__ bin_off,
                                                       const float4* __restrict__ pts, const uint32_t* __restrict__ pclr,
                                                       int olo, int ohi, int accum, uint32_t* __restrict__ out) {
    __shared__ int nrank[27];
    const int4* rec = gtab + (size_t)blockIdx.x * 32;
    const int4 head = __ldg(rec + 27);
    const int slot = head.w;
    if (slot < 0) return;
    if (threadIdx.x < 27) nrank[threadIdx.x] = __ldg(rec + threadIdx.x).x;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sx0 = head.x >> 2, sy0 = head.y >> 2, sz0 = head.z >> 2;
    const int span = ohi - olo + 1, noff = span * span * span;
    uint32_t* dst = out + (size_t)slot * 4096;
    for (int sc = warp; sc < 64; sc += 4) {
        const int lx = sc & 3, ly = (sc >> 2) & 3, lz = sc >> 4;
        const int Sx = sx0 + lx, Sy = sy0 + ly, Sz = sz0 + lz;
        uint32_t sum[4] = {0u, 0u, 0u, 0u}, n = 0;
        for (int g0 = 0; g0 < noff; g0 += 32) {
            const int e = g0 + lane;
            uint32_t beg = 0, cnt = 0;
            int need = 0;
            if (e < noff) {
                const int ox = olo + e % span, oy = olo + (e / span) % span, oz = olo + e / (span * span);
                const int hx = Sx + ox, hy = Sy + oy, hz = Sz + oz;
                if (hx >= 0 && hy >= 0 && hz >= 0) {
                    const int bx = (hx >> 2) - (sx0 >> 2), by = (hy >> 2) - (sy0 >> 2), bz = (hz >> 2) - (sz0 >> 2);
                    const int r = nrank[(bz + 1) * 9 + (by + 1) * 3 + (bx + 1)];
                    if (r >= 0) {
                        const unsigned bin = (unsigned)r * 64u + (unsigned)(((hz & 3) << 4) | ((hy & 3) << 2) | (hx & 3));
                        beg = __ldg(bin_off + bin);
                        cnt = __ldg(bin_off + bin + 1) - beg;
                        need = member_bits(ox, oy, oz);
                    }
                }
            }
            unsigned nonempty = __ballot_sync(0xFFFFFFFFu, cnt > 0);
            while (nonempty) {
                const int l = __ffs(nonempty) - 1;
                nonempty &= nonempty - 1;
                const uint32_t b = __shfl_sync(0xFFFFFFFFu, beg, l);
                const uint32_t c = __shfl_sync(0xFFFFFFFFu, cnt, l);
                const int nd = __shfl_sync(0xFFFFFFFFu, need, l);
                for (uint32_t j = lane; j < c; j += 32) {
                    const int m = __float_as_int(__ldg(&pts[b + j].w));
                    if ((m & nd) == nd) {
                        const uint32_t v = __ldg(pclr + b + j);
                        sum[0] += v & 0xFFu;
                        sum[1] += (v >> 8) & 0xFFu;
                        sum[2] += (v >> 16) & 0xFFu;
                        sum[3] += v >> 24;
                        n++;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) sum[k] = __reduce_add_sync(0xFFFFFFFFu, sum[k]);
        n = __reduce_add_sync(0xFFFFFFFFu, n);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int v = lane + 32 * h;
            const int x = 4 * lx + (v & 3), y = 4 * ly + ((v >> 2) & 3), z = 4 * lz + (v >> 4);
            uint32_t* o = dst + (z << 8) + (y << 4) + x;
            *o = clr_average(sum, n, accum ? *o : 0u, accum);
        }
    }
}

// over materialized lists (the fallback form): one block per linked leaf, a thread
// per voxel, each summing its subcell's list
__global__ void k_gather_colour_lists(TreeView t, const int* __restrict__ linked, const uint32_t* __restrict__ off,
                                      const uint32_t* __restrict__ clr, int ax, int ay, int accum,
                                      uint32_t* __restrict__ out) {
    const int leaf = linked[blockIdx.x];
    const Node nd = t.nodes[0][leaf];
    const int slot = slot_of_value(nd.value, ax, ay);
    if (slot < 0) return;
    uint32_t* dst = out + (size_t)slot * 4096;
    for (int v = threadIdx.x; v < 4096; v += blockDim.x) {
        const int x = v & 15, y = (v >> 4) & 15, z = v >> 8;
        const int s = ((z >> 2) << 4) | ((y >> 2) << 2) | (x >> 2);
        const unsigned idx = blockIdx.x * 64u + (unsigned)s;
        uint32_t sum[4] = {0u, 0u, 0u, 0u};
        for (uint32_t j = off[idx]; j < off[idx + 1]; j++) {
            const uint32_t c = __ldg(clr + j);
            sum[0] += c & 0xFFu;
            sum[1] += (c >> 8) & 0xFFu;
            sum[2] += (c >> 16) & 0xFFu;
            sum[3] += c >> 24;
        }
        dst[v] = clr_average(sum, off[idx + 1] - off[idx], accum ? dst[v] : 0u, accum);
    }
}

// ---- legacy InsertPoints + ScatterDensity (brick binning and a splat) ----

// gvdbInsertPoints (PT.cuh:19-35): the leaf holding each point (w = p + trans; NOHIT,
// negative or outside every leaf -> -1) and the point's rank among its leaf's points
__global__ void k_insert_points(TreeView t, LeafGrid lg, PointSrc p, float3 trans, int* __restrict__ pnode,
                                uint32_t* __restrict__ pndx, uint32_t* __restrict__ gcnt) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (long long)gridDim.x * blockDim.x) {
        float x, y, z;
        load_pos(p.base, i, p.stride, p.off, x, y, z);
        int leaf = -1;
        if (z != kNoHit) {
            const float w[3] = {fadd(x, trans.x), fadd(y, trans.y), fadd(z, trans.z)};
            if (w[0] >= 0 && w[1] >= 0 && w[2] >= 0) {
                const int vx = (int)w[0], vy = (int)w[1], vz = (int)w[2];
                long long l = lg.cells ? lookup_leaf(lg, t, vx, vy, vz) : get_leaf_at_voxel(t, vx, vy, vz);
                leaf = (int)l;
            }
        }
        pnode[i] = leaf;
        if (leaf >= 0) pndx[i] = atomicAdd(gcnt + leaf, 1u);
    }
}

// gvdbSortPoints (PT.cuh:54-68): points grouped by leaf, w = p + trans
__global__ void k_sort_points(PointSrc p, float3 trans, const int* __restrict__ pnode, const uint32_t* __restrict__ pndx,
                              const uint32_t* __restrict__ goff, float* __restrict__ out3) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (long long)gridDim.x * blockDim.x) {
        const int leaf = pnode[i];
        if (leaf < 0) continue;
        float x, y, z;
        load_pos(p.base, i, p.stride, p.off, x, y, z);
        float* o = out3 + 3ull * (goff[leaf] + pndx[i]);
        o[0] = fadd(x, trans.x);
        o[1] = fadd(y, trans.y);
        o[2] = fadd(z, trans.z);
    }
}

// distFunc (PT.cuh:516-523) with one rounding per operation in source order:
// c = (bx*bx + by*by + bz*bz) / (r*r), 1 + c*(-3 + c*(3 - c))
__device__ __forceinline__ float dist_func(float px, float py, float pz, float bx, float by, float bz, float r) {
    bx = fsub(bx, px);
    by = fsub(by, py);
    bz = fsub(bz, pz);
    const float d2 = fadd(fadd(__fmul_rn(bx, bx), __fmul_rn(by, by)), __fmul_rn(bz, bz));
    const float c = __fdiv_rn(d2, __fmul_rn(r, r));
    // the source's 1.0 is a double literal: the last addition is in double, then rounded
    return __double2float_rn(__dadd_rn(1.0, (double)__fmul_rn(c, fadd(-3.0f, __fmul_rn(c, fsub(3.0f, c))))));
}

// gvdbScatterPointDensity (PT.cuh:525-571), one block per leaf over its grouped points:
// each point adds distFunc to the voxel it lies in and, with `expand`, to that voxel's
// six face neighbours inside the leaf's padded 18^3 brick (apron included), so every
// write stays in one slot.  Contributions are summed in FP64 in shared memory and added
// to the stored values once (the reference adds them one by one with unsynchronised
// read-modify-writes of the atlas).
__global__ void __launch_bounds__(256) k_scatter_density(const Node* __restrict__ leaves, long long nleaf,
                                                         const uint32_t* __restrict__ goff,
                                                         const float* __restrict__ pts3, float radius, int expand,
                                                         int res0, int ax, int ay, float* __restrict__ interior,
                                                         float* __restrict__ apron) {
    __shared__ double acc[18 * 18 * 18];
    const long long leaf = blockIdx.x;
    if (leaf >= nleaf) return;
    const uint32_t beg = goff[leaf], end = goff[leaf + 1];
    if (beg == end) return;
    const Node nd = leaves[leaf];
    const int slot = slot_of_value(nd.value, ax, ay);
    if (slot < 0) return;
    for (int v = threadIdx.x; v < 5832; v += blockDim.x) acc[v] = 0.0;
    __syncthreads();
    const float vmx = (float)nd.pos[0], vmy = (float)nd.pos[1], vmz = (float)nd.pos[2];
    const int nb[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    const int nk = expand ? 7 : 1;
    for (uint32_t j = beg + threadIdx.x; j < end; j += blockDim.x) {
        const float px = fsub(pts3[3ull * j], vmx), py = fsub(pts3[3ull * j + 1], vmy), pz = fsub(pts3[3ull * j + 2], vmz);
        const int ix = (int)px, iy = (int)py, iz = (int)pz;
        if (px < 0 || py < 0 || pz < 0 || ix >= res0 || iy >= res0 || iz >= res0) continue;
        for (int k = 0; k < nk; k++) {
            const int qx = ix + nb[k][0], qy = iy + nb[k][1], qz = iz + nb[k][2];
            const float f = dist_func(px, py, pz, (float)qx, (float)qy, (float)qz, radius);
            atomicAdd(&acc[((qz + 1) * 18 + (qy + 1)) * 18 + (qx + 1)], (double)f);
        }
    }
    __syncthreads();
    for (int v = threadIdx.x; v < 5832; v += blockDim.x) {
        const double a = acc[v];
        if (a == 0.0) continue;
        const int x = v % 18, y = (v / 18) % 18, z = v / 324;
        float* dst = (x >= 1 && x <= 16 && y >= 1 && y <= 16 && z >= 1 && z <= 16)
                         ? interior + (size_t)slot * 4096 + ((z - 1) << 8) + ((y - 1) << 4) + (x - 1)
                         : apron + (size_t)slot * kApronStride + apron_index(x, y, z);
        *dst = __double2float_rn(__dadd_rn((double)*dst, a));
    }
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }
inline unsigned gs_blocks(long long n, int t) {
    long long b = (n + t - 1) / t;
    long long cap = 152LL * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}
}  // namespace

void launch_insert_points(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, int* pnode, uint32_t* pndx,
                          uint32_t* gcnt, cudaStream_t s) {
    if (p.n <= 0) return;
    k_insert_points<<<counted(gs_blocks(p.n, 256)), 256, 0, s>>>(t, lg, p, trans, pnode, pndx, gcnt);
}
void launch_sort_points(PointSrc p, float3 trans, const int* pnode, const uint32_t* pndx, const uint32_t* goff,
                        float* out3, cudaStream_t s) {
    if (p.n <= 0) return;
    k_sort_points<<<counted(gs_blocks(p.n, 256)), 256, 0, s>>>(p, trans, pnode, pndx, goff, out3);
}
void launch_scatter_density(const Node* leaves, long long nleaf, const uint32_t* goff, const float* pts3, float radius,
                            int expand, int res0, int ax, int ay, float* interior, float* apron, cudaStream_t s) {
    if (nleaf <= 0) return;
    k_scatter_density<<<counted((unsigned)nleaf), 256, 0, s>>>(leaves, nleaf, goff, pts3, radius, expand, res0, ax, ay,
                                                      interior, apron);
}
void launch_linked_list(const Node* leaves, long long n, const uint32_t* scmap, int* linked, cudaStream_t s) {
    if (n <= 0) return;
    k_linked_list<<<counted(blocks_for(n, 256)), 256, 0, s>>>(leaves, n, scmap, linked);
}
void launch_nb_mask(const TreeView& t, const LeafGrid& lg, long long n, uint32_t* nbmask, uint32_t* bin_cnt,
                    unsigned long long* totals, cudaStream_t s) {
    k_nb_mask<<<counted(blocks_for(std::max(n, 1ll) * 32, 256)), 256, 0, s>>>(t, lg, n, nbmask, bin_cnt, totals);
}
void launch_bin_count(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q,
                      const uint32_t* scmap, const uint32_t* nbmask, uint32_t* bin_cnt, int* bin_of, uint32_t* rank_of,
                      unsigned long long* totals, int unroll, cudaStream_t s) {
    if (p.n <= 0) return;
    const unsigned b = unroll == 4 ? gs_blocks((p.n + 3) / 4, 256) : gs_blocks(p.n, 256);
    if (unroll == 1)
        k_bin_count<1><<<counted(b), 256, 0, s>>>(t, lg, p, trans, R, q, scmap, nbmask, bin_cnt, bin_of, rank_of, totals);
    else if (unroll == 4)
        k_bin_count<4><<<counted(b), 256, 0, s>>>(t, lg, p, trans, R, q, scmap, nbmask, bin_cnt, bin_of, rank_of, totals);
    else
        k_bin_count<2><<<counted(b), 256, 0, s>>>(t, lg, p, trans, R, q, scmap, nbmask, bin_cnt, bin_of, rank_of, totals);
}
void launch_bin_scatter(PointSrc p, float3 trans, float R, Quant q, const int* bin_of, const uint32_t* rank_of,
                        const uint32_t* bin_off, float4* sorted, ClrSrc clr, uint32_t* sorted_clr, int unroll,
                        cudaStream_t s) {
    if (p.n <= 0) return;
    const unsigned b = unroll == 4 ? gs_blocks((p.n + 3) / 4, 256) : gs_blocks(p.n, 256);
    uint32_t* sc = clr.base ? sorted_clr : nullptr;
    if (unroll == 2)
        k_bin_scatter<2><<<counted(b), 256, 0, s>>>(p, trans, R, q, bin_of, rank_of, bin_off, sorted, clr, sc);
    else if (unroll == 8)
        k_bin_scatter<8><<<counted(b), 256, 0, s>>>(p, trans, R, q, bin_of, rank_of, bin_off, sorted, clr, sc);
    else
        k_bin_scatter<4><<<counted(b), 256, 0, s>>>(p, trans, R, q, bin_of, rank_of, bin_off, sorted, clr, sc);
}
void launch_gather_colour(const int4* gtab, long long nbricks, const uint32_t* bin_off, const float4* pts,
                          const uint32_t* pclr, int olo, int ohi, int accum, uint32_t* out, cudaStream_t s) {
    if (nbricks <= 0) return;
    k_gather_colour<<<counted((unsigned)nbricks), 128, 0, s>>>(gtab, bin_off, pts, pclr, olo, ohi, accum, out);
}
void launch_gather_colour_lists(const TreeView& t, const int* linked, long long nbricks, const uint32_t* off,
                                const uint32_t* clr, int ax, int ay, int accum, uint32_t* out, cudaStream_t s) {
    if (nbricks <= 0) return;
    k_gather_colour_lists<<<counted((unsigned)nbricks), 256, 0, s>>>(t, linked, off, clr, ax, ay, accum, out);
}
void launch_push_check(const TreeView& t, const LeafGrid& lg, const uint32_t* scmap, const AtlasNode* amap, int used,
                       int ax, int ay, long long n, int* bad, cudaStream_t s) {
    k_push_check<<<counted(blocks_for(std::max(n, 1ll), 256)), 256, 0, s>>>(t, lg, scmap, amap, used, ax, ay, n, bad);
}
// the gather of one storage type and residency; the packed walk for cutoff radii below
// kPackedReach (a kernel of its own, so that the other keeps its code)
template <typename T, int kMinB>
void launch_gather_kernel(unsigned nb, const int4* gtab, const uint32_t* bin_off, const float4* pts, const int4* offs,
                          int noffs, const GatherParams& gp, void* interior, cudaStream_t s) {
    if (gp.rcut < kPackedReach)
        k_gather<T, kMinB, true><<<counted(nb), kGatherThreads, 0, s>>>(gtab, bin_off, pts, offs, noffs, gp, (T*)interior);
    else
        k_gather<T, kMinB, false><<<counted(nb), kGatherThreads, 0, s>>>(gtab, bin_off, pts, offs, noffs, gp, (T*)interior);
}
void launch_gather(const TreeView& t, const LeafGrid& lg, const int* linked, long long nbricks, const uint32_t* scmap,
                   const uint32_t* bin_off, const float4* pts, const int4* offs, int noffs, const GatherParams& gp,
                   int4* gtab, void* interior, cudaStream_t s) {
    if (nbricks <= 0) return;
    k_gather_prep<<<counted(blocks_for(nbricks * 32, kPrepThreads)), kPrepThreads, 0, s>>>(
        t, lg, linked, nbricks, scmap, bin_off, gp.ax, gp.ay, gp.long_min, gp.order, gtab);
    const unsigned nb = (unsigned)nbricks;
    if (gp.min_blocks == 8) {
        if (gp.dtype == 3) launch_gather_kernel<float, 8>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
        else if (gp.dtype == 100) launch_gather_kernel<__half, 8>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
        else launch_gather_kernel<__nv_bfloat16, 8>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
    } else {
        if (gp.dtype == 3) launch_gather_kernel<float, 10>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
        else if (gp.dtype == 100) launch_gather_kernel<__half, 10>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
        else launch_gather_kernel<__nv_bfloat16, 10>(nb, gtab, bin_off, pts, offs, noffs, gp, interior, s);
    }
}
void launch_list_count(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q,
                       const uint32_t* scmap, uint32_t* cnt, cudaStream_t s) {
    if (p.n <= 0) return;
    k_list_count<<<counted(gs_blocks(p.n, 128)), 128, 0, s>>>(t, lg, p, trans, R, q, scmap, cnt);
}
void launch_list_fill(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q,
                      const uint32_t* scmap, const uint32_t* off, uint32_t* cursor, float* out3, ClrSrc clr,
                      uint32_t* out_clr, cudaStream_t s) {
    if (p.n <= 0) return;
    k_list_fill<<<counted(gs_blocks(p.n, 128)), 128, 0, s>>>(t, lg, p, trans, R, q, scmap, off, cursor, out3, clr,
                                                   clr.base ? out_clr : nullptr);
}
void launch_gather_lists(const TreeView& t, const int* linked, long long nbricks, const uint32_t* off,
                         const float* pts3, const GatherParams& gp, void* interior, cudaStream_t s) {
    if (nbricks <= 0) return;
    if (gp.dtype == 3)
        k_gather_lists<float><<<counted((unsigned)nbricks), 256, 0, s>>>(t, linked, off, pts3, gp, (float*)interior);
    else if (gp.dtype == 100)
        k_gather_lists<__half><<<counted((unsigned)nbricks), 256, 0, s>>>(t, linked, off, pts3, gp, (__half*)interior);
    else
        k_gather_lists<__nv_bfloat16><<<counted((unsigned)nbricks), 256, 0, s>>>(t, linked, off, pts3, gp,
                                                                       (__nv_bfloat16*)interior);
}

}  // namespace gbvdb
