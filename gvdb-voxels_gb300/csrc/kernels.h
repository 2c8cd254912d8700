// kernels.h -- host-side launchers of the libgbvdb kernels (one declaration per launcher).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace gbvdb {

// Kernels this library launched on the calling thread: every launch site passes its
// grid size through counted(), which the launch evaluates once; the C entry points add
// the change over the call to the grid's launch count (gbvdb_get_stats).
extern thread_local long long tl_kernels;
template <class T>
inline T counted(T blocks) {
    ++tl_kernels;
    return blocks;
}

// Key-domain of one level: node coordinates [lo, lo+dim) per axis, bit offset into
// the level bitmaps (x-major linear index so that bit order == key sort order).
struct KeyDomain {
    int lo[3];
    int dim[3];
    long long bitbase;   // first bit of this level
    long long nbits;
};
struct KeyDomains {
    KeyDomain d[kMaxLev];
};

// Sparse form of a key set: an open-addressing table of the set's bit indices (the
// positions the level bitmaps would hold, bitbase included), for key domains too
// large or too sparse for bitmaps.  Free slots hold kKeyEmpty; tab == null: the
// bitmap form.
constexpr unsigned long long kKeyEmpty = ~0ull;
struct KeyHash {
    unsigned long long* tab;
    unsigned long long mask;  // capacity - 1, capacity a power of two
};
// the two sets of a pass in the sparse form: new node keys, touched box positions
struct KeySets {
    KeyHash keys;
    KeyHash touched;
};

struct PointSrc {
    const char* base;
    long long n;
    int stride;
    int off;
};
// point colours (SetPoints' colour DataPtr): the uint32 RGBA8 at base + i*stride + off;
// base == nullptr: none
struct ClrSrc {
    const char* base;
    int stride;
    int off;
};

#ifdef __CUDACC__
// Positions of the four consecutive points i0 .. i0+3 (i0 a multiple of 4): three
// 16-byte loads when the buffer is packed float3 on a 16-byte boundary (the warp then
// reads 1,536 contiguous bytes per step), per-point loads otherwise and at the end of
// the buffer.  Entries past p.n are left unset.
__device__ __forceinline__ void load_pos4(const PointSrc& p, long long i0, float (&w)[4][3]) {
    if (p.stride == 12 && p.off == 0 && ((reinterpret_cast<uintptr_t>(p.base) & 15) == 0) && i0 + 4 <= p.n) {
        const float4* v = reinterpret_cast<const float4*>(p.base + i0 * 12);
        const float4 a = __ldg(v), b = __ldg(v + 1), c = __ldg(v + 2);
        w[0][0] = a.x; w[0][1] = a.y; w[0][2] = a.z;
        w[1][0] = a.w; w[1][1] = b.x; w[1][2] = b.y;
        w[2][0] = b.z; w[2][1] = b.w; w[2][2] = c.x;
        w[3][0] = c.y; w[3][1] = c.z; w[3][2] = c.w;
        return;
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
        if (i0 + u < p.n) load_pos(p.base, i0 + u, p.stride, p.off, w[u][0], w[u][1], w[u][2]);
}
#endif

// ---- scan.cu
size_t scan_tmp_bytes(long long n);
// exclusive scan of n u32 into out[0..n]; out[n] = total.  tmp: scan_tmp_bytes(n) bytes
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s);
// the same over the popcounts of n words (out[i] = set bits in words [0, i))
void scan_exclusive_popc(const uint32_t* words, uint32_t* out, long long n, void* tmp, cudaStream_t s);
// the same over n nodes' flags (mode 0: mFlags != 0, mode 1: mParent defined)
void scan_exclusive_node_flags(const Node* nodes, int mode, uint32_t* out, long long n, void* tmp, cudaStream_t s);
// ascending sort of n distinct u64 keys, each below 2^bits (LSD radix sort, 8-bit digits;
// one block for n <= kSortSmall); keys and alt hold n each; returns the one of the two
// that holds the result.  tmp: sort_tmp_bytes(n) bytes
constexpr long long kSortSmall = 4096;
size_t sort_tmp_bytes(long long n);
unsigned long long* sort_keys_u64(unsigned long long* keys, unsigned long long* alt, long long n, int bits, void* tmp,
                                  cudaStream_t s);

// ---- topology.cu
void launch_bbox(PointSrc p, float3 orig, int* out6, cudaStream_t s);
// ks.keys.tab set: keys go to the table instead of the bitmap (err bit 4: table full)
void launch_keys_pass1(const TreeView& t, PointSrc p, float3 orig, int depth, const KeyDomains& dom,
                       uint32_t* bitmap, const KeySets& ks, int* err, cudaStream_t s);
// touched: scratch bitmap with the layout of `bitmap`, cleared by the caller; dirs (or null):
// scratch of touch_dirs_words(dom) words for the direction-set form (boxes within one node
// of the home node), cleared by the launcher; home_hint: an estimate of the home leaf
// positions (the leaf count), which picks how the direction sets become touched bits
long long touch_dirs_words(const KeyDomains& dom);
void launch_keys_box(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 orig, float radius, int hi_mul,
                     int depth, int root_lo[3], int root_hi[3], const KeyDomains& dom, uint32_t* touched,
                     uint32_t* bitmap, int* markers, int* err, uint32_t* dirs, const KeySets& ks,
                     long long home_hint, cudaStream_t s);
// the key-count readback staged for one copy (k_stage_counts): prefix words of levels
// [0, nlev) and the total (words[nlev]), the error flag, the kept-leaf count and the point
// bounds (both optional)
struct CountStage {
    long long words[kMaxLev + 1];
    int nlev;
    const int* err;
    const unsigned long long* kept;
    const int* bbox;
};
void launch_stage_counts(const uint32_t* pscan, const CountStage& st, uint32_t* out, cudaStream_t s);
// sparse form: the occupied slots of h into out (any order), their number into *count
// (cleared by the caller)
void launch_hash_compact(const KeyHash& h, unsigned long long* out, unsigned int* count, cudaStream_t s);
// at[l] = keys of sorted[0..n) below dom.d[l].bitbase (l < depth), at[depth] = n
void launch_key_bounds(const unsigned long long* sorted, const unsigned int* n, const KeyDomains& dom, int depth,
                       unsigned int* at, cudaStream_t s);
// the nodes of level lev from sorted keys [first, first + count) at pool index base + rank
void launch_alloc_nodes_sorted(const unsigned long long* sorted, long long first, long long count, int lev,
                               int lgrange, const KeyDomain& d, long long base, Node* nodes, cudaStream_t s);
void launch_build_leaf_grid(const TreeView& t, long long n, int* cells, const int lo[3], const int dim[3],
                            int lgrange0, cudaStream_t s);
void launch_alloc_nodes(const uint32_t* bm, const uint32_t* prefix, long long word0, long long nwords,
                        int lev, int lgrange, const KeyDomain& d, long long base, Node* nodes, cudaStream_t s);
void launch_write_node(Node* dst, const Node& v, cudaStream_t s);
// tag: ncnt[lev+1]*res^3 ints, slot_of: count long longs (scratch)
void launch_link(const TreeView& t, int lev, long long count, int* tag, long long* slot_of, cudaStream_t s);
void launch_apply_markers(Node* leaves, long long n, const int* markers, cudaStream_t s);
void launch_delink_leaf(const TreeView& t, long long n, cudaStream_t s);
void launch_delink_upper(const TreeView& t, int lev, long long n, cudaStream_t s);
void launch_count_flags(const Node* nodes, long long n, unsigned long long* out, cudaStream_t s);
// *out += non-zero markers (cleared by the caller)
void launch_count_markers(const int* markers, long long n, unsigned long long* out, cudaStream_t s);
// incremental pass setup: markers (0 or the old flags), *err = 0, *kept = 0, and bbox6
// (when set) to the bounds' initial values
void launch_incr_setup(const Node* leaves, long long n, int* markers, int accum, int* err, unsigned long long* kept,
                       int* bbox6, cudaStream_t s);
void launch_leaf_bounds(const Node* leaves, long long n, int lgrange0, int* out6, cudaStream_t s);

// ---- atlas.cu
void launch_assign_slots(Node* leaves, long long n, const uint32_t* scan, int ax, int ay, AtlasNode* amap,
                         cudaStream_t s);
void launch_fill_u32(uint32_t* p, long long n, uint32_t v, cudaStream_t s);
// fill_only: after a fused-apron gather of this layout (bad: that gather's push check flag)
void launch_apron(const TreeView& t, const LeafGrid& lg, const AtlasNode* amap, int used, int ax, int ay, int esize,
                  const void* interior, void* apron, uint32_t boundbits, const int* fill_only_bad, cudaStream_t s);
void launch_export_bricks(const void* interior, const void* apron, int used, int esize, void* out,
                          cudaStream_t s);
// one brick layer (18 voxel slices) of the reference's atlas layout <-> interior + apron records
void launch_slab_pack(const void* interior, const void* apron, int esize, int ax, int ay, int bz, long long valid,
                      void* slab, cudaStream_t s);
void launch_slab_unpack(const void* slab, int esize, int ax, int ay, int bz, void* interior, void* apron,
                        cudaStream_t s);
// neighbour table (6 leaf indices per leaf), apron faces from it, smoothing pass
void launch_neighbors(const TreeView& t, const LeafGrid& lg, long long n, int d, int* table, cudaStream_t s);
void launch_apron_faces(const Node* leaves, const AtlasNode* amap, int used, int ax, int ay, const int* table,
                        int esize, void* interior, void* apron, cudaStream_t s);
void launch_smooth(const AtlasNode* amap, int used, float* interior, const float* apron, float p1, float p2,
                   cudaStream_t s);
// legacy InsertPoints (leaf of each point, rank, per-leaf counts), SortPoints and ScatterDensity
void launch_insert_points(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, int* pnode, uint32_t* pndx,
                          uint32_t* gcnt, cudaStream_t s);
void launch_sort_points(PointSrc p, float3 trans, const int* pnode, const uint32_t* pndx, const uint32_t* goff,
                        float* out3, cudaStream_t s);
void launch_scatter_density(const Node* leaves, long long nleaf, const uint32_t* goff, const float* pts3, float radius,
                            int expand, int res0, int ax, int ay, float* interior, float* apron, cudaStream_t s);
// deterministic FP64 channel sum: per-slot partials, then one fixed-order block (the
// grid size, blocks_per_sm x 152 at most, does not change the result); amap null: the
// slots below used are all assigned (as UpdateAtlas leaves them), no map is read
void launch_checksum_slots(const AtlasNode* amap, int used, int dtype, const void* interior, double* partials,
                           double* out, cudaStream_t s, int blocks_per_sm = 8);
void launch_fill_interior(const AtlasNode* amap, int used, int dtype, void* interior, float value,
                          cudaStream_t s);
// allocation-free checksum: scratch in a static device array (max slots noalloc_max_slots())
int noalloc_max_slots();
cudaError_t checksum_noalloc(const AtlasNode* amap, int used, int dtype, const void* interior, double* dev_out,
                             cudaStream_t s);

// ---- points.cu
void launch_linked_list(const Node* leaves, long long n, const uint32_t* scmap, int* linked, cudaStream_t s);
// 16-bit position quantisation of the FP16 subcell variants (InsertPointsSubcell_FP16,
// PT.cuh:154-216): q = trunc((w - mn) / rg * 65535), stored and gathered as q / 65535 * rg + mn
struct Quant {
    float3 mn, rg;
    int on;
};
// linked flags of the 27 bricks around every linked leaf (bit (dz+1)*9 + (dy+1)*3 + (dx+1))
// (bin_cnt, totals: when set, cleared too: bin_cnt[0, 64 n) and totals[0..1])
void launch_nb_mask(const TreeView& t, const LeafGrid& lg, long long n, uint32_t* nbmask, uint32_t* bin_cnt,
                    unsigned long long* totals, cudaStream_t s);
// nbmask (or null): from launch_nb_mask; only for R <= 11, where member ranges stay within those 27 bricks
// unroll: points per thread per step (1, 2 or 4)
void launch_bin_count(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q, const uint32_t* scmap,
                      const uint32_t* nbmask, uint32_t* bin_cnt, int* bin_of, uint32_t* rank_of,
                      unsigned long long* totals, int unroll, cudaStream_t s);
// sorted_clr (or null): the binned points' colours from clr, in the order of `sorted`
void launch_bin_scatter(PointSrc p, float3 trans, float R, Quant q, const int* bin_of, const uint32_t* rank_of,
                        const uint32_t* bin_off, float4* sorted, ClrSrc clr, uint32_t* sorted_clr, int unroll,
                        cudaStream_t s);

struct GatherParams {
    int mode;          // 0 density, 1 level set
    int accum;
    float rho;         // gather radius
    float R;           // subcell insert radius (membership)
    uint32_t tbits;    // static cutoff on squared distance (float bits)
    int dtype;         // storage type
    int ax, ay;        // atlas axis counts
    int lo_off, hi_off;  // home-bin offset range H - S (subcell units)
    int dense_min;     // bricks with more candidate points use the gather form
    float rcut;        // per-axis distance at or beyond which d^2 >= cutoff (conservative)
    // fused apron: when apron is non-null each brick also writes its boundary
    // voxels into the apron records of its 26 neighbours (see k_gather)
    void* apron;
    const int* apron_bad;  // set by the push check: the grid is not in the state the push assumes
    int min_blocks;        // resident blocks per SM the gather is compiled for (10 or 8)
    // launch order of the bricks: those with more than long_min candidate points first
    // (< 0: linked order); order: two counters, zero before the launch
    int long_min;
    unsigned* order;
};
// fused-apron precondition (one thread per leaf); *bad must be 0 before the launch
void launch_push_check(const TreeView& t, const LeafGrid& lg, const uint32_t* scmap, const AtlasNode* amap, int used,
                       int ax, int ay, long long n, int* bad, cudaStream_t s);
// offs: candidate home-bin offsets {dx, dy, dz, lb2} (H - S, subcell units), ascending lb2
// gtab: scratch of nbricks * 32 int4 (the per-brick setup, filled by the launcher's prep kernel)
void launch_gather(const TreeView& t, const LeafGrid& lg, const int* linked, long long nbricks, const uint32_t* scmap,
                   const uint32_t* bin_off, const float4* pts, const int4* offs, int noffs, const GatherParams& gp,
                   int4* gtab, void* interior, cudaStream_t s);
// materialized subcell lists (export and the fallback gather)
void launch_list_count(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q, const uint32_t* scmap,
                       uint32_t* cnt, cudaStream_t s);
// out_clr (or null): the list entries' colours from clr
void launch_list_fill(const TreeView& t, const LeafGrid& lg, PointSrc p, float3 trans, float R, Quant q, const uint32_t* scmap,
                      const uint32_t* off, uint32_t* cursor, float* out3, ClrSrc clr, uint32_t* out_clr, cudaStream_t s);
void launch_gather_lists(const TreeView& t, const int* linked, long long nbricks, const uint32_t* off,
                         const float* pts3, const GatherParams& gp, void* interior, cudaStream_t s);
// Colour averages of the gathers (T_UCHAR4 channel, 4096 uint32 per slot): every voxel of
// a subcell gets the mean of the subcell's member colours (plus its old colour with accum,
// else (0, 0, 0, 1)).  Binned form: gtab from the value gather of the same insert;
// member offsets H - S per axis in [olo, ohi].  List form: materialized lists + colours.
void launch_gather_colour(const int4* gtab, long long nbricks, const uint32_t* bin_off, const float4* pts,
                          const uint32_t* pclr, int olo, int ohi, int accum, uint32_t* out, cudaStream_t s);
void launch_gather_colour_lists(const TreeView& t, const int* linked, long long nbricks, const uint32_t* off,
                                const uint32_t* clr, int ax, int ay, int accum, uint32_t* out, cudaStream_t s);

}  // namespace gbvdb
