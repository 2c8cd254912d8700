// scan.cu -- device-wide exclusive prefix sum of u32 (replaces the reference's
// 3-level prefixSum/prefixFixup, cuda_gvdb_particles.cuh:856-902, VG.cpp:4760-4819).
// Reduce-then-scan: per-tile sums, a recursive scan of the tile sums, then a
// tile-local scan that adds the tile's offset.  Tiles of 4096 elements.
//
// Also the ascending sort of distinct u64 keys that the sparse key sets of
// RebuildTopology use in place of the reference's Thrust sort of brick keys
// (gvdb_cutils.cu:11-16): least-significant-digit radix sort, 8-bit digits, each
// pass a per-tile digit histogram, an exclusive scan of the histograms (digit-major,
// so every digit's tiles follow each other), and a stable scatter.
#include "kernels.h"

namespace gbvdb {

thread_local long long tl_kernels = 0;

namespace {
constexpr int kThreads = 1024;
constexpr int kItems = 4;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Element i of a scan's input: kind 0 the u32 value, 1 the popcount of a bitmap word,
// 2 whether node i is flagged (mFlags != 0), 3 whether node i is linked (mParent set)
struct ScanIn {
    const uint32_t* words;
    const Node* nodes;
};
template <int kKind>
__device__ __forceinline__ uint32_t elem(const ScanIn& in, long long i) {
    if (kKind == 0) return in.words[i];
    if (kKind == 1) return (uint32_t)__popc(in.words[i]);
    if (kKind == 2) return in.nodes[i].flags ? 1u : 0u;
    return in.nodes[i].parent != kUndef64 ? 1u : 0u;
}

template <int kKind>
__global__ void k_tile_sums(ScanIn in, long long n, uint32_t* __restrict__ sums) {
    long long base = (long long)blockIdx.x * kTile;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + (long long)k * kThreads + threadIdx.x;
        if (i < n) s += elem<kKind>(in, i);
    }
    // block reduce
    __shared__ uint32_t red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t t = red[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = t;
    }
}

// each thread owns kItems consecutive elements
template <int kKind>
__global__ void k_tile_scan(ScanIn in, long long n, const uint32_t* __restrict__ tile_off, uint32_t* __restrict__ out) {
    __shared__ uint32_t warp_sums[32];
    long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + k;
        v[k] = (i < n) ? elem<kKind>(in, i) : 0u;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = warp_incl_scan(s);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        uint32_t wi = warp_incl_scan(w);
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = (tile_off ? tile_off[blockIdx.x] : 0u) + warp_sums[warp] + inc - s;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    // out[n] = total, written by the thread owning the last element
    if (base <= n - 1 && n - 1 < base + kItems) out[n] = run;
}

// ---- radix sort of u64 keys
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;
constexpr int kSortWarps = kSortThreads / 32;

// hist[digit * tiles + tile] = keys of the tile with that digit
__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const unsigned long long* __restrict__ keys, long long n,
                                                             int shift, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortRounds; r++) {
        const long long i = base + (long long)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: the tile's keys are taken in index order, a block-wide
// round of 256 at a time; within a round a key's place among the keys of its digit is
// its rank among its warp's peers (match_any) plus the counts of the lower warps.
__global__ void __launch_bounds__(kSortThreads) k_digit_scatter(const unsigned long long* __restrict__ in,
                                                                unsigned long long* __restrict__ out, long long n,
                                                                int shift, const uint32_t* __restrict__ offs) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[kSortWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    run[threadIdx.x] = offs[(long long)threadIdx.x * gridDim.x + blockIdx.x];
    for (int w = 0; w < kSortWarps; w++) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortRounds; r++) {
        const long long i = base + (long long)r * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const unsigned long long k = valid ? in[i] : 0ull;
        const unsigned d = valid ? ((unsigned)(k >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned pos = run[d] + rank;
            for (int w = 0; w < warp; w++) pos += wcnt[w][d];
            out[pos] = k;
        }
        __syncthreads();
        uint32_t tot = 0;
        for (int w = 0; w < kSortWarps; w++) {
            tot += wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = 0;
        }
        run[threadIdx.x] += tot;
        __syncthreads();
    }
}

// up to kSortSmall keys: bitonic sort in shared memory, padded with kKeyEmpty (above
// every key)
__global__ void __launch_bounds__(1024) k_sort_small(unsigned long long* keys, int n) {
    __shared__ unsigned long long v[kSortSmall];
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = threadIdx.x; i < m; i += blockDim.x) v[i] = i < n ? keys[i] : kKeyEmpty;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = v[i], b = v[l];
                    if ((a > b) == ((i & k) == 0)) {
                        v[i] = b;
                        v[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = v[i];
}
}  // namespace

static long long ntiles(long long n) { return (n + kTile - 1) / kTile; }

size_t scan_tmp_bytes(long long n) {
    size_t bytes = 0;
    long long m = n;
    while (m > kTile) {
        long long t = ntiles(m);
        bytes += (size_t)(2 * t + 1) * sizeof(uint32_t) + 256;
        m = t;
    }
    return bytes + 256;
}

template <int kKind>
static void scan_exclusive(ScanIn in, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
        return;
    }
    long long t = ntiles(n);
    if (t == 1) {
        k_tile_scan<kKind><<<counted(1), kThreads, 0, s>>>(in, n, nullptr, out);
        return;
    }
    uint32_t* sums = reinterpret_cast<uint32_t*>(tmp);
    uint32_t* offs = sums + t;
    char* rest = reinterpret_cast<char*>(offs + t + 1);
    rest = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(rest) + 255) & ~uintptr_t(255));
    k_tile_sums<kKind><<<counted((unsigned)t), kThreads, 0, s>>>(in, n, sums);
    scan_exclusive<0>(ScanIn{sums, nullptr}, offs, t, rest, s);
    k_tile_scan<kKind><<<counted((unsigned)t), kThreads, 0, s>>>(in, n, offs, out);
}

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    scan_exclusive<0>(ScanIn{in, nullptr}, out, n, tmp, s);
}

void scan_exclusive_popc(const uint32_t* words, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    scan_exclusive<1>(ScanIn{words, nullptr}, out, n, tmp, s);
}

void scan_exclusive_node_flags(const Node* nodes, int mode, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    if (mode == 0) scan_exclusive<2>(ScanIn{nullptr, nodes}, out, n, tmp, s);
    else scan_exclusive<3>(ScanIn{nullptr, nodes}, out, n, tmp, s);
}

static long long sort_tiles(long long n) { return (n + kSortTile - 1) / kSortTile; }

size_t sort_tmp_bytes(long long n) {
    if (n <= kSortSmall) return 256;
    const long long h = 256 * sort_tiles(n);
    return (size_t)(2 * h + 1) * sizeof(uint32_t) + 256 + scan_tmp_bytes(h);
}

unsigned long long* sort_keys_u64(unsigned long long* keys, unsigned long long* alt, long long n, int bits, void* tmp,
                                  cudaStream_t s) {
    if (n <= 1) return keys;
    if (n <= kSortSmall) {
        k_sort_small<<<counted(1), 1024, 0, s>>>(keys, (int)n);
        return keys;
    }
    const long long t = sort_tiles(n), h = 256 * t;
    uint32_t* hist = reinterpret_cast<uint32_t*>(tmp);
    uint32_t* offs = hist + h;
    char* rest = reinterpret_cast<char*>(offs + h + 1);
    rest = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(rest) + 255) & ~uintptr_t(255));
    unsigned long long *src = keys, *dst = alt;
    for (int shift = 0; shift < bits; shift += 8) {
        k_digit_hist<<<counted((unsigned)t), kSortThreads, 0, s>>>(src, n, shift, hist);
        scan_exclusive_u32(hist, offs, h, rest, s);
        k_digit_scatter<<<counted((unsigned)t), kSortThreads, 0, s>>>(src, dst, n, shift, offs);
        unsigned long long* x = src;
        src = dst;
        dst = x;
    }
    return src;
}

}  // namespace gbvdb
