// scan.cu -- device-wide exclusive prefix sum of u32 (replaces the reference's
// 3-level prefixSum/prefixFixup, cuda_gvdb_particles.cuh:856-902, VG.cpp:4760-4819).
// Reduce-then-scan: per-tile sums, a recursive scan of the tile sums, then a
// tile-local scan that adds the tile's offset.  Tiles of 4096 elements.
#include "kernels.h"

namespace gbvdb {

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

__global__ void k_tile_sums(const uint32_t* __restrict__ in, long long n, uint32_t* __restrict__ sums) {
    long long base = (long long)blockIdx.x * kTile;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + (long long)k * kThreads + threadIdx.x;
        if (i < n) s += in[i];
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
__global__ void k_tile_scan(const uint32_t* __restrict__ in, long long n, const uint32_t* __restrict__ tile_off,
                            uint32_t* __restrict__ out) {
    __shared__ uint32_t warp_sums[32];
    long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        long long i = base + k;
        v[k] = (i < n) ? in[i] : 0u;
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

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
        return;
    }
    long long t = ntiles(n);
    if (t == 1) {
        k_tile_scan<<<1, kThreads, 0, s>>>(in, n, nullptr, out);
        return;
    }
    uint32_t* sums = reinterpret_cast<uint32_t*>(tmp);
    uint32_t* offs = sums + t;
    char* rest = reinterpret_cast<char*>(offs + t + 1);
    rest = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(rest) + 255) & ~uintptr_t(255));
    k_tile_sums<<<(unsigned)t, kThreads, 0, s>>>(in, n, sums);
    scan_exclusive_u32(sums, offs, t, rest, s);
    k_tile_scan<<<(unsigned)t, kThreads, 0, s>>>(in, n, offs, out);
}

}  // namespace gbvdb
