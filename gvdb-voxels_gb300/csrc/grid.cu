// grid.cu -- host orchestration of the point-driven path and the C ABI (include/gbvdb.h).
//
// One gbvdb_grid is the state a nvdb::VolumeGVDB object holds for this path
// (source/gvdb_library/src/gvdb_volume_gvdb.h:319-901): grid configuration, node
// pools, the atlas channels and the subcell binning of the last insert.  All
// device work is issued on the grid's stream; the host reads back only the few
// counters it needs to size allocations (bounding box, unique key counts, used
// leaf count, subcell-list length), each as one small pinned copy.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <dlfcn.h>

#include <cstdlib>
#include <memory>

#include "gbvdb.h"
#include "host_topology.h"
#include "kernels.h"

using namespace gbvdb;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

struct Channel {
    bool used = false;
    int dtype = GBVDB_T_FLOAT;
    int apron = 1;
    int esize = 4;
    DevBuf interior, apron_buf;
    long long cap_slots = 0;
};

struct StatusError {
    gbvdb_status st;
    std::string msg;
};

uint16_t f2h_bits(float f) {  // round to nearest even, float -> IEEE half
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    int32_t exp = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
    uint32_t mant = x & 0x7FFFFFu;
    if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0));
    if (exp >= 31) return (uint16_t)(sign | 0x7C00u);
    if (exp <= 0) {
        if (exp < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - exp);
        uint32_t h = mant >> shift;
        uint32_t rem = mant & ((1u << shift) - 1), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1))) h++;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)exp << 10) | (mant >> 13);
    uint32_t rem = mant & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1))) h++;
    return (uint16_t)(sign | h);
}
// ------------------------------------------------------------- tuning table
// Per point-count bucket: the gather's dense-form threshold, the gather's resident
// blocks per SM, the candidate count from which its bricks are launched first and
// the binning passes' points per thread, chosen by a tuning run
// (gvdb-voxels_gb300/tune.py) and read from JSON at the first grid creation:
//   {"buckets": [{"max_points": 100000, "dense_min": 2048, "gather_blocks": 10,
//                 "gather_long_min": 2048, "bin_unroll": 2, "scatter_unroll": 4}, ...]}
// from $GBVDB_TUNE_TABLE, else tune_table.json beside libgbvdb.so.  An insert or gather
// of n points takes the first bucket with max_points >= n (the last one beyond).
// the gather launches bricks with more candidate points than this first (tuning table
// field gather_long_min; -1 keeps the linked order)
constexpr int kGatherLongMin = 2048;
struct TuneEntry {
    long long max_points = 0;
    int dense_min = 2048, gather_blocks = 10, bin_unroll = 2, scatter_unroll = 4;
    int gather_long_min = kGatherLongMin;
};
struct TuneTable {
    std::vector<TuneEntry> b;
    std::string source;
};

bool json_int(const std::string& obj, const char* key, long long* out) {
    const std::string k = std::string("\"") + key + "\"";
    size_t p = obj.find(k);
    if (p == std::string::npos) return false;
    p = obj.find(':', p + k.size());
    if (p == std::string::npos) return false;
    char* end = nullptr;
    const long long v = std::strtoll(obj.c_str() + p + 1, &end, 10);
    if (end == obj.c_str() + p + 1) return false;
    *out = v;
    return true;
}

TuneTable load_tune_table() {
    TuneTable t;
    std::string path;
    if (const char* e = std::getenv("GBVDB_TUNE_TABLE")) {
        path = e;
    } else {
        Dl_info info;
        if (dladdr((void*)&load_tune_table, &info) && info.dli_fname) {
            path = info.dli_fname;
            const size_t sl = path.find_last_of('/');
            path = (sl == std::string::npos ? std::string(".") : path.substr(0, sl)) + "/tune_table.json";
        }
    }
    FILE* f = path.empty() ? nullptr : std::fopen(path.c_str(), "rb");
    if (!f) return t;
    std::string txt;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) txt.append(buf, n);
    std::fclose(f);
    size_t p = txt.find("\"buckets\"");
    while (p != std::string::npos) {
        const size_t a = txt.find('{', p), z = a == std::string::npos ? a : txt.find('}', a);
        if (a == std::string::npos || z == std::string::npos) break;
        const std::string obj = txt.substr(a, z - a + 1);
        TuneEntry e;
        long long v;
        if (!json_int(obj, "max_points", &v)) break;
        e.max_points = v;
        if (json_int(obj, "dense_min", &v) && v >= 0) e.dense_min = (int)std::min<long long>(v, 1ll << 31);
        if (json_int(obj, "gather_blocks", &v)) e.gather_blocks = v == 8 ? 8 : 10;
        if (json_int(obj, "gather_long_min", &v)) e.gather_long_min = (int)std::max(-1ll, std::min(v, 1ll << 30));
        if (json_int(obj, "bin_unroll", &v)) e.bin_unroll = (v == 1 || v == 4) ? (int)v : 2;
        if (json_int(obj, "scatter_unroll", &v)) e.scatter_unroll = (v == 2 || v == 8) ? (int)v : 4;
        t.b.push_back(e);
        p = z + 1;
    }
    std::sort(t.b.begin(), t.b.end(), [](const TuneEntry& x, const TuneEntry& y) { return x.max_points < y.max_points; });
    if (!t.b.empty()) t.source = path;
    return t;
}

const TuneTable& tune_table() {
    static const TuneTable t = load_tune_table();
    return t;
}

uint16_t f2bf_bits(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    if ((x & 0x7F800000u) == 0x7F800000u && (x & 0x7FFFFFu)) return (uint16_t)((x >> 16) | 0x40);
    uint32_t r = x + 0x7FFFu + ((x >> 16) & 1u);
    return (uint16_t)(r >> 16);
}

}  // namespace

struct gbvdb_grid_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string err;

    // configuration (Configure, VG.cpp:2380-2434)
    bool configured = false;
    int levs = 0;
    int log2dim[kMaxLev] = {0};
    int res[kMaxLev] = {0};
    long long range[kMaxLev] = {0};
    int lgrange[kMaxLev] = {0};

    // pools
    DevBuf nodes[kMaxLev], clist[kMaxLev];
    long long ncnt[kMaxLev] = {0}, nused[kMaxLev] = {0};
    bool nused0_stale = false;  // nused[0] awaits a count of the flagged leaves
    // 8 bytes that the next key-count readback brings back with the counts (null: none)
    const void* rb_extra = nullptr;
    unsigned long long rb_extra_val = 0;
    // Speculative incremental passes: the last pass's key domains (bitmap form) and, for
    // the pass that runs on the next frame's points before their bounds are known, the
    // device bounds brought back with its counts and whether its keys all fell inside
    KeyDomains last_kd{};
    int last_kd_depth = -1;
    bool spec_pass = false, spec_failed = false;
    const void* rb_bbox = nullptr;
    int rb_bbox_val[6] = {0};
    int rebuild_topo = 1;
    int curr_depth = -1;
    int last_depth = 0;
    int root_lev = -1;
    int root_pos[3] = {0, 0, 0};
    float posmin[3] = {0, 0, 0}, posmax[3] = {0, 0, 0};
    int bounds[6] = {0, 0, 0, 0, 0, 0};  // ComputeBounds of the last FinishTopology (mObjMin, mObjMax)
    bool bounds_valid = false;

    // points (SetPoints, VG.cpp:4900-4908)
    PointSrc pts{nullptr, 0, 12, 0};
    const void* vel = nullptr;
    ClrSrc clr{nullptr, 4, 0};  // point colours (RGBA8 uint per point), base null: none

    // atlas
    int def_ax = 16, def_ay = 16, def_az = 1;  // SetChannelDefault(16,16,1), VG.cpp:2348
    int ax = 0, ay = 0, az = 0;
    int atlas_last = 0;
    Channel ch[8];
    DevBuf amap;
    long long amap_slots = 0;

    // subcells of the last InsertPointsSubcell
    bool sc_valid = false;
    float sc_R = 0.f;
    float3 sc_trans{0, 0, 0};
    PointSrc sc_pts{nullptr, 0, 12, 0};
    long long sc_nleaf = 0, sc_nbricks = 0, sc_len = 0, sc_orphans = 0;
    bool lists_valid = false;
    Quant sc_quant{};  // position quantisation of the last insert (FP16 variant)
    ClrSrc sc_clr{nullptr, 4, 0};  // colours the last insert carried (base null: none)
    DevBuf scmap, linked, bin_cnt, bin_off, bin_of, rank_of, sorted, sorted_clr;
    DevBuf list_cnt, list_off, list_pts, list_clr;
    DevBuf offs_buf;
    // dense leaf lookup over the brick box of every leaf created since the last Clear
    DevBuf lgrid;
    LeafGrid lgv{nullptr, {0, 0, 0}, {0, 0, 0}, 4};
    int lgdom_lo[3] = {0, 0, 0}, lgdom_hi[3] = {0, 0, 0};
    bool lgdom_init = false;
    int noffs = 0;
    float offs_R = -1.f;
    uint32_t offs_T = 0;

    // scratch
    DevBuf bitmap, pscan, scan_tmp, markers, flags_scan, misc, xfer, link_tag, link_slot;
    long long touched_off = 0;  // the touched bitmap follows the key bitmap in one buffer (words)
    DevBuf touch_dirs;          // per home leaf position: the directions its points' boxes cover
    bool touch_dirs_on = true;  // GBVDB_TUNE_TOUCH_DIRS
    // sparse key sets (hash tables of key bits) for domains too large or too sparse for
    // the bitmaps: the new-key and touched tables, the sorted keys and the sort's
    // scratch, the compaction counter and level bounds (kmeta)
    DevBuf khash, thash, ksorted, kalt, ksort_tmp, kmeta;
    long long khash_cap = 0, thash_cap = 0;
    int keyset_mode = 0;                         // GBVDB_TUNE_KEYSET
    bool hashed = false;                         // the key sets of the current pass
    unsigned long long* sorted_keys = nullptr;   // sparse form: the counted pass's keys, ascending
    long long n_hashed_passes = 0;
    unsigned char* pinned = nullptr;

    // ActivateSpace / RebuildTopologyCPU: host copies of the pools (fetched from the
    // device at the first activation) that the next call reading the topology commits
    std::unique_ptr<HostTopology> host;
    bool host_dirty = false;

    // legacy InsertPoints: leaf and rank per point, points grouped by leaf
    DevBuf pnode, pndx, gcnt, goff, psort;
    long long ins_n = -1, ins_nleaf = -1;

    // neighbour table of UpdateNeighbors (6 leaf indices per leaf) and the leaf count it covers
    DevBuf nbr_table;
    long long nbr_count = -1;
    DevBuf csum_part;  // per-slot partial sums of gbvdb_checksum_device
    // Side stream of gbvdb_checksum_overlap: the checksum of a frame reads the channel
    // interiors (not the atlas map) while the grid's stream goes on with the next frame's
    // topology, atlas and binning; every entry point that writes or reallocates the
    // interiors (all but the topology, atlas, binning and accessor calls; UpdateAtlas when
    // the atlas grows) first makes the grid's stream wait for it on the device (join_side).
    cudaStream_t side = nullptr;
    cudaEvent_t side_start = nullptr, side_done = nullptr;
    // a readback's copies are done: the host waits on this instead of the whole stream
    // when independent work is queued behind them
    cudaEvent_t rb_ev = nullptr;
    bool side_pending = false;
    void join_side() {
        if (!side_pending) return;
        cudaStreamWaitEvent(stream, side_done, 0);
        side_pending = false;
    }
    DevBuf push_bad;   // fused apron: the push check's flag (one int)
    DevBuf nbmask;     // linked flags of the 27 bricks around each leaf (InsertPointsSubcell)
    DevBuf gtab;       // per-brick gather setup (neighbour ranks and bin ranges, origin, slot)

    // tuning
    bool table_on = true;  // GBVDB_TUNE_TABLE: settings from the tuning table when one is loaded
    const TuneEntry* tune_entry(long long n) const {
        const TuneTable& t = tune_table();
        if (!table_on || t.b.empty()) return nullptr;
        for (const TuneEntry& e : t.b)
            if (n <= e.max_points) return &e;
        return &t.b.back();
    }
    // explicit settings (set_tuning) win over the table; -1: table or built-in default
    int bin_unroll_set = -1, scatter_unroll_set = -1, gather_blocks_set = -1;
    int gather_long_min_set = 0;  // GBVDB_TUNE_GATHER_LONG_MIN: 0 table / default, -1 linked order
    int bin_unroll(long long n) const {
        const TuneEntry* e = tune_entry(n);
        return bin_unroll_set > 0 ? bin_unroll_set : (e ? e->bin_unroll : 2);
    }
    int scatter_unroll(long long n) const {
        const TuneEntry* e = tune_entry(n);
        return scatter_unroll_set > 0 ? scatter_unroll_set : (e ? e->scatter_unroll : 4);
    }
    int gather_blocks(long long n) const {
        const TuneEntry* e = tune_entry(n);
        return gather_blocks_set > 0 ? gather_blocks_set : (e ? e->gather_blocks : 10);
    }
    int gather_long_min(long long n) const {
        if (gather_long_min_set != 0) return gather_long_min_set;
        const TuneEntry* e = tune_entry(n);
        return e ? e->gather_long_min : kGatherLongMin;
    }
    int dense_min = 2048;
    // Dense-form threshold autotuner (on until GBVDB_TUNE_DENSE_MIN is set): the
    // gathers of a workload try each candidate once, timed with events on the
    // grid's stream, and the faster one is kept; a linked-brick count that moves
    // by more than 2x starts a new round.  Both forms give the same bits, so only
    // the time depends on the choice.  Which value wins depends on how the points
    // are spread (measured: a thick shell wants 2048, the fluid frame and the
    // surface workload 4096).
    static constexpr int kTuneN = 2;
    static constexpr int kTuneCand[kTuneN] = {2048, 4096};
    bool tune_auto = true;
    bool tune_pending = false;
    int tune_step = kTuneN;  // candidates measured in the current round (kTuneN: none running)
    long long tune_bricks = -1;
    cudaEvent_t tune_ev[2 * kTuneN] = {};

    // the threshold for this gather, and the candidate slot it measures (-1: none)
    int tune_pick(long long bricks, int* slot) {
        *slot = -1;
        if (!tune_auto) return dense_min;
        if (tune_pending) {  // the last round's timings, once its events have completed
            if (cudaEventQuery(tune_ev[2 * kTuneN - 1]) == cudaSuccess) {
                float best = 0.0f;
                int bi = -1;
                for (int i = 0; i < kTuneN; i++) {
                    float ms = 0.0f;
                    if (cudaEventElapsedTime(&ms, tune_ev[2 * i], tune_ev[2 * i + 1]) != cudaSuccess) { bi = -1; break; }
                    if (bi < 0 || ms < best) { best = ms; bi = i; }
                }
                cudaGetLastError();
                if (bi >= 0) dense_min = kTuneCand[bi];
                tune_pending = false;
            } else {
                cudaGetLastError();  // not ready yet (cudaErrorNotReady): decide at a later gather
            }
        }
        if (!tune_pending && tune_step >= kTuneN && (tune_bricks < 0 || bricks > 2 * tune_bricks || 2 * bricks < tune_bricks)) {
            tune_step = 0;  // a new workload: measure the candidates again
            tune_bricks = bricks;
        }
        if (tune_step < kTuneN && !tune_pending) {
            *slot = tune_step;
            return kTuneCand[tune_step];
        }
        return dense_min;
    }

    // Fused apron: a gather also writes each brick's boundary voxels into its
    // neighbours' apron records, and the next UpdateApron of that channel only
    // fills the faces whose neighbour is missing.  layout_ver changes with every
    // topology, atlas or channel change; a channel's pushed_ver is the layout_ver
    // of the gather that pushed (0: none, or the interior was written since).
    // Handing out raw atlas pointers turns the fused form off for the grid.
    bool fused_apron = true;
    unsigned long long layout_ver = 1;
    unsigned long long pushed_ver[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    void layout_changed() { layout_ver++; }
    void interior_written(int c) { if (c >= 0 && c < 8) pushed_ver[c] = 0; }

    // profiling
    bool profile = false;
    std::vector<double> stage_ms;

    // ---------------------------------------------------------------- helpers
    void check(cudaError_t e, const char* what) {
        if (e != cudaSuccess) throw StatusError{GBVDB_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e)};
    }
    long long n_launch = 0, n_readback = 0;  // n_launch: kernels (tl_kernels, per entry point)
    void check_launch(const char* what) { check(cudaGetLastError(), what); }
    void sync() { check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }

    void grow(DevBuf& b, size_t bytes, size_t preserve = 0) {
        if (bytes <= b.cap) return;
        size_t cap = std::max(bytes, b.cap + b.cap / 2);
        cap = (cap + 255) & ~size_t(255);
        void* np = nullptr;
        cudaError_t e = cudaMallocAsync(&np, cap, stream);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw StatusError{GBVDB_OUT_OF_MEMORY, "device allocation of " + std::to_string(cap) + " bytes failed"};
        }
        if (b.p) {
            if (preserve) check(cudaMemcpyAsync(np, b.p, std::min(preserve, b.cap), cudaMemcpyDeviceToDevice, stream),
                                "preserve copy");
            check(cudaFreeAsync(b.p, stream), "cudaFreeAsync");
        }
        b.p = np;
        b.cap = cap;
    }
    void release(DevBuf& b) {
        if (b.p) cudaFreeAsync(b.p, stream);
        b.p = nullptr;
        b.cap = 0;
    }
    template <typename T>
    T* ptr(DevBuf& b) { return reinterpret_cast<T*>(b.p); }

    void readback(void* host, const void* dev, size_t bytes) {
        n_readback++;
        check(cudaMemcpyAsync(pinned, dev, bytes, cudaMemcpyDeviceToHost, stream), "readback");
        sync();
        memcpy(host, pinned, bytes);
    }
    void upload(void* dev, const void* host, size_t bytes) {
        // staged through a device-side copy of pageable memory: small control data only
        check(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, stream), "upload");
    }

    int top_lev() const {
        int t = 1;
        for (int n = levs - 1; n >= 0; n--)
            if (ncnt[n] == 1) t = n;
        return t;
    }
    TreeView view() {
        TreeView t{};
        t.levs = levs;
        t.top_lev = top_lev();
        for (int l = 0; l < kMaxLev; l++) {
            t.res[l] = l < levs ? res[l] : 1;
            t.lgres[l] = l < levs ? log2dim[l] : 0;
            t.lgrange[l] = l < levs ? lgrange[l] : 0;
            t.ncnt[l] = ncnt[l];
            t.nodes[l] = ptr<Node>(nodes[l]);
            t.clist[l] = ptr<unsigned long long>(clist[l]);
        }
        return t;
    }
    long long cl_len(int lev) const { return lev >= 1 ? (1ll << (3 * log2dim[lev])) : 0; }

    void ensure_pool(int lev, long long need) {
        grow(nodes[lev], (size_t)need * sizeof(Node), (size_t)ncnt[lev] * sizeof(Node));
        if (lev >= 1)
            grow(clist[lev], (size_t)(need * cl_len(lev)) * 8, (size_t)(ncnt[lev] * cl_len(lev)) * 8);
    }

    void clear_topology() {  // Clear (VG.cpp:2487-2503)
        layout_changed();
        last_kd_depth = -1;
        for (int l = 0; l < kMaxLev; l++) { ncnt[l] = 0; nused[l] = 0; }
        nused0_stale = false;
        nbr_count = -1;
        ins_n = -1;
        lgdom_init = false;
        lgv.cells = nullptr;
        atlas_last = 0;
        rebuild_topo = 1;
        sc_valid = false;
        lists_valid = false;
    }

    // ---------------------------------------------------------- stage timing
    cudaEvent_t ev[64];
    int nev = 0;
    void mark() {
        if (!profile || nev >= 64) return;
        cudaEventRecord(ev[nev++], stream);
    }
    void stage_begin() {
        nev = 0;
        mark();
    }
    void stage_end() {
        if (!profile) return;
        sync();
        stage_ms.clear();
        for (int i = 1; i < nev; i++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[i - 1], ev[i]);
            stage_ms.push_back(ms);
        }
    }

    // ------------------------------------------- host topology (ActivateSpace)
    // PoolFetchAll: host copies of the device pools for ActivateSpace to extend
    void host_begin() {
        if (host) return;
        if (!configured) throw StatusError{GBVDB_INVALID_ARG, "Configure was not called"};
        refresh_nused0();
        sync();
        host.reset(new HostTopology());
        host->configure(levs, log2dim, range);
        for (int l = 0; l < levs; l++) {
            host->nodes[l].resize((size_t)ncnt[l]);
            if (ncnt[l])
                check(cudaMemcpy(host->nodes[l].data(), nodes[l].p, (size_t)ncnt[l] * sizeof(Node), cudaMemcpyDeviceToHost),
                      "fetch nodes");
            host->used[l] = (size_t)nused[l];
            size_t lists = 0;
            for (const Node& n : host->nodes[l])
                if (n.childlist != kUndefL) lists = std::max(lists, (size_t)(n.childlist >> 16) + 1);
            host->lists_used[l] = lists;
            host->clist[l].resize(lists * (size_t)cl_len(l));
            if (!host->clist[l].empty())
                check(cudaMemcpy(host->clist[l].data(), clist[l].p, host->clist[l].size() * 8, cudaMemcpyDeviceToHost),
                      "fetch child lists");
        }
        host->root = (root_lev >= 0 && ncnt[root_lev] > 0) ? elem(0, root_lev, 0) : HostTopology::kNone;
    }

    // PoolCommitAll of the host pools: they replace the device pools
    void host_commit() {
        if (!host_dirty) return;
        host_dirty = false;
        std::unique_ptr<HostTopology> h = std::move(host);
        layout_changed();
        const long long nl = (long long)h->nodes[0].size();
        for (int l = 0; l < levs; l++) {
            const long long n = (long long)h->nodes[l].size();
            grow(nodes[l], (size_t)std::max(n, 1ll) * sizeof(Node));
            if (l >= 1) grow(clist[l], (size_t)std::max(n, 1ll) * (size_t)cl_len(l) * 8);
            if (n) check(cudaMemcpyAsync(nodes[l].p, h->nodes[l].data(), (size_t)n * sizeof(Node), cudaMemcpyHostToDevice,
                                         stream), "commit nodes");
            if (!h->clist[l].empty())
                check(cudaMemcpyAsync(clist[l].p, h->clist[l].data(), h->clist[l].size() * 8, cudaMemcpyHostToDevice,
                                      stream), "commit child lists");
            if (l >= 1 && (long long)h->lists_used[l] < n)  // lists not taken yet read as empty
                check(cudaMemsetAsync(ptr<unsigned long long>(clist[l]) + h->clist[l].size(), 0xFF,
                                      ((size_t)n * (size_t)cl_len(l) - h->clist[l].size()) * 8, stream),
                      "commit child lists");
            ncnt[l] = n;
            nused[l] = (long long)h->used[l];
        }
        sync();  // the host copies are released below
        nused0_stale = false;
        root_lev = -1;
        if (h->root != HostTopology::kNone) {
            root_lev = (int)((h->root >> 8) & 0xFF);
            const Node& r = h->nodes[root_lev][(size_t)(h->root >> 16)];
            for (int a = 0; a < 3; a++) root_pos[a] = r.pos[a];
        }
        last_depth = std::max(root_lev, 0);
        // the dense leaf lookup covers every leaf's brick
        lgdom_init = false;
        for (long long i = 0; i < nl; i++) {
            const Node& n = h->nodes[0][(size_t)i];
            for (int a = 0; a < 3; a++) {
                const int c = n.pos[a] >> lgrange[0];
                lgdom_lo[a] = lgdom_init ? std::min(lgdom_lo[a], c) : c;
                lgdom_hi[a] = lgdom_init ? std::max(lgdom_hi[a], c) : c;
            }
            lgdom_init = true;
        }
        build_leaf_grid();
        nbr_count = -1;
        ins_n = -1;
        sc_valid = false;
        lists_valid = false;
        rebuild_topo = 1;  // a later RebuildTopology starts from an empty grid
    }

    // ------------------------------------------------------------ topology
    int determine_depth(int out_root[3]) const {  // DetermineDepth (VG.cpp:821-837)
        int pmin[3], pmax[3];
        for (int a = 0; a < 3; a++) { pmin[a] = (int)posmin[a]; pmax[a] = (int)posmax[a]; }
        for (int lev = 0; lev < levs; lev++) {
            long long rg = range[lev];
            bool same = true;
            for (int a = 0; a < 3; a++)
                if (pmin[a] / rg != pmax[a] / rg) same = false;
            if (same) {
                for (int a = 0; a < 3; a++) out_root[a] = (int)((pmin[a] / rg) * rg);
                return lev;
            }
        }
        return -1;
    }

    // GetBoundingBox (VG.cpp:5404-5467): the min / max of the points into d6 (misc)
    int* launch_compute_bbox(long long n, float3 orig) {
        int init[6];
        for (int a = 0; a < 3; a++) { init[a] = 0x7F800000; init[3 + a] = (int)(0xFF800000u ^ 0x7FFFFFFFu); }
        grow(misc, 256);
        int* d6 = ptr<int>(misc);
        memcpy(pinned + 256, init, sizeof(init));
        check(cudaMemcpyAsync(d6, pinned + 256, sizeof(init), cudaMemcpyHostToDevice, stream), "bbox init");
        PointSrc p = pts;
        p.n = n;
        launch_bbox(p, orig, d6, stream);
        check_launch("bbox");
        return d6;
    }
    // mPosMin = max(0, min - 1), mPosMax = max(0, max + 2)
    static void bbox_bounds(const int out[6], float pmin[3], float pmax[3]) {
        for (int a = 0; a < 3; a++) {
            float mn = o2f(out[a]), mx = o2f(out[3 + a]);
            float lo = mn - 1.0f, hi = mx + 2.0f;
            pmin[a] = 0 > lo ? 0 : lo;
            pmax[a] = 0 > hi ? 0 : hi;
        }
    }
    void compute_bbox(long long n, float3 orig) {
        int* d6 = launch_compute_bbox(n, orig);
        int out[6];
        readback(out, d6, sizeof(out));
        bbox_bounds(out, posmin, posmax);
    }

    // key domains of levels [0, depth): node coordinates that any pass can emit,
    // clipped to the root node's extent
    KeyDomains domains(int depth, float margin, const int rpos[3], int rlev, long long* total_bits) {
        KeyDomains kd{};
        long long bit = 0;
        long long rg_root = range[rlev];
        for (int l = 0; l < depth; l++) {
            KeyDomain& d = kd.d[l];
            for (int a = 0; a < 3; a++) {
                double lo = std::max(0.0, (double)posmin[a] - margin);
                double hi = (double)posmax[a] + margin;
                long long clo = (long long)std::floor(lo) >> lgrange[l];
                long long chi = (long long)std::floor(hi) >> lgrange[l];
                long long rlo = (long long)rpos[a] >> lgrange[l];
                long long rhi = ((long long)rpos[a] + rg_root - 1) >> lgrange[l];
                clo = std::max(clo, rlo);
                chi = std::min(chi, rhi);
                if (chi < clo) chi = clo;
                d.lo[a] = (int)clo;
                d.dim[a] = (int)(chi - clo + 1);
            }
            d.bitbase = bit;
            d.nbits = (long long)d.dim[0] * d.dim[1] * d.dim[2];
            bit += (d.nbits + 31) & ~31ll;
        }
        *total_bits = bit;
        return kd;
    }

    // per-level unique-key counts of one pass (bitmap already filled): prefix of the
    // popcounts at each level's first word, and the total; one readback
    std::vector<uint32_t> count_bitmap(int depth, const KeyDomains& kd, long long total_bits) {
        long long nwords = total_bits / 32;
        grow(pscan, (size_t)(nwords + 1) * 4);
        grow(scan_tmp, scan_tmp_bytes(nwords));
        scan_exclusive_popc(ptr<uint32_t>(bitmap), ptr<uint32_t>(pscan), nwords, scan_tmp.p, stream);
        check_launch("popcount scan");
        std::vector<uint32_t> at(depth + 1);
        // the level prefixes, the error flag and the extras staged in kmeta: one copy
        CountStage st{};
        for (int l = 0; l <= depth; l++) st.words[l] = l < depth ? kd.d[l].bitbase / 32 : nwords;
        st.nlev = depth;
        st.err = ptr<int>(misc) + 8;
        st.kept = reinterpret_cast<const unsigned long long*>(rb_extra);
        st.bbox = reinterpret_cast<const int*>(rb_bbox);
        grow(kmeta, 256);
        uint32_t* stage = ptr<uint32_t>(kmeta) + 32;  // (bytes 128..255; 0..127: the sparse form's)
        launch_stage_counts(ptr<uint32_t>(pscan), st, stage, stream);
        check_launch("stage counts");
        check(cudaMemcpyAsync(pinned, stage, 104, cudaMemcpyDeviceToHost, stream), "rb");
        n_readback++;
        sync();
        int errflag = 0;
        memcpy(at.data(), pinned, 4 * (depth + 1));
        memcpy(&errflag, pinned + 64, 4);
        if (rb_extra) memcpy(&rb_extra_val, pinned + 72, 8);
        if (rb_bbox) memcpy(rb_bbox_val, pinned + 80, 24);
        if (spec_pass && errflag) {  // a key outside the guessed domains: the pass is redone
            spec_failed = true;
            return at;
        }
        if (errflag & 2)
            throw StatusError{GBVDB_INVALID_ARG, "a point's activation box spans more than 2^26 nodes of one level"};
        if (errflag) throw StatusError{GBVDB_CAPACITY, "node key outside its key domain"};
        return at;
    }

    // The sparse form's count: the new-key table compacted and sorted (ascending key =
    // the bitmap's bit order), per-level bounds by binary search; *overflow when a table
    // ran out of probes (nothing counted: the caller grows the tables and runs the pass
    // again).  Two readbacks.
    std::vector<uint32_t> count_hashed(int depth, const KeyDomains& kd, long long total_bits, bool* overflow) {
        grow(kmeta, 256);
        unsigned int* cnt = ptr<unsigned int>(kmeta);
        unsigned int* at_d = cnt + 16;
        check(cudaMemsetAsync(cnt, 0, 4, stream), "key count clear");
        grow(ksorted, (size_t)khash_cap * 8);
        const KeyHash kh{ptr<unsigned long long>(khash), (unsigned long long)khash_cap - 1};
        launch_hash_compact(kh, ptr<unsigned long long>(ksorted), cnt, stream);
        check_launch("hash compact");
        check(cudaMemcpyAsync(pinned, cnt, 4, cudaMemcpyDeviceToHost, stream), "rb");
        check(cudaMemcpyAsync(pinned + 4, ptr<int>(misc) + 8, 4, cudaMemcpyDeviceToHost, stream), "rb");
        if (rb_extra) check(cudaMemcpyAsync(pinned + 128, rb_extra, 8, cudaMemcpyDeviceToHost, stream), "rb");
        n_readback++;
        sync();
        unsigned int n = 0;
        int errflag = 0;
        memcpy(&n, pinned, 4);
        memcpy(&errflag, pinned + 4, 4);
        if (rb_extra) memcpy(&rb_extra_val, pinned + 128, 8);
        if (errflag & 2)
            throw StatusError{GBVDB_INVALID_ARG, "a point's activation box spans more than 2^26 nodes of one level"};
        if (errflag & 1) throw StatusError{GBVDB_CAPACITY, "node key outside its key domain"};
        *overflow = (errflag & 4) != 0;
        if (*overflow) return {};
        int bits = 1;
        while (bits < 63 && (1ll << bits) < total_bits) bits++;
        grow(kalt, (size_t)std::max<long long>(n, 1) * 8);
        grow(ksort_tmp, sort_tmp_bytes(n));
        sorted_keys = sort_keys_u64(ptr<unsigned long long>(ksorted), ptr<unsigned long long>(kalt), n, bits,
                                    ksort_tmp.p, stream);
        check_launch("key sort");
        launch_key_bounds(sorted_keys, cnt, kd, depth, at_d, stream);
        check_launch("key bounds");
        std::vector<uint32_t> at(depth + 1);
        readback(at.data(), at_d, 4 * (size_t)(depth + 1));
        n_hashed_passes++;
        return at;
    }

    // append the nodes of the counted pass to the pools in ascending key order
    long long allocate_counted(int depth, const KeyDomains& kd, const std::vector<uint32_t>& at) {
        long long added = 0;
        if (at[1] > at[0]) {  // leaves of this pass lie in the level-0 key domain
            for (int a = 0; a < 3; a++) {
                int lo = kd.d[0].lo[a], hi = kd.d[0].lo[a] + kd.d[0].dim[a] - 1;
                lgdom_lo[a] = lgdom_init ? std::min(lgdom_lo[a], lo) : lo;
                lgdom_hi[a] = lgdom_init ? std::max(lgdom_hi[a], hi) : hi;
            }
            lgdom_init = true;
        }
        for (int l = 0; l < depth; l++) {
            long long cnt = (long long)at[l + 1] - (long long)at[l];
            if (cnt <= 0) continue;
            long long base = ncnt[l];
            ensure_pool(l, base + cnt);
            if (hashed) {
                launch_alloc_nodes_sorted(sorted_keys, at[l], cnt, l, lgrange[l], kd.d[l], base, ptr<Node>(nodes[l]),
                                          stream);
            } else {
                long long w0 = kd.d[l].bitbase / 32;
                long long nw = ((kd.d[l].nbits + 31) / 32);
                launch_alloc_nodes(ptr<uint32_t>(bitmap), ptr<uint32_t>(pscan), w0, nw, l, lgrange[l], kd.d[l], base,
                                   ptr<Node>(nodes[l]), stream);
            }
            check_launch("alloc_nodes");
            if (l >= 1)
                check(cudaMemsetAsync(ptr<unsigned long long>(clist[l]) + base * cl_len(l), 0xFF,
                                      (size_t)(cnt * cl_len(l)) * 8, stream),
                      "childlist init");
            ncnt[l] = base + cnt;
            nused[l] += cnt;
            added += cnt;
        }
        return added;
    }

    // One key pass: clears the key sets of the pass's form, runs gen (the launches that
    // fill them) and counts the keys; in the sparse form a table that ran out of probes
    // is grown fourfold and the pass runs again (its launches only add keys and set leaf
    // markers, so a repeat gives the same sets).  est_keys / est_touched: expected set sizes.
    template <class Gen>
    std::vector<uint32_t> key_pass(int depth, const KeyDomains& kd, long long bits, long long est_keys,
                                   long long est_touched, Gen gen, bool err_ready = false) {
        for (int attempt = 0;; attempt++) {
            if (hashed) {
                clear_hash(khash, khash_cap, std::min(est_keys, bits));
                clear_hash(thash, thash_cap, std::min(est_touched, bits));
                grow(misc, 256);
                check(cudaMemsetAsync(ptr<int>(misc) + 8, 0, 4, stream), "err clear");
            } else {
                clear_bitmap(bits, err_ready);
            }
            gen(key_sets());
            if (!hashed) return count_bitmap(depth, kd, bits);
            bool overflow = false;
            std::vector<uint32_t> at = count_hashed(depth, kd, bits, &overflow);
            if (!overflow) return at;
            if (attempt >= 6) throw StatusError{GBVDB_CAPACITY, "key table overflow"};
            est_keys *= 4;
            est_touched *= 4;
        }
    }
    void clear_hash(DevBuf& b, long long& cap, long long want) {
        long long c = 1024;  // a multiple of 32 (k_hash_compact), load at most one half
        while (c < 2 * want) c <<= 1;
        cap = c;
        grow(b, (size_t)c * 8);
        check(cudaMemsetAsync(b.p, 0xFF, (size_t)c * 8, stream), "key table clear");
    }
    KeySets key_sets() {
        if (!hashed) return KeySets{{nullptr, 0}, {nullptr, 0}};
        return KeySets{{ptr<unsigned long long>(khash), (unsigned long long)khash_cap - 1},
                       {ptr<unsigned long long>(thash), (unsigned long long)thash_cap - 1}};
    }
    // Key-set form of a pass over a domain of `bits` key bits for `keys` point keys (n
    // points x levels): the bitmaps cost about 0.03 ns per bit (clear, popcount, scan, a
    // lane per bit in the allocation and resolve passes), the tables about 2 ns per key
    // plus some 50 us of fixed launches (sort passes); measured on a GB300 with 8,562
    // points in 4096^3 (16.8 M bits): 1.00 ms with the bitmaps, 0.47 ms with the tables.
    // Auto: the tables when bits > 64 keys + 2^21, or beyond kMaxBits (GBVDB_TUNE_KEYSET:
    // 1 the bitmaps while they fit, 2 the tables always).
    bool choose_hashed(long long bits, long long keys) const {
        if (keyset_mode == 2 || bits > kMaxBits) return true;
        if (keyset_mode == 1) return false;
        return bits > 64 * keys + (1ll << 21);
    }

    // rebuild the dense leaf lookup after a topology change (exact: built by traversal)
    void build_leaf_grid() {
        lgv.cells = nullptr;
        if (!lgdom_init || ncnt[0] == 0 || top_lev() == 0) return;
        long long cells = 1;
        int dim[3];
        for (int a = 0; a < 3; a++) {
            dim[a] = lgdom_hi[a] - lgdom_lo[a] + 1;
            cells *= dim[a];
        }
        if (cells > (1ll << 28)) return;  // too sparse for a dense table: kernels traverse the tree
        grow(lgrid, (size_t)cells * 4);
        check(cudaMemsetAsync(lgrid.p, 0xFF, (size_t)cells * 4, stream), "leaf grid clear");
        launch_build_leaf_grid(view(), ncnt[0], ptr<int>(lgrid), lgdom_lo, dim, lgrange[0], stream);
        check_launch("leaf grid");
        lgv.cells = ptr<int>(lgrid);
        for (int a = 0; a < 3; a++) { lgv.lo[a] = lgdom_lo[a]; lgv.dim[a] = dim[a]; }
        lgv.lgrange0 = lgrange[0];
    }

    void link_all(int depth) {
        TreeView t = view();
        for (int lev = depth - 1; lev >= 0; lev--) {
            long long nslots = ncnt[lev + 1] * cl_len(lev + 1);
            grow(link_tag, (size_t)std::max(nslots, 1ll) * 4);
            grow(link_slot, (size_t)std::max(ncnt[lev], 1ll) * 8);
            launch_link(t, lev, ncnt[lev], ptr<int>(link_tag), ptr<long long>(link_slot), stream);
            check_launch("link");
        }
    }

    // the key and touched bitmaps, one buffer, one clear (err_ready: the pass's error
    // flag was cleared by its setup launch)
    void clear_bitmap(long long total_bits, bool err_ready = false) {
        const long long words = ((total_bits / 32) + 63) & ~63ll;  // 256-byte aligned
        touched_off = words;
        grow(bitmap, (size_t)(2 * words) * 4 + 64);
        check(cudaMemsetAsync(bitmap.p, 0, (size_t)(2 * words) * 4, stream), "bitmap clear");
        grow(misc, 256);
        if (!err_ready) check(cudaMemsetAsync(ptr<int>(misc) + 8, 0, 4, stream), "err clear");
    }
    uint32_t* touched_bits() { return ptr<uint32_t>(bitmap) + touched_off; }

    static constexpr long long kMaxBits = 1ll << 34;

    // scratch of the direction-set form of the box pass (null: the per-point walk)
    uint32_t* touch_dirs_buf(const KeyDomains& kd) {
        // a word per level-0 position: beyond 2^28 words (1 GiB) the per-point walk
        if (!touch_dirs_on || touch_dirs_words(kd) > (1ll << 28)) return nullptr;
        grow(touch_dirs, (size_t)touch_dirs_words(kd) * 4);
        return ptr<uint32_t>(touch_dirs);
    }

    void activate_full(long long n, float radius, float3 orig, int D, const int rpos[3]) {
        // root first (VG.cpp:1288-1300)
        ensure_pool(D, 1);
        Node root{};
        root.lev = (uint8_t)D;
        root.flags = 1;
        for (int a = 0; a < 3; a++) { root.pos[a] = rpos[a]; root.value[a] = -1; }
        root.parent = kUndefL;
        root.childlist = elem(1, D, 0);
        launch_write_node(ptr<Node>(nodes[D]), root, stream);
        check_launch("write root");
        check(cudaMemsetAsync(clist[D].p, 0xFF, (size_t)cl_len(D) * 8, stream), "root childlist");
        ncnt[D] = 1;
        nused[D] = 1;
        root_lev = D;
        for (int a = 0; a < 3; a++) root_pos[a] = rpos[a];
        long long bits = 0;
        float margin = 2.0f * std::max(radius, 0.0f) + 4.0f;
        KeyDomains kd = domains(D, margin, rpos, D, &bits);
        hashed = choose_hashed(bits, n * D);
        PointSrc p = pts;
        p.n = n;
        // pass 1 (ActivateBricksGPU, VG.cpp:1229-1413)
        TreeView t = view();
        std::vector<uint32_t> at = key_pass(D, kd, bits, n * D, 0, [&](const KeySets& ks) {
            launch_keys_pass1(t, p, orig, D, kd, ptr<uint32_t>(bitmap), ks, ptr<int>(misc) + 8, stream);
            check_launch("keys_pass1");
        });
        allocate_counted(D, kd, at);
        mark();
        link_all(D);
        build_leaf_grid();
        mark();
        // pass 2 (ActivateExtraBricksGPU, VG.cpp:931-1016), only if radius >= 1 (VG.cpp:1207)
        if (radius >= 1) {
            t = view();
            int rlo[3], rhi[3];
            for (int a = 0; a < 3; a++) { rlo[a] = rpos[a]; rhi[a] = (int)std::min<long long>(rpos[a] + range[D], 0x7FFFFFFF); }
            at = key_pass(D, kd, bits, (long long)at[(size_t)D] + 1024, 4 * n + 1024, [&](const KeySets& ks) {
                launch_keys_box(t, lgv, p, orig, radius, 2, D, rlo, rhi, kd, touched_bits(),
                                ptr<uint32_t>(bitmap), nullptr, ptr<int>(misc) + 8, hashed ? nullptr : touch_dirs_buf(kd),
                                ks, ncnt[0], stream);
                check_launch("keys_extra");
            });
            if (allocate_counted(D, kd, at) > 0) {
                mark();
                link_all(D);
                build_leaf_grid();
            }
            mark();
        }
        last_kd = kd;
        last_kd_depth = hashed ? -1 : D;
    }

    // The last pass's key domains one node wider on each side, clipped to the root: the
    // domains an incremental pass guesses before the frame's bounds are read back
    bool widened_last_domains(int D, int rl, KeyDomains* out, long long* total_bits) const {
        KeyDomains kd{};
        long long bit = 0;
        const long long rg_root = range[rl];
        for (int l = 0; l < D; l++) {
            KeyDomain& d = kd.d[l];
            for (int a = 0; a < 3; a++) {
                long long lo = (long long)last_kd.d[l].lo[a] - 1, hi = (long long)last_kd.d[l].lo[a] + last_kd.d[l].dim[a];
                const long long rlo = (long long)root_pos[a] >> lgrange[l];
                const long long rhi = ((long long)root_pos[a] + rg_root - 1) >> lgrange[l];
                lo = std::max(std::max(lo, rlo), 0ll);
                hi = std::min(hi, rhi);
                if (hi < lo) hi = lo;
                d.lo[a] = (int)lo;
                d.dim[a] = (int)(hi - lo + 1);
            }
            d.bitbase = bit;
            d.nbits = (long long)d.dim[0] * d.dim[1] * d.dim[2];
            bit += (d.nbits + 31) & ~31ll;
        }
        *out = kd;
        *total_bits = bit;
        return bit <= kMaxBits;
    }
    static bool domains_contain(const KeyDomains& outer, const KeyDomains& inner, int D) {
        for (int l = 0; l < D; l++)
            for (int a = 0; a < 3; a++)
                if (inner.d[l].lo[a] < outer.d[l].lo[a] ||
                    (long long)inner.d[l].lo[a] + inner.d[l].dim[a] > (long long)outer.d[l].lo[a] + outer.d[l].dim[a])
                    return false;
        return true;
    }

    // guess (speculative pass): run on the last pass's widened domains while the frame's
    // bounds are computed on the device; they come back with the key counts, and the pass
    // stands only if the frame keeps its depth and all its keys lie in the guessed
    // domains (then the key sets, and so the pools, are those of the exact domains).
    // Returns false when it does not stand; nothing but scratch was written then.
    bool activate_incremental(long long n, float radius, float3 orig, int D, bool accum, bool guess = false) {
        struct RbReset {  // the pass's readback extras end with it, thrown out of or not
            gbvdb_grid_s* g;
            ~RbReset() {
                g->rb_extra = nullptr;
                g->rb_bbox = nullptr;
                g->spec_pass = false;
            }
        } rb_reset{this};
        long long nleaf = ncnt[0];
        if (nleaf == 0) return !guess;  // VG.cpp:1022
        long long bits = 0;
        float margin = 2.0f * std::max(radius, 0.0f) + 4.0f;
        int rl = root_lev >= 0 ? root_lev : D;
        KeyDomains kd{};
        if (guess) {
            if (!widened_last_domains(D, rl, &kd, &bits) || choose_hashed(bits, n * D)) return false;
        } else {
            kd = domains(D, margin, root_pos, rl, &bits);
        }
        // markers, the error flag, the kept-leaf counter and (a guess) the bounds' initial
        // values in one launch, then (a guess) the bounds
        grow(markers, (size_t)nleaf * 4);
        grow(misc, 256);
        unsigned long long* kept = reinterpret_cast<unsigned long long*>(ptr<char>(misc) + 72);
        int* d6 = guess ? ptr<int>(misc) : nullptr;
        launch_incr_setup(ptr<Node>(nodes[0]), nleaf, ptr<int>(markers), accum ? 1 : 0, ptr<int>(misc) + 8, kept, d6,
                          stream);
        check_launch("incr_setup");
        if (guess) {
            PointSrc pb = pts;
            pb.n = n;
            launch_bbox(pb, orig, d6, stream);
            check_launch("bbox");
            rb_bbox = d6;
        }
        hashed = choose_hashed(bits, n * D);
        PointSrc p = pts;
        p.n = n;
        TreeView t = view();
        int rlo[3], rhi[3];
        for (int a = 0; a < 3; a++) { rlo[a] = root_pos[a]; rhi[a] = (int)std::min<long long>(root_pos[a] + range[rl], 0x7FFFFFFF); }
        // count new keys before touching the tree: nothing missing -> return (VG.cpp:1066).
        // The kept leaves (non-zero markers) come back with the counts: with the new
        // leaves they are the flagged-leaf count, so UpdateAtlas needs no readback of its own
        rb_extra = kept;
        spec_pass = guess;
        spec_failed = false;
        std::vector<uint32_t> at = key_pass(D, kd, bits, nleaf / 4 + 1024, 4 * n + 1024, [&](const KeySets& ks) {
            // (the sparse form may run the pass again: its count starts from zero each time)
            if (hashed) check(cudaMemsetAsync(kept, 0, 8, stream), "kept clear");
            launch_keys_box(t, lgv, p, orig, radius, 1, D, rlo, rhi, kd, touched_bits(), ptr<uint32_t>(bitmap),
                            ptr<int>(markers), ptr<int>(misc) + 8, hashed ? nullptr : touch_dirs_buf(kd), ks, nleaf, stream);
            check_launch("keys_incr");
            launch_count_markers(ptr<int>(markers), nleaf, kept, stream);
            check_launch("count_markers");
        }, true);
        rb_extra = nullptr;
        rb_bbox = nullptr;
        spec_pass = false;
        if (guess) {
            if (spec_failed) return false;
            float pmin[3], pmax[3];
            bbox_bounds(rb_bbox_val, pmin, pmax);
            for (int a = 0; a < 3; a++) { posmin[a] = pmin[a]; posmax[a] = pmax[a]; }
            int rpos[3];
            if (determine_depth(rpos) != D) return false;  // the caller's full path clears the tree
            long long exact_bits = 0;
            if (!domains_contain(kd, domains(D, margin, root_pos, rl, &exact_bits), D)) return false;
        }
        mark();
        if (at[(size_t)D] == 0) {
            last_kd = kd;
            last_kd_depth = hashed ? -1 : D;
            return true;
        }
        launch_apply_markers(ptr<Node>(nodes[0]), nleaf, ptr<int>(markers), stream);
        check_launch("apply_markers");
        allocate_counted(D, kd, at);
        link_all(D);
        t = view();
        launch_delink_leaf(t, ncnt[0], stream);
        check_launch("delink_leaf");
        for (int lev = 1; lev < D; lev++) {
            launch_delink_upper(t, lev, ncnt[lev], stream);
            check_launch("delink_upper");
        }
        build_leaf_grid();
        // usedCnt(0,0) = number of flagged leaves (VG.cpp:1144-1148): the kept old leaves
        // plus the new ones
        nused[0] = (long long)rb_extra_val + ((long long)at[1] - (long long)at[0]);
        nused0_stale = false;
        last_kd = kd;
        last_kd_depth = hashed ? -1 : D;
        mark();
        return true;
    }

    // the flagged-leaf count, when an incremental rebuild left it to be counted
    void refresh_nused0() {
        if (!nused0_stale) return;
        check(cudaMemsetAsync(ptr<char>(misc) + 64, 0, 8, stream), "count clear");
        launch_count_flags(ptr<Node>(nodes[0]), ncnt[0], reinterpret_cast<unsigned long long*>(ptr<char>(misc) + 64),
                           stream);
        check_launch("count_flags");
        unsigned long long used = 0;
        readback(&used, ptr<char>(misc) + 64, 8);
        nused[0] = (long long)used;
        nused0_stale = false;
    }

    gbvdb_status rebuild(long long n, float radius, float3 orig, bool accumulate, int min_depth) {
        layout_changed();
        if (!configured) throw StatusError{GBVDB_INVALID_ARG, "Configure was not called"};
        if (n <= 0) return GBVDB_NOOP;
        if (!pts.base) throw StatusError{GBVDB_INVALID_ARG, "SetPoints was not called"};
        if (pts.n > 0 && n > pts.n) throw StatusError{GBVDB_INVALID_ARG, "num_pnts exceeds the point buffer"};
        stage_begin();
        // an incremental frame of unchanged depth: its key pass runs on the last pass's
        // domains, widened, with the frame's bounds read back together with the key counts
        // instead of before the pass (one host round trip less); otherwise, or when the
        // guess does not stand, the pass on the exact domains below
        if (!accumulate && !rebuild_topo && curr_depth > 0 && last_kd_depth == curr_depth &&
            activate_incremental(n, radius, orig, curr_depth, false, true)) {
            last_depth = curr_depth;
            sc_valid = false;
            lists_valid = false;
            stage_end();
            return GBVDB_OK;
        }
        compute_bbox(n, orig);
        mark();
        int rpos[3];
        int D = determine_depth(rpos);
        if (accumulate && D >= 0 && D < min_depth) D = min_depth;
        if (D <= 0 || D > 5 || D >= levs)
            throw StatusError{GBVDB_DEPTH_UNSUPPORTED, D == 0 ? "point extents smaller than 1 brick"
                                                              : "point extents exceed the configured levels"};
        if (accumulate) {  // AccumulateTopology (VG.cpp:1158-1178)
            if (rebuild_topo) return rebuild(n, radius, orig, false, 0);
            last_depth = D;
            activate_incremental(n, radius, orig, D, true);
            sc_valid = false;
            stage_end();
            return GBVDB_OK;
        }
        if (rebuild_topo) {
            clear_topology();
        } else if (D != curr_depth) {  // VG.cpp:1198-1203
            clear_topology();
            rebuild_topo = 1;
            curr_depth = D;
        }
        last_depth = D;
        if (rebuild_topo) {
            activate_full(n, radius, orig, D, rpos);
            rebuild_topo = 0;
        } else {
            activate_incremental(n, radius, orig, D, false);
        }
        sc_valid = false;
        lists_valid = false;
        stage_end();
        return GBVDB_OK;
    }

    // ------------------------------------------------------------- atlas
    void resize_channels(long long slots) {
        layout_changed();
        bool grows = false;
        for (int c = 0; c < 8; c++) grows |= ch[c].used && ch[c].cap_slots < slots;
        if (grows) join_side();  // an overlapped checksum still reads the interiors being moved
        for (int c = 0; c < 8; c++) {
            Channel& C = ch[c];
            if (!C.used || C.cap_slots >= slots) continue;
            grow(C.interior, (size_t)slots * 4096 * C.esize, (size_t)C.cap_slots * 4096 * C.esize);
            grow(C.apron_buf, (size_t)slots * kApronStride * C.esize, (size_t)C.cap_slots * kApronStride * C.esize);
            // bricks new to the atlas start at zero, as the channel does
            const size_t i0 = (size_t)C.cap_slots * 4096 * C.esize, a0 = (size_t)C.cap_slots * kApronStride * C.esize;
            check(cudaMemsetAsync(ptr<char>(C.interior) + i0, 0, (size_t)slots * 4096 * C.esize - i0, stream), "atlas clear");
            check(cudaMemsetAsync(ptr<char>(C.apron_buf) + a0, 0, (size_t)slots * kApronStride * C.esize - a0, stream),
                  "atlas clear");
            C.cap_slots = slots;
        }
    }

    gbvdb_status update_atlas() {  // UpdateAtlas (VG.cpp:2630-2704)
        layout_changed();
        if (!ch[0].used) throw StatusError{GBVDB_INVALID_ARG, "no atlas channel"};
        stage_begin();
        long long total = ncnt[0];
        // the flagged-leaf count is F below; an earlier count is only used when it is current
        long long used = nused0_stale ? 0 : nused[0];
        atlas_last = 0;
        long long layer = (long long)ax * ay;
        if (used > layer * az) az = (int)std::ceil((double)((float)used / (float)layer));
        long long F = 0;
        if (total > 0) {
            grow(flags_scan, (size_t)(total + 1) * 4);
            grow(scan_tmp, scan_tmp_bytes(total));
            scan_exclusive_node_flags(ptr<Node>(nodes[0]), 0, ptr<uint32_t>(flags_scan), total, scan_tmp.p, stream);
            check_launch("atlas scan");
            if (nused0_stale) {
                uint32_t f = 0;
                readback(&f, ptr<uint32_t>(flags_scan) + total, 4);
                F = f;
            } else {
                F = nused[0];  // the flagged-leaf count, kept exact by every topology change
            }
        }
        if (F > layer * az) az = (int)std::ceil((double)((float)F / (float)layer));  // AtlasAlloc growth, AL.cpp:695-698
        if (nused0_stale) {  // F is the flagged-leaf count
            nused[0] = F;
            nused0_stale = false;
        }
        long long slots = layer * az;
        resize_channels(slots);
        grow(amap, (size_t)slots * sizeof(AtlasNode));
        amap_slots = slots;
        launch_fill_u32(ptr<uint32_t>(amap), slots * 4, 0xFFFFFFFFu, stream);
        if (total > 0)
            launch_assign_slots(ptr<Node>(nodes[0]), total, ptr<uint32_t>(flags_scan), ax, ay, ptr<AtlasNode>(amap),
                                stream);
        check_launch("assign_slots");
        atlas_last = (int)F;
        mark();
        stage_end();
        return GBVDB_OK;
    }

    // -------------------------------------------------------- subcells
    void build_linked() {
        long long nleaf = ncnt[0];
        grow(scmap, (size_t)(nleaf + 1) * 4);
        grow(scan_tmp, scan_tmp_bytes(nleaf));
        scan_exclusive_node_flags(ptr<Node>(nodes[0]), 1, ptr<uint32_t>(scmap), nleaf, scan_tmp.p, stream);
        check_launch("scmap");
        // the linked count scmap[nleaf] is read back with the binning totals
        grow(linked, (size_t)(nleaf + 1) * 4);
        launch_linked_list(ptr<Node>(nodes[0]), nleaf, ptr<uint32_t>(scmap), ptr<int>(linked), stream);
        check_launch("linked");
    }

    gbvdb_status insert_subcell(int sc, long long n, float R, float3 trans, long long* out_len, bool fp16 = false) {
        if (!configured) throw StatusError{GBVDB_INVALID_ARG, "Configure was not called"};
        if (!pts.base) throw StatusError{GBVDB_INVALID_ARG, "SetPoints was not called"};
        if (sc != 4 || log2dim[0] != 4) throw StatusError{GBVDB_NOT_SUPPORTED, "subcell size 4 with 16^3 bricks only"};
        if (!(R >= 0)) throw StatusError{GBVDB_INVALID_ARG, "negative radius"};
        if (pts.n > 0 && n > pts.n) throw StatusError{GBVDB_INVALID_ARG, "num_pnts exceeds the point buffer"};
        if (fp16 && clr.base)
            throw StatusError{GBVDB_NOT_SUPPORTED, "InsertPointsSubcell_FP16 with point colours"};
        refresh_nused0();
        if (nused[0] == 0) return GBVDB_NOOP;  // VG.cpp:4973-4977
        stage_begin();
        build_linked();
        mark();
        long long nbins = ncnt[0] * 64;  // upper bound: bins of unlinked leaves stay empty
        grow(bin_cnt, (size_t)(nbins + 1) * 4);
        grow(bin_off, (size_t)(nbins + 1) * 4);
        PointSrc p = pts;
        p.n = std::max(n, 0ll);
        grow(bin_of, (size_t)std::max(p.n, 1ll) * 4);
        grow(rank_of, (size_t)std::max(p.n, 1ll) * 4);
        grow(misc, 256);
        unsigned long long* totals = reinterpret_cast<unsigned long long*>(ptr<char>(misc) + 128);
        if (R > 11.0f) {  // (else the neighbour-mask pass below clears them)
            check(cudaMemsetAsync(bin_cnt.p, 0, (size_t)(nbins + 1) * 4, stream), "bin clear");
            check(cudaMemsetAsync(totals, 0, 16, stream), "totals clear");
        }
        TreeView t = view();
        // InsertPointsSubcell_FP16 quantises over the bounds of the last GetBoundingBox
        // (VG.cpp:5458-5462: PosRange = PosMax - PosMin)
        Quant qz{};
        qz.on = fp16 ? 1 : 0;
        qz.mn = make_float3(posmin[0], posmin[1], posmin[2]);
        qz.rg = make_float3(posmax[0] - posmin[0], posmax[1] - posmin[1], posmax[2] - posmin[2]);
        sc_quant = qz;
        // R <= 11: the list-length count reads the linked flags of the 27 bricks around
        // each home brick from a per-leaf mask instead of looking each brick up
        const uint32_t* nbm = nullptr;
        if (R <= 11.0f) {
            grow(nbmask, (size_t)std::max(ncnt[0], 1ll) * 4);
            launch_nb_mask(t, lgv, ncnt[0], ptr<uint32_t>(nbmask), ptr<uint32_t>(bin_cnt), totals, stream);
            nbm = ptr<uint32_t>(nbmask);
        }
        launch_bin_count(t, lgv, p, trans, R, qz, ptr<uint32_t>(scmap), nbm, ptr<uint32_t>(bin_cnt), ptr<int>(bin_of),
                         ptr<uint32_t>(rank_of), totals, bin_unroll(p.n), stream);
        check_launch("bin_count");
        grow(scan_tmp, scan_tmp_bytes(nbins));
        scan_exclusive_u32(ptr<uint32_t>(bin_cnt), ptr<uint32_t>(bin_off), nbins, scan_tmp.p, stream);
        check_launch("bin scan");
        // The totals are read back while the scatter runs: the host waits for the copies
        // (an event before the scatter), not for the stream, so the caller's next calls
        // queue behind the scatter with no idle gap.  The binned records are at most one
        // per point, so the buffers are sized by the point count.
        grow(sorted, (size_t)std::max<long long>(p.n, 1) * 16);
        // the list entries carry the points' colours when SetPoints gave a colour buffer
        // (InsertPointsSubcell, VG.cpp:5063-5075)
        if (clr.base) grow(sorted_clr, (size_t)std::max<long long>(p.n, 1) * 4);
        unsigned long long tot[2];
        uint32_t nb = 0;
        check(cudaMemcpyAsync(pinned, totals, 16, cudaMemcpyDeviceToHost, stream), "rb");
        check(cudaMemcpyAsync(pinned + 20, ptr<uint32_t>(scmap) + ncnt[0], 4, cudaMemcpyDeviceToHost, stream), "rb");
        check(cudaEventRecord(rb_ev, stream), "readback event");
        n_readback++;
        mark();
        launch_bin_scatter(p, trans, R, qz, ptr<int>(bin_of), ptr<uint32_t>(rank_of), ptr<uint32_t>(bin_off),
                           ptr<float4>(sorted), clr, ptr<uint32_t>(sorted_clr), scatter_unroll(p.n), stream);
        check_launch("bin_scatter");
        check(cudaEventSynchronize(rb_ev), "readback wait");
        memcpy(tot, pinned, 16);
        memcpy(&nb, pinned + 20, 4);
        sc_nbricks = nb;
        mark();
        sc_valid = true;
        lists_valid = false;
        sc_R = R;
        sc_trans = trans;
        sc_pts = p;
        sc_clr = clr;
        sc_nleaf = ncnt[0];
        sc_len = (long long)tot[0];
        sc_orphans = (long long)tot[1];
        if (out_len) *out_len = sc_len;
        stage_end();
        return GBVDB_OK;
    }

    // materialize the reference-shaped subcell lists (export and the fallback gather)
    void materialize_lists() {
        if (lists_valid) return;
        if (sc_len > 0xFFFFFFFFll) throw StatusError{GBVDB_NOT_SUPPORTED, "subcell lists exceed 2^32 entries"};
        long long nsub = sc_nbricks * 64;
        grow(list_cnt, (size_t)(nsub + 1) * 4);
        grow(list_off, (size_t)(nsub + 1) * 4);
        grow(list_pts, (size_t)std::max(sc_len, 1ll) * 12);
        if (sc_clr.base) grow(list_clr, (size_t)std::max(sc_len, 1ll) * 4);
        check(cudaMemsetAsync(list_cnt.p, 0, (size_t)(nsub + 1) * 4, stream), "list clear");
        TreeView t = view();
        launch_list_count(t, lgv, sc_pts, sc_trans, sc_R, sc_quant, ptr<uint32_t>(scmap), ptr<uint32_t>(list_cnt),
                          stream);
        grow(scan_tmp, scan_tmp_bytes(nsub));
        scan_exclusive_u32(ptr<uint32_t>(list_cnt), ptr<uint32_t>(list_off), nsub, scan_tmp.p, stream);
        check(cudaMemsetAsync(list_cnt.p, 0, (size_t)(nsub + 1) * 4, stream), "list clear");
        launch_list_fill(t, lgv, sc_pts, sc_trans, sc_R, sc_quant, ptr<uint32_t>(scmap), ptr<uint32_t>(list_off),
                         ptr<uint32_t>(list_cnt), ptr<float>(list_pts), sc_clr, ptr<uint32_t>(list_clr), stream);
        check_launch("lists");
        lists_valid = true;
    }

    // candidate home-bin offsets d = H - S (subcell units) with their integer lower
    // bound lb2 on the squared distance from any point of bin H to the voxels of
    // subcell S, sorted ascending; offsets with lb2 >= T are dropped
    void build_offsets(int lo_off, int hi_off, float T, float R) {
        if (offs_R == R && offs_T == bits_of(T) && noffs > 0) return;
        std::vector<std::array<int, 4>> v;
        auto gap = [](int d) { return d > 0 ? 4 * d - 3 : (d < 0 ? -4 * d - 4 : 0); };
        for (int dz = lo_off; dz <= hi_off; dz++)
            for (int dy = lo_off; dy <= hi_off; dy++)
                for (int dx = lo_off; dx <= hi_off; dx++) {
                    int lb2 = gap(dx) * gap(dx) + gap(dy) * gap(dy) + gap(dz) * gap(dz);
                    if (!((float)lb2 < T)) continue;
                    v.push_back({dx, dy, dz, lb2});
                }
        std::stable_sort(v.begin(), v.end(), [](const std::array<int, 4>& a, const std::array<int, 4>& b) {
            return a[3] < b[3];
        });
        noffs = (int)v.size();
        grow(offs_buf, (size_t)std::max(noffs, 1) * 16);
        if (noffs) {
            std::vector<int> flat((size_t)noffs * 4);
            for (int i = 0; i < noffs; i++)
                for (int k = 0; k < 4; k++) flat[(size_t)i * 4 + k] = v[(size_t)i][(size_t)k];
            memcpy(pinned, flat.data(), flat.size() * 4);
            check(cudaMemcpyAsync(offs_buf.p, pinned, flat.size() * 4, cudaMemcpyHostToDevice, stream), "offsets");
            sync();
        }
        offs_R = R;
        offs_T = bits_of(T);
    }

    // a float in channel c's storage type: FP32 bits, FP16 / BF16 bits, or for T_UCHAR4
    // make_uchar4(v, v, v, v) (UpdateApronC4's boundary value, OP.cuh:140-143)
    uint32_t storage_bits(int c, float v) const {
        if (ch[c].dtype == GBVDB_T_UCHAR4) {  // the same float -> uchar conversion as the colour gathers
            const uint32_t b = !(v == v) || v <= 0.0f ? 0u : (v >= 4294967296.0f ? 255u : (uint32_t)v & 0xFFu);
            return b | (b << 8) | (b << 16) | (b << 24);
        }
        if (ch[c].esize == 4) return bits_of(v);
        return ch[c].dtype == GBVDB_T_HALF ? f2h_bits(v) : f2bf_bits(v);
    }

    static uint32_t bits_of(float f) {
        uint32_t u;
        memcpy(&u, &f, 4);
        return u;
    }
    static float next_up(float f) {
        uint32_t u = bits_of(f);
        u += 1;
        float r;
        memcpy(&r, &u, 4);
        return r;
    }

    gbvdb_status gather(int mode, int sc, float rho, long long sc_len_arg, int chan, int clr_chan, bool accum) {
        if (sc != 4) throw StatusError{GBVDB_NOT_SUPPORTED, "subcell size 4 only"};
        if (chan < 0 || chan >= 8 || !ch[chan].used) throw StatusError{GBVDB_INVALID_ARG, "bad channel"};
        if (ch[chan].dtype != GBVDB_T_FLOAT && ch[chan].dtype != GBVDB_T_HALF && ch[chan].dtype != GBVDB_T_BFLOAT16)
            throw StatusError{GBVDB_NOT_SUPPORTED, "gathers write float, half or bfloat16 channels"};
        refresh_nused0();
        if (nused[0] == 0) return GBVDB_NOOP;                       // VG.cpp:5321-5322, 5350-5351
        if (mode == 0 && sc_len_arg == 0) return GBVDB_NOOP;        // VG.cpp:5321
        if (!sc_valid || sc_nleaf != ncnt[0]) throw StatusError{GBVDB_INVALID_ARG, "InsertPointsSubcell is stale"};
        // colours: averaged into chanClr when the insert carried point colours (PT.cuh:728, 768)
        const bool colour = sc_clr.base != nullptr;
        if (colour && (clr_chan < 0 || clr_chan >= 8 || !ch[clr_chan].used || ch[clr_chan].dtype != GBVDB_T_UCHAR4))
            throw StatusError{GBVDB_INVALID_ARG, "the points carry colours: chanClr must be a T_UCHAR4 channel"};
        stage_begin();
        GatherParams gp{};
        gp.mode = mode;
        gp.accum = accum ? 1 : 0;
        gp.rho = rho;
        gp.R = sc_R;
        gp.dtype = ch[chan].dtype;
        gp.ax = ax;
        gp.ay = ay;
        // static cutoff T: any d^2 >= T leaves the voxel at its initial value
        float T = INFINITY;
        if (!accum) {
            if (mode == 0) {
                T = (float)((double)rho * rho);
                if (!(rho > 0)) T = 0.0f;
                while (!(std::sqrt(T) >= rho)) T = next_up(T);
            } else {
                double r3 = (double)rho + 3.0;
                T = r3 > 0 ? (float)(r3 * r3) : 0.0f;
                while (!((float)(std::sqrt(T) - rho) >= 3.0f) && T < 3.0e38f) T = next_up(T);
            }
        }
        gp.tbits = bits_of(T);
        gp.rcut = std::isfinite(T) ? (float)(std::sqrt((double)T) + 0.01) : INFINITY;
        gp.lo_off = (int)std::floor((-1.0 - sc_R) / 4.0) - 1;
        gp.hi_off = (int)std::ceil((4.0 + sc_R) / 4.0);
        int span = 4 + gp.hi_off - gp.lo_off;
        TreeView t = view();
        void* interior = ch[chan].interior.p;
        interior_written(chan);
        if (sc_orphans > 0 || span > 12) {
            materialize_lists();
            launch_gather_lists(t, ptr<int>(linked), sc_nbricks, ptr<uint32_t>(list_off), ptr<float>(list_pts), gp,
                                interior, stream);
            if (colour) {
                interior_written(clr_chan);
                launch_gather_colour_lists(t, ptr<int>(linked), sc_nbricks, ptr<uint32_t>(list_off),
                                           ptr<uint32_t>(list_clr), ax, ay, gp.accum, ptr<uint32_t>(ch[clr_chan].interior),
                                           stream);
            }
        } else {
            int tslot = -1;
            const TuneEntry* te = tune_auto ? tune_entry(sc_pts.n) : nullptr;
            gp.dense_min = te ? te->dense_min : tune_pick(sc_nbricks, &tslot);
            gp.min_blocks = gather_blocks(sc_pts.n);
            // long bricks first: the gather form's and the scatter form's fullest
            const int lm = gather_long_min(sc_pts.n);
            gp.long_min = lm < 0 ? -1 : std::min(lm, gp.dense_min);
            // fused apron: needs the dense leaf lookup (the apron pass resolves
            // neighbours with the same table) and an apron of one voxel
            const bool push = fused_apron && lgv.cells && ch[chan].apron == 1 && atlas_last > 0;
            gp.apron = push ? ch[chan].apron_buf.p : nullptr;
            build_offsets(gp.lo_off, gp.hi_off, T, sc_R);
            // push_bad: the push check's flag, then the gather's two launch-order counters
            grow(push_bad, 16);
            if (push || gp.long_min >= 0) check(cudaMemsetAsync(push_bad.p, 0, 12, stream), "push check clear");
            gp.order = ptr<unsigned>(push_bad) + 1;
            if (push) {
                gp.apron_bad = ptr<int>(push_bad);
                launch_push_check(t, lgv, ptr<uint32_t>(scmap), ptr<AtlasNode>(amap), atlas_last, ax, ay, ncnt[0],
                                  ptr<int>(push_bad), stream);
            }
            grow(gtab, (size_t)std::max(sc_nbricks, 1ll) * 32 * 16);
            if (tslot >= 0) check(cudaEventRecord(tune_ev[2 * tslot], stream), "tune event");
            launch_gather(t, lgv, ptr<int>(linked), sc_nbricks, ptr<uint32_t>(scmap), ptr<uint32_t>(bin_off),
                          ptr<float4>(sorted), ptr<int4>(offs_buf), noffs, gp, ptr<int4>(gtab), interior, stream);
            if (tslot >= 0) {
                check(cudaEventRecord(tune_ev[2 * tslot + 1], stream), "tune event");
                if (++tune_step == kTuneN) tune_pending = true;
            }
            if (push) pushed_ver[chan] = layout_ver;
            if (colour) {
                // member offsets H - S: S - H lies in [floor(-R/4), floor((5+R)/4)] on every axis
                const int dlo = (int)std::floor(-(double)sc_R / 4.0), dhi = (int)std::floor((5.0 + sc_R) / 4.0);
                interior_written(clr_chan);
                launch_gather_colour(ptr<int4>(gtab), sc_nbricks, ptr<uint32_t>(bin_off), ptr<float4>(sorted),
                                     ptr<uint32_t>(sorted_clr), -dhi, -dlo, gp.accum,
                                     ptr<uint32_t>(ch[clr_chan].interior), stream);
            }
        }
        check_launch("gather");
        mark();
        stage_end();
        return GBVDB_OK;
    }

    gbvdb_status update_apron(int chan, float boundval) {  // UpdateApron (VG.cpp:4418-4457)
        if (chan < 0 || chan >= 8 || !ch[chan].used) throw StatusError{GBVDB_INVALID_ARG, "bad channel"};
        if (ch[chan].apron == 0) return GBVDB_NOOP;
        if (ncnt[0] == 0 || atlas_last == 0) return GBVDB_NOOP;
        stage_begin();
        const uint32_t bb = storage_bits(chan, boundval);
        TreeView t = view();
        // after a fused-apron gather of this layout only the faces of missing
        // neighbours are left to write
        const bool fill_only = fused_apron && lgv.cells && pushed_ver[chan] == layout_ver;
        launch_apron(t, lgv, ptr<AtlasNode>(amap), atlas_last, ax, ay, ch[chan].esize, ch[chan].interior.p,
                     ch[chan].apron_buf.p, bb, fill_only ? ptr<int>(push_bad) : nullptr, stream);
        check_launch("apron");
        mark();
        stage_end();
        return GBVDB_OK;
    }

    // ------------------------------------------- legacy insert and scatter
    // InsertPoints (VG.cpp:5219-5267): the leaf of every point and the points grouped by
    // leaf (always grouped: ScatterDensity reads the groups; bPrefix only names the
    // reference's optional sort)
    gbvdb_status insert_points(long long n, float3 trans, bool prefix) {
        (void)prefix;
        if (!configured) throw StatusError{GBVDB_INVALID_ARG, "Configure was not called"};
        if (!pts.base && n > 0) throw StatusError{GBVDB_INVALID_ARG, "SetPoints was not called"};
        if (n < 0 || (pts.n > 0 && n > pts.n)) throw StatusError{GBVDB_INVALID_ARG, "num_pnts exceeds the point buffer"};
        long long nl = ncnt[0];
        grow(pnode, (size_t)std::max(n, 1ll) * 4);
        grow(pndx, (size_t)std::max(n, 1ll) * 4);
        grow(gcnt, (size_t)(nl + 1) * 4);
        grow(goff, (size_t)(nl + 1) * 4);
        grow(psort, (size_t)std::max(n, 1ll) * 12);
        check(cudaMemsetAsync(gcnt.p, 0, (size_t)(nl + 1) * 4, stream), "gcnt clear");
        PointSrc p = pts;
        p.n = n;
        TreeView t = view();
        launch_insert_points(t, lgv, p, trans, ptr<int>(pnode), ptr<uint32_t>(pndx), ptr<uint32_t>(gcnt), stream);
        check_launch("insert points");
        grow(scan_tmp, scan_tmp_bytes(nl));
        scan_exclusive_u32(ptr<uint32_t>(gcnt), ptr<uint32_t>(goff), nl, scan_tmp.p, stream);
        launch_sort_points(p, trans, ptr<int>(pnode), ptr<uint32_t>(pndx), ptr<uint32_t>(goff), ptr<float>(psort), stream);
        check_launch("sort points");
        ins_n = n;
        ins_nleaf = nl;
        return GBVDB_OK;
    }

    // ScatterDensity (VG.cpp:5624-5660, gvdbScatterPointDensity PT.cuh:525-571) into
    // channel 0 over the groups of the last InsertPoints; amp is unused by the kernel
    gbvdb_status scatter_density(float radius, bool expand, bool avg_color) {
        if (avg_color) throw StatusError{GBVDB_NOT_SUPPORTED, "colour channels are not part of this path"};
        if (ins_n < 0 || ins_nleaf != ncnt[0]) throw StatusError{GBVDB_INVALID_ARG, "InsertPoints was not called for this topology"};
        if (!ch[0].used || ch[0].dtype != GBVDB_T_FLOAT) throw StatusError{GBVDB_NOT_SUPPORTED, "ScatterDensity: FP32 channel 0"};
        if (atlas_last == 0 || ins_nleaf == 0) return GBVDB_NOOP;
        interior_written(0);
        launch_scatter_density(ptr<Node>(nodes[0]), ins_nleaf, ptr<uint32_t>(goff), ptr<float>(psort), radius,
                               expand ? 1 : 0, res[0], ax, ay, ptr<float>(ch[0].interior), ptr<float>(ch[0].apron_buf),
                               stream);
        check_launch("scatter density");
        return GBVDB_OK;
    }

    // ------------------------------------------------- apron faces and smoothing
    gbvdb_status update_neighbors() {  // UpdateNeighbors (VG.cpp:2527-2556)
        long long n = ncnt[0];
        grow(nbr_table, (size_t)std::max(n, 1ll) * 6 * 4);
        TreeView t = view();
        launch_neighbors(t, lgv, n, (int)range[0], ptr<int>(nbr_table), stream);
        check_launch("neighbors");
        nbr_count = n;
        return GBVDB_OK;
    }

    gbvdb_status update_apron_faces(int chan) {  // UpdateApronFaces (VG.cpp:4461-4496)
        if (chan < 0 || chan >= 8 || !ch[chan].used) throw StatusError{GBVDB_INVALID_ARG, "bad channel"};
        if (nbr_count != ncnt[0]) throw StatusError{GBVDB_INVALID_ARG, "UpdateNeighbors was not called for this topology"};
        if (atlas_last == 0) return GBVDB_NOOP;
        launch_apron_faces(ptr<Node>(nodes[0]), ptr<AtlasNode>(amap), atlas_last, ax, ay, ptr<int>(nbr_table),
                           ch[chan].esize, ch[chan].interior.p, ch[chan].apron_buf.p, stream);
        check_launch("apron faces");
        return GBVDB_OK;
    }

    // Compute(effect, chan, iterations, params, bUpdateApron, skipOverAprons, boundval)
    // (VG.cpp:4532-4558) for FUNC_SMOOTH; the pass covers the interior voxels of the
    // assigned slots whatever skipOverAprons says (the reference's smoothing kernel
    // indexes interiors only)
    gbvdb_status compute(int effect, int chan, int iterations, const float* prm, bool upd_apron, float boundval) {
        if (effect != GBVDB_FUNC_SMOOTH) throw StatusError{GBVDB_NOT_SUPPORTED, "Compute: FUNC_SMOOTH only"};
        if (chan < 0 || chan >= 8 || !ch[chan].used || !prm || iterations < 0)
            throw StatusError{GBVDB_INVALID_ARG, "Compute: bad channel or parameters"};
        if (ch[chan].dtype != GBVDB_T_FLOAT) throw StatusError{GBVDB_NOT_SUPPORTED, "Compute: FP32 channels only"};
        if (atlas_last == 0) return GBVDB_NOOP;
        interior_written(chan);
        for (int it = 0; it < iterations; it++) {
            launch_smooth(ptr<AtlasNode>(amap), atlas_last, ptr<float>(ch[chan].interior),
                          ptr<float>(ch[chan].apron_buf), prm[0], prm[1], stream);
            check_launch("smooth");
            if (upd_apron) update_apron(chan, boundval);
        }
        return GBVDB_OK;
    }

    // ------------------------------------------------------- configuration
    gbvdb_status configure(int nlev, const int* ld) {  // Configure (VG.cpp:2380-2434)
        layout_changed();
        if (nlev < 2 || nlev > kMaxLev || !ld) return GBVDB_INVALID_ARG;
        int d[kMaxLev];
        long long rg = 1;
        int lg = 0;
        for (int l = 0; l < nlev; l++) {
            d[l] = ld[l] == 0 ? 1 : ld[l];  // VG.cpp:2394
            if (d[l] < 1 || d[l] > 6) return GBVDB_INVALID_ARG;
            lg += d[l];
            if (lg > 30) return GBVDB_NOT_SUPPORTED;
        }
        lg = 0;
        for (int l = 0; l < nlev; l++) {
            lg += d[l];
            log2dim[l] = d[l];
            res[l] = 1 << d[l];
            rg <<= d[l];
            range[l] = rg;
            lgrange[l] = lg;
        }
        for (int l = nlev; l < kMaxLev; l++) { log2dim[l] = 0; res[l] = 1; range[l] = rg; lgrange[l] = lg; }
        levs = nlev;
        configured = true;
        clear_topology();  // Configure ends with Clear (VG.cpp:2431)
        return GBVDB_OK;
    }

    gbvdb_status add_channel(int chan, int dtype, int apron, int cax, int cay, int caz) {  // VG.cpp:2437-2453
        layout_changed();
        if (!configured) return GBVDB_INVALID_ARG;
        if (chan < 0 || chan >= 8) return GBVDB_INVALID_ARG;
        if (apron != 1) return GBVDB_NOT_SUPPORTED;  // the reference's apron kernels assume 1 (VG.cpp:4448)
        if (log2dim[0] != 4) return GBVDB_NOT_SUPPORTED;
        int es;
        if (dtype == GBVDB_T_FLOAT || dtype == GBVDB_T_UCHAR4) es = 4;
        else if (dtype == GBVDB_T_HALF || dtype == GBVDB_T_BFLOAT16) es = 2;
        else return GBVDB_NOT_SUPPORTED;
        if (cax == 0 && cay == 0 && caz == 0) {  // VG.cpp:2441-2444
            if (chan == 0) { cax = def_ax; cay = def_ay; caz = def_az; }
            else { cax = ax; cay = ay; caz = az; }
        }
        if (cax <= 0 || cay <= 0 || caz <= 0) return GBVDB_INVALID_ARG;
        if (chan == 0) { ax = cax; ay = cay; az = caz; }
        else if (cax != ax || cay != ay) return GBVDB_NOT_SUPPORTED;  // all channels share the slot layout
        Channel& C = ch[chan];
        C.used = true;
        C.dtype = dtype;
        C.apron = apron;
        C.esize = es;
        long long slots = (long long)ax * ay * az;
        // a channel added again keeps its storage when it is large enough
        grow(C.interior, (size_t)slots * 4096 * es);
        grow(C.apron_buf, (size_t)slots * kApronStride * es);
        check(cudaMemsetAsync(C.interior.p, 0, (size_t)slots * 4096 * es, stream), "channel clear");
        check(cudaMemsetAsync(C.apron_buf.p, 0, (size_t)slots * kApronStride * es, stream), "channel clear");
        C.cap_slots = slots;
        return GBVDB_OK;
    }

    // ------------------------------------------------------------------ VBX
    // SaveVBX / LoadVBX (VG.cpp:1626-1767, 507-683; format GVDB_FILESPEC.txt:12-122),
    // version 1.11: header with the grid transform (identity: this path has none), one
    // grid, topology pools (64-byte nodes, res^3 u64 child lists; level 0 has none),
    // then each channel as the reference's atlas volume (ax*18 x ay*18 x az*18 voxels,
    // x fastest) written one 18-slice brick layer at a time.
    struct File {
        FILE* f = nullptr;
        ~File() {
            if (f) fclose(f);
        }
    };
    static void wr(FILE* f, const void* p, size_t n) {
        if (n && fwrite(p, 1, n, f) != n) throw StatusError{GBVDB_INVALID_ARG, "VBX write failed"};
    }
    static void rd(FILE* f, void* p, size_t n) {
        if (n && fread(p, 1, n, f) != n) throw StatusError{GBVDB_INVALID_ARG, "VBX file truncated"};
    }
    template <typename T>
    static void wv(FILE* f, const T& v) { wr(f, &v, sizeof(T)); }
    template <typename T>
    static T rv(FILE* f) {
        T v;
        rd(f, &v, sizeof(T));
        return v;
    }

    int num_channels() const {  // channels 0..k-1 must be in use (the reference's atlas list)
        int k = 0;
        while (k < 8 && ch[k].used) k++;
        return k;
    }

    gbvdb_status save_vbx(const char* path) {
        if (!configured || !path) return GBVDB_INVALID_ARG;
        const int nch = num_channels();
        if (nch == 0) throw StatusError{GBVDB_INVALID_ARG, "SaveVBX needs channel 0"};
        for (int c = nch; c < 8; c++)
            if (ch[c].used) throw StatusError{GBVDB_NOT_SUPPORTED, "SaveVBX needs channels 0..k-1 without gaps"};
        sync();
        File F;
        F.f = fopen(path, "wb");
        if (!F.f) throw StatusError{GBVDB_INVALID_ARG, std::string("cannot open ") + path};
        FILE* f = F.f;
        const uint8_t major = 1, minor = 11;
        wv(f, major);
        wv(f, minor);
        const float pretrans[3] = {0, 0, 0}, angs[3] = {0, 0, 0}, scal[3] = {1, 1, 1}, trans[3] = {0, 0, 0};
        wr(f, pretrans, 12);
        wr(f, angs, 12);
        wr(f, scal, 12);
        wr(f, trans, 12);
        const int num_grids = 1;
        wv(f, num_grids);
        const long table = ftell(f);
        uint64_t goff = 0;
        wv(f, goff);
        goff = (uint64_t)ftell(f);
        char name[256];
        memset(name, 0, sizeof(name));
        wr(f, name, 256);
        wv(f, (uint8_t)'f');  // data type: float (FP16 / BF16 channels carry their own channel type below)
        wv(f, (uint8_t)1);    // components
        wv(f, (uint8_t)0);    // compression
        const float vs[3] = {1, 1, 1};
        wr(f, vs, 12);
        wv(f, (int32_t)ncnt[0]);  // brick count = level-0 pool total
        const int32_t leafdim[3] = {res[0], res[0], res[0]};
        wr(f, leafdim, 12);
        wv(f, (int32_t)1);  // apron
        wv(f, (int32_t)nch);
        const int32_t axisres[3] = {ax * 18, ay * 18, az * 18};
        wv(f, (uint64_t)ch[0].esize * (uint64_t)axisres[0] * (uint64_t)axisres[1] * (uint64_t)axisres[2]);
        wv(f, (uint8_t)2);  // topology: gvdb
        wv(f, (int32_t)0);  // reuse
        wv(f, (uint8_t)0);  // atlas layout
        const int32_t axiscnt[3] = {ax, ay, az};
        wr(f, axiscnt, 12);
        wr(f, axisres, 12);
        wv(f, (int32_t)levs);
        wv(f, (uint64_t)(root_lev >= 0 ? elem(0, root_lev, 0) : kUndefL));
        for (int l = 0; l < levs; l++) {
            wv(f, (int32_t)log2dim[l]);
            wv(f, (int32_t)res[l]);
            const int32_t rg[3] = {(int32_t)range[l], (int32_t)range[l], (int32_t)range[l]};
            wr(f, rg, 12);
            wv(f, (int32_t)ncnt[l]);
            wv(f, (int32_t)sizeof(Node));
            wv(f, (int32_t)(l >= 1 ? ncnt[l] : 0));
            wv(f, (int32_t)(l >= 1 ? cl_len(l) * 8 : 0));
        }
        std::vector<unsigned char> host;
        for (int l = 0; l < levs; l++) {  // pool 0
            size_t bytes = (size_t)ncnt[l] * sizeof(Node);
            host.resize(bytes);
            if (bytes) check(cudaMemcpy(host.data(), nodes[l].p, bytes, cudaMemcpyDeviceToHost), "VBX nodes");
            wr(f, host.data(), bytes);
        }
        for (int l = 1; l < levs; l++) {  // pool 1
            size_t bytes = (size_t)(ncnt[l] * cl_len(l)) * 8;
            host.resize(bytes);
            if (bytes) check(cudaMemcpy(host.data(), clist[l].p, bytes, cudaMemcpyDeviceToHost), "VBX child lists");
            wr(f, host.data(), bytes);
        }
        const size_t slab_elems = (size_t)axisres[0] * axisres[1] * 18;
        for (int c = 0; c < nch; c++) {
            const Channel& C = ch[c];
            wv(f, (int32_t)C.dtype);
            wv(f, (int32_t)C.esize);
            grow(xfer, slab_elems * C.esize);
            host.resize(slab_elems * C.esize);
            // slots past the assigned ones are written as zero (the reference writes whatever its
            // atlas texture holds there)
            const long long valid = std::min<long long>(std::min<long long>(C.cap_slots, atlas_last),
                                                        (long long)ax * ay * az);
            for (int bz = 0; bz < az; bz++) {
                launch_slab_pack(C.interior.p, C.apron_buf.p, C.esize, ax, ay, bz, valid, xfer.p, stream);
                check_launch("VBX slab");
                check(cudaMemcpyAsync(host.data(), xfer.p, host.size(), cudaMemcpyDeviceToHost, stream), "VBX atlas");
                sync();
                wr(f, host.data(), host.size());
            }
        }
        if (fseek(f, table, SEEK_SET) != 0) throw StatusError{GBVDB_INVALID_ARG, "VBX seek failed"};
        wv(f, goff);
        return GBVDB_OK;
    }

    gbvdb_status load_vbx(const char* path) {
        layout_changed();
        if (!path) return GBVDB_INVALID_ARG;
        File F;
        F.f = fopen(path, "rb");
        if (!F.f) throw StatusError{GBVDB_INVALID_ARG, std::string("cannot open ") + path};
        FILE* f = F.f;
        const uint8_t major = rv<uint8_t>(f), minor = rv<uint8_t>(f);
        if ((major == 1 && minor >= 11) || major > 1) {
            float tf[12];
            rd(f, tf, sizeof(tf));  // grid transform: kept by the renderer, not by this path
        }
        const int32_t num_grids = rv<int32_t>(f);
        uint8_t masks = (major == 1 && minor == 0) ? 1 : 0;
        if (major >= 2) masks = rv<uint8_t>(f);
        if (masks) throw StatusError{GBVDB_NOT_SUPPORTED, "VBX with node bitmasks"};
        if (num_grids < 1) throw StatusError{GBVDB_INVALID_ARG, "VBX without grids"};
        std::vector<uint64_t> offs((size_t)num_grids);
        rd(f, offs.data(), offs.size() * 8);
        if (fseek(f, (long)offs[0], SEEK_SET) != 0) throw StatusError{GBVDB_INVALID_ARG, "VBX seek failed"};
        char name[256];
        rd(f, name, 256);
        const uint8_t dt = rv<uint8_t>(f), comps = rv<uint8_t>(f), comp = rv<uint8_t>(f);
        float vs[3];
        rd(f, vs, 12);
        rv<int32_t>(f);  // brick count (= level-0 pool count, read again below)
        int32_t leafdim[3];
        rd(f, leafdim, 12);
        const int32_t apron = rv<int32_t>(f), nch = rv<int32_t>(f);
        rv<uint64_t>(f);  // atlas size
        const uint8_t topo = rv<uint8_t>(f);
        rv<int32_t>(f);  // topology reuse
        const uint8_t layout = rv<uint8_t>(f);
        int32_t axc[3], axr[3];
        rd(f, axc, 12);
        rd(f, axr, 12);
        if (dt != 'f' || comps != 1 || comp != 0 || topo != 2 || layout != 0 || apron != 1 || leafdim[0] != 16 ||
            nch < 1 || nch > 8)
            throw StatusError{GBVDB_NOT_SUPPORTED, "VBX grid: float, 1 component, uncompressed, gvdb topology, atlas "
                                                   "layout, 16^3 bricks with apron 1 only"};
        const int32_t nlev = rv<int32_t>(f);
        const uint64_t root = rv<uint64_t>(f);
        if (nlev < 2 || nlev > kMaxLev) throw StatusError{GBVDB_NOT_SUPPORTED, "VBX level count"};
        int32_t ld[kMaxLev], cnt0[kMaxLev], w0[kMaxLev], cnt1[kMaxLev], w1[kMaxLev];
        for (int l = 0; l < nlev; l++) {
            ld[l] = rv<int32_t>(f);
            rv<int32_t>(f);  // res
            int32_t rg[3];
            rd(f, rg, 12);
            cnt0[l] = rv<int32_t>(f);
            w0[l] = rv<int32_t>(f);
            cnt1[l] = rv<int32_t>(f);
            w1[l] = rv<int32_t>(f);
        }
        gbvdb_status st = configure(nlev, ld);
        if (st != GBVDB_OK) return st;
        for (int l = 0; l < nlev; l++) {
            if (w0[l] != (int)sizeof(Node) || cnt0[l] < 0)
                throw StatusError{GBVDB_NOT_SUPPORTED, "VBX node records are not 64 bytes"};
            if (l == 0 ? (long long)cnt1[0] * w1[0] != 0 : (cnt1[l] != cnt0[l] || w1[l] != cl_len(l) * 8))
                throw StatusError{GBVDB_NOT_SUPPORTED, "VBX child lists do not match the configuration"};
        }
        std::vector<unsigned char> host;
        root_lev = -1;
        for (int l = 0; l < nlev; l++) {
            ensure_pool(l, std::max(cnt0[l], 1));
            size_t bytes = (size_t)cnt0[l] * sizeof(Node);
            host.resize(bytes);
            rd(f, host.data(), bytes);
            long long flagged = 0;
            for (int i = 0; i < cnt0[l]; i++) flagged += host[(size_t)i * sizeof(Node) + 1] != 0;
            if (bytes) check(cudaMemcpy(nodes[l].p, host.data(), bytes, cudaMemcpyHostToDevice), "VBX nodes");
            ncnt[l] = cnt0[l];
            nused[l] = flagged;
            if (root != kUndefL && (int)((root >> 8) & 0xFF) == l && cnt0[l] > 0) {
                Node r;
                memcpy(&r, host.data() + (size_t)(root >> 16) * sizeof(Node), sizeof(Node));
                root_lev = l;
                for (int a = 0; a < 3; a++) root_pos[a] = r.pos[a];
            }
        }
        for (int l = 1; l < nlev; l++) {
            size_t bytes = (size_t)cnt1[l] * (size_t)w1[l];
            host.resize(bytes);
            rd(f, host.data(), bytes);
            if (bytes) check(cudaMemcpy(clist[l].p, host.data(), bytes, cudaMemcpyHostToDevice), "VBX child lists");
        }
        last_depth = root_lev >= 0 ? root_lev : 0;
        def_ax = axc[0];
        def_ay = axc[1];
        def_az = axc[2];
        for (int c = 0; c < 8; c++) ch[c].used = false;
        const size_t slab_elems = (size_t)axr[0] * axr[1] * 18;
        if (axr[0] != axc[0] * 18 || axr[1] != axc[1] * 18 || axr[2] != axc[2] * 18)
            throw StatusError{GBVDB_NOT_SUPPORTED, "VBX atlas resolution is not axiscnt * 18"};
        for (int c = 0; c < nch; c++) {
            const int32_t ctype = rv<int32_t>(f), cstride = rv<int32_t>(f);
            st = add_channel(c, ctype, 1, axc[0], axc[1], axc[2]);
            if (st != GBVDB_OK) return st;
            Channel& C = ch[c];
            if (cstride != C.esize) throw StatusError{GBVDB_NOT_SUPPORTED, "VBX channel stride"};
            grow(xfer, slab_elems * C.esize);
            host.resize(slab_elems * C.esize);
            for (int bz = 0; bz < axc[2]; bz++) {
                rd(f, host.data(), host.size());
                check(cudaMemcpyAsync(xfer.p, host.data(), host.size(), cudaMemcpyHostToDevice, stream), "VBX atlas");
                launch_slab_unpack(xfer.p, C.esize, ax, ay, bz, C.interior.p, C.apron_buf.p, stream);
                check_launch("VBX slab");
                sync();
            }
        }
        return update_atlas();  // LoadVBX ends with UpdateAtlas (VG.cpp:676)
    }
};

// ------------------------------------------------------------------ C ABI

// the kernels an entry point launches, added to the grid's count when it returns
struct LaunchTally {
    long long& total;
    long long t0;
    explicit LaunchTally(long long& t) : total(t), t0(tl_kernels) {}
    ~LaunchTally() { total += tl_kernels - t0; }
};
#define GBVDB_GUARD_NOCOMMIT(g)                           \
    if (!(g)) return GBVDB_INVALID_ARG;                   \
    std::lock_guard<std::mutex> _lk((g)->mu);             \
    LaunchTally _tally((g)->n_launch);                    \
    try {                                                 \
        cudaSetDevice((g)->device);
// topology, binning and accessor entry points commit pending host activations
// (ActivateSpace) first
#define GBVDB_GUARD_NOJOIN(g)                             \
    GBVDB_GUARD_NOCOMMIT(g)                               \
        (g)->host_commit();
// every other entry point also orders the grid's stream after a pending overlapped
// checksum (gbvdb_checksum_overlap)
#define GBVDB_GUARD(g)                                    \
    GBVDB_GUARD_NOJOIN(g)                                 \
        (g)->join_side();
#define GBVDB_END(g)                                      \
    }                                                     \
    catch (const StatusError& e) {                        \
        (g)->err = e.msg;                                 \
        return e.st;                                      \
    }                                                     \
    catch (const std::exception& e) {                     \
        (g)->err = e.what();                              \
        return GBVDB_OUT_OF_MEMORY;                       \
    }

// Grids allocate with cudaMallocAsync from the device's default memory pool.  By
// default that pool returns freed memory to the CUDA driver at every synchronisation,
// so a grid that is rebuilt or replaced pays for fresh driver allocations; keep
// the freed memory in the pool instead (a setting of this process's pool only).
static void keep_pool_memory(int device) {
    static std::mutex mu;
    static bool done[128] = {false};
    std::lock_guard<std::mutex> lk(mu);
    if (device < 0 || device >= 128 || done[device]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    done[device] = true;
}

static float3 f3(const float* v) { return v ? make_float3(v[0], v[1], v[2]) : make_float3(0, 0, 0); }

extern "C" {

gbvdb_status gbvdb_create(int device, gbvdb_grid* out) {
    if (!out) return GBVDB_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return GBVDB_CUDA_ERROR;
    }
    if (cudaSetDevice(device) != cudaSuccess) return GBVDB_CUDA_ERROR;
    keep_pool_memory(device);
    gbvdb_grid g = new (std::nothrow) gbvdb_grid_s();
    if (!g) return GBVDB_OUT_OF_MEMORY;
    g->device = device;
    if (cudaMallocHost(&g->pinned, 1 << 16) != cudaSuccess) {
        delete g;
        return GBVDB_OUT_OF_MEMORY;
    }
    for (int i = 0; i < 64; i++) cudaEventCreate(&g->ev[i]);
    cudaEventCreateWithFlags(&g->rb_ev, cudaEventDisableTiming);
    for (int i = 0; i < 2 * gbvdb_grid_s::kTuneN; i++) cudaEventCreate(&g->tune_ev[i]);
    *out = g;
    return GBVDB_OK;
}

gbvdb_status gbvdb_destroy(gbvdb_grid g) {
    if (!g) return GBVDB_INVALID_ARG;
    cudaSetDevice(g->device);
    DevBuf* bufs[] = {&g->amap, &g->scmap, &g->linked, &g->bin_cnt, &g->bin_off, &g->bin_of, &g->rank_of,
                      &g->sorted, &g->list_cnt, &g->list_off, &g->list_pts, &g->offs_buf, &g->lgrid, &g->touch_dirs, &g->bitmap, &g->pscan,
                      &g->scan_tmp, &g->markers, &g->flags_scan, &g->misc, &g->xfer,
                      &g->link_tag, &g->link_slot, &g->nbr_table, &g->pnode, &g->pndx, &g->gcnt, &g->goff,
                      &g->psort, &g->csum_part, &g->push_bad, &g->nbmask, &g->gtab, &g->sorted_clr,
                      &g->list_clr, &g->khash, &g->thash, &g->ksorted, &g->kalt, &g->ksort_tmp, &g->kmeta};
    g->join_side();
    for (DevBuf* b : bufs) g->release(*b);
    for (int l = 0; l < kMaxLev; l++) { g->release(g->nodes[l]); g->release(g->clist[l]); }
    for (int c = 0; c < 8; c++) { g->release(g->ch[c].interior); g->release(g->ch[c].apron_buf); }
    cudaStreamSynchronize(g->stream);
    if (g->side) cudaStreamDestroy(g->side);
    if (g->side_start) cudaEventDestroy(g->side_start);
    if (g->side_done) cudaEventDestroy(g->side_done);
    for (int i = 0; i < 64; i++) cudaEventDestroy(g->ev[i]);
    if (g->rb_ev) cudaEventDestroy(g->rb_ev);
    for (int i = 0; i < 2 * gbvdb_grid_s::kTuneN; i++) cudaEventDestroy(g->tune_ev[i]);
    cudaFreeHost(g->pinned);
    delete g;
    return GBVDB_OK;
}

gbvdb_status gbvdb_set_stream(gbvdb_grid g, void* stream) {
    GBVDB_GUARD(g)
    g->sync();
    g->stream = reinterpret_cast<cudaStream_t>(stream);
    return GBVDB_OK;
    GBVDB_END(g)
}

const char* gbvdb_last_error(gbvdb_grid g) { return g ? g->err.c_str() : "null grid"; }

gbvdb_status gbvdb_configure(gbvdb_grid g, int levs, const int* log2dim) {
    GBVDB_GUARD(g)
    return g->configure(levs, log2dim);
    GBVDB_END(g)
}

gbvdb_status gbvdb_configure5(gbvdb_grid g, int q4, int q3, int q2, int q1, int q0) {
    int r[5] = {q0, q1, q2, q3, q4};
    return gbvdb_configure(g, 5, r);
}

gbvdb_status gbvdb_set_channel_default(gbvdb_grid g, int ax, int ay, int az) {
    GBVDB_GUARD(g)
    if (ax <= 0 || ay <= 0 || az <= 0) return GBVDB_INVALID_ARG;
    g->def_ax = ax;
    g->def_ay = ay;
    g->def_az = az;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_add_channel(gbvdb_grid g, int chan, int dtype, int apron, int ax, int ay, int az) {
    GBVDB_GUARD(g)
    return g->add_channel(chan, dtype, apron, ax, ay, az);
    GBVDB_END(g)
}

gbvdb_status gbvdb_insert_points(gbvdb_grid g, int64_t n, const float trans[3], int prefix) {
    GBVDB_GUARD(g)
    return g->insert_points(n, f3(trans), prefix != 0);
    GBVDB_END(g)
}

gbvdb_status gbvdb_scatter_density(gbvdb_grid g, int64_t n, float radius, float amp, const float trans[3], int expand,
                                   int avg_color) {
    GBVDB_GUARD(g)
    (void)n; (void)amp; (void)trans;
    return g->scatter_density(radius, expand != 0, avg_color != 0);
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_point_leaves(gbvdb_grid g, int32_t* pnode_out, int64_t cap, int64_t* offsets,
                                       int64_t cap_offsets, float* points, int64_t cap_points) {
    GBVDB_GUARD(g)
    if (g->ins_n < 0) return GBVDB_INVALID_ARG;
    long long n = g->ins_n, nl = g->ins_nleaf;
    if ((pnode_out && cap < n) || (offsets && cap_offsets < nl + 1)) return GBVDB_CAPACITY;
    if (pnode_out && n)
        g->check(cudaMemcpyAsync(pnode_out, g->pnode.p, (size_t)n * 4, cudaMemcpyDeviceToHost, g->stream), "export");
    std::vector<uint32_t> off((size_t)nl + 1, 0);
    g->check(cudaMemcpyAsync(off.data(), g->goff.p, (size_t)(nl + 1) * 4, cudaMemcpyDeviceToHost, g->stream), "export");
    g->sync();
    if (offsets)
        for (long long i = 0; i <= nl; i++) offsets[i] = off[(size_t)i];
    long long tot = off[(size_t)nl];
    if (points) {
        if (cap_points < tot * 3) return GBVDB_CAPACITY;
        if (tot)
            g->check(cudaMemcpyAsync(points, g->psort.p, (size_t)tot * 12, cudaMemcpyDeviceToHost, g->stream), "export");
        g->sync();
    }
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_update_neighbors(gbvdb_grid g) {
    GBVDB_GUARD(g)
    return g->update_neighbors();
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_neighbors(gbvdb_grid g, int32_t* host_out, int64_t cap) {
    GBVDB_GUARD(g)
    if (!host_out || g->nbr_count < 0) return GBVDB_INVALID_ARG;
    if (cap < g->nbr_count * 6) return GBVDB_CAPACITY;
    if (g->nbr_count == 0) return GBVDB_OK;
    g->check(cudaMemcpyAsync(host_out, g->nbr_table.p, (size_t)g->nbr_count * 24, cudaMemcpyDeviceToHost, g->stream),
             "export neighbors");
    g->sync();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_update_apron_faces(gbvdb_grid g, int chan) {
    GBVDB_GUARD(g)
    return g->update_apron_faces(chan);
    GBVDB_END(g)
}

gbvdb_status gbvdb_compute(gbvdb_grid g, int effect, int chan, int iterations, const float params[3], int update_apron,
                           int skip_aprons, float boundval) {
    GBVDB_GUARD(g)
    (void)skip_aprons;
    return g->compute(effect, chan, iterations, params, update_apron != 0, boundval);
    GBVDB_END(g)
}

gbvdb_status gbvdb_save_vbx(gbvdb_grid g, const char* path) {
    GBVDB_GUARD(g)
    return g->save_vbx(path);
    GBVDB_END(g)
}

gbvdb_status gbvdb_load_vbx(gbvdb_grid g, const char* path) {
    GBVDB_GUARD(g)
    return g->load_vbx(path);
    GBVDB_END(g)
}

gbvdb_status gbvdb_set_points(gbvdb_grid g, const void* pos, int64_t n, int off, int stride, const void* vel,
                              int vel_off, int vel_stride, const void* clr, int clr_off, int clr_stride) {
    GBVDB_GUARD_NOJOIN(g)
    (void)vel_off; (void)vel_stride;
    if ((!pos && n > 0) || n < 0 || stride < 12 || off < 0 || (off % 4) || (stride % 4)) return GBVDB_INVALID_ARG;
    if (clr && (clr_off < 0 || clr_stride < 4 || (clr_off % 4) || (clr_stride % 4))) return GBVDB_INVALID_ARG;
    g->pts.base = reinterpret_cast<const char*>(pos);
    g->pts.n = n;
    g->pts.off = off;
    g->pts.stride = stride;
    g->vel = vel;
    g->clr = ClrSrc{reinterpret_cast<const char*>(clr), clr ? clr_stride : 4, clr ? clr_off : 0};
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_activate_space(gbvdb_grid g, const float pos[3], uint64_t* out_node) {
    GBVDB_GUARD_NOCOMMIT(g)
    if (!pos) return GBVDB_INVALID_ARG;
    g->host_begin();
    const int32_t v[3] = {(int32_t)pos[0], (int32_t)pos[1], (int32_t)pos[2]};  // Vector3DI(Vector3DF) truncates
    const uint64_t id = g->host->activate_space(v);
    g->host_dirty = true;
    if (out_node) *out_node = id;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_rebuild_topology_cpu(gbvdb_grid g, int64_t n, const float orig[3], const void* host_pos,
                                        int stride) {
    GBVDB_GUARD_NOCOMMIT(g)
    if (n < 0 || (n > 0 && !host_pos) || (stride != 0 && stride < 12)) return GBVDB_INVALID_ARG;
    if (stride == 0) stride = 12;
    g->host_begin();
    const float o[3] = {orig ? orig[0] : 0.0f, orig ? orig[1] : 0.0f, orig ? orig[2] : 0.0f};
    const char* base = static_cast<const char*>(host_pos);
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        memcpy(p, base + i * (int64_t)stride, 12);
        const int32_t v[3] = {(int32_t)(p[0] + o[0]), (int32_t)(p[1] + o[1]), (int32_t)(p[2] + o[2])};
        g->host->activate_space(v);
    }
    g->host_dirty = true;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_rebuild_topology(gbvdb_grid g, int64_t n, float radius, const float orig[3]) {
    GBVDB_GUARD_NOJOIN(g)
    g->nbr_count = -1;  // the neighbour table and point groups describe the previous topology
    g->ins_n = -1;
    return g->rebuild(n, radius, f3(orig), false, 0);
    GBVDB_END(g)
}

gbvdb_status gbvdb_accumulate_topology(gbvdb_grid g, int64_t n, float radius, const float orig[3], int min_depth) {
    GBVDB_GUARD_NOJOIN(g)
    g->nbr_count = -1;
    g->ins_n = -1;
    return g->rebuild(n, radius, f3(orig), true, min_depth);
    GBVDB_END(g)
}

gbvdb_status gbvdb_request_full_rebuild(gbvdb_grid g, int tf) {
    GBVDB_GUARD_NOJOIN(g)
    g->rebuild_topo = tf ? 1 : 0;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_finish_topology(gbvdb_grid g, int commit_pool, int compute_bounds) {
    GBVDB_GUARD_NOJOIN(g)
    (void)commit_pool;  // pools live on the device only; nothing to commit
    if (compute_bounds && g->ncnt[0] > 0) {  // ComputeBounds (VG.cpp:1792-1816)
        g->grow(g->misc, 256);
        int* d6 = g->ptr<int>(g->misc) + 16;
        launch_leaf_bounds(g->ptr<Node>(g->nodes[0]), g->ncnt[0], g->lgrange[0], d6, g->stream);
        g->check_launch("bounds");
        g->readback(g->bounds, d6, sizeof(g->bounds));
        g->bounds_valid = true;
    }
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_update_atlas(gbvdb_grid g) {
    GBVDB_GUARD_NOJOIN(g)  // joins an overlapped checksum only when the atlas grows (resize_channels)
    return g->update_atlas();
    GBVDB_END(g)
}

gbvdb_status gbvdb_insert_points_subcell(gbvdb_grid g, int sc, int64_t n, float radius, const float trans[3],
                                         int64_t* out_len) {
    GBVDB_GUARD_NOJOIN(g)
    long long len = 0;
    gbvdb_status st = g->insert_subcell(sc, n, radius, f3(trans), &len);
    if (st == GBVDB_OK && out_len) *out_len = len;
    return st;
    GBVDB_END(g)
}

gbvdb_status gbvdb_insert_points_subcell_fp16(gbvdb_grid g, int sc, int64_t n, float radius, const float trans[3],
                                              int64_t* out_len) {
    GBVDB_GUARD_NOJOIN(g)
    long long len = 0;
    gbvdb_status st = g->insert_subcell(sc, n, radius, f3(trans), &len, true);
    if (st == GBVDB_OK && out_len) *out_len = len;
    return st;
    GBVDB_END(g)
}

gbvdb_status gbvdb_gather_levelset_fp16(gbvdb_grid g, int sc, int64_t n, float radius, const float trans[3],
                                        int64_t sc_len, int chan, int clr_chan) {
    GBVDB_GUARD(g)
    (void)n; (void)trans;
    return g->gather(1, sc, radius, sc_len, chan, clr_chan, false);
    GBVDB_END(g)
}

gbvdb_status gbvdb_gather_density(gbvdb_grid g, int sc, int64_t n, float radius, const float trans[3], int64_t sc_len,
                                  int chan, int clr_chan, int accum) {
    GBVDB_GUARD(g)
    (void)n; (void)trans;
    return g->gather(0, sc, radius, sc_len, chan, clr_chan, accum != 0);
    GBVDB_END(g)
}

gbvdb_status gbvdb_gather_levelset(gbvdb_grid g, int sc, int64_t n, float radius, const float trans[3],
                                   int64_t sc_len, int chan, int clr_chan, int accum) {
    GBVDB_GUARD(g)
    (void)n; (void)trans;
    return g->gather(1, sc, radius, sc_len, chan, clr_chan, accum != 0);
    GBVDB_END(g)
}

gbvdb_status gbvdb_update_apron(gbvdb_grid g, int chan, float boundval) {
    GBVDB_GUARD(g)
    return g->update_apron(chan, boundval);
    GBVDB_END(g)
}

gbvdb_status gbvdb_fill_channel4(gbvdb_grid g, int chan, const float value[4]) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !value) return GBVDB_INVALID_ARG;
    Channel& C = g->ch[chan];
    g->interior_written(chan);
    // every slot of the atlas, interior and apron (the reference's FUNC_FILL_* pass over
    // the whole atlas volume, VG.cpp:2456-2470, OP.cuh:353-380)
    const long long slots = std::min<long long>(C.cap_slots, (long long)g->ax * g->ay * g->az);
    uint32_t bb;
    if (C.dtype == GBVDB_T_UCHAR4) {  // CLR2INT(make_float4(p1, p2, p3, 1.0)) (OP.cuh:20, 372)
        bb = ((uint32_t)(1.0f * 255.0f) << 24) | ((uint32_t)(value[2] * 255.0f) << 16) |
             ((uint32_t)(value[1] * 255.0f) << 8) | (uint32_t)(value[0] * 255.0f);
    } else {
        bb = g->storage_bits(chan, value[0]);
        if (C.esize == 2) bb |= bb << 16;
    }
    launch_fill_u32(g->ptr<uint32_t>(C.interior), slots * 4096 * C.esize / 4, bb, g->stream);
    launch_fill_u32(g->ptr<uint32_t>(C.apron_buf), slots * kApronStride * C.esize / 4, bb, g->stream);
    g->check_launch("fill");
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_fill_channel(gbvdb_grid g, int chan, float value) {
    const float v[4] = {value, 0.0f, 0.0f, 0.0f};
    return gbvdb_fill_channel4(g, chan, v);
}

gbvdb_status gbvdb_clear_channel(gbvdb_grid g, int chan) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used) return GBVDB_INVALID_ARG;
    Channel& C = g->ch[chan];
    g->interior_written(chan);
    const size_t slots = (size_t)C.cap_slots;
    g->check(cudaMemsetAsync(C.interior.p, 0, slots * 4096 * C.esize, g->stream), "clear channel");
    g->check(cudaMemsetAsync(C.apron_buf.p, 0, slots * kApronStride * C.esize, g->stream), "clear channel");
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_depth(gbvdb_grid g, int* depth, int* top_lev) {
    GBVDB_GUARD_NOJOIN(g)
    if (depth) *depth = g->last_depth;
    if (top_lev) *top_lev = g->top_lev();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_node_counts(gbvdb_grid g, int64_t* total, int64_t* used) {
    GBVDB_GUARD_NOJOIN(g)
    for (int l = 0; l < kMaxLev; l++) {
        if (total) total[l] = g->ncnt[l];
        if (used) {
            if (l == 0) g->refresh_nused0();
            used[l] = g->nused[l];
        }
    }
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_vol_bounds(gbvdb_grid g, float* out6) {
    GBVDB_GUARD_NOJOIN(g)
    if (!out6) return GBVDB_INVALID_ARG;
    if (!g->bounds_valid) return GBVDB_NOOP;
    for (int a = 0; a < 6; a++) out6[a] = (float)g->bounds[a];
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_point_bounds(gbvdb_grid g, float* out6) {
    GBVDB_GUARD_NOJOIN(g)
    if (!out6) return GBVDB_INVALID_ARG;
    for (int a = 0; a < 3; a++) { out6[a] = g->posmin[a]; out6[3 + a] = g->posmax[a]; }
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_nodes(gbvdb_grid g, int lev, void* host_out, int64_t cap) {
    GBVDB_GUARD_NOJOIN(g)
    if (lev < 0 || lev >= kMaxLev || !host_out) return GBVDB_INVALID_ARG;
    if (cap < g->ncnt[lev]) return GBVDB_CAPACITY;
    if (g->ncnt[lev] == 0) return GBVDB_OK;
    g->check(cudaMemcpyAsync(host_out, g->nodes[lev].p, (size_t)g->ncnt[lev] * sizeof(Node), cudaMemcpyDeviceToHost,
                             g->stream), "export nodes");
    g->sync();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_childlist(gbvdb_grid g, int lev, uint64_t* host_out, int64_t cap) {
    GBVDB_GUARD_NOJOIN(g)
    if (lev < 1 || lev >= g->levs || !host_out) return GBVDB_INVALID_ARG;
    long long n = g->ncnt[lev] * g->cl_len(lev);
    if (cap < n) return GBVDB_CAPACITY;
    if (n == 0) return GBVDB_OK;
    g->check(cudaMemcpyAsync(host_out, g->clist[lev].p, (size_t)n * 8, cudaMemcpyDeviceToHost, g->stream),
             "export childlist");
    g->sync();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_atlas_info(gbvdb_grid g, int chan, int* info) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !info || !g->ch[chan].used) return GBVDB_INVALID_ARG;
    info[0] = g->ax; info[1] = g->ay; info[2] = g->az; info[3] = g->atlas_last;
    info[4] = g->ch[chan].dtype; info[5] = g->ch[chan].apron; info[6] = kPad; info[7] = g->ch[chan].esize;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_atlas_bricks(gbvdb_grid g, int chan, void* host_out, int64_t cap_bytes) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !host_out) return GBVDB_INVALID_ARG;
    Channel& C = g->ch[chan];
    long long bytes = (long long)g->atlas_last * 5832 * C.esize;
    if (cap_bytes < bytes) return GBVDB_CAPACITY;
    if (bytes == 0) return GBVDB_OK;
    g->grow(g->xfer, (size_t)bytes);
    launch_export_bricks(C.interior.p, C.apron_buf.p, g->atlas_last, C.esize, g->xfer.p, g->stream);
    g->check_launch("export bricks");
    g->check(cudaMemcpyAsync(host_out, g->xfer.p, (size_t)bytes, cudaMemcpyDeviceToHost, g->stream), "export atlas");
    g->sync();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_atlas_map(gbvdb_grid g, void* host_out, int64_t cap) {
    GBVDB_GUARD(g)
    if (!host_out) return GBVDB_INVALID_ARG;
    if (cap < g->amap_slots) return GBVDB_CAPACITY;
    if (g->amap_slots == 0) return GBVDB_OK;
    g->check(cudaMemcpyAsync(host_out, g->amap.p, (size_t)g->amap_slots * 16, cudaMemcpyDeviceToHost, g->stream),
             "export map");
    g->sync();
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_export_subcells(gbvdb_grid g, int64_t* offsets, int64_t cap_offsets, float* points,
                                   int64_t cap_points) {
    GBVDB_GUARD(g)
    if (!g->sc_valid) return GBVDB_INVALID_ARG;
    long long nsub = g->sc_nbricks * 64;
    if (cap_offsets < nsub + 1 || cap_points < g->sc_len) return GBVDB_CAPACITY;
    g->materialize_lists();
    std::vector<uint32_t> off((size_t)nsub + 1);
    g->check(cudaMemcpyAsync(off.data(), g->list_off.p, (size_t)(nsub + 1) * 4, cudaMemcpyDeviceToHost, g->stream),
             "export offsets");
    if (g->sc_len > 0 && points)
        g->check(cudaMemcpyAsync(points, g->list_pts.p, (size_t)g->sc_len * 12, cudaMemcpyDeviceToHost, g->stream),
                 "export points");
    g->sync();
    if (offsets)
        for (long long i = 0; i <= nsub; i++) offsets[i] = off[(size_t)i];
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_checksum(gbvdb_grid g, int chan, double* out) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !out) return GBVDB_INVALID_ARG;
    if (g->ch[chan].dtype == GBVDB_T_UCHAR4) return GBVDB_NOT_SUPPORTED;  // sums of float channels only
    g->grow(g->misc, 256);
    g->grow(g->xfer, (size_t)std::max(g->atlas_last, 1) * 8);
    double* d = reinterpret_cast<double*>(g->ptr<char>(g->misc) + 192);
    launch_checksum_slots(g->ptr<AtlasNode>(g->amap), g->atlas_last, g->ch[chan].dtype, g->ch[chan].interior.p,
                          g->ptr<double>(g->xfer), d, g->stream);
    g->check_launch("checksum");
    g->readback(out, d, 8);
    return GBVDB_OK;
    GBVDB_END(g)
}

// gbvdb_checksum without the readback: the sum goes to a device pointer on the grid's
// stream, so a pipelined caller reads it back when it likes (no host synchronisation)
gbvdb_status gbvdb_checksum_device(gbvdb_grid g, int chan, double* dev_out) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !dev_out) return GBVDB_INVALID_ARG;
    if (g->ch[chan].dtype == GBVDB_T_UCHAR4) return GBVDB_NOT_SUPPORTED;  // sums of float channels only
    g->grow(g->csum_part, (size_t)std::max(g->atlas_last, 1) * 8);
    launch_checksum_slots(g->ptr<AtlasNode>(g->amap), g->atlas_last, g->ch[chan].dtype, g->ch[chan].interior.p,
                          g->ptr<double>(g->csum_part), dev_out, g->stream);
    g->check_launch("checksum");
    return GBVDB_OK;
    GBVDB_END(g)
}

// the checksum on the grid's side stream: ordered after the grid's work so far, while
// the grid's stream goes on; the next entry point that writes interiors waits for it
gbvdb_status gbvdb_checksum_overlap(gbvdb_grid g, int chan, double* dev_out, double* host_out) {
    GBVDB_GUARD(g)  // joins a previous overlapped checksum (its partials are reused)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !dev_out) return GBVDB_INVALID_ARG;
    if (g->ch[chan].dtype == GBVDB_T_UCHAR4) return GBVDB_NOT_SUPPORTED;
    if (!g->side) {
        g->check(cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking), "side stream");
        g->check(cudaEventCreateWithFlags(&g->side_start, cudaEventDisableTiming), "side event");
        g->check(cudaEventCreateWithFlags(&g->side_done, cudaEventDisableTiming), "side event");
    }
    g->grow(g->csum_part, (size_t)std::max(g->atlas_last, 1) * 8);
    g->check(cudaEventRecord(g->side_start, g->stream), "side event");
    g->check(cudaStreamWaitEvent(g->side, g->side_start, 0), "side wait");
    // the atlas map is not read (UpdateAtlas assigns slots 0 .. atlas_last - 1), so the
    // next frame's UpdateAtlas may rewrite it while this runs; the interiors are waited
    // for by their next writer (a gather, a fill, or an atlas that grows)
    // On two blocks per SM: the sum then streams the interiors over the next frame's
    // topology, atlas and binning instead of taking the memory system ahead of their
    // latency-bound kernels (fluid frame e2e: 1.150 -> 1.107 ms per step; four blocks
    // 1.117, one 1.192, when the gather has to wait for it)
    launch_checksum_slots(nullptr, g->atlas_last, g->ch[chan].dtype, g->ch[chan].interior.p,
                          g->ptr<double>(g->csum_part), dev_out, g->side, 2);
    g->check_launch("checksum");
    if (host_out) g->check(cudaMemcpyAsync(host_out, dev_out, 8, cudaMemcpyDeviceToHost, g->side), "checksum copy");
    g->check(cudaEventRecord(g->side_done, g->side), "side event");
    g->side_pending = true;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_join(gbvdb_grid g) {
    GBVDB_GUARD(g)
    return GBVDB_OK;
    GBVDB_END(g)
}

// Allocation-free variant of gbvdb_checksum: see include/gbvdb.h.  It reads the
// grid's atlas and writes one double to dev_out on the grid's stream; its
// scratch is the static per-slot array in atlas.cu, so it calls no allocator.
gbvdb_status gbvdb_checksum_noalloc(gbvdb_grid g, int chan, double* dev_out) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used || !dev_out) return GBVDB_INVALID_ARG;
    if (g->ch[chan].dtype == GBVDB_T_UCHAR4) return GBVDB_NOT_SUPPORTED;  // sums of float channels only
    if (g->atlas_last > noalloc_max_slots()) {
        g->err = "checksum_noalloc: " + std::to_string(g->atlas_last) + " atlas slots exceed the static scratch limit of " +
                 std::to_string(noalloc_max_slots()) + " slots";
        return GBVDB_CAPACITY;
    }
    cudaError_t e = checksum_noalloc(g->ptr<AtlasNode>(g->amap), g->atlas_last, g->ch[chan].dtype,
                                     g->ch[chan].interior.p, dev_out, g->stream);
    if (e != cudaSuccess) {
        g->err = std::string("checksum_noalloc: ") + cudaGetErrorString(e);
        return GBVDB_CUDA_ERROR;
    }
    g->check_launch("checksum_noalloc");
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_vdb_info(gbvdb_grid g, void* host_out, int64_t bytes) {
    GBVDB_GUARD(g)
    if (!host_out || bytes < (int64_t)sizeof(gbvdb_vdb_info)) return GBVDB_INVALID_ARG;
    g->refresh_nused0();
    // a consumer may write the interiors through these pointers at any time, so every
    // later UpdateApron copies the interiors as they are (as with gbvdb_get_atlas_device)
    g->fused_apron = false;
    gbvdb_vdb_info v;
    memset(&v, 0, sizeof(v));
    for (int n = 0; n < g->levs && n < 10; n++) {  // PrepareVDB (VG.cpp:3946-3989)
        v.dim[n] = g->log2dim[n];
        v.res[n] = g->res[n];
        const float rg = (float)g->range[n];
        v.vdel[n] = make_float3(rg / (float)g->res[n], rg / (float)g->res[n], rg / (float)g->res[n]);
        v.noderange[n] = make_int3((int)g->range[n], (int)g->range[n], (int)g->range[n]);
        v.nodecnt[n] = (int)g->ncnt[n];
        v.nodewid[n] = (int)sizeof(Node);
        v.childwid[n] = (int)(g->cl_len(n) * 8);
        v.nodelist[n] = g->ptr<char>(g->nodes[n]);
        v.childlist[n] = g->ptr<char>(g->clist[n]);
    }
    v.atlas_map = g->ptr<gbvdb_atlas_node>(g->amap);
    v.atlas_cnt = make_int3(g->ax, g->ay, g->az);
    v.atlas_res = make_int3(g->ax * kPad, g->ay * kPad, g->az * kPad);
    v.atlas_apron = 1;
    v.brick_res = kPad;
    for (int c = 0; c < 8; c++) {
        if (!g->ch[c].used) continue;
        v.apron_table[c] = g->ch[c].esize;
        v.volIn[c] = (unsigned long long)(uintptr_t)g->ch[c].interior.p;
        v.volOut[c] = (unsigned long long)(uintptr_t)g->ch[c].apron_buf.p;
    }
    v.top_lev = g->top_lev();
    v.clr_chan = 255;  // CHAN_UNDEF
    if (g->bounds_valid) {
        v.bmin = make_float3((float)g->bounds[0], (float)g->bounds[1], (float)g->bounds[2]);
        v.bmax = make_float3((float)g->bounds[3], (float)g->bounds[4], (float)g->bounds[5]);
    }
    memcpy(host_out, &v, sizeof(v));
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_atlas_device(gbvdb_grid g, int chan, void** interior, void** apron) {
    GBVDB_GUARD(g)
    if (chan < 0 || chan >= 8 || !g->ch[chan].used) return GBVDB_INVALID_ARG;
    if (interior) *interior = g->ch[chan].interior.p;
    if (apron) *apron = g->ch[chan].apron_buf.p;
    // the caller may write the interior at any time from now on: every UpdateApron
    // of this grid copies the interiors as they are (no fused apron)
    g->fused_apron = false;
    for (int c = 0; c < 8; c++) g->interior_written(c);
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_set_tuning(gbvdb_grid g, int param, int64_t value) {
    GBVDB_GUARD(g)
    if (param == GBVDB_TUNE_DENSE_MIN) {
        if (value < 0 || value > (1ll << 31)) return GBVDB_INVALID_ARG;
        g->dense_min = (int)value;
        g->tune_auto = false;  // an explicit threshold ends the autotuner
        g->tune_pending = false;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_AUTOTUNE) {
        if (value != 0 && value != 1) return GBVDB_INVALID_ARG;
        g->tune_auto = value != 0;
        g->tune_pending = false;
        g->tune_step = gbvdb_grid_s::kTuneN;
        g->tune_bricks = -1;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_FUSED_APRON) {
        if (value != 0 && value != 1) return GBVDB_INVALID_ARG;
        g->fused_apron = value != 0;
        for (int c = 0; c < 8; c++) g->interior_written(c);
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_TOUCH_DIRS) {
        if (value != 0 && value != 1) return GBVDB_INVALID_ARG;
        g->touch_dirs_on = value != 0;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_GATHER_LONG_MIN) {
        if (value < -1 || value > (1ll << 30)) return GBVDB_INVALID_ARG;
        g->gather_long_min_set = (int)value;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_KEYSET) {
        if (value < 0 || value > 2) return GBVDB_INVALID_ARG;
        g->keyset_mode = (int)value;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_TABLE) {
        if (value != 0 && value != 1) return GBVDB_INVALID_ARG;
        g->table_on = value != 0;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_BIN_UNROLL) {
        if (value != 0 && value != 1 && value != 2 && value != 4) return GBVDB_INVALID_ARG;
        g->bin_unroll_set = value ? (int)value : -1;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_SCATTER_UNROLL) {
        if (value != 0 && value != 2 && value != 4 && value != 8) return GBVDB_INVALID_ARG;
        g->scatter_unroll_set = value ? (int)value : -1;
        return GBVDB_OK;
    }
    if (param == GBVDB_TUNE_GATHER_BLOCKS) {
        if (value != 0 && value != 8 && value != 10) return GBVDB_INVALID_ARG;
        g->gather_blocks_set = value ? (int)value : -1;
        return GBVDB_OK;
    }
    return GBVDB_INVALID_ARG;
    GBVDB_END(g)
}

const char* gbvdb_tune_table_source(void) { return tune_table().source.c_str(); }

gbvdb_status gbvdb_set_profile(gbvdb_grid g, int enable) {
    GBVDB_GUARD_NOJOIN(g)
    g->profile = enable != 0;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_stats(gbvdb_grid g, int64_t* out4) {
    GBVDB_GUARD_NOJOIN(g)
    if (!out4) return GBVDB_INVALID_ARG;
    out4[0] = g->n_launch;
    out4[1] = g->n_readback;
    out4[2] = g->sc_len;
    out4[3] = g->sc_nbricks;
    return GBVDB_OK;
    GBVDB_END(g)
}

gbvdb_status gbvdb_get_stats_ex(gbvdb_grid g, int64_t* out, int cap) {
    GBVDB_GUARD_NOJOIN(g)
    if (!out || cap < 0) return GBVDB_INVALID_ARG;
    const int64_t v[5] = {g->n_launch, g->n_readback, g->sc_len, g->sc_nbricks, g->n_hashed_passes};
    for (int i = 0; i < cap && i < 5; i++) out[i] = v[i];
    return GBVDB_OK;
    GBVDB_END(g)
}

// device bytes held by the grid's buffers (pools, atlas, scratch): the server's memory accounting
size_t gbvdb_internal_device_bytes(gbvdb_grid g);
gbvdb_status gbvdb_get_device_bytes(gbvdb_grid g, int64_t* out) {
    if (!g || !out) return GBVDB_INVALID_ARG;
    *out = (int64_t)gbvdb_internal_device_bytes(g);
    return GBVDB_OK;
}

size_t gbvdb_internal_device_bytes(gbvdb_grid g) {
    if (!g) return 0;
    std::lock_guard<std::mutex> lk(g->mu);
    size_t b = 0;
    const DevBuf* bufs[] = {&g->amap, &g->scmap, &g->linked, &g->bin_cnt, &g->bin_off, &g->bin_of, &g->rank_of,
                            &g->sorted, &g->sorted_clr, &g->list_cnt, &g->list_off, &g->list_pts, &g->list_clr,
                            &g->offs_buf, &g->lgrid,
                            &g->touch_dirs, &g->bitmap, &g->pscan, &g->scan_tmp, &g->markers,
                            &g->flags_scan, &g->misc, &g->xfer, &g->link_tag, &g->link_slot, &g->nbr_table,
                            &g->pnode, &g->pndx, &g->gcnt, &g->goff, &g->psort, &g->csum_part, &g->push_bad,
                            &g->nbmask, &g->gtab, &g->khash, &g->thash, &g->ksorted, &g->kalt, &g->ksort_tmp,
                            &g->kmeta};
    for (const DevBuf* d : bufs) b += d->cap;
    for (int l = 0; l < kMaxLev; l++) b += g->nodes[l].cap + g->clist[l].cap;
    for (int c = 0; c < 8; c++) b += g->ch[c].interior.cap + g->ch[c].apron_buf.cap;
    return b;
}

gbvdb_status gbvdb_get_stage_times(gbvdb_grid g, double* ms, int cap) {
    GBVDB_GUARD_NOJOIN(g)
    if (!ms) return GBVDB_INVALID_ARG;
    int n = std::min<int>(cap, (int)g->stage_ms.size());
    for (int i = 0; i < n; i++) ms[i] = g->stage_ms[(size_t)i];
    for (int i = n; i < cap; i++) ms[i] = -1;
    return GBVDB_OK;
    GBVDB_END(g)
}

}  // extern "C"
