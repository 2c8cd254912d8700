// ref_harness.cu -- runs the REFERENCE's own CUDA kernels (PTX compiled from the
// reference's kernels/cuda_gvdb_module.cu by oracle/ref_build.py into
// oracle/_ref/) under a restatement of VolumeGVDB's host orchestration for the
// point-driven path.
//
// TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py (fixtures that
// pin the CPU oracle to the reference's kernels) and to time the reference's
// CUDA path.  It never links into the product library.
//
// Host logic restated from source/gvdb_library/src/gvdb_volume_gvdb.cpp
// (VG.cpp) and gvdb_allocator.cpp (AL.cpp):
//   RebuildTopology 1181-1218, ActivateBricksGPU 1229-1413, ActivateExtraBricksGPU
//   931-1016, ActivateIncreBricksGPU 1020-1156, RadixSortByByte 904-928 (thrust::sort
//   as gvdb_cutils.cu:11-16), FindUniqueBrick 843-873, PrefixSum 4760-4819,
//   GetBoundingBox 5404-5467 (thrust min/max as gvdb_cutils.cu:22-39),
//   PrepareVDB 3946-3994, UpdateAtlas 2630-2704, InsertPointsSubcell 4971-5092,
//   GatherDensity/LevelSet 5318-5373, UpdateApron 4418-4457; pools AL.cpp:55-192,
//   atlas AL.cpp:311-456, 528-715.
// Inputs must keep every box / subcell position inside the root and >= 0: the
// reference kernels index child lists and subcell counters without bounds checks
// there, and such an index would address memory outside the buffers.
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/extrema.h>
#include <thrust/sort.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define MAXLEV 10
#define UNDEFL 0xFFFFFFFFull
#define UNDEF64 0xFFFFFFFFFFFFFFFFull

// layout of VDBInfo as declared for the device (cuda_gvdb_nodes.cuh:42-67)
struct alignas(16) HVDBInfo {
    int dim[MAXLEV];
    int res[MAXLEV];
    float vdel[MAXLEV][3];
    int noderange[MAXLEV][3];
    int nodecnt[MAXLEV];
    int nodewid[MAXLEV];
    int childwid[MAXLEV];
    unsigned long long nodelist[MAXLEV];
    unsigned long long childlist[MAXLEV];
    unsigned long long atlas_map;
    int atlas_cnt[3];
    int atlas_res[3];
    int atlas_apron;
    int brick_res;
    int apron_table[8];
    int top_lev;
    int max_iter;
    float epsilon;
    bool update;
    unsigned char clr_chan;
    float bmin[3];
    float bmax[3];
    unsigned long long volIn[32];
    unsigned long long volOut[32];
};
static_assert(offsetof(HVDBInfo, nodelist) == 440, "VDBInfo layout");
static_assert(offsetof(HVDBInfo, atlas_map) == 600, "VDBInfo layout");
static_assert(offsetof(HVDBInfo, bmin) == 688, "VDBInfo layout");
static_assert(offsetof(HVDBInfo, volIn) == 712, "VDBInfo layout");
static_assert(offsetof(HVDBInfo, volOut) == 968, "VDBInfo layout");

struct HNode {  // gvdb_node.h:27-40
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    uint64_t parent, childlist, mask;
};
static_assert(sizeof(HNode) == 64, "node");

struct Pool {  // AL.cpp:55-192
    std::vector<char> cpu;
    CUdeviceptr gpu = 0;
    size_t stride = 0, lastEle = 0, usedNum = 0, max = 0;
};

static uint64_t Elem(int grp, int lev, uint64_t ndx) { return (uint64_t)grp | ((uint64_t)lev << 8) | (ndx << 16); }

struct Harness {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    std::string err;
    int levs = 0;
    int logdim[MAXLEV] = {0};
    Pool pool[2][MAXLEV];
    HVDBInfo info{};
    CUdeviceptr cuinfo = 0;
    bool rebuild = true;
    int curr_depth = -1;
    float posmin[3], posmax[3], posrange[3];
    bool fp16_lists = false;  // the last insert was InsertPointsSubcell_FP16 (ushort3 lists)
    // legacy InsertPoints / ScatterDensity buffers
    CUdeviceptr pnode = 0, pndx = 0, gcnt = 0, goff = 0, psort = 0;
    CUdeviceptr nbr = 0;
    // points
    CUdeviceptr pts = 0;
    int npts = 0;
    // atlas: channel 0 T_FLOAT, channel 1 T_UCHAR4 (colour, created on request)
    int ax = 16, ay = 16, az = 1;
    int atlas_last = 0;
    CUarray arr = nullptr, carr = nullptr;
    CUsurfObject surf = 0, csurf = 0;
    bool colour_chan = false;
    CUdeviceptr clr = 0;  // point colours (uint per point), 0 = none
    CUdeviceptr sc_clr = 0;
    CUdeviceptr amap = 0;
    size_t amap_cnt = 0;
    std::vector<int32_t> amap_cpu;
    // aux
    CUdeviceptr keys = 0, sorted = 0, marker = 0, presum = 0, cnt = 0, levcnt = 0, uniq = 0, range_res = 0;
    CUdeviceptr node_mk = 0;  // AUX_NODE_MARKER (separate from the unique pass's AUX_MARKER)
    size_t keys_bytes = 0;
    CUdeviceptr sc_flag = 0, sc_map = 0, sc_cnt = 0, sc_off = 0, sc_pnts = 0, sc_pos = 0, sc_nid = 0;
    int sc_num = 0;
    int sc_len = 0;
    CUdeviceptr scanA1 = 0, scanS1 = 0, scanA2 = 0, scanS2 = 0;
    CUdeviceptr bbx = 0, bby = 0, bbz = 0, bbox = 0;
    size_t bb_cap = 0;
    CUevent ev0 = nullptr, ev1 = nullptr;
    // kernel timing: an event pair around every kernel launch and Thrust call
    bool timing = false;
    std::vector<CUevent> tev;
    size_t ntev = 0;
    void tmark() {
        if (!timing) return;
        if (ntev == tev.size()) {
            CUevent e;
            ck(cuEventCreate(&e, 0), "event");
            tev.push_back(e);
        }
        ck(cuEventRecord(tev[ntev++], 0), "event");
    }
    float kernel_ms() {  // sum over the recorded pairs
        if (!ntev) return 0.0f;
        ck(cuEventSynchronize(tev[ntev - 1]), "event");
        float tot = 0.0f;
        for (size_t i = 0; i + 1 < ntev; i += 2) {
            float ms = 0.0f;
            ck(cuEventElapsedTime(&ms, tev[i], tev[i + 1]), "event");
            tot += ms;
        }
        return tot;
    }

    CUfunction fn(const char* name) {
        CUfunction f;
        if (cuModuleGetFunction(&f, mod, name) != CUDA_SUCCESS) throw std::string("missing kernel ") + name;
        return f;
    }
    void ck(CUresult r, const char* what) {
        if (r != CUDA_SUCCESS) {
            const char* s = nullptr;
            cuGetErrorString(r, &s);
            throw std::string(what) + ": " + (s ? s : "?");
        }
    }
    void launch(const char* name, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, unsigned bz, void** args) {
        CUfunction f = fn(name);
        tmark();
        ck(cuLaunchKernel(f, gx, gy, gz, bx, by, bz, 0, nullptr, args, nullptr), name);
        tmark();
    }
    void realloc_dev(CUdeviceptr& p, size_t& cap, size_t need) {
        if (need <= cap && p) return;
        if (p) cuMemFree(p);
        cap = std::max(need, (size_t)256);
        ck(cuMemAlloc(&p, cap), "cuMemAlloc");
    }
    void aux(CUdeviceptr& p, size_t bytes) {  // PrepareAux: fresh buffer
        if (p) cuMemFree(p);
        ck(cuMemAlloc(&p, std::max(bytes, (size_t)256)), "aux");
    }

    int range(int lev) {
        int r = 1;
        for (int l = 0; l <= lev; l++) r <<= logdim[l];
        return r;
    }
    int res(int lev) { return 1 << logdim[lev]; }
    uint64_t voxcnt(int lev) { uint64_t r = (uint64_t)1 << logdim[lev]; return r * r * r; }

    // ---- pools (AL.cpp:55-192)
    void pool_create(int grp, int lev, size_t width, size_t initmax) {
        Pool& p = pool[grp][lev];
        p.stride = width;
        p.max = initmax;
        p.lastEle = p.usedNum = 0;
        if (width * initmax == 0) return;
        p.cpu.assign(width * initmax, 0);
        ck(cuMemAlloc(&p.gpu, width * initmax), "pool");
        ck(cuMemsetD8(p.gpu, 0, width * initmax), "pool");
    }
    uint64_t pool_alloc(int grp, int lev) {
        Pool& p = pool[grp][lev];
        if (p.lastEle >= p.max) {
            p.max *= 2;
            std::vector<char> nc(p.stride * p.max, 0);
            memcpy(nc.data(), p.cpu.data(), p.stride * p.lastEle);
            p.cpu.swap(nc);
            CUdeviceptr ng;
            ck(cuMemAlloc(&ng, p.stride * p.max), "pool grow");
            ck(cuMemsetD8(ng, 0, p.stride * p.max), "pool grow");
            if (p.lastEle) ck(cuMemcpy(ng, p.gpu, p.stride * p.lastEle), "pool grow");
            cuMemFree(p.gpu);
            p.gpu = ng;
        }
        p.lastEle++;
        p.usedNum++;
        return Elem(grp, lev, p.lastEle - 1);
    }
    void commit_all() {
        for (int g = 0; g < 2; g++)
            for (int l = 0; l < levs; l++) {
                Pool& p = pool[g][l];
                if (p.gpu && p.lastEle) ck(cuMemcpyHtoD(p.gpu, p.cpu.data(), p.stride * p.lastEle), "commit");
            }
    }
    void fetch_all() {
        for (int g = 0; g < 2; g++)
            for (int l = 0; l < levs; l++) {
                Pool& p = pool[g][l];
                if (p.gpu && p.lastEle) ck(cuMemcpyDtoH(p.cpu.data(), p.gpu, p.stride * p.lastEle), "fetch");
            }
    }
    HNode* node(int lev, size_t i) { return reinterpret_cast<HNode*>(pool[0][lev].cpu.data() + i * 64); }
    uint64_t* clist_of(uint64_t elem) {
        int lev = (int)((elem >> 8) & 0xFF);
        return reinterpret_cast<uint64_t*>(pool[1][lev].cpu.data() + (elem >> 16) * pool[1][lev].stride);
    }
    void setup_node(uint64_t id, int lev, const int pos[3]) {  // VG.cpp:2512-2524
        HNode* n = node(lev, id >> 16);
        n->lev = (uint8_t)lev;
        for (int a = 0; a < 3; a++) { n->pos[a] = pos[a]; n->value[a] = -1; }
        n->childlist = UNDEFL;
        n->parent = UNDEFL;
        n->flags = 1;
    }

    // ---- VDBInfo (VG.cpp:3946-4016)
    void prepare(bool partial) {
        int tlev = 1;
        for (int n = levs - 1; n >= 0; n--) {
            info.dim[n] = logdim[n];
            info.res[n] = res(n);
            int rg = range(n);
            for (int a = 0; a < 3; a++) {
                info.vdel[n][a] = (float)rg / (float)res(n);
                info.noderange[n][a] = rg;
            }
            info.nodecnt[n] = (int)pool[0][n].lastEle;
            info.nodewid[n] = (int)pool[0][n].stride;
            info.childwid[n] = (int)pool[1][n].stride;
            info.nodelist[n] = pool[0][n].gpu;
            info.childlist[n] = pool[1][n].gpu;
            if (info.nodecnt[n] == 1) tlev = n;
        }
        info.top_lev = tlev;
        if (!partial) {
            info.atlas_map = amap;
            info.atlas_apron = 1;
            info.atlas_cnt[0] = ax; info.atlas_cnt[1] = ay; info.atlas_cnt[2] = az;
            info.atlas_res[0] = ax * 18; info.atlas_res[1] = ay * 18; info.atlas_res[2] = az * 18;
            info.brick_res = 18;
            info.volOut[0] = surf;
            info.volOut[1] = csurf;
        }
        ck(cuMemcpyHtoD(cuinfo, &info, sizeof(info)), "prepare");
    }

    // ---- PrefixSum (VG.cpp:4760-4819) with the reference's prefixSum / prefixFixup kernels
    void prefix_sum(CUdeviceptr in, CUdeviceptr out, int n) {
        int naux = 1024;
        int blks1 = n / naux + 1;
        int blks2 = blks1 / naux + 1;
        int threads = 512, zon = 1;
        CUdeviceptr nptr = 0;
        aux(scanA1, (size_t)std::max(blks2, 1) * 1024 * 4);
        aux(scanS1, (size_t)std::max(blks2, 1) * 1024 * 4);
        aux(scanA2, 1024 * 4);
        aux(scanS2, 1024 * 4);
        void* a[5] = {&in, &out, &scanA1, &n, &zon};
        launch("prefixSum", blks1, 1, 1, threads, 1, 1, a);
        void* b[5] = {&scanA1, &scanS1, &scanA2, &blks1, &zon};
        launch("prefixSum", blks2, 1, 1, threads, 1, 1, b);
        void* c[5] = {&scanA2, &scanS2, &nptr, &blks2, &zon};
        launch("prefixSum", 1, 1, 1, threads, 1, 1, c);
        void* d[3] = {&scanS1, &scanS2, &blks1};
        launch("prefixFixup", blks2, 1, 1, threads, 1, 1, d);
        void* e[3] = {&out, &scanS1, &n};
        launch("prefixFixup", blks1, 1, 1, threads, 1, 1, e);
    }

    // ---- GetBoundingBox (VG.cpp:5404-5467)
    void bounding_box(float3 orig) {
        realloc_dev(bbx, bb_cap, (size_t)npts * 4);
        size_t c2 = 0, c3 = 0;
        realloc_dev(bby, c2, (size_t)npts * 4);
        realloc_dev(bbz, c3, (size_t)npts * 4);
        if (!bbox) ck(cuMemAlloc(&bbox, 64), "bbox");
        int off = 0, stride = 12;
        void* a[8] = {&npts, &orig, &pts, &off, &stride, &bbx, &bby, &bbz};
        launch("gvdbSplitPos", npts / 256 + 1, 1, 1, 256, 1, 1, a);
        CUdeviceptr ax3[3] = {bbx, bby, bbz};
        float out[6];
        for (int i = 0; i < 3; i++) {
            thrust::device_ptr<float> b = thrust::device_pointer_cast((float*)ax3[i]);
            tmark();
            auto mn = thrust::min_element(b, b + npts);
            auto mx = thrust::max_element(b, b + npts);
            tmark();
            out[i] = *mn;
            out[3 + i] = *mx;
        }
        for (int a = 0; a < 3; a++) {
            posmin[a] = out[a] - 1; posmax[a] = out[3 + a] + 2;
            posmin[a] = 0 > posmin[a] ? 0 : posmin[a];
            posmax[a] = 0 > posmax[a] ? 0 : posmax[a];
            posrange[a] = posmax[a] - posmin[a];  // mPosRange (VG.cpp:5458-5462)
        }
    }
    int determine_depth(int root[3]) {  // VG.cpp:821-837
        int pmin[3], pmax[3];
        for (int a = 0; a < 3; a++) { pmin[a] = (int)posmin[a]; pmax[a] = (int)posmax[a]; }
        for (int lev = 0; lev < levs; lev++) {
            int rg = range(lev);
            bool same = true;
            for (int a = 0; a < 3; a++) if (pmin[a] / rg != pmax[a] / rg) same = false;
            if (same) {
                for (int a = 0; a < 3; a++) root[a] = pmin[a] / rg * rg;
                return lev;
            }
        }
        return -1;
    }

    void clear() {  // VG.cpp:2487-2503
        for (int g = 0; g < 2; g++) for (int l = 0; l < levs; l++) pool[g][l].lastEle = pool[g][l].usedNum = 0;
        atlas_last = 0;
        rebuild = true;
    }

    // sort + unique of `count` keys (RadixSortByByte + FindUniqueBrick); returns uniques (host)
    void sort_unique(int count, int D, std::vector<uint16_t>& uni, std::vector<int>& levcnt_h) {
        if (count <= 0) { uni.clear(); levcnt_h.assign(D, 0); return; }
        aux(sorted, (size_t)count * 8);
        ck(cuMemcpyDtoD(sorted, keys, (size_t)count * 8), "sort copy");
        thrust::device_ptr<uint64_t> b = thrust::device_pointer_cast((uint64_t*)sorted);
        tmark();
        thrust::sort(b, b + count, thrust::less<uint64_t>());
        tmark();
        aux(marker, (size_t)count * 4);
        aux(presum, (size_t)count * 4);
        aux(cnt, 4);
        aux(levcnt, (size_t)D * 4);
        ck(cuMemsetD8(marker, 0, (size_t)count * 4), "m");
        ck(cuMemsetD8(presum, 0, (size_t)count * 4), "m");
        ck(cuMemsetD8(cnt, 0, 4), "m");
        ck(cuMemsetD8(levcnt, 0, (size_t)D * 4), "m");
        void* a[5] = {&count, &sorted, &marker, &cnt, &levcnt};
        launch("gvdbFindUnique", count / 512 + 1, 1, 1, 512, 1, 1, a);
        int nuni = 0;
        ck(cuMemcpyDtoH(&nuni, cnt, 4), "nuni");
        prefix_sum(marker, presum, count);
        aux(uniq, (size_t)std::max(nuni, 1) * 8);
        void* c[5] = {&count, &sorted, &marker, &presum, &uniq};
        launch("gvdbCompactUnique", count / 512 + 1, 1, 1, 512, 1, 1, c);
        levcnt_h.assign(D, 0);
        ck(cuMemcpyDtoH(levcnt_h.data(), levcnt, (size_t)D * 4), "levcnt");
        uni.resize((size_t)nuni * 4);
        if (nuni) ck(cuMemcpyDtoH(uni.data(), uniq, (size_t)nuni * 8), "uniq");
    }

    void alloc_nodes(const std::vector<uint16_t>& uni, const std::vector<int>& levcnt_h, int D) {
        int base = 0;
        for (int lev = 0; lev < D; lev++) {
            int rg = range(lev);
            for (int n = base; n < base + levcnt_h[lev]; n++) {
                uint64_t id = pool_alloc(0, lev);
                int pos[3] = {uni[(size_t)n * 4 + 2] * rg, uni[(size_t)n * 4 + 1] * rg, uni[(size_t)n * 4 + 0] * rg};
                setup_node(id, lev, pos);
                if (lev > 0) {
                    HNode* nd = node(lev, id >> 16);
                    nd->childlist = pool_alloc(1, lev);
                    memset(clist_of(nd->childlist), 0xFF, 8 * voxcnt(lev));
                }
            }
            base += levcnt_h[lev];
        }
    }

    void link(int D, int threads_from_leaves) {
        for (int lev = D - 1; lev >= 0; lev--) {
            int cntn = (int)(threads_from_leaves ? pool[0][0].lastEle : pool[0][lev].lastEle);
            void* a[2] = {&cuinfo, &lev};
            launch("gvdbLinkBricks", cntn / 512 + 1, 1, 1, 512, 1, 1, a);
        }
    }

    void keys_reserve(size_t need) { realloc_dev(keys, keys_bytes, need * 8); }

    void activate_bricks(float3 orig, int D, const int root[3]) {  // VG.cpp:1229-1413
        std::vector<int> rr(D);
        for (int l = 0; l < D; l++) rr[l] = range(l);
        aux(range_res, (size_t)D * 4);
        ck(cuMemcpyHtoD(range_res, rr.data(), (size_t)D * 4), "range_res");
        keys_reserve((size_t)npts * D);
        int off = 0, stride = 12;
        void* a[8] = {&npts, &D, &range_res, &pts, &off, &stride, &orig, &keys};
        launch("gvdbCalcBrickId", npts / 512 + 1, 1, 1, 512, 1, 1, a);
        std::vector<uint16_t> uni;
        std::vector<int> lc;
        sort_unique(npts * D, D, uni, lc);
        uint64_t r = pool_alloc(0, D);
        uint64_t cl = pool_alloc(1, D);
        setup_node(r, D, root);
        HNode* rn = node(D, r >> 16);
        rn->flags = 1;
        rn->childlist = cl;
        memset(clist_of(cl), 0xFF, 8 * voxcnt(D));
        alloc_nodes(uni, lc, D);
        commit_all();
        prepare(true);
        link(D, 0);
        fetch_all();
    }

    // extra (hi2 = true, VG.cpp:931-1016) and incremental (VG.cpp:1020-1156) passes
    int box_pass(float radius, float3 orig, int D, bool incr, bool accum) {
        int nleaf = (int)pool[0][0].lastEle;
        std::vector<int> lc;
        std::vector<uint16_t> uni;
        if (incr) {
            if (nleaf == 0) return 0;
            aux(node_mk, (size_t)nleaf * 4);
            std::vector<int> mk(nleaf, 0);
            if (accum) for (int i = 0; i < nleaf; i++) mk[i] = node(0, i)->flags;
            ck(cuMemcpyHtoD(node_mk, mk.data(), (size_t)nleaf * 4), "markers");
        }
        // worst case keys per point: every node position of the box at every level
        size_t per = 0;
        for (int l = 0; l < D; l++) {
            size_t w = (size_t)std::floor((incr ? 2.0 : 3.0) * radius + 2) / (size_t)range(l) + 2;
            per += w * w * w;
        }
        keys_reserve((size_t)npts * per + 64);
        CUdeviceptr excnt;
        ck(cuMemAlloc(&excnt, 64), "excnt");
        ck(cuMemsetD8(excnt, 0, 64), "excnt");
        prepare(true);
        int off = 0, stride = 12;
        CUdeviceptr mk_dev = node_mk;
        if (incr) {
            void* a[12] = {&cuinfo, &radius, &npts, &D, &range_res, &pts, &off, &stride, &orig, &keys, &excnt, &mk_dev};
            launch("gvdbCalcIncreExtraBrickId", npts / 512 + 1, 1, 1, 512, 1, 1, a);
        } else {
            void* a[11] = {&cuinfo, &radius, &npts, &D, &range_res, &pts, &off, &stride, &orig, &keys, &excnt};
            launch("gvdbCalcExtraBrickId", npts / 512 + 1, 1, 1, 512, 1, 1, a);
        }
        int ex = 0;
        ck(cuMemcpyDtoH(&ex, excnt, 4), "excnt");
        cuMemFree(excnt);
        if (incr && ex == 0) return 0;  // VG.cpp:1066
        sort_unique(ex, D, uni, lc);
        if (incr) {
            std::vector<int> mk(nleaf);
            ck(cuMemcpyDtoH(mk.data(), node_mk, (size_t)nleaf * 4), "markers");
            for (int i = 0; i < nleaf; i++) node(0, i)->flags = (uint8_t)mk[i];
        }
        alloc_nodes(uni, lc, D);
        commit_all();
        prepare(true);
        if (incr) {
            link(D, 1);
            int t = (int)pool[0][0].lastEle;
            void* a[1] = {&cuinfo};
            launch("gvdbDelinkLeafBricks", t / 512 + 1, 1, 1, 512, 1, 1, a);
            for (int lev = 1; lev < D; lev++) {
                void* b[2] = {&cuinfo, &lev};
                launch("gvdbDelinkBricks", t / 512 + 1, 1, 1, 512, 1, 1, b);
            }
            fetch_all();
            uint64_t used = pool[0][0].lastEle;
            for (size_t i = 0; i < pool[0][0].lastEle; i++) if (!node(0, i)->flags) used--;
            pool[0][0].usedNum = used;
        } else {
            link(D, 0);
            fetch_all();
        }
        return ex;
    }

    int accumulate_topology(float radius, float3 orig, int min_depth) {  // VG.cpp:1158-1178
        bounding_box(orig);
        int root[3];
        int D = determine_depth(root);
        if (D < min_depth) D = min_depth;
        if (D == 0 || D > 5) return 4;
        if (rebuild) return rebuild_topology(radius, orig);
        box_pass(radius, orig, D, true, true);
        return 0;
    }

    int rebuild_topology(float radius, float3 orig) {  // VG.cpp:1181-1218
        bounding_box(orig);
        int root[3];
        int D = determine_depth(root);
        if (D <= 0 || D > 5) return 4;
        if (rebuild) clear();
        else if (D != curr_depth) { clear(); rebuild = true; curr_depth = D; }
        if (rebuild) {
            activate_bricks(orig, D, root);
            if (radius >= 1) box_pass(radius, orig, D, false, false);
            rebuild = false;
        } else {
            box_pass(radius, orig, D, true, false);
        }
        return 0;
    }

    // ---- atlas (AL.cpp:311-456, 622-715; VG.cpp:2630-2704)
    // One CUarray per channel; a grown array is cleared and the old one copied in
    // (AllocateTextureGPU, AL.cpp:389-456).  A fresh array is cleared as well.
    void make_array(CUarray& a, CUsurfObject& so, bool colour, int new_az, bool preserve) {
        CUDA_ARRAY3D_DESCRIPTOR d{};
        d.Format = colour ? CU_AD_FORMAT_UNSIGNED_INT8 : CU_AD_FORMAT_FLOAT;
        d.NumChannels = colour ? 4 : 1;
        d.Width = (size_t)ax * 18;
        d.Height = (size_t)ay * 18;
        d.Depth = (size_t)new_az * 18;
        d.Flags = CUDA_ARRAY3D_SURFACE_LDST;
        CUarray na;
        ck(cuArray3DCreate(&na, &d), "atlas");
        {
            std::vector<char> zero((size_t)ax * 18 * 4 * ay * 18 * new_az * 18, 0);
            CUDA_MEMCPY3D cp{};
            cp.srcMemoryType = CU_MEMORYTYPE_HOST;
            cp.srcHost = zero.data();
            cp.srcPitch = (size_t)ax * 18 * 4;
            cp.srcHeight = (size_t)ay * 18;
            cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
            cp.dstArray = na;
            cp.WidthInBytes = (size_t)ax * 18 * 4;
            cp.Height = (size_t)ay * 18;
            cp.Depth = (size_t)new_az * 18;
            ck(cuMemcpy3D(&cp), "atlas clear");
        }
        if (preserve && a) {
            CUDA_MEMCPY3D cp{};
            cp.srcMemoryType = CU_MEMORYTYPE_ARRAY;
            cp.srcArray = a;
            cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
            cp.dstArray = na;
            cp.WidthInBytes = (size_t)ax * 18 * 4;
            cp.Height = (size_t)ay * 18;
            cp.Depth = (size_t)az * 18;
            ck(cuMemcpy3D(&cp), "atlas copy");
        }
        if (so) cuSurfObjectDestroy(so);
        if (a) cuArrayDestroy(a);
        a = na;
        CUDA_RESOURCE_DESC rd{};
        rd.resType = CU_RESOURCE_TYPE_ARRAY;
        rd.res.array.hArray = a;
        ck(cuSurfObjectCreate(&so, &rd), "surf");
    }
    void make_atlas(int new_az, bool preserve) {
        make_array(arr, surf, false, new_az, preserve);
        if (colour_chan) make_array(carr, csurf, true, new_az, preserve);
        az = new_az;
    }
    // FillChannel(chan, v) as the whole atlas array (the reference's FUNC_FILL_F leaves the
    // array's first voxel plane of each axis, an apron plane, unwritten)
    void fill(int chan, float v) {
        size_t W = (size_t)ax * 18, H = (size_t)ay * 18, Dz = (size_t)az * 18;
        std::vector<float> vals(W * H * Dz, v);
        CUDA_MEMCPY3D cp{};
        cp.srcMemoryType = CU_MEMORYTYPE_HOST;
        cp.srcHost = vals.data();
        cp.srcPitch = W * 4;
        cp.srcHeight = H;
        cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
        cp.dstArray = chan == 0 ? arr : carr;
        cp.WidthInBytes = W * 4;
        cp.Height = H;
        cp.Depth = Dz;
        ck(cuMemcpy3D(&cp), "fill");
    }
    void update_atlas() {
        size_t total = pool[0][0].lastEle, used = pool[0][0].usedNum;
        atlas_last = 0;
        int layer = ax * ay;
        if (used > (size_t)layer * az) make_atlas((int)std::ceil((float)used / (float)layer), true);
        for (size_t n = 0; n < total; n++) {
            HNode* nd = node(0, n);
            if (!nd->flags) continue;
            if (atlas_last >= layer * az) make_atlas((int)std::ceil((float)(atlas_last + layer) / (float)layer), true);
            int id = atlas_last++;
            int pz = id / layer, rem = id - pz * layer, py = rem / ax, px = rem - py * ax;
            nd->value[0] = px * 18 + 1; nd->value[1] = py * 18 + 1; nd->value[2] = pz * 18 + 1;
        }
        size_t slots = (size_t)layer * az;
        if (slots != amap_cnt) {
            if (amap) cuMemFree(amap);
            ck(cuMemAlloc(&amap, slots * 16), "amap");
            amap_cnt = slots;
        }
        amap_cpu.assign(slots * 4, -1);
        for (size_t n = 0; n < total; n++) {
            HNode* nd = node(0, n);
            if (!nd->flags) continue;
            int s = ((nd->value[2] / 18) * ay + nd->value[1] / 18) * ax + nd->value[0] / 18;
            for (int a = 0; a < 3; a++) amap_cpu[(size_t)s * 4 + a] = nd->pos[a];
            amap_cpu[(size_t)s * 4 + 3] = (int)n;
        }
        ck(cuMemcpyHtoD(amap, amap_cpu.data(), slots * 16), "amap");
        Pool& p = pool[0][0];
        if (p.lastEle) ck(cuMemcpyHtoD(p.gpu, p.cpu.data(), p.stride * p.lastEle), "pool00");
    }

    // ---- InsertPointsSubcell (VG.cpp:4971-5092)
    int insert_subcell(float radius, float3 trans, bool fp16 = false) {
        int numBrick = (int)pool[0][0].usedNum;
        if (numBrick == 0) return 8;
        prepare(false);
        int sc = 4, scpb = 64, nsc = scpb * numBrick, scdim = 4;
        int nmap = (int)pool[0][0].lastEle;
        aux(sc_flag, (size_t)nmap * 4);
        aux(sc_map, (size_t)nmap * 4);
        void* a[3] = {&cuinfo, &nmap, &sc_flag};
        launch("gvdbSetFlagSubcell", nmap / 512 + 1, 1, 1, 512, 1, 1, a);
        prefix_sum(sc_flag, sc_map, nmap);
        aux(sc_cnt, (size_t)nsc * 4);
        ck(cuMemsetD8(sc_cnt, 0, (size_t)nsc * 4), "cnt");
        int3 rng = make_int3(4, 4, 4);
        int off = 0, stride = 12;
        void* c[14] = {&cuinfo, &sc, &scpb, &npts, &pts, &off, &stride, &sc_cnt, &rng, &trans, &scdim, &radius, &nsc, &sc_map};
        launch("gvdbCountSubcell", npts / 512 + 1, 1, 1, 512, 1, 1, c);
        aux(sc_off, (size_t)nsc * 4);
        ck(cuMemsetD8(sc_off, 0, (size_t)nsc * 4), "off");
        prefix_sum(sc_cnt, sc_off, nsc);
        int ol = 0, cl = 0;
        ck(cuMemcpyDtoH(&ol, sc_off + (size_t)(nsc - 1) * 4, 4), "ol");
        ck(cuMemcpyDtoH(&cl, sc_cnt + (size_t)(nsc - 1) * 4, 4), "cl");
        sc_len = ol + cl;
        sc_num = nsc;
        if (sc_len == 0) return 0;
        ck(cuMemsetD8(sc_cnt, 0, (size_t)nsc * 4), "cnt");
        aux(sc_pnts, (size_t)sc_len * (fp16 ? 6 : 12));
        fp16_lists = fp16;
        CUdeviceptr z = 0;
        int cstride = 4;
        if (clr) aux(sc_clr, (size_t)sc_len * 4);  // VG.cpp:5063
        if (fp16) {  // VG.cpp:5160-5172
            float3 pmin = make_float3(posmin[0], posmin[1], posmin[2]);
            float3 prng = make_float3(posrange[0], posrange[1], posrange[2]);
            float3 vmin = make_float3(0, 0, 0), vrng = make_float3(0, 0, 0);
            void* d[27] = {&cuinfo, &sc, &scpb, &npts, &sc_cnt, &sc_off, &sc_map, &pmin, &prng, &vmin, &vrng,
                           &rng, &trans, &scdim, &radius, &pts, &off, &stride, &sc_pnts, &z, &off, &stride, &z,
                           clr ? &clr : &z, &off, &cstride, clr ? &sc_clr : &z};
            launch("gvdbInsertSubcell_fp16", npts / 512 + 1, 1, 1, 512, 1, 1, d);
        } else {
            void* d[23] = {&cuinfo, &sc, &scpb, &npts, &sc_cnt, &sc_off, &sc_map, &rng, &trans, &scdim, &radius,
                           &pts, &off, &stride, &sc_pnts, &z, &off, &stride, &z, clr ? &clr : &z, &off, &cstride,
                           clr ? &sc_clr : &z};
            launch("gvdbInsertSubcell", npts / 512 + 1, 1, 1, 512, 1, 1, d);
        }
        aux(sc_pos, (size_t)nsc * 12);
        aux(sc_nid, (size_t)nsc * 4);
        void* e[8] = {&cuinfo, &sc_nid, &sc_pos, &nmap, &scdim, &scpb, &sc, &sc_map};
        launch("gvdbCalcSubcellPos", nmap / 512 + 1, 1, 1, 512, 1, 1, e);
        return 0;
    }

    int gather(int mode, float radius, bool accum) {  // VG.cpp:5318-5373
        int num_brick = (int)pool[0][0].usedNum;
        if (num_brick == 0 || sc_len == 0) return 8;
        prepare(false);
        int nsc = 64 * num_brick;
        CUdeviceptr z = 0;
        int chan = 0, cchan = 1;
        CUdeviceptr cl = (clr && colour_chan) ? sc_clr : 0;
        void* a[14] = {&cuinfo, &npts, &nsc, &radius, &sc_nid, &sc_cnt, &sc_off, &sc_pos, &sc_pnts, &z, &cl, &chan,
                       &cchan, &accum};
        launch(mode == 0 ? "gvdbGatherDensity" : "gvdbGatherLevelSet", nsc, 1, 1, 4, 4, 4, a);
        return 0;
    }

    int gather_levelset_fp16(float radius) {  // VG.cpp:5375-5401
        int num_brick = (int)pool[0][0].usedNum;
        if (num_brick == 0) return 8;
        prepare(false);
        int nsc = 64 * num_brick;
        CUdeviceptr z = 0;
        int chan = 0, cchan = 1;
        float3 pmin = make_float3(posmin[0], posmin[1], posmin[2]);
        float3 prng = make_float3(posrange[0], posrange[1], posrange[2]);
        float3 vmin = make_float3(0, 0, 0), vrng = make_float3(0, 0, 0);
        void* a[17] = {&cuinfo, &npts, &nsc, &radius, &pmin, &prng, &vmin, &vrng, &sc_nid, &sc_cnt, &sc_off, &sc_pos,
                       &sc_pnts, &z, &z, &chan, &cchan};
        launch("gvdbGatherLevelSet_fp16", nsc, 1, 1, 4, 4, 4, a);
        return 0;
    }

    // host getNodeAtPoint for a leaf, from mRoot (the root of the last build) through the
    // host child lists; -1 when no leaf holds p
    long long leaf_at(const int p[3]) {
        int D = -1;
        for (int l = levs - 1; l >= 0; l--)
            if (pool[0][l].lastEle > 0) { D = l; break; }
        if (D <= 0) return -1;
        HNode* nd = node(D, 0);
        for (int lev = D; lev >= 1; lev--) {
            const int rg = range(lev), r = res(lev), cr = rg / r;
            int o[3];
            for (int a = 0; a < 3; a++) {
                o[a] = p[a] - nd->pos[a];
                if (o[a] < 0 || o[a] >= rg) return -1;
            }
            if (nd->childlist == UNDEFL) return -1;
            const uint64_t c = clist_of(nd->childlist)[((o[2] / cr) * r + o[1] / cr) * r + o[0] / cr];
            if (c == UNDEF64) return -1;
            nd = node(lev - 1, (size_t)(c >> 16));
            if (lev - 1 == 0) return (long long)(c >> 16);
        }
        return -1;
    }

    // UpdateNeighbors (VG.cpp:2527-2556) + UpdateApronFaces (VG.cpp:4461-4496).  The table
    // holds -1 (ID_UNDEFL) for a missing neighbour, which the kernel skips; the reference
    // stores ElemNdx(ID_UNDEFL) = 65535 there, which its kernel would read as a node.
    int update_apron_faces() {
        prepare(false);
        int bricks = (int)pool[0][0].lastEle;
        if (bricks == 0) return 8;
        std::vector<int> tab((size_t)bricks * 6);
        const int d = 16;
        for (int n = 0; n < bricks; n++) {
            HNode* nd = node(0, n);
            const int ct[3] = {nd->pos[0] + d / 2, nd->pos[1] + d / 2, nd->pos[2] + d / 2};
            const int off[6][3] = {{-d, 0, 0}, {0, -d, 0}, {0, 0, -d}, {d, 0, 0}, {0, d, 0}, {0, 0, d}};
            for (int k = 0; k < 6; k++) {
                const int p[3] = {ct[0] + off[k][0], ct[1] + off[k][1], ct[2] + off[k][2]};
                tab[(size_t)n * 6 + k] = (int)leaf_at(p);
            }
        }
        aux(nbr, tab.size() * 4);
        ck(cuMemcpyHtoD(nbr, tab.data(), tab.size() * 4), "nbr");
        unsigned char chan = 0;
        int brickres = 18, brickwid = 16;
        void* a[6] = {&cuinfo, &chan, &bricks, &brickres, &brickwid, &nbr};
        launch("gvdbUpdateApronFacesF", bricks, (16 + 7) / 8, (16 + 7) / 8, 3, 8, 8, a);
        return 0;
    }

    // Compute(FUNC_SMOOTH, 0, 1, params, false, skipOverAprons = true) (VG.cpp:4532-4558): one
    // pass of gvdbOpSmooth over the packed atlas
    int smooth(float p1, float p2, float p3) {
        prepare(false);
        int3 ares = make_int3(ax * 18, ay * 18, az * 18);
        unsigned char chan = 0;
        const unsigned gx = (unsigned)(ax * 16 + 7) / 8, gy = (unsigned)(ay * 16 + 7) / 8, gz = (unsigned)(az * 16 + 7) / 8;
        void* a[6] = {&cuinfo, &ares, &chan, &p1, &p2, &p3};
        launch("gvdbOpSmooth", gx, gy, gz, 8, 8, 8, a);
        return 0;
    }

    // legacy InsertPoints(bPrefix = true) (VG.cpp:5219-5267)
    int insert_points(float3 trans) {
        prepare(false);
        int bricks = (int)pool[0][0].lastEle;
        aux(pnode, (size_t)std::max(npts, 1) * 4);
        aux(pndx, (size_t)std::max(npts, 1) * 4);
        aux(gcnt, (size_t)std::max(bricks, 1) * 4);
        ck(cuMemsetD8(gcnt, 0, (size_t)std::max(bricks, 1) * 4), "gcnt");
        int off = 0, stride = 12;
        void* a[9] = {&cuinfo, &npts, &pts, &off, &stride, &pnode, &pndx, &gcnt, &trans};
        launch("gvdbInsertPoints", npts / 512 + 1, 1, 1, 512, 1, 1, a);
        aux(goff, (size_t)std::max(bricks, 1) * 4);
        prefix_sum(gcnt, goff, bricks);
        aux(psort, (size_t)std::max(npts, 1) * 12);
        void* b[11] = {&npts, &pts, &off, &stride, &pnode, &pndx, &bricks, &gcnt, &goff, &psort, &trans};
        launch("gvdbSortPoints", npts / 512 + 1, 1, 1, 512, 1, 1, b);
        return 0;
    }

    // ScatterDensity(num_pnts, radius, amp, trans, expand, avgColor = false) (VG.cpp:5624-5660),
    // launched with the VDBInfo pointer that gvdbScatterPointDensity takes first
    // (PT.cuh:525; the reference's host code omits it)
    int scatter_density(float radius, float amp, float3 trans, bool expand) {
        prepare(false);
        CUdeviceptr z = 0;
        int off = 0, stride = 12, coff = 0, cstride = 4;
        void* a[14] = {&cuinfo, &npts, &radius, &amp, &pts, &off, &stride, &z, &coff, &cstride, &pnode, &trans, &expand,
                       &z};
        launch("gvdbScatterPointDensity", npts / 256 + 1, 1, 1, 256, 1, 1, a);
        return 0;
    }

    // padded bricks of slots [0, n) (4-byte voxels, [slot][z][y][x]) into the atlas array
    void write_bricks(int chan, const float* in, int n) {
        size_t W = (size_t)ax * 18, H = (size_t)ay * 18, Dz = (size_t)az * 18;
        std::vector<float> all(W * H * Dz);
        CUDA_MEMCPY3D cp{};
        cp.srcMemoryType = CU_MEMORYTYPE_ARRAY;
        cp.srcArray = chan == 0 ? arr : carr;
        cp.dstMemoryType = CU_MEMORYTYPE_HOST;
        cp.dstHost = all.data();
        cp.dstPitch = W * 4;
        cp.dstHeight = H;
        cp.WidthInBytes = W * 4;
        cp.Height = H;
        cp.Depth = Dz;
        ck(cuMemcpy3D(&cp), "read atlas");
        for (int s = 0; s < n; s++) {
            int pz = s / (ax * ay), rem = s - pz * ax * ay, py = rem / ax, px = rem - py * ax;
            for (int z = 0; z < 18; z++)
                for (int y = 0; y < 18; y++)
                    for (int x = 0; x < 18; x++)
                        all[((size_t)(pz * 18 + z) * H + (py * 18 + y)) * W + (px * 18 + x)] =
                            in[(size_t)s * 5832 + (z * 18 + y) * 18 + x];
        }
        CUDA_MEMCPY3D wp{};
        wp.srcMemoryType = CU_MEMORYTYPE_HOST;
        wp.srcHost = all.data();
        wp.srcPitch = W * 4;
        wp.srcHeight = H;
        wp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
        wp.dstArray = chan == 0 ? arr : carr;
        wp.WidthInBytes = W * 4;
        wp.Height = H;
        wp.Depth = Dz;
        ck(cuMemcpy3D(&wp), "write atlas");
    }

    int update_apron(int c, float boundval) {  // VG.cpp:4418-4457
        prepare(false);
        int bricks = (int)pool[0][0].lastEle;
        if (bricks == 0) return 8;
        unsigned char chan = (unsigned char)c;
        int brickres = 18, brickwid = 16;
        void* a[6] = {&cuinfo, &chan, &bricks, &brickres, &brickwid, &boundval};
        launch(c == 0 ? "gvdbUpdateApronF" : "gvdbUpdateApronC4", bricks, (18 + 7) / 8, (18 + 7) / 8, 6, 8, 8, a);
        return 0;
    }

    // padded bricks of slots [0, used) from the CUarray, [slot][z][y][x]
    void read_bricks(int chan, float* out) {  // 4-byte voxels (FP32 or RGBA8)
        size_t W = (size_t)ax * 18, H = (size_t)ay * 18, Dz = (size_t)az * 18;
        std::vector<float> all(W * H * Dz);
        CUDA_MEMCPY3D cp{};
        cp.srcMemoryType = CU_MEMORYTYPE_ARRAY;
        cp.srcArray = chan == 0 ? arr : carr;
        cp.dstMemoryType = CU_MEMORYTYPE_HOST;
        cp.dstHost = all.data();
        cp.dstPitch = W * 4;
        cp.dstHeight = H;
        cp.WidthInBytes = W * 4;
        cp.Height = H;
        cp.Depth = Dz;
        ck(cuMemcpy3D(&cp), "read atlas");
        for (int s = 0; s < atlas_last; s++) {
            int pz = s / (ax * ay), rem = s - pz * ax * ay, py = rem / ax, px = rem - py * ax;
            for (int z = 0; z < 18; z++)
                for (int y = 0; y < 18; y++)
                    for (int x = 0; x < 18; x++)
                        out[(size_t)s * 5832 + (z * 18 + y) * 18 + x] =
                            all[((size_t)(pz * 18 + z) * H + (py * 18 + y)) * W + (px * 18 + x)];
        }
    }
};

extern "C" {

void* rh_create(const char* ptx_path, int levs, const int* log2dim_leaf_first) {
    Harness* h = new Harness();
    try {
        cudaFree(0);  // primary context
        h->ck(cuCtxGetCurrent(&h->ctx), "ctx");
        h->ck(cuModuleLoad(&h->mod, ptx_path), "cuModuleLoad");
        h->levs = levs;
        for (int l = 0; l < levs; l++) h->logdim[l] = log2dim_leaf_first[l] ? log2dim_leaf_first[l] : 1;
        // Configure (VG.cpp:2364-2434): initial pool sizes 4, 4, 2, 1, 1, ...
        int cnt = 4;
        for (int n = 0; n < levs; n++) {
            int mx = n == 0 ? 4 : cnt;
            if (n >= 1) cnt = std::max(1, cnt >> 1);
            h->pool_create(0, n, 64, mx ? mx : 1);
        }
        h->pool_create(1, 0, 0, 0);
        cnt = 4;
        for (int n = 1; n < levs; n++) {
            h->pool_create(1, n, 8 * h->voxcnt(n), cnt ? cnt : 1);
            cnt = std::max(1, cnt >> 1);
        }
        h->ck(cuMemAlloc(&h->cuinfo, sizeof(HVDBInfo)), "info");
        h->make_atlas(1, false);
        h->ck(cuEventCreate(&h->ev0, 0), "ev");
        h->ck(cuEventCreate(&h->ev1, 0), "ev");
    } catch (const std::string& e) {
        fprintf(stderr, "ref harness: %s\n", e.c_str());
        delete h;
        return nullptr;
    }
    return h;
}

int rh_set_points(void* hp, const float* host_xyz, int n) {
    Harness* h = (Harness*)hp;
    try {
        if (h->pts) cuMemFree(h->pts);
        h->ck(cuMemAlloc(&h->pts, (size_t)std::max(n, 1) * 12), "pts");
        if (n) h->ck(cuMemcpyHtoD(h->pts, host_xyz, (size_t)n * 12), "pts");
        h->npts = n;
    } catch (const std::string& e) { h->err = e; return 3; }
    return 0;
}

#define RH_TRY(h, body) try { body; } catch (const std::string& e) { (h)->err = e; fprintf(stderr, "ref harness: %s\n", e.c_str()); return 3; }

int rh_rebuild_topology(void* hp, float radius, const float* orig) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->rebuild_topology(radius, make_float3(orig[0], orig[1], orig[2])));
}
int rh_update_atlas(void* hp) { Harness* h = (Harness*)hp; RH_TRY(h, h->update_atlas(); return 0); }
int rh_insert_subcell(void* hp, float radius, const float* trans, int* len) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, int r = h->insert_subcell(radius, make_float3(trans[0], trans[1], trans[2])); *len = h->sc_len; return r);
}
int rh_insert_subcell_fp16(void* hp, float radius, const float* trans, int* len) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, int r = h->insert_subcell(radius, make_float3(trans[0], trans[1], trans[2]), true); *len = h->sc_len;
           return r);
}
int rh_gather_levelset_fp16(void* hp, float radius) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->gather_levelset_fp16(radius));
}
int rh_update_apron_faces(void* hp) { Harness* h = (Harness*)hp; RH_TRY(h, return h->update_apron_faces()); }
int rh_smooth(void* hp, float p1, float p2, float p3) { Harness* h = (Harness*)hp; RH_TRY(h, return h->smooth(p1, p2, p3)); }
int rh_insert_points(void* hp, const float* trans) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->insert_points(make_float3(trans[0], trans[1], trans[2])));
}
int rh_scatter_density(void* hp, float radius, float amp, const float* trans, int expand) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->scatter_density(radius, amp, make_float3(trans[0], trans[1], trans[2]), expand != 0));
}
int rh_write_bricks(void* hp, int chan, const float* in, int n) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, h->write_bricks(chan, in, n); return 0);
}
int rh_gather(void* hp, int mode, float radius, int accum) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->gather(mode, radius, accum != 0));
}
int rh_update_apron(void* hp, int chan, float boundval) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->update_apron(chan, boundval));
}
int rh_accumulate_topology(void* hp, float radius, const float* orig, int min_depth) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, return h->accumulate_topology(radius, make_float3(orig[0], orig[1], orig[2]), min_depth));
}
// AddChannel(1, T_UCHAR4): a colour channel with the atlas layout of channel 0
int rh_add_colour_channel(void* hp) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, {
        h->colour_chan = true;
        h->make_array(h->carr, h->csurf, true, h->az, false);
        return 0;
    });
}
// point colours (RGBA8 as one uint per point; n must match the last rh_set_points), NULL clears
int rh_set_colors(void* hp, const uint32_t* host_rgba, int n) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, {
        if (h->clr) cuMemFree(h->clr);
        h->clr = 0;
        if (host_rgba) {
            h->ck(cuMemAlloc(&h->clr, (size_t)std::max(n, 1) * 4), "clr");
            if (n) h->ck(cuMemcpyHtoD(h->clr, host_rgba, (size_t)n * 4), "clr");
        }
        return 0;
    });
}
int rh_fill(void* hp, int chan, float v) { Harness* h = (Harness*)hp; RH_TRY(h, h->fill(chan, v); return 0); }
// per-kernel timing: on = 1 starts a new record; rh_kernel_ms returns the summed device
// time of the kernels and Thrust calls launched since
int rh_timing(void* hp, int on) {
    Harness* h = (Harness*)hp;
    h->timing = on != 0;
    h->ntev = 0;
    return 0;
}
float rh_kernel_ms(void* hp) {
    Harness* h = (Harness*)hp;
    try {
        return h->kernel_ms();
    } catch (const std::string& e) {
        h->err = e;
        return -1.0f;
    }
}
int rh_sync(void* hp) { Harness* h = (Harness*)hp; RH_TRY(h, h->ck(cuCtxSynchronize(), "sync"); return 0); }
// CUDA events on the NULL stream, which every launch and copy of the harness uses
int rh_event_begin(void* hp) { Harness* h = (Harness*)hp; RH_TRY(h, h->ck(cuEventRecord(h->ev0, 0), "ev"); return 0); }
float rh_event_end_ms(void* hp) {
    Harness* h = (Harness*)hp;
    float ms = -1.0f;
    if (cuEventRecord(h->ev1, 0) != CUDA_SUCCESS || cuEventSynchronize(h->ev1) != CUDA_SUCCESS ||
        cuEventElapsedTime(&ms, h->ev0, h->ev1) != CUDA_SUCCESS)
        return -1.0f;
    return ms;
}

long long rh_node_count(void* hp, int lev) { return (long long)((Harness*)hp)->pool[0][lev].lastEle; }
long long rh_used_count(void* hp, int lev) { return (long long)((Harness*)hp)->pool[0][lev].usedNum; }
int rh_top_lev(void* hp) { return ((Harness*)hp)->info.top_lev; }
void rh_nodes(void* hp, int lev, void* out) {
    Harness* h = (Harness*)hp;
    memcpy(out, h->pool[0][lev].cpu.data(), h->pool[0][lev].lastEle * 64);
}
void rh_childlist(void* hp, int lev, void* out) {
    Harness* h = (Harness*)hp;
    memcpy(out, h->pool[1][lev].cpu.data(), h->pool[1][lev].lastEle * h->pool[1][lev].stride);
}
void rh_atlas_dims(void* hp, int* out4) {
    Harness* h = (Harness*)hp;
    out4[0] = h->ax; out4[1] = h->ay; out4[2] = h->az; out4[3] = h->atlas_last;
}
void rh_atlas_map(void* hp, int* out) {
    Harness* h = (Harness*)hp;
    memcpy(out, h->amap_cpu.data(), h->amap_cpu.size() * 4);
}
int rh_atlas_bricks(void* hp, int chan, float* out) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, h->read_bricks(chan, out); return 0);
}
// subcell lists: counts/offsets of the first `nsub` subcells and the list points
int rh_subcells(void* hp, int* cnt_out, int* off_out, float* pts_out) {
    Harness* h = (Harness*)hp;
    RH_TRY(h, {
        h->ck(cuMemcpyDtoH(cnt_out, h->sc_cnt, (size_t)h->sc_num * 4), "cnt");
        h->ck(cuMemcpyDtoH(off_out, h->sc_off, (size_t)h->sc_num * 4), "off");
        if (h->sc_len && pts_out) h->ck(cuMemcpyDtoH(pts_out, h->sc_pnts, (size_t)h->sc_len * 12), "pts");
        return 0;
    });
}
int rh_subcell_num(void* hp) { return ((Harness*)hp)->sc_num; }
const char* rh_error(void* hp) { return ((Harness*)hp)->err.c_str(); }

}  // extern "C"
