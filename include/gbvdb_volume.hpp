// gbvdb_volume.hpp -- header-only C++ facade over include/gbvdb.h with the
// method names and argument order of nvdb::VolumeGVDB for the point-driven path
// (source/gvdb_library/src/gvdb_volume_gvdb.h:387-557), so that a reference
// sample's per-frame sequence (e.g. source/gFluidSurface/main_fluid_surface.cpp
// :325-356) compiles against libgbvdb.so unchanged apart from the namespace.
//
// Errors: the reference prints and carries on (logical errors) or exits (CUDA
// errors).  The facade keeps the status of the last call in last_status() and
// prints the message of every failing call to stderr; it never exits.
#ifndef GBVDB_VOLUME_HPP
#define GBVDB_VOLUME_HPP

#include <cstdint>
#include <cstdio>

#include "gbvdb.h"

namespace gbvdb {

typedef unsigned char uchar;
typedef uint64_t uint64;

struct Vector3DF {
    float x, y, z;
    Vector3DF() : x(0), y(0), z(0) {}
    Vector3DF(float a, float b, float c) : x(a), y(b), z(c) {}
};
struct Vector3DI {
    int x, y, z;
    Vector3DI() : x(0), y(0), z(0) {}
    Vector3DI(int a, int b, int c) : x(a), y(b), z(c) {}
};
struct Vector4DF {
    float x, y, z, w;
    Vector4DF() : x(0), y(0), z(0), w(0) {}
    Vector4DF(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};
typedef int64_t slong;
#define ID_UNDEFL 0xFFFFFFFF

// the fields of the reference's DataPtr (gvdb_allocator.h:35-55) that SetPoints reads
struct DataPtr {
    const void* gpu = nullptr;  // device pointer (CUdeviceptr in the reference)
    uint64 lastEle = 0;         // element count
    uint64 stride = 12;         // bytes between elements
    Vector3DI subdim;           // subdim.x = byte offset of the float3 in an element
};

// channel types and filter constants of gvdb_types.h
enum { T_UCHAR = GBVDB_T_UCHAR, T_UCHAR4 = GBVDB_T_UCHAR4, T_FLOAT = GBVDB_T_FLOAT, T_HALF = GBVDB_T_HALF,
       T_BFLOAT16 = GBVDB_T_BFLOAT16 };
enum { F_NEAREST = 0, F_LINEAR = 1, F_MIDPOINT = 2 };
enum { FUNC_SMOOTH = GBVDB_FUNC_SMOOTH };
enum { F_CLAMP = 0, F_BORDER = 1, F_WRAP = 2 };

class VolumeGVDB {
  public:
    VolumeGVDB() = default;
    VolumeGVDB(const VolumeGVDB&) = delete;
    VolumeGVDB& operator=(const VolumeGVDB&) = delete;
    ~VolumeGVDB() {
        if (g_) gbvdb_destroy(g_);
    }

    // SetCudaDevice + Initialize (VG.cpp:240-334, 2320-2361)
    void SetCudaDevice(int devid) { chk(gbvdb_create(devid < 0 ? 0 : devid, &g_), "SetCudaDevice"); }
    void Initialize() {}
    void SetStream(void* cuda_stream) { chk(gbvdb_set_stream(g_, cuda_stream), "SetStream"); }

    // Configure (VG.cpp:2364-2434)
    void Configure(int q4, int q3, int q2, int q1, int q0) { chk(gbvdb_configure5(g_, q4, q3, q2, q1, q0), "Configure"); }
    void Configure(int levs, int* r, int* numcnt, bool use_masks = false) {
        (void)numcnt;
        (void)use_masks;
        chk(gbvdb_configure(g_, levs, r), "Configure");
    }
    void SetChannelDefault(int cx, int cy, int cz) { chk(gbvdb_set_channel_default(g_, cx, cy, cz), "SetChannelDefault"); }
    void AddChannel(uchar chan, int dt, int apron, int filter = F_LINEAR, int border = F_CLAMP,
                    Vector3DI axiscnt = Vector3DI(0, 0, 0)) {
        (void)filter;
        (void)border;
        chk(gbvdb_add_channel(g_, chan, dt, apron, axiscnt.x, axiscnt.y, axiscnt.z), "AddChannel");
    }

    // SetDataGPU (VG.cpp:4872-4880): a non-owning view of user device memory
    void SetDataGPU(DataPtr& p, uint64 cnt, const void* gpu, int offs, int stride) {
        p.gpu = gpu;
        p.lastEle = cnt;
        p.stride = (uint64)stride;
        p.subdim = Vector3DI(offs, 0, 0);
    }
    // SetPoints (VG.cpp:4900-4908)
    void SetPoints(DataPtr& pnts, DataPtr& vel, DataPtr& clr) {
        chk(gbvdb_set_points(g_, pnts.gpu, (int64_t)pnts.lastEle, pnts.subdim.x, (int)pnts.stride, vel.gpu,
                             vel.subdim.x, (int)vel.stride, clr.gpu, clr.subdim.x, (int)clr.stride),
            "SetPoints");
    }

    // topology (VG.cpp:1158-1218, 1579-1593, 2630-2704)
    void RebuildTopology(int num_pnts, float radius, Vector3DF orig) {
        float o[3] = {orig.x, orig.y, orig.z};
        chk(gbvdb_rebuild_topology(g_, num_pnts, radius, o), "RebuildTopology");
    }
    void AccumulateTopology(int num_pnts, float radius, Vector3DF orig, int iDepth = 1) {
        float o[3] = {orig.x, orig.y, orig.z};
        chk(gbvdb_accumulate_topology(g_, num_pnts, radius, o, iDepth), "AccumulateTopology");
    }
    void RequestFullRebuild(bool tf) { chk(gbvdb_request_full_rebuild(g_, tf ? 1 : 0), "RequestFullRebuild"); }
    void FinishTopology(bool pCommitPool = true, bool pComputeBounds = true) {
        chk(gbvdb_finish_topology(g_, pCommitPool ? 1 : 0, pComputeBounds ? 1 : 0), "FinishTopology");
    }
    void UpdateAtlas() { chk(gbvdb_update_atlas(g_), "UpdateAtlas"); }
    // the host topology path (VG.cpp:1220-1227, 2766-2774): ActivateSpace returns the existing
    // leaf's id, or ID_UNDEFL for a new leaf; the next call that reads the topology commits
    slong ActivateSpace(Vector3DF pos) {
        float p[3] = {pos.x, pos.y, pos.z};
        uint64_t id = ID_UNDEFL;
        if (chk(gbvdb_activate_space(g_, p, &id), "ActivateSpace") != GBVDB_OK) return (slong)ID_UNDEFL;
        return (slong)id;
    }
    void RebuildTopologyCPU(int pNumPnts, Vector3DF pOrig, Vector3DF* pPos) {
        float o[3] = {pOrig.x, pOrig.y, pOrig.z};
        chk(gbvdb_rebuild_topology_cpu(g_, pNumPnts, o, pPos, (int)sizeof(Vector3DF)), "RebuildTopologyCPU");
    }

    // points to voxels (VG.cpp:4971-5092, 5318-5373)
    void InsertPointsSubcell(int subcell_size, int num_pnts, float pRadius, Vector3DF trans, int& pSCPntsLength) {
        float t[3] = {trans.x, trans.y, trans.z};
        int64_t len = pSCPntsLength;
        if (chk(gbvdb_insert_points_subcell(g_, subcell_size, num_pnts, pRadius, t, &len), "InsertPointsSubcell") ==
            GBVDB_OK)
            pSCPntsLength = (int)len;
    }
    void GatherDensity(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                       int chanDensity, int chanClr, bool bAccum = false) {
        float t[3] = {trans.x, trans.y, trans.z};
        chk(gbvdb_gather_density(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanDensity, chanClr,
                                 bAccum ? 1 : 0),
            "GatherDensity");
    }
    void GatherLevelSet(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                        int chanLevelset, int chanClr, bool bAccum = false) {
        float t[3] = {trans.x, trans.y, trans.z};
        chk(gbvdb_gather_levelset(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanLevelset, chanClr,
                                  bAccum ? 1 : 0),
            "GatherLevelSet");
    }
    // FP16 subcell variants (VG.cpp:5094-5189, 5375-5401)
    void InsertPointsSubcell_FP16(int subcell_size, int num_pnts, float pRadius, Vector3DF trans, int& pSCPntsLength) {
        float t[3] = {trans.x, trans.y, trans.z};
        int64_t len = pSCPntsLength;
        if (chk(gbvdb_insert_points_subcell_fp16(g_, subcell_size, num_pnts, pRadius, t, &len),
                "InsertPointsSubcell_FP16") == GBVDB_OK)
            pSCPntsLength = (int)len;
    }
    void GatherLevelSet_FP16(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                             int chanLevelset, int chanClr) {
        float t[3] = {trans.x, trans.y, trans.z};
        chk(gbvdb_gather_levelset_fp16(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanLevelset, chanClr),
            "GatherLevelSet_FP16");
    }
    // legacy InsertPoints / ScatterDensity (VG.cpp:5219-5267, 5624-5660)
    void InsertPoints(int num_pnts, Vector3DF trans, bool bPrefix = false) {
        float t[3] = {trans.x, trans.y, trans.z};
        chk(gbvdb_insert_points(g_, num_pnts, t, bPrefix ? 1 : 0), "InsertPoints");
    }
    void ScatterDensity(int num_pnts, float radius, float amp, Vector3DF trans, bool expand = true,
                        bool avgColor = false) {
        float t[3] = {trans.x, trans.y, trans.z};
        chk(gbvdb_scatter_density(g_, num_pnts, radius, amp, t, expand ? 1 : 0, avgColor ? 1 : 0), "ScatterDensity");
    }
    // UpdateApron (VG.cpp:4411-4457)
    void UpdateApron(uchar chan, float boundval = 0.0f, bool changeCtx = true) {
        (void)changeCtx;
        chk(gbvdb_update_apron(g_, chan, boundval), "UpdateApron");
    }
    void FillChannel(uchar chan, Vector4DF val) {
        float v[4] = {val.x, val.y, val.z, val.w};
        chk(gbvdb_fill_channel4(g_, chan, v), "FillChannel");
    }
    void FillChannel(uchar chan, float value) { chk(gbvdb_fill_channel(g_, chan, value), "FillChannel"); }
    void ClearChannel(uchar chan) { chk(gbvdb_clear_channel(g_, chan), "ClearChannel"); }

    // UpdateNeighbors / UpdateApronFaces / Compute(FUNC_SMOOTH) (VG.cpp:2527-2556, 4461-4496, 4532-4558)
    void UpdateNeighbors() { chk(gbvdb_update_neighbors(g_), "UpdateNeighbors"); }
    void UpdateApronFaces(uchar chan) { chk(gbvdb_update_apron_faces(g_, chan), "UpdateApronFaces"); }
    void Compute(int effect, uchar chan, int num_iterations, Vector3DF params, bool bUpdateApron,
                 bool skipOverAprons = true, float boundval = 0.0f) {
        float p[3] = {params.x, params.y, params.z};
        chk(gbvdb_compute(g_, effect, chan, num_iterations, p, bUpdateApron ? 1 : 0, skipOverAprons ? 1 : 0, boundval),
            "Compute");
    }

    // SaveVBX / LoadVBX (VG.cpp:1626-1767, 507-683)
    void SaveVBX(const char* fname) { chk(gbvdb_save_vbx(g_, fname), "SaveVBX"); }
    bool LoadVBX(const char* fname) { return chk(gbvdb_load_vbx(g_, fname), "LoadVBX") == GBVDB_OK; }

    // accessors (VG.h:563-564, 637-641)
    uint64 getNumTotalNodes(int lev) {
        int64_t tot[10], used[10];
        if (chk(gbvdb_get_node_counts(g_, tot, used), "getNumTotalNodes") != GBVDB_OK || lev < 0 || lev >= 10) return 0;
        return (uint64)tot[lev];
    }
    uint64 getNumUsedNodes(int lev) {
        int64_t tot[10], used[10];
        if (chk(gbvdb_get_node_counts(g_, tot, used), "getNumUsedNodes") != GBVDB_OK || lev < 0 || lev >= 10) return 0;
        return (uint64)used[lev];
    }
    Vector3DF getBoundMin() {
        float b[6] = {0, 0, 0, 0, 0, 0};
        gbvdb_get_point_bounds(g_, b);
        return Vector3DF(b[0], b[1], b[2]);
    }
    Vector3DF getBoundMax() {
        float b[6] = {0, 0, 0, 0, 0, 0};
        gbvdb_get_point_bounds(g_, b);
        return Vector3DF(b[3], b[4], b[5]);
    }

    // getVolMin / getVolMax (gvdb_volume_base.h:57-59): bounds of the last FinishTopology
    Vector3DF getVolMin() {
        float b[6] = {0, 0, 0, 0, 0, 0};
        gbvdb_get_vol_bounds(g_, b);
        return Vector3DF(b[0], b[1], b[2]);
    }
    Vector3DF getVolMax() {
        float b[6] = {0, 0, 0, 0, 0, 0};
        gbvdb_get_vol_bounds(g_, b);
        return Vector3DF(b[3], b[4], b[5]);
    }

    gbvdb_grid handle() const { return g_; }
    gbvdb_status last_status() const { return last_; }

  private:
    gbvdb_status chk(gbvdb_status st, const char* what) {
        last_ = st;
        if (st != GBVDB_OK && st != GBVDB_NOOP)
            std::fprintf(stderr, "gbvdb: %s failed (%d): %s\n", what, (int)st, g_ ? gbvdb_last_error(g_) : "");
        return st;
    }
    gbvdb_grid g_ = nullptr;
    gbvdb_status last_ = GBVDB_OK;
};

}  // namespace gbvdb

#endif  // GBVDB_VOLUME_HPP
