/*
 * gbvdb.h -- C ABI of the GB300-native point-driven dynamic-topology path of
 * GVDB Voxels (libgbvdb.so).
 *
 * Each entry point replaces one method of the reference class nvdb::VolumeGVDB
 * (source/gvdb_library/src/gvdb_volume_gvdb.h) for the path
 *   RebuildTopology -> UpdateAtlas -> InsertPointsSubcell -> Gather* -> UpdateApron
 * with the same argument meaning.  Signatures use plain pointers and sizes
 * only.  Point buffers are borrowed DEVICE pointers (as DataPtr.gpu in the
 * reference); the grid owns all other device memory.  Every call returns a
 * gbvdb_status instead of printing and calling exit() (the reference's
 * cudaCheck, gvdb_allocator.cpp:1006-1034).  All work is issued on the grid's
 * stream (gbvdb_set_stream; default: the legacy NULL stream).
 *
 * Layouts kept from the reference:
 *   - node records: 64 bytes, gvdb_node.h:27-40 (mLev, mFlags, mPriority, pad,
 *     mPos int3, mValue int3, mVRange float3, mParent u64, mChildList u64, mMask u64);
 *   - pool references Elem(grp,lev,ndx) = grp | lev<<8 | ndx<<16 (gvdb_allocator.h:59-62);
 *   - child lists: res^3 u64 per node, 0xFF..FF = empty (no bitmasks);
 *   - atlas addressing: slot id -> (id%ax, (id/ax)%ay, id/(ax*ay))*18 + apron
 *     (gvdb_allocator.cpp:705-715), 16^3 bricks with a 1-voxel apron;
 *   - atlas map entries {int3 pos, int leaf} (cuda_gvdb_nodes.cuh:38-41).
 * The physical atlas storage is brick-major (see gbvdb_export_atlas_bricks);
 * exported bricks are 18^3 with the apron, [z][y][x].
 */
#ifndef GBVDB_H
#define GBVDB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBVDB_API __attribute__((visibility("default")))
#else
#define GBVDB_API
#endif

typedef struct gbvdb_grid_s* gbvdb_grid;

typedef enum {
    GBVDB_OK = 0,
    GBVDB_INVALID_ARG = 1,        /* bad argument or call order */
    GBVDB_OUT_OF_MEMORY = 2,      /* device or host allocation failed */
    GBVDB_CUDA_ERROR = 3,         /* a CUDA runtime call failed; see gbvdb_last_error */
    GBVDB_DEPTH_UNSUPPORTED = 4,  /* point extents < 1 brick or > 5 levels (VG.cpp:1187-1194) */
    GBVDB_CAPACITY = 5,           /* a device capacity was exceeded; retry was not possible */
    GBVDB_TIMEOUT = 6,            /* a bounded device wait gave up */
    GBVDB_NOT_SUPPORTED = 7,      /* configuration outside what this library implements */
    GBVDB_NOOP = 8                /* nothing to do (the reference returns early here) */
} gbvdb_status;

/* channel element types: the reference's T_* codes (gvdb_types.h) plus two storage extensions */
#define GBVDB_T_UCHAR 0
#define GBVDB_T_UCHAR4 2    /* RGBA8 colour channel (gathered colour averages) */
#define GBVDB_T_FLOAT 3
#define GBVDB_T_HALF 100    /* extension: FP16 storage, FP32 accumulation */
#define GBVDB_T_BFLOAT16 101 /* extension: BF16 storage, FP32 accumulation */

/* --- lifetime ------------------------------------------------------------ */
/* SetCudaDevice + Initialize (gvdb_volume_gvdb.cpp:240-334, 2320-2361) */
GBVDB_API gbvdb_status gbvdb_create(int device, gbvdb_grid* out);
GBVDB_API gbvdb_status gbvdb_destroy(gbvdb_grid g);
/* all work of this grid goes to `stream` (a cudaStream_t) */
GBVDB_API gbvdb_status gbvdb_set_stream(gbvdb_grid g, void* stream);
/* message of the last failing call on this grid */
GBVDB_API const char* gbvdb_last_error(gbvdb_grid g);

/* --- configuration ------------------------------------------------------- */
/* Configure(levs, r, numcnt) (gvdb_volume_gvdb.cpp:2380-2434); log2dim[0] = leaf */
GBVDB_API gbvdb_status gbvdb_configure(gbvdb_grid g, int levs, const int* log2dim_leaf_first);
/* Configure(q4, q3, q2, q1, q0) (gvdb_volume_gvdb.cpp:2364-2377) */
GBVDB_API gbvdb_status gbvdb_configure5(gbvdb_grid g, int q4, int q3, int q2, int q1, int q0);
/* SetChannelDefault (gvdb_volume_gvdb.h:390) */
GBVDB_API gbvdb_status gbvdb_set_channel_default(gbvdb_grid g, int ax, int ay, int az);
/* AddChannel(chan, dt, apron, filter, border, axiscnt) (gvdb_volume_gvdb.cpp:2437-2453);
 * apron must be 1 (the reference's kernels assume it, VG.cpp:4448) */
GBVDB_API gbvdb_status gbvdb_add_channel(gbvdb_grid g, int chan, int dtype, int apron,
                                         int ax, int ay, int az);
/* SetPoints / SetDataGPU (gvdb_volume_gvdb.cpp:4900-4908, 4872-4880): position i is the
 * float3 at pos + i*stride + off.  vel and clr may be NULL; clr (device memory) holds one
 * RGBA8 colour per point as the uint32 at clr + i*clr_stride + clr_off (R in the low byte,
 * cuda_gvdb_particles.cuh:236): InsertPointsSubcell then carries colours into its lists
 * and the gathers average them into their chanClr channel. */
GBVDB_API gbvdb_status gbvdb_set_points(gbvdb_grid g, const void* dev_pos, int64_t n, int off, int stride,
                                        const void* dev_vel, int vel_off, int vel_stride,
                                        const void* dev_clr, int clr_off, int clr_stride);

/* --- topology ------------------------------------------------------------ */
/* RebuildTopology(num_pnts, radius, orig) (gvdb_volume_gvdb.cpp:1181-1218) */
GBVDB_API gbvdb_status gbvdb_rebuild_topology(gbvdb_grid g, int64_t n, float radius, const float orig[3]);
/* AccumulateTopology(num_pnts, radius, orig, iDepth) (gvdb_volume_gvdb.cpp:1158-1178) */
GBVDB_API gbvdb_status gbvdb_accumulate_topology(gbvdb_grid g, int64_t n, float radius, const float orig[3],
                                                 int min_depth);
/* RequestFullRebuild (gvdb_volume_gvdb.h:432) */
GBVDB_API gbvdb_status gbvdb_request_full_rebuild(gbvdb_grid g, int tf);
/* FinishTopology(commit, bounds) (gvdb_volume_gvdb.cpp:1579-1593): bounds of the active leaves */
GBVDB_API gbvdb_status gbvdb_finish_topology(gbvdb_grid g, int commit_pool, int compute_bounds);
/* UpdateAtlas (gvdb_volume_gvdb.cpp:2630-2704) */
GBVDB_API gbvdb_status gbvdb_update_atlas(gbvdb_grid g);
/* ActivateSpace(Vector3DF pos) (gvdb_volume_gvdb.cpp:2766-2774, 2795-2855): the host topology
 * path.  Activates the leaf holding the truncated position, creating the nodes above it and
 * growing the root upwards (Reparent) as the reference does, on host copies of the pools
 * (fetched from the device at the first activation).  *out_node (may be NULL) receives the
 * leaf's Elem reference when it existed, else 0xFFFFFFFF (ID_UNDEFL).  Every other entry
 * point first commits pending activations to the device pools (PoolCommitAll); a later
 * RebuildTopology then starts from an empty grid. */
GBVDB_API gbvdb_status gbvdb_activate_space(gbvdb_grid g, const float pos[3], uint64_t* out_node);
/* RebuildTopologyCPU(num_pnts, orig, pos) (gvdb_volume_gvdb.cpp:1220-1227): ActivateSpace of
 * pos[i] + orig for n HOST float3 positions, element i at host_pos + i*stride (0 = 12) */
GBVDB_API gbvdb_status gbvdb_rebuild_topology_cpu(gbvdb_grid g, int64_t n, const float orig[3],
                                                  const void* host_pos, int stride);

/* --- points to voxels ---------------------------------------------------- */
/* InsertPointsSubcell(subcell_size, num_pnts, radius, trans, &len) (gvdb_volume_gvdb.cpp:4971-5092);
 * *out_len receives the total subcell list length pSCPntsLength. */
GBVDB_API gbvdb_status gbvdb_insert_points_subcell(gbvdb_grid g, int subcell_size, int64_t n, float radius,
                                                   const float trans[3], int64_t* out_len);
/* GatherDensity (gvdb_volume_gvdb.cpp:5318-5344): v = max(accum ? old : 0, max_j(radius - |p_j - v|)).
 * When the last insert carried point colours, clr_chan must be a GBVDB_T_UCHAR4 channel: every
 * voxel of a subcell gets the mean of the subcell's member colours, started from its old
 * colour with accum (else from (0, 0, 0, 255)) and divided by (members + accum)
 * (cuda_gvdb_particles.cuh:717-731).  The member bytes are summed exactly as integers and
 * divided by 255 once (the reference adds FP32 terms c/255 in the arbitrary order of its
 * lists), so a byte may differ from the reference's by one. */
GBVDB_API gbvdb_status gbvdb_gather_density(gbvdb_grid g, int subcell_size, int64_t n, float radius,
                                            const float trans[3], int64_t sc_len, int chan, int clr_chan,
                                            int accum);
/* GatherLevelSet (gvdb_volume_gvdb.cpp:5348-5373): v = min(accum ? old : 3, min_j(|p_j - v| - radius));
 * colours as GatherDensity (cuda_gvdb_particles.cuh:757-771) */
GBVDB_API gbvdb_status gbvdb_gather_levelset(gbvdb_grid g, int subcell_size, int64_t n, float radius,
                                             const float trans[3], int64_t sc_len, int chan, int clr_chan,
                                             int accum);
/* InsertPointsSubcell_FP16 (gvdb_volume_gvdb.cpp:5094-5189, cuda_gvdb_particles.cuh:154-216): as
 * InsertPointsSubcell, with positions stored at 16 bits per axis over the bounds of the last
 * RebuildTopology (q = trunc((w - PosMin) / PosRange * 65535)); gathers that follow read the
 * dequantised positions q / 65535 * PosRange + PosMin. */
GBVDB_API gbvdb_status gbvdb_insert_points_subcell_fp16(gbvdb_grid g, int subcell_size, int64_t n, float radius,
                                                        const float trans[3], int64_t* out_len);
/* GatherLevelSet_FP16 (gvdb_volume_gvdb.cpp:5375-5401, cuda_gvdb_particles.cuh:775-811):
 * v = min(3, min_j(|p_j - v| - radius)) over the stored positions, no accumulation */
GBVDB_API gbvdb_status gbvdb_gather_levelset_fp16(gbvdb_grid g, int subcell_size, int64_t n, float radius,
                                                  const float trans[3], int64_t sc_len, int chan, int clr_chan);
/* Legacy InsertPoints(num_pnts, trans, bPrefix) (gvdb_volume_gvdb.cpp:5219-5267,
 * cuda_gvdb_particles.cuh:19-68): the leaf holding each point (w = p + trans, -1 where none)
 * and the points grouped by leaf. */
GBVDB_API gbvdb_status gbvdb_insert_points(gbvdb_grid g, int64_t n, const float trans[3], int prefix);
/* Legacy ScatterDensity(num_pnts, radius, amp, trans, expand, avgColor) (gvdb_volume_gvdb.cpp
 * :5624-5660, cuda_gvdb_particles.cuh:516-571): channel 0 (FP32) += distFunc of every point
 * grouped by the last InsertPoints at the voxel it lies in (and its six face neighbours with
 * expand), c = d^2 / r^2, 1 + c*(-3 + c*(3 - c)); amp is unused as in the reference kernel,
 * colour averaging is not supported. */
GBVDB_API gbvdb_status gbvdb_scatter_density(gbvdb_grid g, int64_t n, float radius, float amp, const float trans[3],
                                             int expand, int avg_color);
/* the last InsertPoints: leaf per point (n int32), group offsets (leaves + 1) and grouped points
 * (float3; order inside a group unspecified, as the reference's atomic ranks); NULL skips one */
GBVDB_API gbvdb_status gbvdb_export_point_leaves(gbvdb_grid g, int32_t* pnode, int64_t cap, int64_t* offsets,
                                                 int64_t cap_offsets, float* points, int64_t cap_points);
/* UpdateApron(chan, boundval) (gvdb_volume_gvdb.cpp:4418-4457, cuda_gvdb_operators.cuh:72-131) */
GBVDB_API gbvdb_status gbvdb_update_apron(gbvdb_grid g, int chan, float boundval);
/* FillChannel(chan, Vector4DF) (gvdb_volume_gvdb.cpp:2456-2470): every voxel of every slot of
 * the atlas, interior and apron; float channels take value[0], T_UCHAR4 channels
 * CLR2INT(value[0], value[1], value[2], 1) (cuda_gvdb_operators.cuh:20, 368-373) */
GBVDB_API gbvdb_status gbvdb_fill_channel4(gbvdb_grid g, int chan, const float value[4]);
/* FillChannel with (value, 0, 0, 0) */
GBVDB_API gbvdb_status gbvdb_fill_channel(gbvdb_grid g, int chan, float value);
/* ClearChannel (gvdb_volume_gvdb.cpp:1596-1603): every voxel of the channel's atlas to 0 */
GBVDB_API gbvdb_status gbvdb_clear_channel(gbvdb_grid g, int chan);

/* --- state and export (for parity checks, VBX and consumers) -------------- */
/* depth of the last build, traversal top level (VG.cpp:3957-3968) */
GBVDB_API gbvdb_status gbvdb_get_depth(gbvdb_grid g, int* depth, int* top_lev);
/* getNumTotalNodes / getNumUsedNodes per level (gvdb_volume_gvdb.h:637-641); arrays of 10 */
GBVDB_API gbvdb_status gbvdb_get_node_counts(gbvdb_grid g, int64_t* total, int64_t* used);
/* getBoundMin/Max (gvdb_volume_gvdb.h:563-564): 6 floats */
GBVDB_API gbvdb_status gbvdb_get_point_bounds(gbvdb_grid g, float* out6);
/* getVolMin/getVolMax (gvdb_volume_base.h:57-59): the bounds ComputeBounds set at the last
 * FinishTopology(.., compute_bounds = 1) (gvdb_volume_gvdb.cpp:1792-1816): both corners start
 * at leaf 0 of the pool, each flagged leaf widens them by [pos, pos + brick range).
 * 6 floats {min xyz, max xyz}; GBVDB_NOOP before any such call. */
GBVDB_API gbvdb_status gbvdb_get_vol_bounds(gbvdb_grid g, float* out6);
/* node pool of one level as 64-byte records (host buffer, `cap` records) */
GBVDB_API gbvdb_status gbvdb_export_nodes(gbvdb_grid g, int lev, void* host_out, int64_t cap);
/* child-list pool of one level (res^3 u64 per node) */
GBVDB_API gbvdb_status gbvdb_export_childlist(gbvdb_grid g, int lev, uint64_t* host_out, int64_t cap);
/* info[8] = {ax, ay, az, used_slots, dtype, apron, brick_res(18), bytes_per_voxel} */
GBVDB_API gbvdb_status gbvdb_get_atlas_info(gbvdb_grid g, int chan, int* info8);
/* padded bricks of slots [0, used): used * 18^3 voxels, [slot][z][y][x], storage type */
GBVDB_API gbvdb_status gbvdb_export_atlas_bricks(gbvdb_grid g, int chan, void* host_out, int64_t cap_bytes);
/* atlas map (16 bytes per slot, ax*ay*az entries) */
GBVDB_API gbvdb_status gbvdb_export_atlas_map(gbvdb_grid g, void* host_out, int64_t cap);
/* materialized subcell lists of the last InsertPointsSubcell: offsets[nsub+1] (nsub = 64 *
 * linked leaves, subcells in reference order) and float3 points; the order inside one list
 * is unspecified, as in the reference (PT.cuh:266 uses atomicAdd slots) */
GBVDB_API gbvdb_status gbvdb_export_subcells(gbvdb_grid g, int64_t* offsets, int64_t cap_offsets,
                                             float* points, int64_t cap_points);
/* UpdateNeighbors (gvdb_volume_gvdb.cpp:2527-2556): per leaf of the pool, the leaves one
 * brick away along -x, -y, -z, +x, +y, +z (-1 where none); the table serves UpdateApronFaces
 * until the topology changes.  Export: 6 int32 per leaf. */
GBVDB_API gbvdb_status gbvdb_update_neighbors(gbvdb_grid g);
GBVDB_API gbvdb_status gbvdb_export_neighbors(gbvdb_grid g, int32_t* host_out, int64_t cap);
/* UpdateApronFaces (gvdb_volume_gvdb.cpp:4461-4496, cuda_gvdb_operators.cuh:27-61): the six
 * apron faces of every assigned slot from its neighbours' interiors (edges and corners are
 * not written; a missing neighbour leaves the face as it is) */
GBVDB_API gbvdb_status gbvdb_update_apron_faces(gbvdb_grid g, int chan);
/* Compute(effect, chan, iterations, params, bUpdateApron, skipOverAprons, boundval)
 * (gvdb_volume_gvdb.cpp:4532-4558) for effect FUNC_SMOOTH (cuda_gvdb_operators.cuh:383-400):
 * per pass v = (p1*c + the six face neighbours) / (p1 + 6) + p2 on the interior voxels of
 * an FP32 channel, then UpdateApron(chan, boundval) when update_apron is set */
#define GBVDB_FUNC_SMOOTH 113
GBVDB_API gbvdb_status gbvdb_compute(gbvdb_grid g, int effect, int chan, int iterations, const float params[3],
                                     int update_apron, int skip_aprons, float boundval);
/* SaveVBX / LoadVBX (gvdb_volume_gvdb.cpp:1626-1767, 507-683; GVDB_FILESPEC.txt): version
 * 1.11, one grid, identity transform, GVDB topology pools and every channel 0..k-1 in the
 * atlas layout (FP16 / BF16 channels carry their extension type codes 100 / 101).  Loading
 * accepts 1.x / 2.x files without node bitmasks, float grids, uncompressed, atlas layout,
 * 16^3 bricks with apron 1, and ends with UpdateAtlas as the reference does. */
GBVDB_API gbvdb_status gbvdb_save_vbx(gbvdb_grid g, const char* path);
GBVDB_API gbvdb_status gbvdb_load_vbx(gbvdb_grid g, const char* path);
/* FP64 sum of the interior voxels of all assigned slots (total-mass check) */
GBVDB_API gbvdb_status gbvdb_checksum(gbvdb_grid g, int chan, double* out);
/* gbvdb_checksum written to the DEVICE pointer dev_out on the grid's stream, without a
 * host synchronisation (no counterpart in the reference): for pipelined callers that read
 * the result back asynchronously.  May allocate (per-slot partials). */
GBVDB_API gbvdb_status gbvdb_checksum_device(gbvdb_grid g, int chan, double* dev_out);
/* gbvdb_checksum_device issued on the grid's own side stream (no counterpart in the
 * reference): ordered after the grid's work so far, it runs while the grid's stream
 * goes on (a frame's checksum overlaps the next frame's topology, atlas and binning);
 * it reads the channel interiors only, so every later entry point of the grid that
 * writes or reallocates them (the gathers, fills, apron and operator calls, and an
 * UpdateAtlas that grows the atlas) makes the grid's stream wait for it first.  dev_out (device) receives the FP64 sum and host_out (pinned host
 * memory, may be NULL) its copy, both on the side stream.  gbvdb_join makes the grid's
 * stream wait for it explicitly: after gbvdb_join and a synchronisation of the grid's
 * stream, host_out holds the sum. */
GBVDB_API gbvdb_status gbvdb_checksum_overlap(gbvdb_grid g, int chan, double* dev_out, double* host_out);
GBVDB_API gbvdb_status gbvdb_join(gbvdb_grid g);
/* Allocation-free variant of gbvdb_checksum (no counterpart in the reference).
 * For callers that may not allocate device memory: a host application that owns
 * every device allocation and forbids its plugins to call cudaMalloc, or a
 * serving loop admitting jobs against a fixed memory budget.  It calls no
 * cudaMalloc, cudaFree or allocating library routine and does not synchronize:
 * the FP64 sum is written to the DEVICE pointer dev_out on the grid's stream.
 * Scratch is a file-scope device array of 65,536 FP64 per-slot partial sums
 * (512 KiB, held by every GPU that loads the library until exit); grids with
 * more assigned atlas slots are rejected with GBVDB_CAPACITY.  The first call on
 * a device looks up that array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU (different streams or grids without ordering) race.
 * The looked-up address is kept for the life of the process: resetting a device
 * (cudaDeviceReset) while the library is loaded is not supported. */
GBVDB_API gbvdb_status gbvdb_checksum_noalloc(gbvdb_grid g, int chan, double* dev_out);
/* The grid as the reference's VDBInfo (cuda_gvdb_nodes.cuh:42-67, uploaded by PrepareVDB,
 * gvdb_volume_gvdb.cpp:3946-3989) for user kernels: struct gbvdb_vdb_info of
 * include/gbvdb_device.cuh (same layout; per channel the interior and apron-record base
 * addresses in place of the texture / surface objects, read and written with
 * gbvdb_atlas_read / gbvdb_atlas_write at the reference's atlas coordinates).  Written to
 * host memory (bytes >= sizeof(gbvdb_vdb_info)); valid until the next call that changes
 * the topology or the atlas.  From this call on every UpdateApron copies all apron voxels,
 * as after gbvdb_get_atlas_device. */
GBVDB_API gbvdb_status gbvdb_get_vdb_info(gbvdb_grid g, void* host_out, int64_t bytes);
/* device pointers of the atlas storage (interior bricks, apron records) for consumers.
 * A caller holding these pointers may write the interior at any time, so from this
 * call on every UpdateApron of the grid copies the interiors as they are (the
 * fused apron of GBVDB_TUNE_FUSED_APRON is turned off for the grid). */
GBVDB_API gbvdb_status gbvdb_get_atlas_device(gbvdb_grid g, int chan, void** interior, void** apron);
/* tuning parameters (no counterpart in the reference) */
#define GBVDB_TUNE_DENSE_MIN 1   /* candidate points per brick above which gathers use the warp-per-subcell
                                    form instead of the scatter form (default 2048; setting it turns the
                                    autotuner off) */
#define GBVDB_TUNE_AUTOTUNE 3    /* 1 (default): the gathers of a workload try 2048 and 4096 for the
                                    threshold above, timed with events on the grid's stream, and keep the
                                    faster; a linked-brick count that changes by more than 2x starts a new
                                    round.  Both forms give the same bits.  0: the threshold stays fixed. */
#define GBVDB_TUNE_FUSED_APRON 2 /* 1 (default): a gather (binned form, apron 1, dense leaf lookup) also
                                    writes every brick's boundary voxels into its neighbours' apron records,
                                    and the next UpdateApron of that channel, with no topology, atlas or
                                    interior change in between, only writes the faces of missing neighbours
                                    (boundval); the atlas ends bit-identical to a full UpdateApron.  0: every
                                    UpdateApron copies all apron voxels (the reference's kernel). */
#define GBVDB_TUNE_TOUCH_DIRS 4  /* 1 (default): the box passes of RebuildTopology (extra and incremental
                                    bricks) record, per home leaf position, the set of the 27 neighbour
                                    directions its points' boxes reach, when no box reaches past a
                                    neighbour; 0: every point walks its box positions.  Same node sets. */
#define GBVDB_TUNE_TABLE 5        /* 1 (default): when a tuning table is loaded (JSON from $GBVDB_TUNE_TABLE, else
                                     tune_table.json beside libgbvdb.so; written by gvdb-voxels_gb300/tune.py), an
                                     insert or gather of n points takes its bucket's settings: the dense-form
                                     threshold (in place of the autotuner), the gather's resident blocks per SM
                                     and launch order, and the binning passes' points per thread.  0: built-in
                                     defaults. */
#define GBVDB_TUNE_BIN_UNROLL 6   /* points per thread of the subcell count pass: 1, 2 or 4 (0: table / default 2) */
#define GBVDB_TUNE_SCATTER_UNROLL 7 /* points per thread of the binning scatter: 2, 4 or 8 (0: table / default 4) */
#define GBVDB_TUNE_GATHER_BLOCKS 8  /* resident blocks per SM the gather is built for: 10 or 8 (0: table / 10) */
#define GBVDB_TUNE_GATHER_LONG_MIN 10 /* launch order of the gather's bricks: those with more candidate points
                                         than this (capped at the dense-form threshold) first, the rest after;
                                         -1: linked order; 0: table / default 2048.  Same bits either way. */
#define GBVDB_TUNE_KEYSET 9  /* key sets of RebuildTopology's passes: per-level bitmaps over the points' key
                                domain (bounding box plus margin, clipped to the root; cost grows with the
                                domain, at most 2^34 node positions), or hash tables of the keys, compacted and
                                radix-sorted (cost grows with the points; no domain limit, as the reference's
                                Thrust sort of brick keys).  0 (default): the tables when the domain has more
                                than 64 positions per point key (n points x levels) + 2^21, or more than 2^34;
                                1: the bitmaps while they fit; 2: always the tables.  Same pools either way. */
GBVDB_API gbvdb_status gbvdb_set_tuning(gbvdb_grid g, int param, int64_t value);
/* where the tuning table was read from, or "" when none was loaded */
GBVDB_API const char* gbvdb_tune_table_source(void);
/* timing of the last call per stage (ms, CUDA events) when profiling is enabled */
GBVDB_API gbvdb_status gbvdb_set_profile(gbvdb_grid g, int enable);
GBVDB_API gbvdb_status gbvdb_get_stage_times(gbvdb_grid g, double* ms, int cap);
/* out4 = {kernel launches issued so far, host readbacks so far, last subcell-list length,
 * linked leaves of the last insert} */
GBVDB_API gbvdb_status gbvdb_get_stats(gbvdb_grid g, int64_t* out4);
/* the same counters and more, the first cap of: {kernel launches, host readbacks, last
 * subcell-list length, last bricks in the subcell lists, RebuildTopology key passes that
 * used the hash-table key sets} */
GBVDB_API gbvdb_status gbvdb_get_stats_ex(gbvdb_grid g, int64_t* out, int cap);
/* device bytes held by the grid (pools, atlas, scratch; no counterpart in the reference) */
GBVDB_API gbvdb_status gbvdb_get_device_bytes(gbvdb_grid g, int64_t* out);

/* --- served form (no counterpart in the reference) -------------------------
 * A request loop over voxelize-and-gather jobs: worker threads, each with its
 * own stream and reusable grid, run queued jobs concurrently on the device.  A
 * job is the per-frame sequence SetPoints, RebuildTopology, UpdateAtlas,
 * InsertPointsSubcell(4), GatherDensity / GatherLevelSet into channel 0,
 * UpdateApron(0, boundval), then the FP64 checksum of channel 0.  With
 * resident_id >= 0 the job runs on a grid kept on the device under that id
 * (created on first use; later jobs on it take the incremental rebuild path);
 * jobs of one resident grid run in submission order.  Jobs are admitted while
 * the device bytes held by all grids plus the job's estimate stay within
 * mem_cap_bytes (one job always runs). */
typedef struct gbvdb_server_s* gbvdb_server;
typedef struct {
    const void* points;          /* float3 positions, element i at points + i*stride */
    int64_t n;                   /* number of points */
    int32_t points_on_device;    /* 1: device pointer (borrowed until the job ends); 0: host memory */
    int32_t stride;              /* bytes between points (0 = 12) */
    int32_t levs;                /* Configure(levs, log2dim): log2 dims, leaf first */
    int32_t log2dim_leaf_first[8];
    int32_t resident_id;         /* -1: fresh grid; >= 0: resident grid id */
    int32_t mode;                /* 0 GatherDensity, 1 GatherLevelSet */
    int32_t dtype;               /* GBVDB_T_FLOAT, GBVDB_T_HALF or GBVDB_T_BFLOAT16 */
    float radius;                /* RebuildTopology radius */
    float insert_radius;         /* InsertPointsSubcell radius */
    float gather_radius;         /* gather radius rho */
    float boundval;              /* UpdateApron boundary value */
    float orig[3];               /* RebuildTopology orig / insert and gather trans */
} gbvdb_job;
typedef struct {
    int32_t status;              /* gbvdb_status of the job */
    int64_t bricks;              /* linked leaves of the insert */
    int64_t sc_len;              /* subcell list length (pSCPntsLength) */
    double checksum;             /* FP64 sum of channel 0 */
    double t_submit_ms, t_start_ms, t_end_ms;  /* server clock */
} gbvdb_job_result;
GBVDB_API gbvdb_status gbvdb_server_create(int device, int workers, int64_t mem_cap_bytes, gbvdb_server* out);
GBVDB_API gbvdb_status gbvdb_server_submit(gbvdb_server s, const gbvdb_job* job, int64_t* ticket);
/* blocks until the job ends; the ticket is released */
GBVDB_API gbvdb_status gbvdb_server_wait(gbvdb_server s, int64_t ticket, gbvdb_job_result* out);
GBVDB_API gbvdb_status gbvdb_server_poll(gbvdb_server s, int64_t ticket, int* done);
/* the grid of an idle resident id (exports, checksums); valid until released */
GBVDB_API gbvdb_status gbvdb_server_resident(gbvdb_server s, int32_t resident_id, gbvdb_grid* out);
GBVDB_API gbvdb_status gbvdb_server_release(gbvdb_server s, int32_t resident_id);
/* out6 = {queued, running, completed, device bytes held, memory cap, resident grids} */
GBVDB_API gbvdb_status gbvdb_server_stats(gbvdb_server s, int64_t* out6);
/* finishes the queued jobs, then frees every grid */
GBVDB_API gbvdb_status gbvdb_server_destroy(gbvdb_server s);

#ifdef __cplusplus
}
#endif
#endif /* GBVDB_H */
