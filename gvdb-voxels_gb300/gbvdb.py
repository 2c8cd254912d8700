"""ctypes binding of libgbvdb.so (include/gbvdb.h).

`Grid` mirrors the reference class nvdb::VolumeGVDB for the point-driven path
(source/gvdb_library/src/gvdb_volume_gvdb.h:387-557): same method names,
argument meaning and order.  Point buffers are device tensors (torch) or raw
device pointers.  There is no CPU fallback: loading fails loudly if the
library is missing, and every failing call raises GbvdbError.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgbvdb.so")

OK, INVALID_ARG, OUT_OF_MEMORY, CUDA_ERROR, DEPTH_UNSUPPORTED, CAPACITY, TIMEOUT, NOT_SUPPORTED, NOOP = range(9)
STATUS_NAMES = ["OK", "INVALID_ARG", "OUT_OF_MEMORY", "CUDA_ERROR", "DEPTH_UNSUPPORTED", "CAPACITY", "TIMEOUT",
                "NOT_SUPPORTED", "NOOP"]
T_UCHAR, T_UCHAR4, T_FLOAT, T_HALF, T_BFLOAT16 = 0, 2, 3, 100, 101

NODE_DTYPE = np.dtype([
    ("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"),
    ("pos", "<i4", 3), ("value", "<i4", 3), ("vrange", "<f4", 3),
    ("parent", "<u8"), ("childlist", "<u8"), ("mask", "<u8"),
])
AMAP_DTYPE = np.dtype([("pos", "<i4", 3), ("leaf", "<i4")])
VDB_INFO_BYTES = 1232  # sizeof(gbvdb_vdb_info), the reference's VDBInfo layout

# every symbol declared in include/gbvdb.h
EXPORTS = [
    "gbvdb_create", "gbvdb_destroy", "gbvdb_set_stream", "gbvdb_last_error", "gbvdb_configure",
    "gbvdb_configure5", "gbvdb_set_channel_default", "gbvdb_add_channel", "gbvdb_set_points",
    "gbvdb_rebuild_topology", "gbvdb_accumulate_topology", "gbvdb_request_full_rebuild",
    "gbvdb_finish_topology", "gbvdb_update_atlas", "gbvdb_insert_points_subcell", "gbvdb_gather_density",
    "gbvdb_gather_levelset", "gbvdb_update_apron", "gbvdb_fill_channel", "gbvdb_get_depth",
    "gbvdb_get_node_counts", "gbvdb_get_point_bounds", "gbvdb_export_nodes", "gbvdb_export_childlist",
    "gbvdb_get_atlas_info", "gbvdb_export_atlas_bricks", "gbvdb_export_atlas_map", "gbvdb_export_subcells",
    "gbvdb_checksum", "gbvdb_get_atlas_device", "gbvdb_set_profile", "gbvdb_get_stage_times",
    "gbvdb_get_stats", "gbvdb_get_stats_ex", "gbvdb_checksum_noalloc", "gbvdb_set_tuning", "gbvdb_save_vbx", "gbvdb_load_vbx",
    "gbvdb_update_neighbors", "gbvdb_export_neighbors", "gbvdb_update_apron_faces", "gbvdb_compute",
    "gbvdb_insert_points_subcell_fp16", "gbvdb_gather_levelset_fp16", "gbvdb_insert_points", "gbvdb_scatter_density",
    "gbvdb_export_point_leaves", "gbvdb_checksum_device", "gbvdb_fill_channel4", "gbvdb_clear_channel",
    "gbvdb_get_vol_bounds", "gbvdb_get_device_bytes", "gbvdb_get_vdb_info", "gbvdb_activate_space",
    "gbvdb_rebuild_topology_cpu", "gbvdb_tune_table_source", "gbvdb_checksum_overlap", "gbvdb_join",
    "gbvdb_server_create", "gbvdb_server_submit", "gbvdb_server_wait", "gbvdb_server_poll",
    "gbvdb_server_resident", "gbvdb_server_release", "gbvdb_server_stats", "gbvdb_server_destroy",
]


class Job(ctypes.Structure):
    """gbvdb_job (include/gbvdb.h)."""
    _fields_ = [("points", ctypes.c_void_p), ("n", ctypes.c_int64), ("points_on_device", ctypes.c_int32),
                ("stride", ctypes.c_int32), ("levs", ctypes.c_int32), ("log2dim_leaf_first", ctypes.c_int32 * 8),
                ("resident_id", ctypes.c_int32), ("mode", ctypes.c_int32), ("dtype", ctypes.c_int32),
                ("radius", ctypes.c_float), ("insert_radius", ctypes.c_float), ("gather_radius", ctypes.c_float),
                ("boundval", ctypes.c_float), ("orig", ctypes.c_float * 3)]


class JobResult(ctypes.Structure):
    """gbvdb_job_result (include/gbvdb.h)."""
    _fields_ = [("status", ctypes.c_int32), ("bricks", ctypes.c_int64), ("sc_len", ctypes.c_int64),
                ("checksum", ctypes.c_double), ("t_submit_ms", ctypes.c_double), ("t_start_ms", ctypes.c_double),
                ("t_end_ms", ctypes.c_double)]
TUNE_DENSE_MIN = 1
TUNE_FUSED_APRON = 2
TUNE_AUTOTUNE = 3
TUNE_TOUCH_DIRS = 4
TUNE_TABLE = 5
TUNE_BIN_UNROLL = 6
TUNE_SCATTER_UNROLL = 7
TUNE_GATHER_BLOCKS = 8
TUNE_KEYSET = 9
TUNE_GATHER_LONG_MIN = 10
FUNC_SMOOTH = 113


class GbvdbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else status, msg))
        self.status = status


_lib = None


def load(path=LIB_PATH):
    """Load libgbvdb.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgbvdb.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
    fp = ctypes.POINTER(ctypes.c_float)
    for name in EXPORTS:
        getattr(L, name).restype = i32
    L.gbvdb_last_error.restype = ctypes.c_char_p
    L.gbvdb_tune_table_source.restype = ctypes.c_char_p
    L.gbvdb_tune_table_source.argtypes = []
    L.gbvdb_create.argtypes = [i32, ctypes.POINTER(vp)]
    L.gbvdb_destroy.argtypes = [vp]
    L.gbvdb_set_stream.argtypes = [vp, vp]
    L.gbvdb_last_error.argtypes = [vp]
    L.gbvdb_configure.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int)]
    L.gbvdb_configure5.argtypes = [vp, i32, i32, i32, i32, i32]
    L.gbvdb_set_channel_default.argtypes = [vp, i32, i32, i32]
    L.gbvdb_add_channel.argtypes = [vp, i32, i32, i32, i32, i32, i32]
    L.gbvdb_set_points.argtypes = [vp, vp, i64, i32, i32, vp, i32, i32, vp, i32, i32]
    L.gbvdb_rebuild_topology.argtypes = [vp, i64, f32, fp]
    L.gbvdb_accumulate_topology.argtypes = [vp, i64, f32, fp, i32]
    L.gbvdb_request_full_rebuild.argtypes = [vp, i32]
    L.gbvdb_finish_topology.argtypes = [vp, i32, i32]
    L.gbvdb_update_atlas.argtypes = [vp]
    L.gbvdb_insert_points_subcell.argtypes = [vp, i32, i64, f32, fp, ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_gather_density.argtypes = [vp, i32, i64, f32, fp, i64, i32, i32, i32]
    L.gbvdb_gather_levelset.argtypes = [vp, i32, i64, f32, fp, i64, i32, i32, i32]
    L.gbvdb_update_apron.argtypes = [vp, i32, f32]
    L.gbvdb_fill_channel.argtypes = [vp, i32, f32]
    L.gbvdb_fill_channel4.argtypes = [vp, i32, fp]
    L.gbvdb_clear_channel.argtypes = [vp, i32]
    L.gbvdb_get_vol_bounds.argtypes = [vp, fp]
    L.gbvdb_get_device_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_get_vdb_info.argtypes = [vp, vp, i64]
    L.gbvdb_checksum_overlap.argtypes = [vp, i32, vp, vp]
    L.gbvdb_join.argtypes = [vp]
    L.gbvdb_activate_space.argtypes = [vp, fp, ctypes.POINTER(ctypes.c_uint64)]
    L.gbvdb_rebuild_topology_cpu.argtypes = [vp, i64, fp, vp, i32]
    L.gbvdb_get_depth.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.gbvdb_get_node_counts.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_get_point_bounds.argtypes = [vp, fp]
    L.gbvdb_export_nodes.argtypes = [vp, i32, vp, i64]
    L.gbvdb_export_childlist.argtypes = [vp, i32, vp, i64]
    L.gbvdb_get_atlas_info.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int)]
    L.gbvdb_export_atlas_bricks.argtypes = [vp, i32, vp, i64]
    L.gbvdb_export_atlas_map.argtypes = [vp, vp, i64]
    L.gbvdb_export_subcells.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), i64, vp, i64]
    L.gbvdb_checksum.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_double)]
    L.gbvdb_get_atlas_device.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.gbvdb_set_profile.argtypes = [vp, i32]
    L.gbvdb_get_stage_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), i32]
    L.gbvdb_get_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_get_stats_ex.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
    L.gbvdb_checksum_noalloc.argtypes = [vp, i32, vp]
    L.gbvdb_set_tuning.argtypes = [vp, i32, i64]
    L.gbvdb_save_vbx.argtypes = [vp, ctypes.c_char_p]
    L.gbvdb_update_neighbors.argtypes = [vp]
    L.gbvdb_checksum_device.argtypes = [vp, i32, vp]
    L.gbvdb_insert_points.argtypes = [vp, i64, fp, i32]
    L.gbvdb_scatter_density.argtypes = [vp, i64, f32, f32, fp, i32, i32]
    L.gbvdb_export_point_leaves.argtypes = [vp, vp, i64, vp, i64, vp, i64]
    L.gbvdb_insert_points_subcell_fp16.argtypes = [vp, i32, i64, f32, fp, ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_gather_levelset_fp16.argtypes = [vp, i32, i64, f32, fp, i64, i32, i32]
    L.gbvdb_export_neighbors.argtypes = [vp, vp, i64]
    L.gbvdb_update_apron_faces.argtypes = [vp, i32]
    L.gbvdb_compute.argtypes = [vp, i32, i32, i32, fp, i32, i32, f32]
    L.gbvdb_load_vbx.argtypes = [vp, ctypes.c_char_p]
    L.gbvdb_server_create.argtypes = [i32, i32, i64, ctypes.POINTER(vp)]
    L.gbvdb_server_submit.argtypes = [vp, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_server_wait.argtypes = [vp, i64, ctypes.POINTER(JobResult)]
    L.gbvdb_server_poll.argtypes = [vp, i64, ctypes.POINTER(ctypes.c_int)]
    L.gbvdb_server_resident.argtypes = [vp, i32, ctypes.POINTER(vp)]
    L.gbvdb_server_release.argtypes = [vp, i32]
    L.gbvdb_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.gbvdb_server_destroy.argtypes = [vp]
    _lib = L
    return L


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in (v if v is not None else (0, 0, 0))])


def _dev_ptr(points):
    """(pointer, n, stride_bytes) of a device point buffer: torch tensor (N, >=3) float32."""
    if hasattr(points, "data_ptr"):
        if not points.is_cuda:
            raise ValueError("points must be a CUDA tensor")
        if points.dtype.itemsize != 4 or points.dim() != 2 or points.shape[1] < 3 or points.stride(1) != 1:
            raise ValueError("points must be float32 (N, >=3) with unit inner stride")
        return points.data_ptr(), points.shape[0], points.stride(0) * 4
    ptr, n, stride = points
    return int(ptr), int(n), int(stride)


class Grid:
    """One GVDB grid on one GPU.  `log2dims` is top -> leaf, as Configure(q4..q0)."""

    def __init__(self, device=0, log2dims=(3, 3, 3, 4), stream=None):
        self.L = load()
        h = ctypes.c_void_p()
        self._check(self.L.gbvdb_create(int(device), ctypes.byref(h)), "create", handle=None)
        self._h = h
        self.levs = len(log2dims)
        self.configure(log2dims)
        if stream is not None:
            self.set_stream(stream)
        self._points = None

    def _check(self, st, what, handle="self", allow_noop=True):
        if st == OK or (allow_noop and st == NOOP):
            return st
        msg = ""
        if handle == "self":
            msg = (self.L.gbvdb_last_error(self._h) or b"").decode()
        raise GbvdbError(st, "%s failed: %s" % (what, msg))

    @classmethod
    def _borrow(cls, handle):
        """A view of a grid owned elsewhere (a server's resident grid): never destroyed here."""
        g = cls.__new__(cls)
        g.L = load()
        g._h = handle
        g._borrowed = True
        g._points = None
        return g

    def close(self):
        if getattr(self, "_borrowed", False):
            self._h = None
            return
        if getattr(self, "_h", None) is not None and self._h.value:
            self.L.gbvdb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration -----------------------------------------------------
    def set_stream(self, stream):
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        self._check(self.L.gbvdb_set_stream(self._h, ctypes.c_void_p(ptr)), "set_stream")

    def configure(self, log2dims):
        leaf_first = list(reversed(log2dims))
        arr = (ctypes.c_int * len(leaf_first))(*leaf_first)
        self._check(self.L.gbvdb_configure(self._h, len(leaf_first), arr), "configure")
        self.levs = len(leaf_first)
        self._leaf_first = [d if d else 1 for d in leaf_first]

    def set_channel_default(self, ax, ay, az):
        self._check(self.L.gbvdb_set_channel_default(self._h, ax, ay, az), "set_channel_default")

    def add_channel(self, chan=0, dtype=T_FLOAT, apron=1, axiscnt=(0, 0, 0)):
        self._check(self.L.gbvdb_add_channel(self._h, chan, dtype, apron, *axiscnt), "add_channel")

    def set_points(self, points, n=None, colours=None):
        """colours: None or a CUDA uint32/int32 tensor, one RGBA8 value per point (R in the low byte)"""
        ptr, cnt, stride = _dev_ptr(points)
        cptr, cstride = None, 0
        if colours is not None:
            if not colours.is_cuda or colours.dtype.itemsize != 4 or colours.dim() != 1 or colours.shape[0] < cnt:
                raise ValueError("colours must be a CUDA tensor of one 4-byte value per point")
            cptr, cstride = ctypes.c_void_p(colours.data_ptr()), colours.stride(0) * 4
        self._points = (points, colours)  # keep the buffers alive
        self._check(self.L.gbvdb_set_points(self._h, ctypes.c_void_p(ptr), cnt if n is None else n, 0, stride,
                                            None, 0, 0, cptr, 0, cstride), "set_points")
        return cnt

    # -- topology ------------------------------------------------------------
    def rebuild_topology(self, n, radius, orig=(0, 0, 0)):
        return self._check(self.L.gbvdb_rebuild_topology(self._h, n, radius, _f3(orig)), "rebuild_topology")

    def accumulate_topology(self, n, radius, orig=(0, 0, 0), min_depth=1):
        return self._check(self.L.gbvdb_accumulate_topology(self._h, n, radius, _f3(orig), min_depth),
                           "accumulate_topology")

    def activate_space(self, pos):
        """ActivateSpace (host path): the existing leaf's Elem id, or 0xFFFFFFFF for a new leaf"""
        out = ctypes.c_uint64(0)
        self._check(self.L.gbvdb_activate_space(self._h, _f3(pos), ctypes.byref(out)), "activate_space")
        return int(out.value)

    def rebuild_topology_cpu(self, points, orig=(0, 0, 0)):
        """RebuildTopologyCPU of host float32 (N, 3) positions"""
        p = np.ascontiguousarray(points[:, :3], dtype=np.float32)
        self._check(self.L.gbvdb_rebuild_topology_cpu(self._h, p.shape[0], _f3(orig), p.ctypes.data, 12),
                    "rebuild_topology_cpu")

    def request_full_rebuild(self, tf=True):
        self._check(self.L.gbvdb_request_full_rebuild(self._h, 1 if tf else 0), "request_full_rebuild")

    def finish_topology(self, commit=False, bounds=True):
        self._check(self.L.gbvdb_finish_topology(self._h, int(commit), int(bounds)), "finish_topology")

    def update_atlas(self):
        return self._check(self.L.gbvdb_update_atlas(self._h), "update_atlas")

    # -- points to voxels ----------------------------------------------------
    def insert_points_subcell(self, subcell, n, radius, trans=(0, 0, 0)):
        out = ctypes.c_int64(-1)
        st = self._check(self.L.gbvdb_insert_points_subcell(self._h, subcell, n, radius, _f3(trans),
                                                            ctypes.byref(out)), "insert_points_subcell")
        return st, int(out.value)

    def insert_points_subcell_fp16(self, subcell, n, radius, trans=(0, 0, 0)):
        """InsertPointsSubcell_FP16: 16-bit positions over the point bounds."""
        out = ctypes.c_int64(-1)
        st = self._check(self.L.gbvdb_insert_points_subcell_fp16(self._h, subcell, n, radius, _f3(trans),
                                                                 ctypes.byref(out)), "insert_points_subcell_fp16")
        return st, int(out.value)

    def gather_levelset_fp16(self, subcell, n, radius, trans, sc_len, chan=0, clr_chan=-1):
        """GatherLevelSet_FP16 (no accumulation)."""
        return self._check(self.L.gbvdb_gather_levelset_fp16(self._h, subcell, n, radius, _f3(trans), sc_len, chan,
                                                             clr_chan), "gather_levelset_fp16")

    def gather_density(self, subcell, n, radius, trans, sc_len, chan=0, clr_chan=-1, accum=False):
        return self._check(self.L.gbvdb_gather_density(self._h, subcell, n, radius, _f3(trans), sc_len, chan,
                                                       clr_chan, int(accum)), "gather_density")

    def gather_levelset(self, subcell, n, radius, trans, sc_len, chan=0, clr_chan=-1, accum=False):
        return self._check(self.L.gbvdb_gather_levelset(self._h, subcell, n, radius, _f3(trans), sc_len, chan,
                                                        clr_chan, int(accum)), "gather_levelset")

    def update_apron(self, chan=0, boundval=0.0):
        return self._check(self.L.gbvdb_update_apron(self._h, chan, boundval), "update_apron")

    def fill_channel(self, chan, value):
        """FillChannel: a float, or a 4-vector (x, y, z, w) as the reference's Vector4DF"""
        if hasattr(value, "__len__"):
            v = (ctypes.c_float * 4)(*[float(x) for x in value])
            return self._check(self.L.gbvdb_fill_channel4(self._h, chan, v), "fill_channel")
        return self._check(self.L.gbvdb_fill_channel(self._h, chan, value), "fill_channel")

    def clear_channel(self, chan):
        """ClearChannel: every voxel of the channel to 0"""
        return self._check(self.L.gbvdb_clear_channel(self._h, chan), "clear_channel")

    def vol_bounds(self):
        """getVolMin / getVolMax after FinishTopology(.., bounds): (min xyz, max xyz), or None"""
        out = (ctypes.c_float * 6)()
        if self._check(self.L.gbvdb_get_vol_bounds(self._h, out), "get_vol_bounds") == NOOP:
            return None
        return np.array(out[:], dtype=np.float32)

    def vdb_info(self):
        """the VDBInfo-layout view (include/gbvdb_device.cuh) as raw bytes"""
        buf = ctypes.create_string_buffer(VDB_INFO_BYTES)
        self._check(self.L.gbvdb_get_vdb_info(self._h, buf, VDB_INFO_BYTES), "get_vdb_info")
        return buf.raw

    def device_bytes(self):
        out = ctypes.c_int64()
        self._check(self.L.gbvdb_get_device_bytes(self._h, ctypes.byref(out)), "get_device_bytes")
        return int(out.value)

    # -- state / export ------------------------------------------------------
    def depth(self):
        d, t = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.gbvdb_get_depth(self._h, ctypes.byref(d), ctypes.byref(t)), "get_depth")
        return d.value, t.value

    def node_counts(self):
        tot = (ctypes.c_int64 * 10)()
        used = (ctypes.c_int64 * 10)()
        self._check(self.L.gbvdb_get_node_counts(self._h, tot, used), "get_node_counts")
        return list(tot), list(used)

    def point_bounds(self):
        out = (ctypes.c_float * 6)()
        self._check(self.L.gbvdb_get_point_bounds(self._h, out), "get_point_bounds")
        return np.array(out[:], dtype=np.float32)

    def nodes(self, lev):
        n = self.node_counts()[0][lev]
        out = np.zeros(n, dtype=NODE_DTYPE)
        if n:
            self._check(self.L.gbvdb_export_nodes(self._h, lev, out.ctypes.data, n), "export_nodes")
        return out

    def childlist(self, lev):
        n = self.node_counts()[0][lev]
        if lev == 0:
            return np.zeros((n, 0), dtype=np.uint64)
        cl = 1 << (3 * self._leaf_first[lev])
        if n == 0:
            return np.zeros((0, cl), dtype=np.uint64)
        out = np.zeros(n * cl, dtype=np.uint64)
        self._check(self.L.gbvdb_export_childlist(self._h, lev, out.ctypes.data, n * cl), "export_childlist")
        return out.reshape(n, cl)

    def atlas_info(self, chan=0):
        info = (ctypes.c_int * 8)()
        self._check(self.L.gbvdb_get_atlas_info(self._h, chan, info), "get_atlas_info")
        keys = ["ax", "ay", "az", "used", "dtype", "apron", "brick_res", "esize"]
        return dict(zip(keys, info[:]))

    def atlas_bricks(self, chan=0):
        """Padded bricks of the assigned slots, shape (used, 18, 18, 18) [slot, z, y, x].
        float32 channels return float32; half returns float16; bfloat16 returns raw uint16; RGBA8
        colour channels return uint32 (R in the low byte)."""
        info = self.atlas_info(chan)
        used = info["used"]
        dt = {T_FLOAT: np.float32, T_HALF: np.float16, T_BFLOAT16: np.uint16, T_UCHAR4: np.uint32}[info["dtype"]]
        out = np.zeros(used * 5832, dtype=dt)
        if used:
            self._check(self.L.gbvdb_export_atlas_bricks(self._h, chan, out.ctypes.data, out.nbytes),
                        "export_atlas_bricks")
        return out.reshape(used, 18, 18, 18)

    def atlas_map(self):
        info = self.atlas_info(0)
        n = info["ax"] * info["ay"] * info["az"]
        out = np.zeros(n, dtype=AMAP_DTYPE)
        if n:
            self._check(self.L.gbvdb_export_atlas_map(self._h, out.ctypes.data, n), "export_atlas_map")
        return out

    def subcells(self, total_len, nsub):
        off = np.zeros(nsub + 1, dtype=np.int64)
        pts = np.zeros((max(total_len, 0), 3), dtype=np.float32)
        self._check(self.L.gbvdb_export_subcells(
            self._h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), nsub + 1,
            pts.ctypes.data if total_len > 0 else None, total_len), "export_subcells")
        return off, pts

    def insert_points(self, n, trans=(0, 0, 0), prefix=True):
        """Legacy InsertPoints (gvdb_volume_gvdb.cpp:5219-5267)."""
        self._check(self.L.gbvdb_insert_points(self._h, n, _f3(trans), int(prefix)), "insert_points")

    def scatter_density(self, n, radius, amp=1.0, trans=(0, 0, 0), expand=True, avg_color=False):
        """Legacy ScatterDensity (gvdb_volume_gvdb.cpp:5624-5660) into channel 0."""
        return self._check(self.L.gbvdb_scatter_density(self._h, n, radius, amp, _f3(trans), int(expand),
                                                        int(avg_color)), "scatter_density")

    def point_leaves(self, n):
        """(leaf per point, group offsets per leaf, grouped points) of the last insert_points."""
        nl = self.node_counts()[0][0]
        pnode = np.zeros(max(n, 1), dtype=np.int32)
        off = np.zeros(nl + 1, dtype=np.int64)
        self._check(self.L.gbvdb_export_point_leaves(self._h, pnode.ctypes.data, n, off.ctypes.data, nl + 1, None, 0),
                    "export_point_leaves")
        pts = np.zeros((max(int(off[-1]), 1), 3), dtype=np.float32)
        self._check(self.L.gbvdb_export_point_leaves(self._h, None, 0, None, 0, pts.ctypes.data, pts.size),
                    "export_point_leaves")
        return pnode[:n], off, pts[:int(off[-1])]

    def update_neighbors(self):
        """UpdateNeighbors (gvdb_volume_gvdb.cpp:2527-2556)."""
        self._check(self.L.gbvdb_update_neighbors(self._h), "update_neighbors")

    def neighbors(self):
        """The neighbour table: (leaves, 6) int32 (-x, -y, -z, +x, +y, +z), -1 = none."""
        n = self.node_counts()[0][0]
        out = np.zeros((n, 6), dtype=np.int32)
        self._check(self.L.gbvdb_export_neighbors(self._h, out.ctypes.data, n * 6), "export_neighbors")
        return out

    def update_apron_faces(self, chan=0):
        """UpdateApronFaces (gvdb_volume_gvdb.cpp:4461-4496)."""
        return self._check(self.L.gbvdb_update_apron_faces(self._h, chan), "update_apron_faces")

    def compute(self, effect, chan, iterations, params, update_apron=True, skip_aprons=True, boundval=0.0):
        """Compute (gvdb_volume_gvdb.cpp:4532-4558); effect FUNC_SMOOTH."""
        return self._check(self.L.gbvdb_compute(self._h, effect, chan, iterations, _f3(params), int(update_apron),
                                                int(skip_aprons), float(boundval)), "compute")

    def save_vbx(self, path):
        """SaveVBX (gvdb_volume_gvdb.cpp:1626-1767)."""
        self._check(self.L.gbvdb_save_vbx(self._h, os.fsencode(path)), "save_vbx")

    def load_vbx(self, path):
        """LoadVBX (gvdb_volume_gvdb.cpp:507-683): replaces configuration, pools and channels."""
        self._check(self.L.gbvdb_load_vbx(self._h, os.fsencode(path)), "load_vbx")

    def checksum_device(self, out, chan=0):
        """FP64 channel sum into `out` (a CUDA float64 tensor element) on the grid's stream."""
        self._check(self.L.gbvdb_checksum_device(self._h, chan, ctypes.c_void_p(out.data_ptr())), "checksum_device")

    def checksum_overlap(self, out, host_out=None, chan=0):
        """FP64 channel sum into `out` (CUDA float64 element) and `host_out` (pinned CPU float64
        element, optional) on the grid's side stream, overlapping the grid's next calls"""
        hp = ctypes.c_void_p(host_out.data_ptr()) if host_out is not None else None
        self._check(self.L.gbvdb_checksum_overlap(self._h, chan, ctypes.c_void_p(out.data_ptr()), hp),
                    "checksum_overlap")

    def join(self):
        """the grid's stream waits for a pending overlapped checksum"""
        self._check(self.L.gbvdb_join(self._h), "join")

    def checksum(self, chan=0):
        out = ctypes.c_double()
        self._check(self.L.gbvdb_checksum(self._h, chan, ctypes.byref(out)), "checksum")
        return out.value

    def set_tuning(self, param, value):
        self._check(self.L.gbvdb_set_tuning(self._h, int(param), int(value)), "set_tuning")

    def set_profile(self, on=True):
        self._check(self.L.gbvdb_set_profile(self._h, int(on)), "set_profile")

    def stats(self):
        out = (ctypes.c_int64 * 5)()
        self._check(self.L.gbvdb_get_stats_ex(self._h, out, 5), "get_stats_ex")
        return {"launches": out[0], "readbacks": out[1], "sc_len": out[2], "bricks": out[3],
                "hashed_key_passes": out[4]}

    def stage_times(self, cap=32):
        out = (ctypes.c_double * cap)()
        self._check(self.L.gbvdb_get_stage_times(self._h, out, cap), "get_stage_times")
        return [v for v in out[:] if v >= 0]


def bf16_to_f32(u16):
    """Raw bfloat16 bits (uint16) -> float32."""
    return (u16.astype(np.uint32) << 16).view(np.float32)


class Server:
    """The served form (include/gbvdb.h, no counterpart in the reference): a request
    loop whose worker threads run voxelize-and-gather jobs concurrently on one GPU.

    submit() takes host points (a C-contiguous float32 (N, 3) numpy array, kept
    alive until the job ends) or a CUDA tensor; wait() returns a dict with the
    job's status, bricks, subcell-list length, FP64 checksum and server-clock
    times (ms)."""

    def __init__(self, device=0, workers=8, mem_cap_bytes=120 << 30):
        self.L = load()
        self.s = ctypes.c_void_p()
        st = self.L.gbvdb_server_create(int(device), int(workers), int(mem_cap_bytes), ctypes.byref(self.s))
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_create")
        self._keep = {}

    def submit(self, points, log2dims=(3, 3, 3, 4), radius=1.0, insert_radius=None, gather_radius=1.0, mode=0,
               dtype=T_FLOAT, boundval=0.0, orig=(0, 0, 0), resident_id=-1):
        j = Job()
        if hasattr(points, "data_ptr"):
            ptr, n, stride = _dev_ptr(points)
            j.points_on_device = 1
        else:
            arr = np.ascontiguousarray(points, dtype=np.float32)
            if arr.ndim != 2 or arr.shape[1] != 3:
                raise ValueError("host points must be (N, 3) float32")
            ptr, n, stride = arr.ctypes.data, arr.shape[0], 12
            j.points_on_device = 0
            points = arr
        j.points, j.n, j.stride = ptr, n, stride
        dims = list(log2dims)[::-1]  # top -> leaf given; leaf first here
        j.levs = len(dims)
        for i, d in enumerate(dims):
            j.log2dim_leaf_first[i] = int(d)
        j.resident_id = int(resident_id)
        j.mode = int(mode)
        j.dtype = int(dtype)
        j.radius = float(radius)
        j.insert_radius = float(radius if insert_radius is None else insert_radius)
        j.gather_radius = float(gather_radius)
        j.boundval = float(boundval)
        for a in range(3):
            j.orig[a] = float(orig[a])
        t = ctypes.c_int64()
        st = self.L.gbvdb_server_submit(self.s, ctypes.byref(j), ctypes.byref(t))
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_submit")
        self._keep[t.value] = points
        return t.value

    def wait(self, ticket):
        r = JobResult()
        st = self.L.gbvdb_server_wait(self.s, int(ticket), ctypes.byref(r))
        self._keep.pop(ticket, None)
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_wait")
        return {"status": r.status, "bricks": r.bricks, "sc_len": r.sc_len, "checksum": r.checksum,
                "t_submit_ms": r.t_submit_ms, "t_start_ms": r.t_start_ms, "t_end_ms": r.t_end_ms}

    def poll(self, ticket):
        d = ctypes.c_int()
        st = self.L.gbvdb_server_poll(self.s, int(ticket), ctypes.byref(d))
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_poll")
        return bool(d.value)

    def resident(self, resident_id):
        """A Grid view of an idle resident grid (not owned: do not destroy)."""
        g = ctypes.c_void_p()
        st = self.L.gbvdb_server_resident(self.s, int(resident_id), ctypes.byref(g))
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_resident")
        return Grid._borrow(g)

    def release(self, resident_id):
        st = self.L.gbvdb_server_release(self.s, int(resident_id))
        if st != OK:
            raise GbvdbError(st, "gbvdb_server_release")

    def stats(self):
        a = (ctypes.c_int64 * 6)()
        self.L.gbvdb_server_stats(self.s, a)
        return dict(zip(["queued", "running", "completed", "held_bytes", "cap_bytes", "resident"], list(a)))

    def close(self):
        if self.s:
            self.L.gbvdb_server_destroy(self.s)
            self.s = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
