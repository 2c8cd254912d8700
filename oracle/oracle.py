"""ctypes front end for the CPU oracle (oracle/gvdb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to check
its result and by bench.py for the timed CPU baseline.  The product library never
imports this module.

`OracleGrid` mirrors the reference's VolumeGVDB call sequence for the
point-driven path (source/gvdb_library/src/gvdb_volume_gvdb.h:387-557):
RebuildTopology, AccumulateTopology, UpdateAtlas, InsertPointsSubcell,
GatherDensity / GatherLevelSet and UpdateApron.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gvdb_oracle.c")
LIB = os.path.join(HERE, "libgvdb_oracle.so")

NODE_DTYPE = np.dtype([
    ("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"),
    ("pos", "<i4", 3), ("value", "<i4", 3), ("vrange", "<f4", 3),
    ("parent", "<u8"), ("childlist", "<u8"), ("mask", "<u8"),
])
assert NODE_DTYPE.itemsize == 64
AMAP_DTYPE = np.dtype([("pos", "<i4", 3), ("leaf", "<i4")])

OK, INVALID_ARG, DEPTH_UNSUPPORTED, NOOP = 0, 1, 4, 8


def build(force=False):
    """Compile the oracle with gcc (-ffp-contract=off keeps FP32 truncations exact)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC",
           SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i64, f32, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_int
        fp3 = ctypes.POINTER(ctypes.c_float)
        L.og_create.restype = vp
        L.og_create.argtypes = [i32, ctypes.POINTER(ctypes.c_int)]
        L.og_destroy.argtypes = [vp]
        L.og_set_threads.argtypes = [vp, i32]
        L.og_set_channel_default.argtypes = [vp, i32, i32, i32]
        L.og_request_full_rebuild.argtypes = [vp, i32]
        L.og_add_channel.argtypes = [vp, i32, i32, i32, i32, i32, i32]
        L.og_rebuild_topology.argtypes = [vp, vp, i64, i32, i32, f32, fp3]
        L.og_accumulate_topology.argtypes = [vp, vp, i64, i32, i32, f32, fp3, i32]
        L.og_update_atlas.argtypes = [vp]
        L.og_insert_points_subcell.argtypes = [vp, i32, vp, i64, i32, i32, f32, fp3, ctypes.POINTER(ctypes.c_int64)]
        L.og_insert_points_subcell_fp16.argtypes = [vp, i32, vp, i64, i32, i32, f32, fp3,
                                                    ctypes.POINTER(ctypes.c_int64)]
        L.og_gather.argtypes = [vp, i32, f32, i32, i32]
        L.og_gather_clr.argtypes = [vp, i32, f32, i32, i32, i32]
        L.og_insert_points_subcell_clr.argtypes = [vp, i32, vp, i64, i32, i32, f32, fp3, vp, i32, i32,
                                                   ctypes.POINTER(ctypes.c_int64)]
        L.og_fill_channel.argtypes = [vp, i32, fp3]
        L.og_clear_channel.argtypes = [vp, i32]
        L.og_compute_bounds.restype = i32
        L.og_compute_bounds.argtypes = [vp, fp3]
        L.og_update_apron.argtypes = [vp, i32, f32]
        for name in ("og_depth", "og_top_lev", "og_childlist_len"):
            getattr(L, name).restype = i32
        L.og_depth.argtypes = [vp]
        L.og_top_lev.argtypes = [vp]
        L.og_childlist_len.argtypes = [vp, i32]
        L.og_node_count.restype = i64
        L.og_node_count.argtypes = [vp, i32]
        L.og_used_count.restype = i64
        L.og_used_count.argtypes = [vp, i32]
        L.og_nodes.restype = vp
        L.og_nodes.argtypes = [vp, i32]
        L.og_childlist.restype = vp
        L.og_childlist.argtypes = [vp, i32]
        L.og_bbox.argtypes = [vp, fp3]
        L.og_atlas_dims.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        L.og_atlas_map.restype = vp
        L.og_atlas_map.argtypes = [vp]
        L.og_atlas_data.restype = vp
        L.og_atlas_data.argtypes = [vp, i32]
        L.og_subcell_count.restype = i64
        L.og_subcell_count.argtypes = [vp]
        L.og_subcell_offsets.restype = vp
        L.og_subcell_offsets.argtypes = [vp]
        L.og_subcell_points.restype = vp
        L.og_subcell_points.argtypes = [vp]
        L.og_subcell_len.restype = i64
        L.og_subcell_len.argtypes = [vp]
        L.og_subcell_map.restype = vp
        L.og_subcell_map.argtypes = [vp]
        L.og_checksum.restype = ctypes.c_double
        L.og_checksum.argtypes = [vp, i32]
        L.og_save_vbx.restype = i32
        L.og_save_vbx.argtypes = [vp, ctypes.c_char_p]
        L.og_update_neighbors.argtypes = [vp, vp]
        L.og_insert_points.argtypes = [vp, vp, i64, i32, i32, fp3, vp, vp]
        L.og_scatter_density.argtypes = [vp, vp, i64, i32, i32, fp3, f32, i32]
        L.og_apron_faces_f32.argtypes = [vp, vp, vp]
        L.og_apron_full_f32.argtypes = [vp, vp, f32]
        L.og_smooth_f32.argtypes = [vp, vp, f32, f32]
        L.og_rebuild_topology_cpu.restype = i64
        L.og_rebuild_topology_cpu.argtypes = [vp, vp, i64, i32, i32, fp3]
        L.og_cpu_root_level.restype = i32
        L.og_cpu_root_level.argtypes = [vp]
        _lib = L
    return _lib


def _f3(v):
    a = (ctypes.c_float * 3)(*[float(x) for x in v])
    return a


def _copy(ptr, dtype, count):
    if count == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    nbytes = int(count) * np.dtype(dtype).itemsize
    buf = (ctypes.c_char * nbytes).from_address(ptr)
    return np.frombuffer(bytes(buf), dtype=dtype).copy()


class OracleGrid:
    """One grid of the CPU oracle.  `log2dims` is given top -> leaf, as in
    Configure(q4, q3, q2, q1, q0) (gvdb_volume_gvdb.cpp:2364-2377)."""

    def __init__(self, log2dims=(3, 3, 3, 4), threads=0):
        L = lib()
        leaf_first = list(reversed(log2dims))
        arr = (ctypes.c_int * len(leaf_first))(*leaf_first)
        self._h = L.og_create(len(leaf_first), arr)
        if not self._h:
            raise ValueError("bad grid config")
        self.levs = len(leaf_first)
        if threads:
            L.og_set_threads(self._h, threads)
        self._keep = None

    def close(self):
        if self._h:
            lib().og_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference API ----------------------------------------------------
    def set_channel_default(self, ax, ay, az):
        lib().og_set_channel_default(self._h, ax, ay, az)

    def add_channel(self, chan=0, dtype=3, apron=1, axiscnt=(0, 0, 0)):
        rc = lib().og_add_channel(self._h, chan, dtype, apron, *axiscnt)
        if rc:
            raise ValueError("add_channel failed: %d" % rc)

    def request_full_rebuild(self, tf=True):
        lib().og_request_full_rebuild(self._h, 1 if tf else 0)

    @staticmethod
    def _pts(points):
        p = np.ascontiguousarray(points, dtype=np.float32)
        assert p.ndim == 2 and p.shape[1] >= 3
        return p, p.shape[0], p.shape[1] * 4

    def rebuild_topology(self, points, radius, orig=(0, 0, 0)):
        p, n, stride = self._pts(points)
        return lib().og_rebuild_topology(self._h, p.ctypes.data, n, stride, 0, float(radius), _f3(orig))

    def rebuild_topology_cpu(self, points, orig=(0, 0, 0)):
        """The reference's host path RebuildTopologyCPU / ActivateSpace (every point
        activates the leaf containing it; the root grows upwards) on an empty grid.
        Returns the number of points that reached a leaf."""
        p, n, stride = self._pts(points)
        return int(lib().og_rebuild_topology_cpu(self._h, p.ctypes.data, n, stride, 0, _f3(orig)))

    def cpu_root_level(self):
        return int(lib().og_cpu_root_level(self._h))

    def accumulate_topology(self, points, radius, orig=(0, 0, 0), min_depth=1):
        p, n, stride = self._pts(points)
        return lib().og_accumulate_topology(self._h, p.ctypes.data, n, stride, 0, float(radius),
                                            _f3(orig), int(min_depth))

    def update_atlas(self):
        return lib().og_update_atlas(self._h)

    def insert_points_subcell(self, points, radius, subcell=4, trans=(0, 0, 0), colours=None):
        """colours: None or one uint32 RGBA8 (R in the low byte) per point"""
        p, n, stride = self._pts(points)
        out = ctypes.c_int64(-1)
        if colours is None:
            rc = lib().og_insert_points_subcell(self._h, subcell, p.ctypes.data, n, stride, 0,
                                                float(radius), _f3(trans), ctypes.byref(out))
        else:
            c = np.ascontiguousarray(colours, dtype=np.uint32)
            assert c.shape[0] >= n
            rc = lib().og_insert_points_subcell_clr(self._h, subcell, p.ctypes.data, n, stride, 0, float(radius),
                                                    _f3(trans), c.ctypes.data, 4, 0, ctypes.byref(out))
        return rc, int(out.value)

    def insert_points_subcell_fp16(self, points, radius, subcell=4, trans=(0, 0, 0)):
        """InsertPointsSubcell_FP16 restated: lists hold 16-bit-quantised positions (dequantised)."""
        p, n, stride = self._pts(points)
        out = ctypes.c_int64(-1)
        rc = lib().og_insert_points_subcell_fp16(self._h, subcell, p.ctypes.data, n, stride, 0,
                                                 float(radius), _f3(trans), ctypes.byref(out))
        return rc, int(out.value)

    def gather_density(self, radius, chan=0, accum=False, clr_chan=-1):
        return lib().og_gather_clr(self._h, 0, float(radius), chan, clr_chan, 1 if accum else 0)

    def gather_levelset(self, radius, chan=0, accum=False, clr_chan=-1):
        return lib().og_gather_clr(self._h, 1, float(radius), chan, clr_chan, 1 if accum else 0)

    def fill_channel(self, chan, value):
        """FillChannel: a float, or a 4-vector (x, y, z, w) as the reference's Vector4DF"""
        v = list(value) if hasattr(value, "__len__") else [float(value), 0.0, 0.0, 0.0]
        a = (ctypes.c_float * 4)(*[float(x) for x in v])
        lib().og_fill_channel(self._h, chan, a)

    def clear_channel(self, chan):
        lib().og_clear_channel(self._h, chan)

    def compute_bounds(self):
        """ComputeBounds restated: (min xyz, max xyz) as floats, or None for an empty pool"""
        out = (ctypes.c_float * 6)()
        if not lib().og_compute_bounds(self._h, out):
            return None
        return np.array(out[:], dtype=np.float32)

    def update_apron(self, chan=0, boundval=0.0):
        return lib().og_update_apron(self._h, chan, float(boundval))

    # -- exports ------------------------------------------------------------
    @property
    def depth(self):
        return lib().og_depth(self._h)

    @property
    def top_lev(self):
        return lib().og_top_lev(self._h)

    def node_count(self, lev):
        return int(lib().og_node_count(self._h, lev))

    def used_count(self, lev=0):
        return int(lib().og_used_count(self._h, lev))

    def nodes(self, lev):
        return _copy(lib().og_nodes(self._h, lev), NODE_DTYPE, self.node_count(lev))

    def childlist(self, lev):
        if lev == 0:
            return np.zeros((0,), dtype=np.uint64)
        n = self.node_count(lev)
        cl = lib().og_childlist_len(self._h, lev)
        return _copy(lib().og_childlist(self._h, lev), np.uint64, n * cl).reshape(n, cl)

    def bbox(self):
        out = (ctypes.c_float * 6)()
        lib().og_bbox(self._h, out)
        return np.array(out[:], dtype=np.float32)

    def atlas_dims(self):
        out = (ctypes.c_int * 4)()
        lib().og_atlas_dims(self._h, out)
        return tuple(out[:])

    def atlas_map(self):
        ax, ay, az, _ = self.atlas_dims()
        return _copy(lib().og_atlas_map(self._h), AMAP_DTYPE, ax * ay * az)

    def atlas_bricks(self, chan=0, slots=None):
        """FP64 padded bricks, shape (slots, 18, 18, 18) indexed [slot, z, y, x] (a T_UCHAR4
        channel holds each RGBA8 voxel as the value of its uint32)."""
        ax, ay, az, used = self.atlas_dims()
        n = used if slots is None else slots
        return _copy(lib().og_atlas_data(self._h, chan), np.float64, n * 5832).reshape(n, 18, 18, 18)

    def subcells(self):
        """(offsets[n+1], points[len,3]) of the subcell lists in subcell order."""
        n = int(lib().og_subcell_count(self._h))
        off = _copy(lib().og_subcell_offsets(self._h), np.int64, n + 1)
        ln = int(lib().og_subcell_len(self._h))
        pts = _copy(lib().og_subcell_points(self._h), np.float32, ln * 3).reshape(ln, 3)
        return off, pts

    def checksum(self, chan=0):
        return float(lib().og_checksum(self._h, chan))

    def insert_points(self, points, trans=(0, 0, 0)):
        """Legacy InsertPoints restated: (leaf per point, point count per leaf)."""
        p, n, stride = self._pts(points)
        pnode = np.zeros(n, dtype=np.int32)
        counts = np.zeros(max(self.node_count(0), 1), dtype=np.int64)
        lib().og_insert_points(self._h, p.ctypes.data, n, stride, 0, _f3(trans), pnode.ctypes.data, counts.ctypes.data)
        return pnode, counts[:self.node_count(0)]

    def scatter_density(self, points, radius, expand=True, trans=(0, 0, 0)):
        """Legacy ScatterDensity restated into channel 0 (FP64)."""
        p, n, stride = self._pts(points)
        lib().og_scatter_density(self._h, p.ctypes.data, n, stride, 0, _f3(trans), float(radius), int(expand))

    def neighbors(self):
        """UpdateNeighbors restated: (leaves, 6) pool indices (-x, -y, -z, +x, +y, +z), -1 = none."""
        n = self.node_count(0)
        out = np.zeros((n, 6), dtype=np.int32)
        if n:
            lib().og_update_neighbors(self._h, out.ctypes.data)
        return out

    @staticmethod
    def _bricks_arg(bricks):
        assert bricks.dtype == np.float32 and bricks.flags.c_contiguous and bricks.shape[1:] == (18, 18, 18)
        return bricks.ctypes.data

    def apron_faces_f32(self, bricks, table):
        """UpdateApronFaces restated, in place on FP32 padded bricks [slot, z, y, x]."""
        t = np.ascontiguousarray(table, dtype=np.int32)
        lib().og_apron_faces_f32(self._h, t.ctypes.data, self._bricks_arg(bricks))

    def apron_full_f32(self, bricks, boundval):
        """UpdateApron restated, in place on FP32 padded bricks."""
        lib().og_apron_full_f32(self._h, self._bricks_arg(bricks), float(boundval))

    def smooth_f32(self, bricks, p1, p2):
        """One Compute(FUNC_SMOOTH) pass restated, in place on FP32 padded bricks."""
        lib().og_smooth_f32(self._h, self._bricks_arg(bricks), float(p1), float(p2))

    def save_vbx(self, path):
        """SaveVBX restated (VG.cpp:1626-1767): FP32 atlas from the FP64 oracle values."""
        assert lib().og_save_vbx(self._h, os.fsencode(path)) == 0
