"""ctypes front end of oracle/ref_harness.cu: the reference's own CUDA kernels
(oracle/_ref/cuda_gvdb_module.ptx) under a restatement of its host code.
TEST INFRASTRUCTURE ONLY (golden fixtures, timing of the reference CUDA path)."""
import ctypes

import numpy as np

import oracle
import ref_build


class RefGrid:
    def __init__(self, log2dims=(3, 3, 3, 4)):
        ptx = ref_build.build_ptx()
        if not ptx:
            raise RuntimeError("reference PTX not available")
        L = ctypes.CDLL(ref_build.build_harness())
        vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        fp = ctypes.POINTER(ctypes.c_float)
        L.rh_create.restype = vp
        L.rh_create.argtypes = [ctypes.c_char_p, i32, ctypes.POINTER(ctypes.c_int)]
        for n in ("rh_set_points", "rh_rebuild_topology", "rh_update_atlas", "rh_insert_subcell", "rh_gather",
                  "rh_update_apron", "rh_sync", "rh_top_lev", "rh_atlas_bricks", "rh_subcells", "rh_subcell_num",
                  "rh_accumulate_topology", "rh_add_colour_channel", "rh_set_colors", "rh_fill", "rh_event_begin",
                  "rh_insert_subcell_fp16", "rh_gather_levelset_fp16", "rh_update_apron_faces", "rh_smooth",
                  "rh_insert_points", "rh_scatter_density", "rh_write_bricks"):
            getattr(L, n).restype = i32
        L.rh_insert_subcell_fp16.argtypes = [vp, f32, fp, ctypes.POINTER(ctypes.c_int)]
        L.rh_gather_levelset_fp16.argtypes = [vp, f32]
        L.rh_update_apron_faces.argtypes = [vp]
        L.rh_smooth.argtypes = [vp, f32, f32, f32]
        L.rh_insert_points.argtypes = [vp, fp]
        L.rh_scatter_density.argtypes = [vp, f32, f32, fp, i32]
        L.rh_write_bricks.argtypes = [vp, i32, vp, i32]
        L.rh_accumulate_topology.argtypes = [vp, f32, fp, i32]
        L.rh_add_colour_channel.argtypes = [vp]
        L.rh_set_colors.argtypes = [vp, vp, i32]
        L.rh_fill.argtypes = [vp, i32, f32]
        L.rh_event_begin.argtypes = [vp]
        L.rh_event_end_ms.restype = f32
        L.rh_event_end_ms.argtypes = [vp]
        L.rh_timing.restype = i32
        L.rh_timing.argtypes = [vp, i32]
        L.rh_kernel_ms.restype = f32
        L.rh_kernel_ms.argtypes = [vp]
        L.rh_set_points.argtypes = [vp, fp, i32]
        L.rh_rebuild_topology.argtypes = [vp, f32, fp]
        L.rh_update_atlas.argtypes = [vp]
        L.rh_insert_subcell.argtypes = [vp, f32, fp, ctypes.POINTER(ctypes.c_int)]
        L.rh_gather.argtypes = [vp, i32, f32, i32]
        L.rh_update_apron.argtypes = [vp, i32, f32]
        L.rh_sync.argtypes = [vp]
        L.rh_node_count.restype = ctypes.c_longlong
        L.rh_node_count.argtypes = [vp, i32]
        L.rh_used_count.restype = ctypes.c_longlong
        L.rh_used_count.argtypes = [vp, i32]
        L.rh_top_lev.argtypes = [vp]
        L.rh_nodes.argtypes = [vp, i32, vp]
        L.rh_childlist.argtypes = [vp, i32, vp]
        L.rh_atlas_dims.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        L.rh_atlas_map.argtypes = [vp, vp]
        L.rh_atlas_bricks.argtypes = [vp, i32, vp]
        L.rh_subcells.argtypes = [vp, vp, vp, vp]
        L.rh_subcell_num.argtypes = [vp]
        L.rh_error.restype = ctypes.c_char_p
        L.rh_error.argtypes = [vp]
        self.L = L
        leaf_first = list(reversed(log2dims))
        self.levs = len(leaf_first)
        self.leaf_first = leaf_first
        arr = (ctypes.c_int * self.levs)(*leaf_first)
        self.h = L.rh_create(ptx.encode(), self.levs, arr)
        if not self.h:
            raise RuntimeError("harness creation failed")
        self.len = 0

    def _ok(self, rc, what):
        if rc not in (0, 8):
            raise RuntimeError("%s: %s" % (what, self.L.rh_error(self.h).decode()))
        return rc

    def set_points(self, pts):
        p = np.ascontiguousarray(pts[:, :3], dtype=np.float32)
        self._keep = p
        self._ok(self.L.rh_set_points(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.shape[0]), "set")

    def set_colors(self, rgba):
        """point colours, one uint32 (RGBA8, R in the low byte) per point; None: no colours"""
        if rgba is None:
            self._ok(self.L.rh_set_colors(self.h, None, 0), "colors")
            return
        c = np.ascontiguousarray(rgba, dtype=np.uint32)
        self._keep_clr = c
        self._ok(self.L.rh_set_colors(self.h, c.ctypes.data, c.shape[0]), "colors")

    def add_colour_channel(self):
        self._ok(self.L.rh_add_colour_channel(self.h), "colour channel")

    def fill(self, chan, value):
        self._ok(self.L.rh_fill(self.h, chan, float(value)), "fill")

    def accumulate_topology(self, radius, orig=(0, 0, 0), min_depth=1):
        o = (ctypes.c_float * 3)(*orig)
        return self._ok(self.L.rh_accumulate_topology(self.h, radius, o, int(min_depth)), "accumulate")

    def event_begin(self):
        self._ok(self.L.rh_event_begin(self.h), "event")

    def event_end_ms(self):
        return float(self.L.rh_event_end_ms(self.h))

    def timing(self, on=True):
        """start (or stop) recording an event pair around every kernel / Thrust call"""
        self.L.rh_timing(self.h, 1 if on else 0)

    def kernel_ms(self):
        """summed device time of the kernels and Thrust calls since timing(True)"""
        return float(self.L.rh_kernel_ms(self.h))

    def rebuild_topology(self, radius, orig=(0, 0, 0)):
        o = (ctypes.c_float * 3)(*orig)
        return self._ok(self.L.rh_rebuild_topology(self.h, radius, o), "rebuild")

    def update_atlas(self):
        return self._ok(self.L.rh_update_atlas(self.h), "atlas")

    def insert_points_subcell(self, radius, trans=(0, 0, 0)):
        t = (ctypes.c_float * 3)(*trans)
        n = ctypes.c_int(0)
        rc = self._ok(self.L.rh_insert_subcell(self.h, radius, t, ctypes.byref(n)), "insert")
        self.len = n.value
        return rc, n.value

    def insert_points_subcell_fp16(self, radius, trans=(0, 0, 0)):
        t = (ctypes.c_float * 3)(*trans)
        n = ctypes.c_int(0)
        rc = self._ok(self.L.rh_insert_subcell_fp16(self.h, radius, t, ctypes.byref(n)), "insert fp16")
        self.len = n.value
        return rc, n.value

    def gather_levelset_fp16(self, radius):
        return self._ok(self.L.rh_gather_levelset_fp16(self.h, radius), "gather fp16")

    def update_apron_faces(self):
        """UpdateNeighbors + UpdateApronFaces on channel 0"""
        return self._ok(self.L.rh_update_apron_faces(self.h), "apron faces")

    def smooth(self, p1, p2, p3=0.0):
        """one Compute(FUNC_SMOOTH) pass on channel 0"""
        return self._ok(self.L.rh_smooth(self.h, p1, p2, p3), "smooth")

    def insert_points(self, trans=(0, 0, 0)):
        t = (ctypes.c_float * 3)(*trans)
        return self._ok(self.L.rh_insert_points(self.h, t), "insert points")

    def scatter_density(self, radius, amp=1.0, trans=(0, 0, 0), expand=True):
        t = (ctypes.c_float * 3)(*trans)
        return self._ok(self.L.rh_scatter_density(self.h, radius, amp, t, 1 if expand else 0), "scatter")

    def write_bricks(self, bricks, chan=0):
        """padded FP32 bricks [slot, z, y, x] of slots [0, n) into the atlas"""
        b = np.ascontiguousarray(bricks, dtype=np.float32)
        return self._ok(self.L.rh_write_bricks(self.h, chan, b.ctypes.data, b.shape[0]), "write bricks")

    def gather_density(self, radius, accum=False):
        return self._ok(self.L.rh_gather(self.h, 0, radius, 1 if accum else 0), "gather")

    def gather_levelset(self, radius, accum=False):
        return self._ok(self.L.rh_gather(self.h, 1, radius, 1 if accum else 0), "gather")

    def update_apron(self, boundval, chan=0):
        return self._ok(self.L.rh_update_apron(self.h, chan, boundval), "apron")

    def sync(self):
        self._ok(self.L.rh_sync(self.h), "sync")

    def node_count(self, lev):
        return int(self.L.rh_node_count(self.h, lev))

    def used_count(self, lev=0):
        return int(self.L.rh_used_count(self.h, lev))

    @property
    def top_lev(self):
        return int(self.L.rh_top_lev(self.h))

    def nodes(self, lev):
        n = self.node_count(lev)
        out = np.zeros(n, dtype=oracle.NODE_DTYPE)
        if n:
            self.L.rh_nodes(self.h, lev, out.ctypes.data)
        return out

    def childlist(self, lev):
        n = self.node_count(lev)
        cl = 1 << (3 * self.leaf_first[lev]) if lev > 0 else 0
        out = np.zeros(n * cl, dtype=np.uint64)
        if n and cl:
            self.L.rh_childlist(self.h, lev, out.ctypes.data)
        return out.reshape(n, cl)

    def atlas_dims(self):
        out = (ctypes.c_int * 4)()
        self.L.rh_atlas_dims(self.h, out)
        return tuple(out[:])

    def atlas_map(self):
        ax, ay, az, _ = self.atlas_dims()
        out = np.zeros(ax * ay * az, dtype=oracle.AMAP_DTYPE)
        self.L.rh_atlas_map(self.h, out.ctypes.data)
        return out

    def atlas_bricks(self, chan=0):
        """padded bricks of the assigned slots, [slot, z, y, x]: FP32 (chan 0) or RGBA8 as uint32 (chan 1)"""
        used = self.atlas_dims()[3]
        out = np.zeros(used * 5832, dtype=np.float32 if chan == 0 else np.uint32)
        if used:
            self._ok(self.L.rh_atlas_bricks(self.h, chan, out.ctypes.data), "bricks")
        return out.reshape(used, 18, 18, 18)

    def subcell_counts(self):
        """(counts, offsets) of all 64 * used subcells, without the list entries"""
        n = int(self.L.rh_subcell_num(self.h))
        cnt = np.zeros(n, dtype=np.int32)
        off = np.zeros(n, dtype=np.int32)
        self._ok(self.L.rh_subcells(self.h, cnt.ctypes.data, off.ctypes.data, None), "subcells")
        return cnt, off

    def subcells(self):
        """(counts, offsets, points) of all 64 * used subcells"""
        n = int(self.L.rh_subcell_num(self.h))
        cnt = np.zeros(n, dtype=np.int32)
        off = np.zeros(n, dtype=np.int32)
        pts = np.zeros((max(self.len, 1), 3), dtype=np.float32)
        self._ok(self.L.rh_subcells(self.h, cnt.ctypes.data, off.ctypes.data, pts.ctypes.data), "subcells")
        return cnt, off, pts[:self.len]
