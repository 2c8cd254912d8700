"""Test infrastructure: an independent reader of VBX files, written from the
format description (GVDB_FILESPEC.txt:12-122) and the field order of the
reference's SaveVBX / LoadVBX (source/gvdb_library/src/gvdb_volume_gvdb.cpp
:1626-1767, 507-683).  The grid header holds a channel count between the apron
and the atlas size (the code's order; the format text omits it), and each
channel starts with its type and element stride.
"""
import numpy as np

NODE_BYTES = 64


class Reader:
    def __init__(self, data):
        self.b = memoryview(data)
        self.p = 0

    def take(self, n):
        v = self.b[self.p:self.p + n]
        if len(v) != n:
            raise ValueError("VBX file truncated at byte %d" % self.p)
        self.p += n
        return bytes(v)

    def arr(self, dtype, count):
        dt = np.dtype(dtype)
        return np.frombuffer(self.take(dt.itemsize * count), dtype=dt).copy()

    def one(self, dtype):
        return self.arr(dtype, 1)[0].item()


def read_vbx(path):
    with open(path, "rb") as f:
        data = f.read()
    r = Reader(data)
    out = {"size": len(data)}
    out["major"], out["minor"] = r.one("u1"), r.one("u1")
    if (out["major"] == 1 and out["minor"] >= 11) or out["major"] > 1:
        t = r.arr("<f4", 12)
        out["pretrans"], out["angs"], out["scale"], out["trans"] = t[0:3], t[3:6], t[6:9], t[9:12]
    out["num_grids"] = r.one("<i4")
    if out["major"] >= 2:
        out["bitmasks"] = r.one("u1")
    out["grid_offsets"] = r.arr("<u8", out["num_grids"])
    r.p = int(out["grid_offsets"][0])
    out["grid_header_offset"] = r.p
    out["name"] = r.take(256)
    out["dtype"] = chr(r.one("u1"))
    out["components"] = r.one("u1")
    out["compression"] = r.one("u1")
    out["voxel_size"] = r.arr("<f4", 3)
    out["brick_count"] = r.one("<i4")
    out["brick_dims"] = r.arr("<i4", 3)
    out["apron"] = r.one("<i4")
    out["num_channels"] = r.one("<i4")
    out["atlas_size"] = r.one("<u8")
    out["topology_type"] = r.one("u1")
    out["topology_reuse"] = r.one("<i4")
    out["layout"] = r.one("u1")
    out["axiscnt"] = r.arr("<i4", 3)
    out["axisres"] = r.arr("<i4", 3)
    levels = r.one("<i4")
    out["levels"] = levels
    out["root"] = r.one("<u8")
    lv = []
    for _ in range(levels):
        d = {"log2dim": r.one("<i4"), "res": r.one("<i4"), "range": r.arr("<i4", 3)}
        d["cnt0"], d["width0"], d["cnt1"], d["width1"] = (r.one("<i4") for _ in range(4))
        lv.append(d)
    out["level_info"] = lv
    out["nodes"] = [np.frombuffer(r.take(d["cnt0"] * d["width0"]), dtype=np.uint8).reshape(d["cnt0"], -1)
                    if d["cnt0"] else np.zeros((0, NODE_BYTES), np.uint8) for d in lv]
    out["childlists"] = [None] + [r.arr("<u8", d["cnt1"] * d["width1"] // 8).reshape(d["cnt1"], -1)
                                  if d["cnt1"] else np.zeros((0, d["width1"] // 8), np.uint64) for d in lv[1:]]
    out["atlas_offset"] = r.p
    W, H, Z = (int(v) for v in out["axisres"])
    chans = []
    for _ in range(out["num_channels"]):
        ctype, stride = r.one("<i4"), r.one("<i4")
        dt = {4: "<f4", 2: "<u2", 1: "u1"}[stride]
        vol = r.arr(dt, W * H * Z).reshape(Z, H, W)
        chans.append({"type": ctype, "stride": stride, "volume": vol})
    out["channels"] = chans
    out["end"] = r.p
    return out


def atlas_bricks(vol, axiscnt, count):
    """Padded 18^3 bricks of slots [0, count) from an atlas volume [z][y][x]."""
    ax, ay, _ = (int(v) for v in axiscnt)
    out = np.zeros((count, 18, 18, 18), dtype=vol.dtype)
    for s in range(count):
        bx, by, bz = s % ax, (s // ax) % ay, s // (ax * ay)
        out[s] = vol[bz * 18:(bz + 1) * 18, by * 18:(by + 1) * 18, bx * 18:(bx + 1) * 18]
    return out
