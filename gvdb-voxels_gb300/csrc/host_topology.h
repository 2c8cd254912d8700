// host_topology.h -- the reference's host-side topology path (ActivateSpace /
// RebuildTopologyCPU), built on host copies of the node pools that the grid
// then commits to its device pools.
//
// Restates, on the reference's pool layout (64-byte nodes, res^3 u64 child lists,
// Elem references):
//   ActivateSpace(Vector3DF)             gvdb_volume_gvdb.cpp:2766-2774
//   ActivateSpace(node, pos, bNew, ...)  gvdb_volume_gvdb.cpp:2795-2855
//   Reparent                             gvdb_volume_gvdb.cpp:2726-2763
//   AddChildNode / getPosFromBit         gvdb_volume_gvdb.cpp:2707-2723, gvdb_volume_gvdb.h:602-608
//   InsertChild (child-list form)        gvdb_volume_gvdb.cpp:2980-3027
//   GetCoveringNode                      gvdb_volume_gvdb.cpp:2915-2931
//   getPosInNode                         gvdb_volume_gvdb.cpp:2858-2875
//   AllocateNode / SetupNode             gvdb_volume_gvdb.cpp:2506-2524
// Each new node takes the next index of its level (pool order = creation order);
// a node's child list is taken from its level's list pool when its first child
// is inserted.  Levels past the configured ones have no range here, so the root
// grows at most to the top configured level (the reference reads unset level
// dimensions there).
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace gbvdb {

class HostTopology {
public:
    static constexpr uint64_t kNone = 0xFFFFFFFFull;  // ID_UNDEFL

    int levs = 0;
    int lgres[kMaxLev] = {0};
    long long range[kMaxLev] = {0};
    std::vector<Node> nodes[kMaxLev];
    std::vector<uint64_t> clist[kMaxLev];
    size_t lists_used[kMaxLev] = {0};
    size_t used[kMaxLev] = {0};  // flagged nodes per level (usedNum)
    uint64_t root = kNone;       // mRoot

    void configure(int nlev, const int* log2dim, const long long* rg) {
        levs = nlev;
        for (int l = 0; l < kMaxLev; l++) {
            lgres[l] = l < nlev ? log2dim[l] : 0;
            range[l] = l < nlev ? rg[l] : 0;
            nodes[l].clear();
            clist[l].clear();
            lists_used[l] = used[l] = 0;
        }
        root = kNone;
    }
    size_t list_len(int lev) const { return lev >= 1 ? (size_t)1 << (3 * lgres[lev]) : 0; }

    // ActivateSpace(pos) for an index-space position already truncated to integers:
    // the leaf that holds it, or kNone when the leaf is new or the position cannot be
    // covered (VG.cpp:2766-2774)
    uint64_t activate_space(const int32_t pos[3]) {
        bool fresh = false;
        const uint64_t leaf = activate(root, pos, &fresh, kNone, 0);
        if (leaf == kNone || fresh) return kNone;
        return leaf;
    }

private:
    static int ref_lev(uint64_t e) { return (int)((e >> 8) & 0xFF); }
    static size_t ref_ndx(uint64_t e) { return (size_t)(e >> 16); }
    static uint64_t elem(int grp, int lev, uint64_t ndx) { return (uint64_t)grp | ((uint64_t)lev << 8) | (ndx << 16); }
    Node& node(uint64_t id) { return nodes[ref_lev(id)][ref_ndx(id)]; }

    uint64_t alloc_node(int lev, const int32_t pos[3]) {
        Node n;
        memset(&n, 0, sizeof(n));
        n.lev = (uint8_t)lev;
        n.flags = 1;
        for (int a = 0; a < 3; a++) { n.pos[a] = pos[a]; n.value[a] = -1; }
        n.parent = kNone;
        n.childlist = kNone;
        nodes[lev].push_back(n);
        used[lev]++;
        return elem(0, lev, nodes[lev].size() - 1);
    }
    // corner of the level-lev node covering pos (floor division); false past the
    // configured levels
    bool cover(int lev, const int32_t pos[3], int32_t out[3]) const {
        if (lev >= levs) return false;
        const long long rg = range[lev];
        for (int a = 0; a < 3; a++) {
            long long q = (long long)pos[a] / rg * rg;
            if (pos[a] < q) q -= rg;
            out[a] = (int32_t)q;
        }
        return true;
    }
    // child bit of pos inside node n; false when pos is outside n
    bool bit_of(const Node& n, const int32_t pos[3], uint32_t* bit) const {
        const long long rg = range[n.lev];
        const long long r = 1ll << lgres[n.lev];
        long long p[3];
        for (int a = 0; a < 3; a++) {
            p[a] = (long long)pos[a] - n.pos[a];
            if (p[a] < 0 || p[a] >= rg) return false;
            p[a] = p[a] * r / rg;
        }
        *bit = (uint32_t)((p[2] * r + p[1]) * r + p[0]);
        return true;
    }
    uint64_t child_of(const Node& n, uint32_t b) const {
        if (n.childlist == kNone) return 0xFFFFFFFFFFFFFFFFull;
        return clist[n.lev][ref_ndx(n.childlist) * list_len(n.lev) + b];
    }
    uint64_t insert_child(uint64_t parent, uint64_t child, uint32_t b) {
        node(child).parent = parent;
        Node& p = node(parent);
        const int lev = p.lev;
        const size_t len = list_len(lev);
        if (p.childlist == kNone) {
            const size_t k = lists_used[lev]++;
            if (clist[lev].size() < (k + 1) * len) clist[lev].resize((k + 1) * len, 0xFFFFFFFFFFFFFFFFull);
            std::fill(clist[lev].begin() + (long long)(k * len), clist[lev].begin() + (long long)((k + 1) * len),
                      0xFFFFFFFFFFFFFFFFull);
            p.childlist = elem(1, lev, k);
        }
        clist[lev][ref_ndx(node(parent).childlist) * len + b] = child;
        return child;
    }
    uint64_t add_child(uint64_t parent, uint32_t b) {
        const Node p = node(parent);
        const int lg = lgres[p.lev];
        const uint32_t mask = (1u << lg) - 1u;
        const long long crg = range[p.lev - 1];
        const int32_t pos[3] = {(int32_t)(p.pos[0] + (long long)(b & mask) * crg),
                                (int32_t)(p.pos[1] + (long long)((b >> lg) & mask) * crg),
                                (int32_t)(p.pos[2] + (long long)((b >> (2 * lg)) & mask) * crg)};
        const uint64_t c = alloc_node(p.lev - 1, pos);
        return insert_child(parent, c, b);
    }
    // a new root above prev covering pos as well; the old root joins it as a child
    uint64_t reparent(int lev, uint64_t prev, const int32_t pos[3], bool* fresh) {
        const int32_t ppos[3] = {node(prev).pos[0], node(prev).pos[1], node(prev).pos[2]};
        int32_t p1[3] = {0, 0, 0}, p2[3];
        bool same = false;
        while (!same) {
            lev++;
            if (!cover(lev, pos, p1) || !cover(lev, ppos, p2)) return kNone;  // the root stays
            same = p1[0] == p2[0] && p1[1] == p2[1] && p1[2] == p2[2];
        }
        const uint64_t nr = alloc_node(lev, p1);
        bool unused = false;
        activate(nr, ppos, &unused, prev, 0);
        const uint64_t leaf = activate(nr, pos, fresh, kNone, 0);
        root = nr;
        if (leaf == kNone) return kNone;
        return node(leaf).parent;
    }
    uint64_t activate(uint64_t id, const int32_t pos[3], bool* fresh, uint64_t stop, int stoplev) {
        for (int guard = 0; guard < 4 * kMaxLev; guard++) {
            if (root == kNone && id == root) {  // an empty tree: a root covering pos
                int32_t p[3];
                if (!cover(stoplev, pos, p)) return kNone;
                root = alloc_node(stoplev, p);
                id = root;
            }
            const Node cur = node(id);
            uint32_t b;
            if (bit_of(cur, pos, &b)) {
                if (stop != kNone) {
                    const Node& s = node(stop);
                    if (pos[0] == s.pos[0] && pos[1] == s.pos[1] && pos[2] == s.pos[2] &&
                        child_of(cur, b) == 0xFFFFFFFFFFFFFFFFull && cur.lev == s.lev + 1)
                        return insert_child(id, stop, b);
                }
                if (cur.lev == stoplev) return id;
                uint64_t c = child_of(cur, b);
                if (c == 0xFFFFFFFFFFFFFFFFull) {
                    c = add_child(id, b);
                    if (cur.lev == 1) *fresh = true;
                }
                if (ref_lev(c) == 0) return c;
                id = c;
            } else {
                uint64_t p = cur.parent;
                if (p == kNone) {
                    p = reparent(cur.lev, id, pos, fresh);
                    if (p == kNone) return kNone;
                }
                id = p;
            }
        }
        return kNone;
    }
};

}  // namespace gbvdb
