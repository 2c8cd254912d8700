/*
 * gvdb_oracle.c -- CPU oracle for the GVDB point-driven dynamic-topology path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference's algorithm, used by tests/, by __graft_entry__.smoke() to check
 * its result, and by bench.py as the timed CPU baseline ("port").  It is never
 * linked into, loaded by, or called from the product library.
 *
 * Every function cites the reference file:line it restates.  Abbreviations:
 *   VG.cpp = source/gvdb_library/src/gvdb_volume_gvdb.cpp
 *   AL.cpp = source/gvdb_library/src/gvdb_allocator.cpp
 *   PT.cuh = source/gvdb_library/kernels/cuda_gvdb_particles.cuh
 *   ND.cuh = source/gvdb_library/kernels/cuda_gvdb_nodes.cuh
 *   OP.cuh = source/gvdb_library/kernels/cuda_gvdb_operators.cuh
 *
 * Integer work (keys, pools, links, subcell membership, atlas slots) follows
 * the reference bit for bit, including its float->int truncations, which are
 * evaluated here in IEEE single precision (compile with -ffp-contract=off).
 * Gathered values are computed in FP64 from the FP32 point positions.
 *
 * Where the reference's behaviour is undefined (a child-list index computed
 * from a position outside the node, e.g. ND.cuh:317-322 has no bounds check)
 * this oracle and the CUDA path both skip the position.  Those guards never
 * fire for positions inside the root node.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OG_MAXLEV 10
#define OG_MAXCHAN 8
#define UNDEFL 0xFFFFFFFFull            /* gvdb_types.h:55 */
#define UNDEF64 0xFFFFFFFFFFFFFFFFull   /* gvdb_types.h:56 */
#define NOHIT 1.0e10f                   /* gvdb_types.h:52 */

/* status codes (mirror include/gbvdb.h) */
#define OG_OK 0
#define OG_INVALID_ARG 1
#define OG_DEPTH_UNSUPPORTED 4
#define OG_NOOP 8

/* 64-byte node record, gvdb_node.h:27-40 */
typedef struct {
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    uint64_t parent;
    uint64_t childlist;
    uint64_t mask;
} ONode;
_Static_assert(sizeof(ONode) == 64, "node record must be 64 bytes");

typedef struct {
    int32_t pos[3];
    int32_t leaf;
} OAtlasNode; /* VDBAtlasNode, ND.cuh:38-41 */

typedef struct {
    int used;           /* channel exists */
    int dtype;
    int apron;
    double* data;       /* slot-major: slot * 18^3 + (z*18+y)*18+x, FP64 */
    size_t cap_slots;
} OChan;

typedef struct OGrid {
    int levs;
    int log2dim[OG_MAXLEV];
    int res[OG_MAXLEV];
    int64_t range[OG_MAXLEV];
    /* pools: group 0 nodes, group 1 child lists (AL.cpp:55-91) */
    ONode* nodes[OG_MAXLEV];
    size_t ncnt[OG_MAXLEV], ncap[OG_MAXLEV];
    size_t nused[OG_MAXLEV];
    uint64_t* clist[OG_MAXLEV];
    int rebuild_topo;
    int curr_depth;
    int last_depth;
    float posmin[3], posmax[3];
    /* atlas (channel 0 owns the slot allocator, AL.cpp:692-715) */
    int ax, ay, az;           /* axiscnt */
    int def_ax, def_ay, def_az;
    int atlas_last;           /* lastEle */
    OAtlasNode* amap;
    size_t amap_cnt;
    OChan chan[OG_MAXCHAN];
    /* subcells (VG.cpp:4971-5092) */
    int sc_size;
    int* sc_map;              /* per leaf: exclusive scan of linked flag */
    size_t sc_nbricks;        /* number of linked leaves */
    int64_t* sc_cnt;
    int64_t* sc_off;
    float* sc_pts;            /* 3 floats per entry, in subcell order */
    uint32_t* sc_clr;         /* RGBA8 per entry when the insert carried colours, else NULL */
    int64_t sc_len;
    size_t sc_nleaf;          /* leaf count when the lists were built */
    int nthreads;
    /* the reference's CPU topology path (og_rebuild_topology_cpu) */
    uint64_t cpu_root;        /* mRoot, an Elem reference; UNDEFL when empty */
    size_t cl_used[OG_MAXLEV]; /* child lists taken from pool 1 per level */
} OGrid;

/* ------------------------------------------------------------------------ */
/* pools                                                                     */

static int64_t og_range(const OGrid* g, int lev) { return g->range[lev]; }
static int og_res(const OGrid* g, int lev) { return g->res[lev]; }
static size_t og_cl_len(const OGrid* g, int lev) {
    size_t r = (size_t)g->res[lev];
    return r * r * r;
}
static uint64_t Elem(int grp, int lev, uint64_t ndx) { /* AL.h:59 */
    return (uint64_t)grp | ((uint64_t)lev << 8) | (ndx << 16);
}

static void pool_reserve(OGrid* g, int lev, size_t need) {
    if (need <= g->ncap[lev]) return;
    size_t cap = g->ncap[lev] ? g->ncap[lev] : 16;
    while (cap < need) cap *= 2;
    g->nodes[lev] = (ONode*)realloc(g->nodes[lev], cap * sizeof(ONode));
    memset(g->nodes[lev] + g->ncap[lev], 0, (cap - g->ncap[lev]) * sizeof(ONode));
    if (lev >= 1) {
        size_t cl = og_cl_len(g, lev);
        g->clist[lev] = (uint64_t*)realloc(g->clist[lev], cap * cl * sizeof(uint64_t));
    }
    g->ncap[lev] = cap;
}

/* PoolAlloc (AL.cpp:158-192) + SetupNode (VG.cpp:2512-2524) */
static size_t alloc_node(OGrid* g, int lev, const int32_t pos[3]) {
    pool_reserve(g, lev, g->ncnt[lev] + 1);
    size_t i = g->ncnt[lev]++;
    g->nused[lev]++;
    ONode* n = &g->nodes[lev][i];
    memset(n, 0, sizeof(ONode));
    n->lev = (uint8_t)lev;
    n->pos[0] = pos[0]; n->pos[1] = pos[1]; n->pos[2] = pos[2];
    n->childlist = UNDEFL;
    n->parent = UNDEFL;
    n->value[0] = n->value[1] = n->value[2] = -1;
    n->flags = 1;
    if (lev >= 1) { /* VG.cpp:979-985: child list from pool 1, filled with 0xFF */
        n->childlist = Elem(1, lev, i);
        size_t cl = og_cl_len(g, lev);
        memset(g->clist[lev] + i * cl, 0xFF, cl * sizeof(uint64_t));
    }
    return i;
}

/* PrepareVDBPartially (VG.cpp:3996-4016): lowest level with exactly one node */
static int top_lev(const OGrid* g) {
    int t = 1;
    for (int n = g->levs - 1; n >= 0; n--)
        if (g->ncnt[n] == 1) t = n;
    return t;
}

/* getChild (ND.cuh:115-124), int-typed result: empty slot -> -1 */
static int64_t get_child(const OGrid* g, const ONode* nd, int b) {
    uint64_t listid = nd->childlist;
    if (listid == UNDEFL) return -1;
    int clev = (int)((listid >> 8) & 0xFF);
    uint64_t cndx = listid >> 16;
    uint64_t e = g->clist[clev][cndx * og_cl_len(g, clev) + (size_t)b];
    if (e == UNDEF64) return -1;
    return (int64_t)(e >> 16);
}

/* child slot of pos inside node nd at level l; -1 if pos is outside the node */
static int child_slot(const OGrid* g, const ONode* nd, int l, const int32_t pos[3]) {
    int64_t rg = og_range(g, l);
    int r = og_res(g, l);
    int64_t p[3];
    for (int a = 0; a < 3; a++) {
        int64_t d = (int64_t)pos[a] - nd->pos[a];
        if (d < 0 || d >= rg) return -1; /* guard: the reference aliases here */
        p[a] = d * r / rg;
    }
    return (int)((p[2] * r + p[1]) * r + p[0]);
}

/* getPosParent (ND.cuh:303-348) */
static int64_t get_pos_parent(const OGrid* g, const int32_t pos[3], int stop_lev) {
    int tl = top_lev(g);
    if (g->ncnt[tl] == 0) return -1;
    const ONode* nd = &g->nodes[tl][0];
    int l = nd->lev;
    if (l == 0) return 0;
    while (l > 0) {
        int b = child_slot(g, nd, l, pos);
        if (b < 0) return -1;
        int64_t c = get_child(g, nd, b);
        l--;
        if (c < 0) return -1;
        if (l == stop_lev) return c;
        nd = &g->nodes[l][c];
    }
    return -1;
}

/* getParent (ND.cuh:350-397) */
static int64_t get_parent(const OGrid* g, int stop_lev, const int32_t pos[3]) {
    int tl = top_lev(g);
    const ONode* nd = &g->nodes[tl][0];
    if (!nd->flags) return 0;
    int l = nd->lev;
    if (l == stop_lev) return 0;
    while (l > stop_lev) {
        int b = child_slot(g, nd, l, pos);
        if (b < 0) return -1;
        l--;
        int64_t c = get_child(g, nd, b);
        if (c < 0) return -1;
        if (l == stop_lev) return c;
        nd = &g->nodes[l][c];
    }
    return -1;
}

/* getPosLeafParent (ND.cuh:255-288) */
static int64_t get_pos_leaf(const OGrid* g, const int32_t pos[3]) {
    int tl = top_lev(g);
    if (g->ncnt[tl] == 0) return -1;
    const ONode* nd = &g->nodes[tl][0];
    int l = nd->lev;
    if (l == 0) { /* single-leaf tree: guard on containment */
        for (int a = 0; a < 3; a++) {
            int64_t d = (int64_t)pos[a] - nd->pos[a];
            if (d < 0 || d >= og_range(g, 0)) return -1;
        }
        return 0;
    }
    while (1) {
        int b = child_slot(g, nd, l, pos);
        if (b < 0) return -1;
        int64_t c = get_child(g, nd, b);
        if (c < 0) return -1;
        l--;
        if (l == 0) return c;
        nd = &g->nodes[l][c];
    }
}

/* getNode(float pos) traversal used by UpdateApron (ND.cuh:199-253), for an
 * integer voxel w (the reference samples at w + 0.5). */
static int64_t get_leaf_at_voxel(const OGrid* g, const int32_t w[3]) {
    int tl = top_lev(g);
    if (g->ncnt[tl] == 0) return -1;
    int lev = tl;
    int64_t id = 0;
    const ONode* nd = &g->nodes[lev][0];
    while (lev > 0) {
        int b = child_slot(g, nd, lev, w);
        if (b < 0) return -1;
        lev--;
        int64_t c = get_child(g, nd, b);
        if (c < 0) return -1;
        id = c;
        nd = &g->nodes[lev][c];
    }
    for (int a = 0; a < 3; a++) { /* leaf containment guard */
        int64_t d = (int64_t)w[a] - nd->pos[a];
        if (d < 0 || d >= og_range(g, 0)) return -1;
    }
    return id;
}

/* gvdbLinkBricks (ND.cuh:470-505) for one node */
static void link_node(OGrid* g, int lev, size_t i) {
    ONode* node = &g->nodes[lev][i];
    if (!node->flags) return;
    int64_t pid = get_parent(g, lev + 1, node->pos);
    if (pid < 0) return;
    ONode* pn = &g->nodes[lev + 1][pid];
    int r = og_res(g, lev + 1);
    int64_t rg = og_range(g, lev + 1);
    int64_t p[3];
    for (int a = 0; a < 3; a++) p[a] = ((int64_t)node->pos[a] - pn->pos[a]) * r / rg;
    if (p[0] > r || p[0] < 0 || p[1] > r || p[1] < 0 || p[2] > r || p[2] < 0) return;
    int b = (int)((p[2] * r + p[1]) * r + p[0]);
    node->parent = ((uint64_t)pid << 16) | ((uint64_t)(lev + 1) << 8);
    uint64_t cndx = pn->childlist >> 16;
    if (cndx >= g->ncnt[lev + 1]) return;
    g->clist[lev + 1][cndx * og_cl_len(g, lev + 1) + b] = ((uint64_t)i << 16) | ((uint64_t)lev << 8);
}

static void link_all(OGrid* g, int D) { /* VG.cpp:1361-1369, top-down */
    for (int lev = D - 1; lev >= 0; lev--)
        for (size_t i = 0; i < g->ncnt[lev]; i++) link_node(g, lev, i);
}

/* gvdbDelinkLeafBricks (ND.cuh:401-429) */
static void delink_leaf(OGrid* g, size_t i) {
    ONode* node = &g->nodes[0][i];
    if (node->flags) return;
    if (node->parent == UNDEF64) return;
    int64_t pid = get_parent(g, 1, node->pos);
    if (pid < 0) { node->parent = UNDEF64; return; } /* guard: no parent reachable */
    ONode* pn = &g->nodes[1][pid];
    int r = og_res(g, 1);
    int64_t rg = og_range(g, 1);
    int64_t p[3];
    for (int a = 0; a < 3; a++) p[a] = ((int64_t)node->pos[a] - pn->pos[a]) * r / rg;
    int b = (int)((p[2] * r + p[1]) * r + p[0]);
    node->parent = UNDEF64;
    uint64_t cndx = pn->childlist >> 16;
    g->clist[1][cndx * og_cl_len(g, 1) + b] = UNDEF64;
}

/* gvdbDelinkBricks (ND.cuh:431-467) */
static void delink_upper(OGrid* g, int lev, size_t i) {
    ONode* node = &g->nodes[lev][i];
    if (node->parent == UNDEF64) { node->flags = 0; return; }
    size_t cl = og_cl_len(g, lev);
    const uint64_t* c = g->clist[lev] + i * cl;
    for (size_t k = 0; k < cl; k++)
        if (c[k] != UNDEF64) { node->flags = 1; return; }
    node->flags = 0;
    int64_t pid = get_parent(g, lev + 1, node->pos);
    if (pid < 0) { node->parent = UNDEF64; return; } /* guard */
    ONode* pn = &g->nodes[lev + 1][pid];
    int r = og_res(g, lev + 1);
    int64_t rg = og_range(g, lev + 1);
    int64_t p[3];
    for (int a = 0; a < 3; a++) p[a] = ((int64_t)node->pos[a] - pn->pos[a]) * r / rg;
    int b = (int)((p[2] * r + p[1]) * r + p[0]);
    node->parent = UNDEF64;
    uint64_t cndx = pn->childlist >> 16;
    g->clist[lev + 1][cndx * og_cl_len(g, lev + 1) + b] = UNDEF64;
}

/* ------------------------------------------------------------------------ */
/* keys                                                                      */

typedef struct { uint64_t* v; size_t n, cap; } KeyVec;
static void kv_push(KeyVec* k, uint64_t x) {
    if (k->n == k->cap) {
        k->cap = k->cap ? k->cap * 2 : 1024;
        k->v = (uint64_t*)realloc(k->v, k->cap * sizeof(uint64_t));
    }
    k->v[k->n++] = x;
}
static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}
/* key layout = u16[4]{z,y,x,lev} read as little-endian u64 (PT.cuh:372-380) */
static uint64_t make_key(int lev, int64_t x, int64_t y, int64_t z) {
    return ((uint64_t)(uint16_t)lev << 48) | ((uint64_t)(uint16_t)x << 32) |
           ((uint64_t)(uint16_t)y << 16) | (uint64_t)(uint16_t)z;
}
/* thrust::sort + gvdbFindUnique/CompactUnique (VG.cpp:843-928, PT.cuh:336-350) */
static void sort_unique(KeyVec* k) {
    if (k->n == 0) return;
    qsort(k->v, k->n, sizeof(uint64_t), cmp_u64);
    size_t w = 1;
    for (size_t i = 1; i < k->n; i++)
        if (k->v[i] != k->v[w - 1]) k->v[w++] = k->v[i];
    k->n = w;
}

/* Allocate nodes for sorted unique keys, level by level (VG.cpp:1306-1330) */
static void alloc_from_keys(OGrid* g, const KeyVec* k, int D) {
    for (int lev = 0; lev < D; lev++) {
        int64_t rg = og_range(g, lev);
        for (size_t i = 0; i < k->n; i++) {
            uint64_t key = k->v[i];
            int kl = (int)((key >> 48) & 0xFF);
            if (kl != lev) continue;
            int32_t pos[3];
            pos[0] = (int32_t)(((key >> 32) & 0xFFFF) * rg);
            pos[1] = (int32_t)(((key >> 16) & 0xFFFF) * rg);
            pos[2] = (int32_t)((key & 0xFFFF) * rg);
            alloc_node(g, lev, pos);
        }
    }
}

static inline void load_point(const char* base, int64_t i, int stride, int off, float p[3]) {
    const float* q = (const float*)(base + (size_t)i * (size_t)stride + (size_t)off);
    p[0] = q[0]; p[1] = q[1]; p[2] = q[2];
}

/* GetCoveringNode, float version (PT.cuh:88-100), as a node coordinate */
static int64_t cover_coord(float w, int64_t rg) {
    float fr = (float)rg;
    float np = ceilf(w / fr) * fr;
    int32_t ni = (int32_t)np;
    if (w < (float)ni) ni -= (int32_t)rg;
    return (int64_t)ni / rg;
}

static int in_root(const OGrid* g, int D, const int64_t np[3]) {
    const ONode* root = &g->nodes[D][0];
    int64_t rg = og_range(g, D);
    for (int a = 0; a < 3; a++) {
        if (np[a] < root->pos[a] || np[a] >= root->pos[a] + rg) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------------------ */
/* public API                                                                */

OGrid* og_create(int levs, const int* log2dim_leaf_first) {
    if (levs < 2 || levs > OG_MAXLEV) return NULL;
    OGrid* g = (OGrid*)calloc(1, sizeof(OGrid));
    g->levs = levs;
    int64_t rg = 1;
    for (int l = 0; l < levs; l++) {
        int d = log2dim_leaf_first[l];
        if (d <= 0) d = 1; /* VG.cpp:2394 */
        g->log2dim[l] = d;
        g->res[l] = 1 << d;
        rg *= g->res[l];
        g->range[l] = rg;
    }
    g->rebuild_topo = 1;
    g->curr_depth = -1;
    g->def_ax = 16; g->def_ay = 16; g->def_az = 1; /* VG.cpp:2348 */
    g->sc_size = 4;
    g->nthreads = 0;
    g->cpu_root = UNDEFL;
    return g;
}

void og_destroy(OGrid* g) {
    if (!g) return;
    for (int l = 0; l < OG_MAXLEV; l++) { free(g->nodes[l]); free(g->clist[l]); }
    for (int c = 0; c < OG_MAXCHAN; c++) free(g->chan[c].data);
    free(g->amap); free(g->sc_map); free(g->sc_cnt); free(g->sc_off); free(g->sc_pts); free(g->sc_clr);
    free(g);
}

void og_set_threads(OGrid* g, int n) { g->nthreads = n; }
void og_set_channel_default(OGrid* g, int ax, int ay, int az) { g->def_ax = ax; g->def_ay = ay; g->def_az = az; }
void og_request_full_rebuild(OGrid* g, int tf) { g->rebuild_topo = tf ? 1 : 0; }

static void chan_resize(OGrid* g, int c, size_t slots) {
    OChan* ch = &g->chan[c];
    if (slots <= ch->cap_slots) return;
    size_t per = 18 * 18 * 18;
    ch->data = (double*)realloc(ch->data, slots * per * sizeof(double));
    memset(ch->data + ch->cap_slots * per, 0, (slots - ch->cap_slots) * per * sizeof(double));
    ch->cap_slots = slots;
}

/* AddChannel (VG.cpp:2437-2453) + AtlasCreate (AL.cpp:528-560) */
int og_add_channel(OGrid* g, int chan, int dtype, int apron, int ax, int ay, int az) {
    if (chan < 0 || chan >= OG_MAXCHAN || apron != 1) return OG_INVALID_ARG;
    if (ax == 0 && ay == 0 && az == 0) {
        if (chan == 0) { ax = g->def_ax; ay = g->def_ay; az = g->def_az; }
        else { ax = g->ax; ay = g->ay; az = g->az; }
    }
    if (chan == 0) { g->ax = ax; g->ay = ay; g->az = az; }
    g->chan[chan].used = 1;
    g->chan[chan].dtype = dtype;
    g->chan[chan].apron = apron;
    chan_resize(g, chan, (size_t)g->ax * g->ay * g->az);
    return OG_OK;
}

/* Clear (VG.cpp:2487-2503) */
static void og_clear(OGrid* g) {
    for (int l = 0; l < OG_MAXLEV; l++) { g->ncnt[l] = 0; g->nused[l] = 0; }
    g->atlas_last = 0;
    g->rebuild_topo = 1;
}

/* GetBoundingBox (VG.cpp:5404-5467) */
static void bbox(OGrid* g, const char* pos, int64_t n, int stride, int off, const float orig[3]) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        for (int a = 0; a < 3; a++) {
            float w = p[a] + orig[a];
            if (w < mn[a]) mn[a] = w;
            if (w > mx[a]) mx[a] = w;
        }
    }
    for (int a = 0; a < 3; a++) {
        float lo = mn[a] - 1.0f, hi = mx[a] + 2.0f;
        g->posmin[a] = 0 > lo ? 0 : lo;
        g->posmax[a] = 0 > hi ? 0 : hi;
    }
}

/* DetermineDepth (VG.cpp:821-837) with GetCoveringNode(int) (VG.cpp:2915-2931) */
static int determine_depth(const OGrid* g, int32_t root_pos[3]) {
    int32_t pmin[3], pmax[3];
    for (int a = 0; a < 3; a++) { pmin[a] = (int32_t)g->posmin[a]; pmax[a] = (int32_t)g->posmax[a]; }
    for (int lev = 0; lev < g->levs; lev++) {
        int64_t rg = og_range(g, lev);
        int same = 1;
        for (int a = 0; a < 3; a++) if (pmin[a] / rg != pmax[a] / rg) same = 0;
        if (same) {
            for (int a = 0; a < 3; a++) root_pos[a] = (int32_t)((pmin[a] / rg) * rg);
            return lev;
        }
    }
    return -1;
}

/* ActivateBricksGPU (VG.cpp:1229-1413) */
static void activate_bricks(OGrid* g, const char* pos, int64_t n, int stride, int off,
                            const float orig[3], int D, const int32_t root_pos[3]) {
    KeyVec k = {0};
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        float w[3] = {p[0] + orig[0], p[1] + orig[1], p[2] + orig[2]};
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue; /* PT.cuh:361-371 */
        for (int lev = 0; lev < D; lev++) {
            int64_t rg = og_range(g, lev);
            kv_push(&k, make_key(lev, cover_coord(w[0], rg), cover_coord(w[1], rg), cover_coord(w[2], rg)));
        }
    }
    sort_unique(&k);
    /* root first (VG.cpp:1288-1300) */
    size_t ri = alloc_node(g, D, root_pos);
    (void)ri;
    alloc_from_keys(g, &k, D);
    link_all(g, D);
    free(k.v);
}

/* box enumeration of gvdbCalcExtraBrickId (PT.cuh:467-512) and
 * gvdbCalcIncreExtraBrickId (PT.cuh:420-465). hi_mul = 2 (extra) or 1 (incr). */
static void box_keys(OGrid* g, const char* pos, int64_t n, int stride, int off, const float orig[3],
                     float radius, int hi_mul, int D, KeyVec* k, int* markers) {
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        float w[3] = {p[0] + orig[0], p[1] + orig[1], p[2] + orig[2]};
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
        int32_t bmin[3], bmax[3];
        for (int a = 0; a < 3; a++) {
            bmin[a] = (int32_t)((float)(int32_t)w[a] - radius);
            bmax[a] = (int32_t)((float)(int32_t)w[a] + (hi_mul == 2 ? 2.0f * radius : radius));
        }
        for (int lev = 0; lev < D; lev++) {
            int32_t rr = (int32_t)og_range(g, lev);
            int32_t lo[3], hi[3];
            for (int a = 0; a < 3; a++) { lo[a] = bmin[a] / rr * rr; hi[a] = bmax[a] / rr * rr; }
            int32_t np[3];
            for (np[0] = lo[0]; np[0] <= hi[0]; np[0] += rr)
                for (np[1] = lo[1]; np[1] <= hi[1]; np[1] += rr)
                    for (np[2] = lo[2]; np[2] <= hi[2]; np[2] += rr) {
                        int64_t npl[3] = {np[0], np[1], np[2]};
                        if (np[0] < 0 || np[1] < 0 || np[2] < 0 || !in_root(g, D, npl)) continue; /* guard */
                        int64_t pid = get_pos_parent(g, np, lev);
                        if (pid < 0) {
                            kv_push(k, make_key(lev, np[0] / rr, np[1] / rr, np[2] / rr));
                        } else if (lev == 0 && markers) {
                            markers[pid] = 1;
                        }
                    }
        }
    }
}

/* ActivateExtraBricksGPU (VG.cpp:931-1016) */
static void activate_extra(OGrid* g, const char* pos, int64_t n, int stride, int off,
                           const float orig[3], float radius, int D) {
    KeyVec k = {0};
    box_keys(g, pos, n, stride, off, orig, radius, 2, D, &k, NULL);
    sort_unique(&k);
    alloc_from_keys(g, &k, D);
    link_all(g, D);
    free(k.v);
}

/* ActivateIncreBricksGPU (VG.cpp:1020-1156) */
static void activate_incre(OGrid* g, const char* pos, int64_t n, int stride, int off,
                           const float orig[3], float radius, int D, int accum) {
    size_t nleaf = g->ncnt[0];
    if (nleaf == 0) return;
    int* markers = (int*)calloc(nleaf, sizeof(int));
    if (accum)
        for (size_t i = 0; i < nleaf; i++) markers[i] = g->nodes[0][i].flags;
    KeyVec k = {0};
    box_keys(g, pos, n, stride, off, orig, radius, 1, D, &k, markers);
    if (k.n == 0) { free(markers); return; } /* VG.cpp:1066: flags untouched */
    sort_unique(&k);
    for (size_t i = 0; i < nleaf; i++) g->nodes[0][i].flags = (uint8_t)markers[i];
    alloc_from_keys(g, &k, D);
    link_all(g, D);
    for (size_t i = 0; i < g->ncnt[0]; i++) delink_leaf(g, i);
    for (int lev = 1; lev < D; lev++)
        for (size_t i = 0; i < g->ncnt[lev]; i++) delink_upper(g, lev, i);
    size_t used = 0;
    for (size_t i = 0; i < g->ncnt[0]; i++) used += g->nodes[0][i].flags ? 1 : 0;
    g->nused[0] = used;
    free(markers);
    free(k.v);
}

static int depth_error(int D) {
    if (D < 0) return OG_DEPTH_UNSUPPORTED;
    if (D == 0) return OG_DEPTH_UNSUPPORTED; /* VG.cpp:1187-1190 */
    if (D > 5) return OG_DEPTH_UNSUPPORTED;  /* VG.cpp:1191-1194 */
    return OG_OK;
}

/* RebuildTopology (VG.cpp:1181-1218) */
int og_rebuild_topology(OGrid* g, const void* pos, int64_t n, int stride, int off, float radius, const float orig[3]) {
    if (n <= 0) return OG_NOOP;
    bbox(g, (const char*)pos, n, stride, off, orig);
    int32_t root_pos[3];
    int D = determine_depth(g, root_pos);
    int e = depth_error(D);
    if (e) return e;
    if (g->rebuild_topo) {
        og_clear(g);
    } else if (D != g->curr_depth) {
        og_clear(g);
        g->rebuild_topo = 1;
        g->curr_depth = D;
    }
    g->last_depth = D;
    if (g->rebuild_topo) {
        activate_bricks(g, (const char*)pos, n, stride, off, orig, D, root_pos);
        if (radius >= 1) activate_extra(g, (const char*)pos, n, stride, off, orig, radius, D);
        g->rebuild_topo = 0;
    } else {
        activate_incre(g, (const char*)pos, n, stride, off, orig, radius, D, 0);
    }
    return OG_OK;
}

/* AccumulateTopology (VG.cpp:1158-1178) */
int og_accumulate_topology(OGrid* g, const void* pos, int64_t n, int stride, int off, float radius,
                           const float orig[3], int min_depth) {
    if (n <= 0) return OG_NOOP;
    bbox(g, (const char*)pos, n, stride, off, orig);
    int32_t root_pos[3];
    int D = determine_depth(g, root_pos);
    if (D >= 0 && D < min_depth) D = min_depth;
    int e = depth_error(D);
    if (e) return e;
    if (g->rebuild_topo) return og_rebuild_topology(g, pos, n, stride, off, radius, orig);
    g->last_depth = D;
    activate_incre(g, (const char*)pos, n, stride, off, orig, radius, D, 1);
    return OG_OK;
}

/* UpdateAtlas (VG.cpp:2630-2704), AtlasResize (AL.cpp:622-650), AtlasAlloc (AL.cpp:692-703),
 * getAtlasPos (AL.cpp:705-715), ClearMapping/AssignMapping (VG.cpp:2557-2590). */
int og_update_atlas(OGrid* g) {
    if (!g->chan[0].used) return OG_INVALID_ARG;
    size_t total = g->ncnt[0];
    size_t used = g->nused[0];
    g->atlas_last = 0;
    size_t amax = (size_t)g->ax * g->ay * g->az;
    if (used > amax) {
        g->az = (int)ceil((double)((float)used / (float)(g->ax * g->ay)));
    }
    int layer = g->ax * g->ay;
    for (size_t i = 0; i < total; i++) {
        ONode* nd = &g->nodes[0][i];
        if (!nd->flags) continue;
        if ((size_t)g->atlas_last >= (size_t)g->ax * g->ay * g->az) {
            size_t ml = (size_t)g->atlas_last + layer;
            g->az = (int)ceil((double)((float)ml / (float)layer));
        }
        int id = g->atlas_last++;
        int a2 = g->ax * g->ay;
        int pz = id / a2, rem = id - pz * a2;
        int py = rem / g->ax, px = rem - py * g->ax;
        nd->value[0] = px * 18 + 1;
        nd->value[1] = py * 18 + 1;
        nd->value[2] = pz * 18 + 1;
    }
    size_t slots = (size_t)g->ax * g->ay * g->az;
    for (int c = 0; c < OG_MAXCHAN; c++) if (g->chan[c].used) chan_resize(g, c, slots);
    g->amap = (OAtlasNode*)realloc(g->amap, slots * sizeof(OAtlasNode));
    g->amap_cnt = slots;
    for (size_t s = 0; s < slots; s++) {
        g->amap[s].pos[0] = g->amap[s].pos[1] = g->amap[s].pos[2] = -1;
        g->amap[s].leaf = -1;
    }
    for (size_t i = 0; i < total; i++) {
        ONode* nd = &g->nodes[0][i];
        if (!nd->flags) continue;
        int s = ((nd->value[2] / 18) * g->ay + nd->value[1] / 18) * g->ax + nd->value[0] / 18;
        g->amap[s].pos[0] = nd->pos[0]; g->amap[s].pos[1] = nd->pos[1]; g->amap[s].pos[2] = nd->pos[2];
        g->amap[s].leaf = (int32_t)i;
    }
    return OG_OK;
}

static int64_t leaf_slot(const OGrid* g, const ONode* nd) {
    if (nd->value[0] < 0) return -1;
    return ((int64_t)(nd->value[2] / 18) * g->ay + nd->value[1] / 18) * g->ax + nd->value[0] / 18;
}

/* subcell candidate range of one coordinate (PT.cuh:286-291) */
static inline void sc_range(float w, float R, int sc, int32_t* lo, int32_t* hi) {
    *lo = ((int32_t)(w - R) / sc) * sc;
    *hi = ((int32_t)(w + 1.0f + R) / sc) * sc;
}

/* InsertPointsSubcell (VG.cpp:4971-5092): SetFlagSubcell (PT.cuh:109-118), CountSubcell
 * (PT.cuh:275-315), PrefixSum, InsertSubcell (PT.cuh:218-273).  Lists are built in a
 * deterministic order (point order); the reference's order within a list is arbitrary. */
/* InsertPointsSubcell_FP16 (VG.cpp:5094-5189, gvdbInsertSubcell_fp16 PT.cuh:154-216) stores
 * each position quantised to 16 bits per axis over the point bounds [PosMin, PosMin +
 * PosRange] (GetBoundingBox, VG.cpp:5404-5467), q = trunc((w - min) / range * 65535);
 * GatherLevelSet_FP16 (PT.cuh:775-811) reads q / 65535 * range + min.  The lists here hold
 * that dequantised position, in FP32 with one rounding per operation. */
static inline float quant16(float w, float mn, float rg) {
    if (!(rg > 0.0f)) return mn;
    float t = ((w - mn) / rg) * 65535.0f;
    unsigned q = t <= 0.0f ? 0u : (t >= 65535.0f ? 65535u : (unsigned)t);
    return ((float)q / 65535.0f) * rg + mn;
}

static int insert_subcell(OGrid* g, int sc, const void* posv, int64_t n, int stride, int off, float R,
                          const float trans[3], int64_t* out_len, int fp16, const char* clr, int clr_stride,
                          int clr_off);

int og_insert_points_subcell(OGrid* g, int sc, const void* posv, int64_t n, int stride, int off,
                             float R, const float trans[3], int64_t* out_len) {
    return insert_subcell(g, sc, posv, n, stride, off, R, trans, out_len, 0, NULL, 0, 0);
}
/* InsertPointsSubcell with a point colour buffer (SetPoints' third DataPtr): each list
 * entry also carries the point's colour, the uint at clr + i*clr_stride + clr_off
 * (gvdbInsertSubcell, PT.cuh:236, 269) */
int og_insert_points_subcell_clr(OGrid* g, int sc, const void* posv, int64_t n, int stride, int off,
                                 float R, const float trans[3], const void* clr, int clr_stride, int clr_off,
                                 int64_t* out_len) {
    return insert_subcell(g, sc, posv, n, stride, off, R, trans, out_len, 0, (const char*)clr, clr_stride, clr_off);
}
int og_insert_points_subcell_fp16(OGrid* g, int sc, const void* posv, int64_t n, int stride, int off,
                                  float R, const float trans[3], int64_t* out_len) {
    return insert_subcell(g, sc, posv, n, stride, off, R, trans, out_len, 1, NULL, 0, 0);
}

static int insert_subcell(OGrid* g, int sc, const void* posv, int64_t n, int stride, int off, float R,
                          const float trans[3], int64_t* out_len, int fp16, const char* clr, int clr_stride,
                          int clr_off) {
    const char* pos = (const char*)posv;
    const float prange[3] = {g->posmax[0] - g->posmin[0], g->posmax[1] - g->posmin[1], g->posmax[2] - g->posmin[2]};
    if (g->nused[0] == 0) return OG_NOOP;
    if (sc <= 0 || (16 % sc) != 0 || og_res(g, 0) != 16) return OG_INVALID_ARG;
    g->sc_size = sc;
    int scres = og_res(g, 0) / sc;
    int scpb = scres * scres * scres;
    size_t nleaf = g->ncnt[0];
    free(g->sc_map);
    g->sc_map = (int*)malloc((nleaf + 1) * sizeof(int));
    size_t nl = 0;
    for (size_t i = 0; i < nleaf; i++) {
        g->sc_map[i] = (int)nl;
        if (g->nodes[0][i].parent != UNDEF64) nl++;
    }
    g->sc_nbricks = nl;
    size_t nsc = nl * (size_t)scpb;
    free(g->sc_cnt); free(g->sc_off); free(g->sc_pts); free(g->sc_clr);
    g->sc_clr = NULL;
    g->sc_cnt = (int64_t*)calloc(nsc + 1, sizeof(int64_t));
    g->sc_off = (int64_t*)calloc(nsc + 1, sizeof(int64_t));
    int D = g->last_depth;
    (void)D;
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            int64_t acc = 0;
            for (size_t s = 0; s < nsc; s++) { g->sc_off[s] = acc; acc += g->sc_cnt[s]; g->sc_cnt[s] = 0; }
            g->sc_off[nsc] = acc;
            g->sc_len = acc;
            g->sc_pts = (float*)malloc((size_t)(acc > 0 ? acc : 1) * 3 * sizeof(float));
            if (clr) g->sc_clr = (uint32_t*)malloc((size_t)(acc > 0 ? acc : 1) * sizeof(uint32_t));
        }
        for (int64_t i = 0; i < n; i++) {
            float p[3];
            load_point(pos, i, stride, off, p);
            if (p[2] == NOHIT) continue;
            float w[3] = {p[0] + trans[0], p[1] + trans[1], p[2] + trans[2]};
            if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
            int32_t lo[3], hi[3];
            for (int a = 0; a < 3; a++) sc_range(w[a], R, sc, &lo[a], &hi[a]);
            int32_t s3[3];
            for (s3[0] = lo[0]; s3[0] <= hi[0]; s3[0] += sc)
                for (s3[1] = lo[1]; s3[1] <= hi[1]; s3[1] += sc)
                    for (s3[2] = lo[2]; s3[2] <= hi[2]; s3[2] += sc) {
                        if (s3[0] < 0 || s3[1] < 0 || s3[2] < 0) continue; /* guard */
                        int64_t leaf = get_pos_leaf(g, s3);
                        if (leaf < 0) continue;
                        const ONode* ln = &g->nodes[0][leaf];
                        int lx = (s3[0] - ln->pos[0]) / sc, ly = (s3[1] - ln->pos[1]) / sc, lz = (s3[2] - ln->pos[2]) / sc;
                        if (lx < 0 || ly < 0 || lz < 0 || lx >= scres || ly >= scres || lz >= scres) continue;
                        if (ln->parent == UNDEF64) continue;
                        size_t idx = (size_t)g->sc_map[leaf] * scpb + (size_t)((lz * scres + ly) * scres + lx);
                        if (pass == 0) {
                            g->sc_cnt[idx]++;
                        } else {
                            int64_t at = g->sc_off[idx] + g->sc_cnt[idx]++;
                            for (int a = 0; a < 3; a++)
                                g->sc_pts[at * 3 + a] = fp16 ? quant16(w[a], g->posmin[a], prange[a]) : w[a];
                            if (clr) memcpy(&g->sc_clr[at], clr + (size_t)i * clr_stride + clr_off, 4);
                        }
                    }
        }
    }
    g->sc_nleaf = nleaf;
    if (out_len) *out_len = g->sc_len;
    return OG_OK;
}

/* gvdbGatherDensity / gvdbGatherLevelSet (PT.cuh:696-773) in FP64.
 * mode 0 = density: v = max(accum ? old : 0, max_j(rho - |p_j - v|))
 * mode 1 = level set: v = min(accum ? old : 3, min_j(|p_j - v| - rho)) */
/* RGBA8 byte of an averaged colour component: the reference's uchar(c * 255.0f)
 * (CLR2CHAR, PT.cuh:16) as its kernels convert it (pinned by the golden fixtures):
 * truncation toward zero to a 32-bit unsigned integer (NaN and negative values to 0,
 * values of 2^32 and more to 0xFFFFFFFF), then its low byte, so that a component
 * above 255 wraps (an opaque average (1 + n) / n of the non-accumulating start). */
static uint32_t clr_byte(float c255) {
    if (!(c255 == c255) || c255 <= 0.0f) return 0u;
    if (c255 >= 4294967296.0f) return 255u;
    return (uint32_t)c255 & 0xFFu;
}

/* The colour of one voxel (gvdbGatherDensity / gvdbGatherLevelSet, PT.cuh:717-731,
 * 757-771): clr = accum ? CHAR2CLR(old) : (0, 0, 0, 1), plus CHAR2CLR of every list
 * entry of the voxel's subcell, divided by (list length + accum), CLR2CHAR.  Here the
 * sum is formed exactly, in integer byte units (the reference adds the FP32 terms
 * c/255 in list order, which is arbitrary), then divided by 255 once; the remaining
 * FP32 operations are the reference's: c / (n + accum), c * 255, truncation. */
static uint32_t clr_average(const uint64_t sum[4], int64_t cnt, uint32_t old, int accum) {
    uint32_t out = 0;
    for (int k = 0; k < 4; k++) {
        uint64_t t = sum[k] + (accum ? ((old >> (8 * k)) & 0xFFu) : (k == 3 ? 255u : 0u));
        float c = (float)t / 255.0f;
        c = c / (float)(cnt + (accum ? 1 : 0));
        out |= clr_byte(c * 255.0f) << (8 * k);
    }
    return out;
}

int og_gather(OGrid* g, int mode, float rho, int chan, int accum);
/* the gather with the colour channel clr_chan (T_UCHAR4; -1 = none): colours are
 * averaged when the last insert carried point colours (VG.cpp:5063, PT.cuh:728) */
int og_gather_clr(OGrid* g, int mode, float rho, int chan, int clr_chan, int accum) {
    int rc = og_gather(g, mode, rho, chan, accum);
    if (rc != OG_OK || clr_chan < 0 || !g->sc_clr) return rc;
    if (clr_chan >= OG_MAXCHAN || !g->chan[clr_chan].used || g->chan[clr_chan].dtype != 2) return OG_INVALID_ARG;
    int sc = g->sc_size;
    int scres = og_res(g, 0) / sc;
    int scpb = scres * scres * scres;
    size_t nleaf = g->ncnt[0];
    double* atl = g->chan[clr_chan].data;
#ifdef _OPENMP
    int nt = g->nthreads > 0 ? g->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
#endif
    for (int64_t i = 0; i < (int64_t)nleaf; i++) {
        const ONode* nd = &g->nodes[0][i];
        if (nd->parent == UNDEF64) continue;
        int64_t slot = leaf_slot(g, nd);
        if (slot < 0) continue;
        double* brick = atl + (size_t)slot * 5832;
        for (int s = 0; s < scpb; s++) {
            size_t idx = (size_t)g->sc_map[i] * scpb + s;
            int sx = s % scres, sy = (s / scres) % scres, sz = s / (scres * scres);
            int64_t beg = g->sc_len ? g->sc_off[idx] : 0, cnt = g->sc_len ? g->sc_off[idx + 1] - g->sc_off[idx] : 0;
            uint64_t sum[4] = {0, 0, 0, 0};
            for (int64_t j = 0; j < cnt; j++) {
                uint32_t c = g->sc_clr[beg + j];
                for (int k = 0; k < 4; k++) sum[k] += (c >> (8 * k)) & 0xFFu;
            }
            for (int tz = 0; tz < sc; tz++)
                for (int ty = 0; ty < sc; ty++)
                    for (int tx = 0; tx < sc; tx++) {
                        int lx = sx * sc + tx, ly = sy * sc + ty, lz = sz * sc + tz;
                        double* cell = brick + ((size_t)(lz + 1) * 18 + (ly + 1)) * 18 + (lx + 1);
                        *cell = (double)clr_average(sum, cnt, (uint32_t)*cell, accum);
                    }
        }
    }
    return OG_OK;
}

int og_gather(OGrid* g, int mode, float rho, int chan, int accum) {
    if (chan < 0 || chan >= OG_MAXCHAN || !g->chan[chan].used) return OG_INVALID_ARG;
    if (g->nused[0] == 0) return OG_NOOP;
    if (mode == 0 && g->sc_len == 0) return OG_NOOP; /* VG.cpp:5321 */
    if (!g->sc_map || g->sc_nleaf != g->ncnt[0]) return OG_INVALID_ARG; /* lists are stale */
    int sc = g->sc_size;
    int scres = og_res(g, 0) / sc;
    int scpb = scres * scres * scres;
    size_t nleaf = g->ncnt[0];
    double* atl = g->chan[chan].data;
    double r = (double)rho;
#ifdef _OPENMP
    int nt = g->nthreads > 0 ? g->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
#endif
    for (int64_t i = 0; i < (int64_t)nleaf; i++) {
        const ONode* nd = &g->nodes[0][i];
        if (nd->parent == UNDEF64) continue;
        int64_t slot = leaf_slot(g, nd);
        if (slot < 0) continue;
        double* brick = atl + (size_t)slot * 5832;
        for (int s = 0; s < scpb; s++) {
            size_t idx = (size_t)g->sc_map[i] * scpb + s;
            int sx = s % scres, sy = (s / scres) % scres, sz = s / (scres * scres);
            int64_t beg = g->sc_len ? g->sc_off[idx] : 0, cnt = g->sc_len ? g->sc_off[idx + 1] - g->sc_off[idx] : 0;
            for (int tz = 0; tz < sc; tz++)
                for (int ty = 0; ty < sc; ty++)
                    for (int tx = 0; tx < sc; tx++) {
                        int lx = sx * sc + tx, ly = sy * sc + ty, lz = sz * sc + tz;
                        double vx = nd->pos[0] + lx, vy = nd->pos[1] + ly, vz = nd->pos[2] + lz;
                        double* cell = brick + ((size_t)(lz + 1) * 18 + (ly + 1)) * 18 + (lx + 1);
                        double val = accum ? *cell : (mode == 0 ? 0.0 : 3.0);
                        for (int64_t j = 0; j < cnt; j++) {
                            const float* q = g->sc_pts + (size_t)(beg + j) * 3;
                            double dx = (double)q[0] - vx, dy = (double)q[1] - vy, dz = (double)q[2] - vz;
                            double c = sqrt(dx * dx + dy * dy + dz * dz);
                            if (mode == 0) { double t = r - c; if (t > val) val = t; }
                            else { double t = c - r; if (t < val) val = t; }
                        }
                        *cell = val;
                    }
        }
    }
    return OG_OK;
}

/* UpdateApron<T> (OP.cuh:72-131): every apron voxel of every assigned slot gets the
 * value of the interior voxel at the same index-space position, or boundval. */
int og_update_apron(OGrid* g, int chan, float boundval) {
    if (chan < 0 || chan >= OG_MAXCHAN || !g->chan[chan].used) return OG_INVALID_ARG;
    double* atl = g->chan[chan].data;
    /* T_UCHAR4: make_uchar4(boundval, ...) (OP.cuh:140-143) */
    const uint32_t b8 = clr_byte(boundval);
    const double bv = g->chan[chan].dtype == 2 ? (double)(b8 | (b8 << 8) | (b8 << 16) | (b8 << 24)) : (double)boundval;
    int used = g->atlas_last;
#ifdef _OPENMP
    int nt = g->nthreads > 0 ? g->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (int s = 0; s < used; s++) {
        if (g->amap[s].leaf < 0) continue;
        const int32_t* bp = g->amap[s].pos;
        double* brick = atl + (size_t)s * 5832;
        for (int z = 0; z < 18; z++)
            for (int y = 0; y < 18; y++)
                for (int x = 0; x < 18; x++) {
                    if (x > 0 && x < 17 && y > 0 && y < 17 && z > 0 && z < 17) continue;
                    int32_t w[3] = {bp[0] + x - 1, bp[1] + y - 1, bp[2] + z - 1};
                    double v = bv;
                    int64_t nl = get_leaf_at_voxel(g, w);
                    if (nl >= 0) {
                        const ONode* nn = &g->nodes[0][nl];
                        int64_t ns = leaf_slot(g, nn);
                        if (ns >= 0) {
                            int lx = w[0] - nn->pos[0] + 1, ly = w[1] - nn->pos[1] + 1, lz = w[2] - nn->pos[2] + 1;
                            v = atl[(size_t)ns * 5832 + ((size_t)lz * 18 + ly) * 18 + lx];
                        }
                    }
                    brick[((size_t)z * 18 + y) * 18 + x] = v;
                }
    }
    return OG_OK;
}

/* FillChannel(chan, v) (VG.cpp:2456-2470) over every slot of the current atlas,
 * interior and apron: FP channels get v[0] (FUNC_FILL_F), T_UCHAR4 channels
 * CLR2INT(v0, v1, v2, 1) (FUNC_FILL_C4, OP.cuh:368-373; CLR2INT OP.cuh:20).  The
 * reference's fill kernel leaves the atlas's first voxel plane on each axis (an
 * apron plane) unwritten; here every voxel is written. */
void og_fill_channel(OGrid* g, int chan, const float v[4]) {
    if (chan < 0 || chan >= OG_MAXCHAN || !g->chan[chan].used) return;
    OChan* ch = &g->chan[chan];
    double val = (double)v[0];
    if (ch->dtype == 2) {
        uint32_t c = ((uint32_t)(1.0f * 255.0f) << 24) | ((uint32_t)(v[2] * 255.0f) << 16) |
                     ((uint32_t)(v[1] * 255.0f) << 8) | (uint32_t)(v[0] * 255.0f);
        val = (double)c;
    }
    size_t n = ch->cap_slots * 5832;
    for (size_t i = 0; i < n; i++) ch->data[i] = val;
}
/* ClearChannel (VG.cpp:1596-1603): every voxel of the atlas to 0 */
void og_clear_channel(OGrid* g, int chan) {
    if (chan < 0 || chan >= OG_MAXCHAN || !g->chan[chan].used) return;
    memset(g->chan[chan].data, 0, g->chan[chan].cap_slots * 5832 * sizeof(double));
}

/* ComputeBounds (VG.cpp:1792-1816): both corners start at the position of leaf 0
 * of the pool (flagged or not); every flagged leaf then widens them by its box
 * [pos, pos + range0).  out6 = {min xyz, max xyz}; returns 0 on an empty pool. */
int og_compute_bounds(const OGrid* g, float out6[6]) {
    if (g->ncnt[0] == 0) return 0;
    const int64_t rg = og_range(g, 0);
    float mn[3], mx[3];
    for (int a = 0; a < 3; a++) mn[a] = mx[a] = (float)g->nodes[0][0].pos[a];
    for (size_t i = 0; i < g->ncnt[0]; i++) {
        const ONode* nd = &g->nodes[0][i];
        if (!nd->flags) continue;
        for (int a = 0; a < 3; a++) {
            if ((float)nd->pos[a] < mn[a]) mn[a] = (float)nd->pos[a];
            if ((float)(nd->pos[a] + rg) > mx[a]) mx[a] = (float)(nd->pos[a] + rg);
        }
    }
    for (int a = 0; a < 3; a++) { out6[a] = mn[a]; out6[3 + a] = mx[a]; }
    return 1;
}

/* ------------------------------------------------------------------------ */
/* exports                                                                   */

int og_depth(const OGrid* g) { return g->last_depth; }
int og_top_lev(const OGrid* g) { return top_lev(g); }
int64_t og_node_count(const OGrid* g, int lev) { return (int64_t)g->ncnt[lev]; }
int64_t og_used_count(const OGrid* g, int lev) { return (int64_t)g->nused[lev]; }
const void* og_nodes(const OGrid* g, int lev) { return g->nodes[lev]; }
const uint64_t* og_childlist(const OGrid* g, int lev) { return g->clist[lev]; }
int og_childlist_len(const OGrid* g, int lev) { return (int)og_cl_len(g, lev); }
void og_bbox(const OGrid* g, float out[6]) {
    for (int a = 0; a < 3; a++) { out[a] = g->posmin[a]; out[3 + a] = g->posmax[a]; }
}
void og_atlas_dims(const OGrid* g, int out[4]) {
    out[0] = g->ax; out[1] = g->ay; out[2] = g->az; out[3] = g->atlas_last;
}
const void* og_atlas_map(const OGrid* g) { return g->amap; }
/* slot-major FP64 brick data (slot * 18^3 + (z*18+y)*18+x) */
const double* og_atlas_data(const OGrid* g, int chan) { return g->chan[chan].data; }
int64_t og_subcell_count(const OGrid* g) { return (int64_t)g->sc_nbricks * 64; }
const int64_t* og_subcell_offsets(const OGrid* g) { return g->sc_off; }
const float* og_subcell_points(const OGrid* g) { return g->sc_pts; }
int64_t og_subcell_len(const OGrid* g) { return g->sc_len; }
const int* og_subcell_map(const OGrid* g) { return g->sc_map; }

/* FP64 sum over the interior voxels of all assigned slots */
double og_checksum(const OGrid* g, int chan) {
    const double* atl = g->chan[chan].data;
    double s = 0;
    for (int k = 0; k < g->atlas_last; k++) {
        if (g->amap[k].leaf < 0) continue;
        const double* b = atl + (size_t)k * 5832;
        for (int z = 1; z < 17; z++)
            for (int y = 1; y < 17; y++)
                for (int x = 1; x < 17; x++) s += b[(z * 18 + y) * 18 + x];
    }
    return s;
}

/* SaveVBX (VG.cpp:1626-1767; format GVDB_FILESPEC.txt:12-122), version 1.11, one grid:
 * header (version, identity transform, grid count, grid offset table), grid header,
 * topology (levels, root id, per-level log2 dim / res / range / pool counts and widths),
 * pool 0 of every level, pool 1 of every level (level 0 has none), then each channel as
 * the atlas volume (ax*18 x ay*18 x az*18 voxels, x fastest) in FP32.  Slots past the
 * assigned ones are written as zero.  Returns 0 on success. */
int og_save_vbx(const OGrid* g, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    int nch = 0;
    while (nch < OG_MAXCHAN && g->chan[nch].used) nch++;
    const uint8_t major = 1, minor = 11;
    fwrite(&major, 1, 1, f);
    fwrite(&minor, 1, 1, f);
    const float pretrans[3] = {0, 0, 0}, angs[3] = {0, 0, 0}, scal[3] = {1, 1, 1}, trans[3] = {0, 0, 0};
    fwrite(pretrans, 4, 3, f);
    fwrite(angs, 4, 3, f);
    fwrite(scal, 4, 3, f);
    fwrite(trans, 4, 3, f);
    const int32_t num_grids = 1;
    fwrite(&num_grids, 4, 1, f);
    const long table = ftell(f);
    uint64_t goff = 0;
    fwrite(&goff, 8, 1, f);
    goff = (uint64_t)ftell(f);
    char name[256];
    memset(name, 0, sizeof(name));
    fwrite(name, 1, 256, f);
    const uint8_t dt = 'f', comps = 1, comp = 0, topo = 2, layout = 0;
    fwrite(&dt, 1, 1, f);
    fwrite(&comps, 1, 1, f);
    fwrite(&comp, 1, 1, f);
    const float vs[3] = {1, 1, 1};
    fwrite(vs, 4, 3, f);
    const int32_t leafcnt = (int32_t)g->ncnt[0];
    fwrite(&leafcnt, 4, 1, f);
    const int32_t leafdim[3] = {g->res[0], g->res[0], g->res[0]};
    fwrite(leafdim, 4, 3, f);
    const int32_t apron = 1, nch32 = nch;
    fwrite(&apron, 4, 1, f);
    fwrite(&nch32, 4, 1, f);
    const int32_t axisres[3] = {g->ax * 18, g->ay * 18, g->az * 18};
    const uint64_t atlas_sz = 4ull * (uint64_t)axisres[0] * (uint64_t)axisres[1] * (uint64_t)axisres[2];
    fwrite(&atlas_sz, 8, 1, f);
    fwrite(&topo, 1, 1, f);
    const int32_t reuse = 0;
    fwrite(&reuse, 4, 1, f);
    fwrite(&layout, 1, 1, f);
    const int32_t axiscnt[3] = {g->ax, g->ay, g->az};
    fwrite(axiscnt, 4, 3, f);
    fwrite(axisres, 4, 3, f);
    const int32_t levels = g->levs;
    fwrite(&levels, 4, 1, f);
    /* mRoot = PoolAlloc(0, D, ...) at a full rebuild (VG.cpp:1290): Elem(0, D, 0) */
    const int D = g->last_depth;
    const uint64_t root = (D >= 0 && D < g->levs && g->ncnt[D] > 0) ? ((uint64_t)D << 8) : 0xFFFFFFFFull;
    fwrite(&root, 8, 1, f);
    for (int l = 0; l < g->levs; l++) {
        const int32_t ld = g->log2dim[l], res = g->res[l];
        const int32_t rg[3] = {(int32_t)g->range[l], (int32_t)g->range[l], (int32_t)g->range[l]};
        const int32_t cnt0 = (int32_t)g->ncnt[l], w0 = (int32_t)sizeof(ONode);
        const int32_t cnt1 = l >= 1 ? (int32_t)g->ncnt[l] : 0, w1 = l >= 1 ? (int32_t)(og_cl_len(g, l) * 8) : 0;
        fwrite(&ld, 4, 1, f);
        fwrite(&res, 4, 1, f);
        fwrite(rg, 4, 3, f);
        fwrite(&cnt0, 4, 1, f);
        fwrite(&w0, 4, 1, f);
        fwrite(&cnt1, 4, 1, f);
        fwrite(&w1, 4, 1, f);
    }
    for (int l = 0; l < g->levs; l++)
        if (g->ncnt[l]) fwrite(g->nodes[l], sizeof(ONode), g->ncnt[l], f);
    for (int l = 1; l < g->levs; l++)
        if (g->ncnt[l]) fwrite(g->clist[l], 8, g->ncnt[l] * og_cl_len(g, l), f);
    const size_t W = (size_t)axisres[0], H = (size_t)axisres[1];
    float* slice = (float*)malloc(W * H * sizeof(float));
    for (int c = 0; c < nch; c++) {
        const int32_t ctype = 3, cstride = 4;
        fwrite(&ctype, 4, 1, f);
        fwrite(&cstride, 4, 1, f);
        for (int z = 0; z < axisres[2]; z++) {
            for (size_t y = 0; y < H; y++)
                for (size_t x = 0; x < W; x++) {
                    const int bx = (int)(x / 18), by = (int)(y / 18), bz = z / 18;
                    const int64_t slot = ((int64_t)bz * g->ay + by) * g->ax + bx;
                    float v = 0.0f;
                    if (slot < g->atlas_last && g->chan[c].data)
                        v = (float)g->chan[c].data[(size_t)slot * 5832 +
                                                   (size_t)(((z % 18) * 18 + (int)(y % 18)) * 18 + (int)(x % 18))];
                    slice[y * W + x] = v;
                }
            fwrite(slice, sizeof(float), W * H, f);
        }
    }
    free(slice);
    fseek(f, table, SEEK_SET);
    fwrite(&goff, 8, 1, f);
    return fclose(f) == 0 ? 0 : -1;
}

/* ------------------------------------------------------------------------ */
/* neighbour table, apron faces, smoothing (FP32 bricks)                     */

/* UpdateNeighbors (VG.cpp:2527-2556): for every leaf of the pool, the leaf at its
 * centre -/+ one brick along x, y, z (order -x, -y, -z, +x, +y, +z), as a pool
 * index, -1 where there is none.  The reference looks up from mRoot; here from the
 * traversal top level, as every lookup of this path. */
void og_update_neighbors(const OGrid* g, int32_t* out) {
    const int d = (int)g->range[0];
    const int dir[6][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (size_t n = 0; n < g->ncnt[0]; n++) {
        const ONode* nd = &g->nodes[0][n];
        for (int k = 0; k < 6; k++) {
            int32_t w[3];
            for (int a = 0; a < 3; a++) w[a] = nd->pos[a] + d / 2 + dir[k][a] * d;
            int64_t nl = (w[0] < 0 || w[1] < 0 || w[2] < 0) ? -1 : get_leaf_at_voxel(g, w);
            out[n * 6 + k] = (int32_t)nl;
        }
    }
}

/* slot owned by leaf nl (its mValue slot, and the atlas map names it), else -1 */
static int64_t owned_slot(const OGrid* g, int64_t nl) {
    if (nl < 0 || (size_t)nl >= g->ncnt[0]) return -1;
    int64_t s = leaf_slot(g, &g->nodes[0][nl]);
    if (s < 0 || s >= g->atlas_last || g->amap[s].leaf != nl) return -1;
    return s;
}

/* UpdateApronFaces (VG.cpp:4461-4496, gvdbUpdateApronFacesF OP.cuh:27-61) on FP32
 * padded bricks [slot][z][y][x]: for every assigned slot and each of its -x, -y, -z
 * neighbours (neighbour table), the slot's first interior plane goes to the
 * neighbour's far apron face and the neighbour's last interior plane to the slot's
 * near apron face.  Edges and corners are not written; a missing neighbour leaves the
 * face as it is. */
void og_apron_faces_f32(const OGrid* g, const int32_t* table, float* bricks) {
    for (int s = 0; s < g->atlas_last; s++) {
        int64_t L = g->amap[s].leaf;
        if (L < 0) continue;
        for (int side = 0; side < 3; side++) {
            int64_t ns = owned_slot(g, table[L * 6 + side]);
            if (ns < 0) continue;
            float* self = bricks + (size_t)s * 5832;
            float* nb = bricks + (size_t)ns * 5832;
            for (int u = 1; u <= 16; u++)
                for (int v = 1; v <= 16; v++) {
                    size_t si, sa, ni, na;
                    if (side == 0) {  /* x: (x, y=u, z=v) */
                        si = ((size_t)v * 18 + u) * 18 + 1;  sa = ((size_t)v * 18 + u) * 18 + 0;
                        ni = ((size_t)v * 18 + u) * 18 + 16; na = ((size_t)v * 18 + u) * 18 + 17;
                    } else if (side == 1) {  /* y: (x=u, y, z=v) */
                        si = ((size_t)v * 18 + 1) * 18 + u;  sa = ((size_t)v * 18 + 0) * 18 + u;
                        ni = ((size_t)v * 18 + 16) * 18 + u; na = ((size_t)v * 18 + 17) * 18 + u;
                    } else {  /* z: (x=u, y=v, z) */
                        si = ((size_t)1 * 18 + v) * 18 + u;  sa = ((size_t)0 * 18 + v) * 18 + u;
                        ni = ((size_t)16 * 18 + v) * 18 + u; na = ((size_t)17 * 18 + v) * 18 + u;
                    }
                    nb[na] = self[si];
                    self[sa] = nb[ni];
                }
        }
    }
}

/* UpdateApron (OP.cuh:72-131) on FP32 padded bricks: every apron voxel = the interior
 * voxel of the leaf at that index-space position, or boundval. */
void og_apron_full_f32(const OGrid* g, float* bricks, float boundval) {
    float* src = (float*)malloc((size_t)g->atlas_last * 5832 * sizeof(float));
    memcpy(src, bricks, (size_t)g->atlas_last * 5832 * sizeof(float));
    for (int s = 0; s < g->atlas_last; s++) {
        if (g->amap[s].leaf < 0) continue;
        const int32_t* bp = g->amap[s].pos;
        float* brick = bricks + (size_t)s * 5832;
        for (int z = 0; z < 18; z++)
            for (int y = 0; y < 18; y++)
                for (int x = 0; x < 18; x++) {
                    if (x > 0 && x < 17 && y > 0 && y < 17 && z > 0 && z < 17) continue;
                    int32_t w[3] = {bp[0] + x - 1, bp[1] + y - 1, bp[2] + z - 1};
                    float v = boundval;
                    int64_t nl = (w[0] < 0 || w[1] < 0 || w[2] < 0) ? -1 : get_leaf_at_voxel(g, w);
                    if (nl >= 0) {
                        const ONode* nn = &g->nodes[0][nl];
                        int64_t ns = leaf_slot(g, nn);
                        if (ns >= 0) {
                            int lx = w[0] - nn->pos[0] + 1, ly = w[1] - nn->pos[1] + 1, lz = w[2] - nn->pos[2] + 1;
                            v = src[(size_t)ns * 5832 + ((size_t)lz * 18 + ly) * 18 + lx];
                        }
                    }
                    brick[((size_t)z * 18 + y) * 18 + x] = v;
                }
    }
    free(src);
}

/* Compute(FUNC_SMOOTH) one iteration (gvdbOpSmooth, OP.cuh:383-400) on FP32 padded
 * bricks, interior voxels of every assigned slot, reading the values before the pass:
 * v = p1*c, then + x-1, x+1, y-1, y+1, z-1, z+1 in FP32; v = v / (p1 + 6.0) + p2 in
 * double (the source's double literal), rounded to float. */
void og_smooth_f32(const OGrid* g, float* bricks, float p1, float p2) {
    float* src = (float*)malloc((size_t)g->atlas_last * 5832 * sizeof(float));
    memcpy(src, bricks, (size_t)g->atlas_last * 5832 * sizeof(float));
    for (int s = 0; s < g->atlas_last; s++) {
        if (g->amap[s].leaf < 0) continue;
        const float* b = src + (size_t)s * 5832;
        float* o = bricks + (size_t)s * 5832;
        for (int z = 1; z < 17; z++)
            for (int y = 1; y < 17; y++)
                for (int x = 1; x < 17; x++) {
                    const size_t i = ((size_t)z * 18 + y) * 18 + x;
                    volatile float v = p1 * b[i];
                    v = v + b[i - 1];
                    v = v + b[i + 1];
                    v = v + b[i - 18];
                    v = v + b[i + 18];
                    v = v + b[i - 324];
                    v = v + b[i + 324];
                    o[i] = (float)((double)v / ((double)p1 + 6.0) + (double)p2);
                }
    }
    free(src);
}

/* ------------------------------------------------------------------------ */
/* legacy InsertPoints + ScatterDensity                                      */

/* gvdbInsertPoints (PT.cuh:19-35): leaf of each point (w = p + trans; NOHIT, negative or
 * outside every leaf -> -1); counts[leaf] = points in it */
void og_insert_points(const OGrid* g, const void* posv, int64_t n, int stride, int off, const float trans[3],
                      int32_t* pnode, int64_t* counts) {
    const char* pos = (const char*)posv;
    for (size_t l = 0; l < g->ncnt[0]; l++) counts[l] = 0;
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        int64_t leaf = -1;
        if (p[2] != NOHIT) {
            float w[3] = {p[0] + trans[0], p[1] + trans[1], p[2] + trans[2]};
            if (w[0] >= 0 && w[1] >= 0 && w[2] >= 0) {
                int32_t v[3] = {(int32_t)w[0], (int32_t)w[1], (int32_t)w[2]};
                leaf = get_leaf_at_voxel(g, v);
            }
        }
        pnode[i] = (int32_t)leaf;
        if (leaf >= 0) counts[leaf]++;
    }
}

/* distFunc (PT.cuh:516-523): c = (bx*bx + by*by + bz*bz) / (r*r) in FP32, then
 * 1.0 + c*(-3 + c*(3 - c)) with the double literal's last addition in double */
static float dist_func(float px, float py, float pz, float bx, float by, float bz, float r) {
    bx -= px;
    by -= py;
    bz -= pz;
    float d2 = bx * bx + by * by;
    d2 = d2 + bz * bz;
    float c = d2 / (r * r);
    float t = c * (-3.0f + c * (3.0f - c));
    return (float)(1.0 + (double)t);
}

/* gvdbScatterPointDensity (PT.cuh:525-571) into channel 0 (FP64 here): every point of a
 * leaf with an atlas slot adds distFunc at the voxel it lies in and, with expand, at the
 * six face neighbours (inside the padded brick, apron included) */
void og_scatter_density(OGrid* g, const void* posv, int64_t n, int stride, int off, const float trans[3],
                        float radius, int expand) {
    const char* pos = (const char*)posv;
    double* atl = g->chan[0].data;
    const int nb[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    const int res0 = g->res[0];
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        if (p[2] == NOHIT) continue;
        float w[3] = {p[0] + trans[0], p[1] + trans[1], p[2] + trans[2]};
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
        int32_t v[3] = {(int32_t)w[0], (int32_t)w[1], (int32_t)w[2]};
        int64_t leaf = get_leaf_at_voxel(g, v);
        if (leaf < 0) continue;
        const ONode* nd = &g->nodes[0][leaf];
        int64_t s = leaf_slot(g, nd);
        if (s < 0) continue;
        float lp[3] = {w[0] - (float)nd->pos[0], w[1] - (float)nd->pos[1], w[2] - (float)nd->pos[2]};
        int ix = (int)lp[0], iy = (int)lp[1], iz = (int)lp[2];
        if (lp[0] < 0 || lp[1] < 0 || lp[2] < 0 || ix >= res0 || iy >= res0 || iz >= res0) continue;
        for (int k = 0; k < (expand ? 7 : 1); k++) {
            int qx = ix + nb[k][0], qy = iy + nb[k][1], qz = iz + nb[k][2];
            float f = dist_func(lp[0], lp[1], lp[2], (float)qx, (float)qy, (float)qz, radius);
            atl[(size_t)s * 5832 + ((size_t)(qz + 1) * 18 + (qy + 1)) * 18 + (qx + 1)] += (double)f;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* The reference's CPU topology path: RebuildTopologyCPU -> ActivateSpace    */
/* (VG.cpp:1220-1227, 2766-2855, 2726-2763, 2707-2723, 2980-3027, 2915-2931, */
/* 2858-2875, 3079-3091; getPosFromBit / getBitPos VG.h:598-608).  Each      */
/* point activates the leaf that contains it, creating the nodes on the way  */
/* down; a point outside the root grows the tree upwards (Reparent).  Node    */
/* references are Elem(0, lev, index); a node's child list is taken from      */
/* pool 1 at its first child (InsertChild, no bitmasks) and filled with 0xFF. */
/* This is the host path the reference uses without a GPU topology pass; it   */
/* runs on an empty grid and is the CPU baseline timed beside the GPU path.   */

static int ref_lev(uint64_t e) { return (int)((e >> 8) & 0xFF); }
static size_t ref_ndx(uint64_t e) { return (size_t)(e >> 16); }
static ONode* cpu_node(OGrid* g, uint64_t id) { return &g->nodes[ref_lev(id)][ref_ndx(id)]; }

/* AllocateNode + SetupNode (VG.cpp:2506-2524): marker (mFlags) = true */
static uint64_t cpu_alloc(OGrid* g, int lev, const int32_t pos[3]) {
    pool_reserve(g, lev, g->ncnt[lev] + 1);
    size_t i = g->ncnt[lev]++;
    g->nused[lev]++;
    ONode* n = &g->nodes[lev][i];
    memset(n, 0, sizeof(ONode));
    n->lev = (uint8_t)lev;
    n->pos[0] = pos[0]; n->pos[1] = pos[1]; n->pos[2] = pos[2];
    n->childlist = UNDEFL;
    n->parent = UNDEFL;
    n->value[0] = n->value[1] = n->value[2] = -1;
    n->flags = 1;
    return Elem(0, lev, i);
}

/* GetCoveringNode (VG.cpp:2915-2931); levels past the configured ones have no
 * range here (the reference reads unset level dimensions): 0 = no cover */
static int cpu_cover(const OGrid* g, int lev, const int32_t pos[3], int32_t out[3]) {
    if (lev == OG_MAXLEV - 1) { out[0] = out[1] = out[2] = 0; return 1; }
    if (lev >= g->levs) return 0;
    int64_t rg = og_range(g, lev);
    for (int a = 0; a < 3; a++) {
        int64_t np = (int64_t)pos[a] / rg * rg; /* C truncation */
        if (pos[a] < np) np -= rg;
        out[a] = (int32_t)np;
    }
    return 1;
}

/* getPosInNode (VG.cpp:2858-2875) */
static int cpu_pos_in_node(const OGrid* g, const ONode* n, const int32_t pos[3], uint32_t* bit) {
    int lev = n->lev;
    int64_t rg = og_range(g, lev);
    int64_t r = og_res(g, lev);
    int64_t p[3];
    for (int a = 0; a < 3; a++) {
        p[a] = (int64_t)pos[a] - n->pos[a];
        if (p[a] < 0 || p[a] >= rg) { *bit = 0; return 0; }
    }
    for (int a = 0; a < 3; a++) p[a] = p[a] * r / rg;
    *bit = (uint32_t)((p[2] * r + p[1]) * r + p[0]);
    return 1;
}

/* getChildNode (VG.cpp:3079-3091) */
static uint64_t cpu_get_child(const OGrid* g, const ONode* n, uint32_t b) {
    if (n->childlist == UNDEFL) return UNDEF64;
    return g->clist[n->lev][ref_ndx(n->childlist) * og_cl_len(g, n->lev) + b];
}

/* InsertChild (VG.cpp:2980-3027), the child-list (non-bitmask) form */
static uint64_t cpu_insert_child(OGrid* g, uint64_t nodeid, uint64_t childid, uint32_t i) {
    cpu_node(g, childid)->parent = nodeid;
    ONode* cur = cpu_node(g, nodeid);
    int lev = cur->lev;
    size_t cl = og_cl_len(g, lev);
    if (cur->childlist == UNDEFL) {
        size_t k = g->cl_used[lev]++; /* PoolAlloc(1, lev): k < node count of the level */
        cur->childlist = Elem(1, lev, k);
        memset(g->clist[lev] + k * cl, 0xFF, cl * sizeof(uint64_t));
    }
    g->clist[lev][ref_ndx(cur->childlist) * cl + i] = childid;
    return childid;
}

/* AddChildNode (VG.cpp:2707-2723) with getPosFromBit (VG.h:602-608) */
static uint64_t cpu_add_child(OGrid* g, uint64_t nodeid, uint32_t b) {
    const ONode* par = cpu_node(g, nodeid);
    int plev = par->lev;
    int logr = g->log2dim[plev];
    uint32_t mask = (1u << logr) - 1u;
    int64_t crg = og_range(g, plev - 1);
    int32_t pos[3] = {(int32_t)(par->pos[0] + (int64_t)(b & mask) * crg),
                      (int32_t)(par->pos[1] + (int64_t)((b >> logr) & mask) * crg),
                      (int32_t)(par->pos[2] + (int64_t)((b >> (2 * logr)) & mask) * crg)};
    uint64_t child = cpu_alloc(g, plev - 1, pos);
    return cpu_insert_child(g, nodeid, child, b);
}

static uint64_t cpu_activate(OGrid* g, uint64_t nodeid, const int32_t pos[3], int* bnew, uint64_t stopnode,
                             int stoplev);

/* Reparent (VG.cpp:2726-2763) */
static uint64_t cpu_reparent(OGrid* g, int lev, uint64_t prevroot, const int32_t pos[3], int* bnew) {
    const ONode* pr = cpu_node(g, prevroot);
    int32_t prevpos[3] = {pr->pos[0], pr->pos[1], pr->pos[2]};
    int32_t p1[3] = {0, 0, 0}, p2[3];
    int cover = 0;
    while (!cover && lev < OG_MAXLEV) {
        lev++;
        if (!cpu_cover(g, lev, pos, p1) || !cpu_cover(g, lev, prevpos, p2)) { lev = OG_MAXLEV; break; }
        cover = p1[0] == p2[0] && p1[1] == p2[1] && p1[2] == p2[2];
    }
    if (lev >= OG_MAXLEV) return UNDEFL; /* level limit: the existing root stays */
    uint64_t newroot = cpu_alloc(g, lev, p1);
    int bn = 0;
    cpu_activate(g, newroot, prevpos, &bn, prevroot, 0); /* the stop node joins the old root */
    uint64_t leaf = cpu_activate(g, newroot, pos, bnew, UNDEFL, 0);
    g->cpu_root = newroot;
    if (leaf == UNDEFL) return UNDEFL;
    return cpu_node(g, leaf)->parent;
}

/* ActivateSpace(nodeid, pos, bNew, stopnode, stoplev) (VG.cpp:2795-2855) */
static uint64_t cpu_activate(OGrid* g, uint64_t nodeid, const int32_t pos[3], int* bnew, uint64_t stopnode,
                             int stoplev) {
    for (int guard = 0; guard < 4 * OG_MAXLEV; guard++) {
        if (g->cpu_root == UNDEFL && nodeid == g->cpu_root) { /* new root covering pos */
            int32_t p[3];
            if (!cpu_cover(g, stoplev, pos, p)) return UNDEFL;
            g->cpu_root = cpu_alloc(g, stoplev, p);
            nodeid = g->cpu_root;
        }
        const ONode* cur = cpu_node(g, nodeid);
        uint32_t b;
        if (cpu_pos_in_node(g, cur, pos, &b)) {
            const int lev = cur->lev;
            if (stopnode != UNDEFL) {
                const ONode* sn = cpu_node(g, stopnode);
                if (pos[0] == sn->pos[0] && pos[1] == sn->pos[1] && pos[2] == sn->pos[2] &&
                    cpu_get_child(g, cur, b) == UNDEF64 && lev == sn->lev + 1)
                    return cpu_insert_child(g, nodeid, stopnode, b);
            }
            if (lev == stoplev) return nodeid;
            uint64_t child;
            if (cpu_get_child(g, cur, b) == UNDEF64) {
                child = cpu_add_child(g, nodeid, b);
                if (lev == 1) *bnew = 1;
            } else {
                child = cpu_get_child(g, cur, b);
            }
            if (ref_lev(child) == 0) return child; /* isLeaf */
            nodeid = child;
        } else {
            uint64_t parent = cur->parent;
            if (parent == UNDEFL) {
                parent = cpu_reparent(g, cur->lev, nodeid, pos, bnew);
                if (parent == UNDEFL) return UNDEFL;
            }
            nodeid = parent;
        }
    }
    return UNDEFL;
}

/* RebuildTopologyCPU (VG.cpp:1220-1227): p = pos + orig, ActivateSpace(Vector3DF p),
 * whose Vector3DF -> Vector3DI conversion truncates each coordinate.  Returns the
 * number of points that reached a leaf. */
int64_t og_rebuild_topology_cpu(OGrid* g, const void* posv, int64_t n, int stride, int off, const float orig[3]) {
    const char* pos = (const char*)posv;
    int64_t ok = 0;
    for (int64_t i = 0; i < n; i++) {
        float p[3];
        load_point(pos, i, stride, off, p);
        float w[3] = {p[0] + orig[0], p[1] + orig[1], p[2] + orig[2]};
        int32_t v[3] = {(int32_t)w[0], (int32_t)w[1], (int32_t)w[2]};
        int bnew = 0;
        if (cpu_activate(g, g->cpu_root, v, &bnew, UNDEFL, 0) != UNDEFL) ok++;
    }
    return ok;
}
/* level of the CPU path's root (-1 when empty) */
int og_cpu_root_level(const OGrid* g) { return g->cpu_root == UNDEFL ? -1 : ref_lev(g->cpu_root); }

