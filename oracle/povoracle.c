/*
 * povoracle.c -- FP64 CPU restatement of the reference per-pixel trace path.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the checker of libpovgpu and the
 * source of the "port" CPU baseline.  The product (libpovgpu.so) never
 * links, loads or calls it.
 *
 * Every function names the reference code it restates (paths relative to
 * the reference source tree).  Arithmetic types follow the reference:
 * geometry in double, bounding boxes in float (BBoxScalar = SNGL,
 * source/core/bounding/boundingbox.h:83), colours in float (COLC).
 *
 * Parity is pinned against the reference itself: tests/golden/ holds
 * per-ray hits and per-pixel colours dumped by oracle/refbuild/pov_oracle
 * (the reference sources compiled unmodified) for the same SDL scenes.
 *
 * Documented simplifications (none changes a result on non-grazing rays):
 *   - the light-source shadow cache of TracePointLightShadowRay
 *     (source/core/render/trace.cpp:1990-2025) is not restated: which
 *     object it holds depends on render order, and its test of that object
 *     accepts hits in [MIN_ISECT_DEPTH, depth) (trace.cpp:1999,346-390)
 *     where the full test needs (SHADOW_TOLERANCE, depth - SHADOW_TOLERANCE).
 *     It changes Shadow_Cache_Hits, and the verdict of a shadow ray that
 *     passes within SHADOW_TOLERANCE of another surface (a few area-light
 *     samples per ten thousand in the golden scenes).
 *   - the mesh best-first loop's early "Depth > Best" exit uses the best
 *     hit so far (source/core/shape/mesh.cpp:1499 keeps the last one).
 */
#include "povoracle.h"
#include "../povray_gb300/csrc/povgpu_noise_table.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* source/core/configcore.h:153-206, source/core/render/trace.cpp:81 */
#define EPSILON          1.0e-10
#define BOUND_HUGE       2.0e+10
#define SMALL_TOLERANCE  0.001
#define MAX_DISTANCE     1.0e7
#define MIN_ISECT_DEPTH  1.0e-4
#define SHADOW_TOLERANCE 1.0e-3
#define AREA_MAX_POINTS  4096   /* largest area-light grid the oracle restates */
/* per-shape DEPTH_TOLERANCE: sphere.cpp:63, plane.cpp:62, mesh.cpp:92 */
#define SPHERE_DEPTH_TOLERANCE 1.0e-6
#define PLANE_DEPTH_TOLERANCE  1.0e-6
#define MESH_DEPTH_TOLERANCE   1.0e-6
#define BUNCHING_FACTOR 4                 /* boundingbox.cpp:68 */

typedef struct { double x, y, z; } V3;

static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vmul(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 vdiv(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 vcross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double vlen(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline V3 vnorm(V3 a) { double l = vlen(a); return l != 0 ? vdiv(a, l) : a; }
static inline double vget(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline V3 vload(const double* p) { return v3(p[0], p[1], p[2]); }

typedef struct { float r, g, b; } RGB;

/* BoundingBox: lowerLeft + size in float (boundingbox.h:90-95). */
typedef struct { float ll[3]; float sz[3]; } BBox;

static BBox bbox_from_min_max(V3 mn, V3 mx)   /* Make_BBox_from_min_max, boundingbox.h:125 */
{
    BBox b;
    b.ll[0] = (float)mn.x; b.ll[1] = (float)mn.y; b.ll[2] = (float)mn.z;
    b.sz[0] = (float)(mx.x - mn.x); b.sz[1] = (float)(mx.y - mn.y); b.sz[2] = (float)(mx.z - mn.z);
    return b;
}

/* ------------------------------------------------------------- trees --- */
/* BBOX_TREE (boundingbox.h:98-104): composite nodes list children, leaves
 * hold one item (an object or a mesh triangle). */
typedef struct {
    BBox    bbox;
    int32_t infinite;
    int32_t entries;   /* 0 = leaf */
    int32_t first;     /* composite: index into kids[]; leaf: item id */
} TNode;

typedef struct {
    TNode*   nodes;
    int32_t  num_nodes, cap_nodes;
    int32_t* kids;
    int32_t  num_kids, cap_kids;
    int32_t  root;     /* -1 = no tree */
} Tree;

static int tree_add(Tree* t, TNode n)
{
    if (t->num_nodes == t->cap_nodes) {
        t->cap_nodes = t->cap_nodes ? t->cap_nodes * 2 : 64;
        t->nodes = (TNode*)realloc(t->nodes, sizeof(TNode) * t->cap_nodes);
    }
    t->nodes[t->num_nodes] = n;
    return t->num_nodes++;
}

static int tree_kids(Tree* t, int n)
{
    if (t->num_kids + n > t->cap_kids) {
        while (t->num_kids + n > t->cap_kids)
            t->cap_kids = t->cap_kids ? t->cap_kids * 2 : 256;
        t->kids = (int32_t*)realloc(t->kids, sizeof(int32_t) * t->cap_kids);
    }
    int at = t->num_kids;
    t->num_kids += n;
    return at;
}

/* compboxes<Axis> (boundingbox.cpp:~670): key 2*lowerLeft + size. */
static const Tree* g_sort_tree;
static int g_sort_axis;
static int compboxes(const void* a, const void* b)
{
    const BBox* ba = &g_sort_tree->nodes[*(const int32_t*)a].bbox;
    const BBox* bb = &g_sort_tree->nodes[*(const int32_t*)b].bbox;
    float am = (float)(2.0 * ba->ll[g_sort_axis] + ba->sz[g_sort_axis]);
    float bm = (float)(2.0 * bb->ll[g_sort_axis] + bb->sz[g_sort_axis]);
    if (am < bm) return -1;
    return am == bm ? 0 : 1;
}

/* find_axis (boundingbox.cpp:~690): axis of largest extent, float. */
static int find_axis(const Tree* t, const int32_t* fin, ptrdiff_t first, ptrdiff_t last)
{
    float mins[3] = {(float)BOUND_HUGE, (float)BOUND_HUGE, (float)BOUND_HUGE};
    float maxs[3] = {(float)-BOUND_HUGE, (float)-BOUND_HUGE, (float)-BOUND_HUGE};
    for (ptrdiff_t i = first; i < last; i++) {
        const BBox* b = &t->nodes[fin[i]].bbox;
        for (int k = 0; k < 3; k++) {
            if (b->ll[k] < mins[k]) mins[k] = b->ll[k];
            if (b->ll[k] + b->sz[k] > maxs[k]) maxs[k] = b->ll[k] + b->sz[k];
        }
    }
    int which = 0;
    float d = (float)-BOUND_HUGE, e;
    e = maxs[0] - mins[0]; if (e > d) { d = e; which = 0; }
    e = maxs[1] - mins[1]; if (e > d) { d = e; which = 1; }
    e = maxs[2] - mins[2]; if (e > d) which = 2;
    return which;
}

/* calc_bbox (boundingbox.cpp:~730): double min/max of float boxes. */
static BBox calc_bbox(const Tree* t, const int32_t* fin, ptrdiff_t first, ptrdiff_t last)
{
    V3 mn = v3(BOUND_HUGE, BOUND_HUGE, BOUND_HUGE), mx = v3(-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE);
    for (ptrdiff_t i = first; i < last; i++) {
        const BBox* b = &t->nodes[fin[i]].bbox;
        double lo, hi;
        lo = b->ll[0]; hi = lo + b->sz[0]; if (lo < mn.x) mn.x = lo; if (hi > mx.x) mx.x = hi;
        lo = b->ll[1]; hi = lo + b->sz[1]; if (lo < mn.y) mn.y = lo; if (hi > mx.y) mx.y = hi;
        lo = b->ll[2]; hi = lo + b->sz[2]; if (lo < mn.z) mn.z = lo; if (hi > mx.z) mx.z = hi;
    }
    return bbox_from_min_max(mn, mx);
}

/* build_area_table (boundingbox.cpp:~760), float. */
static void build_area_table(const Tree* t, const int32_t* fin, ptrdiff_t a, ptrdiff_t b, float* areas)
{
    ptrdiff_t imin, dir;
    if (a < b) { imin = a; dir = 1; } else { imin = b; dir = -1; }
    float bmin[3] = {(float)BOUND_HUGE, (float)BOUND_HUGE, (float)BOUND_HUGE};
    float bmax[3] = {(float)-BOUND_HUGE, (float)-BOUND_HUGE, (float)-BOUND_HUGE};
    for (ptrdiff_t i = a; i != (b + dir); i += dir) {
        const BBox* bb = &t->nodes[fin[i]].bbox;
        for (int k = 0; k < 3; k++) {
            float tmin = bb->ll[k], tmax = tmin + bb->sz[k];
            if (tmin < bmin[k]) bmin[k] = tmin;
            if (tmax > bmax[k]) bmax[k] = tmax;
        }
        float len[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
        areas[i - imin] = len[0] * (len[1] + len[2]) + len[1] * len[2];
    }
}

typedef struct {
    Tree*    t;
    int32_t* fin;
    size_t   n, cap;
    float*   area;
    size_t   area_cap;
    int32_t  root;
} Builder;

/* sort_and_split (boundingbox.cpp:834-928). */
static int sort_and_split(Builder* B, ptrdiff_t first, ptrdiff_t last)
{
    ptrdiff_t size = last - first, best_loc = -1;
    if (size <= 0)
        return 0;
    if (size > BUNCHING_FACTOR) {
        int axis = find_axis(B->t, B->fin, first, last);
        g_sort_tree = B->t;
        g_sort_axis = axis;
        qsort(B->fin + first, (size_t)size, sizeof(int32_t), compboxes);
        if ((size_t)(2 * size) > B->area_cap) {
            B->area_cap = 2 * size;
            B->area = (float*)realloc(B->area, sizeof(float) * B->area_cap);
        }
        float* area_left = B->area;
        float* area_right = area_left + size;
        build_area_table(B->t, B->fin, first, last - 1, area_left);
        build_area_table(B->t, B->fin, last - 1, first, area_right);
        float best_index = area_right[0] * (float)(size - 3);
        for (ptrdiff_t i = 1; i < size; i++) {
            float new_index = (float)i * area_left[i - 1] + (float)(size - i) * area_right[i];
            if (new_index < best_index) {
                best_index = new_index;
                best_loc = i + first;
            }
        }
    }
    if (best_loc < 0) {
        TNode cd;
        memset(&cd, 0, sizeof(cd));
        cd.entries = (int32_t)size;
        cd.first = tree_kids(B->t, (int)size);
        for (ptrdiff_t i = 0; i < size; i++)
            B->t->kids[cd.first + i] = B->fin[first + i];
        cd.bbox = calc_bbox(B->t, B->fin, first, last);
        int id = tree_add(B->t, cd);
        B->root = id;
        if (B->n >= B->cap) {
            B->cap = B->cap + B->cap / 2 + 16;
            B->fin = (int32_t*)realloc(B->fin, sizeof(int32_t) * B->cap);
        }
        B->fin[B->n++] = id;
        return 0;
    }
    sort_and_split(B, first, best_loc);
    sort_and_split(B, best_loc, last);
    return 1;
}

/* Build_BBox_Tree (boundingbox.cpp:262-323).  `finite` lists leaf node ids
 * (consumed), `infinite` the leaf ids of unbounded objects. */
static void build_bbox_tree(Tree* t, int32_t* finite, size_t nfinite, const int32_t* infinite, size_t ninfinite)
{
    t->root = -1;
    if (nfinite > 0) {
        Builder B;
        memset(&B, 0, sizeof(B));
        B.t = t;
        B.cap = 2 * nfinite + 16;
        B.fin = (int32_t*)malloc(sizeof(int32_t) * B.cap);
        memcpy(B.fin, finite, sizeof(int32_t) * nfinite);
        B.n = nfinite;
        ptrdiff_t low = 0, high = (ptrdiff_t)nfinite;
        while (sort_and_split(&B, low, high)) {
            low = high;
            high = (ptrdiff_t)B.n;
        }
        t->root = B.root;
        free(B.fin);
        free(B.area);
        if (ninfinite > 0) {
            /* infinite objects go into a new first child of the root */
            TNode cd;
            memset(&cd, 0, sizeof(cd));
            cd.entries = (int32_t)ninfinite;
            cd.first = tree_kids(t, (int)ninfinite);
            for (size_t i = 0; i < ninfinite; i++)
                t->kids[cd.first + i] = infinite[i];
            cd.bbox = calc_bbox(t, t->kids, cd.first, cd.first + (ptrdiff_t)ninfinite);
            cd.infinite = 1;
            int cid = tree_add(t, cd);
            TNode* root = &t->nodes[t->root];
            int old_first = root->first, old_n = root->entries;
            int nf = tree_kids(t, old_n + 1);
            root = &t->nodes[t->root];
            t->kids[nf] = cid;
            for (int i = 0; i < old_n; i++)
                t->kids[nf + 1 + i] = t->kids[old_first + i];
            root->first = nf;
            root->entries = old_n + 1;
            root->bbox = calc_bbox(t, t->kids, nf, nf + old_n + 1);
            root->infinite = 1;
        }
    } else if (ninfinite > 0) {
        TNode cd;
        memset(&cd, 0, sizeof(cd));
        cd.entries = (int32_t)ninfinite;
        cd.first = tree_kids(t, (int)ninfinite);
        for (size_t i = 0; i < ninfinite; i++)
            t->kids[cd.first + i] = infinite[i];
        cd.bbox = calc_bbox(t, t->kids, cd.first, cd.first + (ptrdiff_t)ninfinite);
        cd.infinite = 1;
        t->root = tree_add(t, cd);
    }
}

/* BBoxPriorityQueue (boundingbox.cpp:74-140): 1-based binary min-heap. */
typedef struct { double depth; int32_t node; } QElem;
typedef struct { QElem* q; size_t size, cap; } PQueue;

static void pq_clear(PQueue* p) { p->size = 0; }
static void pq_insert(PQueue* p, double depth, int32_t node)
{
    if (p->size + 2 > p->cap) {
        p->cap = p->cap ? p->cap * 2 : 256;
        p->q = (QElem*)realloc(p->q, sizeof(QElem) * p->cap);
    }
    size_t i = ++p->size;
    while (i > 1 && depth < p->q[i / 2].depth) {
        p->q[i] = p->q[i / 2];
        i /= 2;
    }
    p->q[i].depth = depth;
    p->q[i].node = node;
}
static int pq_remove_min(PQueue* p, double* depth, int32_t* node)
{
    size_t size = p->size;
    if (size == 0)
        return 0;
    *depth = p->q[1].depth;
    *node = p->q[1].node;
    QElem last = p->q[size];
    p->size = --size;
    size_t i = 1, j;
    while (i <= size / 2) {
        j = 2 * i;
        if (j < size && p->q[j + 1].depth < p->q[j].depth)
            j++;
        if (last.depth <= p->q[j].depth)
            break;
        p->q[i] = p->q[j];
        i = j;
    }
    if (size > 0)
        p->q[i] = last;
    return 1;
}

/* Rayinfo (boundingbox.h:182-216): float origin and inverse direction. */
typedef struct { float origin[3]; float invdir[3]; int nonzero[3]; int positive[3]; } RayInfo;

static void rayinfo_init(RayInfo* ri, V3 o, V3 d)
{
    double dd[3] = {d.x, d.y, d.z};
    ri->origin[0] = (float)o.x; ri->origin[1] = (float)o.y; ri->origin[2] = (float)o.z;
    for (int k = 0; k < 3; k++) {
        ri->nonzero[k] = dd[k] != 0.0;
        ri->invdir[k] = 0.0f;
        ri->positive[k] = 0;
        if (ri->nonzero[k]) {
            ri->invdir[k] = (float)(1.0 / dd[k]);
            ri->positive[k] = dd[k] > 0.0;
        }
    }
}

/* Check_And_Enqueue (boundingbox.cpp:541-648); slab arithmetic is float
 * because every operand is a BBoxScalar. */
static void check_and_enqueue(PQueue* q, const TNode* n, int32_t id, const RayInfo* ri, uint64_t* boxes)
{
    double dmin, dmax;
    if (!n->infinite) {
        if (boxes) (*boxes)++;
        dmin = -BOUND_HUGE;
        dmax = BOUND_HUGE;
        for (int dim = 0; dim < 3; dim++) {
            if (ri->nonzero[dim]) {
                double tmin, tmax;
                if (ri->positive[dim]) {
                    tmax = (float)((n->bbox.ll[dim] + n->bbox.sz[dim] - ri->origin[dim]) * ri->invdir[dim]);
                    if (tmax < EPSILON) return;
                    tmin = (float)((n->bbox.ll[dim] - ri->origin[dim]) * ri->invdir[dim]);
                } else {
                    tmax = (float)((n->bbox.ll[dim] - ri->origin[dim]) * ri->invdir[dim]);
                    if (tmax < EPSILON) return;
                    tmin = (float)((n->bbox.ll[dim] + n->bbox.sz[dim] - ri->origin[dim]) * ri->invdir[dim]);
                }
                if (tmax < dmax) {
                    if (tmin > dmin) {
                        if (tmin > tmax) return;
                        dmin = tmin;
                    } else {
                        if (dmin > tmax) return;
                    }
                    dmax = tmax;
                } else {
                    if (tmin > dmin) {
                        if (tmin > dmax) return;
                        dmin = tmin;
                    }
                }
            } else {
                float lo = n->bbox.ll[dim], hi = n->bbox.ll[dim] + n->bbox.sz[dim];
                if (ri->origin[dim] < lo || ri->origin[dim] > hi)
                    return;
            }
        }
    } else {
        dmin = -MAX_DISTANCE;
    }
    pq_insert(q, dmin, id);
}

/* Intersect_BBox_Dir (object.cpp:1075-1109): per-object box pre-test. */
static int intersect_bbox_dir(const BBox* b, V3 o, V3 d, float maxd)
{
    float origin[3] = {(float)o.x, (float)o.y, (float)o.z};
    float invdir[3] = {(float)(1.0 / d.x), (float)(1.0 / d.y), (float)(1.0 / d.z)};
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) { lo[k] = b->ll[k]; hi[k] = b->ll[k] + b->sz[k]; }
    int bx = invdir[0] < 0.0f, by = invdir[1] < 0.0f, bz = invdir[2] < 0.0f;
    float tmin = ((bx ? hi[0] : lo[0]) - origin[0]) * invdir[0];
    float tmax = ((bx ? lo[0] : hi[0]) - origin[0]) * invdir[0];
    float tymin = ((by ? hi[1] : lo[1]) - origin[1]) * invdir[1];
    float tymax = ((by ? lo[1] : hi[1]) - origin[1]) * invdir[1];
    if (tmin > tymax || tymin > tmax) return 0;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = ((bz ? hi[2] : lo[2]) - origin[2]) * invdir[2];
    float tzmax = ((bz ? lo[2] : hi[2]) - origin[2]) * invdir[2];
    if (tmin > tzmax || tzmin > tmax) return 0;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    return (tmin < maxd) && (tmax > (float)MIN_ISECT_DEPTH);
}

/* ------------------------------------------------------------- scene --- */
/* MESH_TRIANGLE (source/core/shape/mesh.h:83-119), after
 * Compute_Mesh_Triangle (mesh.cpp:838-982). */
typedef struct {
    int32_t p1, p2, p3;     /* vertex indices after the orientation swap */
    int32_t n1, n2, n3;     /* smooth normal indices */
    float   normal[3];      /* geometric normal (Normals[Normal_Ind]) */
    float   distance;
    float   perp[3];
    int32_t dominant_axis, v_axis, smooth;
} MeshTri;

typedef struct {
    float*   verts;         /* 3 per vertex */
    float*   normals;       /* 3 per normal (parser-normalised) */
    MeshTri* tris;
    int32_t  ntris;
    Tree     tree;
    PQueue   scratch_unused;
} OMesh;

typedef struct {
    PovGpuObject   o;
    BBox           bbox;
    const PovGpuMaterial* mat;
} OObj;

struct PovOracle {
    PovGpuSceneDesc desc;
    OObj*    objs;
    int32_t  nobjs;
    PovGpuMaterial* mats;
    PovGpuLight*    lights;
    int32_t  nlights;
    OMesh*   meshes;
    int32_t  nmeshes;
    Tree     top;            /* leaf item = object index */
    int32_t  top_linear;     /* no slabs: linear scan (trace.cpp:263) */
    struct RadCache* rad;    /* radiosity sample cache (mutable during a render) */
    int32_t  gt_count[8];    /* converged mode: directions per query and depth (0 = off) */
    /* interiors: one id per object (CSG children share their parent's),
     * the interiors' parameters, the atmosphere's IOR; transparent = some
     * surface filters or transmits (outside media containers) */
    int32_t* obj_int;
    PovGpuInterior* ints;
    int32_t  nints;
    double   atm_ior;
    int      transparent;
};

static int max3_coordinate(double x, double y, double z)  /* mathutil */
{
    if (x > y) return x > z ? 0 : 2;
    return y > z ? 1 : 2;
}

/* Compute_Mesh_Triangle + compute_smooth_triangle (mesh.cpp:838-1000). */
static void compute_mesh_triangle(MeshTri* T, const float* verts, int smooth)
{
    V3 P1 = v3(verts[3 * T->p1], verts[3 * T->p1 + 1], verts[3 * T->p1 + 2]);
    V3 P2 = v3(verts[3 * T->p2], verts[3 * T->p2 + 1], verts[3 * T->p2 + 2]);
    V3 P3 = v3(verts[3 * T->p3], verts[3 * T->p3 + 1], verts[3 * T->p3 + 2]);
    V3 V1 = vsub(P2, P1), V2 = vsub(P3, P1);
    V3 N = vcross(V2, V1);
    double len = vlen(N);
    T->smooth = 0;
    if (len == 0.0) {
        /* degenerate: normal stays zero, never hit (mesh.cpp:852) */
        T->normal[0] = T->normal[1] = T->normal[2] = 0.0f;
        T->distance = 0.0f;
        T->dominant_axis = 0;
        T->v_axis = 0;
        T->perp[0] = T->perp[1] = T->perp[2] = 0.0f;
        return;
    }
    N = vdiv(N, len);
    double dist = -vdot(N, P1);
    T->distance = (float)dist;
    T->normal[0] = (float)N.x; T->normal[1] = (float)N.y; T->normal[2] = (float)N.z;
    int axis = max3_coordinate(fabs(N.x), fabs(N.y), fabs(N.z));
    T->dominant_axis = axis;
    int swap = 0;
    switch (axis) {
    case 0: swap = (P2.y - P3.y) * (P2.z - P1.z) < (P2.z - P3.z) * (P2.y - P1.y); break;
    case 1: swap = (P2.x - P3.x) * (P2.z - P1.z) < (P2.z - P3.z) * (P2.x - P1.x); break;
    default: swap = (P2.x - P3.x) * (P2.y - P1.y) < (P2.y - P3.y) * (P2.x - P1.x); break;
    }
    V3 pP1 = P1, pP2 = P2;
    if (swap) {
        int32_t t = T->p2; T->p2 = T->p1; T->p1 = t;
        pP1 = P2; pP2 = P1;
        if (smooth) { t = T->n2; T->n2 = T->n1; T->n1 = t; }
    }
    if (smooth)
        T->smooth = 1;
    /* compute_smooth_triangle(Triangle, *pP1, *pP2, P3) */
    V3 P3MinusP2 = vsub(P3, pP2);
    T->v_axis = max3_coordinate(fabs(P3MinusP2.x), fabs(P3MinusP2.y), fabs(P3MinusP2.z));
    V3 VTemp1 = vnorm(vsub(pP2, P3));
    V3 VTemp2 = vsub(pP1, P3);
    double proj = vdot(VTemp2, VTemp1);
    VTemp1 = vmul(VTemp1, proj);
    V3 perp = vnorm(vsub(VTemp1, VTemp2));
    float pf[3] = {(float)perp.x, (float)perp.y, (float)perp.z};
    double uden = -vdot(VTemp2, v3(pf[0], pf[1], pf[2]));
    T->perp[0] = (float)(pf[0] / uden);
    T->perp[1] = (float)(pf[1] / uden);
    T->perp[2] = (float)(pf[2] / uden);
}

/* ---------------------------------------------------------- shapes --- */
typedef struct {
    double  depth;
    V3      ipoint;
    int32_t object;
    int32_t triangle;   /* mesh triangle, or box side (Intersection::i1) */
} Isect;

/* TRANSFORM application (source/core/math/matrix.cpp:415-507); m is a
 * row-major 4x4, row-vector convention. */
static V3 mtrans_point(const double* m, V3 v)
{
    return v3(v.x * m[0] + v.y * m[4] + v.z * m[8] + m[12], v.x * m[1] + v.y * m[5] + v.z * m[9] + m[13],
              v.x * m[2] + v.y * m[6] + v.z * m[10] + m[14]);
}
static V3 mtrans_direction(const double* m, V3 v)
{
    return v3(v.x * m[0] + v.y * m[4] + v.z * m[8], v.x * m[1] + v.y * m[5] + v.z * m[9],
              v.x * m[2] + v.y * m[6] + v.z * m[10]);
}
/* MTransNormal(r, v, T) = MInvTransNormal(r, v, &T->inverse) */
static V3 mtrans_normal(const double* inv, V3 v)
{
    return v3(v.x * inv[0] + v.y * inv[1] + v.z * inv[2], v.x * inv[4] + v.y * inv[5] + v.z * inv[6],
              v.x * inv[8] + v.y * inv[9] + v.z * inv[10]);
}

/* Box::Intersect (source/core/shape/box.cpp:172-533) */
#define BOX_DEPTH_TOLERANCE 1.0e-6
#define CLOSE_TOLERANCE 1.0e-6
enum { SIDE_X0 = 0, SIDE_X1, SIDE_Y0, SIDE_Y1, SIDE_Z0, SIDE_Z1 };
static int box_intersect(V3 P, V3 D, V3 c1, V3 c2, double* d1, double* d2, int* s1, int* s2)
{
    int smin = 0, smax = 0;
    double t, tmin = 0.0, tmax = BOUND_HUGE;
    if (D.x < -EPSILON) {
        t = (c1.x - P.x) / D.x;
        if (t < tmin) return 0;
        if (t <= tmax) { smax = SIDE_X0; tmax = t; }
        t = (c2.x - P.x) / D.x;
        if (t >= tmin) { if (t > tmax) return 0; smin = SIDE_X1; tmin = t; }
    } else if (D.x > EPSILON) {
        t = (c2.x - P.x) / D.x;
        if (t < tmin) return 0;
        if (t <= tmax) { smax = SIDE_X1; tmax = t; }
        t = (c1.x - P.x) / D.x;
        if (t >= tmin) { if (t > tmax) return 0; smin = SIDE_X0; tmin = t; }
    } else if (P.x < c1.x || P.x > c2.x) {
        return 0;
    }
    if (D.y < -EPSILON) {
        t = (c1.y - P.y) / D.y;
        if (t < tmin) return 0;
        if (t <= tmax - CLOSE_TOLERANCE) { smax = SIDE_Y0; tmax = t; }
        else if (t <= tmax + CLOSE_TOLERANCE) { if (-D.y > fabs(D.x)) smax = SIDE_Y0; }
        t = (c2.y - P.y) / D.y;
        if (t >= tmin + CLOSE_TOLERANCE) { if (t > tmax) return 0; smin = SIDE_Y1; tmin = t; }
        else if (t >= tmin - CLOSE_TOLERANCE) { if (-D.y > fabs(D.x)) smin = SIDE_Y1; }
    } else if (D.y > EPSILON) {
        t = (c2.y - P.y) / D.y;
        if (t < tmin) return 0;
        if (t <= tmax - CLOSE_TOLERANCE) { smax = SIDE_Y1; tmax = t; }
        else if (t <= tmax + CLOSE_TOLERANCE) { if (D.y > fabs(D.x)) smax = SIDE_Y1; }
        t = (c1.y - P.y) / D.y;
        if (t >= tmin + CLOSE_TOLERANCE) { if (t > tmax) return 0; smin = SIDE_Y0; tmin = t; }
        else if (t >= tmin - CLOSE_TOLERANCE) { if (D.y > fabs(D.x)) smin = SIDE_Y0; }
    } else if (P.y < c1.y || P.y > c2.y) {
        return 0;
    }
    if (D.z < -EPSILON) {
        t = (c1.z - P.z) / D.z;
        if (t < tmin) return 0;
        if (t <= tmax - CLOSE_TOLERANCE) { smax = SIDE_Z0; tmax = t; }
        else if (t <= tmax + CLOSE_TOLERANCE) {
            if ((smax == SIDE_X0 || smax == SIDE_X1) && -D.z > fabs(D.x)) smax = SIDE_Z0;
            else if ((smax == SIDE_Y0 || smax == SIDE_Y1) && -D.z > fabs(D.y)) smax = SIDE_Z0;
        }
        t = (c2.z - P.z) / D.z;
        if (t >= tmin + CLOSE_TOLERANCE) { if (t > tmax) return 0; smin = SIDE_Z1; tmin = t; }
        else if (t >= tmin - CLOSE_TOLERANCE) {
            if ((smin == SIDE_X0 || smin == SIDE_X1) && -D.z > fabs(D.x)) smin = SIDE_Z1;
            else if ((smin == SIDE_Y0 || smin == SIDE_Y1) && -D.z > fabs(D.y)) smin = SIDE_Z1;
        }
    } else if (D.z > EPSILON) {
        t = (c2.z - P.z) / D.z;
        if (t < tmin) return 0;
        if (t <= tmax - CLOSE_TOLERANCE) { smax = SIDE_Z1; tmax = t; }
        else if (t <= tmax + CLOSE_TOLERANCE) {
            if ((smax == SIDE_X0 || smax == SIDE_X1) && D.z > fabs(D.x)) smax = SIDE_Z1;
            else if ((smax == SIDE_Y0 || smax == SIDE_Y1) && D.z > fabs(D.y)) smax = SIDE_Z1;
        }
        t = (c1.z - P.z) / D.z;
        if (t >= tmin + CLOSE_TOLERANCE) { if (t > tmax) return 0; smin = SIDE_Z0; tmin = t; }
        else if (t >= tmin - CLOSE_TOLERANCE) {
            if ((smin == SIDE_X0 || smin == SIDE_X1) && D.z > fabs(D.x)) smin = SIDE_Z0;
            else if ((smin == SIDE_Y0 || smin == SIDE_Y1) && D.z > fabs(D.y)) smin = SIDE_Z0;
        }
    } else if (P.z < c1.z || P.z > c2.z) {
        return 0;
    }
    if (tmax < BOX_DEPTH_TOLERANCE)
        return 0;
    *d1 = tmin; *d2 = tmax; *s1 = smin; *s2 = smax;
    return 1;
}

/* ------------------------------------------ polynomial solver (FP64) --- */
/* source/core/math/polynomialsolver.cpp: Solve_Polynomial (:1585),
 * solve_quadratic (:810), solve_cubic (:903), difficult_coeffs (:1075),
 * solve_quartic (:1325), Sturm sequence polysolve (:1481) with buildsturm,
 * modp, numchanges, sbisect, regula_falsa, visible_roots, polyeval. */
#define PS_MAX_ORDER 15
#define PS_MAX_ITERATIONS 50
#define PS_SMALL_ENOUGH 1.0e-10
#define PS_RELERROR 1.0e-12
#define PS_FUDGE1 1.0e12
static const double TWO_M_PI_3 = 2.0943951023931954923084;
static const double FOUR_M_PI_3 = 4.1887902047863909846168;

typedef struct { int ord; double coef[PS_MAX_ORDER + 1]; } Poly;

static int ps_modp(const Poly* u, const Poly* v, Poly* r)
{
    int k, j;
    *r = *u;
    if (v->coef[v->ord] < 0.0) {
        for (k = u->ord - v->ord - 1; k >= 0; k -= 2)
            r->coef[k] = -r->coef[k];
        for (k = u->ord - v->ord; k >= 0; k--)
            for (j = v->ord + k - 1; j >= k; j--)
                r->coef[j] = -r->coef[j] - r->coef[v->ord + k] * v->coef[j - k];
    } else {
        for (k = u->ord - v->ord; k >= 0; k--)
            for (j = v->ord + k - 1; j >= k; j--)
                r->coef[j] -= r->coef[v->ord + k] * v->coef[j - k];
    }
    k = v->ord - 1;
    while (k >= 0 && fabs(r->coef[k]) < PS_SMALL_ENOUGH) {
        r->coef[k] = 0.0;
        k--;
    }
    r->ord = (k < 0) ? 0 : k;
    return r->ord;
}

static int ps_buildsturm(int ord, Poly* sseq)
{
    sseq[0].ord = ord;
    sseq[1].ord = ord - 1;
    double f = fabs(sseq[0].coef[ord] * ord);
    for (int i = 1; i <= ord; i++)
        sseq[1].coef[i - 1] = sseq[0].coef[i] * i / f;
    Poly* sp;
    for (sp = sseq + 2; ps_modp(sp - 2, sp - 1, sp); sp++) {
        f = -fabs(sp->coef[sp->ord]);
        for (int k = sp->ord; k >= 0; k--)
            sp->coef[k] /= f;
    }
    sp->coef[0] = -sp->coef[0];
    return (int)(sp - sseq);
}

static int ps_visible_roots(int np, const Poly* sseq)
{
    int atposinf = 0, atzero = 0;
    double f, lf = sseq[0].coef[sseq[0].ord];
    for (const Poly* s = sseq + 1; s <= sseq + np; s++) {
        f = s->coef[s->ord];
        if (lf == 0.0 || lf * f < 0) atposinf++;
        lf = f;
    }
    lf = sseq[0].coef[0];
    for (const Poly* s = sseq + 1; s <= sseq + np; s++) {
        f = s->coef[0];
        if (lf == 0.0 || lf * f < 0) atzero++;
        lf = f;
    }
    return atzero - atposinf;
}

static double ps_polyeval(double x, int n, const double* c)
{
    double val = c[n];
    for (int i = n - 1; i >= 0; i--)
        val = val * x + c[i];
    return val;
}

static int ps_numchanges(int np, const Poly* sseq, double a)
{
    int changes = 0;
    double f, lf = ps_polyeval(a, sseq[0].ord, sseq[0].coef);
    for (const Poly* s = sseq + 1; s <= sseq + np; s++) {
        f = ps_polyeval(a, s->ord, s->coef);
        if (lf == 0.0 || lf * f < 0) changes++;
        lf = f;
    }
    return changes;
}

static int ps_regula_falsa(int order, const double* coef, double a, double b, double* val)
{
    double fa = ps_polyeval(a, order, coef), fb = ps_polyeval(b, order, coef), x = 0, fx, lfx;
    if (fa * fb > 0.0) return 0;
    if (fabs(fa) < PS_SMALL_ENOUGH) { *val = a; return 1; }
    if (fabs(fb) < PS_SMALL_ENOUGH) { *val = b; return 1; }
    lfx = fa;
    for (int its = 0; its < PS_MAX_ITERATIONS; its++) {
        x = (fb * a - fa * b) / (fb - fa);
        fx = ps_polyeval(x, order, coef);
        if (fabs(x) > PS_RELERROR) {
            if (fabs(fx / x) < PS_RELERROR) { *val = x; return 1; }
        } else if (fabs(fx) < PS_RELERROR) {
            *val = x;
            return 1;
        }
        if (fa < 0) {
            if (fx < 0) { a = x; fa = fx; if ((lfx * fx) > 0) fb /= 2; }
            else { b = x; fb = fx; if ((lfx * fx) > 0) fa /= 2; }
        } else {
            if (fx < 0) { b = x; fb = fx; if ((lfx * fx) > 0) fa /= 2; }
            else { a = x; fa = fx; if ((lfx * fx) > 0) fb /= 2; }
        }
        if (fabs(b - a) < PS_RELERROR) { *val = x; return 1; }
        lfx = fx;
    }
    return 0;
}

static int ps_sbisect(int np, const Poly* sseq, double mn, double mx, int atmin, int atmax, double* roots)
{
    double mid = 0.0;
    int n1, n2, its, atmid;
    if ((atmin - atmax) == 1) {
        if (ps_regula_falsa(sseq->ord, sseq->coef, mn, mx, roots))
            return 1;
        for (its = 0; its < PS_MAX_ITERATIONS; its++) {
            mid = (mn + mx) / 2;
            atmid = ps_numchanges(np, sseq, mid);
            if ((atmid < atmax) || (atmid > atmin)) return 0;
            if (fabs(mid) > PS_RELERROR) {
                if (fabs((mx - mn) / mid) < PS_RELERROR) { roots[0] = mid; return 1; }
            } else if (fabs(mx - mn) < PS_RELERROR) {
                roots[0] = mid;
                return 1;
            }
            if ((atmin - atmid) == 0) mn = mid; else mx = mid;
        }
        roots[0] = mid;
        return 1;
    }
    for (its = 0; its < PS_MAX_ITERATIONS; its++) {
        mid = (mn + mx) / 2;
        atmid = ps_numchanges(np, sseq, mid);
        if ((atmid < atmax) || (atmid > atmin)) return 0;
        if (fabs(mid) > PS_RELERROR) {
            if (fabs((mx - mn) / mid) < PS_RELERROR) { roots[0] = mid; return 1; }
        } else if (fabs(mx - mn) < PS_RELERROR) {
            roots[0] = mid;
            return 1;
        }
        n1 = atmin - atmid;
        n2 = atmid - atmax;
        if ((n1 != 0) && (n2 != 0)) {
            n1 = ps_sbisect(np, sseq, mn, mid, atmin, atmid, roots);
            n2 = ps_sbisect(np, sseq, mid, mx, atmid, atmax, &roots[n1]);
            return n1 + n2;
        }
        if (n1 == 0) mn = mid; else mx = mid;
    }
    roots[0] = mid;
    return 1;
}

static int ps_polysolve(int order, const double* c, double* roots)
{
    Poly sseq[PS_MAX_ORDER + 1];
    for (int i = 0; i <= order; i++)
        sseq[0].coef[order - i] = c[i] / c[0];
    int np = ps_buildsturm(order, sseq);
    if (ps_visible_roots(np, sseq) == 0)
        return 0;
    int atmin = ps_numchanges(np, sseq, 0.0);
    int atmax = ps_numchanges(np, sseq, MAX_DISTANCE);
    if (atmin - atmax == 0)
        return 0;
    return ps_sbisect(np, sseq, 0.0, MAX_DISTANCE, atmin, atmax, roots);
}

static int ps_quadratic(const double* x, double* y)
{
    double a = x[0], b = -x[1], c = x[2], d, t;
    if (a == 0.0) {
        if (b == 0.0) return 0;
        y[0] = c / b;
        return 1;
    }
    b /= a;
    c /= a;
    a = 1.0;
    d = b * b - 4.0 * a * c;
    if ((d > -PS_SMALL_ENOUGH) && (d < PS_SMALL_ENOUGH)) {
        y[0] = 0.5 * b / a;
        return 1;
    } else if (d < 0.0) {
        return 0;
    }
    d = sqrt(d);
    t = 2.0 * a;
    y[0] = (b + d) / t;
    y[1] = (b - d) / t;
    return 2;
}

static int ps_cubic(const double* x, double* y)
{
    double Q, R, Q3, R2, sQ, d, an, theta, A2, a0 = x[0], a1, a2, a3;
    if (a0 == 0.0)
        return ps_quadratic(&x[1], y);
    if (a0 != 1.0) { a1 = x[1] / a0; a2 = x[2] / a0; a3 = x[3] / a0; }
    else { a1 = x[1]; a2 = x[2]; a3 = x[3]; }
    A2 = a1 * a1;
    Q = (A2 - 3.0 * a2) / 9.0;
    R = (a1 * (A2 - 4.5 * a2) + 13.5 * a3) / 27.0;
    Q3 = Q * Q * Q;
    R2 = R * R;
    d = Q3 - R2;
    an = a1 / 3.0;
    if (d >= 0.0) {
        d = R / sqrt(Q3);
        theta = acos(d) / 3.0;
        sQ = -2.0 * sqrt(Q);
        y[0] = sQ * cos(theta) - an;
        y[1] = sQ * cos(theta + TWO_M_PI_3) - an;
        y[2] = sQ * cos(theta + FOUR_M_PI_3) - an;
        return 3;
    }
    sQ = pow(sqrt(R2 - Q3) + fabs(R), 1.0 / 3.0);
    if (R < 0) y[0] = (sQ + Q / sQ) - an;
    else y[0] = -(sQ + Q / sQ) - an;
    return 1;
}

/* difficult_coeffs keeps the reference's signed "biggest" (polynomialsolver.cpp:1075-1111). */
static int ps_difficult(int n, const double* x)
{
    double biggest = 0.0;
    for (int i = 0; i <= n; i++)
        if (fabs(x[i]) > biggest) biggest = x[i];
    if (biggest == 0.0) return 0;
    for (int i = 0; i <= n; i++)
        if (x[i] != 0.0 && fabs(biggest / x[i]) > PS_FUDGE1) return 1;
    return 0;
}

static int ps_quartic(const double* x, double* results)
{
    double cubic[4], roots[3], c12, z, p, q, q1, q2, r, d1, d2, c1, c2, c3, c4, c0 = x[0];
    if (c0 != 1.0) { c1 = x[1] / c0; c2 = x[2] / c0; c3 = x[3] / c0; c4 = x[4] / c0; }
    else { c1 = x[1]; c2 = x[2]; c3 = x[3]; c4 = x[4]; }
    c12 = c1 * c1;
    p = -0.375 * c12 + c2;
    q = 0.125 * c12 * c1 - 0.5 * c1 * c2 + c3;
    r = -0.01171875 * c12 * c12 + 0.0625 * c12 * c2 - 0.25 * c1 * c3 + c4;
    cubic[0] = 1.0;
    cubic[1] = -0.5 * p;
    cubic[2] = -r;
    cubic[3] = 0.5 * r * p - 0.125 * q * q;
    if (ps_cubic(cubic, roots) > 0) z = roots[0];
    else return 0;
    d1 = 2.0 * z - p;
    if (d1 < 0.0) {
        if (d1 > -PS_SMALL_ENOUGH) d1 = 0.0;
        else return 0;
    }
    if (d1 < PS_SMALL_ENOUGH) {
        d2 = z * z - r;
        if (d2 < 0.0) return 0;
        d2 = sqrt(d2);
    } else {
        d1 = sqrt(d1);
        d2 = 0.5 * q / d1;
    }
    q1 = d1 * d1;
    q2 = -0.25 * c1;
    int i = 0;
    p = q1 - 4.0 * (z - d2);
    if (p == 0) results[i++] = -0.5 * d1 - q2;
    else if (p > 0) {
        p = sqrt(p);
        results[i++] = -0.5 * (d1 + p) + q2;
        results[i++] = -0.5 * (d1 - p) + q2;
    }
    p = q1 - 4.0 * (z + d2);
    if (p == 0) results[i++] = 0.5 * d1 - q2;
    else if (p > 0) {
        p = sqrt(p);
        results[i++] = 0.5 * (d1 + p) + q2;
        results[i++] = 0.5 * (d1 - p) + q2;
    }
    return i;
}

static int solve_polynomial(int n, const double* c0, double* r, int sturm, double epsilon)
{
    int roots = 0, i = 0;
    while ((i < n) && (fabs(c0[i]) < PS_SMALL_ENOUGH))
        i++;
    n -= i;
    const double* c = &c0[i];
    switch (n) {
    case 0: break;
    case 1: if (c[0] != 0.0) r[roots++] = -c[1] / c[0]; break;
    case 2: roots = ps_quadratic(c, r); break;
    case 3:
        if (epsilon > 0.0 && (c[2] != 0.0) && (fabs(c[3] / c[2]) < epsilon)) { roots = ps_quadratic(c, r); break; }
        roots = sturm ? ps_polysolve(3, c, r) : ps_cubic(c, r);
        break;
    case 4:
        if (epsilon > 0.0 && (c[3] != 0.0) && (fabs(c[4] / c[3]) < epsilon)) {
            roots = sturm ? ps_polysolve(3, c, r) : ps_cubic(c, r);
            break;
        }
        if (ps_difficult(4, c)) sturm = 1;
        roots = sturm ? ps_polysolve(4, c, r) : ps_quartic(c, r);
        break;
    default:
        if (epsilon > 0.0 && (c[n - 1] != 0.0) && (fabs(c[n] / c[n - 1]) < epsilon)) {
            roots = ps_polysolve(n - 1, c, r);
            break;
        }
        roots = ps_polysolve(n, c, r);
        break;
    }
    return roots;
}

/* Torus (source/core/shape/torus.cpp:78-82,241-362,932-1084) */
#define TORUS_DEPTH_TOLERANCE 1.0e-4
#define TORUS_ROOT_TOLERANCE 1.0e-4
static int torus_thick_cylinder(V3 P, V3 D, double h1, double h2, double r1, double r2)
{
    double a, b, c, d, u, v, k, r, h;
    if (fabs(D.y) < EPSILON) {
        if ((P.y < h1) || (P.y > h2)) return 0;
    } else {
        k = (h2 - P.y) / D.y;
        u = P.x + k * D.x;
        v = P.z + k * D.z;
        if ((k > EPSILON) && (k < MAX_DISTANCE)) {
            r = u * u + v * v;
            if ((r >= r1) && (r <= r2)) return 1;
        }
        k = (h1 - P.y) / D.y;
        u = P.x + k * D.x;
        v = P.z + k * D.z;
        if ((k > EPSILON) && (k < MAX_DISTANCE)) {
            r = u * u + v * v;
            if ((r >= r1) && (r <= r2)) return 1;
        }
    }
    a = D.x * D.x + D.z * D.z;
    if (a > EPSILON) {
        b = P.x * D.x + P.z * D.z;
        c = P.x * P.x + P.z * P.z - r2;
        d = b * b - a * c;
        if (d >= 0.0) {
            d = sqrt(d);
            k = (-b + d) / a;
            if ((k > EPSILON) && (k < MAX_DISTANCE)) { h = P.y + k * D.y; if ((h >= h1) && (h <= h2)) return 1; }
            k = (-b - d) / a;
            if ((k > EPSILON) && (k < MAX_DISTANCE)) { h = P.y + k * D.y; if ((h >= h1) && (h <= h2)) return 1; }
        }
        c = P.x * P.x + P.z * P.z - r1;
        d = b * b - a * c;
        if (d >= 0.0) {
            d = sqrt(d);
            k = (-b + d) / a;
            if ((k > EPSILON) && (k < MAX_DISTANCE)) { h = P.y + k * D.y; if ((h >= h1) && (h <= h2)) return 1; }
            k = (-b - d) / a;
            if ((k > EPSILON) && (k < MAX_DISTANCE)) { h = P.y + k * D.y; if ((h >= h1) && (h <= h2)) return 1; }
        }
    }
    return 0;
}

static int torus_intersect(const PovGpuObject* o, V3 O, V3 Dw, double* depth)
{
    const double* inv = o->trans + 16;
    double R = o->p[0], rr = o->p[1];
    V3 P = mtrans_point(inv, O);
    V3 D = mtrans_direction(inv, Dw);
    double len = vlen(D);
    D = vdiv(D, len);
    int i = 0;
    double y1 = -rr, y2 = rr, r1 = (R - rr) * (R - rr), r2 = (R + rr) * (R + rr);
    if (R < rr) r1 = 0;
    if (torus_thick_cylinder(P, D, y1, y2, r1, r2)) {
        double bsr = R + rr + rr;
        double dp = vdot(P, P);
        double closer = 0.0;
        if (dp > bsr * bsr) {
            dp = sqrt(dp);
            closer = dp - bsr;
            P = vadd(P, vmul(D, closer));
        }
        double R2 = R * R, rr2 = rr * rr;
        double Py2 = P.y * P.y, Dy2 = D.y * D.y, PDy2 = P.y * D.y;
        double k1 = P.x * P.x + P.z * P.z + Py2 - R2 - rr2;
        double k2 = P.x * D.x + P.z * D.z + PDy2;
        double c[5], r[4];
        c[0] = 1.0;
        c[1] = 4.0 * k2;
        c[2] = 2.0 * (k1 + 2.0 * (k2 * k2 + R2 * Dy2));
        c[3] = 4.0 * (k2 * k1 + 2.0 * R2 * PDy2);
        c[4] = k1 * k1 + 4.0 * R2 * (Py2 - rr2);
        int n = solve_polynomial(4, c, r, 0, TORUS_ROOT_TOLERANCE);
        while (n--)
            depth[i++] = (r[n] + closer) / len;
    }
    return i;
}

static int torus_inside(const PovGpuObject* o, V3 p)
{
    V3 P = mtrans_point(o->trans + 16, p);
    double r = sqrt(P.x * P.x + P.z * P.z);
    double r2 = P.y * P.y + (r - o->p[0]) * (r - o->p[0]);
    int inside = r2 <= o->p[1] * o->p[1];
    return (o->flags & POV_FLAG_INVERTED) ? !inside : inside;
}

static V3 torus_normal(const PovGpuObject* o, V3 ip)
{
    V3 P = mtrans_point(o->trans + 16, ip);
    double dist = sqrt(P.x * P.x + P.z * P.z);
    V3 M = dist > EPSILON ? v3(o->p[0] * P.x / dist, 0.0, o->p[0] * P.z / dist) : v3(0, 0, 0);
    return vnorm(mtrans_normal(o->trans + 16, vsub(P, M)));
}

#define MAX_RIN 16   /* interiors a ray can be inside at once */

typedef struct {
    PQueue  pq;       /* top-level queue */
    PQueue  mpq;      /* mesh queue (mesh.cpp:110 keeps a thread-local one) */
    uint64_t boxes, prims;
    int     counting;
    /* statistics of the render */
    uint64_t rays, shadow_tests, shadow_succeeded, reflected, transmitted, media_samples;
    /* radiosity task state (RadiosityFunction, radiosity.cpp:297-330):
     * final trace or pretrace, its error bound and pass, the position of
     * each bounce depth's direction sequence, the top-level query count */
    int      rad_final;
    double   rad_error_bound;
    int      rad_pass;
    int      rad_dir_index[8];
    uint64_t rad_top_queries;
    uint64_t gt_rng;          /* converged mode: the pixel's random sequence */
    /* the current ray's interior list (Ray::GetInteriors): interior ids of
     * the objects the ray travels inside, innermost last */
    int      rin[MAX_RIN];
    int      nrin;
    uint64_t refracted, internal_reflected;
} Thread;

/* Sphere::Intersect (sphere.cpp:214-245). */
static int sphere_intersect(V3 O, V3 D, V3 C, double r2, double* d1, double* d2)
{
    V3 oc = vsub(C, O);
    double ocs = vdot(oc, oc);
    double tca = vdot(oc, D);
    if (ocs >= r2 && tca < EPSILON)
        return 0;
    double thcs = r2 - ocs + tca * tca;
    if (thcs > EPSILON) {
        double hc = sqrt(thcs);
        *d1 = tca - hc;
        *d2 = tca + hc;
        return 1;
    }
    return 0;
}

/* Mesh::intersect_mesh_triangle (mesh.cpp:1040-1120). */
static int mesh_triangle(const OMesh* m, const MeshTri* T, V3 O, V3 D, double* depth)
{
    V3 N = v3(T->normal[0], T->normal[1], T->normal[2]);
    double ndd = vdot(N, D);
    if (fabs(ndd) < EPSILON)
        return 0;
    double ndo = vdot(N, O);
    double t = -((double)T->distance + ndo) / ndd;
    *depth = t;
    if (t < MESH_DEPTH_TOLERANCE || t > MAX_DISTANCE)
        return 0;
    const float* v = m->verts;
    V3 P1 = v3(v[3 * T->p1], v[3 * T->p1 + 1], v[3 * T->p1 + 2]);
    V3 P2 = v3(v[3 * T->p2], v[3 * T->p2 + 1], v[3 * T->p2 + 2]);
    V3 P3 = v3(v[3 * T->p3], v[3 * T->p3 + 1], v[3 * T->p3 + 2]);
    double s, u;
    switch (T->dominant_axis) {
    case 0:
        s = O.y + t * D.y; u = O.z + t * D.z;
        if ((P2.y - s) * (P2.z - P1.z) < (P2.z - u) * (P2.y - P1.y)) return 0;
        if ((P3.y - s) * (P3.z - P2.z) < (P3.z - u) * (P3.y - P2.y)) return 0;
        if ((P1.y - s) * (P1.z - P3.z) < (P1.z - u) * (P1.y - P3.y)) return 0;
        return 1;
    case 1:
        s = O.x + t * D.x; u = O.z + t * D.z;
        if ((P2.x - s) * (P2.z - P1.z) < (P2.z - u) * (P2.x - P1.x)) return 0;
        if ((P3.x - s) * (P3.z - P2.z) < (P3.z - u) * (P3.x - P2.x)) return 0;
        if ((P1.x - s) * (P1.z - P3.z) < (P1.z - u) * (P1.x - P3.x)) return 0;
        return 1;
    default:
        s = O.x + t * D.x; u = O.y + t * D.y;
        if ((P2.x - s) * (P2.y - P1.y) < (P2.y - u) * (P2.x - P1.x)) return 0;
        if ((P3.x - s) * (P3.y - P2.y) < (P3.y - u) * (P3.x - P2.x)) return 0;
        if ((P1.x - s) * (P1.y - P3.y) < (P1.y - u) * (P1.x - P3.x)) return 0;
        return 1;
    }
}

/* Mesh::intersect_bbox_tree (mesh.cpp:1452-1566) fused with the closest-hit
 * filter of Find_Intersection (object.cpp:118-168): returns the nearest
 * triangle hit with depth >= min_depth and < closest. */
static int mesh_closest(const OMesh* m, Thread* th, V3 O, V3 D, double min_depth, double closest,
                        double* best_t, int32_t* best_tri)
{
    RayInfo ri;
    rayinfo_init(&ri, O, D);
    pq_clear(&th->mpq);
    int found = 0;
    double best = closest;
    if (m->tree.root < 0)
        return 0;
    check_and_enqueue(&th->mpq, &m->tree.nodes[m->tree.root], m->tree.root, &ri,
                      th->counting ? &th->boxes : NULL);
    double depth;
    int32_t nid;
    while (pq_remove_min(&th->mpq, &depth, &nid)) {
        if (depth > best)
            break;
        const TNode* n = &m->tree.nodes[nid];
        if (n->entries) {
            for (int i = 0; i < n->entries; i++) {
                int32_t c = m->tree.kids[n->first + i];
                check_and_enqueue(&th->mpq, &m->tree.nodes[c], c, &ri, th->counting ? &th->boxes : NULL);
            }
        } else {
            double t;
            if (th->counting) th->prims++;
            if (mesh_triangle(m, &m->tris[n->first], O, D, &t)) {
                if (t >= min_depth && t < best) {
                    best = t;
                    *best_tri = n->first;
                    found = 1;
                }
            }
        }
    }
    *best_t = best;
    return found;
}

/* One entry of an IStack (Intersection: depth, object, aux = box side or
 * mesh triangle). */
typedef struct { double depth; int32_t object; int32_t aux; } Hit;
#define MAX_HITS 64

static int inside_object(const PovOracle* S, int32_t oi, V3 p);

/* All_Intersections of one object (the shape files' All_Intersections and
 * the CSG ones of source/core/shape/csg.cpp:128-403), pushing every hit in
 * the reference's order. */
static int object_all_hits(const PovOracle* S, Thread* th, int32_t oi, V3 O, V3 D, Hit* out, int n, int cap)
{
    const PovGpuObject* o = &S->objs[oi].o;
    switch (o->type) {
    case POV_OBJ_SPHERE: {   /* sphere.cpp:92-212 */
        double d1, d2;
        if (sphere_intersect(O, D, v3(o->p[0], o->p[1], o->p[2]), o->p[3] * o->p[3], &d1, &d2)) {
            if (d1 > SPHERE_DEPTH_TOLERANCE && d1 < MAX_DISTANCE && n < cap) out[n++] = (Hit){d1, oi, -1};
            if (d2 > SPHERE_DEPTH_TOLERANCE && d2 < MAX_DISTANCE && n < cap) out[n++] = (Hit){d2, oi, -1};
        }
        return n;
    }
    case POV_OBJ_PLANE: {    /* plane.cpp:92-211 */
        V3 N = v3(o->p[0], o->p[1], o->p[2]);
        double ndd = vdot(N, D);
        if (fabs(ndd) < EPSILON) return n;
        double t = -(vdot(N, O) + o->p[3]) / ndd;
        if (t >= PLANE_DEPTH_TOLERANCE && t <= MAX_DISTANCE && n < cap) out[n++] = (Hit){t, oi, -1};
        return n;
    }
    case POV_OBJ_BOX: {      /* box.cpp:100-170 */
        double d1, d2;
        int s1, s2;
        if (box_intersect(O, D, v3(o->p[0], o->p[1], o->p[2]), v3(o->p[3], o->p[4], o->p[5]), &d1, &d2, &s1, &s2)) {
            if (d1 > BOX_DEPTH_TOLERANCE && n < cap) out[n++] = (Hit){d1, oi, s1};
            if (n < cap) out[n++] = (Hit){d2, oi, s2};
        }
        return n;
    }
    case POV_OBJ_TORUS: {    /* torus.cpp:133-160 */
        double dep[4];
        int k = torus_intersect(o, O, D, dep);
        for (int i = 0; i < k; i++)
            if (dep[i] > TORUS_DEPTH_TOLERANCE && dep[i] < MAX_DISTANCE && n < cap) out[n++] = (Hit){dep[i], oi, -1};
        return n;
    }
    case POV_OBJ_UNION: {
        for (int c = 0; c < o->num_children; c++)
            n = object_all_hits(S, th, o->first_child + c, O, D, out, n, cap);
        return n;
    }
    case POV_OBJ_INTERSECTION:
    case POV_OBJ_MERGE: {
        Hit local[MAX_HITS];
        int merge = o->type == POV_OBJ_MERGE;
        int c = o->first_child;
        for (int k = 0; k < o->num_children; k++) {
            int ln = object_all_hits(S, th, c, O, D, local, 0, MAX_HITS);
            /* the local stack is drained from the top */
            for (int h = ln - 1; h >= 0; h--) {
                V3 P = vadd(O, vmul(D, local[h].depth));
                int keep = 1;
                /* children are leaves here (checked at create), so siblings are consecutive */
                for (int j = 0; j < o->num_children; j++) {
                    int s = o->first_child + j;
                    if (s != c) {
                        int in = inside_object(S, s, P);
                        if (merge ? in : !in) { keep = 0; break; }
                    }
                }
                if (keep && n < cap) out[n++] = local[h];
            }
            c++;
        }
        return n;
    }
    default:
        return n;
    }
}

/* ObjectBase::Inside for the supported shapes (sphere.cpp:271-303,
 * box.cpp Box::Inside, torus.cpp Torus::Inside, plane.cpp Plane::Inside,
 * csg.cpp:405-450). */
static int inside_object(const PovOracle* S, int32_t oi, V3 p)
{
    const PovGpuObject* o = &S->objs[oi].o;
    int inv = (o->flags & POV_FLAG_INVERTED) != 0;
    switch (o->type) {
    case POV_OBJ_SPHERE: {
        V3 d = vsub(v3(o->p[0], o->p[1], o->p[2]), p);
        double ocs = vdot(d, d), r2 = o->p[3] * o->p[3];
        return inv ? ocs > r2 : ocs < r2;
    }
    case POV_OBJ_BOX:
        if (p.x < o->p[0] || p.x > o->p[3] || p.y < o->p[1] || p.y > o->p[4] || p.z < o->p[2] || p.z > o->p[5])
            return inv;
        return !inv;
    case POV_OBJ_TORUS:
        return torus_inside(o, p);
    case POV_OBJ_PLANE:
        return (vdot(p, v3(o->p[0], o->p[1], o->p[2])) + o->p[3]) < EPSILON;
    case POV_OBJ_UNION:
    case POV_OBJ_MERGE:
        for (int c = 0; c < o->num_children; c++)
            if (inside_object(S, o->first_child + c, p)) return 1;
        return 0;
    case POV_OBJ_INTERSECTION:
        for (int c = 0; c < o->num_children; c++)
            if (!inside_object(S, o->first_child + c, p)) return 0;
        return 1;
    default:
        return 0;
    }
}

/* Per-object closest hit: Find_Intersection (object.cpp:118-168,172-225):
 * the IStack is drained from the top and the closest depth >= min_depth
 * (MIN_ISECT_DEPTH, raised by a postcondition such as SMALL_TOLERANCE for
 * shadow rays) wins on strict '<'. */
static int object_closest(const PovOracle* S, Thread* th, int32_t oi, V3 O, V3 D, double min_depth,
                          double closest, Isect* out)
{
    const OObj* ob = &S->objs[oi];
    const PovGpuObject* o = &ob->o;
    double best = closest;
    int found = 0;
    if (th->counting) th->prims++;
    if (o->type == POV_OBJ_MESH) {
        if (!intersect_bbox_dir(&ob->bbox, O, D, (float)closest))
            return 0;
        double t;
        int32_t tri = -1;
        if (mesh_closest(&S->meshes[o->mesh], th, O, D, min_depth, best, &t, &tri)) {
            out->depth = t;
            out->object = oi;
            out->triangle = tri;
            out->ipoint = vadd(O, vmul(D, t));
            return 1;
        }
        return 0;
    }
    /* ObjectBase::Intersect_BBox pre-test: sphere, plane and box answer true */
    if (o->type == POV_OBJ_TORUS || o->type >= POV_OBJ_UNION)
        if (!intersect_bbox_dir(&ob->bbox, O, D, (float)closest))
            return 0;
    Hit hits[MAX_HITS];
    int n = object_all_hits(S, th, oi, O, D, hits, 0, MAX_HITS);
    for (int i = n - 1; i >= 0; i--) {
        if (hits[i].depth < best && hits[i].depth >= min_depth) {
            best = hits[i].depth;
            out->object = hits[i].object;
            out->triangle = hits[i].aux;
            found = 1;
        }
    }
    if (found) {
        out->depth = best;
        out->ipoint = vadd(O, vmul(D, best));
    }
    return found;
}

/* Intersect_BBox_Tree (boundingbox.cpp:432-539) / linear scan
 * (trace.cpp:263-281).  `shadow` selects the shadow-ray conditions
 * (NoShadowFlag precondition, SmallTolerance postcondition,
 * trace.cpp:1935-1949). */
static int find_intersection(const PovOracle* S, Thread* th, V3 O, V3 D, double max_depth, int shadow, Isect* best)
{
    int found = 0;
    best->depth = max_depth;
    best->object = -1;
    best->triangle = -1;
    if (S->top_linear || S->top.root < 0) {
        for (int32_t i = 0; i < S->nobjs; i++) {
            if (S->objs[i].o.parent >= 0) continue;
            if (shadow && (S->objs[i].o.flags & POV_FLAG_NO_SHADOW)) continue;
            Isect is;
            if (object_closest(S, th, i, O, D, shadow ? nextafter(SMALL_TOLERANCE, 1.0) : MIN_ISECT_DEPTH,
                               HUGE_VAL, &is) && is.depth < best->depth) {
                *best = is;
                found = 1;
            }
        }
        return found;
    }
    RayInfo ri;
    rayinfo_init(&ri, O, D);
    pq_clear(&th->pq);
    check_and_enqueue(&th->pq, &S->top.nodes[S->top.root], S->top.root, &ri, th->counting ? &th->boxes : NULL);
    double depth;
    int32_t nid;
    while (pq_remove_min(&th->pq, &depth, &nid)) {
        if (depth > best->depth)
            break;
        const TNode* n = &S->top.nodes[nid];
        if (n->entries) {
            for (int i = 0; i < n->entries; i++) {
                int32_t c = S->top.kids[n->first + i];
                check_and_enqueue(&th->pq, &S->top.nodes[c], c, &ri, th->counting ? &th->boxes : NULL);
            }
        } else {
            int32_t oi = n->first;
            if (shadow && (S->objs[oi].o.flags & POV_FLAG_NO_SHADOW))
                continue;
            Isect is;
            /* the postcondition "dist > SMALL_TOLERANCE" on top of t >= MIN_ISECT_DEPTH */
            if (object_closest(S, th, oi, O, D, shadow ? nextafter(SMALL_TOLERANCE, 1.0) : MIN_ISECT_DEPTH,
                               HUGE_VAL, &is)) {
                if (is.depth < best->depth) {
                    *best = is;
                    found = 1;
                }
            }
        }
    }
    return found;
}

/* --------------------------------------------------------- shading --- */
static V3 object_normal(const PovOracle* S, const Isect* is)
{
    const PovGpuObject* o = &S->objs[is->object].o;
    switch (o->type) {
    case POV_OBJ_SPHERE:   /* Sphere::Normal (sphere.cpp:333-356) */
        return vdiv(vsub(is->ipoint, v3(o->p[0], o->p[1], o->p[2])), o->p[3]);
    case POV_OBJ_PLANE:
        return v3(o->p[0], o->p[1], o->p[2]);
    case POV_OBJ_BOX:      /* Box::Normal: the side recorded in Intersection::i1 */
        switch (is->triangle) {
        case SIDE_X0: return v3(-1, 0, 0);
        case SIDE_X1: return v3(1, 0, 0);
        case SIDE_Y0: return v3(0, -1, 0);
        case SIDE_Y1: return v3(0, 1, 0);
        case SIDE_Z0: return v3(0, 0, -1);
        default: return v3(0, 0, 1);
        }
    case POV_OBJ_TORUS:
        return torus_normal(o, is->ipoint);
    case POV_OBJ_MESH: {   /* Mesh::Normal, Smooth_Mesh_Normal (mesh.cpp:342-436) */
        const OMesh* m = &S->meshes[o->mesh];
        const MeshTri* T = &m->tris[is->triangle];
        if (T->smooth) {
            const float* nv = m->normals;
            V3 N1 = v3(nv[3 * T->n1], nv[3 * T->n1 + 1], nv[3 * T->n1 + 2]);
            V3 N2 = v3(nv[3 * T->n2], nv[3 * T->n2 + 1], nv[3 * T->n2 + 2]);
            V3 N3 = v3(nv[3 * T->n3], nv[3 * T->n3 + 1], nv[3 * T->n3 + 2]);
            const float* v = m->verts;
            V3 P1 = v3(v[3 * T->p1], v[3 * T->p1 + 1], v[3 * T->p1 + 2]);
            V3 PI = vsub(is->ipoint, P1);
            double u = vdot(PI, v3(T->perp[0], T->perp[1], T->perp[2]));
            V3 R;
            if (u < EPSILON) {
                R = N1;
            } else {
                int ax = T->v_axis;
                double k1 = v[3 * T->p1 + ax], k2 = v[3 * T->p2 + ax], k3 = v[3 * T->p3 + ax];
                double vv = (vget(PI, ax) / u + k1 - k2) / (k3 - k2);
                R = vadd(N1, vmul(vadd(vsub(N2, N1), vmul(vsub(N3, N2), vv)), u));
            }
            return vnorm(R);
        }
        return v3(T->normal[0], T->normal[1], T->normal[2]);
    }
    default:
        return v3(0, 1, 0);
    }
}

/* ====================================================== pattern pigments ==
 * Noise tables: the hash permutation (InitTextureTable, noise.cpp:231-256),
 * the lattice values (RTable, noise.cpp:98-182) and the Perlin gradient
 * tables (InitSolidNoise, noise.cpp:306-347), all from the reference's
 * linear congruential sequence next = next * 1812433253 + 12345 kept in a
 * 32-bit int. */
#define NOISE_ENTRIES 2048
static unsigned short g_hash[8192];
static double g_rtab[2 * POV_NOISE_RTABLE_SIZE];
static int g_perm[2 * (NOISE_ENTRIES + 1)];
static V3 g_ngrad[2 * (NOISE_ENTRIES + 1)];
static pthread_once_t g_noise_once = PTHREAD_ONCE_INIT;

/* the scene's wave sources and frequencies (SceneData::numberOfWaves = 10,
 * Initialize_Waves, noise.cpp:189-205) */
#define NUM_WAVES 10
static V3 g_wave_src[NUM_WAVES];
static double g_wave_freq[NUM_WAVES];
static void waves_init(void);

static int32_t lcg_next(int32_t x) { return (int32_t)(uint32_t)((int64_t)x * 1812433253LL + 12345LL); }

static void noise_init(void)
{
    int32_t next = 0;
    for (int i = 0; i < 4096; i++)
        g_hash[i] = (unsigned short)i;
    for (int i = 4095; i >= 0; i--) {
        next = lcg_next(next);
        int j = ((int)(next >> 16) & 0x7FFF) % 4096;
        unsigned short t = g_hash[i];
        g_hash[i] = g_hash[j];
        g_hash[j] = t;
    }
    for (int i = 0; i < 4096; i++)
        g_hash[4096 + i] = g_hash[i];
    for (int i = 0; i < POV_NOISE_RTABLE_SIZE; i++) {
        g_rtab[2 * i] = kPovNoiseRTable[i];
        g_rtab[2 * i + 1] = kPovNoiseRTable[i] * 0.5;
    }
    next = 1;
    for (int i = 0; i < NOISE_ENTRIES; i++) {
        double v[3], q;
        do {
            for (int k = 0; k < 3; k++) {
                next = lcg_next(next);
                v[k] = (double)((((int)(next >> 16) & 0x7FFF) % (NOISE_ENTRIES << 1)) - NOISE_ENTRIES) /
                       (double)NOISE_ENTRIES;
            }
            q = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        } while (q > 1.0 || q < 1.0e-5);
        q = sqrt(q);
        g_ngrad[i] = v3(v[0] / q, v[1] / q, v[2] / q);
    }
    for (int i = 0; i < NOISE_ENTRIES; i++)
        g_perm[i] = i;
    for (int i = NOISE_ENTRIES; i > 0; i -= 2) {
        int k = g_perm[i];
        next = lcg_next(next);
        int j = ((int)(next >> 16) & 0x7FFF) % NOISE_ENTRIES;
        g_perm[i] = g_perm[j];
        g_perm[j] = k;
    }
    for (int i = 0; i < NOISE_ENTRIES + 2; i++) {
        g_perm[NOISE_ENTRIES + i] = g_perm[i];
        g_ngrad[NOISE_ENTRIES + i] = g_ngrad[i];
    }
    waves_init();
}

/* The pattern random table (gPatternRands = RandomDoubleSequence(0, 1,
 * 32768), pattern.cpp:91): boost's mt19937 at its default seed 5489
 * through uniform_real, x / 2^32 (randomsequence.cpp:138-149 with
 * boost/random/uniform_real_distribution.hpp's generate_uniform_real) --
 * the Mersenne Twister of Matsumoto and Nishimura (1998), restated.
 * Hash3d yields indices below 4096 and crackle reads two past its index,
 * so the patterns read only the first 4098 entries. */
#define PATTERN_RANDS 4100
static double g_prand[PATTERN_RANDS];
static pthread_once_t g_prand_once = PTHREAD_ONCE_INIT;

static void prand_init(void)
{
    uint32_t mt[624];
    mt[0] = 5489u;
    for (int i = 1; i < 624; i++)
        mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    int idx = 624;
    for (int n = 0; n < PATTERN_RANDS; n++) {
        if (idx >= 624) {
            for (int i = 0; i < 624; i++) {
                const uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            idx = 0;
        }
        uint32_t y = mt[idx++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        g_prand[n] = (double)y / 4294967296.0;
    }
}

double pov_oracle_pattern_rand(int32_t i)
{
    pthread_once(&g_prand_once, prand_init);
    return (i >= 0 && i < PATTERN_RANDS) ? g_prand[i] : -1.0;
}

/* Hash3d (texture.h:75-76) over the noise hash table. */
static int hash3d(int a, int b, int c)
{
    return g_hash[g_hash[g_hash[a & 0xfff] ^ (b & 0xfff)] ^ (c & 0xfff)];
}

/* one coordinate's place within its brick or mortar period: the
 * fraction after (int) truncation, lifted into [0, 1) (pattern.cpp:5520-5610) */
static double brick_frac(double v)
{
    v -= (double)(int)v;
    return v < 0.0 ? v + 1.0 : v;
}

/* BrickPattern::Evaluate (pattern.cpp:5495-5623): 0 in the mortar, 1 in a
 * brick; courses of bricks offset by half a brick. */
static double brick_value(const PovGpuPattern* pt, V3 T)
{
    const double mortar = pt->mortar, fudge = EPSILON + mortar;
    const double x = T.x + fudge, y = T.y + fudge, z = T.z + fudge;
    const double bw = pt->brick_size[0], bh = pt->brick_size[1], bd = pt->brick_size[2];
    if (brick_frac(y / bh) <= mortar / bh)
        return 0.0;
    const double by = brick_frac((y / bh) * 0.5);
    if (brick_frac(x / bw) <= mortar / bw && by <= 0.5)
        return 0.0;
    if (brick_frac(x / bw + 0.5) <= mortar / bw && by > 0.5)
        return 0.0;
    if (brick_frac(z / bd) <= mortar / bd && by > 0.5)
        return 0.0;
    if (brick_frac(z / bd + 0.5) <= mortar / bd && by <= 0.5)
        return 0.0;
    return 1.0;
}

/* QuiltedPattern::EvaluateRaw with quilt_cubic (pattern.cpp:8067-8083,
 * 8949-8968); FLOOR is texture.h:73's (one less at negative integers). */
static double quilted_value(const PovGpuPattern* pt, V3 T)
{
#define QFLOOR(x) ((x) >= 0.0 ? floor(x) : (0.0 - floor(0.0 - (x)) - 1.0))
    V3 v = v3(T.x - QFLOOR(T.x) - 0.5, T.y - QFLOOR(T.y) - 0.5, T.z - QFLOOR(T.z) - 0.5);
#undef QFLOOR
    const double t = vlen(v), it = 1.0 - t;
    const double c = (t * t * t + 3.0 * t * it * it * pt->control0 + 3.0 * t * t * it * pt->control1) * 1.154700538;
    v = vmul(v, c);
    return (fabs(v.x) + fabs(v.y) + fabs(v.z)) / 3.0;
}

static double crackle_dist(const PovGpuPattern* pt, V3 dv)
{
    const double m = pt->crackle_metric;
    if (m == 2.0)
        return vdot(dv, dv);
    if (m == 1.0)
        return fabs(dv.x) + fabs(dv.y) + fabs(dv.z);
    return pow(fabs(dv.x), m) + pow(fabs(dv.y), m) + pow(fabs(dv.z), m);
}

static double pov_noise(V3 P, int gen);

/* CracklePattern::EvaluateRaw (pattern.cpp:5760-6010) without repeat: the
 * nuclei of the 81 cubes within a "3d knight move" (InitialiseCrackleCubeTable,
 * pattern.cpp:9348-9373, in its order; IntPickInCube, pattern.cpp:8808-8818),
 * the three smallest distances under the metric kept as the reference keeps
 * them, then the offset and the form (or the noise at the nearest nucleus
 * when solid), clipped to [0, 1]. */
static double crackle_value(const PovGpuPattern* pt, V3 T)
{
    pthread_once(&g_prand_once, prand_init);
    const int fx = (int)floor(T.x - EPSILON), fy = (int)floor(T.y - EPSILON), fz = (int)floor(T.z - EPSILON);
    V3 nuc[81];
    int n = 0;
    for (int ax = -2; ax <= 2; ax++)
        for (int ay = -2; ay <= 2; ay++)
            for (int az = -2; az <= 2; az++) {
                if ((abs(ax) == 2) + (abs(ay) == 2) + (abs(az) == 2) > 1)
                    continue;
                const int cx = fx + ax, cy = fy + ay, cz = fz + az;
                const int seed = hash3d(cx & 0xFFF, cy & 0xFFF, cz & 0xFFF);
                nuc[n++] = v3(cx + g_prand[seed], cy + g_prand[seed + 1], cz + g_prand[seed + 2]);
            }
    double m1 = crackle_dist(pt, vsub(nuc[0], T)), m2 = crackle_dist(pt, vsub(nuc[1], T));
    double m3 = crackle_dist(pt, vsub(nuc[2], T)), tf;
    int idx = 0;
    if (m2 < m1) { tf = m1; m1 = m2; m2 = tf; idx = 1; }
    if (m3 < m1) { tf = m1; m1 = m3; m3 = tf; idx = 2; }
    if (m3 < m2) { tf = m2; m2 = m3; m3 = tf; }
    for (int i = 3; i < 81; i++) {
        const double sum = crackle_dist(pt, vsub(nuc[i], T));
        if (sum < m1) { m3 = m2; m2 = m1; m1 = sum; idx = i; }
        else if (sum < m2) { m3 = m2; m2 = sum; }
        else if (sum < m3) { m3 = sum; }
    }
    const double m = pt->crackle_metric, off = pt->crackle_offset;
    if (off != 0.0) {
        const double a = m == 2.0 ? off * off : (m == 1.0 ? off : pow(off, m));
        m1 += a; m2 += a; m3 += a;
    }
    const double* f = pt->crackle_form;
    if (pt->crackle_solid)
        tf = pov_noise(nuc[idx], pt->noise_generator);
    else if (m == 2.0)
        tf = f[0] * sqrt(m1) + f[1] * sqrt(m2) + f[2] * sqrt(m3);
    else if (m == 1.0)
        tf = f[0] * m1 + f[1] * m2 + f[2] * m3;
    else
        tf = f[0] * pow(m1, 1.0 / m) + f[1] * pow(m2, 1.0 / m) + f[2] * pow(m3, 1.0 / m);
    return fmax(fmin(tf, 1.0), 0.0);
}

static double scurve(double t) { return t * t * (3.0 - 2.0 * t); }
static double lerp(double t, double a, double b) { return a + t * (b - a); }

/* SolidNoise (noise.cpp:392-440): Perlin gradient noise, generator 3. */
static double solid_noise(V3 P)
{
    const double ROLLOVER = 10000000.023157213;
    int b0[3], b1[3];
    double r0[3], r1[3];
    const double p[3] = {P.x, P.y, P.z};
    for (int a = 0; a < 3; a++) {
        double t = p[a] + ROLLOVER;
        int it = (int)floor(t);
        b0[a] = it & (NOISE_ENTRIES - 1);
        b1[a] = (b0[a] + 1) & (NOISE_ENTRIES - 1);
        r0[a] = t - it;
        r1[a] = r0[a] - 1.0;
    }
    int i = g_perm[b0[0]], j = g_perm[b1[0]];
    int b00 = g_perm[i + b0[1]], b10 = g_perm[j + b0[1]], b01 = g_perm[i + b1[1]], b11 = g_perm[j + b1[1]];
    double sx = scurve(r0[0]), sy = scurve(r0[1]), sz = scurve(r0[2]);
#define AT(g, rx, ry, rz) (g.x * (rx) + g.y * (ry) + g.z * (rz))
    double u = AT(g_ngrad[b00 + b0[2]], r0[0], r0[1], r0[2]), v = AT(g_ngrad[b10 + b0[2]], r1[0], r0[1], r0[2]);
    double a = lerp(sx, u, v);
    u = AT(g_ngrad[b01 + b0[2]], r0[0], r1[1], r0[2]);
    v = AT(g_ngrad[b11 + b0[2]], r1[0], r1[1], r0[2]);
    double b = lerp(sx, u, v);
    double c = lerp(sy, a, b);
    u = AT(g_ngrad[b00 + b1[2]], r0[0], r0[1], r1[2]);
    v = AT(g_ngrad[b10 + b1[2]], r1[0], r0[1], r1[2]);
    a = lerp(sx, u, v);
    u = AT(g_ngrad[b01 + b1[2]], r0[0], r1[1], r1[2]);
    v = AT(g_ngrad[b11 + b1[2]], r1[0], r1[1], r1[2]);
    b = lerp(sx, u, v);
    double d = lerp(sy, a, b);
#undef AT
    return lerp(sz, c, d);
}

/* PortableNoise (portablenoise.cpp:103-225): the lattice noise of generators
 * 1 (original) and 2 (range corrected), Perlin noise for 3. */
static double pov_noise(V3 P, int gen)
{
    if (gen == 3) {
        double sum = 0.5 * (1.59 * solid_noise(P) + 0.985);
        return sum < 0.0 ? 0.0 : (sum > 1.0 ? 1.0 : sum);
    }
    const double p[3] = {P.x, P.y, P.z};
    int ii[3];
    double f[3], g[3], sc[3], tc[3];
    for (int a = 0; a < 3; a++) {
        int tmp = p[a] >= 0 ? (int)p[a] : (int)(p[a] - (1 - EPSILON));
        ii[a] = (tmp - (-10000)) & 0xFFF;
        f[a] = p[a] - tmp;
        g[a] = f[a] - 1;
        sc[a] = scurve(f[a]);
        tc[a] = 1 - sc[a];
    }
    const double txty = tc[0] * tc[1], sxty = sc[0] * tc[1], txsy = tc[0] * sc[1], sxsy = sc[0] * sc[1];
#define HASH2(a, b) g_hash[(int)(g_hash[(int)(a)] ^ (b))]
#define RIDX(a, b) ((g_hash[(int)(a) ^ (b)] & 0xFF) * 2)
#define INCR(m, s, x, y, z) ((s) * (g_rtab[(m) + 1] + g_rtab[(m) + 2] * (x) + g_rtab[(m) + 4] * (y) + g_rtab[(m) + 6] * (z)))
    const int h00 = HASH2(ii[0], ii[1]), h10 = HASH2(ii[0] + 1, ii[1]);
    const int h01 = HASH2(ii[0], ii[1] + 1), h11 = HASH2(ii[0] + 1, ii[1] + 1);
    double sum = INCR(RIDX(h00, ii[2]), txty * tc[2], f[0], f[1], f[2]);
    sum += INCR(RIDX(h10, ii[2]), sxty * tc[2], g[0], f[1], f[2]);
    sum += INCR(RIDX(h01, ii[2]), txsy * tc[2], f[0], g[1], f[2]);
    sum += INCR(RIDX(h11, ii[2]), sxsy * tc[2], g[0], g[1], f[2]);
    sum += INCR(RIDX(h00, ii[2] + 1), txty * sc[2], f[0], f[1], g[2]);
    sum += INCR(RIDX(h10, ii[2] + 1), sxty * sc[2], g[0], f[1], g[2]);
    sum += INCR(RIDX(h01, ii[2] + 1), txsy * sc[2], f[0], g[1], g[2]);
    sum += INCR(RIDX(h11, ii[2] + 1), sxsy * sc[2], g[0], g[1], g[2]);
#undef HASH2
#undef RIDX
#undef INCR
    if (gen == 2) {
        sum += 1.05242;
        sum *= 0.48985582;
    } else {
        sum = sum + 0.5;
    }
    return sum < 0.0 ? 0.0 : (sum > 1.0 ? 1.0 : sum);
}

/* PortableDNoise (portablenoise.cpp:260-361): vector noise, the lattice
 * functions of three consecutive table entries per corner (every
 * generator: DNoise has no Perlin variant). */
static V3 pov_dnoise(V3 P)
{
    const double p[3] = {P.x, P.y, P.z};
    int ii[3];
    double f[3], g[3], sc[3], tc[3];
    for (int a = 0; a < 3; a++) {
        int tmp = p[a] >= 0 ? (int)p[a] : (int)(p[a] - (1 - EPSILON));
        ii[a] = (tmp - (-10000)) & 0xFFF;
        f[a] = p[a] - tmp;
        g[a] = f[a] - 1;
        sc[a] = scurve(f[a]);
        tc[a] = 1 - sc[a];
    }
    const double txty = tc[0] * tc[1], sxty = sc[0] * tc[1], txsy = tc[0] * sc[1], sxsy = sc[0] * sc[1];
#define HASH2(a, b) g_hash[(int)(g_hash[(int)(a)] ^ (b))]
#define RIDX(a, b) ((g_hash[(int)(a) ^ (b)] & 0xFF) * 2)
#define INCR(m, s, x, y, z) ((s) * (g_rtab[(m) + 1] + g_rtab[(m) + 2] * (x) + g_rtab[(m) + 4] * (y) + g_rtab[(m) + 6] * (z)))
    const int h00 = HASH2(ii[0], ii[1]), h10 = HASH2(ii[0] + 1, ii[1]);
    const int h01 = HASH2(ii[0], ii[1] + 1), h11 = HASH2(ii[0] + 1, ii[1] + 1);
    /* corners in the reference's order; each adds its three components */
    const int hc[8] = {h00, h10, h11, h01, h01, h11, h10, h00};
    const int zc[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    const double sw[8] = {txty * tc[2], sxty * tc[2], sxsy * tc[2], txsy * tc[2],
                          txsy * sc[2], sxsy * sc[2], sxty * sc[2], txty * sc[2]};
    const int xo[8] = {0, 1, 1, 0, 0, 1, 1, 0}, yo[8] = {0, 0, 1, 1, 1, 1, 0, 0};
    double r[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 8; k++) {
        int m = RIDX(hc[k], ii[2] + zc[k]);
        const double x = xo[k] ? g[0] : f[0], y = yo[k] ? g[1] : f[1], z = zc[k] ? g[2] : f[2];
        for (int c = 0; c < 3; c++, m += 8) {
            const double v = INCR(m, sw[k], x, y, z);
            r[c] = k == 0 ? v : r[c] + v;
        }
    }
#undef HASH2
#undef RIDX
#undef INCR
    return v3(r[0], r[1], r[2]);
}

/* Initialize_Waves (noise.cpp:189-205): source i is the normalised DNoise
 * at (i, 0, 0), its frequency the next value of the start-up sequence. */
static void waves_init(void)
{
    int32_t next = -560851967;
    for (int i = 0; i < NUM_WAVES; i++) {
        g_wave_src[i] = vnorm(pov_dnoise(v3((double)i, 0.0, 0.0)));
        next = lcg_next(next);
        g_wave_freq[i] = (double)((int)(next >> 16) & 0x7FFF) * 0.000030518509476 + 0.01;
    }
}

/* Turbulence and DTurbulence (noise.cpp:522-630): Octaves of the noise at
 * lambda^k-scaled points, weighted by omega^k. */
static double pov_turbulence(V3 P, const PovGpuPattern* t, int gen)
{
    double value;
    if (gen == 1) {
        value = pov_noise(P, gen);
    } else {
        value = 2.0 * pov_noise(P, gen) - 0.5;
        value = value < 0.0 ? 0.0 : (value > 1.0 ? 1.0 : value);
    }
    /* GenericTurbulenceWarp keeps Lambda and Omega in single precision */
    const double lambda = (float)t->lambda, omega = (float)t->omega;
    double l = lambda, o = omega;
    for (int i = 2; i <= t->octaves; i++) {
        const V3 q = vmul(P, l);
        if (gen == 1)
            value += o * pov_noise(q, gen);
        else
            value += o * (2.0 * pov_noise(q, gen) - 0.5);
        if (i < t->octaves) {
            l *= lambda;
            o *= omega;
        }
    }
    return value;
}

static V3 pov_dturbulence(V3 P, const PovGpuPattern* t)
{
    V3 r = pov_dnoise(P);
    /* GenericTurbulenceWarp keeps Lambda and Omega in single precision */
    const double lambda = (float)t->lambda, omega = (float)t->omega;
    double l = lambda, o = omega;
    for (int i = 2; i <= t->octaves; i++) {
        const V3 v = pov_dnoise(vmul(P, l));
        r = vadd(r, vmul(v, o));
        if (i < t->octaves) {
            l *= lambda;
            o *= omega;
        }
    }
    return r;
}

/* cycloidal (texture.cpp:98-108) and Triangle_Wave (texture.cpp:138-156). */
#define TWO_M_PI 6.283185307179586476925286766560
#define M_PI_D 3.141592653589793238462643383280
static double cycloidal(double v)
{
    if (v >= 0.0)
        return sin((double)((v - floor(v)) * 50000.0) / 50000.0 * TWO_M_PI);
    return 0.0 - sin((double)((0.0 - (v + floor(0.0 - v))) * 50000.0) / 50000.0 * TWO_M_PI);
}

static double triangle_wave(double v)
{
    double off = v >= 0.0 ? v - floor(v) : v + 1.0 + floor(fabs(v));
    return off >= 0.5 ? 2.0 * (1.0 - off) : 2.0 * off;
}

/* Compute_Pigment for a pattern pigment (pigment.cpp:395-475): the point
 * through the pattern's inverse TRANSFORM (Warp_EPoint, warp.cpp:103-122),
 * the pattern value, the colour map (BlendMap::Search, pattern.cpp:
 * 1068-1109, linear blend). */
/* Warp_EPoint (warp.cpp:103-122): the pattern's inverse TRANSFORM, then
 * the classic turbulence, then COORDINATE_LIMIT. */
static V3 pattern_warp(const PovGpuPattern* pt, V3 P)
{
    const double* m = pt->inverse;
    double q[3];
    for (int i = 0; i < 3; i++)
        q[i] = P.x * m[0 * 4 + i] + P.y * m[1 * 4 + i] + P.z * m[2 * 4 + i] + m[3 * 4 + i];
    V3 T = v3(q[0], q[1], q[2]);
    /* the classic turbulence warp, applied after the transform (the parser
     * keeps it first in the warp list, Warp_EPoint walks the list backwards) */
    if (pt->has_turbulence) {
        const V3 d = pov_dturbulence(T, pt);
        T = v3(T.x + d.x * pt->turbulence[0], T.y + d.y * pt->turbulence[1], T.z + d.z * pt->turbulence[2]);
    }
    {
        double* c3[3] = {&T.x, &T.y, &T.z};
        for (int i = 0; i < 3; i++) {   /* COORDINATE_LIMIT */
            if (*c3[i] > 1.0e17) *c3[i] = 1.0e17;
            if (*c3[i] < -1.0e17) *c3[i] = -1.0e17;
        }
    }
    return T;
}

/* Evaluate_TPat of a warped point T: the pattern's value with its
 * frequency, phase and wave (ContinuousPattern::Evaluate,
 * pattern.cpp:354-390). */
static double pattern_value(const PovGpuPattern* pt, V3 T)
{
    const int gen = pt->noise_generator;
    double value;
    if (pt->type == POV_PATTERN_CHECKER) {   /* CheckerPattern::Evaluate, pattern.cpp:5691-5706 */
        int c = (int)(floor(T.x + EPSILON) + floor(T.y + EPSILON) + floor(T.z + EPSILON));
        value = (c & 1) ? 1.0 : 0.0;
    } else if (pt->type == POV_PATTERN_SQUARE) {   /* pattern.cpp:6740-6770 */
        const int vx = (int)floor(T.x), vz = (int)floor(T.z);
        value = (vx & 1) ? ((vz & 1) ? 2.0 : 3.0) : ((vz & 1) ? 1.0 : 0.0);
    } else if (pt->type == POV_PATTERN_CUBIC) {    /* pattern.cpp:6699-6714 */
        const double x = T.x, y = T.y, z = T.z, ax = fabs(x), ay = fabs(y), az = fabs(z);
        if (x >= 0 && x >= ay && x >= az) value = 0.0;
        else if (y >= 0 && y >= ax && y >= az) value = 1.0;
        else if (z >= 0 && z >= ax && z >= ay) value = 2.0;
        else if (x < 0 && x <= -ay && x <= -az) value = 3.0;
        else if (y < 0 && y <= -ax && y <= -az) value = 4.0;
        else value = 5.0;
    } else if (pt->type == POV_PATTERN_HEXAGON) {   /* pattern.cpp:6512-6655 */
        /* the colour of each block of the 6 x 6 grid, by zm: blocks 0/5 and
         * 2/3 of xm whole, 1/4 split on the diagonal */
        static const int even[6] = {0, 1, 1, 2, 2, 0}, mid[6] = {2, 2, 0, 0, 1, 1};
        static const int below[6] = {0, 2, 1, 0, 2, 1}, above[6] = {2, 1, 0, 2, 1, 0};
        const double x = fabs(T.x);
        const double z = T.z < 0.0 ? 5.196152424 - fabs(T.z) : T.z;
        double xs = x / 0.5, zs = z / 0.866025404;
        xs -= floor(xs / 6.0) * 6.0;
        zs -= floor(zs / 6.0) * 6.0;
        const int xm = (int)floor(xs) % 6, zm = (int)floor(zs) % 6;
        value = 0.0;
        if (zm >= 0 && zm < 6) {
            if (xm == 0 || xm == 5) {
                value = even[zm];
            } else if (xm == 2 || xm == 3) {
                value = mid[zm];
            } else if (xm == 1 || xm == 4) {
                double xl = xs - xm;
                const double zl = zs - zm;
                if (((xm + zm) % 2) == 1)
                    xl = 1.0 - xl;
                if (xl == 0.0)
                    xl = 0.0001;
                value = (zl / xl) < 1.0 ? below[zm] : above[zm];
            }
        }
        value = fmod(value, 3.0);
    } else if (pt->type == POV_PATTERN_BRICK) {
        value = brick_value(pt, T);
    } else if (pt->type == POV_PATTERN_TRIANGULAR) {   /* pattern.cpp:6799-6866 */
        const double SQ3 = 1.7320508075688772935274463415059, SQ3_2 = 0.86602540378443864676372317075294;
        double xs = T.x - 3.0 * floor(T.x / 3.0);
        double zs = T.z - SQ3 * floor(T.z / SQ3);
        const int a = (int)floor(xs);
        xs -= a;
        const int b = zs < SQ3_2 ? 0 : 1;
        if (b)
            zs = SQ3 - zs;
        const double k = 1.0 - xs;
        double ans = 1.0;
        if (xs != 0.0 && k != 0.0) {
            const double s1 = zs / xs, s2 = zs / k;
            const int c = (s1 < SQ3 ? 1 : 0) + (s2 < SQ3 ? 2 : 0);
            ans = c == 3 ? 0.0 : (c == 2 ? 1.0 : 3.0);
        }
        const int mask = (int)ans;
        ans = (mask & 1) ? fmod(ans + 2.0 * a, 6.0) : fmod(6.0 + ans - 2.0 * a, 6.0);
        if (b)
            ans = 5.0 - ans;
        value = ans;
    } else {
        switch (pt->type) {
        case POV_PATTERN_GRADIENT:   /* pattern.cpp:6386-6393 */
            value = T.x * pt->gradient[0] + T.y * pt->gradient[1] + T.z * pt->gradient[2];
            if (value > 1.0)
                value = fmod(value, 1.0);
            break;
        case POV_PATTERN_BOZO:   /* NoisePattern, pattern.cpp:7858-7861 */
            value = pov_noise(T, gen);
            break;
        case POV_PATTERN_GRANITE: {   /* pattern.cpp:6429-6465 */
            value = 0.0;
            double freq = 1.0;
            const V3 t1 = vmul(T, 4.0);
            for (int i = 0; i < 6; freq *= 2.0, i++) {
                double tmp;
                if (gen == 1) {
                    tmp = fabs(0.5 - pov_noise(vmul(t1, freq), 1));
                } else {
                    tmp = fabs(1.0 - 2.0 * pov_noise(vmul(t1, freq), gen));
                    if (tmp > 0.5)
                        tmp = 0.5;
                }
                value += tmp / freq;
            }
            break;
        }
        case POV_PATTERN_MARBLE:   /* pattern.cpp:7831-7850 */
            value = T.x + (pt->has_turbulence ? pt->turbulence[0] * pov_turbulence(T, pt, gen) : 0.0);
            break;
        case POV_PATTERN_WOOD: {   /* pattern.cpp:8651-8680 */
            double px = 0.0, py = 0.0;
            if (pt->has_turbulence) {
                const V3 wt = pov_dturbulence(T, pt);
                px = cycloidal((T.x + wt.x) * pt->turbulence[0]);
                py = cycloidal((T.y + wt.y) * pt->turbulence[1]);
            }
            px += T.x;
            py += T.y;
            value = sqrt(px * px + py * py + 0.0 * 0.0);
            break;
        }
        case POV_PATTERN_AGATE: {   /* pattern.cpp:5396-5418 */
            const double tv = (double)(float)pt->agate_turb * pov_turbulence(T, pt, gen);   /* SNGL agateTurbScale */
            value = 0.5 * (cycloidal(1.3 * tv + 1.1 * T.z) + 1.0);
            if (value < 0.0) {
                value = 0.0;
            } else {
                value = value < 1.0 ? value : 1.0;
                value = pow(value, 0.77);
            }
            break;
        }
        case POV_PATTERN_RIPPLES: {   /* RipplesPattern::EvaluateRaw, pattern.cpp:8163-8186 */
            const double fr = (float)pt->frequency, ph = (float)pt->phase;
            double sc = 0.0;
            for (int i = 0; i < NUM_WAVES; i++) {
                double len = vlen(vsub(T, g_wave_src[i]));
                if (len == 0.0)
                    len = 1.0;
                sc += cycloidal(len * fr + ph);
            }
            value = 0.5 * (1.0 + (sc / (double)NUM_WAVES));
            break;
        }
        case POV_PATTERN_WAVES: {     /* WavesPattern::EvaluateRaw, pattern.cpp:8593-8618 */
            const double fr = (float)pt->frequency, ph = (float)pt->phase;
            double sc = 0.0;
            for (int i = 0; i < NUM_WAVES; i++) {
                double len = vlen(vsub(T, g_wave_src[i]));
                if (len == 0.0)
                    len = 1.0;
                sc += cycloidal(len * fr * g_wave_freq[i] + ph) / g_wave_freq[i];
            }
            value = 0.2 * (2.5 + (sc / (double)NUM_WAVES));
            break;
        }
        case POV_PATTERN_DENTS: {   /* DentsPattern::EvaluateRaw, pattern.cpp:6307-6313 */
            const double nz = pov_noise(T, gen);
            value = nz * nz * nz;
            break;
        }
        case POV_PATTERN_WRINKLES: {   /* WrinklesPattern::EvaluateRaw, pattern.cpp:8720-8770 */
            double lambda = 2.0, omega = 0.5;
            if (gen == 1) {
                value = pov_noise(T, 1);
            } else {
                const double nz = pov_noise(T, gen) * 2.0 - 0.5;
                value = fmin(fmax(nz, 0.0), 1.0);
            }
            for (int i = 1; i < 10; i++) {
                const V3 q = vmul(T, lambda);
                if (gen == 1) {
                    value += omega * pov_noise(q, 1);
                } else {
                    const double nz = pov_noise(q, gen) * 2.0 - 0.5;
                    value += omega * fmin(fmax(nz, 0.0), 1.0);
                }
                lambda *= 2.0;
                omega *= 0.5;
            }
            value = value / 2.0;
            break;
        }
        case POV_PATTERN_RADIAL:   /* pattern.cpp:8115-8128 */
            if (fabs(T.x) < 0.001 && fabs(T.z) < 0.001)
                value = 0.25;
            else
                value = 0.25 + (atan2(T.x, T.z) + M_PI_D) / TWO_M_PI;
            break;
        case POV_PATTERN_PLANAR:        /* pattern.cpp:8024-8030 */
        case POV_PATTERN_SPHERICAL:     /* pattern.cpp:8551-8558 */
        case POV_PATTERN_CYLINDRICAL:   /* pattern.cpp:6025-6032 */
        case POV_PATTERN_BOXED:         /* pattern.cpp:5454-5461 */
            if (pt->type == POV_PATTERN_PLANAR)
                value = fabs(T.y);
            else if (pt->type == POV_PATTERN_SPHERICAL)
                value = vlen(T);
            else if (pt->type == POV_PATTERN_CYLINDRICAL)
                value = sqrt(T.x * T.x + T.z * T.z);
            else
                value = fmax(fabs(T.x), fmax(fabs(T.y), fabs(T.z)));
            /* CLIP_DENSITY (pattern.cpp:85) */
            value = value < 0.0 ? 1.0 : (value > 1.0 ? 0.0 : 1.0 - value);
            break;
        case POV_PATTERN_ONION:   /* pattern.cpp:7934-7952 */
            value = fmod(sqrt(T.x * T.x + T.y * T.y + T.z * T.z), 1.0);
            break;
        case POV_PATTERN_SPIRAL1:   /* pattern.cpp:8396-8437 */
        case POV_PATTERN_SPIRAL2: { /* pattern.cpp:8473-8515 */
            const double turb = pt->has_turbulence ? pt->turbulence[0] * pov_turbulence(T, pt, gen) : 0.0;
            const double rad = sqrt(T.x * T.x + T.y * T.y);
            double phi = 0.0;   /* the angle about the z axis, 0 .. 2 pi */
            if (rad != 0.0)
                phi = T.x < 0.0 ? 3.0 * (M_PI_D / 2.0) - asin(T.y / rad) : (M_PI_D / 2.0) + asin(T.y / rad);
            const double arm = T.z + rad + (double)pt->arms * phi / TWO_M_PI + turb;
            value = pt->type == POV_PATTERN_SPIRAL1 ? arm : triangle_wave(rad) + triangle_wave(arm);
            break;
        }
        case POV_PATTERN_CRACKLE:
            value = crackle_value(pt, T);
            break;
        case POV_PATTERN_QUILTED:
            value = quilted_value(pt, T);
            break;
        case POV_PATTERN_CELLS:   /* pattern.cpp:5652-5660 */
            pthread_once(&g_prand_once, prand_init);
            value = fmin(g_prand[hash3d((int)floor(T.x + EPSILON), (int)floor(T.y + EPSILON),
                                        (int)floor(T.z + EPSILON))],
                         1.0);
            break;
        default: {   /* leopard, pattern.cpp:7179-7194 */
            const double t1 = sin(T.x), t2 = sin(T.y), t3 = sin(T.z);
            const double v = (t1 + t2 + t3) / 3.0;
            value = v * v;
            break;
        }
        }
        /* ContinuousPattern::Evaluate (pattern.cpp:354-390): frequency and
         * phase, then the wave */
        /* waveFrequency, wavePhase and waveExponent are single precision */
        if ((float)pt->frequency != 0.0f)
            value = fmod(value * (double)(float)pt->frequency + (double)(float)pt->phase, 1.00001);
        if (value < 0.0)
            value -= floor(value);
        switch (pt->wave_type) {
        case POV_WAVE_SINE: value = (1.0 + cycloidal(value)) * 0.5; break;
        case POV_WAVE_TRIANGLE: value = triangle_wave(value); break;
        case POV_WAVE_SCALLOP: value = fabs(cycloidal(value * 0.5)); break;
        case POV_WAVE_CUBIC: value = value * value * ((-2.0 * value) + 3.0); break;
        case POV_WAVE_POLY: value = pow(value, (double)(float)pt->exponent); break;
        default: break;
        }
    }
    return value;
}

/* The colour map at the pattern's value (BlendMap::Search and the linear
 * blend, pattern.cpp:1068-1109): rgb, and through `ft` (when given) the
 * entry's filter and transmit blended the same way. */
static RGB pattern_pigment_ft(const PovGpuPattern* pt, V3 P, float ft[2])
{
    const double value = pattern_value(pt, pattern_warp(pt, P));
    const int n = pt->num_entries;
    RGB c;
    int ip = 0, in = 0;
    if (value >= pt->values[n - 1]) {
        ip = in = n - 1;
    } else {
        while (value > pt->values[in]) {
            ip = in;
            in++;
        }
        if (value == pt->values[in])
            ip = in;
    }
    if (ip == in) {
        c.r = pt->colours[in][0]; c.g = pt->colours[in][1]; c.b = pt->colours[in][2];
        if (ft) {
            ft[0] = pt->filters[in];
            ft[1] = pt->transmits[in];
        }
        return c;
    }
    const double pw = ((double)pt->values[in] - value) / ((double)pt->values[in] - (double)pt->values[ip]);
    const float wp = (float)pw, wn = (float)(1.0 - pw);
    c.r = pt->colours[ip][0] * wp + pt->colours[in][0] * wn;
    c.g = pt->colours[ip][1] * wp + pt->colours[in][1] * wn;
    c.b = pt->colours[ip][2] * wp + pt->colours[in][2] * wn;
    if (ft) {
        ft[0] = pt->filters[ip] * wp + pt->filters[in] * wn;
        ft[1] = pt->transmits[ip] * wp + pt->transmits[in] * wn;
    }
    return c;
}

static RGB pattern_pigment(const PovGpuPattern* pt, V3 P) { return pattern_pigment_ft(pt, P, NULL); }

/* a colour map with an entry that filters or transmits (HAS_FILTER) */
static int pattern_transparent(const PovGpuPattern* pt)
{
    for (int k = 0; k < pt->num_entries; k++)
        if (pt->filters[k] != 0.0f || pt->transmits[k] != 0.0f)
            return 1;
    return 0;
}

/* MInvTransNormal (matrix.cpp:495-508): temp[i] = v . M[i][0..2]; with the
 * forward matrix it takes a normal into the pattern's space (Warp_Normal,
 * TransformWarp::WarpNormal, warp.cpp:582-586), with the inverse back out
 * (UnWarp_Normal, TransformWarp::UnwarpNormal, warp.cpp:622-626). */
static V3 normal_through(const double* m, V3 v)
{
    return v3(v.x * m[0] + v.y * m[1] + v.z * m[2], v.x * m[4] + v.y * m[5] + v.z * m[6],
              v.x * m[8] + v.y * m[9] + v.z * m[10]);
}

/* The four pyramid directions of the slope sampling (normal.cpp:88-91). */
static const double kPyramid[4][3] = {{0.942809041, -0.333333333, 0.0},
                                      {-0.471404521, -0.333333333, 0.816496581},
                                      {-0.471404521, -0.333333333, -0.816496581},
                                      {0.0, 1.0, 0.0}};

/* The layer normal of a textured hit (trace.cpp:812-832): Perturb_Normal
 * (normal.cpp:784-905) of the raw normal N at world point P, normalised
 * afterwards under no_bump_scale. */
static V3 perturb_normal(const PovGpuNormal* nm, const PovGpuPattern* pt, V3 P, V3 N)
{
    const int scale = !nm->dont_scale_bumps;
    /* Warp_Normal (warp.cpp:563-580): normalise, the TRANSFORM, normalise */
    if (scale)
        N = vnorm(N);
    N = normal_through(nm->matrix, N);
    if (scale)
        N = vnorm(N);
    const V3 T = pattern_warp(pt, P);
    const double amount = (double)nm->amount;
    switch (pt->type) {
    case POV_PATTERN_BUMPS:   /* bumps, normal.cpp:235-246 */
        N = vadd(N, vmul(pov_dnoise(T), amount));
        break;
    case POV_PATTERN_DENTS: {  /* dents, normal.cpp:272-288 */
        double v = pov_noise(T, pt->noise_generator);
        v = v * v * v * amount;
        N = vadd(N, vmul(pov_dnoise(T), v));
        break;
    }
    case POV_PATTERN_WRINKLES: {  /* wrinkles, normal.cpp:325-346 */
        double r[3] = {0.0, 0.0, 0.0};
        double sc = 1.0;
        for (int i = 0; i < 10; sc *= 2.0, i++) {
            const V3 d = pov_dnoise(vmul(T, sc));
            r[0] += fabs(d.x / sc);
            r[1] += fabs(d.y / sc);
            r[2] += fabs(d.z / sc);
        }
        N = vadd(N, vmul(v3(r[0], r[1], r[2]), amount));
        break;
    }
    case POV_PATTERN_RIPPLES:    /* ripples, normal.cpp:130-155 */
    case POV_PATTERN_WAVES: {    /* waves, normal.cpp:180-206 */
        const double fr = (float)pt->frequency, ph = (float)pt->phase;
        for (int i = 0; i < NUM_WAVES; i++) {
            const V3 d = vsub(T, g_wave_src[i]);
            double len = vlen(d);
            if (len == 0.0)
                len = 1.0;
            double sc;
            if (pt->type == POV_PATTERN_RIPPLES)
                sc = cycloidal(len * fr + ph) * amount;
            else
                sc = cycloidal(len * fr * g_wave_freq[i] + ph) * amount / g_wave_freq[i];
            N = vadd(N, vmul(d, sc / (len * (double)NUM_WAVES)));
        }
        break;
    }
    default: {  /* the slope of a continuous pattern, normal.cpp:880-902 */
        const double delta = (double)nm->delta;
        const double a = amount * -5.0 * (0.02 / delta);
        for (int i = 0; i < 4; i++) {
            const V3 d = v3(kPyramid[i][0], kPyramid[i][1], kPyramid[i][2]);
            const double v = pattern_value(pt, vadd(T, vmul(d, delta)));
            N = vadd(N, vmul(d, v * a));
        }
        break;
    }
    }
    /* UnWarp_Normal (warp.cpp:603-620) */
    if (scale)
        N = vnorm(N);
    N = normal_through(pt->inverse, N);
    /* UnWarp_Normal's last normalisation; under no_bump_scale the one of
     * trace.cpp:821-822 */
    return vnorm(N);
}

/* Material of an object: its own, else the nearest CSG ancestor's. */
static const PovGpuMaterial* object_material(const PovOracle* S, int32_t oi)
{
    while (oi >= 0) {
        if (S->objs[oi].o.material >= 0)
            return &S->mats[S->objs[oi].o.material];
        oi = S->objs[oi].o.parent;
    }
    return &S->mats[0];
}

static inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Media container: a hollow object whose interior holds media; its surface
 * transmits fully (validated at create).  Returns the media index, -1 for
 * any other object. */
static int container_media(const PovOracle* S, int32_t oi)
{
    const PovGpuObject* o = &S->objs[oi].o;
    return (o->media > 0 && (o->flags & POV_FLAG_HOLLOW)) ? o->media - 1 : -1;
}

/* Transparent surfaces.  TransColour::TransmittedColour (colour.h:1912):
 * pigment * filter + transmit, in float. */
static void transmitted_colour(const float pig[3], float filt, float trm, float out[3])
{
    for (int k = 0; k < 3; k++)
        out[k] = pig[k] * filt + trm;
}

/* a material that can filter or transmit: its plain pigment, or an entry
 * of its pattern's colour map */
static int material_transparent(const PovGpuSceneDesc* d, const PovGpuMaterial* m)
{
    if (m->pattern > 0)
        return pattern_transparent(&d->patterns[m->pattern - 1]);
    return m->pigment[3] != 0.0f || m->pigment[4] != 0.0f;
}

/* the pigment at P with its filter and transmit (the plain pigment's, or
 * the colour map's there) */
static RGB material_pigment(const PovOracle* S, const PovGpuMaterial* m, V3 P, float* filt, float* trm)
{
    RGB c = {m->pigment[0], m->pigment[1], m->pigment[2]};
    *filt = m->pigment[3];
    *trm = m->pigment[4];
    if (m->pattern > 0) {
        float ft[2];
        c = pattern_pigment_ft(&S->desc.patterns[m->pattern - 1], P, ft);
        *filt = ft[0];
        *trm = ft[1];
    }
    return c;
}

/* Object::IsOpaque (OPAQUE_FLAG, parser.cpp:9296-9297): a leaf whose plain
 * pigment neither filters nor transmits; a CSG whose children all are. */
static int object_opaque(const PovOracle* S, int32_t oi)
{
    const PovGpuObject* o = &S->objs[oi].o;
    if (o->type >= POV_OBJ_UNION) {
        for (int c = 0; c < o->num_children; c++)
            if (!object_opaque(S, o->first_child + c))
                return 0;
        return 1;
    }
    return !material_transparent(&S->desc, object_material(S, oi));
}

/* Ray::IsInterior: the current ray's interior list holds `id`. */
static int ray_inside(const Thread* th, int id)
{
    for (int i = 0; i < th->nrin; i++)
        if (th->rin[i] == id)
            return 1;
    return 0;
}

static int top_ancestor(const PovOracle* S, int32_t oi)
{
    while (S->objs[oi].o.parent >= 0)
        oi = S->objs[oi].o.parent;
    return oi;
}

/* Ray flags: the medium a ray travels in (the object id of its media
 * container, the reference's interior list, which containers that do not
 * overlap keep at one entry) rides in bits 8 and up. */
#define RAY_MEDIUM(f)      (((f) >> 8) - 1)
#define WITH_MEDIUM(f, m)  (((f) & 0xff) | (((m) + 1) << 8))

/* Trace::TraceShadowRay / TracePointLightShadowRay (trace.cpp:1892-2076)
 * for opaque objects and media containers: 1 = light blocked.  A container
 * wall is a transparent hit (a test and a success of its own, trace.cpp:
 * 2032-2072): ComputeShadowColour passes the light through it, attenuated by
 * the media of the segment the ray has crossed inside (trace.cpp:2429-2433;
 * for a shadow ray the constant media is one interval, od = extinction *
 * depth), and ComputeShadowMedia toggles the ray's interior
 * (trace.cpp:3064-3066); the ray then continues from the wall. */
static int shadow_trace(const PovOracle* S, Thread* th, V3 P, V3 L, double dist, int medium, int media_on,
                        double lc[3])
{
    const double shadow_adc = S->desc.adc_bailout;
    /* the shadow ray's own interior list (Ray lightsourceray(eye)): a copy
     * of the eye ray's, toggled at every transparent surface it passes
     * (ComputeShadowMedia, trace.cpp:3065-3068) */
    int rin[MAX_RIN], nrin = th->nrin;
    memcpy(rin, th->rin, sizeof(int) * (size_t)nrin);
    V3 O = P;
    double depth = dist;
    for (;;) {
        Isect is;
        th->shadow_tests++;   /* Shadow_Ray_Tests (trace.cpp:2032) */
        if (!find_intersection(S, th, O, L, depth, 1, &is) || !(is.depth < depth - SHADOW_TOLERANCE) ||
            !(is.depth > SHADOW_TOLERANCE))
            return 0;
        th->shadow_succeeded++;
        int mi = container_media(S, is.object);
        if (mi < 0 && !S->transparent)
            return 1;
        if (mi < 0) {
            /* ComputeShadowColour (trace.cpp:2274-2439) for plain textures:
             * an opaque surface clears the light; a transparent one filters
             * it by its TransmittedColour and, when the ray is inside the
             * object's interior, its fade (ComputeShadowTexture,
             * trace.cpp:1180-1250); below ADC_Bailout the light is cleared
             * (trace.cpp:2412-2417).  The ray goes on unless the light is
             * gone and the object (the CSG it belongs to) is opaque
             * (TracePointLightShadowRay, trace.cpp:2040-2072). */
            const PovGpuMaterial* m = object_material(S, is.object);
            float filt, trm;
            const RGB pc = material_pigment(S, m, is.ipoint, &filt, &trm);
            if (filt == 0.0f && trm == 0.0f) {
                lc[0] = lc[1] = lc[2] = 0.0;
            } else {
                float pig[3] = {pc.r, pc.g, pc.b}, fc[3];
                transmitted_colour(pig, filt, trm, fc);
                const int id = S->obj_int[is.object];
                const PovGpuInterior* I = &S->ints[id];
                int in = -1;
                for (int k = 0; k < nrin; k++)
                    if (rin[k] == id) { in = k; break; }
                if (in >= 0 && I->fade_power > 0.0 && fabs(I->fade_distance) > EPSILON) {
                    for (int k = 0; k < 3; k++) {
                        if (I->fade_power >= 1000.0)
                            fc[k] = (float)(fc[k] * exp(-(1.0 - I->fade_colour[k]) * (is.depth / I->fade_distance)));
                        else
                            fc[k] = (float)(fc[k] * (I->fade_colour[k] + (1.0 - I->fade_colour[k]) /
                                                     (1.0 + pow(is.depth / I->fade_distance, I->fade_power))));
                    }
                }
                if (fabs((double)((fabsf(fc[0]) + fabsf(fc[1]) + fabsf(fc[2])) / 3.0)) < shadow_adc) {
                    lc[0] = lc[1] = lc[2] = 0.0;
                } else {
                    for (int k = 0; k < 3; k++)
                        lc[k] = (float)((float)lc[k] * fc[k]);
                    if (!(fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON)) {
                        if (in >= 0) {   /* leaving: removed */
                            for (int k = in; k + 1 < nrin; k++)
                                rin[k] = rin[k + 1];
                            nrin--;
                        } else if (nrin < MAX_RIN) {   /* entering: appended */
                            rin[nrin++] = id;
                        }
                    }
                }
            }
            if (fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON &&
                object_opaque(S, top_ancestor(S, is.object)))
                return 1;
            depth -= is.depth;
            O = is.ipoint;
            continue;
        }
        if (medium >= 0 && media_on) {
            th->media_samples++;   /* the shadow ray's one media sample (media.cpp:384-398) */
            const PovGpuMedia* md = &S->desc.medias[container_media(S, medium)];
            for (int k = 0; k < 3; k++)
                lc[k] *= exp(-md->extinction[k] * is.depth);
        }
        medium = (medium == is.object) ? -1 : is.object;
        depth -= is.depth;
        O = is.ipoint;
    }
}

static int shadow_blocked(const PovOracle* S, Thread* th, V3 P, V3 L, double dist)
{
    double lc[3] = {1.0, 1.0, 1.0};
    return shadow_trace(S, th, P, L, dist, -1, 0, lc);
}

/* Grid point (u, v) of an area light as an offset from its centre
 * (TraceAreaLightSubsetShadowRay, trace.cpp:2166-2205; no jitter). */
static V3 area_offset(const PovGpuLight* L, V3 a1, V3 a2, int u, int v)
{
    double ju = u, jv = v;
    if (L->circular) {
        ju = ju / (L->area_size1 - 1) - 0.5 + 0.001;
        jv = jv / (L->area_size2 - 1) - 0.5 + 0.001;
        double sc = fabs(ju) > fabs(jv) ? fabs(ju) : fabs(jv);
        sc /= sqrt(ju * ju + jv * jv);
        return vadd(vmul(a1, ju * sc), vmul(a2, jv * sc));
    }
    V3 j1 = v3(0.0, 0.0, 0.0), j2 = v3(0.0, 0.0, 0.0);
    if (L->area_size1 > 1)
        j1 = vmul(a1, ju / (double)(L->area_size1 - 1) - 0.5);
    if (L->area_size2 > 1)
        j2 = vmul(a2, jv / (double)(L->area_size2 - 1) - 0.5);
    return vadd(j1, j2);
}

/* TraceAreaLightSubsetShadowRay (trace.cpp:2131-2272) for opaque scenes:
 * the fraction of the light colour that reaches P from the grid region
 * [u1,u2]x[v1,v2].  grid[u*size2+v]: -1 not traced yet (lightGrid's
 * Invalidate), 1 visible, 0 blocked.  A sample colour is the light colour
 * or black, so two corners differ in ColourDistance by |r|+|g|+|b| of the
 * light colour (float SumAbs) or not at all. */
static double area_subset(const PovOracle* S, Thread* th, const PovGpuLight* L, V3 P, V3 a1, V3 a2,
                          signed char* grid, int u1, int v1, int u2, int v2, int level, float lc_dist)
{
    double s[4];
    for (int i = 0; i < 4; i++) {
        int u = (i & 1) ? u2 : u1;
        int v = (i & 2) ? v2 : v1;
        signed char* g = &grid[u * L->area_size2 + v];
        if (*g < 0) {
            V3 C = vadd(vload(L->center), area_offset(L, a1, a2, u, v));
            V3 ld = vsub(C, P);
            double depth = vlen(ld);
            ld = vdiv(ld, depth);
            *g = shadow_blocked(S, th, P, ld, depth) ? 0 : 1;
        }
        s[i] = *g;
    }
    if (u2 - u1 > 1 || v2 - v1 > 1) {
        int differ = s[0] != s[1] || s[1] != s[3] || s[3] != s[2] || s[2] != s[0];
        if (level < L->adaptive_level || (differ && lc_dist > 0.1)) {
            int mu0 = (int)floor((u1 + u2) / 2.0), mu1 = (int)ceil((u1 + u2) / 2.0);
            int mv0 = (int)floor((v1 + v2) / 2.0), mv1 = (int)ceil((v1 + v2) / 2.0);
            s[0] = area_subset(S, th, L, P, a1, a2, grid, u1, v1, mu0, mv0, level + 1, lc_dist);
            s[1] = area_subset(S, th, L, P, a1, a2, grid, mu1, v1, u2, mv0, level + 1, lc_dist);
            s[2] = area_subset(S, th, L, P, a1, a2, grid, u1, mv1, mu0, v2, level + 1, lc_dist);
            s[3] = area_subset(S, th, L, P, a1, a2, grid, mu1, mv1, u2, v2, level + 1, lc_dist);
        }
    }
    return (s[0] + s[1] + s[2] + s[3]) * 0.25;
}

/* LightSource::Direction (parser.cpp:3521-3528): points_at - center, unit
 * length unless shorter than EPSILON. */
static V3 light_direction(const PovGpuLight* L)
{
    V3 d = vsub(vload(L->points_at), vload(L->center));
    double len = vlen(d);
    return len > EPSILON ? vdiv(d, len) : d;
}

/* ComputeOneWhiteLightRay (trace.cpp:2710-2766) without jitter: the unit
 * direction from P towards the light and the distance along it.  A
 * cylinder light's rays run parallel to its axis, their length the
 * projection of P's offset on it; a parallel light's rays all take the
 * light's direction, reversed, their length scaled by the cosine. */
static void light_ray(const PovGpuLight* L, V3 P, V3* dir, double* depth)
{
    V3 C = vload(L->center);
    if (L->light_type == POV_LIGHT_TYPE_CYLINDER) {
        V3 d = vsub(C, vload(L->points_at));
        double len = vlen(d);
        *depth = vdot(vsub(C, P), d) / len;
        *dir = vnorm(d);
    } else {
        V3 d = vsub(C, P);
        *depth = vlen(d);
        *dir = vdiv(d, *depth);
    }
    if (L->parallel) {
        V3 ldir = light_direction(L);
        *depth *= -vdot(ldir, *dir);
        *dir = vmul(ldir, -1.0);
    }
}

/* cubic_spline (lightsource.cpp:497-514). */
static double cubic_spline(double low, double high, double pos)
{
    if (pos < low)
        return 0.0;
    if (pos >= high)
        return 1.0;
    pos = (pos - low) / (high - low);
    return (3 - 2 * pos) * pos * pos;
}

/* Attenuate_Light (lightsource.cpp:544-632): a spotlight's cone, a cylinder
 * light's beam, then the fade with distance.  `P` is the light ray's
 * origin, `dir` and `depth` its direction and length. */
static double attenuate_light(const PovGpuLight* L, V3 P, V3 dir, double depth)
{
    double att = 1.0;
    if (L->light_type == POV_LIGHT_TYPE_SPOT) {
        double costheta = vdot(dir, light_direction(L));
        if (depth > 0.0)
            costheta = -costheta;
        if (costheta <= 0.0)
            return 0.0;
        att = pow(costheta, L->tightness);
        if (L->radius > 0.0 && costheta < L->radius)
            att *= cubic_spline(L->falloff, L->radius, costheta);
    } else if (L->light_type == POV_LIGHT_TYPE_CYLINDER) {
        V3 ldir = light_direction(L);
        V3 v1 = vsub(P, vload(L->center));
        double k = vdot(v1, ldir);
        if (k <= 0.0)
            return 0.0;
        double len = vlen(vsub(v1, vmul(ldir, k)));
        if (len >= L->falloff)
            return 0.0;
        double dist = 1.0 - len / L->falloff;
        att = pow(dist, L->tightness);
        if (L->radius > 0.0 && len > L->radius)
            att *= cubic_spline(0.0, 1.0 - L->radius / L->falloff, dist);
    }
    if (att > 0.0 && L->fade_power > 0.0) {
        if (fabs(L->fade_distance) >= EPSILON)
            att *= 2.0 / (1.0 + pow(depth / L->fade_distance, L->fade_power));
        else
            att *= pow(depth, -L->fade_power);
    }
    return att;
}

/* ComputeOneLightRay (trace.cpp:1873-1889): the light ray and the light's
 * colour attenuated along it (MathColour *= double: float channels). */
static void one_light_ray(const PovGpuLight* L, V3 P, V3* dir, double* depth, double lc[3])
{
    light_ray(L, P, dir, depth);
    const double att = attenuate_light(L, P, *dir, *depth);
    for (int k = 0; k < 3; k++)
        lc[k] = (float)(L->colour[k] * att);
}

/* TraceAreaLightShadowRay (trace.cpp:2078-2129): axes (oriented towards P
 * when `orient`), all grid points invalid, then the whole grid as one
 * region. */
static double area_light_fraction(const PovOracle* S, Thread* th, const PovGpuLight* L, V3 P, const double lc[3])
{
    signed char grid[AREA_MAX_POINTS];
    int npts = L->area_size1 * L->area_size2;
    for (int k = 0; k < npts; k++)
        grid[k] = -1;
    V3 a1 = vload(L->axis1), a2 = vload(L->axis2);
    if (L->orient) {
        V3 dir = vnorm(vsub(vload(L->center), P));
        double len1 = vlen(a1);
        V3 tmp = fabs(fabs(dir.z) - 1.0) < 0.01 ? v3(0.0, 1.0, 0.0) : v3(0.0, 0.0, 1.0);
        a1 = vnorm(vcross(dir, tmp));
        a2 = vnorm(vcross(dir, a1));
        a1 = vmul(a1, len1);
        a2 = vmul(a2, len1);
    }
    /* the samples are the attenuated light colour or black */
    float lc_dist = fabsf((float)lc[0]) + fabsf((float)lc[1]) + fabsf((float)lc[2]);
    return area_subset(S, th, L, P, a1, a2, grid, 0, 0, L->area_size1 - 1, L->area_size2 - 1, 0, lc_dist);
}

/* TraceTicket (source/core/render/ray.h): trace level, its limit, the ADC
 * bailout, radiosity bounce depth and sample quality. */
typedef struct {
    int    level;
    int    max_level;
    double adc;
    int    rad_depth;
    float  rad_quality;
} Ticket;

/* Ray kinds that change shading: radiosity sample rays skip highlights
 * (trace.cpp:1714).  Pretrace camera rays would skip direct light
 * (trace.cpp:1014-1015), but the renderer's default Radiosity_Vain_Pretrace
 * (view.cpp:759) clears their pretrace flag (radiositytask.cpp:76), so
 * they shade fully. */
#define RAY_RADIOSITY 2
#define RAY_CONTINUED 4   /* transmitted ray: TraceRay(continuedRay = true) */

static double trace_ray(const PovOracle* S, Thread* th, V3 O, V3 D, double weight, Ticket* tk, int flags, RGB* col);
static void compute_ambient(const PovOracle* S, Thread* th, V3 ip, V3 raw, V3 layer, double brilliance, float amb[3],
                            double weight, Ticket* tk);

/* ComputeReflection (trace.cpp:1264-1321). */
static void compute_reflection(const PovOracle* S, Thread* th, V3 ip, V3 D, V3 N, V3 raw, double weight,
                               Ticket* tk, int flags, RGB* col)
{
    double n = -2.0 * vdot(D, N);
    V3 nd = vadd(D, vmul(N, n));
    n = vdot(nd, raw);
    if (n < 0.0) {
        double n2 = vdot(nd, N);
        if (n2 < 0.0) {
            n = -2.0 * vdot(D, raw);
            nd = vadd(D, vmul(raw, n));
        } else {
            n *= -2.0;
            nd = vadd(nd, vmul(raw, n));
        }
    }
    nd = vnorm(nd);
    th->reflected++;
    trace_ray(S, th, ip, nd, weight, tk, flags & ~RAY_CONTINUED, col);   /* SetFlags(ReflectionRay, ray) */
}

/* ComputeRefraction / TraceRefractionRay (trace.cpp:1323-1486) through the
 * surface of object `oi` at `is`: the ray's interior list changes as the
 * reference changes it (entering: appended; leaving the innermost:
 * removed; leaving an overlap: removed with ior 1; entering within
 * another: appended), the ior ratio follows; equal iors trace the
 * continued ray (Transmitted_Rays_Traced, same trace level), otherwise
 * Heckbert's refraction, or on total internal reflection the mirror ray of
 * the unchanged ray (Internal_Reflected_Rays_Traced).  Returns 1 on total
 * internal reflection. */
static int compute_refraction(const PovOracle* S, Thread* th, const Isect* is, V3 D, V3 N, V3 raw, double weight,
                              Ticket* tk, int flags, RGB* out)
{
    const int id = S->obj_int[is->object];
    const PovGpuInterior* I = &S->ints[id];
    int saved[MAX_RIN];
    const int nsaved = th->nrin;
    memcpy(saved, th->rin, sizeof(int) * (size_t)nsaved);
    double ior;
    if (th->nrin == 0) {
        th->rin[th->nrin++] = id;
        ior = S->atm_ior / I->ior;
    } else if (th->rin[th->nrin - 1] == id) {
        th->nrin--;
        ior = th->nrin == 0 ? I->ior / S->atm_ior : I->ior / S->ints[th->rin[th->nrin - 1]].ior;
    } else {
        int found = -1;
        for (int i = 0; i < th->nrin; i++)
            if (th->rin[i] == id) { found = i; break; }
        if (found >= 0) {
            for (int i = found; i + 1 < th->nrin; i++)
                th->rin[i] = th->rin[i + 1];
            th->nrin--;
            ior = 1.0;
        } else {
            ior = S->ints[th->rin[th->nrin - 1]].ior / I->ior;
            if (th->nrin < MAX_RIN)
                th->rin[th->nrin++] = id;
        }
    }
    int tir = 0;
    if (fabs(ior - 1.0) < EPSILON) {
        th->transmitted++;   /* Transmitted_Rays_Traced */
        trace_ray(S, th, is->ipoint, D, weight, tk, flags | RAY_CONTINUED, out);
    } else {
        double n = vdot(D, N);
        V3 ln = N;
        if (n <= 0.0)
            n = -n;
        else
            ln = vmul(N, -1.0);
        double t = 1.0 + ior * ior * (n * n - 1.0);
        if (t < 0.0) {
            th->internal_reflected++;   /* Internal_Reflected_Rays_Traced */
            th->nrin = nsaved;          /* the mirror ray keeps the incoming ray's interiors */
            memcpy(th->rin, saved, sizeof(int) * (size_t)nsaved);
            compute_reflection(S, th, is->ipoint, D, N, raw, weight, tk, flags, out);
            tir = 1;
        } else {
            t = ior * n - sqrt(t);
            V3 nd = vadd(vmul(D, ior), vmul(ln, t));
            th->refracted++;   /* Refracted_Rays_Traced */
            trace_ray(S, th, is->ipoint, nd, weight, tk, flags & ~RAY_CONTINUED, out);
        }
    }
    th->nrin = nsaved;
    memcpy(th->rin, saved, sizeof(int) * (size_t)nsaved);
    return tir;
}

/* Trace::ComputeRelativeIOR (trace.cpp:2595-2625): the ratio of iors the
 * ray sees at a surface of interior `id`, from the ray's interior list. */
static double relative_ior(const PovOracle* S, const Thread* th, int id)
{
    const double ior = S->ints[id].ior;
    if (th->nrin == 0)
        return ior / S->atm_ior;   /* entering from the atmosphere */
    if (ray_inside(th, id))
        return th->nrin == 1 ? S->atm_ior / ior : S->ints[th->rin[th->nrin - 1]].ior / ior;
    return ior / S->ints[th->rin[th->nrin - 1]].ior;
}

/* Trace::FresnelR (trace.cpp:2679-2707): the unpolarised Fresnel
 * reflectance for the cosine of incidence and the relative ior. */
static double fresnel_r(double cos_ti, double n)
{
    const double sqrg = n * n + cos_ti * cos_ti - 1.0;
    if (sqrg <= 0.0)
        return 1.0;   /* total reflection */
    const double g = sqrt(sqrg);
    const double q1 = (g - cos_ti) / (g + cos_ti);
    const double q2 = (cos_ti * (g + cos_ti) - 1.0) / (cos_ti * (g - cos_ti) + 1.0);
    const double f = 0.5 * q1 * q1 * (1.0 + q2 * q2);
    return f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
}

/* ComputeMetallic (trace.cpp:2658-2671): colour c moved towards the
 * pigment by `metallic`, less towards grazing angles (float channels). */
static void compute_metallic(float c[3], double metallic, RGB pig, double cos_angle)
{
    if (metallic == 0.0)
        return;
    const double x = fabs(acos(cos_angle)) / (M_PI_D / 2.0);
    double F = 0.014567225 / ((x - 1.12) * (x - 1.12)) - 0.011612903;
    F = fmin(1.0, fmax(0.0, F));
    const double k = metallic * (1.0 - F);
    const float p[3] = {pig.r, pig.g, pig.b};
    for (int i = 0; i < 3; i++)
        c[i] *= (float)(1.0 + (float)((float)(p[i] - 1.0) * k));
}

/* ComputeTextureColour + ComputeLightedTexture (trace.cpp:457-586,739-1179)
 * for one plain layer; a pigment that filters or transmits gives its own
 * light scaled by its opacity and passes the transmitted ray's colour
 * through its filter colour. */
static void shade(const PovOracle* S, Thread* th, const Isect* is, V3 D, double weight, Ticket* tk, int flags,
                  RGB* out)
{
    const int level = tk->level;
    const int radiosity = S->desc.radiosity.enabled;
    if (container_media(S, is->object) >= 0) {
        /* a media container's surface only transmits (all of its finish
         * terms are zero): ComputeRefraction with equal iors traces the
         * continued ray (trace.cpp:1343-1400), entering or leaving the
         * container's interior */
        const int m = RAY_MEDIUM(flags);
        th->transmitted++;   /* Transmitted_Rays_Traced */
        trace_ray(S, th, is->ipoint, D, weight, tk, WITH_MEDIUM(flags, m == is->object ? -1 : is->object) | RAY_CONTINUED,
                  out);
        return;
    }
    const PovGpuObject* o = &S->objs[is->object].o;
    const PovGpuMaterial* m = object_material(S, is->object);
    V3 raw = object_normal(S, is);
    if (o->flags & POV_FLAG_INVERTED)
        raw = vmul(raw, -1.0);
    if (vdot(raw, D) > 0.0)
        raw = vmul(raw, -1.0);
    V3 N = raw;
    V3 ip = is->ipoint;
    float filt, trm;   /* the layer's filter and transmit at the hit */
    RGB pig = material_pigment(S, m, is->ipoint, &filt, &trm);
    if (m->normal > 0) {
        const PovGpuNormal* nm = &S->desc.normals[m->normal - 1];
        N = perturb_normal(nm, &S->desc.patterns[nm->pattern - 1], ip, raw);
    }
    double r = 0.0, g = 0.0, b = 0.0;
    /* a transparent layer's own light is scaled by its opacity, 1 - filter -
     * transmit (TransColour::Opacity; LegacyOpacity before 3.7,
     * trace.cpp:877-881) */

    const int see_through = filt != 0.0f || trm != 0.0f;
    double att = 1.0;
    if (see_through)
        att = S->desc.language_version < 370 ? (float)(1.0 - (filt * fmaxf(pig.r, fmaxf(pig.g, pig.b)) + trm))
                                             : (float)(1.0 - filt - trm);

    /* ComputeReflectivity (trace.cpp:2627-2656) */
    double cos_inc = -vdot(D, N);
    double wmax = fmax(fmax(m->reflection_max[0], m->reflection_max[1]), m->reflection_max[2]);
    double wmin = fmax(fmax(m->reflection_min[0], m->reflection_min[1]), m->reflection_min[2]);
    double rweight = weight * fmax(wmax, wmin);
    double frac = fabs(m->reflection_falloff - 1.0) > EPSILON ? pow(1.0 - cos_inc, m->reflection_falloff)
                                                             : 1.0 - cos_inc;
    RGB reflec;
    if (fabs(frac) < EPSILON) {
        reflec.r = m->reflection_min[0]; reflec.g = m->reflection_min[1]; reflec.b = m->reflection_min[2];
    } else if (fabs(frac - 1.0) < EPSILON) {
        reflec.r = m->reflection_max[0]; reflec.g = m->reflection_max[1]; reflec.b = m->reflection_max[2];
    } else {
        reflec.r = (float)(frac * m->reflection_max[0] + (1.0 - frac) * m->reflection_min[0]);
        reflec.g = (float)(frac * m->reflection_max[1] + (1.0 - frac) * m->reflection_min[1]);
        reflec.b = (float)(frac * m->reflection_max[2] + (1.0 - frac) * m->reflection_min[2]);
    }
    if (m->reflection_fresnel) {
        /* ComputeFresnel (trace.cpp:2673-2677) at the ray's relative ior,
         * in float colour channels; the weight by the result's largest */
        const double f = fresnel_r(cos_inc, relative_ior(S, th, S->obj_int[is->object]));
        const float* rx = m->reflection_max;
        const float* rn = m->reflection_min;
        reflec.r = (float)(f * rx[0]) + (float)((1.0 - f) * rn[0]);
        reflec.g = (float)(f * rx[1]) + (float)((1.0 - f) * rn[1]);
        reflec.b = (float)(f * rx[2]) + (float)((1.0 - f) * rn[2]);
        rweight = weight * fmax(fmax(reflec.r, reflec.g), reflec.b);
    }
    if (m->reflect_metallic != 0.0f) {   /* ComputeMetallic on the reflectivity (trace.cpp:870) */
        float rc[3] = {reflec.r, reflec.g, reflec.b};
        compute_metallic(rc, m->reflect_metallic, pig, cos_inc);
        reflec.r = rc[0]; reflec.g = rc[1]; reflec.b = rc[2];
    }

    /* radiosity ambient (trace.cpp:793-800,896-980): one query per hit
     * while the bounce depth is below recursion_limit and the largest
     * possible contribution beats the ADC bailout */
    if (radiosity && tk->rad_depth < S->desc.radiosity.recursion_limit) {
        double diffuse = m->diffuse;
        float amb[3] = {0.0f, 0.0f, 0.0f};
        double maxc = (0.297 * pig.r + 0.589 * pig.g + 0.114 * pig.b) * 1.0 * diffuse;   /* WeightGreyscale */
        if (maxc > tk->adc)
            compute_ambient(S, th, ip, raw, N, 1.0, amb, weight * maxc, tk);
        r += (float)(pig.r * amb[0]) * diffuse;
        g += (float)(pig.g * amb[1]) * diffuse;
        b += (float)(pig.b * amb[2]) * diffuse;
    }

    /* emission, plus ambient * ambient_light when radiosity is off
     * (trace.cpp:982-1004) */
    double em[3];
    for (int k = 0; k < 3; k++)
        em[k] = m->emission[k] + (radiosity ? 0.0 : m->ambient[k] * S->desc.ambient_light[k]);
    r += pig.r * em[0] * att;
    g += pig.g * em[1] * att;
    b += pig.b * em[2] * att;

    /* ComputeDiffuseLight (trace.cpp:1488-1510,1637-1729) */
    if (m->diffuse != 0.0f || m->diffuse_back != 0.0f || m->specular != 0.0f || m->phong != 0.0f) {
        for (int li = 0; li < S->nlights; li++) {
            const PovGpuLight* L = &S->lights[li];
            V3 ld;
            double ldist, lc[3];
            one_light_ray(L, ip, &ld, &ldist, lc);
            if (fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON)
                continue;   /* outside a spotlight's cone (trace.cpp:1648-1650) */
            /* the light behind the surface: diffuse_back lights it from
             * there, without highlights (trace.cpp:1652-1662,1714) */
            int backside = 0;
            if (!(o->flags & POV_FLAG_DOUBLE_ILLUM)) {
                double cs = vdot(N, ld);
                if (cs < EPSILON) {
                    if (m->diffuse_back == 0.0f)
                        continue;
                    backside = 1;
                }
            }
            const int fill = L->light_type == POV_LIGHT_TYPE_SHADOWLESS;
            /* TraceShadowRay level check (trace.cpp:1897-1901); a shadowless
             * light traces no shadow ray (trace.cpp:1664) */
            if (!fill && level > tk->max_level)
                continue;
            if (!fill) {
                /* the radiosity Trace runs with areaLights off
                 * (GetRadiosityQualityFlags, radiosity.cpp:148-161): inside a
                 * gather an area light casts its centre's shadow */
                if (L->kind == POV_LIGHT_AREA && tk->rad_depth == 0) {
                    double f = area_light_fraction(S, th, L, ip, lc);
                    if (f == 0.0)
                        continue;
                    for (int k = 0; k < 3; k++)
                        lc[k] = (float)(lc[k] * f);
                } else {
                    double t3[3] = {1.0, 1.0, 1.0};
                    if (shadow_trace(S, th, ip, ld, ldist, RAY_MEDIUM(flags), !(flags & RAY_RADIOSITY), t3))
                        continue;
                    for (int k = 0; k < 3; k++)
                        lc[k] = (float)(lc[k] * t3[k]);
                }
            }
            /* ComputeDiffuseColour (trace.cpp:2441-2484) */
            double diffuse = (backside ? m->diffuse_back : m->diffuse) * m->brilliance_adjust;
            if (diffuse > 0.0) {
                double ci = vdot(N, ld);
                double inten = m->brilliance != 1.0f ? pow(fabs(ci), m->brilliance) : fabs(ci);
                inten *= diffuse * att;
                r += inten * pig.r * lc[0];
                g += inten * pig.g * lc[1];
                b += inten * pig.b * lc[2];
            }
            /* ComputePhongColour (trace.cpp:2520-2558); not for radiosity
             * rays nor shadowless lights (trace.cpp:1714) */
            if (m->phong > 0.0f && !(flags & RAY_RADIOSITY) && !fill && !backside) {
                double c2 = -2.0 * vdot(D, N);
                V3 rd = vadd(D, vmul(N, c2));
                double ci = vdot(rd, ld);
                if (ci > 0.0 && (m->phong_size < 60 || ci > 0.0008)) {
                    double inten = m->phong * pow(ci, (double)m->phong_size);
                    float cs[3] = {1.0f, 1.0f, 1.0f};
                    compute_metallic(cs, m->metallic, pig, vdot(N, ld));
                    r += inten * lc[0] * cs[0];
                    g += inten * lc[1] * cs[1];
                    b += inten * lc[2] * cs[2];
                }
            }
            /* ComputeSpecularColour (trace.cpp:2560-2593); not for radiosity
             * rays nor shadowless lights */
            if (m->specular > 0.0f && !(flags & RAY_RADIOSITY) && !fill && !backside) {
                V3 half = vmul(vadd(vmul(D, -1.0), ld), 0.5);
                double hl = vlen(half);
                if (hl > 0.0) {
                    double ci = vdot(half, N) / hl;
                    if (ci > 0.0) {
                        double inten = m->specular * pow(ci, (double)m->roughness);
                        float cs[3] = {1.0f, 1.0f, 1.0f};
                        compute_metallic(cs, m->metallic, pig, vdot(half, ld) / hl);
                        r += inten * lc[0] * cs[0];
                        g += inten * lc[1] * cs[1];
                        b += inten * lc[2] * cs[2];
                    }
                }
            }
        }
    }

    /* transmitted component (trace.cpp:1063-1142): the filter colour
     * TransmittedColour, trans = its greyscale; above ADC_Bailout the
     * refracted ray at weight * max|filter|, attenuated by Old_Refract and,
     * leaving the object's interior, its fade; not filtered after total
     * internal reflection */
    int tir = 0;
    if (see_through) {
        float pf[3] = {pig.r, pig.g, pig.b}, fil[3];
        transmitted_colour(pf, filt, trm, fil);
        if (m->conserve_energy) {
            /* conserve_energy: the filter loses what the surface reflects
             * (trace.cpp:1070-1075) */
            fil[0] *= fminf(1.0f, (float)(1.0 - reflec.r));
            fil[1] *= fminf(1.0f, (float)(1.0 - reflec.g));
            fil[2] *= fminf(1.0f, (float)(1.0 - reflec.b));
        }
        const double trans = fmin(1.0, fabs((double)(float)(0.297 * fil[0] + 0.589 * fil[1] + 0.114 * fil[2])));
        if (trans > tk->adc) {
            const double w1 = fmax(fabs(fil[0]), fmax(fabs(fil[1]), fabs(fil[2])));
            const int id = S->obj_int[is->object];
            const PovGpuInterior* I = &S->ints[id];
            const int leaving = ray_inside(th, id);
            RGB rc = {0, 0, 0};
            tir = compute_refraction(S, th, is, D, N, raw, weight * w1, tk, flags, &rc);
            float ac[3] = {I->old_refract, I->old_refract, I->old_refract};
            if (leaving && fabs(I->fade_distance) > EPSILON) {
                for (int k = 0; k < 3; k++) {
                    if (I->fade_power >= 1000.0)
                        ac[k] = (float)(ac[k] * exp(-(1.0 - I->fade_colour[k]) * (is->depth / I->fade_distance)));
                    else
                        ac[k] = (float)(ac[k] * (I->fade_colour[k] + (1.0 - I->fade_colour[k]) /
                                                 (1.0 + pow(is->depth / I->fade_distance, I->fade_power))));
                }
            }
            if (tir) {
                r += ac[0] * rc.r;
                g += ac[1] * rc.g;
                b += ac[2] * rc.b;
            } else {
                r += ac[0] * rc.r * fil[0];
                g += ac[1] * rc.g * fil[1];
                b += ac[2] * rc.b * fil[2];
            }
        }
    }

    /* reflected component (trace.cpp:1155-1178); after total internal
     * reflection only layers whose normal differs from the top one
     * reflect (a single layer: none) */
    if (!tir && !(reflec.r == 0.0f && reflec.g == 0.0f && reflec.b == 0.0f)) {
        RGB rc = {0, 0, 0};
        compute_reflection(S, th, ip, D, N, raw, rweight, tk, flags, &rc);
        r += reflec.r * rc.r;
        g += reflec.g * rc.g;
        b += reflec.b * rc.b;
    }
    out->r = (float)r;
    out->g = (float)g;
    out->b = (float)b;
}

/* Trace::TraceRay (trace.cpp:135-228): the ticket's level is raised while
 * the hit is shaded.  Returns the hit depth, HUGE_VAL for a miss or a ray
 * that bails at the trace level or ADC check. */
static void compute_media(const PovOracle* S, Thread* th, V3 O, V3 D, double dist, int medium, Ticket* tk, RGB* col);

static double trace_ray(const PovOracle* S, Thread* th, V3 O, V3 D, double weight, Ticket* tk, int flags, RGB* col)
{
    th->rays++;   /* Number_Of_Rays */
    col->r = col->g = col->b = 0.0f;
    weight = (float)weight;   /* TraceRay takes the weight as COLC (float) */
    if (tk->level >= tk->max_level || weight < tk->adc)
        return HUGE_VAL;
    const int cont = flags & RAY_CONTINUED;
    flags &= ~RAY_CONTINUED;
    Isect is;
    double depth = HUGE_VAL;
    if (!cont)
        tk->level++;
    if (find_intersection(S, th, O, D, HUGE_VAL, 0, &is)) {
        depth = is.depth;
        shade(S, th, &is, D, weight, tk, flags, col);
        /* interior media of the segment the ray crossed (ComputeTextureColour,
         * trace.cpp:577-580); the radiosity Trace runs with media off */
        if (RAY_MEDIUM(flags) >= 0 && !(flags & RAY_RADIOSITY))
            compute_media(S, th, O, D, is.depth, RAY_MEDIUM(flags), tk, col);
    } else {
        /* ComputeSky: background only (trace.cpp:2839-2888) */
        col->r = S->desc.background[0];
        col->g = S->desc.background[1];
        col->b = S->desc.background[2];
    }
    if (!cont)
        tk->level--;
    return depth;
}

/* The phase factor of ComputeMediaScatteringAttenuation (media.cpp:1183-
 * 1220) for one media, alpha = the cosine between the light ray (towards
 * the light) and the viewing ray: isotropic 1, Mie hazy, Mie murky,
 * Rayleigh, Henyey-Greenstein with the eccentricity g. */
static double media_phase(const PovGpuMedia* md, double alpha)
{
    switch (md->scattering_type) {
    case 2: return 0.576655375 * (1.0 + 9.0 * pow(0.5 * (1.0 + alpha), 8.0));
    case 3: return 0.495714547 * (1.0 + 50.0 * pow(0.5 * (1.0 + alpha), 32.0));
    case 4: return 0.799372013 * (1.0 + alpha * alpha);
    case 5: {
        const double g = md->eccentricity, g2 = g * g;
        return (1.0 - g2) / pow(1.0 + g2 - 2.0 * g * alpha, 1.5);
    }
    default: return 1.0;
    }
}

/* One media sample (MediaFunction::ComputeOneMediaSample, media.cpp:935-1038,
 * sample method 3, constant density): at fraction d of the interval
 * [s0, s0 + ds], the in-scattered light of every point light not in shadow
 * (TestShadow, trace.cpp:3173-3203, from inside the container) times the
 * media's phase factor (media_phase), times ds; the interval's optical
 * depth estimate extinction * ds. */
static void media_sample(const PovOracle* S, Thread* th, const PovGpuMedia* md, V3 O, V3 D, double s0, double ds,
                         double d, int medium, double lit, Ticket* tk, float C[3], float od[3])
{
    double x = s0 + d * ds;
    V3 P = vadd(O, vmul(D, x));
    th->media_samples++;   /* Media_Samples */
    double em[3] = {md->emission[0], md->emission[1], md->emission[2]};
    int scattering = md->scattering[0] != 0.0f || md->scattering[1] != 0.0f || md->scattering[2] != 0.0f;
    /* lit: the end of the lit span [0, lit] of a point light
     * (ComputeOneMediaLightInterval, media.cpp:715-750), < 0 for an unlit
     * interval; a sample beyond it sees no light (media.cpp:990) */
    if (lit >= 0.0 && x >= 0.0 && x <= lit && scattering) {
        for (int li = 0; li < S->nlights; li++) {
            const PovGpuLight* L = &S->lights[li];
            V3 ld = vsub(vload(L->center), P);
            double ldist = vlen(ld);
            ld = vdiv(ld, ldist);
            double lc[3] = {L->colour[0], L->colour[1], L->colour[2]};
            if (fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON)
                continue;
            if (tk->level > tk->max_level)
                continue;
            if (shadow_trace(S, th, P, ld, ldist, medium, 1, lc))
                continue;
            if (fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON)
                continue;
            const double ph = media_phase(md, vdot(ld, D));
            for (int k = 0; k < 3; k++)
                em[k] += (float)(ph * md->scattering[k]) * (float)lc[k];
        }
    }
    for (int k = 0; k < 3; k++) {
        C[k] = (float)(em[k] * ds);
        od[k] = (float)(md->extinction[k] * ds);
    }
}

static float col3_dist(const float a[3], const float b[3])   /* ColourDistance */
{
    return fabsf(a[0] - b[0]) + fabsf(a[1] - b[1]) + fabsf(a[2] - b[2]);
}

/* MediaFunction::ComputeOneMediaSampleRecursive (media.cpp:1040-1125), jitter 0. */
static void media_recursive(const PovOracle* S, Thread* th, const PovGpuMedia* md, V3 O, V3 D, double s0, double ds,
                            int medium, double lit, Ticket* tk, double d1, double d3, const float C1[3], const float C3[3],
                            const float od1[3], const float od3[3], int depth, float R[3], float ODR[3])
{
    float C2[3], od2[3], R2[3], ODR2[3];
    double d2 = 0.5 * (d1 + d3);
    media_sample(S, th, md, O, D, s0, ds, d2, medium, lit, tk, C2, od2);
    if (depth <= 0) {
        for (int k = 0; k < 3; k++) {
            R[k] = (C1[k] + C2[k] + C3[k]) / 3.0f;
            ODR[k] = (od1[k] + od2[k] + od3[k]) / 3.0f;
        }
        return;
    }
    if (col3_dist(C1, C2) > md->aa_threshold) {
        media_recursive(S, th, md, O, D, s0, ds, medium, lit, tk, d1, d2, C1, C2, od1, od2, depth - 1, R2, ODR2);
        for (int k = 0; k < 3; k++) {
            R[k] = R2[k] / 2.0f;
            ODR[k] = ODR2[k] / 2.0f;
        }
    } else {
        for (int k = 0; k < 3; k++) {
            R[k] = C1[k] / 3.0f + C2[k] / 6.0f;
            ODR[k] = od1[k] / 3.0f + od2[k] / 6.0f;
        }
    }
    if (col3_dist(C2, C3) > md->aa_threshold) {
        media_recursive(S, th, md, O, D, s0, ds, medium, lit, tk, d2, d3, C2, C3, od2, od3, depth - 1, R2, ODR2);
        for (int k = 0; k < 3; k++) {
            R[k] += R2[k] / 2.0f;
            ODR[k] += ODR2[k] / 2.0f;
        }
    } else {
        for (int k = 0; k < 3; k++) {
            R[k] += C2[k] / 6.0f + C3[k] / 3.0f;
            ODR[k] += od2[k] / 6.0f + od3[k] / 3.0f;
        }
    }
}

/* MediaFunction::ComputeMedia (media.cpp:287-364) for the media of one
 * container over the segment [0, dist] of the ray: point lights make one lit
 * interval (ComputeMediaLightInterval, media.cpp:598-751), split into
 * `intervals` uniform intervals (ComputeMediaSampleInterval, media.cpp:
 * 527-596; unlit constant media keep one), each sampled adaptively
 * (ComputeMediaAdaptiveSampling, media.cpp:432-501), then combined
 * (ComputeMediaColour, media.cpp:503-525): colour * exp(-Od) + Te. */
static void compute_media(const PovOracle* S, Thread* th, V3 O, V3 D, double dist, int medium, Ticket* tk, RGB* col)
{
    const PovGpuMedia* md = &S->desc.medias[container_media(S, medium)];
    const int lit = S->nlights > 0;
    /* ComputeMediaSampleInterval (media.cpp:527-596): with a light, the
     * span [0, dist] in `intervals` equal intervals, s1 = delta * (i + 1);
     * when rounding leaves the last s1 short of dist, ComputeMedia
     * (media.cpp:346-352) pads with an unlit interval up to dist.  Without
     * one, constant media takes the whole span as one unlit interval. */
    const int nuni = lit ? (md->intervals > 1 ? md->intervals : 1) : 1;
    const double delta = dist / (double)nuni;
    const int pad = lit && delta * (double)nuni < dist;
    const int nint = nuni + pad;
    int sub = (md->min_samples + 1) / 2;
    if (sub < 1)
        sub = 1;
    const double dd = 1.0 / (double)sub;
    double Od[3] = {0.0, 0.0, 0.0};
    float Te[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < nint; i++) {
        const double s0 = delta * (double)i;
        const double ds = (i < nuni) ? delta : dist - delta * (double)nuni;
        const double lit_end = (lit && i < nuni) ? dist : -1.0;
        float C0[3], od0[3], C1[3], od1[3], R[3], ODR[3];
        float te[3] = {0.0f, 0.0f, 0.0f}, odi[3] = {0.0f, 0.0f, 0.0f};
        media_sample(S, th, md, O, D, s0, ds, 0.0, medium, lit_end, tk, C0, od0);
        double d0 = 0.0;
        for (int j = 1; j <= sub; j++) {
            double d1 = d0 + dd;
            media_sample(S, th, md, O, D, s0, ds, d1, medium, lit_end, tk, C1, od1);
            media_recursive(S, th, md, O, D, s0, ds, medium, lit_end, tk, d0, d1, C0, C1, od0, od1, md->aa_level - 1, R,
                            ODR);
            for (int k = 0; k < 3; k++) {
                R[k] = (float)(R[k] * exp(-odi[k] * dd));
                if (ODR[k] != 0.0f)
                    R[k] = (float)(R[k] * ((1.0 - exp(-ODR[k] * dd)) / (ODR[k] * dd)));
                te[k] += R[k];
                odi[k] += ODR[k];
                C0[k] = C1[k];
                od0[k] = od1[k];
            }
            d0 = d1;
        }
        const double n = 1.0 / (double)sub;
        for (int k = 0; k < 3; k++) {
            Te[k] += (float)(te[k] * n * exp(-Od[k]));
            Od[k] += odi[k] * n;
        }
    }
    col->r = (float)(col->r * exp(-Od[0]) + Te[0]);
    col->g = (float)(col->g * exp(-Od[1]) + Te[1]);
    col->b = (float)(col->b * exp(-Od[2]) + Te[2]);
}

/* ============================================================ radiosity ==
 * RadiosityFunction and RadiosityCache (source/core/lighting/radiosity.cpp)
 * with the octree addressing of source/core/support/octree.cpp.  The cache
 * is one object per render; renders with radiosity run on one thread in
 * the reference's single-thread order (pov_oracle_render). */

#define RAD_EPSILON               0.001      /* radiosity.cpp:110 */
#define AVG_NEAR_EPSILON          0.000001   /* radiosity.cpp:109 */
#define IN_FRONT_LIMIT            (-0.05)    /* radiosity.cpp:100 */
#define WEIGHT_ERROR_BOUND_OFFSET 0.25       /* radiosity.cpp:111 */
#define BRILLIANCE_EPSILON        1e-5       /* radiosity.cpp:116 */
#define OT_BIAS                   10000000.  /* octree.h:81 */
#define RAD_DIRECTIONS            1600       /* RADIOSITY_MAX_SAMPLE_DIRECTIONS */
#define RAD_MAX_DEPTH             8
#define PASS_FIRST                1          /* kOctreePassFirst */
#define PASS_FINAL                65535      /* kOctreePassFinal (unsigned short max) */

/* RadiosityRecursionSettings (radiosity.cpp:177-294). */
typedef struct {
    int    rays_per_sample, reuse_count, trace_level;
    double error_bound_factor, min_reuse_factor, max_reuse_factor, address_factor, weight;
} RadRec;

/* ot_block_struct (octree.h:86-104). */
typedef struct {
    V3    point, normal, to_nearest;
    float ill[3];
    float hmd, nearest, quality, brilliance;
    int   depth, pass;
    int   next;          /* next block of the same octree node */
} RadBlock;

typedef struct { int size, x, y, z; } OtId;   /* OT_ID: biased log2 size, cell */

typedef struct RadCache {
    RadBlock* blocks;
    int       nblocks, cap;
    OtId*     keys;      /* octree nodes: open-addressing hash -> head block */
    int*      heads;
    int       nslots, nnodes;
    int       min_size, max_size;
    RadRec    rec[RAD_MAX_DEPTH];
    V3        dirs[RAD_DIRECTIONS];
    const double* jitter;
    int       njitter;
    uint64_t  gathers, reused, rays, pixels;
    uint64_t  gathers_depth[RAD_MAX_DEPTH];
} RadCache;

/* HaltonGenerator::operator[] (source/core/math/randomsequence.cpp:730-747). */
static double halton(unsigned base, size_t index)
{
    size_t i = 1 + index;
    double h = 0.0, q = 1.0 / base;
    while (i > 0) {
        h += (double)(i % base) * q;
        i /= base;
        q /= base;
    }
    return h;
}

/* SceneRadiositySettings::GetRecursionSettings (radiosity.cpp:177-294) and
 * the direction pool GetSubRandomCosWeightedDirectionGenerator(0, 1600)
 * picks (randomsequence.cpp:1019-1037): 1600 is not below the legacy
 * table's size, so it is the Halton(2, 3) cosine-weighted sequence
 * (HaltonCosWeightedDirectionGenerator, randomsequence.cpp:907-915). */
static void rad_setup(RadCache* R, const PovGpuRadiosity* rs)
{
    for (int d = 0; d < RAD_MAX_DEPTH; d++) {
        RadRec* r = &R->rec[d];
        int n = (int)(rs->count * pow(0.5, (double)d));
        r->rays_per_sample = n > 5 ? n : 5;
        r->reuse_count = d == 0 ? rs->nearest_count : (d == 1 ? (rs->nearest_count < 2 ? rs->nearest_count : 2) : 1);
        r->error_bound_factor = pow(2.0, (double)d);
        r->min_reuse_factor = rs->minimum_reuse * pow(2.0, (double)d);
        r->max_reuse_factor = rs->maximum_reuse * pow(2.0, (double)d);
        double overfill = d == 0 ? 1.0 : 8.0;
        r->trace_level = (int)(1.5 * ((double)d + 1));
        r->weight = pow(0.5 * rs->brightness, (double)d + 1);
        double max_error_bound = rs->error_bound * r->error_bound_factor;
        r->address_factor = max_error_bound / overfill;
    }
    for (int i = 0; i < RAD_DIRECTIONS; i++) {
        double rr = sqrt(halton(2, (size_t)i));
        double th = halton(3, (size_t)i) * (2 * 3.14159265358979323846);   /* 2*M_PI */
        double x = rr * cos(th), z = rr * sin(th);
        R->dirs[i] = v3(x, sqrt(1 - x * x - z * z), z);
    }
}

static void rad_reset(RadCache* R)
{
    R->nblocks = 0;
    R->nnodes = 0;
    for (int i = 0; i < R->nslots; i++)
        R->keys[i].size = -1;
    R->min_size = 1 << 30;
    R->max_size = -1;
    R->gathers = R->reused = R->rays = R->pixels = 0;
    memset(R->gathers_depth, 0, sizeof(R->gathers_depth));
}

static RadCache* rad_create(const PovGpuRadiosity* rs)
{
    RadCache* R = (RadCache*)calloc(1, sizeof(RadCache));
    R->nslots = 1 << 16;
    R->keys = (OtId*)malloc(sizeof(OtId) * R->nslots);
    R->heads = (int*)malloc(sizeof(int) * R->nslots);
    rad_setup(R, rs);
    rad_reset(R);
    return R;
}

static void rad_free(RadCache* R)
{
    if (!R) return;
    free(R->blocks);
    free(R->keys);
    free(R->heads);
    free(R);
}

/* Pow2Floor / BiasedIntLog2 / BiasedIntPow2 (octree.cpp:169-250): float
 * exponent arithmetic. */
static float pow2_floor(float a)
{
    uint32_t i;
    memcpy(&i, &a, 4);
    i &= 0xFF800000u;
    memcpy(&a, &i, 4);
    return a;
}
static int biased_log2(float a)
{
    uint32_t i;
    memcpy(&i, &a, 4);
    return (int)((i & 0x7F800000u) >> 23);
}
static float biased_pow2(int e)
{
    uint32_t i = ((uint32_t)e & 0xFFu) << 23;
    float a;
    memcpy(&a, &i, 4);
    return a;
}

/* ot_point_in_node (octree.cpp:985-997). */
static int ot_point_in_node(V3 p, const OtId* id)
{
    double sized = biased_pow2(id->size);
    if (fabs(p.x + OT_BIAS - ((double)id->x + 0.5) * sized) >= sized) return 0;
    if (fabs(p.y + OT_BIAS - ((double)id->y + 0.5) * sized) >= sized) return 0;
    if (fabs(p.z + OT_BIAS - ((double)id->z + 0.5) * sized) >= sized) return 0;
    return 1;
}

/* ot_index_sphere / ot_index_box with SAFE_METHOD (octree.cpp:1035-1190),
 * ot_parent (octree.cpp:1220-1238). */
static OtId ot_index_sphere(V3 c, double radius)
{
    V3 lo = v3(c.x - radius, c.y - radius, c.z - radius), hi = v3(c.x + radius, c.y + radius, c.z + radius);
    double desired = fmax(fmax(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
    double bsized = pow2_floor((float)desired);
    if (bsized == 0.0)
        bsized = 1.0;
    double maxord = fmax(fmax(fabs(lo.x), fabs(lo.y)), fabs(lo.z)) + OT_BIAS;
    while (maxord / bsized > 1000000000.0)
        bsized *= 2.0;
    V3 ctr = vdiv(vadd(lo, hi), 2);
    OtId id;
    id.x = (int)floor((ctr.x + OT_BIAS) / bsized);
    id.y = (int)floor((ctr.y + OT_BIAS) / bsized);
    id.z = (int)floor((ctr.z + OT_BIAS) / bsized);
    id.size = biased_log2((float)bsized);
    while (!ot_point_in_node(lo, &id) || !ot_point_in_node(hi, &id)) {
        id.size += 1;
        id.x = id.x >= 0 ? id.x >> 1 : (id.x + 1) / 2;
        id.y = id.y >= 0 ? id.y >> 1 : (id.y + 1) / 2;
        id.z = id.z >= 0 ? id.z >> 1 : (id.z + 1) / 2;
    }
    return id;
}

static uint32_t ot_hash(const OtId* k)
{
    uint32_t h = (uint32_t)k->size * 0x9E3779B1u;
    h ^= (uint32_t)k->x * 0x85EBCA77u;
    h ^= (uint32_t)k->y * 0xC2B2AE3Du;
    h ^= (uint32_t)k->z * 0x27D4EB2Fu;
    return h ^ (h >> 15);
}

static int ot_slot(const RadCache* R, const OtId* k)
{
    uint32_t m = (uint32_t)R->nslots - 1, i = ot_hash(k) & m;
    for (;;) {
        const OtId* e = &R->keys[i];
        if (e->size < 0 || (e->size == k->size && e->x == k->x && e->y == k->y && e->z == k->z))
            return (int)i;
        i = (i + 1) & m;
    }
}

static void ot_grow(RadCache* R)
{
    OtId* ok = R->keys;
    int* oh = R->heads;
    int on = R->nslots;
    R->nslots *= 2;
    R->keys = (OtId*)malloc(sizeof(OtId) * R->nslots);
    R->heads = (int*)malloc(sizeof(int) * R->nslots);
    for (int i = 0; i < R->nslots; i++)
        R->keys[i].size = -1;
    for (int i = 0; i < on; i++)
        if (ok[i].size >= 0) {
            int j = ot_slot(R, &ok[i]);
            R->keys[j] = ok[i];
            R->heads[j] = oh[i];
        }
    free(ok);
    free(oh);
}

/* RadiosityCache::AddBlock (radiosity.cpp:1194-1233) and InsertBlock
 * (radiosity.cpp:1421-1429: new blocks go to the head of the node's list). */
static void rad_add_block(RadCache* R, V3 point, V3 normal, double brilliance, V3 to_nearest, const float ill[3],
                          double hmd, double nearest, double quality, int depth, int pass)
{
    if (R->nblocks == R->cap) {
        R->cap = R->cap ? 2 * R->cap : 4096;
        R->blocks = (RadBlock*)realloc(R->blocks, sizeof(RadBlock) * R->cap);
    }
    RadBlock* b = &R->blocks[R->nblocks];
    b->ill[0] = ill[0]; b->ill[1] = ill[1]; b->ill[2] = ill[2];
    b->to_nearest = to_nearest;
    b->brilliance = (float)brilliance;
    b->hmd = (float)hmd;
    b->nearest = (float)nearest;
    b->quality = (float)quality;
    b->depth = depth;
    b->pass = pass;
    b->point = point;
    b->normal = normal;
    OtId id = ot_index_sphere(point, hmd * R->rec[depth].address_factor);
    if (2 * (R->nnodes + 1) > R->nslots)
        ot_grow(R);
    int slot = ot_slot(R, &id);
    if (R->keys[slot].size < 0) {
        R->keys[slot] = id;
        R->heads[slot] = -1;
        R->nnodes++;
    }
    b->next = R->heads[slot];
    R->heads[slot] = R->nblocks++;
    if (id.size < R->min_size) R->min_size = id.size;
    if (id.size > R->max_size) R->max_size = id.size;
}

/* WT_AVG of RadiosityCache::FindReusableBlock (radiosity.cpp:1458-1549). */
typedef struct {
    V3     P, N;
    double brilliance, error_bound, weights;
    float  wi[3];
    int    pass;
} WtAvg;

/* RadiosityCache::AverageNearBlock (radiosity.cpp:1551-1770), pseudo-sigmoid
 * weighting at final trace depth 0, linear otherwise; no gradient. */
static void rad_average_near(const RadBlock* b, WtAvg* w)
{
    if (fabs(b->brilliance - w->brilliance) > BRILLIANCE_EPSILON)
        return;
    V3 delta = vsub(w->P, b->point);
    double sq = vdot(delta, delta);
    double quick = (double)b->hmd * w->error_bound;
    if (!(sq < quick * quick))
        return;
    double dist = sqrt(sq);
    double ri = b->hmd;
    int far = dist > AVG_NEAR_EPSILON;
    V3 du = v3(0, 0, 0);
    if (far) {
        du = vdiv(delta, dist);
        double c = vdot(b->to_nearest, du);
        if (c > 0.0)
            ri = c * (double)b->nearest + (1.0 - c) * ri;
    }
    if (!(dist < ri * w->error_bound))
        return;
    double dd = vdot(w->N, b->normal);
    double e = dist / ri + 2.0 * sqrt(fabs(1.0 - dd));
    if (!(e < w->error_bound))
        return;
    double in_front = 1.0;
    if (far) {
        V3 half = vadd(w->N, b->normal);
        in_front = vdot(du, half) / vlen(half);
    }
    if (!(in_front > IN_FRONT_LIMIT))
        return;
    double wt;
    if (w->pass != PASS_FINAL || b->depth > 0) {
        wt = 1.0 - e / w->error_bound;
    } else {
        wt = e / w->error_bound;
        if (wt < 0.5)
            wt = 1.0 - (wt * 2.0) * (wt * 2.0) / 2.0;
        else
            wt = ((1.0 - wt) * 2.0) * ((1.0 - wt) * 2.0) / 2.0;
    }
    if (in_front <= 0)
        wt *= 1 - in_front / IN_FRONT_LIMIT;
    if (wt > RAD_EPSILON) {
        wt *= b->quality;
        for (int k = 0; k < 3; k++)
            w->wi[k] += (float)(b->ill[k] * wt);
        w->weights += wt;
    }
}

/* RadiosityCache::FindReusableBlock (radiosity.cpp:1458-1512) over the
 * octree nodes whose half-size-extended box holds P (ot_dist_traverse,
 * octree.cpp:800-855, visits exactly those), only blocks of this bounce
 * depth.  Returns the summed weight; sets ill when it is positive. */
static double rad_find_reusable(const RadCache* R, double error_bound, V3 P, V3 N, double brilliance, float ill[3],
                                int depth, int pass)
{
    if (R->nblocks == 0)
        return 0.0;
    WtAvg w;
    memset(&w, 0, sizeof(w));
    w.P = P; w.N = N; w.brilliance = brilliance; w.error_bound = error_bound; w.pass = pass;
    double c[3] = {P.x + OT_BIAS, P.y + OT_BIAS, P.z + OT_BIAS};
    for (int size = R->min_size; size <= R->max_size; size++) {
        double sz = biased_pow2(size);
        int lo[3], n[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = (int)floor(c[a] / sz - 1.5);
            n[a] = 4;
        }
        for (int i = 0; i < n[0]; i++)
            for (int j = 0; j < n[1]; j++)
                for (int k = 0; k < n[2]; k++) {
                    OtId id = {size, lo[0] + i, lo[1] + j, lo[2] + k};
                    if (!ot_point_in_node(P, &id))
                        continue;
                    int slot = ot_slot(R, &id);
                    if (R->keys[slot].size < 0)
                        continue;
                    for (int bi = R->heads[slot]; bi >= 0; bi = R->blocks[bi].next)
                        if (R->blocks[bi].depth == depth)
                            rad_average_near(&R->blocks[bi], &w);
                }
    }
    if (w.weights > 0)
        for (int k = 0; k < 3; k++)
            ill[k] = (float)(w.wi[k] / w.weights);
    return w.weights;
}

/* RadiosityFunction::GatherLight (radiosity.cpp:509-756) with the
 * SampleDirectionGenerator of an unperturbed normal (radiosity.cpp:772-888):
 * every direction of the bounce depth's sequence is usable. */
static double gather_light(const PovOracle* S, Thread* th, V3 ip, V3 raw, double brilliance, float ill[3],
                           Ticket* tk)
{
    RadCache* R = S->rad;
    const PovGpuRadiosity* rs = &S->desc.radiosity;
    const int depth = tk->rad_depth;
    const RadRec* rec = &R->rec[depth];
    double to_eye = vlen(vsub(vload(S->desc.camera.location), ip));
    double reuse_dist_min = to_eye * rec->min_reuse_factor;
    double maximum_distance = to_eye * rec->max_reuse_factor;
    int count = rec->rays_per_sample < RAD_DIRECTIONS ? rec->rays_per_sample : RAD_DIRECTIONS;
    Ticket save = *tk;
    tk->level = rec->trace_level;
    if (tk->max_level < tk->level + 1)
        tk->max_level = tk->level + 1;
    tk->adc = rs->adc_bailout;
    double inverse_distance_sum = 0.0, smallest = BOUND_HUGE;
    V3 min_dist_vec = v3(0, 0, 0);
    double weight = fmax(tk->adc + EPSILON, rec->weight);
    double qsum = 0.0;
    float sums[3] = {0.0f, 0.0f, 0.0f};
    /* InitSequence: frame around the normal */
    V3 fy = raw;
    V3 off = fabs(fy.z) > 0.9 ? v3(0, 1, 0) : v3(0, 0, 1);
    V3 fx = vnorm(vcross(fy, off));
    V3 fz = vnorm(vcross(fx, fy));
    int* idx = &th->rad_dir_index[depth];
    for (int i = 0; i < count; i++) {
        V3 rv = R->dirs[*idx];
        *idx = (*idx + 1) % RAD_DIRECTIONS;
        rv.y = fabs(rv.y);
        V3 dir;
        if (fy.y > 1.0 - RAD_EPSILON)
            dir = rv;
        else if (fy.y < -1.0 + RAD_EPSILON)
            dir = vmul(rv, -1.0);
        else
            dir = vadd(vadd(vmul(fx, rv.x), vmul(fy, rv.y)), vmul(fz, rv.z));
        tk->rad_quality = 1.0f;
        tk->rad_depth++;
        RGB c;
        double d = trace_ray(S, th, ip, dir, weight, tk, RAY_RADIOSITY, &c);
        tk->rad_depth--;
        double quality = tk->rad_quality;
        qsum += quality;
        sums[0] += (float)(c.r * quality);
        sums[1] += (float)(c.g * quality);
        sums[2] += (float)(c.b * quality);
        if (d < smallest) {
            smallest = d;
            min_dist_vec = dir;
        }
        inverse_distance_sum += 1.0 / d;
    }
    R->rays += (uint64_t)count;
    for (int k = 0; k < 3; k++)
        ill[k] = qsum == 0 ? sums[k] : (float)(sums[k] / qsum);
    double mean_dist = count / inverse_distance_sum;
    if (smallest > maximum_distance * 0.0001) {
        if (mean_dist < reuse_dist_min)
            mean_dist = reuse_dist_min;
        if (mean_dist > maximum_distance)
            mean_dist = maximum_distance;
        rad_add_block(R, ip, raw, brilliance, min_dist_vec, ill, mean_dist, smallest, qsum / count, depth,
                      th->rad_pass);
    }
    tk->max_level = save.max_level;
    tk->level = save.level;
    tk->adc = save.adc;
    tk->rad_quality = (float)fmax(save.rad_quality, qsum / count);
    return qsum / count;
}

/* ------------------------------------------- converged radiosity ---
 * The FP64 ground truth for the radiosity images (test infrastructure; no
 * counterpart in the reference).  ComputeAmbient without the sample cache:
 * every query at bounce depth d averages S->gt_count[d] cosine-weighted
 * directions of the radiance Trace returns along them, summed in FP64.  The
 * directions are stratified -- an a x a grid of jittered cells of the unit
 * square (a = round(sqrt(count))) mapped to the hemisphere by Malley's
 * method (uniform disc point lifted to the hemisphere: cosine-weighted
 * density) and turned by a random angle about the normal -- and drawn from
 * a per-pixel random sequence (splitmix64 seeded by the pixel), so the
 * image does not depend on the thread count.  Each sample ray is traced as
 * GatherLight traces its rays (radiosity.cpp:509-756: trace level, ADC
 * bailout and weight of the bounce depth, radiosity ray flags); the query
 * then gets ComputeAmbient's grey threshold and brightness
 * (radiosity.cpp:457-461).  Without reuse the only error left is the
 * sampling noise of gt_count directions per query. */
static const double GT_PI = 3.14159265358979323846;

static double gt_uniform(Thread* th)
{
    uint64_t z = (th->gt_rng += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

static void gather_converged(const PovOracle* S, Thread* th, V3 ip, V3 raw, double amb[3], Ticket* tk)
{
    RadCache* R = S->rad;
    const PovGpuRadiosity* rs = &S->desc.radiosity;
    const int depth = tk->rad_depth;
    const RadRec* rec = &R->rec[depth];
    int a = (int)floor(sqrt((double)S->gt_count[depth]) + 0.5);
    if (a < 1)
        a = 1;
    Ticket save = *tk;
    tk->level = rec->trace_level;
    if (tk->max_level < tk->level + 1)
        tk->max_level = tk->level + 1;
    tk->adc = rs->adc_bailout;
    double weight = fmax(tk->adc + EPSILON, rec->weight);
    V3 fy = raw;
    V3 off = fabs(fy.z) > 0.9 ? v3(0, 1, 0) : v3(0, 0, 1);
    V3 fx = vnorm(vcross(fy, off));
    V3 fz = vnorm(vcross(fx, fy));
    double turn = 2.0 * GT_PI * gt_uniform(th);
    double sum[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < a * a; i++) {
        double u = ((i % a) + gt_uniform(th)) / a, v = ((i / a) + gt_uniform(th)) / a;
        double r = sqrt(u), phi = 2.0 * GT_PI * v + turn;
        double lx = r * cos(phi), ly = sqrt(fmax(0.0, 1.0 - u)), lz = r * sin(phi);
        V3 dir = vnorm(vadd(vadd(vmul(fx, lx), vmul(fy, ly)), vmul(fz, lz)));
        tk->rad_quality = 1.0f;
        tk->rad_depth++;
        RGB c;
        trace_ray(S, th, ip, dir, weight, tk, RAY_RADIOSITY, &c);
        tk->rad_depth--;
        sum[0] += c.r;
        sum[1] += c.g;
        sum[2] += c.b;
    }
    for (int k = 0; k < 3; k++)
        amb[k] = sum[k] / (double)(a * a);
    tk->max_level = save.max_level;
    tk->level = save.level;
    tk->adc = save.adc;
    tk->rad_quality = save.rad_quality;
}

/* RadiosityFunction::ComputeAmbient (radiosity.cpp:385-462), "normal" and
 * "brilliance" settings off (their defaults). */
static void compute_ambient(const PovOracle* S, Thread* th, V3 ip, V3 raw, V3 layer, double brilliance, float amb[3],
                            double weight, Ticket* tk)
{
    (void)layer;
    (void)brilliance;
    RadCache* R = S->rad;
    const PovGpuRadiosity* rs = &S->desc.radiosity;
    if (S->gt_count[0] > 0) {   /* converged mode: no cache */
        double a[3];
        gather_converged(S, th, ip, raw, a, tk);
        double grey = 0.297 * a[0] + 0.589 * a[1] + 0.114 * a[2];
        for (int k = 0; k < 3; k++)
            amb[k] = (float)((a[k] * (1.0 - rs->gray_threshold) + rs->gray_threshold * grey) * rs->brightness);
        return;
    }
    const RadRec* rec = &R->rec[tk->rad_depth];
    double eb = th->rad_error_bound;
    if (weight < WEIGHT_ERROR_BOUND_OFFSET)
        eb += WEIGHT_ERROR_BOUND_OFFSET - weight;
    if (tk->rad_depth == 0)
        th->rad_top_queries++;
    double reuse = rad_find_reusable(R, eb * rec->error_bound_factor, ip, raw, 1.0, amb, tk->rad_depth,
                                     th->rad_pass);
    if (reuse * 4 >= rec->reuse_count || (th->rad_final && !rs->always_sample && reuse > 0)) {
        R->reused++;
    } else {
        float tmp[3];
        double quality = gather_light(S, th, ip, raw, 1.0, tmp, tk);
        for (int k = 0; k < 3; k++)
            amb[k] = reuse > 0 ? (float)((float)((float)(amb[k] * reuse) + (float)(tmp[k] * quality)) / (reuse + quality))
                               : tmp[k];
        reuse += quality;
        R->gathers++;
        R->gathers_depth[tk->rad_depth]++;
    }
    float q = (float)(4 * reuse) / (float)rec->reuse_count;
    tk->rad_quality = q < tk->rad_quality ? q : tk->rad_quality;
    float gray = (float)rs->gray_threshold;
    float grey = (float)(0.297 * amb[0] + 0.589 * amb[1] + 0.114 * amb[2]);
    for (int k = 0; k < 3; k++)
        amb[k] = (float)((amb[k] * (1.0f - gray) + gray * grey) * rs->brightness);
}

/* ----------------------------------------------------------- build --- */
static int build_mesh(OMesh* om, const PovGpuMesh* m)
{
    memset(om, 0, sizeof(*om));
    om->ntris = m->num_triangles;
    om->verts = (float*)malloc(sizeof(float) * 3 * (m->num_vertices > 0 ? m->num_vertices : 1));
    memcpy(om->verts, m->vertices, sizeof(float) * 3 * m->num_vertices);
    om->normals = NULL;
    if (m->num_normals > 0 && m->normals) {
        om->normals = (float*)malloc(sizeof(float) * 3 * m->num_normals);
        for (int i = 0; i < m->num_normals; i++) {
            /* Parse_Mesh2 normalises each normal_vectors entry (parser.cpp:4143) */
            V3 n = v3(m->normals[3 * i], m->normals[3 * i + 1], m->normals[3 * i + 2]);
            if (fabs(n.x) < EPSILON && fabs(n.y) < EPSILON && fabs(n.z) < EPSILON)
                n.x = 1.0;
            n = vnorm(n);
            om->normals[3 * i] = (float)n.x;
            om->normals[3 * i + 1] = (float)n.y;
            om->normals[3 * i + 2] = (float)n.z;
        }
    }
    om->tris = (MeshTri*)calloc((size_t)om->ntris, sizeof(MeshTri));
    for (int i = 0; i < om->ntris; i++) {
        MeshTri* T = &om->tris[i];
        const int32_t* f = &m->face_indices[3 * i];
        if (f[0] < 0 || f[1] < 0 || f[2] < 0 || f[0] >= m->num_vertices || f[1] >= m->num_vertices ||
            f[2] >= m->num_vertices)
            return -1;
        T->p1 = f[0]; T->p2 = f[1]; T->p3 = f[2];
        int smooth = 0;
        if (om->normals && m->normal_indices) {
            const int32_t* ni = &m->normal_indices[3 * i];
            T->n1 = ni[0]; T->n2 = ni[1]; T->n3 = ni[2];
            const float* nv = om->normals;
            V3 N1 = v3(nv[3 * T->n1], nv[3 * T->n1 + 1], nv[3 * T->n1 + 2]);
            V3 N2 = v3(nv[3 * T->n2], nv[3 * T->n2 + 1], nv[3 * T->n2 + 2]);
            V3 N3 = v3(nv[3 * T->n3], nv[3 * T->n3 + 1], nv[3 * T->n3 + 2]);
            V3 D1 = vsub(N1, N2), D2 = vsub(N1, N3);
            double l1 = vdot(D1, D1), l2 = vdot(D2, D2);
            smooth = (fabs(l1) > EPSILON) || (fabs(l2) > EPSILON);   /* parser.cpp:4545 */
        }
        compute_mesh_triangle(T, om->verts, smooth);
    }
    /* Build_Mesh_BBox_Tree (mesh.cpp:1376-1450) */
    int32_t* leaves = (int32_t*)malloc(sizeof(int32_t) * (size_t)(om->ntris > 0 ? om->ntris : 1));
    for (int i = 0; i < om->ntris; i++) {
        const MeshTri* T = &om->tris[i];
        const float* v = om->verts;
        V3 a = v3(v[3 * T->p1], v[3 * T->p1 + 1], v[3 * T->p1 + 2]);
        V3 b = v3(v[3 * T->p2], v[3 * T->p2 + 1], v[3 * T->p2 + 2]);
        V3 c = v3(v[3 * T->p3], v[3 * T->p3 + 1], v[3 * T->p3 + 2]);
        V3 mn = v3(fmin(a.x, fmin(b.x, c.x)), fmin(a.y, fmin(b.y, c.y)), fmin(a.z, fmin(b.z, c.z)));
        V3 mx = v3(fmax(a.x, fmax(b.x, c.x)), fmax(a.y, fmax(b.y, c.y)), fmax(a.z, fmax(b.z, c.z)));
        TNode n;
        memset(&n, 0, sizeof(n));
        n.bbox = bbox_from_min_max(mn, mx);
        n.first = i;
        leaves[i] = tree_add(&om->tree, n);
    }
    build_bbox_tree(&om->tree, leaves, (size_t)om->ntris, NULL, 0);
    free(leaves);
    return 0;
}

static BBox object_bbox(const PovOracle* S, const PovGpuObject* o)
{
    BBox b;
    memset(&b, 0, sizeof(b));
    switch (o->type) {
    case POV_OBJ_SPHERE: {   /* Sphere::Compute_BBox (sphere.cpp:646-658) */
        double r = o->p[3];
        b.ll[0] = (float)(o->p[0] - r); b.ll[1] = (float)(o->p[1] - r); b.ll[2] = (float)(o->p[2] - r);
        b.sz[0] = b.sz[1] = b.sz[2] = (float)(2.0 * r);
        break;
    }
    case POV_OBJ_MESH: {     /* Mesh::Compute_BBox (mesh.cpp:790-808) */
        const OMesh* m = &S->meshes[o->mesh];
        V3 mn = v3(BOUND_HUGE, BOUND_HUGE, BOUND_HUGE), mx = v3(-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE);
        for (int i = 0; i < m->ntris; i++) {
            const MeshTri* T = &m->tris[i];
            int32_t idx[3] = {T->p1, T->p2, T->p3};
            for (int k = 0; k < 3; k++) {
                const float* v = &m->verts[3 * idx[k]];
                mn.x = fmin(mn.x, v[0]); mn.y = fmin(mn.y, v[1]); mn.z = fmin(mn.z, v[2]);
                mx.x = fmax(mx.x, v[0]); mx.y = fmax(mx.y, v[1]); mx.z = fmax(mx.z, v[2]);
            }
        }
        b = bbox_from_min_max(mn, mx);
        break;
    }
    case POV_OBJ_BOX:        /* Box::Compute_BBox (box.cpp:947-957) */
        b = bbox_from_min_max(v3(o->p[0], o->p[1], o->p[2]), v3(o->p[3], o->p[4], o->p[5]));
        break;
    case POV_OBJ_TORUS: {    /* Torus::Compute_BBox + Recompute_BBox (torus.cpp:849-859, boundingbox.cpp:168) */
        double r1 = o->p[1], r2 = o->p[0] + o->p[1];
        float ll[3] = {(float)-r2, (float)-r1, (float)-r2};
        float sz[3] = {(float)(2.0 * r2), (float)(2.0 * r1), (float)(2.0 * r2)};
        V3 mn = v3(BOUND_HUGE, BOUND_HUGE, BOUND_HUGE), mx = v3(-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE);
        for (int i = 1; i <= 8; i++) {
            V3 c = v3(ll[0] + ((i & 1) ? sz[0] : 0.0), ll[1] + ((i & 2) ? sz[1] : 0.0), ll[2] + ((i & 4) ? sz[2] : 0.0));
            c = mtrans_point(o->trans, c);
            mn.x = fmin(mn.x, c.x); mn.y = fmin(mn.y, c.y); mn.z = fmin(mn.z, c.z);
            mx.x = fmax(mx.x, c.x); mx.y = fmax(mx.y, c.y); mx.z = fmax(mx.z, c.z);
        }
        b = bbox_from_min_max(mn, mx);
        break;
    }
    case POV_OBJ_UNION:
    case POV_OBJ_MERGE:
    case POV_OBJ_INTERSECTION: {   /* CSG::Compute_BBox (csg.cpp:872-): union of the
                                      children, or the overlap of the non-inverted ones */
        int isect = o->type == POV_OBJ_INTERSECTION;
        V3 mn = isect ? v3(-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE) : v3(BOUND_HUGE, BOUND_HUGE, BOUND_HUGE);
        V3 mx = isect ? v3(BOUND_HUGE, BOUND_HUGE, BOUND_HUGE) : v3(-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE);
        for (int c = 0; c < o->num_children; c++) {
            const PovGpuObject* ch = &S->objs[o->first_child + c].o;
            if (isect && (ch->flags & POV_FLAG_INVERTED))
                continue;
            BBox cb = object_bbox(S, ch);
            V3 cl = v3(cb.ll[0], cb.ll[1], cb.ll[2]);
            V3 ch_ = v3((double)cb.ll[0] + cb.sz[0], (double)cb.ll[1] + cb.sz[1], (double)cb.ll[2] + cb.sz[2]);
            if (isect) {
                mn.x = fmax(mn.x, cl.x); mn.y = fmax(mn.y, cl.y); mn.z = fmax(mn.z, cl.z);
                mx.x = fmin(mx.x, ch_.x); mx.y = fmin(mx.y, ch_.y); mx.z = fmin(mx.z, ch_.z);
            } else {
                mn.x = fmin(mn.x, cl.x); mn.y = fmin(mn.y, cl.y); mn.z = fmin(mn.z, cl.z);
                mx.x = fmax(mx.x, ch_.x); mx.y = fmax(mx.y, ch_.y); mx.z = fmax(mx.z, ch_.z);
            }
        }
        b = bbox_from_min_max(mn, mx);
        break;
    }
    default: {               /* infinite objects: Make_BBox(-BOUND_HUGE/2, BOUND_HUGE) */
        b.ll[0] = b.ll[1] = b.ll[2] = (float)(-BOUND_HUGE / 2);
        b.sz[0] = b.sz[1] = b.sz[2] = (float)BOUND_HUGE;
        break;
    }
    }
    return b;
}

int pov_oracle_create(const PovGpuSceneDesc* desc, PovOracle** out, int32_t* bad_index)
{
    if (bad_index) *bad_index = -1;
    if (!desc || !out || desc->abi_version != POV_GPU_ABI_VERSION || desc->num_materials < 1)
        return POV_GPU_E_INVALID;
    /* media containers: hollow top-level boxes or spheres whose surface only
     * transmits, holding one constant media (any scattering type) sampled
     * by method 3 without jitter; point lights only */
    int containers = 0;
    for (int i = 0; i < desc->num_objects; i++) {
        const PovGpuObject* o = &desc->objects[i];
        if (o->media < 0 || o->media > desc->num_medias || (o->media > 0 && !desc->medias))
            return POV_GPU_E_INVALID;
        const PovGpuMaterial* m = (o->material >= 0 && o->material < desc->num_materials) ? &desc->materials[o->material]
                                                                                           : NULL;
        int transmits = m && (m->pigment[3] != 0.0f || m->pigment[4] != 0.0f);
        if (o->media == 0 && transmits)
            continue;   /* a transparent surface (checked below) */
        if (o->media > 0) {
            if (bad_index) *bad_index = i;
            const PovGpuMedia* md = o->media > 0 ? &desc->medias[o->media - 1] : NULL;
            if (!md || (o->type != POV_OBJ_BOX && o->type != POV_OBJ_SPHERE) || (o->flags & POV_FLAG_INVERTED) ||
                !(o->flags & POV_FLAG_HOLLOW) || o->parent >= 0 || !m ||
                m->pigment[3] != 0.0f || m->pigment[4] != 1.0f || m->diffuse != 0.0f || m->phong != 0.0f ||
                m->specular != 0.0f || m->emission[0] != 0.0f || m->emission[1] != 0.0f || m->emission[2] != 0.0f ||
                m->ambient[0] != 0.0f || m->ambient[1] != 0.0f || m->ambient[2] != 0.0f ||
                m->reflection_max[0] != 0.0f || m->reflection_max[1] != 0.0f || m->reflection_max[2] != 0.0f ||
                md->method != 3 || md->jitter != 0.0f || md->scattering_type < 1 || md->scattering_type > 5 ||
                md->min_samples != md->max_samples || md->min_samples < 1 || md->aa_level < 1)
                return POV_GPU_E_UNSUPPORTED;
            /* camera rays start outside every container: a camera inside one
             * would need the interior list of its location */
            int inside = 1;
            if (o->type == POV_OBJ_SPHERE) {
                double dd = 0.0;
                for (int k = 0; k < 3; k++)
                    dd += (desc->camera.location[k] - o->p[k]) * (desc->camera.location[k] - o->p[k]);
                inside = dd < o->p[3] * o->p[3];
            } else {
                for (int k = 0; k < 3; k++) {
                    double lo = fmin(o->p[k], o->p[3 + k]), hi = fmax(o->p[k], o->p[3 + k]);
                    inside = inside && desc->camera.location[k] >= lo && desc->camera.location[k] <= hi;
                }
            }
            if (inside)
                return POV_GPU_E_UNSUPPORTED;
            containers++;
        }
    }
    if (bad_index) *bad_index = -1;
    /* transparent surfaces (filter or transmit outside media containers):
     * plain pigments, interiors without dispersion or caustics; not with
     * media containers, radiosity or area lights (whose shadow colours
     * would need the filtered form of TraceAreaLightShadowRay) */
    int transparent = 0;
    for (int i = 0; i < desc->num_materials; i++) {
        const PovGpuMaterial* m = &desc->materials[i];
        int used_by_container = 0;
        for (int k = 0; k < desc->num_objects; k++)
            used_by_container = used_by_container || (desc->objects[k].media > 0 && desc->objects[k].material == i);
        if (material_transparent(desc, m) && !used_by_container)
            transparent = 1;
    }
    /* the classic finish terms; fresnel reflection and conserve_energy on
     * transparent surfaces only (they need the surface's interior) */
    for (int i = 0; i < desc->num_materials; i++) {
        const PovGpuMaterial* m = &desc->materials[i];
        const int see = m->pattern > 0 && m->pattern <= desc->num_patterns && desc->patterns
                            ? pattern_transparent(&desc->patterns[m->pattern - 1])
                            : (m->pigment[3] != 0.0f || m->pigment[4] != 0.0f);
        if (m->fresnel != 0.0f || m->reflect_exp != 1.0f ||
            m->irid != 0.0f || m->crand != 0.0f || (m->diffuse_back != 0.0f && desc->radiosity.enabled) ||
            ((m->reflection_fresnel || m->conserve_energy) && !see))
            return POV_GPU_E_UNSUPPORTED;
    }
    if (desc->num_interiors < 0 || (desc->num_interiors > 0 && !desc->interiors))
        return POV_GPU_E_INVALID;
    if (desc->object_interior)
        for (int i = 0; i < desc->num_objects; i++)
            if (desc->object_interior[i] < 0 || desc->object_interior[i] > desc->num_interiors)
                return POV_GPU_E_INVALID;
    if (transparent) {
        if (containers || desc->radiosity.enabled)
            return POV_GPU_E_UNSUPPORTED;
        for (int i = 0; i < desc->num_interiors; i++)
            if (desc->interiors[i].dispersion != 1.0 || desc->interiors[i].caustics != 0.0)
                return POV_GPU_E_UNSUPPORTED;
        for (int i = 0; i < desc->num_lights; i++)
            if (desc->lights[i].kind != POV_LIGHT_POINT)
                return POV_GPU_E_UNSUPPORTED;
    }
    for (int i = 0; i < desc->num_lights; i++) {
        const PovGpuLight* L = &desc->lights[i];
        if ((L->kind != POV_LIGHT_POINT && L->kind != POV_LIGHT_AREA) || L->light_type < 0 ||
            L->light_type > POV_LIGHT_TYPE_CYLINDER)
            return POV_GPU_E_INVALID;
        const int plain = L->light_type <= POV_LIGHT_TYPE_POINT && !L->parallel && L->fade_power <= 0.0;
        if (containers && (L->kind != POV_LIGHT_POINT || !plain))
            return POV_GPU_E_UNSUPPORTED;   /* media samples test plain point-light shadows only */
        if (L->kind == POV_LIGHT_AREA && (L->parallel || L->light_type == POV_LIGHT_TYPE_CYLINDER))
            return POV_GPU_E_UNSUPPORTED;   /* area lights: no parallel beams */
        if ((L->light_type == POV_LIGHT_TYPE_SPOT || L->light_type == POV_LIGHT_TYPE_CYLINDER || L->parallel) &&
            !(vlen(vsub(vload(L->points_at), vload(L->center))) > EPSILON))
            return POV_GPU_E_UNSUPPORTED;   /* a beam needs its direction */
        if (L->kind == POV_LIGHT_AREA &&
            (L->area_size1 < 1 || L->area_size2 < 1 || L->area_size1 * L->area_size2 > AREA_MAX_POINTS ||
             L->jitter || (L->circular && (L->area_size1 < 2 || L->area_size2 < 2))))
            return POV_GPU_E_UNSUPPORTED;   /* jitter draws on the reference's RNG stream */
    }
    /* patterns: the nine pigment patterns and the three normal-only ones,
     * 0..16 ascending colour map entries, noise generators 1..3; a pigment
     * reads one of the nine with 1..16 entries (checker: 2), a normal any
     * but checker (whose normal form is a normal map) */
    if (desc->num_patterns < 0 || (desc->num_patterns > 0 && !desc->patterns))
        return POV_GPU_E_INVALID;
    for (int i = 0; i < desc->num_patterns; i++) {
        const PovGpuPattern* pt = &desc->patterns[i];
        if (pt->type < POV_PATTERN_CHECKER || pt->type > POV_PATTERN_QUILTED || pt->num_entries < 0 ||
            (pt->type == POV_PATTERN_CRACKLE && !(pt->crackle_metric > 0.0)) ||
            pt->num_entries > POV_PATTERN_MAX_ENTRIES || pt->noise_generator < 1 || pt->noise_generator > 3 ||
            pt->wave_type < POV_WAVE_RAMP || pt->wave_type > POV_WAVE_POLY || pt->octaves < 1 || pt->octaves > 32 ||
            (pt->type == POV_PATTERN_CHECKER && pt->num_entries != 2) ||
            (pt->type == POV_PATTERN_SQUARE && pt->num_entries != 4) ||
            ((pt->type == POV_PATTERN_TRIANGULAR || pt->type == POV_PATTERN_CUBIC) && pt->num_entries != 6) ||
            (pt->type == POV_PATTERN_HEXAGON && pt->num_entries != 3) ||
            (pt->type == POV_PATTERN_BRICK && (pt->num_entries != 2 || !(pt->brick_size[0] > 0.0) ||
                                               !(pt->brick_size[1] > 0.0) || !(pt->brick_size[2] > 0.0))))
            return POV_GPU_E_UNSUPPORTED;
        for (int k = 1; k < pt->num_entries; k++)
            if (pt->values[k] < pt->values[k - 1])
                return POV_GPU_E_INVALID;
    }
    if (desc->num_normals < 0 || (desc->num_normals > 0 && !desc->normals))
        return POV_GPU_E_INVALID;
    for (int i = 0; i < desc->num_normals; i++) {
        const PovGpuNormal* nm = &desc->normals[i];
        if (nm->pattern < 1 || nm->pattern > desc->num_patterns)
            return POV_GPU_E_INVALID;
        const int nt = desc->patterns[nm->pattern - 1].type;
        if (nt == POV_PATTERN_CHECKER || (nt >= POV_PATTERN_SQUARE && nt <= POV_PATTERN_BRICK) ||
            nt == POV_PATTERN_QUILTED ||
            !(nm->delta > 0.0f) ||
            !isfinite(nm->amount))
            return POV_GPU_E_UNSUPPORTED;
    }
    for (int i = 0; i < desc->num_materials; i++) {
        const PovGpuMaterial* m = &desc->materials[i];
        if (m->pattern < 0 || m->pattern > desc->num_patterns || m->normal < 0 || m->normal > desc->num_normals)
            return POV_GPU_E_INVALID;
        if (m->pattern > 0) {
            const PovGpuPattern* pt = &desc->patterns[m->pattern - 1];
            if (pt->type == POV_PATTERN_BUMPS || pt->num_entries < 1 ||
                (pt->type == POV_PATTERN_CHECKER && pt->num_entries != 2))
                return POV_GPU_E_UNSUPPORTED;
        }
    }
    pthread_once(&g_noise_once, noise_init);
    PovOracle* S = (PovOracle*)calloc(1, sizeof(PovOracle));
    S->desc = *desc;
    if (desc->radiosity.enabled)
        S->rad = rad_create(&desc->radiosity);
    S->nobjs = desc->num_objects;
    S->objs = (OObj*)calloc((size_t)(S->nobjs > 0 ? S->nobjs : 1), sizeof(OObj));
    S->mats = (PovGpuMaterial*)malloc(sizeof(PovGpuMaterial) * desc->num_materials);
    memcpy(S->mats, desc->materials, sizeof(PovGpuMaterial) * desc->num_materials);
    S->nlights = desc->num_lights;
    S->lights = (PovGpuLight*)malloc(sizeof(PovGpuLight) * (desc->num_lights > 0 ? desc->num_lights : 1));
    if (desc->num_lights > 0)
        memcpy(S->lights, desc->lights, sizeof(PovGpuLight) * desc->num_lights);
    S->nmeshes = desc->num_meshes;
    S->meshes = (OMesh*)calloc((size_t)(S->nmeshes > 0 ? S->nmeshes : 1), sizeof(OMesh));
    for (int i = 0; i < S->nmeshes; i++)
        if (build_mesh(&S->meshes[i], &desc->meshes[i]) != 0) {
            if (bad_index) *bad_index = i;
            pov_oracle_destroy(S);
            return POV_GPU_E_INVALID;
        }
    int32_t* finite = (int32_t*)malloc(sizeof(int32_t) * (size_t)(S->nobjs + 1));
    int32_t* infinite = (int32_t*)malloc(sizeof(int32_t) * (size_t)(S->nobjs + 1));
    size_t nf = 0, ni = 0;
    for (int i = 0; i < S->nobjs; i++)
        S->objs[i].o = desc->objects[i];
    for (int i = 0; i < S->nobjs; i++) {
        const PovGpuObject* o = &S->objs[i].o;
        int ok = o->type >= POV_OBJ_SPHERE && o->type <= POV_OBJ_MERGE;
        if (o->type == POV_OBJ_TORUS && !(o->flags & POV_FLAG_HAS_TRANS))
            ok = 0;
        if ((o->type == POV_OBJ_SPHERE || o->type == POV_OBJ_BOX || o->type == POV_OBJ_MESH ||
             o->type == POV_OBJ_PLANE) && (o->flags & POV_FLAG_HAS_TRANS))
            ok = 0;
        if (o->type >= POV_OBJ_UNION) {
            /* CSG with leaf children (spheres, boxes, tori, planes) */
            if (o->first_child != i + 1 || o->num_children < 1 || o->first_child + o->num_children > S->nobjs)
                ok = 0;
            for (int c = 0; ok && c < o->num_children; c++) {
                const PovGpuObject* ch = &S->objs[o->first_child + c].o;
                if (ch->type == POV_OBJ_MESH || ch->type >= POV_OBJ_UNION || ch->parent != i)
                    ok = 0;
            }
        }
        if (o->parent >= 0 && S->objs[o->parent].o.type < POV_OBJ_UNION)
            ok = 0;
        if (!ok) {
            if (bad_index) *bad_index = i;
            free(finite); free(infinite);
            pov_oracle_destroy(S);
            return POV_GPU_E_UNSUPPORTED;
        }
    }
    for (int i = S->nobjs - 1; i >= 0; i--)   /* children before parents (CSG boxes) */
        S->objs[i].bbox = object_bbox(S, &S->objs[i].o);
    for (int i = 0; i < S->nobjs; i++) {      /* Build_Bounding_Slabs keeps object order */
        const PovGpuObject* o = &S->objs[i].o;
        if (o->parent >= 0)
            continue;
        TNode n;
        memset(&n, 0, sizeof(n));
        n.bbox = S->objs[i].bbox;
        n.first = i;
        if (o->flags & POV_FLAG_INFINITE) {
            n.infinite = 1;
            infinite[ni++] = tree_add(&S->top, n);
        } else {
            finite[nf++] = tree_add(&S->top, n);
        }
    }
    /* BoundingTask::Run: no slabs below Bounding_Threshold 3 (boundingtask.cpp:170) */
    S->top_linear = (nf + ni) < 3;
    if (!S->top_linear)
        build_bbox_tree(&S->top, finite, nf, infinite, ni);
    free(finite);
    free(infinite);
    /* interiors: the description's, plus a default one (ior = the
     * atmosphere's, Post_Process, parser.cpp:9225-9267) for every top-level
     * object given none; CSG children without their own share their
     * parent's (parser.cpp:9040-9044) */
    S->atm_ior = desc->atmosphere_ior > 0.0 ? desc->atmosphere_ior : 1.0;
    S->transparent = transparent;
    S->ints = (PovGpuInterior*)calloc((size_t)(desc->num_interiors + S->nobjs + 1), sizeof(PovGpuInterior));
    S->obj_int = (int32_t*)malloc(sizeof(int32_t) * (size_t)(S->nobjs + 1));
    if (desc->num_interiors > 0)
        memcpy(S->ints, desc->interiors, sizeof(PovGpuInterior) * (size_t)desc->num_interiors);
    S->nints = desc->num_interiors;
    for (int i = 0; i < S->nobjs; i++) {
        const int32_t given = desc->object_interior ? desc->object_interior[i] : 0;
        const int32_t parent = S->objs[i].o.parent;
        if (given > 0) {
            S->obj_int[i] = given - 1;
        } else if (parent >= 0) {
            S->obj_int[i] = S->obj_int[parent];
        } else {
            PovGpuInterior* d = &S->ints[S->nints];
            d->ior = S->atm_ior;
            d->dispersion = 1.0;
            d->old_refract = 1.0f;
            S->obj_int[i] = S->nints++;
        }
    }
    /* camera rays start with no interior (TracePixel::InitRayContainerState,
     * tracepixel.cpp:929-963, would list the objects around the camera in
     * the bounding tree's order): with transparent surfaces the camera must
     * be inside no object */
    if (transparent)
        for (int i = 0; i < S->nobjs; i++)
            if (S->objs[i].o.parent < 0 && inside_object(S, i, vload(desc->camera.location))) {
                if (bad_index) *bad_index = i;
                pov_oracle_destroy(S);
                return POV_GPU_E_UNSUPPORTED;
            }
    *out = S;
    return POV_GPU_OK;
}

static void free_tree(Tree* t) { free(t->nodes); free(t->kids); }

/* Composite nodes (nodes with entries) of the bounding trees the oracle
 * built: the top tree (none below Bounding_Threshold) and all mesh trees. */
void pov_oracle_tree_info(const PovOracle* S, int32_t* top_nodes, int32_t* mesh_nodes)
{
    int32_t t = 0, m = 0;
    if (!S->top_linear && S->top.root >= 0)
        for (int32_t i = 0; i < S->top.num_nodes; i++)
            t += S->top.nodes[i].entries > 0;
    for (int32_t k = 0; k < S->nmeshes; k++)
        for (int32_t i = 0; i < S->meshes[k].tree.num_nodes; i++)
            m += S->meshes[k].tree.nodes[i].entries > 0;
    *top_nodes = t;
    *mesh_nodes = m;
}

void pov_oracle_destroy(PovOracle* S)
{
    if (!S) return;
    for (int i = 0; i < S->nmeshes; i++) {
        free(S->meshes[i].verts);
        free(S->meshes[i].normals);
        free(S->meshes[i].tris);
        free_tree(&S->meshes[i].tree);
    }
    free(S->meshes);
    free_tree(&S->top);
    free(S->objs);
    free(S->mats);
    free(S->lights);
    free(S->ints);
    free(S->obj_int);
    rad_free(S->rad);
    free(S);
}

static void thread_free(Thread* th) { free(th->pq.q); free(th->mpq.q); }

int pov_oracle_trace_rays(PovOracle* S, const double* org, const double* dir, int32_t n, PovGpuHit* hits)
{
    Thread th;
    memset(&th, 0, sizeof(th));
    for (int32_t i = 0; i < n; i++) {
        Isect is;
        V3 O = vload(org + 3 * i), D = vload(dir + 3 * i);
        if (find_intersection(S, &th, O, D, HUGE_VAL, 0, &is)) {
            hits[i].object = is.object;
            /* the triangle index only means something for mesh hits */
            hits[i].triangle = S->objs[is.object].o.type == POV_OBJ_MESH ? is.triangle : -1;
            hits[i].t = is.depth;
        } else {
            hits[i].object = -1;
            hits[i].triangle = -1;
            hits[i].t = 0.0;
        }
    }
    thread_free(&th);
    return POV_GPU_OK;
}

int pov_oracle_count_work(PovOracle* S, const double* org, const double* dir, int32_t n,
                          uint64_t* boxes, uint64_t* prims)
{
    Thread th;
    memset(&th, 0, sizeof(th));
    th.counting = 1;
    for (int32_t i = 0; i < n; i++) {
        Isect is;
        find_intersection(S, &th, vload(org + 3 * i), vload(dir + 3 * i), HUGE_VAL, 0, &is);
    }
    *boxes = th.boxes;
    *prims = th.prims;
    thread_free(&th);
    return POV_GPU_OK;
}

/* TracePixel::operator() + CreateCameraRay (tracepixel.cpp:311-373,924). */
static void trace_pixel(const PovOracle* S, Thread* th, double x, double y, double w, double h, float* rgbt)
{
    const PovGpuCamera* c = &S->desc.camera;
    double x0 = x / w - 0.5;
    double y0 = 0.5 - y / h;
    V3 D = vadd(vadd(vload(c->direction), vmul(vload(c->right), x0)), vmul(vload(c->up), y0));
    D = vnorm(D);
    RGB col;
    Ticket tk = {0, S->desc.max_trace_level, S->desc.adc_bailout, 0, 1.0f};
    trace_ray(S, th, vload(c->location), D, 1.0, &tk, 0, &col);
    rgbt[0] = col.r;
    rgbt[1] = col.g;
    rgbt[2] = col.b;
    rgbt[3] = 0.0f;
}

typedef struct {
    PovOracle* S;
    const PovGpuRenderParams* p;
    int32_t x0, y0, x1, y1;
    float* out;
    int32_t next_row;
    pthread_mutex_t lock;
    PovGpuStats stats;
    int32_t next_block;
} RenderJob;

/* ---------------------------------------- adaptive antialiasing (M2) --- */
typedef struct { float r, g, b, t; } Col4;

static Col4 trace_sample(const PovOracle* S, Thread* th, double x, double y, double w, double h)
{
    float c[4];
    trace_pixel(S, th, x, y, w, h, c);
    Col4 r = {c[0], c[1], c[2], c[3]};
    return r;
}

/* AA gamma: PowerLawGammaCurve with decoding gamma 2.5 (view.cpp:724-728,
 * colourspace.cpp:310): pow(max(x, 0), 1/2.5) per colour channel. */
static Col4 aa_encode(Col4 c)
{
    const float g = 1.0f / 2.5f;
    Col4 r = {powf(fmaxf(c.r, 0.0f), g), powf(fmaxf(c.g, 0.0f), g), powf(fmaxf(c.b, 0.0f), g), c.t};
    return r;
}

static float col_dist(Col4 a, Col4 b)   /* ColourDistanceRGBT (base/colour.h:1221) */
{
    return fabsf(a.r - b.r) + fabsf(a.g - b.g) + fabsf(a.b - b.b) + fabsf(a.t - b.t);
}

typedef struct {
    Col4*    col;
    uint8_t* sampled;
    int      size;
} SubBuf;

static void subbuf_set(SubBuf* B, int x, int y, Col4 c)
{
    B->col[x + y * B->size] = c;
    B->sampled[x + y * B->size] = 1;
}

/* TraceTask::SubdivideOnePixel (tracetask.cpp:892-1063), jitter off. */
static void subdivide_one_pixel(const PovOracle* S, Thread* th, const PovGpuRenderParams* p, double x, double y,
                                double d, int bx, int by, int bstep, SubBuf* B, Col4* result, int level,
                                uint64_t* samples)
{
    Col4 c00 = B->col[bx + by * B->size], c02 = B->col[bx + (by + bstep) * B->size];
    Col4 c20 = B->col[bx + bstep + by * B->size], c22 = B->col[bx + bstep + (by + bstep) * B->size];
    int h = bstep / 2;
    double thr = (double)p->aa_threshold;
    Col4 g00 = aa_encode(c00), g02 = aa_encode(c02), g20 = aa_encode(c20), g22 = aa_encode(c22);
    double W = p->width, H = p->height;
    if (level > 0 && (col_dist(g00, g02) >= thr || col_dist(g00, g20) >= thr || col_dist(g00, g22) >= thr ||
                      col_dist(g02, g20) >= thr || col_dist(g02, g22) >= thr || col_dist(g20, g22) >= thr)) {
        double d2 = d * 0.5;
        if (!B->sampled[bx + (by + h) * B->size]) {
            subbuf_set(B, bx, by + h, trace_sample(S, th, x + 0.5 - d, y + 0.5, W, H));
            (*samples)++;
        }
        if (!B->sampled[bx + h + by * B->size]) {
            subbuf_set(B, bx + h, by, trace_sample(S, th, x + 0.5, y + 0.5 - d, W, H));
            (*samples)++;
        }
        if (!B->sampled[bx + bstep + (by + h) * B->size]) {
            subbuf_set(B, bx + bstep, by + h, trace_sample(S, th, x + 0.5 + d, y + 0.5, W, H));
            (*samples)++;
        }
        if (!B->sampled[bx + h + (by + bstep) * B->size]) {
            subbuf_set(B, bx + h, by + bstep, trace_sample(S, th, x + 0.5, y + 0.5 + d, W, H));
            (*samples)++;
        }
        if (!B->sampled[bx + h + (by + h) * B->size]) {
            subbuf_set(B, bx + h, by + h, trace_sample(S, th, x + 0.5, y + 0.5, W, H));
            (*samples)++;
        }
        Col4 r00, r01, r10, r11;
        subdivide_one_pixel(S, th, p, x - d2, y - d2, d2, bx, by, h, B, &r00, level - 1, samples);
        subdivide_one_pixel(S, th, p, x - d2, y + d2, d2, bx, by + h, h, B, &r01, level - 1, samples);
        subdivide_one_pixel(S, th, p, x + d2, y - d2, d2, bx + h, by, h, B, &r10, level - 1, samples);
        subdivide_one_pixel(S, th, p, x + d2, y + d2, d2, bx + h, by + h, h, B, &r11, level - 1, samples);
        result->r = (r00.r + r01.r + r10.r + r11.r) / 4.0f;
        result->g = (r00.g + r01.g + r10.g + r11.g) / 4.0f;
        result->b = (r00.b + r01.b + r10.b + r11.b) / 4.0f;
        result->t = (r00.t + r01.t + r10.t + r11.t) / 4.0f;
    } else {
        result->r = (c00.r + c02.r + c20.r + c22.r) / 4.0f;
        result->g = (c00.g + c02.g + c20.g + c22.g) / 4.0f;
        result->b = (c00.b + c02.b + c20.b + c22.b) / 4.0f;
        result->t = (c00.t + c02.t + c20.t + c22.t) / 4.0f;
    }
}

/* TraceTask::AdaptiveSupersamplingM2 (tracetask.cpp:604-657) over the
 * view's 32x32 block grid; pixels outside the requested rectangle are
 * traced (block corners) but not written. */
static void* render_worker_aa(void* arg)
{
    RenderJob* J = (RenderJob*)arg;
    const PovGpuRenderParams* p = J->p;
    Thread th;
    memset(&th, 0, sizeof(th));
    const int bs = 32;
    int nbx = (p->width + bs - 1) / bs, nby = (p->height + bs - 1) / bs;
    int depth = p->aa_depth < 1 ? 1 : p->aa_depth;
    int subsize = 1 << depth;
    SubBuf B;
    B.size = subsize + 1;
    B.col = (Col4*)malloc(sizeof(Col4) * B.size * B.size);
    B.sampled = (uint8_t*)malloc((size_t)B.size * B.size);
    Col4* corners = (Col4*)malloc(sizeof(Col4) * (bs + 1) * (bs + 1));
    uint64_t pixels = 0, samples = 0;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int b = J->next_block++;
        pthread_mutex_unlock(&J->lock);
        if (b >= nbx * nby)
            break;
        int left = (b % nbx) * bs, top = (b / nbx) * bs;
        int right = left + bs - 1 < p->width - 1 ? left + bs - 1 : p->width - 1;
        int bottom = top + bs - 1 < p->height - 1 ? top + bs - 1 : p->height - 1;
        if (right < J->x0 || left >= J->x1 || bottom < J->y0 || top >= J->y1)
            continue;
        int cw = right - left + 2;
        for (int y = top; y <= bottom + 1; y++)
            for (int x = left; x <= right + 1; x++) {
                corners[(y - top) * cw + (x - left)] = trace_sample(J->S, &th, x, y, p->width, p->height);
                pixels++;
            }
        for (int y = top; y <= bottom; y++)
            for (int x = left; x <= right; x++) {
                memset(B.sampled, 0, (size_t)B.size * B.size);
                subbuf_set(&B, 0, 0, corners[(y - top) * cw + (x - left)]);
                subbuf_set(&B, 0, subsize, corners[(y + 1 - top) * cw + (x - left)]);
                subbuf_set(&B, subsize, 0, corners[(y - top) * cw + (x + 1 - left)]);
                subbuf_set(&B, subsize, subsize, corners[(y + 1 - top) * cw + (x + 1 - left)]);
                Col4 r;
                subdivide_one_pixel(J->S, &th, p, x, y, 0.5, 0, 0, subsize, &B, &r, depth - 1, &samples);
                if (x >= J->x0 && x < J->x1 && y >= J->y0 && y < J->y1) {
                    float* o = J->out + ((size_t)(y - J->y0) * (J->x1 - J->x0) + (x - J->x0)) * 4;
                    o[0] = r.r; o[1] = r.g; o[2] = r.b; o[3] = r.t;
                }
            }
    }
    pthread_mutex_lock(&J->lock);
    J->stats.number_of_rays += th.rays;
    J->stats.shadow_ray_tests += th.shadow_tests;
    J->stats.shadow_rays_succeeded += th.shadow_succeeded;
    J->stats.reflected_rays += th.reflected;
    J->stats.refracted_rays += th.refracted;
    J->stats.internal_reflected_rays += th.internal_reflected;
    J->stats.transmitted_rays += th.transmitted;
    J->stats.media_samples += th.media_samples;
    J->stats.number_of_pixels += pixels;
    J->stats.number_of_samples += samples;
    pthread_mutex_unlock(&J->lock);
    free(B.col);
    free(B.sampled);
    free(corners);
    thread_free(&th);
    return NULL;
}

static void* render_worker(void* arg)
{
    RenderJob* J = (RenderJob*)arg;
    Thread th;
    memset(&th, 0, sizeof(th));
    int32_t w = J->x1 - J->x0;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int32_t y = J->next_row++;
        pthread_mutex_unlock(&J->lock);
        if (y >= J->y1)
            break;
        for (int32_t x = J->x0; x < J->x1; x++)
            trace_pixel(J->S, &th, x + 0.5, y + 0.5, J->p->width, J->p->height,
                        J->out + ((size_t)(y - J->y0) * w + (x - J->x0)) * 4);
    }
    pthread_mutex_lock(&J->lock);
    J->stats.number_of_rays += th.rays;
    J->stats.shadow_ray_tests += th.shadow_tests;
    J->stats.shadow_rays_succeeded += th.shadow_succeeded;
    J->stats.reflected_rays += th.reflected;
    J->stats.refracted_rays += th.refracted;
    J->stats.internal_reflected_rays += th.internal_reflected;
    J->stats.transmitted_rays += th.transmitted;
    J->stats.media_samples += th.media_samples;
    pthread_mutex_unlock(&J->lock);
    thread_free(&th);
    return NULL;
}

/* Radiosity render in the reference's single-thread order: the pretrace
 * of View::StartRender (view.cpp:1056-1123) as RadiosityTask::Run
 * (radiositytask.cpp:95-263) runs it without high reproducibility -- pass
 * after pass over the 32x32 blocks in serial order, jitter from the task's
 * table -- then the final trace block by block (TraceTask::SimpleSamplingM0,
 * tracetask.cpp:403-454) with a fresh
 * RadiosityFunction (final trace: full error bound, own direction
 * sequences) on the same cache. */
static int render_radiosity(PovOracle* S, const PovGpuRenderParams* p, int32_t x0, int32_t y0, int32_t x1,
                            int32_t y1, float* out, PovGpuStats* stats)
{
    RadCache* R = S->rad;
    const PovGpuRadiosity* rs = &S->desc.radiosity;
    if (!R->jitter || p->antialias)
        return POV_GPU_E_UNSUPPORTED;
    rad_reset(R);
    /* the view's blocks tile the render area from its top-left corner
     * (ViewData::GetNextRectangle, view.cpp:384-388); pass spacing follows
     * the full image size */
    const int W = p->width, H = p->height, B = 32;
    const int AW = x1 - x0, AH = y1 - y0;
    const int bw = (AW + B - 1) / B, bh = (AH + B - 1) / B, nb = bw * bh;
    Thread th;
    memset(&th, 0, sizeof(th));
    double maxwh = (double)(W > H ? W : H);
    double start = maxwh * rs->pretrace_start, end = maxwh * rs->pretrace_end;
    if (end < 1.0)
        end = 1.0;
    int steps = (int)floor(log(start / end) / log(2.0) + (1.0 - EPSILON)) + 1;
    if (steps > 253) {
        steps = 253;
        start = end * pow(2.0, (double)steps);
    }
    /* pretrace task */
    th.rad_final = 0;
    th.rad_error_bound = rs->error_bound * rs->low_error_factor;
    char* active = (char*)malloc((size_t)nb);
    memset(active, 1, (size_t)nb);
    float rgbt[4];
    for (int pass = 0; pass < steps; pass++) {
        double size = fmax(start * pow(0.5f, (float)pass), end);
        double jit = fmin(1.0, size / 2.0), offset = (size - 1.0) / 2.0;
        for (int serial = 0; serial < nb; serial++) {
            if (!active[serial])
                continue;
            int left = x0 + (serial % bw) * B, top = y0 + (serial / bw) * B;
            int right = left + B - 1 < x1 - 1 ? left + B - 1 : x1 - 1;
            int bottom = top + B - 1 < y1 - 1 ? top + B - 1 : y1 - 1;
            th.rad_pass = PASS_FIRST + pass;
            size_t ji = (size_t)((PASS_FIRST + pass) * 17 + serial * 13) % (size_t)R->njitter;
            double sx = ceil((left - 0.5) / size) * size, sy = ceil((top - 0.5) / size) * size;
            double ex = left + (double)(right - left + 1), ey = top + (double)(bottom - top + 1);
            th.rad_top_queries = 0;
            int count = 0;
            for (double y = sy; y < ey; y += size) {
                if (y < top)
                    continue;
                for (double x = sx; x < ex; x += size) {
                    if (x < left)
                        continue;
                    /* the reference's compiler evaluates the second
                     * argument's jitter first */
                    ji = (ji + 1) % (size_t)R->njitter;
                    double jy = R->jitter[ji];
                    ji = (ji + 1) % (size_t)R->njitter;
                    double jx = R->jitter[ji];
                    trace_pixel(S, &th, x + offset + jit * jx, y + offset + jit * jy, W, H, rgbt);
                    count++;
                }
            }
            R->pixels += (uint64_t)count;
            /* another pass unless the block saw no radiosity query at all */
            if (count >= 9 && th.rad_top_queries == 0)
                active[serial] = 0;
        }
    }
    free(active);
    /* final trace */
    memset(th.rad_dir_index, 0, sizeof(th.rad_dir_index));
    th.rad_final = 1;
    th.rad_error_bound = rs->error_bound;
    th.rad_pass = PASS_FINAL;
    int32_t w = x1 - x0;
    for (int serial = 0; serial < nb; serial++) {
        int left = x0 + (serial % bw) * B, top = y0 + (serial / bw) * B;
        for (int y = top; y < top + B && y < y1; y++)
            for (int x = left; x < left + B && x < x1; x++)
                trace_pixel(S, &th, x + 0.5, y + 0.5, W, H, out + ((size_t)(y - y0) * w + (x - x0)) * 4);
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->number_of_rays = th.rays;
        stats->shadow_ray_tests = th.shadow_tests;
        stats->shadow_rays_succeeded = th.shadow_succeeded;
        stats->reflected_rays = th.reflected;
        stats->refracted_rays = th.refracted;
        stats->internal_reflected_rays = th.internal_reflected;
        stats->transmitted_rays = th.transmitted;
        stats->media_samples = th.media_samples;
        stats->number_of_pixels = (uint64_t)(x1 - x0) * (uint64_t)(y1 - y0) + R->pixels;
        stats->radiosity_gathers = R->gathers;
        stats->radiosity_reuse = R->reused;
        stats->radiosity_rays = R->rays;
        stats->radiosity_gathers_d0 = R->gathers_depth[0];
        stats->radiosity_gathers_d1 = R->gathers_depth[1];
    }
    thread_free(&th);
    return POV_GPU_OK;
}

typedef struct {
    PovOracle* S;
    const PovGpuRenderParams* p;
    const int32_t* px;
    int32_t n, next;
    uint64_t seed;
    float* out;
    PovGpuStats stats;
    pthread_mutex_t lock;
} ConvergedJob;

static void* converged_worker(void* arg)
{
    ConvergedJob* J = (ConvergedJob*)arg;
    Thread th;
    memset(&th, 0, sizeof(th));
    th.rad_final = 1;
    th.rad_pass = PASS_FINAL;
    th.rad_error_bound = J->S->desc.radiosity.error_bound;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int32_t i = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (i >= J->n)
            break;
        int32_t x = J->px[2 * i], y = J->px[2 * i + 1];
        th.gt_rng = J->seed ^ ((uint64_t)(uint32_t)y << 32 | (uint32_t)x) * 0xD1B54A32D192ED03ull;
        trace_pixel(J->S, &th, x + 0.5, y + 0.5, J->p->width, J->p->height, J->out + (size_t)i * 4);
    }
    pthread_mutex_lock(&J->lock);
    J->stats.number_of_rays += th.rays;
    J->stats.shadow_ray_tests += th.shadow_tests;
    J->stats.shadow_rays_succeeded += th.shadow_succeeded;
    pthread_mutex_unlock(&J->lock);
    thread_free(&th);
    return NULL;
}

int pov_oracle_render_converged(PovOracle* S, const PovGpuRenderParams* p, const int32_t* pixels, int32_t n,
                                const int32_t* counts, int32_t ncounts, uint64_t seed, int32_t threads,
                                float* out, PovGpuStats* stats)
{
    if (!S || !p || !S->rad || !S->desc.radiosity.enabled || (n > 0 && (!pixels || !out)) || !counts ||
        ncounts < 1 || ncounts > 8 || counts[0] < 1 || p->antialias)
        return POV_GPU_E_INVALID;
    ConvergedJob J;
    memset(&J, 0, sizeof(J));
    J.S = S; J.p = p; J.px = pixels; J.n = n; J.seed = seed; J.out = out;
    pthread_mutex_init(&J.lock, NULL);
    for (int d = 0; d < 8; d++)
        S->gt_count[d] = counts[d < ncounts ? d : ncounts - 1];
    if (threads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        threads = c > 0 ? (int32_t)c : 1;
    }
    pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    for (int i = 0; i < threads; i++)
        pthread_create(&tids[i], NULL, converged_worker, &J);
    for (int i = 0; i < threads; i++)
        pthread_join(tids[i], NULL);
    free(tids);
    memset(S->gt_count, 0, sizeof(S->gt_count));
    pthread_mutex_destroy(&J.lock);
    J.stats.number_of_pixels = (uint64_t)n;
    if (stats)
        *stats = J.stats;
    return POV_GPU_OK;
}

int pov_oracle_set_pretrace_jitter(PovOracle* S, const double* table, int32_t n)
{
    if (!S || !S->rad || !table || n <= 0)
        return POV_GPU_E_INVALID;
    S->rad->jitter = table;
    S->rad->njitter = n;
    return POV_GPU_OK;
}

int pov_oracle_render(PovOracle* S, const PovGpuRenderParams* p, int32_t x0, int32_t y0, int32_t x1,
                      int32_t y1, int32_t threads, float* out, PovGpuStats* stats)
{
    if (!S || !p || !out || x1 < x0 || y1 < y0)
        return POV_GPU_E_INVALID;
    if (S->desc.radiosity.enabled)
        return render_radiosity(S, p, x0, y0, x1, y1, out, stats);
    int aa = p->antialias != 0;
    if (aa && (p->sampling_method != 2 || p->jitter))
        return POV_GPU_E_UNSUPPORTED;
    RenderJob J;
    memset(&J, 0, sizeof(J));
    J.S = S; J.p = p; J.x0 = x0; J.y0 = y0; J.x1 = x1; J.y1 = y1; J.out = out; J.next_row = y0;
    pthread_mutex_init(&J.lock, NULL);
    if (threads <= 0) {
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (int32_t)n : 1;
    }
    void* (*worker)(void*) = aa ? render_worker_aa : render_worker;
    if (threads == 1) {
        worker(&J);
    } else {
        pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * threads);
        for (int i = 0; i < threads; i++)
            pthread_create(&tids[i], NULL, worker, &J);
        for (int i = 0; i < threads; i++)
            pthread_join(tids[i], NULL);
        free(tids);
    }
    pthread_mutex_destroy(&J.lock);
    if (!aa)
        J.stats.number_of_pixels = (uint64_t)(x1 - x0) * (uint64_t)(y1 - y0);
    if (stats)
        *stats = J.stats;
    return POV_GPU_OK;
}
