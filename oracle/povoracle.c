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
 *     (source/core/render/trace.cpp:1990-2025) is not restated; it only
 *     changes Shadow_Cache_Hits, which depends on render order anyway.
 *   - the mesh best-first loop's early "Depth > Best" exit uses the best
 *     hit so far (source/core/shape/mesh.cpp:1499 keeps the last one).
 */
#include "povoracle.h"

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
    int32_t triangle;
} Isect;

typedef struct {
    PQueue  pq;       /* top-level queue */
    PQueue  mpq;      /* mesh queue (mesh.cpp:110 keeps a thread-local one) */
    uint64_t boxes, prims;
    int     counting;
    /* statistics of the render */
    uint64_t rays, shadow_tests, shadow_succeeded, reflected;
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

/* Per-object closest hit: Find_Intersection (object.cpp:118-168,172-225)
 * with All_Intersections of the shape; `min_depth` is MIN_ISECT_DEPTH,
 * raised by a postcondition (SMALL_TOLERANCE for shadow rays). */
static int object_closest(const PovOracle* S, Thread* th, int32_t oi, V3 O, V3 D, double min_depth,
                          double closest, Isect* out)
{
    const OObj* ob = &S->objs[oi];
    const PovGpuObject* o = &ob->o;
    double best = closest;
    int found = 0;
    if (th->counting) th->prims++;
    switch (o->type) {
    case POV_OBJ_SPHERE: {
        double d1, d2;
        V3 C = v3(o->p[0], o->p[1], o->p[2]);
        if (sphere_intersect(O, D, C, o->p[3] * o->p[3], &d1, &d2)) {
            /* both roots are pushed; the stack is scanned for the closest */
            if (d1 > SPHERE_DEPTH_TOLERANCE && d1 < MAX_DISTANCE && d1 >= min_depth && d1 < best) {
                best = d1; found = 1;
            }
            if (d2 > SPHERE_DEPTH_TOLERANCE && d2 < MAX_DISTANCE && d2 >= min_depth && d2 < best) {
                best = d2; found = 1;
            }
        }
        if (found) { out->triangle = -1; }
        break;
    }
    case POV_OBJ_PLANE: {   /* Plane::Intersect (plane.cpp:139-211) */
        V3 N = v3(o->p[0], o->p[1], o->p[2]);
        double ndd = vdot(N, D);
        if (fabs(ndd) < EPSILON)
            break;
        double ndo = vdot(N, O);
        double t = -(ndo + o->p[3]) / ndd;
        if (t >= PLANE_DEPTH_TOLERANCE && t <= MAX_DISTANCE && t >= min_depth && t < best) {
            best = t; found = 1; out->triangle = -1;
        }
        break;
    }
    case POV_OBJ_MESH: {
        if (!intersect_bbox_dir(&ob->bbox, O, D, (float)closest))
            break;
        double t;
        int32_t tri = -1;
        if (mesh_closest(&S->meshes[o->mesh], th, O, D, min_depth, best, &t, &tri)) {
            best = t; found = 1; out->triangle = tri;
        }
        break;
    }
    default:
        break;
    }
    if (found) {
        out->depth = best;
        out->object = oi;
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

/* Trace::TraceShadowRay / TracePointLightShadowRay for opaque scenes
 * (trace.cpp:1892-2076): 1 = light blocked. */
static int shadow_blocked(const PovOracle* S, Thread* th, V3 P, V3 L, double dist)
{
    Isect is;
    th->shadow_tests++;   /* Shadow_Ray_Tests (trace.cpp:2032) */
    if (find_intersection(S, th, P, L, dist, 1, &is)) {
        if (is.depth < dist - SHADOW_TOLERANCE && is.depth > SHADOW_TOLERANCE) {
            th->shadow_succeeded++;
            return 1;
        }
    }
    return 0;
}

static void trace_ray(const PovOracle* S, Thread* th, V3 O, V3 D, double weight, int level, RGB* col);

/* ComputeReflection (trace.cpp:1264-1321). */
static void compute_reflection(const PovOracle* S, Thread* th, V3 ip, V3 D, V3 N, V3 raw, double weight,
                               int level, RGB* col)
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
    trace_ray(S, th, ip, nd, weight, level, col);
}

/* ComputeTextureColour + ComputeLightedTexture (trace.cpp:457-586,739-1179)
 * for one plain layer with an opaque pigment. */
static void shade(const PovOracle* S, Thread* th, const Isect* is, V3 D, double weight, int level, RGB* out)
{
    const PovGpuObject* o = &S->objs[is->object].o;
    const PovGpuMaterial* m = object_material(S, is->object);
    V3 raw = object_normal(S, is);
    if (o->flags & POV_FLAG_INVERTED)
        raw = vmul(raw, -1.0);
    if (vdot(raw, D) > 0.0)
        raw = vmul(raw, -1.0);
    V3 N = raw;
    V3 ip = is->ipoint;
    RGB pig = {m->pigment[0], m->pigment[1], m->pigment[2]};
    double r = 0.0, g = 0.0, b = 0.0;

    /* ComputeReflectivity (trace.cpp:2627-2656), non-fresnel */
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

    /* emission + ambient * ambient_light (radiosity off, trace.cpp:984-1004) */
    double em[3];
    for (int k = 0; k < 3; k++)
        em[k] = m->emission[k] + m->ambient[k] * S->desc.ambient_light[k];
    r += pig.r * em[0];
    g += pig.g * em[1];
    b += pig.b * em[2];

    /* ComputeDiffuseLight (trace.cpp:1488-1510,1637-1729) */
    if (m->diffuse != 0.0f || m->diffuse_back != 0.0f || m->specular != 0.0f || m->phong != 0.0f) {
        for (int li = 0; li < S->nlights; li++) {
            const PovGpuLight* L = &S->lights[li];
            V3 C = vload(L->center);
            V3 ld = vsub(C, ip);
            double ldist = vlen(ld);
            ld = vdiv(ld, ldist);
            double lc[3] = {L->colour[0], L->colour[1], L->colour[2]};
            if (fabs(lc[0]) < EPSILON && fabs(lc[1]) < EPSILON && fabs(lc[2]) < EPSILON)
                continue;
            if (!(o->flags & POV_FLAG_DOUBLE_ILLUM)) {
                double cs = vdot(N, ld);
                if (cs < EPSILON)
                    continue;
            }
            if (level <= S->desc.max_trace_level) {   /* TraceShadowRay level check */
                if (shadow_blocked(S, th, ip, ld, ldist))
                    continue;
            }
            /* ComputeDiffuseColour (trace.cpp:2441-2484) */
            double diffuse = m->diffuse * m->brilliance_adjust;
            if (diffuse > 0.0) {
                double ci = vdot(N, ld);
                double inten = m->brilliance != 1.0f ? pow(fabs(ci), m->brilliance) : fabs(ci);
                inten *= diffuse;
                r += inten * pig.r * lc[0];
                g += inten * pig.g * lc[1];
                b += inten * pig.b * lc[2];
            }
            /* ComputePhongColour (trace.cpp:2520-2558) */
            if (m->phong > 0.0f) {
                double c2 = -2.0 * vdot(D, N);
                V3 rd = vadd(D, vmul(N, c2));
                double ci = vdot(rd, ld);
                if (ci > 0.0 && (m->phong_size < 60 || ci > 0.0008)) {
                    double inten = m->phong * pow(ci, (double)m->phong_size);
                    r += inten * lc[0];
                    g += inten * lc[1];
                    b += inten * lc[2];
                }
            }
            /* ComputeSpecularColour (trace.cpp:2560-2593) */
            if (m->specular > 0.0f) {
                V3 half = vmul(vadd(vmul(D, -1.0), ld), 0.5);
                double hl = vlen(half);
                if (hl > 0.0) {
                    double ci = vdot(half, N) / hl;
                    if (ci > 0.0) {
                        double inten = m->specular * pow(ci, (double)m->roughness);
                        r += inten * lc[0];
                        g += inten * lc[1];
                        b += inten * lc[2];
                    }
                }
            }
        }
    }

    /* reflected component (trace.cpp:1155-1178) */
    if (!(reflec.r == 0.0f && reflec.g == 0.0f && reflec.b == 0.0f)) {
        RGB rc = {0, 0, 0};
        compute_reflection(S, th, ip, D, N, raw, rweight, level, &rc);
        r += reflec.r * rc.r;
        g += reflec.g * rc.g;
        b += reflec.b * rc.b;
    }
    out->r = (float)r;
    out->g = (float)g;
    out->b = (float)b;
}

/* Trace::TraceRay (trace.cpp:135-228).  `level` is the trace level before
 * this ray (TraceTicket::traceLevel). */
static void trace_ray(const PovOracle* S, Thread* th, V3 O, V3 D, double weight, int level, RGB* col)
{
    th->rays++;   /* Number_Of_Rays */
    col->r = col->g = col->b = 0.0f;
    if (level >= S->desc.max_trace_level || weight < S->desc.adc_bailout)
        return;
    Isect is;
    if (find_intersection(S, th, O, D, HUGE_VAL, 0, &is)) {
        shade(S, th, &is, D, weight, level + 1, col);
    } else {
        /* ComputeSky: background only (trace.cpp:2839-2888) */
        col->r = S->desc.background[0];
        col->g = S->desc.background[1];
        col->b = S->desc.background[2];
    }
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
    PovOracle* S = (PovOracle*)calloc(1, sizeof(PovOracle));
    S->desc = *desc;
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
    for (int i = 0; i < S->nobjs; i++) {
        S->objs[i].o = desc->objects[i];
        const PovGpuObject* o = &S->objs[i].o;
        if (o->type != POV_OBJ_SPHERE && o->type != POV_OBJ_PLANE && o->type != POV_OBJ_MESH) {
            if (bad_index) *bad_index = i;
            free(finite); free(infinite);
            pov_oracle_destroy(S);
            return POV_GPU_E_UNSUPPORTED;
        }
        S->objs[i].bbox = object_bbox(S, o);
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
    *out = S;
    return POV_GPU_OK;
}

static void free_tree(Tree* t) { free(t->nodes); free(t->kids); }

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
            hits[i].triangle = is.triangle;
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
    trace_ray(S, th, vload(c->location), D, 1.0, 0, &col);
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
} RenderJob;

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
    pthread_mutex_unlock(&J->lock);
    thread_free(&th);
    return NULL;
}

int pov_oracle_render(PovOracle* S, const PovGpuRenderParams* p, int32_t x0, int32_t y0, int32_t x1,
                      int32_t y1, int32_t threads, float* out, PovGpuStats* stats)
{
    if (!S || !p || !out || x1 < x0 || y1 < y0)
        return POV_GPU_E_INVALID;
    if (p->antialias)
        return POV_GPU_E_UNSUPPORTED;
    RenderJob J;
    memset(&J, 0, sizeof(J));
    J.S = S; J.p = p; J.x0 = x0; J.y0 = y0; J.x1 = x1; J.y1 = y1; J.out = out; J.next_row = y0;
    pthread_mutex_init(&J.lock, NULL);
    if (threads <= 0) {
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (int32_t)n : 1;
    }
    if (threads == 1) {
        render_worker(&J);
    } else {
        pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * threads);
        for (int i = 0; i < threads; i++)
            pthread_create(&tids[i], NULL, render_worker, &J);
        for (int i = 0; i < threads; i++)
            pthread_join(tids[i], NULL);
        free(tids);
    }
    pthread_mutex_destroy(&J.lock);
    J.stats.number_of_pixels = (uint64_t)(x1 - x0) * (uint64_t)(y1 - y0);
    if (stats)
        *stats = J.stats;
    return POV_GPU_OK;
}
