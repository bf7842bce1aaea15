/*
 * octbuild.c -- host octree builder over loaded scene objects.
 *
 * Restates the reference's oconv algorithm so that scene text can be turned
 * into the same octree the reference programs would read:
 *   - bounding cube from the surfaces' extent plus a 1e-5 margin, centred on
 *     the bounding box (ot/oconv.c:128-150; add2bbox ot/bbox.c:24-95);
 *   - objects added in definition order (ot/oconv.c:216-246);
 *   - a full node is split once it holds objlim objects, unless the child
 *     cube would be smaller than cusize/resolu - 1e-6 (ot/oconv.c:256-330),
 *     surfaces re-added first, then the new object, then volumes;
 *   - face/cube overlap by vertex location, Cohen-Sutherland edge clipping
 *     and the plane test (ot/o_face.c:40-99, common/clip.c:19-72,
 *     common/plocate.c); sphere/cube by ot/sphere.c:50-109; cones, cups,
 *     cylinders, tubes and rings by the strict test of ot/o_cone.c:41-126;
 *   - identical sibling leaves merged (common/octree.c:73-90).
 */
#include "scene.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define O_MISS 0
#define O_HIT 1

typedef struct {
    int32_t kids[8];     /* -1 none; only for trees */
    int32_t *set;        /* leaf set (sorted), NULL for tree/empty */
    int32_t n, cap;
    int     tree;
} bnode;

typedef struct {
    gb_scene_host *S;
    bnode *nodes;
    int32_t nn, cap;
    int objlim;
    double mincusize;
    int err;
} builder;

static int32_t bnew(builder *B)
{
    if (B->nn == B->cap) {
        int32_t nc = B->cap ? B->cap * 2 : 4096;
        bnode *p = (bnode *)realloc(B->nodes, (size_t)nc * sizeof *p);
        if (!p) {
            B->err = 1;
            return -1;
        }
        B->nodes = p;
        B->cap = nc;
    }
    memset(&B->nodes[B->nn], 0, sizeof(bnode));
    return B->nn++;
}

static int set_insert(bnode *nd, int32_t obj)
{
    int32_t i;
    for (i = nd->n; i > 0 && nd->set[i - 1] > obj; i--)
        ;
    if (i > 0 && nd->set[i - 1] == obj)   /* already present */
        return 0;
    if (nd->n == nd->cap) {
        int32_t nc = nd->cap ? nd->cap * 2 : 8;
        int32_t *p = (int32_t *)realloc(nd->set, (size_t)nc * sizeof *p);
        if (!p)
            return -1;
        nd->set = p;
        nd->cap = nc;
    }
    memmove(nd->set + i + 1, nd->set + i, (size_t)(nd->n - i) * sizeof(int32_t));
    nd->set[i] = obj;
    nd->n++;
    return 0;
}

/* ---- geometry tests (ot/o_face.c, common/clip.c, common/plocate.c) ---- */

#define XPOS 03
#define YPOS 014
#define ZPOS 060
#define POSITION(i) (3 << ((i) << 1))
#define BELOW 025
#define ABOVE 052

static int plocate(const double p[3], const double mn[3], const double mx[3])
{
    int loc = 0;
    const double E = GB_FTINY;
    if (p[0] < mn[0] - E) loc |= XPOS & BELOW;
    else if (p[0] > mx[0] + E) loc |= XPOS & ABOVE;
    if (p[1] < mn[1] - E) loc |= YPOS & BELOW;
    else if (p[1] > mx[1] + E) loc |= YPOS & ABOVE;
    if (p[2] < mn[2] - E) loc |= ZPOS & BELOW;
    else if (p[2] > mx[2] + E) loc |= ZPOS & ABOVE;
    return loc;
}

static int clip_seg(double *ep1, double *ep2, const double mn[3], const double mx[3])
{
    int itlim = 6, loc1, loc2, accept, i, j;
    double *dp, d;
    loc1 = plocate(ep1, mn, mx);
    loc2 = plocate(ep2, mn, mx);
    while (!((accept = !(loc1 | loc2)) || (loc1 & loc2))) {
        if (itlim-- <= 0)
            return 0;
        if (!loc1) {
            dp = ep1; ep1 = ep2; ep2 = dp;
            i = loc1; loc1 = loc2; loc2 = i;
        }
        for (i = 0; i < 3; i++) {
            if (loc1 & POSITION(i) & BELOW) {
                d = (mn[i] - ep1[i]) / (ep2[i] - ep1[i]);
                ep1[i] = mn[i];
            } else if (loc1 & POSITION(i) & ABOVE) {
                d = (mx[i] - ep1[i]) / (ep2[i] - ep1[i]);
                ep1[i] = mx[i];
            } else
                continue;
            for (j = 0; j < 3; j++)
                if (j != i)
                    ep1[j] += (ep2[j] - ep1[j]) * d;
            break;
        }
        loc1 = plocate(ep1, mn, mx);
    }
    return accept;
}

/* point in polygon on the dominant projection (common/face.c:121-161) */
static int inface_host(const double p[3], const gb_face *f, const double *va)
{
    int ncross = 0, n = f->nv, tst, xi, yi;
    double x, y;
    const double *p0, *p1;
    if ((xi = f->ax + 1) >= 3) xi -= 3;
    if ((yi = xi + 1) >= 3) yi -= 3;
    x = p[xi];
    y = p[yi];
    p0 = va + 3 * (n - 1);
    p1 = va;
#define FEQ(a, b) (fabs((a) - (b)) <= GB_FTINY)
    while (n--) {
        if (FEQ(p0[yi], y) && FEQ(p1[yi], y) && ((p0[xi] > x) ^ (p1[xi] > x)))
            return 1;
        if ((p0[yi] > y) ^ (p1[yi] > y)) {
            tst = (p0[xi] > x) + (p1[xi] > x);
            if (tst == 2)
                ncross++;
            else if (tst) {
                double prodA = (p0[yi] - y) * (p1[xi] - x);
                double prodB = (p0[xi] - x) * (p1[yi] - y);
                if (FEQ(prodA, prodB))
                    return 1;
                ncross += (p1[yi] > p0[yi]) ^ (prodA > prodB);
            } else if (FEQ(p0[xi], x) && FEQ(p1[xi], x))
                return 1;
        }
        p0 = p1;
        p1 += 3;
    }
#undef FEQ
    return ncross & 1;
}

static int face_cube(const gb_object *o, const gb_face *f, const double org[3], double size)
{
    double cumin[3], cumax[3], v1[3], v2[3], d1, d2;
    const double *va = o->farg;
    int vloc, i, j;
    if (!f->ok)
        return O_MISS;
    for (j = 0; j < 3; j++) {
        cumin[j] = org[j] - GB_FTINY;
        cumax[j] = cumin[j] + size + 2.0 * GB_FTINY;
    }
    vloc = ABOVE | BELOW;
    for (i = 0; i < f->nv; i++) {
        if ((j = plocate(va + 3 * i, cumin, cumax)))
            vloc &= j;
        else
            return O_HIT;
    }
    if (vloc)
        return O_MISS;
    for (i = 0; i < f->nv; i++) {
        if ((j = i + 1) >= f->nv)
            j = 0;
        memcpy(v1, va + 3 * i, sizeof v1);
        memcpy(v2, va + 3 * j, sizeof v2);
        if (clip_seg(v1, v2, cumin, cumax))
            return O_HIT;
    }
    for (j = 0; j < 3; j++)
        if (f->norm[j] > 0.0) {
            v1[j] = cumin[j];
            v2[j] = cumax[j];
        } else {
            v1[j] = cumax[j];
            v2[j] = cumin[j];
        }
    if ((d1 = v1[0] * f->norm[0] + v1[1] * f->norm[1] + v1[2] * f->norm[2] - f->offset) > GB_FTINY)
        return O_MISS;
    if ((d2 = v2[0] * f->norm[0] + v2[1] * f->norm[1] + v2[2] * f->norm[2] - f->offset) < -GB_FTINY)
        return O_MISS;
    for (j = 0; j < 3; j++)
        v1[j] = (v1[j] * d2 - v2[j] * d1) / (d2 - d1);
    return inface_host(v1, f, va) ? O_HIT : O_MISS;
}

static int sphere_cube(const gb_object *o, const double org[3], double size)
{
    const double *c = o->farg;
    double rad = fabs(c[3]), d1, d2, v1[3];
    int i;
    if (rad <= GB_FTINY)
        return O_MISS;
    d1 = 1.732050808 / 2.0 * size;
    d2 = size * 0.5;
    for (i = 0; i < 3; i++)
        v1[i] = org[i] + d2 - c[i];
    d2 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
    if (d2 > (rad + d1 + GB_FTINY) * (rad + d1 + GB_FTINY))
        return O_MISS;
    if (d1 < rad) {
        if (d2 < (rad - d1 - GB_FTINY) * (rad - d1 - GB_FTINY))
            return O_MISS;
        if (d2 < (rad + GB_FTINY) * (rad + GB_FTINY))
            return O_HIT;
    }
    for (i = 0; i < 3; i++)
        if (c[i] < org[i])
            v1[i] = org[i] - c[i];
        else if (c[i] > org[i] + size)
            v1[i] = c[i] - (org[i] + size);
        else
            v1[i] = 0;
    return v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2] <= (rad + GB_FTINY) * (rad + GB_FTINY)
               ? O_HIT : O_MISS;
}

/* bounding box of a cone-family object (ot/bbox.c:56-66, circle2bbox) */
static void cone_bbox(const gb_object *o, const gb_cone *co, double mn[3], double mx[3])
{
    const double *ca = o->farg;
    double ad[3], l;
    int i, k;
    if (o->otype == GT_RING) {
        ad[0] = ca[3]; ad[1] = ca[4]; ad[2] = ca[5];
    } else
        for (i = 0; i < 3; i++)
            ad[i] = ca[co->p1 + i] - ca[co->p0 + i];
    l = sqrt(ad[0] * ad[0] + ad[1] * ad[1] + ad[2] * ad[2]);
    for (i = 0; i < 3; i++)
        ad[i] /= l;
    for (i = 0; i < 3; i++) {
        mn[i] = GB_FHUGE;
        mx[i] = -GB_FHUGE;
    }
    for (k = 0; k < 2; k++) {
        const double *cent;
        double rad;
        if (k == 0) {
            if (o->otype == GT_RING)
                continue;
            cent = ca + co->p0;
            rad = ca[co->r0];
        } else {
            cent = ca + co->p1;
            rad = ca[co->r1];
        }
        for (i = 0; i < 3; i++) {
            double r = sqrt(1. - ad[i] * ad[i]);
            if (cent[i] + r * rad > mx[i]) mx[i] = cent[i] + r * rad;
            if (cent[i] - r * rad < mn[i]) mn[i] = cent[i] - r * rad;
        }
    }
}

static int cone_cube(const gb_object *o, const gb_cone *co, const double org[3], double size, double mincusize);

static int object_cube(builder *B, int32_t obj, const double org[3], double size)
{
    const gb_scene_host *S = B->S;
    const gb_object *o = &S->objs[obj];
    switch (o->otype) {
    case GT_POLYGON:
        return face_cube(o, &S->faces[obj], org, size);
    case GT_SPHERE:
    case GT_BUBBLE:
        return sphere_cube(o, org, size);
    case GT_CONE:
    case GT_CUP:
    case GT_CYLINDER:
    case GT_TUBE:
    case GT_RING: {
        if (!S->cones[obj].ok)
            return O_MISS;
        return cone_cube(o, &S->cones[obj], org, size, B->mincusize);
    }
    default:
        return O_MISS;
    }
}

/* ot/o_cone.c:41-105 with STRICT (as it is compiled): the cone segment
 * nearest the cube centre against the cube's bounding sphere, then clipped
 * to the cube, else the eight sub-cubes down to the minimum cube size */
static int cone_cube(const gb_object *o, const gb_cone *co, const double org[3], double size, double mincusize)
{
    const double *ca = o->farg;
    double ad[3], p[3], v[3], ep0[3], ep1[3], r, d, l, ks;
    int i, j;
    if (o->otype == GT_RING)
        for (i = 0; i < 3; i++) ad[i] = ca[3 + i];
    else
        for (i = 0; i < 3; i++) ad[i] = ca[co->p1 + i] - ca[co->p0 + i];
    l = sqrt(ad[0] * ad[0] + ad[1] * ad[1] + ad[2] * ad[2]);
    for (i = 0; i < 3; i++) ad[i] /= l;
    r = size * 0.5;
    for (i = 0; i < 3; i++) p[i] = org[i] + r;
    r *= 1.732050808;
    /* findcseg: segment of the cone surface nearest p */
    for (i = 0; i < 3; i++) v[i] = p[i] - ca[co->p0 + i];
    d = v[0] * ad[0] + v[1] * ad[1] + v[2] * ad[2];
    for (i = 0; i < 3; i++) v[i] -= d * ad[i];
    l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l != 0.0) {
        double dd = 0, d1 = 0, d2 = 0, q, cumin[3], cumax[3];
        for (i = 0; i < 3; i++) {
            v[i] /= l;
            ep0[i] = ca[co->r0] * v[i] + ca[co->p0 + i];
            ep1[i] = ca[co->r1] * v[i] + ca[co->p1 + i];
        }
        /* common/fvect.c:77-99 dist2lseg */
        for (i = 0; i < 3; i++) {
            dd += (ep1[i] - ep0[i]) * (ep1[i] - ep0[i]);
            d1 += (p[i] - ep0[i]) * (p[i] - ep0[i]);
            d2 += (p[i] - ep1[i]) * (p[i] - ep1[i]);
        }
        if (d2 > d1 && d2 - d1 > dd) q = d1;
        else if (d2 <= d1 && d1 - d2 > dd) q = d2;
        else { double e = dd + d1 - d2; q = d1 - 0.25 * e * e / dd; }
        if (q > (r + GB_FTINY) * (r + GB_FTINY))
            return O_MISS;
        for (i = 0; i < 3; i++) {
            cumin[i] = org[i];
            cumax[i] = org[i] + size;
        }
        if (clip_seg(ep0, ep1, cumin, cumax))
            return O_HIT;
    }
    ks = size * 0.5;                    /* check sub-cubes */
    if (ks < mincusize)
        return O_HIT;
    for (j = 0; j < 8; j++) {
        double ko[3];
        for (i = 0; i < 3; i++) ko[i] = org[i] + (((1 << i) & j) ? ks : 0.0);
        if (cone_cube(o, co, ko, ks, mincusize))
            return O_HIT;
    }
    return O_MISS;
}

static void addobject(builder *B, int32_t nd, const double org[3], double size, int32_t obj);

static void add2full(builder *B, int32_t nd, const double org[3], double size, int32_t obj)
{
    bnode *N = &B->nodes[nd];
    double ks = size * 0.5;
    int32_t *oset, n, i, j;
    if (N->n < B->objlim || ks < (N->n < GB_MAXSET ? B->mincusize : B->mincusize / 256.0)) {
        if (N->n >= GB_MAXSET) {
            B->err = 2;
            return;
        }
        if (set_insert(N, obj) < 0)
            B->err = 1;
        return;
    }
    /* subdivide: take the set out, turn the node into a tree */
    oset = N->set;
    n = N->n;
    N->set = NULL;
    N->n = N->cap = 0;
    N->tree = 1;
    for (i = 0; i < 8; i++) {
        int32_t k = bnew(B);
        if (k < 0) {
            free(oset);
            return;
        }
        B->nodes[nd].kids[i] = k;
    }
    for (i = 0; i < 8; i++) {
        double ko[3];
        int32_t kid = B->nodes[nd].kids[i];
        for (j = 0; j < 3; j++)
            ko[j] = org[j] + (((1 << j) & i) ? ks : 0.0);
        for (j = 0; j < n; j++)              /* surfaces first */
            if (!gb_is_volume(B->S->objs[oset[j]].otype))
                addobject(B, kid, ko, ks, oset[j]);
        addobject(B, kid, ko, ks, obj);      /* then this object */
        for (j = 0; j < n; j++)              /* then (partial) volumes */
            if (gb_is_volume(B->S->objs[oset[j]].otype))
                addobject(B, kid, ko, ks, oset[j]);
    }
    free(oset);
}

static void addobject(builder *B, int32_t nd, const double org[3], double size, int32_t obj)
{
    if (B->err)
        return;
    if (object_cube(B, obj, org, size) == O_MISS)
        return;
    if (B->nodes[nd].tree) {
        double ks = size * 0.5, ko[3];
        int i, j;
        for (i = 0; i < 8; i++) {
            for (j = 0; j < 3; j++)
                ko[j] = org[j] + (((1 << j) & i) ? ks : 0.0);
            addobject(B, B->nodes[nd].kids[i], ko, ks, obj);
        }
        return;
    }
    if (B->nodes[nd].n == 0) {
        if (set_insert(&B->nodes[nd], obj) < 0)
            B->err = 1;
        return;
    }
    add2full(B, nd, org, size, obj);
}

static int leaf_equal(const bnode *a, const bnode *b)
{
    return !a->tree && !b->tree && a->n == b->n &&
           (a->n == 0 || !memcmp(a->set, b->set, (size_t)a->n * sizeof(int32_t)));
}

/* merge a tree whose 8 children are identical leaves into that leaf
 * (common/octree.c:73-90) */
static void combine(builder *B, int32_t nd)
{
    int i;
    bnode *N = &B->nodes[nd], *K0;
    if (!N->tree)
        return;
    for (i = 0; i < 8; i++)
        combine(B, N->kids[i]);
    K0 = &B->nodes[N->kids[0]];
    for (i = 1; i < 8; i++)
        if (!leaf_equal(K0, &B->nodes[N->kids[i]]))
            return;
    N->tree = 0;
    N->set = K0->set;
    N->n = K0->n;
    N->cap = K0->cap;
    K0->set = NULL;
    K0->n = K0->cap = 0;
}

static int32_t flatten(builder *B, int32_t nd, int *ok)
{
    const bnode *N = &B->nodes[nd];
    gb_scene_host *S = B->S;
    if (!N->tree) {
        int32_t code, *tmp;
        if (N->n == 0)
            return -1;
        tmp = (int32_t *)malloc((size_t)(N->n + 1) * sizeof(int32_t));
        if (!tmp) {
            *ok = 0;
            return -1;
        }
        tmp[0] = N->n;
        memcpy(tmp + 1, N->set, (size_t)N->n * sizeof(int32_t));
        code = gb__add_set(S, tmp);
        free(tmp);
        if (code == 0)
            *ok = 0;
        return code;
    } else {
        int32_t out = gb__new_node(S), i;
        if (out < 0) {
            *ok = 0;
            return -1;
        }
        for (i = 0; i < 8; i++) {
            int32_t c = flatten(B, B->nodes[nd].kids[i], ok);
            if (!*ok)
                return -1;
            S->kids[8 * out + i] = c;
        }
        return out;
    }
}

/* Prepares the objects and sets the scene cube from their bounding box
 * (ot/oconv.c:128-150); -1 for objects no octree is built over here. */
int gb_scene_octree_cube(gb_scene_host *S)
{
    double bbmin[3], bbmax[3];
    int32_t i;
    int k;
    if (gb_scene_prepare(S) < 0)
        return -1;
    for (k = 0; k < 3; k++) {
        bbmin[k] = GB_FHUGE;
        bbmax[k] = -GB_FHUGE;
    }
    for (i = 0; i < S->nobjs; i++) {
        const gb_object *o = &S->objs[i];
        double mn[3], mx[3];
        int j;
        switch (o->otype) {
        case GT_POLYGON: {
            const gb_face *f = &S->faces[i];
            for (j = 0; j < f->nv; j++)
                for (k = 0; k < 3; k++) {
                    double v = o->farg[3 * j + k];
                    if (v < bbmin[k]) bbmin[k] = v;
                    if (v > bbmax[k]) bbmax[k] = v;
                }
            break;
        }
        case GT_SPHERE:
        case GT_BUBBLE:
            for (k = 0; k < 3; k++) {
                double r = fabs(o->farg[3]);
                if (o->farg[k] - r < bbmin[k]) bbmin[k] = o->farg[k] - r;
                if (o->farg[k] + r > bbmax[k]) bbmax[k] = o->farg[k] + r;
            }
            break;
        case GT_CONE:
        case GT_CUP:
        case GT_CYLINDER:
        case GT_TUBE:
        case GT_RING:
            if (!S->cones[i].ok)
                break;
            cone_bbox(o, &S->cones[i], mn, mx);
            for (k = 0; k < 3; k++) {
                if (mn[k] < bbmin[k]) bbmin[k] = mn[k];
                if (mx[k] > bbmax[k]) bbmax[k] = mx[k];
            }
            break;
        case GT_INSTANCE:
        case GT_MESH:
            return -1;
        default:
            break;
        }
    }
    S->cusize = 0.0;
    if (bbmin[0] <= bbmax[0]) {
        for (k = 0; k < 3; k++) {
            bbmin[k] -= 10 * GB_FTINY;
            bbmax[k] += 10 * GB_FTINY;
        }
        for (k = 0; k < 3; k++)
            if (bbmax[k] - bbmin[k] > S->cusize)
                S->cusize = bbmax[k] - bbmin[k];
        for (k = 0; k < 3; k++)
            S->cuorg[k] = (bbmax[k] + bbmin[k] - S->cusize) * .5;
    }
    return 0;
}

int gb_scene_build_octree(gb_scene_host *S, int objlim, int resolu)
{
    builder B;
    int32_t i, root;
    int ok = 1;
    if (gb_scene_octree_cube(S) < 0)
        return -1;
    memset(&B, 0, sizeof B);
    B.S = S;
    B.objlim = objlim > 0 ? objlim : 6;
    B.mincusize = S->cusize / (resolu > 0 ? resolu : 16384) - GB_FTINY;
    root = bnew(&B);
    for (i = 0; i < S->nobjs && !B.err; i++)
        if (gb_is_surface(S->objs[i].otype) && S->objs[i].otype != GT_SOURCE)
            addobject(&B, root, S->cuorg, S->cusize, i);
    if (!B.err) {
        S->nnodes = 0;
        S->nsets = 0;
        S->set_len = 0;
        combine(&B, root);
        S->root = flatten(&B, root, &ok);
    }
    for (i = 0; i < B.nn; i++)
        free(B.nodes[i].set);
    free(B.nodes);
    if (B.err || !ok)
        return -1;
    return 0;
}
