/*
 * cast64.cu -- first hits in FP64: the object, distance, point and normal
 * of rays cast into the scene (rtrace's -o s/m/M/L/p/N outputs and the hit
 * ids of gb_rtrace), computed as the reference computes them.
 *
 * The octree walk is rt/raytrace.c:595-793 (localhit, raymove, checkhit,
 * checkset) with FP64 cube bounds and positions, the recursion of raymove
 * turned into a loop over a stack of cubes; the object tests are
 * rt/o_face.c:15-62 with common/face.c:121-161 (inface), rt/sphere.c:15-83
 * with common/zeroes.c:19-53 (quadratic), rt/o_cone.c:16-146 and
 * rt/o_instance.c:15-71, arbitrated by rt/raytrace.c:536-575 (rayreject).
 * The ray direction is normalised as common/fvect.c:132-155 does.  The
 * file is compiled without contracted multiply-adds, so every operation
 * rounds as the reference's: the hit objects are the reference's also
 * where FP32 rounding of a hit point decides an edge rule or a tie
 * (rays at polygon edges and corners, coplanar faces).
 *
 * The objects already tested along the walk are kept, as checkset keeps
 * them, in a sorted list -- of at most CSET_CAP objects here (the
 * reference keeps up to 16,383): past that, an object tested before is
 * tested again, which changes nothing but in a tie between three objects
 * within FTINY of one another.
 *
 * Geometry comes from a per-object FP64 record (gb_dscene g64, g64off)
 * written when the scene is loaded; the octree, the sets and the object
 * flags are the FP32 path's.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "devscene.h"
#include "tracehost.h"

namespace {

#define FTINY64 1e-6
#define FHUGE64 1e10
#define CSET_CAP 128
#define MAX_DEPTH 40

struct Ray64 {
    double org[3], dir[3];
    double rot;          /* distance of the best hit so far */
    int ro;              /* its object, -1 none */
    double rop[3], ron[3], rod;
    double vn[3];        /* a smooth mesh hit: its interpolated vertex normal, unit, in the scene; else 0 */
    double uv[2];        /* a mesh hit with vertex (u,v): them interpolated; else 0 */
};

__device__ __forceinline__ double dot64(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__device__ __forceinline__ const double *rec64(const gb_dscene &S, int o)
{
    return S.g64 + S.g64off[o];
}

/* rt/raytrace.c:536-575 */
__device__ int rayreject64(const gb_dscene &S, int o, const Ray64 &r, double t, double rod)
{
    if ((t <= FTINY64) | (t > r.rot + FTINY64))
        return 1;
    if (t < r.rot - FTINY64)
        return 0;
    if (o == r.ro)
        return 1;
    if (r.ro < 0)
        return 0;
    const int fn = (S.obj[o].x >> 8) & 0xff, fb = (S.obj[r.ro].x >> 8) & 0xff;
    if (!(fn & DF_HASMAT)) {
        if (fb & DF_HASMAT)
            return 1;
    } else if (!(fb & DF_HASMAT)) {
        return 0;
    } else if (fn & DF_TRANSP) {
        if (!(fb & DF_TRANSP))
            return 1;
    } else if (fb & DF_TRANSP) {
        return 0;
    }
    if (rod <= 0) {
        if (r.rod > 0)
            return 1;
    } else if (r.rod <= 0) {
        return 0;
    }
    return S.obj[r.ro].z >= S.obj[o].z;
}

/* common/face.c:121-161 */
__device__ int inface64(const double p[3], int n, int ax, const double *va)
{
    int ncross = 0, tst, xi, yi;
    double x, y;
    const double *p0, *p1;
    if ((xi = ax + 1) >= 3) xi -= 3;
    if ((yi = xi + 1) >= 3) yi -= 3;
    x = p[xi];
    y = p[yi];
    p0 = va + 3 * (n - 1);
    p1 = va;
#define FEQ(a, b) (fabs((a) - (b)) <= FTINY64)
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

/* rt/o_face.c:15-62; record: normal (3), offset, ok, dominant axis, vertex
 * count, vertices */
__device__ int o_face64(const gb_dscene &S, int o, Ray64 &r)
{
    const double *g = rec64(S, o);
    if (g[4] == 0.0)
        return 0;
    const double rdot = -dot64(r.dir, g);
    if ((rdot <= FTINY64) & (rdot >= -FTINY64))
        return 0;
    const double t = (dot64(r.org, g) - g[3]) / rdot;
    if (rayreject64(S, o, r, t, rdot))
        return 0;
    double p[3];
    p[0] = r.org[0] + r.dir[0] * t;
    p[1] = r.org[1] + r.dir[1] * t;
    p[2] = r.org[2] + r.dir[2] * t;
    if (!inface64(p, (int)g[6], (int)g[5], g + 7))
        return 0;
    r.ro = o;
    r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
    r.rot = t;
    for (int i = 0; i < 3; i++) {
        r.rop[i] = p[i];
        r.ron[i] = g[i];
    }
    r.rod = rdot;
    return 1;
}

/* common/zeroes.c:19-53 */
__device__ int quadratic64(double *rt, double a, double b, double c)
{
    double disc;
    int first;
    if (a < -FTINY64)
        first = 1;
    else if (a > FTINY64)
        first = 0;
    else if (fabs(b) > FTINY64) {
        rt[0] = -c / b;
        return 1;
    } else
        return 0;
    b *= 0.5;
    disc = b * b - a * c;
    if (disc < -FTINY64 * FTINY64)
        return 0;
    if (disc <= FTINY64 * FTINY64) {
        rt[0] = -b / a;
        return 1;
    }
    disc = sqrt(disc);
    rt[first] = (-b - disc) / a;
    rt[1 - first] = (-b + disc) / a;
    return 2;
}

/* rt/sphere.c:15-83; record: centre (3), radius */
__device__ int o_sphere64(const gb_dscene &S, int o, bool bubble, Ray64 &r)
{
    const double *ap = rec64(S, o);
    double a = 0, b = 0, c = 0, t = 0, root[2];
    int i, nr;
    for (i = 0; i < 3; i++) {
        const double d = r.org[i] - ap[i];
        a += r.dir[i] * r.dir[i];
        b += 2.0 * r.dir[i] * d;
        c += d * d;
    }
    c -= ap[3] * ap[3];
    nr = quadratic64(root, a, b, c);
    for (i = 0; i < nr; i++)
        if ((t = root[i]) > FTINY64)
            break;
    if (i >= nr)
        return 0;
    if (rayreject64(S, o, r, t, (double)(1 - 2 * ((i > 0) ^ bubble))))
        return 0;
    r.ro = o;
    r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
    r.rot = t;
    const double rad = ap[3] * (1 - 2 * (int)bubble);
    for (i = 0; i < 3; i++) {
        r.rop[i] = r.org[i] + r.dir[i] * t;
        r.ron[i] = (r.rop[i] - ap[i]) / rad;
    }
    r.rod = -dot64(r.dir, r.ron);
    return 1;
}

/* rt/o_cone.c:16-146; record: ok, alpha, slant, the 4x4 world-to-canonical
 * transform (row-major), then for rings centre (3), normal (3), inner and
 * outer radius; for the others the two end points (3 + 3) and the radii at
 * them */
__device__ int o_cone64(const gb_dscene &S, int o, int kind, Ray64 &r)
{
    const double *g = rec64(S, o);
    if (g[0] == 0.0)
        return 0;
    const double al = g[1], sl = g[2];
    const double *tm = g + 3;
    const double *ca = g + 19;
    const double r0 = g[25], r1 = g[26];
    double rox[3], rdx[3], a, b, c, root[2], ad[3];
    int nr, rn, i;
    for (i = 0; i < 3; i++) {
        rdx[i] = r.dir[0] * tm[0 * 4 + i] + r.dir[1] * tm[1 * 4 + i] + r.dir[2] * tm[2 * 4 + i];
        rox[i] = r.org[0] * tm[0 * 4 + i] + r.org[1] * tm[1 * 4 + i] + r.org[2] * tm[2 * 4 + i] + tm[3 * 4 + i];
    }
    for (i = 0; i < 3; i++)
        ad[i] = kind == DK_RING ? ca[3 + i] : ca[3 + i] - ca[i];
    {
        const double l = sqrt(dot64(ad, ad));
        if (l > 0) {
            ad[0] /= l;
            ad[1] /= l;
            ad[2] /= l;
        }
    }
    if (kind == DK_RING) {
        if ((rdx[2] <= FTINY64) & (rdx[2] >= -FTINY64))
            return 0;
        root[0] = -rox[2] / rdx[2];
        if (rayreject64(S, o, r, root[0], -rdx[2]))
            return 0;
        b = root[0] * rdx[0] + rox[0];
        c = root[0] * rdx[1] + rox[1];
        a = b * b + c * c;
        if (a > r1 * r1 || a < r0 * r0)
            return 0;
        r.ro = o;
        r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
        r.rot = root[0];
        for (i = 0; i < 3; i++) {
            r.rop[i] = r.org[i] + r.dir[i] * r.rot;
            r.ron[i] = ad[i];
        }
        r.rod = -rdx[2];
        return 1;
    }
    if (kind == DK_CONE || kind == DK_CUP) {
        a = rdx[0] * rdx[0] + rdx[1] * rdx[1] - rdx[2] * rdx[2];
        b = 2.0 * (rdx[0] * rox[0] + rdx[1] * rox[1] - rdx[2] * rox[2]);
        c = rox[0] * rox[0] + rox[1] * rox[1] - rox[2] * rox[2];
    } else {
        a = rdx[0] * rdx[0] + rdx[1] * rdx[1];
        b = 2.0 * (rdx[0] * rox[0] + rdx[1] * rox[1]);
        c = rox[0] * rox[0] + rox[1] * rox[1] - r0 * r0;
    }
    nr = quadratic64(root, a, b, c);
    for (rn = 0; rn < nr; rn++) {
        double p[3], v[3];
        if (root[rn] <= FTINY64)
            continue;
        if (root[rn] > r.rot + FTINY64)
            break;
        for (i = 0; i < 3; i++) {
            p[i] = r.org[i] + r.dir[i] * root[rn];
            v[i] = p[i] - ca[i];
        }
        b = dot64(v, ad);
        if (b < 0.0 || b > al)
            continue;
        if (rayreject64(S, o, r, root[rn], (double)(1 - 2 * ((rn > 0) ^ (kind == DK_CUP || kind == DK_TUBE)))))
            break;
        r.ro = o;
        r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
        r.rot = root[rn];
        for (i = 0; i < 3; i++)
            r.rop[i] = p[i];
        if (kind == DK_CYL)
            a = r0;
        else if (kind == DK_TUBE)
            a = -r0;
        else {
            c = r1 - r0;
            a = r0 + b * c / al;
            if (kind == DK_CUP) {
                c = -c;
                a = -a;
            }
        }
        for (i = 0; i < 3; i++)
            r.ron[i] = (v[i] - b * ad[i]) / a;
        if (kind == DK_CONE || kind == DK_CUP)
            for (i = 0; i < 3; i++)
                r.ron[i] = (al * r.ron[i] - c * ad[i]) / sl;
        a = dot64(r.ron, r.ron);
        if ((a > 1. + FTINY64) | (a < 1. - FTINY64)) {
            c = 1. / (.5 + .5 * a);
            for (i = 0; i < 3; i++)
                r.ron[i] *= c;
        }
        r.rod = -dot64(r.dir, r.ron);
        return 1;
    }
    return 0;
}

__device__ int incube64(const double org[3], double size, const double pt[3])
{
    for (int i = 0; i < 3; i++)
        if (org[i] > pt[i] || pt[i] >= org[i] + size)
            return 0;
    return 1;
}

/* The objects of a leaf (device leaf code) in the order the reference
 * tests them (descending), those not tested before; records them as
 * tested.  Returns their number in todo. */
struct Checked {
    int n;
    int v[CSET_CAP];               /* ascending */
    __device__ bool has(int o) const
    {
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (v[mid] < o)
                lo = mid + 1;
            else
                hi = mid;
        }
        return lo < n && v[lo] == o;
    }
    __device__ void add(int o)     /* keeps the CSET_CAP smallest */
    {
        int i = n < CSET_CAP ? n : CSET_CAP - 1;
        if (n == CSET_CAP && o > v[CSET_CAP - 1])
            return;
        while (i > 0 && v[i - 1] > o) {
            v[i] = v[i - 1];
            i--;
        }
        v[i] = o;
        if (n < CSET_CAP)
            n++;
    }
};

template <bool INST>
__device__ bool walk64(const gb_dscene &S, Ray64 &r, const double cuorg[3], double cusize, int root);

/* rt/o_mesh.c:185-221: the attributes of mesh triangle o at the hit point
 * p (mesh coordinates), interpolated by its barycentric weights (common/
 * tmesh.c get_baryc: in the plane of the triangle's largest projection):
 * the vertex normals (after its face record) carried to the scene by the
 * forward transform fx (its rotation and scale rows) and normalised, into
 * vn; the vertex (u,v) (after the normals), untransformed, into uv.  A
 * degenerate triangle or a zero normal leaves them 0. */
__device__ void mesh_attrs64(const gb_dscene &S, int o, int fl, const double p[3], const double *fx, double vn[3],
                             double uv[2])
{
    const double *g = rec64(S, o);
    const int nv = (int)g[6];
    const double *v = g + 7, *x = g + 7 + 3 * nv;
    double e1[3], e2[3], cr[3];
    for (int i = 0; i < 3; i++) {
        e1[i] = v[i] - v[3 + i];
        e2[i] = v[6 + i] - v[3 + i];
    }
    cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
    cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
    cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
    int ax = cr[1] * cr[1] > cr[0] * cr[0] ? 1 : 0;
    if (cr[2] * cr[2] > cr[ax] * cr[ax])
        ax = 2;
    const int a0 = (ax + 1) % 3, a1 = (ax + 2) % 3;
    const double x0 = v[a0], y0 = v[a1], x1 = v[3 + a0], y1 = v[3 + a1], x2 = v[6 + a0], y2 = v[6 + a1];
    const double den = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
    if (den == 0.0)
        return;
    const double px = p[a0] - x0, py = p[a1] - y0;
    const double w1 = (px * (y2 - y0) - (x2 - x0) * py) / den;
    const double w2 = ((x1 - x0) * py - px * (y1 - y0)) / den;
    const double w0 = 1.0 - w1 - w2;
    if (fl & DF_VNORM) {
        double m[3], w[3];
        for (int i = 0; i < 3; i++)
            m[i] = w0 * x[i] + w1 * x[3 + i] + w2 * x[6 + i];
        for (int j = 0; j < 3; j++)
            w[j] = m[0] * fx[0 * 4 + j] + m[1] * fx[1 * 4 + j] + m[2] * fx[2 * 4 + j];
        const double l = sqrt(dot64(w, w));
        if (l != 0.0)
            for (int j = 0; j < 3; j++)
                vn[j] = w[j] / l;
        x += 9;
    }
    if (fl & DF_VUV)
        for (int i = 0; i < 2; i++)
            uv[i] = w0 * x[i] + w1 * x[2 + i] + w2 * x[4 + i];
}

/* rt/o_instance.c:15-71; record: backward transform (16), scale, forward
 * transform (16), scale, the octree's cube (3 + 1) and root code, whether
 * the instance's modifier replaces its surfaces' */
__device__ int o_instance64(const gb_dscene &S, int o, Ray64 &r)
{
    const double *g = rec64(S, o);
    const double *bx = g, *fx = g + 17;
    const double bsca = g[16], fsca = g[33];
    Ray64 rc;
    int i, j;
    for (j = 0; j < 3; j++) {
        rc.org[j] = r.org[0] * bx[0 * 4 + j] + r.org[1] * bx[1 * 4 + j] + r.org[2] * bx[2 * 4 + j];
        rc.dir[j] = r.dir[0] * bx[0 * 4 + j] + r.dir[1] * bx[1 * 4 + j] + r.dir[2] * bx[2 * 4 + j];
    }
    for (j = 0; j < 3; j++)
        rc.org[j] += bx[3 * 4 + j];
    for (i = 0; i < 3; i++)
        rc.dir[i] /= bsca;
    rc.ro = -1;
    rc.rot = FHUGE64;
    rc.rod = 1.0;
    const double corg[3] = {g[34], g[35], g[36]};
    if (!walk64<false>(S, rc, corg, g[37], (int)g[38]))
        return 0;
    if (rc.rot * fsca >= r.rot)
        return 0;
    r.ro = g[39] != 0.0 ? o : rc.ro;
    r.rot = rc.rot * fsca;
    r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
    if (rc.ro >= 0 && ((S.obj[rc.ro].x >> 8) & (DF_VNORM | DF_VUV)))
        mesh_attrs64(S, rc.ro, S.obj[rc.ro].x >> 8, rc.rop, fx, r.vn, r.uv);
    for (j = 0; j < 3; j++) {
        r.rop[j] = rc.rop[0] * fx[0 * 4 + j] + rc.rop[1] * fx[1 * 4 + j] + rc.rop[2] * fx[2 * 4 + j];
        r.ron[j] = rc.ron[0] * fx[0 * 4 + j] + rc.ron[1] * fx[1 * 4 + j] + rc.ron[2] * fx[2 * 4 + j];
    }
    for (j = 0; j < 3; j++)
        r.rop[j] += fx[3 * 4 + j];
    const double d = 1. / fsca;
    for (i = 0; i < 3; i++)
        r.ron[i] *= d;
    r.rod = rc.rod;
    return 1;
}

template <bool INST>
__device__ void object_hit64(const gb_dscene &S, int o, Ray64 &r)
{
    const int kind = S.obj[o].x & 0xff;
    switch (kind) {
    case DK_FACE:
        o_face64(S, o, r);
        break;
    case DK_SPHERE:
    case DK_BUBBLE:
        o_sphere64(S, o, kind == DK_BUBBLE, r);
        break;
    case DK_CONE:
    case DK_CUP:
    case DK_CYL:
    case DK_TUBE:
    case DK_RING:
        o_cone64(S, o, kind, r);
        break;
    case DK_INSTANCE:
        if (INST)
            o_instance64(S, o, r);
        break;
    default:
        break;
    }
}

struct Frame {
    double org[3];
    double size;
    int code, br;
};

/* rt/raytrace.c:595-654 (localhit) and :658-739 (raymove), the recursion
 * over subcubes as a stack of frames; checkhit (:743-760) at full leaves */
template <bool INST>
__device__ bool walk64(const gb_dscene &S, Ray64 &r, const double cuorg[3], double cusize, int root)
{
    double pos[3], t, dt;
    int sflags = 0, i;
    for (i = 0; i < 3; i++) {
        pos[i] = r.org[i];
        if (r.dir[i] > 1e-7)
            sflags |= 1 << i;
        else if (r.dir[i] < -1e-7)
            sflags |= 0x10 << i;
    }
    if (!sflags)
        return false;
    t = 0.0;
    if (!incube64(cuorg, cusize, pos)) {
        for (i = 0; i < 3; i++) {
            if (sflags & 1 << i)
                dt = cuorg[i];
            else if (sflags & 0x10 << i)
                dt = cuorg[i] + cusize;
            else
                continue;
            dt = (dt - r.org[i]) / r.dir[i];
            if (dt > t)
                t = dt;
        }
        t += FTINY64;
        if (t >= r.rot)
            return false;
        for (i = 0; i < 3; i++)
            pos[i] += r.dir[i] * t;
        if (!incube64(cuorg, cusize, pos))
            return false;
    }
    Checked cx;
    cx.n = 0;
    Frame f[MAX_DEPTH];
    int d = 0;
    for (i = 0; i < 3; i++)
        f[0].org[i] = cuorg[i];
    f[0].size = cusize;
    f[0].code = root;
    f[0].br = 0;
    for (;;) {
        Frame &F = f[d];
        if (F.code >= 0) {                           /* a tree: the subcube holding pos */
            if (d + 1 >= MAX_DEPTH)
                return r.ro >= 0;
            Frame &C = f[d + 1];
            C.size = F.size * 0.5;
            for (i = 0; i < 3; i++)
                C.org[i] = F.org[i];
            int br = 0;
            if (pos[0] >= C.org[0] + C.size) {
                C.org[0] += C.size;
                br |= 1;
            }
            if (pos[1] >= C.org[1] + C.size) {
                C.org[1] += C.size;
                br |= 2;
            }
            if (pos[2] >= C.org[2] + C.size) {
                C.org[2] += C.size;
                br |= 4;
            }
            C.br = br;
            C.code = S.kids[8 * F.code + br];
            d++;
            continue;
        }
        if (F.code <= -2) {                          /* full leaf: checkhit */
            const int code = -F.code - 2;
            const int off = code >> GB_LEAF_SIZEBITS;
            int cnt = code & ((1 << GB_LEAF_SIZEBITS) - 1);
            if (cnt == (1 << GB_LEAF_SIZEBITS) - 1)
                cnt = S.set_data[off];
            /* the members not tested before, in the set's (descending)
             * order; then all of them count as tested */
            for (int k = 1; k <= cnt; k++) {
                const int sl = S.set_data[off + k];
                const int o = __float_as_int(S.orec[4 * sl].y);
                if (!cx.has(o))
                    object_hit64<INST>(S, o, r);
            }
            for (int k = cnt; k >= 1; k--) {         /* ascending: record them as tested */
                const int sl = S.set_data[off + k];
                const int o = __float_as_int(S.orec[4 * sl].y);
                if (!cx.has(o))
                    cx.add(o);
            }
            if (r.ro >= 0 && incube64(F.org, F.size, r.rop))
                return true;
        }
        /* the exit face of this cube and the position on it */
        int ax = 0;
        if (sflags & 0x11) {
            dt = sflags & 1 ? F.org[0] + F.size : F.org[0];
            t = (dt - pos[0]) / r.dir[0];
            ax = 0;
        } else
            t = FHUGE64;
        if (sflags & 0x22) {
            dt = sflags & 2 ? F.org[1] + F.size : F.org[1];
            dt = (dt - pos[1]) / r.dir[1];
            if (dt < t) {
                t = dt;
                ax = 1;
            }
        }
        if (sflags & 0x44) {
            dt = sflags & 4 ? F.org[2] + F.size : F.org[2];
            dt = (dt - pos[2]) / r.dir[2];
            if (dt < t) {
                t = dt;
                ax = 2;
            }
        }
        pos[0] += r.dir[0] * t;
        pos[1] += r.dir[1] * t;
        pos[2] += r.dir[2] * t;
        /* the parent moves to the sibling across that face, or hands the
         * exit up when the face is its own (raymove's overflow/underflow) */
        for (;;) {
            if (d == 0)
                return r.ro >= 0;
            Frame &C = f[d];
            const int sgn = 1 << ax;
            if (sgn & sflags) {
                if (sgn & C.br) {
                    d--;
                    continue;
                }
                C.org[ax] += C.size;
                C.br |= sgn;
            } else {
                if (sgn & C.br) {
                    C.org[ax] -= C.size;
                    C.br &= ~sgn;
                } else {
                    d--;
                    continue;
                }
            }
            C.code = S.kids[8 * f[d - 1].code + C.br];
            break;
        }
    }
}

/* common/fvect.c:132-155 */
__device__ double normalize64(double v[3])
{
    double len, d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (d == 0.0)
        return 0.0;
    if ((d <= 1.0 + FTINY64) & (d >= 1.0 - FTINY64)) {
        len = 0.5 + 0.5 * d;
        d = 2.0 - len;
    } else {
        len = sqrt(d);
        d = 1.0 / len;
    }
    v[0] *= d;
    v[1] *= d;
    v[2] *= d;
    return len;
}

}  // namespace

/* rt/source.c:317-377 for a primary ray that leaves the scene: the first
 * distant source whose cone holds the direction, a glow's only if no other
 * does; its object, or -1 */
__device__ int cast_source64(const gb_dscene &S, const double dir[3])
{
    int glowsrc = -1;
    for (int i = 0; i < S.nsrc; i++) {
        const gb_dsrc &s = S.src[i];
        if (!(s.flags & DS_DISTANT))
            continue;
        const double dt = (double)s.sloc[0] * dir[0] + (double)s.sloc[1] * dir[1] + (double)s.sloc[2] * dir[2];
        if (2. * 3.14159265358979323846 * (1. - dt) > (double)s.ss2)
            continue;
        if (s.flags & DS_SKIP) {
            if (glowsrc < 0)
                glowsrc = i;
            continue;
        }
        return s.so;
    }
    return glowsrc >= 0 ? S.src[glowsrc].so : -1;
}

__global__ void k_cast64(gb_run P, int *hit_obj, float *hit_t, double *hit_pn)
{
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        const double *sv = P.sensors + 6 * s;
        Ray64 r;
        for (int i = 0; i < 3; i++) {
            r.org[i] = sv[i];
            r.dir[i] = sv[3 + i];
        }
        normalize64(r.dir);
        r.ro = -1;
        r.rot = FHUGE64;
        r.rod = 1.0;
        r.vn[0] = r.vn[1] = r.vn[2] = r.uv[0] = r.uv[1] = 0.0;
        int obj = -1;
        double t = FHUGE64;
        double p[3] = {0, 0, 0}, n[3] = {0, 0, 0};
        const double corg[3] = {P.S.cuorg64[0], P.S.cuorg64[1], P.S.cuorg64[2]};
        if (walk64<true>(P.S, r, corg, P.S.cusize64, P.S.root)) {
            obj = r.ro;
            t = r.rot;
            for (int i = 0; i < 3; i++) {
                p[i] = r.rop[i];
                n[i] = r.ron[i];
            }
        } else {
            obj = cast_source64(P.S, r.dir);
            for (int i = 0; i < 3; i++)
                p[i] = r.org[i] + r.dir[i] * t;
        }
        hit_obj[s] = obj;
        if (hit_t)
            hit_t[s] = (float)t;
        if (hit_pn) {
            double *o = hit_pn + 11 * s;
            for (int i = 0; i < 3; i++) {
                o[i] = p[i];
                o[3 + i] = n[i];
                o[6 + i] = obj >= 0 ? r.vn[i] : 0.0;
            }
            o[9] = obj >= 0 ? r.uv[0] : 0.0;
            o[10] = obj >= 0 ? r.uv[1] : 0.0;
        }
    }
}

int gb_launch_cast64(const gb_run *P, int *hit_obj, float *hit_t, double *hit_pn, cudaStream_t st, int sms)
{
    long long g = (P->nsensors + 127) / 128;
    if (g > (long long)sms * 8)
        g = (long long)sms * 8;
    if (g < 1)
        g = 1;
    k_cast64<<<(unsigned)g, 128, 0, st>>>(*P, hit_obj, hit_t, hit_pn);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
