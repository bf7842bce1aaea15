/*
 * trace.cuh -- device-side ray tracing core: octree traversal, primitive
 * intersection with the reference's hit arbitration, source hits and the
 * bin programs.  FP32 throughout; see trace.cu for the wavefront kernels.
 */
#ifndef GB_TRACE_CUH
#define GB_TRACE_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "devscene.h"
#include "gbcommon.h"

/* The traversal and intersection code is written once for the device; it
 * also compiles for the host so that it can be exercised without a GPU. */
#define GB_DFN __host__ __device__ __forceinline__
/* rarely taken paths kept out of line, so that their registers do not
 * count against the walk loop's */
#define GB_DNI static __host__ __device__ __noinline__
#ifdef __CUDA_ARCH__
#define GB_LDG(p) __ldg(p)
#define GB_F2I_RD(x) __float2int_rd(x)
#define GB_CLZ(x) __clz(x)
#else
#define GB_LDG(p) (*(p))
#define GB_F2I_RD(x) ((int)floorf(x))
#define GB_CLZ(x) __builtin_clz(x)
#endif

#define D_FTINY 1e-6f
#define D_FHUGE 1e10f
#define D_PI 3.14159265358979323846f
#define GRID_BITS 24
#define GRID_N (1 << GRID_BITS)
#define MAX_CUBE_STEPS 65536

struct Hit {
    int   obj;      /* -1 none */
    float t;
    float rod;      /* -dot(dir, normal) */
    float3 n;       /* unflipped surface normal */
};

GB_DFN float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
GB_DFN float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
GB_DFN float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
GB_DFN float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
GB_DFN float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
GB_DFN float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
GB_DFN float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GB_DFN float3 cross3(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GB_DFN float comp(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
GB_DFN float maxc(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
GB_DFN float3 normalize3(float3 v)
{
    float l = sqrtf(dot3(v, v));
    return l > 0.f ? v * (1.f / l) : v;
}

/* ------------------------------------------------------------------------
 * Hit arbitration: rt/raytrace.c:536-575 (rayreject).  Returns true when the
 * candidate (obj, t, rod) is worse than the current best.
 */
GB_DFN bool ray_reject(const gb_dscene &S, int obj, float t, float rod,
                                           const Hit &best, float tmin)
{
    if ((t <= tmin) | (t > best.t + D_FTINY))
        return true;
    if (t < best.t - D_FTINY)
        return false;
    if (obj == best.obj)
        return true;
    if (best.obj < 0)
        return false;
    int fn = (S.obj[obj].x >> 8) & 0xff, fb = (S.obj[best.obj].x >> 8) & 0xff;
    if (!(fn & DF_HASMAT)) {
        if (fb & DF_HASMAT)
            return true;
    } else if (!(fb & DF_HASMAT)) {
        return false;
    } else if (fn & DF_TRANSP) {
        if (!(fb & DF_TRANSP))
            return true;
    } else if (fb & DF_TRANSP) {
        return false;
    }
    if (rod <= 0.f) {
        if (best.rod > 0.f)
            return true;
    } else if (best.rod <= 0.f) {
        return false;
    }
    return S.obj[best.obj].z >= S.obj[obj].z;   /* later modifier wins */
}

/* point in polygon on the dominant projection: common/face.c:121-161 */
GB_DFN bool in_face(const float2 *__restrict__ v, int nv, float x, float y)
{
    int ncross = 0;
    float2 p0 = v[nv - 1];
    for (int k = 0; k < nv; k++) {
        float2 p1 = v[k];
        if ((fabsf(p0.y - y) <= D_FTINY) & (fabsf(p1.y - y) <= D_FTINY) & ((p0.x > x) ^ (p1.x > x)))
            return true;                                           /* edge case #1 */
        if ((p0.y > y) ^ (p1.y > y)) {
            int tst = (p0.x > x) + (p1.x > x);
            if (tst == 2)
                ncross++;
            else if (tst) {
                float prodA = (p0.y - y) * (p1.x - x);
                float prodB = (p0.x - x) * (p1.y - y);
                if (fabsf(prodA - prodB) <= D_FTINY)
                    return true;                                   /* edge case #2 */
                ncross += (p1.y > p0.y) ^ (prodA > prodB);
            } else if ((fabsf(p0.x - x) <= D_FTINY) & (fabsf(p1.x - x) <= D_FTINY))
                return true;                                       /* edge case #3 */
        }
        p0 = p1;
    }
    return ncross & 1;
}

/* in_face for a triangle or quadrilateral whose projected vertices are in
 * registers (va: v0 v1, vb: v2 v3); the same arithmetic in the same order */
GB_DFN bool in_face4(float4 va, float4 vb, int nv, float x, float y)
{
    const float2 v[4] = {make_float2(va.x, va.y), make_float2(va.z, va.w), make_float2(vb.x, vb.y),
                         make_float2(vb.z, vb.w)};
    int ncross = 0;
    float2 p0 = nv == 3 ? v[2] : v[3];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k >= nv)
            break;
        float2 p1 = v[k];
        if ((fabsf(p0.y - y) <= D_FTINY) & (fabsf(p1.y - y) <= D_FTINY) & ((p0.x > x) ^ (p1.x > x)))
            return true;                                           /* edge case #1 */
        if ((p0.y > y) ^ (p1.y > y)) {
            int tst = (p0.x > x) + (p1.x > x);
            if (tst == 2)
                ncross++;
            else if (tst) {
                float prodA = (p0.y - y) * (p1.x - x);
                float prodB = (p0.x - x) * (p1.y - y);
                if (fabsf(prodA - prodB) <= D_FTINY)
                    return true;                                   /* edge case #2 */
                ncross += (p1.y > p0.y) ^ (prodA > prodB);
            } else if ((fabsf(p0.x - x) <= D_FTINY) & (fabsf(p1.x - x) <= D_FTINY))
                return true;                                       /* edge case #3 */
        }
        p0 = p1;
    }
    return ncross & 1;
}

/* rt/o_face.c:15-62; pl is the face's plane, va/vb its first four projected
 * vertices (used when it has at most four) */
GB_DFN void hit_face(const gb_dscene &S, int obj, int4 od, float4 pl, float4 va, float4 vb, float3 org,
                     float3 dir, Hit &best, float tmin)
{
    float3 n = f3(pl.x, pl.y, pl.z);
    float rdot = -dot3(dir, n);
    if ((rdot <= D_FTINY) & (rdot >= -D_FTINY))
        return;
    float t = (dot3(org, n) - pl.w) / rdot;
    if (ray_reject(S, obj, t, rdot, best, tmin))
        return;
    float3 p = org + dir * t;
    int ax = ((od.x >> 8) >> DF_AXSHIFT) & 3;
    int xi = ax + 1 >= 3 ? ax - 2 : ax + 1;
    int yi = xi + 1 >= 3 ? xi - 2 : xi + 1;
    const int nv = (od.x >> 16) & 0xffff;
    const bool in = nv <= 4 ? in_face4(va, vb, nv, comp(p, xi), comp(p, yi))
                            : in_face(S.fvert + od.w, nv, comp(p, xi), comp(p, yi));
    if (!in)
        return;
    best.obj = obj;
    best.t = t;
    best.rod = rdot;
    best.n = n;
}

/* Roots of a*tau^2 + 2*bh*tau + c in ascending order, with the degenerate
 * cases of common/zeroes.c:19-53 (|a| <= FTINY: linear; a discriminant
 * within FTINY^2 of zero: one root).  The root of smaller magnitude is
 * formed as c/q so that it carries no cancellation (the stable form of
 * Numerical Recipes, section 5.6). */
GB_DFN int quadratic_half(float r[2], float a, float bh, float c)
{
    if ((a <= D_FTINY) & (a >= -D_FTINY)) {
        if (fabsf(bh) > 0.5f * D_FTINY) {
            r[0] = -c / (2.f * bh);
            return 1;
        }
        return 0;
    }
    float disc = bh * bh - a * c;
    if (disc < -D_FTINY * D_FTINY)
        return 0;
    if (disc <= D_FTINY * D_FTINY) {
        r[0] = -bh / a;
        return 1;
    }
    float q = -(bh + copysignf(sqrtf(disc), bh));
    float x0 = q / a, x1 = c / q;
    r[0] = fminf(x0, x1);
    r[1] = fmaxf(x0, x1);
    return 2;
}

/* Quadrics in FP32 from a far ray origin.  The reference solves its
 * quadratics in FP64 from the ray origin; in FP32 the constant term
 * |org - centre|^2 - r^2 of a small object seen from a few metres loses
 * most of its digits, and so do the discriminant and the near root.  The
 * ray parameter is therefore split as t = ts + tau, ts the point of closest
 * approach to the centre (sphere) or axis (cone family), and the quadratic
 * is solved in tau with coefficients formed from the closest-approach
 * vector (the method of Haines, Guenther and Akenine-Moeller, "Precision
 * Improvements for Ray/Sphere Intersection", Ray Tracing Gems, 2019,
 * extended to the axial radius of a cone).  The roots are the reference's;
 * only their rounding differs, to a few ulps of the hit position.
 *
 * `self` marks the surface the ray leaves.  One root of its quadratic is
 * the ray origin; in FP64 the reference finds it below FTINY and passes
 * over it.  In FP32 the rounding of the origin, divided by the sine of the
 * angle at which the ray leaves, can put that root well above FTINY for a
 * grazing departure, so it is identified instead: of the two roots, the
 * one nearer zero is the origin and only the other is a candidate.  The
 * first index a test may take is returned. */
GB_DFN int first_root(const float *t, int nr, bool self)
{
    if (!self)
        return 0;
    if (nr < 2)
        return 2;                       /* the only root is the origin */
    return fabsf(t[0]) <= fabsf(t[1]) ? 1 : 2;   /* else the far root is behind */
}

/* rt/sphere.c:15-83 */
GB_DNI void hit_sphere(const gb_dscene &S, int obj, bool bubble, float3 org,
                                           float3 dir, Hit &best, float tmin, bool self)
{
    float4 sp = S.geo[obj];
    float3 f = org - f3(sp.x, sp.y, sp.z);
    float a = dot3(dir, dir);
    float ts = -dot3(f, dir) / a;
    float3 ws = f + dir * ts;           /* centre to closest approach */
    float root[2], tr[2];
    int nr = quadratic_half(root, a, dot3(ws, dir), dot3(ws, ws) - sp.w * sp.w), i;
    tr[0] = ts + root[0];
    tr[1] = ts + root[1];
    float t = 0.f, tau = 0.f;
    for (i = first_root(tr, nr, self); i < nr; i++) {
        tau = root[i];
        if ((t = tr[i]) > tmin)
            break;
    }
    if (i >= nr)
        return;
    if (ray_reject(S, obj, t, (float)(1 - 2 * ((i > 0) ^ bubble)), best, tmin))
        return;
    float rad = bubble ? -sp.w : sp.w;
    float3 n = (ws + dir * tau) * (1.f / rad);
    best.obj = obj;
    best.t = t;
    best.n = n;
    best.rod = -dot3(dir, n);
}

/* rt/o_cone.c:16-146; cone record: tm (12: 3x3 rows then translation),
 * ad (3), p0 (3), al, sl, r0, r1 */
GB_DNI void hit_cone(const gb_dscene &S, int obj, int kind, int ci, float3 org,
                                         float3 dir, Hit &best, float tmin, bool self)
{
    const float *c = S.cone + 24 * ci;
    float3 ad = f3(c[12], c[13], c[14]);
    float3 p0 = f3(c[15], c[16], c[17]);
    float al = c[18], sl = c[19], r0 = c[20], r1 = c[21];
    float a, b, cc, root[2];
    if (kind == DK_RING) {              /* in the ring's own frame */
        float3 rox = f3(org.x * c[0] + org.y * c[3] + org.z * c[6] + c[9],
                        org.x * c[1] + org.y * c[4] + org.z * c[7] + c[10],
                        org.x * c[2] + org.y * c[5] + org.z * c[8] + c[11]);
        float3 rdx = f3(dir.x * c[0] + dir.y * c[3] + dir.z * c[6],
                        dir.x * c[1] + dir.y * c[4] + dir.z * c[7],
                        dir.x * c[2] + dir.y * c[5] + dir.z * c[8]);
        if ((rdx.z <= D_FTINY) & (rdx.z >= -D_FTINY))
            return;
        root[0] = -rox.z / rdx.z;
        if (ray_reject(S, obj, root[0], -rdx.z, best, tmin))
            return;
        b = root[0] * rdx.x + rox.x;
        cc = root[0] * rdx.y + rox.y;
        a = b * b + cc * cc;
        if (a > r1 * r1 || a < r0 * r0)
            return;
        best.obj = obj;
        best.t = root[0];
        best.n = ad;
        best.rod = -rdx.z;
        return;
    }
    /* surface |w(t)| = r0 + k*s(t): s the axial and w the radial part of
     * the ray point relative to p0, k the radius slope (0 for cylinders) */
    const bool cyl = (kind == DK_CYL) | (kind == DK_TUBE);
    const float k = cyl ? 0.f : (r1 - r0) / al;
    float3 v0 = org - p0;
    float s0 = dot3(v0, ad), ds = dot3(dir, ad);
    float3 w0 = v0 - ad * s0, wd = dir - ad * ds;
    float wdd = dot3(wd, wd);
    float ts = wdd > 1e-12f ? -dot3(w0, wd) / wdd : 0.f;   /* closest to the axis */
    float3 ws = w0 + wd * ts;
    float rs = r0 + k * (s0 + ts * ds), kd = k * ds;
    a = wdd - kd * kd;
    b = dot3(ws, wd) - rs * kd;
    cc = dot3(ws, ws) - rs * rs;
    int nr = quadratic_half(root, a, b, cc);
    float tr[2] = {ts + root[0], ts + root[1]};
    for (int rn = first_root(tr, nr, self); rn < nr; rn++) {
        float t = tr[rn];
        if (t <= tmin)
            continue;
        if (t > best.t + D_FTINY)
            break;
        float bb = s0 + t * ds;
        if (bb < 0.f || bb > al)
            continue;
        bool inv = (kind == DK_CUP) | (kind == DK_TUBE);
        if (ray_reject(S, obj, t, (float)(1 - 2 * ((rn > 0) ^ inv)), best, tmin))
            break;
        float aa, c2 = 0.f;
        if (kind == DK_CYL)
            aa = r0;
        else if (kind == DK_TUBE)
            aa = -r0;
        else {
            c2 = r1 - r0;
            aa = r0 + bb * c2 / al;
            if (kind == DK_CUP) {
                c2 = -c2;
                aa = -aa;
            }
        }
        float3 n = (ws + wd * root[rn]) * (1.f / aa);   /* radial part at the hit */
        if ((kind == DK_CONE) | (kind == DK_CUP))
            n = (n * al - ad * c2) * (1.f / sl);
        float nn = dot3(n, n);
        if ((nn > 1.f + D_FTINY) | (nn < 1.f - D_FTINY))
            n = n * (1.f / (.5f + .5f * nn));
        best.obj = obj;
        best.t = t;
        best.n = n;
        best.rod = -dot3(dir, n);
        return;
    }
}

GB_DNI void hit_instance(const gb_dscene &S, int slot, float3 org, float3 dir, Hit &best, int skip);

/* One object's test.  Instances (tested only from the scene's own octree:
 * instances inside instanced octrees are refused when the scene loads) walk
 * their octree in their own coordinates; skip is the surface id the ray
 * leaves, passed on to that walk.  MODE: WALK_FULL tests instances,
 * WALK_NESTED (inside an instance) has none to test, WALK_DEFER marks the
 * walk for the instance-capable kernel instead (best.obj = HIT_DEFER at
 * distance -1, which ends the walk at the end of the leaf), so that the
 * bulk walk carries no nested walk. */
#define WALK_FULL 0
#define WALK_NESTED 1
#define WALK_DEFER 2
#define HIT_DEFER 0x7fffffff    /* with t = -1: every later test fails and the leaf ends the walk */
template <int MODE = WALK_FULL>
GB_DFN void hit_record(const gb_dscene &S, int obj, int4 od, float4 pl, float4 va, float4 vb, float3 org,
                       float3 dir, Hit &best, float tmin, bool self, int skip)
{
    int kind = od.x & 0xff;
    switch (kind) {
    case DK_FACE:
        hit_face(S, obj, od, pl, va, vb, org, dir, best, tmin);
        break;
    case DK_SPHERE:
    case DK_BUBBLE: {                   /* out of line: a copy, so that the */
        Hit b = best;                   /* caller's record stays in registers */
        hit_sphere(S, obj, kind == DK_BUBBLE, org, dir, b, tmin, self);
        best = b;
        break;
    }
    case DK_CONE:
    case DK_CUP:
    case DK_CYL:
    case DK_TUBE:
    case DK_RING: {
        Hit b = best;
        hit_cone(S, obj, kind, od.w, org, dir, b, tmin, self);
        best = b;
        break;
    }
    default:
        if (kind == DK_INSTANCE) {
            if (MODE == WALK_FULL) {
                Hit b = best;
                hit_instance(S, od.w, org, dir, b, skip);
                best = b;
            } else if (MODE == WALK_DEFER) {
                best.obj = HIT_DEFER;
                best.t = -1.f;
            }
        }
        break;
    }
}

/* The object in record slot sl (the records are laid out in the order the
 * octree's leaves first reach their objects, so that the objects of a
 * leaf share cache lines); the record carries the object's index.  The
 * record, plane and packed vertices come from one 64-byte record, all four
 * loads issued together.  The object the ray leaves (skip) is not tested,
 * or, when curved, tested with its root at the origin excluded. */
template <int MODE = WALK_FULL>
GB_DFN void hit_rec(const gb_dscene &S, const float4 *rec, float3 org, float3 dir, Hit &best, float tmin, int skip,
                    bool curved_skip)
{
    const int4 od = GB_LDG(reinterpret_cast<const int4 *>(rec));
    const float4 pl = GB_LDG(rec + 1);
    const float4 va = GB_LDG(rec + 2), vb = GB_LDG(rec + 3);
    const int obj = od.y;
    if (obj != skip)
        hit_record<MODE>(S, obj, od, pl, va, vb, org, dir, best, tmin, false, skip);
    else if (curved_skip)                        /* curved origin surface */
        hit_record<MODE>(S, obj, od, pl, va, vb, org, dir, best, tmin, true, skip);
}

template <int MODE = WALK_FULL>
GB_DFN void hit_slot(const gb_dscene &S, int sl, float3 org, float3 dir, Hit &best, float tmin, int skip,
                     bool curved_skip)
{
    hit_rec<MODE>(S, S.orec + 4 * sl, org, dir, best, tmin, skip, curved_skip);
}

/* the test of object obj (by index) */
template <int MODE = WALK_FULL>
GB_DFN void hit_object(const gb_dscene &S, int obj, float3 org, float3 dir, Hit &best, float tmin)
{
    hit_slot<MODE>(S, GB_LDG(S.oslot + obj), org, dir, best, tmin, -1, false);
}

/* ------------------------------------------------------------------------
 * Octree traversal (rt/raytrace.c:595-793 localhit/raymove/checkhit).
 *
 * Cube positions are kept as integer coordinates on a 2^24 grid over the
 * scene cube, so descending from the root is bit selection and stepping to
 * the neighbour cube is an exact integer increment; only the ray parameter
 * at each cube exit is floating point.  Leaf sets are tested in the
 * reference's order, a hit inside the current cube ends the walk (checkhit),
 * and a hit recorded earlier but never confirmed is still returned when the
 * ray leaves the scene, as localhit does.
 */
/* State of one ray's walk, so that a walk can be advanced one iteration at
 * a time and a lane whose walk ends can start another ray at once.  Every
 * field is indexed with constants only, so that it can live in registers,
 * and it is kept small (the origin relative to the scene cube, the
 * direction signs and the current cube's corner are recomputed where they
 * are used); the descent stack (the node chosen at each level, indexed by
 * level) is kept apart: a WalkStack in local memory, or a column of shared
 * memory.  Every walk runs from FTINY to FHUGE, as every localhit call of
 * the reference on this path does. */
struct Walk {
    float3 org, dir;
    float inv[3];                 /* 1/dir, 0 where the direction is ~0 */
    int skip;                     /* the object the ray leaves */
    bool curved_skip, leaf;
    int q[3];                     /* integer position on the 2^24 grid */
    int rl, k, cnt, span, ax;     /* restart level; leaf set cursor; cube size; exit axis */
    int set;                      /* current leaf: its header record in lrec */
    float texit;
    Hit best;
    uint32_t steps, nodes, tests;
};

struct WalkStack {
    int v[GRID_BITS + 1];
    GB_DFN int &operator[](int i) { return v[i]; }
};

/* The cube a walk runs through: the scene's, or the octree of an instance
 * (in the instance's coordinates). */
struct TopCube {                /* (holds nothing: the scene header is read in place) */
    static constexpr int mode = WALK_FULL;
    GB_DFN float org(const gb_dscene &S, int i) const { return S.cuorg[i]; }
    GB_DFN float size(const gb_dscene &S) const { return S.cusize; }
    GB_DFN float gscale(const gb_dscene &S) const { return S.grid_scale; }
    GB_DFN float cell(const gb_dscene &S) const { return S.cell; }
    GB_DFN int root(const gb_dscene &S) const { return S.wroot; }
};

/* the scene's cube, instances deferred */
struct DeferCube : TopCube {
    static constexpr int mode = WALK_DEFER;
};

/* the cube of a scene without instances: no instance handling compiled */
struct PlainCube : TopCube {
    static constexpr int mode = WALK_NESTED;
};

struct InstCube {
    static constexpr int mode = WALK_NESTED;
    float o[3], sz, gs, cl;
    int rt;
    GB_DFN float org(const gb_dscene &, int i) const { return o[i]; }
    GB_DFN float size(const gb_dscene &) const { return sz; }
    GB_DFN float gscale(const gb_dscene &) const { return gs; }
    GB_DFN float cell(const gb_dscene &) const { return cl; }
    GB_DFN int root(const gb_dscene &) const { return rt; }
};

template <typename Cube>
GB_DFN float walk_rel(const gb_dscene &S, const Cube &C, const Walk &W, int i)   /* origin - cube origin */
{
    return comp(W.org, i) - C.org(S, i);
}

/* Set up the walk of a ray; false when the ray misses the scene cube (no
 * hit, nothing to iterate). */
template <typename Cube, typename Stack>
GB_DFN bool walk_begin(const gb_dscene &S, const Cube &C, float3 org, float3 dir, int skip, Walk &W, Stack &stk)
{
    W.best.obj = -1;
    W.best.t = D_FHUGE;
    W.best.rod = 1.f;
    W.best.n = f3(0.f, 0.f, 0.f);
    W.steps = W.nodes = W.tests = 0;
    const float cs = C.size(S);
    /* Self-intersection: a ray leaving a planar surface cannot meet it
     * again, so that surface is skipped.  A curved origin surface is still
     * tested, since its far side is a legitimate hit, with the root at the
     * origin itself excluded (first_root). */
    W.skip = skip;
    W.curved_skip = false;
    if (skip >= 0 && skip < S.nobjs) {          /* (a surface inside an instance: tested there) */
        int kd = S.obj[skip].x & 0xff;
        W.curved_skip = kd != DK_FACE && kd != DK_RING;
    }
    W.org = org;
    W.dir = dir;
    const float dd[3] = {dir.x, dir.y, dir.z};
    float rr[3];
    int anyd = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        rr[i] = walk_rel(S, C, W, i);
        const bool pos = dd[i] > 1e-7f, neg = dd[i] < -1e-7f;
        W.inv[i] = (pos | neg) ? 1.f / dd[i] : 0.f;
        anyd |= pos | neg;
    }
    if (!anyd)
        return false;
    float t = 0.f;
    bool inside = (rr[0] >= 0.f) & (rr[0] < cs) & (rr[1] >= 0.f) & (rr[1] < cs) & (rr[2] >= 0.f) & (rr[2] < cs);
    if (!inside) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (W.inv[i] == 0.f)
                continue;
            float pl = W.inv[i] > 0.f ? 0.f : cs;
            float dt = (pl - rr[i]) * W.inv[i];
            if (dt > t)
                t = dt;
        }
        t += D_FTINY;
        if (t >= D_FHUGE)
            return false;
        /* the entry point in FP32 carries the rounding of t (about 1e-7 t),
         * far more than the FTINY step the reference takes into the cube,
         * so it is accepted within that rounding; a ray that misses the
         * cube by less walks boundary cells and meets nothing */
        const float eps = 1e-5f * fmaxf(cs, t);
        bool in = true;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float p = rr[i] + dd[i] * t;
            in &= p >= -eps && p < cs + eps;
        }
        if (!in)
            return false;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        int v = GB_F2I_RD((rr[i] + dd[i] * t) * C.gscale(S));
        W.q[i] = min(max(v, 0), GRID_N - 1);
    }
    stk[0] = C.root(S);
    W.rl = 0;
    W.k = 1;
    W.cnt = 0;
    W.span = 0;
    W.ax = 0;
    W.set = 0;
    W.texit = 0.f;
    W.leaf = false;
    return true;
}

/* One iteration of the walk: test objects of the current leaf, and when it
 * is done move to the next leaf (descending from the deepest ancestor it
 * shares with the last one, from the highest coordinate bit that changed).
 * Returns true when the walk has ended. */
#define WALK_TESTS 3
template <typename Cube, typename Stack>
GB_DFN bool walk_iter(const gb_dscene &S, const Cube &C, Walk &W, Stack &stk)
{
    /* up to WALK_TESTS objects of this leaf per iteration, then, if the
     * leaf is done, the step to the next one in the same iteration: fewer
     * iterations (and refill checks) per walk, and lanes testing and lanes
     * stepping share more of each iteration (3 measured best of 1-6) */
#pragma unroll
    for (int u = 0; u < WALK_TESTS; u++) {
        if (W.k > W.cnt)
            break;
        const float4 *rec = S.lrec + 4 * (W.set + W.k);
        W.k++;
        hit_rec<Cube::mode>(S, rec, W.org, W.dir, W.best, D_FTINY, W.skip, W.curved_skip);
    }
    if (W.k <= W.cnt)
        return false;
    const float dd[3] = {W.dir.x, W.dir.y, W.dir.z};
    if (W.leaf) {
        if (W.best.obj >= 0 && W.best.t <= W.texit)
            return true;                         /* hit inside this cube */
        W.steps++;
        if (W.texit >= D_FHUGE || W.steps >= MAX_CUBE_STEPS)
            return true;
        /* step to the face neighbour along the exit axis; the exit point
         * lies on that face, so the other coordinates stay inside this
         * cube's slab (an edge or corner exit takes a second, zero-length
         * step) */
        const int mask = ~(W.span - 1);
        int oq0 = W.q[0], oq1 = W.q[1], oq2 = W.q[2];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const int lo = W.q[i] & mask;        /* this cube's corner */
            if (i == W.ax) {
                W.q[i] = W.inv[i] > 0.f ? lo + W.span : lo - 1;
            } else {
                int v = GB_F2I_RD((walk_rel(S, C, W, i) + dd[i] * W.texit) * C.gscale(S));
                W.q[i] = min(max(v, lo), lo + W.span - 1);
            }
        }
        if ((unsigned)(W.q[0] | W.q[1] | W.q[2]) >= (unsigned)GRID_N)
            return true;                         /* left the scene */
        unsigned diff = (unsigned)((oq0 ^ W.q[0]) | (oq1 ^ W.q[1]) | (oq2 ^ W.q[2]));
        W.rl = GRID_BITS - 1 - (31 - GB_CLZ(diff));
    }
    /* descend from the shared ancestor to the leaf containing q */
    int node = stk[W.rl], level = W.rl;
    while (node >= 0) {
        int sh = GRID_BITS - 1 - level;
        int br = ((W.q[0] >> sh) & 1) | (((W.q[1] >> sh) & 1) << 1) | (((W.q[2] >> sh) & 1) << 2);
        node = GB_LDG(S.wkids + 8 * node + br);
        stk[++level] = node;
        W.nodes++;
    }
    W.span = 1 << (GRID_BITS - level);
    const int mask = ~(W.span - 1);
    W.texit = D_FHUGE;                           /* exit distance of this cube */
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (W.inv[i] == 0.f)
            continue;
        const int lo = W.q[i] & mask;
        float pl = (float)(W.inv[i] > 0.f ? lo + W.span : lo) * C.cell(S);
        float dt = (pl - walk_rel(S, C, W, i)) * W.inv[i];
        if (dt < W.texit) {
            W.texit = dt;
            W.ax = i;
        }
    }
    W.leaf = true;
    W.k = 1;
    W.cnt = 0;
    if (node <= -2) {                            /* full leaf: its set to test */
        const int code = -node - 2;
        W.set = code >> GB_LEAF_SIZEBITS;
        W.cnt = code & ((1 << GB_LEAF_SIZEBITS) - 1);
        if (W.cnt == (1 << GB_LEAF_SIZEBITS) - 1)
            W.cnt = GB_LDG(reinterpret_cast<const int *>(S.lrec + 4 * W.set));
        W.tests += W.cnt;
    }
    return false;
}

/* the walk in the scene's own cube */
template <typename Stack>
GB_DFN bool walk_begin(const gb_dscene &S, float3 org, float3 dir, int skip, Walk &W, Stack &stk)
{
    return walk_begin(S, TopCube{}, org, dir, skip, W, stk);
}

template <typename Stack>
GB_DFN bool walk_iter(const gb_dscene &S, Walk &W, Stack &stk)
{
    return walk_iter(S, TopCube{}, W, stk);
}

/* rt/o_instance.c:15-71: the ray in the instance's coordinates (direction
 * renormalised by the scale) walks the instance's octree; a hit closer than
 * best is transformed back (distance and normal scaled by the forward
 * transform's scale) and recorded with its surface id. */
GB_DNI void hit_instance(const gb_dscene &S, int slot, float3 org, float3 dir, Hit &best, int skip)
{
    const gb_dinst &I = S.inst[slot];
    const float *b = I.bx;
    const float ib = 1.f / I.bsca;
    const float3 o2 = f3(org.x * b[0] + org.y * b[3] + org.z * b[6] + b[9],
                         org.x * b[1] + org.y * b[4] + org.z * b[7] + b[10],
                         org.x * b[2] + org.y * b[5] + org.z * b[8] + b[11]);
    const float3 d2 = f3((dir.x * b[0] + dir.y * b[3] + dir.z * b[6]) * ib,
                         (dir.x * b[1] + dir.y * b[4] + dir.z * b[7]) * ib,
                         (dir.x * b[2] + dir.y * b[5] + dir.z * b[8]) * ib);
    const int local = skip >= I.sidbase && skip < I.sidbase + I.nobjs ? I.firstobj + (skip - I.sidbase) : -1;
    InstCube C;
    C.o[0] = I.cuorg[0];
    C.o[1] = I.cuorg[1];
    C.o[2] = I.cuorg[2];
    C.sz = I.cusize;
    C.gs = I.grid_scale;
    C.cl = I.cell;
    C.rt = I.root;
    Walk W;
    WalkStack stk;
    if (walk_begin(S, C, o2, d2, local, W, stk))
        while (!walk_iter(S, C, W, stk))
            ;
    if (W.best.obj < 0)
        return;
    const float t = W.best.t * I.fsca;
    if (t >= best.t)
        return;
    const float *f = I.fx;
    const float3 n = W.best.n, fi = f3(1.f, 1.f, 1.f) * (1.f / I.fsca);
    best.obj = I.sidbase + (W.best.obj - I.firstobj);
    best.t = t;
    best.rod = W.best.rod;
    best.n = f3((n.x * f[0] + n.y * f[3] + n.z * f[6]) * fi.x, (n.x * f[1] + n.y * f[4] + n.z * f[7]) * fi.y,
                (n.x * f[2] + n.y * f[5] + n.z * f[8]) * fi.z);
}

/* the object Radiance reports for a surface id (r->ro): the object itself,
 * or for a surface inside an instance the instance object when that has a
 * modifier, else the instanced object */
GB_DFN int sid_object(const gb_dscene &S, int sid)
{
    if (sid < S.nobjs || S.ninst == 0)
        return sid;
    int lo = 0, hi = S.ninst - 1;                 /* the last instance with sidbase <= sid */
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S.inst[mid].sidbase <= sid)
            lo = mid;
        else
            hi = mid - 1;
    }
    const gb_dinst &I = S.inst[lo];
    return I.hasmod ? I.obj : I.firstobj + (sid - I.sidbase);
}

/* counters of a finished walk: cube visits, node descents, object tests */
GB_DFN void walk_tally(const Walk &W, uint32_t *tally)
{
    if (tally) {
        tally[0] += W.steps + 1;
        tally[1] += W.nodes;
        tally[2] += W.tests;
    }
}

/* The whole walk of one ray: best hit in `best`, true if there is one. */
GB_DFN bool local_hit(const gb_dscene &S, float3 org, float3 dir, int skip, Hit &best, uint32_t *tally)
{
    Walk W;
    WalkStack stk;
    if (!walk_begin(S, org, dir, skip, W, stk)) {
        best = W.best;
        return false;
    }
    while (!walk_iter(S, W, stk))
        ;
    walk_tally(W, tally);
    best = W.best;
    return best.obj >= 0;
}

/* ------------------------------------------------------------------------
 * Distant source test for rays that leave the scene: rt/source.c:317-377.
 * Returns the source index or -1.
 */
GB_DFN int source_hit(const gb_dscene &S, float3 dir, int rsrc, uint32_t crtype)
{
    int glowsrc = -1;
    int first = 0, last = S.nsrc - 1;
    if (rsrc >= 0)
        first = last = rsrc;
    for (int i = first; i <= last; i++) {
        const gb_dsrc &s = S.src[i];
        if (!(s.flags & DS_DISTANT))
            continue;
        float dt = s.sloc[0] * dir.x + s.sloc[1] * dir.y + s.sloc[2] * dir.z;
        if (2.f * D_PI * (1.f - dt) > s.ss2)
            continue;
        if (i == rsrc)
            return i;
        if (s.flags & DS_SKIP) {
            if (glowsrc < 0)
                glowsrc = i;
            continue;
        }
        return i;
    }
    return glowsrc;
}

/* ------------------------------------------------------------------------
 * Bin programs (rcontrib -b expressions; Reinhart bins as in
 * src/radiance/util/reinhartb.cal:17-47).
 */
GB_DFN float reinhart_bin(float Dx, float Dy, float Dz, const gb_binins *p)
{
    float MF = p[0].op, RHS = p[0].a, rNx = p[0].b, rNy = p[0].c;
    float rNz = p[1].op, Ux = p[1].a, Uy = p[1].b, Uz = p[1].c;
    const float DEG = D_PI / 180.f;
    float inc_dz = -Dx * rNx - Dy * rNy - Dz * rNz;
    float inc_rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
    float inc_ry = Dx * Ux + Dy * Uy + Dz * Uz + inc_dz * (rNx * Ux + rNy * Uy + rNz * Uz);
    float r_alt = (inc_dz - 1.f > 0.f ? D_PI / 2 : (-1.f - inc_dz > 0.f ? -D_PI / 2 : asinf(inc_dz))) / DEG;
    if (!(r_alt > 0.f))
        return -1.f;
    float a = atan2f(inc_rx, inc_ry);
    float r_azi = (-a > 0.f ? a + 2.f * D_PI : a) / DEG;
    float alpha = 90.f / (MF * 7.f + .5f);
    int row = (int)floorf(r_alt / alpha);
    const float tnaz[7] = {30.f, 30.f, 24.f, 24.f, 18.f, 12.f, 6.f};
    /* raccum(row) and rnaz(row) */
    float acc = 0.f;
    float lim = 7.f * MF - .5f;
    float rn = 1.f;
    for (int r = 0; r <= row; r++) {
        float nz;
        if ((float)r - lim > 0.f)
            nz = 1.f;
        else {
            int k = (int)floorf(((float)r + .5f) / MF);
            nz = MF * tnaz[min(max(k, 0), 6)];
        }
        if (r < row)
            acc += nz;
        else
            rn = nz;
    }
    float r_inc = 360.f / rn;
    float azn = (359.9999f - .5f * r_inc - r_azi > 0.f) ? floorf((r_azi + .5f * r_inc) / r_inc) : 0.f;
    return acc + azn;
}

/* CIE sky scanner bin for the incident direction -D about normal rN with up
 * vector U (util/cieskyscan.cal): 8 rows of 12 degrees of altitude with 30,
 * 30, 24, 24, 18, 12, 6 and 1 patches, azimuth from -(right) clockwise,
 * patches starting at azimuth 0 and wound forward in even rows, backward in
 * odd ones; -1 below the horizon. */
GB_DFN float cie_bin(float Dx, float Dy, float Dz, const gb_binins *p)
{
    float RHS = p[0].a, rNx = p[0].b, rNy = p[0].c;
    float rNz = p[1].op, Ux = p[1].a, Uy = p[1].b, Uz = p[1].c;
    const float DEG = D_PI / 180.f;
    float inc_dz = -Dx * rNx - Dy * rNy - Dz * rNz;
    float inc_rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
    float inc_ry = Dx * Ux + Dy * Uy + Dz * Uz + inc_dz * (rNx * Ux + rNy * Uy + rNz * Uz);
    float r_alt = (inc_dz - 1.f > 0.f ? D_PI / 2 : (-1.f - inc_dz > 0.f ? -D_PI / 2 : asinf(inc_dz))) / DEG;
    if (!(r_alt > 0.f))
        return -1.f;
    float a = atan2f(-inc_rx, -inc_ry);
    float c_azi = (-a > 0.f ? a + 2.f * D_PI : a) / DEG;
    const float cnaz[8] = {30.f, 30.f, 24.f, 24.f, 18.f, 12.f, 6.f, 1.f};
    int row = (int)floorf(r_alt / (90.f / 7.5f));
    row = min(max(row, 0), 7);
    float acc = 0.f;
    for (int r = 0; r < row; r++)
        acc += cnaz[r];
    float n = cnaz[row], inc = 360.f / n;
    float azn = 0.f;
    if (359.9999f - c_azi > 0.f)
        azn = (row & 1) ? n - 1.f - floorf(c_azi / inc) : floorf(c_azi / inc);
    return acc + azn;
}

/* Klems bin of the LBNL/Klems full, half or quarter basis for the incident
 * direction -D about normal N with up vector U (util/klems_full.cal:10-40,
 * klems_half.cal, klems_quarter.cal): the polar angle picks the ring (the
 * first whose upper bound is not below it, the last ring otherwise) and the
 * azimuth the patch, patches centred on azimuth 0; -1 behind the surface.
 */
GB_DFN float klems_bin(float Dx, float Dy, float Dz, const gb_binins *p)
{
    const int kind = (int)p[0].op;
    float RHS = p[0].a, Nx = p[0].b, Ny = p[0].c;
    float Nz = p[1].op, Ux = p[1].a, Uy = p[1].b, Uz = p[1].c;
    const float DEG = D_PI / 180.f;
    float c = -Dx * Nx - Dy * Ny - Dz * Nz;
    float pol = c - 1.f > 0.f ? 0.f : (-1.f - c > 0.f ? 180.f : acosf(c) / DEG);
    if (pol - 90.f > 0.f)
        return -1.f;
    float y = -Dx * Ux - Dy * Uy - Dz * Uz + (Nx * Dx + Ny * Dy + Nz * Dz) * (Nx * Ux + Ny * Uy + Nz * Uz);
    float x = -RHS * (Dx * (Uy * Nz - Uz * Ny) + Dy * (Uz * Nx - Ux * Nz) + Dz * (Ux * Ny - Uy * Nx));
    float a = atan2f(y, x);
    float azi = (-a > 0.f ? a + 2.f * D_PI : a) / DEG;
    const float full_pol[9] = {5, 15, 25, 35, 45, 55, 65, 75, 90}, full_naz[9] = {1, 8, 16, 20, 24, 24, 24, 16, 12};
    const float half_pol[7] = {6.5f, 19.5f, 32.5f, 45.5f, 58.5f, 71.5f, 90}, half_naz[7] = {1, 8, 12, 16, 20, 12, 8};
    const float quar_pol[5] = {9, 27, 45, 63, 90}, quar_naz[5] = {1, 8, 12, 12, 8};
    const float *pola = kind == 1 ? full_pol : kind == 2 ? half_pol : quar_pol;
    const float *naz = kind == 1 ? full_naz : kind == 2 ? half_naz : quar_naz;
    const int nrow = kind == 1 ? 9 : kind == 2 ? 7 : 5;
    int row = 0;
    float acc = 0.f;
    while (row < nrow - 1 && pol - pola[row] > 0.f)
        acc += naz[row++];
    float inc = 360.f / naz[row];
    return acc + ((360.f - .5f * inc) - azi > 0.f ? floorf((azi + .5f * inc) / inc) : 0.f);
}

/* Shirley-Chiu bin: the incident direction in the surface frame, its disk
 * position mapped back to the unit square by the inverse of Shirley and
 * Chiu's concentric map, the square cut into SCdim x SCdim cells, the up
 * direction changing fastest; -1 behind the surface (util/disk2square.cal).
 */
GB_DFN float shirchiu_bin(float Dx, float Dy, float Dz, const gb_binins *p)
{
    float SC = p[0].op, RHS = p[0].a, rNx = p[0].b, rNy = p[0].c;
    float rNz = p[1].op, Ux = p[1].a, Uy = p[1].b, Uz = p[1].c;
    const float Q = D_PI / 4.f;
    float dz = -Dx * rNx - Dy * rNy - Dz * rNz;
    if (!(dz > 0.f))
        return -1.f;
    float rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
    float ry = Dx * Ux + Dy * Uy + Dz * Uz + dz * (rNx * Ux + rNy * Uy + rNz * Uz);
    float den2 = rx * rx + ry * ry;
    float radf = den2 - 1e-7f > 0.f ? sqrtf((1.f - dz * dz) / den2) : 0.f;
    float x = rx * radf, y = -ry * radf;
    float r = sqrtf(x * x + y * y);
    float phi = atan2f(y, x);
    if (-phi - Q > 0.f)
        phi += 2.f * D_PI;
    int rgn = (int)floorf((phi + Q) / (2.f * Q)) + 1;
    float a, b;
    switch (rgn) {
    case 1: a = r; b = phi * r / Q; break;
    case 2: a = (2.f * Q - phi) * r / Q; b = r; break;
    case 3: a = -r; b = (D_PI - phi) * r / Q; break;
    case 4: a = (phi - 6.f * Q) * r / Q; b = -r; break;
    default: a = r; b = -r; break;
    }
    return floorf((a + 1.f) * .5f * SC) * SC + floorf((b + 1.f) * .5f * SC);
}

GB_DFN float bin_fn1(int f, float x)
{
    switch (f) {
    case GB_FN_SQRT: return sqrtf(x);
    case GB_FN_SIN: return sinf(x);
    case GB_FN_COS: return cosf(x);
    case GB_FN_TAN: return tanf(x);
    case GB_FN_ASIN: return asinf(x);
    case GB_FN_ACOS: return acosf(x);
    case GB_FN_ATAN: return atanf(x);
    case GB_FN_EXP: return expf(x);
    case GB_FN_LOG: return logf(x);
    case GB_FN_LOG10: return log10f(x);
    default: return ceilf(x);
    }
}

/* the bin program of a contributing ray (binexpr.cpp); -1 when the program
 * is malformed or selects outside its values */
GB_DFN float eval_bin(const gb_binins *prog, float3 d)
{
    float st[GB_BINSTACK], tmp[GB_BINTEMPS];
    int sp = 0;
    for (int pc = 0; pc < GB_BINPROG_MAX; pc++) {
        gb_binins in = prog[pc];
        int op = (int)in.op;
        switch (op) {
        case GB_OP_END:
            return sp > 0 ? st[sp - 1] : -1.f;
        case GB_OP_CONST: st[sp++] = in.a; break;
        case GB_OP_DX: st[sp++] = d.x; break;
        case GB_OP_DY: st[sp++] = d.y; break;
        case GB_OP_DZ: st[sp++] = d.z; break;
        case GB_OP_ADD: sp--; st[sp - 1] += st[sp]; break;
        case GB_OP_SUB: sp--; st[sp - 1] -= st[sp]; break;
        case GB_OP_MUL: sp--; st[sp - 1] *= st[sp]; break;
        case GB_OP_DIV: sp--; st[sp - 1] /= st[sp]; break;
        case GB_OP_NEG: st[sp - 1] = -st[sp - 1]; break;
        case GB_OP_IF: sp -= 2; st[sp - 1] = st[sp - 1] > 0.f ? st[sp] : st[sp + 1]; break;
        case GB_OP_FLOOR: st[sp - 1] = floorf(st[sp - 1]); break;
        case GB_OP_RBIN:
            st[sp++] = reinhart_bin(d.x, d.y, d.z, prog + pc + 1);
            pc += 2;
            break;
        case GB_OP_KBIN:
            st[sp++] = klems_bin(d.x, d.y, d.z, prog + pc + 1);
            pc += 2;
            break;
        case GB_OP_SCBIN:
            st[sp++] = shirchiu_bin(d.x, d.y, d.z, prog + pc + 1);
            pc += 2;
            break;
        case GB_OP_CBIN:
            st[sp++] = cie_bin(d.x, d.y, d.z, prog + pc + 1);
            pc += 2;
            break;
        case GB_OP_POW: sp--; st[sp - 1] = powf(st[sp - 1], st[sp]); break;
        case GB_OP_FN1: st[sp - 1] = bin_fn1((int)in.a, st[sp - 1]); break;
        case GB_OP_ATAN2: sp--; st[sp - 1] = atan2f(st[sp - 1], st[sp]); break;
        case GB_OP_MAXN: case GB_OP_MINN: {
            const int k = (int)in.a;
            float m = st[sp - k];
            for (int j = sp - k + 1; j < sp; j++)
                m = op == GB_OP_MAXN ? fmaxf(m, st[j]) : fminf(m, st[j]);
            sp -= k;
            st[sp++] = m;
            break;
        }
        case GB_OP_SELECT: {                     /* common/calfunc.c select(): index rounded */
            const int k = (int)in.a;
            const int i = (int)(st[sp - k - 1] + .5f);
            const float v = i == 0 ? (float)k : (i > 0 && i <= k ? st[sp - k - 1 + i] : -1.f);
            sp -= k + 1;
            st[sp++] = v;
            break;
        }
        case GB_OP_STORE: tmp[(int)in.a & (GB_BINTEMPS - 1)] = st[--sp]; break;
        case GB_OP_LOAD: st[sp++] = tmp[(int)in.a & (GB_BINTEMPS - 1)]; break;
        default:
            return -1.f;
        }
        if (sp >= GB_BINSTACK - 1 || sp < 0)
            return -1.f;
    }
    return -1.f;
}

#endif
