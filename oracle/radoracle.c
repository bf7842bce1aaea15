/*
 * radoracle.c -- CPU oracle for the GPU ray-tracing path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a scalar FP64 restatement of the
 * reference's algorithms, organised like the reference (recursive ray
 * evaluation with values returned bottom-up, contributions binned by a
 * trace callback that walks the parent chain).  It is used by the tests as
 * the checker, by the benchmark as the timed CPU baseline, and never by the
 * library.  It reads scenes with the library's host loader
 * (pyradiance_gb300/csrc/scene.c), compiles bin expressions with the
 * library's host compiler, and draws random numbers from the same
 * counter-based streams (gbcommon.h) so that it can be compared with the GPU
 * sample for sample.  Its parity with the reference itself is pinned by the
 * golden vectors in tests/golden, produced by the reference programs.
 *
 * Reference functions restated (paths relative to src/radiance):
 *   rayorigin          rt/raytrace.c:39-135
 *   raytrace/raycont   rt/raytrace.c:163-192
 *   raytrans           rt/raytrace.c:194-207
 *   rayreject          rt/raytrace.c:536-575
 *   localhit/raymove   rt/raytrace.c:595-739, checkhit/checkset :743-793
 *   o_face/inface      rt/o_face.c:15-62, common/face.c:121-161
 *   o_sphere           rt/sphere.c:15-83
 *   o_cone             rt/o_cone.c:16-146, quadratic common/zeroes.c:19-53
 *   sourcehit          rt/source.c:317-377
 *   m_light            rt/source.c:749-793
 *   direct             rt/source.c:398-556 (srcray :219, srcvalue :261,
 *                      nextssamp rt/srcsamp.c:37-145 single partition)
 *   m_normal/dirnorm   rt/normal.c:72-360 (plastic, metal, trans)
 *   gaussamp           rt/normal.c:364-495
 *   m_glass            rt/glass.c:45-165
 *   multambient        rt/ambient.c:229-300 (-aa 0 branch)
 *   samp_hemi/ambsample rt/ambcomp.c:177-250, 351-421
 *   getambdiffs/ambsupersamp rt/ambcomp.c:256-346 (-I first hemispheres)
 *   rtcompute/rayirrad rt/rtrace.c:416-468, raytirrad rt/raytrace.c:211-236
 *   eval_irrad/eval_rad/trace_contrib rt/rcontrib.c:272-353
 *   cm_multiply        util/cmatrix.c:421-474
 * Deviations shared with the GPU path: uniform jitter inside each
 * hemisphere stratum instead of urand/ilhash/multisamp, no ambcollision
 * re-draw (it only moves a sample inside its own stratum), every shadow ray
 * tested (-dt thresholding off), one source partition.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gbrad.h"
#include "../pyradiance_gb300/csrc/gbcommon.h"
#include "../pyradiance_gb300/csrc/scene.h"

#define FTINY 1e-6
#define FHUGE 1e10
#define PI 3.14159265358979323846
#define MAXCSET ((GB_MAXSET + 1) * 2 - 1)

/* bin compiler of the library (binexpr.cpp), C-callable shim in orc_bins.cpp */
int orc_compile_bins(const gb_modspec *mods, int nmods, gb_binins *prog, int progcap, int *info, int *nbt,
                     char *err, int errlen);

/* ------------------------------------------------------------------ scene */

typedef struct {
    int flags;               /* DISTANT 1, SKIP 2, FLAT 4, PROX 8, FOLLOW 16, CIR 32 */
    double sloc[3], snorm[3], ss[3][3], ss2, srad, prox;
    double spsiz, spaim[3], spflen;    /* spotlight (rt/srcsupp.c:268-288 makespot) */
    int so;                  /* object */
    int mat;                 /* material object */
} osrc;

typedef struct {
    gb_scene_host H;
    int *mat;                /* per object: material object or -1 */
    int *inst_of;            /* per object: its instance record or -1 */
    osrc *src;
    int nsrc;
    char err[512];
} oscene;

#define S_DISTANT 1
#define S_SKIP 2
#define S_FLAT 4
#define S_PROX 8
#define S_CIR 32
#define S_CYL 64
#define S_SPOT 128

static void vcross(double r[3], const double a[3], const double b[3])
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
static double vdot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double vnormalize(double v[3])
{
    double l = sqrt(vdot(v, v));
    if (l > 0) { v[0] /= l; v[1] /= l; v[2] /= l; }
    return l;
}

/* common/fvect.c:132-155 normalize: the first-order form near unit length,
 * as rtrace normalises the directions it reads (rt/rtrace.c) */
static double normalize_ref(double v[3])
{
    double len, d = vdot(v, v);
    if (d == 0.0) return 0.0;
    if ((d <= 1.0 + FTINY) & (d >= 1.0 - FTINY)) {
        len = 0.5 + 0.5 * d;
        d = 2.0 - len;
    } else {
        len = sqrt(d);
        d = 1.0 / len;
    }
    v[0] *= d; v[1] *= d; v[2] *= d;
    return len;
}

static void perp0(double vp[3], const double v[3])
{
    double v1[3] = {0, 0, 0};
    int i;
    for (i = 3; i--;)
        if (-0.6 < v[i] && v[i] < 0.6)
            break;
    if (i < 0) i = 0;
    v1[i] = 1.0;
    vcross(vp, v1, v);
    vnormalize(vp);
}

static double dist2line(const double p[3], const double a[3], const double b[3])
{
    double d[3], v[3], l2 = 0, t = 0, r = 0;
    int i;
    for (i = 0; i < 3; i++) { d[i] = b[i] - a[i]; v[i] = p[i] - a[i]; l2 += d[i] * d[i]; t += d[i] * v[i]; }
    for (i = 0; i < 3; i++) r += v[i] * v[i];
    return r - t * t / l2;
}

/* rt/source.c:47-142 marksources; rt/srcsupp.c:88-180 fsetsrc/ssetsrc */
static int mark_sources(oscene *O)
{
    gb_scene_host *H = &O->H;
    int32_t i;
    O->src = (osrc *)calloc((size_t)H->nobjs + 1, sizeof(osrc));
    O->nsrc = 0;
    for (i = 0; i < H->nobjs_top; i++) {      /* not the objects of instanced octrees */
        const gb_object *o = &H->objs[i];
        int m = O->mat[i];
        osrc *s;
        if (!gb_is_surface(o->otype) || o->omod < 0 || m < 0)
            continue;
        if (!gb_is_light(H->objs[m].otype))
            continue;
        const gb_object *mo = &H->objs[m];
        if (mo->farg[0] <= FTINY && mo->farg[1] <= FTINY && mo->farg[2] <= FTINY)
            continue;
        if (mo->otype == GT_GLOW && o->otype != GT_SOURCE && mo->farg[3] <= FTINY)
            continue;
        s = &O->src[O->nsrc];
        memset(s, 0, sizeof *s);
        s->so = i;
        s->mat = m;
        if (o->otype == GT_POLYGON) {
            const gb_face *f = &H->faces[i];
            const double *va = o->farg;
            int j, k;
            for (j = 0; j < 3; j++) {
                for (k = 0; k < f->nv; k++) s->sloc[j] += va[3 * k + j];
                s->sloc[j] /= f->nv;
            }
            s->flags = S_FLAT;
            memcpy(s->snorm, f->norm, sizeof s->snorm);
            s->ss2 = f->area;
            for (k = 0; k < f->nv; k++) {
                double d = 0;
                for (j = 0; j < 3; j++) d += (va[3 * k + j] - s->sloc[j]) * (va[3 * k + j] - s->sloc[j]);
                if (d > s->srad) s->srad = d;
            }
            s->srad = sqrt(s->srad);
            if (f->nv == 4) {
                for (j = 0; j < 3; j++) {
                    s->ss[0][j] = .5 * (va[3 + j] - va[j]);
                    s->ss[1][j] = .5 * (va[9 + j] - va[j]);
                }
            } else if (f->nv == 3) {
                int near0 = 2;
                double dmin = dist2line(s->sloc, va + 6, va), l;
                for (k = 0; k < 2; k++) {
                    double d2 = dist2line(s->sloc, va + 3 * k, va + 3 * (k + 1));
                    if (d2 >= dmin) continue;
                    near0 = k;
                    dmin = d2;
                }
                k = (near0 + 1) % 3;
                for (j = 0; j < 3; j++) s->ss[0][j] = va[3 * k + j] - va[3 * near0 + j];
                l = vnormalize(s->ss[0]);
                (void)l;
                for (j = 0; j < 3; j++) s->ss[0][j] *= sqrt(dmin);
                vcross(s->ss[1], f->norm, s->ss[0]);
            } else {
                perp0(s->ss[0], f->norm);
                for (j = 0; j < 3; j++) s->ss[0][j] *= .5 * sqrt(f->area);
                vcross(s->ss[1], f->norm, s->ss[0]);
            }
        } else if (o->otype == GT_SOURCE) {
            double theta;
            int j;
            memcpy(s->sloc, o->farg, 3 * sizeof(double));
            vnormalize(s->sloc);
            theta = PI / 180.0 / 2.0 * o->farg[3];
            s->ss2 = 2.0 * PI * (1.0 - cos(theta));
            s->srad = sqrt(s->ss2 / PI);
            memcpy(s->snorm, s->sloc, sizeof s->snorm);
            perp0(s->ss[0], s->snorm);
            for (j = 0; j < 3; j++) s->ss[0][j] *= .5 * sqrt(s->ss2);
            vcross(s->ss[1], s->snorm, s->ss[0]);
            s->flags = S_DISTANT | S_CIR;
        } else if (o->otype == GT_SPHERE) {            /* rt/srcsupp.c:183-204 sphsetsrc */
            int j;
            if (o->nfargs != 4 || o->farg[3] <= FTINY) {
                snprintf(O->err, sizeof O->err, "oracle: %s: illegal source radius", o->name);
                return -1;
            }
            memcpy(s->sloc, o->farg, 3 * sizeof(double));
            s->srad = o->farg[3];
            s->ss2 = PI * s->srad * s->srad;
            for (j = 0; j < 3; j++) s->ss[j][j] = 0.7236 * o->farg[3];
            s->flags = S_CIR;
        } else if (o->otype == GT_CYLINDER) {          /* rt/srcsupp.c:234-264 cylsetsrc */
            const gb_cone *c = &H->cones[i];
            double ad[3], al = 0, r0;
            int j;
            if (!c->ok || (r0 = o->farg[c->r0]) <= FTINY) {
                snprintf(O->err, sizeof O->err, "oracle: %s: illegal source radius", o->name);
                return -1;
            }
            for (j = 0; j < 3; j++) {
                ad[j] = o->farg[c->p1 + j] - o->farg[c->p0 + j];
                s->sloc[j] = .5 * (o->farg[c->p1 + j] + o->farg[c->p0 + j]);
            }
            al = vnormalize(ad);
            s->srad = .5 * al;
            s->ss2 = 2. * r0 * al;
            for (j = 0; j < 3; j++) s->ss[0][j] = .5 * al * ad[j];
            perp0(s->ss[2], ad);                       /* getperpendicular without the random rotation */
            for (j = 0; j < 3; j++) s->ss[2][j] *= .8559 * r0;
            vcross(s->ss[1], s->ss[2], ad);
            s->flags = S_CYL;
        } else if (o->otype == GT_RING) {              /* rt/srcsupp.c:207-231 rsetsrc */
            const gb_cone *c = &H->cones[i];
            int j;
            if (!c->ok || o->farg[c->r1] <= FTINY || o->farg[c->r0] > 0.0) {
                snprintf(O->err, sizeof O->err, "oracle: %s: illegal ring source", o->name);
                return -1;
            }
            memcpy(s->sloc, o->farg, 3 * sizeof(double));
            memcpy(s->snorm, o->farg + 3, 3 * sizeof(double));
            vnormalize(s->snorm);
            s->srad = o->farg[c->r1];
            s->ss2 = PI * s->srad * s->srad;
            perp0(s->ss[0], s->snorm);                /* setflatss without the random rotation */
            for (j = 0; j < 3; j++) s->ss[0][j] *= .5 * sqrt(s->ss2);
            vcross(s->ss[1], s->snorm, s->ss[0]);
            s->flags = S_FLAT | S_CIR;
        } else {
            snprintf(O->err, sizeof O->err, "oracle: source geometry %s not supported", gb_otype_name(o->otype));
            return -1;
        }
        if (mo->otype == GT_GLOW) {
            s->flags |= S_PROX;
            s->prox = mo->farg[3];
            if (s->flags & S_DISTANT)
                s->flags |= S_SKIP;
        } else if (mo->otype == GT_SPOT) {           /* rt/source.c:104-116 */
            int j;
            double d = 0, d1;
            s->flags |= S_SPOT;
            s->spsiz = 2.0 * PI * (1.0 - cos(PI / 180.0 / 2.0 * mo->farg[3]));
            memcpy(s->spaim, mo->farg + 4, sizeof s->spaim);
            s->spflen = vnormalize(s->spaim);
            for (j = 0; j < 3; j++) d += s->spaim[j] * s->snorm[j];
            d1 = 1. - s->spsiz / (2. * PI);
            if ((s->flags & S_FLAT) && !(d > FTINY) && !(1. - FTINY - d * d < d1 * d1))
                s->flags |= S_SKIP;                     /* checkspot: invalid direction */
        }
        O->nsrc++;
    }
    return 0;
}

static oscene *scene_open(const char *path, int is_rad, char *err, int errlen)
{
    oscene *O = (oscene *)calloc(1, sizeof(oscene));
    int32_t i;
    gb_scene_init(&O->H);
    if (is_rad) {
        if (gb_scene_read_rad_file(&O->H, path) < 0 || gb_scene_build_octree(&O->H, 6, 16384) < 0)
            goto bad;
    } else if (gb_scene_read_oct(&O->H, path) < 0)
        goto bad;
    {
        char dir[4096];
        const char *sl = strrchr(path, '/');
        snprintf(dir, sizeof dir, "%.*s", sl ? (int)(sl - path) : 1, sl ? path : ".");
        if (gb_scene_load_instances(&O->H, dir) < 0)
            goto bad;
    }
    if (gb_scene_prepare(&O->H) < 0)
        goto bad;
    for (i = 0; i < O->H.nobjs; i++)
        if (O->H.objs[i].vnorm) {               /* the shading of smooth meshes is not restated here */
            snprintf(err, errlen, "mesh vertex normals are not supported by the oracle");
            gb_scene_clear(&O->H);
            free(O);
            return NULL;
        }
    O->mat = (int *)malloc(sizeof(int) * ((size_t)O->H.nobjs + 1));
    O->inst_of = (int *)malloc(sizeof(int) * ((size_t)O->H.nobjs + 1));
    for (i = 0; i < O->H.nobjs; i++) {
        O->mat[i] = gb_is_surface(O->H.objs[i].otype) ? gb_find_material(&O->H, i) : -1;
        O->inst_of[i] = -1;
    }
    for (i = 0; i < O->H.ninst; i++)
        O->inst_of[O->H.inst[i].obj] = i;
    if (mark_sources(O) < 0) {
        snprintf(err, errlen, "%s", O->err);
        return NULL;
    }
    return O;
bad:
    snprintf(err, errlen, "%s", gb_scene_error());
    gb_scene_clear(&O->H);
    free(O);
    return NULL;
}

static void scene_close(oscene *O)
{
    if (!O) return;
    gb_scene_clear(&O->H);
    free(O->mat);
    free(O->inst_of);
    free(O->src);
    free(O);
}

/* -------------------------------------------------------------------- ray */

typedef struct RAY {
    double rorg[3], rdir[3], rmax;
    double rop[3], ron[3], rod, rot;
    double rcoef[3], rcol[3];
    double rweight;
    int ro;                  /* object hit, -1 none */
    int rsrc, crtype, rtype, rlvl;
    int rflips;
    const struct RAY *parent;
    uint64_t path;
    uint32_t sensor;
    int origin;              /* object the ray starts on */
    int adepth;              /* ambient recursion depth at this ray */
} RAY;

typedef struct {
    const oscene *O;
    const gb_opts *o;
    int follow;              /* rcontrib: SFOLLOW on all sources */
    uint32_t k0, k1;
    /* rcontrib */
    const gb_binins *prog;
    const int *modinfo;      /* 3 per modifier: program offset, nbins, bin0 */
    const int *trk;          /* per object */
    double *bins;            /* nbins_total x 3 for the current record */
    int64_t rays;
    int ssamp_root;          /* the next hemisphere is an rtrace -I sensor's first */
} ctx;

static double maxc(const double c[3]) { return c[0] > c[1] ? (c[0] > c[2] ? c[0] : c[2]) : (c[1] > c[2] ? c[1] : c[2]); }

static void draw(const ctx *X, uint64_t path, uint32_t sensor, uint32_t group, double u[4], uint32_t *raw)
{
    gb_u4 v = gb_draw(path, sensor, group, X->k0, X->k1);
    int i;
    for (i = 0; i < 4; i++) u[i] = (double)gb_u01(v.v[i]);
    if (raw) *raw = v.v[3];
}

/* getperpendicular(ux, onrm, 1) (common/fvect.c:159-196) with the
 * randomisation drawn from group `group` of ray r */
static void rand_perp(const ctx *X, const RAY *r, uint32_t group, const double onrm[3], double ux[3])
{
    double u[4], v1[3];
    uint32_t raw;
    int ord[3], ii;
    draw(X, r->path, r->sensor, group, u, &raw);
    v1[0] = 0.5 - u[0];
    v1[1] = 0.5 - u[1];
    v1[2] = 0.5 - u[2];
    switch (gb_irand(raw, 6u)) {
    case 0: ord[0] = 0; ord[1] = 1; ord[2] = 2; break;
    case 1: ord[0] = 0; ord[1] = 2; ord[2] = 1; break;
    case 2: ord[0] = 1; ord[1] = 0; ord[2] = 2; break;
    case 3: ord[0] = 1; ord[1] = 2; ord[2] = 0; break;
    case 4: ord[0] = 2; ord[1] = 0; ord[2] = 1; break;
    default: ord[0] = 2; ord[1] = 1; ord[2] = 0; break;
    }
    for (ii = 3; ii--;)
        if ((-0.6 < onrm[ord[ii]]) & (onrm[ord[ii]] < 0.6)) break;
    if (ii < 0) ii = 0;
    v1[ord[ii]] = 1.0;
    vcross(ux, v1, onrm);
    vnormalize(ux);
}

/* rayclear (rt/raytrace.c:138-159) */
static void rayclear(RAY *r)
{
    r->ro = -1;
    r->rot = FHUGE;
    memcpy(r->rop, r->rorg, sizeof r->rop);
    r->ron[0] = -r->rdir[0]; r->ron[1] = -r->rdir[1]; r->ron[2] = -r->rdir[2];
    r->rod = 1.0;
    r->rflips = 0;
    r->rcol[0] = r->rcol[1] = r->rcol[2] = 0;
}

/* rt/raytrace.c:39-135; the random draw of the Russian roulette is the
 * child's own create draw */
static int rayorigin(const ctx *X, RAY *r, int rt, const RAY *ro, const double rc[3], uint32_t code)
{
    double rw;
    if (rc == NULL) {
        rw = 1.0;
        r->rcoef[0] = r->rcoef[1] = r->rcoef[2] = 1.;
    } else {
        rw = maxc(rc);
        if (rw > 1.0) rw = 1.0;
        if (rc != r->rcoef) memcpy(r->rcoef, rc, sizeof r->rcoef);
    }
    r->parent = ro;
    r->rtype = rt;
    if (ro == NULL) {
        r->rlvl = 0;
        r->rweight = rw;
        r->crtype = rt;
        r->rsrc = -1;
        r->adepth = 0;
    } else {
        if (ro->rot >= FHUGE * .99)
            return -1;
        r->rlvl = ro->rlvl;
        r->rsrc = ro->rsrc;
        if (rt & GB_RAYREFL) {
            r->rlvl++;
            if (r->rsrc >= 0) r->rsrc = -1;
            r->rmax = 0.0;
        } else
            r->rmax = 0.0;
        r->crtype = ro->crtype | rt;
        memcpy(r->rorg, ro->rop, sizeof r->rorg);
        r->rweight = ro->rweight * rw;
        r->path = gb_child(ro->path, code);
        r->sensor = ro->sensor;
        r->origin = ro->ro;
        r->adepth = ro->adepth;
    }
    rayclear(r);
    if (r->rweight <= 0.0)
        return -1;
    if (r->crtype & GB_SHADOW)
        return 0;
    if ((X->o->lr <= 0) & (rc != NULL)) {
        double u[4];
        if ((X->o->lr < 0) & (r->rlvl > -X->o->lr))
            return -1;
        if (r->rweight >= X->o->lw)
            return 0;
        draw(X, r->path, r->sensor, GB_G_CREATE, u, NULL);
        if (u[0] > r->rweight / X->o->lw)
            return -1;
        rw = X->o->lw / r->rweight;
        r->rcoef[0] *= rw; r->rcoef[1] *= rw; r->rcoef[2] *= rw;
        r->rweight = X->o->lw;
        return 0;
    }
    return (r->rweight >= X->o->lw) & (r->rlvl <= abs(X->o->lr)) ? 0 : -1;
}

/* ------------------------------------------------------------ intersection */

static int has_mat(const oscene *O, int obj) { return O->mat[obj] >= 0; }
static int is_transp(const oscene *O, int obj) { return O->mat[obj] >= 0 && gb_is_transp(O->H.objs[O->mat[obj]].otype); }

static int rayreject(const oscene *O, int o, const RAY *r, double t, double rod)
{
    if ((t <= FTINY) | (t > r->rot + FTINY)) return 1;
    if (t < r->rot - FTINY) return 0;
    if (o == r->ro) return 1;
    if (r->ro < 0) return 0;
    if (!has_mat(O, o)) {
        if (has_mat(O, r->ro)) return 1;
    } else if (!has_mat(O, r->ro)) {
        return 0;
    } else if (is_transp(O, o)) {
        if (!is_transp(O, r->ro)) return 1;
    } else if (is_transp(O, r->ro)) {
        return 0;
    }
    if (rod <= 0) {
        if (r->rod > 0) return 1;
    } else if (r->rod <= 0) {
        return 0;
    }
    return O->H.objs[r->ro].omod >= O->H.objs[o].omod;
}

static int inface(const double p[3], const gb_face *f, const double *va)
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
#define FEQ(a, b) (fabs((a) - (b)) <= FTINY)
    while (n--) {
        if (FEQ(p0[yi], y) && FEQ(p1[yi], y) && ((p0[xi] > x) ^ (p1[xi] > x))) return 1;
        if ((p0[yi] > y) ^ (p1[yi] > y)) {
            tst = (p0[xi] > x) + (p1[xi] > x);
            if (tst == 2) ncross++;
            else if (tst) {
                double prodA = (p0[yi] - y) * (p1[xi] - x);
                double prodB = (p0[xi] - x) * (p1[yi] - y);
                if (FEQ(prodA, prodB)) return 1;
                ncross += (p1[yi] > p0[yi]) ^ (prodA > prodB);
            } else if (FEQ(p0[xi], x) && FEQ(p1[xi], x)) return 1;
        }
        p0 = p1;
        p1 += 3;
    }
#undef FEQ
    return ncross & 1;
}

static int o_face(const oscene *O, int o, RAY *r)
{
    const gb_face *f = &O->H.faces[o];
    double rdot, t, p[3];
    if (!f->ok) return 0;
    rdot = -vdot(r->rdir, f->norm);
    if ((rdot <= FTINY) & (rdot >= -FTINY)) return 0;
    t = (vdot(r->rorg, f->norm) - f->offset) / rdot;
    if (rayreject(O, o, r, t, rdot)) return 0;
    p[0] = r->rorg[0] + r->rdir[0] * t;
    p[1] = r->rorg[1] + r->rdir[1] * t;
    p[2] = r->rorg[2] + r->rdir[2] * t;
    if (!inface(p, f, O->H.objs[o].farg)) return 0;
    r->ro = o;
    r->rot = t;
    memcpy(r->rop, p, sizeof p);
    memcpy(r->ron, f->norm, sizeof r->ron);
    r->rod = rdot;
    return 1;
}

static int quadratic(double *rt, double a, double b, double c)
{
    double disc;
    int first;
    if (a < -FTINY) first = 1;
    else if (a > FTINY) first = 0;
    else if (fabs(b) > FTINY) { rt[0] = -c / b; return 1; }
    else return 0;
    b *= 0.5;
    disc = b * b - a * c;
    if (disc < -FTINY * FTINY) return 0;
    if (disc <= FTINY * FTINY) { rt[0] = -b / a; return 1; }
    disc = sqrt(disc);
    rt[first] = (-b - disc) / a;
    rt[1 - first] = (-b + disc) / a;
    return 2;
}

static int o_sphere(const oscene *O, int o, RAY *r)
{
    const gb_object *so = &O->H.objs[o];
    const double *ap = so->farg;
    double a = 0, b = 0, c = 0, t = 0, root[2], rad;
    int i, nr, bubble = so->otype == GT_BUBBLE;
    for (i = 0; i < 3; i++) {
        double d = r->rorg[i] - ap[i];
        a += r->rdir[i] * r->rdir[i];
        b += 2.0 * r->rdir[i] * d;
        c += d * d;
    }
    c -= ap[3] * ap[3];
    nr = quadratic(root, a, b, c);
    for (i = 0; i < nr; i++)
        if ((t = root[i]) > FTINY) break;
    if (i >= nr) return 0;
    if (rayreject(O, o, r, t, 1 - 2 * ((i > 0) ^ bubble))) return 0;
    r->ro = o;
    r->rot = t;
    rad = ap[3] * (1 - 2 * bubble);
    for (i = 0; i < 3; i++) {
        r->rop[i] = r->rorg[i] + r->rdir[i] * t;
        r->ron[i] = (r->rop[i] - ap[i]) / rad;
    }
    r->rod = -vdot(r->rdir, r->ron);
    return 1;
}

static int o_cone(const oscene *O, int o, RAY *r)
{
    const gb_object *ob = &O->H.objs[o];
    const gb_cone *co = &O->H.cones[o];
    const double *ca = ob->farg;
    double rox[3], rdx[3], a, b, c, root[2], ad[3], al = co->al;
    int nr, rn, i, otype = ob->otype;
    if (!co->ok) return 0;
    for (i = 0; i < 3; i++) {
        rdx[i] = r->rdir[0] * co->tm[0][i] + r->rdir[1] * co->tm[1][i] + r->rdir[2] * co->tm[2][i];
        rox[i] = r->rorg[0] * co->tm[0][i] + r->rorg[1] * co->tm[1][i] + r->rorg[2] * co->tm[2][i] + co->tm[3][i];
    }
    if (otype == GT_RING) { for (i = 0; i < 3; i++) ad[i] = ca[3 + i]; }
    else for (i = 0; i < 3; i++) ad[i] = ca[co->p1 + i] - ca[co->p0 + i];
    vnormalize(ad);
    if (otype == GT_RING) {
        if ((rdx[2] <= FTINY) & (rdx[2] >= -FTINY)) return 0;
        root[0] = -rox[2] / rdx[2];
        if (rayreject(O, o, r, root[0], -rdx[2])) return 0;
        b = root[0] * rdx[0] + rox[0];
        c = root[0] * rdx[1] + rox[1];
        a = b * b + c * c;
        if (a > ca[co->r1] * ca[co->r1] || a < ca[co->r0] * ca[co->r0]) return 0;
        r->ro = o;
        r->rot = root[0];
        for (i = 0; i < 3; i++) r->rop[i] = r->rorg[i] + r->rdir[i] * r->rot;
        memcpy(r->ron, ad, sizeof ad);
        r->rod = -rdx[2];
        return 1;
    }
    if (otype == GT_CONE || otype == GT_CUP) {
        a = rdx[0] * rdx[0] + rdx[1] * rdx[1] - rdx[2] * rdx[2];
        b = 2.0 * (rdx[0] * rox[0] + rdx[1] * rox[1] - rdx[2] * rox[2]);
        c = rox[0] * rox[0] + rox[1] * rox[1] - rox[2] * rox[2];
    } else {
        a = rdx[0] * rdx[0] + rdx[1] * rdx[1];
        b = 2.0 * (rdx[0] * rox[0] + rdx[1] * rox[1]);
        c = rox[0] * rox[0] + rox[1] * rox[1] - ca[co->r0] * ca[co->r0];
    }
    nr = quadratic(root, a, b, c);
    for (rn = 0; rn < nr; rn++) {
        double p[3], v[3];
        if (root[rn] <= FTINY) continue;
        if (root[rn] > r->rot + FTINY) break;
        for (i = 0; i < 3; i++) { p[i] = r->rorg[i] + r->rdir[i] * root[rn]; v[i] = p[i] - ca[co->p0 + i]; }
        b = vdot(v, ad);
        if (b < 0.0 || b > al) continue;
        if (rayreject(O, o, r, root[rn], 1 - 2 * ((rn > 0) ^ (otype == GT_CUP || otype == GT_TUBE)))) break;
        r->ro = o;
        r->rot = root[rn];
        memcpy(r->rop, p, sizeof p);
        if (otype == GT_CYLINDER) a = ca[co->r0];
        else if (otype == GT_TUBE) a = -ca[co->r0];
        else {
            c = ca[co->r1] - ca[co->r0];
            a = ca[co->r0] + b * c / al;
            if (otype == GT_CUP) { c = -c; a = -a; }
        }
        for (i = 0; i < 3; i++) r->ron[i] = (v[i] - b * ad[i]) / a;
        if (otype == GT_CONE || otype == GT_CUP)
            for (i = 0; i < 3; i++) r->ron[i] = (al * r->ron[i] - c * ad[i]) / co->sl;
        a = vdot(r->ron, r->ron);
        if ((a > 1. + FTINY) | (a < 1. - FTINY)) {
            c = 1. / (.5 + .5 * a);
            for (i = 0; i < 3; i++) r->ron[i] *= c;
        }
        r->rod = -vdot(r->rdir, r->ron);
        return 1;
    }
    return 0;
}

typedef struct { double cuorg[3]; double cusize; int cutree; } CUBE;

static int localhit_cube(const oscene *O, RAY *r, const CUBE *scene);

/* common/mat4.c multp3/multv3: row vector times a 4x4 transform */
static void xf_vec(double out[3], const double v[3], const double m[4][4])
{
    double t[3];
    int j;
    for (j = 0; j < 3; j++) t[j] = v[0] * m[0][j] + v[1] * m[1][j] + v[2] * m[2][j];
    memcpy(out, t, sizeof t);
}

static void xf_pnt(double out[3], const double p[3], const double m[4][4])
{
    xf_vec(out, p, m);
    out[0] += m[3][0];
    out[1] += m[3][1];
    out[2] += m[3][2];
}

/* rt/o_instance.c:15-71: the ray in the instance's coordinates through its
 * octree, the hit transformed back if it is closer */
static int o_instance(const oscene *O, int o, RAY *r)
{
    const gb_instance *ins = &O->H.inst[O->inst_of[o]];
    const gb_subscene *sc = &O->H.subs[ins->sub];
    RAY rc = *r;
    CUBE cu;
    double d;
    int i;
    xf_pnt(rc.rorg, r->rorg, ins->b.xfm);
    xf_vec(rc.rdir, r->rdir, ins->b.xfm);
    for (i = 0; i < 3; i++) rc.rdir[i] /= ins->b.sca;
    rayclear(&rc);
    memcpy(cu.cuorg, sc->cuorg, sizeof cu.cuorg);
    cu.cusize = sc->cusize;
    cu.cutree = sc->root;
    if (!localhit_cube(O, &rc, &cu)) return 0;
    if (rc.rot * ins->f.sca >= r->rot) return 0;
    r->ro = O->H.objs[o].omod >= 0 ? o : rc.ro;
    r->rot = rc.rot * ins->f.sca;
    xf_pnt(r->rop, rc.rop, ins->f.xfm);
    xf_vec(r->ron, rc.ron, ins->f.xfm);
    d = 1. / ins->f.sca;
    for (i = 0; i < 3; i++) r->ron[i] *= d;
    r->rod = rc.rod;
    return 1;
}

static int object_hit(const oscene *O, int o, RAY *r)
{
    switch (O->H.objs[o].otype) {
    case GT_POLYGON: return o_face(O, o, r);
    case GT_SPHERE: case GT_BUBBLE: return o_sphere(O, o, r);
    case GT_CONE: case GT_CUP: case GT_CYLINDER: case GT_TUBE: case GT_RING: return o_cone(O, o, r);
    case GT_INSTANCE: case GT_MESH: return o_instance(O, o, r);
    default: return 0;
    }
}

static int incube(const CUBE *cu, const double pt[3])
{
    int i;
    for (i = 0; i < 3; i++)
        if (cu->cuorg[i] > pt[i] || pt[i] >= cu->cuorg[i] + cu->cusize) return 0;
    return 1;
}

/* checked-set merge (rt/raytrace.c:764-793) */
static void checkset(int32_t *os, int32_t *cs)
{
    static __thread int32_t cset[MAXCSET + GB_MAXSET + 1];
    int i, j, k;
    cset[0] = 0;
    k = 0;
    for (i = j = 1; i <= os[0]; i++) {
        while (j <= cs[0] && cs[j] < os[i]) cset[++cset[0]] = cs[j++];
        if (j > cs[0] || os[i] != cs[j]) {
            os[++k] = os[i];
            cset[++cset[0]] = os[i];
        }
    }
    if (!(os[0] = k)) return;
    while (j <= cs[0]) cset[++cset[0]] = cs[j++];
    if (cset[0] > MAXCSET) cset[0] = MAXCSET;
    memcpy(cs, cset, sizeof(int32_t) * (cset[0] + 1));
}

static int checkhit(const oscene *O, RAY *r, CUBE *cu, int32_t *cxs)
{
    int32_t oset[GB_MAXSET + 1];
    const int32_t *s = gb_scene_set(&O->H, cu->cutree);
    int i;
    memcpy(oset, s, sizeof(int32_t) * (s[0] + 1));
    checkset(oset, cxs);
    for (i = oset[0]; i > 0; i--)
        object_hit(O, oset[i], r);
    if (r->ro < 0) return 0;
    return incube(cu, r->rop);
}

#define RAYHIT (-1)

static int raymove(const oscene *O, double pos[3], int32_t *cxs, int dirf, RAY *r, CUBE *cu)
{
    int ax = 0;
    double dt, t;
    if (cu->cutree >= 0) {
        CUBE ck;
        int br = 0, sgn;
        ck.cusize = cu->cusize * 0.5;
        memcpy(ck.cuorg, cu->cuorg, sizeof ck.cuorg);
        if (pos[0] >= ck.cuorg[0] + ck.cusize) { ck.cuorg[0] += ck.cusize; br |= 1; }
        if (pos[1] >= ck.cuorg[1] + ck.cusize) { ck.cuorg[1] += ck.cusize; br |= 2; }
        if (pos[2] >= ck.cuorg[2] + ck.cusize) { ck.cuorg[2] += ck.cusize; br |= 4; }
        for (;;) {
            ck.cutree = O->H.kids[8 * cu->cutree + br];
            if ((ax = raymove(O, pos, cxs, dirf, r, &ck)) == RAYHIT) return RAYHIT;
            sgn = 1 << ax;
            if (sgn & dirf) {
                if (sgn & br) return ax;
                ck.cuorg[ax] += ck.cusize;
                br |= sgn;
            } else {
                if (sgn & br) { ck.cuorg[ax] -= ck.cusize; br &= ~sgn; }
                else return ax;
            }
        }
    }
    if (cu->cutree <= -2) {
        if (checkhit(O, r, cu, cxs)) return RAYHIT;
    }
    if (dirf & 0x11) {
        dt = dirf & 1 ? cu->cuorg[0] + cu->cusize : cu->cuorg[0];
        t = (dt - pos[0]) / r->rdir[0];
        ax = 0;
    } else t = FHUGE;
    if (dirf & 0x22) {
        dt = dirf & 2 ? cu->cuorg[1] + cu->cusize : cu->cuorg[1];
        dt = (dt - pos[1]) / r->rdir[1];
        if (dt < t) { t = dt; ax = 1; }
    }
    if (dirf & 0x44) {
        dt = dirf & 4 ? cu->cuorg[2] + cu->cusize : cu->cuorg[2];
        dt = (dt - pos[2]) / r->rdir[2];
        if (dt < t) { t = dt; ax = 2; }
    }
    pos[0] += r->rdir[0] * t;
    pos[1] += r->rdir[1] * t;
    pos[2] += r->rdir[2] * t;
    return ax;
}

static int localhit(ctx *X, RAY *r)
{
    CUBE scene;
    X->rays++;
    memcpy(scene.cuorg, X->O->H.cuorg, sizeof scene.cuorg);
    scene.cusize = X->O->H.cusize;
    scene.cutree = X->O->H.root;
    return localhit_cube(X->O, r, &scene);
}

static int localhit_cube(const oscene *O, RAY *r, const CUBE *scube)
{
    int32_t cxset[MAXCSET + 1];
    double curpos[3], t, dt;
    int sflags = 0, i;
    CUBE scene = *scube;
    for (i = 0; i < 3; i++) {
        curpos[i] = r->rorg[i];
        if (r->rdir[i] > 1e-7) sflags |= 1 << i;
        else if (r->rdir[i] < -1e-7) sflags |= 0x10 << i;
    }
    if (!sflags) return 0;
    t = 0.0;
    if (!incube(&scene, curpos)) {
        for (i = 0; i < 3; i++) {
            if (sflags & 1 << i) dt = scene.cuorg[i];
            else if (sflags & 0x10 << i) dt = scene.cuorg[i] + scene.cusize;
            else continue;
            dt = (dt - r->rorg[i]) / r->rdir[i];
            if (dt > t) t = dt;
        }
        t += FTINY;
        if (t >= r->rot) return 0;
        for (i = 0; i < 3; i++) curpos[i] += r->rdir[i] * t;
        if (!incube(&scene, curpos)) return 0;
    }
    cxset[0] = 0;
    raymove(O, curpos, cxset, sflags, r, &scene);
    return r->ro >= 0;
}

/* rt/source.c:317-377 */
static int sourcehit(const ctx *X, RAY *r)
{
    const oscene *O = X->O;
    int glowsrc = -1, first = 0, last = O->nsrc - 1, i;
    if (r->rsrc >= 0) first = last = r->rsrc;
    for (i = first; i <= last; i++) {
        const osrc *s = &O->src[i];
        if (!(s->flags & S_DISTANT)) continue;
        if (2. * PI * (1. - vdot(s->sloc, r->rdir)) > s->ss2) continue;
        if (i == r->rsrc) { r->ro = s->so; break; }
        if (s->flags & S_SKIP) { if (glowsrc < 0) glowsrc = i; continue; }
        r->ro = s->so;
        break;
    }
    if (r->ro < 0) {
        if (glowsrc >= 0) r->ro = O->src[glowsrc].so;
        else return 0;
    }
    return 1;
}

/* ------------------------------------------------------------- shading */

static void raytrace(ctx *X, RAY *r);
static int m_normal(ctx *X, int m, RAY *r);

static void trace_contrib(ctx *X, const RAY *r)
{
    const oscene *O = X->O;
    int slot, bn;
    double contr[3] = {1, 1, 1}, bval;
    const RAY *p;
    if (!X->prog || r->ro < 0 || O->H.objs[r->ro].omod < 0) return;
    if (r->rsrc >= 0 && O->src[r->rsrc].so != r->ro) return;
    slot = X->trk[r->ro];
    if (slot < 0) return;
    if (X->o->V) {
        int i;
        for (i = 0; i < 3; i++) if (r->rcoef[i] * r->rcol[i] > FTINY) break;
        if (i >= 3) return;
    } else if (maxc(r->rcoef) <= FTINY)
        return;
    {
        /* evaluate the bin program in double (gbcommon.h byte code) */
        const gb_binins *pr = X->prog + X->modinfo[3 * slot];
        double st[GB_BINSTACK], tmp[GB_BINTEMPS];
        int sp = 0, pc;
        bval = -1;
        for (pc = 0; pc < GB_BINPROG_MAX; pc++) {
            gb_binins in = pr[pc];
            int op = (int)in.op;
            if (op == GB_OP_END) { bval = sp > 0 ? st[sp - 1] : -1; break; }
            switch (op) {
            case GB_OP_CONST: st[sp++] = in.a; break;
            case GB_OP_DX: st[sp++] = r->rdir[0]; break;
            case GB_OP_DY: st[sp++] = r->rdir[1]; break;
            case GB_OP_DZ: st[sp++] = r->rdir[2]; break;
            case GB_OP_ADD: sp--; st[sp - 1] += st[sp]; break;
            case GB_OP_SUB: sp--; st[sp - 1] -= st[sp]; break;
            case GB_OP_MUL: sp--; st[sp - 1] *= st[sp]; break;
            case GB_OP_DIV: sp--; st[sp - 1] /= st[sp]; break;
            case GB_OP_NEG: st[sp - 1] = -st[sp - 1]; break;
            case GB_OP_IF: sp -= 2; st[sp - 1] = st[sp - 1] > 0 ? st[sp] : st[sp + 1]; break;
            case GB_OP_FLOOR: st[sp - 1] = floor(st[sp - 1]); break;
            case GB_OP_POW: sp--; st[sp - 1] = pow(st[sp - 1], st[sp]); break;
            case GB_OP_FN1: {
                double x = st[sp - 1];
                switch ((int)in.a) {
                case GB_FN_SQRT: x = sqrt(x); break;
                case GB_FN_SIN: x = sin(x); break;
                case GB_FN_COS: x = cos(x); break;
                case GB_FN_TAN: x = tan(x); break;
                case GB_FN_ASIN: x = asin(x); break;
                case GB_FN_ACOS: x = acos(x); break;
                case GB_FN_ATAN: x = atan(x); break;
                case GB_FN_EXP: x = exp(x); break;
                case GB_FN_LOG: x = log(x); break;
                case GB_FN_LOG10: x = log10(x); break;
                default: x = ceil(x); break;
                }
                st[sp - 1] = x;
                break;
            }
            case GB_OP_ATAN2: sp--; st[sp - 1] = atan2(st[sp - 1], st[sp]); break;
            case GB_OP_MAXN: case GB_OP_MINN: {
                int k = (int)in.a, j;
                double m = st[sp - k];
                for (j = sp - k + 1; j < sp; j++) m = op == GB_OP_MAXN ? fmax(m, st[j]) : fmin(m, st[j]);
                sp -= k;
                st[sp++] = m;
                break;
            }
            case GB_OP_SELECT: {
                int k = (int)in.a, i = (int)(st[sp - k - 1] + .5);
                double v = i == 0 ? (double)k : (i > 0 && i <= k ? st[sp - k - 1 + i] : -1.0);
                sp -= k + 1;
                st[sp++] = v;
                break;
            }
            case GB_OP_STORE: tmp[(int)in.a & (GB_BINTEMPS - 1)] = st[--sp]; break;
            case GB_OP_LOAD: st[sp++] = tmp[(int)in.a & (GB_BINTEMPS - 1)]; break;
            case GB_OP_RBIN: {
                /* util/reinhartb.cal:17-47 */
                const gb_binins *q = pr + pc + 1;
                double MF = q[0].op, RHS = q[0].a, rNx = q[0].b, rNy = q[0].c, rNz = q[1].op, Ux = q[1].a,
                       Uy = q[1].b, Uz = q[1].c;
                double Dx = r->rdir[0], Dy = r->rdir[1], Dz = r->rdir[2], DEG = PI / 180;
                double inc_dz = -Dx * rNx - Dy * rNy - Dz * rNz;
                double inc_rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
                double inc_ry = Dx * Ux + Dy * Uy + Dz * Uz + inc_dz * (rNx * Ux + rNy * Uy + rNz * Uz);
                double alt = (inc_dz - 1 > 0 ? PI / 2 : (-1 - inc_dz > 0 ? -PI / 2 : asin(inc_dz))) / DEG;
                static const double tnaz[7] = {30, 30, 24, 24, 18, 12, 6};
                if (!(alt > 0)) st[sp++] = -1;
                else {
                    double a = atan2(inc_rx, inc_ry), azi = (-a > 0 ? a + 2 * PI : a) / DEG;
                    double alpha = 90 / (MF * 7 + .5), acc = 0, rn = 1, inc;
                    int row = (int)floor(alt / alpha), rr;
                    for (rr = 0; rr <= row; rr++) {
                        double nz;
                        if (rr - (7 * MF - .5) > 0) nz = 1;
                        else {
                            int k = (int)floor((rr + .5) / MF);
                            nz = MF * tnaz[k < 0 ? 0 : (k > 6 ? 6 : k)];
                        }
                        if (rr < row) acc += nz; else rn = nz;
                    }
                    inc = 360 / rn;
                    st[sp++] = acc + ((359.9999 - .5 * inc - azi > 0) ? floor((azi + .5 * inc) / inc) : 0);
                }
                pc += 2;
                break;
            }
            case GB_OP_KBIN: {
                /* util/klems_full.cal:10-40 (and klems_half.cal, klems_quarter.cal) */
                static const double fp[9] = {5, 15, 25, 35, 45, 55, 65, 75, 90}, fn[9] = {1, 8, 16, 20, 24, 24, 24, 16, 12};
                static const double hp[7] = {6.5, 19.5, 32.5, 45.5, 58.5, 71.5, 90}, hn[7] = {1, 8, 12, 16, 20, 12, 8};
                static const double qp[5] = {9, 27, 45, 63, 90}, qn[5] = {1, 8, 12, 12, 8};
                const gb_binins *q = pr + pc + 1;
                int kind = (int)q[0].op, nrow = kind == 1 ? 9 : kind == 2 ? 7 : 5, row = 0;
                const double *pola = kind == 1 ? fp : kind == 2 ? hp : qp, *naz = kind == 1 ? fn : kind == 2 ? hn : qn;
                double RHS = q[0].a, Nx = q[0].b, Ny = q[0].c, Nz = q[1].op, Ux = q[1].a, Uy = q[1].b, Uz = q[1].c;
                double Dx = r->rdir[0], Dy = r->rdir[1], Dz = r->rdir[2], DEG = PI / 180;
                double c = -Dx * Nx - Dy * Ny - Dz * Nz;
                double pol = c - 1 > 0 ? 0 : (-1 - c > 0 ? 180 : acos(c) / DEG);
                if (pol - 90 > 0) st[sp++] = -1;
                else {
                    double y = -Dx * Ux - Dy * Uy - Dz * Uz + (Nx * Dx + Ny * Dy + Nz * Dz) * (Nx * Ux + Ny * Uy + Nz * Uz);
                    double x = -RHS * (Dx * (Uy * Nz - Uz * Ny) + Dy * (Uz * Nx - Ux * Nz) + Dz * (Ux * Ny - Uy * Nx));
                    double a = atan2(y, x), azi = (-a > 0 ? a + 2 * PI : a) / DEG, acc = 0, inc;
                    while (row < nrow - 1 && pol - pola[row] > 0) acc += naz[row++];
                    inc = 360 / naz[row];
                    st[sp++] = acc + ((360 - .5 * inc) - azi > 0 ? floor((azi + .5 * inc) / inc) : 0);
                }
                pc += 2;
                break;
            }
            case GB_OP_SCBIN: {
                /* util/disk2square.cal: the inverse concentric map and scbin */
                const gb_binins *q = pr + pc + 1;
                double SC = q[0].op, RHS = q[0].a, rNx = q[0].b, rNy = q[0].c, rNz = q[1].op, Ux = q[1].a,
                       Uy = q[1].b, Uz = q[1].c, Q = PI / 4;
                double Dx = r->rdir[0], Dy = r->rdir[1], Dz = r->rdir[2];
                double dz = -Dx * rNx - Dy * rNy - Dz * rNz;
                if (!(dz > 0)) st[sp++] = -1;
                else {
                    double rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
                    double ry = Dx * Ux + Dy * Uy + Dz * Uz + dz * (rNx * Ux + rNy * Uy + rNz * Uz);
                    double den2 = rx * rx + ry * ry, radf = den2 - 1e-7 > 0 ? sqrt((1 - dz * dz) / den2) : 0;
                    double x = rx * radf, y = -ry * radf, rr = sqrt(x * x + y * y), phi = atan2(y, x), a, b;
                    int rgn;
                    if (-phi - Q > 0) phi += 2 * PI;
                    rgn = (int)floor((phi + Q) / (2 * Q)) + 1;
                    switch (rgn) {
                    case 1: a = rr; b = phi * rr / Q; break;
                    case 2: a = (2 * Q - phi) * rr / Q; b = rr; break;
                    case 3: a = -rr; b = (PI - phi) * rr / Q; break;
                    case 4: a = (phi - 6 * Q) * rr / Q; b = -rr; break;
                    default: a = rr; b = -rr; break;
                    }
                    st[sp++] = floor((a + 1) * .5 * SC) * SC + floor((b + 1) * .5 * SC);
                }
                pc += 2;
                break;
            }
            case GB_OP_CBIN: {
                /* util/cieskyscan.cal: rows of 12 degrees, azimuth from behind, alternate windings */
                const gb_binins *q = pr + pc + 1;
                double RHS = q[0].a, rNx = q[0].b, rNy = q[0].c, rNz = q[1].op, Ux = q[1].a, Uy = q[1].b,
                       Uz = q[1].c, DEG = PI / 180;
                double Dx = r->rdir[0], Dy = r->rdir[1], Dz = r->rdir[2];
                double inc_dz = -Dx * rNx - Dy * rNy - Dz * rNz;
                double inc_rx = -RHS * (Dx * (Uy * rNz - Uz * rNy) + Dy * (Uz * rNx - Ux * rNz) + Dz * (Ux * rNy - Uy * rNx));
                double inc_ry = Dx * Ux + Dy * Uy + Dz * Uz + inc_dz * (rNx * Ux + rNy * Uy + rNz * Uz);
                double alt = (inc_dz - 1 > 0 ? PI / 2 : (-1 - inc_dz > 0 ? -PI / 2 : asin(inc_dz))) / DEG;
                static const double cnaz[8] = {30, 30, 24, 24, 18, 12, 6, 1};
                if (!(alt > 0)) st[sp++] = -1;
                else {
                    double a = atan2(-inc_rx, -inc_ry), azi = (-a > 0 ? a + 2 * PI : a) / DEG, acc = 0, n, inc;
                    int row = (int)floor(alt / (90 / 7.5)), rr;
                    if (row > 7) row = 7;
                    for (rr = 0; rr < row; rr++) acc += cnaz[rr];
                    n = cnaz[row];
                    inc = 360 / n;
                    st[sp++] = acc + (359.9999 - azi > 0 ? ((row & 1) ? n - 1 - floor(azi / inc) : floor(azi / inc)) : 0);
                }
                pc += 2;
                break;
            }
            default: return;
            }
        }
    }
    if (bval <= -.5) return;
    bn = (int)(bval + .5);
    if (bn >= X->modinfo[3 * slot + 1]) return;
    for (p = r; p != NULL && (p->crtype & GB_PRIMARY); p = p->parent) {
        contr[0] *= p->rcoef[0];
        contr[1] *= p->rcoef[1];
        contr[2] *= p->rcoef[2];
    }
    if (X->o->V) { contr[0] *= r->rcol[0]; contr[1] *= r->rcol[1]; contr[2] *= r->rcol[2]; }
    {
        double *d = X->bins + 3 * (X->modinfo[3 * slot + 2] + bn);
        d[0] += contr[0]; d[1] += contr[1]; d[2] += contr[2];
    }
}

static void raytrans(ctx *X, RAY *r)
{
    RAY tr;
    rayorigin(X, &tr, GB_TRANS, r, NULL, GB_C_PASS);
    memcpy(tr.rdir, r->rdir, sizeof tr.rdir);
    raytrace(X, &tr);
    memcpy(r->rcol, tr.rcol, sizeof r->rcol);
}

static void flipsurface(RAY *r)
{
    r->rod = -r->rod;
    r->ron[0] = -r->ron[0]; r->ron[1] = -r->ron[1]; r->ron[2] = -r->ron[2];
    r->rflips++;
}

static int m_light(ctx *X, int m, RAY *r)
{
    const gb_object *mo = &X->O->H.objs[m];
    int glow = mo->otype == GT_GLOW;
    int distglow = glow && mo->farg[3] >= -FTINY && r->rot > mo->farg[3];
    if ((r->crtype & (GB_AMBIENT | GB_SPECULAR)) && !((r->crtype & GB_SHADOW) || r->rod < 0.0 || distglow)) {
        r->rcoef[0] = r->rcoef[1] = r->rcoef[2] = 0;
        return 1;
    }
    if (r->rsrc >= 0 && X->O->src[r->rsrc].so != r->ro) {
        r->rcoef[0] = r->rcoef[1] = r->rcoef[2] = 0;
        return 1;
    }
    if (r->rod < 0.0) return 1;
    if (mo->otype == GT_SPOT) {                      /* rt/source.c:782 spotout (local source) */
        double aim[3] = {mo->farg[4], mo->farg[5], mo->farg[6]};
        vnormalize(aim);
        if (2.0 * PI * (1.0 - cos(PI / 180.0 / 2.0 * mo->farg[3])) < 2.0 * PI * (1.0 + vdot(aim, r->rdir))) return 1;
    }
    r->rcol[0] = mo->farg[0];
    r->rcol[1] = mo->farg[1];
    r->rcol[2] = mo->farg[2];
    return 1;
}

typedef struct {
    double mcolor[3], scolor[3], pnorm[3], prdir[3];
    double rdiff, rspec, alpha2, pdot;
    double trans, tspec, tdiff;
    int pure, refl, rblt, flat, tran, tblt;
} NORMDAT;

#define FRESNE(ci) (exp(-5.85 * (ci)) - 0.00202943064)
#define FRESTHRESH 0.017999

static void dirnorm(const ctx *X, double sc[3], const NORMDAT *np, const RAY *r, const double ldir[3], double omega)
{
    double ldot = vdot(np->pnorm, ldir), lrdiff, ltdiff, dtmp;
    int i;
    sc[0] = sc[1] = sc[2] = 0;
    if (ldot < 0.0 ? np->trans <= FTINY : np->trans >= 1.0 - FTINY) return;    /* wrong side */
    lrdiff = np->rdiff;
    ltdiff = np->tdiff;
    if (np->pure && np->rspec >= FRESTHRESH && ((lrdiff > FTINY) | (ltdiff > FTINY))) {
        dtmp = 1. - FRESNE(fabs(ldot));
        lrdiff *= dtmp;
        ltdiff *= dtmp;
    }
    if ((ldot > FTINY) & (lrdiff > FTINY)) {
        dtmp = ldot * omega * lrdiff * (1.0 / PI);
        for (i = 0; i < 3; i++) sc[i] += np->mcolor[i] * dtmp;
    }
    if ((ldot < -FTINY) & (ltdiff > FTINY)) {                /* diffuse transmission */
        dtmp = -ldot * omega * ltdiff * (1.0 / PI);
        for (i = 0; i < 3; i++) sc[i] += np->mcolor[i] * dtmp;
    }
    if ((ldot < -FTINY) & np->tran & !np->pure) {            /* specular transmission */
        dtmp = np->alpha2 + omega * (1.0 / PI);
        dtmp = exp((2. * vdot(np->prdir, ldir) - 2.) / dtmp) / (PI * dtmp);
        if (dtmp > FTINY) {
            dtmp *= np->tspec * omega * sqrt(-ldot / np->pdot);
            for (i = 0; i < 3; i++) sc[i] += np->mcolor[i] * dtmp;
        }
    }
    if ((ldot > FTINY) & np->refl & !np->pure) {
        double vt[3], d2, d3, d4;
        dtmp = np->alpha2;
        if (np->flat) dtmp += (1. - X->o->dj) * omega * (0.25 / PI);
        for (i = 0; i < 3; i++) vt[i] = ldir[i] - r->rdir[i];
        d2 = vdot(vt, np->pnorm);
        d2 *= d2;
        d3 = vdot(vt, vt);
        d4 = (d3 - d2) / d2;
        dtmp = exp(-d4 / dtmp) * d3 / (PI * d2 * d2 * dtmp);
        if (dtmp > FTINY) {
            dtmp *= ldot * omega;
            for (i = 0; i < 3; i++) sc[i] += np->scolor[i] * dtmp;
        }
    }
}

/* Partitions of a flat local source as seen from point ro (rt/srcsamp.c:
 * 260-330 flatpart, flt_partit): a source larger than -ds times its
 * distance (scaled by the ray weight) is halved along its longer side,
 * recursively, up to MAXSPART pieces.  Each piece is returned as its centre
 * and size in units of 1/MAXSPART of the source's half-size vectors (the
 * coordinates of rt/srcsamp.c:178-210 skipparts), in the reference's order.
 * Sources the point is behind have none. */
#define MAXSPART 64
typedef struct { int ct[2], sz[2]; } spart;

static void flt_partit(const double ro[3], int mp, const double cent[3], const double u[3], const double v[3],
                       double du2, double dv2, int ct0, int ct1, int sz0, int sz1, spart *out, int *np)
{
    double d2 = 0, newax[3], newct[3], nu[3], nv[3];
    int i, axis;
    for (i = 0; i < 3; i++) d2 += (ro[i] - cent[i]) * (ro[i] - cent[i]);
    if (mp < 2 || (d2 >= du2 && d2 >= dv2)) {
        out[*np].ct[0] = ct0; out[*np].ct[1] = ct1;
        out[*np].sz[0] = sz0; out[*np].sz[1] = sz1;
        (*np)++;
        return;
    }
    memcpy(nu, u, sizeof nu);
    memcpy(nv, v, sizeof nv);
    axis = du2 > dv2 ? 0 : 1;
    if (axis == 0) {
        for (i = 0; i < 3; i++) newax[i] = nu[i] = .5 * u[i];
        du2 *= 0.25;
        sz0 >>= 1;
    } else {
        for (i = 0; i < 3; i++) newax[i] = nv[i] = .5 * v[i];
        dv2 *= 0.25;
        sz1 >>= 1;
    }
    for (i = 0; i < 3; i++) newct[i] = cent[i] - newax[i];
    flt_partit(ro, mp / 2, newct, nu, nv, du2, dv2, ct0 - (axis == 0 ? sz0 : 0), ct1 - (axis == 1 ? sz1 : 0),
               sz0, sz1, out, np);
    for (i = 0; i < 3; i++) newct[i] = cent[i] + newax[i];
    flt_partit(ro, mp / 2, newct, nu, nv, du2, dv2, ct0 + (axis == 0 ? sz0 : 0), ct1 + (axis == 1 ? sz1 : 0),
               sz0, sz1, out, np);
}

/* rt/srcsamp.c:187-221 cyl_partit: halves along the cylinder's axis */
static void cyl_partit(const double ro[3], int mp, const double cent[3], const double axis[3], double d2, int ct0,
                       int sz0, spart *out, int *np)
{
    double nc[3], na[3], v[3];
    int i;
    for (i = 0; i < 3; i++) v[i] = ro[i] - cent[i];
    if (mp < 2 || vdot(v, v) >= d2) {
        out[*np].ct[0] = ct0;
        out[*np].ct[1] = 0;
        out[*np].sz[0] = sz0;
        out[*np].sz[1] = MAXSPART;
        (*np)++;
        return;
    }
    for (i = 0; i < 3; i++) na[i] = .5 * axis[i];
    d2 *= 0.25;
    sz0 >>= 1;
    for (i = 0; i < 3; i++) nc[i] = cent[i] - na[i];
    cyl_partit(ro, mp / 2, nc, na, d2, ct0 - sz0, sz0, out, np);
    for (i = 0; i < 3; i++) nc[i] = cent[i] + na[i];
    cyl_partit(ro, mp / 2, nc, na, d2, ct0 + sz0, sz0, out, np);
}

static int source_parts(const ctx *X, const osrc *s, const RAY *r, spart *out)
{
    int np = 0;
    if (X->o->ds > FTINY && (s->flags & S_CYL)) {         /* rt/srcsamp.c:240-273 cylpart */
        double v[3] = {r->rop[0] - s->sloc[0], r->rop[1] - s->sloc[1], r->rop[2] - s->sloc[2]};
        double rad2 = 1.365 * vdot(s->ss[1], s->ss[1]), safe2 = vdot(s->ss[0], s->ss[0]);
        double d = vdot(v, s->ss[0]), cent2 = vdot(v, v), perp2 = cent2 - d * d / safe2;
        if (perp2 <= rad2) return 0;
        safe2 *= 4. * r->rweight * r->rweight / (X->o->ds * X->o->ds);
        if (perp2 <= 4. * rad2 || cent2 >= safe2) {
            out[0].ct[0] = out[0].ct[1] = 0;
            out[0].sz[0] = out[0].sz[1] = MAXSPART;
            return 1;
        }
        cyl_partit(r->rop, MAXSPART, s->sloc, s->ss[0], safe2, 0, MAXSPART, out, &np);
        return np;
    }
    if (X->o->ds <= FTINY || (s->flags & S_DISTANT) || !(s->flags & S_FLAT)) {   /* nopart */
        out[0].ct[0] = out[0].ct[1] = 0;
        out[0].sz[0] = out[0].sz[1] = MAXSPART;
        return 1;
    }
    {
        double v[3] = {r->rop[0] - s->sloc[0], r->rop[1] - s->sloc[1], r->rop[2] - s->sloc[2]};
        double dv2, du2;
        if (vdot(v, s->snorm) <= 0.) return 0;          /* behind the source */
        dv2 = 2. * r->rweight / X->o->ds;
        dv2 *= dv2;
        du2 = dv2 * vdot(s->ss[0], s->ss[0]);
        dv2 *= vdot(s->ss[1], s->ss[1]);
        flt_partit(r->rop, MAXSPART, s->sloc, s->ss[0], s->ss[1], du2, dv2, 0, 0, MAXSPART, MAXSPART, out, &np);
    }
    return np;
}

/* rt/source.c:398-556 with every partition's shadow tested (the reference's
 * -dt threshold, which estimates untested sources from run-wide hit
 * statistics, is taken as 0) */
static void direct(ctx *X, RAY *r, const NORMDAT *nd)
{
    const oscene *O = X->O;
    int sn;
    spart parts[MAXSPART];
    for (sn = 0; sn < O->nsrc; sn++) {
        const osrc *s = &O->src[sn];
        int np, pi;
        if (s->flags & S_SKIP) continue;
        if ((s->flags & (S_PROX | S_DISTANT)) == S_PROX) {
            double dv[3] = {r->rop[0] - s->sloc[0], r->rop[1] - s->sloc[1], r->rop[2] - s->sloc[2]};
            if (vdot(dv, dv) > (s->prox + s->srad) * (s->prox + s->srad)) continue;
        }
        np = source_parts(X, s, r, parts);
        for (pi = 0; pi < np; pi++) {
        double vpos[3] = {0, 0, 0}, dir[3], d, dom, coef[3], val[3];
        const uint32_t code = GB_C_SHADOWP(sn, pi);
        RAY sr;
        int i;
        if (X->o->dj > FTINY) {
            double u[4];
            draw(X, gb_child(r->path, code), r->sensor, GB_G_SRC, u, NULL);
            vpos[0] = X->o->dj * (1. - 2. * u[0]) * parts[pi].sz[0] * (1.0 / MAXSPART);
            vpos[1] = X->o->dj * (1. - 2. * u[1]) * parts[pi].sz[1] * (1.0 / MAXSPART);
            vpos[2] = (s->flags & S_FLAT) ? 0 : X->o->dj * (1. - 2. * u[2]);
        }
        vpos[0] += parts[pi].ct[0] * (1.0 / MAXSPART);
        vpos[1] += parts[pi].ct[1] * (1.0 / MAXSPART);
        if ((s->flags & S_CIR) && (np > 1 || X->o->dj > 0.7)) {   /* rt/srcsamp.c:85-109 */
            if (s->flags & (S_FLAT | S_DISTANT)) {
                double t0 = 1.12837917 * sqrt(1.0 - 0.5 * vpos[1] * vpos[1]);
                double t1 = 1.12837917 * sqrt(1.0 - 0.5 * vpos[0] * vpos[0]);
                vpos[0] *= t0;
                vpos[1] *= t1;
                vpos[2] = 0;
            } else {
                double a = vpos[0] * vpos[0], b = vpos[1] * vpos[1], c = vpos[2] * vpos[2];
                double sum = a + b + c, mx = fmax(a, fmax(b, c));
                double t = sum > FTINY * FTINY ? (1.0 / 0.7236) * sqrt(mx / sum) : 0.0;
                for (i = 0; i < 3; i++) vpos[i] *= t;
            }
        }
        for (i = 0; i < 3; i++)
            dir[i] = s->sloc[i] + vpos[0] * s->ss[0][i] + vpos[1] * s->ss[1][i] + vpos[2] * s->ss[2][i];
        if (!(s->flags & S_DISTANT))
            for (i = 0; i < 3; i++) dir[i] -= r->rop[i];
        if ((d = vnormalize(dir)) == 0.0) continue;
        if (s->flags & S_FLAT) dom = -vdot(s->snorm, dir);
        else if (s->flags & S_CYL) {                   /* rt/srcsamp.c:364-376 scylform */
            double d2 = vdot(dir, s->ss[0]);
            d2 *= d2 / vdot(s->ss[0], s->ss[0]);
            dom = sqrt(1. - d2);
        } else dom = 1.0;
        dom *= parts[pi].sz[0] * parts[pi].sz[1] * (1.0 / MAXSPART / MAXSPART);
        if (s->flags & S_DISTANT) {
            dom *= s->ss2;
            d = FHUGE;
        } else {
            if (dom <= 1e-4) continue;
            dom *= s->ss2 / (d * d);
            if ((s->flags & S_PROX) && d > s->prox) continue;
            if (s->flags & S_SPOT) {                    /* rt/source.c:246-252 */
                if (s->spsiz < 2.0 * PI * (1.0 + vdot(s->spaim, dir))) continue;
                dom *= d * d;
                d += s->spflen;
                dom /= d * d;
            }
        }
        dirnorm(X, coef, nd, r, dir, dom);
        if (maxc(coef) <= 0) continue;
        /* potential: srcvalue on the source alone */
        memset(&sr, 0, sizeof sr);
        rayorigin(X, &sr, GB_SHADOW, r, NULL, code);
        memcpy(sr.rdir, dir, sizeof dir);
        sr.rsrc = sn;
        rayclear(&sr);
        if (s->flags & S_DISTANT) {
            if (!sourcehit(X, &sr)) continue;
        } else if (!object_hit(O, s->so, &sr))
            continue;
        m_light(X, s->mat, &sr);
        for (i = 0; i < 3; i++) val[i] = sr.rcol[i] * coef[i];
        if (0.2126 * val[0] + 0.7152 * val[1] + 0.0722 * val[2] <= 0) continue;
        /* shadow test */
        {
            int thru = (r->rod > 0) ^ (vdot(r->ron, dir) > 0);
            rayorigin(X, &sr, thru ? GB_TSHADOW : GB_RSHADOW, r, NULL, code);
        }
        memcpy(sr.rcoef, coef, sizeof coef);
        memcpy(sr.rdir, dir, sizeof dir);
        sr.rsrc = sn;
        rayclear(&sr);
        if (localhit(X, &sr) && (sr.ro != s->so || X->follow)) {
            int m = O->mat[sr.ro];
            /* raycont */
            if (m < 0) raytrans(X, &sr);
            else {
                int t = O->H.objs[m].otype;
                if (gb_is_light(t)) m_light(X, m, &sr);
                else if (t == GT_GLASS) {
                    /* transmitted part of m_glass for shadow rays */
                    const double *fa = O->H.objs[m].farg;
                    double mc[3], rindex = O->H.objs[m].nfargs == 4 ? fa[3] : 1.52, pdot, cos2, r1e, r1m, sc[3];
                    RAY p;
                    int hastrans;
                    memcpy(mc, fa, sizeof mc);
                    hastrans = maxc(mc) > 1e-15;
                    if (hastrans) {
                        for (i = 0; i < 3; i++) if (mc[i] < 1e-15) mc[i] = 1e-15;
                        if (sr.rod < 0.0) flipsurface(&sr);
                        pdot = sr.rod;
                        cos2 = sqrt((1.0 - 1.0 / (rindex * rindex)) + pdot * pdot / (rindex * rindex));
                        for (i = 0; i < 3; i++) mc[i] = pow(mc[i], 1.0 / cos2);
                        r1e = (pdot - rindex * cos2) / (pdot + rindex * cos2);
                        r1e *= r1e;
                        r1m = (1.0 / pdot - rindex / cos2) / (1.0 / pdot + rindex / cos2);
                        r1m *= r1m;
                        for (i = 0; i < 3; i++)
                            sc[i] = .5 * (1.0 - r1e) * (1.0 - r1e) * mc[i] / (1.0 - r1e * r1e * mc[i] * mc[i]) +
                                    .5 * (1.0 - r1m) * (1.0 - r1m) * mc[i] / (1.0 - r1m * r1m * mc[i] * mc[i]);
                        if (rayorigin(X, &p, GB_TRANS, &sr, sc, GB_C_TRANS) == 0) {
                            memcpy(p.rdir, sr.rdir, sizeof p.rdir);
                            raytrace(X, &p);
                            for (i = 0; i < 3; i++) sr.rcol[i] += p.rcol[i] * p.rcoef[i];
                        }
                    }
                } else if (t == GT_TRANS)
                    m_normal(X, m, &sr);              /* its transmitted part (rt/normal.c:280-301) */
                /* opaque materials: shadow stays black (rt/normal.c:189) */
            }
            trace_contrib(X, &sr);
            if ((sr.rcol[0] + sr.rcol[1] + sr.rcol[2]) / 3.0 <= FTINY) continue;
            for (i = 0; i < 3; i++) val[i] = sr.rcol[i] * sr.rcoef[i];
        } else if (X->follow && (s->flags & S_DISTANT) && sr.ro < 0 && sourcehit(X, &sr)) {
            m_light(X, s->mat, &sr);
            trace_contrib(X, &sr);
        }
        for (i = 0; i < 3; i++) r->rcol[i] += val[i];
        }
    }
}

static void square2disk(double ds[2], double seedx, double seedy)
{
    double phi, rr, a = 2. * seedx - 1, b = 2. * seedy - 1;
    if (a > -b) {
        if (a > b) { rr = a; phi = (PI / 4.) * (b / a); }
        else { rr = b; phi = (PI / 4.) * (2. - (a / b)); }
    } else {
        if (a < b) { rr = -a; phi = (PI / 4.) * (4. + (b / a)); }
        else { rr = -b; phi = b != 0. ? (PI / 4.) * (6. - (a / b)) : 0.; }
    }
    ds[0] = rr * cos(phi);
    ds[1] = rr * sin(phi);
}

/* rt/ambient.c:229-300 (-aa 0) with rt/ambcomp.c:351-421 and :177-250 */
/* rt/ambcomp.c:256-346 getambdiffs + ambsupersamp on the first hemisphere
 * of an rtrace -I sensor (the only hemispheres the GPU path super-samples),
 * in the arithmetic of the GPU's k_ssamp_plan: v holds each stratum's
 * first value (coefficient applied); each stratum's extra samples are
 * traced as children GB_C_SSAMP(k, m) and averaged with it. */
#define PB(c) (0.265074126f * (float)(c)[0] + 0.670114631f * (float)(c)[1] + 0.064811243f * (float)(c)[2])
static void supersample_root(ctx *X, RAY *r, int n, const double acoef[3], const double ux[3], const double uy[3],
                             const double onrm[3], double (*v)[3], double acol[3])
{
    float *earr = (float *)calloc(2 * (size_t)n * n, sizeof(float)), *ep2 = earr + n * n, e2rem = 0.f;
    int *m = (int *)calloc((size_t)n * n, sizeof(int));
    float wt = 1.f, dd = 3.14159265358979323846f * 0.8f / ((float)X->o->ad * (float)X->o->lw + 1e-20f);
    const float normf = 1.f / (PB(acoef) + 1e-6f);
    int cnt, i, j, k, c;
    if (wt > dd) wt = dd;
    cnt = (int)((float)X->o->as * wt + .5f);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) {
            const float b = PB(v[i * n + j]);
            float b1, d2;
            k = i * n + j;
            if (i) {
                b1 = PB(v[k - n]);
                d2 = b - b1;
                d2 *= d2 * normf / (b + b1 + 1e-6f);
                ep2[k] += d2;
                ep2[k - n] += d2;
            }
            if (!j) continue;
            b1 = PB(v[k - 1]);
            d2 = b - b1;
            d2 *= d2 * normf / (b + b1 + 1e-6f);
            ep2[k] += d2;
            ep2[k - 1] += d2;
            if (!i) continue;
            b1 = PB(v[k - n - 1]);
            d2 = b - b1;
            d2 *= d2 * normf / (b + b1 + 1e-6f);
            ep2[k] += d2;
            ep2[k - n - 1] += d2;
        }
    ep2[0] *= 6.f / 3.f;
    ep2[n - 1] *= 6.f / 3.f;
    ep2[(n - 1) * n] *= 6.f / 3.f;
    ep2[(n - 1) * n + n - 1] *= 6.f / 3.f;
    for (i = 1; i < n - 1; i++) {
        ep2[i * n] *= 6.f / 5.f;
        ep2[i * n + n - 1] *= 6.f / 5.f;
    }
    for (j = 1; j < n - 1; j++) {
        ep2[j] *= 6.f / 5.f;
        ep2[(n - 1) * n + j] *= 6.f / 5.f;
    }
    for (i = 0; i < n - 1; i++)
        for (j = 0; j < n - 1; j++) {
            k = i * n + j;
            earr[k] += .5f * ep2[k] + .125f * (ep2[k + 1] + ep2[k + n]);
            earr[k + 1] += .125f * ep2[k];
            earr[k + n] += .125f * ep2[k];
        }
    for (k = n * n; k--;) e2rem += earr[k];
    for (k = 0; k < n * n && cnt > 0; k++) {
        double q[4];
        int nss, mm;
        if (e2rem <= 1e-6f) break;
        draw(X, r->path, r->sensor, GB_G_SSAMP + (uint32_t)(k >> 2), q, NULL);
        nss = (int)(earr[k] / e2rem * (float)cnt + (float)q[k & 3]);
        for (mm = 1; mm <= nss; mm++) {
            RAY ar;
            double u[4], zd;
            float fs[2];
            memset(&ar, 0, sizeof ar);
            if (rayorigin(X, &ar, GB_RAMBIENT, r, acoef, GB_C_SSAMP(k, mm)) < 0) break;
            ar.adepth = r->adepth + 1;
            draw(X, ar.path, ar.sensor, GB_G_CREATE, u, NULL);
            gb_square2disk(fs, ((float)(k % n) + (float)u[2]) / (float)n, ((float)(k / n) + (float)u[1]) / (float)n);
            zd = sqrt(fmax(0., 1. - (double)fs[0] * fs[0] - (double)fs[1] * fs[1]));
            for (c = 0; c < 3; c++) ar.rdir[c] = fs[0] * ux[c] + fs[1] * uy[c] + zd * onrm[c];
            vnormalize(ar.rdir);
            rayclear(&ar);
            raytrace(X, &ar);
            for (c = 0; c < 3; c++) v[k][c] += ar.rcol[c] * ar.rcoef[c];
            m[k]++;
            if (!--cnt) break;
        }
        e2rem -= earr[k];
    }
    acol[0] = acol[1] = acol[2] = 0;
    for (k = 0; k < n * n; k++)
        for (c = 0; c < 3; c++) acol[c] += v[k][c] / (1 + m[k]);
    free(earr);
    free(m);
}
#undef PB

static void multambient(ctx *X, double aval[3], RAY *r, const double nrm[3])
{
    double d, wt, acoef[3], onrm[3], ux[3], uy[3], acol[3] = {0, 0, 0};
    double (*sv)[3] = NULL;
    int n, i, j, k, ok = 0, ssroot = X->ssamp_root, back;
    X->ssamp_root = 0;
    if (X->o->ad <= 0 || r->adepth >= X->o->ab) goto dumbamb;
    d = maxc(aval);
    if (d <= FTINY) goto dumbamb;
    wt = r->rweight;
    d *= 0.8 * r->rweight / (X->o->ad * X->o->lw + 1e-20);
    if (wt > d) wt = d;
    n = (int)(sqrt(X->o->ad * wt) + 0.5);
    if (n < 1) n = 1;
    back = vdot(nrm, r->ron) < 0;                  /* rt/ambcomp.c:351-395 samp_hemi backside */
    for (k = 0; k < 3; k++) onrm[k] = back ? -r->ron[k] : r->ron[k];
    for (k = 0; k < 3; k++) acoef[k] = aval[k] / (n * n);
    rand_perp(X, r, GB_G_FRAME, onrm, ux);
    vcross(uy, onrm, ux);
    if (ssroot && X->o->as > 0 && X->o->aa <= FTINY && n * n > 49)
        sv = (double (*)[3])calloc((size_t)n * n, sizeof *sv);
    {
        gb_lot *L = (gb_lot *)malloc(sizeof(gb_lot));
        float (*rows)[2] = (float (*)[2])malloc(sizeof(float) * 4 * n);
        float (*prev)[2] = rows, (*cur)[2] = rows + n, (*tmp)[2];
        gb_lot_init(L, r->path, r->sensor, X->k0, X->k1);
        for (k = 0; k < 2 * n; k++) rows[k][0] = rows[k][1] = 2.f;
    for (i = n; i--;) {
        for (j = n; j--;) {
            RAY ar;
            double u[4], spt[2], zd;
            float fs[2];
            int kk = i * n + j;
            memset(&ar, 0, sizeof ar);
            if (rayorigin(X, &ar, back ? GB_TAMBIENT : GB_RAMBIENT, r, acoef, GB_C_STRATUM(kk)) < 0) continue;
            ar.adepth = r->adepth + 1;
            draw(X, ar.path, ar.sensor, GB_G_CREATE, u, NULL);
            gb_place_sample(L, n, i, j, (float)u[1], (float)u[2], i + 1 < n ? (const float (*)[2])prev : NULL,
                            (const float (*)[2])cur, fs);
            cur[j][0] = fs[0];
            cur[j][1] = fs[1];
            spt[0] = fs[0];
            spt[1] = fs[1];
            zd = sqrt(fmax(0., 1. - spt[0] * spt[0] - spt[1] * spt[1]));
            for (k = 0; k < 3; k++) ar.rdir[k] = spt[0] * ux[k] + spt[1] * uy[k] + zd * onrm[k];
            vnormalize(ar.rdir);
            rayclear(&ar);
            raytrace(X, &ar);
            for (k = 0; k < 3; k++) acol[k] += ar.rcol[k] * ar.rcoef[k];
            if (sv)
                for (k = 0; k < 3; k++) sv[kk][k] = ar.rcol[k] * ar.rcoef[k];
            ok++;
        }
        tmp = prev; prev = cur; cur = tmp;
        for (k = 0; k < n; k++) cur[k][0] = cur[k][1] = 2.f;
    }
        free(rows);
        free(L);
    }
    if (sv) {
        if (ok == n * n) {                       /* samp_hemi's super-sampling test (rt/ambcomp.c:403-409) */
            float wf = 1.f, df = 3.14159265358979323846f * 0.8f / ((float)X->o->ad * (float)X->o->lw + 1e-20f);
            if (wf > df) wf = df;
            if ((int)((float)X->o->as * wf + .5f) >= 4 * n)
                supersample_root(X, r, n, acoef, ux, uy, onrm, sv, acol);
        }
        free(sv);
    }
    if (ok) {
        memcpy(aval, acol, sizeof acol);
        return;
    }
dumbamb:
    for (k = 0; k < 3; k++) aval[k] *= X->o->av[k];
}

/* The gaussamp trial of rt/normal.c:398-420 (see gaussamp below): returns
 * the cosine of the sampled direction with the surface normal. */
static double spec_trial(const ctx *X, const RAY *r, const NORMDAT *np, const double u[3], const double v[3], int t,
                         double sdir[3])
{
    double q[4], rv0, rv1, d, cosp, sinp, h[3], s;
    int i;
    draw(X, r->path, r->sensor, GB_G_SPEC + (uint32_t)(t >> 1), q, NULL);
    rv0 = q[(t & 1) * 2];
    rv1 = q[(t & 1) * 2 + 1];
    d = 2.0 * PI * rv0;
    cosp = cos(d);
    sinp = sin(d);
    if ((0. <= X->o->ss) & (X->o->ss < 1.)) rv1 = 1.0 - X->o->ss * rv1;
    d = rv1 <= FTINY ? 1.0 : sqrt(np->alpha2 * -log(rv1));
    for (i = 0; i < 3; i++) h[i] = np->pnorm[i] + d * (cosp * u[i] + sinp * v[i]);
    s = -2.0 * vdot(h, r->rdir) / (1.0 + d * d);
    for (i = 0; i < 3; i++) sdir[i] = r->rdir[i] + s * h[i];
    vnormalize(sdir);
    return vdot(sdir, r->ron);
}

/* rt/normal.c:364-440 gaussamp, reflected part (opaque materials): one
 * sample of the rough specular lobe, or with -ss above 1.5 ss times the ray
 * weight of them with the W-G-M-D weighting.  Trials draw from the hit
 * ray's GB_G_SPEC groups instead of urand/frandom; sample k traces as child
 * GB_C_SPEC(k), all samples sharing the first one's rayorigin. */
#define MAXITER 10
static void gaussamp_trans(ctx *X, NORMDAT *np, RAY *r, const double u[3], const double v[3]);

static void gaussamp(ctx *X, NORMDAT *np, RAY *r)
{
    RAY sr;
    double u[3], v[3], scol[3] = {0, 0, 0}, d;
    int nstarget, nstaken, ntrials, maxiter, i;
    if ((!np->refl || np->rblt) && (!np->tran || np->tblt)) return;
    rand_perp(X, r, GB_G_SPECF, np->pnorm, u);
    vcross(v, np->pnorm, u);
    if (np->tran && !np->tblt) gaussamp_trans(X, np, r, u, v);
    if (!np->refl || np->rblt) return;
    if (rayorigin(X, &sr, GB_RSPECULAR, r, np->scolor, GB_C_SPEC(0)) != 0) return;
    nstarget = 1;
    if (X->o->ss > 1.5) {
        nstarget = (int)(X->o->ss * r->rweight + .5);
        if (sr.rweight <= X->o->lw * nstarget) nstarget = (int)(sr.rweight / X->o->lw);
        if (nstarget > 1) {
            d = 1. / nstarget;
            for (i = 0; i < 3; i++) sr.rcoef[i] *= d;
            sr.rweight *= d;
        } else
            nstarget = 1;
    }
    maxiter = MAXITER * nstarget;
    for (nstaken = ntrials = 0; nstaken < nstarget && ntrials < maxiter; ntrials++) {
        double sdir[3];
        d = spec_trial(X, r, np, u, v, ntrials, sdir);
        if (d <= FTINY) continue;
        if (nstaken) {
            rayclear(&sr);
            sr.path = gb_child(r->path, GB_C_SPEC(nstaken));
        }
        memcpy(sr.rdir, sdir, sizeof sr.rdir);
        raytrace(X, &sr);
        if (nstarget > 1) {
            d = 2. / (1. + r->rod / d);
            for (i = 0; i < 3; i++) scol[i] += sr.rcol[i] * d;
        } else
            for (i = 0; i < 3; i++) r->rcol[i] += sr.rcol[i] * sr.rcoef[i];
        ++nstaken;
    }
    if (nstarget > 1) {
        d = (double)nstarget / ntrials;
        for (i = 0; i < 3; i++) r->rcol[i] += scol[i] * sr.rcoef[i] * d;
    }
}

/* rt/normal.c:441-495, the transmitted part of gaussamp: samples about
 * the transmitted direction, rejected at or above the surface, no W-G-M-D
 * weighting; trials from GB_G_TSPEC, sample k traces as GB_C_TSPEC(k) */
static void gaussamp_trans(ctx *X, NORMDAT *np, RAY *r, const double u[3], const double v[3])
{
    RAY sr;
    double tc[3], q[4], rv0, rv1, d, cosp, sinp;
    int nstarget = 1, nstaken, ntrials, maxiter, i, t;
    for (i = 0; i < 3; i++) tc[i] = np->mcolor[i] * np->tspec;
    if (rayorigin(X, &sr, GB_TSPECULAR, r, tc, GB_C_TSPEC(0)) != 0) return;
    if (X->o->ss > 1.5) {
        nstarget = (int)(X->o->ss * r->rweight + .5);
        if (sr.rweight <= X->o->lw * nstarget) nstarget = (int)(sr.rweight / X->o->lw);
        if (nstarget > 1) {
            d = 1. / nstarget;
            for (i = 0; i < 3; i++) sr.rcoef[i] *= d;
            sr.rweight *= d;
        } else
            nstarget = 1;
    }
    maxiter = GB_SPEC_MAXITER * nstarget;
    for (nstaken = ntrials = 0; nstaken < nstarget && ntrials < maxiter; ntrials++) {
        t = ntrials;
        draw(X, r->path, r->sensor, GB_G_TSPEC + (uint32_t)(t >> 1), q, NULL);
        rv0 = q[(t & 1) * 2];
        rv1 = q[(t & 1) * 2 + 1];
        d = 2.0 * PI * rv0;
        cosp = cos(d);
        sinp = sin(d);
        if ((0. <= X->o->ss) & (X->o->ss < 1.)) rv1 = 1.0 - X->o->ss * rv1;
        d = rv1 <= FTINY ? 1.0 : sqrt(np->alpha2 * -log(rv1));
        for (i = 0; i < 3; i++) sr.rdir[i] = np->prdir[i] + d * (cosp * u[i] + sinp * v[i]);
        if (vdot(sr.rdir, r->ron) >= -FTINY) continue;
        vnormalize(sr.rdir);
        if (nstaken) {
            double keep[3];
            memcpy(keep, sr.rdir, sizeof keep);
            rayclear(&sr);
            sr.path = gb_child(r->path, GB_C_TSPEC(nstaken));
            memcpy(sr.rdir, keep, sizeof keep);
        }
        raytrace(X, &sr);
        for (i = 0; i < 3; i++) r->rcol[i] += sr.rcol[i] * sr.rcoef[i];
        ++nstaken;
    }
}

static int m_normal_obj(ctx *X, const gb_object *mo, RAY *r);

static int m_normal(ctx *X, int m, RAY *r)
{
    return m_normal_obj(X, &X->O->H.objs[m], r);
}

/* the Lambertian of reflectance pi that -i substitutes (rt/raytrace.c:24-28
 * Lamb) */
static double lamb_farg[5] = {PI, PI, PI, 0., 0.};
static const gb_object lamb_obj = {GT_PLASTIC, -1, (char *)"Lambertian", 0, NULL, 5, lamb_farg};

static int m_normal_obj(ctx *X, const gb_object *mo, RAY *r)
{
    NORMDAT nd;
    double fest = 0, sct[3];
    int i, istrans = mo->otype == GT_TRANS;
    if ((r->crtype & GB_SHADOW) && !istrans) return 1;      /* trans: shadows pass the transmitted part */
    if (r->rod < 0.0) flipsurface(r);
    memcpy(nd.mcolor, mo->farg, sizeof nd.mcolor);
    nd.alpha2 = mo->farg[4] * mo->farg[4];
    nd.pure = nd.alpha2 <= FTINY;
    memcpy(nd.pnorm, r->ron, sizeof nd.pnorm);
    nd.pdot = r->rod < .001 ? .001 : r->rod;
    nd.flat = r->ro >= 0 && (X->O->H.objs[r->ro].otype == GT_POLYGON || X->O->H.objs[r->ro].otype == GT_RING);
    nd.rspec = mo->farg[3];
    if (nd.pure && nd.rspec >= FRESTHRESH) {
        fest = FRESNE(nd.pdot);
        nd.rspec += fest * (1. - nd.rspec);
    }
    if (istrans) {                                  /* rt/normal.c:259-277 */
        nd.trans = mo->farg[5] * (1.0 - nd.rspec);
        nd.tspec = nd.trans * mo->farg[6];
        nd.tdiff = nd.trans - nd.tspec;
        nd.tran = nd.tspec > FTINY;
        nd.tblt = nd.tran && !nd.pure && X->o->st >= nd.tspec - FTINY;
        memcpy(nd.prdir, r->rdir, sizeof nd.prdir);
    } else {
        nd.trans = nd.tspec = nd.tdiff = 0;
        nd.tran = nd.tblt = 0;
    }
    nd.rdiff = 1.0 - nd.trans - nd.rspec;
    if (nd.tran && nd.pure) {                       /* the transmitted ray */
        RAY lr;
        double tc[3];
        for (i = 0; i < 3; i++) tc[i] = nd.mcolor[i] * nd.tspec;
        if (rayorigin(X, &lr, GB_TRANS, r, tc, GB_C_TRANS) == 0) {
            memcpy(lr.rdir, nd.prdir, sizeof lr.rdir);
            rayclear(&lr);
            raytrace(X, &lr);
            for (i = 0; i < 3; i++) r->rcol[i] += lr.rcol[i] * lr.rcoef[i];
        }
    }
    if (r->crtype & GB_SHADOW) return 1;
    nd.refl = nd.rspec > FTINY;
    nd.rblt = 0;
    nd.scolor[0] = nd.scolor[1] = nd.scolor[2] = 0;
    if (nd.refl) {
        if (mo->otype != GT_METAL) nd.scolor[0] = nd.scolor[1] = nd.scolor[2] = nd.rspec;
        else if (fest > FTINY) {
            double d = mo->farg[3] * (1. - fest);
            for (i = 0; i < 3; i++) nd.scolor[i] = fest + nd.mcolor[i] * d;
        } else
            for (i = 0; i < 3; i++) nd.scolor[i] = nd.mcolor[i] * nd.rspec;
        if (!nd.pure && X->o->st >= nd.rspec - FTINY) nd.rblt = 1;
    }
    if (nd.refl && nd.pure) {
        RAY lr;
        if (rayorigin(X, &lr, GB_REFLECTED, r, nd.scolor, GB_C_REFL) == 0) {
            for (i = 0; i < 3; i++) lr.rdir[i] = r->rdir[i] + 2. * nd.pdot * nd.pnorm[i];
            vnormalize(lr.rdir);
            rayclear(&lr);
            raytrace(X, &lr);
            for (i = 0; i < 3; i++) r->rcol[i] += lr.rcol[i] * lr.rcoef[i];
        }
    }
    if (nd.pure && nd.rdiff <= FTINY && nd.tdiff <= FTINY) return 1;
    if (!nd.pure) gaussamp(X, &nd, r);
    if (nd.rdiff > FTINY) {
        for (i = 0; i < 3; i++) sct[i] = nd.mcolor[i] * nd.rdiff + (nd.rblt ? nd.scolor[i] : 0);
        multambient(X, sct, r, nd.pnorm);
        for (i = 0; i < 3; i++) r->rcol[i] += sct[i];
    }
    if (nd.tdiff > FTINY) {                         /* ambient from the other side */
        double bnorm[3] = {-nd.pnorm[0], -nd.pnorm[1], -nd.pnorm[2]};
        uint64_t path = r->path;
        for (i = 0; i < 3; i++) sct[i] = nd.mcolor[i] * (nd.tblt ? nd.trans : nd.tdiff);
        r->path = gb_child(path, GB_C_BACK);        /* its draws keyed apart from the front's */
        multambient(X, sct, r, bnorm);
        r->path = path;
        for (i = 0; i < 3; i++) r->rcol[i] += sct[i];
    }
    direct(X, r, &nd);
    return 1;
}

static int m_glass(ctx *X, int m, RAY *r)
{
    const gb_object *mo = &X->O->H.objs[m];
    double mc[3], rindex = mo->nfargs == 4 ? mo->farg[3] : 1.52, pdot, cos2, r1e, r1m, sc[3];
    int i, hastrans;
    RAY p;
    memcpy(mc, mo->farg, sizeof mc);
    if ((hastrans = maxc(mc) > 1e-15)) {
        for (i = 0; i < 3; i++) if (mc[i] < 1e-15) mc[i] = 1e-15;
    } else if (r->crtype & GB_SHADOW)
        return 1;
    if (r->rod < 0.0) flipsurface(r);
    pdot = r->rod;
    cos2 = sqrt((1.0 - 1.0 / (rindex * rindex)) + pdot * pdot / (rindex * rindex));
    if (hastrans)
        for (i = 0; i < 3; i++) mc[i] = pow(mc[i], 1.0 / cos2);
    r1e = (pdot - rindex * cos2) / (pdot + rindex * cos2);
    r1e *= r1e;
    r1m = (1.0 / pdot - rindex / cos2) / (1.0 / pdot + rindex / cos2);
    r1m *= r1m;
    if (hastrans) {
        for (i = 0; i < 3; i++)
            sc[i] = .5 * (1.0 - r1e) * (1.0 - r1e) * mc[i] / (1.0 - r1e * r1e * mc[i] * mc[i]) +
                    .5 * (1.0 - r1m) * (1.0 - r1m) * mc[i] / (1.0 - r1m * r1m * mc[i] * mc[i]);
        if (rayorigin(X, &p, GB_TRANS, r, sc, GB_C_TRANS) == 0) {
            memcpy(p.rdir, r->rdir, sizeof p.rdir);
            rayclear(&p);
            raytrace(X, &p);
            for (i = 0; i < 3; i++) r->rcol[i] += p.rcol[i] * p.rcoef[i];
        }
    }
    if (r->crtype & GB_SHADOW) return 1;
    for (i = 0; i < 3; i++) {
        double d = mc[i] * mc[i];
        sc[i] = .5 * r1e * (1.0 + (1.0 - 2.0 * r1e) * d) / (1.0 - r1e * r1e * d) +
                .5 * r1m * (1.0 + (1.0 - 2.0 * r1m) * d) / (1.0 - r1m * r1m * d);
    }
    if (rayorigin(X, &p, GB_REFLECTED, r, sc, GB_C_REFL) == 0) {
        for (i = 0; i < 3; i++) p.rdir[i] = r->rdir[i] + 2. * pdot * r->ron[i];
        vnormalize(p.rdir);
        rayclear(&p);
        raytrace(X, &p);
        for (i = 0; i < 3; i++) r->rcol[i] += p.rcol[i] * p.rcoef[i];
    }
    return 1;
}

/* rt/m_mirror.c m_mirror (no substitute material, no virtual sources):
 * shadow rays stop, the back is black, else the reflected ray */
static int m_mirror(ctx *X, int m, RAY *r)
{
    const gb_object *mo = &X->O->H.objs[m];
    RAY nr;
    int i;
    if (r->rsrc >= 0 && X->O->src[r->rsrc].so != r->ro) return 1;
    if (r->rod < 0.) return 1;
    if (rayorigin(X, &nr, GB_REFLECTED, r, mo->farg, GB_C_REFL) < 0) return 1;
    for (i = 0; i < 3; i++) nr.rdir[i] = r->rdir[i] + 2. * r->rod * r->ron[i];
    vnormalize(nr.rdir);
    rayclear(&nr);
    raytrace(X, &nr);
    for (i = 0; i < 3; i++) r->rcol[i] += nr.rcol[i] * nr.rcoef[i];
    return 1;
}

/* rayshade with the material found for object r->ro */
static void rayshade(ctx *X, RAY *r)
{
    int m = X->O->mat[r->ro];
    int t;
    if (m < 0) { raytrans(X, r); return; }
    t = X->O->H.objs[m].otype;
    /* -i: rt/raytrace.c:211-236 raytirrad for primary rays and those
     * passed on through transparent surfaces */
    if (X->o->i && !(r->crtype & ~(GB_PRIMARY | GB_TRANS))) {
        if (gb_is_transp(t)) { raytrans(X, r); return; }
        if (!gb_is_light(t)) { m_normal_obj(X, &lamb_obj, r); return; }
    }
    if (gb_is_light(t)) m_light(X, m, r);
    else if (t == GT_GLASS) m_glass(X, m, r);
    else if (t == GT_PLASTIC || t == GT_METAL || t == GT_TRANS) m_normal(X, m, r);
    else if (t == GT_MIRROR) m_mirror(X, m, r);
    else raytrans(X, r);
}

static void raytrace(ctx *X, RAY *r)
{
    if (localhit(X, r))
        rayshade(X, r);
    else if (sourcehit(X, r)) {
        int m = X->O->mat[r->ro];
        if (m >= 0) m_light(X, m, r);
    }
    trace_contrib(X, r);
}

/* ---------------------------------------------------------------- entries */

static void setup_ctx(ctx *X, const oscene *O, const gb_opts *o, int follow)
{
    memset(X, 0, sizeof *X);
    X->O = O;
    X->o = o;
    X->follow = follow;
    X->k0 = (uint32_t)o->seed;
    X->k1 = (uint32_t)(o->seed >> 32);
}

/* The -I sensor evaluation (rt/rtrace.c:436-449 + rayirrad :416-433, or
 * rt/rcontrib.c:321-338): Lambertian rho = pi at org + 1e-4 dir. */
static void eval_irrad(ctx *X, const double *rv, uint32_t sensor, double rgb[3])
{
    RAY r;
    NORMDAT nd;
    double dir[3] = {rv[3], rv[4], rv[5]}, sct[3];
    int i;
    memset(&r, 0, sizeof r);
    vnormalize(dir);
    for (i = 0; i < 3; i++) {
        r.rorg[i] = rv[i] + 1.1e-4 * dir[i];
        r.rdir[i] = -dir[i];
    }
    r.path = GB_ROOT_PATH(X->o->replica);
    r.sensor = sensor;
    rayorigin(X, &r, GB_PRIMARY, NULL, NULL, 0);
    r.origin = -1;
    r.rot = 1e-5;
    r.rod = 1.0;
    memcpy(r.ron, dir, sizeof dir);
    for (i = 0; i < 3; i++) r.rop[i] = rv[i] + 1e-4 * dir[i];
    /* m_normal(Lamb) */
    nd.mcolor[0] = nd.mcolor[1] = nd.mcolor[2] = PI;
    nd.scolor[0] = nd.scolor[1] = nd.scolor[2] = 0;
    memcpy(nd.pnorm, dir, sizeof dir);
    nd.rdiff = 1.0;
    nd.rspec = 0;
    nd.alpha2 = 0;
    nd.pdot = 1;
    nd.pure = 1;
    nd.refl = 0;
    nd.rblt = 0;
    nd.flat = 0;
    nd.trans = nd.tspec = nd.tdiff = 0;
    nd.tran = nd.tblt = 0;
    memcpy(nd.prdir, r.rdir, sizeof nd.prdir);
    sct[0] = sct[1] = sct[2] = PI;
    X->ssamp_root = X->o->prog == GB_PROG_RTRACE;
    multambient(X, sct, &r, nd.pnorm);
    X->ssamp_root = 0;
    for (i = 0; i < 3; i++) r.rcol[i] += sct[i];
    direct(X, &r, &nd);
    memcpy(rgb, r.rcol, 3 * sizeof(double));
}

static void eval_rad(ctx *X, const double *rv, uint32_t sensor, double rgb[3])
{
    RAY r;
    memset(&r, 0, sizeof r);
    memcpy(r.rorg, rv, 3 * sizeof(double));
    memcpy(r.rdir, rv + 3, 3 * sizeof(double));
    vnormalize(r.rdir);
    r.path = GB_ROOT_PATH(X->o->replica);
    r.sensor = sensor;
    rayorigin(X, &r, GB_PRIMARY, NULL, NULL, 0);
    r.origin = -1;
    raytrace(X, &r);
    memcpy(rgb, r.rcol, 3 * sizeof(double));
}

static __thread char orc_err[512];
const char *orc_last_error(void) { return orc_err; }

void *orc_scene_open(const char *path, int is_rad)
{
    return scene_open(path, is_rad, orc_err, sizeof orc_err);
}
void orc_scene_close(void *s) { scene_close((oscene *)s); }
int64_t orc_scene_nobjects(void *s) { return ((oscene *)s)->H.nobjs; }
const char *orc_scene_object_name(void *s, int64_t i) { return ((oscene *)s)->H.objs[i].name; }

/* rtrace: values (n x 3) of the input rays; hit ids of the forward cast.
 * nthreads > 1 splits the rays across OpenMP threads. */
int orc_rtrace(void *sp, const gb_opts *o, const double *rays, int64_t n, double *rgb, int32_t *hit,
               double *hit_t, int nthreads, int64_t *nrays)
{
    const oscene *O = (const oscene *)sp;
    int64_t total = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : total)
    {
        ctx X;
        int64_t i;
        setup_ctx(&X, O, o, 0);
#pragma omp for schedule(dynamic, 16)
        for (i = 0; i < n; i++) {
            const double *rv = rays + 6 * i;
            if (hit) {
                RAY c;
                memset(&c, 0, sizeof c);
                memcpy(c.rorg, rv, 3 * sizeof(double));
                memcpy(c.rdir, rv + 3, 3 * sizeof(double));
                normalize_ref(c.rdir);
                rayclear(&c);
                c.rsrc = -1;
                if (!localhit(&X, &c))
                    sourcehit(&X, &c);
                hit[i] = c.ro;
                if (hit_t) hit_t[i] = c.rot;
            }
            if (rgb) {
                if (o->I) eval_irrad(&X, rv, (uint32_t)i, rgb + 3 * i);
                else eval_rad(&X, rv, (uint32_t)i, rgb + 3 * i);
            }
        }
        total += X.rays;
    }
    if (nrays) *nrays = total;
    return 0;
}

/* rcontrib: out (n / accum) x nbins_total x 3 */
int orc_rcontrib(void *sp, const gb_opts *o, const gb_modspec *mods, int nmods, const double *rays, int64_t n,
                 double *out, int nthreads, int64_t *nrays)
{
    const oscene *O = (const oscene *)sp;
    gb_binins *prog = (gb_binins *)malloc(sizeof(gb_binins) * 4096);   /* shared by all threads */
    int info[3 * 256], nbt = 0, m;
    int32_t i;
    int64_t total = 0, rec, nrec;
    int *trk;
    gb_opts oo = *o;
    int accum = o->c > 0 ? o->c : 1;
    oo.dt = 0; oo.as = 0; oo.aa = 0;
    if (nmods > 256 || orc_compile_bins(mods, nmods, prog, 4096, info, &nbt, orc_err, sizeof orc_err) < 0) {
        if (nmods > 256) snprintf(orc_err, sizeof orc_err, "too many modifiers");
        free(prog);
        return -1;
    }
    trk = (int *)malloc(sizeof(int) * ((size_t)O->H.nobjs + 1));
    for (i = 0; i < O->H.nobjs; i++) {
        trk[i] = -1;
        if (O->H.objs[i].omod >= 0)
            for (m = 0; m < nmods; m++)
                if (!strcmp(O->H.objs[O->H.objs[i].omod].name, mods[m].modifier)) trk[i] = m;
    }
    nrec = n / accum;
    memset(out, 0, sizeof(double) * (size_t)nrec * nbt * 3);
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : total)
    {
        ctx X;
        setup_ctx(&X, O, &oo, 1);
        X.prog = prog;
        X.modinfo = info;
        X.trk = trk;
#pragma omp for schedule(dynamic, 1)
        for (rec = 0; rec < nrec; rec++) {
            int64_t k;
            X.bins = out + (size_t)rec * nbt * 3;
            for (k = 0; k < accum; k++) {
                double rgb[3];
                int64_t s = rec * accum + k;
                if (oo.I) eval_irrad(&X, rays + 6 * s, (uint32_t)s, rgb);
                else eval_rad(&X, rays + 6 * s, (uint32_t)s, rgb);
            }
            if (accum > 1)
                for (k = 0; k < nbt * 3; k++) X.bins[k] /= accum;
        }
        total += X.rays;
    }
    free(trk);
    free(prog);
    if (nrays) *nrays = total;
    return 0;
}

/* util/cmatrix.c:421-474: double accumulation, float result; zero rows and
 * columns skipped */
int orc_dctimestep(const float *dc, const float *sky, int64_t M, int64_t K, int64_t N, float *out, int nthreads)
{
    char *rowcheck = (char *)calloc((size_t)M, 1), *colcheck = (char *)calloc((size_t)N, 1);
    int64_t r, c, k;
    for (r = 0; r < M; r++)
        for (k = 0; k < K && !rowcheck[r]; k++)
            if (dc[3 * (r * K + k)] != 0 || dc[3 * (r * K + k) + 1] != 0 || dc[3 * (r * K + k) + 2] != 0) rowcheck[r] = 1;
    for (c = 0; c < N; c++)
        for (k = 0; k < K && !colcheck[c]; k++)
            if (sky[3 * (k * N + c)] != 0 || sky[3 * (k * N + c) + 1] != 0 || sky[3 * (k * N + c) + 2] != 0) colcheck[c] = 1;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static) private(c, k)
    for (r = 0; r < M; r++)
        for (c = 0; c < N; c++) {
            double res[3] = {0, 0, 0};
            float *dp = out + 3 * (r * N + c);
            if (rowcheck[r] && colcheck[c])
                for (k = 0; k < K; k++) {
                    const float *a = dc + 3 * (r * K + k), *b = sky + 3 * (k * N + c);
                    res[0] += (double)a[0] * b[0];
                    res[1] += (double)a[1] * b[1];
                    res[2] += (double)a[2] * b[2];
                }
            dp[0] = (float)res[0];
            dp[1] = (float)res[1];
            dp[2] = (float)res[2];
        }
    free(rowcheck);
    free(colcheck);
    return 0;
}

/* Digest of an octree for builder tests: node count, set count and an
 * FNV-1a hash over the pre-order tree with each leaf's sorted set. */
static void digest_tree(const gb_scene_host *H, int32_t code, uint64_t *h)
{
    int k;
#define MIX(v) (*h = (*h ^ (uint64_t)(uint32_t)(v)) * 1099511628211ull)
    if (code >= 0) {
        MIX(2);
        for (k = 0; k < 8; k++) digest_tree(H, H->kids[8 * code + k], h);
    } else if (code == -1) {
        MIX(0);
    } else {
        const int32_t *s = gb_scene_set(H, code);
        MIX(1);
        for (k = 0; k <= s[0]; k++) MIX(s[k]);
    }
#undef MIX
}

int orc_octree_digest(const char *path, int is_rad, int objlim, int resolu, uint64_t out[3])
{
    gb_scene_host H;
    uint64_t h = 1469598103934665603ull;
    int rc;
    gb_scene_init(&H);
    rc = is_rad ? (gb_scene_read_rad_file(&H, path) < 0 || gb_scene_build_octree(&H, objlim, resolu) < 0)
                : gb_scene_read_oct(&H, path) < 0;
    if (rc) {
        snprintf(orc_err, sizeof orc_err, "%s", gb_scene_error());
        gb_scene_clear(&H);
        return -1;
    }
    digest_tree(&H, H.root, &h);
    out[0] = (uint64_t)H.nnodes;
    out[1] = (uint64_t)H.nsets;
    out[2] = h;
    gb_scene_clear(&H);
    return 0;
}
