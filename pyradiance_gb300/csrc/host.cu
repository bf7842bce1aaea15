/*
 * host.cu -- the C ABI (include/gbrad.h): scene loading and upload, option
 * parsing, and the orchestration of the wavefront kernels of trace.cu.
 */
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <algorithm>
#include <atomic>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbrad.h"
#include "binexpr.h"
#include "dct.h"
#include "scene.h"
#include "tracehost.h"

#define GB_MAX_GENERATIONS 256    /* walk/shade rounds of one run (path length) */
#define GB_TIMED_LAUNCHES 256     /* launches timed with events in one run */

static thread_local std::string g_error;
static thread_local int64_t g_stats[4];

static int set_err(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return set_err(GB_ECUDA, "CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

extern "C" const char *gb_last_error(void) { return g_error.c_str(); }
extern "C" const char *gb_version(void) { return "gbrad 0.1 (sm_103a)"; }

extern "C" int gb_last_stats(int64_t *rays, int64_t *steps, int64_t *contribs, int64_t *launches)
{
    if (rays) *rays = g_stats[0];
    if (steps) *steps = g_stats[1];
    if (contribs) *contribs = g_stats[2];
    if (launches) *launches = g_stats[3];
    return GB_OK;
}

/* ------------------------------------------------------------------ scene */

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= n)
            return 0;
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess)
            return -1;
        n = bytes;
        return 0;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct gb_scene {
    gb_scene_host H;
    std::vector<int> matslot;          /* per object: material slot or -1 */
    std::vector<int> matobj;           /* per slot: material object index */
    std::vector<float4> mat;           /* 2 per slot */
    std::vector<int> unsupported;      /* material objects the shader lacks */
    std::vector<gb_dsrc> src;
    std::string src_error;             /* non-empty if a source is unsupported */
    std::vector<std::string> modname, matname;
    /* host arrays of the device scene */
    std::vector<int> hkids, hsetdata;
    std::vector<gb_dinst> hinst;
    std::vector<int4> hobj;
    std::vector<float4> hgeo;
    std::vector<float2> hfvert;
    std::vector<float4> hfv4, horec, hlrec, hvnrm;
    std::vector<int> hwkids, hvnidx;
    bool has_vnorm = false;        /* some mesh triangle has vertex normals */
    std::string vnorm_error;       /* a smooth mesh triangle on a material whose shading with them is not built */
    std::vector<int> hoslot;
    std::vector<float> hcone;
    std::vector<gb_dsrc> hsrc;
    std::vector<double> hg64;          /* FP64 geometry of the first-hit casts */
    std::vector<long long> hg64off;
    /* device scene */
    DevBuf kids, setdata, obj, geo, fvert, fv4, cone, matd, srcd, trk, instd, orec, oslot, g64, g64off, wkids, lrec,
        vnidx, vnrm;
    gb_dscene ds;
    /* work buffers */
    DevBuf sensors, value, bins, stats, roots, rootspt, qa, qb, qcount, binprog, modinfo, hits, hitt, hitpn, trkrun,
        hitrec, adja, adjb, dlde, gradd, rootdraw, rootlot, tga, tgb, ssval, sscnt, sserr, slow;
    cudaStream_t stream = nullptr;
    int sms = 0;
    int wroot = 0;                 /* the walk's root code (wkids, lrec) */
    void *pin = nullptr;           /* pinned host staging of the first-hit outputs */
    size_t pin_n = 0;
    void *pinb = nullptr;          /* pinned host staging of the bins */
    size_t pinb_n = 0;
    cudaEvent_t ev[2 * GB_TIMED_LAUNCHES + 2];
    int nev = 0;
    int octree_on_device = 0;          /* the octree was built by the device builder */
    /* walk kernel shape picked by the tuner (0: defaults), and whether runs
     * capture their generation loop in a CUDA graph (batched runs) */
    int tuned_refill = 0, tuned_blocks = 0;
    bool use_graph = false;
    std::string tuned_key;             /* options of the queue-size pilot */
    double tuned_per_sensor = 0.0;     /* its queue slots per sensor */
};

/* per-kernel profile of the last run on this thread */
struct KProf {
    double ms[GB_K_N];
    int64_t launches[GB_K_N];
    unsigned long long st[GB_K_N][GB_ST_N];
    double region_ms;
};
static thread_local KProf g_prof;

extern "C" int gb_last_profile(int kernel, double *ms, int64_t *launches, int64_t *counters, int ncounters,
                               double *region_ms)
{
    if (kernel < 0 || kernel >= GB_K_N)
        return set_err(GB_EINVAL, "bad kernel index");
    if (ms) *ms = g_prof.ms[kernel];
    if (launches) *launches = g_prof.launches[kernel];
    for (int i = 0; counters && i < ncounters && i < GB_ST_N; i++)
        counters[i] = (int64_t)g_prof.st[kernel][i];
    if (region_ms) *region_ms = g_prof.region_ms;
    return GB_OK;
}

static float __int_as_float_host(int v)
{
    float f;
    memcpy(&f, &v, sizeof f);
    return f;
}

static int material_kind(const gb_object *m, float4 *m0, float4 *m1, std::string &why)
{
    const double *f = m->farg;
    *m0 = make_float4(0, 0, 0, 0);
    *m1 = make_float4(0, 0, 0, 0);
    switch (m->otype) {
    case GT_PLASTIC:
    case GT_METAL:
        if (m->nfargs != 5) { why = "bad number of arguments"; return -1; }
        *m0 = make_float4(m->otype == GT_PLASTIC ? DM_PLASTIC : DM_METAL, f[0], f[1], f[2]);
        *m1 = make_float4(f[3], f[4], 0, 0);
        return 0;
    case GT_MIRROR:                              /* rt/m_mirror.c: 3 arguments, no substitute */
        if (m->nfargs != 3) { why = "bad number of arguments"; return -1; }
        if (m->nsargs > 0) { why = "mirror with a substitute material is not implemented on the GPU path"; return -1; }
        *m0 = make_float4(DM_MIRROR, f[0], f[1], f[2]);
        return 0;
    case GT_TRANS:                               /* rt/normal.c: 7 arguments */
        if (m->nfargs != 7) { why = "bad number of arguments"; return -1; }
        *m0 = make_float4(DM_TRANS, f[0], f[1], f[2]);
        *m1 = make_float4(f[3], f[4], f[5], f[6]);
        return 0;
    case GT_GLASS:
        if (m->nfargs != 3 && m->nfargs != 4) { why = "bad arguments"; return -1; }
        *m0 = make_float4(DM_GLASS, f[0], f[1], f[2]);
        *m1 = make_float4(m->nfargs == 4 ? f[3] : 1.52, 0, 0, 0);
        return 0;
    case GT_LIGHT:
        if (m->nfargs != 3) { why = "bad # arguments"; return -1; }
        *m0 = make_float4(DM_LIGHT, f[0], f[1], f[2]);
        return 0;
    case GT_SPOT: {                              /* a light with a cone (rt/srcsupp.c:268-288 makespot) */
        if (m->nfargs != 7) { why = "bad # arguments"; return -1; }
        if (f[3] <= GB_FTINY) { why = "zero angle"; return -1; }
        double l = sqrt(f[4] * f[4] + f[5] * f[5] + f[6] * f[6]);
        if (l == 0.0) { why = "zero focus vector"; return -1; }
        *m0 = make_float4(DM_LIGHT, f[0], f[1], f[2]);
        *m1 = make_float4((float)(2.0 * M_PI * (1.0 - cos(M_PI / 180.0 / 2.0 * f[3]))), (float)(f[4] / l),
                          (float)(f[5] / l), (float)(f[6] / l));
        return 0;
    }
    case GT_GLOW:
        if (m->nfargs != 4) { why = "bad # arguments"; return -1; }
        *m0 = make_float4(DM_GLOW, f[0], f[1], f[2]);
        *m1 = make_float4(f[3], 0, 0, 0);
        return 0;
    default:
        why = std::string("material type '") + gb_otype_name(m->otype) + "' is not implemented on the GPU path";
        return -1;
    }
}

/* getperpendicular without randomisation (common/fvect.c:159-196) */
static void perp(double vp[3], const double v[3])
{
    double v1[3] = {0, 0, 0};
    int i;
    for (i = 3; i--;)
        if (-0.6 < v[i] && v[i] < 0.6)
            break;
    if (i < 0) i = 0;
    v1[i] = 1.0;
    vp[0] = v1[1] * v[2] - v1[2] * v[1];
    vp[1] = v1[2] * v[0] - v1[0] * v[2];
    vp[2] = v1[0] * v[1] - v1[1] * v[0];
    double l = sqrt(vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2]);
    for (i = 0; i < 3; i++) vp[i] /= l;
}

static double dist2line(const double p[3], const double a[3], const double b[3])
{
    double d[3], v[3], l2 = 0, t = 0, r = 0;
    for (int i = 0; i < 3; i++) { d[i] = b[i] - a[i]; v[i] = p[i] - a[i]; l2 += d[i] * d[i]; t += d[i] * v[i]; }
    for (int i = 0; i < 3; i++) r += v[i] * v[i];
    return r - t * t / l2;
}

/* rt/source.c:47-142 (marksources) with rt/srcsupp.c:88-180 (fsetsrc,
 * ssetsrc) */
static int mark_sources(gb_scene *G)
{
    gb_scene_host &H = G->H;
    /* the scene's own objects only: the reference marks sources before any
     * instance loads its octree (rt/source.c:47-142) */
    for (int32_t i = 0; i < H.nobjs_top; i++) {
        const gb_object *o = &H.objs[i];
        if (!gb_is_surface(o->otype) || o->omod < 0)
            continue;
        int32_t m = gb_find_material(&H, i);
        if (m < 0)
            continue;
        const gb_object *mo = &H.objs[m];
        if (!gb_is_light(mo->otype))
            continue;
        int need = mo->otype == GT_GLOW ? 4 : mo->otype == GT_SPOT ? 7 : 3;
        if (mo->nfargs != need)
            return set_err(GB_EIO, "%s: bad # arguments", mo->name);
        if (mo->farg[0] <= GB_FTINY && mo->farg[1] <= GB_FTINY && mo->farg[2] <= GB_FTINY)
            continue;
        if (mo->otype == GT_GLOW && o->otype != GT_SOURCE && mo->farg[3] <= GB_FTINY)
            continue;                                /* indirect glow */
        gb_dsrc s;
        memset(&s, 0, sizeof s);
        s.so = i;
        s.mat = G->matslot[i];
        if (o->otype == GT_POLYGON) {
            const gb_face *f = &H.faces[i];
            const double *va = o->farg;
            double c[3] = {0, 0, 0}, su[3] = {0, 0, 0}, sv[3] = {0, 0, 0}, srad = 0;
            if (!f->ok)
                return set_err(GB_EIO, "%s: zero source area", o->name);
            for (int j = 0; j < 3; j++) {
                for (int k = 0; k < f->nv; k++) c[j] += va[3 * k + j];
                c[j] /= f->nv;
            }
            for (int k = 0; k < f->nv; k++) {
                double d = 0;
                for (int j = 0; j < 3; j++) d += (va[3 * k + j] - c[j]) * (va[3 * k + j] - c[j]);
                if (d > srad) srad = d;
            }
            if (f->nv == 4) {
                for (int j = 0; j < 3; j++) {
                    su[j] = .5 * (va[3 + j] - va[j]);
                    sv[j] = .5 * (va[9 + j] - va[j]);
                }
            } else if (f->nv == 3) {
                int near0 = 2;
                double dmin = dist2line(c, va + 6, va);
                for (int k = 0; k < 2; k++) {
                    double d2 = dist2line(c, va + 3 * k, va + 3 * (k + 1));
                    if (d2 >= dmin) continue;
                    near0 = k;
                    dmin = d2;
                }
                int k = (near0 + 1) % 3;
                double l = 0;
                for (int j = 0; j < 3; j++) { su[j] = va[3 * k + j] - va[3 * near0 + j]; l += su[j] * su[j]; }
                l = sqrt(dmin) / sqrt(l);
                for (int j = 0; j < 3; j++) su[j] *= l;
                sv[0] = f->norm[1] * su[2] - f->norm[2] * su[1];
                sv[1] = f->norm[2] * su[0] - f->norm[0] * su[2];
                sv[2] = f->norm[0] * su[1] - f->norm[1] * su[0];
            } else {
                perp(su, f->norm);
                double mult = .5 * sqrt(f->area);
                for (int j = 0; j < 3; j++) su[j] *= mult;
                sv[0] = f->norm[1] * su[2] - f->norm[2] * su[1];
                sv[1] = f->norm[2] * su[0] - f->norm[0] * su[2];
                sv[2] = f->norm[0] * su[1] - f->norm[1] * su[0];
            }
            s.flags = DS_FLAT;
            for (int j = 0; j < 3; j++) {
                s.sloc[j] = (float)c[j];
                s.snorm[j] = (float)f->norm[j];
                s.ss[0][j] = (float)su[j];
                s.ss[1][j] = (float)sv[j];
            }
            s.ss2 = (float)f->area;
            s.srad = (float)sqrt(srad);
        } else if (o->otype == GT_SOURCE) {
            double d[3] = {o->farg[0], o->farg[1], o->farg[2]};
            double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (l == 0.0)
                return set_err(GB_EIO, "%s: zero direction", o->name);
            for (int j = 0; j < 3; j++) d[j] /= l;
            double theta = M_PI / 180.0 / 2.0 * o->farg[3];
            if (theta <= GB_FTINY)
                return set_err(GB_EIO, "%s: zero size", o->name);
            double ss2 = 2.0 * M_PI * (1.0 - cos(theta));
            double su[3], sv[3];
            perp(su, d);
            double mult = .5 * sqrt(ss2);
            for (int j = 0; j < 3; j++) su[j] *= mult;
            sv[0] = d[1] * su[2] - d[2] * su[1];
            sv[1] = d[2] * su[0] - d[0] * su[2];
            sv[2] = d[0] * su[1] - d[1] * su[0];
            s.flags = DS_DISTANT | DS_CIR;
            for (int j = 0; j < 3; j++) {
                s.sloc[j] = (float)d[j];
                s.snorm[j] = (float)d[j];
                s.ss[0][j] = (float)su[j];
                s.ss[1][j] = (float)sv[j];
            }
            s.ss2 = (float)ss2;
            s.srad = (float)sqrt(ss2 / M_PI);
        } else if (o->otype == GT_SPHERE) {          /* rt/srcsupp.c:183-204 sphsetsrc */
            if (o->nfargs != 4)
                return set_err(GB_EIO, "%s: bad # arguments", o->name);
            if (o->farg[3] <= GB_FTINY)
                return set_err(GB_EIO, "%s: illegal source radius", o->name);
            s.flags = DS_CIR;
            for (int j = 0; j < 3; j++) {
                s.sloc[j] = (float)o->farg[j];
                s.ss[j][j] = (float)(0.7236 * o->farg[3]);
            }
            s.srad = (float)o->farg[3];
            s.ss2 = (float)(M_PI * o->farg[3] * o->farg[3]);
        } else if (o->otype == GT_CYLINDER) {        /* rt/srcsupp.c:234-264 cylsetsrc */
            const gb_cone *c = &H.cones[i];
            if (!c->ok)
                return set_err(GB_EIO, "%s: illegal source", o->name);
            const double r0 = o->farg[c->r0];
            if (r0 <= GB_FTINY)
                return set_err(GB_EIO, "%s: illegal source radius", o->name);
            double ad[3], al = 0, sw[3];
            for (int j = 0; j < 3; j++) {
                ad[j] = o->farg[c->p1 + j] - o->farg[c->p0 + j];
                al += ad[j] * ad[j];
            }
            al = sqrt(al);
            for (int j = 0; j < 3; j++) ad[j] /= al;
            perp(sw, ad);                            /* getperpendicular, without the random rotation */
            for (int j = 0; j < 3; j++) sw[j] *= .8559 * r0;
            s.flags = DS_CYL;
            for (int j = 0; j < 3; j++) {
                s.sloc[j] = (float)(.5 * (o->farg[c->p1 + j] + o->farg[c->p0 + j]));
                s.ss[0][j] = (float)(.5 * al * ad[j]);
                s.ss[2][j] = (float)sw[j];
            }
            s.ss[1][0] = (float)(sw[1] * ad[2] - sw[2] * ad[1]);   /* SW x axis */
            s.ss[1][1] = (float)(sw[2] * ad[0] - sw[0] * ad[2]);
            s.ss[1][2] = (float)(sw[0] * ad[1] - sw[1] * ad[0]);
            s.srad = (float)(.5 * al);
            s.ss2 = (float)(2. * r0 * al);
        } else if (o->otype == GT_RING) {            /* rt/srcsupp.c:207-231 rsetsrc */
            const gb_cone *c = &H.cones[i];
            if (!c->ok)
                return set_err(GB_EIO, "%s: illegal source", o->name);
            const double r0 = o->farg[c->r0], r1 = o->farg[c->r1];
            if (r1 <= GB_FTINY)
                return set_err(GB_EIO, "%s: illegal source radius", o->name);
            if (r0 > 0.0)
                return set_err(GB_EIO, "%s: cannot hit source center", o->name);
            double n[3] = {o->farg[3], o->farg[4], o->farg[5]};
            double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int j = 0; j < 3; j++) n[j] /= l;
            double su[3], sv[3], ss2 = M_PI * r1 * r1;
            perp(su, n);                             /* setflatss, without the random rotation */
            for (int j = 0; j < 3; j++) su[j] *= .5 * sqrt(ss2);
            sv[0] = n[1] * su[2] - n[2] * su[1];
            sv[1] = n[2] * su[0] - n[0] * su[2];
            sv[2] = n[0] * su[1] - n[1] * su[0];
            s.flags = DS_FLAT | DS_CIR;
            for (int j = 0; j < 3; j++) {
                s.sloc[j] = (float)o->farg[j];
                s.snorm[j] = (float)n[j];
                s.ss[0][j] = (float)su[j];
                s.ss[1][j] = (float)sv[j];
            }
            s.ss2 = (float)ss2;
            s.srad = (float)r1;
        } else {
            if (G->src_error.empty())
                G->src_error = std::string("light source geometry '") + gb_otype_name(o->otype) + "' (" +
                               o->name + ") is not implemented on the GPU path";
            continue;
        }
        if (mo->otype == GT_GLOW) {
            s.flags |= DS_PROX;
            s.prox = (float)mo->farg[3];
            if (s.flags & DS_DISTANT)
                s.flags |= DS_SKIP;
        } else if (mo->otype == GT_SPOT) {            /* rt/source.c:104-116 */
            if (s.flags & DS_DISTANT) {
                if (G->src_error.empty())
                    G->src_error = std::string("distant spotlight '") + o->name + "' is not implemented on the GPU path";
            } else {
                const double *f = mo->farg;
                double l = sqrt(f[4] * f[4] + f[5] * f[5] + f[6] * f[6]);
                s.flags |= DS_SPOT;
                s.spot[0] = (float)(2.0 * M_PI * (1.0 - cos(M_PI / 180.0 / 2.0 * f[3])));
                for (int j = 0; j < 3; j++) s.spot[1 + j] = (float)(f[4 + j] / l);
                s.spot[4] = (float)l;
                if (s.flags & DS_FLAT) {             /* checkspot (rt/srcsupp.c:452-465) */
                    double d = 0, d1 = 1. - s.spot[0] / (2. * M_PI);
                    for (int j = 0; j < 3; j++) d += (f[4 + j] / l) * s.snorm[j];
                    if (!(d > GB_FTINY) && !(1. - GB_FTINY - d * d < d1 * d1))
                        s.flags |= DS_SKIP;          /* invalid spotlight direction */
                }
            }
        } else if (mo->otype == GT_ILLUM) {
            if (G->src_error.empty())
                G->src_error = std::string("light material '") + gb_otype_name(mo->otype) + "' (" + mo->name +
                               ") is not implemented on the GPU path";
        }
        G->src.push_back(s);
    }
    return GB_OK;
}

template <typename T>
static int upload(DevBuf &b, const std::vector<T> &v)
{
    size_t bytes = v.size() * sizeof(T);
    if (b.ensure(bytes ? bytes : 16) < 0)
        return -1;
    if (bytes && cudaMemcpy(b.p, v.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        return -1;
    return 0;
}

static int build_arrays(gb_scene *G);

static int prepare_device(gb_scene *G)
{
    int rc = build_arrays(G);
    if (rc < 0)
        return rc;
    gb_scene_host &H = G->H;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&G->sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    /* the sequential hemisphere placement keeps a 4 KB lot per thread */
    size_t stack = 0;
    cudaDeviceGetLimit(&stack, cudaLimitStackSize);
    if (stack < 16384)
        CK(cudaDeviceSetLimit(cudaLimitStackSize, 16384));
    if (upload(G->kids, G->hkids) < 0 || upload(G->setdata, G->hsetdata) < 0 || upload(G->instd, G->hinst) < 0 ||
        upload(G->orec, G->horec) < 0 || upload(G->oslot, G->hoslot) < 0 ||
        upload(G->obj, G->hobj) < 0 || upload(G->geo, G->hgeo) < 0 || upload(G->fvert, G->hfvert) < 0 ||
        upload(G->fv4, G->hfv4) < 0 || upload(G->cone, G->hcone) < 0 || upload(G->matd, G->mat) < 0 ||
        upload(G->srcd, G->hsrc) < 0 || upload(G->g64, G->hg64) < 0 || upload(G->g64off, G->hg64off) < 0 ||
        upload(G->wkids, G->hwkids) < 0 || upload(G->lrec, G->hlrec) < 0 || upload(G->vnidx, G->hvnidx) < 0 ||
        upload(G->vnrm, G->hvnrm) < 0)
        return set_err(GB_ENOMEM, "device upload of the scene failed");
    gb_dscene &d = G->ds;
    d.kids = (const int *)G->kids.p;
    d.set_data = (const int *)G->setdata.p;
    d.wkids = (const int *)G->wkids.p;
    d.lrec = (const float4 *)G->lrec.p;
    d.vnidx = (const int *)G->vnidx.p;
    d.vnrm = (const float4 *)G->vnrm.p;
    d.obj = (const int4 *)G->obj.p;
    d.geo = (const float4 *)G->geo.p;
    d.fvert = (const float2 *)G->fvert.p;
    d.fv4 = (const float4 *)G->fv4.p;
    d.orec = (const float4 *)G->orec.p;
    d.oslot = (const int *)G->oslot.p;
    d.cone = (const float *)G->cone.p;
    d.mat = (const float4 *)G->matd.p;
    d.src = (const gb_dsrc *)G->srcd.p;
    d.inst = (const gb_dinst *)G->instd.p;
    d.g64 = (const double *)G->g64.p;
    d.g64off = (const long long *)G->g64off.p;
    (void)H;
    return GB_OK;
}

/* Host-side arrays of the device scene (and the gb_dscene header with
 * host pointers); no CUDA calls. */
static int build_arrays(gb_scene *G)
{
    gb_scene_host &H = G->H;
    if (gb_scene_prepare(&H) < 0)
        return set_err(GB_EIO, "%s", gb_scene_error());
    /* materials */
    G->matslot.assign(H.nobjs, -1);
    std::vector<int> slot_of_mat(H.nobjs, -1);
    for (int32_t i = 0; i < H.nobjs; i++) {
        if (!gb_is_surface(H.objs[i].otype))
            continue;
        int32_t m = gb_find_material(&H, i);
        if (m < 0)
            continue;
        if (slot_of_mat[m] < 0) {
            float4 a, b;
            std::string why;
            if (material_kind(&H.objs[m], &a, &b, why) < 0) {
                a = make_float4(-1.f, 0, 0, 0);
                G->unsupported.push_back(m);
            }
            slot_of_mat[m] = (int)G->matobj.size();
            G->matobj.push_back(m);
            G->mat.push_back(a);
            G->mat.push_back(b);
        }
        G->matslot[i] = slot_of_mat[m];
    }
    if (G->mat.empty()) {
        G->mat.push_back(make_float4(0, 0, 0, 0));
        G->mat.push_back(make_float4(0, 0, 0, 0));
    }
    /* objects */
    std::vector<int4> obj(H.nobjs);
    std::vector<float4> geo(H.nobjs);
    std::vector<float2> fvert;
    std::vector<float4> fv4(2 * (size_t)(H.nobjs > 0 ? H.nobjs : 1), make_float4(0, 0, 0, 0));
    std::vector<float> cone;
    for (int32_t i = 0; i < H.nobjs; i++) {
        const gb_object *o = &H.objs[i];
        int kind = DK_NONE, flags = 0, nv = 0, aux = 0;
        int32_t m = gb_is_surface(o->otype) ? gb_find_material(&H, i) : -1;
        if (m >= 0) {
            flags |= DF_HASMAT;
            if (gb_is_transp(H.objs[m].otype))
                flags |= DF_TRANSP;
        }
        geo[i] = make_float4(0, 0, 0, 0);
        switch (o->otype) {
        case GT_POLYGON: {
            const gb_face *f = &H.faces[i];
            if (!f->ok)
                break;
            kind = DK_FACE;
            nv = f->nv;
            flags |= f->ax << DF_AXSHIFT;
            if (o->vnorm && nv == 3)
                flags |= DF_VNORM;
            if (o->vuv && nv == 3)
                flags |= DF_VUV;
            geo[i] = make_float4((float)f->norm[0], (float)f->norm[1], (float)f->norm[2], (float)f->offset);
            aux = (int)fvert.size();
            int xi = (f->ax + 1) % 3, yi = (xi + 1) % 3;
            for (int k = 0; k < nv; k++)
                fvert.push_back(make_float2((float)o->farg[3 * k + xi], (float)o->farg[3 * k + yi]));
            if (nv <= 4) {
                float v[8] = {0};
                for (int k = 0; k < nv; k++) {
                    v[2 * k] = fvert[aux + k].x;
                    v[2 * k + 1] = fvert[aux + k].y;
                }
                fv4[2 * i] = make_float4(v[0], v[1], v[2], v[3]);
                fv4[2 * i + 1] = make_float4(v[4], v[5], v[6], v[7]);
            }
            break;
        }
        case GT_SPHERE:
        case GT_BUBBLE:
            kind = o->otype == GT_SPHERE ? DK_SPHERE : DK_BUBBLE;
            geo[i] = make_float4((float)o->farg[0], (float)o->farg[1], (float)o->farg[2], (float)o->farg[3]);
            break;
        case GT_CONE: case GT_CUP: case GT_CYLINDER: case GT_TUBE: case GT_RING: {
            const gb_cone *c = &H.cones[i];
            if (!c->ok)
                break;
            kind = o->otype == GT_CONE ? DK_CONE : o->otype == GT_CUP ? DK_CUP :
                   o->otype == GT_CYLINDER ? DK_CYL : o->otype == GT_TUBE ? DK_TUBE : DK_RING;
            aux = (int)(cone.size() / 24);
            const double *ca = o->farg;
            double ad[3];
            if (o->otype == GT_RING) {
                for (int j = 0; j < 3; j++) ad[j] = ca[3 + j];
            } else {
                for (int j = 0; j < 3; j++) ad[j] = ca[c->p1 + j] - ca[c->p0 + j];
            }
            double l = sqrt(ad[0] * ad[0] + ad[1] * ad[1] + ad[2] * ad[2]);
            for (int j = 0; j < 3; j++) ad[j] /= l;
            float rec[24] = {0};
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 3; b++)
                    rec[3 * a + b] = (float)c->tm[a][b];
            for (int j = 0; j < 3; j++) {
                rec[12 + j] = (float)ad[j];
                rec[15 + j] = (float)ca[c->p0 + j];
            }
            rec[18] = (float)c->al;
            rec[19] = (float)c->sl;
            rec[20] = (float)ca[c->r0];
            rec[21] = (float)ca[c->r1];
            cone.insert(cone.end(), rec, rec + 24);
            break;
        }
        case GT_SOURCE:
            kind = DK_SOURCE;
            break;
        case GT_INSTANCE:
        case GT_MESH:                                  /* an instance of its triangles (scene.c) */
            for (int k = 0; k < H.ninst; k++)
                if (H.inst[k].obj == i) {
                    kind = DK_INSTANCE;
                    aux = k;
                }
            break;
        default:
            break;
        }
        if (nv > 0xffff)
            return set_err(GB_EUNSUPPORTED, "%s: polygon with more than 65535 vertices", o->name);
        obj[i] = make_int4(kind | (flags << 8) | (nv << 16), G->matslot[i], o->omod, aux);
    }
    if (fvert.empty()) fvert.push_back(make_float2(0, 0));
    if (cone.empty()) cone.assign(24, 0.f);
    int rc = mark_sources(G);
    if (rc < 0)
        return rc;
    /* octree: sets in descending member order (rt/raytrace.c:585); a full
     * leaf's code carries its set's place in set_data and its size (sizes
     * from 63 up read the count word), so that entering a leaf needs no
     * load before its members' */
    std::vector<int> kids(H.kids, H.kids + 8 * (size_t)H.nnodes);
    if (kids.empty()) kids.assign(8, -1);
    /* record slots: objects in the order a depth-first pass over the leaves
     * (the scene's octree, then each instanced one) first reaches them, so
     * that the objects of neighbouring leaves share cache lines; set
     * members are stored as slots */
    std::vector<int> slot_of((size_t)(H.nobjs > 0 ? H.nobjs : 1), -1);
    {
        int next = 0;
        std::vector<int32_t> stack;
        std::vector<int32_t> roots(1, H.root);
        for (int k = 0; k < H.nsubs; k++)
            roots.push_back(H.subs[k].root);
        for (int32_t rt : roots) {
            stack.assign(1, rt);
            while (!stack.empty()) {
                const int32_t code = stack.back();
                stack.pop_back();
                if (code >= 0) {
                    for (int k = 7; k >= 0; k--)          /* children 0..7 in order */
                        stack.push_back(H.kids[8 * (size_t)code + k]);
                } else if (code <= -2) {
                    const int32_t *st = gb_scene_set(&H, code);
                    for (int k = 1; k <= st[0]; k++)
                        if (slot_of[st[k]] < 0)
                            slot_of[st[k]] = next++;
                }
            }
        }
        for (int32_t i = 0; i < H.nobjs; i++)
            if (slot_of[i] < 0)
                slot_of[i] = next++;
    }
    std::vector<int> setdata((size_t)H.set_len > 0 ? (size_t)H.set_len : 1, 0);
    for (int32_t s = 0; s < H.nsets; s++) {
        const int32_t *st = H.set_data + H.set_off[s];
        setdata[H.set_off[s]] = st[0];
        for (int k = 1; k <= st[0]; k++)
            setdata[H.set_off[s] + k] = slot_of[st[st[0] + 1 - k]];
    }
    if ((int64_t)H.set_len >= GB_LEAF_MAXOFF)
        return set_err(GB_EUNSUPPORTED, "octree sets of %lld entries exceed the %d a leaf code addresses",
                       (long long)H.set_len, GB_LEAF_MAXOFF);
    auto leaf_code = [&](int k) {
        if (k > -2)
            return k;
        int64_t off = H.set_off[-k - 2];
        return gb_leaf_code((int)off, H.set_data[off]);
    };
    for (int &k : kids)
        k = leaf_code(k);
    /* instances: surface ids of their objects above every object index */
    std::vector<gb_dinst> inst((size_t)(H.ninst > 0 ? H.ninst : 1));
    long long sid = H.nobjs;
    for (int k = 0; k < H.ninst; k++) {
        const gb_instance &I = H.inst[k];
        const gb_subscene &sc = H.subs[I.sub];
        gb_dinst &d = inst[k];
        memset(&d, 0, sizeof d);
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 3; c++) {
                d.bx[3 * r + c] = (float)I.b.xfm[r][c];
                d.fx[3 * r + c] = (float)I.f.xfm[r][c];
            }
        d.bsca = (float)I.b.sca;
        d.fsca = (float)I.f.sca;
        for (int c = 0; c < 3; c++) d.cuorg[c] = (float)sc.cuorg[c];
        d.cusize = (float)sc.cusize;
        d.grid_scale = (float)((double)(1 << GRID_BITS_HOST) / sc.cusize);
        d.cell = (float)(sc.cusize / (double)(1 << GRID_BITS_HOST));
        d.root = leaf_code(sc.root);
        d.obj = I.obj;
        d.hasmod = H.objs[I.obj].omod >= 0;
        d.sidbase = (int)sid;
        d.firstobj = sc.firstobj;
        d.nobjs = sc.nobjs;
        sid += sc.nobjs;
    }
    if (sid >= 0x7fffffffll)
        return set_err(GB_EUNSUPPORTED, "%lld instanced surfaces exceed the 2^31 surface ids", sid);
    G->hinst.swap(inst);
    std::vector<float4> orec(4 * obj.size());    /* obj | geo | fv4 (2): the walk's 64-byte record */
    for (size_t i = 0; i < obj.size(); i++) {
        const size_t r = 4 * (size_t)slot_of[i];
        orec[r] = make_float4(__int_as_float_host(obj[i].x), __int_as_float_host((int)i),
                              __int_as_float_host(obj[i].z), __int_as_float_host(obj[i].w));
        orec[r + 1] = geo[i];
        orec[r + 2] = fv4[2 * i];
        orec[r + 3] = fv4[2 * i + 1];
    }
    if (orec.empty())
        orec.assign(4, make_float4(0, 0, 0, 0));
    /* the walk's leaf records: per set a header record (its first word the
     * member count), then the members' records in test order, so that
     * entering a leaf needs no load of its member list; an object in
     * several leaves has a record in each */
    {
        std::vector<int64_t> woff((size_t)(H.nsets > 0 ? H.nsets : 1), 0);
        int64_t nrec = 0;
        for (int32_t k = 0; k < H.nsets; k++) {
            woff[k] = nrec;
            nrec += 1 + H.set_data[H.set_off[k]];
        }
        if (nrec >= GB_LEAF_MAXOFF)
            return set_err(GB_EUNSUPPORTED, "octree leaves of %lld object records exceed the %d a leaf code addresses",
                           (long long)nrec, GB_LEAF_MAXOFF);
        std::vector<float4> lrec(4 * (size_t)(nrec > 0 ? nrec : 1), make_float4(0, 0, 0, 0));
        for (int32_t k = 0; k < H.nsets; k++) {
            const int cnt = setdata[H.set_off[k]];
            lrec[4 * (size_t)woff[k]] = make_float4(__int_as_float_host(cnt), 0.f, 0.f, 0.f);
            for (int j = 1; j <= cnt; j++) {
                const size_t from = 4 * (size_t)setdata[H.set_off[k] + j], to = 4 * (size_t)(woff[k] + j);
                for (int q = 0; q < 4; q++)
                    lrec[to + q] = orec[from + q];
            }
        }
        auto wcode = [&](int code) {
            if (code > -2)
                return code;
            const int32_t k = -code - 2;
            return gb_leaf_code((int)woff[k], setdata[H.set_off[k]]);
        };
        std::vector<int> wkids(H.kids, H.kids + 8 * (size_t)H.nnodes);
        if (wkids.empty()) wkids.assign(8, -1);
        for (int &k : wkids)
            k = wcode(k);
        for (int k = 0; k < H.ninst; k++)
            G->hinst[k].root = wcode(H.subs[H.inst[k].sub].root);
        G->wroot = wcode(H.root);
        G->hlrec.swap(lrec);
        G->hwkids.swap(wkids);
    }
    G->horec.swap(orec);
    /* smooth mesh triangles (rt/o_mesh.c:185-206): their vertex normals for
     * the shading kernels; the materials whose shading uses the perturbed
     * normal here are plastic and metal (light and glow ignore it) */
    {
        std::vector<int> vnidx((size_t)(H.nobjs > 0 ? H.nobjs : 1), -1);
        std::vector<float4> vnrm;
        G->has_vnorm = false;
        G->vnorm_error.clear();
        auto shaded = [&](int32_t carrier) {     /* the material slot's kind allows the perturbation */
            const int ms = G->matslot[carrier];
            const int k = ms >= 0 ? (int)G->mat[2 * ms].x : DM_NONE;
            return k == DM_NONE || k == DM_PLASTIC || k == DM_METAL || k == DM_LIGHT || k == DM_GLOW;
        };
        /* per octree an instance of which replaces its surfaces' materials
         * by one that is not shaded through vertex normals */
        std::vector<char> bad_sub((size_t)(H.nsubs > 0 ? H.nsubs : 1), 0);
        for (int k = 0; k < H.ninst; k++)
            if (H.objs[H.inst[k].obj].omod >= 0 && !shaded(H.inst[k].obj))
                bad_sub[H.inst[k].sub] = 1;
        std::vector<int> sub_of((size_t)(H.nobjs > 0 ? H.nobjs : 1), -1);
        for (int k = 0; k < H.nsubs; k++)
            for (int32_t i = H.subs[k].firstobj; i < H.subs[k].firstobj + H.subs[k].nobjs; i++)
                sub_of[i] = k;
        for (int32_t i = 0; i < H.nobjs; i++) {
            if (!((obj[i].x >> 8) & DF_VNORM))
                continue;
            G->has_vnorm = true;
            vnidx[i] = (int)(vnrm.size() / 3);
            for (int k = 0; k < 3; k++)
                vnrm.push_back(make_float4((float)H.objs[i].vnorm[3 * k], (float)H.objs[i].vnorm[3 * k + 1],
                                           (float)H.objs[i].vnorm[3 * k + 2], 0.f));
            const bool ok = shaded(i) && !(sub_of[i] >= 0 && bad_sub[sub_of[i]]);
            if (!ok && G->vnorm_error.empty())
                G->vnorm_error = "mesh triangles with vertex normals are supported on plastic, metal, light and glow "
                                 "materials only";
        }
        if (vnrm.empty())
            vnrm.assign(3, make_float4(0, 0, 0, 0));
        G->hvnidx.swap(vnidx);
        G->hvnrm.swap(vnrm);
    }
    G->hoslot.swap(slot_of);
    /* FP64 geometry per object for the first-hit casts (cast64.cu) */
    {
        std::vector<double> g64;
        std::vector<long long> g64off((size_t)(H.nobjs > 0 ? H.nobjs : 1), 0);
        g64.push_back(0.0);                      /* offset 0: objects with no record */
        std::vector<int> inst_of((size_t)(H.nobjs > 0 ? H.nobjs : 1), -1);
        for (int k = 0; k < H.ninst; k++)
            inst_of[H.inst[k].obj] = k;
        for (int32_t i = 0; i < H.nobjs; i++) {
            const gb_object *o = &H.objs[i];
            const int kind = obj[i].x & 0xff;
            const long long at = (long long)g64.size();
            if (kind == DK_FACE) {
                const gb_face *f = &H.faces[i];
                for (int j = 0; j < 3; j++) g64.push_back(f->norm[j]);
                g64.push_back(f->offset);
                g64.push_back(f->ok ? 1.0 : 0.0);
                g64.push_back((double)f->ax);
                g64.push_back((double)f->nv);
                for (int j = 0; j < 3 * f->nv; j++) g64.push_back(o->farg[j]);
                if ((obj[i].x >> 8) & DF_VNORM)          /* then its three vertex normals */
                    for (int j = 0; j < 9; j++) g64.push_back(o->vnorm[j]);
                if ((obj[i].x >> 8) & DF_VUV)            /* and their (u,v) */
                    for (int j = 0; j < 6; j++) g64.push_back(o->vuv[j]);
            } else if (kind == DK_SPHERE || kind == DK_BUBBLE) {
                for (int j = 0; j < 4; j++) g64.push_back(o->farg[j]);
            } else if (kind == DK_CONE || kind == DK_CUP || kind == DK_CYL || kind == DK_TUBE || kind == DK_RING) {
                const gb_cone *co = &H.cones[i];
                g64.push_back(co->ok ? 1.0 : 0.0);
                g64.push_back(co->al);
                g64.push_back(co->sl);
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) g64.push_back(co->tm[a][b]);
                if (kind == DK_RING)
                    for (int j = 0; j < 6; j++) g64.push_back(o->farg[j]);
                else {
                    for (int j = 0; j < 3; j++) g64.push_back(o->farg[co->p0 + j]);
                    for (int j = 0; j < 3; j++) g64.push_back(o->farg[co->p1 + j]);
                }
                const double r0 = co->r0 >= 0 ? o->farg[co->r0] : 0.0;
                g64.push_back(r0);
                g64.push_back(co->r1 >= 0 ? o->farg[co->r1] : r0);
            } else if (kind == DK_INSTANCE && inst_of[i] >= 0) {
                const gb_instance &I = H.inst[inst_of[i]];
                const gb_subscene &sc = H.subs[I.sub];
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) g64.push_back(I.b.xfm[a][b]);
                g64.push_back(I.b.sca);
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) g64.push_back(I.f.xfm[a][b]);
                g64.push_back(I.f.sca);
                for (int j = 0; j < 3; j++) g64.push_back(sc.cuorg[j]);
                g64.push_back(sc.cusize);
                g64.push_back((double)leaf_code(sc.root));
                g64.push_back(o->omod >= 0 ? 1.0 : 0.0);
            } else
                continue;
            g64off[i] = at;
        }
        G->hg64.swap(g64);
        G->hg64off.swap(g64off);
    }
    std::vector<gb_dsrc> src = G->src;
    if (src.empty()) src.resize(1);
    G->hkids.swap(kids);
    G->hsetdata.swap(setdata);
    G->hobj.swap(obj);
    G->hgeo.swap(geo);
    G->hfvert.swap(fvert);
    G->hfv4.swap(fv4);
    G->hcone.swap(cone);
    G->hsrc.swap(src);
    gb_dscene &d = G->ds;
    memset(&d, 0, sizeof d);
    for (int j = 0; j < 3; j++) d.cuorg[j] = (float)H.cuorg[j];
    d.cusize = (float)H.cusize;
    d.grid_scale = (float)((double)(1 << GRID_BITS_HOST) / H.cusize);
    d.cell = (float)(H.cusize / (double)(1 << GRID_BITS_HOST));
    d.root = leaf_code(H.root);
    d.nnodes = H.nnodes;
    d.kids = G->hkids.data();
    d.set_data = G->hsetdata.data();
    d.wroot = G->wroot;
    d.wkids = G->hwkids.data();
    d.lrec = G->hlrec.data();
    d.has_vnorm = G->has_vnorm;
    d.vnidx = G->hvnidx.data();
    d.vnrm = G->hvnrm.data();
    d.nobjs = H.nobjs;
    d.obj = G->hobj.data();
    d.geo = G->hgeo.data();
    d.fvert = G->hfvert.data();
    d.fv4 = G->hfv4.data();
    d.orec = G->horec.data();
    d.oslot = G->hoslot.data();
    d.cone = G->hcone.data();
    d.mat = G->mat.data();
    d.nsrc = (int)G->src.size();
    d.src = G->hsrc.data();
    d.ninst = H.ninst;
    d.inst = G->hinst.data();
    for (int j = 0; j < 3; j++) d.cuorg64[j] = H.cuorg[j];
    d.cusize64 = H.cusize;
    d.g64 = G->hg64.data();
    d.g64off = G->hg64off.data();
    /* names for output */
    G->modname.resize(H.nobjs);
    G->matname.resize(H.nobjs);
    for (int32_t i = 0; i < H.nobjs; i++) {
        int32_t m = H.objs[i].omod;
        G->modname[i] = m >= 0 ? H.objs[m].name : "void";
        int32_t mm = gb_find_material(&H, i);
        G->matname[i] = mm >= 0 ? H.objs[mm].name : "void";
    }
    return GB_OK;
}

static int finish_load(gb_scene *G, gb_scene **out)
{
    int rc = prepare_device(G);
    if (rc < 0) {
        gb_scene_free(G);
        return rc;
    }
    *out = G;
    return GB_OK;
}

extern "C" int gb_scene_load(const char *oct_path, gb_scene **out)
{
    if (!oct_path || !out)
        return set_err(GB_EINVAL, "null argument");
    gb_scene *G = new gb_scene();
    gb_scene_init(&G->H);
    if (gb_scene_read_oct(&G->H, oct_path) < 0) {
        int rc = set_err(GB_EIO, "%s", gb_scene_error());
        gb_scene_free(G);
        return rc;
    }
    std::string dir(oct_path);                   /* instance octrees: also beside this one */
    size_t sl = dir.find_last_of('/');
    dir = sl == std::string::npos ? std::string(".") : dir.substr(0, sl);
    if (gb_scene_load_instances(&G->H, dir.c_str()) < 0) {
        int rc = set_err(GB_EIO, "%s", gb_scene_error());
        gb_scene_free(G);
        return rc;
    }
    return finish_load(G, out);
}

/* An octree among the scene files (oconv -i): its objects join the others
 * and the octree is built again over all of them. */
static bool is_octree_file(const char *path)
{
    FILE *fp = fopen(path, "rb");
    if (!fp)
        return false;
    char buf[4096];
    size_t n = fread(buf, 1, sizeof buf - 1, fp);
    fclose(fp);
    buf[n] = '\0';
    const char *end = strstr(buf, "\n\n");
    const char *f = strstr(buf, "FORMAT=Radiance_octree");
    return !strncmp(buf, "#?RADIANCE", 10) && f && (!end || f < end);
}

extern "C" int gb_scene_load_rad(const char *const *paths, int npaths, int objlim, int resolu, gb_scene **out)
{
    if (!paths || npaths <= 0 || !out)
        return set_err(GB_EINVAL, "no scene files");
    gb_scene *G = new gb_scene();
    gb_scene_init(&G->H);
    for (int i = 0; i < npaths; i++)
        if ((is_octree_file(paths[i]) ? gb_scene_read_oct(&G->H, paths[i]) : gb_scene_read_rad_file(&G->H, paths[i])) < 0) {
            int rc = set_err(GB_EIO, "%s", gb_scene_error());
            gb_scene_free(G);
            return rc;
        }
    for (int32_t i = 0; i < G->H.nobjs; i++)
        if (gb_is_volume(G->H.objs[i].otype)) {
            int rc = set_err(GB_EUNSUPPORTED, "%s: instances and meshes are read from an octree made by oconv, "
                             "not built here", G->H.objs[i].name);
            gb_scene_free(G);
            return rc;
        }
    /* the octree: on the device where there is one and the scene is of
     * polygons and spheres (GB_OCTREE_BUILDER=host forces the host
     * builder); both give the same tree */
    int dev_rc = 1, ndev = 0;
    const char *which = getenv("GB_OCTREE_BUILDER");
    if (!(which && !strcmp(which, "host")) && cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0) {
        char why[256] = "";
        dev_rc = gb_scene_build_octree_device(&G->H, objlim, resolu, why, sizeof why);
        if (dev_rc < 0)
            cudaGetLastError();          /* the host builder below starts afresh */
    } else
        cudaGetLastError();
    G->octree_on_device = dev_rc == 0;
    if ((dev_rc != 0 && gb_scene_build_octree(&G->H, objlim, resolu) < 0) || gb_scene_load_instances(&G->H, ".") < 0) {
        int rc = set_err(GB_EIO, "octree build failed: %s", gb_scene_error());
        gb_scene_free(G);
        return rc;
    }
    return finish_load(G, out);
}

/* node count, set count and an FNV-1a hash over the pre-order tree with
 * each leaf's sorted set: equal for equal octrees */
static void digest_code(const gb_scene_host *H, int32_t code, uint64_t *h)
{
    auto mix = [h](uint32_t v) { *h = (*h ^ (uint64_t)v) * 1099511628211ull; };
    if (code >= 0) {
        mix(2);
        for (int k = 0; k < 8; k++)
            digest_code(H, H->kids[8 * code + k], h);
    } else if (code == -1) {
        mix(0);
    } else {
        const int32_t *st = gb_scene_set(H, code);
        mix(1);
        for (int k = 0; k <= st[0]; k++)
            mix((uint32_t)st[k]);
    }
}

extern "C" int gb_scene_octree_info(const gb_scene *G, int64_t *nodes, int64_t *sets, uint64_t *digest,
                                    int *built_on_device)
{
    if (!G)
        return set_err(GB_EINVAL, "null scene");
    if (nodes)
        *nodes = G->H.nnodes;
    if (sets)
        *sets = G->H.nsets;
    if (digest) {
        uint64_t h = 1469598103934665603ull;
        digest_code(&G->H, G->H.root, &h);
        *digest = h;
    }
    if (built_on_device)
        *built_on_device = G->octree_on_device;
    return GB_OK;
}

extern "C" void gb_scene_free(gb_scene *G)
{
    if (!G)
        return;
    DevBuf *bufs[] = {&G->kids, &G->setdata, &G->instd, &G->orec, &G->oslot, &G->obj, &G->geo, &G->fvert, &G->fv4,
                      &G->cone, &G->matd, &G->g64, &G->g64off, &G->wkids, &G->lrec, &G->vnidx, &G->vnrm,
                      &G->srcd, &G->trk, &G->sensors, &G->value, &G->bins, &G->stats, &G->roots, &G->rootspt, &G->qa,
                      &G->qb, &G->qcount, &G->binprog, &G->modinfo, &G->hits, &G->hitt, &G->trkrun, &G->hitrec,
                      &G->adja, &G->adjb, &G->dlde, &G->gradd, &G->rootdraw, &G->rootlot, &G->tga, &G->tgb,
                      &G->ssval, &G->sscnt, &G->sserr, &G->slow, &G->hitpn};
    for (DevBuf *b : bufs)
        b->release();
    if (G->pin)
        cudaFreeHost(G->pin);
    if (G->pinb)
        cudaFreeHost(G->pinb);
    if (G->stream)
        cudaStreamDestroy(G->stream);
    gb_scene_clear(&G->H);
    delete G;
}

extern "C" int64_t gb_scene_nobjects(const gb_scene *G) { return G ? G->H.nobjs : 0; }
extern "C" const char *gb_scene_object_name(const gb_scene *G, int64_t i)
{
    return (G && i >= 0 && i < G->H.nobjs) ? G->H.objs[i].name : "*";
}
extern "C" const char *gb_scene_modifier_name(const gb_scene *G, int64_t i)
{
    return (G && i >= 0 && i < G->H.nobjs) ? G->modname[i].c_str() : "*";
}
extern "C" const char *gb_scene_material_name(const gb_scene *G, int64_t i)
{
    return (G && i >= 0 && i < G->H.nobjs) ? G->matname[i].c_str() : "*";
}

/* ---------------------------------------------------------------- options */

extern "C" int gb_opts_default(int prog, gb_opts *o)
{
    if (!o)
        return set_err(GB_EINVAL, "null options");
    memset(o, 0, sizeof *o);
    o->prog = prog;
    o->fin = o->fout = 'a';
    o->h = 1;
    o->n = 1;
    o->u = 1;
    o->bv = 1;
    o->dv = 1;
    o->lr = -10;
    o->ar = 256;
    o->dc = .75;
    o->dp = 512;
    o->ss = 1.0;
    o->c = 1;
    strcpy(o->outspec, "v");
    if (prog == GB_PROG_RCONTRIB) {   /* rt/rcontrib.c:24-58 + rcmain.c:164-172 */
        o->dj = .9; o->ds = .2; o->dt = 0.; o->dr = 3; o->st = .02; o->lw = 2e-3;
        o->ab = 1; o->aa = 0.; o->ad = 350; o->as = 0;
    } else {                          /* rt/raycalls.c:121-150 */
        o->dj = 0.; o->ds = .2; o->dt = .03; o->dr = 2; o->st = .15; o->lw = 1e-4;
        o->ab = 0; o->aa = .1; o->ad = 1024; o->as = 512;
    }
    return GB_OK;
}

static int boolopt(const char *a, int olen, int *var)
{
    switch (a[olen]) {
    case '\0': *var = !*var; return 0;
    case '+': case '1': *var = 1; return 0;
    case '-': case '0': *var = 0; return 0;
    default: return -1;
    }
}

extern "C" int gb_opts_parse(int argc, const char *const *argv, int prog, gb_opts *o, int *nused)
{
    int i;
    for (i = 0; i < argc; i++) {
        const char *a = argv[i];
        if (!a || a[0] != '-' || !a[1])
            break;
        auto need = [&](int k) { return i + k < argc; };
#define NEED(k) do { if (!need(k)) return set_err(GB_EINVAL, "missing argument for %s", a); } while (0)
#define FARG(k) atof(argv[i + (k)])
#define IARG(k) atoi(argv[i + (k)])
        bool ok = true;
        switch (a[1]) {
        case 'u': ok = boolopt(a, 2, &o->u) == 0; break;
        case 'w': break;                              /* warnings */
        case 'b':
            if (a[2] == 'v') ok = boolopt(a, 3, &o->bv) == 0;
            else ok = false;
            break;
        case 'd':
            switch (a[2]) {
            case 't': NEED(1); o->dt = FARG(1); i++; break;
            case 'c': NEED(1); o->dc = FARG(1); i++; break;
            case 'j': NEED(1); o->dj = FARG(1); i++; break;
            case 'r': NEED(1); o->dr = IARG(1); i++; break;
            case 'p': NEED(1); o->dp = IARG(1); i++; break;
            case 'v': ok = boolopt(a, 3, &o->dv) == 0; break;
            case 's': NEED(1); o->ds = FARG(1); i++; break;
            default: ok = false;
            }
            break;
        case 's':
            if (a[2] == 't') { NEED(1); o->st = FARG(1); i++; }
            else if (a[2] == 's') { NEED(1); o->ss = FARG(1); i++; }
            else ok = false;
            break;
        case 'l':
            if (a[2] == 'r' && !a[3]) { NEED(1); o->lr = IARG(1); i++; }
            else if (a[2] == 'w' && !a[3]) { NEED(1); o->lw = FARG(1); i++; }
            else if (a[2] == 'd') { int v = o->ld != 0; ok = boolopt(a, 3, &v) == 0; o->ld = v; }
            else ok = false;
            break;
        case 'i': ok = boolopt(a, 2, &o->i) == 0; break;
        case 'I': ok = boolopt(a, 2, &o->I) == 0; break;
        case 'a':
            switch (a[2]) {
            case 'v': NEED(3); o->av[0] = FARG(1); o->av[1] = FARG(2); o->av[2] = FARG(3); i += 3; break;
            case 'w': NEED(1); o->aw = IARG(1); i++; break;
            case 'a': NEED(1); o->aa = FARG(1); i++; break;
            case 'r': NEED(1); o->ar = IARG(1); i++; break;
            case 'd': NEED(1); o->ad = IARG(1); i++; break;
            case 's': NEED(1); o->as = IARG(1); i++; break;
            case 'b': NEED(1); o->ab = IARG(1); i++; break;
            case 'i': case 'I': case 'e': case 'E': case 'f':
                return set_err(GB_EUNSUPPORTED, "option %s (ambient lists/files) is not supported", a);
            default: ok = false;
            }
            break;
        case 'm':
            if (prog == GB_PROG_RCONTRIB && !a[2]) { ok = false; break; }
            return set_err(GB_EUNSUPPORTED, "participating media (%s) are not supported", a);
        case 'h': ok = boolopt(a, 2, &o->h) == 0; break;
        case 'n': NEED(1); o->n = IARG(1); i++; break;
        case 'x': NEED(1); o->x = IARG(1); i++; break;
        case 'y': NEED(1); o->y = IARG(1); i++; break;
        case 'c':
            if (prog == GB_PROG_RCONTRIB && !a[2]) { NEED(1); o->c = IARG(1); i++; }
            else return set_err(GB_EUNSUPPORTED, "option %s is not supported", a);
            break;
        case 'V': ok = prog == GB_PROG_RCONTRIB && boolopt(a, 2, &o->V) == 0; break;
        case 'f':
            if (!a[2]) { ok = false; break; }     /* -f calfile: modifier option */
            if (a[2] == 'o') break;               /* -fo force open */
            if (!strchr("afd", a[2])) { ok = false; break; }
            o->fin = a[2];
            o->fout = a[3] ? a[3] : a[2];
            if (!strchr("afdc", o->fout)) ok = false;
            break;
        case 'o':
            if (prog == GB_PROG_RTRACE && a[2]) {
                snprintf(o->outspec, sizeof o->outspec, "%s", a + 2);
                break;
            }
            ok = false;
            break;
        case 'e': case 'p': case 'M':
            ok = false;
            break;
        case 't':
            /* -t N report interval; -ti/-te modifier and -tI/-tE file of
             * the ray-tree trace lists (rt/rtmain.c:210-260), which select
             * what the '~' part of -o prints; the value and the first-hit
             * outputs do not depend on them */
            if (a[2] && (!strchr("iIeE", a[2]) || a[3])) { ok = false; break; }
            NEED(1);
            if (a[2] == 'I' || a[2] == 'E') {
                FILE *f = fopen(argv[i + 1], "r");
                if (!f)
                    return set_err(GB_EIO, "cannot open trace %s file \"%s\"", a[2] == 'I' ? "include" : "exclude",
                                   argv[i + 1]);
                fclose(f);
            }
            i++;
            break;
        default: ok = false;
        }
        if (!ok) {
            if (prog == GB_PROG_RCONTRIB && strchr("fepbmMo", a[1]))
                break;                             /* modifier options: caller */
            return set_err(GB_EINVAL, "command line error at '%s'", a);
        }
#undef NEED
#undef FARG
#undef IARG
    }
    if (nused)
        *nused = i;
    return GB_OK;
}

/* -------------------------------------------------------- run machinery */

static int check_shading(gb_scene *G, const gb_opts *o)
{
    if (!G->unsupported.empty()) {
        const gb_object *m = &G->H.objs[G->unsupported[0]];
        std::string why;
        float4 a, b;
        material_kind(m, &a, &b, why);
        return set_err(GB_EUNSUPPORTED, "%s (\"%s\")", why.c_str(), m->name);
    }
    if (!G->src_error.empty())
        return set_err(GB_EUNSUPPORTED, "%s", G->src_error.c_str());
    if (!G->vnorm_error.empty())
        return set_err(GB_EUNSUPPORTED, "%s", G->vnorm_error.c_str());
    /* the ambient value of a smooth surface in rtrace carries a texture
     * factor made from the whole hemisphere's sample values and distances
     * (rt/ambient.c:269-296, doambient's rotational gradient); the wavefront
     * queues each sample as an independent child ray, so it is not formed.
     * rcontrib's contributions (ray coefficients) do not carry it. */
    if (G->has_vnorm && o->prog == GB_PROG_RTRACE && o->ab >= (o->I ? 2 : 1))
        return set_err(GB_EUNSUPPORTED, "rtrace -ab %d on meshes with vertex normals is not implemented (the ambient "
                       "texture gradient); rcontrib, or rtrace -ab %d, is", o->ab, o->I ? 1 : 0);
    if (o->ab > 0 && o->aa > GB_FTINY)
        return set_err(GB_EUNSUPPORTED, "the ambient cache (-aa %g) is not implemented; use -aa 0", o->aa);
    if (o->as > 0 && o->ab > 0 && o->aa > GB_FTINY)
        return set_err(GB_EUNSUPPORTED, "ambient super-sampling (-as) is not implemented");
    if (!o->bv)
        return set_err(GB_EUNSUPPORTED, "-bv- is not implemented");
    if (!o->dv)
        return set_err(GB_EUNSUPPORTED, "-dv- is not implemented");
    if (o->ld != 0)
        return set_err(GB_EUNSUPPORTED, "-ld is not implemented");
    /* mirrors relay sources as virtual sources under -dr (rt/virtuals.c),
     * which is not built: only -dr 0, or mirrors on curved surfaces (which
     * make none) */
    if (o->dr > 0 && !G->src.empty())
        for (int32_t i = 0; i < G->H.nobjs; i++) {
            const int ms = G->matslot[i];
            if (ms >= 0 && (int)G->mat[2 * ms].x == DM_MIRROR &&
                (G->H.objs[i].otype == GT_POLYGON || G->H.objs[i].otype == GT_RING))
                return set_err(GB_EUNSUPPORTED, "virtual sources of mirror \"%s\" (-dr %d) are not implemented; "
                               "use -dr 0", G->H.objs[i].name, o->dr);
        }
    /* -ds: flat local sources are partitioned, spheres are one piece
     * (rt/srcsupp.c:36 sphsobj nopart), as in the reference */
    /* rough specular sampled with several samples per hit (-ss > 1.5,
     * rt/normal.c:387-398): the reference weights their values, not their
     * ray coefficients, by the W-G-M-D adjustment, so rcontrib's bins (built
     * from the coefficients, rt/raytrace.c:408-442) would differ from the
     * values; rtrace is supported */
    if (o->prog == GB_PROG_RCONTRIB && o->ss > 1.5) {
        for (size_t sl = 0; sl < G->matobj.size(); sl++) {
            float4 a = G->mat[2 * sl], b = G->mat[2 * sl + 1];
            int k = (int)a.x;
            double rspec = b.x;
            if ((k == DM_PLASTIC || k == DM_METAL || k == DM_TRANS) && b.y * b.y > GB_FTINY && rspec > GB_FTINY &&
                !(o->st >= rspec - GB_FTINY))
                return set_err(GB_EUNSUPPORTED,
                               "rcontrib with -ss %g samples the rough specular lobe of \"%s\" several times per "
                               "hit, which is not implemented; use -ss 1 or less",
                               o->ss, G->H.objs[G->matobj[sl]].name);
        }
    }
    return GB_OK;
}

static uint64_t seed_of(const gb_opts *o)
{
    if (o->seed)
        return o->seed;
    if (!o->u)
        return 0;
    return (uint64_t)time(nullptr) * 0x9E3779B97F4A7C15ull;
}

/* Extra samples per -I first hemisphere of n0 x n0 strata under -as
 * (rt/ambcomp.c:403-409): rtrace only (rcontrib forces -as 0,
 * rt/rcmain.c:167), with -aa 0 (the cache is not implemented), hemispheres
 * of more than 7 x 7 strata, and at least four times n0 samples; 0 when
 * there is no super-sampling. */
static int supersamples(const gb_opts *o, int n0)
{
    if (o->prog != GB_PROG_RTRACE || !o->I || o->ab <= 0 || o->aa > GB_FTINY || o->as <= 0 || n0 * n0 <= 49)
        return 0;
    double d = M_PI * 0.8 / (o->ad * o->lw + 1e-20), wt = 1.0;
    if (wt > d) wt = d;
    int cnt = (int)((float)o->as * (float)wt + .5f);
    return cnt >= 4 * n0 ? cnt : 0;
}

/* Whether a hemisphere sampled at ray weight w (with a reflectance of at
 * most 1, or pi for the -I/-i Lambertian) would be super-sampled. */
static bool hemi_supersampled(const gb_opts *o, double w, double rho)
{
    double d = rho * 0.8 * w / (o->ad * o->lw + 1e-20), wt = w;
    if (wt > d) wt = d;
    int n = (int)(sqrt(o->ad * wt) + 0.5);
    return n * n > 49 && (int)(o->as * wt + .5) >= 4 * n;
}

/* -as super-sampling that is not implemented: of any hemisphere but the
 * -I first ones (rtrace with -aa 0 only; rcontrib forces -as 0) */
static int check_supersampling(const gb_opts *o, int n0)
{
    if (o->prog != GB_PROG_RTRACE || o->ab <= 0 || o->aa > GB_FTINY || o->as <= 0)
        return GB_OK;
    bool other;
    if (o->I)                                    /* below the first hemisphere: weight <= pi / n0^2 */
        other = o->ab > 1 && hemi_supersampled(o, fmin(1.0, M_PI / ((double)n0 * n0)), M_PI);
    else                                         /* primary hits at weight 1 */
        other = hemi_supersampled(o, 1.0, o->i ? M_PI : 1.0);
    if (other)
        return set_err(GB_EUNSUPPORTED, "ambient super-sampling (-as %d) is implemented for the first hemisphere "
                       "of -I sensors only; this run would super-sample others: use -as 0", o->as);
    return GB_OK;
}

static int root_divisions(const gb_opts *o)
{
    /* samp_hemi for the Lambertian (rho = pi) at weight 1 (rt/ambcomp.c:366-374) */
    double d = M_PI, wt = 1.0;
    d *= 0.8 * 1.0 / (o->ad * o->lw + 1e-20);
    if (wt > d) wt = d;
    int n = (int)(sqrt(o->ad * wt) + 0.5);
    return n < 1 ? 1 : n;
}

struct RunOut {
    double *value;          /* host n x 3 or null */
    double *bins;           /* host records x nbins x 3 or null */
    int32_t *hit_id;
    double *hit_t;
    const double *dlde;     /* gradient runs: host n x 3 d(loss)/d(value) */
    double *grad;           /* gradient runs: host nslots x 3 */
    double *hit_normal;     /* host n x 3 or null: the first hit's surface normal */
    double *hit_vnormal;    /* host n x 3 or null: a smooth mesh hit's interpolated vertex normal (else 0) */
    double *hit_uv;         /* host n x 2 or null: a mesh hit's interpolated vertex (u,v) (else 0) */
};

/* largest generation and queue capacity of the last run on this thread */
static thread_local long long g_maxgen, g_qcap;

static int run(gb_scene *G, const gb_opts *o, int follow, const double *org_dir, int64_t n,
               const std::vector<gb_binins> *prog, const std::vector<int4> *modinfo, int nbins_total,
               const std::vector<int> *trk, RunOut out, long long qcap_req = 0, int64_t sensor_base = 0)
{
    cudaStream_t st = G->stream;
    if (sensor_base == 0) {                      /* first slice: counters start over */
        g_maxgen = 0;
        g_qcap = 0;
        g_stats[0] = g_stats[1] = g_stats[2] = g_stats[3] = 0;
        memset(&g_prof, 0, sizeof g_prof);
    }
    if (n <= 0)
        return GB_OK;
    const size_t stat_bytes = GB_K_N * GB_ST_N * sizeof(unsigned long long);
    size_t sbytes = (size_t)n * 6 * sizeof(double);
    if (G->sensors.ensure(sbytes) < 0 || G->stats.ensure(stat_bytes) < 0 ||
        G->qcount.ensure(4 * sizeof(unsigned long long)) < 0)
        return set_err(GB_ENOMEM, "device allocation failed");
    if (!G->nev) {
        for (int k = 0; k < (int)(sizeof G->ev / sizeof G->ev[0]); k++)
            CK(cudaEventCreate(&G->ev[k]));
        G->nev = (int)(sizeof G->ev / sizeof G->ev[0]);
    }
    int evused = 2;                                /* ev[0], ev[1]: the kernel region */
    int evkid[GB_TIMED_LAUNCHES];
    bool capturing = false;                        /* launches go into a graph: not timed one by one */
    /* one launch, bracketed by events, counting into its kernel's block */
    auto launch = [&](int kid, gb_run &PR, auto fn) -> int {
        PR.stats = (unsigned long long *)G->stats.p + kid * GB_ST_N;
        int slot = (evused - 2) / 2;
        bool timed = !capturing && slot < GB_TIMED_LAUNCHES;
        if (timed)
            cudaEventRecord(G->ev[evused], st);
        if (fn(PR) < 0)
            return set_err(GB_ECUDA, "launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        if (timed) {
            cudaEventRecord(G->ev[evused + 1], st);
            evkid[slot] = kid;
            evused += 2;
        }
        g_stats[3]++;
        g_prof.launches[kid]++;
        return GB_OK;
    };
    CK(cudaMemcpyAsync(G->sensors.p, org_dir, sbytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(G->stats.p, 0, stat_bytes, st));

    gb_run P;
    memset(&P, 0, sizeof P);
    P.S = G->ds;
    P.ab = o->ab;
    P.ad = o->ad;
    P.minweight = (float)o->lw;
    P.maxdepth = o->lr;
    for (int j = 0; j < 3; j++) P.av[j] = (float)o->av[j];
    P.dstrsrc = (float)o->dj;
    P.srcsizerat = (float)o->ds;
    P.specthresh = (float)o->st;
    P.specjitter = (float)o->ss;
    P.do_irrad = o->i;
    P.follow = follow;
    P.contrib_mode = o->V;
    uint64_t seed = seed_of(o);
    P.k0 = (uint32_t)seed;
    P.k1 = (uint32_t)(seed >> 32);
    P.replica = o->replica;
    P.nsensors = n;
    P.sensor_base = (uint32_t)sensor_base;
    P.sensors = (const double *)G->sensors.p;
    P.stats = (unsigned long long *)G->stats.p;
    P.accum = o->c > 0 ? o->c : 1;
    P.nbins_total = nbins_total;
    P.walk_refill = G->tuned_refill;
    P.walk_blocks_per_sm = G->tuned_blocks;

    /* cast-only outputs */
    std::function<void()> unpack_hits;
    if (out.hit_id) {
        if (G->hits.ensure((size_t)n * sizeof(int)) < 0 || G->hitt.ensure((size_t)n * sizeof(float)) < 0)
            return set_err(GB_ENOMEM, "device allocation failed");
        P.S.trk = nullptr;
        if (out.hit_normal && G->hitpn.ensure((size_t)n * 11 * sizeof(double)) < 0)
            return set_err(GB_ENOMEM, "device allocation failed");
        double *d_pn = out.hit_normal ? (double *)G->hitpn.p : nullptr;
        int rc = launch(GB_K_CAST, P, [&](gb_run &R) {
            return gb_launch_cast64(&R, (int *)G->hits.p, (float *)G->hitt.p, d_pn, st, G->sms); });
        if (rc < 0)
            return rc;
        /* the first hits come back through pinned staging, unpacked after
         * the values' final synchronisation when values follow, so that the
         * host does not wait for the casts before it queues the values */
        const size_t hb = (size_t)n * (sizeof(int) + sizeof(float)) + (d_pn ? (size_t)n * 11 * sizeof(double) : 0);
        if (G->pin_n < hb) {
            if (G->pin)
                cudaFreeHost(G->pin);
            G->pin = nullptr;
            G->pin_n = 0;
            if (cudaHostAlloc(&G->pin, hb, cudaHostAllocDefault) != cudaSuccess) {
                cudaGetLastError();
                G->pin = nullptr;
                return set_err(GB_ENOMEM, "cannot allocate %zu bytes of pinned host memory", hb);
            }
            G->pin_n = hb;
        }
        double *pn = (double *)G->pin;
        int *h = (int *)(pn + (d_pn ? (size_t)n * 11 : 0));
        float *t = (float *)(h + n);
        CK(cudaMemcpyAsync(h, G->hits.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(t, G->hitt.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (d_pn)
            CK(cudaMemcpyAsync(pn, d_pn, (size_t)n * 11 * sizeof(double), cudaMemcpyDeviceToHost, st));
        unpack_hits = [&out, n, h, t, pn]() {
            for (int64_t i = 0; i < n; i++) {
                out.hit_id[i] = h[i];
                if (out.hit_t)
                    out.hit_t[i] = t[i];
                if (out.hit_normal)
                    for (int k = 0; k < 3; k++)
                        out.hit_normal[3 * i + k] = pn[11 * i + 3 + k];
                if (out.hit_vnormal)
                    for (int k = 0; k < 3; k++)
                        out.hit_vnormal[3 * i + k] = pn[11 * i + 6 + k];
                if (out.hit_uv)
                    for (int k = 0; k < 2; k++)
                        out.hit_uv[2 * i + k] = pn[11 * i + 9 + k];
            }
        };
        if (!out.value && !out.bins) {
            CK(cudaStreamSynchronize(st));
            unpack_hits();
            g_stats[0] = n;
            return GB_OK;
        }
    }

    if (out.value) {
        if (G->value.ensure((size_t)n * 3 * sizeof(double)) < 0)
            return set_err(GB_ENOMEM, "device allocation failed");
        CK(cudaMemsetAsync(G->value.p, 0, (size_t)n * 3 * sizeof(double), st));
        P.value = (double *)G->value.p;
    }
    int64_t nrec = n / P.accum;
    if (out.bins) {
        /* room for a trailing partial record, which is not returned */
        size_t bb = (size_t)((n + P.accum - 1) / P.accum + 1) * nbins_total * 3 * sizeof(double);
        if (G->bins.ensure(bb) < 0 || upload(G->binprog, *prog) < 0 || upload(G->modinfo, *modinfo) < 0 ||
            upload(G->trkrun, *trk) < 0)
            return set_err(GB_ENOMEM, "device allocation failed");
        CK(cudaMemsetAsync(G->bins.p, 0, bb, st));
        P.bins = (double *)G->bins.p;
        P.binprog = (const gb_binins *)G->binprog.p;
        P.modinfo = (const int4 *)G->modinfo.p;
        P.S.trk = (const int *)G->trkrun.p;
    } else {
        std::vector<int> none(G->H.nobjs > 0 ? G->H.nobjs : 1, -1);
        if (upload(G->trkrun, none) < 0)
            return set_err(GB_ENOMEM, "device allocation failed");
        P.S.trk = (const int *)G->trkrun.p;
    }

    /* queues: sized for the expected fan-out, bounded by memory */
    int n0 = (o->I && o->ab > 0 && o->ad > 0) ? root_divisions(o) : 0;
    if (n0 > 128)
        return set_err(GB_EUNSUPPORTED, "-ad %d gives %d x %d hemisphere divisions; at most 128 x 128 are "
                       "supported", o->ad, n0, n0);
    long long est = (long long)n * (n0 > 0 ? (long long)n0 * n0 * 4 : (o->ab > 0 ? (long long)o->ad * 2 : 8));
    long long qcap = est < (1ll << 20) ? (1ll << 20) : est;
    if (qcap_req > 0)
        qcap = qcap_req;                         /* measured by a pilot run, or a retry */
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const bool grad = out.grad != nullptr;
    {
        int rc = check_supersampling(o, n0);
        if (rc < 0)
            return rc;
    }
    const int ss = supersamples(o, n0);
    if (ss > 0 && (grad || !out.value))
        return set_err(GB_EUNSUPPORTED, "ambient super-sampling (-as %d) in a gradient run is not implemented; "
                       "use -as 0", o->as);
    /* two queues, the walk results, in gradient runs the factor lists, in
     * super-sampled runs the strata tags */
    const size_t slot = 2 * sizeof(gb_qray) + sizeof(gb_qhit) + (grad ? 2 * sizeof(gb_qadj) : 0) +
                        (ss > 0 ? 2 * sizeof(uint32_t) : 0);
    long long qmax = (long long)(freeb / 3 / slot);
    if (qmax > (1ll << 28)) qmax = 1ll << 28;
    if (qcap > qmax) qcap = qmax;
    if (G->qa.ensure((size_t)qcap * sizeof(gb_qray)) < 0 || G->qb.ensure((size_t)qcap * sizeof(gb_qray)) < 0 ||
        G->hitrec.ensure((size_t)qcap * sizeof(gb_qhit)) < 0)
        return set_err(GB_ENOMEM, "cannot allocate %lld-ray work queues", qcap);
    P.qcap = qcap;
    g_qcap = qcap;
    P.hits = (gb_qhit *)G->hitrec.p;
    const int nslots = (int)(G->mat.size() / 2);
    if (grad) {
        if (G->adja.ensure((size_t)qcap * sizeof(gb_qadj)) < 0 || G->adjb.ensure((size_t)qcap * sizeof(gb_qadj)) < 0 ||
            G->dlde.ensure((size_t)n * 3 * sizeof(double)) < 0 || G->gradd.ensure((size_t)nslots * 3 * sizeof(double)) < 0)
            return set_err(GB_ENOMEM, "cannot allocate the gradient buffers");
        CK(cudaMemcpyAsync(G->dlde.p, out.dlde, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(G->gradd.p, 0, (size_t)nslots * 3 * sizeof(double), st));
        P.dlde = (const double *)G->dlde.p;
        P.grad = (double *)G->gradd.p;
        P.nslots = nslots;
    }
    if (G->H.ninst > 0) {                        /* walks that met an instance */
        if (G->slow.ensure((size_t)qcap * sizeof(unsigned int)) < 0)
            return set_err(GB_ENOMEM, "cannot allocate the instance walk list");
        P.slow = (unsigned int *)G->slow.p;
        P.slow_count = (unsigned long long *)G->qcount.p + 3;
    }
    uint32_t *tags[2] = {nullptr, nullptr};
    if (ss > 0) {
        const size_t nn = (size_t)n0 * n0;
        if (G->tga.ensure((size_t)qcap * sizeof(uint32_t)) < 0 || G->tgb.ensure((size_t)qcap * sizeof(uint32_t)) < 0 ||
            G->ssval.ensure((size_t)n * nn * 3 * sizeof(double)) < 0 ||
            G->sscnt.ensure((size_t)n * nn * sizeof(int)) < 0 || G->sserr.ensure((size_t)n * nn * 2 * sizeof(float)) < 0)
            return set_err(GB_ENOMEM, "cannot allocate the super-sampling buffers");
        CK(cudaMemsetAsync(G->ssval.p, 0, (size_t)n * nn * 3 * sizeof(double), st));
        CK(cudaMemsetAsync(G->sscnt.p, 0, (size_t)n * nn * sizeof(int), st));
        tags[0] = (uint32_t *)G->tga.p;
        tags[1] = (uint32_t *)G->tgb.p;
        P.ss_samples = o->as;
        P.ss_val = (double *)G->ssval.p;
        P.ss_cnt = (int *)G->sscnt.p;
        P.ss_err = (float *)G->sserr.p;
    }
    auto walk = [&](gb_run &R) -> int {
        return launch(GB_K_TRACE, R, [&](gb_run &Q) { return gb_launch_trace(&Q, st, G->sms); });
    };
    gb_qadj *adja = (gb_qadj *)G->adja.p, *adjb = (gb_qadj *)G->adjb.p;
    unsigned long long *cnt = (unsigned long long *)G->qcount.p;   /* [0] A, [1] B, [2] work items */
    CK(cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), st));
    P.work = cnt + 2;
    gb_qray *qa = (gb_qray *)G->qa.p, *qb = (gb_qray *)G->qb.p;

    /* the first generation's queue: -I hemisphere rays or primaries */
    P.qout = qa;
    P.qout_count = cnt;
    P.adj_out = adja;
    P.tag_out = tags[0];
    CK(cudaEventRecord(G->ev[0], st));
    if (o->I) {
        if (n0 > 0) {
            if (G->roots.ensure((size_t)n * sizeof(gb_rootrec)) < 0 ||
                G->rootspt.ensure((size_t)n * n0 * n0 * sizeof(float2)) < 0 ||
                (n0 >= 4 && (G->rootdraw.ensure((size_t)n * n0 * n0 * sizeof(float2)) < 0 ||
                             G->rootlot.ensure((size_t)n * 2 * GB_XLOT * sizeof(float)) < 0)))
                return set_err(GB_ENOMEM, "device allocation failed");
            P.roots = (gb_rootrec *)G->roots.p;
            P.root_spt = (float2 *)G->rootspt.p;
            P.root_draw = (float2 *)G->rootdraw.p;
            P.root_lot = (float *)G->rootlot.p;
        }
        P.root_n = n0;
        int rc = launch(GB_K_ROOT, P, [&](gb_run &R) {
            return grad ? gb_launch_root_grad(&R, st, G->sms) : gb_launch_root(&R, st, G->sms); });
        if (rc < 0)
            return rc;
        if (n0 >= 4) {                           /* the placement of the first hemispheres */
            rc = launch(GB_K_ROOT, P, [&](gb_run &R) { return gb_launch_root_draws(&R, st, G->sms); });
            if (rc < 0)
                return rc;
            rc = launch(GB_K_ROOT, P, [&](gb_run &R) { return gb_launch_root_place(&R, st, G->sms); });
            if (rc < 0)
                return rc;
        }
        if (n0 > 0) {
            rc = launch(GB_K_EXPAND, P, [&](gb_run &R) {
                return grad ? gb_launch_expand_root_grad(&R, st, G->sms) : gb_launch_expand_root(&R, st, G->sms); });
            if (rc < 0)
                return rc;
        }
    } else {
        int rc = launch(GB_K_PRIMARY, P, [&](gb_run &R) {
            return grad ? gb_launch_primary_grad(&R, st, G->sms) : gb_launch_primary(&R, st, G->sms); });
        if (rc < 0)
            return rc;
    }
    /* generations until the queue drains: walk, then shade into the other queue */
    int in = 0;
    auto drain = [&]() -> int {
        for (int gen = 0; gen < GB_MAX_GENERATIONS; gen++) {
            unsigned long long c = 0;
            CK(cudaMemcpyAsync(&c, cnt + in, sizeof c, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (c == 0)
                break;
            if ((long long)c > g_maxgen)
                g_maxgen = (long long)c;
            if ((long long)c > qcap)
                return set_err(GB_EOVERFLOW, "ray queue overflow (%llu rays for %lld slots)", c, qcap);
            P.qin = in ? qb : qa;
            P.qin_count = cnt + in;
            P.qout = in ? qa : qb;
            P.qout_count = cnt + (1 - in);
            P.adj_in = in ? adjb : adja;
            P.adj_out = in ? adja : adjb;
            P.tag_in = tags[in];
            P.tag_out = tags[1 - in];
            CK(cudaMemsetAsync(cnt + (1 - in), 0, sizeof(unsigned long long), st));
            CK(cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st));
            if (P.slow_count)
                CK(cudaMemsetAsync(P.slow_count, 0, sizeof(unsigned long long), st));
            int rc = walk(P);
            if (rc < 0)
                return rc;
            CK(cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st));
            rc = launch(GB_K_SHADE, P, [&](gb_run &R) {
                return grad ? gb_launch_shade_grad(&R, st, G->sms) : gb_launch_shade(&R, st, G->sms); });
            if (rc < 0)
                return rc;
            CK(cudaMemsetAsync(cnt + in, 0, sizeof(unsigned long long), st));
            in = 1 - in;
        }
        return GB_OK;
    };
    /* Batched runs capture the generations in a CUDA graph: the kernels
     * read each queue's count on the device, so no generation waits for
     * the host.  Paths are at most -lr bounces long, so -lr + 3 generations
     * drain the queue; whatever is left (none, when -lr bounds the paths)
     * is drained by the host loop below, which then finds the queue empty
     * at once. */
    if (G->use_graph && o->lr > 0 && ss == 0 && !grad && G->H.ninst == 0) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        capturing = true;
        int rc = GB_OK;
        for (int gen = 0; gen < o->lr + 3 && rc == GB_OK; gen++) {
            P.qin = in ? qb : qa;
            P.qin_count = cnt + in;
            P.qout = in ? qa : qb;
            P.qout_count = cnt + (1 - in);
            P.adj_in = in ? adjb : adja;
            P.adj_out = in ? adja : adjb;
            P.tag_in = tags[in];
            P.tag_out = tags[1 - in];
            if (cudaMemsetAsync(cnt + (1 - in), 0, sizeof(unsigned long long), st) != cudaSuccess ||
                cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st) != cudaSuccess)
                rc = set_err(GB_ECUDA, "graph capture: %s", cudaGetErrorString(cudaGetLastError()));
            if (rc == GB_OK)
                rc = walk(P);
            if (rc == GB_OK && cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st) != cudaSuccess)
                rc = set_err(GB_ECUDA, "graph capture: %s", cudaGetErrorString(cudaGetLastError()));
            if (rc == GB_OK)
                rc = launch(GB_K_SHADE, P, [&](gb_run &R) { return gb_launch_shade(&R, st, G->sms); });
            if (rc == GB_OK && cudaMemsetAsync(cnt + in, 0, sizeof(unsigned long long), st) != cudaSuccess)
                rc = set_err(GB_ECUDA, "graph capture: %s", cudaGetErrorString(cudaGetLastError()));
            in = 1 - in;
        }
        capturing = false;
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc == GB_OK && e != cudaSuccess)
            rc = set_err(GB_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        if (rc == GB_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
            rc = set_err(GB_ECUDA, "graph instantiation: %s", cudaGetErrorString(cudaGetLastError()));
        if (rc == GB_OK && cudaGraphLaunch(exec, st) != cudaSuccess)
            rc = set_err(GB_ECUDA, "graph launch: %s", cudaGetErrorString(cudaGetLastError()));
        if (exec)
            cudaGraphExecDestroy(exec);            /* freed once the launch completes */
        if (graph)
            cudaGraphDestroy(graph);
        if (rc < 0)
            return rc;
    }
    int drc = drain();
    if (drc < 0)
        return drc;
    if (ss > 0) {
        /* the extra samples of the first hemispheres, queued into the
         * drained queue and traced as a second pass, then every stratum's
         * mean into its sensor */
        P.qout = in ? qb : qa;
        P.qout_count = cnt + in;
        P.tag_out = tags[in];
        int rc = launch(GB_K_ROOT, P, [&](gb_run &R) { return gb_launch_ssamp_plan(&R, st, G->sms); });
        if (rc < 0)
            return rc;
        drc = drain();
        if (drc < 0)
            return drc;
        rc = launch(GB_K_ROOT, P, [&](gb_run &R) { return gb_launch_ssamp_final(&R, st, G->sms); });
        if (rc < 0)
            return rc;
    }
    CK(cudaEventRecord(G->ev[1], st));
    unsigned long long stats[GB_K_N][GB_ST_N];
    CK(cudaMemcpyAsync(stats, G->stats.p, sizeof stats, cudaMemcpyDeviceToHost, st));
    if (out.value)
        CK(cudaMemcpyAsync(out.value, G->value.p, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    /* the bins come back through pinned staging (a copy from pageable
     * memory is staged by the driver at a fraction of the link's rate),
     * then into the caller's buffer */
    const size_t binbytes = out.bins && nrec > 0 ? (size_t)nrec * nbins_total * 3 * sizeof(double) : 0;
    bool bins_staged = false;
    if (binbytes) {
        if (G->pinb_n < binbytes) {
            if (G->pinb)
                cudaFreeHost(G->pinb);
            G->pinb = nullptr;
            G->pinb_n = 0;
            if (cudaHostAlloc(&G->pinb, binbytes, cudaHostAllocDefault) == cudaSuccess)
                G->pinb_n = binbytes;
            else {
                cudaGetLastError();
                G->pinb = nullptr;
            }
        }
        bins_staged = G->pinb != nullptr;
        CK(cudaMemcpyAsync(bins_staged ? G->pinb : (void *)out.bins, G->bins.p, binbytes, cudaMemcpyDeviceToHost, st));
    }
    if (grad)
        CK(cudaMemcpyAsync(out.grad, G->gradd.p, (size_t)nslots * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (bins_staged) {                        /* large copies split over host threads */
        const int nt = binbytes >= ((size_t)8 << 20) ? 8 : 1;
        std::vector<std::thread> th;
        const size_t per = (binbytes / nt + 63) & ~(size_t)63;
        for (int k = 1; k < nt; k++) {
            const size_t a0 = per * k;
            if (a0 < binbytes)
                th.emplace_back([&, a0]() {
                    memcpy((char *)out.bins + a0, (const char *)G->pinb + a0, std::min(per, binbytes - a0));
                });
        }
        memcpy(out.bins, G->pinb, std::min(per, binbytes));
        for (auto &x : th)
            x.join();
    }
    if (unpack_hits)
        unpack_hits();
    unsigned long long overflow = 0;
    for (int k = 0; k < GB_K_N; k++) {
        g_stats[0] += (int64_t)stats[k][GB_ST_RAYS];
        g_stats[1] += (int64_t)stats[k][GB_ST_STEPS];
        g_stats[2] += (int64_t)stats[k][GB_ST_CONTRIB];
        overflow += stats[k][GB_ST_OVERFLOW];
        for (int c = 0; c < GB_ST_N; c++)
            g_prof.st[k][c] += stats[k][c];
    }
    for (int s = 0; 2 + 2 * s + 1 < evused; s++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, G->ev[2 + 2 * s], G->ev[3 + 2 * s]);
        g_prof.ms[evkid[s]] += ms;
    }
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, G->ev[0], G->ev[1]);
        g_prof.region_ms += ms;
    }
    if (overflow)
        return set_err(GB_EOVERFLOW, "ray queue overflow (%llu records dropped)", overflow);
    return GB_OK;
}

/* Queue slots per sensor that run() sizes for (the first generation's
 * fan-out times four), or the pilot's measurement. */
static double slots_per_sensor(const gb_scene *G, const gb_opts *o)
{
    int n0 = (o->I && o->ab > 0 && o->ad > 0) ? root_divisions(o) : 0;
    double per = n0 > 0 ? (double)n0 * n0 * 4 : (o->ab > 0 ? (double)o->ad * 2 : 8.0);
    return fmax(per, 4.0 * supersamples(o, n0));    /* the second pass of super-sampled runs */
}

/* run() over slices of at most as many sensors as keep the work buffers
 * within a quarter of free device memory (and 8 GB): the random streams are
 * keyed by the index in the whole set, so the result is that of one run.
 * Slices of -c records stay whole.  per_sensor: queue slots per sensor
 * (0: run()'s estimate). */
static int run_sliced(gb_scene *G, const gb_opts *o, int follow, const double *org_dir, int64_t n,
                      const std::vector<gb_binins> *prog, const std::vector<int4> *modinfo, int nbins_total,
                      const std::vector<int> *trk, RunOut out, double per_sensor)
{
    const int64_t acc = o->c > 0 ? o->c : 1;
    const bool grad = out.grad != nullptr;
    const size_t slot = 2 * sizeof(gb_qray) + sizeof(gb_qhit) + (grad ? 2 * sizeof(gb_qadj) : 0);
    if (per_sensor <= 0)
        per_sensor = slots_per_sensor(G, o);
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    double budget = fmin((double)freeb / 4.0, 8e9);
    int64_t chunk = (int64_t)(budget / (per_sensor * (double)slot));
    chunk = chunk / acc * acc;
    if (chunk < acc)
        chunk = acc;
    if (chunk >= n)
        return run(G, o, follow, org_dir, n, prog, modinfo, nbins_total, trk, out,
                   (long long)(per_sensor * (double)n) + (1ll << 16), 0);
    const int nslots = (int)G->matobj.size();
    std::vector<double> gsum(grad ? (size_t)nslots * 3 : 0), gpart(gsum.size());
    long long maxgen = 0;
    for (int64_t b = 0; b < n; b += chunk) {
        const int64_t m = n - b < chunk ? n - b : chunk;
        RunOut so = out;
        if (out.value) so.value = out.value + 3 * b;
        if (out.bins) so.bins = out.bins + (size_t)(b / acc) * nbins_total * 3;
        if (out.hit_id) so.hit_id = out.hit_id + b;
        if (out.hit_t) so.hit_t = out.hit_t + b;
        if (out.hit_normal) so.hit_normal = out.hit_normal + 3 * b;
        if (grad) {
            so.dlde = out.dlde + 3 * b;
            so.grad = gpart.data();
        }
        int rc = run(G, o, follow, org_dir + 6 * b, m, prog, modinfo, nbins_total, trk, so,
                     (long long)(per_sensor * (double)m) + (1ll << 16), b);
        if (rc < 0)
            return rc;
        if (g_maxgen > maxgen) maxgen = g_maxgen;
        for (size_t i = 0; i < gsum.size(); i++) gsum[i] += gpart[i];
    }
    g_maxgen = maxgen;
    if (grad)
        memcpy(out.grad, gsum.data(), gsum.size() * sizeof(double));
    return GB_OK;
}

extern "C" int gb_rtrace(gb_scene *G, const gb_opts *o, const double *org_dir, int64_t n, double *out_rgb,
                         int32_t *hit_id, double *hit_t)
{
    if (!G || !o || (!org_dir && n > 0))
        return set_err(GB_EINVAL, "null argument");
    if (out_rgb) {
        int rc = check_shading(G, o);
        if (rc < 0)
            return rc;
    }
    RunOut out = {out_rgb, nullptr, hit_id, hit_t, nullptr, nullptr, nullptr};
    double per = 0.0;
    int rc = GB_OK;
    for (int attempt = 0; attempt < 4; attempt++) {
        rc = run_sliced(G, o, 0, org_dir, n, nullptr, nullptr, 0, nullptr, out, per);
        if (rc != GB_EOVERFLOW)
            break;
        per = 2 * (per > 0 ? per : slots_per_sensor(G, o));   /* a larger queue, fewer sensors per slice */
    }
    return rc;
}

extern "C" int gb_rtrace_hits(gb_scene *G, const gb_opts *o, const double *org_dir, int64_t n, int32_t *hit_id,
                              double *hit_t, double *hit_normal, double *hit_pnormal, double *hit_uv)
{
    if (!G || !o || (n > 0 && (!org_dir || !hit_id || !hit_normal)))
        return set_err(GB_EINVAL, "null argument");
    std::vector<double> vn(hit_pnormal && G->has_vnorm ? (size_t)n * 3 : 0);
    RunOut out = {nullptr, nullptr, hit_id, hit_t, nullptr, nullptr, hit_normal, vn.empty() ? nullptr : vn.data(),
                  hit_uv};
    int rc = run_sliced(G, o, 0, org_dir, n, nullptr, nullptr, 0, nullptr, out, 0.0);
    if (rc < 0 || !hit_pnormal)
        return rc;
    /* the shading normal (rt/rtrace.c:807-820 oputn): plastic, metal,
     * trans (rt/normal.c:200-207, with back faces visible) and glass
     * (rt/glass.c:88-89) turn a surface hit from behind toward the ray
     * (flipsurface); the other materials leave it.  A smooth mesh hit's
     * normal is perturbed toward its interpolated vertex normal
     * (rt/o_mesh.c:198-206), the result oriented as the surface is toward
     * the ray (rt/raytrace.c:446-478 raynormal) */
    for (int64_t i = 0; i < n; i++) {
        const double *N = hit_normal + 3 * i, *d0 = org_dir + 6 * i + 3;
        double *pn = hit_pnormal + 3 * i;
        double dl = sqrt(d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2]);
        const double d[3] = {dl > 0 ? d0[0] / dl : 0.0, dl > 0 ? d0[1] / dl : 0.0, dl > 0 ? d0[2] / dl : 0.0};
        double rod = -(d[0] * N[0] + d[1] * N[1] + d[2] * N[2]);
        bool flip = false;
        const int32_t h = hit_id[i];
        if (h >= 0 && h < G->H.nobjs && rod < 0.0) {
            const int32_t m = gb_find_material(&G->H, h);
            const int t = m >= 0 ? G->H.objs[m].otype : -1;
            flip = t == GT_GLASS || (o->bv && (t == GT_PLASTIC || t == GT_METAL || t == GT_TRANS));
        }
        const double *V = vn.empty() ? nullptr : vn.data() + 3 * i;
        double pert2 = 0.0;
        if (V)
            for (int k = 0; k < 3; k++)
                pert2 += (V[k] - N[k]) * (V[k] - N[k]);
        if (V && (V[0] != 0.0 || V[1] != 0.0 || V[2] != 0.0) && pert2 > GB_FTINY * GB_FTINY) {
            double nm[3], r2 = flip ? -rod : rod;
            for (int k = 0; k < 3; k++)
                nm[k] = flip ? -V[k] : V[k];                 /* ron + pert, after any flip */
            double nd = -(nm[0] * d[0] + nm[1] * d[1] + nm[2] * d[2]);
            if ((nd > 0.0) != (r2 > 0.0))
                for (int k = 0; k < 3; k++)
                    nm[k] += 2.0 * nd * d[k];
            for (int k = 0; k < 3; k++)
                pn[k] = nm[k];
        } else
            for (int k = 0; k < 3; k++)
                pn[k] = flip ? -N[k] : N[k];
    }
    return GB_OK;
}

extern "C" int gb_rtrace_grad(gb_scene *G, const gb_opts *o, const double *org_dir, int64_t n,
                              const double *dl_dvalue, double *grad, int64_t nslots)
{
    if (!G || !o || (n > 0 && (!org_dir || !dl_dvalue)) || !grad)
        return set_err(GB_EINVAL, "null argument");
    if (G->has_vnorm)
        return set_err(GB_EUNSUPPORTED, "gradients in scenes with mesh triangles with vertex normals are not "
                       "implemented");
    if (nslots != (int64_t)G->matobj.size())
        return set_err(GB_EINVAL, "the gradient has %lld material slots, the scene %lld", (long long)nslots,
                       (long long)G->matobj.size());
    for (size_t sl = 0; sl < G->matobj.size(); sl++)
        if ((int)G->mat[2 * sl].x == DM_TRANS || (int)G->mat[2 * sl].x == DM_MIRROR)
            return set_err(GB_EUNSUPPORTED, "gradients through trans and mirror materials (\"%s\") are not "
                           "implemented", G->H.objs[G->matobj[sl]].name);
    int rc = check_shading(G, o);
    if (rc < 0)
        return rc;
    memset(grad, 0, (size_t)nslots * 3 * sizeof(double));
    if (nslots == 0)
        return GB_OK;
    RunOut out = {nullptr, nullptr, nullptr, nullptr, dl_dvalue, grad, nullptr};
    return run_sliced(G, o, 0, org_dir, n, nullptr, nullptr, 0, nullptr, out, 0.0);
}

extern "C" int64_t gb_scene_material_slots(const gb_scene *G) { return G ? (int64_t)G->matobj.size() : 0; }

extern "C" int gb_scene_material_slot(const gb_scene *G, const char *name, int *slot)
{
    if (!G || !name || !slot)
        return set_err(GB_EINVAL, "null argument");
    for (size_t sl = 0; sl < G->matobj.size(); sl++)
        if (!strcmp(G->H.objs[G->matobj[sl]].name, name)) {
            *slot = (int)sl;
            return GB_OK;
        }
    return set_err(GB_EINVAL, "no material '%s' in the scene", name);
}

extern "C" int gb_scene_material_rgb(gb_scene *G, int slot, double *get_rgb, const double *set_rgb)
{
    if (!G || slot < 0 || slot >= (int)G->matobj.size())
        return set_err(GB_EINVAL, "bad material slot %d", slot);
    float4 &m0 = G->mat[2 * (size_t)slot];
    if (get_rgb) {
        get_rgb[0] = m0.y;
        get_rgb[1] = m0.z;
        get_rgb[2] = m0.w;
    }
    if (set_rgb) {
        m0.y = (float)set_rgb[0];
        m0.z = (float)set_rgb[1];
        m0.w = (float)set_rgb[2];
        if (G->matd.p)
            CK(cudaMemcpy((float4 *)G->matd.p + 2 * (size_t)slot, &m0, sizeof(float4), cudaMemcpyHostToDevice));
    }
    return GB_OK;
}

static int compile_mods(gb_scene *G, const gb_modspec *mods, int nmods, std::vector<gb_binins> &prog,
                        std::vector<int4> &info, std::vector<int> *trk, int *nbins_total)
{
    int total = 0;
    prog.clear();
    info.clear();
    if (trk)
        trk->assign(G ? (G->H.nobjs > 0 ? G->H.nobjs : 1) : 0, -1);
    for (int m = 0; m < nmods; m++) {
        std::vector<gb_binins> p;
        std::string err;
        int nb = 0;
        if (!mods[m].modifier)
            return set_err(GB_EINVAL, "modifier %d has no name", m);
        if (gb_compile_bin(mods[m].binv, mods[m].params, mods[m].calfile, mods[m].expr, mods[m].nbins, p, &nb,
                           err) < 0)
            return set_err(GB_EUNSUPPORTED, "modifier '%s': %s", mods[m].modifier, err.c_str());
        for (int k = 0; k < m; k++)
            if (!strcmp(mods[k].modifier, mods[m].modifier))
                return set_err(GB_EINVAL, "duplicate modifier '%s'", mods[m].modifier);
        if (!strcmp(mods[m].modifier, "void"))
            return set_err(GB_EINVAL, "cannot track 'void' modifier");
        info.push_back(make_int4((int)prog.size(), nb, total, 0));
        prog.insert(prog.end(), p.begin(), p.end());
        total += nb;
        if (trk && G) {
            for (int32_t i = 0; i < G->H.nobjs; i++) {
                int32_t mo = G->H.objs[i].omod;
                if (mo >= 0 && !strcmp(G->H.objs[mo].name, mods[m].modifier))
                    (*trk)[i] = m;
            }
        }
    }
    *nbins_total = total;
    return GB_OK;
}

extern "C" int gb_rcontrib_nbins(const gb_modspec *mods, int nmods, int *nbins_total)
{
    std::vector<gb_binins> prog;
    std::vector<int4> info;
    return compile_mods(nullptr, mods, nmods, prog, info, nullptr, nbins_total);
}

/* one rcontrib run on one scene: options overridden as rcmain does, bin
 * programs compiled for the scene's modifiers; a queue that overflows is
 * enlarged and the run repeated (the random streams make it identical) */
static int rcontrib_run(gb_scene *G, const gb_opts *o, const gb_modspec *mods, int nmods, const double *org_dir,
                        int64_t n, double *out, int64_t *ray_count, double per_sensor)
{
    gb_opts oo = *o;
    /* rt/rcmain.c:164-172 override_options */
    oo.dt = 0;
    oo.as = 0;
    oo.aa = 0;
    int rc = check_shading(G, &oo);
    if (rc < 0)
        return rc;
    std::vector<gb_binins> prog;
    std::vector<int4> info;
    std::vector<int> trk;
    int nbt = 0;
    rc = compile_mods(G, mods, nmods, prog, info, &trk, &nbt);
    if (rc < 0)
        return rc;
    if (oo.V) {
        /* contributions need the radiance of the tracked surface, which is
         * local only for light sources */
        for (int32_t i = 0; i < G->H.nobjs; i++) {
            if (trk[i] < 0) continue;
            int ms = G->matslot[i];
            int k = ms >= 0 ? (int)G->mat[2 * ms].x : DM_NONE;
            if (k != DM_LIGHT && k != DM_GLOW)
                return set_err(GB_EUNSUPPORTED, "-V with a non-emitting tracked modifier is not implemented");
        }
    }
    RunOut ro = {nullptr, out, nullptr, nullptr, nullptr, nullptr};
    double per = per_sensor;
    for (int attempt = 0; attempt < 4; attempt++) {
        rc = run_sliced(G, &oo, 1, org_dir, n, &prog, &info, nbt, &trk, ro, per);
        if (rc != GB_EOVERFLOW)
            break;
        per = 2 * (per > 0 ? per : slots_per_sensor(G, &oo));   /* a larger queue, fewer sensors per slice */
    }
    if (ray_count)
        *ray_count = g_stats[0];
    if (rc == GB_OK && oo.c > 1) {
        int64_t nrec = n / oo.c;
        double sf = 1.0 / oo.c;
        for (int64_t i = 0; i < nrec * nbt * 3; i++)
            out[i] *= sf;
    }
    return rc;
}

extern "C" int gb_rcontrib(gb_scene *G, const gb_opts *o, const gb_modspec *mods, int nmods,
                           const double *org_dir, int64_t n, double *out, int64_t *ray_count)
{
    if (!G || !o || !mods || nmods <= 0 || (!org_dir && n > 0) || !out)
        return set_err(GB_EINVAL, "null argument or no modifiers");
    return rcontrib_run(G, o, mods, nmods, org_dir, n, out, ray_count, 0.0);
}

/* The tuner of a scene's runs, from pilot runs over 1,024 of the run's
 * sensors (evenly spaced): the queue slots per sensor (the largest
 * generation per sensor, with a margin), then the walk kernel's shape --
 * the idle lanes a warp waits for before refilling them, and the resident
 * blocks per SM -- of five candidates, each timed twice on the pilot
 * (the walk's device milliseconds, CUDA events), the fastest kept.  Kept
 * per scene and option set so that later calls skip the pilots.  0 (run()'s
 * estimate and the default shape) for n <= 4,096. */
static double tune_slots(gb_scene *G, const gb_opts *o, const gb_modspec *mods, int nmods, const double *org_dir,
                         int64_t n, int nbt)
{
    const int64_t m = 1024;
    if (n <= 4 * m)
        return 0.0;
    char key[256];
    snprintf(key, sizeof key, "%d %d %g %d %g %d %d", o->ab, o->ad, o->lw, o->lr, o->dj, o->I, o->c);
    if (G->tuned_key == key)
        return G->tuned_per_sensor;
    int64_t stride = n / m, acc = o->c > 0 ? o->c : 1;
    std::vector<double> sample;
    sample.reserve((size_t)m * acc * 6);
    for (int64_t i = 0; i < m; i++)                 /* whole records of -c sensors */
        for (int64_t j = 0; j < acc; j++) {
            int64_t s = (i * stride / acc) * acc + j;
            if (s >= n) s = n - 1;
            sample.insert(sample.end(), org_dir + 6 * s, org_dir + 6 * s + 6);
        }
    int64_t ns = (int64_t)(sample.size() / 6);
    std::vector<double> scratch((size_t)(ns / acc + 1) * nbt * 3);
    int64_t rays = 0;
    G->tuned_refill = G->tuned_blocks = 0;
    if (rcontrib_run(G, o, mods, nmods, sample.data(), ns, scratch.data(), &rays, 0.0) != GB_OK || g_maxgen <= 0)
        return 0.0;
    const double per = 1.5 * (double)g_maxgen / (double)ns;
    static const int shapes[][2] = {{8, 0}, {4, 0}, {16, 0}, {8, 3}, {8, 2}};
    double best = 1e30;
    int br = 0, bb = 0;
    for (int rep = 0; rep < 2; rep++)
        for (const auto &sh : shapes) {
            G->tuned_refill = sh[0];
            G->tuned_blocks = sh[1];
            if (rcontrib_run(G, o, mods, nmods, sample.data(), ns, scratch.data(), &rays, per) != GB_OK)
                continue;
            if (g_prof.ms[GB_K_TRACE] > 0 && g_prof.ms[GB_K_TRACE] < best) {
                best = g_prof.ms[GB_K_TRACE];
                br = sh[0];
                bb = sh[1];
            }
        }
    G->tuned_refill = br;
    G->tuned_blocks = bb;
    G->tuned_key = key;
    G->tuned_per_sensor = per;
    return G->tuned_per_sensor;
}

extern "C" int gb_rcontrib_batch(int njobs, gb_scene *const *scenes, const gb_opts *o, const gb_modspec *mods,
                                 int nmods, const double *const *org_dir, const int64_t *n, double *const *out,
                                 int64_t *ray_count)
{
    if (njobs < 0 || (njobs > 0 && (!scenes || !org_dir || !n || !out)) || !o || !mods || nmods <= 0)
        return set_err(GB_EINVAL, "null argument or no modifiers");
    const int64_t acc = o->c > 0 ? o->c : 1;
    int nbt = 0;
    {
        std::vector<gb_binins> prog;
        std::vector<int4> info;
        int rc = compile_mods(nullptr, mods, nmods, prog, info, nullptr, &nbt);
        if (rc < 0)
            return rc;
    }
    /* jobs grouped by scene; each group is one run over its jobs' sensors */
    std::vector<gb_scene *> order;
    std::vector<std::vector<int>> groups;
    for (int j = 0; j < njobs; j++) {
        if (!scenes[j] || (n[j] > 0 && (!org_dir[j] || !out[j])) || n[j] < 0)
            return set_err(GB_EINVAL, "job %d: null scene, rays or output", j);
        if (n[j] % acc)
            return set_err(GB_EINVAL, "job %d: %lld rays is not a multiple of -c %lld", j, (long long)n[j],
                           (long long)acc);
        size_t g = 0;
        while (g < order.size() && order[g] != scenes[j]) g++;
        if (g == order.size()) {
            order.push_back(scenes[j]);
            groups.emplace_back();
        }
        groups[g].push_back(j);
    }
    /* generation loops captured in CUDA graphs (GB_GRAPHS=0: host loop) */
    const char *gv = getenv("GB_GRAPHS");
    const bool graphs = !(gv && !strcmp(gv, "0"));
    std::vector<int> rcs(order.size(), GB_OK);
    std::vector<int64_t> rays(order.size(), 0);
    std::vector<std::string> errs(order.size());
    auto work = [&](size_t g) {
        gb_scene *G = order[g];
        int64_t tot = 0;
        for (int j : groups[g]) tot += n[j];
        std::vector<double> in((size_t)tot * 6), res((size_t)(tot / acc) * nbt * 3);
        int64_t at = 0;
        for (int j : groups[g]) {
            if (n[j])
                memcpy(in.data() + 6 * at, org_dir[j], (size_t)n[j] * 6 * sizeof(double));
            at += n[j];
        }
        double per = tune_slots(G, o, mods, nmods, in.data(), tot, nbt);
        G->use_graph = graphs;
        rcs[g] = rcontrib_run(G, o, mods, nmods, in.data(), tot, res.data(), &rays[g], per);
        G->use_graph = false;
        errs[g] = g_error;
        if (rcs[g] != GB_OK)
            return;
        at = 0;
        for (int j : groups[g]) {
            const size_t rec = (size_t)(n[j] / acc) * nbt * 3;
            memcpy(out[j], res.data() + (size_t)(at / acc) * nbt * 3, rec * sizeof(double));
            at += n[j];
        }
    };
    /* scenes run concurrently, each on its own stream, so that one
     * scene's small last generations overlap another's large ones */
    std::vector<std::thread> th;
    for (size_t g = 1; g < order.size(); g++)
        th.emplace_back(work, g);
    if (!order.empty())
        work(0);
    for (auto &t : th)
        t.join();
    int64_t total = 0;
    for (size_t g = 0; g < order.size(); g++) {
        total += rays[g];
        if (rcs[g] != GB_OK)
            return set_err(rcs[g], "%s", errs[g].c_str());
    }
    if (ray_count)
        *ray_count = total;
    g_stats[0] = total;
    return GB_OK;
}

/* ------------------------------------------------- measurement of ceilings */

extern "C" int gb_probe_l2(int64_t table_bytes, int chase, double *gbps)
{
    if (!gbps || table_bytes < 64)
        return set_err(GB_EINVAL, "bad probe arguments");
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint32_t nrec = (uint32_t)(table_bytes / 64);
    float4 *table = nullptr;
    float *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GB_OK;
    do {
        if (cudaMalloc(&table, (size_t)nrec * 64) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess) {
            rc = set_err(GB_ENOMEM, "probe allocation failed");
            break;
        }
        /* random contents: the chase's next place comes from them */
        std::vector<float4> h((size_t)nrec * 4);
        uint32_t x = 2463534242u;
        for (auto &v : h) {
            float *f = &v.x;
            for (int k = 0; k < 4; k++) {
                x ^= x << 13;
                x ^= x >> 17;
                x ^= x << 5;
                uint32_t u = (x & 0x007fffffu) | 0x3f800000u;   /* a float in [1, 2) */
                memcpy(f + k, &u, 4);
            }
        }
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMemcpy(table, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            rc = set_err(GB_ECUDA, "probe set-up failed");
            break;
        }
        const int iters = 256;
        double best = 1e30;
        for (int rep = 0; rep < 6; rep++) {
            cudaEventRecord(e0, st);
            if (gb_launch_probe_l2(table, nrec, iters, chase, sink, st, sms) < 0) {
                rc = set_err(GB_ECUDA, "probe launch failed");
                break;
            }
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = set_err(GB_ECUDA, "probe failed");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep >= 2 && ms < best)
                best = ms;
        }
        if (rc == GB_OK)
            *gbps = (double)4 * sms * 256 * iters * 64 / (best / 1e3) / 1e9;
    } while (0);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(table);
    cudaFree(sink);
    return rc;
}

/* ------------------------------------------------------------- dctimestep */

extern "C" int gb_dctimestep_device(const float *d_dc, const float *d_sky, int64_t M, int64_t K, int64_t N,
                                    int mode, float *d_out, void *stream)
{
    std::string err;
    int rc = gb_dct_device(d_dc, d_sky, M, K, N, mode, d_out, (cudaStream_t)stream, err);
    if (rc < 0)
        return set_err(rc, "%s", err.c_str());
    return GB_OK;
}

extern "C" int gb_dctimestep(const float *dc, const float *sky, int64_t M, int64_t K, int64_t N, int mode,
                             float *out)
{
    if (!dc || !sky || !out || M <= 0 || K <= 0 || N <= 0)
        return set_err(GB_EINVAL, "bad matrix arguments");
    float *a = nullptr, *b = nullptr, *c = nullptr;
    size_t na = (size_t)M * K * 3, nb = (size_t)K * N * 3, nc = (size_t)M * N * 3;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = GB_OK;
    if (cudaMalloc(&a, na * 4) != cudaSuccess || cudaMalloc(&b, nb * 4) != cudaSuccess ||
        cudaMalloc(&c, nc * 4) != cudaSuccess) {
        rc = set_err(GB_ENOMEM, "cannot allocate matrices on the device");
    } else {
        cudaMemcpyAsync(a, dc, na * 4, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(b, sky, nb * 4, cudaMemcpyHostToDevice, st);
        rc = gb_dctimestep_device(a, b, M, K, N, mode, c, st);
        if (rc == GB_OK) {
            cudaMemcpyAsync(out, c, nc * 4, cudaMemcpyDeviceToHost, st);
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess)
                rc = set_err(GB_ECUDA, "dctimestep: %s", cudaGetErrorString(e));
        }
    }
    cudaFree(a);
    cudaFree(b);
    cudaFree(c);
    cudaStreamDestroy(st);
    return rc;
}

/* ------------------------------------------- rtrace without device allocation
 *
 * gb_rtrace_device_noalloc: the values of gb_rtrace for rays that are
 * already on the device, written to a device buffer, for callers that must
 * not allocate device memory while they run -- a service that reserved the
 * GPU's memory for its own pool when it started (a caching allocator holds
 * the rest, so an allocation inside a request fails or forces an eviction),
 * or a loop that shares the GPU with latency-bound streams, which
 * cudaMalloc and cudaFree stall because they synchronise the device.
 *
 * All working memory of a call -- the per-kernel counters, the queue
 * counters, the table of tracked modifiers (none for rtrace), the sensor
 * hemisphere records of -I, the two ray queues and the walk results -- is
 * carved from the one static device array below; the rays and the output
 * are the caller's.  The kernels are those of gb_rtrace, so results agree
 * with it up to the order of the FP64 atomic additions.  Everything is
 * enqueued on the caller's stream, so the call is ordered after whatever
 * the caller enqueued there to write the rays.
 */
#define GB_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)   /* 64 MiB per device */
#define GB_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];
static std::atomic<void *> g_noalloc_addr[GB_NOALLOC_MAX_DEVICES];

/* Device address of the scratch on the current device.  The first call on a
 * device looks it up (which loads this module there if it is not loaded
 * yet); later calls reuse the address for the life of the process, so a
 * cudaDeviceReset() of that device leaves it stale. */
static int noalloc_scratch(int dev, unsigned char **p)
{
    if (dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES)
        return set_err(GB_EUNSUPPORTED, "device %d: at most %d devices", dev, GB_NOALLOC_MAX_DEVICES);
    void *a = g_noalloc_addr[dev].load();
    if (!a) {
        cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
        if (e != cudaSuccess || !a)
            return set_err(GB_ECUDA, "scratch lookup on device %d failed: %s", dev, cudaGetErrorString(e));
        g_noalloc_addr[dev].store(a);
    }
    *p = (unsigned char *)a;
    return GB_OK;
}

static int on_device(const void *p, int dev)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

/* The launches of one call, all on stream st over the scratch at base. */
static int noalloc_run(gb_scene *G, const gb_opts *o, const double *d_org_dir, int64_t n, double *d_rgb,
                       cudaStream_t st, unsigned char *base, int n0, size_t stat_bytes, size_t nobj,
                       const size_t *off, long long qcap)
{
    unsigned long long *stats = (unsigned long long *)(base + off[0]);
    unsigned long long *cnt = (unsigned long long *)(base + off[1]);   /* [0] A, [1] B, [2] work items */
    int *trk = (int *)(base + off[2]);
    gb_qray *qa = (gb_qray *)(base + off[6]);
    gb_qray *qb = qa + qcap;
    gb_qhit *hits = (gb_qhit *)(qb + qcap);
    int rc;
    /* what must start at zero: the counters and the output, which the
     * kernels accumulate into; the table of tracked modifiers is all -1
     * (no modifier is tracked); queues and hemisphere records are written
     * before they are read */
    CK(cudaMemsetAsync(stats, 0, stat_bytes, st));
    CK(cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(trk, 0xff, nobj * sizeof(int), st));
    CK(cudaMemsetAsync(d_rgb, 0, (size_t)n * 3 * sizeof(double), st));

    gb_run P;
    memset(&P, 0, sizeof P);
    P.S = G->ds;
    P.S.trk = trk;
    P.ab = o->ab;
    P.ad = o->ad;
    P.minweight = (float)o->lw;
    P.maxdepth = o->lr;
    for (int j = 0; j < 3; j++) P.av[j] = (float)o->av[j];
    P.dstrsrc = (float)o->dj;
    P.srcsizerat = (float)o->ds;
    P.specthresh = (float)o->st;
    P.specjitter = (float)o->ss;
    P.do_irrad = o->i;
    P.contrib_mode = o->V;
    uint64_t seed = seed_of(o);
    P.k0 = (uint32_t)seed;
    P.k1 = (uint32_t)(seed >> 32);
    P.replica = o->replica;
    P.nsensors = n;
    P.sensors = d_org_dir;
    P.value = d_rgb;
    P.accum = 1;
    P.qcap = qcap;
    P.hits = hits;
    P.work = cnt + 2;
    auto go = [&](int kid, int (*fn)(const gb_run *, cudaStream_t, int)) -> int {
        P.stats = stats + kid * GB_ST_N;
        if (fn(&P, st, G->sms) < 0)
            return set_err(GB_ECUDA, "launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        g_stats[3]++;
        g_prof.launches[kid]++;
        return GB_OK;
    };
    if (o->I) {
        if (n0 > 0) {
            P.roots = (gb_rootrec *)(base + off[3]);
            P.root_spt = (float2 *)(base + off[4]);
            P.root_draw = (float2 *)(base + off[5]);
            P.root_lot = (float *)(base + off[7]);
        }
        P.root_n = n0;
        if ((rc = go(GB_K_ROOT, gb_launch_root)) < 0)
            return rc;
        if (n0 >= 4 && ((rc = go(GB_K_ROOT, gb_launch_root_draws)) < 0 || (rc = go(GB_K_ROOT, gb_launch_root_place)) < 0))
            return rc;
        if (n0 > 0) {
            P.qout = qa;
            P.qout_count = cnt;
            if ((rc = go(GB_K_EXPAND, gb_launch_expand_root)) < 0)
                return rc;
        }
    } else {
        P.qout = qa;
        P.qout_count = cnt;
        if ((rc = go(GB_K_PRIMARY, gb_launch_primary)) < 0)
            return rc;
    }
    int in = 0;
    for (int gen = 0; gen < GB_MAX_GENERATIONS; gen++) {
        unsigned long long c = 0;
        CK(cudaMemcpyAsync(&c, cnt + in, sizeof c, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (c == 0)
            break;
        if ((long long)c > g_maxgen)
            g_maxgen = (long long)c;
        if ((long long)c > qcap)
            return set_err(GB_EOVERFLOW, "ray queue overflow (%llu rays for %lld slots)", c, qcap);
        P.qin = in ? qb : qa;
        P.qin_count = cnt + in;
        P.qout = in ? qa : qb;
        P.qout_count = cnt + (1 - in);
        CK(cudaMemsetAsync(cnt + (1 - in), 0, sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st));
        if ((rc = go(GB_K_TRACE, gb_launch_trace)) < 0)
            return rc;
        CK(cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), st));
        if ((rc = go(GB_K_SHADE, gb_launch_shade)) < 0)
            return rc;
        CK(cudaMemsetAsync(cnt + in, 0, sizeof(unsigned long long), st));
        in = 1 - in;
    }
    unsigned long long hs[GB_K_N][GB_ST_N];
    CK(cudaMemcpyAsync(hs, stats, sizeof hs, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    unsigned long long overflow = 0;
    for (int k = 0; k < GB_K_N; k++) {
        g_stats[0] += (int64_t)hs[k][GB_ST_RAYS];
        g_stats[1] += (int64_t)hs[k][GB_ST_STEPS];
        g_stats[2] += (int64_t)hs[k][GB_ST_CONTRIB];
        overflow += hs[k][GB_ST_OVERFLOW];
        memcpy(g_prof.st[k], hs[k], sizeof hs[k]);
    }
    if (overflow)
        return set_err(GB_EOVERFLOW, "ray queue overflow (%llu records dropped)", overflow);
    return GB_OK;
}

extern "C" int gb_rtrace_device_noalloc(gb_scene *G, const gb_opts *o, const double *d_org_dir, int64_t n,
                                        double *d_rgb, void *stream)
{
    if (!G || !o || (n > 0 && (!d_org_dir || !d_rgb)) || n < 0)
        return set_err(GB_EINVAL, "null argument or negative ray count");
    g_stats[0] = g_stats[1] = g_stats[2] = g_stats[3] = 0;
    memset(&g_prof, 0, sizeof g_prof);
    int rc = check_shading(G, o);
    if (rc < 0)
        return rc;
    if (n == 0)
        return GB_OK;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (!on_device(G->ds.obj, dev))
        return set_err(GB_EINVAL, "the scene was loaded on another device than the current one (%d)", dev);
    if (!on_device(d_org_dir, dev) || !on_device(d_rgb, dev))
        return set_err(GB_EINVAL, "rays and output must be device memory of the current device (%d)", dev);
    unsigned char *base = nullptr;
    rc = noalloc_scratch(dev, &base);
    if (rc < 0)
        return rc;

    const int n0 = (o->I && o->ab > 0 && o->ad > 0) ? root_divisions(o) : 0;
    if (n0 > 128)
        return set_err(GB_EUNSUPPORTED, "-ad %d gives %d x %d hemisphere divisions; at most 128 x 128 are "
                       "supported", o->ad, n0, n0);
    if (G->H.ninst > 0)
        return set_err(GB_EUNSUPPORTED, "scenes with instances are not traced without allocation");
    if ((rc = check_supersampling(o, n0)) < 0)
        return rc;
    if (supersamples(o, n0) > 0)
        return set_err(GB_EUNSUPPORTED, "ambient super-sampling (-as %d) is not implemented without allocation; "
                       "use -as 0", o->as);

    /* every ray needs at least 8 queue slots of 160 bytes: larger counts
     * cannot fit, and rejecting them here keeps the sizes below from
     * overflowing */
    if (n > (int64_t)(GB_NOALLOC_SCRATCH_BYTES / 1024))
        return set_err(GB_EINVAL, "%lld rays need more than the %u MiB static scratch (trace fewer rays per "
                       "call)", (long long)n, (unsigned)(GB_NOALLOC_SCRATCH_BYTES >> 20));

    /* scratch layout, each part on a 256-byte boundary: [0] kernel counters,
     * [1] queue counters, [2] tracked-modifier table, [3] hemisphere records,
     * [4] placed samples, [5] placement draws, [7] collision lots, [6] the
     * two queues and the walk results (qcap slots each) */
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t stat_bytes = GB_K_N * GB_ST_N * sizeof(unsigned long long);
    const size_t nobj = G->H.nobjs > 0 ? (size_t)G->H.nobjs : 1;
    const size_t un = (size_t)n, nn0 = (size_t)n0 * (size_t)n0;
    size_t off[8];
    off[0] = 0;
    off[1] = up(stat_bytes);
    off[2] = off[1] + up(4 * sizeof(unsigned long long));
    off[3] = off[2] + up(nobj * sizeof(int));
    off[4] = off[3] + (n0 > 0 ? up(un * sizeof(gb_rootrec)) : 0);
    off[5] = off[4] + (n0 > 0 ? up(un * nn0 * sizeof(float2)) : 0);
    off[7] = off[5] + (n0 >= 4 ? up(un * nn0 * sizeof(float2)) : 0);
    off[6] = off[7] + (n0 >= 4 ? up(un * 2 * GB_XLOT * sizeof(float)) : 0);
    /* the queue need gb_rtrace sizes for, without its 1M-ray minimum, and
     * never less than 8 slots per ray */
    long long est = (long long)n * (n0 > 0 ? (long long)nn0 * 4 : (o->ab > 0 ? (long long)o->ad * 2 : 8));
    if (est < 8 * (long long)n)
        est = 8 * (long long)n;
    const size_t slot = 2 * sizeof(gb_qray) + sizeof(gb_qhit);   /* two queues and the walk results */
    long long qcap = off[6] < GB_NOALLOC_SCRATCH_BYTES ? (long long)((GB_NOALLOC_SCRATCH_BYTES - off[6]) / slot) : 0;
    if (off[6] >= GB_NOALLOC_SCRATCH_BYTES || est > qcap)
        return set_err(GB_EINVAL, "%lld rays with these options need %.1f MiB of scratch; the static scratch "
                       "is %u MiB (trace fewer rays per call)", (long long)n,
                       (off[6] + (double)est * slot) / 1048576.0, (unsigned)(GB_NOALLOC_SCRATCH_BYTES >> 20));
    qcap = (qcap / 4) * 4;
    if (off[6] + (size_t)qcap * slot > GB_NOALLOC_SCRATCH_BYTES)   /* cannot happen: qcap was cut to fit */
        return set_err(GB_EINVAL, "scratch layout exceeds the static array");

    cudaStream_t st = (cudaStream_t)stream;
    rc = noalloc_run(G, o, d_org_dir, n, d_rgb, st, base, n0, stat_bytes, nobj, off, qcap);
    if (rc < 0) {
        /* work may still be queued over the scratch and d_rgb: let it end
         * before returning, so the next call does not race with it */
        cudaStreamSynchronize(st);
        cudaGetLastError();
    }
    return rc;
}
