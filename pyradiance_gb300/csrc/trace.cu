/*
 * trace.cu -- the GB300 wavefront path engine behind rtrace and rcontrib.
 *
 * Work is organised by ray generation instead of by recursion:
 *   k_root         one thread per sensor: the -I "pretend hit" Lambertian at
 *                  the sensor (rt/rtrace.c:416-433, rt/rcontrib.c:321-338),
 *                  its direct component and its hemisphere's frame and size;
 *   k_root_draws   the random numbers of the first hemispheres' placement,
 *   k_root_place   and the placement itself, sequential per sensor;
 *   k_expand_root  the first generation: one ray per (sensor, stratum);
 *   k_primary      radiance mode: the sensor rays as the first generation;
 * then for every generation, from a queue of 64-byte ray records:
 *   k_trace        the octree walk of every ray (a 32-byte result each),
 *   k_shade        shading, contributions, and every child ray appended to
 *                  the next generation's queue (one atomic per coalesced
 *                  group).
 * Contributions are added to FP64 per-sensor values and per-record bins
 * with warp-aggregated atomics; gradient runs (k_*<true>) replay the same
 * rays and accumulate derivatives instead.
 *
 * Shading follows the reference: m_normal for plastic/metal with pure
 * specular reflection (rt/normal.c:177-360, dirnorm :72-173), m_glass
 * (rt/glass.c:45-165), m_light (rt/source.c:749-793), direct()
 * (rt/source.c:398-556, srcray :219, nextssamp rt/srcsamp.c:37-145 with a
 * single partition), the -aa 0 hemisphere (rt/ambient.c:269-297,
 * rt/ambcomp.c:177-250, 351-421) and rayorigin's weights and Russian
 * roulette (rt/raytrace.c:39-135).  rcontrib's trace callback
 * (rt/rcontrib.c:272-316) is applied to every traced ray.
 */
#include <type_traits>
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#include <algorithm>

#include "trace.cuh"
#include "tracehost.h"

namespace cg = cooperative_groups;

#define FRESTHRESH 0.017999f
__device__ __forceinline__ float fresne(float ci) { return expf(-5.85f * ci) - 0.00202943064f; }

/* stats slots */
/* stats slots: see tracehost.h (GB_ST_*) */
#define ST_RAYS GB_ST_RAYS
#define ST_STEPS GB_ST_STEPS
#define ST_CONTRIB GB_ST_CONTRIB
#define ST_OVERFLOW GB_ST_OVERFLOW
#define ST_BADBIN GB_ST_BADBIN

struct Ray {
    float3 org, dir, coef;
    float weight, lcoef;
    int origin, rsrc;
    uint32_t crtype;
    int rlvl, adepth;
    uint64_t path;
    uint32_t sensor;
    uint32_t tag;           /* super-sampled first-hemisphere stratum the path descends from, or GB_NOTAG */
    gb_qadj adj;            /* gradient runs only: parameter factors of the path */
};

struct Counters {
    unsigned long long rays, steps, nodes, tests, contrib;
    __device__ void add(const uint32_t t[3])
    {
        steps += t[0];
        nodes += t[1];
        tests += t[2];
    }
};

/* one atomic per thread and counter at the end of a kernel */
__device__ __forceinline__ void flush_counters(const gb_run &P, const Counters &c)
{
    if (c.rays) atomicAdd(P.stats + GB_ST_RAYS, c.rays);
    if (c.steps) atomicAdd(P.stats + GB_ST_STEPS, c.steps);
    if (c.nodes) atomicAdd(P.stats + GB_ST_NODES, c.nodes);
    if (c.tests) atomicAdd(P.stats + GB_ST_TESTS, c.tests);
    if (c.contrib) atomicAdd(P.stats + GB_ST_CONTRIB, c.contrib);
}

/* -------------------------------------------------------------- records */

__device__ __forceinline__ void store_ray(gb_qray *q, const Ray &r)
{
    float4 a = make_float4(r.org.x, r.org.y, r.org.z, r.weight);
    float4 b = make_float4(r.dir.x, r.dir.y, r.dir.z, r.lcoef);
    float4 c = make_float4(r.coef.x, r.coef.y, r.coef.z, __int_as_float(r.origin));
    uint4 d = make_uint4((uint32_t)r.path, (uint32_t)(r.path >> 32), r.sensor,
                         (r.crtype & 0xffff) | ((uint32_t)r.rlvl << 16) | ((uint32_t)r.adepth << 24));
    float4 *p = reinterpret_cast<float4 *>(q);
    p[0] = a;
    p[1] = b;
    p[2] = c;
    reinterpret_cast<uint4 *>(q)[3] = d;
}

__device__ __forceinline__ Ray load_ray(const gb_qray *q)
{
    const float4 *p = reinterpret_cast<const float4 *>(q);
    float4 a = p[0], b = p[1], c = p[2];
    uint4 d = reinterpret_cast<const uint4 *>(q)[3];
    Ray r;
    r.org = f3(a.x, a.y, a.z);
    r.weight = a.w;
    r.dir = f3(b.x, b.y, b.z);
    r.lcoef = b.w;
    r.coef = f3(c.x, c.y, c.z);
    r.origin = __float_as_int(c.w);
    r.path = (uint64_t)d.x | ((uint64_t)d.y << 32);
    r.sensor = d.z;
    r.crtype = d.w & 0xffff;
    r.rlvl = (d.w >> 16) & 0xff;
    r.adepth = (d.w >> 24) & 0xff;
    r.rsrc = -1;
    r.tag = GB_NOTAG;
    return r;
}

template <bool G = false>
__device__ __forceinline__ void push_ray(const gb_run &P, const Ray &r)
{
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0)
        base = atomicAdd(P.qout_count, (unsigned long long)g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if (base < (unsigned long long)P.qcap) {
        store_ray(P.qout + base, r);
        if (G)
            P.adj_out[base] = r.adj;
        if (P.tag_out)
            P.tag_out[base] = r.tag;
    } else if (g.thread_rank() == 0)
        atomicAdd(P.stats + ST_OVERFLOW, 1ull);
}

/* ------------------------------------------------------------ gradients
 *
 * A gradient run replays the forward run (same random streams, so the same
 * rays) and, wherever the forward adds a contribution v to a sensor's value,
 * adds w * v * d(ln f)/d(theta) for every parameter-dependent factor f on
 * the contribution's path, w being d(loss)/d(value) of that sensor: the
 * diffuse reflectance of each plastic or metal bounce (f = rho, so
 * d ln f / d rho = 1 / rho) and each transmission through or reflection off
 * glass (f = the rt/glass.c:45-165 coefficient as a function of the
 * transmissivity).  Sampling decisions (Russian roulette, hemisphere sizes)
 * are held fixed.  Accumulators: per block in shared memory when the slots
 * fit, flushed once per block. */
extern __shared__ double grad_smem[];

__device__ __forceinline__ void adj_append(gb_qadj &a, int slot, uint32_t kind, float pd)
{
    if (slot < 0)                            /* a factor that is no parameter */
        return;
    if (a.n < GB_ADJ_MAX) {
        a.e[a.n] = ((uint32_t)slot << 2) | kind;
        a.pd[a.n] = pd;
        a.n++;
    } else {
        a.n = GB_ADJ_MAX + 1;                /* too long: contributes no gradient */
    }
}

/* d ln(coefficient) / d(parameter) of one factor, per channel */
__device__ float3 adj_dlog(const gb_run &P, uint32_t e, float pd)
{
    const int slot = (int)(e >> 2);
    const uint32_t kind = e & 3u;
    const float4 m0 = P.S.mat[2 * slot], m1 = P.S.mat[2 * slot + 1];
    const float c[3] = {m0.y, m0.z, m0.w};
    float out[3];
    if (kind == GB_ADJ_REFL) {
        for (int i = 0; i < 3; i++)
            out[i] = c[i] > 0.f ? 1.f / c[i] : 0.f;
        return f3(out[0], out[1], out[2]);
    }
    const float rindex = m1.x, pdot = pd;
    const float cos2 = sqrtf((1.f - 1.f / (rindex * rindex)) + pdot * pdot / (rindex * rindex));
    float r1e = (pdot - rindex * cos2) / (pdot + rindex * cos2);
    r1e *= r1e;
    float r1m = (1.f / pdot - rindex / cos2) / (1.f / pdot + rindex / cos2);
    r1m *= r1m;
    for (int i = 0; i < 3; i++) {
        const float tau = fmaxf(c[i], 1e-15f);
        const float d = powf(tau, 1.f / cos2), dd = d / (cos2 * tau);
        const float qe = 1.f - r1e * r1e * d * d, qm = 1.f - r1m * r1m * d * d;
        float f, df;
        if (kind == GB_ADJ_GLASST) {
            f = .5f * (1.f - r1e) * (1.f - r1e) * d / qe + .5f * (1.f - r1m) * (1.f - r1m) * d / qm;
            df = .5f * (1.f - r1e) * (1.f - r1e) * (1.f + r1e * r1e * d * d) / (qe * qe) +
                 .5f * (1.f - r1m) * (1.f - r1m) * (1.f + r1m * r1m * d * d) / (qm * qm);
        } else {
            f = .5f * r1e * (1.f + (1.f - 2.f * r1e) * d * d) / qe + .5f * r1m * (1.f + (1.f - 2.f * r1m) * d * d) / qm;
            df = r1e * d * (1.f - r1e) * (1.f - r1e) / (qe * qe) + r1m * d * (1.f - r1m) * (1.f - r1m) / (qm * qm);
        }
        out[i] = f > 0.f ? df * dd / f : 0.f;
    }
    return f3(out[0], out[1], out[2]);
}

__device__ __forceinline__ void grad_slot_add(const gb_run &P, int slot, float3 g)
{
    double *acc = P.grad_shared ? grad_smem : P.grad;
    if (g.x != 0.f) atomicAdd(acc + 3 * slot, (double)g.x);
    if (g.y != 0.f) atomicAdd(acc + 3 * slot + 1, (double)g.y);
    if (g.z != 0.f) atomicAdd(acc + 3 * slot + 2, (double)g.z);
}

/* the gradient of a contribution v to sensor `sensor` along factor list a */
__device__ void grad_add(const gb_run &P, uint32_t sensor, float3 v, const gb_qadj &a)
{
    if (a.n == 0 || a.n > GB_ADJ_MAX)
        return;
    const double *w = P.dlde + 3ull * (sensor - P.sensor_base);
    const float3 wv = f3((float)w[0] * v.x, (float)w[1] * v.y, (float)w[2] * v.z);
    if (wv.x == 0.f && wv.y == 0.f && wv.z == 0.f)
        return;
    for (uint32_t i = 0; i < a.n; i++)
        grad_slot_add(P, (int)(a.e[i] >> 2), wv * adj_dlog(P, a.e[i], a.pd[i]));
}

__device__ __forceinline__ void grad_begin(const gb_run &P)
{
    if (!P.grad_shared)
        return;
    for (int i = threadIdx.x; i < 3 * P.nslots; i += blockDim.x)
        grad_smem[i] = 0.0;
    __syncthreads();
}

__device__ __forceinline__ void grad_end(const gb_run &P)
{
    if (!P.grad_shared)
        return;
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * P.nslots; i += blockDim.x)
        if (grad_smem[i] != 0.0)
            atomicAdd(P.grad + i, grad_smem[i]);
}

/* ------------------------------------------------------- contributions */

__device__ __forceinline__ void add_value(const gb_run &P, uint32_t sensor, uint32_t tag, float3 v)
{
    if (!P.value)
        return;
    if (v.x == 0.f && v.y == 0.f && v.z == 0.f)
        return;
    /* a path from a super-sampled first hemisphere adds to its stratum */
    double *d = tag != GB_NOTAG ? P.ss_val + 3ull * tag : P.value + 3ull * (sensor - P.sensor_base);
    atomicAdd(d, (double)v.x);
    atomicAdd(d + 1, (double)v.y);
    atomicAdd(d + 2, (double)v.z);
}

/* rt/rcontrib.c:272-316: bin the chain coefficient of a ray that hit a
 * tracked modifier; lanes adding to the same (record, bin) are merged first */
__device__ __forceinline__ void add_bin(const gb_run &P, uint32_t sensor, int slot, float3 dir, float3 c,
                                        Counters &cnt)
{
    int4 mi = P.modinfo[slot];           /* x: program offset, y: nbins, z: bin0 */
    float bval = eval_bin(P.binprog + mi.x, dir);
    if (bval <= -.5f)
        return;
    int bn = (int)(bval + .5f);
    if (bn >= mi.y) {
        atomicAdd(P.stats + ST_BADBIN, 1ull);   /* rt/rcontrib.c:305-309 warning */
        return;
    }
    uint32_t rec = (sensor - P.sensor_base) / (uint32_t)P.accum;
    unsigned long long key = (unsigned long long)rec * (unsigned long long)P.nbins_total + (unsigned long long)(mi.z + bn);
    cnt.contrib++;
    /* warp aggregation: lanes with the same key sum through shuffles */
    unsigned int act = __activemask();
    unsigned int grp = __match_any_sync(act, key);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int l = 0; l < 32; l++) {
        if (grp & (1u << l)) {
            sx += __shfl_sync(grp, c.x, l);
            sy += __shfl_sync(grp, c.y, l);
            sz += __shfl_sync(grp, c.z, l);
        }
    }
    int leader = __ffs(grp) - 1;
    if ((int)(threadIdx.x & 31) == leader) {
        double *d = P.bins + 3ull * key;
        atomicAdd(d, (double)sx);
        atomicAdd(d + 1, (double)sy);
        atomicAdd(d + 2, (double)sz);
    }
}

/* rt/source.c:749-793 (m_light) for a ray r that hit light object obj;
 * returns the radiance it carries (rcol) and applies rcontrib's callback */
template <bool G = false>
__device__ __forceinline__ void light_hit(const gb_run &P, const Ray &r, int obj, int ms, float t, float rod,
                                          Counters &cnt, float3 *rcol_out)
{
    const gb_dscene &S = P.S;
    float4 m0 = S.mat[2 * ms], m1 = S.mat[2 * ms + 1];
    int mk = (int)m0.x;
    float3 col = f3(m0.y, m0.z, m0.w);
    float3 rcol = f3(0.f, 0.f, 0.f);
    float3 rc = r.coef;
    bool glow = mk == DM_GLOW;
    bool distglow = glow && (m1.x >= -D_FTINY) && (t > m1.x);
    bool bad = (r.crtype & (GB_AMBIENT | GB_SPECULAR)) && !((r.crtype & GB_SHADOW) || rod < 0.f || distglow);
    bool wrong = r.rsrc >= 0 && S.src[r.rsrc].so != obj;
    if (bad || wrong)
        rc = f3(0.f, 0.f, 0.f);
    else if (rod >= 0.f && !(mk == DM_LIGHT && m1.x > 0.f &&       /* a spotlight seen from outside */
                             m1.x < 2.f * (float)D_PI * (1.f + m1.y * r.dir.x + m1.z * r.dir.y + m1.w * r.dir.z)))
        rcol = col;
    if (rcol_out)
        *rcol_out = rcol;
    if (!(bad || wrong)) {
        if (r.rsrc < 0) {                /* shadow values are added by direct() */
            if (G)
                grad_add(P, r.sensor, rc * rcol, r.adj);
            else
                add_value(P, r.sensor, r.tag, rc * rcol);
        }
        if (P.binprog) {
            int slot = S.trk[obj];
            if (slot >= 0 && (r.rsrc < 0 || S.src[r.rsrc].so == obj) && r.lcoef > D_FTINY) {
                float3 c = P.contrib_mode ? rc * rcol : rc;
                add_bin(P, r.sensor, slot, r.dir, c, cnt);
            }
        }
    }
}

/* rcontrib callback for a ray that hit a non-light surface */
__device__ __forceinline__ void surface_contrib(const gb_run &P, const Ray &r, int obj, Counters &cnt)
{
    if (!P.binprog || P.contrib_mode)
        return;
    int slot = P.S.trk[obj];
    if (slot < 0 || r.lcoef <= D_FTINY)
        return;
    if (r.rsrc >= 0 && P.S.src[r.rsrc].so != obj)
        return;
    add_bin(P, r.sensor, slot, r.dir, r.coef, cnt);
}

/* ----------------------------------------------------------- rayorigin */

/* rt/raytrace.c:39-135 for a child of `parent` of type rt with local
 * coefficient rc (has_rc = 0 for the reference's NULL); decides Russian
 * roulette with the child's own draw.  Returns false if the child dies. */
__device__ __forceinline__ bool ray_origin(const gb_run &P, const Ray &parent, uint32_t rt, float3 rc,
                                           bool has_rc, uint32_t code, Ray &c, float4 *u_out)
{
    float rw = 1.f;
    if (has_rc) {
        rw = maxc(rc);
        if (rw > 1.f)
            rw = 1.f;
    } else
        rc = f3(1.f, 1.f, 1.f);
    c.path = gb_child(parent.path, code);
    c.sensor = parent.sensor;
    c.tag = parent.tag;
    c.rsrc = parent.rsrc;
    c.rlvl = parent.rlvl + ((rt & GB_RAYREFL) ? 1 : 0);
    if ((rt & GB_RAYREFL) && c.rsrc >= 0)
        c.rsrc = -1;
    c.crtype = parent.crtype | rt;
    c.adepth = parent.adepth;
    c.weight = parent.weight * rw;
    c.coef = parent.coef * rc;
    c.lcoef = maxc(rc);
    gb_u4 u = gb_draw(c.path, c.sensor, GB_G_CREATE, P.k0, P.k1);
    if (u_out)
        *u_out = make_float4(gb_u01(u.v[0]), gb_u01(u.v[1]), gb_u01(u.v[2]), gb_u01(u.v[3]));
    if (c.weight <= 0.f)
        return false;
    if (c.crtype & GB_SHADOW)
        return true;
    if ((P.maxdepth <= 0) & has_rc) {
        if ((P.maxdepth < 0) & (c.rlvl > -P.maxdepth))
            return false;
        if (c.weight >= P.minweight)
            return true;
        if (gb_u01(u.v[0]) > c.weight / P.minweight)
            return false;
        float s = P.minweight / c.weight;
        c.coef = c.coef * s;
        c.lcoef *= s;
        c.weight = P.minweight;
        return true;
    }
    return (c.weight >= P.minweight) & (c.rlvl <= abs(P.maxdepth));
}

/* common/fvect.c getperpendicular with randomized orientation */
__device__ __forceinline__ float3 perpendicular(float3 v, float4 u, uint32_t ord_draw)
{
    float v1[3] = {0.5f - u.x, 0.5f - u.y, 0.5f - u.z};
    int ord[3];
    switch (gb_irand(ord_draw, 6u)) {
    case 0: ord[0] = 0; ord[1] = 1; ord[2] = 2; break;
    case 1: ord[0] = 0; ord[1] = 2; ord[2] = 1; break;
    case 2: ord[0] = 1; ord[1] = 0; ord[2] = 2; break;
    case 3: ord[0] = 1; ord[1] = 2; ord[2] = 0; break;
    case 4: ord[0] = 2; ord[1] = 0; ord[2] = 1; break;
    default: ord[0] = 2; ord[1] = 1; ord[2] = 0; break;
    }
    int i;
    for (i = 3; i--;)
        if ((-0.6f < comp(v, ord[i])) & (comp(v, ord[i]) < 0.6f))
            break;
    if (i < 0)
        i = 0;
    v1[ord[i]] = 1.f;
    return normalize3(cross3(f3(v1[0], v1[1], v1[2]), v));
}

/* hemisphere frame of a hit, drawn from the hit ray's frame group */
struct Hemi {
    float3 onrm, ux, uy;
    float3 acoef;       /* aval / n^2 */
    int n;
    uint32_t atyp;
};

__device__ __forceinline__ bool make_hemi(const gb_run &P, const Ray &r, float3 aval, float3 ron, Hemi &h,
                                          bool back = false)
{
    /* rt/ambcomp.c:351-421 (samp_hemi) for the ambacc <= FTINY case */
    float d = maxc(aval);
    if (d <= D_FTINY)
        return false;
    float wt = r.weight;
    d *= 0.8f * r.weight / ((float)P.ad * P.minweight + 1e-20f);
    if (wt > d)
        wt = d;
    int n = (int)(sqrtf((float)P.ad * wt) + 0.5f);
    if (n < 1)
        n = 1;
    h.n = n;
    h.atyp = back ? GB_TAMBIENT : GB_RAMBIENT;   /* the back side: ron is its (flipped) normal */
    h.onrm = ron;
    h.acoef = aval * (1.f / (float)(n * n));
    gb_u4 u = gb_draw(r.path, r.sensor, GB_G_FRAME, P.k0, P.k1);
    h.ux = perpendicular(ron, make_float4(gb_u01(u.v[0]), gb_u01(u.v[1]), gb_u01(u.v[2]), 0.f), u.v[3]);
    h.uy = cross3(h.onrm, h.ux);
    return true;
}

/* child k of a hemisphere (rt/ambcomp.c:177-250 ambsample).  With
 * spt == nullptr the disk position is the plain jitter of the child's own
 * draw (hemispheres below 4 x 4 strata, where the reference makes no
 * collision test); otherwise spt is the position placed by
 * gb_place_sample. */
__device__ __forceinline__ bool hemi_child(const gb_run &P, const Ray &parent, const Hemi &h, float3 hp,
                                           int origin, int k, const float *spt, Ray &c,
                                           uint32_t code = GB_NOTAG)
{
    float4 u;
    if (!ray_origin(P, parent, h.atyp, h.acoef, true, code == GB_NOTAG ? GB_C_STRATUM(k) : code, c, &u))
        return false;
    float s[2];
    if (spt) {
        s[0] = spt[0];
        s[1] = spt[1];
    } else {
        int i = k / h.n, j = k - i * h.n;
        gb_square2disk(s, ((float)j + u.z) / (float)h.n, ((float)i + u.y) / (float)h.n);
    }
    float zd = sqrtf(fmaxf(0.f, 1.f - s[0] * s[0] - s[1] * s[1]));
    c.dir = normalize3(h.ux * s[0] + h.uy * s[1] + h.onrm * zd);
    c.org = hp;
    c.origin = origin;
    c.adepth = parent.adepth + 1;
    return true;
}

#define MAX_HEMI_N 128

/* Spawn all children of a hemisphere of 4 x 4 strata or more met after the
 * first generation: placed sequentially with collision avoidance and
 * queued as they are placed (only two rows of positions are kept). */
template <bool G = false>
__device__ __noinline__ void spawn_hemi_big(const gb_run &P, const Ray &parent, const Hemi &h, float3 hp, int origin,
                                            int slot)
{
    gb_lot L;
    float rows[2][MAX_HEMI_N][2];
    float (*prev)[2] = rows[0], (*cur)[2] = rows[1];
    const int n = h.n;
    if (n > MAX_HEMI_N) {
        atomicAdd(P.stats + GB_ST_OVERFLOW, 1ull);
        return;
    }
    gb_lot_init(&L, parent.path, parent.sensor, P.k0, P.k1);
    for (int k = 0; k < n; k++) {
        rows[0][k][0] = rows[0][k][1] = 2.f;
        rows[1][k][0] = rows[1][k][1] = 2.f;
    }
    for (int i = n - 1; i >= 0; i--) {
        for (int j = n - 1; j >= 0; j--) {
            Ray c;
            float4 u;
            int k = i * n + j;
            float sp[2] = {2.f, 2.f};
            if (ray_origin(P, parent, h.atyp, h.acoef, true, GB_C_STRATUM(k), c, &u)) {
                gb_place_sample(&L, n, i, j, u.y, u.z, i + 1 < n ? (const float(*)[2])prev : nullptr,
                                (const float(*)[2])cur, sp);
                float zd = sqrtf(fmaxf(0.f, 1.f - sp[0] * sp[0] - sp[1] * sp[1]));
                c.dir = normalize3(h.ux * sp[0] + h.uy * sp[1] + h.onrm * zd);
                c.org = hp;
                c.origin = origin;
                c.adepth = parent.adepth + 1;
                if (G) {
                    c.adj = parent.adj;
                    adj_append(c.adj, slot, GB_ADJ_REFL, 0.f);
                }
                push_ray<G>(P, c);
            }
            cur[j][0] = sp[0];
            cur[j][1] = sp[1];
        }
        float(*t)[2] = prev;
        prev = cur;
        cur = t;
        for (int k = 0; k < n; k++)
            cur[k][0] = cur[k][1] = 2.f;
    }
}

/* ------------------------------------------------------------- shading */

struct Surf {                 /* rt/normal.c NORMDAT */
    float3 mcolor, scolor, pnorm;       /* pnorm: the shading normal */
    float rdiff, rspec, alpha2, pdot;
    float trans, tspec, tdiff;    /* trans material; 0 for plastic and metal */
    bool pure, refl, rblt, flat, tran, tblt;
};

/* rt/normal.c:72-173 dirnorm; the transmitted direction of a trans
 * surface without texture is the ray's own (rdir) */
__device__ __forceinline__ float3 dirnorm(const gb_run &P, const Surf &s, float3 rdir, float3 ldir, float omega,
                                          float3 *diffuse = nullptr)
{
    float3 v = f3(0.f, 0.f, 0.f);
    float ldot = dot3(s.pnorm, ldir);
    if (ldot < 0.f ? s.trans <= D_FTINY : s.trans >= 1.f - D_FTINY)
        return v;                                /* wrong side */
    float lrdiff = s.rdiff, ltdiff = s.tdiff;
    if (s.pure && s.rspec >= FRESTHRESH && ((lrdiff > D_FTINY) | (ltdiff > D_FTINY))) {
        const float f = 1.f - fresne(fabsf(ldot));
        lrdiff *= f;
        ltdiff *= f;
    }
    if ((ldot > D_FTINY) & (lrdiff > D_FTINY))
        v = v + s.mcolor * (ldot * omega * lrdiff * (1.f / D_PI));
    if ((ldot < -D_FTINY) & (ltdiff > D_FTINY))          /* diffuse transmission */
        v = v + s.mcolor * (-ldot * omega * ltdiff * (1.f / D_PI));
    if (diffuse)
        *diffuse = v;
    if ((ldot < -D_FTINY) & s.tran & !s.pure) {          /* specular transmission */
        float dt = s.alpha2 + omega * (1.f / D_PI);
        dt = expf((2.f * dot3(rdir, ldir) - 2.f) / dt) / (D_PI * dt);
        if (dt > D_FTINY)
            v = v + s.mcolor * (dt * s.tspec * omega * sqrtf(-ldot / s.pdot));
    }
    if ((ldot > D_FTINY) & s.refl & !s.pure) {
        float dt = s.alpha2;
        if (s.flat)
            dt += (1.f - P.dstrsrc) * omega * (0.25f / D_PI);
        float3 vt = ldir - rdir;
        float d2 = dot3(vt, s.pnorm);
        d2 *= d2;
        float d3 = dot3(vt, vt);
        float d4 = (d3 - d2) / d2;
        dt = expf(-d4 / dt) * d3 / (D_PI * d2 * d2 * dt);
        if (dt > D_FTINY)
            v = v + s.scolor * (dt * ldot * omega);
    }
    return v;
}

/* Follow a shadow ray and its transmitted continuations (rt/source.c:497-545
 * and the raycont() chain it starts).  Returns the value the sample adds
 * to the ray's colour (scp->val): the potential when the first ray reaches
 * the source or nothing, else coefficient x transmission x source radiance;
 * applies the rcontrib callback to every ray of the chain. */
template <bool G = false>
__device__ float3 shadow_chain(const gb_run &P, Ray sr, int s, Counters &cnt, float3 coef, float3 potential,
                               gb_qadj *factors)
{
    const gb_dscene &S = P.S;
    const gb_dsrc &src = S.src[s];
    float3 T = f3(1.f, 1.f, 1.f);           /* product of transmissions so far */
    const float3 zero = f3(0.f, 0.f, 0.f);
    for (int guard = 0; guard < 32; guard++) {
        Hit h;
        uint32_t st[3] = {0, 0, 0};
        cnt.rays++;
        bool hit = local_hit(S, sr.org, sr.dir, sr.origin, h, st);
        cnt.add(st);
        if (!hit) {
            if (guard == 0) {
                if (P.follow && (src.flags & DS_DISTANT)) {
                    if (source_hit(S, sr.dir, s, sr.crtype) >= 0)
                        light_hit(P, sr, src.so, src.mat, D_FHUGE, 1.f, cnt, nullptr);
                }
                return potential;
            }
            if (source_hit(S, sr.dir, s, sr.crtype) < 0)
                return zero;
            float3 rc;
            light_hit(P, sr, src.so, src.mat, D_FHUGE, 1.f, cnt, &rc);
            return coef * T * rc;
        }
        const int ro = sid_object(S, h.obj);   /* h.obj: the surface id, the children's origin */
        int ms = S.obj[ro].y;
        int mk = ms >= 0 ? (int)S.mat[2 * ms].x : DM_NONE;
        if (ro == src.so && guard == 0 && !P.follow)
            return potential;                 /* aimed and reached */
        float3 hp = sr.org + sr.dir * h.t;
        if (mk == DM_LIGHT || mk == DM_GLOW) {
            float3 rc;
            light_hit(P, sr, ro, ms, h.t, h.rod, cnt, &rc);
            return coef * T * rc;
        }
        if (mk == DM_NONE) {
            surface_contrib(P, sr, ro, cnt);
            Ray c;
            ray_origin(P, sr, GB_TRANS, f3(1.f, 1.f, 1.f), false, GB_C_PASS, c, nullptr);
            c.org = hp;
            c.dir = sr.dir;
            c.origin = h.obj;
            sr = c;
            continue;
        }
        if (mk == DM_GLASS) {
            /* rt/glass.c:45-120, transmission only for shadow rays */
            float4 m0 = S.mat[2 * ms], m1 = S.mat[2 * ms + 1];
            float3 mc = f3(m0.y, m0.z, m0.w);
            float rindex = m1.x;
            if (!(maxc(mc) > 1e-15f))
                return zero;
            mc = f3(fmaxf(mc.x, 1e-15f), fmaxf(mc.y, 1e-15f), fmaxf(mc.z, 1e-15f));
            float pdot = fabsf(h.rod);
            float cos2 = sqrtf((1.f - 1.f / (rindex * rindex)) + pdot * pdot / (rindex * rindex));
            mc = f3(powf(mc.x, 1.f / cos2), powf(mc.y, 1.f / cos2), powf(mc.z, 1.f / cos2));
            float r1e = (pdot - rindex * cos2) / (pdot + rindex * cos2);
            r1e *= r1e;
            float r1m = (1.f / pdot - rindex / cos2) / (1.f / pdot + rindex / cos2);
            r1m *= r1m;
            float tc[3], mm[3] = {mc.x, mc.y, mc.z};
            for (int i = 0; i < 3; i++) {
                float d = mm[i];
                tc[i] = .5f * (1.f - r1e) * (1.f - r1e) * d / (1.f - r1e * r1e * d * d) +
                        .5f * (1.f - r1m) * (1.f - r1m) * d / (1.f - r1m * r1m * d * d);
            }
            surface_contrib(P, sr, ro, cnt);
            Ray c;
            float3 tcv = f3(tc[0], tc[1], tc[2]);
            if (!ray_origin(P, sr, GB_TRANS, tcv, true, GB_C_TRANS, c, nullptr))
                return zero;
            c.org = hp;
            c.dir = sr.dir;
            c.origin = h.obj;
            T = T * tcv;
            if (G)
                adj_append(*factors, ms, GB_ADJ_GLASST, pdot);
            sr = c;
            continue;
        }
        surface_contrib(P, sr, ro, cnt);
        if (mk == DM_TRANS) {
            /* rt/normal.c:190-301 for a shadow ray: smooth trans passes its
             * specular transmission on (a continuing TRANS ray) */
            const float4 m0 = S.mat[2 * ms], m1 = S.mat[2 * ms + 1];
            if (m1.y * m1.y <= D_FTINY) {
                const float pdot = fmaxf(fabsf(h.rod), .001f);
                float rspec = m1.x;
                if (rspec >= FRESTHRESH)
                    rspec += fresne(pdot) * (1.f - rspec);
                const float tspec = m1.z * (1.f - rspec) * m1.w;
                if (tspec > D_FTINY) {
                    const float3 tcv = f3(m0.y, m0.z, m0.w) * tspec;
                    Ray c;
                    if (!ray_origin(P, sr, GB_TRANS, tcv, true, GB_C_TRANS, c, nullptr))
                        return zero;
                    c.org = hp;
                    c.dir = sr.dir;
                    c.origin = h.obj;
                    T = T * tcv;
                    sr = c;
                    continue;
                }
            }
        }
        /* opaque (or rough trans): blocked (rt/normal.c:190, m_normal's
         * shadow test) */
        return zero;
    }
    return zero;
}

#define MAXSPART 64                /* pieces of a partitioned source */

/* One sample of source sn's piece pi (centre ct, size sz in 1/MAXSPART of
 * the source's half-size vectors; the whole source is 0, 0, 64, 64):
 * rt/srcsamp.c:37-145 nextssamp, then the coefficient, the potential and
 * the shadow ray of rt/source.c:398-556 (direct). */
template <bool G>
__device__ __noinline__ void direct_sample(const gb_run &P, const Ray &r, float3 hp, const Surf &s, int origin,
                                           Counters &cnt, int slot, int sn, int pi, int ct0, int ct1, int sz0,
                                           int sz1, bool multi)
{
    const gb_dscene &S = P.S;
    const gb_dsrc &src = S.src[sn];
    const float3 sloc = f3(src.sloc[0], src.sloc[1], src.sloc[2]);
    const uint32_t code = GB_C_SHADOWP(sn, pi);
    float vpos[3] = {0.f, 0.f, 0.f};
    if (P.dstrsrc > D_FTINY) {
        gb_u4 u = gb_draw(gb_child(r.path, code), r.sensor, GB_G_SRC, P.k0, P.k1);
        vpos[0] = P.dstrsrc * (1.f - 2.f * gb_u01(u.v[0])) * (float)sz0 * (1.f / MAXSPART);
        vpos[1] = P.dstrsrc * (1.f - 2.f * gb_u01(u.v[1])) * (float)sz1 * (1.f / MAXSPART);
        vpos[2] = (src.flags & DS_FLAT) ? 0.f : P.dstrsrc * (1.f - 2.f * gb_u01(u.v[2]));
    }
    vpos[0] += (float)ct0 * (1.f / MAXSPART);
    vpos[1] += (float)ct1 * (1.f / MAXSPART);
    if ((src.flags & DS_CIR) && (multi || P.dstrsrc > 0.7f)) {
        /* circular sources: samples pulled in from the square's corners
         * (rt/srcsamp.c:85-109) */
        if (src.flags & (DS_FLAT | DS_DISTANT)) {
            const float d = 1.12837917f;
            const float t0 = d * sqrtf(1.f - 0.5f * vpos[1] * vpos[1]);
            const float t1 = d * sqrtf(1.f - 0.5f * vpos[0] * vpos[0]);
            vpos[0] *= t0;
            vpos[1] *= t1;
            vpos[2] = 0.f;
        } else {
            const float a = vpos[0] * vpos[0], b = vpos[1] * vpos[1], c = vpos[2] * vpos[2];
            const float sum = a + b + c, mx = fmaxf(a, fmaxf(b, c));
            const float t = sum > D_FTINY * D_FTINY ? (1.f / 0.7236f) * sqrtf(mx / sum) : 0.f;
            vpos[0] *= t;
            vpos[1] *= t;
            vpos[2] *= t;
        }
    }
    float3 dir = sloc + f3(src.ss[0][0], src.ss[0][1], src.ss[0][2]) * vpos[0] +
                 f3(src.ss[1][0], src.ss[1][1], src.ss[1][2]) * vpos[1] +
                 f3(src.ss[2][0], src.ss[2][1], src.ss[2][2]) * vpos[2];
    if (!(src.flags & DS_DISTANT))
        dir = dir - hp;
    float dist = sqrtf(dot3(dir, dir));
    if (dist == 0.f)
        return;
    dir = dir * (1.f / dist);
    float dom;
    if (src.flags & DS_FLAT)
        dom = -(src.snorm[0] * dir.x + src.snorm[1] * dir.y + src.snorm[2] * dir.z);
    else if (src.flags & DS_CYL) {               /* rt/srcsamp.c:364-376 scylform */
        const float3 su = f3(src.ss[0][0], src.ss[0][1], src.ss[0][2]);
        float d = dot3(dir, su);
        d *= d / dot3(su, su);
        dom = sqrtf(1.f - d);
    } else
        dom = 1.f;
    dom *= (float)(sz0 * sz1) * (1.f / (MAXSPART * MAXSPART));
    if (src.flags & DS_DISTANT) {
        dom *= src.ss2;
    } else {
        if (dom <= 1e-4f)
            return;
        dom *= src.ss2 / (dist * dist);
        if ((src.flags & DS_PROX) && dist > src.prox)
            return;
        if (src.flags & DS_SPOT) {               /* rt/source.c:246-252: outside the cone, none */
            if (src.spot[0] < 2.f * (float)D_PI * (1.f + src.spot[1] * dir.x + src.spot[2] * dir.y +
                                                   src.spot[3] * dir.z))
                return;
            const float df = dist + src.spot[4];   /* the solid angle seen from the focus */
            dom *= dist * dist / (df * df);
        }
    }
    float3 coefd;
    float3 coef = dirnorm(P, s, r.dir, dir, dom, G ? &coefd : nullptr);
    if (maxc(coef) <= 0.f)
        return;
    /* potential (srcvalue): the source alone */
    float4 m0 = S.mat[2 * src.mat];
    float3 L = f3(m0.y, m0.z, m0.w);
    if (src.flags & DS_DISTANT) {
        float dt = dot3(sloc, dir);
        if (2.f * D_PI * (1.f - dt) > src.ss2)
            return;
    } else {
        Hit hs;
        hs.obj = -1;
        hs.t = D_FHUGE;
        hs.rod = 1.f;
        hit_object(S, src.so, hp, dir, hs, D_FTINY);
        if (hs.obj != src.so)
            return;                            /* aiming failure */
        if (hs.rod < 0.f)
            return;                            /* behind the source: black */
    }
    float3 pot = coef * L;
    if (0.2126f * pot.x + 0.7152f * pot.y + 0.0722f * pot.z <= 0.f)
        return;
    /* shadow ray (rt/source.c:497-510) */
    Ray sr;
    bool thru = !(dot3(dir, s.pnorm) > 0.f);          /* thrudir, rt/ray.h:87 */
    ray_origin(P, r, thru ? GB_TSHADOW : GB_RSHADOW, f3(1.f, 1.f, 1.f), false, code, sr, nullptr);
    sr.coef = r.coef * coef;
    sr.lcoef = maxc(coef);
    sr.rsrc = sn;
    sr.org = hp;
    sr.dir = dir;
    sr.origin = origin;
    if (!G) {
        float3 v = shadow_chain(P, sr, sn, cnt, coef, pot, nullptr);
        add_value(P, r.sensor, r.tag, r.coef * v);
        return;
    }
    gb_qadj fac = r.adj;                       /* the path's factors and the shadow's glass */
    const float3 c = r.coef * shadow_chain<true>(P, sr, sn, cnt, coef, pot, &fac);
    grad_add(P, r.sensor, c, fac);
    if (slot >= 0 && fac.n <= GB_ADJ_MAX) {    /* this surface's own reflectance: */
        const double *w = P.dlde + 3ull * (r.sensor - P.sensor_base);     /* the diffuse part */
        float g[3], cc[3] = {c.x, c.y, c.z}, cd[3] = {coefd.x, coefd.y, coefd.z}, ct[3] = {coef.x, coef.y, coef.z};
        float mc[3] = {s.mcolor.x, s.mcolor.y, s.mcolor.z};
        for (int i = 0; i < 3; i++)
            g[i] = (ct[i] > 0.f && mc[i] > 0.f) ? (float)w[i] * cc[i] * (cd[i] / ct[i]) / mc[i] : 0.f;
        grad_slot_add(P, slot, f3(g[0], g[1], g[2]));
    }
}

/* rt/source.c:398-556 (direct) with every piece's shadow tested (the
 * reference's -dt threshold, which estimates untested pieces from run-wide
 * hit statistics, is taken as 0).  A flat local source larger than -ds
 * times its distance is split as rt/srcsamp.c:260-330 (flatpart,
 * flt_partit) splits it: halved along its longer side, recursively, up to
 * MAXSPART pieces, lower half first; other sources are one piece. */
/* The pieces of a cylinder source under -ds (rt/srcsamp.c:187-273 cylpart,
 * cyl_partit): none from inside the cylinder's extended radius, the whole
 * source from close by or far away, else halved along the axis, lower half
 * first, until a piece is farther than its scaled length. */
template <bool G>
__device__ __noinline__ void direct_cyl(const gb_run &P, const Ray &r, float3 hp, const Surf &s, int origin,
                                        Counters &cnt, int slot, int sn)
{
    const gb_dsrc &src = P.S.src[sn];
    const float3 sloc = f3(src.sloc[0], src.sloc[1], src.sloc[2]);
    const float3 su = f3(src.ss[0][0], src.ss[0][1], src.ss[0][2]);
    const float3 sv = f3(src.ss[1][0], src.ss[1][1], src.ss[1][2]);
    const float rad2 = 1.365f * dot3(sv, sv);
    const float3 v = hp - sloc;
    float safe2 = dot3(su, su);
    float d = dot3(v, su);
    const float cent2 = dot3(v, v), perp2 = cent2 - d * d / safe2;
    if (perp2 <= rad2)
        return;                                  /* inside the extended cylinder */
    safe2 *= 4.f * r.weight * r.weight / (P.srcsizerat * P.srcsizerat);
    if (perp2 <= 4.f * rad2 || cent2 >= safe2) {
        direct_sample<G>(P, r, hp, s, origin, cnt, slot, sn, 0, 0, 0, MAXSPART, MAXSPART, false);
        return;
    }
    struct Piece {
        float3 cent, ax;
        float d2;
        int mp, ct0, sz0;
    } stack[8];
    int top = 0, pi = 0;
    stack[top++] = {sloc, su, safe2, MAXSPART, 0, MAXSPART};
    while (top > 0) {
        Piece f = stack[--top];
        for (;;) {
            const float3 dc = hp - f.cent;
            if (f.mp < 2 || dot3(dc, dc) >= f.d2) {
                direct_sample<G>(P, r, hp, s, origin, cnt, slot, sn, pi++, f.ct0, 0, f.sz0, MAXSPART, true);
                break;
            }
            Piece lo = f, hi = f;
            const float3 ax = f.ax * 0.5f;
            lo.ax = hi.ax = ax;
            lo.d2 = hi.d2 = f.d2 * 0.25f;
            lo.mp = hi.mp = f.mp / 2;
            lo.sz0 = hi.sz0 = f.sz0 >> 1;
            lo.ct0 = f.ct0 - lo.sz0;
            hi.ct0 = f.ct0 + lo.sz0;
            lo.cent = f.cent - ax;
            hi.cent = f.cent + ax;
            if (top < 8)
                stack[top++] = hi;
            f = lo;
        }
    }
}

template <bool G = false>
__device__ void direct(const gb_run &P, const Ray &r, float3 hp, const Surf &s, int origin, Counters &cnt,
                       int slot)
{
    const gb_dscene &S = P.S;
    for (int sn = 0; sn < S.nsrc; sn++) {
        const gb_dsrc &src = S.src[sn];
        if (src.flags & DS_SKIP)
            continue;
        const float3 sloc = f3(src.sloc[0], src.sloc[1], src.sloc[2]);
        if ((src.flags & (DS_PROX | DS_DISTANT)) == DS_PROX) {
            float3 dv = hp - sloc;
            float rr = src.prox + src.srad;
            if (dot3(dv, dv) > rr * rr)
                continue;
        }
        if (P.srcsizerat > D_FTINY && (src.flags & DS_CYL)) {
            direct_cyl<G>(P, r, hp, s, origin, cnt, slot, sn);
            continue;
        }
        if (P.srcsizerat <= D_FTINY || (src.flags & DS_DISTANT) || !(src.flags & DS_FLAT)) {
            direct_sample<G>(P, r, hp, s, origin, cnt, slot, sn, 0, 0, 0, MAXSPART, MAXSPART, false);
            continue;
        }
        const float3 snorm = f3(src.snorm[0], src.snorm[1], src.snorm[2]);
        if (dot3(hp - sloc, snorm) <= 0.f)
            continue;                          /* behind the source: no pieces */
        const float3 su = f3(src.ss[0][0], src.ss[0][1], src.ss[0][2]);
        const float3 sv = f3(src.ss[1][0], src.ss[1][1], src.ss[1][2]);
        float dv2 = 2.f * r.weight / P.srcsizerat;
        dv2 *= dv2;
        /* depth-first over the halving tree: a stack of pending upper halves */
        struct Piece {
            float3 cent, u, v;
            float du2, dv2;
            int mp, ct0, ct1, sz0, sz1;
        } stack[8];
        int top = 0, pi = 0;
        stack[top++] = {sloc, su, sv, dv2 * dot3(su, su), dv2 * dot3(sv, sv), MAXSPART, 0, 0, MAXSPART, MAXSPART};
        const float3 dc0 = hp - sloc;
        const bool multi = !(dot3(dc0, dc0) >= stack[0].du2 && dot3(dc0, dc0) >= stack[0].dv2);   /* np > 1 */
        while (top > 0) {
            Piece f = stack[--top];
            for (;;) {
                const float3 dc = hp - f.cent;
                const float d2 = dot3(dc, dc);
                if (f.mp < 2 || (d2 >= f.du2 && d2 >= f.dv2)) {
                    direct_sample<G>(P, r, hp, s, origin, cnt, slot, sn, pi++, f.ct0, f.ct1, f.sz0, f.sz1, multi);
                    break;
                }
                Piece lo = f, hi = f;
                float3 ax;
                if (f.du2 > f.dv2) {                 /* halve along U */
                    ax = f.u * 0.5f;
                    lo.u = hi.u = ax;
                    lo.du2 = hi.du2 = f.du2 * 0.25f;
                    lo.sz0 = hi.sz0 = f.sz0 >> 1;
                    lo.ct0 = f.ct0 - lo.sz0;
                    hi.ct0 = f.ct0 + lo.sz0;
                } else {                             /* halve along V */
                    ax = f.v * 0.5f;
                    lo.v = hi.v = ax;
                    lo.dv2 = hi.dv2 = f.dv2 * 0.25f;
                    lo.sz1 = hi.sz1 = f.sz1 >> 1;
                    lo.ct1 = f.ct1 - lo.sz1;
                    hi.ct1 = f.ct1 + lo.sz1;
                }
                lo.mp = hi.mp = f.mp / 2;
                lo.cent = f.cent - ax;
                hi.cent = f.cent + ax;
                stack[top++] = hi;
                f = lo;
            }
        }
    }
}

/* Shade a hit on plastic or metal: returns false if unsupported */
__device__ __forceinline__ void setup_surf(const gb_run &P, int mk, float4 m0, float4 m1, float3 n, float3 pn,
                                           float pd, bool flat, Surf &s)
{
    s.mcolor = f3(m0.y, m0.z, m0.w);
    s.alpha2 = m1.y * m1.y;
    s.pure = s.alpha2 <= D_FTINY;
    s.pnorm = pn;
    s.pdot = pd < .001f ? .001f : pd;
    s.flat = flat;
    s.rspec = m1.x;
    float fest = 0.f;
    if (s.pure && s.rspec >= FRESTHRESH) {
        fest = fresne(s.pdot);
        s.rspec += fest * (1.f - s.rspec);
    }
    if (mk == DM_TRANS) {                        /* rt/normal.c:259-277 */
        s.trans = m1.z * (1.f - s.rspec);
        s.tspec = s.trans * m1.w;
        s.tdiff = s.trans - s.tspec;
        s.tran = s.tspec > D_FTINY;
        s.tblt = s.tran && !s.pure && P.specthresh >= s.tspec - D_FTINY;
    } else {
        s.trans = s.tspec = s.tdiff = 0.f;
        s.tran = s.tblt = false;
    }
    s.rdiff = 1.f - s.trans - s.rspec;
    s.refl = s.rspec > D_FTINY;
    if (s.refl) {
        if (mk != DM_METAL)
            s.scolor = f3(s.rspec, s.rspec, s.rspec);
        else if (fest > D_FTINY) {
            float d = m1.x * (1.f - fest);
            s.scolor = f3(fest + s.mcolor.x * d, fest + s.mcolor.y * d, fest + s.mcolor.z * d);
        } else
            s.scolor = s.mcolor * s.rspec;
    } else
        s.scolor = f3(0.f, 0.f, 0.f);
    s.rblt = !s.pure && P.specthresh >= s.rspec - D_FTINY;
}

/* One trial of the specular lobe (rt/normal.c:398-420): a half vector
 * drawn about the normal with a Gaussian slope of variance alpha2, the
 * incident direction mirrored about it.  Returns the cosine of the sample
 * with the surface normal (the caller rejects samples at or below FTINY). */
__device__ __forceinline__ float spec_trial(const gb_run &P, const Ray &r, const Surf &su, float3 ron, float3 u,
                                            float3 v, int t, float3 &sdir)
{
    const gb_u4 q = gb_draw(r.path, r.sensor, GB_G_SPEC + (uint32_t)(t >> 1), P.k0, P.k1);
    const int w = (t & 1) * 2;
    float rv0 = gb_u01(q.v[w]), rv1 = gb_u01(q.v[w + 1]);
    float sinp, cosp;
    sincosf(2.f * (float)M_PI * rv0, &sinp, &cosp);
    if ((0.f <= P.specjitter) & (P.specjitter < 1.f))
        rv1 = 1.f - P.specjitter * rv1;
    const float d = rv1 <= D_FTINY ? 1.f : sqrtf(su.alpha2 * -logf(rv1));
    const float3 h = su.pnorm + (u * cosp + v * sinp) * d;
    const float s = -2.f * dot3(h, r.dir) / (1.f + d * d);
    sdir = normalize3(r.dir + h * s);
    return dot3(sdir, ron);                     /* rejection against the surface normal */
}

/* rt/normal.c:441-495, the transmitted part of gaussamp: samples about
 * the ray's own direction (no texture), rejected at or above the surface,
 * without the W-G-M-D weighting; trials from GB_G_TSPEC, sample k is child
 * GB_C_TSPEC(k), all sharing the first one's Russian roulette. */
template <bool G>
__device__ __forceinline__ void gaussamp_trans(const gb_run &P, const Ray &r, const Surf &su, float3 ron,
                                               float3 u, float3 v, float3 hp, int obj)
{
    Ray c;
    if (!ray_origin(P, r, GB_TSPECULAR, su.mcolor * su.tspec, true, GB_C_TSPEC(0), c, nullptr))
        return;
    int nst = 1;
    if (P.specjitter > 1.5f) {
        nst = (int)(P.specjitter * r.weight + .5f);
        if (c.weight <= P.minweight * (float)nst)
            nst = (int)(c.weight / P.minweight);
        if (nst > 1) {
            const float d = 1.f / (float)nst;
            c.coef = c.coef * d;
            c.weight *= d;
        } else
            nst = 1;
    }
    c.org = hp;
    c.origin = obj;
    if (G)
        c.adj = r.adj;
    const int maxiter = GB_SPEC_MAXITER * nst;
    int taken = 0;
    for (int t = 0; taken < nst && t < maxiter; t++) {
        const gb_u4 q = gb_draw(r.path, r.sensor, GB_G_TSPEC + (uint32_t)(t >> 1), P.k0, P.k1);
        const int w = (t & 1) * 2;
        float rv0 = gb_u01(q.v[w]), rv1 = gb_u01(q.v[w + 1]);
        float sinp, cosp;
        sincosf(2.f * (float)M_PI * rv0, &sinp, &cosp);
        if ((0.f <= P.specjitter) & (P.specjitter < 1.f))
            rv1 = 1.f - P.specjitter * rv1;
        const float d = rv1 <= D_FTINY ? 1.f : sqrtf(su.alpha2 * -logf(rv1));
        const float3 sd = r.dir + (u * cosp + v * sinp) * d;
        if (dot3(sd, ron) >= -D_FTINY)
            continue;
        c.dir = normalize3(sd);
        if (taken)
            c.path = gb_child(r.path, GB_C_TSPEC(taken));
        push_ray<G>(P, c);
        taken++;
    }
}

/* rt/normal.c:364-440 gaussamp, reflection: sample the rough specular lobe
 * of a plastic or metal hit (specularity above -st).  One sample, or with
 * -ss above 1.5 ss times the ray weight of them, each weighted by the
 * W-G-M-D adjustment 2/(1 + cos_in/cos_out) and by samples wanted over
 * trials made; every trial is drawn here, so the weights are known before
 * the children are queued.  Children share one Russian-roulette decision,
 * as the reference's samples share one rayorigin. */
template <bool G>
__device__ __noinline__ void gaussamp(const gb_run &P, const Ray &r, const Surf &su, float3 ron, float rod, float3 hp,
                                    int obj)
{
    const gb_u4 uf = gb_draw(r.path, r.sensor, GB_G_SPECF, P.k0, P.k1);
    const float3 u = perpendicular(su.pnorm, make_float4(gb_u01(uf.v[0]), gb_u01(uf.v[1]), gb_u01(uf.v[2]), 0.f),
                                   uf.v[3]);
    const float3 v = cross3(su.pnorm, u);
    if (su.tran && !su.tblt)
        gaussamp_trans<G>(P, r, su, ron, u, v, hp, obj);
    if (!su.refl || su.rblt)
        return;
    Ray c;
    if (!ray_origin(P, r, GB_RSPECULAR, su.scolor, true, GB_C_SPEC(0), c, nullptr))
        return;
    int nst = 1;
    if (P.specjitter > 1.5f) {
        nst = (int)(P.specjitter * r.weight + .5f);
        if (c.weight <= P.minweight * (float)nst)
            nst = (int)(c.weight / P.minweight);
        if (nst > 1) {
            const float d = 1.f / (float)nst;
            c.coef = c.coef * d;
            c.weight *= d;
        } else
            nst = 1;
    }
    const int maxiter = GB_SPEC_MAXITER * nst;
    float post = 1.f;                   /* samples wanted / trials made */
    if (nst > 1) {
        int taken = 0, t = 0;
        for (; taken < nst && t < maxiter; t++) {
            float3 sd;
            if (spec_trial(P, r, su, ron, u, v, t, sd) > D_FTINY)
                taken++;
        }
        post = (float)nst / (float)t;
    }
    c.org = hp;
    c.origin = obj;
    if (G)                              /* specular color: not a parameter */
        c.adj = r.adj;
    const float3 coef = c.coef;
    int taken = 0;
    for (int t = 0; taken < nst && t < maxiter; t++) {
        float3 sd;
        const float cs = spec_trial(P, r, su, ron, u, v, t, sd);
        if (cs <= D_FTINY)
            continue;
        c.dir = sd;
        if (nst > 1) {
            if (taken)
                c.path = gb_child(r.path, GB_C_SPEC(taken));
            c.coef = coef * (2.f / (1.f + rod / cs) * post);
        }
        push_ray<G>(P, c);
        taken++;
    }
}

/* Ambient of one side of a surface (rt/ambient.c:229-300, -aa 0): the
 * hemisphere about nrm (the back side's flipped normal, TAMBIENT rays), or
 * the -av value beyond -ab bounces. */
template <bool G>
__device__ __forceinline__ void ambient_side(const gb_run &P, const Ray &r, float3 aval, float3 nrm, bool back,
                                             float3 hp, int obj, int ms)
{
    if (P.ad > 0 && r.adepth < P.ab) {
        Hemi hm;
        if (make_hemi(P, r, aval, nrm, hm, back) && hm.n >= 4) {
            spawn_hemi_big<G>(P, r, hm, hp, obj, ms);
        } else if (hm.n > 0) {
            int nn = hm.n * hm.n;
            for (int k = 0; k < nn; k++) {
                Ray c;
                if (hemi_child(P, r, hm, hp, obj, k, nullptr, c)) {
                    if (G) {
                        c.adj = r.adj;
                        adj_append(c.adj, ms, GB_ADJ_REFL, 0.f);
                    }
                    push_ray<G>(P, c);
                }
            }
        }
    } else if (P.av[0] != 0.f || P.av[1] != 0.f || P.av[2] != 0.f) {
        add_value(P, r.sensor, r.tag, r.coef * aval * f3(P.av[0], P.av[1], P.av[2]));
    }
}

/* the other side's ambient of a trans surface, out of line (rare): its
 * draws are keyed by a child path of the ray, apart from the front's */
template <bool G>
__device__ __noinline__ void ambient_back(const gb_run &P, const Ray &r, float3 aval, float3 nrm, float3 hp,
                                          int obj, int ms)
{
    Ray rb = r;
    rb.path = gb_child(r.path, GB_C_BACK);
    ambient_side<G>(P, rb, aval, nrm, true, hp, obj, ms);
}

/* The shading normal of a hit on a smooth mesh triangle (rt/o_mesh.c:
 * 185-206, rt/raytrace.c:446-478 raynormal): its vertex normals
 * interpolated at the hit by barycentric weights (in the triangle's
 * dominant-axis projection, in the mesh's coordinates), carried to the
 * scene by the instance's forward transform and normalised, turned with
 * the surface if it was flipped toward the ray, and reflected about the
 * ray's plane if it then faces away from the ray.  sid: the hit's surface
 * id; n0: its unflipped normal; rod > 0 after any flip.  false (pn, pd
 * untouched) when the triangle has no vertex normals or they do not
 * perturb its normal. */
__device__ __noinline__ bool mesh_pnorm(const gb_dscene &S, int sid, float3 hp, float3 dir, float3 n0, bool flipped,
                                        float rod, float3 &pn, float &pd)
{
    if (S.ninst == 0)
        return false;
    int lo = 0, hi = S.ninst - 1;                 /* the last instance with sidbase <= sid */
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S.inst[mid].sidbase <= sid)
            lo = mid;
        else
            hi = mid - 1;
    }
    const gb_dinst &I = S.inst[lo];
    const int o = I.firstobj + (sid - I.sidbase);
    const int fl = S.obj[o].x >> 8;
    if (!(fl & DF_VNORM))
        return false;
    const float *b = I.bx;
    const float3 p = f3(hp.x * b[0] + hp.y * b[3] + hp.z * b[6] + b[9], hp.x * b[1] + hp.y * b[4] + hp.z * b[7] + b[10],
                        hp.x * b[2] + hp.y * b[5] + hp.z * b[8] + b[11]);
    const int ax = (fl >> DF_AXSHIFT) & 3;
    const int xi = ax + 1 >= 3 ? ax - 2 : ax + 1, yi = xi + 1 >= 3 ? xi - 2 : xi + 1;
    const float4 va = S.fv4[2 * o], vb = S.fv4[2 * o + 1];     /* projected v0, v1 | v2 */
    const float e1x = va.z - va.x, e1y = va.w - va.y, e2x = vb.x - va.x, e2y = vb.y - va.y;
    const float den = e1x * e2y - e1y * e2x;
    if (den == 0.f)
        return false;
    const float qx = comp(p, xi) - va.x, qy = comp(p, yi) - va.y;
    const float w1 = (qx * e2y - qy * e2x) / den, w2 = (e1x * qy - e1y * qx) / den, w0 = 1.f - w1 - w2;
    const float4 *vn = S.vnrm + 3 * S.vnidx[o];
    const float3 m = f3(w0 * vn[0].x + w1 * vn[1].x + w2 * vn[2].x, w0 * vn[0].y + w1 * vn[1].y + w2 * vn[2].y,
                        w0 * vn[0].z + w1 * vn[1].z + w2 * vn[2].z);
    const float *f = I.fx;
    float3 w = f3(m.x * f[0] + m.y * f[3] + m.z * f[6], m.x * f[1] + m.y * f[4] + m.z * f[7],
                  m.x * f[2] + m.y * f[5] + m.z * f[8]);
    const float l = sqrtf(dot3(w, w));
    if (l == 0.f)
        return false;
    w = w * (1.f / l);
    const float3 pert = w - n0;
    if (dot3(pert, pert) <= D_FTINY * D_FTINY)
        return false;
    float3 nm = flipped ? -w : w;                  /* ron + pert after any flip: unit */
    float nd = -dot3(nm, dir);
    if ((nd > 0.f) != (rod > 0.f)) {
        nm = nm + dir * (2.f * nd);
        nd = -nd;
    }
    pn = nm;
    pd = nd;
    return true;
}

/* Shade ray r given its trace result (h.obj < 0: the ray left the scene)
 * and push every child ray to the next generation's queue
 * (rt/raytrace.c:163-256 raytrace / rayshade, the material routines). */
template <bool G, bool VN = false>
__device__ void shade_ray(const gb_run &P, const Ray &r, const Hit &h, Counters &cnt)
{
    const gb_dscene &S = P.S;
    if (h.obj < 0) {
        int sidx = source_hit(S, r.dir, r.rsrc, r.crtype);
        if (sidx >= 0)
            light_hit<G>(P, r, S.src[sidx].so, S.src[sidx].mat, D_FHUGE, 1.f, cnt, nullptr);
        return;
    }
    const int ro = sid_object(S, h.obj);       /* h.obj: the surface id, the children's origin */
    int ms = S.obj[ro].y;
    int mk = ms >= 0 ? (int)S.mat[2 * ms].x : DM_NONE;
    float3 hp = r.org + r.dir * h.t;
    /* -i (rt/raytrace.c:211-236 raytirrad): a primary ray, or one passed
     * on through transparent surfaces, passes through glass and meets
     * every other non-light material as a Lambertian of reflectance pi,
     * whose radiance is the irradiance there */
    bool lamb = false;
    if (P.do_irrad && !(r.crtype & ~(GB_PRIMARY | GB_TRANS))) {
        if (mk == DM_GLASS || mk == DM_TRANS)
            mk = DM_NONE;
        else if (mk != DM_LIGHT && mk != DM_GLOW && mk != DM_NONE)
            lamb = true;
    }
    if (mk == DM_LIGHT || mk == DM_GLOW) {
        light_hit<G>(P, r, ro, ms, h.t, h.rod, cnt, nullptr);
        return;
    }
    if (mk == DM_NONE) {
        surface_contrib(P, r, ro, cnt);
        Ray c;
        ray_origin(P, r, GB_TRANS, f3(1.f, 1.f, 1.f), false, GB_C_PASS, c, nullptr);
        c.org = hp;
        c.dir = r.dir;
        c.origin = h.obj;
        if (G)
            c.adj = r.adj;
        push_ray<G>(P, c);
        return;
    }
    float4 m0, m1;
    if (lamb) {
        mk = DM_PLASTIC;
        m0 = make_float4(DM_PLASTIC, (float)M_PI, (float)M_PI, (float)M_PI);
        m1 = make_float4(0.f, 0.f, 0.f, 0.f);
        ms = -1;                                 /* no material parameter on the path */
    } else {
        m0 = S.mat[2 * ms];
        m1 = S.mat[2 * ms + 1];
    }
    float3 n = h.n;
    float rod = h.rod;
    if (rod < 0.f) {                            /* flipsurface (backvis on) */
        rod = -rod;
        n = -n;
    }
    surface_contrib(P, r, ro, cnt);
    if (mk == DM_GLASS) {
        float3 mc = f3(m0.y, m0.z, m0.w);
        float rindex = m1.x;
        bool hastrans = maxc(mc) > 1e-15f;
        mc = f3(fmaxf(mc.x, 1e-15f), fmaxf(mc.y, 1e-15f), fmaxf(mc.z, 1e-15f));
        float pdot = rod;
        float cos2 = sqrtf((1.f - 1.f / (rindex * rindex)) + pdot * pdot / (rindex * rindex));
        if (hastrans)
            mc = f3(powf(mc.x, 1.f / cos2), powf(mc.y, 1.f / cos2), powf(mc.z, 1.f / cos2));
        float r1e = (pdot - rindex * cos2) / (pdot + rindex * cos2);
        r1e *= r1e;
        float r1m = (1.f / pdot - rindex / cos2) / (1.f / pdot + rindex / cos2);
        r1m *= r1m;
        float mm[3] = {mc.x, mc.y, mc.z}, tc[3], rc[3];
        for (int i = 0; i < 3; i++) {
            float d = mm[i];
            tc[i] = .5f * (1.f - r1e) * (1.f - r1e) * d / (1.f - r1e * r1e * d * d) +
                    .5f * (1.f - r1m) * (1.f - r1m) * d / (1.f - r1m * r1m * d * d);
            float d2 = d * d;
            rc[i] = .5f * r1e * (1.f + (1.f - 2.f * r1e) * d2) / (1.f - r1e * r1e * d2) +
                    .5f * r1m * (1.f + (1.f - 2.f * r1m) * d2) / (1.f - r1m * r1m * d2);
        }
        if (hastrans) {
            Ray c;
            if (ray_origin(P, r, GB_TRANS, f3(tc[0], tc[1], tc[2]), true, GB_C_TRANS, c, nullptr)) {
                c.org = hp;
                c.dir = r.dir;
                c.origin = h.obj;
                if (G) {
                    c.adj = r.adj;
                    adj_append(c.adj, ms, GB_ADJ_GLASST, pdot);
                }
                push_ray<G>(P, c);
            }
        }
        Ray c;
        if (ray_origin(P, r, GB_REFLECTED, f3(rc[0], rc[1], rc[2]), true, GB_C_REFL, c, nullptr)) {
            c.org = hp;
            c.dir = normalize3(r.dir + n * (2.f * pdot));
            c.origin = h.obj;
            if (G) {
                c.adj = r.adj;
                adj_append(c.adj, ms, GB_ADJ_GLASSR, pdot);
            }
            push_ray<G>(P, c);
        }
        return;
    }
    if (mk == DM_MIRROR) {                       /* rt/m_mirror.c: black from behind, else reflected */
        if (h.rod < 0.f)
            return;
        Ray c;
        if (ray_origin(P, r, GB_REFLECTED, f3(m0.y, m0.z, m0.w), true, GB_C_REFL, c, nullptr)) {
            c.org = hp;
            c.dir = normalize3(r.dir + h.n * (2.f * h.rod));
            c.origin = h.obj;
            if (G)
                c.adj = r.adj;
            push_ray<G>(P, c);
        }
        return;
    }
    /* plastic / metal */
    int okd = S.obj[ro].x & 0xff;
    float3 pn = n;
    float pd = rod;
    const bool tex = VN && h.obj >= S.nobjs && mesh_pnorm(S, h.obj, hp, r.dir, h.n, h.rod < 0.f, rod, pn, pd);
    Surf su;
    setup_surf(P, mk, m0, m1, n, pn, pd, (okd == DK_FACE || okd == DK_RING) && !tex, su);
    if (su.tran && su.pure) {                    /* the transmitted ray (rt/normal.c:280-301) */
        Ray c;
        if (ray_origin(P, r, GB_TRANS, su.mcolor * su.tspec, true, GB_C_TRANS, c, nullptr)) {
            c.org = hp;
            c.dir = r.dir;
            c.origin = h.obj;
            if (G)
                c.adj = r.adj;
            push_ray<G>(P, c);
        }
    }
    if (su.refl && su.pure) {
        Ray c;
        if (ray_origin(P, r, GB_REFLECTED, su.scolor, true, GB_C_REFL, c, nullptr)) {
            c.org = hp;
            c.dir = normalize3(r.dir + su.pnorm * (2.f * su.pdot));
            if (tex && dot3(c.dir, n) <= D_FTINY)          /* would enter the surface */
                c.dir = normalize3(r.dir + n * (2.f * rod));
            c.origin = h.obj;
            if (G)                               /* specular color: not a parameter */
                c.adj = r.adj;
            push_ray<G>(P, c);
        }
    }
    if (su.pure && su.rdiff <= D_FTINY && su.tdiff <= D_FTINY)
        return;
    if (su.rdiff > D_FTINY) {
        float3 aval = su.mcolor * su.rdiff;
        if (su.rblt)
            aval = aval + su.scolor;
        /* the hemisphere about the surface normal, on the side the
         * shading normal faces (rt/ambient.c:269-279) */
        if (tex && dot3(su.pnorm, n) < 0.f)
            ambient_side<G>(P, r, aval, -n, true, hp, h.obj, ms);
        else
            ambient_side<G>(P, r, aval, n, false, hp, h.obj, ms);
    }
    if (su.tdiff > D_FTINY)                      /* ambient from the other side (trans) */
        ambient_back<G>(P, r, su.mcolor * (su.tblt ? su.trans : su.tdiff), -n, hp, h.obj, ms);
    if (S.nsrc > 0)
        direct<G>(P, r, hp, su, h.obj, cnt, ms);
    /* the rough specular lobes (the reference samples them before the
     * diffuse terms; every draw is keyed by the path, so the order is free,
     * and last keeps the fewest values live across the call) */
    if (!su.pure && ((su.refl && !su.rblt) || (su.tran && !su.tblt)))
        gaussamp<G>(P, r, su, n, rod, hp, h.obj);
}

/* Persistent work loop: each warp takes work items 32 at a time with one
 * atomic, so warps that finish early take more instead of idling.  body(i)
 * processes item i. */
template <typename Body>
__device__ __forceinline__ void persistent_items(unsigned long long *work, unsigned long long total, Body body)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32ull);
        base = __shfl_sync(FULL, base, 0);
        if (base >= total)
            break;
        unsigned long long i = base + lane;
        if (i < total)
            body(i);
    }
}

/* hit record of the trace kernels: 32 bytes, two float4 */
__device__ __forceinline__ void store_hit(gb_qhit *q, const Hit &h)
{
    float4 *p = reinterpret_cast<float4 *>(q);
    p[0] = make_float4(__int_as_float(h.obj), h.t, h.rod, h.n.x);
    p[1] = make_float4(h.n.y, h.n.z, 0.f, 0.f);
}

__device__ __forceinline__ Hit load_hit(const gb_qhit *q)
{
    const float4 *p = reinterpret_cast<const float4 *>(q);
    float4 a = p[0], b = p[1];
    Hit h;
    h.obj = __float_as_int(a.x);
    h.t = a.y;
    h.rod = a.z;
    h.n = f3(a.w, b.x, b.y);
    return h;
}

/* -------------------------------------------------------------- kernels */

/* -I sensor: the Lambertian pretend-hit, its direct part and its frame */
template <bool G>
__global__ void k_root(gb_run P)
{
    if (G)
        grad_begin(P);
    Counters cnt = {0, 0, 0, 0, 0};
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        const double *sv = P.sensors + 6 * s;
        float3 org = f3((float)sv[0], (float)sv[1], (float)sv[2]);
        float3 dir = normalize3(f3((float)sv[3], (float)sv[4], (float)sv[5]));
        Ray r;
        r.org = f3((float)(sv[0] + 1.1e-4 * sv[3]), (float)(sv[1] + 1.1e-4 * sv[4]), (float)(sv[2] + 1.1e-4 * sv[5]));
        r.dir = -dir;
        r.coef = f3(1.f, 1.f, 1.f);
        r.weight = 1.f;
        r.lcoef = 1.f;
        r.origin = -1;
        r.rsrc = -1;
        r.crtype = GB_PRIMARY;
        r.rlvl = 0;
        r.adepth = 0;
        r.path = GB_ROOT_PATH(P.replica);
        r.sensor = (uint32_t)(s + P.sensor_base);
        r.tag = GB_NOTAG;
        r.adj.n = 0;
        float3 hp = f3((float)(sv[0] + 1e-4 * sv[3]), (float)(sv[1] + 1e-4 * sv[4]), (float)(sv[2] + 1e-4 * sv[5]));
        Surf su;
        su.mcolor = f3(D_PI, D_PI, D_PI);
        su.scolor = f3(0.f, 0.f, 0.f);
        su.pnorm = dir;
        su.rdiff = 1.f;
        su.rspec = 0.f;
        su.alpha2 = 0.f;
        su.pdot = 1.f;
        su.pure = true;
        su.refl = false;
        su.rblt = false;
        su.flat = false;
        su.trans = su.tspec = su.tdiff = 0.f;
        su.tran = su.tblt = false;
        if (P.S.nsrc > 0)
            direct<G>(P, r, hp, su, -1, cnt, -1);
        if (P.root_n > 0) {
            Hemi hm;
            make_hemi(P, r, su.mcolor, dir, hm);
            gb_rootrec *rr = P.roots + s;
            rr->hp[0] = hp.x; rr->hp[1] = hp.y; rr->hp[2] = hp.z;
            rr->nrm[0] = dir.x; rr->nrm[1] = dir.y; rr->nrm[2] = dir.z;
            rr->ux[0] = hm.ux.x; rr->ux[1] = hm.ux.y; rr->ux[2] = hm.ux.z;
            rr->n = hm.n;
            /* hm.n >= 4: placed by k_root_draws and k_root_place */
        } else if (P.av[0] != 0.f || P.av[1] != 0.f || P.av[2] != 0.f) {
            add_value(P, r.sensor, GB_NOTAG, su.mcolor * f3(P.av[0], P.av[1], P.av[2]));
        }
    }
    flush_counters(P, cnt);
    if (G)
        grad_end(P);
}

/* the root ray and hemisphere of -I sensor s from its record (as k_root
 * made them) */
__device__ __forceinline__ void root_parent(const gb_run &P, long long s, Ray &parent, Hemi &hm)
{
    const gb_rootrec *rr = P.roots + s;
    parent.org = f3(rr->hp[0], rr->hp[1], rr->hp[2]);
    parent.coef = f3(1.f, 1.f, 1.f);
    parent.weight = 1.f;
    parent.lcoef = 1.f;
    parent.origin = -1;
    parent.rsrc = -1;
    parent.crtype = GB_PRIMARY;
    parent.rlvl = 0;
    parent.adepth = 0;
    parent.path = GB_ROOT_PATH(P.replica);
    parent.sensor = (uint32_t)(s + P.sensor_base);
    parent.tag = GB_NOTAG;
    parent.adj.n = 0;
    hm.n = rr->n;
    hm.atyp = GB_RAMBIENT;
    hm.onrm = f3(rr->nrm[0], rr->nrm[1], rr->nrm[2]);
    hm.ux = f3(rr->ux[0], rr->ux[1], rr->ux[2]);
    hm.uy = cross3(hm.onrm, hm.ux);
    float a = D_PI / (float)(hm.n * hm.n);
    hm.acoef = f3(a, a, a);
}

/* The random numbers of the root placement, drawn in parallel: for every
 * (sensor, stratum) the stratum's creation draw (ray_origin: Russian
 * roulette and the jitter), and for every sensor the first fill of its lot
 * (the 512 positions gb_trade_patchsamp draws on its first call, from the
 * lot stream's blocks 0..255, in gb_lot_u32's order).  The sequential
 * placement then reads them instead of drawing. */
__global__ void k_root_draws(gb_run P)
{
    const long long nn = (long long)P.root_n * P.root_n;
    const long long total = nn * P.nsensors, lots = (long long)P.nsensors * (GB_XLOT / 2);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total + lots;
         g += (long long)gridDim.x * blockDim.x) {
        if (g < total) {
            const long long s = g / nn;
            const int k = (int)(g - s * nn);
            Ray parent, c;
            Hemi hm;
            root_parent(P, s, parent, hm);
            float4 u;
            bool alive = ray_origin(P, parent, hm.atyp, hm.acoef, true, GB_C_STRATUM(k), c, &u);
            P.root_draw[g] = make_float2(alive ? u.y : 3.f, u.z);
        } else {
            const long long h = g - total, s = h / (GB_XLOT / 2);
            const int b = (int)(h - s * (GB_XLOT / 2));          /* lot block: positions 2b, 2b+1 */
            gb_u4 u = gb_draw(GB_ROOT_PATH(P.replica), (uint32_t)(s + P.sensor_base), GB_G_LOT0 + b, P.k0, P.k1);
            float4 *o = reinterpret_cast<float4 *>(P.root_lot + s * (2 * GB_XLOT)) + b;
            *o = make_float4(gb_u01(u.v[3]), gb_u01(u.v[2]), gb_u01(u.v[1]), gb_u01(u.v[0]));
        }
    }
}

/* The sequential placement of every -I sensor's first hemisphere (n >= 4),
 * one thread per sensor, from the precomputed draws and lot. */
__global__ void k_root_place(gb_run P)
{
    const long long nn = (long long)P.root_n * P.root_n;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        const int n = P.roots[s].n;
        if (n < 4 || n > MAX_HEMI_N)
            continue;
        gb_lot L;
        gb_lot_init(&L, GB_ROOT_PATH(P.replica), (uint32_t)(s + P.sensor_base), P.k0, P.k1);
        const float4 *lf = reinterpret_cast<const float4 *>(P.root_lot + s * (2 * GB_XLOT));
        for (int b = 0; b < GB_XLOT / 2; b++) {
            float4 v = lf[b];
            L.lot[2 * b][0] = v.x;
            L.lot[2 * b][1] = v.y;
            L.lot[2 * b + 1][0] = v.z;
            L.lot[2 * b + 1][1] = v.w;
        }
        L.gterm[GB_COTHER] = GB_XLOT;                  /* filled: the lazy fill is skipped */
        L.blk = GB_XLOT / 2;
        float rows[2][MAX_HEMI_N][2];
        float (*prev)[2] = rows[0], (*cur)[2] = rows[1];
        for (int k = 0; k < n; k++) {
            rows[0][k][0] = rows[0][k][1] = 2.f;
            rows[1][k][0] = rows[1][k][1] = 2.f;
        }
        const float2 *dr = P.root_draw + s * nn;
        float2 *out = P.root_spt + s * nn;
        for (int i = n - 1; i >= 0; i--) {
            for (int j = n - 1; j >= 0; j--) {
                const int k = i * n + j;
                const float2 d = dr[k];
                float sp[2] = {2.f, 2.f};
                if (d.x < 1.5f)
                    gb_place_sample(&L, n, i, j, d.x, d.y, i + 1 < n ? (const float(*)[2])prev : nullptr,
                                    (const float(*)[2])cur, sp);
                cur[j][0] = sp[0];
                cur[j][1] = sp[1];
                out[k] = make_float2(sp[0], sp[1]);
            }
            float(*t)[2] = prev;
            prev = cur;
            cur = t;
            for (int k = 0; k < n; k++)
                cur[k][0] = cur[k][1] = 2.f;
        }
    }
}

/* first hemisphere of every -I sensor: one ray per (sensor, stratum) into
 * the queue of the first generation */
template <bool G>
__global__ void __launch_bounds__(256) k_expand_root(gb_run P)
{
    const long long nn = (long long)P.root_n * P.root_n;
    const unsigned long long total = (unsigned long long)(nn * P.nsensors);
    persistent_items(P.work, total, [&](unsigned long long g) {
        long long s = (long long)(g / (unsigned long long)nn);
        int k = (int)(g - (unsigned long long)s * nn);
        Ray parent;
        Hemi hm;
        root_parent(P, s, parent, hm);
        const float *sp = nullptr;
        float2 pk;
        if (hm.n >= 4) {
            pk = P.root_spt[g];
            if (pk.x > 1.5f)
                return;                       /* stratum died in Russian roulette */
            sp = &pk.x;
        }
        Ray c;
        if (hemi_child(P, parent, hm, parent.org, -1, k, sp, c)) {
            c.adj.n = 0;                       /* the -I sensor is not a parameter */
            if (P.ss_val)                      /* its value is kept per stratum */
                c.tag = (uint32_t)g;
            push_ray<G>(P, c);
        }
    });
}

/* Ambient super-sampling of the -I first hemispheres (rt/ambcomp.c:256-346
 * getambdiffs and ambsupersamp, called from samp_hemi :403-409), one
 * thread per sensor, after the first pass has traced every stratum's whole
 * path tree into ss_val.  A hemisphere of more than 7 x 7 strata, all of
 * them alive, gets (int)(as * wt + .5) extra samples when that is at least
 * four times its side: strata are weighted by the squared brightness
 * differences with their neighbours (corrected for the number of
 * neighbours and blurred), and each receives its share with random
 * rounding, in row order, stopping at a sample lost to Russian roulette or
 * when the budget is spent.  Extra sample m of stratum k is child
 * GB_C_SSAMP(k, m) with a fresh jitter in the stratum and no collision
 * test; it is queued for the second pass with the stratum's tag. */
#define GB_MINADIV 7
#define GB_CIE_RF 0.265074126f          /* common/color.h:253 default weights of pbright */
#define GB_CIE_GF 0.670114631f
#define GB_CIE_BF 0.064811243f
__device__ __forceinline__ float pbright(const double *v)
{
    return GB_CIE_RF * (float)v[0] + GB_CIE_GF * (float)v[1] + GB_CIE_BF * (float)v[2];
}

__global__ void k_ssamp_plan(gb_run P)
{
    const long long nn = (long long)P.root_n * P.root_n;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        Ray parent;
        Hemi hm;
        root_parent(P, s, parent, hm);
        const int n = hm.n;
        if (n * n <= GB_MINADIV * GB_MINADIV || n < 4)
            continue;
        const float2 *dr = P.root_draw + s * nn;
        bool all = true;                               /* every stratum sampled (sampOK) */
        for (int k = 0; k < n * n && all; k++)
            all = dr[k].x < 1.5f;
        if (!all)
            continue;
        /* samp_hemi's weight for the Lambertian at weight 1 (make_hemi) */
        float wt = 1.f, d = (float)D_PI * 0.8f / ((float)P.ad * P.minweight + 1e-20f);
        if (wt > d)
            wt = d;
        int cnt = (int)((float)P.ss_samples * wt + .5f);
        if (cnt < 4 * n)
            continue;
        const double *v = P.ss_val + 3ull * (s * nn);
        float *earr = P.ss_err + 2ull * (s * nn), *ep2 = earr + n * n;
        const float normf =
            1.f / (GB_CIE_RF * hm.acoef.x + GB_CIE_GF * hm.acoef.y + GB_CIE_BF * hm.acoef.z + D_FTINY);
        for (int k = 0; k < 2 * n * n; k++)
            earr[k] = 0.f;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const int k = i * n + j;
                const float b = pbright(v + 3 * k);
                float b1, d2;
                if (i) {                               /* from above */
                    b1 = pbright(v + 3 * (k - n));
                    d2 = b - b1;
                    d2 *= d2 * normf / (b + b1 + D_FTINY);
                    ep2[k] += d2;
                    ep2[k - n] += d2;
                }
                if (!j)
                    continue;
                b1 = pbright(v + 3 * (k - 1));         /* from behind */
                d2 = b - b1;
                d2 *= d2 * normf / (b + b1 + D_FTINY);
                ep2[k] += d2;
                ep2[k - 1] += d2;
                if (!i)
                    continue;
                b1 = pbright(v + 3 * (k - n - 1));     /* diagonal */
                d2 = b - b1;
                d2 *= d2 * normf / (b + b1 + D_FTINY);
                ep2[k] += d2;
                ep2[k - n - 1] += d2;
            }
        ep2[0] *= 6.f / 3.f;                           /* corners and edges: fewer neighbours */
        ep2[n - 1] *= 6.f / 3.f;
        ep2[(n - 1) * n] *= 6.f / 3.f;
        ep2[(n - 1) * n + n - 1] *= 6.f / 3.f;
        for (int i = 1; i < n - 1; i++) {
            ep2[i * n] *= 6.f / 5.f;
            ep2[i * n + n - 1] *= 6.f / 5.f;
        }
        for (int j = 1; j < n - 1; j++) {
            ep2[j] *= 6.f / 5.f;
            ep2[(n - 1) * n + j] *= 6.f / 5.f;
        }
        for (int i = 0; i < n - 1; i++)                /* blur into the final map */
            for (int j = 0; j < n - 1; j++) {
                const int k = i * n + j;
                earr[k] += .5f * ep2[k] + .125f * (ep2[k + 1] + ep2[k + n]);
                earr[k + 1] += .125f * ep2[k];
                earr[k + n] += .125f * ep2[k];
            }
        float e2rem = 0.f;
        for (int k = n * n; k--;)
            e2rem += earr[k];
        for (int k = 0; k < n * n; k++) {
            if (e2rem <= D_FTINY)
                break;
            const gb_u4 q = gb_draw(parent.path, parent.sensor, GB_G_SSAMP + (uint32_t)(k >> 2), P.k0, P.k1);
            const int nss = (int)(earr[k] / e2rem * (float)cnt + gb_u01(q.v[k & 3]));
            for (int m = 1; m <= nss; m++) {
                Ray c;
                if (!hemi_child(P, parent, hm, parent.org, -1, k, nullptr, c, GB_C_SSAMP(k, m)))
                    break;
                c.adj.n = 0;
                c.tag = (uint32_t)(s * nn + k);
                push_ray(P, c);
                P.ss_cnt[s * nn + k]++;
                if (!--cnt)
                    break;
            }
            if (!cnt)
                break;
            e2rem -= earr[k];
        }
    }
}

/* each super-sampled stratum's value is the mean of its samples; the
 * first hemisphere's value, their sum, goes to the sensor */
__global__ void k_ssamp_final(gb_run P)
{
    const long long nn = (long long)P.root_n * P.root_n;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        double a[3] = {0., 0., 0.};
        const double *v = P.ss_val + 3ull * (s * nn);
        const int *m = P.ss_cnt + s * nn;
        for (long long k = 0; k < nn; k++) {
            const double w = 1.0 / (1.0 + m[k]);
            a[0] += v[3 * k] * w;
            a[1] += v[3 * k + 1] * w;
            a[2] += v[3 * k + 2] * w;
        }
        double *o = P.value + 3ull * s;
        o[0] += a[0];
        o[1] += a[1];
        o[2] += a[2];
    }
}

/* radiance-mode primaries (rt/rtrace.c:436-468, rt/rcontrib.c:343-353)
 * into the queue of the first generation */
template <bool G>
__global__ void k_primary(gb_run P)
{
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        const double *sv = P.sensors + 6 * s;
        Ray r;
        r.org = f3((float)sv[0], (float)sv[1], (float)sv[2]);
        r.dir = normalize3(f3((float)sv[3], (float)sv[4], (float)sv[5]));
        r.coef = f3(1.f, 1.f, 1.f);
        r.weight = 1.f;
        r.lcoef = 1.f;
        r.origin = -1;
        r.rsrc = -1;
        r.crtype = GB_PRIMARY;
        r.rlvl = 0;
        r.adepth = 0;
        r.path = GB_ROOT_PATH(P.replica);
        r.sensor = (uint32_t)(s + P.sensor_base);
        r.tag = GB_NOTAG;
        r.adj.n = 0;
        push_ray<G>(P, r);
    }
}

/* One generation, first half: the octree walk of every queued ray
 * (rt/raytrace.c:595-793), its result written beside it.  Only the walk
 * runs here, so the lanes of a warp execute one loop body, one iteration
 * (an object test or a step to the next leaf) at a time.  Walks differ in
 * length by an order of magnitude, so a lane whose walk ends takes the next
 * queued ray at once (the warp fetches for all its idle lanes with one
 * atomic once a quarter of them wait, or when none is busy) instead of
 * idling until the longest walk of the warp ends.  The walk is latency
 * bound: four blocks of 256 threads per SM (64 registers) hide more of it
 * than two blocks at 102 registers; the descent stacks of a block sit in
 * shared memory (25.6 KB), one column per thread. */
#define TRACE_BLOCK 256
/* descent stack of one thread: a column of a block-wide shared array */
struct ColumnStack {
    int *p;
    __device__ __forceinline__ int &operator[](int i) { return p[i * TRACE_BLOCK]; }
};

template <bool INST>
__global__ void __launch_bounds__(TRACE_BLOCK, 4) k_trace(gb_run P)
{
    __shared__ int stack_cols[(GRID_BITS + 1) * TRACE_BLOCK];
    ColumnStack stk{stack_cols + threadIdx.x};
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    Counters cnt = {0, 0, 0, 0, 0};
    unsigned long long total = *P.qin_count;
    if (total > (unsigned long long)P.qcap)
        total = P.qcap;
    Walk W;
    /* scenes with instances defer the walks that meet one to k_trace_inst;
     * the others carry no instance handling at all */
    typedef typename std::conditional<INST, DeferCube, PlainCube>::type Cube;
    const Cube C{};
    unsigned long long cur = 0;
    bool active = false, exhausted = false;
    const int refill = P.walk_refill > 0 ? P.walk_refill : 8;
    for (;;) {
        const unsigned idle = __ballot_sync(FULL, !active);
        if (!exhausted && (__popc(idle) >= refill || idle == FULL)) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader)
                base = atomicAdd(P.work, (unsigned long long)__popc(idle));
            base = __shfl_sync(FULL, base, leader);
            if (base + __popc(idle) >= total)
                exhausted = true;
            if (!active) {
                const unsigned long long i = base + __popc(idle & ((1u << lane) - 1u));
                if (i < total) {
                    const float4 *q = reinterpret_cast<const float4 *>(P.qin + i);
                    const float4 a = q[0], b = q[1], c = q[2];
                    cur = i;
                    cnt.rays++;
                    active = walk_begin(P.S, C, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), __float_as_int(c.w), W,
                                        stk);
                    if (!active)
                        store_hit(P.hits + i, W.best);     /* missed the scene cube */
                }
            }
        }
        if (!__any_sync(FULL, active)) {
            if (exhausted)
                break;
            continue;
        }
        if (active && walk_iter(P.S, C, W, stk)) {
            uint32_t st[3] = {0, 0, 0};
            walk_tally(W, st);
            cnt.add(st);
            if (INST && W.best.obj == HIT_DEFER)   /* met an instance: walked again there */
                P.slow[atomicAdd(P.slow_count, 1ull)] = (uint32_t)cur;
            else
                store_hit(P.hits + cur, W.best);
            active = false;
        }
    }
    flush_counters(P, cnt);
}

/* The walks k_trace handed over because they met an instance: walked
 * again from the start with the instances' octrees (hit_instance), one
 * thread per ray.  Runs after k_trace in scenes with instances only. */
__global__ void __launch_bounds__(128) k_trace_inst(gb_run P)
{
    Counters cnt = {0, 0, 0, 0, 0};
    const unsigned long long n = *P.slow_count;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long q = P.slow[i];
        const float4 *r = reinterpret_cast<const float4 *>(P.qin + q);
        const float4 a = r[0], b = r[1], c = r[2];
        Hit h;
        uint32_t st[3] = {0, 0, 0};
        local_hit(P.S, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), __float_as_int(c.w), h, st);
        cnt.add(st);
        store_hit(P.hits + q, h);
    }
    flush_counters(P, cnt);
}

/* One generation, second half: shade every traced ray and queue its
 * children for the next generation. */
template <bool G, bool VN = false>
__global__ void __launch_bounds__(256, 4) k_shade(gb_run P)
{
    if (G)
        grad_begin(P);
    Counters cnt = {0, 0, 0, 0, 0};
    unsigned long long n = *P.qin_count;
    if (n > (unsigned long long)P.qcap)
        n = P.qcap;
    persistent_items(P.work, n, [&](unsigned long long g) {
        Ray r = load_ray(P.qin + g);
        if (G)
            r.adj = P.adj_in[g];
        if (P.tag_in)
            r.tag = P.tag_in[g];
        const Hit h = load_hit(P.hits + g);
        shade_ray<G, VN>(P, r, h, cnt);
    });
    flush_counters(P, cnt);
    if (G)
        grad_end(P);
}

/* castonly rtrace (rt/rtrace.c:398-411 raycast): first intersection only */
__global__ void k_cast(gb_run P, int *hit_obj, float *hit_t, float *hit_pn)
{
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < P.nsensors;
         s += (long long)gridDim.x * blockDim.x) {
        const double *sv = P.sensors + 6 * s;
        float3 org = f3((float)sv[0], (float)sv[1], (float)sv[2]);
        float3 dir = normalize3(f3((float)sv[3], (float)sv[4], (float)sv[5]));
        Hit h;
        uint32_t st[3] = {0, 0, 0};
        int obj = -1;
        float t = D_FHUGE;
        float3 n = f3(0.f, 0.f, 0.f);
        if (local_hit(P.S, org, dir, -1, h, st)) {
            obj = sid_object(P.S, h.obj);
            t = h.t;
            n = h.n;
        } else {
            int sidx = source_hit(P.S, dir, -1, GB_PRIMARY);
            if (sidx >= 0)
                obj = P.S.src[sidx].so;
        }
        hit_obj[s] = obj;
        if (hit_t)
            hit_t[s] = t;
        if (hit_pn) {
            float3 p = org + dir * t;
            float *o = hit_pn + 6 * s;
            o[0] = p.x; o[1] = p.y; o[2] = p.z;
            o[3] = n.x; o[4] = n.y; o[5] = n.z;
        }
    }
}

/* ------------------------------------------------------ host launchers */

static int grid_for(long long n, int block, int sms)
{
    long long g = (n + block - 1) / block;
    long long cap = (long long)sms * 8;
    if (g > cap)
        g = cap;
    if (g < 1)
        g = 1;
    return (int)g;
}

int gb_launch_cast(const gb_run *P, int *hit_obj, float *hit_t, float *hit_pn, cudaStream_t st, int sms)
{
    k_cast<<<grid_for(P->nsensors, 128, sms), 128, 0, st>>>(*P, hit_obj, hit_t, hit_pn);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* dynamic shared memory of a gradient launch: the per-block accumulators
 * when the material slots fit in 32 KB, else none (global accumulation) */
static size_t grad_smem_bytes(const gb_run *P, gb_run &R)
{
    R = *P;
    size_t b = (size_t)P->nslots * 3 * sizeof(double);
    R.grad_shared = b <= 32768;
    return R.grad_shared ? b : 0;
}

int gb_launch_root(const gb_run *P, cudaStream_t st, int sms)
{
    k_root<false><<<grid_for(P->nsensors, 32, sms), 32, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_root_draws(const gb_run *P, cudaStream_t st, int sms)
{
    long long work = (long long)P->root_n * P->root_n * P->nsensors + P->nsensors * (GB_XLOT / 2);
    k_root_draws<<<grid_for(work, 256, sms), 256, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_root_place(const gb_run *P, cudaStream_t st, int sms)
{
    /* a few sensors per warp: the placement is a long dependent chain per
     * sensor, so more warps on every SM hide more of its latency */
    k_root_place<<<grid_for(P->nsensors, 8, sms), 8, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_ssamp_plan(const gb_run *P, cudaStream_t st, int sms)
{
    k_ssamp_plan<<<grid_for(P->nsensors, 32, sms), 32, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_ssamp_final(const gb_run *P, cudaStream_t st, int sms)
{
    k_ssamp_final<<<grid_for(P->nsensors, 128, sms), 128, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_root_grad(const gb_run *P, cudaStream_t st, int sms)
{
    gb_run R;
    size_t sm = grad_smem_bytes(P, R);
    k_root<true><<<grid_for(P->nsensors, 32, sms), 32, sm, st>>>(R);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* persistent kernels: exactly the blocks that fit at once */
template <typename K>
static int resident_grid(K kernel, int block, int sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * sms;
}

int gb_launch_expand_root(const gb_run *P, cudaStream_t st, int sms)
{
    static int grid = 0;
    if (!grid)
        grid = resident_grid(k_expand_root<false>, 256, sms);
    k_expand_root<false><<<grid, 256, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_expand_root_grad(const gb_run *P, cudaStream_t st, int sms)
{
    static int grid = 0;
    if (!grid)
        grid = resident_grid(k_expand_root<true>, 256, sms);
    k_expand_root<true><<<grid, 256, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_primary(const gb_run *P, cudaStream_t st, int sms)
{
    k_primary<false><<<grid_for(P->nsensors, 128, sms), 128, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_primary_grad(const gb_run *P, cudaStream_t st, int sms)
{
    k_primary<true><<<grid_for(P->nsensors, 128, sms), 128, 0, st>>>(*P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* ---- ceilings of the walk: random 64-byte reads from an L2-resident table.
 * Each thread reads `iters` records of 4 x float4: at independent random
 * places (gather), or at places that depend on the last record's contents
 * (chase: a chain of dependent loads, as the walk's descent and object
 * records are).  Launched like the walk kernel (256 threads, 4 blocks per
 * SM). */
__global__ void __launch_bounds__(256, 4) k_probe_l2(const float4 *__restrict__ table, uint32_t nrec, int iters,
                                                    int chase, float *sink)
{
    uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u + 12345u;
    float acc = 0.f;
    for (int it = 0; it < iters; it++) {
        const uint32_t r = x % nrec;
        const float4 *p = table + 4 * (size_t)r;
        const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
        acc += a.x + b.y + c.z + d.w;
        if (chase)
            x = (__float_as_uint(a.y) ^ (x * 1664525u)) + 1013904223u;
        else
            x = x * 1664525u + 1013904223u;
    }
    if (acc == 1234.5f)
        sink[0] = acc;
}

int gb_launch_probe_l2(const float4 *table, uint32_t nrec, int iters, int chase, float *sink, cudaStream_t st,
                       int sms)
{
    k_probe_l2<<<4 * sms, 256, 0, st>>>(table, nrec, iters, chase, sink);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_trace(const gb_run *P, cudaStream_t st, int sms)
{
    static int grid = 0, grid_inst = 0;
    if (!grid)
        grid = resident_grid(k_trace<false>, TRACE_BLOCK, sms);
    if (P->S.ninst == 0) {
        const int g = P->walk_blocks_per_sm > 0 ? std::min(grid, P->walk_blocks_per_sm * sms) : grid;
        k_trace<false><<<g, TRACE_BLOCK, 0, st>>>(*P);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
    if (!grid_inst)
        grid_inst = resident_grid(k_trace<true>, TRACE_BLOCK, sms);
    const int gi = P->walk_blocks_per_sm > 0 ? std::min(grid_inst, P->walk_blocks_per_sm * sms) : grid_inst;
    k_trace<true><<<gi, TRACE_BLOCK, 0, st>>>(*P);
    if (cudaGetLastError() != cudaSuccess)
        return -1;
    {
        k_trace_inst<<<sms * 8, 128, 0, st>>>(*P);
        if (cudaGetLastError() != cudaSuccess)
            return -1;
    }
    return 0;
}

int gb_launch_shade(const gb_run *P, cudaStream_t st, int sms)
{
    /* scenes with smooth mesh triangles: the kernel that perturbs their
     * shading normals; the others carry none of it */
    static int grid = 0, grid_vn = 0;
    if (P->S.has_vnorm) {
        if (!grid_vn)
            grid_vn = resident_grid(k_shade<false, true>, 256, sms);
        k_shade<false, true><<<grid_vn, 256, 0, st>>>(*P);
    } else {
        if (!grid)
            grid = resident_grid(k_shade<false>, 256, sms);
        k_shade<false><<<grid, 256, 0, st>>>(*P);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gb_launch_shade_grad(const gb_run *P, cudaStream_t st, int sms)
{
    gb_run R;
    size_t sm = grad_smem_bytes(P, R);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade<true>, 256, sm) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    k_shade<true><<<per_sm * sms, 256, sm, st>>>(R);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
