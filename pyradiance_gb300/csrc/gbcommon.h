/*
 * gbcommon.h -- definitions shared by the CUDA kernels, the host library and
 * the CPU oracle: ray-type bits, the counter-based random stream, path ids,
 * and the bin-program byte code.  Everything here is integer or
 * format-level, so every user produces bit-identical random numbers and
 * bin programs.
 */
#ifndef GB_COMMON_H
#define GB_COMMON_H

#include <stdint.h>

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD static inline
#endif

/* ray types (rt/ray.h:28-43) */
#define GB_PRIMARY   0x01
#define GB_RSHADOW   0x02
#define GB_REFLECTED 0x04
#define GB_RSPECULAR 0x08
#define GB_TRANS     0x10
#define GB_RAMBIENT  0x20
#define GB_TSPECULAR 0x40
#define GB_TSHADOW   0x80
#define GB_TAMBIENT  0x100
#define GB_SHADOW    (GB_RSHADOW | GB_TSHADOW)
#define GB_AMBIENT   (GB_RAMBIENT | GB_TAMBIENT)
#define GB_SPECULAR  (GB_RSPECULAR | GB_TSPECULAR)
#define GB_RAYREFL   (GB_RSHADOW | GB_REFLECTED | GB_RAMBIENT | GB_RSPECULAR)

/* ------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11).  Counter (c0..c3), key (k0, k1).
 */
typedef struct { uint32_t v[4]; } gb_u4;

GB_HD uint32_t gb_mulhilo(uint32_t a, uint32_t b, uint32_t *hi)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

GB_HD gb_u4 gb_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                      uint32_t k0, uint32_t k1)
{
    gb_u4 r;
    int i;
    for (i = 0; i < 10; i++) {
        uint32_t hi0, hi1;
        uint32_t lo0 = gb_mulhilo(0xD2511F53u, c0, &hi0);
        uint32_t lo1 = gb_mulhilo(0xCD9E8D57u, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    r.v[0] = c0;
    r.v[1] = c1;
    r.v[2] = c2;
    r.v[3] = c3;
    return r;
}

/* uniform in [0,1) with 24 random bits; exactly representable in float */
GB_HD float gb_u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

/* uniform integer in [0, m) from a 32-bit draw (common/urand.c irandom) */
GB_HD uint32_t gb_irand(uint32_t x, uint32_t m) { return (uint32_t)(((uint64_t)x * m) >> 32); }

/* Random draws of a ray: the stream is keyed by the run seed; the counter is
 * (path id low, path id high, sensor, group).  Groups:
 *   0  drawn when the ray is created: [0] Russian roulette, [1] [2] stratum
 *      jitter, [3] spare
 *   1  drawn at the ray's hit for a hemisphere frame: [0..2] perpendicular
 *      randomisation, [3] axis order
 *   2+ per source sample jitter (2 + source index)
 *   GB_G_SPECF  drawn at the hit for the frame of the specular lobe
 *   GB_G_SPEC+j two trials of specular lobe sampling per group: trial t
 *      uses words 2(t&1) and 2(t&1)+1 of group GB_G_SPEC + (t >> 1)
 *   GB_G_SSAMP+j drawn at a super-sampled hemisphere's parent: the random
 *      rounding of each stratum's share of the extra samples
 */
#define GB_G_CREATE 0u
#define GB_G_FRAME  1u
#define GB_G_SRC    2u
#define GB_G_SPECF  0x7F000000u
#define GB_G_SPEC   0x7F000001u
#define GB_G_TSPEC  0x7D000000u   /* transmitted specular lobe trials, as GB_G_SPEC */
#define GB_G_SSAMP  0x7E000000u   /* super-sampling allocation: stratum k uses word k&3 of group + (k >> 2) */

GB_HD gb_u4 gb_draw(uint64_t path, uint32_t sensor, uint32_t group, uint32_t k0, uint32_t k1)
{
    return gb_philox((uint32_t)path, (uint32_t)(path >> 32), sensor, group, k0, k1);
}

/* Child path id: a bijective 64-bit mix of (parent, child code). */
GB_HD uint64_t gb_child(uint64_t parent, uint32_t code)
{
    uint64_t z = parent + 0x9E3779B97F4A7C15ull * ((uint64_t)code + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* child codes */
#define GB_C_STRATUM(k) ((uint32_t)(k))            /* hemisphere stratum k < 2^20 */
#define GB_C_REFL       0x100001u
#define GB_C_TRANS      0x100002u
#define GB_C_PASS       0x100003u                   /* continue through (raytrans) */
#define GB_SPEC_MAXITER 10                            /* rt/normal.c:25 MAXITER */
#define GB_C_TSPEC(k)   (0x120000u + (uint32_t)(k))   /* transmitted specular lobe sample k < 2^16 */
#define GB_C_BACK       0x100004u                   /* the back side's hemisphere (its draws' parent) */
#define GB_C_SSAMP(k, m) (0x400000u + (uint32_t)(k) + ((uint32_t)(m) << 12))  /* extra sample m >= 1 of stratum k < 4096 */
#define GB_NOTAG 0xffffffffu
#define GB_C_SPEC(k)    (0x110000u + (uint32_t)(k))   /* specular lobe sample k < 2^16 */
#define GB_C_SHADOWP(s, p) (0x200000u + (uint32_t)(s) + ((uint32_t)(p) << 12))   /* partition p < 64 */
#define GB_C_SHADOW(s)  GB_C_SHADOWP(s, 0)
/* root path id of replica r of a sensor (replicas give independent samples) */
#define GB_ROOT_PATH(r) ((uint64_t)(r) * 0xD1B54A32D192ED03ull)

/* ------------------------------------------------------------------------
 * Hemisphere sample placement with the reference's collision avoidance
 * (rt/ambcomp.c:141-174 ambcollision, :60-128 trade_patchsamp, :177-215
 * ambsample).  For hemispheres of 4 x 4 strata or more the first sample of
 * each stratum is checked against the disk positions of the neighbouring
 * strata sampled before it (strata are visited from the last row and
 * column down); a sample closer than MINSDIST of a division is traded for a
 * position from a "used car lot" of earlier positions, up to 20 times, and
 * then placed uniformly in the middle 60% of its stratum.  The lot keeps
 * the reference's bookkeeping of corner classes.  The reference shares one
 * lot across the whole run; here each hemisphere owns one, filled from the
 * hemisphere's own random stream, so that hemispheres are independent.
 * Computed in float so that every user places samples identically.
 */
#define GB_XLOT 512
#define GB_MINSDIST 0.2f
#define GB_CFIRST 0
#define GB_COTHER 4
#define GB_CMAXTARGET 128            /* (int)(512 * 0.2 / 0.8) */
#define GB_G_LOT0 0x100u             /* first draw group of the lot stream */

typedef struct {
    float lot[GB_XLOT][2];
    int gterm[GB_COTHER + 1];
    uint64_t path;
    uint32_t sensor, k0, k1, blk;
    uint32_t buf[4];
    int nbuf;
} gb_lot;

GB_HD void gb_lot_init(gb_lot *L, uint64_t path, uint32_t sensor, uint32_t k0, uint32_t k1)
{
    int i;
    for (i = 0; i <= GB_COTHER; i++)
        L->gterm[i] = 0;
    L->path = path;
    L->sensor = sensor;
    L->k0 = k0;
    L->k1 = k1;
    L->blk = 0;
    L->nbuf = 0;
}

GB_HD uint32_t gb_lot_u32(gb_lot *L)
{
    if (L->nbuf == 0) {
        gb_u4 u = gb_draw(L->path, L->sensor, GB_G_LOT0 + L->blk++, L->k0, L->k1);
        L->buf[0] = u.v[0];
        L->buf[1] = u.v[1];
        L->buf[2] = u.v[2];
        L->buf[3] = u.v[3];
        L->nbuf = 4;
    }
    return L->buf[--L->nbuf];
}

GB_HD int gb_psample_class(const float ss[2])
{
    if (ss[0] < GB_MINSDIST) {
        if (ss[1] < GB_MINSDIST) return GB_CFIRST;
        if (ss[1] > 1.f - GB_MINSDIST) return GB_CFIRST + 2;
    } else if (ss[0] > 1.f - GB_MINSDIST) {
        if (ss[1] < GB_MINSDIST) return GB_CFIRST + 1;
        if (ss[1] > 1.f - GB_MINSDIST) return GB_CFIRST + 3;
    }
    return GB_COTHER;
}

GB_HD void gb_trade_patchsamp(gb_lot *L, float ss[2])
{
    float repl[2];
    int sclass, rclass, x;
    for (;;) {
        while (L->gterm[GB_COTHER] < GB_XLOT) {
            L->lot[L->gterm[GB_COTHER]][0] = gb_u01(gb_lot_u32(L));
            L->lot[L->gterm[GB_COTHER]][1] = gb_u01(gb_lot_u32(L));
            ++L->gterm[GB_COTHER];
        }
        sclass = gb_psample_class(ss);
        switch (sclass) {
        case GB_COTHER:
            x = (int)gb_irand(gb_lot_u32(L), L->gterm[GB_COTHER - 1] > GB_CMAXTARGET ?
                                                 (uint32_t)L->gterm[GB_COTHER - 1] : GB_XLOT);
            break;
        case GB_CFIRST:
            x = L->gterm[GB_CFIRST] + (int)gb_irand(gb_lot_u32(L), (uint32_t)(GB_XLOT - L->gterm[GB_CFIRST]));
            break;
        default:
            x = (int)gb_irand(gb_lot_u32(L), (uint32_t)(GB_XLOT - (L->gterm[sclass] - L->gterm[sclass - 1])));
            x += (x >= L->gterm[sclass - 1]) * (L->gterm[sclass] - L->gterm[sclass - 1]);
            break;
        }
        if (x >= GB_XLOT) {              /* trapped in a corner: re-initialise */
            int i;
            for (i = 0; i <= GB_COTHER; i++)
                L->gterm[i] = 0;
            continue;
        }
        break;
    }
    repl[0] = L->lot[x][0];
    repl[1] = L->lot[x][1];
    for (rclass = GB_CFIRST; rclass < GB_COTHER; rclass++)
        if (x < L->gterm[rclass])
            break;
    while (rclass > sclass) {
        L->lot[x][0] = L->lot[L->gterm[rclass - 1]][0];
        L->lot[x][1] = L->lot[L->gterm[rclass - 1]][1];
        x = L->gterm[--rclass]++;
    }
    while (rclass < sclass) {
        --L->gterm[rclass];
        L->lot[x][0] = L->lot[L->gterm[rclass]][0];
        L->lot[x][1] = L->lot[L->gterm[rclass]][1];
        x = L->gterm[rclass++];
    }
    L->lot[x][0] = ss[0];
    L->lot[x][1] = ss[1];
    ss[0] = repl[0];
    ss[1] = repl[1];
}

/* Shirley-Chiu concentric map (common/disk2square.c square2disk) in float */
#if defined(__CUDACC__)
#define GB_SINCOS(p, s, c) sincosf(p, s, c)
#else
#include <math.h>
#define GB_SINCOS(p, s, c) (*(s) = sinf(p), *(c) = cosf(p))
#endif
GB_HD void gb_square2disk(float ds[2], float sx, float sy)
{
    float a = 2.f * sx - 1.f, b = 2.f * sy - 1.f, r, phi, s, c;
    const float Q = 0.785398163397448310f;
    if (a > -b) {
        if (a > b) { r = a; phi = Q * (b / a); }
        else { r = b; phi = Q * (2.f - a / b); }
    } else {
        if (a < b) { r = -a; phi = Q * (4.f + b / a); }
        else { r = -b; phi = b != 0.f ? Q * (6.f - a / b) : 0.f; }
    }
    GB_SINCOS(phi, &s, &c);
    ds[0] = r * c;
    ds[1] = r * s;
}

/* Place stratum (i, j) of an n x n hemisphere: initial jitter ss0/ss1 (the
 * stratum's own draw), then collision avoidance against the disk positions
 * of already placed neighbours (prev_row: row i+1, cur_row: row i; entries
 * with x > 1 are empty).  Writes the final disk position to spt. */
GB_HD void gb_place_sample(gb_lot *L, int n, int i, int j, float ss0, float ss1, const float (*prev_row)[2],
                           const float (*cur_row)[2], float spt[2])
{
    float ss[2] = {ss0, ss1};
    int trade_ok = n >= 4 ? 21 : 0;
    gb_square2disk(spt, ((float)j + ss[1]) / (float)n, ((float)i + ss[0]) / (float)n);
    while (trade_ok--) {
        int jj, hit = 0;
        const float lim = 3.14159265358979323846f * GB_MINSDIST * GB_MINSDIST;
        for (jj = j - 1; jj <= j + 1 && !hit; jj++) {
            float dx, dy;
            if (jj < 0 || jj >= n)
                continue;
            if (prev_row && prev_row[jj][0] <= 1.5f) {
                dx = prev_row[jj][0] - spt[0];
                dy = prev_row[jj][1] - spt[1];
                if ((dx * dx + dy * dy) * (float)(n * n) < lim)
                    hit = 1;
            }
            if (!hit && jj == j + 1 && cur_row[jj][0] <= 1.5f) {
                dx = cur_row[jj][0] - spt[0];
                dy = cur_row[jj][1] - spt[1];
                if ((dx * dx + dy * dy) * (float)(n * n) < lim)
                    hit = 1;
            }
        }
        if (!hit)
            break;
        if (trade_ok)
            gb_trade_patchsamp(L, ss);
        else {
            ss[0] = GB_MINSDIST + (1.f - 2.f * GB_MINSDIST) * gb_u01(gb_lot_u32(L));
            ss[1] = GB_MINSDIST + (1.f - 2.f * GB_MINSDIST) * gb_u01(gb_lot_u32(L));
        }
        gb_square2disk(spt, ((float)j + ss[1]) / (float)n, ((float)i + ss[0]) / (float)n);
    }
}

/* ------------------------------------------------------------------------
 * Bin programs: a small stack byte code evaluated per contributing ray.
 * Each instruction is one float4-sized record {op, a, b, c}; the operands
 * of RBIN are stored in the following records.
 */
enum gb_binop {
    GB_OP_END = 0,
    GB_OP_CONST,     /* push a */
    GB_OP_DX, GB_OP_DY, GB_OP_DZ,    /* push ray direction component */
    GB_OP_ADD, GB_OP_SUB, GB_OP_MUL, GB_OP_DIV, GB_OP_NEG,
    GB_OP_IF,        /* pop c, b, a: push (a > 0 ? b : c) (calcomp if()) */
    GB_OP_FLOOR,
    GB_OP_RBIN,      /* Reinhart bin; params in the next 2 records:
                        {MF, RHS, rNx, rNy} {rNz, Ux, Uy, Uz} */
    GB_OP_POW,       /* pop b, a: push a^b */
    GB_OP_FN1,       /* apply one-argument function a (GB_FN_*) to the top */
    GB_OP_ATAN2,     /* pop x, y: push atan2(y, x) */
    GB_OP_MAXN,      /* pop a values, push their maximum */
    GB_OP_MINN,      /* pop a values, push their minimum */
    GB_OP_SELECT,    /* pop a values and an index i: push value i (1-based); i 0: a */
    GB_OP_STORE,     /* pop into temporary a */
    GB_OP_LOAD,      /* push temporary a */
    GB_OP_KBIN,      /* Klems bin; params in the next 2 records:
                        {basis 1/2/4, RHS, Nx, Ny} {Nz, Ux, Uy, Uz} */
    GB_OP_SCBIN,     /* Shirley-Chiu bin; params in the next 2 records:
                        {SCdim, RHS, rNx, rNy} {rNz, Ux, Uy, Uz} */
    GB_OP_CBIN,      /* CIE sky scanner bin; params in the next 2 records:
                        {0, RHS, rNx, rNy} {rNz, Ux, Uy, Uz} */
    GB_OP_MAX
};
enum gb_binfn { GB_FN_SQRT, GB_FN_SIN, GB_FN_COS, GB_FN_TAN, GB_FN_ASIN, GB_FN_ACOS, GB_FN_ATAN, GB_FN_EXP,
                GB_FN_LOG, GB_FN_LOG10, GB_FN_CEIL };
#define GB_BINPROG_MAX 1024   /* instructions of one bin program */
#define GB_BINSTACK 32        /* evaluation stack */
#define GB_BINTEMPS 32        /* temporaries (arguments used more than once) */

typedef struct { float op, a, b, c; } gb_binins;

#endif
