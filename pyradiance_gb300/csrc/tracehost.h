/*
 * tracehost.h -- the launch record shared by trace.cu (device) and host.cu.
 */
#ifndef GB_TRACEHOST_H
#define GB_TRACEHOST_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "devscene.h"
#include "gbcommon.h"

/* stats slots */
#define GB_ST_RAYS     0   /* rays traced (octree walks) */
#define GB_ST_STEPS    1   /* cube visits */
#define GB_ST_CONTRIB  2   /* contributions binned */
#define GB_ST_OVERFLOW 3   /* queue records dropped */
#define GB_ST_BADBIN   4   /* bin numbers beyond nbins */
#define GB_ST_NODES    5   /* octree node descents */
#define GB_ST_TESTS    6   /* ray-object intersection tests */
#define GB_ST_N        8
/* kernels with their own block of GB_ST_N counters */
#define GB_K_CAST      0   /* first hit only */
#define GB_K_ROOT      1   /* -I sensor roots */
#define GB_K_EXPAND    2   /* first hemisphere of the -I sensors into the queue */
#define GB_K_PRIMARY   3   /* primaries into the queue */
#define GB_K_TRACE     4   /* octree walk of one generation */
#define GB_K_SHADE     5   /* shading of one generation, children queued */
#define GB_K_N         6

#define GRID_BITS_HOST 24      /* must equal GRID_BITS of trace.cuh */

/* one queued ray: 64 bytes, four float4 lanes */
typedef struct __align__(16) {
    float v[16];
} gb_qray;

/* the walk result of a queued ray: 32 bytes (object, distance, -dir.n,
 * normal) */
typedef struct __align__(16) {
    float v[8];
} gb_qhit;

/* the parameter-dependent factors along a queued ray's path (gradient
 * runs): up to GB_ADJ_MAX entries (material slot << 2 | kind) and the
 * cosine at each glass vertex */
#define GB_ADJ_MAX 6
#define GB_ADJ_REFL   0    /* diffuse reflectance of a plastic or metal */
#define GB_ADJ_GLASST 1    /* transmission through glass */
#define GB_ADJ_GLASSR 2    /* reflection off glass */
typedef struct __align__(16) {
    uint32_t n;
    uint32_t e[GB_ADJ_MAX];
    float pd[GB_ADJ_MAX];
    uint32_t pad[3];
} gb_qadj;

/* first hemisphere of a -I sensor */
typedef struct {
    float hp[3], nrm[3], ux[3];
    int n;
} gb_rootrec;

typedef struct {
    gb_dscene S;
    /* options */
    int   ab, ad;
    float minweight;
    int   maxdepth;
    float av[3];
    float dstrsrc;
    float srcsizerat;          /* -ds: split flat local sources larger than this times their distance */
    float specthresh;
    float specjitter;          /* -ss */
    int   follow;              /* rcontrib: every source is followed (SFOLLOW) */
    int   do_irrad;            /* -i: primary hits shaded as a Lambertian irradiance meter */
    int   contrib_mode;        /* rcontrib -V */
    uint32_t k0, k1;           /* random stream key */
    uint32_t replica;
    /* sensors: this run's slice of a larger sensor set starts at index
     * sensor_base of it; random streams are keyed by the index in the set,
     * outputs by the index in the slice */
    long long nsensors;
    uint32_t sensor_base;
    const double *sensors;     /* n x 6 */
    /* outputs */
    double *value;             /* n x 3 or NULL */
    double *bins;              /* records x nbins_total x 3 or NULL */
    int   accum;
    int   nbins_total;
    const gb_binins *binprog;
    const int4 *modinfo;       /* per tracked slot: program offset, nbins, bin0 */
    unsigned long long *stats;
    /* work */
    gb_rootrec *roots;
    float2 *root_spt;          /* n x root_n^2 placed disk positions (root_n >= 4) */
    float2 *root_draw;         /* n x root_n^2 stratum jitters, x > 1.5 for a stratum
                                * that died in Russian roulette (root_n >= 4) */
    float *root_lot;           /* n x 2 * GB_XLOT: the first fill of each sensor's lot */
    int   root_n;
    const gb_qray *qin;
    const unsigned long long *qin_count;
    gb_qray *qout;
    unsigned long long *qout_count;
    gb_qhit *hits;             /* walk results of qin, same indices */
    /* gradient runs: d(loss)/d(value) per sensor, the gradient per material
     * slot (RGB), and the factor lists beside the two queues */
    const double *dlde;
    double *grad;
    int nslots;
    int grad_shared;           /* set per launch: accumulators in shared memory */
    const gb_qadj *adj_in;
    gb_qadj *adj_out;
    long long qcap;
    unsigned long long *work;  /* work-item counter of the persistent kernels (zeroed per launch) */
    /* walk kernel shape, picked per scene by the host's tuner (0: defaults):
     * idle lanes a warp waits for before it refills them from the queue,
     * and resident blocks per SM */
    int   walk_refill;
    int   walk_blocks_per_sm;
    /* ambient super-sampling of the -I first hemispheres (rtrace -as):
     * paths carry the index (sensor * root_n^2 + stratum) of the stratum
     * they descend from in queue-parallel tag arrays, their values add to
     * ss_val there; ss_cnt counts each stratum's extra samples */
    /* scenes with instances: the queue indices whose walks met one, for
     * k_trace_inst (zeroed count per generation) */
    unsigned int *slow;
    unsigned long long *slow_count;
    int   ss_samples;          /* -as */
    const uint32_t *tag_in;
    uint32_t *tag_out;
    double *ss_val;            /* n x root_n^2 x 3, or NULL: no super-sampling */
    int   *ss_cnt;             /* n x root_n^2 */
    float *ss_err;             /* n x 2 root_n^2 scratch of the error map */
} gb_run;

int gb_launch_cast(const gb_run *P, int *hit_obj, float *hit_t, float *hit_pn, cudaStream_t st, int sms);
/* the same first hits in FP64 (cast64.cu) */
int gb_launch_cast64(const gb_run *P, int *hit_obj, float *hit_t, double *hit_pn, cudaStream_t st, int sms);
int gb_launch_root(const gb_run *P, cudaStream_t st, int sms);
/* -I roots with root_n >= 4: the strata's draws and the lots in parallel,
 * then the sequential placement per sensor */
int gb_launch_root_draws(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_root_place(const gb_run *P, cudaStream_t st, int sms);
/* -as super-sampling of the -I first hemispheres: the extra samples after
 * the first pass, and the strata's means into the sensors after the second */
int gb_launch_ssamp_plan(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_ssamp_final(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_expand_root(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_primary(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_trace(const gb_run *P, cudaStream_t st, int sms);
/* the L2 read ceilings of the walk (k_probe_l2) */
int gb_launch_probe_l2(const float4 *table, uint32_t nrec, int iters, int chase, float *sink, cudaStream_t st,
                       int sms);
int gb_launch_shade(const gb_run *P, cudaStream_t st, int sms);
/* gradient runs: the same kernels, shading with the factor lists */
int gb_launch_root_grad(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_expand_root_grad(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_primary_grad(const gb_run *P, cudaStream_t st, int sms);
int gb_launch_shade_grad(const gb_run *P, cudaStream_t st, int sms);

#endif
