/*
 * gbrad.h -- C ABI of the GB300 ray-tracing library (libgbrad.so).
 *
 * Plain pointers and sizes only.  Every function returns 0 on success or a
 * negative GB_E* code; gb_last_error() gives the message of the last failure
 * on the calling thread.  The caller owns every host buffer; a gb_scene owns
 * its device copy of the scene and its work buffers until gb_scene_free().
 * Calls on one scene are serialised by the caller (one CUDA stream each).
 *
 * The entry points stand in for the programs pyradiance runs as
 * subprocesses (src/pyradiance/rt.py:278-362 rtrace, rt.py:165-235
 * Rcontrib, src/pyradiance/util.py:140-192 dctimestep); see each entry.
 */
#ifndef GBRAD_H
#define GBRAD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_OK            0
#define GB_EINVAL       -1   /* bad argument or option */
#define GB_EIO          -2   /* cannot read a file, malformed octree or scene */
#define GB_EUNSUPPORTED -3   /* valid input the GPU path does not implement */
#define GB_ECUDA        -4   /* CUDA runtime failure */
#define GB_ENOMEM       -5   /* device or host allocation failed */
#define GB_EOVERFLOW    -6   /* a work queue or a limit overflowed */

#define GB_PROG_RTRACE   0
#define GB_PROG_RCONTRIB 1

/* Options shared by rtrace and rcontrib.  Field meanings and defaults follow
 * the reference: rt/raycalls.c:121-150 (rtrace defaults), rt/rcontrib.c:24-58
 * and rt/rcmain.c:164-172 (rcontrib defaults and overrides), option letters
 * as parsed by rt/renderopts.c:123-340, rt/rtmain.c:144-330 and
 * rt/rcmain.c:207-320. */
typedef struct {
    int    prog;            /* GB_PROG_* the defaults came from */
    int    ab, ad, as, ar, aw;
    double aa;
    double av[3];
    int    lr;              /* maxdepth */
    double lw;              /* minweight */
    double dj, ds, dt, dc;  /* dstrsrc, srcsizerat, shadthresh, shadcert */
    int    dr, dp, dv;
    double st, ss;          /* specthresh, specjitter */
    int    bv;              /* back face visibility */
    int    I;               /* -I: irradiance at the sensor point */
    int    i;               /* -i: irradiance at the hit surface */
    int    u;               /* -u: uncorrelated (time-seeded) sampling */
    int    h;               /* header output */
    int    n;               /* processes requested (informational) */
    int    c;               /* rcontrib -c: rays accumulated per record */
    int    V;               /* rcontrib -V: contributions, not coefficients */
    char   fin, fout;       /* -f{a,f,d}{a,f,d,c} */
    char   outspec[32];     /* rtrace -o spec */
    int    x, y;            /* flush interval / resolution */
    double ld;              /* unused: -ld (limit distance) flag */
    uint64_t seed;          /* random stream key; set from -u */
    uint32_t replica;       /* independent replica index of the stream */
} gb_opts;

/* One rcontrib modifier (rt/rcontrib.c:92-159 addmodifier, argument order of
 * rt.py:190-228: -f calfile -e expr -bn nbins -b binv -p params -m mod). */
typedef struct {
    const char *modifier;   /* modifier name to track */
    const char *binv;       /* bin expression, NULL = "0" */
    const char *nbins;      /* bin count expression (-bn), NULL = from a constant binv */
    const char *params;     /* -p settings "MF=1,rNz=-1,..." or NULL */
    const char *calfile;    /* -f file (reinhartb.cal is built in) or NULL */
    const char *expr;       /* -e definitions or NULL */
} gb_modspec;

typedef struct gb_scene gb_scene;

/* Load a Radiance octree, frozen or not (common/readoct.c:29, the readoct()
 * call of rt/rtmain.c and rt/rcmain.c:352). */
int  gb_scene_load(const char *oct_path, gb_scene **out);
/* Build the octree from scene text files as oconv does (ot/oconv.c:42-180),
 * then load it.  objlim <= 0 and resolu <= 0 select oconv's 6 and 16384.
 * An octree among the paths contributes its objects (oconv -i, as rfluxmtx
 * runs it: util/rfluxmtx.c:139-178). */
int  gb_scene_load_rad(const char *const *paths, int npaths, int objlim, int resolu, gb_scene **out);
void gb_scene_free(gb_scene *scene);
/* The octree of a loaded scene: node and set counts, an FNV-1a digest of
 * its pre-order structure with each leaf's sorted object set (equal
 * digests, equal trees), and whether gb_scene_load_rad built it on the GPU
 * (scenes of polygons and spheres on a machine with a GPU; the host builder
 * otherwise, or with GB_OCTREE_BUILDER=host).  No counterpart in the
 * reference (oconv writes the tree to a file, ot/writeoct.c). */
int  gb_scene_octree_info(const gb_scene *scene, int64_t *nodes, int64_t *sets, uint64_t *digest,
                          int *built_on_device);
/* Number of objects; name, modifier name and material name of an object
 * (the -os/-om/-oM outputs of rt/rtrace.c:824-860). */
int64_t     gb_scene_nobjects(const gb_scene *scene);
const char *gb_scene_object_name(const gb_scene *scene, int64_t obj);
const char *gb_scene_modifier_name(const gb_scene *scene, int64_t obj);
const char *gb_scene_material_name(const gb_scene *scene, int64_t obj);

/* Parse options; consumed arguments are counted in *nused, the first
 * non-option (the octree) stops parsing.  prog selects the defaults. */
int  gb_opts_default(int prog, gb_opts *out);
int  gb_opts_parse(int argc, const char *const *argv, int prog, gb_opts *out, int *nused);

/* rtrace over n rays (org_dir: n x 6 doubles, ox oy oz dx dy dz): the -ov
 * value (n x 3 doubles) and the first-hit object of each ray cast forward
 * (hit_id, -1 for none; hit_t distance).  Any output pointer may be NULL.
 * Replaces rt/rtrace.c:146-236 (rtrace) and :436-468 (rtcompute). */
int  gb_rtrace(gb_scene *scene, const gb_opts *opts, const double *org_dir, int64_t n,
               double *out_rgb, int32_t *hit_id, double *hit_t);

/* First hits with their surface normals, for rtrace's -oN and -on: for
 * each ray the object hit (-1 none), its distance (1e10 none), the
 * surface's normal at the hit as the object defines it (hit_normal, n x 3:
 * -oN, rt/rtrace.c:787-804) and, if hit_pnormal is not null, the shading
 * normal (-on, :807-820: turned toward the ray where the material turns a
 * surface hit from behind; a mesh triangle's interpolated vertex normal,
 * rt/o_mesh.c:198-206) and, if hit_uv is not null, the local (u,v)
 * coordinates (n x 2: -oc, :766-772: a mesh triangle's vertex (u,v)
 * interpolated at the hit, else 0); zero where nothing is hit or a source
 * at infinity is.  The casts are those of gb_rtrace's hit ids (FP64).
 * Replaces: the -on/-oN/-oc columns of rt/rtrace.c:274-345. */
int  gb_rtrace_hits(gb_scene *scene, const gb_opts *opts, const double *org_dir, int64_t n, int32_t *hit_id,
                    double *hit_t, double *hit_normal, double *hit_pnormal, double *hit_uv);

/* The values of gb_rtrace for rays already in device memory (d_org_dir:
 * n x 6 doubles; d_rgb: n x 3 doubles, overwritten), allocating no device
 * memory.  For callers that cannot allocate while they run: a service that
 * reserved the GPU's memory for its own pool at start-up, or a loop beside
 * latency-bound streams that cudaMalloc/cudaFree would stall by
 * synchronising the device.  Working memory comes from one static 64 MiB
 * device array per device; a call whose rays would not fit (1.25 KiB per
 * ray without ambient bounces, about 650 bytes per first-hemisphere sample with
 * -I and -ab > 0) is rejected with GB_EINVAL and a message giving the
 * need.  All work is enqueued on `stream` (a cudaStream_t; NULL is the
 * legacy default stream), after whatever the caller enqueued there before,
 * so the rays may still be being written on that stream when the call is
 * made; work on other streams must be complete.  The call returns when the
 * output is complete; on an error return d_rgb is undefined, and no work of
 * the call is left running.  The scene must have been loaded on the
 * current device.  The first call on a device looks the array up there
 * (and may load this library's device code) and keeps that address for the
 * life of the process (a cudaDeviceReset() makes it stale); make that first
 * call before capturing work on any stream.  Calls on the same device
 * share the array: calls that overlap in time, from several threads,
 * streams or scenes, race and corrupt each other's results; serialise
 * them.  No counterpart in the reference (its rtrace reads rays from a
 * pipe, rt/rtrace.c:146-236). */
int  gb_rtrace_device_noalloc(gb_scene *scene, const gb_opts *opts, const double *d_org_dir, int64_t n,
                              double *d_rgb, void *stream);

/* Material parameters.  Every material the scene's surfaces use has a
 * slot; gb_scene_material_rgb reads (get_rgb) and/or replaces (set_rgb) its
 * colour: the reflectance of plastic and metal, the transmissivity of
 * glass, the radiance of light and glow.  A new colour takes effect in the
 * next call on the scene.  No counterpart in the reference (its materials
 * are fixed when the octree is read). */
int64_t gb_scene_material_slots(const gb_scene *scene);
int  gb_scene_material_slot(const gb_scene *scene, const char *name, int *slot);
int  gb_scene_material_rgb(gb_scene *scene, int slot, double *get_rgb, const double *set_rgb);

/* Gradient of sum_i dl_dvalue[i] . value[i] -- value being gb_rtrace's -ov
 * output for the same rays and options (with -I, the sensor irradiance) --
 * with respect to the colour of every material slot (grad: nslots x 3,
 * nslots = gb_scene_material_slots): plastic and metal reflectance through
 * their diffuse terms, glass transmissivity through rt/glass.c's
 * transmission and reflection coefficients.  The paths are replayed from the
 * same random streams as the forward call (options, seed and replica must be
 * the same), sampling decisions held fixed.  No counterpart in the
 * reference. */
int  gb_rtrace_grad(gb_scene *scene, const gb_opts *opts, const double *org_dir, int64_t n,
                    const double *dl_dvalue, double *grad, int64_t nslots);

/* rcontrib: out has (n / opts->c) records x (sum of nbins) x 3 doubles,
 * modifiers in the given order (rt/rcontrib.c:379-427, rt/rc2.c:294-357).
 * ray_count (optional) receives the number of rays traced. */
int  gb_rcontrib(gb_scene *scene, const gb_opts *opts, const gb_modspec *mods, int nmods,
                 const double *org_dir, int64_t n, double *out, int64_t *ray_count);
/* Many rcontrib grids at once: job j traces n[j] rays (org_dir[j]) in
 * scenes[j] into out[j] (n[j] / opts->c records, as gb_rcontrib), all with
 * the same options and modifiers.  The jobs of one scene run as a single
 * wavefront over their concatenated sensors, with the queue capacity taken
 * from a pilot run over a sample of them (remembered per scene and option
 * set); different scenes run concurrently on their own streams.  n[j] must
 * be a multiple of opts->c.  ray_count (optional) receives the rays traced
 * by all jobs.  A sensor draws the random streams of its position in its
 * scene's concatenated sensors: a job alone on its scene reproduces its
 * separate gb_rcontrib call up to rounding (the order in which a warp's
 * lanes are summed and bins accumulated), jobs sharing a scene are
 * statistically equivalent to separate calls.  No
 * counterpart in the reference (one rcontrib process per grid). */
int  gb_rcontrib_batch(int njobs, gb_scene *const *scenes, const gb_opts *opts, const gb_modspec *mods, int nmods,
                       const double *const *org_dir, const int64_t *n, double *const *out, int64_t *ray_count);
/* Total bins of a modifier list (validates the bin expressions). */
int  gb_rcontrib_nbins(const gb_modspec *mods, int nmods, int *nbins_total);

/* dctimestep's two-matrix product R[m,n,c] = sum_k DC[m,k,c] * S[k,n,c]
 * (util/dctimestep.c:324-393, util/cmatrix.c:421-474); all matrices are
 * interleaved RGB float32 (row-major, 3 floats per element).  mode selects
 * the arithmetic:
 *   GB_DCT_FP32    FP32 FMA on the CUDA cores
 *   GB_DCT_BF16X3  bf16 hi/lo split, 3 tensor-core products, FP32 accumulate
 *                  (up to about 2e-5 relative error where one product
 *                  dominates an output)
 *   GB_DCT_FP64    FP64 FMA on the CUDA cores
 *   GB_DCT_FP16X3  rows of DC and columns of S scaled by powers of two into
 *                  the FP16 range, fp16 hi/lo split, 3 tensor-core products,
 *                  FP32 accumulate (within 1e-5 relative of FP64)
 *   GB_DCT_FP16    the same scaled fp16 operands, one product (about 1e-3)
 * The tensor-core forms skip all-zero columns of S as cm_multiply does
 * (their outputs are zero); all-zero rows of DC are multiplied (their
 * outputs are the same zeros).  The environment variable GB_DCT_WAIT_NS
 * (nanoseconds, read at each call) shortens the limit of the tensor-core
 * pipeline's waits, normally 2 s, after which a call returns GB_ECUDA: for
 * tests of that error path.  GB_DCT_CLUSTER=1 (read at each call) runs one
 * CTA per row tile instead of clusters of two that share the column tile's
 * copies: the same results, for tests and measurement. */
#define GB_DCT_FP32   0
#define GB_DCT_BF16X3 1
#define GB_DCT_FP64   2
#define GB_DCT_FP16X3 3
#define GB_DCT_FP16   4
int  gb_dctimestep(const float *dc, const float *sky, int64_t M, int64_t K, int64_t N, int mode,
                   float *out);
/* Same on device pointers already resident in HBM (no copies). */
int  gb_dctimestep_device(const float *d_dc, const float *d_sky, int64_t M, int64_t K, int64_t N,
                          int mode, float *d_out, void *stream);

/* Counters of the last call on this thread: rays traced, cube steps,
 * contributions binned, kernel launches. */
int  gb_last_stats(int64_t *rays, int64_t *steps, int64_t *contribs, int64_t *launches);
/* Per-kernel profile of the last rtrace/rcontrib call on this thread:
 * kernel 0 cast, 1 sensor roots, 2 first-hemisphere rays, 3 primaries,
 * 4 octree walks, 5 shading (one launch of 4 and 5 per generation); device
 * milliseconds (CUDA events on the library's stream), launches, counters
 * (rays, cube steps, contributions, queue overflows, bad bins, node
 * descents, object tests, spare) and the milliseconds of the whole kernel
 * region.  No counterpart in the reference (its -t progress report counts
 * rays only). */
int  gb_last_profile(int kernel, double *ms, int64_t *launches, int64_t *counters, int ncounters,
                     double *region_ms);

/* Measurement aid: the rate (GB/s into *gbps) at which this GPU reads
 * random 64-byte records from a table of table_bytes (L2-resident when it
 * is below the L2 size), with the walk kernel's launch shape: independent
 * reads (chase = 0), or each read's place taken from the last record read
 * (chase = 1: a chain of dependent loads, as in the octree walk).  The
 * ceilings the walk's algorithmic bytes are held against.  No counterpart
 * in the reference. */
int  gb_probe_l2(int64_t table_bytes, int chase, double *gbps);

/* ASCII output rows: each row of the nrows x ncols values in C's %e form
 * (six digits after the point, as rt/rtrace.c puta and rt/rc2.c print
 * them), separated by sep, the row ended by end, written to out (cap
 * bytes); *len receives the text's length (GB_EOVERFLOW when above cap,
 * nothing written).  Formatted by several host threads, equal to a
 * sequential loop's text.  No counterpart in the reference (its programs
 * print with printf). */
int  gb_format_rows(const double *vals, int64_t nrows, int64_t ncols, const char *sep, const char *end, char *out,
                    int64_t cap, int64_t *len);

const char *gb_last_error(void);
const char *gb_version(void);

#ifdef __cplusplus
}
#endif
#endif
