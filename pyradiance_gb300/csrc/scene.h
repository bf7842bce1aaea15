/*
 * scene.h -- host-side Radiance scene ingestion shared by the GPU library and
 * the CPU oracle: octree (.oct) reading, scene text (.rad) parsing, the
 * octree builder, and the per-primitive precomputation the intersectors use.
 *
 * The in-memory layout follows what the octree file carries: one flat array
 * of objects (surfaces and modifiers, in definition order, so object indices
 * are exactly the reference's OBJECT numbers) and an octree whose nodes are
 * int32 codes: >= 0 a node index (8 children), -1 empty, <= -2 a leaf object
 * set index (code = -set - 2), as in common/octree.h:11-31.
 */
#ifndef GB_SCENE_H
#define GB_SCENE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_FTINY 1e-6
#define GB_FHUGE 1e10
#define GB_MAXSET 8191          /* common/object.h:82 */

/* object kinds (names as in the reference's common/otypes.c) */
enum gb_otype {
    GT_UNKNOWN = 0,
    /* surfaces */
    GT_POLYGON, GT_SPHERE, GT_BUBBLE, GT_CONE, GT_CUP, GT_CYLINDER, GT_TUBE,
    GT_RING, GT_SOURCE, GT_INSTANCE, GT_MESH,
    /* materials */
    GT_PLASTIC, GT_METAL, GT_TRANS, GT_GLASS, GT_LIGHT, GT_ILLUM, GT_GLOW,
    GT_SPOT, GT_MIRROR, GT_DIELECTRIC, GT_INTERFACE, GT_ANTIMATTER,
    GT_OTHER_MATERIAL,
    /* modifiers that are neither surfaces nor materials */
    GT_ALIAS, GT_PATTERN, GT_TEXTURE, GT_MIXTURE,
    GT_NTYPES
};

int gb_otype_from_name(const char *name);
const char *gb_otype_name(int t);
int gb_is_surface(int t);
int gb_is_material(int t);
int gb_is_light(int t);          /* light, illum, glow, spotlight */
int gb_is_transp(int t);         /* rt/otspecial.h:14 (trans, glass, dielectric, interface) */
int gb_is_volume(int t);         /* instance, mesh (octree volumes) */

typedef struct {
    int      otype;              /* enum gb_otype */
    int32_t  omod;               /* modifier index, -1 = void */
    char    *name;
    int      nsargs;
    char   **sarg;
    int      nfargs;
    double  *farg;
    double  *vnorm;              /* mesh triangles with vertex normals: the three
                                    unit normals in the mesh's coordinates, in the
                                    order of the vertices in farg; else NULL */
    double  *vuv;                /* mesh triangles with (u,v) at every vertex: the
                                    three (u,v) pairs, vertex order; else NULL */
} gb_object;

/* face record: common/face.h + common/face.c:35-112 */
typedef struct {
    double norm[3];
    double offset;
    double area;
    int    nv;                   /* vertex count (after dropping last==first) */
    int    ax;                   /* dominant normal axis */
    int    ok;                   /* 0 for zero-area faces */
} gb_face;

/* cone record: common/cone.h + common/cone.c:44 */
typedef struct {
    double al, sl;               /* alpha and slope terms */
    double tm[4][4];             /* world -> canonical transform */
    int    p0, p1;               /* index of centres in farg (0 and 3) */
    int    r0, r1;               /* index of radii in farg (6 and 7), -1 if none */
    int    ok;
} gb_cone;

/* common/xf.c XF: a 4x4 row-vector transform and its scale */
typedef struct {
    double xfm[4][4];
    double sca;
} gb_xf;

/* an octree referenced by instances, merged into the scene's arrays
 * (common/instance.c:23-60 getscene) */
typedef struct {
    char    *name;               /* the file name as the instance gives it */
    double   cuorg[3], cusize;   /* its own cube */
    int32_t  root;               /* its root code in the merged tree */
    int32_t  firstobj, nobjs;    /* its objects in the merged object array */
} gb_subscene;

/* an instance object (common/instance.c:65-104 getinstance) */
typedef struct {
    int32_t  obj;                /* the instance object */
    int32_t  sub;                /* its octree in subs[] */
    gb_xf    f, b;               /* forward and backward transforms (common/xf.c fullxf) */
} gb_instance;

typedef struct {
    /* bounding cube */
    double   cuorg[3];
    double   cusize;
    /* objects */
    int32_t  nobjs;
    int32_t  cap_objs;
    gb_object *objs;
    /* octree */
    int32_t  root;               /* node code */
    int32_t  nnodes;
    int32_t  cap_nodes;
    int32_t *kids;               /* 8 * nnodes codes */
    int32_t  nsets;
    int32_t  cap_sets;
    int64_t *set_off;            /* offset of each set in set_data */
    int64_t  set_len;
    int64_t  cap_set_data;
    int32_t *set_data;           /* [count, members...] per set, sorted ascending */
    /* derived, filled by gb_scene_prepare */
    gb_face  *faces;             /* per object (only polygons filled) */
    gb_cone  *cones;             /* per object (cones, cups, cylinders, tubes, rings) */
    int       prepared;
    /* files named by an unfrozen octree */
    int       nfiles;
    char    **files;
    /* instances: objects [0, nobjs_top) are the scene's own; the objects of
     * the octrees its instances reference follow, loaded once per file */
    int32_t   nobjs_top;
    int32_t   ninst, nsubs;
    gb_instance *inst;
    gb_subscene *subs;
} gb_scene_host;

/* error text of the last failing call on this thread */
const char *gb_scene_error(void);

void gb_scene_init(gb_scene_host *S);
void gb_scene_clear(gb_scene_host *S);

/* Read a Radiance octree (common/readoct.c:29): header, bounds, scene files
 * (parsed as scene text, resolved against the working directory and then the
 * octree's own directory), object count, the pre-order tree and, for frozen
 * octrees, the binary objects (common/sceneio.c:90).  Returns 0 or -1. */
int gb_scene_read_oct(gb_scene_host *S, const char *path);

/* Append the objects of a Radiance scene text file / buffer. */
int gb_scene_read_rad_file(gb_scene_host *S, const char *path);
int gb_scene_read_rad_text(gb_scene_host *S, const char *text, const char *what);

/* Load the octrees of the scene's instance objects (common/instance.c:
 * 65-104 getinstance: file name, then transform arguments, common/xf.c) and
 * merge their objects, nodes and sets into the scene's arrays.  A relative
 * file name is looked up in the working directory, then in base_dir.
 * Instances inside instanced octrees are refused.  Returns 0 or -1. */
int gb_scene_load_instances(gb_scene_host *S, const char *base_dir);

/* common/xf.c fullxf: forward and inverse transform of ac arguments;
 * returns the number of arguments used. */
int gb_fullxf(gb_xf *f, gb_xf *b, int ac, char *const *av);

/* Build the octree over the loaded objects with the reference's oconv
 * algorithm (ot/oconv.c:216-330): bounding cube from the surfaces' extent,
 * objects added in definition order, full nodes split above objlim objects
 * until the cube is smaller than cusize/resolu. */
int gb_scene_build_octree(gb_scene_host *S, int objlim, int resolu);
/* the first step of gb_scene_build_octree: objects prepared and the scene
 * cube set from their bounding box */
int gb_scene_octree_cube(gb_scene_host *S);
/* the same octree built on the current CUDA device (octbuild_gpu.cu):
 * 0 built, 1 the scene holds objects only the host builder handles, < 0
 * failure (reason in err) */
int gb_scene_build_octree_device(gb_scene_host *S, int objlim, int resolu, char *err, size_t errlen);
/* the builder's storage of nodes and leaf sets (scene.c) */
int32_t gb__add_set(gb_scene_host *S, const int32_t *set);
int32_t gb__new_node(gb_scene_host *S);

/* Precompute faces and cones; checks argument counts. */
int gb_scene_prepare(gb_scene_host *S);

/* Follow the modifier chain to the material (rt/initotypes.c findmaterial);
 * returns the object index or -1. */
int32_t gb_find_material(const gb_scene_host *S, int32_t obj);

/* Object set of a leaf code; returns pointer to [count, members...]. */
const int32_t *gb_scene_set(const gb_scene_host *S, int32_t code);

/* Radiance portable float (common/portio.c:136) of a 4+1 byte code. */
double gb_portable_flt(long mant, int expo);

#ifdef __cplusplus
}
#endif
#endif
