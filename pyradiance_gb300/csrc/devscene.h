/*
 * devscene.h -- the scene as the kernels see it, in HBM.
 *
 * Layout (structure of arrays, all read-only during a run):
 *   kids      int32[8 * nnodes]   octree children codes (>= 0 node, -1 empty,
 *                                 <= -2 full leaf: gb_leaf_code of its set's
 *                                 offset in set_data and size), 32 B per node
 *   set_data  int32[...]          [count, members in DESCENDING object order]
 *                                 (the order rt/raytrace.c:585 tests them),
 *                                 each member given by its record slot
 *   obj       int4[nobjs]         x: kind | flags << 8 | nv << 16,
 *                                 y: material slot (-1 none), z: modifier
 *                                 object index, w: vertex / cone offset
 *   geo       float4[nobjs]       faces: unit normal + plane offset;
 *                                 spheres: centre + radius
 *   fvert     float2[...]         polygon vertices projected on the two
 *                                 axes other than the dominant normal axis
 *   fv4       float4[2 * nobjs]   the same for faces of at most four
 *                                 vertices, packed at a fixed place per
 *                                 object (v0 v1 | v2 v3), so that a face
 *                                 test needs no second indirection
 *   orec      float4[4 * nobjs]   obj (its y: the object's index), geo and
 *                                 fv4 of each object in one 64-byte record,
 *                                 in the order the leaves first reach them
 *   oslot     int32[nobjs]        each object's record slot
 *   vnidx     int32[nobjs]        mesh triangles with vertex normals: the
 *                                 index of their normals in vnrm (else -1)
 *   vnrm      float4[3 * ...]     their three unit vertex normals, in the
 *                                 mesh's coordinates, vertex order
 *   wkids     int32[8 * nnodes]   the FP32 walk's copy of kids: full-leaf
 *                                 codes give the leaf's place in lrec
 *   lrec      float4[4 * ...]     per leaf set: a header record (first
 *                                 word: member count), then its members'
 *                                 64-byte orec records in test order (an
 *                                 object in several leaves has a copy in
 *                                 each), so that a leaf's objects are
 *                                 tested without loading its member list
 *   cone      float[24 * ncones]  3x4 world->canonical transform (rings),
 *                                 axis, base point, length, slant, radii
 *   mat       float4[2 * nmats]   material kind and parameters
 *   src       gb_dsrc[nsrc]       light sources (rt/source.h SRCREC subset)
 *   trk       int32[nobjs]        tracked-modifier slot of each object's
 *                                 direct modifier (-1 untracked)
 *   inst      gb_dinst[ninst]     instances: transforms, octree, surface ids
 *   g64       double[...]         per object (at g64off[object]) its FP64
 *                                 geometry for the first-hit casts: faces
 *                                 normal, offset, ok, axis, count, vertices;
 *                                 spheres centre, radius; cones ok, alpha,
 *                                 slant, transform, end points, radii;
 *                                 instances transforms, scales, octree
 */
#ifndef GB_DEVSCENE_H
#define GB_DEVSCENE_H

#include <stdint.h>

/* object kinds on the device */
enum { DK_NONE = 0, DK_FACE, DK_SPHERE, DK_BUBBLE, DK_CONE, DK_CUP, DK_CYL, DK_TUBE, DK_RING, DK_SOURCE,
       DK_INSTANCE };
/* object flags */
#define DF_HASMAT  0x01   /* has a material (findmaterial != NULL) */
#define DF_TRANSP  0x02   /* material is nominally transparent */
#define DF_AXSHIFT 2      /* bits 2-3: dominant normal axis of a face */
#define DF_VNORM   0x10   /* a mesh triangle with vertex normals (vnidx, vnrm) */
#define DF_VUV     0x20   /* a mesh triangle with (u,v) at its vertices (after its FP64 record) */

/* full-leaf code: -2 - (offset << 6 | min(size, 63)); a size field of 63
 * means "63 or more: read the count word" */
#define GB_LEAF_SIZEBITS 6
#define GB_LEAF_MAXOFF (1 << (31 - GB_LEAF_SIZEBITS))
static inline int gb_leaf_code(int off, int size)
{
    return -2 - ((off << GB_LEAF_SIZEBITS) | (size < 63 ? size : 63));
}

/* material kinds on the device */
enum { DM_NONE = 0, DM_PLASTIC, DM_METAL, DM_GLASS, DM_LIGHT, DM_GLOW, DM_TRANS, DM_MIRROR };

/* source flags (rt/source.h:24-37) */
#define DS_DISTANT 0x01
#define DS_SKIP    0x02
#define DS_FLAT    0x04
#define DS_PROX    0x08
#define DS_FOLLOW  0x10
#define DS_CIR     0x20   /* circular (disk, sphere, distant): SCIR */
#define DS_CYL     0x40   /* cylinder: SCYL */
#define DS_SPOT    0x80   /* spotlight: SSPOT */

typedef struct {
    float sloc[3];      /* centre (local) or direction (distant) */
    float snorm[3];     /* flat source normal */
    float ss[3][3];     /* SU, SV, SW size vectors */
    float ss2;          /* area (flat) or solid angle (distant) */
    float srad;         /* radius */
    float prox;         /* glow proximity radius */
    int   flags;
    int   so;           /* source object index */
    int   mat;          /* material slot of the source */
    int   pad;
    float spot[5];      /* spotlight: cone solid angle, unit aim, focus length (rt/srcsupp.c makespot) */
    float pad2[3];
} gb_dsrc;

/* An instance (rt/o_instance.c): the transforms to and from its octree's
 * coordinates (rows of the 4x4 row-vector matrices of common/xf.c; the
 * fourth row is the translation), that octree's cube and root, and its
 * objects.  Surfaces inside instances are identified by surface ids
 * sidbase + (object - firstobj), above every object index, so that the same
 * instanced object in two instances has two ids. */
typedef struct {
    float bx[12], fx[12];      /* backward (world -> instance) and forward */
    float bsca, fsca;
    float cuorg[3], cusize, grid_scale, cell;
    int   root;                /* root code of its octree in the walk's copy (wkids, lrec) */
    int   obj;                 /* the instance object */
    int   hasmod;              /* the instance's modifier replaces its surfaces' own */
    int   sidbase;             /* first surface id */
    int   firstobj, nobjs;     /* its octree's objects */
} gb_dinst;

typedef struct {
    /* octree */
    float cuorg[3];
    float cusize;
    float grid_scale;          /* 2^24 / cusize */
    float cell;                /* cusize / 2^24 */
    int   root;
    int   nnodes;
    const int   *kids;
    const int   *set_data;
    /* the FP32 walk's copy of the octree: leaf codes address lrec, where
     * each leaf set is a header record (first word: its member count)
     * followed by its members' 64-byte records in test order */
    int   wroot;
    const int   *wkids;
    const float4 *lrec;
    /* objects */
    int   nobjs;
    const int4  *obj;
    const float4 *geo;
    const float2 *fvert;
    const float4 *fv4;
    const float4 *orec;        /* per record slot: obj (y: the object's index), geo, fv4; 64 bytes */
    int   has_vnorm;           /* some mesh triangle has vertex normals */
    const int   *vnidx;        /* per object: its vertex normals in vnrm (DF_VNORM objects) */
    const float4 *vnrm;        /* three unit normals (x, y, z, 0) per smooth mesh triangle, mesh coordinates */
    const int   *oslot;        /* per object: its record slot */
    const float *cone;
    /* materials */
    const float4 *mat;
    /* sources */
    int   nsrc;
    const gb_dsrc *src;
    /* tracked modifiers (per object) */
    const int *trk;
    /* instances, in order of sidbase */
    int   ninst;
    const gb_dinst *inst;
    /* FP64 geometry of the first-hit casts (cast64.cu): the scene cube, and
     * per object a record at g64 + g64off[object] */
    double cuorg64[3], cusize64;
    const double *g64;
    const long long *g64off;
} gb_dscene;

#endif
