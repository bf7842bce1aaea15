/*
 * octbuild_gpu.cu -- the octree of a scene of polygons and spheres built on
 * the GPU, level by level, equal to the one the host builder (octbuild.c)
 * and the reference's oconv make.
 *
 * oconv adds objects one at a time (ot/oconv.c:216-330): an object goes
 * into every leaf cube it overlaps, and a leaf that would hold more than
 * objlim objects is split into eight, its objects re-added to the children,
 * unless the children would fall below the minimum cube size (below 1/256
 * of it once the set has MAXSET objects).  Sets only grow, and for surfaces
 * the overlap of an object and a cube does not depend on what else the cube
 * holds, so the final tree depends only on the counts: a cube is split
 * exactly when more than objlim objects overlap it (more than MAXSET below
 * the minimum size) and its children are not too small.  The tree is
 * therefore built top-down, one level per pass over all (cube, object)
 * pairs of the level:
 *
 *   k_root_pairs   the surfaces that overlap the scene cube, in object
 *                  order;
 *   k_split        which cubes of the level split (their pair counts);
 *   k_child_test   for every pair of a splitting cube and each of its eight
 *                  children, whether the object overlaps the child: the
 *                  overlap tests of ot/o_face.c:40-99 (vertex location,
 *                  common/clip.c edge clipping, the plane and point-in-face
 *                  test) and ot/sphere.c:50-109, in FP64 with the host
 *                  builder's operation order and no contracted multiply-
 *                  adds (this file is compiled with -fmad=false), so every
 *                  decision equals the host builder's;
 *   scan           the flags of each splitting cube are laid out child by
 *                  child, so one exclusive scan gives every surviving pair
 *                  its place in the next level, grouped by child cube and
 *                  still in object order (leaf sets come out sorted);
 *   k_scatter, k_children  the next level's pairs and cubes.
 *
 * The host then merges splits whose eight children are equal leaves
 * (common/octree.c:73-90) and stores the tree in pre-order, as the host
 * builder does.  Scenes with cones, rings or other volumes are left to the
 * host builder (gb_scene_build_octree_device returns 1).
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "scene.h"

namespace {

#define OK_FACE 1
#define OK_SPHERE 2

struct DevObjs {
    const int *kind;          /* OK_FACE, OK_SPHERE, 0 */
    const int *nv, *ax, *ok;  /* faces */
    const long long *voff;    /* first vertex (x3 doubles) */
    const double *norm;       /* 3 per object */
    const double *offset;     /* faces: plane offset; spheres: radius */
    const double *vert;       /* face vertices; sphere centres */
};

#define XPOS 03
#define YPOS 014
#define ZPOS 060
#define POSITION(i) (3 << ((i) << 1))
#define BELOW 025
#define ABOVE 052
#define D_FTINY 1e-6

__device__ int plocate_d(const double p[3], const double mn[3], const double mx[3])
{
    int loc = 0;
    const double E = D_FTINY;
    if (p[0] < mn[0] - E) loc |= XPOS & BELOW;
    else if (p[0] > mx[0] + E) loc |= XPOS & ABOVE;
    if (p[1] < mn[1] - E) loc |= YPOS & BELOW;
    else if (p[1] > mx[1] + E) loc |= YPOS & ABOVE;
    if (p[2] < mn[2] - E) loc |= ZPOS & BELOW;
    else if (p[2] > mx[2] + E) loc |= ZPOS & ABOVE;
    return loc;
}

/* common/clip.c:19-72: clip the segment to the box, true if any part of it
 * is inside */
__device__ int clip_seg_d(double *ep1, double *ep2, const double mn[3], const double mx[3])
{
    int itlim = 6, loc1, loc2, accept, i, j;
    double *dp, d;
    loc1 = plocate_d(ep1, mn, mx);
    loc2 = plocate_d(ep2, mn, mx);
    while (!((accept = !(loc1 | loc2)) || (loc1 & loc2))) {
        if (itlim-- <= 0)
            return 0;
        if (!loc1) {
            dp = ep1; ep1 = ep2; ep2 = dp;
            i = loc1; loc1 = loc2; loc2 = i;
        }
        for (i = 0; i < 3; i++) {
            if (loc1 & POSITION(i) & BELOW) {
                d = (mn[i] - ep1[i]) / (ep2[i] - ep1[i]);
                ep1[i] = mn[i];
            } else if (loc1 & POSITION(i) & ABOVE) {
                d = (mx[i] - ep1[i]) / (ep2[i] - ep1[i]);
                ep1[i] = mx[i];
            } else
                continue;
            for (j = 0; j < 3; j++)
                if (j != i)
                    ep1[j] += (ep2[j] - ep1[j]) * d;
            break;
        }
        loc1 = plocate_d(ep1, mn, mx);
    }
    return accept;
}

/* common/face.c:121-161 on the dominant projection */
__device__ int inface_d(const double p[3], int n, int ax, const double *va)
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
#define FEQ(a, b) (fabs((a) - (b)) <= D_FTINY)
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

/* ot/o_face.c:40-99 */
__device__ int face_cube_d(const DevObjs &O, int obj, const double org[3], double size)
{
    double cumin[3], cumax[3], v1[3], v2[3], d1, d2;
    const double *va = O.vert + 3 * O.voff[obj];
    const double *nrm = O.norm + 3 * obj;
    const int nv = O.nv[obj];
    int vloc, i, j;
    if (!O.ok[obj])
        return 0;
    for (j = 0; j < 3; j++) {
        cumin[j] = org[j] - D_FTINY;
        cumax[j] = cumin[j] + size + 2.0 * D_FTINY;
    }
    vloc = ABOVE | BELOW;
    for (i = 0; i < nv; i++) {
        if ((j = plocate_d(va + 3 * i, cumin, cumax)))
            vloc &= j;
        else
            return 1;
    }
    if (vloc)
        return 0;
    for (i = 0; i < nv; i++) {
        if ((j = i + 1) >= nv)
            j = 0;
        for (int k = 0; k < 3; k++) {
            v1[k] = va[3 * i + k];
            v2[k] = va[3 * j + k];
        }
        if (clip_seg_d(v1, v2, cumin, cumax))
            return 1;
    }
    for (j = 0; j < 3; j++)
        if (nrm[j] > 0.0) {
            v1[j] = cumin[j];
            v2[j] = cumax[j];
        } else {
            v1[j] = cumax[j];
            v2[j] = cumin[j];
        }
    if ((d1 = v1[0] * nrm[0] + v1[1] * nrm[1] + v1[2] * nrm[2] - O.offset[obj]) > D_FTINY)
        return 0;
    if ((d2 = v2[0] * nrm[0] + v2[1] * nrm[1] + v2[2] * nrm[2] - O.offset[obj]) < -D_FTINY)
        return 0;
    for (j = 0; j < 3; j++)
        v1[j] = (v1[j] * d2 - v2[j] * d1) / (d2 - d1);
    return inface_d(v1, nv, O.ax[obj], va);
}

/* ot/sphere.c:50-109 */
__device__ int sphere_cube_d(const DevObjs &O, int obj, const double org[3], double size)
{
    const double *c = O.vert + 3 * O.voff[obj];
    double rad = fabs(O.offset[obj]), d1, d2, v1[3];
    int i;
    if (rad <= D_FTINY)
        return 0;
    d1 = 1.732050808 / 2.0 * size;
    d2 = size * 0.5;
    for (i = 0; i < 3; i++)
        v1[i] = org[i] + d2 - c[i];
    d2 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
    if (d2 > (rad + d1 + D_FTINY) * (rad + d1 + D_FTINY))
        return 0;
    if (d1 < rad) {
        if (d2 < (rad - d1 - D_FTINY) * (rad - d1 - D_FTINY))
            return 0;
        if (d2 < (rad + D_FTINY) * (rad + D_FTINY))
            return 1;
    }
    for (i = 0; i < 3; i++)
        if (c[i] < org[i])
            v1[i] = org[i] - c[i];
        else if (c[i] > org[i] + size)
            v1[i] = c[i] - (org[i] + size);
        else
            v1[i] = 0;
    return v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2] <= (rad + D_FTINY) * (rad + D_FTINY);
}

__device__ int object_cube_d(const DevObjs &O, int obj, const double org[3], double size)
{
    const int k = O.kind[obj];
    if (k == OK_FACE)
        return face_cube_d(O, obj, org, size);
    if (k == OK_SPHERE)
        return sphere_cube_d(O, obj, org, size);
    return 0;
}

/* level 0: surfaces overlapping the scene cube */
__global__ void k_root_flags(DevObjs O, int nobj, double o0, double o1, double o2, double size, int *flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nobj)
        return;
    const double org[3] = {o0, o1, o2};
    flag[i] = O.kind[i] ? object_cube_d(O, i, org, size) : 0;
}

__global__ void k_root_pairs(const int *flag, const int *pos, int nobj, int *pair_obj, int *pair_node)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nobj || !flag[i])
        return;
    pair_obj[pos[i]] = i;
    pair_node[pos[i]] = 0;
}

/* whether each cube of the level splits, and the length of its run of
 * child flags (8 per pair of a splitting cube) */
__global__ void k_split(const int *count, int n, int objlim, int big_ok, int small_ok, int *split, int *runlen)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int c = count[i];
    const int s = (c > objlim && big_ok) || (c > GB_MAXSET && small_ok);
    split[i] = s;
    runlen[i] = s ? 8 * c : 0;
}

/* flag of (pair p, child ch) at run[node] + ch * count + (p - begin) */
__global__ void k_child_test(DevObjs O, const int *pair_obj, const int *pair_node, long long npairs,
                             const int *split, const int *run, const int *begin, const int *count,
                             const double *norg, double ks, int *flag)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs * 8)
        return;
    const long long p = t >> 3;
    const int ch = (int)(t & 7);
    const int nd = pair_node[p];
    if (!split[nd])
        return;
    double org[3];
    for (int j = 0; j < 3; j++)
        org[j] = norg[3 * nd + j] + (((1 << j) & ch) ? ks : 0.0);
    const long long q = (long long)run[nd] + (long long)ch * count[nd] + (p - begin[nd]);
    flag[q] = object_cube_d(O, pair_obj[p], org, ks);
}

__global__ void k_scatter(const int *pair_obj, const int *pair_node, long long npairs, const int *split,
                          const int *run, const int *begin, const int *count, const int *flag, const int *pos,
                          const int *split_rank, int *out_obj, int *out_node)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs * 8)
        return;
    const long long p = t >> 3;
    const int ch = (int)(t & 7);
    const int nd = pair_node[p];
    if (!split[nd])
        return;
    const long long q = (long long)run[nd] + (long long)ch * count[nd] + (p - begin[nd]);
    if (!flag[q])
        return;
    out_obj[pos[q]] = pair_obj[p];
    out_node[pos[q]] = 8 * split_rank[nd] + ch;
}

/* the next level's cube corners: child ch of the r-th splitting cube is
 * cube 8 r + ch (its pairs are counted by k_count at the next level) */
__global__ void k_children(int n, const int *split, const int *split_rank, const double *norg, double ks,
                           double *corg)
{
    const int nd = blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= n || !split[nd])
        return;
    const int r = split_rank[nd];
    for (int ch = 0; ch < 8; ch++)
        for (int j = 0; j < 3; j++)
            corg[3 * (8 * r + ch) + j] = norg[3 * nd + j] + (((1 << j) & ch) ? ks : 0.0);
}

/* per-cube pair counts of a level from the pairs' cube indices (pairs are
 * grouped by cube, in cube order) */
__global__ void k_count(const int *pair_node, long long npairs, int *begin, int *count)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs)
        return;
    const int nd = pair_node[p];
    if (p == 0 || pair_node[p - 1] != nd)
        begin[nd] = (int)p;
    atomicAdd(count + nd, 1);
}

/* ---- exclusive scan of int32 (totals below 2^31) ---- */
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_BLOCK = SCAN_T * SCAN_PER;

__global__ void __launch_bounds__(SCAN_T) k_scan_block(const int *in, int *out, long long n, int *sums)
{
    __shared__ int part[SCAN_T];
    const long long base = (long long)blockIdx.x * SCAN_BLOCK + (long long)threadIdx.x * SCAN_PER;
    int v[SCAN_PER], s = 0;
    for (int k = 0; k < SCAN_PER; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < SCAN_T; o <<= 1) {
        const int x = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    int run = part[threadIdx.x] - s;
    for (int k = 0; k < SCAN_PER; k++) {
        if (base + k < n)
            out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_T - 1 && sums)
        sums[blockIdx.x] = part[SCAN_T - 1];
}

__global__ void k_scan_add(int *out, long long n, const int *offs)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] += offs[i / SCAN_BLOCK];
}

void scan_excl(const int *in, int *out, long long n, cudaStream_t st)
{
    if (n <= 0)
        return;
    const long long nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    if (nb == 1) {
        k_scan_block<<<1, SCAN_T, 0, st>>>(in, out, n, nullptr);
        return;
    }
    int *sums = nullptr, *offs = nullptr;
    cudaMallocAsync(&sums, nb * sizeof(int), st);
    cudaMallocAsync(&offs, nb * sizeof(int), st);
    k_scan_block<<<(unsigned)nb, SCAN_T, 0, st>>>(in, out, n, sums);
    scan_excl(sums, offs, nb, st);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, offs);
    cudaFreeAsync(sums, st);
    cudaFreeAsync(offs, st);
}

/* host side: the levels as downloaded */
struct Level {
    std::vector<int> begin, count, split, rank;
    std::vector<int> pair_obj;
};

struct Builder {
    gb_scene_host *S;
    std::vector<Level> lv;
    bool ok = true;
};

/* a cube after merging: a split (tree) or a leaf with its set (level,
 * begin, count) */
struct Cube {
    bool tree;
    int level, node;                  /* tree: where its children are */
    int slevel, sbegin, scount;       /* leaf: its set */
};

bool same_set(const Builder &B, const Cube &a, const Cube &b)
{
    if (a.scount != b.scount)
        return false;
    if (a.scount == 0)
        return true;
    return !memcmp(B.lv[a.slevel].pair_obj.data() + a.sbegin, B.lv[b.slevel].pair_obj.data() + b.sbegin,
                   (size_t)a.scount * sizeof(int));
}

/* the cube after merging equal leaf children, bottom-up */
Cube merged(Builder &B, int level, int node, std::vector<std::vector<char>> &leafed,
            std::vector<std::vector<int>> &sl, std::vector<std::vector<int>> &sb,
            std::vector<std::vector<int>> &sc)
{
    const Level &L = B.lv[level];
    Cube c;
    if (!L.split[node]) {
        c.tree = false;
        c.slevel = level;
        c.sbegin = L.begin[node];
        c.scount = L.count[node];
        return c;
    }
    const int base = 8 * L.rank[node];
    Cube k[8];
    bool all_leaves = true;
    for (int i = 0; i < 8; i++) {
        k[i] = merged(B, level + 1, base + i, leafed, sl, sb, sc);
        all_leaves &= !k[i].tree;
    }
    bool eq = all_leaves;
    for (int i = 1; eq && i < 8; i++)
        eq = same_set(B, k[0], k[i]);
    if (eq) {                                   /* this split becomes a leaf */
        leafed[level][node] = 1;
        sl[level][node] = k[0].slevel;
        sb[level][node] = k[0].sbegin;
        sc[level][node] = k[0].scount;
        c.tree = false;
        c.slevel = k[0].slevel;
        c.sbegin = k[0].sbegin;
        c.scount = k[0].scount;
        return c;
    }
    c.tree = true;
    c.level = level;
    c.node = node;
    return c;
}

int32_t emit_merged(Builder &B, int level, int node, const std::vector<std::vector<char>> &leafed,
                    const std::vector<std::vector<int>> &sl, const std::vector<std::vector<int>> &sb,
                    const std::vector<std::vector<int>> &sc)
{
    const Level &L = B.lv[level];
    if (!L.split[node] || leafed[level][node]) {
        const int lvl = L.split[node] ? sl[level][node] : level;
        const int beg = L.split[node] ? sb[level][node] : L.begin[node];
        const int c = L.split[node] ? sc[level][node] : L.count[node];
        if (c == 0)
            return -1;
        if (c > GB_MAXSET) {
            B.ok = false;
            return -1;
        }
        std::vector<int32_t> tmp((size_t)c + 1);
        tmp[0] = c;
        memcpy(tmp.data() + 1, B.lv[lvl].pair_obj.data() + beg, (size_t)c * sizeof(int32_t));
        const int32_t code = gb__add_set(B.S, tmp.data());
        if (code == 0)
            B.ok = false;
        return code;
    }
    int32_t out = gb__new_node(B.S);
    if (out < 0) {
        B.ok = false;
        return -1;
    }
    const int base = 8 * L.rank[node];
    for (int i = 0; i < 8; i++) {
        const int32_t c = emit_merged(B, level + 1, base + i, leafed, sl, sb, sc);
        if (!B.ok)
            return -1;
        B.S->kids[8 * out + i] = c;
    }
    return out;
}

}  // namespace

/* Builds the octree of S on the current device.  0: built; 1: the scene
 * holds objects this builder does not handle (the host builder is to be
 * used); < 0: failure, with the reason in err. */
extern "C" int gb_scene_build_octree_device(gb_scene_host *S, int objlim, int resolu, char *err, size_t errlen)
{
    auto fail = [&](const char *what) {
        snprintf(err, errlen, "%s: %s", what, cudaGetErrorString(cudaGetLastError()));
        return -1;
    };
    for (int32_t i = 0; i < S->nobjs; i++) {
        const int t = S->objs[i].otype;
        if (gb_is_surface(t) && t != GT_SOURCE && t != GT_POLYGON && t != GT_SPHERE && t != GT_BUBBLE)
            return 1;
    }
    if (gb_scene_octree_cube(S) < 0) {
        snprintf(err, errlen, "%s", "objects without an octree builder");
        return -1;
    }
    const int nobj = S->nobjs;
    objlim = objlim > 0 ? objlim : 6;
    const double mincusize = S->cusize / (resolu > 0 ? resolu : 16384) - GB_FTINY;
    /* objects on the device */
    std::vector<int> kind(nobj, 0), nv(nobj, 0), ax(nobj, 0), okf(nobj, 0);
    std::vector<long long> voff(nobj, 0);
    std::vector<double> norm(3 * (size_t)nobj, 0.0), offs(nobj, 0.0), vert;
    for (int32_t i = 0; i < nobj; i++) {
        const gb_object *o = &S->objs[i];
        voff[i] = (long long)(vert.size() / 3);
        if (o->otype == GT_POLYGON) {
            const gb_face *f = &S->faces[i];
            kind[i] = OK_FACE;
            nv[i] = f->nv;
            ax[i] = f->ax;
            okf[i] = f->ok;
            for (int j = 0; j < 3; j++)
                norm[3 * (size_t)i + j] = f->norm[j];
            offs[i] = f->offset;
            vert.insert(vert.end(), o->farg, o->farg + 3 * f->nv);
        } else if (o->otype == GT_SPHERE || o->otype == GT_BUBBLE) {
            kind[i] = OK_SPHERE;
            offs[i] = o->farg[3];
            vert.insert(vert.end(), o->farg, o->farg + 3);
        }
    }
    if (vert.empty())
        vert.push_back(0.0);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return fail("stream");
    std::vector<void *> owned;
    auto dalloc = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 4) != cudaSuccess)
            return nullptr;
        owned.push_back(p);
        return p;
    };
    auto upload = [&](const void *h, size_t bytes) -> void * {
        void *p = dalloc(bytes);
        if (p && bytes)
            cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, st);
        return p;
    };
    int rc = 0;
    Builder B;
    B.S = S;
    do {
        DevObjs O;
        O.kind = (const int *)upload(kind.data(), kind.size() * 4);
        O.nv = (const int *)upload(nv.data(), nv.size() * 4);
        O.ax = (const int *)upload(ax.data(), ax.size() * 4);
        O.ok = (const int *)upload(okf.data(), okf.size() * 4);
        O.voff = (const long long *)upload(voff.data(), voff.size() * 8);
        O.norm = (const double *)upload(norm.data(), norm.size() * 8);
        O.offset = (const double *)upload(offs.data(), offs.size() * 8);
        O.vert = (const double *)upload(vert.data(), vert.size() * 8);
        if (!O.kind || !O.nv || !O.ax || !O.ok || !O.voff || !O.norm || !O.offset || !O.vert) {
            rc = fail("object upload");
            break;
        }
        /* level 0 */
        int *flag0 = (int *)dalloc((size_t)nobj * 4), *pos0 = (int *)dalloc((size_t)nobj * 4);
        if (!flag0 || !pos0) {
            rc = fail("allocation");
            break;
        }
        k_root_flags<<<(nobj + 255) / 256, 256, 0, st>>>(O, nobj, S->cuorg[0], S->cuorg[1], S->cuorg[2], S->cusize,
                                                          flag0);
        scan_excl(flag0, pos0, nobj, st);
        int last[2] = {0, 0};
        cudaMemcpyAsync(&last[0], pos0 + nobj - 1, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&last[1], flag0 + nobj - 1, 4, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            rc = fail("root pairs");
            break;
        }
        long long npairs = (long long)last[0] + last[1];
        int *pobj = (int *)dalloc((size_t)(npairs ? npairs : 1) * 4);
        int *pnode = (int *)dalloc((size_t)(npairs ? npairs : 1) * 4);
        double *norg = (double *)upload(S->cuorg, 3 * sizeof(double));
        if (!pobj || !pnode || !norg) {
            rc = fail("allocation");
            break;
        }
        k_root_pairs<<<(nobj + 255) / 256, 256, 0, st>>>(flag0, pos0, nobj, pobj, pnode);
        int nnodes = 1;
        double size = S->cusize;
        for (int level = 0;; level++) {
            const double ks = size * 0.5;
            const int big_ok = !(ks < mincusize), small_ok = !(ks < mincusize / 256.0);
            int *begin = (int *)dalloc((size_t)nnodes * 4), *count = (int *)dalloc((size_t)nnodes * 4);
            int *split = (int *)dalloc((size_t)nnodes * 4), *run = (int *)dalloc((size_t)nnodes * 4);
            int *runlen = (int *)dalloc((size_t)nnodes * 4), *rank = (int *)dalloc((size_t)nnodes * 4);
            if (!begin || !count || !split || !run || !runlen || !rank) {
                rc = fail("allocation");
                break;
            }
            cudaMemsetAsync(begin, 0, (size_t)nnodes * 4, st);
            cudaMemsetAsync(count, 0, (size_t)nnodes * 4, st);
            if (npairs)
                k_count<<<(unsigned)((npairs + 255) / 256), 256, 0, st>>>(pnode, npairs, begin, count);
            k_split<<<(nnodes + 255) / 256, 256, 0, st>>>(count, nnodes, objlim, big_ok, small_ok, split, runlen);
            scan_excl(runlen, run, nnodes, st);
            scan_excl(split, rank, nnodes, st);
            Level L;
            L.begin.resize(nnodes);
            L.count.resize(nnodes);
            L.split.resize(nnodes);
            L.rank.resize(nnodes);
            L.pair_obj.resize((size_t)npairs);
            cudaMemcpyAsync(L.begin.data(), begin, (size_t)nnodes * 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(L.count.data(), count, (size_t)nnodes * 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(L.split.data(), split, (size_t)nnodes * 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(L.rank.data(), rank, (size_t)nnodes * 4, cudaMemcpyDeviceToHost, st);
            if (npairs)
                cudaMemcpyAsync(L.pair_obj.data(), pobj, (size_t)npairs * 4, cudaMemcpyDeviceToHost, st);
            int tail[2] = {0, 0};
            cudaMemcpyAsync(&tail[0], run + nnodes - 1, 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&tail[1], runlen + nnodes - 1, 4, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) {
                rc = fail("level");
                break;
            }
            int nsplit = 0;
            for (int i = 0; i < nnodes; i++)
                nsplit += L.split[i];
            const long long nflags = (long long)tail[0] + tail[1];
            B.lv.push_back(std::move(L));
            if (nsplit == 0)
                break;
            if (nflags > (1ll << 31) - 1 || (long long)nsplit * 8 > (1ll << 31) - 1) {
                snprintf(err, errlen, "octree level %d too large for the device builder", level);
                rc = -1;
                break;
            }
            int *flag = (int *)dalloc((size_t)nflags * 4), *pos = (int *)dalloc((size_t)nflags * 4);
            if (!flag || !pos) {
                rc = fail("allocation");
                break;
            }
            const unsigned g8 = (unsigned)((npairs * 8 + 255) / 256);
            k_child_test<<<g8, 256, 0, st>>>(O, pobj, pnode, npairs, split, run, begin, count, norg, ks, flag);
            scan_excl(flag, pos, nflags, st);
            const int cn = 8 * nsplit;
            double *corg = (double *)dalloc((size_t)cn * 3 * 8);
            int ntail[2] = {0, 0};
            cudaMemcpyAsync(&ntail[0], pos + nflags - 1, 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&ntail[1], flag + nflags - 1, 4, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess || !corg) {
                rc = fail("child tests");
                break;
            }
            const long long nnext = (long long)ntail[0] + ntail[1];
            int *nobj_ = (int *)dalloc((size_t)(nnext ? nnext : 1) * 4);
            int *nnode_ = (int *)dalloc((size_t)(nnext ? nnext : 1) * 4);
            if (!nobj_ || !nnode_) {
                rc = fail("allocation");
                break;
            }
            k_scatter<<<g8, 256, 0, st>>>(pobj, pnode, npairs, split, run, begin, count, flag, pos, rank, nobj_,
                                          nnode_);
            k_children<<<(nnodes + 255) / 256, 256, 0, st>>>(nnodes, split, rank, norg, ks, corg);
            if (cudaStreamSynchronize(st) != cudaSuccess) {
                rc = fail("next level");
                break;
            }
            /* the previous level's device arrays are no longer needed */
            for (void *p : {(void *)pobj, (void *)pnode, (void *)norg, (void *)flag, (void *)pos, (void *)begin,
                            (void *)count, (void *)split, (void *)run, (void *)runlen, (void *)rank}) {
                for (auto &q : owned)
                    if (q == p) {
                        cudaFree(q);
                        q = nullptr;
                    }
            }
            pobj = nobj_;
            pnode = nnode_;
            norg = corg;
            npairs = nnext;
            nnodes = cn;
            size = ks;
        }
    } while (0);
    for (void *p : owned)
        if (p)
            cudaFree(p);
    cudaStreamDestroy(st);
    if (rc < 0)
        return rc;
    /* merge equal leaf children, then store the tree as the host builder does */
    S->nnodes = 0;
    S->nsets = 0;
    S->set_len = 0;
    std::vector<std::vector<char>> leafed(B.lv.size());
    std::vector<std::vector<int>> sl(B.lv.size()), sb(B.lv.size()), sc(B.lv.size());
    for (size_t l = 0; l < B.lv.size(); l++) {
        leafed[l].assign(B.lv[l].split.size(), 0);
        sl[l].assign(B.lv[l].split.size(), 0);
        sb[l].assign(B.lv[l].split.size(), 0);
        sc[l].assign(B.lv[l].split.size(), 0);
    }
    merged(B, 0, 0, leafed, sl, sb, sc);
    S->root = emit_merged(B, 0, 0, leafed, sl, sb, sc);
    if (!B.ok) {
        snprintf(err, errlen, "%s", "set overflow or out of memory while storing the octree");
        return -1;
    }
    return 0;
}
