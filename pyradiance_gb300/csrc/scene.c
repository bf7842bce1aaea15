/*
 * scene.c -- Radiance scene ingestion (see scene.h).
 *
 * Formats follow the reference: octree files as written by ot/writeoct.c and
 * read by common/readoct.c:29-260, frozen object records as in
 * common/sceneio.c:20-110, portable integers/floats as in
 * common/portio.c:94-152, scene text as read by common/readobj.c.
 */
#define _GNU_SOURCE
#include "scene.h"

#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[512];

const char *gb_scene_error(void) { return g_err; }

static int fail(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return -1;
}

/* ------------------------------------------------------------------ types */

static const struct { const char *name; int t; } TYPE_NAMES[] = {
    {"polygon", GT_POLYGON}, {"cone", GT_CONE}, {"sphere", GT_SPHERE},
    {"texfunc", GT_TEXTURE}, {"ring", GT_RING}, {"cylinder", GT_CYLINDER},
    {"instance", GT_INSTANCE}, {"cup", GT_CUP}, {"bubble", GT_BUBBLE},
    {"tube", GT_TUBE}, {"mesh", GT_MESH}, {"alias", GT_ALIAS},
    {"plastic", GT_PLASTIC}, {"metal", GT_METAL}, {"glass", GT_GLASS},
    {"trans", GT_TRANS}, {"dielectric", GT_DIELECTRIC},
    {"plastic2", GT_OTHER_MATERIAL}, {"metal2", GT_OTHER_MATERIAL},
    {"trans2", GT_OTHER_MATERIAL}, {"interface", GT_INTERFACE},
    {"plasfunc", GT_OTHER_MATERIAL}, {"metfunc", GT_OTHER_MATERIAL},
    {"brightfunc", GT_PATTERN}, {"brightdata", GT_PATTERN},
    {"brighttext", GT_PATTERN}, {"colorpict", GT_PATTERN},
    {"glow", GT_GLOW}, {"source", GT_SOURCE}, {"light", GT_LIGHT},
    {"illum", GT_ILLUM}, {"spotlight", GT_SPOT}, {"mist", GT_OTHER_MATERIAL},
    {"mirror", GT_MIRROR}, {"transfunc", GT_OTHER_MATERIAL},
    {"BRTDfunc", GT_OTHER_MATERIAL}, {"BSDF", GT_OTHER_MATERIAL},
    {"aBSDF", GT_OTHER_MATERIAL}, {"WGMDfunc", GT_OTHER_MATERIAL},
    {"plasdata", GT_OTHER_MATERIAL}, {"metdata", GT_OTHER_MATERIAL},
    {"transdata", GT_OTHER_MATERIAL}, {"colorfunc", GT_PATTERN},
    {"antimatter", GT_ANTIMATTER}, {"colordata", GT_PATTERN},
    {"colortext", GT_PATTERN}, {"texdata", GT_TEXTURE},
    {"mixfunc", GT_MIXTURE}, {"mixdata", GT_MIXTURE}, {"mixtext", GT_MIXTURE},
    {"mixpict", GT_MIXTURE}, {"prism1", GT_OTHER_MATERIAL},
    {"prism2", GT_OTHER_MATERIAL}, {"ashik2", GT_OTHER_MATERIAL},
    {"spectrum", GT_PATTERN}, {"specfile", GT_PATTERN},
    {"specfunc", GT_PATTERN}, {"specdata", GT_PATTERN},
    {"specpict", GT_PATTERN},
};

int gb_otype_from_name(const char *name)
{
    size_t i;
    for (i = 0; i < sizeof TYPE_NAMES / sizeof TYPE_NAMES[0]; i++)
        if (!strcmp(TYPE_NAMES[i].name, name))
            return TYPE_NAMES[i].t;
    return GT_UNKNOWN;
}

const char *gb_otype_name(int t)
{
    size_t i;
    for (i = 0; i < sizeof TYPE_NAMES / sizeof TYPE_NAMES[0]; i++)
        if (TYPE_NAMES[i].t == t)
            return TYPE_NAMES[i].name;
    return "unknown";
}

int gb_is_surface(int t) { return t >= GT_POLYGON && t <= GT_MESH; }
int gb_is_material(int t) { return t >= GT_PLASTIC && t <= GT_OTHER_MATERIAL; }
int gb_is_light(int t) { return t == GT_LIGHT || t == GT_ILLUM || t == GT_GLOW || t == GT_SPOT; }
int gb_is_transp(int t)
{
    return t == GT_TRANS || t == GT_GLASS || t == GT_DIELECTRIC || t == GT_INTERFACE;
}
int gb_is_volume(int t)
{
    return t == GT_INSTANCE || t == GT_MESH;     /* T_V in common/otypes.h:126-137 */
}

/* ---------------------------------------------------------------- storage */

void gb_scene_init(gb_scene_host *S)
{
    memset(S, 0, sizeof *S);
    S->root = -1;
}

void gb_scene_clear(gb_scene_host *S)
{
    int32_t i;
    int k;
    for (i = 0; i < S->nobjs; i++) {
        gb_object *o = &S->objs[i];
        free(o->name);
        for (k = 0; k < o->nsargs; k++)
            free(o->sarg[k]);
        free(o->sarg);
        free(o->farg);
        free(o->vnorm);
        free(o->vuv);
    }
    free(S->objs);
    free(S->kids);
    free(S->set_off);
    free(S->set_data);
    free(S->faces);
    free(S->cones);
    for (k = 0; k < S->nfiles; k++)
        free(S->files[k]);
    free(S->files);
    for (k = 0; k < S->nsubs; k++)
        free(S->subs[k].name);
    free(S->subs);
    free(S->inst);
    gb_scene_init(S);
}

static gb_object *new_object(gb_scene_host *S)
{
    if (S->nobjs == S->cap_objs) {
        int32_t nc = S->cap_objs ? S->cap_objs * 2 : 1024;
        gb_object *p = (gb_object *)realloc(S->objs, (size_t)nc * sizeof *p);
        if (!p)
            return NULL;
        S->objs = p;
        S->cap_objs = nc;
    }
    memset(&S->objs[S->nobjs], 0, sizeof(gb_object));
    return &S->objs[S->nobjs++];
}

int32_t gb__new_node(gb_scene_host *S)
{
    if (S->nnodes == S->cap_nodes) {
        int32_t nc = S->cap_nodes ? S->cap_nodes * 2 : 4096;
        int32_t *p = (int32_t *)realloc(S->kids, (size_t)nc * 8 * sizeof *p);
        if (!p)
            return -1;
        S->kids = p;
        S->cap_nodes = nc;
    }
    return S->nnodes++;
}

/* append a sorted set; returns its leaf code */
int32_t gb__add_set(gb_scene_host *S, const int32_t *set)
{
    int64_t need = (int64_t)set[0] + 1;
    if (S->nsets == S->cap_sets) {
        int32_t nc = S->cap_sets ? S->cap_sets * 2 : 4096;
        int64_t *p = (int64_t *)realloc(S->set_off, (size_t)nc * sizeof *p);
        if (!p)
            return 0;
        S->set_off = p;
        S->cap_sets = nc;
    }
    while (S->set_len + need > S->cap_set_data) {
        int64_t nc = S->cap_set_data ? S->cap_set_data * 2 : 65536;
        int32_t *p = (int32_t *)realloc(S->set_data, (size_t)nc * sizeof *p);
        if (!p)
            return 0;
        S->set_data = p;
        S->cap_set_data = nc;
    }
    S->set_off[S->nsets] = S->set_len;
    memcpy(S->set_data + S->set_len, set, (size_t)need * sizeof(int32_t));
    S->set_len += need;
    return -(S->nsets++) - 2;
}

const int32_t *gb_scene_set(const gb_scene_host *S, int32_t code)
{
    return S->set_data + S->set_off[-code - 2];
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* ------------------------------------------------------------ scene text */

typedef struct {
    const char *p, *end;
    const char *what;
    int line;
} lexer;

static int lex_word(lexer *L, char *buf, size_t n)
{
    size_t k = 0;
    while (L->p < L->end) {
        if (*L->p == '\n')
            L->line++;
        if (!isspace((unsigned char)*L->p))
            break;
        L->p++;
    }
    if (L->p >= L->end)
        return 0;
    if (*L->p == '"') {           /* quoted word (common/fgetword.c) */
        L->p++;
        while (L->p < L->end && *L->p != '"') {
            if (k + 1 < n)
                buf[k++] = *L->p;
            L->p++;
        }
        if (L->p < L->end)
            L->p++;
    } else {
        while (L->p < L->end && !isspace((unsigned char)*L->p)) {
            if (k + 1 < n)
                buf[k++] = *L->p;
            L->p++;
        }
    }
    buf[k] = '\0';
    return 1;
}

/* name -> latest modifier index; a simple open hash (common/modobject.c:81) */
typedef struct {
    int32_t cap;
    int32_t *slot;
} modtab;

static uint32_t strhash(const char *s)
{
    uint32_t h = 2166136261u;
    while (*s)
        h = (h ^ (unsigned char)*s++) * 16777619u;
    return h;
}

static int32_t modtab_find(const gb_scene_host *S, const modtab *T, const char *name)
{
    uint32_t h;
    if (!T->cap)
        return -1;
    for (h = strhash(name) & (T->cap - 1);; h = (h + 1) & (T->cap - 1)) {
        int32_t i = T->slot[h];
        if (i < 0)
            return -1;
        if (!strcmp(S->objs[i].name, name))
            return i;
    }
}

static int modtab_put(const gb_scene_host *S, modtab *T, int32_t obj)
{
    uint32_t h;
    if ((S->nobjs + 1) * 2 > T->cap) {     /* rebuild larger */
        int32_t nc = T->cap ? T->cap * 2 : 1024, k;
        int32_t *old = T->slot, oc = T->cap;
        while (nc < (S->nobjs + 1) * 2)
            nc *= 2;
        T->slot = (int32_t *)malloc((size_t)nc * sizeof(int32_t));
        if (!T->slot)
            return -1;
        for (k = 0; k < nc; k++)
            T->slot[k] = -1;
        T->cap = nc;
        for (k = 0; k < oc; k++)
            if (old[k] >= 0)
                modtab_put(S, T, old[k]);
        free(old);
    }
    for (h = strhash(S->objs[obj].name) & (T->cap - 1);; h = (h + 1) & (T->cap - 1)) {
        int32_t i = T->slot[h];
        if (i < 0 || !strcmp(S->objs[i].name, S->objs[obj].name)) {
            T->slot[h] = obj;
            return 0;
        }
    }
}

static int is_modifier_type(int t)
{
    return !gb_is_surface(t) && t != GT_UNKNOWN;
}

static int parse_text(gb_scene_host *S, const char *text, size_t len, const char *what)
{
    lexer L = {text, text + len, what, 1};
    char w[4096];
    modtab T = {0, NULL};
    int32_t i;
    int rc = 0;
    /* modifiers already loaded (from an earlier file) stay visible */
    for (i = 0; i < S->nobjs; i++)
        if (is_modifier_type(S->objs[i].otype))
            modtab_put(S, &T, i);
    for (;;) {
        gb_object *o;
        int32_t idx;
        long n, k;
        char *endp;
        /* skip blanks and comments */
        while (L.p < L.end && isspace((unsigned char)*L.p)) {
            if (*L.p == '\n')
                L.line++;
            L.p++;
        }
        if (L.p >= L.end)
            break;
        if (*L.p == '#') {
            while (L.p < L.end && *L.p != '\n')
                L.p++;
            continue;
        }
        if (*L.p == '!') {
            rc = fail("%s:%d: scene commands ('!...') are not supported; "
                      "expand them into a file first", what, L.line);
            break;
        }
        if (!lex_word(&L, w, sizeof w))
            break;
        o = new_object(S);
        if (!o) {
            rc = fail("out of memory reading %s", what);
            break;
        }
        idx = S->nobjs - 1;
        if (!strcmp(w, "void"))
            o->omod = -1;
        else {
            o->omod = modtab_find(S, &T, w);
            if (o->omod < 0) {
                rc = fail("%s:%d: undefined modifier \"%s\"", what, L.line, w);
                break;
            }
        }
        if (!lex_word(&L, w, sizeof w)) {
            rc = fail("%s:%d: missing object type", what, L.line);
            break;
        }
        o->otype = gb_otype_from_name(w);
        if (o->otype == GT_UNKNOWN) {
            rc = fail("%s:%d: unknown object type \"%s\"", what, L.line, w);
            break;
        }
        if (!lex_word(&L, w, sizeof w)) {
            rc = fail("%s:%d: missing object name", what, L.line);
            break;
        }
        o->name = strdup(w);
        /* string arguments */
        if (!lex_word(&L, w, sizeof w) || (n = strtol(w, &endp, 10), *endp) || n < 0) {
            rc = fail("%s:%d: bad string argument count for %s", what, L.line, o->name);
            break;
        }
        o->nsargs = (int)n;
        o->sarg = n ? (char **)calloc((size_t)n, sizeof(char *)) : NULL;
        for (k = 0; k < n; k++) {
            if (!lex_word(&L, w, sizeof w)) {
                rc = fail("%s:%d: missing string argument", what, L.line);
                goto out;
            }
            o->sarg[k] = strdup(w);
        }
        /* integer arguments (always 0 in the reference, IARGS unset) */
        if (!lex_word(&L, w, sizeof w) || (n = strtol(w, &endp, 10), *endp) || n != 0) {
            rc = fail("%s:%d: bad integer argument count for %s", what, L.line, o->name);
            break;
        }
        if (!lex_word(&L, w, sizeof w) || (n = strtol(w, &endp, 10), *endp) || n < 0) {
            rc = fail("%s:%d: bad real argument count for %s", what, L.line, o->name);
            break;
        }
        o->nfargs = (int)n;
        o->farg = n ? (double *)calloc((size_t)n, sizeof(double)) : NULL;
        for (k = 0; k < n; k++) {
            if (!lex_word(&L, w, sizeof w)) {
                rc = fail("%s:%d: missing real argument", what, L.line);
                goto out;
            }
            o->farg[k] = strtod(w, &endp);
            if (*endp) {
                rc = fail("%s:%d: bad real argument \"%s\"", what, L.line, w);
                goto out;
            }
        }
        if (is_modifier_type(o->otype))
            modtab_put(S, &T, idx);
    }
out:
    free(T.slot);
    return rc;
}

int gb_scene_read_rad_text(gb_scene_host *S, const char *text, const char *what)
{
    return parse_text(S, text, strlen(text), what ? what : "scene text");
}

static char *slurp(const char *path, size_t *len)
{
    FILE *fp = fopen(path, "rb");
    char *buf;
    long n;
    if (!fp)
        return NULL;
    fseek(fp, 0, SEEK_END);
    n = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    buf = (char *)malloc((size_t)n + 1);
    if (buf && fread(buf, 1, (size_t)n, fp) != (size_t)n) {
        free(buf);
        buf = NULL;
    }
    fclose(fp);
    if (buf) {
        buf[n] = '\0';
        *len = (size_t)n;
    }
    return buf;
}

int gb_scene_read_rad_file(gb_scene_host *S, const char *path)
{
    size_t len = 0;
    char *buf = slurp(path, &len);
    int rc;
    if (!buf)
        return fail("cannot open scene file \"%s\"", path);
    rc = parse_text(S, buf, len, path);
    free(buf);
    return rc;
}

/* ---------------------------------------------------------- octree files */

double gb_portable_flt(long l, int e)
{
    double d;
    if (l == 0)
        return 0.0;
    d = (l + .5 - (l < 0)) * (1. / 0x7fffffff);
    return ldexp(d, e);
}

typedef struct {
    const unsigned char *p, *end;
} rdr;

static int r_eof(rdr *R) { return R->p >= R->end; }

static long r_int(rdr *R, int siz, int *ok)
{
    long r;
    int c;
    if (R->p + siz > R->end) {
        *ok = 0;
        return -1;
    }
    c = *R->p++;
    r = c;
    if (c & 0x80)
        r |= -256L;
    while (--siz > 0) {
        c = *R->p++;
        r = (r << 8) | c;
    }
    return r;
}

static double r_flt(rdr *R, int *ok)
{
    long l = r_int(R, 4, ok);
    if (!*ok)
        return 0.0;
    if (l == 0) {
        r_int(R, 1, ok);
        return 0.0;
    }
    return gb_portable_flt(l, (int)r_int(R, 1, ok));
}

static const char *r_str(rdr *R, int *ok)
{
    const unsigned char *s = R->p;
    while (R->p < R->end && *R->p)
        R->p++;
    if (R->p >= R->end) {
        *ok = 0;
        return "";
    }
    R->p++;
    return (const char *)s;
}

static int32_t read_tree(gb_scene_host *S, rdr *R, int objsize, int32_t objorig, int *ok, int depth)
{
    int c;
    if (r_eof(R) || depth > 64) {
        *ok = 0;
        return -1;
    }
    c = *R->p++;
    if (c == 0)
        return -1;                               /* OT_EMPTY */
    if (c == 1) {                                /* OT_FULL */
        int32_t set[GB_MAXSET + 1];
        long n = r_int(R, objsize, ok), k;
        if (!*ok || n < 1 || n > GB_MAXSET) {
            *ok = 0;
            return -1;
        }
        set[0] = (int32_t)n;
        for (k = 1; k <= n; k++)
            set[k] = (int32_t)(r_int(R, objsize, ok) + objorig);
        if (!*ok)
            return -1;
        qsort(set + 1, (size_t)n, sizeof(int32_t), cmp_i32);
        return gb__add_set(S, set);
    }
    if (c == 2) {                                /* OT_TREE */
        int32_t nd = gb__new_node(S), k;
        if (nd < 0) {
            *ok = 0;
            return -1;
        }
        for (k = 0; k < 8; k++) {
            int32_t kid = read_tree(S, R, objsize, objorig, ok, depth + 1);
            if (!*ok)
                return -1;
            S->kids[8 * nd + k] = kid;
        }
        return nd;
    }
    *ok = 0;
    return -1;
}

static int read_frozen(gb_scene_host *S, rdr *R, int objsize, int32_t objorig)
{
    int typemap[128];
    int ntypes = 0, ok = 1;
    for (;;) {
        const char *s = r_str(R, &ok);
        if (!ok)
            return fail("truncated octree (type list)");
        if (!*s)
            break;
        if (ntypes >= 128)
            return fail("damaged octree (type list)");
        typemap[ntypes++] = gb_otype_from_name(s);
    }
    for (;;) {
        long t = r_int(R, 1, &ok), m, n, k;
        gb_object *o;
        if (!ok)
            return fail("truncated octree (objects)");
        if (t == -1)
            break;
        if (t < 0 || t >= ntypes)
            return fail("reference to unknown object type in octree");
        o = new_object(S);
        if (!o)
            return fail("out of memory");
        o->otype = typemap[t];
        m = r_int(R, objsize, &ok);
        o->omod = m == -1 ? -1 : (int32_t)(m + objorig);
        o->name = strdup(r_str(R, &ok));
        n = r_int(R, 2, &ok);
        o->nsargs = (int)n;
        o->sarg = n > 0 ? (char **)calloc((size_t)n, sizeof(char *)) : NULL;
        for (k = 0; k < n; k++)
            o->sarg[k] = strdup(r_str(R, &ok));
        n = r_int(R, 2, &ok);
        o->nfargs = (int)n;
        o->farg = n > 0 ? (double *)calloc((size_t)n, sizeof(double)) : NULL;
        for (k = 0; k < n; k++)
            o->farg[k] = r_flt(R, &ok);
        if (!ok)
            return fail("unexpected EOF in octree objects");
        if (o->otype == GT_UNKNOWN)
            return fail("object \"%s\" has a type this library does not know", o->name);
    }
    return 0;
}

static char *dir_of(const char *path)
{
    const char *s = strrchr(path, '/');
    size_t n = s ? (size_t)(s - path) : 0;
    char *d = (char *)malloc(n + 2);
    if (!s) {
        strcpy(d, ".");
        return d;
    }
    memcpy(d, path, n);
    d[n] = '\0';
    return d;
}

int gb_scene_read_oct(gb_scene_host *S, const char *path)
{
    size_t len = 0;
    char *buf = slurp(path, &len);
    rdr R;
    int ok = 1, objsize, i;
    long magic, nobj;
    int32_t objorig = S->nobjs;
    const char *fmt = NULL;
    char line[256];
    if (!buf)
        return fail("cannot open octree file \"%s\"", path);
    R.p = (const unsigned char *)buf;
    R.end = R.p + len;
    /* information header: lines up to an empty line (common/header.c) */
    for (;;) {
        size_t k = 0;
        while (R.p < R.end && *R.p != '\n') {
            if (k + 1 < sizeof line)
                line[k++] = (char)*R.p;
            R.p++;
        }
        if (R.p >= R.end) {
            free(buf);
            return fail("(%s): not an octree", path);
        }
        R.p++;
        line[k] = '\0';
        if (!k)
            break;
        if (!strncmp(line, "FORMAT=", 7))
            fmt = line + 7, (void)fmt;
        if (!strncmp(line, "FORMAT=", 7) && strcmp(line + 7, "Radiance_octree")) {
            free(buf);
            return fail("(%s): not an octree", path);
        }
    }
    magic = r_int(&R, 2, &ok);
    objsize = (int)(magic - (4 * 8 + 251));
    if (!ok || objsize <= 0 || objsize > 8) {
        free(buf);
        return fail("(%s): incompatible octree format", path);
    }
    for (i = 0; i < 3; i++)
        S->cuorg[i] = atof(r_str(&R, &ok));
    S->cusize = atof(r_str(&R, &ok));
    /* scene file names (unfrozen octree) */
    for (;;) {
        const char *s = r_str(&R, &ok);
        if (!ok) {
            free(buf);
            return fail("(%s): truncated octree", path);
        }
        if (!*s)
            break;
        S->files = (char **)realloc(S->files, (size_t)(S->nfiles + 1) * sizeof(char *));
        S->files[S->nfiles++] = strdup(s);
    }
    for (i = 0; i < S->nfiles; i++) {
        FILE *fp = fopen(S->files[i], "rb");
        if (fp) {
            fclose(fp);
            if (gb_scene_read_rad_file(S, S->files[i]) < 0) {
                free(buf);
                return -1;
            }
        } else {
            char *d = dir_of(path);
            char *alt = (char *)malloc(strlen(d) + strlen(S->files[i]) + 2);
            sprintf(alt, "%s/%s", d, S->files[i]);
            free(d);
            if (gb_scene_read_rad_file(S, alt) < 0) {
                free(alt);
                free(buf);
                return fail("(%s): cannot open scene file \"%s\"", path, S->files[i]);
            }
            free(alt);
        }
    }
    nobj = r_int(&R, objsize, &ok);
    if (!ok || nobj < 0) {
        free(buf);
        return fail("(%s): truncated octree", path);
    }
    S->root = read_tree(S, &R, objsize, objorig, &ok, 0);
    if (!ok) {
        free(buf);
        return fail("(%s): truncated or damaged octree", path);
    }
    if (S->nfiles == 0) {
        if (read_frozen(S, &R, objsize, objorig) < 0) {
            free(buf);
            return -1;
        }
    }
    free(buf);
    if (S->nobjs != objorig + nobj)
        return fail("(%s): bad object count; octree stale?", path);
    return 0;
}

/* -------------------------------------------------------------- modifiers */

int32_t gb_find_material(const gb_scene_host *S, int32_t obj)
{
    int32_t m = S->objs[obj].omod;
    int guard = 0;
    while (m >= 0 && guard++ < 1000) {
        const gb_object *o = &S->objs[m];
        if (gb_is_material(o->otype) || o->otype == GT_ANTIMATTER)
            return m;
        if (o->otype == GT_ALIAS && o->nsargs > 0) {
            /* alias name target: most recent modifier of that name before m */
            int32_t k;
            for (k = m - 1; k >= 0; k--)
                if (!gb_is_surface(S->objs[k].otype) && !strcmp(S->objs[k].name, o->sarg[0]))
                    break;
            if (k < 0)
                return -1;
            m = k;
            continue;
        }
        m = o->omod;
    }
    return -1;
}

/* ------------------------------------------------------------- precompute */

static double vnorm(double v[3])
{
    double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0) {
        v[0] /= l;
        v[1] /= l;
        v[2] /= l;
    }
    return l;
}

/* common/face.c:35-112 */
static void make_face(const gb_object *o, gb_face *f)
{
    const double *va = o->farg;
    double v1[3], v2[3], v3[3], d1;
    int i;
    f->nv = o->nfargs / 3;
    if (f->nv > 3) {
        const double *a = va, *b = va + 3 * (f->nv - 1);
        double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        if (dx * dx + dy * dy + dz * dz <= GB_FTINY * GB_FTINY)
            f->nv--;
    }
    f->norm[0] = f->norm[1] = f->norm[2] = 0.0;
    for (i = 0; i < 3; i++)
        v1[i] = va[3 + i] - va[i];
    for (i = 2; i < f->nv; i++) {
        int k;
        for (k = 0; k < 3; k++)
            v2[k] = va[3 * i + k] - va[k];
        v3[0] = v1[1] * v2[2] - v1[2] * v2[1];
        v3[1] = v1[2] * v2[0] - v1[0] * v2[2];
        v3[2] = v1[0] * v2[1] - v1[1] * v2[0];
        f->norm[0] += v3[0];
        f->norm[1] += v3[1];
        f->norm[2] += v3[2];
        v1[0] = v2[0];
        v1[1] = v2[1];
        v1[2] = v2[2];
    }
    f->area = vnorm(f->norm);
    f->ok = f->area != 0.0;
    if (!f->ok) {
        f->offset = 0.0;
        f->ax = 0;
        return;
    }
    f->area *= 0.5;
    f->offset = f->norm[0] * va[0] + f->norm[1] * va[1] + f->norm[2] * va[2];
    for (i = 1; i < f->nv; i++) {
        d1 = f->norm[0] * va[3 * i] + f->norm[1] * va[3 * i + 1] + f->norm[2] * va[3 * i + 2];
        f->offset += d1;
    }
    f->offset /= (double)f->nv;
    f->ax = fabs(f->norm[1]) > fabs(f->norm[0]);
    if (fabs(f->norm[2]) > fabs(f->norm[f->ax]))
        f->ax = 2;
}

static void ident4(double m[4][4])
{
    int i, j;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++)
            m[i][j] = i == j;
}

static void mult4(double r[4][4], double a[4][4], double b[4][4])
{
    double t[4][4];
    int i, j;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++)
            t[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j] + a[i][3] * b[3][j];
    memcpy(r, t, sizeof t);
}

/* common/cone.c:44-218 (getcone + conexform); may flip the object type as
 * the reference does for negative radii */
static int make_cone(gb_object *o, gb_cone *co)
{
    double *ca = o->farg, ad[3], m4[4][4], d;
    int sgn0, sgn1, i;
    co->ok = 0;
    if (o->otype == GT_CYLINDER || o->otype == GT_TUBE) {
        if (o->nfargs != 7)
            return fail("%s: bad # arguments", o->name);
        if (ca[6] < -GB_FTINY) {
            o->otype = o->otype == GT_CYLINDER ? GT_TUBE : GT_CYLINDER;
            ca[6] = -ca[6];
        } else if (ca[6] <= GB_FTINY)
            return 0;
        co->p0 = 0;
        co->p1 = 3;
        co->r0 = co->r1 = 6;
    } else {
        if (o->nfargs != 8)
            return fail("%s: bad # arguments", o->name);
        sgn0 = ca[6] < -GB_FTINY ? -1 : ca[6] > GB_FTINY;
        sgn1 = ca[7] < -GB_FTINY ? -1 : ca[7] > GB_FTINY;
        if (sgn0 + sgn1 == 0)
            return 0;
        if (sgn0 < 0 || sgn1 < 0) {
            if (o->otype == GT_RING)
                return 0;
            o->otype = o->otype == GT_CONE ? GT_CUP : GT_CONE;
        }
        ca[6] *= sgn0;
        ca[7] *= sgn1;
        if (ca[7] - ca[6] > GB_FTINY) {
            if (o->otype == GT_RING)
                co->p0 = co->p1 = 0;
            else {
                co->p0 = 0;
                co->p1 = 3;
            }
            co->r0 = 6;
            co->r1 = 7;
        } else if (ca[6] - ca[7] > GB_FTINY) {
            if (o->otype == GT_RING)
                co->p0 = co->p1 = 0;
            else {
                co->p0 = 3;
                co->p1 = 0;
            }
            co->r0 = 7;
            co->r1 = 6;
        } else {
            if (o->otype == GT_RING)
                return 0;
            o->otype = o->otype == GT_CONE ? GT_CYLINDER : GT_TUBE;
            o->nfargs = 7;
            co->p0 = 0;
            co->p1 = 3;
            co->r0 = co->r1 = 6;
        }
    }
    if (o->otype == GT_RING) {
        ad[0] = ca[3];
        ad[1] = ca[4];
        ad[2] = ca[5];
    } else
        for (i = 0; i < 3; i++)
            ad[i] = ca[co->p1 + i] - ca[co->p0 + i];
    co->al = vnorm(ad);
    if (co->al == 0.0)
        return 0;
    if (o->otype == GT_RING) {
        co->al = 0.0;
        co->sl = ca[co->r1] - ca[co->r0];
    } else if (o->otype == GT_CONE || o->otype == GT_CUP) {
        co->sl = ca[7] - ca[6];
        co->sl = sqrt(co->sl * co->sl + co->al * co->al);
    } else
        co->sl = co->al;
    /* conexform */
    ident4(co->tm);
    d = co->r0 == co->r1 ? 0.0 : ca[co->r0] / (ca[co->r1] - ca[co->r0]);
    for (i = 0; i < 3; i++)
        co->tm[3][i] = d * (ca[co->p1 + i] - ca[co->p0 + i]) - ca[co->p0 + i];
    ident4(m4);
    d = ad[1] * ad[1] + ad[2] * ad[2];
    if (d <= GB_FTINY * GB_FTINY) {
        m4[0][0] = 0.0;
        m4[0][2] = ad[0];
        m4[2][0] = -ad[0];
        m4[2][2] = 0.0;
    } else {
        d = sqrt(d);
        m4[0][0] = d;
        m4[1][0] = -ad[0] * ad[1] / d;
        m4[2][0] = -ad[0] * ad[2] / d;
        m4[1][1] = ad[2] / d;
        m4[2][1] = -ad[1] / d;
        m4[0][2] = ad[0];
        m4[1][2] = ad[1];
        m4[2][2] = ad[2];
    }
    mult4(co->tm, co->tm, m4);
    if (co->p0 != co->p1 && co->r0 != co->r1) {
        ident4(m4);
        m4[2][2] = (ca[co->r1] - ca[co->r0]) / co->al;
        mult4(co->tm, co->tm, m4);
    }
    co->ok = 1;
    return 0;
}

int gb_scene_prepare(gb_scene_host *S)
{
    int32_t i;
    if (S->prepared)
        return 0;
    S->faces = (gb_face *)calloc((size_t)S->nobjs + 1, sizeof(gb_face));
    S->cones = (gb_cone *)calloc((size_t)S->nobjs + 1, sizeof(gb_cone));
    if (!S->faces || !S->cones)
        return fail("out of memory");
    for (i = 0; i < S->nobjs; i++) {
        gb_object *o = &S->objs[i];
        switch (o->otype) {
        case GT_POLYGON:
            if (o->nfargs < 9 || o->nfargs % 3)
                return fail("%s: bad # arguments", o->name);
            make_face(o, &S->faces[i]);
            break;
        case GT_SPHERE:
        case GT_BUBBLE:
            if (o->nfargs != 4)
                return fail("%s: bad # arguments", o->name);
            if (o->farg[3] < -GB_FTINY) {
                o->otype = o->otype == GT_SPHERE ? GT_BUBBLE : GT_SPHERE;
                o->farg[3] = -o->farg[3];
            } else if (o->farg[3] <= GB_FTINY)
                return fail("%s: zero radius", o->name);
            break;
        case GT_CONE:
        case GT_CUP:
        case GT_CYLINDER:
        case GT_TUBE:
        case GT_RING:
            if (make_cone(o, &S->cones[i]) < 0)
                return -1;
            break;
        case GT_SOURCE:
            if (o->nfargs != 4)
                return fail("%s: bad # arguments", o->name);
            break;
        default:
            break;
        }
    }
    S->prepared = 1;
    return 0;
}

/* ------------------------------------------------------------- instances */

static void mat_ident(double m[4][4])
{
    int i, j;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++)
            m[i][j] = i == j;
}

static void mat_mul(double r[4][4], const double a[4][4], const double b[4][4])   /* r = a b */
{
    double t[4][4];
    int i, j;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++)
            t[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j] + a[i][3] * b[3][j];
    memcpy(r, t, sizeof t);
}

/* the arguments after option av[i] match fmt ('f' real, 'i' integer) */
static int xf_args_ok(int ac, char *const *av, int i, const char *fmt)
{
    int k;
    for (k = 0; fmt[k]; k++) {
        char *e;
        if (i + 1 + k >= ac)
            return 0;
        if (fmt[k] == 'i')
            (void)strtol(av[i + 1 + k], &e, 10);
        else
            (void)strtod(av[i + 1 + k], &e);
        if (e == av[i + 1 + k] || *e)
            return 0;
    }
    return 1;
}

/* common/xf.c xf (inverse = 0) and invxf (inverse = 1): transform options
 * -t x y z, -rx/-ry/-rz degrees, -s factor, -mx/-my/-mz, -i count; each
 * elementary transform multiplies on the right (forward) or on the left
 * (inverse, with the elementary inverse), -i repeats what precedes it.
 * Returns the number of arguments used. */
static int xf_parse(gb_xf *ret, int ac, char *const *av, int inverse)
{
    double xfmat[4][4], m4[4][4], xfsca = 1.0, d;
    int i, icnt = 1;
    mat_ident(ret->xfm);
    ret->sca = 1.0;
    mat_ident(xfmat);
    for (i = 0; i < ac && av[i][0] == '-'; i++) {
        const char *o = av[i] + 1;
        mat_ident(m4);
        if (o[0] == 't' && !o[1] && xf_args_ok(ac, av, i, "fff")) {
            int k;
            for (k = 0; k < 3; k++)
                m4[3][k] = (inverse ? -1.0 : 1.0) * atof(av[++i]);
        } else if (o[0] == 'r' && o[1] >= 'x' && o[1] <= 'z' && !o[2] && xf_args_ok(ac, av, i, "f")) {
            int a = (o[1] - 'x' + 1) % 3, b = (a + 1) % 3;     /* the rotation plane */
            d = (inverse ? -1.0 : 1.0) * (M_PI / 180.0) * atof(av[++i]);
            m4[a][a] = m4[b][b] = cos(d);
            m4[a][b] = sin(d);
            m4[b][a] = -m4[a][b];
        } else if (o[0] == 's' && !o[1] && xf_args_ok(ac, av, i, "f")) {
            d = atof(av[i + 1]);
            if (d == 0.0)
                break;
            i++;
            if (inverse)
                d = 1.0 / d;
            xfsca *= d;
            m4[0][0] = m4[1][1] = m4[2][2] = d;
        } else if (o[0] == 'm' && o[1] >= 'x' && o[1] <= 'z' && !o[2]) {
            int a = o[1] - 'x';
            xfsca *= -1.0;
            m4[a][a] = -1.0;
        } else if (o[0] == 'i' && !o[1] && xf_args_ok(ac, av, i, "i")) {
            while (icnt-- > 0) {
                if (inverse)
                    mat_mul(ret->xfm, xfmat, ret->xfm);
                else
                    mat_mul(ret->xfm, ret->xfm, xfmat);
                ret->sca *= xfsca;
            }
            icnt = atoi(av[++i]);
            mat_ident(xfmat);
            xfsca = 1.0;
            continue;
        } else
            break;
        if (inverse)
            mat_mul(xfmat, m4, xfmat);
        else
            mat_mul(xfmat, xfmat, m4);
    }
    while (icnt-- > 0) {
        if (inverse)
            mat_mul(ret->xfm, xfmat, ret->xfm);
        else
            mat_mul(ret->xfm, ret->xfm, xfmat);
        ret->sca *= xfsca;
    }
    return i;
}

int gb_fullxf(gb_xf *f, gb_xf *b, int ac, char *const *av)
{
    xf_parse(f, ac, av, 0);
    return xf_parse(b, ac, av, 1);
}

static int32_t remap_code(int32_t code, int32_t nodebase, int32_t setbase)
{
    if (code >= 0)
        return code + nodebase;
    if (code == -1)
        return -1;
    return -2 - ((-code - 2) + setbase);
}

/* append the objects, nodes and sets of T to S; returns the sub-scene
 * index or -1 */
static int merge_subscene(gb_scene_host *S, gb_scene_host *T, const char *name)
{
    int32_t objbase = S->nobjs, nodebase = S->nnodes, setbase = S->nsets, i;
    int k;
    gb_subscene *ns;
    for (i = 0; i < T->nobjs; i++) {
        gb_object *o = new_object(S);
        if (!o)
            return fail("out of memory loading \"%s\"", name);
        *o = T->objs[i];                       /* takes the strings and arguments */
        if (o->omod >= 0)
            o->omod += objbase;
    }
    T->nobjs = 0;
    for (i = 0; i < T->nnodes; i++) {
        int32_t nd = gb__new_node(S);
        if (nd < 0)
            return fail("out of memory loading \"%s\"", name);
        for (k = 0; k < 8; k++)
            S->kids[8 * nd + k] = remap_code(T->kids[8 * i + k], nodebase, setbase);
    }
    for (i = 0; i < T->nsets; i++) {
        const int32_t *st = T->set_data + T->set_off[i];
        int32_t *cp = (int32_t *)malloc(((size_t)st[0] + 1) * sizeof(int32_t));
        if (!cp)
            return fail("out of memory loading \"%s\"", name);
        cp[0] = st[0];
        for (k = 1; k <= st[0]; k++)
            cp[k] = st[k] + objbase;
        if (!gb__add_set(S, cp)) {
            free(cp);
            return fail("out of memory loading \"%s\"", name);
        }
        free(cp);
    }
    ns = (gb_subscene *)realloc(S->subs, (size_t)(S->nsubs + 1) * sizeof *ns);
    if (!ns)
        return fail("out of memory loading \"%s\"", name);
    S->subs = ns;
    ns = &S->subs[S->nsubs];
    ns->name = strdup(name);
    memcpy(ns->cuorg, T->cuorg, sizeof ns->cuorg);
    ns->cusize = T->cusize;
    ns->root = remap_code(T->root, nodebase, setbase);
    ns->firstobj = objbase;
    ns->nobjs = S->nobjs - objbase;
    return S->nsubs++;
}

/* ------------------------------------------------------------------ meshes */

/* One patch of a compiled mesh (common/readmesh.c:139-253 getpatch): up to
 * 256 vertices as 32-bit positions in the mesh's cube, local triangles,
 * triangles joining one or two vertices of other patches. */
typedef struct {
    uint32_t (*xyz)[3];
    int32_t *norm;               /* encoded vertex normals (0: none), or NULL */
    uint32_t (*uv)[2];           /* encoded vertex (u,v) (first 0: none), or NULL */
    int nverts, ntris, nj1, nj2;
    unsigned char (*tri)[3];
    int16_t *trimat, solemat;
    int32_t (*j1v)[2];           /* non-local vertex id; local vertices packed as v2 | v3 << 8 */
    int16_t *j1mat;
    int32_t (*j2v)[3];           /* two non-local vertex ids, local vertex */
    int16_t *j2mat;
} mpatch;

static void mpatch_free(mpatch *pp, int n)
{
    int i;
    for (i = 0; i < n; i++) {
        free(pp[i].xyz);
        free(pp[i].norm);
        free(pp[i].uv);
        free(pp[i].tri);
        free(pp[i].trimat);
        free(pp[i].j1v);
        free(pp[i].j1mat);
        free(pp[i].j2v);
        free(pp[i].j2mat);
    }
    free(pp);
}

static int read_patch(rdr *R, mpatch *pp, const char *path)
{
    int ok = 1, i, j;
    long flags = r_int(R, 1, &ok), n;
    if (!ok || !(flags & 1) || (flags & ~7L))
        return fail("(%s): bad patch flags", path);
    pp->nverts = (int)r_int(R, 2, &ok);
    if (!ok || pp->nverts <= 0 || pp->nverts > 256)
        return fail("(%s): bad number of patch vertices", path);
    pp->xyz = (uint32_t(*)[3])malloc((size_t)pp->nverts * sizeof *pp->xyz);
    if (!pp->xyz)
        return fail("out of memory");
    for (i = 0; i < pp->nverts; i++)
        for (j = 0; j < 3; j++)
            pp->xyz[i][j] = (uint32_t)r_int(R, 4, &ok);
    if (flags & 2) {                             /* vertex normals, 32-bit direction codes */
        pp->norm = (int32_t *)malloc((size_t)pp->nverts * sizeof(int32_t));
        if (!pp->norm)
            return fail("out of memory");
        for (i = 0; i < pp->nverts; i++)
            pp->norm[i] = (int32_t)r_int(R, 4, &ok);
    }
    if (flags & 4) {                             /* vertex (u,v), 32-bit codes in the mesh's limits */
        pp->uv = (uint32_t(*)[2])malloc((size_t)pp->nverts * sizeof *pp->uv);
        if (!pp->uv)
            return fail("out of memory");
        for (i = 0; i < pp->nverts; i++)
            for (j = 0; j < 2; j++)
                pp->uv[i][j] = (uint32_t)r_int(R, 4, &ok);
    }
    pp->ntris = (int)r_int(R, 2, &ok);
    if (!ok || pp->ntris < 0 || pp->ntris > 512)
        return fail("(%s): bad number of local triangles", path);
    pp->tri = (unsigned char(*)[3])malloc(((size_t)pp->ntris + 1) * sizeof *pp->tri);
    if (!pp->tri)
        return fail("out of memory");
    for (i = 0; i < pp->ntris; i++)
        for (j = 0; j < 3; j++)
            pp->tri[i][j] = (unsigned char)r_int(R, 1, &ok);
    n = r_int(R, 2, &ok);
    if (n > 1) {
        pp->trimat = (int16_t *)malloc(((size_t)pp->ntris + 1) * sizeof(int16_t));
        if (!pp->trimat)
            return fail("out of memory");
        for (i = 0; i < pp->ntris; i++)
            pp->trimat[i] = (int16_t)r_int(R, 2, &ok);
    } else
        pp->solemat = (int16_t)r_int(R, 2, &ok);
    pp->nj1 = (int)r_int(R, 2, &ok);
    if (!ok || pp->nj1 < 0 || pp->nj1 > 256)
        return fail("(%s): bad number of joiner triangles", path);
    pp->j1v = (int32_t(*)[2])malloc(((size_t)pp->nj1 + 1) * sizeof *pp->j1v);
    pp->j1mat = (int16_t *)malloc(((size_t)pp->nj1 + 1) * sizeof(int16_t));
    if (!pp->j1v || !pp->j1mat)
        return fail("out of memory");
    for (i = 0; i < pp->nj1; i++) {
        int v2, v3;
        pp->j1v[i][0] = (int32_t)r_int(R, 4, &ok);
        v2 = (int)r_int(R, 1, &ok) & 0xff;
        v3 = (int)r_int(R, 1, &ok) & 0xff;
        pp->j1v[i][1] = v2 | v3 << 8;
        pp->j1mat[i] = (int16_t)r_int(R, 2, &ok);
    }
    pp->nj2 = (int)r_int(R, 2, &ok);
    if (!ok || pp->nj2 < 0 || pp->nj2 > 256)
        return fail("(%s): bad number of double joiner triangles", path);
    pp->j2v = (int32_t(*)[3])malloc(((size_t)pp->nj2 + 1) * sizeof *pp->j2v);
    pp->j2mat = (int16_t *)malloc(((size_t)pp->nj2 + 1) * sizeof(int16_t));
    if (!pp->j2v || !pp->j2mat)
        return fail("out of memory");
    for (i = 0; i < pp->nj2; i++) {
        pp->j2v[i][0] = (int32_t)r_int(R, 4, &ok);
        pp->j2v[i][1] = (int32_t)r_int(R, 4, &ok);
        pp->j2v[i][2] = (int32_t)r_int(R, 1, &ok) & 0xff;
        pp->j2mat[i] = (int16_t)r_int(R, 2, &ok);
    }
    return ok ? 0 : fail("(%s): truncated mesh file", path);
}

/* A 32-bit direction code (common/dircode.c decodedir, the format
 * obj2mesh writes vertex normals in): bits 0-2 the signs of x, y and z;
 * two magnitudes of 13 bits at bits 5 and 18 in units of
 * 1 / ((2^13 - 1/2) sqrt 2); bit 3 set: the first is x, else y; bit 4 set:
 * the second is z, else the component the first is not (x or y); the
 * third component completes the unit length.  Code 0 is no normal. */
static void decode_dir(int32_t dc, double v[3])
{
    const double unit = 1. / 11584.5;
    double a, b, c;
    int first, second, third;
    if (!dc) {
        v[0] = v[1] = v[2] = 0.;
        return;
    }
    a = (dc >> 5 & 0x1fff) * unit;
    b = (dc >> 18 & 0x1fff) * unit;
    c = sqrt(1. - a * a - b * b);
    first = (dc & 010) ? 0 : 1;
    if (dc & 020) {
        second = 2;
        third = 1 - first;
    } else {
        second = 1 - first;
        third = 2;
    }
    v[first] = a;
    v[second] = b;
    v[third] = c;
    if (dc & 01)
        v[0] = -v[0];
    if (dc & 02)
        v[1] = -v[1];
    if (dc & 04)
        v[2] = -v[2];
}

/* vertex id -> its decoded normal; 0 when the vertex has none
 * (common/mesh.c:263-267) */
static int mesh_normal(const mpatch *pp, int npatches, int32_t vid, double *n)
{
    int pn = vid >> 8, k = vid & 0xff;
    if (vid < 0 || pn >= npatches || k >= pp[pn].nverts || !pp[pn].norm || !pp[pn].norm[k])
        return 0;
    decode_dir(pp[pn].norm[k], n);
    return 1;
}

/* vertex id -> its (u,v); 0 when the vertex has none (common/mesh.c:
 * 268-275: the codes' cells' centres within the mesh's (u,v) limits) */
static int mesh_uv(const mpatch *pp, int npatches, const double lim[2][2], int32_t vid, double *uv)
{
    int pn = vid >> 8, k = vid & 0xff, i;
    if (vid < 0 || pn >= npatches || k >= pp[pn].nverts || !pp[pn].uv || !pp[pn].uv[k][0])
        return 0;
    for (i = 0; i < 2; i++)
        uv[i] = lim[0][i] + (lim[1][i] - lim[0][i]) * (pp[pn].uv[k][i] + .5) * (1. / 4294967296.);
    return 1;
}

/* vertex id (patch << 8 | index) -> position (common/mesh.c:236-279
 * getmeshvert: the 32-bit cube coordinates at their cells' centres) */
static int mesh_vertex(const mpatch *pp, int npatches, const double org[3], double size, int32_t vid, double *v)
{
    int pn = vid >> 8, k;
    double res = size * (1. / 4294967296.);
    if (vid < 0 || pn >= npatches || (vid & 0xff) >= pp[pn].nverts)
        return 0;
    for (k = 0; k < 3; k++)
        v[k] = org[k] + (pp[pn].xyz[vid & 0xff][k] + .5) * res;
    return 1;
}

/* A compiled mesh file (common/readmesh.c:256-328 readmesh, format written
 * by ot/writemesh.c) as a sub-scene T: the mesh's cube and octree, its
 * materials, then each triangle as a three-vertex polygon whose modifier is
 * the triangle's material, named "M-Tri" as the pseudo object that stands
 * for the triangle in a hit on a mesh without its own modifier
 * (rt/o_mesh.c:186-190, common/mesh.c:281-300 getmeshpseudo).  Triangle ids in the octree's sets (patch << 10 |
 * local index, 0x200 joiners, 0x100 of those joining two patches:
 * common/mesh.c:174-233 getmeshtrivid) become the polygons' indices, in
 * the same order. */
static int read_mesh(gb_scene_host *T, const char *path, const char *mesh_name)
{
    size_t len = 0;
    char *buf = slurp(path, &len);
    rdr R;
    int ok = 1, objsize, i, k, np = 0;
    mpatch *pp = NULL;
    int32_t *map = NULL, nmats, ntri = 0, t;
    double uvlim[2][2] = {{0, 0}, {0, 0}};
    char line[256];
    int rc = -1;
    if (!buf)
        return fail("cannot open mesh file \"%s\"", path);
    R.p = (const unsigned char *)buf;
    R.end = R.p + len;
    for (;;) {                                   /* information header */
        size_t n = 0;
        while (R.p < R.end && *R.p != '\n') {
            if (n + 1 < sizeof line)
                line[n++] = (char)*R.p;
            R.p++;
        }
        if (R.p >= R.end) {
            fail("(%s): not a compiled mesh", path);
            goto done;
        }
        R.p++;
        line[n] = '\0';
        if (!n)
            break;
        if (!strncmp(line, "FORMAT=", 7) && strcmp(line + 7, "Radiance_tmesh")) {
            fail("(%s): not a compiled mesh", path);
            goto done;
        }
    }
    objsize = (int)(r_int(&R, 2, &ok) - (1 * 8 + 311));
    if (!ok || objsize <= 0 || objsize > 8) {
        fail("(%s): incompatible mesh format", path);
        goto done;
    }
    for (i = 0; i < 3; i++)
        T->cuorg[i] = atof(r_str(&R, &ok));
    T->cusize = atof(r_str(&R, &ok));
    for (i = 0; i < 2; i++) {                    /* (u,v) limits: u min, u max, v min, v max */
        uvlim[0][i] = r_flt(&R, &ok);
        uvlim[1][i] = r_flt(&R, &ok);
    }
    T->root = read_tree(T, &R, objsize, 0, &ok, 0);
    if (!ok) {
        fail("(%s): truncated or damaged mesh octree", path);
        goto done;
    }
    if (read_frozen(T, &R, objsize, 0) < 0)
        goto done;
    nmats = T->nobjs;
    np = (int)r_int(&R, 4, &ok);
    if (!ok || np < 0 || np > (1 << 21)) {
        fail("(%s): bad patch count", path);
        goto done;
    }
    pp = (mpatch *)calloc((size_t)np + 1, sizeof *pp);
    map = (int32_t *)malloc(((size_t)np + 1) * 1024 * sizeof(int32_t));
    if (!pp || !map) {
        fail("out of memory");
        goto done;
    }
    for (i = 0; i < np; i++)
        if (read_patch(&R, &pp[i], path) < 0)
            goto done;
    for (i = 0; i < np * 1024; i++)
        map[i] = -1;
    for (i = 0; i < np; i++) {
        for (t = 0; t < 1024; t++) {
            int32_t v[3], m;
            double xyz[9];
            gb_object *o;
            if (!(t & 0x200)) {                  /* local triangle */
                if (t >= pp[i].ntris)
                    continue;
                for (k = 0; k < 3; k++)
                    v[k] = i << 8 | pp[i].tri[t][k];
                m = pp[i].trimat ? pp[i].trimat[t] : pp[i].solemat;
            } else if (!(t & 0x100)) {           /* joins one other patch's vertex */
                int j = t & 0xff;
                if (j >= pp[i].nj1)
                    continue;
                v[0] = pp[i].j1v[j][0];
                v[1] = i << 8 | (pp[i].j1v[j][1] & 0xff);
                v[2] = i << 8 | (pp[i].j1v[j][1] >> 8);
                m = pp[i].j1mat[j];
            } else {                             /* joins two */
                int j = t & 0xff;
                if (j >= pp[i].nj2)
                    continue;
                v[0] = pp[i].j2v[j][0];
                v[1] = pp[i].j2v[j][1];
                v[2] = i << 8 | pp[i].j2v[j][2];
                m = pp[i].j2mat[j];
            }
            for (k = 0; k < 3; k++)
                if (!mesh_vertex(pp, np, T->cuorg, T->cusize, v[k], xyz + 3 * k)) {
                    fail("(%s): missing mesh vertex", path);
                    goto done;
                }
            if (m != -1 && (m < 0 || m >= nmats)) {
                fail("(%s): bad triangle material", path);
                goto done;
            }
            o = new_object(T);
            if (!o) {
                fail("out of memory");
                goto done;
            }
            o->otype = GT_POLYGON;
            o->omod = m;
            o->name = strdup(m >= 0 ? "M-Tri" : mesh_name);
            o->nsargs = 0;
            o->sarg = NULL;
            o->nfargs = 9;
            o->farg = (double *)malloc(9 * sizeof(double));
            if (!o->name || !o->farg) {
                fail("out of memory");
                goto done;
            }
            memcpy(o->farg, xyz, sizeof xyz);
            {                                    /* normals where all three vertices have one */
                double nv[9];
                if (mesh_normal(pp, np, v[0], nv) && mesh_normal(pp, np, v[1], nv + 3) &&
                    mesh_normal(pp, np, v[2], nv + 6)) {
                    o->vnorm = (double *)malloc(sizeof nv);
                    if (!o->vnorm) {
                        fail("out of memory");
                        goto done;
                    }
                    memcpy(o->vnorm, nv, sizeof nv);
                }
            }
            {                                    /* (u,v) where all three vertices have them */
                double uv[6];
                if (mesh_uv(pp, np, uvlim, v[0], uv) && mesh_uv(pp, np, uvlim, v[1], uv + 2) &&
                    mesh_uv(pp, np, uvlim, v[2], uv + 4)) {
                    o->vuv = (double *)malloc(sizeof uv);
                    if (!o->vuv) {
                        fail("out of memory");
                        goto done;
                    }
                    memcpy(o->vuv, uv, sizeof uv);
                }
            }
            map[i * 1024 + t] = ntri++;
        }
    }
    /* set members: triangle ids -> polygon objects (the map is increasing,
     * so the sets stay sorted) */
    for (i = 0; i < T->nsets; i++) {
        int32_t *st = T->set_data + T->set_off[i];
        for (k = 1; k <= st[0]; k++) {
            int32_t id = st[k];
            if (id < 0 || (id >> 10) >= np || map[id] < 0) {
                fail("(%s): octree names a missing triangle", path);
                goto done;
            }
            st[k] = nmats + map[id];
        }
    }
    rc = 0;
done:
    if (pp)
        mpatch_free(pp, np);
    free(map);
    free(buf);
    return rc;
}

int gb_scene_load_instances(gb_scene_host *S, const char *base_dir)
{
    int32_t i, ntop = S->nobjs;
    S->nobjs_top = ntop;
    for (i = 0; i < ntop; i++) {
        gb_object *o = &S->objs[i];
        gb_instance *ni;
        int sub = -1, k;
        /* a mesh (rt/o_mesh.c) is an instance of the sub-scene of its
         * triangles (read_mesh) */
        const int is_mesh = o->otype == GT_MESH;
        if (o->otype != GT_INSTANCE && !is_mesh)
            continue;
        if (o->nsargs < 1)
            return fail("%s: bad # of arguments", o->name);
        ni = (gb_instance *)realloc(S->inst, (size_t)(S->ninst + 1) * sizeof *ni);
        if (!ni)
            return fail("out of memory");
        S->inst = ni;
        ni = &S->inst[S->ninst];
        ni->obj = i;
        if (gb_fullxf(&ni->f, &ni->b, o->nsargs - 1, o->sarg + 1) != o->nsargs - 1)
            return fail("%s: bad transform", o->name);
        if (ni->f.sca < 0.0) {                 /* a mirror: common/instance.c:84-87 */
            ni->f.sca = -ni->f.sca;
            ni->b.sca = -ni->b.sca;
        }
        for (k = 0; k < S->nsubs; k++)
            if (!strcmp(S->subs[k].name, o->sarg[0]))
                sub = k;
        if (sub < 0) {
            gb_scene_host T;
            char *path = o->sarg[0];
            char *alt = NULL;
            FILE *fp = fopen(path, "rb");
            int32_t j;
            if (fp)
                fclose(fp);
            else if (path[0] != '/' && base_dir) {
                alt = (char *)malloc(strlen(base_dir) + strlen(path) + 2);
                sprintf(alt, "%s/%s", base_dir, path);
                path = alt;
            }
            gb_scene_init(&T);
            if ((is_mesh ? read_mesh(&T, path, S->objs[i].name) : gb_scene_read_oct(&T, path)) < 0) {
                char why[256];
                snprintf(why, sizeof why, "%s", gb_scene_error());
                free(alt);
                gb_scene_clear(&T);
                return fail("%s: cannot load %s \"%s\": %s", S->objs[i].name, is_mesh ? "mesh" : "octree",
                            S->objs[i].sarg[0], why);
            }
            free(alt);
            for (j = 0; j < T.nobjs; j++)
                if (gb_is_volume(T.objs[j].otype)) {
                    gb_scene_clear(&T);
                    return fail("%s: instances inside an instanced octree are not supported", S->objs[i].name);
                }
            sub = merge_subscene(S, &T, S->objs[i].sarg[0]);
            gb_scene_clear(&T);
            if (sub < 0)
                return -1;
        }
        S->inst[S->ninst].sub = sub;
        S->ninst++;
    }
    return 0;
}
