/* CPU oracle: parser, camera and light restated from the reference in plain C.
 * TEST INFRASTRUCTURE ONLY -- see csg_oracle.h.  Compiled with -ffp-contract=off so
 * that every `a*b + c` below is two IEEE roundings on every host (x86-64 and aarch64).
 *
 * The render core (traversal, intersections, shading) is in csg_oracle_render.inc,
 * included twice: once with separately rounded operations ("ieee") and once with the
 * fused multiply-adds of nvcc's default contraction ("fma"). */
#include "csg_oracle.h"

#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------
 * Parser: CSGTree::Parse (CSGTree.cu:5-152), split (CSGTree.cu:181-194),
 * color (CSGTree.cu:196-200), Primitive constructors (Primitives.h:42-102),
 * BVHNode (BVHNode.cuh:17-76) and ConstructBVH (CSGTree.cu:154-179).
 * ---------------------------------------------------------------------------------- */

typedef struct { const char* s; size_t n; } tok_t;

/* std::stringstream >> std::string splits on the C-locale isspace set. */
static int orc_is_space(char c)
{
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

static void set_err(char* err, size_t errlen, const char* a, const tok_t* tk)
{
    if (!err || !errlen) return;
    if (tk) {
        size_t la = strlen(a);
        size_t n = tk->n;
        if (la >= errlen) la = errlen - 1;
        memcpy(err, a, la);
        if (la + n >= errlen) n = errlen - 1 - la;
        memcpy(err + la, tk->s, n);
        err[la + n] = 0;
    } else {
        snprintf(err, errlen, "%s", a);
    }
}

/* std::stof / std::stod / std::stoi: strto* with "no conversion" -> invalid_argument
 * (what() = "stof"/"stod"/"stoi") and ERANGE (or int overflow) -> out_of_range. */
static int parse_f32(const tok_t* tk, float* out, char* err, size_t errlen)
{
    char buf[512];
    char* heap = NULL;
    char* s = buf;
    if (tk->n >= sizeof(buf)) { heap = (char*)malloc(tk->n + 1); s = heap; }
    memcpy(s, tk->s, tk->n);
    s[tk->n] = 0;
    char* end = NULL;
    int saved = errno;
    errno = 0;
    float v = strtof(s, &end);
    int e = errno;
    errno = saved;
    int rc = ORC_OK;
    if (end == s) { set_err(err, errlen, "stof", NULL); rc = ORC_E_PARSE; }
    else if (e == ERANGE) { set_err(err, errlen, "stof", NULL); rc = ORC_E_RANGE; }
    free(heap);
    *out = v;
    return rc;
}

static int parse_f64(const tok_t* tk, double* out, char* err, size_t errlen)
{
    char buf[512];
    char* heap = NULL;
    char* s = buf;
    if (tk->n >= sizeof(buf)) { heap = (char*)malloc(tk->n + 1); s = heap; }
    memcpy(s, tk->s, tk->n);
    s[tk->n] = 0;
    char* end = NULL;
    int saved = errno;
    errno = 0;
    double v = strtod(s, &end);
    int e = errno;
    errno = saved;
    int rc = ORC_OK;
    if (end == s) { set_err(err, errlen, "stod", NULL); rc = ORC_E_PARSE; }
    else if (e == ERANGE) { set_err(err, errlen, "stod", NULL); rc = ORC_E_RANGE; }
    free(heap);
    *out = v;
    return rc;
}

/* color(): std::stoi(hex, nullptr, 16) / 255 on a two-character substring. */
static int parse_color2(const char* two, float* out, char* err, size_t errlen)
{
    char s[3] = {two[0], two[1], 0};
    char* end = NULL;
    int saved = errno;
    errno = 0;
    long v = strtol(s, &end, 16);
    int e = errno;
    errno = saved;
    if (end == s) { set_err(err, errlen, "stoi", NULL); return ORC_E_PARSE; }
    if (e == ERANGE || v < -2147483647L - 1 || v > 2147483647L) {
        set_err(err, errlen, "stoi", NULL);
        return ORC_E_RANGE;
    }
    *out = (float)(int)v / 255;
    return ORC_OK;
}

static int tok_eq(const tok_t* t, const char* s)
{
    size_t n = strlen(s);
    return t->n == n && memcmp(t->s, s, n) == 0;
}

/* BVHNode(Primitive, type): sphere box is centre +- 2r computed as (x - r) - r;
 * cylinder box is centre +- max(h/2, r) (not conservative for a tilted cylinder);
 * cube box is centre +- edge/2.  BVHNode.cuh:17-52. */
static void leaf_box(orc_node* n, const orc_prim* p)
{
    float lo[3], hi[3];
    const float c[3] = {p->x, p->y, p->z};
    if (n->type == ORC_SPHERE) {
        float r = p->p[0];
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - r - r; hi[k] = c[k] + r + r; }
    } else if (n->type == ORC_CYLINDER) {
        float h2 = p->p[1] / 2;
        float r = p->p[0];
        float m = (h2 < r) ? r : h2; /* std::max(h/2, r) */
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - m; hi[k] = c[k] + m; }
    } else if (n->type == ORC_CUBE) {
        float hs = p->p[0] / 2;
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - hs; hi[k] = c[k] + hs; }
    } else {
        for (int k = 0; k < 3; ++k) { lo[k] = 0.f; hi[k] = 0.f; }
    }
    n->minx = lo[0]; n->miny = lo[1]; n->minz = lo[2];
    n->maxx = hi[0]; n->maxy = hi[1]; n->maxz = hi[2];
}

/* Exact-box mode of the engine (csg_scene_create_ex with CSG_SCENE_EXACT_BOXES; no
 * counterpart in the reference): a sphere gets +-r, a cylinder about axis V with
 * half-height h/2 gets |V_k| h/2 + r sqrt(1 - V_k^2) per axis, both widened by 2^-12 of
 * their size plus 1e-5; cubes keep the reference box.  Same float operations, in the same
 * order, as the engine's scene compiler. */
static void leaf_box_exact(orc_node* n, const orc_prim* p)
{
    if (n->type != ORC_SPHERE && n->type != ORC_CYLINDER) {
        leaf_box(n, p);
        return;
    }
    const float c[3] = {p->x, p->y, p->z};
    float e[3];
    if (n->type == ORC_SPHERE) {
        for (int k = 0; k < 3; ++k) e[k] = p->p[0];
    } else {
        const float r = p->p[0], h2 = p->p[1] * 0.5f;
        for (int k = 0; k < 3; ++k) {
            const float v = p->p[2 + k];
            const float s = 1.0f - v * v;
            e[k] = fabsf(v) * h2 + r * sqrtf(s > 0.0f ? s : 0.0f);
        }
    }
    for (int k = 0; k < 3; ++k) e[k] = e[k] + e[k] * 0.000244140625f + 1e-5f;
    n->minx = c[0] - e[0]; n->miny = c[1] - e[1]; n->minz = c[2] - e[2];
    n->maxx = c[0] + e[0]; n->maxy = c[1] + e[1]; n->maxz = c[2] + e[2];
}

static void merge_box(orc_node* n, const orc_node* l, const orc_node* r);

void orc_boxes_exact(orc_node* nodes, int n_nodes, const orc_prim* prims)
{
    /* nodes are in preorder: a reverse sweep meets every child before its parent */
    for (int i = n_nodes - 1; i >= 0; --i) {
        if (nodes[i].prim != -1) leaf_box_exact(&nodes[i], &prims[nodes[i].prim]);
        else merge_box(&nodes[i], &nodes[nodes[i].left], &nodes[nodes[i].right]);
    }
}

/* std::min / std::max as the reference uses them (BVHNode.cuh:54-63):
 * min(a,b) = (b < a) ? b : a, max(a,b) = (a < b) ? b : a. */
static float smin(float a, float b) { return (b < a) ? b : a; }
static float smax(float a, float b) { return (a < b) ? b : a; }

static void merge_box(orc_node* n, const orc_node* l, const orc_node* r)
{
    n->minx = smin(l->minx, r->minx); n->miny = smin(l->miny, r->miny); n->minz = smin(l->minz, r->minz);
    n->maxx = smax(l->maxx, r->maxx); n->maxy = smax(l->maxy, r->maxy); n->maxz = smax(l->maxz, r->maxz);
}

/* ConstructBVH (CSGTree.cu:154-179): post-order, leaves from their primitive, operators
 * from the union of their children's boxes.  Iterative with an explicit stack. */
static void construct_bvh(orc_node* nodes, int n_nodes, const orc_prim* prims)
{
    int* stack = (int*)malloc(sizeof(int) * (size_t)(n_nodes + 1) * 2);
    unsigned char* visited = (unsigned char*)calloc((size_t)n_nodes, 1);
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        int id = stack[sp - 1];
        if (visited[id]) {
            --sp;
            merge_box(&nodes[id], &nodes[nodes[id].left], &nodes[nodes[id].right]);
        } else if (nodes[id].prim != -1) {
            --sp;
            leaf_box(&nodes[id], &prims[nodes[id].prim]);
        } else {
            stack[sp++] = nodes[id].left;
            stack[sp++] = nodes[id].right;
            visited[id] = 1;
        }
    }
    free(stack);
    free(visited);
}

/* Primitive cylinder constructor (Primitives.h:54-88): the axis is R * (0,1,0) from
 * Euler angles in double, divided by its SQUARED length, stored as float. */
static void cylinder_axis(double rotX, double rotY, double rotZ, float out[3])
{
    rotX = rotX * 0.017453292519943295769236907684886;
    rotY = rotY * 0.017453292519943295769236907684886;
    rotZ = rotZ * 0.017453292519943295769236907684886;
    double ax = -sin(rotZ) * cos(rotY) + sin(rotY) * sin(rotX) * cos(rotZ);
    double ay = cos(rotX) * cos(rotZ);
    double az = sin(rotY) * sin(rotZ) + sin(rotX) * cos(rotY) * cos(rotZ);
    double len = (ax * ax + ay * ay + az * az);
    ax /= len;
    ay /= len;
    az /= len;
    out[0] = (float)ax;
    out[1] = (float)ay;
    out[2] = (float)az;
}

int orc_parse(const char* text, size_t len, orc_node* nodes, int max_nodes,
              orc_prim* prims, int max_prims, int* n_nodes_out, int* n_prims_out,
              char* err, size_t errlen)
{
    if (err && errlen) err[0] = 0;
    *n_nodes_out = 0;
    *n_prims_out = 0;
    /* split */
    size_t cap = 64, ntok = 0;
    tok_t* toks = (tok_t*)malloc(cap * sizeof(tok_t));
    for (size_t i = 0; i < len;) {
        while (i < len && orc_is_space(text[i])) ++i;
        if (i >= len) break;
        size_t j = i;
        while (j < len && !orc_is_space(text[j])) ++j;
        if (ntok == cap) { cap *= 2; toks = (tok_t*)realloc(toks, cap * sizeof(tok_t)); }
        toks[ntok].s = text + i;
        toks[ntok].n = j - i;
        ++ntok;
        i = j;
    }
    /* (node index, children seen) stack */
    int* st_node = (int*)malloc(sizeof(int) * (ntok + 1));
    int* st_cnt = (int*)malloc(sizeof(int) * (ntok + 1));
    int sp = 0;
    int nprim = 0, nnode = 0;
    int rc = ORC_OK;
    for (size_t i = 0; i < ntok; ++i) {
        if (nnode >= max_nodes) { rc = ORC_E_CAPACITY; set_err(err, errlen, "too many nodes", NULL); break; }
        orc_node* nd = &nodes[nnode];
        nd->type = -1; nd->prim = -1; nd->left = -1; nd->right = -1; nd->parent = -1;
        nd->minx = nd->miny = nd->minz = nd->maxx = nd->maxy = nd->maxz = 0.f;
        if (nnode != 0) {
            if (sp == 0) { rc = ORC_E_PARSE; set_err(err, errlen, "Cannot parse", NULL); break; }
            if (st_cnt[sp - 1] == 0) {
                nodes[st_node[sp - 1]].left = nnode;
                nd->parent = st_node[sp - 1];
                st_cnt[sp - 1]++;
            } else {
                nodes[st_node[sp - 1]].right = nnode;
                nd->parent = st_node[sp - 1];
                --sp;
            }
        }
        const tok_t* tk = &toks[i];
        int kind = -1, nparams = 0;
        if (tok_eq(tk, "Union")) kind = ORC_UNION;
        else if (tok_eq(tk, "Difference")) kind = ORC_DIFFERENCE;
        else if (tok_eq(tk, "Intersection")) kind = ORC_INTERSECTION;
        else if (tok_eq(tk, "Sphere")) { kind = ORC_SPHERE; nparams = 5; }
        else if (tok_eq(tk, "Cylinder")) { kind = ORC_CYLINDER; nparams = 9; }
        else if (tok_eq(tk, "Cube")) { kind = ORC_CUBE; nparams = 5; }
        else {
            rc = ORC_E_PARSE;
            set_err(err, errlen, "Cannot parse - Unrecognized keyword: ", tk);
            break;
        }
        nd->type = kind;
        if (kind <= ORC_INTERSECTION) {
            st_node[sp] = nnode;
            st_cnt[sp] = 0;
            ++sp;
            ++nnode;
            continue;
        }
        if (nprim >= max_prims) { rc = ORC_E_CAPACITY; set_err(err, errlen, "too many primitives", NULL); break; }
        nd->prim = nprim;
        /* Parameters are consumed in the reference's order: x y z, colour length check,
         * colour channels, then size parameters.  A token past the end of the text is
         * undefined behaviour in the reference (an unchecked vector index); here it is
         * reported as a parse error. */
        float v[3];
        orc_prim* p = &prims[nprim];
        memset(p, 0, sizeof(*p));
        p->id = nprim;
#define NEED(k) do { if (i + (k) >= ntok) { rc = ORC_E_PARSE; \
            set_err(err, errlen, "Cannot parse - missing parameters after ", tk); goto done; } } while (0)
        for (int k = 0; k < 3; ++k) {
            NEED(k + 1);
            if ((rc = parse_f32(&toks[i + 1 + k], &v[k], err, errlen)) != ORC_OK) goto done;
        }
        NEED(4);
        if (toks[i + 4].n != 6) {
            rc = ORC_E_PARSE;
            set_err(err, errlen, "Cannot parse color ", &toks[i + 4]);
            goto done;
        }
        {
            float col[3];
            for (int k = 0; k < 3; ++k)
                if ((rc = parse_color2(toks[i + 4].s + 2 * k, &col[k], err, errlen)) != ORC_OK) goto done;
            p->x = v[0]; p->y = v[1]; p->z = v[2];
            p->r = col[0]; p->g = col[1]; p->b = col[2];
        }
        if (kind == ORC_SPHERE || kind == ORC_CUBE) {
            NEED(5);
            if ((rc = parse_f32(&toks[i + 5], &p->p[0], err, errlen)) != ORC_OK) goto done;
        } else {
            double rot[3];
            NEED(5);
            if ((rc = parse_f32(&toks[i + 5], &p->p[0], err, errlen)) != ORC_OK) goto done;
            NEED(6);
            if ((rc = parse_f32(&toks[i + 6], &p->p[1], err, errlen)) != ORC_OK) goto done;
            for (int k = 0; k < 3; ++k) {
                NEED(7 + k);
                if ((rc = parse_f64(&toks[i + 7 + k], &rot[k], err, errlen)) != ORC_OK) goto done;
            }
            static const char* names[3] = {
                "Invalid roation rotX should be in range [0, 360] deg",
                "Invalid roation rotY should be in range [0, 360] deg",
                "Invalid roation rotZ should be in range [0, 360] deg"};
            for (int k = 0; k < 3; ++k)
                if (rot[k] > 360 || rot[k] < 0) {
                    rc = ORC_E_RANGE;
                    set_err(err, errlen, names[k], NULL);
                    goto done;
                }
            cylinder_axis(rot[0], rot[1], rot[2], &p->p[2]);
        }
#undef NEED
        i += (size_t)nparams;
        ++nprim;
        ++nnode;
    }
done:
    if (rc == ORC_OK && nnode != 2 * nprim - 1) {
        rc = ORC_E_COUNT;
        set_err(err, errlen, "Cannot parse - number of primitives do not match number of nodes", NULL);
    }
    if (rc == ORC_OK) construct_bvh(nodes, nnode, prims);
    free(st_node);
    free(st_cnt);
    free(toks);
    *n_nodes_out = nnode;
    *n_prims_out = nprim;
    return rc;
}

/* ------------------------------------------------------------------------------------
 * Camera (Camera.h:9-52, Camera.cpp:4-36) and DirectionalLight (DirectionalLight.h:8-18).
 * Layout: x y z rotX rotY fov forward[3] right[3] up[3].
 * ---------------------------------------------------------------------------------- */
enum { CX = 0, CY = 1, CZ = 2, CROTX = 3, CROTY = 4, CFOV = 5, CF = 6, CR = 9, CU = 12 };

static void normalize_vec(float* v)
{
    float length = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (length > 0) {
        v[0] /= length;
        v[1] /= length;
        v[2] /= length;
    }
}

/* Camera.cpp includes only <cmath>: its unqualified sin/cos on float arguments are the
 * global double functions, so each component is a double expression rounded to float. */
static void update_vectors(float* c)
{
    float* f = c + CF;
    float* r = c + CR;
    float* u = c + CU;
    const double px = c[CROTX], yw = c[CROTY];
    f[0] = (float)(-sin(yw) * cos(px));
    f[1] = (float)sin(px);
    f[2] = (float)(-cos(yw) * cos(px));
    normalize_vec(f);
    r[0] = (float)cos(yw);
    r[1] = 0;
    r[2] = (float)(-sin(yw));
    normalize_vec(r);
    u[0] = f[1] * r[2] - f[2] * r[1];
    u[1] = f[2] * r[0] - f[0] * r[2];
    u[2] = f[0] * r[1] - f[1] * r[0];
    normalize_vec(u);
}

void orc_camera_default(float cam[15])
{
    cam[CX] = 0; cam[CY] = 0; cam[CZ] = 5;
    cam[CROTX] = 0; cam[CROTY] = 0;
    cam[CFOV] = 90.0f * 3.14159f / 180.0f;
    update_vectors(cam);
}

void orc_camera_set_position(float cam[15], float x, float y, float z)
{
    cam[CX] = x; cam[CY] = y; cam[CZ] = z;
}

void orc_camera_set_rotation(float cam[15], float pitch, float yaw)
{
    cam[CROTX] = fmaxf(-89.0f * 3.14159f / 180.0f, fminf(89.0f * 3.14159f / 180.0f, pitch));
    cam[CROTY] = yaw;
    update_vectors(cam);
}

void orc_camera_set_fov(float cam[15], float degrees)
{
    cam[CFOV] = degrees * 3.14159f / 180.0f;
}

void orc_camera_move(float cam[15], float fwd, float right, float up)
{
    cam[CX] += cam[CF + 0] * fwd + cam[CR + 0] * right;
    cam[CY] += cam[CF + 1] * fwd + cam[CR + 1] * right + up;
    cam[CZ] += cam[CF + 2] * fwd + cam[CR + 2] * right;
}

void orc_camera_rotate(float cam[15], float dpitch, float dyaw)
{
    orc_camera_set_rotation(cam, cam[CROTX] + dpitch, cam[CROTY] + dyaw);
}

void orc_light_dir(float polar, float azimuth, float out[3])
{
    out[0] = sinf(polar) * cosf(azimuth);
    out[1] = cosf(polar);
    out[2] = sinf(polar) * sinf(azimuth);
}

void orc_light_default(float out[3])
{
    orc_light_dir(-60.f * 3.14159f / 180.f, -45.f * 3.14159f / 180.f, out);
}

float orc_tan_half_fov(float fov)
{
    return tanf(fov / 2.0f);
}

/* ------------------------------------------------------------------------------------
 * Render core, three arithmetic modes.
 * ---------------------------------------------------------------------------------- */
/* FP32 operations of the reference source on the path a ray executes: every +, -, *,
 * /, sqrt, min, max, pow, tan counts 1 (as written in the reference, so a*b+c is 2);
 * comparisons, negations, conversions 0.  Per OpenMP thread. */
static __thread uint64_t orc_flop_counter;
#define ORC_FL(n) (orc_flop_counter += (uint64_t)(n))

/* Optional operator short-circuit (not the reference's algorithm; off by default): a
 * Difference whose left child, or an Intersection with a child, is a Miss already known at
 * GoTo, and a Difference / Intersection whose left subtree returned a Miss, go straight to
 * Compute without traversing the other child -- the engine's rule for trees whose stacks
 * cannot overflow.  The tests render with and without it and compare every plane, a check
 * of that rule independent of the GPU. */
static int orc_short_circuit;
void orc_set_short_circuit(int on) { orc_short_circuit = on ? 1 : 0; }

/* Optional live-leaf pruning (not the reference's algorithm; off by default): the
 * engine's rule, restated so that the tests can check it against the reference's
 * traversal on the CPU.  Each ray starts with a mask over leaf groups (one bit per
 * 2^shift leaves in preorder, at most ORC_LIVE_GROUPS groups) holding the leaves whose
 * own box passes at tmin = 0 and whose primitive test at tmin = 0 is not a Miss (a cube:
 * its box alone); trees of fewer than ORC_LIVE_MIN_PRIMS primitives start all live, as
 * the engine runs no pre-pass for them (a root leaf is tested without its box, and a
 * cylinder's box does not contain the cylinder).  GoTo treats a child without a live leaf as a Miss without testing it;
 * a culled operator child clears the groups inside its leaf range and a leaf that returns
 * Miss its own bit (single-leaf groups only), and each region of orc_live_region groups
 * records the largest tmin at which one of its live groups was cleared; a loop re-enables
 * the looped child's groups in the regions whose record is above its new tmin.  Mode 4
 * is the engine's rule (its regions are four 32-bit mask words, ORC_LIVE_REGION groups):
 * on trees of at most 15 operator levels, whose stacks cannot overflow, as stated here, and
 * on deeper ones, whose 32-entry stacks can drop pushes, under the guard below.  Mode 1 is the engine's earlier rule,
 * one record per ray raised by every clear, which re-enables whole subtrees that held no
 * stale group; modes 5 and 6 are modes 1 and 4 re-enabling only groups that were live at
 * tmin = 0.  Two unsound variants are kept so that tests can show what the rule's parts
 * prevent: mode 2 leaves out the loop restore, mode 3 prunes trees of any depth without
 * the guard below.
 * Trees deeper than 15 operator levels: mode 4 prunes them too, under a guard
 * (orc_guard_deep, which also covers the operator short-circuit): a skip is taken only
 * while no push of the ray has been dropped and only where the skipped traversal could
 * not drop one (under an operator of height h it adds at most 2h actions and h entries to
 * each of the other stacks, so the action depth plus 2h and the other depths plus h must
 * stay within 32).  Before the first dropped push the traversal's state is the one an
 * unbounded stack would hold, where every skip is exact; from the first one on nothing is
 * skipped, so the rest is the reference's own traversal.  Modes 1, 2, 5 and 6 leave such
 * trees unpruned.  Process-wide. */
#define ORC_LIVE_GROUPS 1024
#define ORC_LIVE_MIN_PRIMS 2
static int orc_live_mode;
static int* orc_live_lo;
static int* orc_live_hi;
static int orc_live_cap, orc_live_shift, orc_live_nodes, orc_live_prims, orc_live_active;
void orc_set_live_pruning(int mode) { orc_live_mode = (mode >= 1 && mode <= 6) ? mode : 0; }
static int* orc_height; /* per node: operator height (0 for a leaf) */
static int orc_height_cap, orc_guard_deep;

/* Operator heights of every node and the tree's operator depth (operators on the longest
 * root-to-leaf path); sets orc_guard_deep for trees deeper than 15 levels. */
static int orc_height_prepare(const orc_node* nodes, int n_nodes)
{
    if (n_nodes > orc_height_cap) {
        int* h = (int*)realloc(orc_height, sizeof(int) * (size_t)n_nodes);
        if (!h) return -1;
        orc_height = h;
        orc_height_cap = n_nodes;
    }
    for (int i = n_nodes - 1; i >= 0; --i) {
        if (nodes[i].prim != -1) {
            orc_height[i] = 0;
        } else {
            const int a = orc_height[nodes[i].left], b = orc_height[nodes[i].right];
            orc_height[i] = 1 + (a > b ? a : b);
        }
    }
    const int depth = n_nodes > 0 ? orc_height[0] : 0;
    orc_guard_deep = depth > 15 && orc_live_mode != 3;
    return depth;
}

/* Leaf ranges (first and last primitive in preorder) of every node, and the group
 * shift, for the tree about to be rendered. */
static int orc_live_prepare(const orc_node* nodes, int n_nodes, int n_prims)
{
    orc_live_active = 0;
    const int depth = orc_height_prepare(nodes, n_nodes);
    if (depth < 0) return -1;
    if (!orc_live_mode) return 0;
    if (n_nodes > orc_live_cap) {
        int* lo = (int*)realloc(orc_live_lo, sizeof(int) * (size_t)n_nodes);
        if (!lo) return -1;
        orc_live_lo = lo;
        int* hi = (int*)realloc(orc_live_hi, sizeof(int) * (size_t)n_nodes);
        if (!hi) return -1;
        orc_live_hi = hi;
        orc_live_cap = n_nodes;
    }
    /* (min and max over both children: a tree whose operators' children were swapped, as
     * the engine may do for Intersections, keeps every subtree's leaves contiguous) */
    for (int i = n_nodes - 1; i >= 0; --i) {
        if (nodes[i].prim != -1) {
            orc_live_lo[i] = orc_live_hi[i] = nodes[i].prim;
        } else {
            const int a = nodes[i].left, b = nodes[i].right;
            orc_live_lo[i] = orc_live_lo[a] < orc_live_lo[b] ? orc_live_lo[a] : orc_live_lo[b];
            orc_live_hi[i] = orc_live_hi[a] > orc_live_hi[b] ? orc_live_hi[a] : orc_live_hi[b];
        }
    }
    int sh = 0;
    while (((n_prims + (1 << sh) - 1) >> sh) > ORC_LIVE_GROUPS) ++sh;
    orc_live_shift = sh;
    orc_live_nodes = n_nodes;
    orc_live_prims = n_prims;
    orc_live_active = (orc_live_mode == 3) || (orc_live_mode == 4) || depth <= 15;
    return 0;
}

/* Single-leaf shortcut (a candidate engine rule, with live-leaf pruning, off by default):
 * an operator subtree of at most orc_shortcut_max leaves, one bit per leaf, with exactly
 * one live leaf l evaluates without descending.  Every other leaf of it is a Miss, and
 * by Kensler's tables (RaycastingKernels.cu:666-677) a Union with a Miss child returns
 * the other child's record, a Difference returns its left child's record when the right
 * one is a Miss and Miss when the left one is, and an Intersection with a Miss child
 * returns Miss (a Miss's t and index reach no decision).  So the subtree's result is l's
 * own result (tested with its box, which every box on the path contains) when every
 * operator on the path down to l is a Union or a Difference entered on its left, and a
 * Miss otherwise.  orc_blk[l] is the depth of the deepest operator above l entered
 * otherwise (-1: none), and the path below a node of depth d is transparent when
 * orc_blk[l] < d.  Mode 1 of orc_set_union_shortcut allows only all-Union subtrees. */
static int orc_shortcut_max, orc_shortcut_general;
static int* orc_uonly;     /* per node: every operator of its subtree is a Union */
static int* orc_depth;     /* per node: operators above it */
static int* orc_leaf_node; /* per primitive: its node */
static int* orc_blk;       /* per primitive: see above */
static int orc_uonly_cap, orc_leaf_cap;
void orc_set_union_shortcut(int max_leaves) { orc_shortcut_max = max_leaves > 0 ? max_leaves : 0; orc_shortcut_general = 0; }
void orc_set_leaf_shortcut(int max_leaves) { orc_shortcut_max = max_leaves > 0 ? max_leaves : 0; orc_shortcut_general = 1; }
static int orc_shortcut_prepare(const orc_node* nodes, int n_nodes, int n_prims)
{
    if (n_nodes > orc_uonly_cap) {
        int* u = (int*)realloc(orc_uonly, sizeof(int) * (size_t)n_nodes);
        if (!u) return -1;
        orc_uonly = u;
        int* d = (int*)realloc(orc_depth, sizeof(int) * (size_t)n_nodes);
        if (!d) return -1;
        orc_depth = d;
        orc_uonly_cap = n_nodes;
    }
    if (n_prims > orc_leaf_cap) {
        int* l = (int*)realloc(orc_leaf_node, sizeof(int) * (size_t)n_prims);
        if (!l) return -1;
        orc_leaf_node = l;
        int* b = (int*)realloc(orc_blk, sizeof(int) * (size_t)n_prims);
        if (!b) return -1;
        orc_blk = b;
        orc_leaf_cap = n_prims;
    }
    for (int i = n_nodes - 1; i >= 0; --i) {
        if (nodes[i].prim != -1) {
            orc_uonly[i] = 1;
            if (nodes[i].prim >= 0 && nodes[i].prim < n_prims) orc_leaf_node[nodes[i].prim] = i;
        } else {
            orc_uonly[i] = nodes[i].type == ORC_UNION && orc_uonly[nodes[i].left] && orc_uonly[nodes[i].right];
        }
    }
    for (int i = 0; i < n_nodes; ++i) orc_depth[i] = nodes[i].parent >= 0 ? orc_depth[nodes[i].parent] + 1 : 0;
    for (int p = 0; p < n_prims; ++p) {
        int blk = -1;
        for (int c = orc_leaf_node[p], a = nodes[c].parent; a >= 0; c = a, a = nodes[a].parent) {
            const int transparent = nodes[a].type == ORC_UNION || (nodes[a].type == ORC_DIFFERENCE && nodes[a].left == c);
            if (!transparent) { blk = orc_depth[a]; break; }
        }
        orc_blk[p] = blk;
    }
    return 0;
}

#define ORC_LIVE_REGION 128 /* groups per region: four 32-bit mask words */
static int orc_live_region = ORC_LIVE_REGION; /* groups per restore record (modes 4 and 6) */
void orc_set_live_region(int groups) { orc_live_region = (groups >= 1 && groups <= ORC_LIVE_GROUPS) ? groups : ORC_LIVE_REGION; }
typedef struct {
    uint64_t w[ORC_LIVE_GROUPS / 64];
    uint64_t p[ORC_LIVE_GROUPS / 64];          /* the mask at tmin = 0 (modes 5 and 6) */
    double tclr;                               /* largest tmin of a traversal clear */
    double treg[ORC_LIVE_GROUPS];              /* the same per region (modes 4 and 6) */
} orc_live;
static int orc_live_any(const orc_live* m, int lo, int hi)
{
    for (int g = lo >> orc_live_shift; g <= (hi >> orc_live_shift); ++g)
        if ((m->w[g >> 6] >> (g & 63)) & 1u) return 1;
    return 0;
}
/* The single-leaf shortcut for operator `node` with leaves [lo, hi]: -1 when it does not
 * apply; else the node of the subtree's one live leaf, with *miss set when the path down
 * to it is not transparent (the subtree is then a Miss). */
static int orc_shortcut_leaf(const orc_live* m, int node, int lo, int hi, int* miss)
{
    *miss = 0;
    if (!orc_shortcut_max || orc_live_shift != 0 || hi - lo + 1 > orc_shortcut_max) return -1;
    if (!orc_shortcut_general && !orc_uonly[node]) return -1;
    int found = -1;
    for (int g = lo; g <= hi; ++g)
        if ((m->w[g >> 6] >> (g & 63)) & 1u) {
            if (found >= 0) return -1;
            found = g;
        }
    if (found < 0) return -1;
    *miss = !(orc_blk[found] < orc_depth[node]);
    return orc_leaf_node[found];
}
static void orc_live_clear(orc_live* m, int lo, int hi, double tmin)
{
    const int sh = orc_live_shift;
    const int ga = (lo + (1 << sh) - 1) >> sh, gb = ((hi + 1) >> sh) - 1;
    if (ga > gb) return;
    const double tc = (tmin == tmin) ? tmin : INFINITY;
    const int regional = (orc_live_mode == 4 || orc_live_mode == 6);
    for (int g = ga; g <= gb; ++g) {
        const uint64_t bit = 1ull << (g & 63);
        /* per-region records are raised only by groups that were live (a group already
         * clear keeps the validity of its earlier clear) */
        if (regional && !(m->w[g >> 6] & bit)) continue;
        m->w[g >> 6] &= ~bit;
        if (tc > m->treg[g / orc_live_region]) m->treg[g / orc_live_region] = tc;
    }
    if (tc > m->tclr) m->tclr = tc;
}
/* A loop to tmin re-enters the subtree with leaves [lo, hi]: mode 1 re-enables all its
 * groups when tmin is below the ray's largest clear tmin, mode 4 those of the regions
 * cleared above tmin; modes 5 and 6 are modes 1 and 4 re-enabling only groups that were
 * live at tmin = 0 (a group the pre-pass cleared is a Miss at every tmin). */
static void orc_live_restore(orc_live* m, int lo, int hi, double tmin)
{
    const int regional = (orc_live_mode == 4 || orc_live_mode == 6);
    const int keep = (orc_live_mode == 5 || orc_live_mode == 6);
    if (!regional && tmin >= m->tclr) return;
    for (int g = lo >> orc_live_shift; g <= (hi >> orc_live_shift); ++g)
        if (!regional || !(tmin >= m->treg[g / orc_live_region]))
            if (!keep || ((m->p[g >> 6] >> (g & 63)) & 1u)) m->w[g >> 6] |= 1ull << (g & 63);
}

#define ORC_FMA 0
#define ORC_SUFFIX(name) name##_ieee
#include "csg_oracle_render.inc"
#undef ORC_FMA
#undef ORC_SUFFIX

#define ORC_FMA 1
#define ORC_SUFFIX(name) name##_fma
#include "csg_oracle_render.inc"
#undef ORC_FMA
#undef ORC_SUFFIX

#define ORC_FMA 0
#define ORC_F64 1
#define ORC_SUFFIX(name) name##_f64
#include "csg_oracle_render.inc"
#undef ORC_FMA
#undef ORC_F64
#undef ORC_SUFFIX
