/* CPU oracle for the CSG ray-casting path: a plain-C restatement of the reference's
 * parser, camera/light math, Kensler traversal, intersection tests and Phong shading.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg use this library, to check results against it; the product never
 * links it.
 *
 * Pinning: the "ieee" arithmetic mode is checked bit for bit against the reference's own
 * code compiled for the host (oracle/build_ref.py, oracle/ref_host_shim.cpp) on every
 * scene file the reference ships and on seeded synthetic scenes (tests/test_oracle_pin.py).
 * The "fma" mode restates the fused multiply-adds that nvcc's default contraction
 * (--fmad=true) forms in the reference CUDA kernel; it is pinned against that kernel's
 * own output on the GPU (tests/golden/ fixtures made by tests/golden/make_golden.py).
 * The "f64" mode carries the same steps in double: the yardstick against which the
 * FP32 results' errors are stated.
 *
 * Record layouts follow the reference byte for byte, so parse results can be compared
 * directly and fed to the reference kernel:
 *   orc_node  == CSGNode   (CSGTree.cuh:15-34 + BVHNode BVHNode.cuh:6-11), 44 bytes
 *   orc_prim  == Primitive (Primitives.h:29-40), 48 bytes
 *   camera    == Camera    (Camera.h:9-16), 15 floats
 */
#ifndef CSG_ORACLE_H
#define CSG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_UNION = 0, ORC_DIFFERENCE = 1, ORC_INTERSECTION = 2,
       ORC_SPHERE = 3, ORC_CYLINDER = 4, ORC_CUBE = 5 };

typedef struct orc_node {
    int32_t type, prim, left, right, parent;
    float minx, miny, minz, maxx, maxy, maxz;
} orc_node;

typedef struct orc_prim {
    int32_t id;
    float x, y, z;
    float r, g, b;
    float p[5]; /* sphere: radius | cylinder: radius, height, axis x/y/z | cube: edge */
} orc_prim;

/* Per-ray work counters (the reference algorithm's own work on that ray). */
typedef struct orc_counts {
    uint32_t iters;   /* CSGRayCast loop iterations (RaycastingKernels.cu:474) */
    uint32_t aabb;    /* isBVHNodeHit calls (RaycastingKernels.cu:718) */
    uint32_t sphere;  /* sphereHit calls */
    uint32_t cyl;     /* cylinderHit calls */
    uint32_t cube;    /* cubeHit calls */
    uint32_t max_actions; /* deepest action stack */
    uint32_t flops_trace; /* FP32 ops of ray generation + traversal (as written in the reference) */
    uint32_t flops;       /* ... plus hit details and shading */
} orc_counts;

/* Parse status codes (match include/csgrt.h). */
enum { ORC_OK = 0, ORC_E_PARSE = 1, ORC_E_RANGE = 2, ORC_E_COUNT = 3, ORC_E_CAPACITY = 9 };

int orc_parse(const char* text, size_t len, orc_node* nodes, int max_nodes,
              orc_prim* prims, int max_prims, int* n_nodes, int* n_prims,
              char* err, size_t errlen);

/* Recomputes the boxes of a parsed tree as the engine's exact-box mode does. */
void orc_boxes_exact(orc_node* nodes, int n_nodes, const orc_prim* prims);

void orc_camera_default(float cam[15]);
void orc_camera_set_position(float cam[15], float x, float y, float z);
void orc_camera_set_rotation(float cam[15], float pitch, float yaw);
void orc_camera_set_fov(float cam[15], float degrees);
void orc_camera_move(float cam[15], float fwd, float right, float up);
void orc_camera_rotate(float cam[15], float dpitch, float dyaw);
void orc_light_dir(float polar, float azimuth, float out[3]);
void orc_light_default(float out[3]);
float orc_tan_half_fov(float fov);

/* Render rows [y0, y1) of a w x h image.  tan_half_fov is tan(fov/2) as the device
 * computes it (the ray generation's only transcendental); pass orc_tan_half_fov(fov)
 * for the host value.  Any output pointer may be NULL.  Planes are indexed by the full
 * image pixel index y*w+x.  On a miss: hit=0, t=+inf, prim=-1, normal=0.
 * rgba8 = lrintf(clamp(c,0,1)*255) per channel, R in the low byte.
 * Returns the number of rays whose traversal hit the iteration cap (0 normally). */
int orc_render_ieee(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                    const float cam[15], float tan_half_fov, const float light[3],
                    int w, int h, int y0, int y1, int nthreads,
                    uint8_t* hit, float* t, int32_t* prim, float* normal3, float* pos3,
                    float* rgba32f, uint32_t* rgba8, orc_counts* counts);
int orc_render_fma(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                   const float cam[15], float tan_half_fov, const float light[3],
                   int w, int h, int y0, int y1, int nthreads,
                   uint8_t* hit, float* t, int32_t* prim, float* normal3, float* pos3,
                   float* rgba32f, uint32_t* rgba8, orc_counts* counts);

/* Render an arbitrary list of pixels (x = pix % w, y = pix / w) of a w x h frame: a
 * bounded sample, used for sampled parity checks of full-size frames and by the timed
 * CPU baseline.  Outputs are indexed by list position; any may be NULL. */
int orc_render_list_ieee(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                         const float cam[15], float tan_half_fov, const float light[3],
                         int w, int h, const int64_t* pix, int64_t n_pix, int nthreads,
                         uint8_t* hit, float* t, int32_t* prim, float* normal3,
                         uint32_t* rgba8, orc_counts* counts);
/* The same steps carried in double (the FP64 yardstick for error statements). */
int orc_render_f64(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                   const float cam[15], float tan_half_fov, const float light[3],
                   int w, int h, int y0, int y1, int nthreads,
                   uint8_t* hit, float* t, int32_t* prim, float* normal3, float* pos3,
                   float* rgba32f, uint32_t* rgba8, orc_counts* counts);
int orc_render_list_f64(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                        const float cam[15], float tan_half_fov, const float light[3],
                        int w, int h, const int64_t* pix, int64_t n_pix, int nthreads,
                        uint8_t* hit, float* t, int32_t* prim, float* normal3,
                        uint32_t* rgba8, orc_counts* counts);
int orc_render_list_fma(const orc_node* nodes, int n_nodes, const orc_prim* prims, int n_prims,
                        const float cam[15], float tan_half_fov, const float light[3],
                        int w, int h, const int64_t* pix, int64_t n_pix, int nthreads,
                        uint8_t* hit, float* t, int32_t* prim, float* normal3,
                        uint32_t* rgba8, orc_counts* counts);

/* Optional operator short-circuit of the traversal (off by default; not the reference's
 * algorithm): see csg_oracle.c.  Process-wide. */
void orc_set_short_circuit(int on);

/* Optional live-leaf pruning of the traversal (0 off, the default; 1 one restore record
 * per ray; 2 the same without its loop restore and 3 the same on trees of any depth, both
 * unsound; 4 one restore record per region of orc_set_live_region groups; 5 and 6 are
 * 1 and 4 restoring only groups live at tmin = 0): see csg_oracle.c.  Process-wide. */
void orc_set_live_pruning(int mode);
void orc_set_live_region(int groups);
/* Union shortcut (with live-leaf pruning; 0 off, the default): an all-Union operator
 * subtree of at most max_leaves leaves with one live leaf is evaluated as that leaf. */
void orc_set_union_shortcut(int max_leaves);
/* The same for any operator subtree: its result is the live leaf's when every operator on
 * the path down to it is a Union or a Difference entered on its left, else a Miss. */
void orc_set_leaf_shortcut(int max_leaves);

#ifdef __cplusplus
}
#endif
#endif
