/* csgrt -- GB300-native (sm_103a) CSG ray-casting engine, C ABI.
 *
 * Drop-in for the render path of Zumi002/CUDA-CSG-Tree-Raycasting: load a CSG tree
 * from the reference's preorder text format, set a camera and a directional light, and
 * ray-cast + Phong-shade into a caller-owned device buffer.  Plain pointers and sizes
 * only; every call returns a csg_status.  No call exits the process, none synchronises
 * the device unless its comment says so, and renders are ordered on the caller's stream.
 *
 * Reference interfaces replaced (file:line within the reference project):
 *   CSGTree::Parse + ConstructBVH        CSGRayCasting/Graphics/RayCasting/CSGTree/CSGTree.cu:5-179
 *   Raycaster::ChangeSize (scene upload) CSGRayCasting/Graphics/RayCasting/Raycaster.cu:3-21
 *   Raycaster::Raycast                   CSGRayCasting/Graphics/RayCasting/Raycaster.cu:23-34
 *   Raycaster::CleanUp                   CSGRayCasting/Graphics/RayCasting/Raycaster.cu:36-44
 *   Camera                               CSGRayCasting/Graphics/RenderManager/Camera/Camera.h:3-53, Camera.cpp:4-36
 *   DirectionalLight::getLightDir        CSGRayCasting/Graphics/RenderManager/DirectionalLight.h:8-18
 */
#ifndef CSGRT_H
#define CSGRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSGRT_ABI_VERSION 1

/* Status codes.  Parse errors carry the reference's exception text in `err`. */
typedef enum csg_status {
    CSG_OK = 0,
    CSG_E_PARSE = 1,    /* malformed scene text (std::invalid_argument in the reference) */
    CSG_E_RANGE = 2,    /* number out of range, or a rotation outside [0, 360] degrees */
    CSG_E_COUNT = 3,    /* node count != 2 * primitive count - 1 */
    CSG_E_CUDA = 4,     /* a CUDA runtime call failed */
    CSG_E_BUDGET = 5,   /* request refused: device-memory budget exceeded */
    CSG_E_TIMEOUT = 6,  /* a bounded device wait gave up, or rays hit the iteration cap */
    CSG_E_DEPTH = 7,    /* scene too large for the device layout (> 32767 primitives) */
    CSG_E_ARG = 8,      /* invalid argument (null pointer, non-positive size, ...) */
    CSG_E_CAPACITY = 9  /* caller-provided array too small */
} csg_status;

/* Same 60-byte layout as the reference's Camera (Camera.h:9-16), so a caller can pass
 * the bytes of a reference Camera object directly. */
typedef struct csg_camera {
    float x, y, z;    /* position */
    float rot_x;      /* pitch, radians */
    float rot_y;      /* yaw, radians */
    float fov;        /* vertical field of view, radians */
    float forward[3];
    float right[3];
    float up[3];
} csg_camera;

typedef struct csg_scene csg_scene; /* opaque, device-resident until destroyed */

typedef struct csg_scene_info {
    int32_t n_nodes;      /* nodes in the tree (2 * n_prims - 1) */
    int32_t n_prims;      /* primitives (sphere, cylinder, cube) */
    int32_t op_depth;     /* most operator nodes on any root-to-leaf path */
    int32_t stack_class;  /* per-ray stack capacity the kernels use for this scene */
    uint64_t device_bytes;/* device memory held by the scene */
    int32_t rolled;       /* kernel variant: GoTo's child tests in a rolled loop */
    int32_t live_words;   /* words of the per-ray live-leaf mask (batched renders) */
    int32_t live_shift;   /* log2 of the leaves per mask bit */
    int32_t fine_words;   /* words of the one-bit-per-leaf mask of single-view renders, 0 if unused */
    int32_t short_circuit;/* the traversal skips the other child of a Difference / Intersection
                             that a Miss child decides */
} csg_scene_info;

/* Optional per-pixel planes.  Any pointer may be NULL.  Row-major, w*h entries, row 0 is
 * the image row the reference computes with v = 0.5/(h-1) (its GL texture's first row). */
typedef struct csg_planes {
    uint32_t* rgba8;   /* packed R | G<<8 | B<<16 | A<<24, q = lrintf(clamp(c,0,1)*255) */
    float* rgba32f;    /* float4 per pixel: the reference's RGBA32F PBO format */
    float* t;          /* hit distance, +inf on a miss */
    int32_t* prim;     /* hit primitive index (file order), -1 on a miss */
    float* normal;     /* three planes (x, y, z) of w*h floats; 0 on a miss */
} csg_planes;

/* ---- scene: CSGTree::Parse (CSGTree.cu:5-152) + ConstructBVH (CSGTree.cu:154-179) +
 *      the scene upload of Raycaster::ChangeSize (Raycaster.cu:16-17) --------------- */
/* Parses `len` bytes of scene text, builds the bounding boxes and the flattened device
 * layout, uploads it on the current device, and synchronises that upload.  On failure
 * *out is NULL and `err` (if given) holds the reference's message, e.g.
 * "Cannot parse - Unrecognized keyword: Spere". */
int csg_scene_create(const char* text, size_t len, csg_scene** out, char* err, size_t errlen);
/* Optional exact-box mode (no counterpart in the reference; off by default because it
 * changes the output): sphere boxes ±r instead of ±2r and cylinder boxes that contain
 * the cylinder (the reference's, BVHNode.cuh:34-49, cut hits), each widened by 2^-12 of
 * its size plus 1e-5.  Cube and operator boxes as the reference builds them. */
#define CSG_SCENE_EXACT_BOXES 1
/* Fine live mask (same output): single-view renders of a rolled tree of 1,025-2,048 leaves
 * keep one live bit per leaf instead of one per two leaves.  Off by default: since the
 * operator short-circuit it is faster for a few trees and slower for most (fewer resident
 * blocks); a caller rendering one large tree many times can time both. */
#define CSG_SCENE_FINE_MASK 2
int csg_scene_create_ex(const char* text, size_t len, int32_t flags, csg_scene** out, char* err, size_t errlen);
/* Frees the scene's device memory (Raycaster::CleanUp, Raycaster.cu:36-44). */
int csg_scene_destroy(csg_scene* scene);
int csg_scene_get_info(const csg_scene* scene, csg_scene_info* info);
/* What csg_scene_create(_ex) would build for this text, computed on the host alone (no
 * device work): the same fields csg_scene_get_info reports for the created scene.  Parse
 * errors as csg_scene_create. */
int csg_tree_plan(const char* text, size_t len, int32_t flags, csg_scene_info* info, char* err, size_t errlen);
/* CSGTree::Parse alone (host only, no device work): parses and builds the boxes into the
 * reference's own record layouts, 44-byte CSGNode (CSGTree.cuh:15-34) and 48-byte
 * Primitive (Primitives.h:29-40).  Pass NULL arrays to query the counts.  Unused
 * parameter slots of a primitive are zero. */
int csg_tree_parse(const char* text, size_t len, void* nodes44, int32_t max_nodes, void* prims48,
                   int32_t max_prims, int32_t* n_nodes, int32_t* n_prims, int32_t* op_depth,
                   char* err, size_t errlen);
/* csg_tree_parse with the csg_scene_create_ex flags (the boxes of the exact-box mode). */
int csg_tree_parse_ex(const char* text, size_t len, int32_t flags, void* nodes44, int32_t max_nodes,
                      void* prims48, int32_t max_prims, int32_t* n_nodes, int32_t* n_prims, int32_t* op_depth,
                      char* err, size_t errlen);
/* Copies the parsed tree out in the reference's own record layouts: 44-byte CSGNode
 * (CSGTree.cuh:15-34) and 48-byte Primitive (Primitives.h:29-40).  Pass NULL arrays to
 * query the counts. */
int csg_scene_export_reference_layout(const csg_scene* scene, void* nodes44, int32_t max_nodes,
                                      void* prims48, int32_t max_prims,
                                      int32_t* n_nodes, int32_t* n_prims);

/* ---- camera and light: Camera (Camera.h, Camera.cpp), DirectionalLight ------------- */
void csg_camera_init(csg_camera* cam);                       /* Camera() */
void csg_camera_set_position(csg_camera* cam, float x, float y, float z);
void csg_camera_set_rotation(csg_camera* cam, float pitch, float yaw); /* clamps pitch to +-89 deg */
void csg_camera_set_fov(csg_camera* cam, float degrees);
void csg_camera_move(csg_camera* cam, float forward, float right, float up);
void csg_camera_rotate(csg_camera* cam, float dpitch, float dyaw);
void csg_light_dir(float polar, float azimuth, float out[3]); /* radians */
void csg_light_default(float out[3]);                         /* polar -60 deg, azimuth -45 deg */

/* ---- render: Raycaster::Raycast (Raycaster.cu:23-34) = RaycastKernel + LightningKernel
 *      fused into one launch on `stream` (a cudaStream_t; NULL = legacy default) -------- */
/* One primary ray per pixel, Kensler single-hit CSG traversal, Phong shading.
 * `light_dir` is the DirectionalLight direction (normalised inside, as the reference
 * does).  All output pointers are device pointers owned by the caller.
 * Frames of at least 32,768 block tiles (8x16 pixels; 2048x2048 and larger) record each
 * tile's render time, and the scene's next frame of the same size on the same stream
 * starts its slowest tiles first; the output is the same, byte for byte.  The first stream
 * that renders such a frame of a scene outside a graph capture owns this state (8 bytes per
 * tile of device memory, allocated on that call, freed by csg_scene_destroy); frames on
 * other streams, and frames captured into graphs, keep the fixed order. */
int csg_render(const csg_scene* scene, const csg_camera* cam, const float light_dir[3],
               int32_t w, int32_t h, uint32_t* rgba8_dev, float* t_dev, int32_t* prim_dev,
               float* normal_dev, void* stream);
/* The reference's own output format: w*h float4 RGBA32F. */
int csg_render_f4(const csg_scene* scene, const csg_camera* cam, const float light_dir[3],
                  int32_t w, int32_t h, float* rgba_f4_dev, void* stream);
/* Every plane at once. */
int csg_render_planes(const csg_scene* scene, const csg_camera* cam, const float light_dir[3],
                      int32_t w, int32_t h, const csg_planes* planes, void* stream);
/* No counterpart in the reference (whose frame stays in a device PBO): renders the RGBA8
 * frame into HOST memory.  A page-locked destination (cudaHostAlloc, cudaMallocHost,
 * cudaHostRegister) is written by the kernel itself over the host link, with no staging
 * buffer and no separate copy, and the call is asynchronous on `stream`; a pageable
 * destination is rendered into a stream-ordered device frame and copied, and the call
 * returns once the frame is in host memory.  A device pointer is CSG_E_ARG. */
int csg_render_host(const csg_scene* scene, const csg_camera* cam, const float light_dir[3],
                    int32_t w, int32_t h, uint32_t* host_rgba8, void* stream);
/* Synchronises `stream` and reports how many rays of the renders issued since the last
 * call stopped at the traversal iteration cap (CSG_E_TIMEOUT if any, else CSG_OK). */
int csg_scene_check(const csg_scene* scene, void* stream, uint64_t* n_capped);
/* No counterpart in the reference (whose traversal loop has no bound).  Sets the per-ray
 * cap on traversal iterations of the renders enqueued after the call (0 restores the
 * default, 2^20, which no well-formed tree reaches); a ray that reaches it is written as a
 * miss and counted (csg_scene_check, csg_batch_check).  A batch keeps the cap in force
 * when it was created.  Process-wide. */
int csg_set_iteration_cap(uint32_t cap);

/* ---- batches: many views of many scenes in one persistent launch --------------------
 * No counterpart in the reference, which renders one view per Raycast call; the per-view
 * results are the same bytes csg_render_planes writes. */
typedef struct csg_view {
    const csg_scene* scene;
    csg_camera cam;
    float light_dir[3];
    int32_t w, h;
    csg_planes out;   /* device planes of this view (any may be NULL) */
} csg_view;

typedef struct csg_batch csg_batch;

typedef struct csg_batch_info {
    int32_t n_views;
    int32_t n_items;      /* work items: 32-pixel warp tiles, all classes */
    int32_t warp_tile_w;  /* warp tile width of the heaviest class (height = 32 / width) */
    int32_t stack_class;  /* largest stack capacity of any class's kernel variant */
    int32_t rolled;       /* some class uses the rolled GoTo loop */
    int32_t grid;         /* persistent blocks of the largest class launch */
    uint64_t device_bytes;
    int32_t n_classes;        /* tree-size classes (one persistent launch each) */
    int32_t warps_per_block;  /* block shape of the heaviest class: warps per block */
    int32_t local_stacks;     /* ... and its per-ray stacks in local (1) or shared (0) memory */
} csg_batch_info;

/* One tree-size class of a batch: its kernel variant and the configuration the autotuner
 * (or csg_batch_set_tile / csg_batch_set_shape) gave it. */
typedef struct csg_batch_class_info {
    int32_t n_views;
    int32_t stack_class;      /* per-ray stack capacity of the kernel variant */
    int32_t rolled;           /* rolled GoTo loop */
    int32_t live_words;       /* live-mask words per ray (a power of two) */
    int32_t warp_tile_w;      /* warp tile width (height 32 / width) */
    int32_t warps_per_block;  /* 2, 4 or 8 */
    int32_t local_stacks;     /* per-ray stacks in local memory (1) or block shared memory (0) */
    int32_t grid;             /* persistent blocks of its launch */
    int32_t n_items;          /* its 32-pixel warp tiles */
    float tuned_ms;           /* the class alone at its tuned configuration; 0 before tuning */
} csg_batch_class_info;

/* Builds the batch on the current device: views are grouped into tree-size classes (same
 * kernel variant and live-mask size), each with its own view table (most expensive first)
 * and persistent launch.  The scenes and the output planes must stay valid while the
 * batch is used.  Output planes may be device memory or page-locked host memory, which
 * the kernel writes over the host link (the frames are complete when the render's stream
 * is); pageable host memory is CSG_E_ARG. */
int csg_batch_create(const csg_view* views, int32_t n_views, csg_batch** out);
int csg_batch_destroy(csg_batch* batch);
/* Renders every view: one CUDA graph, captured on the first call (and again after a tile
 * change), whose branches are the classes' launches; asynchronous on `stream`. */
int csg_batch_render(csg_batch* batch, void* stream);
/* Sets the warp tile width of every class (4, 8, 16 or 32 pixels; height 32 / width). */
int csg_batch_set_tile(csg_batch* batch, int32_t warp_tile_w);
/* Sets the block shape of every class's launch: 4 warps per block with the per-ray stacks
 * in shared memory (local_stacks 0) or in local memory (1), or 2 or 8 warps per block with
 * shared-memory stacks.  Every shape renders the same bytes. */
int csg_batch_set_shape(csg_batch* batch, int32_t warps_per_block, int32_t local_stacks);
/* Autotuner, for each class alone: every warp tile shape with the default block shape,
 * then the other block shapes (warps per block, stack placement) with the best tile;
 * keeps each class's fastest and reports the heaviest class's tile width and the whole
 * batch's time.  Synchronous. */
int csg_batch_tune(csg_batch* batch, void* stream, int32_t* best_tile_w, float* best_ms);
int csg_batch_get_info(const csg_batch* batch, csg_batch_info* info);
/* Class k (0 <= k < n_classes, heaviest first) of the batch. */
int csg_batch_get_class(const csg_batch* batch, int32_t k, csg_batch_class_info* info);
/* Sets class k's warp tile width and block shape (as csg_batch_set_tile and
 * csg_batch_set_shape do for every class), e.g. to give a second batch over the same
 * scenes the configuration another batch was tuned to. */
int csg_batch_set_class(csg_batch* batch, int32_t k, int32_t warp_tile_w, int32_t warps_per_block,
                        int32_t local_stacks);
/* Synchronises `stream`; number of rays of the batch's renders stopped at the iteration
 * cap since the last call (CSG_E_TIMEOUT if any). */
int csg_batch_check(csg_batch* batch, void* stream, uint64_t* n_capped);

/* ---- batched render without allocation ----------------------------------------------
 * No counterpart in the reference.  Renders up to CSG_NOALLOC_MAX_VIEWS views in one
 * persistent launch, like csg_batch_render, but allocates no memory: its scratch (work
 * counter, view table, tile prefix; 1 MiB) is a fixed array in the library's device
 * image.  For callers that cannot allocate at render time -- a server at its
 * device-memory budget, a frame loop that cannot take the device-wide synchronisation of
 * cudaFree.  warp_tile_w is 4, 8, 16 or 32 (0: 8).  More than CSG_NOALLOC_MAX_VIEWS views
 * gives CSG_E_CAPACITY, and a view with pageable host planes CSG_E_ARG, before anything
 * is enqueued (planes may be device or page-locked host memory, as for csg_batch_create).
 * Asynchronous on `stream`; capped
 * rays are counted per scene (csg_scene_check).  Set-up: the first call on a device looks
 * up the array's address there, and the first call with each kernel variant (stack class,
 * rolled GoTo loop, block shape) and live-mask size on a device sets that kernel's
 * attributes and queries its occupancy (a fixed table of 64 such entries per variant; once
 * it is full, new sizes redo the query on every call).  Make a call with every variant a
 * capture will use before any stream capture on that device.  All calls on a device share
 * the one array, so calls whose work may overlap (different streams, unsynchronised
 * threads) race: serialise them.  One call renders all its views with one kernel variant,
 * that of its heaviest view (largest stack class and live mask, rolled if any view is):
 * the planes are the same, but one tree deeper than 15 operator levels gives every view of
 * the call its 32-entry stacks (fewer resident blocks), and one large tree its large live
 * mask, so group views by tree class as csg_batch does.
 * The call uses about 21 KB of the calling thread's stack. */
#define CSG_NOALLOC_MAX_VIEWS 4096
int csg_render_views_noalloc(const csg_view* views, int32_t n_views, int32_t warp_tile_w, void* stream);

/* ---- render server: continuous batching of render requests ---------------------------
 * No counterpart in the reference (one interactive view per frame).  A server owns a
 * pool of scenes, made resident on the device on first use and evicted least recently
 * used when the device-memory budget (resident scenes + in-flight outputs) would be
 * exceeded.  Requests queue as they arrive; a dispatcher thread admits them, as slots
 * (batches in flight, one stream each) and memory free up, into batches rendered by the
 * persistent view-table kernel, so requests that arrive while others run start on a free
 * slot and overlap the running work on the device.  Each request's planes are the bytes
 * csg_render_planes writes for it alone. */
typedef struct csg_server csg_server;

#define CSG_PLANE_RGBA8 1
#define CSG_PLANE_T 2
#define CSG_PLANE_PRIM 4
#define CSG_PLANE_NORMAL 8
#define CSG_PLANE_RGBA32F 16

typedef struct csg_server_config {
    uint64_t hbm_budget;      /* bytes for resident scenes + outputs in flight (0: 40 GiB) */
    int32_t slots;            /* batches in flight, one stream each (0: 4; at most 16) */
    int32_t max_batch_views;  /* views per batch (0: 256; at most 4096) */
    int32_t warp_tile_w;      /* 4, 8, 16 or 32 (0: 8) */
    int32_t planes;           /* CSG_PLANE_* bits rendered per request (0: RGBA8) */
    int32_t keep_results;     /* 1: device planes stay until csg_server_release; 0: freed when done */
    int32_t order;            /* 0: requests admitted and laid out in arrival order; 1: the same,
                                 each batch's views longest first; 2: size-aware: requests of
                                 up to 2^18, up to 2^20 and more rays launched separately,
                                 earliest deadline first (arrival + 8 x its rays at 1.5 Grays/s),
                                 one launch of the largest in flight, each view by the
                                 single-view kernel, the smallest on a raised stream priority */
} csg_server_config;

#define CSG_REQ_ALONE 1       /* render with its own single-view launch (the unbatched form) */

typedef struct csg_request {
    int32_t scene;            /* id from csg_server_add_scene */
    int32_t flags;            /* CSG_REQ_* */
    csg_camera cam;
    float light_dir[3];
    int32_t w, h;
    void* host_rgba8;         /* optional: the RGBA8 plane is also copied here (pinned memory
                                 recommended), before the request counts as done */
} csg_request;

typedef struct csg_result {
    int32_t status;           /* CSG_OK, or why this request failed (CSG_E_BUDGET: it can never fit) */
    int32_t batch_views;      /* views in the launch that rendered it */
    double t_arrive, t_launch, t_done;  /* seconds on the server's clock (csg_server_clock) */
    csg_planes planes;        /* device planes (valid until released, with keep_results) */
} csg_result;

typedef struct csg_server_stats {
    uint64_t budget, scene_bytes, output_bytes, peak_bytes;
    int64_t requests_done, batches, evictions, rejected;
    int32_t scenes, resident_scenes, slots_busy, pending;
    uint64_t capped_rays;  /* rays of all requests stopped at the traversal iteration cap */
} csg_server_stats;

int csg_server_create(const csg_server_config* cfg, csg_server** out);
/* Finishes every queued and in-flight request, then frees everything. */
int csg_server_destroy(csg_server* server);
/* Parses a scene (errors as csg_scene_create) into the pool; resident on first use. */
int csg_server_add_scene(csg_server* server, const char* text, size_t len, int32_t* id, char* err, size_t errlen);
/* Makes a scene resident now (CSG_E_BUDGET if it cannot fit). */
int csg_server_preload(csg_server* server, int32_t id);
/* Queues a request; returns at once with its ticket. */
int csg_server_submit(csg_server* server, const csg_request* req, int64_t* ticket);
/* Waits up to timeout_s (< 0: forever) for a request; CSG_E_TIMEOUT if not done by then. */
int csg_server_wait(csg_server* server, int64_t ticket, double timeout_s, csg_result* out);
/* Forgets a finished request and frees its device planes. */
int csg_server_release(csg_server* server, int64_t ticket);
/* Open-loop replay: submits reqs[i] at arrival_s[i] seconds after the call starts, waits
 * for all, fills results (t_arrive = the scheduled arrival) and the wall time from the
 * start to the last completion.  tickets (optional) receives the tickets, which the caller
 * then releases; without it the requests are released here. */
int csg_server_replay(csg_server* server, const csg_request* reqs, const double* arrival_s, int32_t n,
                      csg_result* results, int64_t* tickets, double* wall_s);
int csg_server_stats_get(csg_server* server, csg_server_stats* out);
double csg_server_clock(const csg_server* server);

/* ---- headless image export ------------------------------------------------------------
 * Replaces the reference's OpenGL display of the frame (RenderManager.cpp:69-84, no
 * graphics stack here): writes a host RGBA8 frame (as csg_render produces it, row 0 on top)
 * to `path` as binary PPM (RGB) or PNG (RGBA, uncompressed deflate).  Synchronous. */
#define CSG_IMAGE_PPM 0
#define CSG_IMAGE_PNG 1
int csg_image_write(const char* path, const uint32_t* rgba8, int32_t w, int32_t h, int32_t format);

/* ---- misc ---------------------------------------------------------------------------- */
/* Diagnostic: tan(fov / 2) as the device's ray generation computes it (RaycastingKernels.cu
 * :15-16 evaluates tan on the device).  Synchronous.  For checkers that restate the ray
 * generation on a host, whose tanf may differ in the last bit. */
int csg_device_tan_half_fov(float fov, float* out);
/* Diagnostic: measures the FP32 fused-multiply-add rate of the current device (TFLOP/s,
 * an FMA counted as 2), the denominator of the FP32 roofline.  Synchronous. */
int csg_probe_fp32_peak(float* tflops, float* ms);
const char* csg_status_string(int status);
int csg_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CSGRT_H */
