// Scene model of the CSG ray-casting engine: the host tree parsed from the reference's
// text format, and the flattened device layout the kernels read.
#pragma once

#include <cstdint>
#include <string>
#include <string_view>
#include <vector>

#include <cuda_runtime.h>

namespace csgrt {

// CSGTree::NodeType (CSGTree.cuh:38-46).
enum NodeType : int32_t { kUnion = 0, kDifference = 1, kIntersection = 2,
                          kSphere = 3, kCylinder = 4, kCube = 5 };

// Host records in the reference's own byte layouts, so a parsed tree can be exported
// to (and compared with) the reference: CSGNode (CSGTree.cuh:15-34, with the BVHNode of
// BVHNode.cuh:6-11 embedded) and Primitive (Primitives.h:29-40).
struct RefNode {
    int32_t type, prim, left, right, parent;
    float minx, miny, minz, maxx, maxy, maxz;
};
struct RefPrim {
    int32_t id;
    float x, y, z;
    float r, g, b;
    float p[5];  // sphere: radius | cylinder: radius, height, axis xyz | cube: edge
};
static_assert(sizeof(RefNode) == 44, "CSGNode layout");
static_assert(sizeof(RefPrim) == 48, "Primitive layout");

struct HostTree {
    std::vector<RefNode> nodes;  // node 0 is the root, preorder
    std::vector<RefPrim> prims;  // file order
    int32_t op_depth = 0;        // most operator nodes on a root-to-leaf path
    // Leaves are numbered in preorder, which is the primitive (file) order, so the leaves
    // of every subtree form one contiguous primitive range [leaf_lo, leaf_hi].
    std::vector<int32_t> leaf_lo, leaf_hi;
};

// Parse status codes (values of csg_status).
enum : int { kOk = 0, kErrParse = 1, kErrRange = 2, kErrCount = 3, kErrDepth = 7 };

// CSGTree::Parse (CSGTree.cu:5-152) followed by ConstructBVH (CSGTree.cu:154-179).
// Returns a status code; `err` receives the reference's exception text.
int parse_tree(std::string_view text, HostTree& out, std::string& err);
// Recomputes every box of a parsed tree in the exact-box mode (CSG_SCENE_EXACT_BOXES).
void use_exact_boxes(HostTree& t);

// ---------------------------------------------------------------------------------
// Device layout (all arrays 16-byte aligned, one cudaMalloc):
//   topo[n]    int4   {left, right, parent, type} for operators,
//                     {prim, -1, parent, type} for leaves (device node numbers: see
//                     CSG_DENSE_OPERATORS)
//   kids[5m]   for each of the m operator nodes, everything GoTo needs in five independent 16-byte
//                     loads (the Ulyanov layout): the two children's boxes with the
//                     child's type and primitive index in .w (as int bits), then the
//                     children's leaf ranges:
//                     {l.min.xyz, l.type} {l.max.xyz, l.prim} {r.min.xyz, r.type}
//                     {r.max.xyz, r.prim} {l.leaf_lo, l.leaf_hi, r.leaf_lo, r.leaf_hi},
//                     l.leaf_lo's bit 30 set when the right child is to be tested first,
//                     the children's depth (operators above them) in bits 16-23 of
//                     l.leaf_hi and, in trees deeper than 15 operator levels, the node's
//                     operator height (up to 127) in bits 24-30 of l.leaf_hi
//   lbox[2p]   per leaf (primitive order) its own box as a kids child record,
//                     {min.xyz, type} {max.xyz, prim | (blk + 1) << 16}, blk the depth of
//                     the deepest operator above it that is an Intersection or a Difference
//                     entered on its right (-1: none), for the single-leaf shortcut
//   geo[2p]    float4 {cx, cy, cz, p0} {p1, p2, p3, p4}
//   color[p]   float4 {r, g, b, 0}
//   bvh[6b]    a binary BVH over the leaves' own boxes (the reference's boxes), used
//                     only to find the primitives a ray can hit; per node the two
//                     children's boxes: {min.xyz, child} {max.xyz, type} x 2, where
//                     child >= 0 is a BVH node and child < 0 is leaf ~prim (type valid);
//                     then per slot (node * 2 + side) a bounding sphere {centre.xyz, r}:
//                     the smallest ball about the box's rounded centre that holds the box,
//                     its radius rounded up, or for a sphere leaf the sphere itself with
//                     its radius negated (the sign marks a sphere leaf)
// ---------------------------------------------------------------------------------
constexpr int kKidsPerNode = 5;
// Node numbering of the device arrays (a build-time knob): 1 numbers the operators first
// (kids records dense, one per operator), 0 keeps the reference's preorder (a kids record
// per node, zeros for leaves).  Either way node 0 is the root.
#ifndef CSG_DENSE_OPERATORS
#define CSG_DENSE_OPERATORS 1
#endif
// Live-leaf mask: at most CSG_LIVE_WORDS_MAX words per ray (32: 1024 bits; 64 is the
// largest the one-register word summary can index).  A build-time tuning knob: more words
// keep one bit per leaf on larger trees at the cost of shared memory per block.
#ifndef CSG_LIVE_WORDS_MAX
#define CSG_LIVE_WORDS_MAX 32
#endif
constexpr int kLiveWordsMax = CSG_LIVE_WORDS_MAX;
static_assert(kLiveWordsMax >= 1 && kLiveWordsMax <= 64, "live-mask words");
// Fine live mask of single-view renders (the render_tiled variants for rolled scenes):
// one bit per leaf, up to kFineWordsMax words, for a scene whose own mask groups leaves
// (more than 32 * kLiveWordsMax of them).  Used by default when the fine mask needs at
// most CSG_FINE_WORDS_USE words (0: never), and on request (CSG_SCENE_FINE_MASK) up to
// kFineWordsMax.  Measured on the batched workload's 35 trees of 1,025-2,015 leaves, as
// single views: before the operator short-circuit, one bit per leaf up to 1,824 leaves
// took their time down 4.7%; with it, the fine mask made 33 of the 35 slower and their
// total 9% longer (fewer resident blocks now cost more than the finer pruning saves), so
// it is off by default.
constexpr int kFineWordsMax = 64;
#ifndef CSG_FINE_WORDS_USE
#define CSG_FINE_WORDS_USE 0
#endif

struct DeviceScene {
    const int4* topo = nullptr;
    const float4* kids = nullptr;
    const float4* geo = nullptr;
    const float4* color = nullptr;
    const float4* lbox = nullptr;
    const float4* bvh = nullptr;
    int32_t n_nodes = 0;
    int32_t n_prims = 0;
    int32_t op_depth = 0;
    int32_t stack_class = 0;
    int32_t n_bvh = 0;        // BVH nodes (0: a single primitive, no BVH)
    int32_t live_words = 0;   // words of the per-ray live mask
    int32_t live_shift = 0;   // log2 of the leaves per live bit
    int32_t fine = 0;         // single-view renders use the fine mask below
    int32_t fine_words = 0;   // its words (at most kFineWordsMax)
    int32_t fine_shift = 0;   // its log2 of the leaves per bit
    int32_t prepass = 0;      // run the liveness pre-pass (scenes with enough leaves)
    int32_t rolled = 0;       // kernel variant: GoTo's tests in a rolled loop (see trace.cuh)
    int32_t short_circuit = 0;  // skip the other child of a Difference / Intersection decided by a Miss
    int32_t cylinders = 0;      // the tree holds a cylinder
};

// Host image of the device arrays (for upload and for tests).
struct PackedScene {
    std::vector<int4> topo;
    std::vector<float4> kids;
    std::vector<float4> geo;
    std::vector<float4> color;
    std::vector<float4> lbox;
    std::vector<float4> bvh;  // 4 * bvh_nodes slot records, then 2 * bvh_nodes bounding spheres
    int32_t bvh_nodes = 0;
    int32_t live_words = 0;
    int32_t live_shift = 0;
    int32_t fine = 0;
    int32_t fine_words = 0;
    int32_t fine_shift = 0;
};
void pack_scene(const HostTree& tree, PackedScene& out);

// Stack capacity class used by the kernels for a tree of this operator depth: the
// per-ray primitive and time stacks never hold more entries than the operator depth,
// and the action stack never more than 2 * depth + 1, so a tree with depth <= 15 never
// reaches the reference's 32-entry limit (RaycastingKernels.cuh:19).  Deeper trees use
// the 32-entry class, which reproduces the reference's drop-on-full behaviour.
int32_t stack_class_for_depth(int32_t op_depth);

// Whether renders of a scene with this many primitives run the liveness pre-pass (for a
// handful of primitives the pre-pass costs more than the pruning saves).
bool use_prepass(int32_t n_prims);

// Kernel variant for a tree: the rolled GoTo loop when the tree has more than two
// primitives, the unrolled one (which overlaps the two children's tests) for the smallest.
// The unrolled code of the primitive tests overflows the instruction cache: 1.7-2.3x slower
// on trees with cylinders, and since the single-leaf shortcut 14% slower on the cheese
// frame of spheres (instruction-fetch stalls the top stall reason).
bool use_rolled(const HostTree& tree);

// Whether the traversal short-circuits Difference and Intersection nodes decided by a Miss
// child (trace.cuh): for trees of which at least one operator in eight is a Difference or
// an Intersection.  Measured: 2.2-6x faster on random trees; on the cheese scene (one
// Difference over a 511-node Union) the extra tests in every GoTo cost 3-5% and saved
// nothing, so such trees keep the plain traversal.  The single-view kernel short-circuits
// in both GoTo variants; the batched view-table kernel only in the rolled one.
bool use_short_circuit(const HostTree& tree);

// Whether a packed tree can use the fine live mask (rolled variant, grouped own mask, one
// bit per leaf within kFineWordsMax words).
bool fine_mask_possible(const HostTree& tree, const PackedScene& pk);

}  // namespace csgrt
