// Scene text parser, bounding boxes and device-layout packer.
//
// Behaviour follows CSGTree::Parse (CSGRayCasting/Graphics/RayCasting/CSGTree/CSGTree.cu:5-152):
// whitespace tokens in preorder; an operator's first child becomes `left`, its second
// `right`; primitive parameters are read with the same C conversions std::stof / stod /
// stoi use, in the same order, so the same text produces the same bits and the same
// first error.  Where the reference indexes past the end of the token list (undefined
// behaviour) this parser reports CSG_E_PARSE instead.
#include "scene.hpp"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <utility>

namespace csgrt {
namespace {

bool is_space(char c)
{
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

std::vector<std::string_view> tokenize(std::string_view text)
{
    std::vector<std::string_view> toks;
    size_t i = 0;
    while (i < text.size()) {
        while (i < text.size() && is_space(text[i])) ++i;
        if (i >= text.size()) break;
        size_t j = i;
        while (j < text.size() && !is_space(text[j])) ++j;
        toks.emplace_back(text.substr(i, j - i));
        i = j;
    }
    return toks;
}

// std::stof: strtof, "no conversion" -> invalid_argument("stof"), ERANGE -> out_of_range.
int to_float(std::string_view tok, float& v, std::string& err)
{
    std::string s(tok);
    char* end = nullptr;
    const int saved = errno;
    errno = 0;
    v = std::strtof(s.c_str(), &end);
    const int e = errno;
    errno = saved;
    if (end == s.c_str()) { err = "stof"; return kErrParse; }
    if (e == ERANGE) { err = "stof"; return kErrRange; }
    return kOk;
}

int to_double(std::string_view tok, double& v, std::string& err)
{
    std::string s(tok);
    char* end = nullptr;
    const int saved = errno;
    errno = 0;
    v = std::strtod(s.c_str(), &end);
    const int e = errno;
    errno = saved;
    if (end == s.c_str()) { err = "stod"; return kErrParse; }
    if (e == ERANGE) { err = "stod"; return kErrRange; }
    return kOk;
}

// color(): std::stoi(two hex characters, nullptr, 16) / 255 (CSGTree.cu:196-200).
int to_channel(std::string_view two, float& v, std::string& err)
{
    std::string s(two);
    char* end = nullptr;
    const int saved = errno;
    errno = 0;
    const long x = std::strtol(s.c_str(), &end, 16);
    const int e = errno;
    errno = saved;
    if (end == s.c_str()) { err = "stoi"; return kErrParse; }
    if (e == ERANGE || x < INT32_MIN || x > INT32_MAX) { err = "stoi"; return kErrRange; }
    v = static_cast<float>(static_cast<int>(x)) / 255;
    return kOk;
}

// Cylinder axis (Primitives.h:54-88): R(rotX, rotY, rotZ) * (0, 1, 0) in double,
// divided by its squared length, rounded to float.
void cylinder_axis(double rx, double ry, double rz, float* axis)
{
    const double deg = 0.017453292519943295769236907684886;
    rx = rx * deg;
    ry = ry * deg;
    rz = rz * deg;
    double x = -std::sin(rz) * std::cos(ry) + std::sin(ry) * std::sin(rx) * std::cos(rz);
    double y = std::cos(rx) * std::cos(rz);
    double z = std::sin(ry) * std::sin(rz) + std::sin(rx) * std::cos(ry) * std::cos(rz);
    const double len2 = (x * x + y * y + z * z);
    x /= len2;
    y /= len2;
    z /= len2;
    axis[0] = static_cast<float>(x);
    axis[1] = static_cast<float>(y);
    axis[2] = static_cast<float>(z);
}

// Leaf bounding boxes (BVHNode.cuh:17-52): sphere +-2r as (c - r) - r, cylinder
// +-max(h/2, r), cube +-edge/2.
void leaf_box(RefNode& n, const RefPrim& p)
{
    const float c[3] = {p.x, p.y, p.z};
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (n.type == kSphere) {
        const float r = p.p[0];
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - r - r; hi[k] = c[k] + r + r; }
    } else if (n.type == kCylinder) {
        const float h2 = p.p[1] / 2, r = p.p[0];
        const float m = (h2 < r) ? r : h2;
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - m; hi[k] = c[k] + m; }
    } else if (n.type == kCube) {
        const float hs = p.p[0] / 2;
        for (int k = 0; k < 3; ++k) { lo[k] = c[k] - hs; hi[k] = c[k] + hs; }
    }
    n.minx = lo[0]; n.miny = lo[1]; n.minz = lo[2];
    n.maxx = hi[0]; n.maxy = hi[1]; n.maxz = hi[2];
}

// Exact-box mode: boxes that contain their primitive, instead of the reference's ±2r
// sphere boxes and its cylinder boxes (BVHNode.cuh:19-49), which are not conservative
// and cut hits.  A sphere gets ±r; a cylinder about axis V with half-height h/2 gets, per
// axis, |V_k| h/2 + r sqrt(1 - V_k^2); both widened by 2^-12 of their size plus 1e-5 so
// that the rounded hit points of the primitive tests stay inside; a cube keeps its own
// box (already exact).  The oracle computes the same floats (oracle/csg_oracle.c,
// orc_boxes_exact).
void leaf_box_exact(RefNode& n, const RefPrim& p)
{
    if (n.type != kSphere && n.type != kCylinder) {
        leaf_box(n, p);
        return;
    }
    const float c[3] = {p.x, p.y, p.z};
    float e[3];
    if (n.type == kSphere) {
        const float r = p.p[0];
        for (int k = 0; k < 3; ++k) e[k] = r;
    } else {
        const float r = p.p[0], h2 = p.p[1] * 0.5f;
        for (int k = 0; k < 3; ++k) {
            const float v = p.p[2 + k];
            const float s = 1.0f - v * v;
            e[k] = std::fabs(v) * h2 + r * std::sqrt(s > 0.0f ? s : 0.0f);
        }
    }
    for (int k = 0; k < 3; ++k) e[k] = e[k] + e[k] * 0.000244140625f + 1e-5f;
    n.minx = c[0] - e[0]; n.miny = c[1] - e[1]; n.minz = c[2] - e[2];
    n.maxx = c[0] + e[0]; n.maxy = c[1] + e[1]; n.maxz = c[2] + e[2];
}

// Operator boxes (BVHNode.cuh:54-63) with std::min / std::max semantics.
inline float min_ref(float a, float b) { return (b < a) ? b : a; }
inline float max_ref(float a, float b) { return (a < b) ? b : a; }

void build_boxes(HostTree& t, bool exact = false)
{
    // Children always follow their parent in preorder, so a reverse sweep visits every
    // child before its parent.
    for (int i = static_cast<int>(t.nodes.size()) - 1; i >= 0; --i) {
        RefNode& n = t.nodes[i];
        if (n.prim != -1) {
            if (exact) leaf_box_exact(n, t.prims[n.prim]);
            else leaf_box(n, t.prims[n.prim]);
        } else {
            const RefNode& l = t.nodes[n.left];
            const RefNode& r = t.nodes[n.right];
            n.minx = min_ref(l.minx, r.minx); n.miny = min_ref(l.miny, r.miny);
            n.minz = min_ref(l.minz, r.minz);
            n.maxx = max_ref(l.maxx, r.maxx); n.maxy = max_ref(l.maxy, r.maxy);
            n.maxz = max_ref(l.maxz, r.maxz);
        }
    }
}

int32_t operator_depth(const HostTree& t)
{
    std::vector<int32_t> d(t.nodes.size(), 0);
    int32_t best = 0;
    for (size_t i = 0; i < t.nodes.size(); ++i) {
        const RefNode& n = t.nodes[i];
        const int32_t here = (n.parent >= 0 ? d[n.parent] : 0) + (n.prim == -1 ? 1 : 0);
        d[i] = here;
        if (here > best) best = here;
    }
    return best;
}

}  // namespace

int parse_tree(std::string_view text, HostTree& out, std::string& err)
{
    out = HostTree{};
    err.clear();
    const std::vector<std::string_view> toks = tokenize(text);
    struct Open { int32_t node; int32_t children; };
    std::vector<Open> open;
    auto& nodes = out.nodes;
    auto& prims = out.prims;
    nodes.reserve(toks.size());

    for (size_t i = 0; i < toks.size(); ++i) {
        const int32_t id = static_cast<int32_t>(nodes.size());
        nodes.push_back(RefNode{-1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0});
        if (id != 0) {
            if (open.empty()) { err = "Cannot parse"; return kErrParse; }
            Open& top = open.back();
            nodes[id].parent = top.node;
            if (top.children == 0) {
                nodes[top.node].left = id;
                top.children = 1;
            } else {
                nodes[top.node].right = id;
                open.pop_back();
            }
        }
        const std::string_view kw = toks[i];
        int32_t type;
        if (kw == "Union") type = kUnion;
        else if (kw == "Difference") type = kDifference;
        else if (kw == "Intersection") type = kIntersection;
        else if (kw == "Sphere") type = kSphere;
        else if (kw == "Cylinder") type = kCylinder;
        else if (kw == "Cube") type = kCube;
        else {
            err = "Cannot parse - Unrecognized keyword: " + std::string(kw);
            return kErrParse;
        }
        nodes[id].type = type;
        if (type <= kIntersection) {
            open.push_back({id, 0});
            continue;
        }

        auto param = [&](size_t k, std::string_view& tok) -> bool {
            if (i + k >= toks.size()) {
                err = "Cannot parse - missing parameters after " + std::string(kw);
                return false;
            }
            tok = toks[i + k];
            return true;
        };
        RefPrim p{};
        p.id = static_cast<int32_t>(prims.size());
        std::string_view tok;
        float xyz[3];
        for (int k = 0; k < 3; ++k) {
            if (!param(1 + k, tok)) return kErrParse;
            if (int rc = to_float(tok, xyz[k], err)) return rc;
        }
        if (!param(4, tok)) return kErrParse;
        if (tok.size() != 6) {
            err = "Cannot parse color " + std::string(tok);
            return kErrParse;
        }
        float rgb[3];
        for (int k = 0; k < 3; ++k)
            if (int rc = to_channel(tok.substr(2 * k, 2), rgb[k], err)) return rc;
        p.x = xyz[0]; p.y = xyz[1]; p.z = xyz[2];
        p.r = rgb[0]; p.g = rgb[1]; p.b = rgb[2];
        size_t consumed = 5;
        if (type == kSphere || type == kCube) {
            if (!param(5, tok)) return kErrParse;
            if (int rc = to_float(tok, p.p[0], err)) return rc;
        } else {
            if (!param(5, tok)) return kErrParse;
            if (int rc = to_float(tok, p.p[0], err)) return rc;
            if (!param(6, tok)) return kErrParse;
            if (int rc = to_float(tok, p.p[1], err)) return rc;
            double rot[3];
            for (int k = 0; k < 3; ++k) {
                if (!param(7 + k, tok)) return kErrParse;
                if (int rc = to_double(tok, rot[k], err)) return rc;
            }
            static const char* const kRotMsg[3] = {
                "Invalid roation rotX should be in range [0, 360] deg",
                "Invalid roation rotY should be in range [0, 360] deg",
                "Invalid roation rotZ should be in range [0, 360] deg"};
            for (int k = 0; k < 3; ++k)
                if (rot[k] > 360 || rot[k] < 0) { err = kRotMsg[k]; return kErrRange; }
            cylinder_axis(rot[0], rot[1], rot[2], &p.p[2]);
            consumed = 9;
        }
        nodes[id].prim = p.id;
        prims.push_back(p);
        i += consumed;
    }
    if (nodes.size() != 2 * prims.size() - 1 || prims.empty()) {
        err = "Cannot parse - number of primitives do not match number of nodes";
        return kErrCount;
    }
    if (prims.size() > 32767) {
        // RayHitMinimal keeps the primitive index in a short (Ray.cuh:36-52).
        err = "scene has more than 32767 primitives";
        return kErrDepth;
    }
    build_boxes(out);
    out.op_depth = operator_depth(out);
    out.leaf_lo.assign(nodes.size(), 0);
    out.leaf_hi.assign(nodes.size(), 0);
    for (int i = static_cast<int>(nodes.size()) - 1; i >= 0; --i) {
        if (nodes[i].prim != -1) {
            out.leaf_lo[i] = out.leaf_hi[i] = nodes[i].prim;
        } else {
            out.leaf_lo[i] = out.leaf_lo[nodes[i].left];
            out.leaf_hi[i] = out.leaf_hi[nodes[i].right];
        }
    }
    return kOk;
}

void use_exact_boxes(HostTree& t)
{
    build_boxes(t, true);
}

// Build-time tuning knob: smallest tree (in primitives) that runs the liveness pre-pass.
// From two primitives on (it was eight): with the empty-mask skip a ray that meets no
// primitive ends after the pre-pass, and the README tree (5 primitives) took 14% less time,
// random trees of 2-6 primitives 11-33% less (with the rolled variant from 3 primitives).
#ifndef CSG_PREPASS_MIN_PRIMS
#define CSG_PREPASS_MIN_PRIMS 2
#endif
bool use_prepass(int32_t n_prims) { return n_prims >= CSG_PREPASS_MIN_PRIMS; }

// Build-time tuning knobs: trees with cylinders and more primitives than
// CSG_ROLLED_MIN_PRIMS use the rolled kernel variant; trees without cylinders do too when
// CSG_ROLLED_WITHOUT_CYLINDERS is 1.
#ifndef CSG_ROLLED_WITHOUT_CYLINDERS
#define CSG_ROLLED_WITHOUT_CYLINDERS 1
#endif
#ifndef CSG_ROLLED_MIN_PRIMS
#define CSG_ROLLED_MIN_PRIMS 2
#endif
bool use_rolled(const HostTree& tree)
{
    if (tree.prims.size() <= (size_t)CSG_ROLLED_MIN_PRIMS) return false;
    if (CSG_ROLLED_WITHOUT_CYLINDERS) return true;
    for (const RefNode& n : tree.nodes)
        if (n.type == kCylinder) return true;
    return false;
}

bool use_short_circuit(const HostTree& tree)
{
    size_t ops = 0, decisive = 0;
    for (const RefNode& n : tree.nodes) {
        if (n.prim != -1) continue;
        ++ops;
        if (n.type == kDifference || n.type == kIntersection) ++decisive;
    }
    return 8 * decisive >= ops;
}

bool fine_mask_possible(const HostTree& tree, const PackedScene& pk)
{
    return use_rolled(tree) && pk.live_shift > 0 && pk.fine_shift == 0;
}

int32_t stack_class_for_depth(int32_t op_depth)
{
    if (op_depth <= 4) return 4;
    if (op_depth <= 8) return 8;
    if (op_depth <= 12) return 12;
    if (op_depth <= 15) return 16;
    return 32;
}

namespace {
inline float as_float(int32_t v)
{
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}
}  // namespace

namespace {

struct Box {
    float lo[3], hi[3];
};

// Binned-SAH BVH over the leaves' boxes.  Each internal node stores both children's
// boxes; a child that is a single leaf stores that leaf's own (reference) box, and an
// internal child stores the exact min/max of its leaves' boxes, so every stored box
// contains the boxes below it.
struct BvhBuilder {
    const std::vector<Box>& box;
    const std::vector<int32_t>& type;
    std::vector<float4>& out;
    std::vector<int32_t> idx;

    static float area(const Box& b)
    {
        const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    Box bounds(int a, int b) const
    {
        Box r{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
        for (int i = a; i < b; ++i)
            for (int k = 0; k < 3; ++k) {
                const Box& x = box[idx[i]];
                r.lo[k] = x.lo[k] < r.lo[k] ? x.lo[k] : r.lo[k];
                r.hi[k] = x.hi[k] > r.hi[k] ? x.hi[k] : r.hi[k];
            }
        return r;
    }
    int split(int a, int b)
    {
        // centroid bounds
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = a; i < b; ++i)
            for (int k = 0; k < 3; ++k) {
                const float c = 0.5f * (box[idx[i]].lo[k] + box[idx[i]].hi[k]);
                clo[k] = c < clo[k] ? c : clo[k];
                chi[k] = c > chi[k] ? c : chi[k];
            }
        constexpr int kBins = 16;
        float best = INFINITY;
        int best_axis = -1;
        float best_cut = 0;
        for (int k = 0; k < 3; ++k) {
            const float ext = chi[k] - clo[k];
            if (!(ext > 0)) continue;
            int cnt[kBins] = {0};
            Box bb[kBins];
            for (auto& x : bb) x = Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
            for (int i = a; i < b; ++i) {
                const Box& x = box[idx[i]];
                const float c = 0.5f * (x.lo[k] + x.hi[k]);
                int bi = static_cast<int>((c - clo[k]) / ext * kBins);
                bi = bi < 0 ? 0 : (bi >= kBins ? kBins - 1 : bi);
                cnt[bi]++;
                for (int q = 0; q < 3; ++q) {
                    bb[bi].lo[q] = x.lo[q] < bb[bi].lo[q] ? x.lo[q] : bb[bi].lo[q];
                    bb[bi].hi[q] = x.hi[q] > bb[bi].hi[q] ? x.hi[q] : bb[bi].hi[q];
                }
            }
            for (int cut = 1; cut < kBins; ++cut) {
                Box L{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}}, R = L;
                int nl = 0, nr = 0;
                for (int q = 0; q < kBins; ++q) {
                    Box& T = q < cut ? L : R;
                    (q < cut ? nl : nr) += cnt[q];
                    if (!cnt[q]) continue;
                    for (int z = 0; z < 3; ++z) {
                        T.lo[z] = bb[q].lo[z] < T.lo[z] ? bb[q].lo[z] : T.lo[z];
                        T.hi[z] = bb[q].hi[z] > T.hi[z] ? bb[q].hi[z] : T.hi[z];
                    }
                }
                if (!nl || !nr) continue;
                const float cost = area(L) * nl + area(R) * nr;
                if (cost < best) {
                    best = cost;
                    best_axis = k;
                    best_cut = clo[k] + ext * cut / kBins;
                }
            }
        }
        int mid = a;
        if (best_axis >= 0) {
            for (int i = a; i < b; ++i) {
                const Box& x = box[idx[i]];
                if (0.5f * (x.lo[best_axis] + x.hi[best_axis]) < best_cut) std::swap(idx[i], idx[mid++]);
            }
        }
        if (mid == a || mid == b) mid = (a + b) / 2;  // degenerate: split by count
        return mid;
    }
    static float as_float(int32_t v)
    {
        float f;
        std::memcpy(&f, &v, 4);
        return f;
    }
    void child(int node, int side, int a, int b, int32_t child_index)
    {
        const Box bb = bounds(a, b);
        const bool leaf = (b - a == 1);
        const int32_t c = leaf ? ~idx[a] : child_index;
        const int32_t ty = leaf ? type[idx[a]] : -1;
        out[4 * node + 2 * side + 0] = float4{bb.lo[0], bb.lo[1], bb.lo[2], as_float(c)};
        out[4 * node + 2 * side + 1] = float4{bb.hi[0], bb.hi[1], bb.hi[2], as_float(ty)};
    }
    // Builds the node for leaves [a, b) (b - a >= 2) at index `node`.
    void build(int node, int a, int b)
    {
        const int mid = split(a, b);
        int lchild = -1, rchild = -1;
        if (mid - a >= 2) {
            lchild = static_cast<int>(out.size() / 4);
            out.resize(out.size() + 4);
        }
        if (b - mid >= 2) {
            rchild = static_cast<int>(out.size() / 4);
            out.resize(out.size() + 4);
        }
        child(node, 0, a, mid, lchild);
        child(node, 1, mid, b, rchild);
        if (lchild >= 0) build(lchild, a, mid);
        if (rchild >= 0) build(rchild, mid, b);
    }
};

}  // namespace

void pack_scene(const HostTree& t, PackedScene& out)
{
    const size_t n = t.nodes.size(), np = t.prims.size();
    const bool rolled = use_rolled(t);
    // Device node numbering: the operators first, in preorder (the root, node 0 of the
    // reference, stays 0), then the leaves.  Only operators have kids records, so those are
    // dense and a cache line holds only records the traversal reads.
    std::vector<int32_t> num(n, -1);
    int32_t next = 0;
    for (size_t i = 0; i < n; ++i)
        if (t.nodes[i].prim == -1 || !CSG_DENSE_OPERATORS) num[i] = next++;
    const size_t n_ops = static_cast<size_t>(CSG_DENSE_OPERATORS ? next : n);
    for (size_t i = 0; i < n; ++i)
        if (num[i] < 0) num[i] = next++;
    auto dev = [&](int32_t old) { return old < 0 ? old : num[old]; };
    // Traversal order of Intersections: Kensler's Intersection table (RaycastingKernels.cu:
    // 670-673) is symmetric in its two children, ties included, so the device tree may
    // list them in either order with the same results (leaf ranges stay contiguous, so the
    // live mask and the primitive numbers are unchanged).  With the operator short-circuit
    // a Miss from the child traversed first skips the other, so an Intersection of two
    // operators puts the child with fewer leaves first: 20% fewer iterations on the
    // batched workload's random trees (oracle, live-leaf pruning and short-circuit on).
    const bool reorder = use_short_circuit(t) && t.op_depth <= 15;
    auto n_leaves = [&](int32_t i) { return t.leaf_hi[i] - t.leaf_lo[i] + 1; };
    // Depths (operators above a node) and, per leaf, the depth of the deepest operator
    // above it that does not pass the leaf's record up when the rest of its subtree is a
    // Miss: an Intersection, or a Difference entered on its right (the single-leaf
    // shortcut in trace.cuh).  Preorder lists parents before children.
    std::vector<int32_t> depth(n, 0), blk(n, -1);
    for (size_t i = 0; i < n; ++i) {
        const int32_t p = t.nodes[i].parent;
        if (p < 0) continue;
        depth[i] = depth[p] + 1;
        const RefNode& pn = t.nodes[p];
        const bool passes = pn.type == kUnion || (pn.type == kDifference && pn.left == static_cast<int32_t>(i));
        blk[i] = passes ? blk[p] : depth[p];
    }
    // Operator heights (0 for a leaf; children follow their parents in preorder).  Trees
    // deeper than 15 operator levels carry each operator's height, up to 127, in bits 24-30
    // of the left child's leaf_hi word: the 32-entry stack class skips work under an
    // operator only where its height leaves the stacks room (trace.cuh, kGuard).
    std::vector<int32_t> height(n, 0);
    for (size_t i = n; i-- > 0;)
        if (t.nodes[i].prim == -1) height[i] = 1 + std::max(height[t.nodes[i].left], height[t.nodes[i].right]);
    const bool deep = t.op_depth > 15;
    out.topo.assign(n, int4{0, 0, 0, 0});
    out.kids.assign(kKidsPerNode * std::max<size_t>(n_ops, 1), float4{0, 0, 0, 0});
    out.geo.assign(2 * np, float4{0, 0, 0, 0});
    out.color.assign(np, float4{0, 0, 0, 0});
    for (size_t i = 0; i < n; ++i) {
        const RefNode& nd = t.nodes[i];
        if (nd.prim != -1) {
            out.topo[num[i]] = int4{nd.prim, -1, dev(nd.parent), nd.type};
            continue;
        }
        int32_t li = nd.left, ri = nd.right;
        if (reorder && nd.type == kIntersection && t.nodes[li].prim == -1 && t.nodes[ri].prim == -1 &&
            n_leaves(ri) < n_leaves(li))
            std::swap(li, ri);
        out.topo[num[i]] = int4{dev(li), dev(ri), dev(nd.parent), nd.type};
        const RefNode& l = t.nodes[li];
        const RefNode& r = t.nodes[ri];
        float4* k = &out.kids[kKidsPerNode * num[i]];
        k[0] = float4{l.minx, l.miny, l.minz, as_float(l.type)};
        k[1] = float4{l.maxx, l.maxy, l.maxz, as_float(l.prim)};
        k[2] = float4{r.minx, r.miny, r.minz, as_float(r.type)};
        k[3] = float4{r.maxx, r.maxy, r.maxz, as_float(r.prim)};
        // Bit 30 of the left child's leaf_lo: test the right child first.  Operator
        // children come before leaves and leaves go sphere, cube, cylinder, so that lanes of
        // a warp at different nodes run the same kind of test together (the two tests are
        // independent: disjoint leaf ranges, separate hit records).
        auto prio = [](const RefNode& c) { return c.prim == -1 ? 0 : c.type == kSphere ? 1 : c.type == kCube ? 2 : 3; };
        const int32_t swap = prio(r) < prio(l) ? (1 << 30) : 0;
        const int32_t dc = std::min<int32_t>(depth[i] + 1, 255);
        const int32_t hb = deep ? std::min<int32_t>(height[i], 127) << 24 : 0;
        k[4] = float4{as_float(t.leaf_lo[li] | swap), as_float(t.leaf_hi[li] | (dc << 16) | hb),
                      as_float(t.leaf_lo[ri]), as_float(t.leaf_hi[ri])};
    }
    // live-mask granularity: one bit per 2^shift leaves, at most kLiveWordsMax words
    int32_t shift = 0;
    while (((static_cast<int64_t>(np) + (1 << shift) - 1) >> shift) > 32 * kLiveWordsMax) ++shift;
    out.live_shift = shift;
    out.live_words = static_cast<int32_t>((((np + (1u << shift) - 1) >> shift) + 31) / 32);
    int32_t fshift = 0;
    while (((static_cast<int64_t>(np) + (1 << fshift) - 1) >> fshift) > 32 * kFineWordsMax) ++fshift;
    out.fine_shift = fshift;
    out.fine_words = static_cast<int32_t>((((np + (1u << fshift) - 1) >> fshift) + 31) / 32);
    out.fine = (rolled && shift > 0 && fshift == 0 && out.fine_words <= CSG_FINE_WORDS_USE) ? 1 : 0;
    // BVH over the leaves' reference boxes (primitive order -> node order)
    out.bvh.clear();
    if (np >= 2) {
        std::vector<Box> boxes(np);
        std::vector<int32_t> types(np);
        for (size_t i = 0; i < n; ++i) {
            const RefNode& nd = t.nodes[i];
            if (nd.prim == -1) continue;
            boxes[nd.prim] = Box{{nd.minx, nd.miny, nd.minz}, {nd.maxx, nd.maxy, nd.maxz}};
            types[nd.prim] = nd.type;
        }
        BvhBuilder b{boxes, types, out.bvh, {}};
        b.idx.resize(np);
        for (size_t i = 0; i < np; ++i) b.idx[i] = static_cast<int32_t>(i);
        out.bvh.resize(4);
        b.build(0, 0, static_cast<int>(np));
        // bounding spheres of the slots, for the pre-pass's warp-wide cone test
        const size_t nb = out.bvh.size() / 4;
        out.bvh_nodes = static_cast<int32_t>(nb);
        for (size_t e = 0; e < 2 * nb; ++e) {
            const float4 lo = out.bvh[2 * e], hi = out.bvh[2 * e + 1];
            int32_t child, ty;
            std::memcpy(&child, &lo.w, 4);
            std::memcpy(&ty, &hi.w, 4);
            if (child < 0 && ty == kSphere) {
                const RefPrim& p = t.prims[static_cast<size_t>(~child)];
                out.bvh.push_back(float4{p.x, p.y, p.z, -std::fabs(p.p[0])});
                continue;
            }
            const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
            float c[3];
            double r2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                c[k] = static_cast<float>(0.5 * (static_cast<double>(l[k]) + static_cast<double>(h[k])));
                const double d = std::max(std::fabs(static_cast<double>(l[k]) - c[k]), std::fabs(static_cast<double>(h[k]) - c[k]));
                r2 += d * d;
            }
            float r = static_cast<float>(std::sqrt(r2));
            if (static_cast<double>(r) < std::sqrt(r2)) r = std::nextafter(r, INFINITY);
            if (!std::isfinite(r) || !std::isfinite(c[0]) || !std::isfinite(c[1]) || !std::isfinite(c[2]))
                r = INFINITY;  // (a non-finite box always passes)
            out.bvh.push_back(float4{c[0], c[1], c[2], r});
        }
    }
    out.lbox.assign(2 * np, float4{0, 0, 0, 0});
    for (size_t i = 0; i < n; ++i) {
        const RefNode& nd = t.nodes[i];
        if (nd.prim == -1) continue;
        const int32_t b = std::min<int32_t>(blk[i] + 1, 255);
        out.lbox[2 * nd.prim + 0] = float4{nd.minx, nd.miny, nd.minz, as_float(nd.type)};
        out.lbox[2 * nd.prim + 1] = float4{nd.maxx, nd.maxy, nd.maxz, as_float(nd.prim | (b << 16))};
    }
    for (size_t i = 0; i < np; ++i) {
        const RefPrim& p = t.prims[i];
        out.geo[2 * i + 0] = float4{p.x, p.y, p.z, p.p[0]};
        out.geo[2 * i + 1] = float4{p.p[1], p.p[2], p.p[3], p.p[4]};
        out.color[i] = float4{p.r, p.g, p.b, 0.f};
    }
}

}  // namespace csgrt
