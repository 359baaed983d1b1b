// C ABI of the CSG ray-casting engine (include/csgrt.h): scene lifecycle, camera and
// light math, render entry points.  Host code; compiled with -ffp-contract=off so the
// camera arithmetic is the reference's separately rounded float sequence on every host.
#include "csgrt.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "render.hpp"
#include "scene.hpp"
#include "scene_handle.hpp"


namespace {

void copy_err(char* err, size_t errlen, const std::string& msg)
{
    if (!err || errlen == 0) return;
    const size_t n = msg.size() < errlen - 1 ? msg.size() : errlen - 1;
    std::memcpy(err, msg.data(), n);
    err[n] = 0;
}

size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// Camera::normalizeVector (Camera.cpp:29-36); the float sum's square root is taken in
// double (global sqrt) and rounded to float, which equals the float square root.
void normalize_vec(float* v)
{
    const float length = static_cast<float>(std::sqrt(static_cast<double>(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])));
    if (length > 0) {
        v[0] /= length;
        v[1] /= length;
        v[2] /= length;
    }
}

// Camera::updateVectors (Camera.cpp:4-27).  Camera.cpp includes only <cmath>, so its
// unqualified sin/cos of a float argument resolve to the global double functions: each
// basis component is computed in double and rounded to float on assignment.
void update_vectors(csg_camera* c)
{
    const double px = c->rot_x, yw = c->rot_y;
    c->forward[0] = static_cast<float>(-std::sin(yw) * std::cos(px));
    c->forward[1] = static_cast<float>(std::sin(px));
    c->forward[2] = static_cast<float>(-std::cos(yw) * std::cos(px));
    normalize_vec(c->forward);
    c->right[0] = static_cast<float>(std::cos(yw));
    c->right[1] = 0;
    c->right[2] = static_cast<float>(-std::sin(yw));
    normalize_vec(c->right);
    const float* f = c->forward;
    const float* r = c->right;
    c->up[0] = f[1] * r[2] - f[2] * r[1];
    c->up[1] = f[2] * r[0] - f[0] * r[2];
    c->up[2] = f[0] * r[1] - f[1] * r[0];
    normalize_vec(c->up);
}

int render_common(const csg_scene* s, const csg_camera* cam, const float light[3], int32_t w, int32_t h,
                  const csgrt::Planes& planes, void* stream, bool host_out = false)
{
    if (!s || !cam || !light || w <= 0 || h <= 0) return CSG_E_ARG;
    if (planes.rgba32f && (reinterpret_cast<uintptr_t>(planes.rgba32f) & 15u)) return CSG_E_ARG;
    static_assert(sizeof(csg_camera) == sizeof(csgrt::Camera), "camera layout");
    csgrt::Camera c;
    std::memcpy(c.v, cam, sizeof(c.v));
    const cudaError_t e = csgrt::launch_render(s->dev, s->center, c, light, w, h, planes, s->status,
                                               static_cast<cudaStream_t>(stream), host_out, &s->dispatch);
    return e == cudaSuccess ? CSG_OK : CSG_E_CUDA;
}

}  // namespace

extern "C" {

int csg_abi_version(void) { return CSGRT_ABI_VERSION; }

const char* csg_status_string(int status)
{
    switch (status) {
        case CSG_OK: return "ok";
        case CSG_E_PARSE: return "scene text could not be parsed";
        case CSG_E_RANGE: return "value out of range";
        case CSG_E_COUNT: return "number of primitives does not match number of nodes";
        case CSG_E_CUDA: return "CUDA runtime error";
        case CSG_E_BUDGET: return "device-memory budget exceeded";
        case CSG_E_TIMEOUT: return "bounded wait or traversal cap reached";
        case CSG_E_DEPTH: return "scene too large for the device layout";
        case CSG_E_ARG: return "invalid argument";
        case CSG_E_CAPACITY: return "output array too small";
        default: return "unknown status";
    }
}

}  // extern "C"

csgrt::SceneLayout csgrt::scene_layout(size_t n_nodes, size_t n_prims, size_t n_kids_f4, size_t n_bvh_f4)
{
    SceneLayout l;
    l.topo = 0;
    l.kids = align16(l.topo + n_nodes * sizeof(int4));
    l.geo = align16(l.kids + n_kids_f4 * sizeof(float4));
    l.color = align16(l.geo + 2 * n_prims * sizeof(float4));
    l.lbox = align16(l.color + n_prims * sizeof(float4));
    l.bvh = align16(l.lbox + 2 * n_prims * sizeof(float4));
    l.status = align16(l.bvh + n_bvh_f4 * sizeof(float4));
    l.total = align16(l.status + sizeof(unsigned long long));
    return l;
}

extern "C" {

int csg_scene_create(const char* text, size_t len, csg_scene** out, char* err, size_t errlen)
{
    return csg_scene_create_ex(text, len, 0, out, err, errlen);
}

int csg_scene_create_ex(const char* text, size_t len, int32_t flags, csg_scene** out, char* err, size_t errlen)
{
    if (!out) return CSG_E_ARG;
    if (flags & ~(CSG_SCENE_EXACT_BOXES | CSG_SCENE_FINE_MASK)) return CSG_E_ARG;
    *out = nullptr;
    if (!text && len) return CSG_E_ARG;
    csg_scene* s = new (std::nothrow) csg_scene();
    if (!s) return CSG_E_CUDA;
    std::string msg;
    const int rc = csgrt::parse_tree(std::string_view(text ? text : "", len), s->tree, msg);
    if (rc != csgrt::kOk) {
        copy_err(err, errlen, msg);
        delete s;
        return rc;
    }
    if (flags & CSG_SCENE_EXACT_BOXES) csgrt::use_exact_boxes(s->tree);
    csgrt::PackedScene pk;
    csgrt::pack_scene(s->tree, pk);
    const size_t n = s->tree.nodes.size(), np = s->tree.prims.size();
    const csgrt::SceneLayout lay = csgrt::scene_layout(n, np, pk.kids.size(), pk.bvh.size());
    const size_t off_topo = lay.topo, off_kids = lay.kids, off_geo = lay.geo, off_color = lay.color;
    const size_t off_bvh = lay.bvh, off_status = lay.status, total = lay.total;
    cudaGetDevice(&s->device);
    cudaError_t e = cudaMalloc(&s->dmem, total);
    if (e != cudaSuccess) {
        copy_err(err, errlen, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        delete s;
        return CSG_E_CUDA;
    }
    char* base = static_cast<char*>(s->dmem);
    e = cudaMemcpy(base + off_topo, pk.topo.data(), n * sizeof(int4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + off_kids, pk.kids.data(), pk.kids.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !pk.bvh.empty())
        e = cudaMemcpy(base + off_bvh, pk.bvh.data(), pk.bvh.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + off_geo, pk.geo.data(), 2 * np * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + off_color, pk.color.data(), np * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + lay.lbox, pk.lbox.data(), 2 * np * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(base + off_status, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        copy_err(err, errlen, std::string("scene upload: ") + cudaGetErrorString(e));
        cudaFree(s->dmem);
        delete s;
        return CSG_E_CUDA;
    }
    s->bytes = total;
    s->dev.topo = reinterpret_cast<const int4*>(base + off_topo);
    s->dev.kids = reinterpret_cast<const float4*>(base + off_kids);
    s->dev.geo = reinterpret_cast<const float4*>(base + off_geo);
    s->dev.color = reinterpret_cast<const float4*>(base + off_color);
    s->dev.lbox = reinterpret_cast<const float4*>(base + lay.lbox);
    s->dev.n_nodes = static_cast<int32_t>(n);
    s->dev.n_prims = static_cast<int32_t>(np);
    s->dev.op_depth = s->tree.op_depth;
    s->dev.stack_class = csgrt::stack_class_for_depth(s->tree.op_depth);
    s->dev.bvh = reinterpret_cast<const float4*>(base + off_bvh);
    s->dev.n_bvh = pk.bvh_nodes;
    s->dev.live_words = pk.live_words;
    s->dev.live_shift = pk.live_shift;
    s->dev.fine = (pk.fine || ((flags & CSG_SCENE_FINE_MASK) && csgrt::fine_mask_possible(s->tree, pk))) ? 1 : 0;
    s->dev.fine_words = pk.fine_words;
    s->dev.fine_shift = pk.fine_shift;
    s->dev.prepass = csgrt::use_prepass(static_cast<int32_t>(np)) ? 1 : 0;
    s->dev.rolled = csgrt::use_rolled(s->tree) ? 1 : 0;
    s->dev.short_circuit = csgrt::use_short_circuit(s->tree) ? 1 : 0;
    if (!s->tree.nodes.empty()) {
        const csgrt::RefNode& r = s->tree.nodes[0];
        s->center[0] = 0.5f * (r.minx + r.maxx);
        s->center[1] = 0.5f * (r.miny + r.maxy);
        s->center[2] = 0.5f * (r.minz + r.maxz);
    }
    s->dev.cylinders = 0;
    for (const csgrt::RefNode& nd : s->tree.nodes)
        if (nd.type == csgrt::kCylinder) s->dev.cylinders = 1;
    s->status = reinterpret_cast<unsigned long long*>(base + off_status);
    *out = s;
    return CSG_OK;
}

int csg_tree_plan(const char* text, size_t len, int32_t flags, csg_scene_info* info, char* err, size_t errlen)
{
    if (!info || (!text && len)) return CSG_E_ARG;
    if (flags & ~(CSG_SCENE_EXACT_BOXES | CSG_SCENE_FINE_MASK)) return CSG_E_ARG;
    csgrt::HostTree tree;
    std::string msg;
    const int rc = csgrt::parse_tree(std::string_view(text ? text : "", len), tree, msg);
    if (rc != csgrt::kOk) {
        copy_err(err, errlen, msg);
        return rc;
    }
    if (flags & CSG_SCENE_EXACT_BOXES) csgrt::use_exact_boxes(tree);
    csgrt::PackedScene pk;
    csgrt::pack_scene(tree, pk);
    const size_t n = tree.nodes.size(), np = tree.prims.size();
    *info = csg_scene_info{};
    info->n_nodes = static_cast<int32_t>(n);
    info->n_prims = static_cast<int32_t>(np);
    info->op_depth = tree.op_depth;
    info->stack_class = csgrt::stack_class_for_depth(tree.op_depth);
    info->device_bytes = csgrt::scene_layout(n, np, pk.kids.size(), pk.bvh.size()).total;
    info->rolled = csgrt::use_rolled(tree) ? 1 : 0;
    info->live_words = pk.live_words;
    info->live_shift = pk.live_shift;
    const bool fine = pk.fine || ((flags & CSG_SCENE_FINE_MASK) && csgrt::fine_mask_possible(tree, pk));
    info->fine_words = fine ? pk.fine_words : 0;
    info->short_circuit = csgrt::use_short_circuit(tree) ? 1 : 0;
    return CSG_OK;
}

int csg_tree_parse(const char* text, size_t len, void* nodes44, int32_t max_nodes, void* prims48,
                   int32_t max_prims, int32_t* n_nodes, int32_t* n_prims, int32_t* op_depth,
                   char* err, size_t errlen)
{
    return csg_tree_parse_ex(text, len, 0, nodes44, max_nodes, prims48, max_prims, n_nodes, n_prims, op_depth,
                             err, errlen);
}

int csg_tree_parse_ex(const char* text, size_t len, int32_t flags, void* nodes44, int32_t max_nodes,
                      void* prims48, int32_t max_prims, int32_t* n_nodes, int32_t* n_prims, int32_t* op_depth,
                      char* err, size_t errlen)
{
    if (!text && len) return CSG_E_ARG;
    if (flags & ~(CSG_SCENE_EXACT_BOXES | CSG_SCENE_FINE_MASK)) return CSG_E_ARG;
    csgrt::HostTree tree;
    std::string msg;
    const int rc = csgrt::parse_tree(std::string_view(text ? text : "", len), tree, msg);
    if (rc != csgrt::kOk) {
        copy_err(err, errlen, msg);
        return rc;
    }
    if (flags & CSG_SCENE_EXACT_BOXES) csgrt::use_exact_boxes(tree);
    const int32_t nn = static_cast<int32_t>(tree.nodes.size());
    const int32_t np = static_cast<int32_t>(tree.prims.size());
    if (n_nodes) *n_nodes = nn;
    if (n_prims) *n_prims = np;
    if (op_depth) *op_depth = tree.op_depth;
    if (nodes44) {
        if (max_nodes < nn) return CSG_E_CAPACITY;
        std::memcpy(nodes44, tree.nodes.data(), nn * sizeof(csgrt::RefNode));
    }
    if (prims48) {
        if (max_prims < np) return CSG_E_CAPACITY;
        std::memcpy(prims48, tree.prims.data(), np * sizeof(csgrt::RefPrim));
    }
    return CSG_OK;
}

int csg_scene_destroy(csg_scene* s)
{
    if (!s) return CSG_E_ARG;
    int rc = CSG_OK;
    if (csgrt::release_dispatch(s->dispatch) != cudaSuccess) rc = CSG_E_CUDA;
    if (s->dmem) {
        int prev = 0;
        cudaGetDevice(&prev);
        if (prev != s->device) cudaSetDevice(s->device);
        if (cudaFree(s->dmem) != cudaSuccess) rc = CSG_E_CUDA;
        if (prev != s->device) cudaSetDevice(prev);
    }
    delete s;
    return rc;
}

int csg_scene_get_info(const csg_scene* s, csg_scene_info* info)
{
    if (!s || !info) return CSG_E_ARG;
    info->n_nodes = s->dev.n_nodes;
    info->n_prims = s->dev.n_prims;
    info->op_depth = s->dev.op_depth;
    info->stack_class = s->dev.stack_class;
    info->device_bytes = s->bytes;
    info->rolled = s->dev.rolled;
    info->live_words = s->dev.live_words;
    info->live_shift = s->dev.live_shift;
    info->fine_words = s->dev.fine ? s->dev.fine_words : 0;
    info->short_circuit = s->dev.short_circuit;
    return CSG_OK;
}

int csg_scene_export_reference_layout(const csg_scene* s, void* nodes44, int32_t max_nodes, void* prims48,
                                      int32_t max_prims, int32_t* n_nodes, int32_t* n_prims)
{
    if (!s) return CSG_E_ARG;
    const int32_t nn = static_cast<int32_t>(s->tree.nodes.size());
    const int32_t np = static_cast<int32_t>(s->tree.prims.size());
    if (n_nodes) *n_nodes = nn;
    if (n_prims) *n_prims = np;
    if (nodes44) {
        if (max_nodes < nn) return CSG_E_CAPACITY;
        std::memcpy(nodes44, s->tree.nodes.data(), nn * sizeof(csgrt::RefNode));
    }
    if (prims48) {
        if (max_prims < np) return CSG_E_CAPACITY;
        std::memcpy(prims48, s->tree.prims.data(), np * sizeof(csgrt::RefPrim));
    }
    return CSG_OK;
}

void csg_camera_init(csg_camera* c)
{
    if (!c) return;
    c->x = 0;
    c->y = 0;
    c->z = 5;
    c->rot_x = 0;
    c->rot_y = 0;
    c->fov = 90.0f * 3.14159f / 180.0f;
    update_vectors(c);
}

void csg_camera_set_position(csg_camera* c, float x, float y, float z)
{
    if (!c) return;
    c->x = x;
    c->y = y;
    c->z = z;
}

void csg_camera_set_rotation(csg_camera* c, float pitch, float yaw)
{
    if (!c) return;
    c->rot_x = std::fmax(-89.0f * 3.14159f / 180.0f, std::fmin(89.0f * 3.14159f / 180.0f, pitch));
    c->rot_y = yaw;
    update_vectors(c);
}

void csg_camera_set_fov(csg_camera* c, float degrees)
{
    if (!c) return;
    c->fov = degrees * 3.14159f / 180.0f;
}

void csg_camera_move(csg_camera* c, float fwd, float right, float up)
{
    if (!c) return;
    c->x += c->forward[0] * fwd + c->right[0] * right;
    c->y += c->forward[1] * fwd + c->right[1] * right + up;
    c->z += c->forward[2] * fwd + c->right[2] * right;
}

void csg_camera_rotate(csg_camera* c, float dpitch, float dyaw)
{
    if (!c) return;
    csg_camera_set_rotation(c, c->rot_x + dpitch, c->rot_y + dyaw);
}

void csg_light_dir(float polar, float azimuth, float out[3])
{
    if (!out) return;
    out[0] = std::sin(polar) * std::cos(azimuth);
    out[1] = std::cos(polar);
    out[2] = std::sin(polar) * std::sin(azimuth);
}

void csg_light_default(float out[3])
{
    csg_light_dir(-60.f * 3.14159f / 180.f, -45.f * 3.14159f / 180.f, out);
}

int csg_render(const csg_scene* s, const csg_camera* cam, const float light_dir[3], int32_t w, int32_t h,
               uint32_t* rgba8_dev, float* t_dev, int32_t* prim_dev, float* normal_dev, void* stream)
{
    csgrt::Planes p;
    p.rgba8 = rgba8_dev;
    p.t = t_dev;
    p.prim = prim_dev;
    p.normal = normal_dev;
    return render_common(s, cam, light_dir, w, h, p, stream);
}

int csg_render_f4(const csg_scene* s, const csg_camera* cam, const float light_dir[3], int32_t w, int32_t h,
                  float* rgba_f4_dev, void* stream)
{
    if (!rgba_f4_dev) return CSG_E_ARG;
    csgrt::Planes p;
    p.rgba32f = reinterpret_cast<float4*>(rgba_f4_dev);
    return render_common(s, cam, light_dir, w, h, p, stream);
}

int csg_render_planes(const csg_scene* s, const csg_camera* cam, const float light_dir[3], int32_t w,
                      int32_t h, const csg_planes* planes, void* stream)
{
    if (!planes) return CSG_E_ARG;
    csgrt::Planes p;
    p.rgba8 = planes->rgba8;
    p.rgba32f = reinterpret_cast<float4*>(planes->rgba32f);
    p.t = planes->t;
    p.prim = planes->prim;
    p.normal = planes->normal;
    return render_common(s, cam, light_dir, w, h, p, stream);
}

int csg_render_host(const csg_scene* s, const csg_camera* cam, const float light_dir[3], int32_t w, int32_t h,
                    uint32_t* host_rgba8, void* stream)
{
    if (!s || !cam || !light_dir || !host_rgba8 || w <= 0 || h <= 0) return CSG_E_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaPointerAttributes a{};
    const cudaError_t qe = cudaPointerGetAttributes(&a, host_rgba8);
    cudaGetLastError();  // an unregistered pointer may leave an error behind on older runtimes
    if (qe == cudaSuccess && (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
        return CSG_E_ARG;  // a device buffer: csg_render writes it
    csgrt::Planes p;
    if (qe == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer) {
        // page-locked and mapped: the kernel stores the frame into host memory itself
        p.rgba8 = static_cast<uint32_t*>(a.devicePointer);
        return render_common(s, cam, light_dir, w, h, p, stream, true);
    }
    // pageable: a stream-ordered device frame, then a copy (which returns when done)
    const size_t bytes = (size_t)w * (size_t)h * sizeof(uint32_t);
    void* d = nullptr;
    if (cudaMallocAsync(&d, bytes, st) != cudaSuccess) return CSG_E_CUDA;
    p.rgba8 = static_cast<uint32_t*>(d);
    int rc = render_common(s, cam, light_dir, w, h, p, stream);
    if (rc == CSG_OK && cudaMemcpyAsync(host_rgba8, d, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = CSG_E_CUDA;
    if (cudaFreeAsync(d, st) != cudaSuccess && rc == CSG_OK) rc = CSG_E_CUDA;
    return rc;
}

int csg_set_iteration_cap(uint32_t cap)
{
    csgrt::set_iteration_cap(cap ? cap : csgrt::kIterCap);
    return CSG_OK;
}

int csg_device_tan_half_fov(float fov, float* out)
{
    if (!out) return CSG_E_ARG;
    return csgrt::device_tan_half_fov(fov, out) == cudaSuccess ? CSG_OK : CSG_E_CUDA;
}

int csg_scene_check(const csg_scene* s, void* stream, uint64_t* n_capped)
{
    if (!s) return CSG_E_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long v = 0;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(&v, s->status, sizeof(v), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(s->status, 0, sizeof(v));
    if (e != cudaSuccess) return CSG_E_CUDA;
    if (n_capped) *n_capped = v;
    return v ? CSG_E_TIMEOUT : CSG_OK;
}

}  // extern "C"
