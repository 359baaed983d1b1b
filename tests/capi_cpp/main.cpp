// A compiled C++ caller of the C ABI (include/csgrt.h), written the way the reference's
// RenderManager would call it in place of its Raycaster (Graphics/RayCasting/Raycaster.cuh:
// 10-25): load a tree (RenderManager::SetTreeToRender / ChangeSize, RenderManager.cpp:
// 136-166), render the frame into a float4 device buffer (RenderManager::CalculateRays,
// RenderManager.cpp:58-67, where the buffer is the mapped GL PBO), and free the scene
// (RenderManager::CleanUp, RenderManager.cpp:168-175).
//
// Built with -DCSG_REFERENCE_HEADERS and the reference's Camera.h / DirectionalLight.h on
// the include path (and its Camera.cpp compiled in), it passes the reference's own Camera
// objects across the boundary, as INTEGRATION.md shows; without them (where the
// reference's sources are absent) a stand-in with the same layout, built by the library's
// csg_camera_* functions, takes their place.
//
//   capi_cpp layout                      layout and camera checks (no GPU work)
//   capi_cpp parse <scene.txt> <out>     host-only parse: 44-byte nodes, 48-byte primitives
//   capi_cpp render <scene.txt> <w> <h> <fov> <out>   float4 frame via csg_render_f4
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "csgrt.h"

#ifdef CSG_REFERENCE_HEADERS
#include "Camera.h"            // CSGRayCasting/Graphics/RenderManager/Camera/Camera.h
#include "DirectionalLight.h"  // CSGRayCasting/Graphics/RenderManager/DirectionalLight.h
#else
// Stand-ins with the reference's data layout (Camera.h:9-16) and methods, for builds
// without its sources.
class Camera {
public:
    float x, y, z;
    float rotX, rotY;
    float fov;
    float forward[3];
    float right[3];
    float up[3];
    Camera() { csg_camera_init(as_c()); }
    void setPosition(float px, float py, float pz) { csg_camera_set_position(as_c(), px, py, pz); }
    void setRotation(float pitch, float yaw) { csg_camera_set_rotation(as_c(), pitch, yaw); }
    void setFOV(float degrees) { csg_camera_set_fov(as_c(), degrees); }
    void move(float f, float r, float u) { csg_camera_move(as_c(), f, r, u); }
    void rotate(float dp, float dy) { csg_camera_rotate(as_c(), dp, dy); }

private:
    csg_camera* as_c() { return reinterpret_cast<csg_camera*>(this); }
};
struct DirectionalLight {
    float3 getLightDir()
    {
        float d[3];
        csg_light_default(d);
        return make_float3(d[0], d[1], d[2]);
    }
};
#endif

static_assert(sizeof(Camera) == sizeof(csg_camera), "same 60-byte layout");
static_assert(offsetof(Camera, x) == offsetof(csg_camera, x), "position");
static_assert(offsetof(Camera, rotX) == offsetof(csg_camera, rot_x), "pitch");
static_assert(offsetof(Camera, rotY) == offsetof(csg_camera, rot_y), "yaw");
static_assert(offsetof(Camera, fov) == offsetof(csg_camera, fov), "field of view");
static_assert(offsetof(Camera, forward) == offsetof(csg_camera, forward), "forward");
static_assert(offsetof(Camera, right) == offsetof(csg_camera, right), "right");
static_assert(offsetof(Camera, up) == offsetof(csg_camera, up), "up");

namespace {

bool read_file(const char* path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

bool write_file(const char* path, const void* data, size_t bytes)
{
    std::ofstream f(path, std::ios::binary);
    f.write(static_cast<const char*>(data), static_cast<std::streamsize>(bytes));
    return static_cast<bool>(f);
}

// The reference's Camera methods and the library's csg_camera_* functions build the same
// bytes along the same sequence of calls.
int check_layout()
{
    Camera cam;
    csg_camera c;
    csg_camera_init(&c);
    int bad = std::memcmp(&cam, &c, sizeof c) != 0;
    const float steps[][5] = {{0.5f, -1.2f, 4.0f, 0.3f, 2.1f},  {-3.0f, 0.25f, 1.5f, -1.7f, -0.4f},
                              {0.0f, 0.0f, -5.0f, 1.6f, 3.9f},  {2.5f, 1.0f, 0.75f, -0.2f, 0.0f}};
    for (const auto& s : steps) {
        cam.setPosition(s[0], s[1], s[2]);
        csg_camera_set_position(&c, s[0], s[1], s[2]);
        cam.setRotation(s[3], s[4]);
        csg_camera_set_rotation(&c, s[3], s[4]);
        cam.setFOV(40.0f + 10.0f * s[3]);
        csg_camera_set_fov(&c, 40.0f + 10.0f * s[3]);
        cam.move(s[1], s[2], s[0]);
        csg_camera_move(&c, s[1], s[2], s[0]);
        cam.rotate(s[4], s[3]);
        csg_camera_rotate(&c, s[4], s[3]);
        bad += std::memcmp(&cam, &c, sizeof c) != 0;
    }
    DirectionalLight light;
    const float3 L = light.getLightDir();
    float d[3];
    csg_light_default(d);
    bad += (std::memcmp(&L.x, &d[0], 4) | std::memcmp(&L.y, &d[1], 4) | std::memcmp(&L.z, &d[2], 4)) != 0;
    // a parse error carries the reference's message
    char err[256] = {0};
    csg_scene_info info;
    const char* typo = "Union Spere 0 0 0 FF0000 1 Sphere 1 0 0 00FF00 1";
    const int rc = csg_tree_plan(typo, std::strlen(typo), 0, &info, err, sizeof err);
    bad += !(rc == CSG_E_PARSE && std::strcmp(err, "Cannot parse - Unrecognized keyword: Spere") == 0);
#ifdef CSG_REFERENCE_HEADERS
    std::printf("reference Camera and DirectionalLight: ");
#else
    std::printf("stand-in Camera and DirectionalLight: ");
#endif
    std::printf("%s\n", bad ? "MISMATCH" : "same bytes");
    return bad ? 1 : 0;
}

int parse(const char* scene_path, const char* out_path)
{
    std::string text;
    if (!read_file(scene_path, text)) return 2;
    char err[256] = {0};
    int32_t nn = 0, np = 0, depth = 0;
    int rc = csg_tree_parse(text.data(), text.size(), nullptr, 0, nullptr, 0, &nn, &np, &depth, err, sizeof err);
    if (rc != CSG_OK) {
        std::fprintf(stderr, "Cannot load tree: %s\n", err);
        return 3;
    }
    std::vector<unsigned char> bytes(static_cast<size_t>(nn) * 44 + static_cast<size_t>(np) * 48);
    rc = csg_tree_parse(text.data(), text.size(), bytes.data(), nn, bytes.data() + static_cast<size_t>(nn) * 44,
                        np, &nn, &np, &depth, err, sizeof err);
    if (rc != CSG_OK) return 3;
    std::printf("%d nodes, %d primitives, operator depth %d\n", nn, np, depth);
    return write_file(out_path, bytes.data(), bytes.size()) ? 0 : 4;
}

int render(const char* scene_path, int width, int height, float fov_deg, const char* out_path)
{
    std::string text;
    if (!read_file(scene_path, text)) return 2;

    // RenderManager::SetTreeToRender / ChangeSize  (RenderManager.cpp:136-166)
    //   was: CSGTree::Parse(text) in Application::LoadCSGTree + raycaster.ChangeSize(w, h, tree)
    csg_scene* scene = nullptr;
    char err[256];
    int rc = csg_scene_create(text.data(), text.size(), &scene, err, sizeof err);
    if (rc != CSG_OK) {
        std::fprintf(stderr, "Cannot load tree: %s\n", err);  // same text as before
        return 3;
    }

    // RenderManager::CalculateRays  (RenderManager.cpp:58-67)
    //   was: raycaster.Raycast(d_ptr, cam, *light)   -- two kernels + two device syncs
    // d_ptr is the mapped GL PBO there; here a device buffer of the same w*h float4 stands in.
    Camera cam;
    cam.setFOV(fov_deg);
    DirectionalLight* light = new DirectionalLight();
    float4* d_ptr = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(&d_ptr), sizeof(float4) * width * height) != cudaSuccess) return 5;
    float3 L = light->getLightDir();
    float ld[3] = {L.x, L.y, L.z};
    rc = csg_render_f4(scene, reinterpret_cast<const csg_camera*>(&cam), ld, width, height,
                       reinterpret_cast<float*>(d_ptr), /*stream*/ nullptr);
    if (rc != CSG_OK) {
        std::fprintf(stderr, "render failed: %s\n", csg_status_string(rc));
        return 6;
    }
    std::vector<float4> frame(static_cast<size_t>(width) * height);
    if (cudaMemcpy(frame.data(), d_ptr, sizeof(float4) * frame.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
    uint64_t capped = 0;
    rc = csg_scene_check(scene, nullptr, &capped);
    cudaFree(d_ptr);
    delete light;

    // RenderManager::CleanUp  (RenderManager.cpp:168-175)
    //   was: raycaster.CleanUp()
    csg_scene_destroy(scene);
    if (rc != CSG_OK) return 8;
    std::printf("rendered %dx%d\n", width, height);
    return write_file(out_path, frame.data(), sizeof(float4) * frame.size()) ? 0 : 4;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc >= 2 && std::strcmp(argv[1], "layout") == 0) return check_layout();
    if (argc == 4 && std::strcmp(argv[1], "parse") == 0) return parse(argv[2], argv[3]);
    if (argc == 7 && std::strcmp(argv[1], "render") == 0)
        return render(argv[2], std::atoi(argv[3]), std::atoi(argv[4]), static_cast<float>(std::atof(argv[5])),
                      argv[6]);
    std::fprintf(stderr, "usage: %s layout | parse <scene> <out> | render <scene> <w> <h> <fov> <out>\n", argv[0]);
    return 1;
}
