// Device-side CSG ray casting: ray generation, Kensler single-hit traversal, primitive
// intersection, hit details and Phong shading.  Shared by the single-view kernel and
// the batched persistent kernel.
//
// Arithmetic.  Every floating-point operation is an explicit round-to-nearest
// intrinsic, so the compiler can neither fuse nor split anything: the sequence of
// roundings is fixed here.  It is the sequence nvcc's default contraction (--fmad=true)
// produces for the reference kernel (CSGRayCasting/Graphics/RayCasting/Kernels/
// RaycastingKernels.cu), where a sum or difference with a product operand becomes one
// fused multiply-add: dot(a, b) = fma(a.z, b.z, fma(a.x, b.x, a.y * b.y)),
// origin + t * dir = fma(t, dir, origin), c - r * r = fma(-r, r, c), and so on.
// Divisions and square roots are IEEE (the reference's default -prec-div/-prec-sqrt);
// a halving x / 2 is computed as x * 0.5, the same correctly rounded value.
// Results -- hit, primitive, t, normal -- are therefore bit-identical to the
// reference kernel's on the same camera and scene bytes.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "scene.hpp"

namespace csgrt {
namespace dev {

// Hit-state bits (CSGUtils.cuh:29-37).
constexpr uint32_t kEnter = 1u << 1, kExit = 1u << 2, kMiss = 1u << 3, kFlip = 1u << 4,
                   kFlag1 = 1u << 5, kFlag2 = 1u << 6;
// Traversal actions (CSGUtils.cuh:5-13).
constexpr uint32_t kGotoL = 1u << 1, kGotoR = 1u << 2, kCompute = 1u << 3, kLoadL = 1u << 4,
                   kLoadR = 1u << 5, kSaveL = 1u << 6;
// Compute() outcomes (CSGUtils.cuh:15-27).
constexpr uint32_t hMiss = 1u << 1, hRetL = 1u << 2, hRetR = 1u << 3, hLoopL = 1u << 4,
                   hLoopR = 1u << 5, hLoopRC = 1u << 6, hLoopLC = 1u << 7, hRetLC = 1u << 8,
                   hRetRC = 1u << 9, hFlipR = 1u << 10;

// Kensler's tables (RaycastingKernels.cu:666-677), indexed [op][left state][right state]
// with op Union=0, Difference=1, Intersection=2 and state Enter=0, Exit=1, Miss=2.
// Loaded into shared memory once per block so that a warp's divergent lookups cost one
// conflict-free access.
__host__ __device__ constexpr uint16_t table_entry(int i)
{
    constexpr uint16_t t[27] = {
        // Union
        hRetLC | hRetRC, hRetRC | hLoopL, hRetL,
        hRetLC | hLoopR, hLoopLC | hLoopRC, hRetL,
        hRetR, hRetR, hMiss,
        // Difference
        hRetLC | hLoopR, hLoopLC | hLoopRC, hRetL,
        hRetLC | hRetRC | hFlipR, hRetRC | hFlipR | hLoopL, hRetL,
        hMiss, hMiss, hMiss,
        // Intersection
        hLoopLC | hLoopRC, hRetLC | hLoopR, hMiss,
        hRetRC | hLoopL, hRetLC | hRetRC, hMiss,
        hMiss, hMiss, hMiss};
    return t[i];
}

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 sub3(V3 a, V3 b)
{
    return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 neg3(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 scale3(float s, V3 a)
{
    return V3{__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)};
}
// Float3Utils.cuh:6-9
__device__ __forceinline__ float dot3(V3 a, V3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y)));
}
// a - s * b
__device__ __forceinline__ V3 sub_scaled(V3 a, float s, V3 b)
{
    return V3{__fmaf_rn(-s, b.x, a.x), __fmaf_rn(-s, b.y, a.y), __fmaf_rn(-s, b.z, a.z)};
}
// Ray::computePosition (Ray.cuh:20-22)
__device__ __forceinline__ V3 at3(V3 o, V3 d, float t)
{
    return V3{__fmaf_rn(t, d.x, o.x), __fmaf_rn(t, d.y, o.y), __fmaf_rn(t, d.z, o.z)};
}
// normalize (Float3Utils.cuh:33-37)
__device__ __forceinline__ V3 normalize3(V3 a)
{
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(a, a)));
    return scale3(inv, a);
}


// RayHitMinimal (Ray.cuh:36-52) held in registers.
struct Hit {
    float t;
    int32_t idx;   // short in the reference; scenes are limited to 32767 primitives
    uint32_t hit;  // state bits
    uint32_t type; // primitive type of the hit
};
__device__ __forceinline__ Hit hit_default() { return Hit{-1.0f, -1, kMiss, 0u}; }
__device__ __forceinline__ uint32_t pack_hit(const Hit& h)
{
    return (h.hit & 0xffu) | ((h.type & 0xffu) << 8) | ((uint32_t)(h.idx & 0xffff) << 16);
}
__device__ __forceinline__ Hit unpack_hit(float t, uint32_t b)
{
    return Hit{t, (int32_t)(int16_t)(b >> 16), b & 0xffu, (b >> 8) & 0xffu};
}

struct Ray {
    V3 o, d;
    V3 inv;      // rn(1/d) per component, for the certified box test
    bool exact;  // a direction component is subnormal: box tests use divisions only
};

__device__ __forceinline__ void ray_finish(Ray& r)
{
    r.inv = V3{__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z)};
    constexpr float kMinNormal = 1.1754943508222875e-38f;
    auto sub = [](float v) { return v != 0.0f && fabsf(v) < kMinNormal; };
    r.exact = sub(r.d.x) || sub(r.d.y) || sub(r.d.z);
}

// The per-view factors of ray generation: tan(fov / 2) and width / height, as the
// reference computes them for every ray (the same bits whoever computes them).
struct RayFrame {
    float thf, aspect;
};
__device__ __forceinline__ RayFrame ray_frame(const float* cam, float width, float height)
{
    return RayFrame{tanf(__fmul_rn(cam[5], 0.5f)), __fdiv_rn(width, height)};
}

// RaycastKernel ray generation (RaycastingKernels.cu:11-27) + the Ray constructor's
// second normalisation (Ray.cuh:12-18).  width/height are floats, as in the reference.
__device__ __forceinline__ Ray primary_ray(const float* cam, int x, int y, float width, float height,
                                           RayFrame f)
{
    const float u = __fdiv_rn(__fadd_rn((float)x, 0.5f), __fsub_rn(width, 1.0f));
    const float v = __fdiv_rn(__fadd_rn((float)y, 0.5f), __fsub_rn(height, 1.0f));
    const float thf = f.thf;
    const float nx = __fmul_rn(__fmul_rn(__fmaf_rn(2.0f, u, -1.0f), f.aspect), thf);
    const float ny = __fmul_rn(__fmaf_rn(-2.0f, v, 1.0f), thf);
    V3 d;
    d.x = __fadd_rn(__fmaf_rn(cam[9], nx, __fmul_rn(cam[12], ny)), cam[6]);
    d.y = __fadd_rn(__fmaf_rn(cam[10], nx, __fmul_rn(cam[13], ny)), cam[7]);
    d.z = __fadd_rn(__fmaf_rn(cam[11], nx, __fmul_rn(cam[14], ny)), cam[8]);
    d = normalize3(d);
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(d, d)));
    Ray r;
    r.o = mk(cam[0], cam[1], cam[2]);
    r.d = mk(__fmul_rn(d.x, inv), __fmul_rn(d.y, inv), __fmul_rn(d.z, inv));
    ray_finish(r);
    return r;
}

// isBVHNodeHit (RaycastingKernels.cu:718-756): slab test with six divisions.
// Returns true when the box must be entered (a cull sets hit = Miss in the caller).
// Out of line: taken only by the rare rays the certified test below cannot decide, and
// its six IEEE divisions are a lot of code to inline at every call site.  Everything is
// passed by value: a reference argument would force the caller's ray into local memory
// on every test, taken or not.
static __device__ __noinline__ bool box_hit_exact(float ox, float oy, float oz, float dx, float dy, float dz,
                                                  float lox, float loy, float loz, float hix, float hiy,
                                                  float hiz, float tmin)
{
    const float t1 = __fdiv_rn(__fsub_rn(lox, ox), dx);
    const float t2 = __fdiv_rn(__fsub_rn(hix, ox), dx);
    const float t3 = __fdiv_rn(__fsub_rn(loy, oy), dy);
    const float t4 = __fdiv_rn(__fsub_rn(hiy, oy), dy);
    const float t5 = __fdiv_rn(__fsub_rn(loz, oz), dz);
    const float t6 = __fdiv_rn(__fsub_rn(hiz, oz), dz);
    const float tmn = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmx = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    if (tmx < 0.0f) return false;
    if (tmn > tmx) return false;
    if (tmn <= tmin && tmx <= tmin) return false;
    return true;
}

// The same decision from per-ray reciprocals, certified.  With s = b - o rounded as in
// the reference, t' = rn(s * rn(1/d)) and t = rn(s / d) differ by at most 3u|t|
// (u = 2^-24) in the normal range.  x -> x -+ 3u|x| are increasing maps and min/max
// commute with increasing maps, so the reciprocal tmn' and tmx' are each within 3u of the
// reference's tmn and tmx in the same relative sense.
// The traversal's tmin is never negative (it starts at 0 and only moves to hit distances
// beyond it), and then the reference's three culls (tmx < 0; tmn > tmx; tmn <= tmin and
// tmx <= tmin) reduce to two: cull iff tmn > tmx or tmx <= tmin.  Each comparison is
// decided from the reciprocal values when their difference exceeds 2^-20 of the
// magnitudes involved plus 2^-120 (a 5x margin over the relative bound, and far above the
// absolute error of subnormal results).  Infinite or NaN values make the margin test
// fail, and a ray with a subnormal direction component (whose reciprocal overflows)
// always uses divisions (Ray::exact); all of these are decided again with divisions.
__device__ __forceinline__ bool box_hit(const Ray& r, float4 lo, float4 hi, float tmin)
{
    if (r.exact)
        return box_hit_exact(r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, tmin);
    const float t1 = __fmul_rn(__fsub_rn(lo.x, r.o.x), r.inv.x);
    const float t2 = __fmul_rn(__fsub_rn(hi.x, r.o.x), r.inv.x);
    const float t3 = __fmul_rn(__fsub_rn(lo.y, r.o.y), r.inv.y);
    const float t4 = __fmul_rn(__fsub_rn(hi.y, r.o.y), r.inv.y);
    const float t5 = __fmul_rn(__fsub_rn(lo.z, r.o.z), r.inv.z);
    const float t6 = __fmul_rn(__fsub_rn(hi.z, r.o.z), r.inv.z);
    const float tmn = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmx = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    constexpr float kRel = 9.5367431640625e-07f;     // 2^-20
    constexpr float kAbs = 7.52316384526264e-37f;    // 2^-120
    const float ax = fabsf(tmx);
    const float d1 = __fsub_rn(tmn, tmx), d2 = __fsub_rn(tmx, tmin);
    const bool sure = fabsf(d1) > __fmaf_rn(kRel, __fadd_rn(fabsf(tmn), ax), kAbs) &&
                      fabsf(d2) > __fmaf_rn(kRel, ax, kAbs);
    if (!sure)
        return box_hit_exact(r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, tmin);
    return d1 < 0.0f && d2 > 0.0f;
}

// Conservative form of the box test at tmin = 0, for the liveness pre-pass: false only
// when the reference's test culls the box for every tmin >= 0, i.e. when tmx <= 0 or
// tmn > tmx; anything it cannot decide cheaply passes (the pre-pass only prunes, so a
// pass is always safe).  From the reciprocal values t' (each with the sign of the
// reference's t, infinities and NaNs where the reference has them, and otherwise within
// 3u|t|): tmx' < 0 means some axis has both reference values <= 0, hence tmx <= 0; and
// tmn' - tmx' > 2^-20 (|tmn'| + |tmx'|) with both magnitudes above 2^-100 means tmn > tmx.
__device__ __forceinline__ bool box_may_pass_at_zero(const Ray& r, float4 lo, float4 hi)
{
    if (r.exact)
        return box_hit_exact(r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, 0.0f);
    const float t1 = __fmul_rn(__fsub_rn(lo.x, r.o.x), r.inv.x);
    const float t2 = __fmul_rn(__fsub_rn(hi.x, r.o.x), r.inv.x);
    const float t3 = __fmul_rn(__fsub_rn(lo.y, r.o.y), r.inv.y);
    const float t4 = __fmul_rn(__fsub_rn(hi.y, r.o.y), r.inv.y);
    const float t5 = __fmul_rn(__fsub_rn(lo.z, r.o.z), r.inv.z);
    const float t6 = __fmul_rn(__fsub_rn(hi.z, r.o.z), r.inv.z);
    const float tmn = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmx = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    if (tmx < 0.0f) return false;
    constexpr float kRel = 9.5367431640625e-07f;     // 2^-20
    constexpr float kTiny = 7.888609052210118e-31f;  // 2^-100
    const float an = fabsf(tmn), ax = fabsf(tmx);
    return !(__fsub_rn(tmn, tmx) > kRel * __fadd_rn(an, ax) && fminf(an, ax) > kTiny);
}

// sphereHit (RaycastingKernels.cu:135-181)
__device__ __forceinline__ void sphere_hit(const Ray& r, float4 g0, int32_t id, Hit& h, float tmin)
{
    h.hit = kMiss;
    h.idx = id;
    const V3 c = mk(g0.x, g0.y, g0.z);
    const V3 oc = sub3(r.o, c);
    const float b = dot3(oc, r.d);
    const float cc = __fmaf_rn(-g0.w, g0.w, dot3(oc, oc));
    const float disc = __fmaf_rn(b, b, -cc);
    if (disc < 0.0f) return;
    const float s = __fsqrt_rn(disc);
    float tt = __fsub_rn(-b, s);
    if (tt <= tmin) {
        tt = __fadd_rn(-b, s);
        if (tt <= tmin) {
            h.t = -1.0f;
            h.hit = kMiss;
            h.idx = -1;
            return;
        }
    }
    h.t = tt;
    const V3 n = sub3(at3(r.o, r.d, tt), c);
    h.hit = (dot3(n, r.d) <= 0.0f) ? kEnter : kExit;
    h.type = kSphere;
}

// Inside cylinderHit and reflect nvcc shares some products between expressions and leaves
// those unfused, so some dot products there have other shapes than dot3 (matched against
// the reference kernel's own intermediates on ~20k cylinder rays and ~37k shaded pixels):
//   dot(d, V), and the cap denominators dot(d, +-V):  rn(fma(y, y', x*x') + z*z')
//   the top cap's numerator dot(-(o - c - (h/2)V), V) and reflect's dot(-L, n):
//                                                    fma(z, z', fma(y, y', x*x'))
// and c - (h/2)V is a product rounded on its own followed by the subtraction.
__device__ __forceinline__ float dot_yx_z(V3 a, V3 b)
{
    return __fadd_rn(__fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float dot_zyx(V3 a, V3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ V3 sub_scaled_unfused(V3 a, float s, V3 b)
{
    return V3{__fsub_rn(a.x, __fmul_rn(s, b.x)), __fsub_rn(a.y, __fmul_rn(s, b.y)),
              __fsub_rn(a.z, __fmul_rn(s, b.z))};
}

// Cap-plane step of cylinderHit (RaycastingKernels.cu:238-266 / 273-301).
__device__ __forceinline__ void cylinder_caps(const Ray& r, V3 V, V3 OC, V3 cen, float h2, float hgt,
                                              float m, float& temp, bool& skip, int& use)
{
    if (m < 0.0f) {
        const V3 nV = neg3(V);
        const float den = dot_yx_z(r.d, nV);
        if (fabsf(den) < 0.0001f) {
            skip = true;
        } else {
            temp = __fdiv_rn(dot3(neg3(OC), nV), den);
            use = 1;
        }
    }
    if (m > hgt) {
        const float den = dot_yx_z(r.d, V);
        if (fabsf(den) < 0.0001f) {
            skip = true;
        } else {
            const V3 ocm = sub_scaled_unfused(sub3(r.o, cen), h2, V);
            temp = __fdiv_rn(dot_zyx(neg3(ocm), V), den);
            use = 2;
        }
    }
}

// cylinderHit (RaycastingKernels.cu:202-336)
__device__ __forceinline__ void cylinder_hit(const Ray& r, float4 g0, float4 g1, int32_t id, Hit& h,
                                             float tmin)
{
    h.hit = kMiss;
    h.idx = id;
    const float rad = g0.w, hgt = g1.x;
    const V3 V = mk(g1.y, g1.z, g1.w);
    const V3 cen = mk(g0.x, g0.y, g0.z);
    const float h2 = __fmul_rn(hgt, 0.5f);
    const V3 C = sub_scaled_unfused(cen, h2, V);
    const V3 OC = sub3(r.o, C);
    const float dV = dot_yx_z(r.d, V);
    const float a = fmaxf(__fmaf_rn(-dV, dV, 1.0f), 0.00001f);
    const float cH = dot3(OC, V);
    const float c = __fmaf_rn(-rad, rad, __fmaf_rn(-cH, cH, dot3(OC, OC)));
    const float b = __fmaf_rn(-dV, cH, dot3(r.d, OC));
    const float disc = __fmaf_rn(b, b, -__fmul_rn(a, c));
    if (disc < 0.0f) return;
    const float s = __fsqrt_rn(disc);
    const float t1 = __fdiv_rn(__fsub_rn(-b, s), a);
    const float t2 = __fdiv_rn(__fadd_rn(-b, s), a);
    const float m1 = __fmaf_rn(t1, dV, cH);
    const float m2 = __fmaf_rn(t2, dV, cH);
    if ((m1 < 0.0f && m2 < 0.0f) || (m1 > hgt && m2 > hgt)) return;
    // The near root, then the far one, each possibly replaced by a cap; one copy of the cap
    // code serves both.
    float temp, m;
    int use;
#pragma unroll 1
    for (int k = 0;; ++k) {
        temp = k ? t2 : t1;
        m = k ? m2 : m1;
        bool skip = false;
        use = 0;
        cylinder_caps(r, V, OC, cen, h2, hgt, m, temp, skip, use);
        if (!(temp <= tmin || skip)) break;
        if (k == 1) return;
    }
    h.t = temp;
    V3 n;
    if (use == 1) n = neg3(V);
    else if (use == 2) n = V;
    else n = sub_scaled(sub3(at3(r.o, r.d, temp), C), m, V);
    h.hit = (dot3(n, r.d) <= 0.0f) ? kEnter : kExit;
    if (use == 1) h.hit |= kFlag1;
    else if (use == 2) h.hit |= kFlag2;
    h.type = kCylinder;
}

// cubeHit (RaycastingKernels.cu:375-434): axis-aligned slab test.
__device__ __forceinline__ void cube_hit(const Ray& r, float4 g0, int32_t id, Hit& h, float tmin)
{
    h.hit = kMiss;
    h.idx = id;
    const float s2 = __fmul_rn(g0.w, 0.5f);
    const V3 C = mk(g0.x, g0.y, g0.z);
    const float t1 = __fdiv_rn(__fsub_rn(__fsub_rn(C.x, s2), r.o.x), r.d.x);
    const float t2 = __fdiv_rn(__fsub_rn(__fadd_rn(C.x, s2), r.o.x), r.d.x);
    const float t3 = __fdiv_rn(__fsub_rn(__fsub_rn(C.y, s2), r.o.y), r.d.y);
    const float t4 = __fdiv_rn(__fsub_rn(__fadd_rn(C.y, s2), r.o.y), r.d.y);
    const float t5 = __fdiv_rn(__fsub_rn(__fsub_rn(C.z, s2), r.o.z), r.d.z);
    const float t6 = __fdiv_rn(__fsub_rn(__fadd_rn(C.z, s2), r.o.z), r.d.z);
    float tmn = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmx = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    if (tmx < 0.0f) return;
    if (tmn > tmx) return;
    if (tmn <= tmin) {
        tmn = tmx;
        if (tmn <= tmin) return;
    }
    h.t = tmn;
    const V3 PC = sub3(at3(r.o, r.d, tmn), C);
    const float bias = 1.00001f;
    const V3 n = mk((float)(int)__fmul_rn(__fdiv_rn(PC.x, s2), bias),
                    (float)(int)__fmul_rn(__fdiv_rn(PC.y, s2), bias),
                    (float)(int)__fmul_rn(__fdiv_rn(PC.z, s2), bias));
    h.hit = (dot3(n, r.d) <= 0.0f) ? kEnter : kExit;
    h.type = kCube;
}

// hitPrimitive (RaycastingKernels.cu:113-133).  CYL: the scene may hold cylinders (false
// leaves the cylinder test out of the code: kernels for trees without cylinders).
template <bool CYL = true>
__device__ __forceinline__ void hit_primitive(const Ray& r, const float4* __restrict__ geo, int32_t type,
                                              int32_t prim, Hit& h, float tmin)
{
    const float4 g0 = __ldg(&geo[2 * prim]);
    if (type == kSphere) {
        sphere_hit(r, g0, prim, h, tmin);
    } else if (CYL && type == kCylinder) {
        const float4 g1 = __ldg(&geo[2 * prim + 1]);
        cylinder_hit(r, g0, g1, prim, h, tmin);
    } else if (type == kCube) {
        cube_hit(r, g0, prim, h, tmin);
    } else {
        h = hit_default();
    }
}

// Per-ray stacks.  The action stack (CudaStack<uchar,32>) is 32 two-bit codes in a
// 64-bit register: Compute=0, LoadLft=1, LoadRgh=2, SaveLft=3 (the only actions ever
// pushed).  The primitive and time stacks live in shared memory, laid out
// [slot][thread] so that a warp touching the same slot hits 32 distinct banks.
// Semantics follow CudaStack (CudaStack.cuh:14-31): a push onto a full stack is
// dropped, a pop from an empty one returns slot 0.
struct ActionStack {
    unsigned long long bits;
    int n;
    __device__ __forceinline__ void push(uint32_t action_bit)
    {
        if (n < 32) {
            const uint32_t code = (uint32_t)(__ffs(action_bit) - 4);  // 8->0 16->1 32->2 64->3
            const int sh = 2 * n;
            bits = (bits & ~(3ull << sh)) | ((unsigned long long)code << sh);
            ++n;
        }
    }
    __device__ __forceinline__ uint32_t pop()
    {
        if (n > 0) --n;
        return 8u << (uint32_t)((bits >> (2 * n)) & 3ull);
    }
};

template <int SD>
struct SmemStacks {
    float* pt;     // [SD][nt] primitive stack: t
    uint32_t* pb;  // [SD][nt] primitive stack: packed state/type/index
    float* tt;     // [SD][nt] time stack
    int nt, tid;
    int np, ntm;
    __device__ __forceinline__ void ppush(const Hit& h)
    {
        if (np < SD) {
            pt[np * nt + tid] = h.t;
            pb[np * nt + tid] = pack_hit(h);
            ++np;
        }
    }
    __device__ __forceinline__ Hit ppop()
    {
        if (np > 0) --np;
        return unpack_hit(pt[np * nt + tid], pb[np * nt + tid]);
    }
    __device__ __forceinline__ void tpush(float v)
    {
        if (ntm < SD) {
            tt[ntm * nt + tid] = v;
            ++ntm;
        }
    }
    __device__ __forceinline__ float tpop()
    {
        if (ntm > 0) --ntm;
        return tt[ntm * nt + tid];
    }
    // Slot 0 of both stacks is what a pop from an empty stack returns.
    __device__ __forceinline__ void reset_bottom()
    {
        pt[tid] = -1.0f;
        pb[tid] = kMiss | (0xffffu << 16);
        tt[tid] = 0.0f;
    }
};

// The same stacks as per-thread arrays in local memory (the thread's stack frame, cached
// in L1), for launches that keep shared memory for the live masks and give the L1 cache
// more room.  Same capacity and overflow semantics as SmemStacks.
template <int SD>
struct LocalStacks {
    float pt[SD];
    uint32_t pb[SD];
    float tt[SD];
    int np, ntm;
    __device__ __forceinline__ void ppush(const Hit& h)
    {
        if (np < SD) {
            pt[np] = h.t;
            pb[np] = pack_hit(h);
            ++np;
        }
    }
    __device__ __forceinline__ Hit ppop()
    {
        if (np > 0) --np;
        return unpack_hit(pt[np], pb[np]);
    }
    __device__ __forceinline__ void tpush(float v)
    {
        if (ntm < SD) {
            tt[ntm] = v;
            ++ntm;
        }
    }
    __device__ __forceinline__ float tpop()
    {
        if (ntm > 0) --ntm;
        return tt[ntm];
    }
    __device__ __forceinline__ void reset_bottom()
    {
        pt[0] = -1.0f;
        pb[0] = kMiss | (0xffffu << 16);
        tt[0] = 0.0f;
    }
};

// Per-ray live-leaf mask.  Bit g stands for leaves [g << shift, (g + 1) << shift); a
// clear bit means every leaf of the group is known to return Miss at the tmin of any
// later visit.  A leaf's result is monotone in tmin (a Miss stays a Miss when tmin grows:
// a sphere needs a root beyond tmin, a cylinder a valid branch beyond tmin, a box tmx
// beyond tmin), so a bit cleared at tmin t stays valid while visits come with tmin >= t.
// The pre-pass clears at tmin = 0, below every tmin.  Bits are also cleared during the
// traversal, when a leaf test returns Miss and when an operator child's box culls (its
// leaves' boxes are nested in it, so they cull too), and those hold only as long as tmin
// does not fall below the tmin of the clear.  It can fall: a node returns its closer
// child's t, which can lie below a tmin its other child's subtree has already looped to,
// and a loop of an ancestor then re-enters that subtree with the lower tmin (the
// reference does this on about one ray in several hundred of random trees).  Subtrees
// are re-entered only through loops, so each region of kLiveRegionWords mask words keeps
// the largest tmin at which the traversal cleared one of its live bits (`region`), and a
// loop whose new tmin is below a region's record marks the looped child's leaves in that
// region live again (restore_range), which only prunes less; `tclr`, the largest record
// of the ray, lets loops at or above every record skip the test.  One record per ray
// re-enabled whole subtrees that held no stale bit: on the 3840x2160 cheese frame the
// slowest rays then took 2.7x the iterations of the rule without the restore, and the
// warps holding them ran for most of the launch.  A subtree whose leaves are all Miss
// evaluates to a Miss whether or not it is traversed, and a Miss's t and index reach no
// decision and no output, so skipping such a subtree changes nothing.  The mask lives in
// shared memory, word k of a lane at w[k * nt] and the record of region r right after the
// words, at w[(words + r) * nt] (as a float); `sum` has bit k set while word k is non-zero
// (SumT: 32 bits for masks of up to 32 words, 64 bits for up to 64).
using live_sum_t = std::conditional<(kLiveWordsMax > 32), unsigned long long, uint32_t>::type;
constexpr int kLiveRegionWords = 4;
__host__ __device__ constexpr int live_regions(int words) { return (words + kLiveRegionWords - 1) / kLiveRegionWords; }

template <typename SumT>
struct LiveMaskT {
    using live_sum_t = SumT;
    uint32_t* w;
    int nt;
    int shift;
    int words;
    live_sum_t sum;
    float tclr;  // largest tmin of a clear made during the traversal (-inf: none)

    __device__ __forceinline__ uint32_t& word(int k) { return w[k * nt]; }
    __device__ __forceinline__ float& region(int k)
    {
        return reinterpret_cast<float*>(w)[(words + k / kLiveRegionWords) * nt];
    }
    // No clear recorded yet (before the traversal starts).
    __device__ __forceinline__ void reset_records()
    {
        tclr = -INFINITY;
        for (int r = 0; r < live_regions(words); ++r) region(r * kLiveRegionWords) = -INFINITY;
    }
    __device__ __forceinline__ void fill(int n_groups)
    {
        sum = 0;
        for (int k = 0; k < words; ++k) {
            const int rem = n_groups - 32 * k;
            const uint32_t v = rem >= 32 ? 0xffffffffu : (rem <= 0 ? 0u : ((1u << rem) - 1u));
            word(k) = v;
            if (v) sum |= (live_sum_t)1 << k;
        }
    }
    __device__ __forceinline__ void clear_all()
    {
        for (int k = 0; k < words; ++k) word(k) = 0u;
        sum = 0;
    }
    __device__ __forceinline__ void set_leaf(int leaf)
    {
        const int g = leaf >> shift;
        word(g >> 5) |= 1u << (g & 31);
        sum |= (live_sum_t)1 << (g >> 5);
    }
    __device__ __forceinline__ bool any(int lo, int hi)
    {
        const int a = lo >> shift, b = hi >> shift;
        const int wa = a >> 5, wb = b >> 5;
        const uint32_t ma = 0xffffffffu << (a & 31);
        const uint32_t mb = 0xffffffffu >> (31 - (b & 31));
        if (wa == wb) return ((sum >> wa) & 1u) && (word(wa) & ma & mb);
        const live_sum_t mid = (live_sum_t)(((1ull << wb) - 1ull) & ~((1ull << (wa + 1)) - 1ull));
        if (sum & mid) return true;
        if (((sum >> wa) & 1u) && (word(wa) & ma)) return true;
        return ((sum >> wb) & 1u) && (word(wb) & mb);
    }
    // Clears the bits m of word k at tmin tc (a NaN tmin counts as +inf: a loop to any
    // tmin then restores the region).  Only bits that were live raise the records: a bit
    // that was already clear keeps the validity of its earlier clear.
    __device__ __forceinline__ void clear_word(int k, uint32_t m, float tc)
    {
        const uint32_t old = word(k), v = old & ~m;
        if (v == old) return;
        word(k) = v;
        if (!v) sum &= ~((live_sum_t)1 << k);
        float& r = region(k);
        r = fmaxf(r, tc);
        tclr = fmaxf(tclr, tc);
    }
    __device__ __forceinline__ void clear_leaf(int leaf, float tmin)
    {
        if (shift == 0) clear_word(leaf >> 5, 1u << (leaf & 31), tmin == tmin ? tmin : INFINITY);
    }
    // Clears the groups lying entirely inside [lo, hi].
    __device__ __forceinline__ void clear_range(int lo, int hi, float tmin)
    {
        const int ga = (lo + (1 << shift) - 1) >> shift, gb = ((hi + 1) >> shift) - 1;
        if (ga > gb) return;
        const float tc = tmin == tmin ? tmin : INFINITY;
        const int wa = ga >> 5, wb = gb >> 5;
        for (int k = wa; k <= wb; ++k) {
            if (!((sum >> k) & 1u)) continue;
            const uint32_t lo_m = (k == wa) ? (0xffffffffu << (ga & 31)) : 0xffffffffu;
            const uint32_t hi_m = (k == wb) ? (0xffffffffu >> (31 - (gb & 31))) : 0xffffffffu;
            clear_word(k, lo_m & hi_m, tc);
        }
    }
    // A loop to tmin re-enters the subtree with leaves [lo, hi]: sets every group that
    // holds one of its leaves (groups reaching outside the range too: more live bits only
    // prune less) in the words whose region recorded a clear above tmin.
    __device__ __forceinline__ void restore_range(int lo, int hi, float tmin)
    {
        const int ga = lo >> shift, gb = hi >> shift;
        const int wa = ga >> 5, wb = gb >> 5;
        for (int k = wa; k <= wb; ++k) {
            if (tmin >= region(k)) continue;
            const uint32_t lo_m = (k == wa) ? (0xffffffffu << (ga & 31)) : 0xffffffffu;
            const uint32_t hi_m = (k == wb) ? (0xffffffffu >> (31 - (gb & 31))) : 0xffffffffu;
            word(k) |= lo_m & hi_m;
            sum |= (live_sum_t)1 << k;
        }
    }
};
// The scene's own mask (at most kLiveWordsMax words), and the fine mask of single-view
// renders of large trees (at most kFineWordsMax words, one bit per leaf up to 2,048 leaves).
using LiveMask = LiveMaskT<live_sum_t>;
using LiveMaskFine = LiveMaskT<unsigned long long>;

// Liveness at tmin = 0 of one leaf whose own box already passed at tmin = 0: a cube's box
// is the cube (the cube test is the same slab test), so it is live; a sphere or cylinder
// is live when its primitive test at tmin = 0 is not a Miss.
// Build-time tuning knob: 0 skips the primitive test (box test only) in the pre-pass.
#ifndef CSG_PREPASS_PRIM_TEST
#define CSG_PREPASS_PRIM_TEST 1
#endif
template <bool CYL>
__device__ __forceinline__ bool leaf_live_at_zero(const Ray& ray, const float4* __restrict__ geo, int prim,
                                                  int type)
{
    if (type == kCube || !CSG_PREPASS_PRIM_TEST) return true;
    Hit h = hit_default();
    const float4 g0 = __ldg(&geo[2 * prim]);
    if (type == kSphere || !CYL) {
        sphere_hit(ray, g0, prim, h, 0.0f);
    } else {
        const float4 g1 = __ldg(&geo[2 * prim + 1]);
        cylinder_hit(ray, g0, g1, prim, h, 0.0f);
    }
    return h.hit != kMiss;
}

// Per-warp scratch of the liveness pre-pass in shared memory (ints): the stack of the
// depth-first walk (its first kWarpStack entries) or of the cone walk (all of it).
constexpr int kWarpStack = 64;
constexpr int kWarpScratch = 192;
static_assert(kWarpScratch >= kWarpStack, "warp scratch");

// Liveness pre-pass, depth first: the warp walks the BVH over the leaves' own boxes
// together (its 32 rays are one pixel tile, so they share most of the walk), each lane
// testing its own ray, and every lane sets the bits of the leaves whose box may pass at
// tmin = 0 (box_may_pass_at_zero) and whose primitive test at tmin = 0 is not a Miss.
// Must be called by all 32 lanes; lanes with active == false only follow.  If the walk
// would overflow the warp's stack, every lane falls back to an all-live mask (the
// traversal then decides everything itself).
template <bool ROLLED, bool CYL, class LM>
__device__ __forceinline__ void live_walk_rays(const Ray& ray, bool active, const DeviceScene& sc, LM& lm,
                                               int* wstack, int n_groups)
{
    const float4* __restrict__ bvh = sc.bvh;
    int node = 0, sp = 0;
    bool overflow = false;
    while (true) {
        const float4 a0 = __ldg(&bvh[4 * node + 0]);
        const float4 a1 = __ldg(&bvh[4 * node + 1]);
        const float4 a2 = __ldg(&bvh[4 * node + 2]);
        const float4 a3 = __ldg(&bvh[4 * node + 3]);
        const int cl = __float_as_int(a0.w), cr = __float_as_int(a2.w);
        bool hl = false, hr = false;
        if (ROLLED) {
            // both box tests side by side (independent work for the scheduler), the
            // primitive tests in a rolled loop so that their code exists once
            hl = active && box_may_pass_at_zero(ray, a0, a1);
            hr = active && box_may_pass_at_zero(ray, a2, a3);
#pragma unroll 1
            for (int j = 0; j < 2; ++j) {
                const int c = j ? cr : cl;
                const bool h = j ? hr : hl;
                const int type = __float_as_int(j ? a3.w : a1.w);
                if (h && c < 0 && leaf_live_at_zero<CYL>(ray, sc.geo, ~c, type)) lm.set_leaf(~c);
            }
        } else {
            hl = active && box_may_pass_at_zero(ray, a0, a1);
            hr = active && box_may_pass_at_zero(ray, a2, a3);
            if (hl && cl < 0 && leaf_live_at_zero<CYL>(ray, sc.geo, ~cl, __float_as_int(a1.w))) lm.set_leaf(~cl);
            if (hr && cr < 0 && leaf_live_at_zero<CYL>(ray, sc.geo, ~cr, __float_as_int(a3.w))) lm.set_leaf(~cr);
        }
        const bool dl = __any_sync(0xffffffffu, hl && cl >= 0);
        const bool dr = __any_sync(0xffffffffu, hr && cr >= 0);
        if (dl && dr) {
            if (sp >= kWarpStack) {
                overflow = true;
                break;
            }
            wstack[sp] = cr;  // every lane writes the same value
            ++sp;
            node = cl;
        } else if (dl) {
            node = cl;
        } else if (dr) {
            node = cr;
        } else {
            if (sp == 0) break;
            __syncwarp();
            node = wstack[--sp];
        }
        __syncwarp();
    }
    if (overflow) lm.fill(n_groups);
}

// Whether a ray of the cone (apex o, unit axis a, half-angle with sine sp and cosine cp)
// may meet the sphere of centre c and radius r at t >= 0, the sphere widened by 1e-4 of its
// radius and by `rel` times its distance from o.  The test is the signed distance of the
// centre from the cone's surface in the plane through the axis: s = d cos - t sin (d the
// centre's distance from the axis, t its position along it) must not exceed the radius, and
// u = t cos + d sin must not lie below minus the radius (the sphere is not wholly behind the
// apex).  The two distances come from the hardware's reciprocal square root (within a few
// units of 2^-23 relative, far inside the 1e-4 margins).  Non-finite values pass (a zero
// distance gives 0 * inf = NaN, which passes too).
__device__ __forceinline__ bool cone_may_hit(V3 o, V3 a, float sp, float cp, float cx, float cy, float cz, float r,
                                             float rel)
{
    const float vx = cx - o.x, vy = cy - o.y, vz = cz - o.z;
    const float dd = vx * vx + vy * vy + vz * vz;
    const float dist = dd * rsqrtf(dd);
    const float R = r * 1.0001f + rel * dist;
    const float t = a.x * vx + a.y * vy + a.z * vz;
    const float qx = a.y * vz - a.z * vy, qy = a.z * vx - a.x * vz, qz = a.x * vy - a.y * vx;
    const float q2 = qx * qx + qy * qy + qz * qz;
    const float d = q2 * rsqrtf(q2);
    const float s = d * cp - t * sp, u = t * cp + d * sp;
    return !(s > R) && !(u < -R);
}

// Liveness pre-pass over a cone: the warp bounds its active lanes' rays by a cone (their
// mean direction as the axis, the largest angle from it plus 1e-4 rad as the half-angle)
// and walks the BVH 32 boxes at a time: each step pops up to 32 boxes off a shared stack,
// one per lane, tests them against the cone (cone_may_hit), pushes the children of the
// boxes that pass, and has every lane test each leaf that passed with its own ray, as the
// depth-first walk does (box_may_pass_at_zero and the primitive test at tmin = 0).  So the
// warp's box tests are shared across the lanes instead of repeated in each.  A box the
// cone rejects holds no leaf any of the warp's rays can meet: the cone contains every ray,
// and its margins (1e-4 rad on the angle, 1e-4 relative on a box's bounding sphere, 1e-3
// for a sphere leaf tested as itself) lie far above the rounding of the rays, of the cone and
// of the reference's box and primitive tests (~1e-7 relative), so no leaf whose tests could
// pass for some ray is left out.  Returns false,
// having decided nothing, when the cone is wide (half-angle above 30 degrees, or
// non-finite) or the stack would overflow; the caller then walks depth first.
template <bool CYL, class LM>
__device__ __forceinline__ bool live_walk_cone(const Ray& ray, bool active, const DeviceScene& sc, LM& lm,
                                               int* stk)
{
    const unsigned lane = threadIdx.x & 31u;
    if (!__any_sync(0xffffffffu, active)) return true;  // no lane renders: the masks go unused
    // cone axis: the mean direction of the active lanes
    float ax = active ? ray.d.x : 0.f, ay = active ? ray.d.y : 0.f, az = active ? ray.d.z : 0.f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, off);
        ay += __shfl_xor_sync(0xffffffffu, ay, off);
        az += __shfl_xor_sync(0xffffffffu, az, off);
    }
    const float inv = rsqrtf(ax * ax + ay * ay + az * az);
    const V3 a = mk(ax * inv, ay * inv, az * inv);
    // half-angle: the largest sine of the angle between the axis and an active lane's ray
    float sn = 0.f;
    bool wide = false;
    if (active) {
        const float qx = a.y * ray.d.z - a.z * ray.d.y, qy = a.z * ray.d.x - a.x * ray.d.z,
                    qz = a.x * ray.d.y - a.y * ray.d.x;
        sn = sqrtf(qx * qx + qy * qy + qz * qz);
        wide = !(a.x * ray.d.x + a.y * ray.d.y + a.z * ray.d.z > 0.5f) || !(sn < 0.5f);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sn = fmaxf(sn, __shfl_xor_sync(0xffffffffu, sn, off));
    const float sp = sn + 1e-4f;
    if (__any_sync(0xffffffffu, wide) || !(sp < 0.5f)) return false;
    const float cp = sqrtf(1.f - sp * sp);

    const float4* __restrict__ bvh = sc.bvh;
    const float4* __restrict__ bsph = sc.bvh + 4 * sc.n_bvh;
    // stack entries: node << 1 | side (a child slot of a BVH node, whose box is at
    // bvh[2 * entry] and bvh[2 * entry + 1] and whose bounding sphere is at bsph[entry])
    if (lane < 2) stk[lane] = (int)lane;  // the root's two children
    __syncwarp();
    int n = 2;
    const unsigned lt = (1u << lane) - 1u;
    while (n > 0) {
        const int take = n < 32 ? n : 32;
        const bool valid = (int)lane < take;
        const int e = valid ? stk[n - take + (int)lane] : 0;
        __syncwarp();  // every entry is read before pushes overwrite the slots
        n -= take;
        const int child = __float_as_int(__ldg(&bvh[2 * e + 0]).w);
        // the bound tested against the cone (precomputed per slot): a box's bounding sphere,
        // or for a sphere leaf (negative radius) the sphere itself (its box, +-2r, is 3.5 times
        // wider), widened by 1e-3 of its distance: a ray that misses the sphere by that much
        // gives a negative discriminant whatever the rounding (~1e-7 of the squared
        // distance), so the leaf is a Miss at every tmin
        const float4 bs = __ldg(&bsph[e]);
        const float rel = __float_as_int(bs.w) < 0 ? 1e-3f : 1e-4f;
        const bool pass = valid && cone_may_hit(ray.o, a, sp, cp, bs.x, bs.y, bs.z, fabsf(bs.w), rel);
        const unsigned mi = __ballot_sync(0xffffffffu, pass && child >= 0);
        unsigned ml = __ballot_sync(0xffffffffu, pass && child < 0);
        if (n + 2 * __popc(mi) > kWarpScratch) return false;  // warp-uniform
        if (pass && child >= 0) {
            const int at = n + 2 * __popc(mi & lt);
            stk[at] = child << 1;
            stk[at + 1] = (child << 1) | 1;
        }
        n += 2 * __popc(mi);
        // every lane tests the leaves that passed, each with its own ray
        while (ml) {
            const int src = __ffs(ml) - 1;
            ml &= ml - 1u;
            const int le = __shfl_sync(0xffffffffu, e, src);
            const float4 llo = __ldg(&bvh[2 * le + 0]);
            const float4 lhi = __ldg(&bvh[2 * le + 1]);
            const int prim = ~__float_as_int(llo.w);
            if (active && box_may_pass_at_zero(ray, llo, lhi) &&
                leaf_live_at_zero<CYL>(ray, sc.geo, prim, __float_as_int(lhi.w)))
                lm.set_leaf(prim);
        }
        __syncwarp();
    }
    return true;
}

// Build-time tuning knob: 1 tries the cone walk first, 0 always walks depth first.
#ifndef CSG_PREPASS_CONE
#define CSG_PREPASS_CONE 1
#endif

// Liveness pre-pass: the mask of the leaves each ray can hit at all, at tmin = 0.  Must be
// called by all 32 lanes; lanes with active == false only follow.
template <bool ROLLED, bool CYL, class LM>
__device__ __forceinline__ void live_prepass(const Ray& ray, bool active, const DeviceScene& sc, LM& lm,
                                             int* wsm)
{
    const int n_groups = (sc.n_prims + (1 << lm.shift) - 1) >> lm.shift;
    lm.reset_records();
    if (!sc.prepass || sc.n_bvh == 0) {
        lm.fill(n_groups);
        return;
    }
    lm.clear_all();
    if (CSG_PREPASS_CONE && live_walk_cone<CYL>(ray, active, sc, lm, wsm)) return;
    lm.clear_all();
    __syncwarp();
    live_walk_rays<ROLLED, CYL>(ray, active, sc, lm, wsm, n_groups);
}

// One child of an operator node during GoTo (RaycastingKernels.cu:540-553): the box
// test of isBVHNodeHit and, for a leaf that passes it, the primitive test.  Returns true
// when the traversal must descend into the child.
//
// The primitive test of a leaf is a function of the ray, the primitive and tmin only, and
// a Miss's t and index never reach a decision or an output (every table cell that
// compares t or loops on t has both sides, or the looping side, non-Miss), so for leaves
// the order of the two tests can change without changing any result:
//  * cube: its box is the cube itself, and cubeHit repeats the identical slab test, so the
//    box test is implied and skipped;
//  * sphere: the sphere test runs first; only a hit is confirmed with the box test;
//  * cylinder: its box is not conservative (BVHNode.cuh:34-49) and does cut hits, so the
//    box test runs first, as in the reference.
//
// With boxed == false the same code serves GoTo landing on a leaf (the root is a leaf, or a
// loop re-enters a leaf child), where the reference calls hitPrimitive with no box test.
// PRUNE: consult and update the live mask.  skip_op / skip_leaf: whether a decision that
// skips work (no live leaf, the single-leaf shortcut) may be taken for an operator child /
// a leaf (always, except in the 32-entry stack class: kGuard).
//
// Single-leaf shortcut (with PRUNE, one mask bit per leaf, in scenes large enough for the
// liveness pre-pass: on smaller ones, whose masks start all live, it cost 4%): an operator
// child of at most
// kShortcutLeaves leaves with exactly one live leaf l is not descended into.  Every other
// leaf of it is a Miss at this tmin, and by Kensler's tables a Union with a Miss child
// returns the other child's record, a Difference returns its left child's record when the
// right one is a Miss and Miss when the left one is, and an Intersection with a Miss child
// returns Miss.  So the child's result is l's own (tested with l's box, which every box on
// the path down to it contains: a box that passes makes every enclosing box pass, a box
// that culls makes the result a Miss either way) when every operator on that path is a
// Union or a Difference entered on its left, and a Miss otherwise: l's record in lbox
// holds the depth of the deepest operator above l that is neither (blk), and the path
// below a child of depth dc is clear of them when blk < dc.  The descent the reference
// makes instead pushes and pops in pairs (none of its pushes is dropped: no stack overflows
// below the 32-entry class, and in it skip_op holds only where none can, kGuard), and it
// leaves the result in the record of the child's side, as this test does.
// (A tuning knob: 256 leaves took the cheese frame 5% below 128, where its Union's two
// 256-leaf halves were not eligible; 512 and 1,024 measured the same as 256.)
#ifndef CSG_SHORTCUT_LEAVES
#define CSG_SHORTCUT_LEAVES 256
#endif
constexpr int kShortcutLeaves = CSG_SHORTCUT_LEAVES;

// The one live leaf of [lo, hi] (a mask of one bit per leaf), or -1 if there are none or
// several.
template <class LM>
__device__ __forceinline__ int single_live_leaf(LM& lm, int lo, int hi)
{
    const int wa = lo >> 5, wb = hi >> 5;
    int found = -1;
    for (int k = wa; k <= wb; ++k) {
        if (!((lm.sum >> k) & 1u)) continue;
        uint32_t m = lm.word(k);
        if (k == wa) m &= 0xffffffffu << (lo & 31);
        if (k == wb) m &= 0xffffffffu >> (31 - (hi & 31));
        if (!m) continue;
        if (found >= 0 || (m & (m - 1u))) return -1;
        found = 32 * k + __ffs(m) - 1;
    }
    return found;
}

template <bool PRUNE, bool CYL, class LM>
__device__ __forceinline__ bool child_test(const Ray& ray, const DeviceScene& sc, float4 lo, float4 hi,
                                           int leaf_lo, int leaf_hi, Hit& H, float tmin, LM& lm,
                                           bool boxed = true, int dc = 0, bool skip_op = true, bool skip_leaf = true)
{
    const float4* __restrict__ geo = sc.geo;
    const bool may_skip = (skip_op && skip_leaf) || (__float_as_int(hi.w) < 0 ? skip_op : skip_leaf);
    if (PRUNE && may_skip && !lm.any(leaf_lo, leaf_hi)) {
        H.hit = kMiss;
        return false;
    }
    int32_t prim = __float_as_int(hi.w);
    if (PRUNE && skip_op && kShortcutLeaves > 0 && prim < 0 && sc.prepass && lm.shift == 0 &&
        leaf_hi - leaf_lo < kShortcutLeaves) {
        const int l = single_live_leaf(lm, leaf_lo, leaf_hi);
        if (l >= 0) {
            const float4 b1 = __ldg(&sc.lbox[2 * l + 1]);
            if ((__float_as_int(b1.w) >> 16) - 1 >= dc) {
                H.hit = kMiss;  // the path down to l holds an Intersection or a right-entered Difference
                return false;
            }
            lo = __ldg(&sc.lbox[2 * l]);
            hi = make_float4(b1.x, b1.y, b1.z, __int_as_float(l));
            prim = l;
        }
    }
    if (prim < 0) {
        const bool go = box_hit(ray, lo, hi, tmin);
        if (!go) {
            H.hit = kMiss;
            if (PRUNE) lm.clear_range(leaf_lo, leaf_hi, tmin);
        }
        return go;
    }
    const int32_t type = __float_as_int(lo.w);
    const float4 g0 = __ldg(&geo[2 * prim]);
    if (type == kSphere) {
        sphere_hit(ray, g0, prim, H, tmin);
        if (boxed && H.hit != kMiss && !box_hit(ray, lo, hi, tmin)) H.hit = kMiss;
    } else if (type == kCube) {
        cube_hit(ray, g0, prim, H, tmin);
    } else if (CYL && type == kCylinder) {
        if (!boxed || box_hit(ray, lo, hi, tmin)) {
            const float4 g1 = __ldg(&geo[2 * prim + 1]);
            cylinder_hit(ray, g0, g1, prim, H, tmin);
        } else {
            H.hit = kMiss;
        }
    } else {
        H = hit_default();
    }
    if (PRUNE && H.hit == kMiss) lm.clear_leaf(prim, tmin);
    return false;
}

// Per-ray traversal state of CSGRayCast (RaycastingKernels.cu:459-512), advanced one loop
// iteration at a time by tracer_step().
struct Tracer {
    Ray ray;
    Hit L, R;
    float tmin;
    int32_t cur;
    int4 ct;          // topology of `cur`; the virtual node CSGNode(0,0,0,0,0) is {0,0,0,Union}
    uint32_t action;
    ActionStack as;
    int32_t np, ntm;  // primitive / time stack depths (entries in shared memory)
    uint32_t it;
    bool run;
    bool ok;          // no push of this ray has been dropped (read by the 32-entry class: kGuard)

    __device__ __forceinline__ bool busy() const { return run || as.n > 0; }
};

template <class Stacks>
__device__ __forceinline__ void tracer_begin(Tracer& T, Stacks& st)
{
    T.as = ActionStack{0ull, 0};
    T.np = 0;
    T.ntm = 0;
    st.reset_bottom();
    T.tmin = 0.0f;
    T.cur = -1;
    T.ct = make_int4(0, 0, 0, kUnion);
    T.L = hit_default();
    T.R = hit_default();
    T.as.push(kCompute);
    T.action = kGotoL;
    T.run = true;
    T.ok = true;
    T.it = 0;
}

// GetParent (RaycastingKernels.cu:708-716)
__device__ __forceinline__ void tracer_parent(Tracer& T, const int4* __restrict__ topo)
{
    if (T.ct.z >= 0) {
        T.cur = T.ct.z;
        T.ct = __ldg(&topo[T.cur]);
    } else {
        T.run = false;
        T.cur = -1;
        T.ct = make_int4(0, 0, 0, kUnion);
    }
}

// Skipping work per stack class.  Live-leaf pruning, the single-leaf shortcut and the
// operator short-circuit skip subtrees, and a skipped traversal would have pushed and
// popped in pairs only if none of its pushes is dropped.  The classes below 32 entries are
// chosen so that no stack can overflow, and skip freely.  The 32-entry class (kGuard)
// reproduces the reference's drop-on-full stacks for trees deeper than 15 operator levels,
// where a push can be dropped; there a skip is taken only while no push of the ray has
// been dropped (Tracer::ok) and only under an operator whose height h leaves room for the
// skipped traversal: the operator's own pushes and its child's traversal add at most 2h
// actions and h entries to each of the other two stacks (two actions and one entry per
// operator level), so the action depth plus 2h and the other depths plus h must stay
// within 32.  Every open operator level holds at least as many actions as primitive and
// time entries together (two actions and a time, or one action and a primitive), and the
// bottom action is the initial Compute, so while no push has been dropped the primitive and
// time depths together stay below the action depth where GoTo and SaveLft decide (the
// oracle checks this on deep chains and random trees): then the action condition implies
// the other two, and a primitive or time push is never the first to be dropped, so only
// action pushes are watched (guard_room).  Before the first dropped push the traversal's
// state is the one an unbounded stack would hold, where every skip is exact; from the first
// one on nothing is skipped, and the rest of the traversal is the reference's own.  A
// leaf's test pushes nothing, so skipping it needs only the first condition.  (Skipping
// without the guard changes the oracle's renders of such trees wherever a stack
// overflows.)  The height is in bits 24-30 of the kids record's left leaf_hi, set for trees
// deeper than 15 levels.
template <int SD>
constexpr bool kGuard = SD >= 32;

__device__ __forceinline__ bool guard_room(const Tracer& T, int h) { return T.ok && T.as.n + 2 * h <= 32; }

// A loop re-enters one child of operator `node` with a tmin below that of a traversal
// clear: its leaves in the regions cleared above tmin become live again (the leaf ranges
// are the node's kids record).
template <class LM>
__device__ __forceinline__ void live_restore_child(LM& lm, const float4* __restrict__ kids, int node, bool right,
                                                   float tmin)
{
    const int4 rg = __ldg(reinterpret_cast<const int4*>(&kids[kKidsPerNode * node + 4]));
    if (right) lm.restore_range(rg.z, rg.w, tmin);
    else lm.restore_range(rg.x & 0x3fffffff, rg.y & 0xffff, tmin);
}

// Operator short-circuit (a tuning knob; 1 on).  Kensler's tables give Miss for a
// Difference whose left child is a Miss and for an Intersection with a Miss child, whatever
// the other child holds (the Miss rows and columns of those tables are all hMiss), and hMiss
// resets both records to the default Miss.  The reference still traverses the other child;
// skipping it changes no output: the node returns the same default Miss, tmin is restored by
// SaveLft or set by a loop before any later GoTo reads it, and the stacks are left as the
// skipped traversal would leave them (it pushes and pops in pairs when none of its pushes
// is dropped: always below the 32-entry class, and there where guard_room holds).  Skipped
// subtrees keep their live bits, which only prunes less.
// Scenes opt in (DeviceScene::short_circuit, chosen by the scene compiler).  The rolled
// variant carries the code always; the unrolled variant, which serves small trees and
// sphere/cube scenes such as the cheese frame, carries it only when instantiated with SCU
// (with it, the cheese frame, which never short-circuits, was 3-5% slower).  0 here
// removes it.
#ifndef CSG_SHORT_CIRCUIT
#define CSG_SHORT_CIRCUIT 1
#endif
constexpr bool kShortCircuit = CSG_SHORT_CIRCUIT != 0;

// One iteration of the CSGRayCast loop: SaveLft, GoTo (:514-595), Compute (:597-661) with
// LookUpActions (:664-706).  `tab` is the 27-entry table in shared memory.
// ROLLED evaluates GoTo's tests (both children of an operator, or the leaf GoTo landed on)
// in one rolled loop, so the primitive tests exist once in the code; the unrolled form
// overlaps the two children's tests and is faster when the code stays small (scenes
// without cylinders).  SCU: the unrolled form with the operator short-circuit.  CYL: the scene
// may hold cylinders.
template <int SD, bool ROLLED, bool SCU, bool CYL, class Stacks, class LM>
__device__ __forceinline__ void tracer_step(Tracer& T, const DeviceScene& sc, Stacks& st,
                                            const uint16_t* tab, LM& lm)
{
    constexpr bool kSC = kShortCircuit && (ROLLED || SCU);
    const int4* __restrict__ topo = sc.topo;
    const float4* __restrict__ kids = sc.kids;
    const float4* __restrict__ geo = sc.geo;
    ++T.it;
    st.np = T.np;
    st.ntm = T.ntm;
    // The step's action pushes.  In the 32-entry class a push onto a full stack (dropped,
    // as the reference drops it) ends all skipping for the ray (kGuard).
    auto apush = [&](uint32_t a) {
        if (kGuard<SD> && T.as.n >= 32) T.ok = false;
        T.as.push(a);
    };
    // the operator height in a kids record's range word (trees deeper than 15 levels)
    auto height = [](int ry) { return (ry >> 24) & 0x7f; };
    if (T.action & kSaveL) {
        T.tmin = st.tpop();
        if (kSC && sc.short_circuit && (T.L.hit & kMiss) &&
            (T.ct.w == kDifference || T.ct.w == kIntersection) &&
            (!kGuard<SD> ||
             (T.cur >= 0 &&
              guard_room(T, height(__ldg(reinterpret_cast<const int4*>(&kids[kKidsPerNode * T.cur + 4])).y))))) {
            // The left subtree returned a Miss: the node's Compute gives Miss whatever the
            // right subtree returns, so it is not traversed (the pending LoadL is dropped;
            // it would reload this same record).
            T.as.pop();
            T.action = kCompute;
        } else {
            st.ppush(T.L);
            T.action = kGotoR;
        }
    }
    if (T.action & (kGotoL | kGotoR)) {
        T.cur = (T.action & kGotoL) ? T.ct.x : T.ct.y;
        T.ct = __ldg(&topo[T.cur]);
        const bool op = T.ct.w <= kIntersection;
        bool gl = false, gr = false;
        // whether work under this node may be skipped (kGuard): for an operator child and
        // for a leaf
        bool skip_op = true;
        const bool skip_leaf = !kGuard<SD> || T.ok;
        if (ROLLED) {
            // the two children in the order the scene compiler chose (operator children,
            // then spheres, cubes, cylinders), so that a warp's lanes run one kind of test
            // at a time
            const float4* kn = &kids[kKidsPerNode * T.cur];
            const int nj = op ? 2 : 1;
            const bool leaf_right = !op && (T.action & kGotoR);
            int4 rg = make_int4(0, 0, 0, 0);
            if (op) rg = __ldg(reinterpret_cast<const int4*>(&kn[4]));
            const int first = (rg.x >> 30) & 1;
            const int dc = kGuard<SD> ? (rg.y >> 16) & 0xff : rg.y >> 16;
            if (kGuard<SD>) skip_op = guard_room(T, height(rg.y));
            rg.x &= 0x3fffffff;
            rg.y &= 0xffff;
#pragma unroll 1
            for (int k = 0; k < nj; ++k) {
                const int j = k ^ first;
                float4 lo, hi;
                int rlo, rhi;
                if (op) {
                    lo = __ldg(&kn[2 * j]);
                    hi = __ldg(&kn[2 * j + 1]);
                    rlo = j ? rg.z : rg.x;
                    rhi = j ? rg.w : rg.y;
                } else {
                    // GoTo landed on a leaf: one unboxed test into L or R
                    lo = make_float4(0.f, 0.f, 0.f, __int_as_float(T.ct.w));
                    hi = make_float4(0.f, 0.f, 0.f, __int_as_float(T.ct.x));
                    rlo = rhi = T.ct.x;
                }
                const bool right = (j == 1) || leaf_right;
                Hit H = right ? T.R : T.L;
                const bool go =
                    child_test<true, CYL>(T.ray, sc, lo, hi, rlo, rhi, H, T.tmin, lm, op, dc, skip_op, skip_leaf);
                if (right) {
                    T.R = H;
                    gr = go;
                } else {
                    T.L = H;
                    gl = go;
                }
            }
        } else if (op) {
            const float4* kn = &kids[kKidsPerNode * T.cur];
            const float4 k0 = __ldg(&kn[0]);
            const float4 k1 = __ldg(&kn[1]);
            const float4 k2 = __ldg(&kn[2]);
            const float4 k3 = __ldg(&kn[3]);
            const int4 rg = __ldg(reinterpret_cast<const int4*>(&kn[4]));
            const int dc = kGuard<SD> ? (rg.y >> 16) & 0xff : rg.y >> 16;
            if (kGuard<SD>) skip_op = guard_room(T, height(rg.y));
            gl = child_test<true, CYL>(T.ray, sc, k0, k1, rg.x & 0x3fffffff, rg.y & 0xffff, T.L, T.tmin, lm, true,
                                       dc, skip_op, skip_leaf);
            gr = child_test<true, CYL>(T.ray, sc, k2, k3, rg.z, rg.w, T.R, T.tmin, lm, true, dc, skip_op, skip_leaf);
        } else {
            Hit& H = (T.action & kGotoL) ? T.L : T.R;
            hit_primitive<CYL>(T.ray, geo, T.ct.w, T.ct.x, H, T.tmin);
            if (H.hit == kMiss) lm.clear_leaf(T.ct.x, T.tmin);
        }
        if (op) {
            // A child that is not descended into and holds a Miss is a Miss at this tmin
            // (a leaf's own test, a culled box or no live leaf).  A Difference whose left
            // child is such a Miss, or an Intersection with one, computes Miss whatever
            // the other child returns: go straight to Compute.
            const bool lmiss = !gl && (T.L.hit & kMiss), rmiss = !gr && (T.R.hit & kMiss);
            const bool decided = kSC && sc.short_circuit && skip_op &&
                                 ((T.ct.w == kDifference && lmiss) || (T.ct.w == kIntersection && (lmiss || rmiss)));
            if (decided) {
                T.action = kCompute;
            } else if (gl || gr) {
                if (!gl) {
                    st.ppush(T.L);
                    apush(kLoadL);
                    T.action = kGotoR;
                } else if (!gr) {
                    st.ppush(T.R);
                    apush(kLoadR);
                    T.action = kGotoL;
                } else {
                    st.tpush(T.tmin);
                    apush(kLoadL);
                    apush(kSaveL);
                    T.action = kGotoL;
                }
            } else {
                T.action = kCompute;
            }
        } else {
            T.action = T.as.pop();
            tracer_parent(T, topo);
        }
    }
    if (T.action & (kLoadL | kLoadR | kCompute)) {
        if (T.action & kLoadL) T.L = st.ppop();
        else if (T.action & kLoadR) T.R = st.ppop();
        // LookUpActions: Enter -> 0, Exit -> 1, Miss -> 2, tested in that order.
        uint32_t li = T.L.hit, ri = T.R.hit;
        li = (li & kEnter) ? 0u : li;
        li = (li & kExit) ? 1u : li;
        li = (li & kMiss) ? 2u : li;
        ri = (ri & kEnter) ? 0u : ri;
        ri = (ri & kExit) ? 1u : ri;
        ri = (ri & kMiss) ? 2u : ri;
        const uint32_t op = (uint32_t)T.ct.w;
        const uint32_t acts = (op <= 2u && li <= 2u && ri <= 2u) ? tab[op * 9 + li * 3 + ri] : 0xffffffffu;
        const bool lt = T.L.t < T.R.t, gt = T.L.t > T.R.t;
        if ((acts & hRetL) || ((acts & hRetLC) && lt)) {
            T.R = T.L;
            T.action = T.as.pop();
            tracer_parent(T, topo);
        } else if ((acts & hRetR) || ((acts & hRetRC) && gt)) {
            if (acts & hFlipR) T.R.hit ^= (kFlip | kExit | kEnter);
            T.L = T.R;
            T.action = T.as.pop();
            tracer_parent(T, topo);
        } else if ((acts & hLoopL) || ((acts & hLoopLC) && lt)) {
            T.tmin = T.L.t;
            if (!(T.tmin >= lm.tclr) && T.cur >= 0) live_restore_child(lm, kids, T.cur, false, T.tmin);
            st.ppush(T.R);
            apush(kLoadR);
            T.action = kGotoL;
        } else if ((acts & hLoopR) || ((acts & hLoopRC) && gt)) {
            T.tmin = T.R.t;
            if (!(T.tmin >= lm.tclr) && T.cur >= 0) live_restore_child(lm, kids, T.cur, true, T.tmin);
            st.ppush(T.L);
            apush(kLoadL);
            T.action = kGotoR;
        } else {
            T.R = hit_default();
            T.L = hit_default();
            T.action = T.as.pop();
            tracer_parent(T, topo);
        }
    }
    T.np = st.np;
    T.ntm = st.ntm;
}

// Whole traversal of one ray.  Returns the final hit (a default Miss if the ray was
// stopped at iter_cap; *capped is then set).
template <int SD, bool ROLLED, bool SCU, bool CYL, class Stacks, class LM>
__device__ __forceinline__ Hit csg_traverse(const DeviceScene& sc, const Ray& ray, Stacks& st,
                                            const uint16_t* tab, LM& lm, uint32_t iter_cap, bool* capped)
{
    Tracer T;
    T.ray = ray;
    tracer_begin(T, st);
    while (T.busy()) {
        if (T.it >= iter_cap) {
            *capped = true;
            return hit_default();
        }
        tracer_step<SD, ROLLED, SCU, CYL>(T, sc, st, tab, lm);
    }
    *capped = false;
    return T.L;
}

// Hit details (sphere/cylinder/cubeHitDetails, RaycastingKernels.cu:183-200, 338-373,
// 436-457): position and the normal, flipped once for Flip and once for Exit.
template <bool CYL = true>
__device__ __forceinline__ void hit_details(const Ray& ray, const float4* __restrict__ geo, const Hit& h,
                                            V3& P, V3& N)
{
    const float4 g0 = __ldg(&geo[2 * h.idx]);
    P = at3(ray.o, ray.d, h.t);
    const V3 cen = mk(g0.x, g0.y, g0.z);
    if (h.type == kSphere) {
        N = normalize3(sub3(P, cen));
    } else if (CYL && h.type == kCylinder) {
        const float4 g1 = __ldg(&geo[2 * h.idx + 1]);
        const V3 V = mk(g1.y, g1.z, g1.w);
        const V3 C = sub_scaled(cen, __fmul_rn(g1.x, 0.5f), V);
        const V3 OC = sub3(ray.o, C);
        if (h.hit & kFlag1) {
            N = neg3(V);
        } else if (h.hit & kFlag2) {
            N = V;
        } else {
            const float m = __fmaf_rn(dot3(ray.d, V), h.t, dot3(OC, V));
            N = normalize3(sub_scaled(sub3(P, C), m, V));
        }
    } else {
        const V3 PC = sub3(P, cen);
        const float bias = 1.00001f;  // `float bias = 1.00001;` rounds to the same float
        const float hs = __fmul_rn(g0.w, 0.5f);
        const V3 n = mk((float)(int)__fmul_rn(__fdiv_rn(PC.x, hs), bias),
                        (float)(int)__fmul_rn(__fdiv_rn(PC.y, hs), bias),
                        (float)(int)__fmul_rn(__fdiv_rn(PC.z, hs), bias));
        N = normalize3(n);
    }
    if (h.hit & kFlip) N = neg3(N);
    if (h.hit & kExit) N = neg3(N);
}

// LightningKernel (RaycastingKernels.cu:62-105): Phong with ka 0.2, kd 0.8, ks 0.7,
// shininess 30 and a white light; clamped to [0, 1].
__device__ __forceinline__ float4 phong(const float* cam, V3 light, V3 P, V3 N, float4 col)
{
    const V3 Ld = normalize3(light);
    const V3 Vd = normalize3(sub3(mk(cam[0], cam[1], cam[2]), P));
    const V3 nL = neg3(Ld);
    const V3 nn = normalize3(N);  // reflect (Float3Utils.cuh:39-44); its dot has the z(y(x)) shape
    const V3 Rd = sub_scaled(nL, __fmul_rn(2.0f, dot_zyx(nL, nn)), nn);
    const float diff = fmaxf(dot3(N, Ld), 0.0f);
    const float spec = powf(fmaxf(dot3(Vd, Rd), 0.0f), 30.0f);
    const float shade = __fmaf_rn(0.7f, spec, __fmaf_rn(0.8f, diff, 0.2f));
    return make_float4(fminf(fmaxf(__fmul_rn(col.x, shade), 0.0f), 1.0f),
                       fminf(fmaxf(__fmul_rn(col.y, shade), 0.0f), 1.0f),
                       fminf(fmaxf(__fmul_rn(col.z, shade), 0.0f), 1.0f), 1.0f);
}

__device__ __forceinline__ uint32_t quantize_rgba8(float4 c)
{
    const uint32_t r = __float2uint_rn(__fmul_rn(fminf(fmaxf(c.x, 0.0f), 1.0f), 255.0f));
    const uint32_t g = __float2uint_rn(__fmul_rn(fminf(fmaxf(c.y, 0.0f), 1.0f), 255.0f));
    const uint32_t b = __float2uint_rn(__fmul_rn(fminf(fmaxf(c.z, 0.0f), 1.0f), 255.0f));
    const uint32_t a = __float2uint_rn(__fmul_rn(fminf(fmaxf(c.w, 0.0f), 1.0f), 255.0f));
    return r | (g << 8) | (b << 16) | (a << 24);
}

}  // namespace dev
}  // namespace csgrt
