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
// Divisions and square roots are IEEE (the reference's default -prec-div/-prec-sqrt).
// Results -- hit, primitive, t, normal -- are therefore bit-identical to the
// reference kernel's on the same camera and scene bytes.
#pragma once

#include <cstdint>
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
};

// RaycastKernel ray generation (RaycastingKernels.cu:11-27) + the Ray constructor's
// second normalisation (Ray.cuh:12-18).  width/height are floats, as in the reference.
__device__ __forceinline__ Ray primary_ray(const float* cam, int x, int y, float width, float height)
{
    const float u = __fdiv_rn(__fadd_rn((float)x, 0.5f), __fsub_rn(width, 1.0f));
    const float v = __fdiv_rn(__fadd_rn((float)y, 0.5f), __fsub_rn(height, 1.0f));
    const float thf = tanf(__fdiv_rn(cam[5], 2.0f));
    const float nx = __fmul_rn(__fmul_rn(__fmaf_rn(2.0f, u, -1.0f), __fdiv_rn(width, height)), thf);
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
    return r;
}

// isBVHNodeHit (RaycastingKernels.cu:718-756): slab test with six divisions.
// Returns true when the box must be entered; a cull sets hit = Miss and keeps t, idx.
__device__ __forceinline__ bool box_hit(const Ray& r, float4 lo, float4 hi, float tmin)
{
    const float t1 = __fdiv_rn(__fsub_rn(lo.x, r.o.x), r.d.x);
    const float t2 = __fdiv_rn(__fsub_rn(hi.x, r.o.x), r.d.x);
    const float t3 = __fdiv_rn(__fsub_rn(lo.y, r.o.y), r.d.y);
    const float t4 = __fdiv_rn(__fsub_rn(hi.y, r.o.y), r.d.y);
    const float t5 = __fdiv_rn(__fsub_rn(lo.z, r.o.z), r.d.z);
    const float t6 = __fdiv_rn(__fsub_rn(hi.z, r.o.z), r.d.z);
    const float tmn = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmx = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    if (tmx < 0.0f) return false;
    if (tmn > tmx) return false;
    if (tmn <= tmin && tmx <= tmin) return false;
    return true;
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

// Cap-plane step of cylinderHit (RaycastingKernels.cu:238-266 / 273-301).
__device__ __forceinline__ void cylinder_caps(const Ray& r, V3 V, V3 OC, V3 cen, float h2, float hgt,
                                              float m, float& temp, bool& skip, int& use)
{
    if (m < 0.0f) {
        const V3 nV = neg3(V);
        const float den = dot3(r.d, nV);
        if (fabsf(den) < 0.0001f) {
            skip = true;
        } else {
            temp = __fdiv_rn(dot3(neg3(OC), nV), den);
            use = 1;
        }
    }
    if (m > hgt) {
        const float den = dot3(r.d, V);
        if (fabsf(den) < 0.0001f) {
            skip = true;
        } else {
            const V3 ocm = sub_scaled(sub3(r.o, cen), h2, V);
            temp = __fdiv_rn(dot3(neg3(ocm), V), den);
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
    const float h2 = __fdiv_rn(hgt, 2.0f);
    const V3 C = sub_scaled(cen, h2, V);
    const V3 OC = sub3(r.o, C);
    const float dV = dot3(r.d, V);
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
    float temp = t1, m = m1;
    bool skip = false;
    int use = 0;
    cylinder_caps(r, V, OC, cen, h2, hgt, m, temp, skip, use);
    if (temp <= tmin || skip) {
        temp = t2;
        m = m2;
        skip = false;
        use = 0;
        cylinder_caps(r, V, OC, cen, h2, hgt, m, temp, skip, use);
        if (temp <= tmin || skip) return;
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
    const float s2 = __fdiv_rn(g0.w, 2.0f);
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

// hitPrimitive (RaycastingKernels.cu:113-133)
__device__ __forceinline__ void hit_primitive(const Ray& r, const float4* __restrict__ geo, int32_t type,
                                              int32_t prim, Hit& h, float tmin)
{
    const float4 g0 = __ldg(&geo[2 * prim]);
    if (type == kSphere) {
        sphere_hit(r, g0, prim, h, tmin);
    } else if (type == kCylinder) {
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
};

// CSGRayCast (RaycastingKernels.cu:459-512) with GoTo (:514-595), Compute (:597-661),
// LookUpActions (:664-706) and GetParent (:708-716).  `tab` is the 27-entry table in
// shared memory.  Returns the final hit; *iters receives the loop count (kIterCap+1 if
// the ray was stopped).
template <int SD>
__device__ __forceinline__ Hit csg_traverse(const DeviceScene& sc, const Ray& ray, SmemStacks<SD>& st,
                                            const uint16_t* tab, uint32_t iter_cap, uint32_t* iters)
{
    const int4* __restrict__ topo = sc.topo;
    const float4* __restrict__ kids = sc.kids;
    const float4* __restrict__ geo = sc.geo;

    ActionStack as{0ull, 0};
    st.np = 0;
    st.ntm = 0;
    // Slot 0 of the primitive and time stacks is what an empty pop returns.
    st.pt[st.tid] = -1.0f;
    st.pb[st.tid] = kMiss | (0xffffu << 16);
    st.tt[st.tid] = 0.0f;

    float tmin = 0.0f;
    int cur = -1;
    int4 ct = make_int4(0, 0, 0, kUnion);  // the virtual node CSGNode(0,0,0,0,0)
    Hit L = hit_default(), R = hit_default();
    as.push(kCompute);
    uint32_t action = kGotoL;
    bool run = true;
    uint32_t it = 0;

    auto parent = [&]() {
        if (ct.z >= 0) {
            cur = ct.z;
            ct = __ldg(&topo[cur]);
        } else {
            run = false;
            cur = -1;
            ct = make_int4(0, 0, 0, kUnion);
        }
    };

    while (run || as.n > 0) {
        if (++it > iter_cap) {
            *iters = it;
            return hit_default();
        }
        if (action & kSaveL) {
            tmin = st.tpop();
            st.ppush(L);
            action = kGotoR;
        }
        if (action & (kGotoL | kGotoR)) {
            cur = (action & kGotoL) ? ct.x : ct.y;
            ct = __ldg(&topo[cur]);
            if (ct.w <= kIntersection) {
                const float4 k0 = __ldg(&kids[4 * cur + 0]);
                const float4 k1 = __ldg(&kids[4 * cur + 1]);
                const float4 k2 = __ldg(&kids[4 * cur + 2]);
                const float4 k3 = __ldg(&kids[4 * cur + 3]);
                bool gl = box_hit(ray, k0, k1, tmin);
                bool gr = box_hit(ray, k2, k3, tmin);
                if (!gl) L.hit = kMiss;
                if (!gr) R.hit = kMiss;
                const int32_t lprim = __float_as_int(k1.w), rprim = __float_as_int(k3.w);
                if (gl && lprim != -1) {
                    hit_primitive(ray, geo, __float_as_int(k0.w), lprim, L, tmin);
                    gl = false;
                }
                if (gr && rprim != -1) {
                    hit_primitive(ray, geo, __float_as_int(k2.w), rprim, R, tmin);
                    gr = false;
                }
                if (gl || gr) {
                    if (!gl) {
                        st.ppush(L);
                        as.push(kLoadL);
                        action = kGotoR;
                    } else if (!gr) {
                        st.ppush(R);
                        as.push(kLoadR);
                        action = kGotoL;
                    } else {
                        st.tpush(tmin);
                        as.push(kLoadL);
                        as.push(kSaveL);
                        action = kGotoL;
                    }
                } else {
                    action = kCompute;
                }
            } else {
                if (action & kGotoL) hit_primitive(ray, geo, ct.w, ct.x, L, tmin);
                else hit_primitive(ray, geo, ct.w, ct.x, R, tmin);
                action = as.pop();
                parent();
            }
        }
        if (action & (kLoadL | kLoadR | kCompute)) {
            if (action & kLoadL) L = st.ppop();
            else if (action & kLoadR) R = st.ppop();
            // LookUpActions: Enter -> 0, Exit -> 1, Miss -> 2, tested in that order.
            uint32_t li = L.hit, ri = R.hit;
            li = (li & kEnter) ? 0u : li;
            li = (li & kExit) ? 1u : li;
            li = (li & kMiss) ? 2u : li;
            ri = (ri & kEnter) ? 0u : ri;
            ri = (ri & kExit) ? 1u : ri;
            ri = (ri & kMiss) ? 2u : ri;
            const uint32_t op = (uint32_t)ct.w;
            const uint32_t acts = (op <= 2u && li <= 2u && ri <= 2u) ? tab[op * 9 + li * 3 + ri] : 0xffffffffu;
            if ((acts & hRetL) || ((acts & hRetLC) && (L.t < R.t))) {
                R = L;
                action = as.pop();
                parent();
            } else if ((acts & hRetR) || ((acts & hRetRC) && (L.t > R.t))) {
                if (acts & hFlipR) R.hit ^= (kFlip | kExit | kEnter);
                L = R;
                action = as.pop();
                parent();
            } else if ((acts & hLoopL) || ((acts & hLoopLC) && (L.t < R.t))) {
                tmin = L.t;
                st.ppush(R);
                as.push(kLoadR);
                action = kGotoL;
            } else if ((acts & hLoopR) || ((acts & hLoopRC) && (L.t > R.t))) {
                tmin = R.t;
                st.ppush(L);
                as.push(kLoadL);
                action = kGotoR;
            } else {
                R = hit_default();
                L = hit_default();
                action = as.pop();
                parent();
            }
        }
    }
    *iters = it;
    return L;
}

// Hit details (sphere/cylinder/cubeHitDetails, RaycastingKernels.cu:183-200, 338-373,
// 436-457): position and the normal, flipped once for Flip and once for Exit.
__device__ __forceinline__ void hit_details(const Ray& ray, const float4* __restrict__ geo, const Hit& h,
                                            V3& P, V3& N)
{
    const float4 g0 = __ldg(&geo[2 * h.idx]);
    P = at3(ray.o, ray.d, h.t);
    const V3 cen = mk(g0.x, g0.y, g0.z);
    if (h.type == kSphere) {
        N = normalize3(sub3(P, cen));
    } else if (h.type == kCylinder) {
        const float4 g1 = __ldg(&geo[2 * h.idx + 1]);
        const V3 V = mk(g1.y, g1.z, g1.w);
        const V3 C = sub_scaled(cen, __fdiv_rn(g1.x, 2.0f), V);
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
        const float hs = __fdiv_rn(g0.w, 2.0f);
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
    const V3 nn = normalize3(N);  // reflect (Float3Utils.cuh:39-44)
    const V3 Rd = sub_scaled(nL, __fmul_rn(2.0f, dot3(nL, nn)), nn);
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
