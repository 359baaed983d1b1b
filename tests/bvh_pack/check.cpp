// Checks the pre-pass BVH that pack_scene builds (csrc/scene.cpp) for each scene file given
// on the command line: every leaf is reached exactly once and every node once from the
// root, every inner slot's box holds its children's boxes, every slot's bounding sphere
// holds its box (a non-finite box gets an infinite radius), and a sphere leaf's slot
// carries the sphere itself with its radius negated.  Host code only; prints one line per
// violation and "scenes N bad M" at the end (scenes the parser rejects, and single
// primitives, which have no BVH, are not counted); exits 1 if any check failed.
#include "scene.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <set>
#include <sstream>
#include <vector>

using namespace csgrt;

static int32_t ival(float f)
{
    int32_t v;
    std::memcpy(&v, &f, 4);
    return v;
}

static bool finite_box(const float4& lo, const float4& hi)
{
    return std::isfinite(lo.x) && std::isfinite(lo.y) && std::isfinite(lo.z) && std::isfinite(hi.x) &&
           std::isfinite(hi.y) && std::isfinite(hi.z);
}

int main(int argc, char** argv)
{
    int bad = 0, scenes = 0;
    for (int i = 1; i < argc; ++i) {
        std::ifstream f(argv[i]);
        std::stringstream ss;
        ss << f.rdbuf();
        HostTree t;
        std::string err;
        if (parse_tree(ss.str(), t, err) != 0) continue;  // (the parser rejects it: no BVH to check)
        PackedScene pk;
        pack_scene(t, pk);
        const int np = static_cast<int>(t.prims.size()), nb = pk.bvh_nodes;
        if (np < 2) continue;
        ++scenes;
        if (pk.bvh.size() != static_cast<size_t>(6 * nb)) {
            std::printf("%s: %zu BVH records for %d nodes\n", argv[i], pk.bvh.size(), nb);
            ++bad;
            continue;
        }
        const float4* sph = pk.bvh.data() + 4 * nb;
        std::multiset<int> leaves;
        std::vector<int> seen(nb, 0), stack{0};
        while (!stack.empty()) {
            const int node = stack.back();
            stack.pop_back();
            if (node < 0 || node >= nb || seen[node]++) {
                std::printf("%s: node %d out of range or reached twice\n", argv[i], node);
                ++bad;
                continue;
            }
            for (int side = 0; side < 2; ++side) {
                const int e = 2 * node + side;
                const float4 lo = pk.bvh[2 * e], hi = pk.bvh[2 * e + 1], s = sph[e];
                const int c = ival(lo.w);
                if (c < 0) {
                    leaves.insert(~c);
                    if (ival(hi.w) == kSphere) {
                        const RefPrim& p = t.prims[static_cast<size_t>(~c)];
                        const bool same = (s.x == p.x || (s.x != s.x && p.x != p.x)) &&
                                          (s.y == p.y || (s.y != s.y && p.y != p.y)) &&
                                          (s.z == p.z || (s.z != s.z && p.z != p.z)) &&
                                          (ival(s.w) < 0 || s.w == 0.0f);
                        if (!same) {
                            std::printf("%s: sphere leaf %d record\n", argv[i], ~c);
                            ++bad;
                        }
                        continue;
                    }
                } else {
                    stack.push_back(c);
                    for (int q = 0; q < 2 && finite_box(lo, hi); ++q) {
                        const float4 l2 = pk.bvh[2 * (2 * c + q)], h2 = pk.bvh[2 * (2 * c + q) + 1];
                        if (finite_box(l2, h2) && (l2.x < lo.x || l2.y < lo.y || l2.z < lo.z || h2.x > hi.x ||
                                                   h2.y > hi.y || h2.z > hi.z)) {
                            std::printf("%s: slot %d does not hold its child's box\n", argv[i], e);
                            ++bad;
                        }
                    }
                }
                if (!finite_box(lo, hi)) {
                    if (!(s.w == INFINITY)) {
                        std::printf("%s: non-finite box of slot %d has radius %g\n", argv[i], e, s.w);
                        ++bad;
                    }
                    continue;
                }
                for (int m = 0; m < 8; ++m) {
                    const double x = (m & 1) ? hi.x : lo.x, y = (m & 2) ? hi.y : lo.y, z = (m & 4) ? hi.z : lo.z;
                    const double d = std::sqrt((x - s.x) * (x - s.x) + (y - s.y) * (y - s.y) + (z - s.z) * (z - s.z));
                    if (d > s.w) {
                        std::printf("%s: slot %d corner %g beyond radius %g\n", argv[i], e, d, s.w);
                        ++bad;
                        break;
                    }
                }
            }
        }
        if (static_cast<int>(leaves.size()) != np || static_cast<int>(std::set<int>(leaves.begin(), leaves.end()).size()) != np) {
            std::printf("%s: %zu leaf slots for %d primitives\n", argv[i], leaves.size(), np);
            ++bad;
        }
        for (int q = 0; q < nb; ++q)
            if (!seen[q]) {
                std::printf("%s: node %d unreached\n", argv[i], q);
                ++bad;
                break;
            }
    }
    std::printf("scenes %d bad %d\n", scenes, bad);
    return bad != 0;
}
