// Host checks of the hierarchy builders of csrc/bvh_build.cpp, without a GPU.
//
//   bvh_check <soup.f32> <threads>
//
// Reads a triangle soup (float32 [n][9]), builds the compressed 8-wide and the
// binary hierarchy with the given number of host threads (0: all cores), and
// checks what the traversal kernels rely on:
//   * the leaf order is a permutation of the triangles, and the leaves of the
//     hierarchy cover every position of it exactly once;
//   * every wide node is reached exactly once from the root, its internal
//     children lie in [child_base, child_base + internal count) and its leaf
//     triangles in [tri_base, tri_base + 24);
//   * every triangle lies inside the dequantised box of every slot on its path
//     (8-wide) and inside the child box of every node on its path (binary);
//   * the reported depths are the depths found, and at most kMaxBuildDepth.
// Prints "digest <hex>" over the bytes of both hierarchies, so that builds
// with different thread counts can be compared, and exits non-zero on the
// first failed check.
#include "dr_internal.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace dr;

namespace {

struct DBox {
    double lo[3], hi[3];
};

int g_fail = 0;

void fail(const char *what, long a = -1, long b = -1)
{
    if (g_fail++ < 10) std::fprintf(stderr, "FAIL: %s (%ld, %ld)\n", what, a, b);
}

bool tri_inside(const float *pos, uint32_t t, const DBox &b)
{
    for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
            const double x = pos[(size_t)t * 9 + v * 3 + a];
            if (!(x >= b.lo[a] && x <= b.hi[a])) return false;
        }
    return true;
}

uint64_t fnv(const void *p, size_t bytes, uint64_t h)
{
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < bytes; ++i) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

uint32_t byte_of(uint32_t w, uint32_t k) { return (w >> (8 * k)) & 0xffu; }

struct Check8 {
    const Bvh8 &b;
    const float *pos;
    uint32_t n;
    std::vector<int> visits, covered;
    std::vector<DBox> path;
    int max_depth = 0;

    void node(uint32_t i, int depth)
    {
        if (i >= b.nodes.size()) return fail("wide node index out of range", i);
        if (visits[i]++) return fail("wide node reached twice", i);
        max_depth = std::max(max_depth, depth);
        const Bvh8Node &nd = b.nodes[i];
        float p[3];
        std::memcpy(p, &nd.w[0], 12);
        const uint32_t imask = nd.w[0].w >> 24;
        const uint32_t child_base = nd.w[1].x, tri_base = nd.w[1].y;
        const uint32_t n_int = (uint32_t)__builtin_popcount(imask);
        if (n_int && (uint64_t)child_base + n_int > b.nodes.size()) fail("children beyond the node array", i);
        for (uint32_t s = 0; s < 8; ++s) {
            const uint32_t meta = byte_of(s < 4 ? nd.w[1].z : nd.w[1].w, s & 3u);
            DBox box;
            for (int a = 0; a < 3; ++a) {
                const int e = (int)byte_of(nd.w[0].w, a) - 127;
                const uint4 &q = nd.w[2 + a];
                const uint32_t qlo = byte_of(s < 4 ? q.x : q.y, s & 3u), qhi = byte_of(s < 4 ? q.z : q.w, s & 3u);
                box.lo[a] = (double)p[a] + std::ldexp((double)qlo, e);
                box.hi[a] = (double)p[a] + std::ldexp((double)qhi, e);
            }
            path.push_back(box);
            if ((imask >> s) & 1u) {
                if (meta != (0x20u | (24u + s))) fail("internal slot metadata", i, s);
                node(child_base + (uint32_t)__builtin_popcount(imask & ((1u << s) - 1u)), depth + 1);
            } else if (meta != 0) {
                const uint32_t cnt = (uint32_t)__builtin_popcount(meta >> 5), off = meta & 31u;
                if ((meta >> 5) != (1u << cnt) - 1u || off + cnt > 24) fail("leaf slot metadata", i, s);
                for (uint32_t k = 0; k < cnt; ++k) {
                    const uint64_t at = (uint64_t)tri_base + off + k;
                    if (at >= n) {
                        fail("leaf triangle beyond the order", i, (long)at);
                        continue;
                    }
                    ++covered[at];
                    for (const DBox &pb : path)
                        if (!tri_inside(pos, b.order[at], pb)) {
                            fail("triangle outside a wide slot box on its path", (long)at, i);
                            break;
                        }
                }
            }
            path.pop_back();
        }
    }
};

struct Check2 {
    const Bvh2 &b;
    const float *pos;
    uint32_t n;
    std::vector<int> visits, covered;
    std::vector<DBox> path;
    int max_depth = 0;

    void child(int32_t link, const DBox &box, int depth)
    {
        path.push_back(box);
        if (link >= 0) {
            node((uint32_t)link, depth + 1);
        } else {
            const uint32_t v = ~(uint32_t)link, first = v >> kLeafCountBits, count = v & kMaxLeafSize;
            for (uint32_t k = 0; k < count; ++k) {
                const uint64_t at = (uint64_t)first + k;
                if (at >= n) {
                    fail("binary leaf beyond the order", (long)at);
                    continue;
                }
                ++covered[at];
                for (const DBox &pb : path)
                    if (!tri_inside(pos, b.order[at], pb)) {
                        fail("triangle outside a binary child box on its path", (long)at);
                        break;
                    }
            }
            max_depth = std::max(max_depth, depth);
        }
        path.pop_back();
    }

    void node(uint32_t i, int depth)
    {
        if (i >= b.nodes.size()) return fail("binary node index out of range", i);
        if (visits[i]++) return fail("binary node reached twice", i);
        const Bvh2Node &nd = b.nodes[i];
        const DBox b0{{nd.c0xy.x, nd.c0xy.z, nd.cz.x}, {nd.c0xy.y, nd.c0xy.w, nd.cz.y}};
        const DBox b1{{nd.c1xy.x, nd.c1xy.z, nd.cz.z}, {nd.c1xy.y, nd.c1xy.w, nd.cz.w}};
        child(nd.link.x, b0, depth);
        child(nd.link.y, b1, depth);
    }
};

void check_order(const std::vector<uint32_t> &order, uint32_t n, const char *what)
{
    if (order.size() != n) return fail(what, (long)order.size(), n);
    std::vector<char> seen(n, 0);
    for (uint32_t t : order) {
        if (t >= n || seen[t]) return fail(what, t);
        seen[t] = 1;
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: bvh_check <soup.f32> <threads>\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<float> pos((size_t)bytes / 4);
    if (std::fread(pos.data(), 4, pos.size(), f) != pos.size()) return 2;
    std::fclose(f);
    const uint32_t n = (uint32_t)(pos.size() / 9);
    float mag = 0.0f;
    for (float v : pos) mag = std::max(mag, std::fabs(v));
    BuildParams bp;
    bp.threads = (uint32_t)std::atoi(argv[2]);
    const float slack = scene_slack(mag);

    const Bvh8 b8 = build_bvh8(pos.data(), n, bp, slack);
    check_order(b8.order, n, "8-wide leaf order is not a permutation");
    if (n > 0) {
        Check8 c{b8, pos.data(), n, std::vector<int>(b8.nodes.size(), 0), std::vector<int>(n, 0), {}, 0};
        c.node(0, 1);
        for (size_t i = 0; i < c.visits.size(); ++i)
            if (c.visits[i] != 1) fail("wide node not reached", (long)i);
        for (uint32_t k = 0; k < n; ++k)
            if (c.covered[k] != 1) fail("8-wide order position covered other than once", k, c.covered[k]);
        if (c.max_depth != b8.depth || b8.depth > kMaxBuildDepth) fail("8-wide depth", b8.depth, c.max_depth);
    }

    const Bvh2 b2 = build_bvh2(pos.data(), n, bp, slack);
    check_order(b2.order, n, "binary leaf order is not a permutation");
    if (n > 0) {
        Check2 c{b2, pos.data(), n, std::vector<int>(b2.nodes.size(), 0), std::vector<int>(n, 0), {}, 0};
        c.node(0, 0);
        for (size_t i = 0; i < c.visits.size(); ++i)
            if (c.visits[i] != 1) fail("binary node not reached", (long)i);
        for (uint32_t k = 0; k < n; ++k)
            if (c.covered[k] != 1) fail("binary order position covered other than once", k, c.covered[k]);
        if (b2.depth > kMaxBuildDepth) fail("binary depth", b2.depth);
    }

    uint64_t h = 1469598103934665603ull;
    h = fnv(b8.nodes.data(), b8.nodes.size() * sizeof(Bvh8Node), h);
    h = fnv(b8.order.data(), b8.order.size() * 4, h);
    h = fnv(b2.nodes.data(), b2.nodes.size() * sizeof(Bvh2Node), h);
    h = fnv(b2.order.data(), b2.order.size() * 4, h);
    std::printf("triangles %u wide_nodes %zu depth %d binary_nodes %zu digest %016llx\n", n, b8.nodes.size(), b8.depth,
                b2.nodes.size(), (unsigned long long)h);
    return g_fail ? 1 : 0;
}
