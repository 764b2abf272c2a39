// kdtree_build.cpp - host kd-tree builder.
//
// Produces the same node stream, word for word, as the reference builder
// (src/ref/kdtree_builder.cpp): SAH over sorted bounding-box edges with the
// empty-space bonus 0.3 and the leaf threshold of 2 primitives (:8-9), the
// depth limit 8 + 1.3*floor(log2 N) capped at 40 (src/ref/kdtree.cpp:199-203),
// triangle clipping of straddling primitives (:17-93), DFS node order with the
// below child at node+1 (:286-301) and leaves that store their sorted
// primitive indices in place (:304-321).
//
// What differs is the execution: children of large nodes are built
// concurrently into private node arrays and spliced into the parent's array
// with their interior above-child indices relocated, and primitive lists are
// per-node vectors instead of one shared scratch buffer.  Neither changes the
// output: every node's primitive list keeps the order the reference produces
// (the order of the split axis' sorted edge list), so stable sorting gives the
// same ties and the same split edge.
#include "yar_gpu.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <new>
#include <vector>

namespace {

constexpr float kEmptyNodeBonus = 0.3f;          // src/ref/kdtree_builder.cpp:8
constexpr uint32_t kLeafPrimitiveThreshold = 2;  // src/ref/kdtree_builder.cpp:9
constexpr int kMaxTraversalDepth = 40;           // src/ref/kdtree.cpp:10
constexpr uint32_t kMaxNodeCount = 0x40000000u;  // src/ref/kdtree.h:23
constexpr uint32_t kMaxPrimitiveCount = 0x3fffffffu;
constexpr uint32_t kParallelThreshold = 32768;   // primitives in a node worth a task

// std::min/std::max argument semantics (return the first argument on ties and
// on unordered comparisons), which the reference relies on for -0.0/+0.0.
inline float fmin_std(float a, float b) { return (b < a) ? b : a; }
inline float fmax_std(float a, float b) { return (a < b) ? b : a; }

struct Box {
    float mn[3];
    float mx[3];
};

struct Prim {
    uint32_t index;  // primitive index in the mesh / object list
    Box bounds;
};

// Edge of a primitive's bounds along one axis (src/ref/kdtree_builder.cpp:96-126).
struct Edge {
    float pos;
    uint32_t bits;  // local primitive index | end flag | perpendicular flag
    static constexpr uint32_t kEnd = 0x80000000u;
    static constexpr uint32_t kPerp = 0x40000000u;
    static constexpr uint32_t kMask = 0x3fffffffu;
    bool is_end() const { return (bits & kEnd) != 0; }
    bool is_start() const { return !is_end(); }
    bool perpendicular() const { return (bits & kPerp) != 0; }
    uint32_t local() const { return bits & kMask; }
};

inline bool edge_less(const Edge& a, const Edge& b) {
    if (a.pos == b.pos) return a.is_end() && b.is_start();
    return a.pos < b.pos;
}

struct Tri_Source {
    const float* vertices;
    const int32_t* indices;
    void positions(uint32_t tri, float p[3][3]) const {
        const int32_t* i = indices + 3 * (size_t)tri;
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) p[k][c] = vertices[3 * (size_t)i[k] + c];
    }
};

// clip_bounds, src/ref/kdtree_builder.cpp:17-93.
void clip_to_triangle(const Tri_Source& mesh, uint32_t tri, float split, int axis, bool left, Box& b) {
    if (left) b.mx[axis] = split;
    else b.mn[axis] = split;

    float p[3][3];
    mesh.positions(tri, p);
    auto swap3 = [](float* x, float* y) { for (int c = 0; c < 3; c++) std::swap(x[c], y[c]); };
    if (p[1][axis] < p[0][axis]) swap3(p[1], p[0]);
    if (p[2][axis] < p[0][axis]) swap3(p[2], p[0]);
    if (p[2][axis] < p[1][axis]) swap3(p[2], p[1]);

    const bool middle_left = p[1][axis] < split;
    const float* a = middle_left ? p[2] : p[0];
    const float* c = middle_left ? p[0] : p[2];
    const float* bb = p[1];

    const float eps = ((left && !middle_left) || (!left && middle_left)) ? 1e-5f : -1e-5f;
    float isect_ab[3], isect_ac[3];
    {
        float ab[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
        float s = (split - a[axis]) / ab[axis] + eps;
        for (int k = 0; k < 3; k++) isect_ab[k] = a[k] + ab[k] * s;
        float ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        float s2 = (split - a[axis]) / ac[axis] + eps;
        for (int k = 0; k < 3; k++) isect_ac[k] = a[k] + ac[k] * s2;
    }
    // Bounding_Box() starts at (+inf, -inf); add_point uses std::min/std::max.
    Box b2;
    for (int k = 0; k < 3; k++) { b2.mn[k] = INFINITY; b2.mx[k] = -INFINITY; }
    auto add = [&](const float* q) {
        for (int k = 0; k < 3; k++) {
            b2.mn[k] = fmin_std(b2.mn[k], q[k]);
            b2.mx[k] = fmax_std(b2.mx[k], q[k]);
        }
    };
    add(isect_ab);
    add(isect_ac);
    if (left) {
        add(p[0]);
        if (middle_left) add(p[1]);
    } else {
        add(p[2]);
        if (!middle_left) add(p[1]);
    }
    // Bounding_Box::compute_intersection (src/lib/bounding_box.h:98-111)
    for (int k = 0; k < 3; k++) {
        b.mn[k] = fmax_std(b.mn[k], b2.mn[k]);
        b.mx[k] = fmin_std(b.mx[k], b2.mx[k]);
    }
}

struct Subtree {
    std::vector<yar_kd_node> nodes;
    std::vector<uint32_t> interior;  // positions of interior nodes (for relocation)
};

struct Builder {
    const Tri_Source* mesh = nullptr;  // null for the scene tree (no clipping)
    int max_parallel = 1;
    std::atomic<int> active_tasks{0};
    std::atomic<bool> overflow{false};

    struct Scratch {
        std::vector<Edge> edges[3];
    };

    static void make_leaf(const std::vector<Prim>& prims, Subtree& out) {
        // KdNode::init_leaf + create_leaf (src/ref/kdtree.h:36-42, src/ref/kdtree_builder.cpp:304-321)
        const uint32_t count = (uint32_t)prims.size();
        const size_t first = out.nodes.size();
        out.nodes.push_back(yar_kd_node{3u | (count << 2), 0xffffffffu});
        if (count > 1) out.nodes.insert(out.nodes.end(), count / 2, yar_kd_node{0u, 0u});
        std::vector<uint32_t> idx(count);
        for (uint32_t i = 0; i < count; i++) idx[i] = prims[i].index;
        std::sort(idx.begin(), idx.end());
        uint32_t* words = &out.nodes[first].word1;
        for (uint32_t i = 0; i < count; i++) words[i] = idx[i];
    }

    // select_split_for_axis, src/ref/kdtree_builder.cpp:359-423
    static float sweep_axis(const Box& nb, const std::vector<Edge>& edges, uint32_t count, int axis,
                            uint32_t* split_edge) {
        static constexpr int other[3][2] = {{1, 2}, {0, 2}, {0, 1}};
        const int o0 = other[axis][0], o1 = other[axis][1];
        const float diag[3] = {nb.mx[0] - nb.mn[0], nb.mx[1] - nb.mn[1], nb.mx[2] - nb.mn[2]};
        const float s0 = 2.0f * (diag[o0] * diag[o1]);
        const float d0 = 2.0f * (diag[o0] + diag[o1]);
        const float inv_total_area = 1.0f / (2.0f * (diag[0] * diag[1] + diag[0] * diag[2] + diag[1] * diag[2]));
        const uint32_t num_edges = 2 * count;
        float best_cost = (float)count;
        uint32_t best_edge = 0xffffffffu;
        uint32_t num_below = 0, num_above = count;
        uint32_t i = 0;
        while (i < num_edges) {
            const float t = edges[i].pos;
            uint32_t group_end = i + 1;
            while (group_end < num_edges && t == edges[group_end].pos) group_end++;
            uint32_t middle = i;
            while (middle != group_end && edges[middle].is_end()) middle++;
            num_above -= middle - i;
            if (t > nb.mn[axis] && t < nb.mx[axis]) {
                const float below_area = s0 + d0 * (t - nb.mn[axis]);
                const float above_area = s0 + d0 * (nb.mx[axis] - t);
                const float p_below = below_area * inv_total_area;
                const float p_above = above_area * inv_total_area;
                const float bonus = (num_below == 0 || num_above == 0) ? kEmptyNodeBonus : 0.0f;
                const float expected = p_below * num_below + p_above * num_above;
                const float cost = (1.f - bonus) * expected;
                if (cost < best_cost) {
                    best_edge = (middle == group_end) ? middle - 1 : middle;
                    best_cost = cost;
                }
            }
            num_below += group_end - middle;
            i = group_end;
        }
        if (best_edge == 0xffffffffu) return INFINITY;
        *split_edge = best_edge;
        return best_cost;
    }

    // build_node, src/ref/kdtree_builder.cpp:207-302
    void build(const Box& nb, std::vector<Prim>& prims, int depth, Subtree& out, Scratch& scratch) {
        if (out.nodes.size() >= kMaxNodeCount) { overflow = true; return; }
        const uint32_t count = (uint32_t)prims.size();
        if (count <= kLeafPrimitiveThreshold || depth == 0) {
            make_leaf(prims, out);
            return;
        }
        // select_split (:323-357): edges of all three axes, stable-sorted
        float best_cost = INFINITY;
        int best_axis = -1;
        uint32_t best_edge = 0;
        for (int axis = 0; axis < 3; axis++) {
            std::vector<Edge>& e = scratch.edges[axis];
            e.resize(2 * (size_t)count);
            for (uint32_t i = 0; i < count; i++) {
                const Box& b = prims[i].bounds;
                uint32_t perp = (b.mn[axis] == b.mx[axis]) ? Edge::kPerp : 0u;
                e[2 * i + 0] = Edge{b.mn[axis], i | perp};
                e[2 * i + 1] = Edge{b.mx[axis], i | Edge::kEnd | perp};
            }
            std::stable_sort(e.begin(), e.end(), edge_less);
            uint32_t edge;
            float cost = sweep_axis(nb, e, count, axis, &edge);
            if (cost < best_cost) {
                best_cost = cost;
                best_axis = axis;
                best_edge = edge;
            }
        }
        if (best_axis == -1) {
            make_leaf(prims, out);
            return;
        }
        const std::vector<Edge>& e = scratch.edges[best_axis];
        const float split = e[best_edge].pos;

        // classification (:256-284)
        std::vector<Prim> below, above;
        below.reserve(count);
        above.reserve(count);
        for (uint32_t i = 0; i < best_edge; i++) {
            const Edge ed = e[i];
            if (ed.is_start() || (ed.pos == split && ed.perpendicular())) {
                Prim p = prims[ed.local()];
                if (p.bounds.mx[best_axis] > split && mesh)
                    clip_to_triangle(*mesh, p.index, split, best_axis, true, p.bounds);
                below.push_back(p);
            }
        }
        for (uint32_t i = best_edge + 1; i < 2 * count; i++) {
            const Edge ed = e[i];
            if (ed.is_end()) {
                Prim p = prims[ed.local()];
                if (p.bounds.mn[best_axis] < split && mesh)
                    clip_to_triangle(*mesh, p.index, split, best_axis, false, p.bounds);
                above.push_back(p);
            }
        }
        std::vector<Prim>().swap(prims);  // release the parent's list early

        const uint32_t this_node = (uint32_t)out.nodes.size();
        out.nodes.push_back(yar_kd_node{0u, 0u});
        out.interior.push_back(this_node);

        Box b0 = nb;
        b0.mx[best_axis] = split;
        Box b1 = nb;
        b1.mn[best_axis] = split;
        uint32_t split_bits;
        memcpy(&split_bits, &split, 4);

        const bool spawn = max_parallel > 1 && above.size() >= kParallelThreshold &&
                           below.size() >= kParallelThreshold && active_tasks.load() < max_parallel - 1;
        if (spawn) {
            active_tasks++;
            Subtree above_tree;
            auto fut = std::async(std::launch::async, [&] {
                Scratch s2;
                build(b1, above, depth - 1, above_tree, s2);
                active_tasks--;
            });
            build(b0, below, depth - 1, out, scratch);
            fut.get();
            const uint32_t above_child = (uint32_t)out.nodes.size();
            out.nodes[this_node] = yar_kd_node{(uint32_t)best_axis | (above_child << 2), split_bits};
            // splice with relocation of the interior nodes' above-child indices
            for (uint32_t k : above_tree.interior) {
                yar_kd_node& n = above_tree.nodes[k];
                n.word0 = (n.word0 & 3u) | (((n.word0 >> 2) + above_child) << 2);
                out.interior.push_back(k + above_child);
            }
            out.nodes.insert(out.nodes.end(), above_tree.nodes.begin(), above_tree.nodes.end());
        } else {
            build(b0, below, depth - 1, out, scratch);
            const uint32_t above_child = (uint32_t)out.nodes.size();
            out.nodes[this_node] = yar_kd_node{(uint32_t)best_axis | (above_child << 2), split_bits};
            build(b1, above, depth - 1, out, scratch);
        }
        if (out.nodes.size() >= kMaxNodeCount) overflow = true;
    }
};

int max_depth_limit(uint32_t primitive_count) {
    // KdTree::get_max_depth_limit, src/ref/kdtree.cpp:199-203
    int depth = (int)std::lround(8.0 + 1.3 * std::floor(std::log2((double)primitive_count)));
    return std::min(depth, kMaxTraversalDepth);
}

int finish(Builder& b, std::vector<Prim>& prims, const Box& total, int threads, float bounds_out[6],
           yar_kd_node** nodes_out, uint32_t* node_count_out) {
    b.max_parallel = std::max(1, threads);
    Subtree tree;
    Builder::Scratch scratch;
    const int depth = max_depth_limit((uint32_t)prims.size());
    b.build(total, prims, depth, tree, scratch);
    if (b.overflow) return YAR_ERR_CAPACITY;
    yar_kd_node* nodes = (yar_kd_node*)malloc(std::max<size_t>(1, tree.nodes.size()) * sizeof(yar_kd_node));
    if (!nodes) return YAR_ERR_NOMEM;
    if (!tree.nodes.empty()) memcpy(nodes, tree.nodes.data(), tree.nodes.size() * sizeof(yar_kd_node));
    memcpy(bounds_out, total.mn, 12);
    memcpy(bounds_out + 3, total.mx, 12);
    *nodes_out = nodes;
    *node_count_out = (uint32_t)tree.nodes.size();
    return YAR_OK;
}

Box empty_box() {
    Box b;
    for (int k = 0; k < 3; k++) { b.mn[k] = INFINITY; b.mx[k] = -INFINITY; }
    return b;
}

void box_union(Box& total, const Box& b) {
    // Bounding_Box::compute_union (src/lib/bounding_box.h:87-96)
    for (int k = 0; k < 3; k++) {
        total.mn[k] = fmin_std(total.mn[k], b.mn[k]);
        total.mx[k] = fmax_std(total.mx[k], b.mx[k]);
    }
}

} // namespace

extern "C" int yar_build_mesh_kdtree(const float* vertices, uint32_t vertex_count, const int32_t* indices,
                                     uint32_t triangle_count, int32_t thread_count, float bounds_out[6],
                                     yar_kd_node** nodes_out, uint32_t* node_count_out) {
    if (!vertices || !indices || !bounds_out || !nodes_out || !node_count_out) return YAR_ERR_INVALID;
    if (triangle_count == 0 || triangle_count > kMaxPrimitiveCount) return YAR_ERR_INVALID;
    for (size_t i = 0; i < 3 * (size_t)triangle_count; i++)
        if (indices[i] < 0 || (uint32_t)indices[i] >= vertex_count) return YAR_ERR_INVALID;
    try {
        Tri_Source src{vertices, indices};
        std::vector<Prim> prims(triangle_count);
        Box total = empty_box();
        for (uint32_t t = 0; t < triangle_count; t++) {
            // Triangle_Mesh::get_triangle_bounds (src/lib/triangle_mesh.h:91-98)
            float p[3][3];
            src.positions(t, p);
            Box b;
            for (int k = 0; k < 3; k++) { b.mn[k] = p[0][k]; b.mx[k] = p[0][k]; }
            for (int v = 1; v < 3; v++)
                for (int k = 0; k < 3; k++) {
                    b.mn[k] = fmin_std(b.mn[k], p[v][k]);
                    b.mx[k] = fmax_std(b.mx[k], p[v][k]);
                }
            prims[t] = Prim{t, b};
            box_union(total, b);
        }
        Builder builder;
        builder.mesh = &src;
        return finish(builder, prims, total, thread_count, bounds_out, nodes_out, node_count_out);
    } catch (const std::bad_alloc&) {
        return YAR_ERR_NOMEM;
    }
}

extern "C" int yar_build_scene_kdtree(const float* object_bounds, uint32_t object_count, float bounds_out[6],
                                      yar_kd_node** nodes_out, uint32_t* node_count_out) {
    if (!object_bounds || !bounds_out || !nodes_out || !node_count_out) return YAR_ERR_INVALID;
    if (object_count == 0 || object_count > kMaxPrimitiveCount) return YAR_ERR_INVALID;
    try {
        std::vector<Prim> prims(object_count);
        Box total = empty_box();
        for (uint32_t i = 0; i < object_count; i++) {
            Box b;
            memcpy(b.mn, object_bounds + 6 * (size_t)i, 12);
            memcpy(b.mx, object_bounds + 6 * (size_t)i + 3, 12);
            prims[i] = Prim{i, b};
            box_union(total, b);
        }
        Builder builder;
        return finish(builder, prims, total, 1, bounds_out, nodes_out, node_count_out);
    } catch (const std::bad_alloc&) {
        return YAR_ERR_NOMEM;
    }
}

extern "C" void yar_free_nodes(yar_kd_node* nodes) { free(nodes); }

extern "C" void yar_transform_bounds(const float m[12], const float in[6], float out[6]) {
    // transform_bounding_box + transform_point (src/lib/matrix.cpp:368-402):
    // the eight corners in the reference's order, accumulated with add_point.
    Box b = empty_box();
    for (int corner = 0; corner < 8; corner++) {
        const float x = (corner & 4) ? in[3] : in[0];
        const float y = (corner & 2) ? in[4] : in[1];
        const float z = (corner & 1) ? in[5] : in[2];
        float p[3];
        for (int r = 0; r < 3; r++) p[r] = m[4 * r + 0] * x + m[4 * r + 1] * y + m[4 * r + 2] * z + m[4 * r + 3];
        for (int k = 0; k < 3; k++) {
            b.mn[k] = fmin_std(b.mn[k], p[k]);
            b.mx[k] = fmax_std(b.mx[k], p[k]);
        }
    }
    memcpy(out, b.mn, 12);
    memcpy(out + 3, b.mx, 12);
}

// ---------------------------------------------------------------- cache files
// The reference's kd-tree cache file (KdTree::save / KdTree::load,
// src/ref/kdtree.cpp:111-160): bounds (min xyz, max xyz as 6 float32),
// the 64-bit geometry hash, the 32-bit node count, then the 8-byte nodes,
// all little-endian.  The reference writes hash 0 (its hash functions are
// stubs returning 0, src/ref/kdtree.cpp:205-215); `hash_out` returns what the
// file holds and the writer takes the value to store.
extern "C" int yar_read_kdtree_cache(const char* path, float bounds_out[6], uint64_t* hash_out,
                                     yar_kd_node** nodes_out, uint32_t* node_count_out) {
    if (!path || !bounds_out || !nodes_out || !node_count_out) return YAR_ERR_INVALID;
    *nodes_out = nullptr;
    *node_count_out = 0;
    FILE* f = fopen(path, "rb");
    if (!f) return YAR_ERR_IO;
    float bounds[6];
    uint64_t hash = 0;
    uint32_t count = 0;
    int rc = YAR_OK;
    if (fread(bounds, 4, 6, f) != 6 || fread(&hash, 8, 1, f) != 1 || fread(&count, 4, 1, f) != 1) rc = YAR_ERR_IO;
    if (rc == YAR_OK && (count == 0 || count > (1u << 31) / sizeof(yar_kd_node))) rc = YAR_ERR_INVALID;
    yar_kd_node* nodes = nullptr;
    if (rc == YAR_OK) {
        nodes = static_cast<yar_kd_node*>(malloc((size_t)count * sizeof(yar_kd_node)));
        if (!nodes) rc = YAR_ERR_NOMEM;
    }
    if (rc == YAR_OK && fread(nodes, sizeof(yar_kd_node), count, f) != count) rc = YAR_ERR_IO;
    if (rc == YAR_OK && fgetc(f) != EOF) rc = YAR_ERR_INVALID;  // trailing bytes: not a cache file
    fclose(f);
    if (rc != YAR_OK) {
        free(nodes);
        return rc;
    }
    memcpy(bounds_out, bounds, sizeof(bounds));
    if (hash_out) *hash_out = hash;
    *nodes_out = nodes;
    *node_count_out = count;
    return YAR_OK;
}

extern "C" int yar_write_kdtree_cache(const char* path, const float bounds[6], uint64_t hash,
                                      const yar_kd_node* nodes, uint32_t node_count) {
    if (!path || !bounds || !nodes || node_count == 0) return YAR_ERR_INVALID;
    FILE* f = fopen(path, "wb");
    if (!f) return YAR_ERR_IO;
    bool ok = fwrite(bounds, 4, 6, f) == 6 && fwrite(&hash, 8, 1, f) == 1 && fwrite(&node_count, 4, 1, f) == 1 &&
              fwrite(nodes, sizeof(yar_kd_node), node_count, f) == node_count;
    ok = (fclose(f) == 0) && ok;
    return ok ? YAR_OK : YAR_ERR_IO;
}
