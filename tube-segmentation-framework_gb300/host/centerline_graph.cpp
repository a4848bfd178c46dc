// centerline_graph.cpp -- the host part of runNewCenterlineAlg when loop
// removal or a VTK centerline file is requested
// (parallelCenterlineExtraction.cpp:1168-1247): keep the vertices and edges of
// trees with at least min-tree-length vertices, optionally split long edges,
// remove loops (removeLoops, :129-285: degree-2 chains are contracted into
// single weighted edges, a minimum spanning forest is grown with a priority
// queue, the chains are restored) and rasterise the edges into centerline
// voxels while smoothing the radius along each edge (createCenterlineVoxels,
// :287-321).
//
// The spanning forest uses std::priority_queue with the reference's ordering
// (smallest distance on top) and its push order, so equal distances resolve
// the same way; new roots are the last unvisited node, as there.  Nodes and
// edges are indices into arrays here rather than heap objects.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <queue>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "tsf/tsf_c.h"

namespace tsf_host {

struct V3 {
    int x, y, z;
};

static float dist(const V3 &a, const V3 &b) {
    const float dx = (float)(a.x - b.x), dy = (float)(a.y - b.y), dz = (float)(a.z - b.z);
    return std::sqrt((dx * dx + dy * dy) + dz * dz);
}

struct GNode {
    V3 pos;
    std::vector<int> out;          // outgoing edge ids
};
struct GEdge {
    int source, target;
    std::vector<int> removed;      // contracted nodes, from source to target
    float distance;
};

class LoopRemover {
public:
    LoopRemover(const std::vector<V3> &v, const std::vector<std::array<int, 2>> &e, V3 size) : size_(size) {
        for (const V3 &p : v) nodes_.push_back(GNode{p, {}});
        for (const auto &ed : e) {
            const float d = dist(nodes_[ed[0]].pos, nodes_[ed[1]].pos);
            add_edge(ed[0], ed[1], {}, d);
            add_edge(ed[1], ed[0], {}, d);
        }
    }

    void run(std::vector<V3> &v_out, std::vector<std::array<int, 2>> &e_out) {
        // contract every node of degree 2 (in index order) into its two neighbours' edge
        std::vector<int> graph;
        for (int n = 0; n < (int)nodes_.size(); n++) {
            if (nodes_[n].out.size() != 2) {
                graph.push_back(n);
                continue;
            }
            const int e0 = nodes_[n].out[0], e1 = nodes_[n].out[1];
            const int a = edges_[e0].target, b = edges_[e1].target;
            const float d = edges_[e0].distance + edges_[e1].distance;
            std::vector<int> ab, ba;
            for (int j = (int)edges_[e0].removed.size() - 1; j >= 0; j--) ab.push_back(edges_[e0].removed[j]);
            ab.push_back(n);
            for (int r : edges_[e1].removed) ab.push_back(r);
            for (int j = (int)edges_[e1].removed.size() - 1; j >= 0; j--) ba.push_back(edges_[e1].removed[j]);
            ba.push_back(n);
            for (int r : edges_[e0].removed) ba.push_back(r);
            drop_edges_to(a, n);
            drop_edges_to(b, n);
            nodes_[n].out.clear();
            add_edge(a, b, ab, d);
            add_edge(b, a, ba, d);
        }
        if (graph.empty())
            throw std::runtime_error("Centerline graph size is 0! Can't continue. Maybe lower min-tree-length?");

        // minimum spanning forest
        // (the next root is the last unvisited node; nodes never become
        // unvisited, so that index only moves down)
        std::unordered_set<int64_t> visited;
        std::vector<int> tree = spanning_tree(graph[0], visited);
        int last = (int)graph.size() - 1;
        while (tree.size() < graph.size()) {
            while (last >= 0 && visited.count(key(nodes_[graph[last]].pos))) last--;
            if (last < 0) break;   // nodes sharing a position count as one
            const std::vector<int> more = spanning_tree(graph[last], visited);
            tree.insert(tree.end(), more.begin(), more.end());
        }

        // restore the contracted chains on the kept edges
        std::vector<int> final_nodes;
        for (int n : tree) {
            final_nodes.push_back(n);
            const std::vector<int> es = nodes_[n].out;
            for (int e : es) restore(e, final_nodes);
        }

        // vertices numbered by first appearance, edges as kept
        std::unordered_map<int64_t, int> index;
        v_out.clear();
        e_out.clear();
        auto idx = [&](int node) {
            const int64_t k = key(nodes_[node].pos);
            auto it = index.find(k);
            if (it != index.end()) return it->second;
            const int i = (int)v_out.size();
            v_out.push_back(nodes_[node].pos);
            index[k] = i;
            return i;
        };
        for (int n : final_nodes) {
            const int ni = idx(n);
            for (int e : nodes_[n].out) e_out.push_back({ni, idx(edges_[e].target)});
        }
    }

private:
    V3 size_;
    std::vector<GNode> nodes_;
    std::vector<GEdge> edges_;

    int64_t key(const V3 &p) const { return p.x + (int64_t)p.y * size_.x + (int64_t)p.z * size_.x * size_.y; }

    int add_edge(int s, int t, std::vector<int> removed, float d) {
        edges_.push_back(GEdge{s, t, std::move(removed), d});
        const int id = (int)edges_.size() - 1;
        nodes_[s].out.push_back(id);
        return id;
    }

    void drop_edges_to(int n, int target) {
        std::vector<int> keep;
        for (int e : nodes_[n].out)
            if (edges_[e].target != target) keep.push_back(e);
        nodes_[n].out = keep;
    }

    struct Longer {
        const std::vector<GEdge> *edges;
        bool operator()(int a, int b) const { return (*edges)[a].distance > (*edges)[b].distance; }
    };

    std::vector<int> spanning_tree(int root, std::unordered_set<int64_t> &visited) {
        std::vector<int> result{root};
        std::priority_queue<int, std::vector<int>, Longer> queue(Longer{&edges_});
        visited.insert(key(nodes_[root].pos));
        for (int e : nodes_[root].out) queue.push(e);
        nodes_[root].out.clear();
        while (!queue.empty()) {
            const int e = queue.top();
            queue.pop();
            const int t = edges_[e].target;
            if (visited.count(key(nodes_[t].pos))) continue;
            for (int en : nodes_[t].out)
                if (!visited.count(key(nodes_[edges_[en].target].pos))) queue.push(en);
            nodes_[t].out.clear();
            nodes_[edges_[e].source].out.push_back(e);
            result.push_back(t);
            visited.insert(key(nodes_[t].pos));
        }
        return result;
    }

    void restore(int e, std::vector<int> &final_nodes) {
        if (edges_[e].removed.empty()) return;
        const int s = edges_[e].source, t = edges_[e].target;
        const std::vector<int> chain = edges_[e].removed;
        drop_edges_to(s, t);
        int prev = s;
        for (int r : chain) {
            add_edge(prev, r, {}, 0.0f);
            prev = r;
            final_nodes.push_back(r);
        }
        add_edge(prev, t, {}, 0.0f);
    }
};

// createCenterlineVoxels: ceil(|ab|) steps from a towards b, in order (a
// cell may repeat when the edge is short and the rounding lands twice)
static void edge_cells(const V3 &a, const V3 &b, V3 size, std::vector<int64_t> &cells) {
    const float d = dist(a, b);
    const float dir[3] = {(float)(b.x - a.x), (float)(b.y - a.y), (float)(b.z - a.z)};
    const int n = (int)std::ceil(d);
    for (int j = 0; j < n; j++) {
        const float ratio = (float)j / (float)n;
        const int x = (int)std::round((float)a.x + dir[0] * ratio);
        const int y = (int)std::round((float)a.y + dir[1] * ratio);
        const int z = (int)std::round((float)a.z + dir[2] * ratio);
        cells.push_back((int64_t)x + (int64_t)size.x * (y + (int64_t)size.y * z));
    }
}

// the radius along each edge replaced by its mean there, edge after edge:
// `at(p)` is the current radius of cell p (earlier edges' means included)
template <typename At>
static void smooth_edges(const std::vector<int64_t> &cells, const std::vector<int64_t> &start, At at) {
    for (size_t k = 0; k + 1 < start.size(); k++) {
        const int64_t c0 = start[k], c1 = start[k + 1];
        float avg = 0.0f;
        for (int64_t i = c0; i < c1; i++) avg = avg + at(cells[(size_t)i]);
        avg = avg / (float)(c1 - c0);
        for (int64_t i = c0; i < c1; i++) at(cells[(size_t)i]) = avg;
    }
}

static void centerline_voxels(const std::vector<V3> &v, const std::vector<std::array<int, 2>> &e, float *radius,
                              int8_t *out, V3 size) {
    std::vector<int64_t> cells, start{0};
    for (const auto &ed : e) {
        edge_cells(v[ed[0]], v[ed[1]], size, cells);
        start.push_back((int64_t)cells.size());
    }
    for (int64_t p : cells) out[p] = 1;
    smooth_edges(cells, start, [&](int64_t p) -> float & { return radius[p]; });
}

}  // namespace tsf_host

using tsf_host::V3;

static int copy_out(const std::vector<V3> &v, const std::vector<std::array<int, 2>> &e, int *out_v, int *out_e,
                    int capacity, int *n_v, int *n_e) {
    *n_v = (int)v.size();
    *n_e = (int)e.size();
    if ((int)v.size() > capacity || (int)e.size() > capacity) return TSF_ERR_CAPACITY;
    for (size_t i = 0; i < v.size(); i++) {
        out_v[3 * i] = v[i].x;
        out_v[3 * i + 1] = v[i].y;
        out_v[3 * i + 2] = v[i].z;
    }
    for (size_t i = 0; i < e.size(); i++) {
        out_e[2 * i] = e[i][0];
        out_e[2 * i + 1] = e[i][1];
    }
    return TSF_OK;
}

extern "C" int tsf_remove_loops(const int *vertices, int n_vertices, const int *edges, int n_edges, int X, int Y,
                                int Z, int *out_vertices, int *out_edges, int capacity, int *n_out_vertices,
                                int *n_out_edges) {
    if (!vertices || !edges || !out_vertices || !out_edges || !n_out_vertices || !n_out_edges || n_vertices < 0 ||
        n_edges < 0)
        return TSF_ERR_INVALID_ARG;
    std::vector<V3> v(n_vertices);
    for (int i = 0; i < n_vertices; i++) v[i] = V3{vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]};
    std::vector<std::array<int, 2>> e(n_edges);
    for (int i = 0; i < n_edges; i++) {
        e[i] = {edges[2 * i], edges[2 * i + 1]};
        if (e[i][0] < 0 || e[i][1] < 0 || e[i][0] >= n_vertices || e[i][1] >= n_vertices) return TSF_ERR_INVALID_ARG;
    }
    try {
        tsf_host::LoopRemover lr(v, e, V3{X, Y, Z});
        lr.run(v, e);
    } catch (const std::exception &) {
        return TSF_ERR_COUNT_RANGE;
    }
    return copy_out(v, e, out_vertices, out_edges, capacity, n_out_vertices, n_out_edges);
}

// the large trees' vertices and edges (parallelCenterlineExtraction.cpp:
// 1187-1225), edges longer than max_edge_distance split, loops removed;
// TSF_ERR_COUNT_RANGE when nothing is left
static int large_tree_graph(const int *vertices, int n_vertices, const int *edges, int n_edges, const int *labels,
                            const int *tree_sizes, int min_tree_length, int max_edge_distance, int X, int Y, int Z,
                            std::vector<V3> &v, std::vector<std::array<int, 2>> &e) {
    std::vector<int> index(n_vertices, -1);
    for (int i = 0; i < n_vertices; i++) {
        if (tree_sizes[labels[i]] >= min_tree_length) {
            index[i] = (int)v.size();
            v.push_back(V3{vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]});
        }
    }
    for (int i = 0; i < n_edges; i++) {
        const int a = edges[2 * i], b = edges[2 * i + 1];
        if (tree_sizes[labels[a]] < min_tree_length || tree_sizes[labels[b]] < min_tree_length) continue;
        const V3 A = v[index[a]], B = v[index[b]];
        const float d = tsf_host::dist(A, B);
        if (max_edge_distance > 0 && d > (float)max_edge_distance) {
            // extra vertices every max_edge_distance along the edge (for the VTK file)
            const float dir[3] = {(float)(B.x - A.x), (float)(B.y - A.y), (float)(B.z - A.z)};
            int prev = index[a];
            for (int j = max_edge_distance; (float)j < d; j += max_edge_distance) {
                const float t = (float)j / d;
                v.push_back(V3{(int)std::round((float)A.x + t * dir[0]), (int)std::round((float)A.y + t * dir[1]),
                               (int)std::round((float)A.z + t * dir[2])});
                const int cur = (int)v.size() - 1;
                e.push_back({prev, cur});
                prev = cur;
            }
            e.push_back({prev, index[b]});
        } else {
            e.push_back({index[a], index[b]});
        }
    }
    try {
        tsf_host::LoopRemover lr(v, e, V3{X, Y, Z});
        lr.run(v, e);
    } catch (const std::exception &) {
        return TSF_ERR_COUNT_RANGE;
    }
    return TSF_OK;
}

extern "C" int tsf_centerline_graph(const int *vertices, int n_vertices, const int *edges, int n_edges,
                                    const int *labels, const int *tree_sizes, int min_tree_length,
                                    int max_edge_distance, int X, int Y, int Z, float *radius,
                                    int8_t *centerlines, int *out_vertices, int *out_edges, int capacity,
                                    int *n_out_vertices, int *n_out_edges) {
    if (!vertices || !edges || !labels || !tree_sizes || !radius || !centerlines || !out_vertices || !out_edges ||
        !n_out_vertices || !n_out_edges || n_vertices < 0 || n_edges < 0)
        return TSF_ERR_INVALID_ARG;
    std::vector<V3> v;
    std::vector<std::array<int, 2>> e;
    const int r = large_tree_graph(vertices, n_vertices, edges, n_edges, labels, tree_sizes, min_tree_length,
                                   max_edge_distance, X, Y, Z, v, e);
    if (r) return r;
    // the counts first: when they exceed the capacity, radius and centerlines
    // are left as they were, so the caller can call again with more
    *n_out_vertices = (int)v.size();
    *n_out_edges = (int)e.size();
    if ((int)v.size() > capacity || (int)e.size() > capacity) return TSF_ERR_CAPACITY;
    tsf_host::centerline_voxels(v, e, radius, centerlines, V3{X, Y, Z});
    return copy_out(v, e, out_vertices, out_edges, capacity, n_out_vertices, n_out_edges);
}

extern "C" int tsf_centerline_graph_cells(const int *vertices, int n_vertices, const int *edges, int n_edges,
                                          const int *labels, const int *tree_sizes, int min_tree_length,
                                          int max_edge_distance, int X, int Y, int Z, int *out_vertices,
                                          int *out_edges, int capacity, int *n_out_vertices, int *n_out_edges,
                                          int64_t *cells, int64_t *edge_start, int64_t cell_capacity,
                                          int64_t *n_cells) {
    if (!vertices || !edges || !labels || !tree_sizes || !out_vertices || !out_edges || !n_out_vertices ||
        !n_out_edges || !cells || !edge_start || !n_cells || n_vertices < 0 || n_edges < 0 || X <= 0 || Y <= 0 ||
        Z <= 0)
        return TSF_ERR_INVALID_ARG;
    std::vector<V3> v;
    std::vector<std::array<int, 2>> e;
    const int r = large_tree_graph(vertices, n_vertices, edges, n_edges, labels, tree_sizes, min_tree_length,
                                   max_edge_distance, X, Y, Z, v, e);
    if (r) return r;
    std::vector<int64_t> c, start{0};
    for (const auto &ed : e) {
        tsf_host::edge_cells(v[ed[0]], v[ed[1]], V3{X, Y, Z}, c);
        start.push_back((int64_t)c.size());
    }
    *n_out_vertices = (int)v.size();
    *n_out_edges = (int)e.size();
    *n_cells = (int64_t)c.size();
    if ((int)v.size() > capacity || (int)e.size() > capacity || (int64_t)c.size() > cell_capacity)
        return TSF_ERR_CAPACITY;
    std::copy(c.begin(), c.end(), cells);
    std::copy(start.begin(), start.end(), edge_start);
    return copy_out(v, e, out_vertices, out_edges, capacity, n_out_vertices, n_out_edges);
}

extern "C" int tsf_centerline_smooth_radius(const int64_t *cells, const int64_t *edge_start, int n_edges,
                                            const float *values, int64_t *unique_cells, float *unique_values,
                                            int64_t *n_unique) {
    if (!cells || !edge_start || !values || !unique_cells || !unique_values || !n_unique || n_edges < 0)
        return TSF_ERR_INVALID_ARG;
    const int64_t n = edge_start[n_edges];
    // current radius per distinct cell, starting from the gathered values
    std::unordered_map<int64_t, size_t> slot;
    std::vector<int64_t> uc;
    std::vector<float> uv;
    for (int64_t i = 0; i < n; i++) {
        if (slot.emplace(cells[i], uc.size()).second) {
            uc.push_back(cells[i]);
            uv.push_back(values[i]);
        }
    }
    const std::vector<int64_t> c(cells, cells + n), start(edge_start, edge_start + n_edges + 1);
    tsf_host::smooth_edges(c, start, [&](int64_t p) -> float & { return uv[slot[p]]; });
    std::copy(uc.begin(), uc.end(), unique_cells);
    std::copy(uv.begin(), uv.end(), unique_values);
    *n_unique = (int64_t)uc.size();
    return TSF_OK;
}

extern "C" int tsf_write_centerline_vtk(const char *path, const int *vertices, int n_vertices, const int *edges,
                                        int n_edges) {
    // writeToVtkFile (inputOutput.cpp:48-63): legacy ASCII polydata
    std::ofstream f(path);
    if (!f) return TSF_ERR_INVALID_ARG;
    f << "# vtk DataFile Version 3.0\nvtk output\nASCII\n";
    f << "DATASET POLYDATA\nPOINTS " << n_vertices << " int\n";
    for (int i = 0; i < n_vertices; i++)
        f << vertices[3 * i] << " " << vertices[3 * i + 1] << " " << vertices[3 * i + 2] << "\n";
    f << "\nLINES " << n_edges << " " << n_edges * 3 << "\n";
    for (int i = 0; i < n_edges; i++) f << "2 " << edges[2 * i] << " " << edges[2 * i + 1] << "\n";
    return f ? TSF_OK : TSF_ERR_INVALID_ARG;
}
