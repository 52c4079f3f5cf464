// Host-side graph work of the PEEC loop/tree basis (pcbqs_gb300_loop_basis): the spanning forest of the copper
// branches and the fundamental cycle of every other branch, restated from src/pcbqs/mqs.py:48-130 (spanning_tree)
// and :592-637 (_loops). Native because the cycle walk touches every tree branch of every cycle (millions of steps
// on a plane pair); same traversal orders as the reference, so the same tree and the same cycles.
#include <cstdint>
#include <deque>
#include <utility>
#include <vector>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"

namespace {

using Adjacency = std::vector<std::vector<std::pair<int32_t, int32_t>>>;   // (neighbour, branch)

// Breadth-first order from `root` and the hop distances of the visited nodes (dist[] reset for them afterwards by
// the caller through `order`).
void bfs(const Adjacency &adj, int32_t root, std::vector<int32_t> &order, std::vector<int32_t> &dist) {
    order.clear();
    dist[root] = 0;
    order.push_back(root);
    for (size_t head = 0; head < order.size(); ++head) {
        const int32_t u = order[head];
        for (const auto &e : adj[u])
            if (dist[e.first] < 0) {
                dist[e.first] = dist[u] + 1;
                order.push_back(e.first);
            }
    }
}

int32_t find(std::vector<int32_t> &parent, int32_t a) {
    while (parent[a] != a) {
        parent[a] = parent[parent[a]];
        a = parent[a];
    }
    return a;
}

}  // namespace

extern "C" int pcbqs_gb300_loop_basis(int64_t n_nodes, int64_t nb, const int32_t *ea, const int32_t *eb,
                                      const uint8_t *is_src, int64_t first, int ideal_terminals, uint8_t *tree_out,
                                      int64_t capacity, int32_t *rows, int32_t *cols, double *vals, int64_t *nnz,
                                      int32_t *col_branch, int64_t *ncol) {
    using pq::fail;
    if (n_nodes <= 0 || nb < 0 || first < 0 || first > nb || (nb && (!ea || !eb || !is_src)) || !tree_out ||
        capacity < 0 || !nnz || !ncol || (capacity && (!rows || !cols || !vals)) || (nb && !col_branch))
        return fail(pq::ERR_ARGUMENT, "loop_basis: invalid argument");
    for (int64_t k = 0; k < nb; ++k)
        if (ea[k] < 0 || ea[k] >= n_nodes || eb[k] < 0 || eb[k] >= n_nodes)
            return fail(pq::ERR_ARGUMENT, "loop_basis: branch %lld ends outside the nodes", (long long)k);
    const int32_t n = (int32_t)n_nodes;
    Adjacency adj(n);
    for (int64_t k = 0; k < first; ++k)
        if (!is_src[k] && ea[k] != eb[k]) {
            adj[ea[k]].emplace_back(eb[k], (int32_t)k);
            adj[eb[k]].emplace_back(ea[k], (int32_t)k);
        }
    std::vector<uint8_t> tree(nb, 0), seen(n, 0);
    std::vector<int32_t> order, o1, o2, d0(n, -1), d1(n, -1), d2(n, -1), mark(n, 0);
    std::deque<int32_t> queue;
    for (int32_t s = 0; s < n; ++s) {
        if (seen[s]) continue;
        bfs(adj, s, order, d0);
        for (int32_t v : order) seen[v] = 1;
        int32_t root = s;
        if (order.size() > 2) {
            // the most central node: the middle of a double sweep's longest path
            bfs(adj, order.back(), o1, d1);
            int32_t far = o1[0];
            for (int32_t v : o1)
                if (d1[v] > d1[far]) far = v;
            bfs(adj, far, o2, d2);
            int32_t best = -1;
            for (int32_t v : order) {
                const int32_t ecc = d1[v] > d2[v] ? d1[v] : d2[v];
                if (best < 0 || ecc < (d1[best] > d2[best] ? d1[best] : d2[best])) best = v;
            }
            root = best;
            for (int32_t v : o1) d1[v] = -1;
            for (int32_t v : o2) d2[v] = -1;
        }
        for (int32_t v : order) d0[v] = -1;
        mark[root] = 1;
        queue.assign(1, root);
        while (!queue.empty()) {
            const int32_t u = queue.front();
            queue.pop_front();
            for (const auto &e : adj[u])
                if (!mark[e.first]) {
                    mark[e.first] = 1;
                    tree[e.second] = 1;
                    queue.push_back(e.first);
                }
        }
    }
    // the other non-source branches join islands the copper leaves apart
    std::vector<int32_t> parent(n);
    for (int32_t i = 0; i < n; ++i) parent[i] = i;
    for (int64_t k = 0; k < nb; ++k)
        if (tree[k]) {
            const int32_t ra = find(parent, ea[k]);
            parent[find(parent, eb[k])] = ra;
        }
    for (int64_t k = first; k < nb; ++k)
        if (!is_src[k]) {
            const int32_t ra = find(parent, ea[k]), rb = find(parent, eb[k]);
            if (ra != rb) {
                parent[rb] = ra;
                tree[k] = 1;
            }
        }
    // rooted forest: parent node, parent branch and its sign, depth, component root
    Adjacency tadj(n);
    for (int64_t k = 0; k < nb; ++k)
        if (tree[k]) {
            tadj[ea[k]].emplace_back(eb[k], (int32_t)k);
            tadj[eb[k]].emplace_back(ea[k], (int32_t)k);
        }
    std::vector<int32_t> up(n, -1), upb(n, -1), ups(n, 0), depth(n, -1), comp(n, -1), stack;
    for (int32_t r = 0; r < n; ++r) {
        if (depth[r] >= 0) continue;
        depth[r] = 0;
        comp[r] = r;
        stack.assign(1, r);
        while (!stack.empty()) {
            const int32_t u = stack.back();
            stack.pop_back();
            for (const auto &e : tadj[u])
                if (depth[e.first] < 0) {
                    const int32_t v = e.first, k = e.second;
                    depth[v] = depth[u] + 1;
                    up[v] = u;
                    upb[v] = k;
                    ups[v] = ea[k] == u ? 1 : -1;
                    comp[v] = r;
                    stack.push_back(v);
                }
        }
    }
    // fundamental cycles: the branch itself, the tree path from its second end up to the meeting node, and the path
    // back down to its first end
    int64_t count = 0, columns = 0;
    std::vector<std::pair<int32_t, int32_t>> pu, pv;
    for (int64_t k = 0; k < nb; ++k) {
        if (tree[k]) continue;
        const int32_t a = ea[k], b = eb[k];
        if (a == b && k < first && ideal_terminals) continue;
        if (comp[a] != comp[b]) continue;
        int32_t u = b, v = a;
        pu.clear();
        pv.clear();
        while (depth[u] > depth[v]) {
            pu.emplace_back(upb[u], -ups[u]);
            u = up[u];
        }
        while (depth[v] > depth[u]) {
            pv.emplace_back(upb[v], ups[v]);
            v = up[v];
        }
        while (u != v) {
            pu.emplace_back(upb[u], -ups[u]);
            u = up[u];
            pv.emplace_back(upb[v], ups[v]);
            v = up[v];
        }
        const int64_t need = 1 + (int64_t)pu.size() + (int64_t)pv.size();
        if (count + need <= capacity) {
            rows[count] = (int32_t)k;
            cols[count] = (int32_t)columns;
            vals[count] = 1.0;
            int64_t at = count + 1;
            for (const auto &e : pu) {
                rows[at] = e.first;
                cols[at] = (int32_t)columns;
                vals[at++] = (double)e.second;
            }
            for (auto it = pv.rbegin(); it != pv.rend(); ++it) {
                rows[at] = it->first;
                cols[at] = (int32_t)columns;
                vals[at++] = (double)it->second;
            }
        }
        count += need;
        col_branch[columns++] = (int32_t)k;
    }
    for (int64_t k = 0; k < nb; ++k) tree_out[k] = tree[k];
    *nnz = count;
    *ncol = columns;
    if (count > capacity) return fail(pq::ERR_ARGUMENT, "loop_basis: %lld entries exceed the capacity of %lld",
                                      (long long)count, (long long)capacity);
    return pq::OK;
}
