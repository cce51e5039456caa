// Host-side mesh ordering utilities (native, deterministic).
//
// - Greedy first-fit cell colouring in cell order: colour(c) is the smallest
//   colour not used by an already-coloured face neighbour.  Used to build the
//   colour-blocked cell numbering under which LU-SGS has one level per colour.
// - Reverse Cuthill-McKee with a specified tie-break: the start node of each
//   connected component is found by the George-Liu pseudo-peripheral search
//   starting from the lowest-index node of minimum degree; neighbours are
//   visited in (degree, index) order; the final order is reversed.
//
// Both run once per mesh, outside the timed path.

#include <algorithm>
#include <cstdint>
#include <vector>

namespace {

struct Graph {
  std::vector<int32_t> ptr, adj, deg;
};

Graph build(int32_t n, const int32_t* own, const int32_t* nei, int32_t F) {
  Graph g;
  g.deg.assign(n, 0);
  for (int32_t f = 0; f < F; ++f) {
    g.deg[own[f]]++;
    g.deg[nei[f]]++;
  }
  g.ptr.assign(n + 1, 0);
  for (int32_t i = 0; i < n; ++i) g.ptr[i + 1] = g.ptr[i] + g.deg[i];
  g.adj.assign(g.ptr[n], 0);
  std::vector<int32_t> fill(g.ptr.begin(), g.ptr.end() - 1);
  for (int32_t f = 0; f < F; ++f) {
    g.adj[fill[own[f]]++] = nei[f];
    g.adj[fill[nei[f]]++] = own[f];
  }
  for (int32_t i = 0; i < n; ++i) std::sort(g.adj.begin() + g.ptr[i], g.adj.begin() + g.ptr[i + 1]);
  return g;
}

// BFS levels from root restricted to unvisited-in-ordering nodes of one component
int32_t bfsLevels(const Graph& g, int32_t root, std::vector<int32_t>& level, std::vector<int32_t>& last) {
  std::vector<int32_t> q;
  q.push_back(root);
  level[root] = 0;
  std::vector<int32_t> touched = {root};
  int32_t depth = 0;
  for (size_t h = 0; h < q.size(); ++h) {
    int32_t u = q[h];
    for (int32_t k = g.ptr[u]; k < g.ptr[u + 1]; ++k) {
      int32_t v = g.adj[k];
      if (level[v] < 0) {
        level[v] = level[u] + 1;
        depth = std::max(depth, level[v]);
        q.push_back(v);
        touched.push_back(v);
      }
    }
  }
  last.clear();
  for (int32_t v : touched)
    if (level[v] == depth) last.push_back(v);
  for (int32_t v : touched) level[v] = -1;
  return depth;
}

}  // namespace

extern "C" {

int32_t ics_mesh_greedy_colour(int32_t n, const int32_t* own, const int32_t* nei, int32_t F, int32_t* colour) {
  if (n <= 0 || !own || !nei || !colour || F < 0) return -1;
  Graph g = build(n, own, nei, F);
  std::vector<int32_t> mark;
  int32_t ncol = 0;
  for (int32_t i = 0; i < n; ++i) colour[i] = -1;
  for (int32_t i = 0; i < n; ++i) {
    mark.assign(ncol + 1, 0);
    for (int32_t k = g.ptr[i]; k < g.ptr[i + 1]; ++k) {
      int32_t c = colour[g.adj[k]];
      if (c >= 0) mark[c] = 1;
    }
    int32_t c = 0;
    while (c < ncol && mark[c]) ++c;
    colour[i] = c;
    if (c == ncol) ++ncol;
  }
  return ncol;
}

int32_t ics_mesh_rcm(int32_t n, const int32_t* own, const int32_t* nei, int32_t F, int32_t* new_to_old) {
  if (n <= 0 || !own || !nei || !new_to_old || F < 0) return -1;
  Graph g = build(n, own, nei, F);
  std::vector<char> placed(n, 0);
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<int32_t> level(n, -1), last;
  std::vector<int32_t> comp;
  for (int32_t seed = 0; seed < n; ++seed) {
    if (placed[seed]) continue;
    // component nodes (BFS), pick min-degree lowest-index node
    comp.clear();
    comp.push_back(seed);
    std::vector<char>& inq = placed;  // temporarily mark component
    inq[seed] = 2;
    for (size_t h = 0; h < comp.size(); ++h) {
      int32_t u = comp[h];
      for (int32_t k = g.ptr[u]; k < g.ptr[u + 1]; ++k) {
        int32_t v = g.adj[k];
        if (!inq[v]) {
          inq[v] = 2;
          comp.push_back(v);
        }
      }
    }
    int32_t root = comp[0];
    for (int32_t v : comp)
      if (g.deg[v] < g.deg[root] || (g.deg[v] == g.deg[root] && v < root)) root = v;
    // pseudo-peripheral node search
    int32_t depth = bfsLevels(g, root, level, last);
    for (;;) {
      int32_t cand = last[0];
      for (int32_t v : last)
        if (g.deg[v] < g.deg[cand] || (g.deg[v] == g.deg[cand] && v < cand)) cand = v;
      int32_t d2 = bfsLevels(g, cand, level, last);
      if (d2 > depth) {
        depth = d2;
        root = cand;
      } else {
        break;
      }
    }
    for (int32_t v : comp) placed[v] = 0;
    // Cuthill-McKee from root
    size_t start = order.size();
    order.push_back(root);
    placed[root] = 1;
    std::vector<int32_t> nb;
    for (size_t h = start; h < order.size(); ++h) {
      int32_t u = order[h];
      nb.clear();
      for (int32_t k = g.ptr[u]; k < g.ptr[u + 1]; ++k)
        if (!placed[g.adj[k]]) nb.push_back(g.adj[k]);
      std::sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) {
        return g.deg[a] < g.deg[b] || (g.deg[a] == g.deg[b] && a < b);
      });
      for (int32_t v : nb) {
        placed[v] = 1;
        order.push_back(v);
      }
    }
  }
  for (int32_t i = 0; i < n; ++i) new_to_old[i] = order[n - 1 - i];
  return 0;
}

}  // extern "C"
