// evoc_labels_oracle.cpp — CPU restatement of evoc-rs 0.2.7's clustering of
// the embedding: the labels that the final correctness check compares.
//
// TEST INFRASTRUCTURE ONLY. The reference keeps this stage on its own Rust CPU
// code; the image has no Rust toolchain, so this restatement stands in for it
// when labels are compared (adjusted Rand index of two embeddings' labels). It
// is compiled into the oracle library beside evoc_oracle.cpp, and nothing in
// the product links, loads or calls it.
//
// Restated (paths inside evoc-rs):
//   KdTree::build, aabb_sq, knn_query(_batch), nearest_other_component,
//     update_node_components            src/clustering/kd_tree.rs:93-535
//   build_mst (Boruvka over mutual reachability)
//                                        src/clustering/mst.rs:82-166
//   DisjointSet (path halving, union by rank)
//                                        src/utils/disjoint_set.rs:12-60
//   mst_to_linkage_tree                  src/clustering/linkage.rs:39-85
//   condense_tree, collect_descendants, eliminate_branch
//                                        src/clustering/condensed_tree.rs:40-251
//   extract_leaves                       src/clustering/condensed_tree.rs:264-292
//   get_cluster_label_vector             src/clustering/condensed_tree.rs:311-368
//   max_lambdas, get_point_membership_strengths
//                                        src/clustering/condensed_tree.rs:380-470
//   min_cluster_size_barcode, compute_total_persistence, find_peaks,
//   estimate_cluster_similarity, select_diverse_peaks,
//   extract_clusters_at_size, build_cluster_layers
//                                        src/clustering/persistence.rs:42-463
//   search_for_n_clusters                src/lib.rs:377-452
// in f32 (the configurations' float type), with the reference's summation
// and comparison orders.
//
// Documented deviations:
//   1. Among several points at an equal mutual-reachability distance, a
//      Boruvka query returns the one with the smallest index; the reference
//      returns the first its tree traversal meets, which depends on the
//      order of points inside its nodes (set by select_nth_unstable_by; the
//      median split here uses std::nth_element). The result no longer
//      depends on the tree. With distinct distances the minimum spanning
//      tree is unique and identical.
//   2. Boruvka merges each round's per-component best edges in ascending
//      order of the component's smallest point index; the reference
//      iterates an FxHashMap keyed by disjoint-set roots (mst.rs:140), whose
//      order depends on rustc-hash. Again only ties are affected.
//   3. The squared distance is the serial left fold sum_d (a_d - b_d)^2, as in
//      evoc_oracle.cpp (ann-search-rs euclidean_simd is not vendored).
//   4. exp() in min_cluster_size_barcode is the C library's expf, which is
//      what Rust's f32::exp calls on Linux.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using f32 = float;

inline f32 sq_dist(const f32* a, const f32* b, int64_t dim) {
  f32 s = 0.0f;
  for (int64_t d = 0; d < dim; ++d) {
    const f32 t = a[d] - b[d];
    s += t * t;
  }
  return s;
}

// ---------------------------------------------------------------------------
// KD-tree (kd_tree.rs:93-535): implicit binary tree, node i has children
// 2i+1, 2i+2; leaves hold at most leaf_size points; bounding boxes per node.
// ---------------------------------------------------------------------------
struct KdTree {
  std::vector<int64_t> idx;
  std::vector<int64_t> start, end;
  std::vector<uint8_t> leaf;
  std::vector<f32> lower, upper;
  int64_t n_nodes = 0, dim = 0;
  const f32* data = nullptr;

  const f32* pt(int64_t i) const { return data + i * dim; }

  void build(const f32* d, int64_t n, int64_t dm, int64_t leaf_size) {  // :139-236
    data = d;
    dim = dm;
    leaf_size = std::max<int64_t>(leaf_size, 1);
    if (n == 0) return;
    int64_t n_levels = 1;
    if (n > leaf_size)
      n_levels = (int64_t)std::log2((double)(n - 1) / (double)leaf_size) + 1;
    n_nodes = ((int64_t)1 << n_levels) - 1;
    idx.resize(n);
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    start.assign(n_nodes, 0);
    end.assign(n_nodes, 0);
    leaf.assign(n_nodes, 1);
    lower.assign(n_nodes * dim, 0.0f);
    upper.assign(n_nodes * dim, 0.0f);
    build_node(0, n, 0);
  }

  void build_node(int64_t s, int64_t e, int64_t node) {  // :191-236
    const int64_t bo = node * dim;
    const f32* first = pt(idx[s]);
    for (int64_t k = 0; k < dim; ++k) lower[bo + k] = upper[bo + k] = first[k];
    for (int64_t i = s + 1; i < e; ++i) {
      const f32* p = pt(idx[i]);
      for (int64_t k = 0; k < dim; ++k) {
        lower[bo + k] = std::min(lower[bo + k], p[k]);
        upper[bo + k] = std::max(upper[bo + k], p[k]);
      }
    }
    start[node] = s;
    end[node] = e;
    const int64_t left = 2 * node + 1;
    if (left >= n_nodes || e - s < 2) {
      leaf[node] = 1;
      return;
    }
    leaf[node] = 0;
    int64_t split = 0;
    f32 spread = 0.0f;
    for (int64_t k = 0; k < dim; ++k) {
      const f32 sp = upper[bo + k] - lower[bo + k];
      if (sp > spread) {
        spread = sp;
        split = k;
      }
    }
    const int64_t mid = s + (e - s) / 2;
    std::nth_element(idx.begin() + s, idx.begin() + mid, idx.begin() + e,
                     [&](int64_t a, int64_t b) { return data[a * dim + split] < data[b * dim + split]; });
    build_node(s, mid, left);
    build_node(mid, e, left + 1);
  }

  f32 aabb_sq(int64_t node, const f32* p) const {  // :247-265
    const int64_t bo = node * dim;
    f32 r = 0.0f;
    for (int64_t k = 0; k < dim; ++k) {
      const f32 lo = lower[bo + k], hi = upper[bo + k];
      const f32 diff = p[k] < lo ? lo - p[k] : (p[k] > hi ? p[k] - hi : 0.0f);
      r += diff * diff;
    }
    return r;
  }

  // k nearest other points of point q, (dist_sq, idx) ascending (:428-535).
  struct Cand {
    f32 d;
    int64_t i;
    bool operator<(const Cand& o) const { return d < o.d || (d == o.d && i < o.i); }
  };
  void knn_recurse(const f32* q, int64_t k, int64_t exclude, int64_t node,
                   std::vector<Cand>& heap) const {
    const f32 lb = aabb_sq(node, q);
    if ((int64_t)heap.size() == k && lb > heap.front().d) return;
    if (leaf[node]) {
      for (int64_t a = start[node]; a < end[node]; ++a) {
        const int64_t j = idx[a];
        if (j == exclude) continue;
        const f32 d = sq_dist(pt(j), q, dim);
        if ((int64_t)heap.size() < k) {
          heap.push_back(Cand{d, j});
          std::push_heap(heap.begin(), heap.end());
        } else {
          const Cand& w = heap.front();
          if (d < w.d || (d == w.d && j < w.i)) {
            std::pop_heap(heap.begin(), heap.end());
            heap.back() = Cand{d, j};
            std::push_heap(heap.begin(), heap.end());
          }
        }
      }
      return;
    }
    const int64_t l = 2 * node + 1, r = l + 1;
    const f32 ll = aabb_sq(l, q), lr = aabb_sq(r, q);
    if (ll <= lr) {
      knn_recurse(q, k, exclude, l, heap);
      knn_recurse(q, k, exclude, r, heap);
    } else {
      knn_recurse(q, k, exclude, r, heap);
      knn_recurse(q, k, exclude, l, heap);
    }
  }
  // squared distance to the k-th nearest other point (0 when k == 0)
  f32 kth_sq(int64_t q, int64_t k) const {
    if (k == 0 || n_nodes == 0) return 0.0f;
    std::vector<Cand> heap;
    heap.reserve(k);
    knn_recurse(pt(q), k, q, 0, heap);
    f32 mx = 0.0f;
    for (const Cand& c : heap) mx = std::max(mx, c.d);
    return mx;
  }

  // Nearest point of another component under mutual reachability (:275-378).
  void noc_recurse(int64_t qi, const f32* core, const int64_t* pc, const int64_t* nc,
                   int64_t node, f32 lb, int64_t& bj, f32& bd) const {
    if (lb > bd) return;
    if (core[qi] > bd) return;
    const int64_t qc = pc[qi];
    if (nc[node] == qc) return;
    if (leaf[node]) {
      const f32* q = pt(qi);
      for (int64_t a = start[node]; a < end[node]; ++a) {
        const int64_t j = idx[a];
        if (pc[j] == qc) continue;
        if (core[j] > bd) continue;
        const f32 sq = sq_dist(q, pt(j), dim);
        const f32 mr = std::max(std::max(sq, core[qi]), core[j]);
        if (mr < bd || (mr == bd && bj != qi && j < bj)) {  // ties: smallest index
          bd = mr;
          bj = j;
        }
      }
      return;
    }
    const int64_t l = 2 * node + 1, r = l + 1;
    const f32* q = pt(qi);
    const f32 ll = aabb_sq(l, q), lr = aabb_sq(r, q);
    if (ll <= lr) {
      noc_recurse(qi, core, pc, nc, l, ll, bj, bd);
      noc_recurse(qi, core, pc, nc, r, lr, bj, bd);
    } else {
      noc_recurse(qi, core, pc, nc, r, lr, bj, bd);
      noc_recurse(qi, core, pc, nc, l, ll, bj, bd);
    }
  }

  void update_node_components(const int64_t* pc, int64_t* nc) const {  // :387-419
    for (int64_t node = n_nodes - 1; node >= 0; --node) {
      if (leaf[node]) {
        const int64_t s = start[node], e = end[node];
        if (s >= e) {
          nc[node] = -1;
          continue;
        }
        const int64_t c = pc[idx[s]];
        bool all = true;
        for (int64_t a = s; a < e && all; ++a) all = pc[idx[a]] == c;
        nc[node] = all ? c : -1;
      } else {
        const int64_t l = 2 * node + 1, r = l + 1;
        nc[node] = (r < n_nodes && nc[l] >= 0 && nc[l] == nc[r]) ? nc[l] : -1;
      }
    }
  }
};

// disjoint_set.rs:12-60
struct DisjointSet {
  std::vector<int64_t> parent, rank, lo;  // lo: smallest element of each root's set
  explicit DisjointSet(int64_t n) : parent(n), rank(n, 0), lo(n) {
    for (int64_t i = 0; i < n; ++i) parent[i] = lo[i] = i;
  }
  int64_t find(int64_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  }
  bool unite(int64_t x, int64_t y) {
    const int64_t rx = find(x), ry = find(y);
    if (rx == ry) return false;
    if (rank[rx] < rank[ry]) {
      parent[rx] = ry;
    } else if (rank[rx] > rank[ry]) {
      parent[ry] = rx;
    } else {
      parent[ry] = rx;
      rank[rx] += 1;
    }
    lo[rx] = lo[ry] = std::min(lo[rx], lo[ry]);
    return true;
  }
};

struct Edge {
  int64_t u, v;
  f32 w;
};

// mst.rs:82-166
std::vector<Edge> build_mst(const f32* data, int64_t n, int64_t dim, int64_t min_samples) {
  std::vector<Edge> mst;
  if (n <= 1) return mst;
  KdTree tree;
  tree.build(data, n, dim, 40);
  const int64_t k = std::min(min_samples, n - 1);
  std::vector<f32> core(n, 0.0f);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) core[i] = tree.kth_sq(i, k);
  DisjointSet ds(n);
  mst.reserve(n - 1);
  std::vector<int64_t> pc(n), nc(std::max<int64_t>(tree.n_nodes, 1), -1);
  std::vector<int64_t> bj(n);
  std::vector<f32> bd(n);
  // Per component, the smallest distance found so far in this round (float
  // bits; the distances are >= 0, so their bits order like the values). A
  // query starts from just above it: a point whose own best is larger cannot
  // be its component's pick, and one whose best equals or beats it walks the
  // same tree order as from FLT_MAX and returns the same neighbour, so the
  // per-component picks are unchanged.
  std::vector<uint32_t> cbest(n);
  const f32 fmax = std::numeric_limits<f32>::max();
  uint32_t fmax_bits;
  std::memcpy(&fmax_bits, &fmax, 4);
  for (;;) {
    for (int64_t i = 0; i < n; ++i) pc[i] = ds.lo[ds.find(i)];  // id: smallest point index
    tree.update_node_components(pc.data(), nc.data());
    std::fill(cbest.begin(), cbest.end(), fmax_bits);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      uint32_t* cb = &cbest[pc[i]];
      const uint32_t bb = __atomic_load_n(cb, __ATOMIC_RELAXED);
      f32 bound;
      std::memcpy(&bound, &bb, 4);
      int64_t j = i;
      f32 d = bound == fmax ? fmax : std::nextafter(bound, std::numeric_limits<f32>::infinity());
      tree.noc_recurse(i, core.data(), pc.data(), nc.data(), 0, tree.aabb_sq(0, tree.pt(i)), j,
                       d);
      bj[i] = j;
      bd[i] = d;
      if (j != i) {
        uint32_t db;
        std::memcpy(&db, &d, 4);
        uint32_t cur = __atomic_load_n(cb, __ATOMIC_RELAXED);
        while (db < cur && !__atomic_compare_exchange_n(cb, &cur, db, true, __ATOMIC_RELAXED,
                                                        __ATOMIC_RELAXED)) {
        }
      }
    }
    // per component: the first point (ascending) with the smallest distance
    std::map<int64_t, Edge> best;
    for (int64_t i = 0; i < n; ++i) {
      if (bj[i] == i) continue;
      auto it = best.find(pc[i]);
      if (it == best.end())
        best.emplace(pc[i], Edge{i, bj[i], bd[i]});
      else if (bd[i] < it->second.w)
        it->second = Edge{i, bj[i], bd[i]};
    }
    if (best.empty()) break;
    bool merged = false;
    for (auto& kv : best) {
      const Edge& e = kv.second;
      if (ds.unite(e.u, e.v)) {
        mst.push_back(e);
        merged = true;
        if ((int64_t)mst.size() == n - 1) break;
      }
    }
    if ((int64_t)mst.size() == n - 1 || !merged) break;
  }
  for (Edge& e : mst) e.w = std::sqrt(e.w);
  return mst;
}

struct LinkRow {
  int64_t left, right;
  f32 dist;
  int64_t size;
};

// linkage.rs:39-85 (the MST sort is stable, like Rust's sort_by)
std::vector<LinkRow> mst_to_linkage(std::vector<Edge>& mst, int64_t n) {
  std::stable_sort(mst.begin(), mst.end(), [](const Edge& a, const Edge& b) { return a.w < b.w; });
  const int64_t total = 2 * n - 1;
  std::vector<int64_t> parent(std::max<int64_t>(total, 0), -1), size(std::max<int64_t>(total, 0), 0);
  for (int64_t i = 0; i < n; ++i) size[i] = 1;
  std::vector<LinkRow> link;
  link.reserve(mst.size());
  for (size_t i = 0; i < mst.size(); ++i) {
    const int64_t next = n + (int64_t)i;
    int64_t l = mst[i].u, r = mst[i].v;
    while (parent[l] != -1) l = parent[l];
    while (parent[r] != -1) r = parent[r];
    const int64_t ns = size[l] + size[r];
    if (l < r) std::swap(l, r);
    link.push_back(LinkRow{l, r, mst[i].w, ns});
    parent[l] = next;
    parent[r] = next;
    size[next] = ns;
  }
  return link;
}

struct CNode {
  int64_t parent, child;
  f32 lambda;
  int64_t size;
};

// condensed_tree.rs:62-80: depth-first, right subtree first (stack pops)
std::vector<int64_t> collect_descendants(const std::vector<LinkRow>& L, int64_t root, int64_t n) {
  std::vector<int64_t> out, stack{root};
  while (!stack.empty()) {
    const int64_t node = stack.back();
    stack.pop_back();
    out.push_back(node);
    if (node >= n) {
      const LinkRow& r = L[node - n];
      stack.push_back(r.left);
      stack.push_back(r.right);
    }
  }
  return out;
}

void eliminate_branch(const std::vector<LinkRow>& L, int64_t node, int64_t parent, f32 lambda,
                      int64_t n, std::vector<CNode>& out) {  // :93-115
  for (int64_t d : collect_descendants(L, node, n))
    if (d < n) out.push_back(CNode{parent, d, lambda, 1});
}

// condensed_tree.rs:127-251
std::vector<CNode> condense_tree(const std::vector<LinkRow>& L, int64_t n, int64_t mcs) {
  std::vector<CNode> out;
  if (L.empty()) return out;
  const int64_t root = 2 * (int64_t)L.size();
  const std::vector<int64_t> trav = collect_descendants(L, root, n);
  std::vector<int64_t> relabel(root + 1, 0);
  relabel[root] = n;
  int64_t next = n + 1;
  std::vector<uint8_t> ignore(root + 1, 0);
  auto mark_ignored = [&](int64_t node) {
    for (int64_t d : collect_descendants(L, node, n))
      if (d >= n) ignore[d] = 1;
  };
  for (int64_t node : trav) {
    if (node < n || ignore[node]) continue;
    const int64_t pl = relabel[node];
    const LinkRow& row = L[node - n];
    const f32 lambda = row.dist > 0.0f ? 1.0f / row.dist : std::numeric_limits<f32>::infinity();
    const int64_t ls = row.left >= n ? L[row.left - n].size : 1;
    const int64_t rs = row.right >= n ? L[row.right - n].size : 1;
    const bool lb = ls >= mcs, rb = rs >= mcs;
    if (lb && rb) {
      relabel[row.left] = next;
      out.push_back(CNode{pl, next, lambda, ls});
      ++next;
      relabel[row.right] = next;
      out.push_back(CNode{pl, next, lambda, rs});
      ++next;
    } else if (lb) {
      relabel[row.left] = pl;
      eliminate_branch(L, row.right, pl, lambda, n, out);
      mark_ignored(row.right);
    } else if (rb) {
      relabel[row.right] = pl;
      eliminate_branch(L, row.left, pl, lambda, n, out);
      mark_ignored(row.left);
    } else {
      eliminate_branch(L, row.left, pl, lambda, n, out);
      eliminate_branch(L, row.right, pl, lambda, n, out);
      mark_ignored(row.left);
      mark_ignored(row.right);
    }
  }
  return out;
}

int64_t tree_max_id(const std::vector<CNode>& T) {
  int64_t m = 0;
  for (const CNode& c : T) m = std::max(m, std::max(c.parent, c.child));
  return m;
}

// condensed_tree.rs:264-292
std::vector<int64_t> extract_leaves(const std::vector<CNode>& T, int64_t n) {
  std::vector<int64_t> leaves;
  if (T.empty()) return leaves;
  const int64_t mx = tree_max_id(T);
  std::vector<uint8_t> is_parent(mx + 1, 0), has_child(mx + 1, 0);
  for (const CNode& c : T) {
    if (c.size > 1) is_parent[c.parent] = 1;
    has_child[c.parent] = 1;
  }
  for (int64_t i = n; i <= mx; ++i)
    if (!is_parent[i] && has_child[i]) leaves.push_back(i);
  return leaves;
}

int64_t tree_root(const std::vector<CNode>& T, int64_t dflt) {
  int64_t r = std::numeric_limits<int64_t>::max();
  for (const CNode& c : T) r = std::min(r, c.parent);
  return T.empty() ? dflt : r;
}

// condensed_tree.rs:311-368
std::vector<int64_t> cluster_labels(const std::vector<CNode>& T, const std::vector<int64_t>& clusters,
                                    int64_t n) {
  std::vector<int64_t> labels(n, -1);
  if (clusters.empty()) return labels;
  const int64_t mx = tree_max_id(T);
  const int64_t root = tree_root(T, n);
  DisjointSet ds(mx + 1);
  const std::unordered_set<int64_t> cset(clusters.begin(), clusters.end());
  for (const CNode& c : T)
    if (!cset.count(c.child)) ds.unite(c.parent, c.child);
  std::vector<int64_t> sorted = clusters;
  std::sort(sorted.begin(), sorted.end());
  std::unordered_map<int64_t, int64_t> lab;
  for (size_t i = 0; i < sorted.size(); ++i) lab[sorted[i]] = (int64_t)i;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = ds.find(i);
    if (c <= root) continue;
    auto it = lab.find(c);
    if (it != lab.end()) labels[i] = it->second;
  }
  return labels;
}

// condensed_tree.rs:380-470
std::vector<f32> membership_strengths(const std::vector<CNode>& T,
                                      const std::vector<int64_t>& clusters,
                                      const std::vector<int64_t>& labels) {
  const int64_t n = (int64_t)labels.size();
  std::vector<f32> out(n, 0.0f);
  const std::unordered_set<int64_t> cset(clusters.begin(), clusters.end());
  std::unordered_map<int64_t, f32> death;
  for (int64_t c : clusters) death[c] = 0.0f;
  for (const CNode& c : T)
    if (c.size == 1 && cset.count(c.parent)) {
      f32& e = death[c.parent];
      if (c.lambda > e) e = c.lambda;
    }
  std::vector<int64_t> sorted = clusters;
  std::sort(sorted.begin(), sorted.end());
  const int64_t root = tree_root(T, n);
  for (const CNode& c : T) {
    const int64_t p = c.child;
    if (p >= root || p >= n) continue;
    if (labels[p] < 0) continue;
    if (labels[p] >= (int64_t)sorted.size()) continue;
    const int64_t cid = sorted[labels[p]];
    auto it = death.find(cid);
    if (it == death.end()) continue;
    const f32 ml = it->second;
    if (ml == 0.0f || !std::isfinite(c.lambda))
      out[p] = 1.0f;
    else
      out[p] = (c.lambda < ml ? c.lambda : ml) / ml;
  }
  return out;
}

struct Barcode {
  f32 birth, death;
  int64_t parent;
  f32 lambda_death;
};

// persistence.rs:42-104
std::vector<Barcode> size_barcode(const std::vector<CNode>& T, int64_t n, int64_t min_size) {
  std::vector<Barcode> bc;
  if (T.empty()) return bc;
  std::vector<const CNode*> cl;
  for (const CNode& c : T)
    if (c.size > 1) cl.push_back(&c);
  if (cl.empty()) return bc;
  int64_t max_child = 0;
  for (const CNode* c : cl) max_child = std::max(max_child, c->child);
  const int64_t nn = max_child - n + 1;
  bc.assign(nn, Barcode{(f32)min_size, 0.0f, n, 0.0f});
  bc[0].lambda_death = 0.0f;
  bc[0].death = (f32)n;
  size_t i = cl.size();
  while (i >= 2) {
    i -= 2;
    const CNode* a = cl[i];
    const CNode* b = cl[i + 1];
    const int64_t ia = a->child - n, ib = b->child - n;
    bc[ia].parent = a->parent;
    bc[ib].parent = b->parent;
    const f32 lv = std::exp(-1.0f / a->lambda);
    bc[ia].lambda_death = lv;
    bc[ib].lambda_death = lv;
    const f32 dt = (f32)std::min(a->size, b->size);
    bc[ia].death = dt;
    bc[ib].death = dt;
    const int64_t pi = a->parent - n;
    const f32 mb = std::max(std::max(bc[ia].birth, bc[ib].birth), dt);
    bc[pi].birth = std::max(bc[pi].birth, mb);
  }
  return bc;
}

// persistence.rs:114-155
void total_persistence(const std::vector<Barcode>& bc, std::vector<f32>& sizes,
                       std::vector<f32>& pers) {
  sizes.clear();
  pers.clear();
  if (bc.empty()) return;
  for (const Barcode& b : bc) sizes.push_back(b.birth);
  std::sort(sizes.begin(), sizes.end());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  pers.assign(sizes.size(), 0.0f);
  for (size_t k = 1; k < bc.size(); ++k) {
    const Barcode& b = bc[k];
    if (b.death <= b.birth) continue;
    const size_t bp = std::lower_bound(sizes.begin(), sizes.end(), b.birth) - sizes.begin();
    const size_t dp = std::lower_bound(sizes.begin(), sizes.end(), b.death) - sizes.begin();
    const f32 contrib = (b.death - b.birth) * b.lambda_death;
    for (size_t q = bp; q < dp; ++q) pers[q] += contrib;
  }
}

// persistence.rs:167-191
std::vector<int64_t> find_peaks(const std::vector<f32>& x) {
  std::vector<int64_t> peaks;
  if (x.size() < 3) return peaks;
  size_t i = 1;
  const size_t imax = x.size() - 1;
  while (i < imax) {
    if (x[i - 1] < x[i]) {
      size_t ia = i + 1;
      while (ia < imax && x[ia] == x[i]) ++ia;
      if (x[ia] < x[i]) {
        peaks.push_back((int64_t)((i + ia - 1) / 2));
        i = ia;
      }
    }
    ++i;
  }
  return peaks;
}

// persistence.rs:203-229
double cluster_similarity(const std::vector<Barcode>& bc, f32 ba, f32 bb) {
  int64_t inter = 0, uni = 0;
  for (const Barcode& b : bc) {
    const bool a = b.birth <= ba && b.death > ba;
    const bool c = b.birth <= bb && b.death > bb;
    inter += a && c;
    uni += a || c;
  }
  return uni == 0 ? 0.0 : (double)inter / (double)uni;
}

// persistence.rs:246-283 (sort by persistence descending, stable)
std::vector<int64_t> select_diverse_peaks(const std::vector<int64_t>& peaks,
                                          const std::vector<f32>& pers,
                                          const std::vector<f32>& sizes,
                                          const std::vector<Barcode>& bc, double thr,
                                          int64_t max_layers) {
  std::vector<int64_t> sel;
  if (peaks.empty()) return sel;
  std::vector<std::pair<int64_t, f32>> ix;
  for (int64_t p : peaks) ix.emplace_back(p, pers[p]);
  std::stable_sort(ix.begin(), ix.end(),
                   [](const std::pair<int64_t, f32>& a, const std::pair<int64_t, f32>& b) {
                     return a.second > b.second;
                   });
  std::vector<f32> births;
  for (auto& pk : ix) {
    if ((int64_t)sel.size() >= max_layers) break;
    const f32 birth = sizes[pk.first];
    bool diverse = true;
    for (f32 sb : births) diverse = diverse && cluster_similarity(bc, birth, sb) <= thr;
    if (diverse) {
      sel.push_back(pk.first);
      births.push_back(birth);
    }
  }
  return sel;
}

struct Layers {
  std::vector<std::vector<int64_t>> labels;
  std::vector<std::vector<f32>> strengths;
  std::vector<double> persistence;
};

int64_t n_clusters_of(const std::vector<int64_t>& l) {
  int64_t m = -1;
  for (int64_t v : l)
    if (v >= 0) m = std::max(m, v);
  return m + 1;
}

// persistence.rs:387-463, from the minimum spanning tree on (:402 builds it)
Layers cluster_layers_from_mst(std::vector<Edge> mst, int64_t n, int64_t base_mcs, double thr,
                               int64_t max_layers) {
  Layers out;
  if (n == 0) return out;
  const std::vector<LinkRow> L = mst_to_linkage(mst, n);
  const std::vector<CNode> T = condense_tree(L, n, base_mcs);
  const std::vector<int64_t> leaves = extract_leaves(T, n);
  std::vector<int64_t> base = cluster_labels(T, leaves, n);
  std::vector<f32> bstr = membership_strengths(T, leaves, base);
  std::vector<std::vector<int64_t>> all_l{base};
  std::vector<std::vector<f32>> all_s{bstr};
  std::vector<double> all_p{0.0};
  const std::vector<Barcode> bc = size_barcode(T, n, base_mcs);
  if (!bc.empty()) {
    std::vector<f32> sizes, pers;
    total_persistence(bc, sizes, pers);
    const std::vector<int64_t> peaks = find_peaks(pers);
    const std::vector<int64_t> sel =
        select_diverse_peaks(peaks, pers, sizes, bc, thr, std::max<int64_t>(max_layers - 1, 0));
    for (int64_t pk : sel) {
      const f32 birth = sizes[pk];
      std::vector<int64_t> act;
      for (size_t i = 0; i < bc.size(); ++i)
        if (bc[i].birth <= birth && bc[i].death > birth) act.push_back((int64_t)i + n);
      std::vector<int64_t> l = cluster_labels(T, act, n);
      all_s.push_back(membership_strengths(T, act, l));
      all_l.push_back(std::move(l));
      all_p.push_back((double)pers[pk]);
    }
  }
  std::vector<size_t> order(all_l.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::vector<int64_t> cnt(all_l.size());
  for (size_t i = 0; i < all_l.size(); ++i) cnt[i] = n_clusters_of(all_l[i]);
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cnt[b] < cnt[a]; });
  for (size_t i : order) {
    out.labels.push_back(all_l[i]);
    out.strengths.push_back(all_s[i]);
    out.persistence.push_back(all_p[i]);
  }
  return out;
}

// persistence.rs:387-463
Layers build_cluster_layers(const f32* emb, int64_t n, int64_t dim, int64_t min_samples,
                            int64_t base_mcs, double thr, int64_t max_layers) {
  if (n == 0) return Layers();
  return cluster_layers_from_mst(build_mst(emb, n, dim, min_samples), n, base_mcs, thr,
                                 max_layers);
}

}  // namespace

extern "C" {

struct OracleLayers {
  Layers l;
};

// Boruvka MST over mutual reachability (mst.rs:82-166); writes n - 1 edges
// (fewer if disconnected) and returns their count.
int64_t oracle_build_mst(const float* emb, int64_t n, int64_t dim, int64_t min_samples,
                         int64_t* u, int64_t* v, float* w) {
  std::vector<Edge> e = build_mst(emb, n, dim, min_samples);
  for (size_t i = 0; i < e.size(); ++i) {
    u[i] = e[i].u;
    v[i] = e[i].v;
    w[i] = e[i].w;
  }
  return (int64_t)e.size();
}

// mst_to_linkage_tree (linkage.rs:39-85) of m edges; rows of (left, right,
// size) and distances.
void oracle_linkage(const int64_t* u, const int64_t* v, const float* w, int64_t m, int64_t n,
                    int64_t* lr, float* dist) {
  std::vector<Edge> e(m);
  for (int64_t i = 0; i < m; ++i) e[i] = Edge{u[i], v[i], w[i]};
  const std::vector<LinkRow> L = mst_to_linkage(e, n);
  for (size_t i = 0; i < L.size(); ++i) {
    lr[3 * i] = L[i].left;
    lr[3 * i + 1] = L[i].right;
    lr[3 * i + 2] = L[i].size;
    dist[i] = L[i].dist;
  }
}

// The MST -> linkage -> condensed tree -> leaves -> labels chain at one
// min_cluster_size (the base layer of build_cluster_layers); labels[n],
// strengths[n]; returns the number of leaf clusters.
int64_t oracle_leaf_labels(const float* emb, int64_t n, int64_t dim, int64_t min_samples,
                           int64_t min_cluster_size, int64_t* labels, float* strengths) {
  if (n == 0) return 0;
  std::vector<Edge> mst = build_mst(emb, n, dim, min_samples);
  const std::vector<LinkRow> L = mst_to_linkage(mst, n);
  const std::vector<CNode> T = condense_tree(L, n, min_cluster_size);
  const std::vector<int64_t> leaves = extract_leaves(T, n);
  const std::vector<int64_t> l = cluster_labels(T, leaves, n);
  const std::vector<f32> s = membership_strengths(T, leaves, l);
  std::memcpy(labels, l.data(), n * sizeof(int64_t));
  std::memcpy(strengths, s.data(), n * sizeof(float));
  return (int64_t)leaves.size();
}

// build_cluster_layers (persistence.rs:387-463).
OracleLayers* oracle_cluster_layers(const float* emb, int64_t n, int64_t dim, int64_t min_samples,
                                    int64_t base_min_cluster_size, double min_similarity,
                                    int64_t max_layers) {
  OracleLayers* o = new OracleLayers();
  o->l = build_cluster_layers(emb, n, dim, min_samples, base_min_cluster_size, min_similarity,
                              max_layers);
  return o;
}
// The same from a given minimum spanning tree (m edges u, v, weight).
OracleLayers* oracle_cluster_layers_mst(const int64_t* u, const int64_t* v, const float* w,
                                        int64_t m, int64_t n, int64_t base_min_cluster_size,
                                        double min_similarity, int64_t max_layers) {
  std::vector<Edge> mst((size_t)m);
  for (int64_t i = 0; i < m; ++i) mst[i] = Edge{u[i], v[i], w[i]};
  OracleLayers* o = new OracleLayers();
  o->l = cluster_layers_from_mst(std::move(mst), n, base_min_cluster_size, min_similarity,
                                 max_layers);
  return o;
}
int64_t oracle_layers_count(const OracleLayers* o) { return (int64_t)o->l.labels.size(); }
void oracle_layers_get(const OracleLayers* o, int64_t i, int64_t* labels, float* strengths,
                       double* persistence) {
  const size_t n = o->l.labels[i].size();
  std::memcpy(labels, o->l.labels[i].data(), n * sizeof(int64_t));
  std::memcpy(strengths, o->l.strengths[i].data(), n * sizeof(float));
  *persistence = o->l.persistence[i];
}
void oracle_layers_free(OracleLayers* o) { delete o; }

// find_peaks (persistence.rs:167-191); returns the count written to out.
int64_t oracle_find_peaks(const float* x, int64_t n, int64_t* out) {
  const std::vector<int64_t> p = find_peaks(std::vector<f32>(x, x + n));
  for (size_t i = 0; i < p.size(); ++i) out[i] = p[i];
  return (int64_t)p.size();
}

// min_cluster_size_barcode + compute_total_persistence of the condensed tree
// at base size mcs: barcodes as (birth, death, parent, lambda_death) rows and
// the persistence curve over sizes; returns the barcode count, *n_sizes the
// curve length (buffers hold at least n entries each).
int64_t oracle_barcodes(const float* emb, int64_t n, int64_t dim, int64_t min_samples,
                        int64_t mcs, double* bc_out, float* sizes_out, float* pers_out,
                        int64_t* n_sizes) {
  std::vector<Edge> mst = build_mst(emb, n, dim, min_samples);
  const std::vector<LinkRow> L = mst_to_linkage(mst, n);
  const std::vector<CNode> T = condense_tree(L, n, mcs);
  const std::vector<Barcode> bc = size_barcode(T, n, mcs);
  std::vector<f32> sizes, pers;
  total_persistence(bc, sizes, pers);
  for (size_t i = 0; i < bc.size(); ++i) {
    bc_out[4 * i] = bc[i].birth;
    bc_out[4 * i + 1] = bc[i].death;
    bc_out[4 * i + 2] = (double)bc[i].parent;
    bc_out[4 * i + 3] = bc[i].lambda_death;
  }
  for (size_t i = 0; i < sizes.size(); ++i) {
    sizes_out[i] = sizes[i];
    pers_out[i] = pers[i];
  }
  *n_sizes = (int64_t)sizes.size();
  return (int64_t)bc.size();
}

// search_for_n_clusters (lib.rs:377-452): labels of the min_cluster_size
// whose leaf count is closest to target_k; returns that leaf count.
int64_t oracle_search_n_clusters(const float* emb, int64_t n, int64_t dim, int64_t min_samples,
                                 int64_t target_k, int64_t* labels, float* strengths) {
  if (n == 0) return 0;
  std::vector<Edge> mst = build_mst(emb, n, dim, min_samples);
  const std::vector<LinkRow> L = mst_to_linkage(mst, n);
  int64_t lo = 2, hi = n / 2;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) / 2;
    if (mid == lo || mid == hi) break;
    const int64_t k = (int64_t)extract_leaves(condense_tree(L, n, mid), n).size();
    if (k < target_k)
      hi = mid;
    else
      lo = mid;
  }
  const std::vector<CNode> tl = condense_tree(L, n, lo), th = condense_tree(L, n, hi);
  const std::vector<int64_t> ll = extract_leaves(tl, n), lh = extract_leaves(th, n);
  const std::vector<int64_t> labl = cluster_labels(tl, ll, n), labh = cluster_labels(th, lh, n);
  const int64_t dl = std::llabs((int64_t)ll.size() - target_k);
  const int64_t dh = std::llabs((int64_t)lh.size() - target_k);
  bool use_lo;
  if (dl != dh) {
    use_lo = dl < dh;
  } else {
    int64_t al = 0, ah = 0;
    for (int64_t i = 0; i < n; ++i) {
      al += labl[i] >= 0;
      ah += labh[i] >= 0;
    }
    use_lo = al >= ah;
  }
  const std::vector<int64_t>& lab = use_lo ? labl : labh;
  const std::vector<f32> s = membership_strengths(use_lo ? tl : th, use_lo ? ll : lh, lab);
  std::memcpy(labels, lab.data(), n * sizeof(int64_t));
  std::memcpy(strengths, s.data(), n * sizeof(float));
  return (int64_t)(use_lo ? ll.size() : lh.size());
}

}  // extern "C"
