// cluster.cpp -- the clustering consumers of a crmsd matrix, behind the C ABI.
//
// Hierarchical agglomerative clustering with the semantics of
// bioshell-clustering/src/hierarchical/hierarchical.rs:22-80 and
// clustering_matrix.rs:11-74, bit for bit in f32:
//   * the pair to merge is the first minimum of the scan "j outer (1..order),
//     i inner (0..j)" with a strict '<' (clustering_matrix.rs:27-42); here
//     it is found from per-column minima kept up to date incrementally
//     (ties: smallest j, then smallest i -- the same pair the scan returns);
//   * update_distances evaluates the rule with size_k = sizes[j] for every k
//     (clustering_matrix.rs:66) and stores the merged cluster at index i;
//   * replace_with_last swaps rows, copies one column and leaves `sizes`
//     where it was (clustering_matrix.rs:47-53);
//   * merged clusters get ids n, n+1, ... in merge order (hierarchical.rs:55).
// The merge rules are strategies/mod.rs:101-167 with the same evaluation
// order (no FMA contraction: this file is compiled with -ffp-contract=off).
//
// OPTICS follows bioshell-clustering/src/optics.rs:51-148 over the matrix,
// with neighbours as CartesianPoints::neighbors_of returns them
// (points_set.rs:150-169): the point itself included, d <= eps, stable sort
// by distance; the seed list is re-sorted after every pop.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cfloat>
#include <new>
#include <vector>

#include "../../include/bioshell_crmsd.h"

namespace {

typedef float (*rule_fn)(int64_t si, int64_t sj, int64_t sk, float dij, float dik, float djk);

float single_link(int64_t, int64_t, int64_t, float, float dik, float djk) { return std::min(dik, djk); }
float complete_link(int64_t, int64_t, int64_t, float, float dik, float djk) { return std::max(dik, djk); }
float average_link(int64_t si, int64_t sj, int64_t, float, float dik, float djk) {
  const float d = 1.0f / (float)(si + sj);
  return d * (float)si * dik + d * (float)sj * djk;
}
float median_link(int64_t, int64_t, int64_t, float dij, float dik, float djk) {
  return 0.5f * dik + 0.5f * djk - 0.25f * dij;
}
float centroid_link(int64_t si, int64_t sj, int64_t, float dij, float dik, float djk) {
  const float d = 1.0f / (float)(si + sj);
  return d * (float)si * dik + d * (float)sj * djk - (float)si * (float)sj * d * d * dij;
}
float wards_method(int64_t si, int64_t sj, int64_t sk, float dij, float dik, float djk) {
  const float d = 1.0f / (float)(si + sj + sk);
  return d * (float)(si + sk) * dik + d * (float)(sj + sk) * djk - (float)sk * d * dij;
}

rule_fn rule_of(int32_t r) {
  switch (r) {
    case BS_LINK_SINGLE: return single_link;
    case BS_LINK_COMPLETE: return complete_link;
    case BS_LINK_AVERAGE: return average_link;
    case BS_LINK_MEDIAN: return median_link;
    case BS_LINK_CENTROID: return centroid_link;
    case BS_LINK_WARD: return wards_method;
    default: return nullptr;
  }
}

// distance (i, j) of the packed triangle as the f32 the clustering sees
struct Tri {
  const void *p;
  int64_t n;
  int32_t type;
  double get(int64_t i, int64_t j) const {
    if (i == j) return 0.0;
    if (i > j) std::swap(i, j);
    const int64_t t = i * n - i * (i + 1) / 2 + (j - i - 1);
    return type == BS_OUT_F64 ? static_cast<const double *>(p)[t] : (double)static_cast<const float *>(p)[t];
  }
};

struct ColMin {
  float v;
  int64_t i;
};

// min over rows r < j of column j, first (smallest r) on ties.  The working
// matrix stays exactly symmetric through every update below, so the column
// is read along row j (contiguous).
inline ColMin column_min(const std::vector<float> &m, int64_t n, int64_t j) {
  ColMin c{FLT_MAX, 0};
  const float *row = m.data() + j * n;
  for (int64_t r = 0; r < j; ++r) {
    const float v = row[r];
    if (v < c.v) {
      c.v = v;
      c.i = r;
    }
  }
  return c;
}

}  // namespace

namespace {

// OPTICS (optics.rs:51-148) with the neighbour lists supplied by a callback
// that fills `nb` with {j, d} for d <= eps, the point itself included,
// stably sorted by distance from a list in ascending j.
template <typename Neighbors>
void optics_run(int64_t n, double eps, int32_t min_points, Neighbors &&neighbors_of,
                std::vector<std::pair<int64_t, double>> &nb, int64_t *order_out, double *reach_out,
                int64_t *cluster_of) {
  const double undefined = eps * 10.0;
  std::vector<double> reach((size_t)n, undefined);
  std::vector<char> processed((size_t)n, 0);
  std::vector<int64_t> order, seeds;
  order.reserve((size_t)n);
  auto by_reach = [&](int64_t a, int64_t b) { return reach[a] < reach[b]; };
  auto update = [&]() {
    const double core = nb[(size_t)min_points - 1].second;
    for (const auto &p : nb) {
      if (processed[p.first]) continue;
      const double nr = std::max(p.second, core);
      if (reach[p.first] == undefined) seeds.push_back(p.first);
      if (reach[p.first] > nr) reach[p.first] = nr;
    }
    std::stable_sort(seeds.begin(), seeds.end(), by_reach);
  };
  for (int64_t i = 0; i < n; ++i) {
    if (processed[i]) continue;
    order.push_back(i);
    neighbors_of(i);
    processed[i] = 1;
    if ((int64_t)nb.size() < min_points) continue;
    seeds.clear();
    update();
    while (!seeds.empty()) {
      const int64_t pi = seeds[0];
      seeds[0] = seeds.back();
      seeds.pop_back();
      std::stable_sort(seeds.begin(), seeds.end(), by_reach);
      order.push_back(pi);
      neighbors_of(pi);
      processed[pi] = 1;
      if ((int64_t)nb.size() < min_points) continue;
      update();
    }
  }
  int64_t label = 0;
  for (int64_t k = 0; k < n; ++k) {
    if (k > 0 && reach[order[k]] == undefined) ++label;
    cluster_of[order[k]] = label;
    order_out[k] = order[k];
    reach_out[k] = reach[order[k]];
  }
}

}  // namespace

extern "C" {

BS_API bs_status bs_hierarchical(const void *tri, int64_t n, int32_t out_type, int32_t rule, int64_t *merges,
                                 float *merge_dist) {
  if (n < 0 || (n > 1 && (!tri || !merges || !merge_dist))) return BS_ERR_INVALID_ARG;
  if (out_type != BS_OUT_F64 && out_type != BS_OUT_F32) return BS_ERR_INVALID_ARG;
  rule_fn rf = rule_of(rule);
  if (!rf) return BS_ERR_INVALID_ARG;
  if (n < 2) return BS_OK;
  if (n > (int64_t)1 << 17) return BS_ERR_UNSUPPORTED;  // dense n x n f32 working matrix
  std::vector<float> m;
  std::vector<int64_t> sizes, ids, node_size;
  std::vector<ColMin> cm;
  try {
    m.assign((size_t)(n * n), 0.0f);
    sizes.assign((size_t)n, 1);
    node_size.assign((size_t)(2 * n - 1), 1);
    ids.resize((size_t)n);
    cm.resize((size_t)n);
  } catch (const std::bad_alloc &) {
    return BS_ERR_OOM;
  }
  const Tri t{tri, n, out_type};
  for (int64_t i = 1; i < n; ++i)
    for (int64_t j = 0; j < i; ++j) {
      const float v = (float)t.get(i, j);
      m[i * n + j] = v;
      m[j * n + i] = v;
    }
  for (int64_t i = 0; i < n; ++i) ids[i] = i;
  for (int64_t j = 1; j < n; ++j) cm[j] = column_min(m, n, j);
  int64_t order = n, cur = n;
  std::vector<float> res((size_t)n);
  for (int64_t step = 0; step < n - 1; ++step) {
    // closest pair: smallest value, then smallest j (scan order), then i
    int64_t bj = 1;
    for (int64_t j = 2; j < order; ++j)
      if (cm[j].v < cm[bj].v) bj = j;
    const int64_t j = bj, i = cm[bj].i;
    const float dij = m[i * n + j];
    merges[4 * step + 0] = ids[i];
    merges[4 * step + 1] = ids[j];
    merges[4 * step + 2] = cur;
    // the tree node's size counts its leaves (hierarchical.rs:52); the
    // matrix's `sizes` slots below keep the reference's bookkeeping
    node_size[cur] = node_size[ids[i]] + node_size[ids[j]];
    merges[4 * step + 3] = node_size[cur];
    merge_dist[step] = dij;
    // update_distances(i, j, rule, new_index = i)
    const int64_t si = sizes[i], sj = sizes[j];
    for (int64_t k = 0; k < order; ++k) res[k] = rf(si, sj, sizes[j], dij, m[i * n + k], m[j * n + k]);
    for (int64_t k = 0; k < order; ++k) {
      m[i * n + k] = res[k];
      m[k * n + i] = res[k];
    }
    m[i * n + i] = 0.0f;
    sizes[i] = sj + si;
    ids[i] = cur;
    // column minima touched by row/column i
    if (i > 0) cm[i] = column_min(m, n, i);
    for (int64_t k = i + 1; k < order; ++k) {
      const float v = m[i * n + k];
      if (v < cm[k].v || (v == cm[k].v && i < cm[k].i)) cm[k] = ColMin{v, i};
      else if (cm[k].i == i) cm[k] = column_min(m, n, k);
    }
    const int64_t last = order - 1;
    if (j < last) {
      // replace_with_last(j): swap rows j and last, copy column last into j
      ids[j] = ids[last];
      order -= 1;
      std::swap_ranges(m.begin() + j * n, m.begin() + j * n + n, m.begin() + order * n);
      for (int64_t r = 0; r < order; ++r) m[r * n + j] = m[r * n + order];
      if (j > 0) cm[j] = column_min(m, n, j);
      for (int64_t k = j + 1; k < order; ++k) {
        const float v = m[j * n + k];
        if (v < cm[k].v || (v == cm[k].v && j < cm[k].i)) cm[k] = ColMin{v, j};
        else if (cm[k].i == j) cm[k] = column_min(m, n, k);
      }
    } else {
      order -= 1;
    }
    cur += 1;
  }
  return BS_OK;
}

BS_API bs_status bs_cut_tree(const int64_t *merges, const float *merge_dist, int64_t n, float cutoff,
                             int64_t *labels) {
  if (n < 0 || (n > 0 && !labels) || (n > 1 && (!merges || !merge_dist))) return BS_ERR_INVALID_ARG;
  if (n == 0) return BS_OK;
  if (n == 1) {
    labels[0] = 0;
    return BS_OK;
  }
  // node ids 0..2n-2; children of merged node n + s are merges[s][0..1]
  const int64_t nodes = 2 * n - 1;
  std::vector<int64_t> left((size_t)nodes, -1), right((size_t)nodes, -1);
  std::vector<float> dist((size_t)nodes, 0.0f);
  for (int64_t s = 0; s < n - 1; ++s) {
    const int64_t id = merges[4 * s + 2];
    if (id < n || id >= nodes) return BS_ERR_INVALID_ARG;
    left[id] = merges[4 * s + 0];
    right[id] = merges[4 * s + 1];
    dist[id] = merge_dist[s];
  }
  // retrieve_clusters (hierarchical.rs:136-169): cluster roots in the order
  // the reference's recursion emits them (left subtree fully before right)
  std::vector<int64_t> roots, stack;
  const int64_t root = nodes - 1;
  if (dist[root] <= cutoff) {
    roots.push_back(root);
  } else {
    // entries >= 0: expand node (clusters_rec); entries < 0: visit child -(c+1)
    stack.push_back(root);
    while (!stack.empty()) {
      const int64_t e = stack.back();
      stack.pop_back();
      if (e < 0) {
        const int64_t c = -(e + 1);
        if (dist[c] <= cutoff) roots.push_back(c);
        else stack.push_back(c);
        continue;
      }
      if (left[e] < 0) {
        roots.push_back(e);
        continue;
      }
      if (!(dist[e] > cutoff)) continue;
      if (right[e] >= 0) stack.push_back(-(right[e] + 1));
      if (left[e] >= 0) stack.push_back(-(left[e] + 1));
    }
  }
  for (size_t r = 0; r < roots.size(); ++r) {
    stack.assign(1, roots[r]);
    while (!stack.empty()) {
      const int64_t v = stack.back();
      stack.pop_back();
      if (left[v] < 0) labels[v] = (int64_t)r;
      else {
        stack.push_back(left[v]);
        stack.push_back(right[v]);
      }
    }
  }
  return BS_OK;
}

BS_API bs_status bs_optics(const void *tri, int64_t n, int32_t out_type, double eps, int32_t min_points,
                           int64_t *order_out, double *reach_out, int64_t *cluster_of) {
  if (n < 0 || min_points < 1 || !(eps > 0.0)) return BS_ERR_INVALID_ARG;
  if (n > 0 && (!tri || !order_out || !reach_out || !cluster_of)) return BS_ERR_INVALID_ARG;
  if (out_type != BS_OUT_F64 && out_type != BS_OUT_F32) return BS_ERR_INVALID_ARG;
  if (n == 0) return BS_OK;
  const Tri t{tri, n, out_type};
  std::vector<std::pair<int64_t, double>> nb;
  auto neighbors_of = [&](int64_t i) {
    nb.clear();
    for (int64_t j = 0; j < n; ++j) {
      const double d = t.get(i, j);
      if (d <= eps) nb.emplace_back(j, d);
    }
    std::stable_sort(nb.begin(), nb.end(), [](const auto &a, const auto &b) { return a.second < b.second; });
  };
  optics_run(n, eps, min_points, neighbors_of, nb, order_out, reach_out, cluster_of);
  return BS_OK;
}

BS_API bs_status bs_optics_neighbors(const int64_t *row_ptr, const int32_t *col, const float *dist, int64_t n,
                                     double eps, int32_t min_points, int64_t *order_out, double *reach_out,
                                     int64_t *cluster_of) {
  if (n < 0 || min_points < 1 || !(eps > 0.0)) return BS_ERR_INVALID_ARG;
  if (n > 0 && (!row_ptr || !order_out || !reach_out || !cluster_of)) return BS_ERR_INVALID_ARG;
  if (n == 0) return BS_OK;
  if (row_ptr[0] != 0 || (row_ptr[n] > 0 && (!col || !dist))) return BS_ERR_INVALID_ARG;
  for (int64_t i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return BS_ERR_INVALID_ARG;
  std::vector<std::pair<int64_t, double>> nb;
  bool bad = false;
  auto neighbors_of = [&](int64_t i) {
    // the row's list, ordered by (d, j), with the point itself (d = 0) put
    // where a stable sort of the ascending-j scan would put it
    nb.clear();
    bool self = false;
    for (int64_t e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
      const int64_t j = col[e];
      const double d = (double)dist[e];
      if (j < 0 || j >= n || j == i) {
        bad = true;
        continue;
      }
      if (!(d <= eps)) continue;
      if (!self && (0.0 < d || (d == 0.0 && i < j))) {
        nb.emplace_back(i, 0.0);
        self = true;
      }
      nb.emplace_back(j, d);
    }
    if (!self) nb.emplace_back(i, 0.0);
  };
  optics_run(n, eps, min_points, neighbors_of, nb, order_out, reach_out, cluster_of);
  return bad ? BS_ERR_INVALID_ARG : BS_OK;
}

}  // extern "C"
