// Cluster trees, level padding and near/far interaction lists (host side).
//
// These are caller-side utilities: the reference obtains its trees from
// H2Trees (ext/BFH2Trees/*) and its far list from nearandfar
// (src/Matrixassembly/intlists.jl:30-217).  The rules here are fixed so that
// the library and the CPU oracle produce identical trees and far lists.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "bf_internal.h"

namespace bfg {

double Tree::radius(int64_t n) const {
  // TwoNTree radius = halfsize * sqrt(3) (ext/BFH2Trees/BFH2Trees.jl:15-16)
  return half[n] * std::sqrt(3.0);
}

int32_t Tree::depth() const {
  int32_t d = 0;
  for (int32_t l : level) d = std::max(d, l);
  return d;
}

int tree_build(const double* xyz, int64_t n, int32_t max_points, int32_t max_depth, Tree& t) {
  if (n <= 0 || xyz == nullptr) {
    set_error("bf_tree_build: empty point set");
    return BF_EINVAL;
  }
  t = Tree();
  t.n_points = n;
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) lo[a] = hi[a] = xyz[a];
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      double v = xyz[3 * i + a];
      if (!std::isfinite(v)) {
        set_error("bf_tree_build: non-finite coordinate at point %lld", (long long)i);
        return BF_EINVAL;
      }
      lo[a] = std::min(lo[a], v);
      hi[a] = std::max(hi[a], v);
    }
  double ext = 0.0;
  for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
  t.perm.resize(n);
  for (int64_t i = 0; i < n; ++i) t.perm[i] = i;
  auto push = [&](const double c[3], double h, int32_t lvl, int32_t par, int64_t b, int64_t e) {
    t.center.insert(t.center.end(), c, c + 3);
    t.half.push_back(h);
    t.level.push_back(lvl);
    t.parent.push_back(par);
    t.first_child.push_back(0);
    t.n_child.push_back(0);
    t.begin.push_back(b);
    t.end.push_back(e);
  };
  double c0[3] = {(lo[0] + hi[0]) * 0.5, (lo[1] + hi[1]) * 0.5, (lo[2] + hi[2]) * 0.5};
  push(c0, ext * 0.5, 0, -1, 0, n);
  std::vector<int64_t> current{0}, next, tmp;
  std::vector<int8_t> oct;
  while (!current.empty()) {
    next.clear();
    for (int64_t nd : current) {
      int64_t b = t.begin[nd], e = t.end[nd], cnt = e - b;
      bool leaf = cnt <= 1;
      if (max_points > 0 && cnt <= max_points) leaf = true;
      if (max_depth >= 0 && t.level[nd] >= max_depth) leaf = true;
      if (!(t.half[nd] > 0.0)) leaf = true;
      t.first_child[nd] = (int32_t)t.nn();
      if (leaf) continue;
      const double c[3] = {t.center[3 * nd], t.center[3 * nd + 1], t.center[3 * nd + 2]};
      oct.resize(cnt);
      int64_t counts[8] = {0};
      for (int64_t i = 0; i < cnt; ++i) {
        const double* p = xyz + 3 * t.perm[b + i];
        int o = (p[0] >= c[0] ? 1 : 0) + (p[1] >= c[1] ? 2 : 0) + (p[2] >= c[2] ? 4 : 0);
        oct[i] = (int8_t)o;
        counts[o]++;
      }
      int64_t start[8];
      int64_t acc = 0;
      for (int o = 0; o < 8; ++o) {
        start[o] = acc;
        acc += counts[o];
      }
      tmp.resize(cnt);
      for (int64_t i = 0; i < cnt; ++i) tmp[start[oct[i]]++] = t.perm[b + i];
      std::memcpy(t.perm.data() + b, tmp.data(), cnt * sizeof(int64_t));
      double hc = t.half[nd] * 0.5;
      int32_t nc = 0;
      int64_t off = b;
      int32_t lvl = t.level[nd] + 1;
      for (int o = 0; o < 8; ++o) {
        if (counts[o] == 0) continue;
        double cc[3] = {c[0] + ((o & 1) ? hc : -hc), c[1] + ((o & 2) ? hc : -hc),
                        c[2] + ((o & 4) ? hc : -hc)};
        push(cc, hc, lvl, (int32_t)nd, off, off + counts[o]);
        next.push_back(t.nn() - 1);
        off += counts[o];
        ++nc;
      }
      t.n_child[nd] = nc;
    }
    current.swap(next);
  }
  return BF_OK;
}

std::vector<std::vector<int64_t>> traverse_and_pad(const Tree& t, int64_t root) {
  // treelevels (src/auxillaries.jl:263-281) + padding (src/auxillaries.jl:340-350)
  std::vector<std::vector<int64_t>> lv;
  std::vector<int64_t> cur{root};
  while (!cur.empty()) {
    lv.push_back(cur);
    std::vector<int64_t> nxt;
    for (int64_t nd : cur)
      if (!t.isleaf(nd))
        for (int32_t c = 0; c < t.n_child[nd]; ++c) nxt.push_back(t.first_child[nd] + c);
    cur.swap(nxt);
  }
  for (size_t l = 1; l + 1 < lv.size(); ++l) {
    size_t n0 = lv[l].size();
    for (size_t i = 0; i < n0; ++i)
      if (t.isleaf(lv[l][i])) lv[l + 1].push_back(lv[l][i]);
  }
  return lv;
}

bool is_far(const Tree& ts, const Tree& to, int64_t snode, int64_t onode, double alpha) {
  // ext/BFH2Trees/h2admissible.jl:11-45
  const double* oc = &to.center[3 * onode];
  const double* sc = &ts.center[3 * snode];
  double ol = to.radius(onode), sl = ts.radius(snode);
  double W = std::max(sl, ol);
  double target = alpha * W;
  double mind_sq = 0.0;
  for (int i = 0; i < 3; ++i) {
    double d = std::fabs(oc[i] - sc[i]) - (sl + ol);
    if (d > 0.0) mind_sq += d * d;
  }
  if (mind_sq < 1e-10) return false;
  return std::sqrt(mind_sq) > target;
}

}  // namespace bfg

using namespace bfg;


extern "C" {

int bf_tree_build(const double* xyz, int64_t n_points, int32_t max_points, int32_t max_depth,
                  bf_tree_t* out) {
  if (!out) {
    set_error("bf_tree_build: out is NULL");
    return BF_EINVAL;
  }
  *out = nullptr;
  auto* h = new (std::nothrow) bf_tree;
  if (!h) return BF_ENOMEM;
  int s = tree_build(xyz, n_points, max_points, max_depth, h->t);
  if (s != BF_OK) {
    delete h;
    return s;
  }
  *out = h;
  return BF_OK;
}

int bf_tree_from_arrays(int64_t n_nodes, int64_t n_points, const double* center,
                        const double* halfsize, const int32_t* parent, const int32_t* first_child,
                        const int32_t* n_child, const int64_t* begin, const int64_t* end,
                        const int64_t* perm, bf_tree_t* out) {
  if (!out || n_nodes <= 0 || n_points <= 0 || !center || !halfsize || !parent || !first_child ||
      !n_child || !begin || !end || !perm) {
    set_error("bf_tree_from_arrays: invalid argument");
    return BF_EINVAL;
  }
  *out = nullptr;
  auto* h = new (std::nothrow) bf_tree;
  if (!h) return BF_ENOMEM;
  Tree& t = h->t;
  t.n_points = n_points;
  t.center.assign(center, center + 3 * n_nodes);
  t.half.assign(halfsize, halfsize + n_nodes);
  t.parent.assign(parent, parent + n_nodes);
  t.first_child.assign(first_child, first_child + n_nodes);
  t.n_child.assign(n_child, n_child + n_nodes);
  t.begin.assign(begin, begin + n_nodes);
  t.end.assign(end, end + n_nodes);
  t.perm.assign(perm, perm + n_points);
  t.level.assign(n_nodes, 0);
  for (int64_t i = 0; i < n_nodes; ++i) {
    bool ok = t.begin[i] >= 0 && t.end[i] <= n_points && t.begin[i] <= t.end[i] &&
              t.n_child[i] >= 0 && (t.n_child[i] == 0 || (t.first_child[i] > i &&
                                                          t.first_child[i] + t.n_child[i] <= n_nodes));
    if (!ok) {
      delete h;
      set_error("bf_tree_from_arrays: inconsistent node %lld", (long long)i);
      return BF_EINVAL;
    }
    for (int32_t c = 0; c < t.n_child[i]; ++c) t.level[t.first_child[i] + c] = t.level[i] + 1;
  }
  for (int64_t i = 0; i < n_points; ++i)
    if (t.perm[i] < 0 || t.perm[i] >= n_points) {
      delete h;
      set_error("bf_tree_from_arrays: perm[%lld] out of range", (long long)i);
      return BF_EINVAL;
    }
  *out = h;
  return BF_OK;
}

int bf_tree_size(bf_tree_t tree, int64_t* n_nodes, int64_t* n_points, int32_t* depth) {
  if (!tree) {
    set_error("bf_tree_size: NULL tree");
    return BF_EINVAL;
  }
  if (n_nodes) *n_nodes = tree->t.nn();
  if (n_points) *n_points = tree->t.n_points;
  if (depth) *depth = tree->t.depth();
  return BF_OK;
}

int bf_tree_export(bf_tree_t tree, double* center, double* halfsize, int32_t* level,
                   int32_t* parent, int32_t* first_child, int32_t* n_child, int64_t* begin,
                   int64_t* end, int64_t* perm) {
  if (!tree) {
    set_error("bf_tree_export: NULL tree");
    return BF_EINVAL;
  }
  const Tree& t = tree->t;
  size_t nn = (size_t)t.nn();
  if (center) std::memcpy(center, t.center.data(), 3 * nn * sizeof(double));
  if (halfsize) std::memcpy(halfsize, t.half.data(), nn * sizeof(double));
  if (level) std::memcpy(level, t.level.data(), nn * sizeof(int32_t));
  if (parent) std::memcpy(parent, t.parent.data(), nn * sizeof(int32_t));
  if (first_child) std::memcpy(first_child, t.first_child.data(), nn * sizeof(int32_t));
  if (n_child) std::memcpy(n_child, t.n_child.data(), nn * sizeof(int32_t));
  if (begin) std::memcpy(begin, t.begin.data(), nn * sizeof(int64_t));
  if (end) std::memcpy(end, t.end.data(), nn * sizeof(int64_t));
  if (perm) std::memcpy(perm, t.perm.data(), (size_t)t.n_points * sizeof(int64_t));
  return BF_OK;
}

int bf_tree_destroy(bf_tree_t tree) {
  delete tree;
  return BF_OK;
}

}  // extern "C"

namespace bfg {

// Dual-tree traversal of src/Matrixassembly/intlists.jl:30-217 (balanced
// splitting), an explicit stack in the recursion's depth-first order.  Far
// pairs go to `far` (when given), near pairs to `near` (when given); both
// are always counted.
void near_far_lists(const Tree& to, const Tree& ts, double alpha, int32_t minbflvl,
                    int32_t leafcomp, int32_t leafimbalance, int32_t unbalancedints,
                    std::vector<std::pair<int64_t, int64_t>>* far,
                    std::vector<std::pair<int64_t, int64_t>>* near, int64_t* n_far,
                    int64_t* n_near) {
  struct Item {
    int64_t o, s;
    int32_t h;
  };
  std::vector<Item> stack;
  int32_t h0 = std::min(to.depth() + 1, ts.depth() + 1);
  stack.push_back({0, 0, h0});
  int64_t nf = 0, nn = 0;
  std::vector<Item> kids;
  auto add_near = [&](const Item& it) {
    if (near) near->push_back({it.o, it.s});
    ++nn;
  };
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    bool lo = to.isleaf(it.o), ls = ts.isleaf(it.s);
    bool adm = is_far(ts, to, it.s, it.o, alpha);
    if (it.h <= minbflvl && !leafcomp) {
      add_near(it);
      continue;
    }
    if (adm) {
      if ((lo || ls) && !leafcomp) {
        add_near(it);
      } else {
        if (far) far->push_back({it.o, it.s});
        ++nf;
      }
      continue;
    }
    if ((lo && ls) || ((lo || ls) && !leafimbalance)) {
      add_near(it);
      continue;
    }
    kids.clear();
    if (unbalancedints) {  // only the larger node splits (intlists.jl:121-149)
      if ((to.radius(it.o) >= ts.radius(it.s) && !lo) || ls) {
        for (int32_t c = 0; c < to.n_child[it.o]; ++c) kids.push_back({to.first_child[it.o] + c, it.s, it.h - 1});
      } else {
        for (int32_t c = 0; c < ts.n_child[it.s]; ++c) kids.push_back({it.o, ts.first_child[it.s] + c, it.h - 1});
      }
    } else if (lo) {
      for (int32_t c = 0; c < ts.n_child[it.s]; ++c) kids.push_back({it.o, ts.first_child[it.s] + c, it.h - 1});
    } else if (ls) {
      for (int32_t c = 0; c < to.n_child[it.o]; ++c) kids.push_back({to.first_child[it.o] + c, it.s, it.h - 1});
    } else {
      for (int32_t co = 0; co < to.n_child[it.o]; ++co)
        for (int32_t cs = 0; cs < ts.n_child[it.s]; ++cs)
          kids.push_back({to.first_child[it.o] + co, ts.first_child[it.s] + cs, it.h - 1});
    }
    for (auto r = kids.rbegin(); r != kids.rend(); ++r) stack.push_back(*r);
  }
  if (n_far) *n_far = nf;
  if (n_near) *n_near = nn;
}

}  // namespace bfg

extern "C" {

int bf_nearandfar(bf_tree_t obs_tree, bf_tree_t src_tree, double alpha, int32_t minbflvl,
                  int32_t leafcomp, int32_t leafimbalance, int32_t unbalancedints,
                  int64_t* far_obs, int64_t* far_src,
                  int64_t capacity, int64_t* n_far, int64_t* n_near) {
  if (!obs_tree || !src_tree) {
    set_error("bf_nearandfar: NULL tree");
    return BF_EINVAL;
  }
  std::vector<std::pair<int64_t, int64_t>> far;
  int64_t nf = 0, nn = 0;
  near_far_lists(obs_tree->t, src_tree->t, alpha, minbflvl, leafcomp, leafimbalance,
                 unbalancedints, (far_obs && far_src) ? &far : nullptr, nullptr, &nf, &nn);
  if (n_far) *n_far = nf;
  if (n_near) *n_near = nn;
  if (capacity > 0 && nf > capacity) {
    set_error("bf_nearandfar: capacity %lld < %lld far pairs", (long long)capacity, (long long)nf);
    return BF_EINVAL;
  }
  for (int64_t i = 0; i < (int64_t)far.size() && i < capacity; ++i) {
    far_obs[i] = far[i].first;
    far_src[i] = far[i].second;
  }
  return BF_OK;
}

int bf_near_pairs(bf_tree_t obs_tree, bf_tree_t src_tree, double alpha, int32_t minbflvl,
                  int32_t leafcomp, int32_t leafimbalance, int32_t unbalancedints,
                  int64_t* near_obs, int64_t* near_src,
                  int64_t capacity, int64_t* n_near) {
  if (!obs_tree || !src_tree) {
    set_error("bf_near_pairs: NULL tree");
    return BF_EINVAL;
  }
  std::vector<std::pair<int64_t, int64_t>> near;
  int64_t nn = 0;
  near_far_lists(obs_tree->t, src_tree->t, alpha, minbflvl, leafcomp, leafimbalance,
                 unbalancedints, nullptr, (near_obs && near_src) ? &near : nullptr, nullptr, &nn);
  if (n_near) *n_near = nn;
  if (capacity > 0 && nn > capacity) {
    set_error("bf_near_pairs: capacity %lld < %lld near pairs", (long long)capacity,
              (long long)nn);
    return BF_EINVAL;
  }
  for (int64_t i = 0; i < (int64_t)near.size() && i < capacity; ++i) {
    near_obs[i] = near[i].first;
    near_src[i] = near[i].second;
  }
  return BF_OK;
}

}  // extern "C"
