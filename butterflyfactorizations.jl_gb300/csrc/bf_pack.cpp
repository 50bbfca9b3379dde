// Packing of a set of butterfly factorisations into the flat device layout.
//
// Input: reference-style blocks (src/ButterflyFactorization/bfstructs.jl:21-29)
// of many far pairs.  The flat pointers of the reference (one Dict per level,
// bfstructs.jl:107-143) become "slots": contiguous segments of one workspace
// array.  Each level becomes one launch of independent tasks:
//   Q stage : one task per source leaf; the Q blocks of all far pairs on that
//             leaf stacked vertically, input gathered from x by values(leaf).
//   R level : one task per connected block set (node pair); its in-slots are
//             the columns, its out-slots the rows (the column split of one
//             compressed T in assemble_BF, bfassembly.jl:296-307).
//   P stage : one task per observer leaf; the P blocks of all far pairs on that
//             leaf concatenated horizontally, output scattered to y by
//             values(leaf).
// Every workspace entry then has exactly one writer per direction, so neither
// the forward nor the adjoint needs atomics, and the adjoint is the same task
// list read backwards with rows and columns swapped.
#include <algorithm>
#include <cstring>
#include <memory>
#include <memory_resource>
#include <numeric>
#include <parallel/algorithm>

#include "bf_internal.h"

namespace bfg {
namespace {

enum : int8_t { SIDE_SLOT = 0, SIDE_X = 1, SIDE_Y = 2 };
struct Side {
  int8_t type;
  int64_t id;  // slot id or tree node id
  int64_t len;
};
struct Member {
  int64_t blk;  // logical block (-1 = explicit identity)
  int32_t row_off, col_off;
  int32_t ident_n;
};
// The tens of millions of R-level tasks take their arrays from per-chunk
// monotonic arenas (a pointer bump per allocation, one release per arena), so
// that building and dropping them does not go through the general allocator.
struct TaskB {
  int32_t stage;
  int32_t kind;
  std::pmr::vector<Side> rows, cols;
  std::pmr::vector<Member> mats;
  int64_t M = 0, n = 0;
  TaskB() = default;
  explicit TaskB(std::pmr::memory_resource* r) : rows(r), cols(r), mats(r) {}
};

struct DSU {
  std::vector<int64_t> p;
  int64_t find(int64_t x) {
    while (p[x] != x) x = p[x] = p[p[x]];
    return x;
  }
  void unite(int64_t a, int64_t b) {
    a = find(a);
    b = find(b);
    if (a != b) p[b] = a;
  }
};

}  // namespace

int pack_plan(const Logical& lg, Plan& plan, int fac_bytes) {
  PhaseLog plog;
  plan = Plan();
  plan.n_rows = lg.n_rows;
  plan.n_cols = lg.n_cols;
  plan.fac_bytes = fac_bytes;
  const auto& B = lg.blocks;
  int64_t nb = (int64_t)B.size();
  plan.blk_pk_off.assign(nb, -1);
  plan.blk_pk_ld.assign(nb, 0);
  int32_t n_bf = lg.n_bf;
  plan.n_bf = n_bf;
  if (nb == 0 || n_bf <= 0) {
    set_error("pack: no blocks");
    return BF_EINVAL;
  }
  // ---- per-BF depth (number of levels = #R + 1)
  // (parallel over blocks; an error names the first offending block, as a
  // serial scan would)
  std::vector<int32_t> nlev(n_bf, 1);
  int64_t bad_bf = nb, bad_size = nb;
#pragma omp parallel for schedule(static) reduction(min : bad_bf, bad_size)
  for (int64_t b = 0; b < nb; ++b) {
    const LBlock& k = B[b];
    if (k.bf < 0 || k.bf >= n_bf) {
      bad_bf = std::min(bad_bf, b);
      continue;
    }
    if (k.stage > 0) {
      const int32_t v = k.stage + 1;
      int32_t cur = __atomic_load_n(&nlev[k.bf], __ATOMIC_RELAXED);
      while (cur < v && !__atomic_compare_exchange_n(&nlev[k.bf], &cur, v, false,
                                                     __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
      }
    }
    if (!k.ident && (k.rows < 0 || k.cols < 0)) bad_size = std::min(bad_size, b);
  }
  if (bad_bf < nb && bad_bf <= bad_size) {
    set_error("pack: block %lld has bf id %d out of range", (long long)bad_bf, B[bad_bf].bf);
    return BF_EINVAL;
  }
  if (bad_size < nb) {
    set_error("pack: block %lld has negative size", (long long)bad_size);
    return BF_EINVAL;
  }
  int32_t Lmax = *std::max_element(nlev.begin(), nlev.end());
  // block order by (stage rank, original order): Q, R1, R2, ..., P -- a
  // counting sort over the Lmax + 1 stage ranks, stable: contiguous block
  // ranges count and scatter in parallel, each range in order
  std::vector<int64_t> order(nb);
  std::vector<int64_t> sbeg(Lmax + 2, 0);  // order[sbeg[r] .. sbeg[r+1]): stage rank r
  {
    auto srank = [&](const LBlock& k) { return k.stage < 0 ? Lmax : k.stage; };
    const int64_t C = std::max<int64_t>(1, std::min<int64_t>(nb / 65536, 256));
    const int R = Lmax + 1;
    std::vector<int64_t> cnt((size_t)C * R, 0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < C; ++c)
      for (int64_t b = nb * c / C; b < nb * (c + 1) / C; ++b) ++cnt[c * R + srank(B[b])];
    for (int r = 0; r < R; ++r) {
      int64_t tot = 0;
      for (int64_t c = 0; c < C; ++c) tot += cnt[c * R + r];
      sbeg[r + 1] = sbeg[r] + tot;
    }
    for (int r = 0; r < R; ++r) {  // cnt -> scatter position of range c, rank r
      int64_t p = sbeg[r];
      for (int64_t c = 0; c < C; ++c) {
        const int64_t n = cnt[c * R + r];
        cnt[c * R + r] = p;
        p += n;
      }
    }
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < C; ++c)
      for (int64_t b = nb * c / C; b < nb * (c + 1) / C; ++b) order[cnt[c * R + srank(B[b])]++] = b;
  }
  plog.mark("pack: checks + block order");
  // ---- slot wiring (bfstructs.jl:107-143)
  // key (bf, level, o, s) packed exactly into 128 bits (node ids < 2^32)
  FlatMap<int64_t> slot_of;
  if (lg.slot_len.empty()) slot_of.reserve((size_t)nb);
  std::vector<int64_t> slot_len;
  std::vector<int64_t> in_slot(nb, -1), out_slot(nb, -1);
  auto get_slot = [&](int32_t bf, int32_t lvl, int64_t o, int64_t s, bool create) -> int64_t {
    if (o < 0 || s < 0 || o > INT32_MAX || s > INT32_MAX) return -2;
    const uint64_t hi = ((uint64_t)(uint32_t)bf << 32) | (uint32_t)lvl;
    const uint64_t lo = ((uint64_t)o << 32) | (uint64_t)s;
    if (int64_t* v = slot_of.find(hi, lo)) return *v;
    if (!create) return -1;
    int64_t id = (int64_t)slot_len.size();
    slot_of.put(hi, lo, id);
    slot_len.push_back(-1);
    return id;
  };
  auto node_ok = [&](const ValuesMap& vm, int64_t node) {
    return node >= 0 && node + 1 < (int64_t)vm.ptr.size();
  };
  if (!lg.slot_len.empty()) {
    // wiring supplied by the producer (the GPU build): slot ids and lengths
    slot_len = lg.slot_len;
    const int64_t ns = (int64_t)slot_len.size();
    int64_t bad = nb;
#pragma omp parallel for schedule(static) reduction(min : bad)
    for (int64_t b = 0; b < nb; ++b) {
      in_slot[b] = B[b].in_slot;
      out_slot[b] = B[b].out_slot;
      if (in_slot[b] >= ns || out_slot[b] >= ns ||
          (B[b].stage != 0 && in_slot[b] < 0) || (B[b].stage >= 0 && out_slot[b] < 0))
        bad = std::min(bad, b);
    }
    if (bad < nb) {
      set_error("pack: block %lld has invalid slot ids", (long long)bad);
      return BF_EINVAL;
    }
  } else
  for (int64_t b : order) {
    const LBlock& k = B[b];
    if (k.stage == 0) {
      if (!node_ok(lg.src_vals, k.si)) {
        set_error("pack: Q block %lld src_in node %lld unknown", (long long)b, (long long)k.si);
        return BF_EINVAL;
      }
      int64_t m = lg.src_vals.n(k.si);
      if (!k.ident && k.cols != m) {
        set_error("pack: Q block %lld has %d cols but values(src_in) has %lld", (long long)b,
                  k.cols, (long long)m);
        return BF_EINVAL;
      }
      int64_t so = get_slot(k.bf, 0, k.oo, k.so, true);
      if (so < 0) {
        set_error("pack: Q block %lld has node ids outside [0, 2^31)", (long long)b);
        return BF_EINVAL;
      }
      int64_t len = k.ident ? m : k.rows;
      if (slot_len[so] >= 0 && slot_len[so] != len) {
        set_error("pack: slot size mismatch at Q block %lld", (long long)b);
        return BF_EINVAL;
      }
      slot_len[so] = len;
      out_slot[b] = so;
    } else if (k.stage > 0) {
      int64_t si = get_slot(k.bf, k.stage - 1, k.oi, k.si, false);
      if (si < 0 || slot_len[si] < 0) {
        set_error("pack: R%d block %lld reads a slot no earlier level writes", k.stage,
                  (long long)b);
        return BF_EINVAL;
      }
      if (!k.ident && k.cols != slot_len[si]) {
        set_error("pack: R%d block %lld has %d cols, input slot has %lld", k.stage, (long long)b,
                  k.cols, (long long)slot_len[si]);
        return BF_EINVAL;
      }
      int64_t so = get_slot(k.bf, k.stage, k.oo, k.so, true);
      if (so < 0) {
        set_error("pack: R%d block %lld has node ids outside [0, 2^31)", k.stage, (long long)b);
        return BF_EINVAL;
      }
      int64_t len = k.ident ? slot_len[si] : k.rows;
      if (slot_len[so] >= 0 && slot_len[so] != len) {
        set_error("pack: slot size mismatch at R%d block %lld", k.stage, (long long)b);
        return BF_EINVAL;
      }
      slot_len[so] = len;
      in_slot[b] = si;
      out_slot[b] = so;
    } else {
      int64_t si = get_slot(k.bf, nlev[k.bf] - 1, k.oi, k.si, false);
      if (si < 0 || slot_len[si] < 0) {
        set_error("pack: P block %lld reads a slot the last level does not write", (long long)b);
        return BF_EINVAL;
      }
      if (!node_ok(lg.obs_vals, k.oo)) {
        set_error("pack: P block %lld obs_out node %lld unknown", (long long)b, (long long)k.oo);
        return BF_EINVAL;
      }
      int64_t m = lg.obs_vals.n(k.oo);
      if (!k.ident && (k.cols != slot_len[si] || k.rows != m)) {
        set_error("pack: P block %lld is %dx%d, expected %lldx%lld", (long long)b, k.rows, k.cols,
                  (long long)m, (long long)slot_len[si]);
        return BF_EINVAL;
      }
      if (k.ident && slot_len[si] != m) {
        set_error("pack: identity P block %lld size mismatch", (long long)b);
        return BF_EINVAL;
      }
      in_slot[b] = si;
    }
  }
  int64_t n_slots = (int64_t)slot_len.size();

  plog.mark("pack: order + slot wiring");
  // ---- tasks
  std::vector<std::unique_ptr<std::pmr::monotonic_buffer_resource>> arenas;  // outlive stages
  std::vector<std::vector<TaskB>> stages(Lmax + 1);
  {  // Q stage: group by source node (node ids validated above)
    std::vector<int64_t> gid(lg.src_vals.ptr.size(), -1);
    for (int64_t i = sbeg[0]; i < sbeg[1]; ++i) {
      const int64_t b = order[i];
      const LBlock& k = B[b];
      if (gid[k.si] < 0) {
        gid[k.si] = (int64_t)stages[0].size();
        TaskB t;
        t.stage = 0;
        t.kind = TASK_DENSE;
        t.n = lg.src_vals.n(k.si);
        t.cols.push_back({SIDE_X, k.si, t.n});
        stages[0].push_back(std::move(t));
      }
      TaskB& t = stages[0][gid[k.si]];
      int64_t r = slot_len[out_slot[b]];
      t.mats.push_back({k.ident ? -1 : b, (int32_t)t.M, 0, k.ident ? (int32_t)t.n : 0});
      t.rows.push_back({SIDE_SLOT, out_slot[b], r});
      t.M += r;
    }
  }
  plog.mark("pack: Q tasks");
  // per-slot bookkeeping shared by all R levels: a slot is a row at exactly one
  // level (the one that writes it) and a column at exactly one level (the one
  // that reads it), so row/column offsets need no reset; the DSU index of a
  // slot is stamped with its level
  std::vector<int32_t> row_off(n_slots, -1), col_off(n_slots, -1);
  std::vector<int64_t> slot_dsu(n_slots, -1);
  std::vector<int32_t> slot_lvl(n_slots, -1);
  for (int32_t l = 1; l < Lmax; ++l) {  // R levels: connected components over slots
    const int64_t lo = sbeg[l], hi = sbeg[l + 1];
    if (lo == hi) continue;
    // Every slot belongs to one far pair, so no component crosses far pairs.
    // When the level's blocks come grouped by far pair (the builder's order),
    // the level splits at far-pair boundaries into chunks, each with its own
    // union-find, joined in order: the same tasks in the same order as one
    // pass.  Otherwise (an import in another order) it is one chunk.
    std::vector<int64_t> cut{lo};
    {
      bool grouped = true;
      std::vector<uint8_t> seen(lg.n_bf > 0 ? lg.n_bf : 1, 0);
      for (int64_t i = lo; i < hi && grouped; ++i) {
        const int32_t f = B[order[i]].bf;
        if (i == lo || f != B[order[i - 1]].bf) {
          if (f < 0 || f >= lg.n_bf || seen[f]) grouped = false;
          else seen[f] = 1;
        }
      }
      const int64_t want = grouped ? std::min<int64_t>(hi - lo, 1024) : 1;
      for (int64_t k = 1; k < want; ++k) {
        int64_t p = std::max(lo + (hi - lo) * k / want, cut.back() + 1);
        while (p < hi && B[order[p]].bf == B[order[p - 1]].bf) ++p;
        if (p >= hi) break;
        cut.push_back(p);
      }
      cut.push_back(hi);
    }
    const int64_t nc = (int64_t)cut.size() - 1;
    std::vector<std::vector<TaskB>> part(nc);
    const size_t a0 = arenas.size();
    for (int64_t c = 0; c < nc; ++c)
      arenas.push_back(std::make_unique<std::pmr::monotonic_buffer_resource>());
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < nc; ++c) {
      DSU d;
      std::vector<TaskB>& out = part[c];
      std::pmr::memory_resource* arena = arenas[a0 + c].get();
      auto idx = [&](int64_t slot) {
        if (slot_lvl[slot] == l) return slot_dsu[slot];
        int64_t i = (int64_t)d.p.size();
        d.p.push_back(i);
        slot_lvl[slot] = l;
        slot_dsu[slot] = i;
        return i;
      };
      for (int64_t i = cut[c]; i < cut[c + 1]; ++i) {
        const int64_t b = order[i];
        if (!B[b].ident) d.unite(idx(in_slot[b]), idx(out_slot[b]));
      }
      std::vector<int64_t> comp(d.p.size(), -1);  // dsu root -> task
      for (int64_t i = cut[c]; i < cut[c + 1]; ++i) {
        const int64_t b = order[i];
        const LBlock& k = B[b];
        if (k.ident) {
          TaskB t(arena);
          t.stage = l;
          t.kind = TASK_COPY;
          int64_t len = slot_len[in_slot[b]];
          t.rows.push_back({SIDE_SLOT, out_slot[b], len});
          t.cols.push_back({SIDE_SLOT, in_slot[b], len});
          t.M = t.n = len;
          out.push_back(std::move(t));
          continue;
        }
        int64_t root = d.find(idx(in_slot[b]));
        if (comp[root] < 0) {
          comp[root] = (int64_t)out.size();
          TaskB t(arena);
          t.stage = l;
          t.kind = TASK_DENSE;
          out.push_back(std::move(t));
        }
        TaskB& t = out[comp[root]];
        const int64_t os = out_slot[b], is = in_slot[b];
        if (row_off[os] < 0) {
          row_off[os] = (int32_t)t.M;
          t.rows.push_back({SIDE_SLOT, os, slot_len[os]});
          t.M += slot_len[os];
        }
        if (col_off[is] < 0) {
          col_off[is] = (int32_t)t.n;
          t.cols.push_back({SIDE_SLOT, is, slot_len[is]});
          t.n += slot_len[is];
        }
        t.mats.push_back({b, row_off[os], col_off[is], 0});
      }
    }
    size_t tot = stages[l].size();
    for (auto& p : part) tot += p.size();
    stages[l].reserve(tot);
    for (auto& p : part)
      for (auto& t : p) stages[l].push_back(std::move(t));
  }
  plog.mark("pack: R tasks");
  {  // P stage: group by observer node (node ids validated above)
    std::vector<int64_t> gid(lg.obs_vals.ptr.size(), -1);
    for (int64_t i = sbeg[Lmax]; i < sbeg[Lmax + 1]; ++i) {  // stage rank Lmax: P blocks
      const int64_t b = order[i];
      const LBlock& k = B[b];
      if (gid[k.oo] < 0) {
        gid[k.oo] = (int64_t)stages[Lmax].size();
        TaskB t;
        t.stage = Lmax;
        t.kind = TASK_DENSE;
        t.M = lg.obs_vals.n(k.oo);
        t.rows.push_back({SIDE_Y, k.oo, t.M});
        stages[Lmax].push_back(std::move(t));
      }
      TaskB& t = stages[Lmax][gid[k.oo]];
      int64_t c = slot_len[in_slot[b]];
      t.mats.push_back({k.ident ? -1 : b, 0, (int32_t)t.n, k.ident ? (int32_t)c : 0});
      t.cols.push_back({SIDE_SLOT, in_slot[b], c});
      t.n += c;
    }
  }
  plog.mark("pack: P tasks");
  // big tasks first inside each launch (longest-processing-time order)
  // (a parallel sort of (size, position) keys, so ties keep their order as in
  // a stable sort; then the tasks move into place)
  // lpt[s] lists the tasks of stage s in that order; the tasks stay in place
  std::vector<std::vector<int64_t>> lpt(Lmax + 1), lpos(Lmax + 1);  // order and its inverse
  for (int32_t s = 0; s <= Lmax; ++s) {
    const std::vector<TaskB>& st = stages[s];
    const int64_t n = (int64_t)st.size();
    std::vector<std::pair<int64_t, int64_t>> key(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) key[i] = {-(st[i].M * st[i].n), i};
    __gnu_parallel::sort(key.begin(), key.end());
    lpt[s].resize(n);
    lpos[s].resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      lpt[s][i] = key[i].second;
      lpos[s][key[i].second] = i;
    }
  }

  plog.mark("pack: LPT sort");
  // ---- workspace layout: [x space | y space | slots in reader order]
  plan.xg_off = 0;
  plan.yg_off = lg.n_cols;
  int64_t ws = lg.n_cols + lg.n_rows;
  std::vector<int64_t> slot_off(n_slots, -1);
  {
    // When every slot is read by exactly one task (the case for the GPU
    // build), the reader-order layout is a prefix sum over the tasks' column
    // sizes and is assigned in parallel; otherwise one serial first-appearance
    // pass gives the same definition.
    std::vector<uint8_t> readers(n_slots, 0);
    int shared_slot = 0;
    for (int32_t s = 1; s <= Lmax; ++s) {
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : shared_slot)
      for (int64_t q = 0; q < (int64_t)lpt[s].size(); ++q)
        for (auto& c : stages[s][lpt[s][q]].cols)
          if (c.type == SIDE_SLOT && __atomic_exchange_n(&readers[c.id], (uint8_t)1, __ATOMIC_RELAXED))
            shared_slot = 1;
    }
    if (!shared_slot) {
      for (int32_t s = 1; s <= Lmax; ++s) {
        const int64_t n = (int64_t)lpt[s].size();
        std::vector<int64_t> base(n + 1, 0);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n; ++q) {
          int64_t tot = 0;
          for (auto& c : stages[s][lpt[s][q]].cols)
            if (c.type == SIDE_SLOT) tot += c.len;
          base[q + 1] = tot;
        }
        base[0] = ws;
        for (int64_t q = 0; q < n; ++q) base[q + 1] += base[q];
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n; ++q) {
          int64_t o = base[q];
          for (auto& c : stages[s][lpt[s][q]].cols)
            if (c.type == SIDE_SLOT) {
              slot_off[c.id] = o;
              o += c.len;
            }
        }
        ws = base[n];
      }
    } else {
      for (int32_t s = 1; s <= Lmax; ++s)
        for (int64_t i : lpt[s])
          for (auto& c : stages[s][i].cols)
            if (c.type == SIDE_SLOT && slot_off[c.id] < 0) {
              slot_off[c.id] = ws;
              ws += c.len;
            }
    }
  }
  for (int64_t s = 0; s < n_slots; ++s)
    if (slot_off[s] < 0) {
      slot_off[s] = ws;
      ws += std::max<int64_t>(slot_len[s], 0);
    }
  plan.ws_entries = ws;
  if (ws >= (int64_t)1 << 31) {
    set_error("pack: workspace of %lld entries exceeds int32 routing", (long long)ws);
    return BF_ENOTSUP;
  }

  plog.mark("pack: workspace layout");
  // ---- leaf order of the x and y regions: the points of each Q-stage source
  // leaf (P-stage observer leaf) become one contiguous range
  std::vector<int64_t> xpos(lg.n_cols, -1), ypos(lg.n_rows, -1);
  {
    int64_t nx = 0, ny = 0;
    for (int64_t i : lpt[0])
      for (auto& c : stages[0][i].cols)
        if (c.type == SIDE_X) {
          const int64_t* v = lg.src_vals.v(c.id);
          for (int64_t i = 0; i < c.len; ++i)
            if (xpos[v[i]] < 0) xpos[v[i]] = nx++;
        }
    for (int64_t i : lpt[Lmax])
      for (auto& r : stages[Lmax][i].rows)
        if (r.type == SIDE_Y) {
          const int64_t* v = lg.obs_vals.v(r.id);
          for (int64_t i = 0; i < r.len; ++i)
            if (ypos[v[i]] < 0) ypos[v[i]] = ny++;
        }
    for (int64_t p = 0; p < lg.n_cols; ++p)
      if (xpos[p] < 0) xpos[p] = nx++;
    for (int64_t p = 0; p < lg.n_rows; ++p)
      if (ypos[p] < 0) ypos[p] = ny++;
    plan.xperm.assign(lg.n_cols, 0);
    plan.yperm.assign(lg.n_rows, 0);
    for (int64_t p = 0; p < lg.n_cols; ++p) plan.xperm[xpos[p]] = (int32_t)p;
    for (int64_t p = 0; p < lg.n_rows; ++p) plan.yperm[ypos[p]] = (int32_t)p;
  }

  plog.mark("pack: leaf order");
  // ---- emit tasks, maps, repack segments
  std::vector<uint8_t> ycov(lg.n_rows, 0), xcov(lg.n_cols, 0);
  auto contiguous_base = [&](int64_t off, int64_t len) -> int {
    if (len <= 0) return -1;
    int32_t b = plan.maps[off];
    for (int64_t i = 1; i < len; ++i)
      if (plan.maps[off + i] != b + i) return -1;
    return b;
  };
  // offsets of every task's maps, segments and matrix (per-task counts in
  // parallel, serial prefix sums), then the tasks are emitted in parallel,
  // each into its own ranges
  struct TRef {
    int32_t s;
    int64_t i, map_off, seg_off, a_off;
  };
  std::vector<TRef> all;
  plan.stage_begin.push_back(0);
  for (int32_t s = 0; s <= Lmax; ++s)
    plan.stage_begin.push_back(plan.stage_begin.back() + (int64_t)stages[s].size());
  all.resize((size_t)plan.stage_begin.back());
  int too_large = 0;
  for (int32_t s = 0; s <= Lmax; ++s) {
    const int64_t base = plan.stage_begin[s];
#pragma omp parallel for schedule(static) reduction(| : too_large)
    for (int64_t i = 0; i < (int64_t)stages[s].size(); ++i) {  // storage order
      const int64_t q = lpos[s][i];
      const TaskB& t = stages[s][i];
      if (t.M > INT32_MAX || t.n > INT32_MAX) too_large = 1;
      // counts for now; turned into offsets below
      TRef r{s, i, t.M + t.n, 0, 0};
      if (t.kind == TASK_DENSE) {
        r.a_off = t.M * t.n;
        for (auto& m : t.mats) {
          const int64_t rr = m.blk < 0 ? m.ident_n : B[m.blk].rows;
          const int64_t cc = m.blk < 0 ? m.ident_n : B[m.blk].cols;
          if (rr > 0 && cc > 0) ++r.seg_off;
        }
      }
      all[base + q] = r;
    }
  }
  if (too_large) {
    set_error("pack: task too large");
    return BF_ENOTSUP;
  }
  int64_t n_maps = 0, n_segs = 0, a_off = 0;
  for (TRef& r : all) {
    const int64_t nm = r.map_off, ns = r.seg_off, na = r.a_off;
    const bool dense = stages[r.s][r.i].kind == TASK_DENSE;
    r.map_off = n_maps;
    r.seg_off = n_segs;
    r.a_off = dense ? a_off : -1;
    n_maps += nm;
    n_segs += ns;
    a_off += na;
  }
  if (n_maps > (int64_t)INT32_MAX * 8) {
    set_error("pack: routing maps too large");
    return BF_ENOTSUP;
  }
  plan.maps.resize((size_t)n_maps);
  plan.segs.resize((size_t)n_segs);
  plan.tasks.resize(all.size());
  std::vector<int64_t> sbytes(Lmax + 1, 0);
  int64_t block_entries = 0, max_rank = 0;
  // tasks are visited in storage order (sequential reads of the task lists);
  // each is written at its launch-order position q
  std::vector<int64_t> qpos(all.size());
  for (int32_t s = 0; s <= Lmax; ++s) {
    const int64_t base = plan.stage_begin[s];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)stages[s].size(); ++i) qpos[base + i] = base + lpos[s][i];
  }
#pragma omp parallel for schedule(dynamic, 512) reduction(+ : block_entries) \
    reduction(max : max_rank)
  for (int64_t g = 0; g < (int64_t)all.size(); ++g) {
    const int64_t q = qpos[g];
    const TRef& r = all[q];
    const TaskB& t = stages[r.s][r.i];
    int64_t tb = 16 * (t.M + t.n);
    DTask d{};
    d.M = (int)t.M;
    d.n = (int)t.n;
    d.kind = t.kind;
    int32_t* mp = plan.maps.data() + r.map_off;
    auto emit = [&](const Side& sd) {
      if (sd.type == SIDE_SLOT) {
        for (int64_t i = 0; i < sd.len; ++i) *mp++ = (int32_t)(slot_off[sd.id] + i);
      } else if (sd.type == SIDE_X) {
        const int64_t* v = lg.src_vals.v(sd.id);
        for (int64_t i = 0; i < sd.len; ++i) *mp++ = (int32_t)(plan.xg_off + xpos[v[i]]);
      } else {
        const int64_t* v = lg.obs_vals.v(sd.id);
        for (int64_t i = 0; i < sd.len; ++i) *mp++ = (int32_t)(plan.yg_off + ypos[v[i]]);
      }
    };
    d.rmap_off = (long long)r.map_off;
    for (auto& rw : t.rows) emit(rw);
    d.cmap_off = (long long)(r.map_off + t.M);
    for (auto& c : t.cols) emit(c);
    d.rbase = contiguous_base(d.rmap_off, t.M);
    d.cbase = contiguous_base(d.cmap_off, t.n);
    d.a_off = r.a_off;
    if (t.kind == TASK_DENSE) {
      int64_t so = r.seg_off;
      for (auto& m : t.mats) {
        DSeg g{};
        g.dst_ld = (int)t.M;
        g.dst_off = r.a_off + (long long)m.col_off * t.M + m.row_off;
        if (m.blk < 0) {
          g.kind = 1;
          g.rows = g.cols = m.ident_n;
        } else {
          const LBlock& k = B[m.blk];
          g.kind = 0;
          g.src_off = k.raw_off;
          g.src_ld = k.raw_ld;
          g.rows = k.rows;
          g.cols = k.cols;
          plan.blk_pk_off[m.blk] = g.dst_off;  // each block is in exactly one task
          plan.blk_pk_ld[m.blk] = g.dst_ld;
          block_entries += (int64_t)k.rows * k.cols;
          tb += (int64_t)plan.fac_bytes * k.rows * k.cols;
          max_rank = std::max<int64_t>(max_rank, k.rows);
        }
        if (g.rows > 0 && g.cols > 0) plan.segs[so++] = g;
      }
    }
    plan.tasks[q] = d;
#pragma omp atomic
    sbytes[r.s] += tb;
  }
  plan.block_entries = block_entries;
  plan.max_rank = max_rank;
  plan.stage_bytes.assign(sbytes.begin(), sbytes.end());
  plan.a_entries = a_off;
  // coverage of x (Q-task columns) and y (P-task rows); every output row has
  // exactly one P-task writer (an atomic exchange finds a second one)
  int64_t dup_row = -1;
  for (int32_t s : {0, Lmax}) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t q = 0; q < (int64_t)stages[s].size(); ++q) {
      const TaskB& t = stages[s][q];
      for (auto& c : t.cols)
        if (c.type == SIDE_X) {
          const int64_t* v = lg.src_vals.v(c.id);
          for (int64_t i = 0; i < c.len; ++i) __atomic_store_n(&xcov[v[i]], 1, __ATOMIC_RELAXED);
        }
      for (auto& rw : t.rows)
        if (rw.type == SIDE_Y) {
          const int64_t* v = lg.obs_vals.v(rw.id);
          for (int64_t i = 0; i < rw.len; ++i)
            if (__atomic_exchange_n(&ycov[v[i]], (uint8_t)1, __ATOMIC_RELAXED))
              __atomic_store_n(&dup_row, v[i], __ATOMIC_RELAXED);
        }
    }
  }
  if (dup_row >= 0) {
    set_error("pack: output row %lld written by two P tasks", (long long)dup_row);
    return BF_EINVAL;
  }
  plog.mark("pack: emit tasks/maps");
  // forward launch lists by task shape (kernels in bf_matvec.cu)
  {
    std::vector<int32_t> cls[Plan::L_NCLASS];
    for (auto& b : plan.list_begin) b.assign(1, 0);
    std::vector<std::vector<int64_t>> ends(Plan::L_NCLASS);
    for (int64_t s = 0; s + 1 < (int64_t)plan.stage_begin.size(); ++s) {
      for (int64_t gi = plan.stage_begin[s]; gi < plan.stage_begin[s + 1]; ++gi) {
        const DTask& d = plan.tasks[gi];
        // adjoint lists (a task with no rows still writes zeros to its columns)
        if (d.kind == TASK_DENSE && d.n > 0) {
          if (d.M <= 32 && d.n > 2 * d.M && d.n >= WIDE_NMIN) {
            // served by L_WIDE below
          } else if (d.M > ADJ_TALL_M) {
            cls[Plan::L_ATALL].push_back((int32_t)gi);
          } else {
            cls[Plan::L_AWARP].push_back((int32_t)gi);
          }
        }
        if (d.M <= 0) continue;
        if (d.kind == TASK_DENSE) cls[Plan::L_DENSE].push_back((int32_t)gi);
        if (d.kind == TASK_COPY) {
          cls[Plan::L_COPY].push_back((int32_t)gi);
        } else if (d.M <= 32 && d.n > 2 * d.M && d.n >= WIDE_NMIN) {
          cls[Plan::L_WIDE].push_back((int32_t)gi);
        } else if (d.M <= 32) {
          cls[Plan::L_SMALL].push_back((int32_t)gi);
        } else if (d.M <= FLAT_MMAX && d.n <= FLAT_NMAX) {
          cls[Plan::L_FLAT].push_back((int32_t)gi);
        } else {
          for (int32_t r0 = 0; r0 < d.M; r0 += TALL_ROWS * TALL_PANELS) {
            cls[Plan::L_TALL].push_back((int32_t)gi);
            cls[Plan::L_TALL].push_back(r0);
          }
        }
      }
      for (int c = 0; c < Plan::L_NCLASS; ++c) ends[c].push_back((int64_t)cls[c].size());
      bool tma = true;
      for (int64_t gi = plan.stage_begin[s]; gi < plan.stage_begin[s + 1]; ++gi) {
        const DTask& d = plan.tasks[gi];
        if (d.kind == TASK_DENSE && d.M > 0 && d.n > 0 && d.cbase < 0) tma = false;
      }
      plan.stage_tma.push_back(tma ? 1 : 0);
    }
    // concatenate; list_begin holds absolute offsets into plan.lists
    for (int c = 0; c < Plan::L_NCLASS; ++c) {
      int64_t base = (int64_t)plan.lists.size();
      plan.list_begin[c].assign(1, base);
      for (int64_t e : ends[c]) plan.list_begin[c].push_back(base + e);
      plan.lists.insert(plan.lists.end(), cls[c].begin(), cls[c].end());
    }
  }
  plan.yg_covered = std::all_of(ycov.begin(), ycov.end(), [](uint8_t c) { return c != 0; });
  plan.xg_covered = std::all_of(xcov.begin(), xcov.end(), [](uint8_t c) { return c != 0; });
  int64_t slot_total = 0;
  for (int64_t s = 0; s < n_slots; ++s) slot_total += std::max<int64_t>(slot_len[s], 0);
  // algorithmic bytes of one forward matvec: factor entries (fac_bytes each:
  // 16 float-float, 8 complex FP32) + x read + y write + every level slot
  // written once and read once (16 B per float-float vector entry)
  plan.alg_bytes_fwd = (int64_t)plan.fac_bytes * plan.block_entries +
                       16 * (lg.n_rows + lg.n_cols + 2 * slot_total);
  plog.mark("pack: class lists + totals");
  // the R tasks' arrays live in the arenas: dropping them releases a few
  // large buffers, not one allocation per array
  stages.clear();
  stages.shrink_to_fit();
  arenas.clear();
  plog.mark("pack: free task lists");
  return BF_OK;
}

}  // namespace bfg
