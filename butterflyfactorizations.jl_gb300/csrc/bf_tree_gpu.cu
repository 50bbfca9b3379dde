// Cluster trees and interaction lists built on the GPU (bf_tree_build_gpu,
// bf_nearandfar_gpu): node for node and pair for pair the same results as the
// host versions (bf_tree.cpp), which follow the reference's tree contract
// (src/treeinterface.jl:39-164) and its dual-tree traversal
// (src/Matrixassembly/intlists.jl:30-217) with the AABB isFarFunctor
// (ext/BFH2Trees/h2admissible.jl:11-45).
//
// Tree: the device does the per-point work -- the bounding box and, level by
// level, one stable octant partition of every node that splits (a CTA per
// node; warp ballots rank the points of a chunk per octant, so the scatter
// keeps the input order without atomics).  The host does the per-node work
// with the host builder's rules (leaf test, child order, numbering), so the
// numbering is identical by construction.
//
// Traversal: level-synchronous on the device.  Every pair carries the digits
// of its depth-first path (the index of each step among its parent's kids,
// six bits per level, in a 128-bit key), so each level's far / near outputs
// come out sorted by key when the level expands in order.  The depth-first
// order of the host traversal is the key order of all outputs; each output's
// final position is the number of keys below it over all levels, found by
// binary search in every level's sorted outputs -- a merge without a sort.
// The admissibility test runs in FP64 with non-contracting intrinsics, so its
// decisions are those of the host test bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "bf_internal.h"

namespace bfg {
namespace {

// ------------------------------------------------------------------ scans
constexpr int SCAN_T = 256;
constexpr int SCAN_PER = 8;  // elements per thread per block tile
constexpr int SCAN_TILE = SCAN_T * SCAN_PER;

__device__ __forceinline__ int64_t block_exclusive(int64_t v, int64_t* sh, int64_t* total) {
  // Hillis-Steele over the block (256 threads)
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int o = 1; o < SCAN_T; o <<= 1) {
    const int64_t a = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += a;
    __syncthreads();
  }
  const int64_t incl = sh[t];
  if (total) *total = sh[SCAN_T - 1];
  __syncthreads();
  return incl - v;
}

__global__ void scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  __shared__ int64_t sh[SCAN_T];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER;
  int64_t v = 0;
  for (int q = 0; q < SCAN_PER; ++q)
    if (base + q < n) v += in[base + q];
  int64_t tot = 0;
  block_exclusive(v, sh, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// exclusive scan of the tile sums in place (one block, any length)
__global__ void scan_sums(int64_t* __restrict__ sums, int64_t nt, int64_t* __restrict__ total) {
  __shared__ int64_t sh[SCAN_T];
  int64_t carry = 0;
  for (int64_t b = 0; b < nt; b += SCAN_T) {
    const int64_t i = b + threadIdx.x;
    const int64_t v = i < nt ? sums[i] : 0;
    int64_t tot = 0;
    const int64_t ex = block_exclusive(v, sh, &tot);
    if (i < nt) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_apply(const int32_t* __restrict__ in, int64_t n,
                           const int64_t* __restrict__ sums, int64_t* __restrict__ out) {
  __shared__ int64_t sh[SCAN_T];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER;
  int64_t v = 0;
  for (int q = 0; q < SCAN_PER; ++q)
    if (base + q < n) v += in[base + q];
  int64_t run = sums[blockIdx.x] + block_exclusive(v, sh, nullptr);
  for (int q = 0; q < SCAN_PER; ++q)
    if (base + q < n) {
      out[base + q] = run;
      run += in[base + q];
    }
}

// device buffers of one call, freed on every exit path
struct DevBufs {
  std::vector<void*> p;
  template <typename T>
  int get(T** out, size_t n, const char* what) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      set_error("%s: device allocation of %zu bytes failed", what, n * sizeof(T));
      return BF_ENOMEM;
    }
    p.push_back(q);
    *out = (T*)q;
    return BF_OK;
  }
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
};

// out[i] = sum of in[0..i), *total = sum of all (host value); scratch sized by the caller
int exclusive_scan(const int32_t* in, int64_t n, int64_t* out, int64_t* sums, int64_t* d_total,
                   int64_t* total, cudaStream_t st) {
  if (n <= 0) {
    *total = 0;
    return BF_OK;
  }
  const int64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
  scan_tile_sums<<<(unsigned)nt, SCAN_T, 0, st>>>(in, n, sums);
  scan_sums<<<1, SCAN_T, 0, st>>>(sums, nt, d_total);
  scan_apply<<<(unsigned)nt, SCAN_T, 0, st>>>(in, n, sums, out);
  BF_TRY_CUDA(cudaGetLastError());
  BF_TRY_CUDA(cudaMemcpyAsync(total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  BF_TRY_CUDA(cudaStreamSynchronize(st));
  return BF_OK;
}

// ------------------------------------------------------------------ tree
__global__ void bbox_kernel(const double* __restrict__ xyz, int64_t n, double* __restrict__ part,
                            int* __restrict__ bad) {
  __shared__ double sh[6][256];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int a = 0; a < 3; ++a) {
      const double v = xyz[3 * i + a];
      if (!isfinite(v)) atomicExch(bad, 1);
      lo[a] = fmin(lo[a], v);
      hi[a] = fmax(hi[a], v);
    }
  for (int a = 0; a < 3; ++a) {
    sh[a][threadIdx.x] = lo[a];
    sh[3 + a][threadIdx.x] = hi[a];
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int a = 0; a < 3; ++a) {
        sh[a][threadIdx.x] = fmin(sh[a][threadIdx.x], sh[a][threadIdx.x + o]);
        sh[3 + a][threadIdx.x] = fmax(sh[3 + a][threadIdx.x], sh[3 + a][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

struct alignas(16) SplitNode {
  long long b, e;
  double c[3];
  double pad;
};

__device__ __forceinline__ int octant(const double* __restrict__ xyz, int32_t p, const double* c) {
  const double* q = xyz + 3 * (long long)p;
  return (q[0] >= c[0] ? 1 : 0) + (q[1] >= c[1] ? 2 : 0) + (q[2] >= c[2] ? 4 : 0);
}

// Stable partition of perm[b, e) of one split node by octant (CTA per node,
// 256 threads): counts, then ranks per octant chunk by chunk (warp ballots),
// scatter to tmp, copy back.  counts[8*node + o] = points in octant o.
__global__ void __launch_bounds__(256) partition_kernel(const SplitNode* __restrict__ nodes,
                                                        const double* __restrict__ xyz,
                                                        int32_t* __restrict__ perm,
                                                        int32_t* __restrict__ tmp,
                                                        int32_t* __restrict__ counts) {
  __shared__ int cnt[8], base[8], wcnt[8][8];
  const SplitNode nd = nodes[blockIdx.x];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < 8) cnt[t] = 0;
  __syncthreads();
  int local[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long i = nd.b + t; i < nd.e; i += 256) local[octant(xyz, perm[i], nd.c)]++;
  for (int o = 0; o < 8; ++o)
    if (local[o]) atomicAdd(&cnt[o], local[o]);
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int o = 0; o < 8; ++o) {
      base[o] = acc;
      acc += cnt[o];
      counts[8 * blockIdx.x + o] = cnt[o];
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (long long c0 = nd.b; c0 < nd.e; c0 += 256) {
    const long long i = c0 + t;
    const bool valid = i < nd.e;
    const int32_t p = valid ? perm[i] : 0;
    const int o = valid ? octant(xyz, p, nd.c) : -1;
    int rank = 0;
    for (int q = 0; q < 8; ++q) {
      const unsigned m = __ballot_sync(0xffffffffu, o == q);
      if (lane == 0) wcnt[warp][q] = __popc(m);
      if (o == q) rank = __popc(m & lt);
    }
    __syncthreads();
    if (valid) {
      int pre = base[o];
      for (int w = 0; w < warp; ++w) pre += wcnt[w][o];
      tmp[nd.b + pre + rank] = p;
    }
    __syncthreads();
    if (t < 8)
      for (int w = 0; w < 8; ++w) base[t] += wcnt[w][t];
    __syncthreads();
  }
  for (long long i = nd.b + t; i < nd.e; i += 256) perm[i] = tmp[i];
}

// ------------------------------------------------------------------ traversal
struct TreeDev {
  const double* center;
  const double* half;
  const int32_t* first_child;
  const int32_t* n_child;
};

struct alignas(16) PairKey {
  unsigned long long hi, lo;  // 21 digits of 6 bits, left-aligned (digit 0 in the top bits of hi)
};

__device__ __forceinline__ bool key_less(const PairKey& a, const PairKey& b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// digit d (< 64) at depth L (0-based) of a left-aligned key
__device__ __forceinline__ PairKey key_with(PairKey k, int L, unsigned long long d) {
  // bits [126 - 6L - 6, 126 - 6L) of the 128-bit key (the top two bits stay zero)
  const int lo_bit = 120 - 6 * L;
  if (lo_bit >= 64) {
    k.hi |= d << (lo_bit - 64);
  } else if (lo_bit + 6 <= 64) {
    k.lo |= d << lo_bit;
  } else {  // straddles the words
    k.lo |= d << lo_bit;
    k.hi |= d >> (64 - lo_bit);
  }
  return k;
}

// the host test of bf_tree.cpp (is_far) with every FP64 operation rounded on its own
__device__ bool is_far_dev(const TreeDev& ts, const TreeDev& to, int s, int o, double alpha,
                           double sqrt3) {
  const double ol = __dmul_rn(to.half[o], sqrt3), sl = __dmul_rn(ts.half[s], sqrt3);
  const double W = fmax(sl, ol);
  const double target = __dmul_rn(alpha, W);
  double mind_sq = 0.0;
  const double r = __dadd_rn(sl, ol);
  for (int i = 0; i < 3; ++i) {
    const double d = __dsub_rn(fabs(__dsub_rn(to.center[3 * o + i], ts.center[3 * s + i])), r);
    if (d > 0.0) mind_sq = __dadd_rn(mind_sq, __dmul_rn(d, d));
  }
  if (mind_sq < 1e-10) return false;
  return __dsqrt_rn(mind_sq) > target;
}

// unbalanced splitting: the observer node splits when it is the larger one
// (largernode: radius(o) >= radius(s), treeinterface.jl:153-154) and not a
// leaf, or when the source node is a leaf
__device__ __forceinline__ bool split_obs(const TreeDev& to, const TreeDev& ts, int o, int s,
                                          bool lo, bool ls, double sqrt3) {
  return (__dmul_rn(to.half[o], sqrt3) >= __dmul_rn(ts.half[s], sqrt3) && !lo) || ls;
}

// classify every pair of a level: flags far / near, kid count
__global__ void classify_kernel(const int32_t* __restrict__ po, const int32_t* __restrict__ ps,
                                int64_t n, TreeDev to, TreeDev ts, int h, double alpha,
                                double sqrt3, int minbflvl, int leafcomp, int leafimbalance,
                                int unbal, int32_t* __restrict__ is_far,
                                int32_t* __restrict__ is_near, int32_t* __restrict__ nkids) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int o = po[i], s = ps[i];
    const bool lo = to.n_child[o] == 0, ls = ts.n_child[s] == 0;
    int f = 0, nr = 0, k = 0;
    if (h <= minbflvl && !leafcomp) {
      nr = 1;
    } else if (is_far_dev(ts, to, s, o, alpha, sqrt3)) {
      if ((lo || ls) && !leafcomp)
        nr = 1;
      else
        f = 1;
    } else if ((lo && ls) || ((lo || ls) && !leafimbalance)) {
      nr = 1;
    } else if (unbal) {  // only the larger node splits (intlists.jl:121-149)
      k = split_obs(to, ts, o, s, lo, ls, sqrt3) ? to.n_child[o] : ts.n_child[s];
    } else {
      k = lo ? ts.n_child[s] : (ls ? to.n_child[o] : to.n_child[o] * ts.n_child[s]);
    }
    is_far[i] = f;
    is_near[i] = nr;
    nkids[i] = k;
  }
}

// outputs of the level at their positions; kids into the next frontier in order
__global__ void expand_kernel(const int32_t* __restrict__ po, const int32_t* __restrict__ ps,
                              const PairKey* __restrict__ pk, int64_t n, int L, TreeDev to,
                              TreeDev ts, int unbal, double sqrt3,
                              const int32_t* __restrict__ is_far,
                              const int32_t* __restrict__ is_near,
                              const int32_t* __restrict__ nkids, const int64_t* __restrict__ far_pos,
                              const int64_t* __restrict__ near_pos,
                              const int64_t* __restrict__ kid_pos, int32_t* __restrict__ fo,
                              int32_t* __restrict__ fs, PairKey* __restrict__ fk,
                              int32_t* __restrict__ no, int32_t* __restrict__ ns,
                              PairKey* __restrict__ nk, int32_t* __restrict__ qo,
                              int32_t* __restrict__ qs, PairKey* __restrict__ qk) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int o = po[i], s = ps[i];
    const PairKey key = pk[i];
    if (is_far[i]) {
      fo[far_pos[i]] = o;
      fs[far_pos[i]] = s;
      fk[far_pos[i]] = key;
    } else if (is_near[i]) {
      no[near_pos[i]] = o;
      ns[near_pos[i]] = s;
      nk[near_pos[i]] = key;
    } else if (nkids[i] > 0) {
      const bool lo = to.n_child[o] == 0, ls = ts.n_child[s] == 0;
      const int nco = to.n_child[o], ncs = ts.n_child[s];
      const bool so = unbal && split_obs(to, ts, o, s, lo, ls, sqrt3);
      int64_t q = kid_pos[i];
      for (int j = 0; j < nkids[i]; ++j, ++q) {
        int co, cs;
        if (unbal) {
          co = so ? to.first_child[o] + j : o;
          cs = so ? s : ts.first_child[s] + j;
        } else if (lo) {
          co = o;
          cs = ts.first_child[s] + j;
        } else if (ls) {
          co = to.first_child[o] + j;
          cs = s;
        } else {
          co = to.first_child[o] + j / ncs;
          cs = ts.first_child[s] + j % ncs;
        }
        (void)nco;
        qo[q] = co;
        qs[q] = cs;
        qk[q] = key_with(key, L, (unsigned long long)j);
      }
    }
  }
}

// final depth-first position of every output of level `lv`: its index in the
// level plus, for every other level, the outputs with smaller keys there
struct LevelKeys {
  const PairKey* k;
  int64_t n, base;  // sorted keys, count, unused
};

__global__ void place_kernel(const int32_t* __restrict__ so, const int32_t* __restrict__ ss,
                             const PairKey* __restrict__ sk, int64_t n, int lv,
                             const LevelKeys* __restrict__ levels, int n_levels,
                             int64_t* __restrict__ out_o, int64_t* __restrict__ out_s,
                             int64_t capacity) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const PairKey key = sk[i];
    int64_t pos = i;
    for (int L = 0; L < n_levels; ++L) {
      if (L == lv) continue;
      int64_t a = 0, b = levels[L].n;  // lower bound of key in level L
      while (a < b) {
        const int64_t m = (a + b) >> 1;
        if (key_less(levels[L].k[m], key))
          a = m + 1;
        else
          b = m;
      }
      pos += a;
    }
    if (pos < capacity) {
      out_o[pos] = so[i];
      out_s[pos] = ss[i];
    }
  }
}

inline unsigned grid_of(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
}

}  // namespace
}  // namespace bfg

using namespace bfg;

extern "C" int bf_tree_build_gpu(bf_ctx_t ctx, const double* xyz, int64_t n, int32_t max_points,
                                 int32_t max_depth, bf_tree_t* out) {
  try {
    if (!ctx || !out) {
      set_error("bf_tree_build_gpu: NULL argument");
      return BF_EINVAL;
    }
    *out = nullptr;
    if (n <= 0 || !xyz) {
      set_error("bf_tree_build_gpu: empty point set");
      return BF_EINVAL;
    }
    if (n >= ((int64_t)1 << 31)) {
      set_error("bf_tree_build_gpu: point sets above 2^31 are not supported");
      return BF_ENOTSUP;
    }
    BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
    cudaStream_t st = nullptr;
    DevBufs mem;
    double *d_xyz, *d_part;
    int32_t *d_perm, *d_tmp, *d_counts;
    int* d_bad;
    BF_TRY(mem.get(&d_xyz, 3 * (size_t)n, "bf_tree_build_gpu"));
    BF_TRY(mem.get(&d_perm, (size_t)n, "bf_tree_build_gpu"));
    BF_TRY(mem.get(&d_tmp, (size_t)n, "bf_tree_build_gpu"));
    const unsigned gb = std::min<unsigned>(1024, (unsigned)((n + 255) / 256));
    BF_TRY(mem.get(&d_part, 6 * (size_t)gb, "bf_tree_build_gpu"));
    BF_TRY(mem.get(&d_bad, 1, "bf_tree_build_gpu"));
    BF_TRY_CUDA(cudaMemcpy(d_xyz, xyz, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemset(d_bad, 0, sizeof(int)));
    bbox_kernel<<<gb, 256, 0, st>>>(d_xyz, n, d_part, d_bad);
    BF_TRY_CUDA(cudaGetLastError());
    std::vector<double> part(6 * (size_t)gb);
    int bad = 0;
    BF_TRY_CUDA(cudaMemcpy(part.data(), d_part, part.size() * sizeof(double),
                           cudaMemcpyDeviceToHost));
    BF_TRY_CUDA(cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) {
      set_error("bf_tree_build_gpu: non-finite coordinate");
      return BF_EINVAL;
    }
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = part[a];
      hi[a] = part[3 + a];
      for (unsigned b = 1; b < gb; ++b) {
        lo[a] = std::min(lo[a], part[6 * b + a]);
        hi[a] = std::max(hi[a], part[6 * b + 3 + a]);
      }
    }
    // identity permutation
    {
      std::vector<int32_t> id((size_t)n);
      for (int64_t i = 0; i < n; ++i) id[i] = (int32_t)i;
      BF_TRY_CUDA(cudaMemcpy(d_perm, id.data(), (size_t)n * sizeof(int32_t),
                             cudaMemcpyHostToDevice));
    }
    auto h = std::make_unique<bf_tree>();
    Tree& t = h->t;
    t.n_points = n;
    double ext = 0.0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
    auto push = [&](const double c[3], double hs, int32_t lvl, int32_t par, int64_t b, int64_t e) {
      t.center.insert(t.center.end(), c, c + 3);
      t.half.push_back(hs);
      t.level.push_back(lvl);
      t.parent.push_back(par);
      t.first_child.push_back(0);
      t.n_child.push_back(0);
      t.begin.push_back(b);
      t.end.push_back(e);
    };
    double c0[3] = {(lo[0] + hi[0]) * 0.5, (lo[1] + hi[1]) * 0.5, (lo[2] + hi[2]) * 0.5};
    push(c0, ext * 0.5, 0, -1, 0, n);
    std::vector<int64_t> current{0}, next;
    std::vector<SplitNode> split;
    std::vector<int64_t> split_id;
    std::vector<int32_t> counts;
    SplitNode* d_split = nullptr;
    size_t split_cap = 0;
    while (!current.empty()) {
      next.clear();
      split.clear();
      split_id.clear();
      for (int64_t nd : current) {  // the host builder's leaf test
        const int64_t cnt = t.end[nd] - t.begin[nd];
        bool leaf = cnt <= 1;
        if (max_points > 0 && cnt <= max_points) leaf = true;
        if (max_depth >= 0 && t.level[nd] >= max_depth) leaf = true;
        if (!(t.half[nd] > 0.0)) leaf = true;
        if (leaf) continue;
        SplitNode s{t.begin[nd], t.end[nd], {t.center[3 * nd], t.center[3 * nd + 1],
                                             t.center[3 * nd + 2]}, 0.0};
        split.push_back(s);
        split_id.push_back(nd);
      }
      if (!split.empty()) {
        if (split.size() > split_cap) {
          split_cap = split.size() * 2;
          BF_TRY(mem.get(&d_split, split_cap, "bf_tree_build_gpu"));
          BF_TRY(mem.get(&d_counts, 8 * split_cap, "bf_tree_build_gpu"));
        }
        BF_TRY_CUDA(cudaMemcpy(d_split, split.data(), split.size() * sizeof(SplitNode),
                               cudaMemcpyHostToDevice));
        partition_kernel<<<(unsigned)split.size(), 256, 0, st>>>(d_split, d_xyz, d_perm, d_tmp,
                                                                 d_counts);
        BF_TRY_CUDA(cudaGetLastError());
        counts.resize(8 * split.size());
        BF_TRY_CUDA(cudaMemcpy(counts.data(), d_counts, counts.size() * sizeof(int32_t),
                               cudaMemcpyDeviceToHost));
      }
      // children in the host builder's order: parents in level order, octants 0..7
      size_t q = 0;
      for (int64_t nd : current) {
        t.first_child[nd] = (int32_t)t.nn();
        if (q >= split_id.size() || split_id[q] != nd) continue;
        const double c[3] = {t.center[3 * nd], t.center[3 * nd + 1], t.center[3 * nd + 2]};
        const double hc = t.half[nd] * 0.5;
        int32_t nc = 0;
        int64_t off = t.begin[nd];
        const int32_t lvl = t.level[nd] + 1;
        for (int o = 0; o < 8; ++o) {
          const int64_t k = counts[8 * q + o];
          if (k == 0) continue;
          double cc[3] = {c[0] + ((o & 1) ? hc : -hc), c[1] + ((o & 2) ? hc : -hc),
                          c[2] + ((o & 4) ? hc : -hc)};
          push(cc, hc, lvl, (int32_t)nd, off, off + k);
          next.push_back(t.nn() - 1);
          off += k;
          ++nc;
        }
        t.n_child[nd] = nc;
        ++q;
      }
      current.swap(next);
    }
    std::vector<int32_t> perm32((size_t)n);
    BF_TRY_CUDA(cudaMemcpy(perm32.data(), d_perm, (size_t)n * sizeof(int32_t),
                           cudaMemcpyDeviceToHost));
    t.perm.assign(perm32.begin(), perm32.end());
    *out = h.release();
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_tree_build_gpu: host allocation failed");
    return BF_ENOMEM;
  }
}

extern "C" int bf_nearandfar_gpu(bf_ctx_t ctx, bf_tree_t obs_tree, bf_tree_t src_tree,
                                 double alpha, int32_t minbflvl, int32_t leafcomp,
                                 int32_t leafimbalance, int32_t unbalancedints,
                                 int64_t* far_obs, int64_t* far_src,
                                 int64_t far_capacity, int64_t* near_obs, int64_t* near_src,
                                 int64_t near_capacity, int64_t* n_far, int64_t* n_near) {
  try {
    if (!ctx || !obs_tree || !src_tree) {
      set_error("bf_nearandfar_gpu: NULL argument");
      return BF_EINVAL;
    }
    const Tree& to = obs_tree->t;
    const Tree& ts = src_tree->t;
    if (to.nn() >= ((int64_t)1 << 31) || ts.nn() >= ((int64_t)1 << 31)) {
      set_error("bf_nearandfar_gpu: trees above 2^31 nodes are not supported");
      return BF_ENOTSUP;
    }
    BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
    cudaStream_t st = nullptr;
    DevBufs mem;
    auto upload_tree = [&](const Tree& t, TreeDev& d) -> int {
      double *c, *hh;
      int32_t *fc, *nc;
      BF_TRY(mem.get(&c, t.center.size(), "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&hh, t.half.size(), "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&fc, t.first_child.size(), "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&nc, t.n_child.size(), "bf_nearandfar_gpu"));
      BF_TRY_CUDA(cudaMemcpy(c, t.center.data(), t.center.size() * sizeof(double),
                             cudaMemcpyHostToDevice));
      BF_TRY_CUDA(cudaMemcpy(hh, t.half.data(), t.half.size() * sizeof(double),
                             cudaMemcpyHostToDevice));
      BF_TRY_CUDA(cudaMemcpy(fc, t.first_child.data(), t.first_child.size() * sizeof(int32_t),
                             cudaMemcpyHostToDevice));
      BF_TRY_CUDA(cudaMemcpy(nc, t.n_child.data(), t.n_child.size() * sizeof(int32_t),
                             cudaMemcpyHostToDevice));
      d = TreeDev{c, hh, fc, nc};
      return BF_OK;
    };
    TreeDev dto{}, dts{};
    BF_TRY(upload_tree(to, dto));
    BF_TRY(upload_tree(ts, dts));
    const double sqrt3 = std::sqrt(3.0);
    const int32_t h0 = std::min(to.depth() + 1, ts.depth() + 1);
    // frontier (level 0: the root pair)
    int32_t *po, *ps;
    PairKey* pk;
    BF_TRY(mem.get(&po, 1, "bf_nearandfar_gpu"));
    BF_TRY(mem.get(&ps, 1, "bf_nearandfar_gpu"));
    BF_TRY(mem.get(&pk, 1, "bf_nearandfar_gpu"));
    BF_TRY_CUDA(cudaMemset(po, 0, sizeof(int32_t)));
    BF_TRY_CUDA(cudaMemset(ps, 0, sizeof(int32_t)));
    BF_TRY_CUDA(cudaMemset(pk, 0, sizeof(PairKey)));
    int64_t nfront = 1;
    struct LevelOut {
      int32_t *fo, *fs, *no, *ns;
      PairKey *fk, *nk;
      int64_t nf, nn;
    };
    std::vector<LevelOut> levels;
    int64_t* d_total;
    BF_TRY(mem.get(&d_total, 1, "bf_nearandfar_gpu"));
    constexpr int MAX_LEVELS = 21;  // 6-bit digits in a 128-bit key
    for (int L = 0; nfront > 0; ++L) {
      if (L >= MAX_LEVELS) {
        set_error("bf_nearandfar_gpu: traversal deeper than %d levels; use bf_nearandfar",
                  MAX_LEVELS);
        return BF_ENOTSUP;
      }
      int32_t *isf, *isn, *nk;
      int64_t *fpos, *npos, *kpos, *sums;
      const int64_t ntile = (nfront + SCAN_TILE - 1) / SCAN_TILE;
      BF_TRY(mem.get(&isf, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&isn, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&nk, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&fpos, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&npos, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&kpos, nfront, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&sums, ntile, "bf_nearandfar_gpu"));
      classify_kernel<<<grid_of(nfront), 256, 0, st>>>(po, ps, nfront, dto, dts, h0 - L, alpha,
                                                       sqrt3, minbflvl, leafcomp, leafimbalance,
                                                       unbalancedints ? 1 : 0, isf, isn, nk);
      BF_TRY_CUDA(cudaGetLastError());
      int64_t nf = 0, nn = 0, nkid = 0;
      BF_TRY(exclusive_scan(isf, nfront, fpos, sums, d_total, &nf, st));
      BF_TRY(exclusive_scan(isn, nfront, npos, sums, d_total, &nn, st));
      BF_TRY(exclusive_scan(nk, nfront, kpos, sums, d_total, &nkid, st));
      LevelOut lo{};
      lo.nf = nf;
      lo.nn = nn;
      BF_TRY(mem.get(&lo.fo, nf, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&lo.fs, nf, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&lo.fk, nf, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&lo.no, nn, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&lo.ns, nn, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&lo.nk, nn, "bf_nearandfar_gpu"));
      int32_t *qo, *qs;
      PairKey* qk;
      BF_TRY(mem.get(&qo, nkid, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&qs, nkid, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&qk, nkid, "bf_nearandfar_gpu"));
      expand_kernel<<<grid_of(nfront), 256, 0, st>>>(po, ps, pk, nfront, L, dto, dts,
                                                     unbalancedints ? 1 : 0, sqrt3, isf, isn,
                                                     nk, fpos, npos, kpos, lo.fo, lo.fs, lo.fk,
                                                     lo.no, lo.ns, lo.nk, qo, qs, qk);
      BF_TRY_CUDA(cudaGetLastError());
      levels.push_back(lo);
      po = qo;
      ps = qs;
      pk = qk;
      nfront = nkid;
    }
    int64_t tf = 0, tn = 0;
    for (const auto& l : levels) {
      tf += l.nf;
      tn += l.nn;
    }
    if (n_far) *n_far = tf;
    if (n_near) *n_near = tn;
    if (far_capacity > 0 && tf > far_capacity) {
      set_error("bf_nearandfar_gpu: capacity %lld < %lld far pairs", (long long)far_capacity,
                (long long)tf);
      return BF_EINVAL;
    }
    if (near_capacity > 0 && tn > near_capacity) {
      set_error("bf_nearandfar_gpu: capacity %lld < %lld near pairs", (long long)near_capacity,
                (long long)tn);
      return BF_EINVAL;
    }
    // depth-first order: place every output by its key rank over all levels
    const int nl = (int)levels.size();
    for (int which = 0; which < 2; ++which) {
      int64_t* ho = which == 0 ? far_obs : near_obs;
      int64_t* hs = which == 0 ? far_src : near_src;
      const int64_t cap = which == 0 ? far_capacity : near_capacity;
      const int64_t tot = which == 0 ? tf : tn;
      if (!ho || !hs || cap <= 0 || tot == 0) continue;
      std::vector<LevelKeys> lk(nl);
      for (int L = 0; L < nl; ++L)
        lk[L] = LevelKeys{which == 0 ? levels[L].fk : levels[L].nk,
                          which == 0 ? levels[L].nf : levels[L].nn, 0};
      LevelKeys* d_lk;
      int64_t *d_o, *d_s;
      BF_TRY(mem.get(&d_lk, nl, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&d_o, tot, "bf_nearandfar_gpu"));
      BF_TRY(mem.get(&d_s, tot, "bf_nearandfar_gpu"));
      BF_TRY_CUDA(cudaMemcpy(d_lk, lk.data(), nl * sizeof(LevelKeys), cudaMemcpyHostToDevice));
      for (int L = 0; L < nl; ++L) {
        const int64_t n = lk[L].n;
        if (n == 0) continue;
        place_kernel<<<grid_of(n), 256, 0, st>>>(
            which == 0 ? levels[L].fo : levels[L].no, which == 0 ? levels[L].fs : levels[L].ns,
            lk[L].k, n, L, d_lk, nl, d_o, d_s, tot);
      }
      BF_TRY_CUDA(cudaGetLastError());
      BF_TRY_CUDA(cudaMemcpy(ho, d_o, (size_t)tot * sizeof(int64_t), cudaMemcpyDeviceToHost));
      BF_TRY_CUDA(cudaMemcpy(hs, d_s, (size_t)tot * sizeof(int64_t), cudaMemcpyDeviceToHost));
    }
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_nearandfar_gpu: host allocation failed");
    return BF_ENOMEM;
  }
}
