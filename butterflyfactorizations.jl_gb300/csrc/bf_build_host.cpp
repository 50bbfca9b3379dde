// Host orchestration of the batched GPU construction (bf_build).
//
// Restates assemble_BF (src/ButterflyFactorization/bfassembly.jl:48-200) for
// all far pairs of an operator at once: the Q stage, every R level and the P
// stage are each one batch of compressions (or dense kernel blocks) executed by
// the kernels of bf_build.cu.  The host keeps only integer bookkeeping: the
// padded level lists, the skeleton map K (bfassembly.jl:76-77) and the block
// keys; matrices never leave the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <unordered_map>
#include <parallel/algorithm>

#include "bf_build.h"
#include "bf_surrogate.h"

namespace bfg {
namespace {

uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// task_key(seed, bf, stage, obs_node, src_node) -- same chain as the oracle
uint64_t task_key(uint64_t seed, int64_t bf, int64_t stage, int64_t o, int64_t s) {
  uint64_t h = mix64(seed);
  h = mix64(h ^ (uint64_t)bf);
  h = mix64(h ^ (uint64_t)stage);
  h = mix64(h ^ (uint64_t)o);
  h = mix64(h ^ (uint64_t)s);
  return h;
}

struct KKey {
  int32_t bf;
  int64_t s, o;
  bool operator==(const KKey& k) const { return bf == k.bf && s == k.s && o == k.o; }
};
struct SkelRef {
  int64_t off = 0;
  int32_t len = 0;
  int64_t slot = -1;  // level slot holding this skeleton's values (pack_plan wiring)
};

// the skeleton map K (bfassembly.jl:76-77): (bf, source node, observer node) ->
// skeleton.  Sharded by far pair, so that a round of updates is applied by
// one thread per shard, each in update order (lookups see the same values as
// with serial updates).
struct KMap {
  static constexpr int NS = 256;
  FlatMap<SkelRef> m[NS];
  static int shard(int32_t bf) { return (int)(((uint32_t)bf * 2654435761u) >> 24); }
  static uint64_t lo(const KKey& k) { return ((uint64_t)k.s << 32) | (uint64_t)(uint32_t)k.o; }
  const SkelRef& at(const KKey& k) const {
    return m[shard(k.bf)].at((uint64_t)(uint32_t)k.bf, lo(k));
  }
  void set_all(const std::vector<std::pair<KKey, SkelRef>>& upd) {
    const int64_t n = (int64_t)upd.size();
    std::vector<int64_t> beg(NS + 1, 0), idx(n);
    for (int64_t i = 0; i < n; ++i) ++beg[shard(upd[i].first.bf) + 1];
    for (int s = 0; s < NS; ++s) beg[s + 1] += beg[s];
    std::vector<int64_t> pos(beg.begin(), beg.end() - 1);
    for (int64_t i = 0; i < n; ++i) idx[pos[shard(upd[i].first.bf)]++] = i;
#pragma omp parallel for schedule(dynamic, 1)
    for (int s = 0; s < NS; ++s) {
      FlatMap<SkelRef>& ms = m[s];
      ms.reserve(ms.count + (size_t)(beg[s + 1] - beg[s]));
      for (int64_t j = beg[s]; j < beg[s + 1]; ++j) {
        const auto& u = upd[idx[j]];
        ms.put((uint64_t)(uint32_t)u.first.bf, lo(u.first), u.second);
      }
    }
  }
};

struct BFState {
  int64_t no, ns;
  std::vector<std::vector<int64_t>> tS, tO;
  int32_t LS, LO, L;
  double eps;
  int32_t n_est;
};

struct HTask {
  int32_t bf, stage;
  int64_t obs_node, src_node;
  int64_t obs_begin;
  int32_t n_obs;
  int64_t cols_off;
  int32_t n_cols;
  uint64_t key;
  double eps;
  int32_t rows0, rows, retries, rank;
  int32_t n_est;            // oversampling-estimator sample count (the fallback)
  int8_t seeded, fell_back; // rows set by the surrogate; fell back to n_est
  int64_t t_off;
  SkelRef skel;
};

struct Item {
  int32_t kind;  // 0 = compression, 1 = identity
  int32_t bf;
  int64_t oo, so, oi, si;
  int64_t split_svert;  // >= 0: split T columns by children of this source node
  int64_t upd_s, upd_o;
  int64_t task;
  SkelRef copy;
};

template <typename T>
int dev_reserve(T*& p, int64_t& cap, int64_t need) {
  if (need <= cap) return BF_OK;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  int64_t n = std::max<int64_t>(need, 1024);
  n += n / 4;
  if (cudaMalloc(&p, (size_t)n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    set_error("build: cannot allocate %lld device entries", (long long)n);
    return BF_ENOMEM;
  }
  cap = n;
  return BF_OK;
}

class Builder {
 public:
  Builder(Context* ctx, const Tree& to, const Tree& ts, double k, double tol,
          const bf_build_opts& opts, Operator& op)
      : ctx_(ctx), to_(to), ts_(ts), k_(k), tol_(tol), opts_(opts), op_(op) {}
  ~Builder() {
    for (void* p : {(void*)d_obs_, (void*)d_src_, (void*)d_obs_perm_, (void*)d_colpool_,
                    (void*)d_ctask_, (void*)d_Z_, (void*)d_rowpool_, (void*)d_permpool_,
                    (void*)d_skel_, (void*)d_sw_, (void*)d_sfeat_, (void*)d_sout_,
                    (void*)d_ranks_, (void*)d_done_, (void*)d_ctask2_})
      if (p) cudaFree(p);
    for (cudaEvent_t e : ev_)
      if (e) cudaEventDestroy(e);
  }

  int run(const double* obs_xyz, int64_t n_obs, const double* src_xyz, int64_t n_src,
          const int64_t* far_obs, const int64_t* far_src, int64_t n_far);

 private:
  // device time of the compression launches (sampling, QR, triangular solve),
  // reported with the phase times when BFGPU_TIMING is set
  cudaEvent_t ev_[2] = {nullptr, nullptr};
  double comp_gpu_s_ = 0;
  int64_t comp_chunks_ = 0;
  void gpu_span_begin() {
    if (ev_[0]) cudaEventRecord(ev_[0], st_);
  }
  void gpu_span_end() {  // after the stream synchronise that follows the span
    if (!ev_[0]) return;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, ev_[0], ev_[1]) == cudaSuccess) comp_gpu_s_ += ms * 1e-3;
  }
  int ensure_raw(int64_t need);
  int run_compressions(std::vector<HTask>& tasks, const std::vector<int32_t>& colpool);
  int run_dense(std::vector<HTask>& tasks, const std::vector<int32_t>& colpool);
  void add_values(std::vector<int32_t>& pool, const Tree& t, int64_t node) {
    const int64_t* v = t.vals(node);
    for (int64_t i = 0; i < t.nvals(node); ++i) pool.push_back((int32_t)v[i]);
  }
  void add_skel(std::vector<int32_t>& pool, const SkelRef& r) {
    pool.insert(pool.end(), skel_.begin() + r.off, skel_.begin() + r.off + r.len);
  }
  HTask make_task(int32_t f, int32_t stage, int64_t obs_node, int64_t src_node, int64_t cols_off,
                  int32_t n_cols) {
    const BFState& st = bfs_[f];
    HTask t{};
    t.bf = f;
    t.stage = stage;
    t.obs_node = obs_node;
    t.src_node = src_node;
    t.obs_begin = to_.begin[obs_node];
    t.n_obs = (int32_t)to_.nvals(obs_node);
    t.cols_off = cols_off;
    t.n_cols = n_cols;
    t.key = task_key(opts_.seed, f, stage, obs_node, src_node);
    t.eps = st.eps;
    const int32_t est = opts_.estimator == BF_EST_GEOMETRIC ? geometric_rank(obs_node, src_node, st.eps)
                                                            : st.n_est;
    t.n_est = std::min(std::max(est, opts_.min_samples), t.n_obs);
    t.rows0 = t.rows = t.n_est;
    t.seeded = t.fell_back = 0;
    t.t_off = -1;
    return t;
  }
  // GeometricRankEstimator (rankestimation.jl:13-25 with the tree method of
  // ext/BFH2Trees/h2rankest.jl:8-38): x1 = (k a_s a_o / max(d, 1e-4))^2 from the
  // node radii and the center distance, x2 = log(1/eps),
  // max(ceil(C x1 + Ceps x2), Rmin)
  int32_t geometric_rank(int64_t obs_node, int64_t src_node, double eps) const {
    double d2 = 0;
    for (int a = 0; a < 3; ++a) {
      const double d = ts_.center[3 * src_node + a] - to_.center[3 * obs_node + a];
      d2 += d * d;
    }
    const double d = std::max(std::sqrt(d2), 1e-4);
    const double g = k_ * (ts_.radius(src_node) * to_.radius(obs_node)) / d;
    const double r = std::ceil(opts_.geo_c * (g * g) + opts_.geo_ceps * std::log(1.0 / eps));
    const double cap = 1e9;  // keeps the count in int range; rows are capped by n_obs anyway
    return std::max((int32_t)std::min(r, cap), opts_.geo_rmin);
  }

  // surrogate-seeded sample counts for one round of compressions (GPU inference)
  int seed_rows(std::vector<HTask>& tasks);

  Context* ctx_;
  const Tree& to_;
  const Tree& ts_;
  double k_, tol_;
  bf_build_opts opts_;
  Operator& op_;
  cudaStream_t st_ = nullptr;
  std::vector<BFState> bfs_;
  KMap K_;
  std::vector<int32_t> skel_;  // host skeleton pool (point ids)
  // device
  double* d_obs_ = nullptr;
  double* d_src_ = nullptr;
  int32_t* d_obs_perm_ = nullptr;
  int32_t* d_colpool_ = nullptr;
  int64_t colpool_cap_ = 0;
  CTask* d_ctask_ = nullptr;
  int64_t ctask_cap_ = 0;
  float2* d_Z_ = nullptr;
  int64_t z_cap_ = 0;
  int32_t* d_rowpool_ = nullptr;
  int64_t row_cap_ = 0;
  int32_t* d_permpool_ = nullptr;
  int64_t perm_cap_ = 0;
  int32_t* d_skel_ = nullptr;
  int64_t skel_cap_ = 0;
  int32_t* d_ranks_ = nullptr;  // ranks of one round
  int64_t ranks_cap_ = 0;
  CDone* d_done_ = nullptr;     // finished compressions of one round
  int64_t done_cap_ = 0;
  CTask* d_ctask2_ = nullptr;   // their records, gathered for the solve
  int64_t ctask2_cap_ = 0;
  float2* d_raw_ = nullptr;
  int64_t raw_cap_ = 0, raw_used_ = 0;
  const Surrogate* surrogate_ = nullptr;
  Surrogate sur_;
  float* d_sw_ = nullptr;     // surrogate weights on the device
  float* d_sfeat_ = nullptr;  // features / predictions of one round
  float* d_sout_ = nullptr;
  int64_t sfeat_cap_ = 0, n_fallback_ = 0;
  // stats
  int64_t n_comp_ = 0, n_retry_ = 0, n_entries_ = 0;
};

int Builder::ensure_raw(int64_t need) {
  if (need <= raw_cap_) return BF_OK;
  int64_t n = std::max<int64_t>(need, raw_cap_ * 3 / 2);
  n = std::max<int64_t>(n, 1 << 20);
  float2* p = nullptr;
  if (cudaMalloc(&p, (size_t)n * sizeof(float2)) != cudaSuccess) {
    cudaGetLastError();
    set_error("build: cannot grow factor store to %lld entries", (long long)n);
    return BF_ENOMEM;
  }
  if (d_raw_) {
    BF_TRY_CUDA(cudaMemcpyAsync(p, d_raw_, (size_t)raw_used_ * sizeof(float2),
                                cudaMemcpyDeviceToDevice, st_));
    BF_TRY_CUDA(cudaStreamSynchronize(st_));
    cudaFree(d_raw_);
  }
  d_raw_ = p;
  raw_cap_ = n;
  return BF_OK;
}

// PartialQR (compressors.jl:81-165) for a batch of compressions: sample,
// pivoted QR, adaptive doubling of the sample while r > floor(0.8 rows), then
// the interpolation matrix and the skeleton.
// adds the wall time of its scope to a statistics field
struct ScopeTimer {
  double& acc;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit ScopeTimer(double& a) : acc(a) {}
  ~ScopeTimer() {
    acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

int Builder::run_compressions(std::vector<HTask>& tasks, const std::vector<int32_t>& colpool) {
  ScopeTimer tm(op_.stats.build_compress_seconds);
  if (tasks.empty()) return BF_OK;
  if (!ev_[0] && std::getenv("BFGPU_TIMING")) {
    BF_TRY_CUDA(cudaEventCreate(&ev_[0]));
    BF_TRY_CUDA(cudaEventCreate(&ev_[1]));
  }
  BF_TRY(seed_rows(tasks));
  BF_TRY(dev_reserve(d_colpool_, colpool_cap_, (int64_t)colpool.size()));
  BF_TRY_CUDA(cudaMemcpyAsync(d_colpool_, colpool.data(), colpool.size() * sizeof(int32_t),
                              cudaMemcpyHostToDevice, st_));
  // empty compressions (compressors.jl:93-96)
  std::vector<int64_t> work;
  for (int64_t i = 0; i < (int64_t)tasks.size(); ++i) {
    HTask& t = tasks[i];
    ++n_comp_;
    if (t.n_obs == 0 || t.n_cols == 0) {
      t.rank = 0;
      t.t_off = raw_used_;
      t.skel = SkelRef{(int64_t)skel_.size(), 0};
      continue;
    }
    work.push_back(i);
  }
  const int64_t ZCAP = (int64_t)96 << 20;  // float2 entries per chunk (768 MB)
  size_t pos = 0;
  std::vector<CTask> ct;
  std::vector<int64_t> pending, next, done;
  std::vector<int32_t> hskel, hranks;
  while (pos < work.size()) {
    pending.clear();
    int64_t zsum = 0;
    while (pos < work.size()) {
      const HTask& t = tasks[work[pos]];
      int64_t z = (int64_t)t.rows * t.n_cols;
      if (!pending.empty() && zsum + z > ZCAP) break;
      zsum += z;
      pending.push_back(work[pos++]);
    }
    while (!pending.empty()) {
      // larger shared-memory needs last, so each QR launch covers one size
      // bucket: sizes ascending, ties in pending order (a stable sort, done as
      // a parallel sort of (size, position) keys)
      const int64_t np = (int64_t)pending.size();
      {
        std::vector<std::pair<int64_t, int64_t>> key(np);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < np; ++q) {
          const HTask& t = tasks[pending[q]];
          key[q] = {(int64_t)t.rows * t.n_cols, q};
        }
        __gnu_parallel::sort(key.begin(), key.end());
        std::vector<int64_t> sorted(np);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < np; ++q) sorted[q] = pending[key[q].second];
        pending.swap(sorted);
      }
      // offsets of every compression's sample, rows and column permutation
      // (sizes gathered in parallel, serial prefix sums), then the records
      std::vector<int64_t> zoff(np + 1, 0), roff(np + 1, 0), poff(np + 1, 0);
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < np; ++q) {
        const HTask& t = tasks[pending[q]];
        zoff[q + 1] = (int64_t)t.rows * t.n_cols;
        roff[q + 1] = t.rows;
        poff[q + 1] = t.n_cols;
      }
      for (int64_t q = 0; q < np; ++q) {
        zoff[q + 1] += zoff[q];
        roff[q + 1] += roff[q];
        poff[q + 1] += poff[q];
      }
      const int64_t zo = zoff[np], ro = roff[np], po = poff[np];
      n_entries_ += zo;
      ct.resize(np);
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < np; ++q) {
        const HTask& t = tasks[pending[q]];
        CTask c{};
        c.z_off = zoff[q];
        c.rows_off = roff[q];
        c.cols_off = t.cols_off;
        c.obs_begin = t.obs_begin;
        c.perm_off = poff[q];
        c.t_off = -1;
        c.skel_off = 0;
        c.key = t.key;
        c.eps = t.eps;
        c.n_obs = t.n_obs;
        c.n_rows = t.rows;
        c.n_cols = t.n_cols;
        c.rank = 0;
        ct[q] = c;
      }
      BF_TRY(dev_reserve(d_ctask_, ctask_cap_, np));
      BF_TRY(dev_reserve(d_Z_, z_cap_, zo));
      BF_TRY(dev_reserve(d_rowpool_, row_cap_, ro));
      BF_TRY(dev_reserve(d_permpool_, perm_cap_, po));
      BF_TRY_CUDA(cudaMemcpyAsync(d_ctask_, ct.data(), np * sizeof(CTask), cudaMemcpyHostToDevice,
                                  st_));
      gpu_span_begin();
      BF_TRY(launch_rows(d_ctask_, (int)np, d_obs_perm_, d_rowpool_, st_));
      BF_TRY(launch_eval(d_ctask_, (int)np, d_obs_, d_src_, d_rowpool_, d_colpool_, d_Z_, k_, 0,
                         st_));
      // QR launches by shared-memory bucket
      int64_t q0 = 0;
      while (q0 < np) {
        size_t need = qr_smem_bytes(ct[q0].n_rows, ct[q0].n_cols, true);
        bool fits = need <= (size_t)QR_MAX_SMEM;
        size_t cap = fits ? std::min<size_t>(QR_MAX_SMEM, std::max<size_t>(need * 2, 16384)) : 0;
        int64_t q1 = q0;
        size_t smax = 0;
        while (q1 < np) {
          size_t s = qr_smem_bytes(ct[q1].n_rows, ct[q1].n_cols, fits);
          bool f1 = qr_smem_bytes(ct[q1].n_rows, ct[q1].n_cols, true) <= (size_t)QR_MAX_SMEM;
          if (f1 != fits || (fits && s > cap)) break;
          smax = std::max(smax, s);
          ++q1;
        }
        if (!fits) smax = std::max(smax, qr_smem_bytes(0, 0, false));
        BF_TRY(launch_qr(d_ctask_ + q0, (int)(q1 - q0), d_Z_, d_permpool_, fits, smax, st_));
        q0 = q1;
      }
      // only the ranks come back (the records stay on the device)
      BF_TRY(dev_reserve(d_ranks_, ranks_cap_, np));
      BF_TRY(launch_ranks(d_ctask_, (int)np, d_ranks_, st_));
      if (ev_[1]) cudaEventRecord(ev_[1], st_);
      hranks.resize(np);
      BF_TRY_CUDA(cudaMemcpyAsync(hranks.data(), d_ranks_, np * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, st_));
      BF_TRY_CUDA(cudaStreamSynchronize(st_));
      gpu_span_end();
      ++comp_chunks_;
      // adaptive decisions (compressors.jl:134-151)
      next.clear();
      done.clear();
      std::vector<uint8_t> retry(np, 0);
      int64_t n_fb = 0, n_rt = 0;
#pragma omp parallel for schedule(static) reduction(+ : n_fb, n_rt)
      for (int64_t q = 0; q < np; ++q) {
        HTask& t = tasks[pending[q]];
        t.rank = hranks[q];
        if (opts_.adaptive && t.rank > (int32_t)std::floor(0.8 * t.rows) && t.rows < t.n_obs) {
          int32_t nr = t.rows * 2;
          if (t.seeded && !t.fell_back) {
            // the surrogate under-predicted: fall back to the oversampling
            // estimator's count (or the doubled sample, if larger)
            nr = std::max(nr, t.n_est);
            t.fell_back = 1;
            ++n_fb;
          }
          t.rows = std::min(nr, t.n_obs);
          t.retries++;
          ++n_rt;
          retry[q] = 1;
        }
      }
      n_fallback_ += n_fb;
      n_retry_ += n_rt;
      for (int64_t q = 0; q < np; ++q) {
        if (retry[q])
          next.push_back(pending[q]);
        else
          done.push_back(q);
      }
      if (!done.empty()) {
        // factor-store and skeleton offsets of the finished compressions, in
        // their order (sizes in parallel, serial prefix sums)
        const int64_t nd = (int64_t)done.size();
        std::vector<int64_t> toff(nd + 1, 0), soff(nd + 1, 0);
        int max_rank = 0;
#pragma omp parallel for schedule(static) reduction(max : max_rank)
        for (int64_t d = 0; d < nd; ++d) {
          const HTask& t = tasks[pending[done[d]]];
          toff[d + 1] = (int64_t)t.rank * t.n_cols;
          soff[d + 1] = t.rank;
          max_rank = std::max(max_rank, t.rank);
        }
        for (int64_t d = 0; d < nd; ++d) {
          toff[d + 1] += toff[d];
          soff[d + 1] += soff[d];
        }
        const int64_t tsum = toff[nd], ssum = soff[nd];
        BF_TRY(ensure_raw(raw_used_ + tsum));
        BF_TRY(dev_reserve(d_skel_, skel_cap_, std::max<int64_t>(ssum, 1)));
        std::vector<CDone> hdone(nd);
        const int64_t raw0 = raw_used_, skel0 = (int64_t)skel_.size();
#pragma omp parallel for schedule(static)
        for (int64_t d = 0; d < nd; ++d) {
          const int64_t q = done[d];
          HTask& t = tasks[pending[q]];
          t.t_off = raw0 + toff[d];
          t.skel = SkelRef{skel0 + soff[d], t.rank};
          hdone[d] = CDone{q, raw0 + toff[d], soff[d]};
        }
        raw_used_ = raw0 + tsum;
        // the finished records are gathered on the device into a second
        // buffer with their output offsets (their sampled blocks stay in place)
        BF_TRY(dev_reserve(d_done_, done_cap_, nd));
        BF_TRY(dev_reserve(d_ctask2_, ctask2_cap_, nd));
        BF_TRY_CUDA(cudaMemcpyAsync(d_done_, hdone.data(), nd * sizeof(CDone),
                                    cudaMemcpyHostToDevice, st_));
        gpu_span_begin();
        BF_TRY(launch_compact_done(d_ctask_, d_done_, (int)nd, d_ctask2_, st_));
        BF_TRY(launch_tsolve(d_ctask2_, (int)nd, d_Z_, d_permpool_, d_colpool_, d_raw_, d_skel_,
                             max_rank, st_));
        if (ev_[1]) cudaEventRecord(ev_[1], st_);
        hskel.resize(ssum);
        if (ssum > 0)
          BF_TRY_CUDA(cudaMemcpyAsync(hskel.data(), d_skel_, ssum * sizeof(int32_t),
                                      cudaMemcpyDeviceToHost, st_));
        BF_TRY_CUDA(cudaStreamSynchronize(st_));
        gpu_span_end();
        skel_.insert(skel_.end(), hskel.begin(), hskel.end());
      }
      pending.swap(next);
    }
  }
  return BF_OK;
}

// Dense kernel blocks K(values(Oleaf), skeleton) for the P stage (bfassembly.jl:186-197).
int Builder::run_dense(std::vector<HTask>& tasks, const std::vector<int32_t>& colpool) {
  ScopeTimer tm(op_.stats.build_compress_seconds);
  if (tasks.empty()) return BF_OK;
  BF_TRY(dev_reserve(d_colpool_, colpool_cap_, (int64_t)colpool.size()));
  BF_TRY_CUDA(cudaMemcpyAsync(d_colpool_, colpool.data(), colpool.size() * sizeof(int32_t),
                              cudaMemcpyHostToDevice, st_));
  int64_t tot = 0;
  for (auto& t : tasks) tot += (int64_t)t.n_obs * t.n_cols;
  BF_TRY(ensure_raw(raw_used_ + tot));
  std::vector<CTask> ct(tasks.size());
  for (size_t i = 0; i < tasks.size(); ++i) {
    HTask& t = tasks[i];
    CTask& c = ct[i];
    c = CTask{};
    c.rows_off = t.obs_begin;  // rows = values(Oleaf), a slice of the observer permutation
    c.cols_off = t.cols_off;
    c.n_rows = t.n_obs;
    c.n_cols = t.n_cols;
    c.t_off = raw_used_;
    t.t_off = raw_used_;
    raw_used_ += (int64_t)t.n_obs * t.n_cols;
    n_entries_ += (int64_t)t.n_obs * t.n_cols;
  }
  const int64_t CH = 1 << 20;
  for (int64_t b = 0; b < (int64_t)ct.size(); b += CH) {
    int64_t n = std::min<int64_t>(CH, (int64_t)ct.size() - b);
    BF_TRY(dev_reserve(d_ctask_, ctask_cap_, n));
    BF_TRY_CUDA(cudaMemcpyAsync(d_ctask_, ct.data() + b, n * sizeof(CTask),
                                cudaMemcpyHostToDevice, st_));
    BF_TRY(launch_eval(d_ctask_, (int)n, d_obs_, d_src_, d_obs_perm_, d_colpool_, d_raw_, k_, 1,
                       st_));
    BF_TRY_CUDA(cudaStreamSynchronize(st_));
  }
  return BF_OK;
}

// Surrogate-seeded sample counts for one round: features of every task (host),
// one batched inference launch, rows = ceil(exp(pred + margin) / 0.8) + 2 so
// that the predicted rank stays under the 0.8 x rows retry line of
// compressors.jl:134; at least min_samples, at most the observer count.
int Builder::seed_rows(std::vector<HTask>& tasks) {
  if (!surrogate_ || tasks.empty()) return BF_OK;
  const int64_t n = (int64_t)tasks.size();
  std::vector<float> feat(4 * n), pred(n);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) {
    const HTask& t = tasks[q];
    surrogate_features(to_, ts_, k_, t.stage, t.obs_node, t.src_node, t.n_obs, t.n_cols,
                       &feat[4 * q]);
  }
  if (n > sfeat_cap_) {
    if (d_sfeat_) cudaFree(d_sfeat_);
    if (d_sout_) cudaFree(d_sout_);
    d_sfeat_ = d_sout_ = nullptr;
    sfeat_cap_ = 0;
    BF_TRY_CUDA(cudaMalloc(&d_sfeat_, (size_t)n * 4 * sizeof(float)));
    BF_TRY_CUDA(cudaMalloc(&d_sout_, (size_t)n * sizeof(float)));
    sfeat_cap_ = n;
  }
  BF_TRY_CUDA(cudaMemcpyAsync(d_sfeat_, feat.data(), feat.size() * sizeof(float),
                              cudaMemcpyHostToDevice, st_));
  BF_TRY(surrogate_predict_gpu(d_sw_, d_sfeat_, d_sout_, n, st_));
  BF_TRY_CUDA(cudaMemcpyAsync(pred.data(), d_sout_, (size_t)n * sizeof(float),
                              cudaMemcpyDeviceToHost, st_));
  BF_TRY_CUDA(cudaStreamSynchronize(st_));
  const double margin = opts_.surrogate_margin;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) {
    HTask& t = tasks[q];
    double r = std::exp(std::min((double)pred[q] + margin, 30.0));
    int64_t rows = (int64_t)std::ceil(r / 0.8) + 2;
    rows = std::max<int64_t>(rows, opts_.min_samples);
    rows = std::min<int64_t>(rows, t.n_obs);
    t.rows0 = t.rows = (int32_t)rows;
    t.seeded = 1;
  }
  return BF_OK;
}

int Builder::run(const double* obs_xyz, int64_t n_obs, const double* src_xyz, int64_t n_src,
                 const int64_t* far_obs, const int64_t* far_src, int64_t n_far) {
  BF_TRY_CUDA(cudaSetDevice(ctx_->device));
  if (!op_.stream) BF_TRY_CUDA(cudaStreamCreateWithFlags(&op_.stream, cudaStreamNonBlocking));
  st_ = op_.stream;
  if (opts_.rank_mode == 1) {
    if (!opts_.surrogate_weights || !sur_.load(opts_.surrogate_weights, opts_.surrogate_nweights)) {
      set_error("bf_build: rank_mode 1 needs valid surrogate weights");
      return BF_EINVAL;
    }
    surrogate_ = &sur_;
    BF_TRY_CUDA(cudaMalloc(&d_sw_, SUR_NW * sizeof(float)));
    BF_TRY_CUDA(cudaMemcpy(d_sw_, sur_.w.data(), SUR_NW * sizeof(float), cudaMemcpyHostToDevice));
  }
  // device copies of the geometry and of the observer permutation
  BF_TRY_CUDA(cudaMalloc(&d_obs_, (size_t)n_obs * 3 * sizeof(double)));
  BF_TRY_CUDA(cudaMalloc(&d_src_, (size_t)n_src * 3 * sizeof(double)));
  BF_TRY_CUDA(cudaMemcpy(d_obs_, obs_xyz, n_obs * 3 * sizeof(double), cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMemcpy(d_src_, src_xyz, n_src * 3 * sizeof(double), cudaMemcpyHostToDevice));
  {
    std::vector<int32_t> p(to_.perm.begin(), to_.perm.end());
    BF_TRY_CUDA(cudaMalloc(&d_obs_perm_, p.size() * sizeof(int32_t)));
    BF_TRY_CUDA(cudaMemcpy(d_obs_perm_, p.data(), p.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
  }
  // per-far-pair state (bfassembly.jl:64-74)
  bfs_.resize(n_far);
  int32_t Lmax = 1;
  for (int64_t f = 0; f < n_far; ++f) {
    BFState& s = bfs_[f];
    s.no = far_obs[f];
    s.ns = far_src[f];
    s.tS = traverse_and_pad(ts_, s.ns);
    s.tO = traverse_and_pad(to_, s.no);
    s.LS = (int32_t)s.tS.size();
    s.LO = (int32_t)s.tO.size();
    s.L = std::max(s.LS, s.LO);
    s.eps = tol_ / s.L;
    // ButterflyRankEstimator (rankestimation.jl:93-98), Rmin = 10
    s.n_est = std::max((int32_t)std::ceil(opts_.c_tau * std::log(1.0 / s.eps)), 10);
    Lmax = std::max(Lmax, s.L);
  }
  PhaseLog blog;
  blog.mark("build: setup + far-pair state");
  Logical& lg = op_.logical;
  lg.n_rows = to_.n_points;
  lg.n_cols = ts_.n_points;
  lg.n_bf = (int32_t)n_far;
  // slot ids follow the skeleton map: every new skeleton (or identity copy) of
  // a level gets a fresh slot, blocks read the slot of the skeleton they use
  std::vector<int64_t> slot_len;
  std::vector<BlockVec> stage_blocks;  // blocks of each stage, joined at the end
  auto make_block = [](int32_t bf, int32_t stage, int64_t oo, int64_t so, int64_t oi, int64_t si,
                       int32_t rows, int32_t cols, int8_t ident, int64_t raw_off, int32_t ld,
                       int64_t in_slot, int64_t out_slot) {
    LBlock b;
    b.in_slot = in_slot;
    b.out_slot = out_slot;
    b.bf = bf;
    b.stage = stage;
    b.oo = oo;
    b.so = so;
    b.oi = oi;
    b.si = si;
    b.rows = rows;
    b.cols = cols;
    b.ident = ident;
    b.raw_off = raw_off;
    b.raw_ld = std::max(ld, 1);
    return b;
  };
  auto rank_rec = [&](const HTask& t) {
    Operator::RankRec r;
    r.bf = t.bf;
    r.stage = t.stage;
    r.obs_node = t.obs_node;
    r.src_node = t.src_node;
    r.n_obs = t.n_obs;
    r.n_cols = t.n_cols;
    r.rows0 = t.rows0;
    r.rows = t.rows;
    r.retries = t.retries;
    r.rank = t.rank;
    r.a_obs = (float)to_.radius(t.obs_node);
    r.a_src = (float)ts_.radius(t.src_node);
    double d2 = 0;
    for (int a = 0; a < 3; ++a) {
      double d = to_.center[3 * t.obs_node + a] - ts_.center[3 * t.src_node + a];
      d2 += d * d;
    }
    r.dist = (float)std::sqrt(d2);
    r.k = (float)k_;
    surrogate_features(to_, ts_, k_, t.stage, t.obs_node, t.src_node, t.n_obs, t.n_cols, r.feat);
    return r;
  };

  // Host loops over the far pairs run in parallel over chunks of far pairs.
  // Each chunk fills its own buffers and the chunks are joined in far-pair
  // order, so tasks, pools, blocks and slot ids are exactly those of a serial
  // loop.  The skeleton map is only read inside the parallel loops; its updates
  // are applied serially after each round.
  const int64_t n_chunks = std::max<int64_t>(1, std::min<int64_t>(n_far, 4096));
  struct Part {
    std::vector<HTask> tasks;
    std::vector<int32_t> pool;
    std::vector<Item> items;
    std::vector<int64_t> in_slots;
  };
  // body(chunk, f_begin, f_end) on every chunk; a failed skeleton-map lookup in
  // any chunk is rethrown here (the caller turns it into BF_EINVAL)
  auto for_chunks = [&](auto&& body) {
    std::atomic<int> failed{0};
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < n_chunks; ++c) {
      try {
        body(c, n_far * c / n_chunks, n_far * (c + 1) / n_chunks);
      } catch (const std::bad_alloc&) {
        failed = 2;
      } catch (...) {
        failed = 1;
      }
    }
    if (failed == 2) throw std::bad_alloc();
    if (failed) throw std::out_of_range("skeleton map lookup");
  };
  // chunk parts -> one round: pool offsets and task indices shift by the
  // chunk's position
  auto join = [&](std::vector<Part>& parts, std::vector<HTask>& tasks, std::vector<int32_t>& pool,
                  std::vector<Item>* items, std::vector<int64_t>* in_slots) {
    const int64_t P = (int64_t)parts.size();
    std::vector<int64_t> tb(P + 1, 0), pb(P + 1, 0), ib(P + 1, 0);
    for (int64_t c = 0; c < P; ++c) {
      tb[c + 1] = tb[c] + (int64_t)parts[c].tasks.size();
      pb[c + 1] = pb[c] + (int64_t)parts[c].pool.size();
      ib[c + 1] = ib[c] + (int64_t)parts[c].items.size();
    }
    tasks.resize(tb[P]);
    pool.resize(pb[P]);
    if (items) items->resize(ib[P]);
    if (in_slots) in_slots->resize(tb[P]);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t c = 0; c < P; ++c) {
      Part& p = parts[c];
      for (size_t q = 0; q < p.tasks.size(); ++q) {
        tasks[tb[c] + q] = p.tasks[q];
        tasks[tb[c] + q].cols_off += pb[c];
      }
      std::copy(p.pool.begin(), p.pool.end(), pool.begin() + pb[c]);
      if (items)
        for (size_t q = 0; q < p.items.size(); ++q) {
          Item it = p.items[q];
          if (it.task >= 0) it.task += tb[c];
          (*items)[ib[c] + q] = it;
        }
      if (in_slots) std::copy(p.in_slots.begin(), p.in_slots.end(), in_slots->begin() + tb[c]);
      p = Part();
    }
  };
  // rank records of one round, in task order
  auto log_tasks = [&](const std::vector<HTask>& tasks) {
    const size_t base = op_.rank_log.size();
    op_.rank_log.resize(base + tasks.size());
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < (int64_t)tasks.size(); ++q) op_.rank_log[base + q] = rank_rec(tasks[q]);
  };

  // ---- Q stage (bfassembly.jl:82-102)
  {
    std::vector<Part> parts(n_chunks);
    for_chunks([&](int64_t c, int64_t f0, int64_t f1) {
      Part& p = parts[c];
      for (int64_t f = f0; f < f1; ++f) {
        const BFState& s = bfs_[f];
        for (int64_t Sleaf : s.tS.back()) {
          int64_t off = (int64_t)p.pool.size();
          add_values(p.pool, ts_, Sleaf);
          p.tasks.push_back(make_task((int32_t)f, 0, s.no, Sleaf, off, (int32_t)ts_.nvals(Sleaf)));
        }
      }
    });
    std::vector<HTask> tasks;
    std::vector<int32_t> pool;
    join(parts, tasks, pool, nullptr, nullptr);
    BF_TRY(run_compressions(tasks, pool));
    const int64_t nt = (int64_t)tasks.size();
    const int64_t sb = (int64_t)slot_len.size();
    slot_len.resize(sb + nt);
    BlockVec& blk = stage_blocks.emplace_back(nt);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nt; ++q) {
      HTask& t = tasks[q];
      t.skel.slot = sb + q;
      slot_len[sb + q] = t.rank;
      blk[q] = make_block(t.bf, 0, t.obs_node, t.src_node, t.obs_node, t.src_node, t.rank,
                          t.n_cols, 0, t.t_off, t.rank, -1, t.skel.slot);
    }
    {
      std::vector<std::pair<KKey, SkelRef>> upd(nt);
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < nt; ++q)
        upd[q] = {KKey{tasks[q].bf, tasks[q].src_node, tasks[q].obs_node}, tasks[q].skel};
      K_.set_all(upd);
    }
    log_tasks(tasks);
  }
  blog.mark("build: Q stage");
  // ---- R levels (bfassembly.jl:107-181)
  for (int32_t l = 1; l < Lmax; ++l) {
    std::vector<Part> parts(n_chunks);
    for_chunks([&](int64_t c, int64_t f0, int64_t f1) {
      Part& p = parts[c];
      std::vector<HTask>& tasks = p.tasks;
      std::vector<int32_t>& pool = p.pool;
      std::vector<Item>& items = p.items;
      auto comp_item = [&](int32_t f, int64_t obs_node, int64_t svert, int64_t cols_off,
                           int32_t ncols, int64_t oo, int64_t so, int64_t oi, int64_t si,
                           int64_t split, int64_t us, int64_t uo) {
        Item it{};
        it.kind = 0;
        it.bf = f;
        it.oo = oo;
        it.so = so;
        it.oi = oi;
        it.si = si;
        it.split_svert = split;
        it.upd_s = us;
        it.upd_o = uo;
        it.task = (int64_t)tasks.size();
        tasks.push_back(make_task(f, l, obs_node, svert, cols_off, ncols));
        items.push_back(it);
      };
      auto ident_item = [&](int32_t f, int64_t Overt, int64_t Svert) {
        Item it{};
        it.kind = 1;
        it.bf = f;
        it.oo = it.oi = Overt;
        it.so = it.si = Svert;
        it.split_svert = -1;
        it.upd_s = Svert;
        it.upd_o = Overt;
        it.task = -1;
        it.copy = K_.at(KKey{f, Svert, Overt});
        items.push_back(it);
      };
      // U(Svert, Overt): concatenated child skeletons (bfassembly.jl:206-230)
      auto push_U = [&](int32_t f, int64_t Svert, int64_t Overt, int64_t& off, int32_t& len) {
        off = (int64_t)pool.size();
        if (!ts_.isleaf(Svert)) {
          for (int32_t ch = 0; ch < ts_.n_child[Svert]; ++ch)
            add_skel(pool, K_.at(KKey{f, ts_.first_child[Svert] + ch, Overt}));
        } else {
          add_skel(pool, K_.at(KKey{f, Svert, Overt}));
        }
        len = (int32_t)((int64_t)pool.size() - off);
      };
      for (int64_t f = f0; f < f1; ++f) {
        const BFState& s = bfs_[f];
        if (l >= s.L) continue;
        const int32_t fi = (int32_t)f;
        bool sfz = l >= s.LS, ofz = l >= s.LO;
        if (!sfz && !ofz) {  // build_nonfrozen_R_blocks (bfassembly.jl:232-349)
          const auto& olv = s.tO[l - 1];
          const auto& slv = s.tS[s.LS - l - 1];
          for (int64_t Svert : slv)
            for (int64_t Overt : olv) {
              bool sleaf = ts_.isleaf(Svert);
              if (!to_.isleaf(Overt)) {
                int64_t off;
                int32_t len;
                push_U(fi, Svert, Overt, off, len);
                for (int32_t ch = 0; ch < to_.n_child[Overt]; ++ch) {
                  int64_t Oc = to_.first_child[Overt] + ch;
                  comp_item(fi, Oc, Svert, off, len, Oc, Svert, Overt, Svert, sleaf ? -1 : Svert,
                            Svert, Oc);
                }
              } else if (!sleaf) {
                int64_t off;
                int32_t len;
                push_U(fi, Svert, Overt, off, len);
                comp_item(fi, Overt, Svert, off, len, Overt, Svert, Overt, Svert, Svert, Svert,
                          Overt);
              } else {
                ident_item(fi, Overt, Svert);
              }
            }
        } else if (sfz && !ofz) {  // build_sourcefrozen_R_blocks (bfassembly.jl:351-412)
          int64_t Svert = s.ns;
          for (int64_t Overt : s.tO[l - 1]) {
            if (!to_.isleaf(Overt)) {
              SkelRef ref = K_.at(KKey{fi, Svert, Overt});
              int64_t off = (int64_t)pool.size();
              add_skel(pool, ref);
              for (int32_t ch = 0; ch < to_.n_child[Overt]; ++ch) {
                int64_t Oc = to_.first_child[Overt] + ch;
                comp_item(fi, Oc, Svert, off, ref.len, Oc, Svert, Overt, Svert, -1, Svert, Oc);
              }
            } else {
              ident_item(fi, Overt, Svert);
            }
          }
        } else {  // build_observerfrozen_R_blocks (bfassembly.jl:414-481)
          const auto& olv = s.tO[s.LO - 1];
          const auto& slv = s.tS[s.LS - l - 1];
          for (int64_t Svert : slv)
            for (int64_t Overt : olv) {
              if (!ts_.isleaf(Svert)) {
                int64_t off;
                int32_t len;
                push_U(fi, Svert, Overt, off, len);
                comp_item(fi, Overt, Svert, off, len, Overt, Svert, Overt, Svert, Svert, Svert,
                          Overt);
              } else {
                ident_item(fi, Overt, Svert);
              }
            }
        }
      }
    });
    std::vector<HTask> tasks;
    std::vector<int32_t> pool;
    std::vector<Item> items;
    join(parts, tasks, pool, &items, nullptr);
    blog.mark("build: R level host prep");
    BF_TRY(run_compressions(tasks, pool));
    blog.mark("build: R level compressions");
    // emit blocks, then apply the skeleton updates (deferred as in
    // bfassembly.jl:177-180).  Every item makes one new slot (slot id = base +
    // item index) and one block, or one block per child of a split source.
    const int64_t ni = (int64_t)items.size();
    std::vector<int64_t> boff(ni + 1, 0);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < ni; ++q) {
      const Item& it = items[q];
      boff[q + 1] = (it.kind == 0 && it.split_svert >= 0) ? ts_.n_child[it.split_svert] : 1;
    }
    for (int64_t q = 0; q < ni; ++q) boff[q + 1] += boff[q];
    const int64_t sb = (int64_t)slot_len.size();
    slot_len.resize(sb + ni);
    BlockVec& blk = stage_blocks.emplace_back(boff[ni]);
    std::vector<std::pair<KKey, SkelRef>> upd(ni);
    std::atomic<int> failed{0};
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < ni; ++q) {
      try {
        const Item& it = items[q];
        const int64_t slot = sb + q;
        int64_t b = boff[q];
        if (it.kind == 1) {
          SkelRef out = it.copy;
          out.slot = slot;
          slot_len[slot] = it.copy.len;
          blk[b] = make_block(it.bf, l, it.oo, it.so, it.oi, it.si, 0, 0, 1, 0, 1, it.copy.slot,
                              slot);
          upd[q] = {KKey{it.bf, it.upd_s, it.upd_o}, out};
        } else {
          HTask& t = tasks[it.task];
          t.skel.slot = slot;
          slot_len[slot] = t.rank;
          if (it.split_svert < 0) {
            blk[b] = make_block(it.bf, l, it.oo, it.so, it.oi, it.si, t.rank, t.n_cols, 0, t.t_off,
                                t.rank, K_.at(KKey{it.bf, it.si, it.oi}).slot, slot);
          } else {
            int64_t c0 = 0;
            const int64_t Sv = it.split_svert;
            for (int32_t ch = 0; ch < ts_.n_child[Sv]; ++ch) {
              const int64_t Sc = ts_.first_child[Sv] + ch;
              const SkelRef& in = K_.at(KKey{it.bf, Sc, it.oi});
              blk[b++] = make_block(it.bf, l, it.oo, it.so, it.oi, Sc, t.rank, in.len, 0,
                                    t.t_off + c0 * t.rank, t.rank, in.slot, slot);
              c0 += in.len;
            }
          }
          upd[q] = {KKey{it.bf, it.upd_s, it.upd_o}, t.skel};
        }
      } catch (...) {
        failed = 1;
      }
    }
    if (failed) throw std::out_of_range("skeleton map lookup");
    blog.mark("build: R level emit blocks");
    log_tasks(tasks);
    blog.mark("build: R level rank records");
    K_.set_all(upd);
    blog.mark("build: R level skeleton map");
  }
  // ---- P stage (bfassembly.jl:186-197)
  {
    std::vector<Part> parts(n_chunks);
    for_chunks([&](int64_t c, int64_t f0, int64_t f1) {
      Part& p = parts[c];
      for (int64_t f = f0; f < f1; ++f) {
        const BFState& s = bfs_[f];
        for (int64_t Oleaf : s.tO.back()) {
          SkelRef ref = K_.at(KKey{(int32_t)f, s.ns, Oleaf});
          p.in_slots.push_back(ref.slot);
          HTask t{};
          t.bf = (int32_t)f;
          t.obs_node = Oleaf;
          t.src_node = s.ns;
          t.obs_begin = to_.begin[Oleaf];
          t.n_obs = (int32_t)to_.nvals(Oleaf);
          t.cols_off = (int64_t)p.pool.size();
          t.n_cols = ref.len;
          add_skel(p.pool, ref);
          p.tasks.push_back(t);
        }
      }
    });
    std::vector<HTask> tasks;
    std::vector<int32_t> pool;
    std::vector<int64_t> in_slots;
    join(parts, tasks, pool, nullptr, &in_slots);
    BF_TRY(run_dense(tasks, pool));
    const int64_t nt = (int64_t)tasks.size();
    BlockVec& blk = stage_blocks.emplace_back(nt);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nt; ++q) {
      const HTask& t = tasks[q];
      blk[q] = make_block(t.bf, -1, t.obs_node, t.src_node, t.obs_node, t.src_node, t.n_obs,
                          t.n_cols, 0, t.t_off, t.n_obs, in_slots[q], -1);
    }
  }
  {  // the stages' blocks, in stage order, into one array (parallel copy)
    int64_t tot = 0;
    for (const BlockVec& v : stage_blocks) tot += (int64_t)v.size();
    lg.blocks.resize(tot);
    int64_t off = 0;
    for (BlockVec& v : stage_blocks) {
      const int64_t n = (int64_t)v.size();
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < n; ++q) lg.blocks[off + q] = v[q];
      off += n;
      BlockVec().swap(v);
    }
  }
  lg.slot_len = std::move(slot_len);
  blog.mark("build: P stage");
  if (blog.on)
    std::fprintf(stderr, "[bfgpu] %-32s %8.3f s (%lld chunks; inside the compression phases)\n",
                 "compress: device time", comp_gpu_s_, (long long)comp_chunks_);
  // node -> values maps for the packer
  auto fill_vm = [](ValuesMap& vm, const Tree& t) {
    vm.ptr.assign(t.nn() + 1, 0);
    for (int64_t i = 0; i < t.nn(); ++i) vm.ptr[i + 1] = vm.ptr[i] + t.nvals(i);
    vm.idx.resize(vm.ptr[t.nn()]);
    for (int64_t i = 0; i < t.nn(); ++i)
      std::memcpy(vm.idx.data() + vm.ptr[i], t.vals(i), t.nvals(i) * sizeof(int64_t));
  };
  fill_vm(lg.obs_vals, to_);
  fill_vm(lg.src_vals, ts_);
  op_.raw_is_double = 0;
  op_.d_raw = d_raw_;
  op_.raw_entries = raw_used_;
  d_raw_ = nullptr;
  op_.stats.compressions = n_comp_;
  op_.stats.retries = n_retry_;
  op_.stats.surrogate_fallbacks = n_fallback_;
  op_.stats.kernel_entries = n_entries_;
  return BF_OK;
}

}  // namespace

int build_operator(Context* ctx, const double* obs_xyz, int64_t n_obs, const double* src_xyz,
                   int64_t n_src, const Tree& to, const Tree& ts, const int64_t* far_obs,
                   const int64_t* far_src, int64_t n_far, double k, double tol,
                   const bf_build_opts& opts, Operator& op) {
  auto t0 = std::chrono::steady_clock::now();
  op.ctx = ctx;
  op.store_ff = opts.factor_storage == BF_STORE_FF ? 1 : 0;
  {
    Builder b(ctx, to, ts, k, tol, opts, op);
    BF_TRY(b.run(obs_xyz, n_obs, src_xyz, n_src, far_obs, far_src, n_far));
  }
  // the build's factors are complex FP32 values: packed as such (exact), or
  // widened to float-float entries when the caller asks for 16-byte storage
  auto tp = std::chrono::steady_clock::now();
  BF_TRY(pack_plan(op.logical, op.plan,
                   (op.raw_is_double || op.store_ff) ? (int)sizeof(float4) : (int)sizeof(float2)));
  auto tu = std::chrono::steady_clock::now();
  const double compress_s = op.stats.build_compress_seconds;
  const int64_t fallbacks = op.stats.surrogate_fallbacks;
  BF_TRY(upload_plan(op));  // rewrites the plan statistics
  BF_TRY_CUDA(cudaDeviceSynchronize());
  auto t1 = std::chrono::steady_clock::now();
  op.stats.build_seconds = std::chrono::duration<double>(t1 - t0).count();
  op.stats.build_compress_seconds = compress_s;
  op.stats.build_pack_seconds = std::chrono::duration<double>(tu - tp).count();
  op.stats.build_upload_seconds = std::chrono::duration<double>(t1 - tu).count();
  op.stats.surrogate_fallbacks = fallbacks;
  return BF_OK;
}

}  // namespace bfg

using namespace bfg;

extern "C" int bf_build(bf_ctx_t ctx, const double* obs_xyz, int64_t n_obs,
                        const double* src_xyz, int64_t n_src, bf_tree_t obs_tree,
                        bf_tree_t src_tree, const int64_t* far_obs, const int64_t* far_src,
                        int64_t n_far, double k, double tol, const bf_build_opts* opts,
                        bf_op_t* out) {
  try {
    if (!out) {
      set_error("bf_build: out is NULL");
      return BF_EINVAL;
    }
    *out = nullptr;
    if (!ctx || !obs_xyz || !src_xyz || !obs_tree || !src_tree || !far_obs || !far_src ||
        n_far <= 0 || !(k > 0) || !(tol > 0)) {
      set_error("bf_build: invalid argument");
      return BF_EINVAL;
    }
    if (obs_tree->t.n_points != n_obs || src_tree->t.n_points != n_src) {
      set_error("bf_build: tree point counts do not match the geometry");
      return BF_EINVAL;
    }
    if (n_obs >= ((int64_t)1 << 31) || n_src >= ((int64_t)1 << 31)) {
      set_error("bf_build: point sets above 2^31 are not supported");
      return BF_ENOTSUP;
    }
    for (int64_t f = 0; f < n_far; ++f)
      if (far_obs[f] < 0 || far_obs[f] >= obs_tree->t.nn() || far_src[f] < 0 ||
          far_src[f] >= src_tree->t.nn()) {
        set_error("bf_build: far pair %lld references an unknown node", (long long)f);
        return BF_EINVAL;
      }
    bf_build_opts o;
    if (opts)
      o = *opts;
    else
      bf_build_opts_default(&o);
    if (o.min_samples < 1) o.min_samples = 1;
    if (o.estimator != BF_EST_BUTTERFLY && o.estimator != BF_EST_GEOMETRIC) {
      set_error("bf_build: unknown rank estimator %d", o.estimator);
      return BF_EINVAL;
    }
    if (o.estimator == BF_EST_GEOMETRIC &&
        (!(o.geo_c >= 0.0) || !(o.geo_ceps >= 0.0) || !std::isfinite(o.geo_c) ||
         !std::isfinite(o.geo_ceps) || o.geo_rmin < 1)) {
      set_error("bf_build: geometric estimator needs finite C, Ceps >= 0 and Rmin >= 1");
      return BF_EINVAL;
    }
    auto* h = new bf_operator;
    int s = build_operator(&ctx->c, obs_xyz, n_obs, src_xyz, n_src, obs_tree->t, src_tree->t,
                           far_obs, far_src, n_far, k, tol, o, h->op);
    if (s != BF_OK) {
      delete h;
      return s;
    }
    *out = h;
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_build: host allocation failed");
    return BF_ENOMEM;
  } catch (const std::out_of_range&) {
    set_error("bf_build: internal skeleton lookup failed");
    return BF_EINVAL;
  } catch (...) {
    set_error("bf_build: unexpected internal error");
    return BF_EINVAL;
  }
}
