// Butterfly recompression on the GPU (bf_op_recompress).
//
// The reference's recompress_BF (src/Butterflyalgebra/algrecomp.jl:19-148)
// lowers the ranks of a butterfly's R levels to a tolerance: a right pass
// over the levels from the last to the second stacks the blocks that share a
// column space (obs_in, src_in), compresses the stack with a pivoted QR at
// rtol tau and moves the transfer matrix into the previous level's blocks
// with that row space; the left pass does the same on the adjoint.  Here
// every far block of an operator is recompressed at once, level by level:
//   - the stacks of all column groups of a level are compressed in one
//     launch of the build's batched pivoted-QR and interpolation kernels
//     (bf_build.cu, FP32 Householder with FP64 column norms and pivots);
//   - the stack's Q factor is formed as A[:, p[1:r]] R11^-1 (forward
//     substitution per row, the rows of block i giving its new entries) and
//     the transfer matrix is R[:, invperm(p)], as in the reference;
//   - the transfer matrices reach the neighbouring level through one batched
//     complex GEMM launch per level.
// Identity blocks (UniformScaling padding of uneven trees) pass one node
// through unchanged and are alone in their column and row groups; such a
// group is left as it is, which is exactly what the reference's pivoted QR of
// an identity gives (Q = I, T = I).  An identity neighbour of a compressed
// group becomes the transfer matrix itself (T * I).  The result is a new
// operator packed from the new blocks.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "bf_build.h"
#include "bf_dfloat.cuh"

namespace bfg {
namespace {

// one block copied from the packed factor array into the pool
struct alignas(16) GatherSeg {
  long long src, dst;
  int ld, rows, cols, pad;
};

// a block placed into a stack: rows [row0, row0 + rows) of a column-major
// stack with leading dimension ld; conj_t places A^H (cols x rows) instead
struct alignas(16) StackSeg {
  long long src, dst;
  int rows, cols, ld, row0, conj_t, pad;
};

// new member block: rows of the stack's Q = A[:, p[1:r]] R11^-1 belonging to
// one block (algrecomp.jl:89-97); by_rows: the block entered the stack as its
// adjoint (left pass) and leaves as Q_i^H (r x cols)
struct alignas(16) QSeg {
  long long src, dst, z, perm;
  int rows, cols, r, ldz, by_rows, pad0, pad1, pad2;
};

// C (m x n) = A (m x k) * B (k x n) (mode 0), A * B^H with B stored n x k
// (mode 1); an identity neighbour takes the transfer matrix itself: C = A
// (mode 2) or C = B^H with B stored n x m (mode 3)
struct alignas(16) GemmSeg {
  long long a, b, c;
  int m, n, k, mode;
};

template <typename FT>
__global__ void gather_kernel(const GatherSeg* __restrict__ segs, const FT* __restrict__ A,
                              float2* __restrict__ pool) {
  const GatherSeg g = segs[blockIdx.x];
  const long long tot = (long long)g.rows * g.cols;
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = (int)(e / g.rows), i = (int)(e - (long long)j * g.rows);
    pool[g.dst + e] = fac_c32(A[g.src + (long long)j * g.ld + i]);
  }
}

__global__ void stack_kernel(const StackSeg* __restrict__ segs, const float2* __restrict__ pool,
                             float2* __restrict__ Z) {
  const StackSeg s = segs[blockIdx.x];
  const long long tot = (long long)s.rows * s.cols;
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = (int)(e / s.rows), i = (int)(e - (long long)j * s.rows);
    const float2 v = pool[s.src + e];
    if (s.conj_t)  // block row i, column j -> stack row row0 + j, column i
      Z[s.dst + (long long)(s.row0 + j) + (long long)i * s.ld] = make_float2(v.x, -v.y);
    else
      Z[s.dst + (long long)(s.row0 + i) + (long long)j * s.ld] = v;
  }
}

// one thread per row of the block's slice of the stack: the row x (1 x n) of
// A_i (or of A_i^H) gives q = x[p[1:r]] R11^-1 by forward substitution
// (q_j = (x_j - sum_{l<j} q_l R_lj) / R_jj, R_jj real), sums in float-float;
// q is kept in the output and read back by the same thread
__global__ void qsolve_kernel(const QSeg* __restrict__ segs, const float2* __restrict__ pool_in,
                              const float2* __restrict__ Zg, const int32_t* __restrict__ permpool,
                              float2* __restrict__ pool_out) {
  const QSeg s = segs[blockIdx.x];
  const float2* __restrict__ R = Zg + s.z;
  const int32_t* __restrict__ p = permpool + s.perm;
  const int nrow = s.by_rows ? s.cols : s.rows;
  for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
    // output of (row i, column j): right pass rows x r; left pass r x cols, conjugated
    auto out_at = [&](int j) -> long long {
      return s.by_rows ? s.dst + j + (long long)i * s.r : s.dst + i + (long long)j * s.rows;
    };
    for (int j = 0; j < s.r; ++j) {
      float2 x = s.by_rows ? pool_in[s.src + p[j] + (long long)i * s.rows]
                           : pool_in[s.src + i + (long long)p[j] * s.rows];
      if (s.by_rows) x.y = -x.y;
      float4 acc = make_float4(x.x, 0.f, x.y, 0.f);
      for (int l = 0; l < j; ++l) {
        float2 q = pool_out[out_at(l)];
        if (s.by_rows) q.y = -q.y;
        const float2 c = R[l + (long long)j * s.ldz];
        cdf_mac(acc, make_float2(-c.x, -c.y), make_float4(q.x, 0.f, q.y, 0.f));
      }
      const float d = R[j + (long long)j * s.ldz].x;
      float2 q = make_float2((acc.x + acc.y) / d, (acc.z + acc.w) / d);
      if (s.by_rows) q.y = -q.y;
      pool_out[out_at(j)] = q;
    }
  }
}

// T = R[:, invperm(p)] (r x n, ld r, algrecomp.jl:86): the upper trapezoid of
// the QR's first r rows with the columns back in their original order
__global__ void transfer_kernel(const CTask* __restrict__ tasks, const float2* __restrict__ Zg,
                                const int32_t* __restrict__ permpool, float2* __restrict__ pool) {
  const CTask t = tasks[blockIdx.x];
  const int r = t.rank, n = t.n_cols, ldz = t.n_rows;
  if (r <= 0) return;  // a zero stack: the host leaves the group as it is
  const float2* __restrict__ R = Zg + t.z_off;
  const int32_t* __restrict__ p = permpool + t.perm_off;
  float2* __restrict__ T = pool + t.t_off;
  for (long long e = threadIdx.x; e < (long long)r * n; e += blockDim.x) {
    const int j = (int)(e / r), i = (int)(e - (long long)j * r);
    T[i + (long long)p[j] * r] = i <= j ? R[i + (long long)j * ldz] : make_float2(0.f, 0.f);
  }
}

// one small complex GEMM per CTA; FP32 products summed in float-float
__global__ void gemm_kernel(const GemmSeg* __restrict__ segs, const float2* __restrict__ pool_in,
                            float2* __restrict__ pool_out) {
  const GemmSeg g = segs[blockIdx.x];
  const long long tot = (long long)g.m * g.n;
  if (g.mode >= 2) {
    for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
      const int c = (int)(e / g.m), i = (int)(e - (long long)c * g.m);
      float2 v = g.mode == 2 ? pool_in[g.a + e] : pool_in[g.b + c + (long long)i * g.n];
      if (g.mode == 3) v.y = -v.y;
      pool_out[g.c + e] = v;
    }
    return;
  }
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    const int c = (int)(e / g.m), i = (int)(e - (long long)c * g.m);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = 0; q < g.k; ++q) {
      const float2 a = pool_in[g.a + i + (long long)q * g.m];
      float2 b = g.mode ? pool_in[g.b + c + (long long)q * g.n]
                        : pool_in[g.b + q + (long long)c * g.k];
      if (g.mode) b.y = -b.y;
      // a * b with the float-float accumulator: x = b as a float-float value
      cdf_mac(acc, a, make_float4(b.x, 0.f, b.y, 0.f));
    }
    pool_out[g.c + e] = make_float2(acc.x + acc.y, acc.z + acc.w);
  }
}

}  // namespace
}  // namespace bfg

namespace bfg {
namespace {

// one block of the operator during recompression; its entries (complex FP32,
// column-major, rows x cols) sit in the pool at `off`
struct RB {
  int32_t bf, stage;
  int64_t oo, so, oi, si;
  int32_t rows, cols;
  int8_t ident;
  int64_t off;
};

// bump-allocated device storage of block entries; grows by copying
struct Pool {
  float2* d = nullptr;
  int64_t used = 0, cap = 0;
  ~Pool() {
    if (d) cudaFree(d);
  }
  int reserve(int64_t extra) {
    if (used + extra <= cap) return BF_OK;
    const int64_t nc = std::max<int64_t>(used + extra, cap + cap / 2 + 1024);
    float2* nd = nullptr;
    if (cudaMalloc(&nd, (size_t)nc * sizeof(float2)) != cudaSuccess) {
      cudaGetLastError();
      set_error("bf_op_recompress: cannot allocate %lld block entries", (long long)nc);
      return BF_ENOMEM;
    }
    if (used > 0) BF_TRY_CUDA(cudaMemcpy(nd, d, (size_t)used * sizeof(float2), cudaMemcpyDeviceToDevice));
    if (d) cudaFree(d);
    d = nd;
    cap = nc;
    return BF_OK;
  }
  int64_t take(int64_t n) {
    const int64_t o = used;
    used += n;
    return o;
  }
};

template <typename T>
int upload(std::vector<void*>& owned, T** out, const std::vector<T>& v) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    set_error("bf_op_recompress: device allocation failed");
    return BF_ENOMEM;
  }
  owned.push_back(p);
  if (!v.empty()) BF_TRY_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = (T*)p;
  return BF_OK;
}

struct Owned {
  std::vector<void*> p;
  ~Owned() {
    for (void* q : p) cudaFree(q);
  }
};

// One pass over one level: `right` compresses the column space of the blocks
// of `stage` that share (bf, obs_in, src_in) and multiplies the transfer
// matrix into the blocks of stage - 1 with that row key (algrecomp.jl:59-139);
// the left pass (right == false) compresses the row space of the blocks that
// share (bf, obs_out, src_out) and multiplies into stage + 1 -- the right pass
// of the adjoint (algrecomp.jl:28-30).  Returns the groups compressed.
int level_pass(std::vector<RB>& B, int32_t stage, bool right, double tau, Pool& pool,
               int64_t* n_groups) {
  const int32_t nst = right ? stage - 1 : stage + 1;
  auto gkey = [&](const RB& b) {
    return right ? std::make_tuple(b.bf, b.oi, b.si) : std::make_tuple(b.bf, b.oo, b.so);
  };
  auto nkey = [&](const RB& b) {
    return right ? std::make_tuple(b.bf, b.oo, b.so) : std::make_tuple(b.bf, b.oi, b.si);
  };
  std::map<std::tuple<int32_t, int64_t, int64_t>, int> gid;
  std::vector<std::vector<int64_t>> mem, nbr;
  std::vector<uint8_t> bad;
  for (int64_t i = 0; i < (int64_t)B.size(); ++i) {
    if (B[i].stage != stage) continue;
    auto it = gid.emplace(gkey(B[i]), (int)mem.size());
    if (it.second) {
      mem.emplace_back();
      nbr.emplace_back();
      bad.push_back(0);
    }
    mem[it.first->second].push_back(i);
    if (B[i].ident) bad[it.first->second] = 1;
  }
  for (int64_t i = 0; i < (int64_t)B.size(); ++i) {
    if (B[i].stage != nst) continue;
    auto it = gid.find(nkey(B[i]));
    if (it == gid.end()) continue;
    nbr[it->second].push_back(i);
  }
  // the stacks: right = members on top of each other (sum rows x cols),
  // left = members' adjoints on top of each other (sum cols x rows)
  std::vector<CTask> ct;
  std::vector<StackSeg> ss;
  std::vector<int> task_of(mem.size(), -1);
  int64_t zsz = 0, psz = 0, tsz = 0;
  for (size_t g = 0; g < mem.size(); ++g) {
    if (bad[g] || mem[g].empty()) continue;
    const RB& b0 = B[mem[g][0]];
    const int n = right ? b0.cols : b0.rows;  // the shared dimension (compressed)
    int64_t m = 0;
    bool same = n > 0;
    for (int64_t i : mem[g]) {
      if ((right ? B[i].cols : B[i].rows) != n) same = false;
      m += right ? B[i].rows : B[i].cols;
    }
    for (int64_t i : nbr[g])  // an identity neighbour has the shared dimension
      if (!B[i].ident && (right ? B[i].rows : B[i].cols) != n) same = false;
    // a group without neighbours has nowhere to put its transfer matrix (the
    // last R level in the left pass): the reference never visits it
    if (!same || m == 0 || m >= (1 << 30) || nbr[g].empty()) continue;
    const int kmax = (int)std::min<int64_t>(m, n);
    if (qr_smem_bytes(0, n, false) > (size_t)QR_MAX_SMEM) continue;  // norms do not fit
    CTask t;
    std::memset(&t, 0, sizeof(t));
    t.z_off = zsz;
    t.perm_off = psz;
    t.t_off = tsz;  // relative; the pool offset is added below
    t.eps = tau;
    t.n_rows = (int)m;
    t.n_cols = n;
    t.n_obs = (int)m;
    int64_t row0 = 0;
    for (int64_t i : mem[g]) {
      StackSeg s{B[i].off, zsz, B[i].rows, B[i].cols, (int)m, (int)row0, right ? 0 : 1, 0};
      ss.push_back(s);
      row0 += right ? B[i].rows : B[i].cols;
    }
    task_of[g] = (int)ct.size();
    ct.push_back(t);
    zsz += m * n;
    psz += n;
    tsz += (int64_t)kmax * n;
  }
  if (n_groups) *n_groups = (int64_t)ct.size();
  if (ct.empty()) return BF_OK;
  BF_TRY(pool.reserve(tsz));
  const int64_t t_base = pool.take(tsz);
  for (auto& t : ct) t.t_off += t_base;
  Owned own;
  CTask* d_ct;
  StackSeg* d_ss;
  int32_t* d_perm;
  float2* d_Z;
  BF_TRY(upload(own.p, &d_ct, ct));
  BF_TRY(upload(own.p, &d_ss, ss));
  BF_TRY(upload(own.p, &d_perm, std::vector<int32_t>((size_t)psz, 0)));
  BF_TRY(upload(own.p, &d_Z, std::vector<float2>((size_t)zsz)));
  cudaStream_t st = nullptr;
  stack_kernel<<<(unsigned)ss.size(), 128, 0, st>>>(d_ss, pool.d, d_Z);
  BF_TRY_CUDA(cudaGetLastError());
  // QR: tasks whose stack fits shared memory, then the others (norms only)
  std::vector<int> fit, nofit;
  size_t smem_fit = 0, smem_nofit = 0;
  for (int q = 0; q < (int)ct.size(); ++q) {
    const size_t sf = qr_smem_bytes(ct[q].n_rows, ct[q].n_cols, true);
    if (sf <= (size_t)QR_MAX_SMEM) {
      fit.push_back(q);
      smem_fit = std::max(smem_fit, sf);
    } else {
      nofit.push_back(q);
      smem_nofit = std::max(smem_nofit, qr_smem_bytes(ct[q].n_rows, ct[q].n_cols, false));
    }
  }
  // the QR kernel takes a contiguous task range: order the tasks fit first
  std::vector<CTask> ord;
  for (int q : fit) ord.push_back(ct[q]);
  for (int q : nofit) ord.push_back(ct[q]);
  BF_TRY_CUDA(cudaMemcpy(d_ct, ord.data(), ord.size() * sizeof(CTask), cudaMemcpyHostToDevice));
  if (!fit.empty()) BF_TRY(launch_qr(d_ct, (int)fit.size(), d_Z, d_perm, true, smem_fit, st));
  if (!nofit.empty())
    BF_TRY(launch_qr(d_ct + fit.size(), (int)nofit.size(), d_Z, d_perm, false, smem_nofit, st));
  std::vector<CTask> done(ord.size());
  BF_TRY_CUDA(cudaMemcpy(done.data(), d_ct, done.size() * sizeof(CTask), cudaMemcpyDeviceToHost));
  transfer_kernel<<<(unsigned)done.size(), 128, 0, st>>>(d_ct, d_Z, d_perm, pool.d);
  BF_TRY_CUDA(cudaGetLastError());
  // new blocks: members get their rows of Q (r columns, or r rows on the
  // left), neighbours are multiplied by T
  std::vector<int> pos_of(ct.size());
  for (size_t a = 0; a < fit.size(); ++a) pos_of[fit[a]] = (int)a;
  for (size_t a = 0; a < nofit.size(); ++a) pos_of[nofit[a]] = (int)(fit.size() + a);
  std::vector<int> grank(mem.size(), -1);
  std::vector<const CTask*> gt(mem.size(), nullptr);
  int64_t need = 0;
  for (size_t g = 0; g < mem.size(); ++g) {
    if (task_of[g] < 0) continue;
    const CTask& t = done[pos_of[task_of[g]]];
    const int r = t.rank, n = t.n_cols;
    // a full rank r = n still replaces the blocks: Q is orthonormal and T
    // carries the weight of this level into the next stacks (the reference
    // does the same); only a zero stack (r = 0) is left as it is
    if (r <= 0) continue;
    grank[g] = r;
    gt[g] = &t;
    for (int64_t i : mem[g]) need += right ? (int64_t)B[i].rows * r : (int64_t)r * B[i].cols;
    for (int64_t i : nbr[g])
      need += B[i].ident ? (int64_t)r * n : right ? (int64_t)r * B[i].cols : (int64_t)B[i].rows * r;
  }
  if (need == 0) return BF_OK;
  BF_TRY(pool.reserve(need));
  std::vector<QSeg> qs;
  std::vector<GemmSeg> gm;
  for (size_t g = 0; g < mem.size(); ++g) {
    const int r = grank[g];
    if (r < 0) continue;
    const int n = right ? B[mem[g][0]].cols : B[mem[g][0]].rows;
    for (int64_t i : mem[g]) {
      const int64_t o = pool.take(right ? (int64_t)B[i].rows * r : (int64_t)r * B[i].cols);
      qs.push_back(QSeg{B[i].off, o, gt[g]->z_off, gt[g]->perm_off, B[i].rows, B[i].cols, r,
                        gt[g]->n_rows, right ? 0 : 1, 0, 0, 0});
      B[i].off = o;
      if (right)
        B[i].cols = r;
      else
        B[i].rows = r;
    }
    for (int64_t i : nbr[g]) {
      if (B[i].ident) {  // I becomes T (right) or T^H (left), a dense block
        const int64_t o = pool.take((int64_t)r * n);
        gm.push_back(right ? GemmSeg{gt[g]->t_off, 0, o, r, n, 0, 2}
                           : GemmSeg{0, gt[g]->t_off, o, n, r, 0, 3});
        B[i].ident = 0;
        B[i].off = o;
        B[i].rows = right ? r : n;
        B[i].cols = right ? n : r;
      } else if (right) {  // T (r x n) * D (n x cols)
        const int64_t o = pool.take((int64_t)r * B[i].cols);
        gm.push_back(GemmSeg{gt[g]->t_off, B[i].off, o, r, B[i].cols, n, 0});
        B[i].off = o;
        B[i].rows = r;
      } else {  // D (rows x n) * T^H, T stored r x n
        const int64_t o = pool.take((int64_t)B[i].rows * r);
        gm.push_back(GemmSeg{B[i].off, gt[g]->t_off, o, B[i].rows, r, n, 1});
        B[i].off = o;
        B[i].cols = r;
      }
    }
  }
  QSeg* d_qs;
  GemmSeg* d_gm;
  BF_TRY(upload(own.p, &d_qs, qs));
  BF_TRY(upload(own.p, &d_gm, gm));
  if (!qs.empty())
    qsolve_kernel<<<(unsigned)qs.size(), 128, 0, st>>>(d_qs, pool.d, d_Z, d_perm, pool.d);
  if (!gm.empty()) gemm_kernel<<<(unsigned)gm.size(), 128, 0, st>>>(d_gm, pool.d, pool.d);
  BF_TRY_CUDA(cudaGetLastError());
  BF_TRY_CUDA(cudaDeviceSynchronize());
  return BF_OK;
}

}  // namespace
}  // namespace bfg

using namespace bfg;

extern "C" int bf_op_recompress(bf_op_t h, double tau, bf_op_t* out) {
  try {
    if (!h || !out || !(tau > 0)) {
      set_error("bf_op_recompress: invalid argument");
      return BF_EINVAL;
    }
    *out = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    Operator& op = h->op;
    if (op.near) {
      set_error("bf_op_recompress: recompress the far field before attaching the near field");
      return BF_ENOTSUP;
    }
    if (!op.d_A && !op.d_A2) {
      set_error("bf_op_recompress: operator has no factors");
      return BF_ESTATE;
    }
    BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
    const Plan& p = op.plan;
    const auto& LB = op.logical.blocks;
    // every block's entries from the packed factors into the pool (complex FP32)
    std::vector<RB> B(LB.size());
    std::vector<GatherSeg> gs;
    int64_t total = 0;
    int32_t max_stage = 0;
    for (size_t b = 0; b < LB.size(); ++b) {
      const LBlock& k = LB[b];
      RB& r = B[b];
      r = RB{k.bf, k.stage, k.oo, k.so, k.oi, k.si, k.rows, k.cols, k.ident, 0};
      max_stage = std::max(max_stage, k.stage);
      if (k.ident || (int64_t)k.rows * k.cols == 0) continue;
      if (p.blk_pk_off[b] < 0) {
        set_error("bf_op_recompress: block %zu has no packed entries", b);
        return BF_ESTATE;
      }
      r.off = total;
      gs.push_back(GatherSeg{p.blk_pk_off[b], total, p.blk_pk_ld[b], k.rows, k.cols, 0});
      total += (int64_t)k.rows * k.cols;
    }
    Pool pool;
    BF_TRY(pool.reserve(total + 1));
    pool.take(total);
    {
      Owned own;
      GatherSeg* d_gs;
      BF_TRY(upload(own.p, &d_gs, gs));
      for (size_t b0 = 0; b0 < gs.size(); b0 += (1u << 30)) {
        const unsigned nb = (unsigned)std::min<size_t>(gs.size() - b0, 1u << 30);
        if (op.d_A2)
          gather_kernel<float2><<<nb, 128>>>(d_gs + b0, op.d_A2, pool.d);
        else
          gather_kernel<float4><<<nb, 128>>>(d_gs + b0, op.d_A, pool.d);
      }
      BF_TRY_CUDA(cudaGetLastError());
      BF_TRY_CUDA(cudaDeviceSynchronize());
    }
    // right pass: R levels from the last to the second (algrecomp.jl:59-139);
    // left pass: the right pass of the adjoint, R levels from the first up
    // (algrecomp.jl:28-30)
    int64_t groups = 0, ng = 0;
    for (int32_t s = max_stage; s >= 2; --s) {
      BF_TRY(level_pass(B, s, true, tau, pool, &ng));
      groups += ng;
    }
    for (int32_t s = 1; s < max_stage; ++s) {
      BF_TRY(level_pass(B, s, false, tau, pool, &ng));
      groups += ng;
    }
    // the new operator: the same keys and trees, packed from the pool
    auto nh = std::make_unique<bf_operator>();
    Operator& o2 = nh->op;
    o2.ctx = op.ctx;
    Logical& lg = o2.logical;
    lg.n_rows = op.logical.n_rows;
    lg.n_cols = op.logical.n_cols;
    lg.n_bf = op.logical.n_bf;
    lg.obs_vals = op.logical.obs_vals;
    lg.src_vals = op.logical.src_vals;
    lg.blocks.resize(B.size());
    for (size_t b = 0; b < B.size(); ++b) {
      const RB& r = B[b];
      LBlock& k = lg.blocks[b];
      k.bf = r.bf;
      k.stage = r.stage;
      k.oo = r.oo;
      k.so = r.so;
      k.oi = r.oi;
      k.si = r.si;
      k.ident = r.ident;
      k.rows = r.ident ? 0 : r.rows;
      k.cols = r.ident ? 0 : r.cols;
      k.raw_off = r.off;
      k.raw_ld = std::max(k.rows, 1);
      k.in_slot = k.out_slot = -1;  // wiring from the routing keys
    }
    o2.raw_is_double = 0;
    o2.store_ff = op.d_A ? 1 : 0;  // keep the storage of the input operator
    o2.d_raw = pool.d;
    o2.raw_entries = pool.used;
    pool.d = nullptr;
    BF_TRY(pack_plan(lg, o2.plan, o2.store_ff ? (int)sizeof(float4) : (int)sizeof(float2)));
    BF_TRY(upload_plan(o2));
    BF_TRY_CUDA(cudaDeviceSynchronize());
    o2.stats.build_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    o2.stats.compressions = groups;
    *out = nh.release();
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_op_recompress: host allocation failed");
    return BF_ENOMEM;
  }
}
