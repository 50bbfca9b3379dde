// Near field of the operator (bf_op_add_near, applied inside bf_matvec).
//
// The reference assembles one dense block K(values(o), values(s)) per near
// pair (src/Matrixassembly/petrovgalerkinbf.jl:57-119) into a
// BlockSparseMatrix and adds its product before the far loop
// (src/matrixalgebra/matrixvector.jl:28-33).  Here the blocks are grouped
// into dense tasks of the far-field layout: one task per observer leaf holds
// the blocks of every near pair whose observer node is the leaf or one of its
// ancestors, side by side (the P-stage shape: few rows, many columns), so every
// output entry has one writer; the adjoint gets its own tasks, one per source
// leaf with the transposed blocks.
//
// Arithmetic is FP64 throughout, as in the reference: the entries are
// evaluated once on the GPU (k*r, sincos, 1/(4 pi r)) and stored as complex
// FP64 (16 B, the bytes of a float-float entry), the inputs are read in FP64
// straight from the caller's vector by point id, and the sums run on the FP64
// FMA pipe.  Near rows sum thousands of large entries of opposing phase, where
// the 48 bits of float-float storage cost up to ~1e-12 of relative accuracy;
// at 8 flop per 16-byte entry the FP64 pipe of GB300 (~1.2 TFLOP/s) keeps
// about the speed of the float-float kernels.  The point kernel is singular at
// r = 0; those entries (a point with itself) are zero.
#include <algorithm>
#include <memory>
#include <stdexcept>
#include <vector>

#include "bf_dfloat.cuh"
#include "bf_fwd_warp.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

// one task's entries: rows from pts_r[rp .. rp + M), columns from pts_c[cp .. cp + n)
struct alignas(16) NearEval {
  long long a_off, rp, cp;
  int M, n, adj, pad;
};

// A[a_off + j*M + i] = G(obs, src) with (obs, src) = (row i, column j) for a
// forward task and (column j, row i) for an adjoint task (its blocks are
// transposed), as float-float complex entries
__global__ void near_eval_kernel(const NearEval* __restrict__ ev, const double* __restrict__ obs,
                                 const double* __restrict__ src, const int32_t* __restrict__ pts_r,
                                 const int32_t* __restrict__ pts_c, double k,
                                 double2* __restrict__ A) {
  const NearEval e = ev[blockIdx.x];
  const long long tot = (long long)e.M * e.n;
  for (long long q = threadIdx.x; q < tot; q += blockDim.x) {
    const int j = (int)(q / e.M), i = (int)(q - (long long)j * e.M);
    const int pr = pts_r[e.rp + i], pc = pts_c[e.cp + j];
    const double* a = e.adj ? obs + 3 * (long long)pc : obs + 3 * (long long)pr;
    const double* b = e.adj ? src + 3 * (long long)pr : src + 3 * (long long)pc;
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    const double r = sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
    double re = 0.0, im = 0.0;
    if (r > 0.0) {
      double sn, cs;
      sincos(k * r, &sn, &cs);
      const double inv = 1.0 / (12.566370614359172954 * r);
      re = cs * inv;
      im = -sn * inv;
    }
    A[e.a_off + q] = make_double2(re, im);
  }
}

// y[perm[q]] += alpha * ws[off + q]
__global__ void near_add_kernel(double2* __restrict__ y, int64_t n, const float4* __restrict__ ws,
                                int64_t off, double2 alpha, const int32_t* __restrict__ perm) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = ws[off + q];
    const double vr = (double)a.x + (double)a.y, vi = (double)a.z + (double)a.w;
    double2 o = y[perm[q]];
    o.x += alpha.x * vr - alpha.y * vi;
    o.y += alpha.x * vi + alpha.y * vr;
    y[perm[q]] = o;
  }
}

// acc += a * v, or conj(a) * v, in FP64
template <bool CONJ>
__device__ __forceinline__ void zmac(double2& acc, const double2 a, const double2 v) {
  const double ai = CONJ ? -a.y : a.y;
  acc.x = fma(a.x, v.x, acc.x);
  acc.x = fma(-ai, v.y, acc.x);
  acc.y = fma(a.x, v.y, acc.y);
  acc.y = fma(ai, v.x, acc.y);
}

__device__ __forceinline__ float4 split_z(const double2 v) {
  const float2 re = df_split(v.x), im = df_split(v.y);
  return make_float4(re.x, re.y, im.x, im.y);
}

constexpr int NX = 256;  // input entries staged per warp and pass
constexpr int NLU = 4;   // factor loads in flight per lane

// Task with M <= 32 rows, one warp.  Inputs x[point of column j] are staged
// per pass; the rows are walked in panels of M's binary digits (below), and
// row i goes to ws[rmap[i]] as a float-float entry.  At least 3 CTAs per SM:
// the six panel accumulators fit 80 registers without spills (left to itself
// the compiler chose 64 and spilled).  Against lane groups G = 32/M with idle
// lanes, the forward near product at 262,144 points went from 2.55 to 1.87 ms.
template <bool CONJ>
__global__ void __launch_bounds__(FW_WARPS * 32, 3) near_small_kernel(
    const int32_t* __restrict__ tlist, int n_tasks, const DTask* __restrict__ tasks,
    const double2* __restrict__ A, const int32_t* __restrict__ maps,
    const int32_t* __restrict__ pts, const double2* __restrict__ x, float4* __restrict__ ws) {
  __shared__ double2 xs[FW_WARPS][NX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.x * FW_WARPS + warp;
  if (ti >= n_tasks) return;
  const DTask t = tasks[tlist[ti]];
  const int M = t.M, n = t.n;
  const int32_t* __restrict__ cpt = pts + t.cmap_off;
  double2* xw = xs[warp];
  // the rows in panels of M's binary digits (21 = 16 + 4 + 1), largest first:
  // panel b has m = 2^b rows from r0 = M with bits 0..b cleared, and G = 32/m
  // lane groups fill all 32 lanes (a warp's FP64 FMA takes the pipe as long
  // with idle lanes as without); the warp walks them one after another on the
  // same staged inputs, one accumulator per panel
  double2 acc[6];
#pragma unroll
  for (int b = 0; b < 6; ++b) acc[b] = make_double2(0.0, 0.0);
  for (int cb = 0; cb < n; cb += NX) {
    const int nb = min(NX, n - cb);
    for (int j = lane; j < nb; j += 32) xw[j] = x[cpt[cb + j]];
    __syncwarp();
#pragma unroll
    for (int b = 5; b >= 0; --b) {
      if (!(M & (1 << b))) continue;  // warp-uniform
      const int pr0 = M & ~((2 << b) - 1);
      const int pG = 32 >> b, pg = lane >> b, pi = lane & ((1 << b) - 1);
      const double2* __restrict__ ap = A + t.a_off + (size_t)(cb + pg) * M + pr0 + pi;
      const size_t step = (size_t)pG * M;
      int j = pg;
      for (; j + (NLU - 1) * pG < nb; j += NLU * pG) {
        double2 a[NLU];
#pragma unroll
        for (int u = 0; u < NLU; ++u) a[u] = __ldg(ap + u * step);
#pragma unroll
        for (int u = 0; u < NLU; ++u) zmac<CONJ>(acc[b], a[u], xw[j + u * pG]);
        ap += NLU * step;
      }
      for (; j < nb; j += pG, ap += step) zmac<CONJ>(acc[b], __ldg(ap), xw[j]);
    }
    __syncwarp();
  }
#pragma unroll
  for (int b = 5; b >= 0; --b) {
    if (!(M & (1 << b))) continue;
    // lanes pg*m + pi of all groups hold row pi's partial sums
    for (int s = 1 << b; s < 32; s <<= 1) {
      acc[b].x += __shfl_xor_sync(0xffffffffu, acc[b].x, s);
      acc[b].y += __shfl_xor_sync(0xffffffffu, acc[b].y, s);
    }
    const int pr0 = M & ~((2 << b) - 1);
    if ((lane >> b) == 0) ws[maps[t.rmap_off + pr0 + (lane & ((1 << b) - 1))]] = split_z(acc[b]);
  }
}

// Task with M > 32 rows: one warp per 64-row panel (item = task, first row),
// two rows per lane, coalesced loads down the columns.
template <bool CONJ>
__global__ void __launch_bounds__(FW_WARPS * 32) near_tall_kernel(
    const int2* __restrict__ items, int n_items, const DTask* __restrict__ tasks,
    const double2* __restrict__ A, const int32_t* __restrict__ maps,
    const int32_t* __restrict__ pts, const double2* __restrict__ x, float4* __restrict__ ws) {
  __shared__ double2 xs[FW_WARPS][NX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * FW_WARPS + warp;
  if (item >= n_items) return;
  const int2 it = items[item];
  const DTask t = tasks[it.x];
  const int M = t.M, n = t.n, r0 = it.y;
  if (r0 >= M) return;
  const int32_t* __restrict__ cpt = pts + t.cmap_off;
  double2* xw = xs[warp];
  const bool act0 = r0 + lane < M, act1 = r0 + lane + 32 < M;
  double2 acc0 = make_double2(0.0, 0.0), acc1 = make_double2(0.0, 0.0);
  for (int cb = 0; cb < n; cb += NX) {
    const int nb = min(NX, n - cb);
    for (int j = lane; j < nb; j += 32) xw[j] = x[cpt[cb + j]];
    __syncwarp();
    const double2* __restrict__ ap = A + t.a_off + (size_t)cb * M + r0 + lane;
#pragma unroll 4
    for (int j = 0; j < nb; ++j, ap += M) {
      const double2 v = xw[j];
      if (act0) zmac<CONJ>(acc0, __ldg(ap), v);
      if (act1) zmac<CONJ>(acc1, __ldg(ap + 32), v);
    }
    __syncwarp();
  }
  if (act0) ws[maps[t.rmap_off + r0 + lane]] = split_z(acc0);
  if (act1) ws[maps[t.rmap_off + r0 + lane + 32]] = split_z(acc1);
}

template <bool CONJ>
int launch_near(const NearField& nf, int small, int tall, cudaStream_t st, const double2* x,
                float4* ws, int64_t* nk) {
  const unsigned WT = FW_WARPS * 32;
  int64_t b = nf.list_begin[small], n = nf.list_begin[small + 1] - b;
  if (n > 0) {
    near_small_kernel<CONJ><<<(unsigned)((n + FW_WARPS - 1) / FW_WARPS), WT, 0, st>>>(
        nf.d_lists + b, (int)n, nf.d_tasks, nf.d_A, nf.d_maps, nf.d_pts, x, ws);
    if (nk) ++*nk;
  }
  b = nf.list_begin[tall];
  n = (nf.list_begin[tall + 1] - b) / 2;
  if (n > 0) {
    near_tall_kernel<CONJ><<<(unsigned)((n + FW_WARPS - 1) / FW_WARPS), WT, 0, st>>>(
        (const int2*)(nf.d_lists + b), (int)n, nf.d_tasks, nf.d_A, nf.d_maps, nf.d_pts, x, ws);
    if (nk) ++*nk;
  }
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

// leaves below node (the node itself when it is one), depth first
void leaves_below(const Tree& t, int64_t node, std::vector<int64_t>& out) {
  if (t.isleaf(node)) {
    out.push_back(node);
    return;
  }
  for (int32_t c = 0; c < t.n_child[node]; ++c) leaves_below(t, t.first_child[node] + c, out);
}

}  // namespace

void near_free(NearField* nf) {
  if (!nf) return;
  if (nf->d_A) cudaFree(nf->d_A);
  if (nf->d_tasks) cudaFree(nf->d_tasks);
  if (nf->d_maps) cudaFree(nf->d_maps);
  if (nf->d_pts) cudaFree(nf->d_pts);
  if (nf->d_lists) cudaFree(nf->d_lists);
  delete nf;
}

int near_upload(NearField& nf) {
  BF_TRY_CUDA(cudaMalloc(&nf.d_tasks, std::max<size_t>(1, nf.tasks.size()) * sizeof(DTask)));
  BF_TRY_CUDA(cudaMemcpy(nf.d_tasks, nf.tasks.data(), nf.tasks.size() * sizeof(DTask),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&nf.d_maps, std::max<size_t>(1, nf.maps.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(nf.d_maps, nf.maps.data(), nf.maps.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&nf.d_pts, std::max<size_t>(1, nf.pts.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(nf.d_pts, nf.pts.data(), nf.pts.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&nf.d_lists, std::max<size_t>(1, nf.lists.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(nf.d_lists, nf.lists.data(), nf.lists.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  return BF_OK;
}

int near_stage(const Operator& op, int trans, cudaStream_t st, const double2* x, float4* ws,
               int64_t* nk) {
  const NearField& nf = *op.near;
  const Plan& p = op.plan;
  if (trans == BF_OP_N) {
    if (!nf.fwd_covered)
      BF_TRY_CUDA(cudaMemsetAsync(ws + nf.ny_off, 0, (size_t)p.n_rows * sizeof(float4), st));
    return launch_near<false>(nf, NearField::N_SMALL_F, NearField::N_TALL_F, st, x, ws, nk);
  }
  if (!nf.adj_covered)
    BF_TRY_CUDA(cudaMemsetAsync(ws + nf.nx_off, 0, (size_t)p.n_cols * sizeof(float4), st));
  if (trans == BF_OP_C)
    return launch_near<true>(nf, NearField::N_SMALL_A, NearField::N_TALL_A, st, x, ws, nk);
  return launch_near<false>(nf, NearField::N_SMALL_A, NearField::N_TALL_A, st, x, ws, nk);
}

// y_c += alpha * near(op) x_c for every column, on top of a far-field result
// already in y (the tensor-core path covers the far field only)
int near_apply_columns(Operator& op, int trans, int64_t nrhs, const double2* x, int64_t lx,
                       double2* y, int64_t ly, double2 alpha, cudaStream_t st) {
  const Plan& p = op.plan;
  const bool fwd = trans == BF_OP_N;
  const int64_t nout = fwd ? p.n_rows : p.n_cols;
  const int64_t out_off = fwd ? op.near->ny_off : op.near->nx_off;
  const unsigned go = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nout + 255) / 256, 2432));
  for (int64_t c = 0; c < nrhs; ++c) {
    BF_TRY(near_stage(op, trans, st, x + c * lx, op.d_ws, nullptr));
    near_add_kernel<<<go, 256, 0, st>>>(y + c * ly, nout, op.d_ws, out_off, alpha,
                                        fwd ? op.d_yperm : op.d_xperm);
  }
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

}  // namespace bfg

using namespace bfg;

extern "C" int bf_op_add_near(bf_op_t h, const double* obs_xyz, int64_t n_obs,
                              const double* src_xyz, int64_t n_src, bf_tree_t obs_tree,
                              bf_tree_t src_tree, const int64_t* near_obs,
                              const int64_t* near_src, int64_t n_near, double k) {
  try {
    if (!h || !obs_xyz || !src_xyz || !obs_tree || !src_tree || n_near < 0 ||
        (n_near > 0 && (!near_obs || !near_src)) || !(k > 0)) {
      set_error("bf_op_add_near: invalid argument");
      return BF_EINVAL;
    }
    Operator& op = h->op;
    Plan& p = op.plan;
    const Tree& to = obs_tree->t;
    const Tree& ts = src_tree->t;
    if (op.near) {
      set_error("bf_op_add_near: the operator already has a near field");
      return BF_ESTATE;
    }
    if (n_obs != p.n_rows || n_src != p.n_cols || to.n_points != n_obs || ts.n_points != n_src) {
      set_error("bf_op_add_near: point counts differ from the operator's (%lld x %lld)",
                (long long)p.n_rows, (long long)p.n_cols);
      return BF_EINVAL;
    }
    if ((int64_t)p.xperm.size() != p.n_cols || (int64_t)p.yperm.size() != p.n_rows) {
      set_error("bf_op_add_near: operator without leaf orders");
      return BF_ESTATE;
    }
    for (int64_t q = 0; q < n_near; ++q)
      if (near_obs[q] < 0 || near_obs[q] >= to.nn() || near_src[q] < 0 || near_src[q] >= ts.nn()) {
        set_error("bf_op_add_near: near pair %lld references an unknown node", (long long)q);
        return BF_EINVAL;
      }
    if (p.ws_entries + p.n_rows + p.n_cols >= ((int64_t)1 << 31)) {
      set_error("bf_op_add_near: workspace would exceed 2^31 entries");
      return BF_ENOTSUP;
    }
    // point -> position in the y / x regions (leaf order)
    std::vector<int32_t> ypos(p.n_rows), xpos(p.n_cols);
    for (int64_t q = 0; q < p.n_rows; ++q) ypos[p.yperm[q]] = (int32_t)q;
    for (int64_t q = 0; q < p.n_cols; ++q) xpos[p.xperm[q]] = (int32_t)q;
    struct NearDel {
      void operator()(NearField* x) const { near_free(x); }
    };
    std::unique_ptr<NearField, NearDel> nf(new NearField);
    NearField& N = *nf;
    N.n_pairs = n_near;
    N.ny_off = p.ws_entries;
    N.nx_off = p.ws_entries + p.n_rows;
    // leaf -> the other side's nodes, per direction
    std::vector<std::vector<int64_t>> fwd_of(to.nn()), adj_of(ts.nn());
    std::vector<int64_t> lv;
    for (int64_t q = 0; q < n_near; ++q) {
      lv.clear();
      leaves_below(to, near_obs[q], lv);
      for (int64_t l : lv) fwd_of[l].push_back(near_src[q]);
      lv.clear();
      leaves_below(ts, near_src[q], lv);
      for (int64_t l : lv) adj_of[l].push_back(near_obs[q]);
    }
    std::vector<NearEval> ev;
    std::vector<int32_t> pts_r, pts_c;
    std::vector<int32_t> small_f, tall_f, small_a, tall_a;
    int64_t covered_f = 0, covered_a = 0;
    // one pass per direction: rows = leaf points, columns = the other side's nodes
    auto make = [&](const Tree& rt, const Tree& ct, std::vector<std::vector<int64_t>>& of,
                    const std::vector<int32_t>& rpos, int64_t rbase_off,
                    const std::vector<int32_t>& cpos, int64_t cbase_off, int adj,
                    std::vector<int32_t>& small, std::vector<int32_t>& tall, int64_t& covered) {
      for (int64_t l = 0; l < rt.nn(); ++l) {
        if (of[l].empty() || rt.nvals(l) == 0) continue;
        int64_t ncol = 0;
        for (int64_t c : of[l]) ncol += ct.nvals(c);
        if (ncol == 0) continue;
        const int64_t M = rt.nvals(l);
        if (M >= (1 << 30) || ncol >= (1 << 30)) throw std::length_error("near task too large");
        DTask t{};
        t.a_off = N.a_entries;
        t.M = (int)M;
        t.n = (int)ncol;
        t.kind = TASK_DENSE;
        t.rmap_off = (long long)N.maps.size();
        const int64_t* rv = rt.vals(l);
        bool contig = true;
        for (int64_t i = 0; i < M; ++i) {
          const int64_t e = rbase_off + rpos[rv[i]];
          N.maps.push_back((int32_t)e);
          N.pts.push_back((int32_t)rv[i]);
          if (e != rbase_off + rpos[rv[0]] + i) contig = false;
        }
        t.rbase = contig ? (int)(rbase_off + rpos[rv[0]]) : -1;
        t.cmap_off = (long long)N.maps.size();
        NearEval e{};
        e.a_off = N.a_entries;
        e.rp = (long long)pts_r.size();
        e.cp = (long long)pts_c.size();
        e.M = (int)M;
        e.n = (int)ncol;
        e.adj = adj;
        for (int64_t i = 0; i < M; ++i) pts_r.push_back((int32_t)rv[i]);
        for (int64_t c : of[l]) {
          const int64_t* cv = ct.vals(c);
          for (int64_t j = 0; j < ct.nvals(c); ++j) {
            N.maps.push_back((int32_t)(cbase_off + cpos[cv[j]]));
            N.pts.push_back((int32_t)cv[j]);
            pts_c.push_back((int32_t)cv[j]);
          }
        }
        t.cbase = -1;
        const int32_t ti = (int32_t)N.tasks.size();
        N.tasks.push_back(t);
        ev.push_back(e);
        N.a_entries += M * ncol;
        N.alg_bytes_fwd += 16 * (M * ncol + M + ncol);
        covered += M;
        if (M <= 32) {
          small.push_back(ti);
        } else {
          for (int64_t r0 = 0; r0 < M; r0 += TALL_ROWS) {
            tall.push_back(ti);
            tall.push_back((int32_t)r0);
          }
        }
      }
    };
    make(to, ts, fwd_of, ypos, N.ny_off, xpos, p.xg_off, 0, small_f, tall_f, covered_f);
    N.n_fwd = (int64_t)N.tasks.size();
    const int64_t fwd_alg = N.alg_bytes_fwd;
    make(ts, to, adj_of, xpos, N.nx_off, ypos, p.yg_off, 1, small_a, tall_a, covered_a);
    N.alg_bytes_fwd = fwd_alg;
    N.fwd_covered = covered_f == p.n_rows ? 1 : 0;
    N.adj_covered = covered_a == p.n_cols ? 1 : 0;
    const std::vector<int32_t>* cls[NearField::N_NCLASS];
    cls[NearField::N_TALL_F] = &tall_f;
    cls[NearField::N_TALL_A] = &tall_a;
    cls[NearField::N_SMALL_F] = &small_f;
    cls[NearField::N_SMALL_A] = &small_a;
    for (int c = 0; c < NearField::N_NCLASS; ++c) {
      N.list_begin[c] = (int64_t)N.lists.size();
      N.lists.insert(N.lists.end(), cls[c]->begin(), cls[c]->end());
    }
    // tall items are read as int2: their lists must start at even offsets
    if ((N.list_begin[NearField::N_TALL_F] | N.list_begin[NearField::N_TALL_A]) & 1)
      throw std::length_error("near field: tall list misaligned");
    N.list_begin[NearField::N_NCLASS] = (int64_t)N.lists.size();
    if (N.a_entries >= ((int64_t)1 << 40)) throw std::length_error("near field too large");
    // device: entries (evaluated here), tasks, maps, lists, the larger workspace
    BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
    struct Tmp {
      std::vector<void*> p;
      ~Tmp() {
        for (void* q : p) cudaFree(q);
      }
    } tmp;
    auto dev = [&](size_t bytes, void** out) -> int {
      if (cudaMalloc(out, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        set_error("bf_op_add_near: cannot allocate %zu bytes", bytes);
        return BF_ENOMEM;
      }
      return BF_OK;
    };
    void *d_obs, *d_src, *d_ev, *d_pr, *d_pc;
    BF_TRY(dev(3 * (size_t)n_obs * sizeof(double), &d_obs));
    tmp.p.push_back(d_obs);
    BF_TRY(dev(3 * (size_t)n_src * sizeof(double), &d_src));
    tmp.p.push_back(d_src);
    BF_TRY(dev(ev.size() * sizeof(NearEval), &d_ev));
    tmp.p.push_back(d_ev);
    BF_TRY(dev(pts_r.size() * sizeof(int32_t), &d_pr));
    tmp.p.push_back(d_pr);
    BF_TRY(dev(pts_c.size() * sizeof(int32_t), &d_pc));
    tmp.p.push_back(d_pc);
    BF_TRY(dev((size_t)N.a_entries * sizeof(double2), (void**)&N.d_A));
    BF_TRY_CUDA(cudaMemcpy(d_obs, obs_xyz, 3 * (size_t)n_obs * sizeof(double),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_src, src_xyz, 3 * (size_t)n_src * sizeof(double),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_ev, ev.data(), ev.size() * sizeof(NearEval), cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_pr, pts_r.data(), pts_r.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_pc, pts_c.data(), pts_c.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
    for (size_t b = 0; b < ev.size(); b += (1u << 30)) {
      const size_t nb = std::min<size_t>(ev.size() - b, 1u << 30);
      near_eval_kernel<<<(unsigned)nb, 128>>>((const NearEval*)d_ev + b, (const double*)d_obs,
                                              (const double*)d_src, (const int32_t*)d_pr,
                                              (const int32_t*)d_pc, k, N.d_A);
    }
    BF_TRY_CUDA(cudaGetLastError());
    BF_TRY_CUDA(cudaDeviceSynchronize());
    BF_TRY(near_upload(N));
    // the workspace grows by the two near output regions
    float4* ws = nullptr;
    const int64_t ws_new = p.ws_entries + p.n_rows + p.n_cols;
    BF_TRY(dev((size_t)ws_new * sizeof(float4), (void**)&ws));
    BF_TRY_CUDA(cudaMemset(ws, 0, (size_t)ws_new * sizeof(float4)));
    if (op.d_ws) cudaFree(op.d_ws);
    op.d_ws = ws;
    p.ws_entries = ws_new;
    op.stats.workspace_entries = ws_new;
    op.stats.near_pairs = n_near;
    op.stats.near_entries = N.a_entries;
    op.stats.near_bytes_fwd = N.alg_bytes_fwd;
    op.near = nf.release();
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_op_add_near: host allocation failed");
    return BF_ENOMEM;
  } catch (const std::length_error& e) {
    set_error("bf_op_add_near: %s", e.what());
    return BF_ENOTSUP;
  }
}
