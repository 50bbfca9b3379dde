// Materialised adjoint / transpose of an operator (bf_op_adjoint_copy).
//
// The reference's adjoint(BF) and transpose(BF) (src/Butterflyalgebra/
// bfadjtr.jl:13-67) build a new factorisation: every block becomes op(data)
// with its routing keys swapped (obs_out <- src_in, src_out <- obs_in,
// obs_in <- src_out, src_in <- obs_out; identities pass through), the R levels
// run in reverse order, P^H becomes the new Q and Q^H the new P, and the two
// trees trade places (reverse_tree).  Here the same is done for every far
// block of an operator at once: the blocks are read from the packed factors
// on the device, conjugate-transposed into a raw block store, and packed into
// a new operator whose forward matvec is op(A) x.  The library's adjoint and
// transpose views (bf_matvec with BF_OP_C / BF_OP_T) need no copy; a copy
// trades twice the factor memory for the forward kernels' speed.
#include <algorithm>
#include <chrono>
#include <memory>
#include <vector>

#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

// block rows x cols at src (leading dimension ld) -> op(block), cols x rows,
// column-major with leading dimension cols, at dst
struct alignas(16) TSeg {
  long long src, dst;
  int ld, rows, cols, pad;
};

__device__ __forceinline__ double2 to_raw(const float4 a, int conj) {
  // a float-float pair is exact in FP64 (at most 48 significant bits)
  const double im = (double)a.z + (double)a.w;
  return make_double2((double)a.x + (double)a.y, conj ? -im : im);
}
__device__ __forceinline__ float2 to_raw(const float2 a, int conj) {
  return make_float2(a.x, conj ? -a.y : a.y);
}

template <typename FT, typename OT>
__global__ void transpose_kernel(const TSeg* __restrict__ segs, const FT* __restrict__ A,
                                 OT* __restrict__ out, int conj) {
  const TSeg g = segs[blockIdx.x];
  const long long tot = (long long)g.rows * g.cols;
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    // entry (c, r) of the cols x rows result is entry (r, c) of the block
    const int r = (int)(e / g.cols), c = (int)(e - (long long)r * g.cols);
    out[g.dst + e] = to_raw(A[g.src + (long long)c * g.ld + r], conj);
  }
}

}  // namespace
}  // namespace bfg

using namespace bfg;

extern "C" int bf_op_adjoint_copy(bf_op_t h, int trans, bf_op_t* out) {
  try {
    if (!h || !out || (trans != BF_OP_C && trans != BF_OP_T)) {
      set_error("bf_op_adjoint_copy: invalid argument (trans must be BF_OP_C or BF_OP_T)");
      return BF_EINVAL;
    }
    *out = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    Operator& op = h->op;
    if (op.near) {
      set_error("bf_op_adjoint_copy: the operator has a near field; apply its adjoint view "
                "(bf_matvec with BF_OP_C / BF_OP_T) instead");
      return BF_ENOTSUP;
    }
    if (!op.d_A && !op.d_A2) {
      set_error("bf_op_adjoint_copy: operator has no factors");
      return BF_ESTATE;
    }
    BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
    const Plan& p = op.plan;
    const auto& LB = op.logical.blocks;
    const bool ff = op.d_A != nullptr;
    // R levels per far block: level l of the copy is level L + 1 - l of the input
    int32_t nbf = 0;
    for (const LBlock& k : LB) nbf = std::max(nbf, k.bf + 1);
    std::vector<int32_t> nr((size_t)std::max(nbf, 1), 0);
    for (const LBlock& k : LB)
      if (k.stage > 0) nr[k.bf] = std::max(nr[k.bf], k.stage);
    auto nh = std::make_unique<bf_operator>();
    Operator& o2 = nh->op;
    o2.ctx = op.ctx;
    Logical& lg = o2.logical;
    lg.n_rows = op.logical.n_cols;
    lg.n_cols = op.logical.n_rows;
    lg.n_bf = op.logical.n_bf;
    lg.obs_vals = op.logical.src_vals;
    lg.src_vals = op.logical.obs_vals;
    lg.blocks.resize(LB.size());
    std::vector<TSeg> segs;
    int64_t total = 0;
    for (size_t b = 0; b < LB.size(); ++b) {
      const LBlock& k = LB[b];
      LBlock& t = lg.blocks[b];
      t.bf = k.bf;
      t.stage = k.stage == 0 ? -1 : k.stage < 0 ? 0 : nr[k.bf] + 1 - k.stage;
      t.oo = k.si;
      t.so = k.oi;
      t.oi = k.so;
      t.si = k.oo;
      t.ident = k.ident;
      t.rows = k.ident ? 0 : k.cols;  // identities carry no entries (sized by their slots)
      t.cols = k.ident ? 0 : k.rows;
      t.raw_off = 0;
      t.raw_ld = std::max(t.rows, 1);
      t.in_slot = t.out_slot = -1;  // wiring from the routing keys
      if (k.ident || (int64_t)k.rows * k.cols == 0) continue;
      if (p.blk_pk_off[b] < 0) {
        set_error("bf_op_adjoint_copy: block %zu has no packed entries", b);
        return BF_ESTATE;
      }
      t.raw_off = total;
      segs.push_back(TSeg{p.blk_pk_off[b], total, p.blk_pk_ld[b], k.rows, k.cols, 0});
      total += (int64_t)k.rows * k.cols;
    }
    // the raw store: FP64 pairs for float-float factors (exact), complex FP32 otherwise
    const size_t esz = ff ? sizeof(double2) : sizeof(float2);
    void* raw = nullptr;
    if (cudaMalloc(&raw, (size_t)std::max<int64_t>(total, 1) * esz) != cudaSuccess) {
      cudaGetLastError();
      set_error("bf_op_adjoint_copy: cannot allocate %lld block entries", (long long)total);
      return BF_ENOMEM;
    }
    o2.d_raw = raw;  // owned by the new operator from here on
    o2.raw_entries = total;
    o2.raw_is_double = ff ? 1 : 0;
    o2.store_ff = 0;
    if (!segs.empty()) {
      TSeg* d_segs = nullptr;
      BF_TRY_CUDA(cudaMalloc(&d_segs, segs.size() * sizeof(TSeg)));
      std::unique_ptr<TSeg, decltype(&cudaFree)> hold(d_segs, cudaFree);
      BF_TRY_CUDA(cudaMemcpy(d_segs, segs.data(), segs.size() * sizeof(TSeg),
                             cudaMemcpyHostToDevice));
      const int conj = trans == BF_OP_C ? 1 : 0;
      for (size_t b0 = 0; b0 < segs.size(); b0 += (1u << 30)) {
        const unsigned nb = (unsigned)std::min<size_t>(segs.size() - b0, 1u << 30);
        if (ff)
          transpose_kernel<float4, double2><<<nb, 128>>>(d_segs + b0, op.d_A, (double2*)raw, conj);
        else
          transpose_kernel<float2, float2><<<nb, 128>>>(d_segs + b0, op.d_A2, (float2*)raw, conj);
      }
      BF_TRY_CUDA(cudaGetLastError());
      BF_TRY_CUDA(cudaDeviceSynchronize());
    }
    BF_TRY(pack_plan(lg, o2.plan, ff ? (int)sizeof(float4) : (int)sizeof(float2)));
    BF_TRY(upload_plan(o2));
    BF_TRY_CUDA(cudaDeviceSynchronize());
    o2.stats.build_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = nh.release();
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_op_adjoint_copy: host allocation failed");
    return BF_ENOMEM;
  }
}
