// bf_compress_block: one compression of the GPU build, on caller-chosen
// observer and source points, with every intermediate returned to the host.
//
// The builder (bf_build_host.cpp) runs millions of these per operator in
// batched rounds; this entry runs exactly the same device launches (row
// sampling, kernel sampling, pivoted partial QR, interpolation solve) for one
// task, so a test can put one GPU compression beside one call of the
// reference's PartialQR compressor (src/ButterflyFactorization/
// compressors.jl:81-165) on identical sampled rows.
#include <algorithm>
#include <cstring>
#include <vector>

#include "bf_build.h"

namespace bfg {
namespace {

// device buffers of one probe, freed on every exit path
struct ProbeMem {
  std::vector<void*> p;
  template <typename T>
  int alloc(T** out, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      set_error("bf_compress_block: device allocation failed");
      return BF_ENOMEM;
    }
    p.push_back(q);
    *out = (T*)q;
    return BF_OK;
  }
  ~ProbeMem() {
    for (void* q : p) cudaFree(q);
  }
};

}  // namespace
}  // namespace bfg

using namespace bfg;

extern "C" int bf_compress_block(bf_ctx_t ctx, const double* obs_xyz, int64_t n_obs_pts,
                                        const double* src_xyz, int64_t n_src_pts,
                                        const int64_t* obs_index, int32_t n_obs,
                                        const int64_t* src_index, int32_t n_src, int32_t n_rows,
                                        uint64_t key, double k, double eps, int32_t* rows_out,
                                        float* Z_out, int32_t* rank_out, int32_t* perm_out,
                                        int32_t* skeleton_out, float* T_out) {
  try {
    if (!ctx || !obs_xyz || !src_xyz || !obs_index || !src_index || !rank_out || !perm_out ||
        !skeleton_out || !T_out || n_obs <= 0 || n_src <= 0 || n_rows <= 0 || n_rows > n_obs ||
        !(k > 0) || !(eps > 0)) {
      set_error("bf_compress_block: invalid argument");
      return BF_EINVAL;
    }
    for (int32_t i = 0; i < n_obs; ++i)
      if (obs_index[i] < 0 || obs_index[i] >= n_obs_pts || obs_index[i] >= (1ll << 31)) {
        set_error("bf_compress_block: observer index %d out of range", i);
        return BF_EINVAL;
      }
    for (int32_t j = 0; j < n_src; ++j)
      if (src_index[j] < 0 || src_index[j] >= n_src_pts || src_index[j] >= (1ll << 31)) {
        set_error("bf_compress_block: source index %d out of range", j);
        return BF_EINVAL;
      }
    BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
    const int kmax = std::min(n_rows, n_src);
    ProbeMem mem;
    double *d_obs, *d_src;
    int32_t *d_operm, *d_cols, *d_rows, *d_perm, *d_skel;
    float2 *d_Z, *d_T;
    CTask* d_task;
    BF_TRY(mem.alloc(&d_obs, 3 * (size_t)n_obs_pts));
    BF_TRY(mem.alloc(&d_src, 3 * (size_t)n_src_pts));
    BF_TRY(mem.alloc(&d_operm, (size_t)n_obs));
    BF_TRY(mem.alloc(&d_cols, (size_t)n_src));
    BF_TRY(mem.alloc(&d_rows, (size_t)n_rows));
    BF_TRY(mem.alloc(&d_perm, (size_t)n_src));
    BF_TRY(mem.alloc(&d_skel, (size_t)kmax));
    BF_TRY(mem.alloc(&d_Z, (size_t)n_rows * n_src));
    BF_TRY(mem.alloc(&d_T, (size_t)kmax * n_src));
    BF_TRY(mem.alloc(&d_task, 1));
    std::vector<int32_t> operm(obs_index, obs_index + n_obs), cols(src_index, src_index + n_src);
    CTask t;
    std::memset(&t, 0, sizeof(t));
    t.key = key;
    t.eps = eps;
    t.n_obs = n_obs;
    t.n_rows = n_rows;
    t.n_cols = n_src;
    BF_TRY_CUDA(cudaMemcpy(d_obs, obs_xyz, 3 * (size_t)n_obs_pts * sizeof(double),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_src, src_xyz, 3 * (size_t)n_src_pts * sizeof(double),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_operm, operm.data(), operm.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_cols, cols.data(), cols.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
    BF_TRY_CUDA(cudaMemcpy(d_task, &t, sizeof(CTask), cudaMemcpyHostToDevice));
    cudaStream_t st = nullptr;  // legacy stream: the probe is synchronous
    BF_TRY(launch_rows(d_task, 1, d_operm, d_rows, st));
    BF_TRY(launch_eval(d_task, 1, d_obs, d_src, d_rows, d_cols, d_Z, k, 0, st));
    BF_TRY_CUDA(cudaDeviceSynchronize());
    if (rows_out)
      BF_TRY_CUDA(cudaMemcpy(rows_out, d_rows, (size_t)n_rows * sizeof(int32_t),
                             cudaMemcpyDeviceToHost));
    if (Z_out)
      BF_TRY_CUDA(cudaMemcpy(Z_out, d_Z, (size_t)n_rows * n_src * sizeof(float2),
                             cudaMemcpyDeviceToHost));
    // the builder's choice: the block in shared memory when it fits; either
    // way the column norms and the permutation (n_src entries) live there
    const bool smem_z = qr_smem_bytes(n_rows, n_src, true) <= (size_t)QR_MAX_SMEM;
    const size_t smem = qr_smem_bytes(n_rows, n_src, smem_z);
    if (smem > (size_t)QR_MAX_SMEM) {
      set_error("bf_compress_block: %d columns exceed the QR kernel's shared memory", n_src);
      return BF_EINVAL;
    }
    BF_TRY(launch_qr(d_task, 1, d_Z, d_perm, smem_z, smem, st));
    BF_TRY_CUDA(cudaMemcpy(&t, d_task, sizeof(CTask), cudaMemcpyDeviceToHost));
    const int r = t.rank;
    if (r > 0) BF_TRY(launch_tsolve(d_task, 1, d_Z, d_perm, d_cols, d_T, d_skel, r, st));
    BF_TRY_CUDA(cudaDeviceSynchronize());
    *rank_out = r;
    BF_TRY_CUDA(cudaMemcpy(perm_out, d_perm, (size_t)n_src * sizeof(int32_t),
                           cudaMemcpyDeviceToHost));
    if (r > 0) {
      BF_TRY_CUDA(cudaMemcpy(skeleton_out, d_skel, (size_t)r * sizeof(int32_t),
                             cudaMemcpyDeviceToHost));
      BF_TRY_CUDA(cudaMemcpy(T_out, d_T, (size_t)r * n_src * sizeof(float2),
                             cudaMemcpyDeviceToHost));
    }
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_compress_block: host allocation failed");
    return BF_ENOMEM;
  } catch (...) {
    set_error("bf_compress_block: unexpected internal error");
    return BF_EINVAL;
  }
}
