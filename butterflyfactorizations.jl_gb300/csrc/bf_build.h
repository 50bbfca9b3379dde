// Device-side construction interface (kernels in bf_build.cu).
#pragma once

#include "bf_internal.h"

namespace bfg {

constexpr int QR_NT = 128;
constexpr int QR_MAX_SMEM = 220 * 1024;
constexpr int TS_MAX_SMEM_R = 120;

// One compression (PartialQR call) of one round of sampling.
struct alignas(16) CTask {
  long long z_off;     // sampled block in the Z batch (float2, column-major, ld n_rows)
  long long rows_off;  // sampled observer point ids in the row pool
  long long cols_off;  // source point ids (src_index) in the column pool
  long long obs_begin; // values(obs_node) = obs_perm[obs_begin .. obs_begin + n_obs)
  long long perm_off;  // column permutation output
  long long t_off;     // interpolation matrix / dense block in the raw store
  long long skel_off;  // skeleton output
  unsigned long long key;
  double eps;
  int n_obs, n_rows, n_cols, rank;
};
static_assert(sizeof(CTask) == 96, "CTask layout");

int launch_rows(const CTask* d_tasks, int ntasks, const int32_t* d_obs_perm, int32_t* d_rowpool,
                cudaStream_t st);
int launch_eval(const CTask* d_tasks, int ntasks, const double* d_obs, const double* d_src,
                const int32_t* d_rowpool, const int32_t* d_colpool, float2* d_out, double k,
                int mode, cudaStream_t st);
size_t qr_smem_bytes(int n, int m, bool with_z);
int launch_qr(CTask* d_tasks, int ntasks, float2* d_Z, int32_t* d_permpool, bool smem_z,
              size_t smem, cudaStream_t st);
int launch_tsolve(const CTask* d_tasks, int ntasks, const float2* d_Z, const int32_t* d_permpool,
                  const int32_t* d_colpool, float2* d_raw, int32_t* d_skel, int max_rank,
                  cudaStream_t st);

// ranks[i] = tasks[i].rank (only the ranks travel back to the host)
int launch_ranks(const CTask* d_tasks, int ntasks, int32_t* d_ranks, cudaStream_t st);

// A finished compression: its index in the round and its output offsets.
struct CDone {
  long long q, t_off, skel_off;
};
// out[i] = tasks[done[i].q] with the offsets of done[i] (out must not alias tasks)
int launch_compact_done(const CTask* d_tasks, const CDone* d_done, int ndone, CTask* d_out,
                        cudaStream_t st);

}  // namespace bfg
