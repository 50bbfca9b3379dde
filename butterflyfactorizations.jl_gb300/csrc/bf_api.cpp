// C ABI entry points of libbfgpu (declared in include/bfgpu.h).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include "bf_internal.h"

namespace bfg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_err; }

}  // namespace bfg

using namespace bfg;


#define BF_GUARD_BEGIN try {
#define BF_GUARD_END                                        \
  }                                                         \
  catch (const std::bad_alloc&) {                           \
    set_error("host allocation failed");                    \
    return BF_ENOMEM;                                       \
  }                                                         \
  catch (...) {                                             \
    set_error("unexpected internal error");                 \
    return BF_EINVAL;                                       \
  }

extern "C" {

int bf_version(void) { return 10000; }

const char* bf_status_string(int s) {
  switch (s) {
    case BF_OK: return "BF_OK";
    case BF_EINVAL: return "BF_EINVAL";
    case BF_ENOMEM: return "BF_ENOMEM";
    case BF_ECUDA: return "BF_ECUDA";
    case BF_ETIMEOUT: return "BF_ETIMEOUT";
    case BF_ENOTSUP: return "BF_ENOTSUP";
    case BF_ESTATE: return "BF_ESTATE";
    default: return "BF_UNKNOWN";
  }
}

const char* bf_last_error(void) { return last_error(); }

int bf_ctx_create(int device, bf_ctx_t* out) {
  BF_GUARD_BEGIN
  if (!out) {
    set_error("bf_ctx_create: out is NULL");
    return BF_EINVAL;
  }
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("bf_ctx_create: no CUDA device (%s)", cudaGetErrorString(e));
    return BF_ECUDA;
  }
  if (device < 0 || device >= n) {
    set_error("bf_ctx_create: device %d out of range (%d devices)", device, n);
    return BF_EINVAL;
  }
  auto* h = new bf_context;
  h->c.device = device;
  if (cudaGetDeviceProperties(&h->c.prop, device) != cudaSuccess ||
      cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("bf_ctx_create: cannot use device %d", device);
    return BF_ECUDA;
  }
  if (h->c.prop.major < 10) {
    set_error("bf_ctx_create: device %d is sm_%d%d; the library is compiled for sm_103a", device,
              h->c.prop.major, h->c.prop.minor);
    delete h;
    return BF_ECUDA;
  }
  *out = h;
  return BF_OK;
  BF_GUARD_END
}

int bf_ctx_destroy(bf_ctx_t ctx) {
  delete ctx;
  return BF_OK;
}

void bf_build_opts_default(bf_build_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->c_tau = 4.0;
  o->min_samples = 10;
  o->adaptive = 1;
  o->seed = 0;
  o->rank_mode = 0;
  o->keep_mixed = 1;
  o->surrogate_margin = 0.15;
  o->factor_storage = BF_STORE_C32;
  o->estimator = BF_EST_BUTTERFLY;
  o->geo_rmin = 3;
  o->geo_c = 1.5;
  o->geo_ceps = 1.5;
}

void bf_train_opts_default(bf_train_opts* o) {
  if (!o) return;
  o->epochs = 30;
  o->batch = 4096;
  o->lr = 3e-3f;
  o->beta1 = 0.9f;
  o->beta2 = 0.999f;
  o->eps = 1e-8f;
  o->seed = 0;
}

int bf_import_factors(bf_ctx_t ctx, const bf_factor_desc* d, bf_op_t* out) {
  BF_GUARD_BEGIN
  if (!ctx || !d || !out) {
    set_error("bf_import_factors: NULL argument");
    return BF_EINVAL;
  }
  *out = nullptr;
  if (d->n_blocks <= 0 || !d->bf || !d->stage || !d->obs_out || !d->src_out || !d->obs_in ||
      !d->src_in || !d->rows || !d->cols || !d->identity || !d->data_off || !d->obs_ptr ||
      !d->obs_idx || !d->src_ptr || !d->src_idx || d->n_rows <= 0 || d->n_cols <= 0) {
    set_error("bf_import_factors: incomplete descriptor");
    return BF_EINVAL;
  }
  auto* h = new bf_operator;
  Operator& op = h->op;
  op.ctx = &ctx->c;
  Logical& lg = op.logical;
  lg.n_rows = d->n_rows;
  lg.n_cols = d->n_cols;
  auto load_vm = [&](ValuesMap& vm, int64_t nn, const int64_t* ptr, const int64_t* idx,
                     int64_t npts) -> bool {
    vm.ptr.assign(ptr, ptr + nn + 1);
    if (vm.ptr[0] != 0) return false;
    for (int64_t i = 0; i < nn; ++i)
      if (vm.ptr[i + 1] < vm.ptr[i]) return false;
    vm.idx.assign(idx, idx + vm.ptr[nn]);
    for (int64_t v : vm.idx)
      if (v < 0 || v >= npts) return false;
    return true;
  };
  if (!load_vm(lg.obs_vals, d->n_obs_nodes, d->obs_ptr, d->obs_idx, d->n_rows) ||
      !load_vm(lg.src_vals, d->n_src_nodes, d->src_ptr, d->src_idx, d->n_cols)) {
    delete h;
    set_error("bf_import_factors: malformed node->values map");
    return BF_EINVAL;
  }
  int64_t raw_n = 0;
  int32_t nbf = 0;
  lg.blocks.resize(d->n_blocks);
  for (int64_t b = 0; b < d->n_blocks; ++b) {
    LBlock& k = lg.blocks[b];
    k.bf = d->bf[b];
    k.stage = d->stage[b];
    k.oo = d->obs_out[b];
    k.so = d->src_out[b];
    k.oi = d->obs_in[b];
    k.si = d->src_in[b];
    k.ident = d->identity[b] ? 1 : 0;
    k.rows = k.ident ? 0 : d->rows[b];
    k.cols = k.ident ? 0 : d->cols[b];
    k.raw_off = d->data_off[b];
    k.raw_ld = std::max(k.rows, 1);
    k.in_slot = k.out_slot = -1;  // wiring derived by pack_plan from the routing keys
    if (!k.ident) {
      if (k.rows < 0 || k.cols < 0 || k.raw_off < 0) {
        delete h;
        set_error("bf_import_factors: block %lld has invalid size/offset", (long long)b);
        return BF_EINVAL;
      }
      raw_n = std::max(raw_n, k.raw_off + (int64_t)k.rows * k.cols);
    }
    nbf = std::max(nbf, k.bf + 1);
  }
  lg.n_bf = nbf;
  if (raw_n > 0 && !d->data) {
    delete h;
    set_error("bf_import_factors: data is NULL");
    return BF_EINVAL;
  }
  int s = pack_plan(lg, op.plan, (int)sizeof(float4));  // FP64 data: float-float entries
  if (s != BF_OK) {
    delete h;
    return s;
  }
  if (cudaSetDevice(ctx->c.device) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("bf_import_factors: cudaSetDevice failed");
    return BF_ECUDA;
  }
  op.raw_is_double = 1;
  op.raw_entries = raw_n;
  if (cudaMalloc(&op.d_raw, (size_t)std::max<int64_t>(raw_n, 1) * 2 * sizeof(double)) !=
      cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("bf_import_factors: cannot allocate raw factor storage");
    return BF_ENOMEM;
  }
  if (raw_n > 0 && cudaMemcpy(op.d_raw, d->data, (size_t)raw_n * 2 * sizeof(double),
                              cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("bf_import_factors: upload failed");
    return BF_ECUDA;
  }
  s = upload_plan(op);
  if (s != BF_OK) {
    delete h;
    return s;
  }
  *out = h;
  return BF_OK;
  BF_GUARD_END
}

int bf_matvec(bf_op_t op, int trans, int64_t nrhs, const double* x, int64_t ldx, double* y,
              int64_t ldy, const double* alpha, const double* beta, int ptr_mode, void* stream) {
  BF_GUARD_BEGIN
  if (!op) {
    set_error("bf_matvec: NULL operator");
    return BF_EINVAL;
  }
  return run_matvec(op->op, trans, nrhs, x, ldx, y, ldy, alpha, beta, ptr_mode,
                    (cudaStream_t)stream);
  BF_GUARD_END
}

int bf_matvec_mixed(bf_op_t op, int trans, int64_t nrhs, const double* x, int64_t ldx, double* y,
                    int64_t ldy, const double* alpha, const double* beta, int ptr_mode,
                    void* stream) {
  BF_GUARD_BEGIN
  if (!op) {
    set_error("bf_matvec_mixed: NULL operator");
    return BF_EINVAL;
  }
  return run_matvec_mixed(op->op, trans, nrhs, x, ldx, y, ldy, alpha, beta, ptr_mode,
                          (cudaStream_t)stream);
  BF_GUARD_END
}

int bf_op_check(bf_op_t op, void* stream) {
  BF_GUARD_BEGIN
  if (!op) {
    set_error("bf_op_check: NULL operator");
    return BF_EINVAL;
  }
  Operator& o = op->op;
  BF_TRY_CUDA(cudaSetDevice(o.ctx->device));
  BF_TRY_CUDA(cudaStreamSynchronize(stream ? (cudaStream_t)stream : o.stream));
  return take_device_error(o, "bf_op_check");
  BF_GUARD_END
}

int bf_op_set_wait_limit(bf_op_t op, int64_t polls) {
  if (!op) {
    set_error("bf_op_set_wait_limit: NULL operator");
    return BF_EINVAL;
  }
  op->op.wait_limit = polls < 0 ? -1 : (long long)polls;
  return BF_OK;
}

int bf_op_profile_mixed(bf_op_t op, int trans, int32_t nrep, double* ms, int64_t* bytes,
                        double* flops, int64_t* kernels) {
  BF_GUARD_BEGIN
  if (!op) {
    set_error("bf_op_profile_mixed: NULL operator");
    return BF_EINVAL;
  }
  if (trans != BF_OP_N && trans != BF_OP_C && trans != BF_OP_T) {
    set_error("bf_op_profile_mixed: invalid trans %d", trans);
    return BF_EINVAL;
  }
  return profile_matvec_mixed(op->op, trans, nrep, ms, bytes, flops, kernels);
  BF_GUARD_END
}

int bf_op_mixed_info(bf_op_t op, int64_t* factor_bytes, int64_t* ws_bytes, int64_t* units) {
  BF_GUARD_BEGIN
  if (!op) {
    set_error("bf_op_mixed_info: NULL operator");
    return BF_EINVAL;
  }
  return mixed_info(op->op, factor_bytes, ws_bytes, units);
  BF_GUARD_END
}

int bf_op_size(bf_op_t op, int64_t* n_rows, int64_t* n_cols) {
  if (!op) {
    set_error("bf_op_size: NULL operator");
    return BF_EINVAL;
  }
  if (n_rows) *n_rows = op->op.plan.n_rows;
  if (n_cols) *n_cols = op->op.plan.n_cols;
  return BF_OK;
}

int bf_op_stats_get(bf_op_t op, bf_op_stats* st) {
  if (!op || !st) {
    set_error("bf_op_stats_get: NULL argument");
    return BF_EINVAL;
  }
  *st = op->op.stats;
  return BF_OK;
}

int bf_op_export_blocks(bf_op_t h, int64_t bf_begin, int64_t bf_end, int64_t* n_blocks,
                        int64_t* n_data, int32_t* bf, int32_t* stage, int64_t* obs_out,
                        int64_t* src_out, int64_t* obs_in, int64_t* src_in, int32_t* rows,
                        int32_t* cols, int8_t* identity, int64_t* data_off, void* data,
                        int32_t as_float32) {
  BF_GUARD_BEGIN
  if (!h || !n_blocks || !n_data) {
    set_error("bf_op_export_blocks: NULL argument");
    return BF_EINVAL;
  }
  Operator& op = h->op;
  const auto& B = op.logical.blocks;
  int64_t tot = 0, nb = 0;
  for (const auto& k : B) {
    if (k.bf < bf_begin || k.bf >= bf_end) continue;
    ++nb;
    if (!k.ident) tot += (int64_t)k.rows * k.cols;
  }
  *n_blocks = nb;
  *n_data = tot;
  if (!data) return BF_OK;
  if (!bf || !stage || !obs_out || !src_out || !obs_in || !src_in || !rows || !cols ||
      !identity || !data_off) {
    set_error("bf_op_export_blocks: NULL output array");
    return BF_EINVAL;
  }
  if (!op.d_A && !op.d_A2) {
    set_error("bf_op_export_blocks: operator has no factors");
    return BF_ESTATE;
  }
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  // one bulk copy of the packed task matrices, then a host-side gather per
  // block (complex FP32 entries are exact; float-float entries are summed)
  const bool f32 = op.d_A2 != nullptr;
  const size_t esz = f32 ? sizeof(float2) : sizeof(float4);
  std::vector<float> pk((size_t)op.plan.a_entries * esz / sizeof(float));
  if (!pk.empty())
    BF_TRY_CUDA(cudaMemcpy(pk.data(), f32 ? (const void*)op.d_A2 : (const void*)op.d_A,
                           pk.size() * sizeof(float), cudaMemcpyDeviceToHost));
  int64_t off = 0, ob = 0;
  for (size_t b = 0; b < B.size(); ++b) {
    const LBlock& k = B[b];
    if (k.bf < bf_begin || k.bf >= bf_end) continue;
    bf[ob] = k.bf;
    stage[ob] = k.stage;
    obs_out[ob] = k.oo;
    src_out[ob] = k.so;
    obs_in[ob] = k.oi;
    src_in[ob] = k.si;
    rows[ob] = k.rows;
    cols[ob] = k.cols;
    identity[ob] = k.ident;
    data_off[ob] = off;
    ++ob;
    if (k.ident || k.rows * (int64_t)k.cols == 0) continue;
    const int64_t pko = op.plan.blk_pk_off[b];
    const size_t pld = (size_t)op.plan.blk_pk_ld[b];
    if (pko < 0) {
      set_error("bf_op_export_blocks: block %zu has no packed entries", b);
      return BF_ESTATE;
    }
    size_t ncol = (size_t)k.cols, nrow = (size_t)k.rows;
    for (size_t e = 0; e < ncol * nrow; ++e) {
      size_t j = e / nrow, i = e - j * nrow;
      size_t src = (size_t)pko + j * pld + i;
      double re, im;
      if (f32) {
        const float* p = pk.data() + 2 * src;
        re = p[0];
        im = p[1];
      } else {
        const float* p = pk.data() + 4 * src;
        re = (double)p[0] + (double)p[1];
        im = (double)p[2] + (double)p[3];
      }
      if (as_float32) {
        ((float*)data)[2 * (off + e)] = (float)re;
        ((float*)data)[2 * (off + e) + 1] = (float)im;
      } else {
        ((double*)data)[2 * (off + e)] = re;
        ((double*)data)[2 * (off + e) + 1] = im;
      }
    }
    off += (int64_t)k.rows * k.cols;
  }
  return BF_OK;
  BF_GUARD_END
}

int bf_op_rank_log(bf_op_t h, int64_t* n_rec, double* rec) {
  if (!h || !n_rec) {
    set_error("bf_op_rank_log: NULL argument");
    return BF_EINVAL;
  }
  const auto& L = h->op.rank_log;
  *n_rec = (int64_t)L.size();
  if (!rec) return BF_OK;
  for (size_t i = 0; i < L.size(); ++i) {
    const auto& r = L[i];
    double* o = rec + BF_RANK_REC_LEN * i;
    o[0] = r.bf;
    o[1] = r.stage;
    o[2] = (double)r.obs_node;
    o[3] = (double)r.src_node;
    o[4] = r.n_obs;
    o[5] = r.n_cols;
    o[6] = r.rows0;
    o[7] = r.rows;
    o[8] = r.retries;
    o[9] = r.rank;
    o[10] = r.a_obs;
    o[11] = r.a_src;
    o[12] = r.dist;
    o[13] = r.k;
    for (int q = 0; q < 4; ++q) o[14 + q] = r.feat[q];
  }
  return BF_OK;
}

int bf_op_profile(bf_op_t h, int trans, int32_t nrep, double* ms_per_stage,
                  int64_t* bytes_per_stage, int64_t* kernels_per_matvec) {
  BF_GUARD_BEGIN
  if (!h) {
    set_error("bf_op_profile: NULL operator");
    return BF_EINVAL;
  }
  if (trans != BF_OP_N && trans != BF_OP_C && trans != BF_OP_T) {
    set_error("bf_op_profile: invalid trans");
    return BF_EINVAL;
  }
  return profile_matvec(h->op, trans, nrep, ms_per_stage, bytes_per_stage, kernels_per_matvec);
  BF_GUARD_END
}

int bf_op_task_shapes(bf_op_t h, int64_t* n_tasks, int32_t* stage, int32_t* kind, int32_t* M,
                      int32_t* n) {
  if (!h || !n_tasks) {
    set_error("bf_op_task_shapes: NULL argument");
    return BF_EINVAL;
  }
  const Plan& p = h->op.plan;
  *n_tasks = (int64_t)p.tasks.size();
  if (!stage) return BF_OK;
  if (!kind || !M || !n) {
    set_error("bf_op_task_shapes: NULL output array");
    return BF_EINVAL;
  }
  for (int64_t s = 0; s < p.n_stages(); ++s)
    for (int64_t t = p.stage_begin[s]; t < p.stage_begin[s + 1]; ++t) {
      stage[t] = (int32_t)s;
      kind[t] = p.tasks[t].kind;
      M[t] = p.tasks[t].M;
      n[t] = p.tasks[t].n;
    }
  return BF_OK;
}

int bf_op_destroy(bf_op_t op) {
  if (op) {
    cudaSetDevice(op->op.ctx->device);
    delete op;
  }
  return BF_OK;
}

}  // extern "C"
