// Internal declarations of libbfgpu (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bfgpu.h"

namespace bfg {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
const char* last_error();

#define BF_TRY_CUDA(call)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      bfg::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                     __LINE__);                                                        \
      return BF_ECUDA;                                                                 \
    }                                                                                  \
  } while (0)

#define BF_TRY(call)              \
  do {                            \
    int s_ = (call);              \
    if (s_ != BF_OK) return s_;   \
  } while (0)

// A CUDA set-up call (a kernel attribute such as its dynamic shared-memory
// limit) made once per device: cudaFuncSetAttribute applies to the current
// device only, so a flag per process would leave a second device without it.
// Safe to race: two threads may both make the (idempotent) call once.
struct DeviceOnce {
  std::atomic<uint64_t> done{0};
  template <typename F>
  int run(F f, const char* what) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("%s: cudaGetDevice failed: %s", what, cudaGetErrorString(e));
      return BF_ECUDA;
    }
    const uint64_t bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return BF_OK;
    e = f();
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("%s: %s", what, cudaGetErrorString(e));
      return BF_ECUDA;
    }
    if (bit) done.fetch_or(bit, std::memory_order_release);
    return BF_OK;
  }
};

// Open-addressing hash map from a 128-bit key (two uint64) to V, linear
// probing, no erase: the host bookkeeping of the builder and the packer
// inserts millions of keys, where node-based maps spend most of their time in
// allocation and pointer chasing.
template <typename V>
struct FlatMap {
  std::vector<uint64_t> khi, klo;
  std::vector<V> val;
  std::vector<uint8_t> used;
  uint64_t mask = 0;
  size_t count = 0;
  static uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  void reserve(size_t n) {
    size_t cap = 16;
    while (cap < 2 * n + 16) cap <<= 1;
    if (cap <= used.size()) return;
    FlatMap<V> t;
    t.khi.assign(cap, 0);
    t.klo.assign(cap, 0);
    t.val.assign(cap, V());
    t.used.assign(cap, 0);
    t.mask = cap - 1;
    for (size_t i = 0; i < used.size(); ++i)
      if (used[i]) t.put(khi[i], klo[i], val[i]);
    *this = std::move(t);
  }
  size_t slot(uint64_t hi, uint64_t lo) const {
    size_t i = (size_t)(mix(hi ^ mix(lo)) & mask);
    while (used[i] && (khi[i] != hi || klo[i] != lo)) i = (i + 1) & mask;
    return i;
  }
  V* find(uint64_t hi, uint64_t lo) {
    if (used.empty()) return nullptr;
    size_t i = slot(hi, lo);
    return used[i] ? &val[i] : nullptr;
  }
  const V& at(uint64_t hi, uint64_t lo) const {
    size_t i = used.empty() ? 0 : slot(hi, lo);
    if (used.empty() || !used[i]) throw std::out_of_range("FlatMap::at");
    return val[i];
  }
  void put(uint64_t hi, uint64_t lo, const V& v) {
    if (2 * (count + 1) > used.size()) reserve(count + 1);
    size_t i = slot(hi, lo);
    if (!used[i]) {
      used[i] = 1;
      khi[i] = hi;
      klo[i] = lo;
      ++count;
    }
    val[i] = v;
  }
};

// Host phase timings, printed to stderr when BFGPU_TIMING is set.
struct PhaseLog {
  bool on;
  std::chrono::steady_clock::time_point t;
  PhaseLog() : on(std::getenv("BFGPU_TIMING") != nullptr), t(std::chrono::steady_clock::now()) {}
  void mark(const char* what) {
    if (!on) return;
    auto n = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[bfgpu] %-32s %8.3f s\n", what,
                 std::chrono::duration<double>(n - t).count());
    t = n;
  }
};

// ---------------------------------------------------------------- trees
struct Tree {
  int64_t n_points = 0;
  std::vector<double> center;  // 3 * n_nodes
  std::vector<double> half;
  std::vector<int32_t> level, parent, first_child, n_child;
  std::vector<int64_t> begin, end, perm;
  int64_t nn() const { return (int64_t)half.size(); }
  bool isleaf(int64_t n) const { return n_child[n] == 0; }
  int64_t nvals(int64_t n) const { return end[n] - begin[n]; }
  const int64_t* vals(int64_t n) const { return perm.data() + begin[n]; }
  double radius(int64_t n) const;
  int32_t depth() const;
};

int tree_build(const double* xyz, int64_t n, int32_t max_points, int32_t max_depth, Tree& t);
// BFS levels below root with shallow leaves pushed down (src/auxillaries.jl:263-350).
std::vector<std::vector<int64_t>> traverse_and_pad(const Tree& t, int64_t root);
bool is_far(const Tree& ts, const Tree& to, int64_t snode, int64_t onode, double alpha);
// far and near pairs of the dual-tree traversal (src/Matrixassembly/intlists.jl:30-217)
void near_far_lists(const Tree& to, const Tree& ts, double alpha, int32_t minbflvl,
                    int32_t leafcomp, int32_t leafimbalance, int32_t unbalancedints,
                    std::vector<std::pair<int64_t, int64_t>>* far,
                    std::vector<std::pair<int64_t, int64_t>>* near, int64_t* n_far,
                    int64_t* n_near);

// ---------------------------------------------------------------- logical factors
// One reference ButterflyBlock (bfstructs.jl:21-29) whose matrix lives in a raw
// device array (column-major, leading dimension raw_ld).
// A plain struct (no member initialisers): every producer sets every field,
// and vectors of blocks are grown without a serial initialisation pass.
struct LBlock {
  int32_t bf;
  int32_t stage;  // 0 = Q, l = R level l, -1 = P
  int64_t oo, so, oi, si;
  int32_t rows, cols;
  int8_t ident;
  int64_t raw_off;
  int32_t raw_ld;
  // slot ids when the producer already knows the wiring (the GPU build);
  // -1: derived by pack_plan from the routing keys
  int64_t in_slot, out_slot;
};

// Allocator whose value-less construct() default-initialises: resize() of a
// vector of plain structs then leaves the new elements for the caller (and the
// first touch of their pages to the threads that fill them).
template <typename T>
struct DefaultInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = DefaultInitAlloc<U>;
  };
  DefaultInitAlloc() = default;
  template <typename U>
  DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
  template <typename U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
};
using BlockVec = std::vector<LBlock, DefaultInitAlloc<LBlock>>;

// node -> values map (CSR), 0-based point indices
struct ValuesMap {
  std::vector<int64_t> ptr, idx;
  int64_t n(int64_t node) const { return ptr[node + 1] - ptr[node]; }
  const int64_t* v(int64_t node) const { return idx.data() + ptr[node]; }
};

struct Logical {
  int64_t n_rows = 0, n_cols = 0;
  int32_t n_bf = 0;
  BlockVec blocks;
  ValuesMap obs_vals, src_vals;
  // with slot ids in the blocks: the length of every slot (else empty)
  std::vector<int64_t> slot_len;
};

// ---------------------------------------------------------------- packed plan
enum : int32_t { TASK_DENSE = 0, TASK_COPY = 1 };

// task shape classes of the forward kernels
constexpr int TALL_ROWS = 64;   // rows per tall-kernel panel
constexpr int TALL_PANELS = 1;  // panels per tall-kernel warp item
constexpr int WIDE_NMIN = 128;  // wide class: M <= 32, n > 2M and n >= WIDE_NMIN
constexpr int ADJ_TALL_M = 128; // adjoint: tasks with more rows get a CTA each
constexpr int FLAT_MMAX = 128;  // flat kernel: 32 < M <= FLAT_MMAX
constexpr int FLAT_NMAX = 256;  //              n <= FLAT_NMAX

// Device task descriptor: row side = rmap[0..M), column side = cmap[0..n);
// forward computes ws[rmap] = A * ws[cmap]; adjoint ws[cmap] = A^H * ws[rmap].
struct alignas(16) DTask {
  long long a_off;     // first complex entry of the M x n column-major matrix
  long long rmap_off;  // offset into the routing array
  long long cmap_off;
  int M, n, kind;
  int cbase;  // workspace offset of column j is cbase + j (contiguous), else -1
  int rbase;  // same for the rows
  int pad;
};
static_assert(sizeof(DTask) == 48, "DTask layout");

// Copy of one logical block into a task matrix (repack on the device).
struct alignas(16) DSeg {
  long long src_off;  // raw array offset (complex entries)
  long long dst_off;  // packed matrix offset of the block's (0,0) entry
  int src_ld, dst_ld, rows, cols;
  int kind;  // 0 = copy, 1 = identity
  int pad[3];
};
static_assert(sizeof(DSeg) == 48, "DSeg layout");

struct Plan {
  int64_t n_rows = 0, n_cols = 0;
  int64_t xg_off = 0, yg_off = 0;  // x-space and y-space regions of the workspace
  // the x / y regions hold points in leaf order: region entry q is point xperm[q]
  // (yperm[q]), so every leaf's values are one contiguous range
  std::vector<int32_t> xperm, yperm;
  int64_t ws_entries = 0;
  std::vector<DTask> tasks;
  std::vector<int64_t> stage_begin;  // n_stages + 1
  std::vector<int64_t> stage_bytes;  // algorithmic bytes of each level launch
  // forward launch lists (one per task shape class, see bf_matvec.cu), all
  // concatenated in `lists`; begin[c][s] indexes class c at stage s (in
  // entries; tall items are (task, row0) pairs and count two entries each)
  // L_ATALL / L_AWARP: adjoint CTA-per-task (M > ADJ_TALL_M) and warp-per-task
  // lists (the adjoint shares L_WIDE and L_COPY with the forward)
  enum { L_TALL = 0, L_FLAT, L_SMALL, L_WIDE, L_COPY, L_DENSE, L_ATALL, L_AWARP, L_NCLASS };
  std::vector<int32_t> lists;
  std::vector<int64_t> list_begin[L_NCLASS];  // n_stages + 1 each
  // stage s can use the bulk-copy pipeline (every dense task input contiguous)
  std::vector<uint8_t> stage_tma;
  std::vector<int32_t> maps;
  int64_t a_entries = 0;
  int fac_bytes = 16;  // bytes per packed factor entry: 16 float-float, 8 complex FP32
  std::vector<DSeg> segs;
  // per logical block: offset and leading dimension of its entries inside the
  // packed task matrices (-1: identity / empty), used by bf_op_export_blocks
  std::vector<int64_t> blk_pk_off;
  std::vector<int32_t> blk_pk_ld;
  bool yg_covered = false, xg_covered = false;
  int64_t alg_bytes_fwd = 0;
  int64_t block_entries = 0;
  int64_t max_rank = 0;
  int32_t n_bf = 0;
  int64_t n_stages() const { return (int64_t)stage_begin.size() - 1; }
};

int pack_plan(const Logical& lg, Plan& plan, int fac_bytes);

// ---------------------------------------------------------------- near field
// The near-field block-sparse part of PetrovGalerkinBF (assembled at
// src/Matrixassembly/petrovgalerkinbf.jl:57-119, applied at
// src/matrixalgebra/matrixvector.jl:28-33), as dense tasks in the layout of
// the far-field levels: tasks [0, n_fwd) are one per observer leaf (rows: its
// points, written to the near-y workspace region; columns: the points of every
// source node near the leaf or one of its ancestors, read from the x region);
// tasks [n_fwd, end) are one per source leaf with the transposed blocks (rows
// written to the near-x region, columns read from the y region), so each
// direction has exactly one writer per output entry.
struct NearField {
  std::vector<DTask> tasks;
  int64_t n_fwd = 0;
  std::vector<int32_t> maps;  // routing entries (workspace entries)
  // point ids, indexed like maps: the kernels read a column's input x[pts[j]]
  // in FP64 straight from the caller's vector
  std::vector<int32_t> pts;
  // launch lists: tall row panels ((task, row0) pairs, read as int2: both
  // tall lists come first, so they start at even offsets) and small tasks
  // (M <= 32), forward and adjoint; list_begin[c] .. list_begin[c + 1]
  enum { N_TALL_F = 0, N_TALL_A, N_SMALL_F, N_SMALL_A, N_NCLASS };
  std::vector<int32_t> lists;
  int64_t list_begin[N_NCLASS + 1] = {};
  int64_t a_entries = 0;      // complex FP64 entries, both directions
  int64_t ny_off = 0, nx_off = 0;
  int32_t fwd_covered = 0, adj_covered = 0;
  int64_t n_pairs = 0;
  int64_t alg_bytes_fwd = 0;  // bytes of one forward near product
  double2* d_A = nullptr;
  DTask* d_tasks = nullptr;
  int32_t* d_maps = nullptr;
  int32_t* d_pts = nullptr;
  int32_t* d_lists = nullptr;
};
void near_free(NearField* nf);
int near_upload(NearField& nf);  // tasks, maps, lists (the entries are uploaded by their producer)
// near-field launches of one matvec: inputs from x (device, the caller's
// vector: n_cols entries forward, n_rows adjoint), results into ws's near region
int near_stage(const struct Operator& op, int trans, cudaStream_t st, const double2* x,
               float4* ws, int64_t* nk);
// y_c += alpha * near(op) x_c for nrhs columns (device pointers), through op's workspace
int near_apply_columns(struct Operator& op, int trans, int64_t nrhs, const double2* x,
                       int64_t lx, double2* y, int64_t ly, double2 alpha, cudaStream_t st);

// ---------------------------------------------------------------- device-side
struct Context {
  int device = 0;
  cudaDeviceProp prop{};
};

}  // namespace bfg
struct bf_batch;  // bf_batch.cu
namespace bfg {

// Operator batches (bf_batch.cu), also used by bf_matvec for chunks of
// MRHS_CHUNK right-hand sides of one operator
constexpr int MRHS_CHUNK = 8;
int batch_create(Context* ctx, struct Operator* const* ops, const int32_t* trans,
                 const int32_t* nrhs, int32_t n_ops, int32_t rhs_chunk, bf_batch** out);
void batch_destroy(bf_batch* b);
int batch_buffers(bf_batch* b, int op, double2** x, double2** y);
int batch_launch(bf_batch* b, cudaStream_t st);

struct Operator {
  Context* ctx = nullptr;
  cudaStream_t stream = nullptr;
  Plan plan;
  Logical logical;
  int raw_is_double = 1;
  void* d_raw = nullptr;  // raw logical block data (double2 or float2); freed after packing
  int64_t raw_entries = 0;
  // plain (FP64-accurate) operator: packed task matrices, float-float entries
  // (d_A, from FP64 factors) or complex FP32 entries (d_A2, from the GPU
  // build, whose factors are FP32 values); exactly one is set
  float4* d_A = nullptr;
  float2* d_A2 = nullptr;
  DTask* d_tasks = nullptr;
  int32_t* d_maps = nullptr;
  float4* d_ws = nullptr;
  int32_t* d_lists = nullptr;  // forward launch lists (Plan::lists)
  int32_t* d_xperm = nullptr;  // leaf order of the x / y regions (Plan::xperm, yperm)
  int32_t* d_yperm = nullptr;
  int* d_err = nullptr;        // device error word of bounded waits (0 = ok)
  // host-visible copy of d_err (pinned, mapped): the last kernel of every
  // plain matvec moves a non-zero d_err here and clears d_err, so that an
  // asynchronous call's timeout is seen by the host after the stream has
  // drained (bf_op_check, or the next call on the handle)
  int* h_err = nullptr;
  int* h_err_dev = nullptr;    // device address of h_err
  long long wait_limit = -1;   // polls of a bounded wait; < 0: the default (about 1 s)
  int store_ff = 0;            // GPU-built factors widened to float-float (16 B) storage
  // one-operator batches of MRHS_CHUNK columns per direction (N, C, T), made at
  // the first bf_matvec call with that many right-hand sides; 1 in mrhs_off:
  // the batch could not be made (its memory), columns run one by one
  bf_batch* mrhs[3] = {nullptr, nullptr, nullptr};
  int mrhs_off[3] = {0, 0, 0};
  // staging of host right-hand sides
  double* d_x = nullptr;
  double* d_y = nullptr;
  int64_t stage_cap = 0;
  // mixed path
  void* mixed = nullptr;
  // near field (bf_op_add_near), or none
  NearField* near = nullptr;
  bf_op_stats stats{};
  // per-compression rank records of the build (surrogate training data)
  struct RankRec {
    int32_t bf, stage;
    int64_t obs_node, src_node;
    int32_t n_obs, n_cols, rows0, rows, retries, rank;
    float a_obs, a_src, dist, k;
    float feat[4];  // rank-surrogate features (bf_surrogate.h)
  };
  std::vector<RankRec> rank_log;
  ~Operator();
};

int upload_plan(Operator& op);  // repacks d_raw into d_A, uploads tasks/maps, allocates ws
int upload_tables(Operator& op);  // the plan without the factors (tasks, maps, lists, ws, ...)
int build_operator(Context* ctx, const double* obs_xyz, int64_t n_obs, const double* src_xyz,
                   int64_t n_src, const Tree& to, const Tree& ts, const int64_t* far_obs,
                   const int64_t* far_src, int64_t n_far, double k, double tol,
                   const bf_build_opts& opts, Operator& op);
int profile_matvec(Operator& op, int trans, int nrep, double* ms, int64_t* bytes,
                   int64_t* kernels);
// The launchers take both factor pointers; the non-null one selects the
// float-float (d_A) or complex FP32 (d_A2) instantiation.
int launch_fwd_tma(const int32_t* d_tlist, int n_tasks, const DTask* d_tasks, const float4* d_A,
                   const float2* d_A2, const int32_t* d_maps, float4* d_ws, int* d_err,
                   long long wait_limit, int n_sm, cudaStream_t st);
// Takes (and clears) the host-visible error word of the plain path: BF_OK, or
// BF_ETIMEOUT with the message set.  Reads host memory only (no CUDA call).
int take_device_error(Operator& op, const char* what);
// adjoint (conj) / transpose launches of level s; returns the kernel count or -1
int launch_adj_stage(const Plan& p, int64_t s, bool conj, const int32_t* d_lists,
                     const DTask* d_tasks, const float4* d_A, const float2* d_A2,
                     const int32_t* d_maps, float4* d_ws, cudaStream_t st);
int run_matvec(Operator& op, int trans, int64_t nrhs, const double* x, int64_t ldx, double* y,
               int64_t ldy, const double* alpha, const double* beta, int ptr_mode,
               cudaStream_t stream);

// many-RHS tensor-core path (bf_mixed.cu); its state hangs off Operator::mixed
void mixed_free(void* p);
int run_matvec_mixed(Operator& op, int trans, int64_t nrhs, const double* x, int64_t ldx,
                     double* y, int64_t ldy, const double* alpha, const double* beta,
                     int ptr_mode, cudaStream_t stream);
int profile_matvec_mixed(Operator& op, int trans, int nrep, double* ms, int64_t* bytes,
                         double* flops, int64_t* kernels);
int mixed_info(Operator& op, int64_t* factor_bytes, int64_t* ws_bytes, int64_t* units);

}  // namespace bfg

// opaque C-ABI handles
struct bf_tree {
  bfg::Tree t;
};
struct bf_context {
  bfg::Context c;
};
struct bf_operator {
  bfg::Operator op;
};
