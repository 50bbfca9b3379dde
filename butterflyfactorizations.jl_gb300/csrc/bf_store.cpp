// Persisted operators: bf_op_save / bf_op_load.
//
// The reference keeps its factors in memory only (ButterflyFactorization,
// src/ButterflyFactorization/bfstructs.jl:91-146, rebuilt by every
// assemble_BF call).  Here an operator is written once in its packed,
// device-ready form -- the level tasks, routing maps, launch lists, leaf
// orders and the packed factor array -- and loaded straight back onto a GPU,
// without the build or the packer.
//
// File layout (little-endian, 64-bit counts):
//   magic "BFGPUOP1", u32 format version, u32 byte-order mark 0x01020304,
//   u32 factor entry bytes (8 complex FP32, 16 float-float), u32 flags;
//   the plan's scalars, then its arrays and the logical blocks, each as
//   (u64 count, u64 element size, bytes); the operator statistics and rank
//   records; with flag 1, the near field's scalars, tasks, maps and lists;
//   then the factor array (u64 bytes, then chunks of FILE_CHUNK bytes, each
//   followed by its 64-bit hash), with flag 1 the near entries the same way;
//   finally the hash of everything before the factors and the end magic
//   "BFGPUEND".
// Loading checks the magic, version, byte order, every size against the
// bytes that remain, both kinds of hash, and every offset a kernel will
// follow (task matrices, routing maps, launch lists, leaf orders) before any
// of it reaches the GPU.
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "bf_internal.h"

namespace bfg {
namespace {

constexpr char MAGIC[8] = {'B', 'F', 'G', 'P', 'U', 'O', 'P', '1'};
constexpr char END_MAGIC[8] = {'B', 'F', 'G', 'P', 'U', 'E', 'N', 'D'};
constexpr uint32_t VERSION = 1;
constexpr uint32_t BOM = 0x01020304u;
constexpr size_t FILE_CHUNK = (size_t)256 << 20;

// 64-bit hash of a byte range, word by word (multiply-xorshift; the tail
// bytes are folded in one at a time)
uint64_t hash_bytes(const void* p, size_t n, uint64_t h) {
  const unsigned char* c = (const unsigned char*)p;
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, c + i, 8);
    h = (h ^ w) * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
  }
  for (; i < n; ++i) h = (h ^ c[i]) * 0x100000001B3ull;
  return h;
}

struct Writer {
  FILE* f = nullptr;
  uint64_t h = 0x243F6A8885A308D3ull;
  bool ok = true;
  void raw(const void* p, size_t n, bool hashed = true) {
    if (!ok || n == 0) return;
    if (std::fwrite(p, 1, n, f) != n) ok = false;
    if (hashed) h = hash_bytes(p, n, h);
  }
  template <typename T>
  void pod(const T& v) {
    raw(&v, sizeof(T));
  }
  template <typename T, typename A>
  void vec(const std::vector<T, A>& v) {
    const uint64_t n = v.size(), es = sizeof(T);
    pod(n);
    pod(es);
    raw(v.data(), n * sizeof(T));
  }
};

struct Reader {
  FILE* f = nullptr;
  uint64_t h = 0x243F6A8885A308D3ull;
  uint64_t left = 0;  // bytes not read yet
  bool ok = true;
  void raw(void* p, size_t n, bool hashed = true) {
    if (!ok) return;
    if (n > left || (n > 0 && std::fread(p, 1, n, f) != n)) {
      ok = false;
      return;
    }
    left -= n;
    if (hashed) h = hash_bytes(p, n, h);
  }
  template <typename T>
  void pod(T& v) {
    raw(&v, sizeof(T));
  }
  template <typename T, typename A>
  void vec(std::vector<T, A>& v) {
    uint64_t n = 0, es = 0;
    pod(n);
    pod(es);
    if (!ok || es != sizeof(T) || n > left / sizeof(T)) {
      ok = false;
      return;
    }
    v.resize(n);
    raw(v.data(), n * sizeof(T));
  }
};

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) std::fclose(f);
  }
};

// The scalars of a plan, laid out for the file.
struct PlanScalars {
  int64_t n_rows, n_cols, xg_off, yg_off, ws_entries, a_entries, alg_bytes_fwd, block_entries,
      max_rank;
  int32_t fac_bytes, n_bf, yg_covered, xg_covered;
};

struct OpScalars {
  int32_t raw_is_double, store_ff, lg_n_bf, pad;
  int64_t lg_n_rows, lg_n_cols;
};

struct NearScalars {
  int64_t n_fwd, a_entries, ny_off, nx_off, n_pairs, alg_bytes_fwd;
  int64_t list_begin[NearField::N_NCLASS + 1];
  int32_t fwd_covered, adj_covered;
};

constexpr uint32_t FLAG_NEAR = 1u;

int validate_near(const Operator& op) {
  const NearField& N = *op.near;
  const Plan& p = op.plan;
  auto bad = [](const char* what) {
    set_error("bf_op_load: inconsistent file (near field: %s)", what);
    return BF_EINVAL;
  };
  const int64_t nt = (int64_t)N.tasks.size(), nm = (int64_t)N.maps.size();
  if (N.n_fwd < 0 || N.n_fwd > nt || N.a_entries < 0) return bad("sizes");
  if (N.ny_off < 0 || N.ny_off + p.n_rows > p.ws_entries || N.nx_off < 0 ||
      N.nx_off + p.n_cols > p.ws_entries)
    return bad("regions");
  for (const DTask& t : N.tasks) {
    if (t.kind != TASK_DENSE || t.M < 0 || t.n < 0) return bad("task");
    if (t.rmap_off < 0 || t.rmap_off + t.M > nm || t.cmap_off < 0 || t.cmap_off + t.n > nm)
      return bad("task maps");
    if (t.a_off < 0 || t.a_off + (int64_t)t.M * t.n > N.a_entries) return bad("task matrix");
    if (t.rbase < -1 || (t.rbase >= 0 && (int64_t)t.rbase + t.M > p.ws_entries))
      return bad("task rows");
    if (t.cbase != -1) return bad("task columns");
  }
  for (int32_t v : N.maps)
    if (v < 0 || v >= p.ws_entries) return bad("routing map entry");
  if (N.pts.size() != N.maps.size()) return bad("point ids");
  // the kernels read x[pts[column]]: source points forward, observer points adjoint
  for (int64_t q = 0; q < nt; ++q) {
    const DTask& t = N.tasks[q];
    const int64_t lim = q < N.n_fwd ? p.n_cols : p.n_rows;
    for (int64_t j = 0; j < t.n; ++j) {
      const int32_t v = N.pts[t.cmap_off + j];
      if (v < 0 || v >= lim) return bad("point id");
    }
  }
  const int64_t nl = (int64_t)N.lists.size();
  if (N.list_begin[0] != 0 || N.list_begin[NearField::N_NCLASS] != nl) return bad("lists");
  for (int c = 0; c < NearField::N_NCLASS; ++c) {
    const int64_t b = N.list_begin[c], e = N.list_begin[c + 1];
    if (e < b || e > nl) return bad("list range");
    const bool tall = c == NearField::N_TALL_F || c == NearField::N_TALL_A;
    const bool adj = c == NearField::N_TALL_A || c == NearField::N_SMALL_A;
    // tall items are (task, row0) pairs read as int2: even start and length
    if (tall && (((e - b) & 1) || (b & 1))) return bad("tall list");
    for (int64_t q = b; q < e; ++q) {
      const int32_t v = N.lists[q];
      if (tall && ((q - b) & 1)) {
        if (v < 0) return bad("tall row");
        continue;
      }
      if (v < (adj ? N.n_fwd : 0) || v >= (adj ? nt : N.n_fwd)) return bad("list entry");
      // the small-task kernel walks the binary digits of M up to 32
      if (!tall && (N.tasks[v].M < 1 || N.tasks[v].M > 32)) return bad("small task rows");
    }
  }
  return BF_OK;
}

// every offset a kernel follows, against the sizes it indexes
int validate(const Operator& op) {
  const Plan& p = op.plan;
  const Logical& lg = op.logical;
  auto bad = [](const char* what) {
    set_error("bf_op_load: inconsistent file (%s)", what);
    return BF_EINVAL;
  };
  if (p.fac_bytes != 8 && p.fac_bytes != 16) return bad("factor entry size");
  if (p.n_rows <= 0 || p.n_cols <= 0 || p.ws_entries < 0 || p.a_entries < 0) return bad("sizes");
  if (p.ws_entries >= ((int64_t)1 << 31)) return bad("workspace size");
  const int64_t nt = (int64_t)p.tasks.size(), nm = (int64_t)p.maps.size();
  for (const DTask& t : p.tasks) {
    if (t.M < 0 || t.n < 0 || (t.kind != TASK_DENSE && t.kind != TASK_COPY)) return bad("task");
    const int64_t ncol = t.kind == TASK_COPY ? t.M : t.n;
    if (t.rmap_off < 0 || t.rmap_off + t.M > nm || t.cmap_off < 0 || t.cmap_off + ncol > nm)
      return bad("task maps");
    if (t.kind == TASK_DENSE && (t.a_off < 0 || t.a_off + (int64_t)t.M * t.n > p.a_entries))
      return bad("task matrix");
    if (t.cbase >= 0 && (int64_t)t.cbase + ncol > p.ws_entries) return bad("task columns");
    if (t.rbase >= 0 && (int64_t)t.rbase + t.M > p.ws_entries) return bad("task rows");
    if (t.cbase < -1 || t.rbase < -1) return bad("task bases");
  }
  for (int32_t v : p.maps)
    if (v < 0 || v >= p.ws_entries) return bad("routing map entry");
  const int64_t ns = p.n_stages();
  if (ns < 0 || p.stage_begin[0] != 0 || p.stage_begin.back() != nt) return bad("stages");
  for (int64_t s = 0; s < ns; ++s)
    if (p.stage_begin[s + 1] < p.stage_begin[s]) return bad("stage order");
  if ((int64_t)p.stage_bytes.size() != ns || (int64_t)p.stage_tma.size() != ns)
    return bad("stage arrays");
  const int64_t nl = (int64_t)p.lists.size();
  for (int c = 0; c < Plan::L_NCLASS; ++c) {
    const auto& b = p.list_begin[c];
    if ((int64_t)b.size() != ns + 1) return bad("launch list bounds");
    for (int64_t s = 0; s < ns; ++s) {
      if (b[s] < 0 || b[s + 1] < b[s] || b[s + 1] > nl) return bad("launch list range");
      // tall items are (task, row0) pairs read as int2: even start and length
      if (c == Plan::L_TALL && ((b[s] | (b[s + 1] - b[s])) & 1)) return bad("tall list");
      for (int64_t q = b[s]; q < b[s + 1]; ++q) {
        const bool row = c == Plan::L_TALL && ((q - b[s]) & 1);  // tall items: (task, row0)
        const int32_t v = p.lists[q];
        if (row) {
          if (v < 0) return bad("tall item row");
        } else if (v < 0 || v >= nt) {
          return bad("launch list entry");
        }
        // the bulk-copy pipeline reads every task input as one contiguous range
        if (!row && c == Plan::L_WIDE && p.stage_tma[s] && p.tasks[v].cbase < 0)
          return bad("bulk-copy task without contiguous inputs");
      }
    }
  }
  if ((int64_t)p.xperm.size() != p.n_cols || (int64_t)p.yperm.size() != p.n_rows)
    return bad("leaf orders");
  for (int32_t v : p.xperm)
    if (v < 0 || v >= p.n_cols) return bad("x leaf order");
  for (int32_t v : p.yperm)
    if (v < 0 || v >= p.n_rows) return bad("y leaf order");
  if (p.xg_off < 0 || p.xg_off + p.n_cols > p.ws_entries || p.yg_off < 0 ||
      p.yg_off + p.n_rows > p.ws_entries)
    return bad("vector regions");
  if (p.blk_pk_off.size() != lg.blocks.size() || p.blk_pk_ld.size() != lg.blocks.size())
    return bad("block offsets");
  for (size_t b = 0; b < lg.blocks.size(); ++b) {
    const LBlock& k = lg.blocks[b];
    if (k.ident || (int64_t)k.rows * k.cols == 0) continue;
    const int64_t o = p.blk_pk_off[b], ld = p.blk_pk_ld[b];
    if (o < 0 || ld < k.rows || o + (int64_t)(k.cols - 1) * ld + k.rows > p.a_entries)
      return bad("block entries");
  }
  return BF_OK;
}

}  // namespace
}  // namespace bfg

using namespace bfg;

extern "C" int bf_op_save(bf_op_t h, const char* path) {
  try {
    if (!h || !path) {
      set_error("bf_op_save: NULL argument");
      return BF_EINVAL;
    }
    Operator& op = h->op;
    const Plan& p = op.plan;
    const void* dA = op.d_A2 ? (const void*)op.d_A2 : (const void*)op.d_A;
    if (!dA) {
      set_error("bf_op_save: operator has no factors");
      return BF_ESTATE;
    }
    std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "wb"));
    if (!f) {
      set_error("bf_op_save: cannot open %s for writing", path);
      return BF_EINVAL;
    }
    Writer w;
    w.f = f.get();
    w.raw(MAGIC, 8);
    w.pod(VERSION);
    w.pod(BOM);
    const uint32_t fb = (uint32_t)p.fac_bytes, flags = op.near ? FLAG_NEAR : 0u;
    w.pod(fb);
    w.pod(flags);
    PlanScalars ps{p.n_rows, p.n_cols, p.xg_off, p.yg_off, p.ws_entries, p.a_entries,
                   p.alg_bytes_fwd, p.block_entries, p.max_rank, p.fac_bytes, p.n_bf,
                   p.yg_covered ? 1 : 0, p.xg_covered ? 1 : 0};
    w.pod(ps);
    w.vec(p.xperm);
    w.vec(p.yperm);
    w.vec(p.tasks);
    w.vec(p.stage_begin);
    w.vec(p.stage_bytes);
    w.vec(p.lists);
    for (int c = 0; c < Plan::L_NCLASS; ++c) w.vec(p.list_begin[c]);
    w.vec(p.stage_tma);
    w.vec(p.maps);
    w.vec(p.blk_pk_off);
    w.vec(p.blk_pk_ld);
    const Logical& lg = op.logical;
    OpScalars os{op.raw_is_double, op.store_ff, lg.n_bf, 0, lg.n_rows, lg.n_cols};
    w.pod(os);
    w.vec(lg.blocks);
    w.vec(lg.obs_vals.ptr);
    w.vec(lg.obs_vals.idx);
    w.vec(lg.src_vals.ptr);
    w.vec(lg.src_vals.idx);
    w.pod(op.stats);
    w.vec(op.rank_log);
    if (op.near) {
      const NearField& N = *op.near;
      NearScalars ns{N.n_fwd, N.a_entries, N.ny_off, N.nx_off, N.n_pairs, N.alg_bytes_fwd, {},
                     N.fwd_covered, N.adj_covered};
      for (int c = 0; c <= NearField::N_NCLASS; ++c) ns.list_begin[c] = N.list_begin[c];
      w.pod(ns);
      w.vec(N.tasks);
      w.vec(N.maps);
      w.vec(N.pts);
      w.vec(N.lists);
    }
    const uint64_t head_hash = w.h;
    // factors (and the near entries): device -> host in chunks, each with its own hash
    BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
    std::vector<unsigned char> buf;
    auto put = [&](const void* d, uint64_t bytes) -> int {
      w.raw(&bytes, 8, false);
      buf.resize((size_t)std::min<uint64_t>(std::max<uint64_t>(bytes, 1), FILE_CHUNK));
      for (uint64_t o = 0; o < bytes && w.ok; o += FILE_CHUNK) {
        const size_t n = (size_t)std::min<uint64_t>(FILE_CHUNK, bytes - o);
        BF_TRY_CUDA(cudaMemcpy(buf.data(), (const unsigned char*)d + o, n,
                               cudaMemcpyDeviceToHost));
        w.raw(buf.data(), n, false);
        const uint64_t ch = hash_bytes(buf.data(), n, 0x13198A2E03707344ull ^ o);
        w.raw(&ch, 8, false);
      }
      return BF_OK;
    };
    BF_TRY(put(dA, (uint64_t)p.a_entries * p.fac_bytes));
    if (op.near) BF_TRY(put(op.near->d_A, (uint64_t)op.near->a_entries * sizeof(double2)));
    w.raw(&head_hash, 8, false);
    w.raw(END_MAGIC, 8, false);
    if (!w.ok || std::fflush(f.get()) != 0) {
      set_error("bf_op_save: write to %s failed", path);
      return BF_EINVAL;
    }
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_op_save: host allocation failed");
    return BF_ENOMEM;
  }
}

extern "C" int bf_op_load(bf_ctx_t ctx, const char* path, bf_op_t* out) {
  try {
    if (!ctx || !path || !out) {
      set_error("bf_op_load: NULL argument");
      return BF_EINVAL;
    }
    *out = nullptr;
    std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "rb"));
    if (!f) {
      set_error("bf_op_load: cannot open %s", path);
      return BF_EINVAL;
    }
    Reader r;
    r.f = f.get();
    if (std::fseek(f.get(), 0, SEEK_END) != 0) {
      set_error("bf_op_load: cannot size %s", path);
      return BF_EINVAL;
    }
    const long sz = std::ftell(f.get());
    std::rewind(f.get());
    r.left = sz > 0 ? (uint64_t)sz : 0;
    char magic[8];
    uint32_t version = 0, bom = 0, fb = 0, flags = 0;
    r.raw(magic, 8);
    r.pod(version);
    r.pod(bom);
    r.pod(fb);
    r.pod(flags);
    if (!r.ok || std::memcmp(magic, MAGIC, 8) != 0) {
      set_error("bf_op_load: %s is not a saved operator", path);
      return BF_EINVAL;
    }
    if (version != VERSION || bom != BOM) {
      set_error("bf_op_load: %s has format version %u / byte order %08x; this library reads "
                "version %u, %08x", path, version, bom, VERSION, BOM);
      return BF_ENOTSUP;
    }
    auto h = std::make_unique<bf_operator>();
    Operator& op = h->op;
    op.ctx = &ctx->c;
    Plan& p = op.plan;
    PlanScalars ps{};
    r.pod(ps);
    p.n_rows = ps.n_rows;
    p.n_cols = ps.n_cols;
    p.xg_off = ps.xg_off;
    p.yg_off = ps.yg_off;
    p.ws_entries = ps.ws_entries;
    p.a_entries = ps.a_entries;
    p.alg_bytes_fwd = ps.alg_bytes_fwd;
    p.block_entries = ps.block_entries;
    p.max_rank = ps.max_rank;
    p.fac_bytes = ps.fac_bytes;
    p.n_bf = ps.n_bf;
    p.yg_covered = ps.yg_covered != 0;
    p.xg_covered = ps.xg_covered != 0;
    r.vec(p.xperm);
    r.vec(p.yperm);
    r.vec(p.tasks);
    r.vec(p.stage_begin);
    r.vec(p.stage_bytes);
    r.vec(p.lists);
    for (int c = 0; c < Plan::L_NCLASS; ++c) r.vec(p.list_begin[c]);
    r.vec(p.stage_tma);
    r.vec(p.maps);
    r.vec(p.blk_pk_off);
    r.vec(p.blk_pk_ld);
    Logical& lg = op.logical;
    OpScalars os{};
    r.pod(os);
    op.raw_is_double = os.raw_is_double;
    op.store_ff = os.store_ff;
    lg.n_bf = os.lg_n_bf;
    lg.n_rows = os.lg_n_rows;
    lg.n_cols = os.lg_n_cols;
    r.vec(lg.blocks);
    r.vec(lg.obs_vals.ptr);
    r.vec(lg.obs_vals.idx);
    r.vec(lg.src_vals.ptr);
    r.vec(lg.src_vals.idx);
    r.pod(op.stats);
    r.vec(op.rank_log);
    if (flags & ~FLAG_NEAR) {
      set_error("bf_op_load: %s uses features this library does not know (flags %08x)", path,
                flags);
      return BF_ENOTSUP;
    }
    if (flags & FLAG_NEAR) {
      op.near = new NearField;
      NearField& N = *op.near;
      NearScalars ns{};
      r.pod(ns);
      N.n_fwd = ns.n_fwd;
      N.a_entries = ns.a_entries;
      N.ny_off = ns.ny_off;
      N.nx_off = ns.nx_off;
      N.n_pairs = ns.n_pairs;
      N.alg_bytes_fwd = ns.alg_bytes_fwd;
      for (int c = 0; c <= NearField::N_NCLASS; ++c) N.list_begin[c] = ns.list_begin[c];
      N.fwd_covered = ns.fwd_covered;
      N.adj_covered = ns.adj_covered;
      r.vec(N.tasks);
      r.vec(N.maps);
      r.vec(N.pts);
      r.vec(N.lists);
    }
    const uint64_t head_hash = r.h;
    uint64_t fbytes = 0;
    r.raw(&fbytes, 8, false);
    if (!r.ok || (uint32_t)p.fac_bytes != fb || p.stage_begin.empty() ||
        fbytes != (uint64_t)p.a_entries * p.fac_bytes) {
      set_error("bf_op_load: %s is truncated or inconsistent", path);
      return BF_EINVAL;
    }
    const uint64_t nbytes = op.near ? (uint64_t)op.near->a_entries * sizeof(double2) : 0;
    if (op.near && (op.near->a_entries < 0 || nbytes / sizeof(double2) != (uint64_t)op.near->a_entries)) {
      set_error("bf_op_load: %s is inconsistent (near field size)", path);
      return BF_EINVAL;
    }
    auto chunked = [](uint64_t b) { return b + 8 * ((b + FILE_CHUNK - 1) / FILE_CHUNK); };
    const uint64_t expect = chunked(fbytes) + (op.near ? 8 + chunked(nbytes) : 0) + 16;
    if (r.left != expect) {
      set_error("bf_op_load: %s has %llu bytes after the tables, expected %llu", path,
                (unsigned long long)r.left, (unsigned long long)expect);
      return BF_EINVAL;
    }
    BF_TRY(validate(op));
    if (op.near) BF_TRY(validate_near(op));
    // factors: host -> device in chunks, each checked against its hash
    BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
    const bool f32 = p.fac_bytes == 8;
    void* dA = nullptr;
    if (cudaMalloc(&dA, (size_t)fbytes + 2 * (size_t)p.fac_bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("bf_op_load: cannot allocate %llu bytes of factors", (unsigned long long)fbytes);
      return BF_ENOMEM;
    }
    if (f32)
      op.d_A2 = (float2*)dA;
    else
      op.d_A = (float4*)dA;
    // the two entries of tail padding the bulk copies may read
    BF_TRY_CUDA(cudaMemset((unsigned char*)dA + fbytes, 0, 2 * (size_t)p.fac_bytes));
    std::vector<unsigned char> buf;
    auto get = [&](void* d, uint64_t bytes) -> int {
      buf.resize((size_t)std::min<uint64_t>(std::max<uint64_t>(bytes, 1), FILE_CHUNK));
      for (uint64_t o = 0; o < bytes; o += FILE_CHUNK) {
        const size_t n = (size_t)std::min<uint64_t>(FILE_CHUNK, bytes - o);
        uint64_t ch = 0;
        r.raw(buf.data(), n, false);
        r.raw(&ch, 8, false);
        if (!r.ok || ch != hash_bytes(buf.data(), n, 0x13198A2E03707344ull ^ o)) {
          set_error("bf_op_load: factor bytes %llu.. of %s fail their check",
                    (unsigned long long)o, path);
          return BF_EINVAL;
        }
        BF_TRY_CUDA(cudaMemcpy((unsigned char*)d + o, buf.data(), n, cudaMemcpyHostToDevice));
      }
      return BF_OK;
    };
    BF_TRY(get(dA, fbytes));
    if (op.near) {
      uint64_t nb = 0;
      r.raw(&nb, 8, false);
      if (!r.ok || nb != nbytes) {
        set_error("bf_op_load: %s is inconsistent (near entries)", path);
        return BF_EINVAL;
      }
      if (cudaMalloc((void**)&op.near->d_A, std::max<uint64_t>(nbytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        set_error("bf_op_load: cannot allocate the near field");
        return BF_ENOMEM;
      }
      BF_TRY(get((void*)op.near->d_A, nbytes));
    }
    uint64_t hh = 0;
    char endm[8];
    r.raw(&hh, 8, false);
    r.raw(endm, 8, false);
    if (!r.ok || hh != head_hash || std::memcmp(endm, END_MAGIC, 8) != 0) {
      set_error("bf_op_load: the tables of %s fail their check", path);
      return BF_EINVAL;
    }
    BF_TRY(upload_tables(op));
    if (op.near) BF_TRY(near_upload(*op.near));
    *out = h.release();
    return BF_OK;
  } catch (const std::bad_alloc&) {
    set_error("bf_op_load: host allocation failed (corrupt sizes?)");
    return BF_ENOMEM;
  } catch (const std::length_error&) {
    set_error("bf_op_load: corrupt sizes");
    return BF_EINVAL;
  }
}
