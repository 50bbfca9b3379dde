/*
 * bfref_c.c -- plain-C restatement of the reference far-field matvec
 * (test infrastructure and timed CPU baseline; the GPU library never links it).
 *
 * Follows, on factors given in the reference block layout (the same arrays as
 * bf_factor_desc in include/bfgpu.h):
 *   - pointer wiring of ButterflyFactorization, one map per level
 *     (src/ButterflyFactorization/bfstructs.jl:99-146);
 *   - the flat-array matvec (src/Butterflyalgebra/bfvector.jl:200-296):
 *     Q gather + GEMV, R levels zeroed then accumulated (identity blocks add
 *     their input), P GEMV + scatter-add;
 *   - the global far-field driver (src/matrixalgebra/matrixvector.jl:39-62):
 *     a static thread schedule over far blocks, one private y buffer per
 *     thread, then a serial reduction y += alpha * buf.
 * Arithmetic is ComplexF64 throughout (the reference's acctype).
 * Parity status: parity unpinned (no Julia available to run the reference).
 */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double re, im;
} cplx;

typedef struct {
  int64_t data;    /* offset (complex entries) of the block matrix, -1 = identity */
  int32_t rows, cols;
  int64_t in_ptr;  /* slot offset in the BF workspace, or source node (Q gather) */
  int64_t out_ptr; /* slot offset, or observer node (P scatter) */
} rblock;

typedef struct {
  int64_t q0, q1, r0, r1, p0, p1; /* block ranges in the plan */
  int64_t* lvl;                   /* n_lvl + 1 offsets of R levels (absolute) */
  int32_t n_lvl;
  int64_t ws_len;
} rbf;

typedef struct {
  int64_t n_rows, n_cols, n_bf, max_ws, max_dim;
  rblock* blk;
  rbf* bf;
  const double* data; /* ComplexF64 interleaved */
  const int64_t *optr, *oidx, *sptr, *sidx;
} rplan;

typedef struct {
  int64_t k[4];
  int64_t off, len;
  int used;
} hent;

static uint64_t hmix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static hent* hfind(hent* t, size_t cap, const int64_t k[4]) {
  uint64_t h = hmix((uint64_t)k[0]) ^ hmix((uint64_t)k[1] + 7) ^ hmix((uint64_t)k[2] * 31) ^
               hmix((uint64_t)k[3] * 131 + 3);
  size_t i = (size_t)(h & (cap - 1));
  while (t[i].used && memcmp(t[i].k, k, sizeof(int64_t) * 4) != 0) i = (i + 1) & (cap - 1);
  return &t[i];
}

void bfref_plan_destroy(void* p) {
  rplan* P = (rplan*)p;
  if (!P) return;
  if (P->bf)
    for (int64_t f = 0; f < P->n_bf; ++f) free(P->bf[f].lvl);
  free(P->bf);
  free(P->blk);
  free(P);
}

/* Wire one operator's blocks (bfstructs.jl:99-146).  Returns NULL on malformed
 * input (a block reading a slot that no earlier level writes). */
void* bfref_plan_create(int64_t n_rows, int64_t n_cols, int64_t n_blocks, const int32_t* bf,
                        const int32_t* stage, const int64_t* oo, const int64_t* so,
                        const int64_t* oi, const int64_t* si, const int32_t* rows,
                        const int32_t* cols, const int8_t* ident, const int64_t* data_off,
                        const double* data, const int64_t* optr, const int64_t* oidx,
                        const int64_t* sptr, const int64_t* sidx) {
  rplan* P = (rplan*)calloc(1, sizeof(rplan));
  if (!P) return NULL;
  P->n_rows = n_rows;
  P->n_cols = n_cols;
  P->data = data;
  P->optr = optr;
  P->oidx = oidx;
  P->sptr = sptr;
  P->sidx = sidx;
  int64_t nbf = 0;
  for (int64_t b = 0; b < n_blocks; ++b)
    if (bf[b] + 1 > nbf) nbf = bf[b] + 1;
  P->n_bf = nbf;
  P->blk = (rblock*)calloc((size_t)n_blocks + 1, sizeof(rblock));
  P->bf = (rbf*)calloc((size_t)nbf + 1, sizeof(rbf));
  int32_t* nlev = (int32_t*)calloc((size_t)nbf + 1, sizeof(int32_t));
  int64_t* key = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n_blocks + 1));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n_blocks + 1));
  int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n_blocks + 1));
  size_t cap = 16;
  while (cap < (size_t)n_blocks * 3 + 16) cap <<= 1;
  hent* H = (hent*)calloc(cap, sizeof(hent));
  int ok = P->blk && P->bf && nlev && key && order && tmp && H;
  if (ok) {
    for (int64_t b = 0; b < n_blocks; ++b)
      if (stage[b] > 0 && stage[b] + 1 > nlev[bf[b]]) nlev[bf[b]] = stage[b] + 1;
    for (int64_t f = 0; f < nbf; ++f)
      if (nlev[f] < 1) nlev[f] = 1;
    /* order blocks by bf, then Q < R1 < ... < P, stable (counting sorts) */
    int64_t maxr = 0;
    for (int64_t b = 0; b < n_blocks; ++b) {
      key[b] = stage[b] < 0 ? nlev[bf[b]] : stage[b];
      if (key[b] > maxr) maxr = key[b];
    }
    int64_t* cnt = (int64_t*)calloc((size_t)(maxr > nbf ? maxr : nbf) + 2, sizeof(int64_t));
    for (int64_t b = 0; b < n_blocks; ++b) cnt[key[b] + 1]++;
    for (int64_t r = 0; r <= maxr; ++r) cnt[r + 1] += cnt[r];
    for (int64_t b = 0; b < n_blocks; ++b) tmp[cnt[key[b]]++] = b;
    memset(cnt, 0, sizeof(int64_t) * ((size_t)(maxr > nbf ? maxr : nbf) + 2));
    for (int64_t b = 0; b < n_blocks; ++b) cnt[bf[b] + 1]++;
    for (int64_t f = 0; f < nbf; ++f) cnt[f + 1] += cnt[f];
    for (int64_t i = 0; i < n_blocks; ++i) order[cnt[bf[tmp[i]]]++] = tmp[i];
    free(cnt);
  }
  int64_t b = 0;
  for (int64_t f = 0; f < nbf && ok; ++f) {
    rbf* F = &P->bf[f];
    int32_t L = nlev[f];
    F->n_lvl = L - 1;
    F->lvl = (int64_t*)calloc((size_t)L + 1, sizeof(int64_t));
    int64_t ws = 0;
    F->q0 = b;
    while (b < n_blocks && bf[order[b]] == f && stage[order[b]] == 0) {
      int64_t g = order[b];
      int64_t ko[4] = {f, 0, oo[g], so[g]};
      int64_t m = sptr[si[g] + 1] - sptr[si[g]];
      int64_t len = ident[g] ? m : rows[g];
      hent* e = hfind(H, cap, ko);
      if (!e->used) {
        e->used = 1;
        memcpy(e->k, ko, sizeof ko);
        e->off = ws;
        e->len = len;
        ws += len;
      }
      rblock* B = &P->blk[b++];
      B->data = ident[g] ? -1 : data_off[g];
      B->rows = (int32_t)len;
      B->cols = (int32_t)m;
      B->in_ptr = si[g];
      B->out_ptr = e->off;
    }
    F->q1 = F->r0 = b;
    for (int32_t l = 1; l < L && ok; ++l) {
      F->lvl[l - 1] = b;
      while (b < n_blocks && bf[order[b]] == f && stage[order[b]] == l) {
        int64_t g = order[b];
        int64_t ki[4] = {f, l - 1, oi[g], si[g]};
        hent* ei = hfind(H, cap, ki);
        if (!ei->used) {
          ok = 0;
          break;
        }
        int64_t in_off = ei->off, in_len = ei->len;
        int64_t len = ident[g] ? in_len : rows[g];
        int64_t ko[4] = {f, l, oo[g], so[g]};
        hent* e = hfind(H, cap, ko);
        if (!e->used) {
          e->used = 1;
          memcpy(e->k, ko, sizeof ko);
          e->off = ws;
          e->len = len;
          ws += len;
        }
        rblock* B = &P->blk[b++];
        B->data = ident[g] ? -1 : data_off[g];
        B->rows = (int32_t)len;
        B->cols = (int32_t)(ident[g] ? in_len : cols[g]);
        B->in_ptr = in_off;
        B->out_ptr = e->off;
      }
    }
    F->lvl[L - 1] = b;
    F->r1 = F->p0 = b;
    while (ok && b < n_blocks && bf[order[b]] == f && stage[order[b]] < 0) {
      int64_t g = order[b];
      int64_t ki[4] = {f, L - 1, oi[g], si[g]};
      hent* ei = hfind(H, cap, ki);
      if (!ei->used) {
        ok = 0;
        break;
      }
      int64_t m = optr[oo[g] + 1] - optr[oo[g]];
      rblock* B = &P->blk[b++];
      B->data = ident[g] ? -1 : data_off[g];
      B->rows = (int32_t)m;
      B->cols = (int32_t)(ident[g] ? m : cols[g]);
      B->in_ptr = ei->off;
      B->out_ptr = oo[g];
    }
    F->p1 = b;
    F->ws_len = ws;
    if (ws > P->max_ws) P->max_ws = ws;
  }
  for (int64_t i = 0; i < n_blocks && ok; ++i) {
    if (P->blk[i].rows > P->max_dim) P->max_dim = P->blk[i].rows;
    if (P->blk[i].cols > P->max_dim) P->max_dim = P->blk[i].cols;
  }
  free(H);
  free(key);
  free(order);
  free(tmp);
  free(nlev);
  if (!ok || b != n_blocks) {
    bfref_plan_destroy(P);
    return NULL;
  }
  return P;
}

/* y[i] += sum_j A[i,j] v[j]  (A column-major rows x cols, ComplexF64) */
static void gemv_acc(const double* A, int32_t rows, int32_t cols, const cplx* v, cplx* y) {
  for (int32_t j = 0; j < cols; ++j) {
    const double* a = A + 2 * (int64_t)j * rows;
    double vr = v[j].re, vi = v[j].im;
    for (int32_t i = 0; i < rows; ++i) {
      double ar = a[2 * i], ai = a[2 * i + 1];
      y[i].re += ar * vr - ai * vi;
      y[i].im += ar * vi + ai * vr;
    }
  }
}

/* bfvector.jl:200-296 for one far block, accumulating into ylocal */
static void bf_apply(const rplan* P, const rbf* F, const cplx* x, cplx* ylocal, cplx* ws,
                     cplx* tmpv) {
  const rblock* B = P->blk;
  for (int64_t b = F->q0; b < F->q1; ++b) {
    const rblock* k = &B[b];
    const int64_t* vals = P->sidx + P->sptr[k->in_ptr];
    for (int32_t j = 0; j < k->cols; ++j) tmpv[j] = x[vals[j]];
    cplx* out = ws + k->out_ptr;
    if (k->data < 0) {
      memcpy(out, tmpv, sizeof(cplx) * (size_t)k->rows);
    } else {
      memset(out, 0, sizeof(cplx) * (size_t)k->rows);
      gemv_acc(P->data + 2 * k->data, k->rows, k->cols, tmpv, out);
    }
  }
  for (int32_t l = 0; l < F->n_lvl; ++l) {
    int64_t b0 = F->lvl[l], b1 = F->lvl[l + 1];
    for (int64_t b = b0; b < b1; ++b) memset(ws + B[b].out_ptr, 0, sizeof(cplx) * (size_t)B[b].rows);
    for (int64_t b = b0; b < b1; ++b) {
      const rblock* k = &B[b];
      cplx* out = ws + k->out_ptr;
      const cplx* in = ws + k->in_ptr;
      if (k->data < 0) {
        for (int32_t i = 0; i < k->rows; ++i) {
          out[i].re += in[i].re;
          out[i].im += in[i].im;
        }
      } else {
        gemv_acc(P->data + 2 * k->data, k->rows, k->cols, in, out);
      }
    }
  }
  for (int64_t b = F->p0; b < F->p1; ++b) {
    const rblock* k = &B[b];
    const int64_t* vals = P->oidx + P->optr[k->out_ptr];
    const cplx* in = ws + k->in_ptr;
    if (k->data < 0) {
      for (int32_t i = 0; i < k->rows; ++i) tmpv[i] = in[i];
    } else {
      memset(tmpv, 0, sizeof(cplx) * (size_t)k->rows);
      gemv_acc(P->data + 2 * k->data, k->rows, k->cols, in, tmpv);
    }
    for (int32_t i = 0; i < k->rows; ++i) {
      ylocal[vals[i]].re += tmpv[i].re;
      ylocal[vals[i]].im += tmpv[i].im;
    }
  }
}

/* y = beta*y + alpha * sum over far blocks [bf_begin, bf_end) of BF * x
 * (ComplexF64 interleaved).  Returns 0 on success. */
int bfref_matvec(void* plan, const double* x, double* y, double alpha_re, double alpha_im,
                 double beta_re, double beta_im, int nthreads, int64_t bf_begin,
                 int64_t bf_end) {
  rplan* P = (rplan*)plan;
  if (!P) return 1;
  if (bf_end > P->n_bf || bf_end < 0) bf_end = P->n_bf;
  if (bf_begin < 0) bf_begin = 0;
  if (nthreads < 1) nthreads = omp_get_max_threads();
  const int64_t nr = P->n_rows;
  cplx* Y = (cplx*)y;
  if (beta_re == 0.0 && beta_im == 0.0) {
    memset(Y, 0, sizeof(cplx) * (size_t)nr);
  } else if (!(beta_re == 1.0 && beta_im == 0.0)) {
    for (int64_t i = 0; i < nr; ++i) {
      double re = Y[i].re, im = Y[i].im;
      Y[i].re = beta_re * re - beta_im * im;
      Y[i].im = beta_re * im + beta_im * re;
    }
  }
  cplx* bufs = (cplx*)calloc((size_t)nthreads * (size_t)nr, sizeof(cplx));
  if (!bufs) return 2;
  int fail = 0;
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    cplx* ylocal = bufs + (size_t)tid * (size_t)nr;
    cplx* ws = (cplx*)malloc(sizeof(cplx) * (size_t)(P->max_ws + 1));
    cplx* tmpv = (cplx*)malloc(sizeof(cplx) * (size_t)(P->max_dim + 1));
    if (!ws || !tmpv) {
#pragma omp atomic write
      fail = 3;
    }
#pragma omp barrier
    if (!fail) {
#pragma omp for schedule(static)
      for (int64_t f = bf_begin; f < bf_end; ++f)
        bf_apply(P, &P->bf[f], (const cplx*)x, ylocal, ws, tmpv);
    }
    free(ws);
    free(tmpv);
  }
  if (!fail)
    for (int t = 0; t < nthreads; ++t) {
      const cplx* bb = bufs + (size_t)t * (size_t)nr;
      for (int64_t i = 0; i < nr; ++i) {
        Y[i].re += alpha_re * bb[i].re - alpha_im * bb[i].im;
        Y[i].im += alpha_re * bb[i].im + alpha_im * bb[i].re;
      }
    }
  free(bufs);
  return fail;
}

int64_t bfref_plan_nbf(void* plan) { return plan ? ((rplan*)plan)->n_bf : 0; }
