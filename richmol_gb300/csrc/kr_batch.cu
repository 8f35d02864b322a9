// Batched mixed-precision Krylov step for ensembles of state vectors
// (thermal ensembles, many initial states) on GB300 (sm_103a).
//
// The reference propagates the vectors of an ensemble one after another with
// the FP64 Lanczos of richmol/tdse.py:379-382 / 417-486. Here all vectors move
// together, each with its own Krylov order:
//   * layout: every vector-valued array is vector-minor, [dim][nb] (nb = nvec
//     rounded up to 128), so a thread owns one vector and the factors K, MF are
//     the same for all threads of a block (broadcast reads);
//   * mat-vec in complex64 (the Kronecker contraction of field.py:1212-1243,
//     term by term): the K contraction on the tensor cores as split-TF32 MMAs,
//     or every product as an FP32 FMA (kr_batch_set_matvec);
//   * Krylov basis in complex64, full classical Gram-Schmidt orthogonalisation
//     against every basis vector, dot products accumulated in FP64 across chunks;
//   * FP64 per-vector scalars: alpha, beta, the tridiagonal exponential
//     exp(fac T) e0 (Taylor series on the vector) and the a-posteriori error
//     estimate |fac| beta_k |[exp(fac T_k)]_{k,0}| ||v|| (Saad, SIAM J. Numer.
//     Anal. 29 (1992) 209) that stops each vector at its own order;
//   * FP64 state and H0 half-phases.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>

#include "kr_internal.cuh"
#include "kr_tc.cuh"

#define KB_MV_THREADS 128      // vectors per mat-vec block
#define KB_RED_CHUNKS 256      // element chunks of the per-vector reductions
#define KB_NK_MAX 32           // largest n_k of the batched mat-vec

struct kr_batch {
  kr_op* op = nullptr;
  int nvec = 0, nb = 0, mmax = 0;
  long long dim = 0;
  std::vector<void*> allocs;
  float4* S = nullptr;       // [dim][nb] state, double-float (re hi, re lo, im hi, im lo)
  float4* phase_df = nullptr; // [dim] H0 half-phase of the current step, double-float
  float2* V = nullptr;       // [mmax + 1][dim][nb] Krylov basis
  float2* W = nullptr;       // [dim][nb] H V_k
  double* norm0 = nullptr;   // [nb]
  double2* h = nullptr;      // [mmax + 1][nb] reduced dot products
  double2* alpha = nullptr;  // [mmax + 1][nb]
  double* beta = nullptr;    // [mmax + 1][nb]
  double2* c = nullptr;      // [mmax + 1][nb] exp(fac T) e0 of the converged order
  double* vscale = nullptr;  // [nb] 1 / beta_k of the newest basis vector
  int* kconv = nullptr;      // [nb] converged Krylov order (0: still active)
  int* active = nullptr;     // [nb]
  int* grp_active = nullptr; // [nb / KB_MV_THREADS rounded up]
  double* err = nullptr;     // [nb]
  double2* part = nullptr;   // [KB_RED_CHUNKS][mmax + 2][nb] partial sums
  int* counts = nullptr;     // [3]: active vectors, vectors that hit mmax, mat-vec error word
  // mat-vec tile table
  int ntask = 0;
  // slab element ranges (populations)
  int nslab = 0;
  long long* slab_off = nullptr;
  long long* slab_len = nullptr;
  double* pop = nullptr;     // [nslab][nb]
  int* task_slab = nullptr;
  int* task_i0 = nullptr;
  int* task_nr = nullptr;
  int mv_kind = KR_MATVEC_TENSOR;
  long long launches = 0;
};

// plain-data view of a batch for kernels
struct BatchDev {
  int nvec, nb, mmax;
  long long dim;
  float4* S;
  float2* V;
  double* norm0;
  double2* h;
  double2* alpha;
  double* beta;
  double2* c;
  double* vscale;
  int* kconv;
  int* active;
  double* err;
  int* counts;
};

static BatchDev dev_view(const kr_batch* b) {
  BatchDev d;
  d.nvec = b->nvec;
  d.nb = b->nb;
  d.mmax = b->mmax;
  d.dim = b->dim;
  d.S = b->S;
  d.V = b->V;
  d.norm0 = b->norm0;
  d.h = b->h;
  d.alpha = b->alpha;
  d.beta = b->beta;
  d.c = b->c;
  d.vscale = b->vscale;
  d.kconv = b->kconv;
  d.active = b->active;
  d.err = b->err;
  d.counts = b->counts;
  return d;
}

// ---------------------------------------------------------------------------
// vector-minor elementwise helpers: block = (32 lanes -> vectors, 8 warps ->
// element streams); grid = (KB_RED_CHUNKS element chunks, nb / 32 groups)
// ---------------------------------------------------------------------------
struct Chunk {
  long long e0, e1;
};
__device__ __forceinline__ Chunk chunk_of(long long dim) {
  const long long per = (dim + gridDim.x - 1) / gridDim.x;
  Chunk c;
  c.e0 = blockIdx.x * per;
  c.e1 = min(dim, c.e0 + per);
  return c;
}

// sum over the 8 warps of one value per (warp, lane), result in warp 0
__device__ __forceinline__ double2 warps_sum(double2 v, double2 (*sh)[32]) {
  sh[threadIdx.y][threadIdx.x] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  if (threadIdx.y == 0)
    for (int w = 0; w < 8; ++w) s = cadd(s, sh[w][threadIdx.x]);
  __syncthreads();
  return s;
}

// ---------------------------------------------------------------------------
// double-float arithmetic for the state: value = hi + lo with |lo| <= ulp(hi)/2,
// about 2^-48 relative. Knuth's TwoSum, the FMA TwoProduct and Dekker's
// normalisation (published error-free transformations); the operations are
// written with round-to-nearest intrinsics so that no FMA contraction alters
// them. The state lives in FP32 pipes this way: GB300's FP64 rate is 1/58 of
// its FP32 rate.
// ---------------------------------------------------------------------------
struct dfl {
  float hi, lo;
};
struct dfc {
  dfl re, im;
};
__device__ __forceinline__ dfl df_fast(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const dfl s = df_two_sum(a.hi, b.hi);
  return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast(p, e);
}
__device__ __forceinline__ dfl df_mulf(dfl a, float b) {
  const float p = __fmul_rn(a.hi, b);
  return df_fast(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfc_ld(float4 q) { return {{q.x, q.y}, {q.z, q.w}}; }
__device__ __forceinline__ float4 dfc_st(dfc a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ dfl df_from(double x) {
  const float hi = __double2float_rn(x);
  return {hi, __double2float_rn(x - (double)hi)};
}
__device__ __forceinline__ double df_to(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfc dfc_from(double2 x) { return {df_from(x.x), df_from(x.y)}; }

// FP64 phase -> double-float (once per step, dim elements)
__global__ void kb_phase_df(const double2* phase, float4* pdf, long long dim) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < dim; e += (long long)gridDim.x * blockDim.x)
    pdf[e] = dfc_st(dfc_from(phase[e]));
}

// S <- phase * S (optional); partial ||S_v||^2
__global__ void kb_phase_norm(float4* S, const float4* phase, long long dim, int nb, double2* part) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  dfl acc = {0.f, 0.f};
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    dfc s = dfc_ld(S[e * nb + v]);
    if (phase) {
      s = dfc_mul(s, dfc_ld(__ldg(phase + e)));
      S[e * nb + v] = dfc_st(s);
    }
    acc = df_add(acc, df_add(df_mul(s.re, s.re), df_mul(s.im, s.im)));
  }
  const double2 t = warps_sum(make_double2(df_to(acc), 0.0), sh);
  if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = t;
}

// out[j][v] = sum over chunks of part[chunk][j][v] (fixed order)
__global__ void kb_reduce(const double2* part, int ncoef, int nb, int stride_coef, double2* out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ncoef * nb) return;
  const int j = idx / nb, v = idx - j * nb;
  double2 s = make_double2(0.0, 0.0);
  for (int c = 0; c < KB_RED_CHUNKS; ++c) s = cadd(s, part[((long long)c * stride_coef + j) * nb + v]);
  out[(long long)j * nb + v] = s;
}

// norm0 = ||S||, V0 = S / norm0 (complex64); resets the per-vector state
__global__ void kb_start(const float4* S, float2* V0, const double2* nsq, double* norm0, int* active, int* kconv,
                         double* vscale, long long dim, int nb, int nvec) {
  const int v = blockIdx.y * 32 + threadIdx.x;
  const double n0 = sqrt(nsq[v].x);
  const double inv = n0 > 0.0 ? 1.0 / n0 : 0.0;
  if (blockIdx.x == 0 && threadIdx.y == 0) {
    norm0[v] = n0;
    active[v] = (v < nvec && n0 > 0.0) ? 1 : 0;
    kconv[v] = 0;
    vscale[v] = 1.0;
  }
  const dfl invd = df_from(inv);
  const Chunk ch = chunk_of(dim);
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    const dfc s = dfc_ld(S[e * nb + v]);
    const dfl re = df_mul(s.re, invd), im = df_mul(s.im, invd);
    V0[e * nb + v] = make_float2(__fadd_rn(re.hi, re.lo), __fadd_rn(im.hi, im.lo));
  }
}

// partial dots h_j = <V_j, W> for j = 0..k: FP32 products, FP32 sums inside a
// thread's elements, FP64 across threads and chunks
__global__ void kb_dots(const float2* V, const float2* W, const int* active, long long dim, int nb, int k,
                        int stride_coef, double2* part) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  const bool act = active[v] != 0;
  for (int j = 0; j <= k; ++j) {
    float2 acc = make_float2(0.f, 0.f);
    if (act) {
      const float2* Vj = V + (long long)j * dim * nb;
      for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
        const float2 a = Vj[e * nb + v], b = W[e * nb + v];
        acc.x = fmaf(a.x, b.x, acc.x);
        acc.x = fmaf(a.y, b.y, acc.x);
        acc.y = fmaf(a.x, b.y, acc.y);
        acc.y = fmaf(-a.y, b.x, acc.y);
      }
    }
    const double2 t = warps_sum(make_double2(acc.x, acc.y), sh);
    if (threadIdx.y == 0) part[((long long)blockIdx.x * stride_coef + j) * nb + v] = t;
  }
}

// V_{k+1} = W - sum_j h_j V_j (unnormalised), partial ||V_{k+1}||^2
__global__ void kb_update(float2* V, const float2* W, const double2* h, const int* active, long long dim, int nb,
                          int k, double2* part) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  const bool act = active[v] != 0;
  dfl nacc = {0.f, 0.f};
  if (act) {
    float2 hv[KB_NK_MAX];
    const int kk = min(k, KB_NK_MAX - 1);
    for (int j = 0; j <= kk; ++j) {
      const double2 t = h[(long long)j * nb + v];
      hv[j] = make_float2((float)t.x, (float)t.y);
    }
    float2* Vn = V + (long long)(k + 1) * dim * nb;
    for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
      float2 r = W[e * nb + v];
      for (int j = 0; j <= kk; ++j) {
        const float2 a = V[((long long)j * dim + e) * nb + v];
        r.x = fmaf(-hv[j].x, a.x, r.x);
        r.x = fmaf(hv[j].y, a.y, r.x);
        r.y = fmaf(-hv[j].x, a.y, r.y);
        r.y = fmaf(-hv[j].y, a.x, r.y);
      }
      Vn[e * nb + v] = r;
      nacc = df_add(nacc, df_add(df_mulf({r.x, 0.f}, r.x), df_mulf({r.y, 0.f}, r.y)));
    }
  }
  const double2 t = warps_sum(make_double2(df_to(nacc), 0.0), sh);
  if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = t;
}

// per vector: T update, exp(fac T) e0, error estimate, convergence
__global__ void kb_small(BatchDev b, int k, double2 fac, double tol, const double2* nsq) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= b.nb || !b.active[v]) return;
  const int nb = b.nb;
  const double2 hk = b.h[(long long)k * nb + v];
  const double bk = sqrt(nsq[v].x);
  b.alpha[(long long)k * nb + v] = hk;
  b.beta[(long long)k * nb + v] = bk;
  const int n = k + 1;
  // Taylor series of exp(A) e0, A = fac T, sub-steps with ||A/s||_1 <= 1
  double2 y[KB_NK_MAX], t[KB_NK_MAX], r[KB_NK_MAX];
  double nrm = 0.0;
  const double fa = sqrt(cabs2(fac));
  for (int i = 0; i < n; ++i) {
    double cs = sqrt(cabs2(cmul(fac, b.alpha[(long long)i * nb + v])));
    if (i > 0) cs += fa * fabs(b.beta[(long long)(i - 1) * nb + v]);
    if (i < n - 1) cs += fa * fabs(b.beta[(long long)i * nb + v]);
    nrm = fmax(nrm, cs);
  }
  int nsub = max(1, (int)ceil(nrm));
  const double inv_s = 1.0 / nsub;
  for (int i = 0; i < n; ++i) y[i] = make_double2(i == 0 ? 1.0 : 0.0, 0.0);
  for (int sub = 0; sub < nsub; ++sub) {
    for (int i = 0; i < n; ++i) t[i] = y[i];
    for (int j = 1; j <= 40; ++j) {
      double tmax = 0.0, amax = 0.0;
      for (int i = 0; i < n; ++i) {
        double2 s = cmul(b.alpha[(long long)i * nb + v], t[i]);
        if (i > 0) s = cadd(s, cscale(t[i - 1], b.beta[(long long)(i - 1) * nb + v]));
        if (i < n - 1) s = cadd(s, cscale(t[i + 1], b.beta[(long long)i * nb + v]));
        r[i] = cscale(cmul(fac, s), inv_s / j);
      }
      for (int i = 0; i < n; ++i) {
        t[i] = r[i];
        y[i] = cadd(y[i], r[i]);
        tmax = fmax(tmax, fmax(fabs(r[i].x), fabs(r[i].y)));
        amax = fmax(amax, fmax(fabs(y[i].x), fabs(y[i].y)));
      }
      if (tmax <= 1e-17 * amax) break;
    }
  }
  const double e = b.norm0[v] * fa * bk * sqrt(cabs2(y[n - 1]));
  b.err[v] = e;
  const bool last = (k + 1 >= b.mmax);
  if (e <= tol || bk == 0.0 || last) {
    for (int i = 0; i < n; ++i) b.c[(long long)i * nb + v] = y[i];
    b.kconv[v] = n;
    b.active[v] = 0;
    if (last && !(e <= tol || bk == 0.0)) atomicAdd(b.counts + 1, 1);
  } else {
    b.vscale[v] = 1.0 / bk;
    atomicAdd(b.counts, 1);
  }
}

// V_{k+1} *= 1 / beta_k for the vectors still active
__global__ void kb_scale(float2* Vn, const double* vscale, const int* active, long long dim, int nb) {
  const int v = blockIdx.y * 32 + threadIdx.x;
  if (!active[v]) return;
  const float s = (float)vscale[v];
  const Chunk ch = chunk_of(dim);
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    float2 a = Vn[e * nb + v];
    Vn[e * nb + v] = make_float2(a.x * s, a.y * s);
  }
}

// S <- phase * (c_0 S + ||v|| sum_{i>=1} c_i V_i)   (double-float state; the
// complex64 Krylov corrections summed in FP32)
__global__ void kb_combine(BatchDev b, const float4* phase) {
  const int v = blockIdx.y * 32 + threadIdx.x;
  const int nb = b.nb;
  const int K = b.kconv[v];
  if (K == 0) return;  // no Krylov step (zero vector or padding)
  float2 cf[KB_NK_MAX];
  for (int i = 1; i < K; ++i) cf[i] = make_float2((float)b.c[(long long)i * nb + v].x, (float)b.c[(long long)i * nb + v].y);
  const dfc c0 = dfc_from(b.c[v]);
  const dfl n0 = df_from(b.norm0[v]);
  const Chunk ch = chunk_of(b.dim);
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    float2 sacc = make_float2(0.f, 0.f);
    for (int i = 1; i < K; ++i) {
      const float2 a = b.V[((long long)i * b.dim + e) * nb + v];
      sacc.x = fmaf(cf[i].x, a.x, sacc.x);
      sacc.x = fmaf(-cf[i].y, a.y, sacc.x);
      sacc.y = fmaf(cf[i].x, a.y, sacc.y);
      sacc.y = fmaf(cf[i].y, a.x, sacc.y);
    }
    dfc u = dfc_mul(c0, dfc_ld(b.S[e * nb + v]));
    u.re = df_add(u.re, df_mulf(n0, sacc.x));
    u.im = df_add(u.im, df_mulf(n0, sacc.y));
    if (phase) u = dfc_mul(u, dfc_ld(__ldg(phase + e)));
    b.S[e * nb + v] = dfc_st(u);
  }
}

// (nvec, dim) row-major <-> [dim][nb] vector-minor, tiled through shared memory
__global__ void kb_transpose_in(const double2* src, float4* S, long long dim, int nvec, int nb) {
  __shared__ double2 tile[32][33];
  const long long e0 = blockIdx.x * 32LL;
  const int v0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int v = v0 + r;
    const long long e = e0 + threadIdx.x;
    tile[r][threadIdx.x] = (v < nvec && e < dim) ? src[(long long)v * dim + e] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const long long e = e0 + r;
    if (e < dim) S[e * nb + v0 + threadIdx.x] = dfc_st(dfc_from(tile[threadIdx.x][r]));
  }
}
__global__ void kb_transpose_out(const float4* S, double2* dst, long long dim, int nvec, int nb) {
  __shared__ double2 tile[32][33];
  const long long e0 = blockIdx.x * 32LL;
  const int v0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const long long e = e0 + r;
    if (e < dim) {
      const dfc s = dfc_ld(S[e * nb + v0 + threadIdx.x]);
      tile[r][threadIdx.x] = make_double2(df_to(s.re), df_to(s.im));
    } else {
      tile[r][threadIdx.x] = make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int v = v0 + r;
    const long long e = e0 + threadIdx.x;
    if (v < nvec && e < dim) dst[(long long)v * dim + e] = tile[threadIdx.x][r];
  }
}

// complex64 copy of the state (input of the observable mat-vec)
__global__ void kb_to_f32(const float4* S, float2* X, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 s = S[i];
    X[i] = make_float2(__fadd_rn(s.x, s.y), __fadd_rn(s.z, s.w));
  }
}

// partial <S_v | Y_v> with Y in complex64 (double-float accumulation)
__global__ void kb_expect_dots(const float4* S, const float2* Y, long long dim, int nb, double2* part) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  dfl ar = {0.f, 0.f}, ai = {0.f, 0.f};
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    const dfc s = dfc_ld(S[e * nb + v]);
    const float2 y = Y[e * nb + v];
    // conj(s) y = (s.re y.x + s.im y.y) + i (s.re y.y - s.im y.x)
    ar = df_add(ar, df_add(df_mulf(s.re, y.x), df_mulf(s.im, y.y)));
    ai = df_add(ai, df_add(df_mulf(s.re, y.y), df_neg(df_mulf(s.im, y.x))));
  }
  const double2 t = warps_sum(make_double2(df_to(ar), df_to(ai)), sh);
  if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = t;
}

// per slab (blockIdx.x) and vector: sum of |S|^2 over the slab's elements
// (double-float accumulation, fixed order); out[slab][nb]
__global__ void kb_slab_pop(const float4* S, const long long* slab_off, const long long* slab_len, int nb,
                            double* out) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const long long e0 = slab_off[blockIdx.x], e1 = e0 + slab_len[blockIdx.x];
  dfl acc = {0.f, 0.f};
  for (long long e = e0 + threadIdx.y; e < e1; e += 8) {
    const dfc s = dfc_ld(S[e * nb + v]);
    acc = df_add(acc, df_add(df_mul(s.re, s.re), df_mul(s.im, s.im)));
  }
  const double2 t = warps_sum(make_double2(df_to(acc), 0.0), sh);
  if (threadIdx.y == 0) out[(long long)blockIdx.x * nb + v] = t.x;
}

// ---------------------------------------------------------------------------
// batched mat-vec, complex64, tiled. One CTA (256 threads = 8 warps) computes
// a tile of R = 128 / NKP consecutive output rows of one slab for 32 vectors
// (lane = vector). Per term:
//   T[j, a] = sum_b K[a, b] X[j, b]     for the input rows j of the band of
//             the tile, each computed once and kept in shared memory; the
//             work goes to the warps in (row, half-row) units
//   Y[i, a] += sum_w MF[i, w] T[col(i, w), a]
// (field.py:1212-1243 orders the same sum as MF (K X^T)^T). Every thread owns
// the outputs of 4 consecutive rows x 4 consecutive k columns (16 complex
// registers) across all terms. Diagonal M groups (slot w of row i holds column
// i + d0 + w, detected by kr_op_create) address the band by offset: the T row
// of (i, w) is i - i0 + w, and each T value loaded serves up to 4 rows. Other
// groups use the stored columns, the band window taken in chunks of NJ rows.
// K^T, the MF rows and their columns are staged as FP32 in shared memory.
// ---------------------------------------------------------------------------
#define KB_WMAX 16   // ELL width of the M band supported by the batched mat-vec

struct BatchMV {
  DevOp op;
  const float2* X;
  float2* Y;
  int nb;
  const int* task_slab;
  const int* task_i0;
  const int* task_nr;
  const int* grp_active;  // per 32-vector group: any vector active (null: all)
};

// complex x real/imaginary/complex K factor accumulation: t += k * x
template <int KT>
__device__ __forceinline__ void kacc(float2& t, float kr, float ki, float2 x) {
  if (KT == 1) {
    t.x = fmaf(kr, x.x, t.x);
    t.y = fmaf(kr, x.y, t.y);
  } else if (KT == 2) {
    t.x = fmaf(-kr, x.y, t.x);
    t.y = fmaf(kr, x.x, t.y);
  } else {
    t.x = fmaf(kr, x.x, fmaf(-ki, x.y, t.x));
    t.y = fmaf(kr, x.y, fmaf(ki, x.x, t.y));
  }
}

// y += m * t for a real, imaginary or complex M-band value m
template <int MT>
__device__ __forceinline__ void macc(float2& y, float2 m, float2 t) {
  if (MT == 1) {
    y.x = fmaf(m.x, t.x, y.x);
    y.y = fmaf(m.x, t.y, y.y);
  } else if (MT == 2) {
    y.x = fmaf(-m.y, t.y, y.x);
    y.y = fmaf(m.y, t.x, y.y);
  } else {
    y.x = fmaf(m.x, t.x, fmaf(-m.y, t.y, y.x));
    y.y = fmaf(m.x, t.y, fmaf(m.y, t.x, y.y));
  }
}

// t[a] = sum_b K[a, b] X[j, b] for AB consecutive k columns a (Ks points at
// the first; rows of NKP floats) and this thread's vector; X is read in groups
// of 4 independent loads, the next group issued before the current one is used
template <int NKP, int AB, int KT>
__device__ __forceinline__ void kb_trow(const float2* xr, long long nb, int nk2, const float* Ks, float2* t) {
#pragma unroll
  for (int a = 0; a < AB; ++a) t[a] = make_float2(0.f, 0.f);
  float2 xn[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) xn[u] = (u < nk2) ? xr[(long long)u * nb] : make_float2(0.f, 0.f);
  for (int b0 = 0; b0 < nk2; b0 += 4) {
    float2 x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = xn[u];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int bn = b0 + 4 + u;
      xn[u] = (bn < nk2) ? xr[(long long)bn * nb] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int b = b0 + u;  // Ks rows beyond nk2 hold zeros
      const float* kr = Ks + b * NKP;
      const float* ki = Ks + (36 + b) * NKP;
#pragma unroll
      for (int a = 0; a < AB; a += 4) {
        const float4 r4 = *reinterpret_cast<const float4*>(kr + a);
        float4 i4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (KT == 0) i4 = *reinterpret_cast<const float4*>(ki + a);
        kacc<KT>(t[a], r4.x, i4.x, x[u]);
        kacc<KT>(t[a + 1], r4.y, i4.y, x[u]);
        kacc<KT>(t[a + 2], r4.z, i4.z, x[u]);
        kacc<KT>(t[a + 3], r4.w, i4.w, x[u]);
      }
    }
  }
}

// T rows jr < nrow for the input rows j0 + jr into Ts[jr]; rows outside the
// input slab [0, dm2) are zero. (row, half-row) units go round-robin over the
// 8 warps.
template <int NKP>
__device__ __forceinline__ void kb_tstep(const float2* Xs2, long long nb, int nk2, int ktype, const float* Ks,
                                         float2* Ts, int j0, int nrow, int dm2, int wid, int lane) {
  constexpr int NH = NKP >= 8 ? 2 : 1;
  constexpr int AB = NKP / NH;
  for (int u = wid; u < nrow * NH; u += 8) {
    const int jr = u / NH, h = u - jr * NH;
    const int j = j0 + jr;
    float2 t[AB];
    if (j >= 0 && j < dm2) {
      const float2* xr = Xs2 + (long long)j * nk2 * nb;
      if (ktype == 1) kb_trow<NKP, AB, 1>(xr, nb, nk2, Ks + h * AB, t);
      else if (ktype == 2) kb_trow<NKP, AB, 2>(xr, nb, nk2, Ks + h * AB, t);
      else kb_trow<NKP, AB, 0>(xr, nb, nk2, Ks + h * AB, t);
    } else {
#pragma unroll
      for (int a = 0; a < AB; ++a) t[a] = make_float2(0.f, 0.f);
    }
    float2* tr = Ts + (jr * NKP + h * AB) * 32 + lane;
#pragma unroll
    for (int a = 0; a < AB; ++a) tr[a * 32] = t[a];
  }
}

// M step of a diagonal group for tile rows r0 .. r0 + 3 (< nr) and k columns
// a0 .. a0 + 3: the T row of (row r, slot w) is r + w
template <int NKP, int MT>
__device__ __forceinline__ void kb_mdia(float2* y, const float2* Ts, const float2* MFs, int W, int r0, int a0,
                                        int nr, int lane) {
  for (int cw = 0; cw < W + 3; ++cw) {
    float2 t[4];
    const float2* tr = Ts + ((r0 + cw) * NKP + a0) * 32 + lane;
#pragma unroll
    for (int aa = 0; aa < 4; ++aa) t[aa] = tr[aa * 32];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int w = cw - r;
      if (w >= 0 && w < W && r0 + r < nr) {
        const float2 m = MFs[(r0 + r) * KB_WMAX + w];
#pragma unroll
        for (int aa = 0; aa < 4; ++aa) macc<MT>(y[r * 4 + aa], m, t[aa]);
      }
    }
  }
}

// M step of an ELL group over one chunk of T rows [jc, jc + nj)
template <int NKP, int MT>
__device__ __forceinline__ void kb_mell(float2* y, const float2* Ts, const float2* MFs, const int* Cs, int W, int jc,
                                        int nj, int r0, int a0, int nr, int lane) {
  for (int w = 0; w < W; ++w) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (r0 + r >= nr) continue;
      const int c = Cs[(r0 + r) * KB_WMAX + w] - jc;
      if (c < 0 || c >= nj) continue;
      const float2 m = MFs[(r0 + r) * KB_WMAX + w];
      const float2* tr = Ts + (c * NKP + a0) * 32 + lane;
#pragma unroll
      for (int aa = 0; aa < 4; ++aa) macc<MT>(y[r * 4 + aa], m, tr[aa * 32]);
    }
  }
}

template <int NKP>
__device__ void kb_tile(const BatchMV& p, int s1, int i0, int nr, float* smem) {
  constexpr int R = 128 / NKP;            // rows of the tile
  constexpr int NJ = R + KR_DIAG_MAX - 1; // T rows held: a diagonal band, or one ELL chunk
  constexpr int NAB = NKP / 4;            // 4-wide k-column blocks
  const DevOp& op = p.op;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const long long nb = p.nb;
  const int v = blockIdx.y * 32 + lane;
  const int r0 = (wid / NAB) * 4, a0 = (wid % NAB) * 4;  // this thread's outputs
  float2* Ts = reinterpret_cast<float2*>(smem);                 // [NJ][NKP][32]
  float* Ks = smem + 2 * NJ * NKP * 32;                          // [2][36][NKP]
  float2* MFs = reinterpret_cast<float2*>(Ks + 2 * 36 * NKP);   // [R][KB_WMAX]
  int* Cs = reinterpret_cast<int*>(MFs + R * KB_WMAX);           // [R][KB_WMAX]
  int* meta = Cs + R * KB_WMAX;                                  // ELL band window jmin, jmax
  const int nk1 = __ldg(op.out_dk + s1);
  float2 y[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) y[q] = make_float2(0.f, 0.f);
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  for (int term = tb; term < te; ++term) {
    const int s2 = __ldg(op.t_in + term);
    const int kb = __ldg(op.t_k + term);
    const int mfi = __ldg(op.t_mf + term);
    const int nk2 = __ldg(op.in_dk + s2);
    const int dm2 = __ldg(op.in_dm + s2);
    const int Wst = __ldg(op.mf_width + mfi);  // stored width (row stride of MF)
    const int d0s = __ldg(op.mf_diag + mfi);
    const bool dia = d0s != KR_NO_DIAG && Wst <= KR_DIAG_MAX;
    // slots that carry a value with the current field (the field kernel's band)
    const int bhi = __ldcg(op.mf_band + 2 * mfi + 1);
    if (bhi < 0) continue;  // MF is zero with this field: no contribution (uniform)
    const int wlo = dia ? Wst - 1 - __ldcg(op.mf_band + 2 * mfi) : 0;
    const int W = dia ? bhi - wlo + 1 : Wst;
    const int d0 = dia ? d0s + wlo : 0;
    const int ktype = __ldg(op.k_type + kb);
    const int mtype = __ldcg(op.mf_type + mfi);
    const int kw = (ktype == 0) ? 2 : 1;
    const float* KT = op.k_f32 + __ldg(op.k_off + kb);
    const int* col = op.m_col + __ldg(op.mf_col_off + mfi);
    const float2* mf = op.mf_f32 + __ldg(op.mf_off + mfi) + wlo;
    __syncthreads();  // the previous term is done with Ks, MFs, Cs, Ts
    // K^T as [plane][b][a], zero outside nk2 x nk1 (rows up to the next multiple of 4)
    const int nb4 = (nk2 + 3) & ~3;
    for (int e = tid; e < kw * nb4 * NKP; e += blockDim.x) {
      const int plane = e / (nb4 * NKP);
      const int rem = e - plane * nb4 * NKP;
      const int b = rem / NKP, a = rem - b * NKP;
      Ks[(plane * 36 + b) * NKP + a] =
          (a < nk1 && b < nk2) ? __ldg(KT + ((long long)b * nk1 + a) * kw + plane) : 0.f;
    }
    for (int e = tid; e < nr * W; e += blockDim.x) {
      const int r = e / W, w = e - r * W;
      const long long src = (long long)(i0 + r) * Wst + w;
      MFs[r * KB_WMAX + w] = __ldcg(mf + src);
      if (!dia) Cs[r * KB_WMAX + w] = __ldg(col + src);
    }
    if (!dia && wid == 0) {
      int lo = 0x7fffffff, hi = -1;
      for (int e = lane; e < nr * W; e += 32) {
        const int c = __ldg(col + (long long)(i0 + e / W) * Wst + (e % W));
        lo = min(lo, c);
        hi = max(hi, c);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
      if (lane == 0) {
        meta[0] = lo;
        meta[1] = hi;
      }
    }
    __syncthreads();
    const float2* Xs2 = p.X + (long long)__ldg(op.in_off + s2) * nb + v;
    if (dia) {
      // T rows of the band: input rows i0 + d0 .. i0 + d0 + nr + W - 2
      kb_tstep<NKP>(Xs2, nb, nk2, ktype, Ks, Ts, i0 + d0, nr + W - 1, dm2, wid, lane);
      __syncthreads();
      if (mtype == 1) kb_mdia<NKP, 1>(y, Ts, MFs, W, r0, a0, nr, lane);
      else if (mtype == 2) kb_mdia<NKP, 2>(y, Ts, MFs, W, r0, a0, nr, lane);
      else kb_mdia<NKP, 0>(y, Ts, MFs, W, r0, a0, nr, lane);
    } else {
      const int jmin = meta[0], jmax = meta[1];
      for (int jc = jmin; jc <= jmax; jc += NJ) {
        const int nj = min(NJ, jmax - jc + 1);
        if (jc != jmin) __syncthreads();  // the previous chunk's M step is done with Ts
        kb_tstep<NKP>(Xs2, nb, nk2, ktype, Ks, Ts, jc, nj, dm2, wid, lane);
        __syncthreads();
        if (mtype == 1) kb_mell<NKP, 1>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
        else if (mtype == 2) kb_mell<NKP, 2>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
        else kb_mell<NKP, 0>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
      }
    }
  }
  float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * nk1) * nb + v;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int aa = 0; aa < 4; ++aa) {
      const int i = r0 + r, a = a0 + aa;
      if (i < nr && a < nk1) Y[((long long)i * nk1 + a) * nb] = y[r * 4 + aa];
    }
  }
}

__global__ void __launch_bounds__(256, 2) kb_matvec(BatchMV p) {
  extern __shared__ __align__(16) float kb_smem[];
  const int task = blockIdx.x;
  if (p.grp_active && !p.grp_active[blockIdx.y]) return;
  const int s1 = __ldg(p.task_slab + task);
  const int i0 = __ldg(p.task_i0 + task);
  const int nr = __ldg(p.task_nr + task);
  const int nk1 = __ldg(p.op.out_dk + s1);
  if (nk1 <= 4) kb_tile<4>(p, s1, i0, nr, kb_smem);
  else if (nk1 <= 8) kb_tile<8>(p, s1, i0, nr, kb_smem);
  else if (nk1 <= 16) kb_tile<16>(p, s1, i0, nr, kb_smem);
  else kb_tile<32>(p, s1, i0, nr, kb_smem);
}

// shared memory of kb_matvec: the largest of the four tile shapes
static size_t kb_matvec_smem() {
  size_t best = 0;
  for (int nkp : {4, 8, 16, 32}) {
    const int R = 128 / nkp, NJ = R + KR_DIAG_MAX - 1;
    size_t b = sizeof(float2) * NJ * nkp * 32 + sizeof(float) * 2 * 36 * nkp + sizeof(float2) * R * KB_WMAX +
               sizeof(int) * (R * KB_WMAX + 2);
    best = std::max(best, b);
  }
  return best;
}

// ---------------------------------------------------------------------------
// batched mat-vec on the tensor cores. One CTA (256 threads = 8 warps) computes
// a tile of R consecutive output rows of one slab, all its k columns, for 128
// vectors. Per term:
//   Z[i][b][v]  = sum_w MF[i, w] X[col(i, w)][b][v]      SIMT, FP32 registers
//   Y[i][a][v] += sum_b K[a, b] Z[i][b][v]               tcgen05.mma
// (field.py:1212-1243 orders the same sum as MF (K X^T)^T). The K contraction
// runs as 128 x NP x 8 TF32 MMAs with the vectors as the M dimension: the real
// and imaginary parts of Z_i, each split hi + lo (3xTF32: hi*hi + hi*lo +
// lo*hi), form the A operands; K^T, split likewise, the B operands; the real
// and imaginary parts of Y_i accumulate in TMEM over all terms of the slab.
// KP = n_k2 padded to 8 (largest over the slab's terms) is the MMA K extent,
// R = 64 / KP, NP = n_k1 padded to 16 the MMA N. The SIMT part of term t + 1
// (X loads and M-band FMAs) runs while the MMAs of term t execute; only the
// A-tile stores wait for them.
// Threads: warp w owns vectors 32 (w % 4) .. + 31 (= TMEM lanes) and input k
// columns [KP/2 (w / 4), KP/2 (w / 4 + 1)).
// ---------------------------------------------------------------------------
struct BatchTC {
  DevOp op;
  const float2* X;
  float2* Y;
  int nb;
  const int* task;        // [4][ntask]: slab, first row, rows, KP
  int ntask;
  const int* grp_active;  // per 32-vector group: any vector active (null: all)
  int* err;
};

constexpr int TC_ABYTES = 128 * 1024;       // A tiles: R rows x 4 parts x 128 x KP FP32 (R KP = 64)
constexpr int TC_BPART = 32 * 32 * 4;       // one B part: NP x KP FP32 at most
constexpr int TC_BBYTES = 6 * TC_BPART;     // one B buffer: K_re, K_im, -K_im, each hi and lo
constexpr int TC_MFBYTES = 2 * 8 * KB_WMAX * 8;
constexpr int TC_CSBYTES = 2 * 8 * KB_WMAX * 4;
constexpr int TC_SMEM = TC_ABYTES + 2 * TC_BBYTES + TC_MFBYTES + TC_CSBYTES + 64;

// X window of one term in registers: input rows j0 + c (c < RP) for this
// thread's vector and KP/2 input columns; RP * KP/2 = 16 loads issued back to
// back (rows outside [0, dm2) and columns beyond n_k2 read as zero)
template <int KP>
struct KbtWin {
  static constexpr int BH = KP / 2, RP = 32 / KP;
  float2 x[RP][BH];
  __device__ __forceinline__ void load(const float2* Xs2, long long nb, int nk2, int dm2, int j0, int nrow, int b0) {
#pragma unroll
    for (int c = 0; c < RP; ++c) {
      const int j = j0 + c;
      const bool rin = c < nrow && j >= 0 && j < dm2;
      const float2* xr = Xs2 + (long long)j * nk2 * nb;
#pragma unroll
      for (int q = 0; q < BH; ++q)
        x[c][q] = (rin && b0 + q < nk2) ? __ldg(xr + (long long)(b0 + q) * nb) : make_float2(0.f, 0.f);
    }
  }
};

// M step of a diagonal term for window rows cw0 .. cw0 + RP - 1 held in xw:
// output row r takes slot w = cw - r
template <int KP, int MT>
__device__ __forceinline__ void kbt_mdia(float2 (&z)[64 / KP][KP / 2], const KbtWin<KP>& xw, int cw0, int nr, int W,
                                         const float2* MFs) {
  constexpr int R = 64 / KP, BH = KP / 2, RP = 32 / KP;
#pragma unroll
  for (int c = 0; c < RP; ++c) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int w = cw0 + c - r;
      if (w >= 0 && w < W && r < nr) {
        const float2 m = MFs[r * KB_WMAX + w];
#pragma unroll
        for (int q = 0; q < BH; ++q) macc<MT>(z[r][q], m, xw.x[c][q]);
      }
    }
  }
}

// M step of a term with stored columns (ELL), one input row per slot
template <int KP, int MT>
__device__ __forceinline__ void kbt_mell(float2 (&z)[64 / KP][KP / 2], const float2* Xs2, long long nb, int nk2,
                                         int nr, int W, int b0, const float2* MFs, const int* Cs) {
  constexpr int R = 64 / KP, BH = KP / 2;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (r >= nr) continue;
    for (int w = 0; w < W; ++w) {
      const float2* xr = Xs2 + (long long)Cs[r * KB_WMAX + w] * nk2 * nb;
      const float2 m = MFs[r * KB_WMAX + w];
      float2 x[BH];
#pragma unroll
      for (int q = 0; q < BH; ++q) x[q] = (b0 + q < nk2) ? __ldg(xr + (long long)(b0 + q) * nb) : make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < BH; ++q) macc<MT>(z[r][q], m, x[q]);
    }
  }
}

template <int KP, int MT>
__device__ __forceinline__ void kbt_mstep(float2 (&z)[64 / KP][KP / 2], KbtWin<KP>& xw, bool loaded,
                                          const float2* Xs2, long long nb, int nk2, int dm2, int i0, int nr, int d0,
                                          int W, int b0, const float2* MFs, const int* Cs, bool dia) {
  constexpr int RP = 32 / KP;
  if (dia) {
    const int nwin = nr + W - 1;
    for (int cw0 = 0; cw0 < nwin; cw0 += RP) {
      if (cw0 > 0 || !loaded) xw.load(Xs2, nb, nk2, dm2, i0 + d0 + cw0, nwin - cw0, b0);
      kbt_mdia<KP, MT>(z, xw, cw0, nr, W, MFs);
    }
  } else {
    kbt_mell<KP, MT>(z, Xs2, nb, nk2, nr, W, b0, MFs, Cs);
  }
}

// one term of a tensor-core tile: its tables and shared-memory staging
struct KbtTerm {
  int s2, nk2, dm2, W, Wst, d0, ktype, mtype;
  bool dia, ok, empty;
  const float* KT;
  const int* col;
  const float2* mf;
  const float2* Xs2;
};

__device__ __forceinline__ KbtTerm kbt_term(const DevOp& op, const BatchTC& p, int term, int KP, int v, long long nb) {
  KbtTerm t;
  t.s2 = __ldg(op.t_in + term);
  const int kb = __ldg(op.t_k + term);
  const int mfi = __ldg(op.t_mf + term);
  t.nk2 = __ldg(op.in_dk + t.s2);
  t.dm2 = __ldg(op.in_dm + t.s2);
  t.Wst = __ldg(op.mf_width + mfi);
  const int d0s = __ldg(op.mf_diag + mfi);
  t.dia = d0s != KR_NO_DIAG && t.Wst <= KR_DIAG_MAX;
  // slots that carry a value with the current field (the field kernel's band)
  const int bhi = __ldcg(op.mf_band + 2 * mfi + 1);
  t.empty = bhi < 0;
  const int wlo = (t.dia && !t.empty) ? t.Wst - 1 - __ldcg(op.mf_band + 2 * mfi) : 0;
  t.W = (t.dia && !t.empty) ? bhi - wlo + 1 : t.Wst;
  t.d0 = t.dia ? d0s + wlo : 0;
  t.ktype = __ldg(op.k_type + kb);
  t.mtype = __ldcg(op.mf_type + mfi);
  t.ok = t.nk2 <= KP && t.Wst <= KB_WMAX;
  t.KT = op.k_f32 + __ldg(op.k_off + kb);
  t.col = op.m_col + __ldg(op.mf_col_off + mfi);
  t.mf = op.mf_f32 + __ldg(op.mf_off + mfi) + wlo;
  t.Xs2 = p.X + (long long)__ldg(op.in_off + t.s2) * nb + v;
  return t;
}

// B operands of a term: K^T (b, a) -> row a, column b; parts K_re, K_im, -K_im,
// each hi and lo; zero outside n_k1 x n_k2. MF rows (and ELL columns).
template <int KP>
__device__ __forceinline__ void kbt_stage(const KbtTerm& t, int nk1, int NP, int i0, int nr, float* Bt, float2* MFs,
                                          int* Cs, int tid, int bpart = TC_BPART) {
  for (int e = tid; e < NP * KP; e += 256) {  // producers only
    const int a = e / KP, b = e - (e / KP) * KP;
    float kr = 0.f, ki = 0.f;
    if (a < nk1 && b < t.nk2) {
      if (t.ktype == 0) {
        kr = __ldg(t.KT + ((long long)b * nk1 + a) * 2);
        ki = __ldg(t.KT + ((long long)b * nk1 + a) * 2 + 1);
      } else if (t.ktype == 1) {
        kr = __ldg(t.KT + (long long)b * nk1 + a);
      } else {
        ki = __ldg(t.KT + (long long)b * nk1 + a);
      }
    }
    const uint32_t o = tc_kmajor_off(a, b, KP) >> 2;
    const float krh = tc_tf32(kr), kih = tc_tf32(ki);
    Bt[0 * (bpart / 4) + o] = krh;
    Bt[1 * (bpart / 4) + o] = kr - krh;
    Bt[2 * (bpart / 4) + o] = kih;
    Bt[3 * (bpart / 4) + o] = ki - kih;
    Bt[4 * (bpart / 4) + o] = -kih;
    Bt[5 * (bpart / 4) + o] = -(ki - kih);
  }
  const int W = t.W;
  for (int e = tid; e < nr * W; e += 256) {
    const int r = e / W, w = e - (e / W) * W;
    const long long src = (long long)(i0 + r) * t.Wst + w;
    MFs[r * KB_WMAX + w] = __ldcg(t.mf + src);
    if (!t.dia) Cs[r * KB_WMAX + w] = __ldg(t.col + src);
  }
}

template <int KP>
__device__ __forceinline__ void kbt_zstep(float2 (&z)[64 / KP][KP / 2], KbtWin<KP>& xw, const KbtTerm& t,
                                          long long nb, int i0, int nr, int b0, const float2* MFs, const int* Cs) {
  constexpr int R = 64 / KP, BH = KP / 2;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int q = 0; q < BH; ++q) z[r][q] = make_float2(0.f, 0.f);
  if (!t.ok || t.empty) return;
  if (t.mtype == 1) kbt_mstep<KP, 1>(z, xw, true, t.Xs2, nb, t.nk2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
  else if (t.mtype == 2) kbt_mstep<KP, 2>(z, xw, true, t.Xs2, nb, t.nk2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
  else kbt_mstep<KP, 0>(z, xw, true, t.Xs2, nb, t.nk2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
}

// producer-only barrier (warps 0-7) that leaves the MMA warp out
__device__ __forceinline__ void kbt_producer_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// issues the MMAs of one term (one thread): D_re += Z_re K_re - Z_im K_im,
// D_im += Z_re K_im + Z_im K_re, each product as three TF32 MMAs per K step
// (A hi B hi, A hi B lo, A lo B hi); zero parts of K skipped
template <int KP>
__device__ __forceinline__ void kbt_issue(uint32_t tmem, uint64_t adesc0, uint64_t bdesc, uint32_t idesc, int NP,
                                          int nr, int ktype, int nk2, uint32_t& dinit, int bpart = TC_BPART) {
  constexpr int ATILE = 128 * KP;
  int pd[4], pa[4], pb[4];
  int np = 0;
  if (ktype != 2) {
    pd[np] = 0; pa[np] = 0; pb[np] = 0; ++np;  // re <- Z_re K_re
    pd[np] = 1; pa[np] = 2; pb[np] = 0; ++np;  // im <- Z_im K_re
  }
  if (ktype != 1) {
    pd[np] = 0; pa[np] = 2; pb[np] = 4; ++np;  // re <- Z_im (-K_im)
    pd[np] = 1; pa[np] = 0; pb[np] = 2; ++np;  // im <- Z_re K_im
  }
  const int nks = (nk2 + 7) >> 3;
  // descriptor start addresses advance by (byte offset >> 4)
  for (int r = 0; r < nr; ++r) {
    for (int q = 0; q < np; ++q) {
      const uint32_t dcol = tmem + (uint32_t)((2 * r + pd[q]) * NP);
      const uint32_t dbit = 1u << (2 * r + pd[q]);
      const uint64_t ad = adesc0 + (uint64_t)(((r * 4 + pa[q]) * ATILE * 4) >> 4);
      const uint64_t bd = bdesc + (uint64_t)((pb[q] * bpart) >> 4);
#pragma unroll
      for (int sp = 0; sp < 3; ++sp) {
        const uint64_t a2 = ad + (sp == 2 ? (uint64_t)((ATILE * 4) >> 4) : 0);
        const uint64_t b2 = bd + (sp == 1 ? (uint64_t)(bpart >> 4) : 0);
#pragma unroll
        for (int ks = 0; ks < KP / 8; ++ks) {
          if (ks < nks) {
            tc_mma_tf32(dcol, a2 + 16u * ks, b2 + 16u * ks, idesc, (dinit & dbit) ? 1u : 0u);
            dinit |= dbit;
          }
        }
      }
    }
  }
}

// Warp-specialised pipeline over the terms of the tile. Warps 0-7 (producers)
// compute Z and store the A tiles; warp 8 issues the MMAs. full: the A tiles
// (and the B buffer) of a term are stored (256 arrivals); empty: the MMAs of a
// term are done (tcgen05.commit). The X window of term t + 1 is requested
// before the A tiles of term t are stored, and the MMAs of term t run while
// the producers compute Z of term t + 1.
template <int KP>
__device__ void kbt_tile(const BatchTC& p, int s1, int i0, int nr, char* smem) {
  constexpr int R = 64 / KP, BH = KP / 2;
  constexpr int ATILE = 128 * KP;  // floats of one A tile
  const DevOp& op = p.op;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const bool producer = wid < 8;
  const int vq = wid & 3, b0 = ((wid >> 2) & 1) * BH;
  const int vloc = vq * 32 + lane;
  const long long nb = p.nb;
  const int v = blockIdx.y * 128 + vloc;
  float* As = reinterpret_cast<float*>(smem);
  char* Bs = smem + TC_ABYTES;
  float2* MFs0 = reinterpret_cast<float2*>(Bs + 2 * TC_BBYTES);          // [2][8][KB_WMAX]
  int* Cs0 = reinterpret_cast<int*>(Bs + 2 * TC_BBYTES + TC_MFBYTES);   // [2][8][KB_WMAX]
  uint64_t* full = reinterpret_cast<uint64_t*>(Bs + 2 * TC_BBYTES + TC_MFBYTES + TC_CSBYTES);
  uint64_t* empty = full + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(full + 2);
  const int nk1 = __ldg(op.out_dk + s1);
  const int NP = nk1 <= 16 ? 16 : 32;
  float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * nk1) * nb + v;
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  if (te == tb) {  // no term reaches this slab
    if (producer)
      for (int e = wid >> 2; e < nr * nk1; e += 2) Y[(long long)e * nb] = make_float2(0.f, 0.f);
    return;
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(2 * R * NP)) ncols <<= 1;
  if (wid == 8) tc_alloc(tslot, ncols);
  if (tid == 256) {
    tc_mbar_init(full, 256);
    tc_mbar_init(empty, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  int ncommit = 0;  // terms whose MMAs were (or will be) committed

  if (!producer) {
    // ---- MMA warp (warp 8; warp 9 idles here) ------------------------------
    if (wid == 8 && lane == 0) {
      const uint32_t idesc = tc_idesc_tf32(128, NP);
      const uint64_t adesc0 = tc_desc(tc_smem_u32(As), 128u, 32u * KP);
      const uint64_t bdesc0 = tc_desc(tc_smem_u32(Bs), 128u, 32u * KP);
      uint32_t dinit = 0;
      for (int term = tb; term < te; ++term) {
        const int s2 = __ldg(op.t_in + term);
        const int nk2 = __ldg(op.in_dk + s2);
        const int W = __ldg(op.mf_width + __ldg(op.t_mf + term));
        if (!(nk2 <= KP && W <= KB_WMAX)) continue;
        if (__ldcg(op.mf_band + 2 * __ldg(op.t_mf + term) + 1) < 0) continue;  // MF zero with this field
        const int ktype = __ldg(op.k_type + __ldg(op.t_k + term));
        if (!tc_mbar_wait(full, (uint32_t)ncommit & 1u)) ok = false;
        tc_fence_after();
        const uint64_t bdesc = bdesc0 + (uint64_t)((((term - tb) & 1) * TC_BBYTES) >> 4);
        kbt_issue<KP>(tmem, adesc0, bdesc, idesc, NP, nr, ktype, nk2, dinit);
        tc_commit(empty);
        ++ncommit;
      }
      if (!ok) atomicExch(p.err, KR_ERR_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    if (wid == 8) tc_dealloc(tmem, ncols);
    return;
  }

  // ---- producers -----------------------------------------------------------
  float2 z[R][BH];
  KbtWin<KP> xw;
  KbtTerm cur = kbt_term(op, p, tb, KP, v, nb);
  if (cur.ok && !cur.empty && cur.dia) xw.load(cur.Xs2, nb, cur.nk2, cur.dm2, i0 + cur.d0, nr + cur.W - 1, b0);
  kbt_stage<KP>(cur, nk1, NP, i0, nr, reinterpret_cast<float*>(Bs), MFs0, Cs0, tid);
  kbt_producer_sync();
  kbt_zstep<KP>(z, xw, cur, nb, i0, nr, b0, MFs0, Cs0);
  for (int term = tb; term < te; ++term) {
    const int buf = (term - tb) & 1;
    const bool has_next = term + 1 < te;
    KbtTerm nxt;
    if (has_next) {
      nxt = kbt_term(op, p, term + 1, KP, v, nb);
      if (nxt.ok && !nxt.empty && nxt.dia) xw.load(nxt.Xs2, nb, nxt.nk2, nxt.dm2, i0 + nxt.d0, nr + nxt.W - 1, b0);
    }
    // the MMAs of the previous committed term are done with the A tiles and its B buffer
    if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
    tc_fence_after();
    if (cur.ok && !cur.empty) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) continue;
        float* At = As + r * 4 * ATILE;
#pragma unroll
        for (int c4 = 0; c4 < BH; c4 += 4) {
          float4 rh, rl, ih, il;
          float* prh = &rh.x;
          float* prl = &rl.x;
          float* pih = &ih.x;
          float* pil = &il.x;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float2 zz = z[r][c4 + q];
            prh[q] = tc_tf32(zz.x);
            prl[q] = zz.x - prh[q];
            pih[q] = tc_tf32(zz.y);
            pil[q] = zz.y - pih[q];
          }
          const uint32_t o = tc_kmajor_off(vloc, b0 + c4, KP) >> 2;
          *reinterpret_cast<float4*>(At + 0 * ATILE + o) = rh;
          *reinterpret_cast<float4*>(At + 1 * ATILE + o) = rl;
          *reinterpret_cast<float4*>(At + 2 * ATILE + o) = ih;
          *reinterpret_cast<float4*>(At + 3 * ATILE + o) = il;
        }
      }
      tc_fence_proxy();
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem_u32(full)) : "memory");
      ++ncommit;
    } else if (!cur.ok && tid == 0) {
      atomicExch(p.err, KR_ERR_ARG);  // outside the tile shape: skipped
    }
    if (has_next) {
      // B buffer buf ^ 1 was last read by the MMAs of term - 1 (done); MF buffer
      // buf ^ 1 by the M step of term - 1 (every producer is past it)
      kbt_stage<KP>(nxt, nk1, NP, i0, nr, reinterpret_cast<float*>(Bs + (buf ^ 1) * TC_BBYTES),
                    MFs0 + (buf ^ 1) * 8 * KB_WMAX, Cs0 + (buf ^ 1) * 8 * KB_WMAX, tid);
      kbt_producer_sync();
      kbt_zstep<KP>(z, xw, nxt, nb, i0, nr, b0, MFs0 + (buf ^ 1) * 8 * KB_WMAX, Cs0 + (buf ^ 1) * 8 * KB_WMAX);
      cur = nxt;
    }
  }
  if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
  tc_fence_after();
  // epilogue: rows r = w / 4, w / 4 + 2, ... of this warp's lane quarter
  for (int r = wid >> 2; r < nr; r += 2) {
    for (int c0 = 0; c0 < NP; c0 += 16) {
      float re[16], im[16];
      const uint32_t lanebase = (uint32_t)(vq * 32) << 16;
      tc_ld16(tmem + lanebase + (uint32_t)(2 * r * NP + c0), re);
      tc_ld16(tmem + lanebase + (uint32_t)((2 * r + 1) * NP + c0), im);
      const bool any = ncommit > 0;
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (c0 + q < nk1)
          Y[((long long)r * nk1 + c0 + q) * nb] = any ? make_float2(re[q], im[q]) : make_float2(0.f, 0.f);
    }
  }
  if (!ok && lane == 0) atomicExch(p.err, KR_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
}


// ---------------------------------------------------------------------------
// Tensor-core tile with the X windows streamed by TMA (KP = 8, 16). Warp 8
// lane 1 walks the window rows of every diagonal term of the tile in order
// and loads each (KP input rows x 128 vectors, KP/8 boxes of 8 rows) into a
// ring of shared-memory slots (full: tx bytes; empty: one arrival per
// producer warp); the producer warps read X from the ring, so no global-load
// latency sits in their M step. Rows outside the input slab read whatever
// lies there (finite data of other slabs, or zeros beyond the array) and meet
// zero MF slots; columns beyond n_k2 are zeroed on read. Terms stored as ELL
// load X directly. Everything else as in kbt_tile.
// ---------------------------------------------------------------------------
constexpr int KBT_MAXT = 64;  // terms of one output slab held in the shared-memory table

// the next term's B and MF values, loaded into registers before they are staged
struct KbtPre {
  float kr[2], ki[2];
  float2 mf;
  int col;
};

template <int KP>
__device__ __forceinline__ void kbt_preload(const KbtTerm& t, int nk1, int NP, int i0, int nr, int tid, KbtPre& q) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = tid + 256 * u;
    const int a = e / KP, b = e - (e / KP) * KP;
    float kr = 0.f, ki = 0.f;
    if (e < NP * KP && a < nk1 && b < t.nk2) {
      if (t.ktype == 0) {
        kr = __ldg(t.KT + ((long long)b * nk1 + a) * 2);
        ki = __ldg(t.KT + ((long long)b * nk1 + a) * 2 + 1);
      } else if (t.ktype == 1) {
        kr = __ldg(t.KT + (long long)b * nk1 + a);
      } else {
        ki = __ldg(t.KT + (long long)b * nk1 + a);
      }
    }
    q.kr[u] = kr;
    q.ki[u] = ki;
  }
  q.mf = make_float2(0.f, 0.f);
  q.col = 0;
  if (tid < nr * t.W) {
    const int r = tid / t.W, w = tid - (tid / t.W) * t.W;
    const long long src = (long long)(i0 + r) * t.Wst + w;
    q.mf = __ldcg(t.mf + src);
    if (!t.dia) q.col = __ldg(t.col + src);
  }
}

template <int KP>
__device__ __forceinline__ void kbt_stage_pre(const KbtTerm& t, const KbtPre& q, int NP, int nr, float* Bt,
                                              float2* MFs, int* Cs, int tid, int bpart) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = tid + 256 * u;
    if (e >= NP * KP) break;
    const int a = e / KP, b = e - (e / KP) * KP;
    const uint32_t o = tc_kmajor_off(a, b, KP) >> 2;
    const float kr = q.kr[u], ki = q.ki[u];
    const float krh = tc_tf32(kr), kih = tc_tf32(ki);
    Bt[0 * (bpart / 4) + o] = krh;
    Bt[1 * (bpart / 4) + o] = kr - krh;
    Bt[2 * (bpart / 4) + o] = kih;
    Bt[3 * (bpart / 4) + o] = ki - kih;
    Bt[4 * (bpart / 4) + o] = -kih;
    Bt[5 * (bpart / 4) + o] = -(ki - kih);
  }
  if (tid < nr * t.W) {
    const int r = tid / t.W, w = tid - (tid / t.W) * t.W;
    MFs[r * KB_WMAX + w] = q.mf;
    if (!t.dia) Cs[r * KB_WMAX + w] = q.col;
  }
}

template <int KP>
struct KbtRing {
  static constexpr int NSLOT = 64 / KP;          // slots of KP rows x 128 vectors x 8 bytes
  static constexpr int SLOT = KP * 1024;
  static constexpr int BPART = 128 * KP;         // one B part: NP (<= 32) x KP FP32
  static constexpr int BBUF = 6 * BPART;
  static constexpr int OFF_B = TC_ABYTES;
  static constexpr int OFF_RING = OFF_B + 2 * BBUF;
  static constexpr int OFF_MF = OFF_RING + NSLOT * SLOT;
  static constexpr int OFF_CS = OFF_MF + TC_MFBYTES;
  static constexpr int OFF_BAR = OFF_CS + TC_CSBYTES;
  static constexpr int OFF_TAB = OFF_BAR + 8 * (2 + 2 * NSLOT) + 16;  // term table (KBT_MAXT entries)
  static constexpr int TOTAL = OFF_TAB + KBT_MAXT * (int)sizeof(KbtTerm);
};
constexpr int TC_SMEM_RING = KbtRing<16>::TOTAL > KbtRing<8>::TOTAL ? KbtRing<16>::TOTAL : KbtRing<8>::TOTAL;

// the ring rows of one term: count, and the first input row (diagonal terms only)
__device__ __forceinline__ int kbt_ring_rows(const KbtTerm& t, int nr) {
  return (t.ok && !t.empty && t.dia) ? nr + t.W - 1 : 0;
}

// M step of a diagonal term from the ring; g: ring row counter (advanced)
template <int KP, int MT>
__device__ __forceinline__ bool kbt_mdia_ring(float2 (&z)[64 / KP][KP / 2], const char* ring, uint64_t* rfull,
                                              uint64_t* rempty, int& g, int nwin, int nr, int W, int nk2, int b0,
                                              int vloc, int lane, const float2* MFs) {
  constexpr int R = 64 / KP, BH = KP / 2, NSLOT = KbtRing<KP>::NSLOT;
  bool ok = true;
  for (int c = 0; c < nwin; ++c, ++g) {
    const int slot = g % NSLOT;
    if (!tc_mbar_wait(rfull + slot, (uint32_t)(g / NSLOT) & 1u)) ok = false;
    const float2* xs = reinterpret_cast<const float2*>(ring + (size_t)slot * KbtRing<KP>::SLOT) + vloc;
    float2 x[BH];
#pragma unroll
    for (int q = 0; q < BH; ++q) x[q] = (b0 + q < nk2) ? xs[(b0 + q) * 128] : make_float2(0.f, 0.f);
    __syncwarp();
    if (lane == 0) tc_mbar_arrive(rempty + slot);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int w = c - r;
      if (w >= 0 && w < W && r < nr) {
        const float2 m = MFs[r * KB_WMAX + w];
#pragma unroll
        for (int q = 0; q < BH; ++q) macc<MT>(z[r][q], m, x[q]);
      }
    }
  }
  return ok;
}

template <int KP>
__device__ __forceinline__ bool kbt_zstep_ring(float2 (&z)[64 / KP][KP / 2], const KbtTerm& t, long long nb, int nr,
                                               int b0, int vloc, int lane, const float2* MFs, const int* Cs,
                                               const char* ring, uint64_t* rfull, uint64_t* rempty, int& g) {
  constexpr int R = 64 / KP, BH = KP / 2;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int q = 0; q < BH; ++q) z[r][q] = make_float2(0.f, 0.f);
  if (!t.ok || t.empty) return true;
  const int nwin = kbt_ring_rows(t, nr);
  if (t.dia) {
    if (t.mtype == 1) return kbt_mdia_ring<KP, 1>(z, ring, rfull, rempty, g, nwin, nr, t.W, t.nk2, b0, vloc, lane, MFs);
    if (t.mtype == 2) return kbt_mdia_ring<KP, 2>(z, ring, rfull, rempty, g, nwin, nr, t.W, t.nk2, b0, vloc, lane, MFs);
    return kbt_mdia_ring<KP, 0>(z, ring, rfull, rempty, g, nwin, nr, t.W, t.nk2, b0, vloc, lane, MFs);
  }
  if (t.mtype == 1) kbt_mell<KP, 1>(z, t.Xs2, nb, t.nk2, nr, t.W, b0, MFs, Cs);
  else if (t.mtype == 2) kbt_mell<KP, 2>(z, t.Xs2, nb, t.nk2, nr, t.W, b0, MFs, Cs);
  else kbt_mell<KP, 0>(z, t.Xs2, nb, t.nk2, nr, t.W, b0, MFs, Cs);
  return true;
}

template <int KP>
__device__ void kbt_tile_ring(const BatchTC& p, const CUtensorMap* xmap, int s1, int i0, int nr, char* smem) {
  using L = KbtRing<KP>;
  constexpr int R = 64 / KP, BH = KP / 2, NSLOT = L::NSLOT;
  constexpr int ATILE = 128 * KP;  // floats of one A tile
  const DevOp& op = p.op;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const bool producer = wid < 8;
  const int vq = wid & 3, b0 = ((wid >> 2) & 1) * BH;
  const int vloc = vq * 32 + lane;
  const long long nb = p.nb;
  const int v = blockIdx.y * 128 + vloc;
  float* As = reinterpret_cast<float*>(smem);
  char* Bs = smem + L::OFF_B;
  char* ring = smem + L::OFF_RING;
  float2* MFs0 = reinterpret_cast<float2*>(smem + L::OFF_MF);  // [2][8][KB_WMAX]
  int* Cs0 = reinterpret_cast<int*>(smem + L::OFF_CS);         // [2][8][KB_WMAX]
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
  uint64_t* empty = full + 1;
  uint64_t* rfull = full + 2;
  uint64_t* rempty = rfull + NSLOT;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(rempty + NSLOT);
  KbtTerm* tab = reinterpret_cast<KbtTerm*>(smem + L::OFF_TAB);
  const int nk1 = __ldg(op.out_dk + s1);
  const int NP = nk1 <= 16 ? 16 : 32;
  float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * nk1) * nb + v;
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  if (te == tb) {  // no term reaches this slab
    if (producer)
      for (int e = wid >> 2; e < nr * nk1; e += 2) Y[(long long)e * nb] = make_float2(0.f, 0.f);
    return;
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(2 * R * NP)) ncols <<= 1;
  if (wid == 8) tc_alloc(tslot, ncols);
  if (tid == 256) {
    tc_mbar_init(full, 256);
    tc_mbar_init(empty, 1);
    for (int i = 0; i < NSLOT; ++i) {
      tc_mbar_init(rfull + i, 1);
      tc_mbar_init(rempty + i, 8);
    }
  }
  // term table: the tables of every term of the slab, read once per tile
  const int nt = te - tb;
  const bool use_tab = nt <= KBT_MAXT;
  if (use_tab)
    for (int i = tid; i < nt; i += blockDim.x) tab[i] = kbt_term(op, p, tb + i, KP, 0, nb);
  auto term_at = [&](int i) {
    KbtTerm tt = use_tab ? tab[i] : kbt_term(op, p, tb + i, KP, 0, nb);
    tt.Xs2 += v;
    return tt;
  };
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  int ncommit = 0;  // terms whose MMAs were (or will be) committed

  if (!producer) {
    if (wid == 8 && lane == 0) {
      // ---- MMA issue -------------------------------------------------------
      const uint32_t idesc = tc_idesc_tf32(128, NP);
      const uint64_t adesc0 = tc_desc(tc_smem_u32(As), 128u, 32u * KP);
      const uint64_t bdesc0 = tc_desc(tc_smem_u32(Bs), 128u, 32u * KP);
      uint32_t dinit = 0;
      for (int term = tb; term < te; ++term) {
        const KbtTerm tt = term_at(term - tb);
        if (!tt.ok || tt.empty) continue;  // skipped by the producers as well
        if (!tc_mbar_wait(full, (uint32_t)ncommit & 1u)) ok = false;
        tc_fence_after();
        const uint64_t bdesc = bdesc0 + (uint64_t)((((term - tb) & 1) * L::BBUF) >> 4);
        kbt_issue<KP>(tmem, adesc0, bdesc, idesc, NP, nr, tt.ktype, tt.nk2, dinit, L::BPART);
        tc_commit(empty);
        ++ncommit;
      }
    } else if (wid == 9 && lane == 0) {
      // ---- X window loads (TMA) into the ring (own warp: a waiting MMA lane
      // would hold up a loader lane of the same warp) ------------------------
      int g = 0;
      for (int term = tb; term < te; ++term) {
        const KbtTerm t = term_at(term - tb);
        const int nwin = kbt_ring_rows(t, nr);
        const long long row0 = __ldg(op.in_off + t.s2);  // first X row of slab s2
        for (int c = 0; c < nwin; ++c, ++g) {
          const int slot = g % NSLOT;
          if (g >= NSLOT && !tc_mbar_wait(rempty + slot, (uint32_t)(g / NSLOT - 1) & 1u)) ok = false;
          tc_mbar_expect_tx(rfull + slot, (uint32_t)L::SLOT);
          const long long y = row0 + (long long)(i0 + t.d0 + c) * t.nk2;  // first X row of the window row
          char* dst = ring + (size_t)slot * L::SLOT;
#pragma unroll
          for (int h = 0; h < KP / 8; ++h)
            tc_tma_load_2d(dst + h * 8192, xmap, blockIdx.y * 128, (int)(y + 8 * h), rfull + slot);
        }
      }
    }
    if (!ok) atomicExch(p.err, KR_ERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (wid == 8) tc_dealloc(tmem, ncols);
    return;
  }

  // ---- producers -------------------------------------------------------------
  float2 z[R][BH];
  int g = 0;  // ring row counter
  KbtTerm cur = term_at(0);
  KbtPre pre;
  kbt_preload<KP>(cur, nk1, NP, i0, nr, tid, pre);
  kbt_stage_pre<KP>(cur, pre, NP, nr, reinterpret_cast<float*>(Bs), MFs0, Cs0, tid, L::BPART);
  kbt_producer_sync();
  if (!kbt_zstep_ring<KP>(z, cur, nb, nr, b0, vloc, lane, MFs0, Cs0, ring, rfull, rempty, g)) ok = false;
  for (int term = tb; term < te; ++term) {
    const int buf = (term - tb) & 1;
    const bool has_next = term + 1 < te;
    KbtTerm nxt;
    if (has_next) {  // the next term's K and MF values in flight during the A-tile hand-off
      nxt = term_at(term + 1 - tb);
      kbt_preload<KP>(nxt, nk1, NP, i0, nr, tid, pre);
    }
    // the MMAs of the previous committed term are done with the A tiles and its B buffer
    if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
    tc_fence_after();
    if (cur.ok && !cur.empty) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) continue;
        float* At = As + r * 4 * ATILE;
#pragma unroll
        for (int c4 = 0; c4 < BH; c4 += 4) {
          float4 rh, rl, ih, il;
          float* prh = &rh.x;
          float* prl = &rl.x;
          float* pih = &ih.x;
          float* pil = &il.x;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float2 zz = z[r][c4 + q];
            prh[q] = tc_tf32(zz.x);
            prl[q] = zz.x - prh[q];
            pih[q] = tc_tf32(zz.y);
            pil[q] = zz.y - pih[q];
          }
          const uint32_t o = tc_kmajor_off(vloc, b0 + c4, KP) >> 2;
          *reinterpret_cast<float4*>(At + 0 * ATILE + o) = rh;
          *reinterpret_cast<float4*>(At + 1 * ATILE + o) = rl;
          *reinterpret_cast<float4*>(At + 2 * ATILE + o) = ih;
          *reinterpret_cast<float4*>(At + 3 * ATILE + o) = il;
        }
      }
      tc_fence_proxy();
      tc_mbar_arrive(full);
      ++ncommit;
    } else if (!cur.ok && tid == 0) {
      atomicExch(p.err, KR_ERR_ARG);  // outside the tile shape: skipped
    }
    if (has_next) {
      // B buffer buf ^ 1 was last read by the MMAs of term - 1 (done); MF buffer
      // buf ^ 1 by the M step of term - 1 (every producer is past it)
      kbt_stage_pre<KP>(nxt, pre, NP, nr, reinterpret_cast<float*>(Bs + (buf ^ 1) * L::BBUF),
                        MFs0 + (buf ^ 1) * 8 * KB_WMAX, Cs0 + (buf ^ 1) * 8 * KB_WMAX, tid, L::BPART);
      kbt_producer_sync();
      if (!kbt_zstep_ring<KP>(z, nxt, nb, nr, b0, vloc, lane, MFs0 + (buf ^ 1) * 8 * KB_WMAX,
                              Cs0 + (buf ^ 1) * 8 * KB_WMAX, ring, rfull, rempty, g))
        ok = false;
      cur = nxt;
    }
  }
  if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
  tc_fence_after();
  // epilogue: rows r = w / 4, w / 4 + 2, ... of this warp's lane quarter
  for (int r = wid >> 2; r < nr; r += 2) {
    for (int c0 = 0; c0 < NP; c0 += 16) {
      float re[16], im[16];
      const uint32_t lanebase = (uint32_t)(vq * 32) << 16;
      tc_ld16(tmem + lanebase + (uint32_t)(2 * r * NP + c0), re);
      tc_ld16(tmem + lanebase + (uint32_t)((2 * r + 1) * NP + c0), im);
      const bool any = ncommit > 0;
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (c0 + q < nk1)
          Y[((long long)r * nk1 + c0 + q) * nb] = any ? make_float2(re[q], im[q]) : make_float2(0.f, 0.f);
    }
  }
  if (!ok && lane == 0) atomicExch(p.err, KR_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
}

__global__ void __launch_bounds__(320, 1) kb_matvec_tc(BatchTC p, const __grid_constant__ CUtensorMap xmap) {
  extern __shared__ __align__(1024) char kbt_smem[];
  if (p.grp_active) {
    const int* g = p.grp_active + 4 * blockIdx.y;
    if (!(g[0] | g[1] | g[2] | g[3])) return;
  }
  const int task = blockIdx.x;
  const int s1 = __ldg(p.task + task);
  const int i0 = __ldg(p.task + p.ntask + task);
  const int nr = __ldg(p.task + 2 * p.ntask + task);
  const int kp = __ldg(p.task + 3 * p.ntask + task);
  if (kp == 8) kbt_tile_ring<8>(p, &xmap, s1, i0, nr, kbt_smem);
  else if (kp == 16) kbt_tile_ring<16>(p, &xmap, s1, i0, nr, kbt_smem);
  else kbt_tile<32>(p, s1, i0, nr, kbt_smem);
}

// any active vector per 32-vector group
__global__ void kb_group_active(const int* active, int* grp, int ngrp) {
  const int g = blockIdx.x * blockDim.y + threadIdx.y;
  if (g >= ngrp) return;
  const int any = __any_sync(0xffffffffu, active[g * 32 + threadIdx.x] != 0);
  if (threadIdx.x == 0) grp[g] = any;
}

// ===========================================================================
// C ABI
// ===========================================================================
namespace {
template <typename T>
int balloc(kr_batch* b, size_t count, T** p) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(T) * std::max<size_t>(count, 1));
  if (e != cudaSuccess) return set_err(b->op->ctx, KR_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  cudaMemset(q, 0, sizeof(T) * std::max<size_t>(count, 1));
  b->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return KR_OK;
}
int mv_groups(const kr_batch* b) { return b->nb / 32; }
const char* const mv_error_text =
    "batched mat-vec: an MMA completion wait gave up or a term exceeded the tile shape";

// TMA descriptor of an X buffer [dim][nb] (complex64 as 8-byte elements):
// boxes of 128 vectors x 8 rows, zero fill outside the array
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
int encode_xmap(kr_ctx* ctx, const float2* X, long long dim, int nb, CUtensorMap* m) {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  if (!fn) return set_err(ctx, KR_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t gdim[2] = {(cuuint64_t)nb, (cuuint64_t)dim};
  const cuuint64_t gstride[1] = {(cuuint64_t)nb * sizeof(float2)};
  const cuuint32_t box[2] = {128, 8};
  const cuuint32_t estride[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<float2*>(X), gdim, gstride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(ctx, KR_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return KR_OK;
}

int launch_matvec(kr_batch* b, kr_op* op, const float2* X, float2* Y, bool masked, cudaStream_t st) {
  if (b->mv_kind == KR_MATVEC_TENSOR && op->tc_ntask > 0) {
    BatchTC q;
    q.op = op->dev;
    q.X = X;
    q.Y = Y;
    q.nb = b->nb;
    q.task = op->tc_task;
    q.ntask = op->tc_ntask;
    q.grp_active = masked ? b->grp_active : nullptr;
    q.err = b->counts + 2;
    CUtensorMap xmap;
    const int rc = encode_xmap(op->ctx, X, b->dim, b->nb, &xmap);
    if (rc != KR_OK) return rc;
    const int smem = std::max(TC_SMEM, TC_SMEM_RING);
    // per device (the attribute belongs to the current device's context)
    KR_CUDA(op->ctx, cudaFuncSetAttribute(kb_matvec_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kb_matvec_tc<<<dim3(op->tc_ntask, b->nb / 128), 320, smem, st>>>(q, xmap);
    b->launches++;
    KR_CUDA(op->ctx, cudaGetLastError());
    return KR_OK;
  }
  BatchMV p;
  p.op = op->dev;
  p.X = X;
  p.Y = Y;
  p.nb = b->nb;
  p.task_slab = b->task_slab;
  p.task_i0 = b->task_i0;
  p.task_nr = b->task_nr;
  p.grp_active = masked ? b->grp_active : nullptr;
  const size_t smem = kb_matvec_smem();
  KR_CUDA(op->ctx, cudaFuncSetAttribute(kb_matvec, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(b->ntask, mv_groups(b));
  kb_matvec<<<grid, 256, smem, st>>>(p);
  b->launches++;
  KR_CUDA(op->ctx, cudaGetLastError());
  return KR_OK;
}
}  // namespace

extern "C" int kr_batch_create(kr_op* op, int64_t nvec, int32_t mmax, kr_batch** out) {
  if (!op || !out || nvec <= 0 || mmax < 2 || mmax > KB_NK_MAX - 1)
    return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_batch_create: bad argument (2 <= mmax <= 31)");
  *out = nullptr;
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_batch_create: operator is not square");
  KR_CUDA(op->ctx, cudaSetDevice(op->ctx->device));
  // the batched mat-vec supports n_k <= 32 and ELL widths <= 16
  std::vector<int> dk(op->dev.nslab_out), dm(op->dev.nslab_out);
  KR_CUDA(op->ctx, cudaMemcpy(dk.data(), op->dev.out_dk, sizeof(int) * dk.size(), cudaMemcpyDeviceToHost));
  KR_CUDA(op->ctx, cudaMemcpy(dm.data(), op->dev.out_dm, sizeof(int) * dm.size(), cudaMemcpyDeviceToHost));
  for (int x : dk)
    if (x > KB_NK_MAX) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_batch_create: n_k above 32 not supported");
  std::vector<int> widths(std::max(1, op->nmf));
  KR_CUDA(op->ctx, cudaMemcpy(widths.data(), op->dev.mf_width, sizeof(int) * op->nmf, cudaMemcpyDeviceToHost));
  for (int i = 0; i < op->nmf; ++i)
    if (widths[i] > KB_WMAX)
      return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_batch_create: M band wider than 16 entries per row");
  kr_batch* b = new kr_batch();
  b->op = op;
  b->nvec = (int)nvec;
  b->nb = (int)((nvec + 127) / 128 * 128);
  b->mmax = mmax;
  b->dim = op->dev.dim_out;
  const size_t nb = b->nb, dim = b->dim, m1 = mmax + 1;
  int rc = KR_OK;
#define BA(count, ptr) \
  if ((rc = balloc(b, (count), (ptr))) != KR_OK) { kr_batch_destroy(b); return rc; }
  BA(dim * nb, &b->S);
  BA(dim, &b->phase_df);
  BA(m1 * dim * nb, &b->V);
  BA(dim * nb, &b->W);
  BA(nb, &b->norm0);
  BA(m1 * nb, &b->h);
  BA(m1 * nb, &b->alpha);
  BA(m1 * nb, &b->beta);
  BA(m1 * nb, &b->c);
  BA(nb, &b->vscale);
  BA(nb, &b->kconv);
  BA(nb, &b->active);
  BA((size_t)mv_groups(b), &b->grp_active);
  BA(nb, &b->err);
  BA((size_t)KB_RED_CHUNKS * (m1 + 1) * nb, &b->part);
  BA(3, &b->counts);
  // output tiles: R = 128 / NKP rows of one slab (NKP = n_k rounded up to 4, 8, 16, 32)
  std::vector<int> ts, ti, tn;
  for (int s = 0; s < (int)dm.size(); ++s) {
    const int nkp = dk[s] <= 4 ? 4 : dk[s] <= 8 ? 8 : dk[s] <= 16 ? 16 : 32;
    const int R = 128 / nkp;
    for (int i0 = 0; i0 < dm[s]; i0 += R) {
      ts.push_back(s);
      ti.push_back(i0);
      tn.push_back(std::min(R, dm[s] - i0));
    }
  }
  b->ntask = (int)ts.size();
  b->nslab = (int)dk.size();
  std::vector<long long> soff(b->nslab), slen(b->nslab);
  {
    long long o = 0;
    for (int s = 0; s < b->nslab; ++s) {
      soff[s] = o;
      slen[s] = (long long)dk[s] * dm[s];
      o += slen[s];
    }
  }
  BA(b->nslab, &b->slab_off);
  BA(b->nslab, &b->slab_len);
  BA((size_t)b->nslab * nb, &b->pop);
  BA(ts.size(), &b->task_slab);
  BA(ti.size(), &b->task_i0);
  BA(tn.size(), &b->task_nr);
#undef BA
  cudaError_t ce = cudaMemcpy(b->task_slab, ts.data(), sizeof(int) * ts.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->slab_off, soff.data(), sizeof(long long) * soff.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->slab_len, slen.data(), sizeof(long long) * slen.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->task_i0, ti.data(), sizeof(int) * ti.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->task_nr, tn.data(), sizeof(int) * tn.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) {
    kr_batch_destroy(b);
    return set_err(op->ctx, KR_ERR_CUDA, std::string("kr_batch_create: ") + cudaGetErrorString(ce));
  }
  *out = b;
  return KR_OK;
}

extern "C" void kr_batch_destroy(kr_batch* b) {
  if (!b) return;
  for (void* p : b->allocs) cudaFree(p);
  delete b;
}

extern "C" int kr_batch_load(kr_batch* b, const void* states, void* stream) {
  if (!b || !states) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_load: bad argument");
  dim3 grid((unsigned)((b->dim + 31) / 32), b->nb / 32);
  kb_transpose_in<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const double2*)states, b->S, b->dim, b->nvec, b->nb);
  b->launches++;
  KR_CUDA(b->op->ctx, cudaGetLastError());
  return KR_OK;
}

extern "C" int kr_batch_store(kr_batch* b, void* states, void* stream) {
  if (!b || !states) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_store: bad argument");
  dim3 grid((unsigned)((b->dim + 31) / 32), b->nb / 32);
  kb_transpose_out<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(b->S, (double2*)states, b->dim, b->nvec, b->nb);
  b->launches++;
  KR_CUDA(b->op->ctx, cudaGetLastError());
  return KR_OK;
}

extern "C" int kr_batch_step(kr_batch* b, kr_op* op, const void* phase, double fac_re, double fac_im, double tol,
                             int32_t* kmax_out, void* stream) {
  if (!b || !op) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_step: bad argument");
  if (op->dev.dim_out != b->dim || !op->square)
    return set_err(op->ctx, KR_ERR_ARG, "kr_batch_step: operator does not match the batch basis");
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = b->nb;
  const long long dim = b->dim;
  const dim3 eg(KB_RED_CHUNKS, nb / 32), eb(32, 8);
  const int stride = b->mmax + 2;
  const double2 fac = make_double2(fac_re, fac_im);
  kr_ctx* ctx = op->ctx;
  KR_CUDA(ctx, cudaMemsetAsync(b->counts, 0, 3 * sizeof(int), st));
  // S <- phase * S, norms, V_0
  const float4* pdf = nullptr;
  if (phase) {
    kb_phase_df<<<(int)std::min<long long>((dim + 255) / 256, 1024), 256, 0, st>>>((const double2*)phase, b->phase_df,
                                                                                dim);
    b->launches++;
    pdf = b->phase_df;
  }
  kb_phase_norm<<<eg, eb, 0, st>>>(b->S, pdf, dim, nb, b->part);
  kb_reduce<<<(nb + 255) / 256, 256, 0, st>>>(b->part, 1, nb, 1, b->h);
  kb_start<<<eg, eb, 0, st>>>(b->S, b->V, b->h, b->norm0, b->active, b->kconv, b->vscale, dim, nb, b->nvec);
  b->launches += 3;
  KR_CUDA(ctx, cudaGetLastError());
  int kused = 0;
  for (int k = 0; k < b->mmax; ++k) {
    kb_group_active<<<(mv_groups(b) + 7) / 8, dim3(32, 8), 0, st>>>(b->active, b->grp_active, mv_groups(b));
    int rc = launch_matvec(b, op, b->V + (long long)k * dim * nb, b->W, true, st);
    if (rc) return rc;
    kb_dots<<<eg, eb, 0, st>>>(b->V, b->W, b->active, dim, nb, k, stride, b->part);
    kb_reduce<<<((k + 1) * nb + 255) / 256, 256, 0, st>>>(b->part, k + 1, nb, stride, b->h);
    kb_update<<<eg, eb, 0, st>>>(b->V, b->W, b->h, b->active, dim, nb, k, b->part);
    // norms of V_{k+1} into the last coefficient slot of h (slot mmax + 1 is not a dot)
    kb_reduce<<<(nb + 255) / 256, 256, 0, st>>>(b->part, 1, nb, 1, b->h + (long long)(b->mmax) * nb);
    KR_CUDA(ctx, cudaMemsetAsync(b->counts, 0, 2 * sizeof(int), st));
    kb_small<<<(nb + 127) / 128, 128, 0, st>>>(dev_view(b), k, fac, tol, b->h + (long long)(b->mmax) * nb);
    kb_scale<<<eg, eb, 0, st>>>(b->V + (long long)(k + 1) * dim * nb, b->vscale, b->active, dim, nb);
    b->launches += 7;
    KR_CUDA(ctx, cudaGetLastError());
    int counts[3] = {0, 0, 0};
    KR_CUDA(ctx, cudaMemcpyAsync(counts, b->counts, sizeof(counts), cudaMemcpyDeviceToHost, st));
    KR_CUDA(ctx, cudaStreamSynchronize(st));
    kused = k + 1;
    if (counts[2] != 0) return set_err(ctx, counts[2], mv_error_text);
    if (counts[1] > 0)
      return set_err(ctx, KR_ERR_MAXORDER,
                     "batched Lanczos: " + std::to_string(counts[1]) + " vectors did not reach the tolerance within " +
                         std::to_string(b->mmax) + " Krylov vectors");
    if (counts[0] == 0) break;
  }
  kb_combine<<<eg, eb, 0, st>>>(dev_view(b), pdf);
  b->launches++;
  KR_CUDA(ctx, cudaGetLastError());
  if (kmax_out) *kmax_out = kused;
  return KR_OK;
}

extern "C" int kr_batch_korder(kr_batch* b, int32_t* korder, void* stream) {
  if (!b || !korder) return KR_ERR_ARG;
  KR_CUDA(b->op->ctx, cudaMemcpyAsync(korder, b->kconv, sizeof(int) * b->nvec, cudaMemcpyDeviceToHost,
                                      (cudaStream_t)stream));
  KR_CUDA(b->op->ctx, cudaStreamSynchronize((cudaStream_t)stream));
  return KR_OK;
}

extern "C" int kr_batch_expect(kr_batch* b, kr_op* obs, double* out, void* stream) {
  if (!b || !obs || !out) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_expect: bad argument");
  if (obs->dev.dim_out != b->dim || !obs->square)
    return set_err(obs->ctx, KR_ERR_ARG, "kr_batch_expect: observable does not match the batch basis");
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = b->dim * b->nb;
  float2* X = b->V;  // basis slot 0 and W are free between steps
  KR_CUDA(obs->ctx, cudaMemsetAsync(b->counts + 2, 0, sizeof(int), st));
  kb_to_f32<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(b->S, X, n);
  int rc = launch_matvec(b, obs, X, b->W, false, st);
  if (rc) return rc;
  const dim3 eg(KB_RED_CHUNKS, b->nb / 32), eb(32, 8);
  kb_expect_dots<<<eg, eb, 0, st>>>(b->S, b->W, b->dim, b->nb, b->part);
  kb_reduce<<<(b->nb + 255) / 256, 256, 0, st>>>(b->part, 1, b->nb, 1, b->h);
  b->launches += 3;
  KR_CUDA(obs->ctx, cudaGetLastError());
  std::vector<double2> h(b->nb);
  int mverr = 0;
  KR_CUDA(obs->ctx, cudaMemcpyAsync(h.data(), b->h, sizeof(double2) * b->nb, cudaMemcpyDeviceToHost, st));
  KR_CUDA(obs->ctx, cudaMemcpyAsync(&mverr, b->counts + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  KR_CUDA(obs->ctx, cudaStreamSynchronize(st));
  if (mverr) return set_err(obs->ctx, mverr, mv_error_text);
  for (int v = 0; v < b->nvec; ++v) {
    out[2 * v] = h[v].x;
    out[2 * v + 1] = h[v].y;
  }
  return KR_OK;
}

// (nvec, dim) complex128 <-> [dim][nb] complex64
__global__ void kb_transpose_in32(const double2* src, float2* X, long long dim, int nvec, int nb) {
  __shared__ float2 tile[32][33];
  const long long e0 = blockIdx.x * 32LL;
  const int v0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int v = v0 + r;
    const long long e = e0 + threadIdx.x;
    const double2 x = (v < nvec && e < dim) ? src[(long long)v * dim + e] : make_double2(0.0, 0.0);
    tile[r][threadIdx.x] = make_float2((float)x.x, (float)x.y);
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const long long e = e0 + r;
    if (e < dim) X[e * nb + v0 + threadIdx.x] = tile[threadIdx.x][r];
  }
}
__global__ void kb_transpose_out32(const float2* Y, double2* dst, long long dim, int nvec, int nb) {
  __shared__ float2 tile[32][33];
  const long long e0 = blockIdx.x * 32LL;
  const int v0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const long long e = e0 + r;
    tile[r][threadIdx.x] = (e < dim) ? Y[e * nb + v0 + threadIdx.x] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int v = v0 + r;
    const long long e = e0 + threadIdx.x;
    if (v < nvec && e < dim) {
      const float2 y = tile[threadIdx.x][r];
      dst[(long long)v * dim + e] = make_double2(y.x, y.y);
    }
  }
}

extern "C" int kr_batch_apply(kr_batch* b, kr_op* op, const void* x, void* y, void* stream) {
  if (!b || !op || !x || !y || !op->square || op->dev.dim_out != b->dim)
    return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_apply: bad argument or basis mismatch");
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid((unsigned)((b->dim + 31) / 32), b->nb / 32);
  KR_CUDA(op->ctx, cudaMemsetAsync(b->counts + 2, 0, sizeof(int), st));
  kb_transpose_in32<<<grid, dim3(32, 8), 0, st>>>((const double2*)x, b->V, b->dim, b->nvec, b->nb);
  const int rc = launch_matvec(b, op, b->V, b->W, false, st);
  if (rc) return rc;
  kb_transpose_out32<<<grid, dim3(32, 8), 0, st>>>(b->W, (double2*)y, b->dim, b->nvec, b->nb);
  b->launches += 2;
  KR_CUDA(op->ctx, cudaGetLastError());
  int mverr = 0;
  KR_CUDA(op->ctx, cudaMemcpyAsync(&mverr, b->counts + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  KR_CUDA(op->ctx, cudaStreamSynchronize(st));
  if (mverr) return set_err(op->ctx, mverr, mv_error_text);
  return KR_OK;
}

extern "C" int kr_batch_populations(kr_batch* b, double* out, void* stream) {
  if (!b || !out) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_populations: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  kb_slab_pop<<<dim3(b->nslab, b->nb / 32), dim3(32, 8), 0, st>>>(b->S, b->slab_off, b->slab_len, b->nb, b->pop);
  b->launches++;
  KR_CUDA(b->op->ctx, cudaGetLastError());
  std::vector<double> h((size_t)b->nslab * b->nb);
  KR_CUDA(b->op->ctx, cudaMemcpyAsync(h.data(), b->pop, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  KR_CUDA(b->op->ctx, cudaStreamSynchronize(st));
  for (int s = 0; s < b->nslab; ++s)
    for (int v = 0; v < b->nvec; ++v) out[(size_t)s * b->nvec + v] = h[(size_t)s * b->nb + v];
  return KR_OK;
}

extern "C" int kr_batch_set_matvec(kr_batch* b, int32_t kind) {
  if (!b || (kind != KR_MATVEC_TENSOR && kind != KR_MATVEC_FP32))
    return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_set_matvec: bad argument");
  b->mv_kind = kind;
  return KR_OK;
}

extern "C" int kr_batch_matvec(kr_batch* b, kr_op* op, void* stream) {
  if (!b || !op || op->dev.dim_out != b->dim || !op->square)
    return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_matvec: operator does not match the batch basis");
  return launch_matvec(b, op, b->V, b->W, false, (cudaStream_t)stream);
}

extern "C" int64_t kr_batch_launch_count(const kr_batch* b) { return b ? b->launches : -1; }

// ---------------------------------------------------------------------------
// tensor-core probe: D (128 x 16) = A (128 x 16) B^T (B: 16 x 16), A, B, D
// row-major FP32 (read as TF32), one CTA: the MMA building block of the
// batched mat-vec (operand staging, descriptors, TMEM, commit, TMEM load)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) kb_mma_probe(const float* A, const float* B, float* D, int* err) {
  __shared__ __align__(128) float sa[128 * 16];
  __shared__ __align__(128) float sb[16 * 16];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  for (int e = tid; e < 128 * 16; e += 128) sa[tc_kmajor_off(e >> 4, e & 15, 16) >> 2] = A[e];
  for (int e = tid; e < 16 * 16; e += 128) sb[tc_kmajor_off(e >> 4, e & 15, 16) >> 2] = B[e];
  if (wid == 0) tc_alloc(&tbase, 32);
  if (tid == 0) tc_mbar_init(&bar, 1);
  tc_fence_proxy();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = tbase;
  if (tid == 0) {
    const uint32_t idesc = tc_idesc_tf32(128, 16);
    for (int s = 0; s < 2; ++s)  // K = 16 in two steps of 8
      tc_mma_tf32(taddr, tc_desc(tc_smem_u32(sa) + 256u * s, 128u, 512u),
                  tc_desc(tc_smem_u32(sb) + 256u * s, 128u, 512u), idesc, (uint32_t)s);
    tc_commit(&bar);
  }
  if (!tc_mbar_wait(&bar, 0) && lane == 0) atomicExch(err, KR_ERR_TIMEOUT);
  tc_fence_after();
  float v[16];
  tc_ld16(taddr + ((uint32_t)(32 * wid) << 16), v);
#pragma unroll
  for (int j = 0; j < 16; ++j) D[(32 * wid + lane) * 16 + j] = v[j];
  tc_fence_before();
  __syncthreads();
  if (wid == 0) tc_dealloc(taddr, 32);
}

extern "C" int kr_probe_mma(kr_ctx* ctx, const float* a, const float* b, float* d) {
  if (!ctx || !a || !b || !d) return set_err(ctx, KR_ERR_ARG, "kr_probe_mma: NULL argument");
  KR_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t na = 128 * 16, nbb = 16 * 16, nd = 128 * 16;
  char* buf = nullptr;
  KR_CUDA(ctx, cudaMalloc(&buf, sizeof(float) * (na + nbb + nd) + 16));
  float* dA = reinterpret_cast<float*>(buf);
  float* dB = dA + na;
  float* dD = dB + nbb;
  int* derr = reinterpret_cast<int*>(dD + nd);
  int herr = 0;
  cudaError_t e = cudaMemcpy(dA, a, sizeof(float) * na, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, b, sizeof(float) * nbb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  if (e == cudaSuccess) {
    kb_mma_probe<<<1, 128>>>(dA, dB, dD, derr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(d, dD, sizeof(float) * nd, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return set_err(ctx, KR_ERR_CUDA, std::string("kr_probe_mma: ") + cudaGetErrorString(e));
  if (herr) return set_err(ctx, herr, "kr_probe_mma: the MMA completion wait gave up");
  return KR_OK;
}
