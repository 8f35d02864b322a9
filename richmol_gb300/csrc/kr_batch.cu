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
//   * state in double-float (an FP32 pair, about 2^-48 relative), H0 half-phases
//     converted from FP64 to double-float once per step.
// The two mat-vec kinds live in kr_batch_simt.cu and kr_batch_tc.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "kr_batch_mv.cuh"

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
  double* vscale = nullptr;  // [mmax + 1][nb] scale of each stored basis vector (V_j = vscale_j x stored)
  int* kconv = nullptr;      // [nb] converged Krylov order (0: still active)
  int* active = nullptr;     // [nb]
  int* grp_active = nullptr; // [nb / KB_MV_THREADS rounded up]
  int* grp_w = nullptr;      // [the same]: groups with a vector of non-zero weight (kr_batch_expect_dev)
  double* err = nullptr;     // [nb]
  double2* part = nullptr;   // [KB_RED_CHUNKS][mmax + 2][nb] partial sums
  // The next step's V_0 = P S and its ||.||^2 partials, written by the state
  // combination (kb_combine) so that the step's prologue need not read S:
  // v0_ready holds the token of the phase they were made with (0: none).
  double2* part0 = nullptr;  // [KB_RED_CHUNKS][nb]
  int* v0_ready = nullptr;   // [1]
  int* counts = nullptr;     // [3]: active vectors, vectors that hit mmax, mat-vec error word
  int* tc_work = nullptr;    // [3] work-item counters of the persistent tensor-core launches
  int* kdev = nullptr;       // [2]: Krylov index of the running iteration, orders used by the last step
  int* status = nullptr;     // [1] sticky error of a step (0: none), read by kr_batch_sync / kr_batch_step
  // the step as a CUDA graph (prologue, a WHILE node over the Krylov
  // iterations, the state combination), instantiated once per step key
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t cap = nullptr, side0 = nullptr, side1 = nullptr;
  const kr_op* g_op = nullptr;
  unsigned long long g_uid = 0;
  const void* g_phase = nullptr;
  double g_fac[2] = {0, 0}, g_tol = 0;
  int g_kind = -1;
  int nodes_fixed = 0, nodes_iter = 0;  // kernel launches of a step outside / per Krylov iteration
  // mat-vec tile table
  int ntask = 0;
  // per-slab populations (slabs of the operator the batch was created with)
  int nslab = 0;
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
  const int* kdev;  // device Krylov index (null: the k argument of the kernel)
  int* status;
  double2* part0;       // partials of the next step's ||V_0||^2
  const int* v0_ready;  // token of the phase of a V_0 made by the last combination
  int v0_token;         // token of this step's phase
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
  d.kdev = b->kdev;
  d.status = b->status;
  d.part0 = b->part0;
  d.v0_ready = b->v0_ready;
  d.v0_token = 0;
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

// S <- phase * S (optional); V_0 = S in complex64 (unnormalised); partial ||S_v||^2.
// Nothing to do when the last state combination already wrote V_0 = phase * S
// and its partials with this phase (*v0_ready == token): S then holds the
// state without the step's first half-phase, which kb_combine applies.
__global__ void kb_phase_norm(float4* S, const float4* phase, float2* V0, long long dim, int nb, double2* part,
                              const int* status, const int* v0_ready, int token) {
  __shared__ double2 sh[8][32];
  if (status && *((volatile const int*)status) != 0) return;  // an error is pending: the step does nothing
  if (*((volatile const int*)v0_ready) == token) return;
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  dfl acc = {0.f, 0.f};
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    dfc s = dfc_ld(S[e * nb + v]);
    if (phase) {
      s = dfc_mul(s, dfc_ld(__ldg(phase + e)));
      S[e * nb + v] = dfc_st(s);
    }
    // the first basis vector, stored unnormalised (its scale 1 / ||S|| is set by kb_start)
    V0[e * nb + v] = make_float2(__fadd_rn(s.re.hi, s.re.lo), __fadd_rn(s.im.hi, s.im.lo));
    acc = df_add(acc, df_add(df_mul(s.re, s.re), df_mul(s.im, s.im)));
  }
  const double2 t = warps_sum(make_double2(df_to(acc), 0.0), sh);
  if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = t;
}

// out[j][v] = sum over chunks of part[chunk][j][v] (fixed order); with kdev
// the coefficients are j = 0 .. *kdev (the dots of the running iteration)
__global__ void kb_reduce(const double2* part, int ncoef, int nb, int stride_coef, double2* out, const int* kdev) {
  if (kdev) ncoef = *kdev + 1;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ncoef * nb) return;
  const int j = idx / nb, v = idx - j * nb;
  double2 s = make_double2(0.0, 0.0);
  for (int c = 0; c < KB_RED_CHUNKS; ++c) s = cadd(s, part[((long long)c * stride_coef + j) * nb + v]);
  out[(long long)j * nb + v] = s;
}

// per vector: ||S||, active flag, the scale of V_0 (phase * S stored by
// kb_phase_norm); counts[0] = active vectors. With an error pending no vector
// is active, so the step leaves the state as it is.
__global__ void kb_start(const double2* nsq, double* norm0, int* active, int* kconv, double* vscale, int nb,
                         int nvec, int* counts, const int* status) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nb) return;
  const bool ok = status == nullptr || *((volatile const int*)status) == 0;
  const double n0 = ok ? sqrt(nsq[v].x) : 0.0;
  norm0[v] = n0;
  const int act = (ok && v < nvec && n0 > 0.0) ? 1 : 0;
  active[v] = act;
  kconv[v] = 0;
  vscale[v] = n0 > 0.0 ? 1.0 / n0 : 0.0;
  if (act && counts) atomicAdd(counts, 1);
}

// partial dots h_j = <V_j, W> for j = 0..k (V_j as stored, times its scale):
// FP32 products, FP32 sums inside a thread's elements, FP64 across threads and
// chunks; per chunk and vector, part[chunk][j][nb]. One pass per j: the chunk
// of W a CTA reads stays in cache from pass to pass, so DRAM sees W once (one
// pass over all V_j with W read once measured 45 % slower at C3). The loads of
// four elements go out before their FMAs (summed in element order, so the
// result is the one-at-a-time sum), at 6 CTAs per SM: 14 % faster at C3.
__global__ void __launch_bounds__(256, 6) kb_dots(const float2* V, const float2* W, const int* active,
                                                  const double* vscale, long long dim, int nb, int k,
                                                  int stride_coef, double2* part, const int* kdev) {
  constexpr int U = 4;
  __shared__ double2 sh[8][32];
  if (kdev) k = *kdev;
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  const bool act = active[v] != 0;
  for (int j = 0; j <= k; ++j) {
    float2 acc = make_float2(0.f, 0.f);
    if (act) {
      const float2* Vj = V + (long long)j * dim * nb;
      long long e = ch.e0 + threadIdx.y;
      for (; e + 8 * (U - 1) < ch.e1; e += 8 * U) {
        float2 a[U], b[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          a[u] = Vj[(e + 8 * u) * nb + v];
          b[u] = W[(e + 8 * u) * nb + v];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          acc.x = fmaf(a[u].x, b[u].x, acc.x);
          acc.x = fmaf(a[u].y, b[u].y, acc.x);
          acc.y = fmaf(a[u].x, b[u].y, acc.y);
          acc.y = fmaf(-a[u].y, b[u].x, acc.y);
        }
      }
      for (; e < ch.e1; e += 8) {
        const float2 a = Vj[e * nb + v], b = W[e * nb + v];
        acc.x = fmaf(a.x, b.x, acc.x);
        acc.x = fmaf(a.y, b.y, acc.x);
        acc.y = fmaf(a.x, b.y, acc.y);
        acc.y = fmaf(-a.y, b.x, acc.y);
      }
    }
    const double2 t = warps_sum(make_double2(acc.x, acc.y), sh);
    if (threadIdx.y == 0) part[((long long)blockIdx.x * stride_coef + j) * nb + v] = cscale(t, vscale[(long long)j * nb + v]);
  }
}

// V_{k+1} = W - sum_j h_j V_j (unnormalised), partial ||V_{k+1}||^2; k < KM.
// KM = 4 with the register budget of 5 CTAs per SM: 48 registers (40 without
// the bound), which lets the loads of W and every basis vector go out ahead of
// their FMAs; 15 % faster at C3.
template <int KM>
__global__ void __launch_bounds__(256, KM == 4 ? 5 : 1) kb_update(float2* V, const float2* W, const double2* h, const double* vscale, const int* active,
                          long long dim, int nb, int k, double2* part, const int* kdev) {
  __shared__ double2 sh[8][32];
  if (kdev) k = *kdev;
  const int v = blockIdx.y * 32 + threadIdx.x;
  const Chunk ch = chunk_of(dim);
  const bool act = active[v] != 0;
  dfl nacc = {0.f, 0.f};
  if (act) {
    float2 hv[KM];
#pragma unroll
    for (int j = 0; j < KM; ++j) {
      const double2 t = j <= k ? cscale(h[(long long)j * nb + v], vscale[(long long)j * nb + v]) : make_double2(0.0, 0.0);
      hv[j] = make_float2((float)t.x, (float)t.y);
    }
    float2* Vn = V + (long long)(k + 1) * dim * nb;
    for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
      float2 r = W[e * nb + v];
#pragma unroll
      for (int j = 0; j < KM; ++j) {
        if (j <= k) {
          const float2 a = V[((long long)j * dim + e) * nb + v];
          r.x = fmaf(-hv[j].x, a.x, r.x);
          r.x = fmaf(hv[j].y, a.y, r.x);
          r.y = fmaf(-hv[j].x, a.y, r.y);
          r.y = fmaf(-hv[j].y, a.x, r.y);
        }
      }
      Vn[e * nb + v] = r;
      nacc = df_add(nacc, df_add(df_mulf({r.x, 0.f}, r.x), df_mulf({r.y, 0.f}, r.y)));
    }
  }
  const double2 t = warps_sum(make_double2(df_to(nacc), 0.0), sh);
  if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = t;
}

// per vector: T update, exp(fac T) e0, error estimate, convergence
__global__ void kb_small(BatchDev b, int k, double2 fac, double tol, const double2* npart) {
  if (b.kdev) k = *b.kdev;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= b.nb || !b.active[v]) return;
  const int nb = b.nb;
  const double2 hk = b.h[(long long)k * nb + v];
  double2 nsq = make_double2(0.0, 0.0);  // ||V_{k+1}||^2 from the chunk partials, in chunk order
  for (int c = 0; c < KB_RED_CHUNKS; ++c) nsq = cadd(nsq, npart[(long long)c * nb + v]);
  const double bk = sqrt(nsq.x);
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
    b.vscale[(long long)(k + 1) * nb + v] = 1.0 / bk;  // V_{k+1} stays stored unnormalised
    atomicAdd(b.counts, 1);
  }
}

// S <- P (c_0 P0 S + ||S|| sum_{1 <= i < K} c_i V_i), K < KM + 1 per vector
// (double-float state; the complex64 Krylov corrections summed in FP32), where
// P0 = P when the step's prologue left S without its first half-phase
// (*v0_ready == v0_token), else 1. Then the next step's prologue in the same
// pass: V_0 = P S in complex64 (unnormalised) and the partials of ||P S||^2,
// the values kb_phase_norm would compute from the stored S, element for
// element and in its order. A vector without a Krylov step (K == 0: zero,
// padding, or an error pending) keeps its S. KM = 4 (the class of Krylov
// orders up to 4) has the register budget of 5 CTAs per SM (48 registers, 8
// bytes of spills; 56 and 4 CTAs without it): 0.05 ms less per step at C3.
template <int KM>
__global__ void __launch_bounds__(256, KM == 4 ? 5 : 1) kb_combine(BatchDev b, const float4* phase) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const int nb = b.nb;
  const int K = b.kconv[v];
  const bool pre = phase && *b.v0_ready == b.v0_token;
  float2 cf[KM];
#pragma unroll
  for (int i = 1; i < KM; ++i)
    cf[i] = i < K ? make_float2((float)(b.c[(long long)i * nb + v].x * b.vscale[(long long)i * nb + v]),
                                (float)(b.c[(long long)i * nb + v].y * b.vscale[(long long)i * nb + v]))
                  : make_float2(0.f, 0.f);
  const dfc c0 = dfc_from(b.c[v]);
  const dfl n0 = df_from(b.norm0[v]);
  const Chunk ch = chunk_of(b.dim);
  dfl acc = {0.f, 0.f};
  for (long long e = ch.e0 + threadIdx.y; e < ch.e1; e += 8) {
    dfc u = dfc_ld(b.S[e * nb + v]);
    const dfc p = phase ? dfc_ld(__ldg(phase + e)) : dfc_ld(make_float4(1.f, 0.f, 0.f, 0.f));
    if (K > 0) {
      float2 sacc = make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 1; i < KM; ++i) {
        if (i < K) {
          const float2 a = b.V[((long long)i * b.dim + e) * nb + v];
          sacc.x = fmaf(cf[i].x, a.x, sacc.x);
          sacc.x = fmaf(-cf[i].y, a.y, sacc.x);
          sacc.y = fmaf(cf[i].x, a.y, sacc.y);
          sacc.y = fmaf(cf[i].y, a.x, sacc.y);
        }
      }
      if (pre) u = dfc_mul(u, p);
      u = dfc_mul(c0, u);
      u.re = df_add(u.re, df_mulf(n0, sacc.x));
      u.im = df_add(u.im, df_mulf(n0, sacc.y));
      if (phase) u = dfc_mul(u, p);
      b.S[e * nb + v] = dfc_st(u);
    }
    if (phase) u = dfc_mul(u, p);
    b.V[e * nb + v] = make_float2(__fadd_rn(u.re.hi, u.re.lo), __fadd_rn(u.im.hi, u.im.lo));
    acc = df_add(acc, df_add(df_mul(u.re, u.re), df_mul(u.im, u.im)));
  }
  const double2 t = warps_sum(make_double2(df_to(acc), 0.0), sh);
  if (threadIdx.y == 0) b.part0[(long long)blockIdx.x * nb + v] = t;
}

// the V_0 of the next step, written by kb_combine, belongs to the phase of token
__global__ void kb_v0_mark(int* v0_ready, int token) { *v0_ready = token; }

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

// 32-vector groups that hold a vector of non-zero weight (w null: every
// vector below nvec): grp[g] = 1, else 0
__global__ void kb_weight_groups(const double* w, int nvec, int nb, int* grp) {
  const int g = blockIdx.x * blockDim.y + threadIdx.y;
  if (g * 32 >= nb) return;
  const int v = g * 32 + threadIdx.x;
  const bool on = v < nvec && (w == nullptr || w[v] != 0.0);
  const unsigned any = __ballot_sync(0xffffffffu, on);
  if (threadIdx.x == 0) grp[g] = any != 0u;
}

// kb_to_f32 over the vectors of active 32-vector groups only (grid.y: group)
__global__ void kb_to_f32_groups(const float4* S, float2* X, long long dim, int nb, const int* grp) {
  if (!grp[blockIdx.y]) return;
  const int v = blockIdx.y * 32 + threadIdx.x;
  for (long long e = blockIdx.x * (long long)blockDim.y + threadIdx.y; e < dim; e += (long long)gridDim.x * blockDim.y) {
    const float4 s = S[e * nb + v];
    X[e * nb + v] = make_float2(__fadd_rn(s.x, s.y), __fadd_rn(s.z, s.w));
  }
}

// partial <S_v | Y_v> with Y in complex64 (double-float accumulation); with
// grp, the vectors of inactive groups get zero partials without reading S or Y
__global__ void kb_expect_dots(const float4* S, const float2* Y, long long dim, int nb, double2* part,
                               const int* grp = nullptr) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  if (grp && !grp[blockIdx.y]) {
    if (threadIdx.y == 0) part[(long long)blockIdx.x * nb + v] = make_double2(0.0, 0.0);
    return;
  }
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
// (double-float accumulation, fixed order); out[slab][nb]. Element q of a slab
// (row q / dk, column q % dk) sits at off + row * stride + column.
__global__ void kb_slab_pop(const float4* S, const long long* slab_off, const int* slab_dm, const int* slab_dk,
                            const int* slab_stride, int nb, double* out) {
  __shared__ double2 sh[8][32];
  const int v = blockIdx.y * 32 + threadIdx.x;
  const long long off = slab_off[blockIdx.x];
  const int dk = slab_dk[blockIdx.x], ld = slab_stride[blockIdx.x];
  const long long n = (long long)slab_dm[blockIdx.x] * dk;
  dfl acc = {0.f, 0.f};
  for (long long q = threadIdx.y; q < n; q += 8) {
    const long long e = off + (q / dk) * ld + q % dk;
    const dfc s = dfc_ld(S[e * nb + v]);
    acc = df_add(acc, df_add(df_mul(s.re, s.re), df_mul(s.im, s.im)));
  }
  const double2 t = warps_sum(make_double2(df_to(acc), 0.0), sh);
  if (threadIdx.y == 0) out[(long long)blockIdx.x * nb + v] = t.x;
}


// any active vector per 32-vector group; in a recorded step, thread 0 also
// selects the Gram-Schmidt kernel of the running iteration (its Krylov-index
// bound 4, 8, 16, 32) for the switch node that follows
__device__ __forceinline__ unsigned kb_bound_class(int k) { return k < 4 ? 0u : k < 8 ? 1u : k < 16 ? 2u : 3u; }
__global__ void kb_group_active(const int* active, int* grp, int ngrp, const int* kdev,
                                cudaGraphConditionalHandle hupd) {
  if (kdev && blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    cudaGraphSetConditional(hupd, kb_bound_class(*kdev));
  const int g = blockIdx.x * blockDim.y + threadIdx.y;
  if (g >= ngrp) return;
  const int any = __any_sync(0xffffffffu, active[g * 32 + threadIdx.x] != 0);
  if (threadIdx.x == 0) grp[g] = any;
}

// ---------------------------------------------------------------------------
// loop control of a recorded step (one thread each)
// ---------------------------------------------------------------------------
// after the prologue: iteration 0 runs if any vector is active and no error is pending
__global__ void kb_ctl_init(int* counts, int* kdev, const int* status, cudaGraphConditionalHandle hloop) {
  const int go = counts[0] > 0 && *((volatile const int*)status) == 0;
  kdev[0] = 0;
  kdev[1] = 0;
  counts[0] = 0;
  counts[1] = 0;
  cudaGraphSetConditional(hloop, go ? 1u : 0u);
}
// after iteration k: errors into the sticky status (mat-vec error word, then
// vectors that reached mmax), k + 1, and whether iteration k + 1 runs
__global__ void kb_ctl(int* counts, int* kdev, int* status, int mmax, cudaGraphConditionalHandle hloop) {
  const int k = kdev[0];
  int e = 0;
  if (counts[2] != 0) e = counts[2];
  else if (counts[1] != 0) e = KR_ERR_MAXORDER;
  if (e != 0 && *status == 0) *status = e;
  const int more = counts[0] > 0 && e == 0 && k + 1 < mmax;
  kdev[0] = k + 1;
  kdev[1] = k + 1;
  counts[0] = 0;
  counts[1] = 0;
  counts[2] = 0;
  cudaGraphSetConditional(hloop, more ? 1u : 0u);
}
// after the loop: the state combination kernel for the orders used (bound class)
__global__ void kb_combine_select(const int* kdev, cudaGraphConditionalHandle hcomb) {
  cudaGraphSetConditional(hcomb, kb_bound_class(kdev[1]));
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

// Y = H X, each vector's output times yscale[v] when yscale is given (the
// scale of a basis vector stored unnormalised). X (and yscale) is the basis
// array b->V (b->vscale); with kslot its slot is the device-side Krylov index
// *kslot, else slot 0.
int launch_matvec(kr_batch* b, kr_op* op, const float2* X, float2* Y, bool masked, const double* yscale,
                  const int* kslot, cudaStream_t st, const int* grp = nullptr) {
  const long long slot_elems = b->dim * (long long)b->nb;
  if ((b->mv_kind == KR_MATVEC_TENSOR || b->mv_kind == KR_MATVEC_TENSOR_TMEM) && op->tc_ntask > 0) {
    BatchTC q;
    q.op = op->dev;
    q.X = X;
    q.Y = Y;
    q.nb = b->nb;
    q.kslot = kslot;
    q.slot_elems = slot_elems;
    q.nslots = kslot ? b->mmax + 1 : 1;
    q.task = op->tc_task;
    q.ntask = op->tc_ntask;
    q.grp_active = grp ? grp : (masked ? b->grp_active : nullptr);
    q.yscale = yscale;
    q.tcb = op->tc_b;
    q.tcb_off = op->tc_boff;
    q.err = b->counts + 2;
    q.tfirst = 0;
    q.tend = op->tc_ntask;
    q.nvb = b->nb / 128;
    q.work = b->tc_work;
    const int rc = kb_launch_tc(op->ctx, q, b->dim, op->tc_class, b->tc_work, b->mv_kind == KR_MATVEC_TENSOR_TMEM, st);
    if (rc == KR_OK)
      b->launches += (op->tc_class[1] > op->tc_class[0]) + (op->tc_class[2] > op->tc_class[1]) +
                     (op->tc_class[3] > op->tc_class[2]);
    return rc;
  }
  BatchMV p;
  p.op = op->dev;
  p.X = X;
  p.Y = Y;
  p.nb = b->nb;
  p.kslot = kslot;
  p.slot_elems = slot_elems;
  p.err = b->counts + 2;
  p.task_slab = b->task_slab;
  p.task_i0 = b->task_i0;
  p.task_nr = b->task_nr;
  p.grp_active = grp ? grp : (masked ? b->grp_active : nullptr);
  p.yscale = yscale;
  if (b->mv_kind == KR_MATVEC_FP32_REG && op->zr_ntask > 0) {
    const int rc = kb_launch_zr(op->ctx, p, op->zr_task, op->zr_ntask, op->zr_class, mv_groups(b), st);
    if (rc == KR_OK)
      b->launches += (op->zr_class[1] > op->zr_class[0]) + (op->zr_class[2] > op->zr_class[1]) +
                     (op->zr_class[3] > op->zr_class[2]);
    return rc;
  }
  const int rc = kb_launch_simt(op->ctx, p, b->ntask, mv_groups(b), st);
  if (rc == KR_OK) b->launches++;
  return rc;
}
}  // namespace

extern "C" int kr_batch_create(kr_op* op, int64_t nvec, int32_t mmax, kr_batch** out) {
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  if (!op || !out || nvec <= 0 || mmax < 2 || mmax > KB_NK_MAX - 1)
    return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_batch_create: bad argument (2 <= mmax <= 31)");
  *out = nullptr;
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_batch_create: operator is not square");
  KR_DEVICE_SCOPE(op->ctx, op->ctx->device);
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
  BA(m1 * nb, &b->vscale);
  BA(nb, &b->kconv);
  BA(nb, &b->active);
  BA((size_t)mv_groups(b), &b->grp_active);
  BA((size_t)mv_groups(b), &b->grp_w);
  BA(nb, &b->err);
  BA((size_t)KB_RED_CHUNKS * (m1 + 1) * nb, &b->part);
  BA((size_t)KB_RED_CHUNKS * nb, &b->part0);
  BA(1, &b->v0_ready);
  BA(3, &b->counts);
  BA(3, &b->tc_work);
  BA(2, &b->kdev);
  BA(1, &b->status);
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
  BA((size_t)b->nslab * nb, &b->pop);
  BA(ts.size(), &b->task_slab);
  BA(ti.size(), &b->task_i0);
  BA(tn.size(), &b->task_nr);
#undef BA
  cudaError_t ce = cudaMemcpy(b->task_slab, ts.data(), sizeof(int) * ts.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->task_i0, ti.data(), sizeof(int) * ti.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(b->task_nr, tn.data(), sizeof(int) * tn.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->side0, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->side1, cudaStreamNonBlocking);
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
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  for (cudaStream_t s : {b->cap, b->side0, b->side1})
    if (s) cudaStreamDestroy(s);
  for (void* p : b->allocs) cudaFree(p);
  delete b;
}

extern "C" int kr_batch_load(kr_batch* b, const void* states, void* stream) {
  if (!b || !states) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_load: bad argument");
  dim3 grid((unsigned)((b->dim + 31) / 32), b->nb / 32);
  kb_transpose_in<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const double2*)states, b->S, b->dim, b->nvec, b->nb);
  b->launches++;
  KR_CUDA(b->op->ctx, cudaGetLastError());
  // a V_0 kept from the last step belongs to the old states
  KR_CUDA(b->op->ctx, cudaMemsetAsync(b->v0_ready, 0, sizeof(int), (cudaStream_t)stream));
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

namespace {
// adds a conditional node (WHILE or SWITCH) at the current end of stream s's
// capture and makes it the new end; its body graphs are returned in body
int add_conditional(kr_ctx* ctx, cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    unsigned size, cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  KR_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  if (cs != cudaStreamCaptureStatusActive) return set_err(ctx, KR_ERR_CUDA, "batched step: stream is not capturing");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = size;
  cudaGraphNode_t node;
  KR_CUDA(ctx, cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np));
  for (unsigned i = 0; i < size; ++i) body[i] = np.conditional.phGraph_out[i];
  KR_CUDA(ctx, cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return KR_OK;
}

// records one Gram-Schmidt kernel or state combination per Krylov-index bound
// class (4, 8, 16, 32) into the four bodies of a switch node, on stream s
template <typename F>
int record_switch(kr_ctx* ctx, cudaStream_t s, cudaGraph_t* bodies, F launch) {
  for (int c = 0; c < 4; ++c) {
    KR_CUDA(ctx, cudaStreamBeginCaptureToGraph(s, bodies[c], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    launch(c, s);
    cudaGraph_t done = nullptr;
    const cudaError_t e1 = cudaGetLastError();
    KR_CUDA(ctx, cudaStreamEndCapture(s, &done));
    KR_CUDA(ctx, e1);
  }
  return KR_OK;
}

// token of a phase array for v0_ready: its address (0 is never a token)
int v0_token(const double2* phase) {
  if (!phase) return 1;
  return (int)((((uintptr_t)phase) >> 4) & 0x3fffffffu) | 0x40000000;
}

// Records one batched step into the graph that stream s is capturing into:
//   prologue   counts = 0; H0 half-phase to double-float; S <- P S, V_0, ||S||^2
//              (skipped when the last step's combination left V_0 = P S and
//              its partials for this phase); per-vector start; loop control
//              (iteration 0 runs?)
//   WHILE      mask of active vector groups (+ Gram-Schmidt kernel class);
//              W = H V_k (mat-vec of the device-side slot k); dots <V_j, W>;
//              their sums; SWITCH: V_{k+1} = W - sum h_j V_j (bound class of k);
//              per-vector T, exp(fac T) e0, error estimate, convergence;
//              loop control (k + 1, errors, iteration k + 1 runs?)
//   SWITCH     state combination S <- P (c_0 S + ||S|| sum c_i V_i) (class of the orders used),
//              with the next step's V_0 = P S and ||V_0||^2 partials; then v0_ready = token
// The Krylov index lives in device memory (b->kdev), so nothing of the loop
// depends on the host: a recorded step replays as it is.
int record_step(kr_batch* b, kr_op* op, const double2* phase, double2 fac, double tol, cudaStream_t s) {
  kr_ctx* ctx = op->ctx;
  const int nb = b->nb;
  const long long dim = b->dim;
  const dim3 eg(KB_RED_CHUNKS, nb / 32), eb(32, 8);
  const int stride = b->mmax + 2;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  KR_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive) return set_err(ctx, KR_ERR_CUDA, "batched step: stream is not capturing");
  cudaGraphConditionalHandle hloop, hupd, hcomb;
  KR_CUDA(ctx, cudaGraphConditionalHandleCreate(&hloop, g, 0, cudaGraphCondAssignDefault));
  KR_CUDA(ctx, cudaGraphConditionalHandleCreate(&hupd, g, 0, 0));
  KR_CUDA(ctx, cudaGraphConditionalHandleCreate(&hcomb, g, 0, 0));
  int fixed = 0, iter = 0;
  // ---- prologue
  KR_CUDA(ctx, cudaMemsetAsync(b->counts, 0, 3 * sizeof(int), s));
  const float4* pdf = nullptr;
  if (phase) {
    kb_phase_df<<<(int)std::min<long long>((dim + 255) / 256, 1024), 256, 0, s>>>(phase, b->phase_df, dim);
    pdf = b->phase_df;
    ++fixed;
  }
  const int token = v0_token(phase);
  kb_phase_norm<<<eg, eb, 0, s>>>(b->S, pdf, b->V, dim, nb, b->part0, b->status, b->v0_ready, token);
  kb_reduce<<<(nb + 255) / 256, 256, 0, s>>>(b->part0, 1, nb, 1, b->h, nullptr);
  kb_start<<<(nb + 255) / 256, 256, 0, s>>>(b->h, b->norm0, b->active, b->kconv, b->vscale, nb, b->nvec, b->counts,
                                            b->status);
  kb_ctl_init<<<1, 1, 0, s>>>(b->counts, b->kdev, b->status, hloop);
  fixed += 4;
  KR_CUDA(ctx, cudaGetLastError());
  // ---- the Krylov iterations
  cudaGraph_t body;
  int rc = add_conditional(ctx, s, hloop, cudaGraphCondTypeWhile, 1, &body);
  if (rc) return rc;
  cudaStream_t s0 = b->side0;
  KR_CUDA(ctx, cudaStreamBeginCaptureToGraph(s0, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  {
    kb_group_active<<<(mv_groups(b) + 7) / 8, dim3(32, 8), 0, s0>>>(b->active, b->grp_active, mv_groups(b), b->kdev,
                                                                     hupd);
    const long long l0 = b->launches;
    rc = launch_matvec(b, op, b->V, b->W, true, b->vscale, b->kdev, s0);
    const int mv_launches = (int)(b->launches - l0);
    b->launches = l0;
    kb_dots<<<eg, eb, 0, s0>>>(b->V, b->W, b->active, b->vscale, dim, nb, 0, stride, b->part, b->kdev);
    kb_reduce<<<((b->mmax + 1) * nb + 255) / 256, 256, 0, s0>>>(b->part, 1, nb, stride, b->h, b->kdev);
    iter += 3 + mv_launches;
    cudaGraph_t ub[4];
    if (rc == KR_OK) rc = add_conditional(ctx, s0, hupd, cudaGraphCondTypeSwitch, 4, ub);
    if (rc == KR_OK)
      rc = record_switch(ctx, b->side1, ub, [&](int c, cudaStream_t t) {
        if (c == 0) kb_update<4><<<eg, eb, 0, t>>>(b->V, b->W, b->h, b->vscale, b->active, dim, nb, 0, b->part, b->kdev);
        else if (c == 1) kb_update<8><<<eg, eb, 0, t>>>(b->V, b->W, b->h, b->vscale, b->active, dim, nb, 0, b->part, b->kdev);
        else if (c == 2) kb_update<16><<<eg, eb, 0, t>>>(b->V, b->W, b->h, b->vscale, b->active, dim, nb, 0, b->part, b->kdev);
        else kb_update<32><<<eg, eb, 0, t>>>(b->V, b->W, b->h, b->vscale, b->active, dim, nb, 0, b->part, b->kdev);
      });
    kb_small<<<(nb + 127) / 128, 128, 0, s0>>>(dev_view(b), 0, fac, tol, b->part);
    kb_ctl<<<1, 1, 0, s0>>>(b->counts, b->kdev, b->status, b->mmax, hloop);
    iter += 3;
  }
  const cudaError_t le = cudaGetLastError();
  cudaGraph_t done = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s0, &done);
  if (rc) return rc;
  KR_CUDA(ctx, le);
  KR_CUDA(ctx, ee);
  // ---- the state combination
  kb_combine_select<<<1, 1, 0, s>>>(b->kdev, hcomb);
  cudaGraph_t cb[4];
  rc = add_conditional(ctx, s, hcomb, cudaGraphCondTypeSwitch, 4, cb);
  if (rc) return rc;
  BatchDev bd = dev_view(b);
  bd.v0_token = token;
  rc = record_switch(ctx, b->side1, cb, [&](int c, cudaStream_t t) {
    if (c == 0) kb_combine<4><<<eg, eb, 0, t>>>(bd, pdf);
    else if (c == 1) kb_combine<8><<<eg, eb, 0, t>>>(bd, pdf);
    else if (c == 2) kb_combine<16><<<eg, eb, 0, t>>>(bd, pdf);
    else kb_combine<32><<<eg, eb, 0, t>>>(bd, pdf);
  });
  if (rc) return rc;
  kb_v0_mark<<<1, 1, 0, s>>>(b->v0_ready, token);
  fixed += 3;
  KR_CUDA(ctx, cudaGetLastError());
  b->nodes_fixed = fixed;
  b->nodes_iter = iter;
  return KR_OK;
}

// the sticky step status: 0, or the error of a step (cleared when read)
int take_status(kr_batch* b, cudaStream_t st, int* kused) {
  int h[3] = {0, 0, 0};
  KR_CUDA(b->op->ctx, cudaMemcpyAsync(h, b->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  KR_CUDA(b->op->ctx, cudaMemcpyAsync(h + 1, b->kdev, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  KR_CUDA(b->op->ctx, cudaStreamSynchronize(st));
  if (kused) *kused = h[2];
  if (h[0] == 0) return KR_OK;
  KR_CUDA(b->op->ctx, cudaMemsetAsync(b->status, 0, sizeof(int), st));
  KR_CUDA(b->op->ctx, cudaStreamSynchronize(st));
  if (h[0] == KR_ERR_MAXORDER)
    return set_err(b->op->ctx, KR_ERR_MAXORDER,
                   "batched Lanczos: vectors did not reach the tolerance within " + std::to_string(b->mmax) +
                       " Krylov vectors");
  return set_err(b->op->ctx, h[0], mv_error_text);
}
}  // namespace

extern "C" int kr_batch_step(kr_batch* b, kr_op* op, const void* phase, double fac_re, double fac_im, double tol,
                             int32_t* kmax_out, void* stream) {
  if (!b || !op) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_step: bad argument");
  if (op->dev.dim_out != b->dim || !op->square)
    return set_err(op->ctx, KR_ERR_ARG, "kr_batch_step: operator does not match the batch basis");
  cudaStream_t st = (cudaStream_t)stream;
  kr_ctx* ctx = op->ctx;
  const double2 fac = make_double2(fac_re, fac_im);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  KR_CUDA(ctx, cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusActive) {
    // the caller records: the step's nodes go into the caller's graph
    if (kmax_out) return set_err(ctx, KR_ERR_ARG, "kr_batch_step: kmax_out must be NULL while the stream captures");
    std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
    return record_step(b, op, (const double2*)phase, fac, tol, st);
  }
  // a call: the step recorded once per (operator, phase, factor, tolerance,
  // mat-vec kind) and launched as one graph
  if (!b->gexec || b->g_op != op || b->g_uid != op->uid || b->g_phase != phase || b->g_fac[0] != fac_re ||
      b->g_fac[1] != fac_im || b->g_tol != tol || b->g_kind != b->mv_kind) {
    // recording and instantiation under the device mutex: no allocation, free or
    // device-wide synchronisation of the library's other threads runs meanwhile
    std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
    if (b->gexec) {
      KR_CUDA(ctx, cudaGraphExecDestroy(b->gexec));
      b->gexec = nullptr;
    }
    KR_CUDA(ctx, cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
    const int rc = record_step(b, op, (const double2*)phase, fac, tol, b->cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
    if (rc != KR_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    KR_CUDA(ctx, e);
    const cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    KR_CUDA(ctx, ie);
    b->g_op = op;
    b->g_uid = op->uid;
    b->g_phase = phase;
    b->g_fac[0] = fac_re;
    b->g_fac[1] = fac_im;
    b->g_tol = tol;
    b->g_kind = b->mv_kind;
  }
  KR_CUDA(ctx, cudaGraphLaunch(b->gexec, st));
  b->launches += b->nodes_fixed;
  if (!kmax_out) return KR_OK;
  int kused = 0;
  const int rc = take_status(b, st, &kused);
  b->launches += (long long)kused * b->nodes_iter;
  *kmax_out = kused;
  return rc;
}

extern "C" int kr_batch_sync(kr_batch* b, int32_t* kmax_out, void* stream) {
  if (!b) return set_err(nullptr, KR_ERR_ARG, "kr_batch_sync: NULL batch");
  int kused = 0;
  const int rc = take_status(b, (cudaStream_t)stream, &kused);
  if (kmax_out) *kmax_out = kused;
  return rc;
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
  float2* X = b->V + b->dim * b->nb;  // basis slot 1 and W are free between steps (slot 0 holds the next V_0)
  KR_CUDA(obs->ctx, cudaMemsetAsync(b->counts + 2, 0, sizeof(int), st));
  kb_to_f32<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(b->S, X, n);
  int rc = launch_matvec(b, obs, X, b->W, false, nullptr, nullptr, st);
  if (rc) return rc;
  const dim3 eg(KB_RED_CHUNKS, b->nb / 32), eb(32, 8);
  kb_expect_dots<<<eg, eb, 0, st>>>(b->S, b->W, b->dim, b->nb, b->part);
  kb_reduce<<<(b->nb + 255) / 256, 256, 0, st>>>(b->part, 1, b->nb, 1, b->h, nullptr);
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

// out = sum_v w_v Re <v|O|v> over the vectors (w: device weights, null = 1),
// summed in vector order by one warp; a mat-vec error of the observable goes
// into the sticky status (reported by kr_batch_sync)
__global__ void kb_expect_wsum(const double2* h, const double* w, int nvec, double* out, const int* mverr,
                               int* status) {
  const int lane = threadIdx.x;
  double s = 0.0;
  for (int v = lane; v < nvec; v += 32)
    if (w == nullptr || w[v] != 0.0) s += (w ? w[v] : 1.0) * h[v].x;  // zero-weight vectors are not computed
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    *out = s;
    if (*mverr != 0 && *status == 0) *status = *mverr;
  }
}

extern "C" int kr_batch_expect_dev(kr_batch* b, kr_op* obs, const double* weights, double* out, void* stream) {
  if (!b || !obs || !out) return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_expect_dev: bad argument");
  if (obs->dev.dim_out != b->dim || !obs->square)
    return set_err(obs->ctx, KR_ERR_ARG, "kr_batch_expect_dev: observable does not match the batch basis");
  cudaStream_t st = (cudaStream_t)stream;
  float2* X = b->V + b->dim * b->nb;  // basis slot 1 and W are free between steps (slot 0 holds the next V_0)
  KR_CUDA(obs->ctx, cudaMemsetAsync(b->counts + 2, 0, sizeof(int), st));
  // only the 32-vector groups with a vector of non-zero weight are computed
  const int ng = b->nb / 32;
  kb_weight_groups<<<(ng + 7) / 8, dim3(32, 8), 0, st>>>(weights, b->nvec, b->nb, b->grp_w);
  kb_to_f32_groups<<<dim3((unsigned)std::min<long long>((b->dim + 7) / 8, 1024), ng), dim3(32, 8), 0, st>>>(
      b->S, X, b->dim, b->nb, b->grp_w);
  int rc = launch_matvec(b, obs, X, b->W, false, nullptr, nullptr, st, b->grp_w);
  if (rc) return rc;
  const dim3 eg(KB_RED_CHUNKS, b->nb / 32), eb(32, 8);
  kb_expect_dots<<<eg, eb, 0, st>>>(b->S, b->W, b->dim, b->nb, b->part, b->grp_w);
  kb_reduce<<<(b->nb + 255) / 256, 256, 0, st>>>(b->part, 1, b->nb, 1, b->h, nullptr);
  kb_expect_wsum<<<1, 32, 0, st>>>(b->h, weights, b->nvec, out, b->counts + 2, b->status);
  b->launches += 6;
  KR_CUDA(obs->ctx, cudaGetLastError());
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
  float2* X = b->V + b->dim * b->nb;  // basis slot 1 (slot 0 holds the next step's V_0)
  kb_transpose_in32<<<grid, dim3(32, 8), 0, st>>>((const double2*)x, X, b->dim, b->nvec, b->nb);
  const int rc = launch_matvec(b, op, X, b->W, false, nullptr, nullptr, st);
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
  const DevOp& o = b->op->dev;
  kb_slab_pop<<<dim3(b->nslab, b->nb / 32), dim3(32, 8), 0, st>>>(b->S, o.out_off, o.out_dm, o.out_dk, o.out_stride,
                                                                  b->nb, b->pop);
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
  if (!b || (kind != KR_MATVEC_TENSOR && kind != KR_MATVEC_FP32 && kind != KR_MATVEC_TENSOR_TMEM &&
             kind != KR_MATVEC_FP32_REG))
    return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_set_matvec: bad argument");
  b->mv_kind = kind;
  return KR_OK;
}

extern "C" int kr_batch_matvec(kr_batch* b, kr_op* op, void* stream) {
  if (!b || !op || op->dev.dim_out != b->dim || !op->square)
    return set_err(b ? b->op->ctx : nullptr, KR_ERR_ARG, "kr_batch_matvec: operator does not match the batch basis");
  return launch_matvec(b, op, b->V + b->dim * b->nb, b->W, false, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int64_t kr_batch_launch_count(const kr_batch* b) { return b ? b->launches : -1; }
