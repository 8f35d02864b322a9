// Krylov time-propagation step for GB300 (sm_103a): field contraction,
// Kronecker mat-vec and the persistent cooperative Lanczos kernel, plus the
// C ABI declared in include/richmol_gb300.h.
//
// Reference behaviour (CFEL-CMI/richmol):
//   richmol/tdse.py:365-414   split-operator / full-H update
//   richmol/tdse.py:417-486   _expmv_lanczos
//   richmol/field.py:1073-1142 CarTens.field
//   richmol/field.py:1145-1245 CarTens.vec
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "kr_internal.cuh"

#define KR_EXPM_MAX 128  // capacity of the tridiagonal exponential (maxorder <= 128)
#define KR_MATVEC_MAXVEC 65535  // vectors of one kr_matvec call (grid.y)

// ===========================================================================
// field contraction: MF = scale * thr(sum_c coef_c M_c)
// ===========================================================================


// class of a complex number: 3 zero, 1 real, 2 imaginary, 0 general
__device__ __forceinline__ int cclass(double2 z) {
  if (z.x == 0.0 && z.y == 0.0) return 3;
  if (z.y == 0.0) return 1;
  if (z.x == 0.0) return 2;
  return 0;
}
// class of a product: zero absorbs, real is neutral, imaginary * imaginary is real
__device__ __forceinline__ int cclass_mul(int a, int b) {
  if (a == 3 || b == 3) return 3;
  if (a == 0 || b == 0) return 0;
  return a == b ? 1 : 2;
}

template <class Coef>
__global__ void __launch_bounds__(256) kr_field_kernel(DevField f, Coef c) {
  // MF instance types: which components of MF = scale * sum_c coef_c M_c can be
  // non-zero; the mat-vec skips the multiplications by exact zeros
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < f.nmf; i += gridDim.x * blockDim.x) {
    const int g = __ldg(f.mf_group + i);
    const int p = __ldg(f.mf_part + i);
    const int nc = __ldg(f.m_ncart + g);
    int t = 3;
    for (int ci = 0; ci < nc; ++ci) {
      const int ct = cclass_mul(cclass(c.c(p, ci)), (int)f.m_ctype[g * KR_MAXCART + ci]);
      if (ct == 3) continue;
      t = (t == 3) ? ct : (t == ct ? t : 0);
    }
    t = cclass_mul(t, cclass(c.s(p)));
    f.mf_type[i] = (t == 3) ? 1 : t;
  }
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < f.nent;
       e += (long long)gridDim.x * blockDim.x) {
    const int inst = __ldg(f.ent_inst + e);
    const int g = __ldg(f.mf_group + inst);
    const int p = __ldg(f.mf_part + inst);
    const long long local = e - __ldg(f.inst_ptr + inst);
    const long long stride = (long long)__ldg(f.m_rows + g) * __ldg(f.m_width + g);
    const double2* M = f.m_val + __ldg(f.m_val_off + g) + local;
    const int nc = __ldg(f.m_ncart + g);
    double2 v = make_double2(0.0, 0.0);
    for (int ci = 0; ci < nc; ++ci) cfma(v, c.c(p, ci), __ldg(M + ci * stride));
    // field.py:1133-1137: elements below the threshold are dropped
    if (c.t(p) > 0.0 && sqrt(cabs2(v)) < c.t(p)) v = make_double2(0.0, 0.0);
    const double2 mfv = cmul(c.s(p), v);
    f.mf_val[e] = mfv;
    const float2 mh = make_float2((float)mfv.x, (float)mfv.y);
    f.mf_f32[e] = mh;
    f.mf_lo[e] = make_float2((float)(mfv.x - (double)mh.x), (float)(mfv.y - (double)mh.y));
    if (mfv.x != 0.0 || mfv.y != 0.0) {  // band of slots that carry a value with this field
      const int W = __ldg(f.m_width + g);
      const int w = (int)(local % W);
      atomicMax(f.mf_band + 2 * inst, W - 1 - w);
      atomicMax(f.mf_band + 2 * inst + 1, w);
    }
  }
}

// ===========================================================================
// stand-alone mat-vec (CarTens.vec): grid.y runs over vectors
// ===========================================================================
__global__ void __launch_bounds__(KR_THREADS, 2) kr_matvec_kernel(DevOp op, const double2* x, double2* y,
                                                                  unsigned* counters) {
  extern __shared__ double2 smem[];
  __shared__ double2 red[KR_WARPS];
  const long long v = blockIdx.y;
  matvec_cta_tasks<false>(op, x + v * op.dim_in, 1.0, y + v * op.dim_out, counters + v, nullptr, smem, red);
}

// v <- (v * ph) * ph : the two H0 half-phases with no field term (tdse.py:375,394)
__global__ void kr_phase2_kernel(double2* v, const double2* ph, long long dim, long long nvec) {
  const long long n = dim * nvec;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 p = ph[e % dim];
    v[e] = cmul(cmul(v[e], p), p);
  }
}

// ===========================================================================
// exp(A) e0 for the (n x n) complex tridiagonal A = fac * T (one warp).
// Truncated Taylor series applied to the vector with s sub-steps so that
// ||A/s||_1 <= 1 (the action-of-exponential approach of Al-Mohy & Higham,
// SIAM J. Sci. Comput. 33 (2011) 488, without its cost optimisation).
// The reference forms the dense expm (scipy Pade, tdse.py:474) and takes
// column 0; both agree to rounding.
// ===========================================================================
__device__ void warp_expm_e0_smem(const double2* alpha, const double* beta, int n, double2 fac, double2* out,
                                  double2* term, double2* tmp) {
  const int lane = threadIdx.x & 31;
  // 1-norm of A
  double nrm = 0.0;
  for (int i = lane; i < n; i += 32) {
    double cs = sqrt(cabs2(cmul(fac, alpha[i])));
    const double fa = sqrt(cabs2(fac));
    if (i > 0) cs += fa * fabs(beta[i - 1]);
    if (i < n - 1) cs += fa * fabs(beta[i]);
    nrm = fmax(nrm, cs);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nrm = fmax(nrm, __shfl_xor_sync(0xffffffffu, nrm, o));
  int nsub = (int)ceil(nrm);
  if (nsub < 1) nsub = 1;
  if (nsub > 4096) nsub = 4096;
  const double inv_s = 1.0 / (double)nsub;
  for (int i = lane; i < n; i += 32) out[i] = make_double2(i == 0 ? 1.0 : 0.0, 0.0);
  __syncwarp();
  for (int sub = 0; sub < nsub; ++sub) {
    for (int i = lane; i < n; i += 32) term[i] = out[i];
    __syncwarp();
    for (int j = 1; j <= 60; ++j) {
      const double sc = inv_s / (double)j;
      double tmax = 0.0, amax = 0.0;
      for (int i = lane; i < n; i += 32) {
        double2 r = cmul(cmul(fac, alpha[i]), term[i]);
        if (i > 0) cfma(r, cscale(fac, beta[i - 1]), term[i - 1]);
        if (i < n - 1) cfma(r, cscale(fac, beta[i]), term[i + 1]);
        tmp[i] = cscale(r, sc);
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        term[i] = tmp[i];
        out[i] = cadd(out[i], tmp[i]);
        tmax = fmax(tmax, fmax(fabs(tmp[i].x), fabs(tmp[i].y)));
        amax = fmax(amax, fmax(fabs(out[i].x), fabs(out[i].y)));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        tmax = fmax(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
        amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      }
      __syncwarp();
      if (tmax <= 1e-18 * amax) break;
    }
  }
}

// n <= 32: one element per lane, neighbours by shuffles. When fac is purely
// imaginary and T is real (Hermitian H: the diagonal's imaginary parts are
// round-off), A = i tau T and each term costs 3 real x complex products.
__device__ void warp_expm_e0_reg(const double2* alpha, const double* beta, int n, double2 fac, double2* out) {
  const int lane = threadIdx.x & 31;
  const bool act = lane < n;
  const double2 al = act ? alpha[lane] : make_double2(0.0, 0.0);
  const double bl = (lane < n - 1) ? beta[lane] : 0.0;      // couples lane and lane+1
  double bm = __shfl_up_sync(0xffffffffu, bl, 1);            // couples lane-1 and lane
  if (lane == 0) bm = 0.0;
  // 1-norm of A and the realness test
  const double fa = sqrt(fac.x * fac.x + fac.y * fac.y);
  double cs = act ? fa * (sqrt(al.x * al.x + al.y * al.y) + fabs(bm) + fabs(bl)) : 0.0;
  double tmagn = act ? fmax(fabs(al.x), fabs(bl)) : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cs = fmax(cs, __shfl_xor_sync(0xffffffffu, cs, o));
    tmagn = fmax(tmagn, __shfl_xor_sync(0xffffffffu, tmagn, o));
  }
  const bool real_t = (fac.x == 0.0) && __all_sync(0xffffffffu, !act || fabs(al.y) <= 1e-13 * tmagn);
  int nsub = (int)ceil(cs);
  if (nsub < 1) nsub = 1;
  if (nsub > 4096) nsub = 4096;
  const double inv_s = 1.0 / (double)nsub;
  double2 y = make_double2(lane == 0 ? 1.0 : 0.0, 0.0);
  if (real_t) {
    const double tau = fac.y * inv_s;  // A / nsub = i tau T
    for (int sub = 0; sub < nsub; ++sub) {
      double2 t = y, acc = y;
      for (int j = 1; j <= 40; ++j) {
        const double2 tu = make_double2(__shfl_up_sync(0xffffffffu, t.x, 1), __shfl_up_sync(0xffffffffu, t.y, 1));
        const double2 td = make_double2(__shfl_down_sync(0xffffffffu, t.x, 1),
                                        __shfl_down_sync(0xffffffffu, t.y, 1));
        double rx = al.x * t.x, ry = al.x * t.y;
        rx = fma(bm, tu.x, rx);
        ry = fma(bm, tu.y, ry);
        rx = fma(bl, td.x, rx);
        ry = fma(bl, td.y, ry);
        const double sc = tau / (double)j;
        t = act ? make_double2(-sc * ry, sc * rx) : make_double2(0.0, 0.0);  // i * sc * (T t)
        acc.x += t.x;
        acc.y += t.y;
        const double lim = 1e-18 * fmax(1.0, fmax(fabs(acc.x), fabs(acc.y)));
        const bool small = fabs(t.x) <= lim && fabs(t.y) <= lim;
        if (__all_sync(0xffffffffu, small)) break;
      }
      y = acc;
    }
  } else {
    const double2 a = cscale(cmul(fac, al), inv_s);
    const double2 bu = cscale(fac, bm * inv_s), bd = cscale(fac, bl * inv_s);
    for (int sub = 0; sub < nsub; ++sub) {
      double2 t = y, acc = y;
      for (int j = 1; j <= 40; ++j) {
        const double2 tu = make_double2(__shfl_up_sync(0xffffffffu, t.x, 1), __shfl_up_sync(0xffffffffu, t.y, 1));
        const double2 td = make_double2(__shfl_down_sync(0xffffffffu, t.x, 1),
                                        __shfl_down_sync(0xffffffffu, t.y, 1));
        double2 r = cmul(a, t);
        cfma(r, bu, tu);
        cfma(r, bd, td);
        const double sc = 1.0 / (double)j;
        t = act ? cscale(r, sc) : make_double2(0.0, 0.0);
        acc = cadd(acc, t);
        const double lim = 1e-18 * fmax(1.0, fmax(fabs(acc.x), fabs(acc.y)));
        const bool small = fabs(t.x) <= lim && fabs(t.y) <= lim;
        if (__all_sync(0xffffffffu, small)) break;
      }
      y = acc;
    }
  }
  if (act) out[lane] = y;
}

// exp(A) e0 for A = fac * T, T (n x n) tridiagonal with diagonal alpha and
// symmetric off-diagonal beta (tdse.py:474 takes column 0 of the same expm).
__device__ void warp_expm_e0(const double2* alpha, const double* beta, int n, double2 fac, double2* out,
                             double2* term, double2* tmp) {
  if (n <= 32)
    warp_expm_e0_reg(alpha, beta, n, fac, out);
  else
    warp_expm_e0_smem(alpha, beta, n, fac, out, term, tmp);
}

// ===========================================================================
// persistent cooperative Lanczos kernel: one TDSE.update of one vector
// ===========================================================================
struct StepArgs {
  DevOp op;
  double2* state;          // (dim) in/out
  const double2* phase;    // (dim) or null
  double2* V;              // maxorder x dim
  double2* Wb[2];          // residual vectors W_{k-1}, W_k
  double2* w;              // H V_k
  double2* ub[2];          // successive solutions
  double2* part_a;         // per-CTA partials
  double2* task_alpha;     // per-task partials of vdot(w, V_k)
  unsigned* counters;      // task counters, one per mat-vec of the step
  double* part_b;
  double* part_c;
  double2* alpha;          // T diagonal   (maxorder)
  double* beta;            // T off-diagonal (maxorder)
  unsigned* bar_count;
  unsigned* bar_gen;
  int* status;
  int* kout;
  float4* xdf;  // double-float copy of the vector the next mat-vec reads (DF kernels)
  double2 fac;
  double tol;
  int maxorder;
  long long dim;
};

struct StepSmem {
  double2 red[KR_WARPS];
  double2 c[KR_EXPM_MAX];
  double2 ta[KR_EXPM_MAX];
  double tb[KR_EXPM_MAX];
  double2 term[KR_EXPM_MAX];
  double2 tmp[KR_EXPM_MAX];
  double scalar[4];
};

// the mat-vec of the plain step: FP64 products, or double-float ones (DF) from
// the copy a.xdf of the vector, which the vector phases write beside it
template <bool DF>
__device__ __forceinline__ void step_matvec(const StepArgs& a, const double2* x, double xscale, unsigned* counter,
                                            double2* smem, double2* red) {
  if constexpr (DF) matvec_cta_tasks_df<true>(a.op, x, a.xdf, xscale, a.w, counter, a.task_alpha, smem, red);
  else matvec_cta_tasks<true>(a.op, x, xscale, a.w, counter, a.task_alpha, smem, red);
}

template <bool DF>
__global__ void __launch_bounds__(KR_THREADS, DF ? 3 : 2) kr_step_kernel(StepArgs a) {
  extern __shared__ double2 smem_dyn[];
  __shared__ StepSmem ss;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nblk = gridDim.x;
  const long long gtid = blockIdx.x * (long long)blockDim.x + tid;
  const long long gstride = (long long)nblk * blockDim.x;
  const long long n = a.dim;

  if (*((volatile int*)a.status) != 0) return;  // sticky error from an earlier launch
  if (blockIdx.x == 0)
    for (int i = tid; i < a.maxorder + 2; i += blockDim.x) a.counters[i] = 0u;

  // ---- V0 = phase * state (tdse.py:375) -----------------------------------
  double2* V0 = a.V;
  for (long long e = gtid; e < n; e += gstride) {
    double2 v = a.state[e];
    if (a.phase) v = cmul(v, a.phase[e]);
    V0[e] = v;
    if (DF) df2_st(a.xdf + e, df2_split(v));
  }
  if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;

  // ---- k = 0: w = H V0, T00 = vdot(w, V0), W0 = w - T00 V0 (tdse.py:443-446)
  step_matvec<DF>(a, V0, 1.0, a.counters, smem_dyn, ss.red);
  if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
  {
    const double2 a0 = grid_partials_sum2(a.task_alpha, a.op.ntask, ss.red);
    if (blockIdx.x == 0 && tid == 0) a.alpha[0] = a0;
    double bp = 0.0;
    double2* W0 = a.Wb[0];
    for (long long e = gtid; e < n; e += gstride) {
      double2 r = ldcg2(a.w + e);
      const double2 v = ldcg2(V0 + e);
      r = csub(r, cmul(a0, v));
      W0[e] = r;
      if (DF) df2_st(a.xdf + e, df2_split(r));
      bp += cabs2(r);
    }
    const double2 s = block_sum2(make_double2(bp, 0.0), ss.red);
    if (tid == 0) a.part_b[blockIdx.x] = s.x;
  }
  if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;

  // ---- Lanczos iterations (tdse.py:450-478) -------------------------------
  int k = 1;
  const double2* uprev = V0;
  double2* unext = a.ub[1];
  bool done = false;
  while (!done) {
    // beta_{k-1} = ||W_{k-1}|| (tdse.py:453)
    double beta_k;
    {
      // sum of part_b (doubles) in a fixed order
      __syncthreads();
      if (warp == 0) {
        double s = 0.0;
        for (int i = lane; i < nblk; i += 32) s += __ldcg(a.part_b + i);
        s = warp_sum(s);
        if (lane == 0) ss.scalar[0] = s;
      }
      __syncthreads();
      beta_k = sqrt(ss.scalar[0]);
      __syncthreads();
    }
    if (blockIdx.x == 0 && tid == 0) a.beta[k - 1] = beta_k;
    double2* Vk = a.V + (long long)k * n;
    const double2* Vkm1 = a.V + (long long)(k - 1) * n;
    const double2* xsrc;
    double xscale;
    if (beta_k != 0.0) {
      const double2* Wprev = a.Wb[(k - 1) & 1];
      xscale = 1.0 / beta_k;
      xsrc = Wprev;
      for (long long e = gtid; e < n; e += gstride) Vk[e] = cscale(ldcg2(Wprev + e), xscale);
    } else {
      // breakdown: orthonormalise a vector of ones against V_0..V_{k-1} (tdse.py:459-465)
      for (long long e = gtid; e < n; e += gstride) Vk[e] = make_double2(1.0, 0.0);
      for (int j = 0; j < k; ++j) {
        if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
        const double2* Vj = a.V + (long long)j * n;
        double2 pp = make_double2(0.0, 0.0);
        for (long long e = gtid; e < n; e += gstride) pp = cadd(pp, cconjmul(ldcg2(Vj + e), ldcg2(Vk + e)));
        pp = block_sum2(pp, ss.red);
        if (tid == 0) a.part_a[blockIdx.x] = pp;
        if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
        const double2 proj = grid_partials_sum2(a.part_a, nblk, ss.red);
        for (long long e = gtid; e < n; e += gstride) Vk[e] = csub(ldcg2(Vk + e), cmul(proj, ldcg2(Vj + e)));
      }
      if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
      double np_ = 0.0;
      for (long long e = gtid; e < n; e += gstride) np_ += cabs2(ldcg2(Vk + e));
      const double2 ns = block_sum2(make_double2(np_, 0.0), ss.red);
      if (tid == 0) a.part_b[blockIdx.x] = ns.x;
      if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
      __syncthreads();
      if (warp == 0) {
        double s = 0.0;
        for (int i = lane; i < nblk; i += 32) s += __ldcg(a.part_b + i);
        s = warp_sum(s);
        if (lane == 0) ss.scalar[1] = sqrt(s);
      }
      __syncthreads();
      const double nrm = ss.scalar[1];
      for (long long e = gtid; e < n; e += gstride) {
        const double2 v = ldcg2(Vk + e);
        Vk[e] = make_double2(v.x / nrm, v.y / nrm);
        if (DF) df2_st(a.xdf + e, df2_split(make_double2(v.x / nrm, v.y / nrm)));
      }
      if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;
      xsrc = Vk;
      xscale = 1.0;
    }

    // w = H V_k and T_kk = vdot(w, V_k) (tdse.py:467-468)
    step_matvec<DF>(a, xsrc, xscale, a.counters + k, smem_dyn, ss.red);
    if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;

    // T_kk, then exp(fac T_{0..k}) e0 in every CTA (tdse.py:474)
    const double2 ak = grid_partials_sum2(a.task_alpha, a.op.ntask, ss.red);
    if (blockIdx.x == 0 && tid == 0) a.alpha[k] = ak;
    __syncthreads();
    if (warp == 0) {
      for (int i = lane; i <= k; i += 32) {
        ss.ta[i] = (i == k) ? ak : __ldcg(a.alpha + i);
        if (i < k) ss.tb[i] = (i == k - 1) ? beta_k : __ldcg(a.beta + i);
      }
      __syncwarp();
      warp_expm_e0(ss.ta, ss.tb, k + 1, a.fac, ss.c, ss.term, ss.tmp);
    }
    __syncthreads();

    // W_k = w - T_kk V_k - beta_{k-1} V_{k-1} (tdse.py:469);
    // u_k = sum_i c_i V_i, conv = ||u_k - u_{k-1}||^2 (tdse.py:475-476)
    {
      double bp = 0.0, cp = 0.0;
      double2* Wk = a.Wb[k & 1];
      for (long long e = gtid; e < n; e += gstride) {
        const double2 vk = ldcg2(Vk + e);
        double2 r = csub(ldcg2(a.w + e), cmul(ak, vk));
        r = csub(r, cscale(ldcg2(Vkm1 + e), beta_k));
        Wk[e] = r;
        if (DF) df2_st(a.xdf + e, df2_split(r));
        bp += cabs2(r);
        double2 u = make_double2(0.0, 0.0);
        for (int i = 0; i <= k; ++i) cfma(u, ss.c[i], ldcg2(a.V + (long long)i * n + e));
        const double2 d = csub(u, ldcg2(uprev + e));
        cp += cabs2(d);
        unext[e] = u;
      }
      const double2 s = block_sum2(make_double2(bp, cp), ss.red);
      if (tid == 0) {
        a.part_b[blockIdx.x] = s.x;
        a.part_c[blockIdx.x] = s.y;
      }
    }
    if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return;

    double conv;
    __syncthreads();
    if (warp == 0) {
      double s = 0.0;
      for (int i = lane; i < nblk; i += 32) s += __ldcg(a.part_c + i);
      s = warp_sum(s);
      if (lane == 0) ss.scalar[2] = s;
    }
    __syncthreads();
    conv = ss.scalar[2];
    __syncthreads();
    k += 1;
    uprev = unext;
    unext = a.ub[k & 1];
    if (!(conv > a.tol)) done = true;
    if (k >= a.maxorder) {
      if (blockIdx.x == 0 && tid == 0) atomicCAS(a.status, 0, KR_ERR_MAXORDER);
      done = true;
    }
  }

  // ---- state = phase * u_k (tdse.py:394) ---------------------------------
  for (long long e = gtid; e < n; e += gstride) {
    double2 u = ldcg2(uprev + e);
    if (a.phase) u = cmul(u, a.phase[e]);
    a.state[e] = u;
  }
  if (blockIdx.x == 0 && tid == 0) *a.kout = k;
}

// ===========================================================================
// Segmented step: independent problems (molecules) whose vectors lie one after
// the other in one vector, under one block-diagonal operator. One persistent
// launch runs the Lanczos recurrence of kr_step_kernel for every segment at
// once, each with its own scalars (alpha, beta, exp(fac T) e0), its own
// stopping test (squared distance of successive solutions, tdse.py:476) and
// Krylov order: the mat-vec tasks of the whole ragged block table are shared,
// the per-element work goes in chunks that lie inside one segment, and every
// per-segment sum is taken over that segment's chunk (or task) partials in a
// fixed order. A segment whose Krylov space closes (beta = 0) ends with the
// exact solution of that space. Segments that have converged are skipped.
// ===========================================================================
struct SegArgs {
  DevOp op;
  double2* state;
  const double2* phase;
  double2* V;
  double2* Wb[2];
  double2* w;
  double2* ub[2];
  double2* task_alpha;
  unsigned* counters;
  unsigned* bar_count;
  unsigned* bar_gen;
  int* status;
  int nseg, nchunk;
  const int* slab_seg;       // [nslab] segment of each slab
  const int* chunk_seg;      // [nchunk]
  const long long* chunk_e0; // [nchunk] element range of each chunk
  const long long* chunk_e1;
  const int* seg_chunk_ptr;  // [nseg + 1] chunks of each segment
  const int* seg_task_ptr;   // [nseg + 1] mat-vec tasks of each segment ...
  const int* seg_tasks;      // ... their indices, ascending
  double2* alpha;            // [nseg][maxorder + 1]
  double* beta;              // [nseg][maxorder + 1]
  double2* coef;             // [nseg][maxorder + 1] exp(fac T) e0 of the last order
  int* done;                 // [nseg]
  int* kout;                 // [nseg] Krylov order used
  int* ufin;                 // [nseg] final solution: ub[ufin], or coef[0] V0 if -1
  double* chunk_b;           // [nchunk] partial sums
  double* chunk_c;
  int* nactive;              // [2] segments still running, by iteration parity
  double2 fac;
  double tol;
  int maxorder;
  long long dim;
};

// sum of the doubles part[p[0] .. p[1]) by one warp in a fixed order (all lanes)
__device__ __forceinline__ double seg_warp_sum(const double* part, int b, int e, int lane) {
  double s = 0.0;
  for (int i = b + lane; i < e; i += 32) s += __ldcg(part + i);
  return warp_sum(s);
}

template <bool F32>
__global__ void __launch_bounds__(KR_THREADS, F32 ? 3 : 2) kr_seg_step_kernel(SegArgs a) {
  extern __shared__ double2 smem_dyn[];
  __shared__ StepSmem ss;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nblk = gridDim.x;
  const int M1 = a.maxorder + 1;
  const long long n = a.dim;
#define SEG_BARRIER() \
  if (!grid_barrier(a.bar_count, a.bar_gen, a.status, KR_ERR_TIMEOUT)) return

  if (*((volatile int*)a.status) != 0) return;  // sticky error from an earlier launch
  if (blockIdx.x == 0) {
    for (int i = tid; i < a.maxorder + 2; i += blockDim.x) a.counters[i] = 0u;
    if (tid < 2) a.nactive[tid] = 0;
  }
  for (int sg = blockIdx.x * blockDim.x + tid; sg < a.nseg; sg += nblk * blockDim.x) {
    a.done[sg] = 0;
    a.kout[sg] = 0;
    a.ufin[sg] = -1;
  }
  double2* V0 = a.V;
  for (int ch = blockIdx.x; ch < a.nchunk; ch += nblk)
    for (long long e = a.chunk_e0[ch] + tid; e < a.chunk_e1[ch]; e += blockDim.x) {
      double2 v = a.state[e];
      if (a.phase) v = cmul(v, a.phase[e]);
      V0[e] = v;
    }
  SEG_BARRIER();

  // w = H V0, alpha_0 = vdot(w, V0), W0 = w - alpha_0 V0 (tdse.py:443-446)
  matvec_cta_tasks<true, F32>(a.op, V0, 1.0, a.w, a.counters, a.task_alpha, smem_dyn, ss.red, a.done, a.slab_seg);
  SEG_BARRIER();
  if (warp == 0)
    for (int sg = blockIdx.x; sg < a.nseg; sg += nblk) {
      double2 t = make_double2(0.0, 0.0);
      for (int i = a.seg_task_ptr[sg] + lane; i < a.seg_task_ptr[sg + 1]; i += 32) t = cadd(t, ldcg2(a.task_alpha + a.seg_tasks[i]));
      t = warp_sum2(t);
      if (lane == 0) a.alpha[(long long)sg * M1] = t;
    }
  SEG_BARRIER();
  for (int ch = blockIdx.x; ch < a.nchunk; ch += nblk) {
    const int sg = a.chunk_seg[ch];
    const double2 a0 = ldcg2(a.alpha + (long long)sg * M1);
    double bp = 0.0;
    for (long long e = a.chunk_e0[ch] + tid; e < a.chunk_e1[ch]; e += blockDim.x) {
      const double2 r = csub(ldcg2(a.w + e), cmul(a0, ldcg2(V0 + e)));
      a.Wb[0][e] = r;
      bp += cabs2(r);
    }
    const double2 sb = block_sum2(make_double2(bp, 0.0), ss.red);
    if (tid == 0) a.chunk_b[ch] = sb.x;
  }
  SEG_BARRIER();

  int k = 1;
  for (;;) {
    // beta_{k-1} = ||W_{k-1}|| per segment; a closed Krylov space ends the segment
    if (warp == 0)
      for (int sg = blockIdx.x; sg < a.nseg; sg += nblk) {
        if (__ldcg(a.done + sg)) continue;
        const double b2 = seg_warp_sum(a.chunk_b, a.seg_chunk_ptr[sg], a.seg_chunk_ptr[sg + 1], lane);
        if (lane == 0) {
          const double b = sqrt(b2);
          a.beta[(long long)sg * M1 + k - 1] = b;
          if (b == 0.0) {
            if (k == 1) {  // V0 spans the space: u = exp(fac alpha_0) V0
              const double2 z = cmul(a.fac, ldcg2(a.alpha + (long long)sg * M1));
              const double m = exp(z.x);
              a.coef[(long long)sg * M1] = make_double2(m * cos(z.y), m * sin(z.y));
              a.ufin[sg] = -1;
            } else {
              a.ufin[sg] = (k - 1) & 1;  // u_{k-1} is exact
            }
            a.kout[sg] = k;
            a.done[sg] = 1;
          }
        }
      }
    SEG_BARRIER();
    double2* Vk = a.V + (long long)k * n;
    const double2* Vkm1 = a.V + (long long)(k - 1) * n;
    const double2* Wprev = a.Wb[(k - 1) & 1];
    for (int ch = blockIdx.x; ch < a.nchunk; ch += nblk) {
      const int sg = a.chunk_seg[ch];
      if (__ldcg(a.done + sg)) continue;
      const double inv = 1.0 / __ldcg(a.beta + (long long)sg * M1 + k - 1);
      for (long long e = a.chunk_e0[ch] + tid; e < a.chunk_e1[ch]; e += blockDim.x) Vk[e] = cscale(ldcg2(Wprev + e), inv);
    }
    SEG_BARRIER();
    // w = H V_k (tdse.py:467-468)
    matvec_cta_tasks<true, F32>(a.op, Vk, 1.0, a.w, a.counters + k, a.task_alpha, smem_dyn, ss.red, a.done,
                                a.slab_seg);
    SEG_BARRIER();
    // alpha_k and exp(fac T_{0..k}) e0 per segment (tdse.py:474)
    if (warp == 0)
      for (int sg = blockIdx.x; sg < a.nseg; sg += nblk) {
        if (__ldcg(a.done + sg)) continue;
        double2 t = make_double2(0.0, 0.0);
        for (int i = a.seg_task_ptr[sg] + lane; i < a.seg_task_ptr[sg + 1]; i += 32)
          t = cadd(t, ldcg2(a.task_alpha + a.seg_tasks[i]));
        const double2 ak = warp_sum2(t);
        for (int i = lane; i <= k; i += 32) {
          ss.ta[i] = (i == k) ? ak : ldcg2(a.alpha + (long long)sg * M1 + i);
          if (i < k) ss.tb[i] = __ldcg(a.beta + (long long)sg * M1 + i);
        }
        __syncwarp();
        warp_expm_e0(ss.ta, ss.tb, k + 1, a.fac, ss.c, ss.term, ss.tmp);
        __syncwarp();
        for (int i = lane; i <= k; i += 32) a.coef[(long long)sg * M1 + i] = ss.c[i];
        if (lane == 0) a.alpha[(long long)sg * M1 + k] = ak;
        __syncwarp();
      }
    SEG_BARRIER();
    // W_k = w - alpha_k V_k - beta_{k-1} V_{k-1} (tdse.py:469); u_k = sum_i c_i V_i,
    // distance to u_{k-1} (tdse.py:475-476)
    {
      const double2* uprev = (k == 1) ? V0 : a.ub[(k - 1) & 1];
      double2* unext = a.ub[k & 1];
      double2* Wk = a.Wb[k & 1];
      for (int ch = blockIdx.x; ch < a.nchunk; ch += nblk) {
        const int sg = a.chunk_seg[ch];
        if (__ldcg(a.done + sg)) continue;
        __syncthreads();  // ss.c of the previous chunk is no longer read
        for (int i = tid; i <= k; i += blockDim.x) ss.c[i] = ldcg2(a.coef + (long long)sg * M1 + i);
        __syncthreads();
        const double2 ak = ldcg2(a.alpha + (long long)sg * M1 + k);
        const double bk = __ldcg(a.beta + (long long)sg * M1 + k - 1);
        double bp = 0.0, cp = 0.0;
        for (long long e = a.chunk_e0[ch] + tid; e < a.chunk_e1[ch]; e += blockDim.x) {
          const double2 vk = ldcg2(Vk + e);
          double2 r = csub(ldcg2(a.w + e), cmul(ak, vk));
          r = csub(r, cscale(ldcg2(Vkm1 + e), bk));
          Wk[e] = r;
          bp += cabs2(r);
          double2 u = make_double2(0.0, 0.0);
          for (int i = 0; i <= k; ++i) cfma(u, ss.c[i], ldcg2(a.V + (long long)i * n + e));
          cp += cabs2(csub(u, ldcg2(uprev + e)));
          unext[e] = u;
        }
        const double2 sc = block_sum2(make_double2(bp, cp), ss.red);
        if (tid == 0) {
          a.chunk_b[ch] = sc.x;
          a.chunk_c[ch] = sc.y;
        }
      }
    }
    SEG_BARRIER();
    // stopping test per segment
    if (warp == 0)
      for (int sg = blockIdx.x; sg < a.nseg; sg += nblk) {
        if (__ldcg(a.done + sg)) continue;
        const double conv = seg_warp_sum(a.chunk_c, a.seg_chunk_ptr[sg], a.seg_chunk_ptr[sg + 1], lane);
        if (lane == 0) {
          if (!(conv > a.tol) || k + 1 >= a.maxorder) {
            if (conv > a.tol) atomicCAS(a.status, 0, KR_ERR_MAXORDER);  // tdse.py:480-484
            a.ufin[sg] = k & 1;
            a.kout[sg] = k + 1;
            a.done[sg] = 1;
          } else {
            atomicAdd(a.nactive + (k & 1), 1);
          }
        }
      }
    SEG_BARRIER();
    const int act = __ldcg(a.nactive + (k & 1));
    if (blockIdx.x == 0 && tid == 0) a.nactive[(k + 1) & 1] = 0;  // counted again two barriers later
    if (act == 0) break;
    k += 1;
  }
  SEG_BARRIER();
  // state = phase * u (tdse.py:394)
  for (int ch = blockIdx.x; ch < a.nchunk; ch += nblk) {
    const int sg = a.chunk_seg[ch];
    const int f = __ldcg(a.ufin + sg);
    const double2 c0 = (f < 0) ? ldcg2(a.coef + (long long)sg * M1) : make_double2(0.0, 0.0);
    for (long long e = a.chunk_e0[ch] + tid; e < a.chunk_e1[ch]; e += blockDim.x) {
      double2 u = (f < 0) ? cmul(c0, ldcg2(V0 + e)) : ldcg2(a.ub[f] + e);
      if (a.phase) u = cmul(u, a.phase[e]);
      a.state[e] = u;
    }
  }
#undef SEG_BARRIER
}

// ===========================================================================
// host side
// ===========================================================================
namespace {
std::mutex g_err_mu;
std::string g_err;
}  // namespace

int kr_set_err(kr_ctx* ctx, int code, const std::string& msg) {
  // one context serves every thread of a process: its message is guarded too
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (ctx) ctx->err = msg;
  g_err = msg;
  return code;
}

std::recursive_mutex& kr_device_mutex() {
  static std::recursive_mutex mu;
  return mu;
}



template <typename T>
static int upload(kr_op* op, const T* host, size_t count, T** dev) {
  *dev = nullptr;
  size_t bytes = sizeof(T) * std::max<size_t>(count, 1);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return set_err(op->ctx, KR_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  op->allocs.push_back(p);
  if (count && host) {
    e = cudaMemcpy(p, host, sizeof(T) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_err(op->ctx, KR_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  } else {
    cudaMemset(p, 0, bytes);
  }
  *dev = static_cast<T*>(p);
  return KR_OK;
}

extern "C" int kr_ctx_create(int device, kr_ctx** out) {
  if (!out) return set_err(nullptr, KR_ERR_ARG, "kr_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_err(nullptr, KR_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return set_err(nullptr, KR_ERR_ARG, "kr_ctx_create: bad device index");
  DeviceScope scope(device);
  if (scope.err != cudaSuccess)
    return set_err(nullptr, KR_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(scope.err));
  kr_ctx* c = new kr_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) {
    delete c;
    return set_err(nullptr, KR_ERR_UNSUPPORTED, "device does not support cooperative launch");
  }
  *out = c;
  return KR_OK;
}

extern "C" void kr_ctx_destroy(kr_ctx* ctx) { delete ctx; }

extern "C" int kr_last_error(const kr_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return KR_ERR_ARG;
  std::string m;
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    m = ctx ? ctx->err : g_err;
  }
  std::snprintf(buf, len, "%s", m.c_str());
  return KR_OK;
}

extern "C" void kr_op_destroy(kr_op* op) {
  if (!op) return;
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  for (void* p : op->allocs) cudaFree(p);
  if (op->expv_ws) cudaFree(op->expv_ws);
  if (op->fs_buf) cudaFree(op->fs_buf);
  delete op;
}

namespace {

// Splits an output slab of dm1 rows x nk1 columns into row tasks for one CTA
// of KR_THREADS threads, each thread owning at most KR_QMAX outputs: picks
// the task count with the best thread occupancy (finer on near-ties).
int pick_task_rows(int nk1, int dm1) {
  const long long P = (long long)dm1 * nk1;
  int best_R = dm1;
  double best_eff = -1.0;
  for (int m = 1; m <= dm1; ++m) {
    const int R = (dm1 + m - 1) / m;
    const int mm = (dm1 + R - 1) / R;
    const int q = (R * nk1 + KR_THREADS - 1) / KR_THREADS;
    if (q > KR_QMAX) continue;
    const double eff = double(P) / (double(mm) * q * KR_THREADS);
    if (eff > best_eff * 1.02 || (eff > best_eff * 0.98 && R < best_R && mm <= 64)) {
      if (eff > best_eff) best_eff = eff;
      best_R = R;
    }
    if (q == 1 && R * nk1 <= KR_THREADS / 4) break;  // finer tasks only lose occupancy
  }
  return best_R;
}

}  // namespace

// The dynamic shared memory attribute of the plain kernels is a property of
// the kernel, not of an operator: it only ever grows (to the largest operator
// seen), so a launch of any operator stays within it, whatever operators were
// created since, by this thread or another.
static std::mutex g_smem_mu;
static size_t g_smem_max = 0;
static cudaError_t ensure_step_smem(size_t smem) {
  std::lock_guard<std::mutex> lk(g_smem_mu);
  if (smem <= g_smem_max) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kr_step_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kr_step_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kr_matvec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kr_seg_step_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kr_seg_step_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) g_smem_max = smem;
  return e;
}

// the plain step kernel of an operator's precision, and its cooperative grid
static void* step_kernel(const kr_op* op) {
  return op->prec == KR_PREC_DF ? (void*)kr_step_kernel<true> : (void*)kr_step_kernel<false>;
}
static int step_grid(const kr_op* op) { return op->prec == KR_PREC_DF ? op->grid_df : op->grid; }

extern "C" int kr_op_set_precision(kr_op* op, int32_t prec) {
  if (!op || (prec != KR_PREC_F64 && prec != KR_PREC_DF))
    return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_op_set_precision: bad argument");
  op->prec = prec;
  return KR_OK;
}

namespace {
// What the validation of a descriptor derives: column chunks present, row
// strides of every slab, and the terms of every output slab.
struct DescCheck {
  bool split = false;
  std::vector<int> out_stride, in_stride;
  std::vector<std::vector<int>> by_out;
};

// Validates a descriptor on the host (no device work): KR_OK, or the status
// and message of the first problem found.
int check_desc(const kr_op_desc* d, DescCheck& c, std::string& err) {
  auto fail = [&err](int code, const std::string& msg) {
    err = msg;
    return code;
  };
  if (d->nslab_out <= 0 || d->nslab_in <= 0) return fail(KR_ERR_ARG, "empty basis");
  if (d->npart < 0 || d->npart > KR_MAXPART) return fail(KR_ERR_ARG, "npart out of range");
  if (d->maxorder < 2 || d->maxorder > KR_EXPM_MAX) return fail(KR_ERR_ARG, "maxorder out of range [2, 128]");
  bool& split = c.split;
  std::vector<int>& out_stride = c.out_stride;
  std::vector<int>& in_stride = c.in_stride;
  split = false;
  out_stride.assign(d->nslab_out, 0);
  in_stride.assign(d->nslab_in, 0);
  if (!d->out_stride != !d->in_stride) return fail(KR_ERR_ARG, "slab strides given on one side only");
  if (!d->out_stride) {
    long long off = 0;
    for (int s = 0; s < d->nslab_out; ++s) {
      if (d->out_off[s] != off || d->out_dm[s] <= 0 || d->out_dk[s] <= 0)
        return fail(KR_ERR_ARG, "malformed output slab table");
      if (d->out_dk[s] > 32 * KR_QMAX) return fail(KR_ERR_UNSUPPORTED, "n_k above 128 not supported");
      off += (long long)d->out_dm[s] * d->out_dk[s];
      out_stride[s] = d->out_dk[s];
    }
    if (off != d->dim_out) return fail(KR_ERR_ARG, "dim_out does not match the slab table");
    off = 0;
    for (int s = 0; s < d->nslab_in; ++s) {
      if (d->in_off[s] != off || d->in_dm[s] <= 0 || d->in_dk[s] <= 0)
        return fail(KR_ERR_ARG, "malformed input slab table");
      off += (long long)d->in_dm[s] * d->in_dk[s];
      in_stride[s] = d->in_dk[s];
    }
    if (off != d->dim_in) return fail(KR_ERR_ARG, "dim_in does not match the slab table");
  } else {
    // column chunks: every element of the vector in exactly one chunk
    for (int side = 0; side < 2; ++side) {
      const int ns = side ? d->nslab_in : d->nslab_out;
      const int32_t *dm = side ? d->in_dm : d->out_dm, *dk = side ? d->in_dk : d->out_dk;
      const int32_t* st = side ? d->in_stride : d->out_stride;
      const int64_t* off = side ? d->in_off : d->out_off;
      const long long dim = side ? d->dim_in : d->dim_out;
      std::vector<unsigned char> seen((size_t)std::max(dim, 1LL), 0);
      for (int s = 0; s < ns; ++s) {
        if (dm[s] <= 0 || dk[s] <= 0 || st[s] < dk[s] || off[s] < 0 ||
            off[s] + (long long)(dm[s] - 1) * st[s] + dk[s] > dim)
          return fail(KR_ERR_ARG, "malformed slab chunk table");
        if (dk[s] > 32 * KR_QMAX) return fail(KR_ERR_UNSUPPORTED, "n_k above 128 not supported");
        for (int i = 0; i < dm[s]; ++i)
          for (int a = 0; a < dk[s]; ++a) {
            unsigned char& c = seen[(size_t)(off[s] + (long long)i * st[s] + a)];
            if (c) return fail(KR_ERR_ARG, "slab chunks overlap");
            c = 1;
          }
        (side ? in_stride : out_stride)[s] = st[s];
        split = split || st[s] != dk[s];
      }
      for (long long e = 0; e < dim; ++e)
        if (!seen[(size_t)e]) return fail(KR_ERR_ARG, "slab chunks do not cover the vector");
    }
  }
  for (int g = 0; g < d->nm; ++g) {
    if (d->m_rows[g] <= 0 || d->m_width[g] < 0 || d->m_ncart[g] < 1 || d->m_ncart[g] > KR_MAXCART)
      return fail(KR_ERR_ARG, "malformed M group");
    const long long ne = (long long)d->m_rows[g] * d->m_width[g];
    if (d->m_col_off[g] < 0 || d->m_col_off[g] + ne > d->m_col_len) return fail(KR_ERR_ARG, "M columns out of range");
    if (d->m_val_off[g] < 0 || d->m_val_off[g] + ne * d->m_ncart[g] > d->m_val_len / 2)
      return fail(KR_ERR_ARG, "M values out of range");
  }
  for (int i = 0; i < d->nmf; ++i)
    if (d->mf_group[i] < 0 || d->mf_group[i] >= d->nm || d->mf_part[i] < 0 || d->mf_part[i] >= d->npart)
      return fail(KR_ERR_ARG, "malformed MF instance");
  for (int b = 0; b < d->nk; ++b) {
    const int words = d->k_type[b] == KR_K_COMPLEX ? 2 : 1;
    if (d->k_type[b] < 0 || d->k_type[b] > 2) return fail(KR_ERR_ARG, "bad K type");
    if (d->k_off[b] < 0 || d->k_off[b] + (long long)d->k_rows[b] * d->k_cols[b] * words > d->k_data_len)
      return fail(KR_ERR_ARG, "K block out of range");
    if (d->k_type[b] == KR_K_COMPLEX && (d->k_off[b] & 1)) return fail(KR_ERR_ARG, "complex K block misaligned");
  }
  std::vector<std::vector<int>>& by_out = c.by_out;
  by_out.assign(d->nslab_out, {});
  for (int t = 0; t < d->nterm; ++t) {
    const int s1 = d->t_out[t], s2 = d->t_in[t], kb = d->t_k[t], mi = d->t_mf[t];
    if (s1 < 0 || s1 >= d->nslab_out || s2 < 0 || s2 >= d->nslab_in || kb < 0 || kb >= d->nk || mi < 0 || mi >= d->nmf)
      return fail(KR_ERR_ARG, "term index out of range");
    const int g = d->mf_group[mi];
    if (d->k_rows[kb] != d->out_dk[s1] || d->k_cols[kb] != d->in_dk[s2])
      return fail(KR_ERR_ARG, "K block shape does not match its slabs");
    if (d->m_rows[g] != d->out_dm[s1]) return fail(KR_ERR_ARG, "M group rows do not match the output slab");
    const long long ne = (long long)d->m_rows[g] * d->m_width[g];
    for (long long e = 0; e < ne; ++e) {
      const int c = d->m_col[d->m_col_off[g] + e];
      if (c < 0 || c >= d->in_dm[s2]) return fail(KR_ERR_ARG, "M column outside the input slab");
    }
    by_out[s1].push_back(t);
  }

  return KR_OK;
}
}  // namespace

extern "C" int kr_op_check(const kr_op_desc* d, char* buf, size_t len) {
  if (buf && len) buf[0] = 0;
  if (!d) return set_err(nullptr, KR_ERR_ARG, "kr_op_check: NULL descriptor");
  DescCheck c;
  std::string msg;
  const int rc = check_desc(d, c, msg);
  if (rc != KR_OK) {
    if (buf && len) {
      std::strncpy(buf, msg.c_str(), len - 1);
      buf[len - 1] = 0;
    }
    return set_err(nullptr, rc, msg);
  }
  return KR_OK;
}

extern "C" int kr_op_create(kr_ctx* ctx, const kr_op_desc* d, kr_op** out) {
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  if (!ctx || !d || !out) return set_err(ctx, KR_ERR_ARG, "kr_op_create: NULL argument");
  *out = nullptr;
  KR_DEVICE_SCOPE(ctx, ctx->device);
  // ---- validation (check_desc) -----------------------------------------------
  DescCheck dchk;
  {
    std::string msg;
    const int rc = check_desc(d, dchk, msg);
    if (rc != KR_OK) return set_err(ctx, rc, msg);
  }
  const bool split = dchk.split;
  const std::vector<int>& out_stride = dchk.out_stride;
  const std::vector<int>& in_stride = dchk.in_stride;
  const std::vector<std::vector<int>>& by_out = dchk.by_out;

  static std::atomic<unsigned long long> next_uid{1};
  kr_op* op = new kr_op();
  op->uid = next_uid.fetch_add(1);
  op->ctx = ctx;
  op->maxorder = d->maxorder;
  op->npart = d->npart;
  op->nmf = d->nmf;
  op->split = split;
  op->square = (d->nslab_out == d->nslab_in) && (d->dim_out == d->dim_in);
  if (op->square)
    for (int s = 0; s < d->nslab_out; ++s)
      if (d->out_dm[s] != d->in_dm[s] || d->out_dk[s] != d->in_dk[s] || d->out_off[s] != d->in_off[s] ||
          out_stride[s] != in_stride[s])
        op->square = false;

  // ---- terms grouped by output slab ---------------------------------------
  std::vector<int> term_ptr(d->nslab_out + 1, 0), t_in, t_k, t_mf;
  for (int s = 0; s < d->nslab_out; ++s) {
    term_ptr[s + 1] = term_ptr[s] + (int)by_out[s].size();
    for (int t : by_out[s]) {
      t_in.push_back(d->t_in[t]);
      t_k.push_back(d->t_k[t]);
      t_mf.push_back(d->t_mf[t]);
    }
  }
  // ---- MF instances -----------------------------------------------------------
  std::vector<long long> inst_ptr(d->nmf + 1, 0), mf_col_off(d->nmf);
  std::vector<int> mf_width(d->nmf);
  for (int i = 0; i < d->nmf; ++i) {
    const int g = d->mf_group[i];
    inst_ptr[i + 1] = inst_ptr[i] + (long long)d->m_rows[g] * d->m_width[g];
    mf_col_off[i] = d->m_col_off[g];
    mf_width[i] = d->m_width[g];
  }
  // ---- diagonal slot order of the M groups --------------------------------
  // A group is diagonal when slot w of row i holds column i + d0 + w wherever
  // that column lies in the input slab, and zero values in every Cartesian
  // component where it does not (the stored column is then any in-slab one).
  // The batched mat-vec addresses such bands by offset.
  std::vector<int> group_diag(d->nm, KR_NO_DIAG);
  {
    std::vector<int> gcols(d->nm, -1);  // input slab rows of the terms of each group (-2: they differ)
    for (int t = 0; t < d->nterm; ++t) {
      const int g = d->mf_group[d->t_mf[t]], c = d->in_dm[d->t_in[t]];
      gcols[g] = (gcols[g] == -1 || gcols[g] == c) ? c : -2;
    }
    for (int g = 0; g < d->nm; ++g) {
      const int rows = d->m_rows[g], W = d->m_width[g], ncols = gcols[g];
      if (ncols <= 0 || W < 1 || W > KR_DIAG_MAX) continue;
      const int* col = d->m_col + d->m_col_off[g];
      const long long ne = (long long)rows * W;
      const int mid = rows / 2;
      for (int w0 = 0; w0 < W && group_diag[g] == KR_NO_DIAG; ++w0) {
        const int cand = col[(long long)mid * W + w0] - mid - w0;
        bool ok = true;
        for (int i = 0; i < rows && ok; ++i)
          for (int w = 0; w < W && ok; ++w) {
            const long long e = (long long)i * W + w;
            const long long c = (long long)i + cand + w;
            if (c >= 0 && c < ncols) {
              ok = col[e] == c;
            } else {
              for (int k = 0; k < d->m_ncart[g] && ok; ++k) {
                const double* v = d->m_val + 2 * (d->m_val_off[g] + k * ne + e);
                ok = v[0] == 0.0 && v[1] == 0.0;
              }
            }
          }
        if (ok) group_diag[g] = cand;
      }
    }
  }
  std::vector<int> mf_diag(d->nmf);
  for (int i = 0; i < d->nmf; ++i) mf_diag[i] = group_diag[d->mf_group[i]];
  op->ndiag_groups = 0;
  for (int g = 0; g < d->nm; ++g) op->ndiag_groups += group_diag[g] != KR_NO_DIAG;

  const long long nent = inst_ptr[d->nmf];
  std::vector<int> ent_inst(nent);
  for (int i = 0; i < d->nmf; ++i)
    for (long long e = inst_ptr[i]; e < inst_ptr[i + 1]; ++e) ent_inst[e] = i;

  // ---- algorithmic work --------------------------------------------------
  std::vector<long long> group_nnz(d->nm, 0);
  for (int g = 0; g < d->nm; ++g) {
    const long long ne = (long long)d->m_rows[g] * d->m_width[g];
    for (long long e = 0; e < ne; ++e) {
      bool nz = false;
      for (int c = 0; c < d->m_ncart[g] && !nz; ++c) {
        const double* v = d->m_val + 2 * (d->m_val_off[g] + c * ne + e);
        nz = v[0] != 0.0 || v[1] != 0.0;
      }
      group_nnz[g] += nz;
    }
  }
  double fma = 0.0, kbytes = 0.0, mbytes = 0.0;
  for (int t = 0; t < d->nterm; ++t) {
    const int s1 = d->t_out[t], s2 = d->t_in[t], kb = d->t_k[t], g = d->mf_group[d->t_mf[t]];
    const double nk1 = d->out_dk[s1], nk2 = d->in_dk[s2], dm1 = d->out_dm[s1];
    const double kf = d->k_type[kb] == KR_K_COMPLEX ? 4.0 : 2.0;
    fma += 4.0 * group_nnz[g] * nk2 + kf * dm1 * nk1 * nk2;
  }
  for (int b = 0; b < d->nk; ++b) kbytes += 8.0 * d->k_rows[b] * d->k_cols[b] * (d->k_type[b] == KR_K_COMPLEX ? 2 : 1);
  for (int g = 0; g < d->nm; ++g) mbytes += 20.0 * group_nnz[g];
  op->fma_per_matvec = fma;
  op->bytes_per_matvec = 16.0 * (d->dim_in + d->dim_out) + kbytes + mbytes;

  // ---- row tasks ----------------------------------------------------------
  // Rows per task from thread occupancy (pick_task_rows); then the slabs whose
  // tasks would cost more than half of the mean work per CTA are cut finer
  // (down to one output per thread), so that the dynamic queue, handed out
  // most expensive first, ends evenly across the CTAs.
  std::vector<int> task_slab, task_row0, task_nrows;
  std::vector<double> task_cost;
  int zmax = 1;
  auto task_cost_of = [&](int s, int nr) {
    const int nk1 = d->out_dk[s];
    const int q = (nr * nk1 + KR_THREADS - 1) / KR_THREADS;
    double cost = 200.0;
    for (int t : by_out[s]) {
      const int nk2 = d->in_dk[d->t_in[t]];
      const int g = d->mf_group[d->t_mf[t]];
      const double kf = d->k_type[d->t_k[t]] == KR_K_COMPLEX ? 4.0 : 2.0;
      const int qz = (nr * nk2 + KR_THREADS - 1) / KR_THREADS;
      cost += 4.0 * qz * d->m_width[g] + kf * q * nk2 + 60.0;
    }
    return cost;
  };
  std::vector<int> rows_per_task(d->nslab_out);
  double total = 0.0;
  for (int s = 0; s < d->nslab_out; ++s) {
    const int dm1 = d->out_dm[s];
    rows_per_task[s] = pick_task_rows(d->out_dk[s], dm1);
    for (int i0 = 0; i0 < dm1; i0 += rows_per_task[s]) total += task_cost_of(s, std::min(rows_per_task[s], dm1 - i0));
  }
  const double cap = 0.5 * total / (2.0 * ctx->nsm);  // half the mean work of one of 2 CTAs per SM
  for (int s = 0; s < d->nslab_out; ++s) {
    const int nk1 = d->out_dk[s], dm1 = d->out_dm[s];
    int R = rows_per_task[s];
    const int rmin = std::max(1, std::min(R, KR_THREADS / nk1));  // one output per thread
    while (R > rmin && task_cost_of(s, R) > cap) R = std::max(rmin, R / 2);
    int maxnk2 = 1;
    for (int t : by_out[s]) maxnk2 = std::max(maxnk2, d->in_dk[d->t_in[t]]);
    for (int i0 = 0; i0 < dm1; i0 += R) {
      const int nr = std::min(R, dm1 - i0);
      task_slab.push_back(s);
      task_row0.push_back(i0);
      task_nrows.push_back(nr);
      task_cost.push_back(task_cost_of(s, nr));
      zmax = std::max(zmax, nr * maxnk2);
    }
  }
  const int ntask = (int)task_slab.size();
  op->smem = (size_t)2 * zmax * sizeof(double2);
  if (op->smem > 100 * 1024) {
    kr_op_destroy(op);
    return set_err(ctx, KR_ERR_UNSUPPORTED, "Z staging buffer exceeds shared memory");
  }
  if (ensure_step_smem(op->smem) != cudaSuccess) {
    kr_op_destroy(op);
    return set_err(ctx, KR_ERR_CUDA, "cannot raise the dynamic shared memory of the step kernels");
  }
  int occ = 0;
  cudaError_t ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kr_step_kernel<false>, KR_THREADS, op->smem);
  int occ_df = 0;
  if (ce == cudaSuccess)
    ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_df, kr_step_kernel<true>, KR_THREADS, op->smem);
  if (ce != cudaSuccess || occ < 1 || occ_df < 1) {
    kr_op_destroy(op);
    return set_err(ctx, KR_ERR_CUDA, "kr_step_kernel cannot be resident");
  }
  // two CTAs per SM for FP64 products; three with double-float products (fewer
  // registers: more warps to hide the latency of the barrier-bound step)
  int grid = ctx->nsm * std::min(occ, 2);
  grid = std::max(1, std::min(grid, ntask));
  op->grid = grid;
  op->grid_df = std::max(1, std::min(ctx->nsm * std::min(occ_df, 3), ntask));
  const int grid_max = std::max(op->grid, op->grid_df);

  // tasks are handed out dynamically, most expensive first
  std::vector<int> task_order(ntask);
  std::iota(task_order.begin(), task_order.end(), 0);
  std::stable_sort(task_order.begin(), task_order.end(),
                   [&](int x, int y) { return task_cost[x] > task_cost[y]; });

  // ---- tiles of the tensor-core batched mat-vec ---------------------------
  // per output slab: KP = largest input n_k of its terms padded to 8 (the MMA K),
  // R = 64 / KP rows per tile; heaviest slabs first
  std::vector<int> tc_task;
  std::vector<int> slab_kp(d->nslab_out, 0);  // KP of each output slab's tiles
  {
    std::vector<int> ts, ti, tn, tk;
    std::vector<double> tcost;
    for (int s = 0; s < d->nslab_out; ++s) {
      int maxnk2 = 1;
      for (int t : by_out[s]) maxnk2 = std::max(maxnk2, d->in_dk[d->t_in[t]]);
      if (maxnk2 > 32 || d->out_dk[s] > 32) {
        tc_task.clear();
        ts.clear();
        break;  // outside the batched mat-vec's shapes (kr_batch_create rejects such operators)
      }
      // an output slab wider than 16 columns takes tiles of at most 4 rows
      // (KP >= 16), so that its accumulators (2 R NP TMEM columns, NP = 32)
      // leave half of the tensor memory to the A tiles of the TMEM form
      const int kp = (maxnk2 <= 8 && d->out_dk[s] <= 16) ? 8 : maxnk2 <= 16 ? 16 : 32;
      slab_kp[s] = kp;
      const int R = 64 / kp, dm1 = d->out_dm[s];
      for (int i0 = 0; i0 < dm1; i0 += R) {
        ts.push_back(s);
        ti.push_back(i0);
        tn.push_back(std::min(R, dm1 - i0));
        tk.push_back(kp);
        tcost.push_back((double)by_out[s].size() * kp * std::min(R, dm1 - i0));
      }
    }
    const int n = (int)ts.size();
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    // classes of KP together (8, 16, 32: one persistent launch per class), heaviest first
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return tk[x] != tk[y] ? tk[x] < tk[y] : tcost[x] > tcost[y]; });
    for (int c = 0; c < 3; ++c) {
      const int kpc = 8 << c;
      op->tc_class[c] = (int)(std::lower_bound(ord.begin(), ord.end(), kpc,
                                               [&](int x, int kv) { return tk[x] < kv; }) - ord.begin());
    }
    op->tc_class[3] = n;
    tc_task.resize((size_t)4 * n);
    for (int q = 0; q < n; ++q) {
      tc_task[q] = ts[ord[q]];
      tc_task[n + q] = ti[ord[q]];
      tc_task[2 * n + q] = tn[ord[q]];
      tc_task[3 * n + q] = tk[ord[q]];
    }
    op->tc_ntask = n;
  }

  // ---- tiles of the register-tiled FP32 batched mat-vec --------------------
  // per output slab: NKP = the largest n_k of the slab and its terms' input
  // slabs, padded to 8, 16 or 32; tiles of 4 * RW rows (RW = 2, or 1 at
  // NKP = 32: one row of outputs per thread and warp); heaviest tiles first
  std::vector<int> zr_task;
  {
    std::vector<int> ts, ti, tn, tk;
    std::vector<double> tcost;
    bool fits = true;
    for (int s = 0; s < d->nslab_out && fits; ++s) {
      int nkmax = d->out_dk[s];
      double terms_nk = 0;
      for (int t : by_out[s]) {
        nkmax = std::max(nkmax, d->in_dk[d->t_in[t]]);
        terms_nk += d->in_dk[d->t_in[t]];
      }
      if (nkmax > 32) {
        fits = false;
        break;
      }
      const int nkp = nkmax <= 8 ? 8 : nkmax <= 16 ? 16 : 32;
      const int rows = 4 * (nkp == 32 ? 1 : 2);
      for (int i0 = 0; i0 < d->out_dm[s]; i0 += rows) {
        const int nr = std::min(rows, d->out_dm[s] - i0);
        ts.push_back(s);
        ti.push_back(i0);
        tn.push_back(nr);
        tk.push_back(nkp);
        tcost.push_back((double)nr * d->out_dk[s] * (terms_nk + 1));
      }
    }
    const int n = fits ? (int)ts.size() : 0;
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    // classes of NKP together (one launch per class), heaviest tiles first
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return tk[x] != tk[y] ? tk[x] < tk[y] : tcost[x] > tcost[y]; });
    for (int c = 0; c < 3; ++c) {
      const int kpc = 8 << c;
      op->zr_class[c] = (int)(std::lower_bound(ord.begin(), ord.end(), kpc,
                                               [&](int x, int kv) { return tk[x] < kv; }) - ord.begin());
    }
    op->zr_class[3] = n;
    zr_task.resize((size_t)4 * n);
    for (int q = 0; q < n; ++q) {
      zr_task[q] = ts[ord[q]];
      zr_task[n + q] = ti[ord[q]];
      zr_task[2 * n + q] = tn[ord[q]];
      zr_task[3 * n + q] = tk[ord[q]];
    }
    op->zr_ntask = n;
  }

  // K blocks transposed: KT[b][a] (complex blocks keep (re, im) pairs)
  std::vector<double> k_t(d->k_data, d->k_data + d->k_data_len);
  for (int b = 0; b < d->nk; ++b) {
    const int r = d->k_rows[b], c = d->k_cols[b];
    const int words = d->k_type[b] == KR_K_COMPLEX ? 2 : 1;
    const double* src = d->k_data + d->k_off[b];
    double* dst = k_t.data() + d->k_off[b];
    for (int a = 0; a < r; ++a)
      for (int bb = 0; bb < c; ++bb)
        for (int w = 0; w < words; ++w) dst[(bb * r + a) * words + w] = src[(a * c + bb) * words + w];
  }
  // value class of every (group, cart) of the M factors
  std::vector<signed char> m_ctype((size_t)std::max(1, d->nm) * KR_MAXCART, 3);
  for (int g = 0; g < d->nm; ++g) {
    const long long ne = (long long)d->m_rows[g] * d->m_width[g];
    for (int c = 0; c < d->m_ncart[g]; ++c) {
      bool any_re = false, any_im = false;
      for (long long e = 0; e < ne; ++e) {
        const double* v = d->m_val + 2 * (d->m_val_off[g] + c * ne + e);
        any_re |= v[0] != 0.0;
        any_im |= v[1] != 0.0;
      }
      m_ctype[g * KR_MAXCART + c] = (!any_re && !any_im) ? 3 : (!any_im ? 1 : (!any_re ? 2 : 0));
    }
  }

  // ---- uploads --------------------------------------------------------------
  DevOp& D = op->dev;
  int rc = KR_OK;
#define UP(host, count, dst) \
  if ((rc = upload(op, host, count, dst)) != KR_OK) { kr_op_destroy(op); return rc; }
  D.nslab_out = d->nslab_out;
  D.nslab_in = d->nslab_in;
  D.dim_out = d->dim_out;
  D.dim_in = d->dim_in;
  int *p_i;
  long long* p_l;
  UP(d->out_dm, d->nslab_out, &p_i); D.out_dm = p_i;
  UP(d->out_dk, d->nslab_out, &p_i); D.out_dk = p_i;
  UP((const long long*)d->out_off, d->nslab_out, &p_l); D.out_off = p_l;
  UP(d->in_dm, d->nslab_in, &p_i); D.in_dm = p_i;
  UP(d->in_dk, d->nslab_in, &p_i); D.in_dk = p_i;
  UP((const long long*)d->in_off, d->nslab_in, &p_l); D.in_off = p_l;
  UP(out_stride.data(), d->nslab_out, &p_i); D.out_stride = p_i;
  UP(in_stride.data(), d->nslab_in, &p_i); D.in_stride = p_i;
  UP((const long long*)d->k_off, d->nk, &p_l); D.k_off = p_l;
  UP(d->k_rows, d->nk, &p_i); D.k_rows = p_i;
  UP(d->k_cols, d->nk, &p_i); D.k_cols = p_i;
  UP(d->k_type, d->nk, &p_i); D.k_type = p_i;
  double* p_d;
  UP(k_t.data(), k_t.size(), &p_d); D.k_data = p_d;
  {
    std::vector<float> k32(k_t.begin(), k_t.end());
    float* p_f;
    UP(k32.data(), k32.size(), &p_f); D.k_f32 = p_f;
    for (size_t i = 0; i < k32.size(); ++i) k32[i] = (float)(k_t[i] - (double)k32[i]);  // the double-float lo part
    UP(k32.data(), k32.size(), &p_f); D.k_lo = p_f;
  }
  UP((const long long*)inst_ptr.data(), d->nmf, &p_l); D.mf_off = p_l;
  UP((const long long*)mf_col_off.data(), d->nmf, &p_l); D.mf_col_off = p_l;
  UP(mf_width.data(), d->nmf, &p_i); D.mf_width = p_i;
  UP(mf_diag.data(), d->nmf, &p_i); D.mf_diag = p_i;
  UP(d->m_col, d->m_col_len, &p_i); D.m_col = p_i;
  double2* p_c;
  UP((const double2*)nullptr, nent, &p_c); D.mf_val = p_c;
  {
    float2* p_f2;
    UP((const float2*)nullptr, nent, &p_f2); D.mf_f32 = p_f2;
    UP((const float2*)nullptr, nent, &p_f2); D.mf_lo = p_f2;
  }
  UP(term_ptr.data(), term_ptr.size(), &p_i); D.term_ptr = p_i;
  UP(t_in.data(), t_in.size(), &p_i); D.t_in = p_i;
  UP(t_k.data(), t_k.size(), &p_i); D.t_k = p_i;
  UP(t_mf.data(), t_mf.size(), &p_i); D.t_mf = p_i;
  UP(task_slab.data(), ntask, &p_i); D.task_slab = p_i;
  UP(task_row0.data(), ntask, &p_i); D.task_row0 = p_i;
  UP(task_nrows.data(), ntask, &p_i); D.task_nrows = p_i;
  UP(task_order.data(), task_order.size(), &p_i); D.task_order = p_i;
  if (op->tc_ntask > 0) {
    UP(tc_task.data(), tc_task.size(), &p_i);
    op->tc_task = p_i;
    // B blocks of the terms of the persistent tiles (KP = 8, 16, 32), 6 NP KP floats each
    const int nterm = (int)t_in.size();
    std::vector<long long> prm((size_t)6 * std::max(1, nterm), 0), boff(std::max(1, nterm), 0);
    long long tot = 0;
    for (int s = 0; s < d->nslab_out; ++s) {
      const int kp = slab_kp[s];
      if (kp != 8 && kp != 16 && kp != 32) continue;
      const int np = d->out_dk[s] <= 16 ? 16 : 32;
      for (size_t k = 0; k < by_out[s].size(); ++k) {
        const int t = by_out[s][k], j = term_ptr[s] + (int)k;  // original and device term index
        const int kb = d->t_k[t];
        prm[j] = d->k_off[kb];
        prm[nterm + j] = d->k_type[kb];
        prm[2 * nterm + j] = d->out_dk[s];
        prm[3 * nterm + j] = d->in_dk[d->t_in[t]];
        prm[4 * nterm + j] = kp;
        prm[5 * nterm + j] = tot;
        boff[j] = tot;
        tot += 6LL * np * kp;
      }
    }
    if (tot > 0) {
      long long* p_prm;
      float* p_b;
      UP(prm.data(), prm.size(), &p_prm);
      UP(boff.data(), boff.size(), &p_l); op->tc_boff = p_l;
      UP((const float*)nullptr, (size_t)tot, &p_b); op->tc_b = p_b;
      if ((rc = kb_build_tc_b(ctx, D.k_f32, p_prm, nterm, op->tc_b)) != KR_OK) {
        kr_op_destroy(op);
        return rc;
      }
    }
  }
  if (op->zr_ntask > 0) {
    UP(zr_task.data(), zr_task.size(), &p_i);
    op->zr_task = p_i;
  }
  D.ntask = ntask;
  unsigned* p_u;
  UP((const unsigned*)nullptr, (size_t)KR_MATVEC_MAXVEC, &p_u); op->mv_counters = p_u;
  UP((const int*)nullptr, (size_t)std::max(1, d->nmf), &p_i); D.mf_type = p_i;
  UP((const int*)nullptr, (size_t)2 * std::max(1, d->nmf), &p_i); D.mf_band = p_i;
  D.zmax = zmax;

  DevField& F = op->field;
  F.nent = nent;
  F.mf_band = const_cast<int*>(D.mf_band);
  UP(ent_inst.data(), nent, &p_i); F.ent_inst = p_i;
  F.inst_ptr = D.mf_off;
  UP(d->mf_group, d->nmf, &p_i); F.mf_group = p_i;
  UP(d->mf_part, d->nmf, &p_i); F.mf_part = p_i;
  UP((const long long*)d->m_val_off, d->nm, &p_l); F.m_val_off = p_l;
  UP(d->m_ncart, d->nm, &p_i); F.m_ncart = p_i;
  UP(d->m_rows, d->nm, &p_i); F.m_rows = p_i;
  UP(d->m_width, d->nm, &p_i); F.m_width = p_i;
  UP((const double2*)d->m_val, d->m_val_len / 2, &p_c); F.m_val = p_c;
  F.mf_val = D.mf_val;
  F.mf_f32 = D.mf_f32;
  F.mf_lo = D.mf_lo;
  F.nmf = d->nmf;
  F.mf_type = const_cast<int*>(D.mf_type);
  signed char* p_s;
  UP(m_ctype.data(), m_ctype.size(), &p_s); F.m_ctype = p_s;
  if (d->npart > KR_PART_INLINE) {  // one block: coef, scale, thresh (see kr_set_field)
    UP((const double*)nullptr, (size_t)d->npart * (KR_MAXCART * 2 + 2 + 1), &p_d);
    op->fc_coef = reinterpret_cast<double2*>(p_d);
    op->fc_scale = op->fc_coef + (size_t)d->npart * KR_MAXCART;
    op->fc_thresh = reinterpret_cast<double*>(op->fc_scale + d->npart);
  }

  // ---- step scratch (sized once: kr_step allocates nothing) -----------------
  if (op->square) {
    const long long n = d->dim_out;
    UP((const double2*)nullptr, (size_t)n * d->maxorder, &p_c); op->V = p_c;
    UP((const double2*)nullptr, (size_t)n, &p_c); op->Wb0 = p_c;
    UP((const double2*)nullptr, (size_t)n, &p_c); op->Wb1 = p_c;
    UP((const double2*)nullptr, (size_t)n, &p_c); op->w = p_c;
    UP((const double2*)nullptr, (size_t)n, &p_c); op->ub0 = p_c;
    UP((const double2*)nullptr, (size_t)n, &p_c); op->ub1 = p_c;
    UP((const double2*)nullptr, (size_t)grid_max, &p_c); op->part_a = p_c;
    UP((const double2*)nullptr, (size_t)ntask, &p_c); op->task_alpha = p_c;
    UP((const unsigned*)nullptr, (size_t)d->maxorder + 2, &p_u); op->counters = p_u;
    UP((const double*)nullptr, (size_t)grid_max, &p_d); op->part_b = p_d;
    UP((const double*)nullptr, (size_t)grid_max, &p_d); op->part_c = p_d;
    UP((const double2*)nullptr, (size_t)d->maxorder + 1, &p_c); op->alpha = p_c;
    UP((const double*)nullptr, (size_t)d->maxorder + 1, &p_d); op->beta = p_d;
    UP((const unsigned*)nullptr, 2, &p_u); op->bar = p_u;
    UP((const int*)nullptr, 2, &p_i); op->status = p_i;
    float4* p_f4;
    UP((const float4*)nullptr, (size_t)n, &p_f4); op->xdf = p_f4;
  }
#undef UP
  KR_CUDA(ctx, cudaDeviceSynchronize());
  *out = op;
  return KR_OK;
}

namespace {
// the field launch of one step: band bounds reset, then MF = field products
template <class Coef>
int launch_field(kr_op* op, const Coef& c, cudaStream_t st) {
  KR_CUDA(op->ctx, cudaMemsetAsync(op->field.mf_band, 0xFF, sizeof(int) * 2 * std::max(1, op->field.nmf), st));
  const int threads = 256;
  const long long work = std::max<long long>(op->field.nent, op->field.nmf);
  const int blocks = (int)std::max<long long>(1, std::min<long long>((work + threads - 1) / threads, 4LL * op->ctx->nsm));
  kr_field_kernel<<<blocks, threads, 0, st>>>(op->field, c);
  op->launches++;
  KR_CUDA(op->ctx, cudaGetLastError());
  return KR_OK;
}
}  // namespace

extern "C" int kr_set_field(kr_op* op, const double* coef, const double* scale, const double* thresh, void* stream) {
  if (!op || !coef || !scale || !thresh) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_set_field: NULL argument");
  if (op->field.nent == 0 && op->field.nmf == 0) return KR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (op->npart <= KR_PART_INLINE) {
    FieldCoef c;
    std::memset(&c, 0, sizeof(c));
    c.npart = op->npart;
    for (int p = 0; p < op->npart; ++p) {
      for (int ci = 0; ci < KR_MAXCART; ++ci)
        c.coef[p][ci] = make_double2(coef[2 * (p * KR_MAXCART + ci)], coef[2 * (p * KR_MAXCART + ci) + 1]);
      c.scale[p] = make_double2(scale[2 * p], scale[2 * p + 1]);
      c.thresh[p] = thresh[p];
    }
    return launch_field(op, c, st);
  } else {
    // stage coef [npart][9] complex, scale [npart] complex, thresh [npart] into
    // one host block, then one copy to the operator's device buffers (the
    // copy completes before the host block is written again: the staging
    // vector is reused only after the stream has passed it)
    const size_t nc = (size_t)op->npart * KR_MAXCART * 2, ns = (size_t)op->npart * 2, nt = op->npart;
    KR_CUDA(op->ctx, cudaStreamSynchronize(st));
    op->fc_host.assign(coef, coef + nc);
    op->fc_host.insert(op->fc_host.end(), scale, scale + ns);
    op->fc_host.insert(op->fc_host.end(), thresh, thresh + nt);
    KR_CUDA(op->ctx, cudaMemcpyAsync(op->fc_coef, op->fc_host.data(), sizeof(double) * op->fc_host.size(),
                                     cudaMemcpyHostToDevice, st));
    FieldCoefDev c{op->fc_coef, op->fc_scale, op->fc_thresh};
    return launch_field(op, c, st);
  }
}

extern "C" int kr_set_field_schedule(kr_op* op, int32_t nsteps, const double* coef, const double* scale,
                                     const double* thresh, void* stream) {
  if (!op || nsteps <= 0 || !coef || !scale || !thresh)
    return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_set_field_schedule: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (op->fs_buf) {  // the old schedule may still be read by queued field launches
    KR_CUDA(op->ctx, cudaDeviceSynchronize());
    KR_CUDA(op->ctx, cudaFree(op->fs_buf));
    op->fs_buf = nullptr;
    op->fs_nsteps = 0;
  }
  const size_t np = (size_t)op->npart, ns = (size_t)nsteps * np;
  if (ns > 0) {
    const size_t bc = sizeof(double2) * ns * KR_MAXCART, bs = sizeof(double2) * ns, bt = sizeof(double) * ns;
    KR_CUDA(op->ctx, cudaMalloc(&op->fs_buf, bc + bs + bt));
    op->fs_coef = reinterpret_cast<double2*>(op->fs_buf);
    op->fs_scale = op->fs_coef + ns * KR_MAXCART;
    op->fs_thresh = reinterpret_cast<double*>(op->fs_scale + ns);
    KR_CUDA(op->ctx, cudaMemcpyAsync(op->fs_coef, coef, bc, cudaMemcpyHostToDevice, st));
    KR_CUDA(op->ctx, cudaMemcpyAsync(op->fs_scale, scale, bs, cudaMemcpyHostToDevice, st));
    KR_CUDA(op->ctx, cudaMemcpyAsync(op->fs_thresh, thresh, bt, cudaMemcpyHostToDevice, st));
    KR_CUDA(op->ctx, cudaStreamSynchronize(st));
  }
  op->fs_nsteps = nsteps;
  return KR_OK;
}

extern "C" int kr_set_field_step(kr_op* op, int32_t step, void* stream) {
  if (!op) return set_err(nullptr, KR_ERR_ARG, "kr_set_field_step: NULL operator");
  if (step < 0 || step >= op->fs_nsteps)
    return set_err(op->ctx, KR_ERR_ARG, "kr_set_field_step: step " + std::to_string(step) + " outside the schedule of " +
                                            std::to_string(op->fs_nsteps) + " steps");
  if (op->field.nent == 0 && op->field.nmf == 0) return KR_OK;
  const size_t np = (size_t)op->npart, s = (size_t)step;
  FieldCoefDev c{op->fs_coef + s * np * KR_MAXCART, op->fs_scale + s * np, op->fs_thresh + s * np};
  return launch_field(op, c, (cudaStream_t)stream);
}

extern "C" int kr_matvec(kr_op* op, const void* x, void* y, int64_t nvec, void* stream) {
  if (!op || !x || !y || nvec < 0) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_matvec: bad argument");
  if (op->split) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_matvec: operator with column chunks (batched path only)");
  if (nvec == 0) return KR_OK;
  if (nvec > KR_MATVEC_MAXVEC) return set_err(op->ctx, KR_ERR_ARG, "kr_matvec: nvec above 65535");
  KR_CUDA(op->ctx, cudaMemsetAsync(op->mv_counters, 0, sizeof(unsigned) * nvec, (cudaStream_t)stream));
  dim3 g(op->grid, (unsigned)nvec);
  KR_CUDA(op->ctx, ensure_step_smem(op->smem));
  kr_matvec_kernel<<<g, KR_THREADS, op->smem, (cudaStream_t)stream>>>(op->dev, (const double2*)x, (double2*)y,
                                                                      op->mv_counters);
  op->launches++;
  KR_CUDA(op->ctx, cudaGetLastError());
  return KR_OK;
}

extern "C" int kr_step(kr_op* op, void* states, int64_t nvec, const void* phase, double fac_re, double fac_im,
                       double tol, uint32_t flags, int32_t* korder, void* stream) {
  if (!op || !states || nvec < 0) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_step: bad argument");
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_step: operator is not square (bra basis != ket basis)");
  if (op->split) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_step: operator with column chunks (batched path only)");
  if (nvec == 0) return KR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = op->dev.dim_out;
  if (flags & KR_STEP_SKIP_KRYLOV) {
    if (phase) {
      const int blocks = (int)std::min<long long>((n * nvec + 255) / 256, 8LL * op->ctx->nsm);
      kr_phase2_kernel<<<blocks, 256, 0, st>>>((double2*)states, (const double2*)phase, n, nvec);
      op->launches++;
      KR_CUDA(op->ctx, cudaGetLastError());
    }
    if (korder)
      for (int64_t v = 0; v < nvec; ++v) korder[v] = 0;
    return KR_OK;
  }
  StepArgs a;
  a.op = op->dev;
  a.phase = (const double2*)phase;
  a.V = op->V;
  a.Wb[0] = op->Wb0;
  a.Wb[1] = op->Wb1;
  a.w = op->w;
  a.ub[0] = op->ub0;
  a.ub[1] = op->ub1;
  a.part_a = op->part_a;
  a.task_alpha = op->task_alpha;
  a.counters = op->counters;
  a.part_b = op->part_b;
  a.part_c = op->part_c;
  a.alpha = op->alpha;
  a.beta = op->beta;
  a.bar_count = op->bar;
  a.bar_gen = op->bar + 1;
  a.status = op->status;
  a.kout = op->status + 1;
  a.xdf = op->xdf;
  a.fac = make_double2(fac_re, fac_im);
  a.tol = tol;
  a.maxorder = op->maxorder;
  a.dim = n;
  for (int64_t v = 0; v < nvec; ++v) {
    a.state = (double2*)states + v * n;
    KR_CUDA(op->ctx, cudaMemsetAsync(op->bar, 0, sizeof(unsigned), st));  // arrival count only
    void* args[] = {&a};
    KR_CUDA(op->ctx, ensure_step_smem(op->smem));
    KR_CUDA(op->ctx, cudaLaunchCooperativeKernel(step_kernel(op), dim3(step_grid(op)), dim3(KR_THREADS), args,
                                                 op->smem, st));
    op->launches++;
    if (korder) {
      int hs[2] = {0, 0};
      KR_CUDA(op->ctx, cudaMemcpyAsync(hs, op->status, sizeof(hs), cudaMemcpyDeviceToHost, st));
      KR_CUDA(op->ctx, cudaStreamSynchronize(st));
      korder[v] = hs[1];
      if (hs[0] != 0) {
        cudaMemsetAsync(op->status, 0, sizeof(int), st);
        cudaStreamSynchronize(st);
        if (hs[0] == KR_ERR_MAXORDER)
          return set_err(op->ctx, KR_ERR_MAXORDER,
                         "Lanczos reached maximum order of '" + std::to_string(op->maxorder) + "' without convergence");
        return set_err(op->ctx, hs[0], "device-side wait gave up (grid barrier timeout)");
      }
    }
  }
  return KR_OK;
}

extern "C" int kr_sync_status(kr_op* op, void* stream) {
  if (!op) return set_err(nullptr, KR_ERR_ARG, "kr_sync_status: NULL op");
  cudaStream_t st = (cudaStream_t)stream;
  KR_CUDA(op->ctx, cudaStreamSynchronize(st));
  KR_CUDA(op->ctx, cudaGetLastError());
  if (!op->status) return KR_OK;
  int hs = 0;
  KR_CUDA(op->ctx, cudaMemcpy(&hs, op->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (hs != 0) {
    cudaMemset(op->status, 0, sizeof(int));
    if (hs == KR_ERR_MAXORDER)
      return set_err(op->ctx, KR_ERR_MAXORDER,
                     "Lanczos reached maximum order of '" + std::to_string(op->maxorder) + "' without convergence");
    return set_err(op->ctx, hs, "device-side wait gave up (grid barrier timeout)");
  }
  return KR_OK;
}

extern "C" int64_t kr_op_launch_count(const kr_op* op) { return op ? op->launches : -1; }

extern "C" int kr_op_work(const kr_op* op, double* fma_per_matvec, double* bytes_per_matvec) {
  if (!op) return KR_ERR_ARG;
  if (fma_per_matvec) *fma_per_matvec = op->fma_per_matvec;
  if (bytes_per_matvec) *bytes_per_matvec = op->bytes_per_matvec;
  return KR_OK;
}

// ===========================================================================
// measurement helper: FP64 FMA throughput of this device (8 independent
// chains per thread; every thread writes one double)
// ===========================================================================
__global__ void kr_fp64_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void kr_fp32_probe_kernel(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

extern "C" int kr_probe_fp32(kr_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return set_err(ctx, KR_ERR_ARG, "kr_probe_fp32: NULL argument");
  KR_DEVICE_SCOPE(ctx, ctx->device);
  const int blocks = ctx->nsm * 8, threads = 256, iters = 65536;
  float* out = nullptr;
  KR_CUDA(ctx, cudaMalloc(&out, sizeof(float) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kr_fp32_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
  cudaEventRecord(e0);
  for (int r = 0; r < 5; ++r) kr_fp32_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return set_err(ctx, KR_ERR_CUDA, cudaGetErrorString(e));
  *tflops = 5.0 * 2.0 * 8.0 * iters * double(blocks) * threads / (ms * 1e-3) / 1e12;
  return KR_OK;
}

extern "C" int kr_probe_fp64(kr_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return set_err(ctx, KR_ERR_ARG, "kr_probe_fp64: NULL argument");
  KR_DEVICE_SCOPE(ctx, ctx->device);
  const int blocks = ctx->nsm * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  KR_CUDA(ctx, cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kr_fp64_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e0);
  for (int r = 0; r < 5; ++r) kr_fp64_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return set_err(ctx, KR_ERR_CUDA, cudaGetErrorString(e));
  *tflops = 5.0 * 2.0 * 8.0 * iters * double(blocks) * threads / (ms * 1e-3) / 1e12;
  return KR_OK;
}

// The grid barrier of the step kernels with a CTA that never arrives (CTA 1
// returns at once, as a rank that never joins): CTA 0's bounded wait gives up
// after KR_BARRIER_TIMEOUT_NS, records KR_ERR_TIMEOUT in status and returns.
// out[0]: 1 if the barrier reported failure, out[1]: ns CTA 0 waited.
__global__ void kr_wait_probe_kernel(unsigned* bar, int* status, unsigned long long* out) {
  if (blockIdx.x != 0) return;
  const unsigned long long t0 = globaltimer_ns();
  const bool ok = grid_barrier(bar, bar + 1, status, KR_ERR_TIMEOUT);
  if (threadIdx.x == 0) {
    out[0] = ok ? 0ull : 1ull;
    out[1] = globaltimer_ns() - t0;
  }
}

extern "C" int kr_probe_wait(kr_ctx* ctx, int32_t* status, double* waited_s) {
  if (!ctx || !status || !waited_s) return set_err(ctx, KR_ERR_ARG, "kr_probe_wait: NULL argument");
  KR_DEVICE_SCOPE(ctx, ctx->device);
  // bar[2] (count, generation), status, pad, out[2]
  void* buf = nullptr;
  KR_CUDA(ctx, cudaMalloc(&buf, 32));
  cudaError_t e = cudaMemset(buf, 0, 32);
  unsigned* bar = static_cast<unsigned*>(buf);
  int* st = reinterpret_cast<int*>(bar + 2);
  unsigned long long* out = reinterpret_cast<unsigned long long*>(static_cast<char*>(buf) + 16);
  if (e == cudaSuccess) {
    kr_wait_probe_kernel<<<2, 32>>>(bar, st, out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int h_st = 0;
  unsigned long long h_out[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(&h_st, st, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(h_out, out, sizeof(h_out), cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return set_err(ctx, KR_ERR_CUDA, std::string("kr_probe_wait: ") + cudaGetErrorString(e));
  *status = h_out[0] ? h_st : KR_OK;
  *waited_s = 1e-9 * (double)h_out[1];
  return KR_OK;
}

// ===========================================================================
// Allocation-free step: kr_step with its Krylov workspace in a fixed,
// file-scope device array instead of the workspace kr_op_create allocated.
// For callers that must not allocate device memory when they step: code that
// records the step into a CUDA graph or runs inside a framework that owns all
// device memory through its own pool. Every GPU that loads this library holds
// the array (KR_STATIC_SCRATCH_BYTES) until the process exits.
// ===========================================================================
#define KR_STATIC_SCRATCH_BYTES (64ull << 20)  // 64 MiB

static __device__ __align__(256) unsigned char g_kr_static_scratch[KR_STATIC_SCRATCH_BYTES];

namespace {
std::mutex g_static_mu;
void* g_static_addr[128] = {};  // device address of g_kr_static_scratch, per device

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }
}  // namespace

// copies a device-side error of the static scratch into the operator's status
// word (kept if that one already holds an error), so kr_sync_status sees it
__global__ void kr_status_merge_kernel(int* dst, const int* src) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && *dst == 0) *dst = *src;
}

extern "C" int kr_static_scratch_bytes(const kr_op* op, size_t* needed, size_t* capacity) {
  if (capacity) *capacity = KR_STATIC_SCRATCH_BYTES;
  if (!op) return KR_ERR_ARG;
  const size_t n = (size_t)op->dev.dim_out, m = (size_t)op->maxorder;
  size_t b = 0;
  b += round256(sizeof(double2) * n * m);                    // V
  b += 5 * round256(sizeof(double2) * n);                    // W[2], w, u[2]
  const size_t gm = (size_t)std::max(op->grid, op->grid_df);
  b += round256(sizeof(double2) * gm);                       // part_a
  b += 2 * round256(sizeof(double) * gm);                    // part_b, part_c
  b += round256(sizeof(double2) * op->dev.ntask);            // task_alpha
  b += round256(sizeof(unsigned) * (m + 2));                 // counters
  b += round256(sizeof(double2) * (m + 1));                  // alpha
  b += round256(sizeof(double) * (m + 1));                   // beta
  b += round256(sizeof(unsigned) * 2);                       // barrier
  b += round256(sizeof(int) * 2);                            // status, Krylov order
  b += round256(sizeof(float4) * n);                         // double-float copy of x
  if (needed) *needed = b;
  return KR_OK;
}

extern "C" int kr_step_static(kr_op* op, void* states, int64_t nvec, const void* phase, double fac_re,
                              double fac_im, double tol, uint32_t flags, int32_t* korder, void* stream) {
  if (!op || !states || nvec < 0) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_step_static: bad argument");
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_step_static: operator is not square");
  if (op->split) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_step_static: operator with column chunks");
  if (nvec == 0) return KR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = op->dev.dim_out;
  if (flags & KR_STEP_SKIP_KRYLOV) {  // no scratch needed
    if (phase) {
      const int blocks = (int)std::min<long long>((n * nvec + 255) / 256, 8LL * op->ctx->nsm);
      kr_phase2_kernel<<<blocks, 256, 0, st>>>((double2*)states, (const double2*)phase, n, nvec);
      op->launches++;
      KR_CUDA(op->ctx, cudaGetLastError());
    }
    if (korder)
      for (int64_t v = 0; v < nvec; ++v) korder[v] = 0;
    return KR_OK;
  }
  size_t need = 0;
  kr_static_scratch_bytes(op, &need, nullptr);
  if (need > KR_STATIC_SCRATCH_BYTES)
    return set_err(op->ctx, KR_ERR_ARG,
                   "kr_step_static: this operator needs " + std::to_string(need) +
                       " bytes of Krylov workspace (dim " + std::to_string(n) + ", maxorder " +
                       std::to_string(op->maxorder) + "), the static scratch holds " +
                       std::to_string((unsigned long long)KR_STATIC_SCRATCH_BYTES) + " bytes; use kr_step");
  const int dev = op->ctx->device;
  if (dev < 0 || dev >= 128) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_step_static: device index above 127");
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_addr[dev]) {
      // set-up, once per device, with that device current (the caller's
      // current device is given back when the scope ends)
      KR_DEVICE_SCOPE(op->ctx, dev);
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_kr_static_scratch);
      if (e != cudaSuccess || !p)
        return set_err(op->ctx, KR_ERR_CUDA,
                       std::string("kr_step_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      g_static_addr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_static_addr[dev]);
  }
  const size_t m = (size_t)op->maxorder;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += round256(bytes);
    return p;
  };
  StepArgs a;
  a.op = op->dev;
  a.phase = (const double2*)phase;
  a.V = (double2*)carve(sizeof(double2) * n * m);
  a.Wb[0] = (double2*)carve(sizeof(double2) * n);
  a.Wb[1] = (double2*)carve(sizeof(double2) * n);
  a.w = (double2*)carve(sizeof(double2) * n);
  a.ub[0] = (double2*)carve(sizeof(double2) * n);
  a.ub[1] = (double2*)carve(sizeof(double2) * n);
  const size_t gm = (size_t)std::max(op->grid, op->grid_df);
  a.part_a = (double2*)carve(sizeof(double2) * gm);
  a.part_b = (double*)carve(sizeof(double) * gm);
  a.part_c = (double*)carve(sizeof(double) * gm);
  a.task_alpha = (double2*)carve(sizeof(double2) * op->dev.ntask);
  a.counters = (unsigned*)carve(sizeof(unsigned) * (m + 2));
  a.alpha = (double2*)carve(sizeof(double2) * (m + 1));
  a.beta = (double*)carve(sizeof(double) * (m + 1));
  unsigned* bar = (unsigned*)carve(sizeof(unsigned) * 2);
  int* status = (int*)carve(sizeof(int) * 2);
  a.xdf = (float4*)carve(sizeof(float4) * n);
  a.bar_count = bar;
  a.bar_gen = bar + 1;
  a.status = status;
  a.kout = status + 1;
  a.fac = make_double2(fac_re, fac_im);
  a.tol = tol;
  a.maxorder = op->maxorder;
  a.dim = n;
  // the array keeps the previous call's contents: clear the arrival count and
  // the status word (task counters are cleared by the kernel itself), then
  // take over an error still pending in the operator's own status word, so
  // that, as kr_step does, the call skips its work until kr_sync_status has
  // reported that error
  KR_CUDA(op->ctx, cudaMemsetAsync(status, 0, 2 * sizeof(int), st));
  KR_CUDA(op->ctx, cudaMemcpyAsync(status, op->status, sizeof(int), cudaMemcpyDeviceToDevice, st));
  for (int64_t v = 0; v < nvec; ++v) {
    a.state = (double2*)states + v * n;
    KR_CUDA(op->ctx, cudaMemsetAsync(bar, 0, sizeof(unsigned), st));
    void* args[] = {&a};
    KR_CUDA(op->ctx, ensure_step_smem(op->smem));
    KR_CUDA(op->ctx, cudaLaunchCooperativeKernel(step_kernel(op), dim3(step_grid(op)), dim3(KR_THREADS), args,
                                                 op->smem, st));
    op->launches++;
    if (korder) {
      int hs[2] = {0, 0};
      KR_CUDA(op->ctx, cudaMemcpyAsync(hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st));
      KR_CUDA(op->ctx, cudaStreamSynchronize(st));
      korder[v] = hs[1];
      if (hs[0] != 0) {
        // reported here: the operator's status word no longer holds it (as kr_step)
        cudaMemsetAsync(op->status, 0, sizeof(int), st);
        cudaStreamSynchronize(st);
        if (hs[0] == KR_ERR_MAXORDER)
          return set_err(op->ctx, KR_ERR_MAXORDER,
                         "Lanczos reached maximum order of '" + std::to_string(op->maxorder) + "' without convergence");
        return set_err(op->ctx, hs[0], "device-side wait gave up (grid barrier timeout)");
      }
    }
  }
  if (!korder) {
    kr_status_merge_kernel<<<1, 32, 0, st>>>(op->status, status);
    op->launches++;
    KR_CUDA(op->ctx, cudaGetLastError());
  }
  return KR_OK;
}


// ===========================================================================
// segmented step (C ABI)
// ===========================================================================
struct kr_seg {
  kr_op* op = nullptr;
  int nseg = 0, nchunk = 0, grid = 1, grid32 = 1;  // cooperative grids: FP64, FP32 products
  std::vector<void*> allocs;
  int *slab_seg = nullptr, *chunk_seg = nullptr, *seg_chunk_ptr = nullptr, *seg_task_ptr = nullptr,
      *seg_tasks = nullptr;
  long long *chunk_e0 = nullptr, *chunk_e1 = nullptr;
  double2 *alpha = nullptr, *coef = nullptr;
  double* beta = nullptr;
  int *done = nullptr, *kout = nullptr, *ufin = nullptr, *nactive = nullptr;
  double *chunk_b = nullptr, *chunk_c = nullptr;
  long long launches = 0;
  bool f32 = false;  // mat-vec products in FP32 (kr_seg_set_precision)
};

extern "C" int kr_seg_set_precision(kr_seg* g, int32_t mode) {
  if (!g || (mode != KR_SEG_F64 && mode != KR_SEG_F32_MATVEC))
    return set_err(g ? g->op->ctx : nullptr, KR_ERR_ARG, "kr_seg_set_precision: bad argument");
  g->f32 = mode == KR_SEG_F32_MATVEC;
  return KR_OK;
}

extern "C" void kr_seg_destroy(kr_seg* g) {
  if (!g) return;
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  for (void* p : g->allocs) cudaFree(p);
  delete g;
}

namespace {
template <typename T>
int seg_upload(kr_seg* g, const T* host, size_t count, T** dev) {
  void* p = nullptr;
  const size_t bytes = sizeof(T) * std::max<size_t>(count, 1);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaSuccess) e = host ? cudaMemcpy(p, host, sizeof(T) * count, cudaMemcpyHostToDevice) : cudaMemset(p, 0, bytes);
  if (e != cudaSuccess) {
    if (p) cudaFree(p);
    return set_err(g->op->ctx, KR_ERR_CUDA, std::string("kr_seg_create: ") + cudaGetErrorString(e));
  }
  g->allocs.push_back(p);
  *dev = static_cast<T*>(p);
  return KR_OK;
}
}  // namespace

extern "C" int kr_seg_create(kr_op* op, int32_t nseg, const int32_t* slab_seg, kr_seg** out) {
  std::lock_guard<std::recursive_mutex> dlk(kr_device_mutex());
  if (!op || !slab_seg || !out || nseg <= 0) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_seg_create: bad argument");
  *out = nullptr;
  if (!op->square || op->split) return set_err(op->ctx, KR_ERR_ARG, "kr_seg_create: operator is not square or has column chunks");
  KR_DEVICE_SCOPE(op->ctx, op->ctx->device);
  const DevOp& D = op->dev;
  const int ns = D.nslab_out;
  std::vector<long long> off(ns);
  std::vector<int> dm(ns), dk(ns), term_ptr(ns + 1), t_in(1), tslab(std::max(1, D.ntask));
  KR_CUDA(op->ctx, cudaMemcpy(off.data(), D.out_off, sizeof(long long) * ns, cudaMemcpyDeviceToHost));
  KR_CUDA(op->ctx, cudaMemcpy(dm.data(), D.out_dm, sizeof(int) * ns, cudaMemcpyDeviceToHost));
  KR_CUDA(op->ctx, cudaMemcpy(dk.data(), D.out_dk, sizeof(int) * ns, cudaMemcpyDeviceToHost));
  KR_CUDA(op->ctx, cudaMemcpy(term_ptr.data(), D.term_ptr, sizeof(int) * (ns + 1), cudaMemcpyDeviceToHost));
  t_in.resize(std::max(1, term_ptr[ns]));
  if (term_ptr[ns] > 0)
    KR_CUDA(op->ctx, cudaMemcpy(t_in.data(), D.t_in, sizeof(int) * term_ptr[ns], cudaMemcpyDeviceToHost));
  if (D.ntask > 0) KR_CUDA(op->ctx, cudaMemcpy(tslab.data(), D.task_slab, sizeof(int) * D.ntask, cudaMemcpyDeviceToHost));
  // segments: contiguous, non-empty slab ranges in order; terms inside segments
  std::vector<long long> seg_off(nseg + 1, -1);
  for (int s = 0; s < ns; ++s) {
    const int g = slab_seg[s];
    if (g < 0 || g >= nseg || (s > 0 && g != slab_seg[s - 1] && g != slab_seg[s - 1] + 1) || (s == 0 && g != 0))
      return set_err(op->ctx, KR_ERR_ARG, "kr_seg_create: slab segments must be 0, 1, ... in slab order");
    if (seg_off[g] < 0) seg_off[g] = off[s];
    for (int t = term_ptr[s]; t < term_ptr[s + 1]; ++t)
      if (slab_seg[t_in[t]] != g) return set_err(op->ctx, KR_ERR_ARG, "kr_seg_create: a term couples two segments");
  }
  if (slab_seg[ns - 1] != nseg - 1) return set_err(op->ctx, KR_ERR_ARG, "kr_seg_create: a segment has no slab");
  seg_off[nseg] = D.dim_out;
  // chunks of at most 4096 elements inside segments; tasks grouped by segment
  std::vector<int> chunk_seg, seg_chunk_ptr(nseg + 1, 0), seg_task_ptr(nseg + 1, 0), seg_tasks;
  std::vector<long long> ce0, ce1;
  for (int g = 0; g < nseg; ++g) {
    seg_chunk_ptr[g] = (int)chunk_seg.size();
    for (long long e = seg_off[g]; e < seg_off[g + 1]; e += 4096) {
      chunk_seg.push_back(g);
      ce0.push_back(e);
      ce1.push_back(std::min(seg_off[g + 1], e + 4096));
    }
  }
  seg_chunk_ptr[nseg] = (int)chunk_seg.size();
  std::vector<std::vector<int>> by_seg(nseg);
  for (int t = 0; t < D.ntask; ++t) by_seg[slab_seg[tslab[t]]].push_back(t);
  for (int g = 0; g < nseg; ++g) {
    seg_task_ptr[g] = (int)seg_tasks.size();
    seg_tasks.insert(seg_tasks.end(), by_seg[g].begin(), by_seg[g].end());
  }
  seg_task_ptr[nseg] = (int)seg_tasks.size();

  kr_seg* g = new kr_seg();
  g->op = op;
  g->nseg = nseg;
  g->nchunk = (int)chunk_seg.size();
  const size_t M1 = (size_t)op->maxorder + 1;
  int rc = KR_OK;
#define SU(host, count, dst) \
  if ((rc = seg_upload(g, host, count, dst)) != KR_OK) { kr_seg_destroy(g); return rc; }
  SU(slab_seg, (size_t)ns, &g->slab_seg);
  SU(chunk_seg.data(), chunk_seg.size(), &g->chunk_seg);
  SU(ce0.data(), ce0.size(), &g->chunk_e0);
  SU(ce1.data(), ce1.size(), &g->chunk_e1);
  SU(seg_chunk_ptr.data(), seg_chunk_ptr.size(), &g->seg_chunk_ptr);
  SU(seg_task_ptr.data(), seg_task_ptr.size(), &g->seg_task_ptr);
  SU(seg_tasks.data(), seg_tasks.size(), &g->seg_tasks);
  SU((const double2*)nullptr, nseg * M1, &g->alpha);
  SU((const double*)nullptr, nseg * M1, &g->beta);
  SU((const double2*)nullptr, nseg * M1, &g->coef);
  SU((const int*)nullptr, (size_t)nseg, &g->done);
  SU((const int*)nullptr, (size_t)nseg, &g->kout);
  SU((const int*)nullptr, (size_t)nseg, &g->ufin);
  SU((const int*)nullptr, (size_t)2, &g->nactive);
  SU((const double*)nullptr, (size_t)g->nchunk, &g->chunk_b);
  SU((const double*)nullptr, (size_t)g->nchunk, &g->chunk_c);
#undef SU
  // persistent grid: every CTA resident (cooperative launch)
  if (ensure_step_smem(op->smem) != cudaSuccess) {
    kr_seg_destroy(g);
    return set_err(op->ctx, KR_ERR_CUDA, "kr_seg_create: cannot raise the dynamic shared memory");
  }
  int occ = 0;
  int occ32 = 0;
  cudaError_t ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kr_seg_step_kernel<false>, KR_THREADS, op->smem);
  if (ce == cudaSuccess)
    ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, kr_seg_step_kernel<true>, KR_THREADS, op->smem);
  if (ce != cudaSuccess || occ < 1 || occ32 < 1) {
    kr_seg_destroy(g);
    return set_err(op->ctx, KR_ERR_CUDA, "kr_seg_step_kernel cannot be resident");
  }
  g->grid = std::max(1, op->ctx->nsm * std::min(occ, 2));
  g->grid32 = std::max(1, op->ctx->nsm * std::min(occ32, 3));  // FP32 products: 3 CTAs per SM
  *out = g;
  return KR_OK;
}

extern "C" int kr_seg_step(kr_seg* g, void* states, const void* phase, double fac_re, double fac_im, double tol,
                           int32_t* korder, void* stream) {
  if (!g || !states) return set_err(g ? g->op->ctx : nullptr, KR_ERR_ARG, "kr_seg_step: bad argument");
  kr_op* op = g->op;
  cudaStream_t st = (cudaStream_t)stream;
  SegArgs a;
  a.op = op->dev;
  a.state = (double2*)states;
  a.phase = (const double2*)phase;
  a.V = op->V;
  a.Wb[0] = op->Wb0;
  a.Wb[1] = op->Wb1;
  a.w = op->w;
  a.ub[0] = op->ub0;
  a.ub[1] = op->ub1;
  a.task_alpha = op->task_alpha;
  a.counters = op->counters;
  a.bar_count = op->bar;
  a.bar_gen = op->bar + 1;
  a.status = op->status;
  a.nseg = g->nseg;
  a.nchunk = g->nchunk;
  a.slab_seg = g->slab_seg;
  a.chunk_seg = g->chunk_seg;
  a.chunk_e0 = g->chunk_e0;
  a.chunk_e1 = g->chunk_e1;
  a.seg_chunk_ptr = g->seg_chunk_ptr;
  a.seg_task_ptr = g->seg_task_ptr;
  a.seg_tasks = g->seg_tasks;
  a.alpha = g->alpha;
  a.beta = g->beta;
  a.coef = g->coef;
  a.done = g->done;
  a.kout = g->kout;
  a.ufin = g->ufin;
  a.chunk_b = g->chunk_b;
  a.chunk_c = g->chunk_c;
  a.nactive = g->nactive;
  a.fac = make_double2(fac_re, fac_im);
  a.tol = tol;
  a.maxorder = op->maxorder;
  a.dim = op->dev.dim_out;
  KR_CUDA(op->ctx, cudaMemsetAsync(op->bar, 0, sizeof(unsigned), st));  // arrival count only
  KR_CUDA(op->ctx, ensure_step_smem(op->smem));
  void* args[] = {&a};
  KR_CUDA(op->ctx, cudaLaunchCooperativeKernel(g->f32 ? (void*)kr_seg_step_kernel<true> : (void*)kr_seg_step_kernel<false>,
                                               dim3(g->f32 ? g->grid32 : g->grid), dim3(KR_THREADS), args, op->smem, st));
  g->launches++;
  int hs = 0;
  KR_CUDA(op->ctx, cudaMemcpyAsync(&hs, op->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (korder) KR_CUDA(op->ctx, cudaMemcpyAsync(korder, g->kout, sizeof(int) * g->nseg, cudaMemcpyDeviceToHost, st));
  KR_CUDA(op->ctx, cudaStreamSynchronize(st));
  if (hs != 0) {
    cudaMemsetAsync(op->status, 0, sizeof(int), st);
    cudaStreamSynchronize(st);
    if (hs == KR_ERR_MAXORDER)
      return set_err(op->ctx, KR_ERR_MAXORDER,
                     "Lanczos reached maximum order of '" + std::to_string(op->maxorder) + "' without convergence");
    return set_err(op->ctx, hs, "device-side wait gave up (grid barrier timeout)");
  }
  return KR_OK;
}

extern "C" int64_t kr_seg_launch_count(const kr_seg* g) { return g ? g->launches : -1; }
