// Device-side building blocks of the Krylov step: complex helpers, the bounded
// grid barrier, deterministic reductions and the Kronecker mat-vec task loop.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define KR_WARPS 8                  // warps per CTA (2 CTAs per SM)
#define KR_THREADS (KR_WARPS * 32)
#define KR_QMAX 4                   // (row, a) outputs per thread of a task
#define KR_BARRIER_TIMEOUT_NS 2000000000ull  // 2 s per grid-barrier wait
#define KR_BARRIER_MAX_SPINS (1u << 24)      // spins per wait (>= 5 s at 0.3 us each)

// ---------------------------------------------------------------------------
// complex helpers (double2 = re, im)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a += b * c
__device__ __forceinline__ void cfma(double2& a, double2 b, double2 c) {
  a.x = fma(b.x, c.x, a.x);
  a.x = fma(-b.y, c.y, a.x);
  a.y = fma(b.x, c.y, a.y);
  a.y = fma(b.y, c.x, a.y);
}
// conj(a) * b
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ double2 ldcg2(const double2* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// operator tables on the device
// ---------------------------------------------------------------------------
#define KR_NO_DIAG (-2147483647 - 1)  // MF instance without diagonal slot order
#define KR_EXPV_MMAX 30                // largest Krylov dimension of kr_expv
#define KR_DIAG_MAX 8                  // widest diagonal band the batched mat-vec takes by offset

struct DevOp {
  int nslab_out, nslab_in;
  const int* out_dm; const int* out_dk; const long long* out_off;
  const int* in_dm;  const int* in_dk;  const long long* in_off;
  const int* out_stride; const int* in_stride;  // slab row strides (= dk unless split into column chunks)
  long long dim_out, dim_in;
  // K blocks
  const long long* k_off; const int* k_rows; const int* k_cols; const int* k_type; const double* k_data;
  const float* k_f32;   // FP32 copy of k_data (same offsets), for the batched complex64 path
  const float* k_lo;    // k_data - k_f32 rounded to FP32: with k_f32 the double-float K
  // MF instances (ELL): values at mf_val + mf_off[i], columns at m_col + mf_col_off[i]
  const long long* mf_off; const long long* mf_col_off; const int* mf_width;
  const int* mf_diag;   // per MF instance: first diagonal d0 if slot w of row i holds column i + d0 + w, else KR_NO_DIAG
  const int* m_col; double2* mf_val;
  float2* mf_f32;       // FP32 copy of mf_val, written with it by the field kernel
  float2* mf_lo;        // mf_val - mf_f32 rounded to FP32 (double-float MF), written with it
  // terms grouped by output slab
  const int* term_ptr; const int* t_in; const int* t_k; const int* t_mf;
  const int* mf_type;   // per MF instance: 0 complex, 1 real, 2 imaginary (set with the field)
  const int* mf_band;   // per MF instance: [W - 1 - lowest, highest] non-zero slot, -1 if none (set with the field)
  // row tasks, handed out dynamically in the order task_order
  const int* task_slab; const int* task_row0; const int* task_nrows;
  const int* task_order; int ntask;
  int zmax;  // complex entries of one Z staging buffer
};

// ---------------------------------------------------------------------------
// grid barrier with a bounded wait. Every CTA of a cooperative launch calls it
// the same number of times. Returns false if the wait gave up or another CTA
// reported an error; the caller then leaves the kernel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

static __device__ bool grid_barrier(unsigned* count, unsigned* gen, int* status, int code_on_timeout) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned my_gen = ld_acquire_u32(gen);
    __threadfence();
    unsigned arrived = atomicAdd(count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      st_release_u32(gen, my_gen + 1u);
    } else {
      unsigned long long t0 = globaltimer_ns();
      // bounded twice: by time, and by a spin count that takes longer than the
      // time limit at any iteration time (an acquire load of L2 takes ~0.3 us)
      for (unsigned spins = 0; ld_acquire_u32(gen) == my_gen; ++spins) {
        if (globaltimer_ns() - t0 > KR_BARRIER_TIMEOUT_NS || spins >= KR_BARRIER_MAX_SPINS) {
          atomicCAS(status, 0, code_on_timeout);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (ok && *((volatile int*)status) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------
// deterministic reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}
// Sum of one double2 per thread over the CTA; result valid in all threads.
static __device__ double2 block_sum2(double2 v, double2* scratch /* KR_WARPS */) {
  v = warp_sum2(v);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  for (int w = 0; w < KR_WARPS; ++w) s = cadd(s, scratch[w]);
  __syncthreads();
  return s;
}
// Sum of n values written by the CTAs of the grid, same order in every CTA.
static __device__ double2 grid_partials_sum2(const double2* part, int n, double2* scratch) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (warp == 0) {
    double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
    int i = lane;
    for (; i + 96 < n; i += 128) {
      s0 = cadd(s0, ldcg2(part + i));
      s1 = cadd(s1, ldcg2(part + i + 32));
      s2 = cadd(s2, ldcg2(part + i + 64));
      s3 = cadd(s3, ldcg2(part + i + 96));
    }
    for (; i < n; i += 32) s0 = cadd(s0, ldcg2(part + i));
    double2 s = cadd(cadd(s0, s1), cadd(s2, s3));
    s = warp_sum2(s);
    if (lane == 0) scratch[0] = s;
  }
  __syncthreads();
  double2 r = scratch[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// The row-task mat-vec below (matvec_cta_tasks) with its products in FP32:
// same tasks, terms and staging; see its F32 argument.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cfmaf(float2& s, float2 a, float2 b) {
  s.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, s.x));
  s.y = fmaf(a.x, b.y, fmaf(a.y, b.x, s.y));
}
template <bool ALPHA>
__device__ void matvec_cta_tasks_f32(const DevOp& op, const double2* __restrict__ x, double xscale,
                                     double2* __restrict__ y, unsigned* counter, double2* task_alpha,
                                     double2* smem, double2* red, const int* seg_done, const int* slab_seg) {
  __shared__ int s_task;
  const int tid = threadIdx.x;
  float2* zb[2] = {reinterpret_cast<float2*>(smem), reinterpret_cast<float2*>(smem) + op.zmax};
  const float xs = (float)xscale;
  for (;;) {
    if (tid == 0) s_task = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_task;
    __syncthreads();
    if (t >= op.ntask) break;
    const int task = __ldg(op.task_order + t);
    const int s1 = __ldg(op.task_slab + task);
    if (seg_done && __ldcg(seg_done + __ldg(slab_seg + s1))) {
      if (ALPHA && tid == 0) task_alpha[task] = make_double2(0.0, 0.0);
      continue;
    }
    const int i0 = __ldg(op.task_row0 + task);
    const int nr = __ldg(op.task_nrows + task);
    const int nk1 = __ldg(op.out_dk + s1);
    const int npair = nr * nk1;
    float2 acc[KR_QMAX];
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) acc[q] = make_float2(0.f, 0.f);
    const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
    for (int term = tb; term < te; ++term) {
      float2* Z = zb[(term - tb) & 1];
      const int s2 = __ldg(op.t_in + term);
      const int kbk = __ldg(op.t_k + term);
      const int mfi = __ldg(op.t_mf + term);
      const int nk2 = __ldg(op.in_dk + s2);
      const double2* X = x + __ldg(op.in_off + s2);
      const int W = __ldg(op.mf_width + mfi);
      const int* col = op.m_col + __ldg(op.mf_col_off + mfi);
      const float2* mf = op.mf_f32 + __ldg(op.mf_off + mfi);
      const int mtype = __ldcg(op.mf_type + mfi);
      const int nz = nr * nk2;
      for (int p = tid; p < nz; p += blockDim.x) {
        const int r = p / nk2;
        const int b = p - r * nk2;
        const int base = (i0 + r) * W;
        float2 z = make_float2(0.f, 0.f);
        for (int w = 0; w < W; ++w) {
          const float2 m = __ldcg(mf + base + w);
          const double2 xd = ldcg2(X + (long long)__ldg(col + base + w) * nk2 + b);
          const float2 xv = make_float2((float)xd.x, (float)xd.y);
          if (mtype == 1) {
            z.x = fmaf(m.x, xv.x, z.x);
            z.y = fmaf(m.x, xv.y, z.y);
          } else if (mtype == 2) {
            z.x = fmaf(-m.y, xv.y, z.x);
            z.y = fmaf(m.y, xv.x, z.y);
          } else {
            cfmaf(z, m, xv);
          }
        }
        Z[p] = make_float2(z.x * xs, z.y * xs);
      }
      const float* KT = op.k_f32 + __ldg(op.k_off + kbk);
      const int ktype = __ldg(op.k_type + kbk);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < KR_QMAX; ++q) {
        const int p = tid + blockDim.x * q;
        if (p < npair) {
          const int r = p / nk1;
          const int a = p - r * nk1;
          const float2* zr = Z + r * nk2;
          float2 s = acc[q];
          if (ktype == 1) {
            for (int b = 0; b < nk2; ++b) {
              const float kv = __ldg(KT + b * nk1 + a);
              const float2 zv = zr[b];
              s.x = fmaf(kv, zv.x, s.x);
              s.y = fmaf(kv, zv.y, s.y);
            }
          } else if (ktype == 2) {
            for (int b = 0; b < nk2; ++b) {
              const float kv = __ldg(KT + b * nk1 + a);
              const float2 zv = zr[b];
              s.x = fmaf(-kv, zv.y, s.x);
              s.y = fmaf(kv, zv.x, s.y);
            }
          } else {
            const float2* KT2 = reinterpret_cast<const float2*>(KT);
            for (int b = 0; b < nk2; ++b) cfmaf(s, __ldg(KT2 + b * nk1 + a), zr[b]);
          }
          acc[q] = s;
        }
      }
    }
    const long long obase = __ldg(op.out_off + s1) + (long long)i0 * nk1;
    double2 al = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) {
      const int p = tid + blockDim.x * q;
      if (p < npair) {
        const double2 yv = make_double2((double)acc[q].x, (double)acc[q].y);
        y[obase + p] = yv;
        if (ALPHA) {
          const double2 v = cscale(ldcg2(x + obase + p), xscale);
          al = cadd(al, cconjmul(yv, v));
        }
      }
    }
    if (ALPHA) {
      al = block_sum2(al, red);
      if (tid == 0) task_alpha[task] = al;
    } else {
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Double-float arithmetic on both FP32 lanes (f32x2): a complex value is held
// as hi + lo pairs, h = (re_h, im_h), l = (re_l, im_l), hi the FP32 rounding of
// the FP64 value and lo the FP32 rounding of the remainder (about 48 bits in
// all). Products are exact to the lo * lo term (Dekker's product with an FMA),
// sums are Knuth's two-sum with the errors gathered in lo. GB300 runs FP32 at
// 58x its FP64 rate; one double-float multiply-add of a complex by a real
// takes 12 f32x2 instructions where FP64 takes 2 DFMA.
// ---------------------------------------------------------------------------
struct DF2 {
  float2 h, l;
};
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d)
      : "l"(*reinterpret_cast<const uint64_t*>(&a)), "l"(*reinterpret_cast<const uint64_t*>(&b)));
  return *reinterpret_cast<const float2*>(&d);
}
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d)
      : "l"(*reinterpret_cast<const uint64_t*>(&a)), "l"(*reinterpret_cast<const uint64_t*>(&b)));
  return *reinterpret_cast<const float2*>(&d);
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d)
      : "l"(*reinterpret_cast<const uint64_t*>(&a)), "l"(*reinterpret_cast<const uint64_t*>(&b)));
  return *reinterpret_cast<const float2*>(&d);
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d)
      : "l"(*reinterpret_cast<const uint64_t*>(&a)), "l"(*reinterpret_cast<const uint64_t*>(&b)),
        "l"(*reinterpret_cast<const uint64_t*>(&c)));
  return *reinterpret_cast<const float2*>(&d);
}
// s += a * b lane by lane, a = ah + al per lane (for a real factor both lanes
// hold it; an imaginary one takes b with its lanes swapped and -a on the re lane)
__device__ __forceinline__ void df2_fma(DF2& s, float2 ah, float2 al, const DF2& b) {
  const float2 q = f2_mul(make_float2(-ah.x, -ah.y), b.h);  // -p, p = ah bh rounded
  float2 e = f2_fma(ah, b.h, q);                            // ah bh - p, exact
  e = f2_fma(ah, b.l, e);
  e = f2_fma(al, b.h, e);
  const float2 t = f2_sub(s.h, q);                          // s.h + p
  const float2 bv = f2_sub(t, s.h);
  const float2 err = f2_sub(f2_sub(s.h, f2_sub(t, bv)), f2_add(q, bv));  // two-sum error
  s.l = f2_add(s.l, f2_add(err, e));
  s.h = t;
}
// renormalise: |l| below half an ulp of h
__device__ __forceinline__ void df2_norm(DF2& s) {
  const float2 t = f2_add(s.h, s.l);
  s.l = f2_sub(s.l, f2_sub(t, s.h));
  s.h = t;
}
__device__ __forceinline__ DF2 df2_swap(const DF2& b) {
  return DF2{make_float2(b.h.y, b.h.x), make_float2(b.l.y, b.l.x)};
}
// s += m b for a complex m = (mh, ml) of class mtype (1 real, 2 imaginary, 0 complex)
__device__ __forceinline__ void df2_cfma(DF2& s, float2 mh, float2 ml, int mtype, const DF2& b) {
  if (mtype != 2) df2_fma(s, make_float2(mh.x, mh.x), make_float2(ml.x, ml.x), b);
  if (mtype != 1) df2_fma(s, make_float2(-mh.y, mh.y), make_float2(-ml.y, ml.y), df2_swap(b));
}
// a + b of two double-float values (two-sum of the hi parts, lo parts added)
__device__ __forceinline__ DF2 df2_add(const DF2& a, const DF2& b) {
  const float2 t = f2_add(a.h, b.h);
  const float2 bv = f2_sub(t, a.h);
  const float2 err = f2_add(f2_sub(a.h, f2_sub(t, bv)), f2_sub(b.h, bv));
  DF2 s{t, f2_add(f2_add(a.l, b.l), err)};
  df2_norm(s);
  return s;
}
__device__ __forceinline__ DF2 df2_split(double2 v) {
  const float2 h = make_float2((float)v.x, (float)v.y);
  return DF2{h, make_float2((float)(v.x - (double)h.x), (float)(v.y - (double)h.y))};
}
__device__ __forceinline__ double2 df2_value(const DF2& s) {
  return make_double2((double)s.h.x + (double)s.l.x, (double)s.h.y + (double)s.l.y);
}
__device__ __forceinline__ DF2 df2_ld(const float4* p) {
  const float4 v = __ldcg(p);
  return DF2{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ void df2_st(float4* p, const DF2& v) { *p = make_float4(v.h.x, v.h.y, v.l.x, v.l.y); }

// The row-task mat-vec below (matvec_cta_tasks) with double-float products:
// x from its double-float copy xdf (the same vector, unscaled), MF and K as
// mf_f32 + mf_lo and k_f32 + k_lo, Z and the sums double-float, Z scaled by
// xscale in FP64, y and the alpha partial in FP64.
template <bool ALPHA>
__device__ void matvec_cta_tasks_df(const DevOp& op, const double2* __restrict__ x, const float4* __restrict__ xdf,
                                    double xscale, double2* __restrict__ y, unsigned* counter,
                                    double2* task_alpha, double2* smem, double2* red) {
  __shared__ int s_task;
  const int tid = threadIdx.x;
  float4* zb[2] = {reinterpret_cast<float4*>(smem), reinterpret_cast<float4*>(smem) + op.zmax};
  const float xsh = (float)xscale, xsl = (float)(xscale - (double)xsh);  // xscale as a double-float
  for (;;) {
    if (tid == 0) s_task = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_task;
    __syncthreads();
    if (t >= op.ntask) break;
    const int task = __ldg(op.task_order + t);
    const int s1 = __ldg(op.task_slab + task);
    const int i0 = __ldg(op.task_row0 + task);
    const int nr = __ldg(op.task_nrows + task);
    const int nk1 = __ldg(op.out_dk + s1);
    const int npair = nr * nk1;
    DF2 acc[KR_QMAX];
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) acc[q] = DF2{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
    for (int term = tb; term < te; ++term) {
      float4* Z = zb[(term - tb) & 1];
      const int s2 = __ldg(op.t_in + term);
      const int kbk = __ldg(op.t_k + term);
      const int mfi = __ldg(op.t_mf + term);
      const int nk2 = __ldg(op.in_dk + s2);
      const float4* X = xdf + __ldg(op.in_off + s2);
      const int W = __ldg(op.mf_width + mfi);
      const int* col = op.m_col + __ldg(op.mf_col_off + mfi);
      const long long mo = __ldg(op.mf_off + mfi);
      const float2* mfh = op.mf_f32 + mo;
      const float2* mfl = op.mf_lo + mo;
      const int mtype = __ldcg(op.mf_type + mfi);
      const int nz = nr * nk2;
      for (int p = tid; p < nz; p += blockDim.x) {
        const int r = p / nk2;
        const int b = p - r * nk2;
        const int base = (i0 + r) * W;
        DF2 z{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        for (int w = 0; w < W; ++w)
          df2_cfma(z, __ldcg(mfh + base + w), __ldcg(mfl + base + w), mtype,
                   df2_ld(X + (long long)__ldg(col + base + w) * nk2 + b));
        df2_norm(z);
        DF2 zs{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // z * xscale, on the FP32 pipes
        df2_fma(zs, make_float2(xsh, xsh), make_float2(xsl, xsl), z);
        df2_norm(zs);
        df2_st(Z + p, zs);
      }
      const long long ko = __ldg(op.k_off + kbk);
      const int ktype = __ldg(op.k_type + kbk);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < KR_QMAX; ++q) {
        const int p = tid + blockDim.x * q;
        if (p < npair) {
          const int r = p / nk1;
          const int a = p - r * nk1;
          const float4* zr = Z + r * nk2;
          // two partial sums (even and odd b): independent chains
          DF2 s0 = acc[q], s1{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
          if (ktype == 1 || ktype == 2) {  // real K, or K = i Ki
            const float* KH = op.k_f32 + ko;
            const float* KL = op.k_lo + ko;
            const float sg = ktype == 1 ? 1.f : -1.f;
            int b = 0;
            for (; b + 1 < nk2; b += 2) {
              const float kh0 = __ldg(KH + b * nk1 + a), kl0 = __ldg(KL + b * nk1 + a);
              const float kh1 = __ldg(KH + (b + 1) * nk1 + a), kl1 = __ldg(KL + (b + 1) * nk1 + a);
              const float4 z0 = zr[b], z1 = zr[b + 1];
              DF2 x0{make_float2(z0.x, z0.y), make_float2(z0.z, z0.w)};
              DF2 x1{make_float2(z1.x, z1.y), make_float2(z1.z, z1.w)};
              if (ktype == 2) {
                x0 = df2_swap(x0);
                x1 = df2_swap(x1);
              }
              df2_fma(s0, make_float2(sg * kh0, kh0), make_float2(sg * kl0, kl0), x0);
              df2_fma(s1, make_float2(sg * kh1, kh1), make_float2(sg * kl1, kl1), x1);
            }
            if (b < nk2) {
              const float kh0 = __ldg(KH + b * nk1 + a), kl0 = __ldg(KL + b * nk1 + a);
              const float4 z0 = zr[b];
              DF2 x0{make_float2(z0.x, z0.y), make_float2(z0.z, z0.w)};
              if (ktype == 2) x0 = df2_swap(x0);
              df2_fma(s0, make_float2(sg * kh0, kh0), make_float2(sg * kl0, kl0), x0);
            }
          } else {  // complex K, interleaved (re, im)
            const float2* KH = reinterpret_cast<const float2*>(op.k_f32 + ko);
            const float2* KL = reinterpret_cast<const float2*>(op.k_lo + ko);
            for (int b = 0; b < nk2; ++b) {
              const float4 zv = zr[b];
              df2_cfma((b & 1) ? s1 : s0, __ldg(KH + b * nk1 + a), __ldg(KL + b * nk1 + a), 0,
                       DF2{make_float2(zv.x, zv.y), make_float2(zv.z, zv.w)});
            }
          }
          acc[q] = df2_add(s0, s1);
        }
      }
    }
    const long long obase = __ldg(op.out_off + s1) + (long long)i0 * nk1;
    double2 al = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) {
      const int p = tid + blockDim.x * q;
      if (p < npair) {
        const double2 yv = df2_value(acc[q]);
        y[obase + p] = yv;
        if (ALPHA) {
          const double2 v = cscale(ldcg2(x + obase + p), xscale);
          al = cadd(al, cconjmul(yv, v));
        }
      }
    }
    if (ALPHA) {
      al = block_sum2(al, red);
      if (tid == 0) task_alpha[task] = al;
    } else {
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Kronecker mat-vec over the row tasks of one CTA. A task is a block of nr
// consecutive rows of one output slab; all threads of the CTA work on it:
//   Z_t[r, b]   = xscale * sum_w MF_t[i0 + r, w] * x[s2][col_t(i0 + r, w), b]
//   y[s1][i0 + r, a] = sum_terms sum_b K_t[a, b] * Z_t[r, b]
// (field.py:1229-1243 computes the same sum as MF (K X^T)^T per term.)
// Z of a term is staged in shared memory (double-buffered, one __syncthreads
// per term); each thread owns up to KR_QMAX (row, a) outputs.
// With ALPHA the CTA also accumulates sum conj(y) * (xscale * x) over its
// outputs: the Lanczos coefficient vdot(w, V_k) of tdse.py:468 for a square
// operator, where V_k = xscale * x.
// ---------------------------------------------------------------------------
// seg_done / slab_seg (optional): tasks of an output slab whose segment is
// done are skipped (their alpha partial is zero), for the segmented step.
// F32: the products in single precision on the FP32 pipes (GB300's FP64 rate
// is 1/58 of its FP32 rate): x read in FP64 and rounded, the FP32 copies of K
// and MF (k_f32, mf_f32), Z and the sums in FP32, y and the alpha partial in
// FP64 (the Lanczos scalars stay FP64).
template <bool ALPHA, bool F32 = false>
__device__ void matvec_cta_tasks(const DevOp& op, const double2* __restrict__ x, double xscale,
                                 double2* __restrict__ y, unsigned* counter, double2* task_alpha,
                                 double2* smem, double2* red, const int* seg_done = nullptr,
                                 const int* slab_seg = nullptr) {
  if constexpr (F32) {
    matvec_cta_tasks_f32<ALPHA>(op, x, xscale, y, counter, task_alpha, smem, red, seg_done, slab_seg);
    return;
  }
  __shared__ int s_task;
  const int tid = threadIdx.x;
  double2* zb[2] = {smem, smem + op.zmax};
  for (;;) {
    // tasks are handed out in order of decreasing cost
    if (tid == 0) s_task = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_task;
    __syncthreads();
    if (t >= op.ntask) break;
    const int task = __ldg(op.task_order + t);
    const int s1 = __ldg(op.task_slab + task);
    if (seg_done && __ldcg(seg_done + __ldg(slab_seg + s1))) {  // uniform over the CTA
      if (ALPHA && tid == 0) task_alpha[task] = make_double2(0.0, 0.0);
      continue;
    }
    const int i0 = __ldg(op.task_row0 + task);
    const int nr = __ldg(op.task_nrows + task);
    const int nk1 = __ldg(op.out_dk + s1);
    const int npair = nr * nk1;
    double2 acc[KR_QMAX];
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) acc[q] = make_double2(0.0, 0.0);

    const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
    for (int term = tb; term < te; ++term) {
      double2* Z = zb[(term - tb) & 1];
      const int s2 = __ldg(op.t_in + term);
      const int kbk = __ldg(op.t_k + term);
      const int mfi = __ldg(op.t_mf + term);
      const int nk2 = __ldg(op.in_dk + s2);
      const double2* X = x + __ldg(op.in_off + s2);
      const int W = __ldg(op.mf_width + mfi);
      const int* col = op.m_col + __ldg(op.mf_col_off + mfi);
      const double2* mf = op.mf_val + __ldg(op.mf_off + mfi);
      const int mtype = __ldcg(op.mf_type + mfi);
      // stage Z (nr x nk2)
      const int nz = nr * nk2;
      for (int p = tid; p < nz; p += blockDim.x) {
        const int r = p / nk2;
        const int b = p - r * nk2;
        const int base = (i0 + r) * W;
        double2 z = make_double2(0.0, 0.0);
        if (mtype == 1) {          // MF real
          for (int w = 0; w < W; ++w) {
            const double m = __ldcg(&mf[base + w].x);
            const double2 xv = ldcg2(X + (long long)__ldg(col + base + w) * nk2 + b);
            z.x = fma(m, xv.x, z.x);
            z.y = fma(m, xv.y, z.y);
          }
        } else if (mtype == 2) {   // MF imaginary
          for (int w = 0; w < W; ++w) {
            const double m = __ldcg(&mf[base + w].y);
            const double2 xv = ldcg2(X + (long long)__ldg(col + base + w) * nk2 + b);
            z.x = fma(-m, xv.y, z.x);
            z.y = fma(m, xv.x, z.y);
          }
        } else {
          for (int w = 0; w < W; ++w)
            cfma(z, ldcg2(mf + base + w), ldcg2(X + (long long)__ldg(col + base + w) * nk2 + b));
        }
        Z[p] = cscale(z, xscale);
      }
      // K is stored transposed (KT[b][a]) so that threads with consecutive a
      // read consecutive words
      const double* KT = op.k_data + __ldg(op.k_off + kbk);
      const int ktype = __ldg(op.k_type + kbk);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < KR_QMAX; ++q) {
        const int p = tid + blockDim.x * q;
        if (p < npair) {
          const int r = p / nk1;
          const int a = p - r * nk1;
          const double2* zr = Z + r * nk2;
          double2 s = acc[q];
          if (ktype == 1) {  // real K
            for (int b = 0; b < nk2; ++b) {
              const double kv = __ldg(KT + b * nk1 + a);
              const double2 zv = zr[b];
              s.x = fma(kv, zv.x, s.x);
              s.y = fma(kv, zv.y, s.y);
            }
          } else if (ktype == 2) {  // K = i * Ki
            for (int b = 0; b < nk2; ++b) {
              const double kv = __ldg(KT + b * nk1 + a);
              const double2 zv = zr[b];
              s.x = fma(-kv, zv.y, s.x);
              s.y = fma(kv, zv.x, s.y);
            }
          } else {  // complex K
            const double2* KT2 = reinterpret_cast<const double2*>(KT);
            for (int b = 0; b < nk2; ++b) cfma(s, __ldg(KT2 + b * nk1 + a), zr[b]);
          }
          acc[q] = s;
        }
      }
    }
    const long long obase = __ldg(op.out_off + s1) + (long long)i0 * nk1;
    double2 al = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < KR_QMAX; ++q) {
      const int p = tid + blockDim.x * q;
      if (p < npair) {
        y[obase + p] = acc[q];
        if (ALPHA) {
          const double2 v = cscale(ldcg2(x + obase + p), xscale);
          al = cadd(al, cconjmul(acc[q], v));
        }
      }
    }
    if (ALPHA) {
      // per-task partial of vdot(w, V_k): summed later in task order, so the
      // result does not depend on which CTA ran the task
      al = block_sum2(al, red);
      if (tid == 0) task_alpha[task] = al;
    } else {
      __syncthreads();
    }
  }
}
