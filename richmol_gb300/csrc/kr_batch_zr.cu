// Batched mat-vec on the FP32 pipes, register-tiled (the KR_MATVEC_FP32_REG
// kind of the batched Krylov step): the Kronecker contraction of
// field.py:1212-1243, Y_i += sum_terms sum_w MF_t[i, w] X_t[i + d0 + w] K_t^T,
// in complex64 with FP32 accumulation.
//
// One CTA = 4 warps computes a tile of 4 * RW consecutive output rows of one
// slab for 32 vectors (lane = vector; vector-minor arrays, so every load and
// store of a warp is one contiguous 256-byte row). Warp w owns rows
// w * RW .. w * RW + RW - 1 of the tile, every thread all NKP output columns of
// those rows for its vector: RW x NKP complex accumulators in registers for
// the whole slab's sum over terms. Per term, Z-first:
//   Z[r, b]  = sum_w MF[r, w] X[r + d0 + w, b]      (the M band; each input row
//              of the band window is loaded once and scattered into the RW
//              rows it feeds)
//   Y[r, a] += sum_b K[a, b] Z[r, b]                (K^T rows from shared memory
//              as float4, each value used by all RW rows)
// so the K work is done once per output row (no band window recomputation)
// and nothing is staged per term but the tables: the term parameters, K^T
// (padded to NKP columns) and the MF band of the tile's rows for up to TCH
// terms at once are put in shared memory once, after which the warps run
// through the terms without synchronising.
#include <cuda_runtime.h>

#include <algorithm>

#include "kr_batch_mv.cuh"

#define ZR_WARPS 4

struct ZrTerm {
  long long xoff;  // first element of the input slab
  int nk2, ld2, dm2, W, Wst, d0, ktype, mtype, dia;
};

template <int NKP>
struct ZrCfg {
  static constexpr int RW = NKP == 32 ? 1 : 2;                   // output rows per warp
  static constexpr int ROWS = ZR_WARPS * RW;                      // rows per tile
  static constexpr int TCH = NKP == 32 ? 4 : NKP == 16 ? 8 : 16;  // terms staged at once
  static constexpr int KSZ = 2 * NKP * NKP;                       // floats of one K^T (two planes)
  static constexpr int OFF_K = 128 * ((TCH * (int)sizeof(ZrTerm) + 127) / 128);
  static constexpr int OFF_MF = OFF_K + TCH * KSZ * 4;
  static constexpr int OFF_C = OFF_MF + TCH * ROWS * KB_WMAX * 8;
  static constexpr int BYTES = OFF_C + TCH * ROWS * KB_WMAX * 4;
};

// z += m x for a real (MT 1), imaginary (2) or complex (0) M-band value m
template <int MT>
__device__ __forceinline__ void zr_macc(float2& z, float2 m, float2 x) {
  if (MT == 1) {
    z.x = fmaf(m.x, x.x, z.x);
    z.y = fmaf(m.x, x.y, z.y);
  } else if (MT == 2) {
    z.x = fmaf(-m.y, x.y, z.x);
    z.y = fmaf(m.y, x.x, z.y);
  } else {
    z.x = fmaf(m.x, x.x, fmaf(-m.y, x.y, z.x));
    z.y = fmaf(m.x, x.y, fmaf(m.y, x.x, z.y));
  }
}

// one input row (its first nk2 of NKP columns) of this thread's vector
template <int NKP>
__device__ __forceinline__ void zr_load_row(float2 (&x)[NKP], const float2* xr, long long nb, int nk2) {
#pragma unroll
  for (int b = 0; b < NKP; ++b) x[b] = b < nk2 ? __ldg(xr + (long long)b * nb) : make_float2(0.f, 0.f);
}

// Z of one term for this warp's RW rows (rows at or beyond nr stay zero)
template <int NKP, int MT>
__device__ __forceinline__ void zr_zstep(float2 (&z)[ZrCfg<NKP>::RW][NKP], const ZrTerm& T, const float2* Xs,
                                         long long nb, int i0, int ra, int nr, const float2* MFt, const int* Ct) {
  constexpr int RW = ZrCfg<NKP>::RW;
#pragma unroll
  for (int rr = 0; rr < RW; ++rr)
#pragma unroll
    for (int b = 0; b < NKP; ++b) z[rr][b] = make_float2(0.f, 0.f);
  if (T.dia) {
    // window rows c = 0 .. RW + W - 2: input row i0 + ra + d0 + c feeds tile row
    // rr through band slot w = c - rr; rows outside the input slab meet band
    // values that are zero (the band is clamped to the slab), so they are skipped
    const int nwin = RW + T.W - 1;
    const int j0 = i0 + ra + T.d0;
    int c = 0;
    while (c < nwin && j0 + c < 0) ++c;
    const int cend = min(nwin, T.dm2 - j0);
    if (c >= cend) return;
    // NKP = 8: the next row's loads go out before the current row is used
    // (two rows of registers); wider tiles load row by row (their registers
    // are taken by the accumulators: 234 at NKP = 16 without spills)
    constexpr bool PREF = NKP <= 8;
    float2 x[NKP], xn[PREF ? NKP : 1];
    zr_load_row<NKP>(x, Xs + (long long)(j0 + c) * T.ld2 * nb, nb, T.nk2);
    for (; c < cend; ++c) {
      if constexpr (PREF) {
        if (c + 1 < cend) zr_load_row<NKP>(xn, Xs + (long long)(j0 + c + 1) * T.ld2 * nb, nb, T.nk2);
      } else if (c > 0) {
        zr_load_row<NKP>(x, Xs + (long long)(j0 + c) * T.ld2 * nb, nb, T.nk2);
      }
#pragma unroll
      for (int rr = 0; rr < RW; ++rr) {
        const int w = c - rr;
        if (w >= 0 && w < T.W && ra + rr < nr) {
          const float2 m = MFt[(ra + rr) * KB_WMAX + w];
#pragma unroll
          for (int b = 0; b < NKP; ++b) zr_macc<MT>(z[rr][b], m, x[b]);
        }
      }
      if constexpr (PREF) {
#pragma unroll
        for (int b = 0; b < NKP; ++b) x[b] = xn[b];
      }
    }
  } else {
    // stored columns (an ELL group): every (row, slot) gathers its own input row
#pragma unroll
    for (int rr = 0; rr < RW; ++rr) {
      if (ra + rr >= nr) continue;
      for (int w = 0; w < T.W; ++w) {
        const float2 m = MFt[(ra + rr) * KB_WMAX + w];
        if (m.x == 0.f && m.y == 0.f) continue;  // ELL padding
        float2 x[NKP];
        zr_load_row<NKP>(x, Xs + (long long)Ct[(ra + rr) * KB_WMAX + w] * T.ld2 * nb, nb, T.nk2);
#pragma unroll
        for (int b = 0; b < NKP; ++b) zr_macc<MT>(z[rr][b], m, x[b]);
      }
    }
  }
}

// y += K z for this warp's rows: K^T rows (b) of NKP columns (a) from shared
// memory, plane 0 the real part (or the single stored part), plane 1 the
// imaginary part of a complex K
template <int NKP, int KT>
__device__ __forceinline__ void zr_kstep(float2 (&y)[ZrCfg<NKP>::RW][NKP], const float2 (&z)[ZrCfg<NKP>::RW][NKP],
                                         const float* Kt, int nk2) {
  constexpr int RW = ZrCfg<NKP>::RW;
#pragma unroll
  for (int b = 0; b < NKP; ++b) {
    if (b < nk2) {
      float kr[NKP], ki[NKP];
      const float4* k0 = reinterpret_cast<const float4*>(Kt + b * NKP);
#pragma unroll
      for (int a4 = 0; a4 < NKP / 4; ++a4) {
        const float4 q = k0[a4];
        kr[4 * a4] = q.x;
        kr[4 * a4 + 1] = q.y;
        kr[4 * a4 + 2] = q.z;
        kr[4 * a4 + 3] = q.w;
      }
      if (KT == 0) {
        const float4* k1 = reinterpret_cast<const float4*>(Kt + (NKP + b) * NKP);
#pragma unroll
        for (int a4 = 0; a4 < NKP / 4; ++a4) {
          const float4 q = k1[a4];
          ki[4 * a4] = q.x;
          ki[4 * a4 + 1] = q.y;
          ki[4 * a4 + 2] = q.z;
          ki[4 * a4 + 3] = q.w;
        }
      }
#pragma unroll
      for (int rr = 0; rr < RW; ++rr) {
        const float2 zz = z[rr][b];
#pragma unroll
        for (int a = 0; a < NKP; ++a) {
          float2& t = y[rr][a];
          if (KT == 1) {
            t.x = fmaf(kr[a], zz.x, t.x);
            t.y = fmaf(kr[a], zz.y, t.y);
          } else if (KT == 2) {
            t.x = fmaf(-kr[a], zz.y, t.x);
            t.y = fmaf(kr[a], zz.x, t.y);
          } else {
            t.x = fmaf(kr[a], zz.x, fmaf(-ki[a], zz.y, t.x));
            t.y = fmaf(kr[a], zz.y, fmaf(ki[a], zz.x, t.y));
          }
        }
      }
    }
  }
}

template <int NKP>
__device__ void zr_tile(const BatchMV& p, int s1, int i0, int nr, char* smem) {
  using C = ZrCfg<NKP>;
  constexpr int RW = C::RW, ROWS = C::ROWS, TCH = C::TCH, KSZ = C::KSZ;
  const DevOp& op = p.op;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const long long nb = p.nb;
  const int v = blockIdx.y * 32 + lane;
  const int slot = kb_slot(p.kslot);
  const float2* X = p.X + (long long)slot * p.slot_elems + v;
  ZrTerm* Ts = reinterpret_cast<ZrTerm*>(smem);
  float* Ks = reinterpret_cast<float*>(smem + C::OFF_K);
  float2* MFs = reinterpret_cast<float2*>(smem + C::OFF_MF);
  int* Cs = reinterpret_cast<int*>(smem + C::OFF_C);
  const int nk1 = __ldg(op.out_dk + s1);
  const int ld1 = __ldg(op.out_stride + s1);
  const int ra = wid * RW;  // this warp's first row in the tile
  float2 y[RW][NKP];
#pragma unroll
  for (int rr = 0; rr < RW; ++rr)
#pragma unroll
    for (int a = 0; a < NKP; ++a) y[rr][a] = make_float2(0.f, 0.f);
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  for (int c0 = tb; c0 < te; c0 += TCH) {
    const int nt = min(TCH, te - c0);
    __syncthreads();  // the previous chunk's terms are done with the buffers
    if (tid < nt) {
      const int term = c0 + tid;
      const int s2 = __ldg(op.t_in + term);
      const int mfi = __ldg(op.t_mf + term);
      ZrTerm T;
      T.xoff = __ldg(op.in_off + s2);
      T.nk2 = __ldg(op.in_dk + s2);
      T.ld2 = __ldg(op.in_stride + s2);
      T.dm2 = __ldg(op.in_dm + s2);
      T.Wst = __ldg(op.mf_width + mfi);
      const int d0s = __ldg(op.mf_diag + mfi);
      T.dia = d0s != KR_NO_DIAG && T.Wst <= KR_DIAG_MAX;
      // slots that carry a value with the current field (the field kernel's band)
      const int bhi = __ldcg(op.mf_band + 2 * mfi + 1);
      const int wlo = (T.dia && bhi >= 0) ? T.Wst - 1 - __ldcg(op.mf_band + 2 * mfi) : 0;
      T.W = bhi < 0 ? 0 : (T.dia ? bhi - wlo + 1 : T.Wst);
      T.d0 = T.dia ? d0s + wlo : 0;  // wlo travels in d0; the MF slots are read from wlo on
      T.ktype = __ldg(op.k_type + __ldg(op.t_k + term));
      T.mtype = __ldcg(op.mf_type + mfi);
      if (T.nk2 > NKP || T.Wst > KB_WMAX) {
        T.W = 0;  // outside the tile shape (the tile table is built so that this never happens)
        if (p.err) atomicExch(p.err, KR_ERR_ARG);
      }
      Ts[tid] = T;
    }
    __syncthreads();
    // K^T rows padded to NKP columns, the MF band (and ELL columns) of the tile's rows
    for (int t = 0; t < nt; ++t) {
      const ZrTerm T = Ts[t];
      if (T.W == 0) continue;
      const int term = c0 + t;
      const int kb = __ldg(op.t_k + term);
      const int kw = T.ktype == 0 ? 2 : 1;
      const float* KT = op.k_f32 + __ldg(op.k_off + kb);
      float* Kd = Ks + t * KSZ;
      for (int e = tid; e < kw * T.nk2 * NKP; e += blockDim.x) {
        const int plane = e / (T.nk2 * NKP);
        const int rem = e - plane * T.nk2 * NKP;
        const int b = rem / NKP, a = rem - b * NKP;
        Kd[(plane * NKP + b) * NKP + a] = a < nk1 ? __ldg(KT + ((long long)b * nk1 + a) * kw + plane) : 0.f;
      }
      const int mfi = __ldg(op.t_mf + term);
      const int wlo = T.dia ? T.d0 - __ldg(op.mf_diag + mfi) : 0;
      const float2* mf = op.mf_f32 + __ldg(op.mf_off + mfi) + wlo;
      const int* col = op.m_col + __ldg(op.mf_col_off + mfi);
      for (int e = tid; e < nr * T.W; e += blockDim.x) {
        const int r = e / T.W, w = e - r * T.W;
        const long long src = (long long)(i0 + r) * T.Wst + w;
        MFs[(t * ROWS + r) * KB_WMAX + w] = __ldcg(mf + src);
        if (!T.dia) Cs[(t * ROWS + r) * KB_WMAX + w] = __ldg(col + src);
      }
    }
    __syncthreads();
    if (ra >= nr) continue;  // this warp has no rows in this tile (uniform per warp)
    for (int t = 0; t < nt; ++t) {
      const ZrTerm T = Ts[t];
      if (T.W == 0) continue;  // MF is zero with this field: no contribution
      const float2* Xs = X + T.xoff * nb;
      const float2* MFt = MFs + t * ROWS * KB_WMAX;
      const int* Ct = Cs + t * ROWS * KB_WMAX;
      float2 z[RW][NKP];
      if (T.mtype == 1) zr_zstep<NKP, 1>(z, T, Xs, nb, i0, ra, nr, MFt, Ct);
      else if (T.mtype == 2) zr_zstep<NKP, 2>(z, T, Xs, nb, i0, ra, nr, MFt, Ct);
      else zr_zstep<NKP, 0>(z, T, Xs, nb, i0, ra, nr, MFt, Ct);
      const float* Kt = Ks + t * KSZ;
      if (T.ktype == 1) zr_kstep<NKP, 1>(y, z, Kt, T.nk2);
      else if (T.ktype == 2) zr_kstep<NKP, 2>(y, z, Kt, T.nk2);
      else zr_kstep<NKP, 0>(y, z, Kt, T.nk2);
    }
  }
  if (ra >= nr) return;
  float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)(i0 + ra) * ld1) * nb + v;
  const float sc = p.yscale ? (float)p.yscale[(long long)slot * nb + v] : 1.f;
#pragma unroll
  for (int rr = 0; rr < RW; ++rr) {
    if (ra + rr < nr) {
#pragma unroll
      for (int a = 0; a < NKP; ++a)
        if (a < nk1) Y[((long long)rr * ld1 + a) * nb] = make_float2(y[rr][a].x * sc, y[rr][a].y * sc);
    }
  }
}

// one launch per NKP class (the tile table holds the tiles of each class
// together): each class's kernel gets the registers its tile shape needs
template <int NKP>
__global__ void __launch_bounds__(ZR_WARPS * 32, 2) kb_matvec_zr(BatchMV p, const int* task, int ntask, int first) {
  extern __shared__ __align__(128) char zr_smem[];
  if (p.grp_active && !p.grp_active[blockIdx.y]) return;
  const int t = first + blockIdx.x;
  const int s1 = __ldg(task + t);
  const int i0 = __ldg(task + ntask + t);
  const int nr = __ldg(task + 2 * ntask + t);
  zr_tile<NKP>(p, s1, i0, nr, zr_smem);
}

int kb_launch_zr(kr_ctx* ctx, const BatchMV& p, const int* task, int ntask, const int* cls, int ngrp,
                 cudaStream_t st) {
  for (int c = 0; c < 3; ++c) {
    const int n = cls[c + 1] - cls[c];
    if (n <= 0) continue;
    const dim3 grid(n, ngrp);
    if (c == 0) {
      KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_zr<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        ZrCfg<8>::BYTES));
      kb_matvec_zr<8><<<grid, ZR_WARPS * 32, ZrCfg<8>::BYTES, st>>>(p, task, ntask, cls[c]);
    } else if (c == 1) {
      KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_zr<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        ZrCfg<16>::BYTES));
      kb_matvec_zr<16><<<grid, ZR_WARPS * 32, ZrCfg<16>::BYTES, st>>>(p, task, ntask, cls[c]);
    } else {
      KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_zr<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        ZrCfg<32>::BYTES));
      kb_matvec_zr<32><<<grid, ZR_WARPS * 32, ZrCfg<32>::BYTES, st>>>(p, task, ntask, cls[c]);
    }
    KR_CUDA(ctx, cudaGetLastError());
  }
  return KR_OK;
}
