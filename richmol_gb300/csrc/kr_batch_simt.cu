// Batched mat-vec on the FP32 pipes (every product an FMA): the
// KR_MATVEC_FP32 kind of the batched Krylov step.
#include <cuda_runtime.h>

#include <algorithm>

#include "kr_batch_mv.cuh"

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

// T rows jr < nrow for the input rows j0 + jr into Ts[jr] (rows ld2 elements
// apart); rows outside the input slab [0, dm2) are zero. (row, half-row) units
// go round-robin over the 8 warps.
template <int NKP>
__device__ __forceinline__ void kb_tstep(const float2* Xs2, long long nb, int nk2, int ld2, int ktype,
                                         const float* Ks, float2* Ts, int j0, int nrow, int dm2, int wid, int lane) {
  constexpr int NH = NKP >= 8 ? 2 : 1;
  constexpr int AB = NKP / NH;
  for (int u = wid; u < nrow * NH; u += 8) {
    const int jr = u / NH, h = u - jr * NH;
    const int j = j0 + jr;
    float2 t[AB];
    if (j >= 0 && j < dm2) {
      const float2* xr = Xs2 + (long long)j * ld2 * nb;
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
  const int ld1 = __ldg(op.out_stride + s1);  // output row stride
  float2 y[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) y[q] = make_float2(0.f, 0.f);
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  for (int term = tb; term < te; ++term) {
    const int s2 = __ldg(op.t_in + term);
    const int kb = __ldg(op.t_k + term);
    const int mfi = __ldg(op.t_mf + term);
    const int nk2 = __ldg(op.in_dk + s2);
    const int ld2 = __ldg(op.in_stride + s2);
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
    const float2* Xs2 = p.X + (long long)kb_slot(p.kslot) * p.slot_elems + (long long)__ldg(op.in_off + s2) * nb + v;
    if (dia) {
      // T rows of the band: input rows i0 + d0 .. i0 + d0 + nr + W - 2
      kb_tstep<NKP>(Xs2, nb, nk2, ld2, ktype, Ks, Ts, i0 + d0, nr + W - 1, dm2, wid, lane);
      __syncthreads();
      if (mtype == 1) kb_mdia<NKP, 1>(y, Ts, MFs, W, r0, a0, nr, lane);
      else if (mtype == 2) kb_mdia<NKP, 2>(y, Ts, MFs, W, r0, a0, nr, lane);
      else kb_mdia<NKP, 0>(y, Ts, MFs, W, r0, a0, nr, lane);
    } else {
      const int jmin = meta[0], jmax = meta[1];
      for (int jc = jmin; jc <= jmax; jc += NJ) {
        const int nj = min(NJ, jmax - jc + 1);
        if (jc != jmin) __syncthreads();  // the previous chunk's M step is done with Ts
        kb_tstep<NKP>(Xs2, nb, nk2, ld2, ktype, Ks, Ts, jc, nj, dm2, wid, lane);
        __syncthreads();
        if (mtype == 1) kb_mell<NKP, 1>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
        else if (mtype == 2) kb_mell<NKP, 2>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
        else kb_mell<NKP, 0>(y, Ts, MFs, Cs, W, jc, nj, r0, a0, nr, lane);
      }
    }
  }
  float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * ld1) * nb + v;
  const float sc = p.yscale ? (float)p.yscale[(long long)kb_slot(p.kslot) * nb + v] : 1.f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int aa = 0; aa < 4; ++aa) {
      const int i = r0 + r, a = a0 + aa;
      if (i < nr && a < nk1) Y[((long long)i * ld1 + a) * nb] = make_float2(y[r * 4 + aa].x * sc, y[r * 4 + aa].y * sc);
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

int kb_launch_simt(kr_ctx* ctx, const BatchMV& p, int ntask, int ngrp, cudaStream_t st) {
  const size_t smem = kb_matvec_smem();
  KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kb_matvec<<<dim3(ntask, ngrp), 256, smem, st>>>(p);
  KR_CUDA(ctx, cudaGetLastError());
  return KR_OK;
}
