// Batched mat-vec with the K contraction on the tcgen05 tensor cores (split
// TF32, accumulators in TMEM, X tiles by TMA): the KR_MATVEC_TENSOR kind of the
// batched Krylov step, and the single-MMA probe kr_probe_mma.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include <cuda.h>

#include "kr_batch_mv.cuh"
#include "kr_tc.cuh"

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
  __device__ __forceinline__ void load(const float2* Xs2, long long nb, int nk2, int ld2, int dm2, int j0, int nrow,
                                       int b0) {
#pragma unroll
    for (int c = 0; c < RP; ++c) {
      const int j = j0 + c;
      const bool rin = c < nrow && j >= 0 && j < dm2;
      const float2* xr = Xs2 + (long long)j * ld2 * nb;
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
template <int KP, int MT, int BH = KP / 2>
__device__ __forceinline__ void kbt_mell(float2 (&z)[64 / KP][BH], const float2* Xs2, long long nb, int nk2,
                                         int ld2, int nr, int W, int b0, const float2* MFs, const int* Cs) {
  constexpr int R = 64 / KP;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (r >= nr) continue;
    for (int w = 0; w < W; ++w) {
      const float2* xr = Xs2 + (long long)Cs[r * KB_WMAX + w] * ld2 * nb;
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
                                          const float2* Xs2, long long nb, int nk2, int ld2, int dm2, int i0, int nr,
                                          int d0, int W, int b0, const float2* MFs, const int* Cs, bool dia) {
  constexpr int RP = 32 / KP;
  if (dia) {
    const int nwin = nr + W - 1;
    for (int cw0 = 0; cw0 < nwin; cw0 += RP) {
      if (cw0 > 0 || !loaded) xw.load(Xs2, nb, nk2, ld2, dm2, i0 + d0 + cw0, nwin - cw0, b0);
      kbt_mdia<KP, MT>(z, xw, cw0, nr, W, MFs);
    }
  } else {
    kbt_mell<KP, MT>(z, Xs2, nb, nk2, ld2, nr, W, b0, MFs, Cs);
  }
}

// one term of a tensor-core tile: its tables and shared-memory staging
struct KbtTerm {
  int s2, nk2, ld2, dm2, W, Wst, d0, ktype, mtype;  // ld2: input row stride
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
  t.ld2 = __ldg(op.in_stride + t.s2);
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
  t.Xs2 = p.X + (long long)kb_slot(p.kslot) * p.slot_elems + (long long)__ldg(op.in_off + t.s2) * nb + v;
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
  if (t.mtype == 1) kbt_mstep<KP, 1>(z, xw, true, t.Xs2, nb, t.nk2, t.ld2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
  else if (t.mtype == 2) kbt_mstep<KP, 2>(z, xw, true, t.Xs2, nb, t.nk2, t.ld2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
  else kbt_mstep<KP, 0>(z, xw, true, t.Xs2, nb, t.nk2, t.ld2, t.dm2, i0, nr, t.d0, t.W, b0, MFs, Cs, t.dia);
}

// producer-only barrier (warps 0-7) that leaves the MMA warp out
template <int PT = 256>
__device__ __forceinline__ void kbt_producer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(PT) : "memory");
}

// MMAs of a term (one thread): per tile row r, D_re += Z_re K_re - Z_im K_im,
// D_im += Z_re K_im + Z_im K_re, each product as three TF32 MMAs per K step
// (A hi B hi, A hi B lo, A lo B hi); zero parts of K skipped.
// Per row, the MMAs into D_re, then those into D_im (runs on one accumulator).
template <int KP>
__device__ __forceinline__ void kbt_issue(uint32_t tmem, uint64_t adesc0, uint64_t bdesc, uint32_t idesc, int NP,
                                          int nr, int ktype, int nk2, uint32_t& dinit, int bpart = TC_BPART,
                                          int r0 = 0, int rs = 1) {
  constexpr int ATILE = 128 * KP;
  // (D part, A part, B part) of each product, D_re ones first
  int pd[4], pa[4], pb[4];
  int np = 0;
  if (ktype != 2) { pd[np] = 0; pa[np] = 0; pb[np] = 0; ++np; }  // re <- Z_re K_re
  if (ktype != 1) { pd[np] = 0; pa[np] = 2; pb[np] = 4; ++np; }  // re <- Z_im (-K_im)
  if (ktype != 2) { pd[np] = 1; pa[np] = 2; pb[np] = 0; ++np; }  // im <- Z_im K_re
  if (ktype != 1) { pd[np] = 1; pa[np] = 0; pb[np] = 2; ++np; }  // im <- Z_re K_im
  const int nks = (nk2 + 7) >> 3;
  for (int r = r0; r < nr; r += rs) {
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

// MMAs of one term with K_hi and K_lo merged along N (one thread): per row r
// and K step, Z_hi [K_hi; K_lo] (N = 2 NP) and Z_lo K_hi (N = NP) into a D
// region of 2 NP columns whose halves the epilogue adds: D_re at column
// 4 r NP, D_im at 4 r NP + 2 NP. KT: K real (1), imaginary (2) or complex (0).
// B parts (bpart bytes each, NP rows): K_re hi, lo; K_im hi, lo; -K_im hi, lo.
// acc0: 0 for the first committed term of the tile (fresh accumulators).
template <int KP, int KT>
__device__ __forceinline__ void kbt_issue_merged(uint32_t tmem, uint64_t adesc0, uint64_t bdesc, uint32_t id1,
                                                 uint32_t id2, int NP, int nr, int nk2, uint32_t acc0, int bpart,
                                                 int r0 = 0, int rs = 1) {
  constexpr uint64_t AP = (uint64_t)((128 * KP * 4) >> 4);  // descriptor step of one A part
  const uint64_t BP = (uint64_t)(bpart >> 4);               // of one B part
  const int nks = (nk2 + 7) >> 3;
  // per row (rows r0, r0 + rs, ...), all MMAs into D_re, then all into D_im:
  // runs of MMAs on one accumulator (faster than switching regions between MMAs)
  for (int r = r0; r < nr; r += rs) {
    const uint32_t dre = tmem + (uint32_t)(4 * r * NP), dim = dre + (uint32_t)(2 * NP);
    const uint64_t a = adesc0 + (uint64_t)(4 * r) * AP;
#pragma unroll
    for (int ks = 0; ks < KP / 8; ++ks) {
      if (ks >= nks) break;
      const uint32_t f = ks == 0 ? acc0 : 1u;
      const uint64_t ak = a + 16u * ks, bk = bdesc + 16u * ks;  // 8 K columns = 256 bytes
      if (KT != 2) {
        tc_mma_tf32(dre, ak + 0 * AP, bk + 0 * BP, id2, f);   // Z_re_hi [K_re_hi; K_re_lo]
        tc_mma_tf32(dre, ak + 1 * AP, bk + 0 * BP, id1, 1u);  // Z_re_lo K_re_hi
      }
      if (KT != 1) {
        tc_mma_tf32(dre, ak + 2 * AP, bk + 4 * BP, id2, KT == 2 ? f : 1u);  // Z_im_hi [-K_im_hi; -K_im_lo]
        tc_mma_tf32(dre, ak + 3 * AP, bk + 4 * BP, id1, 1u);               // Z_im_lo (-K_im_hi)
      }
    }
#pragma unroll
    for (int ks = 0; ks < KP / 8; ++ks) {
      if (ks >= nks) break;
      const uint32_t f = ks == 0 ? acc0 : 1u;
      const uint64_t ak = a + 16u * ks, bk = bdesc + 16u * ks;
      if (KT != 2) {
        tc_mma_tf32(dim, ak + 2 * AP, bk + 0 * BP, id2, f);   // Z_im_hi [K_re_hi; K_re_lo]
        tc_mma_tf32(dim, ak + 3 * AP, bk + 0 * BP, id1, 1u);  // Z_im_lo K_re_hi
      }
      if (KT != 1) {
        tc_mma_tf32(dim, ak + 0 * AP, bk + 2 * BP, id2, KT == 2 ? f : 1u);  // Z_re_hi [K_im_hi; K_im_lo]
        tc_mma_tf32(dim, ak + 1 * AP, bk + 2 * BP, id1, 1u);               // Z_re_lo K_im_hi
      }
    }
  }
}

// A tiles of tile row r: the real and imaginary parts of Z_r, each split into
// TF32 hi (rounded to nearest, ties away, by integer arithmetic on the bit
// pattern: finite values) and lo = value - hi, at K-major positions
template <int KP>
__device__ __forceinline__ void kbt_store_row(float* At, const float2 (&zr)[KP / 2], int vloc, int b0) {
  constexpr int ATILE = 128 * KP, BH = KP / 2;
#pragma unroll
  for (int c4 = 0; c4 < BH; c4 += 4) {
    float4 rh, rl, ih, il;
    float* prh = &rh.x;
    float* prl = &rl.x;
    float* pih = &ih.x;
    float* pil = &il.x;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2 zz = zr[c4 + q];
      const float2 hi = make_float2(__uint_as_float((__float_as_uint(zz.x) + 0x1000u) & 0xFFFFE000u),
                                    __uint_as_float((__float_as_uint(zz.y) + 0x1000u) & 0xFFFFE000u));
      const float2 lo = tc_fsub2(zz, hi);
      prh[q] = hi.x;
      prl[q] = lo.x;
      pih[q] = hi.y;
      pil[q] = lo.y;
    }
    const uint32_t o = tc_kmajor_off(vloc, b0 + c4, KP) >> 2;
    *reinterpret_cast<float4*>(At + 0 * ATILE + o) = rh;
    *reinterpret_cast<float4*>(At + 1 * ATILE + o) = rl;
    *reinterpret_cast<float4*>(At + 2 * ATILE + o) = ih;
    *reinterpret_cast<float4*>(At + 3 * ATILE + o) = il;
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
  // output rows ld1 elements apart; the pointer is formed where it is used
  auto y_rows = [&](int& ld1) {
    ld1 = __ldg(op.out_stride + s1);
    return p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * ld1) * nb + v;
  };
  const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
  if (te == tb) {  // no term reaches this slab
    if (producer) {
      int ld1;
      float2* Y = y_rows(ld1);
      for (int e = wid >> 2; e < nr * nk1; e += 2)
        Y[((long long)(e / nk1) * ld1 + e % nk1) * nb] = make_float2(0.f, 0.f);
    }
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
  if (cur.ok && !cur.empty && cur.dia) xw.load(cur.Xs2, nb, cur.nk2, cur.ld2, cur.dm2, i0 + cur.d0, nr + cur.W - 1, b0);
  kbt_stage<KP>(cur, nk1, NP, i0, nr, reinterpret_cast<float*>(Bs), MFs0, Cs0, tid);
  kbt_producer_sync();
  kbt_zstep<KP>(z, xw, cur, nb, i0, nr, b0, MFs0, Cs0);
  for (int term = tb; term < te; ++term) {
    const int buf = (term - tb) & 1;
    const bool has_next = term + 1 < te;
    KbtTerm nxt;
    if (has_next) {
      nxt = kbt_term(op, p, term + 1, KP, v, nb);
      if (nxt.ok && !nxt.empty && nxt.dia) xw.load(nxt.Xs2, nb, nxt.nk2, nxt.ld2, nxt.dm2, i0 + nxt.d0, nr + nxt.W - 1, b0);
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
  int ld1;
  float2* Y = y_rows(ld1);
  const float sc = p.yscale ? (float)p.yscale[(long long)kb_slot(p.kslot) * nb + v] : 1.f;
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
          Y[((long long)r * ld1 + c0 + q) * nb] = any ? make_float2(re[q] * sc, im[q] * sc) : make_float2(0.f, 0.f);
    }
  }
  if (!ok && lane == 0) atomicExch(p.err, KR_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
}


// ---------------------------------------------------------------------------
// X windows streamed by TMA (KP = 8, 16): the loader warp walks the window
// rows of every diagonal term in order and loads them two by two (each KP input
// columns x 128 vectors, KP/8 boxes of 8 columns) into a ring of shared-memory
// slots (full: tx bytes; empty: one arrival per producer warp; an odd window's
// last slot also carries the row after it); the producer warps read X from
// the ring, so no global-load latency sits in their M step. Rows outside the
// input slab read whatever lies there (finite data of other slabs, or zeros
// beyond the array) and meet zero MF slots. Terms stored as ELL load X
// directly. The layout below is shared by the persistent kernel (KbtPers).
// ---------------------------------------------------------------------------

template <int KP, bool TA = false>
struct KbtRing {
  // slots of two window rows of KP columns x 128 vectors x 8 bytes: with the A
  // tiles in TMEM (TA) the shared memory they took holds a ring about three
  // times as deep
  static constexpr int RS = 2;  // window rows per slot (4 with A in TMEM measured slower)
  static constexpr int NSLOT = TA ? (KP == 32 ? 2 : KP == 16 ? 5 : 11) : 32 / KP;
  static constexpr int ROW = KP * 1024;  // bytes of one window row in a slot
  static constexpr int SLOT = RS * ROW;
  static constexpr int BPART = 128 * KP;         // one B part: NP (<= 32) x KP FP32
  static constexpr int BBUF = 6 * BPART;
  static constexpr int OFF_B = TA ? 0 : TC_ABYTES;
  static constexpr int OFF_RING = OFF_B + 2 * BBUF;
  static constexpr int OFF_MF = OFF_RING + NSLOT * SLOT;
  static constexpr int OFF_CS = OFF_MF + TC_MFBYTES;
  // dense band of a diagonal term: [window row c][tile row r] float4
  // (m_re, m_re, -m_im, m_im) of MF[r, c - r], zero outside the band; two buffers
  static constexpr int R = 64 / KP;
  static constexpr int NWIN = R + KR_DIAG_MAX - 1;  // window rows of the widest band
  static constexpr int OFF_MFD = OFF_CS + TC_CSBYTES;
  static constexpr int MFD = NWIN * R;             // float4 entries of one buffer
};
static_assert(KbtRing<8>::MFD <= 256 && KbtRing<16>::MFD <= 256, "one dense-band entry per producer thread");

// M band of a term into a stage buffer (stager warp, its 32 lanes): for a
// diagonal term the dense band MFd[c][r] = (m_re, m_re, -m_im, m_im) of
// MF[i0 + r, c - r] (zero outside the band and below nr rows), else the ELL
// values and columns of the tile's rows
template <int KP>
__device__ __forceinline__ void kbt_stage_mf(const KbtTerm& t, int i0, int nr, float4* MFd, float2* MFs, int* Cs,
                                             int lane) {
  constexpr int R = 64 / KP;
  if (t.dia) {
    for (int e = lane; e < KbtRing<KP>::MFD; e += 32) {
      const int c = e / R, r = e - (e / R) * R, w = c - r;
      float2 m = make_float2(0.f, 0.f);
      if (r < nr && w >= 0 && w < t.W) m = __ldcg(t.mf + (long long)(i0 + r) * t.Wst + w);
      MFd[e] = make_float4(m.x, m.x, -m.y, m.y);
    }
  } else {
    for (int e = lane; e < nr * t.W; e += 32) {
      const int r = e / t.W, w = e - (e / t.W) * t.W;
      const long long src = (long long)(i0 + r) * t.Wst + w;
      MFs[r * KB_WMAX + w] = __ldcg(t.mf + src);
      Cs[r * KB_WMAX + w] = __ldg(t.col + src);
    }
  }
}


// the ring rows of one term: count, and the first input row (diagonal terms only)
__device__ __forceinline__ int kbt_ring_rows(const KbtTerm& t, int nr) {
  return (t.ok && !t.empty && t.dia) ? nr + t.W - 1 : 0;
}

// z += m x for one complex x and the band value m = (m_re, m_re, -m_im, m_im)
// of a real (MT 1), imaginary (2) or complex (0) M factor, as f32x2 FMAs
template <int MT>
__device__ __forceinline__ void macc2(float2& z, const float4& m, float2 x) {
  if (MT != 2) z = tc_ffma2(make_float2(m.x, m.y), x, z);
  if (MT != 1) z = tc_ffma2(make_float2(m.z, m.w), make_float2(x.y, x.x), z);
}

// position of the producers in the ring: the next row's slot and the phase
// parity that slot's full barrier completes with
struct KbtRingPos {
  int slot;
  uint32_t phase;
};
template <int NSLOT>
__device__ __forceinline__ void kbt_ring_next(KbtRingPos& rp) {
  if (++rp.slot == NSLOT) {
    rp.slot = 0;
    rp.phase ^= 1u;
  }
}

// takes the next ring slot: waits until it has landed, reads this thread's
// vector and BQ columns of its two rows (x[0], x[1]), and gives the slot back
// (one arrival per warp)
template <int KP, int BQ, int RS, int NSLOT>
__device__ __forceinline__ bool kbt_ring_take(float2 (&x)[RS][BQ], const char* ring, uint64_t* rfull,
                                              uint64_t* rempty, KbtRingPos& rp, int b0, int vloc, int lane) {
  const bool ok = tc_mbar_wait(rfull + rp.slot, rp.phase);
  const float2* xs = reinterpret_cast<const float2*>(ring + (size_t)rp.slot * RS * KP * 1024) + vloc;
#pragma unroll
  for (int h = 0; h < RS; ++h)
#pragma unroll
    for (int q = 0; q < BQ; ++q) x[h][q] = xs[h * KP * 128 + (b0 + q) * 128];
  __syncwarp();
  if (lane == 0) tc_mbar_arrive(rempty + rp.slot);
  kbt_ring_next<NSLOT>(rp);
  return ok;
}

// M step of a diagonal term from the ring. Window row c feeds tile rows
// r = c - W + 1 .. c through the dense band MFd[c][r] (zero outside the band);
// rows go in groups of G, a group skipped (warp-uniform) when the band misses
// it. Input columns at or beyond n_k2 hold finite data of the neighbouring rows
// and meet zero rows of K^T in the MMA.
template <int KP, int BH, int MT, int RS, int NSLOT>
__device__ __forceinline__ bool kbt_mdia_ring(float2 (&z)[64 / KP][BH], const char* ring, uint64_t* rfull,
                                              uint64_t* rempty, KbtRingPos& rp, int nwin, int nr, int W, int b0,
                                              int vloc, int lane, const float4* MFd) {
  constexpr int R = 64 / KP;
  constexpr int G = R >= 8 ? 2 : 1;
  bool ok = true;
  for (int c = 0; c < nwin; c += RS) {
    float2 x[RS][BH];
    if (!kbt_ring_take<KP, BH, RS, NSLOT>(x, ring, rfull, rempty, rp, b0, vloc, lane)) ok = false;
#pragma unroll
    for (int h = 0; h < RS; ++h) {
      const int cc = c + h;
      if (cc >= nwin) break;  // an odd window's last slot: its second row is not used
      const float4* mrow = MFd + cc * R;
#pragma unroll
      for (int gr = 0; gr < R / G; ++gr) {
        if (cc >= gr * G && cc < gr * G + G - 1 + W && gr * G < nr) {
#pragma unroll
          for (int rr = 0; rr < G; ++rr) {
            const int r = gr * G + rr;
            const float4 m = mrow[r];
#pragma unroll
            for (int q = 0; q < BH; ++q) macc2<MT>(z[r][q], m, x[h][q]);
          }
        }
      }
    }
  }
  return ok;
}

// the same for a band of WT slots (1, 3, 5), unrolled over the window: the
// band tests fold at compile time. Slots from row nwin on (tiles of fewer than
// R rows) are not taken; a slot's second row at or beyond nwin (an odd
// window) feeds only tile rows at or beyond nr, whose Z is never stored.
template <int KP, int BH, int MT, int WT, int RS, int NSLOT>
__device__ __forceinline__ bool kbt_mdia_ring_u(float2 (&z)[64 / KP][BH], const char* ring, uint64_t* rfull,
                                                uint64_t* rempty, KbtRingPos& rp, int nwin, int b0, int vloc,
                                                int lane, const float4* MFd) {
  constexpr int R = 64 / KP, NW = R + WT - 1;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < NW; c += RS) {
    if (c < nwin) {
      float2 x[RS][BH];
      if (!kbt_ring_take<KP, BH, RS, NSLOT>(x, ring, rfull, rempty, rp, b0, vloc, lane)) ok = false;
#pragma unroll
      for (int h = 0; h < RS; ++h) {
        const int cc = c + h;  // a row at or beyond nwin feeds only tile rows at or beyond nr
        if (cc >= NW) continue;
        const float4* mrow = MFd + cc * R;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r < cc - WT + 1 || r > cc) continue;
          const float4 m = mrow[r];
#pragma unroll
          for (int q = 0; q < BH; ++q) macc2<MT>(z[r][q], m, x[h][q]);
        }
      }
    }
  }
  return ok;
}

template <int KP, int BH, int MT, int RS, int NSLOT>
__device__ __forceinline__ bool kbt_mdia_ring_w(float2 (&z)[64 / KP][BH], const char* ring, uint64_t* rfull,
                                                uint64_t* rempty, KbtRingPos& rp, int nwin, int nr, int W, int b0,
                                                int vloc, int lane, const float4* MFd) {
  if (W == 5) return kbt_mdia_ring_u<KP, BH, MT, 5, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, b0, vloc, lane, MFd);
  if (W == 3) return kbt_mdia_ring_u<KP, BH, MT, 3, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, b0, vloc, lane, MFd);
  if (W == 1) return kbt_mdia_ring_u<KP, BH, MT, 1, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, b0, vloc, lane, MFd);
  return kbt_mdia_ring<KP, BH, MT, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, nr, W, b0, vloc, lane, MFd);
}

template <int KP, int BH, int RS, int NSLOT>
__device__ __forceinline__ bool kbt_zstep_ring(float2 (&z)[64 / KP][BH], const KbtTerm& t, long long nb, int nr,
                                               int b0, int vloc, int lane, const float2* MFs, const int* Cs,
                                               const float4* MFd, const char* ring, uint64_t* rfull,
                                               uint64_t* rempty, KbtRingPos& rp) {
  constexpr int R = 64 / KP;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int q = 0; q < BH; ++q) z[r][q] = make_float2(0.f, 0.f);
  if (!t.ok || t.empty) return true;
  const int nwin = kbt_ring_rows(t, nr);
  if (t.dia) {
    if (t.mtype == 1) return kbt_mdia_ring_w<KP, BH, 1, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, nr, t.W, b0, vloc, lane, MFd);
    if (t.mtype == 2) return kbt_mdia_ring_w<KP, BH, 2, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, nr, t.W, b0, vloc, lane, MFd);
    return kbt_mdia_ring_w<KP, BH, 0, RS, NSLOT>(z, ring, rfull, rempty, rp, nwin, nr, t.W, b0, vloc, lane, MFd);
  }
  if (t.mtype == 1) kbt_mell<KP, 1, BH>(z, t.Xs2, nb, t.nk2, t.ld2, nr, t.W, b0, MFs, Cs);
  else if (t.mtype == 2) kbt_mell<KP, 2, BH>(z, t.Xs2, nb, t.nk2, t.ld2, nr, t.W, b0, MFs, Cs);
  else kbt_mell<KP, 0, BH>(z, t.Xs2, nb, t.nk2, t.ld2, nr, t.W, b0, MFs, Cs);
  return true;
}


// ---------------------------------------------------------------------------
// Persistent form of the ring tile (KP = 8, 16): one CTA per SM loops over the
// work items (tile, block of 128 vectors) of one KP class, taken from a global
// counter in order (heaviest tiles first). Warp 9 takes the next item, writes
// its header and term table into one of two shared-memory buffers (ready: one
// arrival; free: the 8 producer warps and the MMA warp, once done with the
// tile) and streams the item's X window rows into the ring, running ahead of
// the producers across tiles. TMEM, barriers and the ring persist over the
// items; the commit count and the ring row counter run on. The first MMA of a
// tile starts its accumulators afresh.
// ---------------------------------------------------------------------------
constexpr int KBT_MAXT_P = 32;  // term table entries per buffer

template <int KP, bool TA = false>
struct KbtPers {
  using Rg = KbtRing<KP, TA>;
  static constexpr int NSLOT = Rg::NSLOT;
  static constexpr int OFF_BAR = Rg::OFF_MFD + 2 * Rg::MFD * 16;
  // full, empty, rfull[NSLOT], rempty[NSLOT], ready[2], free[2], staged[2],
  // sfree[2], TMEM slot
  static constexpr int OFF_HDR = OFF_BAR + 8 * (2 + 2 * NSLOT + 8) + 16;
  static constexpr int OFF_TAB = OFF_HDR + 2 * 8 * 4;
  static constexpr int TOTAL = OFF_TAB + 2 * KBT_MAXT_P * (int)sizeof(KbtTerm);
  // producer warps: 16 with the A tiles in TMEM (each thread a quarter of the
  // K columns of its vector), 8 with them in shared memory (a half); then the
  // MMA warp and the loader warp
  static constexpr int PW = TA ? 16 : 8;
  static constexpr int PT = 32 * PW;       // producer threads
  static constexpr int NQ = PW / 4;        // K-column groups per vector
  static constexpr int BQ = KP / NQ;       // K columns per producer thread
  // MMA warps: one thread of each issues the MMAs of tile rows r = j, j + NMW,
  // ... (a thread issues about one tcgen05.mma per 120 cycles whatever the
  // tile width; two issuers double that rate)
  static constexpr int NMW = 2;
  // then the loader warp (work items, term tables, X rows) and the stager warp
  // (each term's B operands and M band into one of two stage buffers)
  static constexpr int NT = PT + 32 * (NMW + 2);  // threads of the CTA
};
static_assert(KbtPers<8>::TOTAL <= 232448 && KbtPers<16>::TOTAL <= 232448, "persistent tile exceeds shared memory");
static_assert(KbtPers<8, true>::TOTAL <= 232448 && KbtPers<16, true>::TOTAL <= 232448 &&
                  KbtPers<32, true>::TOTAL <= 232448,
              "persistent tile (A in TMEM) exceeds shared memory");

// A tiles of tile row r in TMEM (the TA form): parts Z_re hi, lo, Z_im hi, lo,
// KP columns each, from column abase + 4 r KP; this thread's lane, its BH of
// the K columns (b0 .. b0 + BH). The TF32 split is the one of kbt_store_row.
template <int KP, int BH>
__device__ __forceinline__ void kbt_store_row_tmem(uint32_t arow, const float2 (&zr)[BH], int b0) {
  float rh[BH], rl[BH], ih[BH], il[BH];
#pragma unroll
  for (int q = 0; q < BH; ++q) {
    const float2 zz = zr[q];
    const float2 hi = make_float2(__uint_as_float((__float_as_uint(zz.x) + 0x1000u) & 0xFFFFE000u),
                                  __uint_as_float((__float_as_uint(zz.y) + 0x1000u) & 0xFFFFE000u));
    const float2 lo = tc_fsub2(zz, hi);
    rh[q] = hi.x;
    rl[q] = lo.x;
    ih[q] = hi.y;
    il[q] = lo.y;
  }
  const uint32_t c = arow + (uint32_t)b0;
  if constexpr (BH == 8) {
    tc_st8(c + 0 * KP, rh);
    tc_st8(c + 1 * KP, rl);
    tc_st8(c + 2 * KP, ih);
    tc_st8(c + 3 * KP, il);
  } else if constexpr (BH == 4) {
    tc_st4(c + 0 * KP, rh);
    tc_st4(c + 1 * KP, rl);
    tc_st4(c + 2 * KP, ih);
    tc_st4(c + 3 * KP, il);
  } else {
    static_assert(BH == 2, "2, 4 or 8 K columns per thread");
    tc_st2(c + 0 * KP, rh);
    tc_st2(c + 1 * KP, rl);
    tc_st2(c + 2 * KP, ih);
    tc_st2(c + 3 * KP, il);
  }
}

// kbt_issue_merged with the A tiles in TMEM (column atm + 4 r KP + part KP)
template <int KP, int KT>
__device__ __forceinline__ void kbt_issue_merged_ta(uint32_t tmem, uint32_t atm, uint64_t bdesc, uint32_t id1,
                                                    uint32_t id2, int NP, int nr, int nk2, uint32_t acc0,
                                                    int bpart, int r0, int rs) {
  const uint64_t BP = (uint64_t)(bpart >> 4);
  const int nks = (nk2 + 7) >> 3;
  for (int r = r0; r < nr; r += rs) {
    const uint32_t dre = tmem + (uint32_t)(4 * r * NP), dim = dre + (uint32_t)(2 * NP);
    const uint32_t a = atm + (uint32_t)(4 * r * KP);
#pragma unroll
    for (int ks = 0; ks < KP / 8; ++ks) {
      if (ks >= nks) break;
      const uint32_t f = ks == 0 ? acc0 : 1u;
      const uint32_t ak = a + 8u * ks;
      const uint64_t bk = bdesc + 16u * ks;
      if (KT != 2) {
        tc_mma_tf32_ta(dre, ak + 0 * KP, bk + 0 * BP, id2, f);
        tc_mma_tf32_ta(dre, ak + 1 * KP, bk + 0 * BP, id1, 1u);
      }
      if (KT != 1) {
        tc_mma_tf32_ta(dre, ak + 2 * KP, bk + 4 * BP, id2, KT == 2 ? f : 1u);
        tc_mma_tf32_ta(dre, ak + 3 * KP, bk + 4 * BP, id1, 1u);
      }
    }
#pragma unroll
    for (int ks = 0; ks < KP / 8; ++ks) {
      if (ks >= nks) break;
      const uint32_t f = ks == 0 ? acc0 : 1u;
      const uint32_t ak = a + 8u * ks;
      const uint64_t bk = bdesc + 16u * ks;
      if (KT != 2) {
        tc_mma_tf32_ta(dim, ak + 2 * KP, bk + 0 * BP, id2, f);
        tc_mma_tf32_ta(dim, ak + 3 * KP, bk + 0 * BP, id1, 1u);
      }
      if (KT != 1) {
        tc_mma_tf32_ta(dim, ak + 0 * KP, bk + 2 * BP, id2, KT == 2 ? f : 1u);
        tc_mma_tf32_ta(dim, ak + 1 * KP, bk + 2 * BP, id1, 1u);
      }
    }
  }
}

// kbt_issue (three MMAs per part and K step, D regions 2 r NP, D_re ones
// first) with the A tiles in TMEM
template <int KP>
__device__ __forceinline__ void kbt_issue_ta(uint32_t tmem, uint32_t atm, uint64_t bdesc, uint32_t idesc, int NP,
                                             int nr, int ktype, int nk2, uint32_t& dinit, int bpart, int r0,
                                             int rs) {
  const int nks = (nk2 + 7) >> 3;
  int pd[4], pa[4], pb[4];
  int np = 0;
  if (ktype != 2) { pd[np] = 0; pa[np] = 0; pb[np] = 0; ++np; }
  if (ktype != 1) { pd[np] = 0; pa[np] = 2; pb[np] = 4; ++np; }
  if (ktype != 2) { pd[np] = 1; pa[np] = 2; pb[np] = 0; ++np; }
  if (ktype != 1) { pd[np] = 1; pa[np] = 0; pb[np] = 2; ++np; }
  for (int r = r0; r < nr; r += rs) {
    for (int q = 0; q < np; ++q) {
      const uint32_t dcol = tmem + (uint32_t)((2 * r + pd[q]) * NP);
      const uint32_t dbit = 1u << (2 * r + pd[q]);
      const uint32_t ad = atm + (uint32_t)((r * 4 + pa[q]) * KP);
      const uint64_t bd = bdesc + (uint64_t)((pb[q] * bpart) >> 4);
#pragma unroll
      for (int sp = 0; sp < 3; ++sp) {
        const uint32_t a2 = ad + (sp == 2 ? (uint32_t)KP : 0u);
        const uint64_t b2 = bd + (sp == 1 ? (uint64_t)(bpart >> 4) : 0);
#pragma unroll
        for (int ks = 0; ks < KP / 8; ++ks) {
          if (ks < nks) {
            tc_mma_tf32_ta(dcol, a2 + 8u * ks, b2 + 16u * ks, idesc, (dinit & dbit) ? 1u : 0u);
            dinit |= dbit;
          }
        }
      }
    }
  }
}

template <int KP, bool TA>
__device__ void kbt_persist(const BatchTC& p, const CUtensorMap* xmap, char* smem) {
  using L = KbtPers<KP, TA>;
  using Rg = KbtRing<KP, TA>;
  constexpr int R = 64 / KP, BH = L::BQ, NSLOT = L::NSLOT, PW = L::PW, PT = L::PT;
  constexpr int ATILE = 128 * KP;
  const DevOp& op = p.op;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int vq = wid & 3, b0 = (wid >> 2) * BH;  // producers: lane quarter, first K column
  const int vloc = vq * 32 + lane;
  const long long nb = p.nb;
  float* As = reinterpret_cast<float*>(smem);
  char* Bs = smem + Rg::OFF_B;
  char* ring = smem + Rg::OFF_RING;
  float2* MFs0 = reinterpret_cast<float2*>(smem + Rg::OFF_MF);
  int* Cs0 = reinterpret_cast<int*>(smem + Rg::OFF_CS);
  float4* MFd0 = reinterpret_cast<float4*>(smem + Rg::OFF_MFD);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
  uint64_t* empty = full + 1;
  uint64_t* rfull = full + 2;
  uint64_t* rempty = rfull + NSLOT;
  uint64_t* tready = rempty + NSLOT;
  uint64_t* tfree = tready + 2;
  uint64_t* staged = tfree + 2;  // stage buffer g & 1 holds term g (B by bulk copy, M band)
  uint64_t* sfree = staged + 2;  // every producer warp is done with it (its term's MMAs included)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sfree + 2);
  int* hdr0 = reinterpret_cast<int*>(smem + L::OFF_HDR);  // [2][8]: item (-1: none), s1, i0, nr, vb, tb, te
  KbtTerm* tab0 = reinterpret_cast<KbtTerm*>(smem + L::OFF_TAB);
  // TMEM: the D regions of a tile (4 R NP <= 512 columns merged, else 2 R NP);
  // with TA, D in columns 0-255 (merged when 4 R NP <= 256) and the A tiles
  // (R rows x 4 parts x KP = 256 columns) from column TA_ACOL on
  constexpr uint32_t NCOLS = 512;
  constexpr uint32_t TA_ACOL = 256;
  constexpr int DMAX = TA ? 256 : 512;
  constexpr int NMW = L::NMW;
  if (wid == PW) tc_alloc(tslot, NCOLS);
  if (tid == PT) {
    tc_mbar_init(full, PW);
    tc_mbar_init(empty, NMW);  // one commit per MMA warp and term
    for (int i = 0; i < NSLOT; ++i) {
      tc_mbar_init(rfull + i, 1);
      tc_mbar_init(rempty + i, PW);
    }
    for (int b = 0; b < 2; ++b) {
      tc_mbar_init(tready + b, 1);
      tc_mbar_init(tfree + b, PW + NMW + 1);
      tc_mbar_init(staged + b, 1);
      tc_mbar_init(sfree + b, PW);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  const int nct = p.tend - p.tfirst;
  const int nwork = nct * p.nvb;

  if (wid == PW + NMW) {
    // ---- work items, term tables and X window loads -------------------------
    const int zslot = kb_slot(p.kslot);  // basis slot of X (third TMA coordinate)
    int g = 0;
    for (int it = 0;; ++it) {
      const int b = it & 1;
      if (it >= 2 && !tc_mbar_wait(tfree + b, (uint32_t)((it - 2) >> 1) & 1u)) ok = false;
      int w = 0;
      for (;;) {  // next item whose vector block has an active vector
        if (lane == 0) w = (int)atomicAdd(reinterpret_cast<unsigned*>(p.work), 1u);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= nwork || !p.grp_active) break;
        const int* gq = p.grp_active + 4 * (w / nct);
        if (gq[0] | gq[1] | gq[2] | gq[3]) break;
      }
      int* hdr = hdr0 + 8 * b;
      KbtTerm* tab = tab0 + KBT_MAXT_P * b;
      if (w >= nwork) {
        if (lane == 0) {
          hdr[0] = -1;
          tc_mbar_arrive(tready + b);
        }
        break;
      }
      const int task = p.tfirst + w % nct, vb = w / nct;
      const int s1 = __ldg(p.task + task);
      const int i0 = __ldg(p.task + p.ntask + task);
      const int nr = __ldg(p.task + 2 * p.ntask + task);
      const int tb = __ldg(op.term_ptr + s1), te = __ldg(op.term_ptr + s1 + 1);
      for (int j = lane; j < te - tb && j < KBT_MAXT_P; j += 32) tab[j] = kbt_term(op, p, tb + j, KP, 0, nb);
      if (lane == 0) {
        hdr[0] = w;
        hdr[1] = s1;
        hdr[2] = i0;
        hdr[3] = nr;
        hdr[4] = vb;
        hdr[5] = tb;
        hdr[6] = te;
      }
      __syncwarp();
      if (lane == 0) {
        tc_mbar_arrive(tready + b);  // release: the header and table above
        for (int term = tb; term < te; ++term) {
          const KbtTerm t = (term - tb < KBT_MAXT_P) ? tab[term - tb] : kbt_term(op, p, term, KP, 0, nb);
          const int nwin = kbt_ring_rows(t, nr);
          const long long row0 = __ldg(op.in_off + t.s2);
          for (int c = 0; c < nwin; c += Rg::RS, ++g) {  // RS window rows per slot
            const int slot = g % NSLOT;
            if (g >= NSLOT && !tc_mbar_wait(rempty + slot, (uint32_t)(g / NSLOT - 1) & 1u)) ok = false;
            // both rows of the slot, also past an odd window's end (a row
            // outside the slot's basis array reads as zeros; the producers'
            // FMAs on such a row reach no stored Z)
            tc_mbar_expect_tx(rfull + slot, (uint32_t)Rg::SLOT);
            for (int rr = 0; rr < Rg::RS; ++rr) {
              const long long y = row0 + (long long)(i0 + t.d0 + c + rr) * t.ld2;
              char* dst = ring + (size_t)slot * Rg::SLOT + rr * Rg::ROW;
#pragma unroll
              for (int h = 0; h < KP / 8; ++h)
                tc_tma_load_3d(dst + h * 8192, xmap, vb * 128, (int)(y + 8 * h), zslot, rfull + slot);
            }
          }
        }
      }
      __syncwarp();
    }
  } else if (wid == PW + NMW + 1) {
    // ---- stage buffers: term g's B operands (one bulk copy of its prebuilt
    // block) and M band into buffer g & 1, once the producers gave it back ----
    int g = 0;
    for (int it = 0;; ++it) {
      const int b = it & 1;
      if (!tc_mbar_wait(tready + b, (uint32_t)(it >> 1) & 1u)) {
        ok = false;
        break;
      }
      const int* hdr = hdr0 + 8 * b;
      if (hdr[0] < 0) break;
      const int s1 = hdr[1], i0 = hdr[2], nr = hdr[3], tb = hdr[5], te = hdr[6];
      const KbtTerm* tab = tab0 + KBT_MAXT_P * b;
      const int NP = __ldg(op.out_dk + s1) <= 16 ? 16 : 32;
      const uint32_t bbytes = (uint32_t)(6 * NP * KP * 4);
      for (int term = tb; term < te; ++term, ++g) {
        const int buf = g & 1;
        if (g >= 2 && !tc_mbar_wait(sfree + buf, (uint32_t)((g - 2) >> 1) & 1u)) ok = false;
        const KbtTerm tt = (term - tb < KBT_MAXT_P) ? tab[term - tb] : kbt_term(op, p, term, KP, 0, nb);
        const bool live = tt.ok && !tt.empty;
        if (live)
          kbt_stage_mf<KP>(tt, i0, nr, MFd0 + buf * Rg::MFD, MFs0 + buf * 8 * KB_WMAX, Cs0 + buf * 8 * KB_WMAX, lane);
        __syncwarp();
        if (lane == 0) {
          if (live) {
            tc_mbar_expect_tx(staged + buf, bbytes);
            tc_bulk_load(Bs + buf * Rg::BBUF, p.tcb + __ldg(p.tcb_off + term), bbytes, staged + buf);
          } else {
            tc_mbar_arrive(staged + buf);
          }
        }
      }
      __syncwarp();
      if (lane == 0) tc_mbar_arrive(tfree + b);
    }
  } else if (wid >= PW) {
    // ---- MMA issue: warp PW + j takes tile rows j, j + NMW, ... ------------------
    const int r0 = wid - PW;
    int ncommit = 0;
    int g = 0;  // term counter (stage buffer g & 1)
    const uint64_t adesc0 = tc_desc(tc_smem_u32(As), 128u, 32u * KP);
    const uint64_t bdesc0 = tc_desc(tc_smem_u32(Bs), 128u, 32u * KP);
    for (int it = 0;; ++it) {
      const int b = it & 1;
      if (!tc_mbar_wait(tready + b, (uint32_t)(it >> 1) & 1u)) {
        ok = false;
        break;
      }
      const int* hdr = hdr0 + 8 * b;
      if (hdr[0] < 0) break;
      const int s1 = hdr[1], nr = hdr[3], tb = hdr[5], te = hdr[6];
      const KbtTerm* tab = tab0 + KBT_MAXT_P * b;
      if (lane == 0) {
        const int nk1 = __ldg(op.out_dk + s1);
        const int NP = nk1 <= 16 ? 16 : 32;
        const bool merged = 4 * R * NP <= DMAX;
        const int bpart = NP * KP * 4;  // the prebuilt blocks' part stride
        const uint32_t idesc = tc_idesc_tf32(128, NP), idesc2 = tc_idesc_tf32(128, 2 * NP);
        const int c0 = ncommit;
        uint32_t dinit = 0;
        for (int term = tb; term < te; ++term, ++g) {
          const KbtTerm tt = (term - tb < KBT_MAXT_P) ? tab[term - tb] : kbt_term(op, p, term, KP, 0, nb);
          if (!tt.ok || tt.empty) continue;  // skipped by the producers as well
          if (!tc_mbar_wait(full, (uint32_t)ncommit & 1u)) ok = false;
          tc_fence_after();
          const uint64_t bdesc = bdesc0 + (uint64_t)(((g & 1) * Rg::BBUF) >> 4);
          if constexpr (TA) {
            const uint32_t atm = tmem + TA_ACOL;
            if (merged) {
              const uint32_t acc0 = ncommit > c0 ? 1u : 0u;
              if (tt.ktype == 1) kbt_issue_merged_ta<KP, 1>(tmem, atm, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
              else if (tt.ktype == 2) kbt_issue_merged_ta<KP, 2>(tmem, atm, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
              else kbt_issue_merged_ta<KP, 0>(tmem, atm, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
            } else {
              kbt_issue_ta<KP>(tmem, atm, bdesc, idesc, NP, nr, tt.ktype, tt.nk2, dinit, bpart, r0, NMW);
            }
          } else if (merged) {
            const uint32_t acc0 = ncommit > c0 ? 1u : 0u;
            if (tt.ktype == 1) kbt_issue_merged<KP, 1>(tmem, adesc0, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
            else if (tt.ktype == 2) kbt_issue_merged<KP, 2>(tmem, adesc0, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
            else kbt_issue_merged<KP, 0>(tmem, adesc0, bdesc, idesc, idesc2, NP, nr, tt.nk2, acc0, bpart, r0, NMW);
          } else {
            kbt_issue<KP>(tmem, adesc0, bdesc, idesc, NP, nr, tt.ktype, tt.nk2, dinit, bpart, r0, NMW);
          }
          tc_commit(empty);  // arrives once this thread's MMAs (if any) are done
          ++ncommit;
        }
      }
      ncommit = __shfl_sync(0xffffffffu, ncommit, 0);
      g = __shfl_sync(0xffffffffu, g, 0);
      __syncwarp();
      if (lane == 0) tc_mbar_arrive(tfree + b);
    }
  } else {
    // ---- producers ---------------------------------------------------------------
    int ncommit = 0;
    KbtRingPos rp{0, 0u};
    float2 z[R][BH];
    int g = 0;     // term counter: stage buffer g & 1
    int rel = -1;  // term whose stage buffer goes back once its MMAs are seen done
    // gives the stage buffer of term gg back to the stager (one arrival per warp)
    auto release = [&](int gg) {
      __syncwarp();
      if (lane == 0) tc_mbar_arrive(sfree + (gg & 1));
    };
    for (int it = 0;; ++it) {
      const int b = it & 1;
      if (!tc_mbar_wait(tready + b, (uint32_t)(it >> 1) & 1u)) {
        ok = false;
        break;
      }
      const int* hdr = hdr0 + 8 * b;
      if (hdr[0] < 0) break;
      const int s1 = hdr[1], i0 = hdr[2], nr = hdr[3], vb = hdr[4], tb = hdr[5], te = hdr[6];
      const KbtTerm* tab = tab0 + KBT_MAXT_P * b;
      const int v = vb * 128 + vloc;
      auto term_at = [&](int i) {
        KbtTerm tt = (i < KBT_MAXT_P) ? tab[i] : kbt_term(op, p, tb + i, KP, 0, nb);
        tt.Xs2 += v;
        return tt;
      };
      const int nk1 = __ldg(op.out_dk + s1);
      const int ld1 = __ldg(op.out_stride + s1);
      float2* Y = p.Y + ((long long)__ldg(op.out_off + s1) + (long long)i0 * ld1) * nb + v;
      const float sc = p.yscale ? (float)p.yscale[(long long)kb_slot(p.kslot) * nb + v] : 1.f;
      const int NP = nk1 <= 16 ? 16 : 32;
      const bool merged = 4 * R * NP <= DMAX;
      if (te == tb) {  // no term reaches this slab
        for (int e = wid >> 2; e < nr * nk1; e += L::NQ)
          Y[((long long)(e / nk1) * ld1 + e % nk1) * nb] = make_float2(0.f, 0.f);
        __syncwarp();
        if (lane == 0) tc_mbar_arrive(tfree + b);
        continue;
      }
      const int c0 = ncommit;
      // M step of the term in stage buffer g & 1, once the stager filled it
      auto zstep = [&](const KbtTerm& t) {
        const int sb = g & 1;
        if (!tc_mbar_wait(staged + sb, (uint32_t)(g >> 1) & 1u)) ok = false;
        if (!kbt_zstep_ring<KP, BH, Rg::RS, L::NSLOT>(z, t, nb, nr, b0, vloc, lane, MFs0 + sb * 8 * KB_WMAX,
                                              Cs0 + sb * 8 * KB_WMAX, MFd0 + sb * Rg::MFD, ring, rfull, rempty, rp))
          ok = false;
      };
      KbtTerm cur = term_at(0);
      zstep(cur);
      for (int term = tb; term < te; ++term) {
        const bool has_next = term + 1 < te;
        // the MMAs of the last committed term are done: the A tiles are free,
        // and that term's stage buffer goes back
        if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
        tc_fence_after();
        if (rel >= 0) {
          release(rel);
          rel = -1;
        }
        if (cur.ok && !cur.empty) {
          if constexpr (TA) {
            const uint32_t arow = tmem + TA_ACOL + ((uint32_t)(vq * 32) << 16);
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (r < nr) kbt_store_row_tmem<KP, BH>(arow + (uint32_t)(4 * r * KP), z[r], b0);
            tc_wait_st();
            tc_fence_before();
          } else {
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (r < nr) kbt_store_row<KP>(As + r * 4 * ATILE, z[r], vloc, b0);
          }
          tc_fence_proxy();  // the A tiles (shared-memory form) to the async proxy
          __syncwarp();
          if (lane == 0) tc_mbar_arrive(full);
          ++ncommit;
          rel = g;
        } else {
          if (!cur.ok && tid == 0) atomicExch(p.err, KR_ERR_ARG);  // outside the tile shape: skipped
          release(g);  // no MMA reads this term's buffer
        }
        if (has_next) {
          ++g;
          cur = term_at(term + 1 - tb);
          zstep(cur);
        }
      }
      ++g;
      if (ncommit > 0 && !tc_mbar_wait(empty, (uint32_t)(ncommit - 1) & 1u)) ok = false;
      tc_fence_after();
      if (rel >= 0) {
        release(rel);
        rel = -1;
      }
      const bool any = ncommit > c0;
      for (int r = wid >> 2; r < nr; r += L::NQ) {
        for (int cc = 0; cc < NP; cc += 16) {
          float re[16], im[16];
          const uint32_t lanebase = (uint32_t)(vq * 32) << 16;
          if (merged) {
            float re2[16], im2[16];
            tc_ld16(tmem + lanebase + (uint32_t)(4 * r * NP + cc), re);
            tc_ld16(tmem + lanebase + (uint32_t)(4 * r * NP + NP + cc), re2);
            tc_ld16(tmem + lanebase + (uint32_t)(4 * r * NP + 2 * NP + cc), im);
            tc_ld16(tmem + lanebase + (uint32_t)(4 * r * NP + 3 * NP + cc), im2);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              re[q] += re2[q];
              im[q] += im2[q];
            }
          } else {
            tc_ld16(tmem + lanebase + (uint32_t)(2 * r * NP + cc), re);
            tc_ld16(tmem + lanebase + (uint32_t)((2 * r + 1) * NP + cc), im);
          }
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (cc + q < nk1)
              Y[((long long)r * ld1 + cc + q) * nb] = any ? make_float2(re[q] * sc, im[q] * sc) : make_float2(0.f, 0.f);
        }
      }
      tc_fence_before();  // the TMEM reads above come before the next tile's MMAs
      __syncwarp();
      if (lane == 0) tc_mbar_arrive(tfree + b);
    }
  }
  if (!ok && lane == 0) atomicExch(p.err, KR_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (wid == PW) tc_dealloc(tmem, NCOLS);
}

template <int KP, bool TA>
__global__ void __launch_bounds__(KbtPers<KP, TA>::NT, 1) kb_matvec_tcp(BatchTC p,
                                                                       const __grid_constant__ CUtensorMap xmap) {
  extern __shared__ __align__(1024) char kbt_smem[];
  kbt_persist<KP, TA>(p, &xmap, kbt_smem);
}

__global__ void __launch_bounds__(320, 1) kb_matvec_tc(BatchTC p, const __grid_constant__ CUtensorMap xmap) {
  extern __shared__ __align__(1024) char kbt_smem[];
  if (p.grp_active) {
    const int* g = p.grp_active + 4 * blockIdx.y;
    if (!(g[0] | g[1] | g[2] | g[3])) return;
  }
  const int task = p.tfirst + blockIdx.x;
  const int s1 = __ldg(p.task + task);
  const int i0 = __ldg(p.task + p.ntask + task);
  const int nr = __ldg(p.task + 2 * p.ntask + task);
  const int kp = __ldg(p.task + 3 * p.ntask + task);
  if (kp == 32) kbt_tile<32>(p, s1, i0, nr, kbt_smem);
  else if (threadIdx.x == 0) atomicExch(p.err, KR_ERR_ARG);  // KP = 8, 16 tiles go to kb_matvec_tcp
}

// ---------------------------------------------------------------------------
// B operands of every term of the persistent tiles, built once per operator
// (K does not change with the field): per term, the six parts K_re hi, lo,
// K_im hi, lo, -K_im hi, lo (TF32 split of the FP32 copy of K), each NP x KP
// in the K-major layout of the MMA, NP x KP x 4 bytes apart. A stager warp of
// the persistent kernel copies a term's block into shared memory in one bulk
// copy. prm: [6][nterm] int64 = K offset, K type, n_k1, n_k2, KP (0: none), B offset.
// ---------------------------------------------------------------------------
__global__ void kbt_build_b(const float* __restrict__ kf32, const long long* __restrict__ prm, int nterm,
                            float* __restrict__ tcb) {
  const int t = blockIdx.x;
  const int KP = (int)prm[4 * nterm + t];
  if (KP == 0) return;
  const float* KT = kf32 + prm[t];
  const int ktype = (int)prm[nterm + t], nk1 = (int)prm[2 * nterm + t], nk2 = (int)prm[3 * nterm + t];
  const int NP = nk1 <= 16 ? 16 : 32;
  const int part = NP * KP;
  float* Bt = tcb + prm[5 * nterm + t];
  for (int e = threadIdx.x; e < NP * KP; e += blockDim.x) {
    const int a = e / KP, b = e - (e / KP) * KP;
    float kr = 0.f, ki = 0.f;
    if (a < nk1 && b < nk2) {
      if (ktype == 0) {
        kr = KT[((long long)b * nk1 + a) * 2];
        ki = KT[((long long)b * nk1 + a) * 2 + 1];
      } else if (ktype == 1) {
        kr = KT[(long long)b * nk1 + a];
      } else {
        ki = KT[(long long)b * nk1 + a];
      }
    }
    const uint32_t o = tc_kmajor_off(a, b, KP) >> 2;
    const float krh = tc_tf32(kr), kih = tc_tf32(ki);
    Bt[0 * part + o] = krh;
    Bt[1 * part + o] = kr - krh;
    Bt[2 * part + o] = kih;
    Bt[3 * part + o] = ki - kih;
    Bt[4 * part + o] = -kih;
    Bt[5 * part + o] = -(ki - kih);
  }
}

int kb_build_tc_b(kr_ctx* ctx, const float* kf32, const long long* prm, int nterm, float* tcb) {
  if (nterm <= 0) return KR_OK;
  kbt_build_b<<<nterm, 256>>>(kf32, prm, nterm, tcb);
  KR_CUDA(ctx, cudaGetLastError());
  return KR_OK;
}

// TMA descriptor of the basis slots behind X, [nslots][dim][nb] (complex64 as
// 8-byte elements): boxes of 128 vectors x 8 rows of one slot, zero fill
// outside the slot's rows (a window never reads into the next slot)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static int encode_xmap(kr_ctx* ctx, const float2* X, long long dim, int nb, int nslots, CUtensorMap* m) {
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
  const cuuint64_t gdim[3] = {(cuuint64_t)nb, (cuuint64_t)dim, (cuuint64_t)std::max(1, nslots)};
  const cuuint64_t gstride[2] = {(cuuint64_t)nb * sizeof(float2), (cuuint64_t)dim * nb * sizeof(float2)};
  const cuuint32_t box[3] = {128, 8, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<float2*>(X), gdim, gstride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(ctx, KR_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return KR_OK;
}

int kb_launch_tc(kr_ctx* ctx, const BatchTC& p, long long dim, const int* cls, int* work, bool tmem_a,
                 cudaStream_t st) {
  CUtensorMap xmap;
  const int rc = encode_xmap(ctx, p.X, dim, p.nb, p.nslots, &xmap);
  if (rc != KR_OK) return rc;
  const int nvb = p.nb / 128;
  KR_CUDA(ctx, cudaMemsetAsync(work, 0, 3 * sizeof(int), st));
  // persistent launches, one per KP class (8, 16, and 32 with the A tiles in
  // TMEM): one CTA per SM at most
  for (int c = 0; c < (tmem_a ? 3 : 2); ++c) {
    const int n = cls[c + 1] - cls[c];
    if (n <= 0) continue;
    BatchTC q = p;
    q.tfirst = cls[c];
    q.tend = cls[c + 1];
    q.nvb = nvb;
    q.work = work + c;
    const int grid = (int)std::min<long long>((long long)n * nvb, ctx->nsm);
    if (tmem_a) {
      if (c == 0) {
        KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tcp<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          KbtPers<8, true>::TOTAL));
        kb_matvec_tcp<8, true><<<grid, KbtPers<8, true>::NT, KbtPers<8, true>::TOTAL, st>>>(q, xmap);
      } else if (c == 2) {
        KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tcp<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          KbtPers<32, true>::TOTAL));
        kb_matvec_tcp<32, true><<<grid, KbtPers<32, true>::NT, KbtPers<32, true>::TOTAL, st>>>(q, xmap);
      } else {
        KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tcp<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          KbtPers<16, true>::TOTAL));
        kb_matvec_tcp<16, true><<<grid, KbtPers<16, true>::NT, KbtPers<16, true>::TOTAL, st>>>(q, xmap);
      }
    } else if (c == 0) {
      KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tcp<8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        KbtPers<8>::TOTAL));
      kb_matvec_tcp<8, false><<<grid, KbtPers<8>::NT, KbtPers<8>::TOTAL, st>>>(q, xmap);
    } else {
      KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tcp<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        KbtPers<16>::TOTAL));
      kb_matvec_tcp<16, false><<<grid, KbtPers<16>::NT, KbtPers<16>::TOTAL, st>>>(q, xmap);
    }
    KR_CUDA(ctx, cudaGetLastError());
  }
  // KP = 32 with the A tiles in shared memory: one CTA per tile and vector block
  const int n32 = cls[3] - cls[2];
  if (n32 > 0 && !tmem_a) {
    BatchTC q = p;
    q.tfirst = cls[2];
    q.tend = cls[3];
    q.nvb = nvb;
    const int smem = TC_SMEM;
    KR_CUDA(ctx, cudaFuncSetAttribute(kb_matvec_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kb_matvec_tc<<<dim3(n32, nvb), 320, smem, st>>>(q, xmap);
    KR_CUDA(ctx, cudaGetLastError());
  }
  return KR_OK;
}

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

// the same product with A in TMEM (written by tcgen05.st, row m in lane m):
// the operand path of MMAs whose A comes from registers of the lane's thread
__global__ void __launch_bounds__(128) kb_mma_probe_ta(const float* A, const float* B, float* D, int* err) {
  __shared__ __align__(128) float sb[16 * 16];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  for (int e = tid; e < 16 * 16; e += 128) sb[tc_kmajor_off(e >> 4, e & 15, 16) >> 2] = B[e];
  if (wid == 0) tc_alloc(&tbase, 64);
  if (tid == 0) tc_mbar_init(&bar, 1);
  tc_fence_proxy();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = tbase;
  const uint32_t lanebase = (uint32_t)(32 * wid) << 16;
  float a[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) a[j] = A[(32 * wid + lane) * 16 + j];
  tc_st8(taddr + lanebase + 32u, a);
  tc_st8(taddr + lanebase + 40u, a + 8);
  tc_wait_st();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid == 0) {
    const uint32_t idesc = tc_idesc_tf32(128, 16);
    for (int s = 0; s < 2; ++s)  // K = 16 in two steps of 8
      tc_mma_tf32_ta(taddr, taddr + 32u + 8u * s, tc_desc(tc_smem_u32(sb) + 256u * s, 128u, 512u), idesc,
                     (uint32_t)s);
    tc_commit(&bar);
  }
  if (!tc_mbar_wait(&bar, 0) && lane == 0) atomicExch(err, KR_ERR_TIMEOUT);
  tc_fence_after();
  float v[16];
  tc_ld16(taddr + lanebase, v);
#pragma unroll
  for (int j = 0; j < 16; ++j) D[(32 * wid + lane) * 16 + j] = v[j];
  tc_fence_before();
  __syncthreads();
  if (wid == 0) tc_dealloc(taddr, 64);
}

extern "C" int kr_probe_mma_ta(kr_ctx* ctx, const float* a, const float* b, float* d) {
  if (!ctx || !a || !b || !d) return set_err(ctx, KR_ERR_ARG, "kr_probe_mma_ta: NULL argument");
  KR_DEVICE_SCOPE(ctx, ctx->device);
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
    kb_mma_probe_ta<<<1, 128>>>(dA, dB, dD, derr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(d, dD, sizeof(float) * nd, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(buf);
  KR_CUDA(ctx, e);
  if (herr) return set_err(ctx, herr, "kr_probe_mma_ta: MMA completion wait gave up");
  return KR_OK;
}

extern "C" int kr_probe_mma(kr_ctx* ctx, const float* a, const float* b, float* d) {
  if (!ctx || !a || !b || !d) return set_err(ctx, KR_ERR_ARG, "kr_probe_mma: NULL argument");
  KR_DEVICE_SCOPE(ctx, ctx->device);
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
