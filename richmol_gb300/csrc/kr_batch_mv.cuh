// Batched mat-vec Y = H X over vector-minor [dim][nb] complex64 arrays: the
// argument blocks and launchers of its two implementations, the SIMT FP32 one
// (kr_batch_simt.cu) and the tensor-core one (kr_batch_tc.cu), used by the
// batch driver (kr_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include "kr_internal.cuh"

#define KB_WMAX 16   // ELL width of the M band supported by the batched mat-vec

// Basis slot a mat-vec reads: X (and yscale) are the base of an array of
// basis slots of slot_elems elements (nb per row); with kslot non-null the
// slot is the device-side Krylov index *kslot (read at launch, so a recorded
// step needs no host-side index), else slot 0.
__device__ __forceinline__ int kb_slot(const int* kslot) { return kslot ? __ldg(kslot) : 0; }

// arguments of the SIMT mat-vec kb_matvec (kr_batch_simt.cu)
struct BatchMV {
  DevOp op;
  const float2* X;
  float2* Y;
  int nb;
  const int* kslot;       // device Krylov index: basis slot of X and yscale (null: slot 0)
  long long slot_elems;   // elements of one basis slot (dim * nb)
  const int* task_slab;
  const int* task_i0;
  const int* task_nr;
  const int* grp_active;  // per 32-vector group: any vector active (null: all)
  const double* yscale;   // per vector: output scale (null: 1)
  int* err;               // error word (a term outside the tile shape), or null
};

// arguments of the tensor-core mat-vec kb_matvec_tc (kr_batch_tc.cu)
struct BatchTC {
  DevOp op;
  const float2* X;
  float2* Y;
  int nb;
  const int* kslot;       // device Krylov index: basis slot of X and yscale (null: slot 0)
  long long slot_elems;   // elements of one basis slot (dim * nb)
  int nslots;             // basis slots behind X (extent of the TMA descriptor)
  const int* task;        // [4][ntask]: slab, first row, rows, KP
  int ntask;
  int tfirst;             // first tile of this launch in task (per-tile kernel: tile tfirst + blockIdx.x)
  int tend;               // persistent kernel: tiles [tfirst, tend) x vector blocks
  int nvb;                // vector blocks of 128
  int* work;              // persistent kernel: work-item counter (zero at launch)
  const int* grp_active;  // per 32-vector group: any vector active (null: all)
  const double* yscale;   // per vector: output scale (null: 1)
  const float* tcb;       // B operands of the persistent tiles' terms (kb_build_tc_b)
  const long long* tcb_off;  // per term: first float of its B block
  int* err;
};

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

// launch kb_matvec over the tile table (ntask tiles x ngrp 32-vector groups)
int kb_launch_simt(kr_ctx* ctx, const BatchMV& p, int ntask, int ngrp, cudaStream_t st);
// launch the tensor-core mat-vec over its tile table: the tiles of KP = 8 and
// 16 (cls[0] .. cls[2]) as one persistent launch per class (work counters
// work[0], work[1], zeroed here), the KP = 32 tiles (cls[2] .. cls[3]) one CTA
// per tile and vector block; encodes the TMA descriptor of p.X (p.nslots
// slots of [dim][nb] complex64)
// tmem_a: the persistent launches keep their A tiles in tensor memory (written by
// tcgen05.st; the shared memory holds a deeper TMA ring), else in shared memory
int kb_launch_tc(kr_ctx* ctx, const BatchTC& p, long long dim, const int* cls, int* work, bool tmem_a,
                 cudaStream_t st);

// launch the register-tiled FP32 mat-vec kb_matvec_zr (kr_batch_zr.cu) over
// its tile table (op->zr_task: [4][ntask] slab, first row, rows, NKP; the
// tiles of NKP = 8, 16, 32 from cls[0], cls[1], cls[2] to cls[3]) x ngrp
// 32-vector groups, one launch per NKP class
int kb_launch_zr(kr_ctx* ctx, const BatchMV& p, const int* task, int ntask, const int* cls, int ngrp,
                 cudaStream_t st);
