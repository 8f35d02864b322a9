// Host/device structures shared by the translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/richmol_gb300.h"
#include "kr_device.cuh"

// field coefficients of up to KR_PART_INLINE parts, passed as kernel parameters
#define KR_PART_INLINE 16
struct FieldCoef {
  int npart;
  double2 coef[KR_PART_INLINE][KR_MAXCART];
  double2 scale[KR_PART_INLINE];
  double thresh[KR_PART_INLINE];
  __device__ __forceinline__ double2 c(int p, int ci) const { return coef[p][ci]; }
  __device__ __forceinline__ double2 s(int p) const { return scale[p]; }
  __device__ __forceinline__ double t(int p) const { return thresh[p]; }
};
// the same for more parts, from device memory: [npart][KR_MAXCART], [npart], [npart]
struct FieldCoefDev {
  const double2* coef;
  const double2* scale;
  const double* thresh;
  __device__ __forceinline__ double2 c(int p, int ci) const { return __ldg(coef + p * KR_MAXCART + ci); }
  __device__ __forceinline__ double2 s(int p) const { return __ldg(scale + p); }
  __device__ __forceinline__ double t(int p) const { return __ldg(thresh + p); }
};

struct DevField {
  long long nent;
  int nmf;
  const signed char* m_ctype;   // [group][KR_MAXCART]: 0 mixed, 1 real, 2 imaginary, 3 all zero
  int* mf_type;                 // out: per MF instance 0 complex, 1 real, 2 imaginary
  const int* ent_inst;          // MF instance of each entry
  const long long* inst_ptr;    // first entry of each instance
  const int* mf_group; const int* mf_part;
  const long long* m_val_off; const int* m_ncart; const int* m_rows; const int* m_width;
  const double2* m_val;
  double2* mf_val;
  float2* mf_f32;
  float2* mf_lo;
  int* mf_band;                 // out: per MF instance [W - 1 - lowest, highest] slot with a non-zero value (-1: none)
};

struct kr_ctx {
  int device = 0;
  int nsm = 0;
  std::string err;
};

// records the error message of a failed call (per context and library-wide)
int kr_set_err(kr_ctx* ctx, int code, const std::string& msg);

// Held while the library records a step into a CUDA graph and while it creates
// or frees device objects (allocation, frees, device-wide synchronisation),
// so that, with several host threads driving one GPU, none of the library's
// own allocations or synchronisations runs in the middle of a recording.
std::recursive_mutex& kr_device_mutex();

// fills the B blocks of the persistent tensor-core tiles' terms (kr_batch_tc.cu);
// prm: [6][nterm] int64 = K offset, K type, n_k1, n_k2, KP (0: no block), B offset
int kb_build_tc_b(kr_ctx* ctx, const float* kf32, const long long* prm, int nterm, float* tcb);
#define set_err kr_set_err

#define KR_CUDA(ctx, call)                                                                 \
  do {                                                                                     \
    cudaError_t _e = (call);                                                               \
    if (_e != cudaSuccess)                                                                 \
      return set_err((ctx), KR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Makes a device current for the rest of a call and gives the caller's current
// device back when the call returns (on every path), so no entry point leaves
// a side effect on the calling thread's device.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) err = cudaSetDevice(dev);
  }
  ~DeviceScope() {
    if (prev >= 0 && err == cudaSuccess) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};
#define KR_DEVICE_SCOPE(ctx, dev) \
  DeviceScope _kr_dev_scope(dev); \
  KR_CUDA(ctx, _kr_dev_scope.err)

struct kr_op {
  kr_ctx* ctx = nullptr;
  unsigned long long uid = 0;  // creation number, unique in the process (keys of recorded steps)
  DevOp dev{};
  DevField field{};
  std::vector<void*> allocs;
  int grid = 1;     // cooperative grid of the plain step (FP64 products)
  int grid_df = 1;  // the same with double-float products
  size_t smem = 0;
  int maxorder = 100;
  bool square = false;
  bool split = false;    // slabs are column chunks (row stride > dk): batched path only
  int npart = 0;
  int nmf = 0;
  int ndiag_groups = 0;  // M groups in diagonal slot order
  // field coefficients in device memory when npart > KR_PART_INLINE
  double2* fc_coef = nullptr;
  double2* fc_scale = nullptr;
  double* fc_thresh = nullptr;
  std::vector<double> fc_host;  // staging: coef, scale, thresh
  // field schedule (kr_set_field_schedule): [nsteps][npart][KR_MAXCART], [nsteps][npart] x2
  void* fs_buf = nullptr;
  int fs_nsteps = 0;
  double2* fs_coef = nullptr;
  double2* fs_scale = nullptr;
  double* fs_thresh = nullptr;
  // tiles of the tensor-core batched mat-vec: [4][tc_ntask] = slab, first row, rows, KP
  int tc_ntask = 0;
  int* tc_task = nullptr;
  int tc_class[4] = {0, 0, 0, 0};  // first tile of KP = 8, 16, 32 in tc_task, and the end
  // B operands of the terms of the KP = 8, 16 tiles (kb_build_tc_b) and each term's offset
  float* tc_b = nullptr;
  long long* tc_boff = nullptr;
  // tiles of the register-tiled FP32 batched mat-vec: [4][zr_ntask] = slab, first row, rows, NKP
  int zr_ntask = 0;
  int* zr_task = nullptr;
  int zr_class[4] = {0, 0, 0, 0};  // first tile of NKP = 8, 16, 32 in zr_task, and the end
  // workspace of kr_expv / kr_op_norm1 (grown on demand, freed with the operator)
  void* expv_ws = nullptr;
  size_t expv_bytes = 0;
  long long launches = 0;
  double fma_per_matvec = 0, bytes_per_matvec = 0;
  // step scratch
  double2 *V = nullptr, *Wb0 = nullptr, *Wb1 = nullptr, *w = nullptr, *ub0 = nullptr, *ub1 = nullptr;
  double2* part_a = nullptr;
  double2* task_alpha = nullptr;
  unsigned* counters = nullptr;
  unsigned* mv_counters = nullptr;
  double *part_b = nullptr, *part_c = nullptr;
  double2* alpha = nullptr;
  double* beta = nullptr;
  unsigned* bar = nullptr;  // [count, gen]
  int* status = nullptr;    // [status, kout]
  float4* xdf = nullptr;    // double-float copy of the vector the next mat-vec reads (KR_PREC_DF)
  int prec = 0;             // products of the plain step: KR_PREC_F64 or KR_PREC_DF
};

