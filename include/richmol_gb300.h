/*
 * richmol_gb300 — C ABI of the GB300 (sm_103a) Krylov time-propagation step.
 *
 * The library replaces, for one GPU, the reference's per-step hot path
 * (CFEL-CMI/richmol):
 *
 *   richmol/tdse.py:265-414   TDSE.update      (split-operator and full-H forms)
 *   richmol/tdse.py:417-486   _expmv_lanczos   (in-house Lanczos exponential)
 *   richmol/field.py:1073-1142 CarTens.field   (field contraction of M factors)
 *   richmol/field.py:1145-1245 CarTens.vec     (Kronecker mat-vec)
 *
 * The reference has no FFI for this path (it is pure Python over scipy); the
 * entry points below are what its Python layer binds through ctypes
 * (richmol_gb300/_native.py is such a binding). Conventions:
 *
 *   - every function returns an int status (KR_OK == 0); no exception or C++
 *     type crosses the boundary; kr_last_error() gives the message;
 *   - vectors and states are DEVICE pointers owned by the caller, complex128
 *     stored as interleaved (re, im) doubles, row-major (nvec, dim);
 *   - descriptor arrays (kr_op_desc) are HOST pointers, copied at creation;
 *   - all work is ordered on the CUDA stream passed in (NULL: legacy stream);
 *   - kr_step and kr_matvec allocate nothing: their scratch is sized and
 *     allocated by kr_op_create;
 *   - one kr_op must not be used from two threads at once.
 */
#ifndef RICHMOL_GB300_H
#define RICHMOL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  KR_OK = 0,
  KR_ERR_ARG = 1,        /* invalid argument / malformed descriptor          */
  KR_ERR_CUDA = 2,       /* a CUDA runtime call failed                       */
  KR_ERR_MAXORDER = 3,   /* Lanczos reached maxorder (tdse.py:480-484)       */
  KR_ERR_TIMEOUT = 4,    /* a bounded device-side wait gave up               */
  KR_ERR_UNSUPPORTED = 5 /* shape outside the compiled limits                */
};

/* K-factor storage kinds: the dense n_k1 x n_k2 block is complex, or purely
 * real, or purely imaginary (then only its imaginary part is stored). */
enum { KR_K_COMPLEX = 0, KR_K_REAL = 1, KR_K_IMAG = 2 };

#define KR_MAXCART 9   /* Cartesian components of a rank-2 tensor         */
#define KR_MAXPART 4096 /* operator parts of one sum (A + B + ...); each
                           part has its own field (kr_set_field), so a
                           set of molecules is one part per tensor of
                           each molecule                                 */

/* Flags of kr_step. */
#define KR_STEP_SKIP_KRYLOV 1u /* H carries no field term (tdse.py:377): apply
                                  only the H0 half-phases                   */

typedef struct kr_ctx kr_ctx;
typedef struct kr_op kr_op;

/*
 * Block-sparse Kronecker operator  Y_{s1} += sum_terms MF_t X_{s2} K_t^T,
 * MF_t = scale_p * thresh_p( sum_c coef_{p,c} M_{g,c} ).
 *
 * Slabs follow the reference's flat vector order: Jlist x symlist[J], each slab
 * a row-major (dim_m, dim_k) block (tdse.py:343-360, field.py:1229).
 * M factors are stored per "group" in ELL form: rows x width entries with a
 * column index (int32) and ncart complex values per entry; padding entries
 * carry value 0. An MF instance is one (group, part) pair; a term names its
 * output slab, input slab, K block and MF instance.
 */
typedef struct {
  int32_t nslab_out, nslab_in;
  const int32_t* out_dm; const int32_t* out_dk; const int64_t* out_off;
  const int32_t* in_dm;  const int32_t* in_dk;  const int64_t* in_off;
  int64_t dim_out, dim_in;

  int32_t nk;                 /* K blocks                                   */
  const int64_t* k_off;       /* offset (in doubles) into k_data            */
  const int32_t* k_rows;      /* n_k1                                       */
  const int32_t* k_cols;      /* n_k2                                       */
  const int32_t* k_type;      /* KR_K_*                                     */
  const double* k_data; int64_t k_data_len;

  int32_t nm;                 /* M groups                                   */
  const int32_t* m_rows;      /* dim_m1                                     */
  const int32_t* m_width;     /* ELL width                                  */
  const int32_t* m_ncart;     /* number of Cartesian components stored      */
  const int64_t* m_col_off;   /* offset into m_col (entries)                */
  const int64_t* m_val_off;   /* offset (in complex values) into m_val      */
  const int32_t* m_col; int64_t m_col_len;
  const double* m_val;  int64_t m_val_len;   /* complex interleaved; layout
                                                [cart][row][width]          */
  int32_t npart;              /* operator parts (<= KR_MAXPART)             */
  int32_t nmf;                /* MF instances                               */
  const int32_t* mf_group; const int32_t* mf_part;

  int32_t nterm;
  const int32_t* t_out; const int32_t* t_in; const int32_t* t_k; const int32_t* t_mf;

  int32_t maxorder;           /* Lanczos basis capacity (reference: 100)    */

  /* Row strides of the slabs (NULL: dim_k, the contiguous row-major slabs
   * above). A slab with stride > dim_k is a column chunk of a wider row-major
   * block: element (i, a) sits at off + i * stride + a. The chunks of an
   * operator must cover each vector element exactly once. Operators with
   * chunks are taken by the batched path only (kr_batch_*), where they carry
   * n_k above 32 as chunks of at most 32 columns; kr_step, kr_matvec,
   * kr_expv and kr_op_norm1 return KR_ERR_UNSUPPORTED for them. */
  const int32_t* out_stride; const int32_t* in_stride;
} kr_op_desc;

/* x <- exp(t A) x, A = i H, for one vector (x: dim complex128 device array,
 * overwritten; with phase != NULL, x is multiplied by phase before and after,
 * the H0 half-phases of the split operator, tdse.py:368-394) with the Krylov scheme of EXPOKIT's ZHEXPV (Sidje 1998), which
 * richmol calls for propag='external' (tdse.py:383-392, pyexpokit.py:55-89;
 * m = 12, t = Im(exp_fac)): fixed Krylov dimension m (<= 30), local error
 * control against tol, at most 500 substeps (then KR_ERR_MAXORDER, the
 * reference's "maximum number of steps reached without convergence").
 * anorm: 1-norm estimate of H (kr_op_norm1). stats (may be NULL): substeps,
 * mat-vecs, rejected substeps. Synchronises the stream. */
int kr_expv(kr_op* op, void* x, const void* phase, double t, int32_t m, double tol,
            double anorm, int32_t* stats, void* stream);
/* Lower-bound estimate of the 1-norm of the (Hermitian) operator with the
 * field of the last kr_set_field: Hager-Higham power iteration (deterministic;
 * the reference uses scipy's randomised onenormest on H.tomat(), tdse.py:387). */
int kr_op_norm1(kr_op* op, double* norm, void* stream);

/* Expectation values of an observable for FP64 states: out[i] = <v_i|O|v_i>
 * (host complex128[nvec], interleaved) for the rows v_i of states (device,
 * (nvec, dim) complex128), O = obs with its field set (e.g. cos^2 theta - 1/3
 * with field [0, 0, 1]); FP64 mat-vec and fixed-order FP64 sums, so the values
 * are reproducible bit for bit. If wsum != NULL, *wsum = sum_i w_i Re out[i]
 * with w = weights (host double[nvec]; NULL: all 1), the Boltzmann-weighted
 * ensemble value. Replaces the observable evaluation of the reference's
 * callers (examples/ocs_alignment.py:70,99-100: v^H (cos^2 theta) v per vector
 * through CarTens.tomat; tests/test_tdse.py:63-67). Synchronises the stream. */
int kr_observables(kr_op* obs, const void* states, int64_t nvec, const double* weights,
                   double* out, double* wsum, void* stream);

/* Segments of a square operator: independent problems (molecules) whose
 * vectors lie one after the other (a block-diagonal operator, e.g. several
 * molecules' slabs in one table). slab_seg[s] is the segment of output slab s:
 * 0, 1, ..., nseg - 1 in slab order, every segment a non-empty slab range, no
 * term coupling two segments. Replaces the per-molecule TDSE.update calls of
 * the reference (tdse.py:265-414) for a set of molecules. */
typedef struct kr_seg kr_seg;
int kr_seg_create(kr_op* op, int32_t nseg, const int32_t* slab_seg, kr_seg** out);
void kr_seg_destroy(kr_seg* seg);
/* One TDSE.update of every segment's vector in one persistent launch (states:
 * dim complex128, in place; phase: H0 half-phases or NULL): the Lanczos
 * recurrence of kr_step per segment, with the segment's own scalars, stopping
 * test (tol) and Krylov order (korder[nseg], host, may be NULL). The operator's
 * kr_step scratch is used: not concurrently with kr_step on the same operator.
 * Synchronises the stream; KR_ERR_MAXORDER if a segment reached maxorder. */
int kr_seg_step(kr_seg* seg, void* states, const void* phase, double fac_re, double fac_im, double tol,
                int32_t* korder, void* stream);
/* Arithmetic of kr_seg_step's mat-vecs (no counterpart in the reference, which
 * is FP64 throughout): KR_SEG_F64 (default), or KR_SEG_F32_MATVEC, the products
 * in FP32 on the FP32 pipes from FP32 copies of the factors (complex64
 * accuracy, about 1e-7 relative per mat-vec) with the states, Krylov vectors,
 * Lanczos scalars, exponential and stopping test in FP64. */
enum { KR_SEG_F64 = 0, KR_SEG_F32_MATVEC = 1 };
int kr_seg_set_precision(kr_seg* seg, int32_t mode);
int64_t kr_seg_launch_count(const kr_seg* seg);

/* Context on one device. Replaces nothing in the reference (which keeps no
 * device state); created once per process and device. */
int kr_ctx_create(int device, kr_ctx** out);
void kr_ctx_destroy(kr_ctx* ctx);
/* Copies the last error message of ctx (or of the library if ctx is NULL). */
int kr_last_error(const kr_ctx* ctx, char* buf, size_t len);

/* Uploads the factors of one operator and allocates its scratch.
 * Replaces the data held by CarTens.kmat / CarTens.mmat (field.py:58-170). */
int kr_op_create(kr_ctx* ctx, const kr_op_desc* desc, kr_op** out);
void kr_op_destroy(kr_op* op);
/* Validates a descriptor on the host, with no device and no context: the
 * checks kr_op_create applies before it uploads anything (slab tables, row
 * strides and coverage of column chunks, M groups, MF instances, K blocks,
 * terms). KR_OK, or the status kr_op_create would return, with its message in
 * buf (len bytes, may be NULL) and in kr_last_error(NULL, ...). */
int kr_op_check(const kr_op_desc* desc, char* buf, size_t len);

/* Field contraction, one call per time step (field.py:1073-1142):
 * MF = scale_p * (|x| < thresh_p ? 0 : x),  x = sum_c coef[p][c] M_c.
 * coef: npart x KR_MAXCART complex (interleaved), scale: npart complex,
 * thresh: npart doubles (<= 0: no element threshold). Host pointers. */
int kr_set_field(kr_op* op, const double* coef, const double* scale,
                 const double* thresh, void* stream);

/* Field schedule: the coefficients of nsteps time steps uploaded at once, for
 * loops whose field is known ahead (the pulse of examples/ocs_alignment.py:
 * 70-100 evaluated on the time grid). coef: nsteps x npart x KR_MAXCART
 * complex, scale: nsteps x npart complex, thresh: nsteps x npart doubles,
 * step-major, each step laid out as for kr_set_field. Host pointers; the call
 * returns once the copy is complete. Replaces a previous schedule (waiting for
 * the device first) and frees its memory: a CUDA graph that recorded
 * kr_set_field_step of the old schedule must not be replayed afterwards. */
int kr_set_field_schedule(kr_op* op, int32_t nsteps, const double* coef,
                          const double* scale, const double* thresh,
                          void* stream);
/* kr_set_field with the coefficients of step `step` of the schedule: no host
 * data travels, so it can be recorded into a CUDA graph for any part count.
 * KR_ERR_ARG if there is no schedule or step is outside [0, nsteps). */
int kr_set_field_step(kr_op* op, int32_t step, void* stream);

/* y = H x for nvec vectors (field.py:1145-1245). x: (nvec, dim_in),
 * y: (nvec, dim_out), device pointers, complex128. */
int kr_matvec(kr_op* op, const void* x, void* y, int64_t nvec, void* stream);

/* One TDSE.update of nvec state vectors in place (tdse.py:265-414 with
 * propag='internal'): if phase != NULL (split operator, tdse.py:365-394)
 *   v <- phase * expmv(fac, H, phase * v), phase = exp(fac/2 diag(H0)),
 * else (full H, tdse.py:396-402)  v <- expmv(fac, H, v), where expmv is the
 * reference Lanczos recurrence (tdse.py:417-486) with tolerance tol on the
 * squared distance of successive solutions. states: (nvec, dim) device,
 * phase: dim complex device or NULL. If korder != NULL the call synchronises
 * the stream and writes the Krylov order used for each vector (host array of
 * nvec int32) and returns KR_ERR_MAXORDER if a vector did not converge;
 * otherwise device-side errors are reported by the next kr_sync_status. */
int kr_step(kr_op* op, void* states, int64_t nvec, const void* phase,
            double fac_re, double fac_im, double tol, uint32_t flags,
            int32_t* korder, void* stream);

/* Allocation-free variant of kr_step, no counterpart in the reference.
 * Same arguments and results as kr_step, but the Krylov workspace lives in a
 * fixed 64 MiB array inside the library (a file-scope __device__ array that
 * every GPU loading the library holds until exit) instead of the workspace
 * kr_op_create allocated. It is for callers that must not allocate device
 * memory at step time: code recorded into CUDA graphs, or hosts whose device
 * memory is owned by their own pool allocator. It calls no cudaMalloc,
 * cudaFree or allocating library routine. Limits and rules:
 *   - operators whose workspace exceeds the array (kr_static_scratch_bytes;
 *     about dim * (maxorder + 5) * 16 bytes) are rejected with KR_ERR_ARG;
 *   - the first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress with that device current); make that first call
 *     before any stream capture;
 *   - all calls share the array and it keeps the previous call's contents:
 *     calls that overlap on the GPU (other streams, other threads) race;
 *   - with korder == NULL a device-side error is copied into op's status and
 *     reported by kr_sync_status;
 *   - an error still pending in op's status (an earlier call with
 *     korder == NULL) makes the call skip its work, as kr_step does;
 *   - the caller's current device is the same after the call as before. */
int kr_step_static(kr_op* op, void* states, int64_t nvec, const void* phase,
                   double fac_re, double fac_im, double tol, uint32_t flags,
                   int32_t* korder, void* stream);

/* Arithmetic of the mat-vec products of kr_step and kr_step_static (no
 * counterpart in the reference, which is FP64 throughout): KR_PREC_F64
 * (default), or KR_PREC_DF, double-float products on the FP32 pipes (each FP64
 * value held as an FP32 pair, about 48 significant bits; 1e-14 relative per
 * product) with the states, Krylov vectors, Lanczos scalars, exponential and
 * stopping test in FP64. */
enum { KR_PREC_F64 = 0, KR_PREC_DF = 1 };
int kr_op_set_precision(kr_op* op, int32_t prec);

/* Bytes of static scratch kr_step_static needs for op, and the capacity. */
int kr_static_scratch_bytes(const kr_op* op, size_t* needed, size_t* capacity);

/* ------------------------------------------------------------------------
 * Batched mixed-precision ensembles. The reference propagates the vectors of
 * an ensemble one by one (tdse.py:379-382 and 398-402, each through
 * _expmv_lanczos, tdse.py:417-486); a batch propagates them together, each
 * with its own Krylov order: complex64 mat-vec with FP32 accumulation,
 * complex64 Krylov basis with full orthogonalisation, FP64 Lanczos scalars,
 * tridiagonal exponential, a-posteriori error estimate and FP64 state.
 * ------------------------------------------------------------------------ */
typedef struct kr_batch kr_batch;

/* Allocates the batch state and Krylov basis for nvec vectors of op's basis
 * (mmax basis vectors, 2 <= mmax <= 31). */
int kr_batch_create(kr_op* op, int64_t nvec, int32_t mmax, kr_batch** out);
void kr_batch_destroy(kr_batch* b);
/* states (nvec, dim) complex128 device <-> the batch's internal layout
 * (kr_batch_load also discards the first Krylov vector kept for the next
 * step, see kr_batch_step). */
int kr_batch_load(kr_batch* b, const void* states, void* stream);
int kr_batch_store(kr_batch* b, void* states, void* stream);
/* One TDSE.update of every vector (split operator when phase != NULL):
 * op carries H with its field set (kr_set_field); each vector stops at the
 * first Krylov order whose error estimate is <= tol (times nothing: absolute,
 * in the norm of the vector). The Krylov loop runs on the device (a CUDA graph
 * with a conditional WHILE node; the Krylov index lives in device memory), so
 * the host takes no part between iterations:
 *   - on a stream that is not capturing, the step is recorded once per
 *     (op, phase, fac, tol, mat-vec kind) and launched as one graph;
 *     kmax_out != NULL synchronises the stream, writes the largest order used
 *     and returns a step error (KR_ERR_MAXORDER if a vector needs more than
 *     mmax); kmax_out == NULL returns at once, errors wait for kr_batch_sync;
 *   - on a capturing stream (the caller records its time loop into a CUDA
 *     graph) the step's nodes go into the caller's graph; kmax_out must be
 *     NULL and errors are read by kr_batch_sync after the replay.
 * A pending error makes later steps leave the states unchanged until it has
 * been read. A step's state combination also writes the next step's first
 * Krylov vector (phase times the new states) and its norm, for the phase
 * array at that address; the next step with the same phase address skips
 * that pass, and kr_batch_load discards it. Rewriting a phase array's
 * contents in place between steps is therefore not allowed. Between steps,
 * kr_batch_expect*, kr_batch_apply, kr_batch_matvec and kr_batch_populations
 * leave it intact. */
int kr_batch_step(kr_batch* b, kr_op* op, const void* phase, double fac_re, double fac_im,
                  double tol, int32_t* kmax_out, void* stream);
/* Synchronises the stream and reports (and clears) the error of an earlier
 * kr_batch_step; *kmax_out (optional): largest Krylov order of the last step.
 * No counterpart in the reference (its steps are synchronous). */
int kr_batch_sync(kr_batch* b, int32_t* kmax_out, void* stream);
/* Krylov order used by each vector in the last step (host int32[nvec]). */
int kr_batch_korder(kr_batch* b, int32_t* korder, void* stream);
/* <v|O|v> for every vector (host complex128[nvec], interleaved), O = obs
 * with its field set (e.g. cos^2 theta with field [0, 0, 1]); complex64
 * mat-vec, FP64 dot products. Synchronises. */
int kr_batch_expect(kr_batch* b, kr_op* obs, double* out, void* stream);
/* sum_v w_v Re <v|O|v> into one device double (out), weights: device
 * double[nvec] or NULL (all 1); stream-ordered, no synchronisation, so a time
 * loop can keep an observable's trace on the device and read it once. A
 * mat-vec error of the observable is kept as the batch's step error (reported
 * by kr_batch_sync). No counterpart in the reference. */
int kr_batch_expect_dev(kr_batch* b, kr_op* obs, const double* weights, double* out, void* stream);
/* Populations of every slab (the (J, sym) blocks of the flat vector order) for
 * every vector: out[slab * nvec + v] = sum over the slab of |S_v|^2 (host array,
 * nslab x nvec doubles); summed over the symmetries of a J they are the
 * J-populations of the reference's observables (tests/test_tdse.py:63-67). */
int kr_batch_populations(kr_batch* b, double* out, void* stream);
/* Mat-vec kinds of a batch: KR_MATVEC_TENSOR (default) contracts the K
 * factors on the tensor cores (tcgen05, TF32 with split operands: about 2^-21
 * relative per product, FP32 accumulation), the A operands staged in shared
 * memory; KR_MATVEC_TENSOR_TMEM the same products with the A operands written
 * to tensor memory (tcgen05.st) and a deeper TMA ring of input rows in the
 * shared memory this frees; KR_MATVEC_FP32 runs every product as an FP32
 * FMA (tiles staged through shared memory); KR_MATVEC_FP32_REG the same
 * products register-tiled (each thread a few output rows of one vector,
 * all terms of the tile's slab summed in registers). No counterpart in the
 * reference (FP64 only). */
enum { KR_MATVEC_TENSOR = 0, KR_MATVEC_FP32 = 1, KR_MATVEC_TENSOR_TMEM = 2, KR_MATVEC_FP32_REG = 3 };
int kr_batch_set_matvec(kr_batch* b, int32_t kind);
/* y = op x for nvec vectors with the batched complex64 mat-vec (CarTens.vec,
 * field.py:1145-1245, in single precision): x, y (nvec, dim) complex128
 * device arrays; uses the batch's basis slot 0 as scratch. Synchronises. */
int kr_batch_apply(kr_batch* b, kr_op* op, const void* x, void* y, void* stream);
/* W = op V_0 for every vector (complex64), the batched mat-vec alone
 * (V_0 holds the normalised, phased states after a step). */
int kr_batch_matvec(kr_batch* b, kr_op* op, void* stream);
int64_t kr_batch_launch_count(const kr_batch* b);

/* Synchronises the stream and returns the pending device-side status of op. */
int kr_sync_status(kr_op* op, void* stream);

/* Number of kernels launched by op since creation (instrumentation). */
int64_t kr_op_launch_count(const kr_op* op);

/* Algorithmic work of one mat-vec of op: FP64 fused multiply-adds and the
 * minimum bytes moved (vector in + out + factors). */
int kr_op_work(const kr_op* op, double* fma_per_matvec, double* bytes_per_matvec);

/* Measurement helper with no counterpart in the reference: FP64 fused
 * multiply-add throughput of the device in TFLOP/s (the roofline denominator
 * of the FP64 path). Allocates and synchronises; not for the hot path. */
int kr_probe_fp64(kr_ctx* ctx, double* tflops);
/* The same for FP32 fused multiply-adds (denominator of the complex64 mat-vec). */
int kr_probe_fp32(kr_ctx* ctx, double* tflops);
/* Tensor-core probe (no counterpart in the reference): D = A B^T with A
 * 128 x 16, B 16 x 16, D 128 x 16, row-major FP32 host arrays read as TF32, by
 * one tcgen05.mma tile; checks the MMA building block of the batched mat-vec. */
int kr_probe_mma(kr_ctx* ctx, const float* a, const float* b, float* d);
/* The same product with A held in tensor memory (row m in TMEM lane m, written
 * by tcgen05.st) instead of shared memory; no counterpart in the reference. */
int kr_probe_mma_ta(kr_ctx* ctx, const float* a, const float* b, float* d);
/* Failure-detection probe (no counterpart in the reference): the bounded grid
 * barrier of the step kernels in a launch of two CTAs of which one never
 * arrives (a rank that never joins). The other's wait gives up after its limit
 * (2 s), records KR_ERR_TIMEOUT and returns instead of hanging; *status gets
 * the status the barrier recorded (KR_ERR_TIMEOUT, or KR_OK had it completed),
 * *waited_s how long it waited. The call itself returns KR_OK and the context
 * stays usable. Synchronises the device. */
int kr_probe_wait(kr_ctx* ctx, int32_t* status, double* waited_s);

#ifdef __cplusplus
}
#endif
#endif /* RICHMOL_GB300_H */
