// Krylov propagator with local error control in the scheme of EXPOKIT's ZHEXPV
// (R. B. Sidje, ACM Trans. Math. Softw. 24 (1998) 130-156), which richmol calls
// for propag='external' (richmol/tdse.py:383-392 via richmol/pyexpokit.py:55-89,
// with A = i H and t = Im(exp_fac)), and a 1-norm estimator of the operator
// (the reference passes scipy's randomised onenormest of H.tomat()).
//
// The step control runs on the host in FP64 exactly as the published scheme:
// fixed Krylov dimension m, Hermitian Lanczos on H with the projected matrix
// i T of A = i H (the reference hands A = i H to a recurrence written for
// Hermitian A, which loses orthogonality and misses the breakdown of small
// invariant subspaces; the exponential is the same), happy breakdown at 1e-7,
// a-priori first step,
// acceptance when the local error estimate of the augmented (m+2) x (m+2)
// exponential is <= 1.2 t_step tol, step shrink/grow by 0.9 (t_step tol /
// err)^(1/m), step sizes rounded to two significant digits, at most 500 steps
// (and 500 rejections of one step, or a non-finite error estimate: error).
// The vector work runs on the device: the FP64 mat-vec of kr_step.cu and small
// FP64 kernels whose reductions sum in a fixed order (bitwise reproducible).
// The small exponential is a (6, 6) Pade approximant with scaling and squaring.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "kr_internal.cuh"

namespace {

constexpr int KX_BLOCKS = 256;
constexpr int KX_THREADS = 256;
enum { KX_DOT = 0, KX_NRM2 = 1, KX_ABS1 = 2, KX_AMAX = 3 };

// per-block partial of a reduction over a grid-stride range (fixed order)
__global__ void __launch_bounds__(KX_THREADS) kx_reduce(int op, const double2* a, const double2* b, long long n,
                                                        double2* part, long long* ipart) {
  __shared__ double2 sv[KX_THREADS];
  __shared__ long long si[KX_THREADS];
  double2 acc = make_double2(op == KX_AMAX ? -1.0 : 0.0, 0.0);
  long long idx = -1;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 x = a[e];
    if (op == KX_DOT) {  // conj(a) b
      const double2 y = b[e];
      acc.x = fma(x.x, y.x, fma(x.y, y.y, acc.x));
      acc.y = fma(x.x, y.y, fma(-x.y, y.x, acc.y));
    } else if (op == KX_NRM2) {
      acc.x = fma(x.x, x.x, fma(x.y, x.y, acc.x));
    } else if (op == KX_ABS1) {
      acc.x += sqrt(x.x * x.x + x.y * x.y);
    } else {
      const double m2 = x.x * x.x + x.y * x.y;
      if (m2 > acc.x) {
        acc.x = m2;
        idx = e;
      }
    }
  }
  sv[threadIdx.x] = acc;
  si[threadIdx.x] = idx;
  __syncthreads();
  for (int s = KX_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double2 o = sv[threadIdx.x + s];
      if (op == KX_AMAX) {
        const long long oi = si[threadIdx.x + s];
        if (o.x > sv[threadIdx.x].x || (o.x == sv[threadIdx.x].x && oi >= 0 && (si[threadIdx.x] < 0 || oi < si[threadIdx.x]))) {
          sv[threadIdx.x] = o;
          si[threadIdx.x] = oi;
        }
      } else {
        sv[threadIdx.x].x += o.x;
        sv[threadIdx.x].y += o.y;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sv[0];
    ipart[blockIdx.x] = si[0];
  }
}

__global__ void kx_final(int op, const double2* part, const long long* ipart, int np, double2* out, long long* iout) {
  if (threadIdx.x != 0) return;
  double2 s = make_double2(op == KX_AMAX ? -1.0 : 0.0, 0.0);
  long long si = -1;
  for (int i = 0; i < np; ++i) {
    if (op == KX_AMAX) {
      if (part[i].x > s.x || (part[i].x == s.x && ipart[i] >= 0 && (si < 0 || ipart[i] < si))) {
        s = part[i];
        si = ipart[i];
      }
    } else {
      s.x += part[i].x;
      s.y += part[i].y;
    }
  }
  *out = s;
  *iout = si;
}

// y = a x + b y   (x may be null: y = b y)
__global__ void kx_axpby(double2 a, const double2* x, double2 b, double2* y, long long n) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 yv = y[e];
    double2 r = make_double2(b.x * yv.x - b.y * yv.y, b.x * yv.y + b.y * yv.x);
    if (x) {
      const double2 xv = x[e];
      r.x = fma(a.x, xv.x, fma(-a.y, xv.y, r.x));
      r.y = fma(a.x, xv.y, fma(a.y, xv.x, r.y));
    }
    y[e] = r;
  }
}

// xi = y / |y| (1 where y = 0)
__global__ void kx_unit(const double2* y, double2* xi, long long n) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 v = y[e];
    const double r = sqrt(v.x * v.x + v.y * v.y);
    xi[e] = r > 0.0 ? make_double2(v.x / r, v.y / r) : make_double2(1.0, 0.0);
  }
}

// x_i = value(i): kind 0 constant c; kind 1 (-1)^i (1 + i / (n - 1)); kind 2 e_j
__global__ void kx_fill(double2* x, long long n, int kind, double c, long long j) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double v;
    if (kind == 0) v = c;
    else if (kind == 1) v = ((e & 1) ? -1.0 : 1.0) * (1.0 + (n > 1 ? (double)e / (double)(n - 1) : 0.0));
    else v = e == j ? 1.0 : 0.0;
    x[e] = make_double2(v, 0.0);
  }
}

// x *= phase (H0 half-phase of the split operator)
__global__ void kx_phase(double2* x, const double2* ph, long long n) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 a = x[e], b = __ldg(ph + e);
    x[e] = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
}

struct KxCoef {
  double2 c[KR_EXPV_MMAX + 2];
};
// w = sum_{i < k} c_i V_i
__global__ void kx_combine(const double2* V, long long n, int k, KxCoef c, double2* w) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int i = 0; i < k; ++i) {
      const double2 v = V[(long long)i * n + e];
      s.x = fma(c.c[i].x, v.x, fma(-c.c[i].y, v.y, s.x));
      s.y = fma(c.c[i].x, v.y, fma(c.c[i].y, v.x, s.y));
    }
    w[e] = s;
  }
}

using cd = std::complex<double>;

// exp(X) for a small dense matrix (row-major mx x mx): (6, 6) Pade approximant
// with scaling and squaring (Moler & Van Loan, SIAM Rev. 45 (2003) 3, method 3)
void expm_pade6(std::vector<cd>& X, int mx, std::vector<cd>& E) {
  double nrm = 0.0;  // infinity norm
  for (int i = 0; i < mx; ++i) {
    double r = 0.0;
    for (int j = 0; j < mx; ++j) r += std::abs(X[i * mx + j]);
    nrm = std::max(nrm, r);
  }
  int s = 0;
  if (nrm > 0.5) s = std::max(0, (int)std::ceil(std::log2(nrm / 0.5)));
  const double sc = std::ldexp(1.0, -s);
  std::vector<cd> A(X.size()), P(X.size()), N(X.size(), 0.0), D(X.size(), 0.0), T(X.size());
  for (size_t i = 0; i < X.size(); ++i) A[i] = X[i] * sc;
  auto matmul = [mx](const std::vector<cd>& L, const std::vector<cd>& R, std::vector<cd>& O) {
    for (int i = 0; i < mx; ++i)
      for (int j = 0; j < mx; ++j) {
        cd acc = 0.0;
        for (int k = 0; k < mx; ++k) acc += L[i * mx + k] * R[k * mx + j];
        O[i * mx + j] = acc;
      }
  };
  const int p = 6;
  double c = 1.0;
  for (int i = 0; i < mx; ++i) {
    N[i * mx + i] = 1.0;
    D[i * mx + i] = 1.0;
    for (int j = 0; j < mx; ++j) P[i * mx + j] = i == j ? 1.0 : 0.0;
  }
  for (int k = 1; k <= p; ++k) {
    c = c * (p + 1 - k) / (k * (2.0 * p + 1 - k));
    matmul(P, A, T);
    P.swap(T);
    const double sgn = (k & 1) ? -1.0 : 1.0;
    for (size_t i = 0; i < P.size(); ++i) {
      N[i] += c * P[i];
      D[i] += sgn * c * P[i];
    }
  }
  // E = D^-1 N (Gaussian elimination, partial pivoting)
  E = N;
  for (int col = 0; col < mx; ++col) {
    int piv = col;
    for (int r = col + 1; r < mx; ++r)
      if (std::abs(D[r * mx + col]) > std::abs(D[piv * mx + col])) piv = r;
    if (piv != col)
      for (int j = 0; j < mx; ++j) {
        std::swap(D[col * mx + j], D[piv * mx + j]);
        std::swap(E[col * mx + j], E[piv * mx + j]);
      }
    const cd d = D[col * mx + col];
    for (int r = col + 1; r < mx; ++r) {
      const cd f = D[r * mx + col] / d;
      if (f == cd(0.0)) continue;
      for (int j = col; j < mx; ++j) D[r * mx + j] -= f * D[col * mx + j];
      for (int j = 0; j < mx; ++j) E[r * mx + j] -= f * E[col * mx + j];
    }
  }
  for (int col = mx - 1; col >= 0; --col) {
    const cd d = D[col * mx + col];
    for (int j = 0; j < mx; ++j) E[col * mx + j] /= d;
    for (int r = 0; r < col; ++r) {
      const cd f = D[r * mx + col];
      if (f == cd(0.0)) continue;
      for (int j = 0; j < mx; ++j) E[r * mx + j] -= f * E[col * mx + j];
    }
  }
  for (int k = 0; k < s; ++k) {
    matmul(E, E, T);
    E.swap(T);
  }
}

double nint(double x) { return std::copysign(std::floor(std::fabs(x) + 0.5), x); }
// step sizes rounded to two significant digits (the published scheme)
double round2(double x) {
  const double p1 = std::pow(10.0, nint(std::log10(x) - std::sqrt(0.1)) - 1.0);
  return std::trunc(x / p1 + 0.55) * p1;
}

// device workspace and reductions of one operator
struct Kx {
  kr_op* op;
  cudaStream_t st;
  long long n;
  double2* V;       // [m + 1][n]
  double2* P;       // [n]
  double2* part;    // [KX_BLOCKS]
  long long* ipart; // [KX_BLOCKS]
  double2* res;     // [1]
  long long* ires;  // [1]
  int grid;
};

// grows the operator's workspace of kr_expv / kr_op_norm1 / kr_observables
// (each of them synchronises its stream before it returns)
int kx_grow(kr_op* op, size_t need) {
  if (op->expv_bytes < need) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, need);
    if (e != cudaSuccess) return set_err(op->ctx, KR_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    if (op->expv_ws) cudaFree(op->expv_ws);
    op->expv_ws = q;
    op->expv_bytes = need;
  }
  return KR_OK;
}

int kx_workspace(kr_op* op, long long n, int m, Kx& k) {
  const size_t need = sizeof(double2) * ((size_t)(m + 2) * n + KX_BLOCKS + 1) + sizeof(long long) * (KX_BLOCKS + 1);
  const int rc = kx_grow(op, need);
  if (rc != KR_OK) return rc;
  char* b = static_cast<char*>(op->expv_ws);
  k.V = reinterpret_cast<double2*>(b);
  k.P = k.V + (size_t)(m + 1) * n;
  k.part = k.P + n;
  k.res = k.part + KX_BLOCKS;
  k.ipart = reinterpret_cast<long long*>(k.res + 1);
  k.ires = k.ipart + KX_BLOCKS;
  k.op = op;
  k.n = n;
  k.grid = std::max(1, std::min(8 * op->ctx->nsm, (int)((n + KX_THREADS - 1) / KX_THREADS)));
  return KR_OK;
}

int kx_red(Kx& k, int op, const double2* a, const double2* b, double2* out, long long* iout) {
  kx_reduce<<<KX_BLOCKS, KX_THREADS, 0, k.st>>>(op, a, b, k.n, k.part, k.ipart);
  kx_final<<<1, 32, 0, k.st>>>(op, k.part, k.ipart, KX_BLOCKS, k.res, k.ires);
  k.op->launches += 2;
  KR_CUDA(k.op->ctx, cudaGetLastError());
  long long idx = 0;
  KR_CUDA(k.op->ctx, cudaMemcpyAsync(out, k.res, sizeof(double2), cudaMemcpyDeviceToHost, k.st));
  KR_CUDA(k.op->ctx, cudaMemcpyAsync(&idx, k.ires, sizeof(long long), cudaMemcpyDeviceToHost, k.st));
  KR_CUDA(k.op->ctx, cudaStreamSynchronize(k.st));
  if (iout) *iout = idx;
  return KR_OK;
}
int kx_nrm2(Kx& k, const double2* a, double* out) {
  double2 r;
  int rc = kx_red(k, KX_NRM2, a, nullptr, &r, nullptr);
  *out = std::sqrt(r.x);
  return rc;
}
int kx_axpby_l(Kx& k, cd a, const double2* x, cd b, double2* y) {
  kx_axpby<<<k.grid, KX_THREADS, 0, k.st>>>(make_double2(a.real(), a.imag()), x, make_double2(b.real(), b.imag()),
                                            y, k.n);
  k.op->launches++;
  KR_CUDA(k.op->ctx, cudaGetLastError());
  return KR_OK;
}
int kx_mv(Kx& k, const double2* x, double2* y) { return kr_matvec(k.op, x, y, 1, k.st); }

}  // namespace

#define KX_TRY(call)          \
  do {                        \
    const int _rc = (call);   \
    if (_rc != KR_OK) return _rc; \
  } while (0)

extern "C" int kr_op_norm1(kr_op* op, double* norm, void* stream) {
  if (!op || !norm) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_op_norm1: bad argument");
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_op_norm1: operator is not square");
  if (op->split) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_op_norm1: operator with column chunks");
  const long long n = op->dev.dim_out;
  Kx k;
  k.st = (cudaStream_t)stream;
  KX_TRY(kx_workspace(op, n, 2, k));
  double2* x = k.V;
  double2* y = k.V + n;
  double2* z = k.V + 2 * n;
  // Hager's estimator in Higham's complex form (ACM Trans. Math. Softw. 14
  // (1988) 381, algorithm CONEST): power iteration on the unit-modulus vector,
  // at most 5 iterations, plus the alternating test vector; H is Hermitian,
  // so its adjoint product is H itself
  kx_fill<<<k.grid, KX_THREADS, 0, k.st>>>(x, n, 0, 1.0 / (double)n, 0);
  double est = 0.0;
  long long jlast = -1;
  for (int it = 1; it <= 5; ++it) {
    KX_TRY(kx_mv(k, x, y));
    double2 r;
    KX_TRY(kx_red(k, KX_ABS1, y, nullptr, &r, nullptr));
    if (it > 1 && r.x <= est) break;
    est = r.x;
    kx_unit<<<k.grid, KX_THREADS, 0, k.st>>>(y, z, n);
    KX_TRY(kx_mv(k, z, y));  // y <- H xi
    long long j = 0;
    double2 zm;
    KX_TRY(kx_red(k, KX_AMAX, y, nullptr, &zm, &j));
    if (it > 1) {
      double2 zx;
      KX_TRY(kx_red(k, KX_DOT, y, x, &zx, nullptr));  // conj(z) . x
      if (std::sqrt(zm.x) <= zx.x || j == jlast) break;
    }
    jlast = j;
    kx_fill<<<k.grid, KX_THREADS, 0, k.st>>>(x, n, 2, 0.0, j);
  }
  kx_fill<<<k.grid, KX_THREADS, 0, k.st>>>(x, n, 1, 0.0, 0);
  KX_TRY(kx_mv(k, x, y));
  double2 r;
  KX_TRY(kx_red(k, KX_ABS1, y, nullptr, &r, nullptr));
  est = std::max(est, 2.0 * r.x / (3.0 * (double)n));
  *norm = est;
  KR_CUDA(op->ctx, cudaGetLastError());
  return KR_OK;
}

extern "C" int kr_observables(kr_op* obs, const void* states, int64_t nvec, const double* weights, double* out,
                              double* wsum, void* stream) {
  if (!obs || (!states && nvec > 0) || nvec < 0 || (!out && nvec > 0))
    return set_err(obs ? obs->ctx : nullptr, KR_ERR_ARG, "kr_observables: bad argument");
  if (!obs->square) return set_err(obs->ctx, KR_ERR_ARG, "kr_observables: operator is not square");
  if (obs->split) return set_err(obs->ctx, KR_ERR_UNSUPPORTED, "kr_observables: operator with column chunks");
  const long long n = obs->dev.dim_out;
  cudaStream_t st = (cudaStream_t)stream;
  // vectors in chunks whose products O v fit 256 MiB: [chunk][n] products,
  // per-block partials, one result per vector
  const long long chunk = std::max(1LL, std::min<long long>(nvec, (256LL << 20) / (16LL * std::max(1LL, n))));
  const size_t need = sizeof(double2) * ((size_t)chunk * n + KX_BLOCKS + (size_t)nvec) +
                      sizeof(long long) * (KX_BLOCKS + (size_t)nvec);
  KX_TRY(kx_grow(obs, need));
  double2* y = static_cast<double2*>(obs->expv_ws);
  double2* part = y + (size_t)chunk * n;
  double2* res = part + KX_BLOCKS;
  long long* ipart = reinterpret_cast<long long*>(res + nvec);
  long long* ires = ipart + KX_BLOCKS;
  const double2* S = static_cast<const double2*>(states);
  for (long long v0 = 0; v0 < nvec; v0 += chunk) {
    const long long c = std::min(chunk, nvec - v0);
    KX_TRY(kr_matvec(obs, S + v0 * n, y, c, st));
    for (long long i = 0; i < c; ++i) {  // <v|O v> = conj(v) . (O v), fixed summation order
      kx_reduce<<<KX_BLOCKS, KX_THREADS, 0, st>>>(KX_DOT, S + (v0 + i) * n, y + i * n, n, part, ipart);
      kx_final<<<1, 32, 0, st>>>(KX_DOT, part, ipart, KX_BLOCKS, res + v0 + i, ires + v0 + i);
    }
    obs->launches += 2 * c;
    KR_CUDA(obs->ctx, cudaGetLastError());
  }
  if (nvec > 0) KR_CUDA(obs->ctx, cudaMemcpyAsync(out, res, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, st));
  KR_CUDA(obs->ctx, cudaStreamSynchronize(st));
  if (wsum) {
    double s = 0.0;
    for (long long i = 0; i < nvec; ++i) s += (weights ? weights[i] : 1.0) * out[2 * i];
    *wsum = s;
  }
  return KR_OK;
}

static int kr_expv_krylov(kr_op* op, void* x, double t, int32_t m, double tol, double anorm, int32_t* stats,
                          void* stream);

extern "C" int kr_expv(kr_op* op, void* x, const void* phase, double t, int32_t m, double tol, double anorm,
                       int32_t* stats, void* stream) {
  if (!op || !x) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_expv: bad argument");
  if (op->split) return set_err(op->ctx, KR_ERR_UNSUPPORTED, "kr_expv: operator with column chunks");
  const long long n = op->dev.dim_out;
  const int grid = std::max(1, std::min(8 * op->ctx->nsm, (int)((n + KX_THREADS - 1) / KX_THREADS)));
  cudaStream_t st = (cudaStream_t)stream;
  if (phase) {
    kx_phase<<<grid, KX_THREADS, 0, st>>>(static_cast<double2*>(x), static_cast<const double2*>(phase), n);
    op->launches++;
    KR_CUDA(op->ctx, cudaGetLastError());
  }
  const int rc = kr_expv_krylov(op, x, t, m, tol, anorm, stats, stream);
  if (rc != KR_OK) return rc;
  if (phase) {
    kx_phase<<<grid, KX_THREADS, 0, st>>>(static_cast<double2*>(x), static_cast<const double2*>(phase), n);
    op->launches++;
    KR_CUDA(op->ctx, cudaGetLastError());
    KR_CUDA(op->ctx, cudaStreamSynchronize(st));
  }
  return KR_OK;
}

static int kr_expv_krylov(kr_op* op, void* x, double t, int32_t m, double tol, double anorm, int32_t* stats,
                          void* stream) {
  if (!op || !x) return set_err(op ? op->ctx : nullptr, KR_ERR_ARG, "kr_expv: bad argument");
  if (!op->square) return set_err(op->ctx, KR_ERR_ARG, "kr_expv: operator is not square");
  const long long n = op->dev.dim_out;
  if (m <= 0 || m >= n || m > KR_EXPV_MMAX) return set_err(op->ctx, KR_ERR_ARG, "kr_expv: bad input arguments");
  if (!(anorm > 0.0)) return set_err(op->ctx, KR_ERR_ARG, "kr_expv: the operator norm must be positive");
  Kx k;
  k.st = (cudaStream_t)stream;
  KX_TRY(kx_workspace(op, n, m, k));
  double2* w = static_cast<double2*>(x);
  const double eps = DBL_EPSILON;
  if (tol <= eps) tol = std::sqrt(eps);
  const double t_out = std::fabs(t), sgn = t >= 0.0 ? 1.0 : -1.0;
  const int mh = m + 2;
  double beta = 0.0;
  KX_TRY(kx_nrm2(k, w, &beta));
  if (!(beta > 0.0)) {  // exp(tA) 0 = 0
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    return KR_OK;
  }
  double xm = 1.0 / m;
  // a-priori first step from the Krylov error bound
  const double pb = tol * std::pow((m + 1) / 2.72, m + 1) * std::sqrt(2.0 * 3.14 * (m + 1));
  double t_new = round2((1.0 / anorm) * std::pow(pb / (4.0 * beta * anorm), xm));
  double t_now = 0.0;
  int nstep = 0, nmult = 0, nreject = 0;
  std::vector<cd> Hm((size_t)mh * mh), F;
  while (t_now < t_out) {
    ++nstep;
    double t_step = std::min(t_out - t_now, t_new);
    KX_TRY(kx_nrm2(k, w, &beta));
    if (!(beta > 0.0)) break;  // zero vector: exp(tA) 0 = 0
    std::fill(Hm.begin(), Hm.end(), cd(0.0));
    KX_TRY(kx_axpby_l(k, 1.0 / beta, w, 0.0, k.V));  // V_0 = w / beta
    int k1 = 2, mbrk = m;
    double avnorm = 0.0, beta_prev = 0.0;
    const cd iu(0.0, 1.0);
    for (int j = 0; j < m; ++j) {
      double2* vj = k.V + (size_t)j * n;
      double2* p = k.V + (size_t)(j + 1) * n;
      // Hermitian Lanczos on H: p = H v_j - beta_{j-1} v_{j-1} - alpha_j v_j
      KX_TRY(kx_mv(k, vj, p));
      ++nmult;
      if (j > 0) KX_TRY(kx_axpby_l(k, -beta_prev, k.V + (size_t)(j - 1) * n, 1.0, p));
      double2 hd;
      KX_TRY(kx_red(k, KX_DOT, vj, p, &hd, nullptr));
      const cd hjj(hd.x, hd.y);
      KX_TRY(kx_axpby_l(k, -hjj, vj, 1.0, p));
      double hj1j = 0.0;
      KX_TRY(kx_nrm2(k, p, &hj1j));
      Hm[(size_t)j * mh + j] = iu * hjj;  // projected matrix of A = i H: i T
      if (hj1j <= 1e-7) {                 // happy breakdown
        k1 = 0;
        mbrk = j + 1;
        t_step = t_out - t_now;
        break;
      }
      Hm[(size_t)j * mh + j + 1] = iu * hj1j;
      Hm[(size_t)(j + 1) * mh + j] = iu * hj1j;
      beta_prev = hj1j;
      KX_TRY(kx_axpby_l(k, 0.0, nullptr, 1.0 / hj1j, p));
    }
    if (k1 != 0) {
      KX_TRY(kx_mv(k, k.V + (size_t)m * n, k.P));
      ++nmult;
      KX_TRY(kx_nrm2(k, k.P, &avnorm));  // ||A v_m|| = ||H v_m||
    }
    // augmented matrix: h_{m+1,m} stays below the diagonal, the entry above it
    // is cleared, and a 1 at (m+2, m+1)
    Hm[(size_t)(m - 1) * mh + m] = 0.0;
    Hm[(size_t)(m + 1) * mh + m] = 1.0;
    double err_loc = 0.0;
    int mx = 0;
    for (int rej = 0;; ++rej) {
      if (rej > 500) return set_err(op->ctx, KR_ERR_MAXORDER, "kr_expv: requested tolerance was too high");
      mx = mbrk + k1;
      std::vector<cd> X((size_t)mx * mx);
      for (int i = 0; i < mx; ++i)
        for (int j = 0; j < mx; ++j) X[(size_t)i * mx + j] = sgn * t_step * Hm[(size_t)i * mh + j];
      expm_pade6(X, mx, F);
      if (k1 == 0) {
        err_loc = tol;
        break;
      }
      const double p1 = std::abs(F[(size_t)m * mx]) * beta;
      const double p2 = std::abs(F[(size_t)(m + 1) * mx]) * beta * avnorm;
      if (p1 > 10.0 * p2) {
        err_loc = p2;
        xm = 1.0 / m;
      } else if (p1 > p2) {
        err_loc = (p1 * p2) / (p1 - p2);
        xm = 1.0 / m;
      } else {
        err_loc = p1;
        xm = 1.0 / (m - 1);
      }
      if (!std::isfinite(err_loc)) return set_err(op->ctx, KR_ERR_MAXORDER, "kr_expv: requested tolerance was too high");
      if (err_loc <= 1.2 * t_step * tol) break;
      t_step = round2(0.9 * t_step * std::pow(t_step * tol / err_loc, xm));
      ++nreject;
    }
    mx = mbrk + std::max(0, k1 - 1);
    KxCoef c;
    for (int i = 0; i < mx; ++i) {
      const cd v = beta * F[(size_t)i * (mbrk + k1)];
      c.c[i] = make_double2(v.real(), v.imag());
    }
    kx_combine<<<k.grid, KX_THREADS, 0, k.st>>>(k.V, n, mx, c, w);
    op->launches++;
    KR_CUDA(op->ctx, cudaGetLastError());
    t_new = round2(0.9 * t_step * std::pow(t_step * tol / err_loc, xm));
    t_now += t_step;
    if (nstep >= 500) {
      if (stats) {
        stats[0] = nstep;
        stats[1] = nmult;
        stats[2] = nreject;
      }
      return set_err(op->ctx, KR_ERR_MAXORDER, "kr_expv: maximum number of steps reached without convergence");
    }
  }
  if (stats) {
    stats[0] = nstep;
    stats[1] = nmult;
    stats[2] = nreject;
  }
  KR_CUDA(op->ctx, cudaStreamSynchronize(k.st));
  return KR_OK;
}
