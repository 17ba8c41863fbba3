// Vector-space operations on flat FP64 device vectors: the VectorInterface methods
// the reference defines for ITensors (ext/ITensorsVectorInterfaceExt/
// ITensorsVectorInterfaceExt.jl:5-84: inner, norm, scale / scale!, add / add!), and
// the two block forms a Krylov solver's classical Gram-Schmidt needs: the inner
// products of one vector with k basis vectors, and the update y += s * sum_j c_j v_j.
//
// All of them only launch kernels: scalars that feed later steps (norms, Gram-Schmidt
// coefficients, Lanczos alpha / beta) stay in device memory, so a whole Krylov
// iteration can be captured into one CUDA graph.  Reductions are deterministic: a
// fixed grid of CTAs writes per-CTA partial sums and a second kernel adds them in a
// fixed order (strided sums, then a fixed-shape tree), so a replay reproduces an eager
// run bit for bit.
//
// Every kernel streams its vectors once from HBM (the basis forms read k vectors and
// one or two more); the bound is HBM bandwidth, 8 bytes per element read or written.
#include "nd_common.h"
#include <algorithm>

namespace {

constexpr int VEC_THREADS = 256;
constexpr int VEC_KMAX = 32;       // basis vectors per dots / update call (a Krylov dimension)

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// part[b * k + j] = sum over this CTA's slice of x_i * V[j][i], j < k; the slice of
// CTA b is [b * chunk, (b + 1) * chunk), chunk a multiple of VEC_THREADS * U.  Each
// thread keeps U elements of x and U * k of the basis in flight per iteration (U * KT
// stays near 32 loads), which is what it takes to cover HBM latency with 2-4 CTAs per SM.
template <int KT>
__global__ void __launch_bounds__(VEC_THREADS) vec_dots_part(int64_t n, int k, const double* __restrict__ V,
                                                             int64_t ldv, const double* __restrict__ x,
                                                             int64_t chunk, double* __restrict__ part) {
  constexpr int U = KT <= 1 ? 8 : KT <= 8 ? 4 : KT <= 16 ? 2 : 1;
  __shared__ double red[VEC_THREADS / 32][KT];
  double acc[KT];
#pragma unroll
  for (int j = 0; j < KT; ++j) acc[j] = 0.0;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  for (int64_t base = i0 + threadIdx.x; base < i1; base += (int64_t)VEC_THREADS * U) {
    double xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * VEC_THREADS;
      xv[u] = i < i1 ? __ldg(x + i) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      if (j < k) {
        double vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = base + (int64_t)u * VEC_THREADS;
          vv[u] = i < i1 ? __ldg(V + (int64_t)j * ldv + i) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc[j] = fma(vv[u], xv[u], acc[j]);
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < KT; ++j) {
    if (j >= k) break;
    const double s = warp_sum_d(acc[j]);
    if (lane == 0) red[warp][j] = s;
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double s = 0.0;
    for (int w = 0; w < VEC_THREADS / 32; ++w) s += red[w][threadIdx.x];
    part[(int64_t)blockIdx.x * k + threadIdx.x] = s;
  }
}

// out[j] = sum_b part[b * k + j] (optionally the square root: a norm), one CTA per j:
// thread t adds the partials t, t + 256, ... in that order, then a fixed-shape tree adds
// the threads' sums, so the result does not depend on thread timing.  (One thread adding
// all partials in sequence was a chain of dependent FP64 adds and loads that took tens of
// microseconds.)
constexpr int FINAL_THREADS = 256;
__global__ void __launch_bounds__(FINAL_THREADS) vec_dots_final(int k, int nparts, const double* __restrict__ part,
                                                                double* out, int root) {
  __shared__ double red[FINAL_THREADS];
  const int j = blockIdx.x, t = threadIdx.x;
  double s = 0.0;
  for (int b = t; b < nparts; b += FINAL_THREADS) s += part[(int64_t)b * k + j];
  red[t] = s;
  __syncthreads();
#pragma unroll
  for (int w = FINAL_THREADS / 2; w > 0; w >>= 1) {
    if (t < w) red[t] += red[t + w];
    __syncthreads();
  }
  if (t == 0) out[j] = root ? sqrt(red[0]) : red[0];
}

// Elementwise kernels: each thread handles VEC_U elements VEC_THREADS apart per
// iteration, loads first, so VEC_U (times the basis size) loads are in flight.
constexpr int VEC_U = 4;

// y_i += sign * sum_j c_j V[j][i]
__global__ void __launch_bounds__(VEC_THREADS) vec_update(int64_t n, int k, const double* __restrict__ V, int64_t ldv,
                                                          const double* __restrict__ coef, double sign, double* y) {
  __shared__ double c[VEC_KMAX];
  if (threadIdx.x < k) c[threadIdx.x] = sign * coef[threadIdx.x];
  __syncthreads();
  const int64_t step = (int64_t)gridDim.x * VEC_THREADS * 2;
  for (int64_t base = (int64_t)blockIdx.x * VEC_THREADS * 2 + threadIdx.x; base < n; base += step) {
    const int64_t i1 = base + VEC_THREADS;
    double s0 = 0.0, s1 = 0.0;
    for (int j = 0; j < k; ++j) {
      const double* v = V + (int64_t)j * ldv;
      const double a = __ldg(v + base), b = i1 < n ? __ldg(v + i1) : 0.0;
      s0 = fma(c[j], a, s0);
      s1 = fma(c[j], b, s1);
    }
    y[base] += s0;
    if (i1 < n) y[i1] += s1;
  }
}

// y = alpha * x (* s or / s, s a device scalar when given)
__global__ void __launch_bounds__(VEC_THREADS) vec_scale(int64_t n, const double* x, double* y, double alpha,
                                                         const double* s, int invert) {
  double a = alpha;
  if (s) a = invert ? alpha / __ldg(s) : alpha * __ldg(s);
  const int64_t step = (int64_t)gridDim.x * VEC_THREADS * VEC_U;
  for (int64_t base = (int64_t)blockIdx.x * VEC_THREADS * VEC_U + threadIdx.x; base < n; base += step) {
    double v[VEC_U];
#pragma unroll
    for (int u = 0; u < VEC_U; ++u) {
      const int64_t i = base + (int64_t)u * VEC_THREADS;
      v[u] = i < n ? x[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < VEC_U; ++u) {
      const int64_t i = base + (int64_t)u * VEC_THREADS;
      if (i < n) y[i] = a * v[u];
    }
  }
}

// y = beta * y + alpha * x  (beta == 0 overwrites y, so NaN in y does not propagate)
__global__ void __launch_bounds__(VEC_THREADS) vec_add(int64_t n, const double* x, double* y, double alpha,
                                                       double beta) {
  const int64_t step = (int64_t)gridDim.x * VEC_THREADS * VEC_U;
  for (int64_t base = (int64_t)blockIdx.x * VEC_THREADS * VEC_U + threadIdx.x; base < n; base += step) {
    double xv[VEC_U], yv[VEC_U];
#pragma unroll
    for (int u = 0; u < VEC_U; ++u) {
      const int64_t i = base + (int64_t)u * VEC_THREADS;
      xv[u] = i < n ? x[i] : 0.0;
      yv[u] = (i < n && beta != 0.0) ? y[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < VEC_U; ++u) {
      const int64_t i = base + (int64_t)u * VEC_THREADS;
      if (i < n) y[i] = beta == 0.0 ? alpha * xv[u] : fma(alpha, xv[u], beta * yv[u]);
    }
  }
}

int vec_ctas(nd_handle h) { return 4 * h->num_sms; }   // upper bound of the reduction grid (partials buffer)

// Reduction grid of one instantiation: the CTAs that are resident at once (at most
// vec_ctas), so the fixed grid runs in one wave.  Queried once per instantiation.
template <int KT>
int dots_ctas(nd_handle h) {
  static const int per_sm = [] {    // initialised once, thread-safely
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vec_dots_part<KT>, VEC_THREADS, 0);
    return std::max(1, std::min(n, 4));
  }();
  return per_sm * h->num_sms;
}

nd_status vec_partials(nd_handle h, double** part) {
  // fixed per-handle buffer: the reductions must not allocate (they are captured in graphs)
  if (!h->vec_part) {
    if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "vector reductions: run one eagerly before graph capture");
    ND_CUDA(h, cudaMalloc(&h->vec_part, (size_t)vec_ctas(h) * VEC_KMAX * sizeof(double)));
  }
  *part = (double*)h->vec_part;
  return ND_OK;
}

nd_status dots(nd_handle h, int64_t n, int32_t k, const double* V, int64_t ldv, const double* x, double* out,
               int root, const char* name) {
  if (n < 0 || k < 1 || k > VEC_KMAX) return nd_fail(h, ND_ERR_ARG, "%s: need n >= 0 and 1 <= k <= %d", name, VEC_KMAX);
  if (!V || !x || !out || (k > 1 && ldv < n)) return nd_fail(h, ND_ERR_ARG, "%s: NULL pointer or ldv < n", name);
  double* part = nullptr;
  nd_status s = vec_partials(h, &part);
  if (s) return s;
  const int ctas = k <= 1 ? dots_ctas<1>(h) : k <= 8 ? dots_ctas<8>(h) : k <= 16 ? dots_ctas<16>(h) : dots_ctas<32>(h);
  // chunk: a multiple of VEC_THREADS * 8 (every unroll factor divides it)
  constexpr int64_t q = VEC_THREADS * 8;
  int64_t chunk = (n + ctas - 1) / ctas;
  chunk = std::max<int64_t>(q, (chunk + q - 1) / q * q);
  nd_prof_begin(h, "vec_dots");
  if (k <= 1) vec_dots_part<1><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else if (k <= 8) vec_dots_part<8><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else if (k <= 16) vec_dots_part<16><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else vec_dots_part<32><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  vec_dots_final<<<k, FINAL_THREADS, 0, h->stream>>>(k, ctas, part, out, root);
  nd_prof_end(h);
  h->launches += 2;
  return nd_cuda_check(h, cudaGetLastError(), name);
}

int grid_for(nd_handle h, int64_t n, int per_thread) {
  const int64_t per_cta = (int64_t)VEC_THREADS * per_thread;
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + per_cta - 1) / per_cta, (int64_t)h->num_sms * 8));
}

// Lowest eigenpair of the k x k symmetric tridiagonal matrix with diagonal a and
// off-diagonal b (a Lanczos matrix), one thread: bisection on the Sturm count of
// T - x I (Barth, Martin and Wilkinson, "Calculation of the eigenvalues of a symmetric
// tridiagonal matrix by the method of bisection", Numer. Math. 9, 1967) to the
// resolution of double precision, then three steps of inverse iteration with the
// Thomas algorithm (near-zero pivots replaced by eps * ||T||, as inverse iteration
// codes do).  The vector is normalised with its largest component positive; the value
// is its Rayleigh quotient.
__global__ void tridiag_lowest(int k, const double* __restrict__ a, const double* __restrict__ b, double* value,
                               double* y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lo = 0.0, hi = 0.0, nrm = 0.0;
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i < k - 1 ? fabs(b[i]) : 0.0);
    lo = i ? fmin(lo, a[i] - r) : a[i] - r;
    hi = i ? fmax(hi, a[i] + r) : a[i] + r;
    nrm = fmax(nrm, fabs(a[i]) + r);
  }
  const double tiny = 2.2250738585072014e-308 / 2.220446049250313e-16;   // safe pivot floor
  for (int it = 0; it < 2100; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    int count = 0;
    double q = a[0] - mid;
    if (q < 0.0) ++count;
    for (int i = 1; i < k; ++i) {
      if (fabs(q) < tiny) q = -tiny;
      q = a[i] - mid - b[i - 1] * b[i - 1] / q;
      if (q < 0.0) ++count;
    }
    if (count >= 1) hi = mid; else lo = mid;
  }
  const double lam = 0.5 * (lo + hi);
  const double piv = 2.220446049250313e-16 * fmax(nrm, tiny);
  double x[32], c[32], d[32];
  for (int i = 0; i < k; ++i) x[i] = 1.0;
  for (int step = 0; step < 3; ++step) {
    // solve (T - lam I) z = x (Thomas), z into x
    double den = a[0] - lam;
    if (fabs(den) < piv) den = den < 0 ? -piv : piv;
    c[0] = k > 1 ? b[0] / den : 0.0;
    d[0] = x[0] / den;
    for (int i = 1; i < k; ++i) {
      den = a[i] - lam - b[i - 1] * c[i - 1];
      if (fabs(den) < piv) den = den < 0 ? -piv : piv;
      c[i] = i < k - 1 ? b[i] / den : 0.0;
      d[i] = (x[i] - b[i - 1] * d[i - 1]) / den;
    }
    x[k - 1] = d[k - 1];
    for (int i = k - 2; i >= 0; --i) x[i] = d[i] - c[i] * x[i + 1];
    double s = 0.0;
    for (int i = 0; i < k; ++i) s = fmax(s, fabs(x[i]));
    for (int i = 0; i < k; ++i) x[i] /= s;
  }
  double n2 = 0.0, big = 0.0;
  int ib = 0;
  for (int i = 0; i < k; ++i) {
    n2 += x[i] * x[i];
    if (fabs(x[i]) > big) { big = fabs(x[i]); ib = i; }
  }
  const double sc = (x[ib] < 0 ? -1.0 : 1.0) / sqrt(n2);
  double rq = 0.0;
  for (int i = 0; i < k; ++i) {
    x[i] *= sc;
    y[i] = x[i];
  }
  for (int i = 0; i < k; ++i) {
    double tx = a[i] * x[i];
    if (i > 0) tx += b[i - 1] * x[i - 1];
    if (i < k - 1) tx += b[i] * x[i + 1];
    rq += x[i] * tx;
  }
  *value = rq;
}

}  // namespace

extern "C" nd_status nd_vec_inner_f64(nd_handle h, int64_t n, const double* x, const double* y, double* out) {
  if (!h) return ND_ERR_ARG;
  return dots(h, n, 1, x, n, y, out, 0, "vec_inner");
}

extern "C" nd_status nd_vec_norm_f64(nd_handle h, int64_t n, const double* x, double* out) {
  if (!h) return ND_ERR_ARG;
  return dots(h, n, 1, x, n, x, out, 1, "vec_norm");
}

extern "C" nd_status nd_vec_dots_f64(nd_handle h, int64_t n, int32_t k, const double* V, int64_t ldv, const double* x,
                                     double* out) {
  if (!h) return ND_ERR_ARG;
  return dots(h, n, k, V, ldv, x, out, 0, "vec_dots");
}

extern "C" nd_status nd_vec_update_f64(nd_handle h, int64_t n, int32_t k, const double* V, int64_t ldv,
                                       const double* coef, double sign, double* y) {
  if (!h) return ND_ERR_ARG;
  if (n < 0 || k < 1 || k > VEC_KMAX) return nd_fail(h, ND_ERR_ARG, "vec_update: need n >= 0 and 1 <= k <= %d", VEC_KMAX);
  if (!V || !coef || !y || (k > 1 && ldv < n)) return nd_fail(h, ND_ERR_ARG, "vec_update: NULL pointer or ldv < n");
  if (n == 0) return ND_OK;
  nd_prof_begin(h, "vec_update");
  vec_update<<<grid_for(h, n, 2), VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, coef, sign, y);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "vec_update");
}

extern "C" nd_status nd_vec_scale_f64(nd_handle h, int64_t n, const double* x, double* y, double alpha,
                                      const double* s, int32_t invert) {
  if (!h) return ND_ERR_ARG;
  if (n < 0 || (n && (!x || !y))) return nd_fail(h, ND_ERR_ARG, "vec_scale: NULL pointer");
  if (n == 0) return ND_OK;
  nd_prof_begin(h, "vec_scale");
  vec_scale<<<grid_for(h, n, VEC_U), VEC_THREADS, 0, h->stream>>>(n, x, y, alpha, s, invert);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "vec_scale");
}

extern "C" nd_status nd_vec_add_f64(nd_handle h, int64_t n, const double* x, double* y, double alpha, double beta) {
  if (!h) return ND_ERR_ARG;
  if (n < 0 || (n && (!x || !y))) return nd_fail(h, ND_ERR_ARG, "vec_add: NULL pointer");
  if (n == 0) return ND_OK;
  nd_prof_begin(h, "vec_add");
  vec_add<<<grid_for(h, n, VEC_U), VEC_THREADS, 0, h->stream>>>(n, x, y, alpha, beta);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "vec_add");
}

extern "C" nd_status nd_tridiag_lowest_f64(nd_handle h, int32_t k, const double* alpha, const double* beta,
                                          double* value, double* y) {
  if (!h) return ND_ERR_ARG;
  if (k < 1 || k > 32 || !alpha || !value || !y || (k > 1 && !beta))
    return nd_fail(h, ND_ERR_ARG, "tridiag_lowest: need 1 <= k <= 32 and device arrays");
  nd_prof_begin(h, "tridiag_lowest");
  tridiag_lowest<<<1, 32, 0, h->stream>>>(k, alpha, beta, value, y);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "tridiag_lowest");
}
