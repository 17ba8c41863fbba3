// Vector-space operations on flat FP64 device vectors: the VectorInterface methods
// the reference defines for ITensors (ext/ITensorsVectorInterfaceExt/
// ITensorsVectorInterfaceExt.jl:5-84: inner, norm, scale / scale!, add / add!), and
// the two block forms a Krylov solver's classical Gram-Schmidt needs: the inner
// products of one vector with k basis vectors, and the update y += s * sum_j c_j v_j.
//
// All of them only launch kernels: scalars that feed later steps (norms, Gram-Schmidt
// coefficients, Lanczos alpha / beta) stay in device memory, so a whole Krylov
// iteration can be captured into one CUDA graph.  Reductions are deterministic: a
// fixed grid of VEC_CTAS CTAs writes per-CTA partial sums in a fixed order and one
// CTA adds them in that order, so a replay reproduces an eager run bit for bit.
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
// CTA b is [b * chunk, (b + 1) * chunk), chunk a multiple of the block size.
template <int KT>
__global__ void __launch_bounds__(VEC_THREADS) vec_dots_part(int64_t n, int k, const double* __restrict__ V,
                                                             int64_t ldv, const double* __restrict__ x,
                                                             int64_t chunk, double* __restrict__ part) {
  __shared__ double red[VEC_THREADS / 32][KT];
  double acc[KT];
#pragma unroll
  for (int j = 0; j < KT; ++j) acc[j] = 0.0;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  for (int64_t i = i0 + threadIdx.x; i < i1; i += VEC_THREADS) {
    const double xi = __ldg(x + i);
#pragma unroll
    for (int j = 0; j < KT; ++j)
      if (j < k) acc[j] = fma(__ldg(V + (int64_t)j * ldv + i), xi, acc[j]);
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

// out[j] = sum_b part[b * k + j] in b order (optionally the square root: a norm)
__global__ void vec_dots_final(int k, int nparts, const double* __restrict__ part, double* out, int root) {
  const int j = threadIdx.x;
  if (j >= k) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[(int64_t)b * k + j];
  out[j] = root ? sqrt(s) : s;
}

// y_i += sign * sum_j c_j V[j][i]
__global__ void __launch_bounds__(VEC_THREADS) vec_update(int64_t n, int k, const double* __restrict__ V, int64_t ldv,
                                                          const double* __restrict__ coef, double sign, double* y) {
  __shared__ double c[VEC_KMAX];
  if (threadIdx.x < k) c[threadIdx.x] = sign * coef[threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s = fma(c[j], __ldg(V + (int64_t)j * ldv + i), s);
    y[i] += s;
  }
}

// y = alpha * x (* s or / s, s a device scalar when given)
__global__ void __launch_bounds__(VEC_THREADS) vec_scale(int64_t n, const double* x, double* y, double alpha,
                                                         const double* s, int invert) {
  double a = alpha;
  if (s) a = invert ? alpha / __ldg(s) : alpha * __ldg(s);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

// y = beta * y + alpha * x  (beta == 0 overwrites y, so NaN in y does not propagate)
__global__ void __launch_bounds__(VEC_THREADS) vec_add(int64_t n, const double* x, double* y, double alpha,
                                                       double beta) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = beta == 0.0 ? alpha * x[i] : fma(alpha, x[i], beta * y[i]);
}

int vec_ctas(nd_handle h) { return 2 * h->num_sms; }

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
  const int ctas = vec_ctas(h);
  int64_t chunk = (n + ctas - 1) / ctas;
  chunk = std::max<int64_t>(VEC_THREADS, (chunk + VEC_THREADS - 1) / VEC_THREADS * VEC_THREADS);
  nd_prof_begin(h, "vec_dots");
  if (k <= 1) vec_dots_part<1><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else if (k <= 8) vec_dots_part<8><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else if (k <= 16) vec_dots_part<16><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  else vec_dots_part<32><<<ctas, VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, x, chunk, part);
  vec_dots_final<<<1, VEC_KMAX, 0, h->stream>>>(k, ctas, part, out, root);
  nd_prof_end(h);
  h->launches += 2;
  return nd_cuda_check(h, cudaGetLastError(), name);
}

int grid_for(nd_handle h, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + VEC_THREADS - 1) / VEC_THREADS, (int64_t)h->num_sms * 8));
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
  vec_update<<<grid_for(h, n), VEC_THREADS, 0, h->stream>>>(n, k, V, ldv, coef, sign, y);
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
  vec_scale<<<grid_for(h, n), VEC_THREADS, 0, h->stream>>>(n, x, y, alpha, s, invert);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "vec_scale");
}

extern "C" nd_status nd_vec_add_f64(nd_handle h, int64_t n, const double* x, double* y, double alpha, double beta) {
  if (!h) return ND_ERR_ARG;
  if (n < 0 || (n && (!x || !y))) return nd_fail(h, ND_ERR_ARG, "vec_add: NULL pointer");
  if (n == 0) return ND_OK;
  nd_prof_begin(h, "vec_add");
  vec_add<<<grid_for(h, n), VEC_THREADS, 0, h->stream>>>(n, x, y, alpha, beta);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "vec_add");
}
