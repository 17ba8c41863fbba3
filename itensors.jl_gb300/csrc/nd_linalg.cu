// Blockwise SVD / QR of a 2-index block matrix, truncation, and block copies
// (combiner gather / scatter), FP64 on the GPU.
//
// Reference behaviour:
//   svd(::Tensor{ElT,2,<:BlockSparse})   NDTensors/src/blocksparse/linearalgebra.jl:45-215
//     per-block dense SVD, all s^2 pooled and sorted descending, truncate!!, per-block
//     kept dims (_truncated_blockdim, :8-33), zero-kept blocks dropped
//   truncate!                             NDTensors/src/truncate.jl:23-107
//   qr / qx                               NDTensors/src/blocksparse/linearalgebra.jl:351-415,
//                                         NDTensors/src/linearalgebra/linearalgebra.jl:321-381
//
// SVD algorithm: one-sided (Hestenes) Jacobi on the columns of every block at
// once (transposed when a block is wide).  Column groups of B follow a round-robin
// tournament; one CTA rotates the pairs of a group pair inside shared memory
// (bj_sweep), and all blocks advance round by round inside one persistent
// cooperative kernel whose CTAs meet at a grid barrier (bounded spin) between
// rounds (blocks too tall for a shared-memory panel use the scalar sweep,
// svd_sweep: one warp per column pair, columns in global memory).  Each sweep
// records the largest |a_i . a_j| / (|a_i| |a_j|) per block; blocks whose sweep
// rotated nothing are done, and the host reports ND_ERR_NOCONV after the sweep
// limit (the reference returns `nothing` when LAPACK fails).  Larger problems first
// run the sweeps in FP32, refine that V to FP64 accuracy with split GEMMs on the
// tensor cores (Ogita-Aishima refinement), then finish with FP64 sweeps on W V, so
// the result is an FP64 Jacobi SVD.
#include "nd_plan.h"
#include <cooperative_groups.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace {

inline double bits_to_double(unsigned long long u) {
  double d;
  memcpy(&d, &u, 8);
  return d;
}

struct SvdBlock {
  int64_t a_off;     // offset of the block in A (column-major m x n, original orientation)
  int64_t w_off;     // offset of the working matrix W (mm x nn, column-major, mm >= nn)
  int64_t v_off;     // offset of V (nn x nn)
  int32_t m, n;      // original dims
  int32_t mm, nn;    // working dims (transposed if m < n)
  int32_t trans;     // 1 if W = A^T
  int32_t npad;      // nn rounded up to even
  int32_t task0;     // first task index of this block in a round
  int32_t ntask;     // npad / 2
  int32_t s_off;     // offset of its singular values in the pooled vector
  int32_t pad;
};

__device__ __forceinline__ double block_reduce_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < (blockDim.x >> 5)) t = red[threadIdx.x];
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  return red[0];
}

// W = A or A^T, V = I
__global__ void svd_init(const SvdBlock* blocks, int nb, const double* A, double* W, double* V) {
  const SvdBlock b = blocks[blockIdx.y];
  const int64_t tot = (int64_t)b.mm * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % b.mm, j = e / b.mm;
    // W(i,j) = trans ? A(j,i) : A(i,j)
    W[b.w_off + e] = b.trans ? A[b.a_off + i * b.m + j] : A[b.a_off + e];
  }
  const int64_t tv = (int64_t)b.nn * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tv; e += (int64_t)gridDim.x * blockDim.x)
    V[b.v_off + e] = (e % b.nn == e / b.nn) ? 1.0 : 0.0;
}

// round-robin tournament: round r, pair k of npad players -> (p, q)
__device__ __forceinline__ void rr_pair(int npad, int r, int k, int& p, int& q) {
  auto pos = [&](int idx) { return idx == 0 ? 0 : ((r + idx - 1) % (npad - 1)) + 1; };
  p = pos(k);
  q = pos(npad - 1 - k);
}

// Bounded grid barrier for a cooperative launch.
__device__ __forceinline__ bool grid_barrier(unsigned int* count, volatile unsigned int* gen, unsigned int nblocks,
                                             DeviceStatus* st) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned int g = *gen;
    __threadfence();
    if (atomicAdd(count, 1u) == nblocks - 1) {
      *count = 0;
      __threadfence();
      atomicAdd((unsigned int*)gen, 1u);
    } else {
      unsigned int it = 0;
      const unsigned int lim = nd_spin_limit(st);
      while (*gen == g) {
        if (++it > lim) {
          if (atomicCAS(&st->code, 0, ND_ERR_TIMEOUT) == 0) st->where = 500;
          ok = 0;
          break;
        }
        if ((it & 1023) == 0 && *(volatile int32_t*)&st->code == ND_ERR_TIMEOUT) { ok = 0; break; }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <typename T>
struct SweepArgs {
  const SvdBlock* blocks;
  int nb;
  int ntasks;        // tasks per round (sum of npad/2)
  int nrounds;       // max npad - 1
  T* W;
  T* V;
  T* nrm;            // |w_j|^2 per column (pooled like the singular values), updated by every rotation
  const int32_t* active;        // per block: 0 once a sweep left it without rotations (converged)
  unsigned long long* offmax;   // per block, bits of the largest relative off-diagonal (as a double) this sweep
  unsigned int* bar_count;
  unsigned int* bar_gen;
  DeviceStatus* st;
  double tol;        // rotations below min(tol * mm^tol_pow, tol_cap) are skipped
  double tol_pow;
  double tol_cap;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// |w_j|^2 of every column of the active blocks (one warp per column), at the start of a sweep.
template <typename T>
__global__ void __launch_bounds__(256) svd_norms(const SvdBlock* blocks, int nb, const int32_t* active,
                                                 const T* W, T* nrm, int total_cols) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int c = gw; c < total_cols; c += nw) {
    int bi = 0;
    while (bi + 1 < nb && blocks[bi + 1].s_off <= c) ++bi;
    if (!active[bi]) continue;
    const SvdBlock& b = blocks[bi];
    const T* w = W + b.w_off + (int64_t)(c - b.s_off) * b.mm;
    constexpr int CH = sizeof(T) == 4 ? 16 : 8;
    T acc = 0;
    for (int base = lane; base < b.mm; base += 32 * CH) {
      T x[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) { const int i = base + 32 * u; x[u] = i < b.mm ? w[i] : T(0); }
#pragma unroll
      for (int u = 0; u < CH; ++u) acc = fma(x[u], x[u], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) nrm[c] = acc;
  }
}

// (x, y) <- (c x - s y, s x + c y) over n elements, one warp, CH loads per lane in flight.
template <typename T, int CH>
__device__ __forceinline__ void rotate_batched(T* xp, T* yp, int n, int lane, T c, T s) {
  for (int base = lane; base < n; base += 32 * CH) {
    T x[CH], y[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int i = base + 32 * u;
      x[u] = i < n ? __ldcg(xp + i) : T(0);
      y[u] = i < n ? __ldcg(yp + i) : T(0);
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int i = base + 32 * u;
      if (i < n) {
        xp[i] = c * x[u] - s * y[u];
        yp[i] = s * x[u] + c * y[u];
      }
    }
  }
}

// One sweep: every round, one warp per column pair (p, q) of every active block:
// gamma = w_p . w_q, the Jacobi rotation from (|w_p|^2, |w_q|^2, gamma), applied
// to the two columns of W and of V.  The squared norms follow the exact
// identities |w_p'|^2 = |w_p|^2 - t gamma, |w_q'|^2 = |w_q|^2 + t gamma, so a
// pair costs one dot product instead of three; they are recomputed every sweep.
template <typename T>
__global__ void __launch_bounds__(512, 2) svd_sweep(SweepArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = 0; r < a.nrounds; ++r) {
    for (int t = gw; t < a.ntasks; t += nw) {
      int bi = 0;
      while (bi + 1 < a.nb && a.blocks[bi + 1].task0 <= t) ++bi;
      const SvdBlock& b = a.blocks[bi];
      if (r >= b.npad - 1 || !a.active[bi]) continue;   // block has fewer rounds / has converged
      int p, q;
      rr_pair(b.npad, r, t - b.task0, p, q);
      if (p >= b.nn || q >= b.nn) continue;            // dummy column
      if (p > q) { int x = p; p = q; q = x; }
      T* wp = a.W + b.w_off + (int64_t)p * b.mm;
      T* wq = a.W + b.w_off + (int64_t)q * b.mm;
      // loads are batched CH per lane so a column costs a few memory round trips, not one per element
      constexpr int CH = sizeof(T) == 4 ? 16 : 8;
      T ga = 0;
      for (int base = lane; base < b.mm; base += 32 * CH) {
        T x[CH], y[CH];
#pragma unroll
        for (int u = 0; u < CH; ++u) {
          const int i = base + 32 * u;
          x[u] = i < b.mm ? __ldcg(wp + i) : T(0);   // L2: other CTAs rotate these columns too
          y[u] = i < b.mm ? __ldcg(wq + i) : T(0);
        }
#pragma unroll
        for (int u = 0; u < CH; ++u) ga = fma(x[u], y[u], ga);
      }
      ga = warp_sum(ga);
      const T al = __ldcg(a.nrm + b.s_off + p), be = __ldcg(a.nrm + b.s_off + q);
      const T nrm = sqrt(al) * sqrt(be);
      T rel = nrm > T(0) ? fabs(ga) / nrm : T(0);
      // tol_pow is 1 or 1/2; tolerance math in T (the FP64 pipe is narrow on this part)
      const T tolb = min((T)a.tol_cap, (T)a.tol * (a.tol_pow != 1.0 ? sqrt((T)b.mm) : (T)b.mm));
      if (rel > tolb && ga != T(0)) {
        const T zeta = (be - al) / (T(2) * ga);
        const T tt = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + tt * tt);
        const T s = c * tt;
        rotate_batched<T, CH>(wp, wq, b.mm, lane, c, s);
        rotate_batched<T, CH>(a.V + b.v_off + (int64_t)p * b.nn, a.V + b.v_off + (int64_t)q * b.nn, b.nn, lane, c, s);
        if (lane == 0) {
          a.nrm[b.s_off + p] = al - tt * ga;
          a.nrm[b.s_off + q] = be + tt * ga;
        }
      } else {
        rel = T(0);
      }
      if (lane == 0 && rel > T(0)) atomicMax(&a.offmax[bi], (unsigned long long)__double_as_longlong((double)rel));
    }
    if (!grid_barrier(a.bar_count, a.bar_gen, gridDim.x, a.st)) return;
  }
}

// Largest |W| of every block (IEEE bits), for the power-of-two scaling of the FP32 copy.
__global__ void block_absmax(const SvdBlock* blocks, const double* W, unsigned long long* mx) {
  const SvdBlock b = blocks[blockIdx.y];
  const int64_t tot = (int64_t)b.mm * b.nn;
  unsigned long long m = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = (unsigned long long)__double_as_longlong(W[b.w_off + e]) & 0x7fffffffffffffffull;
    m = v > m ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) { const unsigned long long u = __shfl_xor_sync(0xffffffffu, m, o); m = u > m ? u : m; }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(&mx[blockIdx.y], m);
}

// W32 = W * 2^-E_b (E_b: exponent of the block's largest |W|), V32 = I.
__global__ void to_f32_scaled(const SvdBlock* blocks, const double* W, const unsigned long long* mx, float* W32,
                              float* V32) {
  const SvdBlock b = blocks[blockIdx.y];
  const int ex = (int)(mx[blockIdx.y] >> 52);
  const double sc = ex ? ldexp(1.0, 1023 - ex) : 1.0;
  const int64_t tot = (int64_t)b.mm * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
    W32[b.w_off + e] = (float)(W[b.w_off + e] * sc);
  const int64_t tv = (int64_t)b.nn * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tv; e += (int64_t)gridDim.x * blockDim.x)
    V32[b.v_off + e] = (e % b.nn == e / b.nn) ? 1.0f : 0.0f;
}

// sigma_j = |w_j|, then per-block descending order (rank by comparison; ties by index)
__global__ void svd_finish(const SvdBlock* blocks, const double* W, double* sig, int32_t* order) {
  const SvdBlock b = blocks[blockIdx.x];
  __shared__ double red[8];
  extern __shared__ double s_sig[];
  for (int j = 0; j < b.nn; ++j) {
    const double* w = W + b.w_off + (int64_t)j * b.mm;
    double acc = 0.0;
    for (int i = threadIdx.x; i < b.mm; i += blockDim.x) acc = fma(w[i], w[i], acc);
    acc = block_reduce_sum(acc, red);
    if (threadIdx.x == 0) s_sig[j] = sqrt(acc);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < b.nn; j += blockDim.x) {
    const double v = s_sig[j];
    int rank = 0;
    for (int k = 0; k < b.nn; ++k) {
      const double u = s_sig[k];
      rank += (u > v) || (u == v && k < j);
    }
    order[b.s_off + rank] = j;
    sig[b.s_off + rank] = v;
  }
}

// U (m x k) and V (n x k) of the original block, columns in descending order.
__global__ void svd_outputs(const SvdBlock* blocks, const double* W, const double* Vw, const double* sig,
                            const int32_t* order, double* Ufull, double* Vfull, const int64_t* u_off,
                            const int64_t* v_off) {
  const SvdBlock b = blocks[blockIdx.y];
  const int k = b.nn;                      // min(m, n)
  // left vectors of the working matrix: w_j / sigma_j ; right vectors: V_w columns
  const int64_t totl = (int64_t)b.mm * k, totr = (int64_t)b.nn * k;
  double* Ul = b.trans ? Vfull + v_off[blockIdx.y] : Ufull + u_off[blockIdx.y];   // mm x k
  double* Ur = b.trans ? Ufull + u_off[blockIdx.y] : Vfull + v_off[blockIdx.y];   // nn x k
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < totl; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % b.mm, c = e / b.mm;
    const int j = order[b.s_off + c];
    const double s = sig[b.s_off + c];
    Ul[e] = s > 0.0 ? W[b.w_off + (int64_t)j * b.mm + i] / s : 0.0;
  }
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < totr; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % b.nn, c = e / b.nn;
    const int j = order[b.s_off + c];
    Ur[e] = Vw[b.v_off + (int64_t)j * b.nn + i];
  }
}

// ---- pooled spectrum: sort s^2 descending (bitonic, one CTA) + truncate! -----
struct TruncParams {
  int32_t mindim, maxdim;        // maxdim < 0: nothing
  double cutoff;                 // < 0 (with has_cutoff = 0): nothing
  int32_t has_cutoff, use_abs, use_rel;
};

__device__ void truncate_serial(double* P, int n, const TruncParams& tp, int* newlen, double* truncerr,
                                double* docut) {
  // NDTensors/src/truncate.jl:23-107, one thread
  const int mindim = tp.mindim;
  const int maxdim = tp.maxdim < 0 ? n : tp.maxdim;
  const double cutoff = tp.has_cutoff ? tp.cutoff : -INFINITY;
  *docut = 0.0;
  if (n == 1) { *newlen = 1; *truncerr = 0.0; *docut = fabs(P[0]) / 2; return; }
  const double s = P[0] < 0.0 ? -1.0 : 1.0;
  if (s < 0) for (int i = 0; i < n; ++i) P[i] *= s;
  for (int i = n - 1; i >= 0; --i) { if (P[i] >= 0.0) break; P[i] = 0.0; }
  int k = n;
  double te = 0.0;
  while (k > maxdim) { te += P[k - 1]; --k; }
  if (tp.use_abs) {
    while (P[k - 1] <= cutoff && k > mindim) { te += P[k - 1]; --k; }
  } else {
    double scale = 1.0;
    if (tp.use_rel) {
      scale = 0.0;
      for (int i = 0; i < n; ++i) scale += P[i];
      if (scale == 0.0) scale = 1.0;
    }
    while ((te + P[k - 1] <= cutoff * scale) && (k > mindim)) { te += P[k - 1]; --k; }
    te /= scale;
  }
  if (k < 1) k = 1;
  if (k < n) {
    double dc = (P[k - 1] + P[k]) / 2;
    if (fabs(P[k - 1] - P[k]) < 1.0e-3 * P[k - 1]) dc += 1.0e-3 * P[k - 1];
    *docut = dc;
  }
  if (s < 0) for (int i = 0; i < n; ++i) P[i] *= s;
  *newlen = k;
  *truncerr = te;
}

__global__ void __launch_bounds__(1024) sort_truncate(const double* sig, int n, int npow2, int squared, int do_sort,
                                                      TruncParams tp, double* P_out, int* newlen, double* truncerr,
                                                      double* docut) {
  extern __shared__ double P[];
  for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
    double v = -INFINITY;
    if (i < n) { v = sig[i]; if (squared) v = v * v; }
    P[i] = v;
  }
  __syncthreads();
  // bitonic sort, descending
  for (int k = 2; do_sort && k <= npow2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool desc = (i & k) == 0;
          const double a = P[i], b = P[l];
          if (desc ? (a < b) : (a > b)) { P[i] = b; P[l] = a; }
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    if (tp.maxdim >= 0 || tp.has_cutoff) truncate_serial(P, n, tp, newlen, truncerr, docut);
    else { *newlen = n; *truncerr = 0.0; *docut = 0.0; }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) P_out[i] = P[i];
}

// kept dims per block (_truncated_blockdim, NDTensors/src/blocksparse/linearalgebra.jl:8-33)
// squared = 1: singular values (s^2 > docut); 0: eigenvalues (|lambda| > docut)
__global__ void kept_dims(const SvdBlock* blocks, int nb, const double* sig, const double* docut, int min_blockdim,
                          int truncate, int32_t* kept, int squared = 1) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= nb) return;
  const SvdBlock b = blocks[bi];
  const int full = b.nn;
  if (!truncate) { kept[bi] = full; return; }
  const int mb = min(min_blockdim, full);
  int k = 0;
  while (k < full) {
    const double v = sig[b.s_off + k];
    if (!((squared ? v * v : fabs(v)) > *docut)) break;
    ++k;
  }
  if (k < mb) k = mb;
  kept[bi] = k;
}

// ---- block copy (combiner gather / uncombine scatter) ----------------------
struct BlockCopyDev {
  int64_t src_off, dst_off, count;
  int64_t start;      // first index of this copy in the flat element space of the list
  Mixed idx;          // st0: source strides, st1: destination strides
};

// All copies of a list as one flat element space (copy r covers [start_r, start_r +
// count_r)).  CTA b takes the contiguous range [b chunk, (b + 1) chunk), so a list of
// many small copies and a few large ones keeps every CTA busy; a thread finds its copy
// by binary search once and then walks forward.  Destination elements of a copy are
// consecutive in its column-major index, so writes coalesce wherever the destination is
// contiguous along the copy's first dimension.
__global__ void __launch_bounds__(256) block_copy(const BlockCopyDev* list, int n, int64_t total, int64_t chunk,
                                                  const double* src, double* dst) {
  const int64_t t0 = (int64_t)blockIdx.x * chunk, t1 = min(total, t0 + chunk);
  int64_t t = t0 + threadIdx.x;
  if (t >= t1) return;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (list[mid].start <= t) lo = mid;
    else hi = mid - 1;
  }
  int r = lo;
  for (; t < t1; t += blockDim.x) {
    while (r + 1 < n && list[r + 1].start <= t) ++r;
    const BlockCopyDev& c = list[r];
    const int64_t e = t - c.start;
    int64_t so, d;
    if (c.count < (1ll << 31)) mixed_offsets32(c.idx, (uint32_t)e, so, d);
    else mixed_offsets(c.idx, e, so, d);
    dst[c.dst_off + d] = src[c.src_off + so];
  }
}

// grid and chunk of a flat copy launch: about 2048 elements per CTA, at most 64 CTAs per SM
static void block_copy_grid(nd_handle h, int64_t total, int& grid, int64_t& chunk) {
  const int64_t g = std::max<int64_t>(1, std::min<int64_t>((total + 2047) / 2048, 64ll * h->num_sms));
  chunk = ((total + g - 1) / g + 255) / 256 * 256;
  grid = (int)((total + chunk - 1) / chunk);
}

// Per-block kernels index their block by blockIdx.y (at most 65535): a factorisation
// call takes at most that many blocks (a QN block matrix has one per charge sector).
constexpr int kMaxBlocksPerCall = 65535;

// ---- blocked Householder QR ----------------------------------------------
// Panels of QR_NB columns: one CTA per block computes the panel's reflectors (LAPACK
// dlarfg convention, as geqrf) and its compact WY factor T, Q_p = H_1 ... H_w =
// I - V T V^T (dlarft, forward columnwise); the trailing columns are then updated as
// C <- Q_p^T C = C - V (T^T (V^T C)) by CTAs that each own QR_SW columns of one block, so
// the large blocks' O(n^3) updates spread over the SMs.  The thin Q is accumulated
// backward from [I; 0]: X <- Q_p X = X - V (T (V^T X)), p from the last panel down,
// with the same strip kernel.  Everything is FP64 on the CUDA cores (GB300's FP64 pipe
// is narrow; the strip kernel keeps it busy from shared memory).
constexpr int QR_NB = 16, QR_SW = 8, QR_RC = 64;    // panel width, strip width, rows per chunk
constexpr int QR_THREADS = 256;                        // panel kernel
constexpr int QR_ATHREADS = 128;                       // strip kernel
constexpr int QR_OPT = QR_NB * QR_SW / QR_ATHREADS;   // V^T X outputs per thread
static_assert(QR_OPT >= 1 && QR_OPT * QR_ATHREADS == QR_NB * QR_SW, "whole V^T X outputs per thread");

struct QrBlock {
  int64_t a_off, w_off, q_off, r_off, t_off;   // t_off: one QR_NB x QR_NB factor per panel
  int32_t m, n, k;
  int32_t tau_off;
};

struct QrTask {
  int32_t block, col0, ncols, pad;
};

// W <- A (working copy), Q <- [I_k; 0]
__global__ void qr_init(const QrBlock* blocks, const double* A, double* Wk, double* Q) {
  const QrBlock b = blocks[blockIdx.y];
  const int64_t mn = (int64_t)b.m * b.n, mk = (int64_t)b.m * b.k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x)
    Wk[b.w_off + e] = A[b.a_off + e];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mk; e += (int64_t)gridDim.x * blockDim.x)
    Q[b.q_off + e] = (e % b.m) == (e / b.m) ? 1.0 : 0.0;
}

// Panel p of block ids[blockIdx.x]: reflectors of columns c0 .. c0 + w - 1 (applied
// within the panel only), then T.
__global__ void __launch_bounds__(QR_THREADS) qr_panel(const QrBlock* blocks, const int32_t* ids, int p, double* Wk,
                                                       double* tau_all, double* Tall) {
  const QrBlock b = blocks[ids[blockIdx.x]];
  const int c0 = p * QR_NB, w = min(QR_NB, b.k - c0);
  __shared__ double red[8];
  __shared__ double sh[4];
  __shared__ double G[QR_NB][QR_NB + 1];
  __shared__ double Ts[QR_NB][QR_NB + 1];
  double* W = Wk + b.w_off;
  double* tau = tau_all + b.tau_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int jj = 0; jj < w; ++jj) {
    const int j = c0 + jj;
    double* x = W + (int64_t)j * b.m;
    double ss = 0.0;
    for (int i = j + 1 + threadIdx.x; i < b.m; i += blockDim.x) ss = fma(x[i], x[i], ss);
    ss = block_reduce_sum(ss, red);
    if (threadIdx.x == 0) {
      // dlarfg: beta = -sign(alpha) * |x|, v(0) = 1, tau = (beta - alpha) / beta
      const double alpha = x[j];
      double t = 0.0, beta = alpha, scal = 0.0;
      if (ss != 0.0) {
        const double nrm = sqrt(alpha * alpha + ss);
        beta = alpha >= 0.0 ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      sh[0] = t; sh[1] = beta; sh[2] = scal;
      tau[j] = t;
    }
    __syncthreads();
    const double t = sh[0], beta = sh[1], scal = sh[2];
    if (t != 0.0)
      for (int i = j + 1 + threadIdx.x; i < b.m; i += blockDim.x) x[i] *= scal;
    __syncthreads();
    if (threadIdx.x == 0) x[j] = beta;
    __syncthreads();
    // H_j = I - tau v v^T on the panel's later columns, one warp per column
    if (t != 0.0) {
      for (int c = j + 1 + warp; c < c0 + w; c += nw) {
        double* y = W + (int64_t)c * b.m;
        double d = lane == 0 ? y[j] : 0.0;
        for (int i = j + 1 + lane; i < b.m; i += 32) d = fma(x[i], y[i], d);
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        d *= t;
        if (lane == 0) y[j] -= d;
        for (int i = j + 1 + lane; i < b.m; i += 32) y[i] = fma(-d, x[i], y[i]);
      }
    }
    __syncthreads();
  }
  // G[a][c] = v_a . v_c (a < c); v_a = e_(c0+a) + W[c0+a+1 .., c0+a], zero above row c0+a
  for (int pr = warp; pr < w * w; pr += nw) {
    const int a = pr / w, c = pr % w;
    if (a >= c) continue;
    const double* va = W + (int64_t)(c0 + a) * b.m;
    const double* vc = W + (int64_t)(c0 + c) * b.m;
    double d = lane == 0 ? va[c0 + c] : 0.0;                 // row c0+c, where v_c is 1
    for (int i = c0 + c + 1 + lane; i < b.m; i += 32) d = fma(va[i], vc[i], d);
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) G[a][c] = d;
  }
  __syncthreads();
  // T(0:jj, jj) = -tau_jj T(0:jj, 0:jj) G(0:jj, jj), T(jj, jj) = tau_jj: lane a owns row a
  if (warp == 0) {
    const bool row = lane < QR_NB;
    if (row)
      for (int c = 0; c < QR_NB; ++c) Ts[lane][c] = 0.0;
    __syncwarp();
    for (int jj = 0; jj < w; ++jj) {
      const double tj = tau[c0 + jj];
      if (lane < jj) {
        double acc = 0.0;
        for (int c = lane; c < jj; ++c) acc = fma(Ts[lane][c], G[c][jj], acc);
        Ts[lane][jj] = -tj * acc;
      } else if (lane == jj) {
        Ts[lane][jj] = tj;
      }
      __syncwarp();
    }
    double* T = Tall + b.t_off + (int64_t)p * QR_NB * QR_NB;   // column-major, ld QR_NB
    if (row)
      for (int c = 0; c < QR_NB; ++c) T[lane + c * QR_NB] = Ts[lane][c];
  }
}

// One strip of columns [col0, col0 + ncols) of the block's W (trailing update, op(T) =
// T^T) or Q (accumulation, op(T) = T): X[c0:, strip] -= V op(T) (V^T X[c0:, strip]).
__global__ void __launch_bounds__(QR_ATHREADS) qr_apply(const QrBlock* blocks, const QrTask* tasks, int p,
                                                       const double* Wk, const double* Tall, double* Xk, int is_q) {
  const QrTask tk = tasks[blockIdx.x];
  const QrBlock b = blocks[tk.block];
  const int c0 = p * QR_NB, w = min(QR_NB, b.k - c0);
  const int L = b.m - c0;
  const double* W = Wk + b.w_off;
  double* X = Xk + (is_q ? b.q_off : b.w_off);
  const double* T = Tall + b.t_off + (int64_t)p * QR_NB * QR_NB;
  __shared__ double Vs[QR_RC][QR_NB + 1];
  __shared__ double Xs[QR_RC][QR_SW + 1];
  __shared__ double Ys[QR_NB][QR_SW + 1];
  __shared__ double Ts[QR_NB][QR_NB + 1];
  const int tid = threadIdx.x;
  const int a0 = tid / QR_SW, cc = tid % QR_SW;          // outputs (a0 + o * QR_ATHREADS / QR_SW, cc)
  constexpr int AS = QR_ATHREADS / QR_SW;
  auto load_v = [&](int r0) {
    for (int e = tid; e < QR_RC * QR_NB; e += QR_ATHREADS) {
      const int i = e % QR_RC, a = e / QR_RC, ri = r0 + i;
      double v = 0.0;
      if (ri < L && a < w) v = ri < a ? 0.0 : (ri == a ? 1.0 : W[(int64_t)(c0 + a) * b.m + c0 + ri]);
      Vs[i][a] = v;
    }
  };
  double y[QR_OPT];
#pragma unroll
  for (int o = 0; o < QR_OPT; ++o) y[o] = 0.0;
  for (int r0 = 0; r0 < L; r0 += QR_RC) {
    __syncthreads();
    load_v(r0);
    for (int e = tid; e < QR_RC * QR_SW; e += QR_ATHREADS) {
      const int i = e % QR_RC, c = e / QR_RC;
      Xs[i][c] = (r0 + i < L && c < tk.ncols) ? X[(int64_t)(tk.col0 + c) * b.m + c0 + r0 + i] : 0.0;
    }
    __syncthreads();
#pragma unroll 16
    for (int i = 0; i < QR_RC; ++i) {
      const double xv = Xs[i][cc];
#pragma unroll
      for (int o = 0; o < QR_OPT; ++o) y[o] = fma(Vs[i][a0 + o * AS], xv, y[o]);
    }
  }
  for (int e = tid; e < QR_NB * QR_NB; e += QR_ATHREADS) {
    const int r = e % QR_NB, c = e / QR_NB;
    const double t = T[r + c * QR_NB];
    if (is_q) Ts[r][c] = t;
    else Ts[c][r] = t;
  }
#pragma unroll
  for (int o = 0; o < QR_OPT; ++o) Ys[a0 + o * AS][cc] = y[o];
  __syncthreads();
  double z[QR_OPT];
#pragma unroll
  for (int o = 0; o < QR_OPT; ++o) z[o] = 0.0;
#pragma unroll 8
  for (int q = 0; q < QR_NB; ++q)
#pragma unroll
    for (int o = 0; o < QR_OPT; ++o) z[o] = fma(Ts[a0 + o * AS][q], Ys[q][cc], z[o]);
  __syncthreads();
#pragma unroll
  for (int o = 0; o < QR_OPT; ++o) Ys[a0 + o * AS][cc] = z[o];
  for (int r0 = 0; r0 < L; r0 += QR_RC) {
    __syncthreads();
    load_v(r0);
    __syncthreads();
    for (int e = tid; e < QR_RC * QR_SW; e += QR_ATHREADS) {
      const int i = e % QR_RC, c = e / QR_RC;
      if (r0 + i < L && c < tk.ncols) {
        double acc = 0.0;
#pragma unroll 8
        for (int a = 0; a < QR_NB; ++a) acc = fma(Vs[i][a], Ys[a][c], acc);
        X[(int64_t)(tk.col0 + c) * b.m + c0 + r0 + i] -= acc;
      }
    }
  }
}

// R = upper triangle of W (k x n); positive: rows of R and columns of Q with a negative
// diagonal entry change sign (qr_positive, NDTensors/src/linearalgebra/linearalgebra.jl:374-381)
__global__ void qr_finish(const QrBlock* blocks, const double* Wk, double* Q, double* R, int positive) {
  const QrBlock b = blocks[blockIdx.y];
  const double* W = Wk + b.w_off;
  const int64_t kn = (int64_t)b.k * b.n, mk = (int64_t)b.m * b.k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < kn; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % b.k), c = (int)(e / b.k);
    double v = i <= c ? W[(int64_t)c * b.m + i] : 0.0;
    if (positive && W[(int64_t)i * b.m + i] < 0.0) v = -v;
    R[b.r_off + e] = v;
  }
  if (positive)
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mk; e += (int64_t)gridDim.x * blockDim.x) {
      const int c = (int)(e / b.m);
      if (W[(int64_t)c * b.m + c] < 0.0) Q[b.q_off + e] = -Q[b.q_off + e];
    }
}

__global__ void set_identity(const SvdBlock* blocks, double* Y) {
  const SvdBlock b = blocks[blockIdx.y];
  const int64_t tv = (int64_t)b.nn * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tv; e += (int64_t)gridDim.x * blockDim.x)
    Y[b.v_off + e] = (e % b.nn == e / b.nn) ? 1.0 : 0.0;
}

// ---- panel Jacobi: column groups of B resident in shared memory -------------------
// The columns of a block are cut into groups of B.  A round-robin tournament over the
// groups pairs them; one CTA loads the 2B columns of a group pair (its "panel") into
// shared memory and rotates every cross pair (p in the first group, q in the second)
// there, B rounds of B independent pairs, one warp per pair.  In the first round of a
// sweep every group also rotates its own pairs (B - 1 rounds), so each column pair is
// visited once per sweep, as in the cyclic scalar sweep.  The CTA accumulates the
// panel's rotations in a 2B x 2B matrix Q and, if anything rotated, writes the panel
// back and applies V[:, panel] <- V[:, panel] Q.  A sweep is one cooperative launch
// with a grid barrier per tournament round: (#groups - 1) rounds instead of
// (#columns - 1).
struct BjTask {
  int32_t block;     // block index
  int32_t k;         // pair index within the block's tournament round
};

template <typename T>
struct BjArgs {
  const SvdBlock* blocks;
  const BjTask* tasks;
  int ntasks;
  int nrounds;       // max over the listed blocks of (#groups rounded up to even) - 1
  int ldp;           // leading dimension of the shared-memory panel (>= every listed mm)
  T* W;
  T* V;
  unsigned long long* offmax;
  unsigned int* bar_count;
  unsigned int* bar_gen;
  DeviceStatus* st;
  double tol;        // pairs with |w_p . w_q| <= min(tol * mm^tol_pow, tol_cap) |w_p||w_q| are left
  double tol_pow;
  double tol_cap;
  const int32_t* active;   // optional: per block, 0 once converged (its tasks are skipped)
  const int32_t* any_active;   // optional: 0 when no block is active (the sweep returns at once)
};

// 16-byte vectors of the panel element type: a lane handles VW consecutive rows.
template <typename T> struct PanVec;
template <> struct PanVec<float> { using type = float4; static constexpr int W = 4; };
template <> struct PanVec<double> { using type = double2; static constexpr int W = 2; };

__device__ __forceinline__ void vdot(const float4& a, const float4& b, float& g0, float& g1) {
  g0 = fmaf(a.x, b.x, g0); g1 = fmaf(a.y, b.y, g1); g0 = fmaf(a.z, b.z, g0); g1 = fmaf(a.w, b.w, g1);
}
__device__ __forceinline__ void vdot(const double2& a, const double2& b, double& g0, double& g1) {
  g0 = fma(a.x, b.x, g0); g1 = fma(a.y, b.y, g1);
}
__device__ __forceinline__ void vrot(float4& x, float4& y, float c, float s) {
  const float4 a = x, b = y;
  x = make_float4(c * a.x - s * b.x, c * a.y - s * b.y, c * a.z - s * b.z, c * a.w - s * b.w);
  y = make_float4(s * a.x + c * b.x, s * a.y + c * b.y, s * a.z + c * b.z, s * a.w + c * b.w);
}
__device__ __forceinline__ void vrot(double2& x, double2& y, double c, double s) {
  const double2 a = x, b = y;
  x = make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
  y = make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
}

// One warp: Jacobi rotation of panel columns p and q (rotation accumulated into Q).
// nv = rows / VW, the panel's rows padded with zeros to a whole vector.
template <typename T, int P2>
__device__ __forceinline__ void bj_pair(T* pan, int ldp, T* q, T* d, const int* cols, int p, int qq, int nv,
                                        T tolb, int lane, int* any, unsigned long long* offmax) {
  using VT = typename PanVec<T>::type;
  if (cols[p] < 0 || cols[qq] < 0) return;
  VT* xp = reinterpret_cast<VT*>(pan + (size_t)p * ldp);
  VT* xq = reinterpret_cast<VT*>(pan + (size_t)qq * ldp);
  T g0 = 0, g1 = 0, g2 = 0, g3 = 0;
  int i = lane;
  for (; i + 32 < nv; i += 64) {
    vdot(xp[i], xq[i], g0, g1);
    vdot(xp[i + 32], xq[i + 32], g2, g3);
  }
  if (i < nv) vdot(xp[i], xq[i], g0, g1);
  const T g = warp_sum((g0 + g2) + (g1 + g3));
  const T al = d[p], be = d[qq];
  const T nrm = sqrt(al) * sqrt(be);
  const T rel = nrm > T(0) ? fabs(g) / nrm : T(0);   // in T: the FP64 pipe is narrow on this part
  if (!(rel > tolb) || g == T(0)) return;
  const T zeta = (be - al) / (T(2) * g);
  const T tt = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  const T c = T(1) / sqrt(T(1) + tt * tt);
  const T sn = c * tt;
  for (int j = lane; j < nv; j += 32) {
    VT x = xp[j], y = xq[j];
    vrot(x, y, c, sn);
    xp[j] = x;
    xq[j] = y;
  }
  if (lane < P2) {
    const T a = q[p * P2 + lane], b = q[qq * P2 + lane];
    q[p * P2 + lane] = c * a - sn * b;
    q[qq * P2 + lane] = sn * a + c * b;
  }
  if (lane == 0) {
    d[p] = al - tt * g;
    d[qq] = be + tt * g;
    *any = 1;
    atomicMax(offmax, (unsigned long long)__double_as_longlong((double)rel));
  }
}

// The cross rounds with column p of warp w (p = w, fixed through them) held in
// registers, NV vectors per lane: each round reads its partner q into registers once
// for both the dot product and the rotation and writes it back once, a third of the
// shared-memory traffic of bj_pair (which the FP32 sweeps are bound by).  Column p,
// its norm and column p of Q are touched by warp w alone during these rounds.
template <typename T, int P2, int NV>
__device__ __forceinline__ void bj_cross_regs(T* pan, int ldp, T* q, T* d, const int* cols, int B, int warp, int nv,
                                              T tolb, int lane, int* any, unsigned long long* offmax) {
  using VT = typename PanVec<T>::type;
  const int p = warp;
  const bool pv = cols[p] >= 0;
  VT* xp = reinterpret_cast<VT*>(pan + (size_t)p * ldp);
  VT rp[NV];
#pragma unroll
  for (int u = 0; u < NV; ++u) {
    const int i = lane + 32 * u;
    if (pv && i < nv) rp[u] = xp[i];
    else memset(&rp[u], 0, sizeof(VT));
  }
  T dp = d[p];
  for (int sr = 0; sr < B; ++sr) {
    const int qq = B + (warp + sr) % B;
    if (pv && cols[qq] >= 0) {
      VT* xq = reinterpret_cast<VT*>(pan + (size_t)qq * ldp);
      VT rq[NV];
      T g0 = 0, g1 = 0;
#pragma unroll
      for (int u = 0; u < NV; ++u) {
        const int i = lane + 32 * u;
        if (i < nv) rq[u] = xq[i];
        else memset(&rq[u], 0, sizeof(VT));
        vdot(rp[u], rq[u], g0, g1);
      }
      const T g = warp_sum(g0 + g1);
      const T al = dp, be = d[qq];
      const T nrm = sqrt(al) * sqrt(be);
      const T rel = nrm > T(0) ? fabs(g) / nrm : T(0);
      if (rel > tolb && g != T(0)) {
        const T zeta = (be - al) / (T(2) * g);
        const T tt = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + tt * tt);
        const T sn = c * tt;
#pragma unroll
        for (int u = 0; u < NV; ++u) {
          vrot(rp[u], rq[u], c, sn);
          const int i = lane + 32 * u;
          if (i < nv) xq[i] = rq[u];
        }
        if (lane < P2) {
          const T a = q[p * P2 + lane], b = q[qq * P2 + lane];
          q[p * P2 + lane] = c * a - sn * b;
          q[qq * P2 + lane] = sn * a + c * b;
        }
        dp = al - tt * g;
        if (lane == 0) {
          d[qq] = be + tt * g;
          *any = 1;
          atomicMax(offmax, (unsigned long long)__double_as_longlong((double)rel));
        }
      }
    }
    __syncthreads();
  }
  if (pv) {
#pragma unroll
    for (int u = 0; u < NV; ++u) {
      const int i = lane + 32 * u;
      if (i < nv) xp[i] = rp[u];
    }
  }
  if (lane == 0) d[p] = dp;
}

template <typename T, int B>
__global__ void __launch_bounds__(32 * B, 1) bj_sweep(BjArgs<T> a) {
  constexpr int P2 = 2 * B;
  extern __shared__ __align__(16) unsigned char bj_smem[];
  T* pan = reinterpret_cast<T*>(bj_smem);            // P2 columns of ldp
  T* q = pan + (size_t)P2 * a.ldp;                   // P2 x P2, column-major
  T* d = q + P2 * P2;                                // |w_c|^2 of the panel columns
  __shared__ int s_cols[P2];                         // column index in the block, -1 if none
  __shared__ int s_any;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const T tol = (T)a.tol, tol_cap = (T)a.tol_cap;
  const bool sqrt_pow = a.tol_pow != 1.0;          // tol_pow is 1 or 1/2
  if (a.any_active && !*a.any_active) return;      // every block converged: nothing to sweep (uniform)
  for (int r = 0; r < a.nrounds; ++r) {
    // tasks are listed longest first; CTA i takes positions i, 2G-1-i, 2G+i, ... (a snake),
    // so the CTAs with the longest first task get the shortest second one
    for (int w = 0;; ++w) {
      const int t = w * (int)gridDim.x + ((w & 1) ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x);
      if (t >= a.ntasks) break;
      const BjTask tk = a.tasks[t];
      if (a.active && !a.active[tk.block]) continue;
      const SvdBlock b = a.blocks[tk.block];
      const int nblk = (b.nn + B - 1) / B, nbp = nblk + (nblk & 1);
      if (r >= nbp - 1) continue;
      int gp, gq;
      rr_pair(nbp, r, tk.k, gp, gq);
      const bool rp = gp < nblk, rq = gq < nblk;
      if (!rp && !rq) continue;
      const bool lone = !(rp && rq);
      if (lone && r != 0) continue;                   // a group without a partner only has its own pairs
      const int mm = b.mm;
      constexpr int VW = PanVec<T>::W;
      const int mmv = (mm + VW - 1) / VW * VW;         // rows padded to whole vectors (zeros)
      const T tolb = min(tol_cap, tol * (sqrt_pow ? sqrt((T)mm) : (T)mm));
      if (threadIdx.x < P2) {
        const int g = threadIdx.x < B ? gp : gq;
        const int col = g * B + (threadIdx.x < B ? threadIdx.x : threadIdx.x - B);
        s_cols[threadIdx.x] = (g < nblk && col < b.nn) ? col : -1;
      }
      if (threadIdx.x == 0) s_any = 0;
      for (int e = threadIdx.x; e < P2 * P2; e += blockDim.x) q[e] = (e % P2 == e / P2) ? T(1) : T(0);
      __syncthreads();
      for (int c = warp; c < P2; c += B) {
        const int col = s_cols[c];
        T* dst = pan + (size_t)c * a.ldp;
        T acc = 0;
        if (col >= 0) {
          const T* src = a.W + b.w_off + (int64_t)col * mm;
          for (int i = lane; i < mmv; i += 32) {
            const T x = i < mm ? __ldcg(src + i) : T(0);   // L2: other CTAs rotated this column earlier
            dst[i] = x;
            acc = fma(x, x, acc);
          }
        } else {
          for (int i = lane; i < mmv; i += 32) dst[i] = T(0);
        }
        acc = warp_sum(acc);
        if (lane == 0) d[c] = acc;
      }
      __syncthreads();
      if (r == 0) {
        // each group's own pairs: a round-robin over its B columns, both groups at once
        for (int sr = 0; sr < B - 1; ++sr) {
          int p, qq;
          rr_pair(B, sr, warp % (B / 2), p, qq);
          if (warp >= B / 2) { p += B; qq += B; }
          bj_pair<T, P2>(pan, a.ldp, q, d, s_cols, p, qq, mmv / VW, tolb, lane, &s_any, &a.offmax[tk.block]);
          __syncthreads();
        }
      }
      if (!lone) {
        // register path for the widest groups when a column fits NVR vectors per lane
        constexpr int NVR = (sizeof(T) == 4 && B == 16) ? 9 : (sizeof(T) == 8 && B == 8) ? 17 : 0;
        bool done = false;
        if constexpr (NVR > 0) {
          if (mmv / VW <= 32 * NVR) {
            bj_cross_regs<T, P2, NVR>(pan, a.ldp, q, d, s_cols, B, warp, mmv / VW, tolb, lane, &s_any,
                                      &a.offmax[tk.block]);
            done = true;
          }
        }
        if (!done) {
          for (int sr = 0; sr < B; ++sr) {
            bj_pair<T, P2>(pan, a.ldp, q, d, s_cols, warp, B + (warp + sr) % B, mmv / VW, tolb, lane, &s_any,
                           &a.offmax[tk.block]);
            __syncthreads();
          }
        }
      }
      if (s_any) {
        for (int c = warp; c < P2; c += B) {
          const int col = s_cols[c];
          if (col < 0) continue;
          T* dst = a.W + b.w_off + (int64_t)col * mm;
          const T* src = pan + (size_t)c * a.ldp;
          for (int i = lane; i < mm; i += 32) dst[i] = src[i];
        }
        // V[:, panel] <- V[:, panel] Q, one row per thread (coalesced along each column)
        const int nn = b.nn;
        T* Vb = a.V + b.v_off;
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
          T v[P2];
#pragma unroll
          for (int c = 0; c < P2; ++c) v[c] = s_cols[c] >= 0 ? __ldcg(Vb + (int64_t)s_cols[c] * nn + i) : T(0);
#pragma unroll
          for (int c2 = 0; c2 < P2; ++c2) {
            if (s_cols[c2] < 0) continue;
            using VT = typename PanVec<T>::type;
            const VT* qc = reinterpret_cast<const VT*>(q + c2 * P2);
            T acc0 = 0, acc1 = 0;
#pragma unroll
            for (int c = 0; c < P2 / VW; ++c) {
              if constexpr (VW == 4)
                vdot(make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]), qc[c], acc0, acc1);
              else
                vdot(make_double2(v[2 * c], v[2 * c + 1]), qc[c], acc0, acc1);
            }
            Vb[(int64_t)s_cols[c2] * nn + i] = acc0 + acc1;
          }
        }
      }
      __syncthreads();
    }
    if (!grid_barrier(a.bar_count, a.bar_gen, gridDim.x, a.st)) return;
  }
}

// ---- mixed-precision refinement of the right singular vectors --------------------
// Ogita and Aishima, "Iterative refinement for symmetric eigenvalue decomposition"
// (Japan J. Indust. Appl. Math. 35, 2018), applied to W^T W without forming it:
// with X the current V, R = I - X^T X and S = (W X)^T (W X),
//   lambda_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i)   (a separated pair),
//   E_ij = R_ij / 2                                         (diagonal, or a close pair),
// and X <- X + X E.  A pair counts as separated when the size of its first-order
// rotation |S_ij + (lambda_i + lambda_j) R_ij / 2| / |lambda_j - lambda_i| is at most
// tau (decided on the unordered pair, so E_ij + E_ji = R_ij still holds); close pairs
// are left to the FP64 Jacobi sweep that follows.  tau < 0 rotates nothing: a
// Newton-Schulz step X <- X + X (I - X^T X) / 2.  A step rotates by first-order
// angles and orthogonalises to first order, so it leaves X non-orthogonal by the
// square of its largest |E_ij|.  The steps run as split GEMMs on the tensor cores
// (which resolve a product to about 2^-38 of its largest terms) until the rotations
// fall below 1e-10; then a step whose R, W X and S are FP64 GEMMs brings X to FP64
// accuracy, and, if that step's E was not tiny, a Newton-Schulz step with an FP64 R
// restores orthogonality.  In those steps E is small, so X E and (W X) E stay split
// GEMMs.  This kernel is the O(n^2) FP64 part.  E overwrites R.
#ifndef ND_SVD_TAU_FP64
#define ND_SVD_TAU_FP64 3e-8
#endif
#ifndef ND_SVD_EXACT_STEP
#define ND_SVD_EXACT_STEP 1
#endif
// Split-GEMM refinement steps before the FP64 one (fewer when the rotations fall below
// 1e-10; with ND_SVD_SPLIT_STALL also when a step does not halve them).  Four measured
// best on the chi = 4096 sweep step (3 / 4 / 5 steps: 127 / 125 / 126 ms).
#ifndef ND_SVD_SPLIT_STEPS
#define ND_SVD_SPLIT_STEPS 4
#endif
#ifndef ND_SVD_SPLIT_STALL
#define ND_SVD_SPLIT_STALL 0
#endif
// FP32 sweeps leave a pair when |w_p . w_q| <= ND_SVD_TOL32 * mm^ND_SVD_TOL32_POW |w_p||w_q|:
// 4 u sqrt(mm) (u = 2^-24), about the rounding level of an FP32 dot product of mm terms.
#ifndef ND_SVD_TOL32
#define ND_SVD_TOL32 2.4e-7
#endif
#ifndef ND_SVD_TOL32_POW
#define ND_SVD_TOL32_POW 0.5
#endif
// FP64 sweeps: mm * eps (eps = 2^-52), capped at 2e-13, so that the left vectors are
// orthogonal to 2e-13 or better however tall the block (LAPACK's dgesvj uses sqrt(mm)
// times the unit roundoff; the cap is the looser bound that this library's accuracy
// targets, 1e-12 relative, allow, and it saves a sweep on the large blocks).
#ifndef ND_SVD_TOL64
#define ND_SVD_TOL64 2.220446049250313e-16
#endif
#ifndef ND_SVD_TOL64_POW
#define ND_SVD_TOL64_POW 1.0
#endif
#ifndef ND_SVD_TOL64_CAP
#define ND_SVD_TOL64_CAP 2e-13
#endif
constexpr double OA_TAU = 1e-2;                   // split-GEMM steps
constexpr double OA_TAU_FP64 = ND_SVD_TAU_FP64;   // FP64 steps: only the small corrections left at that point

// emax[0]: largest first-order rotation applied; emax[1]: largest |E_ij| of any entry.
__global__ void oa_correction(const SvdBlock* blocks, const double* S, double* RE, double tau, unsigned long long* emax) {
  const SvdBlock b = blocks[blockIdx.y];
  const int n = b.nn;
  const double* Sb = S + b.v_off;
  double* Rb = RE + b.v_off;
  const int64_t tot = (int64_t)n * n;
  double m = 0.0, ma = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if (i > j) continue;                       // the thread of the upper entry writes both
    if (i == j) { Rb[e] = 0.5 * Rb[e]; ma = fmax(ma, fabs(Rb[e])); continue; }
    const int64_t et = (int64_t)i * n + j;     // (j, i)
    const double rij = Rb[e];
    const double li = Sb[(int64_t)i * n + i] / (1.0 - Rb[(int64_t)i * n + i]);
    const double lj = Sb[(int64_t)j * n + j] / (1.0 - Rb[(int64_t)j * n + j]);
    const double sij = 0.5 * (Sb[e] + Sb[et]);
    const double den = lj - li;
    const double mid = sij + 0.5 * (li + lj) * rij;
    double eij = 0.5 * rij, eji = 0.5 * rij;
    if (den != 0.0 && fabs(mid) <= tau * fabs(den)) {
      eij = (sij + lj * rij) / den;
      eji = rij - eij;
      m = fmax(m, fabs(mid / den));
    }
    Rb[e] = eij;                               // E(i, j): column j of X gains E_ij x_i
    Rb[et] = eji;
    ma = fmax(ma, fmax(fabs(eij), fabs(eji)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    ma = fmax(ma, __shfl_xor_sync(0xffffffffu, ma, o));
  }
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(emax, (unsigned long long)__double_as_longlong(m));
  if ((threadIdx.x & 31) == 0 && ma > 0.0) atomicMax(emax + 1, (unsigned long long)__double_as_longlong(ma));
}

// Lower triangle of a symmetric nn x nn block from its upper triangle, for the elements
// whose 64 x 64 tile lies below the diagonal (the tiles the FP64 GEMM skipped).
__global__ void sym_mirror(const SvdBlock* blocks, double* R) {
  const SvdBlock b = blocks[blockIdx.y];
  const int n = b.nn;
  double* Rb = R + b.v_off;
  const int64_t tot = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if ((i >> 6) > (j >> 6)) Rb[e] = Rb[(int64_t)i * n + j];
  }
}

// FP32 -> FP64 copy of V, per block
__global__ void v_to_f64(const SvdBlock* blocks, const float* V32, double* V) {
  const SvdBlock b = blocks[blockIdx.y];
  const int64_t tv = (int64_t)b.nn * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tv; e += (int64_t)gridDim.x * blockDim.x)
    V[b.v_off + e] = (double)V32[b.v_off + e];
}

// ---- blockwise Hermitian eigen -------------------------------------------------
// A_b + c_b I with c_b = 1.01 ||A_b||_F (1 for a zero block) is positive definite, so
// its one-sided Jacobi SVD gives the eigenvectors of A_b (left = right singular
// vectors) and lambda = sigma - c_b.
__global__ void eig_shift(const SvdBlock* blocks, const double* A, double* As, double* shift) {
  const SvdBlock b = blocks[blockIdx.x];
  __shared__ double red[8];
  const int64_t n = b.n, tot = n * n;
  const double* a = A + b.a_off;
  double ss = 0.0;
  for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) ss = fma(a[e], a[e], ss);
  ss = block_reduce_sum(ss, red);
  __shared__ double c;
  if (threadIdx.x == 0) c = ss > 0.0 ? 1.01 * sqrt(ss) : 1.0;
  __syncthreads();
  for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) As[b.a_off + e] = a[e] + ((e % (n + 1)) == 0 ? c : 0.0);
  if (threadIdx.x == 0) shift[blockIdx.x] = c;
}

// per block: lambda_j = sigma_j - c_b, re-ordered by |lambda| descending (ties by the
// sigma order): values, their |lambda| (pooled for truncate!) and the Jacobi column
// of each (NDTensors/src/linearalgebra/linearalgebra.jl:183-186: sortperm(rev, by = abs))
__global__ void eig_finish(const SvdBlock* blocks, const double* sig, const int32_t* order, const double* shift,
                           double* lam, double* absl, int32_t* vcol) {
  const SvdBlock b = blocks[blockIdx.x];
  const double c = shift[blockIdx.x];
  for (int j = threadIdx.x; j < b.nn; j += blockDim.x) {
    const double v = sig[b.s_off + j] - c, av = fabs(v);
    int rank = 0;
    for (int k = 0; k < b.nn; ++k) {
      const double u = fabs(sig[b.s_off + k] - c);
      rank += (u > av) || (u == av && k < j);
    }
    lam[b.s_off + rank] = v;
    absl[b.s_off + rank] = av;
    vcol[b.s_off + rank] = order[b.s_off + j];
  }
}

// Unshifted path: the Jacobi SVD of a symmetric block gives w_j = A v_j = sigma_j u_j with
// u_j = +-v_j when the eigenvalue +-sigma_j is not paired with one of opposite sign;
// lambda_j = v_j . w_j then carries the sign.  A column whose |v_j . w_j| falls short of
// sigma_j by more than 1e-6 (near +-lambda pairs mix v_j) marks its block ambiguous
// (*flag = 1); columns below 1e-12 of the block's largest are left as they are
// (their sign does not matter at that size).  One warp per column.
__global__ void eig_sign(const SvdBlock* blocks, const double* W, const double* Vw, const double* sig, double* lamJ,
                         int32_t* flag) {
  const SvdBlock b = blocks[blockIdx.x];
  const int n = b.nn, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double smax = sig[b.s_off];                 // sorted descending by svd_finish
  for (int j = warp; j < n; j += nw) {
    const double* w = W + b.w_off + (int64_t)j * b.mm;
    const double* v = Vw + b.v_off + (int64_t)j * n;
    double ww = 0.0, wv = 0.0;
    for (int i = lane; i < n; i += 32) {
      ww = fma(w[i], w[i], ww);
      wv = fma(w[i], v[i], wv);
    }
    for (int o = 16; o > 0; o >>= 1) {
      ww += __shfl_xor_sync(0xffffffffu, ww, o);
      wv += __shfl_xor_sync(0xffffffffu, wv, o);
    }
    if (lane == 0) {
      const double sj = sqrt(ww);
      lamJ[b.s_off + j] = wv;
      if (sj > 1e-12 * smax && fabs(wv) < (1.0 - 1e-6) * sj) atomicExch(flag, 1);
    }
  }
}

// per block: the signed eigenvalues of the unshifted path, ordered by |lambda| descending
// (ties by the sigma order), as eig_finish does for the shifted one
__global__ void eig_finish_signed(const SvdBlock* blocks, const int32_t* order, const double* lamJ, double* lam,
                                  double* absl, int32_t* vcol) {
  const SvdBlock b = blocks[blockIdx.x];
  for (int j = threadIdx.x; j < b.nn; j += blockDim.x) {
    const double v = lamJ[b.s_off + order[b.s_off + j]], av = fabs(v);
    int rank = 0;
    for (int k = 0; k < b.nn; ++k) {
      const double u = fabs(lamJ[b.s_off + order[b.s_off + k]]);
      rank += (u > av) || (u == av && k < j);
    }
    lam[b.s_off + rank] = v;
    absl[b.s_off + rank] = av;
    vcol[b.s_off + rank] = order[b.s_off + j];
  }
}

// eigenvectors (n x n per block, columns in |lambda| order) from the Jacobi V
__global__ void eig_vectors(const SvdBlock* blocks, const double* Vw, const int32_t* vcol, double* Vfull,
                            const int64_t* v_off) {
  const SvdBlock b = blocks[blockIdx.y];
  const int64_t tot = (int64_t)b.nn * b.nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % b.nn, c = e / b.nn;
    Vfull[v_off[blockIdx.y] + e] = Vw[b.v_off + (int64_t)vcol[b.s_off + c] * b.nn + i];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Jacobi sweeps of element type T on (Wt, Vt) until every block has had a sweep
// without rotations or max_sweeps have run.
template <typename T>
static nd_status run_sweeps(nd_handle h, const SvdBlock* dblk, int nb, int task0, int maxr, int soff, T* Wt, T* Vt,
                            unsigned long long* offmax, unsigned int* bar, double tol, int max_sweeps,
                            bool& converged, int& sweeps, double tol_pow = 1.0, double tol_cap = INFINITY) {
  cudaStream_t s = h->stream;
  converged = maxr == 0;
  sweeps = 0;
  if (converged) return ND_OK;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, svd_sweep<T>, 512, 0);
  per_sm = std::max(per_sm, 1);
  const int grid = std::max(1, std::min((task0 + 15) / 16, per_sm * h->num_sms));
  const char* name = sizeof(T) == 4 ? "svd_sweep_f32" : "svd_sweep";
  std::vector<unsigned long long> om(nb);
  std::vector<int32_t> act(nb, 1);
  T* nrm = nullptr;
  int32_t* dact = nullptr;
  ND_CUDA(h, cudaMallocAsync(&nrm, std::max(soff, 1) * sizeof(T), s));
  ND_CUDA(h, cudaMallocAsync(&dact, nb * 4, s));
  nd_status st = ND_OK;
  for (int sw = 0; sw < max_sweeps; ++sw) {
    cudaError_t e = cudaMemcpyAsync(dact, act.data(), nb * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(offmax, 0, nb * 8, s);
    if (e != cudaSuccess) { st = nd_cuda_check(h, e, "svd sweep set-up"); break; }
    nd_prof_begin(h, "svd_norms");
    svd_norms<T><<<std::max(1, std::min((soff + 7) / 8, 8 * h->num_sms)), 256, 0, s>>>(dblk, nb, dact, Wt, nrm, soff);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    SweepArgs<T> sa{dblk, nb, task0, maxr, Wt, Vt, nrm, dact, offmax, bar, bar + 1, h->d_status, tol, tol_pow, tol_cap};
    void* args[] = {&sa};
    nd_prof_begin(h, name);
    e = cudaLaunchCooperativeKernel((void*)svd_sweep<T>, grid, 512, args, 0, s);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    if (e != cudaSuccess) { st = nd_cuda_check(h, e, "svd_sweep (cooperative launch)"); break; }
    e = cudaMemcpyAsync(om.data(), offmax, nb * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { st = nd_cuda_check(h, e, "svd sweep"); break; }
    ++sweeps;
    if ((st = nd_check_device_status(h, "svd"))) break;
    // a sweep without any rotation above m * unit roundoff leaves its block converged
    bool any = false;
    for (int i = 0; i < nb; ++i) {
      if (act[i] && om[i] == 0ull) act[i] = 0;
      any = any || act[i];
    }
    if (!any) { converged = true; break; }
  }
  cudaFreeAsync(nrm, s);
  cudaFreeAsync(dact, s);
  return st;
}

// Panel-Jacobi sweeps (bj_sweep) of element type T on (Wt, Vt).  Returns
// ND_ERR_UNSUPPORTED without launching anything when the tallest block does not fit a
// panel in shared memory (the caller then uses the scalar sweeps).
template <typename T, int B>
static nd_status launch_bj(nd_handle h, const BjArgs<T>& a, size_t smem) {
  // per device: the dynamic shared memory this instantiation is opted in to, and the
  // resident CTAs per SM for each size (neither set up while capturing)
  static std::mutex mu;
  static std::map<int, size_t> attr;
  static std::map<std::pair<int, size_t>, int> occ_of;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    size_t& opted = attr[h->device];
    if (smem > opted) {
      if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "svd panel sweep: run once before graph capture");
      nd_status st = nd_cuda_check(h, cudaFuncSetAttribute(bj_sweep<T, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                           (int)smem), "svd panel sweep shared memory");
      if (st) return st;
      opted = smem;
    }
    auto it = occ_of.find({h->device, smem});
    if (it == occ_of.end()) {
      if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "svd panel sweep: run once before graph capture");
      int occ = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bj_sweep<T, B>, 32 * B, smem);
      it = occ_of.emplace(std::make_pair(h->device, smem), occ).first;
    }
    per_sm = it->second;
  }
  if (per_sm < 1) return nd_fail(h, ND_ERR_UNSUPPORTED, "svd panel sweep does not fit an SM");
  const int grid = std::max(1, std::min(a.ntasks, per_sm * h->num_sms));
  BjArgs<T> args = a;
  void* kargs[] = {&args};
  return nd_cuda_check(h, cudaLaunchCooperativeKernel((void*)bj_sweep<T, B>, grid, 32 * B, kargs, smem, h->stream),
                       "svd panel sweep (cooperative launch)");
}

// Widest column group B whose panel (2B columns of ldp) stays within ~200 KB of shared
// memory; 0 when even the narrowest does not fit.
template <typename T>
static int panel_group(int ldp) {
  ldp = (ldp + 3) / 4 * 4;
  const size_t budget = 200 * 1024;
  int B = sizeof(T) == 4 ? 16 : 8;
  const int bmin = sizeof(T) == 4 ? 4 : 2;
  while (B >= bmin && (size_t)2 * B * ldp * sizeof(T) > budget) B >>= 1;
  return B >= bmin ? B : 0;
}

// tol_pow: 1 or 1/2 (the panel kernel evaluates mm^tol_pow as mm or sqrt(mm))
template <typename T>
static nd_status run_panel_sweeps(nd_handle h, const std::vector<SvdBlock>& blocks, const SvdBlock* dblk, T* Wt,
                                  T* Vt, unsigned long long* offmax, unsigned int* bar, double tol, int max_sweeps,
                                  bool& converged, int& sweeps, std::vector<int32_t>* act_hist = nullptr,
                                  std::vector<double>* off_hist = nullptr, double tol_pow = 1.0,
                                  double tol_cap = INFINITY) {
  cudaStream_t s = h->stream;
  const int nb = (int)blocks.size();
  sweeps = 0;
  converged = false;
  int ldp = 1;
  for (auto& b : blocks) ldp = std::max(ldp, b.mm);
  ldp = (ldp + 3) / 4 * 4;                  // whole 16-byte vectors per panel column
  const int B = panel_group<T>(ldp);
  if (!B) return ND_ERR_UNSUPPORTED;
  const size_t smem = ((size_t)2 * B * ldp + (size_t)4 * B * B + 2 * B) * sizeof(T);
  std::vector<unsigned long long> om(nb);
  std::vector<int32_t> act(nb, 1);
  // longest tasks first: blocks in decreasing mm * nn
  std::vector<int> ord(nb);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
    return (int64_t)blocks[x].mm * blocks[x].nn > (int64_t)blocks[y].mm * blocks[y].nn;
  });
  int maxtasks = 0;
  for (auto& b : blocks) { const int g = (b.nn + B - 1) / B; maxtasks += (g + (g & 1)) / 2; }
  BjTask* dtasks = nullptr;
  nd_status st = nd_dalloc(h, (void**)&dtasks, std::max(maxtasks, 1) * sizeof(BjTask));
  if (st) return st;
  std::vector<BjTask> tasks;
  const char* name = sizeof(T) == 4 ? "svd_panel_sweep_f32" : "svd_panel_sweep";
  for (int sw = 0; sw < max_sweeps; ++sw) {
    tasks.clear();
    int nrounds = 0;
    for (int bi : ord) {
      if (!act[bi]) continue;
      const int g = (blocks[bi].nn + B - 1) / B, gp = g + (g & 1);
      for (int k = 0; k < gp / 2; ++k) tasks.push_back(BjTask{bi, k});
      nrounds = std::max(nrounds, gp - 1);
    }
    if (tasks.empty()) { converged = true; break; }
    if (act_hist) act_hist->push_back((int32_t)std::count(act.begin(), act.end(), 1));
    if ((st = nd_upload(h, dtasks, tasks.data(), tasks.size() * sizeof(BjTask)))) break;
    if ((st = nd_cuda_check(h, cudaMemsetAsync(offmax, 0, nb * 8, s), "svd sweep set-up"))) break;
    BjArgs<T> a{dblk, dtasks, (int)tasks.size(), nrounds, ldp, Wt, Vt, offmax, bar, bar + 1, h->d_status, tol, tol_pow,
                tol_cap, nullptr, nullptr};
    nd_prof_begin(h, name);
    if constexpr (sizeof(T) == 4) {
      if (B == 16) st = launch_bj<T, 16>(h, a, smem);
      else if (B == 8) st = launch_bj<T, 8>(h, a, smem);
      else st = launch_bj<T, 4>(h, a, smem);
    } else {
      if (B == 8) st = launch_bj<T, 8>(h, a, smem);
      else if (B == 4) st = launch_bj<T, 4>(h, a, smem);
      else st = launch_bj<T, 2>(h, a, smem);
    }
    nd_prof_end(h);
    ND_LAUNCHED(h);
    if (st) break;
    cudaError_t e = cudaMemcpyAsync(om.data(), offmax, nb * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { st = nd_cuda_check(h, e, "svd panel sweep"); break; }
    ++sweeps;
    if ((st = nd_check_device_status(h, "svd"))) break;
    if (off_hist) {
      double m = 0.0;
      for (int i = 0; i < nb; ++i) if (act[i]) m = std::max(m, bits_to_double(om[i]));
      off_hist->push_back(m);
    }
    // a sweep without any rotation above mm * unit roundoff leaves its block converged
    bool any = false;
    for (int i = 0; i < nb; ++i) {
      if (act[i] && om[i] == 0ull) act[i] = 0;
      any = any || act[i];
    }
    if (!any) { converged = true; break; }
  }
  cudaFreeAsync(dtasks, s);
  return st;
}

static Mixed mixed1(int64_t dim, int64_t st0, int64_t st1) {
  Mixed m{};
  m.n = 1;
  m.dim[0] = (int32_t)dim;
  m.st0[0] = st0;
  m.st1[0] = st1;
  mixed_finalize(m);
  return m;
}

// R = alpha * op(A) * B + beta * R for every block in one grouped launch of the given
// precision (c: the launch state, reused while the blocks stay the same).
//   kind 0: Y  (nn x nn) = alpha * V^T V + beta * Y
//   kind 1: Vn (nn x nn) = alpha * V Y   + beta * Vn
//   kind 2: W0 (mm x nn) = alpha * W Q   + beta * W0
//   kind 3: S  (nn x nn) = alpha * W^T W + beta * S
static nd_status block_gemm(nd_handle h, ExecCache& c, const std::vector<SvdBlock>& blocks, const SvdBlock* dblk,
                            int kind, const double* A, const double* B, double* R, double alpha, double beta,
                            int precision) {
  std::vector<PairDesc> pairs(blocks.size());
  for (size_t i = 0; i < blocks.size(); ++i) {
    const SvdBlock& b = blocks[i];
    PairDesc pd{};
    const int64_t M = kind == 2 ? b.mm : b.nn, N = b.nn, K = kind == 3 ? b.mm : b.nn;
    pd.M = (int32_t)M; pd.N = (int32_t)N; pd.K = (int32_t)K;
    pd.group = (int32_t)i; pd.first = 1; pd.job = 0;
    pd.a_off = (kind == 2 || kind == 3) ? b.w_off : b.v_off;
    pd.b_off = kind == 3 ? b.w_off : b.v_off;
    pd.r_off = kind == 2 ? b.w_off : b.v_off;
    const int64_t a_row = kind == 0 ? b.nn : kind == 3 ? b.mm : 1;   // A(i, k) = A[i * a_row + k * a_k]
    const int64_t a_k = (kind == 0 || kind == 3) ? 1 : M;
    const int64_t b_col = kind == 3 ? b.mm : b.nn;                    // B(k, j) = B[k + j * b_col]
    pd.rows = mixed1(M, a_row, 1);                   // A row stride, R row stride
    pd.cols = mixed1(N, b_col, M);                   // B column stride, R column stride
    pd.ks = mixed1(K, a_k, 1);                       // A k stride, B k stride
    pairs[i] = pd;
  }
  // R = V^T V and S = W^T W are symmetric: the FP64 tile kernel computes the 64 x 64 tiles
  // on and above the diagonal, sym_mirror copies the others
  const bool sym = (kind == 0 || kind == 3) && precision == ND_PREC_FP64;
  if (sym)
    for (auto& pd : pairs) pd.sym = 1;
  JobPtrs ptrs{{A, nullptr}, {B, nullptr}, {R, nullptr}};
  nd_status st = nd_execute_cached(h, c, pairs, (int)blocks.size(), ptrs, alpha, beta, precision);
  if (st || !sym) return st;
  int64_t maxv = 1;
  for (auto& b : blocks) maxv = std::max(maxv, (int64_t)b.nn * b.nn);
  const dim3 gv((unsigned)std::min<int64_t>((maxv + 255) / 256, 1024), (unsigned)blocks.size());
  sym_mirror<<<gv, 256, 0, h->stream>>>(dblk, R);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "sym_mirror");
}

static nd_status svd_core(nd_handle h, int nb, const int64_t* rows, const int64_t* cols, const int64_t* offsets,
                          const double* A, std::vector<SvdBlock>& blocks, double** d_sig_out, int32_t** d_order_out,
                          double** d_W_out, double** d_V_out, SvdBlock** d_blocks_out, int& total_k) {
  cudaStream_t s = h->stream;
  blocks.resize(nb);
  int64_t woff = 0, voff = 0;
  int task0 = 0, soff = 0, maxr = 0;
  for (int i = 0; i < nb; ++i) {
    SvdBlock& b = blocks[i];
    if (rows[i] <= 0 || cols[i] <= 0 || rows[i] > INT32_MAX || cols[i] > INT32_MAX)
      return nd_fail(h, ND_ERR_ARG, "svd: block %d has invalid dims %lld x %lld", i, (long long)rows[i], (long long)cols[i]);
    b.a_off = offsets[i];
    b.m = (int)rows[i]; b.n = (int)cols[i];
    b.trans = b.m < b.n;
    b.mm = b.trans ? b.n : b.m;
    b.nn = b.trans ? b.m : b.n;
    b.npad = b.nn + (b.nn & 1);
    b.w_off = woff; woff += (int64_t)b.mm * b.nn;
    b.v_off = voff; voff += (int64_t)b.nn * b.nn;
    b.task0 = task0; b.ntask = b.npad / 2; task0 += b.ntask;
    b.s_off = soff; soff += b.nn;
    maxr = std::max(maxr, b.npad - 1);
  }
  total_k = soff;
  double *W = nullptr, *V = nullptr, *sig = nullptr;
  int32_t* order = nullptr;
  SvdBlock* dblk = nullptr;
  unsigned long long* offmax = nullptr;
  unsigned int* bar = nullptr;
  ND_CUDA(h, cudaMallocAsync(&W, std::max<int64_t>(woff, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&V, std::max<int64_t>(voff, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&sig, std::max(soff, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&order, std::max(soff, 1) * 4, s));
  ND_CUDA(h, cudaMallocAsync(&dblk, nb * sizeof(SvdBlock), s));
  ND_CUDA(h, cudaMallocAsync(&offmax, nb * 8, s));
  ND_CUDA(h, cudaMallocAsync(&bar, 8, s));
  ND_CUDA(h, cudaMemcpyAsync(dblk, blocks.data(), nb * sizeof(SvdBlock), cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemsetAsync(bar, 0, 8, s));
  {
    int64_t maxe = 0;
    for (auto& b : blocks) maxe = std::max(maxe, (int64_t)b.mm * b.nn);
    dim3 grid((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
    nd_prof_begin(h, "svd_init");
    svd_init<<<grid, 256, 0, s>>>(dblk, nb, A, W, V);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  // Larger problems run in three stages.  (1) Jacobi sweeps in FP32 on a power-of-two
  // scaled copy (the FP32 pipe is ~64x the FP64 one on this part) give an approximate V.
  // (2) Mixed-precision refinement (oa_correction) makes V accurate and orthogonal to
  // FP64 working accuracy; its O(n^3) products are split GEMMs with 6 slices on the
  // tensor cores except the last orthogonality check and W V (FP64 GEMMs), its O(n^2)
  // part is FP64.  (3) FP64 Jacobi sweeps on W V finish the
  // pairs the refinement leaves (close singular values) and certify convergence: the
  // result is the FP64 one-sided Jacobi SVD of W V with V orthogonal to working
  // accuracy.  Every sweep stage uses the panel kernel when the tallest block fits a
  // shared-memory panel and the scalar sweep otherwise.
  // FP64 sweep limit (the reference's LAPACK call has no such knob; a limit of 0 makes
  // every block with more than one column report ND_ERR_NOCONV, which tests use)
  const int max_sweeps = h->svd_max_sweeps < 0 ? 60 : h->svd_max_sweeps;
  double work = 0.0;
  for (auto& b : blocks) work += (double)b.mm * b.nn * b.nn;
  bool converged = false;
  int sweeps32 = 0, sweeps64 = 0;
  nd_status st = ND_OK;
  int maxmm = 1;
  for (auto& b : blocks) maxmm = std::max(maxmm, b.mm);
  std::vector<double> ref_angles, off64, off32;
  std::vector<int32_t> act64, act32;
  int nref = 0;
  if (work >= 2e8 && maxr > 0) {
    float *W32 = nullptr, *V32 = nullptr;
    double *Y = nullptr, *Vn = nullptr, *W0 = nullptr, *W1 = nullptr, *S = nullptr;
    unsigned long long *bmax = nullptr, *emax = nullptr;
    ND_CUDA(h, cudaMallocAsync(&W32, std::max<int64_t>(woff, 1) * 4, s));
    ND_CUDA(h, cudaMallocAsync(&V32, std::max<int64_t>(voff, 1) * 4, s));
    ND_CUDA(h, cudaMallocAsync(&Y, std::max<int64_t>(voff, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&Vn, std::max<int64_t>(voff, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&S, std::max<int64_t>(voff, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&W0, std::max<int64_t>(woff, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&W1, std::max<int64_t>(woff, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&bmax, nb * 8, s));
    ND_CUDA(h, cudaMallocAsync(&emax, 16, s));
    ND_CUDA(h, cudaMemsetAsync(bmax, 0, nb * 8, s));
    int64_t maxe = 0, maxv = 0;
    for (auto& b : blocks) { maxe = std::max(maxe, (int64_t)b.mm * b.nn); maxv = std::max(maxv, (int64_t)b.nn * b.nn); }
    const dim3 ge((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
    const dim3 gv((unsigned)std::min<int64_t>((maxv + 255) / 256, 1024), nb);
    nd_prof_begin(h, "svd_precondition");
    block_absmax<<<ge, 256, 0, s>>>(dblk, W, bmax);
    to_f32_scaled<<<ge, 256, 0, s>>>(dblk, W, bmax, W32, V32);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    ND_LAUNCHED(h);
    bool c32 = false;
    const double u32 = ND_SVD_TOL32;
    const int sweeps32_max = std::min(40, max_sweeps);
    if (panel_group<float>(maxmm))
      st = run_panel_sweeps<float>(h, blocks, dblk, W32, V32, offmax, bar, u32, sweeps32_max, c32, sweeps32, &act32,
                                   &off32, ND_SVD_TOL32_POW);
    else
      st = run_sweeps<float>(h, dblk, nb, task0, maxr, soff, W32, V32, offmax, bar, u32, sweeps32_max, c32, sweeps32,
                             ND_SVD_TOL32_POW);
    if (!st) {
      v_to_f64<<<gv, 256, 0, s>>>(dblk, V32, V);
      ND_LAUNCHED(h);
      ExecCache cR, cW, cS, cV, cR64, cW64, cS64, cWE;
      const int saved = h->ozaki_slices;
      h->ozaki_slices = 6;
      // One refinement step.  mode 0: split-GEMM step; 1: FP64 R, W X and S; 2: Newton-
      // Schulz with an FP64 R.  Modes 1 and 2 keep W0 = W X current (W0 += W0 E).
      // Leaves em[0] (largest rotation) and em[1] (largest |E_ij|) on the host.
      double em[2] = {0.0, 0.0};
      auto step = [&](int mode) -> nd_status {
        const int pr = mode ? ND_PREC_FP64 : ND_PREC_OZAKI;
        set_identity<<<gv, 256, 0, s>>>(dblk, Y);
        ND_LAUNCHED(h);
        nd_prof_begin(h, "svd_refine_gemm");
        nd_status e = block_gemm(h, mode ? cR64 : cR, blocks, dblk, 0, V, V, Y, -1.0, 1.0, pr);             // R = I - X^T X
        if (!e && mode < 2) e = block_gemm(h, mode ? cW64 : cW, blocks, dblk, 2, W, V, W0, 1.0, 0.0, pr);  // W0 = W X
        if (!e && mode < 2) e = block_gemm(h, mode ? cS64 : cS, blocks, dblk, 3, W0, W0, S, 1.0, 0.0, pr); // S = W0^T W0
        nd_prof_end(h);
        if (e) return e;
        if ((e = nd_cuda_check(h, cudaMemsetAsync(emax, 0, 16, s), "svd refine"))) return e;
        nd_prof_begin(h, "svd_refine");
        const double tau = mode == 0 ? OA_TAU : mode == 1 ? OA_TAU_FP64 : -1.0;
        oa_correction<<<gv, 256, 0, s>>>(dblk, S, Y, tau, emax);                                      // Y <- E
        ND_LAUNCHED(h);
        e = nd_cuda_check(h, cudaMemcpyAsync(Vn, V, voff * 8, cudaMemcpyDeviceToDevice, s), "svd copy");
        if (!e && mode) e = nd_cuda_check(h, cudaMemcpyAsync(W1, W0, woff * 8, cudaMemcpyDeviceToDevice, s), "svd copy");
        nd_prof_end(h);
        nd_prof_begin(h, "svd_refine_gemm");
        if (!e) e = block_gemm(h, cV, blocks, dblk, 1, V, Y, Vn, 1.0, 1.0, ND_PREC_OZAKI);                 // X + X E
        if (!e && mode) e = block_gemm(h, cWE, blocks, dblk, 2, W0, Y, W1, 1.0, 1.0, ND_PREC_OZAKI);       // W0 + W0 E
        nd_prof_end(h);
        if (e) return e;
        std::swap(V, Vn);
        if (mode) std::swap(W0, W1);
        unsigned long long eb[2] = {0, 0};
        if ((e = nd_cuda_check(h, cudaMemcpyAsync(eb, emax, 16, cudaMemcpyDeviceToHost, s), "svd refine"))) return e;
        if ((e = nd_cuda_check(h, cudaStreamSynchronize(s), "svd refine"))) return e;
        em[0] = bits_to_double(eb[0]);
        em[1] = bits_to_double(eb[1]);
        ++nref;
        ref_angles.push_back(mode == 2 ? em[1] : em[0]);
        return ND_OK;
      };
      // split-GEMM steps while they still converge (their noise floor is ~1e-12 / gap)
      double prev = INFINITY;
      for (int it = 0; it < ND_SVD_SPLIT_STEPS && !st; ++it) {
        st = step(0);
        if (!st && (em[0] <= 1e-10 || (ND_SVD_SPLIT_STALL && em[0] > 0.5 * prev))) break;
        prev = em[0];
      }
      if (!st && ND_SVD_EXACT_STEP) st = step(1);
      // |E| <= 3e-8 leaves X orthogonal to 1e-15; otherwise Newton-Schulz (quadratic)
      for (int it = 0; it < 3 && !st && em[1] > 3e-8; ++it) st = step(2);
      if (!st && !ND_SVD_EXACT_STEP) st = block_gemm(h, cW64, blocks, dblk, 2, W, V, W0, 1.0, 0.0, ND_PREC_FP64);
      if (!st) std::swap(W, W0);                                                                      // W <- W X
      h->ozaki_slices = saved;
      for (ExecCache* c : {&cR, &cW, &cS, &cV, &cR64, &cW64, &cS64, &cWE}) c->free_all(h);
    }
    cudaFreeAsync(W32, s); cudaFreeAsync(V32, s); cudaFreeAsync(Y, s); cudaFreeAsync(Vn, s);
    cudaFreeAsync(S, s); cudaFreeAsync(W0, s); cudaFreeAsync(W1, s); cudaFreeAsync(bmax, s); cudaFreeAsync(emax, s);
  }
  if (!st) {
    const double u64 = ND_SVD_TOL64;
    if (panel_group<double>(maxmm))
      st = run_panel_sweeps<double>(h, blocks, dblk, W, V, offmax, bar, u64, max_sweeps, converged, sweeps64, &act64,
                                    &off64, ND_SVD_TOL64_POW, ND_SVD_TOL64_CAP);
    else
      st = run_sweeps<double>(h, dblk, nb, task0, maxr, soff, W, V, offmax, bar, u64, max_sweeps, converged, sweeps64,
                              ND_SVD_TOL64_POW, ND_SVD_TOL64_CAP);
  }
  h->svd_info_i = {sweeps32, nref, sweeps64, panel_group<double>(maxmm) ? 1 : 0};
  h->svd_info_i.insert(h->svd_info_i.end(), act64.begin(), act64.end());
  h->svd_info_d = ref_angles;
  h->svd_info_d.insert(h->svd_info_d.end(), off64.begin(), off64.end());
  h->svd_info_d.insert(h->svd_info_d.end(), off32.begin(), off32.end());
  if (st) {
    cudaFreeAsync(W, s); cudaFreeAsync(V, s); cudaFreeAsync(sig, s); cudaFreeAsync(order, s);
    cudaFreeAsync(dblk, s); cudaFreeAsync(offmax, s); cudaFreeAsync(bar, s);
    return st;
  }
  if (maxr == 0) converged = true;
  if (!converged) {
    cudaFreeAsync(W, s); cudaFreeAsync(V, s); cudaFreeAsync(sig, s); cudaFreeAsync(order, s);
    cudaFreeAsync(dblk, s); cudaFreeAsync(offmax, s); cudaFreeAsync(bar, s);
    return nd_fail(h, ND_ERR_NOCONV, "svd: one-sided Jacobi did not converge in %d sweeps", max_sweeps);
  }
  {
    int maxn = 1;
    for (auto& b : blocks) maxn = std::max(maxn, b.nn);
    nd_prof_begin(h, "svd_finish");
    svd_finish<<<nb, 256, maxn * 8, s>>>(dblk, W, sig, order);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  cudaFreeAsync(offmax, s);
  cudaFreeAsync(bar, s);
  *d_sig_out = sig; *d_order_out = order; *d_W_out = W; *d_V_out = V; *d_blocks_out = dblk;
  return nd_cuda_check(h, cudaGetLastError(), "svd");
}

extern "C" nd_status nd_bs_svd_f64(nd_handle h, int32_t nb, const int64_t* rows, const int64_t* cols,
                                   const int64_t* offsets, const double* A, double* U, double* S, double* V,
                                   int32_t mindim, int32_t maxdim, double cutoff, int32_t use_absolute_cutoff,
                                   int32_t use_relative_cutoff, int32_t min_blockdim, int32_t* kept, double* spectrum,
                                   int32_t* spectrum_len, double* truncerr, double* docut) {
  if (!h) return ND_ERR_ARG;
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "svd returns kept dimensions to the host and cannot be captured");
  if (nb < 0 || (nb > 0 && (!rows || !cols || !offsets || !A || !U || !S || !V || !kept)))
    return nd_fail(h, ND_ERR_ARG, "svd: NULL argument");
  if (nb > kMaxBlocksPerCall) return nd_fail(h, ND_ERR_UNSUPPORTED, "svd: at most %d blocks per call", kMaxBlocksPerCall);
  if (nb == 0) { if (spectrum_len) *spectrum_len = 0; if (truncerr) *truncerr = 0; if (docut) *docut = 0; return ND_OK; }
  cudaStream_t s = h->stream;
  std::vector<SvdBlock> blocks;
  double *sig = nullptr, *W = nullptr, *Vw = nullptr;
  int32_t* order = nullptr;
  SvdBlock* dblk = nullptr;
  int total = 0;
  nd_status st = svd_core(h, nb, rows, cols, offsets, A, blocks, &sig, &order, &W, &Vw, &dblk, total);
  if (st) return st;
  // full (untruncated) U / V in a scratch buffer, then compacted prefixes
  std::vector<int64_t> uo(nb), vo(nb);
  int64_t ut = 0, vt = 0;
  for (int i = 0; i < nb; ++i) { uo[i] = ut; ut += (int64_t)blocks[i].m * blocks[i].nn; vo[i] = vt; vt += (int64_t)blocks[i].n * blocks[i].nn; }
  double *Uf = nullptr, *Vf = nullptr, *P = nullptr, *res = nullptr;
  int64_t *duo = nullptr, *dvo = nullptr;
  int32_t* dkept = nullptr;
  int* dlen = nullptr;
  ND_CUDA(h, cudaMallocAsync(&Uf, std::max<int64_t>(ut, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&Vf, std::max<int64_t>(vt, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&duo, nb * 8, s));
  ND_CUDA(h, cudaMallocAsync(&dvo, nb * 8, s));
  ND_CUDA(h, cudaMallocAsync(&P, std::max(total, 1) * 8, s));
  ND_CUDA(h, cudaMallocAsync(&res, 4 * 8, s));
  ND_CUDA(h, cudaMallocAsync(&dkept, nb * 4, s));
  ND_CUDA(h, cudaMallocAsync(&dlen, 8, s));
  ND_CUDA(h, cudaMemcpyAsync(duo, uo.data(), nb * 8, cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(dvo, vo.data(), nb * 8, cudaMemcpyHostToDevice, s));
  {
    int64_t maxe = 0;
    for (auto& b : blocks) maxe = std::max(maxe, (int64_t)b.mm * b.nn);
    dim3 grid((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
    nd_prof_begin(h, "svd_outputs");
    svd_outputs<<<grid, 256, 0, s>>>(dblk, W, Vw, sig, order, Uf, Vf, duo, dvo);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  // pooled s^2: sort + truncate on the device
  int npow2 = 1;
  while (npow2 < total) npow2 <<= 1;
  if ((size_t)npow2 * 8 > 200 * 1024) return nd_fail(h, ND_ERR_UNSUPPORTED, "svd: %d singular values exceed the on-chip sort", total);
  TruncParams tp{mindim < 1 ? 1 : mindim, maxdim, cutoff, cutoff >= 0.0 ? 1 : 0, use_absolute_cutoff, use_relative_cutoff};
  const bool trunc = maxdim >= 0 || cutoff >= 0.0;
  static NdOnce sort_attr;
  nd_once(sort_attr, h->device, [] { return cudaFuncSetAttribute(sort_truncate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
  nd_prof_begin(h, "sort_truncate");
  sort_truncate<<<1, 1024, npow2 * 8, s>>>(sig, total, npow2, 1, 1, tp, P, dlen, res, res + 1);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  nd_prof_begin(h, "kept_dims");
  kept_dims<<<(nb + 127) / 128, 128, 0, s>>>(dblk, nb, sig, res + 1, min_blockdim < 0 ? 0 : min_blockdim, trunc ? 1 : 0, dkept);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  int len = 0;
  double hres[2];
  ND_CUDA(h, cudaMemcpyAsync(kept, dkept, nb * 4, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaMemcpyAsync(&len, dlen, 4, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaMemcpyAsync(hres, res, 16, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaStreamSynchronize(s));
  if (spectrum) ND_CUDA(h, cudaMemcpy(spectrum, P, (size_t)len * 8, cudaMemcpyDeviceToHost));
  if (spectrum_len) *spectrum_len = len;
  if (truncerr) *truncerr = hres[0];
  if (docut) *docut = hres[1];
  // compact kept prefixes (column-major prefixes are contiguous)
  int64_t cu = 0, cs = 0, cv = 0;
  for (int i = 0; i < nb; ++i) {
    const int k = kept[i];
    if (k == 0) continue;
    ND_CUDA(h, cudaMemcpyAsync(U + cu, Uf + uo[i], (size_t)blocks[i].m * k * 8, cudaMemcpyDeviceToDevice, s));
    ND_CUDA(h, cudaMemcpyAsync(S + cs, sig + blocks[i].s_off, (size_t)k * 8, cudaMemcpyDeviceToDevice, s));
    ND_CUDA(h, cudaMemcpyAsync(V + cv, Vf + vo[i], (size_t)blocks[i].n * k * 8, cudaMemcpyDeviceToDevice, s));
    cu += (int64_t)blocks[i].m * k; cs += k; cv += (int64_t)blocks[i].n * k;
  }
  for (void* p : {(void*)Uf, (void*)Vf, (void*)duo, (void*)dvo, (void*)P, (void*)res, (void*)dkept, (void*)dlen,
                  (void*)sig, (void*)order, (void*)W, (void*)Vw, (void*)dblk})
    cudaFreeAsync(p, s);
  ND_CUDA(h, cudaStreamSynchronize(s));
  return nd_check_device_status(h, "svd");
}

extern "C" nd_status nd_bs_eigen_f64(nd_handle h, int32_t nb, const int64_t* dims, const int64_t* offsets,
                                     const double* A, double* D, double* V, int32_t mindim, int32_t maxdim,
                                     double cutoff, int32_t use_absolute_cutoff, int32_t use_relative_cutoff,
                                     int32_t min_blockdim, int32_t* kept, double* spectrum, int32_t* spectrum_len,
                                     double* truncerr, double* docut) {
  if (!h) return ND_ERR_ARG;
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "eigen returns kept dimensions to the host and cannot be captured");
  if (nb < 0 || (nb > 0 && (!dims || !offsets || !A || !D || !V || !kept)))
    return nd_fail(h, ND_ERR_ARG, "eigen: NULL argument");
  if (nb > kMaxBlocksPerCall) return nd_fail(h, ND_ERR_UNSUPPORTED, "eigen: at most %d blocks per call", kMaxBlocksPerCall);
  if (nb == 0) { if (spectrum_len) *spectrum_len = 0; if (truncerr) *truncerr = 0; if (docut) *docut = 0; return ND_OK; }
  cudaStream_t s = h->stream;
  int64_t span = 0;
  for (int i = 0; i < nb; ++i) {
    if (dims[i] <= 0) return nd_fail(h, ND_ERR_ARG, "eigen: block %d has dimension %lld", i, (long long)dims[i]);
    span = std::max(span, offsets[i] + dims[i] * dims[i]);
  }
  // First the batched Jacobi SVD of the blocks themselves: when every singular vector
  // pair shows a clean sign (u_j = +-v_j), that is the eigendecomposition, with the full
  // relative gaps of the spectrum (positive semidefinite blocks, such as density
  // matrices, always take this path).  Otherwise every block is shifted to
  // A + c I with c = 1.01 ||A||_F (positive definite) and decomposed again.
  std::vector<SvdBlock> blocks;
  double *sig = nullptr, *W = nullptr, *Vw = nullptr, *shift = nullptr, *lamJ = nullptr;
  int32_t* order = nullptr;
  SvdBlock* dblk = nullptr;
  int total = 0;
  bool shifted = false;
  nd_status st = svd_core(h, nb, dims, dims, offsets, A, blocks, &sig, &order, &W, &Vw, &dblk, total);
  if (st == ND_ERR_NOCONV) {
    shifted = true;                                    // the shifted problem may still converge
  } else if (st) {
    return st;
  } else {
    int32_t* dflag = nullptr;
    int32_t hflag = 0;
    ND_CUDA(h, cudaMallocAsync(&lamJ, std::max(total, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&dflag, 8, s));
    ND_CUDA(h, cudaMemsetAsync(dflag, 0, 4, s));
    nd_prof_begin(h, "eig_sign");
    eig_sign<<<nb, 256, 0, s>>>(dblk, W, Vw, sig, lamJ, dflag);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    ND_CUDA(h, cudaMemcpyAsync(&hflag, dflag, 4, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaStreamSynchronize(s));
    cudaFreeAsync(dflag, s);
    if (hflag) {
      shifted = true;
      for (void* q : {(void*)sig, (void*)order, (void*)W, (void*)Vw, (void*)dblk, (void*)lamJ}) cudaFreeAsync(q, s);
      sig = W = Vw = lamJ = nullptr; order = nullptr; dblk = nullptr;
    }
  }
  if (shifted) {
    h->last_error.clear();
    std::vector<SvdBlock> hb(nb);
    for (int i = 0; i < nb; ++i) { hb[i] = SvdBlock{}; hb[i].a_off = offsets[i]; hb[i].n = (int)dims[i]; }
    double* As = nullptr;
    SvdBlock* dpre = nullptr;
    ND_CUDA(h, cudaMallocAsync(&As, std::max<int64_t>(span, 1) * 8, s));
    ND_CUDA(h, cudaMallocAsync(&shift, nb * 8, s));
    ND_CUDA(h, cudaMallocAsync(&dpre, nb * sizeof(SvdBlock), s));
    ND_CUDA(h, cudaMemcpyAsync(dpre, hb.data(), nb * sizeof(SvdBlock), cudaMemcpyHostToDevice, s));
    nd_prof_begin(h, "eig_shift");
    eig_shift<<<nb, 256, 0, s>>>(dpre, A, As, shift);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    blocks.clear();
    st = svd_core(h, nb, dims, dims, offsets, As, blocks, &sig, &order, &W, &Vw, &dblk, total);
    cudaFreeAsync(As, s);
    cudaFreeAsync(dpre, s);
    if (st) { cudaFreeAsync(shift, s); return st; }
  }
  std::vector<int64_t> vo(nb);
  int64_t vt = 0;
  for (int i = 0; i < nb; ++i) { vo[i] = vt; vt += dims[i] * dims[i]; }
  int npow2 = 1;
  while (npow2 < total) npow2 <<= 1;
  double *lam = nullptr, *absl = nullptr, *Vf = nullptr, *P = nullptr, *res = nullptr;
  int32_t *vcol = nullptr, *dkept = nullptr;
  int64_t* dvo = nullptr;
  int* dlen = nullptr;
  auto cleanup = [&]() {
    for (void* p : {(void*)lam, (void*)absl, (void*)Vf, (void*)P, (void*)res, (void*)vcol, (void*)dkept, (void*)dvo,
                    (void*)dlen, (void*)sig, (void*)order, (void*)W, (void*)Vw, (void*)dblk, (void*)shift, (void*)lamJ})
      if (p) cudaFreeAsync(p, s);
  };
  if ((size_t)npow2 * 8 > 200 * 1024) { cleanup(); return nd_fail(h, ND_ERR_UNSUPPORTED, "eigen: %d eigenvalues exceed the on-chip sort", total); }
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair((void**)&lam, (size_t)total * 8), std::make_pair((void**)&absl, (size_t)total * 8),
                  std::make_pair((void**)&Vf, (size_t)std::max<int64_t>(vt, 1) * 8),
                  std::make_pair((void**)&P, (size_t)total * 8), std::make_pair((void**)&res, (size_t)32),
                  std::make_pair((void**)&vcol, (size_t)total * 4), std::make_pair((void**)&dkept, (size_t)nb * 4),
                  std::make_pair((void**)&dvo, (size_t)nb * 8), std::make_pair((void**)&dlen, (size_t)8)})
    if (e == cudaSuccess) e = cudaMallocAsync(pr.first, std::max<size_t>(pr.second, 8), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dvo, vo.data(), nb * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { cleanup(); return nd_cuda_check(h, e, "eigen buffers"); }
  nd_prof_begin(h, "eig_finish");
  if (shifted) eig_finish<<<nb, 256, 0, s>>>(dblk, sig, order, shift, lam, absl, vcol);
  else eig_finish_signed<<<nb, 256, 0, s>>>(dblk, order, lamJ, lam, absl, vcol);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  {
    int64_t maxe = 1;
    for (int i = 0; i < nb; ++i) maxe = std::max(maxe, dims[i] * dims[i]);
    dim3 grid((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
    nd_prof_begin(h, "eig_vectors");
    eig_vectors<<<grid, 256, 0, s>>>(dblk, Vw, vcol, Vf, dvo);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  // pooled |lambda|: sort + truncate! on the device, then the kept dims per block
  TruncParams tp{mindim < 1 ? 1 : mindim, maxdim, cutoff, cutoff >= 0.0 ? 1 : 0, use_absolute_cutoff, use_relative_cutoff};
  const bool trunc = maxdim >= 0 || cutoff >= 0.0;
  static NdOnce sort_attr;
  nd_once(sort_attr, h->device, [] { return cudaFuncSetAttribute(sort_truncate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
  nd_prof_begin(h, "sort_truncate");
  sort_truncate<<<1, 1024, npow2 * 8, s>>>(absl, total, npow2, 0, 1, tp, P, dlen, res, res + 1);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  nd_prof_begin(h, "kept_dims");
  kept_dims<<<(nb + 127) / 128, 128, 0, s>>>(dblk, nb, absl, res + 1, min_blockdim < 0 ? 0 : min_blockdim, trunc ? 1 : 0,
                                             dkept, 0);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  int len = 0;
  double hres[2];
  e = cudaMemcpyAsync(kept, dkept, nb * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&len, dlen, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hres, res, 16, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && spectrum) e = cudaMemcpy(spectrum, P, (size_t)len * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { cleanup(); return nd_cuda_check(h, e, "eigen results"); }
  if (spectrum_len) *spectrum_len = len;
  if (truncerr) *truncerr = hres[0];
  if (docut) *docut = hres[1];
  // kept prefixes: D values and V columns (column-major prefixes are contiguous)
  int64_t cd = 0, cv = 0;
  for (int i = 0; i < nb && e == cudaSuccess; ++i) {
    const int k = kept[i];
    if (k == 0) continue;
    e = cudaMemcpyAsync(D + cd, lam + blocks[i].s_off, (size_t)k * 8, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(V + cv, Vf + vo[i], (size_t)dims[i] * k * 8, cudaMemcpyDeviceToDevice, s);
    cd += k;
    cv += dims[i] * k;
  }
  cleanup();
  if (e != cudaSuccess) return nd_cuda_check(h, e, "eigen outputs");
  ND_CUDA(h, cudaStreamSynchronize(s));
  return nd_check_device_status(h, "eigen");
}

// ---------------------------------------------------------------------------
// Blockwise SVD plan: the same three stages for fixed block dimensions, with every
// buffer, task table and GEMM launch state built once, fixed sweep and refinement
// counts, convergence tracked per block on the device and the kept dimensions,
// spectrum and truncation error left in device memory: an execution enqueues work
// only, so it can be captured into a CUDA graph with the Krylov loop of a sweep step.
// ---------------------------------------------------------------------------
namespace {

// after a sweep (one CTA): a block whose sweep rotated nothing is done; reset the sweep
// maxima; any = whether a block is still active
__global__ void svd_active_update(int nb, unsigned long long* offmax, int32_t* active, int32_t* any) {
  __shared__ int a;
  if (threadIdx.x == 0) a = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (offmax[b] == 0ull) active[b] = 0;
    offmax[b] = 0ull;
    if (active[b]) a = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) *any = a;
}

__global__ void svd_fill_i32(int n, int32_t* x, int32_t v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

// status = ND_ERR_NOCONV when a block still rotated in the last FP64 sweep
__global__ void svd_noconv_status(int nb, const int32_t* active, int32_t* status) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (active[b]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) *status = any ? ND_ERR_NOCONV : ND_OK;
}

// kept prefixes of U (m x k), S (k) and V (n x k) of every block, concatenated in block
// order (blocks with kept 0 take no space); one CTA row per block
__global__ void svd_compact(const SvdBlock* blocks, int nb, const int32_t* kept, const double* Uf, const double* Vf,
                            const int64_t* uo, const int64_t* vo, const double* sig, double* U, double* S, double* V) {
  const int bi = blockIdx.y;
  __shared__ int64_t off[3];
  if (threadIdx.x == 0) {
    int64_t cu = 0, cs = 0, cv = 0;
    for (int j = 0; j < bi; ++j) {
      const int k = kept[j];
      cu += (int64_t)blocks[j].m * k;
      cs += k;
      cv += (int64_t)blocks[j].n * k;
    }
    off[0] = cu; off[1] = cs; off[2] = cv;
  }
  __syncthreads();
  const SvdBlock b = blocks[bi];
  const int k = kept[bi];
  const int64_t nu = (int64_t)b.m * k, nv = (int64_t)b.n * k;
  const int64_t str = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nu; e += str) U[off[0] + e] = Uf[uo[bi] + e];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nv; e += str) V[off[2] + e] = Vf[vo[bi] + e];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k; e += str) S[off[1] + e] = sig[b.s_off + e];
}

}  // namespace

struct nd_svd_plan_s {
  nd_handle h = nullptr;
  int nb = 0, total = 0, npow2 = 1, maxn = 1;
  bool big = false;
  int n32 = 0, n64 = 0;                       // fixed sweep counts
  int64_t woff = 0, voff = 0, ut = 0, vt = 0;
  std::vector<SvdBlock> blocks;
  SvdBlock* dblk = nullptr;
  // panel sweeps: group sizes, shared memory, task tables (all blocks, longest first)
  int B32 = 0, B64 = 0, ldp = 0, nrounds32 = 0, nrounds64 = 0, ntasks32 = 0, ntasks64 = 0;
  size_t smem32 = 0, smem64 = 0;
  BjTask *tasks32 = nullptr, *tasks64 = nullptr;
  // work buffers
  double *W = nullptr, *V = nullptr, *sig = nullptr, *Y = nullptr, *Vn = nullptr, *W0 = nullptr, *W1 = nullptr,
         *S = nullptr, *Uf = nullptr, *Vf = nullptr, *P = nullptr, *res = nullptr, *Wsrc = nullptr;
  float *W32 = nullptr, *V32 = nullptr;
  int32_t *order = nullptr, *active = nullptr, *any_active = nullptr, *dkept = nullptr;
  int* dlen = nullptr;
  unsigned long long *offmax = nullptr, *bmax = nullptr, *emax = nullptr;
  unsigned int* bar = nullptr;
  int64_t *duo = nullptr, *dvo = nullptr;
  ExecCache cR, cW, cS, cV, cR64, cW64, cS64, cWE;
  void release();
};

void nd_svd_plan_s::release() {
  if (!h) return;
  for (ExecCache* c : {&cR, &cW, &cS, &cV, &cR64, &cW64, &cS64, &cWE}) c->free_all(h);
  for (void* q : {(void*)dblk, (void*)tasks32, (void*)tasks64, (void*)W, (void*)V, (void*)sig, (void*)Y, (void*)Vn,
                  (void*)W0, (void*)W1, (void*)S, (void*)Uf, (void*)Vf, (void*)P, (void*)res, (void*)Wsrc, (void*)W32,
                  (void*)V32, (void*)order, (void*)active, (void*)any_active, (void*)dkept, (void*)dlen, (void*)offmax, (void*)bmax,
                  (void*)emax, (void*)bar, (void*)duo, (void*)dvo})
    if (q) cudaFreeAsync(q, h->stream);
}

namespace {

template <typename T>
nd_status plan_sweeps(nd_svd_plan p, T* Wt, T* Vt, int nsweeps, double tol, double tol_pow, double tol_cap) {
  nd_handle h = p->h;
  const bool f32 = sizeof(T) == 4;
  const int B = f32 ? p->B32 : p->B64;
  BjArgs<T> a{p->dblk, f32 ? p->tasks32 : p->tasks64, f32 ? p->ntasks32 : p->ntasks64,
              f32 ? p->nrounds32 : p->nrounds64, p->ldp, Wt, Vt, p->offmax, p->bar, p->bar + 1, h->d_status,
              tol, tol_pow, tol_cap, p->active, p->any_active};
  const size_t smem = f32 ? p->smem32 : p->smem64;
  const int gb = (p->nb + 127) / 128;
  ND_CUDA(h, cudaMemsetAsync(p->offmax, 0, p->nb * 8, h->stream));
  svd_fill_i32<<<gb, 128, 0, h->stream>>>(p->nb, p->active, 1);
  svd_fill_i32<<<1, 32, 0, h->stream>>>(1, p->any_active, 1);
  ND_LAUNCHED(h);
  ND_LAUNCHED(h);
  for (int sw = 0; sw < nsweeps; ++sw) {
    nd_status st;
    nd_prof_begin(h, f32 ? "svd_panel_sweep_f32" : "svd_panel_sweep");
    if constexpr (sizeof(T) == 4) {
      st = B == 16 ? launch_bj<T, 16>(h, a, smem) : B == 8 ? launch_bj<T, 8>(h, a, smem) : launch_bj<T, 4>(h, a, smem);
    } else {
      st = B == 8 ? launch_bj<T, 8>(h, a, smem) : B == 4 ? launch_bj<T, 4>(h, a, smem) : launch_bj<T, 2>(h, a, smem);
    }
    nd_prof_end(h);
    ND_LAUNCHED(h);
    if (st) return st;
    svd_active_update<<<1, 256, 0, h->stream>>>(p->nb, p->offmax, p->active, p->any_active);
    ND_LAUNCHED(h);
  }
  return nd_cuda_check(h, cudaGetLastError(), "svd plan sweeps");
}

// The whole SVD of A (blocks at the plan's offsets) into the plan's buffers; no host
// synchronisation.  status (device) receives ND_OK or ND_ERR_NOCONV.
nd_status plan_run(nd_svd_plan p, const double* A, const TruncParams& tp, int min_blockdim, bool trunc,
                   int32_t* status) {
  nd_handle h = p->h;
  cudaStream_t s = h->stream;
  const int nb = p->nb;
  double *W = p->W, *V = p->V, *Vn = p->Vn, *W0 = p->W0, *W1 = p->W1;
  int64_t maxe = 1, maxv = 1;
  for (auto& b : p->blocks) { maxe = std::max(maxe, (int64_t)b.mm * b.nn); maxv = std::max(maxv, (int64_t)b.nn * b.nn); }
  const dim3 ge((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
  const dim3 gv((unsigned)std::min<int64_t>((maxv + 255) / 256, 1024), nb);
  nd_prof_begin(h, "svd_init");
  svd_init<<<ge, 256, 0, s>>>(p->dblk, nb, A, W, V);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  nd_status st = ND_OK;
  if (p->big) {
    ND_CUDA(h, cudaMemsetAsync(p->bmax, 0, nb * 8, s));
    block_absmax<<<ge, 256, 0, s>>>(p->dblk, W, p->bmax);
    to_f32_scaled<<<ge, 256, 0, s>>>(p->dblk, W, p->bmax, p->W32, p->V32);
    ND_LAUNCHED(h);
    ND_LAUNCHED(h);
    if ((st = plan_sweeps<float>(p, p->W32, p->V32, p->n32, ND_SVD_TOL32, ND_SVD_TOL32_POW, INFINITY))) return st;
    v_to_f64<<<gv, 256, 0, s>>>(p->dblk, p->V32, V);
    ND_LAUNCHED(h);
    const int saved = h->ozaki_slices;
    h->ozaki_slices = 6;
    // fixed refinement: ND_SVD_SPLIT_STEPS split-GEMM steps, one FP64 step, one Newton-Schulz step
    for (int it = 0; it < ND_SVD_SPLIT_STEPS + 2 && !st; ++it) {
      const int mode = it < ND_SVD_SPLIT_STEPS ? 0 : it == ND_SVD_SPLIT_STEPS ? 1 : 2;
      const int pr = mode ? ND_PREC_FP64 : ND_PREC_OZAKI;
      set_identity<<<gv, 256, 0, s>>>(p->dblk, p->Y);
      ND_LAUNCHED(h);
      nd_prof_begin(h, "svd_refine_gemm");
      st = block_gemm(h, mode ? p->cR64 : p->cR, p->blocks, p->dblk, 0, V, V, p->Y, -1.0, 1.0, pr);
      if (!st && mode < 2) st = block_gemm(h, mode ? p->cW64 : p->cW, p->blocks, p->dblk, 2, W, V, W0, 1.0, 0.0, pr);
      if (!st && mode < 2) st = block_gemm(h, mode ? p->cS64 : p->cS, p->blocks, p->dblk, 3, W0, W0, p->S, 1.0, 0.0, pr);
      nd_prof_end(h);
      if (st) break;
      const double tau = mode == 0 ? OA_TAU : mode == 1 ? OA_TAU_FP64 : -1.0;
      nd_prof_begin(h, "svd_refine");
      oa_correction<<<gv, 256, 0, s>>>(p->dblk, p->S, p->Y, tau, p->emax);
      ND_LAUNCHED(h);
      st = nd_cuda_check(h, cudaMemcpyAsync(Vn, V, p->voff * 8, cudaMemcpyDeviceToDevice, s), "svd copy");
      if (!st && mode) st = nd_cuda_check(h, cudaMemcpyAsync(W1, W0, p->woff * 8, cudaMemcpyDeviceToDevice, s), "svd copy");
      nd_prof_end(h);
      nd_prof_begin(h, "svd_refine_gemm");
      if (!st) st = block_gemm(h, p->cV, p->blocks, p->dblk, 1, V, p->Y, Vn, 1.0, 1.0, ND_PREC_OZAKI);
      if (!st && mode) st = block_gemm(h, p->cWE, p->blocks, p->dblk, 2, W0, p->Y, W1, 1.0, 1.0, ND_PREC_OZAKI);
      nd_prof_end(h);
      if (st) break;
      std::swap(V, Vn);
      if (mode) std::swap(W0, W1);
    }
    h->ozaki_slices = saved;
    if (st) return st;
    W = W0;                                            // W X
  }
  if ((st = plan_sweeps<double>(p, W, V, p->n64, ND_SVD_TOL64, ND_SVD_TOL64_POW, ND_SVD_TOL64_CAP))) return st;
  svd_noconv_status<<<1, 256, 0, s>>>(nb, p->active, status);
  ND_LAUNCHED(h);
  nd_prof_begin(h, "svd_finish");
  svd_finish<<<nb, 256, p->maxn * 8, s>>>(p->dblk, W, p->sig, p->order);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  {
    dim3 grid((unsigned)std::min<int64_t>((maxe + 255) / 256, 1024), nb);
    nd_prof_begin(h, "svd_outputs");
    svd_outputs<<<grid, 256, 0, s>>>(p->dblk, W, V, p->sig, p->order, p->Uf, p->Vf, p->duo, p->dvo);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  nd_prof_begin(h, "sort_truncate");
  sort_truncate<<<1, 1024, p->npow2 * 8, s>>>(p->sig, p->total, p->npow2, 1, 1, tp, p->P, p->dlen, p->res, p->res + 1);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  kept_dims<<<(nb + 127) / 128, 128, 0, s>>>(p->dblk, nb, p->sig, p->res + 1, min_blockdim < 0 ? 0 : min_blockdim,
                                             trunc ? 1 : 0, p->dkept);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "svd plan");
}

}  // namespace

extern "C" nd_status nd_bs_svd_plan_create(nd_handle h, int32_t nb, const int64_t* rows, const int64_t* cols,
                                           nd_svd_plan* out) {
  if (!h || !out) return ND_ERR_ARG;
  *out = nullptr;
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "svd plan: create it before graph capture");
  if (nb <= 0 || !rows || !cols) return nd_fail(h, ND_ERR_ARG, "svd plan: need at least one block");
  if (nb > kMaxBlocksPerCall) return nd_fail(h, ND_ERR_UNSUPPORTED, "svd plan: at most %d blocks per call", kMaxBlocksPerCall);
  cudaStream_t s = h->stream;
  auto p = new nd_svd_plan_s;
  p->h = h;
  p->nb = nb;
  p->blocks.resize(nb);
  int maxmm = 1;
  double work = 0.0;
  int task0 = 0;
  for (int i = 0; i < nb; ++i) {
    SvdBlock& b = p->blocks[i];
    if (rows[i] <= 0 || cols[i] <= 0 || rows[i] > INT32_MAX || cols[i] > INT32_MAX) {
      delete p;
      return nd_fail(h, ND_ERR_ARG, "svd plan: block %d has invalid dims", i);
    }
    b.m = (int)rows[i]; b.n = (int)cols[i];
    b.trans = b.m < b.n;
    b.mm = b.trans ? b.n : b.m;
    b.nn = b.trans ? b.m : b.n;
    b.npad = b.nn + (b.nn & 1);
    b.w_off = p->woff; p->woff += (int64_t)b.mm * b.nn;
    b.v_off = p->voff; p->voff += (int64_t)b.nn * b.nn;
    b.task0 = task0; b.ntask = b.npad / 2; task0 += b.ntask;
    b.s_off = p->total; p->total += b.nn;
    maxmm = std::max(maxmm, b.mm);
    p->maxn = std::max(p->maxn, b.nn);
    work += (double)b.mm * b.nn * b.nn;
  }
  p->big = work >= 2e8;
  p->B32 = panel_group<float>(maxmm);
  p->B64 = panel_group<double>(maxmm);
  if (!p->B64 || (p->big && !p->B32)) {
    delete p;
    return nd_fail(h, ND_ERR_UNSUPPORTED, "svd plan: a block of %d rows is taller than a shared-memory panel "
                                          "(use nd_bs_svd_f64)", maxmm);
  }
  p->ldp = (maxmm + 3) / 4 * 4;
  p->smem32 = ((size_t)2 * p->B32 * p->ldp + (size_t)4 * p->B32 * p->B32 + 2 * p->B32) * sizeof(float);
  p->smem64 = ((size_t)2 * p->B64 * p->ldp + (size_t)4 * p->B64 * p->B64 + 2 * p->B64) * sizeof(double);
  while (p->npow2 < p->total) p->npow2 <<= 1;
  if ((size_t)p->npow2 * 8 > 200 * 1024) {
    delete p;
    return nd_fail(h, ND_ERR_UNSUPPORTED, "svd plan: %d singular values exceed the on-chip sort", p->total);
  }
  const int ms = h->svd_max_sweeps;
  p->n32 = std::min(24, ms < 0 ? 24 : ms);
  p->n64 = ms < 0 ? (p->big ? 8 : 24) : ms;
  // task tables: every block, longest first
  std::vector<int> ord(nb);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
    return (int64_t)p->blocks[x].mm * p->blocks[x].nn > (int64_t)p->blocks[y].mm * p->blocks[y].nn;
  });
  auto table = [&](int B, std::vector<BjTask>& t, int& nrounds) {
    nrounds = 0;
    for (int bi : ord) {
      const int g = (p->blocks[bi].nn + B - 1) / B, gp = g + (g & 1);
      for (int k = 0; k < gp / 2; ++k) t.push_back(BjTask{bi, k});
      nrounds = std::max(nrounds, gp - 1);
    }
  };
  std::vector<BjTask> t32, t64;
  if (p->big) table(p->B32, t32, p->nrounds32);
  table(p->B64, t64, p->nrounds64);
  p->ntasks32 = (int)t32.size();
  p->ntasks64 = (int)t64.size();
  std::vector<int64_t> uo(nb), vo(nb);
  for (int i = 0; i < nb; ++i) {
    uo[i] = p->ut; p->ut += (int64_t)p->blocks[i].m * p->blocks[i].nn;
    vo[i] = p->vt; p->vt += (int64_t)p->blocks[i].n * p->blocks[i].nn;
  }
  nd_status st = ND_OK;
  auto al = [&](void** q, size_t bytes) { if (!st) st = nd_dalloc(h, q, std::max<size_t>(bytes, 16)); };
  al((void**)&p->dblk, nb * sizeof(SvdBlock));
  al((void**)&p->tasks32, std::max<size_t>(t32.size(), 1) * sizeof(BjTask));
  al((void**)&p->tasks64, std::max<size_t>(t64.size(), 1) * sizeof(BjTask));
  al((void**)&p->W, p->woff * 8); al((void**)&p->V, p->voff * 8); al((void**)&p->sig, p->total * 8);
  al((void**)&p->order, p->total * 4); al((void**)&p->active, nb * 4); al((void**)&p->dkept, nb * 4);
  al((void**)&p->any_active, 16);
  al((void**)&p->offmax, nb * 8); al((void**)&p->bar, 8); al((void**)&p->Uf, p->ut * 8); al((void**)&p->Vf, p->vt * 8);
  al((void**)&p->duo, nb * 8); al((void**)&p->dvo, nb * 8); al((void**)&p->P, p->total * 8);
  al((void**)&p->res, 32); al((void**)&p->dlen, 8);
  if (p->big) {
    al((void**)&p->W32, p->woff * 4); al((void**)&p->V32, p->voff * 4); al((void**)&p->bmax, nb * 8);
    al((void**)&p->Y, p->voff * 8); al((void**)&p->Vn, p->voff * 8); al((void**)&p->S, p->voff * 8);
    al((void**)&p->W0, p->woff * 8); al((void**)&p->W1, p->woff * 8); al((void**)&p->emax, 16);
  }
  al((void**)&p->Wsrc, std::max<int64_t>(p->woff, 1) * 8);
  if (!st) st = nd_upload(h, p->dblk, p->blocks.data(), nb * sizeof(SvdBlock));
  if (!st && !t32.empty()) st = nd_upload(h, p->tasks32, t32.data(), t32.size() * sizeof(BjTask));
  if (!st) st = nd_upload(h, p->tasks64, t64.data(), t64.size() * sizeof(BjTask));
  if (!st) st = nd_upload(h, p->duo, uo.data(), nb * 8);
  if (!st) st = nd_upload(h, p->dvo, vo.data(), nb * 8);
  if (!st) st = nd_cuda_check(h, cudaMemsetAsync(p->bar, 0, 8, s), "svd plan");
  // one run on zeros builds every GEMM's launch state (the state a capture needs)
  if (!st) {
    // the plan's blocks sit back to back at the working offsets of a dummy zero matrix
    st = nd_cuda_check(h, cudaMemsetAsync(p->Wsrc, 0, std::max<int64_t>(p->woff, 1) * 8, s), "svd plan");
  }
  if (!st) {
    static NdOnce sort_attr;
    nd_once(sort_attr, h->device, [] { return cudaFuncSetAttribute(sort_truncate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
    std::vector<SvdBlock> zb = p->blocks;               // a_off: the dummy's block offsets
    int64_t o = 0;
    for (auto& b : zb) { b.a_off = o; o += (int64_t)b.m * b.n; }
    p->blocks = zb;
    st = nd_upload(h, p->dblk, p->blocks.data(), nb * sizeof(SvdBlock));
    int32_t* dstat = nullptr;
    if (!st) st = nd_dalloc(h, (void**)&dstat, 8);
    TruncParams tp{1, -1, -1.0, 0, 0, 1};
    if (!st) st = plan_run(p, p->Wsrc, tp, 0, false, dstat);
    if (dstat) cudaFreeAsync(dstat, s);
    if (!st) st = nd_cuda_check(h, cudaStreamSynchronize(s), "svd plan");
    if (!st) st = nd_check_device_status(h, "svd plan");
  }
  if (st) {
    p->release();
    delete p;
    return st;
  }
  *out = p;
  return ND_OK;
}

extern "C" nd_status nd_bs_svd_plan_exec(nd_svd_plan p, const int64_t* offsets, const double* A, double* U, double* S,
                                         double* V, int32_t mindim, int32_t maxdim, double cutoff,
                                         int32_t use_absolute_cutoff, int32_t use_relative_cutoff, int32_t min_blockdim,
                                         int32_t* kept, double* spectrum, int32_t* spectrum_len, double* truncerr,
                                         int32_t* status) {
  if (!p) return ND_ERR_ARG;
  nd_handle h = p->h;
  if (!offsets || !A || !U || !S || !V || !kept || !spectrum || !spectrum_len || !truncerr || !status)
    return nd_fail(h, ND_ERR_ARG, "svd plan exec: NULL argument");
  // block offsets in A: uploaded when they change (not allowed during capture)
  bool same = true;
  for (int i = 0; i < p->nb; ++i) same = same && p->blocks[i].a_off == offsets[i];
  if (!same) {
    if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "svd plan exec: new block offsets during capture (run once first)");
    for (int i = 0; i < p->nb; ++i) p->blocks[i].a_off = offsets[i];
    nd_status st = nd_upload(h, p->dblk, p->blocks.data(), p->nb * sizeof(SvdBlock));
    if (st) return st;
  }
  TruncParams tp{mindim < 1 ? 1 : mindim, maxdim, cutoff, cutoff >= 0.0 ? 1 : 0, use_absolute_cutoff, use_relative_cutoff};
  const bool trunc = maxdim >= 0 || cutoff >= 0.0;
  nd_status st = plan_run(p, A, tp, min_blockdim, trunc, status);
  if (st) return st;
  cudaStream_t s = h->stream;
  dim3 grid((unsigned)std::min<int64_t>((std::max<int64_t>(p->ut, p->vt) / p->nb + 255) / 256 + 1, 512), p->nb);
  svd_compact<<<grid, 256, 0, s>>>(p->dblk, p->nb, p->dkept, p->Uf, p->Vf, p->duo, p->dvo, p->sig, U, S, V);
  ND_LAUNCHED(h);
  ND_CUDA(h, cudaMemcpyAsync(kept, p->dkept, p->nb * 4, cudaMemcpyDeviceToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(spectrum, p->P, (size_t)p->total * 8, cudaMemcpyDeviceToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(spectrum_len, p->dlen, 4, cudaMemcpyDeviceToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(truncerr, p->res, 8, cudaMemcpyDeviceToDevice, s));
  return nd_cuda_check(h, cudaGetLastError(), "svd plan exec");
}

extern "C" nd_status nd_bs_svd_plan_destroy(nd_svd_plan p) {
  if (!p) return ND_OK;
  p->release();
  delete p;
  return ND_OK;
}

extern "C" nd_status nd_truncate_f64(nd_handle h, const double* Pin, int32_t n, int32_t mindim, int32_t maxdim,
                                     double cutoff, int32_t use_absolute_cutoff, int32_t use_relative_cutoff,
                                     int32_t* newlen, double* truncerr, double* docut) {
  if (!h || !newlen) return ND_ERR_ARG;
  if (n <= 0) return nd_fail(h, ND_ERR_ARG, "truncate: empty spectrum");
  cudaStream_t s = h->stream;
  int npow2 = 1;
  while (npow2 < n) npow2 <<= 1;
  if ((size_t)npow2 * 8 > 200 * 1024) return nd_fail(h, ND_ERR_UNSUPPORTED, "truncate: %d values exceed the on-chip sort", n);
  double *P = nullptr, *res = nullptr;
  int* len = nullptr;
  ND_CUDA(h, cudaMallocAsync(&P, n * 8, s));
  ND_CUDA(h, cudaMallocAsync(&res, 16, s));
  ND_CUDA(h, cudaMallocAsync(&len, 8, s));
  TruncParams tp{mindim < 1 ? 1 : mindim, maxdim, cutoff, cutoff >= 0.0 ? 1 : 0, use_absolute_cutoff, use_relative_cutoff};
  static NdOnce sort_attr;
  nd_once(sort_attr, h->device, [] { return cudaFuncSetAttribute(sort_truncate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
  // the caller's order is kept (truncate! takes a descending spectrum; a negative
  // spectrum is descending in magnitude, which a value sort would reverse)
  nd_prof_begin(h, "sort_truncate");
  sort_truncate<<<1, 1024, npow2 * 8, s>>>(Pin, n, npow2, 0, 0, tp, P, len, res, res + 1);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  double hr[2];
  ND_CUDA(h, cudaMemcpyAsync(newlen, len, 4, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaMemcpyAsync(hr, res, 16, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaStreamSynchronize(s));
  if (truncerr) *truncerr = hr[0];
  if (docut) *docut = hr[1];
  cudaFreeAsync(P, s); cudaFreeAsync(res, s); cudaFreeAsync(len, s);
  return ND_OK;
}

extern "C" nd_status nd_bs_qr_f64(nd_handle h, int32_t nb, const int64_t* rows, const int64_t* cols,
                                  const int64_t* offsets, const double* A, double* Q, double* Rf, int32_t positive) {
  if (!h) return ND_ERR_ARG;
  if (nb < 0 || (nb > 0 && (!rows || !cols || !offsets || !A || !Q || !Rf))) return nd_fail(h, ND_ERR_ARG, "qr: NULL argument");
  if (nb > kMaxBlocksPerCall) return nd_fail(h, ND_ERR_UNSUPPORTED, "qr: at most %d blocks per call", kMaxBlocksPerCall);
  if (nb == 0) return ND_OK;
  cudaStream_t s = h->stream;
  std::vector<QrBlock> blocks(nb);
  int64_t w = 0, q = 0, r = 0, t = 0;
  int32_t tau = 0;
  int npanels = 0, maxm = 0, maxk = 0;
  for (int i = 0; i < nb; ++i) {
    QrBlock& b = blocks[i];
    if (rows[i] <= 0 || cols[i] <= 0 || rows[i] >= INT32_MAX || cols[i] >= INT32_MAX)
      return nd_fail(h, ND_ERR_ARG, "qr: block %d has invalid dims", i);
    b.a_off = offsets[i]; b.m = (int)rows[i]; b.n = (int)cols[i]; b.k = std::min(b.m, b.n);
    b.w_off = w; w += (int64_t)b.m * b.n;
    b.q_off = q; q += (int64_t)b.m * b.k;
    b.r_off = r; r += (int64_t)b.k * b.n;
    const int pb = (b.k + QR_NB - 1) / QR_NB;
    b.t_off = t; t += (int64_t)pb * QR_NB * QR_NB;
    b.tau_off = tau; tau += b.k;
    npanels = std::max(npanels, pb);
    maxm = std::max(maxm, b.m);
    maxk = std::max(maxk, b.k);
  }
  // per panel: the blocks that have it, their trailing strips and their Q strips
  std::vector<int32_t> ids;
  std::vector<QrTask> ttask, qtask;
  std::vector<int64_t> id_off(npanels + 1), tt_off(npanels + 1), qt_off(npanels + 1);
  for (int p = 0; p < npanels; ++p) {
    id_off[p] = (int64_t)ids.size(); tt_off[p] = (int64_t)ttask.size(); qt_off[p] = (int64_t)qtask.size();
    for (int i = 0; i < nb; ++i) {
      const QrBlock& b = blocks[i];
      const int c0 = p * QR_NB;
      if (c0 >= b.k) continue;
      const int wp = std::min(QR_NB, b.k - c0);
      ids.push_back(i);
      for (int c = c0 + wp; c < b.n; c += QR_SW) ttask.push_back(QrTask{i, c, std::min(QR_SW, b.n - c), 0});
      for (int c = c0; c < b.k; c += QR_SW) qtask.push_back(QrTask{i, c, std::min(QR_SW, b.k - c), 0});
    }
  }
  id_off[npanels] = (int64_t)ids.size(); tt_off[npanels] = (int64_t)ttask.size(); qt_off[npanels] = (int64_t)qtask.size();
  if (ttask.size() > INT32_MAX / 2 || qtask.size() > INT32_MAX / 2) return nd_fail(h, ND_ERR_ARG, "qr: too many blocks");
  const size_t bytes_blk = nb * sizeof(QrBlock), bytes_ids = std::max<size_t>(ids.size(), 1) * 4,
               bytes_tt = std::max<size_t>(ttask.size(), 1) * sizeof(QrTask), bytes_qt = std::max<size_t>(qtask.size(), 1) * sizeof(QrTask);
  unsigned char* meta = nullptr;
  double *Wk = nullptr, *taus = nullptr, *Tm = nullptr;
  ND_CUDA(h, cudaMallocAsync(&meta, bytes_blk + bytes_ids + bytes_tt + bytes_qt, s));
  QrBlock* dblk = (QrBlock*)meta;
  int32_t* dids = (int32_t*)(meta + bytes_blk);
  QrTask* dtt = (QrTask*)(meta + bytes_blk + bytes_ids);
  QrTask* dqt = (QrTask*)(meta + bytes_blk + bytes_ids + bytes_tt);
  nd_status st = ND_OK;
  auto fail_free = [&](nd_status e) {
    cudaFreeAsync(meta, s);
    if (Wk) cudaFreeAsync(Wk, s);
    if (taus) cudaFreeAsync(taus, s);
    if (Tm) cudaFreeAsync(Tm, s);
    return e;
  };
  cudaError_t ce = cudaMallocAsync(&Wk, std::max<int64_t>(w, 1) * 8, s);
  if (ce == cudaSuccess) ce = cudaMallocAsync(&taus, std::max<int64_t>(tau, 1) * 8, s);
  if (ce == cudaSuccess) ce = cudaMallocAsync(&Tm, std::max<int64_t>(t, 1) * 8, s);
  if (ce != cudaSuccess) return fail_free(nd_cuda_check(h, ce, "qr scratch"));
  if ((st = nd_upload(h, dblk, blocks.data(), bytes_blk)) || (st = nd_upload(h, dids, ids.data(), ids.size() * 4)) ||
      (st = nd_upload(h, dtt, ttask.data(), ttask.size() * sizeof(QrTask))) ||
      (st = nd_upload(h, dqt, qtask.data(), qtask.size() * sizeof(QrTask))))
    return fail_free(st);
  const int gx = (int)std::min<int64_t>(((int64_t)maxm * std::max(maxk, 1) + 255) / 256, 64);
  nd_prof_begin(h, "qr_init");
  qr_init<<<dim3(std::max(gx, 1), nb), 256, 0, s>>>(dblk, A, Wk, Q);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  for (int p = 0; p < npanels; ++p) {
    const int np_ = (int)(id_off[p + 1] - id_off[p]), nt = (int)(tt_off[p + 1] - tt_off[p]);
    nd_prof_begin(h, "qr_panel");
    qr_panel<<<np_, QR_THREADS, 0, s>>>(dblk, dids + id_off[p], p, Wk, taus, Tm);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    if (nt) {
      nd_prof_begin(h, "qr_apply");
      qr_apply<<<nt, QR_ATHREADS, 0, s>>>(dblk, dtt + tt_off[p], p, Wk, Tm, Wk, 0);
      nd_prof_end(h);
      ND_LAUNCHED(h);
    }
  }
  for (int p = npanels - 1; p >= 0; --p) {
    const int nq = (int)(qt_off[p + 1] - qt_off[p]);
    if (!nq) continue;
    nd_prof_begin(h, "qr_apply");
    qr_apply<<<nq, QR_ATHREADS, 0, s>>>(dblk, dqt + qt_off[p], p, Wk, Tm, Q, 1);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  nd_prof_begin(h, "qr_finish");
  qr_finish<<<dim3(std::max(gx, 1), nb), 256, 0, s>>>(dblk, Wk, Q, Rf, positive);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  st = nd_cuda_check(h, cudaGetLastError(), "qr");
  return fail_free(st);
}

// host list -> device form (mixed-radix index per copy); maxc: the total element count
// (each copy's start in the flat element space is the count of the copies before it)
static nd_status prepare_copies(nd_handle h, int32_t n, const nd_block_copy* list, std::vector<BlockCopyDev>& dl,
                                int64_t& maxc) {
  dl.assign(n, BlockCopyDev{});
  maxc = 0;
  for (int i = 0; i < n; ++i) {
    const nd_block_copy& c = list[i];
    if (c.rank < 0 || c.rank > ND_MAX_RANK) return nd_fail(h, ND_ERR_ARG, "block_copy: rank out of range");
    BlockCopyDev& d = dl[i];
    memset(&d, 0, sizeof(d));
    d.src_off = c.src_off; d.dst_off = c.dst_off;
    d.count = 1;
    d.idx.n = c.rank;
    for (int k = 0; k < c.rank; ++k) {
      if (c.dims[k] < 0 || c.dims[k] > INT32_MAX) return nd_fail(h, ND_ERR_ARG, "block_copy: bad dim");
      d.idx.dim[k] = (int32_t)c.dims[k]; d.idx.st0[k] = c.src_strides[k]; d.idx.st1[k] = c.dst_strides[k];
      d.count *= c.dims[k];
    }
    mixed_simplify(d.idx);
    d.start = maxc;                                    // maxc accumulates the flat total
    maxc += d.count;
  }
  return ND_OK;
}

struct nd_copy_plan_s {
  nd_handle h = nullptr;
  int n = 0;
  int64_t maxc = 0;
  BlockCopyDev* list = nullptr;
};

extern "C" nd_status nd_block_copy_plan_create(nd_handle h, int32_t n, const nd_block_copy* list, nd_copy_plan* out) {
  if (!h || !out) return ND_ERR_ARG;
  *out = nullptr;
  if (n < 0 || (n > 0 && !list)) return nd_fail(h, ND_ERR_ARG, "block_copy_plan: NULL argument");
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "block_copy_plan: create it before graph capture");
  std::vector<BlockCopyDev> dl;
  int64_t maxc = 0;
  nd_status st = prepare_copies(h, n, list, dl, maxc);
  if (st) return st;
  auto p = new nd_copy_plan_s;
  p->h = h; p->n = n; p->maxc = maxc;
  if (n > 0) {
    st = nd_dalloc(h, (void**)&p->list, n * sizeof(BlockCopyDev));
    if (!st) st = nd_upload(h, p->list, dl.data(), n * sizeof(BlockCopyDev));
    if (st) { if (p->list) cudaFreeAsync(p->list, h->stream); delete p; return st; }
  }
  *out = p;
  return ND_OK;
}

extern "C" nd_status nd_block_copy_plan_run(nd_copy_plan p, const double* src, double* dst) {
  if (!p) return ND_ERR_ARG;
  nd_handle h = p->h;
  if (p->n == 0 || p->maxc == 0) return ND_OK;
  if (!src || !dst) return nd_fail(h, ND_ERR_ARG, "block_copy_plan: NULL argument");
  int grid;
  int64_t chunk;
  block_copy_grid(h, p->maxc, grid, chunk);
  nd_prof_begin(h, "block_copy");
  block_copy<<<grid, 256, 0, h->stream>>>(p->list, p->n, p->maxc, chunk, src, dst);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "block_copy");
}

extern "C" nd_status nd_block_copy_plan_destroy(nd_copy_plan p) {
  if (!p) return ND_OK;
  if (p->list) cudaFreeAsync(p->list, p->h->stream);
  delete p;
  return ND_OK;
}

extern "C" nd_status nd_block_copy_f64(nd_handle h, int32_t n, const nd_block_copy* list, const double* src, double* dst) {
  if (!h) return ND_ERR_ARG;
  if (n < 0 || (n > 0 && (!list || !src || !dst))) return nd_fail(h, ND_ERR_ARG, "block_copy: NULL argument");
  if (n == 0) return ND_OK;
  std::vector<BlockCopyDev> dl;
  int64_t maxc = 0;
  nd_status pst = prepare_copies(h, n, list, dl, maxc);
  if (pst) return pst;
  if (maxc == 0) return ND_OK;
  cudaStream_t s = h->stream;
  BlockCopyDev* dd = nullptr;
  ND_CUDA(h, cudaMallocAsync(&dd, n * sizeof(BlockCopyDev), s));
  ND_CUDA(h, cudaMemcpyAsync(dd, dl.data(), n * sizeof(BlockCopyDev), cudaMemcpyHostToDevice, s));
  int grid;
  int64_t chunk;
  block_copy_grid(h, maxc, grid, chunk);
  nd_prof_begin(h, "block_copy");
  block_copy<<<grid, 256, 0, s>>>(dd, n, maxc, chunk, src, dst);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  cudaFreeAsync(dd, s);
  return nd_cuda_check(h, cudaGetLastError(), "block_copy");
}
