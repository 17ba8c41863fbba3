// permutedims for FP64 tensors: R = beta*R + alpha*permutedims(T, perm).
//
// Replaces permutedims!(::Exposed{<:Array}) (NDTensors/src/array/permutedims.jl:5-24,
// Strided.jl) and the GPU broadcast permute of NDTensors/ext/NDTensorsCUDAExt/permutedims.jl.
// The kernel is HBM-bound; its roofline is 16 bytes moved per element
// (24 when beta != 0).
//
// Dimensions of size 1 are dropped and dimensions that stay adjacent in both
// layouts are fused.  Then:
//   * perm[0] == 0: both tensors share their contiguous dimension, rows are
//     copied with 128-bit accesses (kernel permute_rows);
//   * otherwise a tiled transpose through shared memory, 32(i) x 64(j) FP64 tiles
//     with i flattened over several T dims (T's contiguous one first) and j over
//     several R dims (R's contiguous one first), so tiles stay full however small
//     each extent is (kernel permute_groups, plain loads);
//   * on request (nd_set_permute_path), a TMA variant tiles T's contiguous dim (i)
//     against the T dim that becomes R's contiguous one (j): tiles staged by
//     cp.async.bulk.tensor (128-byte swizzle, 4-stage mbarrier ring, persistent
//     grid), 128-bit stores along j (kernel permute_tma).  It was the default until
//     the group tiling measured faster on every shape of the 1 GiB rank-3..6 sweep
//     (0.86-0.96 of HBM against 0.83-0.89 for the shapes TMA takes; 0.46 / 0.30
//     for TMA and the one-dimension plain tiling on rank-5 / rank-6 reversals).
#include "nd_common.h"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <cstring>

namespace {

struct PermParams {
  int64_t total;
  int32_t n;                   // fused rank
  int64_t d0, dq;              // extents of i (T dim 0) and j (T dim q)
  int64_t rs_i;                // R stride of the i dimension
  int64_t ts_j;                // T stride of the j dimension
  int32_t nb;                  // number of batch dims
  int64_t bdim[ND_MAX_RANK];   // batch extents
  int64_t bts[ND_MAX_RANK];    // batch T strides
  int64_t brs[ND_MAX_RANK];    // batch R strides
  int32_t bcoord[ND_MAX_RANK]; // batch dim index in T (TMA coordinate slot)
  int32_t q;                   // T dim index of j (TMA coordinate slot)
  int64_t ntile_i, ntile_j, ntiles;
  double alpha, beta;
  int32_t mode;                // 0 copy, 1 scale, 2 beta==1 accumulate, 3 general, 4 zero, 5 beta-only
  int32_t vec;                 // 128-bit stores allowed
  const double* scalar;        // optional device scalar multiplying alpha
  // tile / batch index decomposition by multiply-high (all indices < 2^31 when fast != 0)
  int32_t fast;
  uint32_t mul_j, shr_j, mul_i, shr_i;
  uint32_t bmul[ND_MAX_RANK], bshr[ND_MAX_RANK];
  // permute_groups: i runs over the dims of group I (T's dim 0 first), j over the dims
  // of group J (R's dim 0 first); both flattened, with their T and R strides
  int32_t ni, nj;
  int64_t iext[ND_MAX_RANK], its[ND_MAX_RANK], irs[ND_MAX_RANK];
  int64_t jext[ND_MAX_RANK], jts[ND_MAX_RANK], jrs[ND_MAX_RANK];
  uint32_t imul[ND_MAX_RANK], ishr[ND_MAX_RANK], jmul[ND_MAX_RANK], jshr[ND_MAX_RANK];
};

// q = x / d for 0 <= x < 2^31 with the divisor's precomputed (mul, shr), else plain division
__device__ __forceinline__ int64_t pdiv(const PermParams& p, int64_t x, int64_t d, uint32_t mul, uint32_t shr) {
  if (p.fast) {
    const uint32_t u = (uint32_t)x;
    return (int64_t)((__umulhi(u, mul) + u) >> shr);
  }
  return x / d;
}

// divisor magic for the multiply-high division (Granlund & Montgomery, round-up multiplier)
void fast_divisor(int64_t d, uint32_t& mul, uint32_t& shr) {
  shr = 0;
  while ((1ll << shr) < d) ++shr;
  mul = (uint32_t)((((1ull << 32) * ((1ull << shr) - (uint64_t)d)) / (uint64_t)d) + 1ull);
}

// COPY: mode 0 resolved at compile time, so the plain copy carries no FP64 arithmetic
// (the compiler would otherwise turn the runtime switch into selects and evaluate a * t
// for every element on GB300's narrow FP64 pipe).
template <bool COPY>
__device__ __forceinline__ double combine(const PermParams& p, double a, double t, const double* rp) {
  if (COPY) return t;
  switch (p.mode) {
    case 0: return t;
    case 1: return a * t;
    case 2: return *rp + a * t;
    case 3: return a * t + p.beta * *rp;
    case 4: return 0.0;
    default: return p.beta * *rp;
  }
}

__device__ __forceinline__ double eff_alpha(const PermParams& p) {
  return p.scalar ? p.alpha * __ldg(p.scalar) : p.alpha;
}

__device__ __forceinline__ void batch_offsets(const PermParams& p, int64_t b, int64_t& to, int64_t& ro, int32_t* coord) {
  to = 0; ro = 0;
  for (int d = 0; d < p.nb; ++d) {
    int64_t q = pdiv(p, b, p.bdim[d], p.bmul[d], p.bshr[d]);
    int64_t r = b - q * p.bdim[d];
    to += r * p.bts[d];
    ro += r * p.brs[d];
    if (coord) coord[d] = (int32_t)r;
    b = q;
  }
}

// ---- mbarrier / TMA helpers (bounded waits) -------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Progress wait (drain == false): gives up after the handle's spin limit, or early
// once another CTA has recorded a timeout.  Clean-up wait (drain == true): waits for
// copies already issued with the fixed ND_SPIN_LIMIT and no early exit.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, DeviceStatus* st, int site, bool drain,
                                          uint32_t lim) {
  if (drain) lim = ND_SPIN_LIMIT;
  for (uint32_t it = 0; it < lim; ++it) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    if (ok) return true;
    if (!drain && (it & 1023) == 1023 && *(volatile int32_t*)&st->code == ND_ERR_TIMEOUT) return false;
  }
  if (atomicCAS(&st->code, 0, ND_ERR_TIMEOUT) == 0) st->where = site;
  return false;
}

constexpr int TI = 32, TJ = 64, STAGES = 4;
constexpr int BOX_I = 16;                       // 16 doubles = 128 bytes (swizzle span)
constexpr int TILE_BYTES = TI * TJ * 8;         // 16 KB
constexpr int BOX_BYTES = BOX_I * TJ * 8;       // 8 KB

template <bool COPY>
__global__ void __launch_bounds__(256) permute_tma(const __grid_constant__ CUtensorMap tmap, double* R,
                                                   const double* Rin, PermParams p, DeviceStatus* st) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[STAGES];
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  const double a = eff_alpha(p);
  const uint32_t lim = tid == 0 ? nd_spin_limit(st) : 0u;   // only thread 0 waits
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&full[s])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("prefetch.tensormap [%0];" :: "l"(&tmap) : "memory");
  }
  __syncthreads();
  const int64_t first = blockIdx.x, stride = gridDim.x;
  auto issue = [&](int64_t t, int s) {
    int64_t rest = pdiv(p, t, p.ntile_j, p.mul_j, p.shr_j);
    int64_t tj = t - rest * p.ntile_j;
    int64_t b = pdiv(p, rest, p.ntile_i, p.mul_i, p.shr_i);
    int64_t ti = rest - b * p.ntile_i;
    int32_t c[5] = {0, 0, 0, 0, 0};
    int64_t to, ro;
    int32_t bc[ND_MAX_RANK];
    batch_offsets(p, b, to, ro, bc);
    for (int d = 0; d < p.nb; ++d) c[p.bcoord[d]] = bc[d];
    c[0] = (int32_t)(ti * TI);
    c[p.q] = (int32_t)(tj * TJ);
    uint32_t bar = smem_u32(&full[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(TILE_BYTES) : "memory");
    for (int h = 0; h < 2; ++h) {
      uint32_t dst = smem_u32(smem + s * TILE_BYTES + h * BOX_BYTES);
      int32_t x = c[0] + h * BOX_I;
      asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                   :: "r"(dst), "l"(&tmap), "r"(x), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(bar) : "memory");
    }
  };
  // prologue
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      int64_t t = first + s * stride;
      if (t < p.ntiles) issue(t, s);
    }
  }
  uint32_t phase = 0;                            // bit s: parity of the next completion of stage s
  int s = 0;
  bool ok = true;
  int64_t t_stop = 0;                            // tile whose wait gave up
  for (int64_t t = first; t < p.ntiles; t += stride) {
    // one thread polls the barrier and broadcasts, so every thread leaves together
    if (tid == 0) s_ok = mbar_wait(smem_u32(&full[s]), (phase >> s) & 1u, st, 100, false, lim) ? 1 : 0;
    __syncthreads();
    ok = s_ok != 0;
    if (!ok) { t_stop = t; break; }
    phase ^= 1u << s;                            // stage s consumed
    int64_t rest = pdiv(p, t, p.ntile_j, p.mul_j, p.shr_j);
    int64_t tj = t - rest * p.ntile_j;
    int64_t b = pdiv(p, rest, p.ntile_i, p.mul_i, p.shr_i);
    int64_t ti = rest - b * p.ntile_i;
    int64_t to, ro;
    batch_offsets(p, b, to, ro, nullptr);
    const int64_t i0 = ti * TI, j0 = tj * TJ;
    const unsigned char* tile = smem + s * TILE_BYTES;
    const int warp = tid >> 5, lane = tid & 31;
    for (int ii = warp; ii < TI; ii += 8) {
      const int64_t i = i0 + ii;
      if (i >= p.d0) break;
      const int j = lane * 2;
      const int h = ii / BOX_I, il = ii % BOX_I;
      const unsigned char* box = tile + h * BOX_BYTES;
      double v0 = *(const double*)(box + j * 128 + ((((il >> 1) ^ (j & 7)) << 4)) + (il & 1) * 8);
      double v1 = *(const double*)(box + (j + 1) * 128 + ((((il >> 1) ^ ((j + 1) & 7)) << 4)) + (il & 1) * 8);
      const int64_t jg = j0 + j;
      const int64_t roff = ro + i * p.rs_i + jg;
      if (p.vec && jg + 1 < p.dq) {
        double2 o;
        if (p.mode >= 2) {
          double2 old = *(const double2*)(Rin + roff);
          o.x = combine<COPY>(p, a, v0, &old.x);
          o.y = combine<COPY>(p, a, v1, &old.y);
        } else {
          o.x = combine<COPY>(p, a, v0, nullptr);
          o.y = combine<COPY>(p, a, v1, nullptr);
        }
        *(double2*)(R + roff) = o;
      } else {
        if (jg < p.dq) R[roff] = combine<COPY>(p, a, v0, Rin + roff);
        if (jg + 1 < p.dq) R[roff + 1] = combine<COPY>(p, a, v1, Rin + roff + 1);
      }
    }
    __syncthreads();   // every thread is done with stage s
    if (tid == 0) {
      int64_t tn = t + (int64_t)STAGES * stride;
      if (tn < p.ntiles) issue(tn, s);
    }
    s = (s + 1) % STAGES;
  }
  // After a timeout, wait for the copies still in flight before the CTA exits (on
  // the normal path every issued tile was consumed).  Issued and not consumed are
  // the tiles t_stop, t_stop + stride, ... (at most STAGES of them, the ring ahead
  // of the consumer), in stages s, s + 1, ...; none of those stages has flipped its
  // phase bit since the copy was issued.
  if (!ok && tid == 0) {
    for (int k = 0; k < STAGES; ++k) {
      const int64_t tk = t_stop + (int64_t)k * stride;
      if (tk >= p.ntiles) break;
      const int q = (s + k) % STAGES;
      mbar_wait(smem_u32(&full[q]), (phase >> q) & 1u, st, 101, true, lim);
    }
  }
}

// T and R offsets of flattened index x over extents ext[0..n) (ext[0] fastest).
__device__ __forceinline__ void group_offsets(const PermParams& p, int64_t x, int n, const int64_t* ext,
                                              const int64_t* st, const int64_t* sr, const uint32_t* mul,
                                              const uint32_t* shr, int64_t& ot, int64_t& orr) {
  ot = 0;
  orr = 0;
  for (int k = 0; k < n; ++k) {
    const int64_t q = k + 1 < n ? pdiv(p, x, ext[k], mul[k], shr[k]) : 0;
    const int64_t r = x - q * ext[k];
    ot += r * st[k];
    orr += r * sr[k];
    x = q;
  }
}

// Tiled transpose over dimension groups, plain loads: T -> smem (padded) -> R.  The
// tile's i axis is flattened over the dims of group I (T's dim 0 first, so a warp's 32
// loads along i are contiguous over that dim) and its j axis over group J (R's dim 0
// first, so a warp's stores along j are contiguous over that dim); the groups are
// filled up to 32 and 64 elements, so tiles stay full however small each extent is.
// Per tile the T and R offsets of its i's and j's are decoded once into shared
// memory; each thread issues its eight loads before storing any of them.
template <bool COPY>
__global__ void __launch_bounds__(256) permute_groups(const double* __restrict__ T, double* R,
                                                      const double* Rin, PermParams p) {
  __shared__ double tile[TJ][TI + 1];
  __shared__ int64_t jt[TJ], jr[TJ], it[TI], ir[TI];
  const double a = eff_alpha(p);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
    int64_t rest = pdiv(p, t, p.ntile_j, p.mul_j, p.shr_j);
    int64_t tj = t - rest * p.ntile_j;
    int64_t b = pdiv(p, rest, p.ntile_i, p.mul_i, p.shr_i);
    int64_t ti = rest - b * p.ntile_i;
    int64_t to, ro;
    batch_offsets(p, b, to, ro, nullptr);
    const int64_t i0 = ti * TI, j0 = tj * TJ;
    if (tid < TJ) {
      const int64_t j = j0 + tid;
      int64_t ot = 0, orr = 0;
      if (j < p.dq) group_offsets(p, j, p.nj, p.jext, p.jts, p.jrs, p.jmul, p.jshr, ot, orr);
      jt[tid] = to + ot;
      jr[tid] = ro + orr;
    } else if (tid < TJ + TI) {
      const int64_t i = i0 + tid - TJ;
      int64_t ot = 0, orr = 0;
      if (i < p.d0) group_offsets(p, i, p.ni, p.iext, p.its, p.irs, p.imul, p.ishr, ot, orr);
      it[tid - TJ] = ot;
      ir[tid - TJ] = orr;
    }
    __syncthreads();
    // load: lanes along i
    {
      const bool iok = i0 + lane < p.d0;
      const int64_t oi = it[lane];
      double v[TJ / 8];
#pragma unroll
      for (int k = 0; k < TJ / 8; ++k) {
        const int jj = warp + 8 * k;
        v[k] = (iok && j0 + jj < p.dq) ? __ldg(T + jt[jj] + oi) : 0.0;
      }
#pragma unroll
      for (int k = 0; k < TJ / 8; ++k) tile[warp + 8 * k][lane] = v[k];
    }
    __syncthreads();
    // store: lanes along j
#pragma unroll
    for (int k = 0; k < TI / 8; ++k) {
      const int ii = warp + 8 * k;
      if (i0 + ii < p.d0) {
        const int64_t ri = ir[ii];
#pragma unroll
        for (int h = 0; h < TJ / 32; ++h) {
          const int jj = lane + 32 * h;
          if (j0 + jj < p.dq) {
            const int64_t roff = ri + jr[jj];
            R[roff] = combine<COPY>(p, a, tile[jj][ii], Rin + roff);
          }
        }
      }
    }
    __syncthreads();
  }
}

// Shared contiguous dimension: copy rows of length d0 (i) for every batch index.
template <bool COPY>
__global__ void __launch_bounds__(256) permute_rows(const double* __restrict__ T, double* R,
                                                    const double* Rin, PermParams p) {
  const double a = eff_alpha(p);
  const int64_t nrows = p.ntiles;
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t row = (int64_t)blockIdx.x * warps + warp; row < nrows; row += (int64_t)gridDim.x * warps) {
    int64_t to, ro;
    batch_offsets(p, row, to, ro, nullptr);
    if (p.vec) {
      const int64_t n2 = p.d0 >> 1;
      for (int64_t c = lane; c < n2; c += 32) {
        double2 v = __ldg((const double2*)(T + to) + c);
        double2 o;
        if (p.mode >= 2) {
          double2 old = *((const double2*)(Rin + ro) + c);
          o.x = combine<COPY>(p, a, v.x, &old.x);
          o.y = combine<COPY>(p, a, v.y, &old.y);
        } else {
          o.x = combine<COPY>(p, a, v.x, nullptr);
          o.y = combine<COPY>(p, a, v.y, nullptr);
        }
        *((double2*)(R + ro) + c) = o;
      }
    } else {
      for (int64_t c = lane; c < p.d0; c += 32) R[ro + c] = combine<COPY>(p, a, __ldg(T + to + c), Rin + ro + c);
    }
  }
}

__global__ void permute_scalar(const double* T, double* R, PermParams p) {
  if (threadIdx.x == 0 && blockIdx.x == 0) R[0] = combine<false>(p, eff_alpha(p), T[0], R);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once (a function-local static is initialised once, thread-safely)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)f;
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

}  // namespace

nd_status nd_launch_permute(nd_handle h, double* R, const double* T, int rank, const int64_t* dims,
                            const int* perm0, double alpha, double beta, const double* scalar_dev) {
  // drop singleton dims
  int64_t d[ND_MAX_RANK];
  int nk = 0;
  int64_t total = 1;
  for (int k = 0; k < rank; ++k) total *= dims[k];
  if (total == 0) return ND_OK;
  int newpos[ND_MAX_RANK];
  for (int k = 0; k < rank; ++k) {
    if (dims[k] != 1) { newpos[k] = nk; d[nk] = dims[k]; nk++; }
    else newpos[k] = -1;
  }
  int pr[ND_MAX_RANK], npr = 0;   // R position -> T (reduced) dim
  for (int r = 0; r < rank; ++r) if (newpos[perm0[r]] >= 0) pr[npr++] = newpos[perm0[r]];
  // fuse T dims (t, t+1) that are adjacent in R
  int posR[ND_MAX_RANK];
  for (int r = 0; r < npr; ++r) posR[pr[r]] = r;
  int grp[ND_MAX_RANK];  // fused group id of each reduced T dim
  int ng = 0;
  int64_t gd[ND_MAX_RANK];
  for (int t = 0; t < nk; ++t) {
    if (t > 0 && posR[t] == posR[t - 1] + 1) { grp[t] = grp[t - 1]; gd[grp[t]] *= d[t]; }
    else { grp[t] = ng; gd[ng] = d[t]; ng++; }
  }
  int gperm[ND_MAX_RANK], ngp = 0;   // R order of fused groups
  for (int r = 0; r < npr; ++r) {
    int g = grp[pr[r]];
    if (ngp == 0 || gperm[ngp - 1] != g) gperm[ngp++] = g;
  }
  // strides
  int64_t ts[ND_MAX_RANK], rs[ND_MAX_RANK];
  { int64_t s = 1; for (int g = 0; g < ng; ++g) { ts[g] = s; s *= gd[g]; } }
  { int64_t s = 1; for (int r = 0; r < ngp; ++r) { rs[gperm[r]] = s; s *= gd[gperm[r]]; } }

  PermParams p{};
  p.total = total;
  p.n = ng;
  p.alpha = alpha;
  p.beta = beta;
  p.scalar = scalar_dev;
  if (beta == 0.0) p.mode = (alpha == 0.0 && !scalar_dev) ? 4 : ((alpha == 1.0 && !scalar_dev) ? 0 : 1);
  else if (alpha == 0.0 && !scalar_dev) p.mode = 5;
  else p.mode = (beta == 1.0) ? 2 : 3;
  const double* Rin = R;
  const int threads = 256;

  if (ng <= 1 || gperm[0] == 0) {
    // shared contiguous dim (or scalar / pure copy)
    if (total == 1) {
      nd_prof_begin(h, "permute_scalar");
      permute_scalar<<<1, 32, 0, h->stream>>>(T, R, p);
      nd_prof_end(h);
      ND_LAUNCHED(h);
      return nd_cuda_check(h, cudaGetLastError(), "permute_scalar");
    }
    p.d0 = (ng == 0) ? 1 : gd[0];
    p.nb = 0;
    for (int g = 1; g < ng; ++g) { p.bdim[p.nb] = gd[g]; p.bts[p.nb] = ts[g]; p.brs[p.nb] = rs[g]; p.nb++; }
    p.ntiles = total / p.d0;   // rows
    p.fast = p.ntiles < (int64_t)0x7fffffff;
    for (int b = 0; b < p.nb; ++b) fast_divisor(p.bdim[b], p.bmul[b], p.bshr[b]);
    bool al = ((uintptr_t)T % 16 == 0) && ((uintptr_t)R % 16 == 0) && (p.d0 % 2 == 0);
    p.vec = al ? 1 : 0;
    int64_t blocks = std::min<int64_t>((p.ntiles + 7) / 8, (int64_t)h->num_sms * 8);
    nd_prof_begin(h, "permute_rows");
    if (p.mode == 0) permute_rows<true><<<(unsigned)std::max<int64_t>(blocks, 1), threads, 0, h->stream>>>(T, R, Rin, p);
    else permute_rows<false><<<(unsigned)std::max<int64_t>(blocks, 1), threads, 0, h->stream>>>(T, R, Rin, p);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    return nd_cuda_check(h, cudaGetLastError(), "permute_rows");
  }
  // transpose: i = T group 0, j = T group gperm[0]
  int q = gperm[0];
  bool rvec = ((uintptr_t)R % 16 == 0) && (rs[0] % 2 == 0);
  for (int g = 1; g < ng; ++g) if (g != q && rs[g] % 2) rvec = false;
  auto enc = encode_fn();
  // the TMA tiling (one dimension on each side of the tile) runs when the handle asks
  // for it and TMA can describe the shape; the dimension-group tiling is the default
  bool tma_ok = h->permute_tma && enc && ng <= 5 && (gd[0] % 2 == 0) && ((uintptr_t)T % 16 == 0);
  for (int g = 0; g < ng && tma_ok; ++g) if (gd[g] > (int64_t)0x7fffffff) tma_ok = false;
  if (tma_ok) {
    p.d0 = gd[0];
    p.dq = gd[q];
    p.rs_i = rs[0];
    p.ts_j = ts[q];
    p.q = q;
    p.nb = 0;
    for (int g = 1; g < ng; ++g) {
      if (g == q) continue;
      p.bdim[p.nb] = gd[g]; p.bts[p.nb] = ts[g]; p.brs[p.nb] = rs[g]; p.bcoord[p.nb] = g; p.nb++;
    }
    p.ntile_i = (p.d0 + TI - 1) / TI;
    p.ntile_j = (p.dq + TJ - 1) / TJ;
    int64_t nbatch = total / (p.d0 * p.dq);
    p.ntiles = p.ntile_i * p.ntile_j * nbatch;
    p.fast = p.ntiles < (int64_t)0x7fffffff;
    fast_divisor(p.ntile_j, p.mul_j, p.shr_j);
    fast_divisor(p.ntile_i, p.mul_i, p.shr_i);
    for (int b = 0; b < p.nb; ++b) fast_divisor(p.bdim[b], p.bmul[b], p.bshr[b]);
    p.vec = rvec ? 1 : 0;
    CUtensorMap tmap;
    cuuint64_t gdim[5] = {1, 1, 1, 1, 1};
    cuuint64_t gstride[4] = {0, 0, 0, 0};
    cuuint32_t box[5] = {1, 1, 1, 1, 1};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    for (int g = 0; g < 5; ++g) gdim[g] = g < ng ? (cuuint64_t)gd[g] : 1;
    for (int g = 1; g < 5; ++g) {
      int64_t st = g < ng ? ts[g] * 8 : ts[ng - 1] * gd[ng - 1] * 8;
      gstride[g - 1] = (cuuint64_t)st;
    }
    box[0] = BOX_I;
    box[q] = TJ;
    CUresult r = enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, (void*)T, gdim, gstride, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS) {
      size_t smem = STAGES * TILE_BYTES + 1024;
      static NdOnce attr;
      nd_once(attr, h->device, [smem] {
        cudaError_t e = cudaFuncSetAttribute(permute_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e == cudaSuccess ? cudaFuncSetAttribute(permute_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                : e;
      });
      int64_t blocks = std::min<int64_t>(p.ntiles, (int64_t)h->num_sms * 3);
      nd_prof_begin(h, "permute_tma");
      if (p.mode == 0) permute_tma<true><<<(unsigned)blocks, threads, smem, h->stream>>>(tmap, R, Rin, p, h->d_status);
      else permute_tma<false><<<(unsigned)blocks, threads, smem, h->stream>>>(tmap, R, Rin, p, h->d_status);
      nd_prof_end(h);
      ND_LAUNCHED(h);
      return nd_cuda_check(h, cudaGetLastError(), "permute_tma");
    }
  }
  // plain-load tiling over dimension groups: J = R's dims in R order (skipping T's dim
  // 0) until their product reaches TJ, then I = T's dims in T order (skipping J's)
  // until theirs reaches TI; the remaining dims are the batch
  bool inJ[ND_MAX_RANK] = {false}, inI[ND_MAX_RANK] = {false};
  int64_t DJ = 1, DI = 1;
  p.nj = 0;
  for (int r = 0; r < ngp && DJ < TJ; ++r) {
    const int g = gperm[r];
    if (g == 0) continue;
    inJ[g] = true;
    p.jext[p.nj] = gd[g]; p.jts[p.nj] = ts[g]; p.jrs[p.nj] = rs[g]; p.nj++;
    DJ *= gd[g];
  }
  p.ni = 0;
  for (int g = 0; g < ng && DI < TI; ++g) {
    if (inJ[g]) continue;
    inI[g] = true;
    p.iext[p.ni] = gd[g]; p.its[p.ni] = ts[g]; p.irs[p.ni] = rs[g]; p.ni++;
    DI *= gd[g];
  }
  p.nb = 0;
  for (int g = 0; g < ng; ++g) {
    if (inI[g] || inJ[g]) continue;
    p.bdim[p.nb] = gd[g]; p.bts[p.nb] = ts[g]; p.brs[p.nb] = rs[g]; p.bcoord[p.nb] = g; p.nb++;
  }
  p.d0 = DI;
  p.dq = DJ;
  p.ntile_i = (DI + TI - 1) / TI;
  p.ntile_j = (DJ + TJ - 1) / TJ;
  p.ntiles = p.ntile_i * p.ntile_j * (total / (DI * DJ));
  p.fast = p.ntiles < (int64_t)0x7fffffff && DI < (int64_t)0x7fffffff && DJ < (int64_t)0x7fffffff;
  fast_divisor(p.ntile_j, p.mul_j, p.shr_j);
  fast_divisor(p.ntile_i, p.mul_i, p.shr_i);
  for (int b = 0; b < p.nb; ++b) fast_divisor(p.bdim[b], p.bmul[b], p.bshr[b]);
  for (int k = 0; k < p.ni; ++k) fast_divisor(p.iext[k], p.imul[k], p.ishr[k]);
  for (int k = 0; k < p.nj; ++k) fast_divisor(p.jext[k], p.jmul[k], p.jshr[k]);
  int64_t blocks = std::min<int64_t>(p.ntiles, (int64_t)h->num_sms * 8);
  nd_prof_begin(h, "permute_groups");
  if (p.mode == 0) permute_groups<true><<<(unsigned)blocks, threads, 0, h->stream>>>(T, R, Rin, p);
  else permute_groups<false><<<(unsigned)blocks, threads, 0, h->stream>>>(T, R, Rin, p);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "permute_groups");
}

extern "C" nd_status nd_permutedims_f64(nd_handle h, double* R, const double* T, int32_t rank,
                                        const int64_t* dimsT, const int32_t* perm, double alpha, double beta) {
  if (!h) return ND_ERR_ARG;
  if (rank < 0 || rank > ND_MAX_RANK) return nd_fail(h, ND_ERR_ARG, "permutedims: rank %d out of range", rank);
  if (rank > 0 && (!dimsT || !perm)) return nd_fail(h, ND_ERR_ARG, "permutedims: NULL dims/perm");
  int p0[ND_MAX_RANK];
  bool seen[ND_MAX_RANK] = {false};
  int64_t total = 1;
  for (int k = 0; k < rank; ++k) {
    if (dimsT[k] < 0) return nd_fail(h, ND_ERR_ARG, "permutedims: negative dim");
    total *= dimsT[k];
    int v = perm[k] - 1;
    if (v < 0 || v >= rank || seen[v]) return nd_fail(h, ND_ERR_ARG, "permutedims: perm is not a permutation of 1..%d", rank);
    seen[v] = true;
    p0[k] = v;
  }
  if (total > 0 && (!R || !T)) return nd_fail(h, ND_ERR_ARG, "permutedims: NULL data pointer");
  if (R == T && total > 1) return nd_fail(h, ND_ERR_ARG, "permutedims: R and T must not alias");
  int64_t d1[1] = {1};
  return nd_launch_permute(h, R, T, rank, rank ? dimsT : d1, p0, alpha, beta, nullptr);
}
