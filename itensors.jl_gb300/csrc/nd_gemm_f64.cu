// Plain FP64 grouped GEMM on the FP64 tensor cores (DMMA, mma.sync.m8n8k4.f64).
//
// This is the FP64 drop-in for BLAS.gemm! / cuBLAS mul! reached from
// _contract! (NDTensors/src/abstractarray/tensoralgebra/contract.jl:40-85,115-188)
// and for the per-block-pair loop of the block-sparse contraction
// (NDTensors/src/blocksparse/contract_generic.jl:78-129).  tcgen05 has no FP64
// kind, so DMMA is the FP64 tensor path on sm_103a; it is bound by the FP64
// pipe, not by memory.
//
// One launch runs every block pair of a contraction: a work item is one 64x64
// tile of one output block (group); the CTA walks the group's pairs in plan
// order, accumulating in registers, so the first pair "overwrites" and the
// rest "accumulate" exactly like beta = 0 then 1 in the reference.  Operands
// are read through mixed-radix offset tables, so permuted inputs / outputs
// need no separate permute pass (the permutations of ContractionProperties are
// folded into the addressing).
#include "nd_common.h"
#include <algorithm>

namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BM + 4;

struct GemmArgs {
  const PairDesc* pairs;
  const WorkItem* items;
  int nitems;
  JobPtrs ptrs;
  double alpha, beta;
  int32_t amode;   // 0: alpha == 1
  int32_t bmode;   // 0: beta == 0 (overwrite)
  double* ws;      // split-K partial tiles, BM * BN doubles per slot (column-major in the tile)
};

__device__ __forceinline__ void dmma(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) gemm_f64_grouped(GemmArgs g) {
  __shared__ double As[BK][LDS];
  __shared__ double Bs[BK][LDS];
  __shared__ int64_t rowA[BM], rowR[BM], colB[BN], colR[BN];
  __shared__ int64_t kA[BK], kB[BK];
  __shared__ PairDesc pd;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;

  for (int it = blockIdx.x; it < g.nitems; it += gridDim.x) {
    const WorkItem wi = g.items[it];
    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
    int64_t r_base = 0;
    double* Rp = nullptr;
    int M = 0, N = 0;
    int kcur = 0;                      // start of this pair on the group's concatenated k axis
    for (int pi = 0; pi < wi.pair_count; ++pi) {
      __syncthreads();
      if (tid == 0) pd = g.pairs[wi.pair_begin + pi];
      __syncthreads();
      M = pd.M; N = pd.N;
      int klo = 0, khi = pd.K;
      if (wi.slot >= 0) {
        klo = max(0, wi.kbeg - kcur);
        khi = min(pd.K, wi.kend - kcur);
      }
      kcur += pd.K;
      const int m0 = wi.mt * BM, n0 = wi.nt * BN;
      if (tid < BM) {
        int64_t o0 = 0, o1 = 0;
        if (m0 + tid < M) mixed_offsets32(pd.rows, (uint32_t)(m0 + tid), o0, o1);
        rowA[tid] = o0; rowR[tid] = o1;
      } else {
        int c = tid - BM;
        int64_t o0 = 0, o1 = 0;
        if (n0 + c < N) mixed_offsets32(pd.cols, (uint32_t)(n0 + c), o0, o1);
        colB[c] = o0; colR[c] = o1;
      }
      const double* A = job_A(g.ptrs, pd.job) + pd.a_off;
      const double* B = job_B(g.ptrs, pd.job) + pd.b_off;
      Rp = job_R(g.ptrs, pd.job);
      r_base = pd.r_off;
      const bool a_rows_contig = pd.rows.n > 0 && pd.rows.st0[0] == 1;
      const bool b_cols_contig = pd.cols.n > 0 && pd.cols.st0[0] == 1;
      for (int k0 = klo; k0 < khi; k0 += BK) {
        __syncthreads();
        if (tid < BK) {
          int64_t o0 = 0, o1 = 0;
          if (k0 + tid < khi) mixed_offsets32(pd.ks, (uint32_t)(k0 + tid), o0, o1);
          kA[tid] = o0; kB[tid] = o1;
        }
        __syncthreads();
        // A tile (BM x BK) -> As[k][m]
#pragma unroll
        for (int e = 0; e < (BM * BK) / 128; ++e) {
          int m, k;
          if (a_rows_contig) { m = tid & 63; k = (tid >> 6) + 2 * e; }
          else { k = tid & 15; m = (tid >> 4) + 8 * e; }
          double v = 0.0;
          if (m0 + m < M && k0 + k < khi) v = __ldg(A + rowA[m] + kA[k]);
          As[k][m] = v;
        }
        // B tile (BK x BN) -> Bs[k][n]
#pragma unroll
        for (int e = 0; e < (BN * BK) / 128; ++e) {
          int n, k;
          if (b_cols_contig) { n = tid & 63; k = (tid >> 6) + 2 * e; }
          else { k = tid & 15; n = (tid >> 4) + 8 * e; }
          double v = 0.0;
          if (n0 + n < N && k0 + k < khi) v = __ldg(B + kB[k] + colB[n]);
          Bs[k][n] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 4) {
          double af[4], bf[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) af[i] = As[kk + (lane & 3)][wm + i * 8 + (lane >> 2)];
#pragma unroll
          for (int j = 0; j < 4; ++j) bf[j] = Bs[kk + (lane & 3)][wn + j * 8 + (lane >> 2)];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
        }
      }
    }
    if (wi.slot >= 0) {
      // split-K: the partial tile goes to its workspace slot; splitk_reduce applies alpha / beta
      double* wsl = g.ws + (int64_t)wi.slot * (BM * BN);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int h = 0; h < 2; ++h)
            wsl[(wn + j * 8 + 2 * (lane & 3) + h) * BM + wm + i * 8 + (lane >> 2)] = acc[i][j][h];
      continue;
    }
    // epilogue: R = alpha * acc + beta * R  (beta == 0 overwrites); the uniform choice is
    // made outside the element loops so the plain store path has no FP64 arithmetic
    const int m0 = wi.mt * BM, n0 = wi.nt * BN;
    if (g.bmode == 0 && g.amode == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int m = wm + i * 8 + (lane >> 2);
        if (m0 + m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int n = wn + j * 8 + 2 * (lane & 3) + h;
            if (n0 + n < N) Rp[r_base + rowR[m] + colR[n]] = acc[i][j][h];
          }
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int m = wm + i * 8 + (lane >> 2);
        if (m0 + m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int n = wn + j * 8 + 2 * (lane & 3) + h;
            if (n0 + n >= N) continue;
            double* dst = Rp + r_base + rowR[m] + colR[n];
            const double v = acc[i][j][h];
            *dst = g.bmode == 0 ? g.alpha * v : g.alpha * v + g.beta * *dst;
          }
      }
    }
  }
}

// Sum the split-K partial tiles of one output tile in slot order (deterministic)
// and apply R = alpha * sum + beta * R.
__global__ void __launch_bounds__(256) splitk_reduce(const PairDesc* pairs, const ReduceItem* items, const double* ws,
                                                     JobPtrs ptrs, double alpha, double beta, int amode, int bmode) {
  __shared__ int64_t rowR[BM], colR[BN];
  const ReduceItem ri = items[blockIdx.x];
  const PairDesc& pd = pairs[ri.pair];
  const int m0 = ri.mt * BM, n0 = ri.nt * BN;
  if (threadIdx.x < BM) {
    int64_t a = 0, r = 0;
    if (m0 + threadIdx.x < pd.M) mixed_offsets32(pd.rows, (uint32_t)(m0 + threadIdx.x), a, r);
    rowR[threadIdx.x] = r;
  } else if (threadIdx.x < BM + BN) {
    int64_t b = 0, r = 0;
    const int j = threadIdx.x - BM;
    if (n0 + j < pd.N) mixed_offsets32(pd.cols, (uint32_t)(n0 + j), b, r);
    colR[j] = r;
  }
  __syncthreads();
  double* R = job_R(ptrs, pd.job) + pd.r_off;
  // gridDim.y CTAs share a tile (a few tiles still fill the SMs)
  const int per = (BM * BN + (int)gridDim.y - 1) / (int)gridDim.y;
  const int e1 = min(BM * BN, ((int)blockIdx.y + 1) * per);
  for (int e = (int)blockIdx.y * per + threadIdx.x; e < e1; e += blockDim.x) {
    const int m = e % BM, n = e / BM;
    if (m0 + m >= pd.M || n0 + n >= pd.N) continue;
    double sum = 0.0;
    for (int sl = 0; sl < ri.nslots; ++sl) sum += ws[(int64_t)(ri.slot0 + sl) * (BM * BN) + e];
    double* dst = R + rowR[m] + colR[n];
    if (bmode == 0) *dst = amode ? alpha * sum : sum;
    else *dst = alpha * sum + beta * *dst;
  }
}

}  // namespace

int nd_gemm_f64_tile_elems() { return BM * BN; }

nd_status nd_launch_gemm_f64(nd_handle h, const PairDesc* d_pairs, const WorkItem* d_items, int nitems,
                             const JobPtrs& ptrs, double alpha, double beta, double* ws,
                             const ReduceItem* d_red, int nred) {
  if (nitems == 0) return ND_OK;
  GemmArgs g{d_pairs, d_items, nitems, ptrs, alpha, beta, alpha == 1.0 ? 0 : 1, beta == 0.0 ? 0 : 1, ws};
  int blocks = std::min(nitems, h->num_sms * 4);
  nd_prof_begin(h, "gemm_f64_grouped");
  gemm_f64_grouped<<<blocks, 128, 0, h->stream>>>(g);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  nd_status s = nd_cuda_check(h, cudaGetLastError(), "gemm_f64_grouped");
  if (s || nred == 0) return s;
  nd_prof_begin(h, "splitk_reduce");
  const int parts = std::max(1, std::min(16, (2 * h->num_sms + nred - 1) / nred));
  splitk_reduce<<<dim3(nred, parts), 256, 0, h->stream>>>(d_pairs, d_red, ws, ptrs, alpha, beta, g.amode, g.bmode);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "splitk_reduce");
}

// ---------------------------------------------------------------------------
// Skinny block pairs (N <= 8 and K <= 32): FP64 on the CUDA cores.
//
// Contractions with an MPO tensor (T1 * W1, T2 * W2 in the two-site H_eff)
// are tall and skinny: M is a product of bond dimensions while N and K are
// MPO-link x physical sector sizes (1..3 each).  Their arithmetic intensity
// is a few flops per 8-byte element, far below any tensor-core tile's ridge
// point, so they are HBM-bound and run here in plain FP64 (exact, no split),
// in every precision mode: one thread per output row, the B block of each
// pair staged in shared memory, the group's pairs accumulated in registers.
// ---------------------------------------------------------------------------
namespace {
constexpr int SK_THREADS = 256, SK_ROWS = 8 * SK_THREADS, SK_MAXN = 8, SK_MAXK = 32;

constexpr int SK_BATCH = 4;           // pairs staged per round

// Row index -> (A offset, R offset).  Row maps of at most two dimensions (the MPO
// contractions' blocks) whose A and output blocks hold fewer than 2^31 elements take
// one multiply-high division and four 32-bit multiply-adds with the map's parameters
// held in registers; other maps take mixed_offsets32.
struct SkRowMap {
  bool fast;
  uint32_t d0, mul0, shr0;
  int32_t a0, a1, b0, b1;
  __device__ __forceinline__ void load(const PairDesc& pd) {
    const Mixed& m = pd.rows;
    fast = m.n >= 1 && m.n <= 2 && m.mul[0] != 0u && (int64_t)pd.M * pd.K < (1ll << 31) &&
           (int64_t)pd.M * pd.N < (1ll << 31);
    d0 = (uint32_t)m.dim[0]; mul0 = m.mul[0]; shr0 = m.shr[0];
    a0 = (int32_t)m.st0[0]; b0 = (int32_t)m.st1[0];
    a1 = m.n > 1 ? (int32_t)m.st0[1] : 0; b1 = m.n > 1 ? (int32_t)m.st1[1] : 0;
  }
  __device__ __forceinline__ void offsets(const Mixed& m, uint32_t i, int64_t& ra, int64_t& rr) const {
    if (fast) {
      const uint32_t q = (__umulhi(i, mul0) + i) >> shr0;   // i / d0 (q = 0 for one-dimensional maps)
      const int32_t r = (int32_t)(i - q * d0);
      ra = r * a0 + (int32_t)q * a1;
      rr = r * b0 + (int32_t)q * b1;
    } else {
      mixed_offsets32(m, i, ra, rr);
    }
  }
};

// Shared staging area of one round: the pairs' descriptors, B blocks and k offsets.
struct SkStage {
  PairDesc pd[SK_BATCH];
  double B[SK_BATCH][SK_MAXK][SK_MAXN];
  int64_t kA[SK_BATCH][SK_MAXK];
  int64_t colR[SK_MAXN];
};

// One item = SK_ROWS rows of one group with exactly NN output columns (no predicated
// FMAs: the FP64 pipe is the bound for these pairs on GB300).  These contractions are
// bound by load latency (a few loads per output), so a thread keeps RPT rows in
// flight: 8 for NN = 1 (one pass), 4 for NN <= 3, 2 above; a pass loads KC = 8 / RPT
// operands per row at once.  The pairs of the group are staged SK_BATCH at a time (two
// barriers per round, not per pair); when they fit one round they are staged once per
// item.  MODE (uniform, resolved at compile time so the store path carries no FP64
// work): 0: R = acc, 1: R = alpha acc, 2: R = alpha acc + beta R.
template <int NN, int MODE, int RPT>
__device__ __forceinline__ void skinny_item(const GemmArgs& g, const WorkItem& wi, SkStage& sh) {
  const int tid = threadIdx.x;
  constexpr int PD_VECS = (int)(sizeof(PairDesc) / 16);
  constexpr int KC = RPT >= 8 ? 1 : 8 / RPT;
  const bool whole = wi.pair_count <= SK_BATCH;
  const int M = __ldg(&g.pairs[wi.pair_begin].M);   // every pair of the group has the output's rows
  for (int pass = 0; pass < SK_ROWS / (SK_THREADS * RPT); ++pass) {
    if (wi.mt * SK_ROWS + pass * SK_THREADS * RPT >= M) break;   // uniform: no rows left in this item
    const int i0 = wi.mt * SK_ROWS + pass * SK_THREADS * RPT + tid;
    double acc[RPT][NN];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
      for (int j = 0; j < NN; ++j) acc[r][j] = 0.0;
    for (int p0 = 0; p0 < wi.pair_count; p0 += SK_BATCH) {
      const int nb = min(SK_BATCH, wi.pair_count - p0);
      if (!whole || pass == 0) {
        __syncthreads();                          // the previous round is done with the staging area
        for (int e = tid; e < nb * PD_VECS; e += SK_THREADS)
          ((int4*)sh.pd)[e] = __ldg((const int4*)(g.pairs + wi.pair_begin + p0) + e);
        __syncthreads();
        // B blocks (k, j) and the k offsets of every staged pair, one element per thread
        for (int e = tid; e < nb * SK_MAXK * SK_MAXN; e += SK_THREADS) {
          const int q = e / (SK_MAXK * SK_MAXN), k = (e / SK_MAXN) % SK_MAXK, j = e % SK_MAXN;
          const PairDesc& pd = sh.pd[q];
          if (k < pd.K && j < NN) {
            int64_t ka, kb, cb, cr;
            mixed_offsets32(pd.ks, k, ka, kb);
            mixed_offsets32(pd.cols, j, cb, cr);
            sh.B[q][k][j] = __ldg(job_B(g.ptrs, pd.job) + pd.b_off + kb + cb);
            if (j == 0) sh.kA[q][k] = ka;
            if (q == 0 && k == 0) sh.colR[j] = cr;
          }
        }
        __syncthreads();
      }
      for (int q = 0; q < nb; ++q) {
        const PairDesc& pd = sh.pd[q];
        const int K = pd.K;
        const double* Ab = job_A(g.ptrs, pd.job) + pd.a_off;
        const double* Ar[RPT];
        bool rok[RPT];
        SkRowMap rm;
        rm.load(pd);
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
          const int i = i0 + r * SK_THREADS;
          rok[r] = i < M;
          int64_t ra = 0, rr = 0;
          if (rok[r]) rm.offsets(pd.rows, (uint32_t)i, ra, rr);
          Ar[r] = Ab + ra;
        }
        for (int k0 = 0; k0 < K; k0 += KC) {
          double av[KC][RPT];
#pragma unroll
          for (int kk = 0; kk < KC; ++kk)
#pragma unroll
            for (int r = 0; r < RPT; ++r)
              av[kk][r] = (k0 + kk < K && rok[r]) ? __ldg(Ar[r] + sh.kA[q][k0 + kk]) : 0.0;
#pragma unroll
          for (int kk = 0; kk < KC; ++kk) {
            if (k0 + kk >= K) break;
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
              for (int j = 0; j < NN; ++j) acc[r][j] = fma(av[kk][r], sh.B[q][k0 + kk][j], acc[r][j]);
          }
        }
      }
    }
    // every pair of the group writes the same output block: its row map comes from pair 0
    // of the last round (staged descriptors share the output block's row strides)
    const PairDesc& pd = sh.pd[0];
    double* Rp = job_R(g.ptrs, pd.job) + pd.r_off;
    SkRowMap rm;
    rm.load(pd);
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int i = i0 + r * SK_THREADS;
      if (i >= pd.M) continue;
      int64_t ra, rrow;
      rm.offsets(pd.rows, (uint32_t)i, ra, rrow);
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        double* dst = Rp + rrow + sh.colR[j];
        const double v = acc[r][j];
        if (MODE == 0) *dst = v;
        else if (MODE == 1) *dst = g.alpha * v;
        else *dst = g.alpha * v + g.beta * *dst;
      }
    }
  }
}

__global__ void __launch_bounds__(SK_THREADS, 4) gemm_skinny_f64(GemmArgs g) {
  __shared__ __align__(16) SkStage sh;
  static_assert(sizeof(PairDesc) % 16 == 0, "PairDesc must be a multiple of 16 bytes");
  for (int it = blockIdx.x; it < g.nitems; it += gridDim.x) {
    const WorkItem wi = g.items[it];
    const int N = __ldg(&g.pairs[wi.pair_begin].N);
    const int mode = g.bmode ? 2 : (g.amode ? 1 : 0);
#define ND_SKINNY_CASE(NN)                                               \
  case NN:                                                               \
    if (mode == 0) skinny_item<NN, 0, (NN == 1 ? 8 : NN <= 3 ? 4 : 2)>(g, wi, sh);     \
    else if (mode == 1) skinny_item<NN, 1, (NN == 1 ? 8 : NN <= 3 ? 4 : 2)>(g, wi, sh);\
    else skinny_item<NN, 2, (NN == 1 ? 8 : NN <= 3 ? 4 : 2)>(g, wi, sh);               \
    break;
    switch (N) {
      ND_SKINNY_CASE(1)
      ND_SKINNY_CASE(2)
      ND_SKINNY_CASE(3)
      ND_SKINNY_CASE(4)
      ND_SKINNY_CASE(5)
      ND_SKINNY_CASE(6)
      ND_SKINNY_CASE(7)
      default:
        if (mode == 0) skinny_item<8, 0, 2>(g, wi, sh);
        else if (mode == 1) skinny_item<8, 1, 2>(g, wi, sh);
        else skinny_item<8, 2, 2>(g, wi, sh);
        break;
    }
#undef ND_SKINNY_CASE
  }
}
}  // namespace

bool nd_pair_is_skinny(const PairDesc& p) { return p.N <= SK_MAXN && p.K <= SK_MAXK; }
int nd_skinny_rows() { return SK_ROWS; }

nd_status nd_launch_skinny_f64(nd_handle h, const PairDesc* d_pairs, const WorkItem* d_items, int nitems,
                               const JobPtrs& ptrs, double alpha, double beta) {
  if (nitems == 0) return ND_OK;
  GemmArgs g{d_pairs, d_items, nitems, ptrs, alpha, beta, alpha == 1.0 ? 0 : 1, beta == 0.0 ? 0 : 1};
  int blocks = std::min(nitems, h->num_sms * 8);
  nd_prof_begin(h, "gemm_skinny_f64");
  gemm_skinny_f64<<<blocks, SK_THREADS, 0, h->stream>>>(g);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "gemm_skinny_f64");
}
