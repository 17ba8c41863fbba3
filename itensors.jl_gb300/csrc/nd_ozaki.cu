// Split-precision grouped GEMM on the 5th-generation tensor cores (tcgen05 + TMEM).
//
// Replaces the FP64 BLAS.gemm! of _contract! (NDTensors/src/abstractarray/
// tensoralgebra/contract.jl:40-85) for the block pairs of a contraction when the
// caller asks for ND_PREC_OZAKI or ND_PREC_BF16X3.
//
// Ozaki scheme (error-free splitting, Ozaki-Ogita-Oishi-Rump 2012; integer
// slices after Ootomo et al. 2024):
//   every row i of A (over K) gets an exponent E_i with max|A_i,:| < 2^E_i and is
//   written as A_ik = 2^(E_i-7) * sum_p d_p 2^(-8(p-1)) with S balanced digits
//   d_p in [-128, 128]; B likewise per column (F_j).  Digits are integers of at
//   most 8 significant bits, so they are exact in BF16, digit products are
//   exact in FP32 (< 2^14), and a sum of up to 2^10 of them is exact too.
//   C = 2^(E_i+F_j-14) sum_{p+q<=S+1} 2^(-8(p+q-2)) (A_p B_q).
// sm_103a has no tcgen05 kind::i8, so the int8-range digits run on kind::f16
// with BF16 operands and FP32 accumulators in TMEM.
//
// GB300 has ~1/30 of B200's FP64 rate, so this file performs NO FP64
// arithmetic in its hot loops: the split reads the IEEE bits with integer
// instructions, the recombination is int64 fixed-point, and the final double
// is assembled from integer fields.  FP64 arithmetic appears only in the
// alpha/beta epilogue when alpha != 1 or beta != 0, and in the BF16X3 epilogue.
//
// Levels: level t = p+q carries weight 2^(-8(t-2)).  Slices are stored
// pre-scaled (slice p holds d_p * 2^(-8(p-1)), still exact in BF16), so every
// product already carries its level weight.  All levels accumulate in FP32 TMEM
// over chunks of 512 of K and are drained per chunk into int64 fixed point (unit
// 2^-24 of a level-2 unit): levels 2 and 3 are exact there (|sum| <= 2^24 units),
// levels 4 and >= 5 are rounded once per chunk, below 2^-40 of the leading term.
// A slot is [L2 | L3 | T4 | T5+] (64 columns each); two slots alternate per chunk
// in the 512 TMEM columns, so the drain of one chunk overlaps the MMAs of the next.
// The drains convert with FP32 magic-constant splits, not float->int
// instructions, which sm_103a runs on its narrow FP64 pipe.
//
// Each A-slice stage is [S][128 rows][32 k] BF16 and each B-slice stage is
// [S][64 rows][32 k], pre-swizzled (64-byte swizzle) by the pack kernel, so one
// cp.async.bulk per operand brings a whole stage and the slices of B sit in
// consecutive rows.  Level t sits in block t - 2 of a slot, so A_p x [B_1 .. B_r]
// is ONE tcgen05.mma with N = 64 r whose 64-column parts land in consecutive
// blocks (for S = 5: N = 256, 192, 128, 64 for p = 1..4); the few products past
// the last block go to T5+ with N = 64.  Consecutive MMAs that share A_p reuse it
// through the A collector.  9 MMAs per 16 of K for S = 5.
//
// Warp roles (576 threads): warp 0 = bulk-copy producer, warp 1 = TMEM
// allocator + MMA issuer, warps 2..17 = epilogue (TMEM lane quarter = warp % 4,
// 16-column group = (warp-2)/4).  Persistent CTAs walk a list of output tiles
// balanced across them by longest-processing-time assignment; each tile loops
// over the block pairs of its output block.
#include "nd_plan.h"
#include <cuda_bf16.h>
#include <algorithm>
#include <map>
#include <unordered_map>

namespace {

constexpr int BM = 128, BN = 64, BK = 32;
constexpr int A_SLICE = BM * BK * 2;   // 8192 bytes
constexpr int B_SLICE = BN * BK * 2;   // 4096 bytes
constexpr int CHUNK_STEPS = 16;        // 16 * 32 = 512 of K per exact chunk
constexpr int NTHREADS = 576;          // producer warp, MMA warp, 16 epilogue warps
constexpr int EPI_WARPS = 16;
constexpr int EPI_COLS = BN * 4 / EPI_WARPS;   // columns per epilogue thread (16)
constexpr int SMEM_BUDGET = 220 * 1024;

struct SplitOp {
  int64_t src_off;    // element offset of the block
  int64_t pack_off;   // byte offset of its packed slices
  int64_t exp_off;    // offset of its per-row exponents
  int32_t rows, kdim;
  int32_t row_tiles, k_steps;
  int32_t is_b, job;
  Mixed rk;           // st0: element strides of the rows
  Mixed kk;           // st0: element strides of k
};

// ---- helpers ---------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Progress waits pass the CTA's abort flag and the handle's spin limit; clean-up
// waits (copies or MMAs already issued) pass no flag and wait up to ND_SPIN_LIMIT.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, DeviceStatus* st, int site,
                                          volatile int* abort_flag, uint32_t lim = ND_SPIN_LIMIT) {
  if (!abort_flag) lim = ND_SPIN_LIMIT;
  for (uint32_t it = 0; it < lim; ++it) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    if (ok) return true;
    if ((it & 255) == 255 && abort_flag && *abort_flag) return false;
  }
  if (atomicCAS(&st->code, 0, ND_ERR_TIMEOUT) == 0) st->where = site;
  if (abort_flag) *abort_flag = 1;
  return false;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(b)) : "memory");
}

// FP64 -> FP32 with round-to-nearest-even using integer instructions only.
// Values beyond the FP32 range saturate to +-Inf / flush to zero.
__device__ __forceinline__ float f64_to_f32_int(uint64_t bits) {
  uint32_t sign = (uint32_t)(bits >> 63) << 31;
  int ex = (int)((bits >> 52) & 0x7ff);
  uint64_t m = bits & 0xfffffffffffffull;
  if (ex == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0));
  int e = ex - 1023 + 127;
  if (ex == 0 || e < -24) return __uint_as_float(sign);
  m |= (1ull << 52);
  int shift = 29;                       // 53 -> 24 bits
  if (e <= 0) { shift += 1 - e; e = 0; }
  uint64_t mant = m >> shift;
  uint64_t rem = m & ((1ull << shift) - 1), half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (mant & 1))) mant++;
  if (e == 0) return __uint_as_float(sign | (uint32_t)mant);          // denormal (carry into exponent is fine)
  if (mant >> 24) { mant >>= 1; e++; }
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((uint32_t)e << 23) | ((uint32_t)mant & 0x7fffffu));
}

// v * 2^e rounded to the nearest double, integer instructions only.
__device__ __forceinline__ double i64_scaled_to_f64(long long v, int e) {
  if (v == 0) return 0.0;
  uint64_t sign = v < 0 ? (1ull << 63) : 0ull;
  uint64_t a = v < 0 ? (uint64_t)(-(v + 1)) + 1ull : (uint64_t)v;
  int lz = __clzll((long long)a);
  uint64_t n = a << lz;                  // top bit at 63
  uint64_t mant = n >> 11, rem = n & 0x7ffull;
  int ex2 = e + 63 - lz;                 // value = n/2^63 * 2^ex2 in [2^ex2, 2^(ex2+1))
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
    mant++;
    if (mant >> 53) { mant >>= 1; ex2++; }
  }
  int be = ex2 + 1023;
  if (be >= 2047) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull));
  if (be <= 0) {
    int s = 1 - be;
    if (s > 53) return __longlong_as_double((long long)sign);
    uint64_t r = mant & ((1ull << s) - 1), hf = 1ull << (s - 1);
    uint64_t mm = mant >> s;
    if (r > hf || (r == hf && (mm & 1ull))) mm++;
    return __longlong_as_double((long long)(sign | mm));
  }
  return __longlong_as_double((long long)(sign | ((uint64_t)be << 52) | (mant & 0xfffffffffffffull)));
}

// ---- pack kernels ----------------------------------------------------------
// Two launches over fine-grained items (operand, row tile, chunk of PACK_KC
// k-steps), one CTA per item, so the block scheduler balances them over the SMs
// (4 k-steps per item measured best: 8 left a partial last wave, 2 paid more per-item
// set-up): pack_rowmax folds |x| maxima of its chunk
// into a per-row global maximum (IEEE bit patterns are monotonic for finite
// x, so an integer atomicMax suffices); pack_digits turns each element into S
// digit slices written straight to global memory in the tcgen05 canonical
// K-major SW64 layout.  A thread owns (row, 8-wide k chunk) units: the four
// lanes of a row read its 32 k values (coalesced whether rows or k are
// contiguous in the tensor) and each writes one 16-byte chunk per slice, so
// four lanes fill a 64-byte row and a warp a 512-byte run.  (One exponent per
// (row, 512-wide chunk), digitised in a single pack pass that reads its chunk
// twice, was measured too: the second, L2-resident read made pack_digits 1.5-1.8x
// slower, more than the row-maximum pass it removes.)
constexpr int PACK_KC = 4;                 // k-steps (of 32) per pack item

struct PackItem2 {
  int32_t op, rt, kc;
};

struct PackArgs2 {
  const SplitOp* ops;
  const PackItem2* items;
  int nitems;
  JobPtrs ptrs;
  unsigned char* pack;
  int32_t* exps;
  unsigned long long* rowmax;
  int slices;
  DeviceStatus* st;
};

// Digits of one element as floats d_q * 2^(-8q), q = 0 most significant.
// S > 2: X = round(x * 2^(8S-1-E)) (signed, |X| <= 2^(8S-1)) in balanced base 256.
// Adding C = 0x80 in each of the S-1 low byte positions makes every low byte y_i of
// X + C equal to d_i + 128 (the adder does the carries); the top digit is the
// arithmetic shift of X + C, so all digits lie in [-128, 128].  Integer -> float is
// the exact magic-constant addition: the bits of 1.5 * 2^(23-8q) plus d, read as a
// float, minus 1.5 * 2^(23-8q), equal d * 2^(-8q) for |d| < 2^22.
// S == 2 (3xBF16): the FP32 rounding of x split into a BF16 head and its remainder.
template <int S>
__device__ __forceinline__ void unit_digits_f(uint64_t bits, int E, float* f) {
  if constexpr (S > 2) {
    const uint32_t hi_w = (uint32_t)(bits >> 32);
    const int ex = (int)((hi_w >> 20) & 0x7ff);
    uint64_t mag = 0;
    if (ex != 0x7ff && (bits << 1) != 0) {
      const uint64_t m = (bits & 0xfffffffffffffull) | (ex ? (1ull << 52) : 0ull);
      const int sh = 1075 - (ex ? ex : 1) - (8 * S - 1) + E;   // >= 5
      if (sh < 64) mag = (m + (1ull << (sh - 1))) >> sh;
    }
    const long long X = (hi_w >> 31) ? -(long long)mag : (long long)mag;
    constexpr unsigned long long C = 0x8080808080808080ull & ((1ull << (8 * (S - 1))) - 1ull);
    const long long Y = X + (long long)C;
    const uint32_t ylo = (uint32_t)Y, yhi = (uint32_t)((unsigned long long)Y >> 32);
#pragma unroll
    for (int q = 0; q < S; ++q) {
      const int i = S - 1 - q;                                 // byte position of slice q
      int d;
      if (i == S - 1) d = (int)(Y >> (8 * i));
      else d = (int)(i < 4 ? __byte_perm(ylo, 0, 0x4440 + i) : __byte_perm(yhi, 0, 0x4440 + (i - 4))) - 128;
      const int mq = 0x4B400000 - ((8 * q) << 23);             // bits of 1.5 * 2^(23-8q)
      f[q] = __int_as_float(mq + d) - __int_as_float(mq);
    }
  } else {
    const float xf = f64_to_f32_int(bits);
    const float hd = __bfloat162float(__float2bfloat16_rn(xf));
    f[0] = hd;
    f[1] = xf - hd;
  }
}

__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// shared set-up of one pack item: row offsets and k offsets of the chunk
__device__ __forceinline__ void pack_setup(const SplitOp& op, const PackItem2& pi, int ROWS, int64_t* rowoff,
                                           int64_t* koff, int& ks0, int& ks1) {
  const int tid = threadIdx.x;
  const int r0 = pi.rt * ROWS;
  ks0 = pi.kc * PACK_KC;
  ks1 = min(op.k_steps, ks0 + PACK_KC);
  if (tid < ROWS) {
    int64_t o = 0, dummy;
    if (r0 + tid < op.rows) mixed_offsets32(op.rk, r0 + tid, o, dummy);
    rowoff[tid] = o;
  }
  for (int t = tid; t < PACK_KC * BK; t += blockDim.x) {
    const int k = ks0 * BK + t;
    int64_t o = -1, dummy;
    if (k < op.kdim && t < (ks1 - ks0) * BK) mixed_offsets32(op.kk, k, o, dummy);
    koff[t] = o;                           // -1 marks padding
  }
}

// Row maxima: only the exponent of each row's max |x| is used, so the kernel reads the
// high 32-bit word of every double.  A maximum does not care which lane reads which
// element, so lanes follow the operand's contiguous direction: along k when k is
// unit-stride (a warp takes whole rows, 32 consecutive k per load, then a shuffle
// reduction), else along the rows (a warp takes 32 rows, the item's k split over the
// warps that share them).
__global__ void __launch_bounds__(256) pack_rowmax(PackArgs2 a) {
  __shared__ int64_t rowoff[BM];
  __shared__ int64_t koff[PACK_KC * BK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int it = blockIdx.x; it < a.nitems; it += gridDim.x) {
    const PackItem2 pi = a.items[it];
    const SplitOp& op = a.ops[pi.op];
    const int ROWS = op.is_b ? BN : BM;
    const double* src = (op.is_b ? job_B(a.ptrs, op.job) : job_A(a.ptrs, op.job)) + op.src_off;
    int ks0, ks1;
    __syncthreads();
    pack_setup(op, pi, ROWS, rowoff, koff, ks0, ks1);
    __syncthreads();
    const int nrows = min(ROWS, op.rows - pi.rt * ROWS);
    const int nk = min((ks1 - ks0) * BK, op.kdim - ks0 * BK);
    unsigned long long* rmx = a.rowmax + op.exp_off + pi.rt * ROWS;
    bool bad = false;
    if (nk >= 2 && koff[1] == koff[0] + 1) {
      // four rows per pass, all their loads issued before any is used
      constexpr int RB = 4, KB = PACK_KC * BK / 32;
      for (int r0 = warp * RB; r0 < nrows; r0 += 8 * RB) {
        uint32_t hw[RB][KB];
#pragma unroll
        for (int i = 0; i < RB; ++i) {
          const int r = r0 + i;
          const unsigned int* rowp = (const unsigned int*)(src + rowoff[r < nrows ? r : 0]) + 1;   // high words
#pragma unroll
          for (int j = 0; j < KB; ++j) {
            const int k = lane + 32 * j;
            hw[i][j] = (r < nrows && k < nk) ? __ldg(rowp + 2 * koff[k]) & 0x7ff00000u : 0u;
          }
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
          uint32_t mx = 0u;
#pragma unroll
          for (int j = 0; j < KB; ++j) {
            if (hw[i][j] == 0x7ff00000u) bad = true;
            else mx = max(mx, hw[i][j]);
          }
#pragma unroll
          for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
          if (lane == 0 && mx && r0 + i < nrows) atomicMax(&rmx[r0 + i], (unsigned long long)mx << 32);
        }
      }
    } else {
      const int rgroups = ROWS / 32, kgroups = 8 / rgroups;
      const int r = lane + 32 * (warp % rgroups), kg = warp / rgroups;
      if (r < nrows) {
        const unsigned int* rowp = (const unsigned int*)(src + rowoff[r]) + 1;
        uint32_t mx = 0u;
#pragma unroll 16
        for (int k = kg; k < nk; k += kgroups) {
          const uint32_t hw = __ldg(rowp + 2 * koff[k]) & 0x7ff00000u;
          if (hw == 0x7ff00000u) bad = true;
          else mx = max(mx, hw);
        }
        if (mx) atomicMax(&rmx[r], (unsigned long long)mx << 32);
      }
    }
    if (bad && atomicCAS(&a.st->code, 0, ND_ERR_NONFINITE) == 0) a.st->where = 300;
  }
}

template <int S>
__global__ void __launch_bounds__(256) pack_digits(PackArgs2 a) {
  __shared__ int64_t rowoff[BM];
  __shared__ int64_t koff[PACK_KC * BK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, c = lane & 3;
  for (int it = blockIdx.x; it < a.nitems; it += gridDim.x) {
    const PackItem2 pi = a.items[it];
    const SplitOp& op = a.ops[pi.op];
    const int ROWS = op.is_b ? BN : BM;
    const int units = ROWS / 64;
    const double* src = (op.is_b ? job_B(a.ptrs, op.job) : job_A(a.ptrs, op.job)) + op.src_off;
    int ks0, ks1;
    __syncthreads();
    pack_setup(op, pi, ROWS, rowoff, koff, ks0, ks1);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (j >= units) continue;
      const int r = (lane >> 2) + 8 * warp + 64 * j;
      const bool rv = pi.rt * ROWS + r < op.rows;
      int E = 0;
      if (S > 2) {
        const int ex = (int)(a.rowmax[op.exp_off + pi.rt * ROWS + r] >> 52);
        E = (ex ? ex : 1) - 1022;                      // max|x| < 2^E
        if (pi.kc == 0 && c == 0) a.exps[op.exp_off + pi.rt * ROWS + r] = E;
      }
      const double* rowp = src + rowoff[r];
#pragma unroll 2
      for (int ks = ks0; ks < ks1; ++ks) {
        unsigned char* tile = a.pack + op.pack_off + ((int64_t)(pi.rt * op.k_steps + ks) * S) * (ROWS * 64);
        uint32_t w[S][4];
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          float f0[S], f1[S];
          const int64_t k0 = koff[(ks - ks0) * BK + c * 8 + e], k1 = koff[(ks - ks0) * BK + c * 8 + e + 1];
          const uint64_t b0 = (rv && k0 >= 0) ? (uint64_t)__double_as_longlong(__ldg(rowp + k0)) : 0ull;
          const uint64_t b1 = (rv && k1 >= 0) ? (uint64_t)__double_as_longlong(__ldg(rowp + k1)) : 0ull;
          unit_digits_f<S>(b0, E, f0);
          unit_digits_f<S>(b1, E, f1);
#pragma unroll
          for (int q = 0; q < S; ++q) w[q][e / 2] = bf16x2_bits(f0[q], f1[q]);
        }
        const int so = r * 64 + (((c ^ (r >> 1)) & 3) << 4);
#pragma unroll
        for (int q = 0; q < S; ++q) *(uint4*)(tile + q * ROWS * 64 + so) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
      }
    }
  }
}

// ---- grouped tcgen05 GEMM ----------------------------------------------------
struct GemmArgs {
  const PairDesc* pairs;
  const WorkItem* items;
  int nitems;
  const SplitOp* ops;
  const unsigned char* pack;
  const int32_t* exps;
  JobPtrs ptrs;
  double alpha, beta;
  int32_t amode;      // 0: alpha == 1, 1: general alpha
  int32_t bmode;      // 0: beta == 0 (overwrite), 1: general beta
  DeviceStatus* st;
  unsigned long long* cta_times;   // optional: {start, end} (%globaltimer, ns) per CTA
  long long* ws;                   // split-K: int64 fixed-point tiles, BM x BN per slot (row-major)
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  // tcgen05 shared-memory matrix descriptor: K-major, 64-byte swizzle,
  // 8-row core-matrix groups 512 bytes apart (SBO), LBO unused (1).
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

__device__ __forceinline__ uint32_t idesc(int n) {
  // kind::f16: D=F32 (bit 4), A=BF16 (bit 7), B=BF16 (bit 10), K-major A/B, N>>3 at 17, M>>4 at 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

// The MMA warp runs its loop on all 32 lanes (warp-uniform values stay in uniform
// registers); one elected lane issues each tcgen05 instruction.
// CU selects the A-collector use: 0 none, 1 fill, 2 use, 3 lastuse (consecutive MMAs
// that share A_p read it from shared memory once).
#define ND_ELECT " .reg .pred e;\n elect.sync _|e, 0xffffffff;\n @e "
template <int CU>
__device__ __forceinline__ void mma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t id, uint32_t acc) {
  if constexpr (CU == 1)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else if constexpr (CU == 2)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else if constexpr (CU == 3)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
}

// The same MMA issued by the lane whose `leader` is non-zero (elected once per warp
// instead of once per instruction).
template <int CU>
__device__ __forceinline__ void mmaL(uint32_t leader, uint32_t dt, uint64_t ad, uint64_t bd, uint32_t id, uint32_t acc) {
  if constexpr (CU == 1)
    asm volatile("{\n .reg .pred p, q;\n setp.ne.b32 p, %4, 0;\n setp.ne.b32 q, %5, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc), "r"(leader) : "memory");
  else if constexpr (CU == 2)
    asm volatile("{\n .reg .pred p, q;\n setp.ne.b32 p, %4, 0;\n setp.ne.b32 q, %5, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc), "r"(leader) : "memory");
  else if constexpr (CU == 3)
    asm volatile("{\n .reg .pred p, q;\n setp.ne.b32 p, %4, 0;\n setp.ne.b32 q, %5, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc), "r"(leader) : "memory");
  else
    asm volatile("{\n .reg .pred p, q;\n setp.ne.b32 p, %4, 0;\n setp.ne.b32 q, %5, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc), "r"(leader) : "memory");
}

// Accumulating MMA (enable-input-d true) issued by the `leader` lane: one predicate
// serves as both the issue guard and the accumulate flag.
template <int CU>
__device__ __forceinline__ void mmaA(uint32_t leader, uint32_t dt, uint64_t ad, uint64_t bd, uint32_t id) {
  if constexpr (CU == 1)
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, q;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(leader) : "memory");
  else if constexpr (CU == 2)
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, q;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(leader) : "memory");
  else if constexpr (CU == 3)
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, q;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(leader) : "memory");
  else
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                 " @q tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(leader) : "memory");
}

// One 16-wide k step of the S = 5 schedule, its nine MMAs in one asm block: the slice
// descriptors are formed from the stage's descriptors by 32-bit adds on their low words
// (the start-address field never carries: every stage lies below 2^18 bytes), and
// one predicate is both the issue guard and the accumulate flag.  A slot is
// [L2 | L3 | T4 | T5+] (columns X, X+64, X+128, X+192):
//   A1 x [B1..B4] N=256 -> X (starts the chunk when accx == 0), A1 x B5 -> T5+,
//   A2 x [B1..B3] N=192 -> X+64, A2 x B4 -> T5+, A3 x [B1 B2] N=128 -> X+128,
//   A3 x B3 -> T5+, A4 x B1 -> T5+, A4 x B2 -> T5+, A5 x B1 -> T5+,
// consecutive MMAs of one A slice reading it once through the A collector.
__device__ __forceinline__ void mma_s5_k16(uint32_t leader, uint32_t accx, uint32_t X, uint32_t alo, uint32_t ahi,
                                           uint32_t blo, uint32_t bhi, uint32_t i256, uint32_t i192,
                                           uint32_t i128, uint32_t i64) {
  asm volatile(
      "{\n"
      " .reg .pred q, p;\n"
      " .reg .b32 t<10>, d<3>;\n"
      " .reg .b64 a<5>, b<5>;\n"
      " setp.ne.b32 q, %0, 0;\n"
      " setp.ne.b32 p, %1, 0;\n"
      " add.u32 t1, %3, 512;\n add.u32 t2, %3, 1024;\n add.u32 t3, %3, 1536;\n add.u32 t4, %3, 2048;\n"
      " add.u32 t6, %5, 256;\n add.u32 t7, %5, 512;\n add.u32 t8, %5, 768;\n add.u32 t9, %5, 1024;\n"
      " mov.b64 a0, {%3, %4};\n mov.b64 a1, {t1, %4};\n mov.b64 a2, {t2, %4};\n"
      " mov.b64 a3, {t3, %4};\n mov.b64 a4, {t4, %4};\n"
      " mov.b64 b0, {%5, %6};\n mov.b64 b1, {t6, %6};\n mov.b64 b2, {t7, %6};\n"
      " mov.b64 b3, {t8, %6};\n mov.b64 b4, {t9, %6};\n"
      " add.u32 d0, %2, 64;\n add.u32 d1, %2, 128;\n add.u32 d2, %2, 192;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%2], a0, b0, %7, p;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [d2], a0, b4, %10, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [d0], a1, b0, %8, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [d2], a1, b3, %10, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [d1], a2, b0, %9, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [d2], a2, b2, %10, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [d2], a3, b0, %10, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [d2], a3, b1, %10, q;\n"
      " @q tcgen05.mma.cta_group::1.kind::f16 [d2], a4, b0, %10, q;\n"
      "}\n"
      :: "r"(leader), "r"(accx), "r"(X), "r"(alo), "r"(ahi), "r"(blo), "r"(bhi), "r"(i256), "r"(i192),
         "r"(i128), "r"(i64)
      : "memory");
}

__device__ __forceinline__ void commitL(uint32_t leader, uint64_t* bar) {
  asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %1, 0;\n"
               " @q tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}"
               :: "r"(smem_u32(bar)), "r"(leader) : "memory");
}

#define TMEM_LD8(taddr, r)                                                                                    \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"                           \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])  \
               : "r"(taddr))

#define TMEM_LD32(taddr, r)                                                                                   \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15," \
               "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                      \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),          \
                 "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),       \
                 "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),    \
                 "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),    \
                 "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])                                            \
               : "r"(taddr))

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, %0;" :: "r"(EPI_WARPS * 32) : "memory"); }

// Round-to-nearest-even of v (|v| < 2^33) to an integer on the FP32 and integer
// pipes (sm_103a runs float->int conversions on its narrow FP64 pipe).  Magic-
// constant splitting: v + 1.5*2^35 rounds v to a multiple of 2^12 whose count sits
// in the low mantissa bits (hi); h = that multiple is exact, lo = v - h is exact
// with |lo| <= 2^11, and lo + 1.5*2^23 rounds lo to an integer the same way (li).
// v rounds to hi * 2^12 + li; ties go to even because h is even.
__device__ __forceinline__ void f32_round_split(float v, int& hi, int& li) {
  const float C12 = 51539607552.0f;   // 1.5 * 2^35, bits 0x51400000
  const float C0 = 12582912.0f;       // 1.5 * 2^23, bits 0x4B400000
  const float t = __fadd_rn(v, C12);
  const float h = __fsub_rn(t, C12);
  const float tl = __fadd_rn(__fsub_rn(v, h), C0);
  hi = __float_as_int(t) - 0x51400000;
  li = __float_as_int(tl) - 0x4B400000;
}

// One vote per wait: every lane of the MMA warp polls, and the warp leaves the loop
// together if any lane gave up.
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity, DeviceStatus* st, int site,
                                               volatile int* abort_flag, uint32_t lim) {
  return __all_sync(0xffffffffu, mbar_wait(bar, parity, st, site, abort_flag, lim));
}

template <int S>
struct Cfg {
  static constexpr int STAGE = S * (A_SLICE + B_SLICE);
  static constexpr int STAGES = (SMEM_BUDGET - 1024) / STAGE;
  static constexpr int TBLK = S >= 4 ? 2 : (S == 3 ? 1 : 0);   // tail blocks (T4, T5+)
  static constexpr int TMEM_COLS = 512;                        // two slots of [L2 L3 T4 T5+]
  static constexpr int SMEM = STAGES * STAGE + 1024;
};

// TMEM column of slot x (levels 2, 3) and of its tail blocks (levels 4, >= 5)
__device__ __forceinline__ uint32_t xcol(uint32_t x) { return x * 256u; }
__device__ __forceinline__ uint32_t tcol(uint32_t x) { return x * 256u + 128u; }

template <int S>
__global__ void __launch_bounds__(NTHREADS, 1) split_gemm(GemmArgs g) {
  using C = Cfg<S>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[C::STAGES], empty[C::STAGES];
  __shared__ __align__(8) uint64_t xfull[2], xempty[2], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int64_t colR_s[BN];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t lim = nd_spin_limit(g.st);
  if (g.cta_times && threadIdx.x == 0) g.cta_times[2 * blockIdx.x] = global_ns();

  if (tid == 0) {
    for (int s = 0; s < C::STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&xfull[b], 1); mbar_init(&xempty[b], EPI_WARPS); }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(&tmem_slot)), "r"(C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ------------------------------- producer ------------------------------
    if (lane == 0) {
      uint32_t n = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < g.nitems && ok; it += gridDim.x) {
        const WorkItem wi = g.items[it];
        for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
          const PairDesc& pd = g.pairs[wi.pair_begin + pi];
          const SplitOp& oa = g.ops[pd.a_op];
          const SplitOp& ob = g.ops[pd.b_op];
          const unsigned char* srcA = g.pack + oa.pack_off + (int64_t)wi.mt * oa.k_steps * S * A_SLICE;
          const unsigned char* srcB = g.pack + ob.pack_off + (int64_t)wi.nt * ob.k_steps * S * B_SLICE;
          const int k0 = wi.slot >= 0 ? wi.kbeg : 0, k1 = wi.slot >= 0 ? wi.kend : oa.k_steps;
          for (int ks = k0; ks < k1; ++ks, ++n) {
            const uint32_t s = n % C::STAGES, u = n / C::STAGES;
            if (u >= 1 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1, g.st, 400, &abort_flag, lim)) { ok = false; break; }
            unsigned char* dA = smem + s * C::STAGE;
            unsigned char* dB = dA + S * A_SLICE;
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(fb), "r"(C::STAGE) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_u32(dA)), "l"(srcA + (int64_t)ks * S * A_SLICE), "r"(S * A_SLICE), "r"(fb) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_u32(dB)), "l"(srcB + (int64_t)ks * S * B_SLICE), "r"(S * B_SLICE), "r"(fb) : "memory");
          }
        }
      }
      if (!ok) {
        // let copies already issued land before the CTA can exit
        for (uint32_t q = 0; q < C::STAGES && q < n; ++q) {
          uint32_t m = n - 1 - q;
          mbar_wait(smem_u32(&full[m % C::STAGES]), (m / C::STAGES) & 1, g.st, 401, nullptr);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------- MMA issuer ----------------------------
    {
      uint32_t n = 0, chunk = 0;
      bool ok = true;
      const uint32_t smem_base = smem_u32(smem);
      const uint32_t i64 = idesc(BN);
      constexpr int NBLK = 2 + C::TBLK;     // accumulator blocks of a slot: L2 L3 [T4 [T5+]]
      uint32_t leader;
      asm volatile("{\n .reg .pred e;\n elect.sync _|e, 0xffffffff;\n selp.u32 %0, 1, 0, e;\n}" : "=r"(leader));
      for (int it = blockIdx.x; it < g.nitems && ok; it += gridDim.x) {
        const WorkItem wi = g.items[it];
        for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
          const PairDesc& pd = g.pairs[wi.pair_begin + pi];
          // k steps of this item: the pair's whole K, or a split-K range [kbeg, kend)
          const int nks = wi.slot >= 0 ? wi.kend - wi.kbeg : g.ops[pd.a_op].k_steps;
          const int chunk_steps = S > 2 ? CHUNK_STEPS : nks;
          uint32_t X = tmem;
          for (int ks = 0; ks < nks; ++ks, ++n) {
            const bool cstart = (ks % chunk_steps) == 0;
            const bool cend = ((ks % chunk_steps) == chunk_steps - 1) || ks == nks - 1;
            if (cstart) {
              // every level is drained per chunk: slot xs holds all levels of this chunk
              const uint32_t xs = chunk & 1, xu = chunk >> 1;
              if (xu >= 1 && !mbar_wait_warp(smem_u32(&xempty[xs]), (xu - 1) & 1, g.st, 411, &abort_flag, lim)) { ok = false; break; }
              X = tmem + xcol(xs);
            }
            const uint32_t s = n % C::STAGES, u = n / C::STAGES;
            if (!mbar_wait_warp(smem_u32(&full[s]), u & 1, g.st, 412, &abort_flag, lim)) { ok = false; break; }
            fence_after();
            // descriptors of one stage differ only in the start-address field (addr >> 4)
            const uint32_t a0 = smem_base + s * C::STAGE;
            const uint64_t adesc0 = sdesc(a0), bdesc0 = sdesc(a0 + S * A_SLICE);
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
              const uint32_t accx = (cstart && kk == 0) ? 0u : 1u;
              const uint32_t ko = kk * 32;
              if constexpr (S == 5 && NBLK == 4) {
                mma_s5_k16(leader, accx, X, (uint32_t)adesc0 + (ko >> 4), (uint32_t)(adesc0 >> 32),
                           (uint32_t)bdesc0 + (ko >> 4), (uint32_t)(bdesc0 >> 32), idesc(4 * BN), idesc(3 * BN),
                           idesc(2 * BN), i64);
                continue;
              }
              auto A = [&](int p) { return adesc0 + (uint64_t)((((p - 1) * A_SLICE) + ko) >> 4); };
              auto B = [&](int q) { return bdesc0 + (uint64_t)((((q - 1) * B_SLICE) + ko) >> 4); };
              // A slot is [L2 | L3 | T4 | T5+], 64 columns each, and level t = p + q sits in
              // block t - 2.  A_p x [B_1 .. B_r] therefore lands in consecutive blocks: ONE
              // MMA of N = 64 r at column 64 (p - 1).  The remaining products of A_p (levels
              // past the last block) accumulate into T5+.  The first MMA of a chunk covers
              // every block, so it alone starts the accumulation.
#pragma unroll
              for (int p = 1; p <= S; ++p) {
                const int r = (S + 1 - p) < (NBLK + 1 - p) ? (S + 1 - p) : (NBLK + 1 - p);
                const int r0 = r > 0 ? r : 0;
                const int nm = (r0 > 0 ? 1 : 0) + (S + 1 - p - r0);    // MMAs sharing A_p
                int m = 0;
                if (r0 > 0) {
                  const uint32_t d = X + (p - 1) * BN, id = idesc(r0 * BN);
                  if (p == 1) {          // the chunk's first MMA may start the accumulation
                    if (nm > 1) mmaL<1>(leader, d, A(p), B(1), id, accx);
                    else mmaL<0>(leader, d, A(p), B(1), id, accx);
                  } else {
                    if (nm > 1) mmaA<1>(leader, d, A(p), B(1), id);
                    else mmaA<0>(leader, d, A(p), B(1), id);
                  }
                  ++m;
                }
#pragma unroll
                for (int q = r0 + 1; q <= S + 1 - p; ++q, ++m) {
                  const uint32_t d = X + (NBLK - 1) * BN;
                  if (nm == 1) mmaA<0>(leader, d, A(p), B(q), i64);
                  else if (m == 0) mmaA<1>(leader, d, A(p), B(q), i64);
                  else if (m == nm - 1) mmaA<3>(leader, d, A(p), B(q), i64);
                  else mmaA<2>(leader, d, A(p), B(q), i64);
                }
              }
            }
            commitL(leader, &empty[s]);
            if (cend) { commitL(leader, &xfull[chunk & 1]); ++chunk; }
          }
          if (!ok) break;
        }
      }
      commitL(leader, &done_bar);
      mbar_wait(smem_u32(&done_bar), 0, g.st, 413, nullptr);
    }
  } else {
    // ------------------------------- epilogue ------------------------------
    const int q = warp & 3;                 // TMEM lane quarter
    const int cg = (warp - 2) >> 2;         // 16-column group
    const int row = q * 32 + lane;
    const int etid = tid - 64;
    const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + cg * EPI_COLS;
    uint32_t chunk = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < g.nitems && ok; it += gridDim.x) {
      const WorkItem wi = g.items[it];
      const PairDesc& p0 = g.pairs[wi.pair_begin];
      const int gm = wi.mt * BM + row;
      const bool row_ok = gm < p0.M;
      int64_t roff = 0, dummy;
      if (row_ok) mixed_offsets32(p0.rows, (uint32_t)gm, dummy, roff);
      epi_sync();                                   // previous item done with colR_s
      if (etid < BN) {
        int64_t co = 0, d2;
        const int gn = wi.nt * BN + etid;
        if (gn < p0.N) mixed_offsets32(p0.cols, (uint32_t)gn, d2, co);
        colR_s[etid] = co;
      }
      epi_sync();
      double* Rb = job_R(g.ptrs, p0.job) + p0.r_off + roff;
      const int ncols = min(EPI_COLS, p0.N - (wi.nt * BN + cg * EPI_COLS));
      for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
        const PairDesc& pd = g.pairs[wi.pair_begin + pi];
        const SplitOp& oa = g.ops[pd.a_op];
        const SplitOp& ob = g.ops[pd.b_op];
        const int nks = wi.slot >= 0 ? wi.kend - wi.kbeg : oa.k_steps;
        const int chunk_steps = S > 2 ? CHUNK_STEPS : nks;
        const int nchunks = (nks + chunk_steps - 1) / chunk_steps;
        long long acc[EPI_COLS];
        float facc[EPI_COLS];
#pragma unroll
        for (int c = 0; c < EPI_COLS; ++c) { acc[c] = 0; facc[c] = 0.f; }
        for (int ch = 0; ch < nchunks; ++ch, ++chunk) {
          const uint32_t xs = chunk & 1, xu = chunk >> 1;
          if (!mbar_wait(smem_u32(&xfull[xs]), xu & 1, g.st, 420, &abort_flag, lim)) { ok = false; break; }
          fence_after();
          // 8 columns at a time: L2 and L3 (exact) then the FP32 tail levels T4 and T5+
#pragma unroll
          for (int hb = 0; hb < EPI_COLS; hb += 8) {
            uint32_t l2[8], l3[8];
            TMEM_LD8(lane_addr + xcol(xs) + hb, l2);
            TMEM_LD8(lane_addr + xcol(xs) + BN + hb, l3);
            tmem_wait_ld();
            if (S > 2) {
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                // L2: integer units; L3 was computed with pre-scaled slices: an integer multiple of 2^-8
                // |L2| <= 2^23, |256 L3| <= 2^24: hi parts fit 2^11 and 2^12, li parts 2^11
                int h2, i2, h3, i3;
                f32_round_split(__uint_as_float(l2[c]), h2, i2);
                f32_round_split(__uint_as_float(l3[c]) * 256.0f, h3, i3);
                acc[hb + c] += ((long long)(h2 * 256 + h3) << 28) + ((long long)(i2 * 256 + i3) << 16);
              }
            } else {
#pragma unroll
              for (int c = 0; c < 8; ++c) facc[hb + c] += __uint_as_float(l2[c]) + __uint_as_float(l3[c]);
            }
            if (C::TBLK) {
              // levels >= 4 of this chunk (FP32, rounded once per chunk into the fixed point)
              uint32_t t4[8], t5[8];
              TMEM_LD8(lane_addr + tcol(xs) + hb, t4);
              if (C::TBLK > 1) TMEM_LD8(lane_addr + tcol(xs) + BN + hb, t5);
              tmem_wait_ld();
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                // x 2^24: |T4| < 2^9 and |T5+| < 2^2 per chunk, inside the split's 2^33 range
                int h4, i4, h5 = 0, i5 = 0;
                f32_round_split(__uint_as_float(t4[c]) * 16777216.0f, h4, i4);
                if (C::TBLK > 1) f32_round_split(__uint_as_float(t5[c]) * 16777216.0f, h5, i5);
                acc[hb + c] += ((long long)(h4 + h5) << 12) + (long long)(i4 + i5);
              }
            }
          }
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&xempty[xs]);
        }
        if (!ok) break;
        if (wi.slot >= 0) {
          // split-K: this K range's exact fixed-point tile, added to the others by split_reduce
          long long* wsl = g.ws + (int64_t)wi.slot * (BM * BN) + (int64_t)row * BN + cg * EPI_COLS;
#pragma unroll
          for (int c = 0; c < EPI_COLS; ++c) wsl[c] = acc[c];
          continue;
        }
        // finalize this pair into R
        if (row_ok && ncols > 0) {
          const int Ei = S > 2 ? g.exps[oa.exp_off + gm] : 0;
          const int32_t* Fj = g.exps + ob.exp_off + wi.nt * BN + cg * EPI_COLS;
          const bool first = pd.first != 0;
          // the uniform store choice is made outside the column loop: the common overwrite
          // (first pair, alpha = 1, beta = 0) carries no FP64 arithmetic
          if (first && g.bmode == 0 && g.amode == 0) {
#pragma unroll
            for (int c = 0; c < EPI_COLS; ++c)
              if (c < ncols)
                Rb[colR_s[cg * EPI_COLS + c]] =
                    (S > 2) ? i64_scaled_to_f64(acc[c], Ei + __ldg(Fj + c) - 38) : (double)facc[c];
          } else {
#pragma unroll
            for (int c = 0; c < EPI_COLS; ++c) {
              if (c < ncols) {
                double v = (S > 2) ? i64_scaled_to_f64(acc[c], Ei + __ldg(Fj + c) - 38) : (double)facc[c];
                double* dst = Rb + colR_s[cg * EPI_COLS + c];
                if (first) *dst = g.bmode == 0 ? g.alpha * v : g.alpha * v + g.beta * *dst;
                else *dst = g.amode ? *dst + g.alpha * v : *dst + v;
              }
            }
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(C::TMEM_COLS));
  if (g.cta_times && tid == 0) g.cta_times[2 * blockIdx.x + 1] = global_ns();
}

// Split-K reduction: the K ranges of one output tile were computed by different CTAs as
// exact int64 fixed-point tiles (split_gemm, `ws`).  They begin at the same 512-K chunk
// boundaries the unsplit kernel drains at, so their integer sum is the unsplit kernel's
// accumulator bit for bit; it is converted with the pair's row and column exponents and
// stored with the pair's alpha / beta (split tiles belong to single-pair output blocks).
__global__ void __launch_bounds__(256) split_reduce(const PairDesc* pairs, const ReduceItem* red, int nred,
                                                    const SplitOp* ops, const int32_t* exps, const long long* ws,
                                                    JobPtrs ptrs, double alpha, double beta, int amode, int bmode) {
  __shared__ int64_t colR[BN];
  for (int r = blockIdx.x; r < nred; r += gridDim.x) {
    const ReduceItem ri = red[r];
    const PairDesc& pd = pairs[ri.pair];
    const SplitOp& oa = ops[pd.a_op];
    const SplitOp& ob = ops[pd.b_op];
    __syncthreads();
    if (threadIdx.x < BN) {
      const int gn = ri.nt * BN + threadIdx.x;
      int64_t co = 0, d;
      if (gn < pd.N) mixed_offsets32(pd.cols, (uint32_t)gn, d, co);
      colR[threadIdx.x] = co;
    }
    __syncthreads();
    double* Rb = job_R(ptrs, pd.job) + pd.r_off;
    const int per = (BM * BN + (int)gridDim.y - 1) / (int)gridDim.y;   // gridDim.y CTAs share a tile
    const int e1 = min(BM * BN, ((int)blockIdx.y + 1) * per);
    for (int e = (int)blockIdx.y * per + threadIdx.x; e < e1; e += blockDim.x) {
      const int row = e / BN, col = e - row * BN;
      const int gm = ri.mt * BM + row, gn = ri.nt * BN + col;
      if (gm >= pd.M || gn >= pd.N) continue;
      long long s = 0;
      for (int q = 0; q < ri.nslots; ++q) s += ws[(int64_t)(ri.slot0 + q) * (BM * BN) + e];
      const double v = i64_scaled_to_f64(s, exps[oa.exp_off + gm] + exps[ob.exp_off + gn] - 38);
      int64_t ro, d;
      mixed_offsets32(pd.rows, (uint32_t)gm, d, ro);
      double* dst = Rb + ro + colR[col];
      if (pd.first) *dst = bmode == 0 ? (amode ? alpha * v : v) : alpha * v + beta * *dst;
      else *dst = amode ? *dst + alpha * v : *dst + v;
    }
  }
}

template <int S>
nd_status launch_gemm(nd_handle h, const GemmArgs& g) {
  using C = Cfg<S>;
  static NdOnce attr;
  cudaError_t e = nd_once(attr, h->device, [] {
    return cudaFuncSetAttribute(split_gemm<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  });
  if (e != cudaSuccess) return nd_cuda_check(h, e, "split_gemm smem attribute");
  int blocks = std::min(g.nitems, h->num_sms);
  GemmArgs gt = g;
  gt.cta_times = nd_cta_slot(h, blocks);
  nd_prof_begin(h, "split_gemm");
  split_gemm<S><<<blocks, NTHREADS, C::SMEM, h->stream>>>(gt);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "split_gemm");
}

// ---- 2-CTA variant (tcgen05.mma.cta_group::2, M = 256) -----------------------
// A CTA pair (a cluster of 2) computes a 256 x 64 output tile.  CTA c stages the 128 rows
// of A of row tile 2 m + c and one half (32 rows) of every B slice; one tcgen05.mma of
// M = 256 reads A from each CTA's own shared memory and the two B halves from both, so
// each SM reads half the B bytes the 1-CTA kernel reads per product and a stage is
// S x 10 KB (4 stages for S = 5 instead of 3).  The products run as separate N = 64 MMAs
// (15 per 16 of K for S = 5; the two B halves break the 1-CTA kernel's concatenation of
// B slices), consecutive ones sharing A_p through the A collector.  The even CTA issues
// the MMAs; the odd CTA's MMA warp relays each landed stage to the even CTA (a
// cluster-scope mbarrier arrive).  Completion of a stage's MMAs and of a chunk's
// accumulation is multicast to both CTAs.  Accumulators are per CTA (its 128 rows of the
// pair tile in its own TMEM), so the chunk drains and the epilogue are the 1-CTA kernel's;
// the odd CTA's epilogue warps release a slot with remote arrivals on the even CTA.
constexpr int B_HALF = B_SLICE / 2;   // 32 rows x 32 k, 2048 bytes

template <int S>
struct Cfg2 {
  static constexpr int STAGE = S * (A_SLICE + B_HALF);
  static constexpr int STAGES = (SMEM_BUDGET - 1024) / STAGE;
  static constexpr int TBLK = Cfg<S>::TBLK;
  static constexpr int TMEM_COLS = 512;
  static constexpr int SMEM = STAGES * STAGE + 1024;
};

__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
  uint32_t o;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(o) : "r"(smem_u32(p)), "r"(rank));
  return o;
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" :: "r"(addr) : "memory");
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// mbarrier wait with cluster-scope acquire: the arrivals come from the other CTA
__device__ __forceinline__ bool mbar_wait_cl(uint32_t bar, uint32_t parity, DeviceStatus* st, int site,
                                             volatile int* abort_flag, uint32_t lim) {
  if (!abort_flag) lim = ND_SPIN_LIMIT;
  for (uint32_t it = 0; it < lim; ++it) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    if (ok) return true;
    if ((it & 255) == 255 && abort_flag && *abort_flag) return false;
  }
  if (atomicCAS(&st->code, 0, ND_ERR_TIMEOUT) == 0) st->where = site;
  if (abort_flag) *abort_flag = 1;
  return false;
}

template <int CU>
__device__ __forceinline__ void mma2(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t id, uint32_t acc) {
  if constexpr (CU == 1)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::2.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else if constexpr (CU == 2)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::2.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else if constexpr (CU == 3)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::2.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
  else
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n" ND_ELECT
                 "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(id), "r"(acc) : "memory");
}

// arrive on the mbarrier at this offset in both CTAs once the issued MMAs complete
__device__ __forceinline__ void commit2_both(uint64_t* bar) {
  asm volatile("{\n" ND_ELECT "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;\n}"
               :: "r"(smem_u32(bar)), "h"((unsigned short)3) : "memory");
}
__device__ __forceinline__ void commit2_local(uint64_t* bar) {
  asm volatile("{\n" ND_ELECT "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}"
               :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint32_t idesc2(int n) {
  // as idesc, with M = 256 (the CTA pair)
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
}

template <int S>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NTHREADS, 1) split_gemm2(GemmArgs g) {
  using C = Cfg2<S>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[C::STAGES], empty[C::STAGES], pfull[C::STAGES];
  __shared__ __align__(8) uint64_t xfull[2], xempty[2], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int64_t colR_s[BN];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t lim = nd_spin_limit(g.st);
  if (g.cta_times && threadIdx.x == 0) g.cta_times[2 * blockIdx.x] = global_ns();
  const uint32_t crank = cluster_ctarank();            // 0 issues the MMAs, 1 relays
  const int pair_id = blockIdx.x >> 1, npairs = gridDim.x >> 1;

  if (tid == 0) {
    for (int s = 0; s < C::STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); mbar_init(&pfull[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&xfull[b], 1); mbar_init(&xempty[b], 2 * EPI_WARPS); }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(&tmem_slot)), "r"(C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  cluster_sync_all();                                   // both CTAs' barriers exist before any remote arrive
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ------------------------------- producer (both CTAs) --------------------
    if (lane == 0) {
      uint32_t n = 0;
      bool ok = true;
      for (int it = pair_id; it < g.nitems && ok; it += npairs) {
        const WorkItem wi = g.items[it];
        const int mt = 2 * wi.mt + (int)crank;
        for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
          const PairDesc& pd = g.pairs[wi.pair_begin + pi];
          const SplitOp& oa = g.ops[pd.a_op];
          const SplitOp& ob = g.ops[pd.b_op];
          const unsigned char* srcA = g.pack + oa.pack_off + (int64_t)mt * oa.k_steps * S * A_SLICE;
          const unsigned char* srcB = g.pack + ob.pack_off + (int64_t)wi.nt * ob.k_steps * S * B_SLICE + crank * B_HALF;
          for (int ks = 0; ks < oa.k_steps; ++ks, ++n) {
            const uint32_t s = n % C::STAGES, u = n / C::STAGES;
            if (u >= 1 && !mbar_wait_cl(smem_u32(&empty[s]), (u - 1) & 1, g.st, 430, &abort_flag, lim)) { ok = false; break; }
            unsigned char* dA = smem + s * C::STAGE;
            unsigned char* dB = dA + S * A_SLICE;
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(fb), "r"(C::STAGE) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_u32(dA)), "l"(srcA + (int64_t)ks * S * A_SLICE), "r"(S * A_SLICE), "r"(fb) : "memory");
            const unsigned char* sb = srcB + (int64_t)ks * S * B_SLICE;
#pragma unroll
            for (int q = 0; q < S; ++q)
              asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                           :: "r"(smem_u32(dB + q * B_HALF)), "l"(sb + q * B_SLICE), "r"(B_HALF), "r"(fb) : "memory");
          }
        }
      }
      if (ok) {
        // tail: every multicast release of this CTA's stages has landed before it can exit
        for (uint32_t q = 0; q < C::STAGES && q < n; ++q) {
          const uint32_t m = n - 1 - q;
          mbar_wait_cl(smem_u32(&empty[m % C::STAGES]), (m / C::STAGES) & 1, g.st, 431, nullptr, lim);
        }
      } else {
        // let copies already issued land before the CTA can exit
        for (uint32_t q = 0; q < C::STAGES && q < n; ++q) {
          const uint32_t m = n - 1 - q;
          mbar_wait(smem_u32(&full[m % C::STAGES]), (m / C::STAGES) & 1, g.st, 432, nullptr);
        }
      }
    }
  } else if (warp == 1) {
    if (crank == 0) {
      // ----------------------------- MMA issuer (even CTA) --------------------
      uint32_t n = 0, chunk = 0;
      bool ok = true;
      const uint32_t smem_base = smem_u32(smem);
      const uint32_t i64 = idesc2(BN);
      constexpr int NBLK = 2 + C::TBLK;
      for (int it = pair_id; it < g.nitems && ok; it += npairs) {
        const WorkItem wi = g.items[it];
        for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
          const PairDesc& pd = g.pairs[wi.pair_begin + pi];
          const int nks = g.ops[pd.a_op].k_steps;
          const int chunk_steps = S > 2 ? CHUNK_STEPS : nks;
          uint32_t X = tmem;
          for (int ks = 0; ks < nks; ++ks, ++n) {
            const bool cstart = (ks % chunk_steps) == 0;
            const bool cend = ((ks % chunk_steps) == chunk_steps - 1) || ks == nks - 1;
            if (cstart) {
              const uint32_t xs = chunk & 1, xu = chunk >> 1;
              if (xu >= 1 && !__all_sync(0xffffffffu, mbar_wait_cl(smem_u32(&xempty[xs]), (xu - 1) & 1, g.st, 441, &abort_flag, lim))) { ok = false; break; }
              X = tmem + xcol(xs);
            }
            const uint32_t s = n % C::STAGES, u = n / C::STAGES;
            if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(&full[s]), u & 1, g.st, 442, &abort_flag, lim))) { ok = false; break; }
            if (!__all_sync(0xffffffffu, mbar_wait_cl(smem_u32(&pfull[s]), u & 1, g.st, 443, &abort_flag, lim))) { ok = false; break; }
            fence_after();
            const uint32_t a0 = smem_base + s * C::STAGE;
            const uint64_t adesc0 = sdesc(a0), bdesc0 = sdesc(a0 + S * A_SLICE);
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
              const uint32_t ko = kk * 32;
              auto A = [&](int p) { return adesc0 + (uint64_t)((((p - 1) * A_SLICE) + ko) >> 4); };
              auto B = [&](int q) { return bdesc0 + (uint64_t)((((q - 1) * B_HALF) + ko) >> 4); };
              // product (p, q) accumulates into level block min(p + q - 2, NBLK - 1); the
              // p = 1 products are the first writes of every block of a chunk
#pragma unroll
              for (int p = 1; p <= S; ++p) {
                const int nm = S + 1 - p;                     // MMAs sharing A_p
#pragma unroll
                for (int q = 1; q <= S + 1 - p; ++q) {
                  const int blk = (p + q - 2) < (NBLK - 1) ? (p + q - 2) : (NBLK - 1);
                  const uint32_t d = X + blk * BN;
                  const uint32_t ac = (cstart && kk == 0 && p == 1 && q <= NBLK) ? 0u : 1u;
                  if (nm == 1) mma2<0>(d, A(p), B(q), i64, ac);
                  else if (q == 1) mma2<1>(d, A(p), B(q), i64, ac);
                  else if (q == nm) mma2<3>(d, A(p), B(q), i64, ac);
                  else mma2<2>(d, A(p), B(q), i64, ac);
                }
              }
            }
            commit2_both(&empty[s]);
            if (cend) { commit2_both(&xfull[chunk & 1]); ++chunk; }
          }
          if (!ok) break;
        }
      }
      commit2_local(&done_bar);
      mbar_wait(smem_u32(&done_bar), 0, g.st, 444, nullptr);
    } else {
      // ----------------------------- stage relay (odd CTA) --------------------
      if (lane == 0) {
        uint32_t n = 0;
        bool ok = true;
        const uint32_t leader_pfull0 = cluster_addr(&pfull[0], 0);
        for (int it = pair_id; it < g.nitems && ok; it += npairs) {
          const WorkItem wi = g.items[it];
          for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
            const int nks = g.ops[g.pairs[wi.pair_begin + pi].a_op].k_steps;
            for (int ks = 0; ks < nks; ++ks, ++n) {
              const uint32_t s = n % C::STAGES, u = n / C::STAGES;
              if (!mbar_wait(smem_u32(&full[s]), u & 1, g.st, 445, &abort_flag, lim)) { ok = false; break; }
              mbar_arrive_cluster(leader_pfull0 + s * 8u);
            }
          }
        }
      }
    }
  } else {
    // ------------------------------- epilogue (both CTAs) --------------------
    const int q = warp & 3;
    const int cg = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const int etid = tid - 64;
    const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + cg * EPI_COLS;
    const uint32_t leader_xempty0 = cluster_addr(&xempty[0], 0);
    uint32_t chunk = 0;
    bool ok = true;
    for (int it = pair_id; it < g.nitems && ok; it += npairs) {
      const WorkItem wi = g.items[it];
      if (wi.pair_count == 0) continue;
      const PairDesc& p0 = g.pairs[wi.pair_begin];
      const int gm = (2 * wi.mt + (int)crank) * BM + row;
      const bool row_ok = gm < p0.M;
      int64_t roff = 0, dummy;
      if (row_ok) mixed_offsets32(p0.rows, (uint32_t)gm, dummy, roff);
      epi_sync();
      if (etid < BN) {
        int64_t co = 0, d2;
        const int gn = wi.nt * BN + etid;
        if (gn < p0.N) mixed_offsets32(p0.cols, (uint32_t)gn, d2, co);
        colR_s[etid] = co;
      }
      epi_sync();
      double* Rb = job_R(g.ptrs, p0.job) + p0.r_off + roff;
      const int ncols = min(EPI_COLS, p0.N - (wi.nt * BN + cg * EPI_COLS));
      for (int pi = 0; pi < wi.pair_count && ok; ++pi) {
        const PairDesc& pd = g.pairs[wi.pair_begin + pi];
        const SplitOp& oa = g.ops[pd.a_op];
        const SplitOp& ob = g.ops[pd.b_op];
        const int nks = oa.k_steps;
        const int chunk_steps = S > 2 ? CHUNK_STEPS : nks;
        const int nchunks = (nks + chunk_steps - 1) / chunk_steps;
        long long acc[EPI_COLS];
        float facc[EPI_COLS];
#pragma unroll
        for (int c = 0; c < EPI_COLS; ++c) { acc[c] = 0; facc[c] = 0.f; }
        for (int ch = 0; ch < nchunks; ++ch, ++chunk) {
          const uint32_t xs = chunk & 1, xu = chunk >> 1;
          if (!mbar_wait_cl(smem_u32(&xfull[xs]), xu & 1, g.st, 450, &abort_flag, lim)) { ok = false; break; }
          fence_after();
          // 8 columns at a time: L2 and L3 (exact) then the FP32 tail levels T4 and T5+
#pragma unroll
          for (int hb = 0; hb < EPI_COLS; hb += 8) {
            uint32_t l2[8], l3[8];
            TMEM_LD8(lane_addr + xcol(xs) + hb, l2);
            TMEM_LD8(lane_addr + xcol(xs) + BN + hb, l3);
            tmem_wait_ld();
            if (S > 2) {
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                // L2: integer units; L3 was computed with pre-scaled slices: an integer multiple of 2^-8
                // |L2| <= 2^23, |256 L3| <= 2^24: hi parts fit 2^11 and 2^12, li parts 2^11
                int h2, i2, h3, i3;
                f32_round_split(__uint_as_float(l2[c]), h2, i2);
                f32_round_split(__uint_as_float(l3[c]) * 256.0f, h3, i3);
                acc[hb + c] += ((long long)(h2 * 256 + h3) << 28) + ((long long)(i2 * 256 + i3) << 16);
              }
            } else {
#pragma unroll
              for (int c = 0; c < 8; ++c) facc[hb + c] += __uint_as_float(l2[c]) + __uint_as_float(l3[c]);
            }
            if (C::TBLK) {
              // levels >= 4 of this chunk (FP32, rounded once per chunk into the fixed point)
              uint32_t t4[8], t5[8];
              TMEM_LD8(lane_addr + tcol(xs) + hb, t4);
              if (C::TBLK > 1) TMEM_LD8(lane_addr + tcol(xs) + BN + hb, t5);
              tmem_wait_ld();
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                // x 2^24: |T4| < 2^9 and |T5+| < 2^2 per chunk, inside the split's 2^33 range
                int h4, i4, h5 = 0, i5 = 0;
                f32_round_split(__uint_as_float(t4[c]) * 16777216.0f, h4, i4);
                if (C::TBLK > 1) f32_round_split(__uint_as_float(t5[c]) * 16777216.0f, h5, i5);
                acc[hb + c] += ((long long)(h4 + h5) << 12) + (long long)(i4 + i5);
              }
            }
          }
          fence_before();
          __syncwarp();
          if (lane == 0) {
            if (crank == 0) mbar_arrive(&xempty[xs]);
            else mbar_arrive_cluster(leader_xempty0 + xs * 8u);
          }
        }
        if (!ok) break;
        if (row_ok && ncols > 0) {
          const int Ei = S > 2 ? g.exps[oa.exp_off + gm] : 0;
          const int32_t* Fj = g.exps + ob.exp_off + wi.nt * BN + cg * EPI_COLS;
          const bool first = pd.first != 0;
          if (first && g.bmode == 0 && g.amode == 0) {
#pragma unroll
            for (int c = 0; c < EPI_COLS; ++c)
              if (c < ncols)
                Rb[colR_s[cg * EPI_COLS + c]] =
                    (S > 2) ? i64_scaled_to_f64(acc[c], Ei + __ldg(Fj + c) - 38) : (double)facc[c];
          } else {
#pragma unroll
            for (int c = 0; c < EPI_COLS; ++c) {
              if (c < ncols) {
                double v = (S > 2) ? i64_scaled_to_f64(acc[c], Ei + __ldg(Fj + c) - 38) : (double)facc[c];
                double* dst = Rb + colR_s[cg * EPI_COLS + c];
                if (first) *dst = g.bmode == 0 ? g.alpha * v : g.alpha * v + g.beta * *dst;
                else *dst = g.amode ? *dst + g.alpha * v : *dst + v;
              }
            }
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  cluster_sync_all();                 // no MMA, copy or remote arrival of the pair is in flight
  fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(C::TMEM_COLS));
  if (g.cta_times && threadIdx.x == 0) g.cta_times[2 * blockIdx.x + 1] = global_ns();
}

// Shared-memory attribute of split_gemm2<S> (set once) and the number of CTA pairs that
// can be resident at once, which is the persistent grid (SMs of a GPC pair up, so an odd
// count leaves one idle).  Returns 0 on failure.
template <int S>
int pair_slots_for(nd_handle h) {
  using C = Cfg2<S>;
  static std::mutex mu;
  static std::map<int, int> slots_of;   // per device
  std::lock_guard<std::mutex> lk(mu);
  auto known = slots_of.find(h->device);
  if (known != slots_of.end()) return known->second;
  int slots = 0;
  {
    if (cudaFuncSetAttribute(split_gemm2<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM) == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * std::max(1, h->num_sms / 2));
      cfg.blockDim = dim3(NTHREADS);
      cfg.dynamicSmemBytes = C::SMEM;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, (void*)split_gemm2<S>, &cfg) == cudaSuccess && n > 0) slots = n;
      else cudaGetLastError();
    } else {
      cudaGetLastError();
    }
  }
  slots_of[h->device] = slots;
  return slots;
}

int pair_slots(nd_handle h, int S) {
  switch (S) {
    case 2: return pair_slots_for<2>(h);
    case 3: return pair_slots_for<3>(h);
    case 4: return pair_slots_for<4>(h);
    case 5: return pair_slots_for<5>(h);
    default: return pair_slots_for<6>(h);
  }
}

template <int S>
nd_status launch_gemm2(nd_handle h, const GemmArgs& g, int slots) {
  if (pair_slots_for<S>(h) <= 0) return nd_fail(h, ND_ERR_CUDA, "split_gemm2: no CTA pair can be resident");
  GemmArgs gt = g;
  gt.cta_times = nd_cta_slot(h, 2 * slots);
  nd_prof_begin(h, "split_gemm");
  using C = Cfg2<S>;
  split_gemm2<S><<<2 * slots, NTHREADS, C::SMEM, h->stream>>>(gt);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  return nd_cuda_check(h, cudaGetLastError(), "split_gemm2");
}

// Persistent-CTA schedule.  Items (cost, tile) are assigned longest first to the
// least-loaded of G = min(#items, SMs) CTAs, and laid out so that the kernels'
// stride-G walk (item = blockIdx.x + r G) visits exactly each CTA's list; shorter
// lists are padded with empty items (pair_count 0), which every role skips.
// tmp must be sorted longest first (ties in list order).
std::vector<WorkItem> balance_items(const std::vector<std::pair<int64_t, WorkItem>>& tmp, int num_slots, int* slots_out) {
  std::vector<WorkItem> items;
  if (slots_out) *slots_out = 0;
  if (tmp.empty()) return items;
  const int G = std::max(1, std::min((int)tmp.size(), num_slots));
  if (slots_out) *slots_out = G;
  // Longest processing time first: each tile to the least-loaded slot (ties: lowest
  // index).  Tiles come in runs of equal cost c.  While every load lies within c of the
  // smallest, LPT gives G consecutive tiles of a run to the slots in (load, index) order
  // and keeps that order, so such a run is assigned in O(n) and the order repaired once
  // (a merge); otherwise the run goes tile by tile through a heap.  `order` is kept
  // either sorted or as that heap (the sorted array is a valid heap), and sorted again
  // only when a dealt run follows heap runs.
  std::vector<int> slot_of(tmp.size()), count(G, 0);
  std::vector<std::pair<int64_t, int>> order(G);                 // (load, slot)
  for (int b = 0; b < G; ++b) order[b] = {0, b};
  auto later = [](const auto& x, const auto& y) { return x.first > y.first || (x.first == y.first && x.second > y.second); };
  bool sorted = true;
  int64_t maxload = 0;
  for (size_t t0 = 0; t0 < tmp.size();) {
    size_t t1 = t0;
    while (t1 < tmp.size() && tmp[t1].first == tmp[t0].first) ++t1;
    const int64_t c = tmp[t0].first;
    if (maxload - order.front().first < c) {      // front: the smallest load, sorted or heap
      if (!sorted) { std::sort(order.begin(), order.end()); sorted = true; }
      const size_t n = t1 - t0, q = n / G, r = n % G;
      for (size_t t = t0; t < t1; ++t) {
        const int b = order[(t - t0) % G].second;
        slot_of[t] = b;
        ++count[b];
      }
      for (int k = 0; k < G; ++k) order[k].first += (int64_t)q * c + ((size_t)k < r ? c : 0);
      std::inplace_merge(order.begin(), order.begin() + r, order.end());
      maxload = order.back().first;
    } else {
      if (sorted) { std::make_heap(order.begin(), order.end(), later); sorted = false; }
      for (size_t t = t0; t < t1; ++t) {
        std::pop_heap(order.begin(), order.end(), later);
        slot_of[t] = order.back().second;
        ++count[order.back().second];
        order.back().first += c;
        maxload = std::max(maxload, order.back().first);
        std::push_heap(order.begin(), order.end(), later);
      }
    }
    t0 = t1;
  }
  const int L = *std::max_element(count.begin(), count.end());
  const WorkItem empty{tmp[0].second.group, tmp[0].second.pair_begin, 0, 0, 0};
  items.assign((size_t)L * G, empty);
  std::fill(count.begin(), count.end(), 0);
  for (size_t t = 0; t < tmp.size(); ++t) {      // slot b's r-th item sits at r * G + b
    const int b = slot_of[t];
    items[(size_t)count[b]++ * G + b] = tmp[t].second;
  }
  return items;
}

// Cost of one output tile in k-steps: its MMA steps plus a per-pair and per-tile
// epilogue share.
int64_t tile_cost(int64_t ksteps, int pairs) { return ksteps + 2 * (int64_t)pairs + 2; }

}  // namespace

// Host layout of one split-precision launch: the operand list (one entry per
// distinct A block and B block), the pairs pointing at their operands, the pack
// work list and the balanced output-tile list, with the packed-slice and exponent
// sizes.  Both the allocating path (nd_split_build) and the allocation-free one
// (nd_split_layout_into) place exactly this layout.
struct SplitLayout {
  std::vector<PairDesc> pairs;
  std::vector<SplitOp> ops;
  std::vector<PackItem2> pitems;
  std::vector<WorkItem> items;
  int64_t pack_bytes = 0, exp_count = 0;
  int nops_a = 0, nops_b = 0;
  int pair2 = 0;     // 1: 256 x 64 tiles on CTA pairs (split_gemm2); 0: 128 x 64 tiles (split_gemm)
  int slots = 0;     // persistent CTAs (1-CTA tiles) or CTA pairs (2-CTA tiles)
  std::vector<ReduceItem> red;   // split-K tiles and their workspace slots
  int nws = 0;                   // workspace slots (BM x BN int64 each)
};

// pair2: tiles for CTA pairs.  A operands then hold an even number of 128-row tiles
// (the odd CTA of a pair whose rows run past M stages zero digits, and the epilogue
// stores nothing for those rows); work item mt is the index of a pair of row tiles.
static void split_layout(nd_handle h, const std::vector<PairDesc>& pairs_in, int S, int pair2, SplitLayout& L,
                         bool splitk = false) {
  L = SplitLayout{};
  L.pair2 = pair2 ? 1 : 0;
  L.pairs = pairs_in;
  // (job, offset) -> op, ids in first-appearance order
  std::unordered_map<uint64_t, int> amap, bmap;
  amap.reserve(pairs_in.size());
  bmap.reserve(pairs_in.size());
  auto add_op = [&](bool is_b, const PairDesc& pd) -> int {
    auto& mp = is_b ? bmap : amap;
    const int64_t off = is_b ? pd.b_off : pd.a_off;
    const uint64_t key = ((uint64_t)off << 1) | (uint64_t)(pd.job & 1);   // offsets < 2^62, job 0 / 1
    auto f = mp.find(key);
    if (f != mp.end()) return f->second;
    SplitOp o{};
    o.src_off = off;
    o.is_b = is_b;
    o.job = pd.job;
    o.rows = is_b ? pd.N : pd.M;
    o.kdim = pd.K;
    o.rk = is_b ? pd.cols : pd.rows;          // st0 = strides in this operand
    o.kk = pd.ks;
    if (is_b) for (int d = 0; d < o.kk.n; ++d) o.kk.st0[d] = pd.ks.st1[d];
    const int rows_per_tile = is_b ? BN : BM;
    o.row_tiles = (o.rows + rows_per_tile - 1) / rows_per_tile;
    if (L.pair2 && !is_b) o.row_tiles += o.row_tiles & 1;
    o.k_steps = (o.kdim + BK - 1) / BK;
    o.pack_off = L.pack_bytes;
    L.pack_bytes += (int64_t)o.row_tiles * o.k_steps * S * (is_b ? B_SLICE : A_SLICE);
    o.exp_off = L.exp_count;
    L.exp_count += (int64_t)o.row_tiles * rows_per_tile;
    L.ops.push_back(o);
    mp[key] = (int)L.ops.size() - 1;
    return (int)L.ops.size() - 1;
  };
  for (auto& pd : L.pairs) {
    pd.a_op = add_op(false, pd);
    pd.b_op = add_op(true, pd);
  }
  L.nops_a = (int)amap.size();
  L.nops_b = (int)bmap.size();
  for (int i = 0; i < (int)L.ops.size(); ++i)
    for (int t = 0; t < L.ops[i].row_tiles; ++t)
      for (int kc = 0; kc * PACK_KC < L.ops[i].k_steps; ++kc) L.pitems.push_back({i, t, kc});
  // work items: BM x BN output tiles, balanced over the persistent CTAs.  Every tile of
  // a group costs the same, so the groups are sorted (longest first, ties in group
  // order) and expanded into tiles: the order a stable sort of the tiles would give.
  struct Grp { int64_t cost; size_t i, n; };
  std::vector<Grp> grps;
  for (size_t i = 0; i < L.pairs.size();) {
    size_t j = i;
    int64_t ksteps = 0;
    while (j < L.pairs.size() && L.pairs[j].group == L.pairs[i].group && L.pairs[j].job == L.pairs[i].job) {
      ksteps += (L.pairs[j].K + BK - 1) / BK;
      ++j;
    }
    grps.push_back({tile_cost(ksteps, (int)(j - i)), i, j - i});
    i = j;
  }
  std::stable_sort(grps.begin(), grps.end(), [](const Grp& x, const Grp& y) { return x.cost > y.cost; });
  std::vector<std::pair<int64_t, WorkItem>> tmp;
  int64_t total_ksteps = 0;
  {
    size_t ntiles = 0;
    for (const Grp& g : grps) {
      const PairDesc& p = L.pairs[g.i];
      const size_t mt = (p.M + BM - 1) / BM;
      const size_t tiles = (L.pair2 ? (mt + 1) / 2 : mt) * ((p.N + BN - 1) / BN);
      ntiles += tiles;
      for (size_t q = g.i; q < g.i + g.n; ++q) total_ksteps += (int64_t)tiles * ((L.pairs[q].K + BK - 1) / BK);
    }
    tmp.reserve(ntiles);
  }
  // Split-K (1-CTA tiles, S > 2): a tile of a single-pair output block whose K is long
  // against the launch's fair share (twice the k steps per CTA) is cut into K ranges that
  // start at 512-K chunk boundaries; each range's CTA writes its exact int64 tile to a
  // workspace slot and split_reduce adds them.  A 10 x 10 output with K = 5e5 (a cotangent
  // of an MPO tensor) otherwise runs on one CTA.
  int64_t share = INT64_MAX;
  if (splitk && !L.pair2 && S > 2) {
    const int64_t fair = (total_ksteps + h->num_sms - 1) / h->num_sms;
    share = std::max<int64_t>(2 * CHUNK_STEPS, (2 * fair + CHUNK_STEPS - 1) / CHUNK_STEPS * CHUNK_STEPS);
  }
  bool any_split = false;
  for (const Grp& g : grps) {
    const PairDesc& p = L.pairs[g.i];
    int mt = (p.M + BM - 1) / BM;
    const int nt = (p.N + BN - 1) / BN;
    if (L.pair2) mt = (mt + 1) / 2;
    const int64_t kst = (p.K + BK - 1) / BK;
    for (int a = 0; a < mt; ++a)
      for (int b = 0; b < nt; ++b) {
        if (g.n == 1 && kst > share) {
          const int64_t nch = (kst + share - 1) / share;
          const int64_t kc = ((kst + nch - 1) / nch + CHUNK_STEPS - 1) / CHUNK_STEPS * CHUNK_STEPS;
          const int slot0 = L.nws;
          for (int64_t k0 = 0; k0 < kst; k0 += kc) {
            WorkItem w{p.group, (int)g.i, 1, a, b};
            w.kbeg = (int32_t)k0;
            w.kend = (int32_t)std::min(kst, k0 + kc);
            w.slot = L.nws++;
            tmp.push_back({tile_cost(w.kend - w.kbeg, 1), w});
          }
          L.red.push_back(ReduceItem{(int32_t)g.i, a, b, slot0, L.nws - slot0});
          any_split = true;
        } else {
          tmp.push_back({g.cost, WorkItem{p.group, (int)g.i, (int)g.n, a, b}});
        }
      }
  }
  if (any_split)      // balance_items takes the items longest first
    std::stable_sort(tmp.begin(), tmp.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
  int nslots = h->num_sms;
  if (L.pair2) {
    nslots = pair_slots(h, S);
    if (nslots <= 0) {            // the pair kernel cannot run here: single-CTA tiles
      L = SplitLayout{};
      split_layout(h, pairs_in, S, 0, L);
      return;
    }
  }
  L.items = balance_items(tmp, nslots, &L.slots);
}

static void split_adopt(ExecCache& c, const SplitLayout& L, int S) {
  c.nsplit_items = (int)L.items.size();
  c.npack_items = (int)L.pitems.size();
  c.nops_a = L.nops_a;
  c.nops_b = L.nops_b;
  c.pack_bytes = L.pack_bytes;
  c.exp_count = L.exp_count;
  c.slices = S;
  c.split_pair2 = L.pair2;
  c.split_slots = L.slots;
}

// Build operand list, packed layout and work items (host; once per plan/precision).
nd_status nd_split_build(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs_in, int ngroups, int precision,
                         int pair2) {
  (void)ngroups;
  const int S = precision == ND_PREC_OZAKI ? h->ozaki_slices : 2;
  SplitLayout L;
  split_layout(h, pairs_in, S, pair2, L, true);
  auto up = [&](void** dst, const void* src, size_t bytes) -> nd_status {
    nd_status e = nd_dalloc(h, dst, bytes);
    if (e) return e;
    return nd_upload(h, *dst, src, bytes);
  };
  nd_status s;
  if ((s = up((void**)&c.d_split_pairs, L.pairs.data(), L.pairs.size() * sizeof(PairDesc)))) return s;
  if ((s = up((void**)&c.d_split_items, L.items.data(), L.items.size() * sizeof(WorkItem)))) return s;
  if ((s = up(&c.d_operands, L.ops.data(), L.ops.size() * sizeof(SplitOp)))) return s;
  if ((s = up(&c.d_pack_items, L.pitems.data(), L.pitems.size() * sizeof(PackItem2)))) return s;
  if ((s = nd_dalloc(h, &c.d_rowmax, std::max<int64_t>(L.exp_count, 1) * 8))) return s;
  if ((s = nd_dalloc(h, &c.d_pack, std::max<int64_t>(L.pack_bytes, 16)))) return s;
  if ((s = nd_dalloc(h, (void**)&c.d_exp, std::max<int64_t>(L.exp_count, 4) * 4))) return s;
  if (!L.red.empty()) {
    if ((s = up((void**)&c.d_red, L.red.data(), L.red.size() * sizeof(ReduceItem)))) return s;
    if ((s = nd_dalloc(h, (void**)&c.d_ws, (size_t)L.nws * BM * BN * sizeof(long long)))) return s;
  }
  c.nred = (int)L.red.size();
  split_adopt(c, L, S);
  return ND_OK;
}

nd_status nd_split_run(nd_handle h, ExecCache& c, const JobPtrs& ptrs, double alpha, double beta) {
  const int S = c.slices;
  PackArgs2 pa{(const SplitOp*)c.d_operands, (const PackItem2*)c.d_pack_items, c.npack_items, ptrs,
               (unsigned char*)c.d_pack, c.d_exp, (unsigned long long*)c.d_rowmax, S, h->d_status};
  // one CTA per pack item: the block scheduler hands items to SMs as they free up, so
  // the launch ends within about one item of the ideal (a fixed per-CTA item list left
  // a second partial wave)
  int pblocks = c.npack_items;
  if (pblocks > 0) {
    if (S > 2) {
      ND_CUDA(h, cudaMemsetAsync(c.d_rowmax, 0, c.exp_count * 8, h->stream));
      nd_prof_begin(h, "pack_rowmax");
      pack_rowmax<<<pblocks, 256, 0, h->stream>>>(pa);
      nd_prof_end(h);
      ND_LAUNCHED(h);
    }
    nd_prof_begin(h, "pack_digits");
    switch (S) {
      case 2: pack_digits<2><<<pblocks, 256, 0, h->stream>>>(pa); break;
      case 3: pack_digits<3><<<pblocks, 256, 0, h->stream>>>(pa); break;
      case 4: pack_digits<4><<<pblocks, 256, 0, h->stream>>>(pa); break;
      case 5: pack_digits<5><<<pblocks, 256, 0, h->stream>>>(pa); break;
      default: pack_digits<6><<<pblocks, 256, 0, h->stream>>>(pa); break;
    }
    nd_prof_end(h);
    ND_LAUNCHED(h);
    ND_CUDA(h, cudaGetLastError());
  }
  GemmArgs g{c.d_split_pairs, c.d_split_items, c.nsplit_items, (const SplitOp*)c.d_operands,
             (const unsigned char*)c.d_pack, c.d_exp, ptrs, alpha, beta, alpha == 1.0 ? 0 : 1, beta == 0.0 ? 0 : 1,
             h->d_status, nullptr, (long long*)c.d_ws};
  if (c.nsplit_items == 0) return ND_OK;
  if (c.split_pair2) {
    switch (S) {
      case 2: return launch_gemm2<2>(h, g, c.split_slots);
      case 3: return launch_gemm2<3>(h, g, c.split_slots);
      case 4: return launch_gemm2<4>(h, g, c.split_slots);
      case 5: return launch_gemm2<5>(h, g, c.split_slots);
      case 6: return launch_gemm2<6>(h, g, c.split_slots);
    }
  } else {
    nd_status s = ND_OK;
    switch (S) {
      case 2: s = launch_gemm<2>(h, g); break;
      case 3: s = launch_gemm<3>(h, g); break;
      case 4: s = launch_gemm<4>(h, g); break;
      case 5: s = launch_gemm<5>(h, g); break;
      case 6: s = launch_gemm<6>(h, g); break;
      default: return nd_fail(h, ND_ERR_ARG, "unsupported slice count %d", S);
    }
    if (s || c.nred == 0) return s;
    nd_prof_begin(h, "split_reduce");
    const int parts = std::max(1, std::min(16, (2 * h->num_sms + c.nred - 1) / c.nred));
    split_reduce<<<dim3(std::min(c.nred, 4 * h->num_sms), parts), 256, 0, h->stream>>>(
        c.d_split_pairs, c.d_red, c.nred, (const SplitOp*)c.d_operands, c.d_exp, (const long long*)c.d_ws, ptrs, alpha,
        beta, alpha == 1.0 ? 0 : 1, beta == 0.0 ? 0 : 1);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    return nd_cuda_check(h, cudaGetLastError(), "split_reduce");
  }
  return nd_fail(h, ND_ERR_ARG, "unsupported slice count %d", S);
}

// Lay out one split-precision launch inside caller-provided device memory
// instead of allocating: the same layout as nd_split_build (split_layout), the
// bytes it needs reported in *needed, and when `base` holds enough, the
// descriptors uploaded there and the cache's fields pointed into it.
nd_status nd_split_layout_into(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs_in, int S,
                               unsigned char* base, size_t capacity, size_t* needed) {
  SplitLayout L;
  split_layout(h, pairs_in, S, h->split_pair2, L);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_pairs = 0;
  const size_t o_items = al(o_pairs + L.pairs.size() * sizeof(PairDesc));
  const size_t o_ops = al(o_items + L.items.size() * sizeof(WorkItem));
  const size_t o_pit = al(o_ops + L.ops.size() * sizeof(SplitOp));
  const size_t o_exp = al(o_pit + L.pitems.size() * sizeof(PackItem2));
  const size_t o_rmx = al(o_exp + (size_t)L.exp_count * 4);
  const size_t o_pack = al(o_rmx + (size_t)L.exp_count * 8);
  const size_t total = o_pack + (size_t)L.pack_bytes;
  if (needed) *needed = total;
  if (!base) return ND_OK;
  if (total > capacity) return ND_ERR_ARG;
  cudaStream_t s = h->stream;
  ND_CUDA(h, cudaMemcpyAsync(base + o_pairs, L.pairs.data(), L.pairs.size() * sizeof(PairDesc), cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(base + o_items, L.items.data(), L.items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(base + o_ops, L.ops.data(), L.ops.size() * sizeof(SplitOp), cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(base + o_pit, L.pitems.data(), L.pitems.size() * sizeof(PackItem2), cudaMemcpyHostToDevice, s));
  c.d_split_pairs = (PairDesc*)(base + o_pairs);
  c.d_split_items = (WorkItem*)(base + o_items);
  c.d_operands = base + o_ops;
  c.d_pack_items = base + o_pit;
  c.d_exp = (int32_t*)(base + o_exp);
  c.d_rowmax = base + o_rmx;
  c.d_pack = base + o_pack;
  split_adopt(c, L, S);
  return ND_OK;
}
