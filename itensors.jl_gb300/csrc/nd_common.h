// Internal definitions shared by the translation units of libndtensors_gb300.so.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <map>
#include <mutex>
#include "../../include/ndtensors_gb300.h"

#define ND_HOSTDEV __host__ __device__ __forceinline__

// Bounded device-side waits: a spin that runs past its limit records
// ND_ERR_TIMEOUT in the status word and returns instead of hanging the GPU.
// ND_SPIN_LIMIT is the default limit of the waits that make progress (set per
// handle with nd_set_spin_limit) and the fixed limit of the clean-up waits that
// let issued copies and MMAs land before a CTA exits after a timeout.
#define ND_SPIN_LIMIT (1u << 26)

// Device status word of a handle: [code] = first error code, [where] = the site
// that raised it, [spin_limit] = poll limit of the progress waits (0 = default).
struct DeviceStatus {
  int32_t code;
  int32_t where;
  uint32_t spin_limit;
  uint32_t reserved;
};

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t nd_spin_limit(const DeviceStatus* st) {
  const uint32_t l = *(const volatile uint32_t*)&st->spin_limit;
  return l ? l : ND_SPIN_LIMIT;
}
#endif

// Execution parameters chosen by the autotuner (per block-size histogram).
struct TuneChoice {
  int32_t splitk_mult = 4;   // FP64 tile kernel: split-K balances work over splitk_mult x SMs CTAs (0 = off)
  int32_t skinny = 1;        // 1: skinny groups (N <= 8, K <= 32) on the FP64 CUDA-core kernel
  int32_t pair2 = 0;         // split GEMM tile shape: 1 = 256 x 64 on CTA pairs, 0 = 128 x 64 per CTA
};
struct TuneEntry {
  TuneChoice choice;
  double best_ms = 0.0, default_ms = 0.0;
};

struct nd_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  int ozaki_slices = 5;
  int svd_max_sweeps = -1;            // FP64 Jacobi sweep limit of the SVD (-1 = default 60)
  // per-CTA start / end times of the last split-GEMM launches (nd_set_cta_timing)
  int cta_timing = 0;
  unsigned long long* d_cta_times = nullptr;   // ND_CTA_SLOTS x ND_CTA_MAX x {start, end}
  int cta_nlaunch = 0;
  int cta_nctas[8] = {0};
  // convergence record of the last SVD (nd_svd_last_info)
  std::vector<int32_t> svd_info_i;
  std::vector<double> svd_info_d;
  int split_pair2 = 0;                // untuned split-GEMM tile shape (TuneChoice::pair2)
  std::string last_error;
  DeviceStatus* d_status = nullptr;   // device status word
  int64_t launches = 0;
  // grow-only scratch arena (device) and its pinned host staging buffer (the planner's)
  void* ws = nullptr;
  size_t ws_size = 0;
  void* pin = nullptr;
  size_t pin_size = 0;
  cudaEvent_t order_ev = nullptr;     // orders state used on a previous stream before the current one
  void* vec_part = nullptr;           // per-CTA partial sums of the vector reductions (fixed size)
  // the one-CTA planner runs on its own stream with its own status word, so building a
  // plan waits only for the planner, not for contractions queued on the handle's stream
  cudaStream_t plan_stream = nullptr;
  DeviceStatus* d_plan_status = nullptr;
  int plan_where = 0;                 // nd_set_plan_placement: 0 by size, 1 device, 2 host
  int permute_tma = 0;                // nd_set_permute_path: 1 = TMA tiles where they apply
  int verify = 0;                     // nd_set_verify: rerun split-precision contractions in FP64
  double verify_err = -1.0;           // nd_verify_last: last recorded relative Frobenius distance
  // pinned ring for descriptor uploads (nd_upload): region [begin, end) may be reused
  // once its copy's event has completed
  unsigned char* up_ring = nullptr;
  size_t up_cap = 0, up_head = 0;
  struct UpRec { size_t begin, end; cudaEvent_t ev; };
  std::vector<UpRec> up_fifo;
  std::vector<cudaEvent_t> up_events;
  // graph capture
  cudaGraph_t graph = nullptr;
  bool capturing = false;
  // kernel timing
  bool profiling = false;
  struct ProfRec { const char* name; cudaEvent_t e0, e1; };
  std::vector<ProfRec> prof;
  std::vector<size_t> prof_open;   // indices of the regions begun and not yet ended (regions nest)
  std::vector<cudaEvent_t> event_pool;
  // autotuner
  bool tuning = false;
  std::map<std::string, TuneEntry> tune;
  // device state of recent dense contractions, keyed by their GEMM descriptor and
  // precision (owned by nd_contract.cu; released by nd_dense_cache_clear)
  std::map<std::string, void*> dense_cache;
  std::vector<std::string> dense_order;   // insertion order, for eviction
};

void nd_dense_cache_clear(nd_handle h);

// True while the handle's stream is being captured into a CUDA graph, whether the
// capture was opened by nd_graph_begin or by the caller (e.g. torch.cuda.graph):
// the library then allocates, uploads and synchronises nothing.
bool nd_capturing(nd_handle h);

// Host helpers -------------------------------------------------------------
nd_status nd_fail(nd_handle h, nd_status code, const char* fmt, ...);
nd_status nd_cuda_check(nd_handle h, cudaError_t e, const char* what);
// Host -> device copy of descriptors on the handle's stream through a pinned ring, so
// the host never waits for the driver's pageable staging (which blocks once copies
// queue behind running kernels).  `src` may be reused as soon as the call returns.
nd_status nd_upload(nd_handle h, void* dst, const void* src, size_t bytes);
// Device memory for a contraction's execution state: stream-ordered allocations on
// the handle's stream from the device's default pool, which nd_create keeps from
// returning freed memory to the system, so rebuilding state per plan costs no
// device-wide synchronisation.
nd_status nd_dalloc(nd_handle h, void** p, size_t bytes);
nd_status nd_check_device_status(nd_handle h, const char* what);  // syncs

// One-time set-up of a launch site (a kernel's shared-memory opt-in, an occupancy
// query) per device, since kernel attributes apply per device: thread-safe, so that
// handles driven from different host threads may launch concurrently, and retried
// after a failure.
struct NdOnce {
  std::mutex m;
  uint64_t done = 0;   // bit d: device d is set up
};
template <typename F>
cudaError_t nd_once(NdOnce& o, int device, F&& f) {
  std::lock_guard<std::mutex> lk(o.m);
  const uint64_t bit = 1ull << (device & 63);
  if (o.done & bit) return cudaSuccess;
  const cudaError_t e = f();
  if (e == cudaSuccess) o.done |= bit;
  return e;
}

#define ND_CUDA(h, call)                                              \
  do {                                                                \
    cudaError_t _e = (call);                                          \
    if (_e != cudaSuccess) return nd_cuda_check((h), _e, #call);      \
  } while (0)

#define ND_LAUNCHED(h) do { (h)->launches++; } while (0)

constexpr int ND_CTA_SLOTS = 8, ND_CTA_MAX = 1024;
// Slot for the per-CTA timestamps of the next split-GEMM launch (nullptr when timing is off).
unsigned long long* nd_cta_slot(nd_handle h, int nctas);

// Bracket a launch with timing events when profiling is on (not inside capture).
void nd_prof_begin(nd_handle h, const char* name);
void nd_prof_end(nd_handle h);

// Mixed-radix index decomposition ------------------------------------------
// A GEMM row / column / reduction index enumerates several tensor dimensions,
// first dimension fastest.  st0/st1 are the element strides of those
// dimensions in two tensors (e.g. A and R for rows).
struct Mixed {
  int32_t n;
  int32_t dim[ND_MAX_RANK];
  // division by dim[d] as a multiply-high (Granlund & Montgomery, "Division by
  // invariant integers using multiplication", PLDI 1994, round-up multiplier):
  // for 0 <= x < 2^31, x / d == (umulhi(x, mul) + x) >> shr with shr = ceil(log2 d),
  // mul = floor(2^32 (2^shr - d) / d) + 1.  mul == 0 means "not computed".
  uint32_t mul[ND_MAX_RANK];
  uint32_t shr[ND_MAX_RANK];
  int64_t st0[ND_MAX_RANK];
  int64_t st1[ND_MAX_RANK];
};

// Fill mul / shr of every dimension (host).
inline void mixed_finalize(Mixed& m) {
  for (int d = 0; d < ND_MAX_RANK; ++d) { m.mul[d] = 0; m.shr[d] = 0; }
  for (int d = 0; d < m.n; ++d) {
    const uint64_t dd = (uint64_t)(uint32_t)m.dim[d];
    if (dd == 0) continue;
    uint32_t shr = 0;
    while ((1ull << shr) < dd) ++shr;
    m.shr[d] = shr;
    m.mul[d] = (uint32_t)((((1ull << 32) * ((1ull << shr) - dd)) / dd) + 1ull);
  }
}

ND_HOSTDEV uint32_t nd_umulhi(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

ND_HOSTDEV void mixed_offsets(const Mixed& m, int64_t lin, int64_t& o0, int64_t& o1) {
  int64_t a = 0, b = 0;
  for (int d = 0; d < m.n; ++d) {
    int64_t q = lin / m.dim[d];
    int64_t r = lin - q * m.dim[d];
    a += r * m.st0[d];
    b += r * m.st1[d];
    lin = q;
  }
  o0 = a;
  o1 = b;
}

// Same for indices below 2^31 (GEMM extents are < 2^31), dividing by multiply-high
// when the divisors were computed: integer instructions only, no conversion or
// FP64 pipe work (which GB300 runs at a fraction of the integer rate).
ND_HOSTDEV void mixed_offsets32(const Mixed& m, uint32_t lin, int64_t& o0, int64_t& o1) {
  int64_t a = 0, b = 0;
  for (int d = 0; d < m.n; ++d) {
    const uint32_t dd = (uint32_t)m.dim[d];
    const uint32_t q = m.mul[d] ? (nd_umulhi(lin, m.mul[d]) + lin) >> m.shr[d] : lin / dd;
    const uint32_t r = lin - q * dd;
    a += (int64_t)r * m.st0[d];
    b += (int64_t)r * m.st1[d];
    lin = q;
  }
  o0 = a;
  o1 = b;
}

// Merge adjacent dimensions that are contiguous in both strided views.
inline void mixed_simplify(Mixed& m) {
  Mixed o{};
  o.n = 0;
  for (int d = 0; d < m.n; ++d) {
    if (m.dim[d] == 1) continue;
    if (o.n > 0) {
      int k = o.n - 1;
      if (o.st0[k] * o.dim[k] == m.st0[d] && o.st1[k] * o.dim[k] == m.st1[d]) {
        o.dim[k] *= m.dim[d];
        continue;
      }
    }
    o.dim[o.n] = m.dim[d];
    o.st0[o.n] = m.st0[d];
    o.st1[o.n] = m.st1[d];
    o.n++;
  }
  mixed_finalize(o);
  m = o;
}

// How the labels of one contraction map onto a GEMM (shared by all block pairs).
struct Roles {
  int rankA, rankB, rankR;
  int nfa, nfb, nk;
  int a_free[ND_MAX_RANK];   // positions in A of A-free dims, in output order
  int r_afree[ND_MAX_RANK];  // their positions in R
  int b_free[ND_MAX_RANK];
  int r_bfree[ND_MAX_RANK];
  int a_k[ND_MAX_RANK];      // positions in A of contracted dims, in A order
  int b_k[ND_MAX_RANK];      // matching positions in B
};

// Build roles from ncon labels; returns false on invalid labels.
bool nd_make_roles(int rankA, const int32_t* la, int rankB, const int32_t* lb, int rankR,
                   const int32_t* lr, Roles& ro, std::string& why);

// One block pair of a contraction, ready for the GEMM kernels.
struct PairDesc {
  int64_t a_off, b_off, r_off;   // element offsets of the three blocks
  int32_t M, N, K, group;        // GEMM sizes, output block (group) id
  int32_t a_op, b_op;            // operand-slot ids (packed split operands)
  int32_t first;                 // 1 if first pair of its group (overwrite)
  int32_t job;                   // which (A, B, R) base-pointer triple (0 or 1)
  Mixed rows;   // st0: A strides, st1: R strides
  Mixed cols;   // st0: B strides, st1: R strides
  Mixed ks;     // st0: A strides, st1: B strides
  int32_t sym = 0;   // 1: R is symmetric (M == N); the FP64 tile kernel computes the tiles on
                     // and above the diagonal only, the caller mirrors the rest
  int32_t pad_[3] = {0, 0, 0};   // keeps the size a multiple of 16 bytes
};

// A split operand (one A block or one B block) for the split-precision GEMMs.
struct OperandDesc {
  int64_t src_off;      // element offset of the block in its tensor
  int32_t rows, kdim;   // GEMM view: rows (M or N) x K
  int32_t row_tiles, k_steps;
  int64_t pack_off;     // byte offset of its packed slices
  int64_t exp_off;      // int32 offset of its per-row exponents
  Mixed rk;             // st0: strides of rows, st1 unused ; see pack kernel
  Mixed kk;             // st0: strides of k
};

// Work item of the grouped GEMMs: one output tile of one group.
struct WorkItem {
  int32_t group;        // group id
  int32_t pair_begin;   // first pair (pairs sorted by group)
  int32_t pair_count;
  int32_t mt, nt;       // tile coordinates
  // split-K: the item covers [kbeg, kend) of the group's k axis and writes its
  // partial tile to workspace slot `slot`; slot < 0 means the whole k axis, written
  // to R.  FP64 tile kernel: the k axis is the pairs' K ranges concatenated in plan
  // order, in elements; split GEMM (single-pair groups only): 32-wide k steps, ranges
  // starting on 512-K chunk boundaries.
  int32_t kbeg = 0, kend = 0, slot = -1;
};

// One output tile whose split-K partials are summed into R (in slot order).
struct ReduceItem {
  int32_t pair;         // first pair of the group (rows / cols / job / r_off)
  int32_t mt, nt;
  int32_t slot0, nslots;
};

// Split-precision parameters
#define ND_OZ_BM 128
#define ND_OZ_BN 64
#define ND_OZ_BK 32
#define ND_OZ_CHUNK_STEPS 16   // 16 * 32 = 512 of K per exact chunk

// Kernel launchers (defined in the .cu files) ------------------------------
nd_status nd_launch_permute(nd_handle h, double* R, const double* T, int rank, const int64_t* dims,
                            const int* perm0, double alpha, double beta, const double* scalar_dev);
// Base pointers of up to two contractions executed by one grouped launch.
struct JobPtrs {
  const double* A[2];
  const double* B[2];
  double* R[2];
};

#ifdef __CUDACC__
// Base pointers of a job's operands as selects: indexing a kernel-parameter array with
// a run-time value makes the compiler copy the parameters to local memory.
__device__ __forceinline__ const double* job_A(const JobPtrs& p, int j) { return j ? p.A[1] : p.A[0]; }
__device__ __forceinline__ const double* job_B(const JobPtrs& p, int j) { return j ? p.B[1] : p.B[0]; }
__device__ __forceinline__ double* job_R(const JobPtrs& p, int j) { return j ? p.R[1] : p.R[0]; }
#endif

nd_status nd_launch_gemm_f64(nd_handle h, const PairDesc* d_pairs, const WorkItem* d_items,
                             int nitems, const JobPtrs& ptrs, double alpha, double beta, double* ws,
                             const ReduceItem* d_red, int nred);
int nd_gemm_f64_tile_elems();
