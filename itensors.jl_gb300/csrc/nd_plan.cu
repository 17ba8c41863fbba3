// Block-pair plan built on the device, bit-exact with the reference's
// sequential plan (NDTensors/src/blocksparse/contract_sequential.jl:1-41):
//
//   for block1 in keys(boffs1), block2 in keys(boffs2)        (A-major, B-minor)
//     if are_blocks_contracted(block1, block2)               (contract_utilities.jl:57-70)
//       blockR = contract_blocks(block1, block2)             (contract_utilities.jl:72-91)
//       push!(plan, (block1, block2, blockR))
//       blockR not yet seen -> insert at offset nnzR, nnzR += blockdim(blockR)
//
// GB300 form: one thread per candidate pair computes the match flag; an
// exclusive scan compacts matches in (A-major, B-minor) order, which is the
// reference's order by construction.  Output blocks are identified by their
// column-major linear block index; a device hash table records each key's
// first pair, so "first appearance" is a flag per pair, and a second scan
// numbers the output blocks in first-appearance order.  A third scan over the
// output block sizes gives the offsets.  No step depends on thread timing.
#include "nd_common.h"
#include "nd_plan.h"
#include <algorithm>
#include <climits>
#include <cstring>
#include <unordered_map>

namespace {

constexpr int SCAN_BLOCK = 1024;
constexpr int64_t PLAN1_MAX = 1 << 20;    // candidate pairs planned by one CTA in one launch

__global__ void scan_block_sums(const int64_t* in, int64_t* block_sums, int64_t n) {
  __shared__ int64_t s[SCAN_BLOCK];
  int64_t i = (int64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
  s[threadIdx.x] = i < n ? in[i] : 0;
  __syncthreads();
  for (int o = SCAN_BLOCK / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = s[0];
}

// in-place exclusive scan of each SCAN_BLOCK chunk, plus the chunk's offset
__global__ void scan_apply(int64_t* data, const int64_t* block_offsets, int64_t n) {
  __shared__ int64_t s[SCAN_BLOCK];
  int64_t i = (int64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
  int64_t v = i < n ? data[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
    int64_t t = (int)threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) data[i] = s[threadIdx.x] - v + (block_offsets ? block_offsets[blockIdx.x] : 0);
}

__global__ void write_total(const int64_t* scanned, const int64_t* orig_last, int64_t n, int64_t* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *total = n > 0 ? scanned[n - 1] + *orig_last : 0;
}

__global__ void copy_last(const int64_t* data, int64_t n, int64_t* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = n > 0 ? data[n - 1] : 0;
}

struct PlanKParams {
  int32_t nA, nB, rankA, rankB, rankR;
  int32_t nk, nfa, nfb;
  int32_t a_k[ND_MAX_RANK], b_k[ND_MAX_RANK];
  int32_t a_free[ND_MAX_RANK], r_afree[ND_MAX_RANK];
  int32_t b_free[ND_MAX_RANK], r_bfree[ND_MAX_RANK];
  int64_t r_nblocks[ND_MAX_RANK];      // blocks per R dimension
  int32_t r_bd_off[ND_MAX_RANK];       // offset of each R dimension in r_blockdims
};

__device__ __forceinline__ void blockR_coords(const PlanKParams& p, const int32_t* bA, const int32_t* bB, int32_t* c) {
  for (int t = 0; t < p.nfa; ++t) c[p.r_afree[t]] = bA[p.a_free[t]];
  for (int t = 0; t < p.nfb; ++t) c[p.r_bfree[t]] = bB[p.b_free[t]];
}

__device__ __forceinline__ uint64_t key_of(const PlanKParams& p, const int32_t* c) {
  uint64_t k = 0, mul = 1;
  for (int r = 0; r < p.rankR; ++r) { k += (uint64_t)(c[r] - 1) * mul; mul *= (uint64_t)p.r_nblocks[r]; }
  return k;
}

__global__ void match_kernel(PlanKParams p, const int32_t* blocksA, const int32_t* blocksB, int64_t* flags) {
  const int64_t total = (int64_t)p.nA * p.nB;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i1 = (int32_t)(idx / p.nB), i2 = (int32_t)(idx % p.nB);
    const int32_t* bA = blocksA + (int64_t)i1 * p.rankA;
    const int32_t* bB = blocksB + (int64_t)i2 * p.rankB;
    bool ok = true;
    for (int t = 0; t < p.nk; ++t) ok = ok && (bA[p.a_k[t]] == bB[p.b_k[t]]);
    flags[idx] = ok ? 1 : 0;
  }
}

__device__ __forceinline__ uint32_t hash64(uint64_t k) {
  k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
  return (uint32_t)k;
}

__global__ void compact_kernel(PlanKParams p, const int32_t* blocksA, const int32_t* blocksB, const int64_t* flags,
                               const int64_t* pos, int32_t* pairs, uint64_t* keys, uint64_t* table_keys,
                               int32_t* table_vals, uint32_t mask, DeviceStatus* st) {
  const int64_t total = (int64_t)p.nA * p.nB;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    if (!flags[idx]) continue;
    const int32_t i1 = (int32_t)(idx / p.nB), i2 = (int32_t)(idx % p.nB);
    const int64_t q = pos[idx];
    int32_t c[ND_MAX_RANK];
    blockR_coords(p, blocksA + (int64_t)i1 * p.rankA, blocksB + (int64_t)i2 * p.rankB, c);
    const uint64_t key = key_of(p, c);
    pairs[3 * q + 0] = i1;
    pairs[3 * q + 1] = i2;
    keys[q] = key;
    uint32_t hsh = hash64(key) & mask;
    bool done = false;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      unsigned long long prev = atomicCAS((unsigned long long*)&table_keys[hsh], ~0ull, (unsigned long long)key);
      if (prev == ~0ull || prev == key) { atomicMin(&table_vals[hsh], (int32_t)q); done = true; break; }
      hsh = (hsh + 1) & mask;
    }
    if (!done && atomicCAS(&st->code, 0, ND_ERR_ARG) == 0) st->where = 200;
  }
}

__device__ __forceinline__ int32_t table_lookup(uint64_t key, const uint64_t* tk, const int32_t* tv, uint32_t mask) {
  uint32_t hsh = hash64(key) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    if (tk[hsh] == key) return tv[hsh];
    if (tk[hsh] == ~0ull) return -1;
    hsh = (hsh + 1) & mask;
  }
  return -1;
}

__global__ void first_flags_kernel(int64_t npairs, const uint64_t* keys, const uint64_t* tk, const int32_t* tv,
                                   uint32_t mask, int64_t* isfirst, int32_t* firstof) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < npairs; q += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = table_lookup(keys[q], tk, tv, mask);
    firstof[q] = f;
    isfirst[q] = (f == q) ? 1 : 0;
  }
}

__global__ void assign_kernel(PlanKParams p, int64_t npairs, const int32_t* blocksA, const int32_t* blocksB,
                              int32_t* pairs, const int64_t* isfirst, const int64_t* blockid, const int32_t* firstof,
                              const int64_t* r_blockdims, int32_t* blocksR, int64_t* sizeR) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < npairs; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t id = blockid[firstof[q]];
    pairs[3 * q + 2] = (int32_t)id;
    if (isfirst[q]) {
      int32_t c[ND_MAX_RANK];
      blockR_coords(p, blocksA + (int64_t)pairs[3 * q] * p.rankA, blocksB + (int64_t)pairs[3 * q + 1] * p.rankB, c);
      int64_t sz = 1;
      for (int r = 0; r < p.rankR; ++r) {
        blocksR[id * p.rankR + r] = c[r];
        sz *= r_blockdims[p.r_bd_off[r] + c[r] - 1];
      }
      sizeR[id] = sz;
    }
  }
}

// ---- one-CTA planner ---------------------------------------------------------
// For up to PLAN1_MAX candidate pairs the whole plan is one launch of one CTA:
// match flags and their block-wide scan compact the pairs in (A-major, B-minor)
// order, a hash table in global scratch keeps each output key's first pair, a scan
// of the first-appearance flags numbers the output blocks, and a last scan of their
// sizes gives the offsets.  Every step is a fixed-order scan, so the result does not
// depend on thread timing, and it is the same as the multi-kernel path's.
constexpr int PLAN1_THREADS = 1024;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* excl, T* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  *excl = (warp ? wsum[warp - 1] : (T)0) + x - v;
  const T total = wsum[(blockDim.x >> 5) - 1];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(PLAN1_THREADS) plan_one_cta(PlanKParams p, const int32_t* blocksA,
                                                              const int32_t* blocksB, const int64_t* rbd,
                                                              int32_t* pairs, uint64_t* keys, int32_t* firstof,
                                                              int32_t* blockid, uint64_t* tk, int32_t* tv,
                                                              uint32_t mask, int32_t* blocksR, int64_t* offsR,
                                                              int64_t* counts, DeviceStatus* st) {
  __shared__ int wsum[32];
  __shared__ long long wsum64[32];
  const int tid = threadIdx.x;
  for (uint32_t i = tid; i <= mask; i += blockDim.x) { tk[i] = ~0ull; tv[i] = 0x7fffffff; }
  // 1. contracted pairs, compacted in the reference's order
  const int64_t ncand = (int64_t)p.nA * p.nB;
  int npairs = 0;
  for (int64_t base = 0; base < ncand; base += blockDim.x) {
    const int64_t idx = base + tid;
    int flag = 0, i1 = 0, i2 = 0;
    if (idx < ncand) {
      i1 = (int)(idx / p.nB);
      i2 = (int)(idx - (int64_t)i1 * p.nB);
      const int32_t* bA = blocksA + (int64_t)i1 * p.rankA;
      const int32_t* bB = blocksB + (int64_t)i2 * p.rankB;
      flag = 1;
      for (int t = 0; t < p.nk; ++t) flag &= (bA[p.a_k[t]] == bB[p.b_k[t]]);
    }
    int ex;
    const int tot = block_exclusive_scan<int>(flag, &ex, wsum);
    if (flag) {
      const int q = npairs + ex;
      int32_t c[ND_MAX_RANK];
      blockR_coords(p, blocksA + (int64_t)i1 * p.rankA, blocksB + (int64_t)i2 * p.rankB, c);
      pairs[3 * q] = i1;
      pairs[3 * q + 1] = i2;
      keys[q] = key_of(p, c);
    }
    npairs += tot;
  }
  __syncthreads();
  // 2. the first pair of every output key
  for (int q = tid; q < npairs; q += blockDim.x) {
    const uint64_t key = keys[q];
    uint32_t hsh = hash64(key) & mask;
    bool done = false;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      const unsigned long long prev = atomicCAS((unsigned long long*)&tk[hsh], ~0ull, (unsigned long long)key);
      if (prev == ~0ull || prev == key) { atomicMin(&tv[hsh], q); done = true; break; }
      hsh = (hsh + 1) & mask;
    }
    if (!done && atomicCAS(&st->code, 0, ND_ERR_ARG) == 0) st->where = 210;
  }
  __syncthreads();
  // 3. output blocks numbered in first-appearance order, with their coordinates and sizes
  int nR = 0;
  for (int base = 0; base < npairs; base += blockDim.x) {
    const int q = base + tid;
    int first = 0;
    if (q < npairs) {
      const int f = table_lookup(keys[q], tk, tv, mask);
      firstof[q] = f;
      first = f == q;
    }
    int ex;
    const int tot = block_exclusive_scan<int>(first, &ex, wsum);
    if (first) {
      const int id = nR + ex;
      blockid[q] = id;
      int32_t c[ND_MAX_RANK];
      blockR_coords(p, blocksA + (int64_t)pairs[3 * q] * p.rankA, blocksB + (int64_t)pairs[3 * q + 1] * p.rankB, c);
      int64_t sz = 1;
      for (int r = 0; r < p.rankR; ++r) {
        blocksR[(int64_t)id * p.rankR + r] = c[r];
        sz *= rbd[p.r_bd_off[r] + c[r] - 1];
      }
      offsR[id] = sz;
    }
    nR += tot;
  }
  __syncthreads();
  // 4. each pair's output block
  for (int q = tid; q < npairs; q += blockDim.x) pairs[3 * q + 2] = blockid[firstof[q]];
  // 5. offsets: exclusive scan of the block sizes, in block order
  long long run = 0;
  for (int base = 0; base < nR; base += blockDim.x) {
    const int i = base + tid;
    const long long v = i < nR ? (long long)offsR[i] : 0ll;
    long long ex;
    const long long tot = block_exclusive_scan<long long>(v, &ex, wsum64);
    if (i < nR) offsR[i] = run + ex;
    run += tot;
  }
  if (tid == 0) { counts[0] = npairs; counts[1] = nR; counts[2] = run; }
}

}  // namespace

// Exclusive scan of n int64 values in place; *total_dev receives the sum.
nd_status nd_device_exclusive_scan(nd_handle h, int64_t* data, int64_t n, int64_t* total_dev) {
  if (n <= 0) {
    cudaMemsetAsync(total_dev, 0, sizeof(int64_t), h->stream);
    return ND_OK;
  }
  int64_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
  int64_t* sums = nullptr;
  int64_t* last = nullptr;
  ND_CUDA(h, cudaMallocAsync(&sums, (nb + 2) * sizeof(int64_t), h->stream));
  last = sums + nb;
  nd_prof_begin(h, "copy_last");
  copy_last<<<1, 32, 0, h->stream>>>(data, n, last);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  if (nb == 1) {
    nd_prof_begin(h, "scan_apply");
    scan_apply<<<1, SCAN_BLOCK, 0, h->stream>>>(data, nullptr, n);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  } else {
    nd_prof_begin(h, "scan_block_sums");
    scan_block_sums<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(data, sums, n);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    nd_status s = nd_device_exclusive_scan(h, sums, nb, sums + nb + 1);
    if (s != ND_OK) {
      cudaFreeAsync(sums, h->stream);
      return s;
    }
    nd_prof_begin(h, "scan_apply");
    scan_apply<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(data, sums, n);
    nd_prof_end(h);
    ND_LAUNCHED(h);
  }
  nd_prof_begin(h, "write_total");
  write_total<<<1, 32, 0, h->stream>>>(data, last, n, total_dev);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  ND_CUDA(h, cudaFreeAsync(sums, h->stream));
  return nd_cuda_check(h, cudaGetLastError(), "scan");
}

// Device buffers of the multi-kernel planner, released (stream-ordered) on every exit.
namespace {
struct AsyncBufs {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit AsyncBufs(cudaStream_t st) : s(st) {}
  template <typename T>
  cudaError_t alloc(T** p, size_t bytes) {
    cudaError_t e = cudaMallocAsync((void**)p, bytes, s);
    if (e == cudaSuccess) ptrs.push_back((void*)*p);
    return e;
  }
  ~AsyncBufs() { for (void* p : ptrs) cudaFreeAsync(p, s); }
};
}  // namespace

static nd_status device_plan_multi(nd_handle h, const Roles& ro, const BsDesc& A, const BsDesc& B,
                                   const std::vector<int64_t>& r_nblocks,
                                   const std::vector<std::vector<int64_t>>& r_blockdims, PlanResult& out);

static void plan_params(const Roles& ro, const BsDesc& A, const BsDesc& B, const std::vector<int64_t>& r_nblocks,
                        const std::vector<std::vector<int64_t>>& r_blockdims, PlanKParams& p, std::vector<int64_t>& rbd) {
  p = PlanKParams{};
  p.nA = A.nnzblocks; p.nB = B.nnzblocks; p.rankA = ro.rankA; p.rankB = ro.rankB; p.rankR = ro.rankR;
  p.nk = ro.nk; p.nfa = ro.nfa; p.nfb = ro.nfb;
  for (int t = 0; t < ro.nk; ++t) { p.a_k[t] = ro.a_k[t]; p.b_k[t] = ro.b_k[t]; }
  for (int t = 0; t < ro.nfa; ++t) { p.a_free[t] = ro.a_free[t]; p.r_afree[t] = ro.r_afree[t]; }
  for (int t = 0; t < ro.nfb; ++t) { p.b_free[t] = ro.b_free[t]; p.r_bfree[t] = ro.r_bfree[t]; }
  rbd.clear();
  for (int r = 0; r < ro.rankR; ++r) {
    p.r_nblocks[r] = r_nblocks[r];
    p.r_bd_off[r] = (int32_t)rbd.size();
    rbd.insert(rbd.end(), r_blockdims[r].begin(), r_blockdims[r].end());
  }
  if (rbd.empty()) rbd.push_back(1);
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---- host planner --------------------------------------------------------------
// The same plan from the same block lists, built on the CPU.  A plan is integer
// bookkeeping over a few hundred blocks; on the GPU it costs a launch and a
// synchronisation that, inside a sweep, wait for SMs held by the contraction kernels
// already queued (about 0.09 ms per plan on the chi = 4096 matvec), while here it is a
// sort of B's blocks by their contracted block numbers and one walk over the pairs.
// B blocks in a bucket keep ascending order and A blocks are walked in order, so the
// pairs come out in the reference's (A-major, B-minor) order; output blocks are
// numbered at their first pair, as the device planner's first-appearance scan does.
// Returns false, leaving `out` empty, when the plan has more than max_pairs pairs or
// the contracted block numbers do not fit a 64-bit key (the device planner then runs).
static bool host_plan(const Roles& ro, const BsDesc& A, const BsDesc& B, const std::vector<int64_t>& r_nblocks,
                      const std::vector<std::vector<int64_t>>& r_blockdims, int64_t max_pairs, PlanResult& out) {
  const int nA = A.nnzblocks, nB = B.nnzblocks, rankR = ro.rankR;
  // contracted block numbers of a block as one mixed-radix key (radix: A's block counts)
  uint64_t mul[ND_MAX_RANK];
  {
    long double ks = 1;
    for (int t = 0; t < ro.nk; ++t) {
      mul[t] = (uint64_t)ks;
      ks *= (long double)A.nblocks[ro.a_k[t]];
    }
    if (ks > 9.0e18L) return false;
  }
  std::vector<std::pair<uint64_t, int32_t>> kb;
  kb.reserve(nB);
  for (int i2 = 0; i2 < nB; ++i2) {
    const int32_t* bB = B.blocks + (size_t)i2 * ro.rankB;
    uint64_t k = 0;
    bool ok = true;
    for (int t = 0; t < ro.nk; ++t) {
      const int32_t v = bB[ro.b_k[t]];
      if (v > A.nblocks[ro.a_k[t]]) { ok = false; break; }     // no A block has this number
      k += (uint64_t)(v - 1) * mul[t];
    }
    if (ok) kb.push_back({k, i2});
  }
  std::sort(kb.begin(), kb.end());
  std::vector<std::pair<int32_t, int32_t>> bucket(nA, {0, 0});  // each A block's matching range of kb
  int64_t npairs = 0;
  for (int i1 = 0; i1 < nA; ++i1) {
    const int32_t* bA = A.blocks + (size_t)i1 * ro.rankA;
    uint64_t k = 0;
    for (int t = 0; t < ro.nk; ++t) k += (uint64_t)(bA[ro.a_k[t]] - 1) * mul[t];
    auto lo = std::lower_bound(kb.begin(), kb.end(), std::make_pair(k, (int32_t)INT32_MIN));
    auto hi = lo;
    while (hi != kb.end() && hi->first == k) ++hi;
    bucket[i1] = {(int32_t)(lo - kb.begin()), (int32_t)(hi - kb.begin())};
    npairs += hi - lo;
    if (npairs > max_pairs) return false;
  }
  out = PlanResult{};
  out.pairs.resize((size_t)npairs * 3);
  std::unordered_map<uint64_t, int32_t> ids;
  ids.reserve((size_t)npairs * 2 + 1);
  std::vector<int64_t> sizes;
  int64_t q = 0;
  for (int i1 = 0; i1 < nA; ++i1) {
    const int32_t* bA = A.blocks + (size_t)i1 * ro.rankA;
    for (int32_t j = bucket[i1].first; j < bucket[i1].second; ++j) {
      const int32_t i2 = kb[j].second;
      const int32_t* bB = B.blocks + (size_t)i2 * ro.rankB;
      int32_t c[ND_MAX_RANK];
      for (int t = 0; t < ro.nfa; ++t) c[ro.r_afree[t]] = bA[ro.a_free[t]];
      for (int t = 0; t < ro.nfb; ++t) c[ro.r_bfree[t]] = bB[ro.b_free[t]];
      uint64_t key = 0, m = 1;
      for (int r = 0; r < rankR; ++r) { key += (uint64_t)(c[r] - 1) * m; m *= (uint64_t)r_nblocks[r]; }
      auto ins = ids.emplace(key, out.nR);
      if (ins.second) {
        int64_t sz = 1;
        for (int r = 0; r < rankR; ++r) {
          out.blocksR.push_back(c[r]);
          sz *= r_blockdims[r][c[r] - 1];
        }
        sizes.push_back(sz);
        ++out.nR;
      }
      out.pairs[3 * q] = i1;
      out.pairs[3 * q + 1] = i2;
      out.pairs[3 * q + 2] = ins.first->second;
      ++q;
    }
  }
  out.npairs = (int32_t)npairs;
  out.offsetsR.resize(out.nR);
  int64_t run = 0;
  for (int32_t g = 0; g < out.nR; ++g) { out.offsetsR[g] = run; run += sizes[g]; }
  out.nnzR = run;
  return true;
}

// Plans of up to this many pairs are built on the host when the placement is by size.
// The host planner takes about 0.1 us per pair here, one device round trip 0.03-0.1 ms.
constexpr int64_t kHostPlanMax = 4096;

nd_status nd_block_plan(nd_handle h, const Roles& ro, const BsDesc& A, const BsDesc& B,
                        const std::vector<int64_t>& r_nblocks, const std::vector<std::vector<int64_t>>& r_blockdims,
                        PlanResult& out) {
  const int nA = A.nnzblocks, nB = B.nnzblocks, rankR = ro.rankR;
  out = PlanResult{};
  const int64_t ncand = (int64_t)nA * nB;
  if (ncand == 0) return ND_OK;
  if (ncand > (int64_t)INT_MAX) return nd_fail(h, ND_ERR_UNSUPPORTED, "plan: %lld candidate pairs exceed 2^31", (long long)ncand);
  // key space must fit 64 bits
  {
    long double ks = 1;
    for (int r = 0; r < rankR; ++r) ks *= (long double)r_nblocks[r];
    if (ks > 1.8e19L) return nd_fail(h, ND_ERR_UNSUPPORTED, "plan: output block space exceeds 2^64");
  }
  if (h->plan_where != 1) {
    const int64_t host_max = h->plan_where == 2 ? (int64_t)INT_MAX : kHostPlanMax;
    if (host_plan(ro, A, B, r_nblocks, r_blockdims, host_max, out)) return ND_OK;
    out = PlanResult{};
  }
  if (ncand > PLAN1_MAX || nd_capturing(h)) return device_plan_multi(h, ro, A, B, r_nblocks, r_blockdims, out);
  PlanKParams p;
  std::vector<int64_t> rbd;
  plan_params(ro, A, B, r_nblocks, r_blockdims, p, rbd);
  // one device buffer: inputs (block lists, R block dims) | scratch | results (counts, pairs, blocksR, offsets)
  uint32_t tsize = 1;
  while (tsize < 2 * (uint64_t)ncand) tsize <<= 1;
  const size_t szA = (size_t)nA * ro.rankA * 4, szB = (size_t)nB * ro.rankB * 4, szR = rbd.size() * 8;
  const size_t o_A = 0, o_B = al256(o_A + szA), o_rbd = al256(o_B + szB), in_bytes = al256(o_rbd + szR);
  const size_t o_keys = in_bytes, o_first = al256(o_keys + ncand * 8), o_bid = al256(o_first + ncand * 4);
  const size_t o_tk = al256(o_bid + ncand * 4), o_tv = al256(o_tk + (size_t)tsize * 8);
  const size_t o_out = al256(o_tv + (size_t)tsize * 4);
  const size_t r_counts = 0, r_pairs = 32, r_blocks = al256(r_pairs + ncand * 12);
  const size_t r_offs = al256(r_blocks + ncand * rankR * 4), out_bytes = r_offs + ncand * 8;
  if (!h->plan_stream) {
    ND_CUDA(h, cudaStreamCreateWithFlags(&h->plan_stream, cudaStreamNonBlocking));
    ND_CUDA(h, cudaMalloc(&h->d_plan_status, sizeof(DeviceStatus)));
    const DeviceStatus init{0, 0, ND_SPIN_LIMIT, 0};
    ND_CUDA(h, cudaMemcpy(h->d_plan_status, &init, sizeof(init), cudaMemcpyHostToDevice));
  }
  cudaStream_t st = h->plan_stream;
  // the workspace and the pinned staging buffer belong to the planner alone, and every
  // plan waits for its own work before returning, so growing them needs no other sync
  if (o_out + out_bytes > h->ws_size) {
    if (h->ws) { ND_CUDA(h, cudaFree(h->ws)); h->ws = nullptr; h->ws_size = 0; }
    const size_t sz = std::max(o_out + out_bytes, h->ws_size * 3 / 2);
    ND_CUDA(h, cudaMalloc(&h->ws, sz));
    h->ws_size = sz;
  }
  unsigned char* d = (unsigned char*)h->ws;
  const size_t pin_need = std::max(in_bytes, out_bytes) + sizeof(DeviceStatus);
  if (h->pin_size < pin_need) {
    if (h->pin) { cudaFreeHost(h->pin); h->pin = nullptr; h->pin_size = 0; }
    const size_t sz = std::max<size_t>(pin_need, 1 << 16);
    ND_CUDA(h, cudaHostAlloc(&h->pin, sz, cudaHostAllocDefault));
    h->pin_size = sz;
  }
  nd_status s = ND_OK;
  unsigned char* hp = (unsigned char*)h->pin;
  if (szA) memcpy(hp + o_A, A.blocks, szA);
  if (szB) memcpy(hp + o_B, B.blocks, szB);
  memcpy(hp + o_rbd, rbd.data(), szR);
  ND_CUDA(h, cudaMemcpyAsync(d, hp, in_bytes, cudaMemcpyHostToDevice, st));
  unsigned char* r = d + o_out;
  plan_one_cta<<<1, PLAN1_THREADS, 0, st>>>(p, (const int32_t*)(d + o_A), (const int32_t*)(d + o_B),
                                            (const int64_t*)(d + o_rbd), (int32_t*)(r + r_pairs),
                                            (uint64_t*)(d + o_keys), (int32_t*)(d + o_first), (int32_t*)(d + o_bid),
                                            (uint64_t*)(d + o_tk), (int32_t*)(d + o_tv), tsize - 1,
                                            (int32_t*)(r + r_blocks), (int64_t*)(r + r_offs), (int64_t*)(r + r_counts),
                                            h->d_plan_status);
  ND_LAUNCHED(h);
  ND_CUDA(h, cudaGetLastError());
  // results: in one copy when the bound is small, else the counts first and then exact sizes
  int64_t counts[3];
  const bool one_copy = out_bytes <= (1u << 20);
  DeviceStatus* hst = (DeviceStatus*)(hp + pin_need - sizeof(DeviceStatus));
  ND_CUDA(h, cudaMemcpyAsync(hp, r, one_copy ? out_bytes : 32, cudaMemcpyDeviceToHost, st));
  ND_CUDA(h, cudaMemcpyAsync(hst, h->d_plan_status, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, st));
  ND_CUDA(h, cudaStreamSynchronize(st));
  if (hst->code != ND_OK) {
    const int32_t code = hst->code, where = hst->where;
    const int32_t z[2] = {0, 0};
    cudaMemcpy(h->d_plan_status, z, sizeof(z), cudaMemcpyHostToDevice);
    return nd_fail(h, code, "block plan: device reported error %d at site %d", code, where);
  }
  memcpy(counts, hp + r_counts, sizeof counts);
  const int64_t npairs = counts[0], nR = counts[1];
  if (!one_copy && npairs > 0) {
    ND_CUDA(h, cudaMemcpyAsync(hp + r_pairs, r + r_pairs, npairs * 12, cudaMemcpyDeviceToHost, st));
    ND_CUDA(h, cudaMemcpyAsync(hp + r_blocks, r + r_blocks, nR * rankR * 4, cudaMemcpyDeviceToHost, st));
    ND_CUDA(h, cudaMemcpyAsync(hp + r_offs, r + r_offs, nR * 8, cudaMemcpyDeviceToHost, st));
    ND_CUDA(h, cudaStreamSynchronize(st));
  }
  out.npairs = (int32_t)npairs;
  out.nR = (int32_t)nR;
  out.nnzR = counts[2];
  out.pairs.assign((const int32_t*)(hp + r_pairs), (const int32_t*)(hp + r_pairs) + npairs * 3);
  out.blocksR.assign((const int32_t*)(hp + r_blocks), (const int32_t*)(hp + r_blocks) + nR * rankR);
  out.offsetsR.assign((const int64_t*)(hp + r_offs), (const int64_t*)(hp + r_offs) + nR);
  return ND_OK;
}

// Plans with more than PLAN1_MAX candidate pairs: the same steps as plan_one_cta, one
// grid-wide launch each, with device-wide scans.
static nd_status device_plan_multi(nd_handle h, const Roles& ro, const BsDesc& A, const BsDesc& B,
                                   const std::vector<int64_t>& r_nblocks,
                                   const std::vector<std::vector<int64_t>>& r_blockdims, PlanResult& out) {
  const int nA = A.nnzblocks, nB = B.nnzblocks, rankR = ro.rankR;
  const int64_t ncand = (int64_t)nA * nB;
  PlanKParams p;
  std::vector<int64_t> rbd;
  plan_params(ro, A, B, r_nblocks, r_blockdims, p, rbd);
  cudaStream_t s = h->stream;
  AsyncBufs bufs(s);      // every buffer below is released on return, error paths included
  int32_t *dA = nullptr, *dB = nullptr, *pairs = nullptr, *tv = nullptr, *firstof = nullptr, *blocksR = nullptr;
  int64_t *flags = nullptr, *isfirst = nullptr, *sizeR = nullptr, *tot = nullptr, *rbd_d = nullptr;
  uint64_t *keys = nullptr, *tk = nullptr;
  size_t szA = std::max<size_t>(1, (size_t)nA * ro.rankA), szB = std::max<size_t>(1, (size_t)nB * ro.rankB);
  ND_CUDA(h, bufs.alloc(&dA, szA * 4));
  ND_CUDA(h, bufs.alloc(&dB, szB * 4));
  ND_CUDA(h, bufs.alloc(&flags, ncand * 8));
  ND_CUDA(h, bufs.alloc(&tot, 4 * 8));
  ND_CUDA(h, bufs.alloc(&rbd_d, rbd.size() * 8));
  if (nA * (size_t)ro.rankA) ND_CUDA(h, cudaMemcpyAsync(dA, A.blocks, (size_t)nA * ro.rankA * 4, cudaMemcpyHostToDevice, s));
  if (nB * (size_t)ro.rankB) ND_CUDA(h, cudaMemcpyAsync(dB, B.blocks, (size_t)nB * ro.rankB * 4, cudaMemcpyHostToDevice, s));
  ND_CUDA(h, cudaMemcpyAsync(rbd_d, rbd.data(), rbd.size() * 8, cudaMemcpyHostToDevice, s));
  const int threads = 256;
  int grid = (int)std::min<int64_t>((ncand + threads - 1) / threads, (int64_t)h->num_sms * 16);
  nd_prof_begin(h, "match_kernel");
  match_kernel<<<grid, threads, 0, s>>>(p, dA, dB, flags);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  // positions = exclusive scan of flags (kept in a copy: flags still needed)
  int64_t* pos = nullptr;
  ND_CUDA(h, bufs.alloc(&pos, ncand * 8));
  ND_CUDA(h, cudaMemcpyAsync(pos, flags, ncand * 8, cudaMemcpyDeviceToDevice, s));
  nd_status stt = nd_device_exclusive_scan(h, pos, ncand, tot);
  if (stt != ND_OK) return stt;
  int64_t npairs = 0;
  ND_CUDA(h, cudaMemcpyAsync(&npairs, tot, 8, cudaMemcpyDeviceToHost, s));
  ND_CUDA(h, cudaStreamSynchronize(s));
  out.npairs = (int32_t)npairs;
  if (npairs > 0) {
    uint32_t tsize = 1;
    while (tsize < 2 * (uint64_t)npairs) tsize <<= 1;
    const uint32_t mask = tsize - 1;
    ND_CUDA(h, bufs.alloc(&pairs, npairs * 3 * 4));
    ND_CUDA(h, bufs.alloc(&keys, npairs * 8));
    ND_CUDA(h, bufs.alloc(&tk, (size_t)tsize * 8));
    ND_CUDA(h, bufs.alloc(&tv, (size_t)tsize * 4));
    ND_CUDA(h, bufs.alloc(&isfirst, npairs * 8));
    ND_CUDA(h, bufs.alloc(&firstof, npairs * 4));
    ND_CUDA(h, cudaMemsetAsync(tk, 0xff, (size_t)tsize * 8, s));
    ND_CUDA(h, cudaMemsetAsync(tv, 0x7f, (size_t)tsize * 4, s));
    nd_prof_begin(h, "compact_kernel");
    compact_kernel<<<grid, threads, 0, s>>>(p, dA, dB, flags, pos, pairs, keys, tk, tv, mask, h->d_status);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    int pg = (int)std::min<int64_t>((npairs + threads - 1) / threads, (int64_t)h->num_sms * 16);
    nd_prof_begin(h, "first_flags_kernel");
    first_flags_kernel<<<pg, threads, 0, s>>>(npairs, keys, tk, tv, mask, isfirst, firstof);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    // block ids = exclusive scan of first-appearance flags
    int64_t* blockid = nullptr;
    ND_CUDA(h, bufs.alloc(&blockid, npairs * 8));
    ND_CUDA(h, cudaMemcpyAsync(blockid, isfirst, npairs * 8, cudaMemcpyDeviceToDevice, s));
    stt = nd_device_exclusive_scan(h, blockid, npairs, tot + 1);
    if (stt != ND_OK) return stt;
    int64_t nR = 0;
    ND_CUDA(h, cudaMemcpyAsync(&nR, tot + 1, 8, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaStreamSynchronize(s));
    out.nR = (int32_t)nR;
    ND_CUDA(h, bufs.alloc(&blocksR, std::max<int64_t>(1, nR * rankR) * 4));
    ND_CUDA(h, bufs.alloc(&sizeR, std::max<int64_t>(1, nR) * 8));
    nd_prof_begin(h, "assign_kernel");
    assign_kernel<<<pg, threads, 0, s>>>(p, npairs, dA, dB, pairs, isfirst, blockid, firstof, rbd_d, blocksR, sizeR);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    stt = nd_device_exclusive_scan(h, sizeR, nR, tot + 2);
    if (stt != ND_OK) return stt;
    out.pairs.resize(npairs * 3);
    out.blocksR.resize(nR * rankR);
    out.offsetsR.resize(nR);
    ND_CUDA(h, cudaMemcpyAsync(out.pairs.data(), pairs, npairs * 3 * 4, cudaMemcpyDeviceToHost, s));
    if (nR * rankR) ND_CUDA(h, cudaMemcpyAsync(out.blocksR.data(), blocksR, nR * rankR * 4, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaMemcpyAsync(out.offsetsR.data(), sizeR, nR * 8, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaMemcpyAsync(&out.nnzR, tot + 2, 8, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaStreamSynchronize(s));
  }
  ND_CUDA(h, cudaGetLastError());
  return nd_check_device_status(h, "block plan");
}
