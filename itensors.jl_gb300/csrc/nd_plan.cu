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

namespace {

constexpr int SCAN_BLOCK = 1024;

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
    if (s != ND_OK) return s;
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

nd_status nd_device_plan(nd_handle h, const Roles& ro, const BsDesc& A, const BsDesc& B,
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
  PlanKParams p{};
  p.nA = nA; p.nB = nB; p.rankA = ro.rankA; p.rankB = ro.rankB; p.rankR = rankR;
  p.nk = ro.nk; p.nfa = ro.nfa; p.nfb = ro.nfb;
  for (int t = 0; t < ro.nk; ++t) { p.a_k[t] = ro.a_k[t]; p.b_k[t] = ro.b_k[t]; }
  for (int t = 0; t < ro.nfa; ++t) { p.a_free[t] = ro.a_free[t]; p.r_afree[t] = ro.r_afree[t]; }
  for (int t = 0; t < ro.nfb; ++t) { p.b_free[t] = ro.b_free[t]; p.r_bfree[t] = ro.r_bfree[t]; }
  std::vector<int64_t> rbd;
  for (int r = 0; r < rankR; ++r) {
    p.r_nblocks[r] = r_nblocks[r];
    p.r_bd_off[r] = (int32_t)rbd.size();
    rbd.insert(rbd.end(), r_blockdims[r].begin(), r_blockdims[r].end());
  }
  if (rbd.empty()) rbd.push_back(1);
  cudaStream_t s = h->stream;
  // device buffers
  int32_t *dA = nullptr, *dB = nullptr, *pairs = nullptr, *tv = nullptr, *firstof = nullptr, *blocksR = nullptr;
  int64_t *flags = nullptr, *isfirst = nullptr, *sizeR = nullptr, *tot = nullptr, *rbd_d = nullptr;
  uint64_t *keys = nullptr, *tk = nullptr;
  size_t szA = std::max<size_t>(1, (size_t)nA * ro.rankA), szB = std::max<size_t>(1, (size_t)nB * ro.rankB);
  ND_CUDA(h, cudaMallocAsync(&dA, szA * 4, s));
  ND_CUDA(h, cudaMallocAsync(&dB, szB * 4, s));
  ND_CUDA(h, cudaMallocAsync(&flags, ncand * 8, s));
  ND_CUDA(h, cudaMallocAsync(&tot, 4 * 8, s));
  ND_CUDA(h, cudaMallocAsync(&rbd_d, rbd.size() * 8, s));
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
  ND_CUDA(h, cudaMallocAsync(&pos, ncand * 8, s));
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
    ND_CUDA(h, cudaMallocAsync(&pairs, npairs * 3 * 4, s));
    ND_CUDA(h, cudaMallocAsync(&keys, npairs * 8, s));
    ND_CUDA(h, cudaMallocAsync(&tk, (size_t)tsize * 8, s));
    ND_CUDA(h, cudaMallocAsync(&tv, (size_t)tsize * 4, s));
    ND_CUDA(h, cudaMallocAsync(&isfirst, npairs * 8, s));
    ND_CUDA(h, cudaMallocAsync(&firstof, npairs * 4, s));
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
    ND_CUDA(h, cudaMallocAsync(&blockid, npairs * 8, s));
    ND_CUDA(h, cudaMemcpyAsync(blockid, isfirst, npairs * 8, cudaMemcpyDeviceToDevice, s));
    stt = nd_device_exclusive_scan(h, blockid, npairs, tot + 1);
    if (stt != ND_OK) return stt;
    int64_t nR = 0;
    ND_CUDA(h, cudaMemcpyAsync(&nR, tot + 1, 8, cudaMemcpyDeviceToHost, s));
    ND_CUDA(h, cudaStreamSynchronize(s));
    out.nR = (int32_t)nR;
    ND_CUDA(h, cudaMallocAsync(&blocksR, std::max<int64_t>(1, nR * rankR) * 4, s));
    ND_CUDA(h, cudaMallocAsync(&sizeR, std::max<int64_t>(1, nR) * 8, s));
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
    cudaFreeAsync(pairs, s); cudaFreeAsync(keys, s); cudaFreeAsync(tk, s); cudaFreeAsync(tv, s);
    cudaFreeAsync(isfirst, s); cudaFreeAsync(firstof, s); cudaFreeAsync(blockid, s);
    cudaFreeAsync(blocksR, s); cudaFreeAsync(sizeR, s);
  }
  cudaFreeAsync(dA, s); cudaFreeAsync(dB, s); cudaFreeAsync(flags, s); cudaFreeAsync(pos, s);
  cudaFreeAsync(tot, s); cudaFreeAsync(rbd_d, s);
  ND_CUDA(h, cudaGetLastError());
  return nd_check_device_status(h, "block plan");
}
