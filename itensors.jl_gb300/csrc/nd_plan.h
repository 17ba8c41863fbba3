// Internal: block-sparse descriptors, the device planner and the plan object.
#pragma once
#include "nd_common.h"

// Host-side validated copy of an nd_bs_desc.
struct BsDesc {
  int rank = 0;
  int nnzblocks = 0;
  std::vector<int32_t> nblocks;                   // per dim
  std::vector<std::vector<int64_t>> blockdims;    // per dim, per block number
  const int32_t* blocks = nullptr;                // points into `blocks_store`
  std::vector<int32_t> blocks_store;              // [nnzblocks][rank]
  std::vector<int64_t> offsets;                   // [nnzblocks]
  int64_t block_elems(int b) const {
    int64_t n = 1;
    for (int d = 0; d < rank; ++d) n *= blockdims[d][blocks_store[(size_t)b * rank + d] - 1];
    return n;
  }
  int64_t bdim(int b, int d) const { return blockdims[d][blocks_store[(size_t)b * rank + d] - 1]; }
};

nd_status nd_bs_import(nd_handle h, const nd_bs_desc* in, BsDesc& out, const char* name);

struct PlanResult {
  int32_t npairs = 0;
  int32_t nR = 0;
  int64_t nnzR = 0;
  std::vector<int32_t> pairs;     // [npairs][3] (iA, iB, iR)
  std::vector<int32_t> blocksR;   // [nR][rankR]
  std::vector<int64_t> offsetsR;  // [nR]
};

nd_status nd_device_exclusive_scan(nd_handle h, int64_t* data, int64_t n, int64_t* total_dev);
// The block plan of A x B: on the host up to a few thousand pairs, else on the device
// (nd_set_plan_placement overrides the choice); both give the same plan.
nd_status nd_block_plan(nd_handle h, const Roles& ro, const BsDesc& A, const BsDesc& B,
                        const std::vector<int64_t>& r_nblocks,
                        const std::vector<std::vector<int64_t>>& r_blockdims, PlanResult& out);

// Device-resident execution state of one contraction (built once, reused by
// every call and by captured graphs).
struct ExecCache {
  bool built = false;
  int precision = -1;
  int slices = 0;
  PairDesc* d_pairs = nullptr;
  WorkItem* d_items = nullptr;     // FP64 tensor-core tiles of the regular groups
  int nitems = 0;
  double* d_ws = nullptr;          // split-K partial tiles: FP64 (DMMA path) or int64 fixed point (split GEMM)
  ReduceItem* d_red = nullptr;     // output tiles summed from the partials
  int nred = 0;
  WorkItem* d_sk_items = nullptr;  // skinny groups (FP64 CUDA-core kernel, every precision)
  int nsk_items = 0;
  // split-precision operands (regular groups only)
  PairDesc* d_split_pairs = nullptr;
  WorkItem* d_split_items = nullptr;
  int nsplit_items = 0;
  void* d_operands = nullptr;      // OperandDesc[nops]
  int nops_a = 0, nops_b = 0;
  void* d_pack = nullptr;          // packed slices (bytes)
  size_t pack_bytes = 0;
  int32_t* d_exp = nullptr;        // per-row exponents
  size_t exp_count = 0;
  void* d_pack_items = nullptr;    // pack work list
  int npack_items = 0;
  void* d_rowmax = nullptr;        // per-row |x| maxima (IEEE bits) of the split operands
  int split_pair2 = 0;             // 1: split GEMM on CTA pairs (256 x 64 tiles)
  int req_pair2 = -1;              // the handle's untuned tile shape when this state was built
  int split_slots = 0;             // persistent CTAs / CTA pairs of the split GEMM
  cudaStream_t stream = nullptr;   // stream of the last work that used this state
  // Release every buffer, stream-ordered on the handle's stream (after a device-wide
  // synchronisation when the state was last used on another stream).
  void free_all(nd_handle h);
};

struct nd_bs_plan_s {
  nd_handle h = nullptr;
  Roles roles{};
  BsDesc A, B;
  int rankR = 0;
  std::vector<int32_t> labelsA, labelsB, labelsR;
  std::vector<int64_t> r_nblocks;
  std::vector<std::vector<int64_t>> r_blockdims;
  PlanResult res;
  // grouped pair descriptors, sorted by output block, built on first use
  std::vector<PairDesc> descs;
  int ngroups = 0;
  ExecCache cache[3];
  // adjoint
  bool adj_built = false;
  std::vector<PairDesc> adj_descs;
  int adj_ngroups = 0;
  ExecCache adj_cache[3];
};

// Build the PairDesc of one block pair.
bool nd_make_pair(const Roles& ro, const int64_t* dA, const int64_t* dB, const int64_t* dR, PairDesc& pd,
                  std::string& why);

bool nd_pair_is_skinny(const PairDesc& p);
int nd_skinny_rows();
nd_status nd_launch_skinny_f64(nd_handle h, const PairDesc* d_pairs, const WorkItem* d_items, int nitems,
                               const JobPtrs& ptrs, double alpha, double beta);

// Execute grouped pairs with a cache (built on first call, outside capture).
nd_status nd_execute_cached(nd_handle h, ExecCache& cache, const std::vector<PairDesc>& pairs, int ngroups,
                            const JobPtrs& ptrs, double alpha, double beta, int precision);
