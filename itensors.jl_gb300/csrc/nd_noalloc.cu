// Dense contraction in Ozaki precision that performs no device allocation.
//
// Who needs it: callers that cannot call cudaMalloc at the moment they contract.
// Typical cases are applications whose device memory is owned by another
// allocator with a hard budget (for example a Julia or PyTorch caching pool
// that has already reserved the GPU), and latency-sensitive loops where the
// synchronisation and possible failure of cudaMalloc / cudaFree inside the
// call are not acceptable.  The regular entry point allocates its split-operand
// scratch per call; this one uses a fixed device array instead.
//
// The scratch is a file-scope __device__ array of ND_NOALLOC_SCRATCH_BYTES
// (32 MiB).  Every GPU that loads this library holds it until the process
// exits.  Its device address is looked up once per device, on the first call
// made with a handle on that device (that device is made current for the
// lookup); make that first call before any stream capture.  Every call uploads
// its descriptors from host memory and waits for its own work to finish, so a
// call made while the handle's stream is being captured is refused with
// ND_ERR_ARG instead of being recorded into the caller's graph.  Problems whose
// split operands, descriptors and exponents need more than the array holds are
// rejected with ND_ERR_ARG and a message giving the size.
//
// Every call reuses the same array, which keeps the previous call's contents:
// the per-row maxima are cleared at the start of each call and everything else
// is overwritten before it is read.  Two calls whose GPU work overlaps (for
// example on two streams or two handles of the same device) race on the array;
// serialise them.
#include "nd_plan.h"
#include <mutex>

#define ND_NOALLOC_SCRATCH_BYTES (32u << 20)

static __device__ __align__(256) unsigned char nd_noalloc_scratch[ND_NOALLOC_SCRATCH_BYTES];

nd_status nd_split_layout_into(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs_in, int S,
                               unsigned char* base, size_t capacity, size_t* needed);
nd_status nd_split_run(nd_handle h, ExecCache& c, const JobPtrs& ptrs, double alpha, double beta);

namespace {
std::mutex g_scratch_mu;
unsigned char* g_scratch_addr[128] = {};

// Device address of the scratch array on the handle's device (looked up once per device).
nd_status scratch_address(nd_handle h, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (h->device < 0 || h->device >= 128) return nd_fail(h, ND_ERR_UNSUPPORTED, "noalloc: device ordinal %d", h->device);
  if (!g_scratch_addr[h->device]) {
    int prev = 0;
    ND_CUDA(h, cudaGetDevice(&prev));
    ND_CUDA(h, cudaSetDevice(h->device));
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, nd_noalloc_scratch);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return nd_cuda_check(h, e, "cudaGetSymbolAddress(nd_noalloc_scratch)");
    g_scratch_addr[h->device] = (unsigned char*)p;
  }
  *out = g_scratch_addr[h->device];
  return ND_OK;
}
}  // namespace

extern "C" nd_status nd_contract_dense_ozaki_noalloc_f64(nd_handle h,
                                                         double* R, int32_t rankR, const int64_t* dimsR,
                                                         const int32_t* labelsR, const double* A, int32_t rankA,
                                                         const int64_t* dimsA, const int32_t* labelsA,
                                                         const double* B, int32_t rankB, const int64_t* dimsB,
                                                         const int32_t* labelsB, double alpha, double beta) {
  if (!h) return ND_ERR_ARG;
  if (nd_capturing(h))
    return nd_fail(h, ND_ERR_ARG, "noalloc contract: the handle's stream is being captured; this entry point uploads "
                                  "host descriptors and synchronises, call it outside the capture");
  if (rankA < 0 || rankB < 0 || rankR < 0 || rankA > ND_MAX_RANK || rankB > ND_MAX_RANK || rankR > ND_MAX_RANK)
    return nd_fail(h, ND_ERR_ARG, "noalloc contract: rank out of range (max %d)", ND_MAX_RANK);
  int64_t nA = 1, nB = 1, nR = 1;
  for (int k = 0; k < rankA; ++k) { if (dimsA[k] < 0) return nd_fail(h, ND_ERR_ARG, "noalloc contract: negative dim"); nA *= dimsA[k]; }
  for (int k = 0; k < rankB; ++k) { if (dimsB[k] < 0) return nd_fail(h, ND_ERR_ARG, "noalloc contract: negative dim"); nB *= dimsB[k]; }
  for (int k = 0; k < rankR; ++k) { if (dimsR[k] < 0) return nd_fail(h, ND_ERR_ARG, "noalloc contract: negative dim"); nR *= dimsR[k]; }
  if (nR == 0) return ND_OK;
  if ((nA && !A) || (nB && !B) || !R) return nd_fail(h, ND_ERR_ARG, "noalloc contract: NULL data pointer");
  // A one-element operand is the reference's scalar branch: a scaled permutation,
  // which the regular entry point runs without any scratch.
  if (nA == 1 || nB == 1)
    return nd_contract_dense_f64(h, R, rankR, dimsR, labelsR, A, rankA, dimsA, labelsA, B, rankB, dimsB, labelsB,
                                 alpha, beta, ND_PREC_FP64);
  Roles ro;
  std::string why;
  if (!nd_make_roles(rankA, labelsA, rankB, labelsB, rankR, labelsR, ro, why))
    return nd_fail(h, ND_ERR_ARG, "noalloc contract: %s", why.c_str());
  PairDesc pd;
  if (!nd_make_pair(ro, dimsA, dimsB, dimsR, pd, why)) return nd_fail(h, ND_ERR_ARG, "noalloc contract: %s", why.c_str());
  pd.group = 0; pd.first = 1; pd.job = 0; pd.a_op = 0; pd.b_op = 0;
  if (pd.K == 0) {   // empty contraction: R = beta * R
    int64_t n = nR; int p0 = 0;
    return nd_launch_permute(h, R, R, 1, &n, &p0, 0.0, beta, nullptr);
  }
  unsigned char* scratch = nullptr;
  nd_status s = scratch_address(h, &scratch);
  if (s) return s;
  std::vector<PairDesc> pairs{pd};
  ExecCache c;                     // fields point into the scratch array; nothing here is freed
  size_t needed = 0;
  s = nd_split_layout_into(h, c, pairs, h->ozaki_slices, nullptr, 0, &needed);
  if (s) return s;
  if (needed > ND_NOALLOC_SCRATCH_BYTES)
    return nd_fail(h, ND_ERR_ARG,
                   "noalloc contract: this contraction needs %zu bytes of scratch; the allocation-free entry point "
                   "holds at most %u bytes (use nd_contract_dense_f64)", needed, (unsigned)ND_NOALLOC_SCRATCH_BYTES);
  s = nd_split_layout_into(h, c, pairs, h->ozaki_slices, scratch, ND_NOALLOC_SCRATCH_BYTES, &needed);
  if (s) return s;
  JobPtrs ptrs{{A, nullptr}, {B, nullptr}, {R, nullptr}};
  s = nd_split_run(h, c, ptrs, alpha, beta);
  if (s) return s;
  return nd_check_device_status(h, "noalloc contract");   // synchronises the stream
}
