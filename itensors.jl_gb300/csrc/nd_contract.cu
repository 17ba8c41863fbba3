// Contraction drivers: dense contract!, block-sparse plan / contract / adjoint,
// block-sparse permutedims.  Host-side C++; all arithmetic runs in the kernels.
//
// Reference behaviour reproduced here:
//   dense contract!  NDTensors/src/dense/tensoralgebra/contract.jl:160-216
//     - one-element operand -> scalar branch (drop singleton dims, permute, scale; :100-150)
//     - otherwise one GEMM with the permutations folded into addressing
//   block-sparse     NDTensors/src/blocksparse/contract.jl:3-76, contract_generic.jl:37-129
//     - plan on device (nd_plan.cu), pairs grouped by output block in R's block order,
//       first pair of a group overwrites, the rest accumulate
//   adjoint          ext/ITensorsChainRulesCoreExt/itensor.jl:94-103
#include "nd_plan.h"
#include <algorithm>
#include <numeric>
#include <cstring>
#include <map>
#include <string>
#include <new>
#include <climits>
#include <cmath>

nd_status nd_split_build(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs, int ngroups, int precision,
                         int pair2);
nd_status nd_split_run(nd_handle h, ExecCache& c, const JobPtrs& ptrs, double alpha, double beta);

void ExecCache::free_all(nd_handle h) {
  if (stream && stream != h->stream) cudaDeviceSynchronize();
  for (void* p : {(void*)d_pairs, (void*)d_items, d_operands, d_pack, (void*)d_exp, d_pack_items, d_rowmax,
                  (void*)d_sk_items, (void*)d_split_pairs, (void*)d_split_items, (void*)d_ws, (void*)d_red})
    if (p) cudaFreeAsync(p, h->stream);
  *this = ExecCache{};
}

nd_status nd_bs_import(nd_handle h, const nd_bs_desc* in, BsDesc& out, const char* name) {
  if (!in) return nd_fail(h, ND_ERR_ARG, "%s: NULL descriptor", name);
  if (in->rank < 0 || in->rank > ND_MAX_RANK) return nd_fail(h, ND_ERR_ARG, "%s: rank %d out of range", name, in->rank);
  if (in->nnzblocks < 0) return nd_fail(h, ND_ERR_ARG, "%s: negative block count", name);
  out = BsDesc{};
  out.rank = in->rank;
  out.nnzblocks = in->nnzblocks;
  size_t off = 0;
  for (int d = 0; d < in->rank; ++d) {
    int nb = in->nblocks ? in->nblocks[d] : 0;
    if (nb <= 0) return nd_fail(h, ND_ERR_ARG, "%s: dimension %d has no blocks", name, d);
    out.nblocks.push_back(nb);
    std::vector<int64_t> bd(in->blockdims + off, in->blockdims + off + nb);
    for (auto x : bd) if (x < 0) return nd_fail(h, ND_ERR_ARG, "%s: negative block dim", name);
    out.blockdims.push_back(bd);
    off += nb;
  }
  out.blocks_store.assign(in->blocks, in->blocks + (size_t)in->nnzblocks * in->rank);
  out.blocks = out.blocks_store.data();
  out.offsets.assign(in->offsets, in->offsets + in->nnzblocks);
  for (int b = 0; b < in->nnzblocks; ++b)
    for (int d = 0; d < in->rank; ++d) {
      int v = out.blocks_store[(size_t)b * in->rank + d];
      if (v < 1 || v > out.nblocks[d]) return nd_fail(h, ND_ERR_ARG, "%s: block %d has block number %d out of range in dim %d", name, b, v, d);
    }
  return ND_OK;
}

bool nd_make_pair(const Roles& ro, const int64_t* dA, const int64_t* dB, const int64_t* dR, PairDesc& pd,
                  std::string& why) {
  memset(&pd, 0, sizeof(pd));
  int64_t sA[ND_MAX_RANK + 1], sB[ND_MAX_RANK + 1], sR[ND_MAX_RANK + 1];
  sA[0] = sB[0] = sR[0] = 1;
  for (int k = 0; k < ro.rankA; ++k) sA[k + 1] = sA[k] * dA[k];
  for (int k = 0; k < ro.rankB; ++k) sB[k + 1] = sB[k] * dB[k];
  for (int k = 0; k < ro.rankR; ++k) sR[k + 1] = sR[k] * dR[k];
  int64_t M = 1, N = 1, K = 1;
  pd.rows.n = ro.nfa;
  for (int t = 0; t < ro.nfa; ++t) {
    int64_t d = dA[ro.a_free[t]];
    if (d != dR[ro.r_afree[t]]) { why = "output dimension does not match A"; return false; }
    pd.rows.dim[t] = (int32_t)d; pd.rows.st0[t] = sA[ro.a_free[t]]; pd.rows.st1[t] = sR[ro.r_afree[t]];
    M *= d;
  }
  pd.cols.n = ro.nfb;
  for (int t = 0; t < ro.nfb; ++t) {
    int64_t d = dB[ro.b_free[t]];
    if (d != dR[ro.r_bfree[t]]) { why = "output dimension does not match B"; return false; }
    pd.cols.dim[t] = (int32_t)d; pd.cols.st0[t] = sB[ro.b_free[t]]; pd.cols.st1[t] = sR[ro.r_bfree[t]];
    N *= d;
  }
  pd.ks.n = ro.nk;
  for (int t = 0; t < ro.nk; ++t) {
    int64_t d = dA[ro.a_k[t]];
    if (d != dB[ro.b_k[t]]) { why = "contracted dimensions of A and B differ"; return false; }
    pd.ks.dim[t] = (int32_t)d; pd.ks.st0[t] = sA[ro.a_k[t]]; pd.ks.st1[t] = sB[ro.b_k[t]];
    K *= d;
  }
  if (M > INT32_MAX || N > INT32_MAX || K > INT32_MAX) { why = "GEMM extent exceeds 2^31"; return false; }
  pd.M = (int32_t)M; pd.N = (int32_t)N; pd.K = (int32_t)K;
  mixed_simplify(pd.rows);
  mixed_simplify(pd.cols);
  mixed_simplify(pd.ks);
  return true;
}

static nd_status upload(nd_handle h, void** dst, const void* src, size_t bytes) {
  if (*dst) { cudaFreeAsync(*dst, h->stream); *dst = nullptr; }
  if (!bytes) return ND_OK;                     // an empty list stays NULL (its kernels are not launched)
  nd_status s = nd_dalloc(h, dst, bytes);
  if (s) return s;
  return nd_upload(h, *dst, src, bytes);
}

// Work items: tiles of bm x bn over each group, biggest groups first.  Only the
// groups selected by `pick` (all pairs of a group share M and N) are listed.
template <class Pick>
static void make_items(const std::vector<PairDesc>& pairs, int bm, int bn, Pick pick, std::vector<WorkItem>& items) {
  items.clear();
  // groups longest first (work of a full tile; ties in group order), each expanded into
  // its tiles; the order only steers the schedule, every tile's result is the same
  struct Grp { int64_t cost; size_t i, n; };
  std::vector<Grp> grps;
  for (size_t i = 0; i < pairs.size();) {
    size_t j = i;
    int64_t ksum = 0;
    bool all = true;
    while (j < pairs.size() && pairs[j].group == pairs[i].group && pairs[j].job == pairs[i].job) {
      ksum += pairs[j].K;
      all = all && pick(pairs[j]);
      ++j;
    }
    if (all) {
      const PairDesc& p = pairs[i];
      const int64_t mm = std::min(bm, p.M), nn = std::min(bn, p.N);
      grps.push_back({mm * nn * std::max<int64_t>(ksum, 1), i, j - i});
    }
    i = j;
  }
  std::stable_sort(grps.begin(), grps.end(), [](const Grp& x, const Grp& y) { return x.cost > y.cost; });
  for (const Grp& g : grps) {
    const PairDesc& p = pairs[g.i];
    const int mt = (p.M + bm - 1) / bm, nt = (p.N + bn - 1) / bn;
    for (int a = 0; a < mt; ++a)
      for (int b = 0; b < nt; ++b) {
        if (p.sym && bm == bn && a > b) continue;        // below the diagonal of a symmetric R
        items.push_back(WorkItem{p.group, (int)g.i, (int)g.n, a, b});
      }
  }
}

// Split-K for the FP64 tile kernel.  The launch's work is measured in k-steps
// of 16 summed over its tiles (each tile's k axis is its group's pairs' K
// concatenated in plan order); `ctas` resident CTAs share it.  Any tile longer
// than the chunk share below is cut into chunks of about that share, so one
// long-K tile cannot serialise the launch and a small launch still fills the SMs; the
// partial tiles go to a workspace and splitk_reduce sums them in chunk order
// (deterministic) before applying alpha / beta.
static nd_status plan_split_k(nd_handle h, const std::vector<PairDesc>& pairs, std::vector<WorkItem>& items,
                              ExecCache& c, int ctas) {
  if (ctas <= 0 || items.empty()) return ND_OK;
  std::vector<int64_t> ksum(items.size());
  int64_t total = 0;
  for (size_t i = 0; i < items.size(); ++i) {
    int64_t k = 0;
    for (int p = 0; p < items[i].pair_count; ++p) k += pairs[items[i].pair_begin + p].K;
    ksum[i] = k;
    total += (k + 15) / 16;
  }
  // k-steps per chunk.  A launch of fewer tiles than half the SMs (a small contraction such
  // as a 256 x 256 x 128 pair: 16 tiles) is cut until about one chunk per SM, down to
  // single k-steps; otherwise chunks hold at least 4 k-steps to bound the reduction.
  const bool few = items.size() * 2 < (size_t)h->num_sms;
  const int64_t share = few ? std::max<int64_t>(1, (total + h->num_sms - 1) / h->num_sms)
                            : std::max<int64_t>(4, 2 * ((total + ctas - 1) / ctas));
  std::vector<WorkItem> out;
  std::vector<ReduceItem> red;
  int slot = 0;
  for (size_t i = 0; i < items.size(); ++i) {
    const WorkItem& wi = items[i];
    const int64_t steps = (ksum[i] + 15) / 16;
    if (steps <= share || ksum[i] >= INT32_MAX) { out.push_back(wi); continue; }
    const int64_t s = (steps + share - 1) / share;
    const int64_t kc = ((steps + s - 1) / s) * 16;
    const int64_t nch = (ksum[i] + kc - 1) / kc;
    red.push_back(ReduceItem{wi.pair_begin, wi.mt, wi.nt, slot, (int32_t)nch});
    for (int64_t q = 0; q < nch; ++q) {
      WorkItem x = wi;
      x.kbeg = (int32_t)(q * kc);
      x.kend = (int32_t)std::min(ksum[i], (q + 1) * kc);
      x.slot = slot++;
      out.push_back(x);
    }
  }
  if (red.empty()) return ND_OK;
  items.swap(out);
  if (c.d_ws) { cudaFreeAsync(c.d_ws, h->stream); c.d_ws = nullptr; }
  nd_status s0 = nd_dalloc(h, (void**)&c.d_ws, (size_t)slot * nd_gemm_f64_tile_elems() * sizeof(double));
  if (s0) return s0;
  nd_status st = upload(h, (void**)&c.d_red, red.data(), red.size() * sizeof(ReduceItem));
  if (st) return st;
  c.nred = (int)red.size();
  return ND_OK;
}

// A group runs on the skinny kernel when every one of its pairs is skinny.
static bool group_skinny(const std::vector<PairDesc>& pairs, size_t i) {
  for (size_t j = i; j < pairs.size() && pairs[j].group == pairs[i].group && pairs[j].job == pairs[i].job; ++j)
    if (!nd_pair_is_skinny(pairs[j])) return false;
  return true;
}

// Device state of one contraction for one set of execution parameters.
static nd_status build_exec(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs, int ngroups,
                            int precision, int slices, const TuneChoice& tc) {
  c.free_all(h);
  c.stream = h->stream;
  c.precision = precision;
  c.slices = slices;
  c.req_pair2 = h->split_pair2;
  // which pairs sit in skinny groups (routed to the FP64 CUDA-core kernel)
  std::vector<char> sk(pairs.size(), 0);
  bool any_sk = false;
  for (size_t i = 0; i < pairs.size();) {
    size_t j = i;
    const bool g = tc.skinny && group_skinny(pairs, i);
    any_sk = any_sk || g;
    while (j < pairs.size() && pairs[j].group == pairs[i].group && pairs[j].job == pairs[i].job) sk[j++] = g;
    i = j;
  }
  nd_status s = ND_OK;
  // the FP64 kernels read the pair list; the split-precision path uploads its own copy
  if (precision == ND_PREC_FP64 || any_sk)
    if ((s = upload(h, (void**)&c.d_pairs, pairs.data(), pairs.size() * sizeof(PairDesc)))) return s;
  std::vector<WorkItem> items;
  make_items(pairs, nd_skinny_rows(), 1 << 30, [&](const PairDesc& p) { return sk[&p - pairs.data()] != 0; }, items);
  c.nsk_items = (int)items.size();
  if ((s = upload(h, (void**)&c.d_sk_items, items.data(), items.size() * sizeof(WorkItem)))) return s;
  if (precision == ND_PREC_FP64) {
    make_items(pairs, 64, 64, [&](const PairDesc& p) { return sk[&p - pairs.data()] == 0; }, items);
    if ((s = plan_split_k(h, pairs, items, c, tc.splitk_mult * h->num_sms))) return s;
    c.nitems = (int)items.size();
    if ((s = upload(h, (void**)&c.d_items, items.data(), items.size() * sizeof(WorkItem)))) return s;
  } else {
    if (!any_sk) {
      if ((s = nd_split_build(h, c, pairs, ngroups, precision, tc.pair2))) return s;
    } else {
      std::vector<PairDesc> regular;
      regular.reserve(pairs.size());
      for (size_t i = 0; i < pairs.size(); ++i) if (!sk[i]) regular.push_back(pairs[i]);
      if (!regular.empty() && (s = nd_split_build(h, c, regular, ngroups, precision, tc.pair2))) return s;
    }
  }
  c.built = true;
  return ND_OK;
}

static nd_status launch_exec(nd_handle h, ExecCache& c, const JobPtrs& ptrs, double alpha, double beta) {
  nd_status s = nd_launch_skinny_f64(h, c.d_pairs, c.d_sk_items, c.nsk_items, ptrs, alpha, beta);
  if (s) return s;
  if (c.precision == ND_PREC_FP64)
    return nd_launch_gemm_f64(h, c.d_pairs, c.d_items, c.nitems, ptrs, alpha, beta, c.d_ws, c.d_red, c.nred);
  return nd_split_run(h, c, ptrs, alpha, beta);
}

// Autotuner key: SM count, precision, slices and the block-size histogram
// (block pairs counted per (bit length of M, N, K) bucket).
static std::string tune_key(nd_handle h, const std::vector<PairDesc>& pairs, int precision, int slices) {
  auto bl = [](int64_t v) { int b = 0; while (v > 0) { ++b; v >>= 1; } return b; };
  std::map<int, int> hist;
  for (const PairDesc& p : pairs) hist[(bl(p.M) << 16) | (bl(p.N) << 8) | bl(p.K)]++;
  std::string k = "sm" + std::to_string(h->num_sms) + "/p" + std::to_string(precision) + "/s" + std::to_string(slices) + "/";
  bool first = true;
  for (auto& e : hist) {
    if (!first) k += ",";
    first = false;
    k += std::to_string(e.first >> 16) + "." + std::to_string((e.first >> 8) & 255) + "." +
         std::to_string(e.first & 255) + "x" + std::to_string(e.second);
  }
  return k;
}

// Time every candidate on the real operands (R is overwritten: beta == 0), keep the fastest.
static nd_status tune_exec(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs, int ngroups,
                           const JobPtrs& ptrs, double alpha, int precision, int slices, TuneEntry& out) {
  std::vector<TuneChoice> cands;
  if (precision == ND_PREC_FP64) {
    for (int sk = 1; sk >= 0; --sk)
      for (int m : {4, 0, 2, 8}) cands.push_back(TuneChoice{m, sk, 1});
  } else {
    for (int sk = 1; sk >= 0; --sk)
      for (int p2 : {h->split_pair2, 1 - h->split_pair2}) cands.push_back(TuneChoice{4, sk, p2});
  }
  cudaEvent_t e0, e1;
  ND_CUDA(h, cudaEventCreate(&e0));
  ND_CUDA(h, cudaEventCreate(&e1));
  nd_status st = ND_OK;
  double best = 1e300;
  TuneChoice bestc = cands[0];
  for (size_t i = 0; i < cands.size() && !st; ++i) {
    if ((st = build_exec(h, c, pairs, ngroups, precision, slices, cands[i]))) break;
    if ((st = launch_exec(h, c, ptrs, alpha, 0.0))) break;           // warm-up
    float ms = 0.f, tot = 0.f;
    for (int r = 0; r < 2 && !st; ++r) {
      cudaEventRecord(e0, h->stream);
      st = launch_exec(h, c, ptrs, alpha, 0.0);
      cudaEventRecord(e1, h->stream);
      if (!st) st = nd_cuda_check(h, cudaEventSynchronize(e1), "tune timing");
      if (!st) { cudaEventElapsedTime(&ms, e0, e1); tot += ms; }
    }
    if (st) break;
    if (i == 0) out.default_ms = tot / 2;
    if (tot / 2 < best) { best = tot / 2; bestc = cands[i]; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if ((st = nd_check_device_status(h, "autotune"))) return st;
  out.choice = bestc;
  out.best_ms = best;
  return build_exec(h, c, pairs, ngroups, precision, slices, bestc);
}

nd_status nd_execute_cached(nd_handle h, ExecCache& c, const std::vector<PairDesc>& pairs, int ngroups,
                            const JobPtrs& ptrs, double alpha, double beta, int precision) {
  if (pairs.empty()) return ND_OK;
  if (precision != ND_PREC_FP64 && precision != ND_PREC_OZAKI && precision != ND_PREC_BF16X3)
    return nd_fail(h, ND_ERR_ARG, "unknown precision %d", precision);
  const int want_slices = precision == ND_PREC_OZAKI ? h->ozaki_slices : (precision == ND_PREC_BF16X3 ? 2 : 0);
  if (!c.built || c.precision != precision || c.slices != want_slices ||
      (precision != ND_PREC_FP64 && c.req_pair2 != h->split_pair2)) {
    if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "contraction state must be built before graph capture (run once first)");
    const std::string key = tune_key(h, pairs, precision, want_slices);
    auto it = h->tune.find(key);
    nd_status s;
    if (it != h->tune.end()) {
      s = build_exec(h, c, pairs, ngroups, precision, want_slices, it->second.choice);
    } else if (h->tuning && beta == 0.0) {
      TuneEntry e;
      s = tune_exec(h, c, pairs, ngroups, ptrs, alpha, precision, want_slices, e);
      if (!s) h->tune[key] = e;
    } else {
      TuneChoice dflt;
      dflt.pair2 = h->split_pair2;
      s = build_exec(h, c, pairs, ngroups, precision, want_slices, dflt);
    }
    if (s) return s;
  }
  if (c.stream != h->stream && !nd_capturing(h)) {
    // the state was last used on another stream: order that work before this launch, so
    // the state's release (on the handle's stream) follows every use
    if (!h->order_ev) ND_CUDA(h, cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming));
    ND_CUDA(h, cudaEventRecord(h->order_ev, c.stream));
    ND_CUDA(h, cudaStreamWaitEvent(h->stream, h->order_ev, 0));
    c.stream = h->stream;
  }
  return launch_exec(h, c, ptrs, alpha, beta);
}

// ---------------------------------------------------------------------------
// Verify mode (nd_set_verify): a split-precision contraction is run a second time
// with the FP64 kernels into scratch memory and the relative Frobenius distance of the
// two results is recorded.
// ---------------------------------------------------------------------------
constexpr int kVerifyCtas = 256;

// Per-CTA sums of (x - y)^2 and y^2 over element ranges [start[r], start[r] + len) of
// two buffers; flat index t lies in range r when prefix[r] <= t < prefix[r + 1].
__global__ void __launch_bounds__(256) verify_partial(const double* x, const double* y, const int64_t* start,
                                                      const int64_t* prefix, int nranges, double* part) {
  __shared__ double s0[256], s1[256];
  const int64_t total = prefix[nranges];
  double a = 0.0, b = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nranges - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (prefix[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const int64_t i = start[lo] + (t - prefix[lo]);
    const double yv = y[i], d = x[i] - yv;
    a += d * d;
    b += yv * yv;
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o; o >>= 1) {
    if ((int)threadIdx.x < o) { s0[threadIdx.x] += s0[threadIdx.x + o]; s1[threadIdx.x] += s1[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = s0[0]; part[2 * blockIdx.x + 1] = s1[0]; }
}

// One output of a verified call: the split-precision result x, the FP64 result y and
// the element ranges (offset, length) the call wrote.
struct VerifyOut {
  const double* x;
  const double* y;
  std::vector<std::pair<int64_t, int64_t>> ranges;
};

// Records sqrt(sum |x - y|^2 / sum |y|^2) over every output; synchronises the stream.
static nd_status verify_record(nd_handle h, const std::vector<VerifyOut>& outs) {
  double num = 0.0, den = 0.0;
  std::vector<double> part(2 * kVerifyCtas);
  for (const VerifyOut& o : outs) {
    std::vector<std::pair<int64_t, int64_t>> r = o.ranges;
    std::sort(r.begin(), r.end());
    std::vector<int64_t> start, prefix{0};
    for (const auto& q : r) {
      if (q.second <= 0) continue;
      if (!start.empty() && start.back() + (prefix.back() - prefix[prefix.size() - 2]) == q.first) {
        prefix.back() += q.second;                      // adjacent to the previous range: merge
      } else {
        start.push_back(q.first);
        prefix.push_back(prefix.back() + q.second);
      }
    }
    if (start.empty()) continue;
    const int n = (int)start.size();
    std::vector<int64_t> hostbuf(start);
    hostbuf.insert(hostbuf.end(), prefix.begin(), prefix.end());
    int64_t* d = nullptr;
    ND_CUDA(h, cudaMallocAsync(&d, hostbuf.size() * 8 + part.size() * 8, h->stream));
    double* dpart = (double*)(d + hostbuf.size());
    nd_status s = nd_upload(h, d, hostbuf.data(), hostbuf.size() * 8);
    if (s == ND_OK) {
      nd_prof_begin(h, "verify_partial");
      verify_partial<<<kVerifyCtas, 256, 0, h->stream>>>(o.x, o.y, d, d + n, n, dpart);
      nd_prof_end(h);
      ND_LAUNCHED(h);
      s = nd_cuda_check(h, cudaGetLastError(), "verify_partial");
    }
    cudaError_t e = s == ND_OK ? cudaMemcpyAsync(part.data(), dpart, part.size() * 8, cudaMemcpyDeviceToHost, h->stream)
                               : cudaSuccess;
    cudaFreeAsync(d, h->stream);
    if (s != ND_OK) return s;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return nd_cuda_check(h, e, "verify");
    for (int b = 0; b < kVerifyCtas; ++b) { num += part[2 * b]; den += part[2 * b + 1]; }
  }
  h->verify_err = den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
  return ND_OK;
}

// ---------------------------------------------------------------------------
// Dense contract!
// ---------------------------------------------------------------------------
constexpr size_t kDenseCacheEntries = 64;

static void append_mixed(std::string& k, const Mixed& m) {
  k.append((const char*)&m.n, sizeof m.n);
  for (int d = 0; d < m.n; ++d) {
    k.append((const char*)&m.dim[d], sizeof m.dim[d]);
    k.append((const char*)&m.st0[d], sizeof m.st0[d]);
    k.append((const char*)&m.st1[d], sizeof m.st1[d]);
  }
}

// Cached execution state of a dense contraction (one block pair), oldest evicted first.
static ExecCache* dense_exec(nd_handle h, const PairDesc& pd, int precision) {
  std::string key;
  const int32_t head[5] = {precision, h->ozaki_slices, pd.M, pd.N, h->split_pair2};
  key.append((const char*)head, sizeof head);
  key.append((const char*)&pd.K, sizeof pd.K);
  append_mixed(key, pd.rows);
  append_mixed(key, pd.cols);
  append_mixed(key, pd.ks);
  auto it = h->dense_cache.find(key);
  if (it != h->dense_cache.end()) return (ExecCache*)it->second;
  if (nd_capturing(h)) return nullptr;
  if (h->dense_cache.size() >= kDenseCacheEntries) {
    const std::string old = h->dense_order.front();
    h->dense_order.erase(h->dense_order.begin());
    cudaStreamSynchronize(h->stream);               // the evicted state may still be in use
    ExecCache* e = (ExecCache*)h->dense_cache[old];
    e->free_all(h);
    delete e;
    h->dense_cache.erase(old);
  }
  ExecCache* c = new (std::nothrow) ExecCache();
  if (!c) return nullptr;
  h->dense_cache[key] = c;
  h->dense_order.push_back(key);
  return c;
}

void nd_dense_cache_clear(nd_handle h) {
  for (auto& e : h->dense_cache) {
    ExecCache* c = (ExecCache*)e.second;
    c->free_all(h);
    delete c;
  }
  h->dense_cache.clear();
  h->dense_order.clear();
}

extern "C" nd_status nd_contract_dense_f64(nd_handle h, double* R, int32_t rankR, const int64_t* dimsR,
                                           const int32_t* labelsR, const double* A, int32_t rankA,
                                           const int64_t* dimsA, const int32_t* labelsA, const double* B,
                                           int32_t rankB, const int64_t* dimsB, const int32_t* labelsB,
                                           double alpha, double beta, int32_t precision) {
  if (!h) return ND_ERR_ARG;
  if (h->verify) h->verify_err = 0.0;              // exact branches (scalar, empty K) record 0
  if (rankA < 0 || rankB < 0 || rankR < 0 || rankA > ND_MAX_RANK || rankB > ND_MAX_RANK || rankR > ND_MAX_RANK)
    return nd_fail(h, ND_ERR_ARG, "contract: rank out of range (max %d)", ND_MAX_RANK);
  int64_t nA = 1, nB = 1, nR = 1;
  for (int k = 0; k < rankA; ++k) { if (dimsA[k] < 0) return nd_fail(h, ND_ERR_ARG, "contract: negative dim"); nA *= dimsA[k]; }
  for (int k = 0; k < rankB; ++k) { if (dimsB[k] < 0) return nd_fail(h, ND_ERR_ARG, "contract: negative dim"); nB *= dimsB[k]; }
  for (int k = 0; k < rankR; ++k) { if (dimsR[k] < 0) return nd_fail(h, ND_ERR_ARG, "contract: negative dim"); nR *= dimsR[k]; }
  if (nR == 0) return ND_OK;
  if ((nA && !A) || (nB && !B) || !R) return nd_fail(h, ND_ERR_ARG, "contract: NULL data pointer");
  // scalar branch (dense/tensoralgebra/contract.jl:100-150, 171-174)
  if (nA == 1 || nB == 1) {
    const double* scal = nA == 1 ? A : B;
    const double* T = nA == 1 ? B : A;
    int rankT = nA == 1 ? rankB : rankA;
    const int64_t* dT = nA == 1 ? dimsB : dimsA;
    const int32_t* lT = nA == 1 ? labelsB : labelsA;
    if (nA == 1 && nB == 1) {
      int64_t one = 1;
      int p0 = 0;
      return nd_launch_permute(h, R, B, 1, &one, &p0, alpha, beta, A);
    }
    // drop singletons and derive the permutation from the labels
    std::vector<int> lr, lt;
    std::vector<int64_t> dr, dt;
    for (int k = 0; k < rankR; ++k) if (dimsR[k] != 1) { lr.push_back(labelsR[k]); dr.push_back(dimsR[k]); }
    for (int k = 0; k < rankT; ++k) if (dT[k] != 1) { lt.push_back(lT[k]); dt.push_back(dT[k]); }
    if (lr.size() != lt.size()) return nd_fail(h, ND_ERR_ARG, "contract: scalar branch rank mismatch");
    std::vector<int> perm(lr.size());
    for (size_t r = 0; r < lr.size(); ++r) {
      auto it = std::find(lt.begin(), lt.end(), lr[r]);
      if (it == lt.end()) return nd_fail(h, ND_ERR_ARG, "contract: output label %d not found", lr[r]);
      perm[r] = (int)(it - lt.begin());
      if (dt[perm[r]] != dr[r]) return nd_fail(h, ND_ERR_ARG, "contract: dimension mismatch in scalar branch");
    }
    if (lr.empty()) {
      int64_t one = 1; int p0 = 0;
      return nd_launch_permute(h, R, T, 1, &one, &p0, alpha, beta, scal);
    }
    return nd_launch_permute(h, R, T, (int)lr.size(), dt.data(), perm.data(), alpha, beta, scal);
  }
  Roles ro;
  std::string why;
  if (!nd_make_roles(rankA, labelsA, rankB, labelsB, rankR, labelsR, ro, why))
    return nd_fail(h, ND_ERR_ARG, "contract: %s", why.c_str());
  PairDesc pd;
  if (!nd_make_pair(ro, dimsA, dimsB, dimsR, pd, why)) return nd_fail(h, ND_ERR_ARG, "contract: %s", why.c_str());
  pd.group = 0; pd.first = 1; pd.job = 0; pd.a_op = 0; pd.b_op = 0;
  if (pd.K == 0) {   // empty contraction: R = beta * R
    int64_t n = nR; int p0 = 0;
    return nd_launch_permute(h, R, R, 1, &n, &p0, 0.0, beta, nullptr);
  }
  std::vector<PairDesc> pairs{pd};
  // the device state (descriptors, work list, split-K / split-operand scratch) of a
  // dense contraction is kept per handle and reused by later calls of the same shape,
  // so repeated small contractions cost no allocation and can be graph-captured
  ExecCache* c = dense_exec(h, pd, precision);
  if (!c && nd_capturing(h))
    return nd_fail(h, ND_ERR_ARG, "contract: run this shape once before graph capture (its state is built then)");
  if (!c) return nd_fail(h, ND_ERR_OOM, "contract: host allocation failed");
  const bool verify = h->verify && precision != ND_PREC_FP64;
  if (h->verify && nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "contract: verify mode cannot be graph-captured");
  if (h->verify) h->verify_err = -1.0;             // until this call's figure is known
  double* saved = nullptr;   // verify with beta != 0: R before the call, the FP64 run's input
  if (verify && beta != 0.0) {
    ND_CUDA(h, cudaMallocAsync(&saved, nR * 8, h->stream));
    ND_CUDA(h, cudaMemcpyAsync(saved, R, nR * 8, cudaMemcpyDeviceToDevice, h->stream));
  }
  JobPtrs ptrs{{A, nullptr}, {B, nullptr}, {R, nullptr}};
  nd_status s = nd_execute_cached(h, *c, pairs, 1, ptrs, alpha, beta, precision);
  if (s == ND_OK && verify) {
    ExecCache* c64 = dense_exec(h, pd, ND_PREC_FP64);
    if (!c64) s = nd_fail(h, ND_ERR_OOM, "contract: host allocation failed");
    double* F = saved;
    if (s == ND_OK && !F) {
      cudaError_t e = cudaMallocAsync(&F, nR * 8, h->stream);
      if (e != cudaSuccess) s = nd_cuda_check(h, e, "verify scratch");
    }
    if (s == ND_OK) {
      JobPtrs p64{{A, nullptr}, {B, nullptr}, {F, nullptr}};
      s = nd_execute_cached(h, *c64, pairs, 1, p64, alpha, beta, ND_PREC_FP64);
    }
    if (s == ND_OK) s = verify_record(h, {VerifyOut{R, F, {{0, nR}}}});
    if (F) cudaFreeAsync(F, h->stream);
    saved = nullptr;
  } else if (s == ND_OK && h->verify) {
    h->verify_err = 0.0;
  }
  if (saved) cudaFreeAsync(saved, h->stream);
  if (s != ND_OK) return s;
  if (nd_capturing(h)) return ND_OK;
  return nd_check_device_status(h, "contract");   // synchronises the stream
}

// ---------------------------------------------------------------------------
// Block-sparse plan
// ---------------------------------------------------------------------------
extern "C" nd_status nd_bs_plan_create(nd_handle h, const nd_bs_desc* A, const int32_t* labelsA,
                                       const nd_bs_desc* B, const int32_t* labelsB, int32_t rankR,
                                       const int32_t* labelsR, nd_plan* plan) {
  if (!h || !plan) return ND_ERR_ARG;
  *plan = nullptr;
  auto p = new nd_bs_plan_s();
  p->h = h;
  nd_status s = nd_bs_import(h, A, p->A, "plan(A)");
  if (!s) s = nd_bs_import(h, B, p->B, "plan(B)");
  if (s) { delete p; return s; }
  std::string why;
  if (!nd_make_roles(p->A.rank, labelsA, p->B.rank, labelsB, rankR, labelsR, p->roles, why)) {
    delete p;
    return nd_fail(h, ND_ERR_ARG, "plan: %s", why.c_str());
  }
  p->rankR = rankR;
  p->labelsA.assign(labelsA, labelsA + p->A.rank);
  p->labelsB.assign(labelsB, labelsB + p->B.rank);
  p->labelsR.assign(labelsR, labelsR + rankR);
  const Roles& ro = p->roles;
  // contracted indices must have identical block structure
  for (int t = 0; t < ro.nk; ++t)
    if (p->A.blockdims[ro.a_k[t]] != p->B.blockdims[ro.b_k[t]]) {
      delete p;
      return nd_fail(h, ND_ERR_ARG, "plan: contracted index %d of A and %d of B have different block dims", ro.a_k[t], ro.b_k[t]);
    }
  p->r_nblocks.assign(rankR, 0);
  p->r_blockdims.assign(rankR, {});
  for (int t = 0; t < ro.nfa; ++t) {
    p->r_nblocks[ro.r_afree[t]] = p->A.nblocks[ro.a_free[t]];
    p->r_blockdims[ro.r_afree[t]] = p->A.blockdims[ro.a_free[t]];
  }
  for (int t = 0; t < ro.nfb; ++t) {
    p->r_nblocks[ro.r_bfree[t]] = p->B.nblocks[ro.b_free[t]];
    p->r_blockdims[ro.r_bfree[t]] = p->B.blockdims[ro.b_free[t]];
  }
  s = nd_block_plan(h, ro, p->A, p->B, p->r_nblocks, p->r_blockdims, p->res);
  if (s) { delete p; return s; }
  *plan = p;
  return ND_OK;
}

extern "C" nd_status nd_bs_plan_sizes(nd_plan plan, int32_t* npairs, int32_t* nR, int64_t* nnzR) {
  if (!plan) return ND_ERR_ARG;
  if (npairs) *npairs = plan->res.npairs;
  if (nR) *nR = plan->res.nR;
  if (nnzR) *nnzR = plan->res.nnzR;
  return ND_OK;
}

extern "C" nd_status nd_bs_plan_get(nd_plan plan, int32_t* blocksR, int64_t* offsetsR, int32_t* pairs) {
  if (!plan) return ND_ERR_ARG;
  const PlanResult& r = plan->res;
  if (blocksR && !r.blocksR.empty()) memcpy(blocksR, r.blocksR.data(), r.blocksR.size() * 4);
  if (offsetsR && !r.offsetsR.empty()) memcpy(offsetsR, r.offsetsR.data(), r.offsetsR.size() * 8);
  if (pairs && !r.pairs.empty()) memcpy(pairs, r.pairs.data(), r.pairs.size() * 4);
  return ND_OK;
}

extern "C" nd_status nd_bs_plan_set_output_offsets(nd_plan p, const int64_t* offsetsR) {
  if (!p) return ND_ERR_ARG;
  nd_handle h = p->h;
  if (!offsetsR && p->res.nR > 0) return nd_fail(h, ND_ERR_ARG, "plan_set_output_offsets: NULL offsets");
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "plan_set_output_offsets: not during graph capture");
  for (int32_t g = 0; g < p->res.nR; ++g)
    if (offsetsR[g] < 0) return nd_fail(h, ND_ERR_ARG, "plan_set_output_offsets: negative offset for block %d", g);
  p->res.offsetsR.assign(offsetsR, offsetsR + p->res.nR);
  // execution state carries the old offsets: rebuild it on the next call
  for (auto& c : p->cache) c.free_all(h);
  for (auto& c : p->adj_cache) c.free_all(h);
  p->descs.clear();
  p->adj_descs.clear();
  p->adj_built = false;
  return ND_OK;
}

extern "C" nd_status nd_bs_plan_destroy(nd_plan plan) {
  if (!plan) return ND_OK;
  for (auto& c : plan->cache) c.free_all(plan->h);      // stream-ordered after the plan's last launch
  for (auto& c : plan->adj_cache) c.free_all(plan->h);
  delete plan;
  return ND_OK;
}

// Group the plan's pairs by output block (R block order), plan order inside a group.
static nd_status build_forward_descs(nd_plan p) {
  if (!p->descs.empty() || p->res.npairs == 0) return ND_OK;
  nd_handle h = p->h;
  const PlanResult& r = p->res;
  const int rankR = p->rankR;
  std::vector<std::vector<int>> by_group(r.nR);
  for (int q = 0; q < r.npairs; ++q) by_group[r.pairs[3 * q + 2]].push_back(q);
  std::string why;
  p->descs.reserve(r.npairs);
  for (int g = 0; g < r.nR; ++g) {
    int64_t dR[ND_MAX_RANK];
    for (int k = 0; k < rankR; ++k) dR[k] = p->r_blockdims[k][r.blocksR[(size_t)g * rankR + k] - 1];
    bool first = true;
    for (int q : by_group[g]) {
      int iA = r.pairs[3 * q], iB = r.pairs[3 * q + 1];
      int64_t dA[ND_MAX_RANK], dB[ND_MAX_RANK];
      for (int k = 0; k < p->A.rank; ++k) dA[k] = p->A.bdim(iA, k);
      for (int k = 0; k < p->B.rank; ++k) dB[k] = p->B.bdim(iB, k);
      PairDesc pd;
      if (!nd_make_pair(p->roles, dA, dB, dR, pd, why)) return nd_fail(h, ND_ERR_ARG, "plan: %s", why.c_str());
      pd.a_off = p->A.offsets[iA];
      pd.b_off = p->B.offsets[iB];
      pd.r_off = r.offsetsR[g];
      pd.group = g;
      pd.first = first ? 1 : 0;
      pd.job = 0;
      pd.a_op = iA;
      pd.b_op = iB;
      first = false;
      p->descs.push_back(pd);
    }
  }
  p->ngroups = r.nR;
  return ND_OK;
}

extern "C" nd_status nd_bs_contract_f64(nd_handle h, nd_plan p, double* R, const double* A, const double* B,
                                        double alpha, int32_t precision) {
  if (!h || !p) return ND_ERR_ARG;
  if (p->res.npairs == 0) return ND_OK;
  if (!R || !A || !B) return nd_fail(h, ND_ERR_ARG, "bs_contract: NULL data pointer");
  if (precision < 0 || precision > 2) return nd_fail(h, ND_ERR_ARG, "bs_contract: unknown precision %d", precision);
  nd_status s = build_forward_descs(p);
  if (s) return s;
  if (h->verify && nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "bs_contract: verify mode cannot be graph-captured");
  if (h->verify) h->verify_err = -1.0;
  JobPtrs ptrs{{A, nullptr}, {B, nullptr}, {R, nullptr}};
  s = nd_execute_cached(h, p->cache[precision], p->descs, p->ngroups, ptrs, alpha, 0.0, precision);
  if (s || !h->verify) return s;
  if (precision == ND_PREC_FP64) {
    h->verify_err = 0.0;
    return ND_OK;
  }
  // every output block is written whole (its first pair overwrites), so only those
  // ranges are compared; the scratch spans the highest one
  VerifyOut vo{R, nullptr, {}};
  int64_t extent = 0;
  for (int32_t g = 0; g < p->res.nR; ++g) {
    int64_t n = 1;
    for (int k = 0; k < p->rankR; ++k) n *= p->r_blockdims[k][p->res.blocksR[(size_t)g * p->rankR + k] - 1];
    vo.ranges.push_back({p->res.offsetsR[g], n});
    extent = std::max(extent, p->res.offsetsR[g] + n);
  }
  double* F = nullptr;
  ND_CUDA(h, cudaMallocAsync(&F, std::max<int64_t>(extent, 1) * 8, h->stream));
  vo.y = F;
  JobPtrs p64{{A, nullptr}, {B, nullptr}, {F, nullptr}};
  s = nd_execute_cached(h, p->cache[ND_PREC_FP64], p->descs, p->ngroups, p64, alpha, 0.0, ND_PREC_FP64);
  if (s == ND_OK) s = verify_record(h, {vo});
  cudaFreeAsync(F, h->stream);
  return s;
}

// Pullback: job 0: Abar = Rbar * B grouped by A block; job 1: Bbar = A * Rbar grouped by B block.
static nd_status build_adjoint_descs(nd_plan p) {
  if (p->adj_built) return ND_OK;
  nd_handle h = p->h;
  const PlanResult& r = p->res;
  Roles r1, r2;
  std::string why;
  if (!nd_make_roles(p->rankR, p->labelsR.data(), p->B.rank, p->labelsB.data(), p->A.rank, p->labelsA.data(), r1, why) ||
      !nd_make_roles(p->A.rank, p->labelsA.data(), p->rankR, p->labelsR.data(), p->B.rank, p->labelsB.data(), r2, why))
    return nd_fail(h, ND_ERR_ARG, "adjoint: %s", why.c_str());
  const int nA = p->A.nnzblocks, nB = p->B.nnzblocks;
  std::vector<std::vector<int>> byA(nA), byB(nB);
  for (int q = 0; q < r.npairs; ++q) { byA[r.pairs[3 * q]].push_back(q); byB[r.pairs[3 * q + 1]].push_back(q); }
  auto dimsR = [&](int g, int64_t* d) { for (int k = 0; k < p->rankR; ++k) d[k] = p->r_blockdims[k][r.blocksR[(size_t)g * p->rankR + k] - 1]; };
  for (int a = 0; a < nA; ++a) {
    bool first = true;
    for (int q : byA[a]) {
      int iB = r.pairs[3 * q + 1], g = r.pairs[3 * q + 2];
      int64_t dA[ND_MAX_RANK], dB[ND_MAX_RANK], dR[ND_MAX_RANK];
      for (int k = 0; k < p->A.rank; ++k) dA[k] = p->A.bdim(a, k);
      for (int k = 0; k < p->B.rank; ++k) dB[k] = p->B.bdim(iB, k);
      dimsR(g, dR);
      PairDesc pd;
      if (!nd_make_pair(r1, dR, dB, dA, pd, why)) return nd_fail(h, ND_ERR_ARG, "adjoint: %s", why.c_str());
      pd.a_off = r.offsetsR[g]; pd.b_off = p->B.offsets[iB]; pd.r_off = p->A.offsets[a];
      pd.group = a; pd.first = first; pd.job = 0; pd.a_op = g; pd.b_op = iB;
      first = false;
      p->adj_descs.push_back(pd);
    }
  }
  for (int b = 0; b < nB; ++b) {
    bool first = true;
    for (int q : byB[b]) {
      int iA = r.pairs[3 * q], g = r.pairs[3 * q + 2];
      int64_t dA[ND_MAX_RANK], dB[ND_MAX_RANK], dR[ND_MAX_RANK];
      for (int k = 0; k < p->A.rank; ++k) dA[k] = p->A.bdim(iA, k);
      for (int k = 0; k < p->B.rank; ++k) dB[k] = p->B.bdim(b, k);
      dimsR(g, dR);
      PairDesc pd;
      if (!nd_make_pair(r2, dA, dR, dB, pd, why)) return nd_fail(h, ND_ERR_ARG, "adjoint: %s", why.c_str());
      pd.a_off = p->A.offsets[iA]; pd.b_off = r.offsetsR[g]; pd.r_off = p->B.offsets[b];
      pd.group = nA + b; pd.first = first; pd.job = 1; pd.a_op = iA; pd.b_op = g;
      first = false;
      p->adj_descs.push_back(pd);
    }
  }
  p->adj_ngroups = nA + nB;
  p->adj_built = true;
  return ND_OK;
}

__global__ void zero_ranges(double* base0, double* base1, const int64_t* ranges, int n) {
  // ranges: [n][3] = (job, offset, count)
  for (int r = blockIdx.y; r < n; r += gridDim.y) {
    double* b = ranges[3 * r] ? base1 : base0;
    int64_t off = ranges[3 * r + 1], cnt = ranges[3 * r + 2];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x)
      b[off + i] = 0.0;
  }
}

extern "C" nd_status nd_bs_contract_adjoint_f64(nd_handle h, nd_plan p, const double* Rbar, const double* A,
                                                const double* B, double* Abar, double* Bbar, int32_t precision) {
  if (!h || !p) return ND_ERR_ARG;
  if (!Abar || !Bbar) return nd_fail(h, ND_ERR_ARG, "adjoint: NULL output");
  if (precision < 0 || precision > 2) return nd_fail(h, ND_ERR_ARG, "adjoint: unknown precision %d", precision);
  if (h->verify && nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "adjoint: verify mode cannot be graph-captured");
  if (h->verify) h->verify_err = -1.0;
  nd_status s = build_adjoint_descs(p);
  if (s) return s;
  // blocks of A / B that no pair touches have a zero cotangent
  std::vector<int64_t> ranges;
  {
    std::vector<char> tA(p->A.nnzblocks, 0), tB(p->B.nnzblocks, 0);
    for (int q = 0; q < p->res.npairs; ++q) { tA[p->res.pairs[3 * q]] = 1; tB[p->res.pairs[3 * q + 1]] = 1; }
    for (int a = 0; a < p->A.nnzblocks; ++a) if (!tA[a]) ranges.insert(ranges.end(), {0, p->A.offsets[a], p->A.block_elems(a)});
    for (int b = 0; b < p->B.nnzblocks; ++b) if (!tB[b]) ranges.insert(ranges.end(), {1, p->B.offsets[b], p->B.block_elems(b)});
  }
  if (!ranges.empty()) {
    if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "adjoint with untouched blocks cannot be captured");
    int64_t* d = nullptr;
    ND_CUDA(h, cudaMallocAsync(&d, ranges.size() * 8, h->stream));
    ND_CUDA(h, cudaMemcpyAsync(d, ranges.data(), ranges.size() * 8, cudaMemcpyHostToDevice, h->stream));
    int n = (int)(ranges.size() / 3);
    nd_prof_begin(h, "zero_ranges");
    zero_ranges<<<dim3(64, std::min(n, 1024)), 256, 0, h->stream>>>(Abar, Bbar, d, n);
    nd_prof_end(h);
    ND_LAUNCHED(h);
    ND_CUDA(h, cudaFreeAsync(d, h->stream));
  }
  if (p->adj_descs.empty()) {
    if (h->verify) h->verify_err = 0.0;
    return ND_OK;
  }
  JobPtrs ptrs{{Rbar, A}, {B, Rbar}, {Abar, Bbar}};
  s = nd_execute_cached(h, p->adj_cache[precision], p->adj_descs, p->adj_ngroups, ptrs, 1.0, 0.0, precision);
  if (s || !h->verify) return s;
  if (precision == ND_PREC_FP64) {
    h->verify_err = 0.0;
    return ND_OK;
  }
  // both cotangents over every block of A and B (untouched blocks are zero in both runs)
  VerifyOut va{Abar, nullptr, {}}, vb{Bbar, nullptr, {}};
  int64_t ea = 0, eb = 0;
  for (int a = 0; a < p->A.nnzblocks; ++a) {
    va.ranges.push_back({p->A.offsets[a], p->A.block_elems(a)});
    ea = std::max(ea, p->A.offsets[a] + p->A.block_elems(a));
  }
  for (int b = 0; b < p->B.nnzblocks; ++b) {
    vb.ranges.push_back({p->B.offsets[b], p->B.block_elems(b)});
    eb = std::max(eb, p->B.offsets[b] + p->B.block_elems(b));
  }
  double* F = nullptr;
  ND_CUDA(h, cudaMallocAsync(&F, std::max<int64_t>(ea + eb, 1) * 8, h->stream));
  nd_status s2 = nd_cuda_check(h, cudaMemsetAsync(F, 0, (ea + eb) * 8, h->stream), "verify scratch");
  va.y = F;
  vb.y = F + ea;
  if (s2 == ND_OK) {
    JobPtrs p64{{Rbar, A}, {B, Rbar}, {F, F + ea}};
    s2 = nd_execute_cached(h, p->adj_cache[ND_PREC_FP64], p->adj_descs, p->adj_ngroups, p64, 1.0, 0.0, ND_PREC_FP64);
  }
  if (s2 == ND_OK) s2 = verify_record(h, {va, vb});
  cudaFreeAsync(F, h->stream);
  return s2;
}

// ---------------------------------------------------------------------------
// Block-sparse x block-diagonal DiagBlockSparse
// (NDTensors/src/blocksparse/diagblocksparse.jl:601-696; per block pair the
// diagonal contraction of NDTensors/src/diag/tensoralgebra/contract.jl:103-214)
// ---------------------------------------------------------------------------
// Every index of a diagonal block carries the same coordinate i < min(block dims),
// d_i its value.  So an output element whose D-index coordinates are all equal to i
// is alpha * sum over the group's pairs of d_i * T(x, i, ..., i) (x the T-free
// coordinates; with no D index in the output, the sum also runs over i), and every
// other output element is zero.  One thread per output element, each written once:
// T is read once and R written once, 16 bytes per element.
namespace {
struct DiagGroupDesc {
  int64_t r_off, count;
  int32_t rank, pair_begin, pair_count, dmask;     // dmask: output positions holding a D index
  int32_t dims[ND_MAX_RANK];
  uint32_t mul[ND_MAX_RANK], shr[ND_MAX_RANK];     // multiply-high division by dims (counts < 2^31)
};
struct DiagPairDesc {
  int64_t t_off, d_off, t_istride;                 // t_istride: sum of T strides of the contracted indices
  int64_t tst[ND_MAX_RANK];                        // T stride of each output position (0 for D positions)
  int32_t mind, pad;
};
struct DiagItem {
  int32_t group, pad;
  int64_t e0, e1;
};

__global__ void __launch_bounds__(256) bs_diag_contract(const DiagGroupDesc* groups, const DiagPairDesc* pairs,
                                                        const DiagItem* items, int nitems, const double* __restrict__ T,
                                                        const double* __restrict__ D, double* R, double alpha) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const DiagItem wi = items[it];
    const DiagGroupDesc& g = groups[wi.group];
    for (int64_t e = wi.e0 + threadIdx.x; e < wi.e1; e += blockDim.x) {
      uint32_t rem = (uint32_t)e;
      int32_t cd[ND_MAX_RANK];
      int iy = -1;
      bool diag = true;
      for (int k = 0; k < g.rank; ++k) {
        const uint32_t q = (nd_umulhi(rem, g.mul[k]) + rem) >> g.shr[k];
        const int c = (int)(rem - q * (uint32_t)g.dims[k]);
        rem = q;
        cd[k] = c;
        if ((g.dmask >> k) & 1) {
          if (iy < 0) iy = c;
          else diag = diag && (c == iy);
        }
      }
      double v = 0.0;
      if (diag) {
        for (int pi = 0; pi < g.pair_count; ++pi) {
          const DiagPairDesc& p = pairs[g.pair_begin + pi];
          int64_t toff = 0;
          for (int k = 0; k < g.rank; ++k) toff += (int64_t)cd[k] * p.tst[k];
          if (iy >= 0) {
            if (iy < p.mind) v = fma(__ldg(D + p.d_off + iy), __ldg(T + p.t_off + toff + iy * p.t_istride), v);
          } else {
            for (int i = 0; i < p.mind; ++i) v = fma(__ldg(D + p.d_off + i), __ldg(T + p.t_off + toff + i * p.t_istride), v);
          }
        }
      }
      R[g.r_off + e] = alpha * v;
    }
  }
}
}  // namespace

extern "C" nd_status nd_bs_contract_diag_f64(nd_handle h, nd_plan p, double* R, const double* T, const double* Ddiag,
                                             const int64_t* diag_offsets, double alpha) {
  if (!h || !p) return ND_ERR_ARG;
  if (p->res.npairs == 0) return ND_OK;
  if (!R || !T || !Ddiag || !diag_offsets) return nd_fail(h, ND_ERR_ARG, "bs_contract_diag: NULL argument");
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "bs_contract_diag: not during graph capture");
  const Roles& ro = p->roles;
  const BsDesc& A = p->A;
  const BsDesc& Dd = p->B;
  // D must be block diagonal (the reference's requirement, diagblocksparse.jl:652-657)
  for (int b = 0; b < Dd.nnzblocks; ++b)
    for (int d = 1; d < Dd.rank; ++d)
      if (Dd.blocks[(size_t)b * Dd.rank + d] != Dd.blocks[(size_t)b * Dd.rank]) 
        return nd_fail(h, ND_ERR_ARG, "bs_contract_diag: the DiagBlockSparse operand must be block diagonal");
  const PlanResult& r = p->res;
  const int rankR = p->rankR;
  int dmask = 0;
  for (int t = 0; t < ro.nfb; ++t) dmask |= 1 << ro.r_bfree[t];
  std::vector<std::vector<int>> by_group(r.nR);
  for (int q = 0; q < r.npairs; ++q) by_group[r.pairs[3 * q + 2]].push_back(q);
  std::vector<DiagGroupDesc> groups;
  std::vector<DiagPairDesc> pairs;
  std::vector<DiagItem> items;
  constexpr int64_t ITEM = 8192;
  for (int g = 0; g < r.nR; ++g) {
    DiagGroupDesc gd{};
    gd.r_off = r.offsetsR[g];
    gd.rank = rankR;
    gd.dmask = dmask;
    gd.pair_begin = (int32_t)pairs.size();
    gd.pair_count = (int32_t)by_group[g].size();
    int64_t count = 1;
    for (int k = 0; k < rankR; ++k) {
      const int64_t d = p->r_blockdims[k][r.blocksR[(size_t)g * rankR + k] - 1];
      gd.dims[k] = (int32_t)d;
      count *= d;
    }
    if (count >= (1ll << 31)) return nd_fail(h, ND_ERR_UNSUPPORTED, "bs_contract_diag: output block beyond 2^31 elements");
    Mixed m{};
    m.n = rankR;
    for (int k = 0; k < rankR; ++k) m.dim[k] = gd.dims[k] > 0 ? gd.dims[k] : 1;
    mixed_finalize(m);
    for (int k = 0; k < rankR; ++k) { gd.mul[k] = m.mul[k]; gd.shr[k] = m.shr[k]; }
    gd.count = count;
    for (int q : by_group[g]) {
      const int iA = r.pairs[3 * q], iD = r.pairs[3 * q + 1];
      int64_t sT[ND_MAX_RANK + 1];
      sT[0] = 1;
      for (int k = 0; k < A.rank; ++k) sT[k + 1] = sT[k] * A.bdim(iA, k);
      DiagPairDesc pd{};
      pd.t_off = A.offsets[iA];
      pd.d_off = diag_offsets[iD];
      int64_t mind = INT64_MAX;
      for (int k = 0; k < Dd.rank; ++k) mind = std::min(mind, Dd.bdim(iD, k));
      pd.mind = Dd.rank ? (int32_t)mind : 1;
      for (int t = 0; t < ro.nk; ++t) pd.t_istride += sT[ro.a_k[t]];
      for (int t = 0; t < ro.nfa; ++t) pd.tst[ro.r_afree[t]] = sT[ro.a_free[t]];
      pairs.push_back(pd);
    }
    groups.push_back(gd);
    for (int64_t e = 0; e < count; e += ITEM) items.push_back(DiagItem{g, 0, e, std::min(count, e + ITEM)});
  }
  if (items.empty()) return ND_OK;
  // one upload of the three descriptor lists, stream-ordered scratch
  const size_t bg = groups.size() * sizeof(DiagGroupDesc), bp = pairs.size() * sizeof(DiagPairDesc),
               bi = items.size() * sizeof(DiagItem);
  std::vector<unsigned char> host(bg + bp + bi);
  memcpy(host.data(), groups.data(), bg);
  memcpy(host.data() + bg, pairs.data(), bp);
  memcpy(host.data() + bg + bp, items.data(), bi);
  void* d = nullptr;
  nd_status st = nd_dalloc(h, &d, host.size());
  if (st) return st;
  if ((st = nd_upload(h, d, host.data(), host.size()))) return st;
  const int grid = (int)std::min<size_t>(items.size(), (size_t)h->num_sms * 8);
  nd_prof_begin(h, "bs_diag_contract");
  bs_diag_contract<<<grid, 256, 0, h->stream>>>((const DiagGroupDesc*)d, (const DiagPairDesc*)((unsigned char*)d + bg),
                                                (const DiagItem*)((unsigned char*)d + bg + bp), (int)items.size(), T,
                                                Ddiag, R, alpha);
  nd_prof_end(h);
  ND_LAUNCHED(h);
  cudaFreeAsync(d, h->stream);
  return nd_cuda_check(h, cudaGetLastError(), "bs_diag_contract");
}

extern "C" nd_status nd_bs_permutedims_f64(nd_handle h, const nd_bs_desc* T, const double* Tdata,
                                           const int32_t* perm, const int64_t* offsetsR, double* Rdata) {
  if (!h) return ND_ERR_ARG;
  BsDesc d;
  nd_status s = nd_bs_import(h, T, d, "bs_permutedims");
  if (s) return s;
  if (!perm || !offsetsR) return nd_fail(h, ND_ERR_ARG, "bs_permutedims: NULL perm/offsets");
  int p0[ND_MAX_RANK];
  bool seen[ND_MAX_RANK] = {false};
  for (int k = 0; k < d.rank; ++k) {
    int v = perm[k] - 1;
    if (v < 0 || v >= d.rank || seen[v]) return nd_fail(h, ND_ERR_ARG, "bs_permutedims: bad perm");
    seen[v] = true;
    p0[k] = v;
  }
  // Blocks of 2^22 elements or more go through the tiled transposer, one launch each; all
  // smaller blocks are permuted by one batched gather launch (per block: source strides
  // column-major, destination strides those of the permuted block), since a QN tensor
  // holds hundreds of small blocks and one launch per block would be launch-bound.
  constexpr int64_t kTiledBlock = int64_t(1) << 22;
  std::vector<nd_block_copy> small;
  for (int b = 0; b < d.nnzblocks; ++b) {
    int64_t dims[ND_MAX_RANK];
    int64_t n = 1;
    for (int k = 0; k < d.rank; ++k) { dims[k] = d.bdim(b, k); n *= dims[k]; }
    if (n == 0) continue;
    if (n >= kTiledBlock) {
      s = nd_launch_permute(h, Rdata + offsetsR[b], Tdata + d.offsets[b], d.rank, dims, p0, 1.0, 0.0, nullptr);
      if (s) return s;
      continue;
    }
    nd_block_copy c{};
    c.src_off = d.offsets[b];
    c.dst_off = offsetsR[b];
    c.rank = d.rank;
    int64_t st = 1;
    for (int k = 0; k < d.rank; ++k) { c.dims[k] = dims[k]; c.src_strides[k] = st; st *= dims[k]; }
    st = 1;
    for (int j = 0; j < d.rank; ++j) { c.dst_strides[p0[j]] = st; st *= dims[p0[j]]; }   // R dim j is T dim p0[j]
    small.push_back(c);
  }
  if (small.empty()) return ND_OK;
  if (small.size() > (size_t)INT32_MAX) return nd_fail(h, ND_ERR_ARG, "bs_permutedims: too many blocks");
  return nd_block_copy_f64(h, (int32_t)small.size(), small.data(), Tdata, Rdata);
}
