// Context, memory, error plumbing, label roles and CUDA-graph entry points.
#include "nd_common.h"
#include <cstdarg>
#include <cstring>
#include <algorithm>

static thread_local std::string g_noctx_error;

nd_status nd_fail(nd_handle h, nd_status code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->last_error = buf; else g_noctx_error = buf;
  return code;
}

nd_status nd_cuda_check(nd_handle h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ND_OK;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return nd_fail(h, ND_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  }
  return nd_fail(h, ND_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

nd_status nd_upload(nd_handle h, void* dst, const void* src, size_t bytes) {
  if (!bytes) return ND_OK;
  constexpr size_t kRing = 16u << 20;
  if (bytes > kRing / 4 || nd_capturing(h)) {
    ND_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
    return ND_OK;
  }
  if (!h->up_ring) {
    ND_CUDA(h, cudaHostAlloc((void**)&h->up_ring, kRing, cudaHostAllocDefault));
    h->up_cap = kRing;
    h->up_head = 0;
  }
  const size_t len = (bytes + 255) & ~(size_t)255;
  if (h->up_head + len > h->up_cap) h->up_head = 0;
  const size_t b = h->up_head, e = b + len;
  // wait for (and retire) the oldest uploads whose regions this one overwrites
  while (!h->up_fifo.empty()) {
    const nd_context::UpRec& r = h->up_fifo.front();
    if (r.end <= b || r.begin >= e) break;
    ND_CUDA(h, cudaEventSynchronize(r.ev));
    h->up_events.push_back(r.ev);
    h->up_fifo.erase(h->up_fifo.begin());
  }
  memcpy(h->up_ring + b, src, bytes);
  ND_CUDA(h, cudaMemcpyAsync(dst, h->up_ring + b, bytes, cudaMemcpyHostToDevice, h->stream));
  cudaEvent_t ev;
  if (!h->up_events.empty()) { ev = h->up_events.back(); h->up_events.pop_back(); }
  else ND_CUDA(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  ND_CUDA(h, cudaEventRecord(ev, h->stream));
  h->up_fifo.push_back(nd_context::UpRec{b, e, ev});
  h->up_head = e;
  return ND_OK;
}

unsigned long long* nd_cta_slot(nd_handle h, int nctas) {
  if (!h->cta_timing || !h->d_cta_times || nctas > ND_CTA_MAX || nd_capturing(h)) return nullptr;
  const int slot = h->cta_nlaunch % ND_CTA_SLOTS;
  h->cta_nctas[slot] = nctas;
  ++h->cta_nlaunch;
  return h->d_cta_times + (size_t)slot * 2 * ND_CTA_MAX;
}

nd_status nd_dalloc(nd_handle h, void** p, size_t bytes) {
  *p = nullptr;
  ND_CUDA(h, cudaMallocAsync(p, std::max<size_t>(bytes, 16), h->stream));
  return ND_OK;
}

bool nd_capturing(nd_handle h) {
  if (h->capturing) return true;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &st) != cudaSuccess) return false;
  return st == cudaStreamCaptureStatusActive;
}

nd_status nd_check_device_status(nd_handle h, const char* what) {
  if (nd_capturing(h)) return ND_OK;   // read after replay via nd_sync
  DeviceStatus st{};
  ND_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  ND_CUDA(h, cudaStreamSynchronize(h->stream));
  if (st.code != ND_OK) {
    const int32_t z[2] = {0, 0};              // clear code and site; keep the spin limit
    cudaMemcpy(h->d_status, z, sizeof(z), cudaMemcpyHostToDevice);
    if (st.code == ND_ERR_TIMEOUT)
      return nd_fail(h, ND_ERR_TIMEOUT, "%s: device wait exceeded its iteration limit (site %d)", what, st.where);
    if (st.code == ND_ERR_NONFINITE)
      return nd_fail(h, ND_ERR_NONFINITE, "%s: Inf/NaN input cannot be split exactly; use ND_PREC_FP64", what);
    if (st.code == ND_ERR_NOCONV)
      return nd_fail(h, ND_ERR_NOCONV, "%s: SVD did not converge (block %d)", what, st.where);
    return nd_fail(h, st.code, "%s: device reported error %d at site %d", what, st.code, st.where);
  }
  return ND_OK;
}

extern "C" {

nd_status nd_create(int32_t device, nd_handle* out) {
  if (!out) return nd_fail(nullptr, ND_ERR_ARG, "nd_create: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return nd_fail(nullptr, ND_ERR_CUDA, "nd_create: no CUDA device (%s)", cudaGetErrorString(e));
  if (device < 0 || device >= n) return nd_fail(nullptr, ND_ERR_ARG, "nd_create: bad device %d", device);
  nd_handle h = new nd_context();
  h->device = device;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete h; return nd_fail(nullptr, ND_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e)); }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  if (prop.major * 10 + prop.minor < 100) {
    delete h;
    return nd_fail(nullptr, ND_ERR_UNSUPPORTED, "nd_create: device sm_%d%d is not a Blackwell (sm_10x) GPU", prop.major, prop.minor);
  }
  h->num_sms = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return nd_fail(nullptr, ND_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
  h->own_stream = true;
  e = cudaMalloc(&h->d_status, sizeof(DeviceStatus));
  if (e != cudaSuccess) { cudaStreamDestroy(h->stream); delete h; return nd_fail(nullptr, ND_ERR_OOM, "status word"); }
  {
    const DeviceStatus init{0, 0, ND_SPIN_LIMIT, 0};
    cudaMemcpy(h->d_status, &init, sizeof(init), cudaMemcpyHostToDevice);
  }
  {
    // execution state is allocated stream-ordered from the default pool: keep freed
    // blocks in the pool instead of returning them to the system at every sync
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  cudaDeviceSynchronize();
  *out = h;
  return ND_OK;
}

nd_status nd_destroy(nd_handle h) {
  if (!h) return ND_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  nd_dense_cache_clear(h);
  if (h->ws) cudaFree(h->ws);
  if (h->pin) cudaFreeHost(h->pin);
  if (h->up_ring) cudaFreeHost(h->up_ring);
  for (auto& r : h->up_fifo) cudaEventDestroy(r.ev);
  for (auto e : h->up_events) cudaEventDestroy(e);
  if (h->order_ev) cudaEventDestroy(h->order_ev);
  if (h->vec_part) cudaFree(h->vec_part);
  if (h->plan_stream) { cudaStreamSynchronize(h->plan_stream); cudaStreamDestroy(h->plan_stream); }
  if (h->d_plan_status) cudaFree(h->d_plan_status);
  if (h->d_status) cudaFree(h->d_status);
  for (auto& r : h->prof) { cudaEventDestroy(r.e0); cudaEventDestroy(r.e1); }
  if (h->d_cta_times) cudaFree(h->d_cta_times);
  for (auto e : h->event_pool) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  delete h;
  return ND_OK;
}

const char* nd_last_error(nd_handle h) { return h ? h->last_error.c_str() : g_noctx_error.c_str(); }

nd_status nd_set_stream(nd_handle h, void* s) {
  if (!h) return ND_ERR_ARG;
  if ((cudaStream_t)s == h->stream) return ND_OK;
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "nd_set_stream: cannot change streams during graph capture");
  if (h->own_stream) {
    ND_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaStreamDestroy(h->stream);
    h->own_stream = false;
  }
  h->stream = (cudaStream_t)s;   // NULL selects the legacy default stream, as everywhere in CUDA
  return ND_OK;
}

nd_status nd_get_stream(nd_handle h, void** s) {
  if (!h || !s) return ND_ERR_ARG;
  *s = (void*)h->stream;
  return ND_OK;
}

nd_status nd_sync(nd_handle h) {
  if (!h) return ND_ERR_ARG;
  ND_CUDA(h, cudaStreamSynchronize(h->stream));
  return nd_check_device_status(h, "nd_sync");
}

nd_status nd_alloc(nd_handle h, size_t bytes, void** dptr) {
  if (!h || !dptr) return nd_fail(h, ND_ERR_ARG, "nd_alloc: NULL argument");
  *dptr = nullptr;
  if (bytes == 0) bytes = 16;
  ND_CUDA(h, cudaMalloc(dptr, bytes));
  return ND_OK;
}

nd_status nd_free(nd_handle h, void* p) {
  if (!h) return ND_ERR_ARG;
  if (p) ND_CUDA(h, cudaFree(p));
  return ND_OK;
}

nd_status nd_h2d(nd_handle h, void* dst, const void* src, size_t bytes) {
  if (!h || (bytes && (!dst || !src))) return nd_fail(h, ND_ERR_ARG, "nd_h2d: NULL argument");
  if (bytes) ND_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
  return ND_OK;
}

nd_status nd_d2h(nd_handle h, void* dst, const void* src, size_t bytes) {
  if (!h || (bytes && (!dst || !src))) return nd_fail(h, ND_ERR_ARG, "nd_d2h: NULL argument");
  if (bytes) {
    ND_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    ND_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return ND_OK;
}

nd_status nd_memset0(nd_handle h, void* dst, size_t bytes) {
  if (!h || (bytes && !dst)) return nd_fail(h, ND_ERR_ARG, "nd_memset0: NULL argument");
  if (bytes) ND_CUDA(h, cudaMemsetAsync(dst, 0, bytes, h->stream));
  return ND_OK;
}

nd_status nd_set_spin_limit(nd_handle h, uint32_t polls) {
  if (!h) return ND_ERR_ARG;
  if (nd_capturing(h)) return nd_fail(h, ND_ERR_ARG, "nd_set_spin_limit: not during graph capture");
  const uint32_t v = polls ? polls : ND_SPIN_LIMIT;
  ND_CUDA(h, cudaStreamSynchronize(h->stream));
  ND_CUDA(h, cudaMemcpy(&h->d_status->spin_limit, &v, sizeof(v), cudaMemcpyHostToDevice));
  return ND_OK;
}

nd_status nd_set_svd_max_sweeps(nd_handle h, int32_t sweeps) {
  if (!h) return ND_ERR_ARG;
  h->svd_max_sweeps = sweeps < 0 ? -1 : sweeps;
  return ND_OK;
}

nd_status nd_set_cta_timing(nd_handle h, int32_t enable) {
  if (!h) return ND_ERR_ARG;
  if (enable && !h->d_cta_times)
    ND_CUDA(h, cudaMalloc(&h->d_cta_times, sizeof(unsigned long long) * 2 * ND_CTA_SLOTS * ND_CTA_MAX));
  h->cta_timing = enable != 0;
  h->cta_nlaunch = 0;
  return ND_OK;
}

nd_status nd_cta_times_read(nd_handle h, uint64_t* times, int32_t* nctas, int32_t* nlaunch) {
  if (!h || !times || !nctas || !nlaunch) return ND_ERR_ARG;
  const int n = std::min(h->cta_nlaunch, ND_CTA_SLOTS);
  *nlaunch = n;
  if (!n) return ND_OK;
  ND_CUDA(h, cudaStreamSynchronize(h->stream));
  const int first = h->cta_nlaunch - n;
  for (int k = 0; k < n; ++k) {
    const int slot = (first + k) % ND_CTA_SLOTS;
    nctas[k] = h->cta_nctas[slot];
    ND_CUDA(h, cudaMemcpy(times + (size_t)k * 2 * ND_CTA_MAX, h->d_cta_times + (size_t)slot * 2 * ND_CTA_MAX,
                          sizeof(uint64_t) * 2 * ND_CTA_MAX, cudaMemcpyDeviceToHost));
  }
  return ND_OK;
}

nd_status nd_svd_last_info(nd_handle h, int32_t* ints, int32_t nints, double* dbls, int32_t ndbls) {
  if (!h) return ND_ERR_ARG;
  for (int32_t k = 0; ints && k < nints; ++k) ints[k] = k < (int32_t)h->svd_info_i.size() ? h->svd_info_i[k] : 0;
  for (int32_t k = 0; dbls && k < ndbls; ++k) dbls[k] = k < (int32_t)h->svd_info_d.size() ? h->svd_info_d[k] : 0.0;
  return ND_OK;
}

nd_status nd_set_split_tile(nd_handle h, int32_t shape) {
  if (!h) return ND_ERR_ARG;
  if (shape != 0 && shape != 1) return nd_fail(h, ND_ERR_ARG, "split tile shape must be 0 (128x64) or 1 (256x64 on CTA pairs)");
  h->split_pair2 = shape;
  return ND_OK;
}

nd_status nd_set_plan_placement(nd_handle h, int32_t where) {
  if (!h) return ND_ERR_ARG;
  if (where < 0 || where > 2) return nd_fail(h, ND_ERR_ARG, "plan placement must be 0 (by size), 1 (device) or 2 (host)");
  h->plan_where = where;
  return ND_OK;
}

nd_status nd_set_permute_path(nd_handle h, int32_t path) {
  if (!h) return ND_ERR_ARG;
  if (path != 0 && path != 1) return nd_fail(h, ND_ERR_ARG, "permute path must be 0 (dimension-group tiles) or 1 (TMA tiles)");
  h->permute_tma = path;
  return ND_OK;
}

nd_status nd_set_verify(nd_handle h, int32_t on) {
  if (!h) return ND_ERR_ARG;
  h->verify = on ? 1 : 0;
  h->verify_err = -1.0;
  return ND_OK;
}

nd_status nd_verify_last(nd_handle h, double* rel_err) {
  if (!h || !rel_err) return ND_ERR_ARG;
  *rel_err = h->verify_err;
  return ND_OK;
}

nd_status nd_set_ozaki_slices(nd_handle h, int32_t s) {
  if (!h) return ND_ERR_ARG;
  if (s < 3 || s > 6) return nd_fail(h, ND_ERR_ARG, "ozaki slices must be in 3..6 (got %d)", s);
  h->ozaki_slices = s;
  return ND_OK;
}

// ---- autotuner cache ---------------------------------------------------------
// File format: '#' comment lines, then one line per entry:
//   <key> TAB <splitk_mult> TAB <skinny> TAB <pair2> TAB <best_ms> TAB <default_ms>
// (version 1 files, without the pair2 column, load with the default tile shape)
nd_status nd_tune_enable(nd_handle h, int32_t enable) {
  if (!h) return ND_ERR_ARG;
  h->tuning = enable != 0;
  return ND_OK;
}

nd_status nd_tune_count(nd_handle h, int32_t* entries) {
  if (!h || !entries) return ND_ERR_ARG;
  *entries = (int32_t)h->tune.size();
  return ND_OK;
}

nd_status nd_tune_save(nd_handle h, const char* path) {
  if (!h) return ND_ERR_ARG;
  if (!path) return nd_fail(h, ND_ERR_ARG, "tune_save: NULL path");
  FILE* f = std::fopen(path, "w");
  if (!f) return nd_fail(h, ND_ERR_ARG, "tune_save: cannot open %s", path);
  std::fprintf(f, "# ndtensors_gb300 autotune cache v2: key splitk_mult skinny pair2 best_ms default_ms\n");
  for (const auto& e : h->tune)
    std::fprintf(f, "%s\t%d\t%d\t%d\t%.6f\t%.6f\n", e.first.c_str(), e.second.choice.splitk_mult,
                 e.second.choice.skinny, e.second.choice.pair2, e.second.best_ms, e.second.default_ms);
  const bool ok = std::fclose(f) == 0;
  return ok ? ND_OK : nd_fail(h, ND_ERR_ARG, "tune_save: write to %s failed", path);
}

nd_status nd_tune_load(nd_handle h, const char* path) {
  if (!h) return ND_ERR_ARG;
  if (!path) return nd_fail(h, ND_ERR_ARG, "tune_load: NULL path");
  FILE* f = std::fopen(path, "r");
  if (!f) return nd_fail(h, ND_ERR_ARG, "tune_load: cannot open %s", path);
  std::map<std::string, TuneEntry> got;
  char line[8192];
  int lineno = 0;
  nd_status st = ND_OK;
  while (std::fgets(line, sizeof line, f)) {
    ++lineno;
    size_t n = std::strlen(line);
    if (n + 1 == sizeof line && line[n - 1] != '\n') { st = nd_fail(h, ND_ERR_ARG, "tune_load: line %d too long", lineno); break; }
    while (n && (line[n - 1] == '\n' || line[n - 1] == '\r')) line[--n] = 0;
    if (!n || line[0] == '#') continue;
    char* tab = std::strchr(line, '\t');
    TuneEntry e;
    int used = 0;
    bool parsed = false;
    if (tab) {
      int nf = 0;
      int ntabs = 0;
      for (const char* c = tab + 1; *c; ++c) ntabs += *c == '\t';
      if (ntabs == 4)
        nf = std::sscanf(tab + 1, "%d\t%d\t%d\t%lf\t%lf%n", &e.choice.splitk_mult, &e.choice.skinny,
                         &e.choice.pair2, &e.best_ms, &e.default_ms, &used) == 5;
      else if (ntabs == 3)
        nf = std::sscanf(tab + 1, "%d\t%d\t%lf\t%lf%n", &e.choice.splitk_mult, &e.choice.skinny, &e.best_ms,
                         &e.default_ms, &used) == 4;
      parsed = nf && tab[1 + used] == 0;
    }
    if (!parsed || e.choice.splitk_mult < 0 || e.choice.splitk_mult > 64 ||
        (e.choice.skinny != 0 && e.choice.skinny != 1) || (e.choice.pair2 != 0 && e.choice.pair2 != 1)) {
      st = nd_fail(h, ND_ERR_ARG, "tune_load: malformed entry at %s:%d", path, lineno);
      break;
    }
    got[std::string(line, tab - line)] = e;
  }
  std::fclose(f);
  if (st) return st;
  for (auto& e : got) h->tune[e.first] = e.second;
  return ND_OK;
}

nd_status nd_launch_count(nd_handle h, int64_t* c) {
  if (!h || !c) return ND_ERR_ARG;
  *c = h->launches;
  return ND_OK;
}

nd_status nd_profile_enable(nd_handle h, int32_t enable) {
  if (!h) return ND_ERR_ARG;
  h->profiling = enable != 0;
  return ND_OK;
}

nd_status nd_profile_read(nd_handle h, int32_t cap, char* names, int64_t* counts, double* total_ms, int32_t* n_out) {
  if (!h || !n_out) return ND_ERR_ARG;
  ND_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<std::string> keys;
  std::vector<int64_t> cnt;
  std::vector<double> tot;
  // a region still open (its end not recorded) counts zero time
  std::vector<char> open(h->prof.size(), 0);
  for (size_t i : h->prof_open) open[i] = 1;
  for (size_t i = 0; i < h->prof.size(); ++i) {
    const nd_context::ProfRec& r = h->prof[i];
    float ms = 0.f;
    if (!open[i] && cudaEventElapsedTime(&ms, r.e0, r.e1) != cudaSuccess) {
      (void)cudaGetLastError();
      ms = 0.f;
    }
    size_t k = 0;
    for (; k < keys.size(); ++k) if (keys[k] == r.name) break;
    if (k == keys.size()) { keys.push_back(r.name); cnt.push_back(0); tot.push_back(0.0); }
    cnt[k]++;
    tot[k] += ms;
    h->event_pool.push_back(r.e0);
    h->event_pool.push_back(r.e1);
  }
  h->prof.clear();
  h->prof_open.clear();
  int n = (int)keys.size();
  for (int k = 0; k < n && k < cap; ++k) {
    if (names) { strncpy(names + 64 * k, keys[k].c_str(), 63); names[64 * k + 63] = 0; }
    if (counts) counts[k] = cnt[k];
    if (total_ms) total_ms[k] = tot[k];
  }
  *n_out = n;
  return ND_OK;
}

nd_status nd_graph_begin(nd_handle h) {
  if (!h) return ND_ERR_ARG;
  if (h->capturing) return nd_fail(h, ND_ERR_ARG, "nd_graph_begin: already capturing");
  ND_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  h->capturing = true;
  return ND_OK;
}

nd_status nd_graph_end(nd_handle h, void** exec) {
  if (!h || !exec) return ND_ERR_ARG;
  if (!h->capturing) return nd_fail(h, ND_ERR_ARG, "nd_graph_end: not capturing");
  cudaGraph_t g = nullptr;
  h->capturing = false;
  ND_CUDA(h, cudaStreamEndCapture(h->stream, &g));
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return nd_cuda_check(h, e, "cudaGraphInstantiate");
  *exec = (void*)ge;
  return ND_OK;
}

nd_status nd_graph_launch(nd_handle h, void* exec) {
  if (!h || !exec) return ND_ERR_ARG;
  ND_CUDA(h, cudaGraphLaunch((cudaGraphExec_t)exec, h->stream));
  return ND_OK;
}

nd_status nd_graph_destroy(void* exec) {
  if (exec) cudaGraphExecDestroy((cudaGraphExec_t)exec);
  return ND_OK;
}

}  // extern "C"

void nd_prof_begin(nd_handle h, const char* name) {
  if (!h->profiling || nd_capturing(h)) return;
  auto get = [&]() {
    if (!h->event_pool.empty()) { cudaEvent_t e = h->event_pool.back(); h->event_pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  };
  nd_context::ProfRec r{name, get(), get()};
  cudaEventRecord(r.e0, h->stream);
  h->prof_open.push_back(h->prof.size());
  h->prof.push_back(r);
}

void nd_prof_end(nd_handle h) {
  if (!h->profiling || nd_capturing(h) || h->prof_open.empty()) return;
  cudaEventRecord(h->prof[h->prof_open.back()].e1, h->stream);
  h->prof_open.pop_back();
}


// ---------------------------------------------------------------------------
// Label roles: which dimensions of A and B are free / contracted and where the
// free ones land in R (contract_labels / find_matching_positions,
// NDTensors/src/tensoroperations/contraction_logic.jl:5-55,
// NDTensors/src/blocksparse/contract_utilities.jl:28-55).
// ---------------------------------------------------------------------------
bool nd_make_roles(int rankA, const int32_t* la, int rankB, const int32_t* lb, int rankR,
                   const int32_t* lr, Roles& ro, std::string& why) {
  memset(&ro, 0, sizeof(ro));
  if (rankA < 0 || rankB < 0 || rankR < 0 || rankA > ND_MAX_RANK || rankB > ND_MAX_RANK || rankR > ND_MAX_RANK) {
    why = "rank out of range (max 8)";
    return false;
  }
  ro.rankA = rankA; ro.rankB = rankB; ro.rankR = rankR;
  for (int i = 0; i < rankA; ++i)
    for (int j = i + 1; j < rankA; ++j)
      if (la[i] == la[j]) { why = "repeated label in A"; return false; }
  for (int i = 0; i < rankB; ++i)
    for (int j = i + 1; j < rankB; ++j)
      if (lb[i] == lb[j]) { why = "repeated label in B"; return false; }
  for (int i = 0; i < rankR; ++i)
    for (int j = i + 1; j < rankR; ++j)
      if (lr[i] == lr[j]) { why = "repeated label in R"; return false; }
  auto find = [](const int32_t* l, int n, int x) { for (int i = 0; i < n; ++i) if (l[i] == x) return i; return -1; };
  int nfree = 0;
  for (int i = 0; i < rankA; ++i) {
    int j = find(lb, rankB, la[i]);
    if (j >= 0) { ro.a_k[ro.nk] = i; ro.b_k[ro.nk] = j; ro.nk++; }
    else nfree++;
  }
  for (int j = 0; j < rankB; ++j)
    if (find(la, rankA, lb[j]) < 0) nfree++;
  if (nfree != rankR) { why = "output labels must be exactly the uncontracted labels"; return false; }
  // free dims ordered by their position in R
  for (int r = 0; r < rankR; ++r) {
    int i = find(la, rankA, lr[r]);
    int j = find(lb, rankB, lr[r]);
    if (i >= 0 && find(lb, rankB, lr[r]) < 0) { ro.a_free[ro.nfa] = i; ro.r_afree[ro.nfa] = r; ro.nfa++; }
    else if (j >= 0 && find(la, rankA, lr[r]) < 0) { ro.b_free[ro.nfb] = j; ro.r_bfree[ro.nfb] = r; ro.nfb++; }
    else { why = "output label not found among the uncontracted labels"; return false; }
  }
  return true;
}
