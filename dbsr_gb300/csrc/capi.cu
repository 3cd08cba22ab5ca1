// capi.cu -- the extern "C" entry points declared in include/dbsrg.h.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "internal.cuh"

int set_err(dbsrg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_check(dbsrg_ctx *c, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return DBSRG_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_err(c, DBSRG_ENOMEM, m);
  return set_err(c, DBSRG_ECUDA, m);
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int copy_in_s(dbsrg_ctx *c, void *dst, const void *src, size_t n, cudaStream_t s) {
  if (n == 0) return DBSRG_OK;
  if (!src) return set_err(c, DBSRG_EINVAL, "null input pointer");
  cudaMemcpyKind k = is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  DBSRG_TRY(c, cudaMemcpyAsync(dst, src, n, k, s));
  return DBSRG_OK;
}

int copy_in(dbsrg_ctx *c, void *dst, const void *src, size_t n) {
  return copy_in_s(c, dst, src, n, c->stream);
}

// Waits for both streams, then reads and clears the error word of the
// tensor-core kernels (a bounded wait that ran out, or inconsistent tile
// terms).
int drain(dbsrg_ctx *c) {
  c->pending = false;
  if (c->sstream) DBSRG_TRY(c, cudaStreamSynchronize(c->sstream));
  for (cudaStream_t b : c->bstream)
    if (b) DBSRG_TRY(c, cudaStreamSynchronize(b));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  if (!c->kerr) return DBSRG_OK;
  int h = 0;
  DBSRG_TRY(c, cudaMemcpyAsync(&h, c->kerr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  if (!h) return DBSRG_OK;
  DBSRG_TRY(c, cudaMemsetAsync(c->kerr, 0, sizeof(int), c->stream));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  if (h == 1) return set_err(c, DBSRG_ETIMEOUT, "tensor-core exchange: a wait ran out");
  return set_err(c, DBSRG_ECUDA, "tensor-core exchange: inconsistent tile terms");
}

// blocks of the current window that exist (the last window may run past iicc)
static int window_blocks(const dbsrg_ctx *c) { return std::min(c->wcap, c->iicc - c->wlo + 1); }

// queued work of the asynchronous mode is finished (and its errors read)
// before any call that reads results or changes state
#define SETTLE(c)                  \
  do {                             \
    if ((c)->pending) {            \
      int _r = drain(c);           \
      if (_r) return _r;           \
    }                              \
  } while (0)

int raise_smem_limit(dbsrg_ctx *c, const void *fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{c->device, fn}];
  if (bytes <= cur || bytes <= 48 * 1024) return DBSRG_OK;
  DBSRG_TRY(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return DBSRG_OK;
}

int copy_out(dbsrg_ctx *c, void *dst, const void *src, size_t n) {
  if (n == 0) return DBSRG_OK;
  if (!dst) return set_err(c, DBSRG_EINVAL, "null output pointer");
  cudaMemcpyKind k = is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  DBSRG_TRY(c, cudaMemcpyAsync(dst, src, n, k, c->stream));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

// A scratch buffer that must grow: queued work may still read the old one,
// so it is retired (freed when the context is destroyed or its memory
// trimmed) rather than freed -- growing waits for nothing, neither the
// context's streams nor (through cudaFree) the whole device -- and the new
// one is at least twice the old one, which bounds the retired memory by
// the final size.
int grow_buffer(dbsrg_ctx *c, void **p, size_t *have, size_t bytes) {
  if (*have >= bytes) return DBSRG_OK;
  size_t want = std::max(bytes + bytes / 4, 2 * *have);
  if (*p) {
    c->retired.push_back(*p);
    *p = nullptr;
    *have = 0;
  }
  cudaError_t e = cudaMalloc(p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      *p = nullptr;
      return cuda_check(c, e, "scratch allocation");
    }
    want = bytes;
  }
  *have = want;
  return DBSRG_OK;
}

int ensure_scratch(dbsrg_ctx *c, size_t bytes) {
  return grow_buffer(c, &c->scratch, &c->scratch_bytes, bytes);
}
int ensure_scratch2(dbsrg_ctx *c, size_t bytes) {
  return grow_buffer(c, &c->scratch2, &c->scratch2_bytes, bytes);
}
int ensure_tscratch(dbsrg_ctx *c, size_t bytes) {
  return grow_buffer(c, &c->tscratch, &c->tscratch_bytes, bytes);
}
int ensure_tcscratch(dbsrg_ctx *c, size_t bytes) {
  return grow_buffer(c, &c->tcscratch, &c->tcscratch_bytes, bytes);
}
int ensure_pscratch(dbsrg_ctx *c, int which, size_t bytes) {
  return grow_buffer(c, &c->pscratch[which], &c->pscratch_bytes[which], bytes);
}
void *cache_alloc(dbsrg_ctx *c, size_t bytes) {
  auto it = c->pool.find(bytes);
  void *p = nullptr;
  if (it != c->pool.end()) {
    p = it->second;
    c->pool.erase(it);
  } else if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    pool_trim(c);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  c->psize[p] = bytes;
  return p;
}

void cache_free(dbsrg_ctx *c, void *p) {
  if (!p) return;
  auto it = c->psize.find(p);
  if (it == c->psize.end()) {
    cudaFree(p);
    return;
  }
  c->pool.emplace(it->second, p);
  c->psize.erase(it);
}

void pool_trim(dbsrg_ctx *c) {
  graph_drop(c);
  if (!c->pool.empty() || !c->retired.empty()) {
    // the pooled and retired buffers may be named by queued work on any of
    // the context's streams
    if (c->sstream) cudaStreamSynchronize(c->sstream);
    for (cudaStream_t b : c->bstream)
      if (b) cudaStreamSynchronize(b);
    cudaStreamSynchronize(c->stream);
  }
  for (auto &kv : c->pool) cudaFree(kv.second);
  c->pool.clear();
  for (void *p : c->retired) cudaFree(p);
  c->retired.clear();
}

int ensure_lstate(dbsrg_ctx *c, int par, size_t bytes) {
  return grow_buffer(c, &c->lstate[par], &c->lstate_bytes[par], bytes);
}
bool sync_check_enabled() {
  // read once; the initialisation of a function-local static is thread-safe
  // (the contexts of a batch run on their own host threads)
  static const bool v = [] {
    const char *e = getenv("DBSRG_SYNC_CHECK");
    return e && e[0] == '1';
  }();
  return v;
}
int ensure_pinned(dbsrg_ctx *c, size_t bytes) {
  if (c->pinned_bytes >= bytes) return DBSRG_OK;
  if (c->pinned) cudaFreeHost(c->pinned);
  c->pinned = nullptr;
  c->pinned_bytes = 0;
  DBSRG_TRY(c, cudaMallocHost(&c->pinned, bytes));
  c->pinned_bytes = bytes;
  return DBSRG_OK;
}

cudaEvent_t event_get(dbsrg_ctx *c) {
  cudaEvent_t e = nullptr;
  if (!c->evpool.empty()) {
    e = c->evpool.back();
    c->evpool.pop_back();
    return e;
  }
  cudaEventCreate(&e);
  return e;
}

static void timing_clear(dbsrg_ctx *c) {
  for (auto &t : c->tev) {
    c->evpool.push_back(t.a);
    c->evpool.push_back(t.b);
  }
  c->tev.clear();
}

void free_tables(dbsrg_ctx *c) {
  graph_drop(c);
  for (double *p : c->rtab)
    cache_free(c, p);
  for (double *p : c->stab)
    cache_free(c, p);
  for (double *p : c->quad)
    cache_free(c, p);
  for (double *p : c->rbtab)
    cache_free(c, p);
  for (double *p : c->sbtab)
    cache_free(c, p);
  c->rbtab.clear();
  c->sbtab.clear();
  for (auto &cd : c->rcell)
    cache_free(c, cd.lo1);
  for (auto &cd : c->scell)
    cache_free(c, cd.lo1);
  free_orbital_products(c);
  c->rtab.clear();
  c->stab.clear();
  c->quad.clear();
  c->rcell.clear();
  c->scell.clear();
}

// the mappings of dbsrg_host_alloc and their lengths
static std::mutex &host_mu() {
  static std::mutex m;
  return m;
}
static std::map<void *, size_t> &host_sizes() {
  static std::map<void *, size_t> m;
  return m;
}

extern "C" {

int dbsrg_create(dbsrg_ctx **out, const dbsrg_grid_desc *d) {
  if (!out || !d) return DBSRG_EINVAL;
  *out = nullptr;
  if (d->ns < 2 || d->ks < 2 || d->ks > DBSRG_MAXK || d->ksp < 2 || d->ksp > d->ks ||
      d->ksq < 2 || d->ksq > d->ks || d->ns < d->ks || !d->t)
    return DBSRG_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= d->device || d->device < 0) {
    cudaGetLastError();
    return DBSRG_ECUDA;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, d->device) != cudaSuccess) return DBSRG_ECUDA;
  if (prop.major * 10 + prop.minor < 100) return DBSRG_ECUDA;  // built for sm_103a only
  dbsrg_ctx *c = new (std::nothrow) dbsrg_ctx();
  if (!c) return DBSRG_ENOMEM;
  c->device = d->device;
  c->nsm = prop.multiProcessorCount;
  if (cudaSetDevice(d->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return DBSRG_ECUDA;
  }
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithFlags(&c->sstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->bstream[0], cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->bstream[1], cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->tready[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->tready[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->sready, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->cdone[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->cdone[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->wdone, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->lfree[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->lfree[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->lready, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    dbsrg_destroy(c);
    return DBSRG_ECUDA;
  }
  DeviceGrid &g = c->g;
  g.ns = d->ns;
  g.ks = d->ks;
  g.ksp = d->ksp;
  g.ksq = d->ksq;
  g.nv = g.ns - g.ks + 1;
  g.nsp = g.nv + g.ksp - 1;
  g.nsq = g.nv + g.ksq - 1;
  g.ms = 2 * g.ns;
  int rc = build_grid(c, d->t);
  if (rc) {
    dbsrg_destroy(c);
    return rc;
  }
  *out = c;
  return DBSRG_OK;
}

int dbsrg_destroy(dbsrg_ctx *c) {
  if (!c) return DBSRG_OK;
  cudaSetDevice(c->device);
  if (c->sstream) cudaStreamSynchronize(c->sstream);
  if (c->cstream) cudaStreamSynchronize(c->cstream);
  for (cudaStream_t b : c->bstream)
    if (b) cudaStreamSynchronize(b);
  if (c->stream) cudaStreamSynchronize(c->stream);
  basis_release(c);
  free_tables(c);
  free_structures(c);
  pool_trim(c);
  DeviceGrid &g = c->g;
  double *arrs[] = {g.t, g.tp, g.tq, g.gx, g.gw, g.gr, g.grw, g.grm,
                    g.pbsp, g.qbsp, g.fpbs, g.fqbs, g.fppqq, g.tri};
  for (double *p : arrs)
    if (p) cudaFree(p);
  if (c->pq) cudaFree(c->pq);
  if (c->ipbs) cudaFree(c->ipbs);
  if (c->icc) cudaFree(c->icc);
  if (c->hmem) cudaFree(c->hmem);
  if (c->acf) cudaFree(c->acf);
  if (c->scratch) cudaFree(c->scratch);
  if (c->scratch2) cudaFree(c->scratch2);
  if (c->tscratch) cudaFree(c->tscratch);
  if (c->fscratch) cudaFree(c->fscratch);
  if (c->tcscratch) cudaFree(c->tcscratch);
  for (void *p : c->pscratch)
    if (p) cudaFree(p);
  for (int i = 0; i < 2; i++) {
    if (c->lstate[i]) cudaFree(c->lstate[i]);
    if (c->lfree[i]) cudaEventDestroy(c->lfree[i]);
  }
  if (c->lready) cudaEventDestroy(c->lready);
  for (cudaEvent_t e : {c->cdone[0], c->cdone[1], c->wdone, c->tready[0], c->tready[1], c->sready})
    if (e) cudaEventDestroy(e);
  if (c->kerr) cudaFree(c->kerr);
  if (c->bmap) cudaFree(c->bmap);
  if (c->b2o) cudaFree(c->b2o);
  if (c->pinned) cudaFreeHost(c->pinned);
  timing_clear(c);
  for (cudaEvent_t e : c->evpool) cudaEventDestroy(e);
  if (c->sstream) cudaStreamDestroy(c->sstream);
  if (c->cstream) cudaStreamDestroy(c->cstream);
  for (cudaStream_t b : c->bstream)
    if (b) cudaStreamDestroy(b);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return DBSRG_OK;
}

int dbsrg_release_tables(dbsrg_ctx *c) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  free_tables(c);
  pool_trim(c);
  return DBSRG_OK;
}

int dbsrg_invalidate_tables(dbsrg_ctx *c) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  free_tables(c);  // the buffers stay in the pool for the rebuild
  return DBSRG_OK;
}

int dbsrg_timing(dbsrg_ctx *c, int enable) {
  if (!c) return DBSRG_EINVAL;
  SETTLE(c);
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  timing_clear(c);
  c->timing = enable != 0;
  return DBSRG_OK;
}

int dbsrg_timing_report(dbsrg_ctx *c, char *buf, size_t len) {
  if (!c || !buf || len < 3) return DBSRG_EINVAL;
  SETTLE(c);
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  std::vector<std::string> names;
  std::vector<long long> cnt;
  std::vector<double> ms, by, fl;
  for (auto &t : c->tev) {
    float m = 0.f;
    if (cudaEventElapsedTime(&m, t.a, t.b) != cudaSuccess) {
      cudaGetLastError();
      m = 0.f;
    }
    size_t i = 0;
    while (i < names.size() && names[i] != t.name) i++;
    if (i == names.size()) {
      names.push_back(t.name);
      cnt.push_back(0);
      ms.push_back(0.0);
      by.push_back(0.0);
      fl.push_back(0.0);
    }
    cnt[i]++;
    ms[i] += m;
    by[i] += t.bytes;
    fl[i] += t.flops;
  }
  std::string s = "{";
  for (size_t i = 0; i < names.size(); i++) {
    char tmp[320];
    snprintf(tmp, sizeof tmp, "%s\"%s\": [%lld, %.6f, %.6e, %.6e]", i ? ", " : "",
             names[i].c_str(), cnt[i], ms[i], by[i], fl[i]);
    s += tmp;
  }
  s += "}";
  if (s.size() + 1 > len) return set_err(c, DBSRG_EINVAL, "timing report buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return DBSRG_OK;
}

const char *dbsrg_last_error(const dbsrg_ctx *c) { return c ? c->err.c_str() : "no context"; }

long long dbsrg_kernel_launches(const dbsrg_ctx *c) { return c ? c->launches : 0; }

int dbsrg_sync(dbsrg_ctx *c) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  return drain(c);
}

int dbsrg_set_tuning(dbsrg_ctx *c, const char *name, int value) {
  if (!c || !name) return DBSRG_EINVAL;
  SETTLE(c);
  if (!strcmp(name, "xchunk")) {
    if (value < 2 || value > 4096) return set_err(c, DBSRG_ERANGE, "xchunk: 2..4096");
    c->tune_xchunk = value;
  } else if (!strcmp(name, "dchunk")) {
    if (value < 2 || value > 65535) return set_err(c, DBSRG_ERANGE, "dchunk: 2..65535");
    c->tune_dchunk = value;
  } else if (!strcmp(name, "windows")) {
    if (value < 1 || value > 1024) return set_err(c, DBSRG_ERANGE, "windows: 1..1024");
    c->tune_windows = value;
  } else {
    return set_err(c, DBSRG_EINVAL, "unknown tuning parameter");
  }
  return DBSRG_OK;
}

int dbsrg_set_wait_limit(dbsrg_ctx *c, long long ns) {
  if (!c) return DBSRG_EINVAL;
  if (ns < 1000 || ns > 60000000000LL) return set_err(c, DBSRG_ERANGE, "wait limit: 1 us .. 60 s");
  SETTLE(c);
  c->wait_ns = (unsigned long long)ns;
  return DBSRG_OK;
}

int dbsrg_inject_wait_timeout(dbsrg_ctx *c, int enable) {
  if (!c) return DBSRG_EINVAL;
  SETTLE(c);
  c->inject_wait = enable != 0;
  return DBSRG_OK;
}

int dbsrg_get_tuning(const dbsrg_ctx *c, const char *name, int *value) {
  if (!c || !name || !value) return DBSRG_EINVAL;
  if (!strcmp(name, "xchunk")) *value = c->tune_xchunk;
  else if (!strcmp(name, "dchunk")) *value = c->tune_dchunk;
  else if (!strcmp(name, "windows")) *value = c->tune_windows;
  else return DBSRG_EINVAL;
  return DBSRG_OK;
}

int dbsrg_set_async(dbsrg_ctx *c, int enable) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  c->async = enable != 0;
  return DBSRG_OK;
}

int dbsrg_set_orbitals(dbsrg_ctx *c, int nbf, const double *pq, const int *ipbs) {
  if (!c || nbf < 1 || !pq || !ipbs) return set_err(c, DBSRG_EINVAL, "bad orbital arguments");
  cudaSetDevice(c->device);
  SETTLE(c);
  graph_drop(c);
  if (c->pq) cudaFree(c->pq);
  if (c->ipbs) cudaFree(c->ipbs);
  c->pq = nullptr;
  c->ipbs = nullptr;
  for (double *p : c->quad) cache_free(c, p);
  c->quad.clear();
  size_t n = (size_t)2 * c->g.ns * nbf;
  DBSRG_TRY(c, cudaMalloc((void **)&c->pq, n * sizeof(double)));
  DBSRG_TRY(c, cudaMalloc((void **)&c->ipbs, nbf * sizeof(int)));
  int rc = copy_in(c, c->pq, pq, n * sizeof(double));
  if (rc) return rc;
  c->h_ipbs.assign(nbf, 0);
  if (is_device_ptr(ipbs)) {
    DBSRG_TRY(c, cudaMemcpy(c->h_ipbs.data(), ipbs, nbf * sizeof(int), cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(c->h_ipbs.data(), ipbs, nbf * sizeof(int));
  }
  rc = copy_in(c, c->ipbs, c->h_ipbs.data(), nbf * sizeof(int));
  if (rc) return rc;
  // dense numbering of the bound orbitals (ipbs = 0) for the factored path
  free_orbital_products(c);
  if (c->bmap) cudaFree(c->bmap);
  if (c->b2o) cudaFree(c->b2o);
  c->bmap = nullptr;
  c->b2o = nullptr;
  c->h_bmap.assign(nbf, -1);
  std::vector<int> b2o;
  for (int o = 0; o < nbf; o++)
    if (c->h_ipbs[o] == 0) {
      c->h_bmap[o] = (int)b2o.size();
      b2o.push_back(o + 1);
    }
  c->nbound = (int)b2o.size();
  DBSRG_TRY(c, cudaMalloc((void **)&c->bmap, nbf * sizeof(int)));
  DBSRG_TRY(c, cudaMalloc((void **)&c->b2o, (b2o.size() + 1) * sizeof(int)));
  if ((rc = copy_in(c, c->bmap, c->h_bmap.data(), nbf * sizeof(int)))) return rc;
  if (!b2o.empty() && (rc = copy_in(c, c->b2o, b2o.data(), b2o.size() * sizeof(int)))) return rc;
  if (nbf != c->nbf) c->h_kbs.clear();  // the orbital kappas of dbsrg_set_dhl no longer apply
  c->nbf = nbf;
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_alloc_matrix(dbsrg_ctx *c, int nch, const int *icc, int iicc, int mk) {
  return dbsrg_alloc_matrix_window(c, nch, icc, iicc, mk, iicc);
}

int dbsrg_alloc_matrix_window(dbsrg_ctx *c, int nch, const int *icc, int iicc, int mk,
                              int nwin) {
  if (!c || nch < 1 || !icc || iicc < 1 || mk < 0 || nwin < 1 || nwin > iicc)
    return set_err(c, DBSRG_EINVAL, "bad matrix arguments");
  cudaSetDevice(c->device);
  SETTLE(c);
  graph_drop(c);
  if (c->icc) cudaFree(c->icc);
  if (c->hmem) cudaFree(c->hmem);
  if (c->acf) cudaFree(c->acf);
  // the perturber and target parts are laid out over the channels: a new
  // matrix drops them (dbsrg_alloc_perturbers / dbsrg_set_targets again)
  for (double **p : {&c->hcp, &c->hp, &c->htarg, &c->otarg}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  c->npert = c->iicb = c->iibb = c->ntarg = 0;
  c->h_icb.clear();
  c->h_ibb.clear();
  c->h_iptar.clear();
  c->icc = nullptr;
  c->hch = c->hmem = nullptr;
  c->hcap = 0;
  c->acf = nullptr;
  c->h_icc.assign((size_t)nch * nch, 0);
  if (is_device_ptr(icc)) {
    DBSRG_TRY(c, cudaMemcpy(c->h_icc.data(), icc, sizeof(int) * nch * nch, cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(c->h_icc.data(), icc, sizeof(int) * (size_t)nch * nch);
  }
  for (int v : c->h_icc)
    if (v < 0 || v > iicc) return set_err(c, DBSRG_ERANGE, "icc entry out of range");
  const size_t ms = c->g.ms;
  DBSRG_TRY(c, cudaMalloc((void **)&c->icc, sizeof(int) * (size_t)nch * nch));
  DBSRG_TRY(c, cudaMalloc((void **)&c->hmem, sizeof(double) * ms * ms * nwin));
  c->hch = c->hmem;
  c->hcap = nwin;
  DBSRG_TRY(c, cudaMalloc((void **)&c->acf, sizeof(double) * (size_t)iicc * (mk + 1)));
  int rc = copy_in(c, c->icc, c->h_icc.data(), sizeof(int) * (size_t)nch * nch);
  if (rc) return rc;
  c->nch = nch;
  c->iicc = iicc;
  c->mk = mk;
  c->wlo = 1;
  c->wcap = nwin;
  return dbsrg_zero_matrix(c);
}

int dbsrg_set_window(dbsrg_ctx *c, int blo) {
  if (!c) return DBSRG_EINVAL;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (blo < 1 || blo > c->iicc) return set_err(c, DBSRG_ERANGE, "window start out of range");
  cudaSetDevice(c->device);
  SETTLE(c);
  c->wlo = blo;
  const size_t ms = c->g.ms;
  DBSRG_TRY(c, cudaMemsetAsync(c->hch, 0, sizeof(double) * ms * ms * c->wcap, c->stream));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_zero_matrix(dbsrg_ctx *c) {
  if (!c || !c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  cudaSetDevice(c->device);
  SETTLE(c);
  const size_t ms = c->g.ms;
  DBSRG_TRY(c, cudaMemsetAsync(c->hch, 0, sizeof(double) * ms * ms * c->wcap, c->stream));
  DBSRG_TRY(c, cudaMemsetAsync(c->acf, 0, sizeof(double) * (size_t)c->iicc * (c->mk + 1), c->stream));
  int rc = zero_structures(c);
  if (rc) return rc;
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_set_precision(dbsrg_ctx *c, int p) {
  if (!c) return DBSRG_EINVAL;
  if (p != DBSRG_PLAIN_FP64 && p != DBSRG_SPLIT_BF16 && p != DBSRG_FACTOR_FP64)
    return set_err(c, DBSRG_EINVAL, "unknown precision");
  SETTLE(c);
  c->precision = p;
  return DBSRG_OK;
}

int dbsrg_gen_matrix(dbsrg_ctx *c, int icase, int itype, int kpol, int ncdata, const int *ipt,
                     const int *k1, const int *k2, const int *k3, const int *k4,
                     const double *cdata) {
  if (!c) return DBSRG_EINVAL;
  if (ncdata < 0) return set_err(c, DBSRG_EINVAL, "ncdata < 0");
  if (ncdata == 0) return DBSRG_OK;
  if (!k1 || !k2 || !k3 || !cdata) return set_err(c, DBSRG_EINVAL, "null list pointer");
  cudaSetDevice(c->device);
  return gen_matrix_plain(c, icase, itype, kpol, ncdata, ipt, k1, k2, k3, k4, cdata);
}

int dbsrg_gen_batch(int nctx, dbsrg_ctx *const *ctxs, const int *nlists,
                    const dbsrg_list *lists) {
  if (nctx < 0 || (nctx > 0 && (!ctxs || !nlists))) return DBSRG_EINVAL;
  std::vector<size_t> off((size_t)nctx + 1, 0);
  for (int i = 0; i < nctx; i++) {
    if (!ctxs[i] || nlists[i] < 0) return DBSRG_EINVAL;
    off[i + 1] = off[i] + (size_t)nlists[i];
  }
  if (off[nctx] > 0 && !lists) return DBSRG_EINVAL;
  for (int i = 0; i < nctx; i++)
    for (int j = i + 1; j < nctx; j++)
      if (ctxs[i] == ctxs[j]) return set_err(ctxs[i], DBSRG_EINVAL, "gen_batch: context twice");
  std::vector<int> rc((size_t)nctx, DBSRG_OK);
  // every context pipelines its lists (the set-up of one list overlaps the
  // kernels of the previous one) and is drained at the end
  auto work = [&](int i) {
    dbsrg_ctx *c = ctxs[i];
    cudaSetDevice(c->device);
    const bool was = c->async;
    c->async = true;
    for (size_t l = off[i]; l < off[i + 1] && rc[i] == DBSRG_OK; l++) {
      const dbsrg_list &L = lists[l];
      rc[i] = dbsrg_gen_matrix(c, L.icase, L.itype, L.kpol, L.ncdata, L.ipt, L.k1, L.k2, L.k3,
                               L.k4, L.cdata);
    }
    const int rd = drain(c);
    if (rc[i] == DBSRG_OK) rc[i] = rd;
    c->async = was;
  };
  // one host thread per context (each with its own stream): the host-side
  // list handling of one block overlaps the kernels of the others
  std::vector<std::thread> th;
  for (int i = 1; i < nctx; i++) th.emplace_back(work, i);
  if (nctx > 0) work(0);
  for (auto &t : th) t.join();
  for (int i = 0; i < nctx; i++)
    if (rc[i] != DBSRG_OK) return rc[i];
  return DBSRG_OK;
}

int dbsrg_gen_batch_streamed(int nctx, dbsrg_ctx *const *ctxs, const int *nlists,
                             const dbsrg_list *lists, dbsrg_window_fn fn, void *user) {
  if (nctx < 0 || (nctx > 0 && (!ctxs || !nlists)) || !fn) return DBSRG_EINVAL;
  std::vector<size_t> off((size_t)nctx + 1, 0);
  for (int i = 0; i < nctx; i++) {
    if (!ctxs[i] || nlists[i] < 0) return DBSRG_EINVAL;
    if (!ctxs[i]->hmem) return set_err(ctxs[i], DBSRG_ESTATE, "no matrix allocated");
    off[i + 1] = off[i] + (size_t)nlists[i];
  }
  if (off[nctx] > 0 && !lists) return DBSRG_EINVAL;
  for (int i = 0; i < nctx; i++)
    for (int j = i + 1; j < nctx; j++)
      if (ctxs[i] == ctxs[j]) return set_err(ctxs[i], DBSRG_EINVAL, "gen_batch: context twice");
  std::vector<int> rc((size_t)nctx, DBSRG_OK);
  // per context: every list set up once, the windows in block order, each
  // window zeroed, assembled, drained and handed to the consumer
  auto work = [&](int i) {
    dbsrg_ctx *c = ctxs[i];
    cudaSetDevice(c->device);
    if ((rc[i] = drain(c))) return;
    const size_t blk = (size_t)c->g.ms * c->g.ms;
    const int nwin = c->wcap;
    if (cudaMemsetAsync(c->acf, 0, sizeof(double) * (size_t)c->iicc * (c->mk + 1), c->stream) !=
        cudaSuccess) {
      rc[i] = cuda_check(c, cudaGetLastError(), "acf");
      return;
    }
    if ((rc[i] = zero_structures(c))) return;
    auto before = [&](int, double *slot) -> int {
      DBSRG_TRY(c, cudaMemsetAsync(slot, 0, sizeof(double) * blk * nwin, c->stream));
      return DBSRG_OK;
    };
    auto after = [&](int, int blo, int nb, double *slot) -> int {
      int r = drain(c);
      if (r) return r;
      fn(user, i, blo, nb, slot);
      return DBSRG_OK;
    };
    rc[i] = assemble_windows(c, nlists[i], lists + off[i], nwin, 1, before, after);
    c->wlo = 1 + ((c->iicc - 1) / nwin) * nwin;  // the last window stays held
  };
  std::vector<std::thread> th;
  for (int i = 1; i < nctx; i++) th.emplace_back(work, i);
  if (nctx > 0) work(0);
  for (auto &t : th) t.join();
  for (int i = 0; i < nctx; i++)
    if (rc[i] != DBSRG_OK) return rc[i];
  return DBSRG_OK;
}

// The window partition of the assemblies that copy windows out while the
// next one is assembled: windows of nwin blocks, the first and the last
// max(1, nwin/8) blocks when two device slots alternate over more than two
// windows' worth of blocks -- the first window's assembly and the last
// window's copy are the parts that nothing overlaps.  Empty: plain windows
// of nwin blocks.
static std::vector<int> host_windows(int iicc, int nwin, int nslot) {
  std::vector<int> ws;
  const int edge = std::max(1, nwin / 8);
  if (nslot == 2 && iicc > 2 * nwin) {
    ws.push_back(1);
    ws.push_back(1 + edge);
    while (iicc + 1 - ws.back() > nwin + edge) ws.push_back(ws.back() + nwin);
    ws.push_back(iicc + 1 - edge);
    ws.push_back(iicc + 1);
  }
  return ws;
}

int dbsrg_assemble_to_host(dbsrg_ctx *c, int nlists, const dbsrg_list *lists, int nwin,
                           double *hch_host, double *acf_host) {
  if (!c) return DBSRG_EINVAL;
  if (nlists < 0 || (nlists > 0 && !lists) || !hch_host)
    return set_err(c, DBSRG_EINVAL, "assemble_to_host: bad arguments");
  if (!c->hmem) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  cudaSetDevice(c->device);
  SETTLE(c);
  const int iicc = c->iicc;
  if (nwin <= 0) nwin = std::max(1, (iicc + c->tune_windows - 1) / c->tune_windows);
  nwin = std::min(nwin, iicc);
  const int nslot = nwin < iicc ? 2 : 1;
  if (nslot * nwin > c->hcap)
    return set_err(c, DBSRG_EINVAL, "assemble_to_host: two windows must fit the allocation");
  const size_t blk = (size_t)c->g.ms * c->g.ms;
  const cudaMemcpyKind kind =
      is_device_ptr(hch_host) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  DBSRG_TRY(c, cudaMemsetAsync(c->acf, 0, sizeof(double) * (size_t)iicc * (c->mk + 1), c->stream));
  int rz = zero_structures(c);  // the perturber and target parts start from zero too
  if (rz) return rz;
  // window w (slot w % 2) is assembled on the contraction stream while the
  // copy stream moves window w-1 out; a slot is zeroed again only after its
  // copy
  auto before = [&](int w, double *slot) -> int {
    DBSRG_TRY(c, cudaStreamWaitEvent(c->stream, c->cdone[w % nslot], 0));
    DBSRG_TRY(c, cudaMemsetAsync(slot, 0, sizeof(double) * blk * nwin, c->stream));
    return DBSRG_OK;
  };
  auto after = [&](int w, int blo, int nb, double *slot) -> int {
    DBSRG_TRY(c, cudaEventRecord(c->wdone, c->stream));
    DBSRG_TRY(c, cudaStreamWaitEvent(c->cstream, c->wdone, 0));
    DBSRG_TRY(c, cudaMemcpyAsync(hch_host + (size_t)(blo - 1) * blk, slot,
                                 sizeof(double) * blk * nb, kind, c->cstream));
    DBSRG_TRY(c, cudaEventRecord(c->cdone[w % nslot], c->cstream));
    return DBSRG_OK;
  };
  const std::vector<int> ws = host_windows(iicc, nwin, nslot);
  const int rc =
      assemble_windows(c, nlists, lists, nwin, nslot, before, after, ws.empty() ? nullptr : &ws);
  const cudaError_t ce = cudaStreamSynchronize(c->cstream);
  if (rc) return rc;
  if (ce != cudaSuccess) return cuda_check(c, ce, "assemble_to_host copy");
  if (acf_host) return copy_out(c, acf_host, c->acf, sizeof(double) * (size_t)iicc * (c->mk + 1));
  return DBSRG_OK;
}

int dbsrg_assemble_streamed_host(dbsrg_ctx *c, int nlists, const dbsrg_list *lists, int nwin,
                                 double *stage, dbsrg_window_fn fn, void *user,
                                 double *acf_host) {
  if (!c) return DBSRG_EINVAL;
  if (nlists < 0 || (nlists > 0 && !lists) || !stage || !fn)
    return set_err(c, DBSRG_EINVAL, "assemble_streamed_host: bad arguments");
  if (!c->hmem) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  cudaSetDevice(c->device);
  SETTLE(c);
  const int iicc = c->iicc;
  if (nwin <= 0) nwin = std::max(1, (iicc + c->tune_windows - 1) / c->tune_windows);
  nwin = std::min(nwin, iicc);
  const int nslot = nwin < iicc ? 2 : 1;
  if (nslot * nwin > c->hcap)
    return set_err(c, DBSRG_EINVAL, "assemble_streamed_host: two windows must fit the allocation");
  const size_t blk = (size_t)c->g.ms * c->g.ms;
  const cudaMemcpyKind kind =
      is_device_ptr(stage) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  DBSRG_TRY(c, cudaMemsetAsync(c->acf, 0, sizeof(double) * (size_t)iicc * (c->mk + 1), c->stream));
  int rz = zero_structures(c);
  if (rz) return rz;
  // window w: assembled in device slot w % 2 on the contraction stream,
  // copied into stage half w % 2 on the copy stream; handed to fn once its
  // copy is complete, which the host waits for right after it has queued
  // window w + 1 (so the device assembles w + 1 meanwhile).  Half w % 2 is
  // written again by window w + 2, queued only after that hand-over.
  int pend = -1, pend_blo = 0, pend_nb = 0;  // copied or in flight, not handed over
  auto hand = [&]() -> int {
    if (pend < 0) return DBSRG_OK;
    DBSRG_TRY(c, cudaEventSynchronize(c->cdone[pend % nslot]));
    fn(user, 0, pend_blo, pend_nb, stage + (size_t)(pend % nslot) * nwin * blk);
    pend = -1;
    return DBSRG_OK;
  };
  auto before = [&](int w, double *slot) -> int {
    DBSRG_TRY(c, cudaStreamWaitEvent(c->stream, c->cdone[w % nslot], 0));
    DBSRG_TRY(c, cudaMemsetAsync(slot, 0, sizeof(double) * blk * nwin, c->stream));
    return DBSRG_OK;
  };
  auto after = [&](int w, int blo, int nb, double *slot) -> int {
    DBSRG_TRY(c, cudaEventRecord(c->wdone, c->stream));
    DBSRG_TRY(c, cudaStreamWaitEvent(c->cstream, c->wdone, 0));
    DBSRG_TRY(c, cudaMemcpyAsync(stage + (size_t)(w % nslot) * nwin * blk, slot,
                                 sizeof(double) * blk * nb, kind, c->cstream));
    DBSRG_TRY(c, cudaEventRecord(c->cdone[w % nslot], c->cstream));
    const int r = hand();  // window w - 1
    if (r) return r;
    pend = w;
    pend_blo = blo;
    pend_nb = nb;
    return DBSRG_OK;
  };
  const std::vector<int> ws = host_windows(iicc, nwin, nslot);
  const int rc =
      assemble_windows(c, nlists, lists, nwin, nslot, before, after, ws.empty() ? nullptr : &ws);
  const cudaError_t ce = cudaStreamSynchronize(c->cstream);
  if (rc) return rc;
  if (ce != cudaSuccess) return cuda_check(c, ce, "assemble_streamed_host copy");
  const int rh = hand();  // the last window
  if (rh) return rh;
  if (acf_host) return copy_out(c, acf_host, c->acf, sizeof(double) * (size_t)iicc * (c->mk + 1));
  return DBSRG_OK;
}

int dbsrg_host_alloc(size_t bytes, void **out) {
  if (!out || bytes == 0) return DBSRG_EINVAL;
  *out = nullptr;
  // the transparent huge page size of the kernel (2 MB with 4 KB pages,
  // 512 MB with 64 KB pages); the mapping is over-allocated by one huge
  // page and trimmed so that it starts on a huge-page boundary
  size_t hp = 2u << 20;
  if (FILE *f = fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
    unsigned long long v = 0;
    if (fscanf(f, "%llu", &v) == 1 && v >= 4096 && (v & (v - 1)) == 0) hp = (size_t)v;
    fclose(f);
  }
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  const size_t len = (bytes + page - 1) / page * page;
  char *raw = (char *)mmap(nullptr, len + hp, PROT_READ | PROT_WRITE,
                           MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw == MAP_FAILED) return DBSRG_ENOMEM;
  char *p = (char *)(((uintptr_t)raw + hp - 1) / hp * hp);
  if (p > raw) munmap(raw, (size_t)(p - raw));
  const size_t tail = (size_t)(raw + len + hp - (p + len));
  if (tail) munmap(p + len, tail);
#ifdef MADV_HUGEPAGE
  madvise(p, len, MADV_HUGEPAGE);  // advisory: small pages if refused
#endif
  // touch (zero) the pages from several threads, in huge-page pieces
  const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t npiece = (len + hp - 1) / hp;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nth; t++)
    th.emplace_back([=]() {
      for (size_t q = t; q < npiece; q += nth) {
        const size_t a = q * hp, b = std::min(len, a + hp);
        std::memset(p + a, 0, b - a);
      }
    });
  for (auto &x : th) x.join();
  if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    munmap(p, len);
    return DBSRG_ENOMEM;
  }
  {
    std::lock_guard<std::mutex> lk(host_mu());
    host_sizes()[p] = len;
  }
  *out = p;
  return DBSRG_OK;
}

int dbsrg_host_free(void *p) {
  if (!p) return DBSRG_OK;
  size_t len = 0;
  {
    std::lock_guard<std::mutex> lk(host_mu());
    auto it = host_sizes().find(p);
    if (it == host_sizes().end()) return DBSRG_EINVAL;
    len = it->second;
    host_sizes().erase(it);
  }
  cudaHostUnregister(p);
  munmap(p, len);
  return DBSRG_OK;
}

int dbsrg_graph_capture(dbsrg_ctx *c, int nlists, const dbsrg_list *lists) {
  if (!c) return DBSRG_EINVAL;
  if (nlists < 0 || (nlists > 0 && !lists))
    return set_err(c, DBSRG_EINVAL, "graph_capture: bad arguments");
  cudaSetDevice(c->device);
  SETTLE(c);
  const bool async = c->async;
  int rc = graph_capture(c, nlists, lists);
  if (rc) return rc;
  // the first replay: the cached tables the capture set up hold values only
  // once the graph has run
  c->async = false;
  rc = graph_launch(c, nullptr);
  c->async = async;
  return rc;
}

int dbsrg_graph_launch(dbsrg_ctx *c, const double *pq) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  return graph_launch(c, pq);
}

int dbsrg_graph_release(dbsrg_ctx *c) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  graph_drop(c);
  return DBSRG_OK;
}

int dbsrg_update_hx(dbsrg_ctx *c, int ich, int jch, const double *d, double cc) {
  if (!c || !d) return set_err(c, DBSRG_EINVAL, "bad UPDATE_HX arguments");
  cudaSetDevice(c->device);
  SETTLE(c);
  return update_hx(c, ich, jch, d, cc);
}

int dbsrg_get_block(dbsrg_ctx *c, int ich, int jch, double *out) {
  if (!c || !out) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (ich < 1 || jch < 1 || ich > c->nch || jch > c->nch)
    return set_err(c, DBSRG_ERANGE, "channel out of range");
  int b = c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)];
  if (b < 1) return set_err(c, DBSRG_ERANGE, "channel pair has no block");
  if (!in_window(c, b)) return set_err(c, DBSRG_ESTATE, "block outside the current window");
  const size_t ms = c->g.ms;
  return copy_out(c, out, c->hch + (size_t)(b - c->wlo) * ms * ms, sizeof(double) * ms * ms);
}

int dbsrg_get_matrix(dbsrg_ctx *c, double *out) {
  if (!c || !out) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  const size_t ms = c->g.ms;
  return copy_out(c, out, c->hch, sizeof(double) * ms * ms * window_blocks(c));
}

int dbsrg_get_acf(dbsrg_ctx *c, double *out) {
  if (!c || !out) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  if (!c->acf) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  return copy_out(c, out, c->acf, sizeof(double) * (size_t)c->iicc * (c->mk + 1));
}

int dbsrg_window_blocks(const dbsrg_ctx *c) { return c && c->hch ? window_blocks(c) : 0; }

int dbsrg_matrix_device_ptr(dbsrg_ctx *c, double **p) {
  if (!c || !p) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  *p = c->hch;
  return DBSRG_OK;
}

int dbsrg_get_table(dbsrg_ctx *c, int family, int type, int k, double *out) {
  if (!c || !out || k < 0 || k > 64) return set_err(c, DBSRG_EINVAL, "bad table request");
  cudaSetDevice(c->device);
  SETTLE(c);
  const double *tab = nullptr;
  int rc;
  size_t n;
  const size_t ns = c->g.ns, ks = c->g.ks;
  if (family == DBSRG_RK) {
    if (type < 0 || type > 3) return set_err(c, DBSRG_EINVAL, "R table type 0..3");
    rc = get_rtable(c, type, k, &tab);
    n = ns * ns * ks * ks;
  } else if (family == DBSRG_SK) {
    if (type < 0 || type > 1) return set_err(c, DBSRG_EINVAL, "S table type 0..1");
    rc = get_stable(c, type, k, &tab);
    n = ns * ns * (2 * ks - 1) * (2 * ks - 1);
  } else {
    return set_err(c, DBSRG_EINVAL, "unknown table family");
  }
  if (rc) return rc;
  return copy_out(c, out, tab, n * sizeof(double));
}

int dbsrg_get_moments(dbsrg_ctx *c, int which, int k, double *out) {
  if (!c || !out || which < 0 || which > 3) return set_err(c, DBSRG_EINVAL, "bad moments request");
  cudaSetDevice(c->device);
  SETTLE(c);
  const DeviceGrid &g = c->g;
  size_t n = (size_t)g.ks * g.ks * g.nv;
  int rc = ensure_scratch(c, n * sizeof(double));
  if (rc) return rc;
  if ((rc = compute_moments(c, which, k, (double *)c->scratch))) return rc;
  return copy_out(c, out, c->scratch, n * sizeof(double));
}

int dbsrg_get_diag_cells(dbsrg_ctx *c, int type, int k, double *out) {
  if (!c || !out || type < 0 || type > 5) return set_err(c, DBSRG_EINVAL, "bad diag-cell request");
  cudaSetDevice(c->device);
  SETTLE(c);
  const DeviceGrid &g = c->g;
  size_t kk = (size_t)g.ks * g.ks;
  size_t n = kk * kk * g.nv;
  int rc = ensure_scratch(c, n * sizeof(double));
  if (rc) return rc;
  if ((rc = compute_diag_cells(c, type, k, (double *)c->scratch))) return rc;
  return copy_out(c, out, c->scratch, n * sizeof(double));
}

int dbsrg_get_grid_array(dbsrg_ctx *c, const char *name, double *out) {
  if (!c || !name || !out) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  SETTLE(c);
  const DeviceGrid &g = c->g;
  const size_t nv = g.nv, ks = g.ks, ns = g.ns, ms = g.ms;
  const double *src = nullptr;
  size_t n = 0;
  if (!strcmp(name, "gr")) { src = g.gr; n = nv * ks; }
  else if (!strcmp(name, "grw")) { src = g.grw; n = nv * ks; }
  else if (!strcmp(name, "grm")) { src = g.grm; n = nv * ks; }
  else if (!strcmp(name, "pbsp")) { src = g.pbsp; n = (nv + 1) * ks * g.ksp; }
  else if (!strcmp(name, "qbsp")) { src = g.qbsp; n = (nv + 1) * ks * g.ksq; }
  else if (!strcmp(name, "fpbs")) { src = g.fpbs; n = ns * ns; }
  else if (!strcmp(name, "fqbs")) { src = g.fqbs; n = ns * ns; }
  else if (!strcmp(name, "fppqq")) { src = g.fppqq; n = ms * ms; }
  else if (!strcmp(name, "gx")) { src = g.gx; n = ks; }
  else if (!strcmp(name, "gw")) { src = g.gw; n = ks; }
  else return set_err(c, DBSRG_EINVAL, "unknown grid array");
  return copy_out(c, out, src, n * sizeof(double));
}

}  // extern "C"
