/*
 * C-ABI entry layer of the gravity library.
 *
 * Implements the drop-in boundary declared in include/HostCUDA.h and
 * include/EwaldCUDA.h (reference: HostCUDA.cu:66-630, 1887-1956) and the
 * extension forms in include/changa_gb300.h.
 *
 * Per request the reference does cudaMalloc + four H2D copies + kernel +
 * cudaFree (HostCUDA.cu:578-613), and cudaFree synchronises the device.
 * Here one stream-ordered allocation holds the request's list, markers,
 * starts, sizes and the kernel's work-queue counter; it is released with
 * cudaFreeAsync on the same stream, so an entry point never blocks the host
 * or other streams.  Source-array bounds for the kernels' index guards come
 * from cuMemGetAddressRange on the device pointer the request names.
 */
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include <cuda.h>

#include "chg_internal.h"

namespace chg {

static std::atomic<int> g_error_mode{CHANGA_ERRORS_ABORT};
static std::atomic<int> g_last_error{0};
static std::atomic<int> g_validate{0};
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<changa_completion_hook> g_hook{nullptr};

int record_error(int code, const char* what, const char* file, int line) {
  if (code == 0) return 0;
  int expected = 0;
  g_last_error.compare_exchange_strong(expected, code);
  if (g_error_mode.load() == CHANGA_ERRORS_ABORT) {
    fprintf(stderr, "changa_gb300: fatal error %d (%s) at %s:%d from '%s'\n", code,
            changa_gb300_error_string(code), file, line, what);
    abort();
  }
  return code;
}

void count_launch(unsigned n) { g_launches.fetch_add(n); }

/* ---- optional per-kernel event timing ---- */

static std::atomic<int> g_timing{0};
static std::mutex g_timing_mu;
struct EventPair {
  cudaEvent_t start, stop;
};
static std::vector<EventPair> g_timing_events[kKidCount];

TimingScope::TimingScope(int k, cudaStream_t st) : kid(k), s(st), start(nullptr) {
  if (!g_timing.load() || k < 0 || k >= kKidCount) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  start = e;
}

TimingScope::~TimingScope() {
  if (!start) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaEventDestroy((cudaEvent_t)start);
    return;
  }
  cudaEventRecord(e, s);
  std::lock_guard<std::mutex> lk(g_timing_mu);
  g_timing_events[kid].push_back(EventPair{(cudaEvent_t)start, e});
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
      n = 1;
    cached[dev] = n;
  }
  return cached[dev];
}

/* Keeps memory freed with cudaFreeAsync cached in the default pool so
 * per-request allocations do not return to the OS at every synchronise
 * (a process-local pool attribute). */
void prepare_pool() {
  static bool done[64] = {false};
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

/* Elements of size elem from p to the end of its allocation; LLONG_MAX
 * when the range cannot be determined. */
/* cuMemGetAddressRange, resolved through the runtime so the library loads
 * (and its symbols can be inspected) on machines without a driver. */
typedef CUresult (*AddrRangeFn)(CUdeviceptr*, size_t*, CUdeviceptr);
static AddrRangeFn addr_range_fn() {
  static std::atomic<int> state{0};
  static AddrRangeFn fn = nullptr;
  if (state.load() == 0) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (AddrRangeFn)f;
    else
      cudaGetLastError();
    state.store(1);
  }
  return fn;
}

static long long elems_to_end(const void* p, size_t elem) {
  if (!p) return 0;
  CUdeviceptr base = 0;
  size_t size = 0;
  AddrRangeFn fn = addr_range_fn();
  if (!fn || fn(&base, &size, (CUdeviceptr)p) != CUDA_SUCCESS) return LLONG_MAX;
  size_t off = (size_t)((CUdeviceptr)p - base);
  if (off > size) return 0;
  return (long long)((size - off) / elem);
}

static void signal(cudaStream_t s, void* cb) {
  changa_completion_hook h = g_hook.load();
  if (h) h(s, cb);
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr size_t kDefaultHostChunkBytes = size_t(256) << 20;
static std::atomic<size_t> g_host_chunk_bytes{kDefaultHostChunkBytes};

/* The library-owned streams of the host-array entries on each device
 * (created once): which 0 carries the uploads, which 1 the read-backs, so
 * the two directions of the host link run at once; which 2 is the second
 * compute lane of changa_gravity_step_host. */
static cudaStream_t library_stream(int which = 0) {
  static cudaStream_t st[64][3] = {{nullptr}};
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (which < 0 || which > 2) which = 0;
  std::lock_guard<std::mutex> lk(mu);
  cudaStream_t& x = st[dev][which];
  if (!x && cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) x = nullptr;
  return x;
}

/* Bucket ranges [b0, b1) of a request, about `per` list entries each; with
 * shrink, the last 2 per entries go in halving chunks (down to per / 16),
 * so little arithmetic is left once the final entries have landed. */
static void list_chunks(const ChangaListRequest* r, long long per, bool shrink,
                        std::vector<std::pair<int, int>>& out) {
  const long long total = r->markers[r->n_buckets];
  const long long floor_ = std::max<long long>(1, per / 16);
  int b0 = 0;
  while (b0 < r->n_buckets) {
    const long long left = total - r->markers[b0];
    long long want_n = per;
    if (shrink && left <= 2 * per) want_n = std::max(floor_, left / 2);
    const int* lo = r->markers + b0 + 1;
    const int* hi = r->markers + r->n_buckets + 1;
    const long long want = (long long)r->markers[b0] + want_n;
    const int* it = std::upper_bound(lo, hi, (int)std::min<long long>(want, INT_MAX));
    int b1 = (int)(it - r->markers) - 1;
    if (b1 <= b0) b1 = b0 + 1;
    if (b1 > r->n_buckets) b1 = r->n_buckets;
    out.push_back({b0, b1});
    b0 = b1;
  }
}

/* Device copy of one request (list, markers, starts, sizes, queue). */
struct ReqDev {
  char* block = nullptr;
  int2* list = nullptr;
  int* markers = nullptr;
  int* starts = nullptr;
  int* sizes = nullptr;
  unsigned int* queue = nullptr;
  cudaStream_t stream = 0;
};

static int upload_request(const void* h_list, long long n_entries, const int* h_markers,
                          const int* h_starts, const int* h_sizes, int n_buckets, cudaStream_t s,
                          ReqDev& d, bool copy_list = true) {
  prepare_pool();
  size_t lb = align256((size_t)(n_entries > 0 ? n_entries : 0) * sizeof(ILCell));
  size_t mb = align256((size_t)(n_buckets + 1) * sizeof(int));
  size_t sb = align256((size_t)(n_buckets > 0 ? n_buckets : 0) * sizeof(int));
  size_t total = lb + mb + 2 * sb + 256;
  CHG_CUDA(cudaMallocAsync((void**)&d.block, total, s));
  d.stream = s;
  d.list = (int2*)d.block;
  d.markers = (int*)(d.block + lb);
  d.starts = (int*)(d.block + lb + mb);
  d.sizes = (int*)(d.block + lb + mb + sb);
  d.queue = (unsigned int*)(d.block + lb + mb + 2 * sb);
  if (copy_list && n_entries > 0)
    CHG_CUDA(cudaMemcpyAsync(d.list, h_list, (size_t)n_entries * sizeof(ILCell),
                             cudaMemcpyHostToDevice, s));
  CHG_CUDA(cudaMemcpyAsync(d.markers, h_markers, (size_t)(n_buckets + 1) * sizeof(int),
                           cudaMemcpyHostToDevice, s));
  if (n_buckets > 0) {
    CHG_CUDA(cudaMemcpyAsync(d.starts, h_starts, (size_t)n_buckets * sizeof(int),
                             cudaMemcpyHostToDevice, s));
    CHG_CUDA(cudaMemcpyAsync(d.sizes, h_sizes, (size_t)n_buckets * sizeof(int),
                             cudaMemcpyHostToDevice, s));
  }
  CHG_CUDA(cudaMemsetAsync(d.queue, 0, sizeof(unsigned int), s));
  return 0;
}

static int release_request(ReqDev& d) {
  if (d.block) CHG_CUDA(cudaFreeAsync(d.block, d.stream));
  d.block = nullptr;
  return 0;
}

/* A large drop-in request, pipelined: the markers, starts and sizes go
 * first on the request's stream; the list follows in chunks of about `per`
 * entries (the last ones halving) on the library's copy stream, and the
 * list kernel runs over each chunk's bucket range on the request's stream
 * as soon as that chunk has landed, so the upload overlaps the arithmetic.
 * Every kernel waits for its chunk's copy, so the request's stream (and the
 * completion signalled on it) finishes after every read of the caller's
 * host arrays, which the caller may free in its callback. */
static int run_request_chunked(CudaRequest* r, bool cell, const void* sources, long long n_src,
                               long long n_tgt, int nb, long long per, cudaStream_t c) {
  cudaStream_t s = r->stream;
  ReqDev d;
  /* the block is allocated and its small arrays uploaded on the copy
   * stream, so this request's upload does not wait for the work already on
   * the request's stream (a previous request's kernels); each kernel waits
   * for its chunk's copy, which follows the allocation on the copy stream */
  int rc = upload_request(r->list, r->numInteractions, r->bucketMarkers, r->bucketStarts,
                          r->bucketSizes, nb, c, d, /*copy_list=*/false);
  if (rc) return rc;
  d.stream = s;  // released on the request's stream, after its kernels
  ChangaListRequest h;  // the host arrays, for the chunk boundaries
  h.list = (const ILCell*)r->list;
  h.markers = r->bucketMarkers;
  h.starts = r->bucketStarts;
  h.sizes = r->bucketSizes;
  h.n_buckets = nb;
  h.n_entries = r->numInteractions;
  std::vector<std::pair<int, int>> chunks;
  list_chunks(&h, per, true, chunks);
  /* events are released by the runtime once complete; a wait enqueued
   * before the destroy still sees the recorded work */
  auto mark = [](cudaStream_t on, cudaEvent_t* ev) -> cudaError_t {
    cudaError_t x = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (x != cudaSuccess) return x;
    return cudaEventRecord(*ev, on);
  };
  cudaError_t e = cudaSuccess;
  const ILCell* hl = (const ILCell*)r->list;
  for (size_t i = 0; i < chunks.size() && e == cudaSuccess; ++i) {
    const int b0 = chunks[i].first, b1 = chunks[i].second;
    const long long e0 = std::max(0, h.markers[b0]);
    const long long e1 = std::min<long long>(h.markers[b1], r->numInteractions);
    cudaEvent_t landed = nullptr;
    if (e1 > e0)
      e = cudaMemcpyAsync(d.list + e0, hl + e0, (size_t)(e1 - e0) * sizeof(ILCell),
                          cudaMemcpyHostToDevice, c);
    if (e == cudaSuccess) e = mark(c, &landed);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, landed, 0);
    if (landed) cudaEventDestroy(landed);
    if (e != cudaSuccess) break;
    if (i > 0) e = cudaMemsetAsync(d.queue, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) break;
    ListArgs a;
    a.src = sources;
    a.n_src = n_src;
    a.tgt = r->d_localParts;
    a.n_tgt = n_tgt;
    a.vars = r->d_localVars;
    a.list = d.list;
    a.n_entries = e1 > e0 ? e1 : e0;  // entries past this chunk have not landed yet
    a.markers = d.markers + b0;
    a.starts = d.starts + b0;
    a.sizes = d.sizes + b0;
    a.n_buckets = b1 - b0;
    a.fperiod_f = r->fperiod;
    a.fperiod_d = r->fperiod;
    a.queue = d.queue;
    e = launch_list(kF32, cell, a, s);
  }
  rc = release_request(d);
  if (e != cudaSuccess) return record_error((int)e, "chunked request", __FILE__, __LINE__);
  if (rc) return rc;
  signal(s, r->cb);
  return 0;
}

/* Drop-in request: cell lists when cell, particle lists otherwise. */
static int run_request(CudaRequest* r, bool cell, const void* sources, long long n_src) {
  if (!r) return record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
  int nb = r->numBucketsPlusOne - 1;
  if (nb <= 0) {
    signal(r->stream, r->cb);
    return 0;
  }
  if (!r->list || !r->bucketMarkers || !r->bucketStarts || !r->bucketSizes || !r->d_localParts ||
      !r->d_localVars || !sources)
    return record_error(CHANGA_E_INVALID_ARG, "request pointers", __FILE__, __LINE__);
  /* moments are read as float4 triples: 16-byte alignment is required */
  if (cell && ((uintptr_t)sources & 15))
    return record_error(CHANGA_E_INVALID_ARG, "moments not 16-byte aligned", __FILE__, __LINE__);
  long long n_tgt = elems_to_end(r->d_localParts, sizeof(CompactPartData));
  long long n_var = elems_to_end(r->d_localVars, sizeof(VariablePartData));
  if (n_var < n_tgt) n_tgt = n_var;
  if (g_validate.load()) {
    int rc = changa_validate_request((const ILCell*)r->list, r->numInteractions, r->bucketMarkers,
                                     r->bucketStarts, r->bucketSizes, nb, n_src, n_tgt);
    if (rc) return record_error(rc, "request validation", __FILE__, __LINE__);
  }
  /* a list of more than two chunks streams in chunk by chunk */
  const long long per = (long long)(g_host_chunk_bytes.load() / sizeof(ILCell));
  if (r->numInteractions > 2 * per) {
    cudaStream_t c = library_stream();
    if (c) return run_request_chunked(r, cell, sources, n_src, n_tgt, nb, per, c);
  }
  ReqDev d;
  int rc = upload_request(r->list, r->numInteractions, r->bucketMarkers, r->bucketStarts,
                          r->bucketSizes, nb, r->stream, d);
  if (rc) return rc;
  ListArgs a;
  a.src = sources;
  a.n_src = n_src;
  a.tgt = r->d_localParts;
  a.n_tgt = n_tgt;
  a.vars = r->d_localVars;
  a.list = d.list;
  a.n_entries = r->numInteractions;
  a.markers = d.markers;
  a.starts = d.starts;
  a.sizes = d.sizes;
  a.n_buckets = nb;
  a.fperiod_f = r->fperiod;
  a.fperiod_d = r->fperiod;
  a.queue = d.queue;
  CHG_CUDA(launch_list(kF32, cell, a, r->stream));
  rc = release_request(d);
  if (rc) return rc;
  signal(r->stream, r->cb);
  return 0;
}

/* Stream recorded by TreePieceDataTransferBasic for its Cleanup. */
static std::mutex g_basic_mu;
static std::unordered_map<void*, cudaStream_t> g_basic_streams;

/* FP32 FMA throughput probe: every thread runs 8 independent dependent
 * chains of scalar fma.rn.f32 (the multiplier and addend keep the values
 * bounded); 2 FLOP per FMA.  The result is written so nothing is dropped. */
__global__ void fma_probe_kernel(float* out, int iters) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 1e-3f * (float)(threadIdx.x + k);
  const float m = 0.999f, c = 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace chg

using namespace chg;

/* ------------------------------------------------------------------ */
/* implementations shared by the C names and the C++-mangled names     */
/* ------------------------------------------------------------------ */

extern "C" {

void chg_impl_allocatePinnedHostMemory(void** ptr, size_t size) {
  if (!ptr) return;
  if (size == 0) {
    *ptr = nullptr;
    record_error(CHANGA_E_INVALID_ARG, "allocatePinnedHostMemory(size 0)", __FILE__, __LINE__);
    return;
  }
  cudaError_t e = cudaMallocHost(ptr, size);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    record_error((int)e, "cudaMallocHost", __FILE__, __LINE__);
  }
}

void chg_impl_freePinnedHostMemory(void* ptr) {
  if (!ptr) {
    record_error(CHANGA_E_INVALID_ARG, "freePinnedHostMemory(NULL)", __FILE__, __LINE__);
    return;
  }
  cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) record_error((int)e, "cudaFreeHost", __FILE__, __LINE__);
}

static int transfer_local_tree(void* moments, size_t sMoments, void* compactParts,
                               size_t sCompactParts, void* varParts, size_t sVarParts,
                               void** d_localMoments, void** d_compactParts, void** d_varParts,
                               cudaStream_t stream, int numParticles, void* callback) {
  if (!d_localMoments || !d_compactParts || !d_varParts)
    return record_error(CHANGA_E_INVALID_ARG, "DataManagerTransferLocalTree", __FILE__, __LINE__);
  if ((size_t)numParticles * sizeof(VariablePartData) > sVarParts)
    return record_error(CHANGA_E_INVALID_ARG, "numParticles > sVarParts", __FILE__, __LINE__);
  CHG_CUDA(cudaMalloc(d_localMoments, sMoments));
  CHG_CUDA(cudaMalloc(d_compactParts, sCompactParts));
  CHG_CUDA(cudaMalloc(d_varParts, sVarParts));
  if (sMoments)
    CHG_CUDA(cudaMemcpyAsync(*d_localMoments, moments, sMoments, cudaMemcpyHostToDevice, stream));
  if (sCompactParts)
    CHG_CUDA(cudaMemcpyAsync(*d_compactParts, compactParts, sCompactParts, cudaMemcpyHostToDevice,
                             stream));
  if (sVarParts)
    CHG_CUDA(cudaMemcpyAsync(*d_varParts, varParts, sVarParts, cudaMemcpyHostToDevice, stream));
  /* ZeroVars (HostCUDA.cu:2195-2205): all-zero bits are 0.0f */
  if (numParticles > 0)
    CHG_CUDA(cudaMemsetAsync(*d_varParts, 0, (size_t)numParticles * sizeof(VariablePartData),
                             stream));
  signal(stream, callback);
  return 0;
}

void chg_impl_DataManagerTransferLocalTree(void* moments, size_t sMoments, void* compactParts,
                                           size_t sCompactParts, void* varParts, size_t sVarParts,
                                           void** d_localMoments, void** d_compactParts,
                                           void** d_varParts, cudaStream_t stream,
                                           int numParticles, void* callback) {
  transfer_local_tree(moments, sMoments, compactParts, sCompactParts, varParts, sVarParts,
                      d_localMoments, d_compactParts, d_varParts, stream, numParticles, callback);
}

static int transfer_remote_chunk(void* moments, size_t sMoments, void* compactParts,
                                 size_t sCompactParts, void** d_remoteMoments,
                                 void** d_remoteParts, cudaStream_t stream, void* callback) {
  if (!d_remoteMoments || !d_remoteParts)
    return record_error(CHANGA_E_INVALID_ARG, "DataManagerTransferRemoteChunk", __FILE__, __LINE__);
  CHG_CUDA(cudaMalloc(d_remoteMoments, sMoments));
  CHG_CUDA(cudaMalloc(d_remoteParts, sCompactParts));
  if (sMoments)
    CHG_CUDA(cudaMemcpyAsync(*d_remoteMoments, moments, sMoments, cudaMemcpyHostToDevice, stream));
  if (sCompactParts)
    CHG_CUDA(cudaMemcpyAsync(*d_remoteParts, compactParts, sCompactParts, cudaMemcpyHostToDevice,
                             stream));
  signal(stream, callback);
  return 0;
}

void chg_impl_DataManagerTransferRemoteChunk(void* moments, size_t sMoments, void* compactParts,
                                             size_t sCompactParts, void** d_remoteMoments,
                                             void** d_remoteParts, cudaStream_t stream,
                                             void* callback) {
  transfer_remote_chunk(moments, sMoments, compactParts, sCompactParts, d_remoteMoments,
                        d_remoteParts, stream, callback);
}

void chg_impl_TransferParticleVarsBack(VariablePartData* hostBuffer, size_t size,
                                       void* d_varParts, cudaStream_t stream, void* cb) {
  if (size) {
    cudaError_t e = cudaMemcpyAsync(hostBuffer, d_varParts, size, cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) {
      record_error((int)e, "TransferParticleVarsBack", __FILE__, __LINE__);
      return;
    }
  }
  signal(stream, cb);
}

void chg_impl_TreePieceCellListDataTransferLocal(CudaRequest* d) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  run_request(d, true, d->d_localMoments,
              elems_to_end(d->d_localMoments, sizeof(CudaMultipoleMoments)));
}

void chg_impl_TreePieceCellListDataTransferRemote(CudaRequest* d) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  run_request(d, true, d->d_remoteMoments,
              elems_to_end(d->d_remoteMoments, sizeof(CudaMultipoleMoments)));
}

/* Missed nodes/particles travel with the request (HostCUDA.cu:296-341). */
static void run_resume(CudaRequest* d, bool cell) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  const void* host = cell ? d->missedNodes : d->missedParts;
  if (d->numBucketsPlusOne <= 1) {
    signal(d->stream, d->cb);
    return;
  }
  if (!host || d->sMissed == 0) {
    record_error(CHANGA_E_INVALID_ARG, "resume request without missed data", __FILE__, __LINE__);
    return;
  }
  prepare_pool();
  void* dev = nullptr;
  cudaError_t e = cudaMallocAsync(&dev, d->sMissed, d->stream);
  if (e != cudaSuccess) {
    record_error((int)e, "cudaMallocAsync(missed)", __FILE__, __LINE__);
    return;
  }
  e = cudaMemcpyAsync(dev, host, d->sMissed, cudaMemcpyHostToDevice, d->stream);
  if (e != cudaSuccess) {
    record_error((int)e, "cudaMemcpyAsync(missed)", __FILE__, __LINE__);
    return;
  }
  long long n = (long long)(d->sMissed / (cell ? sizeof(CudaMultipoleMoments) : sizeof(CompactPartData)));
  int rc = run_request(d, cell, dev, n);
  e = cudaFreeAsync(dev, d->stream);
  if (!rc && e != cudaSuccess) record_error((int)e, "cudaFreeAsync(missed)", __FILE__, __LINE__);
}

void chg_impl_TreePieceCellListDataTransferRemoteResume(CudaRequest* d) { run_resume(d, true); }

void chg_impl_TreePiecePartListDataTransferLocal(CudaRequest* d) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  run_request(d, false, d->d_localParts, elems_to_end(d->d_localParts, sizeof(CompactPartData)));
}

void chg_impl_TreePiecePartListDataTransferLocalSmallPhase(CudaRequest* d, CompactPartData* parts,
                                                           int len) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  if (d->numBucketsPlusOne <= 1) {
    signal(d->stream, d->cb);
    return;
  }
  if (!parts || len <= 0) {
    record_error(CHANGA_E_INVALID_ARG, "small-phase particles", __FILE__, __LINE__);
    return;
  }
  prepare_pool();
  size_t bytes = (size_t)len * sizeof(CompactPartData);
  void* dev = nullptr;
  cudaError_t e = cudaMallocAsync(&dev, bytes, d->stream);
  if (e != cudaSuccess) {
    record_error((int)e, "cudaMallocAsync(small phase)", __FILE__, __LINE__);
    return;
  }
  e = cudaMemcpyAsync(dev, parts, bytes, cudaMemcpyHostToDevice, d->stream);
  if (e != cudaSuccess) {
    record_error((int)e, "cudaMemcpyAsync(small phase)", __FILE__, __LINE__);
    return;
  }
  int rc = run_request(d, false, dev, len);
  e = cudaFreeAsync(dev, d->stream);
  if (!rc && e != cudaSuccess) record_error((int)e, "cudaFreeAsync(small phase)", __FILE__, __LINE__);
}

void chg_impl_TreePiecePartListDataTransferRemote(CudaRequest* d) {
  if (!d) {
    record_error(CHANGA_E_INVALID_ARG, "NULL request", __FILE__, __LINE__);
    return;
  }
  run_request(d, false, d->d_remoteParts, elems_to_end(d->d_remoteParts, sizeof(CompactPartData)));
}

void chg_impl_TreePiecePartListDataTransferRemoteResume(CudaRequest* d) { run_resume(d, false); }

void chg_impl_TreePieceDataTransferBasic(CudaRequest* data, CudaDevPtr* ptr) {
  if (!data || !ptr) {
    record_error(CHANGA_E_INVALID_ARG, "TreePieceDataTransferBasic", __FILE__, __LINE__);
    return;
  }
  int nb = data->numBucketsPlusOne - 1;
  ReqDev d;
  if (upload_request(data->list, data->numInteractions, data->bucketMarkers, data->bucketStarts,
                     data->bucketSizes, nb < 0 ? 0 : nb, data->stream, d))
    return;
  ptr->d_list = d.list;
  ptr->d_bucketMarkers = d.markers;
  ptr->d_bucketStarts = d.starts;
  ptr->d_bucketSizes = d.sizes;
  std::lock_guard<std::mutex> lk(g_basic_mu);
  g_basic_streams[d.block] = data->stream;
}

void chg_impl_TreePieceDataTransferBasicCleanup(CudaDevPtr* ptr) {
  if (!ptr || !ptr->d_list) return;
  cudaStream_t s = 0;
  {
    std::lock_guard<std::mutex> lk(g_basic_mu);
    auto it = g_basic_streams.find(ptr->d_list);
    if (it == g_basic_streams.end()) {
      record_error(CHANGA_E_INVALID_ARG, "Cleanup of unknown block", __FILE__, __LINE__);
      return;
    }
    s = it->second;
    g_basic_streams.erase(it);
  }
  cudaError_t e = cudaFreeAsync(ptr->d_list, s);
  if (e != cudaSuccess) record_error((int)e, "cudaFreeAsync(basic)", __FILE__, __LINE__);
  ptr->d_list = nullptr;
  ptr->d_bucketMarkers = ptr->d_bucketStarts = ptr->d_bucketSizes = nullptr;
}

void chg_impl_EwaldHostMemorySetup(EwaldData* h, int size, int nEwhLoop, int largephase) {
  if (!h) return;
  if (largephase) chg_impl_allocatePinnedHostMemory((void**)&h->EwaldMarkers, (size_t)size * sizeof(int));
  else h->EwaldMarkers = nullptr;
  chg_impl_allocatePinnedHostMemory((void**)&h->ewt, (size_t)nEwhLoop * sizeof(EwtData));
  chg_impl_allocatePinnedHostMemory((void**)&h->cachedData, sizeof(EwaldReadOnlyData));
}

void chg_impl_EwaldHostMemoryFree(EwaldData* h, int largephase) {
  if (!h) return;
  if (largephase) chg_impl_freePinnedHostMemory(h->EwaldMarkers);
  chg_impl_freePinnedHostMemory(h->ewt);
  chg_impl_freePinnedHostMemory(h->cachedData);
}

void chg_impl_EwaldHost(CompactPartData* d_localParts, VariablePartData* d_localVars,
                        EwaldData* h, cudaStream_t stream, void* cb, int myIndex, int largephase) {
  (void)myIndex;
  if (!h || !h->cachedData || (h->cachedData->nEwhLoop > 0 && !h->ewt)) {
    record_error(CHANGA_E_INVALID_ARG, "EwaldHost", __FILE__, __LINE__);
    return;
  }
  const EwaldReadOnlyData& ro = *h->cachedData;
  if (ro.nEwhLoop > NEWH) {
    record_error(CHANGA_E_TOO_LARGE, "EwaldHost: nEwhLoop > NEWH", __FILE__, __LINE__);
    return;
  }
  int n = ro.n;
  int* d_markers = nullptr;
  if (largephase && n > 0) {
    prepare_pool();
    cudaError_t e = cudaMallocAsync((void**)&d_markers, (size_t)n * sizeof(int), stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_markers, h->EwaldMarkers, (size_t)n * sizeof(int),
                          cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) {
      record_error((int)e, "EwaldHost markers", __FILE__, __LINE__);
      return;
    }
  }
  int first = largephase ? 0 : h->EwaldRange[0];
  int last = largephase ? n - 1 : h->EwaldRange[1];
  cudaError_t e = launch_ewald_f32(d_localParts, d_localVars, d_markers, largephase, first, last,
                                   ro, h->ewt, stream);
  if (e != cudaSuccess) {
    record_error((int)e, "EwaldKernel launch", __FILE__, __LINE__);
    return;
  }
  if (d_markers) {
    e = cudaFreeAsync(d_markers, stream);
    if (e != cudaSuccess) {
      record_error((int)e, "cudaFreeAsync(markers)", __FILE__, __LINE__);
      return;
    }
  }
  signal(stream, cb);
}

/* ---- public C names (include/HostCUDA.h, include/EwaldCUDA.h) ---- */

void allocatePinnedHostMemory(void** p, size_t s) { chg_impl_allocatePinnedHostMemory(p, s); }
void freePinnedHostMemory(void* p) { chg_impl_freePinnedHostMemory(p); }
void DataManagerTransferLocalTree(void* a, size_t b, void* c, size_t d, void* e, size_t f, void** g,
                                  void** h, void** i, cudaStream_t s, int n, void* cb) {
  chg_impl_DataManagerTransferLocalTree(a, b, c, d, e, f, g, h, i, s, n, cb);
}
void DataManagerTransferRemoteChunk(void* a, size_t b, void* c, size_t d, void** e, void** f,
                                    cudaStream_t s, void* cb) {
  chg_impl_DataManagerTransferRemoteChunk(a, b, c, d, e, f, s, cb);
}
void TransferParticleVarsBack(VariablePartData* h, size_t n, void* d, cudaStream_t s, void* cb) {
  chg_impl_TransferParticleVarsBack(h, n, d, s, cb);
}
void TreePieceCellListDataTransferLocal(CudaRequest* d) { chg_impl_TreePieceCellListDataTransferLocal(d); }
void TreePieceCellListDataTransferRemote(CudaRequest* d) { chg_impl_TreePieceCellListDataTransferRemote(d); }
void TreePieceCellListDataTransferRemoteResume(CudaRequest* d) {
  chg_impl_TreePieceCellListDataTransferRemoteResume(d);
}
void TreePiecePartListDataTransferLocal(CudaRequest* d) { chg_impl_TreePiecePartListDataTransferLocal(d); }
void TreePiecePartListDataTransferLocalSmallPhase(CudaRequest* d, CompactPartData* p, int n) {
  chg_impl_TreePiecePartListDataTransferLocalSmallPhase(d, p, n);
}
void TreePiecePartListDataTransferRemote(CudaRequest* d) { chg_impl_TreePiecePartListDataTransferRemote(d); }
void TreePiecePartListDataTransferRemoteResume(CudaRequest* d) {
  chg_impl_TreePiecePartListDataTransferRemoteResume(d);
}
void TreePieceDataTransferBasic(CudaRequest* d, CudaDevPtr* p) { chg_impl_TreePieceDataTransferBasic(d, p); }
void TreePieceDataTransferBasicCleanup(CudaDevPtr* p) { chg_impl_TreePieceDataTransferBasicCleanup(p); }
void EwaldHostMemorySetup(EwaldData* h, int s, int n, int l) { chg_impl_EwaldHostMemorySetup(h, s, n, l); }
void EwaldHostMemoryFree(EwaldData* h, int l) { chg_impl_EwaldHostMemoryFree(h, l); }
void EwaldHost(CompactPartData* p, VariablePartData* v, EwaldData* h, cudaStream_t s, void* cb, int i,
               int l) {
  chg_impl_EwaldHost(p, v, h, s, cb, i, l);
}

/* ---- extension API (include/changa_gb300.h) ---- */

void changa_gb300_set_error_mode(int mode) { g_error_mode.store(mode); }
int changa_gb300_last_error(void) { return g_last_error.exchange(0); }
const char* changa_gb300_error_string(int code) {
  switch (code) {
    case 0: return "no error";
    case CHANGA_E_INVALID_ARG: return "invalid argument";
    case CHANGA_E_INVALID_LIST: return "interaction list index or marker out of range";
    case CHANGA_E_TOO_LARGE: return "size beyond a fixed limit";
    case CHANGA_E_DEVICE_WAIT: return "a kernel's bounded wait ran out (results incomplete)";
  }
  return cudaGetErrorString((cudaError_t)code);
}
void changa_gb300_set_completion_hook(changa_completion_hook hook) { g_hook.store(hook); }
void changa_gb300_set_validate(int on) { g_validate.store(on); }
int changa_gb300_version(void) { return 100; }

/* Measures the device's FP32 FMA peak: a grid of 8 blocks of 256 threads
 * per SM running fma_probe_kernel, timed with events (best of 5 after a
 * warm-up), in TFLOP/s. */
int changa_gb300_fp32_fma_peak(double* tflops) {
  if (!tflops) return record_error(CHANGA_E_INVALID_ARG, "fp32_fma_peak", __FILE__, __LINE__);
  const int threads = 256, blocks = sm_count() * 8, iters = 1 << 14;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CHG_CUDA(cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)));
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, 0);
    fma_probe_kernel<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return record_error((int)e, "fp32_fma_peak", __FILE__, __LINE__);
  const double flop = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
  *tflops = flop / (best * 1e-3) / 1e12;
  return 0;
}
unsigned long long changa_gb300_kernel_launches(void) { return g_launches.load(); }

void changa_gb300_set_timing(int on) { g_timing.store(on); }

int changa_gb300_list_variant_count(void) { return list_variant_count(); }
int changa_gb300_set_list_variant(int kernel, int variant) {
  return set_list_variant(kernel, variant) ? CHANGA_E_INVALID_ARG : 0;
}
int changa_gb300_get_list_variant(int kernel) { return get_list_variant(kernel); }
int changa_gb300_set_hex_variant(int variant) {
  return set_hex_variant(variant) ? CHANGA_E_INVALID_ARG : 0;
}
int changa_gb300_get_hex_variant(void) { return get_hex_variant(); }
int changa_gb300_device_status(void) {
  unsigned bits = 0;
  cudaError_t e = read_device_status(&bits);
  if (e != cudaSuccess) return record_error((int)e, "device_status", __FILE__, __LINE__);
  if (bits) return record_error(CHANGA_E_DEVICE_WAIT, "device status", __FILE__, __LINE__);
  return 0;
}
void changa_gb300_set_test_wait_limit(int polls) { set_tma_wait_polls(polls); }

int changa_gb300_kernel_time(int kernel, double* total_ms, long long* launches) {
  if (kernel < 0 || kernel >= kKidCount || !total_ms || !launches) return CHANGA_E_INVALID_ARG;
  std::vector<EventPair> ev;
  {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    ev.swap(g_timing_events[kernel]);
  }
  double sum = 0.0;
  for (const EventPair& p : ev) {
    float ms = 0.f;
    cudaEventSynchronize(p.stop);
    if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) sum += ms;
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  *total_ms = sum;
  *launches = (long long)ev.size();
  return 0;
}

int changa_validate_request(const ILCell* list, long long n_entries, const int* markers,
                            const int* starts, const int* sizes, int n_buckets,
                            long long n_sources, long long n_targets) {
  if (n_buckets < 0 || n_entries < 0) return CHANGA_E_INVALID_ARG;
  if (n_buckets == 0) return 0;
  if (!markers || !starts || !sizes || (n_entries > 0 && !list)) return CHANGA_E_INVALID_ARG;
  if (markers[0] < 0 || (long long)markers[n_buckets] > n_entries) return CHANGA_E_INVALID_LIST;
  for (int b = 0; b < n_buckets; ++b) {
    if (markers[b + 1] < markers[b]) return CHANGA_E_INVALID_LIST;
    if (sizes[b] < 0 || starts[b] < 0) return CHANGA_E_INVALID_LIST;
    if ((long long)starts[b] + sizes[b] > n_targets) return CHANGA_E_INVALID_LIST;
  }
  for (long long e = markers[0]; e < markers[n_buckets]; ++e) {
    int idx = list[e].index;
    if (idx < 0 || (long long)idx >= n_sources) return CHANGA_E_INVALID_LIST;
    int code = list[e].offsetID >> 22;
    if (code < 0 || code > 0x1ff) return CHANGA_E_INVALID_LIST;
  }
  return 0;
}

static int check_req(const ChangaListRequest* r) {
  if (!r) return CHANGA_E_INVALID_ARG;
  if (r->n_buckets < 0 || r->n_entries < 0) return CHANGA_E_INVALID_ARG;
  if (r->n_buckets > 0 && (!r->markers || !r->starts || !r->sizes)) return CHANGA_E_INVALID_ARG;
  if (r->n_entries > 0 && !r->list) return CHANGA_E_INVALID_ARG;
  return 0;
}

/* Host particle runs: pointers present, run markers rising from 0 to at
 * most n_runs and flat markers rising from 0 (the copies and chunk bounds
 * read the host arrays through them). */
static int check_runs(const ChangaPartRuns* r) {
  if (!r || r->n_buckets < 0 || r->n_runs < 0) return CHANGA_E_INVALID_ARG;
  if (r->n_buckets == 0) return 0;
  if (!r->run_markers || !r->markers || !r->starts || !r->sizes || (r->n_runs > 0 && !r->runs))
    return CHANGA_E_INVALID_ARG;
  if (r->run_markers[0] != 0 || r->markers[0] != 0) return CHANGA_E_INVALID_ARG;
  for (int b = 0; b < r->n_buckets; ++b)
    if (r->run_markers[b + 1] < r->run_markers[b] || r->markers[b + 1] < r->markers[b])
      return CHANGA_E_INVALID_ARG;
  if (r->run_markers[r->n_buckets] > r->n_runs) return CHANGA_E_INVALID_ARG;
  return 0;
}

/* Particle runs into flat entries: bucket b (of nb; the marker pointers
 * start at the chunk's first bucket) owns runs [rm[b], rm[b+1]) and flat
 * entries [fm[b], fm[b+1]); run {index, off, num} becomes num entries
 * {index + k, off}, k = 0 .. num-1.  One warp per bucket: the lanes take 32
 * runs, an exclusive scan places them, and each write of 32 entries finds
 * its run by a binary search over the lanes' inclusive ends.  Runs past
 * n_runs are not read; writes outside the bucket's flat range or past
 * n_flat are dropped. */
__global__ void expand_runs_kernel(const ILPart* __restrict__ runs, long long n_runs,
                                   const int* __restrict__ rm, const int* __restrict__ fm, int nb,
                                   ILCell* __restrict__ flat, long long n_flat) {
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long b = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nb;
       b += warps) {
    const long long r0 = rm[b] > 0 ? rm[b] : 0;
    const long long r1 = (long long)rm[b + 1] < n_runs ? (long long)rm[b + 1] : n_runs;
    long long pos = fm[b];
    const long long end = (long long)fm[b + 1] < n_flat ? (long long)fm[b + 1] : n_flat;
    for (long long rb = r0; rb < r1; rb += 32) {
      const long long r = rb + lane;
      ILPart run = {0, 0, 0};
      if (r < r1) run = runs[r];
      const int num = run.num > 0 ? (run.num < (1 << 25) ? run.num : (1 << 25)) : 0;
      int incl = num;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(full, incl, 31);
      const int excl = incl - num;
      for (int j0 = 0; j0 < total; j0 += 32) {
        const int j = j0 + lane;
        int owner = 0;
#pragma unroll
        for (int bit = 16; bit > 0; bit >>= 1)
          if (__shfl_sync(full, incl, owner + bit - 1) <= j) owner += bit;
        const int o_excl = __shfl_sync(full, excl, owner);
        const int o_index = __shfl_sync(full, run.index, owner);
        const int o_off = __shfl_sync(full, run.off, owner);
        const long long q = pos + j;
        if (j < total && q >= 0 && q < end) {
          ILCell c;
          c.index = o_index + (j - o_excl);
          c.offsetID = o_off;
          flat[q] = c;
        }
      }
      pos += total;
    }
  }
}

static cudaError_t launch_expand_runs(const ILPart* runs, long long n_runs, const int* rm,
                                      const int* fm, int nb, ILCell* flat, long long n_flat,
                                      cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  long long blocks = ((long long)nb + 7) / 8;
  const long long cap = (long long)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  TimingScope ts(kKidPack, s);
  expand_runs_kernel<<<(int)blocks, 256, 0, s>>>(runs, n_runs, rm, fm, nb, flat, n_flat);
  count_launch();
  return cudaGetLastError();
}

/* One list evaluation over device-resident inputs (FP64 or mixed form). */
static int run_fp(int form, bool cell, const void* src, long long n_src, const void* tgt,
                  long long n_tgt, const ChangaListRequest* req, double fperiod, double* vars,
                  cudaStream_t s, unsigned int* queue) {
  ListArgs a;
  a.src = src;
  a.n_src = n_src;
  a.tgt = tgt;
  a.n_tgt = n_tgt;
  a.vars = vars;
  a.list = (const int2*)req->list;
  a.n_entries = req->n_entries;
  a.markers = req->markers;
  a.starts = req->starts;
  a.sizes = req->sizes;
  a.n_buckets = req->n_buckets;
  a.fperiod_f = (float)fperiod;
  a.fperiod_d = fperiod;
  a.queue = queue;
  CHG_CUDA(cudaMemsetAsync(queue, 0, sizeof(unsigned int), s));
  CHG_CUDA(launch_list(form, cell, a, s));
  return 0;
}

static int forces_entry(int form, bool cell, const double* src, long long n_src,
                        const double* tgt, long long n_tgt, const ChangaListRequest* req,
                        double fperiod, double* vars, cudaStream_t s) {
  int rc = check_req(req);
  if (rc || !src || !tgt || !vars || n_src < 0 || n_tgt < 0)
    return record_error(rc ? rc : CHANGA_E_INVALID_ARG, "forces: arguments", __FILE__, __LINE__);
  if (req->n_buckets == 0) return 0;
  prepare_pool();
  size_t src_b = 0, tgt_b = 0;
  if (form == kMix) {
    src_b = align256((size_t)n_src * (cell ? kCellPackF4 : kPartPackF4) * sizeof(float4));
    tgt_b = align256((size_t)n_tgt * kPartPackF4 * sizeof(float4));
  }
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, src_b + tgt_b + 256, s));
  unsigned int* queue = (unsigned int*)(block + src_b + tgt_b);
  const void* ksrc = src;
  const void* ktgt = tgt;
  if (form == kMix) {
    float4* ps = (float4*)block;
    float4* pt = (float4*)(block + src_b);
    if (cell) CHG_CUDA(launch_pack_cells(src, n_src, ps, s));
    else CHG_CUDA(launch_pack_parts(src, n_src, ps, s));
    CHG_CUDA(launch_pack_parts(tgt, n_tgt, pt, s));
    ksrc = ps;
    ktgt = pt;
  }
  rc = run_fp(form, cell, ksrc, n_src, ktgt, n_tgt, req, fperiod, vars, s, queue);
  if (rc) return rc;
  CHG_CUDA(cudaFreeAsync(block, s));
  return 0;
}

int changa_cell_forces_fp64(const double* moments, long long n_moments, const double* targets,
                            long long n_targets, const ChangaListRequest* req, double fperiod,
                            double* vars, cudaStream_t stream) {
  return forces_entry(kF64, true, moments, n_moments, targets, n_targets, req, fperiod, vars, stream);
}
int changa_part_forces_fp64(const double* sources, long long n_sources, const double* targets,
                            long long n_targets, const ChangaListRequest* req, double fperiod,
                            double* vars, cudaStream_t stream) {
  return forces_entry(kF64, false, sources, n_sources, targets, n_targets, req, fperiod, vars, stream);
}
int changa_cell_forces_mixed(const double* moments, long long n_moments, const double* targets,
                             long long n_targets, const ChangaListRequest* req, double fperiod,
                             double* vars, cudaStream_t stream) {
  return forces_entry(kMix, true, moments, n_moments, targets, n_targets, req, fperiod, vars, stream);
}
int changa_part_forces_mixed(const double* sources, long long n_sources, const double* targets,
                             long long n_targets, const ChangaListRequest* req, double fperiod,
                             double* vars, cudaStream_t stream) {
  return forces_entry(kMix, false, sources, n_sources, targets, n_targets, req, fperiod, vars, stream);
}

int changa_gravity_step(int form, const double* moments, long long n_moments, const double* parts,
                        long long n_parts, const ChangaListRequest* cells,
                        const ChangaListRequest* plist, double fperiod,
                        const ChangaEwaldParams* ewald, double* vars, cudaStream_t s) {
  if (form != CHANGA_FORM_FP64 && form != CHANGA_FORM_MIXED)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step: form", __FILE__, __LINE__);
  if (!moments || !parts || !vars || n_moments < 0 || n_parts < 0)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step: arrays", __FILE__, __LINE__);
  if ((cells && check_req(cells)) || (plist && check_req(plist)))
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step: requests", __FILE__, __LINE__);
  const int f = form == CHANGA_FORM_FP64 ? kF64 : kMix;
  prepare_pool();
  size_t cb = 0, pb = 0;
  if (f == kMix) {
    cb = align256((size_t)n_moments * kCellPackF4 * sizeof(float4));
    pb = align256((size_t)n_parts * kPartPackF4 * sizeof(float4));
  }
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, cb + pb + 512, s));
  unsigned int* q = (unsigned int*)(block + cb + pb);
  const void* ksrc = moments;
  const void* kpart = parts;
  if (f == kMix) {
    CHG_CUDA(launch_pack_cells(moments, n_moments, (float4*)block, s));
    CHG_CUDA(launch_pack_parts(parts, n_parts, (float4*)(block + cb), s));
    ksrc = block;
    kpart = block + cb;
  }
  int rc = 0;
  if (cells && cells->n_buckets > 0)
    rc = run_fp(f, true, ksrc, n_moments, kpart, n_parts, cells, fperiod, vars, s, q);
  if (!rc && plist && plist->n_buckets > 0)
    rc = run_fp(f, false, kpart, n_parts, kpart, n_parts, plist, fperiod, vars, s, q + 64);
  if (!rc && ewald) {
    cudaError_t e = launch_ewald_fp(f, parts, n_parts, nullptr, n_parts, *ewald, vars, s);
    if (e != cudaSuccess) rc = record_error((int)e, "gravity_step: ewald", __FILE__, __LINE__);
  }
  cudaError_t e = cudaFreeAsync(block, s);
  if (!rc && e != cudaSuccess) rc = record_error((int)e, "gravity_step: free", __FILE__, __LINE__);
  return rc;
}

/* Hexadecapole build: cells evaluated with their scaled reduced moments,
 * softened cells as point masses, particles as usual. */
int changa_gravity_step_hexa(int form, const double* moments, long long n_moments,
                             const double* parts, long long n_parts,
                             const ChangaListRequest* cells, const ChangaListRequest* plist,
                             const ChangaListRequest* softcells, double fperiod,
                             const ChangaEwaldParams* ewald, double* vars, cudaStream_t s) {
  if (form != CHANGA_FORM_FP64 && form != CHANGA_FORM_MIXED)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_hexa: form", __FILE__, __LINE__);
  if (!moments || !parts || !vars || n_moments < 0 || n_parts < 0)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_hexa: arrays", __FILE__, __LINE__);
  if ((cells && check_req(cells)) || (plist && check_req(plist)) ||
      (softcells && check_req(softcells)))
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_hexa: requests", __FILE__, __LINE__);
  const int f = form == CHANGA_FORM_FP64 ? kF64 : kMix;
  prepare_pool();
  const size_t qb = align256((size_t)n_moments * 5 * sizeof(double));  // cells as particles
  size_t cb = 0, pb = 0, sb = 0;
  if (f == kMix) {
    cb = align256((size_t)n_moments * kCellHexPackF4 * sizeof(float4));
    pb = align256((size_t)n_parts * kPartPackF4 * sizeof(float4));
    sb = align256((size_t)n_moments * kPartPackF4 * sizeof(float4));
  }
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, qb + cb + pb + sb + 1024, s));
  double* pseudo = (double*)block;
  unsigned int* q = (unsigned int*)(block + qb + cb + pb + sb);
  const void* kcell = moments;
  const void* kpart = parts;
  const void* kpseudo = pseudo;
  int rc = 0;
  cudaError_t e = cudaSuccess;
  do {
    if (softcells && softcells->n_buckets > 0 &&
        (e = launch_cells_as_parts(moments, 27, n_moments, pseudo, s)) != cudaSuccess)
      break;
    if (f == kMix) {
      float4* pc = (float4*)(block + qb);
      float4* pp = (float4*)(block + qb + cb);
      float4* ps = (float4*)(block + qb + cb + pb);
      if ((e = launch_pack_cells_hex(moments, n_moments, pc, s)) != cudaSuccess ||
          (e = launch_pack_parts(parts, n_parts, pp, s)) != cudaSuccess)
        break;
      if (softcells && softcells->n_buckets > 0 &&
          (e = launch_pack_parts(pseudo, n_moments, ps, s)) != cudaSuccess)
        break;
      kcell = pc;
      kpart = pp;
      kpseudo = ps;
    }
    if (cells && cells->n_buckets > 0) {
      ListArgs a;
      a.src = kcell;
      a.n_src = n_moments;
      a.tgt = kpart;
      a.n_tgt = n_parts;
      a.vars = vars;
      a.list = (const int2*)cells->list;
      a.n_entries = cells->n_entries;
      a.markers = cells->markers;
      a.starts = cells->starts;
      a.sizes = cells->sizes;
      a.n_buckets = cells->n_buckets;
      a.fperiod_f = (float)fperiod;
      a.fperiod_d = fperiod;
      a.queue = q;
      if ((e = cudaMemsetAsync(q, 0, sizeof(unsigned int), s)) != cudaSuccess ||
          (e = launch_list_hex(f, a, s)) != cudaSuccess)
        break;
    }
    if (plist && plist->n_buckets > 0)
      rc = run_fp(f, false, kpart, n_parts, kpart, n_parts, plist, fperiod, vars, s, q + 64);
    if (!rc && softcells && softcells->n_buckets > 0)
      rc = run_fp(f, false, kpseudo, n_moments, kpart, n_parts, softcells, fperiod, vars, s,
                  q + 128);
    if (!rc && ewald) {
      e = launch_ewald_fp(f, parts, n_parts, nullptr, n_parts, *ewald, vars, s, true);
      if (e != cudaSuccess)
        rc = record_error((int)e, "gravity_step_hexa: ewald", __FILE__, __LINE__);
      e = cudaSuccess;
    }
  } while (0);
  cudaError_t ef = cudaFreeAsync(block, s);
  if (rc) return rc;
  if (e == cudaSuccess) e = ef;
  if (e != cudaSuccess) return record_error((int)e, "gravity_step_hexa", __FILE__, __LINE__);
  return 0;
}

void changa_gb300_set_host_chunk_bytes(size_t bytes) {
  g_host_chunk_bytes.store(bytes == 0 ? kDefaultHostChunkBytes : bytes < 4096 ? 4096 : bytes);
}

/* Page-locked (or registered) host memory: a read-back into it returns at
 * once, so it can be enqueued between launches without stalling them. */
static bool host_pinned(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

/* Particle range [lo, hi) that the buckets [b0, b1) of r write (clamped to
 * [0, n); empty when lo >= hi). */
static std::pair<long long, long long> target_range(const ChangaListRequest* r, int b0, int b1,
                                                    long long n) {
  long long lo = LLONG_MAX, hi = LLONG_MIN;
  for (int b = b0; b < b1; ++b) {
    const long long st = r->starts[b], sz = r->sizes[b];
    if (sz <= 0 || st < 0 || st + sz > n) continue;  // the kernel skips these buckets
    lo = std::min(lo, st);
    hi = std::max(hi, st + sz);
  }
  if (lo >= hi) return {0, 0};
  return {lo, hi};
}

/* Host-array evaluation, pipelined: the particles go first, in slices that
 * the compute stream packs and gives their Ewald term as they land; then
 * the moments and the small arrays, then each interaction list in chunks of
 * about kChunkBytes, all on a copy stream.  The compute stream packs the
 * moments and launches the list kernel on each chunk's bucket range as
 * soon as its entries have landed, so the list stream from host memory
 * overlaps the force arithmetic.  The last list's
 * chunks shrink toward its end, and when their particle ranges are
 * disjoint and vars is page-locked, each range's results go back on a
 * second copy stream as soon as its kernel is done (every other
 * contribution to those particles is ordered before it), so the read-back
 * overlaps the remaining uploads. */
static int step_host_impl(int form, const double* moments, long long n_moments,
                          const double* parts, long long n_parts, const ChangaListRequest* cells,
                          const ChangaListRequest* plist, const ChangaPartRuns* pruns,
                          double fperiod, const ChangaEwaldParams* ewald, double* vars,
                          cudaStream_t s) {
  const bool overwrite = (form & CHANGA_STEP_OVERWRITE) != 0;
  form &= ~CHANGA_STEP_OVERWRITE;
  if (form != CHANGA_FORM_FP64 && form != CHANGA_FORM_MIXED)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_host: form", __FILE__, __LINE__);
  if (!moments || !parts || !vars || n_moments < 0 || n_parts < 0)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_host: arrays", __FILE__, __LINE__);
  if ((cells && check_req(cells)) || (plist && check_req(plist)) || (pruns && check_runs(pruns)))
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_host: requests", __FILE__, __LINE__);
  /* particle lists as runs: a host view of the flat request they expand to
   * (markers, starts and sizes; the flat entries exist only on the device) */
  ChangaListRequest pview;
  if (pruns) {
    pview.list = nullptr;
    pview.markers = pruns->markers;
    pview.starts = pruns->starts;
    pview.sizes = pruns->sizes;
    pview.n_buckets = pruns->n_buckets;
    pview.n_entries = pruns->n_buckets > 0 ? pruns->markers[pruns->n_buckets] : 0;
    plist = &pview;
  }
  if (ewald && ewald->nEwhLoop > CHANGA_MAX_EWH)
    return record_error(CHANGA_E_TOO_LARGE, "gravity_step_host: nEwhLoop", __FILE__, __LINE__);
  prepare_pool();
  const unsigned long long tma_before = tma_launches();
  const int f = form == CHANGA_FORM_FP64 ? kF64 : kMix;
  cudaStream_t c = library_stream();
  if (!c) return record_error(cudaErrorUnknown, "gravity_step_host: copy stream", __FILE__, __LINE__);
  const size_t kChunkBytes = g_host_chunk_bytes.load();

  cudaStream_t rb = library_stream(1);
  if (!rb) return record_error(cudaErrorUnknown, "gravity_step_host: copy stream", __FILE__, __LINE__);

  /* chunks: [request][bucket range] by entry bytes */
  const ChangaListRequest* reqs[2] = {cells, plist};
  int last = -1;  // the request evaluated last
  for (int k = 0; k < 2; ++k)
    if (reqs[k] && reqs[k]->n_buckets > 0) last = k;
  std::vector<std::pair<int, int>> chunks[2];
  ChangaListRequest rview;  // the runs' own CSR, for chunking the run uploads
  for (int k = 0; k < 2; ++k) {
    const ChangaListRequest* r = reqs[k];
    if (!r || r->n_buckets == 0) continue;
    if (k == 1 && pruns) {
      rview = pview;
      rview.markers = pruns->run_markers;
      rview.n_entries = pruns->n_runs;
      list_chunks(&rview, (long long)(kChunkBytes / sizeof(ILPart)), k == last, chunks[k]);
    } else {
      list_chunks(r, (long long)(kChunkBytes / sizeof(ILCell)), k == last, chunks[k]);
    }
  }

  /* one device block: FP64 inputs, packed inputs, requests, queue counters */
  const size_t mb = align256((size_t)n_moments * 12 * sizeof(double));
  const size_t pb = align256((size_t)n_parts * 5 * sizeof(double));
  const size_t cpb = f == kMix ? align256((size_t)n_moments * kCellPackF4 * sizeof(float4)) : 0;
  const size_t ppb = f == kMix ? align256((size_t)n_parts * kPartPackF4 * sizeof(float4)) : 0;
  size_t off[2][4], sz[2][4];
  size_t total = mb + pb + pb + cpb + ppb;
  for (int k = 0; k < 2; ++k) {
    const ChangaListRequest* r = reqs[k];
    const long long ne = r ? r->n_entries : 0;
    const int nb = r ? r->n_buckets : 0;
    sz[k][0] = (size_t)ne * sizeof(ILCell);
    sz[k][1] = (size_t)(nb + 1) * sizeof(int);
    sz[k][2] = (size_t)nb * sizeof(int);
    sz[k][3] = (size_t)nb * sizeof(int);
    for (int j = 0; j < 4; ++j) {
      off[k][j] = total;
      total += align256(sz[k][j]);
    }
  }
  size_t roff = 0, rmoff = 0;  // runs and their markers (pruns only)
  if (pruns) {
    roff = total;
    total += align256((size_t)pruns->n_runs * sizeof(ILPart));
    rmoff = total;
    total += align256((size_t)(pruns->n_buckets + 1) * sizeof(int));
  }
  const size_t qoff = total;
  total += 256;
  char* block = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&block, total, s));
  double* d_mom = (double*)block;
  double* d_parts = (double*)(block + mb);
  double* d_vars = (double*)(block + mb + pb);
  float4* pc = (float4*)(block + mb + 2 * pb);
  float4* pp = (float4*)(block + mb + 2 * pb + cpb);
  unsigned int* q = (unsigned int*)(block + qoff);

  /* particle slices of about a quarter chunk, uploaded first: each is
   * packed and given its Ewald term as soon as it lands, while the rest of
   * the particles, the moments and the first list chunks are still on the
   * link.  Slices start on multiples of 32 particles, so every warp of the
   * Ewald kernel holds the particles (and culls the replicas) it holds in
   * one launch over all of them: the results do not depend on the slicing. */
  std::vector<std::pair<long long, long long>> slices;
  {
    const long long per =
        std::max<long long>(32, (long long)(kChunkBytes / 4 / (5 * sizeof(double))) & ~31LL);
    for (long long a = 0; a < n_parts; a += per) slices.push_back({a, std::min(n_parts, a + per)});
  }

  std::vector<cudaEvent_t> evs;
  auto event = [&](cudaStream_t on) -> cudaEvent_t {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    evs.push_back(e);
    if (cudaEventRecord(e, on) != cudaSuccess) return nullptr;
    return e;
  };
  int rc = 0;
  cudaError_t e = cudaSuccess;
  do {
    cudaEvent_t ready = event(s);  // the block is allocated on s
    if (!ready || (e = cudaStreamWaitEvent(c, ready, 0)) != cudaSuccess) break;
    /* the particles (and the vars they accumulate into) slice by slice */
    std::vector<cudaEvent_t> sliced;
    for (auto& sl : slices) {
      const size_t o = (size_t)sl.first * 5, b = (size_t)(sl.second - sl.first) * 5 * sizeof(double);
      if ((e = cudaMemcpyAsync(d_parts + o, parts + o, b, cudaMemcpyHostToDevice, c)) !=
              cudaSuccess ||
          (!overwrite &&
           (e = cudaMemcpyAsync(d_vars + o, vars + o, b, cudaMemcpyHostToDevice, c)) != cudaSuccess))
        break;
      sliced.push_back(event(c));
    }
    if (e != cudaSuccess) break;
    /* then the moments and the small arrays */
    if ((e = cudaMemcpyAsync(d_mom, moments, (size_t)n_moments * 12 * sizeof(double),
                             cudaMemcpyHostToDevice, c)) != cudaSuccess)
      break;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      const ChangaListRequest* r = reqs[k];
      if (!r || r->n_buckets == 0) continue;
      const void* src[3] = {r->markers, r->starts, r->sizes};
      for (int j = 1; j < 4 && e == cudaSuccess; ++j)
        e = cudaMemcpyAsync(block + off[k][j], src[j - 1], sz[k][j], cudaMemcpyHostToDevice, c);
    }
    if (e == cudaSuccess && pruns && pruns->n_buckets > 0)
      e = cudaMemcpyAsync(block + rmoff, pruns->run_markers,
                          (size_t)(pruns->n_buckets + 1) * sizeof(int), cudaMemcpyHostToDevice, c);
    if (e != cudaSuccess) break;
    cudaEvent_t small = event(c);
    /* the lists, chunk by chunk */
    std::vector<cudaEvent_t> landed[2];
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      const ChangaListRequest* r = reqs[k];
      for (auto& ch : chunks[k]) {
        if (k == 1 && pruns) {
          const size_t r0 = (size_t)pruns->run_markers[ch.first];
          const size_t r1 = (size_t)pruns->run_markers[ch.second];
          if (r1 > r0 &&
              (e = cudaMemcpyAsync(block + roff + r0 * sizeof(ILPart), pruns->runs + r0,
                                   (r1 - r0) * sizeof(ILPart), cudaMemcpyHostToDevice, c)) !=
                  cudaSuccess)
            break;
          landed[k].push_back(event(c));
          continue;
        }
        const size_t e0 = (size_t)r->markers[ch.first], e1 = (size_t)r->markers[ch.second];
        if (e1 > e0 &&
            (e = cudaMemcpyAsync(block + off[k][0] + e0 * sizeof(ILCell), r->list + e0,
                                 (e1 - e0) * sizeof(ILCell), cudaMemcpyHostToDevice, c)) !=
                cudaSuccess)
          break;
        landed[k].push_back(event(c));
      }
    }
    if (e != cudaSuccess || !small) break;
    /* the last list's particle ranges (host work while the copies run):
     * per-chunk read-backs when they are disjoint */
    std::vector<std::pair<long long, long long>> ranges, gaps;
    bool early = last >= 0 && host_pinned(vars);
    if (early) {
      for (auto& ch : chunks[last])
        ranges.push_back(target_range(reqs[last], ch.first, ch.second, n_parts));
      std::vector<std::pair<long long, long long>> sorted;
      for (auto& g : ranges)
        if (g.first < g.second) sorted.push_back(g);
      std::sort(sorted.begin(), sorted.end());
      for (size_t i = 1; i < sorted.size() && early; ++i)
        early = sorted[i - 1].second <= sorted[i].first;
      /* the particles no chunk of the last list writes: final before it */
      long long at = 0;
      for (auto& g : sorted) {
        if (g.first > at) gaps.push_back({at, g.first});
        at = g.second;
      }
      if (at < n_parts) gaps.push_back({at, n_parts});
    }
    /* Two compute lanes: consecutive chunks of a list alternate between s
     * and a library-owned stream, so each chunk's kernel takes the SMs that
     * the previous chunk's kernel frees while it drains.  Only for a list
     * whose consecutive chunks write disjoint particle ranges (checked
     * here); any other list runs on s alone.  The lanes join before each
     * list and before the last read-back. */
    cudaStream_t s2 = library_stream(2);
    bool dual[2] = {false, false};
    for (int k = 0; k < 2 && s2; ++k) {
      if (chunks[k].size() < 2) continue;
      dual[k] = true;
      std::pair<long long, long long> prev = {0, 0};
      for (size_t i = 0; i < chunks[k].size() && dual[k]; ++i) {
        const auto g = target_range(reqs[k], chunks[k][i].first, chunks[k][i].second, n_parts);
        if (i > 0 && g.first < g.second && prev.first < prev.second)
          dual[k] = g.second <= prev.first || prev.second <= g.first;
        prev = g;
      }
    }
    auto join = [&]() -> cudaError_t {
      if (!s2) return cudaSuccess;
      cudaEvent_t x2 = event(s2);
      if (!x2) return cudaErrorUnknown;
      cudaError_t x = cudaStreamWaitEvent(s, x2, 0);
      if (x != cudaSuccess) return x;
      cudaEvent_t x1 = event(s);
      if (!x1) return cudaErrorUnknown;
      return cudaStreamWaitEvent(s2, x1, 0);
    };
    auto read_back = [&](long long lo, long long hi, cudaStream_t on) -> cudaError_t {
      if (lo >= hi) return cudaSuccess;
      cudaEvent_t done = event(on);
      if (!done) return cudaErrorUnknown;
      cudaError_t x = cudaStreamWaitEvent(rb, done, 0);
      if (x != cudaSuccess) return x;
      return cudaMemcpyAsync(vars + 5 * lo, d_vars + 5 * lo, (size_t)(hi - lo) * 5 * sizeof(double),
                             cudaMemcpyDeviceToHost, rb);
    };
    /* compute stream: each particle slice as it lands, then the moments */
    if (overwrite && (e = cudaMemsetAsync(d_vars, 0, (size_t)n_parts * 5 * sizeof(double), s)) !=
                         cudaSuccess)
      break;
    for (size_t i = 0; i < slices.size() && e == cudaSuccess; ++i) {
      const long long a = slices[i].first, n = slices[i].second - slices[i].first;
      if (!sliced[i]) e = cudaErrorUnknown;
      if (e != cudaSuccess || (e = cudaStreamWaitEvent(s, sliced[i], 0)) != cudaSuccess) break;
      if (f == kMix && (e = launch_pack_parts(d_parts + 5 * a, n, pp + kPartPackF4 * a, s)) !=
                           cudaSuccess)
        break;
      if (ewald && (e = launch_ewald_fp(f, d_parts + 5 * a, n, nullptr, n, *ewald, d_vars + 5 * a,
                                        s)) != cudaSuccess)
        break;
    }
    if (e != cudaSuccess || (e = cudaStreamWaitEvent(s, small, 0)) != cudaSuccess) break;
    const void* ksrc = d_mom;
    const void* kpart = d_parts;
    if (f == kMix) {
      if ((e = launch_pack_cells(d_mom, n_moments, pc, s)) != cudaSuccess) break;
      ksrc = pc;
      kpart = pp;
    }
    for (int k = 0; k < 2 && !rc && e == cudaSuccess; ++k) {
      const ChangaListRequest* r = reqs[k];
      /* both lanes past the packs, the Ewald term and the previous list */
      if ((e = join()) != cudaSuccess) break;
      if (k == last && early) {
        for (size_t i = 0; i < gaps.size() && e == cudaSuccess; ++i)
          e = read_back(gaps[i].first, gaps[i].second, s);
        if (e != cudaSuccess) break;
      }
      for (size_t i = 0; i < chunks[k].size() && !rc && e == cudaSuccess; ++i) {
        const bool second = dual[k] && (i & 1);
        cudaStream_t on = second ? s2 : s;
        if (!landed[k][i]) e = cudaErrorUnknown;
        if (e != cudaSuccess || (e = cudaStreamWaitEvent(on, landed[k][i], 0)) != cudaSuccess)
          break;
        const int b0 = chunks[k][i].first, b1 = chunks[k][i].second;
        if (k == 1 && pruns &&
            (e = launch_expand_runs((const ILPart*)(block + roff), pruns->n_runs,
                                    (const int*)(block + rmoff) + b0,
                                    (const int*)(block + off[k][1]) + b0, b1 - b0,
                                    (ILCell*)(block + off[k][0]), plist->n_entries, on)) !=
                cudaSuccess)
          break;
        ChangaListRequest sub;
        sub.list = (const ILCell*)(block + off[k][0]);
        sub.markers = (const int*)(block + off[k][1]) + b0;
        sub.starts = (const int*)(block + off[k][2]) + b0;
        sub.sizes = (const int*)(block + off[k][3]) + b0;
        sub.n_buckets = b1 - b0;
        sub.n_entries = r->markers[b1];
        /* a queue counter per list and lane (the block's last 256 bytes) */
        unsigned int* qk = q + 32 * k + (second ? 16 : 0);
        rc = k == 0
                 ? run_fp(f, true, ksrc, n_moments, kpart, n_parts, &sub, fperiod, d_vars, on, qk)
                 : run_fp(f, false, kpart, n_parts, kpart, n_parts, &sub, fperiod, d_vars, on, qk);
        if (!rc && k == last && early) e = read_back(ranges[i].first, ranges[i].second, on);
      }
    }
    if (rc || e != cudaSuccess || (e = join()) != cudaSuccess) break;
    if (!early)
      e = cudaMemcpyAsync(vars, d_vars, (size_t)n_parts * 5 * sizeof(double),
                          cudaMemcpyDeviceToHost, s);
  } while (0);
  /* the copy streams and the second lane must be idle before the block goes
   * back to the pool */
  cudaEvent_t copies_done = event(c);
  if (copies_done) cudaStreamWaitEvent(s, copies_done, 0);
  if (cudaStream_t s2 = library_stream(2)) {
    cudaEvent_t lane_done = event(s2);
    if (lane_done) cudaStreamWaitEvent(s, lane_done, 0);
  }
  cudaEvent_t reads_done = event(rb);
  if (reads_done) cudaStreamWaitEvent(s, reads_done, 0);
  cudaError_t ef = cudaFreeAsync(block, s);
  cudaError_t es = cudaStreamSynchronize(s);
  for (cudaEvent_t ev : evs)
    if (ev) cudaEventDestroy(ev);
  if (rc) return rc;
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = es;
  if (e != cudaSuccess) return record_error((int)e, "gravity_step_host", __FILE__, __LINE__);
  if (tma_launches() != tma_before) return changa_gb300_device_status();
  return 0;
}


int changa_gravity_step_host(int form, const double* moments, long long n_moments,
                             const double* parts, long long n_parts, const ChangaListRequest* cells,
                             const ChangaListRequest* plist, double fperiod,
                             const ChangaEwaldParams* ewald, double* vars, cudaStream_t s) {
  return step_host_impl(form, moments, n_moments, parts, n_parts, cells, plist, nullptr, fperiod,
                        ewald, vars, s);
}

int changa_gravity_step_host_runs(int form, const double* moments, long long n_moments,
                                  const double* parts, long long n_parts,
                                  const ChangaListRequest* cells, const ChangaPartRuns* pruns,
                                  double fperiod, const ChangaEwaldParams* ewald, double* vars,
                                  cudaStream_t s) {
  if (!pruns)
    return record_error(CHANGA_E_INVALID_ARG, "gravity_step_host_runs: runs", __FILE__, __LINE__);
  return step_host_impl(form, moments, n_moments, parts, n_parts, cells, nullptr, pruns, fperiod,
                        ewald, vars, s);
}

int changa_ewald_vjp(const double* parts, long long n_parts, const ChangaEwaldParams* p,
                     const double* lam, double* grad, cudaStream_t stream) {
  if (!p || !parts || !lam || !grad || n_parts < 0)
    return record_error(CHANGA_E_INVALID_ARG, "ewald_vjp: arguments", __FILE__, __LINE__);
  if (p->nEwhLoop > CHANGA_MAX_EWH)
    return record_error(CHANGA_E_TOO_LARGE, "ewald_vjp: nEwhLoop", __FILE__, __LINE__);
  /* the quadrupole root expansion: a table without sine terms (a
   * hexadecapole table has them) about a root with mass */
  if (!(p->root[2] > 0) || (p->nEwhLoop > 0 && !p->ewt))
    return record_error(CHANGA_E_INVALID_ARG, "ewald_vjp: root or table", __FILE__, __LINE__);
  for (int i = 0; i < p->nEwhLoop; ++i)
    if (p->ewt[5 * i + 4] != 0.0)
      return record_error(CHANGA_E_INVALID_ARG, "ewald_vjp: sine terms (hexadecapole table)",
                          __FILE__, __LINE__);
  if (n_parts == 0) return 0;
  prepare_pool();
  double* acc = nullptr;
  CHG_CUDA(cudaMallocAsync((void**)&acc, 16 * sizeof(double), stream));
  const cudaError_t e = launch_ewald_vjp(parts, n_parts, *p, lam, grad, acc, stream);
  const cudaError_t ef = cudaFreeAsync(acc, stream);
  if (e != cudaSuccess) return record_error((int)e, "ewald_vjp", __FILE__, __LINE__);
  if (ef != cudaSuccess) return record_error((int)ef, "ewald_vjp: free", __FILE__, __LINE__);
  return 0;
}

int changa_ewald_forces(int form, const double* parts, long long n_parts, const int* idx,
                        long long n_idx, const ChangaEwaldParams* p, double* vars,
                        cudaStream_t stream) {
  if (!p || !parts || !vars || n_idx < 0 || (form != CHANGA_FORM_FP64 && form != CHANGA_FORM_MIXED))
    return record_error(CHANGA_E_INVALID_ARG, "ewald_forces: arguments", __FILE__, __LINE__);
  if (p->nEwhLoop > CHANGA_MAX_EWH)
    return record_error(CHANGA_E_TOO_LARGE, "ewald_forces: nEwhLoop", __FILE__, __LINE__);
  cudaError_t e = launch_ewald_fp(form == CHANGA_FORM_FP64 ? kF64 : kMix, parts, n_parts, idx,
                                  n_idx, *p, vars, stream);
  if (e != cudaSuccess) return record_error((int)e, "ewald_forces: launch", __FILE__, __LINE__);
  return 0;
}

}  // extern "C"

/* ---- CUDA-graph replay of one evaluation (the batching form) ---- */

struct ChangaGravityGraph {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  unsigned kernels;  // kernel nodes in the graph
};

extern "C" ChangaGravityGraph* changa_gravity_graph_create(
    int form, const double* moments, long long n_moments, const double* parts, long long n_parts,
    const ChangaListRequest* cells, const ChangaListRequest* plist, double fperiod,
    const ChangaEwaldParams* ewald, double* vars, int zero_vars) {
  prepare_pool();
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    record_error(CHANGA_E_INVALID_ARG, "graph: stream", __FILE__, __LINE__);
    return nullptr;
  }
  /* warm the occupancy/SM-count caches outside the capture */
  sm_count();
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s);
    record_error((int)e, "graph: begin capture", __FILE__, __LINE__);
    return nullptr;
  }
  int rc = 0;
  if (zero_vars && vars && n_parts > 0) {
    e = cudaMemsetAsync(vars, 0, (size_t)n_parts * 5 * sizeof(double), s);
    if (e != cudaSuccess) rc = (int)e;
  }
  if (!rc)
    rc = changa_gravity_step(form, moments, n_moments, parts, n_parts, cells, plist, fperiod,
                             ewald, vars, s);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(s, &graph);
  cudaStreamDestroy(s);
  if (rc || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    record_error(rc ? rc : (int)e, "graph: capture", __FILE__, __LINE__);
    return nullptr;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    record_error((int)e, "graph: instantiate", __FILE__, __LINE__);
    return nullptr;
  }
  size_t nn = 0;
  unsigned nk = 0;
  if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn) {
    std::vector<cudaGraphNode_t> nodes(nn);
    if (cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
      for (size_t i = 0; i < nn; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
      }
  }
  ChangaGravityGraph* g = new ChangaGravityGraph{graph, exec, nk};
  return g;
}

extern "C" int changa_gravity_graph_launch(ChangaGravityGraph* g, cudaStream_t stream) {
  if (!g) return record_error(CHANGA_E_INVALID_ARG, "graph: NULL", __FILE__, __LINE__);
  CHG_CUDA(cudaGraphLaunch(g->exec, stream));
  count_launch(g->kernels);
  return 0;
}

extern "C" void changa_gravity_graph_destroy(ChangaGravityGraph* g) {
  if (!g) return;
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
}
