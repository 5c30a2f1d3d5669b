/*
 * Cell-list forces in the FP32-mixed form without any device allocation.
 *
 * changa_cell_forces_mixed() takes stream-ordered scratch from the CUDA
 * pool for the packed moments, the packed targets and the work-queue
 * counter.  Some callers cannot let a library allocate: a host code that
 * has handed all device memory to its own pool allocator up front (a new
 * allocation fails or fragments that pool), or one that enqueues work from a
 * thread that must never block on the device (cudaMalloc and cudaFree may
 * synchronise the whole device, stalling every other stream of that code).
 * changa_cell_forces_mixed_noalloc() gives them the same evaluation with the
 * scratch in one fixed array compiled into this library instead.
 *
 * The array is a file-scope __device__ variable: every GPU that loads the
 * library holds its kNoAllocScratchBytes until the process exits.  Host
 * code cannot use the array's name as a device address, so the first call
 * on each device (made with that device current) looks the address up once
 * with cudaGetSymbolAddress and caches it.  Make that first call before any
 * stream capture begins.  The cache is keyed by the context's id, which the
 * driver never reuses within a process: after cudaDeviceReset the next call
 * finds a new context and looks the address up again in it.
 *
 * All calls share the one array and it keeps the previous call's contents:
 * the work-queue counter is cleared on the call's stream before the kernel
 * runs, and the packed arrays are rewritten in full each call.  Two calls
 * whose work overlaps on the GPU (different streams without ordering) race
 * on the array and give wrong results; serialise them.
 */
#include <cuda.h>

#include <mutex>

#include "chg_internal.h"

namespace {

/* Layout: [queue counter, 256 B][packed moments, 64 B each][packed targets,
 * 32 B each]. */
constexpr size_t kQueueBytes = 256;
constexpr size_t kNoAllocScratchBytes = kQueueBytes + (16u << 20);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
struct ScratchAddr {
  void* ptr = nullptr;
  unsigned long long ctx_id = 0;
};
ScratchAddr g_noalloc_addr[64];

/* The current context's process-unique id (cuCtxGetCurrent + cuCtxGetId,
 * resolved through the runtime so the library needs no -lcuda).  Returns
 * false when the driver does not provide them. */
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    else
      cudaGetLastError();
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    else
      cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" int changa_cell_forces_mixed_noalloc(const double* moments, long long n_moments,
                                                const double* targets, long long n_targets,
                                                const ChangaListRequest* req, double fperiod,
                                                double* vars, cudaStream_t stream) {
  using namespace chg;
  if (!req || !moments || !targets || !vars || n_moments < 0 || n_targets < 0 ||
      req->n_buckets < 0 || req->n_entries < 0 ||
      (req->n_buckets > 0 && (!req->markers || !req->starts || !req->sizes)) ||
      (req->n_entries > 0 && !req->list))
    return record_error(CHANGA_E_INVALID_ARG, "cell_forces_mixed_noalloc: arguments", __FILE__,
                        __LINE__);
  /* the counts are compared before any product is formed, so a huge count
   * cannot wrap around into a small size */
  constexpr size_t kRoom = kNoAllocScratchBytes - kQueueBytes;
  constexpr size_t kMomRec = kCellPackF4 * sizeof(float4), kTgtRec = kPartPackF4 * sizeof(float4);
  bool fits = (unsigned long long)n_moments <= kRoom / kMomRec &&
              (unsigned long long)n_targets <= kRoom / kTgtRec;
  const size_t mom_bytes = fits ? round256((size_t)n_moments * kMomRec) : 0;
  const size_t tgt_bytes = fits ? round256((size_t)n_targets * kTgtRec) : 0;
  if (!fits || mom_bytes + tgt_bytes > kRoom)
    return record_error(CHANGA_E_TOO_LARGE,
                        "cell_forces_mixed_noalloc: 64 B x moments + 32 B x targets exceeds the "
                        "16 MiB fixed scratch",
                        __FILE__, __LINE__);
  if (req->n_buckets == 0) return 0;

  int dev = 0;
  CHG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64)
    return record_error(CHANGA_E_INVALID_ARG, "cell_forces_mixed_noalloc: device id", __FILE__,
                        __LINE__);
  unsigned long long ctx_id = 0;
  const bool have_id = current_context_id(&ctx_id);
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    ScratchAddr& c = g_noalloc_addr[dev];
    if (!c.ptr || !have_id || c.ctx_id != ctx_id) {
      void* p = nullptr;
      CHG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      c.ptr = p;
      c.ctx_id = have_id ? ctx_id : 0;
    }
    base = c.ptr;
  }
  char* scratch = static_cast<char*>(base);
  unsigned int* queue = reinterpret_cast<unsigned int*>(scratch);
  float4* packed_moments = reinterpret_cast<float4*>(scratch + kQueueBytes);
  float4* packed_targets = reinterpret_cast<float4*>(scratch + kQueueBytes + mom_bytes);

  CHG_CUDA(launch_pack_cells(moments, n_moments, packed_moments, stream));
  CHG_CUDA(launch_pack_parts(targets, n_targets, packed_targets, stream));
  CHG_CUDA(cudaMemsetAsync(queue, 0, sizeof(unsigned int), stream));
  ListArgs a;
  a.src = packed_moments;
  a.n_src = n_moments;
  a.tgt = packed_targets;
  a.n_tgt = n_targets;
  a.vars = vars;
  a.list = reinterpret_cast<const int2*>(req->list);
  a.n_entries = req->n_entries;
  a.markers = req->markers;
  a.starts = req->starts;
  a.sizes = req->sizes;
  a.n_buckets = req->n_buckets;
  a.fperiod_f = (float)fperiod;
  a.fperiod_d = fperiod;
  a.queue = queue;
  CHG_CUDA(launch_list(kMix, true, a, stream));
  return 0;
}
