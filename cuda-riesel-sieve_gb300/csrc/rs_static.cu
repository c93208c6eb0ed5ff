// rs_static.cu -- the device prime sieve for callers that cannot allocate.
//
// Some hosts of this library cannot call cudaMalloc at the point where they
// want primes: code running under a memory pool or budget that forbids new
// device allocations, plug-ins whose host owns all device memory, or callers
// preparing work for a CUDA graph, where an allocation would have to happen
// outside the captured region.  rs_gpu_primes_static() serves them: the caller
// passes every input and output as device memory it already owns, and the one
// scratch buffer the sieve needs (the bitmap of the window's large-prime pass)
// is a fixed-size array compiled into this file, so the call allocates nothing.
#include <mutex>

#include "rs_internal.h"
#include "rsieve.h"

namespace {

// Window bitmap of the large-prime pass: one bit per odd number, so at most
// kStaticWindowWords * 32 odd numbers per call (a window about 6.7e7 wide).
// Every GPU that loads the library holds these 4 MB until the process exits.
constexpr uint64_t kStaticWindowWords = 1u << 20;
__device__ __align__(256) uint32_t g_static_window_bits[kStaticWindowWords];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
struct StaticAddr {
  unsigned long long ctx_id;  // the context the address belongs to (0: not known)
  uint32_t *ptr;
};
StaticAddr g_static_addr[kMaxDevices] = {};

// Unique id of the current CUDA context (cuCtxGetId, through the runtime's
// driver entry points so that the library needs no link to libcuda), or 0 when
// it cannot be had.  A device reset destroys the primary context and the next
// one gets a new id, which is how a stale cached address is recognised.
unsigned long long current_context_id() {
  typedef int (*GetCurrentFn)(void **);
  typedef int (*GetIdFn)(void *, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(f);
  });
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of g_static_window_bits on the current device.  The array's
// name in host code is only a host-side stand-in, so the address is looked up
// with the device current (cudaGetSymbolAddress) on the first call on each
// device, and again when the device's context has changed since (after a
// cudaDeviceReset the module is loaded anew and the old address is dead).
cudaError_t static_window_bits(int device, uint32_t **out) {
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_static_mu);
  StaticAddr &a = g_static_addr[device];
  if (!a.ptr || (ctx != 0 && ctx != a.ctx_id)) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_window_bits);
    if (e != cudaSuccess) return e;
    a.ptr = static_cast<uint32_t *>(ptr);
    a.ctx_id = ctx ? ctx : current_context_id();
  }
  *out = a.ptr;
  return cudaSuccess;
}

int static_fail(int code, const char *msg, cudaError_t e = cudaSuccess) {
  if (e != cudaSuccess) return rs::set_error(code, "%s: %s", msg, cudaGetErrorString(e));
  return rs::set_error(code, "%s", msg);
}

}  // namespace

extern "C" int rs_gpu_primes_static(uint64_t lo, uint64_t hi, const uint32_t *sieve_primes,
                                    const uint64_t *sieve_rcp, uint32_t n_sieve, uint64_t *out, uint32_t cap,
                                    uint32_t *count, void *stream) {
  if (!sieve_primes || !sieve_rcp || !count || (!out && cap))
    return static_fail(RS_ERR_INVALID, "rs_gpu_primes_static: NULL argument");
  if (hi >= (1ull << 63)) return static_fail(RS_ERR_RANGE, "rs_gpu_primes_static: hi must be < 2^63");
  if (lo < 3) lo = 3;
  if (!(lo & 1)) lo++;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (lo > hi) {
    const cudaError_t e = cudaMemsetAsync(count, 0, 4, st);
    return e == cudaSuccess ? RS_OK : static_fail(RS_ERR_CUDA, "rs_gpu_primes_static: cudaMemsetAsync", e);
  }
  const uint64_t words = rs::sieve_bitmap_words(lo, hi);
  if (words > kStaticWindowWords)
    return static_fail(RS_ERR_RANGE,
                       "rs_gpu_primes_static: window too wide for the static scratch "
                       "(at most 2^25 odd numbers, about 6.7e7 wide); split the range");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return static_fail(RS_ERR_NODEVICE, "rs_gpu_primes_static: cudaGetDevice", e);
  if (device < 0 || device >= kMaxDevices) return static_fail(RS_ERR_INVALID, "rs_gpu_primes_static: device ordinal");
  uint32_t *bits = nullptr;
  e = static_window_bits(device, &bits);
  if (e != cudaSuccess) return static_fail(RS_ERR_CUDA, "rs_gpu_primes_static: cudaGetSymbolAddress", e);
  // With sieve_primes the consecutive odd primes 3, 5, 7, ..., the first 6541
  // are those below 65536, sieved segment by segment; the rest take the bucket
  // pass.  Any other split is still exact, only slower.
  const uint32_t n_small = n_sieve < 6541u ? n_sieve : 6541u;
  e = cudaMemsetAsync(count, 0, 4, st);
  if (e == cudaSuccess)
    e = rs::launch_sieve(lo, hi, sieve_primes, sieve_rcp, n_sieve, n_small, bits, out, count, cap, st);
  if (e != cudaSuccess) return static_fail(RS_ERR_CUDA, "rs_gpu_primes_static: launch", e);
  return RS_OK;
}
