// km_update_noalloc: the centroid update (label sort + exact V.X sums) for
// callers that cannot allocate device memory.
//
// Some hosts own all device memory through their own pool (a serving runtime
// or a framework allocator) and forbid cudaMalloc/cudaFree once they are up:
// those calls synchronise the whole device and fragment the pool.  Others run
// the update inside a latency-critical loop where an allocation is an
// unbounded stall.  km_update (km_capi.cu) allocates its scratch per call; this
// variant keeps all of its scratch in one file-scope device array instead and
// calls no allocating routine at all.  The caller still passes the points,
// labels and output buffers.
//
// The array lives in the library's device image: every GPU that loads the
// library holds its KM_NOALLOC_SCRATCH_BYTES until the process exits.  Host
// code only ever sees a host-side stand-in for it, so the device address is
// looked up with cudaGetSymbolAddress, once per device, with that device
// current, on the first call made on that device.  With lazy module loading
// (the CUDA default) the array may only be placed on the device at that first
// call, so make the first call before a host pool claims the device memory
// (or load modules eagerly, CUDA_MODULE_LOADING=EAGER).  Every call shares the
// array, which keeps the last call's contents: the loop state is cleared at the
// start of each call, and calls that overlap on the GPU (two streams, two host
// threads) race on it.  Each call ends with one synchronisation of its stream
// (it reads the error bits back), so it cannot be recorded into a CUDA graph
// by stream capture.
#include "km_lloyd.cuh"

#include <mutex>

namespace km {

namespace {

constexpr uint64_t NA_MAX_N = KM_NOALLOC_MAX_N;
constexpr uint32_t NA_MAX_K = KM_NOALLOC_MAX_K;
constexpr uint64_t NA_MAX_SEGHIST = 262144;   // k x segments counters

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t NA_OFF_STATE = 0;
constexpr size_t NA_OFF_COUNTS = align256(NA_OFF_STATE + sizeof(DevState));
constexpr size_t NA_OFF_CSTART = align256(NA_OFF_COUNTS + sizeof(uint32_t) * NA_MAX_K);
constexpr size_t NA_OFF_SEGHIST = align256(NA_OFF_CSTART + sizeof(uint32_t) * (NA_MAX_K + 1));
constexpr size_t NA_OFF_PERM = align256(NA_OFF_SEGHIST + sizeof(uint32_t) * NA_MAX_SEGHIST);
constexpr size_t NA_BYTES = align256(NA_OFF_PERM + sizeof(uint32_t) * NA_MAX_N);
static_assert(NA_BYTES <= KM_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

// The scratch array.  Device code could name it directly; host code must not
// pass `g_noalloc_scratch` itself to a kernel (in host code it is only a
// stand-in), it passes the address returned by cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[KM_NOALLOC_SCRATCH_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
unsigned char* g_na_ptr[NA_MAX_DEVICES] = {};

// Per-device set-up: the device address of the scratch array (the device must
// be current) and the kernels' shared-memory opt-in.  No allocation.
km_status noalloc_setup(int dev, unsigned char** out) {
  if (dev < 0 || dev >= NA_MAX_DEVICES) return KM_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    KM_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (!p) return KM_ERR_CUDA;
    KM_TRY(update_sums_prepare());
    g_na_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_na_ptr[dev];
  return KM_OK;
}

}  // namespace
}  // namespace km

using namespace km;

extern "C" km_status km_update_noalloc(const float* X_dev, const uint32_t* labels_dev, uint64_t n,
                                       uint32_t d, uint32_t k, float* C_dev, uint32_t* counts_dev,
                                       void* stream) {
  if (!X_dev || !labels_dev || !C_dev || n == 0 || d == 0 || k == 0 || k > n) return KM_ERR_ARG;
  if (n > NA_MAX_N || k > NA_MAX_K) return KM_ERR_UNSUPPORTED;   // beyond the static scratch
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) { (void)cudaGetLastError(); return KM_ERR_NO_DEVICE; }
  int cc_major = 0, cc_minor = 0;
  KM_CUDA_TRY(cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  KM_CUDA_TRY(cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (cc_major != 10 || cc_minor != 3) return KM_ERR_NO_DEVICE;
  unsigned char* base = nullptr;
  KM_TRY(noalloc_setup(dev, &base));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  DevState* st = reinterpret_cast<DevState*>(base + NA_OFF_STATE);
  uint32_t* counts = reinterpret_cast<uint32_t*>(base + NA_OFF_COUNTS);
  uint32_t* cstart = reinterpret_cast<uint32_t*>(base + NA_OFF_CSTART);
  uint32_t* seghist = reinterpret_cast<uint32_t*>(base + NA_OFF_SEGHIST);
  uint32_t* perm = reinterpret_cast<uint32_t*>(base + NA_OFF_PERM);

  // Segments of `seg` rows with k x nseg <= NA_MAX_SEGHIST (as the engine does).
  uint32_t seg = 1024;
  uint32_t nseg = (uint32_t)((n + seg - 1) / seg);
  while ((uint64_t)k * nseg > NA_MAX_SEGHIST) {
    seg <<= 1;
    nseg = (uint32_t)((n + seg - 1) / seg);
  }
  const size_t per_warp = (size_t)k * 4;     // k <= 1024: at most 4 KB per warp
  const int wpb = 8;
  const size_t smem = per_warp * wpb;

  // The loop state must start at zero (done = 0, no error bits).
  KM_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(DevState), s));
  const unsigned hb = (nseg + wpb - 1) / wpb;
  seg_hist_kernel<<<hb, wpb * 32, smem, s>>>(labels_dev, n, k, seg, nseg, seghist, st);
  seg_scan_kernel<<<(k * 32 + 255) / 256, 256, 0, s>>>(seghist, k, nseg, counts, st, nullptr, nullptr);
  cluster_scan_kernel<<<1, 1024, 0, s>>>(counts, k, cstart, st, nullptr);
  seg_scatter_kernel<<<hb, wpb * 32, smem, s>>>(labels_dev, n, k, seg, nseg, seghist, cstart, perm, st);
  KM_CUDA_TRY(cudaGetLastError());
  // A label >= k only sets an error bit: the sort skips such rows, so every
  // permutation slot the sums read was written by this call and the sums stay
  // in bounds.  The status is read once, after all the work.
  KM_TRY(launch_update_sums(X_dev, perm, cstart, d, k, nullptr, C_dev, nullptr, nullptr, st, s));
  if (counts_dev)
    KM_CUDA_TRY(cudaMemcpyAsync(counts_dev, counts, sizeof(uint32_t) * k, cudaMemcpyDeviceToDevice, s));
  // The one host synchronisation of the call: the error bits of the sort
  // (labels >= k) and of the sums (a bounded wait that ran out).  The copy
  // lands in `err` before the synchronisation returns.
  uint32_t err = 0;
  KM_CUDA_TRY(cudaMemcpyAsync(&err, &st->err, sizeof(err), cudaMemcpyDeviceToHost, s));
  KM_CUDA_TRY(cudaStreamSynchronize(s));
  return status_of_device_error(err);
}
