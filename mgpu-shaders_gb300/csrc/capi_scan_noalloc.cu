// mgpu_scan_noalloc: the single-pass look-back scan for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where allocation is not allowed or not
// possible, for example an operator inside another framework's engine that
// owns all device memory through its own allocator, a plugin whose enqueue
// hook must not allocate (cudaMalloc can synchronise the device and breaks
// stream capture), or a real-time pipeline that forbids allocation after
// start-up.  mgpu_scan needs a context (which allocates its error word and
// may allocate its aux cache) or caller-provided aux; this entry point needs
// neither.
//
// It runs the same persistent deferred look-back scan as mgpu_scan (resident
// CTAs looping over 8192-element tiles), so it scans at the same rate.  Its
// scratch (tile counter, error word, one 64-bit look-back status word per
// tile) lives in the file-scope array below, sized for at most
// MGPU_SCAN_NOALLOC_MAX_COUNT elements: 65,538 words = 512 KiB + 16 bytes
// (the 32,768 tiles of the largest scan use half of the status words).
// Every GPU that loads this library holds that array until the process exits.
// All calls share it, and it keeps the last call's contents: each call clears
// the tile counter and the status words it will use before its kernel runs.
// The error word is not cleared by a scan: a bounded look-back wait that gave
// up stays recorded until mgpu_scan_noalloc_status() reads and clears it.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads, on the same device) race on the array; callers must order them,
// for example by issuing them on one stream.
//
// The array's host-side name is only a stand-in, not a device address; the
// device address comes from cudaGetSymbolAddress, called once per device with
// that device current, the first time this entry point (or the status query)
// runs on it.  Make that first call outside any stream capture.  The address
// is kept for the life of the process, so cudaDeviceReset() on a device after
// its first call here is not supported: the module may be loaded again at
// another address.
#include "mgpu_gb300.h"
#include "mgpu/device/scan.cuh"

#include <algorithm>
#include <mutex>

namespace {

using namespace mgpu::device;

constexpr int kThreads = 256;
constexpr int kItems = 32;
constexpr int kMinBlocks = 4;
constexpr int64_t kTile = (int64_t)kThreads * kItems;
// The array keeps one status word per 4096 elements; the scan uses one per
// 8192-element tile.
constexpr int64_t kMaxTiles = MGPU_SCAN_NOALLOC_MAX_COUNT / 4096;
constexpr int kMaxDevices = 64;
static_assert(MGPU_SCAN_NOALLOC_MAX_COUNT % kTile == 0, "whole tiles");
static_assert(MGPU_SCAN_NOALLOC_MAX_COUNT / kTile <= kMaxTiles, "status words fit");

// Word 0: tile counter (low 32 bits).  Word 1: device error word.
// Words 2 .. 2 + kMaxTiles: look-back status of each tile.
static __device__ __align__(256) uint64_t g_noalloc_scan_scratch[2 + kMaxTiles];

std::mutex g_setup_mutex;
uint64_t* g_scratch_address[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
cudaError_t scratch_address(int device, uint64_t** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if(!g_scratch_address[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
    if(e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&g_sm_count[device], cudaDevAttrMultiProcessorCount, device);
    if(e != cudaSuccess) return e;
    g_scratch_address[device] = (uint64_t*)p;
  }
  *out = g_scratch_address[device];
  return cudaSuccess;
}

// Resident CTAs of the deferred scan kernel per SM (an occupancy query; no
// allocation).
template<typename K>
int resident_ctas(K kernel, size_t smem) {
  int n = 0;
  if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kThreads, smem) != cudaSuccess)
    return 0;
  return n;
}

template<typename T, typename op_t, bool exclusive>
mgpu_status_t launch_defer(cudaStream_t stream, const T* in, T* out, int64_t count, T init,
  T* reduction, tile_status_t<T> status, uint32_t* counter, int* error, int vec, int sm_count) {
  typedef scan_defer_layout<T, kThreads, kItems> L;
  auto k = scan_defer_kernel<T, op_t, kThreads, kItems, exclusive, kMinBlocks>;
  const int per_sm = resident_ctas(k, L::bytes);
  if(per_sm < 1) return MGPU_ERR_CUDA;
  const int64_t num_tiles = div_up(count, kTile);
  const int64_t grid = std::min<int64_t>((int64_t)per_sm * sm_count, num_tiles);
  k<<<(unsigned)grid, kThreads, L::bytes, stream>>>(in, out, count, init, op_t(), status,
    counter, reduction, error, vec);
  return cudaGetLastError() == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
}

template<typename T, typename op_t>
mgpu_status_t launch(cudaStream_t stream, mgpu_scan_type_t scan_type, const void* in, void* out,
  int64_t count, const void* init_p, void* reduction, uint64_t* scratch, int sm_count) {
  T init = op_t::identity();
  if(init_p) memcpy(&init, init_p, sizeof(T));
  if(count == 0) {
    if(reduction) store_value_kernel<T><<<1, 1, 0, stream>>>((T*)reduction, init);
    return cudaGetLastError() == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
  }
  const int64_t num_tiles = div_up(count, kTile);
  // Word 1 (the error word) keeps what earlier calls recorded.
  if(cudaMemsetAsync(scratch, 0, sizeof(uint64_t), stream) != cudaSuccess ||
     cudaMemsetAsync(scratch + 2, 0, sizeof(uint64_t) * num_tiles, stream) != cudaSuccess)
    return MGPU_ERR_CUDA;
  tile_status_t<T> status;
  status.bind(scratch + 2, num_tiles);
  uint32_t* counter = (uint32_t*)scratch;
  int* error = (int*)(scratch + 1);
  int vec = 0 == (((uintptr_t)in | (uintptr_t)out) & 15);
  if(scan_type == MGPU_SCAN_EXC)
    return launch_defer<T, op_t, true>(stream, (const T*)in, (T*)out, count, init, (T*)reduction,
      status, counter, error, vec, sm_count);
  return launch_defer<T, op_t, false>(stream, (const T*)in, (T*)out, count, init, (T*)reduction,
    status, counter, error, vec, sm_count);
}

template<typename T>
mgpu_status_t by_op(mgpu_op_t op, cudaStream_t s, mgpu_scan_type_t st, const void* in,
  void* out, int64_t count, const void* init, void* red, uint64_t* scratch, int sm) {
  switch(op) {
    case MGPU_PLUS: return launch<T, plus_t<T>>(s, st, in, out, count, init, red, scratch, sm);
    case MGPU_MAX: return launch<T, max_t<T>>(s, st, in, out, count, init, red, scratch, sm);
    case MGPU_MIN: return launch<T, min_t<T>>(s, st, in, out, count, init, red, scratch, sm);
  }
  return MGPU_ERR_INVALID_ARG;
}

// Self test of the status path: a bounded wait on a flag that nothing sets
// gives up after `limit` polls and records the timeout in the scan's error
// word, exactly as a scan look-back that gave up would.
__device__ uint32_t g_noalloc_never_set = 0;

__global__ void noalloc_wait_probe(int limit, int* error) {
  int spins = 0;
  while(ld_relaxed(&g_noalloc_never_set) == 0) {
    if(++spins >= limit) {
      raise_error(error, err_lookback_timeout);
      break;
    }
    __nanosleep(64);
  }
}

}  // namespace

extern "C" mgpu_status_t mgpu_scan_noalloc_status(void* stream) {
  int device = 0;
  if(cudaGetDevice(&device) != cudaSuccess) return MGPU_ERR_CUDA;
  if(device < 0 || device >= kMaxDevices) return MGPU_ERR_UNSUPPORTED;
  uint64_t* scratch = nullptr;
  if(scratch_address(device, &scratch) != cudaSuccess) return MGPU_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  int word = 0;
  if(cudaMemcpyAsync(&word, scratch + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
     cudaStreamSynchronize(s) != cudaSuccess)
    return MGPU_ERR_CUDA;
  if(word == 0) return MGPU_OK;
  if(cudaMemsetAsync(scratch + 1, 0, sizeof(uint64_t), s) != cudaSuccess ||
     cudaStreamSynchronize(s) != cudaSuccess)
    return MGPU_ERR_CUDA;
  return word == err_lookback_timeout ? MGPU_ERR_LOOKBACK_TIMEOUT : MGPU_ERR_CUDA;
}

extern "C" mgpu_status_t mgpu_selftest_scan_noalloc_wait(void* stream, int limit) {
  if(limit < 1 || limit > spin_limit) return MGPU_ERR_INVALID_ARG;
  int device = 0;
  if(cudaGetDevice(&device) != cudaSuccess) return MGPU_ERR_CUDA;
  if(device < 0 || device >= kMaxDevices) return MGPU_ERR_UNSUPPORTED;
  uint64_t* scratch = nullptr;
  if(scratch_address(device, &scratch) != cudaSuccess) return MGPU_ERR_CUDA;
  noalloc_wait_probe<<<1, 1, 0, (cudaStream_t)stream>>>(limit, (int*)(scratch + 1));
  return cudaGetLastError() == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
}

extern "C" mgpu_status_t mgpu_scan_noalloc(void* stream, mgpu_dtype_t type,
  mgpu_scan_type_t scan_type, mgpu_op_t op, const void* in, void* out, int64_t count,
  const void* init, void* reduction) {
  if(count < 0 || count > MGPU_SCAN_NOALLOC_MAX_COUNT) return MGPU_ERR_INVALID_ARG;
  if(scan_type != MGPU_SCAN_EXC && scan_type != MGPU_SCAN_INC) return MGPU_ERR_INVALID_ARG;
  if(op != MGPU_PLUS && op != MGPU_MAX && op != MGPU_MIN) return MGPU_ERR_INVALID_ARG;
  if(type != MGPU_I32 && type != MGPU_U32 && type != MGPU_F32) return MGPU_ERR_UNSUPPORTED;
  if(count > 0 && (!in || !out)) return MGPU_ERR_INVALID_ARG;
  int device = 0;
  if(cudaGetDevice(&device) != cudaSuccess) return MGPU_ERR_CUDA;
  if(device < 0 || device >= kMaxDevices) return MGPU_ERR_UNSUPPORTED;
  uint64_t* scratch = nullptr;
  if(scratch_address(device, &scratch) != cudaSuccess) return MGPU_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const int sm = g_sm_count[device];
  switch(type) {
    case MGPU_I32: return by_op<int32_t>(op, s, scan_type, in, out, count, init, reduction, scratch, sm);
    case MGPU_U32: return by_op<uint32_t>(op, s, scan_type, in, out, count, init, reduction, scratch, sm);
    case MGPU_F32: return by_op<float>(op, s, scan_type, in, out, count, init, reduction, scratch, sm);
    default: break;
  }
  return MGPU_ERR_UNSUPPORTED;
}
