// CUDA context for the mgpu primitives on GB300: device, stream, grow-only
// device cache, device-side error word and launch profiling.
//
// Replaces the reference's Vulkan runtime (vk/context.hxx:11-134,
// src/vk/context.cxx:15-439): context_t owned a device, one compute queue, a
// VMA allocator and a pipeline cache; cmd_buffer_t recorded dispatches that
// ran on submit; memcache_t was a grow-only scratch buffer.  Here work is
// enqueued on a CUDA stream in order (no per-dispatch barrier is needed:
// kernels on one stream are ordered), allocation is cudaMalloc / pinned
// cudaMallocHost, and the cache is a stream-ordered grow-only allocation.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "mgpu_gb300.h"
#include "tuning.hxx"
#include <cstdlib>

namespace mgpu {
namespace gb300 {

typedef mgpu_status_t status_t;

struct context_t {
  explicit context_t(int device_ = 0, cudaStream_t stream_ = nullptr) : device(device_) {
    init_status = MGPU_OK;
    if(check(cudaSetDevice(device))) { init_status = MGPU_ERR_CUDA; return; }
    if(check(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device))) {
      init_status = MGPU_ERR_CUDA; return;
    }
    if(stream_) {
      stream = stream_;
    } else {
      if(check(cudaStreamCreateWithFlags(&owned_stream, cudaStreamNonBlocking))) {
        init_status = MGPU_ERR_CUDA; return;
      }
      stream = owned_stream;
    }
    if(check(cudaMalloc(&d_error, sizeof(int)))) { init_status = MGPU_ERR_OOM; return; }
    if(check(cudaMemsetAsync(d_error, 0, sizeof(int), stream))) { init_status = MGPU_ERR_CUDA; return; }
    check(cudaStreamSynchronize(stream));
    if(const char* path = getenv("MGPU_TUNE_FILE")) tuning.load(path);
  }

  ~context_t() {
    if(stream) cudaStreamSynchronize(stream);
    for(auto& r : pending) { release_event(r.begin); release_event(r.end); }
    for(cudaEvent_t e : event_pool) cudaEventDestroy(e);
    if(cache) cudaFree(cache);
    for(void* p : host_allocs) cudaFreeHost(p);
    for(void* p : device_allocs) cudaFree(p);
    if(d_error) cudaFree(d_error);
    if(owned_stream) cudaStreamDestroy(owned_stream);
  }

  context_t(const context_t&) = delete;
  context_t& operator=(const context_t&) = delete;

  operator cudaStream_t() const { return stream; }

  // Records the text of a failing CUDA call; returns true on failure.
  bool check(cudaError_t e) {
    if(e == cudaSuccess) return false;
    last_error = cudaGetErrorString(e);
    return true;
  }

  // ---- allocation (context_t::alloc_gpu / alloc_cpu / free) ----
  void* alloc_gpu(size_t bytes) {
    void* p = nullptr;
    if(check(cudaMalloc(&p, bytes ? bytes : 1))) return nullptr;
    device_allocs.insert(p);
    return p;
  }
  template<typename T> T* alloc_gpu(size_t count) { return (T*)alloc_gpu(sizeof(T) * count); }

  void* alloc_cpu(size_t bytes) {
    void* p = nullptr;
    if(check(cudaMallocHost(&p, bytes ? bytes : 1))) return nullptr;
    host_allocs.insert(p);
    return p;
  }
  template<typename T> T* alloc_cpu(size_t count) { return (T*)alloc_cpu(sizeof(T) * count); }

  status_t free(void* p) {
    if(!p) return MGPU_OK;
    if(host_allocs.erase(p)) return check(cudaFreeHost(p)) ? MGPU_ERR_CUDA : MGPU_OK;
    if(device_allocs.erase(p)) return check(cudaFree(p)) ? MGPU_ERR_CUDA : MGPU_OK;
    return MGPU_ERR_INVALID_ARG;
  }

  status_t memcpy(void* dest, const void* src, size_t bytes) {
    return check(cudaMemcpyAsync(dest, src, bytes, cudaMemcpyDefault, stream))
      ? MGPU_ERR_CUDA : MGPU_OK;
  }

  // ---- grow-only device cache (memcache_t::allocate) ----
  // Growing frees the old block in stream order, so work already enqueued
  // that uses it is unaffected.
  void* cache_allocate(size_t bytes) {
    if(bytes > cache_capacity) {
      if(capturing) {
        last_error = "aux cache too small during graph capture; reserve it first";
        return nullptr;
      }
      if(cache) check(cudaFreeAsync(cache, stream));
      cache = nullptr;
      cache_capacity = 0;
      if(check(cudaMallocAsync(&cache, bytes, stream))) return nullptr;
      cache_capacity = bytes;
    }
    return cache;
  }

  // ---- errors ----
  // Waits for the stream, then reads and clears the device error word.
  status_t synchronize() {
    if(check(cudaStreamSynchronize(stream))) return MGPU_ERR_CUDA;
    int h = 0;
    if(check(cudaMemcpy(&h, d_error, sizeof(int), cudaMemcpyDeviceToHost))) return MGPU_ERR_CUDA;
    if(h) {
      if(check(cudaMemset(d_error, 0, sizeof(int)))) return MGPU_ERR_CUDA;
      return (status_t)h;
    }
    return MGPU_OK;
  }

  // ---- launches and profiling ----
  struct record_t { const char* name; cudaEvent_t begin, end; };

  cudaEvent_t acquire_event() {
    if(!event_pool.empty()) { cudaEvent_t e = event_pool.back(); event_pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    check(cudaEventCreate(&e));
    return e;
  }
  void release_event(cudaEvent_t e) { if(e) event_pool.push_back(e); }

  // Runs `enqueue` (which launches one kernel on `stream`), bracketing it with
  // events when profiling is on.
  template<typename F>
  status_t launch(const char* name, F&& enqueue) {
    record_t r { name, nullptr, nullptr };
    const bool timed = profiling && !capturing;
    if(timed) { r.begin = acquire_event(); cudaEventRecord(r.begin, stream); }
    enqueue();
    ++launches;
    cudaError_t e = cudaGetLastError();
    if(timed) { r.end = acquire_event(); cudaEventRecord(r.end, stream); pending.push_back(r); }
    return check(e) ? MGPU_ERR_CUDA : MGPU_OK;
  }

  // Enqueues `kernel` on `stream` with programmatic dependent launch allowed
  // (unless the stream is being captured into a graph, by this context or
  // by its caller): its CTAs may be placed while the previous kernel on the
  // stream is still running, so the kernel must call device::griddep_wait()
  // before it touches memory that kernel uses.  For chains of short,
  // latency-bound launches (mergesort passes over a few MB) this hides each
  // launch's ramp behind its predecessor's tail.  A failed launch is left
  // for cudaGetLastError(), which launch() reads.
  template<typename... P, typename... A>
  void enqueue_dependent(void (*kernel)(P...), unsigned grid, unsigned block, size_t smem,
    A&&... args) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const bool captured = capturing ||
      cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = captured ? 0 : 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
  }

  // Resolves pending event pairs into per-kernel totals.
  status_t collect_profile() {
    if(check(cudaStreamSynchronize(stream))) return MGPU_ERR_CUDA;
    for(auto& r : pending) {
      float ms = 0;
      cudaEventElapsedTime(&ms, r.begin, r.end);
      auto& t = profile[r.name];
      t.first += 1;
      t.second += ms;
      release_event(r.begin);
      release_event(r.end);
    }
    pending.clear();
    return MGPU_OK;
  }

  // Sets the dynamic shared memory limit of a kernel once per device.
  template<typename kernel_t>
  bool allow_smem(kernel_t kernel, size_t bytes) {
    if(bytes <= 48 * 1024) return true;
    auto key = std::make_pair((const void*)kernel, device);
    if(smem_configured.count(key)) return true;
    if(check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)bytes))) return false;
    smem_configured.insert(key);
    return true;
  }

  // CTAs of `kernel` resident per SM at `nt` threads and `smem` dynamic
  // shared bytes (cached per kernel and device); 0 on error.
  template<typename kernel_t>
  int resident_ctas(kernel_t kernel, int nt, size_t smem) {
    auto key = std::make_pair((const void*)kernel, device);
    auto it = occupancy.find(key);
    if(it != occupancy.end()) return it->second;
    int n = 0;
    if(check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, nt, smem))) return 0;
    occupancy[key] = n;
    return n;
  }

  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t owned_stream = nullptr;
  int* d_error = nullptr;
  // Polls before a radix pass's look-back or copy wait gives up and raises
  // MGPU_ERR_LOOKBACK_TIMEOUT; 0 keeps the library's limit (seconds).
  int wait_limit = 0;
  status_t init_status = MGPU_OK;
  std::string last_error;

  void* cache = nullptr;
  size_t cache_capacity = 0;
  std::set<void*> host_allocs, device_allocs;

  tuning_table_t tuning;
  bool profiling = false;
  bool capturing = false;
  int64_t launches = 0;
  std::vector<record_t> pending;
  std::vector<cudaEvent_t> event_pool;
  std::map<std::string, std::pair<int64_t, double>> profile;
  std::set<std::pair<const void*, int>> smem_configured;
  std::map<std::pair<const void*, int>, int> occupancy;
};

// Source compatibility with code written against cmd_buffer_t
// (vk/context.hxx:93-108): recording is immediate enqueueing on the
// context's stream, so begin/end/submit/host_barrier have nothing to do.
struct cmd_buffer_t {
  explicit cmd_buffer_t(context_t& c) : context(c) {}
  operator context_t&() { return context; }
  void reset() {}
  void begin() {}
  void end() {}
  void submit() {}
  void host_barrier() {}
  void memcpy(void* dest, const void* source, size_t size) { context.memcpy(dest, source, size); }
  context_t& context;
};

// Drop-in for vk::memcache_t (vk/context.hxx:110-134): a grow-only device
// scratch buffer of its own (apart from the context's aux cache, which the
// primitives use).  allocate() returns the buffer's start, grown to at least
// the size asked for; growing releases the old block in stream order, so
// work already enqueued on the context's stream that uses it is unaffected,
// but the pointers an earlier allocate() returned are then stale.  The array
// form carves 256-byte-aligned pieces of one allocation.
struct memcache_t {
  explicit memcache_t(context_t& c) : context(c) {}
  ~memcache_t() { if(data) cudaFreeAsync(data, context.stream); }
  memcache_t(const memcache_t&) = delete;
  memcache_t& operator=(const memcache_t&) = delete;

  template<typename type_t>
  type_t* allocate(size_t count) { return (type_t*)allocate(sizeof(type_t) * count); }

  void* allocate(size_t size) {
    if(size > capacity) {
      if(data) context.check(cudaFreeAsync(data, context.stream));
      data = nullptr;
      capacity = 0;
      if(context.check(cudaMallocAsync(&data, size, context.stream))) return nullptr;
      capacity = size;
    }
    return data;
  }

  template<size_t count>
  std::array<void*, count> allocate(std::array<size_t, count> sizes) {
    std::array<void*, count> out;
    allocate(sizes.data(), (int)count, out.data());
    return out;
  }

  void allocate(const size_t* sizes, int count, void** allocations) {
    size_t total = 0;
    for(int i = 0; i < count; ++i) total += (sizes[i] + 255) & ~(size_t)255;
    char* p = (char*)allocate(total);
    for(int i = 0; i < count; ++i) {
      allocations[i] = p;
      if(p) p += (sizes[i] + 255) & ~(size_t)255;
    }
  }

  context_t& context;
  void* data = nullptr;
  size_t capacity = 0;
};

inline bool aligned16_host(const void* p) { return 0 == ((uintptr_t)p & 15); }

// Carves aligned sub-buffers out of an aux block (advance_pointer,
// common/meta.hxx:119-124, with 256-byte alignment).
struct aux_layout_t {
  size_t total = 0;
  size_t add(size_t bytes) {
    size_t off = total;
    total += (bytes + 255) & ~(size_t)255;
    return off;
  }
};

// Resolves the two-phase aux protocol.  Returns true when the caller should
// return `status` immediately (sizing pass or error); otherwise sets `base`.
inline bool resolve_aux(context_t& ctx, void* aux_data, size_t* aux_size, size_t needed,
  char*& base, status_t& status) {
  status = MGPU_OK;
  if(aux_size == nullptr) {
    base = needed ? (char*)ctx.cache_allocate(needed) : nullptr;
    if(needed && !base) { status = MGPU_ERR_OOM; return true; }
    return false;
  }
  if(!aux_data) { *aux_size += needed; return true; }
  // The kernels bulk-copy from aux and update 8-byte words in it.
  if(*aux_size < needed || ((uintptr_t)aux_data & 15)) {
    status = MGPU_ERR_INVALID_ARG;
    return true;
  }
  base = (char*)aux_data;
  return false;
}

}  // namespace gb300
}  // namespace mgpu
