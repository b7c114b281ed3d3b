// Device-side building blocks shared by the sm_103a kernels: key <-> radix-bit
// transforms, warp intrinsics, relaxed/acquire global accesses for the
// decoupled look-back protocols, bounded waits, and the Blackwell bulk-copy
// (TMA) + mbarrier primitives used to stage tiles into shared memory.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mgpu {
namespace device {

// Device-side error codes written into the context's error word.  They map
// to mgpu_status_t on the host.
enum : int {
  err_none = 0,
  err_invalid_arg = 1,
  err_lookback_timeout = 3,
};

// Spin limit of every look-back / mbarrier wait (iterations; each iteration
// is at least one L2 round trip, so the limit is seconds of wall time).
constexpr int spin_limit = 1 << 22;
// How often a spinning thread looks at the error word to leave early.
constexpr int spin_poll_error = 1 << 10;

__host__ __device__ constexpr int64_t div_up(int64_t x, int64_t y) {
  return (x + y - 1) / y;
}

////////////////////////////////////////////////////////////////////////////////
// Order-preserving key <-> unsigned bits (reference: radix_permute_t,
// common/cta_radix.hxx:6-64).  Unsigned: identity.  Signed: flip the MSB.
// Float: flip the MSB; flip all other bits too when the sign was set.

template<typename K> struct radix_key;

template<> struct radix_key<uint32_t> {
  typedef uint32_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(uint32_t x) { return x; }
  __device__ __forceinline__ static uint32_t from_bits(bits_t x) { return x; }
};
template<> struct radix_key<int32_t> {
  typedef uint32_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(int32_t x) { return (uint32_t)x ^ 0x80000000u; }
  __device__ __forceinline__ static int32_t from_bits(bits_t x) { return (int32_t)(x ^ 0x80000000u); }
};
template<> struct radix_key<float> {
  typedef uint32_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(float f) {
    uint32_t y = __float_as_uint(f);
    return y ^ ((uint32_t)((int32_t)y >> 31) | 0x80000000u);
  }
  __device__ __forceinline__ static float from_bits(bits_t x) {
    x ^= 0x80000000u;
    x ^= (uint32_t)((int32_t)x >> 31) & 0x7fffffffu;
    return __uint_as_float(x);
  }
};
template<> struct radix_key<uint64_t> {
  typedef uint64_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(uint64_t x) { return x; }
  __device__ __forceinline__ static uint64_t from_bits(bits_t x) { return x; }
};
template<> struct radix_key<int64_t> {
  typedef uint64_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(int64_t x) {
    return (uint64_t)x ^ 0x8000000000000000ull;
  }
  __device__ __forceinline__ static int64_t from_bits(bits_t x) {
    return (int64_t)(x ^ 0x8000000000000000ull);
  }
};
template<> struct radix_key<double> {
  typedef uint64_t bits_t;
  __device__ __forceinline__ static bits_t to_bits(double f) {
    uint64_t y = (uint64_t)__double_as_longlong(f);
    return y ^ ((uint64_t)((int64_t)y >> 63) | 0x8000000000000000ull);
  }
  __device__ __forceinline__ static double from_bits(bits_t x) {
    x ^= 0x8000000000000000ull;
    x ^= (uint64_t)((int64_t)x >> 63) & 0x7fffffffffffffffull;
    return __longlong_as_double((long long)x);
  }
};

template<typename U>
__device__ __forceinline__ uint32_t extract_digit(U x, int shift, int bits) {
  return (uint32_t)(x >> shift) & ((1u << bits) - 1);
}

////////////////////////////////////////////////////////////////////////////////
// Warp helpers.

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

////////////////////////////////////////////////////////////////////////////////
// Global accesses for look-back protocols (gpu scope).

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Records a device-side error (first one wins) in the context's error word.
__device__ __forceinline__ void raise_error(int* error, int code) {
  if(error) atomicCAS(error, 0, code);
}
__device__ __forceinline__ bool error_raised(const int* error) {
  return error && ld_relaxed((const uint32_t*)error) != 0;
}

////////////////////////////////////////////////////////////////////////////////
// Blackwell bulk copy (cp.async.bulk, the TMA engine's 1-D form) with
// mbarrier completion.  Both addresses must be 16-byte aligned and the size a
// multiple of 16 bytes; callers check that before issuing.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count)
    : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
    :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and raises the error)
// if `limit` polls pass without completion; the caller then must not read
// the staged data.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* error,
  int limit = spin_limit) {
  for(int it = 0; it < limit; ++it) {
    if(mbar_try_wait(bar, parity)) return true;
  }
  raise_error(error, err_lookback_timeout);
  return false;
}

// Bulk copy global -> shared, completion counted on `bar` in bytes.
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, uint32_t bytes,
  uint64_t* bar) {
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
    :: "r"(smem_addr(smem_dst)), "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Asynchronous copy of one naturally aligned 4-, 8- or 16-byte element
// global -> shared (cp.async); cp_async_wait_all() waits for this thread's
// copies.
template<typename T>
__device__ __forceinline__ void cp_async_elem(T* smem_dst, const T* gmem_src) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "cp.async element size");
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;"
    :: "r"(smem_addr(smem_dst)), "l"(gmem_src), "n"((int)sizeof(T)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

__device__ __forceinline__ bool aligned16(const void* p) {
  return 0 == ((uintptr_t)p & 15);
}

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialisation attribute may start while the kernel before it on the
// stream is still running: griddep_wait() returns once that kernel has
// completed and its memory operations are visible (at once when the launch
// had no such predecessor), so it must precede every access to memory the
// predecessor touches.  griddep_launch_dependents() lets the next kernel's
// CTAs be placed as soon as every CTA of this grid has called it (or exited);
// calling it after griddep_wait() keeps at most one waiting grid resident.
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace device
}  // namespace mgpu
