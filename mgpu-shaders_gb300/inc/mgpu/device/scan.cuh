// Single-pass scan (decoupled look-back) and single-launch reduce for sm_103a.
//
// Reference behaviour: vk::scan (vk/scan.hxx:10-115) is an in-place
// exclusive scan built from cta_scan_t (common/cta_scan.hxx:80-175) as either
// one CTA looping over <= 8 tiles or an upsweep reduce / recursive scan of the
// partials / downsweep with carry-in: three launches per recursion level and
// 12 bytes of traffic per 4-byte element.  Here one launch reads each element
// once and writes it once (8 B/elem): each CTA takes the next tile id from an
// atomic counter, scans its tile in registers, publishes its aggregate, and
// warp 0 walks back over predecessor tiles 32 at a time until it meets an
// inclusive prefix.  The same kernel serves every size.
//
// Operators carry their identity (used for padding and lane 0 of an
// exclusive warp scan); integer addition wraps in two's complement, as the
// GPU's adds do in the reference.
#pragma once

#include "common.cuh"
#include <cfloat>
#include <climits>
#include <type_traits>

namespace mgpu {
namespace device {

template<typename T> struct plus_t {
  __host__ __device__ static T identity() { return T(0); }
  __device__ __forceinline__ T operator()(T a, T b) const {
    if constexpr(std::is_integral<T>::value) {
      typedef typename std::make_unsigned<T>::type U;
      return (T)((U)a + (U)b);
    } else {
      return a + b;
    }
  }
};

template<typename T> struct max_t {
  __host__ __device__ static T identity() {
    if constexpr(std::is_same<T, float>::value) return -__builtin_huge_valf();
    else if constexpr(std::is_same<T, double>::value) return -__builtin_huge_val();
    else if constexpr(std::is_signed<T>::value) return (T)((typename std::make_unsigned<T>::type)1 << (8 * sizeof(T) - 1));
    else return T(0);
  }
  __device__ __forceinline__ T operator()(T a, T b) const { return a > b ? a : b; }
};

template<typename T> struct min_t {
  __host__ __device__ static T identity() {
    if constexpr(std::is_same<T, float>::value) return __builtin_huge_valf();
    else if constexpr(std::is_same<T, double>::value) return __builtin_huge_val();
    else if constexpr(std::is_signed<T>::value) return (T)(~((typename std::make_unsigned<T>::type)1 << (8 * sizeof(T) - 1)));
    else return (T)~T(0);
  }
  __device__ __forceinline__ T operator()(T a, T b) const { return a < b ? a : b; }
};

enum : uint32_t { status_invalid = 0, status_aggregate = 1, status_inclusive = 2 };

// Per-tile look-back status.  4-byte values share one 64-bit word with their
// flag (a single store publishes both).  8-byte values use one value word per
// status (aggregate, inclusive) and a flag word ordered by release/acquire; a
// reader loads the value slot of the flag it saw, so a later inclusive
// publication can never be mistaken for the aggregate.
template<typename T, bool wide = (sizeof(T) == 8)>
struct tile_status_t;

template<typename T>
struct tile_status_t<T, false> {
  uint64_t* words;
  static size_t bytes(int64_t tiles) { return sizeof(uint64_t) * tiles; }
  __host__ __device__ void bind(void* p, int64_t) { words = (uint64_t*)p; }
  __device__ __forceinline__ void publish(int64_t tile, uint32_t flag, T v) const {
    uint32_t b;
    memcpy(&b, &v, 4);
    st_relaxed(words + tile, ((uint64_t)flag << 32) | b);
  }
  __device__ __forceinline__ uint32_t read(int64_t tile, T& v) const {
    uint64_t w = ld_relaxed(words + tile);
    uint32_t b = (uint32_t)w;
    memcpy(&v, &b, 4);
    return (uint32_t)(w >> 32);
  }
};

template<typename T>
struct tile_status_t<T, true> {
  uint64_t* values;          // [2][tiles]: aggregate slot, inclusive slot
  uint32_t* flags;
  int64_t tiles;
  static size_t bytes(int64_t tiles) { return (2 * sizeof(uint64_t) + sizeof(uint32_t)) * tiles + 16; }
  __host__ __device__ void bind(void* p, int64_t n) {
    values = (uint64_t*)p;
    flags = (uint32_t*)(values + 2 * n);
    tiles = n;
  }
  __device__ __forceinline__ void publish(int64_t tile, uint32_t flag, T v) const {
    uint64_t b;
    memcpy(&b, &v, 8);
    st_relaxed(values + (flag == status_inclusive ? tiles : 0) + tile, b);
    st_release(flags + tile, flag);
  }
  __device__ __forceinline__ uint32_t read(int64_t tile, T& v) const {
    uint32_t f = ld_acquire(flags + tile);
    if(f) {
      uint64_t b = ld_relaxed(values + (f == status_inclusive ? tiles : 0) + tile);
      memcpy(&v, &b, 8);
    }
    return f;
  }
};

// Warp 0 of a tile: returns the exclusive prefix of all earlier tiles (which
// already include `init` through tile 0's inclusive value).  Walks back 32
// tiles per step; lane i looks at tile (base - i).
template<typename T, typename op_t, typename status_t>
__device__ T lookback_warp(const status_t& st, int64_t tile, op_t op, int* error) {
  const int lane = threadIdx.x & 31;
  T acc = op_t::identity();
  bool have = false;
  int64_t base = tile - 1;
  while(true) {
    int64_t j = base - lane;
    T v = op_t::identity();
    uint32_t flag = status_inclusive;
    if(j >= 0) {
      int spins = 0;
      while(true) {
        flag = st.read(j, v);
        if(flag != status_invalid) break;
        if(++spins >= spin_limit ||
           (0 == (spins & (spin_poll_error - 1)) && error_raised(error))) {
          raise_error(error, err_lookback_timeout);
          flag = status_inclusive;
          v = op_t::identity();
          break;
        }
      }
    }
    uint32_t inc_mask = __ballot_sync(0xffffffffu, flag == status_inclusive);
    int limit = inc_mask ? __ffs(inc_mask) - 1 : 31;
    // Ordered reduction of lanes [0, limit]: the earlier tile (higher lane)
    // is the left operand.
#pragma unroll
    for(int off = 1; off < 32; off <<= 1) {
      T y = __shfl_down_sync(0xffffffffu, v, off);
      if(lane + off <= limit) v = op(y, v);
    }
    T r = __shfl_sync(0xffffffffu, v, 0);
    acc = have ? op(r, acc) : r;
    have = true;
    if(inc_mask) return acc;
    base -= 32;
  }
}

template<typename T, typename op_t>
__device__ __forceinline__ T warp_inclusive_scan(T x, op_t op) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for(int off = 1; off < 32; off <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, off);
    if(lane >= off) x = op(y, x);
  }
  return x;
}

template<typename T, typename op_t>
__device__ __forceinline__ T warp_reduce(T x, op_t op) {
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) x = op(x, __shfl_down_sync(0xffffffffu, x, off));
  return x;
}

// Loads VT consecutive elements of thread `tid` (thread-contiguous layout),
// with 16-byte vector loads when the whole tile is in range and aligned.
template<typename T, int VT>
__device__ __forceinline__ void load_thread(const T* src, int valid_here, bool vec, T (&x)[VT],
  T fill) {
  if(vec) {
    constexpr int per = 16 / sizeof(T);
    static_assert(VT % per == 0, "vector width");
#pragma unroll
    for(int q = 0; q < VT / per; ++q) {
      uint4 w = reinterpret_cast<const uint4*>(src)[q];
      memcpy(&x[q * per], &w, 16);
    }
  } else {
#pragma unroll
    for(int i = 0; i < VT; ++i) x[i] = i < valid_here ? src[i] : fill;
  }
}

template<typename T, int VT>
__device__ __forceinline__ void store_thread(T* dst, int valid_here, bool vec, const T (&x)[VT]) {
  if(vec) {
    constexpr int per = 16 / sizeof(T);
#pragma unroll
    for(int q = 0; q < VT / per; ++q) {
      uint4 w;
      memcpy(&w, &x[q * per], 16);
      reinterpret_cast<uint4*>(dst)[q] = w;
    }
  } else {
#pragma unroll
    for(int i = 0; i < VT; ++i) if(i < valid_here) dst[i] = x[i];
  }
}

template<typename T, typename op_t, int NT, int VT, bool exclusive>
__global__ void __launch_bounds__(NT)
scan_kernel(const T* in, T* out, int64_t count, T init, op_t op, tile_status_t<T> st,
  uint32_t* tile_counter, T* reduction, int* error, int vec_ok) {
  constexpr int TILE = NT * VT;
  constexpr int NW = NT / 32;
  __shared__ T warp_tot[NW];
  __shared__ T s_prefix;
  __shared__ int64_t s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if(tid == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * TILE;
  const int valid = (int)min((int64_t)TILE, count - base);
  const bool vec = vec_ok && valid == TILE;
  const int valid_here = valid - tid * VT;

  T x[VT];
  load_thread<T, VT>(in + base + tid * VT, valid_here, vec, x, op_t::identity());
#pragma unroll
  for(int i = 1; i < VT; ++i) x[i] = op(x[i - 1], x[i]);

  T winc = warp_inclusive_scan(x[VT - 1], op);
  T wexc = __shfl_up_sync(0xffffffffu, winc, 1);
  if(lane == 31) warp_tot[warp] = winc;
  __syncthreads();
  if(warp == 0) {
    T t = lane < NW ? warp_tot[lane] : op_t::identity();
    t = warp_inclusive_scan(t, op);
    if(lane < NW) warp_tot[lane] = t;
  }
  __syncthreads();
  const T tile_agg = warp_tot[NW - 1];
  T thread_excl = lane ? wexc : op_t::identity();
  if(warp) thread_excl = op(warp_tot[warp - 1], thread_excl);

  if(warp == 0) {
    T prefix;
    if(tile == 0) {
      prefix = init;
      if(lane == 0) st.publish(0, status_inclusive, op(init, tile_agg));
    } else {
      if(lane == 0) st.publish(tile, status_aggregate, tile_agg);
      prefix = lookback_warp<T>(st, tile, op, error);
      if(lane == 0) st.publish(tile, status_inclusive, op(prefix, tile_agg));
    }
    if(lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  const T carry = op(s_prefix, thread_excl);
  if(exclusive) {
#pragma unroll
    for(int i = VT - 1; i > 0; --i) x[i] = op(carry, x[i - 1]);
    x[0] = carry;
  } else {
#pragma unroll
    for(int i = 0; i < VT; ++i) x[i] = op(carry, x[i]);
  }
  store_thread<T, VT>(out + base + tid * VT, valid_here, vec, x);
  if(reduction && tid == 0 && base + TILE >= count) *reduction = op(s_prefix, tile_agg);
}

template<typename T>
__global__ void store_value_kernel(T* p, T v) { *p = v; }

// Device-wide reduce in one launch: each CTA reduces a fixed, strided set of
// tiles into partials[cta]; the last CTA to finish (ticket counter) reduces
// the partials in index order.  Deterministic for a given grid size.
template<typename T, typename op_t, int NT, int VT>
__global__ void __launch_bounds__(NT)
reduce_kernel(const T* in, int64_t count, T init, op_t op, T* partials, uint32_t* counter,
  T* out, int vec_ok) {
  constexpr int TILE = NT * VT;
  constexpr int NW = NT / 32;
  __shared__ T warp_tot[NW];
  __shared__ bool s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t num_tiles = div_up(count, TILE);
  T acc = op_t::identity();
  for(int64_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
    const int64_t base = tile * TILE;
    const int valid = (int)min((int64_t)TILE, count - base);
    T x[VT];
    load_thread<T, VT>(in + base + tid * VT, valid - tid * VT, vec_ok && valid == TILE, x,
      op_t::identity());
#pragma unroll
    for(int i = 0; i < VT; ++i) acc = op(acc, x[i]);
  }
  auto block_reduce = [&](T v) -> T {
    v = warp_reduce(v, op);
    if(lane == 0) warp_tot[warp] = v;
    __syncthreads();
    T r = op_t::identity();
    if(warp == 0) {
      r = lane < NW ? warp_tot[lane] : op_t::identity();
      r = warp_reduce(r, op);
    }
    __syncthreads();
    return r;
  };
  T total = block_reduce(acc);
  if(tid == 0) {
    partials[blockIdx.x] = total;
    __threadfence();
    s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if(s_last) {
    __threadfence();
    T v = op_t::identity();
    for(int i = tid; i < (int)gridDim.x; i += NT) v = op(v, __ldcg(partials + i));
    T r = block_reduce(v);
    if(tid == 0) *out = op(init, r);
  }
}

}  // namespace device
}  // namespace mgpu
