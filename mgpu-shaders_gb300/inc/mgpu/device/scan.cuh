// Single-pass scan (decoupled look-back) and single-launch reduce for sm_103a.
//
// Reference behaviour: vk::scan (vk/scan.hxx:10-115) is an in-place
// exclusive scan built from cta_scan_t (common/cta_scan.hxx:80-175) as either
// one CTA looping over <= 8 tiles or an upsweep reduce / recursive scan of the
// partials / downsweep with carry-in: three launches per recursion level and
// 12 bytes of traffic per 4-byte element.  Here one launch reads each element
// once and writes it once (8 B/elem) with a decoupled look-back over tiles
// whose ids come from an atomic counter (scan_defer_kernel: resident CTAs
// that publish a tile's aggregate in one iteration and look back, scan and
// store it in the next; scan_kernel: one tile per CTA, used where a
// persistent grid is not wanted).
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
// already include `init` through tile 0's inclusive value).  One window of
// 32 * K predecessors is read per round trip to L2: lane l reads tiles
// base - (l * K + q), q = 0..K-1, nearest first.  The window's statuses up to
// the nearest inclusive one are combined; if any of those is not yet
// published, the window is read again.  Tiles arrive every few nanoseconds,
// so a window must reach back past every tile still in its own look-back
// (their number is about the look-back latency over the tile interval) for
// the look-back to end in one round trip.
template<int K, typename T, typename op_t, typename status_t>
__device__ T lookback_warp(const status_t& st, int64_t tile, op_t op, int* error) {
  const int lane = threadIdx.x & 31;
  T acc = op_t::identity();
  bool have = false;
  int64_t base = tile - 1;
  int spins = 0;
  while(true) {
    T v[K];
    uint32_t f[K];
#pragma unroll
    for(int q = 0; q < K; ++q) {
      int64_t j = base - (lane * K + q);
      v[q] = op_t::identity();
      f[q] = status_inclusive;
      if(j >= 0) f[q] = st.read(j, v[q]);
    }
    int qinc = K;
#pragma unroll
    for(int q = K - 1; q >= 0; --q) if(f[q] == status_inclusive) qinc = q;
    const uint32_t inc_mask = __ballot_sync(0xffffffffu, qinc < K);
    const int limit = inc_mask ? __ffs(inc_mask) - 1 : 31;
    // Positions nearer than the first inclusive status (and that one) count.
    const int q_end = lane < limit ? K : (lane == limit ? (inc_mask ? qinc + 1 : K) : 0);
    bool missing = false;
#pragma unroll
    for(int q = 0; q < K; ++q) if(q < q_end && f[q] == status_invalid) missing = true;
    if(__any_sync(0xffffffffu, missing)) {
      if(++spins >= spin_limit ||
         (0 == (spins & (spin_poll_error - 1)) && error_raised(error))) {
        raise_error(error, err_lookback_timeout);
        return acc;
      }
      __nanosleep(32);
      continue;
    }
    // The lane's statuses, earlier tiles (larger q) as left operands.
    T lv = op_t::identity();
#pragma unroll
    for(int q = 0; q < K; ++q) if(q < q_end) lv = op(v[q], lv);
#pragma unroll
    for(int off = 1; off < 32; off <<= 1) {
      T y = __shfl_down_sync(0xffffffffu, lv, off);
      if(lane + off <= limit) lv = op(y, lv);
    }
    T r = __shfl_sync(0xffffffffu, lv, 0);
    acc = have ? op(r, acc) : r;
    have = true;
    if(inc_mask) return acc;
    base -= 32 * K;
  }
}

// All NW warps of a tile look back together: in each round warp w reads the
// 32 predecessors base - (32 w + lane), so one round trip to L2 covers 32 NW
// tiles.  (The chain of inclusive prefixes advances by about one window per
// round trip, which bounds tiles per second; a warp-wide window of 32 limits
// a 2^28-element scan of 8192-element tiles to about 50 tiles per
// microsecond, half of what the HBM bandwidth asks for.)  The warps' window
// values and flags meet in shared memory; every thread derives the same
// result, so the return value is uniform across the CTA.  Called by every
// thread of the CTA, with `s_val` / `s_info` of NW entries.
template<int NW, typename T, typename op_t, typename status_t>
__device__ T lookback_cta(const status_t& st, int64_t tile, op_t op, int* error, T* s_val,
  int* s_info) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T acc = op_t::identity();
  bool have = false;
  int64_t base = tile - 1;
  for(int round = 0;; ++round) {
    const int64_t j = base - (warp * 32 + lane);
    T v = op_t::identity();
    uint32_t f = status_inclusive;
    if(j >= 0) f = st.read(j, v);
    const uint32_t inc_mask = __ballot_sync(0xffffffffu, f == status_inclusive);
    const int limit = inc_mask ? __ffs(inc_mask) - 1 : 31;
    const bool missing = __any_sync(0xffffffffu, lane <= limit && f == status_invalid);
#pragma unroll
    for(int off = 1; off < 32; off <<= 1) {
      T y = __shfl_down_sync(0xffffffffu, v, off);
      if(lane + off <= limit) v = op(y, v);
    }
    if(lane == 0) {
      int info = (inc_mask ? 1 : 0) | (missing ? 2 : 0);
      // Give up (uniformly, through shared memory) after the spin limit or
      // when another CTA has raised the error.
      if(warp == 0 && round &&
         (round >= spin_limit || (0 == (round & (spin_poll_error - 1)) && error_raised(error))))
        info |= 4;
      s_val[warp] = v;
      s_info[warp] = info;
    }
    __syncthreads();
    if(s_info[0] & 4) {
      raise_error(error, err_lookback_timeout);
      return acc;
    }
    bool miss = false;
    int w_last = NW - 1, found = 0;
#pragma unroll
    for(int w = 0; w < NW; ++w) {
      const int info = s_info[w];
      if(!found && !miss) {
        if(info & 2) miss = true;
        else if(info & 1) { w_last = w; found = 1; }
      }
    }
    T r = op_t::identity();
    if(!miss) {
      for(int w = w_last; w >= 0; --w) r = op(r, s_val[w]);
    }
    __syncthreads();                       // s_val / s_info are rewritten next round
    if(miss) {
      __nanosleep(32);
      continue;
    }
    acc = have ? op(r, acc) : r;
    have = true;
    if(found) return acc;
    base -= 32 * NW;
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

// Warp-striped vector layout of a tile: warp w owns elements
// [w * 32 * VT, (w + 1) * 32 * VT) of the tile; in row r of that range lane l
// holds the PER = 16 / sizeof(T) consecutive elements starting at
// (r * 32 + l) * PER, so each warp load or store instruction moves 512
// contiguous bytes.  `valid` elements of the tile exist; the rest read as
// `fill`.
template<typename T, int VT>
struct striped_t {
  static constexpr int PER = 16 / (int)sizeof(T);
  static constexpr int ROWS = VT / PER;
  static_assert(VT % PER == 0, "elements per thread must fill 16-byte vectors");
  static __device__ __forceinline__ int offset(int warp, int lane, int r) {
    return warp * 32 * VT + (r * 32 + lane) * PER;
  }
  static __device__ __forceinline__ void load(const T* tile, int valid, bool vec, int warp,
    int lane, T (&x)[VT], T fill) {
    if(vec) {
      uint4 w[ROWS];
#pragma unroll
      for(int r = 0; r < ROWS; ++r)
        w[r] = __ldcs(reinterpret_cast<const uint4*>(tile + offset(warp, lane, r)));
#pragma unroll
      for(int r = 0; r < ROWS; ++r) memcpy(&x[r * PER], &w[r], 16);
    } else {
#pragma unroll
      for(int r = 0; r < ROWS; ++r)
#pragma unroll
        for(int j = 0; j < PER; ++j) {
          int e = offset(warp, lane, r) + j;
          x[r * PER + j] = e < valid ? tile[e] : fill;
        }
    }
  }
  static __device__ __forceinline__ void store(T* tile, int valid, bool vec, int warp, int lane,
    const T (&x)[VT]) {
    if(vec) {
#pragma unroll
      for(int r = 0; r < ROWS; ++r) {
        uint4 w;
        memcpy(&w, &x[r * PER], 16);
        __stcs(reinterpret_cast<uint4*>(tile + offset(warp, lane, r)), w);
      }
    } else {
#pragma unroll
      for(int r = 0; r < ROWS; ++r)
#pragma unroll
        for(int j = 0; j < PER; ++j) {
          int e = offset(warp, lane, r) + j;
          if(e < valid) tile[e] = x[r * PER + j];
        }
    }
  }
};

// One tile per CTA (tile ids from an atomic counter, so every tile that is
// waited on belongs to a CTA that is already running).  The tile is loaded in
// the warp-striped layout and each warp scans its range in registers; warp 0
// scans the warp totals, publishes the tile aggregate and looks back; the
// carry-in is added and the tile stored with the same striped layout.
template<typename T, typename op_t, int NT, int VT, bool exclusive, int MINB = 1>
__global__ void __launch_bounds__(NT, MINB)
scan_kernel(const T* in, T* out, int64_t count, T init, op_t op, tile_status_t<T> st,
  uint32_t* tile_counter, T* reduction, int* error, int vec_ok) {
  typedef striped_t<T, VT> S;
  constexpr int PER = S::PER, ROWS = S::ROWS;
  constexpr int TILE = NT * VT;
  constexpr int NW = NT / 32;
  __shared__ T warp_tot[NW];
  __shared__ int64_t s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if(tid == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * TILE;
  const int valid = (int)min((int64_t)TILE, count - base);
  const bool vec = vec_ok && valid == TILE;

  T x[VT];
  S::load(in + base, valid, vec, warp, lane, x, op_t::identity());

  // Warp-local inclusive scan, row by row, in place: within each 16-byte
  // vector, then across the lanes' vector totals, then the carry of the
  // earlier rows.
  T acc = op_t::identity();
#pragma unroll
  for(int r = 0; r < ROWS; ++r) {
    T* xr = x + r * PER;
#pragma unroll
    for(int j = 1; j < PER; ++j) xr[j] = op(xr[j - 1], xr[j]);
    T linc = warp_inclusive_scan(xr[PER - 1], op);
    T lexc = __shfl_up_sync(0xffffffffu, linc, 1);
    if(lane == 0) lexc = op_t::identity();
    const T row_carry = op(acc, lexc);
#pragma unroll
    for(int j = 0; j < PER; ++j) xr[j] = op(row_carry, xr[j]);
    acc = op(acc, __shfl_sync(0xffffffffu, linc, 31));
  }
  if(lane == 0) warp_tot[warp] = acc;
  __syncthreads();
  if(warp == 0) {
    T t = lane < NW ? warp_tot[lane] : op_t::identity();
    T tinc = warp_inclusive_scan(t, op);
    const T tile_agg = __shfl_sync(0xffffffffu, tinc, NW - 1);
    T prefix;
    if(tile == 0) {
      prefix = init;
      if(lane == 0) st.publish(0, status_inclusive, op(init, tile_agg));
    } else {
      if(lane == 0) st.publish(tile, status_aggregate, tile_agg);
      prefix = lookback_warp<1, T>(st, tile, op, error);
      if(lane == 0) st.publish(tile, status_inclusive, op(prefix, tile_agg));
    }
    T texc = __shfl_up_sync(0xffffffffu, tinc, 1);
    if(lane < NW) warp_tot[lane] = lane ? op(prefix, texc) : prefix;
    if(lane == 0 && reduction && base + TILE >= count) *reduction = op(prefix, tile_agg);
  }
  __syncthreads();
  const T carry = warp_tot[warp];
#pragma unroll
  for(int i = 0; i < VT; ++i) x[i] = op(carry, x[i]);
  if(exclusive) {
    // Each item takes its predecessor's inclusive value (rows from the last
    // down; the warp's first item takes the warp's carry), as in the
    // deferred scan.
#pragma unroll
    for(int r = ROWS - 1; r >= 0; --r) {
      T* xr = x + r * PER;
      T before = __shfl_up_sync(0xffffffffu, xr[PER - 1], 1);
      const T row_before = r > 0 ? __shfl_sync(0xffffffffu, x[r * PER - 1], 31) : carry;
      if(lane == 0) before = row_before;
#pragma unroll
      for(int j = PER - 1; j > 0; --j) xr[j] = xr[j - 1];
      xr[0] = before;
    }
  }
  S::store(out + base, valid, vec, warp, lane, x);
}

// Persistent scan with a deferred look-back (the large-input path).
//
// A CTA that holds its tile in registers while it looks back keeps an SM slot
// busy for the whole look-back, and look-backs over tens of microseconds of
// tiles take several microseconds, so a one-tile-per-CTA scan reaches only
// about half of the HBM bandwidth.  Here each resident CTA loops over tiles
// (ids from the atomic counter) and splits every tile's work over two
// iterations:
//   iteration k:   tile `cur` arrives in shared memory through one bulk copy
//                  issued an iteration earlier; the CTA reduces it and
//                  publishes its aggregate, then starts the copy of the next
//                  tile into the freed stage;
//   iteration k+1: the CTA re-reads tile `cur` from global memory (it is
//                  still in L2), looks back (its predecessors have had an
//                  iteration to publish), publishes its inclusive prefix at
//                  once, scans it and stores it.
// So a tile's data is held only in L2 while its predecessors finish, and the
// DRAM traffic stays one read and one write per element.  Ids increase in the
// order a CTA processes them, so every tile a look-back waits on belongs to a
// running CTA whose earlier tiles need nothing later: the scan always
// progresses.  Ragged or unaligned tiles are read element by element instead
// of by bulk copy.
template<typename T, int NT, int VT>
struct scan_defer_layout {
  static constexpr size_t stage_bytes = sizeof(T) * NT * VT;
  static constexpr size_t bar_off = stage_bytes;
  static constexpr size_t bytes = bar_off + 16;
};

template<typename T, typename op_t, int NT, int VT, bool exclusive, int MINB>
__global__ void __launch_bounds__(NT, MINB)
scan_defer_kernel(const T* in, T* out, int64_t count, T init, op_t op, tile_status_t<T> st,
  uint32_t* tile_counter, T* reduction, int* error, int vec_ok) {
  typedef striped_t<T, VT> S;
  typedef scan_defer_layout<T, NT, VT> L;
  constexpr int PER = S::PER, ROWS = S::ROWS;
  constexpr int TILE = NT * VT;
  constexpr int NW = NT / 32;
  static_assert(NW >= 2, "the copy thread is outside warp 0");
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);
  __shared__ T warp_tot[NW];
  __shared__ T s_val[NW];
  __shared__ int s_info[NW];
  __shared__ int64_t s_id;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t num_tiles = div_up(count, TILE);
  const int64_t bulk_tiles = vec_ok ? count / TILE : 0;    // whole, aligned tiles
  const int copy_tid = NT - 32;                            // lane 0 of the last warp

  // Records the id of the next tile and starts its copy (copy thread only).
  auto fetch = [&](int64_t id) {
    s_id = id;
    if(id < bulk_tiles) {
      mbar_arrive_expect_tx(bar, (uint32_t)L::stage_bytes);
      bulk_load(smem, in + id * TILE, (uint32_t)L::stage_bytes, bar);
    }
  };
  if(tid == copy_tid) {
    mbar_init(bar, 1);
    fence_mbar_init();
    fetch(atomicAdd(tile_counter, 1u));
  }
  __syncthreads();

  int64_t prev = -1;
  T prev_agg = op_t::identity(), cur_agg = op_t::identity();   // used by thread 0
  uint32_t parity = 0;
  while(true) {
    // The id after `cur`; its atomic overlaps this iteration's work.
    int64_t next_id = 0;
    if(tid == copy_tid) next_id = atomicAdd(tile_counter, 1u);
    const int64_t cur = s_id;
    const bool have_cur = cur < num_tiles;

    // Reduce `cur`.
    if(have_cur) {
      T a = op_t::identity();
      if(cur < bulk_tiles) {
        mbar_wait_bounded(bar, parity, error);   // a timeout raised the error
        parity ^= 1;
        const T* sx = (const T*)smem;
#pragma unroll
        for(int r = 0; r < ROWS; ++r) {
          uint4 w = *reinterpret_cast<const uint4*>(sx + S::offset(warp, lane, r));
          T e[PER];
          memcpy(e, &w, 16);
#pragma unroll
          for(int j = 0; j < PER; ++j) a = op(a, e[j]);
        }
      } else {
        T x[VT];
        const int64_t base = cur * TILE;
        S::load(in + base, (int)min((int64_t)TILE, count - base), false, warp, lane, x,
          op_t::identity());
#pragma unroll
        for(int i = 0; i < VT; ++i) a = op(a, x[i]);
      }
      a = warp_reduce(a, op);
      if(lane == 0) warp_tot[warp] = a;
    }
    __syncthreads();                     // the stage is consumed; warp totals visible
    if(tid == copy_tid) fetch(next_id);
    if(have_cur && tid == 0) {
      T agg = op_t::identity();
#pragma unroll
      for(int w = 0; w < NW; ++w) agg = op(agg, warp_tot[w]);
      if(cur == 0) st.publish(0, status_inclusive, op(init, agg));
      else st.publish(cur, status_aggregate, agg);
      cur_agg = agg;
    }

    // Scan and store `prev`.
    if(prev >= 0) {
      const int64_t base = prev * TILE;
      const int valid = (int)min((int64_t)TILE, count - base);
      const bool vec = vec_ok && valid == TILE;
      T y[VT];
      S::load(in + base, valid, vec, warp, lane, y, op_t::identity());
      T prefix = init;
      if(prev > 0) {
        prefix = lookback_cta<NW, T>(st, prev, op, error, s_val, s_info);
        // Publish at once: successors need not wait for the scan below.
        if(tid == 0) st.publish(prev, status_inclusive, op(prefix, prev_agg));
      } else {
        __syncthreads();
      }
      T acc = op_t::identity();
#pragma unroll
      for(int r = 0; r < ROWS; ++r) {
        // In place: the row's items become their running fold, then (after
        // the warp scan) are offset by the row carry.
        T* yr = y + r * PER;
#pragma unroll
        for(int j = 1; j < PER; ++j) yr[j] = op(yr[j - 1], yr[j]);
        T linc = warp_inclusive_scan(yr[PER - 1], op);
        T lexc = __shfl_up_sync(0xffffffffu, linc, 1);
        if(lane == 0) lexc = op_t::identity();
        T row_carry = op(acc, lexc);
#pragma unroll
        for(int j = 0; j < PER; ++j) yr[j] = op(row_carry, yr[j]);
        acc = op(acc, __shfl_sync(0xffffffffu, linc, 31));
      }
      if(lane == 0) warp_tot[warp] = acc;
      __syncthreads();
      T wexc = prefix, ptot = op_t::identity();
#pragma unroll
      for(int w = 0; w < NW; ++w) {
        const T t = warp_tot[w];
        if(w < warp) wexc = op(wexc, t);
        ptot = op(ptot, t);
      }
      if(tid == 0 && reduction && base + TILE >= count) *reduction = op(prefix, ptot);
#pragma unroll
      for(int i = 0; i < VT; ++i) y[i] = op(wexc, y[i]);
      if(exclusive) {
        // Inclusive -> exclusive: each item takes its predecessor's value,
        // rows from the last down, so the value a row's lane 0 needs (lane
        // 31's last item of the row before) is still the inclusive one; the
        // warp's first item takes the warp's exclusive prefix.  (Shifting
        // inside the row loop instead kept more values live and spilled.)
#pragma unroll
        for(int r = ROWS - 1; r >= 0; --r) {
          T* yr = y + r * PER;
          T before = __shfl_up_sync(0xffffffffu, yr[PER - 1], 1);
          const T row_before = r > 0 ? __shfl_sync(0xffffffffu, y[r * PER - 1], 31) : wexc;
          if(lane == 0) before = row_before;
#pragma unroll
          for(int j = PER - 1; j > 0; --j) yr[j] = yr[j - 1];
          yr[0] = before;
        }
      }
      S::store(out + base, valid, vec, warp, lane, y);
    }
    __syncthreads();
    if(!have_cur) break;
    prev = cur;
    prev_agg = cur_agg;
  }
  // The stage holds no copy in flight here: ids only grow, so once `cur` is
  // past the end the fetched id is too, and no copy was issued for it.
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
    striped_t<T, VT>::load(in + base, valid, vec_ok && valid == TILE, warp, lane, x,
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
