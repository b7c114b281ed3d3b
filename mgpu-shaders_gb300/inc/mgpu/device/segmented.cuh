// Batched segmented sort and segmented scan for sm_103a.
//
// No reference counterpart: the reference sorts one array per call
// (vk/radix.hxx:195-470), so many small arrays cost a launch sequence each.
// Here all segments of a CSR layout (offsets[s] .. offsets[s+1]) are sorted
// by one fixed launch sequence, whatever their number:
//
//  1. seg_classify: one pass over the offsets puts each segment in a size
//     class: <= 32 keys (one warp, rank sort in registers), <= 32*items keys
//     (one warp, merge sort in a shared-memory slice), <= one tile (one CTA,
//     merge sort in shared memory), larger (multi-CTA onesweep).  Large
//     segments get contiguous tile ranges and zeroed histogram rows.
//  2. seg_small_sort: one persistent launch; CTAs pull CTA-class segments,
//     then warps pull warp-class segments, from atomic queues.
//  3. seg_histogram + per-digit onesweep passes over all large segments'
//     tiles together; each tile looks back only within its own segment.
//
// Sort order within a segment is the radix_sort order (radix_permute_t bits),
// stable; values follow their keys.
#pragma once

#include "common.cuh"
#include "merge.cuh"
#include "onesweep.cuh"
#include "scan.cuh"

namespace mgpu {
namespace device {

// Counters and work lists of one segmented sort (device memory).
struct seg_state_t {
  uint32_t* counters;        // see seg_counter_t
  int* warp_list;            // segments of 2..32 keys
  int* slice_list;           // segments of 33..slice keys
  int* cta_list;             // segments of slice+1..tile keys
  int* large_seg;            // segments above one tile
  int* large_tile_base;      // first global tile of each large segment
  int* tile_owner;           // large-segment index of each global tile
  uint32_t* seg_hist;        // [large][passes][256] digit totals
  uint32_t* lookback;        // [passes][max_tiles][256] look-back words
  int64_t max_tiles;         // bound on the large segments' tiles
  int64_t max_large;         // bound on the number of large segments
};

// sc_bad: set when the offsets are not a non-decreasing sequence inside
// [0, count]; every later kernel of the sort then returns at once.
enum seg_counter_t {
  sc_warp = 0, sc_slice, sc_cta, sc_large, sc_tiles,
  sc_next_cta, sc_next_warp, sc_next_slice, sc_bad, sc_pass_tiles /* + pass */,
  sc_count = sc_pass_tiles + 8
};

// CTA_MAX: the largest segment one CTA sorts in shared memory; larger
// segments are cut into onesweep tiles of LARGE_TILE keys.  Offsets outside
// [0, count] or decreasing would make segments overlap or leave the keys:
// the sort is then not done (sc_bad) and the context's error word reports
// MGPU_ERR_INVALID_ARG.  With offsets[s] <= offsets[s + 1] for every s and
// both ends inside [0, count], the segments tile [offsets[0], offsets[n]).
template<int CTA_MAX, int LARGE_TILE, int SLICE, int PASSES>
__global__ void seg_classify(const int64_t* offsets, int64_t num_segments, int64_t count,
  seg_state_t s, int* error) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < num_segments; i += stride) {
    int64_t b = offsets[i], e = offsets[i + 1];
    if(b < 0 || e < b || e > count) {
      atomicOr(&s.counters[sc_bad], 1u);
      raise_error(error, err_invalid_arg);
      continue;
    }
    int64_t n = e - b;
    if(n <= 1) continue;
    if(n <= 32) {
      s.warp_list[atomicAdd(&s.counters[sc_warp], 1u)] = (int)i;
    } else if(n <= SLICE) {
      s.slice_list[atomicAdd(&s.counters[sc_slice], 1u)] = (int)i;
    } else if(n <= CTA_MAX) {
      s.cta_list[atomicAdd(&s.counters[sc_cta], 1u)] = (int)i;
    } else {
      const int tiles = (int)div_up(n, LARGE_TILE);
      const uint32_t lu = atomicAdd(&s.counters[sc_large], 1u);
      const uint32_t tbu = atomicAdd(&s.counters[sc_tiles], (uint32_t)tiles);
      // Non-overlapping segments inside [0, count] stay within the bounds the
      // host sized the lists for; only offsets that fail the check above (in
      // another segment) can get here past them.
      if((int64_t)lu >= s.max_large || (int64_t)tbu + tiles > s.max_tiles) {
        atomicOr(&s.counters[sc_bad], 1u);
        raise_error(error, err_invalid_arg);
        continue;
      }
      const int l = (int)lu, tb = (int)tbu;
      s.large_seg[l] = (int)i;
      s.large_tile_base[l] = tb;
      for(int t = 0; t < tiles; ++t) s.tile_owner[tb + t] = l;
      uint4* h = (uint4*)(s.seg_hist + (int64_t)l * PASSES * radix_bins);
      for(int j = 0; j < PASSES * radix_bins / 4; ++j) h[j] = make_uint4(0, 0, 0, 0);
    }
  }
}

// Stable rank sort of one segment of at most 32 keys by one warp: each lane
// holds one key; rank = keys below + equal keys in lower lanes.
template<typename K, typename V>
__device__ __forceinline__ void warp_rank_sort(K* keys, V* vals, int n) {
  typedef typename radix_key<K>::bits_t U;
  constexpr bool HAS_V = !std::is_same<V, no_values>::value;
  const int lane = threadIdx.x & 31;
  U u = ~(U)0;
  K key{};
  V val{};
  if(lane < n) {
    key = keys[lane];
    u = radix_key<K>::to_bits(key);
    if constexpr(HAS_V) val = vals[lane];
  }
  int rank = 0;
#pragma unroll
  for(int j = 0; j < 32; ++j) {
    U o = __shfl_sync(0xffffffffu, u, j);
    rank += (o < u) || (o == u && j < lane);
  }
  __syncwarp();
  if(lane < n) {
    keys[rank] = key;
    if constexpr(HAS_V) vals[rank] = val;
  }
}

// Stable merge sort of n <= 32 * W * VT keys (radix bits) and values held in
// shared memory, by a group of W warps (gtid: the thread's index in the
// group).  Each thread sorts VT consecutive items in registers by odd-even
// transposition (only adjacent, strictly descending pairs swap, so equal keys
// keep their order; positions past n hold all-ones bits, which never move
// before a real key), then merge passes through shared memory double the
// sorted runs until one run covers n (merge path with A first on ties).  The
// result is the stable order by radix bits, the order of the LSD radix sort.
// About 2 + 3 log2(n / VT) instructions per key against the radix sort's four
// full passes: the choice for segments of a few thousand keys.
template<int W, int VT, typename U, typename V>
__device__ __forceinline__ void group_merge_sort(U* sk, V* sv, int n, int gtid) {
  constexpr bool HAS_V = !std::is_same<V, no_values>::value;
  constexpr int G = 32 * W;
  typedef typename std::conditional<HAS_V, V, char>::type VR;
  auto gsync = [] { if(W == 1) __syncwarp(); else __syncthreads(); };
  const int first = VT * gtid;
  U k[VT];
  VR v[VT];
#pragma unroll
  for(int i = 0; i < VT; ++i) {
    const int j = first + i;
    k[i] = j < n ? sk[j] : ~(U)0;
    if constexpr(HAS_V) v[i] = j < n ? sv[j] : V();
  }
#pragma unroll
  for(int I = 0; I < VT; ++I) {
#pragma unroll
    for(int i = 1 & I; i < VT - 1; i += 2) {
      if(k[i + 1] < k[i]) {
        const U t = k[i]; k[i] = k[i + 1]; k[i + 1] = t;
        if constexpr(HAS_V) { const VR u = v[i]; v[i] = v[i + 1]; v[i + 1] = u; }
      }
    }
  }
#pragma unroll 1
  for(int coop = 2; coop <= G && VT * (coop >> 1) < n; coop <<= 1) {
    gsync();                           // readers of the previous pass are done
#pragma unroll
    for(int i = 0; i < VT; ++i) {
      if(first + i < n) {
        sk[first + i] = k[i];
        if constexpr(HAS_V) sv[first + i] = v[i];
      }
    }
    gsync();
    if(first < n) {
      const int start = VT * (gtid & ~(coop - 1));
      const int half = VT * (coop >> 1);
      const int a_begin = start, a_end = min(start + half, n);
      const int b_begin = a_end, b_end = min(start + 2 * half, n);
      const int a_cnt = a_end - a_begin, b_cnt = b_end - b_begin;
      const int diag = min(first - start, a_cnt + b_cnt);
      const U* A = sk + a_begin;
      const U* B = sk + b_begin;
      int ai = merge_path(A, a_cnt, B, b_cnt, diag, less_t<U>());
      int bi = diag - ai;
      U ak = A[min(ai, max(a_cnt - 1, 0))];
      U bk = B[min(bi, max(b_cnt - 1, 0))];
#pragma unroll
      for(int i = 0; i < VT; ++i) {
        const bool take_a = bi >= b_cnt || (ai < a_cnt && !(bk < ak));
        k[i] = take_a ? ak : bk;
        if constexpr(HAS_V) v[i] = sv[take_a ? a_begin + ai : b_begin + bi];
        if(take_a) { ++ai; ak = A[min(ai, max(a_cnt - 1, 0))]; }
        else { ++bi; bk = B[min(bi, max(b_cnt - 1, 0))]; }
      }
    }
  }
  gsync();
#pragma unroll
  for(int i = 0; i < VT; ++i) {
    if(first + i < n) {
      sk[first + i] = k[i];
      if constexpr(HAS_V) sv[first + i] = v[i];
    }
  }
  gsync();
}

// group_merge_sort with the fewest items per thread, among 3, 7, 13 and
// ITEMS, whose W warps cover n.  The register sort and every merge step cost
// in proportion to the items per thread, while a segment's lanes all run
// the same steps: a 200-key segment sorted by one warp at 21 items per thread
// keeps 10 lanes busy for 4 merge passes of 21 steps each; at 7 items per
// thread 29 lanes take 5 passes of 7 steps.
template<int W, int ITEMS, typename U, typename V>
__device__ __forceinline__ void group_merge_sort_fit(U* sk, V* sv, int n, int gtid) {
  constexpr int G = 32 * W;
  if(ITEMS > 3 && n <= G * 3) group_merge_sort<W, 3>(sk, sv, n, gtid);
  else if(ITEMS > 7 && n <= G * 7) group_merge_sort<W, 7>(sk, sv, n, gtid);
  else if(ITEMS > 13 && n <= G * 13) group_merge_sort<W, 13>(sk, sv, n, gtid);
  else group_merge_sort<W, ITEMS>(sk, sv, n, gtid);
}

// Shared memory of the in-CTA sorts: the tile's keys (radix bits) and values,
// scan scratch and a work-item slot.
template<typename K, typename V, int NT, int ITEMS, int SLICE_ITEMS>
struct seg_small_layout {
  typedef typename radix_key<K>::bits_t U;
  static constexpr bool has_values = !std::is_same<V, no_values>::value;
  static constexpr int tile = NT * ITEMS;
  static constexpr int slice = 32 * SLICE_ITEMS;
  static constexpr int warps = NT / 32;
  static constexpr size_t keys_off = 0;
  static constexpr size_t vals_off = sizeof(U) * tile;
  static constexpr size_t tmp_off = vals_off + (has_values ? sizeof(V) * tile : 0);
  static constexpr size_t misc_off = tmp_off + sizeof(uint32_t) * 32;
  static constexpr size_t bytes = misc_off + 16;
  static_assert(warps * slice <= tile, "warp slices fit in the tile buffers");
};

// Copies the n keys (as radix bits) and values of one segment into shared
// memory, STRIDE threads, t = this thread's index.  Asynchronous element
// copies (cp.async) put every load of the segment in flight at once, so the
// segment costs one memory latency rather than one per row, and hold no
// registers.  Each thread waits for its own copies and converts its own
// keys; the caller's barrier publishes the result.
template<int STRIDE, typename K, typename V, typename U>
__device__ __forceinline__ void seg_stage_in(const K* keys, const V* vals, int n, U* ks, V* vs,
  int t) {
  constexpr bool HAS_V = !std::is_same<V, no_values>::value;
  constexpr bool async_v = HAS_V && (sizeof(V) == 4 || sizeof(V) == 8 || sizeof(V) == 16);
  for(int i = t; i < n; i += STRIDE) {
    cp_async_elem(ks + i, (const U*)keys + i);
    if constexpr(async_v) cp_async_elem(vs + i, vals + i);
    else if constexpr(HAS_V) vs[i] = vals[i];
  }
  cp_async_wait_all();
  if constexpr(!(std::is_integral<K>::value && std::is_unsigned<K>::value)) {
    for(int i = t; i < n; i += STRIDE) {
      K key;
      memcpy(&key, &ks[i], sizeof(K));
      ks[i] = radix_key<K>::to_bits(key);
    }
  }
}

// Whole sort of at most one tile of keys in one CTA (the single-CTA branch
// of vk::radix_sort, vk/radix.hxx:221-282, with all bits of the key): a
// stable merge sort by radix bits in shared memory, whose result is the LSD
// radix sort's (for one CTA it takes about a quarter of the latency of four
// in-shared-memory radix passes).
template<typename K, typename V, int NT, int ITEMS>
__global__ void __launch_bounds__(NT)
radix_sort_cta(K* keys, V* vals, int n) {
  typedef seg_small_layout<K, V, NT, ITEMS, ITEMS> L;
  typedef typename L::U U;
  constexpr bool HAS_V = L::has_values;
  extern __shared__ __align__(16) unsigned char smem[];
  U* ks = (U*)(smem + L::keys_off);
  V* vs = (V*)(smem + L::vals_off);
  const int tid = threadIdx.x;
  seg_stage_in<NT>(keys, vals, n, ks, vs, tid);
  __syncthreads();
  group_merge_sort_fit<NT / 32, ITEMS>(ks, vs, n, tid);
  for(int i = tid; i < n; i += NT) {
    keys[i] = radix_key<K>::from_bits(ks[i]);
    if constexpr(HAS_V) vals[i] = vs[i];
  }
}

// Persistent sort of every segment up to one tile: CTA-class segments first
// (whole CTA), then slice-class and warp-class segments (one warp each).
template<typename K, typename V, int NT, int ITEMS, int SLICE_ITEMS, int PASSES, int MINB = 1>
__global__ void __launch_bounds__(NT, MINB)
seg_small_sort(K* keys, V* vals, const int64_t* offsets, seg_state_t s) {
  typedef seg_small_layout<K, V, NT, ITEMS, SLICE_ITEMS> L;
  typedef typename L::U U;
  constexpr bool HAS_V = L::has_values;
  extern __shared__ __align__(16) unsigned char smem[];
  U* ks = (U*)(smem + L::keys_off);
  V* vs = (V*)(smem + L::vals_off);
  int* s_item = (int*)(smem + L::misc_off);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Bad offsets (sc_bad): no segment is sorted.
  const bool bad = s.counters[sc_bad] != 0;

  // CTA-class segments.
  const uint32_t num_cta = bad ? 0 : s.counters[sc_cta];
  while(true) {
    if(tid == 0) *s_item = (int)atomicAdd(&s.counters[sc_next_cta], 1u);
    __syncthreads();
    const int item = *s_item;
    __syncthreads();
    if((uint32_t)item >= num_cta) break;
    const int seg = s.cta_list[item];
    const int64_t b = offsets[seg];
    const int n = (int)(offsets[seg + 1] - b);
    seg_stage_in<NT>(keys + b, HAS_V ? vals + b : vals, n, ks, vs, tid);
    __syncthreads();
    group_merge_sort_fit<NT / 32, ITEMS>(ks, vs, n, tid);
    for(int i = tid; i < n; i += NT) {
      keys[b + i] = radix_key<K>::from_bits(ks[i]);
      if constexpr(HAS_V) vals[b + i] = vs[i];
    }
    __syncthreads();
  }

  // Slice-class segments: each warp sorts its own in a private slice.
  const uint32_t num_slice = bad ? 0 : s.counters[sc_slice];
  U* wks = ks + warp * L::slice;
  V* wvs = vs + warp * L::slice;
  while(true) {
    int item = 0;
    if(lane == 0) item = (int)atomicAdd(&s.counters[sc_next_slice], 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if((uint32_t)item >= num_slice) break;
    const int seg = s.slice_list[item];
    const int64_t b = offsets[seg];
    const int n = (int)(offsets[seg + 1] - b);
    seg_stage_in<32>(keys + b, HAS_V ? vals + b : vals, n, wks, wvs, lane);
    __syncwarp();
    group_merge_sort_fit<1, SLICE_ITEMS>(wks, wvs, n, lane);
    for(int i = lane; i < n; i += 32) {
      keys[b + i] = radix_key<K>::from_bits(wks[i]);
      if constexpr(HAS_V) vals[b + i] = wvs[i];
    }
    __syncwarp();
  }

  // Warp-class segments: rank sort in registers.
  const uint32_t num_warp = bad ? 0 : s.counters[sc_warp];
  while(true) {
    int item = 0;
    if(lane == 0) item = (int)atomicAdd(&s.counters[sc_next_warp], 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if((uint32_t)item >= num_warp) break;
    const int seg = s.warp_list[item];
    const int64_t b = offsets[seg];
    const int n = (int)(offsets[seg + 1] - b);
    warp_rank_sort<K, V>(keys + b, HAS_V ? vals + b : vals, n);
  }
}

// Digit totals of every large segment, all passes, one read of the keys.
// Each CTA walks a contiguous range of global tiles and flushes its shared
// histogram whenever the owning segment changes.  Also clears the look-back
// words of all used tiles.
template<typename K, int NT, int TILE, int PASSES>
__global__ void __launch_bounds__(NT)
seg_histogram(const K* keys, const int64_t* offsets, seg_state_t s) {
  typedef typename radix_key<K>::bits_t U;
  // One copy of the bins: eight copies spread over the lanes (bank = 8 x
  // (bin mod 4) + copy) measured slower (0.244 -> 0.271 ms on the 10^5-segment
  // batch), and so did a copy per lane in 128 KB with one 1024-thread CTA
  // per SM, the plain histogram's layout (0.243 -> 0.304 ms): their flushes
  // at every segment change and the extra shared traffic cost more than the
  // conflicts they remove.
  constexpr int COPIES = 1;
  constexpr int BINS = PASSES * radix_bins;
  __shared__ uint32_t sh[BINS * COPIES];
  const int tid = threadIdx.x;
  const int copy = 0;
  if(s.counters[sc_bad]) return;
  const int num_tiles = (int)s.counters[sc_tiles];
  const int per = (int)div_up(num_tiles, gridDim.x);
  const int t0 = blockIdx.x * per, t1 = min(num_tiles, t0 + per);
  // Clear this CTA's tiles' look-back rows (all passes).
  for(int p = 0; p < PASSES; ++p) {
    uint4* z = (uint4*)(s.lookback + ((int64_t)p * s.max_tiles + t0) * radix_bins);
    int64_t words = (int64_t)max(0, t1 - t0) * radix_bins / 4;
    for(int64_t i = tid; i < words; i += NT) z[i] = make_uint4(0, 0, 0, 0);
  }
  int cur = -1;
  auto flush = [&] {
    __syncthreads();
    if(cur >= 0) {
      uint32_t* g = s.seg_hist + (int64_t)cur * BINS;
      for(int i = tid; i < BINS; i += NT) {
        uint32_t sum = 0;
#pragma unroll
        for(int j = 0; j < COPIES; ++j) {
          const int c = (i + j) & (COPIES - 1);
          sum += sh[i * COPIES + c];
          sh[i * COPIES + c] = 0;
        }
        if(sum) atomicAdd(&g[i], sum);
      }
    } else {
      for(int i = tid; i < BINS * COPIES; i += NT) sh[i] = 0;
    }
    __syncthreads();
  };
  flush();
  // Loads of a tile are issued UNROLL at a time before their keys are
  // counted, so each thread has several in flight (one at a time left the
  // kernel waiting on memory latency).
  constexpr int UNROLL = 8;
  for(int t = t0; t < t1; ++t) {
    const int l = s.tile_owner[t];
    if(l != cur) { flush(); cur = l; }
    const int seg = s.large_seg[l];
    const int64_t sb = offsets[seg], se = offsets[seg + 1];
    const int64_t b = sb + (int64_t)(t - s.large_tile_base[l]) * TILE;
    const int n = (int)min((int64_t)TILE, se - b);
    for(int i0 = tid; i0 < n; i0 += NT * UNROLL) {
      U u[UNROLL];
#pragma unroll
      for(int k = 0; k < UNROLL; ++k)
        if(i0 + k * NT < n) u[k] = radix_key<K>::to_bits(keys[b + i0 + k * NT]);
#pragma unroll
      for(int k = 0; k < UNROLL; ++k) {
        if(i0 + k * NT < n) {
#pragma unroll
          for(int p = 0; p < PASSES; ++p)
            atomicAdd(&sh[(p * radix_bins + extract_digit(u[k], 8 * p, 8)) * COPIES + copy], 1u);
        }
      }
    }
  }
  flush();
}

// One digit pass over the tiles of all large segments.
template<typename K, typename V, int NT, int ITEMS, int MIN_BLOCKS, int PASSES>
__global__ void __launch_bounds__(NT, MIN_BLOCKS)
seg_onesweep_pass(onesweep_args<K, V> a, const int64_t* offsets, seg_state_t s, int pass) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int TILE = NT * ITEMS;
  if(s.counters[sc_bad] || blockIdx.x >= s.counters[sc_tiles]) return;
  const int tile = onesweep_begin<K, V, NT, ITEMS>(a.tile_counter, smem);
  const int l = s.tile_owner[tile];
  const int seg = s.large_seg[l];
  const int64_t sb = offsets[seg], se = offsets[seg + 1];
  const int local = tile - s.large_tile_base[l];
  onesweep_tile_t t;
  t.base = sb + (int64_t)local * TILE;
  t.valid = (int)min((int64_t)TILE, se - t.base);
  t.local = local;
  t.lb_row = s.lookback + ((int64_t)pass * s.max_tiles + tile) * radix_bins;
  t.hist = s.seg_hist + ((int64_t)l * PASSES + pass) * radix_bins;
  t.out_base = sb;
  onesweep_tile<K, V, NT, ITEMS, 4, true>(a, t, smem);
}

////////////////////////////////////////////////////////////////////////////////
// Segmented scan: a single-pass look-back scan over (head flag, value) pairs
// with the operator (fa, a) . (fb, b) = (fa | fb, fb ? b : a op b), which is
// associative, so one chained scan restarts at every segment head.  A tile's
// look-back also stops early at any predecessor whose aggregate contains a
// head, since nothing before it reaches this tile.  As for the plain scan,
// `op` must be associative and commutative (plus, min, max): a tile's
// aggregate folds its elements in thread order, not element order.

// Head bitmap of a segmented scan: bit e of words[e / 32] is set when a
// non-empty segment begins at element e (element 0 always begins one).  One
// thread per segment; `words` is zeroed before the launch.  (A template, so
// that every translation unit may include it.)
template<int NT = 256>
__global__ void seg_mark_heads(const int64_t* offsets, int64_t num_segments, int64_t count,
  uint32_t* words) {
  const int64_t sg = (int64_t)blockIdx.x * NT + threadIdx.x;
  if(sg == 0) atomicOr(&words[0], 1u);
  if(sg >= num_segments) return;
  const int64_t o = offsets[sg];
  if(o > 0 && o < count && offsets[sg + 1] > o)
    atomicOr(&words[o >> 5], 1u << (o & 31));
}

template<typename T>
struct seg_pair_t {
  T v;
  uint32_t f;
};

template<typename T, typename op_t>
__device__ __forceinline__ seg_pair_t<T> seg_combine(seg_pair_t<T> a, seg_pair_t<T> b, op_t op) {
  return { b.f ? b.v : op(a.v, b.v), a.f | b.f };
}

// Status of a tile.  4-byte values: one 64-bit word per tile, (status |
// head << 2) over the value bits, so one load returns a consistent pair.
// 8-byte values: a flag word (status | head << 2) and one value word per
// status ([2][tiles]: aggregate slot, inclusive slot), so a reader always
// loads the value that belongs to the flag it observed.  `flags` holds
// 8 bytes per tile (zeroed before the scan) in both cases.
template<typename T>
struct seg_status_t {
  uint32_t* flags;
  uint64_t* values;
  int64_t tiles;
  static constexpr bool packed = sizeof(T) <= 4;
  __device__ __forceinline__ void publish(int64_t tile, uint32_t status, seg_pair_t<T> p) const {
    if constexpr(packed) {
      uint32_t b = 0;
      memcpy(&b, &p.v, sizeof(T));
      st_relaxed((uint64_t*)flags + tile, ((uint64_t)(status | (p.f << 2)) << 32) | b);
    } else {
      uint64_t b = 0;
      memcpy(&b, &p.v, sizeof(T));
      st_relaxed(values + (status == status_inclusive ? tiles : 0) + tile, b);
      st_release(flags + tile, status | (p.f << 2));
    }
  }
  __device__ __forceinline__ uint32_t read(int64_t tile, seg_pair_t<T>& p) const {
    if constexpr(packed) {
      const uint64_t w = ld_relaxed((const uint64_t*)flags + tile);
      const uint32_t f = (uint32_t)(w >> 32), b = (uint32_t)w;
      if(f & 3) {
        memcpy(&p.v, &b, sizeof(T));
        p.f = (f >> 2) & 1;
      }
      return f & 3;
    } else {
      uint32_t w = ld_acquire(flags + tile);
      if(w & 3) {
        uint64_t b = ld_relaxed(values + ((w & 3) == status_inclusive ? tiles : 0) + tile);
        memcpy(&p.v, &b, sizeof(T));
        p.f = (w >> 2) & 1;
      }
      return w & 3;
    }
  }
};

// CTA-wide look-back over (head, value) pairs for seg_scan_defer_kernel: in
// each round warp w reads the 32 predecessors base - (32 w + lane).  The walk
// stops at an inclusive status or at a tile whose aggregate holds a head.
// Every thread returns the same pair.
template<int NW, typename T, typename op_t>
__device__ seg_pair_t<T> seg_lookback_cta(const seg_status_t<T>& st, int64_t tile, op_t op,
  int* error, T* s_v, uint32_t* s_f, int* s_info) {
  typedef seg_pair_t<T> P;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  P acc { op_t::identity(), 0u };
  bool have = false;
  int64_t base = tile - 1;
  for(int round = 0;; ++round) {
    const int64_t j = base - (warp * 32 + lane);
    P v { op_t::identity(), 0u };
    uint32_t f = status_inclusive;
    if(j >= 0) f = st.read(j, v);
    const bool stop_here = f == status_inclusive || (f != status_invalid && v.f);
    const uint32_t stop_mask = __ballot_sync(0xffffffffu, stop_here);
    const int limit = stop_mask ? __ffs(stop_mask) - 1 : 31;
    const bool missing = __any_sync(0xffffffffu, lane <= limit && f == status_invalid);
#pragma unroll
    for(int off = 1; off < 32; off <<= 1) {
      P y { __shfl_down_sync(0xffffffffu, v.v, off), __shfl_down_sync(0xffffffffu, v.f, off) };
      if(lane + off <= limit) v = seg_combine<T>(y, v, op);
    }
    if(lane == 0) {
      int info = (stop_mask ? 1 : 0) | (missing ? 2 : 0);
      if(warp == 0 && round &&
         (round >= spin_limit || (0 == (round & (spin_poll_error - 1)) && error_raised(error))))
        info |= 4;
      s_v[warp] = v.v;
      s_f[warp] = v.f;
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
    P r { op_t::identity(), 0u };
    if(!miss)
      for(int w = w_last; w >= 0; --w) r = seg_combine<T>(r, P { s_v[w], s_f[w] }, op);
    __syncthreads();
    if(miss) {
      __nanosleep(32);
      continue;
    }
    acc = have ? seg_combine<T>(r, acc, op) : r;
    have = true;
    if(found) return acc;
    base -= 32 * NW;
  }
}

// Segmented scan with the deferred look-back of scan_defer_kernel: resident
// CTAs loop over tiles; in one iteration a tile's values and its words of the
// head bitmap arrive by bulk copy and its (head, value) aggregate is
// published; in the next the CTA looks back, publishes the tile's inclusive
// pair, re-reads the values from L2 and writes the scanned tile.  Elements
// are held in the warp-striped layout of striped_t.  The bitmap holds one
// word per 32 elements, padded to whole tiles.
template<typename T, int NT, int VT>
struct seg_scan_defer_layout {
  static constexpr int head_words = NT * VT / 32;
  static constexpr size_t stage_bytes = sizeof(T) * NT * VT;
  static constexpr size_t heads_off = stage_bytes;
  static constexpr size_t bar_off = heads_off + sizeof(uint32_t) * head_words;
  static constexpr size_t bytes = bar_off + 16;
  static_assert(head_words % 4 == 0, "bulk-copy granularity");
};

template<typename T, typename op_t, int NT, int VT, bool exclusive, int MINB>
__global__ void __launch_bounds__(NT, MINB)
seg_scan_defer_kernel(const T* in, T* out, int64_t count, const uint32_t* head_bits,
  T init, op_t op, seg_status_t<T> st, uint32_t* tile_counter, int* error, int vec_ok) {
  typedef striped_t<T, VT> S;
  typedef seg_pair_t<T> P;
  typedef seg_scan_defer_layout<T, NT, VT> L;
  constexpr int PER = S::PER, ROWS = S::ROWS;
  constexpr int TILE = NT * VT;
  constexpr int NW = NT / 32;
  constexpr int HW = TILE / 32;
  constexpr uint32_t PER_MASK = (1u << PER) - 1;
  static_assert(NW >= 2, "the copy thread is outside warp 0");
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);
  __shared__ uint32_t heads[2][HW];
  __shared__ T wv[NW];
  __shared__ uint32_t wf[NW];
  __shared__ T s_v[NW];
  __shared__ uint32_t s_f[NW];
  __shared__ int s_info[NW];
  __shared__ int64_t s_id;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t num_tiles = div_up(count, TILE);
  const int64_t bulk_tiles = vec_ok ? count / TILE : 0;
  const int copy_tid = NT - 32;

  auto fetch = [&](int64_t id) {
    s_id = id;
    if(id < bulk_tiles) {
      mbar_arrive_expect_tx(bar, (uint32_t)(L::stage_bytes + sizeof(uint32_t) * HW));
      bulk_load(smem, in + id * TILE, (uint32_t)L::stage_bytes, bar);
      bulk_load(smem + L::heads_off, head_bits + id * HW, (uint32_t)(sizeof(uint32_t) * HW), bar);
    }
  };
  // Head bits of this thread's PER elements of row r.
  auto row_heads = [&](const uint32_t* h, int r) -> uint32_t {
    const int e = S::offset(warp, lane, r);
    return (h[e >> 5] >> (e & 31)) & PER_MASK;
  };
  if(tid == copy_tid) {
    mbar_init(bar, 1);
    fence_mbar_init();
    fetch(atomicAdd(tile_counter, 1u));
  }
  __syncthreads();

  int64_t prev = -1;
  int hb = 0;                                  // heads buffer of `cur`
  P prev_agg { op_t::identity(), 0u }, cur_agg { op_t::identity(), 0u };   // thread 0
  uint32_t parity = 0;
  while(true) {
    int64_t next_id = 0;
    if(tid == copy_tid) next_id = atomicAdd(tile_counter, 1u);
    const int64_t cur = s_id;
    const bool have_cur = cur < num_tiles;

    if(have_cur) {
      const int64_t base = cur * TILE;
      const int valid = (int)min((int64_t)TILE, count - base);
      T x[VT];
      const uint32_t* hs = head_bits + cur * HW;
      if(cur < bulk_tiles) {
        mbar_wait_bounded(bar, parity, error);   // a timeout raised the error
        parity ^= 1;
        const T* sx = (const T*)smem;
#pragma unroll
        for(int r = 0; r < ROWS; ++r) {
          uint4 w = *reinterpret_cast<const uint4*>(sx + S::offset(warp, lane, r));
          memcpy(&x[r * PER], &w, 16);
        }
        hs = (const uint32_t*)(smem + L::heads_off);
      } else {
        S::load(in + base, valid, false, warp, lane, x, op_t::identity());
      }
      // Keep the tile's head words for its scan in the next iteration.
      for(int i = tid; i < HW; i += NT) heads[hb][i] = hs[i];
      // The warp's (head, value) pair: a head if its range holds one, and the
      // fold of its elements from its last head (or its first element) on.
      // The warp's range is words [warp * VT, warp * VT + VT) of the tile.
      const uint32_t hw = lane < VT ? hs[warp * VT + lane] : 0u;
      const int last = __reduce_max_sync(0xffffffffu, hw ? lane * 32 + 31 - __clz(hw) : -1);
      T a = op_t::identity();
#pragma unroll
      for(int r = 0; r < ROWS; ++r) {
        const int e = S::offset(warp, lane, r) - warp * 32 * VT;
#pragma unroll
        for(int j = 0; j < PER; ++j)
          if(e + j >= last) a = op(a, x[r * PER + j]);
      }
      a = warp_reduce(a, op);
      if(lane == 0) { wv[warp] = a; wf[warp] = last >= 0; }
    }
    __syncthreads();                           // stage consumed; warp totals visible
    if(tid == copy_tid) fetch(next_id);
    if(have_cur && tid == 0) {
      P agg { op_t::identity(), 0u };
#pragma unroll
      for(int w = 0; w < NW; ++w) agg = seg_combine<T>(agg, P { wv[w], wf[w] }, op);
      st.publish(cur, cur == 0 ? status_inclusive : status_aggregate, agg);
      cur_agg = agg;
    }

    if(prev >= 0) {
      const int64_t base = prev * TILE;
      const int valid = (int)min((int64_t)TILE, count - base);
      const bool vec = vec_ok && valid == TILE;
      const uint32_t* h = heads[hb ^ 1];
      T x[VT];
      S::load(in + base, valid, vec, warp, lane, x, op_t::identity());
      P prefix { op_t::identity(), 0u };
      if(prev > 0) {
        prefix = seg_lookback_cta<NW, T>(st, prev, op, error, s_v, s_f, s_info);
        if(tid == 0) st.publish(prev, status_inclusive, seg_combine<T>(prefix, prev_agg, op));
      } else {
        __syncthreads();
      }
      // Per row: the pair before this lane's first element, counted from the
      // start of the warp's range.
      // Each row is scanned with value-only shuffles: the lanes' head bits
      // (one ballot) give every lane the first lane of its segment in the
      // row, and a lane combines only partial results from that lane on.
      P before[ROWS];
      P acc { op_t::identity(), 0u };
      const uint32_t lt = lanemask_lt();
#pragma unroll
      for(int r = 0; r < ROWS; ++r) {
        const uint32_t hr = row_heads(h, r);
        T inc = op_t::identity();              // this lane's elements after its last head
#pragma unroll
        for(int j = 0; j < PER; ++j)
          inc = ((hr >> j) & 1u) ? x[r * PER + j] : op(inc, x[r * PER + j]);
        const uint32_t mask = __ballot_sync(0xffffffffu, hr != 0);
        const uint32_t upto = mask & (lt | (1u << lane));
        const int start = upto ? 31 - __clz(upto) : -1;   // segment's first lane in the row
#pragma unroll
        for(int off = 1; off < 32; off <<= 1) {
          const T y = __shfl_up_sync(0xffffffffu, inc, off);
          if(lane - off >= max(start, 0)) inc = op(y, inc);
        }
        T exv = __shfl_up_sync(0xffffffffu, inc, 1);
        if(lane == 0) exv = op_t::identity();
        before[r] = seg_combine<T>(acc, P { exv, (mask & lt) ? 1u : 0u }, op);
        acc = seg_combine<T>(acc, P { __shfl_sync(0xffffffffu, inc, 31), mask ? 1u : 0u }, op);
      }
      if(lane == 0) { wv[warp] = acc.v; wf[warp] = acc.f; }
      __syncthreads();
      P carry = prefix;
#pragma unroll
      for(int w = 0; w < NW; ++w)
        if(w < warp) carry = seg_combine<T>(carry, P { wv[w], wf[w] }, op);
#pragma unroll
      for(int r = 0; r < ROWS; ++r) {
        const uint32_t hr = row_heads(h, r);
        P run = seg_combine<T>(carry, before[r], op);
#pragma unroll
        for(int j = 0; j < PER; ++j) {
          const uint32_t hd = (hr >> j) & 1u;
          const T xv = x[r * PER + j];
          if(exclusive) x[r * PER + j] = hd ? init : op(init, run.v);
          run = seg_combine<T>(run, P { xv, hd }, op);
          if(!exclusive) x[r * PER + j] = op(init, run.v);
        }
      }
      S::store(out + base, valid, vec, warp, lane, x);
    }
    __syncthreads();
    if(!have_cur) break;
    prev = cur;
    prev_agg = cur_agg;
    hb ^= 1;
  }
}

}  // namespace device
}  // namespace mgpu
