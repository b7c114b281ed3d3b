// Merge-path merge and mergesort for sm_103a.
//
// Reference behaviour (seanbaxter/mgpu-shaders):
//  * merge_path (common/cta_merge.hxx:10-31): binary search on the cross
//    diagonal; bounds_lower takes A on ties (pred = !comp(b, a)).
//  * serial_merge (:107-133) merges vt items per thread from shared memory
//    with range checks (merge_predicate, :41-50).
//  * kernel_merge (common/kernel_merge.hxx:9-58) merges one nt*vt output
//    tile per CTA between partitions found by a separate partition launch
//    (vk/partition.hxx:9-20).
//  * kernel_blocksort / cta_sort_t (common/kernel_mergesort.hxx:12-67,
//    common/cta_mergesort.hxx:70-134): odd-even transposition sort of vt
//    registers (stable: swaps on strict comp only), then log2(nt) shared-
//    memory merge passes.
//  * mergesort passes (vk/mergesort.hxx:61-82): partition + merge of pairs
//    of sorted runs, ping-ponging so the result lands in place.
//
// GB300 design: every merge tile stages its A and B ranges (keys and values)
// into shared memory with TMA bulk copies (cp.async.bulk, no multicast),
// covering each range's 16-byte-aligned window and fetching only a ragged
// tail past the last whole 16 bytes of an array with plain loads.  Values are
// gathered from shared memory (not from global memory as the reference does),
// and outputs leave through shared memory as 16-byte vector stores.
#pragma once

#include "common.cuh"
#include "onesweep.cuh"   // no_values
#include <type_traits>

namespace mgpu {
namespace device {

template<typename T> struct less_t {
  __device__ __forceinline__ bool operator()(const T& a, const T& b) const { return a < b; }
};
template<typename T> struct greater_t {
  __device__ __forceinline__ bool operator()(const T& a, const T& b) const { return b < a; }
};

// Lower-bound merge path: the number of A items among the first `diag`
// outputs of a stable merge.
template<typename K, typename comp_t, typename idx_t>
__device__ __forceinline__ idx_t merge_path(const K* a, idx_t a_count, const K* b, idx_t b_count,
  idx_t diag, comp_t comp) {
  idx_t begin = diag > b_count ? diag - b_count : 0;
  idx_t end = diag < a_count ? diag : a_count;
  while(begin < end) {
    idx_t mid = (begin + end) >> 1;
    if(!comp(b[diag - 1 - mid], a[mid])) begin = mid + 1;
    else end = mid;
  }
  return begin;
}

// merge_path by a whole warp: each round the 32 lanes test the last position
// of 32 equal chunks of the candidate range and keep the first chunk whose
// test holds, so a range of n candidates takes about log32(n) rounds of
// independent loads instead of log2(n) dependent ones.  Every lane returns
// the result.
template<typename K, typename comp_t>
__device__ __forceinline__ int64_t merge_path_warp(const K* a, int64_t a_count, const K* b,
  int64_t b_count, int64_t diag, comp_t comp) {
  const int lane = threadIdx.x & 31;
  int64_t begin = diag > b_count ? diag - b_count : 0;
  int64_t end = diag < a_count ? diag : a_count;
  while(end - begin > 32) {
    // Chunk k is [begin + k step, begin + (k + 1) step) clipped to `end`;
    // its last position is tested.
    const int64_t step = (end - begin + 31) >> 5;
    const int64_t start = begin + lane * step;
    const int64_t probe = min(start + step, end) - 1;
    const bool hit = start < end && comp(b[diag - 1 - probe], a[probe]);
    const uint32_t mask = __ballot_sync(0xffffffffu, hit);
    if(!mask) return end;
    const int k = __ffs(mask) - 1;
    const int64_t lo = begin + k * step;
    end = min(end, lo + step);
    begin = lo;
  }
  const int64_t probe = begin + lane;
  const bool hit = probe < end && comp(b[diag - 1 - probe], a[probe]);
  const uint32_t mask = __ballot_sync(0xffffffffu, hit);
  return mask ? begin + __ffs(mask) - 1 : end;
}

// merge_path with either bound (the reference's merge_path<bounds>,
// common/cta_merge.hxx:10-31): UPPER = false is the lower bound above (A's
// item first on ties); UPPER = true takes B's item first on ties (predicate
// comp(a, b)).
template<bool UPPER, typename K, typename comp_t, typename idx_t>
__device__ __forceinline__ idx_t merge_path_bounds(const K* a, idx_t a_count, const K* b,
  idx_t b_count, idx_t diag, comp_t comp) {
  idx_t begin = diag > b_count ? diag - b_count : 0;
  idx_t end = diag < a_count ? diag : a_count;
  while(begin < end) {
    idx_t mid = (begin + end) >> 1;
    const K ak = a[mid], bk = b[diag - 1 - mid];
    const bool pred = UPPER ? comp(ak, bk) : !comp(bk, ak);
    if(pred) begin = mid + 1;
    else end = mid;
  }
  return begin;
}

// Partitions at every `spacing` outputs with a chosen bound, one thread each
// (vk::merge_path_partitions, vk/partition.hxx:9-20); mp_t: the caller's
// partition type (int in the reference).
template<bool UPPER, typename K, typename comp_t, typename mp_t>
__global__ void merge_path_partitions_kernel(const K* a, int64_t a_count, const K* b,
  int64_t b_count, int64_t spacing, int64_t num_partitions, mp_t* mp, comp_t comp) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= num_partitions) return;
  const int64_t diag = min(i * spacing, a_count + b_count);
  mp[i] = (mp_t)merge_path_bounds<UPPER>(a, a_count, b, b_count, diag, comp);
}

// Partitions of a two-array merge: mp[i] for diagonal min(i * spacing,
// total).  WARP: one warp per partition (few partitions: the search latency
// dominates); otherwise one thread per partition (many partitions: the
// kernel is bound by its loads).
template<typename K, typename comp_t, bool WARP>
__global__ void merge_partition_kernel(const K* a, int64_t a_count, const K* b, int64_t b_count,
  int64_t spacing, int64_t num_partitions, int64_t* mp, comp_t comp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = WARP ? t >> 5 : t;
  if(i >= num_partitions) return;
  const int64_t diag = min(i * spacing, a_count + b_count);
  if(WARP) {
    const int64_t r = merge_path_warp(a, a_count, b, b_count, diag, comp);
    if((threadIdx.x & 31) == 0) mp[i] = r;
  } else {
    mp[i] = merge_path(a, a_count, b, b_count, diag, comp);
  }
}

// Partitions of one mergesort pass over runs of `run` items: one per output
// tile start (WARP as for merge_partition_kernel).
template<typename K, typename comp_t, bool WARP>
__global__ void mergesort_partition_kernel(const K* keys, int64_t count, int64_t run,
  int64_t spacing, int64_t num_partitions, int64_t* mp, comp_t comp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = WARP ? t >> 5 : t;
  if(i >= num_partitions) return;
  const int64_t pos = min(i * spacing, count);
  const int64_t pair = pos / (2 * run);
  const int64_t a0 = pair * 2 * run;
  const int64_t a1 = min(a0 + run, count);
  const int64_t b1 = min(a0 + 2 * run, count);
  if(WARP) {
    const int64_t r = merge_path_warp(keys + a0, a1 - a0, keys + a1, b1 - a1, pos - a0, comp);
    if((threadIdx.x & 31) == 0) mp[i] = r;
  } else {
    mp[i] = merge_path(keys + a0, a1 - a0, keys + a1, b1 - a1, pos - a0, comp);
  }
}

// Partition counts up to this use the warp search (inside the mergesort pass
// kernel itself, so such passes need no partition launch).
constexpr int64_t warp_partition_limit = 8192;

// Shared-memory plan of one merge tile: keys and values of the A and B
// ranges, each placed so that its 16-byte-aligned global window starts on a
// 16-byte boundary.
template<typename K, typename V, int NT, int VT>
struct merge_tile_layout {
  static constexpr bool has_values = !std::is_same<V, no_values>::value;
  static constexpr int nv = NT * VT;
  static constexpr int kvec = 16 / sizeof(K);
  static constexpr int vvec = has_values ? 16 / sizeof(V) : 1;
  // A window and B window each round out to a vector on both sides.
  static constexpr int kcap = nv + 4 * kvec;
  static constexpr int vcap = nv + 4 * vvec;
  static constexpr size_t keys_off = 0;
  static constexpr size_t vals_off = (sizeof(K) * kcap + 15) / 16 * 16;
  static constexpr size_t bar_off = vals_off + (has_values ? (sizeof(V) * vcap + 15) / 16 * 16 : 0);
  static constexpr size_t bytes = bar_off + 16;
};

// One range [begin, end) of an array of `count` items staged at smem `dst`
// (16-byte aligned); returns the smem index of item `begin`.  Bytes issued as
// bulk copies are added to *tx.  Plain loads cover what bulk copies cannot.
template<typename T>
__device__ __forceinline__ int stage_range(T* dst, const T* src, int64_t begin, int64_t end,
  int64_t count, bool bulk_ok, uint64_t* bar, uint32_t* tx, bool issue, int tid, int nt) {
  constexpr int vec = 16 / sizeof(T);
  int64_t lo = begin & ~(int64_t)(vec - 1);
  int head = (int)(begin - lo);
  if(end <= begin) return head;
  int64_t whole = count & ~(int64_t)(vec - 1);          // items in whole vectors
  int64_t hi = min((end + vec - 1) & ~(int64_t)(vec - 1), whole);
  int64_t plain_from = begin;
  if(bulk_ok && hi > lo) {
    if(issue) bulk_load(dst, src + lo, (uint32_t)((hi - lo) * sizeof(T)), bar);
    *tx += (uint32_t)((hi - lo) * sizeof(T));
    plain_from = max(hi, begin);
  }
  for(int64_t i = plain_from + tid; i < end; i += nt) dst[i - lo] = src[i];
  return head;
}

template<typename K, typename V, int NT, int VT, typename comp_t>
struct merge_tile_t {
  typedef merge_tile_layout<K, V, NT, VT> L;
  static constexpr bool has_values = L::has_values;

  // Merges A[a_begin, a_end) with B[b_begin, b_end) (total <= nv) and writes
  // the result at out_keys/out_vals[out_base ...].  `ka`, `kb` etc. are the
  // full arrays (their counts bound the plain-load tails).
  __device__ static void run(unsigned char* smem,
    const K* a_keys, const V* a_vals, int64_t a_total, int64_t a_begin, int64_t a_end,
    const K* b_keys, const V* b_vals, int64_t b_total, int64_t b_begin, int64_t b_end,
    K* out_keys, V* out_vals, int64_t out_base, bool bulk_ok, comp_t comp, int* error) {
    const int tid = threadIdx.x;
    K* sk = (K*)(smem + L::keys_off);
    V* sv = (V*)(smem + L::vals_off);
    uint64_t* bar = (uint64_t*)(smem + L::bar_off);
    const int a_cnt = (int)(a_end - a_begin), b_cnt = (int)(b_end - b_begin);
    const int total = a_cnt + b_cnt;

    // B's staging window starts after A's, on a 16-byte boundary.
    const int a_klen = (int)(((a_end + L::kvec - 1) & ~(int64_t)(L::kvec - 1)) -
      (a_begin & ~(int64_t)(L::kvec - 1)));
    const int b_koff = (a_klen + L::kvec - 1) / L::kvec * L::kvec;
    const int a_vlen = (int)(((a_end + L::vvec - 1) & ~(int64_t)(L::vvec - 1)) -
      (a_begin & ~(int64_t)(L::vvec - 1)));
    const int b_voff = (a_vlen + L::vvec - 1) / L::vvec * L::vvec;

    if(tid == 0) { mbar_init(bar, 1); fence_mbar_init(); }
    __syncthreads();
    uint32_t tx = 0;
    const bool issue = tid == 0;
    // Thread 0 first announces the byte count, then issues the copies.
    if(bulk_ok && issue) {
      uint32_t t = 0;
      stage_bytes(a_begin, a_end, a_total, &t, (int)sizeof(K));
      stage_bytes(b_begin, b_end, b_total, &t, (int)sizeof(K));
      if(has_values) {
        stage_bytes(a_begin, a_end, a_total, &t, (int)sizeof(V));
        stage_bytes(b_begin, b_end, b_total, &t, (int)sizeof(V));
      }
      mbar_arrive_expect_tx(bar, t);
    }
    int a_head = stage_range(sk, a_keys, a_begin, a_end, a_total, bulk_ok, bar, &tx, issue, tid, NT);
    int b_head = stage_range(sk + b_koff, b_keys, b_begin, b_end, b_total, bulk_ok, bar, &tx,
      issue, tid, NT);
    int av_head = 0, bv_head = 0;
    if constexpr(has_values) {
      av_head = stage_range(sv, a_vals, a_begin, a_end, a_total, bulk_ok, bar, &tx, issue, tid, NT);
      bv_head = stage_range(sv + b_voff, b_vals, b_begin, b_end, b_total, bulk_ok, bar, &tx,
        issue, tid, NT);
    }
    bool ok = true;
    if(bulk_ok) ok = mbar_wait_bounded(bar, 0, error);
    if(__syncthreads_or(!ok)) {
      mbar_wait_bounded(bar, 0, error);
      return;
    }

    const K* A = sk + a_head;
    const K* B = sk + b_koff + b_head;
    // Each thread merges VT outputs starting at diagonal VT * tid.
    K keys[VT];
    int src[VT];
    int diag = VT * tid;
    if(diag < total) {
      int ai = merge_path(A, a_cnt, B, b_cnt, diag, comp);
      int bi = diag - ai;
      K ak = A[min(ai, a_cnt - 1 < 0 ? 0 : a_cnt - 1)];
      K bk = B[min(bi, b_cnt - 1 < 0 ? 0 : b_cnt - 1)];
      if(ai < a_cnt) ak = A[ai];
      if(bi < b_cnt) bk = B[bi];
#pragma unroll
      for(int i = 0; i < VT; ++i) {
        bool take_a = bi >= b_cnt || (ai < a_cnt && !comp(bk, ak));
        keys[i] = take_a ? ak : bk;
        src[i] = take_a ? ai : a_cnt + bi;
        if(take_a) { ++ai; if(ai < a_cnt) ak = A[ai]; }
        else { ++bi; if(bi < b_cnt) bk = B[bi]; }
      }
    }
    V vals[VT];
    if constexpr(has_values) {
      const V* AV = sv + av_head;
      const V* BV = sv + b_voff + bv_head;
      if(diag < total) {
#pragma unroll
        for(int i = 0; i < VT; ++i) {
          int s = src[i];
          vals[i] = s < a_cnt ? AV[s] : BV[s - a_cnt];
        }
      }
    }
    __syncthreads();
    // Stage outputs in thread order, then store with coalesced vectors.
    if(diag < total) {
#pragma unroll
      for(int i = 0; i < VT; ++i) {
        sk[diag + i] = keys[i];
        if constexpr(has_values) sv[diag + i] = vals[i];
      }
    }
    __syncthreads();
    store_tile(sk, out_keys, out_base, total, tid);
    if constexpr(has_values) store_tile(sv, out_vals, out_base, total, tid);
  }

  __device__ static void stage_bytes(int64_t begin, int64_t end, int64_t count, uint32_t* t,
    int size) {
    int64_t vec = 16 / size;
    if(end <= begin) return;
    int64_t lo = begin & ~(vec - 1);
    int64_t whole = count & ~(vec - 1);
    int64_t hi = min((end + vec - 1) & ~(vec - 1), whole);
    if(hi > lo) *t += (uint32_t)((hi - lo) * size);
  }

  template<typename T>
  __device__ static void store_tile(const T* s, T* out, int64_t base, int total, int tid) {
    constexpr int vec = 16 / sizeof(T);
    T* dst = out + base;
    if(aligned16(dst) && total == L::nv) {
      const uint4* s4 = (const uint4*)s;
      uint4* d4 = (uint4*)dst;
      for(int i = tid; i < L::nv / vec; i += NT) d4[i] = s4[i];
    } else {
      for(int i = tid; i < total; i += NT) dst[i] = s[i];
    }
  }
};

// One CTA per output tile of a two-array merge.
template<typename K, typename V, int NT, int VT, typename comp_t>
__global__ void __launch_bounds__(NT)
merge_kernel(const K* a_keys, const V* a_vals, int64_t a_count, const K* b_keys,
  const V* b_vals, int64_t b_count, K* c_keys, V* c_vals, const int64_t* mp, int bulk_ok,
  comp_t comp, int* error) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NV = NT * VT;
  const int64_t tile = blockIdx.x;
  const int64_t diag0 = tile * NV;
  const int64_t diag1 = min(diag0 + NV, a_count + b_count);
  const int64_t mp0 = mp[tile], mp1 = mp[tile + 1];
  merge_tile_t<K, V, NT, VT, comp_t>::run(smem, a_keys, a_vals, a_count, mp0, mp1,
    b_keys, b_vals, b_count, diag0 - mp0, diag1 - mp1, c_keys, c_vals, diag0, bulk_ok != 0,
    comp, error);
}

// One CTA per output tile of a mergesort pass over runs of `run` items.
template<typename K, typename V, int NT, int VT, typename comp_t>
__global__ void __launch_bounds__(NT)
mergesort_pass_kernel(const K* keys_in, const V* vals_in, K* keys_out, V* vals_out,
  int64_t count, int64_t run, const int64_t* mp, int bulk_ok, comp_t comp, int* error) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NV = NT * VT;
  // Launched as a dependent of the previous pass (or the blocksort).
  griddep_wait();
  griddep_launch_dependents();
  const int64_t tile = blockIdx.x;
  const int64_t pos0 = tile * NV;
  const int64_t pair = pos0 / (2 * run);
  const int64_t a0 = pair * 2 * run;
  const int64_t a1 = min(a0 + run, count);
  const int64_t b1 = min(a0 + 2 * run, count);
  const int64_t diag0 = pos0 - a0;
  const int64_t diag1 = min(diag0 + NV, b1 - a0);
  int64_t mp0, mp1;
  if(mp) {
    mp0 = mp[tile];
    mp1 = diag1 == b1 - a0 ? a1 - a0 : mp[tile + 1];
  } else {
    // No partition launch: warps 0 and 1 search this tile's two splits.
    __shared__ int64_t s_mp[2];
    const int warp = threadIdx.x >> 5;
    if(warp < 2) {
      const int64_t d = warp ? diag1 : diag0;
      const int64_t r = (warp && d == b1 - a0) ? a1 - a0 :
        merge_path_warp(keys_in + a0, a1 - a0, keys_in + a1, b1 - a1, d, comp);
      if((threadIdx.x & 31) == 0) s_mp[warp] = r;
    }
    __syncthreads();
    mp0 = s_mp[0];
    mp1 = s_mp[1];
  }
  merge_tile_t<K, V, NT, VT, comp_t>::run(smem, keys_in, vals_in, count, a0 + mp0, a0 + mp1,
    keys_in, vals_in, count, a1 + diag0 - mp0, a1 + diag1 - mp1, keys_out, vals_out, pos0,
    bulk_ok != 0, comp, error);
}

// Sorts each tile of NT*VT items: stable odd-even transposition network in
// registers, then log2(NT) merge passes through shared memory.  With
// `index_values` the values are synthesised as the global index
// (mergesort_indices).  `vec`: all four arrays start on 16 bytes, so a full
// tile moves between global and shared memory as 16-byte vectors.
template<typename K, typename V, int NT, int VT, bool index_values, typename comp_t>
__global__ void __launch_bounds__(NT)
blocksort_kernel(const K* keys_in, const V* vals_in, K* keys_out, V* vals_out, int64_t count,
  comp_t comp, int vec) {
  constexpr bool has_values = !std::is_same<V, no_values>::value;
  constexpr int NV = NT * VT;
  __shared__ __align__(16) K sk[NV + 1];
  __shared__ __align__(16) typename std::conditional<has_values, V, char>::type
    sv[has_values ? NV : 1];
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * NV;
  const int valid = (int)min((int64_t)NV, count - base);
  // Launched as a dependent of whatever kernel precedes it on the stream.
  griddep_wait();
  griddep_launch_dependents();

  // Load the tile (coalesced), then take VT consecutive items per thread.
  constexpr int KV16 = (int)(sizeof(K) * NV / 16);
  constexpr int VV16 = has_values ? (int)(sizeof(V) * NV / 16) : 0;
  constexpr bool vec_ok = (sizeof(K) * NV) % 16 == 0 && (!has_values || (sizeof(V) * NV) % 16 == 0);
  const bool full_vec = vec_ok && vec && valid == NV;
  if(full_vec) {
    const uint4* gk = (const uint4*)(keys_in + base);
    for(int i = tid; i < KV16; i += NT) reinterpret_cast<uint4*>(sk)[i] = gk[i];
    if constexpr(has_values && !index_values) {
      const uint4* gv = (const uint4*)(vals_in + base);
      for(int i = tid; i < VV16; i += NT) reinterpret_cast<uint4*>(sv)[i] = gv[i];
    }
  } else {
    for(int i = tid; i < valid; i += NT) {
      sk[i] = keys_in[base + i];
      if constexpr(has_values && !index_values) sv[i] = vals_in[base + i];
    }
  }
  __syncthreads();
  K k[VT];
  V v[VT];
#pragma unroll
  for(int i = 0; i < VT; ++i) {
    int j = VT * tid + i;
    k[i] = sk[min(j, NV - 1)];
    if constexpr(has_values) {
      if constexpr(index_values) v[i] = (V)(base + j);
      else v[i] = sv[min(j, NV - 1)];
    }
  }
  // Items past `valid` never swap with in-range items: a swap of i and i+1
  // is allowed only when item i+1 is in range (reference:
  // out_of_range_flags, common/cta_mergesort.hxx:7-15).
  const int first = VT * tid;
#pragma unroll
  for(int I = 0; I < VT; ++I) {
#pragma unroll
    for(int i = 1 & I; i < VT - 1; i += 2) {
      if(first + i + 1 < valid && comp(k[i + 1], k[i])) {
        K t = k[i]; k[i] = k[i + 1]; k[i + 1] = t;
        if constexpr(has_values) { V u = v[i]; v[i] = v[i + 1]; v[i + 1] = u; }
      }
    }
  }
  __syncthreads();

  // Merge passes: lists of VT << p items, coop groups of 2 << p threads.
#pragma unroll 1
  for(int coop = 2; coop <= NT; coop <<= 1) {
#pragma unroll
    for(int i = 0; i < VT; ++i) {
      sk[VT * tid + i] = k[i];
      if constexpr(has_values) sv[VT * tid + i] = v[i];
    }
    __syncthreads();
    int start = VT * (tid & ~(coop - 1));
    int half = VT * (coop >> 1);
    int a_begin = min(start, valid), a_end = min(start + half, valid);
    int b_begin = a_end, b_end = min(start + 2 * half, valid);
    int a_cnt = a_end - a_begin, b_cnt = b_end - b_begin;
    int diag = VT * tid - start;
    if(VT * tid < valid) {
      const K* A = sk + a_begin;
      const K* B = sk + b_begin;
      int ai = merge_path(A, a_cnt, B, b_cnt, min(diag, a_cnt + b_cnt), comp);
      int bi = min(diag, a_cnt + b_cnt) - ai;
      K ak = A[min(ai, max(a_cnt - 1, 0))];
      K bk = B[min(bi, max(b_cnt - 1, 0))];
#pragma unroll
      for(int i = 0; i < VT; ++i) {
        bool take_a = bi >= b_cnt || (ai < a_cnt && !comp(bk, ak));
        int s = take_a ? a_begin + ai : b_begin + bi;
        k[i] = take_a ? ak : bk;
        if constexpr(has_values) v[i] = sv[min(s, NV - 1)];
        if(take_a) { ++ai; ak = A[min(ai, max(a_cnt - 1, 0))]; }
        else { ++bi; bk = B[min(bi, max(b_cnt - 1, 0))]; }
      }
    }
    __syncthreads();
  }

#pragma unroll
  for(int i = 0; i < VT; ++i) {
    sk[VT * tid + i] = k[i];
    if constexpr(has_values) sv[VT * tid + i] = v[i];
  }
  __syncthreads();
  if(full_vec) {
    uint4* gk = (uint4*)(keys_out + base);
    for(int i = tid; i < KV16; i += NT) gk[i] = reinterpret_cast<const uint4*>(sk)[i];
    if constexpr(has_values) {
      uint4* gv = (uint4*)(vals_out + base);
      for(int i = tid; i < VV16; i += NT) gv[i] = reinterpret_cast<const uint4*>(sv)[i];
    }
  } else {
    for(int i = tid; i < valid; i += NT) {
      keys_out[base + i] = sk[i];
      if constexpr(has_values) vals_out[base + i] = sv[i];
    }
  }
}

}  // namespace device
}  // namespace mgpu
