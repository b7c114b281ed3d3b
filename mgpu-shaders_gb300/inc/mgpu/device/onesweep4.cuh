// Onesweep pass over 4-bit digits: the reference's default digit width.
//
// Reference behaviour (seanbaxter/mgpu-shaders): radix_sort's default
// template is <nt = 128, vt = 15, num_bits = 4> (vk/radix.hxx:195-198); its
// 4-bit digits are ranked by cta_radix_rank_t<..., radix_kind_shared>
// (common/cta_radix.hxx:76-206), which counts digits in per-thread packed
// 16-bit histograms in shared memory and scans them across the CTA.  Twice
// as many passes move twice the bytes of 8-bit digits, so the width pays
// where the data stays in L2 and ranking, not memory, bounds a pass.
//
// Here 16 digits need no shared-memory ranking at all: four warp ballots of
// the digit bits give every lane its peers (the lanes holding the same
// digit), and each warp's 16 running counts live in registers of lanes
// 0..15, read with one shuffle.  The rest follows the 8-bit onesweep pass
// (onesweep.cuh): the tile is bulk-copied into region A, keys are scattered
// into region B in local digit order and written out in runs, the values'
// copy reuses A, and global offsets come from a decoupled look-back over
// rows of 16 status words per tile.  Stable, so the permutation equals the
// 8-bit sort's.
#pragma once

#include "onesweep.cuh"

namespace mgpu {
namespace device {

constexpr int radix4_bins = 16;

template<typename K, typename V, int NT, int ITEMS>
struct onesweep4_layout {
  typedef typename radix_key<K>::bits_t U;
  static constexpr bool has_values = !std::is_same<V, no_values>::value;
  static constexpr int tile = NT * ITEMS;
  static constexpr int num_warps = NT / 32;
  static constexpr size_t elem = has_values && sizeof(V) > sizeof(U) ? sizeof(V) : sizeof(U);
  static constexpr size_t a_off = 0;                       // staged keys, then values
  static constexpr size_t b_off = a_off + elem * tile + 16; // keys, then values, sorted
  static constexpr size_t w_off = b_off + elem * tile;      // [warp][16] counts -> offsets
  static constexpr size_t gbase_off = w_off + ((sizeof(uint32_t) * num_warps * radix4_bins + 15) & ~(size_t)15);
  static constexpr size_t bar_off = gbase_off + sizeof(int) * radix4_bins;
  static constexpr size_t tile_off = bar_off + sizeof(uint64_t) * 2;
  static constexpr size_t bytes = tile_off + 16;
  static_assert(NT >= 32 && NT % 32 == 0, "whole warps");
  static_assert((sizeof(U) * tile) % 16 == 0, "bulk-copy granularity");
  static_assert(ITEMS % 2 == 0 && tile <= 65536, "ranks are packed 16-bit pairs");
};

// Lanes whose 4-bit digit is `d`, from the ballots of the four digit bits.
__device__ __forceinline__ uint32_t digit4_lanes(uint32_t d, const uint32_t (&b)[4]) {
  return ((d & 1) ? b[0] : ~b[0]) & ((d & 2) ? b[1] : ~b[1]) &
         ((d & 4) ? b[2] : ~b[2]) & ((d & 8) ? b[3] : ~b[3]);
}

template<typename K, typename V, int NT, int ITEMS, int WINDOW = 4>
__device__ __forceinline__ void onesweep4_tile(const onesweep_args<K, V>& a,
  const onesweep_tile_t& t, unsigned char* smem) {
  typedef onesweep4_layout<K, V, NT, ITEMS> L;
  typedef typename L::U U;
  constexpr int TILE = L::tile;
  constexpr int NWARPS = L::num_warps;
  constexpr bool HAS_V = L::has_values;
  constexpr int CHUNK = 4;
  constexpr int BINS = radix4_bins;

  unsigned char* A = smem + L::a_off;
  unsigned char* B = smem + L::b_off;
  uint32_t* W = (uint32_t*)(smem + L::w_off);
  int* gbase = (int*)(smem + L::gbase_off);
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = t.base;
  const int valid = t.valid;
  const int tile = t.local;
  // Tiles start on whole tiles; a ragged last tile copies its whole 16-byte
  // units and loads the rest (see onesweep_tile).
  constexpr int64_t KV = 16 / sizeof(U);
  constexpr int64_t VV = HAS_V ? 16 / sizeof(V) : 1;
  auto window_end = [&](int64_t per_vec) -> int64_t {
    if(!a.tma || (base & (per_vec - 1))) return base;
    return valid == TILE ? base + TILE : (base + valid) & ~(per_vec - 1);
  };
  const int64_t kend = window_end(KV);
  const int64_t vend = HAS_V ? window_end(VV) : base;
  const bool bulk_k = kend > base, bulk_v = HAS_V && vend > base;
  const int kfill = (int)(kend - base), vfill = (int)(vend - base);
  const uint32_t vparity = bulk_k ? 1 : 0;

  if(bulk_k && tid == 0) {
    const uint32_t kbytes = (uint32_t)(sizeof(U) * (kend - base));
    mbar_arrive_expect_tx(bar, kbytes);
    bulk_load(A, a.keys_in + base, kbytes, bar);
  }
  const int warp_base = warp * 32 * ITEMS;
  const int rem = valid - warp_base - lane;
  U* const ak = (U*)A + warp_base + lane;
  if(kfill < TILE) {
    U fill = ~(U)0;                       // ranks last in every digit place
    if(a.first) {
      const K k = radix_key<K>::from_bits(~(U)0);
      memcpy(&fill, &k, sizeof(U));
    }
    const U* src = a.keys_in + base + warp_base + lane;
#pragma unroll 4
    for(int i = 0; i < ITEMS; ++i)
      if(warp_base + 32 * i + lane >= kfill) ak[32 * i] = 32 * i < rem ? src[32 * i] : fill;
  }
  {
    bool ok = true;
    if(bulk_k && warp == 0) ok = mbar_wait_bounded(bar, 0, a.error, a.wait_limit);
    if(__syncthreads_or(!ok)) {
      if(warp == 0) mbar_wait_bounded(bar, 0, a.error, a.wait_limit);
      return;
    }
  }
  auto key_bits = [&](int i) -> U {
    U u = ak[32 * i];
    if(a.first) {
      K key;
      memcpy(&key, &u, sizeof(K));
      u = radix_key<K>::to_bits(key);
    }
    return u;
  };

  // Ranking in registers: rows of 32 lanes in element order; lane l < 16
  // keeps this warp's running count of digit l.
  uint32_t rp[ITEMS / 2];
  uint32_t wc = 0;
  {
    const uint32_t lt_mask = lanemask_lt();
#pragma unroll
    for(int i = 0; i < ITEMS; ++i) {
      const uint32_t d = extract_digit(key_bits(i), a.shift, 4);
      uint32_t b[4];
#pragma unroll
      for(int k = 0; k < 4; ++k) b[k] = __ballot_sync(0xffffffffu, (d >> k) & 1);
      const uint32_t cnt = __shfl_sync(0xffffffffu, wc, (int)d);
      const uint32_t rank = cnt + __popc(digit4_lanes(d, b) & lt_mask);
      wc += __popc(digit4_lanes((uint32_t)lane & (BINS - 1), b));
      if(i & 1) rp[i >> 1] |= rank << 16;
      else rp[i >> 1] = rank;
    }
  }
  if(lane < BINS) W[warp * BINS + lane] = wc;
  __syncthreads();

  // Warp 0, lane d < 16: counts per warp -> exclusive offsets (in place in
  // W), publish the tile's count, scan the 16 tile counts and digit totals.
  lookback_window_t<WINDOW, 4, BINS> lbw;
  uint32_t valid_cnt = 0, tile_start = 0, glob_start = 0;
  if(warp == 0) {
    uint32_t tile_cnt = 0, h = 0;
    if(lane < BINS) {
#pragma unroll
      for(int w = 0; w < NWARPS; ++w) {
        const uint32_t c = W[w * BINS + lane];
        W[w * BINS + lane] = tile_cnt;
        tile_cnt += c;
      }
      valid_cnt = tile_cnt - (lane == BINS - 1 ? (uint32_t)(TILE - valid) : 0u);
      st_relaxed(&t.lb_row[lane], (tile ? lb_agg : lb_inc) | valid_cnt);
      h = t.hist[lane];
    }
    uint32_t xi = tile_cnt, yi = h;
#pragma unroll
    for(int off = 1; off < BINS; off <<= 1) {
      const uint32_t tx = __shfl_up_sync(0xffffffffu, xi, off);
      const uint32_t ty = __shfl_up_sync(0xffffffffu, yi, off);
      if(lane >= off) { xi += tx; yi += ty; }
    }
    tile_start = xi - tile_cnt;
    glob_start = yi - h;
    if(lane < BINS) {
      if(tile > 0) lbw.issue(t.lb_row + lane - BINS, tile);
#pragma unroll
      for(int w = 0; w < NWARPS; ++w) W[w * BINS + lane] += tile_start;
    }
  }
  __syncthreads();

  // Keys into B in local digit order; ranks become local positions.
  {
    const uint32_t* wh = W + warp * BINS;
#pragma unroll
    for(int i = 0; i < ITEMS; ++i) {
      const U k = key_bits(i);
      const uint32_t sh = (i & 1) * 16;
      const uint32_t r = ((rp[i >> 1] >> sh) & 0xffffu) + wh[extract_digit(k, a.shift, 4)];
      rp[i >> 1] = (rp[i >> 1] & ~(0xffffu << sh)) | (r << sh);
      ((U*)B)[r] = k;
    }
  }
  __syncthreads();
  if(bulk_v && tid == 0) {
    const uint32_t vbytes = (uint32_t)(sizeof(V) * (vend - base));
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, vbytes);
    bulk_load(A, a.vals_in + base, vbytes, bar);
  }
  if(warp == 0 && lane < BINS) {
    uint32_t excl = 0;
    if(tile > 0) {
      excl = lbw.finish(a.error, a.wait_limit);
      st_relaxed(&t.lb_row[lane], lb_inc | (excl + valid_cnt));
    }
    gbase[lane] = (int)(glob_start + excl - tile_start);
  }
  __syncthreads();

  U* keys_out = a.keys_out + t.out_base;
  uint32_t dq[(ITEMS + 3) / 4];
#pragma unroll
  for(int j0 = 0; j0 < ITEMS; j0 += CHUNK) {
    U u[CHUNK];
    uint32_t dst[CHUNK];
#pragma unroll
    for(int c = 0; c < CHUNK; ++c) {
      const int idx = (j0 + c) * NT + tid;
      if(j0 + c < ITEMS && idx < valid) {
        u[c] = ((const U*)B)[idx];
        const uint32_t d = extract_digit(u[c], a.shift, 4);
        const int j = j0 + c;
        if(HAS_V) dq[j >> 2] = (j & 3) ? dq[j >> 2] | (d << (8 * (j & 3))) : d;
        dst[c] = (uint32_t)gbase[d] + idx;
      }
    }
#pragma unroll
    for(int c = 0; c < CHUNK; ++c) {
      if(j0 + c < ITEMS && (j0 + c) * NT + tid < valid) {
        if(a.last) {
          K key = radix_key<K>::from_bits(u[c]);
          U out;
          memcpy(&out, &key, sizeof(U));
          keys_out[dst[c]] = out;
        } else {
          keys_out[dst[c]] = u[c];
        }
      }
    }
  }
  if constexpr(HAS_V) {
    V* const av = (V*)A + warp_base + lane;
    bool ok = true;
    if(bulk_v && warp == 0) ok = mbar_wait_bounded(bar, vparity, a.error, a.wait_limit);
    if(__syncthreads_or(!ok)) {
      if(warp == 0) mbar_wait_bounded(bar, vparity, a.error, a.wait_limit);
      return;
    }
    if(vfill < valid) {
      const V* src = a.vals_in + base + warp_base + lane;
#pragma unroll 4
      for(int i = 0; i < ITEMS; ++i)
        if(32 * i < rem && warp_base + 32 * i + lane >= vfill) av[32 * i] = src[32 * i];
      __syncwarp();
    }
#pragma unroll
    for(int i = 0; i < ITEMS; ++i)
      if(32 * i < rem) ((V*)B)[(rp[i >> 1] >> ((i & 1) * 16)) & 0xffffu] = av[32 * i];
    __syncthreads();
    V* vals_out = a.vals_out + t.out_base;
#pragma unroll
    for(int j0 = 0; j0 < ITEMS; j0 += CHUNK) {
      V v[CHUNK];
      uint32_t dst[CHUNK];
#pragma unroll
      for(int c = 0; c < CHUNK; ++c) {
        const int idx = (j0 + c) * NT + tid;
        if(j0 + c < ITEMS && idx < valid) {
          const int j = j0 + c;
          v[c] = ((const V*)B)[idx];
          dst[c] = (uint32_t)gbase[(dq[j >> 2] >> (8 * (j & 3))) & 0xffu] + idx;
        }
      }
#pragma unroll
      for(int c = 0; c < CHUNK; ++c)
        if(j0 + c < ITEMS && (j0 + c) * NT + tid < valid) vals_out[dst[c]] = v[c];
    }
  }
}

template<typename K, typename V, int NT, int ITEMS, int MIN_BLOCKS>
__global__ void __launch_bounds__(NT, MIN_BLOCKS)
onesweep4_pass(onesweep_args<K, V> a) {
  typedef onesweep4_layout<K, V, NT, ITEMS> L;
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);
  int* s_tile = (int*)(smem + L::tile_off);
  if(threadIdx.x == 0) {
    *s_tile = (int)atomicAdd(a.tile_counter, 1u);
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int tile = *s_tile;
  onesweep_tile_t t;
  t.base = (int64_t)tile * L::tile;
  t.valid = (int)min((int64_t)L::tile, a.count - t.base);
  t.local = tile;
  t.lb_row = a.lookback + (int64_t)tile * radix4_bins;
  t.hist = a.hist;
  t.out_base = 0;
  onesweep4_tile<K, V, NT, ITEMS>(a, t, smem);
}

}  // namespace device
}  // namespace mgpu
