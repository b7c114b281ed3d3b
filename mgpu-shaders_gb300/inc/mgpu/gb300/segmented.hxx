// mgpu::gb300::segmented_sort / segmented_scan - batched primitives over a
// CSR segment layout (offsets[s] .. offsets[s+1], an int64 device array that
// does not decrease and lies in [0, count]; the sort checks that on the
// device and, if it fails, sorts nothing and records MGPU_ERR_INVALID_ARG).
//
// No reference counterpart (the reference handles one array per call).  The
// launch sequence is fixed and independent of the number of segments:
//   sort: memset, classify, persistent small-segment sort, then for the
//         segments larger than one tile a histogram launch and one onesweep
//         pass per 8-bit digit over all of their tiles together;
//   scan: memset, head bitmap (one thread per segment), one persistent
//         look-back scan (seg_scan_defer_kernel).
// No host synchronisation; graph-capturable.
#pragma once

#include "context.hxx"
#include "radix.hxx"
#include "scan.hxx"
#include "../device/segmented.cuh"

namespace mgpu {
namespace gb300 {

// Segments of at most one small-sort tile (nt x vt keys) are merge-sorted in
// shared memory by one CTA (one warp for those of at most 32 x vt keys), with
// vt items per thread for the largest and 3, 7 or 13 for segments those
// cover (device/segmented.cuh, group_merge_sort_fit).  vt is
// odd so that threads' runs of vt items start in distinct banks (an even vt
// shares banks: 16 keys per thread made the kernel 1.6x slower than 21); four
// CTAs per SM at 64 registers.  By the width of the staged elements (the
// wider of key and value), as the onesweep shapes.  Measured on 10^5
// lognormal segments (u32 keys + values), before the fitted items per
// thread: vt 21 -> 4.47 ms per batch, 19 -> 4.49, 17 -> 4.54, 15 -> 4.62;
// three CTAs per SM at vt 21 -> 4.60 (with the fitting, 3.83 ms).
template<int elem_bytes> struct seg_small_tuning;
template<> struct seg_small_tuning<4> { enum { nt = 256, vt = 21, min_blocks = 4 }; };
template<> struct seg_small_tuning<8> { enum { nt = 256, vt = 13, min_blocks = 4 }; };

template<typename K, typename V>
status_t segmented_sort_kv(void* aux_data, size_t* aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count, const int64_t* offsets, int64_t num_segments) {
  using namespace device;
  typedef typename radix_key<K>::bits_t U;
  // Segments of at most one CTA tile sort in the small-segment kernel; larger
  // ones go through onesweep passes over tiles of the plain sort's shape.
  typedef seg_small_tuning<radix_elem_bytes<K, V>()> T;
  constexpr int NT = T::nt, ITEMS = T::vt;
  constexpr int TILE = NT * ITEMS;
  typedef radix_tuning<radix_elem_bytes<K, V>()> OT;
  constexpr int ONT = OT::nt, OITEMS = OT::vt, MINB = OT::min_blocks;
  constexpr int OTILE = ONT * OITEMS;
  constexpr int SLICE_ITEMS = ITEMS;
  constexpr int SMALL_MINB = T::min_blocks;
  constexpr int SLICE = 32 * SLICE_ITEMS;
  constexpr int PASSES = sizeof(K);
  constexpr bool has_values = !std::is_same<V, no_values>::value;
  typedef seg_small_layout<K, V, NT, ITEMS, SLICE_ITEMS> SL;
  typedef onesweep_layout<K, V, ONT, OITEMS> OL;
  if(count < 0 || num_segments < 0 || count > radix_max_count || num_segments > INT32_MAX)
    return MGPU_ERR_INVALID_ARG;
  // Large segments hold more than TILE keys each; each adds at most one
  // partial onesweep tile.
  const int64_t max_large = std::min<int64_t>(num_segments, count / (TILE + 1));
  const int64_t max_tiles = max_large ? div_up(count, OTILE) + max_large : 0;
  aux_layout_t lay;
  size_t cnt_off = lay.add(sizeof(uint32_t) * sc_count);
  size_t warp_off = lay.add(sizeof(int) * num_segments);
  size_t slice_off = lay.add(sizeof(int) * num_segments);
  size_t cta_off = lay.add(sizeof(int) * num_segments);
  size_t large_off = lay.add(sizeof(int) * max_large);
  size_t ltb_off = lay.add(sizeof(int) * max_large);
  size_t owner_off = lay.add(sizeof(int) * max_tiles);
  size_t hist_off = lay.add(sizeof(uint32_t) * max_large * PASSES * radix_bins);
  size_t lb_off = lay.add(sizeof(uint32_t) * PASSES * max_tiles * radix_bins);
  size_t k2_off = max_large ? lay.add(sizeof(K) * count) : 0;
  size_t v2_off = (max_large && has_values) ? lay.add(sizeof(V) * count) : 0;
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(count == 0 || num_segments == 0) return MGPU_OK;
  if(!keys || !offsets || (has_values && !vals)) return MGPU_ERR_INVALID_ARG;

  seg_state_t s;
  s.counters = (uint32_t*)(base + cnt_off);
  s.warp_list = (int*)(base + warp_off);
  s.slice_list = (int*)(base + slice_off);
  s.cta_list = (int*)(base + cta_off);
  s.large_seg = (int*)(base + large_off);
  s.large_tile_base = (int*)(base + ltb_off);
  s.tile_owner = (int*)(base + owner_off);
  s.seg_hist = (uint32_t*)(base + hist_off);
  s.lookback = (uint32_t*)(base + lb_off);
  s.max_tiles = max_tiles;
  s.max_large = max_large;

  if(ctx.check(cudaMemsetAsync(s.counters, 0, sizeof(uint32_t) * sc_count, ctx.stream)))
    return MGPU_ERR_CUDA;
  int cgrid = (int)std::min<int64_t>(div_up(num_segments, 256), (int64_t)ctx.sm_count * 8);
  st = ctx.launch("seg_classify", [&] {
    seg_classify<TILE, OTILE, SLICE, PASSES><<<cgrid, 256, 0, ctx.stream>>>(offsets,
      num_segments, count, s, ctx.d_error);
  });
  if(st) return st;

  auto small = seg_small_sort<K, V, NT, ITEMS, SLICE_ITEMS, PASSES, SMALL_MINB>;
  if(!ctx.allow_smem(small, SL::bytes)) return MGPU_ERR_CUDA;
  const int per_sm = ctx.resident_ctas(small, NT, SL::bytes);
  if(per_sm < 1) return MGPU_ERR_CUDA;
  const int sgrid = ctx.sm_count * per_sm;
  st = ctx.launch("seg_small_sort", [&] {
    small<<<sgrid, NT, SL::bytes, ctx.stream>>>(keys, vals, offsets, s);
  });
  if(st || !max_large) return st;

  st = ctx.launch("seg_histogram", [&] {
    seg_histogram<K, 512, OTILE, PASSES><<<ctx.sm_count * 4, 512, 0, ctx.stream>>>(keys,
      offsets, s);
  });
  if(st) return st;
  auto pass_kernel = seg_onesweep_pass<K, V, ONT, OITEMS, MINB, PASSES>;
  if(!ctx.allow_smem(pass_kernel, OL::bytes)) return MGPU_ERR_CUDA;
  U* k_io[2] = { (U*)keys, (U*)(base + k2_off) };
  V* v_io[2] = { vals, has_values ? (V*)(base + v2_off) : nullptr };
  for(int p = 0; p < PASSES; ++p) {
    onesweep_args<K, V> a;
    a.keys_in = k_io[p & 1];
    a.keys_out = k_io[(p + 1) & 1];
    a.vals_in = v_io[p & 1];
    a.vals_out = v_io[(p + 1) & 1];
    a.count = count;
    a.shift = 8 * p;
    a.hist = nullptr;
    a.lookback = nullptr;
    a.tile_counter = s.counters + sc_pass_tiles + p;
    a.error = ctx.d_error;
    a.wait_limit = ctx.wait_limit > 0 ? ctx.wait_limit : spin_limit;
    a.first = p == 0;
    a.last = p == PASSES - 1;
    a.tma = aligned16_host(a.keys_in) && (!has_values || aligned16_host(a.vals_in));
    st = ctx.launch("seg_onesweep_pass", [&] {
      pass_kernel<<<(unsigned)max_tiles, ONT, OL::bytes, ctx.stream>>>(a, offsets, s, p);
    });
    if(st) return st;
  }
  return MGPU_OK;
}

template<typename K>
status_t segmented_sort(void* aux_data, size_t& aux_size, context_t& ctx, K* keys, int64_t count,
  const int64_t* offsets, int64_t num_segments) {
  return segmented_sort_kv(aux_data, &aux_size, ctx, keys, (device::no_values*)nullptr, count,
    offsets, num_segments);
}

template<typename K, typename V>
status_t segmented_sort(void* aux_data, size_t& aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count, const int64_t* offsets, int64_t num_segments) {
  return segmented_sort_kv(aux_data, &aux_size, ctx, keys, vals, count, offsets, num_segments);
}

// Scan of each segment independently (exclusive: a segment's first output
// is init).  `op` as for scan(): associative and commutative.
template<scan_type_t scan_type = scan_type_inc, typename T, typename op_t = plus_t<T>>
status_t segmented_scan(void* aux_data, size_t* aux_size, context_t& ctx, const T* in,
  int64_t count, T* out, const int64_t* offsets, int64_t num_segments,
  T init = op_t::identity(), op_t op = op_t()) {
  using namespace device;
  static_assert(commutative_op<op_t>::value,
    "segmented_scan combines partials out of element order: op must be associative and "
    "commutative (specialise mgpu::gb300::commutative_op for a user operator that is)");
  // 8192-element tiles at 3 CTAs/SM for 4-byte values (measured against 4
  // CTAs/SM and 4096-element tiles); 8-byte values spill above 2 CTAs/SM.
  constexpr int NT = 256;
  constexpr int VT = sizeof(T) == 4 ? 32 : 16;
  constexpr int MINB = sizeof(T) == 4 ? 3 : 2;
  constexpr int TILE = NT * VT;
  constexpr bool packed = seg_status_t<T>::packed;
  if(count < 0 || num_segments < 0 || num_segments > INT32_MAX) return MGPU_ERR_INVALID_ARG;
  const int64_t num_tiles = div_up(count, TILE);
  if(num_tiles > 0x7fffffffll) return MGPU_ERR_INVALID_ARG;
  aux_layout_t lay;
  size_t cnt_off = lay.add(16);
  size_t flags_off = lay.add(sizeof(uint64_t) * num_tiles);
  size_t bits_off = lay.add(sizeof(uint32_t) * (TILE / 32) * num_tiles);
  size_t head_bytes = lay.total;
  size_t vals_off = packed ? 0 : lay.add(2 * sizeof(uint64_t) * num_tiles);
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(count == 0) return MGPU_OK;
  if(!in || !out || !offsets || num_segments == 0) return MGPU_ERR_INVALID_ARG;
  (void)cnt_off;
  if(ctx.check(cudaMemsetAsync(base, 0, head_bytes, ctx.stream))) return MGPU_ERR_CUDA;
  uint32_t* bits = (uint32_t*)(base + bits_off);
  st = ctx.launch("seg_mark_heads", [&] {
    seg_mark_heads<256><<<(unsigned)div_up(num_segments, 256), 256, 0, ctx.stream>>>(offsets,
      num_segments, count, bits);
  });
  if(st) return st;
  seg_status_t<T> status { (uint32_t*)(base + flags_off),
    packed ? nullptr : (uint64_t*)(base + vals_off), num_tiles };
  typedef seg_scan_defer_layout<T, NT, VT> SL;
  auto k = seg_scan_defer_kernel<T, op_t, NT, VT, scan_type == scan_type_exc, MINB>;
  if(!ctx.allow_smem(k, SL::bytes)) return MGPU_ERR_CUDA;
  const int per_sm = ctx.resident_ctas(k, NT, SL::bytes);
  if(per_sm < 1) return MGPU_ERR_CUDA;
  const int64_t grid = std::min<int64_t>((int64_t)per_sm * ctx.sm_count, num_tiles);
  const int vec = aligned16_host(in) && aligned16_host(out);
  return ctx.launch("seg_scan", [&] {
    k<<<(unsigned)grid, NT, SL::bytes, ctx.stream>>>(in, out, count, bits, init, op, status,
      (uint32_t*)base, ctx.d_error, vec);
  });
}

}  // namespace gb300
}  // namespace mgpu
