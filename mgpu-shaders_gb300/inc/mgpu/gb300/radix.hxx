// mgpu::gb300::radix_sort - the host driver of the onesweep LSD radix sort.
//
// Drop-in for vk::radix_sort (vk/radix.hxx:195-470): same two-phase aux
// protocol (a call with aux_data == nullptr only adds to aux_size), in-place
// result in `keys`, and the same key order (radix_permute_t bits).  The
// template knobs are (nt, vt, num_bits) = (threads per CTA, keys per thread,
// digit width): 8-bit digits by default (the reference's benchmarked setting,
// radix_sort<256,16,8>, examples/vk_radix/vk_radix.cxx:56) or 4-bit ones (its
// default template, <128,15,4>).  Key-value sorting is an addition.
//
// Launch sequence per sort: one memset of the small header (histograms and
// tile counters), radix_histogram (all digit places), then per digit a
// memset of that pass's look-back words and one onesweep pass, ping-ponging
// between `keys`/`vals` and the aux copies.  The pass count is even for 4-
// and 8-byte keys and either digit width, so the result lands in the
// caller's buffers.  No host synchronisation: the sequence is stream-ordered
// and graph-capturable.
#pragma once

#include "context.hxx"
#include "../device/onesweep.cuh"
#include "../device/onesweep4.cuh"
#include "../device/segmented.cuh"

namespace mgpu {
namespace gb300 {

// Default onesweep tile shapes (threads, keys per thread, CTAs per SM) by
// the width of the staged elements (the wider of key and value): 7296-key
// tiles of 12 warps for 4-byte elements (19 keys per thread: an odd count
// keeps the two half-warps' runs in different banks), 4096-key tiles of 8
// warps for 8-byte ones (64-bit reads serve each half-warp separately, so
// any count is conflict-free); three CTAs of about 70 KB of shared memory per
// SM either way.
template<int elem_bytes> struct radix_tuning;
template<> struct radix_tuning<4> { enum { nt = 384, vt = 19, min_blocks = 3 }; };
template<> struct radix_tuning<8> { enum { nt = 256, vt = 16, min_blocks = 3 }; };

template<typename K, typename V>
constexpr int radix_elem_bytes() {
  return (!std::is_same<V, device::no_values>::value && sizeof(V) > sizeof(K)) ? (int)sizeof(V)
                                                                               : (int)sizeof(K);
}

// Shape of the one-CTA sort that takes arrays of at most one such tile: a
// merge sort in shared memory with an odd number of keys per thread (so the
// threads' runs start in distinct banks).  A lone small sort is bound by its
// latency chain, so the CTA is wide and each thread's run short (1024 x 5:
// ten merge passes of five serial steps each).
template<int key_bytes> struct cta_sort_tuning;
template<> struct cta_sort_tuning<4> { enum { nt = 1024, vt = 5 }; };
template<> struct cta_sort_tuning<8> { enum { nt = 1024, vt = 3 }; };

// Largest count the 30-bit look-back status word can carry.
constexpr int64_t radix_max_count = (int64_t(1) << 30) - 1;

template<
  int nt = radix_tuning<sizeof(uint32_t)>::nt,
  int vt = radix_tuning<sizeof(uint32_t)>::vt,
  int min_blocks = radix_tuning<sizeof(uint32_t)>::min_blocks,
  bool dev_count = false,
  int digit_bits = 8,
  typename K, typename V>
status_t radix_sort_kv(void* aux_data, size_t* aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count, const int64_t* d_count = nullptr) {
  using namespace device;
  typedef typename radix_key<K>::bits_t U;
  static_assert(digit_bits == 8 || digit_bits == 4, "8- or 4-bit digits");
  static_assert(digit_bits == 8 || !dev_count, "device-side counts use 8-bit digits");
  constexpr bool has_values = !std::is_same<V, no_values>::value;
  constexpr int bins = 1 << digit_bits;
  constexpr int passes = 8 * (int)sizeof(K) / digit_bits;
  constexpr int tile = nt * vt;
  typedef std::conditional_t<digit_bits == 8, onesweep_layout<K, V, nt, vt>,
    onesweep4_layout<K, V, nt, vt>> L;
  constexpr int cnt = cta_sort_tuning<sizeof(K)>::nt, cvt = cta_sort_tuning<sizeof(K)>::vt;

  if(count < 0 || count > radix_max_count) return MGPU_ERR_INVALID_ARG;

  // dev_count: the number of keys is read on the device from d_count (at
  // most `count`, the capacity everything is sized for), so one captured
  // graph serves any size up to it.
  if(dev_count != (d_count != nullptr)) return MGPU_ERR_INVALID_ARG;
  int64_t num_tiles = div_up(count, tile);
  if(count <= (int64_t)cnt * cvt && !d_count) {
    // One CTA tile: the whole sort runs in shared memory in one CTA; no aux.
    char* unused = nullptr;
    status_t s0;
    if(resolve_aux(ctx, aux_data, aux_size, 0, unused, s0)) return s0;
    if(count <= 1) return MGPU_OK;
    if(!keys || (has_values && !vals)) return MGPU_ERR_INVALID_ARG;
    typedef seg_small_layout<K, V, cnt, cvt, cvt> SL;
    auto k1 = radix_sort_cta<K, V, cnt, cvt>;
    if(!ctx.allow_smem(k1, SL::bytes)) return MGPU_ERR_CUDA;
    return ctx.launch("radix_sort_cta", [&] {
      k1<<<1, cnt, SL::bytes, ctx.stream>>>(keys, vals, (int)count);
    });
  }
  aux_layout_t lay;
  size_t header_off = lay.add(sizeof(uint32_t) * (passes * bins + passes));
  size_t header_bytes = lay.total;
  size_t lookback_off = lay.add(sizeof(uint32_t) * bins * passes * num_tiles);
  size_t keys_off = lay.add(sizeof(K) * count);
  size_t vals_off = has_values ? lay.add(sizeof(V) * count) : 0;
  (void)header_off;

  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(count == 0) return MGPU_OK;
  if(!keys || (has_values && !vals)) return MGPU_ERR_INVALID_ARG;

  uint32_t* hist = (uint32_t*)base;
  uint32_t* counters = hist + passes * bins;
  uint32_t* lookback = (uint32_t*)(base + lookback_off);
  U* alt_keys = (U*)(base + keys_off);
  V* alt_vals = has_values ? (V*)(base + vals_off) : nullptr;

  if(ctx.check(cudaMemsetAsync(base, 0, header_bytes, ctx.stream))) return MGPU_ERR_CUDA;

  // Histogram of every digit place: one CTA of 1024 threads per SM, the
  // bins spread over 32 (4-byte keys) or 16 (8-byte keys) shared copies.
  {
    constexpr int hnt = 1024;
    constexpr int lanes = passes * bins <= 4 * 256 ? 32 : 16;
    constexpr size_t hsmem = sizeof(uint32_t) * passes * bins * lanes;
    auto hk = radix_histogram<K, hnt, passes, lanes, digit_bits>;
    if(!ctx.allow_smem(hk, hsmem)) return MGPU_ERR_CUDA;
    int64_t want = div_up(count, (int64_t)hnt * 16);
    int grid = (int)std::min<int64_t>(std::max<int64_t>(want, 1), (int64_t)ctx.sm_count);
    int vec = aligned16_host(keys);
    st = ctx.launch("radix_histogram", [&] {
      hk<<<grid, hnt, hsmem, ctx.stream>>>(keys, count, hist, vec, d_count);
    });
    if(st) return st;
  }

  auto kernel = [] {
    if constexpr(digit_bits == 8) return onesweep_pass<K, V, nt, vt, min_blocks, 4, dev_count>;
    else return onesweep4_pass<K, V, nt, vt, min_blocks>;
  }();
  if(!ctx.allow_smem(kernel, L::bytes)) return MGPU_ERR_CUDA;

  U* k_io[2] = { (U*)keys, alt_keys };
  V* v_io[2] = { vals, alt_vals };
  for(int p = 0; p < passes; ++p) {
    onesweep_args<K, V> a;
    a.keys_in = k_io[p & 1];
    a.keys_out = k_io[(p + 1) & 1];
    a.vals_in = v_io[p & 1];
    a.vals_out = v_io[(p + 1) & 1];
    a.count = count;
    a.shift = digit_bits * p;
    a.hist = hist + p * bins;
    a.lookback = lookback + (size_t)p * num_tiles * bins;
    a.tile_counter = counters + p;
    a.error = ctx.d_error;
    a.wait_limit = ctx.wait_limit > 0 ? ctx.wait_limit : spin_limit;
    a.first = p == 0;
    a.last = p == passes - 1;
    a.tma = aligned16_host(a.keys_in) && (!has_values || aligned16_host(a.vals_in));
    a.count_ptr = d_count;
    // Clear this pass's look-back words right before it runs, so they are
    // still in L2 when tiles poll them.
    if(ctx.check(cudaMemsetAsync(a.lookback, 0, sizeof(uint32_t) * num_tiles * bins,
      ctx.stream))) return MGPU_ERR_CUDA;
    st = ctx.launch(digit_bits == 8 ? "onesweep_pass" : "onesweep4_pass", [&] {
      kernel<<<(unsigned)num_tiles, nt, L::bytes, ctx.stream>>>(a);
    });
    if(st) return st;
  }
  static_assert(passes % 2 == 0, "result must land in the caller's buffers");
  return MGPU_OK;
}

// The launch shape the reference's knobs select.  radix_sort<nt, vt,
// num_bits> (vk/radix.hxx:195-198) chooses threads per CTA, keys per thread
// and the digit width; the permutation is the same for all of them (a stable
// LSD sort), so the knobs only trade speed.  Here num_bits 1..4 runs the
// 4-bit-digit passes (onesweep4.cuh) and 5..8 the 8-bit ones; nt is rounded
// up to whole warps (at least 256 threads for 8-bit digits, one per digit),
// vt up to an even count (ranks are packed in pairs), and 8-bit tiles hold at
// least 2 KB of match words per warp.  nt = 0 or vt = 0 keeps the tuned
// default of that digit width.  CTAs per SM follow from the shape's shared
// memory and a 56-register budget per thread.
template<typename K, typename V, int nt, int vt, int num_bits>
struct radix_knobs {
  static_assert(num_bits >= 1 && num_bits <= 8, "digit width of the reference's template");
  static constexpr int bits = num_bits <= 4 ? 4 : 8;
  static constexpr int eb = radix_elem_bytes<K, V>();
  static constexpr int nt_min = bits == 8 ? 256 : 32;
  static constexpr int nt_req = nt > 0 ? (nt + 31) / 32 * 32 : (bits == 8 ? radix_tuning<eb>::nt : 128);
  static constexpr int NT = nt_req < nt_min ? nt_min : nt_req;
  static constexpr int vt_req = vt > 0 ? (vt + 1) / 2 * 2 : (bits == 8 ? radix_tuning<eb>::vt : 16);
  static constexpr int vt_min = bits == 8 ? (64 / eb + 1) / 2 * 2 : 2;
  static constexpr int vt_max = 65536 / NT / 2 * 2;
  static constexpr int VT = vt_req < vt_min ? vt_min : (vt_req > vt_max ? vt_max : vt_req);
  typedef std::conditional_t<bits == 8, device::onesweep_layout<K, V, NT, VT>,
    device::onesweep4_layout<K, V, NT, VT>> L;
  static constexpr int by_smem = (int)(233472 / (L::bytes + 1024));
  static constexpr int by_regs = 65536 / (NT * 56);
  static constexpr int m = by_smem < by_regs ? by_smem : by_regs;
  static constexpr int MINB = m < 1 ? 1 : (m > 8 ? 8 : m);
};

// Keys-only form with the reference's signature (vk/radix.hxx:195-198):
// radix_sort<nt, vt, num_bits>(aux_data, aux_size, ctx, keys, count), with
// the knobs mapped as radix_knobs describes.
template<int nt = 0, int vt = 0, int num_bits = 8, typename K>
status_t radix_sort(void* aux_data, size_t& aux_size, context_t& ctx, K* keys, int64_t count) {
  typedef radix_knobs<K, device::no_values, nt, vt, num_bits> R;
  return radix_sort_kv<R::NT, R::VT, R::MINB, false, R::bits>(
    aux_data, &aux_size, ctx, keys, (device::no_values*)nullptr, count);
}

// Key-value form (an addition: the reference sorts keys only).
template<int nt = 0, int vt = 0, int num_bits = 8, typename K, typename V>
status_t radix_sort(void* aux_data, size_t& aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count) {
  typedef radix_knobs<K, V, nt, vt, num_bits> R;
  return radix_sort_kv<R::NT, R::VT, R::MINB, false, R::bits>(
    aux_data, &aux_size, ctx, keys, vals, count);
}

// Memcache forms: aux comes from the context's grow-only cache.
template<typename K>
status_t radix_sort(context_t& ctx, K* keys, int64_t count) {
  constexpr int b = sizeof(K);
  return radix_sort_kv<radix_tuning<b>::nt, radix_tuning<b>::vt, radix_tuning<b>::min_blocks>(
    nullptr, nullptr, ctx, keys, (device::no_values*)nullptr, count);
}
template<typename K, typename V>
status_t radix_sort(context_t& ctx, K* keys, V* vals, int64_t count) {
  constexpr int b = radix_elem_bytes<K, V>();
  return radix_sort_kv<radix_tuning<b>::nt, radix_tuning<b>::vt, radix_tuning<b>::min_blocks>(
    nullptr, nullptr, ctx, keys, vals, count);
}

}  // namespace gb300
}  // namespace mgpu
