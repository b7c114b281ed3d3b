// mgpu::gb300::merge / mergesort - host drivers of the merge-path kernels.
//
// merge: drop-in for vk::merge (vk/merge.hxx:12-59): key-value and keys-only
// overloads, comparator functor, two-phase aux of one partition per tile
// (int64 here, for counts past 2^31).  Partition launch + merge launch.
//
// mergesort_kv / mergesort_keys / mergesort_indices: drop-ins for
// vk/mergesort.hxx:10-103.  One tile fits in one CTA: blocksort in place, no
// aux.  Otherwise: aux = partitions + key/value ping-pong buffers; blocksort
// into the buffer chosen by the parity of the pass count so that the last
// pass lands in the caller's arrays (vk/mergesort.hxx:47-59); then one merge
// launch per pass over pairs of sorted runs, which finds its own splits up to
// 8192 tiles and above that follows a partition launch.  The blocksort and
// the passes are launched as programmatic dependents of the kernel before
// them.
#pragma once

#include "context.hxx"
#include "../device/merge.cuh"

namespace mgpu {
namespace gb300 {

template<typename T> using less_t = device::less_t<T>;
template<typename T> using greater_t = device::greater_t<T>;

// Drop-ins for the reference's partition helpers (common/types.hxx:73-76,
// common/cta_merge.hxx:6-8, vk/partition.hxx:9-20): merge_path_partitions
// writes mp_data[i] = the merge path of diagonal min(i * spacing, a_count +
// b_count) for i < num_merge_partitions(a_count + b_count, spacing), with the
// lower bound (A first on ties) or the upper one (B first).  One thread per
// partition, enqueued on the context's stream.
enum bounds_t { bounds_lower, bounds_upper };

constexpr int64_t num_merge_partitions(int64_t count, int64_t spacing) {
  return (count + spacing - 1) / spacing + 1;
}

template<bounds_t bounds = bounds_lower, typename K, typename mp_t, typename comp_t>
status_t merge_path_partitions(context_t& ctx, const K* a, int64_t a_count, const K* b,
  int64_t b_count, mp_t* mp_data, int64_t spacing, comp_t comp) {
  if(a_count < 0 || b_count < 0 || spacing < 1 || !mp_data) return MGPU_ERR_INVALID_ARG;
  if((a_count && !a) || (b_count && !b)) return MGPU_ERR_INVALID_ARG;
  const int64_t n = num_merge_partitions(a_count + b_count, spacing);
  return ctx.launch("merge_path_partitions", [&] {
    device::merge_path_partitions_kernel<bounds == bounds_upper>
      <<<(unsigned)((n + 255) / 256), 256, 0, ctx.stream>>>(a, a_count, b, b_count, spacing, n,
        mp_data, comp);
  });
}

// Source compatibility with the reference's call shape (cmd_buffer first,
// partitions before spacing: vk/partition.hxx:11-13).
template<bounds_t bounds, typename K, typename mp_t, typename comp_t>
status_t merge_path_partitions(cmd_buffer_t& cmd_buffer, const K* a, int64_t a_count,
  const K* b, int64_t b_count, mp_t* mp_data, int64_t spacing, comp_t comp) {
  return merge_path_partitions<bounds>(cmd_buffer.context, a, a_count, b, b_count, mp_data,
    spacing, comp);
}

template<int key_bytes> struct merge_tuning;
// Odd items per thread keep the per-thread strides of the serial merge and of
// the output staging odd in shared memory, so they do not collide on banks.
template<> struct merge_tuning<4> { enum { nt = 256, vt = 15 }; };
template<> struct merge_tuning<8> { enum { nt = 256, vt = 7 }; };

// Mergesort shapes: the merge shape by default.  `vt_alt` (a tuning variant)
// gives 4-byte keys 17 items per thread where the blocksort's static shared
// arrays (keys and values of one tile) stay within 48 KB: a 4352-item tile
// sorts a power-of-two count in one pass fewer than 3840 (2^20 keys: 8
// passes instead of 9), but each pass costs more, so it wins at 2^20 u32 kv
// (0.1034 against 0.1055 ms) and loses at 2^24 (0.986 against 0.957 ms).
template<typename K, typename V> struct mergesort_tuning {
  static constexpr bool has_values = !std::is_same<V, device::no_values>::value;
  static constexpr int nt = merge_tuning<sizeof(K)>::nt;
  static constexpr int vt = merge_tuning<sizeof(K)>::vt;
  static constexpr int vt_alt = sizeof(K) == 4 &&
    (sizeof(K) + (has_values ? sizeof(V) : 0)) * nt * 17 + sizeof(K) <= 48 * 1024 ? 17 : vt;
};

template<int nt = 0, int vt = 0, typename K, typename V, typename comp_t>
status_t merge_kv(void* aux_data, size_t* aux_size, context_t& ctx,
  const K* a_keys, const V* a_vals, int64_t a_count,
  const K* b_keys, const V* b_vals, int64_t b_count,
  K* c_keys, V* c_vals, comp_t comp) {
  using namespace device;
  constexpr int NT = nt ? nt : (int)merge_tuning<sizeof(K)>::nt;
  constexpr int VT = vt ? vt : (int)merge_tuning<sizeof(K)>::vt;
  constexpr int NV = NT * VT;
  constexpr bool has_values = !std::is_same<V, no_values>::value;
  typedef merge_tile_layout<K, V, NT, VT> L;
  if(a_count < 0 || b_count < 0) return MGPU_ERR_INVALID_ARG;
  const int64_t total = a_count + b_count;
  const int64_t num_tiles = div_up(total, NV);
  const int64_t num_partitions = num_tiles + 1;
  aux_layout_t lay;
  size_t mp_off = lay.add(sizeof(int64_t) * num_partitions);
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(total == 0) return MGPU_OK;
  if((a_count && !a_keys) || (b_count && !b_keys) || !c_keys) return MGPU_ERR_INVALID_ARG;
  if(has_values && ((a_count && !a_vals) || (b_count && !b_vals) || !c_vals))
    return MGPU_ERR_INVALID_ARG;
  int64_t* mp = (int64_t*)(base + mp_off);
  st = ctx.launch("merge_partition", [&] {
    if(num_partitions <= warp_partition_limit)
      merge_partition_kernel<K, comp_t, true><<<(unsigned)div_up(num_partitions, 8), 256, 0,
        ctx.stream>>>(a_keys, a_count, b_keys, b_count, NV, num_partitions, mp, comp);
    else
      merge_partition_kernel<K, comp_t, false><<<(unsigned)div_up(num_partitions, 256), 256, 0,
        ctx.stream>>>(a_keys, a_count, b_keys, b_count, NV, num_partitions, mp, comp);
  });
  if(st) return st;
  auto kernel = merge_kernel<K, V, NT, VT, comp_t>;
  if(!ctx.allow_smem(kernel, L::bytes)) return MGPU_ERR_CUDA;
  int bulk = aligned16_host(a_keys) && aligned16_host(b_keys) &&
    (!has_values || (aligned16_host(a_vals) && aligned16_host(b_vals)));
  return ctx.launch("merge", [&] {
    kernel<<<(unsigned)num_tiles, NT, L::bytes, ctx.stream>>>(a_keys, a_vals, a_count, b_keys,
      b_vals, b_count, c_keys, c_vals, mp, bulk, comp, ctx.d_error);
  });
}

// vk::merge key-value form (vk/merge.hxx:12-46).
template<int nt = 0, int vt = 0, typename K, typename V, typename comp_t>
status_t merge(void* aux_data, size_t& aux_size, context_t& ctx,
  const K* a_keys, const V* a_vals, int64_t a_count,
  const K* b_keys, const V* b_vals, int64_t b_count,
  K* c_keys, V* c_vals, comp_t comp) {
  return merge_kv<nt, vt>(aux_data, &aux_size, ctx, a_keys, a_vals, a_count, b_keys, b_vals,
    b_count, c_keys, c_vals, comp);
}

// vk::merge keys-only form (vk/merge.hxx:48-59).
template<int nt = 0, int vt = 0, typename K, typename comp_t>
status_t merge(void* aux_data, size_t& aux_size, context_t& ctx, const K* a_keys,
  int64_t a_count, const K* b_keys, int64_t b_count, K* c_keys, comp_t comp) {
  typedef device::no_values nv_t;
  return merge_kv<nt, vt>(aux_data, &aux_size, ctx, a_keys, (const nv_t*)nullptr, a_count,
    b_keys, (const nv_t*)nullptr, b_count, c_keys, (nv_t*)nullptr, comp);
}

inline int ceil_log2(int64_t x) {
  int p = 0;
  while(((int64_t)1 << p) < x) ++p;
  return p;
}

template<int nt = 0, int vt = 0, bool sort_indices = false, typename K, typename V,
  typename comp_t>
status_t mergesort_kv(void* aux_data, size_t* aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count, comp_t comp) {
  using namespace device;
  constexpr int NT = nt ? nt : mergesort_tuning<K, V>::nt;
  constexpr int VT = vt ? vt : mergesort_tuning<K, V>::vt;
  constexpr int NV = NT * VT;
  constexpr bool has_values = !std::is_same<V, no_values>::value;
  static_assert(!sort_indices || has_values, "indices need a value array");
  typedef merge_tile_layout<K, V, NT, VT> L;
  if(count < 0) return MGPU_ERR_INVALID_ARG;
  const int64_t num_tiles = div_up(count, NV);
  const int num_passes = num_tiles ? ceil_log2(num_tiles) : 0;
  aux_layout_t lay;
  size_t mp_off = 0, k_off = 0, v_off = 0;
  if(num_passes) {
    mp_off = lay.add(sizeof(int64_t) * (num_tiles + 1));
    k_off = lay.add(sizeof(K) * count);
    if(has_values) v_off = lay.add(sizeof(V) * count);
  }
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(count == 0) return MGPU_OK;
  if(!keys || (has_values && !vals)) return MGPU_ERR_INVALID_ARG;

  K* k2 = num_passes ? (K*)(base + k_off) : nullptr;
  V* v2 = (num_passes && has_values) ? (V*)(base + v_off) : nullptr;
  K* kb = (num_passes & 1) ? k2 : keys;
  V* vb = (num_passes & 1) ? v2 : vals;
  const int vec = aligned16_host(keys) && aligned16_host(kb) &&
    (!has_values || (aligned16_host(vals) && aligned16_host(vb)));
  // The blocksort and the passes are launched as programmatic dependents
  // (each kernel waits for its predecessor in its first instruction).
  st = ctx.launch("blocksort", [&] {
    ctx.enqueue_dependent(blocksort_kernel<K, V, NT, VT, sort_indices, comp_t>,
      (unsigned)num_tiles, NT, 0, (const K*)keys, (const V*)vals, kb, vb, count, comp, vec);
  });
  if(st || !num_passes) return st;

  K* kin = kb;
  V* vin = vb;
  K* kout = (num_passes & 1) ? keys : k2;
  V* vout = (num_passes & 1) ? vals : v2;
  int64_t* mp = (int64_t*)(base + mp_off);
  auto kernel = mergesort_pass_kernel<K, V, NT, VT, comp_t>;
  if(!ctx.allow_smem(kernel, L::bytes)) return MGPU_ERR_CUDA;
  for(int pass = 0; pass < num_passes; ++pass) {
    int64_t run = (int64_t)NV << pass;
    const bool fused = num_tiles + 1 <= warp_partition_limit;
    if(!fused) {
      st = ctx.launch("mergesort_partition", [&] {
        mergesort_partition_kernel<K, comp_t, false><<<(unsigned)div_up(num_tiles + 1, 256), 256,
          0, ctx.stream>>>(kin, count, run, NV, num_tiles + 1, mp, comp);
      });
      if(st) return st;
    }
    int bulk = aligned16_host(kin) && (!has_values || aligned16_host(vin));
    st = ctx.launch("mergesort_pass", [&] {
      ctx.enqueue_dependent(kernel, (unsigned)num_tiles, NT, L::bytes, (const K*)kin,
        (const V*)vin, kout, vout, count, run, (const int64_t*)(fused ? nullptr : mp), bulk,
        comp, ctx.d_error);
    });
    if(st) return st;
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  return MGPU_OK;
}

// vk::mergesort_kv (vk/mergesort.hxx:10-84).
template<int nt = 0, int vt = 0, typename K, typename V, typename comp_t = less_t<K>>
status_t mergesort_kv(void* aux_data, size_t& aux_size, context_t& ctx, K* keys, V* vals,
  int64_t count, comp_t comp = comp_t()) {
  return mergesort_kv<nt, vt, false>(aux_data, &aux_size, ctx, keys, vals, count, comp);
}

// vk::mergesort_keys (vk/mergesort.hxx:86-93).
template<int nt = 0, int vt = 0, typename K, typename comp_t = less_t<K>>
status_t mergesort_keys(void* aux_data, size_t& aux_size, context_t& ctx, K* keys,
  int64_t count, comp_t comp = comp_t()) {
  return mergesort_kv<nt, vt, false>(aux_data, &aux_size, ctx, keys,
    (device::no_values*)nullptr, count, comp);
}

// vk::mergesort_indices (vk/mergesort.hxx:95-103).
template<int nt = 0, int vt = 0, typename K, typename comp_t = less_t<K>>
status_t mergesort_indices(void* aux_data, size_t& aux_size, context_t& ctx, K* keys,
  int* indices, int64_t count, comp_t comp = comp_t()) {
  return mergesort_kv<nt, vt, true>(aux_data, &aux_size, ctx, keys, indices, count, comp);
}

}  // namespace gb300
}  // namespace mgpu
