// Test infrastructure, not product code: a scalar CPU restatement of the
// reference's own tile algorithms (seanbaxter/mgpu-shaders, inc/mgpu).
//
// The reference is Circle C++ compiled to SPIR-V and cannot be built or run
// here (no Circle compiler, no Vulkan), so its known-answer checks
// (examples/vk_radix2/vk_radix2.cxx:25-32,65-75; examples/gl_sort/gl_sort.cxx:
// 18-27,41-42; examples/vk_scan/vk_scan.cxx:25-27) are reproduced against this
// restatement instead.  Each CTA is executed as a sequence of phases, one loop
// over its `nt` threads per phase, with the same partition algebra, the same
// register/shared-memory orders and the same ranking rules as the shaders.
// Tests then show that these algorithms produce exactly what the std:: oracle
// in oracle.cpp computes, which pins that oracle to the reference.
//
// Warp (subgroup) size is 32, as on NVIDIA hardware.

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <type_traits>
#include <vector>

namespace emu {

constexpr int warp_size = 32;

inline int div_up(int x, int y) { return (x + y - 1) / y; }

// find_log2 with round-up (common/meta.hxx:37-41).
inline int find_log2(int x, bool round_up) {
  int a = 31 - __builtin_clz(x);
  if(round_up) a += (x & (x - 1)) != 0;
  return a;
}

// Number of significant bits (common/meta.hxx:43-50).  Note s_log2(nt) is
// log2(nt) + 1 for a power of two, so cta_sort_t makes one extra, empty pass.
inline int s_log2(int x) {
  int i = 0;
  while(x) { x >>= 1; ++i; }
  return i;
}

struct range_t {
  int begin, end;
  int count() const { return end - begin; }
};

// Tile of a CTA (common/types.hxx:14-17).
inline range_t get_tile(int cta, int nv, int count) {
  return range_t { nv * cta, std::min(count, nv * (cta + 1)) };
}

// Partition algebra of a two-list merge (common/types.hxx:19-58).
struct merge_range_t {
  int a_begin, a_end, b_begin, b_end;
  int a_count() const { return a_end - a_begin; }
  int b_count() const { return b_end - b_begin; }
  int total() const { return a_count() + b_count(); }
  merge_range_t to_local() const { return { 0, a_count(), a_count(), total() }; }
  merge_range_t partition(int mp0, int diag) const {
    return { a_begin + mp0, a_end, b_begin + diag - mp0, b_end };
  }
  bool a_valid() const { return a_begin < a_end; }
  bool b_valid() const { return b_begin < b_end; }
};

// Binary search of the cross diagonal `diag` (common/cta_merge.hxx:10-31).
// bounds_lower takes A on ties: pred = !comp(b, a).
template<typename K, typename comp_t>
int merge_path(const K* a, int a_count, const K* b, int b_count, int diag,
  comp_t comp, bool upper = false) {
  int begin = std::max(0, diag - b_count);
  int end = std::min(diag, a_count);
  while(begin < end) {
    int mid = (begin + end) / 2;
    K a_key = a[mid];
    K b_key = b[diag - 1 - mid];
    bool pred = upper ? comp(a_key, b_key) : !comp(b_key, a_key);
    if(pred) begin = mid + 1;
    else end = mid;
  }
  return begin;
}

// common/cta_merge.hxx:52-59.
inline merge_range_t compute_merge_range(int a_count, int b_count, int partition,
  int spacing, int mp0, int mp1) {
  int diag0 = spacing * partition;
  int diag1 = std::min(a_count + b_count, diag0 + spacing);
  return { mp0, mp1, diag0 - mp0, diag1 - mp1 };
}

// common/cta_mergesort.hxx:7-15.
inline int out_of_range_flags(int first, int vt, int count) {
  int out_of_range = std::min(vt, first + vt - count);
  int head_flags = 0;
  if(out_of_range > 0) {
    const int mask = (1 << vt) - 1;
    head_flags = mask & (~mask >> out_of_range);
  }
  return head_flags;
}

// common/cta_mergesort.hxx:17-31.
inline merge_range_t compute_mergesort_frame(int partition, int coop, int spacing) {
  int size = spacing * (coop / 2);
  int start = ~(coop - 1) & partition;
  int a_begin = spacing * start;
  int b_begin = spacing * start + size;
  return { a_begin, a_begin + size, b_begin, b_begin + size };
}

// common/cta_mergesort.hxx:33-43.
inline merge_range_t compute_mergesort_range(int count, int partition, int coop,
  int spacing) {
  merge_range_t f = compute_mergesort_frame(partition, coop, spacing);
  return { f.a_begin, std::min(count, f.a_end), std::min(count, f.b_begin),
    std::min(count, f.b_end) };
}

// common/cta_mergesort.hxx:45-68: the same with the mp0/mp1 fix-up for the
// last CTA of each cooperative merge.
inline merge_range_t compute_mergesort_range(int count, int partition, int coop,
  int spacing, int mp0, int mp1) {
  merge_range_t range = compute_mergesort_range(count, partition, coop, spacing);
  int diag = spacing * partition - range.a_begin;
  if(coop - 1 != ((coop - 1) & partition)) {
    range.a_end = range.a_begin + mp1;
    range.b_end = std::min(count, range.b_begin + diag + spacing - mp1);
  }
  range.a_begin = range.a_begin + mp0;
  range.b_begin = std::min(count, range.b_begin + diag - mp0);
  return range;
}

// Serial merge of vt items from a shared-memory image with range checks
// (common/cta_merge.hxx:41-50 merge_predicate, :107-133 serial_merge).
// `smem` has nv + 1 slots; reads past it return the slot's default.
template<typename K, typename comp_t>
void serial_merge(const std::vector<K>& smem, merge_range_t range, int vt,
  comp_t comp, K* keys, int* indices) {
  auto at = [&](int i) -> K {
    return (i >= 0 && i < (int)smem.size()) ? smem[i] : K();
  };
  K a_key = at(range.a_begin);
  K b_key = at(range.b_begin);
  for(int i = 0; i < vt; ++i) {
    bool p;
    if(!range.a_valid()) p = false;
    else if(!range.b_valid()) p = true;
    else p = !comp(b_key, a_key);
    int index = p ? range.a_begin : range.b_begin;
    keys[i] = p ? a_key : b_key;
    indices[i] = index;
    K c_key = at(++index);
    if(p) a_key = c_key, range.a_begin = index;
    else b_key = c_key, range.b_begin = index;
  }
}

// Odd-even transposition sort of one thread's vt items; bit (i+1) of
// `flags` blocks the swap of items i and i+1 (common/sort_networks.hxx:24-39).
template<typename K, typename V, typename comp_t>
void odd_even_sort(K* keys, V* vals, int vt, comp_t comp, int flags) {
  for(int I = 0; I < vt; ++I)
    for(int i = 1 & I; i < vt - 1; i += 2)
      if((0 == ((2 << i) & flags)) && comp(keys[i + 1], keys[i])) {
        std::swap(keys[i], keys[i + 1]);
        if(vals) std::swap(vals[i], vals[i + 1]);
      }
}

////////////////////////////////////////////////////////////////////////////////
// Mergesort (common/kernel_mergesort.hxx, common/cta_mergesort.hxx,
// vk/mergesort.hxx).

// One CTA of kernel_blocksort (common/kernel_mergesort.hxx:12-67) with
// cta_sort_t::block_sort (common/cta_mergesort.hxx:70-134).
template<typename K, typename comp_t>
void blocksort_cta(const K* keys_in, const int* vals_in, K* keys_out, int* vals_out,
  int count, int nt, int vt, int cta, bool has_values, bool sort_indices,
  comp_t comp) {
  const int nv = nt * vt;
  range_t tile = get_tile(cta, nv, count);
  int tc = tile.count();
  // Registers in thread order: item i of thread tid is slot vt * tid + i.
  std::vector<K> rk(nv, K());
  std::vector<int> rv(nv, 0);
  for(int j = 0; j < tc; ++j) rk[j] = keys_in[tile.begin + j];
  if(sort_indices) {
    for(int tid = 0; tid < nt; ++tid)
      for(int i = 0; i < vt; ++i) rv[vt * tid + i] = vt * (nt * cta + tid) + i;
  } else if(has_values) {
    for(int j = 0; j < tc; ++j) rv[j] = vals_in[tile.begin + j];
  }
  bool vals = has_values || sort_indices;

  // Register sort network, masked for a partial tile.
  for(int tid = 0; tid < nt; ++tid) {
    int flags = tc < nv ? out_of_range_flags(vt * tid, vt, tc) : 0;
    odd_even_sort(&rk[vt * tid], vals ? &rv[vt * tid] : (int*)nullptr, vt, comp, flags);
  }

  // log2(nt) + 1 merge passes in shared memory (cta_sort_t::merge_pass).
  int num_passes = s_log2(nt);
  std::vector<K> skeys(nv + 1, K());
  std::vector<int> svals(nv, 0);
  std::vector<K> nk(nv);
  std::vector<int> nvv(nv), idx(nv);
  for(int pass = 0; pass < num_passes; ++pass) {
    int coop = 2 << pass;
    for(int j = 0; j < nv; ++j) skeys[j] = rk[j];
    for(int tid = 0; tid < nt; ++tid) {
      merge_range_t range = compute_mergesort_range(tc, tid, coop, vt);
      int diag = vt * tid - range.a_begin;
      int mp = merge_path(skeys.data() + range.a_begin, range.a_count(),
        skeys.data() + range.b_begin, range.b_count(), diag, comp);
      serial_merge(skeys, range.partition(mp, diag), vt, comp, &nk[vt * tid],
        &idx[vt * tid]);
    }
    rk = nk;
    if(vals) {
      for(int j = 0; j < nv; ++j) svals[j] = rv[j];
      for(int j = 0; j < nv; ++j) {
        int s = idx[j];
        nvv[j] = (s >= 0 && s < nv) ? svals[s] : 0;
      }
      rv = nvv;
    }
  }
  for(int j = 0; j < tc; ++j) {
    keys_out[tile.begin + j] = rk[j];
    if(vals) vals_out[tile.begin + j] = rv[j];
  }
}

// One CTA of kernel_mergesort_pass (common/kernel_mergesort.hxx:72-121) with
// cta_merge_from_mem (common/cta_merge.hxx:135-162).
template<typename K, typename comp_t>
void mergesort_pass_cta(const int* mp_data, const K* keys_in, const int* vals_in,
  K* keys_out, int* vals_out, int count, int coop, int nt, int vt, int cta,
  bool vals, comp_t comp) {
  const int nv = nt * vt;
  range_t tile = get_tile(cta, nv, count);
  merge_range_t range = compute_mergesort_range(count, cta, coop, nv,
    mp_data[cta], mp_data[cta + 1]);
  int a_count = range.a_count(), total = range.total();
  std::vector<K> smem(nv + 1, K());
  for(int index = 0; index < total; ++index)
    smem[index] = index < a_count ? keys_in[range.a_begin + index]
      : keys_in[range.b_begin + index - a_count];
  merge_range_t local = range.to_local();
  std::vector<K> mk(nv);
  std::vector<int> idx(nv);
  for(int tid = 0; tid < nt; ++tid) {
    int diag = vt * tid;
    int mp = merge_path(smem.data() + local.a_begin, local.a_count(),
      smem.data() + local.b_begin, local.b_count(), diag, comp);
    serial_merge(smem, local.partition(mp, diag), vt, comp, &mk[vt * tid], &idx[vt * tid]);
  }
  for(int j = 0; j < tile.count(); ++j) keys_out[tile.begin + j] = mk[j];
  if(vals)
    for(int j = 0; j < total; ++j) {
      int s = idx[j];
      vals_out[tile.begin + j] = s < a_count ? vals_in[range.a_begin + s]
        : vals_in[range.b_begin + s - a_count];
    }
}

// vk::mergesort_kv driver (vk/mergesort.hxx:10-84).
template<typename K, typename comp_t>
void mergesort(K* keys, int* vals, int count, int nt, int vt, bool has_values,
  bool sort_indices, comp_t comp) {
  if(!count) return;
  int num_ctas = div_up(count, nt * vt);
  int num_passes = find_log2(num_ctas, true);
  bool v = has_values || sort_indices;
  if(0 == num_passes) {
    blocksort_cta(keys, vals, keys, vals, count, nt, vt, 0, has_values,
      sort_indices, comp);
    return;
  }
  int num_partitions = num_ctas + 1;
  std::vector<int> mp(num_partitions);
  std::vector<K> keys2_store(count);
  std::vector<int> vals2_store(count);
  K* keys2 = keys2_store.data();
  int* vals2 = vals2_store.data();
  K* kb = (1 & num_passes) ? keys2 : keys;
  int* vb = (1 & num_passes) ? vals2 : vals;
  // kernel_blocksort reads its whole tile before writing, so in-place is fine.
  std::vector<K> kin(keys, keys + count);
  std::vector<int> vin(v ? std::vector<int>(vals, vals + count) : std::vector<int>());
  for(int cta = 0; cta < num_ctas; ++cta)
    blocksort_cta(kin.data(), v ? vin.data() : nullptr, kb, vb, count, nt, vt, cta,
      has_values, sort_indices, comp);
  if(1 & num_passes) { std::swap(keys, keys2); std::swap(vals, vals2); }
  for(int pass = 0; pass < num_passes; ++pass) {
    int coop = 2 << pass;
    int spacing = nt * vt;
    // Partition transform (vk/mergesort.hxx:65-72).
    for(int index = 0; index < num_partitions; ++index) {
      merge_range_t range = compute_mergesort_range(count, index, coop, spacing);
      int diag = std::min(spacing * index, count) - range.a_begin;
      mp[index] = merge_path(keys + range.a_begin, range.a_count(),
        keys + range.b_begin, range.b_count(), diag, comp);
    }
    for(int cta = 0; cta < num_ctas; ++cta)
      mergesort_pass_cta(mp.data(), keys, vals, keys2, vals2, count, coop, nt, vt,
        cta, v, comp);
    std::swap(keys, keys2);
    std::swap(vals, vals2);
  }
}

////////////////////////////////////////////////////////////////////////////////
// Merge (vk/partition.hxx:9-20, vk/merge.hxx:12-46, common/kernel_merge.hxx).

template<typename K, typename comp_t>
void merge(const K* a_keys, const int* a_vals, int a_count, const K* b_keys,
  const int* b_vals, int b_count, K* c_keys, int* c_vals, int nt, int vt,
  bool vals, comp_t comp) {
  const int nv = nt * vt;
  int total = a_count + b_count;
  int num_partitions = div_up(total, nv) + 1;
  std::vector<int> mp(num_partitions);
  for(int index = 0; index < num_partitions; ++index) {
    int diag = std::min(nv * index, total);
    mp[index] = merge_path(a_keys, a_count, b_keys, b_count, diag, comp);
  }
  int num_blocks = div_up(total, nv);
  for(int cta = 0; cta < num_blocks; ++cta) {
    merge_range_t range = compute_merge_range(a_count, b_count, cta, nv, mp[cta],
      mp[cta + 1]);
    int ac = range.a_count(), tc = range.total();
    std::vector<K> smem(nv + 1, K());
    for(int index = 0; index < tc; ++index)
      smem[index] = index < ac ? a_keys[range.a_begin + index]
        : b_keys[range.b_begin + index - ac];
    merge_range_t local = range.to_local();
    std::vector<K> mk(nv);
    std::vector<int> idx(nv);
    for(int tid = 0; tid < nt; ++tid) {
      int diag = vt * tid;
      int p = merge_path(smem.data() + local.a_begin, local.a_count(),
        smem.data() + local.b_begin, local.b_count(), diag, comp);
      serial_merge(smem, local.partition(p, diag), vt, comp, &mk[vt * tid], &idx[vt * tid]);
    }
    for(int j = 0; j < tc; ++j) {
      c_keys[nv * cta + j] = mk[j];
      if(vals) {
        int s = idx[j];
        c_vals[nv * cta + j] = s < ac ? a_vals[range.a_begin + s]
          : b_vals[range.b_begin + s - ac];
      }
    }
  }
}

////////////////////////////////////////////////////////////////////////////////
// Scan (common/cta_scan.hxx, vk/scan.hxx), int32 with std::plus.  Integer
// adds wrap like the GPU's 32-bit adds (done in uint32_t).

inline int32_t add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

// cta_scan_t::scan, scalar form (common/cta_scan.hxx:87-135), exclusive.
// Returns the per-thread scan and the CTA reduction.  `init` enters lane 0 of
// every warp, which is the reference's behaviour.
inline void cta_scan_scalar(const std::vector<int32_t>& x, int32_t init,
  std::vector<int32_t>& scan, int32_t& reduction) {
  int nt = (int)x.size();
  int num_warps = nt / warp_size;
  std::vector<int32_t> inc(nt);
  for(int w = 0; w < num_warps; ++w) {
    int32_t s = 0;
    for(int lane = 0; lane < warp_size; ++lane) {
      s = add(s, x[w * warp_size + lane]);
      inc[w * warp_size + lane] = s;
    }
  }
  std::vector<int32_t> warps(num_warps);
  int32_t s = 0;
  for(int w = 0; w < num_warps; ++w) {
    s = add(s, inc[w * warp_size + warp_size - 1]);
    warps[w] = s;
  }
  scan.resize(nt);
  for(int tid = 0; tid < nt; ++tid) {
    int lane = tid % warp_size, warp = tid / warp_size;
    int32_t v = lane ? inc[tid - 1] : init;
    if(warp) v = add(warps[warp - 1], v);
    scan[tid] = v;
  }
  reduction = warps[num_warps - 1];
}

// cta_scan_t::scan, vector form with carry-in (common/cta_scan.hxx:139-174),
// exclusive.  x is in thread order (vt items per thread); updated in place.
inline int32_t cta_scan_vec(std::vector<int32_t>& x, int nt, int vt, int32_t carry_in,
  int32_t init) {
  std::vector<int32_t> sums(nt, 0), scan;
  for(int tid = 0; tid < nt; ++tid)
    for(int i = 0; i < vt; ++i) sums[tid] = add(sums[tid], x[vt * tid + i]);
  int32_t reduction;
  cta_scan_scalar(sums, init, scan, reduction);
  reduction = add(carry_in, reduction);
  for(int tid = 0; tid < nt; ++tid) {
    int32_t s = add(carry_in, scan[tid]);
    for(int i = 0; i < vt; ++i) {
      int32_t t = x[vt * tid + i];
      x[vt * tid + i] = s;
      s = add(s, t);
    }
  }
  return reduction;
}

// vk::scan (vk/scan.hxx:10-115): in-place exclusive scan.
inline void scan(int32_t* data, int count, int nt, int vt, int32_t init) {
  const int nv = nt * vt;
  int num_ctas = div_up(count, nv);
  if(num_ctas <= 8) {
    int32_t carry_in = 0;
    for(int cur = 0; cur < count; cur += nv) {
      int n = std::min(nv, count - cur);
      std::vector<int32_t> x(nv, 0);
      for(int j = 0; j < n; ++j) x[j] = data[cur + j];
      carry_in = cta_scan_vec(x, nt, vt, carry_in, init);
      for(int j = 0; j < n; ++j) data[cur + j] = x[j];
    }
    return;
  }
  // Upsweep: one reduction per tile (cta_reduce_t, common/cta_scan.hxx:9-59).
  std::vector<int32_t> partials(num_ctas, 0);
  for(int cta = 0; cta < num_ctas; ++cta) {
    int cur = nv * cta, n = std::min(nv, count - cur);
    int32_t s = 0;
    for(int j = 0; j < n; ++j) s = add(s, data[cur + j]);
    partials[cta] = s;
  }
  // Recursive scan of the partials, then the downsweep with carry-in.
  scan(partials.data(), num_ctas, nt, vt, init);
  for(int cta = 0; cta < num_ctas; ++cta) {
    int cur = nv * cta, n = std::min(nv, count - cur);
    std::vector<int32_t> x(nv, 0);
    for(int j = 0; j < n; ++j) x[j] = data[cur + j];
    cta_scan_vec(x, nt, vt, partials[cta], init);
    for(int j = 0; j < n; ++j) data[cur + j] = x[j];
  }
}

////////////////////////////////////////////////////////////////////////////////
// LSD radix sort (common/cta_radix.hxx, vk/radix.hxx), keys-only as in the
// reference.  An optional int32 payload rides along with each key through the
// same ranks; the reference has no values, so that is an extension used to
// show which permutation the algorithm induces.

template<typename K> struct permute_t;
template<> struct permute_t<uint32_t> {
  typedef uint32_t U;
  static U to(uint32_t x) { return x; }
  static uint32_t from(U x) { return x; }
};
template<> struct permute_t<int32_t> {
  typedef uint32_t U;
  static U to(int32_t x) { return (uint32_t)x ^ 0x80000000u; }
  static int32_t from(U x) { return (int32_t)(x ^ 0x80000000u); }
};
template<> struct permute_t<float> {
  typedef uint32_t U;
  static U to(float f) {
    uint32_t y; memcpy(&y, &f, 4);
    return y ^ ((uint32_t)((int32_t)y >> 31) | 0x80000000u);
  }
  static float from(U x) {
    x ^= 0x80000000u;
    x ^= (uint32_t)((int32_t)x >> 31) & 0x7fffffffu;
    float f; memcpy(&f, &x, 4);
    return f;
  }
};
template<> struct permute_t<uint64_t> {
  typedef uint64_t U;
  static U to(uint64_t x) { return x; }
  static uint64_t from(U x) { return x; }
};

template<typename U>
inline uint32_t extract(U x, int bit, int num_bits) {
  return (uint32_t)((x >> bit) & (((U)1 << num_bits) - 1));
}

// Ranks of a tile's digits.  `digits` is in the ranking order the reference
// uses: for the ballot kind (8-bit) warp w's items are x[i] of lane l at
// warp-contiguous slot vt*32*w + 32*i + l, ranked in (i, lane) order and
// scanned over (digit, warp) (common/cta_radix.hxx:295-350); for the shared
// kind (4-bit) thread tid's items are the thread-contiguous slots vt*tid + i,
// ranked over (digit, thread) (common/cta_radix.hxx:155-205).  Both reduce to
// "earlier slot, same digit => lower rank" once the slot order is fixed, but
// the counts are formed exactly as the shaders form them.
// Returns, per slot, the scatter index, and per digit the tile-local start.
inline void rank_tile(const std::vector<uint32_t>& digits, int nt, int vt,
  int num_bits, std::vector<uint32_t>& scatter, std::vector<uint32_t>& digit_scan) {
  const int num_bins = 1 << num_bits;
  const int nv = nt * vt;
  scatter.assign(nv, 0);
  digit_scan.assign(num_bins, 0);
  if(8 == num_bits) {
    int num_warps = nt / warp_size;
    // hist32[warp][digit], incremented by the lowest lane of each match group.
    std::vector<uint32_t> hist(num_warps * num_bins, 0);
    for(int w = 0; w < num_warps; ++w)
      for(int i = 0; i < vt; ++i)
        for(int lane = 0; lane < warp_size; ++lane) {
          uint32_t d = digits[vt * warp_size * w + warp_size * i + lane];
          hist[w * num_bins + d] += 1;
        }
    // CTA exclusive scan over (digit, warp) in thread order.
    uint32_t run = 0;
    for(int d = 0; d < num_bins; ++d) {
      digit_scan[d] = run;
      for(int w = 0; w < num_warps; ++w) {
        uint32_t c = hist[w * num_bins + d];
        hist[w * num_bins + d] = run;
        run += c;
      }
    }
    // Second pass: offset + popc(lanemask_lt & match), leader bumps the bin.
    for(int w = 0; w < num_warps; ++w)
      for(int i = 0; i < vt; ++i) {
        const uint32_t* row = &digits[vt * warp_size * w + warp_size * i];
        for(int lane = 0; lane < warp_size; ++lane) {
          uint32_t lt = 0, all = 0;
          for(int l2 = 0; l2 < warp_size; ++l2)
            if(row[l2] == row[lane]) { all++; if(l2 < lane) lt++; }
          scatter[vt * warp_size * w + warp_size * i + lane] =
            hist[w * num_bins + row[lane]] + lt;
        }
        for(int lane = 0; lane < warp_size; ++lane) {
          bool leader = true;
          for(int l2 = 0; l2 < lane; ++l2) if(row[l2] == row[lane]) leader = false;
          if(leader) {
            uint32_t all = 0;
            for(int l2 = 0; l2 < warp_size; ++l2) all += row[l2] == row[lane];
            hist[w * num_bins + row[lane]] += all;
          }
        }
      }
  } else {
    // Per-thread histograms hist16[nt * digit + tid], scanned digit-major.
    std::vector<uint32_t> hist(nt * num_bins, 0);
    for(int tid = 0; tid < nt; ++tid)
      for(int i = 0; i < vt; ++i) hist[nt * digits[vt * tid + i] + tid]++;
    uint32_t run = 0;
    for(int k = 0; k < nt * num_bins; ++k) { uint32_t c = hist[k]; hist[k] = run; run += c; }
    for(int d = 0; d < num_bins; ++d) digit_scan[d] = hist[nt * d];
    for(int tid = 0; tid < nt; ++tid)
      for(int i = 0; i < vt; ++i)
        scatter[vt * tid + i] = hist[nt * digits[vt * tid + i] + tid]++;
  }
}

// Slot (ranking order) -> shared-memory index for the load layout the
// downsweep uses: shared_to_reg_warp for 8-bit (common/loadstore.hxx:74-85),
// shared_to_reg_thread for 4-bit (:27-40).  Both are the identity over
// original order, so a slot is simply the original in-tile offset.
inline int slot_to_offset(int slot) { return slot; }

// vk::radix_sort (vk/radix.hxx:195-470), multi-CTA branch and single-CTA
// branch, num_bits 4 or 8.  `vals` may be null.
template<typename K>
void radix_sort(K* data, int32_t* vals, int count, int nt, int vt, int num_bits) {
  typedef typename permute_t<K>::U U;
  const int nv = nt * vt;
  const int num_bins = 1 << num_bits;
  if(!count) return;
  int num_ctas = div_up(count, nv);

  if(1 == num_ctas) {
    // Whole sort in one tile.  The reference loops over 8 * sizeof(int)
    // = 32 bits here whatever the key width (vk/radix.hxx:254); for 64-bit keys
    // that is a defect and this restatement reproduces it.
    std::vector<U> smem(nv);
    std::vector<int32_t> sv(nv, 0);
    for(int j = 0; j < nv; ++j) {
      smem[j] = j < count ? permute_t<K>::to(data[j]) : (U)-1;
      if(vals && j < count) sv[j] = vals[j];
    }
    for(int bit = 0; bit < 32; bit += num_bits) {
      std::vector<uint32_t> digits(nv), scatter, dscan;
      for(int s = 0; s < nv; ++s) digits[s] = extract(smem[slot_to_offset(s)], bit, num_bits);
      rank_tile(digits, nt, vt, num_bits, scatter, dscan);
      std::vector<U> next(nv);
      std::vector<int32_t> nv2(nv);
      for(int s = 0; s < nv; ++s) { next[scatter[s]] = smem[s]; nv2[scatter[s]] = sv[s]; }
      smem = next;
      sv = nv2;
    }
    for(int j = 0; j < count; ++j) {
      data[j] = permute_t<K>::from(smem[j]);
      if(vals) vals[j] = sv[j];
    }
    return;
  }

  std::vector<K> data2_store(nv * num_ctas);
  std::vector<int32_t> vals2_store(nv * num_ctas);
  K* data2 = data2_store.data();
  int32_t* vals2 = vals2_store.data();
  std::vector<uint32_t> partials(num_bins * num_ctas);
  for(int bit = 0; bit < 8 * (int)sizeof(K); bit += num_bits) {
    // Upsweep (vk/radix.hxx:315-365): out-of-range keys count as all ones.
    for(int cta = 0; cta < num_ctas; ++cta) {
      int cur = nv * cta, n = count - cur;
      std::vector<uint32_t> cnt(num_bins, 0);
      for(int j = 0; j < nv; ++j) {
        U k = j < n ? permute_t<K>::to(data[cur + j]) : (U)-1;
        cnt[extract(k, bit, num_bits)]++;
      }
      for(int d = 0; d < num_bins; ++d) {
        int index = 8 == num_bits ? num_bins * cta + d : num_ctas * d + cta;
        partials[index] = cnt[d];
      }
    }
    // Scan of the counts: radix_scan_8 (vk/radix.hxx:13-185) for 8-bit is
    // the exclusive scan in (digit, frame) order over the [frame][digit]
    // layout; for 4-bit the layout is already [digit][cta] and vk::scan runs.
    if(8 == num_bits) {
      uint32_t run = 0;
      for(int d = 0; d < num_bins; ++d)
        for(int f = 0; f < num_ctas; ++f) {
          uint32_t c = partials[num_bins * f + d];
          partials[num_bins * f + d] = run;
          run += c;
        }
    } else {
      uint32_t run = 0;
      for(int k = 0; k < num_bins * num_ctas; ++k) {
        uint32_t c = partials[k]; partials[k] = run; run += c;
      }
    }
    // Downsweep (vk/radix.hxx:380-465).
    for(int cta = 0; cta < num_ctas; ++cta) {
      int cur = nv * cta, n = count - cur;
      std::vector<U> smem(nv);
      std::vector<int32_t> sv(nv, 0);
      for(int j = 0; j < nv; ++j) {
        smem[j] = j < n ? permute_t<K>::to(data[cur + j]) : (U)-1;
        if(vals && j < n) sv[j] = vals[cur + j];
      }
      std::vector<uint32_t> digits(nv), scatter, dscan;
      for(int s = 0; s < nv; ++s) digits[s] = extract(smem[slot_to_offset(s)], bit, num_bits);
      rank_tile(digits, nt, vt, num_bits, scatter, dscan);
      std::vector<U> sorted(nv);
      std::vector<int32_t> svs(nv);
      for(int s = 0; s < nv; ++s) { sorted[scatter[s]] = smem[s]; svs[scatter[s]] = sv[s]; }
      for(int offset = 0; offset < std::min(nv, n); ++offset) {
        uint32_t d = extract(sorted[offset], bit, num_bits);
        int index = 8 == num_bits ? num_bins * cta + d : num_ctas * d + cta;
        int dest = offset + (int)partials[index] - (int)dscan[d];
        data2[dest] = permute_t<K>::from(sorted[offset]);
        if(vals) vals2[dest] = svs[offset];
      }
    }
    // Copy back through the ping-pong pair (the reference swaps pointers; an
    // even pass count lands in `data`).
    std::swap_ranges(data, data + count, data2);
    if(vals) std::swap_ranges(vals, vals + count, vals2);
  }
}

}  // namespace emu

extern "C" {

// comp: 0 = std::less, 1 = std::greater.
#define EMU_COMP(comp, body)                                                   \
  do {                                                                         \
    if(comp) { auto c = std::greater<>(); body; }                              \
    else { auto c = std::less<>(); body; }                                     \
  } while(0)

// key_type: 0 = int32, 1 = uint32, 2 = float (mgpu_dtype_t codes).
int emu_mergesort(int key_type, void* keys, int32_t* vals, int count, int nt, int vt,
  int has_values, int sort_indices, int comp) {
  if(nt < 32 || (nt & (nt - 1)) || vt < 1 || vt > 30) return -1;
  switch(key_type) {
    case 0: EMU_COMP(comp, emu::mergesort((int32_t*)keys, vals, count, nt, vt,
      has_values, sort_indices, c)); return 0;
    case 1: EMU_COMP(comp, emu::mergesort((uint32_t*)keys, vals, count, nt, vt,
      has_values, sort_indices, c)); return 0;
    case 2: EMU_COMP(comp, emu::mergesort((float*)keys, vals, count, nt, vt,
      has_values, sort_indices, c)); return 0;
  }
  return -1;
}

int emu_merge(int key_type, const void* a_keys, const int32_t* a_vals, int a_count,
  const void* b_keys, const int32_t* b_vals, int b_count, void* c_keys, int32_t* c_vals,
  int nt, int vt, int has_values, int comp) {
  switch(key_type) {
    case 0: EMU_COMP(comp, emu::merge((const int32_t*)a_keys, a_vals, a_count,
      (const int32_t*)b_keys, b_vals, b_count, (int32_t*)c_keys, c_vals, nt, vt,
      has_values, c)); return 0;
    case 1: EMU_COMP(comp, emu::merge((const uint32_t*)a_keys, a_vals, a_count,
      (const uint32_t*)b_keys, b_vals, b_count, (uint32_t*)c_keys, c_vals, nt, vt,
      has_values, c)); return 0;
    case 2: EMU_COMP(comp, emu::merge((const float*)a_keys, a_vals, a_count,
      (const float*)b_keys, b_vals, b_count, (float*)c_keys, c_vals, nt, vt,
      has_values, c)); return 0;
  }
  return -1;
}

int emu_scan_exc_i32(int32_t* data, int count, int nt, int vt, int32_t init) {
  if(nt % emu::warp_size || nt / emu::warp_size > emu::warp_size) return -1;
  emu::scan(data, count, nt, vt, init);
  return 0;
}

// key_type: 0 int32, 1 uint32, 2 float, 4 uint64.  vals may be null.
int emu_radix_sort(int key_type, void* keys, int32_t* vals, int count, int nt, int vt,
  int num_bits) {
  if(num_bits != 4 && num_bits != 8) return -1;
  if(8 == num_bits && (nt < 256 || nt % emu::warp_size)) return -1;
  switch(key_type) {
    case 0: emu::radix_sort((int32_t*)keys, vals, count, nt, vt, num_bits); return 0;
    case 1: emu::radix_sort((uint32_t*)keys, vals, count, nt, vt, num_bits); return 0;
    case 2: emu::radix_sort((float*)keys, vals, count, nt, vt, num_bits); return 0;
    case 4: emu::radix_sort((uint64_t*)keys, vals, count, nt, vt, num_bits); return 0;
  }
  return -1;
}

// The reference's data source for its known-answer test: glibc rand()
// after the default seed (examples/vk_radix2/vk_radix2.cxx:25-27).
void emu_libc_rand_fill(uint32_t* out, int64_t n, unsigned seed) {
  srand(seed);
  for(int64_t i = 0; i < n; ++i) out[i] = (uint32_t)rand();
}

}  // extern "C"
