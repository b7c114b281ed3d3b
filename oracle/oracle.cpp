// Test infrastructure, not product code: the host oracle for the mgpu primitives.
//
// This file restates, with host std:: algorithms, the results that the
// reference library (seanbaxter/mgpu-shaders, inc/mgpu) computes on the GPU.
// Only tests, the smoke check and the CPU-baseline leg of bench.py may load it.
// The product library never links or calls anything here.
//
// Semantics followed (reference file:line):
//  * mergesort_kv / mergesort_keys / mergesort_indices (vk/mergesort.hxx:10-103):
//    a stable sort by `comp`.  Stability comes from merge_path's bounds_lower
//    predicate `!comp(b, a)` (common/cta_merge.hxx:23-25, :48) and from the
//    strict-swap odd-even network (common/sort_networks.hxx:17,30), so the
//    result is std::stable_sort.  mergesort_indices sets value = original index
//    (common/kernel_mergesort.hxx:43-49).
//  * merge (vk/merge.hxx:12-59): std::merge, A first on ties (bounds_lower).
//  * radix_sort (vk/radix.hxx:195-470): LSD order over
//    radix_permute_t::to_radix_bits (common/cta_radix.hxx:6-64); every digit
//    pass is stable (ballot ranking in lane-then-item order,
//    cta_radix.hxx:293-296,340-345), so the result is std::stable_sort by the
//    radix bits.  For float keys that is bit order: -0.0 before +0.0, NaNs
//    placed by their bit patterns.  Values (an addition over the reference,
//    which sorts keys only) travel with their keys.
//  * scan (vk/scan.hxx:10-115): exclusive plus-scan.  Integer sums wrap in
//    two's complement exactly as 32-bit GPU adds do, so the oracle adds in the
//    unsigned type and reinterprets.  Float scans accumulate in double.
//
// Type codes match include/mgpu_gb300.h (mgpu_dtype_t).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <numeric>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

enum dtype_t { I32 = 0, U32 = 1, F32 = 2, I64 = 3, U64 = 4, F64 = 5 };
enum op_t { OP_PLUS = 0, OP_MAX = 1, OP_MIN = 2 };

// Order-preserving map of a key to unsigned bits
// (reference: radix_permute_t::to_radix_bits, common/cta_radix.hxx:11-35).
template<typename K> struct radix_traits;
template<> struct radix_traits<uint32_t> {
  typedef uint32_t bits_t;
  static bits_t to_bits(uint32_t x) { return x; }
};
template<> struct radix_traits<uint64_t> {
  typedef uint64_t bits_t;
  static bits_t to_bits(uint64_t x) { return x; }
};
template<> struct radix_traits<int32_t> {
  typedef uint32_t bits_t;
  static bits_t to_bits(int32_t x) { return (uint32_t)x ^ 0x80000000u; }
};
template<> struct radix_traits<int64_t> {
  typedef uint64_t bits_t;
  static bits_t to_bits(int64_t x) { return (uint64_t)x ^ 0x8000000000000000ull; }
};
template<> struct radix_traits<float> {
  typedef uint32_t bits_t;
  static bits_t to_bits(float f) {
    uint32_t y; memcpy(&y, &f, 4);
    uint32_t mask = (uint32_t)((int32_t)y >> 31) | 0x80000000u;
    return y ^ mask;
  }
};
template<> struct radix_traits<double> {
  typedef uint64_t bits_t;
  static bits_t to_bits(double f) {
    uint64_t y; memcpy(&y, &f, 8);
    uint64_t mask = (uint64_t)((int64_t)y >> 63) | 0x8000000000000000ull;
    return y ^ mask;
  }
};

// Opaque value payload of 0, 4 or 8 bytes.
template<int B> struct payload_t { uint8_t b[B]; };
template<> struct payload_t<0> {};

template<typename K, int VB> struct item_t {
  K key;
  payload_t<VB> val;
};

template<typename K, int VB>
void gather_items(const K* keys, const void* vals, int64_t n,
  std::vector<item_t<K, VB>>& items) {
  items.resize(n);
  for(int64_t i = 0; i < n; ++i) {
    items[i].key = keys[i];
    if constexpr(VB > 0) memcpy(items[i].val.b, (const uint8_t*)vals + VB * i, VB);
  }
}

template<typename K, int VB>
void scatter_items(const std::vector<item_t<K, VB>>& items, K* keys, void* vals) {
  int64_t n = (int64_t)items.size();
  for(int64_t i = 0; i < n; ++i) {
    keys[i] = items[i].key;
    if constexpr(VB > 0) memcpy((uint8_t*)vals + VB * i, items[i].val.b, VB);
  }
}

// mode 0: comparator less, 1: comparator greater, 2: radix-bits ascending.
template<typename K>
struct key_comp_t {
  int mode;
  bool operator()(const K& a, const K& b) const {
    if(mode == 0) return a < b;
    if(mode == 1) return b < a;
    return radix_traits<K>::to_bits(a) < radix_traits<K>::to_bits(b);
  }
};

template<typename K, int VB>
void stable_sort_kv(K* keys, void* vals, int64_t n, int mode) {
  std::vector<item_t<K, VB>> items;
  gather_items<K, VB>(keys, vals, n, items);
  key_comp_t<K> kc { mode };
  std::stable_sort(items.begin(), items.end(),
    [&](const item_t<K, VB>& a, const item_t<K, VB>& b) { return kc(a.key, b.key); });
  scatter_items<K, VB>(items, keys, vals);
}

// Parallel stable sort over `threads` std::threads: each thread stable-sorts
// one contiguous chunk, then adjacent runs are merged pairwise (std::merge is
// stable, A first) in log2(threads) rounds.  Same result as stable_sort_kv.
template<typename K, int VB>
void stable_sort_kv_parallel(K* keys, void* vals, int64_t n, int mode, int threads) {
  typedef item_t<K, VB> it_t;
  if(threads < 1) threads = 1;
  std::vector<it_t> a(n), b(n);
  key_comp_t<K> kc { mode };
  auto less = [&](const it_t& x, const it_t& y) { return kc(x.key, y.key); };
  std::vector<int64_t> bounds(threads + 1);
  for(int t = 0; t <= threads; ++t) bounds[t] = n * t / threads;
  {
    std::vector<std::thread> pool;
    for(int t = 0; t < threads; ++t)
      pool.emplace_back([&, t] {
        for(int64_t i = bounds[t]; i < bounds[t + 1]; ++i) {
          a[i].key = keys[i];
          if constexpr(VB > 0) memcpy(a[i].val.b, (const uint8_t*)vals + VB * i, VB);
        }
        std::stable_sort(a.begin() + bounds[t], a.begin() + bounds[t + 1], less);
      });
    for(auto& th : pool) th.join();
  }
  std::vector<int64_t> runs = bounds;
  while(runs.size() > 2) {
    std::vector<int64_t> next;
    std::vector<std::thread> pool;
    size_t num_runs = runs.size() - 1;
    for(size_t r = 0; r < num_runs; r += 2) {
      next.push_back(runs[r]);
      if(r + 1 < num_runs) {
        int64_t s0 = runs[r], s1 = runs[r + 1], s2 = runs[r + 2];
        pool.emplace_back([&, s0, s1, s2] {
          std::merge(a.begin() + s0, a.begin() + s1, a.begin() + s1,
            a.begin() + s2, b.begin() + s0, less);
        });
      } else {
        int64_t s0 = runs[r], s1 = runs[r + 1];
        pool.emplace_back([&, s0, s1] {
          std::copy(a.begin() + s0, a.begin() + s1, b.begin() + s0);
        });
      }
    }
    next.push_back(runs.back());
    for(auto& th : pool) th.join();
    a.swap(b);
    runs = next;
  }
  {
    std::vector<std::thread> pool;
    for(int t = 0; t < threads; ++t)
      pool.emplace_back([&, t] {
        for(int64_t i = bounds[t]; i < bounds[t + 1]; ++i) {
          keys[i] = a[i].key;
          if constexpr(VB > 0) memcpy((uint8_t*)vals + VB * i, a[i].val.b, VB);
        }
      });
    for(auto& th : pool) th.join();
  }
}

template<typename K, int VB>
void merge_kv(const K* ak, const void* av, int64_t an, const K* bk,
  const void* bv, int64_t bn, K* ck, void* cv, int mode) {
  std::vector<item_t<K, VB>> a, b, c(an + bn);
  gather_items<K, VB>(ak, av, an, a);
  gather_items<K, VB>(bk, bv, bn, b);
  key_comp_t<K> kc { mode };
  std::merge(a.begin(), a.end(), b.begin(), b.end(), c.begin(),
    [&](const item_t<K, VB>& x, const item_t<K, VB>& y) { return kc(x.key, y.key); });
  scatter_items<K, VB>(c, ck, cv);
}

// Integer scan with two's-complement wrap: accumulate in the unsigned type.
template<typename T>
T int_op(T a, T b, int op) {
  typedef typename std::make_unsigned<T>::type U;
  if(op == OP_PLUS) return (T)((U)a + (U)b);
  if(op == OP_MAX) return a > b ? a : b;
  return a < b ? a : b;
}

template<typename T>
void scan_int(const T* in, T* out, int64_t n, int exclusive, T init, int op) {
  T acc = init;
  for(int64_t i = 0; i < n; ++i) {
    T x = in[i];
    if(exclusive) { out[i] = acc; acc = int_op(acc, x, op); }
    else { acc = int_op(acc, x, op); out[i] = acc; }
  }
}

template<typename T>
double fp_op(double a, double b, int op) {
  if(op == OP_PLUS) return a + b;
  if(op == OP_MAX) return a > b ? a : b;
  return a < b ? a : b;
}

// Float scan accumulated in double; out_abs (optional) gets the prefix of |x|,
// which scales the tolerance of a float32 comparison.
template<typename T>
void scan_fp(const T* in, double* out, double* out_abs, int64_t n, int exclusive,
  double init, int op) {
  double acc = init, acc_abs = fabs(init);
  for(int64_t i = 0; i < n; ++i) {
    double x = (double)in[i];
    if(exclusive) {
      out[i] = acc;
      if(out_abs) out_abs[i] = acc_abs;
      acc = fp_op<T>(acc, x, op);
      acc_abs += fabs(x);
    } else {
      acc = fp_op<T>(acc, x, op);
      acc_abs += fabs(x);
      out[i] = acc;
      if(out_abs) out_abs[i] = acc_abs;
    }
  }
}

template<typename F>
int dispatch_key(int key_type, F f) {
  switch(key_type) {
    case I32: f((int32_t*)nullptr); return 0;
    case U32: f((uint32_t*)nullptr); return 0;
    case F32: f((float*)nullptr); return 0;
    case I64: f((int64_t*)nullptr); return 0;
    case U64: f((uint64_t*)nullptr); return 0;
    case F64: f((double*)nullptr); return 0;
  }
  return -1;
}

template<typename F>
int dispatch_kv(int key_type, int val_bytes, F f) {
  return dispatch_key(key_type, [&](auto* kp) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    if(val_bytes == 0) f((K*)nullptr, std::integral_constant<int, 0>());
    else if(val_bytes == 4) f((K*)nullptr, std::integral_constant<int, 4>());
    else if(val_bytes == 8) f((K*)nullptr, std::integral_constant<int, 8>());
  });
}

int64_t segment_begin(const int64_t* offsets, int64_t s) { return offsets[s]; }

}  // namespace

extern "C" {

// Stable sort of (keys, vals) by comparator: mode 0 = less, 1 = greater,
// 2 = radix-bits ascending (the radix_sort order).
int oracle_sort(int key_type, void* keys, int val_bytes, void* vals, int64_t n,
  int mode) {
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return -1;
  return dispatch_kv(key_type, val_bytes, [&](auto* kp, auto vb) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    stable_sort_kv<K, decltype(vb)::value>((K*)keys, vals, n, mode);
  });
}

int oracle_sort_parallel(int key_type, void* keys, int val_bytes, void* vals,
  int64_t n, int mode, int threads) {
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return -1;
  return dispatch_kv(key_type, val_bytes, [&](auto* kp, auto vb) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    stable_sort_kv_parallel<K, decltype(vb)::value>((K*)keys, vals, n, mode, threads);
  });
}

// std::merge of two sorted sequences, A first on ties.  mode 0 less, 1 greater.
int oracle_merge(int key_type, const void* a_keys, const void* a_vals, int64_t a_n,
  const void* b_keys, const void* b_vals, int64_t b_n, void* c_keys, void* c_vals,
  int val_bytes, int mode) {
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return -1;
  return dispatch_kv(key_type, val_bytes, [&](auto* kp, auto vb) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    merge_kv<K, decltype(vb)::value>((const K*)a_keys, a_vals, a_n,
      (const K*)b_keys, b_vals, b_n, (K*)c_keys, c_vals, mode);
  });
}

// Integer scans (I32/U32/I64/U64): out has the input's type, wrap-around
// arithmetic.  `init` points to one element of the same type.
int oracle_scan_int(int type, const void* in, void* out, int64_t n, int exclusive,
  const void* init, int op) {
  switch(type) {
    case I32: scan_int<int32_t>((const int32_t*)in, (int32_t*)out, n, exclusive,
      *(const int32_t*)init, op); return 0;
    case U32: scan_int<uint32_t>((const uint32_t*)in, (uint32_t*)out, n, exclusive,
      *(const uint32_t*)init, op); return 0;
    case I64: scan_int<int64_t>((const int64_t*)in, (int64_t*)out, n, exclusive,
      *(const int64_t*)init, op); return 0;
    case U64: scan_int<uint64_t>((const uint64_t*)in, (uint64_t*)out, n, exclusive,
      *(const uint64_t*)init, op); return 0;
  }
  return -1;
}

// Float scans (F32/F64) accumulated in double; out and out_abs are double.
int oracle_scan_fp(int type, const void* in, double* out, double* out_abs, int64_t n,
  int exclusive, double init, int op) {
  if(type == F32) { scan_fp<float>((const float*)in, out, out_abs, n, exclusive, init, op); return 0; }
  if(type == F64) { scan_fp<double>((const double*)in, out, out_abs, n, exclusive, init, op); return 0; }
  return -1;
}

// Segmented stable sort: each segment [offsets[s], offsets[s+1]) is sorted on
// its own (mode as in oracle_sort).
int oracle_segmented_sort(int key_type, void* keys, int val_bytes, void* vals,
  const int64_t* offsets, int64_t num_segments, int mode) {
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return -1;
  return dispatch_kv(key_type, val_bytes, [&](auto* kp, auto vb) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    constexpr int VB = decltype(vb)::value;
    for(int64_t s = 0; s < num_segments; ++s) {
      int64_t b = segment_begin(offsets, s), e = offsets[s + 1];
      stable_sort_kv<K, VB>((K*)keys + b, VB ? (uint8_t*)vals + VB * b : nullptr,
        e - b, mode);
    }
  });
}

// Segmented integer scan: the scan restarts with `init` at every segment head.
int oracle_segmented_scan_int(int type, const void* in, void* out,
  const int64_t* offsets, int64_t num_segments, int exclusive, const void* init,
  int op) {
  for(int64_t s = 0; s < num_segments; ++s) {
    int64_t b = offsets[s], n = offsets[s + 1] - b;
    int rc = 0;
    switch(type) {
      case I32: scan_int<int32_t>((const int32_t*)in + b, (int32_t*)out + b, n,
        exclusive, *(const int32_t*)init, op); break;
      case U32: scan_int<uint32_t>((const uint32_t*)in + b, (uint32_t*)out + b, n,
        exclusive, *(const uint32_t*)init, op); break;
      case I64: scan_int<int64_t>((const int64_t*)in + b, (int64_t*)out + b, n,
        exclusive, *(const int64_t*)init, op); break;
      case U64: scan_int<uint64_t>((const uint64_t*)in + b, (uint64_t*)out + b, n,
        exclusive, *(const uint64_t*)init, op); break;
      default: rc = -1;
    }
    if(rc) return rc;
  }
  return 0;
}

// Host restatement of radix_permute_t::to_radix_bits for 4- and 8-byte keys
// (common/cta_radix.hxx:11-35).  Writes n unsigned words of the key's width.
int oracle_to_radix_bits(int key_type, const void* keys, void* bits, int64_t n) {
  return dispatch_key(key_type, [&](auto* kp) {
    typedef std::remove_pointer_t<decltype(kp)> K;
    typedef typename radix_traits<K>::bits_t B;
    for(int64_t i = 0; i < n; ++i)
      ((B*)bits)[i] = radix_traits<K>::to_bits(((const K*)keys)[i]);
  });
}

// Parallel scan over `threads` threads (two passes: chunk sums, then chunk
// scans with carry-in).  Integer types only; used as the CPU baseline.
int oracle_scan_int_parallel(int type, const void* in, void* out, int64_t n,
  int exclusive, int threads) {
  if(type != I32 && type != U32) return -1;
  if(threads < 1) threads = 1;
  const uint32_t* x = (const uint32_t*)in;
  uint32_t* y = (uint32_t*)out;
  std::vector<uint32_t> sums(threads + 1, 0);
  std::vector<std::thread> pool;
  for(int t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      int64_t b = n * t / threads, e = n * (t + 1) / threads;
      uint32_t s = 0;
      for(int64_t i = b; i < e; ++i) s += x[i];
      sums[t + 1] = s;
    });
  for(auto& th : pool) th.join();
  pool.clear();
  for(int t = 0; t < threads; ++t) sums[t + 1] += sums[t];
  for(int t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      int64_t b = n * t / threads, e = n * (t + 1) / threads;
      uint32_t acc = sums[t];
      if(exclusive) for(int64_t i = b; i < e; ++i) { uint32_t v = x[i]; y[i] = acc; acc += v; }
      else for(int64_t i = b; i < e; ++i) { acc += x[i]; y[i] = acc; }
    });
  for(auto& th : pool) th.join();
  return 0;
}

}  // extern "C"
