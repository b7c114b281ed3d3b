// C ABI: radix sort instantiations for 32-bit keys, every tuned variant.
#include "capi.hxx"
#include "mgpu/gb300/radix.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

// Shapes are given for 4-byte values (and keys-only); with 8-byte values
// the staged elements are twice as wide, so a tile holds half the keys.
template<int NT, int VT4, int MINB, bool DEV = false, typename K, typename V>
mgpu_status_t sort_shape(mgpu_context* c, K* keys, V* vals, int64_t count, void* aux,
  size_t* aux_size, const int64_t* d_count) {
  constexpr int VT = radix_elem_bytes<K, V>() == 8 ? VT4 / 2 : VT4;
  return radix_sort_kv<NT, VT, MINB, DEV>(aux, aux_size, c->ctx, keys, vals, count, d_count);
}

// A 4-bit-digit shape (eight passes over 4-byte keys), CTAs per SM as the
// C++ knobs derive them.
template<int NT, int VT4, typename K, typename V>
mgpu_status_t sort_shape4(mgpu_context* c, K* keys, V* vals, int64_t count, void* aux,
  size_t* aux_size) {
  constexpr int VT = radix_elem_bytes<K, V>() == 8 ? VT4 / 2 : VT4;
  typedef radix_knobs<K, V, NT, VT, 4> R;
  return radix_sort_kv<R::NT, R::VT, R::MINB, false, 4>(aux, aux_size, c->ctx, keys, vals, count);
}

mgpu_status_t radix_sort_w32(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, int variant, void* aux, size_t* aux_size, const int64_t* d_count) {
  auto go_key = [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    auto go = [&](auto* vp) -> mgpu_status_t {
      typedef std::remove_pointer_t<decltype(vp)> V;
      K* k = (K*)keys;
      V* v = (V*)vals;
      if(d_count)   // count read on the device: the default shape
        return sort_shape<384, 20, 3, true>(c, k, v, count, aux, aux_size, d_count);
      switch(variant) {
        case 1: return sort_shape<256, 32, 3>(c, k, v, count, aux, aux_size, nullptr);
        case 2: return sort_shape<256, 24, 3>(c, k, v, count, aux, aux_size, nullptr);
        case 3: return sort_shape4<256, 16>(c, k, v, count, aux, aux_size);
        case 4: return sort_shape4<128, 16>(c, k, v, count, aux, aux_size);
        default: return sort_shape<384, 20, 3>(c, k, v, count, aux, aux_size, nullptr);
      }
    };
    if(val_bytes == 0) return go((no_values*)nullptr);
    if(val_bytes == 4) return go((uint32_t*)nullptr);
    return go((uint64_t*)nullptr);
  };
  switch(key_type) {
    case MGPU_I32: return go_key((int32_t*)nullptr);
    case MGPU_U32: return go_key((uint32_t*)nullptr);
    case MGPU_F32: return go_key((float*)nullptr);
    default: break;
  }
  return MGPU_ERR_INVALID_ARG;
}
