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
