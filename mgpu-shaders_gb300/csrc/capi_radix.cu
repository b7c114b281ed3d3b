// C ABI: mgpu_radix_sort for I32/U32/F32/I64/U64/F64 keys with 0-, 4- or
// 8-byte values.
#include "capi.hxx"
#include "mgpu/gb300/radix.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

namespace {

template<typename K, typename V>
mgpu_status_t run(mgpu_context* c, void* keys, void* vals, int64_t count, void* aux,
  size_t* aux_size) {
  typedef radix_tuning<sizeof(K)> T;
  return radix_sort_kv<T::nt, T::vt, T::min_blocks>(aux, aux_size, c->ctx, (K*)keys, (V*)vals,
    count);
}

}  // namespace

extern "C" mgpu_status_t mgpu_radix_sort(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  return dispatch_dtype(key_type, [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    if(val_bytes == 0) return run<K, no_values>(c, keys, nullptr, count, aux_data, aux_size);
    if(val_bytes == 4) return run<K, uint32_t>(c, keys, vals, count, aux_data, aux_size);
    return run<K, uint64_t>(c, keys, vals, count, aux_data, aux_size);
  });
}
