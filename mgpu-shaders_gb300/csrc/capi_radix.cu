// C ABI: mgpu_radix_sort dispatch (key type, value width, tuned variant) to
// the instantiations in capi_radix_32.cu (4-byte keys) and capi_radix_64.cu
// (8-byte keys).
#include "capi.hxx"
#include "variants.hxx"

mgpu_status_t radix_sort_w32(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, int variant, void* aux, size_t* aux_size, const int64_t* d_count);
mgpu_status_t radix_sort_w64(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, int variant, void* aux, size_t* aux_size, const int64_t* d_count);

static mgpu_status_t radix_dispatch(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, const int64_t* d_count, void* aux_data,
  size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  int variant = c->ctx.tuning.lookup(mgpu::gb300::prim_radix, key_type, val_bytes, count);
  switch(key_type) {
    case MGPU_I32: case MGPU_U32: case MGPU_F32:
      return radix_sort_w32(c, key_type, keys, val_bytes, vals, count, variant, aux_data,
        aux_size, d_count);
    case MGPU_I64: case MGPU_U64: case MGPU_F64:
      return radix_sort_w64(c, key_type, keys, val_bytes, vals, count, variant, aux_data,
        aux_size, d_count);
  }
  return MGPU_ERR_INVALID_ARG;
}

extern "C" mgpu_status_t mgpu_radix_sort(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, void* aux_data, size_t* aux_size) {
  return radix_dispatch(c, key_type, keys, val_bytes, vals, count, nullptr, aux_data, aux_size);
}

extern "C" mgpu_status_t mgpu_radix_sort_count_on_device(mgpu_context_t* c,
  mgpu_dtype_t key_type, void* keys, int val_bytes, void* vals, int64_t max_count,
  const int64_t* d_count, void* aux_data, size_t* aux_size) {
  if(!d_count) return MGPU_ERR_INVALID_ARG;
  return radix_dispatch(c, key_type, keys, val_bytes, vals, max_count, d_count, aux_data,
    aux_size);
}
