// C ABI: mgpu_mergesort and mgpu_mergesort_indices (dispatch by key width to
// the instantiations in capi_mergesort_32.cu / capi_mergesort_64.cu).
#include "capi.hxx"

mgpu_status_t mergesort_w32(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, mgpu_comp_t comp, int indices, void* aux, size_t* aux_size);
mgpu_status_t mergesort_w64(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, mgpu_comp_t comp, int indices, void* aux, size_t* aux_size);

namespace {

mgpu_status_t dispatch(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, mgpu_comp_t comp, int indices, void* aux, size_t* aux_size) {
  if(comp != MGPU_LESS && comp != MGPU_GREATER) return MGPU_ERR_INVALID_ARG;
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  if(indices && count > INT32_MAX) return MGPU_ERR_INVALID_ARG;
  switch(key_type) {
    case MGPU_I32: case MGPU_U32: case MGPU_F32:
      return mergesort_w32(c, key_type, keys, val_bytes, vals, count, comp, indices, aux,
        aux_size);
    case MGPU_I64: case MGPU_U64: case MGPU_F64:
      return mergesort_w64(c, key_type, keys, val_bytes, vals, count, comp, indices, aux,
        aux_size);
  }
  return MGPU_ERR_INVALID_ARG;
}

}  // namespace

extern "C" {

mgpu_status_t mgpu_mergesort(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, mgpu_comp_t comp, void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  return dispatch(c, key_type, keys, val_bytes, vals, count, comp, 0, aux_data, aux_size);
}

mgpu_status_t mgpu_mergesort_indices(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int32_t* indices, int64_t count, mgpu_comp_t comp, void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  return dispatch(c, key_type, keys, 4, indices, count, comp, 1, aux_data, aux_size);
}

}  // extern "C"
