// C ABI: context lifetime, memory, synchronisation and profiling.
#include "capi.hxx"

#include <cstdio>
#include <new>

extern "C" {

mgpu_status_t mgpu_context_create(int device, void* stream, mgpu_context_t** out) {
  if(!out) return MGPU_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if(cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return MGPU_ERR_CUDA;
  mgpu_context* c = new(std::nothrow) mgpu_context(device, (cudaStream_t)stream);
  if(!c) return MGPU_ERR_OOM;
  if(c->ctx.init_status != MGPU_OK) {
    mgpu_status_t s = c->ctx.init_status;
    delete c;
    return s;
  }
  *out = c;
  return MGPU_OK;
}

mgpu_status_t mgpu_context_destroy(mgpu_context_t* c) {
  if(!c) return MGPU_ERR_INVALID_ARG;
  cudaSetDevice(c->ctx.device);
  delete c;
  return MGPU_OK;
}

mgpu_status_t mgpu_context_set_stream(mgpu_context_t* c, void* stream) {
  MGPU_CHECK_CTX(c);
  c->ctx.stream = stream ? (cudaStream_t)stream : c->ctx.owned_stream;
  if(!c->ctx.stream) return MGPU_ERR_INVALID_ARG;
  return MGPU_OK;
}

void* mgpu_context_stream(mgpu_context_t* c) { return c ? (void*)c->ctx.stream : nullptr; }

mgpu_status_t mgpu_synchronize(mgpu_context_t* c) {
  MGPU_CHECK_CTX(c);
  return c->ctx.synchronize();
}

const char* mgpu_status_string(mgpu_status_t s) {
  switch(s) {
    case MGPU_OK: return "ok";
    case MGPU_ERR_INVALID_ARG: return "invalid argument";
    case MGPU_ERR_OOM: return "out of device memory";
    case MGPU_ERR_LOOKBACK_TIMEOUT: return "a bounded device-side wait timed out";
    case MGPU_ERR_CUDA: return "CUDA runtime error";
    case MGPU_ERR_UNSUPPORTED: return "unsupported type or size";
    case MGPU_ERR_BUDGET: return "request exceeds the memory budget";
    case MGPU_ERR_NOT_READY: return "not ready";
  }
  return "unknown status";
}

const char* mgpu_last_error(mgpu_context_t* c) {
  return c ? c->ctx.last_error.c_str() : "null context";
}

int mgpu_sm_count(mgpu_context_t* c) { return c ? c->ctx.sm_count : 0; }

mgpu_status_t mgpu_alloc_gpu(mgpu_context_t* c, size_t bytes, void** out) {
  MGPU_CHECK_CTX(c);
  if(!out) return MGPU_ERR_INVALID_ARG;
  *out = c->ctx.alloc_gpu(bytes);
  return *out ? MGPU_OK : MGPU_ERR_OOM;
}

mgpu_status_t mgpu_alloc_cpu(mgpu_context_t* c, size_t bytes, void** out) {
  MGPU_CHECK_CTX(c);
  if(!out) return MGPU_ERR_INVALID_ARG;
  *out = c->ctx.alloc_cpu(bytes);
  return *out ? MGPU_OK : MGPU_ERR_OOM;
}

mgpu_status_t mgpu_free(mgpu_context_t* c, void* p) {
  MGPU_CHECK_CTX(c);
  return c->ctx.free(p);
}

mgpu_status_t mgpu_memcpy(mgpu_context_t* c, void* dest, const void* src, size_t bytes) {
  MGPU_CHECK_CTX(c);
  if(!bytes) return MGPU_OK;
  if(!dest || !src) return MGPU_ERR_INVALID_ARG;
  return c->ctx.memcpy(dest, src, bytes);
}

mgpu_status_t mgpu_memset(mgpu_context_t* c, void* dest, int value, size_t bytes) {
  MGPU_CHECK_CTX(c);
  if(!bytes) return MGPU_OK;
  if(!dest) return MGPU_ERR_INVALID_ARG;
  return c->ctx.check(cudaMemsetAsync(dest, value, bytes, c->ctx.stream)) ? MGPU_ERR_CUDA : MGPU_OK;
}

mgpu_status_t mgpu_profile_enable(mgpu_context_t* c, int enable) {
  MGPU_CHECK_CTX(c);
  c->ctx.profiling = enable != 0;
  return MGPU_OK;
}

mgpu_status_t mgpu_profile_read(mgpu_context_t* c, char* names, size_t names_bytes,
  int64_t* launches, double* total_ms, int capacity, int* num) {
  MGPU_CHECK_CTX(c);
  mgpu_status_t s = c->ctx.collect_profile();
  if(s) return s;
  int i = 0;
  size_t used = 0;
  if(names && names_bytes) names[0] = 0;
  for(auto& kv : c->ctx.profile) {
    if(i >= capacity) break;
    if(launches) launches[i] = kv.second.first;
    if(total_ms) total_ms[i] = kv.second.second;
    if(names && used + kv.first.size() + 2 <= names_bytes) {
      used += snprintf(names + used, names_bytes - used, "%s\n", kv.first.c_str());
    }
    ++i;
  }
  if(num) *num = i;
  c->ctx.profile.clear();
  return MGPU_OK;
}

int64_t mgpu_launch_count(mgpu_context_t* c) { return c ? c->ctx.launches : 0; }

}  // extern "C"

// ---- CUDA graphs ----

struct mgpu_graph {
  cudaGraphExec_t exec = nullptr;
  int device = 0;
};

extern "C" {

mgpu_status_t mgpu_graph_begin(mgpu_context_t* c) {
  MGPU_CHECK_CTX(c);
  if(c->ctx.capturing) return MGPU_ERR_INVALID_ARG;
  if(c->ctx.check(cudaStreamBeginCapture(c->ctx.stream, cudaStreamCaptureModeThreadLocal)))
    return MGPU_ERR_CUDA;
  c->ctx.capturing = true;
  return MGPU_OK;
}

mgpu_status_t mgpu_graph_end(mgpu_context_t* c, mgpu_graph_t** out) {
  MGPU_CHECK_CTX(c);
  if(!out || !c->ctx.capturing) return MGPU_ERR_INVALID_ARG;
  *out = nullptr;
  c->ctx.capturing = false;
  cudaGraph_t g = nullptr;
  if(c->ctx.check(cudaStreamEndCapture(c->ctx.stream, &g))) return MGPU_ERR_CUDA;
  mgpu_graph* h = new(std::nothrow) mgpu_graph;
  if(!h) { cudaGraphDestroy(g); return MGPU_ERR_OOM; }
  h->device = c->ctx.device;
  cudaError_t e = cudaGraphInstantiate(&h->exec, g, 0);
  cudaGraphDestroy(g);
  if(c->ctx.check(e)) { delete h; return MGPU_ERR_CUDA; }
  *out = h;
  return MGPU_OK;
}

mgpu_status_t mgpu_graph_launch(mgpu_context_t* c, mgpu_graph_t* g) {
  MGPU_CHECK_CTX(c);
  if(!g || g->device != c->ctx.device) return MGPU_ERR_INVALID_ARG;
  return c->ctx.check(cudaGraphLaunch(g->exec, c->ctx.stream)) ? MGPU_ERR_CUDA : MGPU_OK;
}

mgpu_status_t mgpu_graph_destroy(mgpu_graph_t* g) {
  if(!g) return MGPU_ERR_INVALID_ARG;
  cudaSetDevice(g->device);
  cudaGraphExecDestroy(g->exec);
  delete g;
  return MGPU_OK;
}

mgpu_status_t mgpu_cache_reserve(mgpu_context_t* c, size_t bytes) {
  MGPU_CHECK_CTX(c);
  if(c->ctx.capturing) return MGPU_ERR_INVALID_ARG;
  return c->ctx.cache_allocate(bytes) || !bytes ? MGPU_OK : MGPU_ERR_OOM;
}

}  // extern "C"
