/*
 * mgpu_gb300.h - C ABI of the GB300 (sm_103a) data-parallel primitives.
 *
 * These entry points replace the host calls of seanbaxter/mgpu-shaders'
 * Vulkan API (the inc/mgpu/vk headers).  Every primitive keeps the reference's
 * two-phase auxiliary-memory protocol:
 *
 *   size_t aux_size = 0;
 *   mgpu_radix_sort(ctx, ..., NULL, &aux_size);   // only adds the bytes needed
 *   void* aux = <device allocation of aux_size bytes>;
 *   mgpu_radix_sort(ctx, ..., aux, &aux_size);    // runs; aux_size = capacity
 *
 * as in vk/merge.hxx:30-34, vk/mergesort.hxx:35-41, vk/scan.hxx:19-22,54-59
 * and vk/radix.hxx:288-302 (where `aux_data == nullptr` only grows aux_size).
 * aux must start on a 16-byte boundary (device allocations do); a misaligned
 * aux or one smaller than the sizing pass asked for is MGPU_ERR_INVALID_ARG.
 * With aux_size == NULL the context's grow-only device cache supplies the
 * memory (the reference's memcache_t, vk/context.hxx:110-134).
 *
 * All work is enqueued on the context's CUDA stream and returns without a
 * host synchronisation (the reference records into a command buffer and runs
 * on submit, src/vk/context.cxx:336-345).  Buffers are caller-owned device
 * pointers.  Sorts are in place, as in the reference.  mgpu_synchronize()
 * waits for the stream and reports device-side errors (a bounded look-back
 * wait that gave up returns MGPU_ERR_LOOKBACK_TIMEOUT).  No entry point
 * throws.  A context is used by one host thread at a time.
 */
#ifndef MGPU_GB300_H
#define MGPU_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define MGPU_API __attribute__((visibility("default")))
#else
#define MGPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mgpu_status_t {
  MGPU_OK = 0,
  MGPU_ERR_INVALID_ARG = 1,      /* bad pointer, size, type or aux capacity */
  MGPU_ERR_OOM = 2,              /* device allocation failed */
  MGPU_ERR_LOOKBACK_TIMEOUT = 3, /* a bounded device-side wait gave up */
  MGPU_ERR_CUDA = 4,             /* a CUDA runtime call failed */
  MGPU_ERR_UNSUPPORTED = 5,      /* type/size combination not built */
  MGPU_ERR_BUDGET = 6,           /* serving: request exceeds the HBM budget */
  MGPU_ERR_NOT_READY = 7         /* serving: request still in flight */
} mgpu_status_t;

/* Element types.  Codes are shared with the host oracle. */
typedef enum mgpu_dtype_t {
  MGPU_I32 = 0,
  MGPU_U32 = 1,
  MGPU_F32 = 2,
  MGPU_I64 = 3,
  MGPU_U64 = 4,
  MGPU_F64 = 5
} mgpu_dtype_t;

/* Comparators of the merge family: std::less / std::greater. */
typedef enum mgpu_comp_t { MGPU_LESS = 0, MGPU_GREATER = 1 } mgpu_comp_t;

/* Scan/reduce operators (reference: op_t template argument, vk/scan.hxx:10-13). */
typedef enum mgpu_op_t { MGPU_PLUS = 0, MGPU_MAX = 1, MGPU_MIN = 2 } mgpu_op_t;

/* scan_type_t (reference: common/cta_scan.hxx:63-66). */
typedef enum mgpu_scan_type_t { MGPU_SCAN_EXC = 0, MGPU_SCAN_INC = 1 } mgpu_scan_type_t;

typedef struct mgpu_context mgpu_context_t;

/* ---- context (replaces context_t / cmd_buffer_t / memcache_t,
 *      vk/context.hxx:11-134, src/vk/context.cxx:15-439) ---- */

/* Creates a context on `device`.  `stream` is a cudaStream_t to enqueue on,
 * or NULL for a non-blocking stream the context creates and owns (pass
 * cudaStreamLegacy to order work with the legacy default stream). */
MGPU_API mgpu_status_t mgpu_context_create(int device, void* stream, mgpu_context_t** out);
MGPU_API mgpu_status_t mgpu_context_destroy(mgpu_context_t* ctx);
/* Redirects later work to another cudaStream_t (NULL: the owned stream). */
MGPU_API mgpu_status_t mgpu_context_set_stream(mgpu_context_t* ctx, void* stream);
MGPU_API void* mgpu_context_stream(mgpu_context_t* ctx);
/* Waits for the stream; returns the first device-side error since the last
 * call (and clears it), or MGPU_ERR_CUDA. */
MGPU_API mgpu_status_t mgpu_synchronize(mgpu_context_t* ctx);
MGPU_API const char* mgpu_status_string(mgpu_status_t status);
/* Text of the last CUDA error seen by this context. */
MGPU_API const char* mgpu_last_error(mgpu_context_t* ctx);
MGPU_API int mgpu_sm_count(mgpu_context_t* ctx);

/* Device/host memory (context_t::alloc_gpu / alloc_cpu / free,
 * src/vk/context.cxx:156-212) and stream-ordered copies
 * (context_t::memcpy, :225-243; cmd_buffer_t::memcpy, :400-402). */
MGPU_API mgpu_status_t mgpu_alloc_gpu(mgpu_context_t* ctx, size_t bytes, void** out);
MGPU_API mgpu_status_t mgpu_alloc_cpu(mgpu_context_t* ctx, size_t bytes, void** out);
MGPU_API mgpu_status_t mgpu_free(mgpu_context_t* ctx, void* p);
MGPU_API mgpu_status_t mgpu_memcpy(mgpu_context_t* ctx, void* dest, const void* src, size_t bytes);
MGPU_API mgpu_status_t mgpu_memset(mgpu_context_t* ctx, void* dest, int value, size_t bytes);

/* ---- radix sort (vk::radix_sort, vk/radix.hxx:195-470) ----
 * Stable LSD sort of `keys` in place by radix_permute_t order
 * (common/cta_radix.hxx:6-64): unsigned keys by value, signed keys by value,
 * float keys by bit order (-0.0 before +0.0, NaNs by bit pattern).  Values of
 * `val_bytes` bytes (0 = keys only, 4, or 8) travel with their keys; the
 * reference sorts keys only.  Keys: I32, U32, F32, I64, U64, F64.
 * count < 2^30. */
MGPU_API mgpu_status_t mgpu_radix_sort(mgpu_context_t* ctx, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, void* aux_data, size_t* aux_size);

/* The same sort with the number of keys read on the device from *d_count
 * (clamped to [0, max_count]) when the kernels run, so one captured graph
 * (mgpu_graph_begin/end) replays for any size up to max_count without
 * re-capture; keys, vals and aux are sized for max_count, and elements past
 * *d_count are left as they are.  The reference's GL mergesort keeps its
 * pass state in device memory for the same reason (gl/mergesort.hxx:23-27,
 * 48-54).  d_count == NULL is MGPU_ERR_INVALID_ARG. */
MGPU_API mgpu_status_t mgpu_radix_sort_count_on_device(mgpu_context_t* ctx,
  mgpu_dtype_t key_type, void* keys, int val_bytes, void* vals, int64_t max_count,
  const int64_t* d_count, void* aux_data, size_t* aux_size);

/* ---- merge (vk::merge key-value and keys-only, vk/merge.hxx:12-59) ----
 * Stable merge of sorted A and B into C (ties take A first, bounds_lower,
 * common/cta_merge.hxx:23-25).  vals may be NULL with val_bytes 0. */
MGPU_API mgpu_status_t mgpu_merge(mgpu_context_t* ctx, mgpu_dtype_t key_type,
  const void* a_keys, const void* a_vals, int64_t a_count,
  const void* b_keys, const void* b_vals, int64_t b_count,
  void* c_keys, void* c_vals, int val_bytes, mgpu_comp_t comp,
  void* aux_data, size_t* aux_size);

/* ---- mergesort (vk::mergesort_kv / mergesort_keys, vk/mergesort.hxx:10-93) ----
 * Stable comparison sort in place.  vals may be NULL with val_bytes 0. */
MGPU_API mgpu_status_t mgpu_mergesort(mgpu_context_t* ctx, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, mgpu_comp_t comp,
  void* aux_data, size_t* aux_size);

/* vk::mergesort_indices (vk/mergesort.hxx:95-103): sorts keys in place and
 * writes each key's original index into `indices` (int32). */
MGPU_API mgpu_status_t mgpu_mergesort_indices(mgpu_context_t* ctx, mgpu_dtype_t key_type,
  void* keys, int32_t* indices, int64_t count, mgpu_comp_t comp,
  void* aux_data, size_t* aux_size);

/* ---- scan (vk::scan, vk/scan.hxx:10-115) ----
 * out[i] = init (+) in[0] (+) ... (+) in[i-1]   (MGPU_SCAN_EXC)
 * out[i] = init (+) in[0] (+) ... (+) in[i]     (MGPU_SCAN_INC)
 * `init` is a host pointer to one element (NULL: the operator's identity).
 * in == out scans in place, as the reference does.  `reduction`, if not
 * NULL, is a device pointer that receives init (+) all inputs.
 * Integer sums wrap in two's complement. */
MGPU_API mgpu_status_t mgpu_scan(mgpu_context_t* ctx, mgpu_dtype_t type, mgpu_scan_type_t scan_type,
  mgpu_op_t op, const void* in, void* out, int64_t count, const void* init,
  void* reduction, void* aux_data, size_t* aux_size);

/* ---- scan without any allocation.  No counterpart in the reference: it is
 * an addition for callers that cannot allocate device memory (an operator
 * inside another engine that owns all device memory, a plugin whose enqueue
 * must not allocate or synchronise, a pipeline that forbids allocation after
 * start-up).  Same results as mgpu_scan for I32/U32/F32 (plus, max, min;
 * exclusive or inclusive), enqueued on `stream` (a cudaStream_t, NULL = the
 * legacy default stream) on the current device, with no context.  Its
 * scratch is a fixed 512 KiB array inside the library, held on every GPU that
 * loads it until exit; counts above MGPU_SCAN_NOALLOC_MAX_COUNT return
 * MGPU_ERR_INVALID_ARG, 8-byte types MGPU_ERR_UNSUPPORTED.  The first call on
 * a device looks up that array's device address; make it outside any stream
 * capture.  All calls share the array: calls that overlap on the GPU race, so
 * order them (for example, on one stream). */
#define MGPU_SCAN_NOALLOC_MAX_COUNT (1LL << 28)
MGPU_API mgpu_status_t mgpu_scan_noalloc(void* stream, mgpu_dtype_t type,
  mgpu_scan_type_t scan_type, mgpu_op_t op, const void* in, void* out, int64_t count,
  const void* init, void* reduction);

/* Device-side status of mgpu_scan_noalloc on the current device (no
 * counterpart in the reference; it belongs to the allocation-free scan
 * above).  mgpu_scan_noalloc has no context, so a bounded look-back wait
 * that gave up inside it is recorded in a word of its fixed scratch array
 * instead.  This call waits for `stream`, reads that word and clears it:
 * MGPU_OK if no wait gave up since the last query, MGPU_ERR_LOOKBACK_TIMEOUT
 * if one did (the results of the scans since the last query are then not to
 * be trusted; later scans may also leave their waits early until the word is
 * cleared).  It allocates nothing.  Call it outside any stream capture. */
MGPU_API mgpu_status_t mgpu_scan_noalloc_status(void* stream);

/* Self test of that status path: enqueues on `stream` a kernel whose bounded
 * wait on a flag that nothing sets gives up after `limit` polls (1 ..
 * 2^22) and records the timeout where a scan look-back would; the next
 * mgpu_scan_noalloc_status() returns MGPU_ERR_LOOKBACK_TIMEOUT. */
MGPU_API mgpu_status_t mgpu_selftest_scan_noalloc_wait(void* stream, int limit);

/* ---- reduce (cta_reduce_t, common/cta_scan.hxx:9-59, as a device-wide
 * primitive).  Writes init (+) all inputs to the device pointer `out`. */
MGPU_API mgpu_status_t mgpu_reduce(mgpu_context_t* ctx, mgpu_dtype_t type, mgpu_op_t op,
  const void* in, int64_t count, const void* init, void* out,
  void* aux_data, size_t* aux_size);

/* ---- transform (vk::transform / vk::launch, vk/transform.hxx:9-36) ----
 * The generic form takes a C++ device lambda (mgpu::gb300::transform in the
 * C++ headers).  The C ABI carries the element-wise operations of the
 * reference's transform example (examples/vk_transform/vk_transform.cxx:
 * 36-63) for callers without a CUDA compiler. */
/* out[i] = start + i * step, for an element type of the table above. */
MGPU_API mgpu_status_t mgpu_transform_iota(mgpu_context_t* ctx, mgpu_dtype_t type, void* out,
  int64_t count, double start, double step);
/* out[i] = value. */
MGPU_API mgpu_status_t mgpu_transform_fill(mgpu_context_t* ctx, mgpu_dtype_t type, void* out,
  int64_t count, double value);
/* y[i] += a * x[i] (float32). */
MGPU_API mgpu_status_t mgpu_transform_saxpy_f32(mgpu_context_t* ctx, float a, const float* x,
  float* y, int64_t count);

/* ---- segmented primitives (no reference counterpart: batched sort/scan
 * over CSR segments, one launch sequence for all segments) ----
 * `offsets` is a device array of num_segments + 1 int64 begin offsets;
 * segment s is [offsets[s], offsets[s+1]).  Keys are sorted in radix order
 * (as mgpu_radix_sort) within each segment; vals follow.  The offsets must
 * not decrease and must lie in [0, count]; mgpu_segmented_sort checks that
 * on the device and otherwise sorts nothing and records
 * MGPU_ERR_INVALID_ARG for mgpu_synchronize (the segmented scan only marks
 * heads inside [0, count)). */
MGPU_API mgpu_status_t mgpu_segmented_sort(mgpu_context_t* ctx, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, const int64_t* offsets,
  int64_t num_segments, void* aux_data, size_t* aux_size);
/* Scan restarted at every segment head with `init`. */
MGPU_API mgpu_status_t mgpu_segmented_scan(mgpu_context_t* ctx, mgpu_dtype_t type,
  mgpu_scan_type_t scan_type, mgpu_op_t op, const void* in, void* out, int64_t count,
  const int64_t* offsets, int64_t num_segments, const void* init,
  void* aux_data, size_t* aux_size);

/* ---- launch-shape tuning (the reference's (nt, vt[, num_bits]) template
 * knobs, vk/radix.hxx:195, vk/mergesort.hxx:10, vk/merge.hxx:13,
 * vk/scan.hxx:10, chosen at run time).  Several shapes of each primitive are
 * compiled; a per-context table picks one per (primitive, key type, value
 * width, size bucket = ceil(log2 count)), bucket -1 meaning every size.
 * The environment variable MGPU_TUNE_FILE names a table loaded at context
 * creation (there, an entry that names no compiled variant runs the default
 * shape). */
typedef enum mgpu_primitive_t {
  MGPU_PRIM_RADIX = 0,
  MGPU_PRIM_SCAN = 1,
  MGPU_PRIM_MERGE = 2,
  MGPU_PRIM_MERGESORT = 3
} mgpu_primitive_t;
/* Number of compiled variants; their names ("<threads>x<items>") are written
 * '\n'-separated into `names` when it is not NULL. */
MGPU_API int mgpu_tuning_variants(int primitive, mgpu_dtype_t key_type, char* names,
  size_t names_bytes);
MGPU_API mgpu_status_t mgpu_tuning_set(mgpu_context_t* ctx, int primitive,
  mgpu_dtype_t key_type, int val_bytes, int size_bucket, int variant);
/* Variant the context would use for this call shape. */
MGPU_API int mgpu_tuning_get(mgpu_context_t* ctx, int primitive, mgpu_dtype_t key_type,
  int val_bytes, int64_t count);
/* Tables persist as text, one "primitive key_type val_bytes size_bucket
 * variant" line per entry ('#' starts a comment line).  Loading adds the
 * file's entries to the context's table only if every entry names a
 * compiled variant and a bucket in -1..62; otherwise it returns
 * MGPU_ERR_INVALID_ARG and the table is unchanged. */
MGPU_API mgpu_status_t mgpu_tuning_save(mgpu_context_t* ctx, const char* path);
MGPU_API mgpu_status_t mgpu_tuning_load(mgpu_context_t* ctx, const char* path);
/* Times every variant on device-generated data of this type and size (median
 * of `reps` runs, each on a fresh unsorted copy; allocates its own scratch)
 * and records the fastest for the size bucket of `count`. */
MGPU_API mgpu_status_t mgpu_autotune(mgpu_context_t* ctx, int primitive, mgpu_dtype_t key_type,
  int val_bytes, int64_t count, int reps, int* best_variant, double* best_ms);

/* ---- CUDA graphs (no reference counterpart; the reference re-records a
 * Vulkan command buffer per submission, examples/vk_radix/vk_radix.cxx:
 * 51-63).  Everything enqueued on the context between begin and end is
 * captured into one executable graph (multi-pass pipelines such as a radix
 * sort's memset + histogram + passes become one launch).  Calls inside a
 * capture must pass explicit aux or fit in the context cache already
 * (see mgpu_cache_reserve); kernel arguments, including counts, are fixed at
 * capture time. */
typedef struct mgpu_graph mgpu_graph_t;
MGPU_API mgpu_status_t mgpu_graph_begin(mgpu_context_t* ctx);
MGPU_API mgpu_status_t mgpu_graph_end(mgpu_context_t* ctx, mgpu_graph_t** out);
MGPU_API mgpu_status_t mgpu_graph_launch(mgpu_context_t* ctx, mgpu_graph_t* graph);
MGPU_API mgpu_status_t mgpu_graph_destroy(mgpu_graph_t* graph);
/* Grows the context's aux cache to at least `bytes` (stream-ordered). */
MGPU_API mgpu_status_t mgpu_cache_reserve(mgpu_context_t* ctx, size_t bytes);

/* ---- serving: continuous batching of sort / merge / scan requests (no
 * reference counterpart).  A scheduler thread admits queued requests, in
 * arrival order, whenever a stream slot is free and the request's device
 * footprint (inputs, outputs and aux) fits in the remaining HBM budget;
 * admitted requests copy their host inputs into device buffers drawn from a
 * stream-ordered pool that stays resident, run the primitive on the slot's
 * stream, copy the results back and release their memory, so requests that
 * arrive while others run overlap with them.  Small sorts, merges of
 * integer keys by MGPU_LESS and integer scans (at most 2^16 elements) queued
 * together with others of the same kind (sorts and those merges by key type
 * and value width; scans by key type, scan type and operator) are coalesced:
 * up to 512 of them (2^22 elements) run as one segmented sort or scan over a
 * packed buffer, one launch sequence for the batch (a merge is a segment
 * holding A then B, whose stable sort is the A-first merge of sorted inputs);
 * each result is byte-identical to the one the request gets alone.  Host
 * buffers must stay valid until the request completes (pinned memory gives
 * asynchronous copies). */
typedef enum mgpu_request_op_t {
  MGPU_REQ_SORT = 0,   /* radix sort of keys (+ values), in place on device */
  MGPU_REQ_MERGE = 1,  /* merge of sorted A and B (+ values) */
  MGPU_REQ_SCAN = 2    /* scan of `count` elements */
} mgpu_request_op_t;

typedef struct mgpu_request_t {
  int op;                  /* mgpu_request_op_t */
  mgpu_dtype_t key_type;   /* keys (sort, merge) or elements (scan) */
  int val_bytes;           /* values of sort / merge: 0, 4 or 8 */
  int64_t count;           /* sort / scan elements; merge: A count */
  int64_t count_b;         /* merge: B count */
  const void* keys;        /* host: sort keys, scan input, merge A keys */
  const void* vals;        /* host: sort values, merge A values */
  const void* keys_b;      /* host: merge B keys */
  const void* vals_b;      /* host: merge B values */
  void* out_keys;          /* host: sorted keys, merged keys, scan output */
  void* out_vals;          /* host: sorted / merged values */
  int scan_type;           /* scan: mgpu_scan_type_t */
  int op_arg;              /* scan: mgpu_op_t; merge: mgpu_comp_t */
} mgpu_request_t;

typedef struct mgpu_server_stats_t {
  int64_t submitted, completed, failed;
  int64_t elements;        /* sum of request element counts completed */
  double p50_ms, p99_ms, mean_ms, max_ms;   /* submit -> completion, over the most
                                               recent 2^20 completions */
  size_t peak_bytes;       /* largest admitted footprint total */
  int64_t coalesced;       /* requests that ran in coalesced batches */
  int64_t batches;         /* coalesced batches launched */
} mgpu_server_stats_t;

typedef struct mgpu_server mgpu_server_t;
/* `budget_bytes` bounds the summed footprint of admitted requests;
 * `num_slots` streams run requests concurrently. */
MGPU_API mgpu_status_t mgpu_server_create(int device, size_t budget_bytes, int num_slots,
  mgpu_server_t** out);
/* Queues a request; MGPU_ERR_BUDGET if its footprint alone exceeds the
 * budget.  *id identifies it for poll / wait. */
MGPU_API mgpu_status_t mgpu_server_submit(mgpu_server_t* server, const mgpu_request_t* request,
  uint64_t* id);
/* MGPU_OK when done, MGPU_ERR_NOT_READY while queued or running, or the
 * request's error.  A poll that reports completion, or a wait, releases the
 * id; a released id is MGPU_ERR_INVALID_ARG. */
MGPU_API mgpu_status_t mgpu_server_poll(mgpu_server_t* server, uint64_t id);
/* Blocks until the request completes; *latency_ms (optional) = submit to
 * completion. */
MGPU_API mgpu_status_t mgpu_server_wait(mgpu_server_t* server, uint64_t id, double* latency_ms);
/* Blocks until every submitted request has completed. */
MGPU_API mgpu_status_t mgpu_server_drain(mgpu_server_t* server);
MGPU_API mgpu_status_t mgpu_server_stats(mgpu_server_t* server, mgpu_server_stats_t* out);
/* Resets the latency record (not the requests). */
MGPU_API mgpu_status_t mgpu_server_reset_stats(mgpu_server_t* server);
MGPU_API mgpu_status_t mgpu_server_destroy(mgpu_server_t* server);

/* ---- launch profiling (no reference counterpart; the reference times
 * whole command buffers with clock_gettime, examples/vk_radix/vk_radix.cxx:
 * 51-63).  When enabled, every kernel the library launches on this context
 * is bracketed by CUDA events on its stream. */
MGPU_API mgpu_status_t mgpu_profile_enable(mgpu_context_t* ctx, int enable);
/* Synchronises, then returns per-kernel launch counts and total device
 * milliseconds; names are written as a '\n'-separated list into `names`.
 * Clears the record.  Returns the number of kernels in *num (≤ capacity). */
MGPU_API mgpu_status_t mgpu_profile_read(mgpu_context_t* ctx, char* names, size_t names_bytes,
  int64_t* launches, double* total_ms, int capacity, int* num);
/* Kernel launches issued on this context since creation. */
MGPU_API int64_t mgpu_launch_count(mgpu_context_t* ctx);

/* ---- failure-path self test (no reference counterpart) ----
 * Enqueues one kernel that waits, with at most `limit` polls each, on an
 * mbarrier phase and on a device flag that nothing completes -- the two kinds
 * of bounded wait the primitives use (bulk-copy completion, look-back).  The
 * waits give up, record MGPU_ERR_LOOKBACK_TIMEOUT in the context's error word
 * and the kernel returns, so the next mgpu_synchronize reports that status and
 * the context stays usable.  limit: 1 .. 2^22. */
MGPU_API mgpu_status_t mgpu_selftest_bounded_wait(mgpu_context_t* ctx, int limit);
/* Polls (1 .. 2^22) after which the look-back and bulk-copy waits of the
 * radix-sort passes launched from this context give up and raise
 * MGPU_ERR_LOOKBACK_TIMEOUT; 0 restores the library's limit (2^22 polls,
 * seconds of wall time).  A smaller limit detects a stalled predecessor
 * sooner; a limit too small for the load can raise false timeouts. */
MGPU_API mgpu_status_t mgpu_set_wait_limit(mgpu_context_t* ctx, int polls);
/* Runs the production radix-sort pass kernel (u32 keys + u32 values, the
 * default tile shape) over two tiles with its tile counter advanced past
 * tile 0, so the one CTA launched takes tile 1 and its decoupled look-back
 * waits on a predecessor that never publishes.  With the context's wait
 * limit (mgpu_set_wait_limit) the wait runs out, the pass records
 * MGPU_ERR_LOOKBACK_TIMEOUT and returns; the next mgpu_synchronize reports
 * it.  Every store stays inside the call's own buffers.  Synchronises and
 * allocates its own buffers. */
MGPU_API mgpu_status_t mgpu_selftest_lookback_timeout(mgpu_context_t* ctx);

#ifdef __cplusplus
}
#endif

#endif /* MGPU_GB300_H */
