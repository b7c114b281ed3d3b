// C ABI: the serving loop (continuous batching of sort / merge / scan
// requests under an HBM budget).
//
// Threads: callers submit / poll / wait; one scheduler thread admits and
// launches; CUDA's host-callback thread reports completions.  The scheduler
// admits queued requests in arrival order whenever one of `num_slots` stream
// slots is free and the request's footprint fits in the budget that the
// requests in flight leave.  Each slot has its own mgpu context (and stream),
// so admitted requests overlap on the device.  Device buffers come from a
// stream-ordered memory pool whose release threshold is the budget, so memory
// stays resident between requests instead of returning to the driver.
//
// Coalescing: a small sort, integer merge (by less) or integer scan (at most
// coalesce_max elements) at the head of the queue is run together with the
// other queued small requests of the same kind (sorts and such merges of the
// same key type and value width together; scans of the same key type, scan
// type and operator; up to max_batch requests and batch_elems elements) as ONE
// segmented sort or segmented scan over a packed device buffer, one request
// per segment: one fixed launch sequence for the whole batch instead of a
// launch chain per request.  Every result is byte-identical to the request run
// alone: a segment is sorted in the radix order of mgpu_radix_sort (a merge's
// segment holds A then B, and for integer keys the stable sort of that is the
// A-first stable merge), and integer scans are exact.  Floating-point scans
// and merges, merges by greater, and larger requests run alone.
#include "capi.hxx"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

typedef std::chrono::steady_clock clock_type;

struct request_record {
  uint64_t id = 0;
  uint64_t batch = 0;              // id of the coalesced batch it ran in (0: alone)
  mgpu_request_t req {};
  size_t footprint = 0;
  size_t aux_bytes = 0;
  clock_type::time_point submit, finish;
  mgpu_status_t status = MGPU_ERR_NOT_READY;
  bool done = false;
  int slot = -1;
  void* dev[7] = {};
};

int dtype_size(mgpu_dtype_t t) {
  return (t == MGPU_I64 || t == MGPU_U64 || t == MGPU_F64) ? 8 : 4;
}

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// Coalescing limits: a request of at most coalesce_max elements joins a
// batch; a batch holds at most max_batch requests and batch_elems elements.
constexpr int64_t coalesce_max = int64_t(1) << 16;
constexpr int max_batch = 512;
constexpr int64_t batch_elems = int64_t(1) << 22;

bool integer_key(mgpu_dtype_t t) { return t != MGPU_F32 && t != MGPU_F64; }

// Elements a request puts into a batch (a merge: both inputs).
int64_t batch_count(const mgpu_request_t& r) {
  return r.count + (r.op == MGPU_REQ_MERGE ? r.count_b : 0);
}

// A small merge of integer keys by `less` runs as a segment of the batch's
// segmented sort: A followed by B, stably sorted, is the A-first stable merge
// (float keys stay alone: the sort orders -0.0 before +0.0, operator< does
// not).  Floating-point scans stay alone too: a segmented scan adds in
// another order than the plain scan, so their bits would depend on what they
// ran with.
bool sortlike(const mgpu_request_t& r) {
  return r.op == MGPU_REQ_SORT ||
    (r.op == MGPU_REQ_MERGE && integer_key(r.key_type) && r.op_arg == MGPU_LESS);
}

bool coalescible(const mgpu_request_t& r) {
  const bool int_scan = r.op == MGPU_REQ_SCAN && integer_key(r.key_type);
  const int64_t n = batch_count(r);
  return (sortlike(r) || int_scan) && n > 0 && n <= coalesce_max;
}

bool same_kind(const mgpu_request_t& a, const mgpu_request_t& b) {
  if(a.key_type != b.key_type || a.val_bytes != b.val_bytes) return false;
  if(sortlike(a) || sortlike(b)) return sortlike(a) && sortlike(b);
  return a.op == b.op && a.scan_type == b.scan_type && a.op_arg == b.op_arg;
}

// Requests run together as one segmented sort or scan.
struct batch_record {
  uint64_t id = 0;
  std::vector<request_record*> recs;
  int64_t total = 0;
  size_t footprint = 0, aux_bytes = 0;
  int slot = -1;
  void* dev[4] = {};               // keys, values, offsets, aux
};

}  // namespace

struct mgpu_server {
  int device = 0;
  size_t budget = 0;
  int num_slots = 0;
  std::vector<mgpu_context*> slots;
  std::vector<char> slot_busy;
  int* h_err = nullptr;          // pinned: each slot's device error word after a request
  int64_t* h_off = nullptr;      // pinned: each slot's batch offsets (max_batch + 1)
  mgpu_context* sizing = nullptr;
  cudaMemPool_t pool = nullptr;

  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, request_record*> records;
  std::unordered_map<uint64_t, batch_record*> batches;
  std::deque<uint64_t> completions;
  std::deque<uint64_t> batch_completions;
  uint64_t next_batch = 1;
  int64_t coalesced = 0, batch_launches = 0;
  size_t used = 0, peak = 0;
  int in_flight = 0;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread scheduler;

  int64_t submitted = 0, completed = 0, failed = 0, elements = 0;
  // Latencies of the most recent completions (a ring of latency_window
  // samples), so a long-running server's record stays bounded.
  static constexpr size_t latency_window = size_t(1) << 20;
  std::vector<double> latencies;
  size_t latency_next = 0;

  // Device bytes a request needs: its inputs, outputs and the primitive's aux.
  mgpu_status_t footprint(const mgpu_request_t& r, size_t& bytes, size_t& aux) {
    const size_t kb = dtype_size(r.key_type), vb = r.val_bytes;
    aux = 0;
    mgpu_status_t st = MGPU_OK;
    switch(r.op) {
      case MGPU_REQ_SORT:
        st = mgpu_radix_sort(sizing, r.key_type, nullptr, (int)vb, nullptr, r.count, nullptr, &aux);
        bytes = round256(kb * r.count) + round256(vb * r.count) + round256(aux);
        break;
      case MGPU_REQ_MERGE:
        st = mgpu_merge(sizing, r.key_type, nullptr, nullptr, r.count, nullptr, nullptr, r.count_b,
          nullptr, nullptr, (int)vb, (mgpu_comp_t)r.op_arg, nullptr, &aux);
        bytes = 2 * (round256(kb * r.count) + round256(vb * r.count) + round256(kb * r.count_b) +
          round256(vb * r.count_b)) + round256(aux);
        break;
      case MGPU_REQ_SCAN:
        st = mgpu_scan(sizing, r.key_type, (mgpu_scan_type_t)r.scan_type, (mgpu_op_t)r.op_arg,
          nullptr, nullptr, r.count, nullptr, nullptr, nullptr, &aux);
        bytes = round256(kb * r.count) + round256(aux);   // scanned in place
        break;
      default:
        return MGPU_ERR_INVALID_ARG;
    }
    // A null aux pointer would make the run a sizing call: always give the
    // primitive a (small) block, even when it needs none.
    if(!st && !aux) {
      aux = 256;
      bytes += aux;
    }
    return st;
  }

  static void CUDART_CB on_complete(void* arg);

  struct callback_arg { mgpu_server* server; uint64_t id; bool batch; };

  // Enqueues one admitted request on its slot's stream.
  mgpu_status_t launch(request_record* rec) {
    mgpu_context* c = slots[rec->slot];
    cudaStream_t s = c->ctx.stream;
    const mgpu_request_t& r = rec->req;
    const size_t kb = dtype_size(r.key_type), vb = r.val_bytes;
    if(cudaSetDevice(device) != cudaSuccess) return MGPU_ERR_CUDA;
    auto alloc = [&](int i, size_t bytes) -> bool {
      if(!bytes) return true;
      return cudaMallocFromPoolAsync(&rec->dev[i], bytes, pool, s) == cudaSuccess;
    };
    auto h2d = [&](void* d, const void* h, size_t bytes) -> bool {
      return !bytes || cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
    };
    auto d2h = [&](void* h, const void* d, size_t bytes) -> bool {
      return !bytes || cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s) == cudaSuccess;
    };
    mgpu_status_t st = MGPU_OK;
    size_t aux = rec->aux_bytes;
    if(!alloc(6, aux)) return MGPU_ERR_OOM;
    const int64_t total = r.count + (r.op == MGPU_REQ_MERGE ? r.count_b : 0);
    switch(total ? r.op : -1) {
      case -1:
        break;                     // nothing to do: completes through the callback

      case MGPU_REQ_SORT: {
        size_t kbytes = kb * r.count, vbytes = vb * r.count;
        if(!alloc(0, kbytes) || !alloc(1, vbytes)) return MGPU_ERR_OOM;
        if(!h2d(rec->dev[0], r.keys, kbytes) || !h2d(rec->dev[1], r.vals, vbytes))
          return MGPU_ERR_CUDA;
        st = mgpu_radix_sort(c, r.key_type, rec->dev[0], (int)vb, rec->dev[1], r.count,
          rec->dev[6], &aux);
        if(st) return st;
        if(!d2h(r.out_keys, rec->dev[0], kbytes) || !d2h(r.out_vals, rec->dev[1], vbytes))
          return MGPU_ERR_CUDA;
        break;
      }
      case MGPU_REQ_MERGE: {
        size_t ak = kb * r.count, av = vb * r.count, bk = kb * r.count_b, bv = vb * r.count_b;
        if(!alloc(0, ak) || !alloc(1, av) || !alloc(2, bk) || !alloc(3, bv) ||
           !alloc(4, ak + bk) || !alloc(5, av + bv)) return MGPU_ERR_OOM;
        if(!h2d(rec->dev[0], r.keys, ak) || !h2d(rec->dev[1], r.vals, av) ||
           !h2d(rec->dev[2], r.keys_b, bk) || !h2d(rec->dev[3], r.vals_b, bv))
          return MGPU_ERR_CUDA;
        st = mgpu_merge(c, r.key_type, rec->dev[0], rec->dev[1], r.count, rec->dev[2],
          rec->dev[3], r.count_b, rec->dev[4], rec->dev[5], (int)vb, (mgpu_comp_t)r.op_arg,
          rec->dev[6], &aux);
        if(st) return st;
        if(!d2h(r.out_keys, rec->dev[4], ak + bk) || !d2h(r.out_vals, rec->dev[5], av + bv))
          return MGPU_ERR_CUDA;
        break;
      }
      case MGPU_REQ_SCAN: {
        size_t bytes = kb * r.count;
        if(!alloc(0, bytes)) return MGPU_ERR_OOM;
        if(!h2d(rec->dev[0], r.keys, bytes)) return MGPU_ERR_CUDA;
        st = mgpu_scan(c, r.key_type, (mgpu_scan_type_t)r.scan_type, (mgpu_op_t)r.op_arg,
          rec->dev[0], rec->dev[0], r.count, nullptr, nullptr, rec->dev[6], &aux);
        if(st) return st;
        if(!d2h(r.out_keys, rec->dev[0], bytes)) return MGPU_ERR_CUDA;
        break;
      }
      default:
        return MGPU_ERR_INVALID_ARG;
    }
    release(rec);
    // The slot's device error word travels back (and is cleared) in stream
    // order, so the completion needs no host synchronisation.
    if(cudaMemcpyAsync(h_err + rec->slot, c->ctx.d_error, sizeof(int), cudaMemcpyDeviceToHost,
         s) != cudaSuccess ||
       cudaMemsetAsync(c->ctx.d_error, 0, sizeof(int), s) != cudaSuccess)
      return MGPU_ERR_CUDA;
    callback_arg* arg = new(std::nothrow) callback_arg { this, rec->id, false };
    if(!arg) return MGPU_ERR_OOM;
    if(cudaLaunchHostFunc(s, on_complete, arg) != cudaSuccess) { delete arg; return MGPU_ERR_CUDA; }
    return MGPU_OK;
  }

  // Returns the request's buffers to the pool in stream order.
  void release(request_record* rec) {
    cudaStream_t s = slots[rec->slot]->ctx.stream;
    for(void*& p : rec->dev) {
      if(p) cudaFreeAsync(p, s);
      p = nullptr;
    }
  }

  // Device bytes of a batch: packed keys (and values), offsets and the
  // segmented primitive's aux for the batch's total and segment count.
  mgpu_status_t batch_footprint(batch_record* b) {
    const mgpu_request_t& r = b->recs.front()->req;
    const size_t kb = dtype_size(r.key_type), vb = r.val_bytes;
    const int64_t n = (int64_t)b->recs.size();
    size_t aux = 0;
    mgpu_status_t st;
    if(sortlike(r))
      st = mgpu_segmented_sort(sizing, r.key_type, nullptr, (int)vb, nullptr, b->total, nullptr,
        n, nullptr, &aux);
    else
      st = mgpu_segmented_scan(sizing, r.key_type, (mgpu_scan_type_t)r.scan_type,
        (mgpu_op_t)r.op_arg, nullptr, nullptr, b->total, nullptr, n, nullptr, nullptr, &aux);
    if(st) return st;
    if(!aux) aux = 256;
    b->aux_bytes = aux;
    b->footprint = round256(kb * b->total) + round256(vb * b->total) +
      round256(sizeof(int64_t) * (n + 1)) + round256(aux);
    return MGPU_OK;
  }

  // Enqueues one admitted batch on its slot's stream: packed uploads, one
  // segmented sort or scan, per-request downloads, one completion.
  mgpu_status_t launch_batch(batch_record* b) {
    mgpu_context* c = slots[b->slot];
    cudaStream_t s = c->ctx.stream;
    const mgpu_request_t& r0 = b->recs.front()->req;
    const size_t kb = dtype_size(r0.key_type), vb = r0.val_bytes;
    const int64_t n = (int64_t)b->recs.size();
    if(cudaSetDevice(device) != cudaSuccess) return MGPU_ERR_CUDA;
    auto alloc = [&](int i, size_t bytes) -> bool {
      return !bytes || cudaMallocFromPoolAsync(&b->dev[i], bytes, pool, s) == cudaSuccess;
    };
    if(!alloc(0, kb * b->total) || !alloc(1, vb * b->total) ||
       !alloc(2, sizeof(int64_t) * (n + 1)) || !alloc(3, b->aux_bytes))
      return MGPU_ERR_OOM;
    int64_t* off = h_off + (size_t)b->slot * (max_batch + 1);
    char* dk = (char*)b->dev[0];
    char* dv = (char*)b->dev[1];
    off[0] = 0;
    auto h2d = [&](void* d, const void* h, size_t bytes) -> bool {
      return !bytes || cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
    };
    for(int64_t i = 0; i < n; ++i) {
      const mgpu_request_t& r = b->recs[i]->req;
      off[i + 1] = off[i] + batch_count(r);
      if(!h2d(dk + kb * off[i], r.keys, kb * r.count) ||
         (vb && !h2d(dv + vb * off[i], r.vals, vb * r.count)))
        return MGPU_ERR_CUDA;
      if(r.op == MGPU_REQ_MERGE &&      // B right after A in the same segment
         (!h2d(dk + kb * (off[i] + r.count), r.keys_b, kb * r.count_b) ||
          (vb && !h2d(dv + vb * (off[i] + r.count), r.vals_b, vb * r.count_b))))
        return MGPU_ERR_CUDA;
    }
    if(cudaMemcpyAsync(b->dev[2], off, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s) !=
       cudaSuccess)
      return MGPU_ERR_CUDA;
    size_t aux = b->aux_bytes;
    mgpu_status_t st;
    if(sortlike(r0))
      st = mgpu_segmented_sort(c, r0.key_type, dk, (int)vb, vb ? dv : nullptr, b->total,
        (const int64_t*)b->dev[2], n, b->dev[3], &aux);
    else
      st = mgpu_segmented_scan(c, r0.key_type, (mgpu_scan_type_t)r0.scan_type,
        (mgpu_op_t)r0.op_arg, dk, dk, b->total, (const int64_t*)b->dev[2], n, nullptr,
        b->dev[3], &aux);
    if(st) return st;
    for(int64_t i = 0; i < n; ++i) {
      const mgpu_request_t& r = b->recs[i]->req;
      const int64_t m = batch_count(r);
      if(cudaMemcpyAsync(r.out_keys, dk + kb * off[i], kb * m, cudaMemcpyDeviceToHost, s) !=
           cudaSuccess ||
         (vb && cudaMemcpyAsync(r.out_vals, dv + vb * off[i], vb * m,
           cudaMemcpyDeviceToHost, s) != cudaSuccess))
        return MGPU_ERR_CUDA;
    }
    release_batch(b);
    if(cudaMemcpyAsync(h_err + b->slot, c->ctx.d_error, sizeof(int), cudaMemcpyDeviceToHost,
         s) != cudaSuccess ||
       cudaMemsetAsync(c->ctx.d_error, 0, sizeof(int), s) != cudaSuccess)
      return MGPU_ERR_CUDA;
    callback_arg* arg = new(std::nothrow) callback_arg { this, b->id, true };
    if(!arg) return MGPU_ERR_OOM;
    if(cudaLaunchHostFunc(s, on_complete, arg) != cudaSuccess) { delete arg; return MGPU_ERR_CUDA; }
    return MGPU_OK;
  }

  void release_batch(batch_record* b) {
    cudaStream_t s = slots[b->slot]->ctx.stream;
    for(void*& p : b->dev) {
      if(p) cudaFreeAsync(p, s);
      p = nullptr;
    }
  }

  // Completes every request of a batch (lock held).
  void finish_batch_locked(batch_record* b, mgpu_status_t st) {
    used -= b->footprint;
    slot_busy[b->slot] = 0;
    for(request_record* rec : b->recs) {
      rec->footprint = 0;          // the batch held the memory
      rec->slot = -1;
      finish_locked(rec, st);
    }
    batches.erase(b->id);
    delete b;
  }

  // Gathers the queued requests that run together with the queue head (at
  // least the head itself), looking at most gather_window entries deep so a
  // long backlog does not make each admission scan all of it.  Lock held.
  static constexpr int gather_window = 4 * max_batch;
  batch_record* gather_batch() {
    request_record* head = records[queue.front()];
    batch_record* b = new(std::nothrow) batch_record;
    if(!b) return nullptr;
    int seen = 0;
    for(uint64_t id : queue) {
      if(++seen > gather_window) break;
      request_record* rec = records[id];
      if(!coalescible(rec->req) || !same_kind(rec->req, head->req)) continue;
      if((int)b->recs.size() == max_batch || b->total + batch_count(rec->req) > batch_elems) break;
      b->recs.push_back(rec);
      b->total += batch_count(rec->req);
    }
    return b;
  }

  void finish_locked(request_record* rec, mgpu_status_t st) {
    rec->status = st;
    rec->done = true;
    used -= rec->footprint;
    if(rec->slot >= 0) slot_busy[rec->slot] = 0;
    --in_flight;
    if(st == MGPU_OK) {
      ++completed;
      elements += rec->req.count + (rec->req.op == MGPU_REQ_MERGE ? rec->req.count_b : 0);
      const double ms = std::chrono::duration<double, std::milli>(rec->finish - rec->submit)
        .count();
      if(latencies.size() < latency_window) latencies.push_back(ms);
      else latencies[latency_next] = ms;
      latency_next = (latency_next + 1) % latency_window;
    } else {
      ++failed;
    }
    cv_done.notify_all();
  }

  void run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while(true) {
      // Completions reported by the host callbacks.
      while(!completions.empty()) {
        uint64_t id = completions.front();
        completions.pop_front();
        request_record* rec = records[id];
        // The callback ran after the slot's error word reached h_err.
        const int e = h_err[rec->slot];
        finish_locked(rec, e ? (mgpu_status_t)e : MGPU_OK);
      }
      while(!batch_completions.empty()) {
        batch_record* b = batches[batch_completions.front()];
        batch_completions.pop_front();
        const int e = h_err[b->slot];
        finish_batch_locked(b, e ? (mgpu_status_t)e : MGPU_OK);
      }
      if(stop && queue.empty() && in_flight == 0) break;
      bool progressed = false;
      while(!queue.empty()) {
        request_record* rec = records[queue.front()];
        int slot = -1;
        for(int i = 0; i < num_slots; ++i) if(!slot_busy[i]) { slot = i; break; }
        if(slot < 0) break;
        if(coalescible(rec->req)) {
          batch_record* b = gather_batch();
          if(b && b->recs.size() > 1 && !batch_footprint(b) && used + b->footprint <= budget) {
            // Admit the batch: its requests leave the queue together.
            b->id = next_batch++;
            for(request_record* r : b->recs) {
              r->slot = slot;
              r->batch = b->id;
            }
            // One pass over the gathered window removes them all.
            const auto window_end = queue.begin() +
              (std::ptrdiff_t)std::min<size_t>(queue.size(), gather_window);
            queue.erase(std::remove_if(queue.begin(), window_end,
              [&](uint64_t id) { return records[id]->batch == b->id; }), window_end);
            used += b->footprint;
            peak = std::max(peak, used);
            slot_busy[slot] = 1;
            b->slot = slot;
            in_flight += (int)b->recs.size();
            batches[b->id] = b;
            ++batch_launches;
            coalesced += (int64_t)b->recs.size();
            lk.unlock();
            mgpu_status_t st = launch_batch(b);
            if(st) {
              release_batch(b);
              cudaStreamSynchronize(slots[slot]->ctx.stream);
            }
            lk.lock();
            if(st) {
              const auto now = clock_type::now();
              for(request_record* r : b->recs) r->finish = now;
              finish_batch_locked(b, st);
            }
            progressed = true;
            continue;
          }
          delete b;          // alone (or the batch does not fit yet): the single path
        }
        if(used + rec->footprint > budget) break;
        queue.pop_front();
        used += rec->footprint;
        peak = std::max(peak, used);
        slot_busy[slot] = 1;
        rec->slot = slot;
        ++in_flight;
        lk.unlock();
        mgpu_status_t st = launch(rec);
        if(st) {
          release(rec);
          cudaStreamSynchronize(slots[slot]->ctx.stream);
        }
        lk.lock();
        if(st) {
          rec->finish = clock_type::now();
          finish_locked(rec, st);
        }
        progressed = true;
      }
      if(!progressed && completions.empty())
        cv_sched.wait_for(lk, std::chrono::milliseconds(2));
    }
  }
};

void CUDART_CB mgpu_server::on_complete(void* p) {
  callback_arg* arg = (callback_arg*)p;
  mgpu_server* s = arg->server;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const auto now = clock_type::now();
    if(arg->batch) {
      auto it = s->batches.find(arg->id);
      if(it != s->batches.end())
        for(request_record* rec : it->second->recs) rec->finish = now;
      s->batch_completions.push_back(arg->id);
    } else {
      auto it = s->records.find(arg->id);
      if(it != s->records.end()) it->second->finish = now;
      s->completions.push_back(arg->id);
    }
  }
  s->cv_sched.notify_one();
  delete arg;
}

extern "C" {

mgpu_status_t mgpu_server_create(int device, size_t budget_bytes, int num_slots,
  mgpu_server_t** out) {
  if(!out || num_slots < 1 || num_slots > 64 || !budget_bytes) return MGPU_ERR_INVALID_ARG;
  *out = nullptr;
  mgpu_server* s = new(std::nothrow) mgpu_server;
  if(!s) return MGPU_ERR_OOM;
  s->device = device;
  s->budget = budget_bytes;
  s->num_slots = num_slots;
  mgpu_status_t st = mgpu_context_create(device, nullptr, &s->sizing);
  for(int i = 0; i < num_slots && !st; ++i) {
    mgpu_context_t* c = nullptr;
    st = mgpu_context_create(device, nullptr, &c);
    if(!st) s->slots.push_back(c);
  }
  if(!st) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if(cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) st = MGPU_ERR_CUDA;
    else {
      uint64_t threshold = budget_bytes;
      cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
  }
  if(st) {
    for(auto* c : s->slots) mgpu_context_destroy(c);
    if(s->sizing) mgpu_context_destroy(s->sizing);
    delete s;
    return st;
  }
  if(cudaMallocHost(&s->h_err, sizeof(int) * num_slots) != cudaSuccess ||
     cudaMallocHost(&s->h_off, sizeof(int64_t) * (max_batch + 1) * num_slots) != cudaSuccess) {
    if(s->h_err) cudaFreeHost(s->h_err);
    for(auto* c : s->slots) mgpu_context_destroy(c);
    mgpu_context_destroy(s->sizing);
    cudaMemPoolDestroy(s->pool);
    delete s;
    return MGPU_ERR_OOM;
  }
  for(int i = 0; i < num_slots; ++i) s->h_err[i] = 0;
  s->slot_busy.assign(num_slots, 0);
  s->scheduler = std::thread([s] { s->run(); });
  *out = s;
  return MGPU_OK;
}

mgpu_status_t mgpu_server_submit(mgpu_server_t* s, const mgpu_request_t* r, uint64_t* id) {
  if(!s || !r || !id) return MGPU_ERR_INVALID_ARG;
  if(r->count < 0 || r->count_b < 0) return MGPU_ERR_INVALID_ARG;
  if(r->val_bytes != 0 && r->val_bytes != 4 && r->val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  if(r->op < MGPU_REQ_SORT || r->op > MGPU_REQ_SCAN) return MGPU_ERR_INVALID_ARG;
  if(r->op == MGPU_REQ_SCAN && r->val_bytes) return MGPU_ERR_INVALID_ARG;
  if(r->op != MGPU_REQ_MERGE && r->count_b) return MGPU_ERR_INVALID_ARG;
  {
    const int64_t total = r->count + r->count_b;
    const bool has_vals = r->val_bytes && r->op != MGPU_REQ_SCAN;
    if(total && (!r->out_keys || (has_vals && !r->out_vals))) return MGPU_ERR_INVALID_ARG;
    if(r->count && (!r->keys || (has_vals && !r->vals))) return MGPU_ERR_INVALID_ARG;
    if(r->count_b && (!r->keys_b || (has_vals && !r->vals_b))) return MGPU_ERR_INVALID_ARG;
  }
  request_record* rec = new(std::nothrow) request_record;
  if(!rec) return MGPU_ERR_OOM;
  rec->req = *r;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    mgpu_status_t st = s->footprint(*r, rec->footprint, rec->aux_bytes);
    if(st) { delete rec; return st; }
    if(rec->footprint > s->budget) { delete rec; return MGPU_ERR_BUDGET; }
    rec->id = s->next_id++;
    rec->submit = clock_type::now();
    s->records[rec->id] = rec;
    s->queue.push_back(rec->id);
    ++s->submitted;
    *id = rec->id;
  }
  s->cv_sched.notify_one();
  return MGPU_OK;
}

mgpu_status_t mgpu_server_poll(mgpu_server_t* s, uint64_t id) {
  if(!s) return MGPU_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->records.find(id);
  if(it == s->records.end()) return MGPU_ERR_INVALID_ARG;
  if(!it->second->done) return MGPU_ERR_NOT_READY;
  mgpu_status_t st = it->second->status;
  delete it->second;
  s->records.erase(it);
  return st;
}

mgpu_status_t mgpu_server_wait(mgpu_server_t* s, uint64_t id, double* latency_ms) {
  if(!s) return MGPU_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->records.find(id);
  if(it == s->records.end()) return MGPU_ERR_INVALID_ARG;
  request_record* rec = it->second;
  s->cv_done.wait(lk, [&] { return rec->done; });
  if(latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(rec->finish - rec->submit).count();
  mgpu_status_t st = rec->status;
  s->records.erase(id);
  delete rec;
  return st;
}

mgpu_status_t mgpu_server_drain(mgpu_server_t* s) {
  if(!s) return MGPU_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->queue.empty() && s->in_flight == 0; });
  return MGPU_OK;
}

mgpu_status_t mgpu_server_stats(mgpu_server_t* s, mgpu_server_stats_t* out) {
  if(!s || !out) return MGPU_ERR_INVALID_ARG;
  std::vector<double> l;
  {
    // Copy under the lock; sort outside it, so the scheduler is not held up.
    std::lock_guard<std::mutex> lk(s->mu);
    *out = {};
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->elements = s->elements;
    out->peak_bytes = s->peak;
    out->coalesced = s->coalesced;
    out->batches = s->batch_launches;
    l = s->latencies;
  }
  if(!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = l.back();
    double sum = 0;
    for(double x : l) sum += x;
    out->mean_ms = sum / l.size();
  }
  return MGPU_OK;
}

mgpu_status_t mgpu_server_reset_stats(mgpu_server_t* s) {
  if(!s) return MGPU_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->latency_next = 0;
  s->completed = s->failed = s->elements = 0;
  s->submitted = 0;
  s->coalesced = s->batch_launches = 0;
  s->peak = s->used;
  return MGPU_OK;
}

mgpu_status_t mgpu_server_destroy(mgpu_server_t* s) {
  if(!s) return MGPU_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_sched.notify_one();
  if(s->scheduler.joinable()) s->scheduler.join();
  for(auto& kv : s->records) delete kv.second;
  for(auto& kv : s->batches) delete kv.second;
  for(auto* c : s->slots) mgpu_context_destroy(c);
  if(s->sizing) mgpu_context_destroy(s->sizing);
  if(s->pool) cudaMemPoolDestroy(s->pool);
  if(s->h_err) cudaFreeHost(s->h_err);
  if(s->h_off) cudaFreeHost(s->h_off);
  delete s;
  return MGPU_OK;
}

}  // extern "C"
