// mgpu::gb300::scan / reduce - host drivers of the single-pass scan and the
// single-launch reduce.
//
// Drop-in for vk::scan (vk/scan.hxx:10-115): in-place exclusive scan with
// `init` and `op`, same two-phase aux protocol.  Additions: the scan type
// template (scan_type_exc / scan_type_inc, the enum of
// common/cta_scan.hxx:63-66), an out-of-place overload, an optional device
// reduction output, and reduce().  `init` enters once, as the left-most
// operand: exclusive out[0] = init; inclusive out[i] = init (+) in[0..i].
// `op` must be associative and commutative with an identity() (plus_t,
// maximum_t, minimum_t): a tile's aggregate folds each thread's elements
// before the warps' partials, not in element order.  Float sums therefore
// round differently from a sequential sum (within the usual bound).  The
// requirement is checked at compile time through commutative_op<op_t>, so an
// operator that does not commute fails to build instead of scanning wrongly.
#pragma once

#include "context.hxx"
#include "../device/scan.cuh"

namespace mgpu {
namespace gb300 {

enum scan_type_t { scan_type_exc = 0, scan_type_inc = 1 };

template<typename T> using plus_t = device::plus_t<T>;
template<typename T> using maximum_t = device::max_t<T>;
template<typename T> using minimum_t = device::min_t<T>;

// Operators the scans and reductions may combine out of element order.  The
// built-in plus, maximum and minimum commute; a caller's own operator that is
// associative and commutative (and has a static identity()) opts in with
//   template<> struct mgpu::gb300::commutative_op<my_op> : std::true_type {};
template<typename op_t> struct commutative_op : std::false_type {};
template<typename T> struct commutative_op<device::plus_t<T>> : std::true_type {};
template<typename T> struct commutative_op<device::max_t<T>> : std::true_type {};
template<typename T> struct commutative_op<device::min_t<T>> : std::true_type {};

// Launch shapes: threads, elements per thread, persistent (1: resident CTAs
// looping over tiles with a deferred look-back, scan_defer_kernel; 0: one
// tile per CTA, scan_kernel), CTAs per SM asked of the compiler.
template<int bytes> struct scan_tuning;
template<> struct scan_tuning<4> { enum { nt = 256, vt = 32, persistent = 1, minb = 4 }; };
template<> struct scan_tuning<8> { enum { nt = 512, vt = 16, persistent = 1, minb = 2 }; };

template<scan_type_t scan_type = scan_type_exc,
  int nt = 0, int vt = 0, int persistent = -1, int minb = -1, typename T,
  typename op_t = plus_t<T>>
status_t scan(void* aux_data, size_t* aux_size, context_t& ctx, const T* in, int64_t count,
  T* out, T init = op_t::identity(), op_t op = op_t(), T* reduction = nullptr) {
  using namespace device;
  static_assert(commutative_op<op_t>::value,
    "scan combines partials out of element order: op must be associative and commutative "
    "(specialise mgpu::gb300::commutative_op for a user operator that is)");
  constexpr int NT = nt ? nt : (int)scan_tuning<sizeof(T)>::nt;
  constexpr int VT = vt ? vt : (int)scan_tuning<sizeof(T)>::vt;
  constexpr int PERSISTENT = persistent >= 0 ? persistent : (int)scan_tuning<sizeof(T)>::persistent;
  constexpr int MINB = minb >= 0 ? minb : (int)scan_tuning<sizeof(T)>::minb;
  constexpr int tile = NT * VT;
  if(count < 0) return MGPU_ERR_INVALID_ARG;
  int64_t num_tiles = div_up(count, tile);
  if(num_tiles > 0x7fffffffll) return MGPU_ERR_INVALID_ARG;
  aux_layout_t lay;
  lay.add(16);                                     // tile counter
  size_t status_off = lay.add(tile_status_t<T>::bytes(num_tiles));
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(count == 0) {
    if(!reduction) return MGPU_OK;
    return ctx.launch("store_value", [&] {
      store_value_kernel<T><<<1, 1, 0, ctx.stream>>>(reduction, init);
    });
  }
  if(!in || !out) return MGPU_ERR_INVALID_ARG;
  if(ctx.check(cudaMemsetAsync(base, 0, lay.total, ctx.stream))) return MGPU_ERR_CUDA;
  tile_status_t<T> status;
  status.bind(base + status_off, num_tiles);
  int vec = aligned16_host(in) && aligned16_host(out);
  const char* name = scan_type == scan_type_exc ? "scan_exc" : "scan_inc";
  if constexpr(PERSISTENT > 0) {
    typedef scan_defer_layout<T, NT, VT> DL;
    auto k = scan_defer_kernel<T, op_t, NT, VT, scan_type == scan_type_exc, MINB>;
    if(!ctx.allow_smem(k, DL::bytes)) return MGPU_ERR_CUDA;
    int per_sm = ctx.resident_ctas(k, NT, DL::bytes);
    if(per_sm < 1) return MGPU_ERR_CUDA;
    // Resident CTAs only, each looping over tiles.
    int64_t grid = std::min<int64_t>((int64_t)per_sm * ctx.sm_count, num_tiles);
    return ctx.launch(name, [&] {
      k<<<(unsigned)grid, NT, DL::bytes, ctx.stream>>>(in, out, count, init, op, status,
        (uint32_t*)base, reduction, ctx.d_error, vec);
    });
  } else {
    return ctx.launch(name, [&] {
      scan_kernel<T, op_t, NT, VT, scan_type == scan_type_exc, MINB>
        <<<(unsigned)num_tiles, NT, 0, ctx.stream>>>(in, out, count, init, op, status,
          (uint32_t*)base, reduction, ctx.d_error, vec);
    });
  }
}

// The reference's in-place form: scan(aux_data, aux_size, cmd, data, count,
// init, op) is exclusive (vk/scan.hxx:12-13).
template<scan_type_t scan_type = scan_type_exc, int nt = 0, int vt = 0, int persistent = -1,
  typename T, typename op_t = plus_t<T>>
status_t scan(void* aux_data, size_t& aux_size, context_t& ctx, T* data, int64_t count,
  T init = op_t::identity(), op_t op = op_t()) {
  return scan<scan_type, nt, vt, persistent>(aux_data, &aux_size, ctx, (const T*)data, count, data, init, op);
}

// The launch shape the reference's scan<nt, vt> knobs select: nt threads
// (rounded up to whole warps, at least two), vt elements per thread rounded up
// to whole 16-byte vectors, on the persistent deferred look-back kernel; CTAs
// per SM from its shared memory (one nt x vt stage) and a 64-register budget.
template<typename T, int nt, int vt>
struct scan_knobs {
  static constexpr int per = 16 / (int)sizeof(T);
  static constexpr int nt_w = (nt + 31) / 32 * 32;
  static constexpr int NT = nt_w < 64 ? 64 : (nt_w > 1024 ? 1024 : nt_w);
  static constexpr int vt_v = (vt + per - 1) / per * per;
  static constexpr int VT = vt_v < per ? per : vt_v;
  static constexpr int by_smem = (int)(233472 / ((size_t)sizeof(T) * NT * VT + 16 + 1024));
  static constexpr int by_regs = 65536 / (NT * 64);
  static constexpr int m = by_smem < by_regs ? by_smem : by_regs;
  static constexpr int MINB = m < 1 ? 1 : (m > 8 ? 8 : m);
};

// The reference's exact template shape, scan<nt, vt>(aux_data, aux_size,
// cmd, data, count, init, op) (vk/scan.hxx:10-13): the in-place exclusive
// scan with the launch shape scan_knobs derives from nt and vt (the reference
// default <128, 7> runs 128 x 8).  The result does not depend on the shape
// beyond float rounding.  (nt and vt have no defaults here, so a call without
// template arguments selects the form above.)
template<int nt, int vt, typename T, typename op_t = plus_t<T>>
status_t scan(void* aux_data, size_t& aux_size, context_t& ctx, T* data, int64_t count,
  T init = op_t::identity(), op_t op = op_t()) {
  typedef scan_knobs<T, nt, vt> S;
  return scan<scan_type_exc, S::NT, S::VT, 1, S::MINB>(aux_data, &aux_size, ctx, (const T*)data,
    count, data, init, op);
}

// Memcache form.
template<scan_type_t scan_type = scan_type_exc, typename T, typename op_t = plus_t<T>>
status_t scan(context_t& ctx, const T* in, int64_t count, T* out, T init = op_t::identity(),
  op_t op = op_t(), T* reduction = nullptr) {
  return scan<scan_type>(nullptr, (size_t*)nullptr, ctx, in, count, out, init, op, reduction);
}

template<int nt = 0, int vt = 0, typename T, typename op_t = plus_t<T>>
status_t reduce(void* aux_data, size_t* aux_size, context_t& ctx, const T* in, int64_t count,
  T* out, T init = op_t::identity(), op_t op = op_t()) {
  using namespace device;
  static_assert(commutative_op<op_t>::value,
    "reduce combines partials out of element order: op must be associative and commutative "
    "(specialise mgpu::gb300::commutative_op for a user operator that is)");
  constexpr int NT = nt ? nt : (int)scan_tuning<sizeof(T)>::nt;
  constexpr int VT = vt ? vt : (int)scan_tuning<sizeof(T)>::vt;
  constexpr int tile = NT * VT;
  if(count < 0) return MGPU_ERR_INVALID_ARG;
  int64_t num_tiles = div_up(count, tile);
  int grid = (int)std::min<int64_t>(std::max<int64_t>(num_tiles, 1), (int64_t)ctx.sm_count * 8);
  aux_layout_t lay;
  lay.add(16);
  size_t part_off = lay.add(sizeof(T) * grid);
  char* base = nullptr;
  status_t st;
  if(resolve_aux(ctx, aux_data, aux_size, lay.total, base, st)) return st;
  if(!out || (count > 0 && !in)) return MGPU_ERR_INVALID_ARG;
  if(ctx.check(cudaMemsetAsync(base, 0, 16, ctx.stream))) return MGPU_ERR_CUDA;
  int vec = aligned16_host(in);
  return ctx.launch("reduce", [&] {
    reduce_kernel<T, op_t, NT, VT><<<grid, NT, 0, ctx.stream>>>(in, count, init, op,
      (T*)(base + part_off), (uint32_t*)base, out, vec);
  });
}

}  // namespace gb300
}  // namespace mgpu
