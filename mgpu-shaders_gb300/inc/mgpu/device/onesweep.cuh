// LSD radix sort for sm_103a: one histogram kernel for all digit places, then
// one single-pass "onesweep" scatter kernel per 8-bit digit.
//
// Reference behaviour (seanbaxter/mgpu-shaders): vk::radix_sort
// (vk/radix.hxx:195-470) runs, per digit, an upsweep histogram, a scan of
// the per-tile counts (radix_scan_8, :13-185) and a downsweep that ranks the
// digits with warp ballots (cta_radix_rank_t<..., radix_kind_ballot>,
// common/cta_radix.hxx:212-351) and scatters through shared memory.  The
// result is a stable LSD sort over radix_permute_t bits.  This file computes
// the same permutation with a different schedule:
//
//  * radix_histogram: every digit place's 256-bin histogram from a single
//    read of the keys (4 B/key instead of one upsweep read per digit).
//  * onesweep_pass: one launch per digit.  Each CTA takes the next tile id
//    from an atomic counter (so every predecessor tile is already resident)
//    and bulk-copies the tile's keys into shared memory with the TMA engine.
//    The kernel is bound by shared-memory traffic and by how many warps and
//    keys each SM holds, so it keeps almost nothing per key in registers:
//    keys are read from the staged tile each time they are needed and ranks
//    are packed 16-bit pairs.  Each half-warp ranks its rows of 16 keys
//    (stable, element order) through one 32-bit word per digit, a 16-bit
//    peer mask under a 16-bit running count; the CTA publishes its per-digit
//    counts and walks back over predecessor tiles' published counts
//    (decoupled look-back, several predecessors per L2 round trip,
//    overlapping the scatter) to find its global offset per digit.
//    Keys are scattered into a second shared-memory region in local digit
//    order and written out in runs, so global stores coalesce; the values'
//    bulk copy reuses the first region once the keys have left it, and the
//    values follow the same permutation.  Per pass the kernel reads and
//    writes each key and value once.
//
// The look-back status of (tile, digit) is one 32-bit word: two flag bits
// (aggregate / inclusive prefix) over a 30-bit count, hence count < 2^30.
#pragma once

#include "common.cuh"
#include <type_traits>

namespace mgpu {
namespace device {

// Value type of a keys-only sort.
struct no_values {};

constexpr int radix_bins = 256;

constexpr uint32_t lb_agg = 1u << 30;
constexpr uint32_t lb_inc = 2u << 30;
constexpr uint32_t lb_count = (1u << 30) - 1;

template<typename K, typename V>
struct onesweep_args {
  typedef typename radix_key<K>::bits_t U;
  const U* keys_in;          // K on the first pass, radix bits after
  U* keys_out;               // radix bits, or K on the last pass
  const V* vals_in;
  V* vals_out;
  int64_t count;
  int shift;                 // bit offset of this pass's digit
  const uint32_t* hist;      // this pass's 256 global digit counts
  uint32_t* lookback;        // this pass's [num_tiles][256] status words
  uint32_t* tile_counter;    // this pass's dynamic tile counter
  int* error;
  int wait_limit = spin_limit;   // polls before a look-back or copy wait gives up
  int first;                 // convert K -> bits on load
  int last;                  // convert bits -> K on store
  int tma;                   // pointers allow 16-byte bulk copies
  // If set, the number of keys is read here at kernel start (clamped to
  // [0, count]); `count` is then the capacity the launch was sized for.
  const int64_t* count_ptr = nullptr;
};

// Shared memory of one onesweep tile of NT threads x ITEMS keys:
//   A  the staged tile: keys (raw on the first pass), later the values; 16
//      spare bytes take the aligned window of a tile that does not start on
//      16 bytes;
//   B  the match words while ranking (1 KB per half-warp), then the keys
//      in local digit order, then the values in that order;
//   W  each half-warp's digit offsets within the tile (16-bit);
//   plus the digits' global bases, scan scratch, the mbarrier and the tile id.
template<typename K, typename V, int NT, int ITEMS>
struct onesweep_layout {
  typedef typename radix_key<K>::bits_t U;
  static constexpr bool has_values = !std::is_same<V, no_values>::value;
  static constexpr int tile = NT * ITEMS;
  static constexpr int num_warps = NT / 32;
  static constexpr size_t elem = has_values && sizeof(V) > sizeof(U) ? sizeof(V) : sizeof(U);
  static constexpr size_t a_off = 0;
  static constexpr size_t b_off = a_off + elem * tile + 16;
  static constexpr size_t w_off = b_off + elem * tile;
  static constexpr size_t w_bytes = (size_t)2 * num_warps * radix_bins * 2;
  static constexpr size_t gbase_off = w_off + w_bytes;
  static constexpr size_t scan_off = gbase_off + sizeof(int) * radix_bins;
  static constexpr size_t bar_off = scan_off + sizeof(uint32_t) * 32;
  static constexpr size_t tile_off = bar_off + sizeof(uint64_t) * 2;
  static constexpr size_t bytes = tile_off + 16;
  static_assert(NT >= radix_bins && NT % 32 == 0, "one thread per digit");
  static_assert((sizeof(U) * tile) % 16 == 0, "bulk-copy granularity");
  static_assert(elem * tile >= (size_t)num_warps * 2 * radix_bins * 4,
    "the half-warps' match words fit in region B");
  static_assert(tile <= 65536, "ranks are packed 16-bit pairs");
};

// Exclusive scan of two 256-entry arrays held by threads 0..255 (one digit
// each).  Every thread of the CTA must call it.
__device__ __forceinline__ void scan_256_pair(uint32_t& x, uint32_t& y, uint32_t* tmp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t xi = x, yi = y;
#pragma unroll
  for(int off = 1; off < 32; off <<= 1) {
    uint32_t tx = __shfl_up_sync(0xffffffffu, xi, off);
    uint32_t ty = __shfl_up_sync(0xffffffffu, yi, off);
    if(lane >= off) { xi += tx; yi += ty; }
  }
  if(tid < radix_bins && lane == 31) { tmp[warp] = xi; tmp[8 + warp] = yi; }
  __syncthreads();
  if(tid < radix_bins) {
    uint32_t px = 0, py = 0;
    for(int w = 0; w < warp; ++w) { px += tmp[w]; py += tmp[8 + w]; }
    x = px + xi - x;
    y = py + yi - y;
  }
}

// Histogram of every digit place in one read.  Each bin has LANES copies
// and lane l updates copy l % LANES, so the 32 lanes of a warp hit 32 (or,
// with 16 copies, at worst 2 x 16) different banks and the shared-memory
// atomics do not conflict; the copies are summed before one global atomic
// per bin and CTA.  Dynamic shared memory: PASSES * 2^BITS * LANES counters
// (BITS: digit width, 8 or 4).
template<typename K, int NT, int PASSES, int LANES, int BITS = 8>
__global__ void __launch_bounds__(NT)
radix_histogram(const K* keys, int64_t count, uint32_t* hist, int vectorised,
  const int64_t* count_ptr) {
  typedef typename radix_key<K>::bits_t U;
  if(count_ptr) count = max((int64_t)0, min(*count_ptr, count));
  constexpr int BINS = PASSES << BITS;
  extern __shared__ __align__(16) uint32_t sh[];
  const int tid = threadIdx.x;
  for(int i = tid; i < BINS * LANES / 4; i += NT)
    reinterpret_cast<uint4*>(sh)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  const int copy = tid % LANES;
  const int64_t gid = (int64_t)blockIdx.x * NT + tid;
  const int64_t stride = (int64_t)gridDim.x * NT;

  auto count_key = [&](K key) {
    U u = radix_key<K>::to_bits(key);
#pragma unroll
    for(int p = 0; p < PASSES; ++p)
      atomicAdd(&sh[((p << BITS) + extract_digit(u, BITS * p, BITS)) * LANES + copy], 1u);
  };
  constexpr int per_vec = 16 / sizeof(K);
  int64_t num_vec = vectorised ? count / per_vec : 0;
  const uint4* kv = (const uint4*)keys;
  // Four 16-byte loads in flight per thread before their keys are counted:
  // with one, the kernel waited on memory latency (45 % of DRAM peak).
  constexpr int UNROLL = 4;
  int64_t i = gid;
  for(; i + (UNROLL - 1) * stride < num_vec; i += UNROLL * stride) {
    uint4 v[UNROLL];
#pragma unroll
    for(int u = 0; u < UNROLL; ++u) v[u] = __ldcs(kv + i + u * stride);
#pragma unroll
    for(int u = 0; u < UNROLL; ++u) {
      const K* e = (const K*)&v[u];
#pragma unroll
      for(int j = 0; j < per_vec; ++j) count_key(e[j]);
    }
  }
  for(; i < num_vec; i += stride) {
    uint4 v = kv[i];
    const K* e = (const K*)&v;
#pragma unroll
    for(int j = 0; j < per_vec; ++j) count_key(e[j]);
  }
  for(int64_t i = num_vec * per_vec + gid; i < count; i += stride) count_key(keys[i]);
  __syncthreads();
  for(int i = tid; i < BINS; i += NT) {
    uint32_t sum = 0;
#pragma unroll 8
    for(int j = 0; j < LANES; ++j) sum += sh[i * LANES + ((i + j) & (LANES - 1))];
    if(sum) atomicAdd(&hist[i], sum);
  }
}

// Where one tile of a sort sits.  A plain sort is one sequence; a segmented
// sort runs one independent sort per large segment over the same kernel.
struct onesweep_tile_t {
  int64_t base;            // first element of the tile (absolute index)
  int valid;               // elements in the tile
  int local;               // tile index within its sort (tile 0 publishes inclusive)
  uint32_t* lb_row;        // this tile's look-back row; predecessor k is lb_row - 256 k
  const uint32_t* hist;    // this pass's 256 digit totals of the tile's sort
  int64_t out_base;        // absolute index of the sort's first element
};

// Claims the next tile id and initialises the tile's mbarrier.  Returns the
// tile id; every thread of the CTA must call it.
template<typename K, typename V, int NT, int ITEMS>
__device__ __forceinline__ int onesweep_begin(uint32_t* tile_counter, unsigned char* smem) {
  typedef onesweep_layout<K, V, NT, ITEMS> L;
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);
  int* s_tile = (int*)(smem + L::tile_off);
  if(threadIdx.x == 0) {
    *s_tile = (int)atomicAdd(tile_counter, 1u);
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  return *s_tile;
}

// Orders this thread's earlier generic-proxy accesses to shared memory
// before its later bulk copies (async proxy) into the same bytes.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Decoupled look-back of one digit: the sum of the counts of all predecessor
// tiles.  `pred` is this digit's word in the nearest predecessor's row; there
// are `num_pred` predecessors, ROW words apart.  issue() loads the status of
// the nearest WINDOW predecessors (one L2 round trip) early, so its latency
// overlaps other work; finish() consumes them in order (aggregates are added,
// an inclusive prefix ends the walk, an unpublished status stops the round)
// and continues, if needed, with rounds of WIDE predecessors each.  On a
// 2^28-key sort the walk reaches back about 20 tiles in 5-6 rounds; rounds of
// 16 or 32 predecessors took fewer rounds but longer ones, and the walks grew,
// so WIDE stays 4.  Bounded.  ROW: status words per tile (one per digit: 256
// for 8-bit digits, 16 for 4-bit ones).
template<int WINDOW, int WIDE = 4, int ROW = radix_bins>
struct lookback_window_t {
  uint32_t s[WINDOW];
  const uint32_t* pred;
  int left;

  __device__ __forceinline__ void issue(const uint32_t* p, int num_pred) {
    pred = p;
    left = num_pred;
#pragma unroll
    for(int k = 0; k < WINDOW; ++k)
      s[k] = k < left ? ld_relaxed(pred - k * ROW) : lb_inc;
  }
  // Consumes statuses in order; returns true when an inclusive prefix ended
  // the walk, else advances `pred` / `left` past the aggregates used and
  // sets `stalled` if an unpublished status stopped the round.
  template<int N>
  __device__ __forceinline__ bool consume(const uint32_t (&w)[N], uint32_t& excl, bool& stalled) {
    int used = 0;
    bool done = false;
    stalled = false;
#pragma unroll
    for(int k = 0; k < N; ++k) {
      if(!done && !stalled) {
        const uint32_t flag = w[k] & ~lb_count;
        if(!flag) {
          stalled = true;
        } else {
          excl += w[k] & lb_count;
          ++used;
          done = flag == lb_inc;
        }
      }
    }
    pred -= used * ROW;
    left -= used;
    return done;
  }
  __device__ __forceinline__ uint32_t finish(int* error, int limit) {
    uint32_t excl = 0;
    bool stalled;
    if(consume(s, excl, stalled)) return excl;
    int spins = 0;
    while(true) {
      if(stalled) {
        ++spins;
        if(spins >= limit ||
           (0 == (spins & (spin_poll_error - 1)) && error_raised(error))) {
          raise_error(error, err_lookback_timeout);
          return excl;
        }
        // The predecessor has not published yet: yield issue slots to the
        // other warps on this SM for a short while before polling again.
        __nanosleep(128);
      }
      uint32_t w[WIDE];
#pragma unroll
      for(int k = 0; k < WIDE; ++k)
        w[k] = k < left ? ld_relaxed(pred - k * ROW) : lb_inc;
      if(consume(w, excl, stalled)) return excl;
    }
  }
};

// UNALIGNED: tiles may start anywhere (the segmented sort's large segments);
// a plain sort's tiles start on whole tiles, so it skips the window logic.
template<typename K, typename V, int NT, int ITEMS, int WINDOW = 4, bool UNALIGNED = false>
__device__ __forceinline__ void onesweep_tile(const onesweep_args<K, V>& a,
  const onesweep_tile_t& t, unsigned char* smem) {
  typedef onesweep_layout<K, V, NT, ITEMS> L;
  typedef typename L::U U;
  constexpr int TILE = L::tile;
  constexpr int NWARPS = L::num_warps;
  constexpr bool HAS_V = L::has_values;
  constexpr int CHUNK = 4;                  // write-out: loads in flight per thread

  unsigned char* A = smem + L::a_off;
  unsigned char* B = smem + L::b_off;
  uint16_t* W = (uint16_t*)(smem + L::w_off);
  int* gbase = (int*)(smem + L::gbase_off);
  uint32_t* stmp = (uint32_t*)(smem + L::scan_off);
  uint64_t* bar = (uint64_t*)(smem + L::bar_off);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = t.base;
  const int valid = t.valid;
  const int tile = t.local;
  // a.tma: both arrays start on 16 bytes.  The tile's keys are bulk-copied
  // as the 16-byte-aligned window [kstart, kend) around it (the tile starts
  // koff elements in); values likewise.  A full tile whose whole window lies
  // inside the array copies it all; otherwise (a ragged last tile) the window
  // ends at the last whole 16 bytes before the tile's end, and threads load
  // the positions after it with plain loads.  Without UNALIGNED a tile must
  // start on 16 bytes to be copied.
  constexpr int64_t KV = 16 / sizeof(U);
  constexpr int64_t VV = HAS_V ? 16 / sizeof(V) : 1;
  auto window = [&](int64_t per_vec, int64_t& start, int64_t& end) -> bool {
    start = UNALIGNED ? (base & ~(per_vec - 1)) : base;
    if(!UNALIGNED && (base & (per_vec - 1))) return false;
    const int64_t full = (base + TILE + per_vec - 1) & ~(per_vec - 1);
    end = valid == TILE && full <= a.count ? full : (base + valid) & ~(per_vec - 1);
    return a.tma && end > base;
  };
  int64_t kstart = base, kend = base, vstart = base, vend = base;
  const bool bulk_k = window(KV, kstart, kend);
  const bool bulk_v = HAS_V && window(VV, vstart, vend);
  const int koff = bulk_k ? (int)(base - kstart) : 0;
  const int voff = bulk_v ? (int)(base - vstart) : 0;
  // Tile positions from kfill (vfill) on are loaded by the threads.
  const int kfill = bulk_k ? (int)min((int64_t)TILE, kend - base) : 0;
  const int vfill = bulk_v ? (int)min((int64_t)TILE, vend - base) : 0;
  const uint32_t vparity = bulk_k ? 1 : 0;       // mbarrier phase of the values' copy

  if(bulk_k && tid == 0) {
    const uint32_t kbytes = (uint32_t)(sizeof(U) * (kend - kstart));
    mbar_arrive_expect_tx(bar, kbytes);
    bulk_load(A, a.keys_in + kstart, kbytes, bar);
  }

  // This warp's match words (its two half-warps' 256 words each), in B.
  uint32_t* mw = (uint32_t*)B + warp * 2 * radix_bins;
  for(int j = lane; j < 2 * radix_bins / 4; j += 32)
    reinterpret_cast<uint4*>(mw)[j] = make_uint4(0, 0, 0, 0);

  // Concentration of this pass's digits: when some digit holds more than
  // 1/128 of the keys, rows of 16 equal digits become likely (equal keys sit
  // together after earlier passes) and the ranking checks for them.  Warp
  // maxima and sums of the digit totals go to scan scratch words 16..31.
  uint32_t hval = 0;
  if(tid < radix_bins) {
    hval = t.hist[tid];
    const uint32_t m = __reduce_max_sync(0xffffffffu, hval);
    const uint32_t sum = __reduce_add_sync(0xffffffffu, hval);
    if(lane == 0) { stmp[16 + warp] = m; stmp[24 + warp] = sum; }
  }

  // Ranking rows are 16 lanes wide: each half-warp (a "virtual warp" vw)
  // owns the contiguous run of 16 * rpv elements, and item i < rpv of this
  // thread is element vw * 16 * rpv + 16 * i + (lane & 15).  A full tile has
  // rpv = ITEMS rows per half-warp (an odd ITEMS puts the two halves' runs 16
  // banks apart); a partial tile of the segmented sort (most large segments
  // end in one) spreads its elements evenly over all half-warps with fewer
  // rows, so it costs in proportion to its size (seg_onesweep_pass 2.91 ->
  // 2.64 ms on 10^5 lognormal segments).  Item i is in range while RS * i <
  // rem.
  constexpr int RS = 16;
  constexpr int NVW = 2 * NWARPS;
  // (Only the segmented sort spreads: in a plain sort only the last tile is
  // partial, and a compile-time row count keeps the loops free of checks.)
  const int rpv = (!UNALIGNED || valid == TILE) ? ITEMS
                                : max(1, min(ITEMS, (valid + RS * NVW - 1) / (RS * NVW)));
  const int vw = 2 * warp + (lane >> 4);
  const int rl = lane & 15;                              // lane within the row
  const int thr_base = vw * RS * rpv + rl;
  const int rem = valid - thr_base;
  U* const ak = (U*)A + koff + thr_base;                 // this thread's staged keys
  if(kfill < TILE) {
    // Plain loads; positions past the tile's end take the largest radix
    // bits, so they rank last (after every real key with digit 255).
    U fill = ~(U)0;
    if(a.first) {
      const K k = radix_key<K>::from_bits(~(U)0);
      memcpy(&fill, &k, sizeof(U));
    }
    const U* src = a.keys_in + base + thr_base;
#pragma unroll 4
    for(int i = 0; i < ITEMS; ++i)
      if(i < rpv && thr_base + RS * i >= kfill) ak[RS * i] = RS * i < rem ? src[RS * i] : fill;
  }
  {
    // Only warp 0 polls the barrier; the other warps sleep at the CTA
    // barrier below instead of spending issue slots.  The mbarrier phase
    // completion makes the copied bytes visible to warp 0, and the CTA
    // barrier passes that on to every thread.
    bool ok = true;
    if(bulk_k && warp == 0) ok = mbar_wait_bounded(bar, 0, a.error, a.wait_limit);
    if(__syncthreads_or(!ok)) {
      // The copy did not complete in time: wait once more (bounded) so no
      // bulk copy is still writing this CTA's shared memory, then leave.
      if(warp == 0) mbar_wait_bounded(bar, 0, a.error, a.wait_limit);
      return;
    }
  }
  bool check_uniform;
  {
    uint32_t mx = 0, total = 0;
#pragma unroll
    for(int w = 0; w < radix_bins / 32; ++w) { mx = max(mx, stmp[16 + w]); total += stmp[24 + w]; }
    check_uniform = (uint64_t)mx * 128 > total;
  }
  // Radix bits of item i (the staged copy holds raw keys on the first pass).
  auto key_bits = [&](int i) -> U {
    U u = ak[RS * i];
    if(a.first) {
      K key;
      memcpy(&key, &u, sizeof(K));
      u = radix_key<K>::to_bits(key);
    }
    return u;
  };

  // Stable ranking by half-warps: item i of the 16 lanes of a half forms one
  // row; lanes holding equal digits are peers.  Per (half-warp, digit) one
  // 32-bit word: the low half collects the row's peer mask (every lane ORs
  // its bit in), the high half is the half-warp's running count.  A lane reads
  // both in one load; the lowest peer writes back the advanced count with a
  // cleared mask.  Three 32-bit shared-memory operations per key (32-lane rows
  // need a 64-bit mask + count word, whose random accesses cost about 1.6x the
  // wavefronts: 1.295 -> 1.240 ms per 2^28 pass).  The rank counts earlier
  // rows and lower lanes of the same row (element order).  Ranks (< 2^16) are
  // kept as packed pairs.
  uint32_t rp[(ITEMS + 1) / 2];
  {
    uint32_t* mv = (uint32_t*)B + vw * radix_bins;
    const uint32_t lt_mask = (1u << rl) - 1;
    const uint32_t lane_bit = 1u << rl;
#pragma unroll
    for(int i = 0; i < ITEMS; ++i) {
      if(i >= rpv) continue;
      const uint32_t d = extract_digit(key_bits(i), a.shift, 8);
      uint32_t rank;
      if(check_uniform && __all_sync(0xffffffffu, d == __shfl_sync(0xffffffffu, d, lane & 16))) {
        // One digit across each half-row (common once equal keys sit
        // together): the peers are the whole half, same-address atomics are
        // skipped, and its lane 0 advances the count.
        uint32_t* cw = &mv[d];
        const uint32_t cnt = *cw >> 16;
        __syncwarp();
        if(rl == 0) *cw = (cnt + 16) << 16;
        __syncwarp();
        rank = cnt + rl;
      } else {
        atomicOr(&mv[d], lane_bit);
        __syncwarp();
        const uint32_t w = mv[d];
        __syncwarp();
        const uint32_t peers = w & 0xffffu, cnt = w >> 16;
        const uint32_t below = peers & lt_mask;
        if(!below) mv[d] = (cnt + __popc(peers)) << 16;
        __syncwarp();
        rank = cnt + __popc(below);
      }
      if(i & 1) rp[i >> 1] |= rank << 16;
      else rp[i >> 1] = rank;
    }
  }
  __syncthreads();

  // Digit `tid`: counts per (virtual) warp -> exclusive offsets over them;
  // publish the tile's count (inclusive for tile 0) before scanning, so
  // successors can proceed as early as possible.
  auto vw_count = [&](int w) -> uint32_t {
    return ((const uint32_t*)B)[w * radix_bins + tid] >> 16;
  };
  uint32_t tile_cnt = 0, valid_cnt = 0;
  if(tid < radix_bins) {
#pragma unroll
    for(int w = 0; w < NVW; ++w) tile_cnt += vw_count(w);
    // Padding positions (all-ones bits, digit 255) ranked after the real keys.
    valid_cnt = tile_cnt - (tid == radix_bins - 1 ? (uint32_t)(RS * NVW * rpv - valid) : 0u);
    st_relaxed(&t.lb_row[tid], (tile ? lb_agg : lb_inc) | valid_cnt);
  }
  uint32_t tile_start = tile_cnt, glob_start = hval;
  scan_256_pair(tile_start, glob_start, stmp);

  // Issue the first look-back window now; its L2 round trip overlaps the
  // key scatter below.  Each (virtual) warp's offset of each digit within the
  // tile goes to W (16-bit entries with 16-lane rows).
  lookback_window_t<WINDOW> lbw;
  if(tid < radix_bins) {
    if(tile > 0) lbw.issue(t.lb_row + tid - radix_bins, tile);
    uint32_t run = tile_start;
#pragma unroll
    for(int w = 0; w < NVW; ++w) {
      const uint32_t c = vw_count(w);
      W[w * radix_bins + tid] = (uint16_t)run;
      run += c;
    }
  }
  __syncthreads();

  // Keys into B in local digit order; the ranks become local positions.
  {
    const uint16_t* wh = W + vw * radix_bins;
#pragma unroll
    for(int i = 0; i < ITEMS; ++i) {
      if(i >= rpv) continue;
      const U k = key_bits(i);
      const uint32_t sh = (i & 1) * 16;
      const uint32_t dg = extract_digit(k, a.shift, 8);
      const uint32_t r = ((rp[i >> 1] >> sh) & 0xffffu) + wh[dg];
      rp[i >> 1] = (rp[i >> 1] & ~(0xffffu << sh)) | (r << sh);
      ((U*)B)[r] = k;
    }
  }
  __syncthreads();
  // A is free: the values' bulk copy overlaps the look-back and the key
  // write-out.
  if(bulk_v && tid == 0) {
    const uint32_t vbytes = (uint32_t)(sizeof(V) * (vend - vstart));
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, vbytes);
    bulk_load(A, a.vals_in + vstart, vbytes, bar);
  }

  // Finish the look-back, publish the inclusive prefix, and form each
  // digit's global base (global digit start + predecessors - local start).
  if(tid < radix_bins) {
    uint32_t excl = 0;
    if(tile > 0) {
      excl = lbw.finish(a.error, a.wait_limit);
      st_relaxed(&t.lb_row[tid], lb_inc | (excl + valid_cnt));
    }
    gbase[tid] = (int)(glob_start + excl - tile_start);
  }
  __syncthreads();

  // Write out in local order: consecutive threads hit consecutive addresses
  // inside each digit's run.  CHUNK loads, then CHUNK stores.  The values
  // are written out by the same threads at the same positions, so each
  // thread keeps its positions' digits, packed four per register.
  U* keys_out = a.keys_out + t.out_base;
  uint32_t dq[(ITEMS + 3) / 4];
#pragma unroll
  for(int j0 = 0; j0 < ITEMS; j0 += CHUNK) {
    U u[CHUNK];
    uint32_t dst[CHUNK];
#pragma unroll
    for(int c = 0; c < CHUNK; ++c) {
      const int idx = (j0 + c) * NT + tid;
      if(j0 + c < ITEMS && idx < valid) {
        u[c] = ((const U*)B)[idx];
        const uint32_t d = extract_digit(u[c], a.shift, 8);
        const int j = j0 + c;
        if(HAS_V) dq[j >> 2] = (j & 3) ? dq[j >> 2] | (d << (8 * (j & 3))) : d;
        dst[c] = (uint32_t)gbase[d] + idx;
      }
    }
#pragma unroll
    for(int c = 0; c < CHUNK; ++c) {
      if(j0 + c < ITEMS && (j0 + c) * NT + tid < valid) {
        if(a.last) {
          K key = radix_key<K>::from_bits(u[c]);
          // Convert in registers and store one word (a memcpy straight to
          // global memory may be split into narrow stores).
          U out;
          memcpy(&out, &key, sizeof(U));
          keys_out[dst[c]] = out;
        } else {
          keys_out[dst[c]] = u[c];
        }
      }
    }
  }
  if constexpr(HAS_V) {
    V* const av = (V*)A + voff + thr_base;             // this thread's staged values
    // The sorted keys must have left B, and (when copied) the values arrived.
    bool ok = true;
    if(bulk_v && warp == 0) ok = mbar_wait_bounded(bar, vparity, a.error, a.wait_limit);
    if(__syncthreads_or(!ok)) {
      if(warp == 0) mbar_wait_bounded(bar, vparity, a.error, a.wait_limit);
      return;
    }
    if(vfill < valid) {
      const V* src = a.vals_in + base + thr_base;
#pragma unroll 4
      for(int i = 0; i < ITEMS; ++i)
        if(i < rpv && RS * i < rem && thr_base + RS * i >= vfill) av[RS * i] = src[RS * i];
      __syncwarp();                        // each warp reads only its own rows
    }
#pragma unroll
    for(int i = 0; i < ITEMS; ++i)
      if(i < rpv && RS * i < rem) ((V*)B)[(rp[i >> 1] >> ((i & 1) * 16)) & 0xffffu] = av[RS * i];
    __syncthreads();
    V* vals_out = a.vals_out + t.out_base;
#pragma unroll
    for(int j0 = 0; j0 < ITEMS; j0 += CHUNK) {
      V v[CHUNK];
      uint32_t dst[CHUNK];
#pragma unroll
      for(int c = 0; c < CHUNK; ++c) {
        const int idx = (j0 + c) * NT + tid;
        if(j0 + c < ITEMS && idx < valid) {
          const int j = j0 + c;
          v[c] = ((const V*)B)[idx];
          dst[c] = (uint32_t)gbase[(dq[j >> 2] >> (8 * (j & 3))) & 0xffu] + idx;
        }
      }
#pragma unroll
      for(int c = 0; c < CHUNK; ++c)
        if(j0 + c < ITEMS && (j0 + c) * NT + tid < valid) vals_out[dst[c]] = v[c];
    }
  }
}

template<typename K, typename V, int NT, int ITEMS, int MIN_BLOCKS, int WINDOW = 4,
  bool DEV_COUNT = false>
__global__ void __launch_bounds__(NT, MIN_BLOCKS)
onesweep_pass(onesweep_args<K, V> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int TILE = NT * ITEMS;
  // DEV_COUNT: the count is read from device memory; the grid covers the
  // capacity, and CTAs that claim a tile id past the last tile leave (ids
  // are claimed in order, so no tile waits on them).
  if constexpr(DEV_COUNT) a.count = max((int64_t)0, min(*a.count_ptr, a.count));
  const int tile = onesweep_begin<K, V, NT, ITEMS>(a.tile_counter, smem);
  if constexpr(DEV_COUNT)
    if((int64_t)tile * TILE >= a.count) return;
  onesweep_tile_t t;
  t.base = (int64_t)tile * TILE;
  t.valid = (int)min((int64_t)TILE, a.count - t.base);
  t.local = tile;
  t.lb_row = a.lookback + (int64_t)tile * radix_bins;
  t.hist = a.hist;
  t.out_base = 0;
  onesweep_tile<K, V, NT, ITEMS, WINDOW>(a, t, smem);
}

}  // namespace device
}  // namespace mgpu
