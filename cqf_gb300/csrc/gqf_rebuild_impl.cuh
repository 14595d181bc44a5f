// Region rebuild: the bulk insert / delete hot path.
//
// The reference applies a batch with one thread per 8192-slot region that
// inserts its sorted keys one at a time, shifting slots byte by byte
// (insert_from_buffers_hashed / delete_from_buffers_hashed,
// src/gqf.cu:2759-2906, two launches: even regions then odd).  The layout
// that produces is canonical: it depends only on the multiset of
// (quotient, remainder, count), never on the order of operations.  So this
// kernel rebuilds a region's layout in one pass instead:
//
//   * one CTA per region of 2^LOGS quotients, even regions then odd ones (the
//     reference's schedule), so two CTAs never touch the same slots;
//   * the CTA stages a window in shared memory: the region plus the head of
//     the next one, which its growth may push.  A first launch per parity
//     uses a short head (TAIL slots), enough for almost every region; a
//     second launch takes the regions it could not hold with the full head
//     (PUSH slots);
//   * it groups the region's new keys by quotient with a counting sort in
//     shared memory, merges them with the old counters of the touched runs
//     only (decode_counter / encode_counter, src/gqf.cu:1216-1345), and
//     recomputes every run position with one block-wide max-plus scan:
//     end(q) = max(q + L_q - 1, end(prev) + L_q);
//   * untouched runs move byte-parallel (every slot knows its run's shift);
//   * it writes back only the blocks that changed.
//
// A rebuild whose changes would reach past the full window (a cluster longer
// than PUSH slots, or the end of the table) is deferred: nothing is written and the
// region is applied afterwards by a single-thread serial pass built from the
// reference's own single-key algorithms (gqf_device.cuh), which handles any
// cluster length and reports a full table like the reference does.
#pragma once
#include <algorithm>
#include <type_traits>

#include "gqf_kernels.cuh"

namespace gqf {
namespace {

constexpr int kNeg = -(1 << 28);  // "minus infinity" of the max-plus scan

// OR of a 64-bit mask into a shared-memory word as native 32-bit atomics on
// the halves that carry bits.
__device__ __forceinline__ void or64(unsigned long long* p, unsigned long long v) {
  uint32_t* h = reinterpret_cast<uint32_t*>(p);
  if ((uint32_t)v) atomicOr(h, (uint32_t)v);
  if ((uint32_t)(v >> 32)) atomicOr(h + 1, (uint32_t)(v >> 32));
}
// Sets bit i of a shared-memory bitmap of 64-bit words.
__device__ __forceinline__ void set_bit(unsigned long long* m, int i) {
  atomicOr(reinterpret_cast<uint32_t*>(m) + (i >> 5), 1u << (i & 31));
}

// Bulk staging of a window: one thread starts a cp.async.bulk copy from
// global into this CTA's shared memory that completes on an mbarrier, while
// the other threads clear their tables; then all wait on the barrier's phase.
// The wait is bounded (kStageSpin polls): a copy that never lands makes the
// region fall back to the serial path and sets the timeout status bit.
struct BulkStage {
  unsigned long long* bar;  // mbarrier in shared memory, one arrival per phase
  uint32_t phase;           // the phase the next copy completes
  uint32_t* status;
};
constexpr uint32_t kStageSpin = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}

// Thread 0: copies `bytes` (a multiple of 16, both addresses 16-byte
// aligned) from src to dst and arms the barrier for them.
__device__ __forceinline__ void bulk_stage_start(const BulkStage& sg, void* dst, const void* src, uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of dst come first
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(sg.bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(sg.bar))
      : "memory");
}

// All threads: waits for the copy; false when the wait ran out.
__device__ __forceinline__ bool bulk_stage_wait(BulkStage& sg) {
  uint32_t done = 0;
  for (uint32_t i = 0; i < kStageSpin && !done; i++) {
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(sg.bar)), "r"(sg.phase)
        : "memory");
  }
  sg.phase ^= 1u;
  if (!done && threadIdx.x == 0) atomicOr(sg.status, kStTimeout);
  return done != 0;
}

template <int LOGS>
struct Cfg;
// PUSH: the slots past the region a window holds; TAIL: the shorter tail
// tried first, enough whenever the region's growth is absorbed that close;
// MINB: CTAs per SM the full-window kernels are built for; MINB_INS /
// MINB_CNT: the short-window insert and delete / counted-insert kernels'
// (their shared memory allows five / four at 2^11 and 2^12 quotients; the
// delete kernel keeps its quotient and slot loops rolled to fit 48
// registers).
template <>
struct Cfg<11> {
  static constexpr int PUSH = 1024, TAIL = 256, KMAX = 2048, MINB = 4, MINB_INS = 5, MINB_CNT = 4;
};
template <>
struct Cfg<12> {
  static constexpr int PUSH = 2048, TAIL = 256, KMAX = 2048, MINB = 4, MINB_INS = 5, MINB_CNT = 4;
};
template <>
struct Cfg<13> {
  static constexpr int PUSH = 2048, TAIL = 256, KMAX = 4096, MINB = 2, MINB_INS = 2, MINB_CNT = 2;
};
// CTAs per SM a rebuild kernel is built for.
template <int LOGS, bool DEL, bool CNT, int SPAN>
constexpr int rebuild_min_blocks() {
  constexpr bool kShort = SPAN < (1 << LOGS) + Cfg<LOGS>::PUSH;
  return CNT ? (kShort ? Cfg<LOGS>::MINB_CNT : 3) : (kShort ? Cfg<LOGS>::MINB_INS : Cfg<LOGS>::MINB);
}

// The layout of one kernel's shared memory.  Its tables are sized for the
// window span TS the kernel works in (the short or the full window), so the
// short-window kernels take less shared memory and more of them fit an SM.
template <int LOGS, bool CNT, int TS = (1 << LOGS) + Cfg<LOGS>::PUSH>
struct Lay {
  static constexpr int NT = 256;
  static constexpr int REG = 1 << LOGS;
  static constexpr int PUSH = Cfg<LOGS>::PUSH;
  static constexpr int KMAX = Cfg<LOGS>::KMAX;
  static constexpr int WIN = REG + PUSH;
  static constexpr int SHORT = REG + Cfg<LOGS>::TAIL;
  static constexpr int WB = TS / 64;
  static constexpr int KCW = REG / 2 + 2;  // packed 16-bit per-quotient key counters
  static_assert(WIN % NT == 0 && SHORT % NT == 0 && SHORT <= WIN && (REG / 2) % NT == 0,
                "work splits evenly over threads");
  static_assert(TS % NT == 0 && TS >= SHORT && TS <= WIN, "a table span is the short or the full window");
  static_assert(KCW * 4 <= (TS + 8) * 2, "the key counters fit the shift table they share");
  static_assert(PUSH < REG, "a window must not reach the region after next");
  static_assert(WIN + PUSH + 64 < 32767, "window positions fit int16");
  static_assert(WB < NT, "window words fit one scan");
  static_assert(WIN + PUSH < 16384, "shifts and old starts fit apart in int16");
  // shared memory carve-up (bytes)
  static constexpr int IMG = WB * 96;
  static constexpr int OFF_IMG0 = 0;
  static constexpr int OFF_IMG1 = OFF_IMG0 + IMG;
  static constexpr int OFF_KG = OFF_IMG1 + IMG;                  // u32[KMAX] keys grouped by quotient
  static constexpr int OFF_PREF = OFF_KG + KMAX * 4;             // u16[TS] lengths, then ends + 1
  // one table, three lives: the key counters while the keys are grouped,
  // then the old run ends by rank, then each old run's start and shift
  static constexpr int OFF_DELTA = OFF_PREF + TS * 2;            // i16[TS + 8]
  static constexpr int OFF_KC = OFF_DELTA;                       // u32[KCW]
  static constexpr int OFF_RPOS = OFF_DELTA;                     // u16[TS + 8]
  // the single-round kernel keeps two u16 per key in the same table
  static constexpr int DELTA_BYTES = (TS + 8) * 2 > 4 * KMAX ? (TS + 8) * 2 : 4 * KMAX;
  static constexpr int OFF_NOCC = (OFF_DELTA + DELTA_BYTES + 7) & ~7;  // u64[WB] new occupieds
  static constexpr int OFF_TCH = OFF_NOCC + WB * 8;              // u64[WB] touched quotients
  static constexpr int OFF_ORANK = OFF_TCH + WB * 8;             // u16[WB + 8]
  static constexpr int OFF_RRANK = OFF_ORANK + (WB + 8) * 2;     // u16[WB + 8]
  static constexpr int OFF_KN = (OFF_RRANK + (WB + 8) * 2 + 3) & ~3;  // u32[KMAX] key counts (CNT)
  static constexpr int BYTES = OFF_KN + (CNT ? KMAX * 4 : 0);
};

// A run rewritten by its merge keeps kTouched + its old start in the shift
// table; untouched runs hold their shift, always below kTouched.
constexpr int kTouched = 16384;
// The work list of one phase lives in the partition's cursor array (free once
// the keys are scattered): [0] regions listed by k_sparse, [1] the next one
// a rebuild CTA takes, [2 ...] the region indices.
constexpr int kListCount = 0, kListNext = 1, kListBase = 2;

// ----------------------------------------------------- shared-memory image

// A window in shared memory in split form: the slots contiguous (slot i of
// the window at s[i]) and the blocks' 32-byte headers after them (header w
// at h + 32 w: occupieds, runends, offset), so that the per-slot loops index
// one byte instead of recomputing a block address.  The image of WB blocks
// takes the same 96 WB bytes as the blocks themselves.
struct Img {
  uint8_t* s;
  uint8_t* h;
  __device__ uint8_t& slot(int i) const { return s[i]; }
  __device__ unsigned long long& occ(int w) const { return *reinterpret_cast<unsigned long long*>(h + w * 32); }
  __device__ unsigned long long& run(int w) const { return *reinterpret_cast<unsigned long long*>(h + w * 32 + 8); }
  __device__ uint32_t& off(int w) const { return *reinterpret_cast<uint32_t*>(h + w * 32 + 16); }
  __device__ int is_end(int i) const { return (int)((run(i >> 6) >> (i & 63)) & 1ULL); }
  // The place in this image of 16-byte word i of the same window laid out
  // as blocks (word 6 w + c of block w: c = 0, 1 its header, 2-5 its slots).
  __device__ uint4& part(int i) const {
    const int w = i / 6, c = i - 6 * w;
    return c < 2 ? reinterpret_cast<uint4*>(h + w * 32)[c] : reinterpret_cast<uint4*>(s + w * 64)[c - 2];
  }
};
// The image of a window of WB blocks at `base` (16-byte aligned).
template <int WB>
__device__ __forceinline__ Img img_at(uint8_t* base) {
  return Img{base, base + WB * 64};
}

// Merge one run's old counters with the run's new keys (sorted by remainder;
// each key counts once, or cnts[j] times when cnts is given) and return the
// new run length; with WRITE, also emit the bytes at out[pos..].
template <bool DEL, bool WRITE>
__device__ int merge_run(Img cur, bool has_old, int s, int e, const uint32_t* keys, const uint32_t* cnts,
                         int ki, int kj, Img out, int pos) {
  if (!cnts && kj == ki + 1) {  // one key, counted once: the common case
    const int r = (int)(keys[ki] & 255u);
    if (!has_old) {
      if (DEL) return 0;
      if (WRITE) out.slot(pos) = (uint8_t)r;
      return 1;
    }
    // Remainders that strictly increase along the run are all counted once
    // (a counter of two or more repeats its remainder or steps down after
    // it), so the key only adds or drops one slot.
    int prev = -1, at = -1, ins = e + 1;
    bool single = true;
    for (int t = s; t <= e; t++) {
      const int v = cur.slot(t);
      if (v <= prev) { single = false; break; }
      if (v == r) at = t;
      if (v > r && ins > e) ins = t;
      prev = v;
    }
    if (single && (DEL || at < 0)) {
      const int len = e - s + 1;
      if (DEL && at < 0) {  // not in the run: nothing changes
        if (WRITE)
          for (int t = 0; t < len; t++) out.slot(pos + t) = cur.slot(s + t);
        return len;
      }
      if (DEL) {
        if (WRITE)
          for (int t = s, o = pos; t <= e; t++)
            if (t != at) out.slot(o++) = cur.slot(t);
        return len - 1;
      }
      if (WRITE) {
        int o = pos;
        for (int t = s; t < ins; t++) out.slot(o++) = cur.slot(t);
        out.slot(o++) = (uint8_t)r;
        for (int t = ins; t <= e; t++) out.slot(o++) = cur.slot(t);
      }
      return len + 1;
    }
  }
  auto get = [&](uint64_t i) -> uint64_t { return cur.slot((int)i); };
  auto end = [&](uint64_t i) -> int { return cur.is_end((int)i); };
  const uint64_t lim = (uint64_t)e + 1;  // the walk never leaves the run [s, e]
  int total = 0;
  bool have_old = has_old;
  int opos = s;
  uint32_t orem = 0;
  uint64_t ocnt = 0;
  int oend = 0;
  if (have_old) oend = (int)decode_counter(get, end, (uint64_t)opos, &orem, &ocnt, lim);
  int j = ki;
  uint8_t enc[16];
  while (have_old || j < kj) {
    uint32_t nrem = 0;
    uint64_t ncnt = 0;
    int jn = j;
    if (j < kj) {
      nrem = keys[j] & 255u;
      while (jn < kj && (keys[jn] & 255u) == nrem) {
        ncnt += cnts ? cnts[jn] : 1u;
        jn++;
      }
    }
    bool take_old = have_old && (j >= kj || orem < nrem);
    bool both = have_old && j < kj && orem == nrem;
    if (take_old) {
      int len = oend - opos + 1;
      if (WRITE)
        for (int t = 0; t < len; t++) out.slot(pos + total + t) = cur.slot(opos + t);
      total += len;
    } else {
      uint64_t c = both ? (DEL ? (ocnt > ncnt ? ocnt - ncnt : 0) : ocnt + ncnt) : (DEL ? 0 : ncnt);
      int len = encode_counter(nrem, c, enc);
      if (WRITE)
        for (int t = 0; t < len; t++) out.slot(pos + total + t) = enc[t];
      total += len;
      j = jn;
    }
    if (take_old || both) {
      if (cur.is_end(oend) || oend >= e) {
        have_old = false;
      } else {
        opos = oend + 1;
        oend = (int)decode_counter(get, end, (uint64_t)opos, &orem, &ocnt, lim);
      }
    }
  }
  return total;
}

// Block-wide exclusive scan of max-plus maps f(x) = max(a, x + b).  Both
// parts saturate at kNeg ("minus infinity"), so maps that reset their
// argument (b = kNeg) compose without overflow.
__device__ __forceinline__ int sat(int v) { return max(v, kNeg); }
template <int NT>
__device__ void scan_maps(int& a, int& b, int* sa, int* sb) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int ia = a, ib = b;  // inclusive
  for (int o = 1; o < 32; o <<= 1) {
    int pa = __shfl_up_sync(0xffffffffu, ia, o);
    int pb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {  // (pa,pb) first, then (ia,ib)
      ia = max(ia, sat(pa + ib));
      ib = sat(pb + ib);
    }
  }
  if (lane == 31) { sa[wid] = ia; sb[wid] = ib; }
  __syncthreads();
  if (wid == 0) {
    int wa = lane < NT / 32 ? sa[lane] : kNeg, wb = lane < NT / 32 ? sb[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int pa = __shfl_up_sync(0xffffffffu, wa, o);
      int pb = __shfl_up_sync(0xffffffffu, wb, o);
      if (lane >= o) { wa = max(wa, sat(pa + wb)); wb = sat(pb + wb); }
    }
    sa[lane] = wa;
    sb[lane] = wb;
  }
  __syncthreads();
  int ea = __shfl_up_sync(0xffffffffu, ia, 1), eb = __shfl_up_sync(0xffffffffu, ib, 1);
  if (lane == 0) { ea = kNeg; eb = 0; }
  if (wid > 0) {
    int pa = sa[wid - 1], pb = sb[wid - 1];
    ea = max(ea, sat(pa + eb));
    eb = sat(pb + eb);
  }
  a = ea;
  b = eb;
  __syncthreads();
}

// Block-wide exclusive sum; returns this thread's prefix and the total.
template <int NT>
__device__ int scan_sum(int v, int* tmp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) tmp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < NT / 32 ? tmp[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    tmp[lane] = w;
  }
  __syncthreads();
  int r = x - v + (wid ? tmp[wid - 1] : 0);
  *total = tmp[NT / 32 - 1];
  __syncthreads();
  return r;
}

// CNT: the batch carries a multiplicity per key (p.counts), as produced by
// the duplicate-merging pass of bulk_insert_reduce.
// Rebuilds region R of the launch (all threads of the CTA) in a window of
// SPAN slots (a multiple of the thread count, at most the full window);
// returns false, having written nothing, when the changes would reach past
// the window.
template <int LOGS, bool DEL, bool CNT, int SPAN, class Loc>
__device__ __forceinline__ bool rebuild_window(const Loc& loc, const Partition& p, const uint32_t R) {
  using L = Lay<LOGS, CNT, SPAN>;
  constexpr int NT = L::NT, WB = L::WB, REG = L::REG, KMAX = L::KMAX, span = SPAN;
  constexpr int qpt = SPAN / NT;  // slots and quotients per thread
  extern __shared__ __align__(128) uint8_t sm[];
  __shared__ int s_i[8];
  __shared__ int sa[32], sb[32];

  const uint32_t kbeg = p.region_start[R], kend = kbeg + p.region_count[R];
  if (kbeg == kend) return true;
  Geom g;
  uint32_t r;  // the region within its filter
  const quotient_filter* dq;
  if (!loc.locate(R, LOGS, &g, &r, &dq)) return true;
  const int tid = threadIdx.x;

  const uint64_t base = (uint64_t)r << LOGS;
  const uint64_t bw0 = base >> 6;
  const int wb = (int)min((uint64_t)(span / 64), g.nblocks - bw0);
  const int wslots = wb * 64;
  const int win_valid = (int)min((uint64_t)wslots, g.xnslots - base);
  const int win_q = (int)min((uint64_t)span, g.nslots - base);
  const int wq_words = (win_q + 63) >> 6;
  const int nq = (int)min((uint64_t)REG, g.nslots - base);

  uint32_t* kg = reinterpret_cast<uint32_t*>(sm + L::OFF_KG);
  uint32_t* kc = reinterpret_cast<uint32_t*>(sm + L::OFF_KC);
  uint16_t* pref = reinterpret_cast<uint16_t*>(sm + L::OFF_PREF);
  int16_t* delta = reinterpret_cast<int16_t*>(sm + L::OFF_DELTA);
  unsigned long long* nocc = reinterpret_cast<unsigned long long*>(sm + L::OFF_NOCC);
  unsigned long long* tch = reinterpret_cast<unsigned long long*>(sm + L::OFF_TCH);
  uint16_t* orank = reinterpret_cast<uint16_t*>(sm + L::OFF_ORANK);
  uint16_t* rrank = reinterpret_cast<uint16_t*>(sm + L::OFF_RRANK);
  uint16_t* rpos = reinterpret_cast<uint16_t*>(sm + L::OFF_RPOS);
  uint32_t* kn = CNT ? reinterpret_cast<uint32_t*>(sm + L::OFF_KN) : nullptr;

  // ---- stage the window (wb blocks of 96 bytes) into image 0
  {
    const uint4* src = reinterpret_cast<const uint4*>(g.blocks + bw0);
    const Img D = img_at<WB>(sm + L::OFF_IMG0);
    for (int i = tid; i < wb * 6; i += NT) D.part(i) = src[i];
  }
  __syncthreads();
  const int c0 = (int)img_at<WB>(sm + L::OFF_IMG0).off(0) - 1;  // last slot used by earlier regions' runs
  // The previous region's runs fill the whole window: every run of this
  // region lies beyond it, so only the serial path can place them.  (This
  // also keeps all window positions far below the 16-bit tables' range.)
  bool deferred = c0 + 1 >= win_valid;
  const bool multi = kend - kbeg > (uint32_t)KMAX;
  int cur = 0;
  bool changed = false;

  // runends of word w that lie after c0
  auto runs_after_c0 = [&](Img C, int w) -> unsigned long long {
    unsigned long long rw = C.run(w);
    int lo = 64 * w;
    if (c0 >= lo + 63) return 0ULL;
    if (c0 >= lo) rw &= ~0ULL << (c0 - lo + 1);
    return rw;
  };
  // A thread's bits of a bitmap, [from, from + n) (0 < n <= 64, inside the
  // window), in one register shifted by one per step of its loops.
  using Bits = typename std::conditional<(qpt <= 32), uint32_t, unsigned long long>::type;
  auto window_bits = [&](auto word, int from, int n) -> Bits {
    const int w = from >> 6, sh = from & 63;
    unsigned long long v = word(w) >> sh;
    if (sh && sh + n > 64) v |= word(w + 1) << (64 - sh);
    return (Bits)(n >= 64 ? v : v & ((1ULL << n) - 1ULL));
  };

  for (uint32_t kr = kbeg; kr < kend && !deferred; kr += KMAX) {
    const int nk = (int)min((uint32_t)KMAX, kend - kr);
    const Img C = img_at<WB>(sm + (cur ? L::OFF_IMG1 : L::OFF_IMG0));
    const Img N = img_at<WB>(sm + (cur ? L::OFF_IMG0 : L::OFF_IMG1));

    // ---- group this round's keys by quotient (counting sort in shared memory)
    for (int i = tid; i < L::KCW; i += NT) kc[i] = 0;
    for (int i = tid; i < WB; i += NT) { nocc[i] = 0; tch[i] = 0; }
    __syncthreads();
    for (int i = tid; i < nk; i += NT) {
      uint32_t q = p.keys[kr + i] >> 8;
      atomicAdd(&kc[q >> 1], 1u << ((q & 1) * 16));
    }
    __syncthreads();
    {  // exclusive prefix over the REG counters, 2 per word
      constexpr int WPT = (REG / 2) / NT;
      int a = tid * WPT, sum = 0;
      for (int w = a; w < a + WPT; w++) sum += (int)(kc[w] & 0xFFFFu) + (int)(kc[w] >> 16);
      int tot;
      int run = scan_sum<NT>(sum, sa, &tot);
      for (int w = a; w < a + WPT; w++) {
        uint32_t v = kc[w];
        uint32_t lo = (uint32_t)run;
        run += (int)(v & 0xFFFFu);
        uint32_t hi = (uint32_t)run;
        run += (int)(v >> 16);
        kc[w] = lo | (hi << 16);
      }
    }
    __syncthreads();
    for (int i = tid; i < nk; i += NT) {
      uint32_t key = p.keys[kr + i];
      uint32_t q = key >> 8;
      uint32_t sh = (q & 1) * 16;
      uint32_t old = atomicAdd(&kc[q >> 1], 1u << sh);
      kg[(old >> sh) & 0xFFFFu] = key;
      if (CNT) kn[(old >> sh) & 0xFFFFu] = p.counts[kr + i];
    }
    // now the keys of each quotient are contiguous in kg, in quotient order

    // ---- rank tables of the current image: per window word, the occupied
    // quotients and the runends after c0 before it (one packed block scan)
    {
      int packed = 0;
      if (tid < WB) {
        const int co = tid < wq_words ? __popcll(C.occ(tid)) : 0;
        const int cr = tid < wb ? __popcll(runs_after_c0(C, tid)) : 0;
        packed = co | (cr << 16);
      }
      int tot;
      const int ex = scan_sum<NT>(packed, sa, &tot);
      if (tid < WB) {
        orank[tid] = (uint16_t)(ex & 0xFFFF);
        rrank[tid] = (uint16_t)(ex >> 16);
      }
      if (tid == 0) { s_i[0] = tot >> 16; s_i[1] = tot & 0xFFFF; }  // visible runends, occupied quotients
    }
    __syncthreads();
    const int nvis = s_i[0], nold = s_i[1];
    // Each thread owns qpt consecutive slots / quotients from here on, so
    // ranks, run ends and shifts carry from one to the next in registers.
    const int ca = tid * qpt;
    {  // rpos[k] = the k-th runend after c0, for this thread's slots
      const int cb = min(ca + qpt, wslots);
      int x = ca;
      while (x < cb) {
        const int w = x >> 6;
        const int xe = min(cb, 64 * w + 64);
        unsigned long long m = runs_after_c0(C, w);
        int k = rrank[w] + __popcll(m & ((1ULL << (x & 63)) - 1ULL));
        m &= ~0ULL << (x & 63);
        if (xe < 64 * w + 64) m &= (1ULL << (xe & 63)) - 1ULL;
        while (m) {
          rpos[k++] = (uint16_t)(64 * w + __ffsll((long long)m) - 1);
          m &= m - 1;
        }
        x = xe;
      }
    }
    __syncthreads();

    // Runs ending beyond the window get positions past it, in order.
    const int fake0 = win_valid + 16;
    auto runpos = [&](int k) -> int { return k < nvis ? (int)rpos[k] : fake0 + (k - nvis); };
    // the end of a quotient's key group in kg
    auto group_end = [&](int ks, uint32_t q) -> int {
      int ke = ks + 1;
      while (ke < nk && (kg[ke] >> 8) == q) ke++;
      return ke;
    };
    auto rank_of = [&](int q) -> int {
      return (int)orank[q >> 6] + __popcll(C.occ(q >> 6) & ((1ULL << (q & 63)) - 1ULL));
    };

    // ---- merge tasks: new length of every touched quotient (first key of
    // each group), before the positions are scanned
    bool my_defer = false;
    for (int i = tid; i < nk; i += NT) {
      const uint32_t q = kg[i] >> 8;
      if (i > 0 && (kg[i - 1] >> 8) == q) continue;
      const int ks = i, ke = group_end(i, q);
      set_bit(tch, (int)q);
      const bool occ = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
      int s = 0, e = -1;
      if (occ) {
        const int k = rank_of((int)q);
        e = runpos(k);
        s = max((int)q, (k ? runpos(k - 1) : c0) + 1);
      }
      if (occ && e >= win_valid) {
        my_defer = true;
        continue;
      }
      for (int a = ks + 1; a < ke; a++) {  // the quotient's keys by remainder
        const uint32_t v = kg[a];
        const uint32_t vc = CNT ? kn[a] : 0u;
        int b = a;
        while (b > ks && kg[b - 1] > v) {
          kg[b] = kg[b - 1];
          if (CNT) kn[b] = kn[b - 1];
          b--;
        }
        kg[b] = v;
        if (CNT) kn[b] = vc;
      }
      pref[q] = (uint16_t)merge_run<DEL, false>(C, occ, s, e, kg, kn, ks, ke, N, 0);
    }
    if (__syncthreads_or(my_defer)) { deferred = true; break; }

    // ---- this thread's quotients: old runs, new lengths, composed max-plus map
    const int qb_ = min(ca + qpt, win_q);
    const int k0 = ca < win_q ? rank_of(ca) : nold;
    const int e_old = nold ? runpos(nold - 1) : c0;  // end of the window's old runs
    int fa = kNeg, fb = 0;
    {
      int k = k0;
      int pe = k ? runpos(k - 1) : c0;
      // From here the table turns from run ends into run starts, each thread
      // over its own runs [k0, k1): the run ends other threads read (k0 - 1
      // above, e_old) are read before any is overwritten.
      __syncthreads();
      Bits ob = 0, tb = 0;  // occupied and touched quotients from ca on
      if (ca < qb_) {
        ob = window_bits([&](int w) { return C.occ(w); }, ca, qb_ - ca);
        tb = window_bits([&](int w) { return tch[w]; }, ca, qb_ - ca);
      }
      #pragma unroll 1  // rolled: fewer registers, five CTAs per SM
      for (int q = ca; q < qb_; q++) {
        const bool oq = ob & 1u, tq = tb & 1u;
        ob >>= 1;
        tb >>= 1;
        int len = 0;
        if (oq) {
          const int e = runpos(k);
          const int s = max(q, pe + 1);
          len = e - s + 1;
          delta[k] = (int16_t)s;
          pe = e;
          k++;
        }
        if (tq) len = pref[q];
        pref[q] = (uint16_t)len;
        if (len > 0) { fa = max(q + len - 1, fa + len); fb += len; }
      }
    }

    // ---- run positions: one block-wide max-plus scan over the quotients
    scan_maps<NT>(fa, fb, sa, sb);
    // ---- clear the next image; keep the previous region's spill
    for (int i = tid; i < wb * 6; i += NT) N.part(i) = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int sl = tid; sl <= c0 && sl < wslots; sl += NT) N.slot(sl) = C.slot(sl);
    for (int w = tid; w < wb && 64 * w <= c0; w += NT) {
      int nb = c0 - 64 * w;  // bits 0..nb belong to the previous region's runs
      N.run(w) = nb >= 63 ? C.run(w) : (C.run(w) & ((2ULL << nb) - 1ULL));
    }
    __syncthreads();
    // ---- apply: new ends, runend bits, occupancy, shift of every old run
    {
      int x = max(fa, c0 + fb);  // end of all runs before this thread's first quotient
      int k = k0;
      unsigned long long occ_bits = 0;
      int occ_word = ca >> 6, cw = -1;
      unsigned long long ebits = 0;  // new runend bits of window word ew
      int ew = -1;
      int nlen = ca < qb_ ? pref[ca] : 0;  // the next quotient's length, loaded a step ahead
      int nd = delta[k];                   // the next run's old start, loaded ahead
      Bits ob = 0, tb = 0;  // occupied and touched quotients from ca on
      if (ca < qb_) {
        ob = window_bits([&](int w) { return C.occ(w); }, ca, qb_ - ca);
        tb = window_bits([&](int w) { return tch[w]; }, ca, qb_ - ca);
      }
      #pragma unroll 1  // rolled: fewer registers, five CTAs per SM
      for (int q = ca; q < qb_; q++) {
        if ((q >> 6) != cw) {
          if (cw >= 0 && occ_bits) or64(&nocc[occ_word], occ_bits);
          occ_bits = 0;
          cw = occ_word = q >> 6;
        }
        const bool oq = ob & 1u, tq = tb & 1u;
        ob >>= 1;
        tb >>= 1;
        const int len = nlen;
        if (q + 1 < qb_) nlen = pref[q + 1];
        const int ns = max(q, x + 1);
        if (len > 0) {
          x = ns + len - 1;
          occ_bits |= 1ULL << (q & 63);
          if (x < wslots) {
            if ((x >> 6) != ew) {
              if (ebits) or64(&N.run(ew), ebits);
              ew = x >> 6;
              ebits = 0;
            }
            ebits |= 1ULL << (x & 63);
          }
        }
        if (oq) {
          delta[k] = (int16_t)(tq ? kTouched + nd : ns - nd);
          k++;
          nd = delta[k];
        }
        pref[q] = (uint16_t)(x + 1);
      }
      if (occ_bits) or64(&nocc[occ_word], occ_bits);
      if (ebits) or64(&N.run(ew), ebits);
    }
    __syncthreads();
    {
      const int e_new = (int)pref[win_q - 1] - 1;
      // A change that reaches the window's end would move runs this CTA does
      // not hold (or overflow the table): leave the region to the serial pass.
      if (e_new != e_old && max(e_new, e_old) >= win_valid) { deferred = true; break; }
    }
    // ---- merge tasks again, now writing the touched runs at their new start
    for (int i = tid; i < nk; i += NT) {
      const uint32_t q = kg[i] >> 8;
      if (i > 0 && (kg[i - 1] >> 8) == q) continue;
      if (!((nocc[q >> 6] >> (q & 63)) & 1ULL)) continue;  // deleted entirely
      const int ks = i, ke = group_end(i, q);
      const bool occ = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
      int s = 0, e = -1;
      if (occ) {  // the old run: its start kept by the apply, its end the next runend
        s = (int)delta[rank_of((int)q)] - kTouched;
        int w = s >> 6;
        unsigned long long m = C.run(w) & (~0ULL << (s & 63));
        while (!m) m = C.run(++w);  // ends below win_valid: the first merge deferred the rest
        e = 64 * w + __ffsll((long long)m) - 1;
      }
      const int ns = max((int)q, (q ? (int)pref[q - 1] - 1 : c0) + 1);
      merge_run<DEL, true>(C, occ, s, e, kg, kn, ks, ke, N, ns);
    }
    // ---- slot pass: this thread's slots move by their run's shift.  A slot
    // after c0 holds part of a run of this window exactly when more of the
    // window's occupied quotients lie at or before it than runs end before it
    // (runs never pass a gap), so `o - k` tracks it from the rank tables.
    {
      const int cb = min(ca + qpt, wslots);
      if (ca < cb) {
        const int w = ca >> 6;
        int k = rrank[w] + __popcll(runs_after_c0(C, w) & ((1ULL << (ca & 63)) - 1ULL));
        int o = ca < win_q ? rank_of(ca) : nold;  // occupied window quotients below sl
        Bits mb = window_bits([&](int ww) { return runs_after_c0(C, ww); }, ca, cb - ca);
        Bits ob = window_bits([&](int ww) { return ww < wq_words ? C.occ(ww) : 0ULL; }, ca, cb - ca);
        #pragma unroll 1  // rolled: fewer registers, five CTAs per SM
        for (int sl = ca; sl < cb; sl++) {
          o += (int)(ob & 1u);
          ob >>= 1;
          if (sl > c0 && o > k) {
            const int d = delta[k];
            if (d < kTouched) {
              const int t = sl + d;
              if (t >= 0 && t < wslots) N.slot(t) = C.slot(sl);
            }
          }
          k += (int)(mb & 1u);
          mb >>= 1;
        }
      }
    }
    __syncthreads();
    // ---- block headers: occupieds and offsets
    for (int w = tid; w < wb; w += NT) {
      N.occ(w) = w < wq_words ? nocc[w] : 0ULL;
      if (w == 0) {
        N.off(0) = C.off(0);
      } else {
        const int x = min(64 * w - 1, win_q - 1);
        const int E = (int)pref[x] - 1;
        N.off(w) = E >= win_valid ? C.off(w) : (uint32_t)max(0, E - 64 * w + 1);
      }
    }
    __syncthreads();
    cur ^= 1;
    changed = true;
  }

  if (deferred) return false;
  if (!changed) return true;
  // ---- write back the blocks that differ from what was loaded
  {
    const Img fin = img_at<WB>(sm + (cur ? L::OFF_IMG1 : L::OFF_IMG0));
    const Img org = img_at<WB>(sm + L::OFF_IMG0);
    uint4* dst = reinterpret_cast<uint4*>(g.blocks + bw0);
    for (int w = tid; w < wb; w += NT) {
      bool diff = multi;  // after several rounds the loaded image is gone
      if (!diff)
        for (int c = 0; c < 6; c++) {
          const uint4 a = fin.part(w * 6 + c), b = org.part(w * 6 + c);
          diff |= (a.x != b.x) | (a.y != b.y) | (a.z != b.z) | (a.w != b.w);
        }
      if (diff)
        for (int c = 0; c < 6; c++) dst[w * 6 + c] = fin.part(w * 6 + c);
    }
  }
  return true;
}

// The last word w of [0, nw) whose exclusive rank rank[w] is <= k: the word
// holding the k-th set bit, when k is below the total.
__device__ __forceinline__ int rank_word(const uint16_t* rank, int nw, int k) {
  int lo = 0, hi = nw;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((int)rank[mid] <= k) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Single-round insert into region R (all threads of the CTA) in a window of
// SPAN slots, by shifting slots instead of re-placing every run.
//
// The batch changes only the runs of its quotients (the touched runs: their
// counters merged with the keys, merge_run) and adds runs for quotients that
// had none.  Everything else keeps its bytes and moves right by a shift D(x)
// that a recurrence over the old slots gives, one map per slot:
//   D <- max(0, D + ins(x) - empty(x))
// (growth ins(x) enters before slot x; an empty slot absorbs one slot of
// push).  Each map has the form max(a, D + b), so one block-wide max-plus
// scan gives every thread the shift at its first slot.  This is the
// canonical layout's rule end(q) = max(q + L_q - 1, end(prev) + L_q) written
// per slot: a touched run of old length l and new length L adds L - l before
// the slot X after its end, a new run of quotient q adds L before slot
// X = max(q, end of the runs before it + 1), and a run's new bytes go where
// its old first slot moves.
//
// Threads own SPAN / 256 consecutive slots; the per-quotient work is per
// touched run only (about one per thread), which finds its run from its
// block's exact offset.  Returns false, having written nothing, when the
// changes would reach past the window.  Deletes, and regions of more than
// KMAX keys, go to rebuild_window.
template <int LOGS, bool CNT, int SPAN, class Loc>
__device__ __forceinline__ bool shift_window(const Loc& loc, const Partition& p, const uint32_t R, BulkStage& sg) {
  using L = Lay<LOGS, CNT, SPAN>;
  constexpr int NT = L::NT, WB = L::WB, REG = L::REG, KMAX = L::KMAX;
  constexpr int qpt = SPAN / NT;  // slots per thread
  constexpr int kFar = 1 << 20;   // a position past every window
  static_assert(SPAN % NT == 0 && SPAN <= L::WIN, "slots split evenly over threads");
  static_assert(4 * KMAX <= L::DELTA_BYTES, "per-key tables fit the shared table");
  extern __shared__ __align__(128) uint8_t sm[];
  __shared__ int s_i[8];
  __shared__ int sa[32], sb[32];

  const uint32_t kbeg = p.region_start[R];
  const int nk = (int)p.region_count[R];
  if (nk == 0) return true;
  Geom g;
  uint32_t r;
  const quotient_filter* dq;
  if (!loc.locate(R, LOGS, &g, &r, &dq)) return true;
  const int tid = threadIdx.x;

  const uint64_t base = (uint64_t)r << LOGS;
  const uint64_t bw0 = base >> 6;
  const int wb = (int)min((uint64_t)(SPAN / 64), g.nblocks - bw0);
  const int wslots = wb * 64;
  const int win_valid = (int)min((uint64_t)wslots, g.xnslots - base);
  const int win_q = (int)min((uint64_t)SPAN, g.nslots - base);
  const int wq_words = (win_q + 63) >> 6;

  const Img C = img_at<WB>(sm + L::OFF_IMG0);
  const Img N = img_at<WB>(sm + L::OFF_IMG1);
  uint32_t* kg = reinterpret_cast<uint32_t*>(sm + L::OFF_KG);
  uint32_t* kc = reinterpret_cast<uint32_t*>(sm + L::OFF_KC);
  // growth entering before each slot, then the shift just before it
  int16_t* ins = reinterpret_cast<int16_t*>(sm + L::OFF_PREF);
  uint32_t* ins32 = reinterpret_cast<uint32_t*>(sm + L::OFF_PREF);
  // after the grouping: each key's event slot X (its group's) and each
  // group's old run length
  uint16_t* gx = reinterpret_cast<uint16_t*>(sm + L::OFF_DELTA);
  uint16_t* gl = reinterpret_cast<uint16_t*>(sm + L::OFF_DELTA + 2 * KMAX);
  unsigned long long* nocc = reinterpret_cast<unsigned long long*>(sm + L::OFF_NOCC);
  unsigned long long* trm = reinterpret_cast<unsigned long long*>(sm + L::OFF_TCH);  // touched runs' slots
  uint16_t* orank = reinterpret_cast<uint16_t*>(sm + L::OFF_ORANK);
  uint16_t* rrank = reinterpret_cast<uint16_t*>(sm + L::OFF_RRANK);
  uint32_t* kn = CNT ? reinterpret_cast<uint32_t*>(sm + L::OFF_KN) : nullptr;

  // ---- stage the window (wb blocks of 96 bytes) with one bulk copy into
  // image N's memory, clearing the tables meanwhile, then split it into
  // image C (N is cleared before its first use)
  const uint4* raw = reinterpret_cast<const uint4*>(sm + L::OFF_IMG1);
  if (tid == 0) bulk_stage_start(sg, sm + L::OFF_IMG1, g.blocks + bw0, (uint32_t)wb * 96u);
  for (int i = tid; i < L::KCW; i += NT) kc[i] = 0;
  for (int i = tid; i < (wslots >> 1); i += NT) ins32[i] = 0;
  const bool staged = bulk_stage_wait(sg);
  __syncthreads();
  if (!staged) return false;
  for (int i = tid; i < wb * 6; i += NT) C.part(i) = raw[i];
  __syncthreads();
  const int c0 = (int)C.off(0) - 1;  // last slot used by earlier regions' runs
  if (c0 + 1 >= win_valid) return false;  // every run of this region lies past the window

  auto runs_after_c0 = [&](int w) -> unsigned long long {
    unsigned long long rw = C.run(w);
    const int lo = 64 * w;
    if (c0 >= lo + 63) return 0ULL;
    if (c0 >= lo) rw &= ~0ULL << (c0 - lo + 1);
    return rw;
  };

  // ---- group the keys by quotient (counting sort in shared memory)
  for (int i = tid; i < nk; i += NT) {
    const uint32_t q = p.keys[kbeg + i] >> 8;
    atomicAdd(&kc[q >> 1], 1u << ((q & 1) * 16));
  }
  __syncthreads();
  {
    constexpr int WPT = (REG / 2) / NT;
    const int a = tid * WPT;
    int sum = 0;
    for (int w = a; w < a + WPT; w++) sum += (int)(kc[w] & 0xFFFFu) + (int)(kc[w] >> 16);
    int tot;
    int run = scan_sum<NT>(sum, sa, &tot);
    for (int w = a; w < a + WPT; w++) {
      const uint32_t v = kc[w];
      const uint32_t lo = (uint32_t)run;
      run += (int)(v & 0xFFFFu);
      const uint32_t hi = (uint32_t)run;
      run += (int)(v >> 16);
      kc[w] = lo | (hi << 16);
    }
  }
  __syncthreads();
  for (int i = tid; i < nk; i += NT) {
    const uint32_t key = p.keys[kbeg + i];
    const uint32_t q = key >> 8;
    const uint32_t sh = (q & 1) * 16;
    const uint32_t old = atomicAdd(&kc[q >> 1], 1u << sh);
    kg[(old >> sh) & 0xFFFFu] = key;
    if (CNT) kn[(old >> sh) & 0xFFFFu] = p.counts[kbeg + i];
  }
  // ---- rank tables of the old image: per window word, the occupied
  // quotients and the runends after c0 before it
  {
    int packed = 0;
    if (tid < WB) {
      const int co = tid < wq_words ? __popcll(C.occ(tid)) : 0;
      const int cr = tid < wb ? __popcll(runs_after_c0(tid)) : 0;
      packed = co | (cr << 16);
    }
    int tot;
    const int ex = scan_sum<NT>(packed, sa, &tot);  // synchronises: the grouping is done
    if (tid < WB) {
      orank[tid] = (uint16_t)(ex & 0xFFFF);
      rrank[tid] = (uint16_t)(ex >> 16);
      nocc[tid] = tid < wq_words ? C.occ(tid) : 0ULL;
      trm[tid] = 0ULL;
    }
    if (tid == 0) s_i[1] = tot & 0xFFFF;
  }
  __syncthreads();
  const int nold = s_i[1];  // occupied quotients of the window
  auto rank_of = [&](int q) -> int {
    return (int)orank[q >> 6] + __popcll(C.occ(q >> 6) & ((1ULL << (q & 63)) - 1ULL));
  };
  // the n-th (0-based) runend at or after slot `from` (> c0), or kFar
  auto nth_end = [&](int from, int n) -> int {
    int w = from >> 6;
    if (w >= wb) return kFar;
    unsigned long long m = C.run(w) & (~0ULL << (from & 63));
    int c = __popcll(m);
    while (n >= c) {
      n -= c;
      if (++w >= wb) return kFar;
      m = C.run(w);
      c = __popcll(m);
    }
    return 64 * w + select64(m, n);
  };
  auto group_end = [&](int ks, uint32_t q) -> int {
    int ke = ks + 1;
    while (ke < nk && (kg[ke] >> 8) == q) ke++;
    return ke;
  };

  // ---- pass 1 over the touched quotients: the run each key group changes,
  // its new length, and the growth it adds before slot X
  bool my_defer = false;
  for (int i = tid; i < nk; i += NT) {
    const uint32_t q = kg[i] >> 8;
    if (i > 0 && (kg[i - 1] >> 8) == q) continue;
    const int ke = group_end(i, q);
    for (int a = i + 1; a < ke; a++) {  // the quotient's keys by remainder
      const uint32_t v = kg[a];
      const uint32_t vc = CNT ? kn[a] : 0u;
      int b = a;
      while (b > i && kg[b - 1] > v) {
        kg[b] = kg[b - 1];
        if (CNT) kn[b] = kn[b - 1];
        b--;
      }
      kg[b] = v;
      if (CNT) kn[b] = vc;
    }
    // the runs of block qb's quotients end at the runends from its offset on
    const int qb = (int)(q >> 6);
    const unsigned long long ow = C.occ(qb);
    const bool occ = (ow >> (q & 63)) & 1ULL;
    const int rib = __popcll(ow & ((1ULL << (q & 63)) - 1ULL));
    const int p0 = 64 * qb + (int)C.off(qb);
    const int prev_end = rib ? nth_end(p0, rib - 1) : p0 - 1;
    int s, e, X;
    if (occ) {
      e = prev_end >= kFar ? kFar : nth_end(prev_end + 1, 0);
      s = max((int)q, prev_end + 1);
      X = e + 1;
    } else {
      X = max((int)q, prev_end + 1);
      s = X;
      e = X - 1;
    }
    if (X >= win_valid) { my_defer = true; continue; }
    const int len = merge_run<false, false>(C, occ, s, e, kg, kn, i, ke, N, 0);
    const int delta = len - (e - s + 1);
    if (delta < 0) { my_defer = true; continue; }  // counters never shrink on insert
    if (delta) atomicAdd(&ins32[X >> 1], (uint32_t)delta << ((X & 1) * 16));
    for (int a = i; a < ke; a++) gx[a] = (uint16_t)X;
    gl[i] = (uint16_t)(e - s + 1);
    if (occ) {
      for (int w = s >> 6; w <= (e >> 6); w++) {
        const int lo = max(s, 64 * w) - 64 * w, hi = min(e, 64 * w + 63) - 64 * w;
        or64(&trm[w], (~0ULL >> (63 - hi)) & (~0ULL << lo));
      }
    } else {
      set_bit(nocc, (int)q);
    }
  }
  if (__syncthreads_or(my_defer)) return false;

  // ---- the shift recurrence over this thread's slots [lo, hi): those after
  // c0 and inside the window (the others neither move nor shift).  The map
  // of slot x is max(a, D + b).
  const int ca = tid * qpt;
  const int lo = max(ca, c0 + 1), hi = min(ca + qpt, win_valid);
  // The thread's occupied, runend (after c0) and touched-run bits, from lo
  // on, in one register each, shifted by one slot per step.
  using Bits = typename std::conditional<(qpt <= 32), uint32_t, unsigned long long>::type;
  struct Walk {
    int o, k;
    Bits ob, mb, tb;
    bool prev_end, prev_tr;
  };
  // bits [from, from + n) of a bitmap given word by word (n <= 64, within the window)
  auto window_bits = [&](auto word, int from, int n) -> Bits {
    const int w = from >> 6, sh = from & 63;
    unsigned long long v = word(w) >> sh;
    if (sh && sh + n > 64) v |= word(w + 1) << (64 - sh);
    return (Bits)(n >= 64 ? v : v & ((1ULL << n) - 1ULL));
  };
  auto walk_init = [&](Walk& W) {
    const int n = hi - lo;
    W.ob = window_bits([&](int w) { return w < wq_words ? C.occ(w) : 0ULL; }, lo, n);
    W.mb = window_bits([&](int w) { return runs_after_c0(w); }, lo, n);
    W.tb = window_bits([&](int w) { return trm[w]; }, lo, n);
    W.k = (int)rrank[lo >> 6] + __popcll(runs_after_c0(lo >> 6) & ((1ULL << (lo & 63)) - 1ULL));
    W.o = lo < win_q ? rank_of(lo) : nold;  // occupied window quotients below lo
    if (lo == c0 + 1) {
      W.prev_end = false;
      W.prev_tr = false;
    } else {
      const int y = lo - 1;
      W.prev_end = (runs_after_c0(y >> 6) >> (y & 63)) & 1ULL;
      W.prev_tr = (trm[y >> 6] >> (y & 63)) & 1ULL;
    }
  };
  // Advances W over slot x (c0 < x < win_valid): whether it holds a run's
  // slot, ends a run, belongs to a touched run, or receives growth (b: its
  // map max(0, D + b)), and whether a touched run's writer needs the shift
  // before it.
  auto step = [&](Walk& W, int x, int& b, bool& used, bool& is_end, bool& tr, bool& evt) {
    W.o += (int)(W.ob & 1u);
    is_end = W.mb & 1u;
    tr = W.tb & 1u;
    W.ob >>= 1;
    W.mb >>= 1;
    W.tb >>= 1;
    const int gv = (int)ins[x];
    evt = gv != 0 || (W.prev_tr && W.prev_end);
    used = W.o > W.k;
    b = gv - (used ? 0 : 1);
    W.k += (int)is_end;
    W.prev_end = is_end;
    W.prev_tr = tr;
  };
  int fa = 0, fb = 0;  // composed map of this thread's slots (b >= -1: nothing saturates)
  if (lo < hi) {
    Walk W;
    walk_init(W);
    for (int x = lo; x < hi; x++) {
      int b;
      bool used, is_end, tr, evt;
      step(W, x, b, used, is_end, tr, evt);
      fa = max(0, fa + b);
      fb += b;
    }
  }
  int ea = fa, eb = fb;
  scan_maps<NT>(ea, eb, sa, sb);
  const int d_in = max(ea, eb);  // the shift entering this thread's slots (D = 0 before the window)
  if (tid == NT - 1) s_i[2] = max(fa, sat(d_in + fb));  // the shift after the window's last slot
  // ---- clear the new image; keep the previous region's spill
  for (int i = tid; i < wb * 6; i += NT) N.part(i) = make_uint4(0, 0, 0, 0);
  __syncthreads();
  if (s_i[2] != 0) return false;  // the changes reach past the window
  for (int sl = tid; sl <= c0 && sl < wslots; sl += NT) N.slot(sl) = C.slot(sl);
  for (int w = tid; w < wb && 64 * w <= c0; w += NT) {
    const int nb = c0 - 64 * w;  // bits 0..nb belong to the previous region's runs
    N.run(w) = nb >= 63 ? C.run(w) : (C.run(w) & ((2ULL << nb) - 1ULL));
  }
  __syncthreads();
  // ---- pass 2 over the slots: untouched slots move by their shift; the
  // shift before each event slot is kept for the touched runs' writers
  if (lo < hi) {
    Walk W;
    walk_init(W);
    int D = d_in;
    unsigned long long ebits = 0;
    int ew = -1;
    for (int x = lo; x < hi; x++) {
      int b;
      bool used, is_end, tr, evt;
      step(W, x, b, used, is_end, tr, evt);
      const int dp = D;
      D = max(0, D + b);
      if (evt) ins[x] = (int16_t)dp;
      if (used && !tr) {
        const int t = x + D;
        N.slot(t) = C.slot(x);
        if (is_end) {
          if ((t >> 6) != ew) {
            if (ebits) or64(&N.run(ew), ebits);
            ew = t >> 6;
            ebits = 0;
          }
          ebits |= 1ULL << (t & 63);
        }
      }
    }
    if (ebits) or64(&N.run(ew), ebits);
  }
  __syncthreads();
  // ---- pass 2 over the touched quotients: each run's new bytes where its
  // old first slot moved.  Runs whose growth enters before the same slot X
  // (a touched run and the new runs right after it) are written in quotient
  // order by the first of them.
  for (int i = tid; i < nk; i += NT) {
    const uint32_t q = kg[i] >> 8;
    if (i > 0 && (kg[i - 1] >> 8) == q) continue;
    const bool occ = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
    const int X = (int)gx[i];
    if (i > 0 && (int)gx[i - 1] == X) continue;  // written by the first run of its slot
    const int ell = (int)gl[i];
    int ke = group_end(i, q);
    int pos = X - ell + (int)ins[X];
    int len = merge_run<false, true>(C, occ, X - ell, X - 1, kg, kn, i, ke, N, pos);
    if (len > 0) or64(&N.run((pos + len - 1) >> 6), 1ULL << ((pos + len - 1) & 63));
    pos += len;
    while (ke < nk && (int)gx[ke] == X) {  // new runs entering before the same slot
      const int ks = ke;
      ke = group_end(ks, kg[ks] >> 8);
      len = merge_run<false, true>(C, false, 0, -1, kg, kn, ks, ke, N, pos);
      if (len > 0) or64(&N.run((pos + len - 1) >> 6), 1ULL << ((pos + len - 1) & 63));
      pos += len;
    }
  }
  __syncthreads();
  // ---- block headers: occupieds, then offsets from the new run ends
  {
    int packed = 0;
    if (tid < WB) {
      const unsigned long long nw = tid < wq_words ? nocc[tid] : 0ULL;
      unsigned long long rw = 0ULL;
      if (tid < wb) {
        N.occ(tid) = nw;
        rw = N.run(tid);
        const int l0 = 64 * tid;
        if (c0 >= l0 + 63) rw = 0ULL;
        else if (c0 >= l0) rw &= ~0ULL << (c0 - l0 + 1);
      }
      packed = __popcll(nw) | (__popcll(rw) << 16);
    }
    int tot;
    const int ex = scan_sum<NT>(packed, sa, &tot);
    if (tid < WB) {
      orank[tid] = (uint16_t)(ex & 0xFFFF);  // now: new occupied quotients before word tid
      rrank[tid] = (uint16_t)(ex >> 16);     // new runends after c0 before word tid
    }
    if (tid == 0) s_i[3] = tot >> 16;
  }
  __syncthreads();
  {
    const int nvis_new = s_i[3];
    for (int w = tid; w < wb; w += NT) {
      if (w == 0) {
        N.off(0) = C.off(0);
        continue;
      }
      const int kq = (int)orank[w];  // new runs of quotients before block w
      int E;
      if (kq == 0) {
        E = c0;
      } else if (kq - 1 < nvis_new) {
        const int ww = rank_word(rrank, wb, kq - 1);
        unsigned long long rw = N.run(ww);
        const int l0 = 64 * ww;
        if (c0 >= l0 + 63) rw = 0ULL;
        else if (c0 >= l0) rw &= ~0ULL << (c0 - l0 + 1);
        E = 64 * ww + select64(rw, kq - 1 - (int)rrank[ww]);
      } else {
        E = win_valid;  // ends past the window: unchanged
      }
      N.off(w) = E >= win_valid ? C.off(w) : (uint32_t)max(0, E - 64 * w + 1);
    }
  }
  __syncthreads();
  // ---- write back the blocks that differ from what was loaded
  {
    uint4* dst = reinterpret_cast<uint4*>(g.blocks + bw0);
    for (int w = tid; w < wb; w += NT) {
      bool diff = false;
      for (int c = 0; c < 6; c++) {
        const uint4 a = N.part(w * 6 + c), b = C.part(w * 6 + c);
        diff |= (a.x != b.x) | (a.y != b.y) | (a.z != b.z) | (a.w != b.w);
      }
      if (diff)
        for (int c = 0; c < 6; c++) dst[w * 6 + c] = N.part(w * 6 + c);
    }
  }
  return true;
}

// Where a rebuild launch finds its regions: one CTA per region of the
// parity, in region order; or a persistent grid whose CTAs take regions
// one at a time from a work list (k_sparse's, or the short pass's retries)
// until it is exhausted.
enum : int { kFromGrid = 0, kFromList = 1, kFromRetry = 2 };

// The rebuild of one phase in windows of SPAN slots.  The short pass
// (SPAN < the full window) lists for the full pass the regions it cannot
// hold, and those whose keys need several rounds (they may grow further);
// the full pass leaves what it cannot hold to the serial fallback.
template <int LOGS, bool DEL, bool CNT, int SPAN, class Loc>
__global__ void __launch_bounds__(256, (rebuild_min_blocks<LOGS, DEL, CNT, SPAN>()))
    k_rebuild(Loc loc, Partition p, int parity, int from, uint32_t* status) {
  using L = Lay<LOGS, CNT>;
  constexpr bool kShort = SPAN < L::WIN;
  __shared__ __align__(8) unsigned long long s_bar;
  BulkStage sg{&s_bar, 0u, status};
  if (!DEL) {
    if (threadIdx.x == 0) mbar_init(&s_bar);
    __syncthreads();
  }
  auto one = [&](uint32_t R) {
    // inserts of one round of keys shift the window; deletes, and keys
    // needing several rounds (full window only), re-place every run
    bool ok;
    if constexpr (!DEL) {
      if (p.region_count[R] <= (uint32_t)L::KMAX) ok = shift_window<LOGS, CNT, SPAN>(loc, p, R, sg);
      else ok = kShort ? false : rebuild_window<LOGS, DEL, CNT, SPAN>(loc, p, R);
    } else {
      ok = (kShort && p.region_count[R] > (uint32_t)L::KMAX) ? false
                                                             : rebuild_window<LOGS, DEL, CNT, SPAN>(loc, p, R);
    }
    if (ok || threadIdx.x != 0) return;
    if (kShort) {
      const uint32_t at = atomicAdd(&p.retry[kListCount], 1u);
      p.retry[kListBase + at] = R;
      if (p.stats) atomicAdd(&p.stats[2], 1ULL);
    } else {
      const uint32_t at = atomicAdd(&p.deferred[0], 1u);
      p.deferred[1 + at] = R;
      atomicOr(status, kStDeferred);
      if (p.stats) atomicAdd(&p.stats[0], 1ULL);
    }
  };
  if (from == kFromGrid) {
    const uint32_t R = 2 * blockIdx.x + parity;
    if (R < p.nregions) one(R);
    return;
  }
  uint32_t* list = from == kFromList ? p.cursor : p.retry;
  __shared__ uint32_t s_take;
  const uint32_t count = list[kListCount];  // complete: the launch that fills it has ended
  for (;;) {
    __syncthreads();  // the previous region is written back before its memory is reused
    if (threadIdx.x == 0) s_take = atomicAdd(&list[kListNext], 1u);
    __syncthreads();
    const uint32_t i = s_take;
    if (i >= count) return;
    one(list[kListBase + i]);
  }
}

// Sparse regions.  The rebuild visits every quotient and slot of its window
// whatever the number of keys, so a region holding only a few keys (a small
// batch, or a large table) is cheaper to update key by key: one thread per
// region applies the reference's single-key algorithms (gqf_device.cuh,
// src/gqf.cu:1523 insert1, :1768 insert, :1876 _remove) in place, as the
// reference's insert_from_buffers_hashed does for every region
// (src/gqf.cu:2759-2804).
//
// Before writing anything the thread proves (Serial::sparse_fits) that the
// region's changes stay inside the window a rebuild would own, [base, base +
// REG + PUSH); otherwise it lists the region, untouched, for the rebuild that
// follows in the same phase, as it lists every region with more keys.
template <int LOGS, bool DEL, bool CNT, class Loc>
__global__ void __launch_bounds__(128) k_sparse(Loc loc, Partition p, int parity, uint32_t sparse_max,
                                                uint32_t* status) {
  const uint32_t R = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + parity;
  const uint32_t cnt = R < p.nregions ? p.region_count[R] : 0;
  Geom g;
  uint32_t r = 0;
  const quotient_filter* dq = nullptr;
  const bool real = cnt && loc.locate(R, LOGS, &g, &r, &dq);
  bool listed = real && cnt > sparse_max;
  bool mine = real && !listed;
  uint64_t grow = 0;  // slots the batch may add (0 for deletes)
  if (mine && !DEL)
    for (uint32_t k = p.region_start[R]; k < p.region_start[R] + cnt; k++)
      grow += Serial::insert_growth(CNT ? p.counts[k] : 1);
  if (mine) {
    const Serial S(dq);
    const uint64_t base = (uint64_t)r << LOGS;
    // a block boundary at or below nslots (a filter smaller than a region is
    // one region)
    const uint64_t region_end = min((uint64_t)(base + (1ULL << LOGS)), (uint64_t)S.nslots);
    const uint64_t bound = min(base + (uint64_t)Lay<LOGS, false>::WIN, min(S.xnslots, 64 * S.nblocks));
    if (!S.sparse_fits(region_end, grow, bound)) {
      listed = true;
      mine = false;
    }
  }
  // append the listed regions (one atomic per warp)
  const unsigned want = __ballot_sync(0xffffffffu, listed);
  const unsigned lane = threadIdx.x & 31;
  uint32_t at = 0;
  if (lane == 0 && want) at = atomicAdd(&p.cursor[kListCount], (uint32_t)__popc(want));
  at = __shfl_sync(0xffffffffu, at, 0);
  if (listed) p.cursor[kListBase + at + __popc(want & ((1u << lane) - 1u))] = R;
  if (!mine) return;
  const Serial S(dq);
  const uint32_t kbeg = p.region_start[R];
  const int shift = 8 + LOGS;
  for (uint32_t k = kbeg; k < kbeg + cnt; k++) {
    const uint64_t h = ((uint64_t)r << shift) | p.keys[k];
    if (DEL) {
      S.remove(h, 1);
    } else {
      const uint64_t c = CNT ? p.counts[k] : 1;
      const int rc = c == 1 ? S.insert1(h) : S.insert(h, c);
      if (rc < 0) atomicOr(status, kStFull);
    }
  }
}

// Serial fallback for deferred regions: the reference's single-key
// operations, one key at a time, in region order.
template <class Loc>
__global__ void k_fallback(Loc loc, Partition p, int del, uint32_t* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t n = p.deferred[0];
  if (n == 0) return;
  // ascending region order (insertion sort; the list is short)
  uint32_t* ids = p.deferred + 1;
  for (uint32_t i = 1; i < n; i++) {
    uint32_t v = ids[i];
    uint32_t j = i;
    while (j > 0 && ids[j - 1] > v) { ids[j] = ids[j - 1]; j--; }
    ids[j] = v;
  }
  const int shift = 8 + p.log_region;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t R = ids[i];
    Geom g;
    uint32_t r;
    const quotient_filter* dq;
    if (!loc.locate(R, p.log_region, &g, &r, &dq)) continue;
    Serial S(dq);
    if (p.stats) p.stats[1] += p.region_count[R];
    for (uint32_t k = p.region_start[R]; k < p.region_start[R] + p.region_count[R]; k++) {
      uint64_t h = ((uint64_t)r << shift) | p.keys[k];
      uint64_t c = p.counts ? p.counts[k] : 1;
      if (del) {
        for (uint64_t t = 0; t < c; t++) S.remove(h, 1);
      } else {
        int rc = c == 1 ? S.insert1(h) : S.insert(h, c);
        if (rc < 0) atomicOr(status, kStFull);
      }
    }
  }
}

// The shared-memory limit is an attribute of the kernel on one device: set
// it once per instantiation and device.
template <int LOGS, bool DEL, bool CNT, int SPAN, class Loc>
void configure() {
  static std::atomic<bool> done[kMaxDevices];
  once_per_device(done, [] {
    cudaFuncSetAttribute(k_rebuild<LOGS, DEL, CNT, SPAN, Loc>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         Lay<LOGS, CNT, SPAN>::BYTES);
    cudaFuncSetAttribute(k_rebuild<LOGS, DEL, CNT, SPAN, Loc>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         100);
  });
}

// CTAs of k_rebuild resident at once on the current device.
template <int LOGS, bool DEL, bool CNT, int SPAN, class Loc>
uint32_t resident() {
  static std::atomic<uint32_t> n[kMaxDevices];  // per instantiation and device
  const int d = current_device();
  uint32_t v = n[d].load(std::memory_order_relaxed);
  if (!v) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rebuild<LOGS, DEL, CNT, SPAN, Loc>, 256,
                                                  Lay<LOGS, CNT, SPAN>::BYTES);
    v = (uint32_t)std::max(1, sm_count()) * (uint32_t)std::max(1, per);
    n[d].store(v, std::memory_order_relaxed);
  }
  return v;
}

// The two passes of one parity: the short windows over the grid or the
// listed regions, then the full windows over the short pass's retries.
template <int LOGS, bool DEL, bool CNT, class Loc>
void launch_passes(const Loc& loc, const Partition& p, int parity, int use_list, uint32_t grid, uint32_t* status,
                   cudaStream_t st) {
  using L = Lay<LOGS, CNT>;
  configure<LOGS, DEL, CNT, L::SHORT, Loc>();
  configure<LOGS, DEL, CNT, L::WIN, Loc>();
  constexpr int kShortBytes = Lay<LOGS, CNT, L::SHORT>::BYTES, kFullBytes = Lay<LOGS, CNT, L::WIN>::BYTES;
  const uint32_t g1 = use_list ? std::min(grid, resident<LOGS, DEL, CNT, L::SHORT, Loc>()) : grid;
  k_rebuild<LOGS, DEL, CNT, L::SHORT, Loc><<<g1, 256, kShortBytes, st>>>(loc, p, parity,
                                                                         use_list ? kFromList : kFromGrid, status);
  count_launch();
  const uint32_t g2 = std::min(grid, resident<LOGS, DEL, CNT, L::WIN, Loc>());
  k_rebuild<LOGS, DEL, CNT, L::WIN, Loc><<<g2, 256, kFullBytes, st>>>(loc, p, parity, kFromRetry, status);
  count_launch();
}

template <int LOGS, class Loc>
cudaError_t run_phases(const Loc& loc, const Partition& p, Op op, uint32_t sparse_max, uint32_t* status,
                       cudaStream_t st) {
  const bool cnt = p.counts != nullptr;
  if (op == Op::kDelete && cnt) return cudaErrorInvalidValue;  // deletes carry no counts
  const uint32_t half = (p.nregions + 1) / 2;
  for (int parity = 0; parity < 2; parity++) {
    uint32_t grid = parity ? p.nregions / 2 : half;
    if (!grid) continue;
    const int use_list = sparse_max != 0;
    cudaError_t e = cudaMemsetAsync(p.retry, 0, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (use_list) {
      e = cudaMemsetAsync(p.cursor, 0, 2 * sizeof(uint32_t), st);
      if (e != cudaSuccess) return e;
      const uint32_t sg = (grid + 127) / 128;
      if (op == Op::kDelete)
        k_sparse<LOGS, true, false, Loc><<<sg, 128, 0, st>>>(loc, p, parity, sparse_max, status);
      else if (cnt)
        k_sparse<LOGS, false, true, Loc><<<sg, 128, 0, st>>>(loc, p, parity, sparse_max, status);
      else
        k_sparse<LOGS, false, false, Loc><<<sg, 128, 0, st>>>(loc, p, parity, sparse_max, status);
      count_launch();
    }
    // persistent grids over lists: as many CTAs as fit at once, or as
    // regions exist
    if (op == Op::kDelete) launch_passes<LOGS, true, false>(loc, p, parity, use_list, grid, status, st);
    else if (cnt) launch_passes<LOGS, false, true>(loc, p, parity, use_list, grid, status, st);
    else launch_passes<LOGS, false, false>(loc, p, parity, use_list, grid, status, st);
  }
  return cudaGetLastError();
}

// The whole-launch driver over any region locator: the key-by-key kernel
// and the rebuild for even regions, then for odd ones, then the fallback.
template <class Loc>
cudaError_t run_rebuild(const Loc& loc, const Partition& p, Op op, uint32_t* status, cudaStream_t st,
                        uint32_t sparse_max) {
  cudaError_t e = cudaMemsetAsync(p.deferred, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  switch (p.log_region) {
    case 11: e = run_phases<11>(loc, p, op, sparse_max, status, st); break;
    case 12: e = run_phases<12>(loc, p, op, sparse_max, status, st); break;
    case 13: e = run_phases<13>(loc, p, op, sparse_max, status, st); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  k_fallback<Loc><<<1, 32, 0, st>>>(loc, p, op == Op::kDelete ? 1 : 0, status);
  count_launch();
  return cudaGetLastError();
}

}  // namespace
}  // namespace gqf
