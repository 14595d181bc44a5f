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
//   * the CTA stages a window of LOGS-region + PUSH slots in shared memory
//     (the region plus the head of the next one, which its growth may push);
//   * it sorts the region's new keys in shared memory (bitonic), merges them
//     run by run with the old counters (decode_counter / encode_counter,
//     src/gqf.cu:1216-1345), and recomputes every run position with one
//     block-wide max-plus scan: end(q) = max(q + L_q - 1, end(prev) + L_q);
//   * it writes back only the blocks that changed.
//
// A rebuild whose changes would reach past the window (a cluster longer than
// PUSH slots, or the end of the table) is deferred: nothing is written and the
// region is applied afterwards by a single-thread serial pass built from the
// reference's own single-key algorithms (gqf_device.cuh), which handles any
// cluster length and reports a full table like the reference does.
#include "gqf_kernels.cuh"

namespace gqf {
namespace {

constexpr int kNeg = -(1 << 28);  // "minus infinity" of the max-plus scan

template <int LOGS>
struct Cfg;
template <>
struct Cfg<11> { static constexpr int PUSH = 1024, NT = 256, KMAX = 2048; };
template <>
struct Cfg<12> { static constexpr int PUSH = 1024, NT = 256, KMAX = 4096; };
template <>
struct Cfg<13> { static constexpr int PUSH = 2048, NT = 512, KMAX = 4096; };

template <int LOGS>
struct Lay {
  static constexpr int REG = 1 << LOGS;
  static constexpr int PUSH = Cfg<LOGS>::PUSH;
  static constexpr int NT = Cfg<LOGS>::NT;
  static constexpr int KMAX = Cfg<LOGS>::KMAX;
  static constexpr int WIN = REG + PUSH;
  static constexpr int WB = WIN / 64;
  static constexpr int QPT = WIN / NT;
  static_assert(WIN % NT == 0, "quotients split evenly over threads");
  static_assert(PUSH < REG, "a window must not reach the region after next");
  // shared memory carve-up (bytes)
  static constexpr int IMG = WB * 96;
  static constexpr int OFF_IMG0 = 0;
  static constexpr int OFF_IMG1 = OFF_IMG0 + IMG;
  static constexpr int OFF_KEYS = OFF_IMG1 + IMG;                 // u64[KMAX]
  static constexpr int OFF_NOCC = OFF_KEYS + KMAX * 8;            // u64[WB]
  static constexpr int OFF_TCH = OFF_NOCC + WB * 8;               // u64[WB]
  static constexpr int OFF_RPOS = OFF_TCH + WB * 8;               // u16[WIN + 8]
  static constexpr int OFF_PREF = OFF_RPOS + (WIN + 8) * 2;       // u16[WIN]
  static constexpr int OFF_ORANK = OFF_PREF + WIN * 2;            // u16[WB + 1]
  static constexpr int OFF_RRANK = OFF_ORANK + (WB + 8) * 2;      // u16[WB + 1]
  static constexpr int BYTES = OFF_RRANK + (WB + 8) * 2;
};

// ----------------------------------------------------- shared-memory image

struct Img {
  uint8_t* p;
  __device__ uint8_t& slot(int i) const { return p[(i >> 6) * 96 + 32 + (i & 63)]; }
  __device__ unsigned long long& occ(int w) const { return *reinterpret_cast<unsigned long long*>(p + w * 96); }
  __device__ unsigned long long& run(int w) const { return *reinterpret_cast<unsigned long long*>(p + w * 96 + 8); }
  __device__ uint32_t& off(int w) const { return *reinterpret_cast<uint32_t*>(p + w * 96 + 16); }
  __device__ int is_end(int i) const { return (int)((run(i >> 6) >> (i & 63)) & 1ULL); }
  __device__ void set_end(int i) const {
    uint32_t* w = reinterpret_cast<uint32_t*>(p + (i >> 6) * 96 + 8) + ((i >> 5) & 1);
    atomicOr(w, 1u << (i & 31));
  }
};

// Merge one run's old counters with the run's sorted new keys and return the
// new run length; with WRITE, also emit the bytes at out[pos..].
//   keys[ki..kj): (local << 32) | multiplicity, sorted, all with this quotient.
template <bool DEL, bool WRITE>
__device__ int merge_run(Img cur, bool has_old, int s, int e, const unsigned long long* keys, int ki,
                         int kj, Img out, int pos) {
  auto get = [&](uint64_t i) -> uint64_t { return cur.slot((int)i); };
  auto end = [&](uint64_t i) -> int { return cur.is_end((int)i); };
  int total = 0;
  bool have_old = has_old;
  int opos = s;
  uint32_t orem = 0;
  uint64_t ocnt = 0;
  int oend = 0;
  // the walk never leaves the run [s, e]
  const uint64_t lim = (uint64_t)e + 1;
  if (have_old) oend = (int)decode_counter(get, end, (uint64_t)opos, &orem, &ocnt, lim);
  int j = ki;
  uint8_t enc[16];
  while (have_old || j < kj) {
    uint32_t nrem = 0;
    uint64_t ncnt = 0;
    int jn = j;
    if (j < kj) {
      nrem = (uint32_t)((keys[j] >> 32) & 255);
      while (jn < kj && (uint32_t)((keys[jn] >> 32) & 255) == nrem) {
        ncnt += keys[jn] & 0xFFFFFFFFULL;
        jn++;
      }
    }
    if (have_old && (j >= kj || orem < nrem)) {
      int len = oend - opos + 1;
      if (WRITE)
        for (int t = 0; t < len; t++) out.slot(pos + total + t) = cur.slot(opos + t);
      total += len;
      if (cur.is_end(oend) || oend >= e) {
        have_old = false;
      } else {
        opos = oend + 1;
        oend = (int)decode_counter(get, end, (uint64_t)opos, &orem, &ocnt, lim);
      }
    } else {
      uint64_t c;
      bool advance_old = have_old && orem == nrem;
      if (advance_old)
        c = DEL ? (ocnt > ncnt ? ocnt - ncnt : 0) : ocnt + ncnt;
      else
        c = DEL ? 0 : ncnt;
      int len = encode_counter(nrem, c, enc);
      if (WRITE)
        for (int t = 0; t < len; t++) out.slot(pos + total + t) = enc[t];
      total += len;
      j = jn;
      if (advance_old) {
        if (cur.is_end(oend) || oend >= e) {
          have_old = false;
        } else {
          opos = oend + 1;
          oend = (int)decode_counter(get, end, (uint64_t)opos, &orem, &ocnt, lim);
        }
      }
    }
  }
  return total;
}

// Block-wide exclusive scan of max-plus maps f(x) = max(a, x + b).
template <int NT>
__device__ void scan_maps(int& a, int& b, int* sa, int* sb) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int ia = a, ib = b;  // inclusive
  for (int o = 1; o < 32; o <<= 1) {
    int pa = __shfl_up_sync(0xffffffffu, ia, o);
    int pb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {  // (pa,pb) first, then (ia,ib)
      ia = max(ia, pa + ib);
      ib = pb + ib;
    }
  }
  if (lane == 31) { sa[wid] = ia; sb[wid] = ib; }
  __syncthreads();
  if (wid == 0) {
    int wa = lane < NT / 32 ? sa[lane] : kNeg, wb = lane < NT / 32 ? sb[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int pa = __shfl_up_sync(0xffffffffu, wa, o);
      int pb = __shfl_up_sync(0xffffffffu, wb, o);
      if (lane >= o) { wa = max(wa, pa + wb); wb = pb + wb; }
    }
    sa[lane] = wa;
    sb[lane] = wb;
  }
  __syncthreads();
  // exclusive within warp
  int ea = __shfl_up_sync(0xffffffffu, ia, 1), eb = __shfl_up_sync(0xffffffffu, ib, 1);
  if (lane == 0) { ea = kNeg; eb = 0; }
  if (wid > 0) {  // prefix of earlier warps first
    int pa = sa[wid - 1], pb = sb[wid - 1];
    ea = max(ea, pa + eb);
    eb = pb + eb;
  }
  a = ea;
  b = eb;
  __syncthreads();
}

template <int LOGS, bool DEL>
__global__ void __launch_bounds__(Lay<LOGS>::NT, 1) k_rebuild(Geom g, Partition p, int parity,
                                                            uint32_t* status) {
  using L = Lay<LOGS>;
  constexpr int NT = L::NT, WB = L::WB, QPT = L::QPT, KMAX = L::KMAX;
  extern __shared__ __align__(128) uint8_t sm[];
  __shared__ int s_i[8];
  __shared__ int sa[32], sb[32];

  const uint32_t r = 2 * blockIdx.x + parity;
  if (r >= p.nregions) return;
  const uint32_t kbeg = p.region_start[r], kend = p.region_start[r + 1];
  if (kbeg == kend) return;
  const int tid = threadIdx.x;

  const uint64_t base = (uint64_t)r << LOGS;
  const uint64_t bw0 = base >> 6;
  const int wb = (int)min((uint64_t)WB, g.nblocks - bw0);
  const int win_valid = (int)min((uint64_t)wb * 64, g.xnslots - base);
  const int win_q = (int)min((uint64_t)L::WIN, g.nslots - base);
  const int wq_words = (win_q + 63) >> 6;

  unsigned long long* keys = reinterpret_cast<unsigned long long*>(sm + L::OFF_KEYS);
  unsigned long long* nocc = reinterpret_cast<unsigned long long*>(sm + L::OFF_NOCC);
  unsigned long long* tch = reinterpret_cast<unsigned long long*>(sm + L::OFF_TCH);
  uint16_t* rpos = reinterpret_cast<uint16_t*>(sm + L::OFF_RPOS);
  uint16_t* pref = reinterpret_cast<uint16_t*>(sm + L::OFF_PREF);
  uint16_t* orank = reinterpret_cast<uint16_t*>(sm + L::OFF_ORANK);
  uint16_t* rrank = reinterpret_cast<uint16_t*>(sm + L::OFF_RRANK);

  // ---- stage the window (wb blocks of 96 bytes) into image 0
  {
    const uint4* src = reinterpret_cast<const uint4*>(g.blocks + bw0);
    uint4* dst = reinterpret_cast<uint4*>(sm + L::OFF_IMG0);
    for (int i = tid; i < wb * 6; i += NT) dst[i] = src[i];
  }
  __syncthreads();
  const int c0 = (int)Img{sm + L::OFF_IMG0}.off(0) - 1;  // last slot used by earlier regions' runs
  int cur = 0;
  int dirty_lo = 1 << 30, dirty_hi = -1;
  // The previous region's runs fill the whole window: every run of this
  // region lies beyond it, so only the serial path can place them.  (This
  // also keeps all window positions far below the 16-bit tables' range.)
  bool deferred = c0 + 1 >= win_valid;

  for (uint32_t kr = kbeg; kr < kend && !deferred; kr += KMAX) {
    const int nk = (int)min((uint32_t)KMAX, kend - kr);
    int P = 2;
    while (P < nk) P <<= 1;
    for (int i = tid; i < P; i += NT)
      keys[i] = i < nk ? (((unsigned long long)p.keys[kr + i]) << 32) |
                             (p.counts ? (unsigned long long)p.counts[kr + i] : 1ULL)
                       : ~0ULL;
    for (int i = tid; i < WB; i += NT) { nocc[i] = 0; tch[i] = 0; }
    __syncthreads();
    // bitonic sort of the round's keys
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = tid; i < P; i += NT) {
          int ixj = i ^ j;
          if (ixj > i) {
            unsigned long long a = keys[i], b = keys[ixj];
            bool up = (i & k) == 0;
            if ((a > b) == up) { keys[i] = b; keys[ixj] = a; }
          }
        }
        __syncthreads();
      }
    }

    const Img C{sm + (cur ? L::OFF_IMG1 : L::OFF_IMG0)};
    const Img N{sm + (cur ? L::OFF_IMG0 : L::OFF_IMG1)};

    // ---- rank tables: occupied quotients per word, runends after c0 per word
    if (tid < 32) {
      const int lane = tid;
      int per = (WB + 31) / 32;
      int a = lane * per, b = min(a + per, WB);
      int so = 0, sr = 0;
      for (int w = a; w < b; w++) {
        if (w < wq_words) so += __popcll(C.occ(w));
        if (w < wb) {
          unsigned long long rw = C.run(w);
          int lo = 64 * w;
          if (c0 >= lo + 63) rw = 0;
          else if (c0 >= lo) rw &= ~0ULL << (c0 - lo + 1);
          sr += __popcll(rw);
        }
      }
      int io = so, ir = sr;
      for (int o = 1; o < 32; o <<= 1) {
        int t1 = __shfl_up_sync(0xffffffffu, io, o), t2 = __shfl_up_sync(0xffffffffu, ir, o);
        if (lane >= o) { io += t1; ir += t2; }
      }
      int eo = io - so, er = ir - sr;
      for (int w = a; w < b; w++) {
        orank[w] = (uint16_t)eo;
        rrank[w] = (uint16_t)er;
        if (w < wq_words) eo += __popcll(C.occ(w));
        if (w < wb) {
          unsigned long long rw = C.run(w);
          int lo = 64 * w;
          if (c0 >= lo + 63) rw = 0;
          else if (c0 >= lo) rw &= ~0ULL << (c0 - lo + 1);
          er += __popcll(rw);
        }
      }
      if (lane == 31) { s_i[0] = ir; }  // visible runends after c0
    }
    __syncthreads();
    const int nvis = s_i[0];
    for (int w = tid; w < wb; w += NT) {
      unsigned long long rw = C.run(w);
      int lo = 64 * w;
      if (c0 >= lo + 63) rw = 0;
      else if (c0 >= lo) rw &= ~0ULL << (c0 - lo + 1);
      int k = rrank[w];
      while (rw) {
        int bit = __ffsll((long long)rw) - 1;
        rpos[k++] = (uint16_t)(lo + bit);
        rw &= rw - 1;
      }
    }
    __syncthreads();

    const int fake0 = win_valid + 16;
    auto runpos = [&](int k) -> int { return k < nvis ? (int)rpos[k] : fake0 + (k - nvis); };
    auto rank_of = [&](int q) -> int {
      return (int)orank[q >> 6] + __popcll(C.occ(q >> 6) & ((1ULL << (q & 63)) - 1ULL));
    };
    auto old_run = [&](int q, int& s, int& e) {
      int k = rank_of(q);
      e = runpos(k);
      int pe = k ? runpos(k - 1) : c0;
      s = max(q, pe + 1);
    };

    // ---- per-quotient new run lengths; compose this thread's max-plus map
    const int qa = tid * QPT, qb = min(qa + QPT, win_q);
    int lo_k = 0, hi_k = nk;  // first key with quotient >= qa
    {
      unsigned long long probe = ((unsigned long long)qa) << 40;
      while (lo_k < hi_k) {
        int mid = (lo_k + hi_k) >> 1;
        if (keys[mid] < probe) lo_k = mid + 1; else hi_k = mid;
      }
    }
    int fa = kNeg, fb = 0;
    bool my_defer = false;
    {
      int ki = lo_k;
      for (int q = qa; q < qb; q++) {
        const bool occ = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
        int kj = ki;
        while (kj < nk && (int)(keys[kj] >> 40) == q) kj++;
        int s = 0, e = -1, len = 0;
        if (occ) { old_run(q, s, e); len = e - s + 1; }
        if (kj > ki) {
          atomicOr(&tch[q >> 6], 1ULL << (q & 63));
          if (occ && e >= win_valid) {
            my_defer = true;
          } else {
            len = merge_run<DEL, false>(C, occ, s, e, keys, ki, kj, N, 0);
          }
        }
        pref[q] = (uint16_t)len;
        if (len > 0) {
          atomicOr(&nocc[q >> 6], 1ULL << (q & 63));
          // compose f_q after the running map: f_q(x) = max(q + len - 1, x + len)
          fa = max(q + len - 1, fa + len);
          fb = fb + len;
        }
        ki = kj;
      }
    }
    if (__syncthreads_or(my_defer)) { deferred = true; break; }

    // ---- block scan: where does each thread's first quotient start from?
    scan_maps<NT>(fa, fb, sa, sb);
    {
      int x = max(fa, c0 + fb);  // end of all runs before qa
      for (int q = qa; q < qb; q++) {
        int len = pref[q];
        if (len > 0) x = max(q + len - 1, x + len);
        pref[q] = (uint16_t)(x + 1);
      }
    }
    __syncthreads();

    // ---- what changed?
    int qlo = 1 << 30, hi = -1;
    for (int q = qa; q < qb; q++) {
      const bool oo = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
      const bool no = (nocc[q >> 6] >> (q & 63)) & 1ULL;
      if (!oo && !no) continue;
      const bool touched = (tch[q >> 6] >> (q & 63)) & 1ULL;
      int s = 0, e = -1;
      if (oo) old_run(q, s, e);
      int ne = (int)pref[q] - 1;
      int prev = q ? (int)pref[q - 1] - 1 : c0;
      int ns = max(q, prev + 1);
      bool changed = touched || oo != no || (no && (ns != s || ne != e));
      if (changed) {
        qlo = min(qlo, q);
        if (oo) hi = max(hi, e);
        if (no) hi = max(hi, ne);
      }
    }
    // block min / max
    for (int o = 16; o; o >>= 1) {
      qlo = min(qlo, __shfl_xor_sync(0xffffffffu, qlo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (tid == 0) { s_i[1] = 1 << 30; s_i[2] = -1; }
    __syncthreads();
    if ((tid & 31) == 0) { atomicMin(&s_i[1], qlo); atomicMax(&s_i[2], hi); }
    __syncthreads();
    qlo = s_i[1];
    hi = s_i[2];
    if (hi < 0) continue;  // nothing changed in this round
    if (hi >= win_valid) { deferred = true; break; }
    // first slot that may change: start of the first changed run (old or new)
    int lo_slot;
    {
      int prev = qlo ? (int)pref[qlo - 1] - 1 : c0;
      int ns = max(qlo, prev + 1);
      lo_slot = ns;
      if ((C.occ(qlo >> 6) >> (qlo & 63)) & 1ULL) {
        int s, e;
        old_run(qlo, s, e);
        lo_slot = min(lo_slot, s);
      }
    }

    // ---- build the next image: copy, clear [lo_slot, hi], write runs
    {
      const uint4* src = reinterpret_cast<const uint4*>(C.p);
      uint4* dst = reinterpret_cast<uint4*>(N.p);
      for (int i = tid; i < wb * 6; i += NT) dst[i] = src[i];
    }
    __syncthreads();
    for (int i = lo_slot + tid; i <= hi; i += NT) N.slot(i) = 0;
    for (int w = (lo_slot >> 6) + tid; w <= (hi >> 6); w += NT) {
      int a = max(lo_slot, 64 * w) - 64 * w, b = min(hi, 64 * w + 63) - 64 * w;  // inclusive bit range
      unsigned long long m = (b == 63 ? ~0ULL : ((1ULL << (b + 1)) - 1ULL)) & (~0ULL << a);
      N.run(w) &= ~m;
    }
    __syncthreads();
    for (int q = max(qa, qlo); q < qb; q++) {
      if (!((nocc[q >> 6] >> (q & 63)) & 1ULL)) continue;
      int ne = (int)pref[q] - 1;
      int prev = q ? (int)pref[q - 1] - 1 : c0;
      int ns = max(q, prev + 1);
      if (ns > hi) break;
      if ((tch[q >> 6] >> (q & 63)) & 1ULL) {
        int kj, ki;
        {  // keys of q
          unsigned long long probe = ((unsigned long long)q) << 40;
          int l = 0, h = nk;
          while (l < h) { int m = (l + h) >> 1; if (keys[m] < probe) l = m + 1; else h = m; }
          ki = l;
          kj = ki;
          while (kj < nk && (int)(keys[kj] >> 40) == q) kj++;
        }
        const bool oo = (C.occ(q >> 6) >> (q & 63)) & 1ULL;
        int s = 0, e = -1;
        if (oo) old_run(q, s, e);
        merge_run<DEL, true>(C, oo, s, e, keys, ki, kj, N, ns);
      } else {
        int s, e;
        old_run(q, s, e);
        if (e >= win_valid || ne >= win_valid) continue;  // cannot happen: checked above
        for (int t = 0; t <= e - s; t++) N.slot(ns + t) = C.slot(s + t);
      }
      N.set_end(ne);
    }
    // occupieds of the window's quotient words
    for (int w = tid; w < wq_words; w += NT) N.occ(w) = nocc[w];
    // offsets of blocks 1 .. hi/64 (block 0 belongs to the previous region)
    for (int w = 1 + tid; w <= min(wb - 1, hi >> 6); w += NT) {
      int x = min(64 * w - 1, win_q - 1);
      int E = (int)pref[x] - 1;
      if (E < win_valid) N.off(w) = (uint32_t)max(0, E - 64 * w + 1);
    }
    __syncthreads();
    dirty_lo = min(dirty_lo, min(qlo, lo_slot) >> 6);
    dirty_hi = max(dirty_hi, hi >> 6);
    cur ^= 1;
  }

  if (deferred) {
    if (tid == 0) {
      uint32_t at = atomicAdd(&p.deferred[0], 1u);
      p.deferred[1 + at] = r;
      atomicOr(status, kStDeferred);
    }
    return;
  }
  if (dirty_hi < 0) return;
  {
    const uint4* src = reinterpret_cast<const uint4*>(sm + (cur ? L::OFF_IMG1 : L::OFF_IMG0)) + dirty_lo * 6;
    uint4* dst = reinterpret_cast<uint4*>(g.blocks + bw0 + dirty_lo);
    const int n16 = (dirty_hi - dirty_lo + 1) * 6;
    for (int i = tid; i < n16; i += NT) dst[i] = src[i];
  }
}

// Serial fallback for deferred regions: the reference's single-key
// operations, one key at a time, in region order.
__global__ void k_fallback(quotient_filter* dqf, Partition p, int del, uint32_t* status) {
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
  Serial S(dqf);
  const int shift = 8 + p.log_region;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t r = ids[i];
    for (uint32_t k = p.region_start[r]; k < p.region_start[r + 1]; k++) {
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

template <int LOGS>
cudaError_t run_phases(const Geom& g, const Partition& p, Op op, uint32_t* status, cudaStream_t st) {
  using L = Lay<LOGS>;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_rebuild<LOGS, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    cudaFuncSetAttribute(k_rebuild<LOGS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    configured = true;
  }
  const uint32_t half = (p.nregions + 1) / 2;
  for (int parity = 0; parity < 2; parity++) {
    uint32_t grid = parity ? p.nregions / 2 : half;
    if (!grid) continue;
    if (op == Op::kDelete)
      k_rebuild<LOGS, true><<<grid, L::NT, L::BYTES, st>>>(g, p, parity, status);
    else
      k_rebuild<LOGS, false><<<grid, L::NT, L::BYTES, st>>>(g, p, parity, status);
    count_launch();
  }
  return cudaGetLastError();
}

}  // namespace

size_t rebuild_smem_bytes(int log_region) {
  switch (log_region) {
    case 11: return Lay<11>::BYTES;
    case 12: return Lay<12>::BYTES;
    case 13: return Lay<13>::BYTES;
  }
  return 0;
}

cudaError_t launch_rebuild(const Geom& g, const Partition& p, Op op, quotient_filter* dqf,
                           uint32_t* status, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(p.deferred, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  switch (p.log_region) {
    case 11: e = run_phases<11>(g, p, op, status, st); break;
    case 12: e = run_phases<12>(g, p, op, status, st); break;
    case 13: e = run_phases<13>(g, p, op, status, st); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  k_fallback<<<1, 32, 0, st>>>(dqf, p, op == Op::kDelete ? 1 : 0, status);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
