// Host build of the device's single-key algorithms (gqf::Serial, used by the
// point API and the bulk path's serial fallback) for CPU tests: the same
// source, compiled for the host, on a host array of blocks.
#include "../cqf_gb300/csrc/gqf_device.cuh"
#include <cmath>
#include <cstring>
#include <cstdlib>
using namespace gqf;
extern "C" {
void* sh_new(int nbits) {
  quotient_filter* q = (quotient_filter*)calloc(1, sizeof(quotient_filter));
  q->nslots = 1ULL << nbits; q->xnslots = q->nslots + (uint64_t)(10*std::sqrt((double)q->nslots));
  q->nblocks = (q->xnslots + 63)/64; q->range = q->nslots << 8;
  q->blocks = (Block*)calloc(q->nblocks, sizeof(Block));
  return q;
}
int sh_insert1(void* p, uint64_t h) { return Serial((quotient_filter*)p).insert1(h); }
int sh_insert(void* p, uint64_t h, uint64_t c) { return Serial((quotient_filter*)p).insert(h, c); }
int sh_remove(void* p, uint64_t h) { return Serial((quotient_filter*)p).remove(h, 1); }
uint64_t sh_count(void* p, uint64_t h) { return Serial((quotient_filter*)p).count(h); }
void sh_export(void* p, uint8_t* out) {
  quotient_filter* q = (quotient_filter*)p;
  for (uint64_t b = 0; b < q->nblocks; b++) {
    uint8_t* d = out + b*81; Block& s = q->blocks[b];
    d[0] = s.offset < 255 ? s.offset : 255;
    memcpy(d+1, &s.occupieds, 8); memcpy(d+9, &s.runends, 8); memcpy(d+17, s.slots, 64);
  }
}
}
extern "C" {
int sh_sparse_fits(void* p, uint64_t region_end, uint64_t grow, uint64_t bound) {
  return Serial((quotient_filter*)p).sparse_fits(region_end, grow, bound) ? 1 : 0;
}
uint64_t sh_insert_growth(uint64_t count) { return Serial::insert_growth(count); }
int64_t sh_snapshot(void* p, Block* out) {
  quotient_filter* q = (quotient_filter*)p;
  memcpy(out, q->blocks, q->nblocks * sizeof(Block));
  return (int64_t)q->nblocks;
}
// Highest slot whose byte, occupied or runend bit differs from the snapshot
// (a changed block offset counts as the block's first slot); -1 if none.
int64_t sh_highest_change(void* p, const Block* before) {
  quotient_filter* q = (quotient_filter*)p;
  for (int64_t b = (int64_t)q->nblocks - 1; b >= 0; b--) {
    const Block& x = q->blocks[b];
    const Block& y = before[b];
    for (int j = 63; j >= 0; j--)
      if (x.slots[j] != y.slots[j] || (((x.runends ^ y.runends) >> j) & 1ULL) ||
          (((x.occupieds ^ y.occupieds) >> j) & 1ULL))
        return 64 * b + j;
    if (x.offset != y.offset) return 64 * b;
  }
  return -1;
}
}
