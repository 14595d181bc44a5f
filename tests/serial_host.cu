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
