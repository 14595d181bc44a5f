// Export / import in the reference's packed format, and the serial-apply
// testing kernel.
//
// Packed format (include/gqf_int.cuh:38-57): per block an 8-bit offset that
// saturates at 255 (insert1 / insert_replace, src/gqf.cu:1078-1088,
// :1747-1753), occupieds, runends, 64 slot bytes -- 81 bytes, unaligned.
#include "gqf_kernels.cuh"

namespace gqf {
namespace {

__global__ void k_export(Geom g, uint8_t* __restrict__ out) {
  uint64_t b = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (b >= g.nblocks) return;
  const Block& s = g.blocks[b];
  uint8_t* d = out + b * 81;
  uint32_t off = s.offset;
  d[0] = (uint8_t)(off < 255 ? off : 255);
  unsigned long long o = s.occupieds, r = s.runends;
  for (int i = 0; i < 8; i++) {
    d[1 + i] = (uint8_t)(o >> (8 * i));
    d[9 + i] = (uint8_t)(r >> (8 * i));
  }
  const uint4* src = reinterpret_cast<const uint4*>(s.slots);
  for (int c = 0; c < 4; c++) {
    uint4 v = src[c];
    uint32_t w[4] = {v.x, v.y, v.z, v.w};
    for (int k = 0; k < 16; k++) d[17 + 16 * c + k] = (uint8_t)(w[k >> 2] >> (8 * (k & 3)));
  }
}

__global__ void k_import(Geom g, const uint8_t* __restrict__ in) {
  uint64_t b = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (b >= g.nblocks) return;
  const uint8_t* s = in + b * 81;
  Block& d = g.blocks[b];
  unsigned long long o = 0, r = 0;
  for (int i = 0; i < 8; i++) {
    o |= (unsigned long long)s[1 + i] << (8 * i);
    r |= (unsigned long long)s[9 + i] << (8 * i);
  }
  d.occupieds = o;
  d.runends = r;
  d.offset = s[0];
  d.pad0 = 0;
  d.pad1 = 0;
  for (int i = 0; i < 64; i++) d.slots[i] = s[17 + i];
}

// Saturated (255) offsets of an imported image are replaced by exact ones,
// block by block in order: block_offset's fallback (src/gqf.cu:619-630).
__global__ void k_import_fix(quotient_filter* dqf, const uint8_t* __restrict__ in) {
  if (threadIdx.x || blockIdx.x) return;
  Serial S(dqf);
  for (uint64_t b = 1; b < S.nblocks; b++) {
    if (in[b * 81] != 255) continue;
    uint64_t e = S.run_end(64 * b - 1);
    S.b[b].offset = (uint32_t)(e >= 64 * b ? e - 64 * b + 1 : 0);
  }
}

__global__ void k_serial_apply(quotient_filter* dqf, const uint64_t* __restrict__ hashes, uint64_t n,
                               int op) {
  if (threadIdx.x || blockIdx.x) return;
  Serial S(dqf);
  for (uint64_t i = 0; i < n; i++) {
    uint64_t h = hashes[i];
    if (h >= dqf->range) {
      atomicOr(dqf->status, kStBadKey);
      continue;
    }
    if (op == 0) {
      if (S.insert1(h) < 0) atomicOr(dqf->status, kStFull);
    } else {
      S.remove(h, 1);
    }
  }
}

}  // namespace

cudaError_t launch_export(const Geom& g, uint8_t* packed, cudaStream_t st) {
  k_export<<<(unsigned)((g.nblocks + 255) / 256), 256, 0, st>>>(g, packed);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_import(const Geom& g, const uint8_t* packed, cudaStream_t st) {
  k_import<<<(unsigned)((g.nblocks + 255) / 256), 256, 0, st>>>(g, packed);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_import_fix(quotient_filter* dqf, const uint8_t* packed, cudaStream_t st) {
  k_import_fix<<<1, 32, 0, st>>>(dqf, packed);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_serial_apply(quotient_filter* dqf, const uint64_t* hashes, uint64_t n, int op,
                                cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_serial_apply<<<1, 32, 0, st>>>(dqf, hashes, n, op);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
