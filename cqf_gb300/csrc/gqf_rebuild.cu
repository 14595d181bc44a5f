// Region rebuild for one filter (the instantiation for a set of filters is
// in gqf_set.cu); the kernels are in gqf_rebuild_impl.cuh.
#include "gqf_rebuild_impl.cuh"

namespace gqf {

size_t rebuild_smem_bytes(int log_region) {
  switch (log_region) {
    case 11: return Lay<11, false>::BYTES;
    case 12: return Lay<12, false>::BYTES;
    case 13: return Lay<13, false>::BYTES;
  }
  return 0;
}

cudaError_t launch_rebuild(const Geom& g, const Partition& p, Op op, quotient_filter* dqf,
                           uint32_t* status, cudaStream_t st, uint32_t sparse_max) {
  return run_rebuild(OneFilter{g, dqf}, p, op, status, st, sparse_max);
}

}  // namespace gqf
