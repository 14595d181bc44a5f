// Prints the byte layout of the reference's host structs (as its own headers
// and this compiler lay them out) as JSON, for baseline/refgpu.py, which
// builds those structs in device memory to drive the reference's kernels.
// Compiled from the reference's headers where they lie; adds nothing to them.
#include <cstddef>
#include <cstdio>

#include "gqf_int.cuh"

int main() {
  std::printf("{\n");
  std::printf(" \"sizeof_QF\": %zu,\n", sizeof(QF));
  std::printf(" \"QF_runtimedata\": %zu,\n", offsetof(QF, runtimedata));
  std::printf(" \"QF_metadata\": %zu,\n", offsetof(QF, metadata));
  std::printf(" \"QF_blocks\": %zu,\n", offsetof(QF, blocks));
  std::printf(" \"sizeof_qfruntime\": %zu,\n", sizeof(qfruntime));
  std::printf(" \"qfruntime_num_locks\": %zu,\n", offsetof(qfruntime, num_locks));
  std::printf(" \"qfruntime_locks\": %zu,\n", offsetof(qfruntime, locks));
  std::printf(" \"qfruntime_buffers\": %zu,\n", offsetof(qfruntime, buffers));
  std::printf(" \"qfruntime_buffer_sizes\": %zu,\n", offsetof(qfruntime, buffer_sizes));
  std::printf(" \"sizeof_qfmetadata\": %zu,\n", sizeof(qfmetadata));
  std::printf(" \"sizeof_qfblock\": %zu,\n", sizeof(qfblock));
  std::printf(" \"qfruntime_wait_times\": %zu\n", offsetof(qfruntime, wait_times));
  std::printf("}\n");
  return 0;
}
