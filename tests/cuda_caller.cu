// A CUDA caller of the device point API, built the way the reference's own
// callers are (include/point_wrapper.cuh:137-156 calling point_insert from a
// user kernel, linked with -rdc=true as in Makefile:35):
//
//   nvcc -rdc=true -gencode arch=compute_103a,code=sm_103a cuda_caller.cu -I include \
//        -L cqf_gb300/_lib -lgqf_gb300_device -lgqf_gb300 -o cuda_caller
//
// Usage: cuda_caller NBITS KEYS_IN DUMP_OUT COUNTS_OUT
//   KEYS_IN:    raw uint64 keys (host byte order)
//   DUMP_OUT:   the filter after every key was inserted once by point_insert
//               from this program's kernel, in the packed export format
//   COUNTS_OUT: uint64 point_query count of each key, from another kernel
// Exit status 0 on success; every insert must return QF_ITEM_INSERTED.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gqf.cuh"

__global__ void insert_all(QF* qf, const uint64_t* keys, uint64_t n, int* bad) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (point_insert(qf, keys[i], 0, QF_WAIT_FOR_LOCK) != QF_ITEM_INSERTED) atomicAdd(bad, 1);
}

__global__ void query_all(QF* qf, const uint64_t* keys, uint64_t n, uint64_t* counts) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t v = 0;
  counts[i] = point_query(qf, keys[i], 0, v, QF_NO_LOCK);
}

static int fail(const char* what) {
  std::fprintf(stderr, "cuda_caller: %s (%s)\n", what, gqf_last_error());
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 5) return fail("usage: cuda_caller NBITS KEYS_IN DUMP_OUT COUNTS_OUT");
  const int nbits = std::atoi(argv[1]);
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return fail("cannot open the keys file");
  std::vector<uint64_t> keys;
  uint64_t k;
  while (std::fread(&k, sizeof k, 1, f) == 1) keys.push_back(k);
  std::fclose(f);
  const uint64_t n = keys.size();

  QF* qf = nullptr;
  qf_malloc_device(&qf, nbits, true);
  if (!qf) return fail("qf_malloc_device");
  uint64_t *d_keys = nullptr, *d_counts = nullptr;
  int* d_bad = nullptr;
  if (cudaMalloc(&d_keys, n * sizeof(uint64_t)) != cudaSuccess ||
      cudaMalloc(&d_counts, n * sizeof(uint64_t)) != cudaSuccess || cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess)
    return fail("cudaMalloc");
  cudaMemcpy(d_keys, keys.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice);
  cudaMemset(d_bad, 0, sizeof(int));
  const unsigned grid = (unsigned)((n + 255) / 256);
  insert_all<<<grid, 256>>>(qf, d_keys, n, d_bad);
  query_all<<<grid, 256>>>(qf, d_keys, n, d_counts);
  if (cudaDeviceSynchronize() != cudaSuccess) return fail("kernels");
  int bad = 0;
  cudaMemcpy(&bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost);
  if (bad) return fail("an insert did not return QF_ITEM_INSERTED");

  std::vector<unsigned char> dump(gqf_export_size(qf));
  if (gqf_export(qf, dump.data(), dump.size()) != 0) return fail("gqf_export");
  std::vector<uint64_t> counts(n);
  cudaMemcpy(counts.data(), d_counts, n * sizeof(uint64_t), cudaMemcpyDeviceToHost);
  FILE* o = std::fopen(argv[3], "wb");
  FILE* c = std::fopen(argv[4], "wb");
  if (!o || !c) return fail("cannot open an output file");
  std::fwrite(dump.data(), 1, dump.size(), o);
  std::fwrite(counts.data(), sizeof(uint64_t), n, c);
  std::fclose(o);
  std::fclose(c);
  cudaFree(d_keys);
  cudaFree(d_counts);
  cudaFree(d_bad);
  qf_destroy_device(qf);
  return 0;
}
