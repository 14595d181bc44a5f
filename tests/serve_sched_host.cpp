// The serving loop's scheduling policy (cqf_gb300/csrc/serve_sched.h)
// compiled for the host, behind a C interface for tests/test_serve_sched.py.
#include <cstdint>
#include <vector>

#include "../cqf_gb300/csrc/serve_sched.h"

using namespace gqf::serve;

extern "C" {
void* ring_new(uint64_t cap) { return new Ring(cap); }
void ring_free(void* r) { delete static_cast<Ring*>(r); }
int ring_alloc(void* r, uint64_t bytes, uint64_t* off) { return static_cast<Ring*>(r)->alloc(bytes, off) ? 1 : 0; }
int ring_release(void* r, uint64_t off, uint64_t bytes) {
  return static_cast<Ring*>(r)->release(off, bytes) ? 1 : 0;
}
uint64_t ring_used(void* r) { return static_cast<Ring*>(r)->used(); }
uint64_t plan(const int* ops, const int* kih, const uint64_t* ns, uint64_t len, uint64_t max_keys,
              uint64_t max_bytes) {
  std::vector<Pending> q;
  for (uint64_t i = 0; i < len; i++) q.push_back({ops[i], kih[i], ns[i]});
  return plan_group(q, max_keys, max_bytes);
}
uint64_t split(int op, uint64_t ring_bytes) { return split_keys(op, ring_bytes); }
uint64_t req_bytes(int op, uint64_t n) { return request_bytes(op, n); }
int cls(int op, int kih) { return op_class(op, kih); }
}
