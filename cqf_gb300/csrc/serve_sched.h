// Host-side policy of the serving loop (gqf_serve.cu): the staging ring that
// admits requests by free device memory, and the grouping of queued requests
// into coalesced launches.  Plain C++17 without CUDA, so the policy is tested
// on hosts without a GPU (tests/serve_sched_host.cpp).
#pragma once
#include <cstdint>
#include <deque>

namespace gqf {
namespace serve {

enum Op : int { kGet = 0, kInsert = 1, kDelete = 2, kInsertReduce = 3 };

// Coalescing class: consecutive requests of one class run as one launch and
// give the same results as run one by one, in order.  Inserts and counted
// inserts share a class (both add their multiset); gets, deletes and
// QF_KEY_IS_HASH batches stay apart.
inline int op_class(int op, int key_is_hash) {
  const int base = op == kInsertReduce ? kInsert : op;
  return base * 2 + (key_is_hash ? 1 : 0);
}

// Device bytes a request of n keys holds while in flight: its keys, and its
// counts for a get.
inline uint64_t request_bytes(int op, uint64_t n) {
  const uint64_t b = n * 8 * (op == kGet ? 2 : 1);
  return (b + 255) & ~255ULL;
}

// A ring of `cap` staging bytes.  Blocks are contiguous and are released in
// the order they were allocated (requests complete in order on one stream),
// so the free space is at most two runs: after the newest block and before
// the oldest one.
class Ring {
 public:
  explicit Ring(uint64_t cap = 0) : cap_(cap) {}
  uint64_t capacity() const { return cap_; }
  // Bytes not available: the live blocks and, when wrapped, the unused end
  // of the ring behind the newest block that wrapped.
  uint64_t used() const {
    if (blocks_.empty()) return 0;
    const uint64_t head = blocks_.back().off + blocks_.back().bytes, tail = blocks_.front().off;
    return head > tail ? head - tail : cap_ - tail + head;
  }
  size_t live() const { return blocks_.size(); }

  bool alloc(uint64_t bytes, uint64_t* off) {
    if (bytes == 0 || bytes > cap_) return false;
    if (blocks_.empty()) return push(0, bytes, off);
    const uint64_t head = blocks_.back().off + blocks_.back().bytes;  // end of the newest
    const uint64_t tail = blocks_.front().off;                         // start of the oldest
    if (head > tail) {  // not wrapped: free is [head, cap) and [0, tail)
      if (cap_ - head >= bytes) return push(head, bytes, off);
      if (tail >= bytes) return push(0, bytes, off);
      return false;
    }
    if (tail - head >= bytes) return push(head, bytes, off);  // wrapped: free is [head, tail)
    return false;
  }

  // Releases the oldest block; returns false if (off, bytes) is not it.
  bool release(uint64_t off, uint64_t bytes) {
    if (blocks_.empty() || blocks_.front().off != off || blocks_.front().bytes != bytes) return false;
    blocks_.pop_front();
    return true;
  }

 private:
  struct Block {
    uint64_t off, bytes;
  };
  bool push(uint64_t o, uint64_t bytes, uint64_t* off) {
    blocks_.push_back({o, bytes});
    *off = o;
    return true;
  }
  uint64_t cap_;
  std::deque<Block> blocks_;
};

// What the scheduler needs to know of a queued request.
struct Pending {
  int op;
  int key_is_hash;
  uint64_t n;
};

// Number of leading requests of `q` that form the next launch: all of one
// coalescing class, at most max_keys keys and max_bytes staging bytes in
// total (the first request alone always qualifies; the submitter splits
// requests larger than the ring).
template <class Q>
size_t plan_group(const Q& q, uint64_t max_keys, uint64_t max_bytes) {
  if (q.empty()) return 0;
  const int cls = op_class(q[0].op, q[0].key_is_hash);
  uint64_t keys = q[0].n, bytes = request_bytes(q[0].op, q[0].n);
  size_t k = 1;
  while (k < q.size() && op_class(q[k].op, q[k].key_is_hash) == cls) {
    const uint64_t nb = request_bytes(q[k].op, q[k].n);
    if (keys + q[k].n > max_keys || bytes + nb > max_bytes) break;
    keys += q[k].n;
    bytes += nb;
    k++;
  }
  return k;
}

// Keys per part when a request must be split to fit the ring (a quarter of
// it, so that a split request still overlaps copies with compute).
inline uint64_t split_keys(int op, uint64_t ring_bytes) {
  const uint64_t per = op == kGet ? 16 : 8;
  uint64_t k = (ring_bytes / 4) / per;
  k &= ~31ULL;
  return k ? k : 32;
}

}  // namespace serve
}  // namespace gqf
