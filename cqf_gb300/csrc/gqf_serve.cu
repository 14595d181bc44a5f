// Serving loop: continuous batching of bulk requests against one resident
// filter.
//
// The reference offers only bulk calls on caller-owned device buffers, one
// at a time (src/gqf.cu:3184-3419); a service built on it runs requests back
// to back.  Here a server owns a staging ring in HBM and two host threads:
//
//   scheduler  takes queued requests in arrival order, groups consecutive
//              requests of one coalescing class (serve_sched.h) into one
//              launch, admits the group when its bytes fit the free part of
//              the ring (admission by free device memory), copies the keys
//              in on a copy stream, enqueues the bulk call on the compute
//              stream and a get's result copies on a third stream, so that
//              they overlap the next launch;
//   completer  waits for each group's completion event in order, stamps the
//              requests' latencies, releases their ring space and wakes
//              waiting clients and the scheduler.
//
// Groups run in arrival order on one compute stream, so every request sees
// exactly the filter that running the requests one by one would give it (a
// group of inserts, or of deletes, applies its multiset in one pass; deletes
// clamp at zero, so removing A then B equals removing A + B).  Copies of later
// groups overlap the compute of earlier ones.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gqf_kernels.cuh"
#include "serve_sched.h"
#include "../../include/gqf.h"

using namespace gqf;
using namespace gqf::serve;

namespace {

using Clock = std::chrono::steady_clock;

// One launchable piece of a submitted request (a request larger than a
// quarter of the ring is split into several, all under one ticket).
struct Request {
  int64_t ticket;
  int op;
  int key_is_hash;
  const uint64_t* keys;
  uint64_t* counts;
  uint64_t n;
  bool on_device;
};

struct Ticket {
  int parts_left = 0;
  bool done = false;
  bool failed = false;
  double latency_ms = 0;
  Clock::time_point t_submit;
};

struct Group {
  std::vector<Request> reqs;
  uint64_t off = 0, bytes = 0;
  cudaEvent_t done = nullptr;
  bool failed = false;
};

}  // namespace

struct gqf_server {
  QF* qf = nullptr;
  uint8_t* staging = nullptr;
  uint64_t staging_bytes = 0;
  uint64_t max_group_keys = 1ULL << 25;
  cudaStream_t copy = nullptr, comp = nullptr, out = nullptr;
  int device = 0;

  std::mutex mu;
  std::condition_variable cv_work, cv_space, cv_done, cv_inflight;
  std::deque<Request> pending;
  std::deque<Group> inflight;
  std::unordered_map<int64_t, Ticket> tickets;
  Ring ring;
  int64_t next_ticket = 0;
  int launching = 0;  // groups taken from pending, not yet in flight
  bool stop = false;
  bool sched_done = false;
  std::thread scheduler, completer;
  std::vector<cudaEvent_t> spare_events;
  std::string error;

  // statistics
  std::vector<double> lat_ms;
  uint64_t n_requests = 0, n_groups = 0, n_keys = 0;
  uint64_t peak_used = 0;
};

namespace {

cudaEvent_t take_event(gqf_server* s) {
  if (!s->spare_events.empty()) {
    cudaEvent_t e = s->spare_events.back();
    s->spare_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  return e;
}

// Enqueues one admitted group; returns false on a launch error.
bool launch_group(gqf_server* s, Group& g, cudaEvent_t copied, cudaEvent_t computed) {
  const int op = g.reqs[0].op;
  const int key_is_hash = g.reqs[0].key_is_hash;
  bool reduce = false;
  uint64_t total = 0;
  for (const Request& r : g.reqs) {
    total += r.n;
    reduce |= r.op == kInsertReduce;
  }
  uint64_t* keys = reinterpret_cast<uint64_t*>(s->staging + g.off);
  uint64_t* outs = keys + total;
  uint64_t at = 0;
  for (const Request& r : g.reqs) {
    if (cudaMemcpyAsync(keys + at, r.keys, r.n * 8, r.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        s->copy) != cudaSuccess)
      return false;
    at += r.n;
  }
  if (cudaEventRecord(copied, s->copy) != cudaSuccess || cudaStreamWaitEvent(s->comp, copied, 0) != cudaSuccess)
    return false;
  const uint8_t flags = QF_NO_LOCK | (key_is_hash ? QF_KEY_IS_HASH : 0);
  int rc = 0;
  if (op == kGet) {
    rc = gqf_bulk_get_async(s->qf, total, keys, outs, flags, s->comp);
    if (cudaEventRecord(computed, s->comp) != cudaSuccess || cudaStreamWaitEvent(s->out, computed, 0) != cudaSuccess)
      return false;
    at = 0;
    for (const Request& r : g.reqs) {
      if (rc == 0 && cudaMemcpyAsync(r.counts, outs + at, r.n * 8,
                                     r.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                     s->out) != cudaSuccess)
        rc = -1;
      at += r.n;
    }
    if (cudaEventRecord(g.done, s->out) != cudaSuccess) return false;
    return rc == 0;
  } else if (op == kDelete) {
    rc = gqf_bulk_delete_async(s->qf, total, keys, flags, s->comp);
  } else if (reduce) {
    rc = gqf_bulk_insert_reduce_async(s->qf, total, keys, flags, s->comp);
  } else {
    rc = gqf_bulk_insert_async(s->qf, total, keys, flags, s->comp);
  }
  if (cudaEventRecord(g.done, s->comp) != cudaSuccess) return false;
  return rc == 0;
}

void scheduler_main(gqf_server* s) {
  cudaSetDevice(s->device);
  std::vector<cudaEvent_t> copied_events, computed_events;
  size_t ce = 0;
  for (;;) {
    Group g;
    cudaEvent_t copied, computed;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
      if (s->pending.empty()) {  // stop requested and nothing left
        s->sched_done = true;
        s->cv_inflight.notify_all();
        break;
      }
      std::deque<Pending> view;
      for (size_t i = 0; i < s->pending.size() && i < 4096; i++)
        view.push_back({s->pending[i].op, s->pending[i].key_is_hash, s->pending[i].n});
      // at most half the ring per launch, so that the next one's copies can
      // proceed while it runs
      const size_t k = plan_group(view, s->max_group_keys, s->ring.capacity() / 2);
      uint64_t total = 0;
      for (size_t i = 0; i < k; i++) total += s->pending[i].n;
      const uint64_t bytes = request_bytes(s->pending[0].op, total);
      // admission: wait until the group's bytes are free in the ring
      s->cv_space.wait(lk, [&] { return s->ring.alloc(bytes, &g.off); });
      s->peak_used = std::max(s->peak_used, s->ring.used());
      g.bytes = bytes;
      for (size_t i = 0; i < k; i++) {
        g.reqs.push_back(s->pending.front());
        s->pending.pop_front();
      }
      g.done = take_event(s);
      s->launching++;
      if (copied_events.size() < 64) {
        cudaEvent_t e = nullptr, f = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&f, cudaEventDisableTiming);
        copied_events.push_back(e);
        computed_events.push_back(f);
      }
      copied = copied_events[ce % copied_events.size()];
      computed = computed_events[ce % computed_events.size()];
      ce++;
    }
    g.failed = !launch_group(s, g, copied, computed);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (g.failed && s->error.empty()) s->error = gqf_last_error();
      s->n_groups++;
      s->launching--;
      s->inflight.push_back(std::move(g));
    }
    s->cv_inflight.notify_one();
  }
  // a stream wait captured each record when it was enqueued: safe to destroy
  for (cudaEvent_t e : copied_events) cudaEventDestroy(e);
  for (cudaEvent_t e : computed_events) cudaEventDestroy(e);
}

void finish_request(gqf_server* s, const Request& r, bool failed, Clock::time_point now) {
  auto it = s->tickets.find(r.ticket);
  if (it == s->tickets.end()) return;
  Ticket& t = it->second;
  t.failed |= failed;
  if (--t.parts_left > 0) return;
  t.done = true;
  t.latency_ms = std::chrono::duration<double, std::milli>(now - t.t_submit).count();
  s->lat_ms.push_back(t.latency_ms);
  s->n_requests++;
}

void completer_main(gqf_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    Group* g = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_inflight.wait(lk, [&] { return !s->inflight.empty() || s->sched_done; });
      if (s->inflight.empty()) return;  // the scheduler has exited and all groups completed
      g = &s->inflight.front();  // only this thread pops; push_back keeps references valid
    }
    const bool failed = g->failed || cudaEventSynchronize(g->done) != cudaSuccess;
    const Clock::time_point now = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (const Request& r : g->reqs) {
        finish_request(s, r, failed, now);
        s->n_keys += r.n;
      }
      s->ring.release(g->off, g->bytes);
      s->spare_events.push_back(g->done);
      s->inflight.pop_front();
    }
    s->cv_space.notify_all();
    s->cv_done.notify_all();
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const double x = p * (double)(v.size() - 1);
  const size_t i = (size_t)x;
  const double f = x - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int gqf_server_create(QF* qf, uint64_t staging_bytes, gqf_server** out) {
  if (!out || !qf) return -1;
  *out = nullptr;
  gqf_server* s = new gqf_server();
  s->qf = qf;
  cudaGetDevice(&s->device);
  if (staging_bytes == 0) {  // a quarter of the free device memory, at most 4 GiB
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    staging_bytes = std::min<uint64_t>(fr / 4, 4ULL << 30);
  }
  staging_bytes &= ~255ULL;
  if (staging_bytes < (1ULL << 20) || cudaMalloc((void**)&s->staging, staging_bytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->comp, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->out, cudaStreamNonBlocking) != cudaSuccess) {
    if (s->staging) cudaFree(s->staging);
    delete s;
    return -1;
  }
  s->staging_bytes = staging_bytes;
  s->ring = Ring(staging_bytes);
  s->scheduler = std::thread(scheduler_main, s);
  s->completer = std::thread(completer_main, s);
  *out = s;
  return 0;
}

int64_t gqf_server_submit(gqf_server* s, int op, const uint64_t* keys, uint64_t n, uint64_t* counts,
                          uint32_t flags) {
  if (!s || op < GQF_OP_GET || op > GQF_OP_INSERT_REDUCE || (n && !keys) || (op == GQF_OP_GET && n && !counts))
    return -1;
  const Clock::time_point now = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return -1;
  const int64_t id = s->next_ticket++;
  Ticket& t = s->tickets[id];
  t.t_submit = now;
  const bool dev = (flags & GQF_SERVE_DEVICE_PTRS) != 0;
  const int kih = (flags & QF_KEY_IS_HASH) ? 1 : 0;
  if (n == 0) {  // nothing to do: done at once
    t.done = true;
    s->cv_done.notify_all();
    return id;
  }
  const uint64_t part = split_keys(op, s->staging_bytes);
  t.parts_left = (int)((n + part - 1) / part);
  for (uint64_t a = 0; a < n; a += part)
    s->pending.push_back({id, op, kih, keys + a, counts ? counts + a : nullptr, std::min(part, n - a), dev});
  s->cv_work.notify_one();
  return id;
}

int gqf_server_poll(gqf_server* s, int64_t ticket) {
  if (!s) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return -1;
  if (!it->second.done) return 0;
  return it->second.failed ? -1 : 1;
}

int gqf_server_wait(gqf_server* s, int64_t ticket, double* latency_ms) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return -1;
  s->cv_done.wait(lk, [&] { return it->second.done; });
  const bool failed = it->second.failed;
  if (latency_ms) *latency_ms = it->second.latency_ms;
  s->tickets.erase(it);
  return failed ? -1 : 0;
}

int gqf_server_drain(gqf_server* s) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->pending.empty() && s->inflight.empty() && s->launching == 0; });
  return s->error.empty() ? 0 : -1;
}

int gqf_server_stats(gqf_server* s, double* out, int n) {
  if (!s || !out) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  const double v[GQF_SERVE_STATS] = {
      (double)s->n_requests, (double)s->n_groups, (double)s->n_keys,
      percentile(s->lat_ms, 0.5), percentile(s->lat_ms, 0.99),
      s->lat_ms.empty() ? 0.0 : *std::max_element(s->lat_ms.begin(), s->lat_ms.end()),
      (double)s->staging_bytes, (double)s->peak_used};
  for (int i = 0; i < n && i < GQF_SERVE_STATS; i++) out[i] = v[i];
  return 0;
}

int gqf_server_reset_stats(gqf_server* s) {
  if (!s) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat_ms.clear();
  s->n_requests = s->n_groups = s->n_keys = 0;
  s->peak_used = s->ring.used();
  return 0;
}

void gqf_server_destroy(gqf_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->scheduler.join();  // drains what is queued, then marks itself done
  s->completer.join();  // completes what is in flight
  cudaStreamSynchronize(s->comp);
  cudaStreamSynchronize(s->copy);
  cudaStreamSynchronize(s->out);
  for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
  cudaStreamDestroy(s->copy);
  cudaStreamDestroy(s->comp);
  cudaStreamDestroy(s->out);
  cudaFree(s->staging);
  delete s;
}

}  // extern "C"
