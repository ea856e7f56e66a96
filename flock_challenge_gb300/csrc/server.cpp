// Proof server: continuous batching of proof requests on one GPU.
//
// No reference counterpart: the reference's serving loop is a process per
// proof (benchmark-tools/worker) fed by the harness over IPC. Here a request
// (a seed and size, or host compressions) is queued; worker threads, each
// with its own prover state and CUDA stream, take requests as soon as the
// device-memory budget admits them, so the kernels of several proofs run
// concurrently and a small proof does not wait behind a large one. A worker's
// witness, codeword and Merkle buffers stay resident between its proofs and
// are released only when a queued request does not fit the budget otherwise.
// Every proof is the plain path's proof (same kernels, same transcript).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "flock_internal.h"
#include "prover.h"

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int log2_slots(size_t n) {
  size_t nn = n < 8 ? 8 : n;
  int l = 0;
  while (((size_t)1 << l) < nn) l++;
  return l;
}

struct Request {
  uint64_t id = 0;
  int n_log = 0;
  bool by_seed = true;
  uint64_t seed = 0;
  std::vector<flock_compression> inputs;
  int status = FLOCK_PENDING;
  std::vector<uint8_t> proof;
  double t_submit = 0, t_start = 0, t_done = 0;
};

struct Worker {
  ProverState* prover = nullptr;
  size_t reserved = 0;  // device bytes this worker's state holds (or is about to)
  bool busy = false;
  std::thread thread;
};

}  // namespace

struct flock_server {
  int device = 0;
  size_t budget = 0;  // 0 = no limit
  std::vector<Worker> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> reqs;
  uint64_t next_id = 1;
  bool stop = false;

  size_t reserved_total() const {
    size_t t = 0;
    for (const Worker& w : workers) t += w.reserved;
    return t;
  }
  bool fits(const Worker& w, size_t fp) const {
    if (budget == 0) return true;
    size_t mine = std::max(w.reserved, fp);
    return reserved_total() - w.reserved + mine <= budget;
  }
  void run(int wi);
};

// Requests of at least 2^kHighPriorityLog compressions run on their worker's
// high-priority stream: the p99 of a mixed load is set by the largest
// requests. Measured with 4 workers, Poisson 2^10..2^20 requests: p99 at the
// plain path's rate 399 ms with no priority, 380 ms from 2^19, 374 ms from
// 2^17 (at 1.05 of it: 428, 420, 413 ms); sustained throughput unchanged.
#ifndef FLOCK_SERVER_PRIORITY_LOG
#define FLOCK_SERVER_PRIORITY_LOG 17
#endif
constexpr int kHighPriorityLog = FLOCK_SERVER_PRIORITY_LOG;

void flock_server::run(int wi) {
  Worker& w = workers[wi];
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  while (true) {
    std::shared_ptr<Request> r;
    size_t fp = 0;
    // first queued request (in arrival order) that the budget admits
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      size_t f = flock_footprint_bytes((uint32_t)(*it)->n_log);
      if (fits(w, f)) {
        r = *it;
        fp = f;
        queue.erase(it);
        break;
      }
    }
    if (!r) {
      if (stop && queue.empty()) return;
      if (!queue.empty() && w.reserved > 0) {
        // a queued request does not fit: give this idle worker's memory back
        lk.unlock();
        flock_prover_trim(w.prover);
        lk.lock();
        w.reserved = 0;
        cv_work.notify_all();
        continue;
      }
      cv_work.wait(lk);
      continue;
    }
    w.busy = true;
    w.reserved = std::max(w.reserved, fp);
    r->t_start = now_ms();
    lk.unlock();
    std::vector<uint8_t> out;
    int rc;
    // the largest requests set the tail of the latency: their kernels go first
    flock_prover_set_priority(w.prover, r->n_log >= kHighPriorityLog);
    if (r->by_seed) rc = flock_prover_prove_seed(w.prover, r->n_log, r->seed, out);
    else rc = flock_prover_prove(w.prover, r->inputs.data(), r->inputs.size(), r->n_log, out, false);
    const size_t actual = flock_prover_reserved_bytes(w.prover);
    lk.lock();
    w.busy = false;
    w.reserved = std::max(fp, actual);
    r->proof.swap(out);
    r->inputs.clear();
    r->inputs.shrink_to_fit();
    r->t_done = now_ms();
    r->status = rc;
    cv_done.notify_all();
    cv_work.notify_all();
  }
}

namespace {

int submit(flock_server* s, std::shared_ptr<Request> r, uint64_t* id) {
  if (s->budget && flock_footprint_bytes((uint32_t)r->n_log) > s->budget) return FLOCK_ERR_OOM;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return FLOCK_ERR_ARG;
  r->id = s->next_id++;
  r->t_submit = now_ms();
  s->reqs[r->id] = r;
  s->queue.push_back(r);
  *id = r->id;
  s->cv_work.notify_one();
  return FLOCK_OK;
}

// Copies a finished request's proof out and forgets the request (caller holds mu).
int collect(flock_server* s, const std::shared_ptr<Request>& r, uint8_t* out, size_t cap, size_t* len) {
  if (r->status != FLOCK_OK) {
    int rc = r->status;
    s->reqs.erase(r->id);
    return rc;
  }
  *len = r->proof.size();
  if (!out || cap < r->proof.size()) return FLOCK_ERR_CAPACITY;
  std::memcpy(out, r->proof.data(), r->proof.size());
  s->reqs.erase(r->id);
  return FLOCK_OK;
}

}  // namespace

extern "C" {

size_t flock_footprint_bytes(uint32_t log2_size) {
  // Device bytes one prover state holds after a proof of 2^log2_size
  // compressions (m = 14 + log2_size): the witness planes and stripe
  // (4 x 2^m / 8), the rate-1/2 codeword (2^m / 4), the zerocheck tables
  // (2^m / 2 + 2^m / 4), the combined basis and first Ligerito fold (2^m / 4),
  // round 1's eq table and its per-block basis (9 x 16 B per 2^13 bits: 2^m / 57),
  // smaller per-level buffers, the inputs, and the fixed matrices and partials.
  const int n_log = log2_slots((size_t)1 << log2_size);
  const double two_m = (double)((uint64_t)1 << (14 + n_log));
  return (size_t)(1.87 * two_m) + ((size_t)128 << n_log) + ((size_t)320 << 20);
}

int flock_server_create(int device, size_t hbm_budget, int n_workers, flock_server** out) {
  if (!out || n_workers < 1 || n_workers > 64) return FLOCK_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return FLOCK_ERR_CUDA;
  flock_server* s = new (std::nothrow) flock_server;
  if (!s) return FLOCK_ERR_OOM;
  s->device = device;
  s->budget = hbm_budget;
  s->workers.resize(n_workers);
  for (Worker& w : s->workers) {
    w.prover = flock_prover_create(device);
    if (!w.prover) {
      for (Worker& v : s->workers) flock_prover_destroy(v.prover);
      delete s;
      return FLOCK_ERR_CUDA;
    }
  }
  for (int i = 0; i < n_workers; i++) s->workers[i].thread = std::thread([s, i] { s->run(i); });
  *out = s;
  return FLOCK_OK;
}

void flock_server_destroy(flock_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  for (Worker& w : s->workers)
    if (w.thread.joinable()) w.thread.join();
  for (Worker& w : s->workers) flock_prover_destroy(w.prover);
  delete s;
}

int flock_server_submit_seed(flock_server* s, uint32_t log2_size, uint64_t seed, uint64_t* id) {
  if (!s || !id || log2_size < 8 || log2_size > 21) return FLOCK_ERR_ARG;
  auto r = std::make_shared<Request>();
  r->n_log = (int)log2_size;
  r->seed = seed;
  return submit(s, r, id);
}

int flock_server_submit(flock_server* s, const flock_compression* in, size_t n, uint64_t* id) {
  if (!s || !id || (n && !in) || n > ((size_t)1 << 21)) return FLOCK_ERR_ARG;
  auto r = std::make_shared<Request>();
  r->n_log = log2_slots(n);
  if (r->n_log < 8) return FLOCK_ERR_SHAPE;
  r->by_seed = false;
  r->inputs.assign(in, in + n);
  return submit(s, r, id);
}

int flock_server_poll(flock_server* s, uint64_t id, uint8_t* out, size_t cap, size_t* len) {
  if (!s || !len) return FLOCK_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FLOCK_ERR_ARG;
  if (it->second->status == FLOCK_PENDING) return FLOCK_PENDING;
  return collect(s, it->second, out, cap, len);
}

int flock_server_wait(flock_server* s, uint64_t id, uint8_t* out, size_t cap, size_t* len) {
  if (!s || !len) return FLOCK_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FLOCK_ERR_ARG;
  std::shared_ptr<Request> r = it->second;
  s->cv_done.wait(lk, [&] { return r->status != FLOCK_PENDING; });
  return collect(s, r, out, cap, len);
}

int flock_server_request_times(flock_server* s, uint64_t id, double* queue_ms, double* run_ms) {
  if (!s) return FLOCK_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FLOCK_ERR_ARG;
  const Request& r = *it->second;
  if (r.status == FLOCK_PENDING) return FLOCK_PENDING;
  if (queue_ms) *queue_ms = r.t_start - r.t_submit;
  if (run_ms) *run_ms = r.t_done - r.t_start;
  return FLOCK_OK;
}

size_t flock_server_reserved_bytes(flock_server* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  return s->reserved_total();
}

int flock_prove_batch(flock_server* s, size_t count, const uint32_t* log2_sizes, const uint64_t* seeds, uint8_t* out,
                      size_t cap, size_t* lens) {
  if (!s || (count && (!log2_sizes || !seeds || !lens))) return FLOCK_ERR_ARG;
  // Largest first, so the big proofs start early and the small ones fill in.
  std::vector<size_t> order(count);
  for (size_t i = 0; i < count; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return log2_sizes[a] > log2_sizes[b]; });
  std::vector<uint64_t> ids(count, 0);
  int first_err = FLOCK_OK;
  for (size_t k = 0; k < count; k++) {
    size_t i = order[k];
    int rc = flock_server_submit_seed(s, log2_sizes[i], seeds[i], &ids[i]);
    if (rc != FLOCK_OK) {
      ids[i] = 0;
      if (first_err == FLOCK_OK) first_err = rc;
    }
  }
  size_t off = 0;
  for (size_t i = 0; i < count; i++) {
    lens[i] = 0;
    if (!ids[i]) continue;
    size_t len = 0;
    uint8_t* dst = out && off <= cap ? out + off : nullptr;
    int rc = flock_server_wait(s, ids[i], dst, dst ? cap - off : 0, &len);
    lens[i] = len;
    if (rc == FLOCK_OK) {
      off += len;
    } else {
      if (rc == FLOCK_ERR_CAPACITY) {  // no room: drop the finished proof
        std::lock_guard<std::mutex> lk(s->mu);
        s->reqs.erase(ids[i]);
      }
      if (first_err == FLOCK_OK) first_err = rc;
    }
  }
  return first_err;
}

}  // extern "C"
