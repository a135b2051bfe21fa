// Serving batch: independent HemoCell solves resident on one device and
// stepped together (continuous batching).
//
// Each admitted solve keeps its own handle, and so its own lattice, meshes and
// non-blocking stream.  hc_batch_pump keeps every solve's stream fed with up to
// kDepth chunks of steps (each chunk replays the handle's step graph), so the
// kernels of all resident solves overlap on the device; a solve that finishes
// leaves at once, without waiting for the others, and its memory goes back to
// the budget when the caller releases it.  Admission is by device memory: a
// solve is admitted only while the bytes of the resident solves stay within
// the batch's budget and a slot is free.
//
// There is no counterpart in the reference, which runs one simulation per MPI
// job; each solve here runs exactly the steps hc_step would run on its own.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hemocell_gb300.h"
#include "hc_dev.h"

namespace {

constexpr int kDepth = 2;  // chunks in flight per solve

struct Solve {
  hc_handle* h = nullptr;
  long long tag = 0;
  long long bytes = 0;
  int total = 0;     // steps requested
  int enqueued = 0;  // steps handed to the stream
  int rc = HC_OK;    // first failure of this solve
  std::deque<cudaEvent_t> inflight;
};

}  // namespace

struct hc_batch {
  int device = 0;
  long long budget = 0;
  long long in_use = 0;  // bytes of admitted, finished and popped solves not yet released
  int max_slots = 0;
  int chunk = 0;
  std::vector<Solve> active;
  std::deque<Solve> finished;  // done, waiting for hc_batch_pop
  std::vector<Solve> popped;   // handed to the caller, waiting for hc_batch_release
  std::vector<cudaEvent_t> spare_events;
  std::string err;
  long long admitted = 0, completed = 0, refused = 0, steps_enqueued = 0;
};

namespace {

int batch_fail(hc_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

cudaError_t take_event(hc_batch* b, cudaEvent_t* ev) {
  if (!b->spare_events.empty()) {
    *ev = b->spare_events.back();
    b->spare_events.pop_back();
    return cudaSuccess;
  }
  return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
}

// Hand the stream of one solve up to kDepth chunks.  Returns the solve's status.
int feed(hc_batch* b, Solve& s) {
  while (s.rc == HC_OK && (int)s.inflight.size() < kDepth && s.enqueued < s.total) {
    const int n = std::min(b->chunk, s.total - s.enqueued);
    int rc = hc_step(s.h, n);
    if (rc != HC_OK) {
      s.rc = rc;
      break;
    }
    cudaEvent_t ev;
    cudaError_t e = take_event(b, &ev);
    if (e == cudaSuccess) e = cudaEventRecord(ev, hcd::handle_stream(s.h));
    if (e != cudaSuccess) {
      s.rc = HC_ERR_CUDA;
      b->err = std::string("event: ") + cudaGetErrorString(e);
      break;
    }
    s.inflight.push_back(ev);
    s.enqueued += n;
    b->steps_enqueued += n;
  }
  return s.rc;
}

// Retire the chunks that have completed; true when the solve is done.
bool retire(hc_batch* b, Solve& s) {
  while (!s.inflight.empty()) {
    cudaError_t e = cudaEventQuery(s.inflight.front());
    if (e == cudaErrorNotReady) break;
    if (e != cudaSuccess && s.rc == HC_OK) {
      s.rc = HC_ERR_CUDA;
      b->err = std::string("chunk: ") + cudaGetErrorString(e);
    }
    b->spare_events.push_back(s.inflight.front());
    s.inflight.pop_front();
  }
  if (s.rc != HC_OK) {
    // a failed solve leaves once its stream has nothing left in flight
    if (!s.inflight.empty()) return false;
    return true;
  }
  return s.enqueued >= s.total && s.inflight.empty();
}

void drop(hc_batch* b, Solve& s) {
  if (s.h) cudaStreamSynchronize(hcd::handle_stream(s.h));
  for (cudaEvent_t ev : s.inflight) b->spare_events.push_back(ev);
  s.inflight.clear();
  if (s.h) hc_destroy(s.h);
  s.h = nullptr;
}

}  // namespace

extern "C" {

hc_batch* hc_batch_create(int device, long long budget_bytes, int max_slots, int chunk_steps) {
  if (budget_bytes <= 0 || max_slots <= 0 || chunk_steps <= 0) {
    hcd::set_handleless_error("hc_batch_create: budget, slots and chunk must be positive");
    return nullptr;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || device < 0 || device >= ndev) {
    hcd::set_handleless_error("hc_batch_create: no such device");
    return nullptr;
  }
  hc_batch* b = new hc_batch();
  b->device = device;
  b->budget = budget_bytes;
  b->max_slots = max_slots;
  b->chunk = chunk_steps;
  return b;
}

int hc_batch_destroy(hc_batch* b) {
  if (!b) return HC_OK;
  cudaSetDevice(b->device);
  for (Solve& s : b->active) drop(b, s);
  for (Solve& s : b->finished) drop(b, s);
  for (Solve& s : b->popped) drop(b, s);
  for (cudaEvent_t ev : b->spare_events) cudaEventDestroy(ev);
  delete b;
  return HC_OK;
}

const char* hc_batch_last_error(const hc_batch* b) { return b ? b->err.c_str() : ""; }

int hc_batch_fits(const hc_batch* b, long long bytes) {
  if (!b || bytes < 0) return HC_ERR_INVALID;
  return ((int)b->active.size() < b->max_slots && b->in_use + bytes <= b->budget) ? 1 : 0;
}

int hc_batch_admit(hc_batch* b, hc_handle* h, int nsteps, long long tag) {
  if (!b || !h || nsteps < 0) return HC_ERR_INVALID;
  if (hcd::handle_device(h) != b->device) return batch_fail(b, HC_ERR_INVALID, "handle is on another device");
  const long long bytes = hcd::handle_bytes(h);
  if (hc_batch_fits(b, bytes) != 1) {
    b->refused++;
    return batch_fail(b, HC_ERR_MEMORY, "solve does not fit: " + std::to_string(bytes) + " bytes, " +
                                            std::to_string(b->budget - b->in_use) + " free of the budget, " +
                                            std::to_string(b->max_slots - (int)b->active.size()) + " slots free");
  }
  Solve s;
  s.h = h;
  s.tag = tag;
  s.bytes = bytes;
  s.total = nsteps;
  b->in_use += bytes;
  b->admitted++;
  b->active.push_back(std::move(s));
  return HC_OK;
}

int hc_batch_pump(hc_batch* b, double wait_ms) {
  if (!b) return HC_ERR_INVALID;
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return batch_fail(b, HC_ERR_CUDA, cudaGetErrorString(e));
  const auto t0 = std::chrono::steady_clock::now();
  int done = 0;
  for (;;) {
    for (Solve& s : b->active) feed(b, s);
    for (size_t i = 0; i < b->active.size();) {
      if (retire(b, b->active[i])) {
        b->finished.push_back(std::move(b->active[i]));
        b->active.erase(b->active.begin() + (long)i);
        b->completed++;
        done++;
      } else {
        ++i;
      }
    }
    // a chunk that just retired leaves room for the next one
    for (Solve& s : b->active) feed(b, s);
    if (done > 0 || b->active.empty()) break;
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (ms >= wait_ms) break;
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  return done;
}

int hc_batch_pop(hc_batch* b, long long* tag, hc_handle** h, int* status) {
  if (!b || !h) return HC_ERR_INVALID;
  if (b->finished.empty()) return 0;
  Solve s = std::move(b->finished.front());
  b->finished.pop_front();
  if (tag) *tag = s.tag;
  if (status) *status = s.rc;
  *h = s.h;
  b->popped.push_back(std::move(s));
  return 1;
}

int hc_batch_release(hc_batch* b, hc_handle* h, int destroy) {
  if (!b || !h) return HC_ERR_INVALID;
  for (size_t i = 0; i < b->popped.size(); ++i) {
    if (b->popped[i].h != h) continue;
    b->in_use -= b->popped[i].bytes;
    if (destroy) hc_destroy(h);
    b->popped.erase(b->popped.begin() + (long)i);
    return HC_OK;
  }
  return batch_fail(b, HC_ERR_INVALID, "handle was not popped from this batch");
}

int hc_batch_get_stats(const hc_batch* b, hc_batch_stats* out) {
  if (!b || !out) return HC_ERR_INVALID;
  out->active = (int)b->active.size();
  out->finished = (int)b->finished.size();
  out->popped = (int)b->popped.size();
  out->max_slots = b->max_slots;
  out->budget_bytes = b->budget;
  out->bytes_in_use = b->in_use;
  out->admitted = b->admitted;
  out->completed = b->completed;
  out->refused = b->refused;
  out->steps_enqueued = b->steps_enqueued;
  return HC_OK;
}

}  // extern "C"
