// Serving loop: cell-simulation requests arrive at any time, are admitted as
// worker slots and device memory allow, and run concurrently on the GPU while
// others are running (continuous batching): either each on its own stream, or
// (lockstep) through one shared gw_batch whose stage launches a newcomer joins
// at the next round.
//
// Admission is by bytes of device state (FRU arrays, MT19937 rows and their
// snapshot copies).  The server holds at most `mem_budget_bytes` of cell
// contexts at any time, counting running cells and the idle contexts it keeps
// for reuse alike.  A request waits in arrival order until one of these
// holds: an idle context of its FRU count is pooled (no allocation); its
// cell fits in the budget beside every context held (one allocation); or
// freeing idle contexts of other sizes makes it fit (those are destroyed
// first).  Allocating or freeing device memory synchronises the device and
// so stalls the running requests: gw_server_reserve creates contexts up
// front, so that a workload of known sizes allocates nothing while it runs.
// Each request starts from the rest state with its own seeds, so its result
// is the same alone and in any mix.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "gw_ctx_impl.h"
#include "gw_fru.h"

extern "C" int gw_internal_error(int code, const char* msg);

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

extern "C" size_t gw_cell_bytes(int nfru) {
  const size_t s = (size_t)((nfru + 31) & ~31);
  const size_t nb = (size_t)((nfru + 7) / 8);
  // frus, chan, mti, their snapshots, MT rows and hold rows, hold epochs,
  // partial sums, scratch words
  return s * (5 * 8 + 4 * 4 + 4) * 2 + (size_t)nfru * 640 * 4 * 2 + s * 4 + nb * 16 * 8 + 512;
}

struct gw_server {
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<gw_request*> queue;
  std::vector<std::thread> workers;
  std::map<int, std::vector<gw_ctx*>> pool;  // idle contexts by FRU count
  gw_batch* batch = nullptr;
  int precision = 0;
  int lockstep = 0;  // 1: members share batched launches; 0: each cell on its own stream
  size_t budget = 0;
  size_t held = 0;        // bytes of every context the server holds (running and idle)
  size_t peak_held = 0;
  unsigned long long allocs = 0, frees = 0;
  int pending = 0;  // submitted and not finished
  bool stop = false;
  int device = 0;
};

static size_t idle_bytes_except(const gw_server* s, int nfru) {
  size_t b = 0;
  for (const auto& kv : s->pool)
    if (kv.first != nfru) b += kv.second.size() * gw_cell_bytes(kv.first);
  return b;
}

// Under the lock: can the request of nfru FRUs start now?  On success either
// *ctx is a pooled context, or *make is set (allocate one; the bytes are
// already counted) and `victims` holds idle contexts to destroy first.
static bool admit(gw_server* s, int nfru, gw_ctx** ctx, bool* make, std::vector<gw_ctx*>& victims) {
  auto& v = s->pool[nfru];
  if (!v.empty()) {
    *ctx = v.back();
    v.pop_back();
    return true;
  }
  const size_t need = gw_cell_bytes(nfru);
  if (s->held + need > s->budget) {
    if (s->held - idle_bytes_except(s, nfru) + need > s->budget) return false;
    // free idle contexts of other sizes, largest first, until the cell fits
    while (s->held + need > s->budget) {
      int big = -1;
      for (const auto& kv : s->pool)
        if (kv.first != nfru && !kv.second.empty() && kv.first > big) big = kv.first;
      gw_ctx* c = s->pool[big].back();
      s->pool[big].pop_back();
      s->held -= gw_cell_bytes(big);
      victims.push_back(c);
    }
  }
  s->held += need;
  if (s->held > s->peak_held) s->peak_held = s->held;
  *make = true;
  return true;
}

static gw_ctx* new_ctx(gw_server* s, int nfru, int* rc) {
  gw_ctx* c = nullptr;
  *rc = gw_create(&c, nfru);
  if (*rc) return nullptr;
  gw_set_precision(c, s->precision);
  return c;
}

static void run_request(gw_server* s, gw_request* r, gw_ctx* c, int rc) {
  r->t_start = now_s();
  if (c) {
    double state[37], t = 0.0, oldstep = r->set.step_max;
    const int steps = (int)(r->duration_ms / r->set.time_step + 0.5);
    rc = gw_set_pca_scale(c, r->pca_scale > 0.0 ? r->pca_scale : 1.0);
    if (!rc) rc = gw_init_rest(c, &r->set, r->seed_scheme, r->seed, state);
    if (!rc && s->lockstep) rc = gw_batch_add(s->batch, c);
    if (!rc) {
      double* states = r->v_trace ? new (std::nothrow) double[(size_t)steps * 37] : nullptr;
      rc = gw_run(c, &r->set, &t, state, &oldstep, steps, states, nullptr, nullptr);
      if (s->lockstep) gw_batch_remove(s->batch, c);
      if (states) {
        for (int k = 0; k < steps; k++) r->v_trace[k] = states[(size_t)k * 37];
        delete[] states;
      }
      if (!rc && r->final_state) memcpy(r->final_state, state, sizeof state);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->pool[r->nfru].push_back(c);  // stays held, idle, for the next request of its size
  }
  r->t_done = now_s();
  if (rc) snprintf(r->message, sizeof r->message, "%s", gw_last_error());  // per-thread message
  r->status = rc;
}

static void worker(gw_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    gw_request* r = nullptr;
    gw_ctx* ctx = nullptr;
    bool make = false;
    std::vector<gw_ctx*> victims;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // first come, first served: the head waits until its cell can be held
      s->cv_work.wait(lk, [&] {
        return s->stop || (!s->queue.empty() && admit(s, s->queue.front()->nfru, &ctx, &make, victims));
      });
      if (!ctx && !make) return;  // stopping with an empty queue
      r = s->queue.front();
      s->queue.pop_front();
      s->frees += victims.size();
      if (make) s->allocs++;
    }
    s->cv_work.notify_all();
    for (gw_ctx* v : victims) gw_destroy(v);
    int rc = 0;
    if (make) {
      ctx = new_ctx(s, r->nfru, &rc);
      if (!ctx) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->held -= gw_cell_bytes(r->nfru);
      }
    }
    run_request(s, r, ctx, rc);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->pending--;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
}

extern "C" int gw_server_create(gw_server** out, int precision, int slots, size_t mem_budget_bytes, int lockstep) {
  if (!out || slots <= 0 || (precision != 0 && precision != 1) || mem_budget_bytes == 0)
    return gw_internal_error(GW_EINVAL, "gw_server_create: bad argument");
  gw_server* s = new (std::nothrow) gw_server();
  if (!s) return gw_internal_error(GW_ENOMEM, "gw_server_create: host allocation failed");
  int rc = gw_batch_create(&s->batch, precision);
  if (rc) {
    delete s;
    return rc;
  }
  cudaGetDevice(&s->device);
  s->precision = precision;
  s->lockstep = lockstep ? 1 : 0;
  s->budget = mem_budget_bytes;
  for (int i = 0; i < slots; i++) s->workers.emplace_back(worker, s);
  *out = s;
  return GW_OK;
}

extern "C" int gw_server_reserve(gw_server* s, int nfru, int count) {
  if (!s || nfru <= 0 || count < 0) return gw_internal_error(GW_EINVAL, "gw_server_reserve: bad argument");
  for (int i = 0; i < count; i++) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->held + gw_cell_bytes(nfru) > s->budget)
        return gw_internal_error(GW_EINVAL, "gw_server_reserve: the contexts exceed the memory budget");
      s->held += gw_cell_bytes(nfru);
      if (s->held > s->peak_held) s->peak_held = s->held;
      s->allocs++;
    }
    int rc = 0;
    gw_ctx* c = new_ctx(s, nfru, &rc);
    std::lock_guard<std::mutex> lk(s->mu);
    if (!c) {
      s->held -= gw_cell_bytes(nfru);
      return rc;
    }
    s->pool[nfru].push_back(c);
  }
  s->cv_work.notify_all();
  return GW_OK;
}

extern "C" int gw_server_stats(gw_server* s, size_t* held, size_t* peak_held, unsigned long long* allocs,
                               unsigned long long* frees) {
  if (!s) return gw_internal_error(GW_EINVAL, "gw_server_stats: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  if (held) *held = s->held;
  if (peak_held) *peak_held = s->peak_held;
  if (allocs) *allocs = s->allocs;
  if (frees) *frees = s->frees;
  return GW_OK;
}

extern "C" int gw_server_submit(gw_server* s, gw_request* r) {
  if (!s || !r || r->nfru <= 0 || r->duration_ms <= 0.0)
    return gw_internal_error(GW_EINVAL, "gw_server_submit: bad request");
  if (gw_cell_bytes(r->nfru) > s->budget)
    return gw_internal_error(GW_EINVAL, "gw_server_submit: the cell alone exceeds the memory budget");
  r->t_submit = now_s();
  r->t_start = r->t_done = 0.0;
  r->status = -1;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->queue.push_back(r);
    s->pending++;
  }
  s->cv_work.notify_all();
  return GW_OK;
}

extern "C" int gw_server_wait(gw_server* s) {
  if (!s) return gw_internal_error(GW_EINVAL, "gw_server_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->pending == 0; });
  return GW_OK;
}

extern "C" int gw_server_destroy(gw_server* s) {
  if (!s) return GW_OK;
  gw_server_wait(s);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& w : s->workers) w.join();
  for (auto& kv : s->pool)
    for (gw_ctx* c : kv.second) gw_destroy(c);
  gw_batch_destroy(s->batch);
  delete s;
  return GW_OK;
}
