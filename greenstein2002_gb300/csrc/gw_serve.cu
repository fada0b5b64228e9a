// Serving loop: cell-simulation requests arrive at any time, are admitted as
// worker slots and device memory allow, and run concurrently on the GPU while
// others are running (continuous batching): either each on its own stream, or
// (lockstep) through one shared gw_batch whose stage launches a newcomer joins
// at the next round.
//
// Admission is by bytes of device state (FRU arrays, MT19937 rows and their
// snapshot copies): a request waits in arrival order until its cell fits in
// the budget next to the running ones.  Device contexts are pooled per FRU
// count and reused, so no allocation or free (which would synchronise the
// device) happens while other requests are running, once a size has been
// seen.  Each request starts from the rest state with its own seeds, so its
// result is the same alone and in any mix.
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
  std::vector<gw_ctx*> all;
  gw_batch* batch = nullptr;
  int precision = 0;
  int lockstep = 0;  // 1: members share batched launches; 0: each cell on its own stream
  size_t budget = 0, in_use = 0;
  int pending = 0;  // submitted and not finished
  bool stop = false;
  int device = 0;
};

static gw_ctx* take_ctx(gw_server* s, int nfru, int* rc) {
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto& v = s->pool[nfru];
    if (!v.empty()) {
      gw_ctx* c = v.back();
      v.pop_back();
      return c;
    }
  }
  gw_ctx* c = nullptr;
  *rc = gw_create(&c, nfru);
  if (*rc) return nullptr;
  gw_set_precision(c, s->precision);
  std::lock_guard<std::mutex> lk(s->mu);
  s->all.push_back(c);
  return c;
}

static void run_request(gw_server* s, gw_request* r) {
  int rc = 0;
  gw_ctx* c = take_ctx(s, r->nfru, &rc);
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
    s->pool[r->nfru].push_back(c);
  }
  r->t_done = now_s();
  if (rc) snprintf(r->message, sizeof r->message, "%s", gw_last_error());  // per-thread message
  r->status = rc;
}

static void worker(gw_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    gw_request* r = nullptr;
    size_t need = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // first come, first served: the head waits until its cell fits
      s->cv_work.wait(lk, [&] {
        return s->stop || (!s->queue.empty() && s->in_use + gw_cell_bytes(s->queue.front()->nfru) <= s->budget);
      });
      if (s->stop && s->queue.empty()) return;
      if (s->queue.empty()) continue;
      r = s->queue.front();
      s->queue.pop_front();
      need = gw_cell_bytes(r->nfru);
      s->in_use += need;
    }
    s->cv_work.notify_all();
    run_request(s, r);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->in_use -= need;
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
  for (gw_ctx* c : s->all) gw_destroy(c);
  gw_batch_destroy(s->batch);
  delete s;
  return GW_OK;
}
