// Many cells, one launch per stage round.
//
// Each member cell keeps its own host-side Dormand-Prince driver (one host
// thread per cell, gw_rk54pd / gw_run unchanged).  When a member asks for a
// stage or flux operation, the request is posted to the batch; once every
// member has posted, one launch of the batched stage kernel advances all of
// them (each with its own interval, voltages, flags and snapshot epoch) and
// every waiting cell resumes with its own fluxes.  One cell's FRUs occupy the
// GPU only while their slowest FRU finishes; a batch keeps all SM
// sub-partitions busy with many cells' FRUs and hides those tails.
//
// Each cell's arithmetic and reduction order is exactly its single-cell one,
// so a cell's results are the same alone and in any batch.  Cells may join
// and leave between rounds (continuous batching).
#include <cuda_runtime.h>
#include <stdio.h>

#include <condition_variable>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "gw_ctx_impl.h"
#include "gw_fru.h"
#include "gw_kernels.h"

extern "C" int gw_internal_error(int code, const char* msg);

struct gw_batch {
  std::mutex mu;
  std::condition_variable cv;
  int precision = 0;
  cudaStream_t stream = nullptr;
  std::vector<gw_ctx*> members;
  std::vector<gw::StageParams> ops;
  std::vector<char> posted;
  int nposted = 0;
  unsigned long long round = 0;
  bool dirty = true;
  int nblocks = 0;
  int warps = 1;  // warps per block of the batched launches
  int cap = 0;  // capacity of the device/pinned arrays (cells)
  gw::DevState* d_cells = nullptr;
  gw::StageParams* d_params = nullptr;
  int* d_block0 = nullptr;
  double* d_outs = nullptr;
  gw::StageParams* h_params = nullptr;
  double* h_outs = nullptr;
  int* h_block0 = nullptr;
  gw::DevState* h_cells = nullptr;
  cudaEvent_t ev[2] = {};
  bool profiling = false;
  double kernel_ms = 0.0;
  unsigned long long launches = 0;
  int error = 0;  // sticky CUDA failure of a round
};

static void free_arrays(gw_batch* b) {
  if (b->d_cells) cudaFree(b->d_cells);
  if (b->d_params) cudaFree(b->d_params);
  if (b->d_block0) cudaFree(b->d_block0);
  if (b->d_outs) cudaFree(b->d_outs);
  if (b->h_params) cudaFreeHost(b->h_params);
  if (b->h_outs) cudaFreeHost(b->h_outs);
  if (b->h_block0) cudaFreeHost(b->h_block0);
  if (b->h_cells) cudaFreeHost(b->h_cells);
  b->d_cells = nullptr;
  b->d_params = nullptr;
  b->d_block0 = nullptr;
  b->d_outs = nullptr;
  b->h_params = nullptr;
  b->h_outs = nullptr;
  b->h_block0 = nullptr;
  b->h_cells = nullptr;
}

static cudaError_t ensure_capacity(gw_batch* b, int n) {
  if (n <= b->cap) return cudaSuccess;
  const int cap = n < 64 ? 64 : 2 * n;
  cudaStreamSynchronize(b->stream);
  free_arrays(b);
  cudaError_t e = cudaMalloc(&b->d_cells, sizeof(gw::DevState) * cap);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_params, sizeof(gw::StageParams) * cap);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_block0, sizeof(int) * (cap + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_outs, sizeof(double) * gw::kBatchOutStride * cap);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_params, sizeof(gw::StageParams) * cap);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_outs, sizeof(double) * gw::kBatchOutStride * cap);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_block0, sizeof(int) * (cap + 1));
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_cells, sizeof(gw::DevState) * cap);
  if (e == cudaSuccess) e = cudaMemset(b->d_outs, 0, sizeof(double) * gw::kBatchOutStride * cap);
  if (e != cudaSuccess) {
    free_arrays(b);
    b->cap = 0;
    return e;
  }
  b->cap = cap;
  return cudaSuccess;
}

// Run one round: every member has posted.  Called with the mutex held.
static cudaError_t launch_round(gw_batch* b) {
  const int n = (int)b->members.size();
  cudaError_t e = cudaSuccess;
  if (b->dirty) {
    e = ensure_capacity(b, n);
    if (e != cudaSuccess) return e;
    int acc = 0;
    for (int i = 0; i < n; i++) {
      b->h_cells[i] = b->members[i]->d;
      b->h_block0[i] = acc;
      acc += gw::stage_blocks(b->members[i]->d.nfru, b->warps);
    }
    b->h_block0[n] = acc;
    b->nblocks = acc;
    e = cudaMemcpyAsync(b->d_cells, b->h_cells, sizeof(gw::DevState) * n, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->d_block0, b->h_block0, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return e;
    b->dirty = false;
  }
  for (int i = 0; i < n; i++) b->h_params[i] = b->ops[i];
  e = cudaMemcpyAsync(b->d_params, b->h_params, sizeof(gw::StageParams) * n, cudaMemcpyHostToDevice, b->stream);
  if (e != cudaSuccess) return e;
  gw::BatchArgs a;
  a.cells = b->d_cells;
  a.params = b->d_params;
  a.block0 = b->d_block0;
  a.outs = b->d_outs;
  a.ncells = n;
  if (b->profiling) cudaEventRecord(b->ev[0], b->stream);
  e = (b->precision == 1) ? gw::launch_stage_mixed_batch(a, b->nblocks, b->warps, b->stream)
                          : gw::launch_stage4_batch(a, b->nblocks, b->warps, b->stream);
  if (e != cudaSuccess) return e;
  b->launches++;
  if (b->profiling) cudaEventRecord(b->ev[1], b->stream);
  e = cudaMemcpyAsync(b->h_outs, b->d_outs, sizeof(double) * gw::kBatchOutStride * n, cudaMemcpyDeviceToHost,
                      b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e == cudaSuccess && b->profiling) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
    b->kernel_ms += ms;
  }
  return e;
}

static void finish_round(gw_batch* b) {
  cudaError_t e = launch_round(b);
  if (e != cudaSuccess) b->error = (int)e;
  // hand every member its outputs now: slots are renumbered when a member
  // leaves, so a waiter must not look its outputs up by index later
  for (size_t i = 0; i < b->members.size(); i++)
    for (int k = 0; k < gw::kBatchOutStride; k++)
      b->members[i]->batch_out[k] = b->h_outs[gw::kBatchOutStride * i + k];
  b->round++;
  b->nposted = 0;
  for (auto& x : b->posted) x = 0;
  b->cv.notify_all();
}

int gw_batch_post(gw_ctx* c, const gw::StageParams& p, double* out) {
  gw_batch* b = c->batch;
  std::unique_lock<std::mutex> lk(b->mu);
  const int slot = c->slot;
  b->ops[slot] = p;
  b->posted[slot] = 1;
  b->nposted++;
  const unsigned long long my_round = b->round;
  if (b->nposted == (int)b->members.size()) finish_round(b);
  else b->cv.wait(lk, [&] { return b->round != my_round; });
  if (b->error)
    return gw_internal_error(GW_ECUDA, "batched FRU stage launch failed");
  for (int k = 0; k < gw::kBatchOutStride; k++) out[k] = c->batch_out[k];
  c->launches++;
  return GW_OK;
}

extern "C" int gw_batch_create(gw_batch** out, int precision) {
  if (!out || (precision != 0 && precision != 1)) return gw_internal_error(GW_EINVAL, "gw_batch_create: bad argument");
  gw_batch* b = new (std::nothrow) gw_batch();
  if (!b) return gw_internal_error(GW_ENOMEM, "gw_batch_create: host allocation failed");
  b->precision = precision;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess ||
      ensure_capacity(b, 64) != cudaSuccess) {
    delete b;
    return gw_internal_error(GW_ECUDA, "gw_batch_create: CUDA setup failed");
  }
  *out = b;
  return GW_OK;
}

extern "C" int gw_batch_destroy(gw_batch* b) {
  if (!b) return GW_OK;
  {
    std::lock_guard<std::mutex> lk(b->mu);
    for (gw_ctx* c : b->members) {
      c->batch = nullptr;
      c->slot = -1;
    }
    b->members.clear();
  }
  cudaStreamSynchronize(b->stream);
  free_arrays(b);
  cudaEventDestroy(b->ev[0]);
  cudaEventDestroy(b->ev[1]);
  cudaStreamDestroy(b->stream);
  delete b;
  return GW_OK;
}

extern "C" int gw_batch_set_warps(gw_batch* b, int warps) {
  if (!b || warps < 1 || warps > gw::kMaxStageWarps || (warps & (warps - 1)))
    return gw_internal_error(GW_EINVAL, "gw_batch_set_warps: warps per block must be 1, 2, 4 or 8");
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->warps != warps) {
    b->warps = warps;
    b->dirty = true;  // block prefix sums change
  }
  return GW_OK;
}

extern "C" int gw_batch_add(gw_batch* b, gw_ctx* c) {
  if (!b || !c || c->batch) return gw_internal_error(GW_EINVAL, "gw_batch_add: bad cell or cell already batched");
  if (c->fru_lanes != 4 || c->precision != b->precision)
    return gw_internal_error(GW_EINVAL, "gw_batch_add: cell precision / kernel differs from the batch's");
  if (c->sum_order != GW_SUM_TREE)
    return gw_internal_error(GW_EINVAL, "gw_batch_add: reference-order sums are a single-cell mode");
  std::lock_guard<std::mutex> lk(b->mu);
  cudaStreamSynchronize(c->stream);  // the cell's own pending work lands first
  c->batch = b;
  c->slot = (int)b->members.size();
  b->members.push_back(c);
  b->ops.push_back(gw::StageParams{});
  b->posted.push_back(0);
  b->dirty = true;
  return GW_OK;
}

extern "C" int gw_batch_remove(gw_batch* b, gw_ctx* c) {
  if (!b || !c || c->batch != b) return gw_internal_error(GW_EINVAL, "gw_batch_remove: cell is not in this batch");
  std::lock_guard<std::mutex> lk(b->mu);
  const int s = c->slot;
  if (b->posted[s]) b->nposted--;
  b->members.erase(b->members.begin() + s);
  b->ops.erase(b->ops.begin() + s);
  b->posted.erase(b->posted.begin() + s);
  for (int i = s; i < (int)b->members.size(); i++) b->members[i]->slot = i;
  c->batch = nullptr;
  c->slot = -1;
  b->dirty = true;
  // the cells still waiting may now all have posted
  if (!b->members.empty() && b->nposted == (int)b->members.size()) finish_round(b);
  return GW_OK;
}

extern "C" int gw_batch_profile(gw_batch* b, int enable, double* kernel_ms, unsigned long long* launches) {
  if (!b) return gw_internal_error(GW_EINVAL, "gw_batch_profile: null batch");
  std::lock_guard<std::mutex> lk(b->mu);
  if (kernel_ms) *kernel_ms = b->kernel_ms;
  if (launches) *launches = b->launches;
  b->profiling = enable != 0;
  if (enable) {
    b->kernel_ms = 0.0;
    b->launches = 0;
  }
  return GW_OK;
}

// Run n cells concurrently through the batch: one host thread per cell runs
// the caf.c main loop (gw_run) for n_steps output steps; optional traces
// [n][n_steps][37] and [n][n_steps][12] receive each step's states and
// otherstates.
extern "C" int gw_batch_run(gw_batch* b, int n, gw_ctx** cells, const gw_settings* sets, double* t, double* states,
                            double* oldsteps, int n_steps, double* state_trace, double* other_trace) {
  if (!b || n <= 0 || !cells || !sets || !t || !states || !oldsteps)
    return gw_internal_error(GW_EINVAL, "gw_batch_run: bad argument");
  for (int i = 0; i < n; i++) {
    int rc = gw_batch_add(b, cells[i]);
    if (rc) {
      for (int j = 0; j < i; j++) gw_batch_remove(b, cells[j]);
      return rc;
    }
  }
  std::vector<int> rcs(n, 0);
  std::vector<std::string> msgs(n);
  std::vector<std::thread> th;
  th.reserve(n);
  int dev = 0;
  cudaGetDevice(&dev);
  for (int i = 0; i < n; i++)
    th.emplace_back([&, i] {
      cudaSetDevice(dev);
      rcs[i] = gw_run(cells[i], &sets[i], &t[i], states + (size_t)i * 37, &oldsteps[i], n_steps,
                      state_trace ? state_trace + (size_t)i * n_steps * 37 : nullptr,
                      other_trace ? other_trace + (size_t)i * n_steps * 12 : nullptr, nullptr);
      if (rcs[i]) msgs[i] = gw_last_error();  // the message is per thread
      gw_batch_remove(b, cells[i]);
    });
  for (auto& x : th) x.join();
  for (int i = 0; i < n; i++)
    if (rcs[i]) {
      const std::string m = "gw_batch_run: cell " + std::to_string(i) + ": " + msgs[i];
      gw_internal_error(rcs[i], m.c_str());
      return rcs[i];
    }
  return GW_OK;
}

// The same concurrency without shared rounds: every cell launches its own
// stage kernels on its own stream from its own host thread, so a cell whose
// slowest FRU is still running does not hold back the others; the GPU runs
// the cells' kernels concurrently.
extern "C" int gw_run_concurrent(int n, gw_ctx** cells, const gw_settings* sets, double* t, double* states,
                                 double* oldsteps, int n_steps, double* state_trace, double* other_trace) {
  if (n <= 0 || !cells || !sets || !t || !states || !oldsteps)
    return gw_internal_error(GW_EINVAL, "gw_run_concurrent: bad argument");
  std::vector<int> rcs(n, 0);
  std::vector<std::string> msgs(n);
  std::vector<std::thread> th;
  th.reserve(n);
  int dev = 0;
  cudaGetDevice(&dev);
  for (int i = 0; i < n; i++)
    th.emplace_back([&, i] {
      cudaSetDevice(dev);
      rcs[i] = gw_run(cells[i], &sets[i], &t[i], states + (size_t)i * 37, &oldsteps[i], n_steps,
                      state_trace ? state_trace + (size_t)i * n_steps * 37 : nullptr,
                      other_trace ? other_trace + (size_t)i * n_steps * 12 : nullptr, nullptr);
      if (rcs[i]) msgs[i] = gw_last_error();  // the message is per thread
    });
  for (auto& x : th) x.join();
  for (int i = 0; i < n; i++)
    if (rcs[i]) {
      const std::string m = "gw_run_concurrent: cell " + std::to_string(i) + ": " + msgs[i];
      gw_internal_error(rcs[i], m.c_str());
      return rcs[i];
    }
  return GW_OK;
}
