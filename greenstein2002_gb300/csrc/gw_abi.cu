// Native C-ABI of the FRU hot path: device memory of one cell, uploads and
// downloads in the reference's array layout, and the stage / flux / average
// / save / resume operations that replace the MPI layer of mpi_master.c.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>
#include <vector>

#include "gw_diag.h"
#include "gw_fru.h"
#include "gw_kernels.h"
#include "gw_fru_model.cuh"
#include "gw_ctx_impl.h"

using gw::DevState;
using gw::StageParams;

static thread_local char g_err[512];

static int set_err(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return set_err(GW_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                          __FILE__, __LINE__);                                  \
  } while (0)

static cudaError_t launch_stage_variant(gw_ctx* c, const StageParams& p0) {
  StageParams p = p0;
  p.launch = c->pack_launch;
  if (c->packed_warps > 0 && c->fru_lanes == 4 && (p.flags & gw::kFlagAdvance)) {
    // packed: advance from the queue, then the sums over the stored states
    cudaError_t e = (c->precision == 1) ? gw::launch_stage_mixed_packed(c->d, p, c->packed_warps, c->stream)
                                        : gw::launch_stage4_packed(c->d, p, c->packed_warps, c->stream);
    if (e != cudaSuccess) return e;
    p.flags = gw::kFlagQueueReset;
    c->pack_launch++;
    c->launches++;
  }
  if (c->precision == 1) return gw::launch_stage_mixed(c->d, p, c->stage_warps, c->stream);
  return c->fru_lanes == 4 ? gw::launch_stage4(c->d, p, c->stage_warps, c->stream)
                           : gw::launch_stage(c->d, p, c->stream);
}

extern "C" const char* gw_last_error(void) { return g_err; }

// error reporting for entry points defined in other translation units
extern "C" int gw_internal_error(int code, const char* msg) { return set_err(code, "%s", msg); }

extern "C" int gw_nfru(const gw_ctx* c) { return c ? c->d.nfru : 0; }

static void free_dev(gw_ctx* c) {
  void* ptrs[] = {c->d.frus, c->d.chan, c->d.mti, c->d.mt, c->d.frus_s, c->d.chan_s, c->d.mti_s,
                  c->d.mt_hold, c->d.hold_epoch, c->d.partials, c->d.ticket, c->d.out, c->d.substeps,
                  c->d.trace_sub, c->d.trace_ns, c->d.qctl, c->d.heavy_list, c->d.heavy_tag};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->flush_buf) cudaFree(c->flush_buf);
  for (cudaEvent_t e : c->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->pev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
}

extern "C" int gw_create(gw_ctx** out, int nfru) {
  if (!out || nfru <= 0) return set_err(GW_EINVAL, "gw_create: nfru must be > 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return set_err(GW_ENODEV, "gw_create: no CUDA device available");
  gw_ctx* c = new (std::nothrow) gw_ctx();
  if (!c) return set_err(GW_ENOMEM, "gw_create: host allocation failed");
  cudaGetDevice(&c->device);
  DevState& d = c->d;
  d.nfru = nfru;
  d.stride = (nfru + 31) & ~31;
  d.nblocks = (nfru + gw::kStageThreads - 1) / gw::kStageThreads;
  const size_t nf = (size_t)d.stride;
  cudaError_t e = cudaSuccess;
#define AL(ptr, bytes) \
  if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
  AL(d.frus, 5 * nf * sizeof(double));
  AL(d.chan, 4 * nf * sizeof(uint32_t));
  AL(d.mti, nf * sizeof(int));
  AL(d.mt, nf * gw::kMtStride * sizeof(uint32_t));
  AL(d.frus_s, 5 * nf * sizeof(double));
  AL(d.chan_s, 4 * nf * sizeof(uint32_t));
  AL(d.mti_s, nf * sizeof(int));
  AL(d.mt_hold, nf * gw::kMtStride * sizeof(uint32_t));
  AL(d.hold_epoch, nf * sizeof(uint32_t));
  // partial sums of the widest grid: 8-FRU blocks of the cleft-parallel kernel
  AL(d.partials, (size_t)((nfru + 7) / 8) * 16 * sizeof(double));
  AL(d.ticket, sizeof(unsigned));
  AL(d.out, 32 * sizeof(double));
  AL(d.substeps, sizeof(unsigned long long));
  AL(d.qctl, 8 * sizeof(unsigned));
  AL(d.heavy_list, 2 * nf * sizeof(int));
  AL(d.heavy_tag, 2 * nf * sizeof(uint32_t));
#undef AL
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_out, 32 * sizeof(double));
  for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventCreate(&c->pev[i]);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.ticket, 0, sizeof(unsigned), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.out, 0, 32 * sizeof(double), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.substeps, 0, sizeof(unsigned long long), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.hold_epoch, 0xff, nf * sizeof(uint32_t), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.qctl, 0, 8 * sizeof(unsigned), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.heavy_tag, 0, 2 * nf * sizeof(uint32_t), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.frus, 0, 5 * nf * sizeof(double), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.chan, 0, 4 * nf * sizeof(uint32_t), c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? GW_ENOMEM : GW_ECUDA;
    set_err(code, "gw_create(%d): %s", nfru, cudaGetErrorString(e));
    free_dev(c);
    delete c;
    return code;
  }
  c->nfru_scale = 12500.0 / (double)nfru;
  *out = c;
  return GW_OK;
}

extern "C" int gw_destroy(gw_ctx* c) {
  if (!c) return GW_OK;
  cudaStreamSynchronize(c->stream);
  free_dev(c);
  delete c;
  return GW_OK;
}

extern "C" int gw_set_scale(gw_ctx* c, double nfru_scale) {
  if (!c) return set_err(GW_EINVAL, "gw_set_scale: null context");
  c->nfru_scale = nfru_scale;
  return GW_OK;
}

extern "C" int gw_set_fru_lanes(gw_ctx* c, int lanes) {
  if (!c || (lanes != 1 && lanes != 4)) return set_err(GW_EINVAL, "gw_set_fru_lanes: lanes must be 1 or 4");
  if (lanes == 1 && (c->precision != 0 || c->pca_scale != 1.0))
    return set_err(GW_EINVAL, "gw_set_fru_lanes: the one-thread-per-FRU kernel is FP64 with the reference PCa only");
  c->fru_lanes = lanes;
  return GW_OK;
}

extern "C" int gw_set_stage_warps(gw_ctx* c, int warps) {
  if (!c || warps < 1 || warps > gw::kMaxStageWarps || (warps & (warps - 1)))
    return set_err(GW_EINVAL, "gw_set_stage_warps: warps per block must be 1, 2, 4 or 8");
  c->stage_warps = warps;
  return GW_OK;
}

extern "C" int gw_set_stage_packing(gw_ctx* c, int warps) {
  if (!c || warps < 0) return set_err(GW_EINVAL, "gw_set_stage_packing: warps must be >= 0");
  const int groups = (c->d.nfru + 7) / 8;
  c->packed_warps = warps > groups ? groups : warps;
  return GW_OK;
}

extern "C" int gw_set_precision(gw_ctx* c, int precision) {
  if (!c || (precision != 0 && precision != 1)) return set_err(GW_EINVAL, "gw_set_precision: 0 (FP64) or 1 (mixed)");
  if (precision == 1 && c->fru_lanes == 1) c->fru_lanes = 4;
  c->precision = precision;
  return GW_OK;
}

extern "C" int gw_set_pca_scale(gw_ctx* c, double scale) {
  if (!c || !(scale > 0.0)) return set_err(GW_EINVAL, "gw_set_pca_scale: scale must be > 0");
  if (scale != 1.0 && c->fru_lanes == 1) c->fru_lanes = 4;
  c->pca_scale = scale;
  return GW_OK;
}

extern "C" int gw_set_sum_order(gw_ctx* c, int order) {
  if (!c || (order != GW_SUM_TREE && order != GW_SUM_REFERENCE))
    return set_err(GW_EINVAL, "gw_set_sum_order: order must be GW_SUM_TREE or GW_SUM_REFERENCE");
  if (c->batch) return set_err(GW_EINVAL, "gw_set_sum_order: the cell is in a batch");
  c->sum_order = order;
  return GW_OK;
}

extern "C" int gw_sync(gw_ctx* c) {
  if (!c) return set_err(GW_EINVAL, "gw_sync: null context");
  CK(cudaStreamSynchronize(c->stream));
  return GW_OK;
}

static int check_states(int n, const int* ltype, const int* ryr, const int* ito2, const int* mti) {
  for (int f = 0; f < n; f++) {
    for (int c = 0; c < 4; c++) {
      int l = ltype[8 * f + 2 * c], v = ltype[8 * f + 2 * c + 1], x = ito2[4 * f + c];
      if (l < 1 || l > 12 || v < 1 || v > 2 || x < 1 || x > 2)
        return set_err(GW_EINVAL, "FRU %d cleft %d: channel state out of range (LCC %d, VDI %d, ClCh %d)", f, c, l,
                       v, x);
      for (int i = 0; i < 5; i++) {
        int r = ryr[20 * f + 5 * c + i];
        if (r < 1 || r > 8) return set_err(GW_EINVAL, "FRU %d cleft %d RyR %d: state %d out of range", f, c, i, r);
      }
    }
    if (mti[f] < 0 || mti[f] > gw::kMtN) return set_err(GW_EINVAL, "FRU %d: mti %d out of range", f, mti[f]);
  }
  return GW_OK;
}

extern "C" int gw_upload(gw_ctx* c, const double* frus, const int* ltype, const int* ryr, const int* ito2,
                         const int* mti, const uint32_t* mt) {
  if (!c || !frus || !ltype || !ryr || !ito2 || !mti || !mt) return set_err(GW_EINVAL, "gw_upload: null argument");
  const int n = c->d.nfru;
  int rc = check_states(n, ltype, ryr, ito2, mti);
  if (rc) return rc;
  const size_t nf = (size_t)c->d.stride;
  std::vector<double> hf(5 * nf, 0.0);
  std::vector<uint32_t> hc(4 * nf, 0u);
  for (int f = 0; f < n; f++) {
    for (int i = 0; i < 5; i++) hf[i * nf + f] = frus[5 * f + i];
    for (int k = 0; k < 4; k++) {
      uint32_t w = (uint32_t)ltype[8 * f + 2 * k] | ((uint32_t)ltype[8 * f + 2 * k + 1] << 4) |
                   ((uint32_t)ito2[4 * f + k] << 28);
      for (int i = 0; i < 5; i++) w |= (uint32_t)ryr[20 * f + 5 * k + i] << (8 + 4 * i);
      hc[k * nf + f] = w;
    }
  }
  CK(cudaMemcpyAsync(c->d.frus, hf.data(), hf.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d.chan, hc.data(), hc.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d.mti, mti, n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpy2DAsync(c->d.mt, gw::kMtStride * sizeof(uint32_t), mt, gw::kMtN * sizeof(uint32_t),
                       gw::kMtN * sizeof(uint32_t), n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d.hold_epoch, 0xff, nf * sizeof(uint32_t), c->stream));
  c->pending = 0;
  CK(cudaStreamSynchronize(c->stream));  // host staging vectors go out of scope
  return GW_OK;
}

// Apply a pending save/resume with a zero-length stage (no substeps).
static int flush_pending(gw_ctx* c) {
  if (!c->pending) return GW_OK;
  StageParams p = {};
  p.flags = c->pending;
  p.epoch = c->epoch;
  p.nfru_scale = c->nfru_scale;
  p.pca_scale = c->pca_scale;
  c->pending = 0;
  if (c->batch) {
    double out[32];
    return gw_batch_post(c, p, out);
  }
  CK(launch_stage_variant(c, p));
  c->launches++;
  return GW_OK;
}

extern "C" int gw_download(gw_ctx* c, double* frus, int* ltype, int* ryr, int* ito2, int* mti, uint32_t* mt) {
  if (!c) return set_err(GW_EINVAL, "gw_download: null context");
  int rc = flush_pending(c);
  if (rc) return rc;
  const int n = c->d.nfru;
  const size_t nf = (size_t)c->d.stride;
  std::vector<double> hf(5 * nf);
  std::vector<uint32_t> hc(4 * nf);
  CK(cudaMemcpyAsync(hf.data(), c->d.frus, hf.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(hc.data(), c->d.chan, hc.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  if (mti) CK(cudaMemcpyAsync(mti, c->d.mti, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (mt)
    CK(cudaMemcpy2DAsync(mt, gw::kMtN * sizeof(uint32_t), c->d.mt, gw::kMtStride * sizeof(uint32_t),
                         gw::kMtN * sizeof(uint32_t), n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int f = 0; f < n; f++) {
    if (frus)
      for (int i = 0; i < 5; i++) frus[5 * f + i] = hf[i * nf + f];
    for (int k = 0; k < 4; k++) {
      const uint32_t w = hc[k * nf + f];
      if (ltype) {
        ltype[8 * f + 2 * k] = (int)(w & 15u);
        ltype[8 * f + 2 * k + 1] = (int)((w >> 4) & 15u);
      }
      if (ryr)
        for (int i = 0; i < 5; i++) ryr[20 * f + 5 * k + i] = (int)((w >> (8 + 4 * i)) & 15u);
      if (ito2) ito2[4 * f + k] = (int)(w >> 28);
    }
  }
  return GW_OK;
}

extern "C" int gw_download_range(gw_ctx* c, int first, int count, double* frus, int* ltype, int* ryr, int* ito2) {
  if (!c) return set_err(GW_EINVAL, "gw_download_range: null context");
  if (first < 0 || count <= 0 || first + count > c->d.nfru)
    return set_err(GW_EINVAL, "gw_download_range: FRUs %d..%d outside 0..%d", first, first + count - 1,
                   c->d.nfru - 1);
  int rc = flush_pending(c);
  if (rc) return rc;
  const size_t nf = (size_t)c->d.stride;
  std::vector<double> hf(5 * (size_t)count);
  std::vector<uint32_t> hc(4 * (size_t)count);
  CK(cudaMemcpy2DAsync(hf.data(), count * sizeof(double), c->d.frus + first, nf * sizeof(double),
                       count * sizeof(double), 5, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpy2DAsync(hc.data(), count * sizeof(uint32_t), c->d.chan + first, nf * sizeof(uint32_t),
                       count * sizeof(uint32_t), 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int f = 0; f < count; f++) {
    if (frus)
      for (int i = 0; i < 5; i++) frus[5 * f + i] = hf[(size_t)i * count + f];
    for (int k = 0; k < 4; k++) {
      const uint32_t w = hc[(size_t)k * count + f];
      if (ltype) {
        ltype[8 * f + 2 * k] = (int)(w & 15u);
        ltype[8 * f + 2 * k + 1] = (int)((w >> 4) & 15u);
      }
      if (ryr)
        for (int i = 0; i < 5; i++) ryr[20 * f + 5 * k + i] = (int)((w >> (8 + 4 * i)) & 15u);
      if (ito2) ito2[4 * f + k] = (int)(w >> 28);
    }
  }
  return GW_OK;
}

extern "C" int gw_seed(gw_ctx* c, int scheme, uint32_t base) {
  if (!c || (scheme != gw::kSeedBase && scheme != gw::kSeedReference))
    return set_err(GW_EINVAL, "gw_seed: bad context or scheme %d", scheme);
  CK(gw::launch_seed(c->d, scheme, base, c->stream));
  c->launches++;
  CK(cudaStreamSynchronize(c->stream));
  return GW_OK;
}

static int run_stage(gw_ctx* c, double t0, double tf, const double dep0[3], const double depf[3], int advance,
                     double out[4], double num[5]) {
  StageParams p;
  p.t0 = t0;
  p.tf = tf;
  for (int i = 0; i < 3; i++) {
    p.dep0[i] = dep0[i];
    p.depf[i] = depf[i];
    p.span[i] = depf[i] - dep0[i];
  }
  p.nfru_scale = c->nfru_scale;
  p.pca_scale = c->pca_scale;
  p.epoch = c->epoch;
  p.flags = c->pending | (advance ? gw::kFlagAdvance : 0);
  c->pending = 0;
  if (c->batch) {
    int rc = gw_batch_post(c, p, c->h_out);
    if (rc) return rc;
    if (c->h_out[gw::kOutError] != 0.0)
      return set_err(GW_EINVAL, "FRU stage [%g, %g]: substep limit reached (corrupted FRU state: NaN or "
                     "out-of-range concentrations)", t0, tf);
    if (num)
      for (int k = 0; k < 5; k++) num[k] = c->h_out[k];
    if (out)
      for (int k = 0; k < 4; k++) out[k] = c->h_out[5 + k];
    return GW_OK;
  }
  if (c->profiling) CK(cudaEventRecord(c->pev[0], c->stream));
  CK(launch_stage_variant(c, p));
  c->launches++;
  if (c->sum_order == GW_SUM_REFERENCE) {
    CK(gw::launch_flux_seq(c->d, p, c->stream));
    c->launches++;
  }
  if (c->profiling) CK(cudaEventRecord(c->pev[1], c->stream));
  CK(cudaMemcpyAsync(c->h_out, c->d.out, 32 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->h_out[gw::kOutError] != 0.0) {
    double z = 0.0;
    CK(cudaMemcpy(c->d.out + gw::kOutError, &z, sizeof z, cudaMemcpyHostToDevice));
    return set_err(GW_EINVAL, "FRU stage [%g, %g]: substep limit reached (corrupted FRU state: NaN or "
                   "out-of-range concentrations)", t0, tf);
  }
  if (c->profiling) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->pev[0], c->pev[1]));
    c->prof_ms += ms;
    c->prof_launches++;
  }
  if (num)
    for (int k = 0; k < 5; k++) num[k] = c->h_out[k];
  if (out)
    for (int k = 0; k < 4; k++) out[k] = c->h_out[5 + k];
  return GW_OK;
}

extern "C" int gw_stage(gw_ctx* c, double t0, double tf, const double dep0[3], const double depf[3], double out[4],
                        double num[5]) {
  if (!c || !dep0 || !depf) return set_err(GW_EINVAL, "gw_stage: null argument");
  return run_stage(c, t0, tf, dep0, depf, 1, out, num);
}

extern "C" int gw_flux(gw_ctx* c, const double dep[3], double out[4], double num[5]) {
  if (!c || !dep) return set_err(GW_EINVAL, "gw_flux: null argument");
  return run_stage(c, 0.0, 0.0, dep, dep, 0, out, num);
}

extern "C" int gw_avg_sums(gw_ctx* c, double num[11]) {
  if (!c || !num) return set_err(GW_EINVAL, "gw_avg_sums: null argument");
  int rc = flush_pending(c);
  if (rc) return rc;
  if (c->sum_order == GW_SUM_REFERENCE)
    CK(gw::launch_avg_seq(c->d, c->stream));
  else
    CK(gw::launch_avg(c->d, c->stream));
  c->launches++;
  CK(cudaMemcpyAsync(c->h_out + 16, c->d.out + 16, 11 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 11; k++) num[k] = c->h_out[16 + k];
  return GW_OK;
}

extern "C" int gw_save(gw_ctx* c) {
  if (!c) return set_err(GW_EINVAL, "gw_save: null context");
  if (c->pending) {
    int rc = flush_pending(c);  // a pending resume runs under the old epoch
    if (rc) return rc;
  }
  // A new epoch: the first MT regeneration of each FRU after this point
  // copies the pre-regeneration words aside (copy-on-twist).
  c->epoch++;
  c->pending = gw::kFlagSave;
  return GW_OK;
}

extern "C" int gw_resume(gw_ctx* c) {
  if (!c) return set_err(GW_EINVAL, "gw_resume: null context");
  if (c->pending) {
    int rc = flush_pending(c);  // a pending save must land before rolling back to it
    if (rc) return rc;
  }
  c->pending = gw::kFlagResume;
  return GW_OK;
}

extern "C" int gw_substeps(gw_ctx* c, unsigned long long* count) {
  if (!c || !count) return set_err(GW_EINVAL, "gw_substeps: null argument");
  CK(cudaMemcpyAsync(count, c->d.substeps, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GW_OK;
}

// Device time of work that several cells run concurrently on their own
// streams: phase 0 records a start event on a timing stream and makes every
// cell's stream wait for it; phase 1 makes the timing stream wait for every
// cell's stream, records the end event and returns the elapsed ms.
extern "C" int gw_group_timer(int n, gw_ctx** cells, int phase, float* ms) {
  static cudaStream_t ts = nullptr;
  static cudaEvent_t ev[2] = {nullptr, nullptr};
  static cudaEvent_t link = nullptr;
  if (n <= 0 || !cells || (phase != 0 && phase != 1) || (phase == 1 && !ms))
    return set_err(GW_EINVAL, "gw_group_timer: bad argument");
  if (!ts) {
    CK(cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    CK(cudaEventCreateWithFlags(&link, cudaEventDisableTiming));
  }
  if (phase == 0) {
    CK(cudaEventRecord(ev[0], ts));
    for (int i = 0; i < n; i++) CK(cudaStreamWaitEvent(cells[i]->stream, ev[0], 0));
    return GW_OK;
  }
  for (int i = 0; i < n; i++) {
    CK(cudaEventRecord(link, cells[i]->stream));
    CK(cudaStreamWaitEvent(ts, link, 0));
  }
  CK(cudaEventRecord(ev[1], ts));
  CK(cudaEventSynchronize(ev[1]));
  CK(cudaEventElapsedTime(ms, ev[0], ev[1]));
  return GW_OK;
}

extern "C" int gw_stage_trace(gw_ctx* c, int enable) {
  if (!c) return set_err(GW_EINVAL, "gw_stage_trace: null context");
  if (c->batch) return set_err(GW_EINVAL, "gw_stage_trace: change it before the cell joins a batch");
  CK(cudaStreamSynchronize(c->stream));
  if (enable && !c->d.trace_sub) {
    const size_t ng = (size_t)(c->d.nfru + 7) / 8;
    CK(cudaMalloc((void**)&c->d.trace_sub, sizeof(uint32_t) * c->d.nfru));
    cudaError_t e = cudaMalloc((void**)&c->d.trace_ns, sizeof(unsigned long long) * 2 * ng);
    if (e != cudaSuccess) {
      cudaFree(c->d.trace_sub);
      c->d.trace_sub = nullptr;
      CK(e);
    }
    CK(cudaMemsetAsync(c->d.trace_sub, 0, sizeof(uint32_t) * c->d.nfru, c->stream));
    CK(cudaMemsetAsync(c->d.trace_ns, 0, sizeof(unsigned long long) * 2 * ng, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  } else if (!enable && c->d.trace_sub) {
    cudaFree(c->d.trace_sub);
    cudaFree(c->d.trace_ns);
    c->d.trace_sub = nullptr;
    c->d.trace_ns = nullptr;
  }
  return GW_OK;
}

extern "C" int gw_stage_trace_read(gw_ctx* c, uint32_t* substeps, unsigned long long* warp_ns) {
  if (!c || !c->d.trace_sub) return set_err(GW_EINVAL, "gw_stage_trace_read: tracing is not enabled");
  const size_t ng = (size_t)(c->d.nfru + 7) / 8;
  if (substeps)
    CK(cudaMemcpyAsync(substeps, c->d.trace_sub, sizeof(uint32_t) * c->d.nfru, cudaMemcpyDeviceToHost, c->stream));
  if (warp_ns)
    CK(cudaMemcpyAsync(warp_ns, c->d.trace_ns, sizeof(unsigned long long) * 2 * ng, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GW_OK;
}

extern "C" int gw_event_record(gw_ctx* c, int slot) {
  if (!c || slot < 0 || slot > 7) return set_err(GW_EINVAL, "gw_event_record: bad slot");
  CK(cudaEventRecord(c->ev[slot], c->stream));
  return GW_OK;
}

extern "C" int gw_event_elapsed(gw_ctx* c, int a, int b, float* ms) {
  if (!c || !ms || a < 0 || a > 7 || b < 0 || b > 7) return set_err(GW_EINVAL, "gw_event_elapsed: bad slot");
  CK(cudaEventSynchronize(c->ev[b]));
  CK(cudaEventElapsedTime(ms, c->ev[a], c->ev[b]));
  return GW_OK;
}

extern "C" int gw_profile(gw_ctx* c, int enable) {
  if (!c) return set_err(GW_EINVAL, "gw_profile: null context");
  c->profiling = enable != 0;
  c->prof_ms = 0.0;
  c->prof_launches = 0;
  return GW_OK;
}

extern "C" int gw_profile_read(gw_ctx* c, double* ms, unsigned long long* launches) {
  if (!c) return set_err(GW_EINVAL, "gw_profile_read: null context");
  if (ms) *ms = c->prof_ms;
  if (launches) *launches = c->prof_launches;
  return GW_OK;
}

extern "C" int gw_launches(gw_ctx* c, unsigned long long* count) {
  if (!c || !count) return set_err(GW_EINVAL, "gw_launches: null argument");
  *count = c->launches;
  return GW_OK;
}

extern "C" int gw_l2_flush(gw_ctx* c) {
  const size_t bytes = (size_t)512 << 20;
  if (!c) return set_err(GW_EINVAL, "gw_l2_flush: null context");
  if (!c->flush_buf) CK(cudaMalloc(&c->flush_buf, bytes));
  CK(cudaMemsetAsync(c->flush_buf, c->launches & 0xff, bytes, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GW_OK;
}

extern "C" int gw_probe_fcn(double* device_us, double* host_us) {
  if (!device_us || !host_us) return set_err(GW_EINVAL, "gw_probe_fcn: null argument");
  CK(gw::probe_fcn(device_us, host_us));
  return GW_OK;
}

extern "C" int gw_probe_exp(const double* x, double* device_y, double* host_y, int n) {
  if (!x || !device_y || !host_y || n <= 0) return set_err(GW_EINVAL, "gw_probe_exp: bad argument");
  CK(gw::probe_exp(x, device_y, host_y, n));
  return GW_OK;
}

extern "C" int gw_probe_fp64_issue(double* cycles) {
  if (!cycles) return set_err(GW_EINVAL, "gw_probe_fp64_issue: null argument");
  CK(gw::probe_fp64_issue(cycles));
  return GW_OK;
}

extern "C" int gw_probe_div(unsigned long long seed, long long n, unsigned long long* mismatches) {
  if (!mismatches || n <= 0) return set_err(GW_EINVAL, "gw_probe_div: bad argument");
  CK(gw::probe_div(seed, n, mismatches));
  return GW_OK;
}

extern "C" int gw_probe_fcn_warp(double* us) {
  if (!us) return set_err(GW_EINVAL, "gw_probe_fcn_warp: null argument");
  CK(gw::probe_fcn_warp(us));
  return GW_OK;
}

extern "C" int gw_probe_fcn_compare(const double* states, int n, double time, int clamp, double* Fs, double* Fw,
                                    double* Cs, double* Cw) {
  if (!states || n <= 0 || !Fs || !Fw || !Cs || !Cw) return set_err(GW_EINVAL, "gw_probe_fcn_compare: bad argument");
  CK(gw::probe_fcn_compare(states, n, time, clamp, Fs, Fw, Cs, Cw));
  return GW_OK;
}

extern "C" int gw_probe_fp64_peak(double* tflops) {
  if (!tflops) return set_err(GW_EINVAL, "gw_probe_fp64_peak: null argument");
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double best = 0.0;
  CK(gw::probe_fp64(sms, &best));
  *tflops = best;
  return GW_OK;
}
