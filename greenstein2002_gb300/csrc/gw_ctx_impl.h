// Private definition of gw_ctx (one cell's device state and settings),
// shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_kernels.h"

struct gw_batch;

struct gw_ctx {
  gw::DevState d;
  cudaStream_t stream = nullptr;
  double* h_out = nullptr;  // pinned [32]
  double nfru_scale = 1.0;
  uint32_t epoch = 0;
  int pending = 0;          // kFlagSave / kFlagResume to fold into the next launch
  int device = 0;
  cudaEvent_t ev[8] = {};
  cudaEvent_t pev[2] = {};  // bracket of the last stage launch while profiling
  bool profiling = false;
  double prof_ms = 0.0;
  unsigned long long prof_launches = 0, launches = 0;
  void* flush_buf = nullptr;
  int fru_lanes = 4;        // lanes per FRU of the stage kernel: 1 or 4
  int stage_warps = 1;      // warps per block of the 4-lane stage kernels
  int packed_warps = 0;     // > 0: packed stage launches of that many warps
  uint32_t pack_launch = 0; // packed launches so far
  int precision = 0;        // 0: FP64, 1: mixed (FP32 rates and local ODE)
  double pca_scale = 1.0;   // LCC permeability scale of the cell
  int sum_order = 0;        // GW_SUM_TREE or GW_SUM_REFERENCE
  gw_batch* batch = nullptr;  // set while the cell is a member of a batch
  int slot = -1;              // its index in the batch
  double batch_out[32];       // its outputs of the last batch round
};

// Post one stage operation of a batched cell and wait for the batch round
// that runs it; out receives the cell's 32 output slots (gw_batch.cu).
int gw_batch_post(gw_ctx* c, const gw::StageParams& p, double* out);

