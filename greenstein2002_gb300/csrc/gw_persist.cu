// Persistent multi-cell kernel: every cell's FRU stages, flux reductions and
// Dormand-Prince 5(4) integrator steps run inside one launch, without host
// round trips and without lockstep rounds.
//
// The reference advances one cell per MPI job: rk54pd (rk_pd54m.c:29-345)
// calls distrib_simFRU (mpi_master.c:369-469) five or six times per attempt,
// and every call waits for the slowest FRU.  Here one resident grid serves
// all cells at once.  Each cell's integrator posts one "operation" at a time
// (a flux evaluation at an attempt's start, or an FRU stage over [t0, tf]),
// and warps take the operation's FRUs in batches of consecutive 8-FRU
// groups from a per-cell counter.  A warp advances its batch's FRUs with the
// substep loop of the cleft kernels (advance4's substep_a / substep_b,
// warp-wide MT19937 regeneration), its eight 4-lane groups taking the
// batch's FRUs one after another as they finish (the packed launches'
// scheme, with a warp-uniform counter instead of a queue in memory); then
// forms each group's flux (and output-average) partial sums exactly as the
// fixed-layout stage kernel does -- same lanes, same shuffle tree -- from
// the stored FRUs.  The warp that stores the operation's last batch adds
// the partials in the fixed order of cell_finish, forms the currents, runs
// the cell's integrator step on the whole warp (dp_after_warp: the
// arithmetic of gw_dp.c, the 37-state vectors split over the lanes and
// fcn's exponentials one per lane) and posts the cell's next operation.
// Operations that do not advance (the flux at an attempt's start) take
// their batches the same way and only apply a pending save / resume.
// A warp that finds nothing in one cell works on whatever else is open, so
// one cell's slowest FRU no longer holds the GPU.  Every cell's arithmetic,
// reduction order and integrator are those of its single-cell run, so its
// results are the same bits alone, in any mix, and in the round-based
// device runner (gw_run_device).
//
// Waiting: a warp with nothing to do sleeps and checks a global progress
// counter (batches and operations finished); if it has not moved for
// `wait_ns` (2 s by default; real operations take microseconds to
// milliseconds) the kernel sets an error status and every warp returns, so
// the context stays usable and the host reports the error.  No warp ever
// waits for a specific other warp, so the grid needs no co-residency
// guarantee; it is sized to the occupancy (one single-warp block per
// resident slot) all the same.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "gw_cell_model.h"
#include "gw_ctx_impl.h"
#include "gw_diag.h"
#include "gw_dp_device.cuh"
#include "gw_fru.h"
#include "gw_fru_cleft.cuh"

extern "C" int gw_internal_error(int code, const char* msg);

namespace gw {
namespace persist {

constexpr int kMaxBatchGroups = 8;  // 8-FRU groups a warp takes at once, at most
constexpr int kMaxCells = 1024;     // cells of one run (16 mask words)
constexpr unsigned kFull = 0xffffffffu;
enum : int { kStatusOk = 0, kStatusWatchdog = 3 };
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;

// Scheduling state of one cell.  `take` is reset only when an operation
// opens, so a warp that increments it late either gets an index past the
// end (nothing to do) or a valid batch of an open operation, and it reads
// the operation's parameters after the increment.
struct PCell {
  unsigned long long take;  // next 8-FRU group of the open operation (>= ngroups: none)
  unsigned done;            // groups of the open operation stored and summed
  unsigned overflow;        // an FRU of the operation reached the substep limit
  int finished;
};

struct Args {
  const DevState* cells;
  DpCell* dp;
  PCell* pc;
  int ncells;
  int batch;                     // 8-FRU groups per take (1 .. kMaxBatchGroups)
  unsigned* running;             // cells with output steps left
  unsigned long long* open_mask; // bit per cell: its operation has groups left to take
  int nwords;                    // 64-bit words of the mask
  unsigned long long* progress;  // batches finished
  unsigned long long* ops;       // operations completed
  int* status;                   // kStatus*
  unsigned long long wait_ns;
  const int* release;            // null, or operations are posted only while *release != 0
};

__device__ __forceinline__ int vload(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ unsigned vload(const unsigned* p) { return *(const volatile unsigned*)p; }
__device__ __forceinline__ unsigned long long vload(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}
__device__ __forceinline__ int ngroups_of(const DevState& s) { return (s.nfru + 7) >> 3; }

// ---- the open-cell mask --------------------------------------------------------------
// A cell's bit is set after its counter is reset (open), and the warp that
// finds the counter exhausted clears the bit and then looks at the counter
// again, setting the bit back if a new operation opened meanwhile; so an
// operation with groups left always has its bit set.
__device__ __forceinline__ void mask_set(unsigned long long* m, int ci) {
  atomicOr(&m[ci >> 6], 1ull << (ci & 63));
}
__device__ __forceinline__ void mask_clear(const Args& a, int ci, int ngroups) {
  atomicAnd(&a.open_mask[ci >> 6], ~(1ull << (ci & 63)));
  __threadfence();
  if (vload(&a.pc[ci].take) < (unsigned long long)ngroups) mask_set(a.open_mask, ci);
}
// a set bit of the mask at or after `from` (cyclically); -1: none
__device__ __forceinline__ int mask_pick(const unsigned long long* m, int nwords, int ncells, int from) {
  const int w0 = from >> 6;
  for (int k = 0; k <= nwords; k++) {
    const int w = (w0 + k) % nwords;
    unsigned long long bits = vload(&m[w]);
    if (k == 0) bits &= ~0ull << (from & 63);
    else if (k == nwords) bits &= ~(~0ull << (from & 63));
    if (bits) {
      const int ci = (w << 6) + __ffsll((long long)bits) - 1;
      return ci < ncells ? ci : -1;
    }
  }
  return -1;
}

// Post the operation dp_after has just set up in the cell's DpCell (one thread).
static __device__ void post(const Args& a, int ci) {
  PCell& pc = a.pc[ci];
  pc.done = 0u;
  pc.overflow = 0u;
  __threadfence();
  atomicExch(&pc.take, 0ull);
  __threadfence();
  mask_set(a.open_mask, ci);
}

// The cell's totals from its group partials in cell_finish's order, the
// currents, and the integrator step; then the next operation is posted (or
// the cell is done).  Whole warp.
template <int NV>
__device__ __forceinline__ void finish_op(const Args& a, int ci, int lane) {
  const DevState& s = a.cells[ci];
  DpCell& c = a.dp[ci];
  const int ngroups = ngroups_of(s);
  __threadfence();
  double tot[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) tot[k] = 0.0;
  for (int b = lane; b < ngroups; b += 32)
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] += __ldcg(&s.partials[b * NV + k]);
  cleft::warp_sum<NV>(tot);
#pragma unroll
  for (int k = 0; k < NV; k++) tot[k] = __shfl_sync(kFull, tot[k], 0);
  PCell& pc = a.pc[ci];
  double cur[4];
  currents_from_sums(s.nfru, c.sp.nfru_scale, c.sp.depf, tot, cur);
  cur[2] = cur[2] * c.sp.pca_scale;  // ICa is proportional to the LCC permeability
  const bool ovf = vload(&pc.overflow) != 0u;
  __syncwarp();
  if (ovf) {
    if (lane == 0) c.err = 1;  // substep limit: corrupted FRU state
    __syncwarp();
  } else {
    dp_after_warp(c, cur, NV == 16 ? tot + 5 : nullptr, lane);
  }
  if (lane == 0) {
    atomicAdd(a.ops, 1ull);
    if (c.done || c.err) {
      pc.finished = 1;
      __threadfence();
      atomicSub(a.running, 1u);
    } else if (!a.release || vload(a.release) != 0) {
      post(a, ci);
    }
    // else: held by the caller's release flag (never posted)
  }
  __syncwarp();
}

// One 8-FRU group's partial sums into partials[grp * NV ..], by the whole
// warp in the lanes of the fixed-layout kernel (FRU grp*8 + lane/4, cleft
// lane%4), from the FRUs as stored: stage_body_fin's epilogue.
template <int NV>
__device__ __forceinline__ void group_partials(const DevState& s, int grp, const cleft::Group& g, int lane) {
  const int f = grp * 8 + (lane >> 2);
  const bool active = f < s.nfru;
  const size_t nf = (size_t)s.stride;
  double cajsr = 0.0, cass = 0.0;
  uint32_t w = 0u;
  if (active) {
    cajsr = s.frus[f];
    cass = s.frus[(g.c + 1) * nf + f];
    w = s.chan[g.c * nf + f];
  }
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = 0.0;
  if (active) {
    v[0] = cass;
    v[1] = (g.c == 0) ? cajsr : 0.0;
    if (lcc_open(w)) {
      v[2] = cass;
      v[3] = 1.0;
    }
    if (cl_of(w) == 2) v[4] = 1.0;
  }
  if (NV == 16) {
    double t[11];
    cleft::avg_terms(g.c, cajsr, cass, w, t);
#pragma unroll
    for (int k = 0; k < 11; k++) v[(5 + k) % NV] = active ? t[k] : 0.0;
  }
  cleft::warp_sum<NV>(v);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) s.partials[grp * NV + k] = v[k];
}

// One batch of cell ci's open operation: groups [grp0, grp0 + ng).  The
// FRUs are loaded (applying the operation's save / resume), advanced when
// the operation is a stage, and stored; then the groups' partial sums; the
// warp that stores the operation's last batch finishes the operation.
template <typename R>
__device__ __forceinline__ void run_batch(const Args& a, int ci, int grp0, int ng, int lane) {
  using namespace cleft;
  const DevState& s = a.cells[ci];
  const StageParams& p = a.dp[ci].sp;
  const int n = s.nfru;
  const int ngroups = ngroups_of(s);
  const int f_begin = grp0 * 8;
  const int f_end = min(n, (grp0 + ng) * 8);
  const size_t nf = (size_t)s.stride;
  const bool restore_op = (p.flags & kFlagResume) != 0;
  Group g;
  g.c = lane & 3;
  g.base = lane & ~3;
  g.mask = 0xfu << g.base;
  bool overflow = false;
  unsigned long long nsub_sum = 0ull;
  if (p.flags & kFlagAdvance) {
    LaneStage<R> LS;
    lane_stage(p, g, LS);
    StageCtx sc;
    sc.p = &p;
    sc.m = s.mt;
    sc.hold_base = s.mt_hold;
    sc.hold_epoch_base = s.hold_epoch;
    sc.f = 0;
    sc.my_hold_epoch = s.hold_epoch;
    Fru4<R> F;
    F.clk = {};
    F.jsr.set(0.0);
    F.ss.set(0.0);
    F.w = 0u;
    F.nsub = 0u;
    F.mti = 0;
    int f = -1;
    auto load = [&](int ff) {
      f = ff;
      sc.f = ff;
      sc.my_hold_epoch = s.hold_epoch + ff;
      bool restore = false;
      if (restore_op) {
        F.jsr.set(s.frus_s[ff]);
        F.ss.set(s.frus_s[(g.c + 1) * nf + ff]);
        F.w = s.chan_s[g.c * nf + ff];
        F.mti = s.mti_s[ff];
        restore = (*sc.my_hold_epoch == p.epoch);
      } else {
        F.jsr.set(__ldcg(&s.frus[ff]));
        F.ss.set(__ldcg(&s.frus[(g.c + 1) * nf + ff]));
        F.w = __ldcg(&s.chan[g.c * nf + ff]);
        F.mti = __ldcg(&s.mti[ff]);
      }
      if (p.flags & kFlagSave) {
        if (g.c == 0) {
          s.frus_s[ff] = F.jsr.get();
          s.mti_s[ff] = F.mti;
        }
        s.frus_s[(g.c + 1) * nf + ff] = F.ss.get();
        s.chan_s[g.c * nf + ff] = F.w;
      }
      use_row(sc, s.mt + (size_t)ff * kMtStride, s.mt_hold + (size_t)ff * kMtStride, restore, g);
      F.nsub = 0u;
      fru_begin(F, LS);
    };
    auto finish = [&]() {
      if (g.c == 0) {
        s.frus[f] = F.jsr.get();
        s.mti[f] = F.mti;
        nsub_sum += F.nsub;
      }
      s.frus[(g.c + 1) * nf + f] = F.ss.get();
      s.chan[g.c * nf + f] = F.w;
    };
    // the batch's first eight FRUs one per group; then each group that
    // stores its FRU takes the next, in group order (a warp-uniform count of
    // the FRUs handed out, advanced by a ballot of the groups that need one)
    int next = f_begin + 8;
    {
      const int ff = f_begin + (lane >> 2);
      if (ff < f_end) load(ff);
    }
    __syncwarp();
    while (true) {
      const bool has = f >= 0;
      bool go = has && F.clk.running(LS);
      if (go && F.nsub >= (1u << 22)) {
        overflow = true;
        go = false;
      }
      if (!__any_sync(kFull, has)) break;
      Sub4<R> S;
      S.etot = 0;
#pragma unroll
      for (int i = 0; i < kRyR; i++) S.exw[i] = 0u;
      S.p34 = R(0);
      if (go) substep_a(F, S, LS, g, sc);
      regen_step(sc, lane, g, go, F, S);
      if (go) substep_b(F, S, LS, g, sc);
      const bool stored = has && !(go && F.clk.running(LS));
      if (stored) {
        finish();
        f = -1;
      }
      const unsigned need = __ballot_sync(kFull, stored && g.c == 0);
      if (need) {
        const int ff = next + __popc(need & ((1u << g.base) - 1u));
        next += __popc(need);
        if (stored && ff < f_end) load(ff);
      }
      __syncwarp();
    }
  } else {
    // no advance: apply a pending save / resume (stage_body_fin without the
    // substeps), in the fixed layout
    for (int grp = grp0; grp < grp0 + ng; grp++) {
      const int ff = grp * 8 + (lane >> 2);
      if (ff < n) {
        double cajsr, cass;
        uint32_t w;
        int mti;
        bool restore = false;
        if (restore_op) {
          cajsr = s.frus_s[ff];
          cass = s.frus_s[(g.c + 1) * nf + ff];
          w = s.chan_s[g.c * nf + ff];
          mti = s.mti_s[ff];
          restore = (s.hold_epoch[ff] == p.epoch);
        } else {
          cajsr = __ldcg(&s.frus[ff]);
          cass = __ldcg(&s.frus[(g.c + 1) * nf + ff]);
          w = __ldcg(&s.chan[g.c * nf + ff]);
          mti = __ldcg(&s.mti[ff]);
        }
        if (p.flags & kFlagSave) {
          if (g.c == 0) {
            s.frus_s[ff] = cajsr;
            s.mti_s[ff] = mti;
          }
          s.frus_s[(g.c + 1) * nf + ff] = cass;
          s.chan_s[g.c * nf + ff] = w;
        }
        if (restore) copy_row16(s.mt + (size_t)ff * kMtStride, s.mt_hold + (size_t)ff * kMtStride, g);
        if (restore_op) {
          if (g.c == 0) {
            s.frus[ff] = cajsr;
            s.mti[ff] = mti;
          }
          s.frus[(g.c + 1) * nf + ff] = cass;
          s.chan[g.c * nf + ff] = w;
        }
      }
    }
  }
  __syncwarp();  // the stores above are visible to the whole warp
  const bool avg = (p.flags & kFlagAvg) != 0;
  for (int grp = grp0; grp < grp0 + ng; grp++) {
    if (avg) group_partials<16>(s, grp, g, lane);
    else group_partials<5>(s, grp, g, lane);
  }
  if (s.substeps) {
    for (int o = 16; o > 0; o >>= 1) nsub_sum += __shfl_down_sync(kFull, nsub_sum, o);
    if (lane == 0 && nsub_sum) atomicAdd(s.substeps, nsub_sum);
  }
  PCell& pc = a.pc[ci];
  if (__any_sync(kFull, overflow) && lane == 0) atomicOr(&pc.overflow, 1u);
  __threadfence();
  __syncwarp();
  unsigned last = 0u;
  if (lane == 0) {
    last = (atomicAdd(&pc.done, (unsigned)ng) + (unsigned)ng == (unsigned)ngroups) ? 1u : 0u;
    atomicAdd(a.progress, 1ull);
  }
  last = __shfl_sync(kFull, last, 0);
  if (last) {
    if (avg) finish_op<16>(a, ci, lane);
    else finish_op<5>(a, ci, lane);
  }
}

template <typename R>
__device__ __forceinline__ void persist_body(const Args& a) {
  const int lane = threadIdx.x & 31;
  const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int cursor = warp % a.ncells;
  unsigned long long seen = 0ull, idle_since = 0ull;
  bool idle_clock = false;
  while (true) {
    // the next batch of any open operation (lane 0 takes it for the warp)
    int ci = -1, grp0 = 0, ng = 0;
    if (lane == 0) {
      for (int tries = 0; tries < 4; tries++) {
        const int cj = mask_pick(a.open_mask, a.nwords, a.ncells, cursor);
        if (cj < 0) break;
        const int ngr = ngroups_of(a.cells[cj]);
        const unsigned long long idx = atomicAdd(&a.pc[cj].take, (unsigned long long)a.batch);
        if (idx + (unsigned long long)a.batch >= (unsigned long long)ngr) mask_clear(a, cj, ngr);
        cursor = cj;
        if (idx >= (unsigned long long)ngr) continue;
        ci = cj;
        grp0 = (int)idx;
        ng = min(a.batch, ngr - grp0);
        break;
      }
    }
    ci = __shfl_sync(kFull, ci, 0);
    if (ci >= 0) {
      grp0 = __shfl_sync(kFull, grp0, 0);
      ng = __shfl_sync(kFull, ng, 0);
      __threadfence();  // the operation's parameters after the take
      run_batch<R>(a, ci, grp0, ng, lane);
      idle_clock = false;
      if (lane == 0) cursor = (cursor + 1) % a.ncells;  // spread the warps over the open cells
      if (__shfl_sync(kFull, vload(a.status), 0) != kStatusOk) break;
      continue;
    }
    int st = kStatusOk;
    unsigned run = 0u;
    if (lane == 0) {
      st = vload(a.status);
      run = vload(a.running);
    }
    st = __shfl_sync(kFull, st, 0);
    run = __shfl_sync(kFull, run, 0);
    if (st != kStatusOk || run == 0u) break;  // an error somewhere, or every cell is done
    // nothing to do: sleep, and give up if nothing anywhere has progressed
    // for wait_ns
    int give_up = 0;
    if (lane == 0) {
      const unsigned long long now = cleft::global_ns();
      const unsigned long long pr = vload(a.progress) + vload(a.ops);
      if (!idle_clock || pr != seen) {
        idle_clock = true;
        seen = pr;
        idle_since = now;
      } else if (now - idle_since > a.wait_ns) {
        atomicCAS(a.status, kStatusOk, kStatusWatchdog);
        give_up = 1;
      }
    }
    if (__shfl_sync(kFull, give_up, 0)) break;
    __nanosleep(1000);
  }
}

// Single-warp blocks, at least ten per SM (the register cap).
__global__ void __launch_bounds__(32, 10) persist_kernel_fp64(Args a) { persist_body<double>(a); }
__global__ void __launch_bounds__(32, 10) persist_kernel_mixed(Args a) { persist_body<float>(a); }

}  // namespace persist
}  // namespace gw

using gw::DpCell;
using gw::persist::PCell;

namespace {

// 8-FRU groups a warp takes at once: up to four (32 FRUs, the packed
// launches' best shape for full GPUs), fewer when the cells have too few
// groups to give every resident warp two batches.  GW_PERSIST_GROUPS
// (1..8) overrides the choice.
int persist_batch(long long total_groups, long long warps) {
  const char* env = getenv("GW_PERSIST_GROUPS");
  if (env) {
    const int v = atoi(env);
    if (v >= 1 && v <= gw::persist::kMaxBatchGroups) return v;
  }
  long long b = warps > 0 ? total_groups / (2 * warps) : 1;
  return (int)(b < 1 ? 1 : b > 4 ? 4 : b);
}

// One persistent run of n cells; wait_ns / release as in persist::Args.
int run_persistent(int n, gw_ctx** cells, const gw_settings* sets, double* t, double* states, double* oldsteps,
                   int n_steps, double* state_trace, double* other_trace, double* cur_trace,
                   unsigned long long wait_ns, bool hold, int* status_out, unsigned long long* ops_out) {
  const char* who = "gw_run_persistent";
  if (n <= 0 || n > gw::persist::kMaxCells || !cells || !sets || !t || !states || !oldsteps || n_steps <= 0)
    return gw_internal_error(GW_EINVAL, "gw_run_persistent: bad argument (1 to 1024 cells)");
  const int prec = cells[0]->precision;
  for (int i = 0; i < n; i++)
    if (!cells[i] || cells[i]->precision != prec || cells[i]->fru_lanes != 4 || cells[i]->batch ||
        cells[i]->sum_order != GW_SUM_TREE)
      return gw_internal_error(GW_EINVAL,
                               "gw_run_persistent: cells must share one precision, use the 4-lane kernel and "
                               "tree-order sums and not be batched");
  std::vector<gw::DevState> hcells(n);
  std::vector<DpCell> hdp(n);
  std::vector<PCell> hpc(n);
  long long total_groups = 0;
  for (int i = 0; i < n; i++) {
    gw_ctx* c = cells[i];
    cudaStreamSynchronize(c->stream);
    hcells[i] = c->d;
    DpCell& d = hdp[i];
    memset(&d, 0, sizeof d);
    memcpy(d.y, states + (size_t)i * GW_NSTATE, sizeof d.y);
    d.set = sets[i];
    d.tnow = t[i];
    d.oldstep = oldsteps[i];
    d.epoch = c->epoch;
    d.steps_left = n_steps;
    d.nfru = c->d.nfru;
    d.sp.nfru_scale = c->nfru_scale;
    d.sp.pca_scale = c->pca_scale;
    // the first operation: the flux at the first attempt's start, carrying
    // the context's pending save / resume (gw_run_device's preamble)
    d.tstep = d.tnow + d.set.time_step;
    double step = d.oldstep < d.tstep - d.tnow ? d.oldstep : d.tstep - d.tnow;
    step = d.set.step_max < step ? d.set.step_max : step;
    d.step = step;
    d.ostep = step;
    d.start = d.tnow;
    d.success = 1;
    d.keepc = 1;
    d.phase = gw::kPhFlux;
    const double dep[3] = {d.y[GW_V], d.y[GW_Cai], d.y[GW_CaNSR]};
    for (int k = 0; k < 3; k++) {
      d.sp.dep0[k] = d.sp.depf[k] = dep[k];
      d.sp.span[k] = 0.0;
    }
    d.sp.epoch = d.epoch;
    d.sp.flags = c->pending;
    d.pending = 0;
    PCell& p = hpc[i];
    memset(&p, 0, sizeof p);  // take = 0: the first operation (a flux) is open
    total_groups += (c->d.nfru + 7) / 8;
  }
  const size_t ns = (size_t)n * n_steps;
  gw::DevState* dcells = nullptr;
  DpCell* ddp = nullptr;
  PCell* dpc = nullptr;
  // counters: [0] running, [3] status, [4] release; then progress, ops; the open-cell mask
  int* dcnt = nullptr;
  unsigned long long* dmask = nullptr;
  const int nwords = (n + 63) / 64;
  unsigned long long* d64 = nullptr;
  double *dst = nullptr, *dot = nullptr, *dcu = nullptr;
  DpCell* hout = nullptr;  // pinned copy-back of the integrators
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int rc = GW_OK;
  int dev = 0, sms = 0, per_sm = 0;
  const bool mixed = prec == 1;
  const size_t smem = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = mixed ? gw::stage_cache_attributes(gw::persist::persist_kernel_mixed)
              : gw::stage_cache_attributes(gw::persist::persist_kernel_fp64);
  if (e == cudaSuccess)
    e = mixed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gw::persist::persist_kernel_mixed, 32, smem)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gw::persist::persist_kernel_fp64, 32, smem);
  if (e == cudaSuccess && per_sm <= 0) e = cudaErrorInvalidConfiguration;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&dcells, sizeof(gw::DevState) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ddp, sizeof(DpCell) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dpc, sizeof(PCell) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dcnt, sizeof(int) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dmask, sizeof(unsigned long long) * nwords);
  if (e == cudaSuccess) e = cudaMalloc(&d64, sizeof(unsigned long long) * 2);
  if (e == cudaSuccess) e = cudaMallocHost(&hout, sizeof(DpCell) * n);
  if (e == cudaSuccess && state_trace) e = cudaMalloc(&dst, sizeof(double) * ns * GW_NSTATE);
  if (e == cudaSuccess && other_trace) e = cudaMalloc(&dot, sizeof(double) * ns * GW_NOTHER);
  if (e == cudaSuccess && cur_trace) e = cudaMalloc(&dcu, sizeof(double) * ns * GW_NCUR);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    DpCell& d = hdp[i];
    d.tr_states = dst ? dst + (size_t)i * n_steps * GW_NSTATE : nullptr;
    d.tr_other = dot ? dot + (size_t)i * n_steps * GW_NOTHER : nullptr;
    d.tr_cur = dcu ? dcu + (size_t)i * n_steps * GW_NCUR : nullptr;
  }
  const int cnt[8] = {n, 0, n, gw::persist::kStatusOk, hold ? 0 : 1, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(dcells, hcells.data(), sizeof(gw::DevState) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ddp, hdp.data(), sizeof(DpCell) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dpc, hpc.data(), sizeof(PCell) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dcnt, cnt, sizeof cnt, cudaMemcpyHostToDevice);
  {
    // every cell's first operation (a flux) is open
    std::vector<unsigned long long> m(nwords, 0ull);
    for (int i = 0; i < n; i++) m[i >> 6] |= 1ull << (i & 63);
    if (e == cudaSuccess) e = cudaMemcpy(dmask, m.data(), sizeof(unsigned long long) * m.size(), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(d64, 0, sizeof(unsigned long long) * 2);
  gw::persist::Args args;
  args.cells = dcells;
  args.dp = ddp;
  args.pc = dpc;
  args.ncells = n;
  args.running = (unsigned*)dcnt;
  args.open_mask = dmask;
  args.nwords = nwords;
  args.batch = persist_batch(total_groups, (long long)sms * per_sm);
  args.status = dcnt + 3;
  args.release = hold ? dcnt + 4 : nullptr;
  args.progress = d64;
  args.ops = d64 + 1;
  args.wait_ns = wait_ns;
  // the run as one graph: the persistent launch, then the integrators' copy-back
  if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const dim3 grid(sms * per_sm), block(32);
    if (mixed) gw::persist::persist_kernel_mixed<<<grid, block, smem, st>>>(args);
    else gw::persist::persist_kernel_fp64<<<grid, block, smem, st>>>(args);
    cudaMemcpyAsync(hout, ddp, sizeof(DpCell) * n, cudaMemcpyDeviceToHost, st);
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = ec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int hc[8] = {0};
  unsigned long long h64[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(hc, dcnt, sizeof hc, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(h64, d64, sizeof h64, cudaMemcpyDeviceToHost);
  if (status_out) *status_out = hc[3];
  if (ops_out) *ops_out = h64[1];
  if (e == cudaSuccess && dst) e = cudaMemcpy(state_trace, dst, sizeof(double) * ns * GW_NSTATE, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dot) e = cudaMemcpy(other_trace, dot, sizeof(double) * ns * GW_NOTHER, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dcu) e = cudaMemcpy(cur_trace, dcu, sizeof(double) * ns * GW_NCUR, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    rc = gw_internal_error(GW_ECUDA, (std::string(who) + ": " + cudaGetErrorString(e)).c_str());
  } else if (hc[3] != gw::persist::kStatusOk) {
    rc = gw_internal_error(GW_ECUDA, "gw_run_persistent: no progress within the wait limit (watchdog); the cells' "
                                     "state is that of an unfinished run");
  } else {
    for (int i = 0; i < n; i++) {
      const DpCell& d = hout[i];
      if (d.err || !d.done) {
        rc = gw_internal_error(GW_EINVAL, d.err == 1   ? "gw_run_persistent: substep limit reached (corrupted FRU state)"
                                          : d.err == 2 ? "gw_run_persistent: global state not finite"
                                                       : "gw_run_persistent: a cell did not finish its output steps");
        break;
      }
      memcpy(states + (size_t)i * GW_NSTATE, d.y, sizeof d.y);
      t[i] = d.tnow;
      oldsteps[i] = d.oldstep;
      cells[i]->epoch = d.epoch;
      cells[i]->pending = 0;
      cells[i]->launches += 1;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaFree(dcells);
  cudaFree(ddp);
  cudaFree(dpc);
  cudaFree(dcnt);
  cudaFree(dmask);
  cudaFree(d64);
  cudaFree(dst);
  cudaFree(dot);
  cudaFree(dcu);
  if (hout) cudaFreeHost(hout);
  if (st) cudaStreamDestroy(st);
  return rc;
}

}  // namespace

extern "C" int gw_run_persistent(int n, gw_ctx** cells, const gw_settings* sets, double* t, double* states,
                                 double* oldsteps, int n_steps, double* state_trace, double* other_trace,
                                 double* cur_trace) {
  return run_persistent(n, cells, sets, t, states, oldsteps, n_steps, state_trace, other_trace, cur_trace,
                        gw::persist::kDefaultWaitNs, false, nullptr, nullptr);
}

extern "C" int gw_probe_persist_watchdog(gw_ctx* cell, const gw_settings* set, double wait_s, int* status) {
  if (!cell || !set || !status || !(wait_s > 0.0) || wait_s > 10.0)
    return gw_internal_error(GW_EINVAL, "gw_probe_persist_watchdog: bad argument (wait_s in (0, 10])");
  double t = 0.0, oldstep = set->step_max, state[GW_NSTATE];
  gw_rest_state(state);
  const int rc = run_persistent(1, &cell, set, &t, state, &oldstep, 1, nullptr, nullptr, nullptr,
                                (unsigned long long)(wait_s * 1e9), true, status, nullptr);
  return rc == GW_ECUDA && *status == gw::persist::kStatusWatchdog ? GW_OK : rc;
}
