// Persistent multi-cell kernel: every cell's FRU stages, flux reductions and
// Dormand-Prince 5(4) integrator steps run inside one launch, without host
// round trips and without lockstep rounds.
//
// The reference advances one cell per MPI job: rk54pd (rk_pd54m.c:29-345)
// calls distrib_simFRU (mpi_master.c:369-469) five or six times per attempt,
// and every call waits for the slowest FRU.  Here one resident grid serves
// all cells at once.  Each cell's integrator posts one "operation" at a time
// (a flux evaluation at an attempt's start, or an FRU stage over [t0, tf]);
// an operation has two phases:
//   FRU phase      (stages only) 4-lane groups of any warp take the cell's
//                  FRUs one at a time from a per-cell counter, advance them
//                  with the substep loop of the cleft kernels (advance4's
//                  substep_a / substep_b, warp-wide MT19937 regeneration) and
//                  store them;
//   reduction      whole warps take chunks of 32 8-FRU groups and form each
//                  group's flux (and output-average) partial sums exactly as
//                  the fixed-layout stage kernel does -- same lanes, same
//                  shuffle tree -- applying a pending save / resume for
//                  operations that do not advance; the warp that finishes
//                  the last chunk adds the partials in the fixed order of
//                  cell_finish, forms the currents, runs the cell's
//                  integrator step on the whole warp (dp_after_warp: the
//                  arithmetic of gw_dp.c, the 37-state vectors split over
//                  the lanes and fcn's exponentials one per lane) and posts
//                  the cell's next operation.
// A warp whose groups find nothing to take works on whatever else is open,
// so one cell's slowest FRU no longer holds the GPU: other cells' FRUs fill
// the idle lanes.  Every cell's arithmetic, reduction order and integrator
// are those of its single-cell run, so its results are the same bits alone,
// in any mix, and in the round-based device runner (gw_run_device).
//
// Waiting: a warp with nothing to do sleeps and checks a global progress
// counter (FRUs and chunks finished); if it has not moved for `wait_ns`
// (2 s by default; real operations take microseconds to milliseconds) the
// kernel sets an error status and every warp returns, so the context stays
// usable and the host reports the error.  No warp ever waits for a specific
// other warp, so the grid needs no co-residency guarantee; it is sized to the
// occupancy (one single-warp block per resident slot) all the same.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <new>
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

constexpr int kChunkGroups = 32;  // 8-FRU groups per reduction chunk (256 FRUs)
constexpr int kTakeFrus = 4;      // FRUs a 4-lane group takes at once (one counter update, one fence)
constexpr int kMaxCells = 1024;   // cells of one run (16 mask words)
constexpr unsigned kFull = 0xffffffffu;
enum : int { kStatusOk = 0, kStatusWatchdog = 3 };
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;

// Scheduling state of one cell.  `take` and `red_take` are reset only when
// their phase opens, so a warp that increments one of them late either gets
// an index past the end (nothing to do) or a valid index of a phase that is
// open, and it reads the operation's parameters after the increment.
struct PCell {
  unsigned long long take;  // next FRU of the open FRU phase (>= nfru: none)
  unsigned done;            // FRUs of the open operation stored
  unsigned red_take;        // next reduction chunk (>= nchunks: none)
  unsigned red_done;        // reduction chunks finished
  unsigned overflow;        // an FRU of the operation reached the substep limit
  int nchunks;
  int finished;
};

struct Args {
  const DevState* cells;
  DpCell* dp;
  PCell* pc;
  int ncells;
  unsigned* running;             // cells with output steps left
  unsigned long long* fru_mask;  // bit per cell: its FRU phase has FRUs left to take
  unsigned long long* red_mask;  // bit per cell: its reduction has chunks left to take
  int nwords;                    // 64-bit words of each mask
  unsigned long long* progress;  // FRUs and chunks finished
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

// ---- posting operations (one thread) -----------------------------------------------
// A cell's bit in a mask is set after its counter is reset (open), and the
// warp that finds the counter exhausted clears the bit and then looks at the
// counter again, setting the bit back if a new phase opened meanwhile; so a
// phase with work left always has its bit set.
__device__ __forceinline__ void mask_set(unsigned long long* m, int ci) {
  atomicOr(&m[ci >> 6], 1ull << (ci & 63));
}
__device__ __forceinline__ void mask_clear_fru(const Args& a, int ci) {
  atomicAnd(&a.fru_mask[ci >> 6], ~(1ull << (ci & 63)));
  __threadfence();
  if (vload(&a.pc[ci].take) < (unsigned long long)a.cells[ci].nfru) mask_set(a.fru_mask, ci);
}
__device__ __forceinline__ void mask_clear_red(const Args& a, int ci) {
  atomicAnd(&a.red_mask[ci >> 6], ~(1ull << (ci & 63)));
  __threadfence();
  if (vload(&a.pc[ci].red_take) < (unsigned)a.pc[ci].nchunks) mask_set(a.red_mask, ci);
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

static __device__ void open_reduction(const Args& a, int ci) {
  PCell& pc = a.pc[ci];
  pc.red_done = 0u;
  atomicExch(&pc.red_take, 0u);
  __threadfence();
  mask_set(a.red_mask, ci);
}

// Post the operation dp_after has just set up in the cell's DpCell.
static __device__ void post(const Args& a, int ci) {
  PCell& pc = a.pc[ci];
  pc.done = 0u;
  pc.overflow = 0u;
  __threadfence();
  if (a.dp[ci].sp.flags & kFlagAdvance) {
    atomicExch(&pc.take, 0ull);
    __threadfence();
    mask_set(a.fru_mask, ci);
  } else {
    open_reduction(a, ci);
  }
}

// ---- reduction ---------------------------------------------------------------------
// One 8-FRU group's partial sums into partials[grp * NV ..], by the whole
// warp in the lanes of the fixed-layout kernel (FRU grp*8 + lane/4, cleft
// lane%4): stage_body_fin's epilogue, with its save / resume handling for an
// operation that does not advance.
template <int NV>
__device__ __forceinline__ void reduce_group(const DevState& s, const StageParams& p, int grp, const cleft::Group& g,
                                             int lane) {
  const int f = grp * 8 + (lane >> 2);
  const bool active = f < s.nfru;
  const size_t nf = (size_t)s.stride;
  const bool apply = !(p.flags & kFlagAdvance);  // an advancing op applied them in its FRU phase
  double cajsr = 0.0, cass = 0.0;
  uint32_t w = 0u;
  int mti = 0;
  bool restore = false;
  if (active) {
    if (apply && (p.flags & kFlagResume)) {
      cajsr = s.frus_s[f];
      cass = s.frus_s[(g.c + 1) * nf + f];
      w = s.chan_s[g.c * nf + f];
      mti = s.mti_s[f];
      restore = (s.hold_epoch[f] == p.epoch);
    } else {
      cajsr = __ldcg(&s.frus[f]);
      cass = __ldcg(&s.frus[(g.c + 1) * nf + f]);
      w = __ldcg(&s.chan[g.c * nf + f]);
      mti = __ldcg(&s.mti[f]);
    }
    if (apply && (p.flags & kFlagSave)) {
      if (g.c == 0) {
        s.frus_s[f] = cajsr;
        s.mti_s[f] = mti;
      }
      s.frus_s[(g.c + 1) * nf + f] = cass;
      s.chan_s[g.c * nf + f] = w;
    }
  }
  if (apply) {
    if (active && restore) cleft::copy_row16(s.mt + (size_t)f * kMtStride, s.mt_hold + (size_t)f * kMtStride, g);
    if (active) {
      if (g.c == 0) {
        s.frus[f] = cajsr;
        s.mti[f] = mti;
      }
      s.frus[(g.c + 1) * nf + f] = cass;
      s.chan[g.c * nf + f] = w;
    }
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

// The cell's totals from its group partials in cell_finish's order, the
// currents, and the integrator step; then the next operation is posted (or
// the cell is done).  Whole warp; the integrator runs on lane 0.
template <int NV>
__device__ __forceinline__ void finish_op(const Args& a, int ci, int lane) {
  const DevState& s = a.cells[ci];
  DpCell& c = a.dp[ci];
  const int ngroups = (s.nfru + 7) >> 3;
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

// Take and reduce one chunk of cell ci's open reduction; false if none left.
static __device__ bool reduce_chunk(const Args& a, int ci, const cleft::Group& g, int lane) {
  PCell& pc = a.pc[ci];
  unsigned k = 0u;
  if (lane == 0) {
    k = atomicAdd(&pc.red_take, 1u);
    if (k >= (unsigned)pc.nchunks - 1u) mask_clear_red(a, ci);
  }
  k = __shfl_sync(kFull, k, 0);
  if (k >= (unsigned)pc.nchunks) return false;
  __threadfence();  // the operation's parameters and stored FRUs after the take
  const DevState& s = a.cells[ci];
  const StageParams& p = a.dp[ci].sp;
  const int ngroups = (s.nfru + 7) >> 3;
  const int g1 = min(ngroups, (int)(k + 1u) * kChunkGroups);
  const bool avg = (p.flags & kFlagAvg) != 0;
  for (int grp = (int)k * kChunkGroups; grp < g1; grp++) {
    if (avg) reduce_group<16>(s, p, grp, g, lane);
    else reduce_group<5>(s, p, grp, g, lane);
  }
  __threadfence();
  __syncwarp();
  unsigned last = 0u;
  if (lane == 0) {
    last = (atomicAdd(&pc.red_done, 1u) == (unsigned)pc.nchunks - 1u) ? 1u : 0u;
    atomicAdd(a.progress, 1ull);
  }
  last = __shfl_sync(kFull, last, 0);
  if (last) {
    if (avg) finish_op<16>(a, ci, lane);
    else finish_op<5>(a, ci, lane);
  }
  return true;
}

// A cell with reduction chunks left (warp-uniform; -1: none).
static __device__ int find_reduction(const Args& a, int from, int lane) {
  int ci = -1;
  if (lane == 0) ci = mask_pick(a.red_mask, a.nwords, a.ncells, from);
  return __shfl_sync(kFull, ci, 0);
}

// MT19937 regeneration of the rows whose draws run past word 624 in this
// substep, by the whole warp (regen_step of the cleft kernels, with each
// group's copy-on-twist target taken from its own cell).
__device__ __forceinline__ void regen_multi(cleft::StageCtx& sc, int lane, const cleft::Group& g, bool go, int mti,
                                            int etot, uint32_t epoch) {
  const bool cross = go && (mti + etot + 32 > kMtN);
  const unsigned cross_mask = __ballot_sync(kFull, cross && g.c == 0);
  const unsigned copy_mask = __ballot_sync(kFull, cross && g.c == 0 && *sc.my_hold_epoch != epoch);
  unsigned cm = cross_mask;
  while (cm) {
    const int l0 = __ffs(cm) - 1;
    cm &= cm - 1u;
    uint32_t* row = sc.rows + (l0 >> 2) * kMtSmemStride;
    const int fg = __shfl_sync(kFull, sc.f, l0);
    uint32_t* hold = (uint32_t*)__shfl_sync(kFull, (unsigned long long)sc.hold_base, l0);
    uint32_t* hold_ep = (uint32_t*)__shfl_sync(kFull, (unsigned long long)sc.hold_epoch_base, l0);
    const uint32_t ep = __shfl_sync(kFull, epoch, l0);
    __syncwarp();  // the group has read its old words
    cleft::complete_row(sc, lane, l0, row);
    if (copy_mask & (1u << l0)) {
      const uint4* s4 = reinterpret_cast<const uint4*>(row);
      uint4* d4 = reinterpret_cast<uint4*>(hold + (size_t)fg * kMtStride);
      for (int i = lane; i < kMtN / 4; i += 32) d4[i] = s4[i];
      if (lane == 0) hold_ep[fg] = ep;
    }
    cleft::regen32(row, lane);
  }
  if (cross) sc.dirty = true;
}

template <typename R>
__device__ __forceinline__ void persist_body(const Args& a) {
  using namespace cleft;
  extern __shared__ __align__(16) uint32_t mt_stage[];  // [8][kMtSmemStride] per warp
  const int lane = threadIdx.x & 31;
  const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  Group g;
  g.c = lane & 3;
  g.base = lane & ~3;
  g.mask = 0xfu << g.base;
  StageCtx sc;
  sc.p = nullptr;
  sc.rows = mt_stage + (threadIdx.x >> 5) * 8 * kMtSmemStride;
  sc.m = sc.rows + (lane >> 2) * kMtSmemStride;
  sc.hold_base = nullptr;
  sc.hold_epoch_base = nullptr;
  sc.my_hold_epoch = nullptr;
  sc.f = 0;
  sc.dirty = false;
  sc.start = 0;
  sc.src = nullptr;
  LaneStage<R> LS;
  Fru4<R> F;
  F.clk = {};
  F.jsr.set(0.0);
  F.ss.set(0.0);
  F.w = 0u;
  F.nsub = 0u;
  F.mti = 0;
  LS.tf = 0.0;
  LS.interval = 0.0;
  int ci = -1, f = -1, f_end = -1, nfru = 0, taken = 0;
  uint32_t epoch = 0u;
  bool ovf = false;
  const DevState* S = nullptr;
  int cursor = (warp * 8 + (lane >> 2)) % a.ncells;
  unsigned long long seen = 0ull, idle_since = 0ull;
  bool idle_clock = false;

  // load FRU ff of the group's operation into the group's lanes
  auto load = [&](int ff) {
    const StageParams& p = a.dp[ci].sp;
    f = ff;
    sc.f = ff;
    sc.my_hold_epoch = S->hold_epoch + ff;
    const size_t nf = (size_t)S->stride;
    bool restore = false;
    if (p.flags & kFlagResume) {
      F.jsr.set(S->frus_s[ff]);
      F.ss.set(S->frus_s[(g.c + 1) * nf + ff]);
      F.w = S->chan_s[g.c * nf + ff];
      F.mti = S->mti_s[ff];
      restore = (*sc.my_hold_epoch == epoch);
    } else {
      F.jsr.set(__ldcg(&S->frus[ff]));
      F.ss.set(__ldcg(&S->frus[(g.c + 1) * nf + ff]));
      F.w = __ldcg(&S->chan[g.c * nf + ff]);
      F.mti = __ldcg(&S->mti[ff]);
    }
    if (p.flags & kFlagSave) {
      if (g.c == 0) {
        S->frus_s[ff] = F.jsr.get();
        S->mti_s[ff] = F.mti;
      }
      S->frus_s[(g.c + 1) * nf + ff] = F.ss.get();
      S->chan_s[g.c * nf + ff] = F.w;
    }
    stage_row(sc, restore ? S->mt_hold + (size_t)ff * kMtStride : S->mt + (size_t)ff * kMtStride, F.mti, restore, g);
    sc.dirty = restore;
    F.nsub = 0u;
    fru_begin(F, LS);
  };
  // the next kTakeFrus FRUs of any open FRU phase (group-uniform; false: none)
  auto take = [&]() -> bool {
    int got_c = -1, got_f = -1;
    if (g.c == 0) {
      for (int tries = 0; tries < 4; tries++) {
        const int cj = mask_pick(a.fru_mask, a.nwords, a.ncells, cursor);
        if (cj < 0) break;
        const unsigned n = (unsigned)a.cells[cj].nfru;
        const unsigned idx = (unsigned)atomicAdd(&a.pc[cj].take, (unsigned long long)kTakeFrus);
        if (idx + kTakeFrus >= n) mask_clear_fru(a, cj);  // the phase has no FRUs left to take
        cursor = cj;
        if (idx >= n) continue;
        got_c = cj;
        got_f = (int)idx;
        break;
      }
    }
    got_c = __shfl_sync(g.mask, got_c, g.base);
    got_f = __shfl_sync(g.mask, got_f, g.base);
    if (got_c < 0) return false;
    __threadfence();  // the operation's parameters after the take
    ci = got_c;
    S = &a.cells[ci];
    nfru = S->nfru;
    f_end = min(nfru, got_f + kTakeFrus);
    taken = f_end - got_f;
    const StageParams& p = a.dp[ci].sp;
    lane_stage(p, g, LS);
    epoch = p.epoch;
    sc.p = &p;
    sc.hold_base = S->mt_hold;
    sc.hold_epoch_base = S->hold_epoch;
    ovf = false;
    load(got_f);
    return true;
  };
  // store the group's FRU and load the next one it holds; after its last,
  // count them done -- the group that completes a phase opens the reduction
  auto finish = [&]() {
    const size_t nf = (size_t)S->stride;
    if (sc.dirty) copy_row16(S->mt + (size_t)f * kMtStride, sc.m, g);
    if (g.c == 0) {
      S->frus[f] = F.jsr.get();
      S->mti[f] = F.mti;
      if (S->substeps) atomicAdd(S->substeps, (unsigned long long)F.nsub);
    }
    S->frus[(g.c + 1) * nf + f] = F.ss.get();
    S->chan[g.c * nf + f] = F.w;
    if (f + 1 < f_end) {
      __syncwarp(g.mask);
      load(f + 1);
      return;
    }
    __threadfence();
    __syncwarp(g.mask);
    unsigned last = 0u;
    if (g.c == 0) {
      PCell& pc = a.pc[ci];
      if (ovf) atomicOr(&pc.overflow, 1u);
      last = (atomicAdd(&pc.done, (unsigned)taken) + (unsigned)taken == (unsigned)nfru) ? 1u : 0u;
      if (last) {
        __threadfence();
        open_reduction(a, ci);
      }
      atomicAdd(a.progress, (unsigned long long)taken);
    }
    __syncwarp(g.mask);
    ci = -1;
    f = -1;
  };

  while (true) {
    // flags for the end of this iteration, loaded now so that their latency
    // hides behind the substep
    int st = kStatusOk;
    unsigned run = 1u;
    int red = 0;
    if (lane == 0) {
      st = vload(a.status);
      run = vload(a.running);
      for (int w = 0; w < a.nwords; w++) red |= vload(&a.red_mask[w]) != 0ull;
    }
    bool worked = false;
    // groups without an FRU take some
    if (ci < 0) take();
    const bool has = ci >= 0;
    bool go = has && F.clk.running(LS);
    if (go && F.nsub >= (1u << 22)) {
      ovf = true;
      go = false;
    }
    if (__any_sync(kFull, go)) {
      Sub4<R> Sb;
      Sb.etot = 0;
#pragma unroll
      for (int i = 0; i < kRyR; i++) Sb.exw[i] = 0u;
      Sb.p34 = R(0);
      if (go) substep_a(F, Sb, LS, g, sc);
      regen_multi(sc, lane, g, go, F.mti, Sb.etot, epoch);
      if (go) substep_b(F, Sb, LS, g, sc);
      worked = true;
    }
    if (has && !(go && F.clk.running(LS))) {
      finish();
      worked = true;
    }
    __syncwarp();
    st = __shfl_sync(kFull, st, 0);
    run = __shfl_sync(kFull, run, 0);
    if (st != kStatusOk) break;  // an error somewhere: every warp returns
    if (run == 0u && !__any_sync(kFull, ci >= 0)) break;  // every cell is done
    // reduction chunks: they are on a cell's critical path
    if (__shfl_sync(kFull, red, 0)) {
      const int rc = find_reduction(a, cursor, lane);
      if (rc >= 0) worked = reduce_chunk(a, rc, g, lane) || worked;
    }
    if (__any_sync(kFull, worked)) {
      idle_clock = false;
      continue;
    }
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

// Single-warp blocks: 191 registers and 19,968 B of MT staging per warp let
// ten warps share an SM, as many as the packed stage kernels run.
__global__ void __launch_bounds__(32, 10) persist_kernel_fp64(Args a) { persist_body<double>(a); }
__global__ void __launch_bounds__(32, 10) persist_kernel_mixed(Args a) { persist_body<float>(a); }

}  // namespace persist
}  // namespace gw

using gw::DpCell;
using gw::persist::PCell;

namespace {

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
    memset(&p, 0, sizeof p);
    p.take = (unsigned long long)c->d.nfru;  // no FRU phase open
    p.nchunks = ((c->d.nfru + 7) / 8 + gw::persist::kChunkGroups - 1) / gw::persist::kChunkGroups;
    p.red_take = 0u;                         // the first operation's reduction is open
  }
  const size_t ns = (size_t)n * n_steps;
  gw::DevState* dcells = nullptr;
  DpCell* ddp = nullptr;
  PCell* dpc = nullptr;
  // counters: [0] running, [3] status, [4] release; then progress, ops; the two cell masks
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
  const size_t smem = gw::kStageSmemPerWarp;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = mixed ? gw::stage_smem_attributes(gw::persist::persist_kernel_mixed)
              : gw::stage_smem_attributes(gw::persist::persist_kernel_fp64);
  if (e == cudaSuccess)
    e = mixed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gw::persist::persist_kernel_mixed, 32, smem)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gw::persist::persist_kernel_fp64, 32, smem);
  if (e == cudaSuccess && per_sm <= 0) e = cudaErrorInvalidConfiguration;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&dcells, sizeof(gw::DevState) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ddp, sizeof(DpCell) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dpc, sizeof(PCell) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dcnt, sizeof(int) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dmask, sizeof(unsigned long long) * 2 * nwords);
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
    // no FRU phase open; every cell's first operation (a flux) is in its reduction
    std::vector<unsigned long long> m(2 * nwords, 0ull);
    for (int i = 0; i < n; i++) m[nwords + (i >> 6)] |= 1ull << (i & 63);
    if (e == cudaSuccess) e = cudaMemcpy(dmask, m.data(), sizeof(unsigned long long) * m.size(), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(d64, 0, sizeof(unsigned long long) * 2);
  gw::persist::Args args;
  args.cells = dcells;
  args.dp = ddp;
  args.pc = dpc;
  args.ncells = n;
  args.running = (unsigned*)dcnt;
  args.fru_mask = dmask;
  args.red_mask = dmask + nwords;
  args.nwords = nwords;
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
