// Launch-shape autotuner of the FRU stage kernels.
//
// A stage lasts as long as its slowest FRU's chain of FP64 (or FP32)
// instructions, and how many FRUs share a warp and how many warps share a
// block decides how those chains share the SM sub-partitions' issue slots.
// Which shape is fastest depends on the cell size, the precision and how many
// cells run at once, so the tuner measures it: it saves the cells' complete
// state (FRU Ca, channels, MT19937 words and positions), runs the same short
// window of the real workload once per candidate from that state, restores
// the state and keeps the fastest candidate.  Candidates:
//   - 4 lanes per FRU (8 FRUs per warp) with 1, 2, 4 or 8 warps per block;
//   - 1 lane per FRU (32 FRUs per warp), FP64 cells with the reference PCa
//     only, single-cell or per-stream runs only;
//   - packed launches (4 lanes per FRU, FRUs taken from a queue) with a half,
//     a quarter or an eighth as many warps as the cell has 8-FRU groups (16,
//     32 or 64 FRUs per warp on average), not in a batch.
// Every candidate computes the same bits (per-FRU arithmetic is the same and
// the flux sums use one fixed order), so tuning never changes a result.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <chrono>
#include <new>
#include <vector>

#include "gw_ctx_impl.h"
#include "gw_fru.h"

extern "C" int gw_internal_error(int code, const char* msg);
extern "C" int gw_batch_set_warps(gw_batch* b, int warps);

namespace {

struct Saved {
  std::vector<double> frus;
  std::vector<int> ltype, ryr, ito2, mti;
  std::vector<uint32_t> mt;
};

int save_cell(gw_ctx* c, Saved& s) {
  const size_t n = (size_t)gw_nfru(c);
  try {
    s.frus.resize(5 * n);
    s.ltype.resize(8 * n);
    s.ryr.resize(20 * n);
    s.ito2.resize(4 * n);
    s.mti.resize(n);
    s.mt.resize(624 * n);
  } catch (const std::bad_alloc&) {
    return gw_internal_error(GW_ENOMEM, "gw_autotune: host copy of the cell state does not fit");
  }
  return gw_download(c, s.frus.data(), s.ltype.data(), s.ryr.data(), s.ito2.data(), s.mti.data(), s.mt.data());
}

int restore_cell(gw_ctx* c, const Saved& s) {
  return gw_upload(c, s.frus.data(), s.ltype.data(), s.ryr.data(), s.ito2.data(), s.mti.data(), s.mt.data());
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" int gw_autotune(int n, gw_ctx** cells, const gw_settings* sets, const double* t, const double* states,
                           const double* oldsteps, double window_ms, gw_batch* batch, int* lanes_out,
                           int* warps_out, double* ms_out) {
  if (n <= 0 || !cells || !sets || !t || !states || !oldsteps || !(window_ms > 0.0))
    return gw_internal_error(GW_EINVAL, "gw_autotune: bad argument");
  bool one_lane_ok = !batch;
  for (int i = 0; i < n; i++) {
    if (!cells[i]) return gw_internal_error(GW_EINVAL, "gw_autotune: null cell");
    one_lane_ok = one_lane_ok && cells[i]->precision == 0 && cells[i]->pca_scale == 1.0;
  }
  std::vector<Saved> saved(n);
  std::vector<int> lanes0(n), warps0(n), pack0(n);
  for (int i = 0; i < n; i++) {
    int rc = save_cell(cells[i], saved[i]);
    if (rc) return rc;
    lanes0[i] = cells[i]->fru_lanes;
    warps0[i] = cells[i]->stage_warps;
    pack0[i] = cells[i]->packed_warps;
  }
  struct Cand {
    int lanes, warps, pack_div;  // pack_div > 0: packed, groups / pack_div warps
  };
  const Cand cands[GW_TUNE_CANDIDATES] = {{4, 1, 0}, {4, 2, 0}, {4, 4, 0}, {4, 8, 0},
                                          {1, 1, 0}, {4, 1, 2}, {4, 1, 4}, {4, 1, 8}};
  auto pack_warps = [&](int i, const Cand& k) {
    const int groups = (gw_nfru(cells[i]) + 7) / 8;
    return k.pack_div ? (groups + k.pack_div - 1) / k.pack_div : 0;
  };
  double best = 1e300;
  int best_i = 0, rc = GW_OK;
  std::vector<double> tt(n), st(37 * (size_t)n), os(n);
  const int nsteps = (int)(window_ms / sets[0].time_step + 0.5) > 0 ? (int)(window_ms / sets[0].time_step + 0.5) : 1;
  for (int k = 0; k < GW_TUNE_CANDIDATES; k++) {
    if (ms_out) ms_out[k] = -1.0;
    if (cands[k].lanes == 1 && !one_lane_ok) continue;
    if (cands[k].pack_div && batch) continue;
    for (int i = 0; i < n && !rc; i++) {
      rc = restore_cell(cells[i], saved[i]);
      if (!rc) rc = gw_set_fru_lanes(cells[i], cands[k].lanes);
      if (!rc) rc = gw_set_stage_warps(cells[i], cands[k].warps);
      if (!rc) rc = gw_set_stage_packing(cells[i], pack_warps(i, cands[k]));
    }
    if (!rc && batch) rc = gw_batch_set_warps(batch, cands[k].warps);
    if (rc) break;
    memcpy(tt.data(), t, sizeof(double) * n);
    memcpy(st.data(), states, sizeof(double) * 37 * n);
    memcpy(os.data(), oldsteps, sizeof(double) * n);
    const double t0 = now_s();
    if (n == 1 && !batch)
      rc = gw_run(cells[0], &sets[0], tt.data(), st.data(), os.data(), nsteps, nullptr, nullptr, nullptr);
    else if (batch)
      rc = gw_batch_run(batch, n, cells, sets, tt.data(), st.data(), os.data(), nsteps, nullptr, nullptr);
    else
      rc = gw_run_concurrent(n, cells, sets, tt.data(), st.data(), os.data(), nsteps, nullptr, nullptr);
    const double el = (now_s() - t0) * 1e3;
    if (rc) break;
    if (ms_out) ms_out[k] = el;
    if (el < best) {
      best = el;
      best_i = k;
    }
  }
  // back to the saved state, with the winner (or, after an error, the
  // settings the cells had)
  for (int i = 0; i < n; i++) {
    int r2 = restore_cell(cells[i], saved[i]);
    if (!r2) r2 = gw_set_fru_lanes(cells[i], rc ? lanes0[i] : cands[best_i].lanes);
    if (!r2) r2 = gw_set_stage_warps(cells[i], rc ? warps0[i] : cands[best_i].warps);
    if (!r2) r2 = gw_set_stage_packing(cells[i], rc ? pack0[i] : pack_warps(i, cands[best_i]));
    if (!rc) rc = r2;
  }
  if (batch) {
    int r2 = gw_batch_set_warps(batch, rc ? 1 : cands[best_i].warps);
    if (!rc) rc = r2;
  }
  if (rc) return rc;
  if (lanes_out) *lanes_out = cands[best_i].lanes;
  if (warps_out) *warps_out = cands[best_i].pack_div ? -cands[best_i].pack_div : cands[best_i].warps;
  return GW_OK;
}
