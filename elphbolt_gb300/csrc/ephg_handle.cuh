// ephg_handle.cuh - the library handle (internal; the C ABI sees an opaque pointer).
#pragma once
#include <mutex>
#include <vector>

#include "../../include/ephg.h"
#include "ephg_kernels.cuh"
#include "ephg_tc.cuh"
#include "ephg_ws.cuh"

// Resident Wannier data of one crystal on one device, its stream, workspace
// and error word.
struct ephg_handle {
  int device = 0;
  cudaStream_t st = nullptr;
  int nw = 0, nb = 0, nwsk = 0, nwsq = 0, nwsg = 0, nat = 0;
  int cq[3] = {0, 0, 0};
  double lattvecs[9];
  std::vector<double> masses_h;
  std::vector<double> basis_h;   // (3,nat) crystal coordinates
  int64_t Nn = 0;   // nw*nw*nb*nwsg, the stage-A row length
  // resident device data
  int *Rk = nullptr, *Rq = nullptr, *Rg = nullptr;         // (n,3) int
  double *degk = nullptr, *degq = nullptr, *degg = nullptr;
  double2 *Hext = nullptr;   // [Re][4*nw*nw]: H, i rx H, i ry H, i rz H
  double2 *Hbox = nullptr;   // H(Re) / deg(Re) on the box of Re coordinates [hlo, hlo + hext) (mesh Fourier sums)
  int hlo[3] = {0, 0, 0}, hext[3] = {1, 1, 1};
  double2 *Dbox = nullptr;   // mass-normalised D terms on the box of wrapped cell vectors [dlo, dlo + dext)
  int dlo[3] = {0, 0, 0}, dext[3] = {1, 1, 1};
  double2 *graw = nullptr;   // epmatwp order (i,j,Re,s,Rp)
  double2 *G64 = nullptr;    // stage-A matrix [Re][Nn]
  double *masses = nullptr;
  // phonon wrap terms
  int *pair_off = nullptr, *ent_iuc = nullptr, *ent_woff = nullptr, *wrapR = nullptr;
  double *ent_rden = nullptr, *rcartq = nullptr;
  double2 *D = nullptr;
  ephg::PhTerms terms;
  int *kposk = nullptr, *kposq = nullptr;   // split-form contraction order (far cells first)
  int *err = nullptr;        // device error word
  ephg::Workspace ws;
  ephg::tc::SplitOperands split;   // split-TF32 operand planes (lazy)
  ephg::LaunchTimer timer_a, timer_b;   // device time of the contraction launches of the last request
  int64_t launches = 0;
  int64_t resident_bytes = 0;   // device bytes taken by ephg_create (Wannier data, tables)
  std::mutex split_mu;          // guards the one-time build of `split`
  // polar crystals (ephg_set_polar): the long-range terms' device data
  bool polar_on = false;
  ephg::PolarDev polar;
  double *polar_G = nullptr, *polar_Gcell = nullptr, *polar_born = nullptr, *polar_tau = nullptr;
  double2 *polar_Da = nullptr;
  // crystal symmetry (ephg_set_symmetry): real-space rotations (3,3,n), crystal coordinates
  std::vector<int64_t> sym_rot;
};

namespace ephg {
// Where a rate request runs: stream, device error word, workspace, timers and
// launch counter.  The handle's own fields form the default view
// (ephg_el_rates); the serving loop gives each of its slots one of its own, so
// that requests on one crystal overlap on the device.  The crystal's resident
// data is shared read-only.
struct ExecView {
  cudaStream_t st;
  int *err;
  Workspace *ws;
  LaunchTimer *ta, *tb;
  int64_t *launches;
  int chunk_us = 0;   // > 0: persistent kernels run as launches of about this length (serving)
  Yield yield;        // called between chunks and stages (serving); no-op by default
  tc::BatchMember bm;                        // batched form: the member of a grouped-launch batcher
  int64_t chunk_bytes = (int64_t)1 << 31;    // per-chunk GEMM output bound of the generic split path
};
// The phonon side of a rate request (ephg_ph_rates): the ph-e rates (N, nb) and
// the optional per-vertex Y list, formed in the same sweep as the electron side.
struct PhOut {
  double *rates_phe;
  double *y;
  double spindeg;
};
// A caller's |g|^2 vertex list to average over degenerate subspaces
// (ephg_g2_average_degenerate) instead of running the contractions.
struct DegAvgReq {
  double *g2;
  int64_t nv;
  int mode;
  double thres;
};
// Parameter sets of a merged request (ephg_el_rates_sets): the request is set
// 0; reqs[1..n-1] differ from it only in T, sigma and chempot, and rates[p]
// receives set p's rates (rates[0] is el_rates_view's own `rates`).
struct SetsOut {
  int n;
  const ephg_rate_request *reqs;
  double *const *rates;
};
// ph == nullptr: the electron side only (ephg_el_rates); otherwise rates and
// indexlist may be NULL.  avg != nullptr: the request's set-up only, then the
// averaging of avg->g2 (rates and indexlist may be NULL).  sets != nullptr:
// the electron side under every set (not with ph, avg or vertex lists).
int el_rates_view(ephg_handle *h, const ExecView &x, const ephg_rate_request *req, double *rates,
                  int64_t *indexlist, ephg_rate_stats *stats, double *g2, double *xplus, double *xminus, int64_t cap,
                  const PhOut *ph = nullptr, const DegAvgReq *avg = nullptr, const SetsOut *sets = nullptr);
// reqs[0..n-1] may share one contraction: equal but for T, sigma and chempot,
// each with valid T / sigma.  Returns 0 or EPHG_ERR_ARG with the reason recorded.
int check_sets(int64_t n, const ephg_rate_request *reqs);
// record a failure message for ephg_last_error() and return code
int api_fail(int code, const char *fmt, ...);
// read, clear and translate the handle's device error word
int api_check_err(ephg_handle *h);
}  // namespace ephg
