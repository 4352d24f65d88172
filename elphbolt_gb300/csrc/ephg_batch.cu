// ephg_batch.cu - the batched form: many rate requests, on many crystals, solved together.
//
// The reference answers one request on one crystal per run.  Here n requests
// (each against its own resident crystal handle) run on up to nslots execution
// slots at once, one host thread, stream, device error word and workspace per
// slot, largest estimated work first so that the long requests do not start
// last.  The split form's generic contractions of the running requests meet in
// rounds through a GemmBatcher (ephg_tc.cu): when every request inside a
// contraction stage has reached its next GEMM, those GEMMs run as one
// persistent tcgen05 launch over all their tiles, whatever their crystals and
// shapes.  Small requests then share the SMs with large ones inside one launch
// instead of queueing launch after launch, and the host work of one request
// (set-up, window compaction, its reads of sizes) overlaps the others' kernels.
//
// The slots' workspaces share an HBM budget: every growth reserves its bytes
// first; a request whose growth is refused gives its slot's workspace back and
// runs again after the others, alone, with the whole budget.  Each result is
// the same as the request run alone: the kernels and their chunking are the
// same, only the launches that carry them differ.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ephg.h"
#include "../../include/ephg_debug.h"
#include "ephg_gate.cuh"
#include "ephg_handle.cuh"

namespace {

struct Budget {
  std::mutex mu;
  int64_t budget = 0, reserved = 0, peak = 0;
};

bool reserve(void *ctx, int64_t delta) {
  Budget *b = (Budget *)ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (delta > 0 && b->reserved + delta > b->budget) return false;
  b->reserved += delta;
  b->peak = std::max(b->peak, b->reserved);
  return true;
}

struct Slot {
  cudaStream_t st = nullptr;
  int *err = nullptr;
  ephg::Workspace ws;
  ephg::LaunchTimer ta, tb;
  int64_t launches = 0;
};

void release_slot(Slot &s, Budget &b) {
  std::lock_guard<std::mutex> lk(b.mu);
  b.reserved -= (int64_t)s.ws.total();
  s.ws.release();
}

// relative cost of a request: window-independent, for the largest-first order
double work(const ephg_handle *h, const ephg_rate_request &r) {
  const double N = (double)r.mesh[0] * (double)r.mesh[1] * (double)r.mesh[2];
  return N * N * (double)h->nw * h->nw * h->nb * (double)h->nwsq;
}

}  // namespace

extern "C" int ephg_el_rates_batch(int64_t n, ephg_handle *const *crystals, const ephg_rate_request *reqs,
                                   double *const *rates, int64_t *const *indexlists, ephg_rate_stats *stats,
                                   int *status, const ephg_batch_opts *opts, ephg_batch_stats *bstats) {
  using ephg::api_fail;
  const auto t_start = std::chrono::steady_clock::now();
  if (n <= 0 || n > (1 << 20) || !crystals || !reqs || !rates || !indexlists || !status)
    return api_fail(EPHG_ERR_ARG, "el_rates_batch: bad arguments");
  for (int64_t i = 0; i < n; ++i)
    if (!crystals[i] || !rates[i] || !indexlists[i])
      return api_fail(EPHG_ERR_ARG, "el_rates_batch: request %lld has a null crystal or output", (long long)i);
  const int dev = crystals[0]->device;
  for (int64_t i = 1; i < n; ++i)
    if (crystals[i]->device != dev) return api_fail(EPHG_ERR_ARG, "el_rates_batch: crystals on different devices");
  int nslots = opts && opts->nslots > 0 ? (int)std::min<int64_t>(opts->nslots, 1 << 30) : 8;
  if (nslots > 64) return api_fail(EPHG_ERR_ARG, "el_rates_batch: nslots must be 1..64");
  nslots = (int)std::min<int64_t>(nslots, n);
  const bool grouped = !opts || opts->grouped != 0;
  if (cudaSetDevice(dev) != cudaSuccess) return api_fail(EPHG_ERR_CUDA, "el_rates_batch: no device");
  Budget budget;
  if (opts && opts->hbm_budget_bytes > 0) {
    budget.budget = opts->hbm_budget_bytes;
  } else {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return api_fail(EPHG_ERR_CUDA, "el_rates_batch: cudaMemGetInfo");
    budget.budget = (int64_t)(0.8 * (double)fr);
  }
  // per-chunk GEMM outputs: a 48th of the budget (a request holds about two
  // chunks, so eight at once take a third of it), within [64 MB, 2 GB]
  const int64_t chunk_bytes =
      std::max<int64_t>((int64_t)1 << 26, std::min<int64_t>((int64_t)1 << 31, budget.budget / 48));

  std::vector<Slot> slots(nslots);
  for (auto &s : slots) {
    if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void **)&s.err, sizeof(int)) != cudaSuccess || cudaMemset(s.err, 0, sizeof(int)) != cudaSuccess) {
      for (auto &q : slots) {
        if (q.st) cudaStreamDestroy(q.st);
        if (q.err) cudaFree(q.err);
      }
      return api_fail(EPHG_ERR_CUDA, "el_rates_batch: slot set-up failed");
    }
    s.ws.st = s.st;
    s.ws.grow = reserve;
    s.ws.grow_ctx = &budget;
  }
  ephg::tc::GemmBatcher *gb = grouped ? ephg::tc::batcher_create(nslots) : nullptr;
  if (grouped && !gb) {
    for (auto &q : slots) {
      cudaStreamDestroy(q.st);
      cudaFree(q.err);
    }
    return api_fail(EPHG_ERR_CUDA, "el_rates_batch: batcher set-up failed");
  }

  std::vector<int64_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return work(crystals[a], reqs[a]) > work(crystals[b], reqs[b]);
  });
  std::vector<std::string> msg(n);
  std::vector<int64_t> retry;
  std::mutex retry_mu;
  std::atomic<int64_t> next{0};
  auto view_of = [&](int w, bool batched) {
    ephg::ExecView x{slots[w].st, slots[w].err, &slots[w].ws, &slots[w].ta, &slots[w].tb, &slots[w].launches};
    x.chunk_bytes = chunk_bytes;
    if (batched && gb) {
      x.bm.gb = gb;
      x.bm.id = w;
    }
    return x;
  };
  auto run_one = [&](int w, int64_t i, bool batched) {
    const ephg::ExecView x = view_of(w, batched);
    int rc = ephg::el_rates_view(crystals[i], x, &reqs[i], rates[i], indexlists[i], stats ? &stats[i] : nullptr,
                                 nullptr, nullptr, nullptr, 0);
    if (rc != EPHG_OK) msg[i] = ephg_last_error();
    return rc;
  };
  auto worker = [&](int w) {
    cudaSetDevice(dev);
    for (;;) {
      const int64_t k = next.fetch_add(1);
      if (k >= n) break;
      const int64_t i = order[k];
      const int rc = run_one(w, i, true);
      if (rc == EPHG_ERR_NOMEM) {   // give the slot's workspace back; run it alone later
        cudaStreamSynchronize(slots[w].st);
        release_slot(slots[w], budget);
        std::lock_guard<std::mutex> lk(retry_mu);
        retry.push_back(i);
      } else {
        status[i] = rc;
      }
    }
    if (gb) ephg::tc::batcher_deactivate(ephg::tc::BatchMember{gb, w});
  };
  std::vector<std::thread> th;
  for (int w = 0; w < nslots; ++w) th.emplace_back(worker, w);
  for (auto &t : th) t.join();
  // requests that did not fit beside the others: alone, with the whole budget
  if (!retry.empty()) {
    for (auto &s : slots) {
      cudaStreamSynchronize(s.st);
      release_slot(s, budget);
    }
    std::sort(retry.begin(), retry.end());
    for (int64_t i : retry) {
      status[i] = run_one(0, i, false);
      cudaStreamSynchronize(slots[0].st);
      release_slot(slots[0], budget);
    }
  }
  int gerr = 0;
  int64_t gl = 0, gp = 0, gt = 0, gm = 0;
  if (gb) {
    gerr = ephg::tc::batcher_device_error(gb);
    ephg::tc::batcher_stats(gb, &gl, &gp, &gt, &gm);
    ephg::tc::batcher_destroy(gb);
  }
  for (auto &s : slots) {
    cudaStreamSynchronize(s.st);
    release_slot(s, budget);
    cudaStreamDestroy(s.st);
    cudaFree(s.err);
  }
  if (gerr & ephg::DERR_TIMEOUT)   // a grouped launch gave up a bounded wait: none of its outputs can be trusted
    for (int64_t i = 0; i < n; ++i)
      if (status[i] == EPHG_OK && reqs[i].precision == EPHG_PREC_SPLIT_TF32) {
        status[i] = EPHG_ERR_TIMEOUT;
        msg[i] = "grouped tcgen05 GEMM: a bounded mbarrier wait gave up";
      }
  const double wall_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  int64_t failed = 0, verts = 0, first_bad = -1;
  for (int64_t i = 0; i < n; ++i) {
    if (status[i] != EPHG_OK) {
      ++failed;
      if (first_bad < 0) first_bad = i;
    } else if (stats) {
      verts += stats[i].vertices;
    }
  }
  if (bstats) {
    bstats->requests = n;
    bstats->failed = failed;
    bstats->vertices = verts;
    bstats->wall_ms = wall_ms;
    bstats->vertices_per_s = wall_ms > 0 ? (double)verts / (wall_ms * 1e-3) : 0.0;
    bstats->group_launches = gl;
    bstats->group_problems = gp;
    bstats->group_tiles = gt;
    bstats->max_group = gm;
    bstats->retried_alone = (int64_t)retry.size();
    bstats->peak_workspace_bytes = budget.peak;
  }
  if (first_bad >= 0)
    return api_fail(status[first_bad], "el_rates_batch: request %lld: %s", (long long)first_bad,
                    msg[first_bad].c_str());
  return EPHG_OK;
}

// The round logic of the grouped launches (ephg::RoundGate) under host
// threads only: members alternate active stretches of 1-4 submissions, with
// random pauses, and inactive stretches; some become active by submitting.
// The launch callback checks that each member's items arrive once each, in
// order; each submit checks that its item was launched before it returned.
extern "C" int ephg_debug_batcher_selftest(int nmembers, int iters, uint64_t seed, int64_t *rounds,
                                           int64_t *max_group) {
  using ephg::api_fail;
  if (nmembers < 1 || nmembers > 64 || iters < 1) return api_fail(EPHG_ERR_ARG, "batcher_selftest: bad arguments");
  struct Item {
    int64_t seq;
  };
  struct Shared {
    std::mutex mu;
    std::condition_variable cv;
    std::vector<int64_t> launched;   // last sequence number launched, per member
    int64_t items = 0, max_group = 0, finished = 0;
    std::string why;
  };
  auto *sh = new Shared;   // leaked on a deadlock: the blocked threads still refer to it
  sh->launched.assign(nmembers, -1);
  auto *gate = new ephg::RoundGate<Item>(nmembers, [sh](std::vector<std::pair<int, Item>> &r) {
    std::lock_guard<std::mutex> lk(sh->mu);
    std::vector<char> seen(sh->launched.size(), 0);
    for (auto &it : r) {
      if (seen[it.first]) sh->why = "a member has two items in one round";
      seen[it.first] = 1;
      if (it.second.seq != sh->launched[it.first] + 1) sh->why = "a member's items launched out of order or lost";
      sh->launched[it.first] = it.second.seq;
    }
    sh->items += (int64_t)r.size();
    sh->max_group = std::max<int64_t>(sh->max_group, (int64_t)r.size());
    return 0;
  });
  std::vector<std::thread> th;
  std::vector<int64_t> submitted(nmembers, 0);
  for (int w = 0; w < nmembers; ++w)
    th.emplace_back([=, &submitted] {
      std::mt19937_64 rng(seed * 1000003ull + (uint64_t)w);
      int64_t seq = 0;
      for (int it = 0; it < iters; ++it) {
        if (rng() & 1) gate->activate(w);
        const int k = 1 + (int)(rng() % 4);
        for (int j = 0; j < k; ++j) {
          std::this_thread::sleep_for(std::chrono::microseconds(rng() % 200));
          const int rc = gate->submit(w, Item{seq});
          std::lock_guard<std::mutex> lk(sh->mu);
          if (rc != 0) sh->why = "submit returned an error";
          if (sh->launched[w] < seq) sh->why = "submit returned before its round was launched";
          ++seq;
        }
        gate->deactivate(w);
        std::this_thread::sleep_for(std::chrono::microseconds(rng() % 300));
      }
      submitted[w] = seq;
      std::lock_guard<std::mutex> lk(sh->mu);
      ++sh->finished;
      sh->cv.notify_all();
    });
  bool done;
  {
    std::unique_lock<std::mutex> lk(sh->mu);
    done = sh->cv.wait_for(lk, std::chrono::seconds(60), [&] { return sh->finished == nmembers; });
  }
  if (!done) {   // a deadlock: the members stay blocked; report it and leave them be
    for (auto &t : th) t.detach();
    return api_fail(EPHG_ERR_TIMEOUT, "batcher_selftest: members still blocked after 60 s");
  }
  for (auto &t : th) t.join();
  int64_t total = 0;
  for (int64_t x : submitted) total += x;
  const uint64_t nr = gate->rounds();
  std::string why = sh->why;
  const int64_t items = sh->items, mg = sh->max_group;
  delete gate;
  delete sh;
  if (rounds) *rounds = (int64_t)nr;
  if (max_group) *max_group = mg;
  if (!why.empty()) return api_fail(EPHG_ERR_INDEX, "batcher_selftest: %s", why.c_str());
  if (items != total)
    return api_fail(EPHG_ERR_INDEX, "batcher_selftest: %lld items launched of %lld submitted", (long long)items,
                    (long long)total);
  return EPHG_OK;
}
