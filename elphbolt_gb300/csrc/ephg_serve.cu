// ephg_serve.cu - the serving loop: RTA-rate requests against resident crystals.
//
// A server keeps a set of crystals (handles of ephg_create) resident on the
// device and answers ephg_rate_request's as they arrive.  It is a continuous
// batcher, not a queue alone: it owns `nslots` execution slots (a stream, a
// device error word, a request workspace and timers each), a worker thread per
// slot takes the oldest waiting request as soon as its slot is free, and the
// requests of different slots run concurrently on the device (on one crystal
// or several: the crystals' resident data is shared read-only).  One request's
// GPU work overlaps another's host steps and small kernels; each result is the
// same as that of the request run alone (the kernels are deterministic).
//
// Admission is by an HBM budget covering the crystals' resident data and the
// slots' workspaces: every growth of a slot's workspace reserves its bytes
// against the budget first (under the server's lock, so that concurrent
// requests cannot overrun it together).  ephg_submit refuses a request whose
// set-up arrays alone exceed what the budget leaves (EPHG_ERR_NOMEM).  A
// request whose workspace cannot be reserved makes the idle slots release
// their cached workspaces and tries again; if that is still too little it waits
// until no other request runs (no new request starts meanwhile), takes the
// whole budget, and fails with EPHG_ERR_NOMEM only if even that is too little.
//
// Scheduling is preemptive highest-response-ratio-next: a request's ratio is
// its age divided by its estimated isolated solve time (per crystal, a linear
// fit time = a + b x work, work = mesh points^2 x nw^2 nb N_Rp, over the
// requests that ran alone so far; a crystal without two such runs borrows the
// others' slope, and without any model the estimate is the work itself).  A
// free slot takes the waiting request of highest ratio.  Every served request
// runs its persistent contraction kernels as launches of about kChunkUs, and
// between launches and stages it reaches a yield point: it drains its stream
// there (the host never queues more than a launch ahead), and the GPU belongs
// to the running request of highest ratio; any other waits there, except an
// urgent one (under a quarter of the largest running request's work), which
// runs beside it on a high-priority stream.  A small
// request overtakes a large one after waiting about (the large one's ratio) x
// its own solve time, and a large one's ratio keeps growing until it is served
// again, so that slowdowns even out instead of piling up on either end.  A
// small request therefore gets the whole GPU within one launch of a large one
// instead of waiting for all of it, while the host steps of all running
// requests still overlap.
//
// Latency is wall time from ephg_submit to completion; the server reports p50 /
// p99 and the vertices/s of completed requests.  The queue, slots, admission
// and statistics are written against an executor interface: the library's
// executor runs ephg::el_rates_view on the slots; a test executor
// (ephg_debug_server_selftest) simulates service times and memory so that the
// host logic is checked without a GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/ephg.h"
#include "../../include/ephg_debug.h"
#include "ephg_handle.cuh"

namespace {

using clk = std::chrono::steady_clock;

struct Result {
  std::vector<double> rates;
  std::vector<int64_t> idx;
  ephg_rate_stats stats{};
};

constexpr int kChunkUs = 3000;      // served requests: persistent kernels in launches of about 3 ms

struct Executor {
  virtual ~Executor() {}
  virtual int ncrystals() const = 0;
  virtual double work(int c, const ephg_rate_request &r) const = 0;   // relative cost estimate
  virtual int64_t resident() const = 0;                 // device bytes of all crystals' resident data
  virtual int64_t cached(int slot) const = 0;           // device bytes of a slot's workspace
  virtual int64_t min_bytes(int c, const ephg_rate_request &r) const = 0;   // lower bound of a request's workspace
  virtual void set_grow(int slot, bool (*fn)(void *, int64_t), void *ctx) = 0;   // reservation hook of a workspace
  virtual void release(int slot) = 0;
  // reqs[0..n-1] on crystal c, equal but for T, sigma and chempot (one contraction); out[i] per request
  virtual int run(int slot, int c, const ephg_rate_request *reqs, int n, bool urgent, const ephg::Yield &y,
                  Result *out, std::string &msg) = 0;
  virtual void drain(int slot) = 0;   // wait for the slot's queued device work
};

struct Ticket {
  int crystal = 0;
  ephg_rate_request req{};
  int state = EPHG_TICKET_QUEUED;
  int rc = EPHG_OK;
  std::string msg;
  Result res;
  double work = 0.0;
  double est = 1.0;        // estimated isolated solve time (ms; the work itself without any time model)
  bool urgent = false;
  bool alone = true;       // no other request ran at any time while this one did
  std::vector<Ticket *> partners;   // queued requests merged into this one's run (it leads them)
  clk::time_point t_submit, t_done;
};

// Can b share a's contraction (ephg_el_rates_sets)?  Same crystal, mesh,
// window, delta and precision; both with a valid T (and sigma for the
// Gaussian), so that one bad request cannot fail another.
bool mergeable(const Ticket &a, const Ticket &b) {
  const ephg_rate_request &x = a.req, &y = b.req;
  auto valid = [](const ephg_rate_request &r) { return r.T > 0 && (r.delta_kind != 0 || r.sigma > 0); };
  return a.crystal == b.crystal && x.mesh[0] == y.mesh[0] && x.mesh[1] == y.mesh[1] && x.mesh[2] == y.mesh[2] &&
         x.enref == y.enref && x.fsthick == y.fsthick && x.delta_kind == y.delta_kind &&
         x.precision == y.precision && valid(x) && valid(y);
}

// Least-squares fit of isolated solve time (ms) against work, per crystal.
struct TimeModel {
  double n = 0, sw = 0, sl = 0, sww = 0, swl = 0;
  void add(double w, double l) {
    n += 1;
    sw += w;
    sl += l;
    sww += w * w;
    swl += w * l;
  }
  bool ready() const { return n >= 2 && n * sww - sw * sw > 0; }
  double slope() const { return (n * swl - sw * sl) / (n * sww - sw * sw); }
  double predict(double w) const {
    const double b = slope(), a = (sl - b * sw) / n;
    return std::max(0.0, a + b * w);
  }
};

}  // namespace

struct ephg_server {
  std::unique_ptr<Executor> ex;
  int nslots = 1;
  int64_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_idle;
  std::deque<int64_t> queue;
  std::unordered_map<int64_t, std::unique_ptr<Ticket>> tickets;
  int64_t next_id = 1;
  bool stop = false;
  int running = 0;                 // slots running a request (not counting one waiting for exclusivity)
  int excl_waiting = 0;            // slots waiting to take the whole budget: no new request starts meanwhile
  int excl_owner = -1;             // slot holding the whole budget
  int64_t reserved = 0;            // bytes reserved by all slots' workspaces
  int max_sets = EPHG_MAX_SETS;    // requests per merged run (1: no merging)
  std::vector<char> busy;          // slot runs a request
  std::vector<double> run_work;    // estimated work of each slot's running request (0: idle or waiting)
  std::vector<double> run_est;     // its estimated isolated time
  std::vector<Ticket *> run_ticket;
  std::vector<TimeModel> model;    // per crystal
  clk::time_point t0 = clk::now();
  std::condition_variable cv_gpu;  // the GPU owner changed
  struct YieldCtx {
    ephg_server *s;
    int slot;
  };
  std::vector<YieldCtx> yctx;

  static double ratio(const Ticket &t, clk::time_point now) {
    return std::chrono::duration<double, std::milli>(now - t.t_submit).count() / t.est;
  }
  // under mu: does `slot` run the request of highest ratio (ties: lower slot)?
  bool owns_gpu(int slot) const {
    const clk::time_point now = clk::now();
    const double mine = ratio(*run_ticket[slot], now);
    for (int o = 0; o < nslots; ++o)
      if (o != slot && run_work[o] > 0.0 && run_ticket[o]) {
        const double r = ratio(*run_ticket[o], now);
        if (r > mine || (r == mine && o < slot)) return false;
      }
    return true;
  }
  // under mu: estimated isolated solve time of a request
  double est_of(const Ticket &t) const {
    double e;
    if (model[t.crystal].ready()) {
      e = model[t.crystal].predict(t.work);
    } else {
      double b = 0.0;   // a crystal without a model borrows the others' mean slope
      int k = 0;
      for (const TimeModel &m : model)
        if (m.ready()) {
          b += std::max(0.0, m.slope());
          ++k;
        }
      e = k ? (b / k) * t.work : t.work;   // no model anywhere yet: the work itself
    }
    return std::max(e, 1e-3);
  }
  void rekey() {   // under mu, after a model changed
    for (int64_t id : queue) tickets[id]->est = est_of(*tickets[id]);
    for (int o = 0; o < nslots; ++o)
      if (run_ticket[o]) run_est[o] = run_ticket[o]->est = est_of(*run_ticket[o]);
    cv_gpu.notify_all();
  }
  // Launches are asynchronous, so without a check the host would queue a whole
  // request's device work at once, before a later small request could be let
  // in.  Every yield point drains the caller's stream (at most one chunk of a
  // few ms stays queued ahead, at the cost of a host round trip per chunk) and
  // the caller goes on only while it owns the GPU.
  void yield_point(int slot) {
    ex->drain(slot);
    std::unique_lock<std::mutex> lk(mu);
    // An urgent request (under a quarter of the largest running one's work, on a
    // high-priority stream) does not wait: its kernels take SMs as the others'
    // blocks and launches end, so small requests run beside large ones instead
    // of queueing for the GPU behind their response ratio (serving stream at 80%
    // load: p50 slowdown 1.95 -> 1.62, p90 4.6 -> 3.4, p99 about 7 either way).
    while (!stop && !(run_ticket[slot] && run_ticket[slot]->urgent) &&
           !owns_gpu(slot)) {   // ratios change with time: re-check on notice or every 2 ms
      cv_gpu.notify_all();
      cv_gpu.wait_for(lk, std::chrono::milliseconds(2));
    }
  }
  static void yield_fn(void *p) {
    YieldCtx *y = (YieldCtx *)p;
    y->s->yield_point(y->slot);
  }
  ephg::Yield hook(int slot) {
    ephg::Yield y;
    y.fn = &yield_fn;
    y.ctx = &yctx[slot];
    return y;
  }
  std::vector<std::thread> workers;
  // statistics
  std::vector<double> lat_ms;
  int64_t submitted = 0, completed = 0, failed = 0, rejected = 0, vertices = 0, peak = 0, merged = 0;
  bool any_submit = false;
  clk::time_point t_first, t_last;

  // reservation hook of the slots' workspaces (called without mu held)
  static bool grow_fn(void *p, int64_t delta) {
    ephg_server *s = (ephg_server *)p;
    std::lock_guard<std::mutex> lk(s->mu);
    if (delta > 0 && s->ex->resident() + s->reserved + delta > s->budget) return false;
    s->reserved += delta;
    s->peak = std::max(s->peak, s->ex->resident() + s->reserved);
    return true;
  }
  void release_slot(int o) {   // under mu; the slot is idle
    reserved -= ex->cached(o);
    ex->release(o);
  }

  // Run t on `slot` (called with running already counting it); if its workspace
  // cannot be reserved, idle slots give back theirs, then it runs alone.
  int execute(int slot, Ticket &t, std::unique_lock<std::mutex> &lk) {
    const int n = 1 + (int)t.partners.size();
    std::vector<ephg_rate_request> reqs{t.req};
    for (Ticket *o : t.partners) reqs.push_back(o->req);
    std::vector<Result> res(n);
    auto run = [&]() {
      lk.unlock();
      const int rc = ex->run(slot, t.crystal, reqs.data(), n, t.urgent, hook(slot), res.data(), t.msg);
      lk.lock();
      if (rc == EPHG_OK) {
        t.res = std::move(res[0]);
        for (int i = 1; i < n; ++i) t.partners[i - 1]->res = std::move(res[i]);
      }
      return rc;
    };
    int rc = run();
    if (rc != EPHG_ERR_NOMEM) return rc;
    bool freed = false;
    for (int o = 0; o < nslots; ++o)
      if (o != slot && !busy[o] && ex->cached(o) > 0) {
        release_slot(o);
        freed = true;
      }
    if (freed) {
      t.msg.clear();
      rc = run();
      if (rc != EPHG_ERR_NOMEM) return rc;
    }
    // exclusive: stop new starts, wait until no other slot runs, take the whole budget
    // (while waiting this slot neither runs nor owns the GPU)
    const double w = run_work[slot];
    run_work[slot] = 0.0;
    cv_gpu.notify_all();
    running--;
    excl_waiting++;
    cv_idle.notify_all();
    cv_idle.wait(lk, [&] { return excl_owner < 0 && running == 0; });
    excl_waiting--;
    excl_owner = slot;
    running++;
    run_work[slot] = w;
    for (int o = 0; o < nslots; ++o)
      if (o != slot) release_slot(o);   // idle: no other slot runs now
    t.msg.clear();
    rc = run();
    excl_owner = -1;
    cv_work.notify_all();
    cv_idle.notify_all();
    return rc;
  }

  void loop(int slot) {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_work.wait(lk, [&] { return stop || (excl_waiting == 0 && excl_owner < 0 && !queue.empty()); });
      if (stop) return;
      size_t pick = 0;   // highest ratio
      {
        const clk::time_point now = clk::now();
        for (size_t i = 1; i < queue.size(); ++i)
          if (ratio(*tickets[queue[i]], now) > ratio(*tickets[queue[pick]], now)) pick = i;
      }
      const int64_t id = queue[pick];
      queue.erase(queue.begin() + (std::ptrdiff_t)pick);
      Ticket *t = tickets[id].get();
      t->state = EPHG_TICKET_RUNNING;
      // queued requests that differ only in T, sigma and chempot share this run's contraction
      t->partners.clear();
      for (size_t i = 0; i < queue.size() && 1 + (int)t->partners.size() < max_sets;) {
        Ticket *o = tickets[queue[i]].get();
        if (mergeable(*t, *o)) {
          o->state = EPHG_TICKET_RUNNING;
          t->partners.push_back(o);
          queue.erase(queue.begin() + (std::ptrdiff_t)i);
        } else {
          ++i;
        }
      }
      if (!t->partners.empty()) t->alone = false;   // a merged run trains no time model
      double bigger = 0.0;
      for (int o = 0; o < nslots; ++o) bigger = std::max(bigger, run_work[o]);
      t->urgent = t->work < 0.25 * bigger;
      run_work[slot] = t->work;
      run_est[slot] = t->est;
      for (int o = 0; o < nslots; ++o)   // whatever runs now does not run alone
        if (run_ticket[o]) {
          run_ticket[o]->alone = false;
          t->alone = false;
        }
      run_ticket[slot] = t;
      busy[slot] = 1;
      running++;
      const int rc = execute(slot, *t, lk);
      running--;
      busy[slot] = 0;
      run_work[slot] = 0.0;
      run_ticket[slot] = nullptr;
      cv_gpu.notify_all();
      const clk::time_point now = clk::now();
      std::vector<Ticket *> group{t};
      group.insert(group.end(), t->partners.begin(), t->partners.end());
      for (Ticket *g : group) {
        g->t_done = now;
        g->rc = rc;
        if (rc == EPHG_OK) {
          g->state = EPHG_TICKET_DONE;
          completed++;
          merged += g != t;
          vertices += g->res.stats.vertices;
          lat_ms.push_back(std::chrono::duration<double, std::milli>(now - g->t_submit).count());
          t_last = now;
        } else {
          g->msg = t->msg;
          g->state = EPHG_TICKET_FAILED;
          failed++;
        }
      }
      if (rc == EPHG_OK && t->alone) {   // an isolated solve time
        model[t->crystal].add(t->work, std::chrono::duration<double, std::milli>(now - t->t_submit).count());
        rekey();
      }
      t->partners.clear();
      cv_done.notify_all();
      cv_idle.notify_all();
      cv_work.notify_all();
    }
  }
};

namespace {

// One execution slot of the library's executor.
struct Slot {
  cudaStream_t st = nullptr, st_hi = nullptr;   // normal and high priority
  int *err = nullptr;
  ephg::Workspace ws;
  ephg::LaunchTimer ta, tb;
  int64_t launches = 0;
};

// The library's executor: ephg::el_rates_view on resident handles, one slot per worker.
struct HandleExecutor : Executor {
  std::vector<ephg_handle *> hs;
  std::vector<std::unique_ptr<Slot>> slots;
  int device = 0;
  ~HandleExecutor() override {
    cudaSetDevice(device);
    for (auto &s : slots) {
      if (s->st) cudaStreamSynchronize(s->st);
      if (s->st_hi) cudaStreamSynchronize(s->st_hi);
      s->ws.release();
      if (s->err) cudaFree(s->err);
      if (s->st) cudaStreamDestroy(s->st);
      if (s->st_hi) cudaStreamDestroy(s->st_hi);
    }
  }
  int init(int nslots) {
    device = hs[0]->device;
    for (ephg_handle *h : hs)
      if (h->device != device) return ephg::api_fail(EPHG_ERR_ARG, "server_create: crystals on different devices");
    cudaSetDevice(device);
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    for (int i = 0; i < nslots; ++i) {
      auto s = std::make_unique<Slot>();
      const bool ok = cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, least) == cudaSuccess;
      s->ws.st = s->st;
      if (!ok ||
          cudaStreamCreateWithPriority(&s->st_hi, cudaStreamNonBlocking, greatest) != cudaSuccess ||
          cudaMalloc(&s->err, sizeof(int)) != cudaSuccess || cudaMemset(s->err, 0, sizeof(int)) != cudaSuccess) {
        slots.push_back(std::move(s));
        return ephg::api_fail(EPHG_ERR_CUDA, "server_create: slot set-up: %s", cudaGetErrorString(cudaGetLastError()));
      }
      slots.push_back(std::move(s));
    }
    return EPHG_OK;
  }
  int ncrystals() const override { return (int)hs.size(); }
  double work(int c, const ephg_rate_request &r) const override {
    const ephg_handle *h = hs[c];
    const double N = (double)r.mesh[0] * r.mesh[1] * r.mesh[2];
    return N * N * h->nw * h->nw * h->nb * h->nwsq;
  }
  int64_t resident() const override {
    int64_t r = 0;
    for (ephg_handle *h : hs) r += h->resident_bytes + h->split.bytes;
    return r;
  }
  int64_t cached(int s) const override { return (int64_t)slots[s]->ws.total(); }
  int64_t min_bytes(int c, const ephg_rate_request &r) const override {
    const ephg_handle *h = hs[c];
    const int64_t N = r.mesh[0] * r.mesh[1] * r.mesh[2];
    // set-up arrays of el_rates on the whole mesh: H(k) + eigenvectors, D(q) + eigenvectors + u
    return N * (2 * (int64_t)h->nw * h->nw + 3 * (int64_t)h->nb * h->nb) * 16;
  }
  void set_grow(int s, bool (*fn)(void *, int64_t), void *ctx) override {
    slots[s]->ws.grow = fn;
    slots[s]->ws.grow_ctx = ctx;
  }
  void release(int s) override {
    cudaSetDevice(device);
    cudaStreamSynchronize(slots[s]->st);
    cudaStreamSynchronize(slots[s]->st_hi);
    slots[s]->ws.release();
  }
  void drain(int s) override {
    cudaSetDevice(device);
    cudaStreamSynchronize(slots[s]->st);
    cudaStreamSynchronize(slots[s]->st_hi);
  }
  int run(int s, int c, const ephg_rate_request *reqs, int n, bool urgent, const ephg::Yield &y, Result *out,
          std::string &msg) override {
    ephg_handle *h = hs[c];
    Slot &S = *slots[s];
    cudaSetDevice(device);
    const ephg_rate_request &r = reqs[0];
    const int64_t N = r.mesh[0] * r.mesh[1] * r.mesh[2];
    std::vector<double *> rates(n);
    for (int i = 0; i < n; ++i) {
      out[i].rates.assign((size_t)(N * h->nw), 0.0);
      rates[i] = out[i].rates.data();
    }
    out[0].idx.assign((size_t)N, 0);
    // the previous request of this slot ended with a host sync, so its buffers may move between the slot's streams
    S.ws.st = urgent ? S.st_hi : S.st;
    const ephg::ExecView x{S.ws.st, S.err, &S.ws, &S.ta, &S.tb, &S.launches, kChunkUs, y};
    const ephg::SetsOut so{n, reqs, rates.data()};
    const int rc = ephg::el_rates_view(h, x, &r, rates[0], out[0].idx.data(), &out[0].stats, nullptr, nullptr,
                                       nullptr, 0, nullptr, nullptr, n > 1 ? &so : nullptr);
    if (rc != EPHG_OK) msg = ephg_last_error();
    for (int i = 1; i < n; ++i) {   // the indexlist and stats are common to a merged run
      out[i].idx = out[0].idx;
      out[i].stats = out[0].stats;
    }
    return rc;
  }
};

// Test executor: service time and workspace simulated on the host.
struct FakeExecutor : Executor {
  int n = 1;
  double service_ms = 1.0;
  int64_t res_bytes = 0, per_request = 0;
  std::vector<int64_t> ws;
  bool (*grow)(void *, int64_t) = nullptr;
  void *grow_ctx = nullptr;
  std::mutex m;
  int concurrent = 0, max_concurrent = 0;
  int ncrystals() const override { return n; }
  double work(int, const ephg_rate_request &r) const override { return (double)r.mesh[0] * r.mesh[1] * r.mesh[2]; }
  int64_t resident() const override { return res_bytes * n; }
  int64_t cached(int s) const override { return ws[s]; }
  int64_t min_bytes(int, const ephg_rate_request &r) const override {
    return per_request * r.mesh[0] * r.mesh[1] * r.mesh[2] / 1000;
  }
  void set_grow(int, bool (*fn)(void *, int64_t), void *ctx) override {
    grow = fn;
    grow_ctx = ctx;
  }
  void release(int s) override { ws[s] = 0; }
  void drain(int) override {}
  int merged_runs = 0;
  // simulated device time service_ms x (mesh / 8)^3, in four parts with yield points between them; a merged
  // run takes the time of one request, and request i's result is crystal + 1000 T_i
  int run(int s, int c, const ephg_rate_request *reqs, int nreq, bool, const ephg::Yield &y, Result *out,
          std::string &msg) override {
    const ephg_rate_request &r = reqs[0];
    const int64_t need = per_request * r.mesh[0] * r.mesh[1] * r.mesh[2] / 1000;
    if (need > ws[s]) {
      if (!grow(grow_ctx, need - ws[s])) {
        msg = "simulated workspace over budget";
        return EPHG_ERR_NOMEM;
      }
      ws[s] = need;
    }
    {
      std::lock_guard<std::mutex> g(m);
      max_concurrent = std::max(max_concurrent, ++concurrent);
    }
    const double us = service_ms * 1000.0 * (double)(r.mesh[0] * r.mesh[1] * r.mesh[2]) / 512.0;
    for (int part = 0; part < 4; ++part) {
      if (part) y();
      std::this_thread::sleep_for(std::chrono::microseconds((int64_t)(us / 4)));
    }
    {
      std::lock_guard<std::mutex> g(m);
      --concurrent;
      merged_runs += nreq > 1;
    }
    for (int i = 0; i < nreq; ++i) {
      out[i].stats = ephg_rate_stats{};
      out[i].stats.vertices = r.mesh[0] * r.mesh[1] * r.mesh[2];
      out[i].rates.assign(1, (double)c + 1000.0 * reqs[i].T);
      out[i].idx.assign(1, 1);
    }
    return EPHG_OK;
  }
};

ephg_server *make_server(std::unique_ptr<Executor> ex, int64_t budget, int nslots) {
  ephg_server *s = new ephg_server();
  s->ex = std::move(ex);
  s->nslots = nslots;
  s->budget = budget;
  s->busy.assign(nslots, 0);
  s->run_est.assign(nslots, 1.0);
  s->run_ticket.assign(nslots, nullptr);
  s->model.assign(s->ex->ncrystals(), TimeModel());
  s->run_work.assign(nslots, 0.0);
  for (int i = 0; i < nslots; ++i) s->yctx.push_back({s, i});
  for (int i = 0; i < nslots; ++i) s->ex->set_grow(i, &ephg_server::grow_fn, s);
  for (int i = 0; i < nslots; ++i) s->workers.emplace_back([s, i] { s->loop(i); });
  return s;
}

int submit(ephg_server *s, int crystal, const ephg_rate_request *req, int64_t *ticket) {
  if (!s || !req || !ticket) return ephg::api_fail(EPHG_ERR_ARG, "submit: null argument");
  if (crystal < 0 || crystal >= s->ex->ncrystals()) return ephg::api_fail(EPHG_ERR_ARG, "submit: bad crystal index");
  for (int i = 0; i < 3; ++i)
    if (req->mesh[i] <= 0) return ephg::api_fail(EPHG_ERR_ARG, "submit: bad mesh");
  std::lock_guard<std::mutex> lk(s->mu);
  const clk::time_point now = clk::now();
  if (!s->any_submit) {
    s->t_first = now;
    s->any_submit = true;
  }
  s->submitted++;
  const int64_t need = s->ex->min_bytes(crystal, *req), avail = s->budget - s->ex->resident();
  if (need > avail) {
    s->rejected++;
    return ephg::api_fail(EPHG_ERR_NOMEM, "submit: the request needs at least %lld device bytes; the budget leaves %lld",
                          (long long)need, (long long)avail);
  }
  auto t = std::make_unique<Ticket>();
  t->crystal = crystal;
  t->req = *req;
  t->work = s->ex->work(crystal, *req);
  t->t_submit = now;
  t->est = s->est_of(*t);
  const int64_t id = s->next_id++;
  s->tickets[id] = std::move(t);
  s->queue.push_back(id);
  *ticket = id;
  s->cv_work.notify_one();
  return EPHG_OK;
}

void fill_stats(ephg_server *s, ephg_server_stats *o) {
  std::lock_guard<std::mutex> lk(s->mu);
  *o = ephg_server_stats{};
  o->submitted = s->submitted;
  o->completed = s->completed;
  o->failed = s->failed;
  o->rejected = s->rejected;
  o->vertices = s->vertices;
  o->peak_device_bytes = s->peak;
  o->merged = s->merged;
  std::vector<double> l = s->lat_ms;
  std::sort(l.begin(), l.end());
  if (!l.empty()) {
    auto rank = [&](double q) { return l[(size_t)std::max(0.0, std::ceil(q * (double)l.size()) - 1.0)]; };
    o->p50_ms = rank(0.50);
    o->p99_ms = rank(0.99);
    o->max_ms = l.back();
    double m = 0.0;
    for (double x : l) m += x;
    o->mean_ms = m / (double)l.size();
    o->wall_s = std::chrono::duration<double>(s->t_last - s->t_first).count();
    o->vertices_per_s = o->wall_s > 0 ? (double)s->vertices / o->wall_s : 0.0;
  }
}

void destroy(ephg_server *s) {
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_idle.notify_all();
  s->cv_gpu.notify_all();
  for (auto &w : s->workers)
    if (w.joinable()) w.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto &kv : s->tickets)
      if (kv.second->state == EPHG_TICKET_QUEUED) {
        kv.second->state = EPHG_TICKET_FAILED;
        kv.second->rc = EPHG_ERR_ARG;
        kv.second->msg = "server destroyed before the request ran";
      }
  }
  s->cv_done.notify_all();
  delete s;
}

}  // namespace

extern "C" {

int ephg_server_create(ephg_handle *const *crystals, int ncrystals, int64_t hbm_budget_bytes, int nslots,
                       ephg_server **out) {
  if (!crystals || ncrystals <= 0 || !out || hbm_budget_bytes <= 0 || nslots < 1 || nslots > 16)
    return ephg::api_fail(EPHG_ERR_ARG, "server_create: bad arguments");
  *out = nullptr;
  auto ex = std::make_unique<HandleExecutor>();
  for (int c = 0; c < ncrystals; ++c) {
    if (!crystals[c]) return ephg::api_fail(EPHG_ERR_ARG, "server_create: null crystal handle");
    ex->hs.push_back(crystals[c]);
  }
  if (ex->resident() > hbm_budget_bytes)
    return ephg::api_fail(EPHG_ERR_NOMEM, "server_create: the crystals' resident data (%lld bytes) exceed the budget",
                          (long long)ex->resident());
  int rc = ex->init(nslots);
  if (rc) return rc;
  *out = make_server(std::move(ex), hbm_budget_bytes, nslots);
  return EPHG_OK;
}

int ephg_server_destroy(ephg_server *s) {
  if (s) destroy(s);
  return EPHG_OK;
}

int ephg_submit(ephg_server *s, int crystal, const ephg_rate_request *req, int64_t *ticket) {
  return submit(s, crystal, req, ticket);
}

int ephg_poll(ephg_server *s, int64_t ticket, int *state) {
  if (!s || !state) return ephg::api_fail(EPHG_ERR_ARG, "poll: null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return ephg::api_fail(EPHG_ERR_ARG, "poll: unknown ticket");
  *state = it->second->state;
  return EPHG_OK;
}

int ephg_wait(ephg_server *s, int64_t ticket, double *rates, int64_t *indexlist, ephg_rate_stats *stats,
              double *latency_ms) {
  if (!s) return ephg::api_fail(EPHG_ERR_ARG, "wait: null server");
  std::unique_ptr<Ticket> t;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return ephg::api_fail(EPHG_ERR_ARG, "wait: unknown ticket");
    Ticket *tp = it->second.get();
    s->cv_done.wait(lk, [&] { return tp->state == EPHG_TICKET_DONE || tp->state == EPHG_TICKET_FAILED; });
    t = std::move(it->second);
    s->tickets.erase(it);
  }
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(t->t_done - t->t_submit).count();
  if (t->state == EPHG_TICKET_FAILED) return ephg::api_fail(t->rc, "%s", t->msg.c_str());
  if (rates) std::copy(t->res.rates.begin(), t->res.rates.end(), rates);
  if (indexlist) std::copy(t->res.idx.begin(), t->res.idx.end(), indexlist);
  if (stats) *stats = t->res.stats;
  return EPHG_OK;
}

int ephg_server_set_merge(ephg_server *s, int max_sets) {
  if (!s || max_sets < 1 || max_sets > EPHG_MAX_SETS) return ephg::api_fail(EPHG_ERR_ARG, "server_set_merge: bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  s->max_sets = max_sets;
  return EPHG_OK;
}

int ephg_server_stats_get(ephg_server *s, ephg_server_stats *out) {
  if (!s || !out) return ephg::api_fail(EPHG_ERR_ARG, "server_stats: null argument");
  fill_stats(s, out);
  return EPHG_OK;
}

int ephg_debug_server_selftest(int nreq, int nslots, double service_ms, int64_t budget, int64_t per_request_bytes,
                               const int64_t *meshes, const double *temps, int max_sets, ephg_server_stats *out,
                               int *max_concurrent, double *lat_ms) {
  if (nreq <= 0 || nslots < 1 || !meshes || !out) return ephg::api_fail(EPHG_ERR_ARG, "selftest: bad arguments");
  auto ex = std::make_unique<FakeExecutor>();
  FakeExecutor *fx = ex.get();
  ex->n = 2;
  ex->service_ms = service_ms;
  ex->res_bytes = 1000;
  ex->per_request = per_request_bytes;
  ex->ws.assign(nslots, 0);
  ephg_server *s = make_server(std::move(ex), budget, nslots);
  if (max_sets >= 1 && max_sets <= EPHG_MAX_SETS) s->max_sets = max_sets;
  std::vector<std::pair<int64_t, int>> tk(nreq, {0, -1});   // (ticket, crystal) per request
  for (int i = 0; i < nreq; ++i) {
    ephg_rate_request r{};
    r.mesh[0] = r.mesh[1] = r.mesh[2] = meshes[i];
    if (temps) {   // a valid T (and sigma) makes the request mergeable
      r.T = temps[i];
      r.sigma = 0.01;
    }
    int64_t id = 0;
    if (submit(s, i % 2, &r, &id) == EPHG_OK) tk[i] = {id, i % 2};
    if (i == 0) std::this_thread::sleep_for(std::chrono::microseconds(200));   // the first one starts alone
  }
  int bad = 0;
  for (int i = 0; i < nreq; ++i) {
    double rate = -1.0, lat = -1.0;
    int64_t idx = 0;
    if (tk[i].second < 0) {
      if (lat_ms) lat_ms[i] = -1.0;
      continue;
    }
    const int rc = ephg_wait(s, tk[i].first, &rate, &idx, nullptr, &lat);
    // the fake writes the crystal index + 1000 T
    if (rc == EPHG_OK && rate != (double)tk[i].second + (temps ? 1000.0 * temps[i] : 0.0)) bad++;
    if (lat_ms) lat_ms[i] = rc == EPHG_OK ? lat : -1.0;
  }
  fill_stats(s, out);
  if (max_concurrent) *max_concurrent = fx->max_concurrent;
  destroy(s);
  return bad ? ephg::api_fail(EPHG_ERR_INDEX, "selftest: results went to the wrong ticket") : EPHG_OK;
}

}  // extern "C"
