// ephg_gate.cuh - the round logic of the batched form's grouped launches, free of CUDA.
//
// n members (concurrently running requests, one host thread each).  A member is
// active while it may submit; submit(id, item) queues one item and blocks until
// the round that carries it has been launched.  A round is launched, by the
// thread that completes it, as soon as every active member has an item queued:
// either the last member to submit or a member that deactivates while the
// others wait.  The launch callback runs under the gate's lock with the round's
// items (in submission order) and returns the round's status, which every
// member of the round gets back from submit.
#pragma once
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <utility>
#include <vector>

namespace ephg {

template <class Item>
class RoundGate {
 public:
  using Launch = std::function<int(std::vector<std::pair<int, Item>> &)>;

  RoundGate(int n, Launch launch) : act_(n, 0), rc_(n, 0), launch_(std::move(launch)) {}

  void activate(int id) {
    std::lock_guard<std::mutex> lk(mu_);
    if (!act_[id]) {
      act_[id] = 1;
      ++active_;
    }
  }

  void deactivate(int id) {
    std::lock_guard<std::mutex> lk(mu_);
    if (!act_[id]) return;
    act_[id] = 0;
    --active_;
    if (!pend_.empty() && (int)pend_.size() == active_) launch_locked();
  }

  // An inactive member becomes active by submitting.
  int submit(int id, const Item &item) {
    std::unique_lock<std::mutex> lk(mu_);
    if (!act_[id]) {
      act_[id] = 1;
      ++active_;
    }
    pend_.emplace_back(id, item);
    const uint64_t my = round_;
    if ((int)pend_.size() == active_) launch_locked();
    else cv_.wait(lk, [&] { return round_ != my; });
    return rc_[id];
  }

  uint64_t rounds() const {
    std::lock_guard<std::mutex> lk(mu_);
    return round_;
  }

 private:
  void launch_locked() {
    const int rc = launch_(pend_);
    for (auto &p : pend_) rc_[p.first] = rc;
    pend_.clear();
    ++round_;
    cv_.notify_all();
  }
  mutable std::mutex mu_;
  std::condition_variable cv_;
  std::vector<char> act_;
  std::vector<int> rc_;
  std::vector<std::pair<int, Item>> pend_;
  int active_ = 0;
  uint64_t round_ = 0;
  Launch launch_;
};

}  // namespace ephg
