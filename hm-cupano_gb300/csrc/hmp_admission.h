// hmp_admission.h -- admission policy of the stitch server (host only, no CUDA).
//
// The server keeps, per pano configuration, up to `max_instances` resident stitchers (tables,
// seam and pyramid scratch on the device); each runs one request at a time. Resident bytes are
// admitted against an HBM budget. For a pending request the policy answers, in order:
//   1. an idle resident instance of its configuration          -> use it;
//   2. room for one more instance (count and budget)            -> create one;
//   3. room after evicting idle instances, least recently used  -> evict them, then create;
//   4. otherwise                                               -> wait (the request stays queued).
// The dispatcher applies it to pending requests in arrival order but skips, rather than blocks
// behind, one that must wait, so that requests of other configurations keep flowing.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace hmp {

class AdmissionPolicy {
 public:
  struct Instance {
    int config = -1;
    bool busy = false;
    uint64_t last_used = 0;
    double bytes = 0;
    bool alive = false;
  };

  enum Kind { kUse, kCreate, kWait };
  struct Decision {
    Kind kind = kWait;
    int instance = -1;          // kUse: the instance to run on
    std::vector<int> evict;     // kCreate: instances to destroy first
  };

  AdmissionPolicy(double budget_bytes, int max_instances) : budget_(budget_bytes), max_instances_(max_instances) {}

  // `bytes` = device bytes one instance of `config` holds (known from a first instance, or an
  // estimate before it exists).
  Decision decide(int config, double bytes) const {
    Decision d;
    int count = 0;
    for (size_t i = 0; i < inst_.size(); ++i) {
      const Instance& s = inst_[i];
      if (!s.alive || s.config != config) continue;
      ++count;
      if (!s.busy && d.kind != kUse) {
        d.kind = kUse;
        d.instance = int(i);
      }
    }
    if (d.kind == kUse) return d;
    if (count >= max_instances_ || bytes > budget_) return d;  // kWait
    double free_bytes = budget_ - resident_;
    if (bytes <= free_bytes) {
      d.kind = kCreate;
      return d;
    }
    // Evict idle instances, least recently used first, until the new one fits.
    std::vector<int> idle;
    for (size_t i = 0; i < inst_.size(); ++i)
      if (inst_[i].alive && !inst_[i].busy) idle.push_back(int(i));
    for (size_t a = 1; a < idle.size(); ++a)
      for (size_t b = a; b > 0 && inst_[idle[b]].last_used < inst_[idle[b - 1]].last_used; --b) {
        const int t = idle[b];
        idle[b] = idle[b - 1];
        idle[b - 1] = t;
      }
    for (int i : idle) {
      if (bytes <= free_bytes) break;
      d.evict.push_back(i);
      free_bytes += inst_[i].bytes;
    }
    if (bytes <= free_bytes) {
      d.kind = kCreate;
      return d;
    }
    d.evict.clear();
    return d;  // kWait: busy instances hold the budget
  }

  // Book-keeping the server reports back.
  int add(int config, double bytes) {
    Instance s;
    s.config = config;
    s.bytes = bytes;
    s.alive = true;
    s.last_used = ++clock_;
    for (size_t i = 0; i < inst_.size(); ++i)
      if (!inst_[i].alive) {
        inst_[i] = s;
        resident_ += bytes;
        peak_ = resident_ > peak_ ? resident_ : peak_;
        return int(i);
      }
    inst_.push_back(s);
    resident_ += bytes;
    peak_ = resident_ > peak_ ? resident_ : peak_;
    return int(inst_.size()) - 1;
  }
  void remove(int i) {
    if (i < 0 || size_t(i) >= inst_.size() || !inst_[i].alive) return;
    resident_ -= inst_[i].bytes;
    inst_[i] = Instance{};
  }
  void acquire(int i) {
    inst_[i].busy = true;
    inst_[i].last_used = ++clock_;
  }
  void release(int i) { inst_[i].busy = false; }

  double resident() const { return resident_; }
  double peak() const { return peak_; }
  double budget() const { return budget_; }
  const std::vector<Instance>& instances() const { return inst_; }

 private:
  double budget_;
  int max_instances_;
  std::vector<Instance> inst_;
  double resident_ = 0, peak_ = 0;
  uint64_t clock_ = 0;
};

}  // namespace hmp
