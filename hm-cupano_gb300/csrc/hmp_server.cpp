// hmp_server.cpp -- continuous-batching stitch server (include/hmpano.h, hmp_server_*). No
// counterpart in the reference, which stitches one configuration per process.
//
// Clients register pano configurations (host tables are copied) and submit requests: a
// configuration id, device input frames and a device canvas. A dispatcher thread owns the GPU
// side: it admits pending requests against the HBM budget (hmp_admission.h), keeps stitchers
// resident per configuration (tables, seam, pyramid scratch), launches each admitted request on
// a stream slot with room (each runs one request and holds the next queued behind it), and
// watches the requests' completion events. Requests that arrive while others
// are on the GPU start as soon as a slot and an instance are free, so their work overlaps on the
// device. Latency = observed completion - submission, host steady clock.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "hmp_admission.h"
#include "hmpano.h"

namespace {

using Clock = std::chrono::steady_clock;

hmp_status mk(int code, const char* msg) {
  hmp_status s;
  s.code = code;
  std::snprintf(s.message, sizeof(s.message), "%s", msg);
  return s;
}

struct ConfigEntry {
  hmp_config cfg{};
  std::vector<hmp_remap> remaps;
  std::vector<std::vector<uint16_t>> mx, my;
  std::vector<uint8_t> seam;
  double bytes = 0;  // device bytes of one instance (0 = not known yet)
  int n = 0;
  double canvas_mpix = 0;
};

struct Request {
  long long id = 0;
  int config = 0;
  std::vector<hmp_image> inputs;
  hmp_image canvas{};
  Clock::time_point t_submit;
};

struct InFlight {
  Request req;
  int slot = -1;
  int instance = -1;
  int event = -1;  // its completion event
};

// Requests a stream slot holds: one running and the next queued behind it on the same stream, so
// that the slot's next request is already on the GPU when the running one completes.
constexpr int kSlotDepth = 2;

}  // namespace

struct hmp_server {
  hmp_server_options opt{};
  int device = 0;
  hmp::AdmissionPolicy policy;
  std::vector<ConfigEntry> configs;
  std::vector<hmp_stitcher*> stitchers;  // indexed like the policy's instances
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;  // kSlotDepth per slot
  std::vector<char> event_busy;
  std::vector<int> slot_count;      // requests in flight on the slot

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> pending;            // submitted, not yet taken by the dispatcher
  std::unordered_map<long long, hmp_status> done;
  std::unordered_multiset<long long> waited_ids;  // requests a hmp_server_wait call waits for
  long long next_id = 1;
  long long submitted = 0, completed = 0, failed = 0, created = 0, evicted = 0, outstanding = 0;
  int max_in_flight = 0;
  double resident_bytes = 0, resident_peak = 0;  // the policy's figures, published under `mu`
  std::vector<double> lat_ms;
  double mpix_done = 0;
  Clock::time_point t_first{}, t_last{};
  bool have_first = false;
  bool stop = false;
  std::thread worker;

  // Dispatcher-owned.
  std::deque<Request> queue;
  std::vector<InFlight> inflight;

  explicit hmp_server(const hmp_server_options& o)
      : opt(o), policy(double(o.hbm_budget_bytes), std::max(1, o.max_instances_per_config)) {}

  void finish(const Request& r, const hmp_status& s, Clock::time_point now) {
    std::lock_guard<std::mutex> lk(mu);
    done[r.id] = s;
    --outstanding;
    if (s.code == HMP_OK) {
      ++completed;
      lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r.t_submit).count());
      mpix_done += configs[r.config].canvas_mpix * (configs[r.config].cfg.batch_size);
      t_last = now;
    } else {
      ++failed;
    }
    // Wake waiters only when one of them can return: drains once nothing is outstanding, a wait
    // once its request is done. Waking every waiter on every completion had them contend for `mu`
    // with this thread at each of thousands of completions a second.
    if (outstanding == 0 || waited_ids.count(r.id) > 0) cv_done.notify_all();
  }

  // One dispatcher step; returns true if it did any work.
  bool step() {
    bool worked = false;
    {
      std::lock_guard<std::mutex> lk(mu);
      while (!pending.empty()) {
        queue.push_back(std::move(pending.front()));
        pending.pop_front();
      }
    }
    // Completions.
    const Clock::time_point now = Clock::now();
    for (size_t i = 0; i < inflight.size();) {
      const cudaError_t q = cudaEventQuery(events[inflight[i].event]);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      InFlight f = std::move(inflight[i]);
      inflight.erase(inflight.begin() + long(i));
      --slot_count[f.slot];
      event_busy[f.event] = 0;
      policy.release(f.instance);
      hmp_status s = q == cudaSuccess ? mk(HMP_OK, "") : mk(int(q), cudaGetErrorString(q));
      if (s.code == HMP_OK) s = hmp_stitcher_status(stitchers[f.instance]);
      finish(f.req, s, now);
      worked = true;
    }
    // Admission, in arrival order, skipping requests that must wait.
    for (auto it = queue.begin(); it != queue.end();) {
      int slot = -1;  // the least loaded slot with room: an empty one first
      for (size_t k = 0; k < slot_count.size(); ++k)
        if (slot_count[k] < kSlotDepth && (slot < 0 || slot_count[k] < slot_count[slot])) slot = int(k);
      if (slot < 0) break;
      ConfigEntry& c = configs[it->config];
      if (c.bytes > policy.budget()) {
        // An instance of this configuration was measured larger than the whole budget: the
        // request can never be admitted, so it fails instead of waiting.
        finish(*it, mk(HMP_ERR_MEMORY_ALLOCATION, "configuration exceeds the server's HBM budget"), Clock::now());
        it = queue.erase(it);
        worked = true;
        continue;
      }
      const double est = c.bytes > 0 ? c.bytes : 0.0;
      const hmp::AdmissionPolicy::Decision d = policy.decide(it->config, est);
      int inst = -1;
      if (d.kind == hmp::AdmissionPolicy::kUse) {
        inst = d.instance;
      } else if (d.kind == hmp::AdmissionPolicy::kCreate) {
        for (int e : d.evict) {
          hmp_stitcher_destroy(stitchers[e]);
          stitchers[e] = nullptr;
          policy.remove(e);
          std::lock_guard<std::mutex> lk(mu);
          ++evicted;
        }
        hmp_stitcher* st = nullptr;
        const hmp_status cs = hmp_stitcher_create(&c.cfg, &st);
        if (cs.code != HMP_OK) {
          hmp_stitcher_destroy(st);
          finish(*it, cs, Clock::now());
          it = queue.erase(it);
          worked = true;
          continue;
        }
        hmp_stitcher_info info{};
        hmp_stitcher_get_info(st, &info);
        if (c.bytes <= 0) c.bytes = info.device_bytes;
        if (info.device_bytes > policy.budget() - policy.resident()) {
          // First instance of this configuration: its size was unknown and does not fit now.
          hmp_stitcher_destroy(st);
          if (info.device_bytes > policy.budget()) {
            finish(*it, mk(HMP_ERR_MEMORY_ALLOCATION, "configuration exceeds the server's HBM budget"),
                   Clock::now());
            it = queue.erase(it);
            worked = true;
          } else {
            ++it;
          }
          continue;
        }
        inst = policy.add(it->config, info.device_bytes);
        if (size_t(inst) >= stitchers.size()) stitchers.resize(inst + 1, nullptr);
        stitchers[inst] = st;
        std::lock_guard<std::mutex> lk(mu);
        ++created;
      } else {
        ++it;
        continue;
      }
      // Launch on the slot.
      policy.acquire(inst);
      const hmp_status ps = hmp_stitcher_process(stitchers[inst], it->inputs.data(), int(it->inputs.size()),
                                                 &it->canvas, streams[slot]);
      if (ps.code != HMP_OK) {
        policy.release(inst);
        // A failed process() leaves the instance's sticky status set: retire it.
        hmp_stitcher_destroy(stitchers[inst]);
        stitchers[inst] = nullptr;
        policy.remove(inst);
        finish(*it, ps, Clock::now());
        it = queue.erase(it);
        worked = true;
        continue;
      }
      int ev = slot * kSlotDepth;
      while (event_busy[ev]) ++ev;  // the slot has fewer than kSlotDepth requests in flight
      cudaEventRecord(events[ev], streams[slot]);
      event_busy[ev] = 1;
      ++slot_count[slot];
      InFlight f;
      f.req = std::move(*it);
      f.slot = slot;
      f.instance = inst;
      f.event = ev;
      inflight.push_back(std::move(f));
      it = queue.erase(it);
      worked = true;
      std::lock_guard<std::mutex> lk(mu);
      max_in_flight = std::max(max_in_flight, int(inflight.size()));
    }
    if (worked) {
      std::lock_guard<std::mutex> lk(mu);
      resident_bytes = policy.resident();
      resident_peak = policy.peak();
    }
    return worked;
  }

  void run() {
    cudaSetDevice(device);
    for (;;) {
      const bool worked = step();
      std::unique_lock<std::mutex> lk(mu);
      if (stop && pending.empty() && queue.empty() && inflight.empty()) break;
      if (!worked) {
        // Idle: sleep until work arrives. Waiting on the GPU: poll the in-flight events again
        // after yielding the core, not after a timed sleep (a 20 us wait sleeps 50 us or more
        // with the kernel's timer slack, and every slot that drains meanwhile idles the GPU).
        if (inflight.empty() && pending.empty() && queue.empty()) {
          cv_work.wait_for(lk, std::chrono::milliseconds(5));
        } else if (!inflight.empty()) {
          lk.unlock();
          std::this_thread::yield();
        } else {
          cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
      }
    }
  }

  ~hmp_server() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (hmp_stitcher* st : stitchers) hmp_stitcher_destroy(st);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    for (cudaStream_t s : streams) cudaStreamDestroy(s);
  }
};

extern "C" {

HMP_API hmp_status hmp_server_create(const hmp_server_options* opt, hmp_server** out) {
  if (out) *out = nullptr;
  if (!opt || !out || opt->slots < 1 || opt->slots > 64 || opt->hbm_budget_bytes == 0)
    return mk(HMP_ERR_INVALID_VALUE, "server options: slots in 1..64 and a non-zero HBM budget");
  hmp_server* s = new (std::nothrow) hmp_server(*opt);
  if (!s) return mk(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  cudaError_t e = cudaGetDevice(&s->device);
  for (int k = 0; k < opt->slots && e == cudaSuccess; ++k) {
    cudaStream_t st;
    cudaEvent_t ev;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) break;
    s->streams.push_back(st);
    for (int d = 0; d < kSlotDepth && e == cudaSuccess; ++d) {
      e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e == cudaSuccess) s->events.push_back(ev);
    }
  }
  if (e != cudaSuccess) {
    const hmp_status r = mk(int(e), cudaGetErrorString(e));
    delete s;
    return r;
  }
  s->slot_count.assign(opt->slots, 0);
  s->event_busy.assign(size_t(opt->slots) * kSlotDepth, 0);
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return mk(HMP_OK, "");
}

HMP_API void hmp_server_destroy(hmp_server* s) { delete s; }

HMP_API hmp_status hmp_server_add_config(hmp_server* s, const hmp_config* cfg, int* config_id) {
  if (!s || !cfg || !config_id) return mk(HMP_ERR_INVALID_VALUE, "null argument");
  int cw = 0, ch = 0, geo[9];
  hmp_status g = hmp_plan_geometry(cfg, &cw, &ch, geo);
  if (g.code != HMP_OK) return g;
  ConfigEntry c;
  c.cfg = *cfg;
  c.n = cfg->n_images;
  c.canvas_mpix = double(cw) * ch / 1e6;
  c.remaps.assign(cfg->remaps, cfg->remaps + cfg->n_images);
  c.mx.resize(c.n);
  c.my.resize(c.n);
  for (int i = 0; i < c.n; ++i) {
    const size_t px = size_t(cfg->remaps[i].width) * cfg->remaps[i].height;
    c.mx[i].assign(cfg->remaps[i].map_x, cfg->remaps[i].map_x + px);
    c.my[i].assign(cfg->remaps[i].map_y, cfg->remaps[i].map_y + px);
    c.remaps[i].map_x = c.mx[i].data();
    c.remaps[i].map_y = c.my[i].data();
  }
  c.seam.assign(cfg->seam, cfg->seam + size_t(cfg->seam_width) * cfg->seam_height);
  c.cfg.remaps = c.remaps.data();
  c.cfg.seam = c.seam.data();
  std::lock_guard<std::mutex> lk(s->mu);
  // The dispatcher indexes configs without the lock; registering while requests run would
  // reallocate under it, so configurations are registered before submitting.
  if (s->outstanding > 0) return mk(HMP_ERR_INVALID_VALUE, "register configurations while no request is outstanding");
  s->configs.push_back(std::move(c));
  // Vectors of hmp_remap moved with the entry keep their heap buffers; re-point the config.
  ConfigEntry& e = s->configs.back();
  e.cfg.remaps = e.remaps.data();
  e.cfg.seam = e.seam.data();
  *config_id = int(s->configs.size()) - 1;
  return mk(HMP_OK, "");
}

HMP_API hmp_status hmp_server_submit(hmp_server* s, int config_id, const hmp_image* inputs, int n_inputs,
                                     const hmp_image* canvas, long long* request_id) {
  if (!s || !inputs || !canvas) return mk(HMP_ERR_INVALID_VALUE, "null argument");
  Request r;
  r.t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (config_id < 0 || config_id >= int(s->configs.size())) return mk(HMP_ERR_INVALID_VALUE, "unknown configuration");
    if (n_inputs != s->configs[config_id].n) return mk(HMP_ERR_INVALID_VALUE, "inputs size != N");
    r.id = s->next_id++;
    r.config = config_id;
    r.inputs.assign(inputs, inputs + n_inputs);
    r.canvas = *canvas;
    if (!s->have_first) {
      s->t_first = r.t_submit;
      s->have_first = true;
    }
    ++s->submitted;
    ++s->outstanding;
    if (request_id) *request_id = r.id;
    s->pending.push_back(std::move(r));
  }
  s->cv_work.notify_one();
  return mk(HMP_OK, "");
}

HMP_API hmp_status hmp_server_wait(hmp_server* s, long long request_id, int timeout_ms) {
  if (!s) return mk(HMP_ERR_INVALID_VALUE, "server is null");
  std::unique_lock<std::mutex> lk(s->mu);
  const auto w = s->waited_ids.insert(request_id);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)),
                                      [&] { return s->done.count(request_id) > 0; });
  s->waited_ids.erase(w);
  if (!ok) return mk(HMP_ERR_TIMEOUT, "request did not finish within the timeout");
  const hmp_status r = s->done[request_id];
  s->done.erase(request_id);
  return r;
}

HMP_API hmp_status hmp_server_drain(hmp_server* s, int timeout_ms) {
  if (!s) return mk(HMP_ERR_INVALID_VALUE, "server is null");
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)),
                                      [&] { return s->outstanding == 0; });
  if (!ok) return mk(HMP_ERR_TIMEOUT, "requests still outstanding after the timeout");
  s->done.clear();
  return mk(HMP_OK, "");
}

HMP_API hmp_status hmp_server_get_stats(hmp_server* s, hmp_server_stats* out) {
  if (!s || !out) return mk(HMP_ERR_INVALID_VALUE, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->instances_created = s->created;
  out->instances_evicted = s->evicted;
  out->max_in_flight = s->max_in_flight;
  out->canvas_mpix = s->mpix_done;
  out->resident_bytes = s->resident_bytes;
  out->resident_bytes_peak = s->resident_peak;
  if (!s->lat_ms.empty()) {
    std::vector<double> v = s->lat_ms;
    std::sort(v.begin(), v.end());
    const auto pct = [&](double p) { return v[std::min(v.size() - 1, size_t(p * double(v.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / double(v.size());
  }
  if (s->have_first && s->completed > 0)
    out->span_ms = std::chrono::duration<double, std::milli>(s->t_last - s->t_first).count();
  return mk(HMP_OK, "");
}

HMP_API void hmp_server_reset_stats(hmp_server* s) {
  if (!s) return;
  std::lock_guard<std::mutex> lk(s->mu);
  s->submitted -= s->completed + s->failed;
  s->completed = s->failed = s->created = s->evicted = 0;
  s->max_in_flight = 0;
  s->lat_ms.clear();
  s->mpix_done = 0;
  s->have_first = false;
}

}  // extern "C"
