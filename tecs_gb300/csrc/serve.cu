// serve.cu -- the served stream behind the C ABI (tecs_serve_*): a
// continuous-batching request loop over engines, run by a server thread.
//
// Requests arrive through tecs_serve_submit from any thread.  Each goes to
// the first lane (size class) that takes its cell count; a lane is one
// engine (engine.cu) with its own stream.  The server thread loops:
//
//   admit    per lane, first come first served, while the engine has the
//            request's cells and a free run of its bins;
//   step     per lane with fewer than in_flight batches queued: k steps of
//            every resident simulation, k = steps_per_issue at most and never
//            past a resident request's next snapshot or its end;
//   snapshot a request at a multiple of snapshot_every: unpacked on the
//            device and copied to pinned memory on the engine's side stream;
//            the writer thread waits for the copy and writes the HDF5 group;
//   retire   a request at its step count: its state downloaded and kept for
//            tecs_serve_fetch, its engine slot removed.
//
// Time-to-completion is measured from the submit to the retirement.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tecs/hdf5_writer.hpp"
#include "../../include/tecs_gpu.h"

namespace tecs {
int set_last_error(const std::string& m);
}

namespace {

int fail(const std::string& m) { return tecs::set_last_error(m); }

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0, tag = 0;
  tecs_sim_desc desc{};
  std::vector<float> pos, pol;
  unsigned n = 0, steps = 0, start = 0;
  double arrival = 0.0;
};

struct Live {
  std::unique_ptr<Request> req;
  int slot = -1;
  unsigned done = 0;  // steps taken, counted from the request's start step
  double admitted = 0.0;
};

struct Lane {
  tecs_engine* engine = nullptr;
  unsigned max_cells = 0;  // 0: any
  unsigned cells = 0, bins = 0;
  std::deque<std::unique_ptr<Request>> waiting;
  std::map<int, Live> live;
  std::deque<cudaEvent_t> pending;  // queued step batches
  unsigned stage_next = 0;          // next free staging cell for snapshots
};

// pinned host buffers for snapshots, reused by size
struct PinnedPool {
  std::mutex mu;
  std::multimap<size_t, float*> free_bufs;
  float* get(size_t floats) {
    {
      std::lock_guard<std::mutex> lock(mu);
      auto it = free_bufs.find(floats);
      if (it != free_bufs.end()) {
        float* p = it->second;
        free_bufs.erase(it);
        return p;
      }
    }
    float* p = nullptr;
    if (cudaMallocHost(&p, std::max<size_t>(floats, 1) * 4) != cudaSuccess) return nullptr;
    return p;
  }
  void put(size_t floats, float* p) {
    std::lock_guard<std::mutex> lock(mu);
    free_bufs.emplace(floats, p);
  }
  ~PinnedPool() {
    for (auto& kv : free_bufs) cudaFreeHost(kv.second);
  }
};

struct Snapshot {
  void* event = nullptr;
  uint64_t id = 0, tag = 0;
  unsigned step = 0, n = 0;
  float* pos = nullptr;
  float* pol = nullptr;
  bool close = false;  // the request is retired: close its file
};

}  // namespace

struct tecs_serve {
  tecs_serve_desc d{};
  std::deque<Lane> lanes;  // a deque: lanes hold move-only members and never move
  Clock::time_point t0;
  std::mutex mu;                 // submitted, results, counters below
  std::condition_variable cv;    // work for the server thread; completions for drain
  std::deque<std::unique_ptr<Request>> submitted;
  std::deque<tecs_serve_result> completed_unpolled;
  std::map<uint64_t, std::pair<std::vector<float>, std::vector<float>>> finals;
  uint64_t next_id = 1;
  unsigned n_submitted = 0, n_completed = 0, n_resident = 0, n_waiting = 0;
  unsigned long long cell_steps = 0, engine_steps = 0;
  std::atomic<unsigned long long> snaps_written{0}, snaps_errors{0}, snaps_pending{0};
  std::atomic<bool> stop{false};
  std::string error;             // a server-thread failure, reported by drain
  std::thread worker;
  // snapshot writer
  std::mutex wmu;
  std::condition_variable wcv;
  std::deque<Snapshot> wq;
  bool wstop = false;
  std::thread writer;
  PinnedPool pool;
  std::map<uint64_t, std::unique_ptr<tecs::io::h5detail::File>> files;  // writer thread only

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// HDF5 snapshots, one file per request (writer thread)
void writer_loop(tecs_serve* s) {
  for (;;) {
    Snapshot sn;
    {
      std::unique_lock<std::mutex> lock(s->wmu);
      s->wcv.wait(lock, [&] { return s->wstop || !s->wq.empty(); });
      if (s->wq.empty()) return;
      sn = s->wq.front();
      s->wq.pop_front();
    }
    if (sn.close) {
      s->files.erase(sn.id);  // the file's superblock is written as it closes
      continue;
    }
    // the copy's event, waited for at most a minute (a copy that never
    // completes loses its snapshot, not the writer)
    bool ok = true;
    for (int polls = 0;; ++polls) {
      int ready = 0;
      if (tecs_engine_event_query(sn.event, &ready) != 0) { ok = false; break; }
      if (ready) break;
      if (polls >= 300000) { ok = false; break; }
      std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    tecs_engine_event_destroy(sn.event);
    if (ok && s->d.snapshot_dir) {
      try {
        auto& f = s->files[sn.id];
        if (!f) {
          char name[48];
          std::snprintf(name, sizeof name, "/request_%05llu.h5", (unsigned long long)sn.tag);
          f = std::make_unique<tecs::io::h5detail::File>(std::string(s->d.snapshot_dir) + name);
        }
        std::vector<tecs::io::h5detail::Dataset> ds;
        ds.push_back({"position", sn.pos, sn.n, 3, tecs::io::h5detail::Kind::f32});
        if (sn.pol) ds.push_back({"polarity", sn.pol, sn.n, 2, tecs::io::h5detail::Kind::f32});
        f->write_group("t" + std::to_string(sn.step), ds);
      } catch (const std::exception&) {
        ok = false;  // a failing write loses this snapshot, not the server
      }
    }
    s->pool.put(3 * (size_t)sn.n, sn.pos);
    if (sn.pol) s->pool.put(2 * (size_t)sn.n, sn.pol);
    if (ok) ++s->snaps_written;
    else ++s->snaps_errors;
    --s->snaps_pending;
    // taken and released so that a drain between its check and its wait
    // cannot miss this notification
    { std::lock_guard<std::mutex> lock(s->mu); }
    s->cv.notify_all();
  }
}

int snapshot(tecs_serve* s, Lane& lane, Live& lv, unsigned step) {
  const unsigned n = lv.req->n;
  const bool pol = lv.req->desc.has_polarity != 0;
  if (lane.stage_next + n > lane.cells) {
    lane.stage_next = 0;
    if (tecs_engine_synchronize(lane.engine)) return -1;  // staging reused: queued copies first
  }
  Snapshot sn;
  sn.id = lv.req->id;
  sn.tag = lv.req->tag;
  sn.step = step;
  sn.n = n;
  sn.pos = s->pool.get(3 * (size_t)n);
  sn.pol = pol ? s->pool.get(2 * (size_t)n) : nullptr;
  if (!sn.pos || (pol && !sn.pol)) return fail("cannot allocate pinned snapshot buffers");
  if (tecs_engine_snapshot_async(lane.engine, lv.slot, sn.pos, sn.pol, lane.stage_next, &sn.event)) return -1;
  lane.stage_next += n;
  ++s->snaps_pending;
  {
    std::lock_guard<std::mutex> lock(s->wmu);
    s->wq.push_back(sn);
  }
  s->wcv.notify_one();
  return 0;
}

int retire(tecs_serve* s, Lane& lane, int slot) {
  Live& lv = lane.live.at(slot);
  const Request& r = *lv.req;
  std::vector<float> pos(3 * (size_t)r.n), pol(r.desc.has_polarity ? 2 * (size_t)r.n : 0);
  unsigned n = 0;
  if (tecs_engine_download(lane.engine, slot, pos.data(), pol.empty() ? nullptr : pol.data(), &n)) return -1;
  if (tecs_engine_remove(lane.engine, slot)) return -1;
  tecs_serve_result res{};
  res.id = r.id;
  res.tag = r.tag;
  res.cells = r.n;
  res.steps = r.steps - r.start;
  res.arrival_s = r.arrival;
  res.admitted_s = lv.admitted;
  res.completed_s = s->now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->finals[r.id] = {std::move(pos), std::move(pol)};
    s->completed_unpolled.push_back(res);
    ++s->n_completed;
    --s->n_resident;
  }
  lane.live.erase(slot);
  if (s->d.snapshot_every && s->d.snapshot_dir) {
    Snapshot sn;
    sn.id = res.id;
    sn.close = true;
    std::lock_guard<std::mutex> lock(s->wmu);
    s->wq.push_back(sn);
    s->wcv.notify_one();
  }
  s->cv.notify_all();
  return 0;
}

// one pass of the loop; returns -1 on a failure, else whether a step was issued
int serve_once(tecs_serve* s) {
  {
    std::lock_guard<std::mutex> lock(s->mu);
    while (!s->submitted.empty()) {
      auto r = std::move(s->submitted.front());
      s->submitted.pop_front();
      for (auto& lane : s->lanes)
        if (lane.max_cells == 0 || r->n <= lane.max_cells) {
          lane.waiting.push_back(std::move(r));
          break;
        }
    }
  }
  // admission, per lane: first come first served, while cells and bins are free
  for (auto& lane : s->lanes) {
    while (!lane.waiting.empty()) {
      Request& r = *lane.waiting.front();
      unsigned free_cells = 0, free_bins = 0, need_bins = 0;
      if (tecs_engine_free(lane.engine, &free_cells, &free_bins)) return -1;
      if (tecs_engine_bins_needed(&r.desc, &need_bins)) return -1;
      if (r.n > free_cells || need_bins > free_bins) {
        if (lane.live.empty()) return fail("request " + std::to_string(r.id) + " does not fit an idle engine");
        break;
      }
      int slot = -1;
      if (tecs_engine_add(lane.engine, &r.desc, r.pos.data(), r.pol.empty() ? nullptr : r.pol.data(), r.n, &slot))
        return -1;
      Live lv;
      lv.req = std::move(lane.waiting.front());
      lane.waiting.pop_front();
      lv.slot = slot;
      lv.done = lv.req->start;
      lv.admitted = s->now();
      lv.req->pos.clear();
      lv.req->pos.shrink_to_fit();
      lv.req->pol.clear();
      lv.req->pol.shrink_to_fit();
      lane.live.emplace(slot, std::move(lv));
      std::lock_guard<std::mutex> lock(s->mu);
      --s->n_waiting;
      ++s->n_resident;
    }
    // a request resumed at its end
    std::vector<int> finished;
    for (auto& kv : lane.live)
      if (kv.second.done >= kv.second.req->steps) finished.push_back(kv.first);
    for (int slot : finished)
      if (retire(s, lane, slot)) return -1;
  }
  int issued = 0;
  for (auto& lane : s->lanes) {
    while (!lane.pending.empty() && cudaEventQuery(lane.pending.front()) == cudaSuccess) {
      cudaEventDestroy(lane.pending.front());
      lane.pending.pop_front();
    }
    if (lane.live.empty() || lane.pending.size() >= s->d.in_flight) continue;
    unsigned k = s->d.steps_per_issue;
    for (auto& kv : lane.live) {
      const Live& lv = kv.second;
      k = std::min(k, lv.req->steps - lv.done);
      if (s->d.snapshot_every) k = std::min(k, s->d.snapshot_every - lv.done % s->d.snapshot_every);
    }
    k = std::max(k, 1u);
    if (tecs_engine_step(lane.engine, s->d.dt, (int)k)) return -1;
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(ev, static_cast<cudaStream_t>(tecs_engine_stream(lane.engine))) != cudaSuccess)
      return fail("cannot record a step event");
    lane.pending.push_back(ev);
    issued = 1;
    unsigned long long cs = 0;
    std::vector<int> finished;
    for (auto& kv : lane.live) {
      Live& lv = kv.second;
      lv.done += k;
      cs += (unsigned long long)lv.req->n * k;
      if (s->d.snapshot_every && lv.done % s->d.snapshot_every == 0 && lv.done < lv.req->steps)
        if (snapshot(s, lane, lv, lv.done)) return -1;
      if (lv.done >= lv.req->steps) finished.push_back(kv.first);
    }
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->cell_steps += cs;
      s->engine_steps += k;
    }
    for (int slot : finished)
      if (retire(s, lane, slot)) return -1;
  }
  return issued;
}

void server_loop(tecs_serve* s) {
  cudaSetDevice(s->d.device);
  while (!s->stop) {
    const int r = serve_once(s);
    if (r < 0) {
      std::lock_guard<std::mutex> lock(s->mu);
      s->error = tecs_last_error();
      s->cv.notify_all();
      return;
    }
    if (r == 0) {
      std::unique_lock<std::mutex> lock(s->mu);
      bool idle = s->submitted.empty();
      for (auto& lane : s->lanes) idle = idle && lane.live.empty();
      if (idle) s->cv.wait_for(lock, std::chrono::milliseconds(2));
      else {
        lock.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(50));
      }
    }
  }
}

}  // namespace

int tecs_serve_desc_default(tecs_serve_desc* d) {
  if (!d) return fail("null desc");
  std::memset(d, 0, sizeof *d);
  d->cell_capacity = 1u << 22;
  d->bin_capacity = 3u << 22;
  d->max_sims = 4096;
  d->dt = 0.05;
  d->snapshot_every = 100;
  d->n_lanes = 1;
  d->lane_share[0] = 1.0f;
  d->steps_per_issue = 1;
  d->in_flight = 2;
  return 0;
}

int tecs_serve_create(const tecs_serve_desc* desc, tecs_serve** out) {
  if (!desc || !out) return fail("null argument");
  *out = nullptr;
  if (desc->n_lanes < 1 || desc->n_lanes > 4) return fail("1 to 4 lanes");
  if (desc->lane_max_cells[desc->n_lanes - 1] != 0) return fail("the last lane must take any request");
  if (desc->steps_per_issue < 1 || desc->in_flight < 1) return fail("steps_per_issue and in_flight must be >= 1");
  auto s = std::make_unique<tecs_serve>();
  s->d = *desc;
  s->t0 = Clock::now();
  for (unsigned l = 0; l < desc->n_lanes; ++l) {
    Lane lane;
    lane.max_cells = desc->lane_max_cells[l];
    lane.cells = std::max(1u, (unsigned)(desc->cell_capacity * (double)desc->lane_share[l]));
    lane.bins = std::max(1u, (unsigned)(desc->bin_capacity * (double)desc->lane_share[l]));
    tecs_engine_desc ed{};
    tecs_engine_desc_default(&ed);
    ed.cell_capacity = lane.cells;
    ed.bin_capacity = lane.bins;
    ed.max_sims = desc->max_sims;
    ed.device = desc->device;
    if (tecs_engine_create(&ed, &lane.engine)) {
      for (auto& l2 : s->lanes) tecs_engine_destroy(l2.engine);
      return -1;
    }
    s->lanes.emplace_back(std::move(lane));
  }
  tecs_serve* raw = s.release();
  raw->writer = std::thread(writer_loop, raw);
  raw->worker = std::thread(server_loop, raw);
  *out = raw;
  return 0;
}

int tecs_serve_submit(tecs_serve* s, const tecs_sim_desc* desc, const float* positions, const float* polarity,
                      unsigned n, unsigned steps, unsigned start_step, uint64_t tag, uint64_t* id) {
  if (!s || !desc || (!positions && n)) return fail("null argument");
  if (desc->has_polarity && n && !polarity) return fail("the request has a polarity field: polarity required");
  if (start_step > steps) return fail("start step beyond the step count");
  bool fits = false;
  for (const auto& lane : s->lanes) {
    if (lane.max_cells != 0 && n > lane.max_cells) continue;
    unsigned need = 0;
    if (tecs_engine_bins_needed(desc, &need)) return -1;
    if (n > lane.cells || need > lane.bins) return fail("the request exceeds its lane's engine");
    fits = true;
    break;
  }
  if (!fits) return fail("no lane takes the request");
  auto r = std::make_unique<Request>();
  r->desc = *desc;
  r->n = n;
  r->steps = steps;
  r->start = start_step;
  r->tag = tag;
  r->pos.assign(positions, positions + 3 * (size_t)n);
  if (desc->has_polarity) r->pol.assign(polarity, polarity + 2 * (size_t)n);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (!s->error.empty()) return fail("server stopped: " + s->error);
    r->id = s->next_id++;
    r->arrival = s->now();
    if (id) *id = r->id;
    s->submitted.push_back(std::move(r));
    ++s->n_submitted;
    ++s->n_waiting;
  }
  s->cv.notify_all();
  return 0;
}

int tecs_serve_poll(tecs_serve* s, tecs_serve_result* results, unsigned capacity, unsigned* n) {
  if (!s || !n || (capacity && !results)) return fail("null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  unsigned k = 0;
  while (k < capacity && !s->completed_unpolled.empty()) {
    results[k++] = s->completed_unpolled.front();
    s->completed_unpolled.pop_front();
  }
  *n = k;
  return s->error.empty() ? 0 : fail("server stopped: " + s->error);
}

int tecs_serve_fetch(tecs_serve* s, uint64_t id, float* positions, float* polarity, unsigned* n) {
  if (!s || !positions) return fail("null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->finals.find(id);
  if (it == s->finals.end()) return fail("no completed request " + std::to_string(id));
  const auto& [pos, pol] = it->second;
  std::memcpy(positions, pos.data(), pos.size() * 4);
  if (polarity && !pol.empty()) std::memcpy(polarity, pol.data(), pol.size() * 4);
  if (n) *n = (unsigned)(pos.size() / 3);
  s->finals.erase(it);
  return 0;
}

int tecs_serve_drain(tecs_serve* s, double timeout_s) {
  if (!s) return fail("null server");
  std::unique_lock<std::mutex> lock(s->mu);
  const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
  const bool done = s->cv.wait_until(lock, until, [&] {
    return !s->error.empty() || (s->n_completed == s->n_submitted && s->snaps_pending == 0);
  });
  if (!s->error.empty()) return fail("server stopped: " + s->error);
  if (!done) return fail("drain timed out");
  return 0;
}

int tecs_serve_stats_get(tecs_serve* s, tecs_serve_stats* st) {
  if (!s || !st) return fail("null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  st->cell_steps = s->cell_steps;
  st->engine_steps = s->engine_steps;
  st->snapshots_written = s->snaps_written;
  st->snapshot_errors = s->snaps_errors;
  st->submitted = s->n_submitted;
  st->completed = s->n_completed;
  st->resident = s->n_resident;
  st->waiting = s->n_waiting;
  return 0;
}

int tecs_serve_destroy(tecs_serve* s) {
  if (!s) return 0;
  s->stop = true;
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& lane : s->lanes) tecs_engine_synchronize(lane.engine);
  {
    std::lock_guard<std::mutex> lock(s->wmu);
    s->wstop = true;
  }
  s->wcv.notify_all();
  if (s->writer.joinable()) s->writer.join();
  s->files.clear();
  for (auto& lane : s->lanes) {
    for (cudaEvent_t ev : lane.pending) cudaEventDestroy(ev);
    tecs_engine_destroy(lane.engine);
  }
  delete s;
  return 0;
}
