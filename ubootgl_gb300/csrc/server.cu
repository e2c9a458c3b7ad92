// Step server (extension): continuous batching of step requests over
// sessions whose fields stay resident on the device.
//
// A session is one simulation handle (its own fields and stream).  Sessions
// are admitted against a device-memory budget when they are opened: over
// budget, an open is refused (UBG_ADMIT_REJECT, the default) or the session
// waits in FIFO order, with its inputs kept in host memory, until closed
// sessions free enough budget (UBG_ADMIT_QUEUE).  A request asks for k steps
// of one session.  The worker thread admits queued requests in arrival
// order whenever a slot is free (one request in flight per session; at most
// max_active stream requests and 4 * max_active fused requests; requests
// of sessions still waiting for memory stay queued without blocking the
// others).  Requests of sessions that the fused form covers (FP32, fixed
// V-cycle count, at most 1M cells; see FusedStepper) are stepped together:
// every worker iteration enqueues ONE step of every such request as one
// launch per kernel over all of them, so a request that arrives joins at
// the next step boundary and leaves after its k-th step (iteration-level
// continuous batching, at most two steps in flight).  Other requests (mixed
// precision, tolerance mode, larger grids, or every request in the stream
// mode) go to a pool of max_active host threads, each of which runs one
// request's steps on its session's own stream: the tolerance solver waits
// on the device once per V-cycle, and a pool thread blocked there holds up
// neither the worker nor the other sessions, whose work overlaps on the
// device.  Sessions touch only their own memory and the fused step is
// bit-identical to stepping alone, so a session's result does not depend on
// what else is in flight.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "ubg_internal.cuh"

using namespace ubg;

namespace {
double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace

// A fused request in flight costs one step of a shared launch sequence per
// worker iteration, not a stream of its own: max_active bounds the stream
// requests in flight, and kFusedPerSlot * max_active the fused ones.
constexpr int kFusedPerSlot = 4;
// Steps of a stream request enqueued at a time (at most two chunks queued).
constexpr int kChunkSteps = 2;

struct ubg_server {
  struct Session {
    ubg_sim *sim = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t evc[2] = {nullptr, nullptr};  // completion of queued work
    size_t bytes = 0;
    long long cells = 0;
    bool busy = false;
    // waiting for device memory (queue admission): the inputs to build it
    bool pending = false, building = false;
    int width = 0, height = 0;
    float pwidth = 1.0f, mu = 0.0f;
    std::vector<float> flag, vx, vy;
    bool has_opt = false;
    ubg_options opt{};
  };
  struct Request {
    int session = 0;
    int steps = 0;
    float cfl = 0.5f;
    double t_submit = 0, t_admit = 0, t_end = 0;
    bool fused = false;  // stepped by the fused stepper
    int remaining = 0;   // fused steps not yet enqueued
    bool finished = false;
    int error = 0;
  };

  size_t budget = 0, used = 0;
  int max_active = 1;
  int mode = UBG_SERVE_FUSED;
  int admission = UBG_ADMIT_REJECT;
  std::deque<int> pending;  // sessions waiting for memory, in open order
  long long admitted_from_queue = 0;
  std::condition_variable cv_pool;
  std::deque<uint64_t> stream_jobs;  // admitted stream requests for the pool
  std::vector<std::thread> pool;
  long long fuse_max_cells = kFuseMaxCells;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::map<int, Session> sessions;
  int next_session = 1;
  std::map<uint64_t, Request> reqs;
  uint64_t next_req = 1;
  std::deque<uint64_t> queue;
  std::vector<uint64_t> active;
  std::vector<double> latencies;
  long long rejected = 0, cell_steps = 0, completed = 0;
  long long fused_steps = 0, fused_member_steps = 0;
  double worker_fused_ms = 0.0, worker_streams_ms = 0.0;
  double t_first = -1.0, t_last = 0.0;
  bool stop = false, stop_pool = false;
  std::unique_ptr<FusedStepper> fs;
  std::thread worker;

  // Runs one stream request's steps on its session's stream, in chunks of
  // kChunkSteps with at most two chunks queued (a full launch queue would
  // block every launching thread, the worker's fused steps included), then
  // waits for the last chunk.  Called by a pool thread without the lock.
  int run_stream_request(Request &r, Session &s) {
    int rc = UBG_OK;
    int enq = 0, chunks = 0;
    while (enq < r.steps && rc == UBG_OK) {
      if (chunks >= 2 && cudaEventSynchronize(s.evc[chunks % 2]) != cudaSuccess) {
        cudaGetLastError();
        return UBG_ECUDA;
      }
      const double t0 = now_ms();
      const int n = std::min(kChunkSteps, r.steps - enq);
      for (int k = 0; k < n && rc == UBG_OK; k++) rc = ubg_step_cfl(s.sim, r.cfl);
      if (rc == UBG_OK && cudaEventRecord(s.evc[chunks % 2], s.st) != cudaSuccess) rc = UBG_ECUDA;
      enq += n;
      chunks++;
      {
        std::lock_guard<std::mutex> lk(mu);
        worker_streams_ms += now_ms() - t0;
      }
    }
    if (rc == UBG_OK && chunks > 0 && cudaEventSynchronize(s.evc[(chunks - 1) % 2]) != cudaSuccess) {
      cudaGetLastError();
      rc = UBG_ECUDA;
    }
    return rc;
  }

  // Pool thread: takes admitted stream requests until the server stops.
  void pool_run() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_pool.wait(lk, [&] { return stop_pool || !stream_jobs.empty(); });
      if (stream_jobs.empty()) return;
      const uint64_t id = stream_jobs.front();
      stream_jobs.pop_front();
      Request &r = reqs[id];
      Session &s = sessions[r.session];
      lk.unlock();
      const int rc = run_stream_request(r, s);
      lk.lock();
      finish(id, rc);
      cv_work.notify_all();  // a slot is free
    }
  }

  // Completion bookkeeping of an active request (lock held).
  void finish(uint64_t id, int rc) {
    Request &r = reqs[id];
    Session &s = sessions[r.session];
    r.t_end = now_ms();
    r.finished = true;
    r.error = rc;
    s.busy = false;
    if (rc == UBG_OK) {
      latencies.push_back(r.t_end - r.t_submit);
      cell_steps += s.cells * r.steps;
      completed++;
      t_last = r.t_end;
    }
    active.erase(std::remove(active.begin(), active.end(), id), active.end());
    cv_done.notify_all();
  }

  void fail(Request &r, Session &s, int code) {
    r.t_end = now_ms();
    r.finished = true;
    r.error = code;
    s.busy = false;
    cv_done.notify_all();
  }

  // One fused step of every fused request with steps left (grouped by
  // V-cycle count); requests whose last step was enqueued start draining.
  bool fused_tick() {
    std::map<int, std::vector<uint64_t>> groups;
    for (uint64_t id : active) {
      Request &r = reqs[id];
      if (r.fused && r.remaining > 0) groups[FusedStepper::group(sessions[r.session].sim)].push_back(id);
    }
    if (groups.empty() || !fs->ready()) return false;
    const double t0 = now_ms();
    for (auto &g : groups) {
      std::vector<ubg_sim *> sims;
      std::vector<float> cfl;
      for (uint64_t id : g.second) {
        sims.push_back(sessions[reqs[id].session].sim);
        cfl.push_back(reqs[id].cfl);
      }
      try {
        fs->step(sims, cfl);
        fused_steps++;
        fused_member_steps += (long long)g.second.size();
        for (uint64_t id : g.second) {
          Request &r = reqs[id];
          if (--r.remaining == 0) {
            Session &ses = sessions[r.session];
            fs->leave(ses.sim, ses.evc[0]);
          }
        }
      } catch (const std::exception &e) {
        set_last_error(e.what());
        cudaGetLastError();
        for (uint64_t id : g.second) {
          Request &r = reqs[id];
          r.remaining = 0;
          fail(r, sessions[r.session], UBG_ECUDA);
        }
        active.erase(std::remove_if(active.begin(), active.end(),
                                    [&](uint64_t id) { return reqs[id].finished; }),
                     active.end());
      }
    }
    worker_fused_ms += now_ms() - t0;
    return true;
  }

  void run() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      // admit in arrival order while slots are free
      int n_fused = 0;
      for (uint64_t id : active) n_fused += reqs[id].fused;
      int n_streams = (int)active.size() - n_fused;
      for (auto it = queue.begin();
           it != queue.end() && (n_streams < max_active || n_fused < kFusedPerSlot * max_active);) {
        Request &r = reqs[*it];
        auto sit = sessions.find(r.session);
        if (sit == sessions.end()) {  // session closed before admission
          r.finished = true;
          r.error = UBG_ESTATE;
          it = queue.erase(it);
          cv_done.notify_all();
          continue;
        }
        Session &s = sit->second;
        if (s.pending) {  // still waiting for device memory
          ++it;
          continue;
        }
        const bool fuse = mode == UBG_SERVE_FUSED && s.cells <= fuse_max_cells &&
                          FusedStepper::eligible(s.sim);
        if (s.busy || (fuse ? n_fused >= kFusedPerSlot * max_active : n_streams >= max_active)) {
          ++it;
          continue;
        }
        s.busy = true;
        r.t_admit = now_ms();
        if (t_first < 0.0) t_first = r.t_admit;
        int rc = UBG_OK;
        if (fuse) {
          try {
            if (!fs) fs.reset(new FusedStepper());
            fs->join(s.sim);
            r.fused = true;
            r.remaining = r.steps;
          } catch (const std::exception &e) {
            set_last_error(e.what());
            cudaGetLastError();
            rc = UBG_ECUDA;
          }
        } else {
          stream_jobs.push_back(*it);
          cv_pool.notify_one();
        }
        if (rc != UBG_OK) {
          fail(r, s, rc);
          it = queue.erase(it);
          continue;
        }
        active.push_back(*it);
        (fuse ? n_fused : n_streams)++;
        it = queue.erase(it);
      }
      bool fused_active = false;
      for (uint64_t id : active) fused_active |= reqs[id].fused;
      if (!fused_active) {
        if (stop && queue.empty() && active.empty()) return;
        // stream requests complete on the pool threads, which wake us
        cv_work.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
      bool stepped = fused_tick();
      // completion polling of the fused requests
      bool any = false;
      for (size_t i = 0; i < active.size();) {
        const uint64_t id = active[i];
        Request &r = reqs[id];
        Session &s = sessions[r.session];
        if (!r.fused || r.remaining > 0) {
          i++;
          continue;
        }
        // the request's last work: the stepper's event
        cudaError_t q = cudaEventQuery(s.evc[0]);
        if (q == cudaErrorNotReady) {
          i++;
          continue;
        }
        int rc = UBG_OK;
        if (q != cudaSuccess) {
          cudaGetLastError();
          rc = UBG_ECUDA;
        } else if (fs->failed()) {
          set_last_error("fused step: a launch found a table it was not made for");
          rc = UBG_ECUDA;
        }
        finish(id, rc);  // removes it from active
        any = true;
      }
      if (!any && !stepped) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
        lk.lock();
      }
    }
  }

  // Builds the device state of waiting sessions in open order while the
  // budget allows (called without the lock, after memory was freed).
  void admit_pending();
};

namespace {
int srv_fail(int code, const std::string &m) {
  set_last_error(m);
  return code;
}
}  // namespace

int ubg_server_create(size_t budget_bytes, int max_active, ubg_server **out) {
  if (!out || max_active < 1) return srv_fail(UBG_EINVAL, "bad argument");
  try {
    ubg_server *s = new ubg_server();
    s->budget = budget_bytes;
    s->max_active = max_active;
    s->worker = std::thread([s] { s->run(); });
    for (int i = 0; i < max_active; i++) s->pool.emplace_back([s] { s->pool_run(); });
    *out = s;
  } catch (const std::exception &e) {
    return srv_fail(UBG_ESTATE, e.what());
  }
  set_last_error("");
  return UBG_OK;
}

int ubg_server_destroy(ubg_server *s) {
  if (!s) return srv_fail(UBG_EINVAL, "null handle");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop_pool = true;
  }
  s->cv_pool.notify_all();
  for (auto &t : s->pool)
    if (t.joinable()) t.join();
  s->fs.reset();
  for (auto &kv : s->sessions) {
    for (cudaEvent_t e : kv.second.evc)
      if (e) cudaEventDestroy(e);
    if (kv.second.sim) ubg_destroy(kv.second.sim);
  }
  delete s;
  set_last_error("");
  return UBG_OK;
}

int ubg_server_set_mode(ubg_server *s, int mode) {
  if (!s || (mode != UBG_SERVE_STREAMS && mode != UBG_SERVE_FUSED))
    return srv_fail(UBG_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->mode = mode;
  return UBG_OK;
}

int ubg_server_set_fuse_cells(ubg_server *s, long long max_cells) {
  if (!s || max_cells < 0) return srv_fail(UBG_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->fuse_max_cells = max_cells;
  return UBG_OK;
}

int ubg_server_set_admission(ubg_server *s, int admission) {
  if (!s || (admission != UBG_ADMIT_REJECT && admission != UBG_ADMIT_QUEUE))
    return srv_fail(UBG_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->admission = admission;
  return UBG_OK;
}

namespace {
// Device bytes a session holds: the fields and hierarchy, plus the 16-bit
// hierarchy of the fixed-mode mixed solver or the tolerance solver's arrays.
size_t session_bytes(int width, int height, const ubg_options *opt, int *rc) {
  size_t bytes = 0;
  *rc = ubg_device_bytes(width, height, &bytes);
  if (*rc) return 0;
  const size_t P = (size_t)(width + 31) / 32 * 32;
  if (opt && opt->solver_mode == UBG_SOLVE_TOLERANCE)
    bytes += fcg_bytes(width, height, (int)P, opt->precision);
  else if (opt && opt->precision != UBG_FP32)
    bytes += (size_t)(3.0 * 2.0 * 4.0 / 3.0 * (double)P * height) + P * height * 4;
  return bytes;
}

// Creates the session's simulation, uploads its inputs and makes its events.
int build_session(ubg_server::Session &ses, const float *flag, const float *vx, const float *vy,
                  const ubg_options *opt) {
  ubg_sim *sim = nullptr;
  int rc = ubg_create(flag, ses.width, ses.height, ses.pwidth, ses.mu, &sim);
  if (rc == UBG_OK && opt) rc = ubg_set_options(sim, opt);
  if (rc == UBG_OK && vx) rc = ubg_upload(sim, UBG_VX, vx);
  if (rc == UBG_OK && vx) rc = ubg_upload(sim, UBG_VX_BACK, vx);
  if (rc == UBG_OK && vy) rc = ubg_upload(sim, UBG_VY, vy);
  if (rc == UBG_OK && vy) rc = ubg_upload(sim, UBG_VY_BACK, vy);
  cudaEvent_t evc[2] = {nullptr, nullptr};
  void *st = nullptr;
  if (rc == UBG_OK) rc = ubg_stream(sim, &st);
  for (cudaEvent_t &e : evc)
    if (rc == UBG_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      rc = srv_fail(UBG_ECUDA, "event creation failed");
    }
  if (rc != UBG_OK) {
    for (cudaEvent_t e : evc)
      if (e) cudaEventDestroy(e);
    if (sim) ubg_destroy(sim);
    return rc;
  }
  ses.sim = sim;
  ses.st = (cudaStream_t)st;
  ses.evc[0] = evc[0];
  ses.evc[1] = evc[1];
  return UBG_OK;
}
}  // namespace

void ubg_server::admit_pending() {
  for (;;) {
    int id = 0;
    ubg_server::Session inputs;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (pending.empty()) return;
      id = pending.front();
      Session &p = sessions[id];
      if (used + p.bytes > budget) return;
      used += p.bytes;  // reserved while the session is built
      pending.pop_front();
      inputs.width = p.width;
      inputs.height = p.height;
      inputs.pwidth = p.pwidth;
      inputs.mu = p.mu;
      inputs.flag.swap(p.flag);
      inputs.vx.swap(p.vx);
      inputs.vy.swap(p.vy);
      inputs.has_opt = p.has_opt;
      inputs.opt = p.opt;
      p.building = true;
    }
    int rc = build_session(inputs, inputs.flag.data(), inputs.vx.empty() ? nullptr : inputs.vx.data(),
                           inputs.vy.empty() ? nullptr : inputs.vy.data(),
                           inputs.has_opt ? &inputs.opt : nullptr);
    std::lock_guard<std::mutex> lk(mu);
    Session &p = sessions[id];
    if (rc != UBG_OK) {  // its queued requests fail with UBG_ESTATE
      used -= p.bytes;
      sessions.erase(id);
    } else {
      p.sim = inputs.sim;
      p.st = inputs.st;
      p.evc[0] = inputs.evc[0];
      p.evc[1] = inputs.evc[1];
      p.pending = false;
      p.building = false;
      admitted_from_queue++;
    }
    cv_work.notify_all();
  }
}

int ubg_server_open(ubg_server *s, const float *flag, int width, int height, float pwidth,
                    float mu, const float *vx, const float *vy, const ubg_options *opt,
                    int *session) {
  if (!s || !flag || !session) return srv_fail(UBG_EINVAL, "null argument");
  int rc = UBG_OK;
  const size_t bytes = session_bytes(width, height, opt, &rc);
  if (rc) return rc;
  ubg_server::Session ses;
  ses.width = width;
  ses.height = height;
  ses.pwidth = pwidth;
  ses.mu = mu;
  ses.bytes = bytes;
  ses.cells = (long long)width * height;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const bool fits = s->used + bytes <= s->budget;
    if (s->admission == UBG_ADMIT_QUEUE && bytes <= s->budget && (!fits || !s->pending.empty())) {
      // wait in open order for memory: keep the inputs on the host
      const size_t n = (size_t)width * height;
      ses.pending = true;
      ses.flag.assign(flag, flag + n);
      if (vx) ses.vx.assign(vx, vx + (size_t)(width - 1) * height);
      if (vy) ses.vy.assign(vy, vy + (size_t)width * (height - 1));
      if (opt) {
        ses.has_opt = true;
        ses.opt = *opt;
      }
      *session = s->next_session++;
      s->sessions[*session] = std::move(ses);
      s->pending.push_back(*session);
      set_last_error("");
      return UBG_OK;
    }
    if (!fits) {
      s->rejected++;
      return srv_fail(UBG_EBUSY, "device-memory budget exhausted: session not admitted");
    }
    s->used += bytes;  // reserved while the session is built
  }
  rc = build_session(ses, flag, vx, vy, opt);
  std::lock_guard<std::mutex> lk(s->mu);
  if (rc != UBG_OK) {
    s->used -= bytes;
    return rc;
  }
  *session = s->next_session++;
  s->sessions[*session] = ses;
  return UBG_OK;
}

int ubg_server_close(ubg_server *s, int session) {
  if (!s) return srv_fail(UBG_EINVAL, "null handle");
  ubg_server::Session ses;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->sessions.find(session);
    if (it == s->sessions.end()) return srv_fail(UBG_EINVAL, "unknown session");
    bool queued = false;
    for (auto id : s->queue)
      if (s->reqs[id].session == session) queued = true;
    if (it->second.building) return srv_fail(UBG_EBUSY, "session is being admitted");
    if (it->second.pending) {
      // never built: drop it from the waiting line (its queued requests
      // fail with UBG_ESTATE)
      s->pending.erase(std::remove(s->pending.begin(), s->pending.end(), session),
                       s->pending.end());
      s->sessions.erase(it);
      s->cv_work.notify_all();
    } else {
      if (it->second.busy || queued) return srv_fail(UBG_EBUSY, "session has requests in flight");
      ses = std::move(it->second);
      s->sessions.erase(it);
      s->used -= ses.bytes;
    }
  }
  for (cudaEvent_t e : ses.evc)
    if (e) cudaEventDestroy(e);
  if (ses.sim) ubg_destroy(ses.sim);
  s->admit_pending();  // freed memory may admit waiting sessions
  return UBG_OK;
}

int ubg_server_submit(ubg_server *s, int session, int steps, float cfl, uint64_t *request) {
  if (!s || !request || steps < 1 || !(cfl > 0.0f)) return srv_fail(UBG_EINVAL, "bad argument");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->sessions.count(session)) return srv_fail(UBG_EINVAL, "unknown session");
    uint64_t id = s->next_req++;
    ubg_server::Request r;
    r.session = session;
    r.steps = steps;
    r.cfl = cfl;
    r.t_submit = now_ms();
    s->reqs[id] = r;
    s->queue.push_back(id);
    *request = id;
  }
  s->cv_work.notify_all();
  return UBG_OK;
}

int ubg_server_wait(ubg_server *s, uint64_t request, double *latency_ms) {
  if (!s) return srv_fail(UBG_EINVAL, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(request);
  if (it == s->reqs.end()) return srv_fail(UBG_EINVAL, "unknown request");
  s->cv_done.wait(lk, [&] { return it->second.finished; });
  if (latency_ms) *latency_ms = it->second.t_end - it->second.t_submit;
  int e = it->second.error;
  return e ? srv_fail(e, "request failed") : UBG_OK;
}

int ubg_server_drain(ubg_server *s) {
  if (!s) return srv_fail(UBG_EINVAL, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  // every request of an admitted session done (requests of sessions still
  // waiting for memory stay queued)
  s->cv_done.wait(lk, [&] {
    if (!s->active.empty()) return false;
    for (uint64_t id : s->queue) {
      auto it = s->sessions.find(s->reqs[id].session);
      if (it != s->sessions.end() && !it->second.pending) return false;
    }
    return true;
  });
  return UBG_OK;
}

int ubg_server_session_sim(ubg_server *s, int session, ubg_sim **sim) {
  if (!s || !sim) return srv_fail(UBG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->sessions.find(session);
  if (it == s->sessions.end()) return srv_fail(UBG_EINVAL, "unknown session");
  if (!it->second.sim) return srv_fail(UBG_ESTATE, "session still waiting for device memory");
  *sim = it->second.sim;
  return UBG_OK;
}

int ubg_server_stats(ubg_server *s, ubg_serve_stats *out) {
  if (!s || !out) return srv_fail(UBG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->sessions = (int)s->sessions.size();
  out->queued = (int)s->queue.size();
  out->active = (int)s->active.size();
  out->completed = s->completed;
  out->rejected_sessions = s->rejected;
  out->cell_steps = s->cell_steps;
  out->device_bytes_used = s->used;
  out->busy_ms = s->t_first < 0.0 ? 0.0 : s->t_last - s->t_first;
  out->fused_steps = s->fused_steps;
  out->fused_member_steps = s->fused_member_steps;
  out->worker_fused_ms = s->worker_fused_ms;
  out->worker_streams_ms = s->worker_streams_ms;
  out->pending_sessions = (int)s->pending.size();
  out->admitted_from_queue = s->admitted_from_queue;
  if (!s->latencies.empty()) {
    std::vector<double> v = s->latencies;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
      size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(q * (double)v.size()) - 1);
      return v[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = v.back();
  }
  return UBG_OK;
}
