// Step server (extension): continuous batching of step requests over
// sessions whose fields stay resident on the device.
//
// A session is one simulation handle (its own fields and stream).  Sessions
// are admitted against a device-memory budget when they are opened.  A
// request asks for k steps of one session.  The worker thread admits queued
// requests in arrival order whenever a slot is free (one request in flight
// per session; at most max_active stream requests and 4 * max_active fused
// requests).  Requests of sessions that the fused form covers (FP32, fixed
// V-cycle count, at most 1M cells; see FusedStepper) are stepped together:
// every worker iteration enqueues ONE step of every such request as one
// launch per kernel over all of them, so a request that arrives joins at
// the next step boundary and leaves after its k-th step (iteration-level
// continuous batching, at most two steps in flight).  Other sessions (mixed
// precision, tolerance mode, larger grids) enqueue their k steps on their
// own stream.  The worker polls completion events.  Sessions touch only
// their own memory and the fused step is bit-identical to stepping alone,
// so a session's result does not depend on what else is in flight.
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
  };
  struct Request {
    int session = 0;
    int steps = 0;
    float cfl = 0.5f;
    double t_submit = 0, t_admit = 0, t_end = 0;
    bool fused = false;  // stepped by the fused stepper
    int remaining = 0;   // fused steps not yet enqueued
    int enq = 0;         // stream steps enqueued so far
    int chunks = 0;      // stream chunks enqueued so far
    bool finished = false;
    int error = 0;
  };

  size_t budget = 0, used = 0;
  int max_active = 1;
  int mode = UBG_SERVE_FUSED;
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
  bool stop = false;
  std::unique_ptr<FusedStepper> fs;
  std::thread worker;

  // Enqueues the next chunk of a stream request's steps once at most one
  // chunk is still queued (chunk i records evc[i % 2]).  Keeping only a few
  // steps queued per session keeps the worker out of a full launch queue,
  // where every launch would block it.
  int stream_topup(Request &r, Session &s) {
    if (r.enq >= r.steps) return UBG_OK;
    if (r.chunks >= 2) {
      cudaError_t q = cudaEventQuery(s.evc[r.chunks % 2]);
      if (q == cudaErrorNotReady) return UBG_OK;
      if (q != cudaSuccess) {
        cudaGetLastError();
        return UBG_ECUDA;
      }
    }
    const double t0 = now_ms();
    const int n = std::min(kChunkSteps, r.steps - r.enq);
    int rc = UBG_OK;
    for (int k = 0; k < n && rc == UBG_OK; k++) rc = ubg_step_cfl(s.sim, r.cfl);
    if (rc == UBG_OK && cudaEventRecord(s.evc[r.chunks % 2], s.st) != cudaSuccess) rc = UBG_ECUDA;
    r.enq += n;
    r.chunks++;
    worker_streams_ms += now_ms() - t0;
    return rc;
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
          rc = stream_topup(r, s);
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
      if (active.empty()) {
        if (stop && queue.empty()) return;
        cv_work.wait(lk);
        continue;
      }
      bool stepped = fused_tick();
      // stream top-ups and completion polling
      bool any = false;
      for (size_t i = 0; i < active.size();) {
        Request &r = reqs[active[i]];
        Session &s = sessions[r.session];
        if (r.fused && r.remaining > 0) {
          i++;
          continue;
        }
        cudaError_t q = cudaSuccess;
        if (!r.fused && r.enq < r.steps) {
          const int c0 = r.chunks;
          if (stream_topup(r, s) != UBG_OK) {
            q = cudaErrorUnknown;
          } else {
            stepped |= r.chunks != c0;
            i++;
            continue;
          }
        } else {
          // the request's last work: the stepper's event, or its last chunk
          q = cudaEventQuery(r.fused ? s.evc[0] : s.evc[(r.chunks - 1) % 2]);
          if (q == cudaErrorNotReady) {
            i++;
            continue;
          }
        }
        r.t_end = now_ms();
        r.finished = true;
        if (q != cudaSuccess) {
          cudaGetLastError();
          r.error = UBG_ECUDA;
        } else if (r.fused && fs->failed()) {
          set_last_error("fused step: a launch found a table it was not made for");
          r.error = UBG_ECUDA;
        }
        s.busy = false;
        latencies.push_back(r.t_end - r.t_submit);
        cell_steps += s.cells * r.steps;
        completed++;
        t_last = r.t_end;
        active.erase(active.begin() + i);
        any = true;
      }
      if (any) {
        cv_done.notify_all();
      } else if (!stepped) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
        lk.lock();
      }
    }
  }
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
  s->fs.reset();
  for (auto &kv : s->sessions) {
    for (cudaEvent_t e : kv.second.evc) cudaEventDestroy(e);
    ubg_destroy(kv.second.sim);
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

int ubg_server_open(ubg_server *s, const float *flag, int width, int height, float pwidth,
                    float mu, const float *vx, const float *vy, const ubg_options *opt,
                    int *session) {
  if (!s || !flag || !session) return srv_fail(UBG_EINVAL, "null argument");
  size_t bytes = 0;
  int rc = ubg_device_bytes(width, height, &bytes);
  if (rc) return rc;
  if (opt && opt->precision != UBG_FP32)
    bytes += (size_t)(3.0 * 2.0 * 4.0 / 3.0 * (double)((width + 31) / 32 * 32) * height) +
             (size_t)((width + 31) / 32 * 32) * height * 4;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->used + bytes > s->budget) {
      s->rejected++;
      return srv_fail(UBG_EBUSY, "device-memory budget exhausted: session not admitted");
    }
    s->used += bytes;  // reserved while the session is built
  }
  ubg_sim *sim = nullptr;
  auto unreserve = [&] {
    std::lock_guard<std::mutex> lk(s->mu);
    s->used -= bytes;
  };
  rc = ubg_create(flag, width, height, pwidth, mu, &sim);
  if (rc == UBG_OK && opt) rc = ubg_set_options(sim, opt);
  if (rc == UBG_OK && vx) rc = ubg_upload(sim, UBG_VX, vx);
  if (rc == UBG_OK && vx) rc = ubg_upload(sim, UBG_VX_BACK, vx);
  if (rc == UBG_OK && vy) rc = ubg_upload(sim, UBG_VY, vy);
  if (rc == UBG_OK && vy) rc = ubg_upload(sim, UBG_VY_BACK, vy);
  ubg_server::Session ses;
  if (rc == UBG_OK) {
    void *st = nullptr;
    ubg_stream(sim, &st);
    ses.st = (cudaStream_t)st;
    for (cudaEvent_t &e : ses.evc)
      if (rc == UBG_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        rc = srv_fail(UBG_ECUDA, "event creation failed");
      }
  }
  if (rc != UBG_OK) {
    for (cudaEvent_t e : ses.evc)
      if (e) cudaEventDestroy(e);
    if (sim) ubg_destroy(sim);
    unreserve();
    return rc;
  }
  ses.sim = sim;
  ses.bytes = bytes;
  ses.cells = (long long)width * height;
  std::lock_guard<std::mutex> lk(s->mu);
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
    if (it->second.busy || queued) return srv_fail(UBG_EBUSY, "session has requests in flight");
    ses = it->second;
    s->sessions.erase(it);
    s->used -= ses.bytes;
  }
  for (cudaEvent_t e : ses.evc)
    if (e) cudaEventDestroy(e);
  ubg_destroy(ses.sim);
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
  s->cv_done.wait(lk, [&] { return s->queue.empty() && s->active.empty(); });
  return UBG_OK;
}

int ubg_server_session_sim(ubg_server *s, int session, ubg_sim **sim) {
  if (!s || !sim) return srv_fail(UBG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->sessions.find(session);
  if (it == s->sessions.end()) return srv_fail(UBG_EINVAL, "unknown session");
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
