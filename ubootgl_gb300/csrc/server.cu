// Step server (extension): continuous batching of step requests over
// sessions whose fields stay resident on the device.
//
// A session is one simulation handle (its own fields, stream and captured
// step graph).  Sessions are admitted against a device-memory budget when
// they are opened.  A request asks for k steps of one session.  The worker
// thread admits queued requests in arrival order whenever a slot is free
// (at most max_active requests in flight, one per session), enqueues all k
// steps of an admitted request on its session's stream at once, and polls
// the streams' completion events: requests that arrive while others run on
// the GPU join as soon as a slot frees, and the device overlaps the work of
// every in-flight session.  Sessions touch only their own memory, so a
// session's result does not depend on what else is in flight.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
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

struct ubg_server {
  struct Session {
    ubg_sim *sim = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    size_t bytes = 0;
    long long cells = 0;
    bool busy = false;
  };
  struct Request {
    int session = 0;
    int steps = 0;
    float cfl = 0.5f;
    double t_submit = 0, t_admit = 0, t_end = 0;
    bool finished = false;
    int error = 0;
  };

  size_t budget = 0, used = 0;
  int max_active = 1;
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
  double t_first = -1.0, t_last = 0.0;
  bool stop = false;
  std::thread worker;

  void run() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      // admit in arrival order while slots are free
      for (auto it = queue.begin(); it != queue.end() && (int)active.size() < max_active;) {
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
        if (s.busy) {
          ++it;
          continue;
        }
        s.busy = true;
        r.t_admit = now_ms();
        if (t_first < 0.0) t_first = r.t_admit;
        // enqueue every step of the request on the session's stream
        int rc = UBG_OK;
        for (int k = 0; k < r.steps && rc == UBG_OK; k++) rc = ubg_step_cfl(s.sim, r.cfl);
        if (rc == UBG_OK && cudaEventRecord(s.ev, s.st) != cudaSuccess) rc = UBG_ECUDA;
        if (rc != UBG_OK) {
          r.finished = true;
          r.error = rc;
          s.busy = false;
          it = queue.erase(it);
          cv_done.notify_all();
          continue;
        }
        active.push_back(*it);
        it = queue.erase(it);
      }
      if (active.empty()) {
        if (stop && queue.empty()) return;
        cv_work.wait(lk);
        continue;
      }
      // completion polling
      bool any = false;
      for (size_t i = 0; i < active.size();) {
        Request &r = reqs[active[i]];
        Session &s = sessions[r.session];
        cudaError_t q = cudaEventQuery(s.ev);
        if (q == cudaErrorNotReady) {
          i++;
          continue;
        }
        r.t_end = now_ms();
        r.finished = true;
        if (q != cudaSuccess) {
          cudaGetLastError();
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
      } else {
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
  for (auto &kv : s->sessions) {
    cudaEventDestroy(kv.second.ev);
    ubg_destroy(kv.second.sim);
  }
  delete s;
  set_last_error("");
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
    if (cudaEventCreateWithFlags(&ses.ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      rc = srv_fail(UBG_ECUDA, "event creation failed");
    }
  }
  if (rc != UBG_OK) {
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
  cudaEventDestroy(ses.ev);
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
