// cp_serve.cpp -- the served form of World.step: a request server that keeps
// world state resident in HBM and batches requests continuously.
//
// A request is one world plus a horizon (a rollout of `nsteps` steps at `dt`).
// cp_serve_submit checks and lays the world out on the caller's thread and
// queues it.  One server thread then loops over ticks:
//
//   1. admission: queued requests, first come first served, are committed to
//      the device while their state and scratch fit the HBM budget (and the
//      optional cap on bodies stepping at once);
//   2. step: every admitted world advances up to `steps_per_tick` steps in
//      one launch sequence per distinct dt (the same persistent kernels as
//      cp_batch_step); a world stops at its own horizon through its step
//      limit, so requests of any horizon share a tick;
//   3. retire: finished worlds are read back into the request's result, their
//      device memory returns to the pool, and waiters are woken.
//
// Requests arriving while a tick runs join at the next tick, so work of old
// and new requests overlaps on the device.  A world's result does not depend
// on which other worlds share its ticks: every world is stepped by the same
// kernels on its own data, so results match stepping it alone bit for bit.
//
// Optional wide lanes (wide_lanes > 0): large worlds (at least `wide_bodies`
// bodies) then do not join the ticks; each lane thread takes one at a time,
// on a context (a CUDA stream) of its own, and steps it to its horizon
// through the wide kernels (the world spread over the whole GPU), in chunks
// of a few steps so that a cancellation takes effect.  The lanes' work
// overlaps with the ticks of the small worlds on the device.  A lane gives
// one large world a short step, but steps only that world, so under load
// the ticks, which step every admitted world at once, deliver several times
// the throughput; the lanes are off unless configured.  Both classes share
// the HBM budget.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <cstring>
#include <thread>

#include "cp_internal.h"

using namespace cpi;

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum { REQ_PENDING = CP_REQ_PENDING, REQ_ACTIVE = CP_REQ_ACTIVE, REQ_DONE = CP_REQ_DONE, REQ_FAILED = CP_REQ_FAILED,
       REQ_CANCELLED = CP_REQ_CANCELLED };

struct Request {
  int64_t ticket = 0;
  PreparedWorld prep;
  double dt = 0;
  int nsteps = 0;
  int nb = 0;
  size_t bytes = 0;
  int state = REQ_PENDING;
  std::atomic<bool> cancel{false};
  int world = -1;
  long long remaining = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int status = CP_OK;
  std::string error;
  std::vector<cp_body_desc> result;
  cp_step_info info{};
};

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  double pos = q * (double)(v.size() - 1);
  size_t i = (size_t)pos;
  double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

struct cp_server {
  cp_ctx* ctx = nullptr;
  cp_serve_config cfg{};
  std::thread thread;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::atomic<bool> stop{false};
  std::deque<Request*> pending;
  std::vector<Request*> active;  // modified by the server thread only, under mu
  // large worlds: queued for, and stepped by, the wide lanes
  std::deque<Request*> pending_wide;
  std::vector<cp_ctx*> lane_ctx;
  std::vector<std::thread> lanes;
  std::vector<Request*> lane_req;  // the request each lane is stepping, or null
  int wide_bodies = 0;
  std::map<int64_t, std::unique_ptr<Request>> requests;
  int64_t next_ticket = 1;
  size_t bytes_in_use = 0, bytes_peak = 0;
  long long active_bodies = 0;
  // statistics since the last reset
  long long submitted = 0, admitted = 0, completed = 0, failed = 0, cancelled = 0, ticks = 0;
  long long body_steps = 0;
  std::vector<double> latency;
  double t_first = -1, t_last = -1;
  double device_s = 0;

  void finish(Request* r, int state) {
    r->state = state;
    r->t_done = now_s();
    bytes_in_use -= r->bytes;
    active_bodies -= r->nb;
    if (state == REQ_DONE) {
      completed++;
      latency.push_back(r->t_done - r->t_submit);
      body_steps += (long long)r->nb * r->nsteps;
      t_last = r->t_done;
    } else if (state == REQ_FAILED) {
      failed++;
    } else {
      cancelled++;
    }
  }

  void fail_all_active(int status, const std::string& msg) {
    std::lock_guard<std::mutex> lk(mu);
    for (Request* r : active) {
      r->status = status;
      r->error = msg;
      finish(r, REQ_FAILED);
    }
    active.clear();
    cv_done.notify_all();
  }

  bool is_wide(const Request* r) const { return wide_bodies > 0 && !lane_ctx.empty() && r->nb >= wide_bodies; }

  // One wide lane: a large world at a time, stepped to its horizon on the
  // lane's own context.
  void run_lane(int lane) {
    cp_ctx* c = lane_ctx[lane];
    for (;;) {
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
          if (stop) return;
          while (!pending_wide.empty() && pending_wide.front()->cancel) {
            Request* q = pending_wide.front();
            pending_wide.pop_front();
            q->state = REQ_CANCELLED;
            cancelled++;
            cv_done.notify_all();
          }
          if (!pending_wide.empty() && bytes_in_use + pending_wide.front()->bytes <= (size_t)cfg.hbm_budget_bytes) break;
          cv_work.wait(lk);
        }
        r = pending_wide.front();
        pending_wide.pop_front();
        bytes_in_use += r->bytes;
        bytes_peak = std::max(bytes_peak, bytes_in_use);
        active_bodies += r->nb;
        lane_req[lane] = r;
      }
      int st;
      int id = -1;
      {
        std::lock_guard<std::mutex> lc(c->mu);
        cudaSetDevice(c->device);
        DWorldParams* P = (DWorldParams*)&r->prep.host[r->prep.off.P];
        P->step_limit = P->stepnumber + r->nsteps;
        r->prep.w.step_limit = P->step_limit;
        st = commit_world(c, r->prep, &id);
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        if (!st) {
          r->world = id;
          r->state = REQ_ACTIVE;
          r->t_admit = now_s();
          r->remaining = r->nsteps;
          admitted++;
        }
      }
      std::string msg;
      while (!st && r->remaining > 0 && !r->cancel && !stop) {
        const int chunk = (int)std::min<long long>(r->remaining, 16);
        std::lock_guard<std::mutex> lc(c->mu);
        cudaSetDevice(c->device);
        st = world_step_plain(c, id, r->dt, chunk);
        if (!st) r->remaining -= chunk;
      }
      if (stop && !st && r->remaining > 0) {
        std::lock_guard<std::mutex> lc(c->mu);
        destroy_world(c, id);
        return;
      }
      if (!st && !r->cancel) {
        std::lock_guard<std::mutex> lc(c->mu);
        r->result.resize(r->nb);
        st = read_bodies(c, id, r->result.data());
        if (!st) st = read_info(c, id, &r->info);
      }
      if (st) msg = last_error();
      if (id >= 0) {
        std::lock_guard<std::mutex> lc(c->mu);
        destroy_world(c, id);
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        r->status = st;
        r->error = msg;
        lane_req[lane] = nullptr;
        finish(r, r->cancel ? REQ_CANCELLED : (st ? REQ_FAILED : REQ_DONE));
        cv_done.notify_all();
      }
      cv_work.notify_all();  // budget freed: a queued request may fit now
    }
  }

  void run() {
    for (;;) {
      std::vector<Request*> admit;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !pending.empty() || !active.empty(); });
        if (stop) return;
        while (!pending.empty()) {
          Request* r = pending.front();
          if (r->cancel) {
            pending.pop_front();
            r->state = REQ_CANCELLED;
            cancelled++;
            cv_done.notify_all();
            continue;
          }
          const bool idle = active.empty() && admit.empty();
          if (bytes_in_use + r->bytes > (size_t)cfg.hbm_budget_bytes) break;
          if (cfg.max_active_bodies > 0 && !idle && active_bodies + r->nb > cfg.max_active_bodies) break;
          pending.pop_front();
          bytes_in_use += r->bytes;
          bytes_peak = std::max(bytes_peak, bytes_in_use);
          active_bodies += r->nb;
          admit.push_back(r);
        }
      }
      // commit the admitted worlds (device allocation from the pool + upload)
      {
        std::lock_guard<std::mutex> lc(ctx->mu);
        cudaSetDevice(ctx->device);
        for (Request* r : admit) {
          DWorldParams* P = (DWorldParams*)&r->prep.host[r->prep.off.P];
          P->step_limit = P->stepnumber + r->nsteps;
          r->prep.w.step_limit = P->step_limit;
          int id = -1;
          int st = commit_world(ctx, r->prep, &id);
          std::lock_guard<std::mutex> lk(mu);
          if (st) {
            r->status = st;
            r->error = last_error();
            finish(r, REQ_FAILED);
            cv_done.notify_all();
            continue;
          }
          r->world = id;
          r->state = REQ_ACTIVE;
          r->t_admit = now_s();
          r->remaining = r->nsteps;
          admitted++;
          active.push_back(r);
        }
      }
      std::vector<Request*> act;
      {
        std::lock_guard<std::mutex> lk(mu);
        act = active;
      }
      if (act.empty()) continue;
      // one launch sequence per distinct dt; every world advances m steps or
      // up to its horizon
      long long most = 0;
      for (Request* r : act) most = std::max(most, r->remaining);
      const int m = (int)std::min<long long>(std::max(1, cfg.steps_per_tick), most);
      std::map<double, std::vector<int>> by_dt;
      for (Request* r : act)
        if (r->remaining > 0 && !r->cancel) by_dt[r->dt].push_back(r->world);
      int st = CP_OK;
      std::vector<int> failed;
      std::string fail_msg;
      const double t0 = now_s();
      {
        std::lock_guard<std::mutex> lc(ctx->mu);
        cudaSetDevice(ctx->device);
        for (auto& kv : by_dt) {
          const size_t before = failed.size();
          st = step_worlds(ctx, kv.second.data(), (int)kv.second.size(), kv.first, m, false, &failed);
          if (failed.size() > before && fail_msg.empty()) fail_msg = last_error();
          if (st) break;
        }
      }
      device_s += now_s() - t0;
      if (st) {
        // an error no single world explains (a CUDA error, bad arguments)
        // fails every world of the tick; their memory is released
        std::string msg = last_error();
        {
          std::lock_guard<std::mutex> lc(ctx->mu);
          for (Request* r : act) destroy_world(ctx, r->world);
        }
        fail_all_active(st, msg);
        continue;
      }
      if (!failed.empty()) {
        // a world that cannot complete its steps (a capacity beyond its limit)
        // fails alone: its request ends with the error, the others go on
        std::lock_guard<std::mutex> lc(ctx->mu);
        std::lock_guard<std::mutex> lk(mu);
        for (int id : failed) {
          auto it = std::find_if(act.begin(), act.end(), [&](Request* r) { return r->world == id; });
          if (it == act.end()) continue;
          Request* r = *it;
          destroy_world(ctx, r->world);
          r->status = CP_ERR_CAPACITY;
          r->error = fail_msg;
          finish(r, REQ_FAILED);
          active.erase(std::find(active.begin(), active.end(), r));
          act.erase(it);
        }
        cv_done.notify_all();
      }
      // retire finished and cancelled worlds
      std::vector<Request*> done;
      for (Request* r : act) {
        if (!r->cancel) r->remaining -= std::min<long long>(m, r->remaining);
        if (r->remaining == 0 || r->cancel) done.push_back(r);
      }
      {
        std::lock_guard<std::mutex> lc(ctx->mu);
        for (Request* r : done) {
          int s2 = CP_OK;
          if (!r->cancel) {
            r->result.resize(r->nb);
            s2 = read_bodies(ctx, r->world, r->result.data());
            if (!s2) s2 = read_info(ctx, r->world, &r->info);
          }
          std::string msg = s2 ? last_error() : std::string();
          destroy_world(ctx, r->world);
          std::lock_guard<std::mutex> lk(mu);
          r->status = s2;
          r->error = msg;
          finish(r, r->cancel ? REQ_CANCELLED : (s2 ? REQ_FAILED : REQ_DONE));
          active.erase(std::find(active.begin(), active.end(), r));
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        ticks++;
        if (!done.empty()) cv_done.notify_all();
      }
    }
  }
};

extern "C" {

int cp_serve_start(const cp_serve_config* cfg, cp_server** out) {
  if (!cfg || !out) return fail(CP_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->hbm_budget_bytes <= 0 || cfg->steps_per_tick < 0 || cfg->max_active_bodies < 0 || cfg->max_list_entries < 0)
    return fail(CP_ERR_ARG, "bad server configuration");
  cp_config cc{};
  cc.device = cfg->device;
  cp_ctx* ctx = nullptr;
  int st = cp_create(&cc, &ctx);
  if (st) return st;
  {
    std::lock_guard<std::mutex> lc(ctx->mu);
    st = enable_pool(ctx);
    if (!st && cfg->variant >= 0) {
      if (cfg->variant >= cpk_num_variants()) st = fail(CP_ERR_ARG, "variant %d out of range", cfg->variant);
      ctx->forced = cfg->variant;
    }
    if (cfg->group_bodies > 0) ctx->group_bodies = cfg->group_bodies;
    ctx->list_cap_limit = cfg->max_list_entries;
  }
  if (st) {
    cp_destroy(ctx);
    return st;
  }
  cp_server* s = new cp_server();
  s->ctx = ctx;
  s->cfg = *cfg;
  if (s->cfg.steps_per_tick == 0) s->cfg.steps_per_tick = 2;
  const int nlanes = cfg->wide_lanes > 0 ? cfg->wide_lanes : 0;
  s->wide_bodies = cfg->wide_bodies > 0 ? cfg->wide_bodies : CP_WIDE_BODIES_DEFAULT;
  for (int l = 0; l < nlanes; l++) {
    cp_ctx* lc = nullptr;
    st = cp_create(&cc, &lc);
    if (!st) {
      std::lock_guard<std::mutex> g(lc->mu);
      st = enable_pool(lc);
      lc->wide_bodies = s->wide_bodies;
      lc->list_cap_limit = cfg->max_list_entries;
    }
    if (st) {
      if (lc) cp_destroy(lc);
      for (cp_ctx* x : s->lane_ctx) cp_destroy(x);
      cp_destroy(ctx);
      delete s;
      return st;
    }
    s->lane_ctx.push_back(lc);
  }
  s->lane_req.assign(s->lane_ctx.size(), nullptr);
  s->thread = std::thread([s] { s->run(); });
  for (int l = 0; l < (int)s->lane_ctx.size(); l++) s->lanes.emplace_back([s, l] { s->run_lane(l); });
  *out = s;
  return CP_OK;
}

int cp_serve_stop(cp_server* s) {
  if (!s) return CP_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->thread.joinable()) s->thread.join();
  for (auto& t : s->lanes)
    if (t.joinable()) t.join();
  {
    std::lock_guard<std::mutex> lc(s->ctx->mu);
    for (Request* r : s->active) destroy_world(s->ctx, r->world);
  }
  for (cp_ctx* x : s->lane_ctx) cp_destroy(x);
  cp_destroy(s->ctx);
  delete s;
  return CP_OK;
}

int cp_serve_submit(cp_server* s, const cp_world_desc* desc, double dt, int32_t nsteps, int64_t* ticket) {
  if (!s || !desc || !ticket) return fail(CP_ERR_ARG, "null argument");
  if (!(dt > 0) || nsteps < 1) return fail(CP_ERR_ARG, "need dt > 0 and nsteps >= 1");
  auto r = std::make_unique<Request>();
  int st = prepare_world(desc, r->prep);
  if (st) return st;
  r->dt = dt;
  r->nsteps = nsteps;
  r->nb = r->prep.w.nb;
  r->bytes = r->prep.w.state_bytes + r->prep.w.scratch_bytes;
  if (r->bytes > (size_t)s->cfg.hbm_budget_bytes)
    return fail(CP_ERR_CAPACITY, "the request needs %zu bytes of device memory, more than the whole budget of %lld",
                r->bytes, (long long)s->cfg.hbm_budget_bytes);
  r->t_submit = now_s();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->submitted++;
    if (s->t_first < 0) s->t_first = r->t_submit;
    (s->is_wide(r.get()) ? s->pending_wide : s->pending).push_back(r.get());
    s->requests[r->ticket] = std::move(r);
  }
  s->cv_work.notify_all();
  return CP_OK;
}

int cp_serve_poll(cp_server* s, int64_t ticket, int32_t* state) {
  if (!s || !state) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) return fail(CP_ERR_ARG, "no request %lld", (long long)ticket);
  *state = it->second->state;
  return CP_OK;
}

int cp_serve_wait(cp_server* s, int64_t ticket, double timeout_s, int32_t* state) {
  if (!s) return fail(CP_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) return fail(CP_ERR_ARG, "no request %lld", (long long)ticket);
  Request* r = it->second.get();
  auto finished = [&] { return r->state >= REQ_DONE; };
  bool ok = timeout_s < 0 ? (s->cv_done.wait(lk, finished), true)
                          : s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
  if (state) *state = r->state;
  if (!ok) return fail(CP_ERR_TIMEOUT, "request %lld not finished after %.3f s", (long long)ticket, timeout_s);
  return CP_OK;
}

int cp_serve_result(cp_server* s, int64_t ticket, cp_body_desc* out, int32_t n, cp_step_info* info) {
  if (!s) return fail(CP_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) return fail(CP_ERR_ARG, "no request %lld", (long long)ticket);
  Request* r = it->second.get();
  if (r->state == REQ_FAILED) {
    int st = fail(r->status ? r->status : CP_ERR_CUDA, "request %lld failed: %s", (long long)ticket, r->error.c_str());
    s->requests.erase(it);
    return st;
  }
  if (r->state == REQ_CANCELLED) {
    s->requests.erase(it);
    return fail(CP_ERR_ARG, "request %lld was cancelled", (long long)ticket);
  }
  if (r->state != REQ_DONE) return fail(CP_ERR_ARG, "request %lld has not finished", (long long)ticket);
  if ((!out && n > 0) || n != r->nb) return fail(CP_ERR_ARG, "expected %d bodies", r->nb);
  if (n) std::memcpy(out, r->result.data(), sizeof(cp_body_desc) * n);
  if (info) *info = r->info;
  s->requests.erase(it);
  return CP_OK;
}

int cp_serve_cancel(cp_server* s, int64_t ticket) {
  if (!s) return fail(CP_ERR_ARG, "null server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return fail(CP_ERR_ARG, "no request %lld", (long long)ticket);
    Request* r = it->second.get();
    if (r->state >= REQ_DONE) return CP_OK;
    r->cancel = true;
    if (r->state == REQ_PENDING) {  // never admitted: drop it now
      auto& q = s->is_wide(r) ? s->pending_wide : s->pending;
      auto qi = std::find(q.begin(), q.end(), r);
      if (qi == q.end()) return CP_OK;  // a lane has just taken it; it ends at its next chunk
      q.erase(qi);
      r->state = REQ_CANCELLED;
      s->cancelled++;
      s->cv_done.notify_all();
      return CP_OK;
    }
  }
  s->cv_work.notify_all();
  return CP_OK;
}

int cp_serve_get_stats(cp_server* s, cp_serve_stats* out, int32_t reset) {
  if (!s || !out) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->admitted = s->admitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->cancelled = s->cancelled;
  out->pending = (int64_t)(s->pending.size() + s->pending_wide.size());
  out->active = (int64_t)s->active.size();
  for (Request* r : s->lane_req) out->active += r != nullptr;
  out->ticks = s->ticks;
  out->bytes_in_use = (int64_t)s->bytes_in_use;
  out->bytes_peak = (int64_t)s->bytes_peak;
  out->bytes_budget = s->cfg.hbm_budget_bytes;
  out->body_steps = s->body_steps;
  out->span_s = s->t_first >= 0 && s->t_last >= s->t_first ? s->t_last - s->t_first : 0.0;
  out->device_s = s->device_s;
  out->p50_ms = 1e3 * percentile(s->latency, 0.50);
  out->p99_ms = 1e3 * percentile(s->latency, 0.99);
  out->max_ms = s->latency.empty() ? 0.0 : 1e3 * *std::max_element(s->latency.begin(), s->latency.end());
  double sum = 0;
  for (double v : s->latency) sum += v;
  out->mean_ms = s->latency.empty() ? 0.0 : 1e3 * sum / (double)s->latency.size();
  if (reset) {
    s->submitted = s->admitted = s->completed = s->failed = s->cancelled = s->ticks = 0;
    s->body_steps = 0;
    s->latency.clear();
    s->t_first = s->t_last = -1;
    s->device_s = 0;
    s->bytes_peak = s->bytes_in_use;
  }
  return CP_OK;
}

}  // extern "C"
