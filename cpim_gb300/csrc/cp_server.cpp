// Request server: propagate (AC / GAC), SAC and MAC-solve requests on one GPU,
// continuously batched.
//
// Networks are either registered once and stay resident in HBM (level 0 keeps
// the pristine domains, levels 1..slots are working levels handed to
// requests), or carried by the request and uploaded for its lifetime. A
// request may fix variables to values (the client's choices) before the
// propagation or search runs.
//
// A scheduler thread admits queued requests in arrival order while their
// estimated device footprint fits the HBM budget (a request on a resident
// network also needs a free working level; it waits without holding back the
// requests behind it) and hands them to three lanes, each with its own thread
// and engine (stream):
//   - propagate lane: everything queued when the lane is free runs as one
//     multi-instance batch whose members are (network, level) pairs, loaded
//     from level 0 with the choices applied in one launch, propagated with
//     one launch per phase and read back in one copy (high-priority stream);
//   - SAC lane: the same for SAC requests, on a default-priority stream whose
//     sweep CTAs retire after a few tiles, so that the propagate and solve
//     lanes get SMs during long sweeps instead of waiting behind them;
//   - solve lane(s): MAC solves, run whole on the device, one CTA per search,
//     everything queued when a solver is free in one launch; each request
//     finishes as soon as its own search ends (high-priority streams).
// Requests that arrive while a lane is busy join its next batch. Without
// batching one lane runs every propagate and SAC request alone, in order: the
// one-request-per-launch path. Built only on the public C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cpgpu.h"
#include "cp_gen.h"

struct cp_instance {
  cpgen::Instance I;
};

namespace {

using Clock = std::chrono::steady_clock;

struct Resident {
  int64_t id = 0;
  cpgen::Instance I;          // host copy: solver uploads and choice checks
  cp_net* net = nullptr;      // batch engine; level 0 pristine, 1..slots working
  std::vector<int> free_slots;
  int64_t footprint = 0;
  int refs = 0;               // queued or running requests on it
};

struct Req {
  int64_t id = 0;
  int type = 0;  // 0 propagate, 1 SAC, 2 MAC solve
  const cpgen::Instance* inst = nullptr;  // the request's own network or the resident's host copy
  Resident* res = nullptr;
  std::vector<int> cvar, cval;  // choices: variable cvar[j] fixed to cval[j]
  int slot = -1;                // working level on a resident network
  int64_t footprint = 0;
  Clock::time_point t_submit, t_start, t_done;
  int status = 0;  // 0 queued, 1 admitted, 2 done, < 0 error code
  int inconsistent = 0;
  int64_t deletions = 0, npos = 0, nneg = 0;
  int mac_status = 0;
  std::vector<uint64_t> dom;
  std::vector<int> sol;
  std::string error;
};

int internal_w(int W) { return W <= 2 ? W : (W <= 4 ? 4 : 8); }

int64_t total_values(const cpgen::Instance& I) {
  int64_t tv = 0;
  for (int d : I.dom) tv += d;
  return tv;
}

// Device bytes of a network: relations (both directions), the level stack,
// and the per-network scratch (work lists, queues, bitmaps).
int64_t net_footprint(const cpgen::Instance& I, int levels) {
  const int64_t Wi = internal_w(I.W);
  int64_t rel = 0;
  for (int c = 0; c < I.n_bin(); ++c) rel += (I.dom[I.bx[c]] + I.dom[I.by[c]]) * Wi * 8;
  const int64_t lv = int64_t(levels) * I.n * Wi * 8;
  const int64_t scratch = total_values(I) * 22 + int64_t(I.n) * 64 + int64_t(I.n_bin()) * 48 +
                          int64_t(I.ttup.size()) * 2 + 65536;
  return rel + lv + scratch;
}

// Device bytes a request adds to a batch (work lists, tiles, descriptors).
int64_t batch_share(const cpgen::Instance& I) {
  return total_values(I) * 16 + int64_t(I.n) * (32 + 16 * internal_w(I.W)) + 4096;
}

// Device bytes of one device MAC search: its level stack, assigned flags and
// path.
int64_t search_share(const cpgen::Instance& I) {
  return int64_t(I.n + 3) * I.n * (internal_w(I.W) * 8 + 1) + int64_t(I.n) * 8 + 4096;
}

int upload(cp_engine* e, const cpgen::Instance& I, int levels, cp_net** out) {
  std::vector<int> scope(2 * size_t(I.n_bin()));
  for (int c = 0; c < I.n_bin(); ++c) {
    scope[2 * c] = I.bx[c];
    scope[2 * c + 1] = I.by[c];
  }
  return cp_net_upload(e, I.n, I.dom.data(), I.W, I.init.data(), I.n_bin(), scope.data(), I.brows.data(), I.n_tab(),
                       I.tarity.data(), I.tscope.data(), I.tntup.data(), I.ttup.data(), levels, out);
}

int64_t popcount_all(const uint64_t* d, size_t words) {
  int64_t s = 0;
  for (size_t i = 0; i < words; ++i) s += __builtin_popcountll(d[i]);
  return s;
}

// A choice outside a variable's initial domain, or two different values for
// one variable, leaves a domain empty: the request is inconsistent as posed.
bool choices_empty_a_domain(const cpgen::Instance& I, const std::vector<int>& var, const std::vector<int>& val) {
  for (size_t j = 0; j < var.size(); ++j) {
    const uint64_t w = I.init[size_t(var[j]) * I.W + (val[j] >> 6)];
    if (!((w >> (val[j] & 63)) & 1ull)) return true;
    for (size_t k = 0; k < j; ++k)
      if (var[k] == var[j] && val[k] != val[j]) return true;
  }
  return false;
}

}  // namespace

struct Lane {
  cp_engine* eng = nullptr;
  std::list<Req*> q;  // admitted, waiting for the lane
  std::condition_variable cv;
  std::thread th;
  double busy_s = 0;
};

struct cp_server {
  cp_engine* eA = nullptr;  // propagate lane and resident networks
  cp_engine* eB = nullptr;  // first solver
  cp_engine* eS = nullptr;  // SAC lane (created by the server)
  int64_t budget = 0;
  int max_batch = 256;
  bool batching = true;
  int64_t solve_limit_ms = 600000;
  std::mutex mu;      // queues, requests, residents, accounting
  std::mutex eng_mu;  // use of eA (propagate lane, registration)
  std::condition_variable cv_sched, cv_solve, cv_done;
  std::list<Req*> pending;
  std::list<Req*> solve_q;
  Lane lanes[2];  // 0: propagate (and SAC without batching), 1: SAC
  double solve_busy_s = 0;
  int64_t mac_timeouts = 0;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  std::unordered_map<int64_t, std::unique_ptr<Resident>> residents;
  int64_t in_use = 0, peak_in_use = 0;
  int64_t next_id = 1, next_res = 1;
  std::atomic<int64_t> ticks{0}, batched_requests{0};
  bool stop = false;
  std::thread sched;
  std::vector<std::thread> solvers;     // one per solve engine
  std::vector<cp_engine*> own_engines;  // solve engines the server created

  void account(int64_t bytes) {  // caller holds mu
    in_use += bytes;
    peak_in_use = std::max(peak_in_use, in_use);
  }

  // Caller holds mu.
  void finish_locked(Req* r) {
    in_use -= r->footprint;
    if (r->res) {
      if (r->slot >= 0) r->res->free_slots.push_back(r->slot);
      r->slot = -1;
      --r->res->refs;
    }
    r->t_done = Clock::now();
    if (r->status >= 0) r->status = 2;
    cv_done.notify_all();
    cv_sched.notify_all();
  }

  void finish(Req* r) {
    std::lock_guard<std::mutex> lk(mu);
    finish_locked(r);
  }

  int lane_of(int type) const { return (type == 1 && batching) ? 1 : 0; }

  // Moves queued requests to the lanes while memory and working levels allow.
  // Caller holds mu.
  void admit() {
    for (auto it = pending.begin(); it != pending.end();) {
      Req* r = *it;
      if (r->res && r->type != 2 && r->res->free_slots.empty()) {  // waits for a working level
        ++it;
        continue;
      }
      if (in_use + r->footprint > budget && in_use > 0) break;  // head of line waits for memory
      it = pending.erase(it);
      account(r->footprint);
      r->status = 1;
      r->t_start = Clock::now();
      if (r->type == 2) {
        solve_q.push_back(r);
        cv_solve.notify_one();
        continue;
      }
      if (r->res) {
        r->slot = r->res->free_slots.back();
        r->res->free_slots.pop_back();
      }
      Lane& L = lanes[lane_of(r->type)];
      L.q.push_back(r);
      L.cv.notify_one();
    }
  }

  void fail_req(Req* r, int rc) {
    r->status = rc;
    r->error = cp_last_error_string();
  }

  // One batch of same-type members (network, level), loaded from level 0
  // with the requests' choices.
  void run_batch(cp_engine* eng, int type, std::vector<Req*>& rq, std::vector<cp_net*>& nets,
                 std::vector<int>& levels) {
    cp_batch* b = nullptr;
    const int k = static_cast<int>(rq.size());
    std::vector<int> em, ev, ea;
    for (int i = 0; i < k; ++i)
      for (size_t j = 0; j < rq[i]->cvar.size(); ++j) {
        em.push_back(i);
        ev.push_back(rq[i]->cvar[j]);
        ea.push_back(rq[i]->cval[j]);
      }
    std::vector<uint8_t> inc(k, 0);
    std::vector<int64_t> off(k + 1, 0);
    for (int i = 0; i < k; ++i) off[i + 1] = off[i] + int64_t(rq[i]->inst->n) * rq[i]->inst->W;
    std::vector<uint64_t> doms(static_cast<size_t>(off[k]));
    cp_stats st{};
    int rc = cp_batch_create_levels(eng, k, nets.data(), levels.data(), &b);
    if (rc == CP_OK) rc = cp_batch_set_graphs(b, 0);
    if (rc == CP_OK) rc = cp_batch_load(b, 0, static_cast<int>(em.size()), em.data(), ev.data(), ea.data());
    if (rc == CP_OK) rc = type == 0 ? cp_batch_ac(b, &st, inc.data()) : cp_batch_sac1(b, &st, inc.data());
    if (rc == CP_OK) rc = cp_batch_dom_get(b, doms.data());
    if (b) cp_batch_destroy(b);
    for (int i = 0; i < k; ++i) {
      Req* r = rq[i];
      if (rc != CP_OK) {
        fail_req(r, rc);
        continue;
      }
      r->inconsistent = inc[i];
      r->dom.assign(doms.begin() + off[i], doms.begin() + off[i + 1]);
    }
    batched_requests += k;
  }

  // The one-request-per-launch path: level copy, choices, one propagation.
  void run_plain(Req* r, cp_net* net, int level) {
    int rc = cp_level_copy(net, 0, level);
    for (size_t j = 0; rc == CP_OK && j < r->cvar.size(); ++j) rc = cp_reduce_to(net, level, r->cvar[j], r->cval[j]);
    cp_stats st{};
    if (rc == CP_OK) rc = r->type == 0 ? cp_enforce_ac(net, level, 0, nullptr, &st) : cp_enforce_sac1(net, level, &st);
    if (rc == CP_OK) {
      r->inconsistent = st.inconsistent;
      r->dom.assign(size_t(r->inst->n) * r->inst->W, 0);
      rc = cp_dom_get(net, level, r->dom.data());
    }
    if (rc != CP_OK) fail_req(r, rc);
  }

  void run_tick(int lane, std::vector<Req*>& tick) {
    cp_engine* eng = lanes[lane].eng;
    std::unique_lock<std::mutex> eg(eng_mu, std::defer_lock);
    if (eng == eA) eg.lock();
    const size_t k = tick.size();
    std::vector<cp_net*> owned(k, nullptr), mnet(k, nullptr);
    std::vector<int> mlevel(k, 0);
    for (size_t i = 0; i < k; ++i) {
      Req* r = tick[i];
      if (r->res) {
        mnet[i] = r->res->net;
        mlevel[i] = r->slot;
      } else {
        const int rc = upload(eng, *r->inst, 2, &owned[i]);
        if (rc != CP_OK) {
          fail_req(r, rc);
          continue;
        }
        mnet[i] = owned[i];
        mlevel[i] = 1;
      }
    }
    if (batching) {
      for (int type = 0; type < 2; ++type) {
        std::vector<Req*> rq;
        std::vector<cp_net*> nets;
        std::vector<int> levels;
        for (size_t i = 0; i < k; ++i)
          if (mnet[i] && tick[i]->type == type) {
            rq.push_back(tick[i]);
            nets.push_back(mnet[i]);
            levels.push_back(mlevel[i]);
          }
        if (!rq.empty()) run_batch(eng, type, rq, nets, levels);
      }
    } else {
      for (size_t i = 0; i < k; ++i)
        if (mnet[i]) run_plain(tick[i], mnet[i], mlevel[i]);
    }
    for (size_t i = 0; i < k; ++i) {
      Req* r = tick[i];
      if (r->status >= 0 && !r->inconsistent && !r->dom.empty())
        r->deletions = popcount_all(r->inst->init.data(), r->inst->init.size()) -
                       popcount_all(r->dom.data(), r->dom.size());
      if (owned[i]) cp_net_destroy(owned[i]);
      finish(r);
    }
    ++ticks;
  }

  void sched_loop() {
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      admit();
      cv_sched.wait_for(lk, std::chrono::milliseconds(2));
    }
  }

  void lane_loop(int li) {
    Lane& L = lanes[li];
    cudaSetDevice(cp_engine_device(L.eng));
    const size_t cap = batching ? static_cast<size_t>(max_batch) : 1;
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      if (L.q.empty()) {
        L.cv.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      std::vector<Req*> tick;
      while (!L.q.empty() && tick.size() < cap) {
        tick.push_back(L.q.front());
        L.q.pop_front();
      }
      lk.unlock();
      const auto t0 = Clock::now();
      run_tick(li, tick);
      const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
      lk.lock();
      L.busy_s += dt;
    }
  }

  // MAC solves: everything queued when a solver is free runs as one batch of
  // device searches (one CTA per search; resident networks are read in place
  // from their pristine level 0, each search in its own level stack), and
  // each request finishes as soon as its own search ends.
  void solve_batch(std::vector<Req*>& rq, cp_engine* eng) {
    std::vector<cp_net*> nets, owned;
    std::vector<int> nch, cv, ca;
    std::vector<Req*> live;
    for (Req* r : rq) {
      cp_net* net = nullptr;
      if (r->res) {
        net = r->res->net;
      } else {
        const int rc = upload(eng, *r->inst, 2, &net);
        if (rc != CP_OK) {
          fail_req(r, rc);
          finish(r);
          continue;
        }
        owned.push_back(net);
      }
      live.push_back(r);
      nets.push_back(net);
      nch.push_back(static_cast<int>(r->cvar.size()));
      cv.insert(cv.end(), r->cvar.begin(), r->cvar.end());
      ca.insert(ca.end(), r->cval.begin(), r->cval.end());
    }
    const int k = static_cast<int>(live.size());
    if (k > 0) {
      int64_t limit;
      {
        std::lock_guard<std::mutex> lk(mu);
        limit = solve_limit_ms;
      }
      cp_mac_batch* b = nullptr;
      int rc = cp_mac_batch_start(eng, k, nets.data(), nch.data(), cv.data(), ca.data(), 1, 0, limit, &b);
      std::vector<uint8_t> done(k, 0), fin(k, 0);
      std::vector<cp_search_result> res(k);
      int left = k;
      while (rc == CP_OK && left > 0) {
        int nd = 0;
        rc = cp_mac_batch_poll(b, done.data(), res.data(), &nd);
        for (int i = 0; rc == CP_OK && i < k; ++i) {
          if (!done[i] || fin[i]) continue;
          Req* r = live[i];
          r->mac_status = res[i].status;
          r->npos = res[i].num_positive;
          r->nneg = res[i].num_negative;
          r->inconsistent = res[i].status == 0;
          r->sol.assign(r->inst->n, -1);
          if (res[i].status == 1) cp_mac_batch_solution(b, i, r->sol.data());
          if (res[i].status == 2) {
            std::lock_guard<std::mutex> lk(mu);
            ++mac_timeouts;
          }
          finish(r);
          fin[i] = 1;
          --left;
        }
        if (rc == CP_OK && left > 0) std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
      for (int i = 0; i < k; ++i)
        if (!fin[i]) {
          fail_req(live[i], rc != CP_OK ? rc : CP_E_STATE);
          finish(live[i]);
        }
      if (b) cp_mac_batch_destroy(b);
    }
    for (cp_net* n : owned) cp_net_destroy(n);
  }

  void solve_loop(cp_engine* eng) {
    cudaSetDevice(cp_engine_device(eng));
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      if (solve_q.empty()) {
        cv_solve.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      std::vector<Req*> rq;
      while (!solve_q.empty() && static_cast<int>(rq.size()) < max_batch) {
        rq.push_back(solve_q.front());
        solve_q.pop_front();
      }
      lk.unlock();
      const auto t0 = Clock::now();
      solve_batch(rq, eng);
      const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
      lk.lock();
      solve_busy_s += dt;
    }
  }

  int submit(const cp_request* q, int64_t* ticket) {
    if (!q || !ticket || q->type < 0 || q->type > 2 || q->n_choice < 0 ||
        (q->n_choice > 0 && (!q->choice_var || !q->choice_val)))
      return CP_E_ARG;
    auto r = std::make_unique<Req>();
    r->type = q->type;
    r->cvar.assign(q->choice_var, q->choice_var + q->n_choice);
    r->cval.assign(q->choice_val, q->choice_val + q->n_choice);
    std::lock_guard<std::mutex> lk(mu);
    if (q->net_id != 0) {
      auto it = residents.find(q->net_id);
      if (it == residents.end()) return CP_E_ARG;
      r->res = it->second.get();
      r->inst = &r->res->I;
    } else {
      if (!q->inst) return CP_E_ARG;
      r->inst = &q->inst->I;
    }
    const cpgen::Instance& I = *r->inst;
    for (int j = 0; j < q->n_choice; ++j)
      if (r->cvar[j] < 0 || r->cvar[j] >= I.n || r->cval[j] < 0 || r->cval[j] >= I.dom[r->cvar[j]]) return CP_E_ARG;
    const int64_t share = r->type == 2 ? search_share(I) : batch_share(I);
    r->footprint = r->res ? share : net_footprint(I, 2) + share;
    r->t_submit = Clock::now();
    r->id = next_id++;
    if (r->res) ++r->res->refs;
    Req* raw = r.get();
    reqs[raw->id] = std::move(r);
    *ticket = raw->id;
    if (choices_empty_a_domain(I, raw->cvar, raw->cval)) {  // answered without the device
      raw->inconsistent = 1;
      raw->t_start = raw->t_submit;
      raw->footprint = 0;
      finish_locked(raw);
      return CP_OK;
    }
    pending.push_back(raw);
    cv_sched.notify_one();
    return CP_OK;
  }
};

extern "C" {

int cp_server_create(cp_engine* batch_engine, cp_engine* solve_engine, int64_t hbm_budget_bytes, int max_batch,
                     int batching, cp_server** out) {
  if (!batch_engine || !solve_engine || !out || batch_engine == solve_engine || hbm_budget_bytes <= 0 ||
      max_batch < 1)
    return CP_E_ARG;
  auto s = std::make_unique<cp_server>();
  s->eA = batch_engine;
  s->eB = solve_engine;
  s->budget = hbm_budget_bytes;
  s->max_batch = max_batch;
  s->batching = batching != 0;
  // Latency lanes on high-priority streams (engines that already hold
  // networks keep their stream).
  cp_engine_set_priority(batch_engine, 1);
  cp_engine_set_priority(solve_engine, 1);
  s->lanes[0].eng = batch_engine;
  if (s->batching) {
    int rc = cp_engine_create(cp_engine_device(batch_engine), &s->eS);
    if (rc == CP_OK) rc = cp_engine_set_priority(s->eS, -1);
    if (rc == CP_OK) rc = cp_engine_set_cta_quota(s->eS, 2);
    if (rc != CP_OK) {
      if (s->eS) cp_engine_destroy(s->eS);
      return rc;
    }
    s->own_engines.push_back(s->eS);
    s->lanes[1].eng = s->eS;
  }
  cp_server* raw = s.get();
  s->sched = std::thread([raw] { raw->sched_loop(); });
  s->lanes[0].th = std::thread([raw] { raw->lane_loop(0); });
  if (s->batching) s->lanes[1].th = std::thread([raw] { raw->lane_loop(1); });
  s->solvers.emplace_back([raw] { raw->solve_loop(raw->eB); });
  *out = s.release();
  return CP_OK;
}

int cp_server_destroy(cp_server* s) {
  if (!s) return CP_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_sched.notify_all();
  s->cv_solve.notify_all();
  for (auto& L : s->lanes) L.cv.notify_all();
  s->sched.join();
  for (auto& L : s->lanes)
    if (L.th.joinable()) L.th.join();
  for (auto& t : s->solvers) t.join();
  for (auto& kv : s->residents)
    if (kv.second->net) cp_net_destroy(kv.second->net);
  for (cp_engine* e : s->own_engines) cp_engine_destroy(e);
  delete s;
  return CP_OK;
}

int cp_server_set_solve_limit(cp_server* s, int64_t ms) {
  if (!s || ms <= 0) return CP_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->solve_limit_ms = ms;
  return CP_OK;
}

int cp_server_set_solvers(cp_server* s, int k) {
  if (!s || k < 1 || k > 64) return CP_E_ARG;
  while (static_cast<int>(s->solvers.size()) < k) {
    cp_engine* e = nullptr;
    int rc = cp_engine_create(cp_engine_device(s->eB), &e);
    if (rc == CP_OK) rc = cp_engine_set_priority(e, 1);
    if (rc != CP_OK) {
      if (e) cp_engine_destroy(e);
      return rc;
    }
    s->own_engines.push_back(e);
    cp_server* raw = s;
    s->solvers.emplace_back([raw, e] { raw->solve_loop(e); });
  }
  return CP_OK;
}

int cp_server_register(cp_server* s, const cp_instance* inst, int slots, int64_t* net_id) {
  if (!s || !inst || !net_id || slots < 1 || slots > 4096) return CP_E_ARG;
  auto res = std::make_unique<Resident>();
  res->I = inst->I;
  res->footprint = net_footprint(res->I, 1 + slots);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->in_use + res->footprint > s->budget) return CP_E_OOM;
    s->account(res->footprint);
  }
  int rc;
  {
    std::lock_guard<std::mutex> eg(s->eng_mu);
    rc = upload(s->eA, res->I, 1 + slots, &res->net);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (rc != CP_OK) {
    s->in_use -= res->footprint;
    return rc;
  }
  for (int l = slots; l >= 1; --l) res->free_slots.push_back(l);
  res->id = s->next_res++;
  *net_id = res->id;
  s->residents[res->id] = std::move(res);
  return CP_OK;
}

int cp_server_unregister(cp_server* s, int64_t net_id) {
  if (!s) return CP_E_ARG;
  std::unique_ptr<Resident> gone;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->residents.find(net_id);
    if (it == s->residents.end()) return CP_E_ARG;
    if (it->second->refs > 0) return CP_E_STATE;  // requests still queued or running on it
    gone = std::move(it->second);
    s->residents.erase(it);
    s->in_use -= gone->footprint;
  }
  std::lock_guard<std::mutex> eg(s->eng_mu);
  cp_net_destroy(gone->net);
  return CP_OK;
}

int cp_submit(cp_server* s, const cp_request* req, int64_t* ticket) {
  if (!s) return CP_E_ARG;
  return s->submit(req, ticket);
}

int cp_submit_instance(cp_server* s, int type, const cp_instance* inst, int64_t* ticket) {
  if (!s || !inst) return CP_E_ARG;
  cp_request q{};
  q.type = type;
  q.inst = inst;
  return s->submit(&q, ticket);
}

int cp_cancel(cp_server* s, int64_t ticket) {
  if (!s) return CP_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return CP_E_ARG;
  Req* r = it->second.get();
  if (r->status != 0) return CP_E_STATE;  // admitted requests run to the end
  s->pending.remove(r);
  r->status = CP_E_CANCELLED;
  r->footprint = 0;
  s->finish_locked(r);
  return CP_OK;
}

int cp_wait(cp_server* s, int64_t ticket, int64_t timeout_ms, cp_result* res) {
  if (!s || !res) return CP_E_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return CP_E_ARG;
  Req* r = it->second.get();
  const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
  while (r->status == 0 || r->status == 1) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && (r->status == 0 || r->status == 1))
      return CP_E_TIMEOUT;
  }
  res->status = r->status;
  res->inconsistent = r->inconsistent;
  res->deletions = r->deletions;
  res->num_positive = r->npos;
  res->num_negative = r->nneg;
  res->mac_status = r->mac_status;
  res->type = r->type;
  res->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
  res->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  return CP_OK;
}

int cp_poll(cp_server* s, int64_t ticket, cp_result* res) {
  if (!s || !res) return CP_E_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return CP_E_ARG;
    if (it->second->status == 0 || it->second->status == 1) return 1;
  }
  return cp_wait(s, ticket, 0, res);
}

int cp_result_domains(cp_server* s, int64_t ticket, uint64_t* out) {
  if (!s || !out) return CP_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->status != 2 || it->second->dom.empty()) return CP_E_STATE;
  std::memcpy(out, it->second->dom.data(), it->second->dom.size() * 8);
  return CP_OK;
}

int cp_result_solution(cp_server* s, int64_t ticket, int* out) {
  if (!s || !out) return CP_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->status != 2 || it->second->sol.empty()) return CP_E_STATE;
  std::memcpy(out, it->second->sol.data(), it->second->sol.size() * sizeof(int));
  return CP_OK;
}

int cp_release(cp_server* s, int64_t ticket) {
  if (!s) return CP_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return CP_E_ARG;
  if (it->second->status == 0 || it->second->status == 1) return CP_E_STATE;
  s->reqs.erase(it);
  return CP_OK;
}

int cp_server_run_trace(cp_server* s, int k, const double* t_arrival_s, const cp_request* reqs, double* latency_ms,
                        int32_t* status, double* stats) {
  if (!s || k < 0 || (k > 0 && (!t_arrival_s || !reqs || !latency_ms || !status))) return CP_E_ARG;
  const int64_t ticks0 = s->ticks, batched0 = s->batched_requests;
  double busy0[3];
  int64_t mto0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    busy0[0] = s->lanes[0].busy_s;
    busy0[1] = s->lanes[1].busy_s;
    busy0[2] = s->solve_busy_s;
    mto0 = s->mac_timeouts;
  }
  const auto t0 = Clock::now();
  std::vector<int64_t> tickets(k, 0);
  std::vector<int> rc(k, CP_OK);
  for (int i = 0; i < k; ++i) {
    const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t_arrival_s[i]));
    while (Clock::now() < due) {
      const auto left = due - Clock::now();
      if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
    }
    rc[i] = s->submit(&reqs[i], &tickets[i]);
  }
  for (int i = 0; i < k; ++i) {
    if (rc[i] != CP_OK) {
      latency_ms[i] = 0;
      status[i] = rc[i];
      continue;
    }
    cp_result r{};
    const int w = cp_wait(s, tickets[i], 3600 * 1000, &r);
    latency_ms[i] = r.latency_ms;
    status[i] = w == CP_OK ? r.status : w;
    cp_release(s, tickets[i]);
  }
  if (stats) {
    stats[0] = static_cast<double>(s->ticks - ticks0);
    stats[1] = static_cast<double>(s->batched_requests - batched0);
    stats[2] = std::chrono::duration<double>(Clock::now() - t0).count();
    std::lock_guard<std::mutex> lk(s->mu);
    stats[3] = static_cast<double>(s->peak_in_use);
    stats[4] = s->lanes[0].busy_s - busy0[0];
    stats[5] = s->lanes[1].busy_s - busy0[1];
    stats[6] = s->solve_busy_s - busy0[2];
    stats[7] = static_cast<double>(s->mac_timeouts - mto0);
  }
  return CP_OK;
}

}  // extern "C"
