// server.cpp -- continuous batching of puncture solves behind the C ABI
// (olgpu_server_*).  Host code only: it drives hierarchies through the
// library's own entry points (olgpu_hierarchy_create, olgpu_cycle_launch /
// olgpu_cycle_poll), so a served solve runs exactly the kernels, graphs and
// stop rule of a solve made alone and gives the same bits.
//
// Threads: `builders` threads make hierarchies (host geometry, plans, device
// allocation, coefficients, graph capture); one scheduler thread admits
// requests (arrival order; a slot and the device footprint must fit) and
// keeps the next cycle of every admitted solve queued on its stream.  With
// batch_max >= 2 the scheduler admits requests in groups instead and a
// builder thread makes and solves each group as one batch (olgpu_batch_*),
// whose results are the solo solves' bit for bit too.
#include "olgpu.h"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

// device bytes per point: 12 FP64 fields and a mask byte; mixed precision
// adds 11 FP32 fields, the colour-packed (A, 1/(c+u)) pairs and 9 FP32
// Anderson vectors; plus a fixed allowance
// for plans, tables and graphs
constexpr long long kBytesPerPointFP64 = 12 * 8 + 1;
constexpr long long kBytesPerPointMixed = 12 * 8 + 11 * 4 + 2 * 4 + 9 * 4 + 1;
constexpr long long kFixedBytes = 64LL << 20;

struct Request {
  long long id = 0;
  olgpu_problem p{};
  long long bytes = 0;
  int blocks = 0;
  double arrival = 0, admitted = 0;
};

struct Built {
  Request r;
  olgpu_hierarchy *h = nullptr;
  olgpu_status st = OLGPU_OK;
};

// olgpu_solve's stop rule for one served solve
struct Track {
  int stop = OLGPU_STOP_TOLERANCE, max_cycles = 200;
  double tol = 0, du_tol = 0, res = 1e12, res_prev = 1e12, du = 0;
  int cycles = 0;
  // r: the cycle's norm; part, change: its residual part and its largest
  // change of u (olgpu_last_cycle)
  bool step(olgpu_status s, double r, double part, double change)
  {
    res_prev = res;
    res = r;
    du = change;
    cycles++;
    if (s != OLGPU_OK || cycles >= max_cycles) return true;
    if (stop == OLGPU_STOP_FIXED) return false;
    if (stop == OLGPU_STOP_ERROR) return part <= tol && change <= du_tol;
    if (!(res > tol)) return true;
    if (stop == OLGPU_STOP_REFERENCE && !(res < res_prev)) return true;
    return false;
  }
};

struct Active {
  Request r;
  olgpu_hierarchy *h = nullptr;
  Track T;
};

// requests admitted together, solved as one batch
struct Group {
  std::vector<Request> rs;
  long long bytes = 0;
};

}  // namespace

struct olgpu_server {
  olgpu_server_config cfg{};
  Clock::time_point t0 = Clock::now();
  std::mutex mu;
  std::condition_variable cv_sched, cv_build, cv_done;
  bool stopping = false;
  long long next_id = 1;
  long long used = 0;                 // device bytes of admitted solves
  std::deque<Request> waiting;        // submitted, not yet admitted
  std::deque<Request> to_build;       // admitted, waiting for a builder
  std::deque<Group> to_solve;         // batching: admitted groups, waiting for a builder
  std::vector<Built> built;           // built, not yet stepping
  int n_building = 0;                 // admitted and not yet stepping
  int n_active = 0, peak_active = 0;  // stepping (scheduler's list size)
  std::map<long long, olgpu_server_result> results;
  std::vector<std::thread> builders;
  std::thread scheduler;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  bool batching() const { return cfg.batch_max >= 2; }
  void builder_loop();
  void scheduler_loop();
  void solve_group(Group &G);
  void finish(const Request &r, olgpu_status st, int cycles, double res, const double *adm, olgpu_hierarchy *keep,
              double du = 0.0);
};

void olgpu_server::finish(const Request &r, olgpu_status st, int cycles, double res, const double *adm,
                          olgpu_hierarchy *keep, double du)
{
  olgpu_server_result out{};
  out.id = r.id;
  out.status = st;
  out.cycles = cycles;
  out.final_res = res;
  out.final_du = du;
  if (adm)
    for (int i = 0; i < OLGPU_MAX_BH; i++) out.adm[i] = adm[i];
  out.queue_s = r.admitted > 0 ? r.admitted - r.arrival : 0.0;
  out.latency_s = now() - r.arrival;
  out.h = keep;
  {
    std::lock_guard<std::mutex> g(mu);
    results[r.id] = out;
  }
  cv_done.notify_all();
}

// One admitted group as one batch: made, solved to the stop rule and
// destroyed on this builder thread; every member's result is reported when
// the batch ends.  A group whose batch cannot be made is retried one request
// at a time, so that one bad request fails alone.
void olgpu_server::solve_group(Group &G)
{
  const int n = (int)G.rs.size();
  std::vector<olgpu_problem> ps(n);
  for (int i = 0; i < n; i++) ps[i] = G.rs[i].p;
  olgpu_batch_config bc;
  olgpu_batch_config_defaults(&bc);
  bc.device = cfg.device;
  bc.precision = cfg.precision;
  bc.nu1 = cfg.nu1;
  bc.nu2 = cfg.nu2;
  bc.blocks = cfg.blocks;
  olgpu_batch *b = nullptr;
  const olgpu_status st = olgpu_batch_create(ps.data(), n, &bc, &b);
  if (st != OLGPU_OK) {
    if (n > 1) {
      for (const Request &r : G.rs) {
        Group one;
        one.rs.push_back(r);
        one.bytes = r.bytes;
        solve_group(one);
      }
      return;
    }
    {
      std::lock_guard<std::mutex> g(mu);
      used -= G.bytes;
      n_building -= n;
    }
    finish(G.rs[0], st, 0, 0.0, nullptr, nullptr);
    cv_sched.notify_one();
    return;
  }
  {
    std::lock_guard<std::mutex> g(mu);
    n_building -= n;
    n_active += n;
    if (n_active > peak_active) peak_active = n_active;
  }
  const olgpu_stop_rule rule{cfg.stop, cfg.max_cycles, cfg.tol, cfg.du_tol};
  std::vector<olgpu_report> reps(n);
  olgpu_batch_solve(b, &rule, reps.data());   // each report holds its own status
  olgpu_batch_destroy(b);
  {
    std::lock_guard<std::mutex> g(mu);
    used -= G.bytes;
    n_active -= n;
  }
  for (int i = 0; i < n; i++)
    finish(G.rs[i], (olgpu_status)reps[i].status, reps[i].cycles, reps[i].final_res, reps[i].adm, nullptr,
           reps[i].final_du);
  cv_sched.notify_one();
}

void olgpu_server::builder_loop()
{
  for (;;) {
    Request r;
    {
      std::unique_lock<std::mutex> g(mu);
      cv_build.wait(g, [&] { return stopping || !to_build.empty() || !to_solve.empty(); });
      if (stopping) return;
      if (!to_solve.empty()) {
        Group G = to_solve.front();
        to_solve.pop_front();
        g.unlock();
        solve_group(G);
        continue;
      }
      r = to_build.front();
      to_build.pop_front();
    }
    Built b;
    b.r = r;
    b.st = olgpu_hierarchy_create(&r.p, cfg.device, &b.h);
    if (b.st == OLGPU_OK && cfg.precision == OLGPU_PREC_MIXED) {
      // the schedule first: it is captured with the mixed cycle
      b.st = olgpu_set_smoother_blocks(b.h, r.blocks);
      if (b.st == OLGPU_OK && cfg.nu1 >= 0) b.st = olgpu_set_inner_sweeps(b.h, cfg.nu1, cfg.nu2);
    }
    if (b.st == OLGPU_OK) b.st = olgpu_set_precision(b.h, cfg.precision);
    if (b.st != OLGPU_OK && b.h) {
      olgpu_hierarchy_destroy(b.h);
      b.h = nullptr;
    }
    {
      std::lock_guard<std::mutex> g(mu);
      built.push_back(b);
    }
    cv_sched.notify_one();
  }
}

void olgpu_server::scheduler_loop()
{
  std::vector<Active> active;
  for (;;) {
    std::vector<Built> ready;
    {
      std::unique_lock<std::mutex> g(mu);
      if (stopping) break;
      // batching: admission in groups, once batch_max requests wait or the
      // oldest has waited batch_window (arrival order, slots and footprint
      // as below); a builder thread makes and solves each group
      while (batching() && !waiting.empty() &&
             ((int)waiting.size() >= cfg.batch_max || now() - waiting.front().arrival >= cfg.batch_window)) {
        Group G;
        while (!waiting.empty() && (int)G.rs.size() < cfg.batch_max && n_active + n_building < cfg.max_active &&
               used + waiting.front().bytes <= cfg.mem_budget) {
          Request r = waiting.front();
          waiting.pop_front();
          used += r.bytes;
          G.bytes += r.bytes;
          r.admitted = now();
          n_building++;
          G.rs.push_back(r);
        }
        if (G.rs.empty()) break;
        to_solve.push_back(G);
        cv_build.notify_one();
      }
      // admission: arrival order, a slot and the footprint must fit
      while (!batching() && !waiting.empty() && n_active + n_building < cfg.max_active &&
             used + waiting.front().bytes <= cfg.mem_budget) {
        Request r = waiting.front();
        waiting.pop_front();
        used += r.bytes;
        r.admitted = now();
        // the smoother layout follows the load unless fixed: per-colour
        // launches while few solves run (one solve is bound by its chain
        // of launches), the cluster-resident smoother beyond
        r.blocks = cfg.blocks >= 0 ? cfg.blocks : (n_active + n_building < cfg.busy ? 0 : 16);
        n_building++;
        to_build.push_back(r);
        cv_build.notify_one();
      }
      ready.swap(built);
    }
    for (Built &b : ready) {
      if (b.st != OLGPU_OK) {
        {
          std::lock_guard<std::mutex> g(mu);
          used -= b.r.bytes;
          n_building--;
        }
        finish(b.r, b.st, 0, 0.0, nullptr, nullptr);
        continue;
      }
      Active a;
      a.r = b.r;
      a.h = b.h;
      a.T.stop = cfg.stop;
      a.T.max_cycles = cfg.max_cycles;
      a.T.tol = cfg.tol > 0 ? cfg.tol : b.r.p.tol;
      a.T.du_tol = cfg.du_tol > 0 ? cfg.du_tol : a.T.tol;
      const olgpu_status st = olgpu_cycle_launch(a.h);
      {
        std::lock_guard<std::mutex> g(mu);
        n_building--;
        if (st == OLGPU_OK) {
          n_active++;
          if (n_active > peak_active) peak_active = n_active;
        } else {
          used -= b.r.bytes;
        }
      }
      if (st == OLGPU_OK)
        active.push_back(a);
      else {
        olgpu_hierarchy_destroy(a.h);
        finish(b.r, st, 0, 0.0, nullptr, nullptr);
      }
    }
    bool progressed = !ready.empty();
    for (size_t i = 0; i < active.size();) {
      Active &a = active[i];
      int done = 0;
      double res = 0;
      olgpu_status st = olgpu_cycle_poll(a.h, 0, &done, &res);
      if (st == OLGPU_OK && !done) {
        i++;
        continue;
      }
      progressed = true;
      double part = res, change = 0;
      olgpu_last_cycle(a.h, &part, &change);
      if (!a.T.step(st, res, part, change)) {
        st = olgpu_cycle_launch(a.h);   // the next cycle; a failure ends the solve
        if (st == OLGPU_OK) {
          i++;
          continue;
        }
      }
      double adm[OLGPU_MAX_BH] = {0};
      olgpu_adm_mass(a.h, adm);
      const olgpu_status rs = st;
      olgpu_hierarchy *keep = cfg.keep_solutions ? a.h : nullptr;
      if (!keep) olgpu_hierarchy_destroy(a.h);
      {
        std::lock_guard<std::mutex> g(mu);
        used -= a.r.bytes;
        n_active--;
      }
      finish(a.r, rs, a.T.cycles, a.T.res, adm, keep, a.T.du);
      active[i] = active.back();
      active.pop_back();
    }
    if (!progressed) {
      std::unique_lock<std::mutex> g(mu);
      if (active.empty() && waiting.empty() && built.empty() && !stopping)
        cv_sched.wait(g, [&] { return stopping || !waiting.empty() || !built.empty(); });
      else
        cv_sched.wait_for(g, std::chrono::microseconds(20));
    }
  }
  for (Active &a : active) olgpu_hierarchy_destroy(a.h);
}

extern "C" {

void olgpu_server_config_defaults(olgpu_server_config *c)
{
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->device = -1;
  c->mem_budget = 64LL << 30;
  c->max_active = 32;
  c->precision = OLGPU_PREC_MIXED;
  c->stop = OLGPU_STOP_TOLERANCE;
  c->max_cycles = 200;
  c->tol = 0.0;
  c->builders = 2;
  c->nu1 = -1;
  c->nu2 = -1;
  c->blocks = -1;
  c->busy = 4;
  c->keep_solutions = 0;
  c->du_tol = 0.0;
  c->batch_max = 0;
  c->batch_window = 0.02;
}

olgpu_status olgpu_server_create(const olgpu_server_config *c, olgpu_server **out)
{
  if (!c || !out) return OLGPU_ERR_INVALID_ARG;
  if (c->max_active < 1 || c->builders < 1 || c->max_cycles < 1 || c->mem_budget <= 0 ||
      (c->precision != OLGPU_PREC_FP64 && c->precision != OLGPU_PREC_MIXED) || c->stop < OLGPU_STOP_REFERENCE ||
      c->stop > OLGPU_STOP_ERROR || c->batch_window < 0.0 ||
      (c->batch_max >= 2 && c->keep_solutions))   // a batch's hierarchies are not handed out
    return OLGPU_ERR_INVALID_ARG;
  olgpu_server *s = new olgpu_server();
  s->cfg = *c;
  for (int i = 0; i < c->builders; i++) s->builders.emplace_back([s] { s->builder_loop(); });
  s->scheduler = std::thread([s] { s->scheduler_loop(); });
  *out = s;
  return OLGPU_OK;
}

olgpu_status olgpu_server_submit(olgpu_server *s, const olgpu_problem *p, long long *id)
{
  if (!s || !p || !id) return OLGPU_ERR_INVALID_ARG;
  if (p->method != OLGPU_METHOD_VCYCLE) return OLGPU_ERR_INVALID_ARG;   // the scheduler steps V-cycles
  if (p->equation == OLGPU_EQ_BOWEN_YORK) return OLGPU_ERR_INVALID_ARG;   // four unknowns in turn: olgpu_solve
  static const int kMaxBoxes = 1024;
  std::vector<olgpu_box_info> boxes(kMaxBoxes);
  int nb = 0;
  const olgpu_status st = olgpu_plan_boxes(p, boxes.data(), kMaxBoxes, &nb, nullptr, nullptr);
  if (st != OLGPU_OK) return st;
  long long pts = 0;
  for (int g = 0; g < nb; g++) pts += (long long)boxes[g].nx * boxes[g].ny * boxes[g].nz;
  Request r;
  r.p = *p;
  r.bytes = pts * (s->cfg.precision == OLGPU_PREC_MIXED ? kBytesPerPointMixed : kBytesPerPointFP64) + kFixedBytes;
  r.arrival = s->now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r.id = s->next_id++;
    *id = r.id;
    if (r.bytes <= s->cfg.mem_budget) s->waiting.push_back(r);
  }
  if (r.bytes > s->cfg.mem_budget)   // can never fit: refused at once
    s->finish(r, OLGPU_ERR_OOM, 0, 0.0, nullptr, nullptr);
  else
    s->cv_sched.notify_one();
  return OLGPU_OK;
}

olgpu_status olgpu_server_poll(olgpu_server *s, long long id, int wait, int *done, olgpu_server_result *out)
{
  if (!s || !done || !out) return OLGPU_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> g(s->mu);
  if (id < 1 || id >= s->next_id) return OLGPU_ERR_INVALID_ARG;
  auto ready = [&] { return s->results.count(id) > 0; };
  if (wait) s->cv_done.wait(g, ready);
  *done = 0;
  if (!ready()) return OLGPU_OK;
  *out = s->results[id];
  s->results.erase(id);
  *done = 1;
  return OLGPU_OK;
}

olgpu_status olgpu_server_stats(olgpu_server *s, int *active, int *building, int *waiting, int *peak_active)
{
  if (!s) return OLGPU_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  if (active) *active = s->n_active;
  if (building) *building = s->n_building;
  if (waiting) *waiting = (int)s->waiting.size();
  if (peak_active) *peak_active = s->peak_active;
  return OLGPU_OK;
}

olgpu_status olgpu_server_destroy(olgpu_server *s)
{
  if (!s) return OLGPU_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stopping = true;
  }
  s->cv_build.notify_all();
  s->cv_sched.notify_all();
  for (std::thread &t : s->builders) t.join();
  s->scheduler.join();
  for (Built &b : s->built)
    if (b.h) olgpu_hierarchy_destroy(b.h);
  for (auto &kv : s->results)
    if (kv.second.h) olgpu_hierarchy_destroy(kv.second.h);
  delete s;
  return OLGPU_OK;
}

}  // extern "C"
