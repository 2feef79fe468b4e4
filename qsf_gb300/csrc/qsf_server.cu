// qsf_server.cu -- request loop with continuous batching over the public C ABI.
//
// One worker thread owns all device work.  Each round it admits queued requests while
// a slot is free and cudaMemGetInfo reports enough free HBM beyond the reserve
// (creating the solve's grid, uploading or preparing its start state and adding it
// to a qsf_batch), runs the batch for a fixed number of steps, and retires the
// solves whose last step is done (results from their observables rows; grid freed).
// Solves therefore join and leave the running batch between rounds while the others
// keep their wavefunctions resident on the device.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "qsf_gpu.h"

namespace qsf {  // qsf_api.cu, qsf_bluestein.cu
int grid_clear(qsf_grid* g);
int batch_add_nowait(qsf_batch* b, qsf_grid* g, const qsf_step_desc* d, int64_t* slot);
int batch_launch(qsf_batch* b, int64_t steps);
int batch_finish(qsf_batch* b, int64_t* active);
bool fused_length(int n);
int bs_size(int n, int dim);
bool grid_fused(const qsf_grid* g);
int generic_begin(qsf_grid* g, const qsf_step_desc* d);
int generic_enqueue(qsf_grid* g, const qsf_step_desc* d, int64_t first, int64_t count);
int generic_wait(qsf_grid* g, bool* bad);
int generic_rows(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t nsteps);
}

namespace {

using clk = std::chrono::steady_clock;

struct Pending {
  int64_t ticket;
  qsf_request req;
  std::vector<double> coupling;
  std::vector<double> psi0;
  clk::time_point submitted;
};

struct Running {
  int64_t ticket;
  qsf_grid* grid = nullptr;
  int64_t slot = -1;
  int64_t nsteps = 0;
  int64_t remaining = 0;
  int64_t m = 0;
  int nb = 0;
  double dt = 0.0;
  qsf_grid_desc desc{};          // for returning the grid to the pool
  std::vector<double> coupling;  // kept alive while in the batch
  clk::time_point submitted, admitted;
  bool cancel = false;           // qsf_server_cancel: leave after this round
  // a grid without fused kernels (Bluestein lengths): its steps run as member
  // operations on the grid's own stream, beside the batch, with this step program
  bool generic = false;
  qsf_step_desc d{};
  bool bad = false;  // NaN / non-positive norm seen
  int rc = 0;        // error of a queued round
  bool in_round = false;  // has steps in the current round (joined before it was queued)
};

int64_t grid_points(const qsf_grid_desc& d) {
  int64_t m = 1;
  for (int k = 0; k < d.dim; ++k) m *= d.n[k];
  return m;
}

// device bytes a solve holds: psi, static X factor and potential, observables rows,
// coupling rows, plus small tables
size_t solve_bytes(const qsf_request& r) {
  const int64_t m = grid_points(r.grid);
  const int stride = r.grid.gauge == QSF_GAUGE_LENGTH ? 6 : 3;
  size_t b = (size_t)m * (16 + 16 + 8) + (size_t)r.nsteps * (size_t)(3 + r.nborders + stride) * 8 + (1u << 20);
  // Bluestein lengths: the convolution scratch (up to 4 m points) and the member
  // operations' X / P phase tables
  if (!qsf::fused_length((int)r.grid.n[0])) b += (size_t)m * 16 * 6;
  return b;
}

}  // namespace

// Build-time worker trace (-DQSF_SERVER_TRACE): host seconds per phase of the worker
// loop, printed to stderr when the server stops.
#ifdef QSF_SERVER_TRACE
#include <cstdio>
#define QSF_TRACE_T(v) const auto v = clk::now()
#define QSF_TRACE_ADD(s, k, t0) ((s)->trace[k] += std::chrono::duration<double>(clk::now() - (t0)).count())
#else
#define QSF_TRACE_T(v)
#define QSF_TRACE_ADD(s, k, t0)
#endif

struct qsf_server {
  qsf_server_config cfg{};
  int device = 0;  // the caller's current device at qsf_server_start; the worker thread selects it
#ifdef QSF_SERVER_TRACE
  // decide, admit, enqueue, batch, wait, retire, rounds, admits, batch launch (rebuilds)
  // admits of member-operation / batched solves (incl. their first queued steps)
  // admission parts: grid (pool or new), psi upload, batch add / member program begin,
  // grids created new
  double trace[15] = {0};
#endif
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::map<int64_t, qsf_result> results;  // finished, not yet handed out
  std::map<int64_t, Running> running;     // worker thread only
  std::vector<int64_t> cancel_running;    // cancels of admitted solves (under mu)
  std::map<int64_t, bool> admitted_set;   // tickets admitted and not finished (under mu)
  int64_t next_ticket = 1;
  bool stopping = false;
  std::thread worker;
  qsf_batch* batch = nullptr;
  qsf_server_stats stats{};
  // finished solves' grids kept for the next request with the same descriptor: their
  // allocations, static X / potential tables and flux point lists are reused (worker
  // thread only)
  std::vector<std::pair<qsf_grid_desc, qsf_grid*>> pool;
};

namespace {

bool same_grid(const qsf_grid_desc& a, const qsf_grid_desc& b) {
  if (a.dim != b.dim || a.nCAP != b.nCAP || a.potential != b.potential || a.gauge != b.gauge ||
      a.n_fields != b.n_fields || a.p_axis_swap != b.p_axis_swap || a.Ncharge != b.Ncharge ||
      a.Echarge != b.Echarge || a.Nsoft != b.Nsoft || a.Esoft != b.Esoft || a.free_axes != b.free_axes ||
      a.multi_region != b.multi_region || a.absorber != b.absorber || a.mask_dt != b.mask_dt)
    return false;
  for (int k = 0; k < a.dim; ++k)
    if (a.n[k] != b.n[k] || a.dx[k] != b.dx[k]) return false;
  for (int k = 0; k < 4; ++k)
    if (a.border_nodes[k] != b.border_nodes[k]) return false;
  return true;
}

size_t pooled_bytes(const qsf_server* s) {
  size_t b = 0;
  for (const auto& e : s->pool) {
    int64_t m = 1;
    for (int k = 0; k < e.first.dim; ++k) m *= e.first.n[k];
    b += (size_t)m * (16 + 16 + 8);
  }
  return b;
}

void drain_pool(qsf_server* s) {
  for (auto& e : s->pool) qsf_grid_destroy(e.second);
  s->pool.clear();
}

// a grid for this descriptor: a pooled one (the most recently returned) or a new one
int take_grid(qsf_server* s, const qsf_grid_desc& d, qsf_grid** out) {
  for (size_t i = s->pool.size(); i-- > 0;) {
    if (!same_grid(s->pool[i].first, d)) continue;
    qsf_grid* g = s->pool[i].second;
    s->pool.erase(s->pool.begin() + (long)i);
    *out = g;  // psi is overwritten (upload) or cleared on the grid's stream by admit
    return QSF_OK;
  }
  int rc = qsf_grid_create(&d, nullptr, out);
  if (rc == QSF_ENOMEM && !s->pool.empty()) {  // pooled grids hold the memory: free them and retry
    drain_pool(s);
    rc = qsf_grid_create(&d, nullptr, out);
  }
  return rc;
}

// a finished solve's grid goes to the back of the pool; a full pool gives up its least
// recently returned grid (so that a stream of one-off sizes does not crowd out the
// sizes that come back)
void release_grid(qsf_server* s, const qsf_grid_desc& d, qsf_grid* g) {
  s->pool.emplace_back(d, g);
  if ((int)s->pool.size() > s->cfg.max_slots) {
    qsf_grid_destroy(s->pool.front().second);
    s->pool.erase(s->pool.begin());
  }
}

void finish(qsf_server* s, Running& r, int status, const double* rows, int64_t steps) {
#ifdef QSF_SERVER_TRACE
  if (status && status != QSF_ECANCELED)
    std::fprintf(stderr, "qsf_server trace: ticket %lld status %d generic %d in_round %d remaining %lld n %lld: %s\n",
                 (long long)r.ticket, status, (int)r.generic, (int)r.in_round, (long long)r.remaining,
                 (long long)r.desc.n[0], qsf_last_error());
#endif
  qsf_result res{};
  res.status = status;
  res.steps = steps;
  if (rows && steps > 0) {
    const int ncol = 3 + r.nb;
    const double* last = rows + (steps - 1) * ncol;
    res.final_norm = last[0];
    res.final_epot = last[1];
    res.yield = 1.0 - last[0];
    for (int b = 0; b < r.nb; ++b) {
      double acc = 0.0;
      for (int64_t k = 0; k < steps; ++k) acc += rows[k * ncol + 3 + b] * r.dt;
      res.flux_integral[b] = acc;
    }
  }
  const auto now = clk::now();
  res.queue_s = std::chrono::duration<double>(r.admitted - r.submitted).count();
  res.latency_s = std::chrono::duration<double>(now - r.submitted).count();
  std::lock_guard<std::mutex> lk(s->mu);
  s->results[r.ticket] = res;
  s->admitted_set.erase(r.ticket);
  s->stats.completed++;
  s->stats.in_flight--;
  if (status == QSF_OK) s->stats.grid_point_steps += (double)r.m * (double)steps;
  s->cv_done.notify_all();
}

// admit one request: grid, start state, batch membership (nowait: while a round of the
// batch runs; the new member joins the next round)
int admit(qsf_server* s, Pending& p, Running& r, bool nowait) {
  qsf_grid* g = nullptr;
  QSF_TRACE_T(t_grid);
#ifdef QSF_SERVER_TRACE
  const size_t pooled = s->pool.size();
#endif
  int rc = take_grid(s, p.req.grid, &g);
  QSF_TRACE_ADD(s, 11, t_grid);
#ifdef QSF_SERVER_TRACE
  if (s->pool.size() == pooled) s->trace[14] += 1.0;
#endif
  if (rc) return rc;
  QSF_TRACE_T(t_upload);
  const int64_t m = grid_points(p.req.grid);
  if (!p.psi0.empty()) {
    rc = qsf_upload(g, p.psi0.data(), m);
  } else {  // gaussian(0, 1) added to a cleared psi, on the grid's own stream
    rc = qsf::grid_clear(g);
    if (!rc) rc = qsf_add_gaussian(g, 0.0, 1.0);
    if (!rc) rc = qsf_normalize(g, nullptr);
  }
  QSF_TRACE_ADD(s, 12, t_upload);
  if (rc) {
    qsf_grid_destroy(g);
    return rc;
  }
  r.ticket = p.ticket;
  r.grid = g;
  r.desc = p.req.grid;
  r.nsteps = p.req.nsteps;
  r.remaining = p.req.nsteps;
  r.m = m;
  r.nb = (p.req.obs & QSF_OBS_FLUX) ? p.req.nborders : 0;
  r.dt = p.req.dt;
  r.coupling = std::move(p.coupling);
  r.submitted = p.submitted;
  r.admitted = clk::now();
  qsf_step_desc d{};
  d.mode = p.req.mode;
  d.dt = p.req.dt;
  d.nsteps = p.req.nsteps;
  d.coupling = r.coupling.empty() ? nullptr : r.coupling.data();
  d.obs = p.req.obs;
  d.nborders = p.req.nborders;
  for (int b = 0; b < QSF_MAX_BORDERS; ++b) d.border_types[b] = p.req.border_types[b];
  d.box_size = p.req.box_size;
  QSF_TRACE_T(t_add);
  if (!qsf::grid_fused(g)) {
    r.generic = true;
    r.d = d;
    rc = qsf::generic_begin(g, &r.d);
  } else {
    rc = nowait ? qsf::batch_add_nowait(s->batch, g, &d, &r.slot) : qsf_batch_add(s->batch, g, &d, &r.slot);
  }
  QSF_TRACE_ADD(s, 13, t_add);
  if (rc) {
    qsf_grid_destroy(g);
    r.grid = nullptr;
  }
  return rc;
}

void worker_loop(qsf_server* s) {
  // a new host thread starts on device 0: select the device the server was started on
  // (one process per GPU selects its own before qsf_server_start)
  cudaSetDevice(s->device);
  std::vector<double> rows;
  for (;;) {
    // admission
    std::vector<Pending> take;
    QSF_TRACE_T(t_decide);
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->running.empty() && s->queue.empty()) {
        if (s->stopping) break;
        s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
      size_t free_b = 0, total_b = 0;
      cudaMemGetInfo(&free_b, &total_b);
      const double reserve = s->cfg.hbm_reserve_gb * 1e9;
      double budget = (double)free_b - reserve + (double)pooled_bytes(s);  // pooled grids can be freed
      const double capacity = (double)total_b - reserve;  // what an otherwise empty device could give
      while (!s->queue.empty() && (int)(s->running.size() + take.size()) < s->cfg.max_slots) {
        const double need = (double)solve_bytes(s->queue.front().req);
        if (need > capacity) {  // can never be admitted: finish it now, do not block the queue
          Pending p = std::move(s->queue.front());
          s->queue.pop_front();
          s->stats.queued--;
          s->stats.completed++;
          qsf_result res{};
          res.status = QSF_ENOMEM;
          res.latency_s = res.queue_s = std::chrono::duration<double>(clk::now() - p.submitted).count();
          s->results[p.ticket] = res;
          s->cv_done.notify_all();
          continue;
        }
        if (need > budget) break;  // fits later: stays queued
        budget -= need;
        take.push_back(std::move(s->queue.front()));
        s->queue.pop_front();
        s->admitted_set[take.back().ticket] = true;
        s->stats.queued--;
        s->stats.admitted++;
        s->stats.in_flight++;
      }
      // nothing resident and the queue head has to wait for memory: sleep until a
      // submit, a cancel or a stop (or 20 ms) instead of spinning on cudaMemGetInfo
      if (take.empty() && s->running.empty()) {
        if (s->stopping) break;
        s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
      for (int64_t t : s->cancel_running) {
        auto it = s->running.find(t);
        if (it != s->running.end()) it->second.cancel = true;
      }
      s->cancel_running.clear();
    }
    QSF_TRACE_ADD(s, 0, t_decide);
    // Admissions cost host time (grid creation or reuse, psi upload, tables).  While
    // solves are resident, the new ones are prepared after this round's work is queued,
    // so that this host work overlaps the GPU's round: a member-operation solve starts
    // its first steps at once on its own stream, a batched one joins the next round.
    const bool overlap = !s->running.empty();
    auto admit_all = [&]() {
      QSF_TRACE_T(t_admit);
      for (Pending& p : take) {
        Running r;
        r.ticket = p.ticket;
        r.submitted = p.submitted;
        r.admitted = clk::now();
        QSF_TRACE_T(t_one);
        const int rc = admit(s, p, r, overlap);
        if (rc) {
          finish(s, r, rc, nullptr, 0);
          continue;
        }
        if (r.generic && overlap) {
          const int64_t count = std::min<int64_t>(s->cfg.steps_per_round, r.remaining);
          r.d.coupling = r.coupling.empty() ? nullptr : r.coupling.data();
          r.rc = qsf::generic_enqueue(r.grid, &r.d, 0, count);
          r.in_round = true;
        } else {
          r.in_round = !overlap;
        }
#ifdef QSF_SERVER_TRACE
        QSF_TRACE_ADD(s, r.generic ? 9 : 10, t_one);
#endif
        s->running.emplace(r.ticket, std::move(r));
      }
      QSF_TRACE_ADD(s, 1, t_admit);
#ifdef QSF_SERVER_TRACE
      s->trace[7] += (double)take.size();
#endif
    };
    if (!overlap) admit_all();
    if (s->running.empty()) continue;
    QSF_TRACE_T(t_enqueue);
    // one round of steps for every resident solve: the member-operation solves' steps
    // queued on their own streams (they overlap with one another and with the batch),
    // then the batch's round; then the admissions; then the waits
    bool any_fused = false;
    for (auto& kv : s->running) {
      Running& r = kv.second;
      r.in_round = true;
      if (!r.generic) {
        any_fused = true;
        continue;
      }
      const int64_t first = r.nsteps - r.remaining;
      const int64_t count = std::min<int64_t>(s->cfg.steps_per_round, r.remaining);
      r.d.coupling = r.coupling.empty() ? nullptr : r.coupling.data();
      if (!r.cancel && !r.rc && count > 0) r.rc = qsf::generic_enqueue(r.grid, &r.d, first, count);
    }
    QSF_TRACE_ADD(s, 2, t_enqueue);
    QSF_TRACE_T(t_batch);
    int64_t active = 0;
    QSF_TRACE_T(t_launch);
    int rc_run = any_fused ? qsf::batch_launch(s->batch, s->cfg.steps_per_round) : QSF_OK;
    QSF_TRACE_ADD(s, 8, t_launch);
    if (overlap) admit_all();
    if (any_fused && rc_run == QSF_OK) rc_run = qsf::batch_finish(s->batch, &active);
    QSF_TRACE_ADD(s, 3, t_batch);
    QSF_TRACE_T(t_wait);
    for (auto& kv : s->running) {
      Running& r = kv.second;
      if (!r.generic || !r.in_round) continue;
      const int rw = qsf::generic_wait(r.grid, &r.bad);
      if (rw && !r.rc) r.rc = rw;
    }
    QSF_TRACE_ADD(s, 4, t_wait);
    QSF_TRACE_T(t_retire);
#ifdef QSF_SERVER_TRACE
    s->trace[6] += 1.0;
#endif
    // retire finished, cancelled and failed solves.  A numeric failure (QSF_ENUMERIC)
    // belongs to single members, which qsf_batch_result names; any other error of the
    // round ends every resident solve.
    const bool fatal = rc_run && rc_run != QSF_ENUMERIC;
    std::vector<int64_t> done;
    for (auto& kv : s->running) {
      Running& r = kv.second;
      if (!r.in_round && !fatal) continue;  // joined the batch during this round: runs from the next
      const int64_t ran = r.cancel && r.generic ? 0 : std::min<int64_t>(s->cfg.steps_per_round, r.remaining);
      if (r.in_round) r.remaining -= r.generic ? ran : s->cfg.steps_per_round;
      bool bad = r.generic && (r.bad || r.rc);
      if (!r.generic && r.in_round && rc_run == QSF_ENUMERIC) {
        int64_t st = 0;
        bad = qsf_batch_result(s->batch, r.slot, nullptr, &st) != QSF_OK;
      }
      if (r.remaining <= 0 || fatal || bad || r.cancel) done.push_back(kv.first);
    }
    for (int64_t t : done) {
      Running& r = s->running[t];
      rows.assign((size_t)r.nsteps * (3 + r.nb), 0.0);
      int64_t steps = 0;
      int rc;
      if (fatal) {
        rc = rc_run;
      } else if (r.generic) {
        steps = r.nsteps - std::max<int64_t>(r.remaining, 0);
        rc = r.rc ? r.rc : qsf::generic_rows(r.grid, &r.d, rows.data(), steps);
        if (rc == QSF_OK && r.bad) rc = QSF_ENUMERIC;
      } else {
        rc = qsf_batch_result(s->batch, r.slot, rows.data(), &steps);
      }
      if (rc == QSF_OK && r.cancel && r.remaining > 0) rc = QSF_ECANCELED;
      if (!r.generic) qsf_batch_remove(s->batch, r.slot);
      if (rc && rc != QSF_ECANCELED) qsf_grid_destroy(r.grid);
      else release_grid(s, r.desc, r.grid);
      finish(s, r, rc, rows.data(), steps);
      s->running.erase(t);
    }
    QSF_TRACE_ADD(s, 5, t_retire);
  }
}

}  // namespace

extern "C" {

int qsf_server_start(const qsf_server_config* cfg, qsf_server** out) {
  if (!cfg || !out || cfg->max_slots < 1 || cfg->steps_per_round < 1 || cfg->queue_capacity < 1)
    return QSF_EINVAL;
  qsf_server* s = new qsf_server();
  s->cfg = *cfg;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    return QSF_ECUDA;
  }
  int rc = qsf_batch_create(nullptr, &s->batch);
  if (rc) {
    delete s;
    return rc;
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return QSF_OK;
}

int qsf_server_submit(qsf_server* s, const qsf_request* r, int64_t* ticket) {
  if (!s || !r || !ticket || r->nsteps < 1 || r->nborders < 0 || r->nborders > QSF_MAX_BORDERS) return QSF_EINVAL;
  // lengths with fused kernels join the batch; the others need a Bluestein length
  if (r->grid.dim < 1 || r->grid.dim > 3) return QSF_EINVAL;
  if (!qsf::fused_length((int)r->grid.n[0]) && !qsf::bs_size((int)r->grid.n[0], r->grid.dim)) return QSF_EINVAL;
  Pending p;
  p.req = *r;
  const int stride = r->grid.gauge == QSF_GAUGE_LENGTH ? 6 : 3;
  if (r->coupling) p.coupling.assign(r->coupling, r->coupling + r->nsteps * stride);
  if (r->psi0) p.psi0.assign(r->psi0, r->psi0 + 2 * grid_points(r->grid));
  p.req.coupling = nullptr;
  p.req.psi0 = nullptr;
  p.submitted = clk::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stopping) return QSF_ESTATE;
  if ((int)s->queue.size() >= s->cfg.queue_capacity) return QSF_EBUSY;
  p.ticket = s->next_ticket++;
  *ticket = p.ticket;
  s->queue.push_back(std::move(p));
  s->stats.submitted++;
  s->stats.queued++;
  s->cv_work.notify_one();
  return QSF_OK;
}

int qsf_server_poll(qsf_server* s, int64_t ticket, qsf_result* out, int* done) {
  if (!s || !out || !done) return QSF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->results.find(ticket);
  *done = it != s->results.end();
  if (*done) {
    *out = it->second;
    s->results.erase(it);  // handed out once
  }
  return QSF_OK;
}

int qsf_server_wait(qsf_server* s, int64_t ticket, double timeout_s, qsf_result* out) {
  if (!s || !out) return QSF_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto until = clk::now() + std::chrono::duration<double>(timeout_s);
  while (s->results.find(ticket) == s->results.end()) {
    if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout && s->results.find(ticket) == s->results.end())
      return QSF_ETIMEDOUT;
  }
  auto it = s->results.find(ticket);
  *out = it->second;
  s->results.erase(it);  // handed out once
  return QSF_OK;
}

int qsf_server_cancel(qsf_server* s, int64_t ticket) {
  if (!s) return QSF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    if (it->ticket != ticket) continue;
    qsf_result res{};
    res.status = QSF_ECANCELED;
    res.latency_s = res.queue_s = std::chrono::duration<double>(clk::now() - it->submitted).count();
    s->results[ticket] = res;
    s->queue.erase(it);
    s->stats.queued--;
    s->stats.completed++;
    s->cv_done.notify_all();
    return QSF_OK;
  }
  if (s->admitted_set.count(ticket)) {
    s->cancel_running.push_back(ticket);
    s->cv_work.notify_one();
    return QSF_OK;
  }
  return QSF_EINVAL;
}

int qsf_server_stats_get(qsf_server* s, qsf_server_stats* out) {
  if (!s || !out) return QSF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return QSF_OK;
}

int qsf_server_stop(qsf_server* s) {
  if (!s) return QSF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    for (Pending& p : s->queue) {
      qsf_result res{};
      res.status = QSF_ESTATE;
      s->results[p.ticket] = res;
    }
    s->stats.queued -= (int64_t)s->queue.size();
    s->queue.clear();
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
#ifdef QSF_SERVER_TRACE
  std::fprintf(stderr,
               "qsf_server trace: decide %.3f s, admit %.3f s (%.0f; member programs %.3f s, batched %.3f s), "
               "enqueue %.3f s, batch %.3f s (launch %.3f s), wait %.3f s, retire %.3f s, rounds %.0f\n",
               s->trace[0], s->trace[1], s->trace[7], s->trace[9], s->trace[10], s->trace[2], s->trace[3],
               s->trace[8], s->trace[4], s->trace[5], s->trace[6]);
  std::fprintf(stderr, "qsf_server trace: admission parts: grid %.3f s (%.0f new), upload %.3f s, add %.3f s\n",
               s->trace[11], s->trace[14], s->trace[12], s->trace[13]);
#endif
  drain_pool(s);
  qsf_batch_destroy(s->batch);
  delete s;
  return QSF_OK;
}

}  // extern "C"
