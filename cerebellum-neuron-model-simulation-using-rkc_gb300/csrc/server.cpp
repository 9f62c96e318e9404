// Request server: simulation jobs of uneven cell counts and durations admitted
// into a device-resident arena and advanced together (include/gbrkc.h,
// "request server").  No counterpart in the reference, which integrates one
// fixed block per cell type per process (main.cu:105-311).
//
// Design.  At start the server sizes one slot arena per system shape
// ("class") from its HBM budget and builds ONE engine holding every slot as
// an idle system; nothing is allocated on the device after that except the
// raster log.  A request names a class, a number of systems and a duration
// in 0.125 ms intervals.  Each serving round (gbrkc_request_advance):
//   1. admits queued requests whose systems fit the free slots of their
//      arena (first come first served with bounded backfilling), refilling
//      their slots in place (gbrkc_systems_reset, a few bulk copies per run
//      of consecutive slots) with the request's interval budget;
//   2. advances every resident request by one quantum in the engine's
//      persistent launch -- systems whose budget runs out inside the
//      quantum stop there, so every request gets exactly its intervals;
//   3. routes the device raster's threshold crossings to their requests;
//   4. completes the requests with no intervals left: final v_new read back
//      per run, slots released for the next round's admissions.
// A request's systems integrate exactly as they would in an engine of their
// own started at t = 0: each system keeps its own clock, and the server only
// shifts the stimulus windows by the request's admission time.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <exception>
#include <map>
#include <new>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbrkc.h"
#include "serve_sched.h"

namespace {

using gbrkc::serve::Run;

constexpr double INTERVAL_MS = 0.125;  // RKC_DT, param.h:12

std::string g_srv_error;

int srv_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_srv_error = buf;
  return code;
}

// A C entry point lets no C++ exception out (host allocations sized by the
// caller report GBRKC_ENOMEM).
template <class F>
int srv_no_throw(F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    return srv_fail(GBRKC_ENOMEM, "host memory exhausted");
  } catch (const std::exception &x) {
    return srv_fail(GBRKC_EINVAL, "%s", x.what());
  }
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct ServeClass {
  gbrkc_system_desc shape{};
  std::vector<double> rows;
  std::vector<int> gj;
  long long slots_req = 0;
  double share = 0.0;
  int slots = 0, first_id = -1, cells = 0, nc = 0;
  long long slot_bytes = 0;
  gbrkc::serve::SlotArena arena;
  gbrkc::serve::Admission queue;
  std::vector<int> owner;  // per slot: request id or -1
  std::vector<int> rank;   // per slot: position of the system within its request
};

struct Request {
  int cls = 0, n_sys = 0, n_iv = 0;
  std::vector<double> jitter, stim_amp, stim_t0, stim_t1, cond_scale, io_gap_g;
  std::vector<int> stim_comp;
  int state = GBRKC_REQ_QUEUED;
  int status = 0;
  std::vector<Run> runs;
  double t_submit = 0, t_admit = 0, t_done = 0;
  double sim_t0 = 0;  // server time at admission (ms)
  int remaining = 0;
  std::vector<double> vnew;
  std::vector<double> spk_t;
  std::vector<int> spk_cell;
};

}  // namespace

struct gbrkc_server {
  int precision = GBRKC_MIXED;
  long long budget = 0;
  int quantum = 8;
  bool started = false;
  gbrkc_engine *e = nullptr;
  std::vector<std::unique_ptr<ServeClass>> classes;
  std::map<int, Request> reqs;
  int next_id = 0;
  double T = 0.0;  // server time (ms)
  long spike_cap = 0;
  std::vector<double> spk_t;
  std::vector<int> spk_sys, spk_cell;
  // statistics
  long long submitted = 0, admitted = 0, completed = 0, failed = 0, cancelled = 0, rounds = 0;
  long long lost_spikes = 0;
  std::vector<double> latency_ms;
  double busy_s = 0.0, advance_s = 0.0;
  long long cu = 0;
  long long reserved = 0;
  ~gbrkc_server() {
    if (e) gbrkc_engine_destroy(e);
  }
};

namespace {

bool resident(const Request &r) { return r.state == GBRKC_REQ_RESIDENT; }

// fill the request's slots (one reset per run), budget = its intervals
int admit(gbrkc_server *S, int rid) {
  Request &r = S->reqs[rid];
  ServeClass &c = *S->classes[r.cls];
  r.state = GBRKC_REQ_RESIDENT;
  r.t_admit = now_s();
  r.sim_t0 = S->T;
  r.remaining = r.n_iv;
  int done = 0;  // systems filled so far
  std::vector<double> t0, t1;
  for (const Run &run : r.runs) {
    const long cell0 = (long)done * c.cells, ncell = (long)run.second * c.cells;
    gbrkc_reset_desc d{};
    d.jitter = r.jitter.data() + cell0;
    if (!r.stim_comp.empty()) {
      // request-relative windows on the server's clock
      t0.assign(r.stim_t0.begin() + cell0, r.stim_t0.begin() + cell0 + ncell);
      t1.assign(r.stim_t1.begin() + cell0, r.stim_t1.begin() + cell0 + ncell);
      for (double &x : t0) x += S->T;
      for (double &x : t1) x += S->T;
      d.stim_comp = r.stim_comp.data() + cell0;
      d.stim_amp = r.stim_amp.data() + cell0;
      d.stim_t0 = t0.data();
      d.stim_t1 = t1.data();
    }
    if (!r.cond_scale.empty()) d.cond_scale = r.cond_scale.data() + cell0;
    if (!r.io_gap_g.empty()) d.io_gap_g = r.io_gap_g.data() + 4 * cell0;
    d.n_intervals = r.n_iv;
    int rc = gbrkc_systems_reset(S->e, c.first_id + run.first, run.second, &d);
    if (rc) return srv_fail(rc, "admitting request %d: %s", rid, gbrkc_last_error());
    for (int k = 0; k < run.second; k++) {
      c.owner[run.first + k] = rid;
      c.rank[run.first + k] = done + k;
    }
    done += run.second;
  }
  S->admitted++;
  return 0;
}

void release(gbrkc_server *S, Request &r) {
  ServeClass &c = *S->classes[r.cls];
  for (const Run &run : r.runs)
    for (int k = 0; k < run.second; k++) c.owner[run.first + k] = -1;
  c.arena.release(r.runs);
  r.runs.clear();
}

// read the final voltages, free the slots, stamp the latency
int complete(gbrkc_server *S, int rid, int state) {
  Request &r = S->reqs[rid];
  ServeClass &c = *S->classes[r.cls];
  r.vnew.assign((size_t)r.n_sys * c.nc, 0.0);
  long off = 0;
  for (const Run &run : r.runs) {
    const long n = (long)run.second * c.nc;
    int rc = gbrkc_read_run(S->e, c.first_id + run.first, run.second, GBRKC_F_VNEW, r.vnew.data() + off, n);
    if (rc) return srv_fail(rc, "reading request %d: %s", rid, gbrkc_last_error());
    off += n;
  }
  // stop the slots (a budget of 0) before anyone else gets them
  for (const Run &run : r.runs) {
    int rc = gbrkc_set_budget(S->e, c.first_id + run.first, run.second, 0);
    if (rc) return srv_fail(rc, "parking request %d: %s", rid, gbrkc_last_error());
  }
  release(S, r);
  r.state = state;
  r.t_done = now_s();
  if (state == GBRKC_REQ_DONE) {
    S->completed++;
    S->latency_ms.push_back((r.t_done - r.t_submit) * 1e3);
  } else {
    S->failed++;
  }
  return 0;
}

}  // namespace

extern "C" const char *gbrkc_server_last_error(void) { return g_srv_error.c_str(); }

extern "C" int gbrkc_server_create(int precision, long long hbm_budget, int quantum_intervals, gbrkc_server **out) {
  if (!out || (precision != GBRKC_FP64 && precision != GBRKC_MIXED) || hbm_budget < 0 || quantum_intervals <= 0)
    return srv_fail(GBRKC_EINVAL, "bad arguments");
  gbrkc_server *S = new gbrkc_server;
  S->precision = precision;
  S->budget = hbm_budget;
  S->quantum = quantum_intervals;
  *out = S;
  return 0;
}

extern "C" void gbrkc_server_destroy(gbrkc_server *S) { delete S; }

static int server_add_class_impl(gbrkc_server *S, const gbrkc_slot_class *c, int *class_id) {
  if (!S || !c || !c->shape.rows) return srv_fail(GBRKC_EINVAL, "null argument");
  if (S->started) return srv_fail(GBRKC_ESTATE, "server already started");
  const gbrkc_system_desc &d = c->shape;
  if (d.cell_type < GBRKC_GR || d.cell_type > GBRKC_IO || d.nx <= 0 || d.ny <= 0 || d.ncomp <= 0)
    return srv_fail(GBRKC_EINVAL, "bad class shape");
  if (c->slots < 0 || c->share < 0.0 || (c->slots == 0 && c->share <= 0.0))
    return srv_fail(GBRKC_EINVAL, "a class needs slots or a share of the budget");
  static const int row_fields[4] = {17, 20, 7, 6};  // Gr.txt, Go_131.txt, Pkj.txt, IO.txt
  auto C = std::make_unique<ServeClass>();
  C->shape = d;
  C->rows.assign(d.rows, d.rows + (size_t)d.ncomp * row_fields[d.cell_type]);
  C->shape.rows = C->rows.data();
  if (d.gj_pairs && d.n_gj_pairs > 0) {
    C->gj.assign(d.gj_pairs, d.gj_pairs + 2 * d.n_gj_pairs);
    C->shape.gj_pairs = C->gj.data();
  } else {
    C->shape.gj_pairs = nullptr;
    C->shape.n_gj_pairs = 0;
  }
  // per-slot inputs come with each request
  C->shape.io_gap_g = nullptr;
  C->shape.jitter = nullptr;
  C->shape.stim_comp = nullptr;
  C->shape.stim_amp = C->shape.stim_t0 = C->shape.stim_t1 = nullptr;
  C->shape.cond_scale = nullptr;
  C->shape.cond_scale_ch = nullptr;
  C->shape.idle = 1;
  C->slots_req = c->slots;
  C->share = c->share;
  C->cells = d.nx * d.ny;
  C->nc = C->cells * d.ncomp;
  C->slot_bytes = gbrkc_system_bytes(S->precision, d.cell_type, d.ncomp, C->cells);
  if (C->slot_bytes <= 0) return srv_fail(GBRKC_EINVAL, "bad class shape");
  S->classes.push_back(std::move(C));
  if (class_id) *class_id = (int)S->classes.size() - 1;
  return 0;
}

extern "C" int gbrkc_server_add_class(gbrkc_server *S, const gbrkc_slot_class *c, int *class_id) {
  return srv_no_throw([&] { return server_add_class_impl(S, c, class_id); });
}

namespace {

// The arenas' systems in the server's engine (idle until a request fills
// them), the engine built, and the raster log sized for `cells` cells.
int fill_arenas(gbrkc_server *S, long long cells) {
  int rc = 0;
  for (auto &C : S->classes) {
    std::vector<double> jit(C->cells, 0.0);
    gbrkc_system_desc d = C->shape;
    d.jitter = jit.data();
    for (int k = 0; k < C->slots; k++) {
      int id = -1;
      rc = gbrkc_add_system(S->e, &d, &id);
      if (rc) return srv_fail(rc, "arena: %s", gbrkc_last_error());
      if (k == 0) C->first_id = id;
    }
    C->arena = gbrkc::serve::SlotArena(C->slots);
    C->owner.assign(C->slots, -1);
    C->rank.assign(C->slots, -1);
  }
  rc = gbrkc_build(S->e);
  if (rc) return srv_fail(rc, "build: %s", gbrkc_last_error());
  // a cell crosses upward at most every other interval
  S->spike_cap = (long)std::min<long long>(cells * ((S->quantum + 1) / 2 + 1), 1 << 24);
  rc = gbrkc_record_spikes(S->e, S->spike_cap);
  if (rc) return srv_fail(rc, "raster: %s", gbrkc_last_error());
  S->spk_t.resize(S->spike_cap);
  S->spk_sys.resize(S->spike_cap);
  S->spk_cell.resize(S->spike_cap);
  return 0;
}

}  // namespace

static int server_start_impl(gbrkc_server *S) {
  if (!S) return srv_fail(GBRKC_EINVAL, "null server");
  if (S->started) return srv_fail(GBRKC_ESTATE, "server already started");
  if (S->classes.empty()) return srv_fail(GBRKC_EINVAL, "no classes");
  long long budget = S->budget;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) return srv_fail(GBRKC_ECUDA, "cudaMemGetInfo: %s", cudaGetErrorString(e));
    budget = (long long)(0.8 * (double)fr);
  }
  // arenas: explicit slot counts first, then shares of what is left
  long long fixed = 0;
  for (auto &C : S->classes)
    if (C->slots_req > 0) fixed += C->slots_req * C->slot_bytes;
  if (fixed > budget)
    return srv_fail(GBRKC_ENOMEM, "the classes' slots need %lld bytes; the HBM budget is %lld", fixed, budget);
  const long long rest = budget - fixed;
  long long total = 0, cells = 0;
  for (auto &C : S->classes) {
    long long n = C->slots_req > 0 ? C->slots_req : (long long)(C->share * (double)rest) / C->slot_bytes;
    n = std::min<long long>(n, 1 << 22);
    if (n <= 0) return srv_fail(GBRKC_ENOMEM, "a class gets no slot within the HBM budget");
    C->slots = (int)n;
    total += n * C->slot_bytes;
    cells += n * C->cells;
  }
  if (total > budget) return srv_fail(GBRKC_ENOMEM, "arenas need %lld bytes; the HBM budget is %lld", total, budget);
  S->reserved = total;
  int rc = gbrkc_engine_create(S->precision, &S->e);
  if (rc) return srv_fail(rc, "engine: %s", gbrkc_last_error());
  rc = fill_arenas(S, cells);
  if (rc) {
    // back to the state before the call, so that start can be retried
    gbrkc_engine_destroy(S->e);
    S->e = nullptr;
    S->reserved = 0;
    return rc;
  }
  S->started = true;
  return 0;
}

extern "C" int gbrkc_server_start(gbrkc_server *S) { return srv_no_throw([&] { return server_start_impl(S); }); }

static int request_create_impl(gbrkc_server *S, const gbrkc_request_desc *d, int *req_id) {
  if (!S || !d || !d->jitter) return srv_fail(GBRKC_EINVAL, "null argument");
  if (!S->started) return srv_fail(GBRKC_ESTATE, "server not started");
  if (d->class_id < 0 || d->class_id >= (int)S->classes.size()) return srv_fail(GBRKC_EINVAL, "bad class");
  ServeClass &c = *S->classes[d->class_id];
  if (d->n_systems <= 0 || d->n_systems > c.slots)
    return srv_fail(GBRKC_EINVAL, "request of %d systems; the class holds %d", d->n_systems, c.slots);
  if (d->n_intervals <= 0) return srv_fail(GBRKC_EINVAL, "a request needs at least one interval");
  if (d->stim_comp && (!d->stim_amp || !d->stim_t0 || !d->stim_t1)) return srv_fail(GBRKC_EINVAL, "incomplete stimulus");
  const long cells = (long)d->n_systems * c.cells;
  Request r;
  r.cls = d->class_id;
  r.n_sys = d->n_systems;
  r.n_iv = d->n_intervals;
  r.jitter.assign(d->jitter, d->jitter + cells);
  if (d->stim_comp) {
    r.stim_comp.assign(d->stim_comp, d->stim_comp + cells);
    r.stim_amp.assign(d->stim_amp, d->stim_amp + cells);
    r.stim_t0.assign(d->stim_t0, d->stim_t0 + cells);
    r.stim_t1.assign(d->stim_t1, d->stim_t1 + cells);
    for (int x : r.stim_comp)
      if (x >= c.shape.ncomp) return srv_fail(GBRKC_EINVAL, "stimulus compartment out of range");
  }
  if (d->cond_scale) r.cond_scale.assign(d->cond_scale, d->cond_scale + cells);
  if (d->io_gap_g) r.io_gap_g.assign(d->io_gap_g, d->io_gap_g + 4 * cells);
  r.t_submit = now_s();
  const int id = S->next_id++;
  S->reqs.emplace(id, std::move(r));
  c.queue.push(id);
  S->submitted++;
  if (req_id) *req_id = id;
  return 0;
}

extern "C" int gbrkc_request_create(gbrkc_server *S, const gbrkc_request_desc *d, int *req_id) {
  return srv_no_throw([&] { return request_create_impl(S, d, req_id); });
}

static int request_advance_impl(gbrkc_server *S, int *n_done) {
  if (!S) return srv_fail(GBRKC_EINVAL, "null server");
  if (!S->started) return srv_fail(GBRKC_ESTATE, "server not started");
  const double t_round = now_s();
  int rc = 0;
  // 1. admission
  for (int ci = 0; ci < (int)S->classes.size(); ci++) {
    ServeClass &c = *S->classes[ci];
    std::vector<int> in = c.queue.admit([&](int rid) { return c.arena.alloc(S->reqs[rid].n_sys, S->reqs[rid].runs); });
    for (int rid : in)
      if ((rc = admit(S, rid))) return rc;
  }
  int live = 0;
  for (auto &kv : S->reqs) live += resident(kv.second);
  int done = 0;
  if (live > 0) {
    // 2. one quantum for every resident request
    const long long cu0 = gbrkc_compartment_updates(S->e, -1);
    const double ta = now_s();
    int arc = gbrkc_advance(S->e, S->T, S->quantum);
    S->advance_s += now_s() - ta;
    if (arc && arc != GBRKC_ESOLVER) return srv_fail(arc, "advance: %s", gbrkc_last_error());
    const long long cu1 = gbrkc_compartment_updates(S->e, -1);
    if (cu0 >= 0 && cu1 >= cu0) S->cu += cu1 - cu0;
    S->T += S->quantum * INTERVAL_MS;
    // 3. raster, routed to the requests
    for (int type = GBRKC_GR; type <= GBRKC_IO; type++) {
      long n = 0;
      int src = gbrkc_read_spikes(S->e, type, S->spike_cap, S->spk_t.data(), S->spk_sys.data(), S->spk_cell.data(), &n);
      if (src == GBRKC_EOVERFLOW) S->lost_spikes++;
      else if (src) return srv_fail(src, "raster: %s", gbrkc_last_error());
      for (long k = 0; k < n; k++) {
        for (auto &cp : S->classes) {
          ServeClass &c = *cp;
          const int slot = S->spk_sys[k] - c.first_id;
          if (slot < 0 || slot >= c.slots) continue;
          const int rid = c.owner[slot];
          if (rid >= 0) {
            Request &r = S->reqs[rid];
            r.spk_t.push_back(S->spk_t[k] - r.sim_t0);
            r.spk_cell.push_back(c.rank[slot] * c.cells + S->spk_cell[k]);
          }
          break;
        }
      }
    }
    // 4. completions (and systems the solver stopped)
    for (auto &kv : S->reqs) {
      Request &r = kv.second;
      if (!resident(r)) continue;
      r.remaining = std::max(0, r.remaining - S->quantum);
      int state = (r.remaining == 0) ? GBRKC_REQ_DONE : -1;
      if (arc == GBRKC_ESOLVER) {
        ServeClass &c = *S->classes[r.cls];
        for (const Run &run : r.runs) {
          std::vector<int> st(run.second);
          if ((rc = gbrkc_run_status(S->e, c.first_id + run.first, run.second, st.data(), nullptr)))
            return srv_fail(rc, "status: %s", gbrkc_last_error());
          for (int x : st)
            if (x) { r.status = x; state = GBRKC_REQ_FAILED; }
        }
      }
      if (state >= 0) {
        if ((rc = complete(S, kv.first, state))) return rc;
        done++;
      }
    }
  }
  S->rounds++;
  S->busy_s += now_s() - t_round;
  if (n_done) *n_done = done;
  return 0;
}

extern "C" int gbrkc_request_advance(gbrkc_server *S, int *n_done) {
  return srv_no_throw([&] { return request_advance_impl(S, n_done); });
}

extern "C" int gbrkc_request_state(gbrkc_server *S, int rid, int *state, double *latency_ms, int *status) {
  if (!S) return srv_fail(GBRKC_EINVAL, "null server");
  auto it = S->reqs.find(rid);
  if (it == S->reqs.end()) return srv_fail(GBRKC_EINVAL, "no request %d", rid);
  const Request &r = it->second;
  if (state) *state = r.state;
  if (latency_ms) *latency_ms = (r.state == GBRKC_REQ_DONE || r.state == GBRKC_REQ_FAILED) ? (r.t_done - r.t_submit) * 1e3 : -1.0;
  if (status) *status = r.status;
  return 0;
}

extern "C" int gbrkc_request_read(gbrkc_server *S, int rid, double *host, long cap) {
  if (!S || !host) return srv_fail(GBRKC_EINVAL, "null argument");
  auto it = S->reqs.find(rid);
  if (it == S->reqs.end()) return srv_fail(GBRKC_EINVAL, "no request %d", rid);
  const Request &r = it->second;
  if (r.state != GBRKC_REQ_DONE && r.state != GBRKC_REQ_FAILED) return srv_fail(GBRKC_ESTATE, "request %d not finished", rid);
  if (cap < (long)r.vnew.size()) return srv_fail(GBRKC_EINVAL, "buffer holds %ld of %zu values", cap, r.vnew.size());
  memcpy(host, r.vnew.data(), r.vnew.size() * sizeof(double));
  return 0;
}

extern "C" int gbrkc_request_spikes(gbrkc_server *S, int rid, long cap, double *t, int *cell, long *n) {
  if (!S || !n || (cap > 0 && (!t || !cell))) return srv_fail(GBRKC_EINVAL, "bad arguments");
  auto it = S->reqs.find(rid);
  if (it == S->reqs.end()) return srv_fail(GBRKC_EINVAL, "no request %d", rid);
  const Request &r = it->second;
  const long m = std::min<long>(cap, (long)r.spk_t.size());
  for (long k = 0; k < m; k++) {
    t[k] = r.spk_t[k];
    cell[k] = r.spk_cell[k];
  }
  *n = (long)r.spk_t.size();
  return m < (long)r.spk_t.size() ? srv_fail(GBRKC_EOVERFLOW, "%ld spikes, buffer holds %ld", *n, cap) : 0;
}

extern "C" int gbrkc_request_destroy(gbrkc_server *S, int rid) {
  if (!S) return srv_fail(GBRKC_EINVAL, "null server");
  auto it = S->reqs.find(rid);
  if (it == S->reqs.end()) return srv_fail(GBRKC_EINVAL, "no request %d", rid);
  Request &r = it->second;
  if (r.state == GBRKC_REQ_QUEUED) {
    S->classes[r.cls]->queue.remove(rid);
    S->cancelled++;
  } else if (r.state == GBRKC_REQ_RESIDENT) {
    ServeClass &c = *S->classes[r.cls];
    for (const Run &run : r.runs) {
      int rc = gbrkc_set_budget(S->e, c.first_id + run.first, run.second, 0);
      if (rc) return srv_fail(rc, "parking request %d: %s", rid, gbrkc_last_error());
    }
    release(S, r);
    S->cancelled++;
  }
  S->reqs.erase(it);
  return 0;
}

extern "C" int gbrkc_server_stats(gbrkc_server *S, gbrkc_server_stats_t *o) {
  if (!S || !o) return srv_fail(GBRKC_EINVAL, "null argument");
  memset(o, 0, sizeof *o);
  o->submitted = S->submitted;
  o->admitted = S->admitted;
  o->completed = S->completed;
  o->failed = S->failed;
  o->cancelled = S->cancelled;
  o->rounds = S->rounds;
  for (auto &kv : S->reqs) {
    o->queued += kv.second.state == GBRKC_REQ_QUEUED;
    o->resident += kv.second.state == GBRKC_REQ_RESIDENT;
  }
  o->p50_ms = gbrkc::serve::percentile(S->latency_ms, 50.0);
  o->p99_ms = gbrkc::serve::percentile(S->latency_ms, 99.0);
  double sum = 0.0, mx = 0.0;
  for (double x : S->latency_ms) { sum += x; mx = std::max(mx, x); }
  o->mean_ms = S->latency_ms.empty() ? 0.0 : sum / (double)S->latency_ms.size();
  o->max_ms = mx;
  o->busy_s = S->busy_s;
  o->advance_s = S->advance_s;
  o->compartment_updates = S->cu;
  o->hbm_reserved = S->reserved;
  long long used = 0, slots = 0, free_slots = 0;
  for (auto &C : S->classes) {
    used += (long long)(C->slots - C->arena.free_slots()) * C->slot_bytes;
    slots += C->slots;
    free_slots += C->arena.free_slots();
  }
  o->hbm_in_use = used;
  o->slots = slots;
  o->free_slots = free_slots;
  o->sim_ms = S->T;
  o->lost_spike_reads = S->lost_spikes;
  return 0;
}

extern "C" int gbrkc_server_class_slots(gbrkc_server *S, int class_id, int *slots, int *first_system) {
  if (!S || class_id < 0 || class_id >= (int)S->classes.size()) return srv_fail(GBRKC_EINVAL, "bad class");
  if (slots) *slots = S->classes[class_id]->slots;
  if (first_system) *first_system = S->classes[class_id]->first_id;
  return 0;
}

extern "C" gbrkc_engine *gbrkc_server_engine(gbrkc_server *S) { return S ? S->e : nullptr; }
