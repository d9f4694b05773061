// Request server: continuous batching of frequency-solve requests on one GPU.
//
// A request is what one HAMS-MREL run asks for (src/HAMS_Prog.f90:255-304,
// :613-704): a mesh, a depth, a list of frequencies and headings.  Its unit
// of work is one frequency-solve (hg_solve_frequency).  The server keeps
// nslots solve slots (library contexts, each with its own device buffers and
// CUDA stream, driven by its own host thread), and:
//   - admits queued requests in arrival order while the device memory they
//     may hold stays within the budget: a request reserves
//     min(nslots, nfreq) x hg_solve_footprint(its size) plus its mesh, and
//     gives the reservation back when its last frequency is done;
//   - hands the frequencies of all admitted requests to whichever slot is
//     free, preferring the request whose mesh the slot already holds (the
//     mesh then stays resident on the device, no re-upload), else the
//     oldest admitted request: requests that arrive while others run join
//     the mix as soon as memory and a slot allow, and their solves overlap
//     on the device;
//   - lets a slot give its buffers back to the device when no admitted
//     request needs them any more (its buffers only grow otherwise).
// Every frequency-solve of a request gives the same result whether it runs
// alone or in the mix: a slot computes exactly what a single context does.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hamsgpu.h"

namespace hg {
size_t hmatrix_bytes_estimate(int n, const double* xyz, int nc);  // hg_hmatrix.cu
}

// Milliseconds from ref (an event recorded earlier on the context's device)
// to the context's hg_mark event in slot (hg_abi.cu).
int hg_mark_since(const hg_ctx* c, int slot, cudaEvent_t ref, float* ms);

namespace {

typedef std::chrono::steady_clock Clock;

struct Request {
  long long id = 0;
  // mesh
  int n = 0, ntnd = 0, nl = 0, nbody = 0;
  std::vector<double> nodes, xyz, ds, pnsz, dxyz, lid;
  std::vector<int> ncon, ncn, ranges;
  // frequencies and headings
  double h = -1.0;
  int nfreq = 0, nk = 0, irsp = 0, isol = 1, nbeta = 0;
  std::vector<double> v, wk, w1, wvn, betas;
  // results (per frequency, column-major as hg_forces)
  std::vector<double> amas, bdmp, exfc;
  // state
  size_t reserve = 0;       // bytes reserved at admission
  size_t slot_bytes = 0;    // one solve's footprint
  int next = 0;             // next frequency to hand out
  int done = 0;             // frequencies finished
  int rc = 0;               // first error
  std::string err;
  bool admitted = false, finished = false;
  Clock::time_point t_submit, t_admit, t_done;
};

struct Slot {
  hg_ctx* ctx = nullptr;
  long long mesh_of = -1;   // request whose mesh the context holds
  size_t holds = 0;         // footprint of the largest solve it has buffers for
  std::thread th;
};

}  // namespace

struct hg_server {
  hg_opts opts;
  int nslots = 0;
  size_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;         // submitted, not admitted
  std::vector<std::shared_ptr<Request>> active;       // admitted, not finished
  std::map<long long, std::shared_ptr<Request>> all;  // until collected by hg_server_wait
  std::vector<Slot> slots;
  size_t reserved = 0, peak_reserved = 0;
  long long next_id = 1;
  long long n_done = 0, n_units = 0;
  int max_active = 0;
  bool stop = false;
  std::string err;
  // device timeline: ref recorded at creation; per finished frequency-solve
  // (ticket, frequency, start, end) in milliseconds since ref
  cudaEvent_t ref = nullptr;
  std::vector<double> timeline;
};

namespace {

size_t mesh_bytes(const Request& r) {
  return (size_t)r.n * (4 * sizeof(int) + 12 * sizeof(double) + 36 * sizeof(double)) +
         (size_t)(r.n + r.nl) * 3 * sizeof(double);
}

// Admit queued requests in order while the budget allows (caller holds mu).
void admit(hg_server* s) {
  while (!s->queue.empty()) {
    auto r = s->queue.front();
    if (s->reserved + r->reserve > s->budget) break;
    s->queue.pop_front();
    s->reserved += r->reserve;
    s->peak_reserved = std::max(s->peak_reserved, s->reserved);
    r->admitted = true;
    r->t_admit = Clock::now();
    s->active.push_back(r);
    s->max_active = std::max(s->max_active, (int)s->active.size());
  }
}

// Next unit for slot k (caller holds mu): the slot's current request first.
bool next_unit(hg_server* s, int k, std::shared_ptr<Request>* out, int* freq) {
  std::shared_ptr<Request> pick;
  for (auto& r : s->active)
    if (r->id == s->slots[k].mesh_of && r->next < r->nfreq && r->rc == 0) { pick = r; break; }
  if (!pick)
    for (auto& r : s->active)
      if (r->next < r->nfreq && r->rc == 0) { pick = r; break; }
  if (!pick) return false;
  *out = pick;
  *freq = pick->next++;
  return true;
}

void finish_unit(hg_server* s, const std::shared_ptr<Request>& r) {
  r->done++;
  s->n_units++;
  const bool all_handed = r->next >= r->nfreq || r->rc != 0;
  const bool complete = r->rc != 0 ? (r->done >= r->next) : (r->done >= r->nfreq);
  if (all_handed && complete && !r->finished) {
    r->finished = true;
    r->t_done = Clock::now();
    s->reserved -= r->reserve;
    s->active.erase(std::remove(s->active.begin(), s->active.end(), r), s->active.end());
    s->n_done++;
    admit(s);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

// Largest per-solve footprint among admitted requests (caller holds mu).
size_t needed_bytes(hg_server* s) {
  size_t m = 0;
  for (auto& r : s->active) m = std::max(m, r->slot_bytes);
  return m;
}

void worker(hg_server* s, int k) {
  Slot& sl = s->slots[k];
  cudaSetDevice(s->opts.device);
  for (;;) {
    std::shared_ptr<Request> r;
    int f = -1;
    bool release = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || next_unit(s, k, &r, &f); });
      if (s->stop && !r) break;
      if (sl.holds > 0 && sl.holds > 2 * needed_bytes(s)) release = true;
    }
    if (release) {
      // no admitted request needs buffers this large: hand them back
      hg_destroy(sl.ctx);
      sl.ctx = nullptr;
      sl.holds = 0;
      sl.mesh_of = -1;
    }
    int rc = 0;
    std::string msg;
    if (!sl.ctx) {
      rc = hg_create(&sl.ctx, &s->opts);
      if (rc) msg = "creating a solve slot failed";
    }
    if (!rc && sl.mesh_of != r->id) {
      rc = hg_set_mesh(sl.ctx, r->n, r->ntnd, r->nodes.data(), r->ncon.data(), r->ncn.data(), r->xyz.data(),
                       r->ds.data(), r->pnsz.data(), r->dxyz.data(), r->nl, r->nl ? r->lid.data() : nullptr,
                       r->nbody, r->ranges.data());
      if (rc) msg = hg_last_error(sl.ctx);
      else sl.mesh_of = r->id;
    }
    float t0 = 0.f, t1 = 0.f;
    bool timed = false;
    if (!rc) {
      const int nd = 6 * r->nbody;
      hg_mark(sl.ctx, 14);
      rc = hg_solve_frequency(sl.ctx, r->v[f], r->wk[f], r->w1[f], r->h, r->h > 0 ? &r->wvn[(size_t)f * r->nk] : nullptr,
                              r->h > 0 ? r->nk : 0, r->irsp, r->betas.data(), r->nbeta, r->isol,
                              &r->amas[(size_t)f * nd * nd], &r->bdmp[(size_t)f * nd * nd],
                              r->nbeta > 0 ? &r->exfc[(size_t)f * r->nbeta * nd * 2] : nullptr, nullptr, 0);
      if (rc) msg = hg_last_error(sl.ctx);
      sl.holds = std::max(sl.holds, r->slot_bytes);
      if (!rc && s->ref && hg_mark(sl.ctx, 15) == 0 && hg_mark_since(sl.ctx, 14, s->ref, &t0) == 0 &&
          hg_mark_since(sl.ctx, 15, s->ref, &t1) == 0)
        timed = true;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (timed) {
        const double e[4] = {(double)r->id, (double)f, (double)t0, (double)t1};
        s->timeline.insert(s->timeline.end(), e, e + 4);
      }
      if (rc && r->rc == 0) {
        r->rc = rc;
        r->err = "frequency " + std::to_string(f) + ": " + msg;
      }
      finish_unit(s, r);
    }
  }
}

template <typename T>
void copy_in(std::vector<T>& dst, const T* src, size_t count) {
  dst.assign(src, src + count);
}

}  // namespace

// Device memory of the GMRES paths beyond hg_solve_footprint: the Krylov
// and preconditioned bases (restart 8 for the refinement, 25 for solver 2),
// for solver 2 the preconditioner (the diagonal, or the per-body diagonal
// blocks and their pivots), and in the FP64 form without lids the n x nc
// right-hand-side block of the square system, which hg_solve_footprint
// counts only for the mixed form and for lids; with the H-matrix its blocks
// and scratch (hmatrix_bytes_estimate, from the request's panel centres).
static size_t iter_bytes(const hg_opts& o, const hg_request& q) {
  const size_t n = (size_t)q.n, nc = (size_t)6 * q.nbody + (size_t)(q.nbeta > 0 ? q.nbeta : 0);
  size_t b = 0;
  if (o.solver == 2) {
    b += (size_t)(2 * 25 + 2) * n * nc * 16;
    if (o.precision != HG_PREC_MIXED && q.irsp != 1) b += n * nc * 16;
    if (q.nbody <= 1) {
      b += n * 16;
    } else {
      size_t blocks = 0;
      for (int k = 0; k < q.nbody; ++k) {
        const size_t sz = (size_t)(q.body_ranges[2 * k + 1] - q.body_ranges[2 * k] + 1);
        blocks += sz * sz;
      }
      b += blocks * (o.precision == HG_PREC_MIXED ? 8 : 16) + n * sizeof(int);
    }
    if (o.hmatrix) b += hg::hmatrix_bytes_estimate(q.n, q.xyz_p, (int)nc);
  } else if (o.refine_method == 1 && o.precision == HG_PREC_MIXED) {
    b += (size_t)(2 * 8 + 2) * n * nc * 16;
  }
  return b;
}

extern "C" {

int hg_server_create(hg_server** out, const hg_opts* opts, int nslots, double budget_bytes) {
  if (!out) return -1;
  *out = nullptr;
  if (nslots < 1 || nslots > 64) return -3;
  if (!(budget_bytes > 0)) return -4;
  hg_server* s = new (std::nothrow) hg_server();
  if (!s) return HG_ERR_ALLOC;
  hg_default_opts(&s->opts);
  if (opts) s->opts = *opts;
  s->nslots = nslots;
  s->budget = (size_t)budget_bytes;
  if (cudaSetDevice(s->opts.device) == cudaSuccess && cudaEventCreate(&s->ref) == cudaSuccess) {
    if (cudaEventRecord(s->ref, 0) != cudaSuccess || cudaEventSynchronize(s->ref) != cudaSuccess) {
      cudaEventDestroy(s->ref);
      s->ref = nullptr;
    }
  }
  cudaGetLastError();
  s->slots.resize(nslots);
  for (int k = 0; k < nslots; ++k) s->slots[k].th = std::thread(worker, s, k);
  *out = s;
  return 0;
}

void hg_server_destroy(hg_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& sl : s->slots)
    if (sl.th.joinable()) sl.th.join();
  for (auto& sl : s->slots)
    if (sl.ctx) hg_destroy(sl.ctx);
  if (s->ref) cudaEventDestroy(s->ref);
  delete s;
}

const char* hg_server_last_error(const hg_server* s) { return s ? s->err.c_str() : "null server"; }

int hg_server_submit(hg_server* s, const hg_request* q, long long* ticket) {
  if (!s) return -1;
  if (!q || !ticket) return -2;
  if (q->n <= 0 || q->ntnd <= 0 || !q->nodes || !q->ncon || !q->ncn || !q->xyz_p || !q->ds || !q->pnsz ||
      !q->dxyz_p || q->nbody <= 0 || !q->body_ranges || q->nl < 0 || (q->nl > 0 && !q->lid_xyz_p)) {
    s->err = "bad mesh arrays";
    return -2;
  }
  if (q->nfreq <= 0 || !q->v || !q->wk || !q->w1 || (q->h > 0 && (!q->wvn || q->nk < 20)) || q->nbeta < 0 ||
      (q->nbeta > 0 && !q->betas) || (q->irsp != 0 && q->irsp != 1) || (q->irsp == 1 && q->nl == 0)) {
    s->err = "bad frequency, heading or irsp arguments";
    return -2;
  }
  auto r = std::make_shared<Request>();
  r->n = q->n; r->ntnd = q->ntnd; r->nl = q->nl; r->nbody = q->nbody;
  copy_in(r->nodes, q->nodes, (size_t)q->ntnd * 3);
  copy_in(r->ncon, q->ncon, (size_t)q->n * 4);
  copy_in(r->ncn, q->ncn, (size_t)q->n);
  copy_in(r->xyz, q->xyz_p, (size_t)q->n * 3);
  copy_in(r->ds, q->ds, (size_t)q->n);
  copy_in(r->pnsz, q->pnsz, (size_t)q->n);
  copy_in(r->dxyz, q->dxyz_p, (size_t)q->n * 6);
  if (q->nl > 0) copy_in(r->lid, q->lid_xyz_p, (size_t)q->nl * 3);
  copy_in(r->ranges, q->body_ranges, (size_t)2 * q->nbody);
  r->h = q->h; r->nfreq = q->nfreq; r->irsp = q->irsp; r->isol = q->isol; r->nbeta = q->nbeta;
  r->nk = q->h > 0 ? q->nk : 0;
  copy_in(r->v, q->v, (size_t)q->nfreq);
  copy_in(r->wk, q->wk, (size_t)q->nfreq);
  copy_in(r->w1, q->w1, (size_t)q->nfreq);
  if (q->h > 0) copy_in(r->wvn, q->wvn, (size_t)q->nfreq * q->nk);
  if (q->nbeta > 0) copy_in(r->betas, q->betas, (size_t)q->nbeta);
  const int nd = 6 * q->nbody;
  r->amas.assign((size_t)q->nfreq * nd * nd, 0.0);
  r->bdmp.assign((size_t)q->nfreq * nd * nd, 0.0);
  r->exfc.assign((size_t)q->nfreq * (q->nbeta > 0 ? q->nbeta : 0) * nd * 2, 0.0);
  r->slot_bytes = hg_solve_footprint(s->opts.precision, q->n, q->nl, q->nbody, q->nbeta, q->irsp, s->opts.lu_tensor) +
                  iter_bytes(s->opts, *q);
  r->reserve = (size_t)std::min(s->nslots, q->nfreq) * r->slot_bytes + mesh_bytes(*r);
  if (r->reserve > s->budget) {
    s->err = "request needs " + std::to_string(r->reserve) + " bytes of device memory, above the budget of " +
             std::to_string(s->budget);
    return -3;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  r->t_submit = Clock::now();
  s->queue.push_back(r);
  s->all[r->id] = r;
  admit(s);
  s->cv_work.notify_all();
  *ticket = r->id;
  return 0;
}

int hg_server_wait(hg_server* s, long long ticket, double timeout_s, double* amas, double* bdmp, double* exfc,
                   double* latency_ms) {
  if (!s) return -1;
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) {
      s->err = "unknown ticket " + std::to_string(ticket);
      return -2;
    }
    r = it->second;
    auto pred = [&] { return r->finished; };
    if (timeout_s > 0) {
      if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return 1;  // not yet
    } else {
      s->cv_done.wait(lk, pred);
    }
    s->all.erase(ticket);
  }
  if (r->rc) {
    s->err = "request " + std::to_string(ticket) + ": " + r->err;
    return r->rc;
  }
  if (amas) std::memcpy(amas, r->amas.data(), r->amas.size() * sizeof(double));
  if (bdmp) std::memcpy(bdmp, r->bdmp.data(), r->bdmp.size() * sizeof(double));
  if (exfc && !r->exfc.empty()) std::memcpy(exfc, r->exfc.data(), r->exfc.size() * sizeof(double));
  if (latency_ms) {
    latency_ms[0] = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    latency_ms[1] = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
  }
  return 0;
}

int hg_server_stats(hg_server* s, double* stats) {
  if (!s || !stats) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  stats[0] = (double)s->n_done;
  stats[1] = (double)s->n_units;
  stats[2] = (double)s->reserved;
  stats[3] = (double)s->peak_reserved;
  stats[4] = (double)s->max_active;
  stats[5] = (double)s->queue.size();
  stats[6] = (double)s->active.size();
  stats[7] = (double)s->budget;
  return 0;
}

int hg_server_timeline(hg_server* s, int max_entries, double* out) {
  if (!s) return -1;
  if (max_entries < 0 || (max_entries > 0 && !out)) return -2;
  std::lock_guard<std::mutex> lk(s->mu);
  const int count = (int)(s->timeline.size() / 4);
  const int m = std::min(count, max_entries);
  if (m > 0) std::memcpy(out, s->timeline.data(), (size_t)4 * m * sizeof(double));
  return count;
}

}  // extern "C"
