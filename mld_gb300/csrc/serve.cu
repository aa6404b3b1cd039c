// Serving loop: energies, forces and stresses of structures with a fitted potential under
// continuous batching (the evaluation side of MILADY, mld.F90:1579-1867, as driven step by step
// by mld_md_driver.F90:324-375,579-651).
//
// A server owns n_slots evaluation slots, each a library handle with its own CUDA stream and
// device buffers (neighbour lists, descriptors and design rows stay on the device).  Requests
// queue on the host; progress() retires the batches whose completion event has fired (results
// come back through a pinned buffer) and fills every idle slot with the next requests in arrival
// order, admitted while the batch stays within the slot's share of the HBM budget and the atom
// cap.  Batches in different slots run concurrently on their streams, so requests that arrive
// while others are on the GPU start as soon as a slot and memory free up.  A request whose own
// size exceeds the per-slot share but fits the whole budget waits at the head of the queue
// until every slot is idle, then runs alone: nothing else is launched while it is on the GPU,
// and its slot's buffers are released when it retires, so the bytes on the device never exceed
// the budget.  A request larger than the whole budget fails with MLD_ERR_OOM.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mld_gpu.h"
#include "mld_internal.h"

namespace mld {
int eval_launch(mld_gpu_handle* h, cudaEvent_t done, double** pinned_out);
void eval_collect(const mld_gpu_handle* h, int s, double* E, double* F, double* Sout);
int eval_weights_upload(mld_gpu_handle* h, const double* w_full);
int handle_dims(const mld_gpu_handle* h, int* D, int* ldx, int* KK, int* nch);
void handle_release_buffers(mld_gpu_handle* h);
}  // namespace mld

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int nat = 0;
  std::vector<double> pos, cell;
  std::vector<int> types;
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 on the GPU, 2 done, 3 failed
  int err = 0;
  double E = 0;
  std::vector<double> F;
  double S[6] = {0, 0, 0, 0, 0, 0};
  double bytes = 0;
};

struct Slot {
  mld_gpu_handle* h = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<long long> batch;
  bool busy = false;
  double bytes = 0;  // estimated device bytes of the batch on the GPU
};

}  // namespace

struct mld_gpu_server {
  mld_gpu_config cfg;
  std::string err;
  std::vector<Slot> slots;
  std::deque<long long> queue;
  std::unordered_map<long long, Request> reqs;
  long long next_id = 1;
  long long max_batch_atoms = 0;
  double budget = 0;  // bytes of HBM for the slots' batch buffers
  int D = 0, ldx = 0, KK = 0, nch = 1;
  long long batches = 0, atoms_done = 0;
  int exclusive_slot = -1;       // slot running a request larger than the per-slot share
  double peak_in_flight = 0;     // largest sum of the busy slots' estimated bytes
  double largest_request = 0;    // largest estimated bytes of a request admitted so far
};

namespace {

int sfail(mld_gpu_server* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

// device bytes of one structure's batch buffers: neighbour pairs (expected neighbours from the
// number density within r_cut, 1.5x margin), per-atom descriptors and effective weights, the
// FP64 outputs (evaluation without design rows)
double request_bytes(const mld_gpu_server* s, int nat, const double* cell) {
  const double* c = cell;
  const double vol = std::fabs(c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                               c[2] * (c[3] * c[7] - c[4] * c[6]));
  const double rc = s->cfg.r_cut;
  const double nn = std::min<double>(s->cfg.imm_neigh, 1.5 * nat / std::max(vol, 1e-9) * 4.18879 * rc * rc * rc + 8);
  const double eb = s->cfg.precision == MLD_PRECISION_MIXED ? 4.0 : 8.0;
  const double pairs = nat * nn;
  // per pair: index, FP64 and FP32 displacement, reverse pair, the single-pass search row
  return pairs * 44.0 + nat * (2.0 * s->KK * eb + 24.0 + 64.0) + 128.0;
}

void retire(mld_gpu_server* s, int idx) {
  Slot& sl = s->slots[idx];
  const cudaError_t q = cudaEventQuery(sl.done);
  if (q == cudaErrorNotReady) return;
  const double t = now_ms();
  for (size_t i = 0; i < sl.batch.size(); ++i) {
    Request& r = s->reqs[sl.batch[i]];
    if (q == cudaSuccess) {
      r.F.assign(3 * (size_t)r.nat, 0.0);
      mld::eval_collect(sl.h, (int)i, &r.E, r.F.data(), r.S);
      r.state = 2;
      s->atoms_done += r.nat;
    } else {
      r.state = 3;
      r.err = MLD_ERR_CUDA;
    }
    r.t_done = t;
  }
  if (q != cudaSuccess) s->err = std::string("batch failed: ") + cudaGetErrorString(q);
  sl.batch.clear();
  sl.busy = false;
  sl.bytes = 0;
  if (s->exclusive_slot == idx) {
    // the slot grew its buffers past its share: give them back before others are admitted
    mld::handle_release_buffers(sl.h);
    s->exclusive_slot = -1;
  }
}

double bytes_in_flight(const mld_gpu_server* s) {
  double b = 0;
  for (const Slot& o : s->slots)
    if (o.busy) b += o.bytes;
  return b;
}

int launch(mld_gpu_server* s, int idx) {
  Slot& sl = s->slots[idx];
  if (s->exclusive_slot >= 0) return MLD_OK;  // an over-share request is running alone
  const double share = s->budget / std::max<size_t>(1, s->slots.size());
  bool exclusive = false;
  double used = 0;
  long long atoms = 0;
  std::vector<long long> batch;
  while (!s->queue.empty()) {
    const long long id = s->queue.front();
    Request& r = s->reqs[id];
    const bool first = batch.empty();
    if (!first && (used + r.bytes > share || atoms + r.nat > s->max_batch_atoms)) break;
    if (first && r.bytes > s->budget) {
      s->queue.pop_front();
      r.state = 3;
      r.err = MLD_ERR_OOM;
      r.t_done = now_ms();
      continue;
    }
    if (first && r.bytes > share) {
      // runs alone: hold it at the head (and launch nothing else) until every slot is idle
      if (bytes_in_flight(s) > 0) return MLD_OK;
      exclusive = true;
    }
    batch.push_back(id);
    used += r.bytes;
    atoms += r.nat;
    s->queue.pop_front();
    if (first && (r.bytes > share || r.nat > s->max_batch_atoms)) break;  // a large request runs alone
  }
  if (batch.empty()) return MLD_OK;
  std::vector<int> nat(batch.size());
  std::vector<double> pos, cell;
  std::vector<int> types;
  pos.reserve(3 * (size_t)atoms);
  types.reserve((size_t)atoms);
  cell.reserve(9 * batch.size());
  for (size_t i = 0; i < batch.size(); ++i) {
    Request& r = s->reqs[batch[i]];
    nat[i] = r.nat;
    pos.insert(pos.end(), r.pos.begin(), r.pos.end());
    cell.insert(cell.end(), r.cell.begin(), r.cell.end());
    types.insert(types.end(), r.types.begin(), r.types.end());
    r.state = 1;
  }
  int rc = mld_gpu_set_structures(sl.h, (int)batch.size(), nat.data(), pos.data(), cell.data(), types.data());
  double* pinned = nullptr;
  if (rc == MLD_OK) rc = mld::eval_launch(sl.h, sl.done, &pinned);
  if (rc != MLD_OK) {
    s->err = mld_gpu_last_error(sl.h);
    const double t = now_ms();
    for (long long id : batch) {
      Request& r = s->reqs[id];
      r.state = 3;
      r.err = rc;
      r.t_done = t;
    }
    return MLD_OK;  // the failure is recorded on the requests; the server stays usable
  }
  sl.batch = std::move(batch);
  sl.busy = true;
  sl.bytes = used;
  if (exclusive) s->exclusive_slot = idx;
  s->peak_in_flight = std::max(s->peak_in_flight, bytes_in_flight(s));
  s->largest_request = std::max(s->largest_request, used);
  ++s->batches;
  return MLD_OK;
}

}  // namespace

extern "C" {

int mld_gpu_server_create(const mld_gpu_config* cfg, const double* w_params, int n_slots, long long max_batch_atoms,
                          double hbm_fraction, mld_gpu_server** out) {
  if (!cfg || !w_params || !out || n_slots < 1 || max_batch_atoms < 1 || !(hbm_fraction > 0 && hbm_fraction <= 1))
    return MLD_ERR_INVALID;
  if (cfg->ml_type != 0) return MLD_ERR_UNSUPPORTED;  // linear and quadratic (QNML) potentials
  *out = nullptr;
  mld_gpu_server* s = new mld_gpu_server();
  s->cfg = *cfg;
  s->max_batch_atoms = max_batch_atoms;
  for (int i = 0; i < n_slots; ++i) {
    Slot sl;
    int rc = mld_gpu_create(cfg, &sl.h);
    if (rc != MLD_OK) {
      mld_gpu_server_destroy(s);
      return rc;
    }
    if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
      mld_gpu_destroy(sl.h);
      mld_gpu_server_destroy(s);
      return MLD_ERR_CUDA;
    }
    rc = mld::eval_weights_upload(sl.h, w_params);
    s->slots.push_back(sl);
    if (rc != MLD_OK) {
      mld_gpu_server_destroy(s);
      return rc;
    }
  }
  mld::handle_dims(s->slots[0].h, &s->D, &s->ldx, &s->KK, &s->nch);
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    mld_gpu_server_destroy(s);
    return MLD_ERR_CUDA;
  }
  s->budget = hbm_fraction * (double)fr;
  *out = s;
  return MLD_OK;
}

void mld_gpu_server_destroy(mld_gpu_server* s) {
  if (!s) return;
  for (Slot& sl : s->slots) {
    if (sl.h) mld_gpu_synchronize(sl.h);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.h) mld_gpu_destroy(sl.h);
  }
  delete s;
}

const char* mld_gpu_server_last_error(const mld_gpu_server* s) { return s ? s->err.c_str() : "null server"; }

int mld_gpu_server_submit(mld_gpu_server* s, int nat, const double* pos, const double* cell, const int* types,
                          long long* ticket) {
  if (!s || nat < 1 || !pos || !cell || !types || !ticket) return MLD_ERR_INVALID;
  Request r;
  r.nat = nat;
  r.pos.assign(pos, pos + 3 * (size_t)nat);
  r.cell.assign(cell, cell + 9);
  r.types.assign(types, types + nat);
  r.t_submit = now_ms();
  r.bytes = request_bytes(s, nat, cell);
  const long long id = s->next_id++;
  s->reqs.emplace(id, std::move(r));
  s->queue.push_back(id);
  *ticket = id;
  return MLD_OK;
}

int mld_gpu_server_progress(mld_gpu_server* s, int* n_busy, int* n_queued) {
  if (!s) return MLD_ERR_INVALID;
  for (size_t i = 0; i < s->slots.size(); ++i)
    if (s->slots[i].busy) retire(s, (int)i);
  for (size_t i = 0; i < s->slots.size(); ++i)
    if (!s->slots[i].busy && !s->queue.empty()) {
      const int rc = launch(s, (int)i);
      if (rc != MLD_OK) return rc;
    }
  if (n_busy) {
    int b = 0;
    for (const Slot& sl : s->slots) b += sl.busy;
    *n_busy = b;
  }
  if (n_queued) *n_queued = (int)s->queue.size();
  return MLD_OK;
}

int mld_gpu_server_result(mld_gpu_server* s, long long ticket, double* E, double* F, double* S, double* latency_ms,
                          int* ready) {
  if (!s || !ready) return MLD_ERR_INVALID;
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MLD_ERR_INVALID, "unknown ticket");
  Request& r = it->second;
  *ready = 0;
  if (r.state < 2) return MLD_OK;
  if (r.state == 3) {
    const int e = r.err;
    s->reqs.erase(it);
    return sfail(s, e, "request failed: " + s->err);
  }
  if (E) *E = r.E;
  if (F) std::memcpy(F, r.F.data(), sizeof(double) * r.F.size());
  if (S) std::memcpy(S, r.S, sizeof(double) * 6);
  if (latency_ms) *latency_ms = r.t_done - r.t_submit;
  *ready = 1;
  s->reqs.erase(it);
  return MLD_OK;
}

int mld_gpu_server_wait(mld_gpu_server* s, long long ticket, double* E, double* F, double* S, double* latency_ms,
                        double timeout_ms) {
  if (!s) return MLD_ERR_INVALID;
  const double t0 = now_ms();
  for (;;) {
    int ready = 0;
    int rc = mld_gpu_server_result(s, ticket, E, F, S, latency_ms, &ready);
    if (rc != MLD_OK || ready) return rc;
    rc = mld_gpu_server_progress(s, nullptr, nullptr);
    if (rc != MLD_OK) return rc;
    if (timeout_ms > 0 && now_ms() - t0 > timeout_ms) return sfail(s, MLD_ERR_TIMEOUT, "request not finished in time");
  }
}

int mld_gpu_server_stats(const mld_gpu_server* s, long long* batches, long long* atoms_done, double* budget_bytes) {
  if (!s) return MLD_ERR_INVALID;
  if (batches) *batches = s->batches;
  if (atoms_done) *atoms_done = s->atoms_done;
  if (budget_bytes) *budget_bytes = s->budget;
  return MLD_OK;
}

int mld_gpu_server_admission(const mld_gpu_server* s, double* peak_bytes_in_flight, double* share_bytes,
                             double* largest_batch_bytes) {
  if (!s) return MLD_ERR_INVALID;
  if (peak_bytes_in_flight) *peak_bytes_in_flight = s->peak_in_flight;
  if (share_bytes) *share_bytes = s->budget / std::max<size_t>(1, s->slots.size());
  if (largest_batch_bytes) *largest_batch_bytes = s->largest_request;
  return MLD_OK;
}

}  // extern "C"
