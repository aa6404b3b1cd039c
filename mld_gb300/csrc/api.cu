// C ABI of libmld_gpu (declared in include/mld_gpu.h): handle, staging, orchestration.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/mld_gpu.h"
#include "mld_internal.h"


using namespace mld;

namespace {

struct Buf {
  void* p = nullptr;
  size_t cap = 0;
};

struct RowLayout {
  std::vector<long long> rowE, rowF, rowS;
  long long M = 0;
};

}  // namespace

struct mld_gpu_handle {
  mld_gpu_config cfg;
  std::string err;
  cudaStream_t st = nullptr;
  int device = 0;
  Bso4Tables tab;
  DevTables dt;
  BsoParams bp;
  int nch = 1, K = 0, KK = 0, D = 0, ldx = 0;
  // quadratic model (mld_order = 2): linear block DL = 1 + KK, upper-triangle quadratic block DQ
  bool quad = false;
  int DL = 0, DQ = 0, Dfull = 0;
  // kernel ridge regression (ml_type 1): nk standardised reference points, columns DL .. DL+nk
  bool krr = false;
  int nk = 0;
  double lam_eff = 0.0;  // ridge added to the normal-matrix diagonal (lambda, or lambda^2 for KRR)
  bool mixed = false;

  // staged batch
  int S = 0, A = 0;
  std::vector<int> h_atom_start;
  DevBatch b;
  bool has_batch = false;
  bool nbr_valid = false;
  int max_nn = 0;
  // neighbours per atom that the single-pass search reserves: 1.5 x the densest structure's
  // mean count within r_cut, + 8 (at most imm_neigh); an atom above it reruns the two passes
  int nn_bound = 0;

  // labels
  bool has_labels = false;
  std::vector<int> h_has;  // 3*S
  RowLayout fit_rows;

  // profiling: CUDA event pairs around each phase interval of a fit, accumulated after its
  // final sync; kernel launches are counted per interval at the launch sites
  bool prof = false;
  std::vector<cudaEvent_t> evpool;
  struct Interval {
    int phase, ev;
    long long launches;
  };
  std::vector<Interval> pending;
  int cur_phase = -1, cur_ev = -1;
  long long cur_launches = 0;
  cudaEvent_t tev[2] = {};
  double ms[MLD_NPHASE] = {0};
  long long launches[MLD_NPHASE] = {0};
  long long calls[MLD_NPHASE] = {0};

  // serving: row layout of the last launched batch and its pinned prediction buffer
  RowLayout serve_rows;
  double* pinned = nullptr;
  size_t pinned_cap = 0;

  // device properties and the last mixed-method solve
  int nsm = 0;
  int pcg_iters[2] = {0, 0};
  double precond_shift[2] = {0, 0};
  double ew0 = 0.0;        // constant weight of the evaluation weights (B_EW)
  bool ew_ready = false;
  double pcg_rel[2] = {0, 0};
  int chol_retries = 0;
  int last_rank = 0;  // rank of the last symmetric solve (eigenvalues kept by the rcond cut)

  // descriptor-kernel launch shape per output mode (0: B and dB, 1: evaluation, 2: B only),
  // chosen by timing the candidates once on a batch of at least kTuneMinAtoms per SM
  struct Tune {
    bool done = false;
    Bso4Launch best;
    std::vector<Bso4Launch> cand;
    std::vector<float> ms;
  } tune[3];

  // CUDA graph of the row-assembly stage (descriptor kernel, reverse pairs, row gathers) of the
  // staged batch, replayed by later fits of the same batch; key = buffer generation and sizes
  long long buf_gen = 0;  // bumped whenever a device buffer is (re)allocated or freed
  cudaGraphExec_t rows_graph = nullptr;
  long long rows_graph_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long rows_graph_launches = 0;
  bool rows_graph_off = false;  // a capture failed once: run the stage directly from then on

  std::vector<void*> owned;  // table allocations
  Buf bufs[80];
  enum {
    B_ATOM_START, B_ATOM_STRUCT, B_TYPES, B_POS, B_CELL, B_RECIP, B_SMALL, B_NSIZE, B_VOL,
    B_NN, B_NBR_OFF, B_NBR_IDX, B_NBR_U, B_SCAN_TMP, B_MAXNN,
    B_E, B_F, B_S, B_WEFS,
    B_ROWE, B_ROWF, B_ROWS, B_X, B_Y, B_WROW, B_KIND,
    B_G, B_H, B_W, B_EVALS, B_INFO, B_SQ, B_PRED, B_BOUT, B_DBOUT,
    B_REV, B_HQ, B_YQ, B_GF, B_RES, B_DW,
    B_GWS, B_TERR, B_PCG, B_POS32, B_YSCR, B_RINV, B_KZD, B_KZF, B_KWS, B_WSERVE, B_P32,
    B_EW, B_EBETA, B_EB, B_EOUT, B_KTC, B_SKW, B_ORDER, B_QCNT, B_SP, B_EPAIR, B_EATOM, B_GP,
    B_CNC, B_CELLOFF, B_CELLOF, B_CELLSTART, B_CELLATOMS, B_SORTTMP, B_NBR_U32, B_MVWS, B_GTCP, B_NBRTMP,
    B_COUNT
  };
  static_assert(B_COUNT <= 80, "buffer table too small");
};

namespace {

int fail(mld_gpu_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(mld_gpu_handle* h, cudaError_t e, const char* where) {
  return fail(h, e == cudaErrorMemoryAllocation ? MLD_ERR_OOM : MLD_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) return cuda_fail(h, _e, #call); \
  } while (0)

cudaError_t ensure(mld_gpu_handle* h, int id, size_t bytes) {
  Buf& bf = h->bufs[id];
  if (bytes <= bf.cap && bf.p) return cudaSuccess;
  ++h->buf_gen;
  if (bf.p) cudaFree(bf.p);
  bf.p = nullptr;
  bf.cap = 0;
  size_t want = std::max<size_t>(bytes, 256);
  want = want + want / 8;  // headroom for slowly growing batches
  cudaError_t e = cudaMalloc(&bf.p, want);
  if (e != cudaSuccess) return e;
  bf.cap = want;
  return cudaSuccess;
}

template <typename P>
P* bp_(mld_gpu_handle* h, int id) {
  return reinterpret_cast<P*>(h->bufs[id].p);
}

template <typename V>
cudaError_t upload(mld_gpu_handle* h, int id, const V* src, size_t n) {
  cudaError_t e = ensure(h, id, sizeof(V) * n);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  return cudaMemcpyAsync(h->bufs[id].p, src, sizeof(V) * n, cudaMemcpyHostToDevice, h->st);
}

template <typename V>
cudaError_t dev_alloc_copy(mld_gpu_handle* h, V** dst, const V* src, size_t n) {
  cudaError_t e = cudaMalloc((void**)dst, sizeof(V) * std::max<size_t>(n, 1));
  if (e != cudaSuccess) return e;
  h->owned.push_back(*dst);
  if (n) e = cudaMemcpy(*dst, src, sizeof(V) * n, cudaMemcpyHostToDevice);
  return e;
}

void recips(const double* cell, double* bg) {
  const double *a1 = cell, *a2 = cell + 3, *a3 = cell + 6;
  double c23[3] = {a2[1] * a3[2] - a2[2] * a3[1], a2[2] * a3[0] - a2[0] * a3[2], a2[0] * a3[1] - a2[1] * a3[0]};
  double c31[3] = {a3[1] * a1[2] - a3[2] * a1[1], a3[2] * a1[0] - a3[0] * a1[2], a3[0] * a1[1] - a3[1] * a1[0]};
  double c12[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
  double vol = a1[0] * c23[0] + a1[1] * c23[1] + a1[2] * c23[2];
  for (int c = 0; c < 3; ++c) {
    bg[c] = c23[c] / vol;
    bg[3 + c] = c31[c] / vol;
    bg[6 + c] = c12[c] / vol;
  }
}

// Row layout: energy row, 3*nat force rows, 6 stress rows per structure, in structure order.
RowLayout make_layout(const mld_gpu_handle* h, const std::vector<int>& has, bool force_all) {
  RowLayout L;
  L.rowE.assign(h->S, -1);
  L.rowF.assign(h->S, -1);
  L.rowS.assign(h->S, -1);
  long long r = 0;
  for (int s = 0; s < h->S; ++s) {
    int nat = h->h_atom_start[s + 1] - h->h_atom_start[s];
    bool e = force_all || has[3 * s];
    bool f = force_all || (has[3 * s + 1] && h->cfg.desc_forces);
    bool st = force_all || (has[3 * s + 2] && h->cfg.desc_forces);
    if (e) L.rowE[s] = r++;
    if (f) {
      L.rowF[s] = r;
      r += 3LL * nat;
    }
    if (st) {
      L.rowS[s] = r;
      r += 6;
    }
  }
  L.M = r;
  return L;
}

// Phase intervals: mark(h, p, 0) opens an interval of phase p, mark(h, p, 1) closes it; a
// phase may be entered several times per fit.  nl() counts the kernels launched inside.
void mark(mld_gpu_handle* h, int phase, int end) {
  if (!h->prof) return;
  if (!end) {
    const int idx = (int)h->pending.size();
    while ((int)h->evpool.size() < 2 * (idx + 1)) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      h->evpool.push_back(e);
    }
    cudaEventRecord(h->evpool[2 * idx], h->st);
    h->cur_phase = phase;
    h->cur_ev = idx;
    h->cur_launches = 0;
  } else if (h->cur_phase == phase && h->cur_ev >= 0) {
    cudaEventRecord(h->evpool[2 * h->cur_ev + 1], h->st);
    h->pending.push_back({phase, h->cur_ev, h->cur_launches});
    h->cur_phase = -1;
    h->cur_ev = -1;
  }
}

inline void nl(mld_gpu_handle* h, long long n) { h->cur_launches += n; }

int build_neighbours(mld_gpu_handle* h) {
  if (!h->has_batch) return fail(h, MLD_ERR_STATE, "no structures staged");
  DevBatch& b = h->b;
  CK(ensure(h, mld_gpu_handle::B_NN, sizeof(int) * std::max(1, h->A)));
  CK(ensure(h, mld_gpu_handle::B_NBR_OFF, sizeof(int) * (h->A + 1)));
  CK(ensure(h, mld_gpu_handle::B_SCAN_TMP, sizeof(int) * ((h->A + 1023) / 1024 + 2)));
  CK(ensure(h, mld_gpu_handle::B_MAXNN, sizeof(int) * 2));
  CK(ensure(h, mld_gpu_handle::B_POS32, sizeof(float4) * 2 * (size_t)std::max(1, h->A)));
  b.pos32 = bp_<float4>(h, mld_gpu_handle::B_POS32);
  b.frac32 = b.pos32 + std::max(1, h->A);
  b.nn = bp_<int>(h, mld_gpu_handle::B_NN);
  b.nbr_off = bp_<int>(h, mld_gpu_handle::B_NBR_OFF);
  int* dmax = bp_<int>(h, mld_gpu_handle::B_MAXNN);
  CK(cudaMemsetAsync(dmax, 0, sizeof(int), h->st));
  if (b.ncells > 0) {
    CK(ensure(h, mld_gpu_handle::B_SCAN_TMP, sizeof(int) * ((std::max(h->A, b.ncells) + 1023) / 1024 + 2)));
    CK(launch_cells(b, bp_<int>(h, mld_gpu_handle::B_SCAN_TMP), h->st));
    nl(h, 5);
  }
  // one scan of the candidates into rows of nn_bound pairs per atom when that workspace can be
  // had, else (or when an atom has more) a counting scan and a filling scan
  b.nbr_cap = 0;
  b.nbr_tmp = nullptr;
  if (h->nn_bound > 0 && h->A > 0) {
    const size_t tb = sizeof(int2) * (size_t)h->A * (size_t)h->nn_bound;
    if (ensure(h, mld_gpu_handle::B_NBRTMP, tb) == cudaSuccess) {
      b.nbr_cap = h->nn_bound;
      b.nbr_tmp = bp_<int2>(h, mld_gpu_handle::B_NBRTMP);
    } else {
      cudaGetLastError();  // the failed allocation leaves no error for later launches
    }
  }
  CK(launch_neighbours(b, h->cfg.r_cut, b.nn, dmax, h->st, b.nbr_cap > 0 ? 2 : 0));
  CK(launch_scan(b.nn, b.nbr_off, h->A, bp_<int>(h, mld_gpu_handle::B_SCAN_TMP), h->st));
  nl(h, 5);
  int hv[2] = {0, 0};
  CK(cudaMemcpyAsync(&hv[0], b.nbr_off + h->A, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(&hv[1], dmax, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (b.nbr_cap > 0 && hv[1] > b.nbr_cap && hv[1] <= h->cfg.imm_neigh) b.nbr_cap = 0;  // the rows overflowed
  if (hv[1] > h->cfg.imm_neigh)
    return fail(h, MLD_ERR_NEIGHBOUR_CAP,
                "an atom has " + std::to_string(hv[1]) + " neighbours within r_cut, more than imm_neigh=" +
                    std::to_string(h->cfg.imm_neigh));
  h->max_nn = hv[1];
  b.maxnn = hv[1];
  b.P = hv[0];
  CK(ensure(h, mld_gpu_handle::B_NBR_IDX, sizeof(int) * std::max<long long>(b.P, 1)));
  CK(ensure(h, mld_gpu_handle::B_NBR_U, sizeof(double) * 3 * std::max<long long>(b.P, 1)));
  b.nbr_idx = bp_<int>(h, mld_gpu_handle::B_NBR_IDX);
  b.nbr_u = bp_<double>(h, mld_gpu_handle::B_NBR_U);
  b.nbr_u32 = nullptr;
  if (h->mixed) {
    CK(ensure(h, mld_gpu_handle::B_NBR_U32, sizeof(float4) * std::max<long long>(b.P, 1)));
    b.nbr_u32 = bp_<float4>(h, mld_gpu_handle::B_NBR_U32);
  }
  if (b.ncells > 0 && b.P > 0) {
    // workspace of the sort of the celled structures' lists (inside the filling pass)
    CK(ensure(h, mld_gpu_handle::B_SORTTMP, sizeof(int) * (size_t)b.P));
    b.sort_tmp = bp_<int>(h, mld_gpu_handle::B_SORTTMP);
    nl(h, 1);
  }
  CK(launch_neighbours(b, h->cfg.r_cut, b.nn, dmax, h->st, b.nbr_cap > 0 ? 3 : 1));
  nl(h, b.P > 0 ? 2 : 1);  // filling pass (or compaction) and pair displacements
  // longest-first order of the descriptor kernel's work queue; one counter int + sort workspace
  CK(ensure(h, mld_gpu_handle::B_ORDER, sizeof(int) * std::max(1, h->A)));
  CK(ensure(h, mld_gpu_handle::B_QCNT, sizeof(int) * (4 + atom_order_tmp_ints(h->max_nn))));
  CK(launch_atom_order(b.nn, h->A, h->max_nn, bp_<int>(h, mld_gpu_handle::B_ORDER),
                       bp_<int>(h, mld_gpu_handle::B_QCNT) + 4, h->st));
  nl(h, 3);
  h->nbr_valid = true;
  return MLD_OK;
}



// workspace of the tensor-core kernel-row product (derivative-vector planes of one atom chunk)
constexpr size_t kKrrTcWorkspaceCap = size_t(6) << 30;

// global Y scratch of the descriptor kernel when its per-atom Y does not fit in shared memory
template <typename T>
int y_scratch(mld_gpu_handle* h, void** p, size_t* bytes) {
  *bytes = bso4_y_scratch_bytes(h->dt, h->nch, (int)sizeof(T), 2 * std::max(1, h->nsm));
  *p = nullptr;
  if (*bytes) {
    CK(ensure(h, mld_gpu_handle::B_YSCR, *bytes));
    *p = bp_<void>(h, mld_gpu_handle::B_YSCR);
  }
  return MLD_OK;
}

// Autotuner of the descriptor kernel's launch shape for the design rows of a fit: on the first
// batch large enough (at least kTuneMinAtoms atoms per SM) each candidate shape (column tile 4 or 2, as many persistent CTAs
// per SM as fit or one, longest-first or index-order queue) runs once on the real batch, timed
// with CUDA events on the handle's stream, and the fastest is kept for the handle.  Every shape
// computes bitwise the same outputs, so the last candidate's run is the result.
constexpr int kTuneMinAtoms = 64;

template <typename T>
int tuned_launch(mld_gpu_handle* h, int mode, T* Bout, T* dB, const DevEval<T>* ev, void* ys, size_t ysb) {
  auto& tn = h->tune[mode];
  const int* order = bp_<int>(h, mld_gpu_handle::B_ORDER);
  int* counter = bp_<int>(h, mld_gpu_handle::B_QCNT);
  // only the design-row stage of a fit is tuned: it is repeated on the same batch, while
  // evaluation batches (serving) and descriptor dumps change from call to call
  if (tn.done || mode != 0 || h->A < kTuneMinAtoms * std::max(1, h->nsm)) {
    CK(launch_bso4<T>(h->dt, h->b, h->bp, Bout, dB, ev, order, counter, h->st, ys, ysb, &tn.best));
    return MLD_OK;
  }
  tn.cand.clear();
  tn.ms.clear();
  for (int ct : {4, 2})
    for (int cps : {0, 1})
      for (int sorted : {1, 0}) tn.cand.push_back(Bso4Launch{ct, cps, sorted});
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  float best = 0.f;
  for (const Bso4Launch& c : tn.cand) {
    CK(cudaEventRecord(ev0, h->st));
    CK(launch_bso4<T>(h->dt, h->b, h->bp, Bout, dB, ev, order, counter, h->st, ys, ysb, &c));
    CK(cudaEventRecord(ev1, h->st));
    CK(cudaEventSynchronize(ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev0, ev1));
    tn.ms.push_back(ms);
    if (tn.ms.size() == 1 || ms < best) {
      best = ms;
      tn.best = c;
    }
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  nl(h, (long long)tn.cand.size() - 1);
  tn.done = true;
  return MLD_OK;
}

template <typename T>
int prepare_descriptors(mld_gpu_handle* h, bool want_dB, void** ys, size_t* ysb) {
  int rcy = y_scratch<T>(h, ys, ysb);
  if (rcy) return rcy;
  if (want_dB) CK(ensure(h, mld_gpu_handle::B_DBOUT, sizeof(T) * std::max<size_t>((size_t)h->b.P * 3 * h->KK, 1)));
  return MLD_OK;
}

// B and w_ch * dB of the staged batch into B_BOUT / B_DBOUT (dB optional) through the
// descriptor kernel's queue
template <typename T>
int run_descriptors(mld_gpu_handle* h, bool want_dB, const DevEval<T>* ev, T* Bout) {
  void* ys = nullptr;
  size_t ysb = 0;
  int rcy = prepare_descriptors<T>(h, want_dB, &ys, &ysb);
  if (rcy) return rcy;
  T* dB = want_dB ? bp_<T>(h, mld_gpu_handle::B_DBOUT) : nullptr;
  const int mode = ev ? 1 : (want_dB ? 0 : 2);
  int rc = tuned_launch<T>(h, mode, Bout, dB, ev, ys, ysb);
  if (rc) return rc;
  nl(h, 1);
  return MLD_OK;
}

template <typename T>
int run_rows(mld_gpu_handle* h, const RowLayout& L, bool with_labels, T** Xout) {
  if (h->krr && h->nk == 0) return fail(h, MLD_ERR_STATE, "kernel model without reference points");
  DevRows rows;
  rows.M = L.M;
  rows.D = h->D;
  rows.ldx = h->ldx;
  CK(upload(h, mld_gpu_handle::B_ROWE, L.rowE.data(), h->S));
  CK(upload(h, mld_gpu_handle::B_ROWF, L.rowF.data(), h->S));
  CK(upload(h, mld_gpu_handle::B_ROWS, L.rowS.data(), h->S));
  rows.rowE = bp_<long long>(h, mld_gpu_handle::B_ROWE);
  rows.rowF = bp_<long long>(h, mld_gpu_handle::B_ROWF);
  rows.rowS = bp_<long long>(h, mld_gpu_handle::B_ROWS);
  size_t xbytes = sizeof(T) * (size_t)std::max<long long>(L.M, 1) * h->ldx;
  CK(ensure(h, mld_gpu_handle::B_X, xbytes));
  CK(ensure(h, mld_gpu_handle::B_Y, sizeof(double) * std::max<long long>(L.M, 1)));
  CK(ensure(h, mld_gpu_handle::B_WROW, sizeof(double) * std::max<long long>(L.M, 1)));
  CK(ensure(h, mld_gpu_handle::B_KIND, sizeof(int) * std::max<long long>(L.M, 1)));
  T* X = bp_<T>(h, mld_gpu_handle::B_X);
  mark(h, MLD_PHASE_ROWS, 0);
  CK(cudaMemsetAsync(X, 0, xbytes, h->st));
  const double* dE = with_labels ? bp_<double>(h, mld_gpu_handle::B_E) : nullptr;
  if (with_labels) {
    CK(launch_rows_prep<T>(h->S, h->b.atom_start, rows, bp_<double>(h, mld_gpu_handle::B_E),
                           bp_<double>(h, mld_gpu_handle::B_F), bp_<double>(h, mld_gpu_handle::B_S),
                           bp_<double>(h, mld_gpu_handle::B_WEFS), X, bp_<double>(h, mld_gpu_handle::B_Y),
                           bp_<double>(h, mld_gpu_handle::B_WROW), bp_<int>(h, mld_gpu_handle::B_KIND), h->st));
  } else {
    // energy-row constant column only; labels unused
    std::vector<double> zeros(1, 0.0);
    (void)zeros;
    (void)dE;
    CK(ensure(h, mld_gpu_handle::B_E, sizeof(double) * std::max(1, h->S)));
    CK(ensure(h, mld_gpu_handle::B_F, sizeof(double) * 3 * std::max(1, h->A)));
    CK(ensure(h, mld_gpu_handle::B_S, sizeof(double) * 6 * std::max(1, h->S)));
    CK(ensure(h, mld_gpu_handle::B_WEFS, sizeof(double) * 3 * std::max(1, h->S)));
    CK(launch_rows_prep<T>(h->S, h->b.atom_start, rows, bp_<double>(h, mld_gpu_handle::B_E),
                           bp_<double>(h, mld_gpu_handle::B_F), bp_<double>(h, mld_gpu_handle::B_S),
                           bp_<double>(h, mld_gpu_handle::B_WEFS), X, bp_<double>(h, mld_gpu_handle::B_Y),
                           bp_<double>(h, mld_gpu_handle::B_WROW), bp_<int>(h, mld_gpu_handle::B_KIND), h->st));
  }
  nl(h, 1);
  mark(h, MLD_PHASE_ROWS, 1);
  mark(h, MLD_PHASE_DESCRIPTORS, 0);
  {
    // B of every atom and w_ch * dB of every pair, then the rows gathered through the reverse
    // pairs in a fixed order (rows.cu); the quadratic and kernel columns use the same B and dB
    const size_t nB = (size_t)std::max(1, h->A) * h->KK;
    CK(ensure(h, mld_gpu_handle::B_BOUT, sizeof(T) * nB));
    CK(ensure(h, mld_gpu_handle::B_REV, sizeof(int) * (size_t)std::max<long long>(1, h->b.P)));
    CK(ensure(h, mld_gpu_handle::B_SP, sizeof(T) * nB * 6));
    if (h->quad) CK(ensure(h, mld_gpu_handle::B_HQ, sizeof(T) * (size_t)std::max(1, h->A) * 6 * h->KK));
    T* Bq = bp_<T>(h, mld_gpu_handle::B_BOUT);
    void* ys = nullptr;
    size_t ysb = 0;
    int rcd = prepare_descriptors<T>(h, true, &ys, &ysb);
    if (rcd) return rcd;
    T* dBq = bp_<T>(h, mld_gpu_handle::B_DBOUT);
    // the stage of this batch: descriptor kernel, reverse pairs, linear (and quadratic) rows
    auto stage = [&]() -> int {
      int rc = run_descriptors<T>(h, true, nullptr, Bq);
      if (rc) return rc;
      CK(launch_reverse_pairs(h->b, bp_<int>(h, mld_gpu_handle::B_REV), h->st));
      CK(launch_lin_rows<T>(h->b, rows, h->bp, h->KK, bp_<int>(h, mld_gpu_handle::B_REV), Bq, dBq,
                            bp_<T>(h, mld_gpu_handle::B_SP), X, h->st));
      nl(h, 3);
      if (h->quad) {
        CK(launch_quad_rows<T>(h->b, rows, h->bp, h->KK, bp_<int>(h, mld_gpu_handle::B_REV), Bq, dBq,
                               bp_<T>(h, mld_gpu_handle::B_HQ), X, h->DL, h->st));
        nl(h, 2);
      }
      return MLD_OK;
    };
    if (h->krr || !h->tune[0].done || h->rows_graph_off) {
      // the kernel model's rows synchronise on a timeout flag, and the autotuner times its
      // candidates: both run directly
      int rc = stage();
      if (rc) return rc;
    } else {
      // replayed as a CUDA graph, captured once per batch (and buffer generation)
      const long long key[8] = {h->buf_gen, h->A, h->b.P, h->S, L.M, h->b.maxnn, h->quad ? 1 : 0,
                                (long long)(uintptr_t)X};
      if (!h->rows_graph || !std::equal(key, key + 8, h->rows_graph_key)) {
        if (h->rows_graph) cudaGraphExecDestroy(h->rows_graph);
        h->rows_graph = nullptr;
        const long long l0 = h->cur_launches;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeRelaxed));
        const int rc = stage();
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(h->st, &g);
        if (rc) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        cudaError_t ei = ec;
        if (ec == cudaSuccess) ei = cudaGraphInstantiate(&h->rows_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        const long long captured = h->cur_launches - l0;  // kernels of the graph
        h->cur_launches = l0;
        if (ei != cudaSuccess) {
          // the capture did not take: clear the error and run the stage directly from now on
          (void)cudaGetLastError();
          h->rows_graph = nullptr;
          h->rows_graph_off = true;
          int rc2 = stage();
          if (rc2) return rc2;
        } else {
          std::copy(key, key + 8, h->rows_graph_key);
          h->rows_graph_launches = captured;
        }
      }
      if (h->rows_graph) {
        CK(cudaGraphLaunch(h->rows_graph, h->st));
        nl(h, h->rows_graph_launches);
      }
    }
    if (h->krr) {
      // kernel columns (compute_kernel.F90, mld_energy/forces/stress kernel packing)
      const size_t wse = krr_workspace_elems(h->A, h->nk, h->KK);
      CK(ensure(h, mld_gpu_handle::B_KWS, sizeof(T) * wse));
      const T* Zp = bp_<T>(h, sizeof(T) == 8 ? mld_gpu_handle::B_KZD : mld_gpu_handle::B_KZF);
      int nkl = 0;
      // FP32 rows: force rows on the tensor cores, in atom chunks that fit a bounded workspace
      void* tcws = nullptr;
      size_t tcb = 0;
      int* terr = nullptr;
      if (sizeof(T) == 4 && krr_force_tc_available() && h->KK <= kKrrTcMaxK) {
        // all atoms at once when that fits the cap, else chunks of at least 64 atoms
        const int maxnv = h->b.maxnn + 1;
        tcb = std::min(kKrrTcWorkspaceCap, krr_force_tc_workspace_bytes(h->A, maxnv, (int)h->nk, h->KK));
        tcb = std::max(tcb, krr_force_tc_workspace_bytes(std::min<long long>(h->A, 64), maxnv, (int)h->nk, h->KK));
        CK(ensure(h, mld_gpu_handle::B_KTC, tcb));
        CK(ensure(h, mld_gpu_handle::B_TERR, sizeof(int)));
        tcws = bp_<void>(h, mld_gpu_handle::B_KTC);
        terr = bp_<int>(h, mld_gpu_handle::B_TERR);
        CK(cudaMemsetAsync(terr, 0, sizeof(int), h->st));
      }
      CK(launch_krr_rows<T>(h->b, rows, bp_<int>(h, mld_gpu_handle::B_REV), Bq, dBq, Zp, h->nk, h->KK,
                            h->cfg.kernel_power, h->cfg.length_kernel, h->cfg.sigma_kernel, h->cfg.sign_stress,
                            h->cfg.sign_stress_big_box, bp_<T>(h, mld_gpu_handle::B_KWS), X, h->DL, h->st, &nkl, tcws,
                            tcb, terr, h->nsm));
      nl(h, nkl);
      if (terr) {
        int herr = 0;
        CK(cudaMemcpyAsync(&herr, terr, sizeof(int), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        if (herr) return fail(h, MLD_ERR_TIMEOUT, "tensor-core kernel rows: a pipeline wait timed out");
      }
    }
  }
  mark(h, MLD_PHASE_DESCRIPTORS, 1);
  *Xout = X;
  return MLD_OK;
}

// workspace of the fixed-order Gram / rhs reductions over M rows of D columns
double* gram_ws(mld_gpu_handle* h, long long M, int D) {
  if (ensure(h, mld_gpu_handle::B_GP, sizeof(double) * gram_workspace_doubles(M, D)) != cudaSuccess) return nullptr;
  return bp_<double>(h, mld_gpu_handle::B_GP);
}

// Symmetric solve of (G + lambda I) w = rhs with the reference's dgelsd semantics
// (stats_tools.F90:1153-1213: minimum-norm solution, singular values below rcond * s_max cut).
//  * D <= 112: one-CTA Jacobi eigen-solve.  When it cuts no eigenvalue (full rank), the same
//    solution is recomputed from the Cholesky factor with two FP64 refinement steps, which is
//    more accurate than the eigen-solve on an ill-conditioned matrix; a cut keeps the
//    minimum-norm eigen-solution.
//  * above: blocked Cholesky with two refinement steps (diagonal shift lambda, or a 1e-12
//    relative jitter when lambda <= 0 or the factorisation fails).
// G is left intact.
int chol_refined(mld_gpu_handle* h, const double* G, const double* rhs, int D, double shift, double* w, int* hinfo) {
  CK(ensure(h, mld_gpu_handle::B_GF, sizeof(double) * (size_t)D * D));
  CK(ensure(h, mld_gpu_handle::B_RES, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_DW, sizeof(double) * 3 * (size_t)D));
  CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
  double* Lf = bp_<double>(h, mld_gpu_handle::B_GF);
  double* r = bp_<double>(h, mld_gpu_handle::B_RES);
  double* dw = bp_<double>(h, mld_gpu_handle::B_DW);
  double* tmp = dw + D;
  int* info = bp_<int>(h, mld_gpu_handle::B_INFO);
  CK(cudaMemcpyAsync(Lf, G, sizeof(double) * (size_t)D * D, cudaMemcpyDeviceToDevice, h->st));
  CK(launch_cholesky(Lf, D, shift, info, h->st));
  CK(cudaMemcpyAsync(hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  nl(h, cholesky_launches(D));
  if (*hinfo != 0) return MLD_OK;
  CK(launch_chol_solve_blocked(Lf, D, rhs, w, tmp, h->st));
  for (int it = 0; it < 2; ++it) {
    CK(launch_residual(G, D, shift, w, rhs, r, h->st));
    CK(launch_chol_solve_blocked(Lf, D, r, dw, tmp, h->st));
    CK(launch_axpy(D, 1.0, dw, w, h->st));
  }
  nl(h, 3 * chol_solve_launches(D) + 4);
  return MLD_OK;
}

int solve_any(mld_gpu_handle* h, double* G, const double* rhs, int D, double* w) {
  if (D <= 112) {
    CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
    int* info = bp_<int>(h, mld_gpu_handle::B_INFO);
    CK(launch_solve_sym(G, rhs, D, h->lam_eff, h->cfg.svd_rcond, w, bp_<double>(h, mld_gpu_handle::B_EVALS), info,
                        h->st));
    nl(h, 1);
    int hv[2] = {0, 0};
    CK(cudaMemcpyAsync(hv, info, sizeof(int) * 2, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->last_rank = hv[1];
    if (hv[1] < D) return MLD_OK;  // eigenvalues cut: the minimum-norm solution stands
    int hinfo = 0;
    return chol_refined(h, G, rhs, D, h->lam_eff > 0 ? h->lam_eff : 0.0, w, &hinfo);  // on failure w is kept
  }
  // diagonal shift: lambda, but at least 1e-12 of the largest diagonal entry (a rank-deficient
  // normal matrix: the min-norm solution of dgelsd differs only in the near-null space); x10 on
  // a failed factorisation
  std::vector<double> diag(D);
  CK(cudaMemcpy2DAsync(diag.data(), sizeof(double), G, sizeof(double) * (D + 1), sizeof(double), D,
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double mx = 0;
  for (double v : diag) mx = std::max(mx, std::fabs(v));
  double jitter = 1e-12 * (mx > 0 ? mx : 1.0);
  int hinfo = 0;
  h->last_rank = D;
  for (int attempt = 0; attempt < 5; ++attempt, jitter *= 10.0) {
    const double shift = std::max(h->lam_eff > 0 ? h->lam_eff : 0.0, jitter);
    int rc = chol_refined(h, G, rhs, D, shift, w, &hinfo);
    if (rc) return rc;
    if (hinfo == 0) break;
  }
  if (hinfo != 0)
    return fail(h, MLD_ERR_SOLVE, "normal matrix not positive definite at column " + std::to_string(hinfo));
  return MLD_OK;
}

// weights of the reference's full quadratic layout <-> the deduplicated working layout
void dedup_to_full(const mld_gpu_handle* h, const double* wd, double* wf) {
  const int KK = h->KK, DL = h->DL;
  for (int c = 0; c < DL; ++c) wf[c] = wd[c];
  const double r2 = std::sqrt(2.0);
  for (int i = 0, q = 0; i < KK; ++i)
    for (int j = i; j < KK; ++j, ++q) {
      const double v = wd[DL + q];
      if (i == j) wf[DL + KK * i + j] = v;
      else wf[DL + KK * i + j] = wf[DL + KK * j + i] = v / r2;
    }
}
void full_to_dedup(const mld_gpu_handle* h, const double* wf, double* wd) {
  const int KK = h->KK, DL = h->DL;
  for (int c = 0; c < DL; ++c) wd[c] = wf[c];
  const double r2 = std::sqrt(2.0);
  for (int i = 0, q = 0; i < KK; ++i)
    for (int j = i; j < KK; ++j, ++q)
      wd[DL + q] = (i == j) ? wf[DL + KK * i + j] : (wf[DL + KK * i + j] + wf[DL + KK * j + i]) / r2;
}

// a working-layout design row -> the reference's row (full K*K quadratic block)
void export_row(const mld_gpu_handle* h, const double* xd, double* xf) {
  const int KK = h->KK, DL = h->DL;
  if (h->krr) {
    for (int c = 0; c < h->D; ++c) xf[c] = xd[c];
    return;
  }
  for (int c = 0; c < DL; ++c) xf[c] = xd[c];
  if (!h->quad) return;
  const double r2 = std::sqrt(2.0);
  for (int i = 0, q = 0; i < KK; ++i)
    for (int j = i; j < KK; ++j, ++q) {
      const double v = xd[DL + q];
      if (i == j) xf[DL + KK * i + j] = v;
      else xf[DL + KK * i + j] = xf[DL + KK * j + i] = v / r2;
    }
}

__global__ void k_sub(long long n, const double* a, const double* b, double* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

// Kernel launches per phase of one fit (neighbours: count, 3 scan kernels, fill; rows: labels
// kernel; descriptors: fused bispectrum kernel; Gram: tiles, rhs, symmetrise; solve; predict).
void accumulate_profile(mld_gpu_handle* h) {
  if (!h->prof) return;
  for (const auto& iv : h->pending) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, h->evpool[2 * iv.ev], h->evpool[2 * iv.ev + 1]) == cudaSuccess) {
      h->ms[iv.phase] += t;
      h->launches[iv.phase] += iv.launches;
      h->calls[iv.phase] += 1;
    }
  }
  h->pending.clear();
}

// Plain method, one block of columns [c0, c0 + Db): FP64 Gram on the CUDA cores and the
// symmetric solve (min-norm Jacobi / Cholesky), parameters.F90:1018-1099.
int fit_block_plain(mld_gpu_handle* h, const double* X, int c0, int Db, const double* y, long long M, double* w) {
  double* G = bp_<double>(h, mld_gpu_handle::B_G);
  double* hv = bp_<double>(h, mld_gpu_handle::B_H);
  mark(h, MLD_PHASE_GRAM, 0);
  double* gws = gram_ws(h, M, Db);
  if (!gws) return fail(h, MLD_ERR_OOM, "Gram workspace");
  CK(launch_gram<double>(X + c0, h->ldx, bp_<double>(h, mld_gpu_handle::B_WROW), y, M, Db, G, hv, h->st, gws));
  nl(h, 5);  // tiles, tile reduction, rhs partials, rhs reduction, symmetrise
  mark(h, MLD_PHASE_GRAM, 1);
  mark(h, MLD_PHASE_SOLVE, 0);
  int rc = solve_any(h, G, hv, Db, w);
  if (rc) return rc;
  mark(h, MLD_PHASE_SOLVE, 1);
  return MLD_OK;
}

constexpr size_t kGramWorkspaceCap = size_t(8) << 30;  // bf16 planes of one row chunk
constexpr int kPcgMaxIter = 150;
constexpr double kPcgObjTol = 1e-7;  // relative objective decrease over three steps that ends CG
// relative diagonal shift of the preconditioner: max(min, per_column * D), x3 while not SPD
constexpr double kPrecondShiftMin = 1e-6;
constexpr double kPrecondShiftPerColumn = 2e-7;
constexpr double kPcgTol2 = 1e-22;   // (preconditioned residual / initial)^2 that ends the iteration
constexpr double kPcgFloor2 = 1e-14; // below this, stagnation also ends it
constexpr int kSketchMinD = 768;     // blocks this wide get the sketched preconditioner (sketch.cu)
constexpr uint64_t kSketchSeed = 0x5EED5EED12345ull;

// Mixed method, one block of columns [c0, c0 + Db) of the FP32 design matrix; blocks of
// kSketchMinD columns or more take fit_block_sketch instead.
//  * normal matrix G~ = X^T W X on the tensor cores in BF16 split precision (gram_tc.cu) and
//    rhs = X^T W y with FP64 accumulation;
//  * preconditioner: FP64 Cholesky of G~ + diag(max(lambda, rel * G~_ii)), rel = max(1e-6,
//    2e-7 * D) (x3 on a failed factorisation);
//    applied through the explicit inverse of the factor (two dense FP64 triangular matvecs);
//  * conjugate gradients on (X^T W X + lambda I) w = X^T W y with FP64-accumulated matvecs
//    over X itself, so the converged coefficients are those of the FP64 normal equations of
//    this X, whatever the precision of G~.
int pcg_solve(mld_gpu_handle* h, const float* X, int c0, int Db, const double* y, long long M, double lam,
              double* w, int stage, const std::function<cudaError_t(const double*, double*)>& precond);

// Mixed method, wide block (Db >= kSketchMinD): the preconditioner is the FP64 Cholesky factor
// of Y^T Y + mu I for the sketch Y = S W^1/2 X (sketch.cu), whose error grows with the condition
// number of X rather than of X^T X, and CG runs on (X^T W X + mu I) w = X^T W y with
// mu = max(lambda, 1e-12 max_i G_ii), the diagonal shift of the plain solver (solve_any).
int fit_block_sketch(mld_gpu_handle* h, const float* X, int c0, int Db, const double* y, long long M, double* w,
                     int stage) {
  double* G = bp_<double>(h, mld_gpu_handle::B_G);
  double* hv = bp_<double>(h, mld_gpu_handle::B_H);
  const double* wrow = bp_<double>(h, mld_gpu_handle::B_WROW);
  mark(h, MLD_PHASE_GRAM, 0);
  CK(ensure(h, mld_gpu_handle::B_TERR, sizeof(int)));
  CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * (size_t)std::max<long long>(M, 1)));
  double* rws = gram_ws(h, M, Db);
  if (!rws) return fail(h, MLD_ERR_OOM, "rhs workspace");
  CK(launch_rhs<float>(X + c0, h->ldx, wrow, y, M, Db, hv, h->nsm, h->st, bp_<float2>(h, mld_gpu_handle::B_PRED), rws));
  nl(h, 3);
  if (M >= (1LL << 31)) return fail(h, MLD_ERR_INVALID, "sketch: more than 2^31 design rows");
  const SketchParams P = sketch_params(M, Db, kSketchSeed + (uint64_t)stage);
  CK(ensure(h, mld_gpu_handle::B_SKW, sketch_workspace_bytes(M, Db)));
  int nsk = 0;
  CK(launch_sketch_gram(X, h->ldx, c0, Db, wrow, M, P, bp_<void>(h, mld_gpu_handle::B_SKW), G, h->st, &nsk));
  nl(h, nsk + 1);
  mark(h, MLD_PHASE_GRAM, 1);

  mark(h, MLD_PHASE_SOLVE, 0);
  CK(ensure(h, mld_gpu_handle::B_GF, sizeof(double) * (size_t)Db * Db));
  CK(ensure(h, mld_gpu_handle::B_PCG, sizeof(double) * (7 * (size_t)Db + 8)));
  CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
  CK(ensure(h, mld_gpu_handle::B_P32, precond32_workspace_bytes(Db)));
  double* Lf = bp_<double>(h, mld_gpu_handle::B_GF);
  double* tmp = bp_<double>(h, mld_gpu_handle::B_PCG) + 4 * (size_t)Db;  // 2 Db
  int* info = bp_<int>(h, mld_gpu_handle::B_INFO);
  std::vector<double> diag(Db);
  CK(cudaMemcpy2DAsync(diag.data(), sizeof(double), G, sizeof(double) * (Db + 1), sizeof(double), Db,
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double mx = 0;
  for (double v : diag) mx = std::max(mx, std::fabs(v));
  const double lam = h->lam_eff > 0 ? h->lam_eff : 0.0;
  double jitter = 1e-12 * (mx > 0 ? mx : 1.0);
  const double mu = std::max(lam, jitter);
  int retries = 0, hinfo = 0;
  for (double shift = mu;; shift = std::max(mu, jitter *= 10.0), ++retries) {
    CK(cudaMemcpyAsync(Lf, G, sizeof(double) * (size_t)Db * Db, cudaMemcpyDeviceToDevice, h->st));
    CK(launch_cholesky(Lf, Db, shift, info, h->st, true));
    nl(h, cholesky_launches(Db));
    CK(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (hinfo == 0) {
      h->precond_shift[stage] = shift / (mx > 0 ? mx : 1.0);
      break;
    }
    if (retries >= 5)
      return fail(h, MLD_ERR_SOLVE, "sketched preconditioner not positive definite at column " + std::to_string(hinfo));
  }
  h->chol_retries += retries;
  void* pws = bp_<void>(h, mld_gpu_handle::B_P32);
  int ninv = 0;
  CK(launch_precond32_from_factor(Lf, Db, pws, h->st, &ninv));
  nl(h, ninv);
  auto precond = [&](const double* rr, double* zz) { return launch_precond32_apply(pws, Db, rr, zz, tmp, h->st); };
  return pcg_solve(h, X, c0, Db, y, M, mu, w, stage, precond);
}

int fit_block_mixed(mld_gpu_handle* h, const float* X, int c0, int Db, const double* y, long long M, double* w,
                    int stage) {
  if (Db >= kSketchMinD) return fit_block_sketch(h, X, c0, Db, y, M, w, stage);
  double* G = bp_<double>(h, mld_gpu_handle::B_G);
  double* hv = bp_<double>(h, mld_gpu_handle::B_H);
  const double* wrow = bp_<double>(h, mld_gpu_handle::B_WROW);
  const double lam = h->lam_eff > 0 ? h->lam_eff : 0.0;
  mark(h, MLD_PHASE_GRAM, 0);
  const size_t need = (size_t)4 * Db * (size_t)((std::max<long long>(M, 1) + 63) / 64 * 64) + 256;
  const size_t wsb = std::max(gram_tc_min_workspace(Db), std::min(need, kGramWorkspaceCap));
  CK(ensure(h, mld_gpu_handle::B_GWS, wsb));
  CK(ensure(h, mld_gpu_handle::B_TERR, sizeof(int)));
  int* terr = bp_<int>(h, mld_gpu_handle::B_TERR);
  CK(cudaMemsetAsync(G, 0, sizeof(double) * (size_t)Db * Db, h->st));
  CK(cudaMemsetAsync(terr, 0, sizeof(int), h->st));
  if (!gram_tc_available()) return fail(h, MLD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const size_t npart = gram_tc_part_doubles(Db, h->nsm);
  CK(ensure(h, mld_gpu_handle::B_GTCP, sizeof(double) * std::max<size_t>(npart, 1)));
  CK(launch_gram_tc<float>(X, h->ldx, c0, Db, wrow, M, G, bp_<void>(h, mld_gpu_handle::B_GWS), wsb, terr, h->nsm,
                           h->st, bp_<double>(h, mld_gpu_handle::B_GTCP), npart));
  const long long chunk = (long long)((wsb - 256) / (4 * (size_t)Db)) / 64 * 64;
  nl(h, 2 * ((M + chunk - 1) / chunk));
  CK(launch_symmetrize(G, Db, h->st));
  CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * (size_t)std::max<long long>(M, 1)));
  double* rws = gram_ws(h, M, Db);
  if (!rws) return fail(h, MLD_ERR_OOM, "rhs workspace");
  CK(launch_rhs<float>(X + c0, h->ldx, wrow, y, M, Db, hv, h->nsm, h->st, bp_<float2>(h, mld_gpu_handle::B_PRED),
                       rws));
  nl(h, 3);
  mark(h, MLD_PHASE_GRAM, 1);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, terr, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (herr) return fail(h, MLD_ERR_TIMEOUT, "tensor-core Gram: a pipeline wait timed out");

  mark(h, MLD_PHASE_SOLVE, 0);
  CK(ensure(h, mld_gpu_handle::B_GF, sizeof(double) * (size_t)Db * Db));
  CK(ensure(h, mld_gpu_handle::B_PCG, sizeof(double) * (7 * (size_t)Db + 8)));
  CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
  CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * (size_t)std::max<long long>(M, 1)));
  double* Lf = bp_<double>(h, mld_gpu_handle::B_GF);
  double* tmp = bp_<double>(h, mld_gpu_handle::B_PCG) + 4 * (size_t)Db;  // 2 Db
  int* info = bp_<int>(h, mld_gpu_handle::B_INFO);
  // the error of the BF16x3 Gram is coherent across the matrix (the tensor core truncates its
  // FP32 sums), so the shift that keeps G~ positive definite grows with D
  double rel = std::max(kPrecondShiftMin, kPrecondShiftPerColumn * Db);
  int retries = 0;
  for (;; ++retries) {
    CK(cudaMemcpyAsync(Lf, G, sizeof(double) * (size_t)Db * Db, cudaMemcpyDeviceToDevice, h->st));
    CK(launch_shift_diag_rel(Lf, Db, lam, rel, h->st));
    CK(launch_cholesky(Lf, Db, 0.0, info, h->st));
    nl(h, 1 + cholesky_launches(Db));
    int hinfo = 0;
    CK(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (hinfo == 0) break;
    if (retries >= 6)
      return fail(h, MLD_ERR_SOLVE, "preconditioner not positive definite at column " + std::to_string(hinfo));
    rel *= 3.0;
  }
  h->precond_shift[stage] = rel;
  h->chol_retries += retries;
  // explicit inverse of the factor: each preconditioner application is two dense matvecs
  CK(ensure(h, mld_gpu_handle::B_RINV, sizeof(double) * 2 * (size_t)Db * Db));
  double* Rinv = bp_<double>(h, mld_gpu_handle::B_RINV);
  double* Rinvt = Rinv + (size_t)Db * Db;
  int ninv = 0;
  CK(launch_cholesky_inverse(Lf, Db, Rinv, Rinvt, h->st, &ninv));
  nl(h, ninv);
  auto precond = [&](const double* rr, double* zz) { return launch_precond_apply(Rinv, Rinvt, Db, rr, zz, tmp, h->st); };
  return pcg_solve(h, X, c0, Db, y, M, lam, w, stage, precond);
}

// Conjugate gradients on (X^T W X + lam I) w = X^T W y (the right-hand side in B_H) from w = 0,
// with FP64-accumulated matvecs over the FP32 rows of X and the given preconditioner; stops on
// the preconditioned residual, on the objective's decrease or on stagnation.
int pcg_solve(mld_gpu_handle* h, const float* X, int c0, int Db, const double* y, long long M, double lam,
              double* w, int stage, const std::function<cudaError_t(const double*, double*)>& precond) {
  const double* hv = bp_<double>(h, mld_gpu_handle::B_H);
  const double* wrow = bp_<double>(h, mld_gpu_handle::B_WROW);
  int* terr = bp_<int>(h, mld_gpu_handle::B_TERR);
  double* r = bp_<double>(h, mld_gpu_handle::B_PCG);
  double* z = r + Db;
  double* p = z + Db;
  double* q = p + Db;
  double* scal = q + 3 * (size_t)Db;  // [0..3] CG scalars, [4] objective at w = 0
  float2* sv = bp_<float2>(h, mld_gpu_handle::B_PRED);  // per-row double-FP32 scratch
  // per-block partial sums of the matvecs and of the objective, reduced in block order
  const size_t nmvws = std::max<size_t>(normal_matvec_workspace_doubles(M, Db, h->nsm), kSumsqBlocksMax);
  CK(ensure(h, mld_gpu_handle::B_MVWS, sizeof(double) * nmvws));
  double* mvws = bp_<double>(h, mld_gpu_handle::B_MVWS);
  int herr = 0;
  // objective sum_r w_r y_r^2 at w = 0, for the stopping test on its decrease
  CK(launch_weighted_sumsq(wrow, y, M, scal + 4, mvws, h->st));
  nl(h, 2);
  // x0 = 0, r0 = rhs
  CK(cudaMemsetAsync(w, 0, sizeof(double) * Db, h->st));
  CK(cudaMemcpyAsync(r, hv, sizeof(double) * Db, cudaMemcpyDeviceToDevice, h->st));
  CK(precond(r, z));
  CK(launch_pcg_beta(Db, z, r, p, scal, 1, h->st));
  nl(h, 3);
  CK(launch_split_weights(wrow, M, sv, h->st));  // the fused matvecs read w as pairs
  CK(cudaMemsetAsync(terr, 0, sizeof(int), h->st));
  nl(h, 1);
  double hs[5] = {0, 0, 0, 0, 0};
  double prev = 0.0, fobj = -1.0, dec_hist[3] = {0, 0, 0};
  int it = 0, slow = 0;
  for (; it < kPcgMaxIter; ++it) {
    int nmv = 0;
    CK(launch_normal_matvec(X, h->ldx, c0, Db, wrow, p, M, lam, sv, q, mvws, h->nsm, h->st, &nmv, terr));
    CK(launch_pcg_alpha(Db, p, q, w, r, scal, h->st));
    CK(precond(r, z));
    CK(launch_pcg_beta(Db, z, r, p, scal, 0, h->st));
    nl(h, nmv + 4);
    CK(cudaMemcpyAsync(hs, scal, sizeof(double) * 5, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const double ratio = hs[1] > 0 ? hs[0] / hs[1] : 0.0;
    if (!(ratio > kPcgTol2)) {
      ++it;
      break;
    }
    // least-squares objective: f_k = f_0 - sum of the step decreases alpha_j (r.z)_j; stop once
    // three steps together lower it by less than kPcgObjTol of its value
    if (fobj < 0) fobj = hs[4];
    fobj -= hs[3];
    dec_hist[it % 3] = hs[3];
    if (it >= 2 && fobj > 0 && dec_hist[0] + dec_hist[1] + dec_hist[2] < kPcgObjTol * fobj) {
      ++it;
      break;
    }
    // stagnation at the FP64 rounding floor of the matvec: three steps without halving r.z
    slow = (it > 0 && ratio < kPcgFloor2 && hs[0] > 0.5 * prev) ? slow + 1 : 0;
    prev = hs[0];
    if (slow >= 3) {
      ++it;
      break;
    }
  }
  CK(cudaMemcpyAsync(&herr, terr, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (herr) return fail(h, MLD_ERR_TIMEOUT, "normal-equation matvec: a pipeline wait timed out");
  h->pcg_iters[stage] = it;
  h->pcg_rel[stage] = hs[1] > 0 ? std::sqrt(std::max(hs[0], 0.0) / hs[1]) : 0.0;
  mark(h, MLD_PHASE_SOLVE, 1);
  return MLD_OK;
}

template <typename T>
int fit_block(mld_gpu_handle* h, const T* X, int c0, int Db, const double* y, long long M, double* w, int stage);
template <>
int fit_block<double>(mld_gpu_handle* h, const double* X, int c0, int Db, const double* y, long long M, double* w,
                      int) {
  return fit_block_plain(h, X, c0, Db, y, M, w);
}
template <>
int fit_block<float>(mld_gpu_handle* h, const float* X, int c0, int Db, const double* y, long long M, double* w,
                     int stage) {
  return fit_block_mixed(h, X, c0, Db, y, M, w, stage);
}

void set_lam_eff(mld_gpu_handle* h) {
  const double l = h->cfg.lambda_krr > 0 ? h->cfg.lambda_krr : 0.0;
  h->lam_eff = h->krr ? l * l : l;  // parameters.F90:1018-1099 (lambda) / :1217-1395 (lambda^2)
}

template <typename T>
int fit_impl(mld_gpu_handle* h, double* w_params, double* rmse) {
  if (h->krr && h->nk == 0) return fail(h, MLD_ERR_STATE, "kernel model without reference points");
  set_lam_eff(h);
  h->pending.clear();
  h->pcg_iters[0] = h->pcg_iters[1] = 0;
  h->chol_retries = 0;
  mark(h, MLD_PHASE_NEIGHBOURS, 0);
  int rc = build_neighbours(h);
  if (rc) return rc;
  mark(h, MLD_PHASE_NEIGHBOURS, 1);
  T* X = nullptr;
  rc = run_rows<T>(h, h->fit_rows, true, &X);
  if (rc) return rc;
  const long long M = h->fit_rows.M;
  const int D = h->D;
  const size_t gdim = (size_t)std::max(h->krr ? h->D : h->DL, h->DQ);
  CK(ensure(h, mld_gpu_handle::B_G, sizeof(double) * gdim * gdim));
  CK(ensure(h, mld_gpu_handle::B_H, sizeof(double) * gdim));
  CK(ensure(h, mld_gpu_handle::B_W, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_EVALS, sizeof(double) * gdim));
  CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
  CK(ensure(h, mld_gpu_handle::B_SQ, sizeof(double) * predict_sq_doubles()));
  double* w = bp_<double>(h, mld_gpu_handle::B_W);
  double* y = bp_<double>(h, mld_gpu_handle::B_Y);
  // linear block (QNML stage 1, or the whole linear model): parameters.F90:1018-1099; the
  // kernel model is one block of all its columns (parameters.F90:1217-1395)
  rc = fit_block<T>(h, X, 0, h->krr ? h->D : h->DL, y, M, w, 0);
  if (rc) return rc;
  if (h->quad) {
    // QNML stage 2 (parameters.F90:404-421, 476-1015): the quadratic block is fitted to the
    // residual of the linear fit with the same ridge solver
    CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * std::max<long long>(M, 1)));
    CK(ensure(h, mld_gpu_handle::B_YQ, sizeof(double) * std::max<long long>(M, 1)));
    double* pred = bp_<double>(h, mld_gpu_handle::B_PRED);
    double* yq = bp_<double>(h, mld_gpu_handle::B_YQ);
    mark(h, MLD_PHASE_PREDICT, 0);
    CK(launch_predict_sq<T>(X, h->ldx, w, M, h->DL, pred, nullptr, nullptr, nullptr, h->st));
    k_sub<<<(unsigned)((M + 255) / 256), 256, 0, h->st>>>(M, y, pred, yq);
    CK(cudaGetLastError());
    nl(h, 2);
    mark(h, MLD_PHASE_PREDICT, 1);
    rc = fit_block<T>(h, X, h->DL, h->DQ, yq, M, w + h->DL, 1);
    if (rc) return rc;
  }
  double* sq = bp_<double>(h, mld_gpu_handle::B_SQ);
  mark(h, MLD_PHASE_PREDICT, 0);
  CK(cudaMemsetAsync(sq, 0, sizeof(double) * 6, h->st));
  CK(launch_predict_sq<T>(X, h->ldx, w, M, D, nullptr, bp_<double>(h, mld_gpu_handle::B_Y), bp_<int>(h, mld_gpu_handle::B_KIND),
                          sq, h->st));
  nl(h, 2);
  mark(h, MLD_PHASE_PREDICT, 1);
  double hsq[6];
  std::vector<double> wd(D);
  CK(cudaMemcpyAsync(wd.data(), w, sizeof(double) * D, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(hsq, sq, sizeof(double) * 6, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (w_params) {
    if (h->quad) dedup_to_full(h, wd.data(), w_params);
    else std::copy(wd.begin(), wd.end(), w_params);
  }
  accumulate_profile(h);
  if (rmse)
    for (int k = 0; k < 3; ++k) rmse[k] = hsq[3 + k] > 0 ? std::sqrt(hsq[k] / hsq[3 + k]) : 0.0;
  return MLD_OK;
}

}  // namespace

namespace mld {
int eval_weights_upload(mld_gpu_handle* h, const double* w_full);
int eval_launch(mld_gpu_handle* h, cudaEvent_t done, double** pinned_out);
}  // namespace mld

extern "C" {

void mld_gpu_config_defaults(mld_gpu_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->descriptor_type = 9;
  c->j_max = 1.5;
  c->r_cut = 5.0;
  c->inv_r0_input = 1.0 - 0.02 / 3.14159265358979323846;
  c->weighted = 0;
  c->weighted_3ch = 0;
  c->n_elements = 1;
  for (int i = 0; i < MLD_MAX_ELEMENTS; ++i) {
    c->weight_per_element[i] = 1.0;
    c->weight_per_element_3ch[i] = 1.0;
  }
  c->r_cut_width_in = 0.4;
  c->desc_forces = 1;
  c->ml_type = 0;
  c->mld_order = 1;
  c->lambda_krr = -1.0;
  c->svd_rcond = -1.0;
  c->sign_stress = 1.0;
  c->sign_stress_big_box = 1.0;
  c->imm_neigh = 300;
  c->precision = MLD_PRECISION_PLAIN_FP64;
  c->kernel_type = 4;
  c->kernel_power = 2.0;
  c->length_kernel = std::sqrt(0.5);
  c->sigma_kernel = 0.0;
}

const char* mld_gpu_last_error(const mld_gpu_handle* h) { return h ? h->err.c_str() : "null handle"; }

int mld_gpu_create(const mld_gpu_config* cfg, mld_gpu_handle** out) {
  if (!cfg || !out) return MLD_ERR_INVALID;
  *out = nullptr;
  if (cfg->descriptor_type != 9) return MLD_ERR_UNSUPPORTED;
  if (cfg->ml_type != 0 && cfg->ml_type != 1) return MLD_ERR_UNSUPPORTED;
  if (cfg->ml_type == 0 && cfg->mld_order != 1 && cfg->mld_order != 2) return MLD_ERR_UNSUPPORTED;
  if (cfg->ml_type == 1 && cfg->kernel_type != 4) return MLD_ERR_UNSUPPORTED;  // polynomial kernel only
  if (cfg->ml_type == 1 && !(cfg->length_kernel > 0)) return MLD_ERR_INVALID;
  if (!(cfg->inv_r0_input > 0.0 && cfg->inv_r0_input < 1.0)) return MLD_ERR_INVALID;  // test_parameters_bso4
  if (cfg->j_max < 0 || !(cfg->r_cut > 0)) return MLD_ERR_INVALID;
  if (cfg->n_elements < 1 || cfg->n_elements > MLD_MAX_ELEMENTS) return MLD_ERR_INVALID;
  if (cfg->weighted_3ch && !cfg->weighted) return MLD_ERR_INVALID;
  if (cfg->precision != MLD_PRECISION_PLAIN_FP64 && cfg->precision != MLD_PRECISION_MIXED) return MLD_ERR_INVALID;
  if (cfg->imm_neigh < 1) return MLD_ERR_INVALID;
  mld_gpu_handle* h = new mld_gpu_handle();
  h->cfg = *cfg;
  h->mixed = cfg->precision == MLD_PRECISION_MIXED;
  if (!build_bso4_tables(cfg->j_max, &h->tab, &h->err)) {
    delete h;
    return MLD_ERR_INVALID;
  }
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return MLD_ERR_CUDA;
  }
  const Bso4Tables& t = h->tab;
  h->nch = cfg->weighted ? (cfg->weighted_3ch ? 3 : 2) : 1;
  h->K = t.K;
  h->KK = h->nch * t.K;
  h->DL = 1 + h->KK;
  h->krr = cfg->ml_type == 1;
  h->quad = !h->krr && cfg->mld_order == 2;
  set_lam_eff(h);
  h->DQ = h->quad ? h->KK * (h->KK + 1) / 2 : 0;
  h->D = h->DL + h->DQ;                                       // working (deduplicated) row width
  h->Dfull = h->DL + (h->quad ? h->KK * h->KK : 0);           // reference layout (dim_design_line)
  h->ldx = round_up4(h->D);
  // device tables
  e = fill_dev_tables(t, &h->dt, [h](const auto& vec, auto** dst) { return dev_alloc_copy(h, dst, vec.data(), vec.size()); });
  if (e != cudaSuccess) {
    int code = cuda_fail(h, e, "table upload");
    mld_gpu_destroy(h);
    return code;
  }
  // parameters
  BsoParams& p = h->bp;
  std::memset(&p, 0, sizeof(p));
  p.rcut = cfg->r_cut;
  p.inv_r0 = 3.14159265358979323846 * cfg->inv_r0_input;
  p.nch = h->nch;
  p.ntypes = cfg->n_elements;
  for (int tt = 0; tt < cfg->n_elements; ++tt) {
    p.chw[0 * p.ntypes + tt] = 1.0;
    if (h->nch > 1) p.chw[1 * p.ntypes + tt] = cfg->weight_per_element[tt];
    if (h->nch > 2) p.chw[2 * p.ntypes + tt] = cfg->weight_per_element_3ch[tt];
  }
  p.has_rin = 0;
  for (int a = 0; a < cfg->n_elements; ++a)
    for (int c2 = 0; c2 < cfg->n_elements; ++c2) {
      double v = cfg->r_cut_pair_in[a * MLD_MAX_ELEMENTS + c2];
      p.rin[a * p.ntypes + c2] = v;
      if (v > 0) p.has_rin = 1;
    }
  p.rin_width = cfg->r_cut_width_in;
  p.sign_stress = cfg->sign_stress;
  p.sign_big = cfg->sign_stress_big_box;
  *out = h;
  return MLD_OK;
}

void mld_gpu_destroy(mld_gpu_handle* h) {
  if (!h) return;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->rows_graph) cudaGraphExecDestroy(h->rows_graph);
  for (auto& bf : h->bufs)
    if (bf.p) cudaFree(bf.p);
  for (void* p : h->owned) cudaFree(p);
  if (h->pinned) cudaFreeHost(h->pinned);
  for (auto& e : h->evpool)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->tev)
    if (e) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

int mld_gpu_dims(const mld_gpu_handle* h, int* K, int* dim_desc, int* dim_design_line) {
  if (!h) return MLD_ERR_INVALID;
  if (K) *K = h->K;
  if (dim_desc) *dim_desc = h->KK;
  if (dim_design_line) *dim_design_line = h->Dfull;
  return MLD_OK;
}

int mld_gpu_set_structures(mld_gpu_handle* h, int nstruct, const int* nat, const double* pos, const double* cell,
                           const int* types) {
  if (!h) return MLD_ERR_INVALID;
  if (nstruct < 0 || (nstruct > 0 && (!nat || !cell))) return fail(h, MLD_ERR_INVALID, "bad structure arrays");
  std::vector<int> start(nstruct + 1, 0);
  for (int s = 0; s < nstruct; ++s) {
    if (nat[s] < 0) return fail(h, MLD_ERR_INVALID, "negative atom count");
    start[s + 1] = start[s] + nat[s];
  }
  const int A = start[nstruct];
  if (A > 0 && (!pos || !types)) return fail(h, MLD_ERR_INVALID, "missing positions or types");
  std::vector<int> astruct(A);
  for (int s = 0; s < nstruct; ++s)
    for (int i = start[s]; i < start[s + 1]; ++i) astruct[i] = s;
  for (int i = 0; i < A; ++i)
    if (types[i] < 0 || types[i] >= h->cfg.n_elements) return fail(h, MLD_ERR_INVALID, "type index out of range");
  for (long long i = 0; i < 3LL * A; ++i)
    if (!std::isfinite(pos[i])) return fail(h, MLD_ERR_INVALID, "non-finite position");
  std::vector<double> rec(9 * (size_t)nstruct), vol(nstruct);
  std::vector<int> small(nstruct), nsize(3 * (size_t)nstruct);
  // linked cells of large boxes with at least kCellMinAtoms atoms and three cells along some
  // direction: cells at least r_cut + 1e-3 A wide (perpendicular width / count)
  constexpr int kCellMinAtoms = 64;
  std::vector<int> cnc(3 * (size_t)nstruct, 0), cell_off(nstruct + 1, 0);
  for (int s = 0; s < nstruct; ++s) {
    const double* cl = cell + 9 * (size_t)s;
    recips(cl, &rec[9 * (size_t)s]);
    double v = cl[0] * (cl[4] * cl[8] - cl[5] * cl[7]) - cl[1] * (cl[3] * cl[8] - cl[5] * cl[6]) +
               cl[2] * (cl[3] * cl[7] - cl[4] * cl[6]);
    if (!(std::fabs(v) > 0)) return fail(h, MLD_ERR_INVALID, "singular cell");
    vol[s] = std::fabs(v);
    // neighbours.F90:787-847
    int sm = 0;
    for (int i = 0; i < 3; ++i) {
      const double* bgi = &rec[9 * (size_t)s + 3 * i];
      double bval = 1.0 / std::sqrt(bgi[0] * bgi[0] + bgi[1] * bgi[1] + bgi[2] * bgi[2]);
      int nc = (int)(2.0 * h->cfg.r_cut / bval) + 1;
      if (nc > 1) sm = 1;
      nsize[3 * s + i] = nc / 2 + 1;
      // the neighbour search packs each periodic image index in 8 bits
      if (nsize[3 * s + i] > 127)
        return fail(h, MLD_ERR_INVALID, "structure " + std::to_string(s) +
                                            ": cell too thin for r_cut (more than 127 periodic images along a lattice vector)");
    }
    small[s] = sm;
    int ncell = 0;
    if (!sm && nat[s] >= kCellMinAtoms) {
      int n[3], mx = 0;
      for (int i = 0; i < 3; ++i) {
        const double* bgi = &rec[9 * (size_t)s + 3 * i];
        const double width = 1.0 / std::sqrt(bgi[0] * bgi[0] + bgi[1] * bgi[1] + bgi[2] * bgi[2]);
        n[i] = std::max(1, std::min(1024, (int)std::floor(width / (h->cfg.r_cut + 1e-3))));
        mx = std::max(mx, n[i]);
      }
      if (mx >= 3 && (long long)n[0] * n[1] * n[2] <= 4LL * nat[s] + 64) {
        for (int i = 0; i < 3; ++i) cnc[3 * s + i] = n[i];
        ncell = n[0] * n[1] * n[2];
      }
    }
    cell_off[s + 1] = cell_off[s] + ncell;
  }
  {
    const double rc3 = h->cfg.r_cut * h->cfg.r_cut * h->cfg.r_cut;
    double worst = 0.0;
    for (int s = 0; s < nstruct; ++s) worst = std::max(worst, nat[s] / vol[s]);
    h->nn_bound = (int)std::min<double>(h->cfg.imm_neigh, 1.5 * worst * 4.18879 * rc3 + 8.0);
  }
  h->S = nstruct;
  h->A = A;
  h->h_atom_start = start;
  DevBatch& b = h->b;
  b.S = nstruct;
  b.A = A;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_ATOM_START, start.data(), start.size());
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_ATOM_STRUCT, astruct.data(), astruct.size());
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_TYPES, types, (size_t)A);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_POS, pos, 3 * (size_t)A);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_CELL, cell, 9 * (size_t)nstruct);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_RECIP, rec.data(), rec.size());
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_SMALL, small.data(), small.size());
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_NSIZE, nsize.data(), nsize.size());
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_VOL, vol.data(), vol.size());
  const int ncells = cell_off[nstruct];
  if (ncells > 0) {
    if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_CNC, cnc.data(), cnc.size());
    if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_CELLOFF, cell_off.data(), cell_off.size());
    if (e == cudaSuccess) e = ensure(h, mld_gpu_handle::B_CELLOF, sizeof(int) * (size_t)std::max(1, A));
    if (e == cudaSuccess) e = ensure(h, mld_gpu_handle::B_CELLSTART, sizeof(int) * (2 * (size_t)ncells + 1));
    if (e == cudaSuccess) e = ensure(h, mld_gpu_handle::B_CELLATOMS, sizeof(int) * (size_t)std::max(1, A));
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "mld_gpu_set_structures");
  b.ncells = ncells;
  b.cnc = ncells ? bp_<int>(h, mld_gpu_handle::B_CNC) : nullptr;
  b.cell_off = ncells ? bp_<int>(h, mld_gpu_handle::B_CELLOFF) : nullptr;
  b.cell_of = ncells ? bp_<int>(h, mld_gpu_handle::B_CELLOF) : nullptr;
  b.cell_start = ncells ? bp_<int>(h, mld_gpu_handle::B_CELLSTART) : nullptr;
  b.cell_atoms = ncells ? bp_<int>(h, mld_gpu_handle::B_CELLATOMS) : nullptr;
  b.atom_start = bp_<int>(h, mld_gpu_handle::B_ATOM_START);
  b.atom_struct = bp_<int>(h, mld_gpu_handle::B_ATOM_STRUCT);
  b.types = bp_<int>(h, mld_gpu_handle::B_TYPES);
  b.pos = bp_<double>(h, mld_gpu_handle::B_POS);
  b.cell = bp_<double>(h, mld_gpu_handle::B_CELL);
  b.recip = bp_<double>(h, mld_gpu_handle::B_RECIP);
  b.small = bp_<int>(h, mld_gpu_handle::B_SMALL);
  b.nsize = bp_<int>(h, mld_gpu_handle::B_NSIZE);
  b.volume = bp_<double>(h, mld_gpu_handle::B_VOL);
  // the host arrays of this call are read by the stream above: wait before returning
  e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return cuda_fail(h, e, "mld_gpu_set_structures");
  h->has_batch = true;
  h->nbr_valid = false;
  h->has_labels = false;
  return MLD_OK;
}

int mld_gpu_set_labels(mld_gpu_handle* h, const double* energy, const double* force, const double* stress,
                       const int* has_efs, const double* w_efs) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->has_batch) return fail(h, MLD_ERR_STATE, "no structures staged");
  if (!has_efs || !w_efs) return fail(h, MLD_ERR_INVALID, "has_efs and w_efs are required");
  const int S = h->S, A = h->A;
  h->h_has.assign(has_efs, has_efs + 3 * (size_t)S);
  bool anyE = false, anyF = false, anyS = false;
  for (int s = 0; s < S; ++s) {
    anyE |= has_efs[3 * s] != 0;
    anyF |= has_efs[3 * s + 1] != 0;
    anyS |= has_efs[3 * s + 2] != 0;
  }
  if ((anyE && !energy) || (anyF && h->cfg.desc_forces && !force) || (anyS && h->cfg.desc_forces && !stress))
    return fail(h, MLD_ERR_INVALID, "missing label array for a flagged block");
  std::vector<double> zE, zF, zS;
  if (!energy) zE.assign(std::max(S, 1), 0.0), energy = zE.data();
  if (!force) zF.assign(3 * (size_t)std::max(A, 1), 0.0), force = zF.data();
  if (!stress) zS.assign(6 * (size_t)std::max(S, 1), 0.0), stress = zS.data();
  cudaError_t e = upload(h, mld_gpu_handle::B_E, energy, (size_t)S);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_F, force, 3 * (size_t)A);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_S, stress, 6 * (size_t)S);
  if (e == cudaSuccess) e = upload(h, mld_gpu_handle::B_WEFS, w_efs, 3 * (size_t)S);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return cuda_fail(h, e, "mld_gpu_set_labels");
  h->fit_rows = make_layout(h, h->h_has, false);
  h->has_labels = true;
  return MLD_OK;
}

int mld_gpu_descriptors(mld_gpu_handle* h, double* B_out, int* n_neigh_out) {
  if (!h) return MLD_ERR_INVALID;
  int rc = build_neighbours(h);
  if (rc) return rc;
  const size_t nB = (size_t)h->A * h->KK;
  if (h->mixed) {
    CK(ensure(h, mld_gpu_handle::B_BOUT, sizeof(float) * std::max<size_t>(nB, 1)));
    rc = run_descriptors<float>(h, true, nullptr, bp_<float>(h, mld_gpu_handle::B_BOUT));
    if (rc) return rc;
    if (B_out) {
      std::vector<float> tmp(nB);
      CK(cudaMemcpyAsync(tmp.data(), bp_<float>(h, mld_gpu_handle::B_BOUT), sizeof(float) * nB,
                         cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      for (size_t i = 0; i < nB; ++i) B_out[i] = tmp[i];
    }
  } else {
    CK(ensure(h, mld_gpu_handle::B_BOUT, sizeof(double) * std::max<size_t>(nB, 1)));
    rc = run_descriptors<double>(h, true, nullptr, bp_<double>(h, mld_gpu_handle::B_BOUT));
    if (rc) return rc;
    if (B_out)
      CK(cudaMemcpyAsync(B_out, bp_<double>(h, mld_gpu_handle::B_BOUT), sizeof(double) * nB, cudaMemcpyDeviceToHost,
                         h->st));
  }
  if (n_neigh_out)
    CK(cudaMemcpyAsync(n_neigh_out, h->b.nn, sizeof(int) * h->A, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return MLD_OK;
}

int mld_gpu_descriptor_derivatives(mld_gpu_handle* h, long long* P_inout, int* nbr_out, double* u_out,
                                   double* dB_out) {
  if (!h || !P_inout) return MLD_ERR_INVALID;
  if (!h->nbr_valid) return fail(h, MLD_ERR_STATE, "call mld_gpu_descriptors first");
  const long long P = h->b.P;
  if (*P_inout < P) {
    *P_inout = P;
    return fail(h, MLD_ERR_INVALID, "pair capacity too small");
  }
  *P_inout = P;
  if (nbr_out) CK(cudaMemcpyAsync(nbr_out, h->b.nbr_idx, sizeof(int) * P, cudaMemcpyDeviceToHost, h->st));
  if (u_out) CK(cudaMemcpyAsync(u_out, h->b.nbr_u, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, h->st));
  const size_t nd = (size_t)P * 3 * h->KK;
  if (dB_out) {
    if (h->mixed) {
      std::vector<float> tmp(nd);
      CK(cudaMemcpyAsync(tmp.data(), bp_<float>(h, mld_gpu_handle::B_DBOUT), sizeof(float) * nd,
                         cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      for (size_t i = 0; i < nd; ++i) dB_out[i] = tmp[i];
    } else {
      CK(cudaMemcpyAsync(dB_out, bp_<double>(h, mld_gpu_handle::B_DBOUT), sizeof(double) * nd,
                         cudaMemcpyDeviceToHost, h->st));
    }
  }
  CK(cudaStreamSynchronize(h->st));
  return MLD_OK;
}

int mld_gpu_num_rows(mld_gpu_handle* h, long long* M) {
  if (!h || !M) return MLD_ERR_INVALID;
  if (!h->has_labels) return fail(h, MLD_ERR_STATE, "labels not set");
  *M = h->fit_rows.M;
  return MLD_OK;
}

int mld_gpu_design_matrix(mld_gpu_handle* h, double* A, double* y, double* w) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->has_labels) return fail(h, MLD_ERR_STATE, "labels not set");
  int rc = build_neighbours(h);
  if (rc) return rc;
  const long long M = h->fit_rows.M;
  if (h->mixed) {
    float* X = nullptr;
    rc = run_rows<float>(h, h->fit_rows, true, &X);
    if (rc) return rc;
    if (A) {
      std::vector<float> tmp((size_t)M * h->ldx);
      CK(cudaMemcpyAsync(tmp.data(), X, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      std::vector<double> row(h->D);
      for (long long r = 0; r < M; ++r) {
        for (int c = 0; c < h->D; ++c) row[c] = tmp[(size_t)r * h->ldx + c];
        export_row(h, row.data(), A + (size_t)r * h->Dfull);
      }
    }
  } else {
    double* X = nullptr;
    rc = run_rows<double>(h, h->fit_rows, true, &X);
    if (rc) return rc;
    if (A && M > 0) {
      std::vector<double> tmp((size_t)M * h->ldx);
      CK(cudaMemcpyAsync(tmp.data(), X, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      for (long long r = 0; r < M; ++r) export_row(h, tmp.data() + (size_t)r * h->ldx, A + (size_t)r * h->Dfull);
    }
  }
  if (y) CK(cudaMemcpyAsync(y, bp_<double>(h, mld_gpu_handle::B_Y), sizeof(double) * M, cudaMemcpyDeviceToHost, h->st));
  if (w)
    CK(cudaMemcpyAsync(w, bp_<double>(h, mld_gpu_handle::B_WROW), sizeof(double) * M, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return MLD_OK;
}

int mld_gpu_gram(mld_gpu_handle* h, double* G, double* rhs) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->has_labels) return fail(h, MLD_ERR_STATE, "labels not set");
  int rc = build_neighbours(h);
  if (rc) return rc;
  const int D = h->D;
  const long long M = h->fit_rows.M;
  CK(ensure(h, mld_gpu_handle::B_G, sizeof(double) * D * D));
  CK(ensure(h, mld_gpu_handle::B_H, sizeof(double) * D));
  if (h->mixed) {
    // tensor-core BF16 split-precision Gram (the mixed method's normal matrix)
    float* X = nullptr;
    rc = run_rows<float>(h, h->fit_rows, true, &X);
    if (rc) return rc;
    double* dG = bp_<double>(h, mld_gpu_handle::B_G);
    const size_t need = (size_t)4 * D * (size_t)((std::max<long long>(M, 1) + 63) / 64 * 64) + 256;
    const size_t wsb = std::max(gram_tc_min_workspace(D), std::min(need, kGramWorkspaceCap));
    CK(ensure(h, mld_gpu_handle::B_GWS, wsb));
    CK(ensure(h, mld_gpu_handle::B_TERR, sizeof(int)));
    int* terr = bp_<int>(h, mld_gpu_handle::B_TERR);
    CK(cudaMemsetAsync(dG, 0, sizeof(double) * (size_t)D * D, h->st));
    CK(cudaMemsetAsync(terr, 0, sizeof(int), h->st));
    if (!gram_tc_available()) return fail(h, MLD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const size_t npart = gram_tc_part_doubles(D, h->nsm);
    CK(ensure(h, mld_gpu_handle::B_GTCP, sizeof(double) * std::max<size_t>(npart, 1)));
    CK(launch_gram_tc<float>(X, h->ldx, 0, D, bp_<double>(h, mld_gpu_handle::B_WROW), M, dG,
                             bp_<void>(h, mld_gpu_handle::B_GWS), wsb, terr, h->nsm, h->st,
                             bp_<double>(h, mld_gpu_handle::B_GTCP), npart));
    CK(launch_symmetrize(dG, D, h->st));
    CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * (size_t)std::max<long long>(M, 1)));
    double* rws = gram_ws(h, M, D);
    if (!rws) return fail(h, MLD_ERR_OOM, "rhs workspace");
    CK(launch_rhs<float>(X, h->ldx, bp_<double>(h, mld_gpu_handle::B_WROW), bp_<double>(h, mld_gpu_handle::B_Y), M, D,
                         bp_<double>(h, mld_gpu_handle::B_H), h->nsm, h->st, bp_<float2>(h, mld_gpu_handle::B_PRED),
                         rws));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, terr, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (herr) return fail(h, MLD_ERR_TIMEOUT, "tensor-core Gram: a pipeline wait timed out");
  } else {
    double* X = nullptr;
    rc = run_rows<double>(h, h->fit_rows, true, &X);
    if (rc) return rc;
    double* gws = gram_ws(h, M, D);
    if (!gws) return fail(h, MLD_ERR_OOM, "Gram workspace");
    CK(launch_gram<double>(X, h->ldx, bp_<double>(h, mld_gpu_handle::B_WROW), bp_<double>(h, mld_gpu_handle::B_Y), M, D,
                           bp_<double>(h, mld_gpu_handle::B_G), bp_<double>(h, mld_gpu_handle::B_H), h->st, gws));
  }
  if (G) CK(cudaMemcpyAsync(G, bp_<double>(h, mld_gpu_handle::B_G), sizeof(double) * D * D, cudaMemcpyDeviceToHost, h->st));
  if (rhs) CK(cudaMemcpyAsync(rhs, bp_<double>(h, mld_gpu_handle::B_H), sizeof(double) * D, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return MLD_OK;
}

int mld_gpu_solve(mld_gpu_handle* h, const double* G, const double* rhs, int D, double* w, int* rank_out) {
  if (!h || !G || !rhs || !w || D < 1) return MLD_ERR_INVALID;
  CK(ensure(h, mld_gpu_handle::B_G, sizeof(double) * (size_t)D * D));
  CK(ensure(h, mld_gpu_handle::B_H, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_W, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_EVALS, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_INFO, sizeof(int) * 4));
  double* dG = bp_<double>(h, mld_gpu_handle::B_G);
  double* dh = bp_<double>(h, mld_gpu_handle::B_H);
  double* dw = bp_<double>(h, mld_gpu_handle::B_W);
  CK(cudaMemcpyAsync(dG, G, sizeof(double) * (size_t)D * D, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(dh, rhs, sizeof(double) * D, cudaMemcpyHostToDevice, h->st));
  int rc = solve_any(h, dG, dh, D, dw);
  if (rc) return rc;
  CK(cudaMemcpyAsync(w, dw, sizeof(double) * D, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (rank_out) *rank_out = h->last_rank;
  return MLD_OK;
}

int mld_gpu_fit(mld_gpu_handle* h, double* w_params, double* rmse_efs) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->has_labels) return fail(h, MLD_ERR_STATE, "labels not set");
  return h->mixed ? fit_impl<float>(h, w_params, rmse_efs) : fit_impl<double>(h, w_params, rmse_efs);
}

int mld_gpu_evaluate(mld_gpu_handle* h, const double* w_params, double* E, double* F, double* Sout) {
  if (!h || !w_params) return MLD_ERR_INVALID;
  int rc = mld::eval_weights_upload(h, w_params);
  if (rc) return rc;
  rc = mld::eval_launch(h, nullptr, nullptr);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->st));
  const double* out = bp_<double>(h, mld_gpu_handle::B_EOUT);
  std::vector<double> ho((size_t)h->S + 3 * (size_t)h->A + 6 * (size_t)h->S);
  CK(cudaMemcpy(ho.data(), out, sizeof(double) * ho.size(), cudaMemcpyDeviceToHost));
  if (E) std::copy(ho.begin(), ho.begin() + h->S, E);
  if (F) std::copy(ho.begin() + h->S, ho.begin() + h->S + 3 * (size_t)h->A, F);
  if (Sout) std::copy(ho.begin() + h->S + 3 * (size_t)h->A, ho.end(), Sout);
  return MLD_OK;
}

int mld_gpu_predict(mld_gpu_handle* h, const double* w_params, double* E, double* F, double* Sout) {
  if (!h || !w_params) return MLD_ERR_INVALID;
  int rc = build_neighbours(h);
  if (rc) return rc;
  std::vector<int> all(3 * (size_t)h->S, 1);
  RowLayout L = make_layout(h, all, true);
  const int D = h->D;
  CK(ensure(h, mld_gpu_handle::B_W, sizeof(double) * D));
  CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * std::max<long long>(L.M, 1)));
  double* dw = bp_<double>(h, mld_gpu_handle::B_W);
  double* pred = bp_<double>(h, mld_gpu_handle::B_PRED);
  std::vector<double> wd(D);
  if (h->quad) full_to_dedup(h, w_params, wd.data());
  else std::copy(w_params, w_params + D, wd.begin());
  CK(cudaMemcpyAsync(dw, wd.data(), sizeof(double) * D, cudaMemcpyHostToDevice, h->st));
  if (h->mixed) {
    float* X = nullptr;
    rc = run_rows<float>(h, L, false, &X);
    if (rc) return rc;
    CK(launch_predict_sq<float>(X, h->ldx, dw, L.M, D, pred, nullptr, nullptr, nullptr, h->st));
  } else {
    double* X = nullptr;
    rc = run_rows<double>(h, L, false, &X);
    if (rc) return rc;
    CK(launch_predict_sq<double>(X, h->ldx, dw, L.M, D, pred, nullptr, nullptr, nullptr, h->st));
  }
  std::vector<double> hp(L.M);
  CK(cudaMemcpyAsync(hp.data(), pred, sizeof(double) * L.M, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int s = 0; s < h->S; ++s) {
    int a0 = h->h_atom_start[s], nat = h->h_atom_start[s + 1] - a0;
    if (E) E[s] = hp[L.rowE[s]];
    if (F && L.rowF[s] >= 0)
      for (int i = 0; i < 3 * nat; ++i) F[3 * (size_t)a0 + i] = hp[L.rowF[s] + i];
    if (Sout && L.rowS[s] >= 0)
      for (int k = 0; k < 6; ++k) Sout[6 * s + k] = hp[L.rowS[s] + k];
  }
  return MLD_OK;
}

}  // extern "C"

namespace mld {

// Asynchronous halves of mld_gpu_predict for the serving loop: predict_launch stages nothing on
// the host side but the neighbour counts (one stream synchronisation), queues the descriptor,
// design-row and prediction kernels and the copy of the predictions into a pinned host buffer
// on the handle's stream, and records `done`; predict_collect scatters the predictions of
// structure s into its energy / forces / stress once `done` has completed.
int predict_launch(mld_gpu_handle* h, const double* w_dev, cudaEvent_t done, double** pinned_out) {
  int rc = build_neighbours(h);
  if (rc) return rc;
  std::vector<int> all(3 * (size_t)h->S, 1);
  h->serve_rows = make_layout(h, all, true);
  const RowLayout& L = h->serve_rows;
  CK(ensure(h, mld_gpu_handle::B_PRED, sizeof(double) * std::max<long long>(L.M, 1)));
  double* pred = bp_<double>(h, mld_gpu_handle::B_PRED);
  if (h->mixed) {
    float* X = nullptr;
    rc = run_rows<float>(h, L, false, &X);
    if (rc) return rc;
    CK(launch_predict_sq<float>(X, h->ldx, w_dev, L.M, h->D, pred, nullptr, nullptr, nullptr, h->st));
  } else {
    double* X = nullptr;
    rc = run_rows<double>(h, L, false, &X);
    if (rc) return rc;
    CK(launch_predict_sq<double>(X, h->ldx, w_dev, L.M, h->D, pred, nullptr, nullptr, nullptr, h->st));
  }
  if ((size_t)L.M > h->pinned_cap) {
    if (h->pinned) cudaFreeHost(h->pinned);
    h->pinned = nullptr;
    h->pinned_cap = 0;
    CK(cudaMallocHost(&h->pinned, sizeof(double) * (size_t)std::max<long long>(L.M, 1)));
    h->pinned_cap = (size_t)std::max<long long>(L.M, 1);
  }
  CK(cudaMemcpyAsync(h->pinned, pred, sizeof(double) * L.M, cudaMemcpyDeviceToHost, h->st));
  CK(cudaEventRecord(done, h->st));
  *pinned_out = h->pinned;
  return MLD_OK;
}

void predict_collect(const mld_gpu_handle* h, int s, double* E, double* F, double* Sout) {
  const RowLayout& L = h->serve_rows;
  const double* hp = h->pinned;
  const int a0 = h->h_atom_start[s], nat = h->h_atom_start[s + 1] - a0;
  (void)a0;
  if (E) *E = hp[L.rowE[s]];
  if (F && L.rowF[s] >= 0)
    for (int i = 0; i < 3 * nat; ++i) F[i] = hp[L.rowF[s] + i];
  if (Sout && L.rowS[s] >= 0)
    for (int k = 0; k < 6; ++k) Sout[k] = hp[L.rowS[s] + k];
}

// device copy of fitted weights (reference full layout) in the handle's working layout
int upload_weights(mld_gpu_handle* h, const double* w_full, double** w_dev) {
  std::vector<double> wd(h->D);
  if (h->quad) full_to_dedup(h, w_full, wd.data());
  else std::copy(w_full, w_full + h->D, wd.begin());
  CK(ensure(h, mld_gpu_handle::B_WSERVE, sizeof(double) * h->D));
  CK(cudaMemcpyAsync(bp_<double>(h, mld_gpu_handle::B_WSERVE), wd.data(), sizeof(double) * h->D,
                     cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  *w_dev = bp_<double>(h, mld_gpu_handle::B_WSERVE);
  return MLD_OK;
}

// ---- evaluation with fitted weights, without design rows (bispectrum.cu eval mode, eval.cu) ----
// Weights of the reference's full layout [w0, w_lin (KK), W (KK x KK, quadratic)] are kept on
// the device as w_lin (FP64), w_lin in the descriptor precision, and Wsym = W + W^T (FP64).
int eval_weights_upload(mld_gpu_handle* h, const double* w_full) {
  if (h->krr) return fail(h, MLD_ERR_UNSUPPORTED, "evaluation without design rows covers ml_type 0 only");
  const int KK = h->KK;
  const size_t n2 = h->quad ? (size_t)KK * KK : 0;
  std::vector<double> hw((size_t)KK + n2);
  std::copy(w_full + 1, w_full + 1 + KK, hw.begin());
  if (h->quad) {
    const double* W = w_full + 1 + KK;
    for (int i = 0; i < KK; ++i)
      for (int j = 0; j < KK; ++j) hw[KK + (size_t)i * KK + j] = W[(size_t)i * KK + j] + W[(size_t)j * KK + i];
  }
  const size_t eb = h->mixed ? sizeof(float) : sizeof(double);
  CK(ensure(h, mld_gpu_handle::B_EW, sizeof(double) * hw.size() + eb * KK + 256));
  double* dw = bp_<double>(h, mld_gpu_handle::B_EW);
  CK(cudaMemcpyAsync(dw, hw.data(), sizeof(double) * hw.size(), cudaMemcpyHostToDevice, h->st));
  void* wt = dw + hw.size();
  if (h->mixed) {
    std::vector<float> f(w_full + 1, w_full + 1 + KK);
    CK(cudaMemcpyAsync(wt, f.data(), sizeof(float) * KK, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  } else {
    CK(cudaMemcpyAsync(wt, w_full + 1, sizeof(double) * KK, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  h->ew0 = w_full[0];
  h->ew_ready = true;
  return MLD_OK;
}

template <typename T>
static int eval_run(mld_gpu_handle* h, double* out) {
  const int KK = h->KK;
  double* E = out;
  double* F = out + h->S;
  double* S = F + 3 * (size_t)h->A;
  const double* wlin = bp_<double>(h, mld_gpu_handle::B_EW);
  const double* wsym = wlin + KK;
  const T* wlinT = reinterpret_cast<const T*>(wlin + KK + (h->quad ? (size_t)KK * KK : 0));
  CK(ensure(h, mld_gpu_handle::B_EPAIR, sizeof(double) * 9 * (size_t)std::max<long long>(1, h->b.P)));
  CK(ensure(h, mld_gpu_handle::B_EATOM, sizeof(double) * (size_t)std::max(1, h->A)));
  CK(ensure(h, mld_gpu_handle::B_REV, sizeof(int) * (size_t)std::max<long long>(1, h->b.P)));
  double* Eatom = bp_<double>(h, mld_gpu_handle::B_EATOM);
  DevEval<T> ev;
  ev.pair = bp_<double>(h, mld_gpu_handle::B_EPAIR);
  ev.w0 = h->ew0;
  if (h->quad) {
    // pass 1: B of every atom; beta_a and the atom energies; pass 2: per-pair forces and stress
    CK(ensure(h, mld_gpu_handle::B_EB, sizeof(T) * std::max<size_t>(1, (size_t)h->A * KK)));
    CK(ensure(h, mld_gpu_handle::B_EBETA, sizeof(T) * std::max<size_t>(1, (size_t)h->A * KK)));
    T* B = bp_<T>(h, mld_gpu_handle::B_EB);
    T* beta = bp_<T>(h, mld_gpu_handle::B_EBETA);
    int rc = run_descriptors<T>(h, false, nullptr, B);
    if (rc) return rc;
    CK(launch_eval_beta<T>(B, h->A, KK, wlin, wsym, h->ew0, beta, Eatom, h->st));
    ev.beta = beta;
    ev.beta_per_atom = 1;
    rc = run_descriptors<T>(h, false, &ev, (T*)nullptr);
    if (rc) return rc;
    nl(h, 1);
  } else {
    ev.beta = wlinT;
    ev.beta_per_atom = 0;
    ev.wlin = wlin;
    ev.Eatom = Eatom;
    int rc = run_descriptors<T>(h, false, &ev, (T*)nullptr);
    if (rc) return rc;
  }
  CK(launch_reverse_pairs(h->b, bp_<int>(h, mld_gpu_handle::B_REV), h->st));
  CK(launch_eval_gather(h->b, h->bp, bp_<int>(h, mld_gpu_handle::B_REV), ev.pair, Eatom, E, F, S, h->st));
  nl(h, 3);
  return MLD_OK;
}

// Queue the evaluation of the staged batch on the handle's stream: outputs [E (S) | F (3A) |
// S (6S)] in FP64 in B_EOUT and, when `pinned_out` is given, copied into a pinned host buffer;
// `done` (optional) is recorded after the copy.
int eval_launch(mld_gpu_handle* h, cudaEvent_t done, double** pinned_out) {
  if (!h->ew_ready) return fail(h, MLD_ERR_STATE, "evaluation weights not uploaded");
  int rc = build_neighbours(h);
  if (rc) return rc;
  const size_t nout = (size_t)h->S + 3 * (size_t)h->A + 6 * (size_t)h->S;
  CK(ensure(h, mld_gpu_handle::B_EOUT, sizeof(double) * std::max<size_t>(nout, 1)));
  double* out = bp_<double>(h, mld_gpu_handle::B_EOUT);
  CK(cudaMemsetAsync(out, 0, sizeof(double) * nout, h->st));
  rc = h->mixed ? eval_run<float>(h, out) : eval_run<double>(h, out);
  if (rc) return rc;
  if (pinned_out) {
    if (nout > h->pinned_cap) {
      if (h->pinned) cudaFreeHost(h->pinned);
      h->pinned = nullptr;
      h->pinned_cap = 0;
      CK(cudaMallocHost(&h->pinned, sizeof(double) * std::max<size_t>(nout, 1)));
      h->pinned_cap = std::max<size_t>(nout, 1);
    }
    CK(cudaMemcpyAsync(h->pinned, out, sizeof(double) * nout, cudaMemcpyDeviceToHost, h->st));
    *pinned_out = h->pinned;
  }
  if (done) CK(cudaEventRecord(done, h->st));
  return MLD_OK;
}

void eval_collect(const mld_gpu_handle* h, int s, double* E, double* F, double* Sout) {
  const double* hp = h->pinned;
  const int a0 = h->h_atom_start[s], nat = h->h_atom_start[s + 1] - a0;
  if (E) *E = hp[s];
  if (F)
    for (int i = 0; i < 3 * nat; ++i) F[i] = hp[h->S + 3 * (size_t)a0 + i];
  if (Sout)
    for (int k = 0; k < 6; ++k) Sout[k] = hp[h->S + 3 * (size_t)h->A + 6 * (size_t)s + k];
}

cudaStream_t handle_stream(const mld_gpu_handle* h) { return h->st; }
int handle_dims(const mld_gpu_handle* h, int* D, int* ldx, int* KK, int* nch) {
  *D = h->D;
  *ldx = h->ldx;
  *KK = h->KK;
  *nch = h->nch;
  return MLD_OK;
}

// Free every per-batch device buffer of an idle handle (the evaluation weights stay); the next
// batch allocates what it needs again.
void handle_release_buffers(mld_gpu_handle* h) {
  cudaStreamSynchronize(h->st);
  ++h->buf_gen;
  for (int id = 0; id < mld_gpu_handle::B_COUNT; ++id) {
    if (id == mld_gpu_handle::B_EW) continue;
    Buf& bf = h->bufs[id];
    if (bf.p) cudaFree(bf.p);
    bf.p = nullptr;
    bf.cap = 0;
  }
  h->has_batch = false;
  h->nbr_valid = false;
}

}  // namespace mld

extern "C" {

int mld_gpu_set_profiling(mld_gpu_handle* h, int on) {
  if (!h) return MLD_ERR_INVALID;
  h->prof = on != 0;
  h->pending.clear();
  h->cur_phase = h->cur_ev = -1;
  return MLD_OK;
}

int mld_gpu_profile(mld_gpu_handle* h, double* ms, long long* launches, long long* calls, int reset) {
  if (!h) return MLD_ERR_INVALID;
  for (int p = 0; p < MLD_NPHASE; ++p) {
    if (ms) ms[p] = h->ms[p];
    if (launches) launches[p] = h->launches[p];
    if (calls) calls[p] = h->calls[p];
    if (reset) {
      h->ms[p] = 0;
      h->launches[p] = 0;
      h->calls[p] = 0;
    }
  }
  return MLD_OK;
}

int mld_gpu_timer_start(mld_gpu_handle* h) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->tev[0]) {
    CK(cudaEventCreate(&h->tev[0]));
    CK(cudaEventCreate(&h->tev[1]));
  }
  CK(cudaEventRecord(h->tev[0], h->st));
  return MLD_OK;
}

int mld_gpu_timer_stop(mld_gpu_handle* h, double* ms) {
  if (!h || !ms || !h->tev[0]) return MLD_ERR_INVALID;
  CK(cudaEventRecord(h->tev[1], h->st));
  CK(cudaEventSynchronize(h->tev[1]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->tev[0], h->tev[1]));
  *ms = t;
  return MLD_OK;
}

int mld_gpu_work_counts(const mld_gpu_handle* h, long long* out) {
  if (!h || !out) return MLD_ERR_INVALID;
  const Bso4Tables& t = h->tab;
  long long na_sum = 0, is_a = 0;
  for (const auto& z : t.zterms) na_sum += z.na;
  for (const auto& s : t.yslots) is_a += s.is_a;
  out[0] = t.HU;
  out[1] = t.u_one;
  out[2] = t.u_two;
  out[3] = t.cg_terms;
  out[4] = na_sum;
  out[5] = (long long)t.zterms.size();
  out[6] = (long long)t.yslots.size();
  out[7] = is_a;
  out[8] = t.K;
  out[9] = h->nch;
  out[10] = h->b.P;
  out[11] = h->A;
  return MLD_OK;
}

int mld_gpu_synchronize(mld_gpu_handle* h) {
  if (!h) return MLD_ERR_INVALID;
  cudaError_t e = cudaStreamSynchronize(h->st);
  return e == cudaSuccess ? MLD_OK : cuda_fail(h, e, "cudaStreamSynchronize");
}

}  // extern "C"

namespace mld {
template <typename T>
cudaError_t measure_fma_peak(cudaStream_t st, double* tflops);
}

extern "C" int mld_gpu_peak_flops(mld_gpu_handle* h, int precision, double* tflops) {
  if (!h || !tflops) return MLD_ERR_INVALID;
  cudaError_t e = precision == MLD_PRECISION_MIXED ? mld::measure_fma_peak<float>(h->st, tflops)
                                                   : mld::measure_fma_peak<double>(h->st, tflops);
  return e == cudaSuccess ? MLD_OK : cuda_fail(h, e, "mld_gpu_peak_flops");
}

extern "C" int mld_gpu_set_kernel_points(mld_gpu_handle* h, int nk, const double* z_raw) {
  if (!h) return MLD_ERR_INVALID;
  if (!h->krr) return fail(h, MLD_ERR_STATE, "reference points need ml_type = 1");
  if (nk < 1 || !z_raw) return fail(h, MLD_ERR_INVALID, "need at least one reference point");
  const int KK = h->KK;
  // standardisation over the reference set (compute_kernel.F90:1058-1256, init_kernel)
  std::vector<double> mean(KK, 0.0), sd(KK, 0.0), zd((size_t)nk * KK);
  for (int k = 0; k < nk; ++k)
    for (int c = 0; c < KK; ++c) mean[c] += z_raw[(size_t)k * KK + c];
  for (int c = 0; c < KK; ++c) mean[c] /= nk;
  for (int k = 0; k < nk; ++k)
    for (int c = 0; c < KK; ++c) {
      const double d = z_raw[(size_t)k * KK + c] - mean[c];
      sd[c] += d * d;
    }
  for (int c = 0; c < KK; ++c) {
    sd[c] = std::sqrt(sd[c] / nk);
    if (!(sd[c] > 0.0))
      return fail(h, MLD_ERR_INVALID, "kernel reference points: descriptor component " + std::to_string(c) +
                                          " has zero spread over the set");
  }
  for (int k = 0; k < nk; ++k)
    for (int c = 0; c < KK; ++c) zd[(size_t)k * KK + c] = (z_raw[(size_t)k * KK + c] - mean[c]) / sd[c];
  std::vector<float> zf(zd.begin(), zd.end());
  CK(upload(h, mld_gpu_handle::B_KZD, zd.data(), zd.size()));
  CK(upload(h, mld_gpu_handle::B_KZF, zf.data(), zf.size()));
  CK(cudaStreamSynchronize(h->st));
  h->nk = nk;
  h->D = h->DL + nk;
  h->Dfull = h->D;
  h->ldx = round_up4(h->D);
  return MLD_OK;
}

extern "C" int mld_gpu_tuning(const mld_gpu_handle* h, int mode, int* shape, int* ncand, double* ms) {
  if (!h || mode < 0 || mode > 2 || !shape || !ncand) return MLD_ERR_INVALID;
  const auto& tn = h->tune[mode];
  shape[0] = tn.best.col_tile;
  shape[1] = tn.best.ctas_per_sm;
  shape[2] = tn.best.sorted_queue;
  shape[3] = tn.done ? 1 : 0;
  const int n = std::min<int>(*ncand, (int)tn.ms.size());
  for (int i = 0; i < n; ++i) {
    if (ms) ms[i] = tn.ms[i];
  }
  *ncand = (int)tn.ms.size();
  return MLD_OK;
}

extern "C" int mld_gpu_test_pipeline_timeout(int skip_loads, long long wait_limit_clocks) {
  if (skip_loads < 0 || wait_limit_clocks < 0) return MLD_ERR_INVALID;
  mld::gram_tc_test_timeout(skip_loads, wait_limit_clocks);
  return MLD_OK;
}

extern "C" int mld_gpu_solve_info(const mld_gpu_handle* h, int* pcg_iterations, double* pcg_residual,
                                  double* precond_shift, int* chol_retries) {
  if (!h) return MLD_ERR_INVALID;
  for (int s = 0; s < 2; ++s) {
    if (pcg_iterations) pcg_iterations[s] = h->pcg_iters[s];
    if (pcg_residual) pcg_residual[s] = h->pcg_rel[s];
    if (precond_shift) precond_shift[s] = h->precond_shift[s];
  }
  if (chol_retries) *chol_retries = h->chol_retries;
  return MLD_OK;
}

namespace {
int set_err(char* err, int err_len, int code, const std::string& msg) {
  if (err && err_len > 0) {
    std::strncpy(err, msg.c_str(), (size_t)err_len - 1);
    err[err_len - 1] = 0;
  }
  return code;
}
}  // namespace

extern "C" int mld_gpu_gram_rows(int method, const void* X, int x_is_fp32, long long M, int D, int ldx,
                                 const double* w, const double* y, double* G, double* rhs, void* stream, char* err,
                                 int err_len) {
  if (!X || !w || !G || D < 1 || M < 0 || ldx < D || (rhs && !y))
    return set_err(err, err_len, MLD_ERR_INVALID, "invalid argument");
  if (method != MLD_PRECISION_PLAIN_FP64 && method != MLD_PRECISION_MIXED)
    return set_err(err, err_len, MLD_ERR_INVALID, "method must be MLD_PRECISION_PLAIN_FP64 or MLD_PRECISION_MIXED");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  void* ws = nullptr;
  double* hbuf = nullptr;
  int* terr = nullptr;
  double* part = nullptr;  // tensor-core split partials and right-hand-side partials
  auto cleanup = [&]() {
    if (ws) cudaFree(ws);
    if (hbuf) cudaFree(hbuf);
    if (terr) cudaFree(terr);
    if (part) cudaFree(part);
  };
  auto cuda_err = [&](cudaError_t ce, const char* where) {
    cleanup();
    return set_err(err, err_len, ce == cudaErrorMemoryAllocation ? MLD_ERR_OOM : MLD_ERR_CUDA,
                   std::string(where) + ": " + cudaGetErrorString(ce));
  };
  if (e != cudaSuccess) return cuda_err(e, "device query");
  if (method == MLD_PRECISION_PLAIN_FP64) {
    double* hv = rhs;
    const double* yy = y;
    if (!hv) {
      e = cudaMalloc(&hbuf, sizeof(double) * (size_t)D + sizeof(double) * (size_t)std::max<long long>(M, 1));
      if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
      hv = hbuf;
      double* yz = hbuf + D;
      e = cudaMemsetAsync(yz, 0, sizeof(double) * (size_t)std::max<long long>(M, 1), st);
      if (e != cudaSuccess) return cuda_err(e, "cudaMemsetAsync");
      yy = yz;
    }
    e = cudaMalloc(&ws, sizeof(double) * gram_workspace_doubles(M, D));
    if (e != cudaSuccess) return cuda_err(e, "workspace");
    double* gws = static_cast<double*>(ws);
    e = x_is_fp32 ? launch_gram<float>(static_cast<const float*>(X), ldx, w, yy, M, D, G, hv, st, gws)
                  : launch_gram<double>(static_cast<const double*>(X), ldx, w, yy, M, D, G, hv, st, gws);
    if (e != cudaSuccess) return cuda_err(e, "launch_gram");
  } else {
    if (!gram_tc_available())
      return set_err(err, err_len, MLD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const size_t need = (size_t)4 * D * (size_t)((std::max<long long>(M, 1) + 63) / 64 * 64) + 256;
    const size_t wsb = std::max(gram_tc_min_workspace(D), std::min(need, kGramWorkspaceCap));
    const size_t npart = gram_tc_part_doubles(D, nsm);
    const size_t nrhs = rhs ? gram_workspace_doubles(M, D) : 0;
    e = cudaMalloc(&ws, wsb);
    if (e == cudaSuccess) e = cudaMalloc(&part, sizeof(double) * std::max<size_t>(std::max(npart, nrhs), 1));
    if (e == cudaSuccess) e = cudaMalloc(&terr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(terr, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(G, 0, sizeof(double) * (size_t)D * D, st);
    if (e != cudaSuccess) return cuda_err(e, "workspace");
    e = x_is_fp32 ? launch_gram_tc<float>(static_cast<const float*>(X), ldx, 0, D, w, M, G, ws, wsb, terr, nsm, st,
                                          part, npart)
                  : launch_gram_tc<double>(static_cast<const double*>(X), ldx, 0, D, w, M, G, ws, wsb, terr, nsm, st,
                                           part, npart);
    if (e == cudaSuccess) e = launch_symmetrize(G, D, st);
    float2* sv = nullptr;
    // the right-hand side reuses the partial buffer after the Gram (same stream)
    if (e == cudaSuccess && rhs && x_is_fp32) {
      e = cudaMalloc(&sv, sizeof(float2) * (size_t)std::max<long long>(M, 1));
      if (e == cudaSuccess)
        e = launch_rhs<float>(static_cast<const float*>(X), ldx, w, y, M, D, rhs, nsm, st, sv, part);
    } else if (e == cudaSuccess && rhs) {
      e = launch_rhs<double>(static_cast<const double*>(X), ldx, w, y, M, D, rhs, nsm, st, nullptr, part);
    }
    if (sv) {
      cudaStreamSynchronize(st);
      cudaFree(sv);
    }
    if (e != cudaSuccess) return cuda_err(e, "launch_gram_tc");
    int herr = 0;
    e = cudaMemcpyAsync(&herr, terr, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_err(e, "synchronize");
    if (herr) {
      cleanup();
      return set_err(err, err_len, MLD_ERR_TIMEOUT, "tensor-core Gram: a pipeline wait timed out");
    }
  }
  e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return set_err(err, err_len, MLD_ERR_CUDA, cudaGetErrorString(e));
  return set_err(err, err_len, MLD_OK, "");
}
