// mld_gpu_descriptors_noalloc: bispectrum descriptors of one structure without any device
// allocation.
//
// Why it exists: cudaMalloc and cudaFree synchronise the device and can stall unrelated work.
// Some callers therefore cannot use them on their hot path, or at all.  Examples are MD
// drivers and serving loops that evaluate one structure per step, hosts whose device memory is
// owned by another runtime's pool, and code that must not synchronise.  Such a caller passes
// device pointers it already holds.  All the scratch this path needs (contraction tables,
// neighbour list, scan workspace, FP32 staging) lives in the file-scope array below.  Every GPU
// that loads this library reserves the array until the process exits.
//
// The device address of the array is obtained once per device, with that device current, by
// cudaGetSymbolAddress in noalloc_setup(); host code never uses the symbol itself.  The first
// call on a device does this set-up and uploads the tables (cudaMemcpy into the array, no
// allocation).  Make that first call before any stream capture.
//
// All calls share the array and it keeps the last call's contents.  Counters that must start
// at zero are cleared on every call.  Calls that overlap on the GPU (concurrent streams or host
// threads on the same device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mld_gpu.h"
#include "mld_internal.h"

namespace mld {

namespace {

constexpr size_t kScratchBytes = (size_t)48 << 20;  // MLD_NOALLOC_SCRATCH_MIB
constexpr int kMaxDevices = 64;

// The scratch array (device memory reserved at module load; never passed by host name).
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceState {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_noalloc_scratch on this device
  double j_max = -1.0;
  DevTables dt;
  size_t table_bytes = 0;
};

std::mutex g_mu;
DeviceState g_dev[kMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

void set_err(char* err, int len, const std::string& msg) {
  if (err && len > 0) {
    std::strncpy(err, msg.c_str(), (size_t)len - 1);
    err[len - 1] = '\0';
  }
}

template <typename V>
cudaError_t put(unsigned char* base, size_t* off, const std::vector<V>& v, V** dst) {
  // synchronous copy into the static array; callers have waited for earlier calls' kernels
  *off = align256(*off);
  *dst = reinterpret_cast<V*>(base + *off);
  const size_t bytes = sizeof(V) * v.size();
  *off += bytes;
  if (*off > kScratchBytes) return cudaErrorMemoryAllocation;
  return bytes ? cudaMemcpy(*dst, v.data(), bytes, cudaMemcpyHostToDevice) : cudaSuccess;
}

// Once per device (and again when j_max changes): resolve the array's device address and
// upload the contraction tables into its first region.
int noalloc_setup(int dev, double j_max, DeviceState** out, std::string* msg) {
  DeviceState& S = g_dev[dev];
  if (!S.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *msg = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return MLD_ERR_CUDA;
    }
    S.base = static_cast<unsigned char*>(p);
    S.ready = true;
  }
  if (S.j_max != j_max) {
    Bso4Tables t;
    if (!build_bso4_tables(j_max, &t, msg)) return MLD_ERR_INVALID;
    if (S.j_max >= 0.0) {
      // A previous call's kernels may still read the old tables (and the per-call region behind
      // them) on whatever stream that call was given; the synchronous copies below run on the
      // legacy default stream, which does not wait for non-blocking streams.  Wait for the
      // whole device before overwriting.
      cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        *msg = std::string("cudaDeviceSynchronize before the table re-upload: ") + cudaGetErrorString(e);
        return MLD_ERR_CUDA;
      }
    }
    size_t off = 0;
    cudaError_t e = fill_dev_tables(t, &S.dt, [&](const auto& vec, auto** dst) { return put(S.base, &off, vec, dst); });
    if (e != cudaSuccess) {
      *msg = std::string("table upload into the scratch array: ") + cudaGetErrorString(e);
      S.j_max = -1.0;
      return e == cudaErrorMemoryAllocation ? MLD_ERR_OOM : MLD_ERR_CUDA;
    }
    S.table_bytes = align256(off);
    S.j_max = j_max;
  }
  *out = &S;
  return MLD_OK;
}

__global__ void k_widen(const float* __restrict__ in, double* __restrict__ out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

}  // namespace
}  // namespace mld

using namespace mld;

extern "C" int mld_gpu_descriptors_noalloc(const mld_gpu_config* cfg, int nat, const double* pos, const double* cell,
                                           const int* types, double* B, void* stream, char* err, int err_len) {
  if (!cfg || nat < 0 || (nat > 0 && (!pos || !cell || !types || !B))) {
    set_err(err, err_len, "invalid argument");
    return MLD_ERR_INVALID;
  }
  if (cfg->descriptor_type != 9) {
    set_err(err, err_len, "descriptor_type must be 9");
    return MLD_ERR_UNSUPPORTED;
  }
  if (!(cfg->inv_r0_input > 0.0 && cfg->inv_r0_input < 1.0) || !(cfg->r_cut > 0) || cfg->j_max < 0 ||
      cfg->n_elements < 1 || cfg->n_elements > MLD_MAX_ELEMENTS || (cfg->weighted_3ch && !cfg->weighted) ||
      cfg->imm_neigh < 1 ||
      (cfg->precision != MLD_PRECISION_PLAIN_FP64 && cfg->precision != MLD_PRECISION_MIXED)) {
    set_err(err, err_len, "invalid configuration");
    return MLD_ERR_INVALID;
  }
  if (nat > MLD_NOALLOC_MAX_ATOMS) {
    set_err(err, err_len, "nat = " + std::to_string(nat) + " exceeds MLD_NOALLOC_MAX_ATOMS = " +
                              std::to_string(MLD_NOALLOC_MAX_ATOMS));
    return MLD_ERR_NOALLOC_LIMIT;
  }
  if (nat == 0) return MLD_OK;
  const int nch = cfg->weighted ? (cfg->weighted_3ch ? 3 : 2) : 1;
  const bool mixed = cfg->precision == MLD_PRECISION_MIXED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  std::lock_guard<std::mutex> lock(g_mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_err(err, err_len, "no usable CUDA device");
    return MLD_ERR_CUDA;
  }
  DeviceState* S = nullptr;
  std::string msg;
  int rc = noalloc_setup(dev, cfg->j_max, &S, &msg);
  if (rc != MLD_OK) {
    set_err(err, err_len, msg);
    return rc;
  }
  const DevTables& dt = S->dt;
  const int KK = nch * dt.K;

  // cell geometry on the host (neighbours.F90:787-847)
  const double *a1 = cell, *a2 = cell + 3, *a3 = cell + 6;
  double c23[3] = {a2[1] * a3[2] - a2[2] * a3[1], a2[2] * a3[0] - a2[0] * a3[2], a2[0] * a3[1] - a2[1] * a3[0]};
  double c31[3] = {a3[1] * a1[2] - a3[2] * a1[1], a3[2] * a1[0] - a3[0] * a1[2], a3[0] * a1[1] - a3[1] * a1[0]};
  double c12[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
  const double det = a1[0] * c23[0] + a1[1] * c23[1] + a1[2] * c23[2];
  if (!(std::fabs(det) > 0)) {
    set_err(err, err_len, "singular cell");
    return MLD_ERR_INVALID;
  }
  struct HostBatch {
    int atom_start[2];
    int small;
    int nsize[3];
    double volume;
    double cell[9];
    double recip[9];
  } hb;
  hb.atom_start[0] = 0;
  hb.atom_start[1] = nat;
  hb.volume = std::fabs(det);
  hb.small = 0;
  for (int c = 0; c < 9; ++c) hb.cell[c] = cell[c];
  for (int c = 0; c < 3; ++c) {
    hb.recip[c] = c23[c] / det;
    hb.recip[3 + c] = c31[c] / det;
    hb.recip[6 + c] = c12[c] / det;
  }
  for (int i = 0; i < 3; ++i) {
    const double* b = hb.recip + 3 * i;
    const double bval = 1.0 / std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    const int nc = (int)(2.0 * cfg->r_cut / bval) + 1;
    if (nc > 1) hb.small = 1;
    hb.nsize[i] = nc / 2 + 1;
    if (hb.nsize[i] > 127) {
      set_err(err, err_len, "cell too thin for r_cut: more than 127 periodic images along a lattice vector");
      return MLD_ERR_INVALID;
    }
  }

  // carve the per-call region after the tables
  unsigned char* p = S->base + S->table_bytes;
  auto take = [&](size_t bytes) {
    unsigned char* q = p;
    p += align256(bytes);
    return q;
  };
  DevBatch b;
  b.S = 1;
  b.A = nat;
  HostBatch* d_hb = reinterpret_cast<HostBatch*>(take(sizeof(HostBatch)));
  b.atom_start = d_hb->atom_start;
  b.small = &d_hb->small;
  b.nsize = d_hb->nsize;
  b.volume = &d_hb->volume;
  b.cell = d_hb->cell;
  b.recip = d_hb->recip;
  b.pos = const_cast<double*>(pos);
  b.types = const_cast<int*>(types);
  b.atom_struct = reinterpret_cast<int*>(take(sizeof(int) * nat));
  b.nn = reinterpret_cast<int*>(take(sizeof(int) * nat));
  b.nbr_off = reinterpret_cast<int*>(take(sizeof(int) * (nat + 1)));
  b.pos32 = reinterpret_cast<float4*>(take(sizeof(float4) * nat));   // neighbour pre-filter copies
  b.frac32 = reinterpret_cast<float4*>(take(sizeof(float4) * nat));
  int* scan_tmp = reinterpret_cast<int*>(take(sizeof(int) * ((nat + 1023) / 1024 + 2)));
  int* dmax = reinterpret_cast<int*>(take(sizeof(int) * 2));
  int* qcount = reinterpret_cast<int*>(take(sizeof(int)));  // descriptor kernel's queue counter
  float* bstage = mixed ? reinterpret_cast<float*>(take(sizeof(float) * (size_t)nat * KK)) : nullptr;
  // global Y slices of the descriptor kernel only when they do not fit in shared memory (FP64
  // with several channels); at most 64 persistent CTAs
  const size_t ysb = bso4_y_scratch_bytes(dt, nch, mixed ? 4 : 8, 64, true);
  void* yscr = ysb ? take(ysb) : nullptr;
  const size_t fixed = (size_t)(p - S->base);
  if (fixed > kScratchBytes) {
    set_err(err, err_len, "descriptor staging exceeds the scratch array");
    return MLD_ERR_NOALLOC_LIMIT;
  }
  // remaining space holds the neighbour list: 4 B index + 24 B displacement per pair
  const long long pair_cap = std::min<long long>((long long)(kScratchBytes - fixed - 512) / 28,
                                                 (long long)MLD_NOALLOC_MAX_PAIRS);

#define CKN(call)                                                            \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess) {                                                 \
      set_err(err, err_len, std::string(#call) + ": " + cudaGetErrorString(_e)); \
      return MLD_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

  CKN(cudaMemcpyAsync(d_hb, &hb, sizeof(HostBatch), cudaMemcpyHostToDevice, st));
  CKN(cudaMemsetAsync(b.atom_struct, 0, sizeof(int) * nat, st));  // one structure
  CKN(cudaMemsetAsync(dmax, 0, sizeof(int) * 2, st));               // neighbour maximum starts at zero
  CKN(launch_neighbours(b, cfg->r_cut, b.nn, dmax, st, 0));
  CKN(launch_scan(b.nn, b.nbr_off, nat, scan_tmp, st));
  int hv[2] = {0, 0};
  CKN(cudaMemcpyAsync(&hv[0], b.nbr_off + nat, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKN(cudaMemcpyAsync(&hv[1], dmax, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKN(cudaStreamSynchronize(st));
  if (hv[1] > cfg->imm_neigh) {
    set_err(err, err_len, "an atom has " + std::to_string(hv[1]) + " neighbours within r_cut, more than imm_neigh=" +
                              std::to_string(cfg->imm_neigh));
    return MLD_ERR_NEIGHBOUR_CAP;
  }
  if ((long long)hv[0] > pair_cap) {
    set_err(err, err_len, std::to_string(hv[0]) + " neighbour pairs exceed the scratch limit of " +
                              std::to_string(pair_cap) + " pairs (MLD_NOALLOC_MAX_PAIRS)");
    return MLD_ERR_NOALLOC_LIMIT;
  }
  b.P = hv[0];
  b.nbr_idx = reinterpret_cast<int*>(take(sizeof(int) * (size_t)std::max(1, hv[0])));
  b.nbr_u = reinterpret_cast<double*>(take(sizeof(double) * 3 * (size_t)std::max(1, hv[0])));
  CKN(launch_neighbours(b, cfg->r_cut, b.nn, dmax, st, 1));

  BsoParams prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.rcut = cfg->r_cut;
  prm.inv_r0 = 3.14159265358979323846 * cfg->inv_r0_input;
  prm.nch = nch;
  prm.ntypes = cfg->n_elements;
  for (int t = 0; t < cfg->n_elements; ++t) {
    prm.chw[t] = 1.0;
    if (nch > 1) prm.chw[prm.ntypes + t] = cfg->weight_per_element[t];
    if (nch > 2) prm.chw[2 * prm.ntypes + t] = cfg->weight_per_element_3ch[t];
  }
  for (int a = 0; a < cfg->n_elements; ++a)
    for (int c = 0; c < cfg->n_elements; ++c) {
      const double v = cfg->r_cut_pair_in[a * MLD_MAX_ELEMENTS + c];
      prm.rin[a * prm.ntypes + c] = v;
      if (v > 0) prm.has_rin = 1;
    }
  prm.rin_width = cfg->r_cut_width_in;
  prm.sign_stress = cfg->sign_stress;
  prm.sign_big = cfg->sign_stress_big_box;
  if (mixed) {
    CKN(launch_bso4<float>(dt, b, prm, bstage, (float*)nullptr, nullptr, nullptr, qcount, st, yscr, ysb));
    const size_t n = (size_t)nat * KK;
    k_widen<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(bstage, B, n);
    CKN(cudaGetLastError());
  } else {
    CKN(launch_bso4<double>(dt, b, prm, B, (double*)nullptr, nullptr, nullptr, qcount, st, yscr, ysb));
  }
#undef CKN
  return MLD_OK;
}
