// Internal declarations shared by the CUDA translation units of libmld_gpu.
// Nothing here is part of the public C ABI (include/mld_gpu.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

namespace mld {

constexpr int kMaxJ = 10;          // doubled angular momentum bound (j_max <= 5)
constexpr int kMaxTypes = 8;       // element types per handle
constexpr int kMaxCh = 3;          // plain, weighted, weighted_3ch

// One output element of the Z contraction (compute_bispectrum_so4.F90:1014-1143).
// Z(m1,m2) = sum_{a<na, b<nb} cg1[a]*cg2[b] * c[i1 + a*s1 + b] * c[i2 - a*s2 - b]
// where layer jA supplies the first factor and layer jB the second.
struct ZTerm {
  uint16_t i1, i2;       // flattened c index of the first (ma,mb) / matching second factor
  uint16_t cg1, cg2;     // offsets into the 1-D CG coefficient table
  uint8_t na, nb, s1, s2;  // loop extents and layer strides (j+1)
  uint8_t snum, sden;    // scale snum/sden: 1 for ZA, (l+1)/(l1+1) for ZB, (l+1)/(l2+1) for ZC
  uint16_t pad;
};

// One slot of the merged Y array: for triple k and layer j, the sum of the scaled Z blocks
// of k living on layer j at entry (p,q).  nterm in {1,2,3}; term[] index ZTerm entries.
struct YSlot {
  uint16_t term[3];
  uint8_t nterm;
  uint8_t is_a;          // first term is the ZA block (contributes to B_k)
  uint16_t uidx;         // flattened (j,p,q) index into c / V
  uint16_t k;            // triple index
};

// Host-built constant tables of the SO(4) bispectrum for a given j_max.
struct Bso4Tables {
  int J = 0, NU = 0, K = 0;
  int off[kMaxJ + 2] = {0};
  std::vector<int> l1, l2, l;           // triples (reference order)
  std::vector<double> cg;               // 1-D CG coefficient lists
  std::vector<ZTerm> zterms;            // all ZA/ZB/ZC outputs
  std::vector<YSlot> yslots;            // merged slots, grouped by k (contiguous per k)
  std::vector<int> kslot_begin;         // K+1 offsets into yslots
  std::vector<int> yorder;              // yslot evaluation order (cost-descending)
  long long cg_terms_A = 0, cg_terms_B = 0, cg_terms_C = 0;
};

bool build_bso4_tables(double j_max, Bso4Tables* t, std::string* err);
double cg_coefficient(int j1, int m1, int j2, int m2, int j, int m);  // doubled indices

// Device copies of the tables.
struct DevTables {
  int J = 0, NU = 0, K = 0, NY = 0;
  ZTerm* zterms = nullptr;
  YSlot* yslots = nullptr;
  int* kslot_begin = nullptr;
  int* yorder = nullptr;
  double* cg64 = nullptr;
  float* cg32 = nullptr;
  // U-recursion coefficients per flattened index: U = tz*Zsel*U[sz] - i*tx*Xsel*U[sx]
  double* rec_tz64 = nullptr;
  double* rec_tx64 = nullptr;
  float* rec_tz32 = nullptr;
  float* rec_tx32 = nullptr;
  int16_t* rec_sz = nullptr;
  int16_t* rec_sx = nullptr;
  int8_t* rec_qneg = nullptr;
  int16_t* uj = nullptr;     // layer j of each flattened index
  int16_t* up = nullptr;     // p of each flattened index
  int16_t* uq = nullptr;     // q of each flattened index
};

// Per-batch structure description on the device.
struct DevBatch {
  int S = 0;                 // structures
  int A = 0;                 // atoms
  int* atom_start = nullptr; // S+1
  int* atom_struct = nullptr;// A
  int* types = nullptr;      // A
  double* pos = nullptr;     // 3A
  double* cell = nullptr;    // 9S  (cell[9s+3i+c] = a_i[c])
  double* recip = nullptr;   // 9S  (b_k with a_i.b_k = delta)
  int* small = nullptr;      // S
  int* nsize = nullptr;      // 3S
  double* volume = nullptr;  // S
  // neighbour list (CSR over atoms)
  int* nn = nullptr;         // A
  int* nbr_off = nullptr;    // A+1
  int* nbr_idx = nullptr;    // P
  double* nbr_u = nullptr;   // 3P  (x_neighbour - x_centre, FP64)
  long long P = 0;
  size_t P_cap = 0;
};

// Design-row placement of each structure (-1 when a block is absent).
struct DevRows {
  long long M = 0;           // rows
  int D = 0;                 // row width (1 + nch*K for linear)
  long long* rowE = nullptr; // S
  long long* rowF = nullptr; // S (first of 3*nat force rows)
  long long* rowS = nullptr; // S (first of 6 stress rows)
};

struct BsoParams {
  double rcut, inv_r0;       // inv_r0 = pi * inv_r0_input
  int nch, ntypes;
  double chw[kMaxCh * kMaxTypes];
  double rin[kMaxTypes * kMaxTypes];
  double rin_width;
  int has_rin;
  double sign_stress, sign_big;
};

// Kernels / launchers (return cudaError_t of the launch).
cudaError_t launch_neighbours(const DevBatch& b, double rcut, int* counts, int* maxcount, cudaStream_t st,
                              int pass /*0 count, 1 fill*/);
cudaError_t launch_scan(const int* in, int* out, int n, int* d_tmp, cudaStream_t st);

template <typename T>
cudaError_t launch_bso4_rows(const DevTables& tb, const DevBatch& b, const DevRows& rows, const BsoParams& p,
                             T* X, T* Bout, T* dBout, int want_rows, cudaStream_t st);

template <typename T>
cudaError_t launch_gram(const T* X, const double* w, const double* y, long long M, int D, double* G, double* h,
                        cudaStream_t st);
cudaError_t launch_solve_sym(double* G, const double* h, int D, double lambda, double rcond, double* wout,
                             double* work, int* info, cudaStream_t st);
template <typename T>
cudaError_t launch_predict(const T* X, const double* w, long long M, int D, double* pred, cudaStream_t st);

size_t bso4_smem_bytes(int NU, int NY, int K, int nch, int elem_bytes, int nwarps);

}  // namespace mld
