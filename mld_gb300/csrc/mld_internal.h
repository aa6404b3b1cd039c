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
constexpr int kRowTile = 4;        // rows (triples) per register tile of the dB contraction
constexpr int kColTile = 4;        // columns (neighbour, component) per register tile

// Symmetry used throughout: U^j(-p,-q) = (-1)^((p-q)/2) conj(U^j(p,q)); the same holds for c,
// the Z blocks and vecall.  Only the "half" of each layer is stored: the first
// H_j = ceil((j+1)^2/2) entries in row-major (p, q) order.  A source reference into a half
// layer is encoded as (half_index << 2) | (conj << 1) | negate, or -1 when absent.

// One output element of the Z contraction (compute_bispectrum_so4.F90:1014-1143).
// Z(m1,m2) = sum_{a<na, b<nb} cg1[a]*cg2[b] * c[i1 + a*s1 + b] * c[i2 - a*s2 - b]
// (full-layer indices of c) where layer jA supplies the first factor and jB the second.
struct ZTerm {
  uint16_t i1, i2;         // flattened c index of the first (ma,mb) / matching second factor
  uint16_t cg1, cg2;       // offsets into the 1-D CG coefficient table
  uint8_t na, nb, s1, s2;  // loop extents and layer strides (j+1)
  uint8_t snum, sden;      // scale snum/sden: 1 for ZA, (l+1)/(l1+1) for ZB, (l+1)/(l2+1) for ZC
  uint16_t pad;
};

// One slot of the folded Y array: triple k, layer j, half entry e.  Y = wgt * sum of the scaled
// Z blocks of k living on layer j at that entry; wgt = 2 off the symmetry centre, 1 on it.
struct YSlot {
  uint16_t term[3];
  uint8_t nterm;
  uint8_t is_a;            // term[0] is the ZA block (contributes to B_k)
  uint16_t ufull;          // full (j,p,q) index into c
  uint16_t k;              // triple index
  uint16_t ypos;           // position in the layer-blocked Y array
  uint8_t wgt;             // 2 or 1
  uint8_t pad;
};

// One lane of a phase-2 round, self-contained so that a lane fetches its work with one 32-byte
// load: the Z term (c indices of its first product, CG offsets, loop extents and strides) and
// its slot (Y position, c index of the slot's (j,p,q) for B, triple, scale); wgt = 0 marks a
// padding lane.
struct alignas(16) ZItem {
  uint16_t i1, i2, cg1, cg2;  // first (ma,mb) c index / matching second factor, CG offsets
  uint8_t na, nb, s1, s2;     // loop extents and layer strides (j+1)
  uint16_t ypos, ufull, k;    // slot: Y position, c index of its (j,p,q), triple
  uint8_t wgt, is_a;          // fold weight, ZA flag
  uint8_t snum, sden;         // scale snum / sden (formed in the kernel's precision)
  uint8_t pad[10];
};
static_assert(sizeof(ZItem) == 32, "phase-2 entries are 32 bytes");

// Packed per-entry recursion record of the half layers (one 16-byte load per entry).
struct RecEntry32 {
  float tz, tx;
  int16_t sz, sx;
  int32_t qneg;
};
struct RecEntry64 {
  double tz, tx;
  int16_t sz, sx;
  int32_t qneg;
  int64_t pad;
};

constexpr int kZWarps = 8;  // warps of the phase-2 schedule (= warps of a k_bso4 CTA)

// Host-built constant tables of the SO(4) bispectrum for a given j_max.
struct Bso4Tables {
  std::vector<ZItem> zitems;    // phase-2 rounds of 32 equal-shape terms, grouped per warp (LPT)
  std::vector<int> zitem_off;   // kZWarps + 1 round offsets (a round is 32 consecutive zitems)
  int J = 0, NU = 0, HU = 0, K = 0, NYP = 0;
  int off[kMaxJ + 2] = {0};     // full-layer offsets
  int hoff[kMaxJ + 2] = {0};    // half-layer offsets
  int Mp[kMaxJ + 1] = {0};      // padded row count per layer (multiple of kRowTile)
  int yoff[kMaxJ + 1] = {0};    // Y offset of each layer block (complex elements)
  std::vector<int> l1, l2, l;   // triples (reference order)
  std::vector<double> cg;       // 1-D CG coefficient lists
  std::vector<ZTerm> zterms;    // ZA/ZB/ZC outputs on half layers
  std::vector<YSlot> yslots;    // folded slots
  std::vector<int> yorder;      // slot evaluation order (cost-descending)
  std::vector<int16_t> rowk;    // per layer-block row: triple index or -1 (padding)
  int rowk_off[kMaxJ + 2] = {0};  // offset of each layer's rows in rowk
  std::vector<int> tiles;       // row tiles (j << 8 | rt), cost-descending
  // recursion on half layers: U = tz*Zsel*U[src_z] + tx*(-i)*Xsel*U[src_x]
  std::vector<double> rec_tz, rec_tx;
  std::vector<int16_t> rec_sz, rec_sx;
  std::vector<int8_t> rec_qneg;
  std::vector<int16_t> expand;  // full index -> encoded half source
  std::vector<int8_t> half_diag;  // half entries on the diagonal p == q (get the +1 of c)
  long long cg_terms = 0;       // CG products evaluated per channel (half outputs)
  long long cg_terms_full = 0;  // CG products of the unfolded contraction (reference count)
  long long u_one = 0, u_two = 0;  // half-layer recursion entries with one / two source terms
};

bool build_bso4_tables(double j_max, Bso4Tables* t, std::string* err);
double cg_coefficient(int j1, int m1, int j2, int m2, int j, int m);  // doubled indices

// Device copies of the tables.
struct DevTables {
  int J = 0, NU = 0, HU = 0, K = 0, NS = 0, NYP = 0, NTILE = 0;
  int NCG = 0;  // entries of the 1-D CG coefficient table
  int hoff[kMaxJ + 2] = {0};
  int Mp[kMaxJ + 1] = {0};
  int yoff[kMaxJ + 1] = {0};
  int rowk_off[kMaxJ + 2] = {0};
  ZTerm* zterms = nullptr;
  YSlot* yslots = nullptr;
  int* yorder = nullptr;
  int16_t* rowk = nullptr;
  int* tiles = nullptr;
  double* cg64 = nullptr;
  float* cg32 = nullptr;
  double* rec_tz64 = nullptr;
  double* rec_tx64 = nullptr;
  float* rec_tz32 = nullptr;
  float* rec_tx32 = nullptr;
  int16_t* rec_sz = nullptr;
  int16_t* rec_sx = nullptr;
  int8_t* rec_qneg = nullptr;
  int16_t* expand = nullptr;
  int8_t* half_diag = nullptr;
  RecEntry32* rec32 = nullptr;  // packed recursion records (FP32 method)
  RecEntry64* rec64 = nullptr;  // packed recursion records (FP64 method)
  ZItem* zitems = nullptr;
  int* zitem_off = nullptr;     // kZWarps + 1
};

// Packed recursion records from the table vectors.
inline void pack_recursion(const Bso4Tables& t, std::vector<RecEntry32>* r32, std::vector<RecEntry64>* r64) {
  r32->resize(t.HU);
  r64->resize(t.HU);
  for (int h = 0; h < t.HU; ++h) {
    (*r32)[h] = RecEntry32{(float)t.rec_tz[h], (float)t.rec_tx[h], t.rec_sz[h], t.rec_sx[h], (int32_t)t.rec_qneg[h]};
    (*r64)[h] = RecEntry64{t.rec_tz[h], t.rec_tx[h], t.rec_sz[h], t.rec_sx[h], (int32_t)t.rec_qneg[h], 0};
  }
}

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
  // FP32 copies for the neighbour pre-filter (written by the counting pass)
  float4* pos32 = nullptr;   // A  (x, y, z, 0)
  float4* frac32 = nullptr;  // A  (fractional coordinates b_k . x, 0)
  // neighbour list (CSR over atoms)
  int* nn = nullptr;         // A
  int* nbr_off = nullptr;    // A+1
  int* nbr_idx = nullptr;    // P
  double* nbr_u = nullptr;   // 3P  (x_neighbour - x_centre, FP64)
  long long P = 0;
  int maxnn = 0;             // largest neighbour count (after the counting pass)
};

// Design-row placement of each structure (-1 when a block is absent).
struct DevRows {
  long long M = 0;           // rows
  int D = 0;                 // row width (1 + nch*K for linear)
  int ldx = 0;               // row stride of the design matrix (D rounded up to 4)
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

inline int round_up4(int d) { return (d + 3) & ~3; }

// Kernels / launchers (return cudaError_t of the launch).
cudaError_t launch_neighbours(const DevBatch& b, double rcut, int* counts, int* maxcount, cudaStream_t st,
                              int pass /*0 count, 1 fill*/);
cudaError_t launch_scan(const int* in, int* out, int n, int* d_tmp, cudaStream_t st);

// Y scratch the descriptor kernel needs in global memory for up to max_ctas CTAs (0 when Y fits
// in shared memory); pass it to launch_bso4_rows, which then runs that many persistent CTAs.
size_t bso4_y_scratch_bytes(const DevTables& tb, int nch, int eb, int max_ctas);
// Evaluation with fitted weights instead of design rows: the energy, forces and stress that
// the rows times the weights would give, formed from the per-atom effective weights
// beta_a = dE/dB_a (w_lin for the linear model; w_lin + (W + W^T) B_a for the quadratic one).
template <typename T>
struct DevEval {
  const T* beta = nullptr;       // one vector (nch*K) or one per atom (A x nch*K)
  int beta_per_atom = 0;
  const double* wlin = nullptr;  // linear weights: the kernel adds w0 + w_lin . B_a to E (linear model)
  double w0 = 0.0;
  double* F = nullptr;           // 3A forces, accumulated (zeroed by the caller)
  double* S = nullptr;           // 6S stress rows' predictions, accumulated
  double* E = nullptr;           // S energies, accumulated
};

template <typename T>
cudaError_t launch_bso4_rows(const DevTables& tb, const DevBatch& b, const DevRows& rows, const BsoParams& p,
                             T* X, T* Bout, T* dBout, int want_rows, cudaStream_t st, void* yscratch = nullptr,
                             size_t yscratch_bytes = 0, const DevEval<T>* ev = nullptr);
// beta_a = w_lin + Wsym B_a and E_s += sum_a (w0 + B_a . (beta_a + w_lin) / 2)   (eval.cu)
template <typename T>
cudaError_t launch_eval_beta(const T* B, int A, int nchK, const double* wlin, const double* wsym, double w0,
                             const int* atom_struct, T* beta, double* E, cudaStream_t st);

template <typename T>
cudaError_t launch_gram(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* G,
                        double* h, cudaStream_t st);
cudaError_t launch_solve_sym(double* G, const double* h, int D, double lambda, double rcond, double* wout,
                             double* evals, int* info, cudaStream_t st);
template <typename T>
cudaError_t launch_rhs(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* h,
                       int nsm, cudaStream_t st, float2* sv);
cudaError_t launch_symmetrize(double* G, int D, cudaStream_t st);
cudaError_t launch_weighted_sumsq(const double* w, const double* y, long long M, double* out, cudaStream_t st);
cudaError_t launch_split_weights(const double* w, long long M, float2* wds, cudaStream_t st);
cudaError_t launch_normal_matvec(const float* X, int ldx, int c0, int D, const double* w, const double* p, long long M,
                                 double lambda, float2* sv, double* q, int nsm, cudaStream_t st, int* launches,
                                 int* err);
template <typename T>
cudaError_t launch_predict_sq(const T* X, int ldx, const double* w, long long M, int D, double* pred, const double* y,
                              const int* kind, double* sq, cudaStream_t st);
template <typename T>
cudaError_t launch_rows_prep(int S, const int* atom_start, const DevRows& rows, const double* E, const double* F,
                             const double* Sv, const double* wefs, T* X, double* y, double* wrow, int* kind,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_quad_rows(const DevBatch& b, const DevRows& rows, const BsoParams& p, int KK, const int* rev,
                             const T* B, const T* dB, T* H, T* X, int qoff, cudaStream_t st);
cudaError_t launch_reverse_pairs(const DevBatch& b, int* rev, cudaStream_t st);

// dense FP64 factorisation / solves (solve.cu)
// ds_update: trailing updates in double-FP32 on the FP32 pipe (preconditioner factors)
cudaError_t launch_cholesky(double* A, int D, double shift, int* info, cudaStream_t st, bool ds_update = false);
cudaError_t launch_chol_solve(const double* L, int D, const double* b, double* x, cudaStream_t st);
cudaError_t launch_chol_solve_blocked(const double* L, int D, const double* b, double* x, double* tmp,
                                      cudaStream_t st);
inline int chol_solve_launches(int D) { return 2 * ((D + 63) / 64); }
cudaError_t launch_cholesky_inverse(const double* L, int D, double* R, double* Rt, cudaStream_t st, int* launches);
cudaError_t launch_precond_apply(const double* R, const double* Rt, int D, const double* r, double* z, double* tmp,
                                 cudaStream_t st);
inline int cholesky_launches(int D) { return 3 * ((D + 31) / 32) - 2; }

// FP32 inverse of a wide block's preconditioner factor (precond32.cu)
size_t precond32_workspace_bytes(int D);
cudaError_t launch_precond32_from_factor(const double* Lf, int D, void* ws, cudaStream_t st, int* launches);
cudaError_t launch_precond32_apply(const void* ws, int D, const double* r, double* z, double* tmp, cudaStream_t st);
cudaError_t launch_residual(const double* G, int D, double lambda, const double* w, const double* h, double* r,
                            cudaStream_t st);
cudaError_t launch_axpy(int n, double a, const double* x, double* y, cudaStream_t st);
cudaError_t launch_shift_diag_rel(double* A, int D, double lambda, double rel, cudaStream_t st);
cudaError_t launch_pcg_alpha(int D, const double* p, const double* q, double* x, double* r, double* scal,
                             cudaStream_t st);
cudaError_t launch_pcg_beta(int D, const double* z, const double* r, double* p, double* scal, int first,
                            cudaStream_t st);

// kernel ridge regression rows (kernel_rows.cu)
size_t krr_workspace_elems(int A, int nk, int KK);
template <typename T>
cudaError_t launch_krr_rows(const DevBatch& b, const DevRows& rows, const int* rev, const T* Bq, const T* dBq,
                            const T* Z, int nk, int KK, double power, double length, double sigma,
                            double sign_stress, double sign_big, T* ws, T* X, int c0, cudaStream_t st,
                            int* launches, void* tcws = nullptr, size_t tcws_bytes = 0, int* err = nullptr,
                            int nsm = 0);
// kernel-block force rows on the tensor cores (krr_tc.cu); the workspace that holds all `atoms`
// (maxnv derivative vectors at most) in one chunk
// sketched preconditioner of wide mixed blocks (sketch.cu)
constexpr int kSketchZeta = 8;
struct SketchParams {
  int zeta;        // signed copies of each row of X
  int s;           // sketch rows
  long long M;     // rows of X
  uint64_t seed;   // signs
  long long a[kSketchZeta], ainv[kSketchZeta], b[kSketchZeta];  // affine permutations of the rows
};
SketchParams sketch_params(long long M, int D, uint64_t seed);
size_t sketch_workspace_bytes(long long M, int D);
// G (D x D, FP64, full) = Y^T Y of the sketch Y = S W^1/2 X[:, c0 : c0 + D]
cudaError_t launch_sketch_gram(const float* X, int ldx, int c0, int D, const double* w, long long M,
                               const SketchParams& P, void* ws, double* G, cudaStream_t st, int* launches);
constexpr int kKrrTcMaxK = 192;  // three K blocks of 64 in shared memory
bool krr_force_tc_available();
size_t krr_force_tc_workspace_bytes(long long atoms, int maxnv, int nk, int KK);
cudaError_t launch_krr_force_tc(const DevBatch& b, const DevRows& rows, const int* rev, const float* Bq,
                                const float* dBq, const float* Z, const float* F, const float* at, const float* szz,
                                const float* Ts, const float* tx, double sign_stress, int nk, int KK, double power,
                                double length, double sigma, void* ws, size_t ws_bytes, float* X, int c0, int* err,
                                int nsm, cudaStream_t st, int* launches);

// tensor-core Gram in BF16 split precision (gram_tc.cu)
size_t gram_tc_min_workspace(int D);
bool gram_tc_available();
template <typename T>
cudaError_t launch_gram_tc(const T* X, int ldx, int c0, int D, const double* w, long long M, double* G, void* ws,
                           size_t ws_bytes, int* err, int nsm, cudaStream_t st);

}  // namespace mld
