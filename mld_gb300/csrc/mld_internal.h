// Internal declarations shared by the CUDA translation units of libmld_gpu.
// Nothing here is part of the public C ABI (include/mld_gpu.h).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <stdint.h>
#include <string>
#include <vector>

namespace mld {

constexpr int kMaxJ = 10;          // doubled angular momentum bound (j_max <= 5)
constexpr int kMaxTypes = 8;       // element types per handle
constexpr int kMaxCh = 3;          // plain, weighted, weighted_3ch
constexpr int kRowTile = 4;        // rows (triples) per register tile of the dB contraction


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

// One lane of a phase-2 round (16 bytes): the Z term's c indices of its first product, CG
// offsets, loop extents and strides, and the term's index in the per-atom term buffer
// (kNoTerm marks a padding lane).
struct alignas(16) ZItem {
  uint16_t i1, i2, cg1, cg2;  // first (ma,mb) c index / matching second factor, CG offsets
  uint8_t na, nb, s1, s2;     // loop extents and layer strides (j+1)
  uint16_t term;              // index of the term (its Z value) in the term buffer
  uint16_t pad;
};
static_assert(sizeof(ZItem) == 16, "phase-2 entries are 16 bytes");
// the descriptor kernel decodes entries from their four 32-bit words at these byte offsets
static_assert(offsetof(ZItem, i2) == 2 && offsetof(ZItem, cg1) == 4 && offsetof(ZItem, cg2) == 6 &&
                  offsetof(ZItem, na) == 8 && offsetof(ZItem, nb) == 9 && offsetof(ZItem, s1) == 10 &&
                  offsetof(ZItem, s2) == 11 && offsetof(ZItem, term) == 12,
              "ZItem layout");
constexpr uint16_t kNoTerm = 0xFFFF;

// One folded Y slot for the kernel (16 bytes): Y[ypos] = wgt * sum_t (snum_t / sden_t) Z[term_t].
struct SlotEntry {
  uint16_t term[3];
  uint16_t ypos;
  uint8_t nterm, wgt;
  uint8_t snum[3], sden[3];
};
static_assert(sizeof(SlotEntry) == 16, "slot entries are 16 bytes");
static_assert(offsetof(SlotEntry, ypos) == 6 && offsetof(SlotEntry, nterm) == 8 && offsetof(SlotEntry, wgt) == 9 &&
                  offsetof(SlotEntry, snum) == 10 && offsetof(SlotEntry, sden) == 13,
              "SlotEntry layout (decoded from its words by the descriptor kernel)");
// snum and sden are doubled angular momenta + 1 <= kMaxJ + 1; the descriptor kernel looks
// snum / sden up in a 16 x 16 table
static_assert(kMaxJ + 1 < 16, "slot scales index a 16 x 16 table");

// One ZA half entry of a triple: B_k = sum over its entries of wgt * Re(conj(c[ufull]) Z[term]).
struct BkItem {
  uint16_t term, ufull;
  uint8_t wgt, pad[3];
};
static_assert(sizeof(BkItem) == 8, "B items are 8 bytes");
static_assert(offsetof(BkItem, ufull) == 2 && offsetof(BkItem, wgt) == 4, "BkItem layout (decoded by the descriptor kernel)");

// Packed per-entry recursion record of the half layers (one 16-byte load per entry).  tz and tx
// (>= 0 in the tables) are stored with the sign that selects the entry's Z / conj(Z) and X
// (+ for qneg != 0), so the kernel takes their magnitudes with fabs.
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

constexpr int kZWarps = 8;   // warps of the phase-2 schedule (= warps of a k_bso4 CTA)
constexpr int kRounds = 3;   // ranks of a triple's layer rows (its distinct layers in ascending order)
constexpr int kRankShift = 12;  // row destination code: (rank << kRankShift) | index within the rank's buffer

// Host-built constant tables of the SO(4) bispectrum for a given j_max.
struct Bso4Tables {
  std::vector<ZItem> zitems;    // phase-2 rounds of 32 terms of one nb (na descending), grouped per warp (LPT)
  std::vector<int> zitem_off;   // kZWarps + 1 round offsets (a round is 32 consecutive zitems)
  int J = 0, NU = 0, HU = 0, K = 0, NYP = 0;
  int off[kMaxJ + 2] = {0};     // full-layer offsets
  int hoff[kMaxJ + 2] = {0};    // half-layer offsets
  int Mp[kMaxJ + 1] = {0};      // padded row count per layer (multiple of kRowTile per round group)
  int yoff[kMaxJ + 1] = {0};    // Y offset of each layer block (complex elements)
  std::vector<int> l1, l2, l;   // triples (reference order)
  std::vector<double> cg;       // 1-D CG coefficient lists
  std::vector<ZTerm> zterms;    // ZA/ZB/ZC outputs on half layers
  int nzu = 0;                  // distinct Z computations among them (the term buffer's entries)
  std::vector<YSlot> yslots;    // folded slots
  std::vector<SlotEntry> slots; // the same slots in the kernel's form
  std::vector<int> bk_off;      // K + 1 offsets into bk_items
  std::vector<BkItem> bk_items; // ZA entries of each triple
  // per layer-block row: destination code (rank << kRankShift) | index, -1 for padding; the
  // index is the triple for rank 0 and the triple's slot in the rank-1 / rank-2 buffers
  std::vector<int16_t> rowk;
  int rowk_off[kMaxJ + 2] = {0};  // offset of each layer's rows in rowk
  std::vector<int> tiles;       // row tiles (j << 8 | rt), heaviest layers first
  int nrank[kRounds] = {0};     // triples with a row of rank r (rank 0: all K)
  std::vector<int16_t> rank_slot;  // K x (kRounds - 1): slot of triple k in the rank-1 / rank-2 buffers, -1 none
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
  int J = 0, NU = 0, HU = 0, K = 0, NS = 0, NYP = 0, NTILE = 0, NZT = 0, NROWS = 0;
  int NCG = 0;  // entries of the 1-D CG coefficient table
  int hoff[kMaxJ + 2] = {0};
  int Mp[kMaxJ + 1] = {0};
  int yoff[kMaxJ + 1] = {0};
  int rowk_off[kMaxJ + 2] = {0};
  int nrank[kRounds] = {0};
  int16_t* rowk = nullptr;
  int16_t* rank_slot = nullptr;  // K x (kRounds - 1)
  int* tiles = nullptr;
  double* cg64 = nullptr;
  float* cg32 = nullptr;
  int16_t* expand = nullptr;
  int8_t* half_diag = nullptr;
  RecEntry32* rec32 = nullptr;  // packed recursion records (FP32 method)
  RecEntry64* rec64 = nullptr;  // packed recursion records (FP64 method)
  ZItem* zitems = nullptr;
  int* zitem_off = nullptr;     // kZWarps + 1
  SlotEntry* slots = nullptr;   // NS
  int* bk_off = nullptr;        // K + 1
  BkItem* bk_items = nullptr;
};

// Packed recursion records from the table vectors.
inline void pack_recursion(const Bso4Tables& t, std::vector<RecEntry32>* r32, std::vector<RecEntry64>* r64) {
  r32->resize(t.HU);
  r64->resize(t.HU);
  for (int h = 0; h < t.HU; ++h) {
    // tz, tx >= 0 carry the sign of the entry's q (+ for q >= 0), which selects Z / conj(Z) and X
    const double sq = t.rec_qneg[h] ? 1.0 : -1.0;
    (*r32)[h] = RecEntry32{(float)(sq * t.rec_tz[h]), (float)(sq * t.rec_tx[h]), t.rec_sz[h], t.rec_sx[h], (int32_t)t.rec_qneg[h]};
    (*r64)[h] = RecEntry64{sq * t.rec_tz[h], sq * t.rec_tx[h], t.rec_sz[h], t.rec_sx[h], (int32_t)t.rec_qneg[h], 0};
  }
}

// Fill the scalar part of *d from t and place every device table through put(vector, &ptr),
// which allocates (or carves) device memory of the vector's size and copies it there.
template <class Put>
cudaError_t fill_dev_tables(const Bso4Tables& t, DevTables* d, Put put) {
  *d = DevTables();
  d->J = t.J;
  d->NU = t.NU;
  d->HU = t.HU;
  d->K = t.K;
  d->NS = (int)t.slots.size();
  d->NYP = t.NYP;
  d->NTILE = (int)t.tiles.size();
  d->NZT = t.nzu;
  d->NROWS = (int)t.rowk.size();
  d->NCG = (int)t.cg.size();
  for (int j = 0; j <= t.J + 1; ++j) {
    d->hoff[j] = t.hoff[j];
    d->rowk_off[j] = t.rowk_off[j];
  }
  for (int j = 0; j <= t.J; ++j) {
    d->Mp[j] = t.Mp[j];
    d->yoff[j] = t.yoff[j];
  }
  for (int r = 0; r < kRounds; ++r) d->nrank[r] = t.nrank[r];
  // the CG table padded to whole 16-byte chunks (the descriptor kernel stages it with 16-byte
  // asynchronous copies)
  std::vector<double> cg64(t.cg);
  cg64.resize((cg64.size() + 1) / 2 * 2, 0.0);
  std::vector<float> cg32(t.cg.begin(), t.cg.end());
  cg32.resize((cg32.size() + 3) / 4 * 4, 0.0f);
  std::vector<RecEntry32> r32;
  std::vector<RecEntry64> r64;
  pack_recursion(t, &r32, &r64);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = put(t.rowk, &d->rowk);
  if (e == cudaSuccess) e = put(t.rank_slot, &d->rank_slot);
  if (e == cudaSuccess) e = put(t.tiles, &d->tiles);
  if (e == cudaSuccess) e = put(cg64, &d->cg64);
  if (e == cudaSuccess) e = put(cg32, &d->cg32);
  if (e == cudaSuccess) e = put(t.expand, &d->expand);
  if (e == cudaSuccess) e = put(t.half_diag, &d->half_diag);
  if (e == cudaSuccess) e = put(r32, &d->rec32);
  if (e == cudaSuccess) e = put(r64, &d->rec64);
  if (e == cudaSuccess) e = put(t.zitems, &d->zitems);
  if (e == cudaSuccess) e = put(t.zitem_off, &d->zitem_off);
  if (e == cudaSuccess) e = put(t.slots, &d->slots);
  if (e == cudaSuccess) e = put(t.bk_off, &d->bk_off);
  if (e == cudaSuccess) e = put(t.bk_items, &d->bk_items);
  return e;
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
  float4* nbr_u32 = nullptr; // P (x, y, z, 1/r) rounded from the FP64 values, for the FP32
                             // descriptor kernel (null: it converts nbr_u itself)
  long long P = 0;
  int maxnn = 0;             // largest neighbour count (after the counting pass)
  // linked cells of large boxes (null cnc: every structure scans all its atoms)
  int* cnc = nullptr;        // 3S cells per lattice direction, 0 for a structure without cells
  int* cell_off = nullptr;   // S+1 first cell of each structure
  int ncells = 0;
  int* cell_of = nullptr;    // A cell of each atom (-1 without cells)
  int* cell_start = nullptr; // ncells+1 first entry of each cell in cell_atoms (then a cursor of ncells)
  int* cell_atoms = nullptr; // A atoms grouped by cell
  int* sort_tmp = nullptr;   // P  neighbour indices while the lists of celled structures are sorted
  // single-pass search: each atom's pairs (neighbour, packed image) in a row of nbr_cap entries
  int2* nbr_tmp = nullptr;   // A * nbr_cap
  int nbr_cap = 0;
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
// pass 0 counts and 1 fills the CSR lists (two scans of the candidates); pass 2 counts and
// writes each atom's pairs into b.nbr_tmp in one scan, pass 3 then compacts them into the CSR.
// Passes 1 and 3 end with the sorted lists of celled structures and the displacements.
cudaError_t launch_neighbours(const DevBatch& b, double rcut, int* counts, int* maxcount, cudaStream_t st,
                              int pass);
cudaError_t launch_scan(const int* in, int* out, int n, int* d_tmp, cudaStream_t st);
// Bin the atoms of celled structures (b.cnc) into their cells; scan_tmp as for launch_scan over
// b.ncells entries.  Then launch_neighbours scans the 27 (or fewer, unique) cells around each
// atom, and launch_sort_lists restores the ascending neighbour order of those atoms' lists.
cudaError_t launch_cells(const DevBatch& b, int* scan_tmp, cudaStream_t st);
cudaError_t launch_sort_lists(const DevBatch& b, cudaStream_t st);

// Y scratch the descriptor kernel needs in global memory for up to max_ctas CTAs (0 when Y fits
// in shared memory); pass it to launch_bso4, which then runs at most that many persistent CTAs.
// Bytes of the descriptor kernel's global Y slices for max_ctas persistent CTAs: needed when Y
// does not fit in shared memory, and preferred (unless only_if_required) when it would cost a
// resident CTA per SM; 0 otherwise.
size_t bso4_y_scratch_bytes(const DevTables& tb, int nch, int eb, int max_ctas, bool only_if_required = false);
// Evaluation with fitted weights instead of design rows: per-pair force and stress
// contributions of dE/dB_a (beta_a = w_lin for the linear model; w_lin + (W + W^T) B_a for the
// quadratic one), gathered into E/F/S by launch_eval_gather.
template <typename T>
struct DevEval {
  const T* beta = nullptr;       // one vector (nch*K) or one per atom (A x nch*K)
  int beta_per_atom = 0;
  const double* wlin = nullptr;  // linear weights: the kernel writes Eatom = w0 + w_lin . B_a (linear model)
  double w0 = 0.0;
  double* pair = nullptr;        // P x 9: force contribution f_q (3), stress contribution (6: xx yy zz yz xz xy)
  double* Eatom = nullptr;       // A: energy of each atom (linear model; may be null)
};

// Launch shape of the descriptor kernel, chosen per handle by the autotuner (api.cu); every
// shape gives bitwise the same results.
struct Bso4Launch {
  int col_tile = 4;      // columns per register tile of the dB contraction: 2 or 4
  int ctas_per_sm = 0;   // persistent CTAs per SM (0: as many as fit)
  int sorted_queue = 1;  // atoms longest first (1) or in index order (0)
};
// Descriptor kernel (bispectrum.cu): B (A x nch*K) and w_ch * dB (P x 3 x nch*K) of the batch,
// either may be null; or evaluation (ev->pair set, dBout null).  Atoms are taken in `order`
// (null: index order) through `counter` (one int of device memory, reset by the launch).
template <typename T>
cudaError_t launch_bso4(const DevTables& tb, const DevBatch& b, const BsoParams& p, T* Bout, T* dBout,
                        const DevEval<T>* ev, const int* order, int* counter, cudaStream_t st,
                        void* yscratch = nullptr, size_t yscratch_bytes = 0, const Bso4Launch* shape = nullptr);
// Linear design rows of the batch from B, w_ch * dB and the reverse pairs (rows.cu); Sp is a
// workspace of A x 6 x KK stress partials.  Columns [1, 1 + KK) of the energy, force and stress
// rows are written.
template <typename T>
cudaError_t launch_lin_rows(const DevBatch& b, const DevRows& rows, const BsoParams& p, int KK, const int* rev,
                            const T* B, const T* dB, T* Sp, T* X, cudaStream_t st);
// E (S; from Eatom when given), F (3A) and S (6S) from the per-pair contributions of evaluation.
cudaError_t launch_eval_gather(const DevBatch& b, const BsoParams& p, const int* rev, const double* pair,
                               const double* Eatom, double* E, double* F, double* S, cudaStream_t st);
// Atoms ordered by descending neighbour count (the descriptor kernel's queue); tmp holds
// atom_order_tmp_ints(maxnn) ints.
size_t atom_order_tmp_ints(int maxnn);
cudaError_t launch_atom_order(const int* nn, int A, int maxnn, int* order, int* tmp, cudaStream_t st);
// beta_a = w_lin + Wsym B_a and Eatom_a = w0 + B_a . (beta_a + w_lin) / 2   (eval.cu)
template <typename T>
cudaError_t launch_eval_beta(const T* B, int A, int nchK, const double* wlin, const double* wsym, double w0, T* beta,
                             double* Eatom, cudaStream_t st);

// FP64 Gram and rhs on the CUDA cores; with ws (gram_workspace_doubles(M, D) doubles) the
// row-chunk partials are summed in a fixed order (bitwise reproducible), else with atomics
size_t gram_workspace_doubles(long long M, int D);
template <typename T>
cudaError_t launch_gram(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* G,
                        double* h, cudaStream_t st, double* ws = nullptr);
cudaError_t launch_solve_sym(double* G, const double* h, int D, double lambda, double rcond, double* wout,
                             double* evals, int* info, cudaStream_t st);
template <typename T>
cudaError_t launch_rhs(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* h,
                       int nsm, cudaStream_t st, float2* sv, double* ws = nullptr);
cudaError_t launch_symmetrize(double* G, int D, cudaStream_t st);
// ws: at least kSumsqBlocks doubles (per-block partials, added in block order)
constexpr int kSumsqBlocksMax = 1024;
cudaError_t launch_weighted_sumsq(const double* w, const double* y, long long M, double* out, double* ws,
                                  cudaStream_t st);
cudaError_t launch_split_weights(const double* w, long long M, float2* wds, cudaStream_t st);
// ws: normal_matvec_workspace_doubles(M, D, nsm) doubles for the per-block partial column sums,
// reduced in block order (null: FP64 atomics, order not fixed)
size_t normal_matvec_workspace_doubles(long long M, int D, int nsm);
cudaError_t launch_normal_matvec(const float* X, int ldx, int c0, int D, const double* w, const double* p, long long M,
                                 double lambda, float2* sv, double* q, double* ws, int nsm, cudaStream_t st,
                                 int* launches, int* err);
// doubles of the squared-error buffer of launch_predict_sq (3 sums, 3 counts, per-CTA partials)
size_t predict_sq_doubles();
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
// doubles of the per-split partial tiles launch_gram_tc needs for a deterministic sum (0: none)
size_t gram_tc_part_doubles(int D, int nsm);
void gram_tc_test_timeout(int skip_loads, long long wait_limit);
bool gram_tc_available();
template <typename T>
cudaError_t launch_gram_tc(const T* X, int ldx, int c0, int D, const double* w, long long M, double* G, void* ws,
                           size_t ws_bytes, int* err, int nsm, cudaStream_t st, double* part = nullptr,
                           size_t part_doubles = 0);

}  // namespace mld
