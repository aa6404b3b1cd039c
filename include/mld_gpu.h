/*
 * mld_gpu.h -- C ABI of the GB300 bispectrum-SO(4) descriptor-to-fit path.
 *
 * Plain C types and pointers only; one opaque handle per fitting job.  Every entry point
 * returns an int status (MLD_OK = 0) and never aborts the host process; the text of the last
 * failure is available from mld_gpu_last_error().  All arrays are caller-owned host memory
 * unless the name ends in _device (device pointers, e.g. from cudaMalloc).
 *
 * Layouts follow the reference's Fortran column-major arrays, so a Fortran caller passes its
 * arrays through ISO_C_BINDING (c_loc) without copies:
 *   pos_cart(3, nat)   -> pos[3*i + c]
 *   cell(3, 3)         -> cell[3*i + c] = component c of lattice vector a_i  (columns = vectors)
 *   force(3, nat)      -> force[3*i + c]
 *   stress(6)          -> xx, yy, zz, yz, xz, xy
 *   energy(dim, nat)   -> B[dim*i + k]   (descriptor k of atom i; channel-major within dim)
 *   Amat(D, M)         -> A[D*r + c]     (design row r, column c)
 * Types are 0-based indices into the element list of the configuration.
 *
 * Reference interfaces replaced (paths inside the MILADY project):
 *   &input_ml namelist subset      src/mld/read_ml_file.F90:174-252 (defaults :307-611)
 *   compute_descriptors, case 9    src/mld/descriptors.F90:87-382, :658-671;
 *                                  src/mld/compute/compute_bispectrum_so4.F90:43
 *   calc_neighbours                src/mld/neighbours.F90:852 (small :1147, large :1091)
 *   train_fill_Amat_with_energy    src/mld/mld_energy.F90:364
 *   train_fill_Amat_with_force     src/mld/mld_forces.F90:649
 *   train_fill_Amat_with_stress    src/mld/mld_stress.F90:181
 *   train_snap_get_parameters      src/mld/parameters.F90:354 (linear :1018)
 *   gram%accumulate / reduce_and_solve  src/mld/module_online_fit.F90:138-265, :432-598
 *   md_mld_compute_energy/force/stress  src/mld/mld.F90:1579, :1673, :1777
 */
#ifndef MLD_GPU_H
#define MLD_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define MLD_OK 0
#define MLD_ERR_INVALID 1        /* bad argument or configuration */
#define MLD_ERR_CUDA 2           /* CUDA runtime error (message in mld_gpu_last_error) */
#define MLD_ERR_NEIGHBOUR_CAP 3  /* an atom has more than imm_neigh neighbours within r_cut */
#define MLD_ERR_OOM 4            /* device allocation failed */
#define MLD_ERR_SOLVE 5          /* the normal matrix could not be solved */
#define MLD_ERR_STATE 6          /* call order: e.g. fit before structures were staged */
#define MLD_ERR_UNSUPPORTED 7    /* option outside this build (e.g. descriptor_type != 9) */
#define MLD_ERR_TIMEOUT 9        /* a bounded device-side wait expired (kernel returned early) */

#define MLD_PRECISION_PLAIN_FP64 0  /* all-FP64 on the GPU */
#define MLD_PRECISION_MIXED 1       /* FP32 descriptors and rows; normal matrix on the tensor cores in
                                       BF16 split precision (hi*hi + hi*lo + lo*hi, FP32 accumulation,
                                       FP64 across row blocks) or, for blocks of 768 columns or more, a
                                       sparse-sign sketch in double-FP32; FP64 Cholesky of the
                                       preconditioner; conjugate gradients with double-FP32 matvecs over
                                       the FP32 rows, so the coefficients solve the FP32 rows' normal
                                       equations */

#define MLD_MAX_ELEMENTS 8

/* The &input_ml subset read by the descriptor-to-fit path (read_ml_file.F90:174-252). */
typedef struct mld_gpu_config {
  int descriptor_type;      /* must be 9 (bispectrum SO(4)) */
  double j_max;             /* j_max (half-integers allowed); default 1.5 */
  double r_cut;             /* r_cut [Angstrom]; default 5.0 */
  double inv_r0_input;      /* default 1 - 0.02/pi; must lie in (0,1) */
  int weighted;             /* weighted: second channel with per-element weights */
  int weighted_3ch;         /* weighted_3ch: third channel */
  int n_elements;           /* fix_no_of_elements (types are 0..n_elements-1) */
  double weight_per_element[MLD_MAX_ELEMENTS];      /* channel-2 weights (after any weighted_auto renorm) */
  double weight_per_element_3ch[MLD_MAX_ELEMENTS];  /* channel-3 weights */
  double r_cut_pair_in[MLD_MAX_ELEMENTS * MLD_MAX_ELEMENTS];  /* inner cutoff per element pair, 0 = off */
  double r_cut_width_in;    /* default 0.4 */
  int desc_forces;          /* 1: force and stress design rows */
  int ml_type;              /* 0 linear / quadratic models, 1 kernel ridge regression (KRR) */
  int mld_order;            /* ml_type 0: 1 linear, 2 quadratic (QNML two-stage) */
  double lambda_krr;        /* ridge: lambda added to the normal-matrix diagonal (ml_type 0) or
                               lambda^2 (ml_type 1, [sqrt(W) A; lambda I] least squares); < 0 -> 0;
                               default -1 */
  double svd_rcond;         /* singular-value cut of the min-norm solve; < 0 -> machine precision; default -1 */
  double sign_stress;       /* default 1 */
  double sign_stress_big_box; /* default 1 */
  int imm_neigh;            /* neighbour cap per atom; default 300 */
  int precision;            /* MLD_PRECISION_PLAIN_FP64 or MLD_PRECISION_MIXED */
  /* kernel ridge regression (ml_type 1): &input_ml kernel_type, kernel_power, length_kernel,
     sigma_kernel (read_ml_file.F90:338-347); only kernel_type 4 (normalised polynomial) */
  int kernel_type;          /* default 4 */
  double kernel_power;      /* default 2 */
  double length_kernel;     /* default sqrt(1/2) */
  double sigma_kernel;      /* default 0 */
} mld_gpu_config;

typedef struct mld_gpu_handle mld_gpu_handle;

/* Fill *cfg with the reference's namelist defaults (read_ml_file.F90:307-611). */
void mld_gpu_config_defaults(mld_gpu_config* cfg);

/* Create a handle on the current CUDA device (init_descriptors, descriptors.F90:658-671). */
int mld_gpu_create(const mld_gpu_config* cfg, mld_gpu_handle** out);
void mld_gpu_destroy(mld_gpu_handle* h);
const char* mld_gpu_last_error(const mld_gpu_handle* h);

/* Dimensions: K = bispectrum components per channel (bisso4_dim), dim_desc = channels*K
 * (dim_xdesc), dim_design_line = width of one design row (1 + dim_desc for the linear model). */
int mld_gpu_dims(const mld_gpu_handle* h, int* K, int* dim_desc, int* dim_design_line);

/* Stage a batch of structures (the per-configuration loop of mld.F90:376-404).
 * nat[S]; pos[3*sum(nat)]; cell[9*S]; types[sum(nat)].  Copies to the device. */
int mld_gpu_set_structures(mld_gpu_handle* h, int nstruct, const int* nat, const double* pos, const double* cell,
                           const int* types);

/* Labels and per-structure weights of the design rows
 * (train_fill_Amat_with_energy/force/stress):
 *   energy[S]   = energy(iread_energy) (already minus the per-element reference energies),
 *   force[3*sum(nat)], stress[6*S],
 *   has_efs[3*S] = has_energy, has_force, has_stress flags (0/1),
 *   w_efs[3*S]   = w_e_model, w_f_model, w_s_model.
 * Any pointer may be NULL when no structure uses that block. */
int mld_gpu_set_labels(mld_gpu_handle* h, const double* energy, const double* force, const double* stress,
                       const int* has_efs, const double* w_efs);

/* Neighbour lists + descriptors of the staged batch (compute_descriptors).
 * B_out[dim_desc*sum(nat)] (may be NULL); n_neigh_out[sum(nat)] (may be NULL). */
int mld_gpu_descriptors(mld_gpu_handle* h, double* B_out, int* n_neigh_out);

/* Per-pair derivatives dB/du of the last mld_gpu_descriptors call, in neighbour-list order:
 * nbr_out[P] (global atom index of each neighbour, per centre atom in order), u_out[3*P]
 * (x_neighbour - x_centre), dB_out[3*dim_desc*P] (derivative with the sign of
 * descriptors.F90:298-302).  *P_inout: capacity in pairs on input, pairs on output. */
int mld_gpu_descriptor_derivatives(mld_gpu_handle* h, long long* P_inout, int* nbr_out, double* u_out,
                                   double* dB_out);

/* Number of design rows of the staged batch (energy + 3N force + 6 stress rows per structure,
 * as the has_efs flags and desc_forces select). */
int mld_gpu_num_rows(mld_gpu_handle* h, long long* M);

/* Build and return the design matrix A[M*dim_design_line], labels y[M] and row weights w[M]
 * (any may be NULL). */
int mld_gpu_design_matrix(mld_gpu_handle* h, double* A, double* y, double* w);

/* Weighted normal matrix G[D*D] = A^T W A and rhs[D] = A^T W y of the staged batch
 * (no ridge term; module_online_fit.F90 gram%accumulate). */
int mld_gpu_gram(mld_gpu_handle* h, double* G, double* rhs);

/* Min-norm ridge solve of (G + lambda*I) w = rhs with the handle's lambda_krr / svd_rcond
 * (serial_lsystem_by_svd).  rank_out may be NULL. */
int mld_gpu_solve(mld_gpu_handle* h, const double* G, const double* rhs, int D, double* w, int* rank_out);

/* Full fit of the staged batch: neighbours, descriptors, rows, Gram, ridge solve
 * (main_train_mld / train_snap_get_parameters).  w_params[dim_design_line];
 * rmse_efs[3] (may be NULL) = train RMSE of energy, force components, stress. */
int mld_gpu_fit(mld_gpu_handle* h, double* w_params, double* rmse_efs);

/* Predictions of the staged batch with coefficients w_params (md_mld_compute_energy/force/stress):
 * E[S] (w . energy row, excluding reference energies), F[3*sum(nat)], S[6*S]; any may be NULL. */
int mld_gpu_predict(mld_gpu_handle* h, const double* w_params, double* E, double* F, double* S);
/* The same energies, forces and stress as mld_gpu_predict (ml_type 0), evaluated without design
 * rows: the descriptor derivatives are contracted with the per-atom effective weights
 * beta_a = dE/dB_a (w_lin; w_lin + (W + W^T) B_a for the quadratic model, the neighbour's beta in
 * the stress as the reference's quadratic stress rows use the neighbour's B) and summed in FP64.
 * This is how the reference's MD evaluation (md_mld_compute_energy/force/stress, mld.F90:1579-1867)
 * can be computed when only E/F/S are wanted; the serving loop uses it. */
int mld_gpu_evaluate(mld_gpu_handle* h, const double* w_params, double* E, double* F, double* S);

/* Block until the handle's stream has finished. */
int mld_gpu_synchronize(mld_gpu_handle* h);

/* ---- measurement (the reference's phase timers, time_check_general / repport_time,
 *      ml_in_ndm_module.F90:271-320, re-done with CUDA events on the handle's stream) ---- */
#define MLD_NPHASE 6
#define MLD_PHASE_NEIGHBOURS 0   /* count, scan, fill */
#define MLD_PHASE_ROWS 1         /* zero the design matrix, labels and weights */
#define MLD_PHASE_DESCRIPTORS 2  /* fused bispectrum + design-row kernel */
#define MLD_PHASE_GRAM 3         /* weighted Gram and right-hand side */
#define MLD_PHASE_SOLVE 4        /* ridge / min-norm solve */
#define MLD_PHASE_PREDICT 5      /* train predictions and squared errors */

/* Record CUDA events around each phase of mld_gpu_fit (on = 1) and accumulate their times. */
int mld_gpu_set_profiling(mld_gpu_handle* h, int on);
/* Accumulated per-phase device time [ms], kernel launches and fits (arrays of MLD_NPHASE;
 * any may be NULL); reset != 0 clears the accumulators after reading. */
int mld_gpu_profile(mld_gpu_handle* h, double* ms, long long* launches, long long* calls, int reset);
/* Event-based interval timer on the handle's stream (stop synchronises on its event). */
int mld_gpu_timer_start(mld_gpu_handle* h);
int mld_gpu_timer_stop(mld_gpu_handle* h, double* ms);
/* Sizes behind the algorithmic work model of the descriptor kernel, out[12] =
 * {NU, one-term U entries, two-term U entries, CG terms (ZA+ZB+ZC), sum of Z row extents,
 *  Z outputs, merged Y slots, Y slots carrying ZA, K, channels, neighbour pairs, atoms}. */
int mld_gpu_work_counts(const mld_gpu_handle* h, long long* out);
/* Measured CUDA-core FMA throughput [TFLOP/s] of this GPU for the precision's descriptor type
 * (FP64 for MLD_PRECISION_PLAIN_FP64, FP32 for MLD_PRECISION_MIXED): the roofline denominator
 * of the descriptor kernel. */
int mld_gpu_peak_flops(mld_gpu_handle* h, int precision, double* tflops);

/* Reference points of the kernel model (ml_type 1): nk raw descriptors of selected atoms
 * (nk x dim_desc, row-major), the rows of kernel_matrix.dat (compute_kernel.F90:1058-1256).
 * They are standardised per component over the set, z = (z_raw - mean) / std (population
 * std); a component with zero spread is rejected (MLD_ERR_INVALID).  Sets dim_design_line to
 * 1 + dim_desc + nk. */
int mld_gpu_set_kernel_points(mld_gpu_handle* h, int nk, const double* z_raw);

/* Solver record of the last mixed-method fit: conjugate-gradient iterations, final relative
 * preconditioned residual and the relative diagonal shift of the Cholesky preconditioner, per
 * stage (0 = linear block, 1 = quadratic block of QNML), and how often the preconditioner had
 * to be re-factorised with a larger shift.
 * (No reference counterpart: the reference solves with dgelsd, stats_tools.F90:1153-1213.) */
int mld_gpu_solve_info(const mld_gpu_handle* h, int* pcg_iterations /*[2]*/, double* pcg_residual /*[2]*/,
                       double* precond_shift /*[2]*/, int* chol_retries);

/* Launch shape of the descriptor kernel chosen by the handle's autotuner for one output mode
 * (0: design rows, i.e. B and dB; 1: evaluation with fitted weights; 2: descriptors only).  Only
 * mode 0 is tuned (modes 1 and 2 run the default shape: column tile 4, as many CTAs per SM as
 * fit, longest-first queue).  The tuner times every candidate once on the first batch with
 * enough atoms (64 per SM) and keeps the fastest;
 * all candidates give bitwise the same results.  shape[4] = {column tile (4 or 2), persistent
 * CTAs per SM (0 = as many as fit), longest-first queue (1) or index order (0), tuned (1/0)};
 * *ncand: capacity of ms on input, candidates timed on output; ms[i] the time [ms] of candidate
 * i in the order (column tile 4, 2) x (CTAs per SM max, 1) x (queue sorted, index).
 * (No reference counterpart.) */
int mld_gpu_tuning(const mld_gpu_handle* h, int mode, int* shape, int* ncand, double* ms);

/* Test hook of the device-side timeout path (no reference counterpart).  skip_loads = 1 makes
 * the producer warp of the tensor-core Gram (the mixed method's narrow-block normal matrix and
 * mld_gpu_gram_rows) issue no loads, so its consumers' bounded waits expire after
 * wait_limit_clocks SM clocks (0 = the default of about one second); the kernel then reports the
 * expiry, frees its tensor memory and returns, and the call fails with MLD_ERR_TIMEOUT while the
 * handle stays usable.  (0, 0) restores normal operation.  Process-wide; not for production use. */
int mld_gpu_test_pipeline_timeout(int skip_loads, long long wait_limit_clocks);

/* ---------------------------------------------------------------------------------------
 * Serving loop (evaluation with a fitted potential under continuous batching; the evaluation
 * side of mld.F90:1579-1867 as driven by mld_md_driver.F90:324-375,579-651).
 * A server holds n_slots evaluation slots (one stream and one set of device buffers each).
 * Requests (one structure each) are queued by submit and evaluated by progress(), which
 * retires finished batches and fills idle slots with queued requests in arrival order while a
 * batch stays within its share of hbm_fraction * (free HBM at creation) and max_batch_atoms.
 * w_params: fitted weights in the reference's full layout (dim_design_line of cfg). */
typedef struct mld_gpu_server mld_gpu_server;
int mld_gpu_server_create(const mld_gpu_config* cfg, const double* w_params, int n_slots, long long max_batch_atoms,
                          double hbm_fraction, mld_gpu_server** out);
void mld_gpu_server_destroy(mld_gpu_server* s);
const char* mld_gpu_server_last_error(const mld_gpu_server* s);
/* copies the structure (positions 3*nat, cell 3x3 rows = lattice vectors, types) */
int mld_gpu_server_submit(mld_gpu_server* s, int nat, const double* pos, const double* cell, const int* types,
                          long long* ticket);
/* non-blocking: retire finished batches, launch queued requests into idle slots */
int mld_gpu_server_progress(mld_gpu_server* s, int* n_busy_slots, int* n_queued);
/* *ready = 1 and the results (E, F[3*nat], S[6], latency from submit to completion) once the
 * request is done; the ticket is then released.  A failed request returns its error code. */
int mld_gpu_server_result(mld_gpu_server* s, long long ticket, double* E, double* F, double* S, double* latency_ms,
                          int* ready);
/* progress() until the request is done or timeout_ms (> 0) passes (MLD_ERR_TIMEOUT) */
int mld_gpu_server_wait(mld_gpu_server* s, long long ticket, double* E, double* F, double* S, double* latency_ms,
                        double timeout_ms);
int mld_gpu_server_stats(const mld_gpu_server* s, long long* batches, long long* atoms_done, double* budget_bytes);
/* Admission record: the largest sum of estimated device bytes of the batches on the GPU at one
 * time (never above budget_bytes), the per-slot share of the budget, and the largest estimated
 * bytes of one batch.  A request above the share waits until every slot is idle and then runs
 * alone.  (No reference counterpart: the reference evaluates one structure per MD step.) */
int mld_gpu_server_admission(const mld_gpu_server* s, double* peak_bytes_in_flight, double* share_bytes,
                             double* largest_batch_bytes);

/* Weighted Gram matrix and right-hand side of caller-owned DEVICE rows, the per-block
 * accumulation of the online fit (gram%accumulate, module_online_fit.F90:49-53,138-265):
 *   G   (D x D, row-major FP64, device)   = sum_r w[r] x_r x_r^T
 *   rhs (D, FP64, device; may be NULL)    = sum_r w[r] y[r] x_r
 * X holds M rows of D values with a row stride of ldx elements, FP64 (x_is_fp32 = 0) or FP32.
 * method MLD_PRECISION_PLAIN_FP64: FP64 accumulation on the CUDA cores; MLD_PRECISION_MIXED:
 * tensor cores in BF16 split precision (x = hi + lo, hi*hi + hi*lo + lo*hi) with FP32
 * accumulation per row split and FP64 accumulation across splits.  Allocates and frees its own
 * workspace; `stream` may be NULL; returns after the stream has synchronised. */
int mld_gpu_gram_rows(int method, const void* X, int x_is_fp32, long long M, int D, int ldx, const double* w,
                      const double* y, double* G, double* rhs, void* stream, char* err, int err_len);

/* ---- descriptors without device allocation --------------------------------------------
 * No counterpart in the MILADY reference.  Some callers cannot call cudaMalloc: it
 * synchronises the device, and hosts whose device memory is owned by another runtime's pool
 * have nothing to call it with.  Examples are MD steps, serving loops and such pool-managed
 * hosts.  This entry point computes the bispectrum descriptors of ONE structure on the
 * current device and allocates nothing.  Its scratch (contraction tables, neighbour list, scan
 * and FP32 staging) lives in one static device array of MLD_NOALLOC_SCRATCH_MIB MiB, which
 * every GPU that loads the library holds until the process exits.
 *   cfg    configuration as for mld_gpu_create (descriptor_type 9; both precisions)
 *   pos    DEVICE pointer, 3*nat doubles (pos_cart(3,nat))
 *   cell   HOST pointer, 9 doubles (cell(3,3), columns = lattice vectors)
 *   types  DEVICE pointer, nat ints (0-based element index)
 *   B      DEVICE pointer, nat*dim_desc doubles (energy(dim_desc, nat)), written on `stream`
 *   stream cudaStream_t or NULL for the default stream
 *   err    optional buffer of err_len bytes that receives a message when the call fails
 * Limits: nat <= MLD_NOALLOC_MAX_ATOMS and at most MLD_NOALLOC_MAX_PAIRS neighbour pairs
 * (fewer when many channels need FP32 staging).  Larger inputs return MLD_ERR_NOALLOC_LIMIT.
 * The first call on a device resolves the array's address (cudaGetSymbolAddress) and uploads
 * the tables; make that first call before any stream capture.  A call whose j_max differs from
 * the previous call's on that device re-uploads the tables, and first waits for the whole device
 * (cudaDeviceSynchronize), because the previous call may have run on another stream.  Every call
 * shares the array and it keeps the last call's contents.  Counters that must start at zero are
 * cleared on every call.  Calls that overlap on the GPU (two streams, or two host threads on one
 * device) race on the array: serialise them.  The call synchronises once on `stream` to read the
 * pair count; B is complete when `stream` is next synchronised. */
#define MLD_NOALLOC_SCRATCH_MIB 48
#define MLD_NOALLOC_MAX_ATOMS 16384
#define MLD_NOALLOC_MAX_PAIRS 1048576
#define MLD_ERR_NOALLOC_LIMIT 8  /* input larger than the static scratch array allows */
int mld_gpu_descriptors_noalloc(const mld_gpu_config* cfg, int nat, const double* pos, const double* cell,
                                const int* types, double* B, void* stream, char* err, int err_len);

#ifdef __cplusplus
}
#endif
#endif /* MLD_GPU_H */
