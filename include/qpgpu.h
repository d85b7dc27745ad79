/*
 * qpgpu.h -- C ABI of the GB300 (sm_103a) Davidson sigma library.
 *
 * Drop-in boundary for Quantum Package's sigma path.  Each entry point names
 * the reference routine (path:line in the quantum_package source tree) whose
 * role it takes; the Fortran host binds them through iso_c_binding.
 *
 * Conventions
 *  - Every call returns an int status: QPGPU_OK (0) or a negative QPGPU_ERR_*;
 *    qpgpu_last_error() gives the message of the last failure of a context.
 *    The reference stops the program instead (diagonalization_hs2.irp.f:110-114,
 *    404-409); the Fortran shim turns a non-zero status into `stop`.
 *  - Orbitals are 1-based; determinants are psi_det(N_int,2,N) int64 bit
 *    strings (Fortran order: for det k, alpha words then beta words).
 *  - Vectors u_0(sze,N_st) are column-major double precision, leading
 *    dimension `ld` >= N_det, determinants in psi_det order.
 *  - "host" arguments are host pointers (the call copies); "device" arguments
 *    are device pointers on the context's GPU.  A NULL `stream` selects the
 *    context's own stream; pass cudaStreamLegacy ((void*)1) for the legacy
 *    default stream.
 *  - A context may be used by one host thread at a time (calls lock it).
 */
#ifndef QPGPU_H
#define QPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QPGPU_OK 0
#define QPGPU_ERR_ARG (-1)      /* invalid argument (shape, null pointer, range) */
#define QPGPU_ERR_STATE (-2)    /* integrals / determinants not set */
#define QPGPU_ERR_CUDA (-3)     /* CUDA runtime error */
#define QPGPU_ERR_NOMEM (-4)    /* device allocation failed */
#define QPGPU_ERR_DAVIDSON (-5) /* Davidson failed (residual > 1e8) */
#define QPGPU_ERR_TIMEOUT (-6)  /* a bounded device wait ran out (the tensor-core Gram's mbarrier waits) */
#define QPGPU_ERR_NUMERIC (-7)  /* NaN / Inf in an input vector: checked by the entry points that take
                                   host arrays (qpgpu_h_s2_u0, _work, qpgpu_u0_h_u0 and the guess of
                                   qpgpu_davidson_hs2); the asynchronous device entry points do not check */

/* Arithmetic of a sigma application. */
#define QPGPU_FP64 0  /* FP64 matrix elements and products */
#define QPGPU_FP32 1  /* FP32 elements and products, Kahan-compensated per-row sums,
                         FP64 diagonal */
#define QPGPU_FF 2    /* float-float (hi + lo FP32 pairs, about 47 significant bits) elements,
                         coefficients and sums on the FP32 pipes, FP64 diagonal: FP64-class
                         accuracy (1e-13 relative) at FP32-pipe speed.  No counterpart in the
                         reference.  In qpgpu_davidson_hs2 it selects FP32 sigma with a
                         float-float sigma as the restart (defect-correction) sigma. */

typedef struct qpgpu_ctx qpgpu_ctx;

typedef struct qpgpu_info {
  int64_t n_det;          /* N_det */
  int32_t n_alpha_unique; /* N_det_alpha_unique */
  int32_t n_beta_unique;  /* N_det_beta_unique */
  int64_t n_pairs;        /* directed connected pairs (I != J, degree 1-2) */
  int64_t n_s2_pairs;     /* pairs with <I|S^2|J> != 0 */
  double setup_ms;        /* device time of the last qpgpu_set_dets */
  double ref_energy;      /* ref_bitmask_energy */
  int64_t device_bytes;   /* device memory held by the context */
  int64_t n_split_rows;   /* rows whose pairs span several sigma work chunks */
  int32_t direct_sigma;   /* 1: pairs not stored, sigma enumerates them at each call */
  int32_t n_keyed_lines;  /* beta columns + alpha rows with deletion-key tables */
} qpgpu_info;

/* Context for one orbital space; replaces the IRPF90 providers N_int,
 * elec_alpha_num, elec_beta_num, mo_tot_num (src/Bitmask/bitmasks.irp.f:3-15).
 * n_int must be (n_mo-1)/64+1 and at most 2 (n_mo <= 128).  n_alpha >= n_beta
 * as in src/Bitmask/bitmasks.irp.f:82. */
int qpgpu_create(int n_mo, int n_alpha, int n_beta, int n_int, qpgpu_ctx** out);
int qpgpu_destroy(qpgpu_ctx* ctx);
const char* qpgpu_last_error(qpgpu_ctx* ctx);
int qpgpu_get_info(qpgpu_ctx* ctx, qpgpu_info* info);

/* How sigma reaches the connected pairs (no counterpart in the reference,
 * which recomputes every matrix element at each call, u0Hu0.irp.f:177-444).
 * QPGPU_SIGMA_STORED: qpgpu_set_dets stores the pairs and their FP64 / FP32
 * elements once, and sigma streams them (the fast path).  QPGPU_SIGMA_DIRECT:
 * nothing is stored; every sigma enumerates the pairs again from the
 * bilinear index and evaluates the Slater rules in FP64, as the reference
 * does, for determinant sets whose pairs do not fit in device memory (FP32
 * requests run in FP64; qpgpu_connected_pairs, the no-alloc sigma and
 * batches need stored pairs).  QPGPU_SIGMA_AUTO (default): stored unless the
 * pairs would leave less than 1/16 of the device memory free.  Takes effect at
 * the next qpgpu_set_dets. */
#define QPGPU_SIGMA_AUTO 0
#define QPGPU_SIGMA_STORED 1
#define QPGPU_SIGMA_DIRECT 2
int qpgpu_set_sigma_mode(qpgpu_ctx* ctx, int mode);

/* How the pair scans reach the partners of a determinant (no counterpart in
 * the reference, whose loops test every string of the lines involved,
 * u0Hu0.irp.f:177-332).  A beta column (alpha row) holding more than
 * min_single determinants gets a table of its alpha (beta) strings with one
 * electron removed, which the alpha x beta scan probes instead of scanning the
 * line; one holding more than min_double gets a table with two electrons
 * removed, which its own determinants probe for their same-spin pairs.  The
 * pairs, and so sigma, are the same either way; only the work changes (a few
 * heavy lines carry most of the scan work of large sets).  -1 keeps a default
 * (min_single 64 (n_elec + 2), min_double 16384); INT64_MAX turns tables off.
 * hash_bits (1..64, default 64) keeps the low bits of the key hashes only, to
 * test that colliding keys still give the exact pairs; below 64,
 * qpgpu_set_dets refuses (QPGPU_ERR_ARG) a table of more than 2^22 keys,
 * whose merged groups would make the scans quadratic.  Tables that would
 * take more than half of the free device memory are left out.  Takes effect
 * at the next qpgpu_set_dets. */
int qpgpu_set_line_keys(qpgpu_ctx* ctx, int64_t min_single, int64_t min_double, int hash_bits);

/* u_0_H_u_0 (src/Davidson/diagonalization_hs2.irp.f:446-484), the psi_energy
 * provider's routine: e_0[i] = <u_0(:,i)|H|u_0(:,i)> over the N_det rows of the
 * host array u_0(ld, n_st) (column-major, psi_det order), FP64 sigma on the
 * device.  As in the reference the value is not divided by <u|u> (psi_coef is
 * normalised) and a zero column gives 0; electronic energy (no nuclear
 * repulsion). */
int qpgpu_u0_h_u0(qpgpu_ctx* ctx, double* e_0, const double* u_0, int n_st, int64_t ld);

/* Integrals (host).  h_pq: n_mo x n_mo column-major, symmetric
 * (mo_mono_elec_integral, src/Integrals_Monoelec/mo_mono_ints.irp.f:1-26).
 * eri_packed: chemist (pq|rs) at bielec_integrals_index key - 1
 * (src/Integrals_Bielec/map_integrals.irp.f:19-34), P2*(P2+1)/2 entries with
 * P2 = n_mo*(n_mo+1)/2.  Derives on the device mo_bielec_integral_jj /
 * _jj_anti (mo_bi_integrals.irp.f:1344-1369), big_array_coulomb/exchange
 * (integrals_3_index.irp.f:1-22), the closed-shell Fock operator
 * (mono_excitations.irp.f:22-95) and ref_bitmask_energy (ref_bitmask.irp.f:1-56).
 * Replaces the integral hash map / dense cache.  Invalidates determinant data. */
int qpgpu_set_integrals(qpgpu_ctx* ctx, const double* h_pq, const double* eri_packed);

/* Determinants (host, psi_det(N_int,2,n_det)).  Builds on the device the
 * bilinear alpha x beta index (spindeterminants.irp.f:56-596), the connected
 * pairs with their FP64/FP32 matrix elements, H_II and <I|S^2|I>.  This is the
 * provider rebuild the reference performs after TOUCH psi_det. */
int qpgpu_set_dets(qpgpu_ctx* ctx, const uint64_t* psi_det, int64_t n_det);

/* H_S2_u_0_nstates_openmp (src/Davidson/u0Hu0.irp.f:15-66), host arrays:
 * v_0 = H u_0 and s_0 = S^2 u_0 (S^2 without the S_z(S_z-1) shift, as the
 * reference), each (ld, n_st) column-major.  u_0 is read only. */
int qpgpu_h_s2_u0(qpgpu_ctx* ctx, double* v0, double* s0, const double* u0, int n_st, int64_t ld);

/* H_S2_u_0_nstates_openmp_work (src/Davidson/u0Hu0.irp.f:69-96), host arrays
 * in bilinear order, states fastest: u_t(n_st, N_det), v_t, s_t.  Only rows
 * k = istart+ishift, istart+ishift+istep, ..., <= iend (1-based) are written;
 * other rows of v_t, s_t are left untouched. */
int qpgpu_h_s2_u0_work(qpgpu_ctx* ctx, double* v_t, double* s_t, const double* u_t, int n_st, int istart,
                       int iend, int ishift, int istep);

/* Device variant of qpgpu_h_s2_u0: same layout, device pointers, runs on the
 * given CUDA stream (NULL: the context's stream), precision QPGPU_FP64 or
 * QPGPU_FP32.  Asynchronous. */
int qpgpu_h_s2_u0_device(qpgpu_ctx* ctx, double* v0, double* s0, const double* u0, int n_st, int64_t ld,
                         int precision, void* stream);

/* Sigma in the internal layout: u_t, v_t, s_t are device arrays (N_det, n_st)
 * with states fastest, determinants in bilinear order (the order of
 * qpgpu_bilinear_order).  u_t32 (FP32 copy of u_t) is required for
 * QPGPU_FP32 and ignored otherwise; both must be 16-byte aligned.
 * Asynchronous on `stream`. */
int qpgpu_sigma_bilinear(qpgpu_ctx* ctx, double* v_t, double* s_t, const double* u_t, const float* u_t32,
                         int n_st, int precision, void* stream);

/* No counterpart in the reference.  qpgpu_sigma_bilinear without any device
 * allocation, for callers that cannot let the library call cudaMalloc (a host
 * code whose device memory belongs to its own pool allocator, or a worker that
 * overlaps sigma with work on other streams and cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree).  Same arguments and results as
 * qpgpu_sigma_bilinear, except that only QPGPU_FP64 and QPGPU_FP32 are accepted
 * (QPGPU_FF gives QPGPU_ERR_ARG) and the pairs must be stored (a direct-sigma
 * set gives QPGPU_ERR_STATE).  Its
 * scratch (partial sums of rows split over several work chunks) is a fixed
 * 8 MiB device array of the library, held by every GPU that loads it until
 * exit: the call fails with QPGPU_ERR_ARG when work chunks x n_st exceeds
 * 524288 (about 100k determinants at 4 states).  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make that first
 * call before any stream capture.  All calls share the array: calls that may
 * overlap on the GPU (other streams, other contexts on the same device) race. */
int qpgpu_sigma_bilinear_noalloc(qpgpu_ctx* ctx, double* v_t, double* s_t, const double* u_t,
                                 const float* u_t32, int n_st, int precision, void* stream);

/* Dressing of one state for the MRCC / MRCEPA0 sigma, H_S2_u_0_mrcc_nstates
 * (plugins/MRCC_Utils/davidson.irp.f:955-1127), host arrays: determinants
 * idx_ref[0..n_ref) (psi_det indices, 0-based; idx_ref of the reference) and
 * idx_non_ref[0..n_non_ref) (idx_non_ref), all distinct; delta_ij and
 * delta_ij_s2 (n_non_ref, n_ref) column-major, the slice delta_ij(istate,:,:)
 * of the reference's provider; delta_ii (n_ref, may be NULL for zeros), the
 * diagonal dressing davidson_diag_mrcc_hs2 adds to H_jj (:547-549).  The
 * dressing stays with the determinant set (qpgpu_set_dets drops it). */
int qpgpu_set_dressing(qpgpu_ctx* ctx, int n_ref, const int32_t* idx_ref, int64_t n_non_ref,
                       const int32_t* idx_non_ref, const double* delta_ij, const double* delta_ij_s2,
                       const double* delta_ii);
int qpgpu_clear_dressing(qpgpu_ctx* ctx);

/* H_S2_u_0_mrcc_nstates with host arrays, as qpgpu_h_s2_u0: v_0 = (H + dressing) u_0,
 * s_0 = (S^2 + dressing_s2) u_0, the diagonal of H dressed by delta_ii. */
int qpgpu_h_s2_u0_dressed(qpgpu_ctx* ctx, double* v0, double* s0, const double* u0, int n_st, int64_t ld);

/* X(m, n) = A^T B for tall A (N x m) and B (N x n), device arrays whose rows
 * are lda / ldb doubles apart (the u_t(N_st, N) layout, states fastest), on
 * the given stream (NULL: the context's): the dgemm('T','N') Gram blocks of
 * davidson_diag_hjj_sjj (src/Davidson/diagonalization_hs2.irp.f:232-238)
 * computed to FP64 accuracy on the tensor cores.  Each column is split into
 * eight balanced 7-bit BF16 digit planes against its largest exponent (Ozaki
 * splitting), the digit products are summed exactly (FP32 tensor-core
 * accumulators flushed into integers every 128 rows) and the per-SM results
 * combined in FP64.  m <= 128, n <= 16; X (m x n, row-major) is written on
 * the device and the call waits for the stream; a bounded tensor-core wait
 * that runs out gives QPGPU_ERR_TIMEOUT.  Uses the context only for its
 * scratch and stream. */
int qpgpu_gram_tc(qpgpu_ctx* ctx, const double* A, int64_t lda, int m, const double* B, int64_t ldb, int n,
                  int64_t N, double* X, void* stream);

/* Davidson parameters: the EZFIO knobs of src/Davidson/EZFIO.cfg:1-36 and
 * src/Determinants/EZFIO.cfg:13-41 plus the precision options. */
typedef struct qpgpu_davidson_params {
  int32_t n_states;         /* N_st */
  int32_t n_states_diag;    /* N_st_diag (<= 8) */
  int32_t davidson_sze_max; /* micro-iterations before re-contraction (8) */
  int32_t s2_eig;           /* keep Ritz vectors with |S^2 - expected| < 0.6 (1) */
  double threshold;         /* threshold_davidson on the squared step norm (1e-12) */
  int32_t precision;        /* QPGPU_FP64, or QPGPU_FP32: FP32 sigma with an FP64 sigma at each restart */
  int32_t defect_every;     /* FP32 mode: restart (FP64 sigma) at least every k iterations (0: sze_max) */
  int32_t preconditioner;   /* 0: the reference's diagonal step; 1: learned (MLP) step in place of the
                               diagonal one, with fallback; 2: learned step as an extra direction in the
                               slot of Ritz vector n_states + k (states k < n_states_diag - n_states) */
  int32_t max_iter;         /* cap on sigma applications (0: 1000) */
  int32_t collect_every;    /* > 0: capture training pairs every k iterations (from the 2nd) */
  int32_t collect_max;      /* captures kept (default 8) */
  int32_t state_following;  /* state_following (src/Davidson/EZFIO.cfg:19-22): keep the Ritz vectors
                               that overlap most with the guess states (diagonalization_hs2.irp.f:328-370) */
  int32_t algebra;          /* QPGPU_ALGEBRA_FAST (mixed modes): projections, Gram-Schmidt, Ritz vectors
                               and the step on the FP32 pipes (float-float / FP32); QPGPU_ALGEBRA_FP64:
                               all of them in FP64 as in the plain loop, so only sigma runs in FP32;
                               QPGPU_ALGEBRA_TC (any precision): FP64-level accuracy with the
                               projections, Gram-Schmidt Grams and updates, Ritz vectors and
                               re-contraction on the tensor cores (qpgpu_gram_tc / qpgpu_lincomb_tc),
                               the small Cholesky-QR Gram and update, step and residual norms in
                               FP64, the Ritz vectors of FP32-sigma iterations in FP32 (they only
                               feed the step) */
  int32_t dressed;          /* 1: davidson_diag_mrcc_hs2 (plugins/MRCC_Utils/davidson.irp.f:496-553):
                               sigma and H_jj carry the context's dressing (qpgpu_set_dressing) */
  int32_t reserved;         /* 0 */
} qpgpu_davidson_params;
#define QPGPU_ALGEBRA_FAST 0
#define QPGPU_ALGEBRA_FP64 1
#define QPGPU_ALGEBRA_TC 2

/* Optional per-iteration record of a Davidson run. */
typedef struct qpgpu_davidson_trace {
  int32_t cap;              /* entries available in the arrays below */
  int32_t n;                /* iterations recorded */
  int32_t n_sigma;          /* sigma applications */
  int32_t converged;        /* 1 when the threshold was met */
  int32_t* sigma_precision; /* [cap] precision of each iteration's sigma */
  double* energies;         /* [cap][n_states] Ritz values */
  double* residuals;        /* [cap][n_states] squared step norms */
  double* elapsed_ms;       /* [cap] device time from the start of the call */
  int32_t n_fallback;       /* states switched back to the diagonal step */
  int32_t pad;
  int64_t n_samples;        /* training samples added by this run */
} qpgpu_davidson_trace;

/* davidson_diag_hs2 / davidson_diag_hjj_sjj
 * (src/Davidson/diagonalization_hs2.irp.f:1-444) on the context's determinant
 * set, host arrays: u_in(dim_in, n_states_diag) column-major in psi_det order
 * holds ALL guess vectors (the reference draws the extra ones with
 * random_number, :188-200) and returns the eigenvectors; energies and s2_out
 * get n_states_diag entries (electronic energies, S^2 with the S_z(S_z-1)
 * shift).  H_jj is diag_H_mat_elem.  Returns the number of sigma
 * applications (> 0) or a negative status (QPGPU_ERR_DAVIDSON when a residual
 * exceeds 1e8, as the reference's 'Davidson failed'). */
int qpgpu_davidson_hs2(qpgpu_ctx* ctx, double* u_in, int64_t dim_in, double* energies, double* s2_out,
                       const qpgpu_davidson_params* params, qpgpu_davidson_trace* trace);

/* Learned Davidson preconditioner (no counterpart in the reference): an MLP
 * 8 -> 64 -> 64 -> 1 (GELU, FP32, 4801 parameters packed W1[64][8], b1[64],
 * W2[64][64], b2[64], W3[64], b3) that scales the diagonal correction of the
 * Davidson step per determinant.  Features (8 floats): alpha and beta
 * excitation rank / 4, (H_II - E)/10, hole/particle orbital-energy sum / 10,
 * log10(sum_J H_IJ^2)/4, log10|c_I|/8, log10|r_I|/8, log10|d_I|/8.  Samples are
 * (features, target multiplier g, weight w); the loss is mean(w (y - g)^2).
 * The training set and the parameters belong to the context and survive
 * qpgpu_set_dets (earlier determinant sets train later ones). */
#define QPGPU_MLP_NPARAM 4801
int qpgpu_mlp_init(qpgpu_ctx* ctx, uint64_t seed);
int qpgpu_mlp_set_weights(qpgpu_ctx* ctx, const float* w);
int qpgpu_mlp_get_weights(qpgpu_ctx* ctx, float* w);
int qpgpu_mlp_add_samples(qpgpu_ctx* ctx, const float* X, const float* g, const float* w, int64_t n);
int qpgpu_mlp_clear_samples(qpgpu_ctx* ctx);
int64_t qpgpu_mlp_n_samples(qpgpu_ctx* ctx);
int qpgpu_mlp_gradient(qpgpu_ctx* ctx, const float* X, const float* g, const float* w, int64_t n, float* grad,
                       float* loss);
int qpgpu_mlp_predict(qpgpu_ctx* ctx, const float* X, int64_t n, float* y);
int qpgpu_mlp_train(qpgpu_ctx* ctx, int epochs, int batch, float lr, uint64_t seed, float* loss);

/* Batches of independent CI problems (no counterpart in the reference, which
 * solves one problem per process).  A batch wraps contexts whose integrals
 * and determinants are set; sigma for all problems is one persistent launch
 * over a work queue of (problem, row chunk) items, the Davidson algebra of all
 * problems runs in batched kernels, the device part of each iteration is
 * replayed from CUDA graphs, and the persistent kernel's launch shape is
 * autotuned on the first call.  All problems must share S_z. */
typedef struct qpgpu_batch qpgpu_batch;
typedef struct qpgpu_batch_stats {
  int32_t n_iter;              /* Davidson iterations (all problems advance together) */
  int32_t n_sigma_launches;    /* persistent sigma launches */
  int32_t n_converged;         /* problems that met the threshold */
  int32_t tuned_warps;         /* chosen warps per block of the persistent sigma */
  int32_t tuned_blocks_per_sm; /* chosen resident blocks per SM */
  int32_t pad;
  double elapsed_ms;           /* device time of the iterations */
  double tune_ms;              /* time spent by the autotuner (first call) */
  int32_t* iters;              /* optional [n]: iterations of each problem */
} qpgpu_batch_stats;
int qpgpu_batch_create(qpgpu_ctx* const* ctxs, int n, qpgpu_batch** out);
int qpgpu_batch_destroy(qpgpu_batch* batch);
const char* qpgpu_batch_last_error(qpgpu_batch* batch);
/* davidson_diag_hjj_sjj (diagonalization_hs2.irp.f:52-444) on every problem:
 * u_in[p] host (dim_in[p], n_states_diag) guesses in psi_det order, replaced
 * by the eigenvectors; energies and s2_out: n x n_states_diag (row p for
 * problem p); n_states[p] <= params->n_states_diag; diagonal step only. */
int qpgpu_batch_davidson(qpgpu_batch* batch, double* const* u_in, const int64_t* dim_in, const int* n_states,
                         double* energies, double* s2_out, const qpgpu_davidson_params* params,
                         qpgpu_batch_stats* stats);

/* psi_bilinear_matrix_order (spindeterminants.irp.f:387-445), 0-based, host:
 * order[k] = psi_det index of bilinear position k. */
int qpgpu_bilinear_order(qpgpu_ctx* ctx, int32_t* order);

/* H_jj(i) = diag_H_mat_elem(psi_det(:,:,i)) (davidson_diag_hs2,
 * src/Davidson/diagonalization_hs2.irp.f:37-45) and diag_S_mat_elem, host,
 * psi_det order.  Either pointer may be NULL. */
int qpgpu_diag(qpgpu_ctx* ctx, double* h_jj, double* s_jj);

/* Debug export of the connected pairs sigma visits, host, psi_det indices
 * (0-based): class 1 alpha single, 2 beta single, 3 alpha double, 4 beta
 * double, 5 alpha-beta double; phase +1/-1; exc = (h1,p1,h2,p2) 1-based
 * (get_mono/double_excitation_spin, slater_rules.irp.f:2783-2987; for class 5
 * alpha (h,p) then beta (h,p)); hij = FP64 <I|H|J>.  *n_pairs returns the
 * total; at most `cap` records are written (pass cap = 0 to query). */
int qpgpu_connected_pairs(qpgpu_ctx* ctx, int64_t* n_pairs, int32_t* I, int32_t* J, int8_t* cls,
                          int8_t* phase, int16_t* exc, double* hij, int64_t cap);

/* The same export for selected determinants only: the records of
 * qpgpu_connected_pairs whose I is one of rows[0..n_rows) (0-based psi_det
 * indices; a repeated index counts once), for spot checks of large sets where
 * the full list does not fit in host memory.  *n_pairs returns the count; at
 * most `cap` records are written (cap = 0 queries).  Same routines as above
 * (slater_rules.irp.f:2783-2987). */
int qpgpu_connected_pairs_rows(qpgpu_ctx* ctx, const int32_t* rows, int64_t n_rows, int64_t* n_pairs, int32_t* I,
                               int32_t* J, int8_t* cls, int8_t* phase, int16_t* exc, double* hij, int64_t cap);

/* O = [A_0 .. A_nb-1] C for tall blocks A_b (N x nsd, rows nsd doubles
 * apart, blocks sA doubles apart; m = nb nsd) and C (m x nsd, row-major),
 * device arrays, computed to FP64 accuracy on the tensor cores.  These are
 * the Davidson's linear combinations: the Ritz vectors and the re-contraction
 * (src/Davidson/diagonalization_hs2.irp.f:376-381,419-420, dgemm('N','N'))
 * and the Gram-Schmidt updates.  Each row of A gets the exponent of its
 * largest value and each column of C its own; the digit products are summed
 * exactly, as in qpgpu_gram_tc.  The error of an entry is within a few
 * 2^-56 of max|a_r| max|c_j| (norm-wise, at or below FP64's rounding of the
 * largest product); an entry far below that scale has a larger relative
 * error than an FP64 dot product would give it.  O (rows ldO doubles apart)
 * may be the last block of A.  m <= 128, nsd <= 16.  The call waits for the stream (NULL:
 * the context's); a bounded tensor-core wait that runs out gives
 * QPGPU_ERR_TIMEOUT. */
int qpgpu_lincomb_tc(qpgpu_ctx* ctx, const double* A, int64_t sA, int m, int nsd, const double* C, double* O,
                     int64_t ldO, int64_t N, void* stream);

/* CIPSI selection with the Epstein-Nesbet second-order energy over the
 * context's wave function, which must be in psi_det_sorted order: the
 * generators are determinants 0..n_gen-1 and the selectors 0..n_sel-1
 * (1 <= n_gen <= n_sel <= N_det).  Replaces select_connected and the walk it
 * drives (plugins/Full_CI_ZMQ/selection.irp.f:24-79, :258-1172).  Holes are
 * every occupied orbital of a generator and particles every empty one (the
 * full generators_bitmask of Full_CI).  coef (N_det, n_st) is column-major
 * (psi_coef_sorted) and e0 (n_st) holds the denominators (pt2_E0_denominator,
 * electronic).  Every determinant a outside the wave function within a double
 * excitation of a generator is counted once, by the first generator that
 * reaches it, with the numerators mat(st) = sum over the selectors of
 * c_D,st <a|H|D>.  Each such a with a non-zero numerator adds
 * e = (sign(d) sqrt(d^2 + 4 mat^2) - d) / 2 (d = e0 - H_aa,
 * fill_buffer_double, :582-645) to pt2 (n_st).  The buffer keeps the
 * buf_size most negative values min(0, min_st e) (selection_buffer.irp.f),
 * ascending, ties in determinant-bit order, with their determinants
 * (N_int, 2) each in buf_dets.  *n_ext returns the number of external
 * determinants with a non-zero numerator.  1 <= n_st <= 8.  Returns the
 * number of buffer entries written (>= 0) or a negative status. */
int qpgpu_select_pt2(qpgpu_ctx* ctx, const double* coef, int n_st, const double* e0, int n_gen, int n_sel,
                     int buf_size, double* pt2, uint64_t* buf_dets, double* buf_vals, int64_t* n_ext);

/* The second-order energy of each listed generator separately (pt2_detail of
 * the stochastic PT2, plugins/Full_CI_ZMQ/pt2_stoch_routines.irp.f:6-155,
 * which runs select_connected on sampled generators).  gens[0..n_list) are
 * 0-based psi_det indices below n_sel.  Generator g gets the contributions
 * of the external determinants it reaches first: the same rules and
 * arguments as qpgpu_select_pt2, with every generator before g banning,
 * listed or not.  pt2_detail is (n_list, n_st) row-major (state fastest).
 * The comb sampling that picks the generators is host logic. */
int qpgpu_pt2_generators(qpgpu_ctx* ctx, const double* coef, int n_st, const double* e0, int n_sel,
                         const int32_t* gens, int n_list, double* pt2_detail);

#ifdef __cplusplus
}
#endif

#endif /* QPGPU_H */
