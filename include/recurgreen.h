/*
 * recurgreen.h -- C ABI of the GB300-native recursive Green-function sweep.
 *
 * A drop-in for the `waveguide` module of RecurGreen (src/waveguide.f90): the
 * same ten waveguide parameters, one transmission computation per disorder
 * realization, the transmission-eigenvalue distribution task, and the
 * full-Green-function methods (profiles, deposition, wavefunction).  Every entry
 * point takes plain pointers and sizes; all arithmetic is IEEE double /
 * double complex (complex values are interleaved (re, im) pairs, matrices are
 * column-major with leading dimension = number of rows, as in Fortran).
 *
 * Error convention: every call returns an int status (RG_OK == 0).  The
 * reference prints a message and stops the process (src/base_utils.f90:56-57,
 * src/waveguide.f90:91-142,408-421); here the message is kept in a
 * thread-local buffer returned by rg_last_error() and the caller decides.
 *
 * Threading: a handle, like a Fortran `waveguide_t` object, is not shared
 * between host threads (src/main.f90:148-150 gives each OpenMP thread its own
 * copy).  Each handle owns one CUDA stream and its device buffers.
 */
#ifndef RECURGREEN_H
#define RECURGREEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define RG_OK 0
#define RG_ERR_INVALID_ARG 1  /* stop errmsg_invalid_arg in the reference */
#define RG_ERR_SINGULAR 2     /* zgetrf info > 0 / zero or NaN pivot */
#define RG_ERR_CUDA 3         /* CUDA runtime failure (message has details) */
#define RG_ERR_NOMEM 4        /* host or device allocation failed */
#define RG_ERR_NOCONV 5       /* singular-value iteration did not converge */

/* Transverse boundary conditions (src/waveguide.f90:150-236). */
#define RG_BOUND_DIRICHLET 0
#define RG_BOUND_PERIODIC 1

/* The `&waveguide` namelist (src/main.f90:83), plus `ny`: the number of
 * transverse grid points.  ny == 0 keeps the reference's ny = nmu
 * (src/waveguide.f90:162,202). */
typedef struct rg_params {
  int boundtype; /* RG_BOUND_DIRICHLET or RG_BOUND_PERIODIC */
  int nxdiso;    /* slices in the disordered region */
  int nxfree;    /* free slices on each side */
  double wol;    /* W / lambda */
  double exfac;  /* mode-basis extension factor, in [1, 1e4] */
  double aratio; /* L / W */
  double dscat;  /* L / l_scat */
  double dabso;  /* L / l_abso */
  double napera; /* fraction of controlled modes (input port a), in (0, 1] */
  double naperb; /* fraction of observed modes (output port b), in (0, 1] */
  int ny;        /* transverse grid points; 0 => nmu */
} rg_params;

typedef struct rg_waveguide rg_waveguide;

/* Message of the last failing call on this host thread ("" if none). */
const char* rg_last_error(void);

/* init_waveguide (src/waveguide.f90:81-255): validates the parameters and
 * builds the mode set, mumesh, dos and the B diagonal on the current CUDA
 * device.  Warnings the reference prints (Shannon limit, weak disorder) are
 * not errors here either. */
int rg_init(const rg_params* params, rg_waveguide** out);

/* init_copy_waveguide (src/waveguide.f90:262-270). */
int rg_init_copy(const rg_waveguide* src, rg_waveguide** out);

/* del_waveguide (src/waveguide.f90:275-286).  Accepts NULL. */
void rg_del(rg_waveguide* wg);

/* Getters: get_nmu, get_neigv, get_nx (src/waveguide.f90:291-320), plus the
 * derived sizes the reference keeps private (ny, nprop and the filtering
 * window imin..imax x jmin..jmax, 1-based as in Fortran). */
int rg_get_nmu(const rg_waveguide* wg);
int rg_get_neigv(const rg_waveguide* wg);
int rg_get_nx(const rg_waveguide* wg);
int rg_get_ny(const rg_waveguide* wg);
int rg_get_nprop(const rg_waveguide* wg);
int rg_get_window(const rg_waveguide* wg, int* imin, int* imax, int* jmin, int* jmax);
/* get_xmesh (src/waveguide.f90:325-329): len must equal nx. */
int rg_get_xmesh(const rg_waveguide* wg, double* xmesh, int64_t len);
/* get_parameters (src/waveguide.f90:335-350). */
int rg_get_parameters(const rg_waveguide* wg, rg_params* out);
/* Internal scalars of the reference object: kdx, dos and the standard
 * deviation stdu of the dimensionless potential (src/waveguide.f90:118,243,370). */
int rg_get_scalars(const rg_waveguide* wg, double* kdx, double* dos, double* stdu);

/* The mode set's direction cosines mumesh and the diagonal of B
 * (src/waveguide.f90:240-248), nmu complex values each (either may be NULL). */
int rg_get_modes(const rg_waveguide* wg, double* mumesh, double* bmat);

/* compute_tdistrib (src/waveguide.f90:392-462): draws the disorder of seed
 * `iseed`, runs the recursive Green sweep on the GPU, and writes the neigv
 * transmission eigenvalues (descending) into chunk iseed of the host array
 * tallvals[len].  Same checks as the reference: len must be a positive
 * multiple of neigv and 1 <= iseed <= len / neigv. */
int rg_compute_tdistrib(rg_waveguide* wg, int iseed, double* tallvals, int64_t len);

/* compute_refl_trans_v1 (src/waveguide.f90:469-519): full nmu x nmu
 * transmission matrix t (and, if rmat != NULL, reflection matrix r) of seed
 * iseed, Fisher-Lee with sqrt(real(mu)).  Host buffers of nmu*nmu complex
 * doubles, column-major.  r comes from a second sweep over the slices in
 * reverse order (its last Gss is G(x_1; x_1)), instead of the reference's two
 * extra matrix products per slice. */
int rg_compute_refl_trans_v1(rg_waveguide* wg, int iseed, double* rmat, double* tmat);

/* compute_refl_trans_v1 for many seeds (the loop of the tpattern task,
 * src/main.f90:796-830): for k < n, t and r of seed seeds[k] go to
 * tmat + 2*k*nmu*nmu and rmat + 2*k*nmu*nmu (host, column-major complex;
 * rmat may be NULL).  The realizations run in batched launches of bounded
 * device memory.  status[k] (may be NULL) receives each realization's status;
 * returns the first non-OK one after all have run. */
int rg_refl_trans_v1_batch(rg_waveguide* wg, const int32_t* seeds, int n, double* rmat, double* tmat,
                           int32_t* status);

/* ------------------------------------------------------------------------
 * Full Green function (src/waveguide.f90:636-997).  The reference solves the
 * whole block tridiagonal system (solve_block_tridiag,
 * src/base_utils.f90:296-335) and keeps G(x_n; x_s) for every slice.  Here a
 * forward sweep keeps each slice's (S_n, Z_n), and the backward pass runs
 * only on the source vectors a result needs.  Positions are 1-based slice
 * indices, as in the reference.
 * ------------------------------------------------------------------------ */

/* Profile kinds of rg_tprofile_batch:
 *   RG_PROFILE_TPROFILE  compute_tprofile (src/waveguide.f90:843-907): the
 *                        eigenvectors of t^H t (full nmu x nmu t) with
 *                        a[w] <= T <= b[w], profile times 4/nt (nt != 0);
 *   RG_PROFILE_ITX       compute_itx_profile (src/waveguide.f90:764-825): the
 *                        same selection, times 2/(pi wol |b[w]-a[w]|);
 *   RG_PROFILE_GROUP     compute_tprofile_group (src/waveguide.f90:924-997):
 *                        t filtered to imin..imax x jmin..jmax, eigenvectors
 *                        with |T - a[w]| <= b[w], times 4/nt (nt != 0). */
#define RG_PROFILE_TPROFILE 0
#define RG_PROFILE_ITX 1
#define RG_PROFILE_GROUP 2

/* Transmission-eigenstate profiles of n realizations: for seed seeds[k] and
 * window w < nprofile, profiles[(k*nprofile + w)*nx + ix] (the reference's
 * tprofiledata(nx, nprofile, nseed) layout), nt[k*nprofile + w] eigenvalues
 * in the window and tavg[k] = sum(T)/ncol (the group's Tavg).  Host
 * pointers; nt, tavg and status may be NULL.  The window bounds are checked
 * as the reference checks them.  Returns the first non-OK status after all
 * realizations have run. */
int rg_tprofile_batch(rg_waveguide* wg, const int32_t* seeds, int n, int kind, int nprofile, const double* a,
                      const double* b, double* profiles, int32_t* nt, double* tavg, int32_t* status);

/* The reference's single-realization methods on top of it. */
int rg_compute_tprofile(rg_waveguide* wg, int iseed, double tmin, double tmax, double* tprofile, int64_t len,
                        int* nt);
int rg_compute_itx_profile(rg_waveguide* wg, int iseed, double tmin, double tmax, double* itx, int64_t len);
int rg_compute_tprofile_group(rg_waveguide* wg, int iseed, int nprofile, const double* tm, const double* dt,
                              double* tprofile, int64_t len, int32_t* nt, double* tavg);

/* compute_deposition (src/waveguide.f90:710-745): depmat = 2i sqrt(real(mu))
 * G(x_fpos; x_ipos) sqrt(real(mu)), nmu x nmu complex, column-major (host). */
int rg_compute_deposition(rg_waveguide* wg, int iseed, int fpos, int ipos, double* depmat);

/* Deposition for n realizations (the deposition branch of the tpattern
 * task, src/main.f90:804-809): col in 1..nmu gives column col of each
 * realization's depmat (out + 2*k*nmu), col == 0 the whole matrix
 * (out + 2*k*nmu*nmu).  Host pointers; status may be NULL. */
int rg_deposition_batch(rg_waveguide* wg, const int32_t* seeds, int n, int fpos, int ipos, int col, double* out,
                        int32_t* status);

/* compute_refl_trans_v2 (src/waveguide.f90:526-553): t and r (r may be NULL)
 * from the full block tridiagonal solve with the identity source at slice 1,
 * t = 2i sqrt(real(mu)) G(x_nx; x_1) sqrt(real(mu)) and
 * r = -1 + 2i sqrt(real(mu)) G(x_1; x_1) sqrt(real(mu)); nmu x nmu complex,
 * column-major (host).  The reference's cross-check of v1 (its
 * test_green_v1_v2, src/waveguide.f90:598-623). */
int rg_compute_refl_trans_v2(rg_waveguide* wg, int iseed, double* rmat, double* tmat);

/* compute_wavefunction (src/waveguide.f90:636-698): the field of a unit
 * source in mode imode at slice ipos, as the (nx*ny) x 5 table [x, y, Re psi,
 * Im psi, upot] (host, column-major; rows = nx*ny). */
int rg_compute_wavefunction(rg_waveguide* wg, int iseed, int ipos, int imode, double* wfundata, int64_t rows);

/* diagonalize_ahca (src/base_utils.f90:394-444) on the GPU: the eigenvalues
 * T[n] (descending) and eigenvectors U (n x n, column-major, same order) of
 * A^H A for the m x n complex matrix a (column-major).  One-sided Jacobi with
 * accumulated rotations instead of zgesvd; eigenvectors are defined up to a
 * phase (and within degenerate eigenspaces). */
int rg_diagonalize_ahca(const double* a, int m, int n, double* T, double* U);

/* As rg_compute_tdistrib / rg_compute_refl_trans_v1, but for a caller-given
 * potential upot(nxdiso, ny) (host, column-major: x fastest), already scaled
 * by stdu as set_hamiltonian_waveguide stores it (src/waveguide.f90:366-372).
 * teigvals receives neigv values; tfilt, if not NULL, the filtered Fisher-Lee
 * t of tdistrib ((imax-imin+1) x (jmax-jmin+1) complex, column-major). */
int rg_tdistrib_upot(rg_waveguide* wg, const double* upot, double* teigvals, double* tfilt);
int rg_refl_trans_v1_upot(rg_waveguide* wg, const double* upot, double* rmat, double* tmat);

/* The potential of seed iseed as the GPU draws it (host output, nxdiso*ny
 * doubles, column-major), for inspection and tests. */
int rg_potential(rg_waveguide* wg, int iseed, double* upot);

/* Batched tdistrib (the OpenMP seed loop of src/main.f90:134-179, as one
 * persistent launch): realization k uses seed seeds[k] and writes its neigv
 * eigenvalues to tallvals[k*neigv ...].  Host pointers; status[k] (may be
 * NULL) receives the per-realization status.  Returns the first non-OK
 * status, after every realization has run. */
int rg_tdistrib_batch(rg_waveguide* wg, const int32_t* seeds, int n, double* tallvals, int32_t* status);

/* Same on device pointers, enqueued on `stream` (a cudaStream_t; NULL means
 * the handle's own stream).  Synchronises the stream before returning. */
int rg_tdistrib_batch_device(rg_waveguide* wg, const int32_t* d_seeds, int n, double* d_tallvals,
                             int32_t* d_status, void* stream);

/* Batched tdistrib over several waveguides at once (realizations of guides
 * of uneven size; the reference would run one OpenMP seed loop per guide,
 * src/main.f90:134-179): item k is realization seeds[k] of waveguide wgs[k],
 * and its neigv eigenvalues (descending) go to tallvals[offsets[k] ...],
 * which must lie inside tallvals[len].  Host arrays.  Items are grouped by
 * kernel class (up to 16, 32, 64 modes, more), ordered by decreasing cost
 * within a group, and each group runs as one persistent launch on wgs[0]'s
 * stream; all handles must share a device.  status[k] (may be NULL) gets the
 * per-item status; the first non-OK status is returned after all items ran. */
int rg_tdistrib_multi(rg_waveguide* const* wgs, const int32_t* seeds, int n, const int64_t* offsets,
                      double* tallvals, int64_t len, int32_t* status);

/* Adjoint support (no counterpart in the reference, whose FP64 path has no
 * gradients).  Device pointers; work is enqueued on `stream` taken literally
 * (0 is CUDA's default stream, as frameworks pass it), no synchronisation.
 *
 * rg_sweep_segment runs the recursion of n realizations over slices
 * [n_begin, n_end) on caller-given potentials d_upot (n x nxdiso x ny,
 * C order), starting from d_state_in (n x 2 x nmu x nmu complex, row-major:
 * Gss then Gs1 after slice n_begin-1; NULL exactly when n_begin == 0).  It
 * writes the state after every slice to d_state_dump (n x (n_end-n_begin) x
 * 2 x nmu x nmu, optional) and after the last one to d_state_out (optional).
 * When n_end == nx it also forms the filtered Fisher-Lee t (d_tfilt,
 * n x ncol x nrow complex, i.e. column-major per realization, optional) and
 * the eigenvalues (d_teig, n x neigv).  This is the forward recomputation
 * from checkpoints of the adjoint sweep.
 *
 * rg_adjoint_grad_rows turns the adjoints Xbar = dL/dX* of n slice matrices
 * (n x nmu x nmu complex, row-major) into the potential gradients
 * dL/dU(n, :) = -2 sum Re(Xbar[a][c]) chi_a chi_c, n rows of ny doubles
 * grad_stride apart (Dirichlet guides). */
int rg_sweep_segment(rg_waveguide* wg, const double* d_upot, int n, int n_begin, int n_end,
                     const double* d_state_in, double* d_state_dump, double* d_state_out, double* d_tfilt,
                     double* d_teig, int32_t* d_status, void* stream);
int rg_adjoint_grad_rows(rg_waveguide* wg, const double* d_xbar, int n, double* d_grad, int64_t grad_stride,
                         void* stream);

/* A whole sweep on caller-given potentials d_upot (n x nxdiso x ny, C order)
 * that keeps the state of every slice: d_states (n x nx x 2 x nmu x nmu
 * complex, row-major; NULL: none kept) receives (Gss, Gs1) after each slice, i.e. the
 * (S_n, Z_n) of solve_block_tridiag (src/base_utils.f90:318-324) for the
 * identity source at slice 1; d_tfilt (n x ncol x nrow complex, optional) the
 * filtered Fisher-Lee t, d_teig (n x neigv) the eigenvalues, d_status (n) the
 * statuses.  Dirichlet guides run the symmetric sweep.  Device pointers,
 * enqueued on `stream` (taken literally), which is synchronised before
 * returning.  The full-Green-function adjoint's forward pass. */
int rg_sweep_states(rg_waveguide* wg, const double* d_upot, int n, double* d_states, double* d_tfilt,
                    double* d_teig, int32_t* d_status, void* stream);

/* Tracing (the reference times its seed loop with date_and_time,
 * src/main.f90:145,174-176): device time in milliseconds of the sweep
 * launches of the last rg_tdistrib_batch[_device] call on this handle (one
 * kernel, or the symmetric kernel and its pivoted re-run), measured with CUDA
 * events recorded around them on their stream.  Fails before the first batch. */
int rg_last_sweep_time(rg_waveguide* wg, float* ms);

/* No counterpart in the reference.  The launch configuration of the last
 * rg_tdistrib_batch[_device] call on this handle: the sweep kernel that ran,
 * its grid, and how many realizations the symmetric kernel handed to the
 * pivoted kernel (their diagonal pivots fell below the threshold).  Waits for
 * that batch to finish.  rerun is valid until the next computation on the
 * handle. */
#define RG_KERNEL_PIVOTED 0   /* shared-memory Gauss-Jordan with implicit partial pivoting */
#define RG_KERNEL_SYMMETRIC 1 /* symmetric sweep (Dirichlet), pivoted re-run of flagged items */
#define RG_KERNEL_BLOCKED 2   /* blocked global-memory kernel, `cluster` CTAs per realization */
#define RG_KERNEL_BLOCKED_SYMMETRIC 3 /* blocked symmetric sweep (Dirichlet), blocked pivoted re-run */
typedef struct rg_batch_info {
  int kernel;  /* RG_KERNEL_* */
  int grid;    /* CTAs of the launch */
  int cluster; /* CTAs per realization */
  int rerun;   /* realizations re-run by the pivoted kernel */
} rg_batch_info;
int rg_last_batch_info(rg_waveguide* wg, rg_batch_info* info);

/* No counterpart in the reference.  One seed's transmission eigenvalues, as
 * rg_compute_tdistrib computes them, for callers that cannot allocate device
 * memory when they need the result: hosts whose device memory is handed to
 * their own pool allocator, and loops that must not take cudaMalloc's
 * implicit synchronisation.  The call allocates nothing:
 * create the handle with rg_init at set-up, then call this with device
 * buffers d_teigvals[neigv] and d_status[1]; work is enqueued on `stream`
 * (NULL: the handle's stream) and the call returns without synchronising.
 * The potential is drawn into a fixed 16 MiB device array of the library,
 * shared by all calls, so nxdiso*ny may be at most 2,097,120 (above 64 modes
 * the elimination matrices, about 64*nmu^2 bytes, share the array too);
 * larger guides get RG_ERR_INVALID_ARG.  The handle's device must be current; the first
 * call on each device looks the array up (make it before any stream capture).
 * Calls that overlap on the GPU race on the shared array.  iseed must be >= 1.
 * The array's address is kept per device index for the life of the process:
 * do not call this after the device was reset (cudaDeviceReset). */
int rg_tdistrib_seed_noalloc(rg_waveguide* wg, int iseed, double* d_teigvals, int32_t* d_status, void* stream);

/* No counterpart in the reference: throughput of one arithmetic pipe of the
 * current device, in TFLOP/s, from a full grid of independent dependency
 * chains on register operands (the denominators of the sweep's roofline).
 * kind 0: FP64 FMA; 1: FP64 mma.sync m8n8k4; 2: FP64 mma.sync m16n8k16;
 * 3: FP16 mma.sync m16n8k16 with FP32 accumulation; 4: FP32 FMA.  iters is
 * the loop count per thread (about 1e5 gives ~0.1 s for kind 0). */
int rg_probe_rate(int kind, int iters, double* tflops);

/* No counterpart in the reference: C = A B for M x M complex matrices (host,
 * column-major, 1 <= M <= 512) through the tensor-core path the blocked
 * symmetric sweep uses for its propagator product Gss (B Gs1): each row of A
 * and column of B is cut into six balanced 9-bit digits of a 53-bit fixed
 * point, 26 digit-pair products run as FP16 mma.sync with exact FP32 level
 * sums, and an exact int64 fold gives C rounded once -- FP64 accuracy
 * (normwise at an FP64 product's level).  For tests and measurements. */
int rg_ozaki_zgemm(int M, const double* a, const double* b, double* c);

/* No counterpart in the reference (the adjoint's per-slice products): for
 * k < nbatch,
 *     C_k = alpha * op(A_k) diag(s) op(B_k) + beta * D_k
 * with M x M complex matrices (1 <= M <= 512) on the device, through the same
 * tensor-core path as rg_ozaki_zgemm.  Operand X of item k is the matrix at
 * x + (k % mod_x) * stride_x (complex elements; mod_x <= 0 means nbatch), so
 * an operand can be shared by several items; op 0 = X, 1 = X^T, 2 = X^H;
 * rowscale_b (M complex, may be NULL) is diag(s); D may be NULL when beta is
 * 0.  colmajor != 0: column-major matrices, else row-major (C order).  C may
 * alias A, B or D.  workspace (device, 16-byte aligned) holds at least
 * rg_zgemm_workspace_bytes(M, nbatch) bytes; the call allocates nothing and
 * enqueues three kernels on `stream` (taken literally), without
 * synchronising. */
int64_t rg_zgemm_workspace_bytes(int M, int nbatch);
int rg_zgemm_batched(int M, int nbatch, const double* a, int64_t stride_a, int mod_a, int op_a, const double* b,
                     int64_t stride_b, int mod_b, int op_b, const double* rowscale_b, double alpha_re,
                     double alpha_im, const double* d, int64_t stride_d, int mod_d, double beta, double* c,
                     int64_t stride_c, int colmajor, void* workspace, int64_t workspace_bytes, void* stream);

/* histogram (src/base_utils.f90:491-516) with the reference's exact edge
 * semantics, computed on the GPU: samples[n] and bins[nbins+1] are host
 * arrays; histo[nbins] and *missing receive counts as doubles. */
int rg_histogram(const double* samples, int64_t n, const double* bins, int nbins, double* histo,
                 double* missing);

#ifdef __cplusplus
}
#endif

#endif /* RECURGREEN_H */
