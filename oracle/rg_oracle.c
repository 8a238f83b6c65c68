/*
 * CPU oracle for the recursive Green-function sweep of RecurGreen.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference Fortran algorithm, used as the parity checker by tests/, by
 * __graft_entry__.smoke() and as the CPU baseline leg of bench.py.  Nothing in
 * the product library (recurgreen_gb300/) links, loads or calls it.
 *
 * Every routine cites the reference file:line it follows (paths relative to
 * the RecurGreen project root).  Dense linear algebra goes through the same
 * LAPACK routines the reference calls (zgetrf, zgetri, zgesvd, plus zgemm in
 * place of gfortran's intrinsic matmul), resolved at run time with dlopen()
 * from an LP64 OpenBLAS build (the one bundled with scipy), because the image
 * has no system LAPACK.  LAPACK is not pinned by the reference
 * (Makefile:27 links "-lblas -llapack" with no version).
 *
 * The Gaussian random numbers follow src/random_normal.f90:20-67: an ANSI-C
 * LCG fills the seed array of gfortran's random_seed(put=), the uniforms come
 * from gfortran's random_number, and Box-Muller makes the normals.  gfortran's
 * generator since GCC 9 is xoshiro256** (Blackman & Vigna) seeded by the
 * 8-word put array XOR-scrambled into the 256-bit state; it is restated here.
 * No gfortran >= 9 runtime exists in this image to pin that restatement, so
 * potential-level parity with binaries built by the reference is UNPINNED; the
 * parity tests feed the same potential to the oracle and the GPU path instead.
 */
#include <complex.h>
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_SINGULAR 2
#define ORC_ERR_LAPACK 3
#define ORC_ERR_NOMEM 4

static const double PI = 3.14159265358979323846264338327950288;

/* ------------------------------------------------------------------------ */
/* LAPACK / BLAS through dlopen (Fortran ABI, 32-bit integers).             */
/* ------------------------------------------------------------------------ */
typedef void (*zgetrf_fn)(const int*, const int*, cplx*, const int*, int*, int*);
typedef void (*zgetri_fn)(const int*, cplx*, const int*, const int*, cplx*, const int*, int*);
typedef void (*zgesvd_fn)(const char*, const char*, const int*, const int*, cplx*, const int*,
                          double*, cplx*, const int*, cplx*, const int*, cplx*, const int*,
                          double*, int*, size_t, size_t);
typedef void (*zgemm_fn)(const char*, const char*, const int*, const int*, const int*,
                         const cplx*, const cplx*, const int*, const cplx*, const int*,
                         const cplx*, cplx*, const int*, size_t, size_t);
typedef void (*setthreads_fn)(int);

static zgetrf_fn p_zgetrf;
static zgetri_fn p_zgetri;
static zgesvd_fn p_zgesvd;
static zgemm_fn p_zgemm;
static char g_err[512];

const char* orc_last_error(void) { return g_err; }

static void* sym2(void* h, const char* prefix, const char* name) {
  char buf[128];
  snprintf(buf, sizeof buf, "%s%s", prefix, name);
  return dlsym(h, buf);
}

/* Load LAPACK from the shared library at `path`; symbol names are
 * `<prefix>zgetrf_` etc. (prefix "scipy_" for scipy's OpenBLAS). */
int orc_load_lapack(const char* path, const char* prefix) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    snprintf(g_err, sizeof g_err, "dlopen(%s) failed: %s", path, dlerror());
    return ORC_ERR_LAPACK;
  }
  p_zgetrf = (zgetrf_fn)sym2(h, prefix, "zgetrf_");
  p_zgetri = (zgetri_fn)sym2(h, prefix, "zgetri_");
  p_zgesvd = (zgesvd_fn)sym2(h, prefix, "zgesvd_");
  p_zgemm = (zgemm_fn)sym2(h, prefix, "zgemm_");
  if (!p_zgetrf || !p_zgetri || !p_zgesvd || !p_zgemm) {
    snprintf(g_err, sizeof g_err, "LAPACK symbols with prefix '%s' missing in %s", prefix, path);
    return ORC_ERR_LAPACK;
  }
  /* One BLAS thread per caller: the oracle parallelises over seeds. */
  setthreads_fn st = (setthreads_fn)sym2(h, prefix, "openblas_set_num_threads");
  if (!st) st = (setthreads_fn)dlsym(h, "scipy_openblas_set_num_threads");
  if (!st) st = (setthreads_fn)dlsym(h, "openblas_set_num_threads");
  if (st) st(1);
  return ORC_OK;
}

static int need_lapack(void) {
  if (!p_zgetrf) {
    snprintf(g_err, sizeof g_err, "LAPACK not loaded (call orc_load_lapack first)");
    return ORC_ERR_LAPACK;
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Random numbers: src/random_normal.f90                                    */
/* ------------------------------------------------------------------------ */

/* randi_ansic, src/random_normal.f90:20-31: s <- 1103515245*s + 12345 with
 * 32-bit two's-complement wrap-around. */
void orc_randi_ansic(int32_t* out, int n, int32_t seed) {
  uint32_t s = (uint32_t)seed;
  for (int i = 0; i < n; ++i) {
    s = 1103515245u * s + 12345u;
    out[i] = (int32_t)s;
  }
}

/* gfortran (GCC >= 9) runtime generator: xoshiro256** state seeded by
 * random_seed(put=seed(1:8)).  The put array is read last-element-first into
 * four 64-bit words which are XORed with fixed keys. */
typedef struct { uint64_t s[4]; } orc_xoshiro;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xoshiro_next(orc_xoshiro* st) {
  uint64_t* s = st->s;
  const uint64_t result = rotl64(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return result;
}

void orc_gfortran_seed(orc_xoshiro* st, const int32_t put[8]) {
  static const uint64_t keys[4] = {0xbd0c5b6e50c2df49ULL, 0xd46061cd46e1df38ULL,
                                   0xbb4f4d4ed6103544ULL, 0x114a583d0756ad39ULL};
  uint32_t w[8];
  for (int i = 0; i < 8; ++i) w[i] = (uint32_t)put[7 - i];
  for (int i = 0; i < 4; ++i) {
    uint64_t v = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
    st->s[i] = v ^ keys[i];
  }
}

/* random_number for real(8): top 53 bits of the 64-bit draw times 2^-53. */
static inline double gfortran_uniform(orc_xoshiro* st) {
  return (double)(xoshiro_next(st) >> 11) * 0x1.0p-53;
}

/* rand_normal, src/random_normal.f90:40-67. */
void orc_rand_normal(double* out, int64_t n, int32_t seed) {
  int32_t seedarr[8];
  orc_randi_ansic(seedarr, 8, seed);
  orc_xoshiro st;
  orc_gfortran_seed(&st, seedarr);
  for (int64_t i = 0; i < n; ++i) {
    double u1 = gfortran_uniform(&st);
    double u2 = gfortran_uniform(&st);
    out[i] = sqrt(-2.0 * log(u1)) * cos(2.0 * PI * u2);
  }
}

/* ------------------------------------------------------------------------ */
/* Waveguide: src/waveguide.f90:13-255                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  int boundtype; /* 0 dirichlet, 1 periodic */
  int nxdiso, nxfree, nx, ny, nmu, imin, imax, jmin, jmax, nprop, neigv;
  double wol, exfac, aratio, dscat, dabso, napera, naperb, kdx, dos, stdu;
  double* xmesh;  /* nx */
  double* ymesh;  /* ny */
  double* kpmesh; /* nmu */
  cplx* mumesh;   /* nmu */
  cplx* modal;    /* ny x nmu, column-major */
  cplx* bmat;     /* nmu */
  cplx* adiag_edge; /* nmu: i*mu - mu/tan(mu*kdx), src/waveguide.f90:357 */
  cplx* adiag_bulk; /* nmu: -2*mu/tan(mu*kdx), src/waveguide.f90:359 */
} orc_wg;

void orc_free(orc_wg* w) {
  if (!w) return;
  free(w->xmesh); free(w->ymesh); free(w->kpmesh); free(w->mumesh);
  free(w->modal); free(w->bmat); free(w->adiag_edge); free(w->adiag_bulk);
  free(w);
}

/* init_waveguide, src/waveguide.f90:81-255.  `ny_override` > 0 replaces the
 * reference's ny = nmu (src/waveguide.f90:162,202). */
int orc_init(int boundtype, int nxdiso, int nxfree, double wol, double exfac, double aratio,
             double dscat, double dabso, double napera, double naperb, int ny_override,
             orc_wg** out) {
  const double eps = 2.220446049250313e-16;
  *out = NULL;
  if (wol < eps) { snprintf(g_err, sizeof g_err, "Invalid width-to-wavelength ratio."); return ORC_ERR_ARG; }
  if (aratio < eps) { snprintf(g_err, sizeof g_err, "Invalid aspect ratio."); return ORC_ERR_ARG; }
  if (exfac < 1.0 || exfac > 1e4) { snprintf(g_err, sizeof g_err, "Invalid modal basis extension factor."); return ORC_ERR_ARG; }
  if (nxfree < 0) { snprintf(g_err, sizeof g_err, "Invalid number of x points, cannot be negative."); return ORC_ERR_ARG; }
  if (dscat < 0.0 || dabso < 0.0) { snprintf(g_err, sizeof g_err, "Invalid optical depth, cannot be negative."); return ORC_ERR_ARG; }
  if (napera <= 0.0 || napera > 1.0) { snprintf(g_err, sizeof g_err, "Invalid filtering parameter napera."); return ORC_ERR_ARG; }
  if (naperb <= 0.0 || naperb > 1.0) { snprintf(g_err, sizeof g_err, "Invalid filtering parameter naperb."); return ORC_ERR_ARG; }
  if (nxdiso < 1 || nxdiso + 2 * nxfree < 2) { snprintf(g_err, sizeof g_err, "Invalid number of x points."); return ORC_ERR_ARG; }

  orc_wg* w = (orc_wg*)calloc(1, sizeof(orc_wg));
  w->boundtype = boundtype;
  w->wol = wol; w->aratio = aratio; w->exfac = exfac;
  const double kl = 2.0 * PI * wol * aratio;
  w->nxdiso = nxdiso; w->nxfree = nxfree; w->nx = nxdiso + 2 * nxfree;
  w->kdx = kl / nxdiso;
  w->dscat = dscat; w->dabso = dabso; w->napera = napera; w->naperb = naperb;

  w->xmesh = (double*)malloc(sizeof(double) * w->nx);
  for (int i = 1; i <= w->nx; ++i) w->xmesh[i - 1] = aratio * (i - 0.5 - nxfree) / nxdiso;

  if (boundtype == 1) { /* periodic, src/waveguide.f90:151-189 */
    if (fmod(wol, 1.0) == 0.0) { snprintf(g_err, sizeof g_err, "Invalid width wol (integer) for periodic."); orc_free(w); return ORC_ERR_ARG; }
    w->nmu = 2 * (int)floor(exfac * wol) + 1;
    w->ny = ny_override > 0 ? ny_override : w->nmu;
    w->imin = w->nmu / 2 + 1 - (int)floor(naperb * wol);
    w->imax = w->nmu / 2 + 1 + (int)floor(naperb * wol);
    w->jmin = w->nmu / 2 + 1 - (int)floor(napera * wol);
    w->jmax = w->nmu / 2 + 1 + (int)floor(napera * wol);
    w->neigv = 2 * (int)floor(fmin(napera, naperb) * wol) + 1;
    w->nprop = 2 * (int)floor(wol) + 1;
  } else if (boundtype == 0) { /* dirichlet, src/waveguide.f90:191-229 */
    if (fmod(wol, 0.5) == 0.0) { snprintf(g_err, sizeof g_err, "Invalid width wol (half integer) for dirichlet."); orc_free(w); return ORC_ERR_ARG; }
    w->nmu = (int)floor(2 * exfac * wol);
    w->ny = ny_override > 0 ? ny_override : w->nmu;
    w->imin = 1;
    w->imax = (int)floor(2 * naperb * wol);
    w->jmin = 1;
    w->jmax = (int)floor(2 * napera * wol);
    w->neigv = (int)floor(2 * fmin(napera, naperb) * wol);
    w->nprop = (int)floor(2 * wol);
  } else {
    snprintf(g_err, sizeof g_err, "Unknown boundary condition type."); orc_free(w); return ORC_ERR_ARG;
  }
  const int nmu = w->nmu, ny = w->ny;
  if (nmu < 1) { snprintf(g_err, sizeof g_err, "No modes."); orc_free(w); return ORC_ERR_ARG; }
  w->ymesh = (double*)malloc(sizeof(double) * ny);
  for (int i = 1; i <= ny; ++i) w->ymesh[i - 1] = (i - 0.5) / ny;
  w->kpmesh = (double*)malloc(sizeof(double) * nmu);
  w->modal = (cplx*)malloc(sizeof(cplx) * ny * nmu);
  if (boundtype == 1) {
    for (int n = 1; n <= nmu; ++n) w->kpmesh[n - 1] = (n - nmu / 2 - 1) / wol;
    const double nrm = sqrt((double)ny);
    for (int n = 0; n < nmu; ++n)
      for (int i = 0; i < ny; ++i)
        w->modal[i + (size_t)ny * n] = cexp(I * (2 * PI * wol * w->kpmesh[n] * w->ymesh[i])) / nrm;
  } else {
    for (int n = 1; n <= nmu; ++n) w->kpmesh[n - 1] = 0.5 * n / wol;
    const double nrm = sqrt(2.0 / ny);
    for (int n = 0; n < nmu; ++n)
      for (int i = 0; i < ny; ++i)
        w->modal[i + (size_t)ny * n] = nrm * sin(2 * PI * wol * w->kpmesh[n] * w->ymesh[i]);
  }
  /* mumesh, dos, bmat: src/waveguide.f90:240-248 */
  w->mumesh = (cplx*)malloc(sizeof(cplx) * nmu);
  w->bmat = (cplx*)malloc(sizeof(cplx) * nmu);
  w->adiag_edge = (cplx*)malloc(sizeof(cplx) * nmu);
  w->adiag_bulk = (cplx*)malloc(sizeof(cplx) * nmu);
  double dos = 0.0;
  for (int n = 0; n < nmu; ++n) {
    const double kp = w->kpmesh[n];
    w->mumesh[n] = csqrt(CMPLX(1.0 - kp * kp, dabso / kl));
    dos += creal(1.0 / csqrt(CMPLX(1.0 - kp * kp, 0.0)));
  }
  w->dos = dos / (wol * (2.0 * PI) * (2.0 * PI));
  for (int n = 0; n < nmu; ++n) {
    const cplx mu = w->mumesh[n];
    w->bmat[n] = mu / csin(mu * w->kdx);
    const cplx cot = mu / ctan(mu * w->kdx);
    w->adiag_edge[n] = I * mu - cot;
    w->adiag_bulk[n] = -2.0 * cot;
  }
  /* standard deviation of upot, src/waveguide.f90:370 */
  w->stdu = sqrt(dscat * ny / (2.0 * PI * PI * w->dos * wol * nxdiso));
  *out = w;
  return ORC_OK;
}

int orc_get_int(const orc_wg* w, const char* key) {
  if (!strcmp(key, "nmu")) return w->nmu;
  if (!strcmp(key, "ny")) return w->ny;
  if (!strcmp(key, "nx")) return w->nx;
  if (!strcmp(key, "neigv")) return w->neigv;
  if (!strcmp(key, "nprop")) return w->nprop;
  if (!strcmp(key, "imin")) return w->imin;
  if (!strcmp(key, "imax")) return w->imax;
  if (!strcmp(key, "jmin")) return w->jmin;
  if (!strcmp(key, "jmax")) return w->jmax;
  return -1;
}

double orc_get_real(const orc_wg* w, const char* key) {
  if (!strcmp(key, "kdx")) return w->kdx;
  if (!strcmp(key, "dos")) return w->dos;
  if (!strcmp(key, "stdu")) return w->stdu;
  return NAN;
}

void orc_get_tables(const orc_wg* w, cplx* mumesh, cplx* bmat, cplx* adiag_edge, cplx* adiag_bulk) {
  memcpy(mumesh, w->mumesh, sizeof(cplx) * w->nmu);
  memcpy(bmat, w->bmat, sizeof(cplx) * w->nmu);
  memcpy(adiag_edge, w->adiag_edge, sizeof(cplx) * w->nmu);
  memcpy(adiag_bulk, w->adiag_bulk, sizeof(cplx) * w->nmu);
}

/* The potential upot(nxdiso, ny), column-major (x fastest), for seed iseed:
 * src/waveguide.f90:366-372. */
void orc_potential(const orc_wg* w, int32_t iseed, double* upot) {
  const int64_t n = (int64_t)w->ny * w->nxdiso;
  orc_rand_normal(upot, n, iseed);
  for (int64_t i = 0; i < n; ++i) upot[i] *= w->stdu;
}

/* ------------------------------------------------------------------------ */
/* Linear algebra helpers: src/base_utils.f90                               */
/* ------------------------------------------------------------------------ */

/* inverse_complex, src/base_utils.f90:235-274: zgetrf then zgetri with
 * lwork = n.  Returns ORC_ERR_SINGULAR on info != 0 (the reference stops). */
int orc_inverse_complex(cplx* a, int n) {
  if (need_lapack()) return ORC_ERR_LAPACK;
  int info = 0;
  int ipiv_stack[512];
  cplx work_stack[512];
  int* ipiv = n <= 512 ? ipiv_stack : (int*)malloc(sizeof(int) * n);
  cplx* work = n <= 512 ? work_stack : (cplx*)malloc(sizeof(cplx) * n);
  p_zgetrf(&n, &n, a, &n, ipiv, &info);
  int rc = ORC_OK;
  if (info != 0) {
    snprintf(g_err, sizeof g_err, "zgetrf: Matrix is numerically singular (LAPACK info=%d)", info);
    rc = ORC_ERR_SINGULAR;
  } else {
    p_zgetri(&n, a, &n, ipiv, work, &n, &info);
    if (info != 0) {
      snprintf(g_err, sizeof g_err, "zgetri: Matrix inversion failed (LAPACK info=%d)", info);
      rc = ORC_ERR_SINGULAR;
    }
  }
  if (ipiv != ipiv_stack) free(ipiv);
  if (work != work_stack) free(work);
  return rc;
}

/* singular_values, src/base_utils.f90:341-380: zgesvd('N','N').  `a` (m x n,
 * column-major) is destroyed; s receives min(m,n) values in descending order. */
int orc_singular_values(cplx* a, int m, int n, double* s) {
  if (need_lapack()) return ORC_ERR_LAPACK;
  const int mn = m < n ? m : n;
  int lwork = 2 * mn + (m > n ? m : n);
  if (lwork < 1) lwork = 1;
  cplx* work = (cplx*)malloc(sizeof(cplx) * lwork);
  double* rwork = (double*)malloc(sizeof(double) * 5 * (mn > 0 ? mn : 1));
  cplx u[1], vt[1];
  int info = 0, ldu = m, ldvt = n;
  p_zgesvd("N", "N", &m, &n, a, &m, s, u, &ldu, vt, &ldvt, work, &lwork, rwork, &info, 1, 1);
  free(work);
  free(rwork);
  if (info != 0) {
    snprintf(g_err, sizeof g_err, "zgesvd failed (LAPACK info=%d)", info);
    return ORC_ERR_LAPACK;
  }
  return ORC_OK;
}

/* diagonalize_ahca, src/base_utils.f90:394-444: zgesvd('N','A') of the m x n
 * matrix a (destroyed); T (n entries, the first min(m,n) written, the rest
 * zero here) receives the squared singular values in descending order and U
 * (n x n, column-major) = (W^H)^H, the eigenvectors of A^H A. */
int orc_diagonalize_ahca(cplx* a, int m, int n, double* T, cplx* U) {
  if (need_lapack()) return ORC_ERR_LAPACK;
  const int mn = m < n ? m : n;
  int lwork = 2 * mn + (m > n ? m : n);
  if (lwork < 1) lwork = 1;
  cplx* work = (cplx*)malloc(sizeof(cplx) * lwork);
  double* rwork = (double*)malloc(sizeof(double) * 5 * (mn > 0 ? mn : 1));
  cplx* wh = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
  cplx v[1];
  int info = 0, ldv = m, ldwh = n;
  for (int k = 0; k < n; ++k) T[k] = 0.0;
  p_zgesvd("N", "A", &m, &n, a, &m, T, v, &ldv, wh, &ldwh, work, &lwork, rwork, &info, 1, 1);
  if (info == 0) {
    for (int k = 0; k < n; ++k) T[k] = T[k] * T[k];
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) U[i + (size_t)n * j] = conj(wh[j + (size_t)n * i]);
  }
  free(work);
  free(rwork);
  free(wh);
  if (info != 0) {
    snprintf(g_err, sizeof g_err, "zgesvd failed (LAPACK info=%d)", info);
    return ORC_ERR_LAPACK;
  }
  return ORC_OK;
}

/* The modal matrix modal(iy, imu) (ny x nmu, column-major),
 * src/waveguide.f90:179-185 and :221-227. */
void orc_get_modal(const orc_wg* w, cplx* modal) {
  memcpy(modal, w->modal, sizeof(cplx) * (size_t)w->ny * w->nmu);
}

/* xmesh (nx) and ymesh (ny), src/waveguide.f90:145-146 and :172,212. */
void orc_get_meshes(const orc_wg* w, double* xmesh, double* ymesh) {
  if (xmesh) memcpy(xmesh, w->xmesh, sizeof(double) * w->nx);
  if (ymesh) memcpy(ymesh, w->ymesh, sizeof(double) * w->ny);
}

/* C = alpha * op(A) * B via zgemm (the reference uses gfortran's intrinsic
 * matmul, src/waveguide.f90:379,438; any FP64 summation order is equally
 * valid). */
static void gemm(const char* ta, int m, int n, int k, cplx alpha, const cplx* a, int lda,
                 const cplx* b, int ldb, cplx* c, int ldc) {
  const cplx beta = 0.0;
  p_zgemm(ta, "N", &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc, 1, 1);
}

/* ------------------------------------------------------------------------ */
/* Slice matrices and the sweep                                             */
/* ------------------------------------------------------------------------ */

/* A_ix (0-based ix in [0, nx)) into `amat` (nmu x nmu, column-major), as
 * set_hamiltonian_waveguide builds it, src/waveguide.f90:355-380:
 *   diagonal  i*mu - mu*cot(mu kdx)  on the two edge slices,
 *             -2*mu*cot(mu kdx)      in the bulk,
 *   minus modal^H diag(upot(ix - nxfree, :)) modal on disordered slices.
 * `work` holds ny*nmu complex. */
static void slice_matrix(const orc_wg* w, const double* upot, int ix, cplx* amat, cplx* work) {
  const int nmu = w->nmu, ny = w->ny;
  const cplx* diag = (ix == 0 || ix == w->nx - 1) ? w->adiag_edge : w->adiag_bulk;
  const int id = ix - w->nxfree;
  if (upot && id >= 0 && id < w->nxdiso) {
    /* work = diag(upot(id,:)) * modal  (diag_mul_left, src/base_utils.f90:155-176) */
    for (int n = 0; n < nmu; ++n)
      for (int i = 0; i < ny; ++i)
        work[i + (size_t)ny * n] = upot[id + (size_t)w->nxdiso * i] * w->modal[i + (size_t)ny * n];
    gemm("C", nmu, nmu, ny, -1.0, w->modal, ny, work, ny, amat, nmu);
  } else {
    memset(amat, 0, sizeof(cplx) * nmu * nmu);
  }
  for (int n = 0; n < nmu; ++n) amat[n + (size_t)nmu * n] += diag[n];
}

/* Recursive Green sweep shared by tdistrib and v1.  On return gs1 holds
 * G(x_nx; x_1) and, when g11 != NULL, g11 holds G(x_1; x_1).
 * src/waveguide.f90:426-440 (tdistrib) and :489-507 (v1). */
static int sweep(const orc_wg* w, const double* upot, cplx* gs1, cplx* g11) {
  const int nmu = w->nmu;
  const size_t mm = (size_t)nmu * nmu;
  cplx* gss = (cplx*)malloc(sizeof(cplx) * mm);
  cplx* tmp = (cplx*)malloc(sizeof(cplx) * mm);
  cplx* g1s = g11 ? (cplx*)malloc(sizeof(cplx) * mm) : NULL;
  cplx* work = (cplx*)malloc(sizeof(cplx) * (size_t)w->ny * nmu);
  int rc = ORC_OK;
  slice_matrix(w, upot, 0, gss, work);
  if ((rc = orc_inverse_complex(gss, nmu))) goto done;
  memcpy(gs1, gss, sizeof(cplx) * mm);
  if (g11) { memcpy(g1s, gss, sizeof(cplx) * mm); memcpy(g11, gss, sizeof(cplx) * mm); }
  for (int ix = 1; ix < w->nx; ++ix) {
    /* Gss = inv(A_ix - B Gss B) */
    slice_matrix(w, upot, ix, tmp, work);
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a)
        tmp[a + (size_t)nmu * c] -= (w->bmat[a] * gss[a + (size_t)nmu * c]) * w->bmat[c];
    memcpy(gss, tmp, sizeof(cplx) * mm);
    if ((rc = orc_inverse_complex(gss, nmu))) goto done;
    /* Gs1 = -Gss * (B Gs1) */
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = w->bmat[a] * gs1[a + (size_t)nmu * c];
    gemm("N", nmu, nmu, nmu, -1.0, gss, nmu, tmp, nmu, gs1, nmu);
    if (g11) {
      /* G11 = G11 - G1s * (B Gs1) */
      for (int c = 0; c < nmu; ++c)
        for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = w->bmat[a] * gs1[a + (size_t)nmu * c];
      cplx* t2 = work; /* ny >= 1 so work holds at least nmu*nmu when ny >= nmu */
      cplx* t2h = NULL;
      if (w->ny < nmu) { t2h = (cplx*)malloc(sizeof(cplx) * mm); t2 = t2h; }
      gemm("N", nmu, nmu, nmu, 1.0, g1s, nmu, tmp, nmu, t2, nmu);
      for (size_t e = 0; e < mm; ++e) g11[e] -= t2[e];
      /* G1s = -G1s * (B Gss) */
      for (int c = 0; c < nmu; ++c)
        for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = w->bmat[a] * gss[a + (size_t)nmu * c];
      gemm("N", nmu, nmu, nmu, -1.0, g1s, nmu, tmp, nmu, t2, nmu);
      memcpy(g1s, t2, sizeof(cplx) * mm);
      free(t2h);
    }
  }
done:
  free(gss); free(tmp); free(g1s); free(work);
  return rc;
}

/* compute_tdistrib_waveguide, src/waveguide.f90:392-462, for a given
 * potential: fills teigvals[neigv] (descending) and optionally the filtered
 * Fisher-Lee t (imax-imin+1 x jmax-jmin+1, column-major) in tmat_out. */
int orc_tdistrib_upot(const orc_wg* w, const double* upot, double* teigvals, cplx* tmat_out) {
  const int nmu = w->nmu;
  cplx* gs1 = (cplx*)malloc(sizeof(cplx) * nmu * nmu);
  int rc = sweep(w, upot, gs1, NULL);
  if (rc) { free(gs1); return rc; }
  const int mr = w->imax - w->imin + 1, mc = w->jmax - w->jmin + 1;
  cplx* t = (cplx*)malloc(sizeof(cplx) * mr * mc);
  /* Fisher-Lee with complex sqrt(mu), src/waveguide.f90:443-445 */
  for (int j = 0; j < mc; ++j)
    for (int i = 0; i < mr; ++i) {
      const int gi = w->imin - 1 + i, gj = w->jmin - 1 + j;
      const cplx v = (csqrt(w->mumesh[gi]) * gs1[gi + (size_t)nmu * gj]) * csqrt(w->mumesh[gj]);
      t[i + (size_t)mr * j] = CMPLX(0.0, 2.0) * v;
    }
  if (tmat_out) memcpy(tmat_out, t, sizeof(cplx) * mr * mc);
  const int mn = mr < mc ? mr : mc;
  double* s = (double*)malloc(sizeof(double) * mn);
  rc = orc_singular_values(t, mr, mc, s);
  if (!rc) {
    /* src/waveguide.f90:448-454: T = s^2 */
    for (int k = 0; k < w->neigv && k < mn; ++k) teigvals[k] = s[k] * s[k];
  }
  free(s); free(t); free(gs1);
  return rc;
}

/* compute_refl_trans_v1_waveguide, src/waveguide.f90:469-519, for a given
 * potential: full nmu x nmu t and r with sqrt(real(mu)). */
int orc_refl_trans_v1_upot(const orc_wg* w, const double* upot, cplx* rmat, cplx* tmat) {
  const int nmu = w->nmu;
  const size_t mm = (size_t)nmu * nmu;
  cplx* gs1 = (cplx*)malloc(sizeof(cplx) * mm);
  cplx* g11 = (cplx*)malloc(sizeof(cplx) * mm);
  int rc = sweep(w, upot, gs1, g11);
  if (!rc) {
    for (int j = 0; j < nmu; ++j)
      for (int i = 0; i < nmu; ++i) {
        const cplx si = sqrt(creal(w->mumesh[i])), sj = sqrt(creal(w->mumesh[j]));
        tmat[i + (size_t)nmu * j] = CMPLX(0.0, 2.0) * ((si * gs1[i + (size_t)nmu * j]) * sj);
        const cplx rv = CMPLX(0.0, 2.0) * ((si * g11[i + (size_t)nmu * j]) * sj);
        rmat[i + (size_t)nmu * j] = (i == j ? -1.0 : 0.0) + rv;
      }
  }
  free(gs1); free(g11);
  return rc;
}

/* solve_block_tridiag, src/base_utils.f90:296-335, specialised to the
 * independent term I_1 = identity, I_k = 0 (compute_refl_trans_v2,
 * src/waveguide.f90:526-553).  Returns X_1 (-> r) and X_nx (-> t). */
int orc_refl_trans_v2_upot(const orc_wg* w, const double* upot, cplx* rmat, cplx* tmat) {
  const int nmu = w->nmu, nx = w->nx;
  const size_t mm = (size_t)nmu * nmu;
  cplx* smat = (cplx*)malloc(sizeof(cplx) * mm * nx);
  cplx* zmat = (cplx*)malloc(sizeof(cplx) * mm * nx);
  cplx* x = (cplx*)malloc(sizeof(cplx) * mm);
  cplx* tmp = (cplx*)malloc(sizeof(cplx) * mm);
  cplx* work = (cplx*)malloc(sizeof(cplx) * (size_t)w->ny * nmu + mm);
  int rc = ORC_OK;
  slice_matrix(w, upot, 0, smat, work);
  if ((rc = orc_inverse_complex(smat, nmu))) goto done;
  memcpy(zmat, smat, sizeof(cplx) * mm); /* S_1 * I */
  for (int i = 1; i < nx; ++i) {
    cplx* si = smat + mm * i;
    const cplx* sp = smat + mm * (i - 1);
    slice_matrix(w, upot, i, si, work);
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a) si[a + (size_t)nmu * c] -= (w->bmat[a] * sp[a + (size_t)nmu * c]) * w->bmat[c];
    if ((rc = orc_inverse_complex(si, nmu))) goto done;
    const cplx* zp = zmat + mm * (i - 1);
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = -(w->bmat[a] * zp[a + (size_t)nmu * c]);
    gemm("N", nmu, nmu, nmu, 1.0, si, nmu, tmp, nmu, zmat + mm * i, nmu);
  }
  /* backward loop: X_n = Z_n; X_i = Z_i - S_i * (B X_{i+1}) */
  memcpy(x, zmat + mm * (nx - 1), sizeof(cplx) * mm);
  for (size_t e = 0; e < mm; ++e) tmat[e] = x[e];
  for (int i = nx - 2; i >= 0; --i) {
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = w->bmat[a] * x[a + (size_t)nmu * c];
    gemm("N", nmu, nmu, nmu, 1.0, smat + mm * i, nmu, tmp, nmu, work, nmu);
    for (size_t e = 0; e < mm; ++e) x[e] = zmat[mm * i + e] - work[e];
  }
  /* Fisher-Lee with sqrt(real(mu)), src/waveguide.f90:544-547 */
  for (int j = 0; j < nmu; ++j)
    for (int i = 0; i < nmu; ++i) {
      const cplx si = sqrt(creal(w->mumesh[i])), sj = sqrt(creal(w->mumesh[j]));
      const cplx tv = tmat[i + (size_t)nmu * j];
      tmat[i + (size_t)nmu * j] = CMPLX(0.0, 2.0) * ((si * tv) * sj);
      rmat[i + (size_t)nmu * j] = (i == j ? -1.0 : 0.0) + CMPLX(0.0, 2.0) * ((si * x[i + (size_t)nmu * j]) * sj);
    }
done:
  free(smat); free(zmat); free(x); free(tmp); free(work);
  return rc;
}

/* solve_block_tridiag, src/base_utils.f90:296-335: nb diagonal blocks amat
 * (nmu x nmu each), the diagonal bdiag of B, the independent term `ind` and
 * the solution `x` (nb blocks of nmu x k); every block column-major, block i
 * at offset i*nmu*nmu (amat) or i*nmu*k (ind, x).  Forward loop
 * S_1 = inv(A_1), Z_1 = S_1 I_1; S_i = inv(A_i - B S_{i-1} B),
 * Z_i = S_i (I_i - B Z_{i-1}); backward loop X_n = Z_n,
 * X_i = Z_i - S_i (B X_{i+1}). */
int orc_block_tridiag(const cplx* amat, const cplx* bdiag, const cplx* ind, int nb, int nmu, int k, cplx* x) {
  const size_t mm = (size_t)nmu * nmu, mk = (size_t)nmu * k;
  if (need_lapack()) return ORC_ERR_LAPACK;
  if (k < 1 || nb < 1 || nmu < 1) { snprintf(g_err, sizeof g_err, "solve_block_tridiag: empty system"); return ORC_ERR_ARG; }
  cplx* smat = (cplx*)malloc(sizeof(cplx) * mm * nb);
  cplx* zmat = (cplx*)malloc(sizeof(cplx) * mk * nb);
  cplx* tmp = (cplx*)malloc(sizeof(cplx) * mk);
  int rc = ORC_OK;
  memcpy(smat, amat, sizeof(cplx) * mm);
  if ((rc = orc_inverse_complex(smat, nmu))) goto done;
  gemm("N", nmu, k, nmu, 1.0, smat, nmu, ind, nmu, zmat, nmu);
  for (int i = 1; i < nb; ++i) {
    cplx* si = smat + mm * i;
    const cplx* sp = smat + mm * (i - 1);
    const cplx* ai = amat + mm * i;
    for (int c = 0; c < nmu; ++c)
      for (int a = 0; a < nmu; ++a)
        si[a + (size_t)nmu * c] = ai[a + (size_t)nmu * c] - (bdiag[a] * sp[a + (size_t)nmu * c]) * bdiag[c];
    if ((rc = orc_inverse_complex(si, nmu))) goto done;
    const cplx* zp = zmat + mk * (i - 1);
    const cplx* ii = ind + mk * i;
    for (int c = 0; c < k; ++c)
      for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = ii[a + (size_t)nmu * c] - bdiag[a] * zp[a + (size_t)nmu * c];
    gemm("N", nmu, k, nmu, 1.0, si, nmu, tmp, nmu, zmat + mk * i, nmu);
  }
  memcpy(x + mk * (nb - 1), zmat + mk * (nb - 1), sizeof(cplx) * mk);
  for (int i = nb - 2; i >= 0; --i) {
    const cplx* xn = x + mk * (i + 1);
    for (int c = 0; c < k; ++c)
      for (int a = 0; a < nmu; ++a) tmp[a + (size_t)nmu * c] = bdiag[a] * xn[a + (size_t)nmu * c];
    cplx* xi = x + mk * i;
    gemm("N", nmu, k, nmu, 1.0, smat + mm * i, nmu, tmp, nmu, xi, nmu);
    for (size_t e = 0; e < mk; ++e) xi[e] = zmat[mk * i + e] - xi[e];
  }
done:
  free(smat); free(zmat); free(tmp);
  return rc;
}

/* The diagonal block A_ix - V_ix of slice ix (0-based) for potential upot,
 * nmu x nmu column-major (set_hamiltonian_waveguide, src/waveguide.f90:349-384). */
void orc_amat(const orc_wg* w, const double* upot, int ix, cplx* amat) {
  cplx* work = (cplx*)malloc(sizeof(cplx) * ((size_t)w->ny * w->nmu + (size_t)w->nmu * w->nmu));
  slice_matrix(w, upot, ix, amat, work);
  free(work);
}

/* solve_block_tridiag on the waveguide's blocks: amat of
 * set_hamiltonian_waveguide (src/waveguide.f90:349-384) for potential upot,
 * B = bmat, independent term `ind` of nx blocks nmu x k. */
int orc_solve_block_tridiag(const orc_wg* w, const double* upot, const cplx* ind, int k, cplx* x) {
  const size_t mm = (size_t)w->nmu * w->nmu;
  cplx* amat = (cplx*)malloc(sizeof(cplx) * mm * w->nx);
  cplx* work = (cplx*)malloc(sizeof(cplx) * ((size_t)w->ny * w->nmu + mm));
  for (int i = 0; i < w->nx; ++i) slice_matrix(w, upot, i, amat + mm * i, work);
  const int rc = orc_block_tridiag(amat, w->bmat, ind, w->nx, w->nmu, k, x);
  free(amat); free(work);
  return rc;
}

/* Seed-driven tdistrib (compute_tdistrib_waveguide with the chunk checks of
 * src/waveguide.f90:408-421,452-454): writes chunk iseed of tallvals. */
int orc_compute_tdistrib(const orc_wg* w, int32_t iseed, double* tallvals, int64_t len) {
  const int64_t nchunk = len / w->neigv;
  if (nchunk == 0 || nchunk * w->neigv != len) {
    snprintf(g_err, sizeof g_err, "Invalid eigenvalue array length, received %lld", (long long)len);
    return ORC_ERR_ARG;
  }
  if (iseed < 1 || nchunk < iseed) {
    snprintf(g_err, sizeof g_err, "Invalid chunk index, received %d, expected in [1, %lld]", iseed, (long long)nchunk);
    return ORC_ERR_ARG;
  }
  double* upot = (double*)malloc(sizeof(double) * (size_t)w->ny * w->nxdiso);
  if (!upot) return ORC_ERR_NOMEM;
  orc_potential(w, iseed, upot);
  int rc = orc_tdistrib_upot(w, upot, tallvals + (int64_t)(iseed - 1) * w->neigv, NULL);
  free(upot);
  return rc;
}

/* compute_eigvals_omp, src/main.f90:134-179: OpenMP over seeds with
 * schedule(dynamic,1).  seeds[k] is the realization placed at chunk k of
 * tallvals (length n*neigv).  Returns the first failing status. */
int orc_tdistrib_batch(const orc_wg* w, const int32_t* seeds, int n, double* tallvals, int nthreads) {
  int status = ORC_OK;
  if (need_lapack()) return ORC_ERR_LAPACK;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    double* upot = (double*)malloc(sizeof(double) * (size_t)w->ny * w->nxdiso);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int k = 0; k < n; ++k) {
      orc_potential(w, seeds[k], upot);
      int rc = orc_tdistrib_upot(w, upot, tallvals + (int64_t)k * w->neigv, NULL);
      if (rc) {
#ifdef _OPENMP
#pragma omp critical
#endif
        if (!status) status = rc;
      }
    }
    free(upot);
  }
  return status;
}

/* histogram, src/base_utils.f90:491-516 (exact comparison semantics: out of
 * [b_1, b_{n+1}] is missing; x == b_{n+1} goes to the last bin; otherwise the
 * first j with x < b_{j+1}; NaN falls through uncounted). */
int orc_histogram(const double* samples, int64_t n, const double* bins, int nbins, double* histo,
                  double* missing) {
  for (int j = 1; j <= nbins; ++j)
    if (bins[j - 1] > bins[j]) { snprintf(g_err, sizeof g_err, "Unsorted array of bins"); return ORC_ERR_ARG; }
  double miss = 0.0;
  for (int j = 0; j < nbins; ++j) histo[j] = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double x = samples[i];
    if (x < bins[0] || bins[nbins] < x) {
      miss += 1.0;
    } else if (x == bins[nbins]) {
      histo[nbins - 1] += 1.0;
    } else {
      for (int j = 0; j < nbins; ++j)
        if (x < bins[j + 1]) { histo[j] += 1.0; break; }
    }
  }
  *missing = miss;
  return ORC_OK;
}

/* prepare_distrib, src/main.f90:223-251: Chebyshev edges, histogram,
 * +eps/10, normalisation (src/base_utils.f90:524-537) and bin centres by a
 * 2-point moving average (src/base_utils.f90:543-570).  rho is (nbins, 2)
 * column-major: rho[j] = centre, rho[nbins+j] = density. */
int orc_prepare_distrib(const double* tallvals, int64_t n, int nbins, double* rho, double* missing) {
  if (nbins < 1) { snprintf(g_err, sizeof g_err, "Invalid number of bins"); return ORC_ERR_ARG; }
  double* bins = (double*)malloc(sizeof(double) * (nbins + 1));
  double* histo = (double*)malloc(sizeof(double) * nbins);
  for (int i = 1; i <= nbins + 1; ++i) bins[i - 1] = (1.0 - cos(PI * (i - 1) / nbins)) / 2;
  int rc = orc_histogram(tallvals, n, bins, nbins, histo, missing);
  if (!rc) {
    const double eps10 = 2.220446049250313e-16 / 10.0;
    double npoints = 0.0;
    for (int j = 0; j < nbins; ++j) histo[j] += eps10;
    for (int j = 0; j < nbins; ++j) npoints += histo[j];
    for (int j = 0; j < nbins; ++j) histo[j] = histo[j] / (npoints * (bins[j + 1] - bins[j]));
    for (int j = 0; j < nbins; ++j) {
      rho[j] = (bins[j] + bins[j + 1]) / 2;
      rho[nbins + j] = histo[j];
    }
  }
  free(bins); free(histo);
  return rc;
}
