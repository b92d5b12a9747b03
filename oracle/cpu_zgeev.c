/*
 * TEST INFRASTRUCTURE — the CPU oracle and CPU baseline. Never linked into
 * or called by the product library.
 *
 * Restates the reference's CPU comparison driver,
 * stream_test_with_MKL/get_eig_MKL.c:27-47 (identical copy at
 * tokura_zgeev_batched_library_test/get_eig_MKL.c): one LAPACK
 * zgeev(JOBVL='N', JOBVR='N') per matrix, column-major, lda = n, the
 * batch split over host threads. The reference links MKL (unpinned
 * version, stream_test_with_MKL/compile_mkl.sh:2), which is not available
 * here; the same published LAPACK routine is taken from the OpenBLAS build
 * bundled with scipy (OpenBLAS 0.3.34, LAPACKE symbol prefix "scipy_"),
 * located at run time and opened with dlopen. BLAS threading inside each
 * call is pinned to 1, as the reference uses sequential MKL.
 *
 * Also exposes zgeevx(BALANC='N', SENSE='E') to obtain the reciprocal
 * eigenvalue condition numbers RCONDE used to filter parity checks,
 * zgeev('V','V') for the eigenvector path, and the real dgeev('N','N') for
 * the real-input path (same library, same threading).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int (*zgeev_fn)(int layout, char jobvl, char jobvr, int n, double* a, int lda, double* w, double* vl,
                        int ldvl, double* vr, int ldvr);
typedef int (*zgeevx_fn)(int layout, char balanc, char jobvl, char jobvr, char sense, int n, double* a, int lda,
                         double* w, double* vl, int ldvl, double* vr, int ldvr, int* ilo, int* ihi, double* scale,
                         double* abnrm, double* rconde, double* rcondv);
typedef int (*dgeev_fn)(int layout, char jobvl, char jobvr, int n, double* a, int lda, double* wr, double* wi,
                        double* vl, int ldvl, double* vr, int ldvr);
typedef void (*setthreads_fn)(int);

enum { LAPACK_COL_MAJOR_ = 102 };

static void* g_lib = NULL;
static zgeev_fn g_zgeev = NULL;
static zgeevx_fn g_zgeevx = NULL;
static dgeev_fn g_dgeev = NULL;

/* Opens the LAPACK library; returns 0 on success. */
int cpu_zgeev_open(const char* path) {
  if (g_lib) return 0;
  g_lib = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!g_lib) return -1;
  g_zgeev = (zgeev_fn)dlsym(g_lib, "scipy_LAPACKE_zgeev");
  g_zgeevx = (zgeevx_fn)dlsym(g_lib, "scipy_LAPACKE_zgeevx");
  g_dgeev = (dgeev_fn)dlsym(g_lib, "scipy_LAPACKE_dgeev");
  setthreads_fn st = (setthreads_fn)dlsym(g_lib, "scipy_openblas_set_num_threads");
  if (st) st(1);
  return (g_zgeev && g_zgeevx && g_dgeev) ? 0 : -2;
}

typedef struct {
  int n, batch, mode; /* mode 0: eigenvalues, 1: + RCONDE, 2: + left/right eigenvectors, 3: real dgeev */
  const double* A;    /* batch * n * n complex (interleaved re, im), column-major */
  double* w;          /* batch * n complex */
  double* rconde;     /* batch * n (mode 1) */
  double* vl;         /* batch * n * n complex (mode 2) */
  double* vr;         /* batch * n * n complex (mode 2) */
  double* wi;         /* batch * n (mode 3; w holds wr) */
  int* info;          /* batch */
  atomic_long next;
} job_t;

static void* worker(void* arg) {
  job_t* J = (job_t*)arg;
  const int n = J->n;
  const size_t nn2 = (size_t)n * n * 2;
  double* a = (double*)malloc(sizeof(double) * nn2);
  double* vl = NULL; double* vr = NULL; double* scale = NULL; double* rcv = NULL;
  if (J->mode == 1) {
    vl = (double*)malloc(sizeof(double) * nn2);
    vr = (double*)malloc(sizeof(double) * nn2);
    scale = (double*)malloc(sizeof(double) * n);
    rcv = (double*)malloc(sizeof(double) * n);
  }
  for (;;) {
    /* dynamic schedule in chunks of 16 matrices */
    long k0 = atomic_fetch_add(&J->next, 16);
    if (k0 >= J->batch) break;
    long k1 = k0 + 16 < J->batch ? k0 + 16 : J->batch;
    for (long k = k0; k < k1; ++k) {
      if (J->mode == 3) { /* real: A holds batch * n * n doubles */
        memcpy(a, J->A + (size_t)k * n * n, sizeof(double) * (size_t)n * n);
        J->info[k] = g_dgeev(LAPACK_COL_MAJOR_, 'N', 'N', n, a, n, J->w + (size_t)k * n, J->wi + (size_t)k * n, NULL, 1,
                             NULL, 1);
        continue;
      }
      memcpy(a, J->A + (size_t)k * nn2, sizeof(double) * nn2);
      if (J->mode == 0) {
        J->info[k] = g_zgeev(LAPACK_COL_MAJOR_, 'N', 'N', n, a, n, J->w + (size_t)k * n * 2, NULL, 1, NULL, 1);
      } else if (J->mode == 2) {
        J->info[k] = g_zgeev(LAPACK_COL_MAJOR_, 'V', 'V', n, a, n, J->w + (size_t)k * n * 2, J->vl + (size_t)k * nn2, n,
                             J->vr + (size_t)k * nn2, n);
      } else {
        int ilo, ihi;
        double abnrm;
        J->info[k] = g_zgeevx(LAPACK_COL_MAJOR_, 'N', 'V', 'V', 'E', n, a, n, J->w + (size_t)k * n * 2, vl, n, vr, n,
                              &ilo, &ihi, scale, &abnrm, J->rconde + (size_t)k * n, rcv);
      }
    }
  }
  free(a); free(vl); free(vr); free(scale); free(rcv);
  return NULL;
}

static int run(job_t* J, int nthreads, double* seconds) {
  if (!g_zgeev) return -3;
  if (nthreads < 1) nthreads = 1;
  atomic_store(&J->next, 0);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, worker, J);
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(th);
  if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  return 0;
}

/* Eigenvalues of `batch` matrices with zgeev('N','N'); info[k] is LAPACK's INFO. */
int cpu_zgeev_batched(int n, int batch, const double* A, double* w, int* info, int nthreads, double* seconds) {
  job_t J;
  J.n = n; J.batch = batch; J.mode = 0; J.A = A; J.w = w; J.rconde = NULL; J.vl = NULL; J.vr = NULL; J.info = info;
  J.wi = NULL;
  return run(&J, nthreads, seconds);
}

/* Real eigenvalues with dgeev('N','N'): A is batch * n * n doubles, column-major. */
int cpu_dgeev_batched(int n, int batch, const double* A, double* wr, double* wi, int* info, int nthreads,
                      double* seconds) {
  job_t J;
  J.n = n; J.batch = batch; J.mode = 3; J.A = A; J.w = wr; J.wi = wi; J.rconde = NULL; J.vl = NULL; J.vr = NULL;
  J.info = info;
  return run(&J, nthreads, seconds);
}

/* Eigenvalues and left/right eigenvectors with zgeev('V','V'). */
int cpu_zgeev_vectors_batched(int n, int batch, const double* A, double* w, double* vl, double* vr, int* info,
                              int nthreads, double* seconds) {
  job_t J;
  J.n = n; J.batch = batch; J.mode = 2; J.A = A; J.w = w; J.rconde = NULL; J.vl = vl; J.vr = vr; J.info = info;
  J.wi = NULL;
  return run(&J, nthreads, seconds);
}

/* Eigenvalues plus RCONDE (reciprocal eigenvalue condition numbers) from zgeevx. */
int cpu_zgeevx_batched(int n, int batch, const double* A, double* w, double* rconde, int* info, int nthreads,
                       double* seconds) {
  job_t J;
  J.n = n; J.batch = batch; J.mode = 1; J.A = A; J.w = w; J.rconde = rconde; J.vl = NULL; J.vr = NULL; J.info = info;
  J.wi = NULL;
  return run(&J, nthreads, seconds);
}
