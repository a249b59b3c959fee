/*
 * C restatement of FEREBUS-v7's CPU likelihood path -- the timed CPU
 * baseline (TEST / BENCHMARK INFRASTRUCTURE ONLY; never part of the engine).
 *
 * The reference is Fortran and cannot be compiled on these machines (no
 * Fortran compiler, its toml-f submodule is absent), so this file restates
 * its per-particle algorithm with the same data structures and the same
 * LAPACK/BLAS calls, OpenMP-parallel over particles as README.md:50 runs it:
 *
 *  - once per data set: the d x N x N distance tensor D(f,i,j) = (x_if-x_jf)^2
 *    for i > j, 0 on the diagonal (src/kernels/distance_matrix.f90:64-93) and
 *    P = sin(sqrt(D)/2)^2 (distance_matrix.f90:130-142);
 *  - per leaf kernel: when active dims != all features, copy the active
 *    slice dm(nact, N, N) (stationary_kernel.f90:114-119), then
 *    dgemv('t', nact, N*N, alpha, dm, nact, lengthscale, 1, 0, R, 1) with
 *    alpha = -0.5 (rbf) or -2 (periodic) and R = exp(R)
 *    (stationary_kernel.f90:101-122, periodic_kernel.f90:181-206);
 *  - sum / product into fresh N x N temporaries (kernel_module.f90:309-375);
 *  - K = R + nugget * identity(N) with an N x N identity (gpr.f90:185-189,
 *    utils/array.f90:60-70);
 *  - dpotrf('L'), log-det = 2 sum log L_ii, dpotrs('L') and the marginal or
 *    concentrated formula (likelihood.f90:130-253).
 *
 * BLAS/LAPACK come from an OpenBLAS loaded at run time (scipy's bundled
 * copy), one thread per particle (OPENBLAS_NUM_THREADS=1 semantics).
 * Supported leaves: rbf, periodic (the benchmark's kernels).
 */
#include <dlfcn.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef void (*dgemv_t)(const char*, const int*, const int*, const double*, const double*, const int*,
                        const double*, const int*, const double*, double*, const int*);
typedef void (*dpotrf_t)(const char*, const int*, double*, const int*, int*);
typedef void (*dpotrs_t)(const char*, const int*, const int*, const double*, const int*, double*, const int*,
                         int*);
typedef void (*setthreads_t)(int);

static dgemv_t p_dgemv;
static dpotrf_t p_dpotrf;
static dpotrs_t p_dpotrs;
static char g_err[256];

static void* sym(void* h, const char* a, const char* b) {
  void* f = dlsym(h, a);
  return f ? f : dlsym(h, b);
}

/* Load BLAS/LAPACK from the given shared object. Returns 0 on success. */
int ref_load_blas(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_GLOBAL);
  if (!h) {
    snprintf(g_err, sizeof g_err, "dlopen %s failed: %s", path, dlerror());
    return -1;
  }
  p_dgemv = (dgemv_t)sym(h, "scipy_dgemv_", "dgemv_");
  p_dpotrf = (dpotrf_t)sym(h, "scipy_dpotrf_", "dpotrf_");
  p_dpotrs = (dpotrs_t)sym(h, "scipy_dpotrs_", "dpotrs_");
  setthreads_t st = (setthreads_t)sym(h, "scipy_openblas_set_num_threads", "openblas_set_num_threads");
  if (!p_dgemv || !p_dpotrf || !p_dpotrs) {
    snprintf(g_err, sizeof g_err, "BLAS symbols not found in %s", path);
    return -2;
  }
  if (st) st(1);
  return 0;
}

const char* ref_last_error(void) { return g_err; }

typedef struct {
  int N, d, likelihood, optimise_noise, nkspec;
  double noise;
  int* kspec;
  double *X, *y, *mu;
  double *D, *P; /* d x N x N, Fortran order D(f, i, j) */
} ref_ctx;

static size_t idx3(int d, int N, int f, int i, int j) { return (size_t)f + (size_t)d * ((size_t)i + (size_t)N * j); }

ref_ctx* ref_create(int N, int d, const double* X, const double* y, const double* mu, const int* kspec, int nkspec,
                    int likelihood, double noise, int optimise_noise) {
  ref_ctx* c = (ref_ctx*)calloc(1, sizeof(ref_ctx));
  if (!c) return NULL;
  c->N = N;
  c->d = d;
  c->likelihood = likelihood;
  c->noise = noise;
  c->optimise_noise = optimise_noise;
  c->nkspec = nkspec;
  c->kspec = (int*)malloc(sizeof(int) * nkspec);
  memcpy(c->kspec, kspec, sizeof(int) * nkspec);
  c->X = (double*)malloc(sizeof(double) * N * d);
  memcpy(c->X, X, sizeof(double) * N * d);
  c->y = (double*)malloc(sizeof(double) * N);
  memcpy(c->y, y, sizeof(double) * N);
  c->mu = (double*)malloc(sizeof(double) * N);
  for (int i = 0; i < N; ++i) c->mu[i] = mu ? mu[i] : 0.0;
  const size_t T = (size_t)d * N * N;
  c->D = (double*)malloc(sizeof(double) * T);
  c->P = (double*)malloc(sizeof(double) * T);
  if (!c->D || !c->P) {
    snprintf(g_err, sizeof g_err, "distance tensors (%zu bytes each) do not fit", sizeof(double) * T);
    return NULL;
  }
  /* distance_matrix.f90:64-93 (lower + diagonal), then the periodic tensor */
#pragma omp parallel for schedule(dynamic)
  for (int j = 0; j < N; ++j) {
    for (int f = 0; f < d; ++f) c->D[idx3(d, N, f, j, j)] = 0.0;
    for (int i = 0; i < j; ++i)
      for (int f = 0; f < d; ++f) c->D[idx3(d, N, f, i, j)] = 0.0; /* never read */
    for (int i = j + 1; i < N; ++i)
      for (int f = 0; f < d; ++f) {
        const double df = X[i + (size_t)N * f] - X[j + (size_t)N * f];
        c->D[idx3(d, N, f, i, j)] = df * df;
      }
    for (int i = 0; i < N; ++i)
      for (int f = 0; f < d; ++f) {
        const double s = sin(sqrt(c->D[idx3(d, N, f, i, j)]) / 2.0);
        c->P[idx3(d, N, f, i, j)] = s * s;
      }
  }
  return c;
}

void ref_destroy(ref_ctx* c) {
  if (!c) return;
  free(c->kspec);
  free(c->X);
  free(c->y);
  free(c->mu);
  free(c->D);
  free(c->P);
  free(c);
}

/* one leaf: R = exp(alpha * T(dims)^T l) */
static int leaf_R(const ref_ctx* c, int op, int n, const int* dims1, const double* theta, double* R) {
  const int N = c->N, d = c->d;
  double* ls = (double*)malloc(sizeof(double) * n);
  for (int k = 0; k < n; ++k) {
    if (op == 1) {
      ls[k] = exp(theta[k]);
    } else {
      const double l = 1.0 / exp(theta[k]);
      ls[k] = l * l;
    }
  }
  const double alpha = op == 1 ? -0.5 : -2.0, zero = 0.0;
  const int one = 1, NN = N * N;
  const double* T = op == 1 ? c->D : c->P;
  int all = (n == d);
  for (int k = 0; all && k < n; ++k) all = (dims1[k] == k + 1);
  if (all) {
    p_dgemv("T", &d, &NN, &alpha, T, &d, ls, &one, &zero, R, &one);
  } else {
    double* dm = (double*)malloc(sizeof(double) * (size_t)n * N * N);
    if (!dm) {
      free(ls);
      return -1;
    }
    for (size_t e = 0; e < (size_t)N * N; ++e)
      for (int k = 0; k < n; ++k) dm[(size_t)k + (size_t)n * e] = T[(size_t)(dims1[k] - 1) + (size_t)d * e];
    p_dgemv("T", &n, &NN, &alpha, dm, &n, ls, &one, &zero, R, &one);
    free(dm);
  }
  for (size_t e = 0; e < (size_t)N * N; ++e) R[e] = exp(R[e]);
  free(ls);
  return 0;
}

/* evaluate the postfix tree; returns a malloc'd N x N matrix or NULL */
static double* kernel_R(const ref_ctx* c, const double* theta) {
  const int N = c->N;
  double* stack[16];
  int top = 0, i = 0, p = 0;
  while (i < c->nkspec) {
    const int op = c->kspec[i];
    if (op == 1 || op == 2) {
      const int n = c->kspec[i + 1];
      double* R = (double*)malloc(sizeof(double) * (size_t)N * N);
      if (!R || leaf_R(c, op, n, c->kspec + i + 2, theta + p, R)) return NULL;
      stack[top++] = R;
      p += n;
      i += 2 + n;
    } else if (op == 10 || op == 11) {
      double* b = stack[--top];
      double* a = stack[--top];
      double* R = (double*)malloc(sizeof(double) * (size_t)N * N);
      if (!R) return NULL;
      for (size_t e = 0; e < (size_t)N * N; ++e) R[e] = op == 10 ? a[e] + b[e] : a[e] * b[e];
      free(a);
      free(b);
      stack[top++] = R;
      i += 1;
    } else {
      snprintf(g_err, sizeof g_err, "opcode %d not in the CPU restatement", op);
      return NULL;
    }
  }
  return stack[0];
}

static int nkparams(const ref_ctx* c) {
  int i = 0, p = 0;
  while (i < c->nkspec) {
    const int op = c->kspec[i];
    if (op >= 1 && op <= 4) {
      p += c->kspec[i + 1];
      i += 2 + c->kspec[i + 1];
    } else if (op == 5) {
      p += 1;
      i += 2;
    } else {
      i += 1;
    }
  }
  return p;
}

static int one_particle(const ref_ctx* c, const double* theta, double* ll_out, int* info_out) {
  const int N = c->N, one = 1;
  const int nk = nkparams(c);
  const double noise = c->optimise_noise ? theta[nk] : c->noise;
  double* K = kernel_R(c, theta);
  if (!K) return -1;
  /* gpr.f90:188: K = K + nugget * identity(N) */
  double* I = (double*)calloc((size_t)N * N, sizeof(double));
  if (!I) return -1;
  for (int j = 0; j < N; ++j) I[j + (size_t)N * j] = 1.0;
  for (size_t e = 0; e < (size_t)N * N; ++e) K[e] = K[e] + noise * I[e];
  free(I);
  int info = 0;
  p_dpotrf("L", &N, K, &N, &info);
  *info_out = info;
  if (info != 0) {
    *ll_out = NAN;
    free(K);
    return 0;
  }
  double logdet = 0.0;
  for (int j = 0; j < N; ++j) logdet += log(K[j + (size_t)N * j]);
  logdet *= 2.0;
  double* t = (double*)malloc(sizeof(double) * N);
  if (c->likelihood == 0) {
    for (int j = 0; j < N; ++j) t[j] = c->y[j] - c->mu[j];
    p_dpotrs("L", &N, &one, K, &N, t, &N, &info);
    double q = 0.0;
    for (int j = 0; j < N; ++j) q += (c->y[j] - c->mu[j]) * t[j];
    *ll_out = -0.5 * q - 0.5 * logdet - 0.5 * N * log(2.0 * 3.141592653589793);
  } else {
    double* t1 = (double*)malloc(sizeof(double) * N);
    for (int j = 0; j < N; ++j) {
      t[j] = c->y[j];
      t1[j] = 1.0;
    }
    p_dpotrs("L", &N, &one, K, &N, t, &N, &info);
    p_dpotrs("L", &N, &one, K, &N, t1, &N, &info);
    double a = 0.0, b = 0.0;
    for (int j = 0; j < N; ++j) {
      a += t[j];
      b += t1[j];
    }
    const double m = a / b;
    for (int j = 0; j < N; ++j) t[j] = c->y[j] - m;
    p_dpotrs("L", &N, &one, K, &N, t, &N, &info);
    double q = 0.0;
    for (int j = 0; j < N; ++j) q += (c->y[j] - m) * t[j];
    const double s2 = q / N;
    *ll_out = -0.5 * N * log(s2) - 0.5 * logdet;
    free(t1);
  }
  free(t);
  free(K);
  return 0;
}

/* S particles (theta row-major S x ldtheta), OpenMP over particles. */
int ref_loglik_batch(const ref_ctx* c, int S, const double* theta, int ldtheta, double* ll, int* info,
                     int nthreads) {
  int rc = 0;
  if (!p_dpotrf) {
    snprintf(g_err, sizeof g_err, "BLAS not loaded");
    return -1;
  }
#pragma omp parallel for schedule(dynamic) num_threads(nthreads) reduction(| : rc)
  for (int s = 0; s < S; ++s) rc |= one_particle(c, theta + (size_t)s * ldtheta, ll + s, info + s);
  return rc;
}
