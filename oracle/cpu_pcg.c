/* A clean CPU solver for the time step: the comparison point for the GPU path beside the faithful
 * restatement of the reference in hf_oracle.c.  Measurement and test infrastructure, not the
 * reference's algorithm (the reference solves with a COO Jacobi-BiCG, mod_Sparse.f90:372-434):
 *   - the operator in the geometric form (diagonal and the +x/+y/+z face of each cell, from
 *     or_geometric), so an SpMV is a 7-point stencil with no atomics;
 *   - Jacobi-preconditioned CG in FP64 on A = -H (symmetric positive definite), vector updates
 *     fused into the SpMV and dot-product loops, OpenMP over z-planes;
 *   - stopped on the true relative residual ||S - H x|| / ||S|| (the recursive residual only
 *     triggers the check; a restart follows when the true one is not there yet).
 * Per step, S and x0 (with the reference's x0 + TINY rule) come from the oracle's RHS (or_rhs),
 * and the solution rotates into the oracle's state as simulate() does (mod_evolve.f90:169-170). */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/heatflow_gb300.h"

int or_rhs(void* h, int64_t itime, double* B, double* Q, double* Qdens, double* scat, double* S,
           double* x);
void or_geometric(void* h, double* diag, double* cx, double* cy, double* cz);
void or_get_state(void* h, double* tp, double* tpp);
void or_set_state(void* h, const double* tp, const double* tpp);

typedef struct cp_sys {
  int64_t nx, ny, nz, n;
  int px, py, pz, threads;
  double *diag, *cx, *cy, *cz, *dinv;
  double *B, *Q, *Qd, *Sc, *S, *x, *r, *z, *p, *q, *tp, *tpp;
} cp_sys;

void cp_destroy(void* h) {
  cp_sys* c = (cp_sys*)h;
  if (!c) return;
  double* bufs[] = {c->diag, c->cx, c->cy, c->cz, c->dinv, c->B, c->Q, c->Qd, c->Sc,
                    c->S,    c->x,  c->r,  c->z,  c->p,    c->q, c->tp, c->tpp};
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) free(bufs[k]);
  free(c);
}

void* cp_create(void* oracle, int64_t nx, int64_t ny, int64_t nz, const int32_t* periodic,
                int threads) {
  cp_sys* c = (cp_sys*)calloc(1, sizeof(cp_sys));
  if (!c) return NULL;
  c->nx = nx; c->ny = ny; c->nz = nz; c->n = nx * ny * nz;
  c->px = periodic[0] != 0; c->py = periodic[1] != 0; c->pz = periodic[2] != 0;
  c->threads = threads > 0 ? threads : 1;
  const size_t bytes = sizeof(double) * (size_t)c->n;
  double** bufs[] = {&c->diag, &c->cx, &c->cy, &c->cz, &c->dinv, &c->B, &c->Q, &c->Qd, &c->Sc,
                     &c->S,    &c->x,  &c->r,  &c->z,  &c->p,    &c->q, &c->tp, &c->tpp};
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) {
    *bufs[k] = (double*)malloc(bytes);
    if (!*bufs[k]) { cp_destroy(c); return NULL; }
  }
  or_geometric(oracle, c->diag, c->cx, c->cy, c->cz);
  for (int64_t i = 0; i < c->n; ++i) c->dinv[i] = 1.0 / (-c->diag[i]);
  return c;
}

/* out = A v = -(H v); returns v.out when want_dot. */
static double apply_a(const cp_sys* c, const double* v, double* out, int want_dot) {
  const int64_t nx = c->nx, ny = c->ny, nz = c->nz, nxy = nx * ny;
  const double *diag = c->diag, *cx = c->cx, *cy = c->cy, *cz = c->cz;
  double dot = 0.0;
#pragma omp parallel for collapse(2) num_threads(c->threads) schedule(static) reduction(+ : dot)
  for (int64_t z = 0; z < nz; ++z) {
    for (int64_t y = 0; y < ny; ++y) {
      const int64_t row = z * nxy + y * nx;
      for (int64_t x = 0; x < nx; ++x) {
        const int64_t l = row + x;
        double acc = diag[l] * v[l];
        if (x + 1 < nx) acc += cx[l] * v[l + 1];
        else if (c->px && nx > 1) acc += cx[l] * v[l - (nx - 1)];
        if (x > 0) acc += cx[l - 1] * v[l - 1];
        else if (c->px && nx > 1) acc += cx[l + nx - 1] * v[l + nx - 1];
        if (ny > 1) {
          if (y + 1 < ny) acc += cy[l] * v[l + nx];
          else if (c->py) acc += cy[l] * v[l - (ny - 1) * nx];
          if (y > 0) acc += cy[l - nx] * v[l - nx];
          else if (c->py) acc += cy[l + (ny - 1) * nx] * v[l + (ny - 1) * nx];
        }
        if (nz > 1) {
          if (z + 1 < nz) acc += cz[l] * v[l + nxy];
          else if (c->pz) acc += cz[l] * v[l - (nz - 1) * nxy];
          if (z > 0) acc += cz[l - nxy] * v[l - nxy];
          else if (c->pz) acc += cz[l + (nz - 1) * nxy] * v[l + (nz - 1) * nxy];
        }
        out[l] = -acc;
        if (want_dot) dot += v[l] * out[l];
      }
    }
  }
  return dot;
}

/* r = b - A x for b = -S, A = -H: r = -(S - H x), so ||r|| is the true residual norm; returns
 * ||r||^2. */
static double true_residual(const cp_sys* c) {
  apply_a(c, c->x, c->q, 0);
  const int64_t n = c->n;
  double rr = 0.0;
#pragma omp parallel for num_threads(c->threads) schedule(static) reduction(+ : rr)
  for (int64_t i = 0; i < n; ++i) {
    const double r = -c->S[i] - c->q[i];
    c->r[i] = r;
    rr += r * r;
  }
  return rr;
}

/* One time step.  Returns 0 or the oracle's HF_ENAN_* code from the RHS; *iters = CG iterations,
 * *relres = the final true relative residual. */
int cp_step(void* h, void* oracle, int64_t itime, double tol, int64_t itmax, int64_t* iters,
            double* relres) {
  cp_sys* c = (cp_sys*)h;
  const int64_t n = c->n;
  int rc = or_rhs(oracle, itime, c->B, c->Q, c->Qd, c->Sc, c->S, c->x);
  if (rc) return rc;
  double bb = 0.0;
#pragma omp parallel for num_threads(c->threads) schedule(static) reduction(+ : bb)
  for (int64_t i = 0; i < n; ++i) bb += c->S[i] * c->S[i];
  const double bn = sqrt(bb);
  int64_t it = 0;
  double rel = bn > 0.0 ? sqrt(true_residual(c)) / bn : 0.0;
  while (rel > tol && it < itmax) {
    const int64_t it0 = it;
    double rz = 0.0;
#pragma omp parallel for num_threads(c->threads) schedule(static) reduction(+ : rz)
    for (int64_t i = 0; i < n; ++i) {
      const double zi = c->dinv[i] * c->r[i];
      c->z[i] = zi;
      c->p[i] = zi;
      rz += c->r[i] * zi;
    }
    while (it < itmax) {
      const double pq = apply_a(c, c->p, c->q, 1);
      if (!(pq > 0.0)) break;
      const double alpha = rz / pq;
      double rr = 0.0, rz2 = 0.0;
#pragma omp parallel for num_threads(c->threads) schedule(static) reduction(+ : rr, rz2)
      for (int64_t i = 0; i < n; ++i) {
        c->x[i] += alpha * c->p[i];
        const double ri = c->r[i] - alpha * c->q[i];
        c->r[i] = ri;
        const double zi = c->dinv[i] * ri;
        c->z[i] = zi;
        rr += ri * ri;
        rz2 += ri * zi;
      }
      ++it;
      if (sqrt(rr) <= 0.5 * tol * bn) break;
      const double beta = rz2 / rz;
      rz = rz2;
#pragma omp parallel for num_threads(c->threads) schedule(static)
      for (int64_t i = 0; i < n; ++i) c->p[i] = c->z[i] + beta * c->p[i];
    }
    rel = sqrt(true_residual(c)) / bn;
    if (it == it0) break;             /* breakdown (p.Ap <= 0): no progress to restart from */
  }
  for (int64_t i = 0; i < n; ++i)
    if (isnan(c->x[i])) return HF_ENAN_X;   /* a NaN in x: the reference stops */
  or_get_state(oracle, c->tp, c->tpp);
  or_set_state(oracle, c->x, c->tp);   /* Temp_pp = Temp_p; Temp_p = x */
  if (iters) *iters = it;
  if (relres) *relres = rel;
  return 0;
}
