/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the HeatFlow reference's
 * time-stepping hot path (ExeQuantCode/HeatFlow v0.5.0, Fortran), used as the parity checker
 * for the CUDA path and as the timed CPU baseline ("port").  Nothing in the product links or
 * calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
 *
 * Every routine follows the reference statement by statement, including its quirks, and cites
 * the file:line it restates (paths relative to the reference project root).  Floating-point
 * expressions keep the reference's evaluation order (Fortran evaluates left to right within one
 * precedence level); the file is compiled with -ffp-contract=off so no product is fused.
 *
 * Pinned against: test/data/TempDis.dat (10 Fourier steps of test/data/{param,mat,system}.in),
 * the manual's Chapter 6 steady 1-D cases 1-4, test/test_mod_cattaneo.f90:64-73,
 * test/test_mod_boundary.f90:64-72 and test/test_mod_hmatrix.f90:56-64 (see tests/).
 *
 * Indices are 1-based inside this file, as in the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/heatflow_gb300.h"

#define OR_TINY 1.0e-12                /* mod_constants.f90:17 */
/* Threads of the loops that run in parallel (or_set_threads): the per-cell loops of the RHS, whose
 * cells are independent (same bits at any thread count), and the reference's OpenMP SpMV. */
static int g_threads = 1;
#define OR_PI 3.141592653589793        /* mod_constants.f90:12 */
#define OR_STEFBOLTZ 5.670373e-8       /* mod_constants.f90:16 */

typedef struct or_sys {
  int64_t nx, ny, nz, na;
  double len[3];          /* grid(:,:,:)%Length, mod_inputs.f90:619-621 */
  double volume;          /* grid%volume, mod_inputs.f90:622 */
  double *kappa, *rho, *hc, *tau_s, *em, *rhoc, *power;
  int64_t* iheater;
  int any_heater;
  double power_in, freq, time_step, inverse_time;
  int64_t heated_steps;
  int icattaneo, isteady, periodic[3], cg[6], qdens_mode;
  double kb[6], tb[6], t_bath, t_bath_cg, br;
  /* sprs2_dp ra (mod_SPtype.f90:19-24) */
  int64_t len_cap, count;
  int64_t *irow, *jcol;
  double* val;
  double *temp_p, *temp_pp;
  /* tabulated properties (extension): tables of rows (T, kappa, rho, c), a table per cell or -1 */
  int32_t ntables;
  int32_t* toff;
  double* trows;
  int32_t* cell_table;
} or_sys;

/* altmod, mod_hmatrix.f90:330-338 */
static int64_t altmod(int64_t a, int64_t b) {
  int64_t c = a % b;
  if (c == 0) c = b;
  return c;
}

#define G(s, x, y, z) (((z) - 1) * (s)->nx * (s)->ny + ((y) - 1) * (s)->nx + ((x) - 1))

/* boundry_diag_term, mod_hmatrix.f90:347-391 (kappa_ab is inout; unset branches keep it) */
static double boundry_diag_term(const or_sys* s, int64_t xb, int64_t yb, int64_t zb, int64_t x,
                                int64_t y, int64_t z, double kappa_ab) {
  double kappa = s->kappa[G(s, x, y, z)];
  if (xb != x) {
    if (xb < 1) {
      kappa_ab = ((2.0 * s->kb[0] * kappa) / (s->kb[0] + kappa)) / (s->len[0] * s->len[0]);
      if (kappa != s->kb[0]) kappa_ab = kappa_ab * s->br;
    } else if (xb > s->nx) {
      kappa_ab = ((2.0 * s->kb[1] * kappa) / (s->kb[1] + kappa)) / (s->len[0] * s->len[0]);
      if (kappa != s->kb[1]) kappa_ab = kappa_ab * s->br;
    }
  } else if (yb != y) {
    if (yb < 1) {
      kappa_ab = ((2.0 * s->kb[2] * kappa) / (s->kb[2] + kappa)) / (s->len[1] * s->len[1]);
      if (kappa != s->kb[2]) kappa_ab = kappa_ab * s->br;
    } else if (yb > s->ny) {
      kappa_ab = ((2.0 * s->kb[3] * kappa) / (s->kb[3] + kappa)) / (s->len[1] * s->len[1]);
      if (kappa != s->kb[3]) kappa_ab = kappa_ab * s->br;
    }
  } else if (zb != z) {
    if (zb < 1) {
      kappa_ab = ((2.0 * s->kb[4] * kappa) / (s->kb[4] + kappa)) / (s->len[2] * s->len[2]);
      if (kappa != s->kb[4]) kappa_ab = kappa_ab * s->br;
    } else if (zb > s->nz) {
      kappa_ab = ((2.0 * s->kb[5] * kappa) / (s->kb[5] + kappa)) / (s->len[2] * s->len[2]);
      if (kappa != s->kb[5]) kappa_ab = kappa_ab * s->br;
    }
  }
  return kappa_ab;
}

/* calculate_conductivity, mod_hmatrix.f90:273-321 */
static double calculate_conductivity(const or_sys* s, int64_t xi, int64_t yi, int64_t zi,
                                     int64_t xo, int64_t yo, int64_t zo) {
  double kappa_ab = 0.0;
  if (xi >= 1 && xi <= s->nx && yi >= 1 && yi <= s->ny && zi >= 1 && zi <= s->nz) {
    double kin = s->kappa[G(s, xi, yi, zi)];
    double kout = s->kappa[G(s, xo, yo, zo)];
    int ax = -1;
    if (xi != xo) ax = 0;
    else if (yi != yo) ax = 1;
    else if (zi != zo) ax = 2;
    if (ax >= 0) {
      double L = s->len[ax]; /* Length(ax) of both cells: uniform grid */
      kappa_ab = (L + L) * kin * kout / (L * kout + L * kin);
      kappa_ab = kappa_ab / (L * L);
    }
    if (kin != kout) kappa_ab = kappa_ab * s->br;
    return kappa_ab;
  }
  return boundry_diag_term(s, xi, yi, zi, xo, yo, zo, kappa_ab);
}

/* calculate_alpha, mod_hmatrix.f90:254-267 */
static double calculate_alpha(const or_sys* s, int64_t x, int64_t y, int64_t z, int64_t i) {
  double alpha = 0.0;
  double tau = s->tau_s[G(s, x, y, z)];
  if (s->isteady == 0) {
    if (s->icattaneo == 0) tau = 0.0;
    alpha = (tau * s->rhoc[i - 1]) + (s->inverse_time * s->rhoc[i - 1]);
  }
  return alpha;
}

/* hmatrixfunc, mod_hmatrix.f90:62-248 */
static double hmatrixfunc(const or_sys* s, int64_t i, int64_t j) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  int64_t x = altmod(i, nx);
  int64_t y = ((i - altmod(i, nx)) / nx) % ny + 1;
  int64_t z = (i - altmod(i, nx * ny)) / (nx * ny) + 1;
  double alpha = calculate_alpha(s, x, y, z, i);
  int64_t xp = x + 1, xm = x - 1, yp = y + 1, ym = y - 1, zp = z + 1, zm = z - 1;
  if (s->periodic[0]) { if (xp > nx) xp = 1; if (xm < 1) xm = nx; }
  if (s->periodic[1]) { if (yp > ny) yp = 1; if (ym < 1) ym = ny; }
  if (s->periodic[2]) { if (zp > nz) zp = 1; if (zm < 1) zm = nz; }
  double A = calculate_conductivity(s, xm, y, z, x, y, z);
  double B = calculate_conductivity(s, xp, y, z, x, y, z);
  double D = calculate_conductivity(s, x, ym, z, x, y, z);
  double E = calculate_conductivity(s, x, yp, z, x, y, z);
  double F = calculate_conductivity(s, x, y, zm, x, y, z);
  double Gc = calculate_conductivity(s, x, y, zp, x, y, z);
  int64_t d = i - j;
  double H = 0.0;
  if (d == 0) H = -(A + B + D + E + F + Gc) - alpha;
  if (d == 1) H = (x == 1) ? 0.0 : A;
  if (d == -1) H = (x == nx) ? 0.0 : B;
  if (d == nx) H = (y == 1) ? 0.0 : D;
  if (d == -nx) H = (y == ny) ? 0.0 : E;
  if (d == nx * ny) H = (z == 1) ? 0.0 : F;
  if (d == -(nx * ny)) H = (z == nz) ? 0.0 : Gc;
  if (s->periodic[0]) {
    if (d == -(nx - 1) && x == 1) H = A;
    if (d == (nx - 1) && x == nx) H = B;
  }
  if (s->periodic[1]) {
    if (d == -(ny - 1) * nx && y == 1) H = D;
    if (d == (ny - 1) * nx && y == ny) H = E;
  }
  if (s->periodic[2]) {
    if (d == -(nz - 1) * nx * ny && z == 1) H = F;
    if (d == (nz - 1) * nx * ny && z == nz) H = Gc;
  }
  return H;
}

/* sparse_Hmatrix, mod_setup.f90:89-152.  Returns 0, or -1 if the reference would write past
 * its COO capacity (grids with nx=1 and more than one cell). */
static int sparse_hmatrix(or_sys* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz, na = s->na;
  int64_t len = 7 * nx * ny * nz - 2 * (nx * ny + ny * nz + nz * nx);
  if (s->periodic[0]) len += 2 * ny * nz;
  if (s->periodic[1]) len += 2 * nz * nx;
  if (s->periodic[2]) len += 2 * nx * ny;
  s->len_cap = len;
  free(s->irow); free(s->jcol); free(s->val);
  s->irow = (int64_t*)malloc(sizeof(int64_t) * (size_t)(len > 0 ? len : 1));
  s->jcol = (int64_t*)malloc(sizeof(int64_t) * (size_t)(len > 0 ? len : 1));
  s->val = (double*)malloc(sizeof(double) * (size_t)(len > 0 ? len : 1));
  for (int64_t c = 0; c < len; ++c) { s->val[c] = 0.0; s->irow[c] = -2; s->jcol[c] = -1; }
  int64_t addit[6]; int nadd = 0;
  addit[nadd++] = 1;
  if (s->periodic[0]) addit[nadd++] = nx - 1;
  if (ny > 1) addit[nadd++] = nx;
  if (s->periodic[1] && ny > 1) addit[nadd++] = (ny - 1) * nx;
  if (nz > 1) addit[nadd++] = nx * ny;
  if (s->periodic[2] && nz > 1) addit[nadd++] = (nz - 1) * ny * nx;
  int64_t count = 0;
  for (int64_t j = 1; j <= na; ++j) {
    int64_t i = j;
    if (count >= len) return -1;
    double h0 = hmatrixfunc(s, i, j);
    s->val[count] = h0; s->irow[count] = i; s->jcol[count] = j; ++count;
    for (int k = 0; k < nadd; ++k) {
      i = j + addit[k];
      if (i > na) break;                 /* cycle parent_loop */
      h0 = hmatrixfunc(s, i, j);
      if (fabs(h0) < OR_TINY) continue;  /* cycle neighbour_loop */
      if (count + 2 > len) return -1;
      s->val[count] = h0; s->irow[count] = i; s->jcol[count] = j; ++count;
      s->val[count] = h0; s->irow[count] = j; s->jcol[count] = i; ++count;
    }
  }
  s->count = count;
  return 0;
}

/* ---- construction: set_global_variables (mod_setup.f90:34-83) ------------------------------ */
static double* dup_d(const double* src, int64_t n, double fill) {
  double* d = (double*)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) d[i] = src ? src[i] : fill;
  return d;
}

void or_destroy(void* h) {
  or_sys* s = (or_sys*)h;
  if (!s) return;
  free(s->kappa); free(s->rho); free(s->hc); free(s->tau_s); free(s->em); free(s->rhoc);
  free(s->power); free(s->iheater); free(s->irow); free(s->jcol); free(s->val);
  free(s->temp_p); free(s->temp_pp);
  free(s->toff); free(s->trows); free(s->cell_table);
  free(s);
}

/* Returns NULL for grids the reference cannot represent (see sparse_hmatrix). */
void* or_create(const hf_problem* p) {
  or_sys* s = (or_sys*)calloc(1, sizeof(or_sys));
  s->nx = p->nx; s->ny = p->ny; s->nz = p->nz; s->na = p->nx * p->ny * p->nz;
  const int64_t na = s->na;
  s->len[0] = p->lx / (double)(float)p->nx; /* Lx/real(nx): default-real conversion */
  s->len[1] = p->ly / (double)(float)p->ny;
  s->len[2] = p->lz / (double)(float)p->nz;
  s->volume = s->len[0] * s->len[1] * s->len[2];
  s->time_step = p->time_step;
  s->inverse_time = 1.0 / p->time_step;   /* mod_setup.f90:45 */
  s->kappa = dup_d(p->kappa, na, 0.0);
  s->rho = dup_d(p->rho, na, 0.0);
  s->hc = dup_d(p->heat_capacity, na, 0.0);
  s->em = dup_d(p->em, na, 0.0);
  s->power = dup_d(p->power, na, p->power_in);
  s->tau_s = (double*)malloc(sizeof(double) * (size_t)na);
  s->rhoc = (double*)malloc(sizeof(double) * (size_t)na);
  s->iheater = (int64_t*)calloc((size_t)na, sizeof(int64_t));
  s->any_heater = 0;
  for (int64_t i = 0; i < na; ++i) {
    double tau = p->tau ? p->tau[i] : 0.0;
    s->tau_s[i] = tau * s->inverse_time * s->inverse_time;  /* mod_setup.f90:62 */
    s->rhoc[i] = s->rho[i] * s->hc[i];                       /* mod_setup.f90:64 */
    if (p->iheater) s->iheater[i] = p->iheater[i];
    if (s->iheater[i] > 0) s->any_heater = 1;
  }
  s->power_in = p->power_in; s->freq = p->freq; s->heated_steps = p->heated_steps;
  s->icattaneo = p->icattaneo; s->isteady = p->isteady; s->qdens_mode = p->qdens_mode;
  for (int a = 0; a < 3; ++a) s->periodic[a] = p->periodic[a];
  for (int f = 0; f < 6; ++f) { s->cg[f] = p->cg_face[f]; s->kb[f] = p->kappa_bound[f]; s->tb[f] = p->t_bath_face[f]; }
  s->t_bath = p->t_bath; s->t_bath_cg = p->t_bath_cg; s->br = p->br;
  s->temp_p = (double*)calloc((size_t)na, sizeof(double));
  s->temp_pp = (double*)calloc((size_t)na, sizeof(double));
  if (sparse_hmatrix(s) != 0) { or_destroy(s); return NULL; }
  return s;
}

int64_t or_num_cells(void* h) { return ((or_sys*)h)->na; }

/* Copy the COO out.  Returns the entry count; *cap receives the reference capacity. */
int64_t or_coo(void* h, int64_t* irow, int64_t* jcol, double* val, int64_t* cap) {
  or_sys* s = (or_sys*)h;
  if (cap) *cap = s->len_cap;
  for (int64_t c = 0; c < s->len_cap; ++c) {
    if (irow) irow[c] = s->irow[c];
    if (jcol) jcol[c] = s->jcol[c];
    if (val) val[c] = s->val[c];
  }
  return s->count;
}

void or_set_state(void* h, const double* tp, const double* tpp) {
  or_sys* s = (or_sys*)h;
  memcpy(s->temp_p, tp, sizeof(double) * (size_t)s->na);
  memcpy(s->temp_pp, tpp, sizeof(double) * (size_t)s->na);
}
void or_get_state(void* h, double* tp, double* tpp) {
  or_sys* s = (or_sys*)h;
  if (tp) memcpy(tp, s->temp_p, sizeof(double) * (size_t)s->na);
  if (tpp) memcpy(tpp, s->temp_pp, sizeof(double) * (size_t)s->na);
}

/* ---- RHS pieces ------------------------------------------------------------------------- */
/* boundary(B), mod_boundary.f90:24-152.  B must be zeroed by the caller (mod_evolve.f90:55). */
void or_boundary(void* h, double* B) {
  or_sys* s = (or_sys*)h;
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  double pd[6] = {0, 0, 0, 0, 0, 0};
  /* power densities of the Neumann "CG" faces, mod_boundary.f90:43-66 (all cells equal) */
  if (s->cg[4]) pd[4] = s->t_bath_cg / (s->volume * (double)nx * (double)ny);
  if (s->cg[5]) pd[5] = s->t_bath_cg / (s->volume * (double)nx * (double)ny);
  if (s->cg[2]) pd[2] = s->t_bath_cg / (s->volume * (double)nx * (double)nz);
  if (s->cg[3]) pd[3] = s->t_bath_cg / (s->volume * (double)nx * (double)nz);
  if (s->cg[0]) pd[0] = s->t_bath_cg / (s->volume * (double)ny * (double)nz);
  if (s->cg[1]) pd[1] = s->t_bath_cg / (s->volume * (double)ny * (double)nz);
#pragma omp parallel for collapse(2) num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t iz = 1; iz <= nz; ++iz)
    for (int64_t iy = 1; iy <= ny; ++iy)
      for (int64_t ix = 1; ix <= nx; ++ix) {
        const int64_t I = ((iz - 1) * ny + (iy - 1)) * nx + ix;
        double kappa = s->kappa[I - 1], kh;
        int64_t c[3] = {ix, iy, iz}, n[3] = {nx, ny, nz};
        for (int a = 0; a < 3; ++a) {
          if (s->periodic[a]) continue;
          double L = s->len[a];
          if (c[a] == 1) {
            if (s->cg[2 * a]) {
              B[I - 1] = pd[2 * a];
            } else {
              kh = (2.0 * kappa * s->kb[2 * a] / (kappa + s->kb[2 * a])) / (L * L);
              if (kappa != s->kb[2 * a]) kh = kh * s->br;
              B[I - 1] = B[I - 1] + (kh) * s->tb[2 * a];
            }
          }
          if (c[a] == n[a]) {
            if (s->cg[2 * a + 1]) {
              B[I - 1] = pd[2 * a + 1];
            } else {
              kh = (2.0 * kappa * s->kb[2 * a + 1] / (kappa + s->kb[2 * a + 1])) / (L * L);
              if (kappa != s->kb[2 * a + 1]) kh = kh * s->br;
              B[I - 1] = B[I - 1] + (kh) * s->tb[2 * a + 1];
            }
          }
        }
      }
}

/* heater(itime,Q,Qdens), mod_heating.f90:27-169.  Q and Qdens are fully written. */
void or_heater(void* h, int64_t itime, const double* tp, double* Q, double* Qdens) {
  or_sys* s = (or_sys*)h;
  const int64_t na = s->na;
  double time = s->time_step * (double)itime;
  double time_pulse = (double)s->heated_steps * s->time_step;
  double heated_volume = 0.0;
  double L1 = s->len[0], L2 = s->len[1];
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t ia = 0; ia < na; ++ia) {
    double power = s->power[ia];
    double tau = s->tau_s[ia] * pow(s->time_step, 2.0);
    double q = 0.0;
    switch (s->iheater[ia]) {
      case 0: q = 0.0; break;
      case 1: q = power; break;
      case 2: q = (time <= time_pulse) ? power : 0.0; break;
      case 3: {
        double x = time * 2.0 * OR_PI * s->freq;
        double x2 = s->time_step * 2.0 * OR_PI * s->freq;
        q = power * 0.5 * ((x2) - sin(x + x2) * cos(x + x2) + sin(x) * cos(x)) / x2;
        break;
      }
      case 4: q = power * pow(sin(time * 2.0 * OR_PI * s->freq), 2.0); break;
      case 5:
        q = power * pow(sin(time * 2.0 * OR_PI * s->freq), 2.0) +
            power * 2.0 * OR_PI * s->freq * tau * sin(2.0 * time * 2.0 * OR_PI * s->freq);
        break;
      case 6: q = (itime == 1) ? power : 0.0; break;
      default: q = 0.0; break;   /* no case matches: Q keeps its initial 0 */
    }
    q = q - s->em[ia] * L1 * L2 * OR_STEFBOLTZ * (pow(tp[ia], 4.0) - pow(s->t_bath, 4.0));
    Q[ia] = q;
  }
  for (int64_t ia = 0; ia < na; ++ia)   /* in cell order, as the reference sums it */
    if (s->iheater[ia] > 0) heated_volume = heated_volume + s->volume;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t ia = 0; ia < na; ++ia) {
    double qd = 0.0;
    if (s->qdens_mode == HF_QDENS_CELL_VOLUME) qd = Q[ia] / s->volume;
    else if (heated_volume > 0.0) qd = Q[ia] / heated_volume;
    Qdens[ia] = qd;
  }
}

/* S_catS, mod_cattaneo.f90:23-42 */
void or_cattaneo(void* h, const double* tp, const double* tpp, double* scat) {
  or_sys* s = (or_sys*)h;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t i = 0; i < s->na; ++i)
    scat[i] = (tpp[i] - 2.0 * tp[i]) * (s->tau_s[i] * s->rhoc[i]);
}

/* Steps 55-141 of simulate (mod_evolve.f90): B, Q, Qdens, S_CAT, S and the initial guess x.
 * Returns a HF_ENAN_* code if the reference would stop, else 0. */
/* Any NaN in v (the reference's isnan checks of a whole vector). */
static int any_nan(const double* v, int64_t n) {
  int bad = 0;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(| : bad) if (g_threads > 1)
  for (int64_t i = 0; i < n; ++i) bad |= isnan(v[i]) ? 1 : 0;
  return bad;
}

int or_rhs(void* h, int64_t itime, double* B, double* Q, double* Qdens, double* scat, double* S,
           double* x) {
  or_sys* s = (or_sys*)h;
  const int64_t na = s->na;
  const double* tp = s->temp_p;
  const double* tpp = s->temp_pp;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t i = 0; i < na; ++i) { B[i] = 0; Q[i] = 0; Qdens[i] = 0; scat[i] = 0; S[i] = 0; }
  or_boundary(h, B);
  if (any_nan(B, na)) return HF_ENAN_B;
  if (s->any_heater) {
    or_heater(h, itime, tp, Q, Qdens);
    if (any_nan(Q, na)) return HF_ENAN_Q;
    if (any_nan(Qdens, na)) return HF_ENAN_QDENS;
  }
  if (s->icattaneo == 1) {
    or_cattaneo(h, tp, tpp, scat);
    if (any_nan(scat, na)) return HF_ENAN_SCAT;
  }
  const int cat = s->icattaneo == 1, steady = s->isteady != 0;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
  for (int64_t i = 0; i < na; ++i) {
    if (!steady) {
      S[i] = -s->inverse_time * tp[i] * s->rhoc[i] - Qdens[i] - B[i];
      if (cat) S[i] = S[i] + scat[i];
    } else {
      S[i] = -Qdens[i] - B[i];
    }
  }
  if (any_nan(S, na)) return HF_ENAN_S;
  int any = 0;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(| : any) if (g_threads > 1)
  for (int64_t i = 0; i < na; ++i) {
    x[i] = tp[i] + (tp[i] - tpp[i]);
    if (x[i] - tp[i] < OR_TINY) any |= 1;
  }
  if (any) {
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (int64_t i = 0; i < na; ++i) x[i] = x[i] + OR_TINY;
  }
  return 0;
}

/* ---- solver: module solver, mod_Sparse.f90 ---------------------------------------------- */
int or_set_threads(int n) {
  g_threads = n > 0 ? n : 1;
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* SRSax / SRStx, mod_Sparse.f90:293-337: b(irow) += val*x(jcol) over all slots, skipping
 * slots whose target row is out of range; with OpenMP each update is atomic. */
void or_atimes(void* h, const double* x, double* b, int transpose) {
  or_sys* s = (or_sys*)h;
  const int64_t m = s->na, n = s->len_cap;
  const int64_t* tgt = transpose ? s->jcol : s->irow;
  const int64_t* src = transpose ? s->irow : s->jcol;
  const double* val = s->val;
  for (int64_t i = 0; i < m; ++i) b[i] = 0.0;
#ifdef _OPENMP
  if (g_threads > 1) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < n; ++j) {
      int64_t i = tgt[j];
      if (i > 0 && i <= m) {
        double v = val[j] * x[src[j] - 1];
#pragma omp atomic
        b[i - 1] += v;
      }
    }
    return;
  }
#endif
  for (int64_t j = 0; j < n; ++j) {
    int64_t i = tgt[j];
    if (i > 0 && i <= m) b[i - 1] = b[i - 1] + val[j] * x[src[j] - 1];
  }
}

/* SRSdiag, mod_Sparse.f90:350-366: the diagonal by a scan of all slots, in storage order. */
static void srs_diag(const or_sys* s, double* d) {
  int64_t k = 0;
  for (int64_t c = 0; c < s->len_cap; ++c)
    if (s->irow[c] == s->jcol[c]) d[k++] = s->val[c];
}

/* asolve, mod_Sparse.f90:452-466 */
static void asolve(const or_sys* s, const double* b, double* x, double* dscratch) {
  srs_diag(s, dscratch);
  for (int64_t i = 0; i < s->na; ++i) x[i] = b[i] / dscratch[i];
}

static double dot(const double* a, const double* b, int64_t n) {
  double acc = 0.0;
  for (int64_t i = 0; i < n; ++i) acc = acc + a[i] * b[i];
  return acc;
}

/* linbcg, mod_Sparse.f90:372-434 (Jacobi-preconditioned biconjugate gradient). */
int or_linbcg(void* h, const double* b, double* x, int itol, double tol, int64_t itmax,
              int64_t* iter_out, double* err_out) {
  or_sys* s = (or_sys*)h;
  const int64_t n = s->na;
  size_t bytes = sizeof(double) * (size_t)n;
  double *p = malloc(bytes), *pp = malloc(bytes), *r = malloc(bytes), *rr = malloc(bytes);
  double *z = malloc(bytes), *zz = malloc(bytes), *dg = malloc(bytes);
  double ak, akden, bk, bkden = 1.0, bknum, bnrm, err = 0.0;
  int64_t iter;
  or_atimes(h, x, r, 0);
  for (int64_t i = 0; i < n; ++i) { r[i] = b[i] - r[i]; rr[i] = r[i]; }
  bnrm = sqrt(dot(b, b, n));
  asolve(s, r, z, dg);
  asolve(s, rr, zz, dg);
  bknum = dot(z, rr, n);
  for (int64_t i = 0; i < n; ++i) { p[i] = z[i]; pp[i] = zz[i]; }
  for (iter = 1; iter <= itmax; ++iter) {
    or_atimes(h, p, z, 0);
    bkden = bknum;
    akden = dot(z, pp, n);
    ak = bknum / akden;
    or_atimes(h, pp, zz, 1);
    for (int64_t i = 0; i < n; ++i) {
      x[i] = x[i] + ak * p[i];
      r[i] = r[i] - ak * z[i];
      rr[i] = rr[i] - ak * zz[i];
    }
    asolve(s, r, z, dg);
    if (itol == 1) err = sqrt(dot(r, r, n)) / bnrm;
    else err = sqrt(dot(z, z, n)) / bnrm;
    if (err <= tol) break;
    asolve(s, rr, zz, dg);
    bknum = dot(z, rr, n);
    bk = bknum / bkden;
    for (int64_t i = 0; i < n; ++i) { p[i] = bk * p[i] + z[i]; pp[i] = bk * pp[i] + zz[i]; }
  }
  if (iter > itmax) iter = itmax + 1; /* Fortran DO leaves iter = itmax+1 on exhaustion */
  if (iter_out) *iter_out = iter;
  if (err_out) *err_out = err;
  free(p); free(pp); free(r); free(rr); free(z); free(zz); free(dg);
  return 0;
}

/* ||b - Hx|| / ||b|| in FP64 with the COO operator. */
double or_true_relres(void* h, const double* b, const double* x) {
  or_sys* s = (or_sys*)h;
  double* y = malloc(sizeof(double) * (size_t)s->na);
  or_atimes(h, x, y, 0);
  double rr = 0.0, bb = 0.0;
  for (int64_t i = 0; i < s->na; ++i) { double d = b[i] - y[i]; rr += d * d; bb += b[i] * b[i]; }
  free(y);
  return sqrt(rr) / sqrt(bb);
}

/* The operator in the geometric form: diag[I] = H_II and the stored slot coupling I with its + x/y/z
 * neighbour (the first cell of a periodic axis for the last one), with sparse_Hmatrix's drop rule
 * (|H| < TINY is not stored, mod_setup.f90:137); 0 where there is no such face. */
void or_geometric(void* h, double* diag, double* cx, double* cy, double* cz) {
  const or_sys* s = (const or_sys*)h;
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  for (int64_t l = 0; l < s->na; ++l) {
    const int64_t I = l + 1, x = l % nx + 1, y = (l / nx) % ny + 1, z = l / (nx * ny) + 1;
    double v;
    diag[l] = hmatrixfunc(s, I, I);
    v = 0.0;
    if (x < nx) v = hmatrixfunc(s, I + 1, I);
    else if (s->periodic[0] && nx > 1) v = hmatrixfunc(s, I, I - (nx - 1));
    cx[l] = fabs(v) < OR_TINY ? 0.0 : v;
    v = 0.0;
    if (ny > 1) {
      if (y < ny) v = hmatrixfunc(s, I + nx, I);
      else if (s->periodic[1]) v = hmatrixfunc(s, I, I - (ny - 1) * nx);
    }
    cy[l] = fabs(v) < OR_TINY ? 0.0 : v;
    v = 0.0;
    if (nz > 1) {
      if (z < nz) v = hmatrixfunc(s, I + nx * ny, I);
      else if (s->periodic[2]) v = hmatrixfunc(s, I, I - (nz - 1) * nx * ny);
    }
    cz[l] = fabs(v) < OR_TINY ? 0.0 : v;
  }
}

/* Jacobi-PCG on the same COO operator (the symmetric specialisation of linbcg: rr == r,
 * pp == p), stopping on the TRUE relative residual.  Test helper for larger grids. */
int or_pcg(void* h, const double* b, double* x, double tol, int64_t itmax, int64_t* iter_out,
           double* relres_out) {
  or_sys* s = (or_sys*)h;
  const int64_t n = s->na;
  size_t bytes = sizeof(double) * (size_t)n;
  double *p = malloc(bytes), *q = malloc(bytes), *r = malloc(bytes), *z = malloc(bytes);
  double* dg = malloc(bytes);
  srs_diag(s, dg);
  double bnrm = sqrt(dot(b, b, n));
  int64_t iter = 0;
  double relres = 0.0;
  for (int restart = 0; restart < 50; ++restart) {
    or_atimes(h, x, r, 0);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    relres = sqrt(dot(r, r, n)) / bnrm;
    if (relres <= tol || iter >= itmax) break;
    for (int64_t i = 0; i < n; ++i) { z[i] = r[i] / dg[i]; p[i] = z[i]; }
    double rz = dot(r, z, n);
    while (iter < itmax) {
      or_atimes(h, p, q, 0);
      double ak = rz / dot(p, q, n);
      for (int64_t i = 0; i < n; ++i) { x[i] += ak * p[i]; r[i] -= ak * q[i]; z[i] = r[i] / dg[i]; }
      ++iter;
      double rec = sqrt(dot(r, r, n)) / bnrm;
      if (rec <= 0.5 * tol) break;
      double rz2 = dot(r, z, n);
      double bk = rz2 / rz;
      rz = rz2;
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + bk * p[i];
    }
  }
  if (iter_out) *iter_out = iter;
  if (relres_out) *relres_out = relres;
  free(p); free(q); free(r); free(z); free(dg);
  return 0;
}

/* simulate(itime), mod_evolve.f90:45-177.  mode 0: linbcg with (itol=1, tol, itmax) as the
 * reference calls it (tol=1e-32, itmax=50000 at :142-144); mode 1: or_pcg to a true relative
 * residual tol.  Returns 0 or a HF_ENAN_* code (the reference's `stop 1`). */
/* Property of one table column at temperature T: rows (T ascending) held constant below the first
 * and above the last row, linear in between: v_k + (T - T_k) / (T_k1 - T_k) * (v_k1 - v_k). */
static double table_value(const double* rows, int32_t m, int col, double T) {
  if (T <= rows[0]) return rows[col];
  if (T >= rows[4 * (m - 1)]) return rows[4 * (m - 1) + col];
  int32_t k = 0;
  while (k + 1 < m - 1 && !(T < rows[4 * (k + 1)])) ++k;
  const double f = (T - rows[4 * k]) / (rows[4 * (k + 1)] - rows[4 * k]);
  return rows[4 * k + col] + f * (rows[4 * (k + 1) + col] - rows[4 * k + col]);
}

/* Tabulated kappa, rho, c (extension of TempDepProp, whose reference lookup is commented out,
 * mod_tempdep.f90:66-95): after every step, cells with a table take their properties at their
 * new temperature and H is rebuilt (ChangeProp -> sparse_Hmatrix, mod_evolve.f90:172-174). */
int or_set_property_tables(void* h, int32_t ntables, const int32_t* offsets, const double* rows,
                           const int32_t* cell_table) {
  or_sys* s = (or_sys*)h;
  free(s->toff); free(s->trows); free(s->cell_table);
  s->ntables = ntables;
  s->toff = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntables + 1));
  memcpy(s->toff, offsets, sizeof(int32_t) * (size_t)(ntables + 1));
  s->trows = (double*)malloc(sizeof(double) * 4 * (size_t)offsets[ntables]);
  memcpy(s->trows, rows, sizeof(double) * 4 * (size_t)offsets[ntables]);
  s->cell_table = (int32_t*)malloc(sizeof(int32_t) * (size_t)s->na);
  memcpy(s->cell_table, cell_table, sizeof(int32_t) * (size_t)s->na);
  return 0;
}

static void change_prop(or_sys* s) {
  for (int64_t i = 0; i < s->na; ++i) {
    const int32_t t = s->cell_table[i];
    if (t < 0) continue;
    const double* rows = s->trows + 4 * (size_t)s->toff[t];
    const int32_t m = s->toff[t + 1] - s->toff[t];
    const double T = s->temp_p[i];
    s->kappa[i] = table_value(rows, m, 1, T);
    s->rho[i] = table_value(rows, m, 2, T);
    s->hc[i] = table_value(rows, m, 3, T);
    s->rhoc[i] = s->rho[i] * s->hc[i];
  }
  sparse_hmatrix(s);
}

int or_simulate(void* h, int64_t itime, int mode, double tol, int64_t itmax, int64_t* iter,
                double* err) {
  or_sys* s = (or_sys*)h;
  const int64_t na = s->na;
  size_t bytes = sizeof(double) * (size_t)na;
  double *B = malloc(bytes), *Q = malloc(bytes), *Qd = malloc(bytes), *Sc = malloc(bytes);
  double *S = malloc(bytes), *x = malloc(bytes);
  int rc = or_rhs(h, itime, B, Q, Qd, Sc, S, x);
  if (rc == 0) {
    if (mode == 0) or_linbcg(h, S, x, 1, tol, itmax, iter, err);
    else or_pcg(h, S, x, tol, itmax, iter, err);
    for (int64_t i = 0; i < na; ++i) if (isnan(x[i])) { rc = HF_ENAN_X; break; }
  }
  if (rc == 0) {
    memcpy(s->temp_pp, s->temp_p, bytes);  /* Temp_pp = Temp_p; Temp_p = x (:169-170) */
    memcpy(s->temp_p, x, bytes);
    if (s->cell_table) change_prop(s);
  }
  free(B); free(Q); free(Qd); free(Sc); free(S); free(x);
  return rc;
}
