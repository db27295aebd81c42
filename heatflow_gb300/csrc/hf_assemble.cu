// One-time set-up kernels: per-cell properties, the 7-point operator in geometric SoA form,
// the boundary vector, the Jacobi-scaled operator, and the parity probes (COO assembly in the
// reference's storage order, SpMV in the reference's accumulation order).
//
// This file is compiled with -fmad=false: every product and sum is rounded separately, in the
// order the reference writes it, so the assembled coefficients equal the reference's bit for bit.
#include "hf_ctx.cuh"

namespace hf {

// ---- reference arithmetic (1-based indices, as in the reference) -----------------------------
struct HM {
  const InstDesc& d;
  const InstBC& bc;
  const double* kappa;  // instance base
  const double* rhoc;
  const double* tau_s;

  __device__ int64_t G(int64_t x, int64_t y, int64_t z) const {
    return ((z - 1) * d.ny + (y - 1)) * (int64_t)d.nx + (x - 1);
  }

  // boundry_diag_term, mod_hmatrix.f90:347-391
  __device__ double bdiag(int64_t xb, int64_t yb, int64_t zb, int64_t x, int64_t y, int64_t z,
                          double kab) const {
    double k = kappa[G(x, y, z)];
    int f = -1, ax = 0;
    if (xb != x) { ax = 0; f = xb < 1 ? 0 : (xb > d.nx ? 1 : -1); }
    else if (yb != y) { ax = 1; f = yb < 1 ? 2 : (yb > d.ny ? 3 : -1); }
    else if (zb != z) { ax = 2; f = zb < 1 ? 4 : (zb > d.nz ? 5 : -1); }
    if (f >= 0) {
      double L = d.len[ax];
      kab = ((2.0 * bc.kb[f] * k) / (bc.kb[f] + k)) / (L * L);
      if (k != bc.kb[f]) kab = kab * bc.br;
    }
    return kab;
  }

  // calculate_conductivity, mod_hmatrix.f90:273-321
  __device__ double cond(int64_t xi, int64_t yi, int64_t zi, int64_t xo, int64_t yo,
                         int64_t zo) const {
    double kab = 0.0;
    if (xi >= 1 && xi <= d.nx && yi >= 1 && yi <= d.ny && zi >= 1 && zi <= d.nz) {
      double kin = kappa[G(xi, yi, zi)];
      double kout = kappa[G(xo, yo, zo)];
      int ax = xi != xo ? 0 : (yi != yo ? 1 : (zi != zo ? 2 : -1));
      if (ax >= 0) {
        double L = d.len[ax];
        kab = (L + L) * kin * kout / (L * kout + L * kin);
        kab = kab / (L * L);
      }
      if (kin != kout) kab = kab * bc.br;
      return kab;
    }
    return bdiag(xi, yi, zi, xo, yo, zo, kab);
  }

  // hmatrixfunc(i,j), mod_hmatrix.f90:62-248 (calculate_alpha :254-267 inlined)
  __device__ double hmf(int64_t i, int64_t j) const {
    const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
    int64_t am = i % nx; if (am == 0) am = nx;
    int64_t x = am;
    int64_t y = ((i - am) / nx) % ny + 1;
    int64_t amxy = i % (nx * ny); if (amxy == 0) amxy = nx * ny;
    int64_t z = (i - amxy) / (nx * ny) + 1;
    double alpha = 0.0;
    if (d.isteady == 0) {
      double tau = tau_s[G(x, y, z)];
      if (d.icattaneo == 0) tau = 0.0;
      alpha = (tau * rhoc[i - 1]) + (d.inv_dt * rhoc[i - 1]);
    }
    int64_t xp = x + 1, xm = x - 1, yp = y + 1, ym = y - 1, zp = z + 1, zm = z - 1;
    if (d.px) { if (xp > nx) xp = 1; if (xm < 1) xm = nx; }
    if (d.py) { if (yp > ny) yp = 1; if (ym < 1) ym = ny; }
    if (d.pz) { if (zp > nz) zp = 1; if (zm < 1) zm = nz; }
    double A = cond(xm, y, z, x, y, z), B = cond(xp, y, z, x, y, z);
    double D = cond(x, ym, z, x, y, z), E = cond(x, yp, z, x, y, z);
    double F = cond(x, y, zm, x, y, z), Gc = cond(x, y, zp, x, y, z);
    int64_t dd = i - j;
    double H = 0.0;
    if (dd == 0) H = -(A + B + D + E + F + Gc) - alpha;
    if (dd == 1) H = (x == 1) ? 0.0 : A;
    if (dd == -1) H = (x == nx) ? 0.0 : B;
    if (dd == nx) H = (y == 1) ? 0.0 : D;
    if (dd == -nx) H = (y == ny) ? 0.0 : E;
    if (dd == nx * ny) H = (z == 1) ? 0.0 : F;
    if (dd == -(nx * ny)) H = (z == nz) ? 0.0 : Gc;
    if (d.px) {
      if (dd == -(nx - 1) && x == 1) H = A;
      if (dd == (nx - 1) && x == nx) H = B;
    }
    if (d.py) {
      if (dd == -(ny - 1) * nx && y == 1) H = D;
      if (dd == (ny - 1) * nx && y == ny) H = E;
    }
    if (d.pz) {
      if (dd == -(nz - 1) * nx * ny && z == 1) H = F;
      if (dd == (nz - 1) * nx * ny && z == nz) H = Gc;
    }
    return H;
  }

  // The COO slot list of sparse_Hmatrix for column j (mod_setup.f90:107-112): offsets in
  // storage order; returns the count.
  __device__ int slots(int64_t* off) const {
    const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
    int k = 0;
    off[k++] = 1;
    if (d.px) off[k++] = nx - 1;
    if (ny > 1) off[k++] = nx;
    if (d.py && ny > 1) off[k++] = (ny - 1) * nx;
    if (nz > 1) off[k++] = nx * ny;
    if (d.pz && nz > 1) off[k++] = (nz - 1) * ny * nx;
    return k;
  }

  // Stored value of COO entry (i,j), i > j (0 when sparse_Hmatrix drops it, |H| < TINY).
  __device__ double stored(int64_t i, int64_t j) const {
    if (i > (int64_t)d.n) return 0.0;
    double h = hmf(i, j);
    return fabs(h) < kTiny ? 0.0 : h;
  }
};

// ---- per-cell properties: set_global_variables, mod_setup.f90:53-68 ------------------------
// The coefficient of T^n in S (mod_evolve.f90:112-116 with S_cat, mod_cattaneo.f90:35-36):
// -rho c / dt - 2 tau' rho c, or -rho c / dt in Fourier mode.
__device__ __forceinline__ double scoef(const InstDesc& d, double rc, double cc) {
  const double a = -d.inv_dt * rc;
  return d.icattaneo == 1 ? a - 2.0 * cc : a;
}

__global__ void k_props(DevArrays A, const double* rho, const double* hc, const double* tau,
                        const double* em) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const InstDesc& d = A.inst[A.tile_inst[g / kTile]];
  if (g - d.off >= d.n) return;
  double rc = rho[g] * hc[g];
  double ts = tau[g] * d.inv_dt * d.inv_dt;
  A.rhoc[g] = rc;
  A.tau_s[g] = ts;
  A.ccat[g] = ts * rc;                                   // (tau*lin_rhoc), mod_cattaneo.f90:35-36
  A.scoef[g] = scoef(d, rc, ts * rc);
  if (A.emc) A.emc[g] = em[g] * d.len[0] * d.len[1] * kStefBoltz;   // mod_heating.f90:121-122
}

// ---- geometric operator + boundary vector --------------------------------------------------
// For cell I (1-based) and axis a: c_a[I] is the COO value coupling I with its + neighbour,
// where the + neighbour of the last cell of a periodic axis is the first (wrap slot of
// sparse_Hmatrix).  For nx >= 2 every COO slot maps to exactly one such face; a slot that is
// nonzero where no face exists raises devcheck.
__global__ void k_assemble(DevArrays A, const InstBC* bcs, const double* kappa) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  int inst = A.tile_inst[g / kTile];
  const InstDesc& d = A.inst[inst];
  const InstBC& bc = bcs[inst];
  HM h{d, bc, kappa + d.off, A.rhoc + d.off, A.tau_s + d.off};
  const int64_t l = g - d.off;
  if (l >= d.n) return;
  const int64_t I = l + 1;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t x = l % nx + 1, y = (l / nx) % ny + 1, z = l / (nx * ny) + 1;
  int bad = 0;
  A.diag[g] = h.hmf(I, I);
  // x: interior slot (offset 1) or, at x = nx, the wrap slot (offset nx-1) of column I-(nx-1)
  double cxv = 0.0, cyv = 0.0, czv = 0.0;
  if (x < nx) cxv = h.stored(I + 1, I);
  else if (d.px && nx > 1) cxv = h.stored(I, I - (nx - 1));
  if (ny > 1) {
    if (y < ny) cyv = h.stored(I + nx, I);
    else if (d.py) cyv = h.stored(I, I - (ny - 1) * nx);
  }
  if (nz > 1) {
    if (z < nz) czv = h.stored(I + nx * ny, I);
    else if (d.pz) czv = h.stored(I, I - (nz - 1) * nx * ny);
  }
  // consistency: slots that would be stored with no geometric face behind them
  if (x == nx && !d.px && h.stored(I + 1, I) != 0.0) bad = 1;
  if (ny > 1 && y == ny && !d.py && h.stored(I + nx, I) != 0.0) bad = 1;
  A.cx[g] = cxv;
  A.cy[g] = cyv;
  A.cz[g] = czv;

  // boundary(B), mod_boundary.f90:72-150 (B starts at 0, mod_evolve.f90:55)
  double Bv = 0.0;
  const double kap = kappa[g];
  const int64_t c[3] = {x, y, z}, n[3] = {nx, ny, nz};
  const int per[3] = {d.px, d.py, d.pz};
  for (int a = 0; a < 3; ++a) {
    if (per[a]) continue;
    double L = d.len[a];
    if (c[a] == 1) {
      int f = 2 * a;
      if (bc.cg[f]) {
        Bv = bc.pd[f];
      } else {
        double kh = (2.0 * kap * bc.kb[f] / (kap + bc.kb[f])) / (L * L);
        if (kap != bc.kb[f]) kh = kh * bc.br;
        Bv = Bv + (kh) * bc.tb[f];
      }
    }
    if (c[a] == n[a]) {
      int f = 2 * a + 1;
      if (bc.cg[f]) {
        Bv = bc.pd[f];
      } else {
        double kh = (2.0 * kap * bc.kb[f] / (kap + bc.kb[f])) / (L * L);
        if (kap != bc.kb[f]) kh = kh * bc.br;
        Bv = Bv + (kh) * bc.tb[f];
      }
    }
  }
  A.bvec[g] = Bv;
  if (isnan(Bv)) atomicOr(&A.scal[inst].status, 1 << (HF_ENAN_B - HF_ENAN_B));
  if (bad) atomicOr(&A.scal[inst].devcheck, 1);
}

// ---- operator rebuild of a step (temperature-dependent properties) -----------------------------
// The coefficients of k_assemble + k_sinv, bit for bit, with each conductivity evaluated once.
// Interior face P|Q (Q the + neighbour): calculate_conductivity(P->Q) (kin = kappa_P) is both the
// stored slot of P (hmatrixfunc(Q,P)) and the - face term of Q's diagonal; (Q->P) is P's + face
// term.  The products (L+L)*kin*kout round differently in the two orders, so both are evaluated.
// Pass 1 writes P->Q per axis into the a64 arrays (k_scale rewrites them afterwards); on the last
// cell of a periodic axis it writes last->first, the - face term of the first cell.  Pass 2 forms
// the + face terms, the diagonal in hmatrixfunc's summation order, the wrap slots (the + face term
// of the last cell), the boundary vector and 1/sqrt|H_II|.  k_assemble instead evaluates
// hmatrixfunc whole per stored slot (six conductivities each) and checks slot consistency, which
// the one-time set-up affords and a rebuild on every step does not.
__global__ void k_faces_step(DevArrays A, const InstBC* bcs, const double* kappa) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const int inst = A.tile_inst[g / kTile];
  const InstDesc& d = A.inst[inst];
  HM h{d, bcs[inst], kappa + d.off, A.rhoc + d.off, A.tau_s + d.off};
  const int64_t l = g - d.off;
  if (l >= d.n) return;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t x = l % nx + 1, y = (l / nx) % ny + 1, z = l / (nx * ny) + 1;
  A.a64x[g] = x < nx ? h.cond(x, y, z, x + 1, y, z) : (d.px ? h.cond(x, y, z, 1, y, z) : 0.0);
  A.a64y[g] = y < ny ? h.cond(x, y, z, x, y + 1, z) : (d.py ? h.cond(x, y, z, x, 1, z) : 0.0);
  A.a64z[g] = z < nz ? h.cond(x, y, z, x, y, z + 1) : (d.pz ? h.cond(x, y, z, x, y, 1) : 0.0);
}

__global__ void k_diag_step(DevArrays A, const InstBC* bcs, const double* kappa) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const int inst = A.tile_inst[g / kTile];
  const InstDesc& d = A.inst[inst];
  const InstBC& bc = bcs[inst];
  HM h{d, bc, kappa + d.off, A.rhoc + d.off, A.tau_s + d.off};
  const int64_t l = g - d.off;
  if (l >= d.n) { A.sinv[g] = 0.0; return; }
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  const int64_t x = l % nx + 1, y = (l / nx) % ny + 1, z = l / nxy + 1;
  // hmatrixfunc(I,I): alpha, then the six face terms (mod_hmatrix.f90:62-248)
  double alpha = 0.0;
  if (d.isteady == 0) {
    double tau = A.tau_s[g];
    if (d.icattaneo == 0) tau = 0.0;
    alpha = (tau * A.rhoc[g]) + (d.inv_dt * A.rhoc[g]);
  }
  int64_t xp = x + 1, xm = x - 1, yp = y + 1, ym = y - 1, zp = z + 1, zm = z - 1;
  if (d.px) { if (xp > nx) xp = 1; if (xm < 1) xm = nx; }
  if (d.py) { if (yp > ny) yp = 1; if (ym < 1) ym = ny; }
  if (d.pz) { if (zp > nz) zp = 1; if (zm < 1) zm = nz; }
  const double Af = x > 1 ? A.a64x[g - 1] : (d.px ? A.a64x[g + nx - 1] : h.cond(xm, y, z, x, y, z));
  const double Bf = h.cond(xp, y, z, x, y, z);
  const double Df = y > 1 ? A.a64y[g - nx] : (d.py ? A.a64y[g + (ny - 1) * nx] : h.cond(x, ym, z, x, y, z));
  const double Ef = h.cond(x, yp, z, x, y, z);
  const double Ff = z > 1 ? A.a64z[g - nxy] : (d.pz ? A.a64z[g + (nz - 1) * nxy] : h.cond(x, y, zm, x, y, z));
  const double Gf = h.cond(x, y, zp, x, y, z);
  const double dg = -(Af + Bf + Df + Ef + Ff + Gf) - alpha;
  A.diag[g] = dg;
  auto keep = [](double v) { return fabs(v) < kTiny ? 0.0 : v; };   // sparse_Hmatrix's drop rule
  double cxv = 0.0, cyv = 0.0, czv = 0.0;
  if (x < nx) cxv = keep(A.a64x[g]);
  else if (d.px && nx > 1) cxv = keep(Bf);
  if (ny > 1) {
    if (y < ny) cyv = keep(A.a64y[g]);
    else if (d.py) cyv = keep(Ef);
  }
  if (nz > 1) {
    if (z < nz) czv = keep(A.a64z[g]);
    else if (d.pz) czv = keep(Gf);
  }
  A.cx[g] = cxv;
  A.cy[g] = cyv;
  A.cz[g] = czv;
  // boundary(B), mod_boundary.f90:72-150
  double Bv = 0.0;
  const double kap = kappa[g];
  const int64_t c[3] = {x, y, z}, n[3] = {nx, ny, nz};
  const int per[3] = {d.px, d.py, d.pz};
  for (int a = 0; a < 3; ++a) {
    if (per[a]) continue;
    double L = d.len[a];
    if (c[a] == 1) {
      int f = 2 * a;
      if (bc.cg[f]) {
        Bv = bc.pd[f];
      } else {
        double kh = (2.0 * kap * bc.kb[f] / (kap + bc.kb[f])) / (L * L);
        if (kap != bc.kb[f]) kh = kh * bc.br;
        Bv = Bv + (kh) * bc.tb[f];
      }
    }
    if (c[a] == n[a]) {
      int f = 2 * a + 1;
      if (bc.cg[f]) {
        Bv = bc.pd[f];
      } else {
        double kh = (2.0 * kap * bc.kb[f] / (kap + bc.kb[f])) / (L * L);
        if (kap != bc.kb[f]) kh = kh * bc.br;
        Bv = Bv + (kh) * bc.tb[f];
      }
    }
  }
  A.bvec[g] = Bv;
  if (isnan(Bv)) atomicOr(&A.scal[inst].status, 1 << (HF_ENAN_B - HF_ENAN_B));
  if (dg >= 0.0) atomicOr(&A.scal[inst].devcheck, 2);
  A.sinv[g] = 1.0 / sqrt(fabs(dg));
  A.sinv32[g] = (float)A.sinv[g];
}

// ---- Jacobi scaling: sinv = 1/sqrt|H_II|, a = -c * sinv_I * sinv_E ----------------------------
__global__ void k_sinv(DevArrays A) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const InstDesc& d = A.inst[A.tile_inst[g / kTile]];
  if (g - d.off >= d.n) { A.sinv[g] = 0.0; return; }
  double dg = A.diag[g];
  if (dg >= 0.0) atomicOr(&A.scal[A.tile_inst[g / kTile]].devcheck, 2);   // NaN passes: B check reports it
  A.sinv[g] = 1.0 / sqrt(fabs(dg));
  A.sinv32[g] = (float)A.sinv[g];
}

__global__ void k_scale(DevArrays A) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const InstDesc& d = A.inst[A.tile_inst[g / kTile]];
  const int64_t l = g - d.off;
  if (l >= d.n) return;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  const int64_t x = l % nx, y = (l / nx) % ny, z = l / nxy;
  const double si = A.sinv[g];
  int64_t ex = x + 1 < nx ? g + 1 : g - (nx - 1);
  int64_t ey = y + 1 < ny ? g + nx : g - (ny - 1) * nx;
  int64_t ez = z + 1 < nz ? g + nxy : g - (nz - 1) * nxy;
  double ax = -A.cx[g] * si * A.sinv[ex];
  double ay = -A.cy[g] * si * A.sinv[ey];
  double az = -A.cz[g] * si * A.sinv[ez];
  A.a64x[g] = ax; A.a64y[g] = ay; A.a64z[g] = az;
  const int64_t g4 = d.off4 + (z * ny + y) * d.sx + x;   // the FP32 layout (rows of sx cells)
  A.a32x[g4] = (float)ax; A.a32y[g4] = (float)ay; A.a32z[g4] = (float)az;
  // H*1: the diagonal plus every face of the row
  double rs = A.diag[g];
  if (nx > 1 && (x + 1 < nx || d.px)) rs += A.cx[g];
  if (nx > 1 && (x > 0 || d.px)) rs += A.cx[x > 0 ? g - 1 : g + nx - 1];
  if (ny > 1 && (y + 1 < ny || d.py)) rs += A.cy[g];
  if (ny > 1 && (y > 0 || d.py)) rs += A.cy[y > 0 ? g - nx : g + (ny - 1) * nx];
  if (nz > 1 && (z + 1 < nz || d.pz)) rs += A.cz[g];
  if (nz > 1 && (z > 0 || d.pz)) rs += A.cz[z > 0 ? g - nxy : g + (nz - 1) * nxy];
  A.rsum[g] = rs;
}

// ---- parity probe: COO in the reference's storage order (sparse_Hmatrix) --------------------
__global__ void k_coo_count(DevArrays A, const InstBC* bcs, const double* kappa, int inst,
                            int64_t* counts) {
  const InstDesc& d = A.inst[inst];
  int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= d.n) return;
  HM h{d, bcs[inst], kappa + d.off, A.rhoc + d.off, A.tau_s + d.off};
  int64_t j = l + 1, off[6];
  int ns = h.slots(off);
  int64_t cnt = 1;
  for (int k = 0; k < ns; ++k) {
    int64_t i = j + off[k];
    if (i > d.n) break;
    if (fabs(h.hmf(i, j)) < kTiny) continue;
    cnt += 2;
  }
  counts[l] = cnt;
}

__global__ void k_coo_write(DevArrays A, const InstBC* bcs, const double* kappa, int inst,
                            const int64_t* pos, int64_t* irow, int64_t* jcol, double* val) {
  const InstDesc& d = A.inst[inst];
  int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= d.n) return;
  HM h{d, bcs[inst], kappa + d.off, A.rhoc + d.off, A.tau_s + d.off};
  int64_t j = l + 1, off[6];
  int ns = h.slots(off);
  int64_t c = pos[l];
  irow[c] = j; jcol[c] = j; val[c] = h.hmf(j, j); ++c;
  for (int k = 0; k < ns; ++k) {
    int64_t i = j + off[k];
    if (i > d.n) break;
    double h0 = h.hmf(i, j);
    if (fabs(h0) < kTiny) continue;
    irow[c] = i; jcol[c] = j; val[c] = h0; ++c;
    irow[c] = j; jcol[c] = i; val[c] = h0; ++c;
  }
}

// ---- parity probe: y = H x in SRSax's accumulation order -------------------------------------
// Row I of the reference COO holds its entries in ascending column order (entries of earlier
// columns first, then the diagonal, then the upper entries), and SRSax adds them one at a time
// into b(I) = 0 (mod_Sparse.f90:304-313).
__global__ void k_apply_exact(DevArrays A, const double* xin, double* yout) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const InstDesc& d = A.inst[A.tile_inst[g / kTile]];
  const int64_t l = g - d.off;
  if (l >= d.n) return;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  const int64_t x = l % nx, y = (l / nx) % ny, z = l / nxy;
  const double* xs = xin + d.off;
  int64_t idx[7];
  double cf[7];
  int m = 0;
  idx[m] = l; cf[m] = A.diag[g]; ++m;
  auto add = [&](int64_t j, double c) { if (c != 0.0) { idx[m] = j; cf[m] = c; ++m; } };
  // + neighbours (face stored at this cell)
  if (nx > 1) add(x + 1 < nx ? l + 1 : l - (nx - 1), (x + 1 < nx || d.px) ? A.cx[g] : 0.0);
  if (ny > 1) add(y + 1 < ny ? l + nx : l - (ny - 1) * nx, (y + 1 < ny || d.py) ? A.cy[g] : 0.0);
  if (nz > 1) add(z + 1 < nz ? l + nxy : l - (nz - 1) * nxy, (z + 1 < nz || d.pz) ? A.cz[g] : 0.0);
  // - neighbours (face stored at the neighbour)
  if (nx > 1 && (x > 0 || d.px)) { int64_t w = x > 0 ? l - 1 : l + (nx - 1); add(w, A.cx[d.off + w]); }
  if (ny > 1 && (y > 0 || d.py)) { int64_t w = y > 0 ? l - nx : l + (ny - 1) * nx; add(w, A.cy[d.off + w]); }
  if (nz > 1 && (z > 0 || d.pz)) { int64_t w = z > 0 ? l - nxy : l + (nz - 1) * nxy; add(w, A.cz[d.off + w]); }
  // insertion sort by column (stable: equal columns hold equal values)
  for (int a = 1; a < m; ++a) {
    int64_t ki = idx[a]; double kc = cf[a]; int b = a - 1;
    while (b >= 0 && idx[b] > ki) { idx[b + 1] = idx[b]; cf[b + 1] = cf[b]; --b; }
    idx[b + 1] = ki; cf[b + 1] = kc;
  }
  double acc = 0.0;
  for (int a = 0; a < m; ++a) acc = acc + cf[a] * xs[idx[a]];
  yout[g] = acc;
}

// ---- launchers ------------------------------------------------------------------------------
static inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// ---- tabulated properties (extension of TempDepProp) ------------------------------------------
// After a step, every cell with a table takes kappa, rho and c at its new temperature T^n: rows
// (T ascending, kappa, rho, c) held constant below the first and above the last row, linear in
// between, in the oracle's operation order (compiled without contraction, so the values match
// bit for bit); then rho*c and tau'*rho*c follow, and the operator is rebuilt by k_assemble.
// Interval of T in a table (rows of T, kappa, rho, c with ascending T) and its fraction; the same
// search and fraction serve all three columns.  Outside the table: the end row, f = 0.
struct TableAt {
  const double* r0;
  const double* r1;
  double f;
  bool inside;
};

__device__ __forceinline__ TableAt table_at(const double* rows, int m, double T) {
  if (T <= rows[0]) return {rows, rows, 0.0, false};
  if (T >= rows[4 * (m - 1)]) return {rows + 4 * (m - 1), rows + 4 * (m - 1), 0.0, false};
  int k = 0;
  while (k + 1 < m - 1 && !(T < rows[4 * (k + 1)])) ++k;
  const double f = (T - rows[4 * k]) / (rows[4 * (k + 1)] - rows[4 * k]);
  return {rows + 4 * k, rows + 4 * (k + 1), f, true};
}

__device__ __forceinline__ double table_col(const TableAt& t, int col) {
  if (!t.inside) return t.r0[col];
  return t.r0[col] + t.f * (t.r1[col] - t.r0[col]);
}

__global__ void k_tempdep(DevArrays A, const int32_t* toff, const double* trows,
                          const int32_t* cell_table, double* kappa) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ncells) return;
  const int inst = A.tile_inst[g / kTile];
  const InstDesc& d = A.inst[inst];
  if (g - d.off >= d.n) return;
  if (g == d.off) A.scal[inst].hx_ok = 0;      // H changes: the stored products H T are stale
  const int32_t t = cell_table[g];
  if (t < 0) return;
  const double* rows = trows + 4 * (int64_t)toff[t];
  const int m = toff[t + 1] - toff[t];
  const double T = A.tbuf[A.scal[inst].role[0]][g];
  const TableAt at = table_at(rows, m, T);
  kappa[g] = table_col(at, 1);
  const double rc = table_col(at, 2) * table_col(at, 3);
  A.rhoc[g] = rc;
  A.ccat[g] = A.tau_s[g] * rc;
  A.scoef[g] = scoef(d, rc, A.ccat[g]);
}

cudaError_t launch_tempdep(Ctx& c) {
  k_tempdep<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A, c.d_toff, c.d_trows, c.d_cell_table,
                                                       c.asm_.kappa);
  k_faces_step<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A, c.d_bc, c.asm_.kappa);
  k_diag_step<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A, c.d_bc, c.asm_.kappa);
  k_scale<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}

cudaError_t launch_props(Ctx& c, const double* rho, const double* hc, const double* tau,
                         const double* em) {
  k_props<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A, rho, hc, tau, em);
  return cudaGetLastError();
}

cudaError_t launch_assemble(Ctx& c) {
  k_assemble<<<nblk(c.ncells, 128), 128, 0, c.stream>>>(c.A, c.d_bc, c.asm_.kappa);
  k_sinv<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A);
  k_scale<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A);
  return cudaGetLastError();
}

cudaError_t launch_coo(Ctx& c, int64_t inst, int64_t* d_counts, int64_t* d_irow, int64_t* d_jcol,
                       double* d_val, int64_t* d_pos, int phase) {
  const int64_t n = c.h_inst[inst].n;
  if (phase == 0)
    k_coo_count<<<nblk(n, 128), 128, 0, c.stream>>>(c.A, c.d_bc, c.asm_.kappa, (int)inst, d_counts);
  else
    k_coo_write<<<nblk(n, 128), 128, 0, c.stream>>>(c.A, c.d_bc, c.asm_.kappa, (int)inst, d_pos,
                                                    d_irow, d_jcol, d_val);
  return cudaGetLastError();
}

cudaError_t launch_apply(Ctx& c, const double* x, double* y) {
  k_apply_exact<<<nblk(c.ncells, 256), 256, 0, c.stream>>>(c.A, x, y);
  return cudaGetLastError();
}

}  // namespace hf
