// Oracle (test infrastructure): JACOBI_TRANS restated from
// src/diablo.F90:1088-1570 of the reference.  Arrays are zero-filled at
// allocation, which makes the reads of not-yet-set entries that the Fortran
// performs (e.g. the J=0 row read by the K=0 extrapolation loop,
// diablo.F90:1282-1293) deterministic.
#include "ekref.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct A3 {  // (1:NZ+1, 1:NY+1, 1:2) allocatable of JACOBI_TRANS
  int nz1, ny1;
  std::vector<double> v;
  A3(int nz, int ny) : nz1(nz + 1), ny1(ny + 1), v(size_t(2) * (nz + 1) * (ny + 1), 0.0) {}
  double &operator()(int k, int j, int f) { return v[((size_t)(f - 1) * ny1 + (j - 1)) * nz1 + (k - 1)]; }
};

struct Terms {  // inverse metrics on the faces, (1:NZ+1, 1:NY+1, 1:2)
  A3 zeta_x, zeta_y, eta_x, eta_y, in_jaco;
  Terms(int nz, int ny) : zeta_x(nz, ny), zeta_y(nz, ny), eta_x(nz, ny), eta_y(nz, ny), in_jaco(nz, ny) {}
};

// diablo.F90:1164-1241: face derivatives of the grid, truncated to 1e-8,
// the face Jacobians and the inverse metrics.
void grid_terms(const ek_params *p, const double *xpoint, const double *ypoint, Terms &t) {
  const int NY = p->ny, NZ = p->nz;
  auto XP = [&](int k, int j) { return xpoint[(size_t)j * (NZ + 2) + k]; };
  auto YP = [&](int k, int j) { return ypoint[(size_t)j * (NZ + 2) + k]; };
  A3 x_zeta(NZ, NY), y_zeta(NZ, NY), x_eta(NZ, NY), y_eta(NZ, NY);
  A3 &zeta_x = t.zeta_x, &zeta_y = t.zeta_y, &eta_x = t.eta_x, &eta_y = t.eta_y, &in_jaco = t.in_jaco;
  // diablo.F90:1164-1189
  for (int j = 1; j <= NY; ++j)
    for (int k = 1; k <= NZ; ++k) {
      x_zeta(k, j, 1) = XP(k + 1, j) - XP(k, j);
      x_zeta(k, j, 2) = 0.250 * (XP(k + 1, j + 1) + XP(k + 1, j) - XP(k - 1, j + 1) - XP(k - 1, j));
      y_zeta(k, j, 1) = YP(k + 1, j) - YP(k, j);
      y_zeta(k, j, 2) = 0.250 * (YP(k + 1, j + 1) + YP(k + 1, j) - YP(k - 1, j + 1) - YP(k - 1, j));
      x_eta(k, j, 2) = XP(k, j + 1) - XP(k, j);
      x_eta(k, j, 1) = 0.250 * (XP(k, j + 1) + XP(k + 1, j + 1) - XP(k, j - 1) - XP(k + 1, j - 1));
      y_eta(k, j, 1) = 0.250 * (YP(k, j + 1) + YP(k + 1, j + 1) - YP(k, j - 1) - YP(k + 1, j - 1));
      y_eta(k, j, 2) = (YP(k, j + 1) - YP(k, j));
    }
  // diablo.F90:1192-1216 (one-sided linear extrapolations, in Fortran order)
  for (int k = 1; k <= NZ + 1; ++k) {
    x_eta(k, 1, 1) = 2.0 * x_eta(k, 2, 1) - x_eta(k, 3, 1);
    for (int f = 1; f <= 2; ++f) {
      x_eta(k, NY + 1, f) = 2.0 * x_eta(k, NY, f) - x_eta(k, NY - 1, f);
      x_zeta(k, NY + 1, f) = 2.0 * x_zeta(k, NY, f) - x_zeta(k, NY - 1, f);
    }
    y_eta(k, 1, 1) = 2.0 * y_eta(k, 2, 1) - y_eta(k, 3, 1);
    for (int f = 1; f <= 2; ++f) {
      y_eta(k, NY + 1, f) = 2.0 * y_eta(k, NY, f) - y_eta(k, NY - 1, f);
      y_zeta(k, NY + 1, f) = 2.0 * y_zeta(k, NY, f) - y_zeta(k, NY - 1, f);
    }
  }
  for (int j = 1; j <= NY + 1; ++j) {
    x_zeta(1, j, 2) = 2.0 * x_zeta(2, j, 2) - x_zeta(3, j, 2);
    for (int f = 1; f <= 2; ++f) {
      x_zeta(NZ + 1, j, f) = 2.0 * x_zeta(NZ, j, f) - x_zeta(NZ - 1, j, f);
      x_eta(NZ + 1, j, f) = 2.0 * x_eta(NZ, j, f) - x_eta(NZ - 1, j, f);
    }
    y_zeta(1, j, 2) = 2.0 * y_zeta(2, j, 2) - y_zeta(3, j, 2);
    for (int f = 1; f <= 2; ++f) {
      y_zeta(NZ + 1, j, f) = 2.0 * y_zeta(NZ, j, f) - y_zeta(NZ - 1, j, f);
      y_eta(NZ + 1, j, f) = 2.0 * y_eta(NZ, j, f) - y_eta(NZ - 1, j, f);
    }
  }
  // diablo.F90:1219-1229: truncate to 1e-8 with AINT (toward zero).
  const double e8 = 1.0e-8;
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f) {
        x_zeta(k, j, f) = std::trunc(x_zeta(k, j, f) * 100000000.0) * e8;
        x_eta(k, j, f) = std::trunc(x_eta(k, j, f) * 100000000.0) * e8;
        y_zeta(k, j, f) = std::trunc(y_zeta(k, j, f) * 100000000.0) * e8;
        y_eta(k, j, f) = std::trunc(y_eta(k, j, f) * 100000000.0) * e8;
      }
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f) {
        in_jaco(k, j, f) = x_zeta(k, j, f) * y_eta(k, j, f) - x_eta(k, j, f) * y_zeta(k, j, f);
        zeta_x(k, j, f) = y_eta(k, j, f) / in_jaco(k, j, f);
        eta_x(k, j, f) = -y_zeta(k, j, f) / in_jaco(k, j, f);
        zeta_y(k, j, f) = -x_eta(k, j, f) / in_jaco(k, j, f);
        eta_y(k, j, f) = x_zeta(k, j, f) / in_jaco(k, j, f);
      }
}

}  // namespace

extern "C" int ekref_metrics_from_grid(const ek_params *p, const double *xpoint,
                                       const double *ypoint, double *int_jacob,
                                       double *gmat_11, double *gmat_12, double *gmat_22,
                                       double *cjob_11, double *cjob_12, double *cjob_21,
                                       double *cjob_22, double *th_bar) {
  const int NY = p->ny, NZ = p->nz;
  if (NY < 3 || NZ < 3) return EK_ERR_ARG;
  const int LD = NZ + 3;                        // leading dim of (0:NZ+2, 0:NY+2)
  const size_t N2 = (size_t)LD * (NY + 3);
  auto YP = [&](int k, int j) { return ypoint[(size_t)j * (NZ + 2) + k]; };
  auto M2 = [&](double *a, int k, int j) -> double & { return a[(size_t)j * LD + k]; };
  auto M3 = [&](double *a, int k, int j, int f) -> double & { return a[(size_t)(f - 1) * N2 + (size_t)j * LD + k]; };

  for (double *a : {int_jacob}) std::memset(a, 0, sizeof(double) * N2);
  for (double *a : {gmat_11, gmat_12, gmat_22, cjob_11, cjob_12, cjob_21, cjob_22})
    std::memset(a, 0, sizeof(double) * 2 * N2);
  if (th_bar) std::memset(th_bar, 0, sizeof(double) * N2);

  Terms t(NZ, NY);
  grid_terms(p, xpoint, ypoint, t);
  A3 &zeta_x = t.zeta_x, &zeta_y = t.zeta_y, &eta_x = t.eta_x, &eta_y = t.eta_y, &in_jaco = t.in_jaco;

  // TH_BAR (diablo.F90:1152-1160): CONT_STRAT profile; otherwise the caller
  // supplies density_data_input.dat values, which this helper leaves at 0.
  if (th_bar && p->cont_strat)
    for (int j = 0; j <= NY + 1; ++j)
      for (int k = 0; k <= NZ + 1; ++k) M2(th_bar, k, j) = (-YP(k, j) + YP(0, NY + 1));

  // diablo.F90:1246-1263
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k) {
      for (int f = 1; f <= 2; ++f) {
        M3(gmat_11, k, j, f) = (zeta_x(k, j, f) * zeta_x(k, j, f) + zeta_y(k, j, f) * zeta_y(k, j, f)) * in_jaco(k, j, f);
        M3(gmat_12, k, j, f) = (zeta_x(k, j, f) * eta_x(k, j, f) + zeta_y(k, j, f) * eta_y(k, j, f)) * in_jaco(k, j, f);
        M3(gmat_22, k, j, f) = (eta_x(k, j, f) * eta_x(k, j, f) + eta_y(k, j, f) * eta_y(k, j, f)) * in_jaco(k, j, f);
        M3(cjob_11, k, j, f) = zeta_x(k, j, f) * in_jaco(k, j, f);
        M3(cjob_12, k, j, f) = zeta_y(k, j, f) * in_jaco(k, j, f);
        M3(cjob_21, k, j, f) = eta_x(k, j, f) * in_jaco(k, j, f);
        M3(cjob_22, k, j, f) = eta_y(k, j, f) * in_jaco(k, j, f);
      }
    }
  // diablo.F90:1267-1287
  for (int j = 1; j <= NY; ++j)
    for (int k = 1; k <= NZ; ++k)
      M2(int_jacob, k, j) = 0.250 * (in_jaco(k, j, 1) + in_jaco(k, j, 2) + in_jaco(k, j + 1, 1) + in_jaco(k + 1, j, 2));
  for (int j = 0; j <= NY + 1; ++j) {
    M2(int_jacob, NZ + 1, j) = 2.0 * M2(int_jacob, NZ, j) - M2(int_jacob, NZ - 1, j);
    M2(int_jacob, 0, j) = 2.0 * M2(int_jacob, 1, j) - M2(int_jacob, 2, j);
  }
  for (int k = 0; k <= NZ + 1; ++k) {
    M2(int_jacob, k, NY + 1) = 2.0 * M2(int_jacob, k, NY) - M2(int_jacob, k, NY - 1);
    M2(int_jacob, k, 0) = 2.0 * M2(int_jacob, k, 1) - M2(int_jacob, k, 2);
  }
  M2(int_jacob, 0, 0) = 0.5 * (2.0 * M2(int_jacob, 1, 0) - M2(int_jacob, 2, 0) + 2.0 * M2(int_jacob, 0, 1) - M2(int_jacob, 0, 2));
  M2(int_jacob, NZ + 1, NY + 1) = 0.5 * (2.0 * M2(int_jacob, NZ, NY + 1) - M2(int_jacob, NZ - 1, NY + 1) +
                                         2.0 * M2(int_jacob, NZ + 1, NY) - M2(int_jacob, NZ + 1, NY - 1));
  double *all7[7] = {cjob_11, cjob_12, cjob_21, cjob_22, gmat_11, gmat_12, gmat_22};
  // diablo.F90:1295-1321 (K=0 column first, then the J=0 row)
  for (int j = 0; j <= NY + 1; ++j)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all7) M3(a, 0, j, f) = 2.0 * M3(a, 1, j, f) - M3(a, 2, j, f);
  for (int k = 0; k <= NZ + 1; ++k)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all7) M3(a, k, 0, f) = 2.0 * M3(a, k, 1, f) - M3(a, k, 2, f);
  // diablo.F90:1323-1341 corner fixes; the GMAT_22 line is written twice
  // (the first one with GMAT_12 values) and GMAT_12(0,0) is left alone,
  // as in the reference.
  for (int f = 1; f <= 2; ++f) {
    auto corner = [&](double *src) {
      return 0.5 * (2.0 * M3(src, 0, 1, f) - M3(src, 0, 2, f) + 2.0 * M3(src, 1, 0, f) - M3(src, 2, 0, f));
    };
    M3(gmat_11, 0, 0, f) = corner(gmat_11);
    M3(gmat_22, 0, 0, f) = corner(gmat_12);
    M3(gmat_22, 0, 0, f) = corner(gmat_22);
    M3(cjob_11, 0, 0, f) = corner(cjob_11);
    M3(cjob_12, 0, 0, f) = corner(cjob_12);
    M3(cjob_21, 0, 0, f) = corner(cjob_21);
    M3(cjob_22, 0, 0, f) = corner(cjob_22);
  }
  // diablo.F90:1344-1376: index NZ+2 / NY+2 copies used by the MG coefficients.
  for (int f = 1; f <= 2; ++f) {
    for (int k = 0; k <= NZ + 1; ++k)
      for (double *a : all7) M3(a, k, NY + 2, f) = M3(a, k, NY + 1, f);
    for (int j = 0; j <= NY + 1; ++j)
      for (double *a : all7) M3(a, NZ + 2, j, f) = M3(a, NZ + 1, j, f);
    for (double *a : all7) M3(a, NZ + 2, NY + 2, f) = M3(a, NZ + 1, NY + 1, f);
  }
  return EK_OK;
}

// The LES metric variants of JACOBI_TRANS (diablo.F90:1379-1467): GMAT_*_z
// double the zeta_x/eta_x products, GMAT_*_y the zeta_y/eta_y products.  The
// K = 0 column is extrapolated first (its J = 0 entry from rows not yet set,
// overwritten by the J = 0 row that follows), then the J = 0 row; the (0,0)
// corner lines write GMAT_22_* twice (the first time with GMAT_12_* values)
// and leave GMAT_12_*(0,0) at its row extrapolation, as in the reference.
extern "C" int ekref_les_metrics_from_grid(const ek_params *p, const double *xpoint, const double *ypoint,
                                           double *g11y, double *g12y, double *g22y, double *g11z,
                                           double *g12z, double *g22z) {
  const int NY = p->ny, NZ = p->nz;
  if (NY < 3 || NZ < 3) return EK_ERR_ARG;
  const int LD = NZ + 3;
  const size_t N2 = (size_t)LD * (NY + 3);
  auto M3 = [&](double *a, int k, int j, int f) -> double & { return a[(size_t)(f - 1) * N2 + (size_t)j * LD + k]; };
  double *all6[6] = {g11z, g12z, g22z, g11y, g12y, g22y};
  for (double *a : all6) std::memset(a, 0, sizeof(double) * 2 * N2);
  Terms t(NZ, NY);
  grid_terms(p, xpoint, ypoint, t);
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f) {
        const double zx = t.zeta_x(k, j, f), zy = t.zeta_y(k, j, f), ex = t.eta_x(k, j, f), ey = t.eta_y(k, j, f);
        const double ij = t.in_jaco(k, j, f);
        M3(g11z, k, j, f) = (2.0 * zx * zx + zy * zy) * ij;
        M3(g12z, k, j, f) = (2.0 * zx * ex + zy * ey) * ij;
        M3(g22z, k, j, f) = (2.0 * ex * ex + ey * ey) * ij;
        M3(g11y, k, j, f) = (zx * zx + 2.0 * zy * zy) * ij;
        M3(g12y, k, j, f) = (zx * ex + 2.0 * zy * ey) * ij;
        M3(g22y, k, j, f) = (ex * ex + 2.0 * ey * ey) * ij;
      }
  for (int j = 0; j <= NY + 1; ++j)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all6) M3(a, 0, j, f) = 2.0 * M3(a, 1, j, f) - M3(a, 2, j, f);
  for (int k = 0; k <= NZ + 1; ++k)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all6) M3(a, k, 0, f) = 2.0 * M3(a, k, 1, f) - M3(a, k, 2, f);
  for (int f = 1; f <= 2; ++f) {
    auto corner = [&](double *src) {
      return 0.5 * (2.0 * M3(src, 0, 1, f) - M3(src, 0, 2, f) + 2.0 * M3(src, 1, 0, f) - M3(src, 2, 0, f));
    };
    M3(g11z, 0, 0, f) = corner(g11z);
    M3(g22z, 0, 0, f) = corner(g12z);
    M3(g22z, 0, 0, f) = corner(g22z);
    M3(g11y, 0, 0, f) = corner(g11y);
    M3(g22y, 0, 0, f) = corner(g12y);
    M3(g22y, 0, 0, f) = corner(g22y);
  }
  for (int f = 1; f <= 2; ++f) {
    for (int k = 0; k <= NZ + 1; ++k)
      for (double *a : all6) M3(a, k, NY + 2, f) = M3(a, k, NY + 1, f);
    for (int j = 0; j <= NY + 1; ++j)
      for (double *a : all6) M3(a, NZ + 2, j, f) = M3(a, NZ + 1, j, f);
    for (double *a : all6) M3(a, NZ + 2, NY + 2, f) = M3(a, NZ + 1, NY + 1, f);
  }
  return EK_OK;
}
