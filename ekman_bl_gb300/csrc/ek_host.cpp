// Host-side precomputation for the GB300 duct substep: metrics from grid
// points (JACOBI_TRANS), boundary-row tables (APPLY_BC_*), Thomas factors of
// the ADI lines and the multigrid plan (levels, kx-independent 9-point
// coefficients of dismd2cr, and the k-cycle schedule of mud2cr1/kcymd2cr).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ek_internal.h"

namespace ek {

namespace {

// The face derivatives of the grid (x_zeta, y_zeta, x_eta, y_eta on faces
// 1 and 2), their one-sided extrapolations and the AINT truncation to 1e-8
// (diablo.F90:1164-1229), in arrays (1:NZ+1, 1:NY+1, 2).
struct GridDeriv {
  int n1, m1;
  std::vector<double> xz, yz, xe, ye;
  GridDeriv(int nz, int ny) : n1(nz + 1), m1(ny + 1), xz(2 * (size_t)(nz + 1) * (ny + 1), 0.0), yz(xz), xe(xz), ye(xz) {}
  double &operator()(std::vector<double> &v, int k, int j, int f) {
    return v[((size_t)(f - 1) * m1 + (j - 1)) * n1 + (k - 1)];
  }
};

void grid_derivatives(const ek_params *p, const double *xpoint, const double *ypoint, GridDeriv &g) {
  const int NY = p->ny, NZ = p->nz;
  auto &xz = g.xz, &yz = g.yz, &xe = g.xe, &ye = g.ye;
  auto T = [&](std::vector<double> &v, int k, int j, int f) -> double & { return g(v, k, j, f); };
  auto XP = [&](int k, int j) { return xpoint[(size_t)j * (NZ + 2) + k]; };
  auto YP = [&](int k, int j) { return ypoint[(size_t)j * (NZ + 2) + k]; };
  for (int j = 1; j <= NY; ++j)
    for (int k = 1; k <= NZ; ++k) {
      T(xz, k, j, 1) = XP(k + 1, j) - XP(k, j);
      T(xz, k, j, 2) = 0.250 * (XP(k + 1, j + 1) + XP(k + 1, j) - XP(k - 1, j + 1) - XP(k - 1, j));
      T(yz, k, j, 1) = YP(k + 1, j) - YP(k, j);
      T(yz, k, j, 2) = 0.250 * (YP(k + 1, j + 1) + YP(k + 1, j) - YP(k - 1, j + 1) - YP(k - 1, j));
      T(xe, k, j, 2) = XP(k, j + 1) - XP(k, j);
      T(xe, k, j, 1) = 0.250 * (XP(k, j + 1) + XP(k + 1, j + 1) - XP(k, j - 1) - XP(k + 1, j - 1));
      T(ye, k, j, 1) = 0.250 * (YP(k, j + 1) + YP(k + 1, j + 1) - YP(k, j - 1) - YP(k + 1, j - 1));
      T(ye, k, j, 2) = (YP(k, j + 1) - YP(k, j));
    }
  for (int k = 1; k <= NZ + 1; ++k) {
    T(xe, k, 1, 1) = 2.0 * T(xe, k, 2, 1) - T(xe, k, 3, 1);
    for (int f = 1; f <= 2; ++f) {
      T(xe, k, NY + 1, f) = 2.0 * T(xe, k, NY, f) - T(xe, k, NY - 1, f);
      T(xz, k, NY + 1, f) = 2.0 * T(xz, k, NY, f) - T(xz, k, NY - 1, f);
    }
    T(ye, k, 1, 1) = 2.0 * T(ye, k, 2, 1) - T(ye, k, 3, 1);
    for (int f = 1; f <= 2; ++f) {
      T(ye, k, NY + 1, f) = 2.0 * T(ye, k, NY, f) - T(ye, k, NY - 1, f);
      T(yz, k, NY + 1, f) = 2.0 * T(yz, k, NY, f) - T(yz, k, NY - 1, f);
    }
  }
  for (int j = 1; j <= NY + 1; ++j) {
    T(xz, 1, j, 2) = 2.0 * T(xz, 2, j, 2) - T(xz, 3, j, 2);
    for (int f = 1; f <= 2; ++f) {
      T(xz, NZ + 1, j, f) = 2.0 * T(xz, NZ, j, f) - T(xz, NZ - 1, j, f);
      T(xe, NZ + 1, j, f) = 2.0 * T(xe, NZ, j, f) - T(xe, NZ - 1, j, f);
    }
    T(yz, 1, j, 2) = 2.0 * T(yz, 2, j, 2) - T(yz, 3, j, 2);
    for (int f = 1; f <= 2; ++f) {
      T(yz, NZ + 1, j, f) = 2.0 * T(yz, NZ, j, f) - T(yz, NZ - 1, j, f);
      T(ye, NZ + 1, j, f) = 2.0 * T(ye, NZ, j, f) - T(ye, NZ - 1, j, f);
    }
  }
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f)
        for (auto *v : {&xz, &xe, &yz, &ye}) T(*v, k, j, f) = std::trunc(T(*v, k, j, f) * 100000000.0) * 1.0e-8;
}

}  // namespace

// JACOBI_TRANS (src/diablo.F90:1088-1570).  Same statement order as the
// Fortran; arrays start zero-filled as a fresh ALLOCATE.
int metrics_from_grid_host(const ek_params *p, const double *xpoint, const double *ypoint, double *int_jacob,
                           double *gmat_11, double *gmat_12, double *gmat_22, double *cjob_11, double *cjob_12,
                           double *cjob_21, double *cjob_22, double *th_bar) {
  const int NY = p->ny, NZ = p->nz;
  if (NY < 3 || NZ < 3 || !xpoint || !ypoint) return EK_ERR_ARG;
  const int LD = NZ + 3;
  const size_t N2 = (size_t)LD * (NY + 3);
  const int n1 = NZ + 1, m1 = NY + 1;  // extents of the temporaries (1:NZ+1, 1:NY+1, 2)
  std::vector<double> ij(2 * (size_t)n1 * m1, 0.0);
  auto T = [&](std::vector<double> &v, int k, int j, int f) -> double & {
    return v[((size_t)(f - 1) * m1 + (j - 1)) * n1 + (k - 1)];
  };
  auto YP = [&](int k, int j) { return ypoint[(size_t)j * (NZ + 2) + k]; };
  auto M2 = [&](double *a, int k, int j) -> double & { return a[(size_t)j * LD + k]; };
  auto M3 = [&](double *a, int k, int j, int f) -> double & { return a[(size_t)(f - 1) * N2 + (size_t)j * LD + k]; };
  std::memset(int_jacob, 0, sizeof(double) * N2);
  for (double *a : {gmat_11, gmat_12, gmat_22, cjob_11, cjob_12, cjob_21, cjob_22}) std::memset(a, 0, sizeof(double) * 2 * N2);
  if (th_bar) {
    std::memset(th_bar, 0, sizeof(double) * N2);
    if (p->cont_strat)
      for (int j = 0; j <= NY + 1; ++j)
        for (int k = 0; k <= NZ + 1; ++k) M2(th_bar, k, j) = (-YP(k, j) + YP(0, NY + 1));
  }
  GridDeriv gd(NZ, NY);
  grid_derivatives(p, xpoint, ypoint, gd);
  auto &xz = gd.xz, &yz = gd.yz, &xe = gd.xe, &ye = gd.ye;
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f) {
        const double J = T(xz, k, j, f) * T(ye, k, j, f) - T(xe, k, j, f) * T(yz, k, j, f);
        T(ij, k, j, f) = J;
        const double zxv = T(ye, k, j, f) / J, exv = -T(yz, k, j, f) / J;
        const double zyv = -T(xe, k, j, f) / J, eyv = T(xz, k, j, f) / J;
        M3(gmat_11, k, j, f) = (zxv * zxv + zyv * zyv) * J;
        M3(gmat_12, k, j, f) = (zxv * exv + zyv * eyv) * J;
        M3(gmat_22, k, j, f) = (exv * exv + eyv * eyv) * J;
        M3(cjob_11, k, j, f) = zxv * J;
        M3(cjob_12, k, j, f) = zyv * J;
        M3(cjob_21, k, j, f) = exv * J;
        M3(cjob_22, k, j, f) = eyv * J;
      }
  for (int j = 1; j <= NY; ++j)
    for (int k = 1; k <= NZ; ++k)
      M2(int_jacob, k, j) = 0.250 * (T(ij, k, j, 1) + T(ij, k, j, 2) + T(ij, k, j + 1, 1) + T(ij, k + 1, j, 2));
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
  for (int j = 0; j <= NY + 1; ++j)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all7) M3(a, 0, j, f) = 2.0 * M3(a, 1, j, f) - M3(a, 2, j, f);
  for (int k = 0; k <= NZ + 1; ++k)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all7) M3(a, k, 0, f) = 2.0 * M3(a, k, 1, f) - M3(a, k, 2, f);
  for (int f = 1; f <= 2; ++f) {
    auto corner = [&](double *s) {
      return 0.5 * (2.0 * M3(s, 0, 1, f) - M3(s, 0, 2, f) + 2.0 * M3(s, 1, 0, f) - M3(s, 2, 0, f));
    };
    M3(gmat_11, 0, 0, f) = corner(gmat_11);
    M3(gmat_22, 0, 0, f) = corner(gmat_12);  // overwritten on the next line, as in the reference
    M3(gmat_22, 0, 0, f) = corner(gmat_22);
    M3(cjob_11, 0, 0, f) = corner(cjob_11);
    M3(cjob_12, 0, 0, f) = corner(cjob_12);
    M3(cjob_21, 0, 0, f) = corner(cjob_21);
    M3(cjob_22, 0, 0, f) = corner(cjob_22);
  }
  for (int f = 1; f <= 2; ++f) {
    for (int k = 0; k <= NZ + 1; ++k)
      for (double *a : all7) M3(a, k, NY + 2, f) = M3(a, k, NY + 1, f);
    for (int j = 0; j <= NY + 1; ++j)
      for (double *a : all7) M3(a, NZ + 2, j, f) = M3(a, NZ + 1, j, f);
    for (double *a : all7) M3(a, NZ + 2, NY + 2, f) = M3(a, NZ + 1, NY + 1, f);
  }
  return EK_OK;
}


// The LES metric variants GMAT_*_y / GMAT_*_z of JACOBI_TRANS
// (diablo.F90:1379-1467): the zeta_x/eta_x products doubled (_z) or the
// zeta_y/eta_y products doubled (_y); the K = 0 column and then the J = 0
// row extrapolated linearly; the (0,0) corner averaged for GMAT_11_* and
// GMAT_22_* (the reference writes the GMAT_22_* corner twice, first from
// GMAT_12_*, and keeps GMAT_12_*(0,0) from the row extrapolation); index
// NZ+2 / NY+2 copies.
int les_metrics_from_grid_host(const ek_params *p, const double *xpoint, const double *ypoint, double *g11y,
                               double *g12y, double *g22y, double *g11z, double *g12z, double *g22z) {
  const int NY = p->ny, NZ = p->nz;
  if (NY < 3 || NZ < 3 || !xpoint || !ypoint || !g11y || !g12y || !g22y || !g11z || !g12z || !g22z) return EK_ERR_ARG;
  const int LD = NZ + 3;
  const size_t N2 = (size_t)LD * (NY + 3);
  auto M3 = [&](double *a, int k, int j, int f) -> double & { return a[(size_t)(f - 1) * N2 + (size_t)j * LD + k]; };
  double *all6[6] = {g11z, g12z, g22z, g11y, g12y, g22y};
  for (double *a : all6) std::memset(a, 0, sizeof(double) * 2 * N2);
  GridDeriv gd(NZ, NY);
  grid_derivatives(p, xpoint, ypoint, gd);
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 1; k <= NZ + 1; ++k)
      for (int f = 1; f <= 2; ++f) {
        const double xz = gd(gd.xz, k, j, f), yz = gd(gd.yz, k, j, f), xe = gd(gd.xe, k, j, f), ye = gd(gd.ye, k, j, f);
        const double J = xz * ye - xe * yz;
        const double zx = ye / J, ex = -yz / J, zy = -xe / J, ey = xz / J;
        M3(g11z, k, j, f) = (2.0 * zx * zx + zy * zy) * J;
        M3(g12z, k, j, f) = (2.0 * zx * ex + zy * ey) * J;
        M3(g22z, k, j, f) = (2.0 * ex * ex + ey * ey) * J;
        M3(g11y, k, j, f) = (zx * zx + 2.0 * zy * zy) * J;
        M3(g12y, k, j, f) = (zx * ex + 2.0 * zy * ey) * J;
        M3(g22y, k, j, f) = (ex * ex + 2.0 * ey * ey) * J;
      }
  for (int j = 0; j <= NY + 1; ++j)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all6) M3(a, 0, j, f) = 2.0 * M3(a, 1, j, f) - M3(a, 2, j, f);
  for (int k = 0; k <= NZ + 1; ++k)
    for (int f = 1; f <= 2; ++f)
      for (double *a : all6) M3(a, k, 0, f) = 2.0 * M3(a, k, 1, f) - M3(a, k, 2, f);
  for (int f = 1; f <= 2; ++f) {
    auto corner = [&](double *s) {
      return 0.5 * (2.0 * M3(s, 0, 1, f) - M3(s, 0, 2, f) + 2.0 * M3(s, 1, 0, f) - M3(s, 2, 0, f));
    };
    M3(g11z, 0, 0, f) = corner(g11z);
    M3(g22z, 0, 0, f) = corner(g22z);
    M3(g11y, 0, 0, f) = corner(g11y);
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

static void bc_lhs(int field, int dir, const ek_params &p, const Dims &d, int row, double &L, double &D, double &U);

// Boundary rows of APPLY_BC_{TH,1,2,3}_{LOWER,UPPER,LEFT,RIGHT}
// (src/boundary.F90:124-1763) for the supported codes with IC_TYPE = 7.
// field: 0 TH, 1 U1, 2 U2, 3 U3; dir 0 = y lines, 1 = z lines.  Rows are
// listed in the order the routine writes them (later rows win).
int build_bc_sets(Ctx &c, std::vector<double> &w, const std::vector<double> &jac, const std::vector<double> &c22) {
  const ek_params &p = c.p;
  const Dims &d = c.d;
  const int NY = d.NY, NZ = d.NZ;
  auto J2 = [&](int k, int j) { return jac[d.m2(k, j)]; };
  auto C22 = [&](int k, int j, int f) { return c22[d.m3(k, j, f)]; };
  w.clear();
  for (int f = 0; f < 4; ++f) {
    const int *bc = (f == 0) ? p.th_bc : (f == 1) ? p.u_bc : (f == 2) ? p.v_bc : p.w_bc;
    const double *c1 = (f == 0) ? p.th_bc_c1 : (f == 1) ? p.u_bc_c1 : (f == 2) ? p.v_bc_c1 : p.w_bc_c1;
    // ---- y lines (LOWER then UPPER) ----
    BcSet &y = c.bc[f][0];
    y = BcSet{};
    auto addy = [&](int row, int kind, int src, double val, double l, double dd, double u) {
      (void)l; (void)dd; (void)u;
      y.r[y.n++] = BcRow{row, kind, src, val};
    };
    const int lo = bc[EK_YMIN], hi = bc[EK_YMAX];
    if (lo == 0) addy(0, 0, 0, c1[EK_YMIN], 0, 1, 0);
    else if (lo == 1 || (f == 0 && lo == 5)) {
      if (f == 0) {  // VECY(0) = C1/(0.5*(CJOB_22(K,1,2)+CJOB_22(K+1,1,1)))*INT_JACOB(K,1)
        // stored as the factor that multiplies C1: (1/(0.5*(..)))*J, so that
        // C1*w rounds like C1/(0.5*(..))*J up to one ulp
        const int off = (int)w.size();
        y.weight_off = off;
        for (int k = 0; k < d.NZ2; ++k) w.push_back(1.0 / (0.5 * (C22(k, 1, 2) + C22(k + 1, 1, 1))) * J2(k, 1));
        addy(0, 2, off, c1[EK_YMIN], 0, -1, 1);
      } else if (f == 3) addy(0, 0, 0, c1[EK_YMIN], 0, -1, 1);
      else addy(1, 0, 0, c1[EK_YMIN], 0, -1, 1);
    } else if (lo == 6) addy(0, 1, NY, 0.0, 0, 1, 0);
    else return EK_ERR_ARG;
    if (hi == 0) {
      addy(NY + 1, 0, 0, c1[EK_YMAX], 0, 1, 0);
      if (f == 2 || f == 3) addy(NY, 0, 0, c1[EK_YMAX], 0, 1, 0);
    } else if (hi == 1) {
      if (f == 0) {
        // two Neumann rows with metric weights (APPLY_BC_TH_UPPER)
        const int off = (int)w.size();
        for (int k = 0; k < d.NZ2; ++k) w.push_back(0.5 * (J2(k, NY) + J2(k, NY - 1)) / C22(k, NY - 1, 1));
        for (int k = 0; k < d.NZ2; ++k) w.push_back(0.5 * (J2(k, NY + 1) + J2(k, NY)) / C22(k, NY, 1));
        y.r[y.n++] = BcRow{NY, 2, off, c1[EK_YMAX]};
        y.r[y.n++] = BcRow{NY + 1, 2, off + d.NZ2, c1[EK_YMAX]};
      } else if (f == 2) addy(NY, 0, 0, c1[EK_YMAX], -1, 1, 0);
      else addy(NY + 1, 0, 0, c1[EK_YMAX], -1, 1, 0);
    } else if (hi == 6) addy(NY + 1, 1, 1, 0.0, 0, 1, 0);
    else return EK_ERR_ARG;
    // ---- z lines (LEFT then RIGHT) ----
    BcSet &z = c.bc[f][1];
    z = BcSet{};
    const int zl = bc[EK_ZMIN], zr = bc[EK_ZMAX];
    if (zl == 0) {
      if (f == 2 || f == 3) return EK_ERR_ARG;  // needs the U2_BAR/U3_BAR profiles
      z.r[z.n++] = BcRow{0, 0, 0, (f == 0) ? 0.0 : c1[EK_ZMIN]};
      z.r[z.n++] = BcRow{1, 0, 0, c1[EK_ZMIN]};
    } else if (zl == 1) z.r[z.n++] = BcRow{0, 0, 0, c1[EK_ZMIN]};
    else if (zl == 6) z.r[z.n++] = BcRow{0, 1, NZ, 0.0};
    else return EK_ERR_ARG;
    if (zr == 0) {
      z.r[z.n++] = BcRow{NZ + 1, 0, 0, (f == 3) ? c1[EK_ZMAX] : 0.0};
      z.r[z.n++] = BcRow{NZ, 0, 0, c1[EK_ZMAX]};
    } else if (zr == 1) {
      if (f == 1) z.r[z.n++] = BcRow{NZ + 1, 0, 0, 0.0};  // APPLY_BC_1_RIGHT ends with a Dirichlet 0 row
      else z.r[z.n++] = BcRow{NZ + 1, 0, 0, c1[EK_ZMAX]};
    } else if (zr == 6) z.r[z.n++] = BcRow{NZ + 1, 1, 1, 0.0};
    else return EK_ERR_ARG;
    // the boundary rows' matrix entries, for the solvers that build rows on the device
    for (int dir = 0; dir < 2; ++dir) {
      BcSet &bs = c.bc[f][dir];
      for (int t = 0; t < bs.n; ++t) bc_lhs(f, dir, p, d, bs.r[t].row, bs.r[t].l, bs.r[t].dg, bs.r[t].u);
    }
  }
  return EK_OK;
}

// Matrix rows (L, D, U) of the boundary rows above.
static void bc_lhs(int field, int dir, const ek_params &p, const Dims &d, int row, double &L, double &D, double &U) {
  const int *bc = (field == 0) ? p.th_bc : (field == 1) ? p.u_bc : (field == 2) ? p.v_bc : p.w_bc;
  L = 0.0; D = 1.0; U = 0.0;
  if (dir == 0) {
    const int lo = bc[EK_YMIN], hi = bc[EK_YMAX];
    if (row <= 1) {
      if (lo == 1 || (field == 0 && lo == 5)) { L = 0.0; D = -1.0; U = 1.0; }
    } else {
      if (hi == 1) { L = -1.0; D = 1.0; U = 0.0; }
    }
  } else {
    const int zl = bc[EK_ZMIN], zr = bc[EK_ZMAX];
    if (row <= 1) {
      if (zl == 1) { L = 0.0; D = -1.0; U = 1.0; }
    } else {
      if (zr == 1 && field != 1) { L = -1.0; D = 1.0; U = 0.0; }
    }
  }
  (void)d;
}

// Thomas factors (THOMAS_REAL, src/boundary.F90:53-84) of the lines of one
// field and direction for RK substep rk.  Line index: K for y lines, J for
// z lines; rows 0..N+1.  Interior rows follow duct.F90 (e.g. 1704-1716 for
// y, 1795-1805 for z); boundary rows come from bc_lhs; other rows stay at
// the initial (0, 1, 0).
void adi_factor_host(const Ctx &c, int field, int rk, int dir, const std::vector<double> &jac,
                     const std::vector<double> &g11, const std::vector<double> &g22, std::vector<double> &a,
                     std::vector<double> &ib, std::vector<double> &u) {
  const Dims &d = c.d;
  const ek_params &p = c.p;
  double coef = p.nu * c.H_BAR[rk] / 2.0;
  if (field == 0) coef = coef / p.pr;
  const int nline = (dir == 0) ? d.NZ2 : d.NY2;
  const int nrow = (dir == 0) ? d.NY2 : d.NZ2;
  const int js = (field == 0) ? d.JST : d.JS, je = (field == 0) ? d.JET : d.JE;
  const int zs = (field == 0) ? d.ZST : d.ZS, ze = (field == 0) ? d.ZET : d.ZE;
  a.assign((size_t)nline * nrow, 0.0);
  ib.assign((size_t)nline * nrow, 1.0);
  u.assign((size_t)nline * nrow, 0.0);
  std::vector<double> L(nrow), D(nrow), U(nrow);
  const BcSet &bs = c.bc[field][dir];
  for (int l = 0; l < nline; ++l) {
    const bool active = (dir == 0) ? (l >= zs && l <= ze) : (l >= js && l <= je);
    if (!active) continue;
    for (int r = 0; r < nrow; ++r) { L[r] = 0.0; D[r] = 1.0; U[r] = 0.0; }
    if (dir == 0) {
      const int k = l;
      for (int j = js; j <= je; ++j) {
        L[j] = -coef * g22[d.m3(k, j, 1)];
        D[j] = jac[d.m2(k, j)] + coef * (g22[d.m3(k, j + 1, 1)] + g22[d.m3(k, j, 1)]);
        U[j] = -coef * g22[d.m3(k, j + 1, 1)];
      }
    } else {
      const int j = l;
      for (int k = zs; k <= ze; ++k) {
        L[k] = -coef * g11[d.m3(k, j, 2)];
        D[k] = jac[d.m2(k, j)] + coef * (g11[d.m3(k + 1, j, 2)] + g11[d.m3(k, j, 2)]);
        U[k] = -coef * g11[d.m3(k + 1, j, 2)];
      }
    }
    for (int t = 0; t < bs.n; ++t) bc_lhs(field, dir, p, d, bs.r[t].row, L[bs.r[t].row], D[bs.r[t].row], U[bs.r[t].row]);
    // forward elimination on the matrix only
    double B = D[0];
    ib[(size_t)l * nrow + 0] = 1.0 / B;
    u[(size_t)l * nrow + 0] = U[0];
    for (int r = 0; r + 1 < nrow; ++r) {
      const double aa = -L[r + 1] / B;
      B = D[r + 1] + aa * U[r];
      a[(size_t)l * nrow + r + 1] = aa;
      ib[(size_t)l * nrow + r + 1] = 1.0 / B;
      u[(size_t)l * nrow + r + 1] = U[r + 1];
    }
  }
}

// n = p*2^(e-1)+1 with p >= 2; prefer the smallest p >= 3.
bool mg_pick_shape(int n, int &p, int &e) {
  const int m = n - 1;
  int bp = -1, be = -1;
  for (int ee = 1; ee < 31 && (1 << (ee - 1)) <= m; ++ee) {
    if (m % (1 << (ee - 1))) continue;
    const int pp = m >> (ee - 1);
    if (pp < 2) continue;
    if (pp >= 3 && (bp < 3 || pp < bp)) { bp = pp; be = ee; }
    if (bp < 0) { bp = pp; be = ee; }
  }
  if (bp < 0) return false;
  p = bp;
  e = be;
  return true;
}

// Sponge profiles (diablo.F90:1489-1556).  b, co_b and xx are REAL*8 there,
// but REAL(...) of a difference has the default kind (the Makefiles set no
// -r8), so the spans are rounded to REAL*4 before they divide.
int sponge_profiles_host(const ek_params *p, const double *xpoint, const double *ypoint, double *sig,
                         double *sig_out) {
  const int NY = p->ny, NZ = p->nz;
  auto X = [&](int k, int j) { return xpoint[(size_t)j * (NZ + 2) + k]; };
  auto Y = [&](int k, int j) { return ypoint[(size_t)j * (NZ + 2) + k]; };
  for (int k = 0; k <= NZ + 1; ++k) sig_out[k] = 0.0;
  const int R = p->nz_s_r, Lft = p->nz_s_l, T = p->ny_s_t;
  if (p->sponge_type == 1 && R < NZ + 1) {
    const double b = 1.0 / (double)(float)(X(NZ + 1, NY + 1) - X(R, NY + 1));
    for (int k = 0; k <= NZ + 1; ++k) {
      if (k >= R) {
        const double xx = (X(k, NY + 1) - X(R, NY + 1)) * b;
        sig_out[k] = xx * xx;
      } else if (k <= Lft) {
        const double xx = (X(Lft, NY + 1) - X(k, NY + 1)) * b;
        sig_out[k] = xx * xx;
      }
    }
  } else if (p->sponge_type == 2 && R < NZ + 1) {
    const double co_b = 25.0;
    const double b = std::log(co_b) / (double)(float)(NZ + 1 - R);
    for (int k = 0; k <= NZ + 1; ++k) {
      if (k >= R) sig_out[k] = (std::exp(b * std::abs(k - R)) - 1.0) / (co_b - 1.0);
      else if (k <= Lft) sig_out[k] = (std::exp(b * std::abs(Lft - k)) - 1.0) / (co_b - 1.0);
    }
  }
  for (int j = 0; j <= NY + 1; ++j) sig[j] = 0.0;
  if (p->sponge_type == 1) {
    if (T < 0 || T > NY + 1) return EK_ERR_ARG;
    const double b = 1.0 / (double)(float)(Y(NZ + 1, NY + 1) - Y(NZ + 1, T));
    for (int j = T; j <= NY + 1; ++j) {
      const double xx = (Y(NZ + 1, j) - Y(NZ + 1, T)) * b;
      sig[j] = xx * xx;
    }
  } else if (p->sponge_type == 2) {
    if (T < 0 || T > NY + 1) return EK_ERR_ARG;
    const double co_b = 30.0;
    const double b = std::log(co_b) / (double)(float)(NY + 1 - T);
    for (int j = T; j <= NY + 1; ++j) sig[j] = (std::exp(b * (j - T)) - 1.0) / (co_b - 1.0);
  }
  return EK_OK;
}

// Multigrid plan: level sizes (mud2cr.f:150-158), kx-independent
// coefficients of dismd2cr (mud2cr.f:544-998) for nxa=nxb=0, nyc=nyd=2 with
// bndcr's alfa=0, beta=1, gama=0, and cofcr (duct.F90:3900-3934).  Per
// point: c1..c8 after boundary folding, s4 = c1+c3+c5+c7 of the unfolded
// values, corr9 (corner correction added to c9) and J at the coefficient
// point, so that c9 = (-kx2*J - s4) + corr9 as in the Fortran.
void mg_build_plan_host(Ctx &c, const std::vector<double> &jac, const std::vector<double> &g11,
                        const std::vector<double> &g12, const std::vector<double> &g22) {
  MgPlan &P = c.mg;
  const Dims &d = c.d;
  P.ngrid = std::max(P.iex, P.jey);
  P.nfx = P.ixp * (1 << (P.iex - 1)) + 1;
  P.nfy = P.jyq * (1 << (P.jey - 1)) + 1;
  P.lv.assign(P.ngrid, MgLevel{});
  P.cof_host.assign(P.ngrid, {});
  const double xa = 0.0, xb = P.nfx - 1, yc = 0.0, yd = P.nfy - 1;
  auto G = [&](const std::vector<double> &a, int k, int j, int f) { return a[d.m3(k, j, f)]; };
  auto coef = [&](double x, double y, double &cxx, double &cxy, double &cyy, double &cx, double &cy, double &jc) {
    const int k = (int)x, j = (int)y;
    cxx = 0.25 * (G(g11, k, j, 2) + G(g11, k + 1, j, 2) + G(g11, k, j, 1) + G(g11, k, j + 1, 1));
    cxy = 0.5 * (G(g12, k, j, 2) + G(g12, k + 1, j, 2) + G(g12, k, j, 1) + G(g12, k, j + 1, 1));
    cyy = 0.25 * (G(g22, k, j, 2) + G(g22, k + 1, j, 2) + G(g22, k, j, 1) + G(g22, k, j + 1, 1));
    cx = G(g11, k + 1, j, 2) - G(g11, k, j, 2) + G(g12, k, j + 1, 1) - G(g12, k, j, 1);
    cy = G(g22, k, j + 1, 1) - G(g22, k, j, 1) + G(g12, k + 1, j, 2) - G(g12, k, j, 2);
    jc = jac[d.m2(k, j)];
  };
  bool orth = true;
  for (int lk = 1; lk <= P.ngrid; ++lk) {
    MgLevel &L = P.lv[lk - 1];
    L.nx = P.ixp * (1 << (std::max(lk + P.iex - P.ngrid, 1) - 1)) + 1;
    L.ny = P.jyq * (1 << (std::max(lk + P.jey - P.ngrid, 1) - 1)) + 1;
    const int nx = L.nx, ny = L.ny;
    std::vector<double> &cf = P.cof_host[lk - 1];
    cf.assign((size_t)11 * nx * ny, 0.0);
    auto C = [&](int i, int j, int l) -> double & { return cf[((size_t)(l - 1) * ny + (j - 1)) * nx + (i - 1)]; };
    const double dlx = (xb - xa) / (nx - 1), dlx2 = dlx + dlx, dlxx = dlx * dlx;
    const double dly = (yd - yc) / (ny - 1), dly2 = dly + dly, dlyy = dly * dly;
    const double dlxy = dlx * dly, dlxy2 = dlxy + dlxy, dlxy4 = dlxy2 + dlxy2;
    double cxx, cxy, cyy, cx, cy, jc;
    for (int j = 1; j <= ny; ++j) {
      const double y = yc + (j - 1) * dly;
      for (int i = 1; i <= nx; ++i) {
        const double x = xa + (i - 1) * dlx;
        coef(x, y, cxx, cxy, cyy, cx, cy, jc);
        cxx = std::max(cxx, std::fabs(cx) * dlx * 0.5);
        cyy = std::max(cyy, std::fabs(cy) * dly * 0.5);
        const double c1 = cxx / dlxx + cx / dlx2, c2 = cxy / dlxy4, c3 = cyy / dlyy + cy / dly2;
        const double c5 = cxx / dlxx - cx / dlx2, c7 = cyy / dlyy - cy / dly2;
        C(i, j, 1) = c1; C(i, j, 2) = c2; C(i, j, 3) = c3; C(i, j, 4) = -c2; C(i, j, 5) = c5;
        C(i, j, 6) = c2; C(i, j, 7) = c7; C(i, j, 8) = -c2;
        C(i, j, 9) = c1 + c3 + c5 + c7;  // s4
        C(i, j, 10) = 0.0;               // corr9
        C(i, j, 11) = jc;
      }
    }
    auto corner = [&](int i, int j, double x, double y, bool c4type) {
      coef(x, y, cxx, cxy, cyy, cx, cy, jc);
      if (c4type) {
        const double c4 = -cxy / dlxy2;
        C(i, j, 1) = C(i, j, 1) - c4; C(i, j, 2) = 0.0; C(i, j, 3) = C(i, j, 3) - c4; C(i, j, 4) = c4;
        C(i, j, 5) = C(i, j, 5) - c4; C(i, j, 6) = 0.0; C(i, j, 7) = C(i, j, 7) - c4; C(i, j, 8) = c4;
        C(i, j, 10) = 2.0 * c4;
      } else {
        const double c2 = cxy / dlxy2;
        C(i, j, 1) = C(i, j, 1) - c2; C(i, j, 2) = c2; C(i, j, 3) = C(i, j, 3) - c2; C(i, j, 4) = 0.0;
        C(i, j, 5) = C(i, j, 5) - c2; C(i, j, 6) = c2; C(i, j, 7) = C(i, j, 7) - c2; C(i, j, 8) = 0.0;
        C(i, j, 10) = 2.0 * c2;
      }
    };
    corner(1, 1, xa, yc, true);
    corner(nx, 1, xb, yc, false);
    corner(1, ny, xa, yd, false);
    corner(nx, ny, xb, yd, true);
    for (int i = 2; i <= nx - 1; ++i) {
      const double c6 = C(i, 1, 6), c7 = C(i, 1, 7), c8 = C(i, 1, 8);
      C(i, 1, 2) = C(i, 1, 2) + c8; C(i, 1, 3) = C(i, 1, 3) + c7; C(i, 1, 4) = C(i, 1, 4) + c6;
      C(i, 1, 6) = 0.0; C(i, 1, 7) = 0.0; C(i, 1, 8) = 0.0;
    }
    for (int i = 2; i <= nx - 1; ++i) {
      const double c2 = C(i, ny, 2), c3 = C(i, ny, 3), c4 = C(i, ny, 4);
      C(i, ny, 2) = 0.0; C(i, ny, 3) = 0.0; C(i, ny, 4) = 0.0;
      C(i, ny, 6) = C(i, ny, 6) + c4; C(i, ny, 7) = C(i, ny, 7) + c3; C(i, ny, 8) = C(i, ny, 8) + c2;
    }
    {
      const double c7 = C(1, 1, 7), c8 = C(1, 1, 8);
      C(1, 1, 2) = C(1, 1, 2) + c8; C(1, 1, 3) = C(1, 1, 3) + c7;
      C(1, 1, 6) = 0.0; C(1, 1, 7) = 0.0; C(1, 1, 8) = 0.0;
      const double d6 = C(nx, 1, 6), d7 = C(nx, 1, 7);
      C(nx, 1, 3) = C(nx, 1, 3) + d7; C(nx, 1, 4) = C(nx, 1, 4) + d6;
      C(nx, 1, 6) = 0.0; C(nx, 1, 7) = 0.0; C(nx, 1, 8) = 0.0;
    }
    {
      const double c2 = C(1, ny, 2), c3 = C(1, ny, 3);
      C(1, ny, 2) = 0.0; C(1, ny, 3) = 0.0; C(1, ny, 4) = 0.0;
      C(1, ny, 7) = C(1, ny, 7) + c3; C(1, ny, 8) = C(1, ny, 8) + c2;
      const double d3 = C(nx, ny, 3), d4 = C(nx, ny, 4);
      C(nx, ny, 2) = 0.0; C(nx, ny, 3) = 0.0; C(nx, ny, 4) = 0.0;
      C(nx, ny, 6) = C(nx, ny, 6) + d4; C(nx, ny, 7) = C(nx, ny, 7) + d3;
    }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        for (int l : {2, 4, 6, 8})
          if (C(i, j, l) != 0.0) orth = false;
  }
  P.orth = orth;
}

// The operation list of mud2cr1 with iguess = 0 (mud2cr.f:211-338): trsfc2
// down all levels, one FMG pass of kcymd2cr + prolon2, then maxcy k-cycles
// each followed by the convergence check.  kcymd2cr's level counters
// (mud2cr.f:340-499) are simulated exactly, so the relaxation counts per
// level match the Fortran control flow.
static void kcycle_ops(std::vector<MgOp> &ops, int kcur, int kcycle, int iprer, int ipost, int ngrid) {
  std::vector<int> kount(ngrid + 2, 0);
  int klevel = kcur;
  ops.push_back({OP_RELAX, klevel, iprer});
  if (kcur != 1) {
    ops.push_back({OP_RESTRICT, klevel, 0});
    for (int l = 1; l <= kcur; ++l) kount[l] = 0;
    klevel = kcur - 1;
    int nrel = iprer;
    while (klevel != kcur) {
      kount[klevel]++;
      ops.push_back({OP_RELAX, klevel, nrel});
      if (kount[klevel] == kcycle + 1) {
        ops.push_back({OP_COR2, klevel + 1, 0});
        kount[klevel] = 0;
        klevel++;
        nrel = ipost;
      } else if (klevel > 1) {
        ops.push_back({OP_RESTRICT, klevel, 0});
        klevel--;
        nrel = iprer;
      } else {
        ops.push_back({OP_RELAX, 1, ipost});
        ops.push_back({OP_COR2, 2, 0});
        nrel = ipost;
        klevel = 2;
      }
    }
  }
  ops.push_back({OP_RELAX, kcur, ipost});
}

void mg_build_schedule(MgPlan &plan, int kcycle, int iprer, int ipost, int maxcy) {
  std::vector<MgOp> &ops = plan.ops;
  ops.clear();
  ops.push_back({OP_TRSFC, plan.ngrid, 0});
  for (int k = 1; k <= plan.ngrid - 1; ++k) {
    kcycle_ops(ops, k, kcycle, iprer, ipost, plan.ngrid);
    ops.push_back({OP_PROLONG, k, 0});
  }
  for (int it = 1; it <= maxcy; ++it) {
    kcycle_ops(ops, plan.ngrid, kcycle, iprer, ipost, plan.ngrid);
    ops.push_back({OP_CHECK, plan.ngrid, it});
  }
  // merge consecutive relaxations of one level
  std::vector<MgOp> merged;
  for (const MgOp &o : ops) {
    if (!merged.empty() && o.kind == OP_RELAX && merged.back().kind == OP_RELAX && merged.back().level == o.level)
      merged.back().count += o.count;
    else
      merged.push_back(o);
  }
  ops.swap(merged);
}

// ---------------------------------------------------------------------------
// Left null vector of the finest kx = 0 operator.  With kx = 0 the problem is
// periodic in x and pure Neumann in y, so A 1 = 0 and A^T has a one-
// dimensional null space too.  The residual rule solves that mode as a well-
// posed problem: b' = b - (z.b) z with A^T z = 0, |z| = 1, and a zero-mean
// solution.  z is found once per metric set from A^T with the equation of
// the centre point replaced by z = 1 there, factored as a band.
namespace {

// A general band matrix with kl sub- and ku super-diagonals, stored by
// columns with room for the fill of row interchanges (LAPACK's band layout).
struct BandMatrix {
  long n;
  int kl, ku, ld;
  std::vector<double> a;
  std::vector<long> piv;
  BandMatrix(long n_, int kl_, int ku_) : n(n_), kl(kl_), ku(ku_), ld(2 * kl_ + ku_ + 1), a((size_t)ld * n_, 0.0) {}
  double &at(long i, long j) { return a[(size_t)j * ld + (size_t)(kl + ku + i - j)]; }
  // LU with partial pivoting, column by column; false on a zero pivot
  bool factor() {
    piv.assign(n, 0);
    long last = 0;  // last column touched by an interchange so far
    for (long j = 0; j < n; ++j) {
      const long m = std::min<long>(kl, n - 1 - j);
      long best = 0;
      for (long t = 1; t <= m; ++t)
        if (std::fabs(at(j + t, j)) > std::fabs(at(j + best, j))) best = t;
      piv[j] = j + best;
      last = std::max(last, std::min<long>(j + ku + best, n - 1));
      if (best)
        for (long c = j; c <= last; ++c) std::swap(at(j, c), at(j + best, c));
      const double d = at(j, j);
      if (d == 0.0) return false;
      const double rd = 1.0 / d;
      double *l = &at(j + 1, j);
      for (long t = 0; t < m; ++t) l[t] *= rd;
#pragma omp parallel for schedule(static) if (m * (last - j) > 32768)
      for (long c = j + 1; c <= last; ++c) {
        const double u = at(j, c);
        if (u != 0.0) {
          double *col = &at(j + 1, c);
          for (long t = 0; t < m; ++t) col[t] -= l[t] * u;
        }
      }
    }
    return true;
  }
  void solve(std::vector<double> &x) {
    for (long j = 0; j < n; ++j) {
      std::swap(x[j], x[piv[j]]);
      const long m = std::min<long>(kl, n - 1 - j);
      for (long t = 1; t <= m; ++t) x[j + t] -= at(j + t, j) * x[j];
    }
    for (long j = n - 1; j >= 0; --j) {
      x[j] /= at(j, j);
      for (long i = std::max<long>(0, j - kl - ku); i < j; ++i) x[i] -= at(i, j) * x[j];
    }
  }
};

}  // namespace

bool mg_left_null_host(const MgPlan &P, std::vector<double> &z) {
  const int nx = P.nfx, ny = P.nfy;
  const long n = (long)nx * ny;
  const std::vector<double> &cf = P.cof_host[P.ngrid - 1];
  auto C = [&](int i, int j, int l) { return cf[((size_t)(l - 1) * ny + (j - 1)) * nx + (i - 1)]; };
  // place of unknown (i, j): rows j one after another; inside a row the
  // periodic x ring is visited 1, nx, 2, nx-1, 3, ... so that the couplings
  // through the ghost columns stay within three places of the diagonal
  std::vector<long> place(nx + 2);
  {
    long k = 0;
    place[1] = k++;
    place[nx] = k++;
    for (int lo = 2, hi = nx - 1; lo <= hi; ++lo, --hi) {
      place[lo] = k++;
      if (hi != lo) place[hi] = k++;
    }
  }
  place[0] = place[nx - 1];  // ghost columns: e(0) = e(nx-1), e(nx+1) = e(2)
  place[nx + 1] = place[2];
  auto idx = [&](int i, int j) { return (long)(j - 1) * nx + place[i]; };
  static const int di[8] = {1, 1, 0, -1, -1, -1, 0, 1}, dj[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  const long pin = idx((nx + 1) / 2, (ny + 1) / 2);
  struct Entry { long r, c; double v; };
  std::vector<Entry> ent;
  ent.reserve((size_t)n * 9);
  int kl = 0, ku = 0;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long row_of_a = idx(i, j);
      // A^T: A's coupling of (i, j) to its neighbour q lands in row q, column (i, j)
      const double c9 = -C(i, j, 9) + C(i, j, 10);
      if (row_of_a != pin) ent.push_back({row_of_a, row_of_a, c9});
      for (int l = 0; l < 8; ++l) {
        const int jj = j + dj[l];
        const double v = C(i, j, l + 1);
        if (jj < 1 || jj > ny || v == 0.0) continue;  // the y ghosts carry no coupling after the folding
        const long q = idx(i + di[l], jj);
        if (q == pin) continue;
        ent.push_back({q, row_of_a, v});
        kl = std::max<int>(kl, (int)(q - row_of_a));
        ku = std::max<int>(ku, (int)(row_of_a - q));
      }
    }
  BandMatrix M(n, kl, ku);
  for (const Entry &e : ent) M.at(e.r, e.c) += e.v;
  M.at(pin, pin) = 1.0;
  if (!M.factor()) return false;
  std::vector<double> x(n, 0.0);
  x[pin] = 1.0;
  M.solve(x);
  z.assign(n, 0.0);
  double ss = 0.0;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const double v = x[idx(i, j)];
      z[(size_t)(j - 1) * nx + (i - 1)] = v;
      ss += v * v;
    }
  const double inv = 1.0 / std::sqrt(ss);
  for (double &v : z) v *= inv;
  return true;
}

}  // namespace ek
