// Oracle (test infrastructure): MUDPACK subset restated.  Each routine cites
// the reference routine it follows; Fortran expression order is kept.
#include "ekref_mud.h"

#include <algorithm>
#include <cmath>

namespace ekref {

Mud2cr::Mud2cr(const MudOpts &o) : o_(o) {
  // mud2cr.f:118-160: sizes of the grid levels (nxk, nyk)
  ngrid_ = std::max(o.iex, o.jey);
  nfx_ = o.ixp * (1 << (o.iex - 1)) + 1;
  nfy_ = o.jyq * (1 << (o.jey - 1)) + 1;
  lv_.resize(ngrid_);
  for (int k = 1; k <= ngrid_; ++k) {
    Level &L = lv_[k - 1];
    L.nx = o.ixp * (1 << (std::max(k + o.iex - ngrid_, 1) - 1)) + 1;
    L.ny = o.jyq * (1 << (std::max(k + o.jey - ngrid_, 1) - 1)) + 1;
    L.phi.assign((size_t)(L.nx + 2) * (L.ny + 2), 0.0);
    L.cof.assign((size_t)10 * L.nx * L.ny, 0.0);
  }
  work_.assign((size_t)(nfx_ + 2) * (nfy_ + 2), 0.0);
  // MULTIGRID_MUDPACK (mg_solver2d.F90:162-170): xa=0, xb=nnx-1, yc=0, yd=nny-1
  xa_ = 0.0;
  xb_ = nfx_ - 1;
  yc_ = 0.0;
  yd_ = nfy_ - 1;
}

// dismd2cr (mud2cr.f:501-1270) for nxa=nxb=0, nyc=nyd=2 with bndcr's
// alfa=0, beta=1, gama=0.  The mixed-condition folding terms that carry
// alfa or gama are zero products added to the coefficient, so only the
// reflection moves (c6->c4, c7->c3, c8->c2 at j=1 and the mirror at j=ny)
// change values; they are kept, the zero additions are omitted.
void Mud2cr::dismd2cr(Level &L, const CoefFn &coef) {
  const int nx = L.nx, ny = L.ny;
  const double dlx = (xb_ - xa_) / (nx - 1), dlx2 = dlx + dlx, dlxx = dlx * dlx;
  const double dly = (yd_ - yc_) / (ny - 1), dly2 = dly + dly, dlyy = dly * dly;
  const double dlxy = dlx * dly, dlxy2 = dlxy + dlxy, dlxy4 = dlxy2 + dlxy2;
  double cxx, cxy, cyy, cx, cy, ce;
  for (int j = 1; j <= ny; ++j) {
    const double y = yc_ + (j - 1) * dly;
    for (int i = 1; i <= nx; ++i) {
      const double x = xa_ + (i - 1) * dlx;
      coef(x, y, cxx, cxy, cyy, cx, cy, ce);
      cxx = std::max(cxx, std::fabs(cx) * dlx * 0.5);
      cyy = std::max(cyy, std::fabs(cy) * dly * 0.5);
      const double c1 = cxx / dlxx + cx / dlx2;
      const double c2 = cxy / dlxy4;
      const double c3 = cyy / dlyy + cy / dly2;
      const double c4 = -c2;
      const double c5 = cxx / dlxx - cx / dlx2;
      const double c6 = c2;
      const double c7 = cyy / dlyy - cy / dly2;
      const double c8 = -c2;
      const double c9 = ce - (c1 + c3 + c5 + c7);
      L.C(i, j, 1) = c1; L.C(i, j, 2) = c2; L.C(i, j, 3) = c3; L.C(i, j, 4) = c4; L.C(i, j, 5) = c5;
      L.C(i, j, 6) = c6; L.C(i, j, 7) = c7; L.C(i, j, 8) = c8; L.C(i, j, 9) = c9;
    }
  }
  // corners: virtual-virtual points not used (mud2cr.f:583-629)
  {
    coef(xa_, yc_, cxx, cxy, cyy, cx, cy, ce);
    const double c4 = -cxy / dlxy2;
    L.C(1, 1, 1) = L.C(1, 1, 1) - c4; L.C(1, 1, 2) = 0.0; L.C(1, 1, 3) = L.C(1, 1, 3) - c4;
    L.C(1, 1, 4) = c4; L.C(1, 1, 5) = L.C(1, 1, 5) - c4; L.C(1, 1, 6) = 0.0;
    L.C(1, 1, 7) = L.C(1, 1, 7) - c4; L.C(1, 1, 8) = c4; L.C(1, 1, 9) = L.C(1, 1, 9) + 2.0 * c4;
  }
  {
    coef(xb_, yc_, cxx, cxy, cyy, cx, cy, ce);
    const double c2 = cxy / dlxy2;
    L.C(nx, 1, 1) = L.C(nx, 1, 1) - c2; L.C(nx, 1, 2) = c2; L.C(nx, 1, 3) = L.C(nx, 1, 3) - c2;
    L.C(nx, 1, 4) = 0.0; L.C(nx, 1, 5) = L.C(nx, 1, 5) - c2; L.C(nx, 1, 6) = c2;
    L.C(nx, 1, 7) = L.C(nx, 1, 7) - c2; L.C(nx, 1, 8) = 0.0; L.C(nx, 1, 9) = L.C(nx, 1, 9) + 2.0 * c2;
  }
  {
    coef(xa_, yd_, cxx, cxy, cyy, cx, cy, ce);
    const double c2 = cxy / dlxy2;
    L.C(1, ny, 1) = L.C(1, ny, 1) - c2; L.C(1, ny, 2) = c2; L.C(1, ny, 3) = L.C(1, ny, 3) - c2;
    L.C(1, ny, 4) = 0.0; L.C(1, ny, 5) = L.C(1, ny, 5) - c2; L.C(1, ny, 6) = c2;
    L.C(1, ny, 7) = L.C(1, ny, 7) - c2; L.C(1, ny, 8) = 0.0; L.C(1, ny, 9) = L.C(1, ny, 9) + 2.0 * c2;
  }
  {
    coef(xb_, yd_, cxx, cxy, cyy, cx, cy, ce);
    const double c4 = -cxy / dlxy2;
    L.C(nx, ny, 1) = L.C(nx, ny, 1) - c4; L.C(nx, ny, 2) = 0.0; L.C(nx, ny, 3) = L.C(nx, ny, 3) - c4;
    L.C(nx, ny, 4) = c4; L.C(nx, ny, 5) = L.C(nx, ny, 5) - c4; L.C(nx, ny, 6) = 0.0;
    L.C(nx, ny, 7) = L.C(nx, ny, 7) - c4; L.C(nx, ny, 8) = c4; L.C(nx, ny, 9) = L.C(nx, ny, 9) + 2.0 * c4;
  }
  // nyc=2 edge j=1 (mud2cr.f:719-760)
  for (int i = 2; i <= nx - 1; ++i) {
    const double c6 = L.C(i, 1, 6), c7 = L.C(i, 1, 7), c8 = L.C(i, 1, 8);
    L.C(i, 1, 2) = L.C(i, 1, 2) + c8;
    L.C(i, 1, 3) = L.C(i, 1, 3) + c7;
    L.C(i, 1, 4) = L.C(i, 1, 4) + c6;
    L.C(i, 1, 6) = 0.0; L.C(i, 1, 7) = 0.0; L.C(i, 1, 8) = 0.0;
  }
  // nyd=2 edge j=ny (mud2cr.f:762-803)
  for (int i = 2; i <= nx - 1; ++i) {
    const double c2 = L.C(i, ny, 2), c3 = L.C(i, ny, 3), c4 = L.C(i, ny, 4);
    L.C(i, ny, 2) = 0.0; L.C(i, ny, 3) = 0.0; L.C(i, ny, 4) = 0.0;
    L.C(i, ny, 6) = L.C(i, ny, 6) + c4;
    L.C(i, ny, 7) = L.C(i, ny, 7) + c3;
    L.C(i, ny, 8) = L.C(i, ny, 8) + c2;
  }
  // periodic-mixed corners at yc (mud2cr.f:818-854)
  {
    const double c7 = L.C(1, 1, 7), c8 = L.C(1, 1, 8);
    L.C(1, 1, 2) = L.C(1, 1, 2) + c8;
    L.C(1, 1, 3) = L.C(1, 1, 3) + c7;
    L.C(1, 1, 6) = 0.0; L.C(1, 1, 7) = 0.0; L.C(1, 1, 8) = 0.0;
    const double d6 = L.C(nx, 1, 6), d7 = L.C(nx, 1, 7);
    L.C(nx, 1, 3) = L.C(nx, 1, 3) + d7;
    L.C(nx, 1, 4) = L.C(nx, 1, 4) + d6;
    L.C(nx, 1, 6) = 0.0; L.C(nx, 1, 7) = 0.0; L.C(nx, 1, 8) = 0.0;
  }
  // periodic-mixed corners at yd (mud2cr.f:956-998)
  {
    const double c2 = L.C(1, ny, 2), c3 = L.C(1, ny, 3);
    L.C(1, ny, 2) = 0.0; L.C(1, ny, 3) = 0.0; L.C(1, ny, 4) = 0.0;
    L.C(1, ny, 7) = L.C(1, ny, 7) + c3;
    L.C(1, ny, 8) = L.C(1, ny, 8) + c2;
    const double d3 = L.C(nx, ny, 3), d4 = L.C(nx, ny, 4);
    L.C(nx, ny, 2) = 0.0; L.C(nx, ny, 3) = 0.0; L.C(nx, ny, 4) = 0.0;
    L.C(nx, ny, 6) = L.C(nx, ny, 6) + d4;
    L.C(nx, ny, 7) = L.C(nx, ny, 7) + d3;
  }
}

void Mud2cr::discretize(const CoefFn &coef) {
  for (int kb = 1; kb <= ngrid_; ++kb) dismd2cr(lv_[ngrid_ - kb], coef);
}

// relmd2crp (mud2cr.f:1693-1795): four-colour point Gauss-Seidel.
void Mud2cr::relmd2crp(Level &L) {
  const int nx = L.nx, ny = L.ny;
  int i1 = 1, i2 = 4, i3 = 3, i4 = 2;
  auto upd = [&](int i, int j) {
    L.P(i, j) = (L.C(i, j, 10) - (L.C(i, j, 1) * L.P(i + 1, j) + L.C(i, j, 2) * L.P(i + 1, j + 1) +
                                  L.C(i, j, 3) * L.P(i, j + 1) + L.C(i, j, 4) * L.P(i - 1, j + 1) +
                                  L.C(i, j, 5) * L.P(i - 1, j) + L.C(i, j, 6) * L.P(i - 1, j - 1) +
                                  L.C(i, j, 7) * L.P(i, j - 1) + L.C(i, j, 8) * L.P(i + 1, j - 1))) /
                L.C(i, j, 9);
  };
  for (int lcolor = 1; lcolor <= 4; ++lcolor) {
    for (int j = 1; j <= ny; j += 4)
      for (int i = i1; i <= nx; i += 4) upd(i, j);
    for (int j = 2; j <= ny; j += 4)
      for (int i = i2; i <= nx; i += 4) upd(i, j);
    for (int j = 3; j <= ny; j += 4)
      for (int i = i3; i <= nx; i += 4) upd(i, j);
    for (int j = 4; j <= ny; j += 4)
      for (int i = i4; i <= nx; i += 4) upd(i, j);
    for (int j = 1; j <= ny; ++j) {  // nxa == 0: periodic virtual boundaries
      L.P(0, j) = L.P(nx - 1, j);
      L.P(nx + 1, j) = L.P(2, j);
    }
    const int it = i4;
    i4 = i3; i3 = i2; i2 = i1; i1 = it;
  }
}

// res2 (mudcom.f:120-257): full-weighting restriction of resf to C.rhs.
void Mud2cr::res2(int nx, int ny, const double *resf, Level &Cl) {
  const int ncx = Cl.nx, ncy = Cl.ny;
  auto R = [&](int i, int j) { return resf[(size_t)j * (nx + 2) + i]; };
  auto fw = [&](int im1, int ip1, int jm1, int jp1, int i, int j) {
    return (R(im1, jm1) + R(ip1, jm1) + R(im1, jp1) + R(ip1, jp1) +
            2. * (R(im1, j) + R(ip1, j) + R(i, jm1) + R(i, jp1)) + 4. * R(i, j)) * .0625;
  };
  const int ix = (ncx == nx) ? 0 : 1;
  const int jy = (ncy == ny) ? 0 : 1;
  if (ncy < ny && ncx < nx) {
    for (int jc = 2; jc <= ncy - 1; ++jc) {
      const int j = jc + jc - 1;
      for (int ic = 2; ic <= ncx - 1; ++ic) {
        const int i = ic + ic - 1;
        Cl.C(ic, jc, 10) = fw(i - 1, i + 1, j - 1, j + 1, i, j);
      }
    }
  } else if (ncy == ny) {
    for (int jc = 2; jc <= ncy - 1; ++jc) {
      const int j = jc;
      for (int ic = 2; ic <= ncx - 1; ++ic) {
        const int i = ic + ic - 1;
        Cl.C(ic, jc, 10) = fw(i - 1, i + 1, j - 1, j + 1, i, j);
      }
    }
  } else {
    for (int jc = 2; jc <= ncy - 1; ++jc) {
      const int j = jc + jc - 1;
      for (int ic = 2; ic <= ncx - 1; ++ic) {
        const int i = ic;
        Cl.C(ic, jc, 10) = fw(i - 1, i + 1, j - 1, j + 1, i, j);
      }
    }
  }
  for (int jc = 1; jc <= ncy; jc += ncy - 1) {
    const int j = jc + jy * (jc - 1);
    const int jm1 = std::max(j - 1, 2);
    const int jp1 = std::min(j + 1, ny - 1);
    for (int ic = 1; ic <= ncx; ic += ncx - 1) {
      const int i = ic + ix * (ic - 1);
      int im1 = std::max(i - 1, 2);
      int ip1 = std::min(i + 1, nx - 1);
      if (i == 1) im1 = nx - 1;   // nxa == 0
      if (i == nx) ip1 = 2;
      Cl.C(ic, jc, 10) = fw(im1, ip1, jm1, jp1, i, j);
    }
    for (int ic = 2; ic <= ncx - 1; ++ic) {
      const int i = ic + ix * (ic - 1);
      Cl.C(ic, jc, 10) = fw(i - 1, i + 1, jm1, jp1, i, j);
    }
  }
  for (int ic = 1; ic <= ncx; ic += ncx - 1) {
    const int i = ic + ix * (ic - 1);
    int im1 = std::max(i - 1, 2);
    int ip1 = std::min(i + 1, nx - 1);
    if (i == 1) im1 = nx - 1;
    if (i == nx) ip1 = 2;
    for (int jc = 2; jc <= ncy - 1; ++jc) {
      const int j = jc + jy * (jc - 1);
      Cl.C(ic, jc, 10) = fw(im1, ip1, j - 1, j + 1, i, j);
    }
  }
}

// resmd2cr (mud2cr.f:1618-1665)
void Mud2cr::resmd2cr(Level &F, Level &Cl) {
  std::fill(Cl.phi.begin(), Cl.phi.end(), 0.0);
  const int nx = F.nx, ny = F.ny;
  double *resf = work_.data();
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i)
      resf[(size_t)j * (nx + 2) + i] =
          F.C(i, j, 10) - (F.C(i, j, 1) * F.P(i + 1, j) + F.C(i, j, 2) * F.P(i + 1, j + 1) +
                           F.C(i, j, 3) * F.P(i, j + 1) + F.C(i, j, 4) * F.P(i - 1, j + 1) +
                           F.C(i, j, 5) * F.P(i - 1, j) + F.C(i, j, 6) * F.P(i - 1, j - 1) +
                           F.C(i, j, 7) * F.P(i, j - 1) + F.C(i, j, 8) * F.P(i + 1, j - 1) +
                           F.C(i, j, 9) * F.P(i, j));
  res2(nx, ny, resf, Cl);
}

// trsfc2 (mudcom.f:61-118): injection of phi and rhs to the coarser level.
void Mud2cr::trsfc2(Level &F, Level &Cl) {
  const int nx = F.nx, ny = F.ny, ncx = Cl.nx, ncy = Cl.ny;
  for (int jc = 0; jc <= ncy + 1; ++jc) { Cl.P(0, jc) = 0.0; Cl.P(ncx + 1, jc) = 0.0; }
  for (int ic = 0; ic <= ncx + 1; ++ic) { Cl.P(ic, 0) = 0.0; Cl.P(ic, ncy + 1) = 0.0; }
  for (int jc = 1; jc <= ncy; ++jc) {
    const int j = (ncy < ny) ? jc + jc - 1 : jc;
    for (int ic = 1; ic <= ncx; ++ic) {
      const int i = (ncx < nx) ? ic + ic - 1 : ic;
      Cl.P(ic, jc) = F.P(i, j);
      Cl.C(ic, jc, 10) = F.C(i, j, 10);
    }
  }
}

// prolon1 (mudcom.f:404-499), nxa = nxb = 0.  p, q point at index 0.
void Mud2cr::prolon1(int ncx, const double *p, int nx, double *q) {
  if (o_.intpol == 1 || ncx < 4) {
    if (ncx < nx) {
      for (int i = 1; i <= nx; i += 2) q[i] = p[(i + 1) / 2];
      for (int i = 2; i <= nx; i += 2) q[i] = 0.5 * (q[i - 1] + q[i + 1]);
    } else {
      for (int i = 1; i <= nx; ++i) q[i] = p[i];
    }
    q[0] = q[nx - 1];
    q[nx + 1] = q[2];
  } else {
    if (ncx < nx) {
      for (int i = 1; i <= nx; i += 2) q[i] = p[(i + 1) / 2];
      for (int i = 4; i <= nx - 3; i += 2) q[i] = (-q[i - 3] + 9. * (q[i - 1] + q[i + 1]) - q[i + 3]) * .0625;
      q[2] = (-q[nx - 2] + 9. * (q[1] + q[3]) - q[5]) * .0625;
      q[nx - 1] = (-q[nx - 4] + 9. * (q[nx - 2] + q[nx]) - q[3]) * .0625;
      q[nx + 1] = q[2];
      q[0] = q[nx - 1];
    } else {
      for (int i = 1; i <= nx; ++i) q[i] = p[i];
      q[0] = q[nx - 1];
      q[nx + 1] = q[2];
    }
  }
}

// prolon2 (mudcom.f:261-399), nyc = nyd = 2.  q is (0:nx+1, 0:ny+1).
void Mud2cr::prolon2(int ncx, int ncy, Level &Pc, int nx, int ny, double *q) {
  auto Q = [&](int i, int j) -> double & { return q[(size_t)j * (nx + 2) + i]; };
  auto prow = [&](int jc) { return &Pc.phi[(size_t)jc * (ncx + 2)]; };
  if (o_.intpol == 1 || ncy < 4) {
    if (ncy < ny) {
      for (int j = 1; j <= ny; j += 2) prolon1(ncx, prow(j / 2 + 1), nx, &Q(0, j));
      for (int j = 2; j <= ny; j += 2)
        for (int i = 1; i <= nx; ++i) Q(i, j) = 0.5 * (Q(i, j - 1) + Q(i, j + 1));
    } else {
      for (int j = 1; j <= ny; ++j) prolon1(ncx, prow(j), nx, &Q(0, j));
    }
  } else {
    if (ncy < ny) {
      for (int j = 1; j <= ny; j += 2) prolon1(ncx, prow(j / 2 + 1), nx, &Q(0, j));
      for (int j = 4; j <= ny - 3; j += 2)
        for (int i = 1; i <= nx; ++i)
          Q(i, j) = (-Q(i, j - 3) + 9. * (Q(i, j - 1) + Q(i, j + 1)) - Q(i, j + 3)) * .0625;
      for (int i = 1; i <= nx; ++i) {
        Q(i, 2) = (5. * Q(i, 1) + 15. * Q(i, 3) - 5. * Q(i, 5) + Q(i, 7)) * .0625;
        Q(i, ny - 1) = (5. * Q(i, ny) + 15. * Q(i, ny - 2) - 5. * Q(i, ny - 4) + Q(i, ny - 6)) * .0625;
      }
    } else {
      for (int j = 1; j <= ny; ++j) prolon1(ncx, prow(j), nx, &Q(0, j));
    }
  }
}

// cor2 (mudcom.f:502-552)
void Mud2cr::cor2(Level &F, Level &Cl) {
  const int nx = F.nx, ny = F.ny;
  double *phcor = work_.data();
  std::fill(phcor, phcor + (size_t)(nx + 2) * (ny + 2), 0.0);
  prolon2(Cl.nx, Cl.ny, Cl, nx, ny, phcor);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) F.P(i, j) = F.P(i, j) + phcor[(size_t)j * (nx + 2) + i];
  for (int j = 1; j <= ny; ++j) {
    F.P(0, j) = F.P(nx - 1, j);
    F.P(nx + 1, j) = F.P(2, j);
  }
}

// kcymd2cr (mud2cr.f:340-499): one k-cycle from level kcur.
void Mud2cr::kcymd2cr(int kcur) {
  const int kcycle = o_.kcycle, iprer = o_.iprer, ipost = o_.ipost;
  std::vector<int> kount(ngrid_ + 1, 0);
  int klevel = kcur;
  for (int l = 1; l <= iprer; ++l) relmd2crp(lv_[klevel - 1]);
  if (kcur != 1) {
    resmd2cr(lv_[klevel - 1], lv_[klevel - 2]);
    for (int l = 1; l <= kcur; ++l) kount[l] = 0;
    klevel = kcur - 1;
    int nrel = iprer;
    while (klevel != kcur) {
      kount[klevel] = kount[klevel] + 1;
      for (int l = 1; l <= nrel; ++l) relmd2crp(lv_[klevel - 1]);
      if (kount[klevel] == kcycle + 1) {
        cor2(lv_[klevel], lv_[klevel - 1]);
        kount[klevel] = 0;
        klevel = klevel + 1;
        nrel = ipost;
      } else if (klevel > 1) {
        resmd2cr(lv_[klevel - 1], lv_[klevel - 2]);
        klevel = klevel - 1;
        nrel = iprer;
      } else {
        for (int l = 1; l <= ipost; ++l) relmd2crp(lv_[0]);
        cor2(lv_[1], lv_[0]);
        nrel = ipost;
        klevel = 2;
      }
    }
  }
  for (int l = 1; l <= ipost; ++l) relmd2crp(lv_[kcur - 1]);
}

// mud2cr1 (mud2cr.f:211-338) with swk2 (mudcom.f:32-59).
MudResult Mud2cr::solve(const double *rhsf, double *phif, bool singular, const double *z) {
  MudResult r;
  const int nfx = nfx_, nfy = nfy_;
  const size_t nf = (size_t)nfx * nfy;
  auto PF = [&](int i, int j) -> double & { return phif[(size_t)(j - 1) * nfx + (i - 1)]; };
  Level &F = lv_[ngrid_ - 1];
  // the residual rule's well-posed kx = 0 problem: b' = b - (z.b / z.z) z
  const bool wellposed = singular && o_.stop_rule == 1;
  std::vector<double> bproj;
  if (wellposed) {
    double zb = 0.0, zz = 0.0;
    for (size_t t = 0; t < nf; ++t) {
      zb += z[t] * rhsf[t];
      zz += z[t] * z[t];
    }
    const double a = (zz > 0.0) ? zb / zz : 0.0;
    bproj.resize(nf);
    for (size_t t = 0; t < nf; ++t) bproj[t] = rhsf[t] - a * z[t];
    rhsf = bproj.data();
  }
  for (int j = 1; j <= nfy; ++j)
    for (int i = 1; i <= nfx; ++i) {
      F.P(i, j) = PF(i, j);
      F.C(i, j, 10) = rhsf[(size_t)(j - 1) * nfx + (i - 1)];
    }
  for (int j = 0; j <= nfy + 1; ++j) { F.P(0, j) = 0.0; F.P(nfx + 1, j) = 0.0; }
  for (int i = 0; i <= nfx + 1; ++i) { F.P(i, 0) = 0.0; F.P(i, nfy + 1) = 0.0; }
  // iguess = 0: transfer down, adjust rhs (adjmd2cr adds only zero terms for
  // gbdy = 0 and does nothing else for these boundary types), then one FMG
  // sweep up the levels.
  for (int kb = 2; kb <= ngrid_; ++kb) {
    const int k = ngrid_ - kb + 1;
    trsfc2(lv_[k], lv_[k - 1]);
  }
  for (int k = 1; k <= ngrid_ - 1; ++k) {
    kcymd2cr(k);
    Level &Fk = lv_[k];
    prolon2(lv_[k - 1].nx, lv_[k - 1].ny, lv_[k - 1], Fk.nx, Fk.ny, Fk.phi.data());
  }
  const int kcur = ngrid_;
  double bnorm = 0.0;
  if (o_.stop_rule == 1) {
    for (int j = 1; j <= nfy; ++j)
      for (int i = 1; i <= nfx; ++i) bnorm += F.C(i, j, 10) * F.C(i, j, 10);
    bnorm = std::sqrt(bnorm);
  }
  const bool rel = (o_.stop_rule == 0);
  const double tol = o_.tol;
  const int maxcy = o_.maxcy;
  for (int iter = 1; iter <= maxcy; ++iter) {
    r.cycles = iter;
    kcymd2cr(kcur);
    if (rel) {
      if (tol > 0.0) {
        double relmax = 0.0, phmax = 0.0;
        for (int j = 1; j <= nfy; ++j)
          for (int i = 1; i <= nfx; ++i) {
            phmax = std::max(phmax, std::fabs(F.P(i, j)));
            relmax = std::max(relmax, std::fabs(F.P(i, j) - PF(i, j)));
            PF(i, j) = F.P(i, j);
          }
        if (phmax > 0.0) relmax = relmax / phmax;
        r.relmax = relmax;
        if (relmax <= tol) { r.converged = true; return r; }
      }
    } else {
      double rn = 0.0;
      for (int j = 1; j <= nfy; ++j)
        for (int i = 1; i <= nfx; ++i) {
          const double res =
              F.C(i, j, 10) - (F.C(i, j, 1) * F.P(i + 1, j) + F.C(i, j, 2) * F.P(i + 1, j + 1) +
                               F.C(i, j, 3) * F.P(i, j + 1) + F.C(i, j, 4) * F.P(i - 1, j + 1) +
                               F.C(i, j, 5) * F.P(i - 1, j) + F.C(i, j, 6) * F.P(i - 1, j - 1) +
                               F.C(i, j, 7) * F.P(i, j - 1) + F.C(i, j, 8) * F.P(i + 1, j - 1) +
                               F.C(i, j, 9) * F.P(i, j));
          rn += res * res;
        }
      rn = std::sqrt(rn);
      r.resid = (bnorm > 0.0) ? rn / bnorm : 0.0;
      if (r.resid <= o_.tol) {
        r.converged = true;
        break;
      }
    }
  }
  for (int j = 1; j <= nfy; ++j)
    for (int i = 1; i <= nfx; ++i) PF(i, j) = F.P(i, j);
  if (wellposed) {
    // the solution is defined up to a constant: zero mean
    double m = 0.0;
    for (size_t t = 0; t < nf; ++t) m += phif[t];
    m = m / (double)nf;
    for (size_t t = 0; t < nf; ++t) phif[t] = phif[t] - m;
  }
  return r;
}

void Mud2cr::finest_coo(std::vector<int> &row, std::vector<int> &col, std::vector<double> &val) const {
  const Level &F = lv_[ngrid_ - 1];
  const int nx = nfx_, ny = nfy_;
  static const int di[9] = {1, 1, 0, -1, -1, -1, 0, 1, 0}, dj[9] = {0, 1, 1, 1, 0, -1, -1, -1, 0};
  row.clear();
  col.clear();
  val.clear();
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i)
      for (int l = 0; l < 9; ++l) {
        const double v = F.cof[((size_t)l * ny + (j - 1)) * nx + (i - 1)];
        int ii = i + di[l];
        const int jj = j + dj[l];
        if (jj < 1 || jj > ny) continue;  // zero after the Neumann folding
        if (v == 0.0) continue;
        if (ii == 0) ii = nx - 1;
        if (ii == nx + 1) ii = 2;
        row.push_back((j - 1) * nx + (i - 1));
        col.push_back((jj - 1) * nx + (ii - 1));
        val.push_back(v);
      }
}

std::vector<double> Mud2cr::left_null() const {
  const int nx = nfx_, ny = nfy_;
  const long n = (long)nx * ny;
  // unknowns ordered row by row (j outer); inside a row the periodic ring
  // 1, nx, 2, nx-1, 3, ... so that every x-coupling (the wrap included)
  // spans at most 3 places and the band is nx + 3 wide
  std::vector<int> pos(nx + 1);
  const int L = nx - 2, left = (L + 1) / 2;
  pos[1] = 0;
  pos[nx] = 1;
  for (int i = 2; i <= nx - 1; ++i) pos[i] = (i - 2 < left) ? 2 + 2 * (i - 2) : 3 + 2 * ((nx - 1) - i);
  auto q = [&](int u) { return (long)(u / nx) * nx + pos[u % nx + 1]; };
  std::vector<int> r, c;
  std::vector<double> v;
  finest_coo(r, c, v);
  const long pin = q(((ny + 1) / 2 - 1) * nx + (nx + 1) / 2 - 1);
  // M = A^T: entry (q(col), q(row)); the pinned equation becomes z = 1
  int kl = 0, ku = 0;
  for (size_t t = 0; t < v.size(); ++t) {
    const long a = q(c[t]), b = q(r[t]);
    if (a == pin) continue;
    kl = std::max<int>(kl, (int)(a - b));
    ku = std::max<int>(ku, (int)(b - a));
  }
  const int kv = kl + ku, ldab = 2 * kl + ku + 1;
  std::vector<double> ab((size_t)ldab * n, 0.0);
  auto AB = [&](long i, long j) -> double & { return ab[(size_t)j * ldab + (size_t)(kv + i - j)]; };
  for (size_t t = 0; t < v.size(); ++t) {
    const long a = q(c[t]), b = q(r[t]);
    if (a == pin) continue;
    AB(a, b) += v[t];
  }
  AB(pin, pin) = 1.0;
  // LU with partial pivoting of the band (the unblocked LAPACK gbtf2 scheme)
  std::vector<long> ipiv(n);
  long ju = 0;
  for (long j = 0; j < n; ++j) {
    const long km = std::min<long>(kl, n - 1 - j);
    long jp = 0;
    double best = std::fabs(AB(j, j));
    for (long t = 1; t <= km; ++t)
      if (std::fabs(AB(j + t, j)) > best) {
        best = std::fabs(AB(j + t, j));
        jp = t;
      }
    ipiv[j] = j + jp;
    ju = std::max(ju, std::min<long>(j + ku + jp, n - 1));
    if (jp != 0)
      for (long cc = j; cc <= ju; ++cc) std::swap(AB(j, cc), AB(j + jp, cc));
    const double piv = AB(j, j);
    if (piv == 0.0) continue;  // cannot happen for a connected grid
    for (long t = 1; t <= km; ++t) AB(j + t, j) = AB(j + t, j) / piv;
    const double *lcol = &AB(j + 1, j);
#pragma omp parallel for schedule(static) if (km * (ju - j) > 20000)
    for (long cc = j + 1; cc <= ju; ++cc) {
      const double m = AB(j, cc);
      if (m == 0.0) continue;
      double *dst = &AB(j + 1, cc);
      for (long t = 0; t < km; ++t) dst[t] = dst[t] - lcol[t] * m;
    }
  }
  // solve M y = e_pin
  std::vector<double> y(n, 0.0);
  y[pin] = 1.0;
  for (long j = 0; j < n; ++j) {
    if (ipiv[j] != j) std::swap(y[j], y[ipiv[j]]);
    const long km = std::min<long>(kl, n - 1 - j);
    for (long t = 1; t <= km; ++t) y[j + t] = y[j + t] - AB(j + t, j) * y[j];
  }
  for (long j = n - 1; j >= 0; --j) {
    y[j] = y[j] / AB(j, j);
    const double yj = y[j];
    for (long i = std::max<long>(0, j - kv); i < j; ++i) y[i] = y[i] - AB(i, j) * yj;
  }
  std::vector<double> z(n);
  double zz = 0.0;
  for (long u = 0; u < n; ++u) {
    z[u] = y[q(u)];
    zz += z[u] * z[u];
  }
  const double s = 1.0 / std::sqrt(zz);
  for (long u = 0; u < n; ++u) z[u] = z[u] * s;
  return z;
}

void Mud2cr::apply_finest(const double *phif, double *out) const {
  Level F = lv_[ngrid_ - 1];  // copy: keeps the solver state untouched
  const int nx = nfx_, ny = nfy_;
  std::fill(F.phi.begin(), F.phi.end(), 0.0);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) F.P(i, j) = phif[(size_t)(j - 1) * nx + (i - 1)];
  for (int j = 1; j <= ny; ++j) {
    F.P(0, j) = F.P(nx - 1, j);
    F.P(nx + 1, j) = F.P(2, j);
  }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i)
      out[(size_t)(j - 1) * nx + (i - 1)] =
          F.C(i, j, 1) * F.P(i + 1, j) + F.C(i, j, 2) * F.P(i + 1, j + 1) + F.C(i, j, 3) * F.P(i, j + 1) +
          F.C(i, j, 4) * F.P(i - 1, j + 1) + F.C(i, j, 5) * F.P(i - 1, j) + F.C(i, j, 6) * F.P(i - 1, j - 1) +
          F.C(i, j, 7) * F.P(i, j - 1) + F.C(i, j, 8) * F.P(i + 1, j - 1) + F.C(i, j, 9) * F.P(i, j);
}

}  // namespace ekref
