// Oracle (test infrastructure): restatement of the MUDPACK 5.0 subset that
// MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201) reaches: mud2cr with
// method=0 (point relaxation), FMG start (iguess=0), k-cycles, full-weighting
// restriction and linear/cubic prolongation, periodic x (nxa=nxb=0) and the
// pure-Neumann mixed condition of bndcr in y (nyc=nyd=2, alfa=0, beta=1,
// gama=0, gbdy=0; src/mg_solver2d.F90:206-255).
#pragma once
#include <functional>
#include <vector>

namespace ekref {

// Coefficients cofcr (src/duct.F90:3900-3934) at MUDPACK coordinate (x,y).
using CoefFn = std::function<void(double x, double y, double &cxx, double &cxy, double &cyy,
                                  double &cx, double &cy, double &ce)>;

struct MudOpts {
  int ixp, jyq, iex, jey;  // nfx = ixp*2^(iex-1)+1, nfy = jyq*2^(jey-1)+1
  int kcycle = 2, iprer = 2, ipost = 1, intpol = 3;
  int maxcy = 6;
  int stop_rule = 0;       // 0 relative change (MUDPACK), 1 residual norm
  double tol = 0.0;
};

struct MudResult {
  int cycles = 0;          // k-cycles executed after FMG
  bool converged = false;
  double relmax = 0.0;     // last relative change
  double resid = 0.0;      // last relative residual (stop_rule 1)
};

class Mud2cr {
 public:
  explicit Mud2cr(const MudOpts &o);
  // intl=0 call: discretize at every level (mud2cr.f:180-196 -> dismd2cr).
  void discretize(const CoefFn &coef);
  // intl=1 call: rhsf, phif are (nfx, nfy) column-major; phif is input guess
  // (the reference always passes zeros) and output solution.
  // singular: the problem has ce = 0 (kx = 0, pure Neumann/periodic).  Under
  // the relative-change rule it runs as MUDPACK does.  Under the residual
  // rule it is made well posed (not a reference behaviour): the right-hand
  // side's component along the left null vector z of the finest operator
  // (A^T z = 0, from left_null) is removed, b' = b - (z.b / z.z) z, the
  // k-cycles run until ||b' - A phi|| <= tol ||b'||, and the solution is
  // shifted to zero mean over the nfx x nfy points.  z must then be given.
  MudResult solve(const double *rhsf, double *phif, bool singular = false, const double *z = nullptr);
  // out = A phi at the finest level on (1..nfx, 1..nfy).
  void apply_finest(const double *phif, double *out) const;
  // The finest operator as coordinate triplets over the nfx*nfy unknowns
  // (unknown (i, j) -> (j-1)*nfx + i-1): the periodic ghosts of columns 0
  // and nfx+1 folded onto i = nfx-1 and i = 2, the y ghosts (zero couplings
  // after the Neumann folding) dropped.
  void finest_coo(std::vector<int> &row, std::vector<int> &col, std::vector<double> &val) const;
  // Left null vector of the finest operator as last discretized (kx = 0):
  // A^T z = 0 with |z|_2 = 1, by a banded LU with partial pivoting of A^T
  // with the equation of the centre point replaced by z = 1 there.
  std::vector<double> left_null() const;
  int nfx() const { return nfx_; }
  int nfy() const { return nfy_; }
  int ngrid() const { return ngrid_; }

 private:
  struct Level {
    int nx, ny;
    std::vector<double> phi;  // (0:nx+1, 0:ny+1)
    std::vector<double> cof;  // cf(nx, ny, 10), 10th = right-hand side
    double &P(int i, int j) { return phi[(size_t)j * (nx + 2) + i]; }
    double &C(int i, int j, int l) { return cof[((size_t)(l - 1) * ny + (j - 1)) * nx + (i - 1)]; }
  };
  MudOpts o_;
  int ngrid_, nfx_, nfy_;
  std::vector<Level> lv_;     // index k-1 for MUDPACK level k (1 = coarsest)
  std::vector<double> work_;  // wk(kps): residual / correction scratch
  double xa_ = 0, xb_ = 0, yc_ = 0, yd_ = 0;

  void dismd2cr(Level &L, const CoefFn &coef);
  void relmd2crp(Level &L);
  void resmd2cr(Level &F, Level &C);
  void res2(int nx, int ny, const double *resf, Level &C);
  void trsfc2(Level &F, Level &C);
  void prolon2(int ncx, int ncy, Level &P, int nx, int ny, double *q);
  void prolon1(int ncx, const double *p, int nx, double *q);
  void cor2(Level &F, Level &C);
  void kcymd2cr(int kcur);
};

}  // namespace ekref
