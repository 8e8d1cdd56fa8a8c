// Host-side setup of one ghost-cell cylinder case: classification, ghost
// extension stencils, the irregular rows of the pressure and Helmholtz
// operators, the boundary Schur rows and the surface quadrature stencils.
// Compiled with -ffp-contract=off so that every classification and index
// decision is made with the same IEEE operations, in the same order, as the
// reference's numpy code.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gm {

struct Csr {
  std::vector<int64_t> ptr{0};
  std::vector<int64_t> col;
  std::vector<double> val;
  int64_t rows() const { return (int64_t)ptr.size() - 1; }
  int64_t nnz() const { return (int64_t)col.size(); }
};

// Separable rectangle of one MAC field (solver/rectangular_inverse.py:8-58).
struct Rect {
  int kind = 0;            // 0 pressure, 1 u, 2 v
  int rows = 0, cols = 0;  // rectangle grid
  int64_t base = 0;        // offset of rectangle (0,0) in the field grid
  int64_t pitch = 0;       // row pitch of the field grid
  // Tridiagonal x/y operators: sub (entry i,i-1), main, sup (entry i,i+1), already /h^2.
  std::vector<double> xsub, xmain, xsup, ysub, ymain, ysup;
  double scale = 1.0;      // pressure: 1/rho multiplies lap; Helmholtz: c = 0.5*dt*nu
  bool helmholtz = false;
  // Value of the assembled rectangle entry (row r, col c) in rectangle flat indices.
  double entry(int64_t r, int64_t c) const;
  double diag_max() const;
};

struct Geometry {
  // configuration
  int nx = 0, ny = 0;
  double Lx = 0, Ly = 0, dx = 0, dy = 0, D = 0, R = 0, xc = 0, yc = 0, nu = 0, rho = 1, U_inf = 1,
         U_m = 1, U_ref = 1;
  int inflow = 0, pressure_solver = 0, pressure_extension = 0, velocity_interpolation = 0;
  int64_t usize = 0, vsize = 0, psize = 0;
  std::vector<double> xu, yu, xv, yv;
  std::vector<double> dist_u, dist_v, dist_p;
  std::vector<uint8_t> act_u, act_v, act_p, mask;
  std::vector<int64_t> ui, vi, pi;
  std::vector<int64_t> lab_u, lab_v, lab_p;
  std::vector<double> u_inlet;
  // ghost rows (grid flat index) and their stencils over grid flat indices
  std::vector<int64_t> gu_rows, gv_rows, gp_rows;
  Csr gu, gv, gp;
  std::vector<int32_t> ghost_of_u, ghost_of_v, ghost_of_p;  // grid -> ghost row or -1
  // pressure-extension fit statistics (quadratic option)
  double fit_condition_max = 0, fit_reproduction_max = 0;
  int fit_neighbors_max = 0;
  // pressure operator A = D G on active cells: irregular rows (grid flat row ->
  // CSR over grid flat p indices); regular rows equal the rectangle stencil.
  std::vector<int64_t> a_rows;
  Csr a_irr;
  std::vector<int32_t> a_nnz_row;  // nnz of every active row of A (roundoff weights)
  // boundary Schur data for the pressure rectangle
  Rect rect_p;
  std::vector<int64_t> schur_p_rows;  // rectangle flat indices
  Csr schur_p_c;                      // delta rows, columns = rectangle flat indices
  double schur_p_tol = 0;
  // surface quadrature
  int n_surface = 0;
  std::vector<double> surf_y, surf_x, normal_wx, normal_wy, normal_x, normal_y;
  Csr surf_p, dudn, dvdn;  // columns: grid flat indices of p, u, v
  // diff_offset factor per row j for u faces at i=1 (nu * (1/dx^2)) and whether (j,1) is active
  std::string error;
};

// Helmholtz data depends on dt (solver/optimized_ghost_cell.py:243-255).
struct HelmholtzSetup {
  double dt = 0;
  Rect rect[2];                       // u, v
  std::vector<int64_t> rows_irr[2];   // grid flat rows (u grid, v grid) that differ from the rectangle
  Csr irr[2];                         // actual rows over grid flat indices of the same field
  std::vector<int64_t> schur_rows[2]; // rectangle flat indices
  Csr schur_c[2];
  double tol[2] = {0, 0};
};

// Returns empty string on success, else the error text; err_class set to GM_E*.
bool build_geometry(Geometry& g, int& err_class);
bool build_helmholtz(const Geometry& g, double dt, HelmholtzSetup& hs, int& err_class, std::string& err);

// Pressure side of a cut-cell case (solver/cut_cell_solver.py:132-216, 376-400): the cut-cell
// Poisson operator over the fluid and cut cells (face-aperture-weighted five-point rows, the
// outlet Dirichlet row, covered cells decoupled) as irregular rows against the rectangle of
// the pressure grid with its boundary Schur rows, the active face maps of the u / v unknowns
// (ax[:, 1:] > 0, ay[1:-1, :] > 0), the inlet profile and the surface quadrature points with
// their point-pressure reconstruction.  The density enters through the caller's right-hand
// side: the operator is built with unit density and g.rho is set to 1.  ax: ny x (nx+1), ay: (ny+1) x nx, cell_type:
// ny x nx (1 fluid, 0 cut, -1 covered).
// The rows of cut cells (cell_type 0) are divided by their fluid fraction kappa (and so must be
// their right-hand sides): a residual of this system is then the reference's divergence measure
// |b - A x| / kappa (solver/cut_cell_solver.py:721-722), which the refinement drives down.
bool build_cutcell_geometry(Geometry& g, const double* ax, const double* ay, const int32_t* cell_type,
                            const double* kappa, int& err_class);

// Quadratic point-pressure reconstruction at the points (py[k], px[k]) (solver/cut_cell_solver.py:25-55):
// rows = points, columns = grid flat p indices; false with err set for invalid points.
bool pressure_reconstruction(const Geometry& g, const std::vector<double>& py, const std::vector<double>& px,
                             Csr& out, std::string& err);

// Least-squares helpers (min-norm solution of B w = t with B m x n, m <= n).
bool min_norm_lstsq(int m, int n, const double* B /*row-major m x n*/, const double* t, double* w,
                    double rcond, int* rank);

// Dense LU with partial pivoting (row-major n x n, in place); returns false on an exact zero pivot.
bool lu_factor(int n, double* a, int* piv);
void lu_inverse(int n, const double* lu, const int* piv, double* inv);

}  // namespace gm
