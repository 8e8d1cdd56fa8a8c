// Host setup of a ghost-cell cylinder case (see geometry.hpp).
// Build with -ffp-contract=off: classification and stencil indices must come
// out of the same IEEE operations as the reference's numpy code.
#include "geometry.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>

namespace gm {

static const double EPS = std::numeric_limits<double>::epsilon();
static const double PI = 3.141592653589793238462643383279502884;

// ---------------------------------------------------------------------------
// small dense linear algebra
// ---------------------------------------------------------------------------

// Householder QR of the n x m matrix At (column-major, n >= m) in place.
// On return the upper triangle of the first m rows holds R; v vectors below.
static void householder_qr(int n, int m, double* At, double* beta) {
  for (int k = 0; k < m; ++k) {
    double* col = At + (size_t)k * n;
    double norm2 = 0;
    for (int i = k; i < n; ++i) norm2 += col[i] * col[i];
    double norm = std::sqrt(norm2);
    if (norm == 0) { beta[k] = 0; continue; }
    double alpha = col[k] > 0 ? -norm : norm;
    double v0 = col[k] - alpha;
    // v = [v0, col[k+1..]]; store v normalised so v[0]=1
    for (int i = k + 1; i < n; ++i) col[i] /= v0;
    double vnorm2 = 1.0;
    for (int i = k + 1; i < n; ++i) vnorm2 += col[i] * col[i];
    beta[k] = 2.0 / vnorm2;
    col[k] = alpha;
    for (int j = k + 1; j < m; ++j) {
      double* cj = At + (size_t)j * n;
      double s = cj[k];
      for (int i = k + 1; i < n; ++i) s += col[i] * cj[i];
      s *= beta[k];
      cj[k] -= s;
      for (int i = k + 1; i < n; ++i) cj[i] -= s * col[i];
    }
  }
}

// Singular values of the m x m upper-triangular R (column-major with leading dim ld)
// by one-sided Jacobi; returns them in s (unsorted).
static void triangular_singular_values(int m, const double* R, int ld, double* s) {
  std::vector<double> a((size_t)m * m, 0.0);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i <= j; ++i) a[(size_t)j * m + i] = R[(size_t)j * ld + i];
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        double* ap = &a[(size_t)p * m];
        double* aq = &a[(size_t)q * m];
        double alpha = 0, beta = 0, gamma = 0;
        for (int i = 0; i < m; ++i) { alpha += ap[i] * ap[i]; beta += aq[i] * aq[i]; gamma += ap[i] * aq[i]; }
        if (gamma == 0) continue;
        off = std::max(off, std::fabs(gamma) / std::sqrt(alpha * beta));
        double zeta = (beta - alpha) / (2 * gamma);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
        double c = 1 / std::sqrt(1 + t * t), sn = c * t;
        for (int i = 0; i < m; ++i) {
          double x = ap[i], y = aq[i];
          ap[i] = c * x - sn * y;
          aq[i] = sn * x + c * y;
        }
      }
    if (off < 1e-15) break;
  }
  for (int j = 0; j < m; ++j) {
    double t = 0;
    for (int i = 0; i < m; ++i) t += a[(size_t)j * m + i] * a[(size_t)j * m + i];
    s[j] = std::sqrt(t);
  }
}

// Min-norm solution of B w = t, B row-major m x n (m <= n), via QR of B^T.
// rank = number of singular values above rcond * max; the solution assumes full rank.
static bool lstsq_full(int m, int n, const double* B, const double* t, double* w, double rcond, int* rank,
                       double* cond) {
  std::vector<double> At((size_t)n * m), beta(m);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) At[(size_t)i * n + j] = B[(size_t)i * n + j];  // column i of B^T
  householder_qr(n, m, At.data(), beta.data());
  std::vector<double> s(m);
  triangular_singular_values(m, At.data(), n, s.data());
  double smax = *std::max_element(s.begin(), s.end());
  double smin = *std::min_element(s.begin(), s.end());
  int r = 0;
  for (double v : s) r += v > rcond * smax;
  *rank = r;
  if (cond) *cond = smin > 0 ? smax / smin : std::numeric_limits<double>::infinity();
  if (r < m) return false;
  // R^T z = t (forward substitution), R = upper triangle of At (column-major, ld n)
  std::vector<double> z(m);
  for (int i = 0; i < m; ++i) {
    double acc = t[i];
    for (int k = 0; k < i; ++k) acc -= At[(size_t)i * n + k] * z[k];  // R[k][i]
    z[i] = acc / At[(size_t)i * n + i];
  }
  // w = Q [z; 0]: apply reflections in reverse order
  for (int j = 0; j < n; ++j) w[j] = j < m ? z[j] : 0.0;
  for (int k = m - 1; k >= 0; --k) {
    if (beta[k] == 0) continue;
    const double* v = At.data() + (size_t)k * n;
    double sdot = w[k];
    for (int i = k + 1; i < n; ++i) sdot += v[i] * w[i];
    sdot *= beta[k];
    w[k] -= sdot;
    for (int i = k + 1; i < n; ++i) w[i] -= sdot * v[i];
  }
  return true;
}

bool min_norm_lstsq(int m, int n, const double* B, const double* t, double* w, double rcond, int* rank) {
  return lstsq_full(m, n, B, t, w, rcond, rank, nullptr);
}

bool lu_factor(int n, double* a, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(a[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      double v = std::fabs(a[(size_t)i * n + k]);
      if (v > best) { best = v; p = i; }
    }
    piv[k] = p;
    if (best == 0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
    double inv = 1.0 / a[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double f = a[(size_t)i * n + k] * inv;
      a[(size_t)i * n + k] = f;
      if (f != 0)
        for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= f * a[(size_t)k * n + j];
    }
  }
  return true;
}

void lu_inverse(int n, const double* lu, const int* piv, double* inv) {
  std::vector<double> col(n);
  for (int c = 0; c < n; ++c) {
    std::fill(col.begin(), col.end(), 0.0);
    col[c] = 1.0;
    for (int k = 0; k < n; ++k) std::swap(col[k], col[piv[k]]);
    for (int i = 0; i < n; ++i) {
      double acc = col[i];
      for (int k = 0; k < i; ++k) acc -= lu[(size_t)i * n + k] * col[k];
      col[i] = acc;
    }
    for (int i = n - 1; i >= 0; --i) {
      double acc = col[i];
      for (int k = i + 1; k < n; ++k) acc -= lu[(size_t)i * n + k] * col[k];
      col[i] = acc / lu[(size_t)i * n + i];
    }
    for (int r = 0; r < n; ++r) inv[(size_t)r * n + c] = col[r];
  }
}

// ---------------------------------------------------------------------------
// rectangle operator entries (solver/rectangular_inverse.py:9-38)
// ---------------------------------------------------------------------------
static void make_rect(Rect& r, int kind, int nx, int ny, double dx, double dy, double nu, double dt, double rho) {
  r.kind = kind;
  double left, right, lower, upper;
  if (kind == 0) { r.rows = ny; r.cols = nx; left = 1; right = 3; lower = 1; upper = 1; r.base = 0; r.pitch = nx; }
  else if (kind == 1) { r.rows = ny; r.cols = nx; left = 2; right = 2; lower = 3; upper = 3; r.base = 1; r.pitch = nx + 1; }
  else { r.rows = ny - 1; r.cols = nx; left = 3; right = 1; lower = 2; upper = 2; r.base = nx; r.pitch = nx; }
  const double dx2 = dx * dx, dy2 = dy * dy;
  int X = r.cols, Y = r.rows;
  r.xsub.assign(X, 0); r.xmain.assign(X, 0); r.xsup.assign(X, 0);
  r.ysub.assign(Y, 0); r.ymain.assign(Y, 0); r.ysup.assign(Y, 0);
  for (int i = 0; i < X; ++i) {
    double d = -2.0;
    if (i == 0) d = -left;
    if (i == X - 1) d = -right;
    r.xmain[i] = d / dx2;
    if (i >= 1) r.xsub[i] = ((kind == 1 && i == X - 1) ? 2.0 : 1.0) / dx2;
    if (i <= X - 2) r.xsup[i] = 1.0 / dx2;
  }
  for (int j = 0; j < Y; ++j) {
    double d = -2.0;
    if (j == 0) d = -lower;
    if (j == Y - 1) d = -upper;
    r.ymain[j] = d / dy2;
    if (j >= 1) r.ysub[j] = 1.0 / dy2;
    if (j <= Y - 2) r.ysup[j] = 1.0 / dy2;
  }
  if (kind == 0) { r.helmholtz = false; r.scale = rho; }
  else { r.helmholtz = true; r.scale = (0.5 * dt) * nu; }
}

double Rect::entry(int64_t rr, int64_t cc) const {
  int64_t j = rr / cols, i = rr % cols, jc = cc / cols, ic = cc % cols;
  double lap;
  bool diag = false;
  if (rr == cc) { lap = xmain[i] + ymain[j]; diag = true; }
  else if (j == jc && ic == i - 1) lap = xsub[i];
  else if (j == jc && ic == i + 1) lap = xsup[i];
  else if (i == ic && jc == j - 1) lap = ysub[j];
  else if (i == ic && jc == j + 1) lap = ysup[j];
  else return 0.0;
  if (!helmholtz) return lap / scale;
  double m = scale * lap;
  return diag ? 1.0 - m : -m;
}

double Rect::diag_max() const {
  double best = 0;
  for (int j = 0; j < rows; ++j)
    for (int i = 0; i < cols; ++i) best = std::max(best, std::fabs(entry((int64_t)j * cols + i, (int64_t)j * cols + i)));
  return best;
}

// ---------------------------------------------------------------------------
// ghost extension (solver/optimized_ghost_cell.py:14-58)
// ---------------------------------------------------------------------------
static inline double circle_distance(double x, double y, double xc, double yc, double R) {
  double ax = x - xc, ay = y - yc;
  return std::sqrt(ax * ax + ay * ay) - R;
}

static bool extension(const std::vector<double>& x, const std::vector<double>& y, double xc, double yc,
                      double R, const std::vector<double>& dist, const std::vector<int64_t>& label,
                      bool neumann, bool quad, std::vector<int64_t>& rows, Csr& st,
                      std::vector<int32_t>& ghost_of, std::string& err) {
  const int X = (int)x.size(), Y = (int)y.size();
  const double sx = x[1] - x[0], sy = y[1] - y[0];
  const double h = std::max(sx, sy);
  const int width = quad ? 3 : 2;
  ghost_of.assign((size_t)X * Y, -1);
  rows.clear();
  st = Csr();
  for (int j = 0; j < Y; ++j)
    for (int i = 0; i < X; ++i) {
      double dd = dist[(size_t)j * X + i];
      if (!(dd <= 1e-13 && dd >= -2 * h)) continue;
      double d = (-dd > 0.0) ? -dd : 0.0;
      double ax = x[i] - xc, ay = y[j] - yc;
      double r = std::sqrt(ax * ax + ay * ay);
      if (!(r >= 1e-14)) r = 1e-14;
      double nxv = ax / r, nyv = ay / r;
      double s = (d >= 1.5 * h) ? d : 1.5 * h;
      int64_t cols[2][9];
      double w[2][9];
      bool ok = false;
      for (int attempt = 0; attempt < 8 && !ok; ++attempt) {
        bool all = true;
        for (int pr = 0; pr < 2; ++pr) {
          double ell = pr == 0 ? s : 2 * s;
          double px = x[i] + (d + ell) * nxv;
          double py = y[j] + (d + ell) * nyv;
          double fi = (px - x[0]) / sx;
          double fj = (py - y[0]) / sy;
          int64_t i0, j0;
          if (quad) { i0 = (int64_t)std::floor(fi + 0.5) - 1; j0 = (int64_t)std::floor(fj + 0.5) - 1; }
          else { i0 = (int64_t)std::floor(fi); j0 = (int64_t)std::floor(fj); }
          if (!(0 <= i0 && i0 <= X - width && 0 <= j0 && j0 <= Y - width)) {
            err = "Ghost probe reaches an outer boundary";
            return false;
          }
          double a = fi - i0, b = fj - j0;
          int k = 0;
          for (int rj = 0; rj < width; ++rj)
            for (int ri = 0; ri < width; ++ri) {
              int64_t lab = label[(size_t)(j0 + rj) * X + (i0 + ri)];
              cols[pr][k] = lab < 0 ? -1 : (j0 + rj) * (int64_t)X + (i0 + ri);
              if (lab < 0) all = false;
              ++k;
            }
          if (quad) {
            double wx[3] = {(0.5 * (a - 1)) * (a - 2), (-a) * (a - 2), (0.5 * a) * (a - 1)};
            double wy[3] = {(0.5 * (b - 1)) * (b - 2), (-b) * (b - 2), (0.5 * b) * (b - 1)};
            for (int rj = 0; rj < 3; ++rj)
              for (int ri = 0; ri < 3; ++ri) w[pr][rj * 3 + ri] = wy[rj] * wx[ri];
          } else {
            w[pr][0] = (1 - a) * (1 - b);
            w[pr][1] = a * (1 - b);
            w[pr][2] = (1 - a) * b;
            w[pr][3] = a * b;
          }
        }
        if (all) ok = true;
        else s *= 1.25;
      }
      if (!ok) { err = "No exterior ghost stencil"; return false; }
      double f[2];
      if (neumann) {
        f[0] = (((4 * s) * s) - d * d) / ((3 * s) * s);
        f[1] = (d * d - s * s) / ((3 * s) * s);
      } else {
        f[0] = ((-d) * (d + 2 * s)) / (s * s);
        f[1] = (d * (d + s)) / ((2 * s) * s);
      }
      // sum duplicates; column order ascending (scipy canonical CSR)
      std::map<int64_t, double> acc;
      const int n = width * width;
      for (int pr = 0; pr < 2; ++pr)
        for (int k = 0; k < n; ++k) {
          double v = f[pr] * w[pr][k];
          auto it = acc.find(cols[pr][k]);
          if (it == acc.end()) acc.emplace(cols[pr][k], v);
          else it->second = it->second + v;
        }
      ghost_of[(size_t)j * X + i] = (int32_t)rows.size();
      rows.push_back((int64_t)j * X + i);
      for (auto& kv : acc) { st.col.push_back(kv.first); st.val.push_back(kv.second); }
      st.ptr.push_back((int64_t)st.col.size());
    }
  return true;
}

// k nearest candidates (with ties within 1e-12 relative) of point (py, px)
static void neighbours(const std::vector<double>& cy, const std::vector<double>& cx, double py, double px, int k,
                       std::vector<int>& out) {
  const int n = (int)cy.size();
  std::vector<double> d2(n);
  for (int c = 0; c < n; ++c) {
    double a = cy[c] - py, b = cx[c] - px;
    d2[c] = a * a + b * b;
  }
  std::vector<double> tmp(d2);
  int kk = std::min(k, n);
  std::nth_element(tmp.begin(), tmp.begin() + (kk - 1), tmp.end());
  double r = std::sqrt(tmp[kk - 1]) * (1 + 1e-12);
  double r2 = r * r;
  out.clear();
  for (int c = 0; c < n; ++c)
    if (d2[c] <= r2) out.push_back(c);
}

// quadratic exterior pressure continuation (solver/ghost_reconstruction.py:7-45)
static bool quadratic_extension(Geometry& g, std::vector<int64_t>& rows, Csr& st, std::vector<int32_t>& ghost_of,
                                std::string& err) {
  const int X = g.nx, Y = g.ny;
  const double hx = g.xv[1] - g.xv[0], hy = g.yu[1] - g.yu[0];
  const double h = std::max(hx, hy);
  std::vector<double> cy, cx;
  std::vector<int64_t> pool;
  for (int j = 0; j < Y; ++j)
    for (int i = 0; i < X; ++i) {
      size_t f = (size_t)j * X + i;
      if (g.act_p[f] && g.dist_p[f] < 6 * h) { pool.push_back((int64_t)f); cy.push_back(g.yu[j]); cx.push_back(g.xv[i]); }
    }
  if (pool.size() < 12) { err = "Pressure continuation needs twelve exterior centers"; return false; }
  ghost_of.assign((size_t)X * Y, -1);
  rows.clear();
  st = Csr();
  std::vector<int> near;
  for (int j = 0; j < Y; ++j)
    for (int i = 0; i < X; ++i) {
      size_t f = (size_t)j * X + i;
      double dd = g.dist_p[f];
      if (!(dd <= 1e-13 && dd >= -2 * h)) continue;
      double py = g.yu[j], px = g.xv[i];
      bool done = false;
      std::vector<double> w;
      double cond = 0, errv = 0;
      for (int count : {12, 20, 32}) {
        neighbours(cy, cx, py, px, std::min(count, (int)pool.size()), near);
        int n = (int)near.size();
        std::vector<double> B(6 * (size_t)n);
        for (int c = 0; c < n; ++c) {
          double oy = (cy[near[c]] - py) / hy, ox = (cx[near[c]] - px) / hx;
          B[0 * n + c] = 1.0; B[1 * n + c] = ox; B[2 * n + c] = oy;
          B[3 * n + c] = ox * ox; B[4 * n + c] = ox * oy; B[5 * n + c] = oy * oy;
        }
        double t[6] = {1, 0, 0, 0, 0, 0};
        w.assign(n, 0.0);
        int rank = 0;
        bool full = lstsq_full(6, n, B.data(), t, w.data(), 1e-12, &rank, &cond);
        if (!full) continue;
        int big = 0;
        for (int c = 1; c < n; ++c) if (std::fabs(w[c]) > std::fabs(w[big])) big = c;
        double sum = 0;
        for (int c = 0; c < n; ++c) sum += w[c];
        w[big] += 1 - sum;
        errv = 0;
        for (int r = 0; r < 6; ++r) {
          double acc = 0;
          for (int c = 0; c < n; ++c) acc += B[r * (size_t)n + c] * w[c];
          errv = std::max(errv, std::fabs(acc - t[r]));
        }
        if (rank == 6 && std::isfinite(cond) && cond <= 1e8 && errv <= 1e-10) { done = true; break; }
      }
      if (!done) { err = "Unresolved exterior pressure polynomial"; return false; }
      g.fit_condition_max = std::max(g.fit_condition_max, cond);
      g.fit_reproduction_max = std::max(g.fit_reproduction_max, errv);
      g.fit_neighbors_max = std::max(g.fit_neighbors_max, (int)near.size());
      ghost_of[f] = (int32_t)rows.size();
      rows.push_back((int64_t)f);
      std::vector<std::pair<int64_t, double>> e;
      for (size_t c = 0; c < near.size(); ++c) e.emplace_back(pool[near[c]], w[c]);
      std::sort(e.begin(), e.end());
      for (auto& kv : e) { st.col.push_back(kv.first); st.val.push_back(kv.second); }
      st.ptr.push_back((int64_t)st.col.size());
    }
  return true;
}

// ---------------------------------------------------------------------------
// sparse rows of the folded operators
// ---------------------------------------------------------------------------
using Row = std::vector<std::pair<int64_t, double>>;  // ordered by first appearance

static inline void acc_add(Row& row, std::map<int64_t, size_t>& where, int64_t col, double v) {
  auto it = where.find(col);
  if (it == where.end()) { where.emplace(col, row.size()); row.emplace_back(col, 0.0 + v); }
  else row[it->second].second += v;
}

// E (or P) row of a grid point: identity for active points, ghost stencil for ghost
// points, empty otherwise.  Columns are grid flat indices of the same field.
static Row ext_row(const std::vector<uint8_t>& act, const std::vector<int32_t>& ghost_of, const Csr& st, int64_t f) {
  Row r;
  if (act[f]) { r.emplace_back(f, 1.0); return r; }
  int32_t g = ghost_of[f];
  if (g >= 0)
    for (int64_t k = st.ptr[g]; k < st.ptr[g + 1]; ++k) r.emplace_back(st.col[k], st.val[k]);
  return r;
}

// gradient row (G = raw_g P / rho) of an active face; field 0 = u, 1 = v
static Row grad_row(const Geometry& g, int field, int64_t f) {
  const int nx = g.nx;
  std::vector<std::pair<int64_t, double>> raw;
  if (field == 0) {
    int64_t j = f / (nx + 1), i = f % (nx + 1);
    if (i < nx) { raw.emplace_back(j * nx + i - 1, -1.0 / g.dx); raw.emplace_back(j * nx + i, 1.0 / g.dx); }
    else raw.emplace_back(j * nx + nx - 1, -2.0 / g.dx);
  } else {
    int64_t j = f / nx, i = f % nx;
    raw.emplace_back((j - 1) * nx + i, -1.0 / g.dy);
    raw.emplace_back(j * nx + i, 1.0 / g.dy);
  }
  Row out;
  std::map<int64_t, size_t> where;
  for (auto& e : raw) {
    Row pr = ext_row(g.act_p, g.ghost_of_p, g.gp, e.first);
    for (auto& q : pr) acc_add(out, where, q.first, e.second * q.second);
  }
  for (auto& e : out) e.second = e.second / g.rho;
  return out;
}

// A = D G row of an active p cell (solver/optimized_ghost_cell.py:85-108)
static Row pressure_row(const Geometry& g, int64_t c) {
  const int nx = g.nx;
  int64_t j = c / nx, i = c % nx;
  struct F { int field; int64_t f; double coef; };
  F faces[4] = {{0, j * (nx + 1) + i, -1.0 / g.dx}, {0, j * (nx + 1) + i + 1, 1.0 / g.dx},
                {1, j * nx + i, -1.0 / g.dy}, {1, (j + 1) * nx + i, 1.0 / g.dy}};
  // D row = Dfull row @ E (face -> active faces)
  Row drow;
  std::map<int64_t, size_t> dwhere;  // key: field*2^40 + flat
  for (auto& fc : faces) {
    Row er = fc.field == 0 ? ext_row(g.act_u, g.ghost_of_u, g.gu, fc.f) : ext_row(g.act_v, g.ghost_of_v, g.gv, fc.f);
    for (auto& e : er) acc_add(drow, dwhere, ((int64_t)fc.field << 40) + e.first, fc.coef * e.second);
  }
  Row arow;
  std::map<int64_t, size_t> awhere;
  for (auto& d : drow) {
    if (d.second == 0.0) continue;
    int field = (int)(d.first >> 40);
    int64_t f = d.first & ((1LL << 40) - 1);
    Row gr = grad_row(g, field, f);
    for (auto& e : gr) acc_add(arow, awhere, e.first, d.second * e.second);
  }
  Row out;
  for (auto& e : arow) if (e.second != 0.0) out.push_back(e);
  return out;
}

// Helmholtz actual row I - dt/2 * (nu raw_l E) of an active face (solver/optimized_ghost_cell.py:113-128, 248-251)
static Row helmholtz_row(const Geometry& g, int field, int64_t f, double dt) {
  const int nx = g.nx, ny = g.ny;
  const double dx2 = g.dx * g.dx, dy2 = g.dy * g.dy;
  std::vector<std::pair<int64_t, double>> raw;  // sorted by column
  if (field == 0) {
    int64_t j = f / (nx + 1), i = f % (nx + 1);
    if (j > 0) raw.emplace_back(f - nx - 1, 1 / dy2);
    raw.emplace_back(f - 1, (i == nx ? 2.0 : 1.0) / dx2);
    raw.emplace_back(f, -2 / dx2 - ((j == 0 || j == ny - 1) ? 3.0 : 2.0) / dy2);
    if (i < nx) raw.emplace_back(f + 1, 1 / dx2);
    if (j < ny - 1) raw.emplace_back(f + nx + 1, 1 / dy2);
  } else {
    int64_t i = f % nx;
    raw.emplace_back(f - nx, 1 / dy2);
    if (i > 0) raw.emplace_back(f - 1, 1 / dx2);
    raw.emplace_back(f, -(i == 0 ? 3.0 : (i == nx - 1 ? 1.0 : 2.0)) / dx2 - 2 / dy2);
    if (i < nx - 1) raw.emplace_back(f + 1, 1 / dx2);
    raw.emplace_back(f + nx, 1 / dy2);
  }
  Row lrow;
  std::map<int64_t, size_t> where;
  for (auto& e : raw) {
    Row er = field == 0 ? ext_row(g.act_u, g.ghost_of_u, g.gu, e.first) : ext_row(g.act_v, g.ghost_of_v, g.gv, e.first);
    double scaled = g.nu * e.second;
    for (auto& q : er) acc_add(lrow, where, q.first, scaled * q.second);
  }
  const double c = 0.5 * dt;
  Row out;
  bool has_diag = false;
  for (auto& e : lrow) {
    if (e.second == 0.0) continue;
    double m = c * e.second;
    if (e.first == f) { out.emplace_back(e.first, 1.0 - m); has_diag = true; }
    else out.emplace_back(e.first, -m);
  }
  if (!has_diag) out.emplace_back(f, 1.0);
  return out;
}

// rectangle flat index of a field flat index (-1 when outside the rectangle)
static int64_t rect_index(const Rect& r, int field_kind, int nx, int64_t f) {
  if (field_kind == 0) return f;
  if (field_kind == 1) { int64_t j = f / (nx + 1), i = f % (nx + 1); return i >= 1 ? j * nx + i - 1 : -1; }
  int64_t j = f / nx, i = f % nx;
  return (j >= 1 && j <= r.rows) ? (j - 1) * nx + i : -1;
}
static int64_t field_index(const Rect& r, int field_kind, int nx, int64_t rf) {
  int64_t j = rf / r.cols, i = rf % r.cols;
  if (field_kind == 0) return rf;
  if (field_kind == 1) return j * (nx + 1) + i + 1;
  return (j + 1) * nx + i;
}

// Schur rows and delta (solver/pressure_schur.py:77-91) for one rectangle.
// actual(f) returns the active row of field flat index f (columns field flat).
template <class RowFn>
static void schur_setup(const Geometry& g, const Rect& rect, int field_kind, const std::vector<uint8_t>& act,
                        RowFn actual, std::vector<int64_t>& irr_rows, Csr& irr, std::vector<int64_t>& srows, Csr& C,
                        double& tol, std::vector<int32_t>* nnz_out) {
  const int nx = g.nx;
  const int64_t n = (int64_t)rect.rows * rect.cols;
  tol = 8 * EPS * std::max(1.0, rect.diag_max());
  irr_rows.clear(); irr = Csr(); srows.clear(); C = Csr();
  std::vector<uint8_t> cov(n);
  for (int64_t r = 0; r < n; ++r) cov[r] = !act[field_index(rect, field_kind, nx, r)];
  for (int64_t r = 0; r < n; ++r) {
    int64_t f = field_index(rect, field_kind, nx, r);
    int64_t j = r / rect.cols, i = r % rect.cols;
    // rectangle row: (col, value)
    std::vector<std::pair<int64_t, double>> rrow;
    if (j > 0) rrow.emplace_back(r - rect.cols, rect.entry(r, r - rect.cols));
    if (i > 0) rrow.emplace_back(r - 1, rect.entry(r, r - 1));
    rrow.emplace_back(r, rect.entry(r, r));
    if (i < rect.cols - 1) rrow.emplace_back(r + 1, rect.entry(r, r + 1));
    if (j < rect.rows - 1) rrow.emplace_back(r + rect.cols, rect.entry(r, r + rect.cols));
    std::map<int64_t, double> delta;
    Row arow;
    if (!cov[r]) {
      arow = actual(f);
      for (auto& e : arow) {
        int64_t rc = rect_index(rect, field_kind, nx, e.first);
        delta[rc] += e.second;  // ext entries are distinct columns
      }
      for (auto& e : rrow) {
        auto it = delta.find(e.first);
        if (it == delta.end()) delta.emplace(e.first, 0.0 - e.second);
        else it->second = it->second - e.second;
      }
      if (nnz_out) (*nnz_out)[f] = (int32_t)arow.size();
    } else {
      for (auto& e : rrow)
        if (!cov[e.first]) delta.emplace(e.first, 0.0 - e.second);
    }
    bool any = false;
    std::vector<std::pair<int64_t, double>> kept;
    for (auto& kv : delta)
      if (std::fabs(kv.second) >= tol && kv.second != 0.0) { kept.push_back(kv); any = true; }
    if (!any) continue;
    srows.push_back(r);
    for (auto& kv : kept) { C.col.push_back(kv.first); C.val.push_back(kv.second); }
    C.ptr.push_back((int64_t)C.col.size());
    if (!cov[r]) {
      irr_rows.push_back(f);
      std::sort(arow.begin(), arow.end());
      for (auto& e : arow) { irr.col.push_back(e.first); irr.val.push_back(e.second); }
      irr.ptr.push_back((int64_t)irr.col.size());
    }
  }
}

// Quadratic point-pressure reconstruction (solver/cut_cell_solver.py:25-55): at every point
// (py[k], px[k]) the 12 nearest exterior active pressure centres of a padded window (with ties
// at the cutoff), weights from the minimum-norm least-squares fit of a quadratic.  Rows of out
// are the points, columns grid flat p indices.
bool pressure_reconstruction(const Geometry& g, const std::vector<double>& py, const std::vector<double>& px,
                             Csr& out, std::string& err) {
  const size_t count = py.size();
  if (count == 0 || px.size() != count) { err = "At least one pressure sample is required"; return false; }
  for (size_t k = 0; k < count; ++k) {
    if (!std::isfinite(py[k]) || !std::isfinite(px[k])) {
      err = "Pressure sample points must be finite (y, x) pairs";
      return false;
    }
  }
  for (size_t k = 0; k < count; ++k)
    if (py[k] < 0 || py[k] > g.Ly || px[k] < 0 || px[k] > g.Lx) {
      err = "Pressure sample points must lie inside the domain";
      return false;
    }
  for (size_t k = 0; k < count; ++k)
    if (std::hypot(px[k] - g.xc, py[k] - g.yc) < g.R * (1 - 1e-12)) {
      err = "Physical pressure cannot be sampled inside the solid";
      return false;
    }
  const double pad = 4 * std::max(g.dx, g.dy);
  const double ymin = *std::min_element(py.begin(), py.end());
  const double xmin = *std::min_element(px.begin(), px.end());
  const double ymax = *std::max_element(py.begin(), py.end());
  const double xmax = *std::max_element(px.begin(), px.end());
  const int64_t jlo = std::max<int64_t>(0, (int64_t)std::floor((ymin - pad) / g.dy));
  const int64_t ilo = std::max<int64_t>(0, (int64_t)std::floor((xmin - pad) / g.dx));
  const int64_t jhi = std::min<int64_t>(g.ny, (int64_t)std::ceil((ymax + pad) / g.dy) + 1);
  const int64_t ihi = std::min<int64_t>(g.nx, (int64_t)std::ceil((xmax + pad) / g.dx) + 1);
  std::vector<double> cy, cx;
  std::vector<int64_t> ids;
  for (int64_t j = jlo; j < jhi; ++j)
    for (int64_t i = ilo; i < ihi; ++i) {
      double y = (j + .5) * g.dy, x = (i + .5) * g.dx;
      if (g.act_p[(size_t)j * g.nx + i] && std::hypot(x - g.xc, y - g.yc) >= g.R * (1 - 1e-12)) {
        cy.push_back(y); cx.push_back(x); ids.push_back(j * g.nx + i);
      }
    }
  if (ids.size() < 12) { err = "Pressure reconstruction needs at least 12 exterior centers"; return false; }
  std::vector<int> near;
  out = Csr();
  for (size_t k = 0; k < count; ++k) {
    neighbours(cy, cx, py[k], px[k], 12, near);
    int n = (int)near.size();
    std::vector<double> B(6 * (size_t)n), w(n);
    for (int c = 0; c < n; ++c) {
      double oy = (cy[near[c]] - py[k]) / g.dy, ox = (cx[near[c]] - px[k]) / g.dx;
      B[0 * n + c] = 1.0; B[1 * n + c] = ox; B[2 * n + c] = oy;
      B[3 * n + c] = ox * ox; B[4 * n + c] = ox * oy; B[5 * n + c] = oy * oy;
    }
    double t[6] = {1, 0, 0, 0, 0, 0};
    int rank = 0;
    if (!lstsq_full(6, n, B.data(), t, w.data(), 1e-12, &rank, nullptr) || rank != 6) {
      err = "Pressure stencil cannot resolve a quadratic polynomial";
      return false;
    }
    for (int c = 0; c < n; ++c) { out.col.push_back(ids[near[c]]); out.val.push_back(w[c]); }
    out.ptr.push_back((int64_t)out.col.size());
  }
  return true;
}

// ---------------------------------------------------------------------------
// surface quadrature (solver/cut_cell_solver.py:25-77, solver/optimized_ghost_cell.py:144-172)
// ---------------------------------------------------------------------------
static bool surface_setup(Geometry& g, std::string& err) {
  const double h_min = std::min(g.dx, g.dy), h = std::max(g.dx, g.dy);
  int count = std::max(360, 4 * (int)std::ceil(2 * PI * g.R / h_min));
  g.n_surface = count;
  g.surf_y.resize(count); g.surf_x.resize(count);
  g.normal_wx.resize(count); g.normal_wy.resize(count); g.normal_x.resize(count); g.normal_y.resize(count);
  const double step = 2 * PI / count, wscale = 2 * PI * g.R / count, nscale = PI * (2 * g.R) / count;
  const double Dd = g.D;
  for (int k = 0; k < count; ++k) {
    double th = k * step;
    double c = std::cos(th), s = std::sin(th);
    g.surf_y[k] = g.yc + g.R * s;
    g.surf_x[k] = g.xc + g.R * c;
    g.normal_wx[k] = c * wscale;
    g.normal_wy[k] = s * wscale;
    g.normal_x[k] = g.normal_wx[k] / (PI * Dd / count);
    g.normal_y[k] = g.normal_wy[k] / (PI * Dd / count);
  }
  (void)nscale;
  // pressure point reconstruction at the surface points
  if (!pressure_reconstruction(g, g.surf_y, g.surf_x, g.surf_p, err)) return false;
  // wall-normal derivative stencils for u and v
  for (int field = 0; field < 2; ++field) {
    const std::vector<double>& x = field == 0 ? g.xu : g.xv;
    const std::vector<double>& y = field == 0 ? g.yu : g.yv;
    const std::vector<uint8_t>& act = field == 0 ? g.act_u : g.act_v;
    const int X = (int)x.size(), Y = (int)y.size();
    std::vector<double> cy, cx;
    std::vector<int64_t> ids;
    for (int j = 0; j < Y; ++j)
      for (int i = 0; i < X; ++i) {
        size_t f = (size_t)j * X + i;
        if (act[f] && std::hypot(x[i] - g.xc, y[j] - g.yc) < g.R + 6 * h) {
          cy.push_back(y[j]); cx.push_back(x[i]); ids.push_back((int64_t)f);
        }
      }
    Csr& out = field == 0 ? g.dudn : g.dvdn;
    out = Csr();
    std::vector<int> near;
    for (int k = 0; k < count; ++k) {
      double py = g.surf_y[k], px = g.surf_x[k];
      neighbours(cy, cx, py, px, 14, near);
      int n = (int)near.size();
      double theta = std::atan2(py - g.yc, px - g.xc);
      std::vector<double> B(3 * (size_t)n), w(n);
      for (int c = 0; c < n; ++c) {
        double ys = cy[near[c]], xs = cx[near[c]];
        double ang = std::atan2(ys - g.yc, xs - g.xc) - theta;
        double nn = (std::hypot(xs - g.xc, ys - g.yc) - g.R) / h;
        double tt = g.R * std::atan2(std::sin(ang), std::cos(ang)) / h;
        B[0 * n + c] = nn; B[1 * n + c] = nn * nn; B[2 * n + c] = nn * tt;
      }
      double t[3] = {1 / h, 0, 0};
      int rank = 0;
      if (!lstsq_full(3, n, B.data(), t, w.data(), 1e-12, &rank, nullptr) || rank != 3) {
        err = "Unresolved wall-gradient stencil";
        return false;
      }
      for (int c = 0; c < n; ++c) { out.col.push_back(ids[near[c]]); out.val.push_back(w[c]); }
      out.ptr.push_back((int64_t)out.col.size());
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// build
// ---------------------------------------------------------------------------
bool build_geometry(Geometry& g, int& err_class) {
  err_class = 1;  // ValueError unless stated
  const int nx = g.nx, ny = g.ny;
  if (nx < 4 || ny < 4) { g.error = "nx and ny must be integers >= 4"; return false; }
  for (double v : {g.Lx, g.Ly, g.D, g.nu, g.rho, g.U_inf})
    if (!(std::isfinite(v) && v > 0)) { g.error = "Domain lengths, D, nu, rho and U_inf must be finite and positive"; return false; }
  if (g.inflow != 0 && g.inflow != 1) { g.error = "inflow must be uniform or parabolic"; return false; }
  if (std::isnan(g.U_m) || (std::isfinite(g.U_m) == false)) { g.error = "U_m must be finite and positive"; return false; }
  if (!(g.D / 2 < g.xc && g.xc < g.Lx - g.D / 2 && g.D / 2 < g.yc && g.yc < g.Ly - g.D / 2)) {
    g.error = "Cylinder must lie strictly inside the channel";
    return false;
  }
  if (g.pressure_solver != 0 && g.pressure_solver != 1) { g.error = "Ghost AB2/CN requires direct/iterative pressure and no-slip channel walls"; return false; }
  if (g.pressure_extension != 0 && g.pressure_extension != 1) { g.error = "Unknown Ghost pressure extension or velocity interpolation"; return false; }
  if (g.velocity_interpolation != 0 && g.velocity_interpolation != 1) { g.error = "Unknown Ghost pressure extension or velocity interpolation"; return false; }
  g.dx = g.Lx / nx;
  g.dy = g.Ly / ny;
  if (g.inflow == 1) { g.U_m = g.U_m > 0 ? g.U_m : 1.5 * g.U_inf; g.U_ref = (2.0 / 3.0) * g.U_m; }
  else { g.U_m = g.U_inf; g.U_ref = g.U_inf; }
  g.R = g.D / 2.0;
  g.usize = (int64_t)ny * (nx + 1);
  g.vsize = (int64_t)(ny + 1) * nx;
  g.psize = (int64_t)ny * nx;
  // mask of cell centres inside the cylinder (solver/main.py:123-129)
  g.mask.assign(g.psize, 0);
  bool any = false, edge = false;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      double xcn = (i + 0.5) * g.dx, ycn = (j + 0.5) * g.dy;
      double a = (xcn - g.xc) / (g.D / 2.0), b = (ycn - g.yc) / (g.D / 2.0);
      bool m = (a * a + b * b) <= (1.0 + 1e-13);
      g.mask[(size_t)j * nx + i] = m;
      any |= m;
      if (m && (j == 0 || j == ny - 1 || i == 0 || i == nx - 1)) edge = true;
    }
  if (!any || edge) { g.error = "Grid must resolve the cylinder and a fluid layer at every outer boundary"; return false; }
  g.u_inlet.assign(ny, 0.0);
  for (int j = 0; j < ny; ++j) {
    double y = (j + 0.5) * g.dy;
    g.u_inlet[j] = g.inflow == 1 ? (((4.0 * g.U_m) * y) * (g.Ly - y)) / (g.Ly * g.Ly) : g.U_inf;
  }
  // coordinates and distances (solver/ghost_cell.py:48-62)
  g.xu.resize(nx + 1); g.yu.resize(ny); g.xv.resize(nx); g.yv.resize(ny + 1);
  for (int i = 0; i <= nx; ++i) g.xu[i] = i * g.dx;
  for (int j = 0; j < ny; ++j) g.yu[j] = (j + 0.5) * g.dy;
  for (int i = 0; i < nx; ++i) g.xv[i] = (i + 0.5) * g.dx;
  for (int j = 0; j <= ny; ++j) g.yv[j] = j * g.dy;
  auto fill = [&](const std::vector<double>& x, const std::vector<double>& y, std::vector<double>& d) {
    d.resize(x.size() * y.size());
    for (size_t j = 0; j < y.size(); ++j)
      for (size_t i = 0; i < x.size(); ++i) d[j * x.size() + i] = circle_distance(x[i], y[j], g.xc, g.yc, g.R);
  };
  fill(g.xu, g.yu, g.dist_u);
  fill(g.xv, g.yv, g.dist_v);
  fill(g.xv, g.yu, g.dist_p);
  // active classification (solver/optimized_ghost_cell.py:66-70)
  g.act_u.resize(g.usize); g.act_v.resize(g.vsize); g.act_p.resize(g.psize);
  for (int64_t f = 0; f < g.usize; ++f) g.act_u[f] = g.dist_u[f] > 1e-13 && (f % (nx + 1)) != 0;
  for (int64_t f = 0; f < g.vsize; ++f) { int64_t j = f / nx; g.act_v[f] = g.dist_v[f] > 1e-13 && j != 0 && j != ny; }
  for (int64_t f = 0; f < g.psize; ++f) g.act_p[f] = g.dist_p[f] > 1e-13;
  auto labels = [](const std::vector<uint8_t>& a, std::vector<int64_t>& ids, std::vector<int64_t>& lab) {
    ids.clear(); lab.assign(a.size(), -1);
    for (size_t f = 0; f < a.size(); ++f) if (a[f]) { lab[f] = (int64_t)ids.size(); ids.push_back((int64_t)f); }
  };
  labels(g.act_u, g.ui, g.lab_u);
  labels(g.act_v, g.vi, g.lab_v);
  labels(g.act_p, g.pi, g.lab_p);
  // ghost extension stencils (solver/optimized_ghost_cell.py:72-79)
  bool quad = g.velocity_interpolation == 1;
  if (!extension(g.xu, g.yu, g.xc, g.yc, g.R, g.dist_u, g.lab_u, false, quad, g.gu_rows, g.gu, g.ghost_of_u, g.error)) return false;
  if (!extension(g.xv, g.yv, g.xc, g.yc, g.R, g.dist_v, g.lab_v, false, quad, g.gv_rows, g.gv, g.ghost_of_v, g.error)) return false;
  if (g.pressure_extension == 1) {
    if (!quadratic_extension(g, g.gp_rows, g.gp, g.ghost_of_p, g.error)) return false;
  } else {
    if (!extension(g.xv, g.yu, g.xc, g.yc, g.R, g.dist_p, g.lab_p, true, false, g.gp_rows, g.gp, g.ghost_of_p, g.error)) return false;
  }
  // pressure operator rows and Schur rows
  make_rect(g.rect_p, 0, nx, ny, g.dx, g.dy, g.nu, 0.0, g.rho);
  g.a_nnz_row.assign(g.psize, 0);
  schur_setup(g, g.rect_p, 0, g.act_p, [&](int64_t f) { return pressure_row(g, f); }, g.a_rows, g.a_irr,
              g.schur_p_rows, g.schur_p_c, g.schur_p_tol, &g.a_nnz_row);
  if (g.schur_p_rows.size() > 2048) { g.error = "Ghost inverse exceeds the bounded boundary-row rank"; return false; }
  if (!surface_setup(g, g.error)) return false;
  err_class = 0;
  return true;
}

// cut-cell Poisson row of fluid cell c (solver/cut_cell_solver.py:166-214), unit density
// A coupling to a covered neighbour is left out: the covered cell's row is the identity with a
// zero right-hand side, so its value is zero and the coupling adds nothing, while the diagonal
// keeps the face's share as in the assembled matrix.
static Row cutcell_pressure_row(const Geometry& g, const double* ax, const double* ay, const int32_t* cell_type,
                               const double* kappa, int64_t c) {
  const int nx = g.nx, ny = g.ny;
  const int64_t j = c / nx, i = c % nx;
  const double idx2 = 1.0 / (g.dx * g.dx), idy2 = 1.0 / (g.dy * g.dy);
  Row r;
  double diag = 0.0;
  const double aw = ax[j * (nx + 1) + i], ae = ax[j * (nx + 1) + i + 1];
  const double as = ay[j * nx + i], an = ay[(j + 1) * nx + i];
  auto couple = [&](int64_t nb, double k) {
    if (g.act_p[nb]) r.emplace_back(nb, k);
    diag -= k;
  };
  if (i > 0 && aw > 0.0) couple(c - 1, aw * idx2);
  if (i == nx - 1) diag -= 2.0 * ae * idx2;
  else if (ae > 0.0) couple(c + 1, ae * idx2);
  if (j > 0 && as > 0.0) couple(c - nx, as * idy2);
  if (j < ny - 1 && an > 0.0) couple(c + nx, an * idy2);
  r.emplace_back(c, diag);
  if (cell_type[c] == 0)
    for (auto& e : r) e.second = e.second / kappa[c];
  return r;
}

bool build_cutcell_geometry(Geometry& g, const double* ax, const double* ay, const int32_t* cell_type,
                            const double* kappa, int& err_class) {
  err_class = 1;
  const int nx = g.nx, ny = g.ny;
  if (nx < 4 || ny < 4) { g.error = "nx and ny must be integers >= 4"; return false; }
  for (double v : {g.Lx, g.Ly, g.D, g.nu, g.rho, g.U_inf})
    if (!(std::isfinite(v) && v > 0)) { g.error = "Domain lengths, D, nu, rho and U_inf must be finite and positive"; return false; }
  if (g.inflow != 0 && g.inflow != 1) { g.error = "inflow must be uniform or parabolic"; return false; }
  g.dx = g.Lx / nx;
  g.dy = g.Ly / ny;
  if (g.inflow == 1) { g.U_m = g.U_m > 0 ? g.U_m : 1.5 * g.U_inf; g.U_ref = (2.0 / 3.0) * g.U_m; }
  else { g.U_m = g.U_inf; g.U_ref = g.U_inf; }
  g.R = g.D / 2.0;
  g.usize = (int64_t)ny * (nx + 1);
  g.vsize = (int64_t)(ny + 1) * nx;
  g.psize = (int64_t)ny * nx;
  g.u_inlet.assign(ny, 0.0);
  for (int j = 0; j < ny; ++j) {
    double y = (j + 0.5) * g.dy;
    g.u_inlet[j] = g.inflow == 1 ? (((4.0 * g.U_m) * y) * (g.Ly - y)) / (g.Ly * g.Ly) : g.U_inf;
  }
  g.xu.resize(nx + 1); g.yu.resize(ny); g.xv.resize(nx); g.yv.resize(ny + 1);
  for (int i = 0; i <= nx; ++i) g.xu[i] = i * g.dx;
  for (int j = 0; j < ny; ++j) g.yu[j] = (j + 0.5) * g.dy;
  for (int i = 0; i < nx; ++i) g.xv[i] = (i + 0.5) * g.dx;
  for (int j = 0; j <= ny; ++j) g.yv[j] = j * g.dy;
  g.mask.assign(g.psize, 0);
  g.act_u.assign(g.usize, 0); g.act_v.assign(g.vsize, 0); g.act_p.assign(g.psize, 0);
  for (int64_t f = 0; f < g.usize; ++f) g.act_u[f] = (f % (nx + 1)) != 0 && ax[f] > 0.0;
  for (int64_t f = 0; f < g.vsize; ++f) { int64_t j = f / nx; g.act_v[f] = j != 0 && j != ny && ay[f] > 0.0; }
  for (int64_t c = 0; c < g.psize; ++c) {
    g.act_p[c] = cell_type[c] != -1;
    g.mask[c] = cell_type[c] == -1;
    if (cell_type[c] == 0 && !(kappa[c] > 0.0)) { g.error = "cut cell without fluid volume"; return false; }
  }
  auto labels = [](const std::vector<uint8_t>& a, std::vector<int64_t>& ids, std::vector<int64_t>& lab) {
    ids.clear(); lab.assign(a.size(), -1);
    for (size_t f = 0; f < a.size(); ++f) if (a[f]) { lab[f] = (int64_t)ids.size(); ids.push_back((int64_t)f); }
  };
  labels(g.act_u, g.ui, g.lab_u);
  labels(g.act_v, g.vi, g.lab_v);
  labels(g.act_p, g.pi, g.lab_p);
  g.ghost_of_u.assign(g.usize, -1);
  g.ghost_of_v.assign(g.vsize, -1);
  g.ghost_of_p.assign(g.psize, -1);
  g.gu_rows.clear(); g.gv_rows.clear(); g.gp_rows.clear();
  g.gu = Csr(); g.gv = Csr(); g.gp = Csr();
  // unit density (g.rho = 1 from here on): the rectangle is the plain Laplacian and
  // A phi = rhs with rhs = (rho/dt) div, the caller's rho entering through the right-hand side
  g.rho = 1.0;
  make_rect(g.rect_p, 0, nx, ny, g.dx, g.dy, g.nu, 0.0, 1.0);
  g.a_nnz_row.assign(g.psize, 0);
  schur_setup(g, g.rect_p, 0, g.act_p, [&](int64_t c) { return cutcell_pressure_row(g, ax, ay, cell_type, kappa, c); }, g.a_rows,
              g.a_irr, g.schur_p_rows, g.schur_p_c, g.schur_p_tol, &g.a_nnz_row);
  if (g.schur_p_rows.size() > 2048) { g.error = "Cut-cell inverse exceeds the bounded boundary-row rank"; return false; }
  // surface quadrature points and point-pressure reconstruction (solver/cut_cell_solver.py:25-77)
  const double h_min = std::min(g.dx, g.dy);
  const int count = std::max(360, 4 * (int)std::ceil(2 * PI * g.R / h_min));
  g.n_surface = count;
  g.surf_y.resize(count); g.surf_x.resize(count);
  g.normal_wx.resize(count); g.normal_wy.resize(count); g.normal_x.resize(count); g.normal_y.resize(count);
  const double step = 2 * PI / count, wscale = 2 * PI * g.R / count;
  for (int k = 0; k < count; ++k) {
    const double th = k * step, c = std::cos(th), s = std::sin(th);
    g.surf_y[k] = g.yc + g.R * s;
    g.surf_x[k] = g.xc + g.R * c;
    g.normal_x[k] = c;
    g.normal_y[k] = s;
    g.normal_wx[k] = c * wscale;
    g.normal_wy[k] = s * wscale;
  }
  if (!pressure_reconstruction(g, g.surf_y, g.surf_x, g.surf_p, g.error)) return false;
  g.dudn = Csr(); g.dvdn = Csr();
  err_class = 0;
  return true;
}

bool build_helmholtz(const Geometry& g, double dt, HelmholtzSetup& hs, int& err_class, std::string& err) {
  err_class = 1;
  hs.dt = dt;
  for (int c = 0; c < 2; ++c) {
    make_rect(hs.rect[c], 1 + c, g.nx, g.ny, g.dx, g.dy, g.nu, dt, g.rho);
    const std::vector<uint8_t>& act = c == 0 ? g.act_u : g.act_v;
    schur_setup(g, hs.rect[c], 1 + c, act, [&](int64_t f) { return helmholtz_row(g, c, f, dt); }, hs.rows_irr[c],
                hs.irr[c], hs.schur_rows[c], hs.schur_c[c], hs.tol[c], nullptr);
    if (hs.schur_rows[c].size() > 2048) { err = "Ghost inverse exceeds the bounded boundary-row rank"; return false; }
  }
  err_class = 0;
  return true;
}

}  // namespace gm
