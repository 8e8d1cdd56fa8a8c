// The reference's native MAC kernels of its legacy staircase path, on the GPU.
//
// solver/src/bindings.cpp:47-390 (module mac_engine) holds four OpenMP loops that the
// reference's legacy immersed/staircase step calls (solver/main.py:303-381):
//   predictor_rhs_cpp          upwind or centred momentum predictor u*, v* with staircase wall
//                              reflections, and the Poisson right-hand side rho/dt div u*;
//   corrector_cpp              u = u* - dt/rho grad phi with the exact Dirichlet outlet;
//   calculate_mac_forces_cpp   staircase pressure and shear force sums over the solid cells;
//   calculate_mac_divergence_cpp  fluid-cell divergence statistics.
// Here each is one or two grid-parallel kernels; gm_mac_ab2_rhs adds the loop's own AB2 step on
// u*, v* and its recomputed Poisson right-hand side (solver/main.py:315-339).  The per-point arithmetic is written in the
// reference's order and this file is compiled without FMA contraction, so u*, v*, rhs, u and v
// are bit-identical to the reference's compiled code; the force and divergence sums are
// reduced per block and then over blocks in a fixed order (deterministic, and equal to the
// sequential sums up to reassociation).
//
// Arrays may be host or device memory: host arrays are staged through a per-thread device
// buffer (grown on demand) on the caller's stream, and every call returns after its results
// are in the caller's arrays.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/ghostmac.h"
#include "internal.hpp"

namespace gmk {
void kernel_launch_adjust(long long delta);  // the library's launch counter (kernels.cu)
}
void gm_internal_set_error(const char* msg);  // defined in ghostmac.cu

namespace {

constexpr int LT = 256;

#define P_(j, i) p[(size_t)(j) * nx + (i)]
#define M_(j, i) mask[(size_t)(j) * nx + (i)]
#define U_(j, i) u[(size_t)(j) * (nx + 1) + (i)]
#define V_(j, i) v[(size_t)(j) * nx + (i)]
#define US_(j, i) us[(size_t)(j) * (nx + 1) + (i)]
#define VS_(j, i) vs[(size_t)(j) * nx + (i)]
#define PHI_(j, i) phi[(size_t)(j) * nx + (i)]

// u* on every vertical face (bindings.cpp:98-139): interior faces by the predictor, the inlet
// column from the inlet profile, the outlet column from the previous u
__global__ void k_predict_u(const double* __restrict__ u, const double* __restrict__ v, double* __restrict__ us,
                            const double* __restrict__ p, const uint8_t* __restrict__ mask,
                            const double* __restrict__ inlet, int nx, int ny, double dx, double dy, double dx2,
                            double dy2, double dt, double nu, double rho, int slip, int centered) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ny * (nx + 1)) return;
  const int j = (int)(t / (nx + 1)), i = (int)(t - (long long)j * (nx + 1));
  if (i == 0) { US_(j, 0) = inlet[j]; return; }
  if (i == nx) { US_(j, nx) = U_(j, nx - 1); return; }
  if (M_(j, i - 1) || M_(j, i)) { US_(j, i) = 0.0; return; }
  const double uc = U_(j, i);
  const double vavg = 0.25 * (V_(j, i - 1) + V_(j, i) + V_(j + 1, i - 1) + V_(j + 1, i));
  double ub, ut;
  if (j == 0) ub = slip ? uc : -uc;
  else ub = (M_(j - 1, i - 1) && M_(j - 1, i)) ? -uc : U_(j - 1, i);
  if (j == ny - 1) ut = slip ? uc : -uc;
  else ut = (M_(j + 1, i - 1) && M_(j + 1, i)) ? -uc : U_(j + 1, i);
  const double lap = (U_(j, i + 1) - 2.0 * uc + U_(j, i - 1)) / dx2 + (ut - 2.0 * uc + ub) / dy2;
  const double dpdx = (P_(j, i) - P_(j, i - 1)) / dx;
  double conv;
  if (centered) {
    const double e = .5 * (uc + U_(j, i + 1)), w = .5 * (uc + U_(j, i - 1));
    conv = (e * e - w * w) / dx +
           .25 * ((uc + ut) * (V_(j + 1, i - 1) + V_(j + 1, i)) - (uc + ub) * (V_(j, i - 1) + V_(j, i))) / dy;
  } else {
    const double dudx = (uc > 0.0) ? (uc - U_(j, i - 1)) / dx : (U_(j, i + 1) - uc) / dx;
    const double dudy = (vavg > 0.0) ? (uc - ub) / dy : (ut - uc) / dy;
    conv = uc * dudx + vavg * dudy;
  }
  US_(j, i) = uc + dt * (-conv + nu * lap - dpdx / rho);
}

// v* on every horizontal face (bindings.cpp:142-193): walls zero
__global__ void k_predict_v(const double* __restrict__ u, const double* __restrict__ v, double* __restrict__ vs,
                            const double* __restrict__ p, const uint8_t* __restrict__ mask, int nx, int ny,
                            double dx, double dy, double dx2, double dy2, double dt, double nu, double rho,
                            int centered) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)(ny + 1) * nx) return;
  const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
  if (j == 0 || j == ny) { VS_(j, i) = 0.0; return; }
  if (M_(j - 1, i) || M_(j, i)) { VS_(j, i) = 0.0; return; }
  const double vc = V_(j, i);
  const double uavg = 0.25 * (U_(j - 1, i) + U_(j, i) + U_(j - 1, i + 1) + U_(j, i + 1));
  double vl, vr;
  if (i == 0) vl = -vc;
  else vl = (M_(j - 1, i - 1) && M_(j, i - 1)) ? -vc : V_(j, i - 1);
  if (i == nx - 1) vr = vc;
  else vr = (M_(j - 1, i + 1) && M_(j, i + 1)) ? -vc : V_(j, i + 1);
  const double lap = (vr - 2.0 * vc + vl) / dx2 + (V_(j + 1, i) - 2.0 * vc + V_(j - 1, i)) / dy2;
  const double dpdy = (P_(j, i) - P_(j - 1, i)) / dy;
  double conv;
  if (centered) {
    const double n = .5 * (vc + V_(j + 1, i)), s = .5 * (vc + V_(j - 1, i));
    conv = (n * n - s * s) / dy +
           .25 * ((vc + vr) * (U_(j - 1, i + 1) + U_(j, i + 1)) - (vc + vl) * (U_(j - 1, i) + U_(j, i))) / dx;
  } else {
    const double dvdx = (uavg > 0.0) ? (vc - vl) / dx : (vr - vc) / dx;
    const double dvdy = (vc > 0.0) ? (vc - V_(j - 1, i)) / dy : (V_(j + 1, i) - vc) / dy;
    conv = uavg * dvdx + vc * dvdy;
  }
  VS_(j, i) = vc + dt * (-conv + nu * lap - dpdy / rho);
}

// Poisson right-hand side rho/dt div u* on the fluid cells (bindings.cpp:201-215)
__global__ void k_poisson_rhs(const double* __restrict__ us, const double* __restrict__ vs,
                              const uint8_t* __restrict__ mask, double* __restrict__ rhs, int nx, int ny, double dx,
                              double dy, double inv_dt) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ny * nx) return;
  const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
  if (M_(j, i)) { rhs[t] = 0.0; return; }
  const double div = (US_(j, i + 1) - US_(j, i)) / dx + (VS_(j + 1, i) - VS_(j, i)) / dy;
  rhs[t] = inv_dt * div;
}

// The legacy loop's AB2 step on the interior faces (solver/main.py:315-322): d = (u* - u) / dt,
// u* += dt alpha (d - d_prev) when a previous step exists, d_prev = d
__global__ void k_ab2(const double* __restrict__ u, const double* __restrict__ v, double* __restrict__ us,
                      double* __restrict__ vs, double* __restrict__ pdu, double* __restrict__ pdv, int nx, int ny,
                      double dt, double dt_alpha, int has_prev) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nu_ = (long long)ny * (nx + 1), nv_ = (long long)(ny + 1) * nx;
  if (t < nu_) {
    const int i = (int)(t % (nx + 1));
    if (i < 1 || i > nx - 1) return;
    const double d = (us[t] - u[t]) / dt;
    if (has_prev) us[t] = us[t] + dt_alpha * (d - pdu[t]);
    pdu[t] = d;
  } else if (t < nu_ + nv_) {
    const long long f = t - nu_;
    const int j = (int)(f / nx);
    if (j < 1 || j > ny - 1) return;
    const double d = (vs[f] - v[f]) / dt;
    if (has_prev) vs[f] = vs[f] + dt_alpha * (d - pdv[f]);
    pdv[f] = d;
  }
}

// the recomputed Poisson right-hand side of the legacy loop (solver/main.py:337-339):
// rho/dt ((u*_e - u*_w)/dx + (v*_n - v*_s)/dy), zero on masked cells
__global__ void k_legacy_rhs(const double* __restrict__ us, const double* __restrict__ vs,
                             const uint8_t* __restrict__ mask, double* __restrict__ rhs, int nx, int ny, double dx,
                             double dy, double rho_dt) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ny * nx) return;
  const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
  if (M_(j, i)) { rhs[t] = 0.0; return; }
  rhs[t] = rho_dt * ((US_(j, i + 1) - US_(j, i)) / dx + (VS_(j + 1, i) - VS_(j, i)) / dy);
}

// ---- the legacy loop's ghost-cell branch (solver/ghost_cell.py:32-234, solver/main.py:347-370) --
// Image-point ghost velocities g = wall - gamma (ip - wall), ip the bilinear value at the image
// point.  The reference sets the ghost faces one after another, so a face may read a ghost face
// set earlier in the same pass (its new value) or a later one (its old value): the host orders
// the faces into levels (a face is one level above every earlier ghost face it reads), the old
// values are saved first, and each level is one launch.
__global__ void k_ghost_save(const double* __restrict__ f, long long nf, const long long* __restrict__ target,
                             long long n, double* __restrict__ snap) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) {
    const long long t = target[g];
    snap[g] = (t >= 0 && t < nf) ? f[t] : 0.0;
  }
}
// one level of ghost faces; entries whose indexes fall outside the field or the table are skipped
__global__ void k_ghost_level(double* __restrict__ f, long long nf, const long long* __restrict__ target,
                              const long long* __restrict__ src, const int* __restrict__ snap_of,
                              const double* __restrict__ w, const double* __restrict__ gamma,
                              const int* __restrict__ level, long long n, int lvl, const double* __restrict__ snap,
                              double wall) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n || level[g] != lvl) return;
  const long long t = target[g];
  if (t < 0 || t >= nf) return;
  double v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int sidx = snap_of[4 * g + q];
    const long long c = src[4 * g + q];
    if (sidx >= n || c < 0 || c >= nf) return;
    v[q] = sidx >= 0 ? snap[sidx] : f[c];
  }
  // the reference's order: w00 f00 + w10 f10 + w01 f01 + w11 f11, then the reflection
  const double ip = w[4 * g] * v[0] + w[4 * g + 1] * v[1] + w[4 * g + 2] * v[2] + w[4 * g + 3] * v[3];
  f[t] = wall - gamma[g] * (ip - wall);
}

// the ghost branch's corrector (solver/main.py:347-366): u = u* on interior faces, minus
// dt/rho grad phi on faces between two fluid cells, zero between two masked cells, the inlet
// and the Dirichlet outlet; v likewise with zero wall rows
__global__ void k_ghost_correct(double* __restrict__ u, double* __restrict__ v, const double* __restrict__ us,
                                const double* __restrict__ vs, const double* __restrict__ phi,
                                const uint8_t* __restrict__ mask, const double* __restrict__ inlet, int nx, int ny,
                                double dx, double dy, double dt_over_rho) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nu_ = (long long)ny * (nx + 1);
  if (t < nu_) {
    const int j = (int)(t / (nx + 1)), i = (int)(t - (long long)j * (nx + 1));
    if (i == 0) U_(j, 0) = inlet[j];
    else if (i == nx) U_(j, nx) = US_(j, nx) + dt_over_rho * 2.0 * PHI_(j, nx - 1) / dx;
    else {
      const bool l = M_(j, i - 1), r = M_(j, i);
      double val = US_(j, i);
      if (!l && !r) val -= dt_over_rho * (PHI_(j, i) - PHI_(j, i - 1)) / dx;
      else if (l && r) val = 0.0;
      U_(j, i) = val;
    }
  } else if (t < nu_ + (long long)(ny + 1) * nx) {
    const long long f = t - nu_;
    const int j = (int)(f / nx), i = (int)(f - (long long)j * nx);
    if (j == 0 || j == ny) { V_(j, i) = 0.0; return; }
    const bool b = M_(j - 1, i), a = M_(j, i);
    double val = VS_(j, i);
    if (!a && !b) val -= dt_over_rho * (PHI_(j, i) - PHI_(j - 1, i)) / dy;
    else if (a && b) val = 0.0;
    V_(j, i) = val;
  }
}
// faces between a fluid and a masked cell keep u* (solver/main.py:368-370)
__global__ void k_ghost_boundary(double* __restrict__ u, double* __restrict__ v, const double* __restrict__ us,
                                 const double* __restrict__ vs, const uint8_t* __restrict__ mask, int nx, int ny) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nu_ = (long long)ny * (nx + 1);
  if (t < nu_) {
    const int j = (int)(t / (nx + 1)), i = (int)(t - (long long)j * (nx + 1));
    if (i >= 1 && i <= nx - 1 && M_(j, i - 1) != M_(j, i)) U_(j, i) = US_(j, i);
  } else if (t < nu_ + (long long)(ny + 1) * nx) {
    const long long f = t - nu_;
    const int j = (int)(f / nx), i = (int)(f - (long long)j * nx);
    if (j >= 1 && j <= ny - 1 && M_(j - 1, i) != M_(j, i)) V_(j, i) = VS_(j, i);
  }
}

// bilinear value of a staggered field at (y, x): the linear RegularGridInterpolator of the
// reference (solver/ghost_cell.py:199-201), zero outside the grid
__device__ double grid_linear(const double* __restrict__ f, int nxf, int nyf, double x0, double y0, double hx,
                              double hy, double y, double x) {
  const double gx = (x - x0) / hx, gy = (y - y0) / hy;
  if (!(gx >= 0.0 && gx <= nxf - 1 && gy >= 0.0 && gy <= nyf - 1)) return 0.0;
  int i = (int)floor(gx), j = (int)floor(gy);
  if (i > nxf - 2) i = nxf - 2;
  if (j > nyf - 2) j = nyf - 2;
  const double tx = (x - (x0 + i * hx)) / hx, ty = (y - (y0 + j * hy)) / hy;
  const double* r0 = f + (size_t)j * nxf;
  const double* r1 = r0 + nxf;
  return (r0[i] * (1.0 - tx) + r0[i + 1] * tx) * (1.0 - ty) + (r1[i] * (1.0 - tx) + r1[i + 1] * tx) * ty;
}

// surface forces on the true circle (extract_true_surface_forces, solver/ghost_cell.py:186-234):
// pressure and probed central-difference velocity gradients at n points; one block, sums in a
// fixed order; out = fx_p, fy_p, fx_v, fy_v
__global__ void k_ghost_forces(const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ p,
                               int nx, int ny, double dx, double dy, double xc, double yc, double radius, int n,
                               double mu, double* __restrict__ out) {
  __shared__ double sh[4][256];
  double ax = 0.0, ay = 0.0, bx = 0.0, by = 0.0;
  const double eps = 1e-4 * dx;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double th = k * (2 * M_PI / n);  // np.linspace(0, 2 pi, n, endpoint=False)
    const double c = cos(th), s = sin(th);
    const double x = xc + radius * c, y = yc + radius * s;
    const double pk = grid_linear(p, nx, ny, 0.5 * dx, 0.5 * dy, dx, dy, y, x);
    auto U = [&](double yy, double xx) { return grid_linear(u, nx + 1, ny, 0.0, 0.5 * dy, dx, dy, yy, xx); };
    auto V = [&](double yy, double xx) { return grid_linear(v, nx, ny + 1, 0.5 * dx, 0.0, dx, dy, yy, xx); };
    const double dudx = (U(y, x + eps) - U(y, x - eps)) / (2.0 * eps);
    const double dudy = (U(y + eps, x) - U(y - eps, x)) / (2.0 * eps);
    const double dvdx = (V(y, x + eps) - V(y, x - eps)) / (2.0 * eps);
    const double dvdy = (V(y + eps, x) - V(y - eps, x)) / (2.0 * eps);
    const double txx = 2.0 * mu * dudx, tyy = 2.0 * mu * dvdy, txy = mu * (dudy + dvdx);
    ax += pk * c;
    ay += pk * s;
    bx += txx * c + txy * s;
    by += txy * c + tyy * s;
  }
  sh[0][threadIdx.x] = ax; sh[1][threadIdx.x] = ay; sh[2][threadIdx.x] = bx; sh[3][threadIdx.x] = by;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ds = radius * (2 * M_PI / n);
    out[0] = -sh[0][0] * ds;
    out[1] = -sh[1][0] * ds;
    out[2] = sh[2][0] * ds;
    out[3] = sh[3][0] * ds;
  }
}

// u = u* - dt/rho d phi/dx, v = v* - dt/rho d phi/dy (bindings.cpp:248-281)
__global__ void k_correct(double* __restrict__ u, double* __restrict__ v, const double* __restrict__ us,
                          const double* __restrict__ vs, const double* __restrict__ phi,
                          const uint8_t* __restrict__ mask, const double* __restrict__ inlet, int nx, int ny,
                          double dx, double dy, double dt_over_rho) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nu_ = (long long)ny * (nx + 1);
  if (t < nu_) {
    const int j = (int)(t / (nx + 1)), i = (int)(t - (long long)j * (nx + 1));
    if (i == 0) U_(j, 0) = inlet[j];
    else if (i == nx) U_(j, nx) = US_(j, nx) + dt_over_rho * 2.0 * PHI_(j, nx - 1) / dx;
    else if (M_(j, i - 1) || M_(j, i)) U_(j, i) = 0.0;
    else U_(j, i) = US_(j, i) - dt_over_rho * (PHI_(j, i) - PHI_(j, i - 1)) / dx;
    return;
  }
  const long long r = t - nu_;
  if (r >= (long long)(ny + 1) * nx) return;
  const int j = (int)(r / nx), i = (int)(r - (long long)j * nx);
  if (j == 0 || j == ny) V_(j, i) = 0.0;
  else if (M_(j - 1, i) || M_(j, i)) V_(j, i) = 0.0;
  else V_(j, i) = VS_(j, i) - dt_over_rho * (PHI_(j, i) - PHI_(j - 1, i)) / dy;
}

template <int NF>
__device__ void block_sum(double (&val)[NF], double* __restrict__ out /* NF per block */) {
  __shared__ double sm[NF][LT];
#pragma unroll
  for (int f = 0; f < NF; ++f) sm[f][threadIdx.x] = val[f];
  __syncthreads();
  for (int s = LT / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
#pragma unroll
      for (int f = 0; f < NF; ++f) sm[f][threadIdx.x] += sm[f][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int f = 0; f < NF; ++f) out[(size_t)blockIdx.x * NF + f] = sm[f][0];
}

// staircase traction of every solid cell's fluid-facing sides (bindings.cpp:310-338)
__global__ void k_forces_part(const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ p, const uint8_t* __restrict__ mask, int nx, int ny,
                              double dx, double dy, double mu, double* __restrict__ part) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double f[4] = {0.0, 0.0, 0.0, 0.0};  // fx_p, fy_p, fx_v, fy_v
  if (t < (long long)ny * nx) {
    const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
    if (M_(j, i)) {
      if (i > 0 && !M_(j, i - 1)) {
        f[0] += P_(j, i - 1) * dy;
        const double vf = 0.5 * (V_(j, i - 1) + V_(j + 1, i - 1));
        f[3] += mu * (vf / (0.5 * dx)) * dy;
      }
      if (i < nx - 1 && !M_(j, i + 1)) {
        f[0] -= P_(j, i + 1) * dy;
        const double vf = 0.5 * (V_(j, i + 1) + V_(j + 1, i + 1));
        f[3] += mu * (vf / (0.5 * dx)) * dy;
      }
      if (j > 0 && !M_(j - 1, i)) {
        f[1] += P_(j - 1, i) * dx;
        const double uf = 0.5 * (U_(j - 1, i) + U_(j - 1, i + 1));
        f[2] += mu * (uf / (0.5 * dy)) * dx;
      }
      if (j < ny - 1 && !M_(j + 1, i)) {
        f[1] -= P_(j + 1, i) * dx;
        const double uf = 0.5 * (U_(j + 1, i) + U_(j + 1, i + 1));
        f[2] += mu * (uf / (0.5 * dy)) * dx;
      }
    }
  }
  block_sum<4>(f, part);
}

// divergence of every fluid cell: max |div|, sum div^2, count, core sum, core count
// (bindings.cpp:343-390)
__global__ void k_div_part(const double* __restrict__ u, const double* __restrict__ v,
                           const uint8_t* __restrict__ mask, int nx, int ny, double dx, double dy,
                           double* __restrict__ part) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s[4] = {0.0, 0.0, 0.0, 0.0};  // sum div^2, count, core sum, core count
  double mx = 0.0;
  if (t < (long long)ny * nx) {
    const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
    if (!M_(j, i)) {
      const double d = (U_(j, i + 1) - U_(j, i)) / dx + (V_(j + 1, i) - V_(j, i)) / dy;
      mx = fabs(d);
      s[0] = d * d;
      s[1] = 1.0;
      const bool core = !((i > 0 && M_(j, i - 1)) || (i < nx - 1 && M_(j, i + 1)) || (j > 0 && M_(j - 1, i)) ||
                          (j < ny - 1 && M_(j + 1, i)));
      if (core) {
        s[2] = d * d;
        s[3] = 1.0;
      }
    }
  }
  __shared__ double smx[LT];
  smx[threadIdx.x] = mx;
  __syncthreads();
  for (int k = LT / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) smx[threadIdx.x] = fmax(smx[threadIdx.x], smx[threadIdx.x + k]);
    __syncthreads();
  }
  double* out = part + (size_t)gridDim.x * 4;  // maxima after the sums
  if (threadIdx.x == 0) out[blockIdx.x] = smx[0];
  block_sum<4>(s, part);
}

// per-field sums of the block partials (one block of LT threads: thread t adds the partials of
// blocks t, t + LT, ... in order, then a tree in a fixed order; the same sums every run); the
// maximum of the divergence after them when nmax is set
__global__ void k_fold(const double* __restrict__ part, int nblocks, int nf, int nmax, double* __restrict__ out) {
  __shared__ double sh[LT];
  const int nout = nf + (nmax ? 1 : 0);
  for (int f = 0; f < nout; ++f) {
    const bool is_max = f == nf;
    double a = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const double v = is_max ? part[(size_t)nblocks * nf + b] : part[(size_t)b * nf + f];
      a = is_max ? fmax(a, v) : a + v;
    }
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
      if ((int)threadIdx.x < k)
        sh[threadIdx.x] = is_max ? fmax(sh[threadIdx.x], sh[threadIdx.x + k]) : sh[threadIdx.x] + sh[threadIdx.x + k];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[f] = sh[0];
    __syncthreads();
  }
}


int fail(int code, const char* msg) {
  gm_internal_set_error(msg);
  return code;
}

bool is_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

// Device views of the call's arrays: device arrays pass through; host arrays get a slice of a
// per-thread device buffer, copied in (inputs) before and out (outputs) after the kernels.
struct Staging {
  struct Arena {
    void* p = nullptr;
    size_t cap = 0;
    int dev = -1;
  };
  static Arena& arena() {
    static thread_local Arena a;
    return a;
  }
  struct Item {
    const void* host;
    void* dev;
    size_t bytes;
    bool in, out;
  };
  std::vector<Item> items;
  size_t total = 0;
  cudaStream_t st;
  explicit Staging(cudaStream_t s) : st(s) {}
  // registers an array; returns its index
  int add(const void* p, size_t bytes, bool in, bool out) {
    if (is_device(p)) {
      items.push_back({p, const_cast<void*>(p), bytes, false, false});
    } else {
      items.push_back({p, nullptr, bytes, in, out});
      total += (bytes + 255) & ~(size_t)255;
    }
    return (int)items.size() - 1;
  }
  cudaError_t begin(size_t extra_bytes, double** extra) {
    Arena& a = arena();
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t need = total + ((extra_bytes + 255) & ~(size_t)255);
    if (a.dev != dev || a.cap < need) {
      if (a.p && a.dev == dev) cudaFree(a.p);
      a.p = nullptr;
      a.cap = 0;
      cudaError_t e = cudaMalloc(&a.p, need);
      if (e != cudaSuccess) return e;
      a.cap = need;
      a.dev = dev;
    }
    size_t off = 0;
    char* base = static_cast<char*>(a.p);
    for (auto& it : items) {
      if (it.dev) continue;
      it.dev = base + off;
      off += (it.bytes + 255) & ~(size_t)255;
      if (it.in) {
        cudaError_t e = cudaMemcpyAsync(it.dev, it.host, it.bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
      }
    }
    *extra = reinterpret_cast<double*>(base + off);
    return cudaSuccess;
  }
  cudaError_t finish() {
    for (auto& it : items)
      if (it.out && it.host != it.dev) {
        cudaError_t e = cudaMemcpyAsync(const_cast<void*>(it.host), it.dev, it.bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
      }
    return cudaStreamSynchronize(st);
  }
  template <typename T>
  T* dev(int k) const { return static_cast<T*>(items[k].dev); }
};

int check_grid(int nx, int ny, double dx, double dy) {
  if (nx < 2 || ny < 2) return fail(GM_EVALUE, "mask must be a 2D grid with at least 2 cells per direction");
  if (!(std::isfinite(dx) && dx > 0 && std::isfinite(dy) && dy > 0))
    return fail(GM_EVALUE, "dx and dy must be finite and positive");
  return GM_OK;
}
int check_step(double dt, double rho) {
  if (!(std::isfinite(dt) && dt > 0 && std::isfinite(rho) && rho > 0))
    return fail(GM_EVALUE, "dt and rho must be finite and positive");
  return GM_OK;
}
int cuda_fail(cudaError_t e) {
  cudaGetLastError();
  return fail(GM_ECUDA, cudaGetErrorString(e));
}
unsigned blocks(long long n) { return (unsigned)((n + LT - 1) / LT); }

// p = phi (c = 0) or p += phi (c = 1)
__global__ void k_pupdate(double* __restrict__ p, const double* __restrict__ phi, long long n, int add) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = add ? p[t] + phi[t] : phi[t];
}

void ghost_pass(const gm_legacy_state& s, int k, double* field, double* snap, cudaStream_t st) {
  const long long n = s.n_ghost[k];
  if (n <= 0) return;
  const long long nf = k == 0 ? (long long)s.ny * (s.nx + 1) : (long long)(s.ny + 1) * s.nx;
  const long long* tg = reinterpret_cast<const long long*>(s.target[k]);
  k_ghost_save<<<blocks(n), LT, 0, st>>>(field, nf, tg, n, snap);
  for (int l = 0; l < s.n_levels[k]; ++l)
    k_ghost_level<<<blocks(n), LT, 0, st>>>(field, nf, tg, reinterpret_cast<const long long*>(s.src[k]), s.snap_of[k],
                                            s.weights[k], s.gamma[k], s.level[k], n, l, snap, 0.0);
  gmk::kernel_launch_adjust(1 + s.n_levels[k]);
}

}  // namespace

namespace gml {

size_t scratch_doubles(const gm_legacy_state& s) {
  const long long nP = (long long)s.ny * s.nx;
  const long long ng = std::max<long long>(s.ghost ? std::max(s.n_ghost[0], s.n_ghost[1]) : 0, 1);
  return (size_t)(ng + (long long)blocks(nP) * 4 + 16);
}

void predict(const gm_legacy_state& s, double dt, double* scratch, cudaStream_t st) {
  const int nx = s.nx, ny = s.ny;
  const long long nU = (long long)ny * (nx + 1), nV = (long long)(ny + 1) * nx, nP = (long long)ny * nx;
  const double* pin = s.centered ? s.zero_p : s.p;
  k_predict_u<<<blocks(nU), LT, 0, st>>>(s.u, s.v, s.u_star, pin, s.mask, s.inlet, nx, ny, s.dx, s.dy, s.dx * s.dx,
                                         s.dy * s.dy, dt, s.nu, s.rho, s.slip_walls ? 1 : 0, s.centered ? 1 : 0);
  k_predict_v<<<blocks(nV), LT, 0, st>>>(s.u, s.v, s.v_star, pin, s.mask, nx, ny, s.dx, s.dy, s.dx * s.dx,
                                         s.dy * s.dy, dt, s.nu, s.rho, s.centered ? 1 : 0);
  gmk::kernel_launch_adjust(2);
  if (s.ghost) {
    ghost_pass(s, 0, s.u_star, scratch, st);
    ghost_pass(s, 1, s.v_star, scratch, st);
  }
  if (s.centered) {
    const bool hp = s.has_prev != 0;
    k_ab2<<<blocks(nU + nV), LT, 0, st>>>(s.u, s.v, s.u_star, s.v_star, s.prev_du, s.prev_dv, nx, ny, dt,
                                          hp ? dt * (dt / (2 * s.prev_dt)) : 0.0, hp ? 1 : 0);
    gmk::kernel_launch_adjust(1);
    if (s.ghost) {
      ghost_pass(s, 0, s.u_star, scratch, st);
      ghost_pass(s, 1, s.v_star, scratch, st);
    }
  }
  k_legacy_rhs<<<blocks(nP), LT, 0, st>>>(s.u_star, s.v_star, s.mask, s.rhs, nx, ny, s.dx, s.dy, s.rho / dt);
  gmk::kernel_launch_adjust(1);
}

void correct(const gm_legacy_state& s, double dt, double* scratch, cudaStream_t st) {
  const int nx = s.nx, ny = s.ny;
  const long long n = (long long)ny * (nx + 1) + (long long)(ny + 1) * nx, nP = (long long)ny * nx;
  if (s.ghost) {
    k_ghost_correct<<<blocks(n), LT, 0, st>>>(s.u, s.v, s.u_star, s.v_star, s.phi, s.mask, s.inlet, nx, ny, s.dx,
                                              s.dy, dt / s.rho);
    gmk::kernel_launch_adjust(1);
    ghost_pass(s, 0, s.u, scratch, st);
    ghost_pass(s, 1, s.v, scratch, st);
    k_ghost_boundary<<<blocks(n), LT, 0, st>>>(s.u, s.v, s.u_star, s.v_star, s.mask, nx, ny);
  } else {
    k_correct<<<blocks(n), LT, 0, st>>>(s.u, s.v, s.u_star, s.v_star, s.phi, s.mask, s.inlet, nx, ny, s.dx, s.dy,
                                        dt / s.rho);
  }
  k_pupdate<<<blocks(nP), LT, 0, st>>>(s.p, s.phi, nP, s.centered ? 0 : 1);
  gmk::kernel_launch_adjust(2);
}

void forces(const gm_legacy_state& s, double* scratch, double* out, cudaStream_t st) {
  const int nx = s.nx, ny = s.ny;
  const double mu = s.nu * s.rho;
  if (s.ghost) {
    k_ghost_forces<<<1, 256, 0, st>>>(s.u, s.v, s.p, nx, ny, s.dx, s.dy, s.xc, s.yc, s.radius, s.n_theta, mu, out);
    gmk::kernel_launch_adjust(1);
    return;
  }
  const unsigned nb = blocks((long long)ny * nx);
  double* part = scratch + std::max<long long>(s.ghost ? std::max(s.n_ghost[0], s.n_ghost[1]) : 0, 1);
  k_forces_part<<<nb, LT, 0, st>>>(s.u, s.v, s.p, s.mask, nx, ny, s.dx, s.dy, mu, part);
  k_fold<<<1, LT, 0, st>>>(part, (int)nb, 4, 0, out);
  gmk::kernel_launch_adjust(2);
}

}  // namespace gml

extern "C" {

int gm_mac_predictor_rhs(const double* u, const double* v, double* u_star, double* v_star, double* rhs,
                         const double* p, const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx,
                         double dy, double dt, double nu, double rho, int32_t slip_walls, int32_t centered,
                         void* stream) {
  if (!u || !v || !u_star || !v_star || !rhs || !p || !mask || !inlet) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (int rc = check_step(dt, rho)) return rc;
  if (!(std::isfinite(nu) && nu >= 0)) return fail(GM_EVALUE, "nu must be finite and nonnegative");
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, false), iv = sg.add(v, nV * 8, true, false);
  const int ius = sg.add(u_star, nU * 8, false, true), ivs = sg.add(v_star, nV * 8, false, true);
  const int ir = sg.add(rhs, nP * 8, false, true), ip = sg.add(p, nP * 8, true, false);
  const int im = sg.add(mask, nP, true, false), ii = sg.add(inlet, (size_t)ny * 8, true, false);
  double* extra = nullptr;
  if (cudaError_t e = sg.begin(0, &extra)) return cuda_fail(e);
  cudaStream_t st = sg.st;
  k_predict_u<<<blocks((long long)nU), LT, 0, st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ius),
                                                    sg.dev<double>(ip), sg.dev<uint8_t>(im), sg.dev<double>(ii), nx,
                                                    ny, dx, dy, dx * dx, dy * dy, dt, nu, rho, slip_walls ? 1 : 0,
                                                    centered ? 1 : 0);
  k_predict_v<<<blocks((long long)nV), LT, 0, st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ivs),
                                                    sg.dev<double>(ip), sg.dev<uint8_t>(im), nx, ny, dx, dy, dx * dx,
                                                    dy * dy, dt, nu, rho, centered ? 1 : 0);
  k_poisson_rhs<<<blocks((long long)nP), LT, 0, st>>>(sg.dev<double>(ius), sg.dev<double>(ivs), sg.dev<uint8_t>(im),
                                                      sg.dev<double>(ir), nx, ny, dx, dy, rho / dt);
  gmk::kernel_launch_adjust(3);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_corrector(double* u, double* v, const double* u_star, const double* v_star, const double* phi,
                     const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx, double dy, double dt,
                     double rho, int32_t slip_walls, void* stream) {
  (void)slip_walls;  // accepted for the reference's signature; the walls are no-slip v = 0 either way
  if (!u || !v || !u_star || !v_star || !phi || !mask || !inlet) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (int rc = check_step(dt, rho)) return rc;
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, false, true), iv = sg.add(v, nV * 8, false, true);
  const int ius = sg.add(u_star, nU * 8, true, false), ivs = sg.add(v_star, nV * 8, true, false);
  const int iph = sg.add(phi, nP * 8, true, false), im = sg.add(mask, nP, true, false);
  const int ii = sg.add(inlet, (size_t)ny * 8, true, false);
  double* extra = nullptr;
  if (cudaError_t e = sg.begin(0, &extra)) return cuda_fail(e);
  k_correct<<<blocks((long long)(nU + nV)), LT, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv),
                                                              sg.dev<double>(ius), sg.dev<double>(ivs),
                                                              sg.dev<double>(iph), sg.dev<uint8_t>(im),
                                                              sg.dev<double>(ii), nx, ny, dx, dy, dt / rho);
  gmk::kernel_launch_adjust(1);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_ab2_rhs(const double* u, const double* v, double* u_star, double* v_star, double* prev_du,
                   double* prev_dv, double* rhs, const uint8_t* mask, int32_t nx, int32_t ny, double dx, double dy,
                   double dt, double rho, double alpha, int32_t has_prev, int32_t what, void* stream) {
  if (!u || !v || !u_star || !v_star || !prev_du || !prev_dv || !rhs || !mask) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (int rc = check_step(dt, rho)) return rc;
  if (has_prev && !std::isfinite(alpha)) return fail(GM_EVALUE, "alpha must be finite");
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, false), iv = sg.add(v, nV * 8, true, false);
  const int ius = sg.add(u_star, nU * 8, true, true), ivs = sg.add(v_star, nV * 8, true, true);
  const int idu = sg.add(prev_du, nU * 8, true, true), idv = sg.add(prev_dv, nV * 8, true, true);
  const int ir = sg.add(rhs, nP * 8, true, true), im = sg.add(mask, nP, true, false);
  double* extra = nullptr;
  if (cudaError_t e = sg.begin(0, &extra)) return cuda_fail(e);
  cudaStream_t st = sg.st;
  if (what & 1) {
    k_ab2<<<blocks((long long)(nU + nV)), LT, 0, st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ius),
                                                       sg.dev<double>(ivs), sg.dev<double>(idu), sg.dev<double>(idv),
                                                       nx, ny, dt, dt * alpha, has_prev ? 1 : 0);
    gmk::kernel_launch_adjust(1);
  }
  if (what & 2) {
    k_legacy_rhs<<<blocks((long long)nP), LT, 0, st>>>(sg.dev<double>(ius), sg.dev<double>(ivs),
                                                       sg.dev<uint8_t>(im), sg.dev<double>(ir), nx, ny, dx, dy,
                                                       rho / dt);
    gmk::kernel_launch_adjust(1);
  }
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_ghost_apply(double* field, int64_t field_size, int64_t n_ghost, const int64_t* target, const int64_t* src,
                       const int32_t* snap_of, const double* weights, const double* gamma, const int32_t* level,
                       int32_t n_levels, double wall, void* stream) {
  if (n_ghost < 0 || field_size <= 0 || n_levels < 0) return fail(GM_EVALUE, "invalid ghost table sizes");
  if (n_ghost == 0) return GM_OK;
  if (!field || !target || !src || !snap_of || !weights || !gamma || !level) return fail(GM_EVALUE, "null argument");
  if (!std::isfinite(wall)) return fail(GM_EVALUE, "the wall velocity must be finite");
  const size_t ng = (size_t)n_ghost;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iff = sg.add(field, (size_t)field_size * 8, true, true);
  const int it = sg.add(target, ng * 8, true, false), is = sg.add(src, 4 * ng * 8, true, false);
  const int io = sg.add(snap_of, 4 * ng * 4, true, false), iw = sg.add(weights, 4 * ng * 8, true, false);
  const int ig = sg.add(gamma, ng * 8, true, false), il = sg.add(level, ng * 4, true, false);
  double* snap = nullptr;
  if (cudaError_t e = sg.begin(ng * 8, &snap)) return cuda_fail(e);
  const unsigned nb = blocks((long long)n_ghost);
  const long long* tg = sg.dev<const long long>(it);
  k_ghost_save<<<nb, LT, 0, sg.st>>>(sg.dev<double>(iff), field_size, tg, n_ghost, snap);
  for (int l = 0; l < n_levels; ++l)
    k_ghost_level<<<nb, LT, 0, sg.st>>>(sg.dev<double>(iff), field_size, tg, sg.dev<const long long>(is),
                                        sg.dev<const int>(io), sg.dev<const double>(iw), sg.dev<const double>(ig),
                                        sg.dev<const int>(il), n_ghost, l, snap, wall);
  gmk::kernel_launch_adjust(1 + n_levels);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_ghost_correct(double* u, double* v, const double* u_star, const double* v_star, const double* phi,
                         const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx, double dy,
                         double dt, double rho, int32_t boundary_faces, void* stream) {
  if (!u || !v || !u_star || !v_star || !phi || !mask || !inlet) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (int rc = check_step(dt, rho)) return rc;
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, true), iv = sg.add(v, nV * 8, true, true);
  const int ius = sg.add(u_star, nU * 8, true, false), ivs = sg.add(v_star, nV * 8, true, false);
  const int iph = sg.add(phi, nP * 8, true, false), im = sg.add(mask, nP, true, false);
  const int ii = sg.add(inlet, (size_t)ny * 8, true, false);
  double* extra = nullptr;
  if (cudaError_t e = sg.begin(0, &extra)) return cuda_fail(e);
  const long long n = (long long)(nU + nV);
  if (boundary_faces)
    k_ghost_boundary<<<blocks(n), LT, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ius),
                                                  sg.dev<double>(ivs), sg.dev<uint8_t>(im), nx, ny);
  else
    k_ghost_correct<<<blocks(n), LT, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ius),
                                                 sg.dev<double>(ivs), sg.dev<double>(iph), sg.dev<uint8_t>(im),
                                                 sg.dev<double>(ii), nx, ny, dx, dy, dt / rho);
  gmk::kernel_launch_adjust(1);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_ghost_forces(const double* u, const double* v, const double* p, int32_t nx, int32_t ny, double dx,
                        double dy, double xc, double yc, double radius, int32_t n_theta, double mu, double out[4],
                        void* stream) {
  if (!u || !v || !p || !out) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (n_theta <= 0) return fail(GM_EVALUE, "n_theta must be positive");
  if (!(std::isfinite(mu) && mu >= 0)) return fail(GM_EVALUE, "mu must be finite and nonnegative");
  if (!(std::isfinite(xc) && std::isfinite(yc) && std::isfinite(radius) && radius > 0))
    return fail(GM_EVALUE, "the circle must be finite with a positive radius");
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, false), iv = sg.add(v, nV * 8, true, false);
  const int ip = sg.add(p, nP * 8, true, false);
  double* res = nullptr;
  if (cudaError_t e = sg.begin(8 * 8, &res)) return cuda_fail(e);
  k_ghost_forces<<<1, 256, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ip), nx, ny, dx, dy,
                                       xc, yc, radius, n_theta, mu, res);
  gmk::kernel_launch_adjust(1);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = cudaMemcpyAsync(out, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, sg.st))
    return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_forces(const double* u, const double* v, const double* p, const uint8_t* mask, int32_t nx, int32_t ny,
                  double dx, double dy, double mu, double out[4], void* stream) {
  if (!u || !v || !p || !mask || !out) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  if (!(std::isfinite(mu) && mu >= 0)) return fail(GM_EVALUE, "mu must be finite and nonnegative");
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  const unsigned nb = blocks((long long)nP);
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, false), iv = sg.add(v, nV * 8, true, false);
  const int ip = sg.add(p, nP * 8, true, false), im = sg.add(mask, nP, true, false);
  double* part = nullptr;
  if (cudaError_t e = sg.begin(((size_t)nb * 4 + 8) * 8, &part)) return cuda_fail(e);
  double* res = part + (size_t)nb * 4;
  k_forces_part<<<nb, LT, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<double>(ip), sg.dev<uint8_t>(im),
                                      nx, ny, dx, dy, mu, part);
  k_fold<<<1, LT, 0, sg.st>>>(part, (int)nb, 4, 0, res);
  gmk::kernel_launch_adjust(2);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  if (cudaError_t e = cudaMemcpyAsync(out, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, sg.st))
    return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  return GM_OK;
}

int gm_mac_divergence(const double* u, const double* v, const uint8_t* mask, int32_t nx, int32_t ny, double dx,
                      double dy, double out[3], int64_t counts[2], void* stream) {
  if (!u || !v || !mask || !out || !counts) return fail(GM_EVALUE, "null argument");
  if (int rc = check_grid(nx, ny, dx, dy)) return rc;
  const size_t nU = (size_t)ny * (nx + 1), nV = (size_t)(ny + 1) * nx, nP = (size_t)ny * nx;
  const unsigned nb = blocks((long long)nP);
  Staging sg(static_cast<cudaStream_t>(stream));
  const int iu = sg.add(u, nU * 8, true, false), iv = sg.add(v, nV * 8, true, false);
  const int im = sg.add(mask, nP, true, false);
  double* part = nullptr;
  if (cudaError_t e = sg.begin(((size_t)nb * 5 + 8) * 8, &part)) return cuda_fail(e);
  double* res = part + (size_t)nb * 5;
  k_div_part<<<nb, LT, 0, sg.st>>>(sg.dev<double>(iu), sg.dev<double>(iv), sg.dev<uint8_t>(im), nx, ny, dx, dy, part);
  k_fold<<<1, LT, 0, sg.st>>>(part, (int)nb, 4, 1, res);
  gmk::kernel_launch_adjust(2);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e);
  double r[5];
  if (cudaError_t e = cudaMemcpyAsync(r, res, sizeof r, cudaMemcpyDeviceToHost, sg.st)) return cuda_fail(e);
  if (cudaError_t e = sg.finish()) return cuda_fail(e);
  out[0] = r[4];
  out[1] = r[0];
  out[2] = r[2];
  counts[0] = (int64_t)std::llround(r[1]);
  counts[1] = (int64_t)std::llround(r[3]);
  return GM_OK;
}

}  // extern "C"
