// Cut-cell (embedded-boundary) AB2/CN step on the GPU: MAC_CylinderFlow(boundary='cut_cell',
// time_scheme='ab2_cn') of the reference (solver/cut_cell_solver.py:790-1015 with
// solver/time_integration.py:7-145).
//
// State and every vector of the step live on the face grid (u then v, ny x (nx+1) and
// (ny+1) x nx, C order) with the non-unknown faces held at zero: the inlet column, covered
// faces and the channel-wall rows of v.  The packed unknown vector of the reference is this
// grid restricted to its active faces, so dot products and norms over the grid equal the
// reference's over q.
//
// Momentum right-hand side (compute_momentum_rhs, solver/cut_cell_solver.py:790-957), one
// evaluation = three launches:
//   k_cc_flux    the four face-flux families on the aperture-weighted staggered faces
//   k_cc_fix     curved faces near the cylinder, one warp per face: advective fluxes from the
//                streamfunction fit at Gauss points, or viscous fluxes from the fitted /
//                ring-corrected gradient, then the wall shear at the circle's Gauss points
//   k_cc_rhs     flux differences into the staggered control volumes (natural outlet row), the
//                wall shear added in the reference's order and the covered-volume transfers
//                (on the few flagged faces), division by rho * owned volume, small-cell
//                merging, covered faces zero, and the packed output (or the CN operator
//                x - dt/2 a for GMRES)
// The CN system is solved by GMRES(30) without a preconditioner (scipy.sparse.linalg.gmres of
// solver/time_integration.py:99-101, rtol 1e-12, atol 1e-13) with its control on the device:
// one WHILE node per restart cycle, one IF node per Arnoldi step, two classical Gram-Schmidt
// passes.  The three pressure solves per step use the pressure-only handle of ghostmac.cu
// over the cut-cell Poisson operator (internal.hpp).  One step is one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ghostmac.h"
#include "geometry.hpp"
#include "internal.hpp"
#include "kernels.cuh"

using namespace gmk;

namespace {

struct CcFail : std::exception {
  int cls;
  std::string msg;
  CcFail(int c, std::string m) : cls(c), msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

#define CCK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) throw CcFail(GM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() { if (p) cudaFree(p); }
  void alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    if (count) CCK(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const std::vector<T>& v, cudaStream_t st) {
    alloc(v.size());
    if (!v.empty()) CCK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void zero(cudaStream_t st) { if (n) CCK(cudaMemsetAsync(p, 0, n * sizeof(T), st)); }
};

constexpr int CC_TPB = 256;
constexpr int CC_FORCE_THREADS = 512;
inline unsigned nblk(int64_t n, int t = CC_TPB) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }
inline void counted() { note_launch_ext(); }

enum : uint8_t { F_ACTIVE = 1, F_FLUID = 2, F_SOLID = 4, F_AUX = 8 };

// geometry of the face grid (kernel argument)
// GB300 issues FP64 at 1/64 of the FP32 rate, so every per-point factor that does not depend on
// the field is folded on the host: the kernels multiply, they never divide.
struct CcGeo {
  int nx, ny;
  int64_t usize, vsize, psize, F;
  double dx, dy, idx, idy;
  const double *ax, *ay;
  // viscous flux factors (aperture x face length / spacing): F = rho nu (difference) c
  const double *cxx, *cyy;   // ny x nx: ax_mid dy / dx, ay_mid dx / dy
  const double *cxy, *cyx;   // (ny+1) x (nx+1): ay_u dx / dy, ax_v dy / dx
  // advective flux factors (rho x aperture x face length): F = -(transported product) a
  const double *axx, *ayy;   // ny x nx: rho ax_mid dy, rho ay_mid dx
  const double *axy, *ayx;   // (ny+1) x (nx+1): rho ay_u dx, rho ax_v dy
  const double* aout;        // ny: rho ax[:, nx] dy (natural outlet)
  const uint8_t* flags;      // F: F_ACTIVE unknown, F_FLUID divided by its own volume, F_SOLID covered face
  const int32_t* cell_type;  // psize
  const double* kappa;       // psize: fluid fraction
  const double* ikappa;      // psize: 1 / fluid fraction on cut cells, 1 elsewhere
  const double* ivol_rho;    // F: 1 / (rho * owned volume)
  const int32_t* merge_of;   // F: the last merge that writes the face, or -1
  const int64_t* ms;         // merges: small face, master face (face-grid flat), 1 / (rho * merged volume)
  const int64_t* mm;
  const double* imvol_rho;
};

// curved-face flux overrides, the four families concatenated (0 F_xx, 1 F_xy, 2 F_yx, 3 F_yy)
struct CcFix {
  int n_dif;
  const uint8_t* dfam;
  const int64_t* dface;
  const int64_t* dptr;
  const int64_t* dcol;
  const double* dval;
  int n_adv;
  const uint8_t* afam;
  const int64_t* aface;
  const int64_t* apptr;  // n_adv + 1: each face's Gauss points
  const int64_t* uptr;
  const int64_t* ucol;
  const double* uval;
  const int64_t* vptr;
  const int64_t* vcol;
  const double* vval;
  const double* alen;
};

struct CcWall {
  int n;  // Gauss points on the circle
  const int64_t* ptr;
  const int64_t* col;
  const double* val;
  const double* tx;
  const double* ty;
  const double* ds;
  int n_tgt;  // faces receiving wall shear, each with its points in the reference's order
  const int64_t* tgt;
  const int64_t* tptr;
  const int32_t* tk;
  int n_own;  // owners of covered volumes, each with its donors in order
  const int64_t* own;
  const int64_t* optr;
  const int64_t* odon;
  int n_don;
  const int64_t* don;
  double* tau;  // n scratch
  // faces flagged F_AUX (wall targets, owners, donors), sorted, with their target and owner
  // list entries (-1: none) and whether they are donors
  int n_aux;
  const int64_t* aux_face;
  const int32_t* aux_tgt;
  const int32_t* aux_own;
  const uint8_t* aux_don;
};

struct CcFlux {
  double *xx, *xy, *yx, *yy;
};

// Per-step device diagnostics (maxima as the bits of non-negative doubles)
struct CcDiagDev {
  unsigned long long rhs_max, mres, coupled, umax, vmax, divmax;
  unsigned long long pdiv[3];  // predicted divergence of the start-up, first and second solve
  double forces[6];
  double res_linf, res_l2;     // the legacy step's pressure residual b - A phi (unscaled rows)
};

// field value c of the concatenated face grid, with the inlet column from `inl` when given
__device__ __forceinline__ double fld(const CcGeo& g, const double* __restrict__ X, const double* __restrict__ inl,
                                      int64_t c) {
  if (inl && c < g.usize && c % (g.nx + 1) == 0) return inl[c / (g.nx + 1)];
  return X[c];
}

__device__ __forceinline__ void atomic_max_abs(unsigned long long* out, double v) {
  atomicMax(out, (unsigned long long)__double_as_longlong(fabs(v)));
}

// the block's maximum |m| (a NaN stays visible) committed with one atomic: warp maxima, then
// the first warp over the block's warps
__device__ __forceinline__ void block_commit_max_abs(double m, unsigned long long* out) {
  __shared__ double wm[32];
  for (int o = 16; o; o >>= 1) {
    const double q = __shfl_down_sync(0xffffffffu, m, o);
    m = (q != q) ? q : fmax(m, q);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();  // an earlier call's readers are done with wm
  if (lane == 0) wm[w] = m;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    m = lane < nw ? wm[lane] : 0.0;
    for (int o = 16; o; o >>= 1) {
      const double q = __shfl_down_sync(0xffffffffu, m, o);
      m = (q != q) ? q : fmax(m, q);
    }
    if (lane == 0) atomic_max_abs(out, m);
  }
}

// One CSR row times the field by a whole warp: lanes stride over the row's entries, then a
// butterfly sum leaves the same total in every lane (the pairs add in mirrored order, which
// IEEE addition does not distinguish), in a fixed order from run to run.
__device__ __forceinline__ double warp_row_dot(const int64_t* __restrict__ ptr, const int64_t* __restrict__ col,
                                               const double* __restrict__ val, int64_t r, const CcGeo& g,
                                               const double* __restrict__ X, const double* __restrict__ inl,
                                               int lane) {
  double acc = 0.0;
  for (int64_t e = ptr[r] + lane; e < ptr[r + 1]; e += 32) acc += val[e] * fld(g, X, inl, col[e]);
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// ---- momentum right-hand side -------------------------------------------------------------
// One thread per vertex (j, i) of the (ny+1) x (nx+1) grid: F_xx and F_yy of cell (j, i),
// F_xy and F_yx of vertex (j, i) (solver/cut_cell_solver.py:808-914).  ADV: the advective
// form (nu = 0: no viscous part), with the transported velocity centred or, UPW, taken from
// the upwind side of the face's advecting velocity (transport='upwind'); otherwise the
// viscous form without advection.
template <bool ADV, bool UPW = false>
__global__ void k_cc_flux(CcGeo g, const double* __restrict__ X, const double* __restrict__ inl, double rnu,
                          int slip, CcFlux F) {
  const int nx = g.nx, ny = g.ny;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)(ny + 1) * (nx + 1)) return;
  const int j = (int)(t / (nx + 1)), i = (int)(t % (nx + 1));
  const double* V = X + g.usize;
  auto U = [&](int jj, int ii) -> double {
    const int64_t f = (int64_t)jj * (nx + 1) + ii;
    return (ii == 0 && inl) ? inl[jj] : X[f];
  };
  auto W = [&](int jj, int ii) -> double { return V[(int64_t)jj * nx + ii]; };
  if (j < ny && i < nx) {
    const int64_t c = (int64_t)j * nx + i;
    const double ul = U(j, i), ur = U(j, i + 1), vb = W(j, i), vt = W(j + 1, i);
    if (ADV) {
      const double uf = 0.5 * (ul + ur), vf = 0.5 * (vb + vt);
      const double ua = UPW ? (uf >= 0.0 ? ul : ur) : uf, va = UPW ? (vf >= 0.0 ? vb : vt) : vf;
      F.xx[c] = -(uf * ua * g.axx[c]);
      F.yy[c] = -(vf * va * g.ayy[c]);
    } else {
      F.xx[c] = rnu * (ur - ul) * g.cxx[c];
      F.yy[c] = rnu * (vt - vb) * g.cyy[c];
    }
  }
  {
    double f;
    if (j == 0) f = (ADV || slip) ? 0.0 : rnu * U(0, i) * (2.0 * g.cxy[t]);
    else if (j == ny) f = (ADV || slip) ? 0.0 : -(rnu * U(ny - 1, i) * (2.0 * g.cxy[t]));
    else if (ADV) {
      const double vf = i == 0 ? W(j, 0) : (i == nx ? W(j, nx - 1) : 0.5 * (W(j, i - 1) + W(j, i)));
      const double ua = UPW ? (vf >= 0.0 ? U(j - 1, i) : U(j, i)) : 0.5 * (U(j - 1, i) + U(j, i));
      f = -(vf * ua * g.axy[t]);
    } else {
      f = rnu * (U(j, i) - U(j - 1, i)) * g.cxy[t];
    }
    F.xy[t] = f;
  }
  {
    double f;
    if (i == 0) {
      f = ADV ? 0.0 : rnu * W(j, 0) * (2.0 * g.cyx[t]);
    } else if (i == nx) {
      f = 0.0;
      if (ADV) {
        const double uo = j == 0 ? U(0, nx) : (j == ny ? U(ny - 1, nx) : 0.5 * (U(j - 1, nx) + U(j, nx)));
        f = -(uo * W(j, nx - 1) * g.ayx[t]);
      }
    } else if (ADV) {
      const double uf = j == 0 ? U(0, i) : (j == ny ? U(ny - 1, i) : 0.5 * (U(j - 1, i) + U(j, i)));
      const double va = UPW ? (uf >= 0.0 ? W(j, i - 1) : W(j, i)) : 0.5 * (W(j, i - 1) + W(j, i));
      f = -(uf * va * g.ayx[t]);
    } else {
      f = rnu * (W(j, i) - W(j, i - 1)) * g.cyx[t];
    }
    F.yx[t] = f;
  }
}

// Curved faces (solver/staggered_wall.py:134-140 and the viscous correction of
// solver/cut_cell_solver.py:822-825), one warp per face: ADV: -rho * sum over the face's Gauss
// points of length * (u u | u v | v v) with u, v from the fit; otherwise rho nu (gradient row .
// field), and then one warp per wall Gauss point for its shear stress (wscale = -rho nu).
template <bool ADV>
__global__ void k_cc_fix(CcGeo g, CcFix fx, CcWall w, const double* __restrict__ X, const double* __restrict__ inl,
                         double rnu, double rho, double wscale, CcFlux F) {
  const int lane = threadIdx.x & 31;
  const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  double* fam[4] = {F.xx, F.xy, F.yx, F.yy};
  if (!ADV) {
    if (r < fx.n_dif) {
      const double acc = warp_row_dot(fx.dptr, fx.dcol, fx.dval, r, g, X, inl, lane);
      if (lane == 0) fam[fx.dfam[r]][fx.dface[r]] = rnu * acc;
    } else if (r < fx.n_dif + w.n) {
      // wall shear stress -rho nu (rate . field) at Gauss point k (solver/cut_cell_solver.py:921-924)
      const int k = r - fx.n_dif;
      const double acc = warp_row_dot(w.ptr, w.col, w.val, k, g, X, inl, lane);
      if (lane == 0) w.tau[k] = wscale * acc;
    }
  } else {
    if (r >= fx.n_adv) return;
    const int fm = fx.afam[r];
    double s = 0.0;
    for (int64_t p = fx.apptr[r]; p < fx.apptr[r + 1]; ++p) {
      const double ue = warp_row_dot(fx.uptr, fx.ucol, fx.uval, p, g, X, inl, lane);
      const double ve = warp_row_dot(fx.vptr, fx.vcol, fx.vval, p, g, X, inl, lane);
      const double prod = fm == 0 ? ue * ue : (fm == 3 ? ve * ve : ue * ve);
      s += fx.alen[p] * prod;
    }
    if (lane == 0) fam[fm][fx.aface[r]] = -(rho * s);
  }
}

// Flux differences of face f (solver/cut_cell_solver.py:853-861, 916-917; the natural outlet
// row of u at :857-861)
template <bool ADV>
__device__ __forceinline__ double rhs_base(const CcGeo& g, const CcFlux& F, const double* __restrict__ X, int64_t f) {
  const int nx = g.nx, ny = g.ny;
  if (f < g.usize) {
    const int j = (int)(f / (nx + 1)), i = (int)(f % (nx + 1));
    if (i >= 1 && i < nx)
      return (F.xx[(int64_t)j * nx + i] - F.xx[(int64_t)j * nx + i - 1]) + (F.xy[f + nx + 1] - F.xy[f]);
    if (i == nx) {
      double ext = 0.0;
      if (ADV) {
        const double un = X[f];
        ext = -(un * un * g.aout[j]);
      }
      return (ext - F.xx[(int64_t)j * nx + nx - 1]) + 0.5 * (F.xy[f + nx + 1] - F.xy[f]);
    }
    return 0.0;
  }
  const int64_t c = f - g.usize;
  const int j = (int)(c / nx), i = (int)(c % nx);
  if (j >= 1 && j < ny)
    return (F.yx[(int64_t)j * (nx + 1) + i + 1] - F.yx[(int64_t)j * (nx + 1) + i]) + (F.yy[c] - F.yy[c - nx]);
  return 0.0;
}

__device__ __forceinline__ int aux_find(const CcWall& w, int64_t f) {
  int lo = 0, hi = w.n_aux - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (w.aux_face[mid] < f) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// right-hand side of face f after the wall shear (added in the order of the Gauss points,
// np.add.at of solver/cut_cell_solver.py:922-924)
template <bool ADV>
__device__ double rhs_walled(const CcGeo& g, const CcFlux& F, const CcWall& w, const double* __restrict__ X,
                             int64_t f, int shear, int a) {
  double r = rhs_base<ADV>(g, F, X, f);
  const int t = a >= 0 ? w.aux_tgt[a] : -1;
  if (shear && t >= 0) {
    const double* dir = f < g.usize ? w.tx : w.ty;
    for (int64_t q = w.tptr[t]; q < w.tptr[t + 1]; ++q) {
      const int k = w.tk[q];
      r += w.tau[k] * dir[k] * w.ds[k];
    }
  }
  return r;
}

// the full right-hand side of face f: flux differences, wall shear, then the covered-volume
// transfers (donors give their whole value to their owner in donor order and hold zero;
// solid/staggered_wall.py:302-304)
template <bool ADV>
__device__ double rhs_full(const CcGeo& g, const CcFlux& F, const CcWall& w, const double* __restrict__ X, int64_t f,
                           int shear) {
  if (!(g.flags[f] & F_AUX)) return rhs_base<ADV>(g, F, X, f);
  const int a = aux_find(w, f);
  if (w.aux_don[a]) return 0.0;
  double r = rhs_walled<ADV>(g, F, w, X, f, shear, a);
  const int o = w.aux_own[a];
  if (o >= 0)
    for (int64_t q = w.optr[o]; q < w.optr[o + 1]; ++q) {
      const int64_t d = w.odon[q];
      r += rhs_walled<ADV>(g, F, w, X, d, shear, (g.flags[d] & F_AUX) ? aux_find(w, d) : -1);
    }
  return r;
}

// Right-hand side and accelerations in one pass (solver/cut_cell_solver.py:853-955): flux
// differences, wall shear and covered transfers (flagged faces only), division by rho x owned
// volume (a multiply by the host-formed reciprocal), small-cell merging, covered faces zero.
// mode 0: Y = packed a; 1: Y = packed (X - hdt a) (the CN operator); 2: Y = a and Rout = rhs,
// both unpacked.
template <bool ADV>
__global__ void k_cc_rhs(CcGeo g, CcFlux F, CcWall w, const double* __restrict__ X, int shear, double hdt, int mode,
                         double* __restrict__ Y, double* __restrict__ Rout) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.F) return;
  const uint8_t fl = g.flags[f];
  const double r = rhs_full<ADV>(g, F, w, X, f, shear);
  double a = 0.0;
  if (fl & F_FLUID) a = r * g.ivol_rho[f];
  const int m = g.merge_of[f];
  if (m >= 0) {
    const int64_t fs = g.ms[m], fm = g.mm[m];
    const double rs = fs == f ? r : rhs_full<ADV>(g, F, w, X, fs, shear);
    const double rm = fm == f ? r : rhs_full<ADV>(g, F, w, X, fm, shear);
    a = (rs + rm) * g.imvol_rho[m];
  }
  if (fl & F_SOLID) a = 0.0;
  if (mode == 0) Y[f] = (fl & F_ACTIVE) ? a : 0.0;
  else if (mode == 1) Y[f] = (fl & F_ACTIVE) ? X[f] - hdt * a : 0.0;
  else {
    Y[f] = a;
    Rout[f] = (fl & F_SOLID) ? 0.0 : r;
  }
}

// ---- projection pieces ----------------------------------------------------------------------
// (rho / dt) times the aperture-weighted divergence of the unpacked field, zero on covered
// cells (compute_rhs, solver/cut_cell_solver.py:732-738), divided by kappa on cut cells (the row
// scaling of the pressure system built by gm::build_cutcell_geometry)
__global__ void k_cc_divrhs(CcGeo g, const double* __restrict__ X, const double* __restrict__ inl, double inv_dt,
                            double* __restrict__ B) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.psize) return;
  if (g.cell_type[c] == -1) { B[c] = 0.0; return; }
  const int nx = g.nx;
  const int j = (int)(c / nx), i = (int)(c % nx);
  const int64_t fu = (int64_t)j * (nx + 1) + i;
  const double uw = (i == 0 && inl) ? inl[j] : X[fu];
  const double* V = X + g.usize;
  const double fx = (g.ax[fu + 1] * X[fu + 1] - g.ax[fu] * uw) * g.idx;
  const double fy = (g.ay[c + nx] * V[c + nx] - g.ay[c] * V[c]) * g.idy;
  B[c] = inv_dt * (fx + fy) * g.ikappa[c];
}
// a caller's right-hand side in the row scaling of the pressure system: cut cells / kappa,
// covered cells zero
__global__ void k_cc_scale_rhs(CcGeo g, double* __restrict__ B) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.psize) return;
  B[c] = g.cell_type[c] == -1 ? 0.0 : B[c] * g.ikappa[c];
}

// corrector (solver/cut_cell_solver.py:740-753), packed output; sx = dt / (rho dx), sy = dt / (rho dy)
__global__ void k_cc_correct(CcGeo g, const double* __restrict__ X, const double* __restrict__ phi, double sx,
                             double sy, double* __restrict__ Y) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.F) return;
  const int nx = g.nx, ny = g.ny;
  double r = 0.0;
  if (f < g.usize) {
    const int j = (int)(f / (nx + 1)), i = (int)(f % (nx + 1));
    const int64_t c = (int64_t)j * nx + i;
    if (i >= 1 && i < nx) r = g.ax[f] > 0.0 ? X[f] - sx * (phi[c] - phi[c - 1]) : 0.0;
    else if (i == nx) r = X[f] + (2.0 * sx) * phi[c - 1];
  } else {
    const int64_t c = f - g.usize;
    const int j = (int)(c / nx);
    if (j >= 1 && j < ny) r = g.ay[c] > 0.0 ? X[f] - sy * (phi[c] - phi[c - nx]) : 0.0;
  }
  Y[f] = (g.flags[f] & F_ACTIVE) ? r : 0.0;
}

// pressure gradient / rho on the unknown faces (advance_ab2_cn's gradient,
// solver/cut_cell_solver.py:979-984); gx = 1 / (rho dx), gy = 1 / (rho dy)
__global__ void k_cc_grad(CcGeo g, const double* __restrict__ P, double gx, double gy, double* __restrict__ Y) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.F) return;
  const int nx = g.nx, ny = g.ny;
  double r = 0.0;
  if (f < g.usize) {
    const int j = (int)(f / (nx + 1)), i = (int)(f % (nx + 1));
    const int64_t c = (int64_t)j * nx + i;
    if (i >= 1 && i < nx) r = (P[c] - P[c - 1]) * gx;
    else if (i == nx) r = -2.0 * P[c - 1] * gx;
  } else {
    const int64_t c = f - g.usize;
    const int j = (int)(c / nx);
    if (j >= 1 && j < ny) r = (P[c] - P[c - nx]) * gy;
  }
  Y[f] = (g.flags[f] & F_ACTIVE) ? r : 0.0;
}

// pack (X = masked U) and unpack (U = X with the inlet column)
__global__ void k_cc_pack(CcGeo g, const double* __restrict__ U, double* __restrict__ X) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f < g.F) X[f] = (g.flags[f] & F_ACTIVE) ? U[f] : 0.0;
}
__global__ void k_cc_unpack(CcGeo g, const double* __restrict__ X, const double* __restrict__ inl,
                            double* __restrict__ U) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.F) return;
  if (f < g.usize && f % (g.nx + 1) == 0) U[f] = inl[f / (g.nx + 1)];
  else U[f] = (g.flags[f] & F_ACTIVE) ? X[f] : 0.0;
}

// ---- vector steps of solver/time_integration.py:7-145 -------------------------------------
// op 0: out = a + s0 ((b + c) - d)            midpoint start-up
// op 1: out = (1 + s0) a - s0 b               AB2 advection
// op 2: out = (a + s0 ((b + 0.5 c) - d)) + s1 e   CN right-hand side
// op 3: out = a + (b - c)                     projected result plus the momentum defect
__global__ void k_cc_vec(int op, int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                         const double* __restrict__ c, const double* __restrict__ d, const double* __restrict__ e,
                         double s0, double s1, double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double r;
  if (op == 0) r = a[t] + s0 * ((b[t] + c[t]) - d[t]);
  else if (op == 1) r = (1 + s0) * a[t] - s0 * b[t];
  else if (op == 2) r = (a[t] + s0 * ((b[t] + 0.5 * c[t]) - d[t])) + s1 * e[t];
  else r = a[t] + (b[t] - c[t]);
  out[t] = r;
}
// half = p + inc; out = half + factor inc
__global__ void k_cc_pressure_out(int64_t n, const double* __restrict__ p, const double* __restrict__ inc,
                                  double factor, double* __restrict__ half, double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double h = p[t] + inc[t];
  half[t] = h;
  out[t] = h + factor * inc[t];
}
// max |a - b| (b may be null), max |(a - b) + s c| with c set
__global__ void k_cc_maxdiff(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                             const double* __restrict__ c, double s, unsigned long long* out) {
  double m = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double v = b ? a[t] - b[t] : a[t];
    if (c) v = v + s * c[t];
    m = fmax(m, fabs(v));
    if (v != v) m = v;  // keep a NaN visible
  }
  block_commit_max_abs(m, out);
}
// predicted divergence dt/rho max_fluid |res| / kappa (solver/cut_cell_solver.py:721-722); the
// residual of the row-scaled system already carries the 1 / kappa
__global__ void k_cc_pdiv(CcGeo g, const double* __restrict__ res, double scale, unsigned long long* out) {
  double m = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.psize; c += (int64_t)gridDim.x * blockDim.x)
    if (g.cell_type[c] != -1) {
      const double v = scale * fabs(res[c]);
      m = (v != v) ? v : fmax(m, v);
    }
  block_commit_max_abs(m, out);
}
// step gate quantities of solver/main.py:416-424: max_fluid |flux divergence| / kappa, max |u|, max |v|
__global__ void k_cc_stepmax(CcGeo g, const double* __restrict__ U, unsigned long long* divmax,
                             unsigned long long* umax, unsigned long long* vmax) {
  const int nx = g.nx;
  double dm = 0.0, um = 0.0, vm = 0.0;
  const double* V = U + g.usize;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < g.F; f += (int64_t)gridDim.x * blockDim.x) {
    if (f < g.usize) um = fmax(um, fabs(U[f]));
    else vm = fmax(vm, fabs(U[f]));
    if (f < g.psize && g.cell_type[f] != -1) {
      const int64_t c = f;
      const int j = (int)(c / nx), i = (int)(c % nx);
      const int64_t fu = (int64_t)j * (nx + 1) + i;
      const double d = (g.ax[fu + 1] * U[fu + 1] - g.ax[fu] * U[fu]) * g.idx +
                       (g.ay[c + nx] * V[c + nx] - g.ay[c] * V[c]) * g.idy;
      const double v = fabs(d) * g.ikappa[c];
      dm = (v != v) ? v : fmax(dm, v);
    }
  }
  block_commit_max_abs(dm, divmax);
  block_commit_max_abs(um, umax);
  block_commit_max_abs(vm, vmax);
}

// The legacy predictor (advance_momentum_predictor, solver/cut_cell_solver.py:1017-1033) and
// apply_predictor_boundary (:663-670): a = advective + viscous acceleration, u* = u + dt a
// (forward Euler) or u + dt ((1 + alpha) a - alpha a_prev) (AB2), a_prev = a; then the inlet
// column, zero on closed faces and on the channel-wall v rows.
__global__ void k_cc_legacy_pred(CcGeo g, const double* __restrict__ U, const double* __restrict__ aa,
                                 const double* __restrict__ ad, double* __restrict__ prev,
                                 const double* __restrict__ inl, double dt, double alpha, int ab2,
                                 double* __restrict__ star) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.F) return;
  const double a = aa[f] + ad[f];
  double s = ab2 ? U[f] + dt * ((1 + alpha) * a - alpha * prev[f]) : U[f] + dt * a;
  prev[f] = a;
  if (f < g.usize) {
    if (f % (g.nx + 1) == 0) s = inl[f / (g.nx + 1)];
    if (g.ax[f] == 0.0) s = 0.0;
  } else {
    const int64_t c = f - g.usize;
    const int j = (int)(c / g.nx);
    if (g.ay[c] == 0.0 || j == 0 || j == g.ny) s = 0.0;
  }
  star[f] = s;
}

// max |r| and sum r^2 of the pressure residual in the unscaled rows (the row-scaled residual
// times kappa), per block, then folded by one block in a fixed order (deterministic)
constexpr int CC_RES_BLOCKS = 152;
__global__ void k_cc_resnorm_part(CcGeo g, const double* __restrict__ res, double* __restrict__ part) {
  __shared__ double smax[CC_TPB], ssum[CC_TPB];
  double m = 0.0, q = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.psize; c += (int64_t)gridDim.x * blockDim.x)
    if (g.cell_type[c] != -1) {
      const double r = res[c] * g.kappa[c];
      m = (r != r) ? r : fmax(m, fabs(r));
      q += r * r;
    }
  smax[threadIdx.x] = m;
  ssum[threadIdx.x] = q;
  __syncthreads();
  for (int k = CC_TPB / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) {
      const double o = smax[threadIdx.x + k];
      smax[threadIdx.x] = (o != o) ? o : fmax(smax[threadIdx.x], o);
      ssum[threadIdx.x] += ssum[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = smax[0];
    part[2 * blockIdx.x + 1] = ssum[0];
  }
}
__global__ void k_cc_resnorm_fold(const double* __restrict__ part, int nb, double* __restrict__ linf,
                                  double* __restrict__ l2) {
  __shared__ double smax[CC_TPB], ssum[CC_TPB];
  double m = 0.0, q = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const double o = part[2 * b];
    m = (o != o) ? o : fmax(m, o);
    q += part[2 * b + 1];
  }
  smax[threadIdx.x] = m;
  ssum[threadIdx.x] = q;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) {
      const double o = smax[threadIdx.x + k];
      smax[threadIdx.x] = (o != o) ? o : fmax(smax[threadIdx.x], o);
      ssum[threadIdx.x] += ssum[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *linf = smax[0];
    *l2 = sqrt(ssum[0]);
  }
}

// fixed-order block sum of one value per thread (blockDim a power of two <= 1024)
__device__ double block_sum(double v, double* sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] = sh[tid] + sh[tid + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// mu (rate . field) at every wall Gauss point, one warp each: the wall shear stress of the
// forces (the same warp dot product as the forces kernel's, so the same values)
__global__ void k_cc_wall_tau(CcWall w, const double* __restrict__ U, double mu, double* __restrict__ tau) {
  const int lane = threadIdx.x & 31;
  const int k = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (k >= w.n) return;  // whole warps leave together
  const double acc = warp_row_dot(w.ptr, w.col, w.val, k, CcGeo{}, U, nullptr, lane);
  if (lane == 0) tau[k] = mu * acc;
}

// Forces on the true circle (extract_true_surface_forces, solver/cut_cell_solver.py:755-765):
// pressure from the point reconstruction with its mean removed, shear mu (rate . field) at
// the wall Gauss points.  One block; out = fx, fy, fx_p, fy_p, fx_v, fy_v.
__global__ void k_cc_forces(gmi::SurfaceCsr S, CcWall w, const double* __restrict__ P,
                            const double* __restrict__ tau, double* __restrict__ pb, double* __restrict__ out) {
  __shared__ double sh[CC_FORCE_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  double s = 0.0;
  for (int k = tid; k < S.n; k += nt) {
    double acc = 0.0;
    for (int64_t e = S.ptr[k]; e < S.ptr[k + 1]; ++e) acc += S.val[e] * P[S.col[e]];
    pb[k] = acc;
    s += acc;
  }
  const double mean = block_sum(s, sh) / S.n;
  double px = 0.0, py = 0.0;
  for (int k = tid; k < S.n; k += nt) {
    const double d = pb[k] - mean;
    px += d * S.nwx[k];
    py += d * S.nwy[k];
  }
  const double fxp = -block_sum(px, sh), fyp = -block_sum(py, sh);
  double vx = 0.0, vy = 0.0;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  if (lane == 0)
    for (int k = warp; k < w.n; k += nwarp) {
      vx += tau[k] * w.tx[k] * w.ds[k];
      vy += tau[k] * w.ty[k] * w.ds[k];
    }
  const double fxv = block_sum(vx, sh), fyv = block_sum(vy, sh);
  if (tid == 0) {
    out[0] = fxp + fxv;
    out[1] = fyp + fyv;
    out[2] = fxp;
    out[3] = fyp;
    out[4] = fxv;
    out[5] = fyv;
  }
}

// calculate_cut_cell_divergence (solver/cut_cell_solver.py:219-260): max |div|, sum div^2,
// fluid count, max |net flux|, one block in a fixed order
__global__ void k_cc_divstats(CcGeo g, const double* __restrict__ U, double* __restrict__ out) {
  __shared__ double sh[CC_FORCE_THREADS];
  const int nx = g.nx;
  const double* V = U + g.usize;
  double mdiv = 0.0, sq = 0.0, cnt = 0.0, mflux = 0.0;
  for (int64_t c = threadIdx.x; c < g.psize; c += blockDim.x) {
    if (g.cell_type[c] == -1) continue;
    const int j = (int)(c / nx), i = (int)(c % nx);
    const int64_t fu = (int64_t)j * (nx + 1) + i;
    const double fx = g.ax[fu + 1] * g.dy * U[fu + 1] - g.ax[fu] * g.dy * U[fu];
    const double fy = g.ay[c + nx] * g.dx * V[c + nx] - g.ay[c] * g.dx * V[c];
    const double net = fx + fy;
    const double vol = g.kappa[c] * g.dx * g.dy;  // diagnostics only: the reference's division
    const double d = vol > 0.0 ? net / vol : 0.0;
    mdiv = fmax(mdiv, fabs(d));
    mflux = fmax(mflux, fabs(net));
    sq += d * d;
    cnt += 1.0;
  }
  const double tsq = block_sum(sq, sh), tcnt = block_sum(cnt, sh);
  sh[threadIdx.x] = mdiv;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  const double tmd = sh[0];
  __syncthreads();
  sh[threadIdx.x] = mflux;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = tmd;
    out[1] = tsq;
    out[2] = tcnt;
    out[3] = sh[0];
  }
}

// ---- Gram-Schmidt of the CN GMRES -------------------------------------------------------
// Two classical passes per Arnoldi step with the basis read once per pass: k_gs_dot forms the
// partial dots V^T w; k_gs_pass<NV, NORM> reduces the previous partials to the coefficients
// (every block in the same fixed order, so all blocks hold identical values), subtracts V c
// from w and, in the same sweep, forms the partials of the next pass (V^T w) or of |w|^2.
// One block per SM; NV (the basis size, a compile-time constant per Arnoldi step) keeps the
// accumulators in registers.
constexpr int GS_BLOCKS = 152;
constexpr int GS_THREADS = 512;
constexpr int GS_MAXV = 32;

template <int NV>
__device__ __forceinline__ void gs_block_partials(double (&acc)[NV], double* __restrict__ part) {
  __shared__ double red[GS_THREADS / 32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double a = acc[i];
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp][i] = a;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NV; i += blockDim.x) {
    double a = 0.0;
    for (int q = 0; q < GS_THREADS / 32; ++q) a += red[q][i];
    part[(int64_t)blockIdx.x * GS_MAXV + i] = a;
  }
}

// coefficients c_i = sum over blocks of part[b][i], in a fixed order
template <int NV>
__device__ __forceinline__ void gs_coefficients(const double* __restrict__ part, double* cf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < NV) {
    double a = 0.0;
    for (int b = lane; b < GS_BLOCKS; b += 32) a += part[(int64_t)b * GS_MAXV + warp];
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) cf[warp] = a;
  }
  __syncthreads();
}

template <int NV>
__global__ void __launch_bounds__(GS_THREADS) k_gs_dot(const double* __restrict__ V, int64_t n,
                                                       const double* __restrict__ w, double* __restrict__ part) {
  double acc[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) acc[i] = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double wt = w[t];
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] += V[(int64_t)i * n + t] * wt;
  }
  gs_block_partials<NV>(acc, part);
}

// w -= V c (c from part_in); then part_out = partials of V^T w (NORM = false) or of |w|^2
// (NORM = true, one value per block); block 0 stores c for the Hessenberg column
template <int NV, bool NORM>
__global__ void __launch_bounds__(GS_THREADS) k_gs_pass(const double* __restrict__ V, int64_t n,
                                                        const double* __restrict__ part_in, double* __restrict__ w,
                                                        double* __restrict__ part_out, double* __restrict__ coef) {
  __shared__ double cf[NV];
  gs_coefficients<NV>(part_in, cf);
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < NV; i += blockDim.x) coef[i] = cf[i];
  constexpr int NA = NORM ? 1 : NV;
  double acc[NA];
#pragma unroll
  for (int i = 0; i < NA; ++i) acc[i] = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double v[NV];
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      v[i] = V[(int64_t)i * n + t];
      s += cf[i] * v[i];
    }
    const double wt = w[t] - s;
    w[t] = wt;
    if (NORM) acc[0] += wt * wt;
    else {
#pragma unroll
      for (int i = 0; i < NA; ++i) acc[i] += v[i] * wt;
    }
  }
  gs_block_partials<NA>(acc, part_out);
}

// V0 = b - w with the partials of |V0|^2 (the residual that starts a restart cycle)
__global__ void __launch_bounds__(GS_THREADS) k_gs_residual(const double* __restrict__ b, const double* __restrict__ w,
                                                            int64_t n, double* __restrict__ r,
                                                            double* __restrict__ part) {
  double acc[1] = {0.0};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double v = b[t] - w[t];
    r[t] = v;
    acc[0] += v * v;
  }
  gs_block_partials<1>(acc, part);
}

// the sum of one partial per block, in a fixed order, into out[0]
__global__ void k_gs_sum(const double* __restrict__ part, double* __restrict__ out) {
  double a = 0.0;
  for (int b = threadIdx.x; b < GS_BLOCKS; b += 32) a += part[(int64_t)b * GS_MAXV];
  for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (threadIdx.x == 0) out[0] = a;
}

template <int NV>
void gs_step_nv(const double* V, int64_t n, double* w, double* part1, double* part2, double* d1, double* d2,
                cudaStream_t st) {
  counted();
  k_gs_dot<NV><<<GS_BLOCKS, GS_THREADS, 0, st>>>(V, n, w, part1);
  counted();
  k_gs_pass<NV, false><<<GS_BLOCKS, GS_THREADS, 0, st>>>(V, n, part1, w, part2, d1);
  counted();
  k_gs_pass<NV, true><<<GS_BLOCKS, GS_THREADS, 0, st>>>(V, n, part2, w, part1, d2);
}

// both Gram-Schmidt passes of Arnoldi step j (basis V_0..V_j) on w; d1, d2 the coefficients,
// |w|^2 into wn2.  Up to 12 basis vectors the fused passes keep their values in registers;
// beyond that (steps that converged problems rarely reach) the separate dot / update kernels
// (part1 then holds multidot_blocks(n) x 64 partials).
void gs_step(int nv, const double* V, int64_t n, double* w, double* part1, double* part2, double* d1, double* d2,
             double* wn2, cudaStream_t st) {
  switch (nv) {
#define GS_CASE(K) case K: gs_step_nv<K>(V, n, w, part1, part2, d1, d2, st); break;
    GS_CASE(1) GS_CASE(2) GS_CASE(3) GS_CASE(4) GS_CASE(5) GS_CASE(6) GS_CASE(7) GS_CASE(8) GS_CASE(9)
    GS_CASE(10) GS_CASE(11) GS_CASE(12)
#undef GS_CASE
    default:
      launch_multidot(V, n, nv, w, n, part1, d1, st);
      launch_multiaxpy(V, n, nv, d1, -1.0, 1.0, w, n, st);
      launch_multidot(V, n, nv, w, n, part1, d2, st);
      launch_multiaxpy(V, n, nv, d2, -1.0, 1.0, w, n, st);
      launch_multidot(w, n, 1, w, n, part1, wn2, st);
      return;
  }
  counted();
  k_gs_sum<<<1, 32, 0, st>>>(part1, wn2);
}

}  // namespace

// =============================================================================================
// handle
// =============================================================================================
struct gm_cc {
  std::string err;
  gm_handle* P = nullptr;  // pressure-only handle (stream, Poisson inverse, control block)
  cudaStream_t st = nullptr;
  int nx = 0, ny = 0;
  int64_t usize = 0, vsize = 0, psize = 0, F = 0;
  double dx = 0, dy = 0, rho = 1, nu = 0, D = 1, U_ref = 1;
  int slip = 0;
  int64_t n_active = 0;
  std::vector<int64_t> act_idx;  // face-grid flat indices of the unknowns (packed order)
  // geometry on the device
  Buf<double> ax, ay, kappa, ikappa, vol_rho, mvol_rho, inlet;
  Buf<double> cxx, cyy, cxy, cyx, axx, ayy, axy, ayx, aout;
  Buf<uint8_t> flags;
  Buf<int32_t> cell_type, merge_of;
  Buf<int64_t> ms, mm, d_act;
  // overrides
  Buf<uint8_t> dfam, afam;
  Buf<int64_t> dface, dptr, dcol, aface, apptr, uptr, ucol, vptr, vcol;
  Buf<double> dval, uval, vval, alen;
  // wall and transfers
  Buf<int64_t> wptr, wcol, tgt, tptr, own, optr, odon, don;
  Buf<int32_t> tk, aux_tgt, aux_own;
  Buf<int64_t> aux_face;
  Buf<uint8_t> aux_don;
  Buf<double> wval, wtx, wty, wds, tau;
  CcGeo geo{};
  CcFix fix{};
  CcWall wall{};
  // state: U (unpacked face grid), P; history
  Buf<double> U, Pst, prev_adv, halfp, halfp_next;
  bool has_history = false;
  double prev_dt = 0;
  // work vectors (face grid) and pressure-grid work
  Buf<double> q0, now, d0, gp, mid, halfq, expl, offset, dq, rhs, star, w, result, action, tmp, zero, Rw;
  Buf<double> fxx, fxy, fyx, fyy;
  Buf<double> B, phi, inc, pb, io_f, io_p;
  // the legacy predictor: advective and viscous accelerations, scratch, previous acceleration,
  // predicted field, residual-norm partials; its history
  Buf<double> la, ld, lr, lprev, lstar, lres;
  Buf<double> ftau;  // the wall shear of the forces, per Gauss point
  bool l_has_prev = false;
  double l_prev_dt = 0;
  CcFlux flux{};
  // GMRES(30)
  static constexpr int GM_M = 30;
  Buf<double> V, gpart, gpart2, gd1, gd2, gwn, gbeta, gbn, gy, gone;
  Buf<int> gnv;
  Buf<GmresDev> gdev;
  // per-step diagnostics
  Buf<CcDiagDev> diag;
  CcDiagDev* host_diag = nullptr;
  // step graphs keyed by (dt, history, previous dt)
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    double dt = 0, prev_dt = 0;
    bool hist = false;
    long long outer = 0, per_step = 0, per_cycle = 0;
  };
  Graph graphs[3];
  int next_graph = 0;
  // optional phase events inside the step graph (environment GHOSTMAC_PHASE_TIMING=1 at create)
  static constexpr int NPHASE = 8;
  bool phase_on = false;
  cudaEvent_t pev[NPHASE + 1] = {};
  double phase_ms[NPHASE] = {};
};

namespace {

int guarded(gm_cc* c, const std::function<void()>& f) {
  try {
    f();
    return GM_OK;
  } catch (const CcFail& e) {
    if (c) c->err = e.msg;
    else gm_internal_set_error(e.msg.c_str());
    return e.cls;
  } catch (const std::exception& e) {
    if (c) c->err = e.what();
    else gm_internal_set_error(e.what());
    return GM_ECUDA;
  }
}

// copies n doubles from a host or device pointer into a device buffer
void copy_in(double* dst, const double* src, size_t n, cudaStream_t st) {
  CCK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, st));
}

// ---- momentum evaluation (five launches) ----------------------------------------------------
void momentum(gm_cc* c, bool adv, const double* X, const double* inl, double nu, int mode, double hdt, double* Y,
              double* Rout, cudaStream_t st, bool upwind = false) {
  const double rnu = c->rho * nu;
  const int64_t nv = (int64_t)(c->ny + 1) * (c->nx + 1);
  const bool shear = !adv && nu != 0.0;
  counted();
  if (adv && upwind) k_cc_flux<true, true><<<nblk(nv), CC_TPB, 0, st>>>(c->geo, X, inl, rnu, c->slip, c->flux);
  else if (adv) k_cc_flux<true><<<nblk(nv), CC_TPB, 0, st>>>(c->geo, X, inl, rnu, c->slip, c->flux);
  else k_cc_flux<false><<<nblk(nv), CC_TPB, 0, st>>>(c->geo, X, inl, rnu, c->slip, c->flux);
  const int nrows = adv ? c->fix.n_adv : c->fix.n_dif + (shear ? c->wall.n : 0);
  if (nrows > 0) {
    counted();
    const unsigned nb = nblk((int64_t)nrows * 32, 256);
    if (adv) k_cc_fix<true><<<nb, 256, 0, st>>>(c->geo, c->fix, c->wall, X, inl, rnu, c->rho, 0.0, c->flux);
    else k_cc_fix<false><<<nb, 256, 0, st>>>(c->geo, c->fix, c->wall, X, inl, rnu, c->rho, (-c->rho) * nu, c->flux);
  }
  counted();
  if (adv) k_cc_rhs<true><<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, c->flux, c->wall, X, 0, hdt, mode, Y, Rout);
  else k_cc_rhs<false><<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, c->flux, c->wall, X, shear ? 1 : 0, hdt, mode, Y, Rout);
}

void vec(gm_cc* c, int op, int64_t n, const double* a, const double* b, const double* cc, const double* d,
         const double* e, double s0, double s1, double* out, cudaStream_t st) {
  counted();
  k_cc_vec<<<nblk(n), CC_TPB, 0, st>>>(op, n, a, b, cc, d, e, s0, s1, out);
}

void grad(gm_cc* c, const double* P, double* Y, cudaStream_t st) {
  counted();
  k_cc_grad<<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, P, 1.0 / (c->rho * c->dx), 1.0 / (c->rho * c->dy), Y);
}

void maxdiff(gm_cc* c, int64_t n, const double* a, const double* b, const double* cc, double s, unsigned long long* out,
             cudaStream_t st) {
  counted();
  k_cc_maxdiff<<<std::min<unsigned>(nblk(n), 1216), CC_TPB, 0, st>>>(n, a, b, cc, s, out);
}

// project(q, step) of advance_ab2_cn (solver/cut_cell_solver.py:993-1002): q -> out (packed),
// phi; slot selects the control block entry and the predicted-divergence record
void project(gm_cc* c, const double* q, double step, double* out, double* phi, int slot, int rec, cudaStream_t st) {
  counted();
  k_cc_divrhs<<<nblk(c->psize), CC_TPB, 0, st>>>(c->geo, q, c->inlet.p, c->rho / step, c->B.p);
  gmi::pressure_solve(c->P, c->B.p, phi, slot);
  counted();
  k_cc_pdiv<<<std::min<unsigned>(nblk(c->psize), 1216), CC_TPB, 0, st>>>(c->geo, gmi::pressure_residual(c->P),
                                                                        step / c->rho, &c->diag.p->pdiv[rec]);
  counted();
  k_cc_correct<<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, q, phi, (step / c->rho) / c->dx, (step / c->rho) / c->dy, out);
}

// forces on the circle into diag->forces: the wall shear of every Gauss point (one warp each),
// then the one-block sums
void forces(gm_cc* c, const double* U, const double* P, double mu, cudaStream_t st) {
  if (c->wall.n > 0) {
    counted();
    k_cc_wall_tau<<<nblk((int64_t)c->wall.n * 32, 256), 256, 0, st>>>(c->wall, U, mu, c->ftau.p);
  }
  counted();
  k_cc_forces<<<1, CC_FORCE_THREADS, 0, st>>>(gmi::surface(c->P), c->wall, P, c->ftau.p, c->pb.p, c->diag.p->forces);
}

// H x = x - dt/2 L x on packed vectors (L the viscous operator without the inlet)
void hmatvec(gm_cc* c, const double* x, double dt, double* y, cudaStream_t st) {
  momentum(c, false, x, nullptr, c->nu, 1, 0.5 * dt, y, nullptr, st);
}

cudaGraphNode_t add_cond(cudaStream_t st, cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType type,
                         cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CCK(cudaGraphAddNode(&node, graph, deps, nullptr, nd, &cp));
  *body = cp.conditional.phGraph_out[0];
  CCK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return node;
}

// GMRES(30) for H x = b from x0 = x, captured on st (solver/time_integration.py:99-101:
// rtol 1e-12, atol 1e-13, restart 30, at most 100 cycles)
void gmres(gm_cc* c, const double* b, double* x, double dt, gm_cc::Graph& gr, cudaStream_t st) {
  const int m = gm_cc::GM_M;
  const int64_t n = c->F;
  double* V = c->V.p;
  auto vec_i = [&](int i) { return V + (int64_t)i * n; };
  cudaStream_t sb1 = gmi::body_stream(c->P, 0), sb2 = gmi::body_stream(c->P, 1);
  counted();
  k_gs_dot<1><<<GS_BLOCKS, GS_THREADS, 0, st>>>(b, n, b, c->gpart.p);
  counted();
  k_gs_sum<<<1, 32, 0, st>>>(c->gpart.p, c->gbn.p);
  cudaStreamCaptureStatus cs;
  cudaGraph_t top;
  CCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &top, nullptr, nullptr, nullptr));
  cudaGraphConditionalHandle cyc;
  CCK(cudaGraphConditionalHandleCreate(&cyc, top, 0, 0));
  launch_gm_init(c->gdev.p, c->gbn.p, cyc, st, 1e-12, 1e-13);
  cudaGraph_t cycle_body;
  add_cond(st, cyc, cudaGraphCondTypeWhile, &cycle_body);
  CCK(cudaStreamBeginCaptureToGraph(sb1, cycle_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const long long c1 = kernel_launch_count();
  hmatvec(c, x, dt, vec_i(1), sb1);
  counted();
  k_gs_residual<<<GS_BLOCKS, GS_THREADS, 0, sb1>>>(b, vec_i(1), n, vec_i(0), c->gpart.p);
  counted();
  k_gs_sum<<<1, 32, 0, sb1>>>(c->gpart.p, c->gbeta.p);
  GmresHandles hs{};
  hs.count = m;
  cudaGraph_t cyc_graph;
  CCK(cudaStreamGetCaptureInfo(sb1, &cs, nullptr, &cyc_graph, nullptr, nullptr, nullptr));
  for (int j = 0; j < m; ++j) CCK(cudaGraphConditionalHandleCreate(&hs.step[j], cyc_graph, 0, 0));
  launch_gm_cycle_begin(c->gdev.p, c->gbeta.p, hs, sb1);
  launch_gm_scale(vec_i(0), n, c->gdev.p, sb1);
  long long per_step = 0;
  for (int j = 0; j < m; ++j) {
    cudaGraph_t step_body;
    add_cond(sb1, hs.step[j], cudaGraphCondTypeIf, &step_body);
    CCK(cudaStreamBeginCaptureToGraph(sb2, step_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const long long c2 = kernel_launch_count();
    double* wv = vec_i(j + 1);
    hmatvec(c, vec_i(j), dt, wv, sb2);
    gs_step(j + 1, V, n, wv, c->gpart.p, c->gpart2.p, c->gd1.p, c->gd2.p, c->gwn.p, sb2);
    launch_gm_step_end(c->gdev.p, j, c->gd1.p, c->gd2.p, c->gwn.p, j + 1 < m ? hs.step[j + 1] : hs.step[0],
                       j + 1 < m, sb2);
    launch_gm_scale(wv, n, c->gdev.p, sb2);
    per_step = kernel_launch_count() - c2;
    cudaGraph_t done;
    CCK(cudaStreamEndCapture(sb2, &done));
  }
  launch_gm_cycle_end(c->gdev.p, c->gy.p, c->gnv.p, cyc, sb1);
  launch_multiaxpy_dev(V, n, c->gnv.p, c->gy.p, x, n, sb1);
  gr.per_step = per_step;
  gr.per_cycle = kernel_launch_count() - c1 - (long long)m * per_step;
  cudaGraph_t done1;
  CCK(cudaStreamEndCapture(sb1, &done1));
}

// One AB2/CN step (advance_ab2_cn, solver/cut_cell_solver.py:959-1015, with ab2_cn_step,
// solver/time_integration.py:7-145), captured on st.
void step_body(gm_cc* c, double dt, gm_cc::Graph& gr, cudaStream_t st) {
  const int64_t F = c->F, Pn = c->psize;
  const double* inl = c->inlet.p;
  auto mark = [&](int k) {
    // inside a capture an event record node needs the external flag (a plain record only
    // orders the captured streams)
    if (c->phase_on) CCK(cudaEventRecordWithFlags(c->pev[k], st, cudaEventRecordExternal));
  };
  mark(0);
  CCK(cudaMemsetAsync(c->diag.p, 0, offsetof(CcDiagDev, forces), st));
  counted();
  k_cc_pack<<<nblk(F), CC_TPB, 0, st>>>(c->geo, c->U.p, c->q0.p);
  momentum(c, true, c->q0.p, inl, 0.0, 0, 0.0, c->now.p, nullptr, st);
  mark(1);
  const double* pressure = c->has_history ? c->halfp.p : c->Pst.p;
  if (!c->has_history) {
    // projected midpoint start-up
    momentum(c, false, c->q0.p, inl, c->nu, 0, 0.0, c->d0.p, nullptr, st);
    grad(c, pressure, c->gp.p, st);
    vec(c, 0, F, c->q0.p, c->now.p, c->d0.p, c->gp.p, nullptr, 0.5 * dt, 0.0, c->mid.p, st);
    project(c, c->mid.p, 0.5 * dt, c->halfq.p, c->phi.p, S_P0, 0, st);
    momentum(c, true, c->halfq.p, inl, 0.0, 0, 0.0, c->expl.p, nullptr, st);
  } else {
    vec(c, 1, F, c->now.p, c->prev_adv.p, nullptr, nullptr, nullptr, dt / (2 * c->prev_dt), 0.0, c->expl.p, st);
  }
  momentum(c, false, c->zero.p, inl, c->nu, 0, 0.0, c->offset.p, nullptr, st);
  momentum(c, false, c->q0.p, inl, c->nu, 0, 0.0, c->dq.p, nullptr, st);
  grad(c, pressure, c->gp.p, st);
  vec(c, 2, F, c->q0.p, c->expl.p, c->dq.p, c->gp.p, c->offset.p, dt, 0.5 * dt, c->rhs.p, st);
  maxdiff(c, F, c->rhs.p, nullptr, nullptr, 0.0, &c->diag.p->rhs_max, st);
  CCK(cudaMemcpyAsync(c->star.p, c->q0.p, F * sizeof(double), cudaMemcpyDeviceToDevice, st));
  mark(2);
  gmres(c, c->rhs.p, c->star.p, dt, gr, st);
  mark(3);
  hmatvec(c, c->star.p, dt, c->w.p, st);
  maxdiff(c, F, c->w.p, c->rhs.p, nullptr, 0.0, &c->diag.p->mres, st);
  mark(4);
  project(c, c->star.p, dt, c->result.p, c->phi.p, S_P1, 1, st);
  mark(5);
  hmatvec(c, c->result.p, dt, c->action.p, st);
  vec(c, 3, F, c->result.p, c->rhs.p, c->action.p, nullptr, nullptr, 0.0, 0.0, c->tmp.p, st);
  mark(6);
  project(c, c->tmp.p, dt, c->w.p, c->inc.p, S_P2, 2, st);
  mark(7);
  const double factor = c->has_history ? dt / (dt + c->prev_dt) : 1.0;
  counted();
  k_cc_pressure_out<<<nblk(Pn), CC_TPB, 0, st>>>(Pn, pressure, c->inc.p, factor, c->halfp_next.p, c->Pst.p);
  grad(c, c->inc.p, c->gp.p, st);
  maxdiff(c, F, c->action.p, c->rhs.p, c->gp.p, dt, &c->diag.p->coupled, st);
  CCK(cudaMemcpyAsync(c->halfp.p, c->halfp_next.p, Pn * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CCK(cudaMemcpyAsync(c->prev_adv.p, c->now.p, F * sizeof(double), cudaMemcpyDeviceToDevice, st));
  counted();
  k_cc_unpack<<<nblk(F), CC_TPB, 0, st>>>(c->geo, c->result.p, inl, c->U.p);
  counted();
  k_cc_stepmax<<<std::min<unsigned>(nblk(F), 1216), CC_TPB, 0, st>>>(c->geo, c->U.p, &c->diag.p->divmax,
                                                                      &c->diag.p->umax, &c->diag.p->vmax);
  forces(c, c->U.p, c->Pst.p, c->nu * c->rho, st);
  mark(8);
}

gm_cc::Graph& step_graph(gm_cc* c, double dt) {
  for (auto& g : c->graphs)
    if (g.exec && g.dt == dt && g.hist == c->has_history && (!g.hist || g.prev_dt == c->prev_dt)) return g;
  gm_cc::Graph& gr = c->graphs[c->next_graph];
  c->next_graph = (c->next_graph + 1) % 3;
  if (gr.exec) { cudaGraphExecDestroy(gr.exec); gr.exec = nullptr; }
  cudaStream_t st = c->st;
  const long long c0 = kernel_launch_count();
  gmi::set_capturing(c->P, true);
  cudaGraph_t g = nullptr;
  CCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    step_body(c, dt, gr, st);
  } catch (...) {
    gmi::set_capturing(c->P, false);
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  gmi::set_capturing(c->P, false);
  CCK(cudaStreamEndCapture(st, &g));
  const long long captured = kernel_launch_count() - c0;
  kernel_launch_adjust(-captured);
  gr.outer = captured - (long long)gm_cc::GM_M * gr.per_step - gr.per_cycle;
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) throw CcFail(GM_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  gr.exec = ex;
  gr.dt = dt;
  gr.hist = c->has_history;
  gr.prev_dt = c->prev_dt;
  return gr;
}

// One step of the legacy cut-cell loop (solver/main.py:297-333, boundary='cut_cell',
// time_scheme='legacy'): the predictor on the stored state (its inlet column is the previous
// step's), compute_rhs / solve_pressure / apply_corrector (the projection of the AB2/CN path),
// p = phi, the step maxima and the forces on the true circle.
void legacy_body(gm_cc* c, double dt, bool centered, cudaStream_t st) {
  const int64_t F = c->F;
  CCK(cudaMemsetAsync(c->diag.p, 0, sizeof(CcDiagDev), st));
  momentum(c, true, c->U.p, nullptr, 0.0, 2, 0.0, c->la.p, c->lr.p, st, !centered);
  momentum(c, false, c->U.p, nullptr, c->nu, 2, 0.0, c->ld.p, c->lr.p, st);
  const bool ab2 = centered && c->l_has_prev;
  counted();
  k_cc_legacy_pred<<<nblk(F), CC_TPB, 0, st>>>(c->geo, c->U.p, c->la.p, c->ld.p, c->lprev.p, c->inlet.p, dt,
                                               ab2 ? dt / (2 * c->l_prev_dt) : 0.0, ab2 ? 1 : 0, c->lstar.p);
  project(c, c->lstar.p, dt, c->w.p, c->Pst.p, S_P1, 1, st);
  counted();
  k_cc_resnorm_part<<<CC_RES_BLOCKS, CC_TPB, 0, st>>>(c->geo, gmi::pressure_residual(c->P), c->lres.p);
  counted();
  k_cc_resnorm_fold<<<1, CC_TPB, 0, st>>>(c->lres.p, CC_RES_BLOCKS, &c->diag.p->res_linf, &c->diag.p->res_l2);
  counted();
  k_cc_unpack<<<nblk(F), CC_TPB, 0, st>>>(c->geo, c->w.p, c->inlet.p, c->U.p);
  counted();
  k_cc_stepmax<<<std::min<unsigned>(nblk(F), 1216), CC_TPB, 0, st>>>(c->geo, c->U.p, &c->diag.p->divmax,
                                                                      &c->diag.p->umax, &c->diag.p->vmax);
  forces(c, c->U.p, c->Pst.p, c->nu * c->rho, st);
}

double bits_to_double(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

// the initial state of solver/main.py:166-177 and its projection (:236-240)
void initial_state(gm_cc* c, const std::vector<double>& inlet, const int32_t* cell_type, const double* ax,
                   const double* ay) {
  const int nx = c->nx, ny = c->ny;
  std::vector<double> U(c->F, 0.0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i <= nx; ++i) U[(size_t)j * (nx + 1) + i] = inlet[j];
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      if (cell_type[(size_t)j * nx + i] == -1) {
        U[(size_t)j * (nx + 1) + i] = 0.0;
        U[(size_t)j * (nx + 1) + i + 1] = 0.0;
        U[c->usize + (size_t)j * nx + i] = 0.0;
        U[c->usize + (size_t)(j + 1) * nx + i] = 0.0;
      }
  for (int64_t f = 0; f < c->usize; ++f)
    if (ax[f] == 0.0) U[f] = 0.0;
  for (int64_t f = 0; f < c->vsize; ++f)
    if (ay[f] == 0.0) U[c->usize + f] = 0.0;
  cudaStream_t st = c->st;
  CCK(cudaMemcpyAsync(c->U.p, U.data(), U.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  // compute_rhs(u, v, 1, rho); solve; apply_corrector(u, v, u, v, phi, 1, rho, inlet): the
  // corrector reads the unpacked field (inlet column included)
  CCK(cudaMemsetAsync(c->diag.p, 0, sizeof(CcDiagDev), st));
  CCK(cudaMemsetAsync(gmi::control(c->P), 0, sizeof(StepCtl), st));
  counted();
  k_cc_divrhs<<<nblk(c->psize), CC_TPB, 0, st>>>(c->geo, c->U.p, nullptr, c->rho / 1.0, c->B.p);
  gmi::pressure_solve(c->P, c->B.p, c->phi.p, S_P1);
  counted();
  k_cc_pdiv<<<std::min<unsigned>(nblk(c->psize), 1216), CC_TPB, 0, st>>>(c->geo, gmi::pressure_residual(c->P),
                                                                        1.0 / c->rho, &c->diag.p->pdiv[1]);
  counted();
  k_cc_correct<<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, c->U.p, c->phi.p, (1.0 / c->rho) / c->dx, (1.0 / c->rho) / c->dy,
                                             c->tmp.p);
  counted();
  k_cc_unpack<<<nblk(c->F), CC_TPB, 0, st>>>(c->geo, c->tmp.p, c->inlet.p, c->U.p);
  CCK(cudaMemsetAsync(c->Pst.p, 0, c->psize * sizeof(double), st));
  std::string m;
  int rc = gmi::check(c->P, "initial projection", m);
  if (rc != GM_OK) throw CcFail(rc, m);
  CCK(cudaMemcpyAsync(c->host_diag, c->diag.p, sizeof(CcDiagDev), cudaMemcpyDeviceToHost, st));
  CCK(cudaStreamSynchronize(st));
  const double pd = bits_to_double(c->host_diag->pdiv[1]);
  if (!(pd < 1e-10))
    {
      char pbuf[96];
      std::snprintf(pbuf, sizeof pbuf, "Pressure residual exceeds divergence budget: %g", pd);
      throw CcFail(GM_ERUNTIME, pbuf);
    }
}

template <typename T>
std::vector<T> vec_of(const T* p, size_t n) {
  return p ? std::vector<T>(p, p + n) : std::vector<T>();
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

const char* gm_cc_last_error(const gm_cc* c) { return c ? c->err.c_str() : gm_last_error(nullptr); }

int gm_cc_create(const gm_cc_config* cfg, gm_cc** out) {
  if (!cfg || !out) { gm_internal_set_error("null argument"); return GM_EVALUE; }
  *out = nullptr;
  if (!cfg->ax || !cfg->ay || !cfg->ax_mid || !cfg->ay_mid || !cfg->ay_u || !cfg->ax_v || !cfg->cell_type ||
      !cfg->volume_fraction || !cfg->u_volume_fraction || !cfg->v_volume_fraction || !cfg->u_vol || !cfg->v_vol ||
      !cfg->u_vol_eff || !cfg->v_vol_eff) {
    gm_internal_set_error("missing geometry array");
    return GM_EVALUE;
  }
  auto c = std::make_unique<gm_cc>();
  gm_cc* C = c.get();
  const int nx = cfg->nx, ny = cfg->ny;
  gm::Geometry g;
  g.nx = nx; g.ny = ny; g.Lx = cfg->Lx; g.Ly = cfg->Ly; g.D = cfg->D; g.xc = cfg->xc; g.yc = cfg->yc;
  g.nu = cfg->nu; g.rho = cfg->rho; g.U_inf = cfg->U_inf; g.inflow = cfg->inflow; g.U_m = cfg->U_m;
  int ec = 0;
  if (!gm::build_cutcell_geometry(g, cfg->ax, cfg->ay, cfg->cell_type, cfg->volume_fraction, ec)) {
    gm_internal_set_error(g.error.c_str());
    return ec ? ec : GM_EVALUE;
  }
  C->nx = nx; C->ny = ny;
  C->usize = g.usize; C->vsize = g.vsize; C->psize = g.psize; C->F = g.usize + g.vsize;
  C->dx = g.dx; C->dy = g.dy; C->rho = cfg->rho; C->nu = cfg->nu; C->D = cfg->D; C->U_ref = g.U_ref;
  C->slip = cfg->slip_walls ? 1 : 0;
  std::vector<double> inlet = g.u_inlet;
  for (int64_t f : g.ui) C->act_idx.push_back(f);
  for (int64_t f : g.vi) C->act_idx.push_back(g.usize + f);
  C->n_active = (int64_t)C->act_idx.size();
  std::vector<uint8_t> act_u = g.act_u, act_v = g.act_v;
  std::string perr;
  int rc = gmi::pressure_create(std::move(g), &C->P, perr);
  if (rc != GM_OK) {
    gm_internal_set_error(perr.c_str());
    return rc;
  }
  rc = guarded(nullptr, [&] {
    cudaStream_t st = C->st = gmi::stream(C->P);
    const int64_t F = C->F, Pn = C->psize, us = C->usize;
    const int64_t nvert = (int64_t)(ny + 1) * (nx + 1);
    C->ax.upload(vec_of(cfg->ax, us), st);
    C->ay.upload(vec_of(cfg->ay, C->vsize), st);
    C->kappa.upload(vec_of(cfg->volume_fraction, Pn), st);
    {
      // folded factors of the structured kernels (see CcGeo)
      const double dx = C->dx, dy = C->dy, rho = cfg->rho;
      std::vector<double> cxx(Pn), cyy(Pn), axx(Pn), ayy(Pn), cxy(nvert), cyx(nvert), axy(nvert), ayx(nvert), aout(ny),
          ik(Pn);
      for (int64_t c = 0; c < Pn; ++c) {
        cxx[c] = cfg->ax_mid[c] * dy / dx;
        cyy[c] = cfg->ay_mid[c] * dx / dy;
        axx[c] = rho * cfg->ax_mid[c] * dy;
        ayy[c] = rho * cfg->ay_mid[c] * dx;
        ik[c] = cfg->cell_type[c] == 0 ? 1.0 / cfg->volume_fraction[c] : 1.0;
      }
      for (int64_t t = 0; t < nvert; ++t) {
        cxy[t] = cfg->ay_u[t] * dx / dy;
        cyx[t] = cfg->ax_v[t] * dy / dx;
        axy[t] = rho * cfg->ay_u[t] * dx;
        ayx[t] = rho * cfg->ax_v[t] * dy;
      }
      for (int j = 0; j < ny; ++j) aout[j] = rho * cfg->ax[(int64_t)j * (nx + 1) + nx] * dy;
      C->cxx.upload(cxx, st); C->cyy.upload(cyy, st); C->axx.upload(axx, st); C->ayy.upload(ayy, st);
      C->cxy.upload(cxy, st); C->cyx.upload(cyx, st); C->axy.upload(axy, st); C->ayx.upload(ayx, st);
      C->aout.upload(aout, st); C->ikappa.upload(ik, st);
    }
    C->cell_type.upload(vec_of(cfg->cell_type, Pn), st);
    C->inlet.upload(inlet, st);
    // face flags and volumes (fluid: fraction >= 0.3 and open; solid: covered face)
    std::vector<uint8_t> fl(F, 0);
    std::vector<double> vr(F, 1.0);
    for (int64_t f = 0; f < F; ++f) {
      const bool u = f < us;
      const int64_t k = u ? f : f - us;
      const double ap = u ? cfg->ax[k] : cfg->ay[k];
      const double fr = u ? cfg->u_volume_fraction[k] : cfg->v_volume_fraction[k];
      if (u ? act_u[k] : act_v[k]) fl[f] |= F_ACTIVE;
      if (fr >= 0.3 && ap > 0.0) fl[f] |= F_FLUID;
      if (ap == 0.0) fl[f] |= F_SOLID;
      vr[f] = 1.0 / (cfg->rho * (u ? cfg->u_vol[k] : cfg->v_vol[k]));
    }
    C->vol_rho.upload(vr, st);
    // merges in list order; a face written by several keeps the last
    std::vector<int32_t> mof(F, -1);
    std::vector<int64_t> ms, mm;
    std::vector<double> mv;
    auto add_merges = [&](int64_t n, const int64_t* tab, bool u) {
      const int64_t pitch = u ? nx + 1 : nx, off = u ? 0 : us;
      const double* eff = u ? cfg->u_vol_eff : cfg->v_vol_eff;
      for (int64_t k = 0; k < n; ++k) {
        const int64_t s = tab[4 * k] * pitch + tab[4 * k + 1], m = tab[4 * k + 2] * pitch + tab[4 * k + 3];
        const int32_t idx = (int32_t)ms.size();
        ms.push_back(off + s);
        mm.push_back(off + m);
        mv.push_back(1.0 / (cfg->rho * eff[s]));
        mof[off + s] = idx;
        mof[off + m] = idx;
      }
    };
    if (cfg->n_u_merge > 0 && !cfg->u_merge) throw CcFail(GM_EVALUE, "missing merge table");
    if (cfg->n_v_merge > 0 && !cfg->v_merge) throw CcFail(GM_EVALUE, "missing merge table");
    add_merges(cfg->n_u_merge, cfg->u_merge, true);
    add_merges(cfg->n_v_merge, cfg->v_merge, false);
    C->merge_of.upload(mof, st);
    C->ms.upload(ms, st);
    C->mm.upload(mm, st);
    C->mvol_rho.upload(mv, st);
    // covered-volume transfers: owners with their donors in order
    std::map<int64_t, std::vector<int64_t>> owners;
    std::vector<int64_t> donors;
    auto add_cov = [&](int64_t n, const int64_t* d, const int64_t* o, int64_t off) {
      for (int64_t k = 0; k < n; ++k) {
        owners[off + o[k]].push_back(off + d[k]);
        donors.push_back(off + d[k]);
      }
    };
    add_cov(cfg->n_u_covered, cfg->u_covered, cfg->u_owner, 0);
    add_cov(cfg->n_v_covered, cfg->v_covered, cfg->v_owner, us);
    std::vector<int64_t> own, optr{0}, odon;
    for (auto& kv : owners) {
      own.push_back(kv.first);
      odon.insert(odon.end(), kv.second.begin(), kv.second.end());
      optr.push_back((int64_t)odon.size());
    }
    C->own.upload(own, st);
    C->optr.upload(optr, st);
    C->odon.upload(odon, st);
    C->don.upload(donors, st);
    // wall: shear-rate rows, targets with their points in order
    const int64_t nw = cfg->n_wall;
    C->wptr.upload(vec_of(cfg->wall_rate.ptr, nw + 1), st);
    const int64_t wnnz = nw > 0 ? cfg->wall_rate.ptr[nw] : 0;
    C->wcol.upload(vec_of(cfg->wall_rate.col, wnnz), st);
    C->wval.upload(vec_of(cfg->wall_rate.val, wnnz), st);
    C->wtx.upload(vec_of(cfg->wall_tx, nw), st);
    C->wty.upload(vec_of(cfg->wall_ty, nw), st);
    C->wds.upload(vec_of(cfg->wall_ds, nw), st);
    C->tau.alloc(std::max<int64_t>(1, nw));
    std::map<int64_t, std::vector<int32_t>> targets;
    for (int64_t k = 0; k < nw; ++k) targets[cfg->wall_u[k]].push_back((int32_t)k);
    std::map<int64_t, std::vector<int32_t>> vtargets;
    for (int64_t k = 0; k < nw; ++k) vtargets[us + cfg->wall_v[k]].push_back((int32_t)k);
    std::vector<int64_t> tgt, tptr{0};
    std::vector<int32_t> tk;
    for (auto* mp : {&targets, &vtargets})
      for (auto& kv : *mp) {
        tgt.push_back(kv.first);
        tk.insert(tk.end(), kv.second.begin(), kv.second.end());
        tptr.push_back((int64_t)tk.size());
      }
    C->tgt.upload(tgt, st);
    C->tptr.upload(tptr, st);
    C->tk.upload(tk, st);
    // faces with wall shear, owners and donors: the sorted list the fused right-hand side
    // kernel searches (flag F_AUX)
    std::map<int64_t, std::array<int32_t, 3>> aux;  // face -> target entry, owner entry, donor
    for (size_t t = 0; t < tgt.size(); ++t) aux.emplace(tgt[t], std::array<int32_t, 3>{-1, -1, 0})
                                               .first->second[0] = (int32_t)t;
    for (size_t o = 0; o < own.size(); ++o) aux.emplace(own[o], std::array<int32_t, 3>{-1, -1, 0})
                                               .first->second[1] = (int32_t)o;
    for (int64_t d : donors) aux.emplace(d, std::array<int32_t, 3>{-1, -1, 0}).first->second[2] = 1;
    std::vector<int64_t> aux_face;
    std::vector<int32_t> aux_tgt, aux_own;
    std::vector<uint8_t> aux_don;
    for (auto& kv : aux) {
      aux_face.push_back(kv.first);
      aux_tgt.push_back(kv.second[0]);
      aux_own.push_back(kv.second[1]);
      aux_don.push_back((uint8_t)kv.second[2]);
      fl[kv.first] |= F_AUX;
    }
    C->flags.upload(fl, st);
    C->aux_face.upload(aux_face, st);
    C->aux_tgt.upload(aux_tgt, st);
    C->aux_own.upload(aux_own, st);
    C->aux_don.upload(aux_don, st);
    // curved-face overrides of the four families
    std::vector<uint8_t> dfam, afam;
    std::vector<int64_t> dface, dptr{0}, dcol, aface, apptr{0}, uptr{0}, ucol, vptr{0}, vcol;
    std::vector<double> dval, uval, vval, alen;
    for (int fm = 0; fm < 4; ++fm) {
      const gm_cc_faces& fc = cfg->faces[fm];
      for (int64_t r = 0; r < fc.n_dif; ++r) {
        dfam.push_back((uint8_t)fm);
        dface.push_back(fc.dif_face[r]);
        for (int64_t e = fc.dif_grad.ptr[r]; e < fc.dif_grad.ptr[r + 1]; ++e) {
          dcol.push_back(fc.dif_grad.col[e]);
          dval.push_back(fc.dif_grad.val[e]);
        }
        dptr.push_back((int64_t)dcol.size());
      }
      // advective faces: the Gauss points of face r are those with patch == r (contiguous)
      int64_t p = 0;
      for (int64_t r = 0; r < fc.n_adv; ++r) {
        afam.push_back((uint8_t)fm);
        aface.push_back(fc.adv_face[r]);
        while (p < fc.n_adv_points && fc.adv_patch[p] == r) {
          for (int64_t e = fc.adv_u.ptr[p]; e < fc.adv_u.ptr[p + 1]; ++e) {
            ucol.push_back(fc.adv_u.col[e]);
            uval.push_back(fc.adv_u.val[e]);
          }
          uptr.push_back((int64_t)ucol.size());
          for (int64_t e = fc.adv_v.ptr[p]; e < fc.adv_v.ptr[p + 1]; ++e) {
            vcol.push_back(fc.adv_v.col[e]);
            vval.push_back(fc.adv_v.val[e]);
          }
          vptr.push_back((int64_t)vcol.size());
          alen.push_back(fc.adv_len[p]);
          ++p;
        }
        apptr.push_back((int64_t)alen.size());
      }
      if (p != fc.n_adv_points) throw CcFail(GM_EVALUE, "advective face points must be grouped by face in order");
    }
    C->dfam.upload(dfam, st); C->dface.upload(dface, st); C->dptr.upload(dptr, st);
    C->dcol.upload(dcol, st); C->dval.upload(dval, st);
    C->afam.upload(afam, st); C->aface.upload(aface, st); C->apptr.upload(apptr, st);
    C->uptr.upload(uptr, st); C->ucol.upload(ucol, st); C->uval.upload(uval, st);
    C->vptr.upload(vptr, st); C->vcol.upload(vcol, st); C->vval.upload(vval, st);
    C->alen.upload(alen, st);
    // kernel arguments
    CcGeo& G = C->geo;
    G.nx = nx; G.ny = ny; G.usize = us; G.vsize = C->vsize; G.psize = Pn; G.F = F; G.dx = C->dx; G.dy = C->dy;
    G.idx = 1.0 / C->dx; G.idy = 1.0 / C->dy;
    G.ax = C->ax.p; G.ay = C->ay.p;
    G.cxx = C->cxx.p; G.cyy = C->cyy.p; G.cxy = C->cxy.p; G.cyx = C->cyx.p;
    G.axx = C->axx.p; G.ayy = C->ayy.p; G.axy = C->axy.p; G.ayx = C->ayx.p; G.aout = C->aout.p;
    G.flags = C->flags.p; G.cell_type = C->cell_type.p; G.kappa = C->kappa.p; G.ikappa = C->ikappa.p;
    G.ivol_rho = C->vol_rho.p; G.merge_of = C->merge_of.p; G.ms = C->ms.p; G.mm = C->mm.p;
    G.imvol_rho = C->mvol_rho.p;
    CcFix& X = C->fix;
    X.n_dif = (int)dface.size(); X.dfam = C->dfam.p; X.dface = C->dface.p; X.dptr = C->dptr.p; X.dcol = C->dcol.p;
    X.dval = C->dval.p;
    X.n_adv = (int)aface.size(); X.afam = C->afam.p; X.aface = C->aface.p; X.apptr = C->apptr.p;
    X.uptr = C->uptr.p; X.ucol = C->ucol.p; X.uval = C->uval.p; X.vptr = C->vptr.p; X.vcol = C->vcol.p;
    X.vval = C->vval.p; X.alen = C->alen.p;
    CcWall& W = C->wall;
    W.n = (int)nw; W.ptr = C->wptr.p; W.col = C->wcol.p; W.val = C->wval.p; W.tx = C->wtx.p; W.ty = C->wty.p;
    W.ds = C->wds.p; W.n_tgt = (int)tgt.size(); W.tgt = C->tgt.p; W.tptr = C->tptr.p; W.tk = C->tk.p;
    W.n_own = (int)own.size(); W.own = C->own.p; W.optr = C->optr.p; W.odon = C->odon.p;
    W.n_don = (int)donors.size(); W.don = C->don.p; W.tau = C->tau.p;
    W.n_aux = (int)aux_face.size(); W.aux_face = C->aux_face.p; W.aux_tgt = C->aux_tgt.p; W.aux_own = C->aux_own.p;
    W.aux_don = C->aux_don.p;
    // state and work arrays
    for (Buf<double>* b : {&C->U, &C->prev_adv, &C->q0, &C->now, &C->d0, &C->gp, &C->mid, &C->halfq, &C->expl,
                           &C->offset, &C->dq, &C->rhs, &C->star, &C->w, &C->result, &C->action, &C->tmp, &C->zero,
                           &C->Rw, &C->la, &C->ld, &C->lr, &C->lprev, &C->lstar}) {
      b->alloc(F);
      b->zero(st);
    }
    for (Buf<double>* b : {&C->Pst, &C->halfp, &C->halfp_next, &C->B, &C->phi, &C->inc}) {
      b->alloc(Pn);
      b->zero(st);
    }
    C->fxx.alloc(Pn); C->fyy.alloc(Pn); C->fxy.alloc(nvert); C->fyx.alloc(nvert);
    C->flux = CcFlux{C->fxx.p, C->fxy.p, C->fyx.p, C->fyy.p};
    C->pb.alloc(std::max(1, gmi::surface(C->P).n));
    const int m = gm_cc::GM_M;
    C->V.alloc((size_t)(m + 1) * F);
    C->gpart.alloc(std::max<size_t>((size_t)GS_BLOCKS * GS_MAXV, (size_t)multidot_blocks(F) * 64));
    C->gpart2.alloc((size_t)GS_BLOCKS * GS_MAXV);
    for (Buf<double>* b : {&C->gd1, &C->gd2, &C->gy}) b->alloc(64);
    for (Buf<double>* b : {&C->gwn, &C->gbeta, &C->gbn, &C->gone}) b->alloc(1);
    C->gnv.alloc(1);
    C->gdev.alloc(1);
    const double one = 1.0;
    CCK(cudaMemcpyAsync(C->gone.p, &one, sizeof one, cudaMemcpyHostToDevice, st));
    C->lres.alloc(2 * CC_RES_BLOCKS);
    C->ftau.alloc(std::max<int64_t>(1, nw));
    C->diag.alloc(1);
    CCK(cudaMallocHost(&C->host_diag, sizeof(CcDiagDev)));
    C->d_act.upload(C->act_idx, st);
    if (const char* e = std::getenv("GHOSTMAC_PHASE_TIMING")) C->phase_on = e[0] == '1';
    if (C->phase_on)
      for (auto& e : C->pev) CCK(cudaEventCreate(&e));
    initial_state(C, inlet, cfg->cell_type, cfg->ax, cfg->ay);
  });
  if (rc != GM_OK) {
    gm_cc_destroy(c.release());
    return rc;
  }
  *out = c.release();
  return GM_OK;
}

int gm_cc_destroy(gm_cc* c) {
  if (!c) return GM_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  for (auto& g : c->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (c->host_diag) cudaFreeHost(c->host_diag);
  for (auto& e : c->pev)
    if (e) cudaEventDestroy(e);
  gm_handle* P = c->P;
  delete c;  // device buffers first, then the pressure handle and its stream
  if (P) gmi::pressure_destroy(P);
  return GM_OK;
}

int gm_cc_get_sizes(const gm_cc* c, gm_sizes* o) {
  if (!c || !o) return GM_EVALUE;
  std::memset(o, 0, sizeof *o);
  o->nx = c->nx; o->ny = c->ny; o->usize = c->usize; o->vsize = c->vsize; o->psize = c->psize;
  const gm::Geometry& g = gmi::geometry(c->P);
  o->nu_active = (int64_t)g.ui.size(); o->nv_active = (int64_t)g.vi.size(); o->np_active = (int64_t)g.pi.size();
  o->qsize = c->n_active;
  o->n_surface = g.n_surface;
  o->rank_p = gmi::schur_rank(c->P);
  o->dx = c->dx; o->dy = c->dy; o->U_ref = c->U_ref;
  return GM_OK;
}

int gm_cc_get_indices(const gm_cc* c, int64_t* ui, int64_t* vi, int64_t* pi) {
  if (!c) return GM_EVALUE;
  const gm::Geometry& g = gmi::geometry(c->P);
  if (ui) std::copy(g.ui.begin(), g.ui.end(), ui);
  if (vi) std::copy(g.vi.begin(), g.vi.end(), vi);
  if (pi) std::copy(g.pi.begin(), g.pi.end(), pi);
  return GM_OK;
}

int gm_cc_get_surface_points(const gm_cc* c, double* yx) {
  if (!c || !yx) return GM_EVALUE;
  const gm::Geometry& g = gmi::geometry(c->P);
  for (int k = 0; k < g.n_surface; ++k) {
    yx[2 * k] = g.surf_y[k];
    yx[2 * k + 1] = g.surf_x[k];
  }
  return GM_OK;
}

int gm_cc_set_state(gm_cc* c, const double* u, const double* v, const double* p) {
  if (!c) return GM_EVALUE;
  return guarded(c, [&] {
    if (u) copy_in(c->U.p, u, c->usize, c->st);
    if (v) copy_in(c->U.p + c->usize, v, c->vsize, c->st);
    if (p) copy_in(c->Pst.p, p, c->psize, c->st);
    CCK(cudaStreamSynchronize(c->st));
  });
}

int gm_cc_get_state(gm_cc* c, double* u, double* v, double* p) {
  if (!c) return GM_EVALUE;
  return guarded(c, [&] {
    if (u) CCK(cudaMemcpyAsync(u, c->U.p, c->usize * sizeof(double), cudaMemcpyDefault, c->st));
    if (v) CCK(cudaMemcpyAsync(v, c->U.p + c->usize, c->vsize * sizeof(double), cudaMemcpyDefault, c->st));
    if (p) CCK(cudaMemcpyAsync(p, c->Pst.p, c->psize * sizeof(double), cudaMemcpyDefault, c->st));
    CCK(cudaStreamSynchronize(c->st));
  });
}

int gm_cc_set_inlet(gm_cc* c, const double* u_inlet) {
  if (!c || !u_inlet) return GM_EVALUE;
  return guarded(c, [&] {
    copy_in(c->inlet.p, u_inlet, c->ny, c->st);
    CCK(cudaStreamSynchronize(c->st));
  });
}

int gm_cc_set_history(gm_cc* c, int32_t has_history, const double* prev_adv, const double* half_p, double prev_dt) {
  if (!c) return GM_EVALUE;
  return guarded(c, [&] {
    if (has_history) {
      if (!prev_adv || !half_p || !(std::isfinite(prev_dt) && prev_dt > 0))
        throw CcFail(GM_EVALUE, "AB2 history requires a finite positive previous timestep");
      // packed previous advection -> face grid
      std::vector<double> q((size_t)c->n_active), grid((size_t)c->F, 0.0);
      CCK(cudaMemcpy(q.data(), prev_adv, q.size() * sizeof(double), cudaMemcpyDefault));
      for (int64_t k = 0; k < c->n_active; ++k) grid[(size_t)c->act_idx[k]] = q[(size_t)k];
      CCK(cudaMemcpyAsync(c->prev_adv.p, grid.data(), grid.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
      copy_in(c->halfp.p, half_p, c->psize, c->st);
      c->prev_dt = prev_dt;
    }
    c->has_history = has_history != 0;
    CCK(cudaStreamSynchronize(c->st));
  });
}

int gm_cc_get_history(gm_cc* c, int32_t* has_history, double* prev_adv, double* half_p, double* prev_dt) {
  if (!c) return GM_EVALUE;
  return guarded(c, [&] {
    if (has_history) *has_history = c->has_history ? 1 : 0;
    if (prev_dt) *prev_dt = c->prev_dt;
    if (!c->has_history) return;
    if (prev_adv) {
      std::vector<double> grid((size_t)c->F);
      CCK(cudaMemcpyAsync(grid.data(), c->prev_adv.p, grid.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
      CCK(cudaStreamSynchronize(c->st));
      std::vector<double> q((size_t)c->n_active);
      for (int64_t k = 0; k < c->n_active; ++k) q[(size_t)k] = grid[(size_t)c->act_idx[k]];
      CCK(cudaMemcpy(prev_adv, q.data(), q.size() * sizeof(double), cudaMemcpyDefault));
    }
    if (half_p) CCK(cudaMemcpyAsync(half_p, c->halfp.p, c->psize * sizeof(double), cudaMemcpyDefault, c->st));
    CCK(cudaStreamSynchronize(c->st));
  });
}

int gm_cc_step(gm_cc* c, double dt, int32_t n_steps, double start_time, gm_cc_step_diag* diag) {
  if (!c) return GM_EVALUE;
  if (!(std::isfinite(dt) && dt > 0) || n_steps <= 0) {
    c->err = "Finite fields and a positive timestep are required";
    return GM_EVALUE;
  }
  return guarded(c, [&] {
    cudaStream_t st = c->st;
    for (int32_t k = 0; k < n_steps; ++k) {
      gm_cc::Graph& gr = step_graph(c, dt);
      CCK(cudaMemsetAsync(gmi::control(c->P), 0, sizeof(StepCtl), st));
      CCK(cudaGraphLaunch(gr.exec, st));
      int r[5];
      CCK(cudaMemcpyAsync(r, &c->gdev.p->jend, sizeof r, cudaMemcpyDeviceToHost, st));
      CCK(cudaMemcpyAsync(c->host_diag, c->diag.p, sizeof(CcDiagDev), cudaMemcpyDeviceToHost, st));
      std::string m;
      const int prc = gmi::check(c->P, "cut-cell step", m);  // synchronises the stream
      const int cycles = r[1], its = r[2], converged = r[3];
      if (c->phase_on)
        for (int q = 0; q < gm_cc::NPHASE; ++q) {
          float ms = 0.f;
          c->phase_ms[q] = cudaEventElapsedTime(&ms, c->pev[q], c->pev[q + 1]) == cudaSuccess ? ms : 0.0;
        }
      kernel_launch_adjust(gr.outer + (long long)cycles * gr.per_cycle + (long long)its * gr.per_step);
      const CcDiagDev& d = *c->host_diag;
      gm_cc_step_diag out{};
      out.time = start_time + (k + 1) * dt;
      out.dt = dt;
      out.momentum_iterations = its;
      out.pressure_residual_linf = out.pressure_residual_l2 = std::nan("");
      out.momentum_residual_linf = bits_to_double(d.mres);
      out.coupled_momentum_residual_linf = bits_to_double(d.coupled);
      out.predicted_divergence = std::max(bits_to_double(d.pdiv[1]), bits_to_double(d.pdiv[2]));
      if (!c->has_history) out.predicted_divergence = std::max(out.predicted_divergence, bits_to_double(d.pdiv[0]));
      out.pressure_solves = c->has_history ? 2 : 3;
      out.max_divergence = bits_to_double(d.divmax);
      out.cfl = dt * (bits_to_double(d.umax) / c->dx + bits_to_double(d.vmax) / c->dy);
      for (int q = 0; q < 6; ++q) out.forces[q] = d.forces[q];
      const double denom = 0.5 * c->rho * (c->U_ref * c->U_ref) * c->D;
      out.cd = d.forces[0] / denom;
      out.cl = d.forces[1] / denom;
      out.cd_pressure = d.forces[2] / denom;
      out.cd_viscous = d.forces[4] / denom;
      out.cl_pressure = d.forces[3] / denom;
      out.cl_viscous = d.forces[5] / denom;
      // the step has replaced the state; history for the next step
      c->has_history = true;
      c->prev_dt = dt;
      int cls = GM_OK, gate = 0;
      std::string msg;
      const double rmax = bits_to_double(d.rhs_max);
      char buf[128];  // messages in the reference's %g form
      if (prc != GM_OK) { cls = prc; gate = GM_GATE_PRESSURE; msg = m; }
      else if (!(out.predicted_divergence < 1e-10)) {
        std::snprintf(buf, sizeof buf, "Pressure residual exceeds divergence budget: %g", out.predicted_divergence);
        cls = GM_ERUNTIME; gate = GM_GATE_PRESSURE; msg = buf;
      } else if (!converged || !(out.momentum_residual_linf <= 1e-10 * std::max(1.0, rmax)) ||
                 !std::isfinite(out.momentum_residual_linf)) {
        std::snprintf(buf, sizeof buf, "CN momentum solve failed: info=%d, residual=%g", converged ? 0 : 1,
                      out.momentum_residual_linf);
        cls = GM_ERUNTIME; gate = GM_GATE_MOMENTUM; msg = buf;
      } else if (!std::isfinite(out.cd) || !std::isfinite(out.cl)) {
        std::snprintf(buf, sizeof buf, "Non-finite force at t=%g; results not saved", out.time);
        cls = GM_EFLOAT; gate = GM_GATE_FORCE; msg = buf;
      } else if (!(out.max_divergence < 1e-10) || !(out.cfl < 0.5)) {
        cls = GM_ERUNTIME; gate = GM_GATE_STEP;
        msg = "Step failed the divergence/CFL acceptance gate";
      }
      out.status = cls;
      out.gate = gate;
      if (diag) diag[k] = out;
      if (cls != GM_OK) throw CcFail(cls, msg);
    }
  });
}

int gm_cc_legacy_step(gm_cc* c, double dt, int32_t n_steps, double start_time, int32_t centered,
                      gm_cc_step_diag* diag) {
  if (!c) return GM_EVALUE;
  if (!(std::isfinite(dt) && dt > 0) || n_steps <= 0) {
    c->err = "Finite fields and a positive timestep are required";
    return GM_EVALUE;
  }
  return guarded(c, [&] {
    cudaStream_t st = c->st;
    for (int32_t k = 0; k < n_steps; ++k) {
      CCK(cudaMemsetAsync(gmi::control(c->P), 0, sizeof(StepCtl), st));
      legacy_body(c, dt, centered != 0, st);
      CCK(cudaGetLastError());
      CCK(cudaMemcpyAsync(c->host_diag, c->diag.p, sizeof(CcDiagDev), cudaMemcpyDeviceToHost, st));
      std::string m;
      const int prc = gmi::check(c->P, "cut-cell legacy step", m);  // synchronises the stream
      // the predictor has replaced its history (solver/cut_cell_solver.py:1029-1031)
      c->l_has_prev = true;
      c->l_prev_dt = dt;
      const CcDiagDev& d = *c->host_diag;
      gm_cc_step_diag out{};
      out.time = start_time + (k + 1) * dt;
      out.dt = dt;
      out.predicted_divergence = bits_to_double(d.pdiv[1]);
      out.pressure_solves = 1;
      out.max_divergence = bits_to_double(d.divmax);
      out.cfl = dt * (bits_to_double(d.umax) / c->dx + bits_to_double(d.vmax) / c->dy);
      for (int q = 0; q < 6; ++q) out.forces[q] = d.forces[q];
      const double denom = 0.5 * c->rho * (c->U_ref * c->U_ref) * c->D;
      out.cd = d.forces[0] / denom;
      out.cl = d.forces[1] / denom;
      out.cd_pressure = d.forces[2] / denom;
      out.cd_viscous = d.forces[4] / denom;
      out.cl_pressure = d.forces[3] / denom;
      out.cl_viscous = d.forces[5] / denom;
      out.pressure_residual_linf = d.res_linf;
      out.pressure_residual_l2 = d.res_l2;
      int cls = GM_OK, gate = 0;
      std::string msg;
      char buf[96];
      if (prc != GM_OK) { cls = prc; gate = GM_GATE_PRESSURE; msg = m; }
      else if (!(out.predicted_divergence < 1e-10)) {
        std::snprintf(buf, sizeof buf, "Pressure residual exceeds divergence budget: %g", out.predicted_divergence);
        cls = GM_ERUNTIME; gate = GM_GATE_PRESSURE; msg = buf;
      } else if (!std::isfinite(out.cd) || !std::isfinite(out.cl)) {
        std::snprintf(buf, sizeof buf, "Non-finite force at t=%g; results not saved", out.time);
        cls = GM_EFLOAT; gate = GM_GATE_FORCE; msg = buf;
      }
      out.status = cls;
      out.gate = gate;
      if (diag) diag[k] = out;
      if (cls != GM_OK) throw CcFail(cls, msg);
    }
  });
}

int gm_cc_set_legacy_history(gm_cc* c, int32_t has_history, const double* prev_accel, double prev_dt) {
  if (!c) return GM_EVALUE;
  if (has_history && (!prev_accel || !(std::isfinite(prev_dt) && prev_dt > 0))) {
    c->err = "Incomplete predictor checkpoint history";
    return GM_EVALUE;
  }
  return guarded(c, [&] {
    if (has_history) copy_in(c->lprev.p, prev_accel, c->F, c->st);
    else CCK(cudaMemsetAsync(c->lprev.p, 0, c->F * sizeof(double), c->st));
    CCK(cudaStreamSynchronize(c->st));
    c->l_has_prev = has_history != 0;
    c->l_prev_dt = has_history ? prev_dt : 0.0;
  });
}

int gm_cc_get_legacy_history(gm_cc* c, int32_t* has_history, double* prev_accel, double* prev_dt) {
  if (!c) return GM_EVALUE;
  return guarded(c, [&] {
    if (has_history) *has_history = c->l_has_prev ? 1 : 0;
    if (prev_dt) *prev_dt = c->l_prev_dt;
    if (prev_accel) {
      CCK(cudaMemcpyAsync(prev_accel, c->lprev.p, c->F * sizeof(double), cudaMemcpyDefault, c->st));
      CCK(cudaStreamSynchronize(c->st));
    }
  });
}

int gm_cc_phase_timing(const gm_cc* c, double out[8]) {
  if (!c || !out) return GM_EVALUE;
  for (int q = 0; q < gm_cc::NPHASE; ++q) out[q] = c->phase_ms[q];
  return GM_OK;
}

int gm_cc_apply(gm_cc* c, int32_t op, double param, const double* x, double* y, double* y2) {
  if (!c || !x || !y) return GM_EVALUE;
  return guarded(c, [&] {
    cudaStream_t st = c->st;
    const int64_t F = c->F, Pn = c->psize;
    auto gather = [&](const double* grid, double* outp) {
      std::vector<double> g((size_t)F), q((size_t)c->n_active);
      CCK(cudaMemcpyAsync(g.data(), grid, F * sizeof(double), cudaMemcpyDeviceToHost, st));
      CCK(cudaStreamSynchronize(st));
      for (int64_t k = 0; k < c->n_active; ++k) q[(size_t)k] = g[(size_t)c->act_idx[k]];
      CCK(cudaMemcpy(outp, q.data(), q.size() * sizeof(double), cudaMemcpyDefault));
    };
    auto scatter = [&](const double* q, double* grid) {
      std::vector<double> h((size_t)c->n_active), g((size_t)F, 0.0);
      CCK(cudaMemcpy(h.data(), q, h.size() * sizeof(double), cudaMemcpyDefault));
      for (int64_t k = 0; k < c->n_active; ++k) g[(size_t)c->act_idx[k]] = h[(size_t)k];
      CCK(cudaMemcpyAsync(grid, g.data(), F * sizeof(double), cudaMemcpyHostToDevice, st));
    };
    switch (op) {
      case GM_CC_OP_MOMENTUM_ADVECTION:
      case GM_CC_OP_MOMENTUM_ADVECTION_UPWIND:
      case GM_CC_OP_MOMENTUM_DIFFUSION: {
        copy_in(c->tmp.p, x, F, st);
        const bool adv = op != GM_CC_OP_MOMENTUM_DIFFUSION;
        momentum(c, adv, c->tmp.p, nullptr, adv ? 0.0 : param, 2, 0.0, c->w.p, c->action.p, st,
                 op == GM_CC_OP_MOMENTUM_ADVECTION_UPWIND);
        CCK(cudaMemcpyAsync(y, c->w.p, F * sizeof(double), cudaMemcpyDefault, st));
        if (y2) CCK(cudaMemcpyAsync(y2, c->action.p, F * sizeof(double), cudaMemcpyDefault, st));
        break;
      }
      case GM_CC_OP_ADVECTION:
      case GM_CC_OP_DIFFUSION: {
        scatter(x, c->tmp.p);
        const bool adv = op == GM_CC_OP_ADVECTION;
        momentum(c, adv, c->tmp.p, c->inlet.p, adv ? 0.0 : c->nu, 0, 0.0, c->w.p, nullptr, st);
        gather(c->w.p, y);
        break;
      }
      case GM_CC_OP_H_MATVEC: {
        scatter(x, c->tmp.p);
        hmatvec(c, c->tmp.p, param, c->w.p, st);
        gather(c->w.p, y);
        break;
      }
      case GM_CC_OP_PROJECT: {
        scatter(x, c->tmp.p);
        CCK(cudaMemsetAsync(gmi::control(c->P), 0, sizeof(StepCtl), st));
        CCK(cudaMemsetAsync(c->diag.p, 0, sizeof(CcDiagDev), st));
        project(c, c->tmp.p, param, c->w.p, c->phi.p, S_P1, 1, st);
        std::string m;
        int rc = gmi::check(c->P, "project", m);
        if (rc != GM_OK) throw CcFail(rc, m);
        gather(c->w.p, y);
        if (y2) CCK(cudaMemcpyAsync(y2, c->phi.p, Pn * sizeof(double), cudaMemcpyDefault, st));
        break;
      }
      case GM_CC_OP_PRESSURE_SOLVE: {
        // solve_pressure(rhs, dt = param, rho): A phi = rhs on the fluid cells, phi = 0 on covered
        copy_in(c->B.p, x, Pn, st);
        counted();
        k_cc_scale_rhs<<<nblk(Pn), CC_TPB, 0, st>>>(c->geo, c->B.p);
        CCK(cudaMemsetAsync(gmi::control(c->P), 0, sizeof(StepCtl), st));
        CCK(cudaMemsetAsync(c->diag.p, 0, sizeof(CcDiagDev), st));
        gmi::pressure_solve(c->P, c->B.p, c->phi.p, S_P1);
        counted();
        k_cc_pdiv<<<std::min<unsigned>(nblk(Pn), 1216), CC_TPB, 0, st>>>(
            c->geo, gmi::pressure_residual(c->P), param / c->rho, &c->diag.p->pdiv[1]);
        std::string m;
        int rc = gmi::check(c->P, "pressure solve", m);
        if (rc != GM_OK) throw CcFail(rc, m);
        CCK(cudaMemcpyAsync(c->host_diag, c->diag.p, sizeof(CcDiagDev), cudaMemcpyDeviceToHost, st));
        CCK(cudaStreamSynchronize(st));
        const double pd = bits_to_double(c->host_diag->pdiv[1]);
        if (!(pd < 1e-10)) {
      char pbuf[96];
      std::snprintf(pbuf, sizeof pbuf, "Pressure residual exceeds divergence budget: %g", pd);
      throw CcFail(GM_ERUNTIME, pbuf);
    }
        CCK(cudaMemcpyAsync(y, c->phi.p, Pn * sizeof(double), cudaMemcpyDefault, st));
        break;
      }
      default:
        throw CcFail(GM_EVALUE, "unknown cut-cell operator");
    }
    CCK(cudaGetLastError());
    CCK(cudaStreamSynchronize(st));
  });
}

int gm_cc_surface_forces(gm_cc* c, const double* u, const double* v, const double* p, double mu, double out[6]) {
  if (!c || !u || !v || !p || !out) return GM_EVALUE;
  return guarded(c, [&] {
    cudaStream_t st = c->st;
    copy_in(c->tmp.p, u, c->usize, st);
    copy_in(c->tmp.p + c->usize, v, c->vsize, st);
    copy_in(c->B.p, p, c->psize, st);
    forces(c, c->tmp.p, c->B.p, mu, st);
    CCK(cudaMemcpyAsync(out, c->diag.p->forces, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CCK(cudaStreamSynchronize(st));
  });
}

int gm_cc_divergence_stats(gm_cc* c, const double* u, const double* v, double out[3]) {
  if (!c || !out) return GM_EVALUE;
  return guarded(c, [&] {
    cudaStream_t st = c->st;
    const double* U = c->U.p;
    if (u || v) {
      copy_in(c->tmp.p, u ? u : c->U.p, c->usize, st);
      copy_in(c->tmp.p + c->usize, v ? v : c->U.p + c->usize, c->vsize, st);
      U = c->tmp.p;
    }
    counted();
    k_cc_divstats<<<1, CC_FORCE_THREADS, 0, st>>>(c->geo, U, c->pb.p);
    double r[4];
    CCK(cudaMemcpyAsync(r, c->pb.p, sizeof r, cudaMemcpyDeviceToHost, st));
    CCK(cudaStreamSynchronize(st));
    out[0] = r[0];
    out[1] = r[2] > 0 ? std::sqrt(r[1] / r[2]) : 0.0;
    out[2] = r[3];
  });
}

}  // extern "C"

// =============================================================================================
// the pressure system alone (the legacy staircase loop's Poisson solve)
// =============================================================================================
struct gm_poisson {
  std::string err;
  gm_handle* P = nullptr;
  int64_t psize = 0;
  Buf<double> b, x;
  Buf<double> ikappa;
  Buf<int32_t> cell_type;
  // the legacy loop's device scratch and per-step records (four forces and the residual bits)
  Buf<double> lscratch, lrec;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};

extern "C" {

const char* gm_poisson_last_error(const gm_poisson* p) { return p ? p->err.c_str() : gm_last_error(nullptr); }

int gm_poisson_create(int32_t nx, int32_t ny, double Lx, double Ly, double D, double xc, double yc, const double* ax,
                      const double* ay, const int32_t* cell_type, const double* kappa, gm_poisson** out) {
  if (!out || !ax || !ay || !cell_type || !kappa) { gm_internal_set_error("null argument"); return GM_EVALUE; }
  *out = nullptr;
  auto q = std::make_unique<gm_poisson>();
  gm::Geometry g;
  g.nx = nx; g.ny = ny; g.Lx = Lx; g.Ly = Ly; g.D = D; g.xc = xc; g.yc = yc;
  g.nu = 1.0; g.rho = 1.0; g.U_inf = 1.0; g.inflow = 0; g.U_m = 0.0;
  int ec = 0;
  if (!gm::build_cutcell_geometry(g, ax, ay, cell_type, kappa, ec)) {
    gm_internal_set_error(g.error.c_str());
    return ec ? ec : GM_EVALUE;
  }
  q->psize = g.psize;
  std::string perr;
  int rc = gmi::pressure_create(std::move(g), &q->P, perr);
  if (rc != GM_OK) {
    gm_internal_set_error(perr.c_str());
    return rc;
  }
  rc = guarded(nullptr, [&] {
    cudaStream_t st = gmi::stream(q->P);
    q->b.alloc(q->psize);
    q->x.alloc(q->psize);
    std::vector<double> ik(q->psize);
    for (int64_t c = 0; c < q->psize; ++c) ik[c] = cell_type[c] == 0 ? 1.0 / kappa[c] : 1.0;
    q->ikappa.upload(ik, st);
    q->cell_type.upload(std::vector<int32_t>(cell_type, cell_type + q->psize), st);
    CCK(cudaStreamSynchronize(st));
  });
  if (rc != GM_OK) {
    gm_poisson_destroy(q.release());
    return rc;
  }
  *out = q.release();
  return GM_OK;
}

int gm_poisson_destroy(gm_poisson* p) {
  if (!p) return GM_OK;
  gm_handle* P = p->P;
  if (P) cudaStreamSynchronize(gmi::stream(P));
  if (p->ev_in) cudaEventDestroy(p->ev_in);
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  delete p;
  if (P) gmi::pressure_destroy(P);
  return GM_OK;
}

int gm_poisson_legacy_step(gm_poisson* p, gm_legacy_state* s, double dt, int32_t n_steps, gm_legacy_step_diag* diag,
                           void* stream) {
  if (!p) return GM_EVALUE;
  if (!s || n_steps <= 0 || !(std::isfinite(dt) && dt > 0)) {
    p->err = "a state, a positive step count and a finite positive dt are required";
    return GM_EVALUE;
  }
  if ((int64_t)s->nx * s->ny != p->psize || !s->u || !s->v || !s->p || !s->u_star || !s->v_star || !s->rhs ||
      !s->phi || !s->prev_du || !s->prev_dv || !s->zero_p || !s->mask || !s->inlet ||
      (s->centered && s->has_prev && !(std::isfinite(s->prev_dt) && s->prev_dt > 0))) {
    p->err = "the legacy state does not match the pressure system or is incomplete";
    return GM_EVALUE;
  }
  if (s->ghost)
    for (int k = 0; k < 2; ++k)
      if (s->n_ghost[k] < 0 || (s->n_ghost[k] > 0 && (!s->target[k] || !s->src[k] || !s->snap_of[k] ||
                                                      !s->weights[k] || !s->gamma[k] || !s->level[k]))) {
        p->err = "incomplete ghost tables";
        return GM_EVALUE;
      }
  try {
    cudaStream_t st = gmi::stream(p->P);
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (!p->ev_in) CCK(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming));
    if (!p->ev_out) CCK(cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming));
    CCK(cudaEventRecord(p->ev_in, cs));
    CCK(cudaStreamWaitEvent(st, p->ev_in, 0));
    const size_t need = gml::scratch_doubles(*s);
    if (p->lscratch.n < need) p->lscratch.alloc(need);
    if (p->lrec.n < (size_t)n_steps * 5) p->lrec.alloc((size_t)n_steps * 5);
    CcGeo g{};
    g.psize = p->psize;
    g.cell_type = p->cell_type.p;
    g.ikappa = p->ikappa.p;
    std::vector<double> rec((size_t)n_steps * 5);
    for (int32_t k = 0; k < n_steps; ++k) {
      double* r = p->lrec.p + (size_t)k * 5;
      gml::predict(*s, dt, p->lscratch.p, st);
      if (s->centered) {  // the loop keeps the AB2 history before its pressure solve (solver/main.py:320)
        s->has_prev = 1;
        s->prev_dt = dt;
      }
      counted();
      k_cc_scale_rhs<<<nblk(p->psize), CC_TPB, 0, st>>>(g, s->rhs);
      CCK(cudaMemsetAsync(gmi::control(p->P), 0, sizeof(StepCtl), st));
      CCK(cudaMemsetAsync(r + 4, 0, sizeof(double), st));
      gmi::pressure_solve(p->P, s->rhs, s->phi, S_P1);
      counted();
      k_cc_maxdiff<<<std::min<unsigned>(nblk(p->psize), 1216), CC_TPB, 0, st>>>(
          p->psize, gmi::pressure_residual(p->P), nullptr, nullptr, 0.0, reinterpret_cast<unsigned long long*>(r + 4));
      std::string m;
      const int rc = gmi::check(p->P, "pressure solve", m);  // synchronises the stream
      if (rc != GM_OK) throw CcFail(rc, m);
      gml::correct(*s, dt, p->lscratch.p, st);
      gml::forces(*s, p->lscratch.p, r, st);
    }
    CCK(cudaMemcpyAsync(rec.data(), p->lrec.p, rec.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CCK(cudaGetLastError());
    CCK(cudaStreamSynchronize(st));
    CCK(cudaEventRecord(p->ev_out, st));
    CCK(cudaStreamWaitEvent(cs, p->ev_out, 0));
    if (diag)
      for (int32_t k = 0; k < n_steps; ++k) {
        for (int q = 0; q < 4; ++q) diag[k].forces[q] = rec[(size_t)k * 5 + q];
        unsigned long long bits;
        std::memcpy(&bits, &rec[(size_t)k * 5 + 4], sizeof bits);
        diag[k].pressure_residual_linf = bits_to_double(bits);
      }
  } catch (const CcFail& e) {
    p->err = e.msg;
    return e.cls;
  } catch (const std::exception& e) {
    p->err = e.what();
    return GM_ECUDA;
  }
  return GM_OK;
}

int gm_poisson_solve(gm_poisson* p, const double* rhs, double* phi, double* residual_linf) {
  if (!p || !rhs || !phi) return GM_EVALUE;
  int rc = GM_OK;
  try {
    cudaStream_t st = gmi::stream(p->P);
    copy_in(p->b.p, rhs, p->psize, st);
    CcGeo g{};
    g.psize = p->psize;
    g.cell_type = p->cell_type.p;
    g.ikappa = p->ikappa.p;
    counted();
    k_cc_scale_rhs<<<nblk(p->psize), CC_TPB, 0, st>>>(g, p->b.p);
    CCK(cudaMemsetAsync(gmi::control(p->P), 0, sizeof(StepCtl), st));
    gmi::pressure_solve(p->P, p->b.p, p->x.p, S_P1);
    std::string m;
    rc = gmi::check(p->P, "pressure solve", m);
    if (rc != GM_OK) throw CcFail(rc, m);
    if (residual_linf) {
      unsigned long long* bits = nullptr;
      CCK(cudaMallocAsync(reinterpret_cast<void**>(&bits), sizeof(unsigned long long), st));
      CCK(cudaMemsetAsync(bits, 0, sizeof(unsigned long long), st));
      counted();
      k_cc_maxdiff<<<std::min<unsigned>(nblk(p->psize), 1216), CC_TPB, 0, st>>>(
          p->psize, gmi::pressure_residual(p->P), nullptr, nullptr, 0.0, bits);
      unsigned long long hb = 0;
      CCK(cudaMemcpyAsync(&hb, bits, sizeof hb, cudaMemcpyDeviceToHost, st));
      CCK(cudaFreeAsync(bits, st));
      CCK(cudaStreamSynchronize(st));
      *residual_linf = bits_to_double(hb);
    }
    CCK(cudaMemcpyAsync(phi, p->x.p, p->psize * sizeof(double), cudaMemcpyDefault, st));
    CCK(cudaStreamSynchronize(st));
  } catch (const CcFail& e) {
    p->err = e.msg;
    return e.cls;
  } catch (const std::exception& e) {
    p->err = e.what();
    return GM_ECUDA;
  }
  return GM_OK;
}

}  // extern "C"
