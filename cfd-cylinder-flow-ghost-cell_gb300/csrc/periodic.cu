// Periodic Taylor-Green case on the GPU (verification/taylor_green.py:14-59): the AB2/CN
// step of solver/time_integration.py:7-145 with the periodic staggered operators of
// periodic_momentum_operator (solver/cut_cell_solver.py:108-130, the full-fluid flux form of
// compute_momentum_rhs :790-957) and Fourier-space pressure and CN solves.
//
// Grid: u[j][i] at (i h, (j + 1/2) h), v[j][i] at ((i + 1/2) h, j h), p at cell centres,
// h = 2 pi / n; the velocity buffer holds u (n x n) then v (n x n), float64.
//
// Precision 0 runs everything in FP64.  Precision 1 runs the stencils of the momentum
// right-hand side and the Fourier solves in FP32 and refines both solves against the FP64
// operators (the CN system to the reference's residual gate, the pressure until the
// projected divergence is below 1e-11).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ghostmac.h"
#include "fftplan.hpp"
#include "transforms.cuh"

namespace gmk {
void kernel_launch_adjust(long long delta);  // the library's launch counter (kernels.cu)
}

namespace {
using namespace gmk;

constexpr int PT = 256;

struct TgError : std::exception {
  int cls;
  std::string msg;
  TgError(int c, std::string m) : cls(c), msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};
#define TG_CK(call)                                                                              \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) throw TgError(GM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
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
    if (count) TG_CK(cudaMalloc(&p, count * sizeof(T)));
  }
};

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ unsigned long long dbits_(double v) { return (unsigned long long)__double_as_longlong(v); }
// |v| as bits, on the integer pipe: the mask is PTX because the compiler turns fabs, or a C++
// mask of the sign bit, into an FP64 instruction
__device__ __forceinline__ unsigned long long absbits_(double v) {
  unsigned long long r;
  asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(r) : "l"(dbits_(v)));
  return r;
}

__device__ void commit_max(unsigned long long v, unsigned long long* dst) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}

// ---- periodic flux-form operators (T arithmetic, S storage) -----------------------------
// -N(u) at u[j][i]: east/west face fluxes -uE^2 h, north/south corner fluxes -vN uN h, / h^2
template <typename T, typename S>
__device__ __forceinline__ T adv_u_p(const S* u, const S* v, int n, int j, int i, T h) {
  const int ip = wrapi(i + 1, n), im = wrapi(i - 1, n), jp = wrapi(j + 1, n), jm = wrapi(j - 1, n);
  const T uc = (T)u[j * n + i];
  const T uE = (T)0.5 * (uc + (T)u[j * n + ip]), uW = (T)0.5 * ((T)u[j * n + im] + uc);
  const T vN = (T)0.5 * ((T)v[jp * n + im] + (T)v[jp * n + i]), uN = (T)0.5 * (uc + (T)u[jp * n + i]);
  const T vS = (T)0.5 * ((T)v[j * n + im] + (T)v[j * n + i]), uS = (T)0.5 * ((T)u[jm * n + i] + uc);
  const T fE = -(uE * uE * h), fW = -(uW * uW * h), fN = -(vN * uN * h), fS = -(vS * uS * h);
  return ((fE - fW) + (fN - fS)) / (h * h);
}
template <typename T, typename S>
__device__ __forceinline__ T adv_v_p(const S* u, const S* v, int n, int j, int i, T h) {
  const int ip = wrapi(i + 1, n), im = wrapi(i - 1, n), jp = wrapi(j + 1, n), jm = wrapi(j - 1, n);
  const T vc = (T)v[j * n + i];
  const T vN = (T)0.5 * (vc + (T)v[jp * n + i]), vS = (T)0.5 * ((T)v[jm * n + i] + vc);
  const T uE = (T)0.5 * ((T)u[jm * n + ip] + (T)u[j * n + ip]), vE = (T)0.5 * (vc + (T)v[j * n + ip]);
  const T uW = (T)0.5 * ((T)u[jm * n + i] + (T)u[j * n + i]), vW = (T)0.5 * ((T)v[j * n + im] + vc);
  const T fN = -(vN * vN * h), fS = -(vS * vS * h), fE = -(uE * vE * h), fW = -(uW * vW * h);
  return ((fE - fW) + (fN - fS)) / (h * h);
}
// nu L at a point of one component (5-point, the face fluxes nu (f_next - f) / h * h)
template <typename T, typename S>
__device__ __forceinline__ T lap_p(const S* f, int n, int j, int i, T h, T nu) {
  const int ip = wrapi(i + 1, n), im = wrapi(i - 1, n), jp = wrapi(j + 1, n), jm = wrapi(j - 1, n);
  const T c = (T)f[j * n + i];
  const T fE = nu * ((T)f[j * n + ip] - c) / h * h, fW = nu * (c - (T)f[j * n + im]) / h * h;
  const T fN = nu * ((T)f[jp * n + i] - c) / h * h, fS = nu * (c - (T)f[jm * n + i]) / h * h;
  return ((fE - fW) + (fN - fS)) / (h * h);
}

// ---- kernels ------------------------------------------------------------------------------
// AB2/CN right-hand sides (solver/time_integration.py:20-67): mode 0 AB2, mode 1 start-up
// midpoint, mode 2 start-up CN right-hand side from the half-step velocity
template <typename T>
__global__ void k_tg_rhs(int n, double h, double nu, int mode, double dt, double alpha, const double* __restrict__ q,
                         const double* __restrict__ qh, const double* __restrict__ p, const double* __restrict__ prev,
                         double* __restrict__ now, double* __restrict__ out) {
  const int nn = n * n;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nn) return;
  const int comp = t >= nn, k = t - comp * nn, j = k / n, i = k - j * n;
  const double* u = q;
  const double* v = q + nn;
  const T hh = (T)h, nuu = (T)nu, ddt = (T)dt;
  T lq, gp, a = 0;
  if (comp == 0) {
    lq = lap_p<T>(u, n, j, i, hh, nuu);
    gp = ((T)p[j * n + i] - (T)p[j * n + wrapi(i - 1, n)]) / hh;
    if (mode != 2) a = adv_u_p<T>(u, v, n, j, i, hh);
  } else {
    lq = lap_p<T>(v, n, j, i, hh, nuu);
    gp = ((T)p[j * n + i] - (T)p[wrapi(j - 1, n) * n + i]) / hh;
    if (mode != 2) a = adv_v_p<T>(u, v, n, j, i, hh);
  }
  const double qv = q[t];
  if (mode == 1) {
    now[t] = (double)a;
    out[t] = qv + (double)((T)0.5 * ddt * ((a + lq) - gp));
    return;
  }
  T expl;
  if (mode == 0) {
    expl = ((T)1 + (T)alpha) * a - (T)alpha * (T)prev[t];
    now[t] = (double)a;
  } else {
    expl = comp == 0 ? adv_u_p<T>(qh, qh + nn, n, j, i, hh) : adv_v_p<T>(qh, qh + nn, n, j, i, hh);
  }
  out[t] = qv + (double)(ddt * (expl + (T)0.5 * lq - gp));
}

// r = b - H x (H = I - dt/2 nu L, FP64) with max |r| and, on request, max |b|
__global__ void k_tg_hres(int n, double h, double nu, double hdt, const double* __restrict__ b,
                          const double* __restrict__ x, double* __restrict__ r, unsigned long long* rmax,
                          unsigned long long* bmax) {
  const int nn = n * n;
  unsigned long long rm = 0, bm = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nn; t += gridDim.x * blockDim.x) {
    const int comp = t >= nn, k = t - comp * nn, j = k / n, i = k - j * n;
    const double* f = x + comp * nn;
    const double hx = x[t] - hdt * lap_p<double>(f, n, j, i, h, nu);
    const double rv = b[t] - hx;
    if (r) r[t] = rv;
    rm = max(rm, absbits_(rv));
    if (bmax) bm = max(bm, absbits_(b[t]));
  }
  commit_max(rm, rmax);
  if (bmax) commit_max(bm, bmax);
}

// d = div(q) / step on the cell grid, max |div q| on request
__global__ void k_tg_div(int n, double h, double inv_step, const double* __restrict__ q, double* __restrict__ d,
                         unsigned long long* dmax) {
  const int nn = n * n;
  unsigned long long m = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int j = k / n, i = k - j * n;
    const double dv = (q[j * n + wrapi(i + 1, n)] - q[k] + q[nn + wrapi(j + 1, n) * n + i] - q[nn + k]) / h;
    if (d) d[k] = dv * inv_step;
    m = max(m, absbits_(dv));
  }
  if (dmax) commit_max(m, dmax);
}

// r = b - A phi with A = div grad (periodic 5-point / h^2), max |r|
__global__ void k_tg_pres(int n, double h, const double* __restrict__ b, const double* __restrict__ x,
                          double* __restrict__ r, unsigned long long* rmax) {
  const int nn = n * n;
  unsigned long long rm = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int j = k / n, i = k - j * n;
    const double ax = ((x[j * n + wrapi(i + 1, n)] - x[k]) - (x[k] - x[j * n + wrapi(i - 1, n)]) +
                       (x[wrapi(j + 1, n) * n + i] - x[k]) - (x[k] - x[wrapi(j - 1, n) * n + i])) / (h * h);
    const double rv = b[k] - ax;
    r[k] = rv;
    rm = max(rm, absbits_(rv));
  }
  commit_max(rm, rmax);
}

// out = q - step grad(phi)
__global__ void k_tg_update(int n, double h, double step, const double* __restrict__ q, const double* __restrict__ phi,
                            double* __restrict__ out) {
  const int nn = n * n;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nn) return;
  const int comp = t >= nn, k = t - comp * nn, j = k / n, i = k - j * n;
  const double g = comp == 0 ? (phi[k] - phi[j * n + wrapi(i - 1, n)]) / h : (phi[k] - phi[wrapi(j - 1, n) * n + i]) / h;
  out[t] = q[t] - step * g;
}

// action = H result, proj = result + (rhs - action)   (solver/time_integration.py:107-113)
__global__ void k_tg_defect(int n, double h, double nu, double hdt, const double* __restrict__ res,
                            const double* __restrict__ rhs, double* __restrict__ action, double* __restrict__ proj) {
  const int nn = n * n;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nn) return;
  const int comp = t >= nn, k = t - comp * nn, j = k / n, i = k - j * n;
  const double a = res[t] - hdt * lap_p<double>(res + comp * nn, n, j, i, h, nu);
  action[t] = a;
  proj[t] = res[t] + (rhs[t] - a);
}

// half = p + inc, out = half + factor inc, max |action - rhs + dt grad inc|
__global__ void k_tg_pout(int n, double h, double dt, double factor, const double* __restrict__ p,
                          const double* __restrict__ inc, const double* __restrict__ action,
                          const double* __restrict__ rhs, double* __restrict__ half, double* __restrict__ pout,
                          unsigned long long* cmax) {
  const int nn = n * n;
  unsigned long long m = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nn; t += gridDim.x * blockDim.x) {
    const int comp = t >= nn, k = t - comp * nn, j = k / n, i = k - j * n;
    const double g = comp == 0 ? (inc[k] - inc[j * n + wrapi(i - 1, n)]) / h : (inc[k] - inc[wrapi(j - 1, n) * n + i]) / h;
    m = max(m, absbits_(action[t] - rhs[t] + dt * g));
    if (comp == 0) {
      const double hv = p[k] + inc[k];
      half[k] = hv;
      pout[k] = hv + factor * inc[k];
    }
  }
  commit_max(m, cmax);
}

// ---- Fourier solves: rows (x) -> transpose -> rows (y) with the symbol -> transpose -> rows ----
// The symbol of the periodic 5-point Laplacian is lam(k, l) = -4 (s_k + s_l) / h^2 with
// s_k = sin^2(pi k / n).  kind 0: phi = F^-1[F b / lam] with the mean mode set to zero
// (verification/taylor_green.py:41-45); kind 1: x = F^-1[F b / (1 - c lam)].
template <typename T>
__host__ __device__ inline size_t tg_row_smem(int n, int tw) {
  return ((size_t)tw * sizeof(cplx<T>) + 15) / 16 * 16 + 2 * (size_t)n * sizeof(cplx<T>);
}

// mode 0: real row in -> forward FFT -> complex out; mode 1: complex row in -> forward FFT ->
// divide by the symbol -> inverse FFT -> complex out; mode 2: complex row in -> inverse FFT ->
// real part times scale out.  One block per row.
template <typename T, int MODE>
__global__ void k_tg_rows(int n, FftPlan plan, const cplx<T>* __restrict__ tw_g, const void* __restrict__ in,
                          void* __restrict__ out, const T* __restrict__ s2, int kind, T hh2, T coef, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  for (int q = threadIdx.x; q < plan.tw_len; q += blockDim.x) tw[q] = tw_g[q];
  cplx<T>* a = reinterpret_cast<cplx<T>*>(smem_raw + ((size_t)plan.tw_len * sizeof(cplx<T>) + 15) / 16 * 16);
  cplx<T>* b = a + n;
  const int row = blockIdx.x;
  if (MODE == 0) {
    const T* src = reinterpret_cast<const T*>(in) + (size_t)row * n;
    for (int e = threadIdx.x; e < n; e += blockDim.x) a[e] = {src[e], (T)0};
  } else {
    const cplx<T>* src = reinterpret_cast<const cplx<T>*>(in) + (size_t)row * n;
    for (int e = threadIdx.x; e < n; e += blockDim.x) a[e] = src[e];
  }
  __syncthreads();
  const Grp G{(int)threadIdx.x, (int)blockDim.x, 1};
  cplx<T>* r = fft_run<T>(a, b, plan, 1, tw, MODE == 2 ? +1 : -1, G);
  if (MODE == 1) {
    cplx<T>* o = r == a ? b : a;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const T lam = (T)-4 * (s2[row] + s2[e]) / hh2;
      T f;
      if (kind == 0) f = (row == 0 && e == 0) ? (T)0 : (T)1 / lam;
      else f = (T)1 / ((T)1 - coef * lam);
      r[e] = {r[e].x * f, r[e].y * f};
    }
    __syncthreads();
    r = fft_run<T>(r, o, plan, 1, tw, +1, G);
  }
  if (MODE == 2) {
    T* dst = reinterpret_cast<T*>(out) + (size_t)row * n;
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = r[e].x * scale;
  } else {
    cplx<T>* dst = reinterpret_cast<cplx<T>*>(out) + (size_t)row * n;
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = r[e];
  }
}

template <typename T>
__global__ void k_tg_transpose(int n, const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out) {
  __shared__ cplx<T> tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int y = by + yy, x = bx + threadIdx.x;
    if (y < n && x < n) tile[yy][threadIdx.x] = in[(size_t)y * n + x];
  }
  __syncthreads();
  for (int xx = threadIdx.y; xx < 32; xx += blockDim.y) {
    const int x = bx + xx, y = by + threadIdx.x;
    if (y < n && x < n) out[(size_t)x * n + y] = tile[threadIdx.x][xx];
  }
}

template <typename T>
__global__ void k_tg_to_t(int64_t n, const double* __restrict__ src, T* __restrict__ dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = (T)src[t];
}
template <typename T>
__global__ void k_tg_from_t(int64_t n, const T* __restrict__ src, double* __restrict__ dst, int accumulate) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = accumulate ? dst[t] + (double)src[t] : (double)src[t];
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + PT - 1) / PT, 152 * 8); }

}  // namespace

struct gm_tg {
  int n = 0, precision = 0;
  double nu = 0, h = 0;
  std::string err;
  cudaStream_t st = nullptr;
  FftPlan plan{};
  size_t smem = 0, smem32 = 0;
  int threads = 256;
  Buf<double> q, qn, hist, now, rhs, star, mid, half_q, action, proj, phalf, phalf_n, pout, phi, inc, div, work, corr;
  Buf<double> tw64, s2_64;
  Buf<float> tw32, s2_32, real32;
  Buf<double> real64;
  Buf<unsigned char> cbuf_a, cbuf_b;  // complex n x n work arrays (T precision)
  Buf<unsigned long long> red;        // reductions: 0 cn residual, 1 rhs max, 2 div, 3 coupled, 4 pressure residual
  bool has_history = false;
  double prev_dt = 0;
  double last_cn_residual = 0, last_coupled = 0;
};

namespace {

// x = S^-1 b on the cell grid (n x n, FP64 in and out, T arithmetic); kind 0 Poisson, 1 Helmholtz
template <typename T>
void fourier_solve(gm_tg* t, int kind, double coef, const double* b, double* x, bool accumulate) {
  const int n = t->n;
  const int64_t nn = (int64_t)n * n;
  cudaStream_t st = t->st;
  T* rb = sizeof(T) == 4 ? (T*)t->real32.p : (T*)t->real64.p;
  const cplx<T>* tw = sizeof(T) == 4 ? (const cplx<T>*)t->tw32.p : (const cplx<T>*)t->tw64.p;
  const T* s2 = sizeof(T) == 4 ? (const T*)t->s2_32.p : (const T*)t->s2_64.p;
  const size_t smem = sizeof(T) == 4 ? t->smem32 : t->smem;
  cplx<T>* A = reinterpret_cast<cplx<T>*>(t->cbuf_a.p);
  cplx<T>* B = reinterpret_cast<cplx<T>*>(t->cbuf_b.p);
  gmk::kernel_launch_adjust(1);
  k_tg_to_t<T><<<grid_for(nn), PT, 0, st>>>(nn, b, rb);
  gmk::kernel_launch_adjust(1);
  k_tg_rows<T, 0><<<n, t->threads, smem, st>>>(n, t->plan, tw, rb, A, s2, kind, (T)(t->h * t->h), (T)coef, (T)1);
  const dim3 tg((n + 31) / 32, (n + 31) / 32), tb(32, 8);
  gmk::kernel_launch_adjust(1);
  k_tg_transpose<T><<<tg, tb, 0, st>>>(n, A, B);
  gmk::kernel_launch_adjust(1);
  k_tg_rows<T, 1><<<n, t->threads, smem, st>>>(n, t->plan, tw, B, B, s2, kind, (T)(t->h * t->h), (T)coef, (T)1);
  gmk::kernel_launch_adjust(1);
  k_tg_transpose<T><<<tg, tb, 0, st>>>(n, B, A);
  gmk::kernel_launch_adjust(1);
  k_tg_rows<T, 2><<<n, t->threads, smem, st>>>(n, t->plan, tw, A, rb, s2, kind, (T)(t->h * t->h), (T)coef,
                                                (T)(1.0 / ((double)n * n)));
  gmk::kernel_launch_adjust(1);
  k_tg_from_t<T><<<grid_for(nn), PT, 0, st>>>(nn, rb, x, accumulate ? 1 : 0);
  TG_CK(cudaGetLastError());
}

unsigned long long read_max(gm_tg* t, int slot) {
  unsigned long long v = 0;
  TG_CK(cudaMemcpyAsync(&v, t->red.p + slot, sizeof v, cudaMemcpyDeviceToHost, t->st));
  TG_CK(cudaStreamSynchronize(t->st));
  return v;
}
double bitsd(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

// project(q, step): phi = A^-1 (div q / step), out = q - step grad phi (refined in FP32 mode
// until the projected divergence max |step (b - A phi)| is below 1e-11)
void tg_project(gm_tg* t, const double* q, double step, double* out, double* phi) {
  const int n = t->n;
  const int64_t nn = (int64_t)n * n;
  cudaStream_t st = t->st;
  gmk::kernel_launch_adjust(1);
  k_tg_div<<<grid_for(nn), PT, 0, st>>>(n, t->h, 1.0 / step, q, t->div.p, nullptr);
  if (t->precision == 0) {
    fourier_solve<double>(t, 0, 0.0, t->div.p, phi, false);
  } else {
    fourier_solve<float>(t, 0, 0.0, t->div.p, phi, false);
    for (int sweep = 0; sweep < 8; ++sweep) {
      TG_CK(cudaMemsetAsync(t->red.p + 4, 0, sizeof(unsigned long long), st));
      gmk::kernel_launch_adjust(1);
      k_tg_pres<<<grid_for(nn), PT, 0, st>>>(n, t->h, t->div.p, phi, t->work.p, t->red.p + 4);
      if (bitsd(read_max(t, 4)) * step <= 1e-11) break;
      fourier_solve<float>(t, 0, 0.0, t->work.p, phi, true);
    }
  }
  gmk::kernel_launch_adjust(1);
  k_tg_update<<<(unsigned)((2 * nn + PT - 1) / PT), PT, 0, st>>>(n, t->h, step, q, phi, out);
}

// star = H^-1 rhs (two components), refined in FP32 mode to the CN gate
void tg_helmholtz(gm_tg* t, double dt, const double* rhs, double* star) {
  const int n = t->n;
  const int64_t nn = (int64_t)n * n;
  cudaStream_t st = t->st;
  const double c = 0.5 * dt * t->nu;
  for (int comp = 0; comp < 2; ++comp) {
    if (t->precision == 0) fourier_solve<double>(t, 1, c, rhs + comp * nn, star + comp * nn, false);
    else fourier_solve<float>(t, 1, c, rhs + comp * nn, star + comp * nn, false);
  }
  if (t->precision == 1) {
    for (int sweep = 0; sweep < 6; ++sweep) {
      TG_CK(cudaMemsetAsync(t->red.p, 0, 2 * sizeof(unsigned long long), st));
      gmk::kernel_launch_adjust(1);
      k_tg_hres<<<grid_for(2 * nn), PT, 0, st>>>(n, t->h, t->nu, 0.5 * dt, rhs, star, t->work.p, t->red.p, t->red.p + 1);
      unsigned long long v[2];
      TG_CK(cudaMemcpyAsync(v, t->red.p, sizeof v, cudaMemcpyDeviceToHost, st));
      TG_CK(cudaStreamSynchronize(st));
      if (bitsd(v[0]) <= 32 * 2.220446049250313e-16 * std::max(1.0, bitsd(v[1]))) break;
      for (int comp = 0; comp < 2; ++comp) fourier_solve<float>(t, 1, c, t->work.p + comp * nn, star + comp * nn, true);
    }
  }
}

// ab2_cn_step (solver/time_integration.py:7-145) with the periodic operators
void tg_step(gm_tg* t, double dt, double* max_div) {
  const int n = t->n;
  const int64_t nn = (int64_t)n * n;
  cudaStream_t st = t->st;
  const unsigned g2 = (unsigned)((2 * nn + PT - 1) / PT);
  auto rhs_kernel = [&](int mode, double alpha, const double* qh, double* out) {
    gmk::kernel_launch_adjust(1);
    if (t->precision == 1)
      k_tg_rhs<float><<<g2, PT, 0, st>>>(n, t->h, t->nu, mode, dt, alpha, t->q.p, qh, t->phalf.p, t->hist.p, t->now.p,
                                         out);
    else
      k_tg_rhs<double><<<g2, PT, 0, st>>>(n, t->h, t->nu, mode, dt, alpha, t->q.p, qh, t->phalf.p, t->hist.p,
                                          t->now.p, out);
  };
  const bool first = !t->has_history;
  if (first) {
    rhs_kernel(1, 0.0, nullptr, t->mid.p);
    tg_project(t, t->mid.p, 0.5 * dt, t->half_q.p, t->phi.p);
    rhs_kernel(2, 0.0, t->half_q.p, t->rhs.p);
  } else {
    rhs_kernel(0, dt / (2 * t->prev_dt), nullptr, t->rhs.p);
  }
  tg_helmholtz(t, dt, t->rhs.p, t->star.p);
  // CN gate: max |H star - rhs| <= 1e-10 max(1, max |rhs|)  (solver/time_integration.py:100-104)
  TG_CK(cudaMemsetAsync(t->red.p, 0, 5 * sizeof(unsigned long long), st));
  gmk::kernel_launch_adjust(1);
  k_tg_hres<<<grid_for(2 * nn), PT, 0, st>>>(n, t->h, t->nu, 0.5 * dt, t->rhs.p, t->star.p, nullptr, t->red.p,
                                             t->red.p + 1);
  unsigned long long v[2];
  TG_CK(cudaMemcpyAsync(v, t->red.p, sizeof v, cudaMemcpyDeviceToHost, st));
  TG_CK(cudaStreamSynchronize(st));
  t->last_cn_residual = bitsd(v[0]);
  if (!std::isfinite(bitsd(v[0])) || bitsd(v[0]) > 1e-10 * std::max(1.0, bitsd(v[1])))
    throw TgError(GM_ERUNTIME, "CN momentum solve failed: residual=" + std::to_string(bitsd(v[0])));
  tg_project(t, t->star.p, dt, t->qn.p, t->phi.p);
  gmk::kernel_launch_adjust(1);
  k_tg_defect<<<g2, PT, 0, st>>>(n, t->h, t->nu, 0.5 * dt, t->qn.p, t->rhs.p, t->action.p, t->proj.p);
  tg_project(t, t->proj.p, dt, t->work.p, t->inc.p);
  const double factor = first ? 1.0 : dt / (dt + t->prev_dt);
  gmk::kernel_launch_adjust(1);
  k_tg_pout<<<grid_for(2 * nn), PT, 0, st>>>(n, t->h, dt, factor, t->phalf.p, t->inc.p, t->action.p, t->rhs.p,
                                             t->phalf_n.p, t->pout.p, t->red.p + 3);
  TG_CK(cudaMemsetAsync(t->red.p + 2, 0, sizeof(unsigned long long), st));
  gmk::kernel_launch_adjust(1);
  k_tg_div<<<grid_for(nn), PT, 0, st>>>(n, t->h, 1.0, t->qn.p, nullptr, t->red.p + 2);
  unsigned long long r[2];
  TG_CK(cudaMemcpyAsync(r, t->red.p + 2, sizeof r, cudaMemcpyDeviceToHost, st));
  TG_CK(cudaStreamSynchronize(st));
  *max_div = std::max(*max_div, bitsd(r[0]));
  t->last_coupled = bitsd(r[1]);
  std::swap(t->q.p, t->qn.p);
  std::swap(t->phalf.p, t->phalf_n.p);
  std::swap(t->hist.p, t->now.p);
  t->has_history = true;
  t->prev_dt = dt;
}

int tg_guard(gm_tg* t, const std::function<void()>& f) {
  try {
    f();
    return GM_OK;
  } catch (const TgError& e) {
    if (t) t->err = e.msg;
    return e.cls;
  } catch (const std::exception& e) {
    if (t) t->err = e.what();
    return GM_ECUDA;
  }
}

std::string g_tg_create_error;

}  // namespace

extern "C" {

int gm_tg_create(int32_t n, double nu, int32_t precision, gm_tg** out) {
  if (!out) return GM_EVALUE;
  *out = nullptr;
  if (n < 8 || !(std::isfinite(nu) && nu > 0)) { g_tg_create_error = "Require n>=8 and finite positive nu"; return GM_EVALUE; }
  if (precision != 0 && precision != 1) { g_tg_create_error = "precision must be 0 or 1"; return GM_EVALUE; }
  auto t = std::make_unique<gm_tg>();
  t->n = n;
  t->nu = nu;
  t->h = 2 * 3.141592653589793 / n;
  t->precision = precision;
  int rc = tg_guard(t.get(), [&] {
    TG_CK(cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking));
    t->plan = make_plan(n);
    std::vector<double> tw = plan_twiddles(t->plan);
    t->tw64.alloc(tw.size());
    TG_CK(cudaMemcpy(t->tw64.p, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> tw32(tw.begin(), tw.end());
    t->tw32.alloc(tw32.size());
    TG_CK(cudaMemcpy(t->tw32.p, tw32.data(), tw32.size() * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<double> s2(n);
    for (int k = 0; k < n; ++k) s2[k] = std::pow(std::sin(3.141592653589793 * k / n), 2);
    t->s2_64.alloc(n);
    TG_CK(cudaMemcpy(t->s2_64.p, s2.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> s2f(s2.begin(), s2.end());
    t->s2_32.alloc(n);
    TG_CK(cudaMemcpy(t->s2_32.p, s2f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    t->smem = tg_row_smem<double>(n, t->plan.tw_len);
    t->smem32 = tg_row_smem<float>(n, t->plan.tw_len);
    int optin = 0;
    TG_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0));
    if (t->smem > (size_t)optin) throw TgError(GM_EVALUE, "grid too large for the row transforms");
    // the limit is a process-wide attribute of the kernel shared by every handle: the device
    // maximum, so that a smaller handle created later cannot lower it below a larger one's need
    for (auto f : {(const void*)k_tg_rows<double, 0>, (const void*)k_tg_rows<double, 1>, (const void*)k_tg_rows<double, 2>,
                   (const void*)k_tg_rows<float, 0>, (const void*)k_tg_rows<float, 1>, (const void*)k_tg_rows<float, 2>}) {
      cudaFuncAttributes fa;
      TG_CK(cudaFuncGetAttributes(&fa, f));
      const int dyn = optin - (int)fa.sharedSizeBytes;
      if (t->smem > (size_t)dyn) throw TgError(GM_EVALUE, "grid too large for the row transforms");
      TG_CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    }
    t->threads = std::min(512, std::max(64, ((n / 4 + 31) / 32) * 32));
    const int64_t nn = (int64_t)n * n;
    for (Buf<double>* b : {&t->q, &t->qn, &t->hist, &t->now, &t->rhs, &t->star, &t->mid, &t->half_q, &t->action,
                           &t->proj, &t->work}) {
      b->alloc(2 * nn);
      TG_CK(cudaMemset(b->p, 0, 2 * nn * sizeof(double)));
    }
    for (Buf<double>* b : {&t->phalf, &t->phalf_n, &t->pout, &t->phi, &t->inc, &t->div, &t->real64}) {
      b->alloc(nn);
      TG_CK(cudaMemset(b->p, 0, nn * sizeof(double)));
    }
    t->real32.alloc(nn);
    t->cbuf_a.alloc((size_t)nn * 16);
    t->cbuf_b.alloc((size_t)nn * 16);
    t->red.alloc(8);
    TG_CK(cudaMemset(t->red.p, 0, 8 * sizeof(unsigned long long)));
  });
  if (rc != GM_OK) { g_tg_create_error = t->err; return rc; }
  *out = t.release();
  return GM_OK;
}

int gm_tg_destroy(gm_tg* t) {
  if (!t) return GM_OK;
  if (t->st) {
    cudaStreamSynchronize(t->st);
    cudaStreamDestroy(t->st);
  }
  delete t;
  return GM_OK;
}

const char* gm_tg_last_error(const gm_tg* t) { return t ? t->err.c_str() : g_tg_create_error.c_str(); }

int gm_tg_set_state(gm_tg* t, const double* q, const double* p) {
  if (!t || !q || !p) return GM_EVALUE;
  return tg_guard(t, [&] {
    const int64_t nn = (int64_t)t->n * t->n;
    TG_CK(cudaMemcpyAsync(t->q.p, q, 2 * nn * sizeof(double), cudaMemcpyDefault, t->st));
    TG_CK(cudaMemcpyAsync(t->phalf.p, p, nn * sizeof(double), cudaMemcpyDefault, t->st));
    TG_CK(cudaMemcpyAsync(t->pout.p, p, nn * sizeof(double), cudaMemcpyDefault, t->st));
    TG_CK(cudaStreamSynchronize(t->st));
    t->has_history = false;
    t->prev_dt = 0;
  });
}

int gm_tg_get_state(gm_tg* t, double* q, double* p_half, double* p_out) {
  if (!t) return GM_EVALUE;
  return tg_guard(t, [&] {
    const int64_t nn = (int64_t)t->n * t->n;
    if (q) TG_CK(cudaMemcpyAsync(q, t->q.p, 2 * nn * sizeof(double), cudaMemcpyDefault, t->st));
    if (p_half) TG_CK(cudaMemcpyAsync(p_half, t->phalf.p, nn * sizeof(double), cudaMemcpyDefault, t->st));
    if (p_out) TG_CK(cudaMemcpyAsync(p_out, t->pout.p, nn * sizeof(double), cudaMemcpyDefault, t->st));
    TG_CK(cudaStreamSynchronize(t->st));
  });
}

int gm_tg_step(gm_tg* t, double dt, int32_t n_steps, double* max_divergence) {
  if (!t || n_steps <= 0 || !(std::isfinite(dt) && dt > 0)) {
    if (t) t->err = "Finite fields and a positive timestep are required";
    return GM_EVALUE;
  }
  return tg_guard(t, [&] {
    double md = max_divergence ? *max_divergence : 0.0;
    for (int s = 0; s < n_steps; ++s) tg_step(t, dt, &md);
    if (max_divergence) *max_divergence = md;
  });
}

}  // extern "C"
