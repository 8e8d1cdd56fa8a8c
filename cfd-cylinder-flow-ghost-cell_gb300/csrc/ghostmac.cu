// C ABI of libghostmac.so: handle lifetime, device upload, Schur precompute and
// the AB2/CN step sequence (solver/time_integration.py:7-145 as orchestrated by
// solver/optimized_ghost_cell.py:236-278 and solver/main.py:271-429).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <array>
#include <vector>

#include "../../include/ghostmac.h"
#include "geometry.hpp"
#include "fftplan.hpp"
#include "kernels.cuh"
#include "internal.hpp"

using namespace gmk;

// Last error of a call made without a handle (gm_create, gm_create_host and the
// allocation-free entry point), one per host thread so that threads failing at the same time
// do not overwrite each other's text; a fixed buffer so that setting it allocates nothing.
static thread_local char g_global_error[512];
void gm_internal_set_error(const char* msg) {
  std::strncpy(g_global_error, msg ? msg : "", sizeof g_global_error - 1);
  g_global_error[sizeof g_global_error - 1] = 0;
}

namespace {

struct GlobalError {
  GlobalError& operator=(const std::string& m) { gm_internal_set_error(m.c_str()); return *this; }
  GlobalError& operator=(const char* m) { gm_internal_set_error(m); return *this; }
};
GlobalError g_create_error;

struct CudaError : std::exception {
  std::string msg;
  explicit CudaError(std::string m) : msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};
struct GateError : std::exception {
  int cls;
  std::string msg;
  GateError(int c, std::string m) : cls(c), msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { if (p) cudaFree(p); }
  void alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    if (count) CK(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const std::vector<T>& v, cudaStream_t st) {
    alloc(v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void zero(cudaStream_t st) { if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), st)); }
};

struct Csrd {
  DBuf<int64_t> rows, ptr, col;
  DBuf<double> val;
  DBuf<int32_t> index;  // per grid point: its row in this CSR, or -1 (irregular operator rows)
  int n = 0;
};

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// radix plan of an FFT length
std::vector<double> cexp_table(int count, double scale_num, double scale_den, double offset, int sign) {
  // entries exp(sign * i * pi * (k*scale_num + offset) / scale_den), interleaved (re, im)
  std::vector<double> t(2 * (size_t)count);
  for (int k = 0; k < count; ++k) {
    long double a = 3.14159265358979323846264338327950288L * ((long double)k * scale_num + offset) / scale_den;
    t[2 * k] = (double)std::cos(a);
    t[2 * k + 1] = sign * (double)std::sin(a);
  }
  return t;
}

struct RectDev {
  TransformTables tt{};
  RectView view{};
  DBuf<double> Wx, prex, postx, t0, t1, t2;
  // FP32 copies for the mixed-precision mode
  TransformTables tt32{};
  DBuf<float> Wx32, prex32, postx32, t0_32, t1_32, t2_32;
  // Schur data
  int rank = 0;
  DBuf<int64_t> rows, cptr, ccol;
  DBuf<double> cval, sinv;
  int mcount = 0;             // distinct points read by the C rows
  DBuf<int64_t> mcols;        // their field-grid flat indices
  DBuf<double> mmat;          // M = S^{-1} C, rank x mcount
  // band solve of the Schur term (pivots, decay factors, band work array)
  DBuf<double> bpiv, phi, psi, band;
  DBuf<float> bpiv32, phi32, psi32, band32;
  // direct sums of the boundary term (build_direct_tables): the inverse row transform at the
  // mcount points (spectrum row of each, coefficients mcount x cols), the forward row transform
  // of a unit value at each boundary row (band-row order: bptr over band rows), M with its rows
  // in the same band-row order (so the GEMV writes the Schur values c already in that order),
  // c, and the transformed values at the points
  bool direct = false;
  DBuf<int32_t> mrow, bptr;
  DBuf<double> binv, bfwd, mband, cvec, firstm;
  DBuf<float> binv32, bfwd32, firstm32;
  // FP32 mode, pressure: the row passes as split-TF32 GEMMs on the tensor cores (rowgemm.cu),
  // and their boundary-term table W (rows x cols: the phi rows, the band rows that the band
  // solve writes in place, the psi rows)
  RowGemm gemm;
  DBuf<float> wcorr32;
  // G = M binv folded over the spectrum rows cj0..cj1 (rank x glen, glen = (cj1 - cj0 + 1) cols;
  // 0: not built, the first / GEMV chain runs), in the mode's precision, and the slice sums
  int glen = 0;
  DBuf<double> gmat;
  DBuf<float> gmat32;
  DBuf<double> cpart;
};

}  // namespace

struct gm_handle {
  gm::Geometry g;
  gm::HelmholtzSetup hs;
  bool helm_ready = false;
  double helm_dt = 0;
  long long helm_gen = 0;  // bumped whenever the device Helmholtz tables are rebuilt
  std::string err;
  cudaStream_t st = nullptr;
  bool own_stream = true;
  int device = 0;
  size_t smem_optin = 48 * 1024;
  CaseDev cd{};
  // geometry on device
  DBuf<uint8_t> cls_f, cls_p, mask;  // cls_f: u then v class maps
  const uint8_t* cls_u = nullptr;
  const uint8_t* cls_v = nullptr;
  DBuf<double> inlet;
  Csrd gf, gp, irr[3];
  DBuf<int32_t> a_nnz;
  DBuf<int64_t> sp_ptr, sp_col, su_ptr, su_col, sv_ptr, sv_col, d_ui, d_vi, d_pi;
  DBuf<double> sp_val, su_val, sv_val, nwx, nwy, nxx, nyy;
  DBuf<double> surf_part;      // per-point force terms
  DBuf<unsigned> surf_ticket;  // k_forces block counter
  RectDev rp, ru, rv;
  // state and work buffers (face grid F, pressure grid P)
  DBuf<double> U, Unext, hist, now, rhs, star, fres, ffirst, fw2, fmid, fhalf, faction, fproj, fproj2, ftmp;
  DBuf<double> phalf, phalf_next, pout, prhs, pphi, pres, pfirst, pw2, pinc, ptmp, spectral;
  DBuf<float> pres32, fres32;  // FP32-mode residuals (inputs of the FP32 inverse)
  DBuf<float> U32, P32;        // FP32-mode copies of the state for the momentum stencils
  // FP32 mode: Jacobi iterations of the Helmholtz systems (per dt; jac_iters 0 keeps the FFT
  // inverse), their irregular-row tables and two face-grid iterates (u and v use disjoint parts,
  // so the two lanes share them)
  int jac_iters = 0;
  double jac_rho = 0.0;
  HelmJacobi hj{};
  DBuf<float> jval[2], jidiag[2], jd0, jd1;
  DBuf<int32_t> jsidx[2], jrpos[2];
  size_t jac_smem = 0;  // dynamic shared memory of the temporally blocked form (0: K launches)
  int jac_tile = 0;     // its regular tile, width * 1000 + height (autotuned at set-up)
  // flexible GMRES (pressure_solver = iterative): Krylov basis V (m+1 vectors), preconditioned
  // directions Z (m), the refinement correction and reduction scratch
  static constexpr int GMRES_M = 50;
  DBuf<double> gV, gZ, gdx, gpart, gdots, gcoef;
  // FGMRES with its control on the device: state, scalars, and one instantiated graph per
  // (right-hand side, solution) pair it has solved for
  DBuf<GmresDev> gdev;
  DBuf<double> gd1, gd2, gwn, gbeta, gbn, gy, gone;
  DBuf<int> gnv;
  struct GmresExec {
    const double* b = nullptr;
    double* x = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long fixed = 0, per_cycle = 0, per_step = 0;  // kernels of the graph's parts
  };
  std::vector<GmresExec> gexec;
  // learned preconditioner attached to the GMRES path (network and weights owned by the caller)
  gm_unet* lnet = nullptr;
  std::vector<const uint16_t*> lw;
  std::vector<const float*> lb;
  DBuf<float> lout;              // network output (pressure grid)
  DBuf<unsigned long long> lscale;  // max |r| bits
  // recorder of the pressure solves of launch-by-launch steps: (right-hand side, solution)
  double* rec_rhs = nullptr;
  double* rec_sol = nullptr;
  int rec_cap = 0, rec_count = 0;
  ResidualCoef rcoef[3];       // regular-row coefficients: pressure, Helmholtz u, Helmholtz v
  DBuf<float> spectral32, ffirst32, pfirst32;
  DBuf<StepCtl> ctl;
  DBuf<unsigned long long> state_max;  // persistent max|u|, max|v| of the current state
  StepCtl* host_ctl = nullptr;
  // step records and graphs
  static constexpr int RING_CAP = 64;
  DBuf<StepCtl> ring;
  DBuf<int> ridx;
  DBuf<long long> counter;
  StepCtl* host_ring = nullptr;
  cudaStream_t st_body = nullptr;  // capture stream of conditional-node bodies
  // second lane: the v Helmholtz solve runs beside the u solve (own stream, body stream and
  // spectral work arrays); fork/join by events
  cudaStream_t st2 = nullptr, st2_body = nullptr;
  double step_dt = 0.0;  // dt of the step being issued (step phases)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  DBuf<double> spectral_b;
  DBuf<float> spectral32_b;
  long long body_nodes_slot[5] = {0, 0, 0, 0, 0};  // kernels per refinement sweep of each solve slot
  bool use_graphs = true;
  bool capturing = false;
  // launch-by-launch steps decide every refinement sweep on the host (one synchronisation
  // per sweep) instead of launching all sweeps gated: then every launched kernel does work,
  // which per-kernel timing and profiling need (environment GHOSTMAC_HOST_REFINE=1)
  bool host_refine = false;
  // optional timing events between the phases of a step (environment GHOSTMAC_PHASE_TIMING=1
  // when the step graphs are captured): start, momentum, Helmholtz solves, projection 1,
  // defect, projection 2, end
  static constexpr int NPHASE_EV = 7;
  bool phase_on = false;
  cudaEvent_t phase_ev[NPHASE_EV] = {};
  double phase_ms[NPHASE_EV - 1] = {};
  // with phase timing on, the first sweep of projection 1 also times each of its kernels:
  // row pass, column solve, band row pass, Schur GEMV, band row pass, band solve, final
  // row pass, residual
  static constexpr int NSWEEP_EV = 9;
  bool sweep_marking = false;
  cudaEvent_t sweep_ev[NSWEEP_EV] = {};
  double sweep_ms[NSWEEP_EV - 1] = {};
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    const double* key[6] = {};
    double dt = 0;
    long long outer_nodes = 0;     // kernel nodes outside the refinement loops
    long long body_nodes[5] = {};  // kernel nodes of one refinement sweep, per solve slot
  } graphs[2];
  bool has_history = false;
  bool host_only = false;
  int precision = 0;  // 0 plain FP64, 1 FP32 inverse with FP64 refinement
  int nchk = 3;       // residual checks per solve (1 + refinement sweeps)
  double prev_dt = 0;
  int64_t F = 0, Pn = 0;
  // scratch for host<->device arrays
  DBuf<double> io[4];
};

namespace {

void set_error(gm_handle* h, const std::string& m) {
  if (h) h->err = m;
  else g_create_error = m;
}

Gate gate_of(gm_handle* h, int slot = 0, int sweep = 0) { return Gate{h->ctl.p, slot, sweep}; }

void upload_csr(Csrd& d, const std::vector<int64_t>& rows, const gm::Csr& c, cudaStream_t st,
                int64_t col_offset = 0, int64_t row_offset = 0) {
  d.n = (int)c.rows();
  std::vector<int64_t> r(rows), cols(c.col);
  for (auto& x : r) x += row_offset;
  for (auto& x : cols) x += col_offset;
  d.rows.upload(r, st);
  d.ptr.upload(c.ptr, st);
  d.col.upload(cols, st);
  d.val.upload(c.val, st);
}
// row index of every point of a grid of `npts` points into the irregular rows (or -1)
void upload_row_index(Csrd& d, const std::vector<int64_t>& rows, int64_t npts, cudaStream_t st) {
  std::vector<int32_t> idx((size_t)npts, -1);
  for (size_t k = 0; k < rows.size(); ++k) idx[(size_t)rows[k]] = (int32_t)k;
  d.index.upload(idx, st);
}

std::vector<float> to_f32(const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); }

// Chunk layout of an n-row column: P chunks of inner rows separated by P-1 interface rows.
YChunks make_chunks(int n) {
  YChunks c{};
  int P = std::max(1, (n + 1) / (32 + 1));
  P = std::min(P, YCHUNK_MAX);
  int inner = n - (P - 1);  // rows that are not interfaces
  int r = 0;
  for (int p = 0; p < P; ++p) {
    int m = inner / P + (p < inner % P ? 1 : 0);
    c.start[p] = r;
    c.end[p] = r + m - 1;
    r += m + 1;  // skip the interface row after the chunk
  }
  c.P = P;
  return c;
}

// Partition-method tables of the column systems (see k_ysolve).  main(j) is the
// diagonal of row j for this x-mode, gamma the constant off-diagonal.
void ysolve_tables(const YChunks& ch, int n, int cols, int kx, const std::vector<double>& main, double gamma,
                   double* t0, double* t1, double* t2) {
  auto at = [&](int j) { return (size_t)j * cols + kx; };
  std::vector<double> inv(n, 0.0), v(n, 0.0), w(n, 0.0), tmp(n);
  for (int p = 0; p < ch.P; ++p) {
    int a = ch.start[p], b = ch.end[p];
    double piv = main[a];
    inv[a] = 1.0 / piv;
    for (int j = a + 1; j <= b; ++j) {
      piv = main[j] - gamma * gamma * inv[j - 1];
      inv[j] = 1.0 / piv;
    }
    // spikes: A_in v = gamma e_a (p > 0), A_in w = gamma e_b (p < P-1)
    auto solve_unit = [&](int at_row, std::vector<double>& out) {
      double prev = 0;
      for (int j = a; j <= b; ++j) {
        double d = (j == at_row) ? gamma : 0.0;
        prev = (d - gamma * prev) * inv[j];
        tmp[j] = prev;
      }
      out[b] = tmp[b];
      for (int j = b - 1; j >= a; --j) out[j] = tmp[j] - gamma * inv[j] * out[j + 1];
    };
    if (p > 0) solve_unit(a, v);
    if (p < ch.P - 1) solve_unit(b, w);
    for (int j = a; j <= b; ++j) { t0[at(j)] = inv[j]; t1[at(j)] = v[j]; t2[at(j)] = w[j]; }
  }
  // interface system: sub_q y_{q-1} + main_q y_q + sup_q y_{q+1} = rhs_q
  double cr_prev = 0;
  for (int q = 0; q < ch.P - 1; ++q) {
    int e = ch.end[q] + 1;
    int bL = ch.end[q], aR = ch.start[q + 1];
    double sub = -gamma * v[bL];
    double mid = main[e] - gamma * w[bL] - gamma * v[aR];
    double sup = -gamma * w[aR];
    double piv = mid - sub * cr_prev;
    double rinv = 1.0 / piv;
    double cr = sup * rinv;
    t0[at(e)] = rinv;
    t1[at(e)] = sub;
    t2[at(e)] = cr;
    cr_prev = cr;
  }
}

// Diagonal of the column system of x-mode kx: pressure (L_y + lambda_x)/rho, Helmholtz
// (1 - c lambda_x) - c L_y with c = dt/2 nu; the off-diagonal is column_gamma.  The wall
// rows follow the 1-D operators of solver/rectangular_inverse.py:8-58.
void column_diagonal(const gm::Geometry& g, int kind, double dt, int rows, int kx, std::vector<double>& mainj) {
  const double PI = 3.141592653589793;
  const double idy2 = 1.0 / (g.dy * g.dy);
  const double c = (0.5 * dt) * g.nu;
  const double sx = ((double)kx + 0.5) * PI / (2 * g.nx);
  const double lam = -4 * std::pow(std::sin(sx), 2) / (g.dx * g.dx);
  mainj.resize(rows);
  for (int j = 0; j < rows; ++j) {
    double m = -2.0;
    if (kind == 0 && (j == 0 || j == rows - 1)) m = -1.0;
    if (kind == 1 && (j == 0 || j == rows - 1)) m = -3.0;
    const double ly = m * idy2;
    mainj[j] = kind == 0 ? (ly + lam) / g.rho : 1.0 - c * (lam + ly);
  }
}
double column_gamma(const gm::Geometry& g, int kind, double dt) {
  const double idy2 = 1.0 / (g.dy * g.dy);
  return kind == 0 ? idy2 / g.rho : -((0.5 * dt) * g.nu) * idy2;
}

// T^{-1} b on a rectangle view without the boundary term: x pass, column solves, x pass.
template <typename T, typename TI, typename TO>
void plain_inverse(const TransformTables& tt, const RectView& v, const TI* b, bool mask_in, T* spectral, TO* out,
                   const uint8_t* ocls, const double* add, const Gate& g, cudaStream_t st) {
  const YCorr<T> none{nullptr, nullptr, nullptr, 0, -1};
  launch_xpass<T, TI, T>(tt, false, 0, v.rows, b, v.base, v.pitch, mask_in ? v.cls : nullptr, spectral, 0, v.cols,
                         nullptr, nullptr, none, g, st);
  launch_ysolve<T>(tt, v.cols, v.rows, spectral, g, st);
  launch_xpass<T, T, TO>(tt, true, 0, v.rows, spectral, 0, v.cols, nullptr, out, v.base, v.pitch, ocls, add, none, g,
                         st);
}

// Launch shapes of the separable inverse, picked by timing: the x pass over line-group
// sizes of 1-8 warps and 1-4 groups per block, the column solve over 2-8 columns per
// block.  Every shape computes the same values (each line / column is handled by the same
// arithmetic whatever the grouping), so only the time differs.
void autotune_shapes(gm_handle* h, RectDev& rd, int kind, bool fp32) {
  TransformTables& tt = fp32 ? rd.tt32 : rd.tt;
  const RectView& v = rd.view;
  cudaStream_t st = h->st;
  const size_t per = std::max(xpass_smem_per_group(tt.tx_fwd, v.cols, fp32), xpass_smem_per_group(tt.tx_inv, v.cols, fp32));
  const size_t tabs = std::max(xpass_smem_tables(tt.tx_fwd, v.cols, tt.plan_x.tw_len, fp32),
                               xpass_smem_tables(tt.tx_inv, v.cols, tt.plan_x.tw_len, fp32));
  double* field = kind == 0 ? h->ptmp.p : h->ftmp.p;
  float* field32 = kind == 0 ? h->pfirst32.p : h->ffirst32.p;
  const Gate open{nullptr, 0, 0};
  const YCorr<double> none64{nullptr, nullptr, nullptr, 0, -1};
  const YCorr<float> none32{nullptr, nullptr, nullptr, 0, -1};
  CK(cudaMemsetAsync(field, 0, (size_t)(kind == 0 ? h->Pn : h->F) * sizeof(double), st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  // a shape whose launch the device refuses (threads x registers) is skipped; each timing is
  // the best of 5 runs of 4 back-to-back launches (single launches are too noisy to rank the
  // shapes the same way in every process)
  auto time_ms = [&](auto&& body) {
    float best = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
      CK(cudaEventRecord(e0, st));
      for (int k = 0; k < 4; ++k) body();
      if (cudaGetLastError() != cudaSuccess) return 1e30f;
      CK(cudaEventRecord(e1, st));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) best = std::min(best, ms);  // the first run warms caches and code
    }
    return best;
  };
  // x pass
  float best = 1e30f;
  int bt = 32, bg = 1;
  for (int gt : {64, 128, 256, 512}) {
    for (int gp : {1, 2, 4}) {
      if (gt * gp > 512 || tabs + per * gp > h->smem_optin) continue;
      tt.xg_threads = gt;
      tt.xg_pb = gp;
      tt.smem_x = tabs + per * gp;
      float ms = time_ms([&] {
        if (fp32) {
          launch_xpass<float, double, float>(tt, false, 0, v.rows, field, v.base, v.pitch, nullptr, h->spectral32.p, 0,
                                             v.cols, nullptr, nullptr, none32, open, st);
          launch_xpass<float, float, float>(tt, true, 0, v.rows, h->spectral32.p, 0, v.cols, nullptr, field32, v.base,
                                            v.pitch, nullptr, nullptr, none32, open, st);
        } else {
          launch_xpass<double, double, double>(tt, false, 0, v.rows, field, v.base, v.pitch, nullptr, h->spectral.p, 0,
                                               v.cols, nullptr, nullptr, none64, open, st);
          launch_xpass<double, double, double>(tt, true, 0, v.rows, h->spectral.p, 0, v.cols, nullptr, field, v.base,
                                               v.pitch, nullptr, nullptr, none64, open, st);
        }
      });
      if (ms < best) { best = ms; bt = gt; bg = gp; }
    }
  }
  if (best >= 1e30f) throw CudaError("row transforms do not fit the shared memory");
  tt.xg_threads = bt;
  tt.xg_pb = bg;
  tt.smem_x = tabs + per * bg;
  // column solve: L columns per block and the block's threads (at least L x P: one per chunk in
  // the solve phases; more threads only shorten the load and store phases)
  best = 1e30f;
  int bl = 0, bthr = 0;
  for (int L : {2, 4, 8, 16}) {
    const int base = ((L * tt.ych.P + 31) / 32) * 32;
    const size_t sm = ysolve_smem(v.rows, L, fp32);
    if (base > 1024 || sm > h->smem_optin) continue;
    for (int want : {0, 256, 512, 1024}) {
      const int thr = std::max(base, want);
      if (thr > 1024 || (want > 0 && thr == base)) continue;
      tt.lpb_y = L;
      tt.threads_y = thr;
      tt.smem_y = sm;
      float ms = time_ms([&] {
        if (fp32) launch_ysolve<float>(tt, v.cols, v.rows, h->spectral32.p, open, st);
        else launch_ysolve<double>(tt, v.cols, v.rows, h->spectral.p, open, st);
      });
      if (ms < best) { best = ms; bl = L; bthr = thr; }
    }
  }
  if (bl == 0) throw CudaError("separable inverse does not fit the launch limits");
  tt.lpb_y = bl;
  tt.threads_y = bthr;
  tt.smem_y = ysolve_smem(v.rows, bl, fp32);
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  CK(cudaGetLastError());
  // GHOSTMAC_SHAPES="gthreads,gpb,L" replaces the timed choice (shape studies; every shape
  // computes the same values)
  if (const char* e = std::getenv("GHOSTMAC_SHAPES")) {
    int gt = 0, gp = 0, L = 0;
    if (std::sscanf(e, "%d,%d,%d", &gt, &gp, &L) == 3 && gt >= 32 && gt % 32 == 0 && gp >= 1 && gt * gp <= 512 &&
        tabs + per * gp <= h->smem_optin && (L == 2 || L == 4 || L == 8 || L == 16) &&
        ((L * tt.ych.P + 31) / 32) * 32 <= 1024 && ysolve_smem(v.rows, L, fp32) <= h->smem_optin) {
      tt.xg_threads = gt;
      tt.xg_pb = gp;
      tt.smem_x = tabs + per * gp;
      tt.lpb_y = L;
      tt.threads_y = ((L * tt.ych.P + 31) / 32) * 32;
      tt.smem_y = ysolve_smem(v.rows, L, fp32);
    }
  }
}

// Launch shape (row-pass group threads, groups per block, columns per column-solve block) of a
// rectangle kind, if it fits the device's limits; every shape computes the same values.
bool apply_shape(gm_handle* h, RectDev& rd, bool fp32, int gt, int gp, int L) {
  TransformTables& tt = fp32 ? rd.tt32 : rd.tt;
  const RectView& v = rd.view;
  const size_t per = std::max(xpass_smem_per_group(tt.tx_fwd, v.cols, fp32), xpass_smem_per_group(tt.tx_inv, v.cols, fp32));
  const size_t tabs = std::max(xpass_smem_tables(tt.tx_fwd, v.cols, tt.plan_x.tw_len, fp32),
                               xpass_smem_tables(tt.tx_inv, v.cols, tt.plan_x.tw_len, fp32));
  const int thr = ((L * tt.ych.P + 31) / 32) * 32;
  if (!(gt >= 32 && gt % 32 == 0 && gp >= 1 && gt * gp <= 512 && tabs + per * gp <= h->smem_optin &&
        (L == 2 || L == 4 || L == 8 || L == 16) && thr <= 1024 && ysolve_smem(v.rows, L, fp32) <= h->smem_optin))
    return false;
  tt.xg_threads = gt;
  tt.xg_pb = gp;
  tt.smem_x = tabs + per * gp;
  tt.lpb_y = L;
  tt.threads_y = thr;
  tt.smem_y = ysolve_smem(v.rows, L, fp32);
  return true;
}

// x transform tables and y partition tables of a rectangle kind
// (solver/rectangular_inverse.py:8-58: same operator, y direction solved exactly per x-mode)
void build_rect_tables(gm_handle* h, RectDev& rd, int kind, double dt) {
  const gm::Geometry& g = h->g;
  const int nx = g.nx, ny = g.ny;
  int rows = kind == 2 ? ny - 1 : ny, cols = nx;
  int tx_f, tx_i;
  if (kind == 0) { tx_f = DCT4; tx_i = DCT4; }
  else if (kind == 1) { tx_f = DST3; tx_i = DST2; }
  else { tx_f = DST4; tx_i = DST4; }
  TransformTables& tt = rd.tt;
  tt.tx_fwd = tx_f; tt.tx_inv = tx_i;
  int Mx = r2r_fft_length(tx_f, cols);
  tt.plan_x = make_plan(Mx);
  cudaStream_t st = h->st;
  rd.Wx.upload(plan_twiddles(tt.plan_x), st);
  // type IV: pre exp(-i pi (4m+1)/(4n)), post exp(-i pi k/n); Makhoul: (cos, sin)(pi k/(2n))
  if (r2r_family(tx_f) == 2) {
    rd.prex.upload(cexp_table(cols / 2, 4.0, 4.0 * cols, 1.0, -1), st);
    rd.postx.upload(cexp_table(cols / 2, 1.0, cols, 0.0, -1), st);
  } else {
    rd.prex.upload(cexp_table(1, 0, 1, 0, 1), st);
    rd.postx.upload(cexp_table(cols, 1.0, 2.0 * cols, 0.0, +1), st);
  }
  tt.Wx = rd.Wx.p; tt.prex = rd.prex.p; tt.postx = rd.postx.p;
  tt.prex_inv = rd.prex.p; tt.postx_inv = rd.postx.p;
  // column systems: pressure (L_y + lambda_x)/rho; Helmholtz (1 - c lambda_x) - c L_y, c = dt/2 nu
  tt.gamma = column_gamma(g, kind, dt);
  tt.yscale = 1.0 / (2.0 * nx);
  tt.ych = make_chunks(rows);
  std::vector<double> t0((size_t)rows * cols), t1((size_t)rows * cols), t2((size_t)rows * cols), mainj(rows);
  for (int kx = 0; kx < cols; ++kx) {
    column_diagonal(g, kind, dt, rows, kx, mainj);
    ysolve_tables(tt.ych, rows, cols, kx, mainj, tt.gamma, t0.data(), t1.data(), t2.data());
  }
  rd.t0.upload(t0, st);
  rd.t1.upload(t1, st);
  rd.t2.upload(t2, st);
  tt.t0 = rd.t0.p; tt.t1 = rd.t1.p; tt.t2 = rd.t2.p;
  if (h->precision == 1) {
    rd.t0_32.upload(to_f32(t0), st);
    rd.t1_32.upload(to_f32(t1), st);
    rd.t2_32.upload(to_f32(t2), st);
  }
  tt.n = cols;
  tt.bj0 = 0; tt.bj1 = -1; tt.cj0 = 0; tt.cj1 = -1;
  tt.bpiv = tt.phi = tt.psi = nullptr;
  if (h->precision == 1) {
    // FP32 tables and launch shapes (same plans, half the shared memory per line)
    TransformTables& t32 = rd.tt32;
    t32 = tt;
    rd.Wx32.upload(to_f32(plan_twiddles(tt.plan_x)), st);
    if (r2r_family(tx_f) == 2) {
      rd.prex32.upload(to_f32(cexp_table(cols / 2, 4.0, 4.0 * cols, 1.0, -1)), st);
      rd.postx32.upload(to_f32(cexp_table(cols / 2, 1.0, cols, 0.0, -1)), st);
    } else {
      rd.prex32.upload(to_f32(cexp_table(1, 0, 1, 0, 1)), st);
      rd.postx32.upload(to_f32(cexp_table(cols, 1.0, 2.0 * cols, 0.0, +1)), st);
    }
    t32.Wx = rd.Wx32.p; t32.prex = rd.prex32.p; t32.postx = rd.postx32.p;
    t32.prex_inv = rd.prex32.p; t32.postx_inv = rd.postx32.p;
    t32.t0 = rd.t0_32.p; t32.t1 = rd.t1_32.p; t32.t2 = rd.t2_32.p;
  }
  // view
  rd.view.rows = rows;
  rd.view.cols = cols;
  if (kind == 0) { rd.view.base = 0; rd.view.pitch = nx; rd.view.cls = h->cls_p.p; }
  else if (kind == 1) { rd.view.base = 1; rd.view.pitch = nx + 1; rd.view.cls = h->cls_f.p; }
  else { rd.view.base = h->g.usize + nx; rd.view.pitch = nx; rd.view.cls = h->cls_f.p; }
  autotune_shapes(h, rd, kind, false);
  if (h->precision == 1) autotune_shapes(h, rd, kind, true);
}

// Band solve of the Schur term T^{-1} U c.  U c is nonzero only in the rows bj0..bj1 that
// hold boundary rows, so after the x transform each column system has its right-hand side
// in the band.  Eliminating the rows below the band (pivots e, from row 0 up) and above it
// (pivots f, from the last row down) leaves the band system with modified end pivots, and
// outside the band the solution decays geometrically from the band's end values:
//   y[j] = phi[j] y[bj0],  phi[j] = prod_{i=j}^{bj0-1} (-gamma / e_i)       (j < bj0)
//   y[j] = psi[j] y[bj1],  psi[j] = prod_{i=bj1+1}^{j} (-gamma / f_i)       (j > bj1)
// The C rows read the uncorrected solution in rows cj0..cj1 only.
void build_band_tables(gm_handle* h, RectDev& rd, const std::vector<int64_t>& rows, const gm::Csr& C) {
  TransformTables& tt = rd.tt;
  const int R = rd.view.rows, cols = rd.view.cols;
  const int kind = &rd == &h->rp ? 0 : (&rd == &h->ru ? 1 : 2);
  const double dt = kind == 0 ? 0.0 : h->helm_dt;
  cudaStream_t st = h->st;
  if (rows.empty()) {
    tt.bj0 = 0; tt.bj1 = -1; tt.cj0 = 0; tt.cj1 = -1;
    rd.tt32.bj0 = 0; rd.tt32.bj1 = -1; rd.tt32.cj0 = 0; rd.tt32.cj1 = -1;
    return;
  }
  int bj0 = R, bj1 = -1, cj0 = R, cj1 = -1;
  for (int64_t r : rows) { const int j = (int)(r / cols); bj0 = std::min(bj0, j); bj1 = std::max(bj1, j); }
  for (int64_t c : C.col) { const int j = (int)(c / cols); cj0 = std::min(cj0, j); cj1 = std::max(cj1, j); }
  const int nb = bj1 - bj0 + 1;
  const double gamma = tt.gamma;
  std::vector<double> bpiv((size_t)nb * cols), phi((size_t)std::max(bj0, 1) * cols, 0.0),
      psi((size_t)std::max(R - 1 - bj1, 1) * cols, 0.0), d, e(R), f(R);
  for (int kx = 0; kx < cols; ++kx) {
    column_diagonal(h->g, kind, dt, R, kx, d);
    if (bj0 > 0) {
      e[0] = d[0];
      for (int i = 1; i < bj0; ++i) e[i] = d[i] - gamma * gamma / e[i - 1];
      double q = 1.0;
      for (int j = bj0 - 1; j >= 0; --j) {
        q *= -gamma / e[j];
        phi[(size_t)j * cols + kx] = q;
      }
    }
    if (bj1 < R - 1) {
      f[R - 1] = d[R - 1];
      for (int i = R - 2; i > bj1; --i) f[i] = d[i] - gamma * gamma / f[i + 1];
      double q = 1.0;
      for (int j = bj1 + 1; j < R; ++j) {
        q *= -gamma / f[j];
        psi[(size_t)(j - bj1 - 1) * cols + kx] = q;
      }
    }
    double prev = 0.0;
    for (int j = bj0; j <= bj1; ++j) {
      double dm = d[j];
      if (j == bj0 && bj0 > 0) dm -= gamma * gamma / e[bj0 - 1];
      if (j == bj1 && bj1 < R - 1) dm -= gamma * gamma / f[bj1 + 1];
      const double pv = j == bj0 ? dm : dm - gamma * gamma * prev;
      prev = 1.0 / pv;
      bpiv[(size_t)(j - bj0) * cols + kx] = prev;
    }
  }
  rd.bpiv.upload(bpiv, st);
  rd.phi.upload(phi, st);
  rd.psi.upload(psi, st);
  rd.band.alloc((size_t)nb * cols);
  tt.bj0 = bj0; tt.bj1 = bj1; tt.cj0 = cj0; tt.cj1 = cj1;
  tt.bpiv = rd.bpiv.p; tt.phi = rd.phi.p; tt.psi = rd.psi.p;
  if (h->precision == 1) {
    rd.bpiv32.upload(to_f32(bpiv), st);
    rd.phi32.upload(to_f32(phi), st);
    rd.psi32.upload(to_f32(psi), st);
    rd.band32.alloc((size_t)nb * cols);
    if (kind == 0) {
      std::vector<float> w((size_t)R * cols, 0.0f);
      for (int j = 0; j < bj0; ++j)
        for (int k = 0; k < cols; ++k) w[(size_t)j * cols + k] = (float)phi[(size_t)j * cols + k];
      for (int j = bj1 + 1; j < R; ++j)
        for (int k = 0; k < cols; ++k) w[(size_t)j * cols + k] = (float)psi[(size_t)(j - bj1 - 1) * cols + k];
      rd.wcorr32.upload(w, st);
    }
    TransformTables& t32 = rd.tt32;
    t32.bj0 = bj0; t32.bj1 = bj1; t32.cj0 = cj0; t32.cj1 = cj1;
    t32.bpiv = rd.bpiv32.p; t32.phi = rd.phi32.p; t32.psi = rd.psi32.p;
  }
  CK(cudaStreamSynchronize(st));
}

// The row transforms of a rectangle kind as explicit cols x cols matrices, by running the FP64
// row-transform kernel on the rows of the identity: row k of tinv (tfwd) is the inverse (forward)
// transform of e_k.
void transform_matrices(gm_handle* h, const RectDev& rd, std::vector<double>& tinv, std::vector<double>& tfwd) {
  const int n = rd.view.cols;
  const TransformTables& tt = rd.tt;
  cudaStream_t st = h->st;
  const Gate open{nullptr, 0, 0};
  const YCorr<double> none{nullptr, nullptr, nullptr, 0, -1};
  std::vector<double> eye((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) eye[(size_t)i * n + i] = 1.0;
  DBuf<double> deye, dinv, dfwd;
  deye.upload(eye, st);
  dinv.alloc((size_t)n * n);
  dfwd.alloc((size_t)n * n);
  launch_xpass<double, double, double>(tt, true, 0, n, deye.p, 0, n, nullptr, dinv.p, 0, n, nullptr, nullptr, none,
                                       open, st);
  launch_xpass<double, double, double>(tt, false, 0, n, deye.p, 0, n, nullptr, dfwd.p, 0, n, nullptr, nullptr, none,
                                       open, st);
  tinv.assign((size_t)n * n, 0.0);
  tfwd.assign((size_t)n * n, 0.0);
  CK(cudaMemcpyAsync(tinv.data(), dinv.p, tinv.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(tfwd.data(), dfwd.p, tfwd.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
}

// FP32 mode, opt-in (GHOSTMAC_ROW_GEMM=1): the pressure inverse's two row passes as split-TF32
// GEMMs against these matrices on the tensor cores (rowgemm.cu), where the grid allows it (cols
// a multiple of 4, at most 1024; the row pitch of the pressure grid is cols).  Measured on the
// 800x820 case it is the slower choice: 38 us per pass against 15 us for the FFT pass, and the
// tensor cores' FP32 accumulation over 800 products leaves the inverse less accurate than the
// FP32 FFT, so the refinement needs 4.0 instead of 2.65 pressure sweeps per step.
void build_row_gemm(gm_handle* h, RectDev& rd) {
  row_gemm_free(rd.gemm);
  const char* e = std::getenv("GHOSTMAC_ROW_GEMM");
  if (!(e && e[0] == '1')) return;
  if (h->precision != 1 || rd.view.base != 0 || rd.view.pitch != rd.view.cols) return;
  if (rd.rank > 0 && !rd.wcorr32.p) return;
  if (rd.view.cols % 4 || rd.view.cols > 1024 || row_gemm_smem_bytes() > h->smem_optin) return;
  std::vector<double> tinv, tfwd;
  transform_matrices(h, rd, tinv, tfwd);
  row_gemm_build(rd.gemm, rd.view.cols, rd.view.rows, tfwd.data(), tinv.data(), h->smem_optin, h->st);
}

// Tables of the boundary term by direct sums.  The row transforms are taken as explicit
// cols x cols matrices by running the row-transform kernel on the rows of the identity (so the
// direct sums use exactly the transforms of the FFT path), then
//   binv (mcount x cols): row q holds the inverse-transform coefficients of the point q;
//   bfwd (rank x cols, band-row order): the forward transform of a unit value at a boundary row.
// Per solve the boundary chain then costs a dot product per point, the GEMV with M and one
// sum per band entry, instead of row transforms of the C rows and of the band rows.  Grids
// whose tables would exceed 64 MB keep the row-transform chain.
void build_direct_tables(gm_handle* h, RectDev& rd, const std::vector<int64_t>& rows,
                         const std::vector<int64_t>& ucol, const std::vector<double>& M) {
  rd.direct = false;
  const int n = rd.view.cols, m = rd.mcount, rank = rd.rank;
  const TransformTables& tt = rd.tt;
  if (rank <= 0 || m <= 0 || tt.bj1 < tt.bj0) return;
  const char* e = std::getenv("GHOSTMAC_BAND_TRANSFORMS");
  if (e && e[0] == '1') return;
  if ((size_t)(m + rank) * n * 8 > ((size_t)64 << 20) ||
      band_fwd_smem(tt.bj1 - tt.bj0 + 1, rank, false) > 48 * 1024)
    return;
  cudaStream_t st = h->st;
  std::vector<double> tinv, tfwd;
  transform_matrices(h, rd, tinv, tfwd);
  // row k of tinv is the inverse transform of e_k: value at column i = tinv[k][i]
  std::vector<int32_t> mrow(m);
  std::vector<double> binv((size_t)m * n);
  for (int q = 0; q < m; ++q) {
    const int r = (int)(ucol[q] / n), i = (int)(ucol[q] % n);
    mrow[q] = r;
    for (int k = 0; k < n; ++k) binv[(size_t)q * n + k] = tinv[(size_t)k * n + i];
  }
  // boundary rows grouped by band row; row i of tfwd is the forward transform of e_i
  const int nb = tt.bj1 - tt.bj0 + 1;
  std::vector<int32_t> perm(rank), ptr(nb + 1, 0);
  for (int r = 0; r < rank; ++r) perm[r] = r;
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return rows[a] / n < rows[b] / n; });
  std::vector<double> bfwd((size_t)rank * n);
  for (int e2 = 0; e2 < rank; ++e2) {
    const int r = perm[e2];
    const int j = (int)(rows[r] / n) - tt.bj0, i = (int)(rows[r] % n);
    ++ptr[j + 1];
    for (int k = 0; k < n; ++k) bfwd[(size_t)e2 * n + k] = tfwd[(size_t)i * n + k];
  }
  for (int j = 0; j < nb; ++j) ptr[j + 1] += ptr[j];
  rd.mrow.upload(mrow, st);
  rd.bptr.upload(ptr, st);
  std::vector<double> mband((size_t)rank * rd.mcount);
  for (int e2 = 0; e2 < rank; ++e2)
    std::copy_n(&M[(size_t)perm[e2] * rd.mcount], rd.mcount, &mband[(size_t)e2 * rd.mcount]);
  rd.mband.upload(mband, st);
  rd.binv.upload(binv, st);
  rd.bfwd.upload(bfwd, st);
  rd.cvec.alloc(rank);
  rd.firstm.alloc(m);
  if (h->precision == 1) {
    rd.binv32.upload(to_f32(binv), st);
    rd.bfwd32.upload(to_f32(bfwd), st);
    rd.firstm32.alloc(m);
  }
  // Opt-in (GHOSTMAC_BAND_FOLDED=1): G = M binv over the spectrum rows cj0..cj1, one sum per
  // Schur value per solve instead of the point values and a GEMV.  Measured on the 800x820
  // case it loses: in the FP32 mode the rounding of G and the long FP32 sums leave the inverse
  // less accurate (4.0 instead of 2.8 pressure sweeps per step, 0.774 against 0.701 ms), and the
  // plain FP64 step gains nothing (0.973 against 0.957 ms).
  rd.glen = 0;
  const char* eg = std::getenv("GHOSTMAC_BAND_FOLDED");
  const int L = (tt.cj1 - tt.cj0 + 1) * n;
  if ((eg && eg[0] == '1') && tt.cj1 >= tt.cj0 && (size_t)rank * L * 8 <= ((size_t)64 << 20)) {
    std::vector<double> G((size_t)rank * L, 0.0);
    for (int r = 0; r < rank; ++r) {
      double* gr = &G[(size_t)r * L];
      for (int q = 0; q < m; ++q) {
        const double a = mband[(size_t)r * m + q];
        if (a == 0.0) continue;
        double* dst = gr + (size_t)(mrow[q] - tt.cj0) * n;
        const double* src = &binv[(size_t)q * n];
        for (int k = 0; k < n; ++k) dst[k] += a * src[k];
      }
    }
    if (h->precision == 1) rd.gmat32.upload(to_f32(G), st);
    else rd.gmat.upload(G, st);
    rd.cpart.alloc((size_t)rank * BAND_SPLIT);
    rd.glen = L;
  }
  CK(cudaStreamSynchronize(st));
  rd.direct = true;
}

// Schur matrix S = I + C T^{-1} U by impulse solves, LU, explicit inverse (solver/pressure_schur.py:92-101)
void build_schur(gm_handle* h, RectDev& rd, const std::vector<int64_t>& rows, const gm::Csr& C, double* field_buf) {
  cudaStream_t st = h->st;
  rd.rank = (int)rows.size();
  // device copies hold field-grid flat indices (no index arithmetic in the kernels)
  auto field_index = [&](int64_t rc) { return rd.view.base + (rc / rd.view.cols) * rd.view.pitch + rc % rd.view.cols; };
  std::vector<int64_t> frows(rows.size()), fcol(C.col.size());
  for (size_t k = 0; k < rows.size(); ++k) frows[k] = field_index(rows[k]);
  for (size_t k = 0; k < C.col.size(); ++k) fcol[k] = field_index(C.col[k]);
  rd.rows.upload(frows, st);
  rd.cptr.upload(C.ptr, st);
  rd.ccol.upload(fcol, st);
  rd.cval.upload(C.val, st);
  const int n = rd.rank;
  if (n == 0) { rd.sinv.alloc(0); return; }
  DBuf<double> S;
  S.alloc((size_t)n * n);
  // field_buf is a full-grid buffer used as the impulse; h->ftmp / ptmp holds T^{-1} e
  double* first = (rd.view.cls == h->cls_p.p) ? h->ptmp.p : h->ftmp.p;
  size_t span = (rd.view.cls == h->cls_p.p) ? (size_t)h->Pn : (size_t)h->F;
  CK(cudaMemsetAsync(field_buf, 0, span * sizeof(double), st));
  const double one = 1.0, zero = 0.0;
  Gate open{nullptr, 0, 0};
  for (int c = 0; c < n; ++c) {
    int64_t rc = rows[c];
    int64_t fi = rd.view.base + (rc / rd.view.cols) * rd.view.pitch + rc % rd.view.cols;
    CK(cudaMemcpyAsync(field_buf + fi, &one, sizeof(double), cudaMemcpyHostToDevice, st));
    plain_inverse<double, double, double>(rd.tt, rd.view, field_buf, false, h->spectral.p, first, nullptr, nullptr,
                                          open, st);
    launch_schur_column(first, rd.view, n, rd.cptr.p, rd.ccol.p, rd.cval.p, S.p, c, st);
    CK(cudaMemcpyAsync(field_buf + fi, &zero, sizeof(double), cudaMemcpyHostToDevice, st));
  }
  CK(cudaGetLastError());
  std::vector<double> hs((size_t)n * n);
  CK(cudaMemcpyAsync(hs.data(), S.p, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int i = 0; i < n; ++i) hs[(size_t)i * n + i] += 1.0;
  std::vector<int> piv(n);
  if (!gm::lu_factor(n, hs.data(), piv.data())) throw GateError(GM_ERUNTIME, "Singular boundary Schur matrix");
  std::vector<double> inv((size_t)n * n);
  gm::lu_inverse(n, hs.data(), piv.data(), inv.data());
  rd.sinv.upload(inv, st);
  // M = S^{-1} C as a dense rank x m matrix over the m distinct points C reads, so that one
  // gather and one GEMV give c = S^{-1} (C first) per solve
  std::vector<int64_t> ucol(C.col.begin(), C.col.end());
  std::sort(ucol.begin(), ucol.end());
  ucol.erase(std::unique(ucol.begin(), ucol.end()), ucol.end());
  const int m = (int)ucol.size();
  if ((size_t)m * sizeof(double) > 48 * 1024) throw CudaError("boundary Schur term reads too many points");
  std::vector<double> cd((size_t)n * m, 0.0), M((size_t)n * m, 0.0);
  for (int r = 0; r < n; ++r)
    for (int64_t e = C.ptr[r]; e < C.ptr[r + 1]; ++e) {
      const int q = (int)(std::lower_bound(ucol.begin(), ucol.end(), C.col[e]) - ucol.begin());
      cd[(size_t)r * m + q] += C.val[e];
    }
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k) {
      const double a = inv[(size_t)r * n + k];
      if (a == 0.0) continue;
      const double* src = &cd[(size_t)k * m];
      double* dst = &M[(size_t)r * m];
      for (int q = 0; q < m; ++q) dst[q] += a * src[q];
    }
  std::vector<int64_t> mcol(m);
  for (int q = 0; q < m; ++q) mcol[q] = field_index(ucol[q]);
  rd.mcols.upload(mcol, st);
  rd.mmat.upload(M, st);
  rd.mcount = m;
  build_band_tables(h, rd, rows, C);
  build_direct_tables(h, rd, rows, ucol, M);
}

// Regular-row coefficients of the residual kernels (see ResidualCoef): the pressure operator
// (solver/optimized_ghost_cell.py:80-107, A = D G with the outlet -2/dx) and the Helmholtz
// rows I - c L, c = dt nu / 2 (raw_l of solver/optimized_ghost_cell.py:116-123).
ResidualCoef residual_coef(const gm::Geometry& g, int kind, double hc) {
  ResidualCoef r{};
  const double idx2 = 1.0 / (g.dx * g.dx), idy2 = 1.0 / (g.dy * g.dy), irho = 1.0 / g.rho;
  if (kind == 0) {
    const double mx[3] = {-1.0, -2.0, -3.0}, my[2] = {-1.0, -2.0};
    for (int ic = 0; ic < 3; ++ic)
      for (int jc = 0; jc < 2; ++jc) r.cc[ic][jc] = (mx[ic] * idx2 + my[jc] * idy2) * irho;
    for (int ic = 0; ic < 3; ++ic) r.cw[ic] = idx2 * irho;
    r.ce = idx2 * irho;
    r.cy = idy2 * irho;
  } else if (kind == 1) {
    const double my[2] = {-3.0, -2.0};
    for (int ic = 0; ic < 3; ++ic)
      for (int jc = 0; jc < 2; ++jc) r.cc[ic][jc] = 1.0 - hc * (-2.0 * idx2 + my[jc] * idy2);
    r.cw[0] = r.cw[1] = -hc * idx2;
    r.cw[2] = -hc * (2.0 * idx2);  // outlet face: raw_l doubles the west coupling
    r.ce = -hc * idx2;
    r.cy = -hc * idy2;
  } else {
    const double mx[3] = {-3.0, -2.0, -1.0};
    for (int ic = 0; ic < 3; ++ic)
      for (int jc = 0; jc < 2; ++jc) r.cc[ic][jc] = 1.0 - hc * (mx[ic] * idx2 - 2.0 * idy2);
    for (int ic = 0; ic < 3; ++ic) r.cw[ic] = -hc * idx2;
    r.ce = -hc * idx2;
    r.cy = -hc * idy2;
  }
  for (int a = 0; a < 3; ++a) {
    for (int c = 0; c < 2; ++c) r.fcc[a][c] = (float)r.cc[a][c];
    r.fcw[a] = (float)r.cw[a];
  }
  r.fce = (float)r.ce;
  r.fcy = (float)r.cy;
  return r;
}

void fill_case_dev(gm_handle* h) {
  const gm::Geometry& g = h->g;
  CaseDev& c = h->cd;
  c.nx = g.nx; c.ny = g.ny; c.dx = g.dx; c.dy = g.dy; c.rho = g.rho; c.nu = g.nu;
  c.idx = 1.0 / g.dx; c.idy = 1.0 / g.dy;
  c.idx2 = 1.0 / (g.dx * g.dx); c.idy2 = 1.0 / (g.dy * g.dy);
  c.gx = (1.0 / g.dx) / g.rho; c.gy = (1.0 / g.dy) / g.rho;
  c.iarea = 1.0 / (g.dx * g.dy); c.irho = 1.0 / g.rho;
  c.usize = g.usize; c.vsize = g.vsize; c.psize = g.psize;
  c.cls_u = h->cls_u; c.cls_v = h->cls_v; c.cls_p = h->cls_p.p;
  c.inlet = h->inlet.p;
  c.n_ghost_f = h->gf.n; c.gf_rows = h->gf.rows.p; c.gf_ptr = h->gf.ptr.p; c.gf_col = h->gf.col.p; c.gf_val = h->gf.val.p;
  c.n_ghost_p = h->gp.n; c.gp_rows = h->gp.rows.p; c.gp_ptr = h->gp.ptr.p; c.gp_col = h->gp.col.p; c.gp_val = h->gp.val.p;
  for (int k = 0; k < 3; ++k) {
    c.n_irr[k] = h->irr[k].n; c.irr_rows[k] = h->irr[k].rows.p; c.irr_ptr[k] = h->irr[k].ptr.p;
    c.irr_index[k] = h->irr[k].index.p;
    c.irr_col[k] = h->irr[k].col.p; c.irr_val[k] = h->irr[k].val.p;
  }
  c.a_nnz = h->a_nnz.p;
  c.n_surf = g.n_surface;
  c.sp_ptr = h->sp_ptr.p; c.sp_col = h->sp_col.p; c.sp_val = h->sp_val.p;
  c.su_ptr = h->su_ptr.p; c.su_col = h->su_col.p; c.su_val = h->su_val.p;
  c.sv_ptr = h->sv_ptr.p; c.sv_col = h->sv_col.p; c.sv_val = h->sv_val.p;
  c.nwx = h->nwx.p; c.nwy = h->nwy.p; c.nxx = h->nxx.p; c.nyy = h->nyy.p;
  c.surf_part = h->surf_part.p; c.surf_ticket = h->surf_ticket.p;
  h->rcoef[0] = residual_coef(g, 0, 0.0);
  if (h->helm_ready) {
    const double hc = (0.5 * h->helm_dt) * g.nu;
    h->rcoef[1] = residual_coef(g, 1, hc);
    h->rcoef[2] = residual_coef(g, 2, hc);
  }
  c.D = g.D; c.U_ref = g.U_ref;
  c.fdx = (float)c.dx; c.fdy = (float)c.dy; c.fidx2 = (float)c.idx2; c.fidy2 = (float)c.idy2;
  c.fiarea = (float)c.iarea; c.fnu = (float)c.nu; c.fgx = (float)c.gx; c.fgy = (float)c.gy;
}

void build_class_maps(gm_handle* h) {
  const gm::Geometry& g = h->g;
  std::vector<uint8_t> cu(g.usize), cv(g.vsize), cp(g.psize);
  for (int64_t f = 0; f < g.usize; ++f) cu[f] = (g.act_u[f] ? CLS_ACTIVE : 0) | (g.ghost_of_u[f] >= 0 ? CLS_GHOST : 0);
  for (int64_t f = 0; f < g.vsize; ++f) cv[f] = (g.act_v[f] ? CLS_ACTIVE : 0) | (g.ghost_of_v[f] >= 0 ? CLS_GHOST : 0);
  for (int64_t f = 0; f < g.psize; ++f) cp[f] = (g.act_p[f] ? CLS_ACTIVE : 0) | (g.ghost_of_p[f] >= 0 ? CLS_GHOST : 0);
  for (int64_t r : g.a_rows) cp[r] |= CLS_IRREG;
  if (h->helm_ready) {
    for (int64_t r : h->hs.rows_irr[0]) cu[r] |= CLS_IRREG;
    for (int64_t r : h->hs.rows_irr[1]) cv[r] |= CLS_IRREG;
  }
  std::vector<uint8_t> cf(cu);
  cf.insert(cf.end(), cv.begin(), cv.end());
  if (h->cls_f.n != cf.size()) h->cls_f.alloc(cf.size());
  CK(cudaMemcpyAsync(h->cls_f.p, cf.data(), cf.size(), cudaMemcpyHostToDevice, h->st));
  if (h->cls_p.n != cp.size()) h->cls_p.alloc(cp.size());
  CK(cudaMemcpyAsync(h->cls_p.p, cp.data(), cp.size(), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->cls_u = h->cls_f.p;
  h->cls_v = h->cls_f.p + g.usize;
}

// device copy-in/out helpers
const double* dev_in(gm_handle* h, int slot, const double* p, size_t n) {
  if (is_device_ptr(p)) return p;
  if (h->io[slot].n < n) h->io[slot].alloc(n);
  CK(cudaMemcpyAsync(h->io[slot].p, p, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  return h->io[slot].p;
}
struct DevOut {
  gm_handle* h;
  double* user;
  double* dev;
  size_t n;
  bool copy;
  DevOut(gm_handle* hh, int slot, double* p, size_t count) : h(hh), user(p), n(count) {
    copy = !is_device_ptr(p);
    if (copy) {
      if (h->io[slot].n < n) h->io[slot].alloc(n);
      dev = h->io[slot].p;
    } else {
      dev = p;
    }
  }
  void finish() {
    if (copy && user) CK(cudaMemcpyAsync(user, dev, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  }
};

void check_ctl(gm_handle* h, const char* where) {
  CK(cudaMemcpyAsync(h->host_ctl, h->ctl.p, sizeof(StepCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const StepCtl& c = *h->host_ctl;
  if (c.err) {
    static const char* names[] = {"", "Ghost projection failed", "CN momentum solve failed", "Pressure solve failed",
                                  "Pressure RHS must be finite", "Ghost step failed divergence/CFL gate",
                                  "Non-finite force", "Explicit timestep unsafe", "Finite fields and a positive timestep are required"};
    std::string m = std::string(names[c.gate < 9 ? c.gate : 0]) + " (" + where + ")";
    throw GateError(c.err, m);
  }
}

// --- building blocks of the step ---------------------------------------------

void ghost_faces(gm_handle* h, double* U, const Gate& gt) {
  launch_ghost(U, h->gf.n, h->gf.rows.p, h->gf.ptr.p, h->gf.col.p, h->gf.val.p, gt, h->st);
}
void ghost_p(gm_handle* h, double* P, const Gate& gt) {
  launch_ghost(P, h->gp.n, h->gp.rows.p, h->gp.ptr.p, h->gp.col.p, h->gp.val.p, gt, h->st);
}

// one boundary-row solve of kind k into x with residual checks (solver/pressure_schur.py:103-124)
// In the FP32 mode every application of the inverse runs in FP32 and the residual
// b - A x in FP64, so the refinement sweeps recover an FP64 solution.
// One application of the (FP64 or FP32) boundary-corrected inverse: x = [x +] T^{-1} r - T^{-1} U S^{-1} C T^{-1} r.
// x = [x +] A_rect^{-1} r with the boundary Schur correction (solver/pressure_schur.py:75-124):
//   S1 = Y^{-1} F_x r (spectral, all rows); first = F_x^{-1} S1 on the rows the C rows read;
//   c = S^{-1} C first; B = band solve of F_x (U c); x = F_x^{-1} (S1 - B extended by phi/psi).
void sweep_mark(gm_handle* h, int k, cudaStream_t st);

template <typename T>
void schur_inverse(gm_handle* h, RectDev& rd, const TransformTables& tt, const void* r, bool r_f32, double* x,
                   bool accumulate, T* spectral, T* first, T* band, double* w2, const Gate& g, cudaStream_t st) {
  const RectView& v = rd.view;
  const YCorr<T> none{nullptr, nullptr, nullptr, 0, -1};
  // FP32 pressure inverse: both row passes on the tensor cores when their arrays have tensor maps
  bool gemm_fwd = false, gemm_inv = false;
  if constexpr (sizeof(T) == 4) {
    if (rd.gemm.n > 0) {
      gemm_fwd = row_gemm_ready(rd.gemm, r, r_f32 ? 4 : 8);
      gemm_inv = row_gemm_ready(rd.gemm, spectral, 4) && (rd.rank == 0 || row_gemm_ready(rd.gemm, rd.wcorr32.p, 4));
    }
    // with the tensor-core inverse pass the band solve writes its rows into the table W
    if (gemm_inv && rd.rank > 0) band = (T*)(rd.wcorr32.p + (int64_t)tt.bj0 * v.cols);
  }
  sweep_mark(h, 0, st);
  if constexpr (sizeof(T) == 4) {
    if (gemm_fwd) {
      if (r_f32) launch_row_gemm_fwd<float>(rd.gemm, (const float*)r, (float*)spectral, g, st);
      else launch_row_gemm_fwd<double>(rd.gemm, (const double*)r, (float*)spectral, g, st);
    } else if (r_f32)
      launch_xpass<float, float, float>(tt, false, 0, v.rows, (const float*)r, v.base, v.pitch, v.cls, spectral, 0,
                                        v.cols, nullptr, nullptr, none, g, st);
    else
      launch_xpass<float, double, float>(tt, false, 0, v.rows, (const double*)r, v.base, v.pitch, v.cls, spectral, 0,
                                         v.cols, nullptr, nullptr, none, g, st);
  } else {
    launch_xpass<double, double, double>(tt, false, 0, v.rows, (const double*)r, v.base, v.pitch, v.cls, spectral, 0,
                                         v.cols, nullptr, nullptr, none, g, st);
  }
  sweep_mark(h, 1, st);
  launch_ysolve<T>(tt, v.cols, v.rows, spectral, g, st);
  sweep_mark(h, 2, st);
  YCorr<T> corr = none;
  if (rd.rank > 0 && rd.direct) {
    const bool f32 = sizeof(T) == 4;
    const double* cv = rd.cvec.p;
    int nsplit = 1;
    if (rd.glen > 0) {
      launch_band_direct<T>(rd.rank, rd.glen, f32 ? (const T*)rd.gmat32.p : (const T*)rd.gmat.p,
                            spectral + (int64_t)tt.cj0 * v.cols, rd.cpart.p, g, st);
      sweep_mark(h, 3, st);
      sweep_mark(h, 4, st);
      cv = rd.cpart.p;
      nsplit = BAND_SPLIT;
    } else {
      T* fm = f32 ? (T*)rd.firstm32.p : (T*)rd.firstm.p;
      launch_band_first<T>(rd.mcount, v.cols, rd.mrow.p, f32 ? (const T*)rd.binv32.p : (const T*)rd.binv.p, spectral,
                           fm, g, st);
      sweep_mark(h, 3, st);
      launch_band_gemv<T>(rd.rank, rd.mcount, rd.mband.p, fm, rd.cvec.p, g, st);
      sweep_mark(h, 4, st);
    }
    launch_band_fwd_solve<T>(tt, v.cols, rd.rank, rd.bptr.p, cv, f32 ? (const T*)rd.bfwd32.p : (const T*)rd.bfwd.p,
                             band, g, st, nsplit);
    sweep_mark(h, 5, st);
    corr = YCorr<T>{band, (const T*)tt.phi, (const T*)tt.psi, tt.bj0, tt.bj1};
  } else if (rd.rank > 0) {
    launch_xpass<T, T, T>(tt, true, tt.cj0, tt.cj1 - tt.cj0 + 1, spectral, 0, v.cols, nullptr, first, v.base, v.pitch,
                          nullptr, nullptr, none, g, st);
    sweep_mark(h, 3, st);
    launch_schur<T>(first, rd.rank, rd.mcount, rd.mcols.p, rd.mmat.p, rd.rows.p, w2, g, st);
    sweep_mark(h, 4, st);
    launch_xpass<T, double, T>(tt, false, tt.bj0, tt.bj1 - tt.bj0 + 1, w2, v.base, v.pitch, nullptr, band,
                               -(int64_t)tt.bj0 * v.cols, v.cols, nullptr, nullptr, none, g, st);
    sweep_mark(h, 5, st);
    launch_yband<T>(tt, v.cols, band, g, st);
    corr = YCorr<T>{band, (const T*)tt.phi, (const T*)tt.psi, tt.bj0, tt.bj1};
  } else {
    for (int k = 3; k <= 5; ++k) sweep_mark(h, k, st);
  }
  sweep_mark(h, 6, st);
  bool inv_done = false;
  if constexpr (sizeof(T) == 4)
    if (gemm_inv)
      inv_done = launch_row_gemm_inv(rd.gemm, (const float*)spectral, rd.rank > 0 ? rd.wcorr32.p : nullptr, tt.bj0,
                                     tt.bj1, x, v.base, v.pitch, v.cls, accumulate ? x : nullptr, g, st);
  if (!inv_done)
    launch_xpass<T, T, double>(tt, true, 0, v.rows, spectral, 0, v.cols, nullptr, x, v.base, v.pitch, v.cls,
                               accumulate ? x : nullptr, corr, g, st);
  sweep_mark(h, 7, st);
}

// r is the FP64 right-hand side, or in the FP32 mode the FP32 residual when r_f32 is set
void helm_jacobi_apply(gm_handle* h, int kind, const void* r, bool r_f32, double* x, bool accumulate,
                       const Gate& g, cudaStream_t st);
void apply_inverse(gm_handle* h, int lane, RectDev& rd, int kind, const void* r, bool r_f32, double* x,
                   bool accumulate, double* first, double* w2, const Gate& gt, cudaStream_t st) {
  if (h->precision == 1 && kind != 0 && h->jac_iters > 0) {
    helm_jacobi_apply(h, kind, r, r_f32, x, accumulate, gt, st);
    return;
  }
  if (h->precision == 1) {
    float* first32 = kind == 0 ? h->pfirst32.p : h->ffirst32.p;
    float* spec = lane == 0 ? h->spectral32.p : h->spectral32_b.p;
    schur_inverse<float>(h, rd, rd.tt32, r, r_f32, x, accumulate, spec, first32, rd.band32.p, w2, gt, st);
  } else {
    double* spec = lane == 0 ? h->spectral.p : h->spectral_b.p;
    schur_inverse<double>(h, rd, rd.tt, r, false, x, accumulate, spec, first, rd.band.p, w2, gt, st);
  }
}

// The same solve while the step is being captured into a CUDA graph: the refinement
// sweeps form a WHILE conditional node whose body runs only while the residual check
// exceeds the target, so no sweep kernel launches when none is needed.
void schur_solve_graph(gm_handle* h, int lane, RectDev& rd, int kind, double hc, const double* b, double* x,
                       double* res, double* first, double* w2, int slot) {
  cudaStream_t st = lane == 0 ? h->st : h->st2;
  cudaStream_t body_st = lane == 0 ? h->st_body : h->st2_body;
  SolveCtl* sc = &h->ctl.p->solve[slot];
  Gate g0 = gate_of(h, slot, 0);
  const bool f32 = h->precision == 1;
  void* resb = f32 ? (void*)(kind == 0 ? h->pres32.p : h->fres32.p) : (void*)res;
  (void)hc;
  h->sweep_marking = h->phase_on && slot == S_P1;
  apply_inverse(h, lane, rd, kind, b, false, x, false, first, w2, g0, st);
  launch_residual(h->cd, h->rcoef[kind], kind, b, x, resb, f32, sc, 0, true, g0, st);
  sweep_mark(h, 8, st);
  h->sweep_marking = false;
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, nullptr, nullptr, nullptr));
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, graph, 0, 0));
  launch_refine_decide(h->ctl.p, slot, h->nchk, cond, st);
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  CK(cudaGraphAddNode(&cnode, graph, deps, nullptr, nd, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  CK(cudaStreamBeginCaptureToGraph(body_st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  long long c0 = kernel_launch_count();
  apply_inverse(h, lane, rd, kind, resb, f32, x, true, first, w2, g0, body_st);
  launch_residual(h->cd, h->rcoef[kind], kind, b, x, resb, f32, sc, -1, false, g0, body_st);
  launch_refine_decide(h->ctl.p, slot, h->nchk, cond, body_st);
  h->body_nodes_slot[slot] = kernel_launch_count() - c0;
  CK(cudaStreamEndCapture(body_st, &body));
}

// Flexible GMRES(50) for A x = b on the pressure grid, right-preconditioned by the separable
// rectangle inverse (no boundary term) -- solver/pressure_schur.py:20-41 with
// gmres(rtol=atol=1e-12, restart=50, maxiter=100): at most 100 restart cycles, convergence
// on the residual 2-norm <= max(rtol ||b||, atol).  Classical Gram-Schmidt with one
// re-orthogonalisation; the Hessenberg least-squares update (Givens rotations) runs on the
// host, one small read-back per iteration.  Returns 0 when converged, else the iteration count.
// With a learned network attached and `learned` set, the first Arnoldi direction of the first
// cycle (whose residual is b itself, the distribution the network was trained on) is
// preconditioned by T^-1 + s net; every later direction by T^-1 alone (a flexible
// preconditioner may change from one direction to the next).
int fgmres(gm_handle* h, const double* b, double* x, int& iterations, bool learned) {
  const int m = gm_handle::GMRES_M;
  const int64_t n = h->Pn;
  cudaStream_t st = h->st;
  if (!h->gV.p) {
    h->gV.alloc((size_t)(m + 1) * n);
    h->gZ.alloc((size_t)m * n);
    h->gdx.alloc(n);
    h->gpart.alloc((size_t)multidot_blocks(n) * 64);
    h->gdots.alloc(64);
    h->gcoef.alloc(64);
  }
  RectDev& rd = h->rp;
  const Gate open{nullptr, 0, 0};
  double* V = h->gV.p;
  double* Z = h->gZ.p;
  auto vec = [&](double* base, int i) { return base + (int64_t)i * n; };
  auto dots = [&](const double* Vb, int nv, const double* w, double* out_host) {
    launch_multidot(Vb, n, nv, w, n, h->gpart.p, h->gdots.p, st);
    CK(cudaMemcpyAsync(out_host, h->gdots.p, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  };
  auto precondition = [&](const double* v, double* z, bool use_net) {
    if (h->precision == 1)
      plain_inverse<float, double, double>(rd.tt32, rd.view, v, true, h->spectral32.p, z, rd.view.cls, nullptr, open,
                                           st);
    else
      plain_inverse<double, double, double>(rd.tt, rd.view, v, true, h->spectral.p, z, rd.view.cls, nullptr, open, st);
    if (use_net) {
      // z += s net([v / s, mask]), s = max |v|  (FP32 network, FGMRES absorbs its nonlinearity)
      float* xin = nullptr;
      gm_unet_input(h->lnet, &xin);
      CK(cudaMemsetAsync(h->lscale.p, 0, sizeof(unsigned long long), st));
      launch_learned_prep(h->cd, v, xin, h->lscale.p, st);
      if (gm_unet_forward(h->lnet, h->lw.data(), h->lb.data(), nullptr, h->lout.p, st) != GM_OK)
        throw CudaError(std::string("learned preconditioner: ") + gm_unet_last_error(h->lnet));
      launch_learned_apply(h->cd, h->lout.p, h->lscale.p, z, st);
    }
  };
  double bn2 = 0;
  dots(b, 1, b, &bn2);
  const double tol = std::max(1e-12 * std::sqrt(bn2), 1e-12);
  CK(cudaMemsetAsync(x, 0, n * sizeof(double), st));
  iterations = 0;
  bool converged = false, x_zero = true;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hc(m + 1), hc2(m + 1), y(m);
  for (int cycle = 0; cycle < 100 && !converged; ++cycle) {
    // V0 = b - A x
    CK(cudaMemcpyAsync(vec(V, 0), b, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (!x_zero) {
      launch_apply_pressure(h->cd, h->rcoef[0], x, vec(V, 1), open, st);
      const double one = 1.0;
      CK(cudaMemcpyAsync(h->gcoef.p, &one, sizeof one, cudaMemcpyHostToDevice, st));
      launch_multiaxpy(vec(V, 1), n, 1, h->gcoef.p, -1.0, 1.0, vec(V, 0), n, st);
    }
    double beta2 = 0;
    dots(vec(V, 0), 1, vec(V, 0), &beta2);
    const double beta = std::sqrt(beta2);
    if (!(beta > tol)) { converged = std::isfinite(beta); break; }
    launch_multiaxpy(nullptr, n, 0, h->gcoef.p, 0.0, 1.0 / beta, vec(V, 0), n, st);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jend = -1;
    for (int j = 0; j < m; ++j) {
      precondition(vec(V, j), vec(Z, j), learned && h->lnet && cycle == 0 && j == 0);
      double* w = vec(V, j + 1);
      launch_apply_pressure(h->cd, h->rcoef[0], vec(Z, j), w, open, st);
      // two classical Gram-Schmidt passes against V_0..V_j
      dots(V, j + 1, w, hc.data());
      launch_multiaxpy(V, n, j + 1, h->gdots.p, -1.0, 1.0, w, n, st);
      dots(V, j + 1, w, hc2.data());
      launch_multiaxpy(V, n, j + 1, h->gdots.p, -1.0, 1.0, w, n, st);
      for (int i = 0; i <= j; ++i) hc[i] += hc2[i];
      double wn2 = 0;
      dots(w, 1, w, &wn2);
      hc[j + 1] = std::sqrt(wn2);
      if (hc[j + 1] > 0) launch_multiaxpy(nullptr, n, 0, h->gcoef.p, 0.0, 1.0 / hc[j + 1], w, n, st);
      // Givens rotations on the new Hessenberg column
      for (int i = 0; i < j; ++i) {
        const double a = cs[i] * hc[i] + sn[i] * hc[i + 1];
        hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
        hc[i] = a;
      }
      const double den = std::hypot(hc[j], hc[j + 1]);
      cs[j] = den > 0 ? hc[j] / den : 1.0;
      sn[j] = den > 0 ? hc[j + 1] / den : 0.0;
      hc[j] = den;
      hc[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hc[i];
      ++iterations;
      jend = j;
      if (!std::isfinite(g[j + 1])) break;
      if (std::abs(g[j + 1]) <= tol) { converged = true; break; }
    }
    if (jend < 0) break;
    // y = R^{-1} g, x += Z y
    for (int i = jend; i >= 0; --i) {
      double acc = g[i];
      for (int k = i + 1; k <= jend; ++k) acc -= H[(size_t)i * m + k] * y[k];
      y[i] = acc / H[(size_t)i * m + i];
    }
    CK(cudaMemcpyAsync(h->gcoef.p, y.data(), (jend + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_multiaxpy(Z, n, jend + 1, h->gcoef.p, 1.0, 1.0, x, n, st);
    CK(cudaStreamSynchronize(st));
    x_zero = false;
  }
  return converged ? 0 : std::max(1, iterations);
}

// The same FGMRES(50) with its control on the device (kernels.cu, GmresDev): one graph per
// (b, x) pair, built on first use and replayed after.  Restart cycles form a WHILE node; each
// of the 50 Arnoldi steps of a cycle is an IF node whose condition the previous step sets, so
// a solve launches the kernels of the steps it takes and reads nothing back until it ends.
// The learned preconditioner keeps the host-driven fgmres above.
static_assert(gm_handle::GMRES_M == GmresDev::M, "GMRES restart length");

cudaGraphNode_t add_conditional(cudaStream_t st, cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType type,
                                cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, graph, deps, nullptr, nd, &cp));
  *body = cp.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return node;
}

gm_handle::GmresExec& gmres_graph(gm_handle* h, const double* b, double* x) {
  for (auto& ge : h->gexec)
    if (ge.b == b && ge.x == x && ge.exec) return ge;
  const int m = gm_handle::GMRES_M;
  const int64_t n = h->Pn;
  if (!h->gdev.p) {
    h->gdev.alloc(1);
    for (DBuf<double>* d : {&h->gd1, &h->gd2, &h->gy}) d->alloc(64);
    for (DBuf<double>* d : {&h->gwn, &h->gbeta, &h->gbn, &h->gone}) d->alloc(1);
    h->gnv.alloc(1);
    const double one = 1.0;
    CK(cudaMemcpyAsync(h->gone.p, &one, sizeof one, cudaMemcpyHostToDevice, h->st));
  }
  RectDev& rd = h->rp;
  const Gate open{nullptr, 0, 0};
  double* V = h->gV.p;
  double* Z = h->gZ.p;
  auto vec = [&](double* base, int i) { return base + (int64_t)i * n; };
  cudaStream_t st = h->st, sb1 = h->st_body, sb2 = h->st2_body;
  auto precondition = [&](const double* v, double* z, cudaStream_t s) {
    if (h->precision == 1)
      plain_inverse<float, double, double>(rd.tt32, rd.view, v, true, h->spectral32.p, z, rd.view.cls, nullptr, open,
                                           s);
    else
      plain_inverse<double, double, double>(rd.tt, rd.view, v, true, h->spectral.p, z, rd.view.cls, nullptr, open, s);
  };
  gm_handle::GmresExec ge;
  ge.b = b;
  ge.x = x;
  const long long c0 = kernel_launch_count();
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  launch_multidot(b, n, 1, b, n, h->gpart.p, h->gbn.p, st);
  CK(cudaMemsetAsync(x, 0, n * sizeof(double), st));
  cudaStreamCaptureStatus cs;
  cudaGraph_t top;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &top, nullptr, nullptr, nullptr));
  cudaGraphConditionalHandle cyc;
  CK(cudaGraphConditionalHandleCreate(&cyc, top, 0, 0));
  launch_gm_init(h->gdev.p, h->gbn.p, cyc, st);
  ge.fixed = kernel_launch_count() - c0;
  cudaGraph_t cycle_body;
  add_conditional(st, cyc, cudaGraphCondTypeWhile, &cycle_body);
  CK(cudaStreamBeginCaptureToGraph(sb1, cycle_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const long long c1 = kernel_launch_count();
  // V0 = (b - A x) / ||b - A x||
  launch_apply_pressure(h->cd, h->rcoef[0], x, vec(V, 1), open, sb1);
  CK(cudaMemcpyAsync(vec(V, 0), b, n * sizeof(double), cudaMemcpyDeviceToDevice, sb1));
  launch_multiaxpy(vec(V, 1), n, 1, h->gone.p, -1.0, 1.0, vec(V, 0), n, sb1);
  launch_multidot(vec(V, 0), n, 1, vec(V, 0), n, h->gpart.p, h->gbeta.p, sb1);
  GmresHandles hs{};
  hs.count = m;
  cudaGraph_t cyc_graph;
  CK(cudaStreamGetCaptureInfo(sb1, &cs, nullptr, &cyc_graph, nullptr, nullptr, nullptr));
  for (int j = 0; j < m; ++j) CK(cudaGraphConditionalHandleCreate(&hs.step[j], cyc_graph, 0, 0));
  launch_gm_cycle_begin(h->gdev.p, h->gbeta.p, hs, sb1);
  launch_gm_scale(vec(V, 0), n, h->gdev.p, sb1);
  long long per_step = 0;
  for (int j = 0; j < m; ++j) {
    cudaGraph_t step_body;
    add_conditional(sb1, hs.step[j], cudaGraphCondTypeIf, &step_body);
    CK(cudaStreamBeginCaptureToGraph(sb2, step_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const long long c2 = kernel_launch_count();
    double* w = vec(V, j + 1);
    precondition(vec(V, j), vec(Z, j), sb2);
    launch_apply_pressure(h->cd, h->rcoef[0], vec(Z, j), w, open, sb2);
    // two classical Gram-Schmidt passes against V_0..V_j, then the norm
    launch_multidot(V, n, j + 1, w, n, h->gpart.p, h->gd1.p, sb2);
    launch_multiaxpy(V, n, j + 1, h->gd1.p, -1.0, 1.0, w, n, sb2);
    launch_multidot(V, n, j + 1, w, n, h->gpart.p, h->gd2.p, sb2);
    launch_multiaxpy(V, n, j + 1, h->gd2.p, -1.0, 1.0, w, n, sb2);
    launch_multidot(w, n, 1, w, n, h->gpart.p, h->gwn.p, sb2);
    launch_gm_step_end(h->gdev.p, j, h->gd1.p, h->gd2.p, h->gwn.p, j + 1 < m ? hs.step[j + 1] : hs.step[0], j + 1 < m,
                       sb2);
    launch_gm_scale(w, n, h->gdev.p, sb2);
    per_step = kernel_launch_count() - c2;
    cudaGraph_t done;
    CK(cudaStreamEndCapture(sb2, &done));
  }
  // y = R^{-1} g, x += Z y
  launch_gm_cycle_end(h->gdev.p, h->gy.p, h->gnv.p, cyc, sb1);
  launch_multiaxpy_dev(Z, n, h->gnv.p, h->gy.p, x, n, sb1);
  ge.per_step = per_step;
  ge.per_cycle = kernel_launch_count() - c1 - (long long)m * per_step;
  cudaGraph_t done1;
  CK(cudaStreamEndCapture(sb1, &done1));
  cudaGraph_t graph;
  CK(cudaStreamEndCapture(st, &graph));
  cudaError_t e = cudaGraphInstantiate(&ge.exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  kernel_launch_adjust(-(kernel_launch_count() - c0));  // captured, not yet launched
  if (h->gexec.size() >= 8) {
    cudaGraphExecDestroy(h->gexec.front().exec);
    h->gexec.erase(h->gexec.begin());
  }
  h->gexec.push_back(ge);
  return h->gexec.back();
}

int fgmres_device(gm_handle* h, const double* b, double* x, int& iterations) {
  if (!h->gV.p) {
    const int m = gm_handle::GMRES_M;
    const int64_t n = h->Pn;
    h->gV.alloc((size_t)(m + 1) * n);
    h->gZ.alloc((size_t)m * n);
    h->gdx.alloc(n);
    h->gpart.alloc((size_t)multidot_blocks(n) * 64);
    h->gdots.alloc(64);
    h->gcoef.alloc(64);
  }
  gm_handle::GmresExec& ge = gmres_graph(h, b, x);
  CK(cudaGraphLaunch(ge.exec, h->st));
  int r[5];
  CK(cudaMemcpyAsync(r, &h->gdev.p->jend, sizeof r, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int cycles = r[1], its = r[2], converged = r[3];
  kernel_launch_adjust(ge.fixed + (long long)cycles * ge.per_cycle + (long long)its * ge.per_step);
  iterations = its;
  return converged ? 0 : std::max(1, its);
}

// monitored_pressure_solver, iterative branch (solver/pressure_schur.py:16-72): GMRES, the
// true residual, up to two GMRES refinements of the residual to max(1e-10, 64 eps max(1,|b|));
// the gate (k_gate_pressure) then sees the final check, its roundoff bound and the status.
void gmres_monitored(gm_handle* h, const double* b, double* x, double* res, int slot) {
  cudaStream_t st = h->st;
  SolveCtl* sc = &h->ctl.p->solve[slot];
  const Gate g0 = gate_of(h);
  int its = 0, total = 0;
  // device-controlled FGMRES unless a learned network seeds the first direction (or
  // GHOSTMAC_GMRES_HOST=1)
  const char* eh = std::getenv("GHOSTMAC_GMRES_HOST");
  const bool dev = !h->lnet && !(eh && eh[0] == '1') && !h->capturing && h->st != nullptr && !ktimer_active();
  auto solve = [&](const double* rb, double* rx, int& it, bool learned) {
    return dev ? fgmres_device(h, rb, rx, it) : fgmres(h, rb, rx, it, learned);
  };
  int status = solve(b, x, its, true);
  total += its;
  launch_residual(h->cd, h->rcoef[0], 0, b, x, res, false, sc, 0, true, g0, st);
  auto read = [&](SolveCtl& hs) {
    CK(cudaMemcpyAsync(&hs, sc, sizeof hs, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  };
  SolveCtl hs;
  read(hs);
  const double target = std::max(1e-10, 64 * 2.220446049250313e-16 * std::max(1.0, bits2d(hs.bmax)));
  int k = 0;
  for (int r = 0; r < 2; ++r) {
    if (status || bits2d(hs.rmax[k]) <= target) break;
    status = solve(res, h->gdx.p, its, false);
    total += its;
    const double one = 1.0;
    CK(cudaMemcpyAsync(h->gcoef.p, &one, sizeof one, cudaMemcpyHostToDevice, st));
    launch_multiaxpy(h->gdx.p, h->Pn, 1, h->gcoef.p, 1.0, 1.0, x, h->Pn, st);
    ++k;
    launch_residual(h->cd, h->rcoef[0], 0, b, x, res, false, sc, k, false, g0, st);
    read(hs);
  }
  const int ints[2] = {k + 1, total};
  CK(cudaMemcpyAsync(&sc->gk1, ints, sizeof ints, cudaMemcpyHostToDevice, st));
  if (status) {
    const unsigned long long bad = 1;
    CK(cudaMemcpyAsync(&sc->xbad, &bad, sizeof bad, cudaMemcpyHostToDevice, st));
  }
  CK(cudaStreamSynchronize(st));
}

// One solve A x = b with the FFT + boundary Schur inverse and refinement sweeps to the
// reference's residual target (solver/pressure_schur.py:16-72, direct branch).
void schur_solve(gm_handle* h, int lane, RectDev& rd, int kind, double hc, const double* b, double* x, double* res,
                 double* first, double* w2, int slot) {
  if (kind == 0 && h->g.pressure_solver == 1) {
    gmres_monitored(h, b, x, res, slot);
    return;
  }
  if (h->capturing) {
    schur_solve_graph(h, lane, rd, kind, hc, b, x, res, first, w2, slot);
    return;
  }
  cudaStream_t st = lane == 0 ? h->st : h->st2;
  SolveCtl* sc = &h->ctl.p->solve[slot];
  const bool f32 = h->precision == 1;
  void* resb = f32 ? (void*)(kind == 0 ? h->pres32.p : h->fres32.p) : (void*)res;
  for (int sweep = 0; sweep < h->nchk; ++sweep) {
    Gate gt = gate_of(h, slot, sweep);
    apply_inverse(h, lane, rd, kind, sweep == 0 ? (const void*)b : (const void*)resb, sweep > 0 && f32, x, sweep > 0,
                  first, w2, gt, st);
    launch_residual(h->cd, h->rcoef[kind], kind, b, x, resb, f32, sc, sweep, sweep == 0, gt, st);
    if (h->host_refine && sweep + 1 < h->nchk) {
      // the rule of k_refine_decide, read back on the host
      SolveCtl hs;
      CK(cudaMemcpyAsync(&hs, sc, sizeof hs, cudaMemcpyDeviceToHost, st));
      int err = 0;
      CK(cudaMemcpyAsync(&err, &h->ctl.p->err, sizeof err, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      const double bm = bits2d(hs.bmax), tg = std::max(1e-10, 32 * 2.220446049250313e-16 * std::max(1.0, bm));
      if (err || !(bits2d(hs.rmax[sweep]) > tg)) break;
    }
  }
}

// project(q, dt) (solver/optimized_ghost_cell.py:218-229); q is a face grid with active values.
// In two halves around its pressure solve so that a batch can run the solve of many cases as
// one case-indexed launch sequence.
struct SolveCall {  // one monitored solve (the arguments of schur_solve)
  int lane;
  RectDev* rd;
  int kind;
  const double* b;
  double* x;
  double* res;
  double* first;
  double* w2;
  int slot;
};
void solve_call(gm_handle* h, const SolveCall& c) {
  schur_solve(h, c.lane, *c.rd, c.kind, 0.0, c.b, c.x, c.res, c.first, c.w2, c.slot);
}
SolveCall project_pre(gm_handle* h, double* q, double dt, double* phi, int slot) {
  cudaStream_t st = h->st;
  Gate g0 = gate_of(h);
  launch_set_inlet(h->cd, q, false, st);
  ghost_faces(h, q, g0);
  launch_divergence(h->cd, q, h->prhs.p, dt, nullptr, nullptr, 1, g0, st);
  return SolveCall{0, &h->rp, 0, h->prhs.p, phi, h->pres.p, h->pfirst.p, h->pw2.p, slot};
}
void project_post(gm_handle* h, double* q, double dt, double* out, double* phi, int slot, int divk) {
  cudaStream_t st = h->st;
  Gate g0 = gate_of(h);
  if (h->rec_rhs && !h->capturing && h->rec_count < h->rec_cap) {
    const size_t off = (size_t)h->rec_count * h->Pn;
    CK(cudaMemcpyAsync(h->rec_rhs + off, h->prhs.p, h->Pn * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(h->rec_sol + off, phi, h->Pn * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ++h->rec_count;
  }
  launch_gate_pressure(h->ctl.p, slot, h->nchk, st);
  ghost_p(h, phi, g0);
  launch_project_update(h->cd, q, phi, dt, out, nullptr, g0, st);
  ghost_faces(h, out, g0);
  launch_divergence(h->cd, out, nullptr, 0.0, nullptr, &h->ctl.p->div_max[divk], 0, g0, st);
  launch_gate_projection(h->ctl.p, divk, st);
}
void project(gm_handle* h, double* q, double dt, double* out, double* phi, int slot, int divk) {
  solve_call(h, project_pre(h, q, dt, phi, slot));
  project_post(h, q, dt, out, phi, slot, divk);
}

// Jacobi tables of the FP32 mode's Helmholtz solves for the current dt: 1 / diagonal per
// regular-row class, the irregular rows in FP32 with their diagonal entry zeroed, and the
// number of iterations per application.  The row-sum norm rho of the iteration matrix
// D^{-1} (D - H), taken over every regular class and every irregular row, bounds the error
// contraction per iteration; `iters` takes rho^iters <= 2^-23 (the FP32 rounding level).
// With rho > 1/4 (large dt nu / h^2) the FFT inverse stays.  GHOSTMAC_HELM_JACOBI=0 keeps the
// FFT inverse, =N forces N iterations.
// Tiles of the temporally blocked Jacobi application on the u (k = 0) or v (k = 1) grid:
// regular tw x th tiles, and the body box around the irregular rows with iters - 1 points of
// margin, whose loaded region is what iters - 1 stencil steps reach from the box (breadth-first
// over the five-point stencil and the irregular rows' entries).  Returns false when the
// region would not fit the block's shared memory.
bool jacobi_tiles(gm_handle* h, int k, int iters, int tw, int th) {
  const gm::Geometry& g = h->g;
  const int W = k == 0 ? g.nx + 1 : g.nx, R = k == 0 ? g.ny : g.ny + 1, hal = iters - 1;
  JacobiTiles& T = h->hj.jt[k];
  T = JacobiTiles{};
  T.tw = tw;
  T.th = th;
  T.ntx = (W + T.tw - 1) / T.tw;
  T.nty = (R + T.th - 1) / T.th;
  const gm::Csr& c = h->hs.irr[k];
  const std::vector<int64_t>& rows = h->hs.rows_irr[k];
  std::vector<int32_t> sidx(c.col.size(), -1), rpos(rows.size(), -1);
  if (!rows.empty()) {
    int jmin = R, jmax = -1, imin = W, imax = -1;
    for (int64_t f : rows) {
      const int j = (int)(f / W), i = (int)(f % W);
      jmin = std::min(jmin, j); jmax = std::max(jmax, j); imin = std::min(imin, i); imax = std::max(imax, i);
    }
    T.bj0 = std::max(jmin - hal, 0); T.bj1 = std::min(jmax + hal + 1, R);
    T.bi0 = std::max(imin - hal, 0); T.bi1 = std::min(imax + hal + 1, W);
    // breadth-first reach of hal stencil steps from the box, on a window around it
    int reach = 1;
    for (size_t r = 0; r < rows.size(); ++r) {
      const int j = (int)(rows[r] / W), i = (int)(rows[r] % W);
      for (int64_t e = c.ptr[r]; e < c.ptr[r + 1]; ++e) {
        const int cj = (int)(c.col[e] / W), ci = (int)(c.col[e] % W);
        reach = std::max(reach, std::max(std::abs(cj - j), std::abs(ci - i)));
      }
    }
    const int wj0 = std::max(T.bj0 - hal * reach, 0), wj1 = std::min(T.bj1 + hal * reach, R);
    const int wi0 = std::max(T.bi0 - hal * reach, 0), wi1 = std::min(T.bi1 + hal * reach, W);
    const int ww = wi1 - wi0, wh = wj1 - wj0;
    std::vector<int32_t> irow((size_t)ww * wh, -1);
    for (size_t r = 0; r < rows.size(); ++r) {
      const int j = (int)(rows[r] / W), i = (int)(rows[r] % W);
      if (j >= wj0 && j < wj1 && i >= wi0 && i < wi1) irow[(size_t)(j - wj0) * ww + (i - wi0)] = (int32_t)r;
    }
    std::vector<uint8_t> mark((size_t)ww * wh, 0), next;
    for (int j = T.bj0; j < T.bj1; ++j)
      for (int i = T.bi0; i < T.bi1; ++i) mark[(size_t)(j - wj0) * ww + (i - wi0)] = 1;
    for (int step = 0; step < hal; ++step) {
      next = mark;
      for (int j = 0; j < wh; ++j)
        for (int i = 0; i < ww; ++i) {
          if (!mark[(size_t)j * ww + i]) continue;
          const int32_t r = irow[(size_t)j * ww + i];
          auto put = [&](int gj, int gi) {
            if (gj >= wj0 && gj < wj1 && gi >= wi0 && gi < wi1) next[(size_t)(gj - wj0) * ww + (gi - wi0)] = 1;
          };
          if (r >= 0) {
            for (int64_t e = c.ptr[r]; e < c.ptr[r + 1]; ++e) put((int)(c.col[e] / W), (int)(c.col[e] % W));
          } else {
            put(wj0 + j - 1, wi0 + i); put(wj0 + j + 1, wi0 + i); put(wj0 + j, wi0 + i - 1); put(wj0 + j, wi0 + i + 1);
          }
        }
      mark.swap(next);
    }
    T.rj0 = wj1; T.rj1 = wj0; T.ri0 = wi1; T.ri1 = wi0;
    for (int j = 0; j < wh; ++j)
      for (int i = 0; i < ww; ++i)
        if (mark[(size_t)j * ww + i]) {
          T.rj0 = std::min(T.rj0, wj0 + j); T.rj1 = std::max(T.rj1, wj0 + j + 1);
          T.ri0 = std::min(T.ri0, wi0 + i); T.ri1 = std::max(T.ri1, wi0 + i + 1);
        }
    const int rw = T.ri1 - T.ri0;
    for (size_t e = 0; e < c.col.size(); ++e) {
      const int cj = (int)(c.col[e] / W), ci = (int)(c.col[e] % W);
      if (cj >= T.rj0 && cj < T.rj1 && ci >= T.ri0 && ci < T.ri1) sidx[e] = (cj - T.rj0) * rw + (ci - T.ri0);
    }
    for (size_t r = 0; r < rows.size(); ++r) {
      const int j = (int)(rows[r] / W), i = (int)(rows[r] % W);
      rpos[r] = (j - T.rj0) * rw + (i - T.ri0);  // inside: the box holds every irregular row
    }
    T.nrow = (int)rows.size();
    T.nnz = (int)c.col.size();
  }
  h->jsidx[k].upload(sidx, h->st);
  h->jrpos[k].upload(rpos, h->st);
  T.sidx = h->jsidx[k].p;
  T.rpos = h->jrpos[k].p;
  return helm_jacobi_tiled_smem(T, iters) <= 200 * 1024;
}

void build_helm_jacobi(gm_handle* h) {
  h->jac_iters = 0;
  if (h->precision != 1) return;
  double rho = 0.0;
  bool ok = true;
  for (int k = 0; k < 2; ++k) {
    const ResidualCoef& rc = h->rcoef[k + 1];
    for (int ic = 0; ic < 3; ++ic)
      for (int jc = 0; jc < 2; ++jc) {
        const double cc = rc.cc[ic][jc];
        if (!(std::fabs(cc) > 0.5)) ok = false;
        h->hj.icc[k][ic][jc] = (float)(1.0 / cc);
        rho = std::max(rho, (std::fabs(rc.cw[ic]) + std::fabs(rc.ce) + 2.0 * std::fabs(rc.cy)) / std::fabs(cc));
      }
    const gm::Csr& c = h->hs.irr[k];
    const std::vector<int64_t>& rows = h->hs.rows_irr[k];
    std::vector<float> val(c.col.size()), idiag(rows.size());
    for (size_t r = 0; r < rows.size(); ++r) {
      double diag = 0.0, off = 0.0;
      for (int64_t e = c.ptr[r]; e < c.ptr[r + 1]; ++e) {
        if (c.col[e] == rows[r]) {
          diag += c.val[e];
          val[e] = 0.0f;
        } else {
          off += std::fabs(c.val[e]);
          val[e] = (float)c.val[e];
        }
      }
      if (!(std::fabs(diag) > 0.5)) ok = false;
      idiag[r] = (float)(1.0 / diag);
      rho = std::max(rho, off / std::fabs(diag));
    }
    h->jval[k].upload(val, h->st);
    h->jidiag[k].upload(idiag, h->st);
    h->hj.val[k] = h->jval[k].p;
    h->hj.idiag[k] = h->jidiag[k].p;
  }
  h->jac_rho = rho;
  int iters = 0;
  if (ok && rho < 0.25) iters = rho > 0.0 ? (int)std::ceil(std::log(0x1p-23) / std::log(rho)) : 1;
  iters = std::min(std::max(iters, ok && rho < 0.25 ? 1 : 0), 12);
  if (const char* e = std::getenv("GHOSTMAC_HELM_JACOBI")) {
    const int forced = std::atoi(e);
    iters = forced <= 0 ? 0 : std::min(forced, 32);
  }
  h->jac_iters = iters;
  h->hj.iters = iters;
  h->jac_smem = 0;
  if (iters > 0) {
    bool tiled = true;
    if (const char* e = std::getenv("GHOSTMAC_HELM_JACOBI_TILED")) tiled = std::atoi(e) != 0;
    // Regular tile shapes (width x height), timed on both grids; the fastest is kept.  A
    // smaller tile gives more blocks (a more even spread over the SMs) but a larger share of
    // recomputed halo; a width of 32k - 2 (iters - 1) makes each region row a whole number of
    // warps.  Every shape computes the same values.
    std::vector<std::array<int, 2>> shapes = {{64, 32}, {32, 32}, {64, 16}, {128, 16}, {32, 16}, {128, 8}, {64, 8}};
    for (int k32 : {2, 3, 4})
      for (int th : {8, 16, 32})
        if (32 * k32 - 2 * (iters - 1) >= 16) shapes.push_back({32 * k32 - 2 * (iters - 1), th});
    size_t smem_max = 0;
    std::vector<int> fits;
    for (int s = 0; s < (int)shapes.size() && tiled; ++s) {
      bool ok2 = true;
      size_t sm = 0;
      for (int k = 0; k < 2 && ok2; ++k) {
        ok2 = jacobi_tiles(h, k, iters, shapes[s][0], shapes[s][1]);
        if (ok2) sm = std::max(sm, helm_jacobi_tiled_smem(h->hj.jt[k], iters));
      }
      if (ok2 && sm <= h->smem_optin) {
        fits.push_back(s);
        smem_max = std::max(smem_max, sm);
      }
    }
    if (tiled && !fits.empty() && helm_jacobi_tiled_optin(smem_max) == 0) {
      int best = fits[0];
      if (fits.size() > 1 && !h->capturing) {
        cudaStream_t st = h->st;
        const Gate open{nullptr, 0, 0};
        double *r = nullptr, *x = nullptr;
        CK(cudaMalloc(&r, (size_t)h->F * sizeof(double)));
        CK(cudaMalloc(&x, (size_t)h->F * sizeof(double)));
        CK(cudaMemsetAsync(r, 0, (size_t)h->F * sizeof(double), st));
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        float best_ms = 1e30f;
        for (int s : fits) {
          size_t sm = 0;
          for (int k = 0; k < 2; ++k) {
            jacobi_tiles(h, k, iters, shapes[s][0], shapes[s][1]);
            sm = std::max(sm, helm_jacobi_tiled_smem(h->hj.jt[k], iters));
          }
          float ms_best = 1e30f;
          for (int rep = 0; rep < 6; ++rep) {
            CK(cudaEventRecord(e0, st));
            for (int q = 0; q < 4; ++q)
              for (int kind = 1; kind <= 2; ++kind)
                launch_helm_jacobi_tiled<double>(h->cd, h->rcoef[kind], h->hj, kind, r, x, false, sm, open, st);
            CK(cudaGetLastError());
            CK(cudaEventRecord(e1, st));
            CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) ms_best = std::min(ms_best, ms);  // the first run warms caches and code
          }
          if (ms_best < best_ms) { best_ms = ms_best; best = s; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(r);
        cudaFree(x);
      }
      size_t smem = 0;
      for (int k = 0; k < 2; ++k) {
        jacobi_tiles(h, k, iters, shapes[best][0], shapes[best][1]);
        smem = std::max(smem, helm_jacobi_tiled_smem(h->hj.jt[k], iters));
      }
      h->jac_smem = smem;
      h->jac_tile = shapes[best][0] * 1000 + shapes[best][1];
    }
  }
  if (iters > 0 && !h->jac_smem && h->jd0.n != (size_t)h->F) {
    h->jd0.alloc(h->F);
    h->jd1.alloc(h->F);
  }
}

// One FP32 application of the Helmholtz inverse by Jacobi iterations: x = [x +] d, with d the
// jac_iters-th iterate from d = 0 for the right-hand side r (FP64 b, or the FP32 residual).
void helm_jacobi_apply(gm_handle* h, int kind, const void* r, bool r_f32, double* x, bool accumulate,
                       const Gate& g, cudaStream_t st) {
  if (h->jac_smem) {
    if (r_f32)
      launch_helm_jacobi_tiled<float>(h->cd, h->rcoef[kind], h->hj, kind, (const float*)r, x, accumulate, h->jac_smem,
                                      g, st);
    else
      launch_helm_jacobi_tiled<double>(h->cd, h->rcoef[kind], h->hj, kind, (const double*)r, x, accumulate,
                                       h->jac_smem, g, st);
    return;
  }
  const float* din = nullptr;
  for (int it = 0; it < h->jac_iters; ++it) {
    const bool last = it + 1 == h->jac_iters;
    float* dout = last ? nullptr : (it % 2 == 0 ? h->jd0.p : h->jd1.p);
    if (r_f32)
      launch_helm_jacobi<float>(h->cd, h->rcoef[kind], h->hj, kind, (const float*)r, din, dout, last ? x : nullptr,
                                accumulate, g, st);
    else
      launch_helm_jacobi<double>(h->cd, h->rcoef[kind], h->hj, kind, (const double*)r, din, dout,
                                 last ? x : nullptr, accumulate, g, st);
    din = dout;
  }
}

void ensure_helmholtz(gm_handle* h, double dt) {
  if (h->helm_ready && h->helm_dt == dt) return;
  int ec = 0;
  std::string err;
  gm::HelmholtzSetup hs;
  if (!gm::build_helmholtz(h->g, dt, hs, ec, err)) throw GateError(ec ? ec : GM_EVALUE, err);
  h->hs = std::move(hs);
  h->helm_ready = true;
  h->helm_dt = dt;
  ++h->helm_gen;
  if (h->host_only) return;
  // the Helmholtz tables are reallocated below: captured step graphs would point at freed buffers
  for (auto& gr : h->graphs)
    if (gr.exec) { cudaGraphExecDestroy(gr.exec); gr.exec = nullptr; }
  build_class_maps(h);
  upload_csr(h->irr[1], h->hs.rows_irr[0], h->hs.irr[0], h->st);
  upload_csr(h->irr[2], h->hs.rows_irr[1], h->hs.irr[1], h->st);
  upload_row_index(h->irr[1], h->hs.rows_irr[0], h->g.usize, h->st);
  upload_row_index(h->irr[2], h->hs.rows_irr[1], h->g.vsize, h->st);
  // v irregular rows are v-grid flat indices (columns too)
  fill_case_dev(h);
  build_helm_jacobi(h);
  build_rect_tables(h, h->ru, 1, dt);
  build_rect_tables(h, h->rv, 2, dt);
  build_schur(h, h->ru, h->hs.schur_rows[0], h->hs.schur_c[0], h->fw2.p);
  build_schur(h, h->rv, h->hs.schur_rows[1], h->hs.schur_c[1], h->fw2.p);
  CK(cudaMemsetAsync(h->fw2.p, 0, h->F * sizeof(double), h->st));
  CK(cudaStreamSynchronize(h->st));
}

void momentum(gm_handle* h, const MomentumArgs& ma, const Gate& g0) {
  if (h->precision == 1) launch_momentum_f32(h->cd, ma, g0, h->st);
  else launch_momentum(h->cd, ma, g0, h->st);
}

// One AB2/CN step (solver/time_integration.py:7-145) on the handle state.
// screen: 1/0 run or skip the CFL screen, -1 decide on the device from the step counter.
// The error word of the control block is sticky: only the per-step slots are cleared, so
// every kernel after a failed gate (also in later captured steps) does nothing.
void sweep_mark(gm_handle* h, int k, cudaStream_t st) {
  if (h->sweep_marking) CK(cudaEventRecordWithFlags(h->sweep_ev[k], st, h->capturing ? cudaEventRecordExternal : 0));
}

void phase_mark(gm_handle* h, int k, cudaStream_t st) {
  // inside a capture an event record node needs the external flag (a plain record only
  // orders the captured streams)
  if (h->phase_on) CK(cudaEventRecordWithFlags(h->phase_ev[k], st, h->capturing ? cudaEventRecordExternal : 0));
}

// One AB2/CN step in four phases around its solves (step_once runs them in order):
//   phase 0: control block, CFL screen, momentum right-hand side -> Helmholtz u (lane 0), v (lane 1)
//   phase 1: momentum gate, first projection up to its pressure solve
//   phase 2: first projection after its solve, defect, second projection up to its solve
//   phase 3: second projection after its solve, pressure output, forces, gates, step record
void step_phase0(gm_handle* h, double dt, int screen, SolveCall calls[2]) {
  cudaStream_t st = h->st;
  phase_mark(h, 0, st);
  Gate g0 = gate_of(h);
  const size_t keep = offsetof(StepCtl, solve);
  CK(cudaMemsetAsync(reinterpret_cast<char*>(h->ctl.p) + keep, 0, sizeof(StepCtl) - keep, st));
  launch_cfl_screen(h->ctl.p, &h->state_max.p[0], &h->state_max.p[1], dt, h->g.dx, h->g.dy, screen, h->counter.p, st);
  const bool first = !h->has_history;
  // pressure at the previous half step: the stored half pressure, or p at active cells
  // when there is no history (solver/optimized_ghost_cell.py:256); ghost values for G p
  if (first) launch_copy_active(h->cls_p.p, h->Pn, h->pout.p, h->phalf.p, g0, st);
  ghost_p(h, h->phalf.p, g0);
  MomentumArgs ma{};
  ma.U = h->U.p;
  ma.P = h->phalf.p;
  ma.dt = dt;
  if (first) {
    ma.mode = 1;
    ma.now = h->now.p;
    ma.out = h->fmid.p;
    momentum(h, ma, g0);
    project(h, h->fmid.p, 0.5 * dt, h->fhalf.p, h->pphi.p, S_P0, 0);
    ma.mode = 2;
    ma.Uhalf = h->fhalf.p;
    ma.now = nullptr;
    ma.out = h->rhs.p;
    momentum(h, ma, g0);
  } else {
    ma.mode = 0;
    ma.alpha = dt / (2 * h->prev_dt);
    ma.prev = h->hist.p;
    ma.now = h->now.p;
    ma.out = h->rhs.p;
    if (h->precision == 1) {
      launch_shadow(h->U.p, h->U32.p, h->F, h->phalf.p, h->P32.p, h->Pn, g0, st);
      ma.U32 = h->U32.p;
      ma.P32 = h->P32.p;
    }
    momentum(h, ma, g0);
  }
  phase_mark(h, 1, st);
  // CN Helmholtz solves for u and v (solver/optimized_ghost_cell.py:247-254)
  // (independent systems on disjoint parts of the face arrays: u on this stream, v on the
  // second lane, joined before the momentum gate)
  CK(cudaEventRecord(h->ev_fork, st));
  CK(cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
  calls[0] = SolveCall{0, &h->ru, 1, h->rhs.p, h->star.p, h->fres.p, h->ffirst.p, h->fw2.p, S_HELM_U};
  calls[1] = SolveCall{1, &h->rv, 2, h->rhs.p, h->star.p, h->fres.p, h->ffirst.p, h->fw2.p, S_HELM_V};
}
SolveCall step_phase1(gm_handle* h) {
  cudaStream_t st = h->st;
  CK(cudaEventRecord(h->ev_join, h->st2));
  CK(cudaStreamWaitEvent(st, h->ev_join, 0));
  launch_gate_momentum(h->ctl.p, h->nchk, st);
  phase_mark(h, 2, st);
  // projection of the CN velocity, defect correction and the pressure increment
  return project_pre(h, h->star.p, h->step_dt, h->pphi.p, S_P1);
}
SolveCall step_phase2(gm_handle* h) {
  cudaStream_t st = h->st;
  const double dt = h->step_dt;
  project_post(h, h->star.p, dt, h->Unext.p, h->pphi.p, S_P1, 1);
  phase_mark(h, 3, st);
  launch_defect(h->cd, h->rcoef[1], h->rcoef[2], h->Unext.p, h->rhs.p, h->faction.p, h->fproj.p, gate_of(h), st);
  phase_mark(h, 4, st);
  return project_pre(h, h->fproj.p, dt, h->pinc.p, S_P2);
}
void step_phase3(gm_handle* h) {
  cudaStream_t st = h->st;
  const double dt = h->step_dt;
  Gate g0 = gate_of(h);
  project_post(h, h->fproj.p, dt, h->fproj2.p, h->pinc.p, S_P2, 2);
  phase_mark(h, 5, st);
  // pinc already carries its ghost values: project_post extended it, and the extension rows
  // read active cells only, so extending it again would rewrite the same values
  const bool first = !h->has_history;
  double factor = first ? 1.0 : dt / (dt + h->prev_dt);
  launch_pressure_out(h->cd, h->phalf.p, h->pinc.p, factor, dt, h->faction.p, h->rhs.p, h->phalf_next.p, h->pout.p,
                      &h->ctl.p->coupled_max, g0, st);
  ghost_p(h, h->pout.p, g0);
  // diagnostics on the new state, forces and the step gates (solver/main.py:383-415)
  launch_maxabs(h->cd, h->Unext.p, &h->ctl.p->umax, &h->ctl.p->vmax, g0, st);
  launch_forces(h->cd, h->Unext.p, h->pout.p, h->g.nu * h->g.rho, dt, h->ctl.p, 1, nullptr, g0, st);
  launch_step_end(h->ctl.p, h->state_max.p, h->ring.p, h->ridx.p, h->counter.p, gm_handle::RING_CAP, st);
  phase_mark(h, 6, st);
  CK(cudaGetLastError());
}
// One AB2/CN step (solver/time_integration.py:7-145) on the handle state.
// screen: 1/0 run or skip the CFL screen, -1 decide on the device from the step counter.
// The error word of the control block is sticky: only the per-step slots are cleared, so
// every kernel after a failed gate (also in later captured steps) does nothing.
void step_once(gm_handle* h, double dt, int screen) {
  h->step_dt = dt;
  SolveCall helm[2];
  step_phase0(h, dt, screen, helm);
  solve_call(h, helm[0]);
  solve_call(h, helm[1]);
  solve_call(h, step_phase1(h));
  solve_call(h, step_phase2(h));
  step_phase3(h);
}

void swap_state(gm_handle* h) {
  std::swap(h->U.p, h->Unext.p);
  std::swap(h->phalf.p, h->phalf_next.p);
  std::swap(h->hist.p, h->now.p);
}

// Graph of one steady step for the current buffer assignment and dt (captured on demand,
// two alternate between the ping-pong buffer assignments).
cudaGraphExec_t step_graph(gm_handle* h, double dt) {
  const double* key[6] = {h->U.p, h->Unext.p, h->phalf.p, h->phalf_next.p, h->hist.p, h->now.p};
  for (auto& gr : h->graphs)
    if (gr.exec && gr.dt == dt && std::equal(key, key + 6, gr.key)) return gr.exec;
  gm_handle::StepGraph* slot = !h->graphs[0].exec || h->graphs[0].dt != dt ? &h->graphs[0]
                               : (!h->graphs[1].exec || h->graphs[1].dt != dt ? &h->graphs[1] : &h->graphs[0]);
  if (slot->exec) { cudaGraphExecDestroy(slot->exec); slot->exec = nullptr; }
  const long long c0 = kernel_launch_count();
  long long body_total = 0;
  std::fill(h->body_nodes_slot, h->body_nodes_slot + 5, 0LL);
  h->capturing = true;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  try {
    step_once(h, dt, -1);
  } catch (...) {
    h->capturing = false;
    cudaStreamEndCapture(h->st, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  h->capturing = false;
  CK(cudaStreamEndCapture(h->st, &g));
  const long long captured = kernel_launch_count() - c0;
  kernel_launch_adjust(-captured);
  for (int q = 0; q < 5; ++q) {
    body_total += h->body_nodes_slot[q];
    slot->body_nodes[q] = h->body_nodes_slot[q];
  }
  slot->outer_nodes = captured - body_total;
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) throw CudaError(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  slot->exec = ex;
  slot->dt = dt;
  std::copy(key, key + 6, slot->key);
  return ex;
}

void fill_diag(gm_handle* h, const StepCtl& c, double t, double dt, bool first, gm_step_diag* d) {
  std::memset(d, 0, sizeof *d);
  d->time = t;
  d->dt = dt;
  d->max_divergence = bits2d(c.div_max[1]);
  d->cfl = dt * (bits2d(c.umax) / h->g.dx + bits2d(c.vmax) / h->g.dy);
  double denom = ((0.5 * h->g.rho) * (h->g.U_ref * h->g.U_ref)) * h->g.D;
  d->cd = c.cd;
  d->cl = c.cl;
  d->cd_pressure = c.forces[2] / denom;
  d->cd_viscous = c.forces[4] / denom;
  d->cl_pressure = c.forces[3] / denom;
  d->cl_viscous = c.forces[5] / denom;
  for (int q = 0; q < 6; ++q) d->forces[q] = c.forces[q];
  double mres = 0;
  int mref = 0;
  for (int s = 0; s < 2; ++s) {
    const SolveCtl& sc = c.solve[s];
    double b = bits2d(sc.bmax), tg = std::max(1e-10, 32 * 2.220446049250313e-16 * std::max(1.0, b));
    int k = 0;
    while (k + 1 < h->nchk && bits2d(sc.rmax[k]) > tg) ++k;
    mres = std::max(mres, bits2d(sc.rmax[k]));
    mref += k;
  }
  d->momentum_residual_linf = mres;
  d->momentum_refinement_iterations = mref;
  d->coupled_momentum_residual_linf = bits2d(c.coupled_max);
  int count = 0, refine = 0;
  double plinf = 0, prel = 0;
  int its = 0;
  for (int s = first ? 2 : 3; s < 5; ++s) {
    const SolveCtl& sc = c.solve[s];
    double b = bits2d(sc.bmax), tg = std::max(1e-10, 32 * 2.220446049250313e-16 * std::max(1.0, b));
    int k = 0;
    while (k + 1 < h->nchk && bits2d(sc.rmax[k]) > tg) ++k;
    if (sc.gk1) k = sc.gk1 - 1;
    its += sc.gits;
    ++count;
    refine += k;
    plinf = std::max(plinf, bits2d(sc.rmax[k]));
    double den = std::max(std::sqrt(sc.bsq), 2.2250738585072014e-308);
    prel = std::max(prel, std::sqrt(sc.rsq[k]) / den);
  }
  d->pressure_solve_count = count;
  d->pressure_refinement_iterations = refine;
  d->pressure_iterations = its;
  d->pressure_residual_linf = plinf;
  d->pressure_residual_relative_l2 = prel;
  d->status = c.err;
  d->gate = c.gate;
}

}  // namespace

namespace {
int run_guarded(gm_handle* h, const std::function<void()>& f) {
  try {
    f();
    return GM_OK;
  } catch (const GateError& e) {
    set_error(h, e.msg);
    return e.cls;
  } catch (const CudaError& e) {
    set_error(h, e.msg);
    return GM_ECUDA;
  } catch (const std::exception& e) {
    set_error(h, e.what());
    return GM_ECUDA;
  }
}

void initial_state(gm_handle* h) {
  // u = inlet rows with the faces of masked cells zero, v = 0, p = 0 (solver/main.py:166-177)
  const gm::Geometry& g = h->g;
  std::vector<double> F(h->F, 0.0);
  for (int j = 0; j < g.ny; ++j)
    for (int i = 0; i <= g.nx; ++i) F[(size_t)j * (g.nx + 1) + i] = g.u_inlet[j];
  for (int j = 0; j < g.ny; ++j)
    for (int i = 0; i < g.nx; ++i)
      if (g.mask[(size_t)j * g.nx + i]) {
        F[(size_t)j * (g.nx + 1) + i] = 0.0;
        F[(size_t)j * (g.nx + 1) + i + 1] = 0.0;
        F[g.usize + (size_t)j * g.nx + i] = 0.0;
        F[g.usize + (size_t)(j + 1) * g.nx + i] = 0.0;
      }
  CK(cudaMemcpyAsync(h->ftmp.p, F.data(), F.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  // q = pack(u, v); project(q, 1) (solver/main.py:229-230)
  Gate g0{nullptr, 0, 0};
  launch_copy_active(h->cls_f.p, h->F, h->ftmp.p, h->fmid.p, g0, h->st);
  CK(cudaMemsetAsync(h->ctl.p, 0, sizeof(StepCtl), h->st));
  project(h, h->fmid.p, 1.0, h->U.p, h->pphi.p, S_P1, 1);
  check_ctl(h, "initial projection");
  CK(cudaMemsetAsync(h->phalf.p, 0, h->Pn * sizeof(double), h->st));
  CK(cudaMemsetAsync(h->pout.p, 0, h->Pn * sizeof(double), h->st));
  launch_maxabs(h->cd, h->U.p, &h->state_max.p[0], &h->state_max.p[1], Gate{nullptr, 0, 0}, h->st);
  CK(cudaStreamSynchronize(h->st));
}

// Device side of a handle whose geometry is built: streams, geometry and operator uploads,
// work arrays, the pressure rectangle tables and its boundary Schur data.
void create_device(gm_handle* H) {
  const gm::Geometry& g = H->g;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); throw CudaError("no CUDA device"); }
  CK(cudaGetDevice(&H->device));
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, H->device));
  int dyn = configure_kernels(optin);
  cudaGetLastError();
  if (dyn < 48 * 1024) throw CudaError("cannot enable large shared memory for the transform kernels");
  H->smem_optin = (size_t)dyn;
  CK(cudaStreamCreateWithFlags(&H->st, cudaStreamNonBlocking));
  cudaStream_t st = H->st;
  H->F = g.usize + g.vsize;
  H->Pn = g.psize;
  build_class_maps(H);
  H->mask.upload(g.mask, st);
  H->inlet.upload(g.u_inlet, st);
  // ghost stencils: u rows and v rows on the face grid
  {
    gm::Csr f;
    std::vector<int64_t> rows;
    for (size_t r = 0; r < g.gu_rows.size(); ++r) {
      rows.push_back(g.gu_rows[r]);
      for (int64_t e = g.gu.ptr[r]; e < g.gu.ptr[r + 1]; ++e) { f.col.push_back(g.gu.col[e]); f.val.push_back(g.gu.val[e]); }
      f.ptr.push_back((int64_t)f.col.size());
    }
    for (size_t r = 0; r < g.gv_rows.size(); ++r) {
      rows.push_back(g.usize + g.gv_rows[r]);
      for (int64_t e = g.gv.ptr[r]; e < g.gv.ptr[r + 1]; ++e) { f.col.push_back(g.usize + g.gv.col[e]); f.val.push_back(g.gv.val[e]); }
      f.ptr.push_back((int64_t)f.col.size());
    }
    upload_csr(H->gf, rows, f, st);
  }
  upload_csr(H->gp, g.gp_rows, g.gp, st);
  upload_csr(H->irr[0], g.a_rows, g.a_irr, st);
  upload_row_index(H->irr[0], g.a_rows, g.psize, st);
  H->a_nnz.upload(g.a_nnz_row, st);
  H->sp_ptr.upload(g.surf_p.ptr, st); H->sp_col.upload(g.surf_p.col, st); H->sp_val.upload(g.surf_p.val, st);
  H->su_ptr.upload(g.dudn.ptr, st); H->su_col.upload(g.dudn.col, st); H->su_val.upload(g.dudn.val, st);
  H->sv_ptr.upload(g.dvdn.ptr, st); H->sv_col.upload(g.dvdn.col, st); H->sv_val.upload(g.dvdn.val, st);
  H->nwx.upload(g.normal_wx, st); H->nwy.upload(g.normal_wy, st);
  H->nxx.upload(g.normal_x, st); H->nyy.upload(g.normal_y, st);
  H->surf_part.alloc(4 * (size_t)std::max(1, g.n_surface));
  H->surf_ticket.alloc(1);
  H->surf_ticket.zero(st);
  H->d_ui.upload(g.ui, st); H->d_vi.upload(g.vi, st); H->d_pi.upload(g.pi, st);
  for (DBuf<double>* b : {&H->U, &H->Unext, &H->hist, &H->now, &H->rhs, &H->star, &H->fres, &H->ffirst, &H->fw2,
                          &H->fmid, &H->fhalf, &H->faction, &H->fproj, &H->fproj2, &H->ftmp}) {
    b->alloc(H->F);
    b->zero(st);
  }
  for (DBuf<double>* b : {&H->phalf, &H->phalf_next, &H->pout, &H->prhs, &H->pphi, &H->pres, &H->pfirst, &H->pw2,
                          &H->pinc, &H->ptmp}) {
    b->alloc(H->Pn);
    b->zero(st);
  }
  H->spectral.alloc(std::max<int64_t>(H->Pn, (int64_t)g.ny * g.nx));
  H->spectral_b.alloc(H->spectral.n);
  if (H->precision == 1) {
    H->spectral32.alloc(H->spectral.n);
    H->spectral32_b.alloc(H->spectral.n);
    H->pres32.alloc(H->Pn);
    H->pres32.zero(st);
    H->fres32.alloc(H->F);
    H->fres32.zero(st);
    H->U32.alloc(H->F);
    H->P32.alloc(H->Pn);
    H->ffirst32.alloc(H->F);
    H->ffirst32.zero(st);
    H->pfirst32.alloc(H->Pn);
    H->pfirst32.zero(st);
  }
  H->ctl.alloc(1);
  H->ctl.zero(st);
  H->ring.alloc(gm_handle::RING_CAP);
  H->ridx.alloc(1);
  H->ridx.zero(st);
  H->counter.alloc(1);
  H->counter.zero(st);
  CK(cudaMallocHost(&H->host_ring, gm_handle::RING_CAP * sizeof(StepCtl)));
  CK(cudaStreamCreateWithFlags(&H->st_body, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&H->st2, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&H->st2_body, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&H->ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&H->ev_join, cudaEventDisableTiming));
  if (const char* e = std::getenv("GHOSTMAC_NO_GRAPHS")) H->use_graphs = !(e[0] == '1');
  if (g.pressure_solver == 1) H->use_graphs = false;  // GMRES decides its iterations on the host

  H->state_max.alloc(2);
  H->state_max.zero(st);
  CK(cudaMallocHost(&H->host_ctl, sizeof(StepCtl)));
  fill_case_dev(H);
  build_rect_tables(H, H->rp, 0, 0.0);
  build_schur(H, H->rp, g.schur_p_rows, g.schur_p_c, H->pw2.p);
  build_row_gemm(H, H->rp);
  CK(cudaMemsetAsync(H->pw2.p, 0, H->Pn * sizeof(double), st));
}

// The step loop of gm_step: n_steps steps in graph batches of up to RING_CAP, the step records
// read back after each batch, the state returned to the last good step on a failed gate.
// before_last_sync (may be empty) enqueues work on the stream after the last batch, before the
// loop's final synchronisation.
void step_loop(gm_handle* h, double dt, int32_t n_steps, int64_t first_step_index, double start_time,
               gm_step_diag* diag, const std::function<void()>& before_last_sync) {
    ensure_helmholtz(h, dt);
    cudaStream_t st = h->st;
    CK(cudaMemsetAsync(h->ctl.p, 0, sizeof(StepCtl), st));  // clears the sticky error word
    long long counter = first_step_index;
    CK(cudaMemcpyAsync(h->counter.p, &counter, sizeof counter, cudaMemcpyHostToDevice, st));
    int s = 0;
    while (s < n_steps) {
      // steps that differ from the steady pattern run launch by launch: the start-up step,
      // a changed dt, or per-kernel event timing
      const bool direct = !h->has_history || h->prev_dt != dt || !h->use_graphs || ktimer_active() || h->rec_rhs;
      const bool first = !h->has_history;
      const int batch = direct ? 1 : std::min(n_steps - s, (int)gm_handle::RING_CAP);
      CK(cudaMemsetAsync(h->ridx.p, 0, sizeof(int), st));
      if (direct) {
        step_once(h, dt, ((first_step_index + s) % 100) == 0 ? 1 : 0);
        swap_state(h);
      } else {
        for (int k = 0; k < batch; ++k) {
          CK(cudaGraphLaunch(step_graph(h, dt), st));
          swap_state(h);
        }
      }
      CK(cudaMemcpyAsync(h->host_ring, h->ring.p, batch * sizeof(StepCtl), cudaMemcpyDeviceToHost, st));
      if (s + batch == n_steps && before_last_sync) before_last_sync();
      CK(cudaStreamSynchronize(st));
      ktimer_collect();
      if (h->phase_on && !first)
        for (int k = 0; k + 1 < gm_handle::NPHASE_EV; ++k) {
          float ms = 0;
          if (cudaEventElapsedTime(&ms, h->phase_ev[k], h->phase_ev[k + 1]) == cudaSuccess) h->phase_ms[k] = ms;
        }
      if (h->phase_on && !first)
        for (int k = 0; k + 1 < gm_handle::NSWEEP_EV; ++k) {
          float ms = 0;
          if (cudaEventElapsedTime(&ms, h->sweep_ev[k], h->sweep_ev[k + 1]) == cudaSuccess) h->sweep_ms[k] = ms;
        }
      cudaGetLastError();
      int good = 0;
      while (good < batch && h->host_ring[good].err == 0) ++good;
      if (!direct) {
        // kernel nodes the replays executed: outer nodes + one sweep body per refinement iteration
        const gm_handle::StepGraph& gr = h->graphs[0].exec ? h->graphs[0] : h->graphs[1];
        long long nodes = 0;
        for (int k = 0; k < batch; ++k) {
          const StepCtl& c = h->host_ring[k];
          nodes += gr.outer_nodes;
          for (int sl = 0; sl < 5; ++sl) nodes += gr.body_nodes[sl] * c.solve[sl].k;
        }
        kernel_launch_adjust(nodes);
      }
      for (int k = 0; k < std::min(batch, good + 1); ++k)
        if (diag) fill_diag(h, h->host_ring[k], start_time + (s + k + 1) * dt, dt, first && k == 0, &diag[s + k]);
      if (good < batch) {
        // back to the state after the last good step
        if ((batch - good) % 2) swap_state(h);
        if (good > 0) { h->has_history = true; h->prev_dt = dt; }
        *h->host_ctl = h->host_ring[good];
        static const char* names[] = {"", "Ghost projection failed", "CN momentum solve failed",
                                      "Pressure solve failed", "Pressure RHS must be finite",
                                      "Ghost step failed divergence/CFL gate", "Non-finite force",
                                      "Explicit timestep unsafe",
                                      "Finite fields and a positive timestep are required"};
        const StepCtl& c = h->host_ring[good];
        throw GateError(c.err, std::string(names[c.gate < 9 ? c.gate : 0]) + " (step)");
      }
      h->has_history = true;
      h->prev_dt = dt;
      s += batch;
    }
}

// environment switches of the step loop, read per call
void step_switches(gm_handle* h) {
  const char* hr = std::getenv("GHOSTMAC_HOST_REFINE");
  h->host_refine = hr && hr[0] == '1';
  const char* pt = std::getenv("GHOSTMAC_PHASE_TIMING");
  const bool phase = pt && pt[0] == '1';
  if (phase != h->phase_on) {
    // the events become graph nodes: recapture the step graphs with or without them
    for (auto& gr : h->graphs)
      if (gr.exec) { cudaGraphExecDestroy(gr.exec); gr.exec = nullptr; }
    if (phase && !h->phase_ev[0]) {
      for (auto& e : h->phase_ev) cudaEventCreate(&e);
      for (auto& e : h->sweep_ev) cudaEventCreate(&e);
    }
    h->phase_on = phase;
  }
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char* gm_last_error(const gm_handle* h) { return h ? h->err.c_str() : g_global_error; }


int gm_create(const gm_config* cfg, gm_handle** out) {
  if (!cfg || !out) { g_create_error = "null argument"; return GM_EVALUE; }
  *out = nullptr;
  auto h = std::make_unique<gm_handle>();
  gm::Geometry& g = h->g;
  g.nx = cfg->nx; g.ny = cfg->ny; g.Lx = cfg->Lx; g.Ly = cfg->Ly; g.D = cfg->D; g.xc = cfg->xc; g.yc = cfg->yc;
  g.nu = cfg->nu; g.rho = cfg->rho; g.U_inf = cfg->U_inf; g.inflow = cfg->inflow; g.U_m = cfg->U_m;
  g.pressure_solver = cfg->pressure_solver; g.pressure_extension = cfg->pressure_extension;
  g.velocity_interpolation = cfg->velocity_interpolation;
  if (cfg->precision != 0 && cfg->precision != 1) { g_create_error = "precision must be 0 (FP64) or 1 (FP32 with FP64 refinement)"; return GM_EVALUE; }
  h->precision = cfg->precision;
  h->nchk = cfg->precision == 1 ? MAXCHK : 3;
  if (cfg->nx % 2 != 0) { g_create_error = "odd nx is not supported by the type-IV transform"; return GM_ENOTIMPL; }
  int ec = 0;
  if (!gm::build_geometry(g, ec)) { g_create_error = g.error; return ec ? ec : GM_EVALUE; }
  if (g.usize + g.vsize >= (int64_t(1) << 31)) { g_create_error = "grids of 2^31 or more faces are not supported"; return GM_EVALUE; }
  gm_handle* H = h.get();
  int rc = run_guarded(nullptr, [&] {
    create_device(H);
    initial_state(H);
  });
  if (rc != GM_OK) return rc;
  *out = h.release();
  return GM_OK;
}

int gm_create_host(const gm_config* cfg, gm_handle** out) {
  if (!cfg || !out) { g_create_error = "null argument"; return GM_EVALUE; }
  *out = nullptr;
  auto h = std::make_unique<gm_handle>();
  gm::Geometry& g = h->g;
  g.nx = cfg->nx; g.ny = cfg->ny; g.Lx = cfg->Lx; g.Ly = cfg->Ly; g.D = cfg->D; g.xc = cfg->xc; g.yc = cfg->yc;
  g.nu = cfg->nu; g.rho = cfg->rho; g.U_inf = cfg->U_inf; g.inflow = cfg->inflow; g.U_m = cfg->U_m;
  g.pressure_solver = cfg->pressure_solver; g.pressure_extension = cfg->pressure_extension;
  g.velocity_interpolation = cfg->velocity_interpolation;
  int ec = 0;
  if (!gm::build_geometry(g, ec)) { g_create_error = g.error; return ec ? ec : GM_EVALUE; }
  h->host_only = true;
  *out = h.release();
  return GM_OK;
}

int gm_prepare_dt(gm_handle* h, double dt) {
  if (!h) return GM_EVALUE;
  if (!(std::isfinite(dt) && dt > 0)) { h->err = "dt must be finite and positive"; return GM_EVALUE; }
  return run_guarded(h, [&] { ensure_helmholtz(h, dt); });
}

int gm_destroy(gm_handle* h) {
  if (!h) return GM_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->host_ctl) cudaFreeHost(h->host_ctl);
  if (h->host_ring) cudaFreeHost(h->host_ring);
  for (auto& gr : h->graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  for (auto& ge : h->gexec)
    if (ge.exec) cudaGraphExecDestroy(ge.exec);
  if (h->st2) cudaStreamSynchronize(h->st2);
  if (h->st_body) cudaStreamDestroy(h->st_body);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->st2_body) cudaStreamDestroy(h->st2_body);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  for (auto& e : h->phase_ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->sweep_ev)
    if (e) cudaEventDestroy(e);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  cudaStream_t st = h->st;
  bool own = h->own_stream;
  delete h;
  if (st && own) cudaStreamDestroy(st);
  return GM_OK;
}

int gm_set_stream(gm_handle* h, void* stream) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    CK(cudaStreamSynchronize(h->st));
    if (h->own_stream) CK(cudaStreamDestroy(h->st));
    h->st = (cudaStream_t)stream;
    h->own_stream = false;
  });
}

int gm_get_sizes(const gm_handle* h, gm_sizes* o) {
  if (!h || !o) return GM_EVALUE;
  const gm::Geometry& g = h->g;
  o->nx = g.nx; o->ny = g.ny; o->usize = g.usize; o->vsize = g.vsize; o->psize = g.psize;
  o->nu_active = (int64_t)g.ui.size(); o->nv_active = (int64_t)g.vi.size(); o->np_active = (int64_t)g.pi.size();
  o->qsize = o->nu_active + o->nv_active;
  o->n_surface = g.n_surface;
  o->rank_p = (int64_t)g.schur_p_rows.size();
  o->rank_u = h->helm_ready ? (int64_t)h->hs.schur_rows[0].size() : -1;
  o->rank_v = h->helm_ready ? (int64_t)h->hs.schur_rows[1].size() : -1;
  o->ghost_u = (int64_t)g.gu_rows.size(); o->ghost_v = (int64_t)g.gv_rows.size(); o->ghost_p = (int64_t)g.gp_rows.size();
  o->dx = g.dx; o->dy = g.dy; o->U_ref = g.U_ref;
  return GM_OK;
}

int gm_get_indices(const gm_handle* h, int64_t* ui, int64_t* vi, int64_t* pi) {
  if (!h) return GM_EVALUE;
  if (ui) std::copy(h->g.ui.begin(), h->g.ui.end(), ui);
  if (vi) std::copy(h->g.vi.begin(), h->g.vi.end(), vi);
  if (pi) std::copy(h->g.pi.begin(), h->g.pi.end(), pi);
  return GM_OK;
}

int gm_get_ghost_stencils(const gm_handle* h, int32_t which, int64_t* n_rows, int64_t* nnz, int64_t* rows,
                          int64_t* ptr, int64_t* cols, double* vals) {
  if (!h || which < 0 || which > 2) return GM_EVALUE;
  const gm::Geometry& g = h->g;
  const std::vector<int64_t>& r = which == 0 ? g.gu_rows : (which == 1 ? g.gv_rows : g.gp_rows);
  const gm::Csr& c = which == 0 ? g.gu : (which == 1 ? g.gv : g.gp);
  if (n_rows) *n_rows = (int64_t)r.size();
  if (nnz) *nnz = c.nnz();
  if (rows) std::copy(r.begin(), r.end(), rows);
  if (ptr) std::copy(c.ptr.begin(), c.ptr.end(), ptr);
  if (cols) std::copy(c.col.begin(), c.col.end(), cols);
  if (vals) std::copy(c.val.begin(), c.val.end(), vals);
  return GM_OK;
}

int gm_get_schur_rows(const gm_handle* h, int32_t which, int64_t* n, int64_t* rows) {
  if (!h || which < 0 || which > 2) return GM_EVALUE;
  const std::vector<int64_t>* r = nullptr;
  if (which == 0) r = &h->g.schur_p_rows;
  else if (h->helm_ready) r = &h->hs.schur_rows[which - 1];
  else { if (n) *n = -1; return GM_OK; }
  if (n) *n = (int64_t)r->size();
  if (rows) std::copy(r->begin(), r->end(), rows);
  return GM_OK;
}

int gm_get_surface_points(const gm_handle* h, double* yx) {
  if (!h || !yx) return GM_EVALUE;
  for (int k = 0; k < h->g.n_surface; ++k) { yx[2 * k] = h->g.surf_y[k]; yx[2 * k + 1] = h->g.surf_x[k]; }
  return GM_OK;
}

int gm_pressure_reconstruction(gm_handle* h, const double* yx, int32_t n_points, int64_t* nnz, int64_t* ptr,
                               int64_t* cols, double* vals) {
  if (!h || !yx || !nnz || n_points < 0) return GM_EVALUE;
  std::vector<double> py((size_t)n_points), px((size_t)n_points);
  for (int32_t k = 0; k < n_points; ++k) { py[k] = yx[2 * k]; px[k] = yx[2 * k + 1]; }
  gm::Csr out;
  std::string err;
  if (!gm::pressure_reconstruction(h->g, py, px, out, err)) {
    h->err = err;
    return GM_EVALUE;
  }
  *nnz = out.nnz();
  if (ptr) std::copy(out.ptr.begin(), out.ptr.end(), ptr);
  if (cols) std::copy(out.col.begin(), out.col.end(), cols);
  if (vals) std::copy(out.val.begin(), out.val.end(), vals);
  return GM_OK;
}

int gm_host_alloc(size_t bytes, void** out) {
  if (!out) return GM_EVALUE;
  *out = nullptr;
  if (bytes == 0) return GM_OK;
  if (cudaMallocHost(out, bytes) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return GM_ECUDA;
  }
  return GM_OK;
}
int gm_host_free(void* p) {
  if (!p) return GM_OK;
  if (cudaFreeHost(p) != cudaSuccess) {
    cudaGetLastError();
    return GM_ECUDA;
  }
  return GM_OK;
}

int gm_set_state(gm_handle* h, const double* u, const double* v, const double* p) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    if (u || v) {
      // the state is unpack(pack(u, v)): active entries taken, ghosts and inlet rebuilt; each
      // given array is copied straight into the work grid (host arrays by one DMA)
      if (!(u && v)) CK(cudaMemcpyAsync(h->ftmp.p, h->U.p, h->F * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (u) CK(cudaMemcpyAsync(h->ftmp.p, u, g.usize * sizeof(double), cudaMemcpyDefault, st));
      if (v) CK(cudaMemcpyAsync(h->ftmp.p + g.usize, v, g.vsize * sizeof(double), cudaMemcpyDefault, st));
      Gate g0{nullptr, 0, 0};
      launch_copy_active(h->cls_f.p, h->F, h->ftmp.p, h->U.p, g0, st);
      launch_set_inlet(h->cd, h->U.p, false, st);
      ghost_faces(h, h->U.p, g0);
      CK(cudaMemsetAsync(h->state_max.p, 0, 2 * sizeof(unsigned long long), st));
      launch_maxabs(h->cd, h->U.p, &h->state_max.p[0], &h->state_max.p[1], g0, st);
    }
    if (p) CK(cudaMemcpyAsync(h->pout.p, p, g.psize * sizeof(double), cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
  });
}

int gm_get_state(gm_handle* h, double* u, double* v, double* p) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    if (u) {
      if (is_device_ptr(u)) CK(cudaMemcpyAsync(u, h->U.p, g.usize * 8, cudaMemcpyDeviceToDevice, st));
      else CK(cudaMemcpyAsync(u, h->U.p, g.usize * 8, cudaMemcpyDeviceToHost, st));
    }
    if (v) {
      if (is_device_ptr(v)) CK(cudaMemcpyAsync(v, h->U.p + g.usize, g.vsize * 8, cudaMemcpyDeviceToDevice, st));
      else CK(cudaMemcpyAsync(v, h->U.p + g.usize, g.vsize * 8, cudaMemcpyDeviceToHost, st));
    }
    if (p) {
      if (is_device_ptr(p)) CK(cudaMemcpyAsync(p, h->pout.p, g.psize * 8, cudaMemcpyDeviceToDevice, st));
      else CK(cudaMemcpyAsync(p, h->pout.p, g.psize * 8, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
  });
}

int gm_set_inlet(gm_handle* h, const double* u_inlet) {
  if (!h || !u_inlet) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    CK(cudaMemcpyAsync(h->inlet.p, dev_in(h, 0, u_inlet, h->g.ny), h->g.ny * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    launch_set_inlet(h->cd, h->U.p, false, h->st);
    CK(cudaStreamSynchronize(h->st));
  });
}

int gm_set_history(gm_handle* h, int32_t has_history, const double* prev_adv, const double* half_p, double prev_dt) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    if (!has_history) { h->has_history = false; h->prev_dt = 0; return; }
    if (!prev_adv || !half_p || !(std::isfinite(prev_dt) && prev_dt > 0))
      throw GateError(GM_EVALUE, "AB2 history requires advection, half pressure and a finite positive previous timestep");
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    const int64_t nu = (int64_t)g.ui.size(), nv = (int64_t)g.vi.size(), np = (int64_t)g.pi.size();
    const double* q = dev_in(h, 0, prev_adv, nu + nv);
    CK(cudaMemsetAsync(h->hist.p, 0, h->F * sizeof(double), st));
    launch_scatter(q, h->d_ui.p, nu, h->hist.p, st);
    launch_scatter(q + nu, h->d_vi.p, nv, h->hist.p + g.usize, st);
    const double* ph = dev_in(h, 1, half_p, np);
    CK(cudaMemsetAsync(h->phalf.p, 0, h->Pn * sizeof(double), st));
    launch_scatter(ph, h->d_pi.p, np, h->phalf.p, st);
    CK(cudaStreamSynchronize(st));
    h->has_history = true;
    h->prev_dt = prev_dt;
  });
}

int gm_get_history(gm_handle* h, int32_t* has_history, double* prev_adv, double* half_p, double* prev_dt) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    if (has_history) *has_history = h->has_history ? 1 : 0;
    if (prev_dt) *prev_dt = h->prev_dt;
    if (!h->has_history) return;
    const gm::Geometry& g = h->g;
    const int64_t nu = (int64_t)g.ui.size(), nv = (int64_t)g.vi.size(), np = (int64_t)g.pi.size();
    if (prev_adv) {
      DevOut o(h, 0, prev_adv, nu + nv);
      launch_gather(h->hist.p, h->d_ui.p, nu, o.dev, h->st);
      launch_gather(h->hist.p + g.usize, h->d_vi.p, nv, o.dev + nu, h->st);
      o.finish();
    }
    if (half_p) {
      DevOut o(h, 1, half_p, np);
      launch_gather(h->phalf.p, h->d_pi.p, np, o.dev, h->st);
      o.finish();
    }
    CK(cudaStreamSynchronize(h->st));
  });
}

int gm_step(gm_handle* h, double dt, int32_t n_steps, int64_t first_step_index, double start_time,
            gm_step_diag* diag) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  if (!(std::isfinite(dt) && dt > 0) || n_steps <= 0) { h->err = "dt must be finite and positive"; return GM_EVALUE; }
  step_switches(h);
  return run_guarded(h, [&] { step_loop(h, dt, n_steps, first_step_index, start_time, diag, {}); });
}

int gm_solve_io(gm_handle* h, const double* u_in, const double* v_in, const double* p_in, const double* u_inlet,
                double dt, int32_t n_steps, int64_t first_step_index, double start_time, gm_step_diag* diag,
                double* u_out, double* v_out, double* p_out) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  if (!(std::isfinite(dt) && dt > 0) || n_steps <= 0) { h->err = "dt must be finite and positive"; return GM_EVALUE; }
  step_switches(h);
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    Gate g0{nullptr, 0, 0};
    if (u_in || v_in) {
      // the state is unpack(pack(u, v)), as gm_set_state
      if (!(u_in && v_in)) CK(cudaMemcpyAsync(h->ftmp.p, h->U.p, h->F * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (u_in) CK(cudaMemcpyAsync(h->ftmp.p, u_in, g.usize * sizeof(double), cudaMemcpyDefault, st));
      if (v_in) CK(cudaMemcpyAsync(h->ftmp.p + g.usize, v_in, g.vsize * sizeof(double), cudaMemcpyDefault, st));
      launch_copy_active(h->cls_f.p, h->F, h->ftmp.p, h->U.p, g0, st);
    }
    if (p_in) CK(cudaMemcpyAsync(h->pout.p, p_in, g.psize * sizeof(double), cudaMemcpyDefault, st));
    if (u_inlet) CK(cudaMemcpyAsync(h->inlet.p, u_inlet, g.ny * sizeof(double), cudaMemcpyDefault, st));
    if (u_in || v_in || u_inlet) {
      launch_set_inlet(h->cd, h->U.p, false, st);
      ghost_faces(h, h->U.p, g0);
      CK(cudaMemsetAsync(h->state_max.p, 0, 2 * sizeof(unsigned long long), st));
      launch_maxabs(h->cd, h->U.p, &h->state_max.p[0], &h->state_max.p[1], g0, st);
    }
    step_loop(h, dt, n_steps, first_step_index, start_time, diag, [&] {
      if (u_out) CK(cudaMemcpyAsync(u_out, h->U.p, g.usize * 8, cudaMemcpyDefault, st));
      if (v_out) CK(cudaMemcpyAsync(v_out, h->U.p + g.usize, g.vsize * 8, cudaMemcpyDefault, st));
      if (p_out) CK(cudaMemcpyAsync(p_out, h->pout.p, g.psize * 8, cudaMemcpyDefault, st));
    });
  });
}

int gm_apply(gm_handle* h, int32_t op, double param, const double* x, double* y) {
  if (!h || !x || !y) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    const int64_t nu = (int64_t)g.ui.size(), nv = (int64_t)g.vi.size(), np = (int64_t)g.pi.size(), nq = nu + nv;
    Gate g0{nullptr, 0, 0};
    auto unpack_into = [&](const double* q, double* F) {
      CK(cudaMemsetAsync(F, 0, h->F * sizeof(double), st));
      launch_scatter(q, h->d_ui.p, nu, F, st);
      launch_scatter(q + nu, h->d_vi.p, nv, F + g.usize, st);
      launch_set_inlet(h->cd, F, false, st);
      ghost_faces(h, F, g0);
    };
    auto pack_from = [&](const double* F, double* q) {
      launch_gather(F, h->d_ui.p, nu, q, st);
      launch_gather(F + g.usize, h->d_vi.p, nv, q + nu, st);
    };
    switch (op) {
      case GM_OP_PACK: {
        const double* F = dev_in(h, 0, x, h->F);
        DevOut o(h, 1, y, nq);
        pack_from(F, o.dev);
        o.finish();
        break;
      }
      case GM_OP_UNPACK: {
        const double* q = dev_in(h, 0, x, nq);
        DevOut o(h, 1, y, h->F);
        unpack_into(q, o.dev);
        o.finish();
        break;
      }
      case GM_OP_ADVECTION:
      case GM_OP_DIFFUSION:
      case GM_OP_H_MATVEC: {
        const double* q = dev_in(h, 0, x, nq);
        unpack_into(q, h->ftmp.p);
        if (op == GM_OP_ADVECTION) launch_advection(h->cd, h->ftmp.p, h->fmid.p, g0, st);
        else if (op == GM_OP_DIFFUSION) launch_diffusion(h->cd, h->ftmp.p, h->fmid.p, true, 0.0, g0, st);
        else launch_diffusion(h->cd, h->ftmp.p, h->fmid.p, false, 0.5 * param, g0, st);
        DevOut o(h, 1, y, nq);
        pack_from(h->fmid.p, o.dev);
        o.finish();
        break;
      }
      case GM_OP_GRADIENT:
      case GM_OP_PRESSURE_EXTEND: {
        const double* pp = dev_in(h, 0, x, np);
        CK(cudaMemsetAsync(h->ptmp.p, 0, h->Pn * sizeof(double), st));
        launch_scatter(pp, h->d_pi.p, np, h->ptmp.p, st);
        ghost_p(h, h->ptmp.p, g0);
        if (op == GM_OP_GRADIENT) {
          launch_gradient(h->cd, h->ptmp.p, h->fmid.p, g0, st);
          DevOut o(h, 1, y, nq);
          pack_from(h->fmid.p, o.dev);
          o.finish();
        } else {
          DevOut o(h, 1, y, h->Pn);
          CK(cudaMemcpyAsync(o.dev, h->ptmp.p, h->Pn * sizeof(double), cudaMemcpyDeviceToDevice, st));
          o.finish();
        }
        break;
      }
      case GM_OP_DIVERGENCE: {
        const double* q = dev_in(h, 0, x, nq);
        unpack_into(q, h->ftmp.p);
        launch_divergence(h->cd, h->ftmp.p, h->ptmp.p, 0.0, nullptr, nullptr, 0, g0, st);
        DevOut o(h, 1, y, np);
        launch_gather(h->ptmp.p, h->d_pi.p, np, o.dev, st);
        o.finish();
        break;
      }
      default:
        throw GateError(GM_EVALUE, "unknown operator");
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
  });
}

static void solve_info_from(gm_handle* h, int slot, gm_solve_info* info) {
  if (!info) return;
  const SolveCtl& sc = h->host_ctl->solve[slot];
  double b = bits2d(sc.bmax), tg = std::max(1e-10, 32 * 2.220446049250313e-16 * std::max(1.0, b));
  int k = 0;
  while (k + 1 < h->nchk && bits2d(sc.rmax[k]) > tg) ++k;
  if (sc.gk1) k = sc.gk1 - 1;
  double bound = bits2d(sc.bound[k]);
  double t64 = std::max(1e-10, 64 * 2.220446049250313e-16 * std::max(1.0, b));
  info->residual_linf = bits2d(sc.rmax[k]);
  info->residual_relative_l2 = std::sqrt(sc.rsq[k]) / std::max(std::sqrt(sc.bsq), 2.2250738585072014e-308);
  info->roundoff_bound_linf = bound;
  info->residual_target_linf = std::max(t64, bound);
  info->backward_error_linf = 0;
  info->iterations = sc.gits;
  info->refinement_iterations = k;
  info->status = sc.xbad && sc.gk1 ? 1 : 0;
  info->rank = (int32_t)h->rp.rank;
}

int gm_project(gm_handle* h, double dt, const double* q, double* q_out, double* phi, gm_solve_info* info) {
  if (!h || !q) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    const int64_t nu = (int64_t)g.ui.size(), nv = (int64_t)g.vi.size(), np = (int64_t)g.pi.size(), nq = nu + nv;
    const double* qd = dev_in(h, 0, q, nq);
    CK(cudaMemsetAsync(h->fmid.p, 0, h->F * sizeof(double), st));
    launch_scatter(qd, h->d_ui.p, nu, h->fmid.p, st);
    launch_scatter(qd + nu, h->d_vi.p, nv, h->fmid.p + g.usize, st);
    CK(cudaMemsetAsync(h->ctl.p, 0, sizeof(StepCtl), st));
    project(h, h->fmid.p, dt, h->fproj2.p, h->pinc.p, S_P1, 1);
    CK(cudaMemcpyAsync(h->host_ctl, h->ctl.p, sizeof(StepCtl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    solve_info_from(h, S_P1, info);
    check_ctl(h, "project");
    if (q_out) {
      DevOut o(h, 1, q_out, nq);
      launch_gather(h->fproj2.p, h->d_ui.p, nu, o.dev, st);
      launch_gather(h->fproj2.p + g.usize, h->d_vi.p, nv, o.dev + nu, st);
      o.finish();
    }
    if (phi) {
      DevOut o(h, 2, phi, np);
      launch_gather(h->pinc.p, h->d_pi.p, np, o.dev, st);
      o.finish();
    }
    CK(cudaStreamSynchronize(st));
  });
}

int gm_pressure_solve(gm_handle* h, const double* rhs, double* phi, gm_solve_info* info) {
  if (!h || !rhs || !phi) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    const int64_t np = (int64_t)g.pi.size();
    const double* b = dev_in(h, 0, rhs, np);
    CK(cudaMemsetAsync(h->prhs.p, 0, h->Pn * sizeof(double), st));
    launch_scatter(b, h->d_pi.p, np, h->prhs.p, st);
    CK(cudaMemsetAsync(h->ctl.p, 0, sizeof(StepCtl), st));
    schur_solve(h, 0, h->rp, 0, 0.0, h->prhs.p, h->pphi.p, h->pres.p, h->pfirst.p, h->pw2.p, S_P1);
    launch_gate_pressure(h->ctl.p, S_P1, h->nchk, st);
    CK(cudaMemcpyAsync(h->host_ctl, h->ctl.p, sizeof(StepCtl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    solve_info_from(h, S_P1, info);
    check_ctl(h, "pressure solve");
    DevOut o(h, 1, phi, np);
    launch_gather(h->pphi.p, h->d_pi.p, np, o.dev, st);
    o.finish();
    CK(cudaStreamSynchronize(st));
  });
}

int gm_rectangle_solve(gm_handle* h, int32_t kind, double dt, const double* b, double* x) {
  if (!h || !b || !x || kind < 0 || kind > 2) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    if (kind > 0) ensure_helmholtz(h, dt);
    RectDev& rd = kind == 0 ? h->rp : (kind == 1 ? h->ru : h->rv);
    const int64_t n = (int64_t)rd.view.rows * rd.view.cols;
    const double* bd = dev_in(h, 0, b, n);
    RectView dense = rd.view;
    dense.base = 0;
    dense.pitch = dense.cols;
    dense.cls = nullptr;
    DevOut o(h, 1, x, n);
    plain_inverse<double, double, double>(rd.tt, dense, bd, false, h->spectral.p, o.dev, nullptr, nullptr,
                                          Gate{nullptr, 0, 0}, h->st);
    o.finish();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
  });
}

int gm_surface_forces(gm_handle* h, const double* u, const double* v, const double* p, double mu, double out[6]) {
  if (!h || !u || !v || !p || !out) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    CK(cudaMemcpyAsync(h->ftmp.p, dev_in(h, 0, u, g.usize), g.usize * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(h->ftmp.p + g.usize, dev_in(h, 1, v, g.vsize), g.vsize * 8, cudaMemcpyDeviceToDevice, st));
    const double* pd = dev_in(h, 2, p, g.psize);
    DBuf<double> o6;
    o6.alloc(6);
    launch_forces(h->cd, h->ftmp.p, pd, mu, 0.0, nullptr, 0, o6.p, Gate{nullptr, 0, 0}, st);
    CK(cudaMemcpyAsync(out, o6.p, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  });
}

int gm_divergence_stats(gm_handle* h, const double* u, const double* v, double out[3], int64_t counts[2]) {
  if (!h || !u || !v || !out || !counts) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  return run_guarded(h, [&] {
    const gm::Geometry& g = h->g;
    cudaStream_t st = h->st;
    CK(cudaMemcpyAsync(h->ftmp.p, dev_in(h, 0, u, g.usize), g.usize * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(h->ftmp.p + g.usize, dev_in(h, 1, v, g.vsize), g.vsize * 8, cudaMemcpyDeviceToDevice, st));
    DBuf<double> o5;
    o5.alloc(5);
    o5.zero(st);
    launch_divergence_stats(h->cd, h->ftmp.p, h->mask.p, o5.p, st);
    double r[5];
    CK(cudaMemcpyAsync(r, o5.p, sizeof r, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    unsigned long long mb;
    std::memcpy(&mb, &r[0], 8);
    out[0] = bits2d(mb);
    out[1] = r[1];
    out[2] = r[3];
    counts[0] = (int64_t)std::llround(r[2]);
    counts[1] = (int64_t)std::llround(r[4]);
  });
}

}  // extern "C"

extern "C" {

int64_t gm_kernel_launches(void) { return (int64_t)kernel_launch_count(); }

int gm_set_pressure_recorder(gm_handle* h, double* rhs, double* sol, int32_t capacity) {
  if (!h) return GM_EVALUE;
  if (capacity < 0 || ((!rhs || !sol) && capacity > 0)) { h->err = "recorder needs two device buffers"; return GM_EVALUE; }
  h->rec_rhs = capacity > 0 ? rhs : nullptr;
  h->rec_sol = capacity > 0 ? sol : nullptr;
  h->rec_cap = capacity;
  h->rec_count = 0;
  return GM_OK;
}
int32_t gm_pressure_recorded(const gm_handle* h) { return h ? h->rec_count : 0; }

int gm_set_learned_preconditioner(gm_handle* h, gm_unet* net, const uint16_t* const* w_bf16, const float* const* bias) {
  if (!h) return GM_EVALUE;
  if (h->host_only) { h->err = "host-only handle has no device state"; return GM_ECUDA; }
  if (!net) {
    h->lnet = nullptr;
    return GM_OK;
  }
  if (!w_bf16 || !bias) { h->err = "weights and biases are required"; return GM_EVALUE; }
  if (h->g.pressure_solver != 1) { h->err = "the learned preconditioner serves the GMRES path (pressure_solver=iterative)"; return GM_EVALUE; }
  int32_t nl = 0;
  gm_unet_layers(&nl, nullptr, nullptr);
  return run_guarded(h, [&] {
    h->lw.assign(w_bf16, w_bf16 + nl);
    h->lb.assign(bias, bias + nl);
    if (h->lout.n != (size_t)h->Pn) h->lout.alloc(h->Pn);
    if (!h->lscale.p) h->lscale.alloc(1);
    h->lnet = net;
  });
}

int gm_phase_timing(const gm_handle* h, double out[14]) {
  if (!h || !out) return GM_EVALUE;
  for (int k = 0; k < 6; ++k) out[k] = h->phase_ms[k];
  for (int k = 0; k < 8; ++k) out[6 + k] = h->sweep_ms[k];
  return GM_OK;
}

int gm_solver_info(const gm_handle* h, int32_t* jacobi_iters, double* jacobi_rho) {
  if (!h) return GM_EVALUE;
  if (jacobi_iters) *jacobi_iters = h->jac_iters;
  if (jacobi_rho) *jacobi_rho = h->jac_rho;
  return GM_OK;
}

int gm_kernel_timing(int32_t kernel_class, int32_t enable, double* total_ms, int64_t* count, double* bytes) {
  if (enable) ktimer_enable(1);
  // launches timed outside a step (pressure solves, operator calls) are folded in here
  if (ktimer_active() && cudaDeviceSynchronize() == cudaSuccess) ktimer_collect();
  cudaGetLastError();
  double t = 0, by = 0;
  long long n = 0;
  ktimer_read(kernel_class, &t, &n, &by);
  if (total_ms) *total_ms = t;
  if (count) *count = (int64_t)n;
  if (bytes) *bytes = by;
  if (!enable && kernel_class == 0) ktimer_enable(0);
  return GM_OK;
}

}  // extern "C"

// =============================================================================
// Many cases per GPU: every steady step of all cases is one CUDA graph launch in
// which each case is a concurrent branch (with its own refinement loops).
// =============================================================================
// Cases of a batch that share nx, ny and the precision (at most GM_PACK): their solves run as
// case-indexed launches, one launch per kernel for the whole group.
struct BatchGroup {
  std::vector<int> idx;                // case indices in the batch
  cudaStream_t st[2] = {nullptr, nullptr}, body[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

struct gm_batch {
  std::vector<gm_handle*> cases;
  std::vector<long long> gens;  // Helmholtz table generations the graphs were captured with
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  std::vector<BatchGroup> groups;  // empty: every case steps on its own graph branch
  int shape[3] = {0, 0, 0};        // launch shapes the batch gives its cases (0: not chosen yet)
  std::vector<float> probe_ms;     // the timed candidates, in candidate order (-1: does not fit)
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    std::vector<const double*> key;
    std::vector<long long> gens;
    double dt = 0;
    std::vector<long long> outer;               // per-case kernel nodes outside the refinement loops
    std::vector<std::array<long long, 5>> body;  // per-case kernel nodes of one sweep, per solve slot
    long long group_outer = 0;                          // case-indexed solves: nodes outside the loops
    std::vector<std::array<long long, 5>> group_body;   // and per group, one sweep per solve slot
  } graphs[2];
  std::string err;
};

namespace {

// ---- case-indexed solves of a batch group --------------------------------------------
// One application of the boundary-corrected inverse for every case of the group (the direct
// path of schur_inverse, case-indexed): x = [x +] T^{-1} r - band correction.
template <typename T, typename TI>
void apply_inverse_group(gm_batch* b, const BatchGroup& G, int lane, const std::vector<SolveCall>& calls,
                         bool body, cudaStream_t st) {
  const int n = (int)calls.size();
  const bool f32 = sizeof(T) == 4;
  bool jacobi = false;
  for (int c = 0; c < n; ++c) jacobi = jacobi || (f32 && calls[c].kind != 0 && b->cases[G.idx[c]]->jac_iters > 0);
  if (jacobi) {
    // FP32 Helmholtz solves by Jacobi iterations: every case in turn through the single-case
    // application (each case keeps its own iteration count), the same launches as the case
    // stepped alone
    for (int c = 0; c < n; ++c) {
      gm_handle* h = b->cases[G.idx[c]];
      const SolveCall& call = calls[c];
      const Gate g{h->ctl.p, call.slot, body ? -1 : 0};
      const void* r = body ? (const void*)h->fres32.p : (const void*)call.b;
      apply_inverse(h, lane, *call.rd, call.kind, r, body, call.x, body, call.first, call.w2, g, st);
    }
    return;
  }
  auto fwd = std::make_unique<ArgPack<XpassArgs<T, TI, T>>>();
  auto ys = std::make_unique<ArgPack<YsolveArgs<T>>>();
  auto bf = std::make_unique<ArgPack<BandFirstArgs<T>>>();
  auto bg = std::make_unique<ArgPack<BandGemvArgs<T>>>();
  auto bw = std::make_unique<ArgPack<BandFwdArgs<T>>>();
  auto bd = std::make_unique<ArgPack<BandDirectArgs<T>>>();
  bool direct_g = true;
  auto fin = std::make_unique<ArgPack<XpassArgs<T, T, double>>>();
  const TransformTables* tt0 = nullptr;
  for (int c = 0; c < n; ++c) {
    gm_handle* h = b->cases[G.idx[c]];
    const SolveCall& call = calls[c];
    RectDev& rd = *call.rd;
    const TransformTables& tt = f32 ? rd.tt32 : rd.tt;
    if (!tt0) tt0 = &tt;
    const RectView& v = rd.view;
    const Gate g{h->ctl.p, call.slot, body ? -1 : 0};
    T* spec = f32 ? (T*)(lane == 0 ? h->spectral32.p : h->spectral32_b.p) : (T*)(lane == 0 ? h->spectral.p : h->spectral_b.p);
    const TI* r;
    if (!body) r = (const TI*)call.b;
    else if (f32) r = (const TI*)(call.kind == 0 ? (void*)h->pres32.p : (void*)h->fres32.p);
    else r = (const TI*)call.res;
    const YCorr<T> none{nullptr, nullptr, nullptr, 0, -1};
    fwd->a[c] = xpass_args<T, TI, T>(tt, false, 0, v.rows, r, v.base, v.pitch, v.cls, spec, 0, v.cols, nullptr,
                                     nullptr, none, g);
    ys->a[c] = ysolve_args<T>(tt, v.cols, v.rows, spec, g);
    T* fm = f32 ? (T*)rd.firstm32.p : (T*)rd.firstm.p;
    bf->a[c] = BandFirstArgs<T>{rd.mcount, v.cols, rd.mrow.p, f32 ? (const T*)rd.binv32.p : (const T*)rd.binv.p, spec,
                                fm, g};
    bg->a[c] = BandGemvArgs<T>{rd.rank, rd.mcount, rd.mband.p, fm, rd.cvec.p, g};
    bd->a[c] = BandDirectArgs<T>{rd.rank, rd.glen, f32 ? (const T*)rd.gmat32.p : (const T*)rd.gmat.p,
                                 spec + (int64_t)tt.cj0 * v.cols, rd.cpart.p, g};
    direct_g = direct_g && rd.glen > 0;
    T* band = f32 ? (T*)rd.band32.p : (T*)rd.band.p;
    bw->a[c] = BandFwdArgs<T>{tt.bj1 - tt.bj0 + 1, v.cols, rd.rank, rd.bptr.p, rd.cvec.p,
                              f32 ? (const T*)rd.bfwd32.p : (const T*)rd.bfwd.p, (T)tt.gamma, (T)tt.yscale,
                              (const T*)tt.bpiv, band, g, band_fwd_blocks(v.cols), 1};
    const YCorr<T> corr{band, (const T*)tt.phi, (const T*)tt.psi, tt.bj0, tt.bj1};
    fin->a[c] = xpass_args<T, T, double>(tt, true, 0, v.rows, spec, 0, v.cols, nullptr, call.x, v.base, v.pitch, v.cls,
                                         body ? call.x : nullptr, corr, g);
  }
  launch_xpass_multi<T, TI, T>(*fwd, n, *tt0, st);
  launch_ysolve_multi<T>(*ys, n, *tt0, st);
  if (direct_g) {
    // the same direct sums as the cases stepped alone
    for (int c = 0; c < n; ++c) {
      bw->a[c].c = bd->a[c].part;
      bw->a[c].nsplit = BAND_SPLIT;
    }
    launch_band_direct_multi<T>(*bd, n, st);
  } else {
    launch_band_first_multi<T>(*bf, n, st);
    launch_band_gemv_multi<T>(*bg, n, st);
  }
  launch_band_fwd_solve_multi<T>(*bw, n, st);
  launch_xpass_multi<T, T, double>(*fin, n, *tt0, st);
}

void residual_group(gm_batch* b, const BatchGroup& G, const std::vector<SolveCall>& calls, bool body,
                    cudaStream_t st) {
  const int n = (int)calls.size();
  auto p = std::make_unique<ArgPack<ResidualArgs>>();
  bool f32 = false;
  for (int c = 0; c < n; ++c) {
    gm_handle* h = b->cases[G.idx[c]];
    const SolveCall& call = calls[c];
    f32 = h->precision == 1;
    void* resb = f32 ? (void*)(call.kind == 0 ? h->pres32.p : h->fres32.p) : (void*)call.res;
    p->a[c] = residual_args(h->cd, h->rcoef[call.kind], call.kind, call.b, call.x, resb, f32, &h->ctl.p->solve[call.slot],
                            body ? -1 : 0, !body, Gate{h->ctl.p, call.slot, body ? -1 : 0});
  }
  launch_residual_multi(*p, n, calls[0].kind, f32, st);
}

// The monitored solve of every case of the group (schur_solve_graph, case-indexed): first
// application and check, then a WHILE node whose body sweeps the cases still above their
// targets; returns the kernel nodes of one body sweep.
long long solve_group(gm_batch* b, BatchGroup& G, int lane, const std::vector<SolveCall>& calls) {
  cudaStream_t st = G.st[lane], body_st = G.body[lane];
  const int n = (int)calls.size();
  gm_handle* h0 = b->cases[G.idx[0]];
  const bool f32 = h0->precision == 1;
  const int slot = calls[0].slot, kind = calls[0].kind, nchk = h0->nchk;
  if (f32) apply_inverse_group<float, double>(b, G, lane, calls, false, st);
  else apply_inverse_group<double, double>(b, G, lane, calls, false, st);
  residual_group(b, G, calls, false, st);
  ArgPack<StepCtl*> ctls{};
  for (int c = 0; c < n; ++c) ctls.a[c] = b->cases[G.idx[c]]->ctl.p;
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, nullptr, nullptr, nullptr));
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, graph, 0, 0));
  launch_refine_decide_multi(ctls, n, slot, nchk, cond, st);
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  CK(cudaGraphAddNode(&cnode, graph, deps, nullptr, nd, &cp));
  cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  CK(cudaStreamBeginCaptureToGraph(body_st, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  const long long c0 = kernel_launch_count();
  if (f32) apply_inverse_group<float, float>(b, G, lane, calls, true, body_st);
  else apply_inverse_group<double, double>(b, G, lane, calls, true, body_st);
  residual_group(b, G, calls, true, body_st);
  launch_refine_decide_multi(ctls, n, slot, nchk, cond, body_st);
  const long long body_nodes = kernel_launch_count() - c0;
  CK(cudaStreamEndCapture(body_st, &bodyg));
  return body_nodes;
}

// Groups of a batch for case-indexed solves (empty when some case cannot join one: every case
// needs the direct pressure path, graphs and the direct boundary tables).  Cases of a group take
// the launch shapes of its first case (every shape computes the same values).
void free_groups(gm_batch* b) {
  for (auto& G : b->groups)
    for (int l = 0; l < 2; ++l) {
      if (G.st[l]) cudaStreamDestroy(G.st[l]);
      if (G.body[l]) cudaStreamDestroy(G.body[l]);
      if (G.ev[l]) cudaEventDestroy(G.ev[l]);
    }
  b->groups.clear();
}

// GHOSTMAC_BATCH_GROUPED=1 selects them; by default every case runs on its own graph branch
// (measured faster on GB300 for the 64-case sweep: the branches overlap kernels of different
// kinds, while a case-indexed row transform is bound by its blocks' latency at full load).
void batch_groups(gm_batch* b) {
  const char* e = std::getenv("GHOSTMAC_BATCH_GROUPED");
  if (!(e && e[0] == '1')) { free_groups(b); return; }
  std::vector<BatchGroup> gs;
  for (int c = 0; c < (int)b->cases.size(); ++c) {
    gm_handle* h = b->cases[c];
    if (!h->use_graphs || !h->rp.direct || !h->ru.direct || !h->rv.direct) {
      free_groups(b);
      return;
    }
    BatchGroup* dst = nullptr;
    for (auto& g : gs) {
      gm_handle* f = b->cases[g.idx[0]];
      if (f->g.nx == h->g.nx && f->g.ny == h->g.ny && f->precision == h->precision && (int)g.idx.size() < GM_PACK)
        dst = &g;
    }
    if (!dst) { gs.emplace_back(); dst = &gs.back(); }
    dst->idx.push_back(c);
  }
  // keep the streams and events of existing groups
  for (size_t k = 0; k < gs.size(); ++k) {
    if (k < b->groups.size()) {
      for (int l = 0; l < 2; ++l) {
        gs[k].st[l] = b->groups[k].st[l];
        gs[k].body[l] = b->groups[k].body[l];
        gs[k].ev[l] = b->groups[k].ev[l];
        b->groups[k].st[l] = nullptr;
        b->groups[k].body[l] = nullptr;
        b->groups[k].ev[l] = nullptr;
      }
    }
    for (int l = 0; l < 2; ++l) {
      if (!gs[k].st[l]) CK(cudaStreamCreateWithFlags(&gs[k].st[l], cudaStreamNonBlocking));
      if (!gs[k].body[l]) CK(cudaStreamCreateWithFlags(&gs[k].body[l], cudaStreamNonBlocking));
      if (!gs[k].ev[l]) CK(cudaEventCreateWithFlags(&gs[k].ev[l], cudaEventDisableTiming));
    }
  }
  for (size_t k = gs.size(); k < b->groups.size(); ++k)
    for (int l = 0; l < 2; ++l) {
      if (b->groups[k].st[l]) cudaStreamDestroy(b->groups[k].st[l]);
      if (b->groups[k].body[l]) cudaStreamDestroy(b->groups[k].body[l]);
      if (b->groups[k].ev[l]) cudaEventDestroy(b->groups[k].ev[l]);
    }
  b->groups = std::move(gs);
  auto copy_shape = [](TransformTables& d, const TransformTables& s) {
    d.xg_threads = s.xg_threads;
    d.xg_pb = s.xg_pb;
    d.smem_x = s.smem_x;
    d.lpb_y = s.lpb_y;
    d.threads_y = s.threads_y;
    d.smem_y = s.smem_y;
  };
  for (auto& g : b->groups) {
    gm_handle* f = b->cases[g.idx[0]];
    for (size_t k = 1; k < g.idx.size(); ++k) {
      gm_handle* h = b->cases[g.idx[k]];
      RectDev* dst[3] = {&h->rp, &h->ru, &h->rv};
      const RectDev* src[3] = {&f->rp, &f->ru, &f->rv};
      for (int q = 0; q < 3; ++q) {
        copy_shape(dst[q]->tt, src[q]->tt);
        copy_shape(dst[q]->tt32, src[q]->tt32);
      }
    }
  }
}

// Launch shapes a batch gives its cases (row-pass group threads, groups per block, columns per
// column-solve block).  The single-case autotuner minimises one case's latency with large
// blocks, which in a batch keep other cases' kernels off their SMs; a batch instead times a
// few small-block candidates under its own concurrency: each candidate is applied to every
// case, and a probe graph runs every case's separable inverses (pressure, and the Helmholtz
// ones where the case uses them) on its scratch fields, one branch per case; the fastest of
// three replays wins.  Chosen once per batch.  GHOSTMAC_BATCH_SHAPES="gthreads,gpb,L" fixes the
// shapes instead, "tuned" keeps every case's own.
float batch_probe_ms(gm_batch* b) {
  const Gate open{nullptr, 0, 0};
  const long long c0 = kernel_launch_count();
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
  CK(cudaEventRecord(b->fork, b->root));
  for (size_t c = 0; c < b->cases.size(); ++c) {
    gm_handle* h = b->cases[c];
    CK(cudaStreamWaitEvent(h->st, b->fork, 0));
    RectDev* rs[3] = {&h->rp, &h->ru, &h->rv};
    for (int k = 0; k < 3; ++k) {
      if (k > 0 && (!h->helm_ready || (h->precision == 1 && h->jac_iters > 0))) continue;
      RectDev& rd = *rs[k];
      double* field = k == 0 ? h->ptmp.p : h->ftmp.p;
      if (h->precision == 1)
        plain_inverse<float, double, double>(rd.tt32, rd.view, field, false, h->spectral32.p, field, nullptr, nullptr,
                                             open, h->st);
      else
        plain_inverse<double, double, double>(rd.tt, rd.view, field, false, h->spectral.p, field, nullptr, nullptr,
                                              open, h->st);
    }
    CK(cudaEventRecord(b->join[c], h->st));
    CK(cudaStreamWaitEvent(b->root, b->join[c], 0));
  }
  CK(cudaStreamEndCapture(b->root, &g));
  kernel_launch_adjust(-(kernel_launch_count() - c0));
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return -1.0f;
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    CK(cudaEventRecord(e0, b->root));
    CK(cudaGraphLaunch(ex, b->root));
    CK(cudaEventRecord(e1, b->root));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0) best = std::min(best, ms);  // the first replay warms caches and code
  }
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  cudaGraphExecDestroy(ex);
  return best;
}

bool batch_apply_shape(gm_batch* b, int gt, int gp, int L) {
  for (gm_handle* h : b->cases) {
    RectDev* rs[3] = {&h->rp, &h->ru, &h->rv};
    for (RectDev* rd : rs) {
      if (!apply_shape(h, *rd, false, gt, gp, L)) return false;
      if (h->precision == 1 && !apply_shape(h, *rd, true, gt, gp, L)) return false;
    }
  }
  return true;
}

void batch_shapes(gm_batch* b) {
  if (const char* e = std::getenv("GHOSTMAC_BATCH_SHAPES")) {
    if (std::strncmp(e, "tuned", 5) == 0) return;
    int a = 0, c = 0, d = 0;
    if (std::sscanf(e, "%d,%d,%d", &a, &c, &d) == 3) {
      batch_apply_shape(b, a, c, d);
      return;
    }
  }
  if (b->shape[0] == 0) {
    static const int cand[][3] = {{64, 4, 8}, {64, 4, 4}, {32, 8, 4}, {128, 2, 4}, {128, 2, 8}, {64, 2, 8}};
    float best = 1e30f;
    b->probe_ms.clear();
    for (const auto& cs : cand) {
      float ms = -1.0f;
      if (batch_apply_shape(b, cs[0], cs[1], cs[2])) ms = batch_probe_ms(b);
      b->probe_ms.push_back(ms);
      if (ms > 0 && ms < best) {
        best = ms;
        b->shape[0] = cs[0];
        b->shape[1] = cs[1];
        b->shape[2] = cs[2];
      }
    }
    if (b->shape[0] == 0) { b->shape[0] = 64; b->shape[1] = 4; b->shape[2] = 8; }
    for (gm_handle* h : b->cases) CK(cudaStreamSynchronize(h->st));
  }
  batch_apply_shape(b, b->shape[0], b->shape[1], b->shape[2]);
}

// the case-indexed capture of one steady step of every case (phases on the cases' streams,
// solves on the groups' streams)
void capture_grouped_step(gm_batch* b, double dt, gm_batch::Graph& gr) {
  const int nc = (int)b->cases.size();
  const int ng = (int)b->groups.size();
  gr.group_body.assign(ng, std::array<long long, 5>{});
  gr.group_outer = 0;
  std::vector<std::array<SolveCall, 2>> helm(nc);
  std::vector<SolveCall> pcall(nc);
  auto phase = [&](int c, auto&& f) {
    gm_handle* h = b->cases[c];
    const long long c0 = kernel_launch_count();
    f(h);
    gr.outer[c] += kernel_launch_count() - c0;
  };
  // joins the cases of group g (their stream `which`: 0 st, 1 st2) into its lane streams
  auto join_group = [&](BatchGroup& G, bool both) {
    for (int c : G.idx) {
      gm_handle* h = b->cases[c];
      CK(cudaEventRecord(b->join[c], h->st));
      CK(cudaStreamWaitEvent(G.st[0], b->join[c], 0));
      if (both) CK(cudaStreamWaitEvent(G.st[1], b->join[c], 0));
    }
  };
  auto fork_group = [&](BatchGroup& G, bool both) {
    CK(cudaEventRecord(G.ev[0], G.st[0]));
    if (both) CK(cudaEventRecord(G.ev[1], G.st[1]));
    for (int c : G.idx) {
      gm_handle* h = b->cases[c];
      CK(cudaStreamWaitEvent(h->st, G.ev[0], 0));
      if (both) CK(cudaStreamWaitEvent(h->st2, G.ev[1], 0));
    }
  };
  auto solves = [&](int slot_kind, bool both) {
    for (int g = 0; g < ng; ++g) {
      BatchGroup& G = b->groups[g];
      std::vector<SolveCall> c0v, c1v;
      for (int c : G.idx) {
        if (both) { c0v.push_back(helm[c][0]); c1v.push_back(helm[c][1]); }
        else c0v.push_back(pcall[c]);
      }
      join_group(G, both);
      const long long o0 = kernel_launch_count();
      long long bn = solve_group(b, G, 0, c0v);
      gr.group_body[g][c0v[0].slot] = bn;
      long long bn1 = 0;
      if (both) {
        bn1 = solve_group(b, G, 1, c1v);
        gr.group_body[g][c1v[0].slot] = bn1;
      }
      gr.group_outer += kernel_launch_count() - o0 - bn - bn1;
      fork_group(G, both);
    }
    (void)slot_kind;
  };
  for (int c = 0; c < nc; ++c) phase(c, [&](gm_handle* h) { h->step_dt = dt; step_phase0(h, dt, -1, helm[c].data()); });
  solves(0, true);
  for (int c = 0; c < nc; ++c) phase(c, [&](gm_handle* h) { pcall[c] = step_phase1(h); });
  solves(1, false);
  for (int c = 0; c < nc; ++c) phase(c, [&](gm_handle* h) { pcall[c] = step_phase2(h); });
  solves(2, false);
  for (int c = 0; c < nc; ++c) phase(c, [&](gm_handle* h) { step_phase3(h); });
}

std::vector<const double*> batch_key(gm_batch* b) {
  std::vector<const double*> k;
  for (gm_handle* h : b->cases) {
    const double* t[6] = {h->U.p, h->Unext.p, h->phalf.p, h->phalf_next.p, h->hist.p, h->now.p};
    k.insert(k.end(), t, t + 6);
  }
  return k;
}

gm_batch::Graph& batch_graph(gm_batch* b, double dt) {
  std::vector<const double*> key = batch_key(b);
  std::vector<long long> gens;
  for (gm_handle* h : b->cases) gens.push_back(h->helm_gen);
  for (auto& gr : b->graphs)
    if (gr.exec && gr.dt == dt && gr.key == key && gr.gens == gens) return gr;
  gm_batch::Graph* slot = !b->graphs[0].exec ? &b->graphs[0] : (!b->graphs[1].exec ? &b->graphs[1] : nullptr);
  if (!slot) {
    slot = (b->graphs[0].key == key || b->graphs[0].dt != dt) ? &b->graphs[0] : &b->graphs[1];
    cudaGraphExecDestroy(slot->exec);
    slot->exec = nullptr;
  }
  slot->outer.assign(b->cases.size(), 0);
  slot->body.assign(b->cases.size(), std::array<long long, 5>{});
  slot->group_outer = 0;
  slot->group_body.clear();
  batch_shapes(b);
  batch_groups(b);
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
  try {
    CK(cudaEventRecord(b->fork, b->root));
    if (!b->groups.empty()) {
      for (size_t c = 0; c < b->cases.size(); ++c) {
        gm_handle* h = b->cases[c];
        CK(cudaStreamWaitEvent(h->st, b->fork, 0));
        std::fill(h->body_nodes_slot, h->body_nodes_slot + 5, 0LL);
        h->capturing = true;
      }
      const long long c0 = kernel_launch_count();
      capture_grouped_step(b, dt, *slot);
      kernel_launch_adjust(-(kernel_launch_count() - c0));
      for (size_t c = 0; c < b->cases.size(); ++c) {
        gm_handle* h = b->cases[c];
        h->capturing = false;
        CK(cudaEventRecord(b->join[c], h->st));
        CK(cudaStreamWaitEvent(b->root, b->join[c], 0));
      }
    }
    for (size_t c = 0; c < b->cases.size() && b->groups.empty(); ++c) {
      gm_handle* h = b->cases[c];
      CK(cudaStreamWaitEvent(h->st, b->fork, 0));
      const long long c0 = kernel_launch_count();
      std::fill(h->body_nodes_slot, h->body_nodes_slot + 5, 0LL);
      h->capturing = true;
      step_once(h, dt, -1);
      h->capturing = false;
      const long long captured = kernel_launch_count() - c0;
      kernel_launch_adjust(-captured);
      long long body_total = 0;
      for (int q = 0; q < 5; ++q) {
        slot->body[c][q] = h->body_nodes_slot[q];
        body_total += h->body_nodes_slot[q];
      }
      slot->outer[c] = captured - body_total;
      CK(cudaEventRecord(b->join[c], h->st));
      CK(cudaStreamWaitEvent(b->root, b->join[c], 0));
    }
  } catch (...) {
    for (gm_handle* h : b->cases) h->capturing = false;
    cudaStreamEndCapture(b->root, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  CK(cudaStreamEndCapture(b->root, &g));
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) throw CudaError(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  slot->exec = ex;
  slot->dt = dt;
  slot->key = key;
  slot->gens = gens;
  return *slot;
}

}  // namespace

extern "C" {

int gm_batch_create(gm_handle* const* cases, int32_t n_cases, gm_batch** out) {
  if (!cases || n_cases <= 0 || !out) { g_create_error = "null argument"; return GM_EVALUE; }
  *out = nullptr;
  auto b = std::make_unique<gm_batch>();
  for (int i = 0; i < n_cases; ++i) {
    if (!cases[i] || cases[i]->host_only) { g_create_error = "batch cases must be device handles"; return GM_EVALUE; }
    if (cases[i]->g.pressure_solver != 0) { g_create_error = "batch cases must use the direct pressure solver"; return GM_EVALUE; }
    for (int j = 0; j < i; ++j)
      if (cases[j] == cases[i]) { g_create_error = "a case appears twice in the batch"; return GM_EVALUE; }
    b->cases.push_back(cases[i]);
  }
  int rc = run_guarded(nullptr, [&] {
    CK(cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->join.resize(n_cases);
    for (auto& e : b->join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  });
  if (rc != GM_OK) return rc;
  *out = b.release();
  return GM_OK;
}

int gm_batch_shapes(const gm_batch* b, int32_t shape[3], float* probe_ms, int32_t n) {
  if (!b || !shape) return GM_EVALUE;
  for (int k = 0; k < 3; ++k) shape[k] = b->shape[k];
  for (int k = 0; probe_ms && k < n; ++k) probe_ms[k] = k < (int)b->probe_ms.size() ? b->probe_ms[k] : -1.0f;
  return GM_OK;
}

int gm_batch_destroy(gm_batch* b) {
  if (!b) return GM_OK;
  if (b->root) cudaStreamSynchronize(b->root);
  for (auto& gr : b->graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  for (auto& e : b->join) cudaEventDestroy(e);
  free_groups(b);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->root) cudaStreamDestroy(b->root);
  delete b;
  return GM_OK;
}

const char* gm_batch_last_error(const gm_batch* b) { return b ? b->err.c_str() : g_global_error; }

int gm_batch_step(gm_batch* b, double dt, int32_t n_steps, int64_t first_step_index, const double* start_times,
                  gm_step_diag* diag, int32_t* steps_done) {
  if (!b) return GM_EVALUE;
  if (!(std::isfinite(dt) && dt > 0) || n_steps <= 0) { b->err = "dt must be finite and positive"; return GM_EVALUE; }
  const int nc = (int)b->cases.size();
  if (steps_done) std::fill(steps_done, steps_done + nc, 0);
  const char* hr = std::getenv("GHOSTMAC_HOST_REFINE");
  for (gm_handle* h : b->cases) h->host_refine = hr && hr[0] == '1';
  int first_error = GM_OK;
  try {
    for (gm_handle* h : b->cases) {
      ensure_helmholtz(h, dt);
      CK(cudaMemsetAsync(h->ctl.p, 0, sizeof(StepCtl), h->st));  // clears the sticky error words
      long long counter = first_step_index;
      CK(cudaMemcpyAsync(h->counter.p, &counter, sizeof counter, cudaMemcpyHostToDevice, h->st));
    }
    int s = 0;
    while (s < n_steps && first_error == GM_OK) {
      bool steady = !ktimer_active();
      for (gm_handle* h : b->cases) steady = steady && h->has_history && h->prev_dt == dt && h->use_graphs;
      const int batch = steady ? std::min(n_steps - s, (int)gm_handle::RING_CAP) : 1;
      for (gm_handle* h : b->cases) CK(cudaMemsetAsync(h->ridx.p, 0, sizeof(int), h->st));
      long long nodes = 0;
      if (!steady) {
        // start-up or changed dt: every case launch by launch on its own stream
        for (gm_handle* h : b->cases) {
          step_once(h, dt, ((first_step_index + s) % 100) == 0 ? 1 : 0);
          swap_state(h);
        }
      } else {
        for (gm_handle* h : b->cases) CK(cudaStreamSynchronize(h->st));
        for (int k = 0; k < batch; ++k) {
          CK(cudaGraphLaunch(batch_graph(b, dt).exec, b->root));
          for (gm_handle* h : b->cases) swap_state(h);
        }
        CK(cudaStreamSynchronize(b->root));
      }
      for (gm_handle* h : b->cases)
        CK(cudaMemcpyAsync(h->host_ring, h->ring.p, batch * sizeof(StepCtl), cudaMemcpyDeviceToHost, h->st));
      if (!steady) {
        for (gm_handle* h : b->cases) CK(cudaStreamSynchronize(h->st));
        ktimer_collect();
      }
      for (int c = 0; c < nc; ++c) {
        gm_handle* h = b->cases[c];
        CK(cudaStreamSynchronize(h->st));
        const bool first = !h->has_history;
        int good = 0;
        while (good < batch && h->host_ring[good].err == 0) ++good;
        const double t0 = start_times ? start_times[c] : 0.0;
        for (int k = 0; k < std::min(batch, good + 1); ++k)
          if (diag) fill_diag(h, h->host_ring[k], t0 + (s + k + 1) * dt, dt, first && k == 0,
                              &diag[(size_t)c * n_steps + s + k]);
        if (steady) {
          const gm_batch::Graph& gr = b->graphs[0].exec ? b->graphs[0] : b->graphs[1];
          for (int k = 0; k < batch; ++k) {
            nodes += gr.outer[c];
            for (int sl = 0; sl < 5; ++sl) nodes += gr.body[c][sl] * h->host_ring[k].solve[sl].k;
          }
        }
        if (steps_done) steps_done[c] = s + good;
        if (good > 0) { h->has_history = true; h->prev_dt = dt; }
        if (good < batch) {
          // the sticky error word froze this case after its last good step: undo the swaps since
          if ((batch - good) % 2) swap_state(h);
          *h->host_ctl = h->host_ring[good];
          if (first_error == GM_OK) {
            first_error = h->host_ring[good].err;
            b->err = "case " + std::to_string(c) + ": gate " + std::to_string(h->host_ring[good].gate) +
                     " failed at step " + std::to_string(first_step_index + s + good);
          }
        }
      }
      if (steady) {
        // case-indexed solves: the loop of a group runs while any of its cases sweeps
        const gm_batch::Graph& gr = b->graphs[0].exec ? b->graphs[0] : b->graphs[1];
        for (size_t g = 0; g < b->groups.size() && g < gr.group_body.size(); ++g)
          for (int k = 0; k < batch; ++k) {
            for (int sl = 0; sl < 5; ++sl) {
              int it = 0;
              for (int c : b->groups[g].idx) it = std::max(it, b->cases[c]->host_ring[k].solve[sl].k);
              nodes += gr.group_body[g][sl] * it;
            }
          }
        for (int k = 0; k < batch; ++k) nodes += gr.group_outer;
        kernel_launch_adjust(nodes);
      }
      s += batch;
    }
  } catch (const GateError& e) {
    b->err = e.msg;
    return e.cls;
  } catch (const std::exception& e) {
    b->err = e.what();
    return GM_ECUDA;
  }
  return first_error;
}

}  // extern "C"

// =============================================================================
// pressure-only handles for the cut-cell path (internal.hpp)
// =============================================================================
namespace gmi {

int pressure_create(gm::Geometry&& g, gm_handle** out, std::string& err) {
  *out = nullptr;
  if (g.nx % 2 != 0) { err = "odd nx is not supported by the type-IV transform"; return GM_ENOTIMPL; }
  if (g.usize + g.vsize >= (int64_t(1) << 31)) { err = "grids of 2^31 or more faces are not supported"; return GM_EVALUE; }
  auto h = std::make_unique<gm_handle>();
  h->g = std::move(g);
  h->g.pressure_solver = 0;
  h->precision = 0;
  h->nchk = 3;
  gm_handle* H = h.get();
  int rc = run_guarded(H, [&] { create_device(H); });
  if (rc != GM_OK) {
    err = H->err;
    gm_destroy(h.release());
    return rc;
  }
  *out = h.release();
  return GM_OK;
}

void pressure_destroy(gm_handle* h) { gm_destroy(h); }
const gm::Geometry& geometry(const gm_handle* h) { return h->g; }
cudaStream_t stream(gm_handle* h) { return h->st; }
cudaStream_t body_stream(gm_handle* h, int level) { return level == 0 ? h->st_body : h->st2_body; }
void set_capturing(gm_handle* h, bool on) { h->capturing = on; }

void pressure_solve(gm_handle* h, const double* b, double* x, int slot) {
  schur_solve(h, 0, h->rp, 0, 0.0, b, x, h->pres.p, h->pfirst.p, h->pw2.p, slot);
  launch_gate_pressure(h->ctl.p, slot, h->nchk, h->st);
}

const double* pressure_residual(gm_handle* h) { return h->pres.p; }
StepCtl* control(gm_handle* h) { return h->ctl.p; }

int check(gm_handle* h, const char* where, std::string& err) {
  int rc = run_guarded(h, [&] { check_ctl(h, where); });
  if (rc != GM_OK) err = h->err;
  return rc;
}

int64_t schur_rank(const gm_handle* h) { return h->rp.rank; }

SurfaceCsr surface(const gm_handle* h) {
  return SurfaceCsr{h->g.n_surface, h->sp_ptr.p, h->sp_col.p, h->sp_val.p, h->nwx.p, h->nwy.p};
}

}  // namespace gmi
