// Device data layout and kernel launchers of the ghost-cell AB2/CN step.
//
// Fields live on the staggered grid in HBM, float64, C order:
//   u : ny x (nx+1)   v : (ny+1) x nx   (one buffer "face grid", u then v)
//   p : ny x nx
// A face-grid buffer that represents an unpacked velocity holds the active
// values, the ghost values (extension stencils), the inlet column and zero
// walls; a buffer that represents a packed vector holds the active values and
// zeros elsewhere.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "transforms.cuh"

namespace gmk {

// class bits of every grid point
enum : uint8_t { CLS_ACTIVE = 1, CLS_IRREG = 2, CLS_GHOST = 4 };

// Residual checks of one solve: check 0 after the first application of the
// inverse, check k after refinement sweep k.  Plain FP64 runs at most 2 sweeps (as
// solver/pressure_schur.py:117-122); the FP32 mode refines up to MAXCHK - 1 times.
static constexpr int MAXCHK = 8;

// Reduction slots of one monitored solve (zeroed at the start of every step).
struct SolveCtl {
  unsigned long long bmax;            // max |b| (bits of a non-negative double)
  unsigned long long rmax[MAXCHK];    // max |b - A x| at each check
  unsigned long long bound[MAXCHK];   // roundoff bound max_i w_i (|A||x| + |b|)_i
  double rsq[MAXCHK];                 // sum (b - A x)^2
  double bsq;                         // sum b^2
  unsigned long long xbad;            // non-finite solution (or unconverged GMRES) flag
  int k;                              // current check index (graph-driven refinement loop)
  int gk1;                            // GMRES path: final check index + 1 (0: direct path)
  int gits;                           // GMRES path: Krylov iterations of the solve
  int act;                            // case-indexed refinement loop: this case sweeps again
};

// Per-step control and diagnostics, one per step in flight.
struct StepCtl {
  int err;                       // first failing GM_E* class (0 none)
  int gate;                      // failing gate id
  SolveCtl solve[5];             // 0 helm u, 1 helm v, 2 pressure (start-up), 3 pressure #1, 4 pressure #2
  unsigned long long div_max[3]; // projection divergence checks (start-up, #1, #2)
  unsigned long long coupled_max;
  unsigned long long umax, vmax; // max |u|, |v| over the whole grids after the step
  double forces[6];
  double cd, cl;
};

enum Slot { S_HELM_U = 0, S_HELM_V = 1, S_P0 = 2, S_P1 = 3, S_P2 = 4 };

__device__ __forceinline__ unsigned long long dbits(double v) { return __double_as_longlong(v); }
__host__ __device__ inline double bits2d(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// FP64 <-> FP32 conversions on the integer pipe.  GB300 runs cvt.f32.f64 / cvt.f64.f32 on the
// FP64 pipe (2 per SM per clock), so the FP32 mode moves values between the formats by
// rebuilding the IEEE-754 fields with integer operations instead.  f64 -> f32 rounds half away
// from zero at the 24th significant bit (error <= 2^-24 relative, like round-to-nearest), flushes
// magnitudes below 2^-126 to a signed zero and keeps Inf / NaN; f32 -> f64 is exact for normal
// numbers and flushes FP32 subnormals to a signed zero.
template <typename To, typename From>
__host__ __device__ __forceinline__ To bit_as(From v) {
  static_assert(sizeof(To) == sizeof(From), "bit_as needs equal sizes");
  To t;
  memcpy(&t, &v, sizeof t);
  return t;
}
__host__ __device__ __forceinline__ float f64_to_f32i(double x) {
  const uint64_t b = bit_as<uint64_t>(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint32_t e0 = (uint32_t)(b >> 52) & 0x7ffu;
#ifdef __CUDA_ARCH__
  // the mask as PTX: the compiler folds a C++ mask of the sign bit into fabs, an FP64 add
  // (counted on a GB300: one dadd per conversion in the FP32-mode residual, gone with this)
  uint64_t m;
  asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(m) : "l"(b));
  const uint64_t a = m + (1ull << 28);  // rounding carry may bump the exponent
#else
  const uint64_t a = (b & 0x7fffffffffffffffull) + (1ull << 28);  // rounding carry may bump the exponent
#endif
  const uint32_t e = (uint32_t)(a >> 52);
  uint32_t r;
  if (e0 == 0x7ffu) r = (b & 0xfffffffffffffull) ? 0x7fc00000u : 0x7f800000u;
  else if (e <= 896u) r = 0u;
  else if (e >= 1151u) r = 0x7f800000u;
  else r = ((e - 896u) << 23) | ((uint32_t)(a >> 29) & 0x7fffffu);
  return bit_as<float>(sign | r);
}
__host__ __device__ __forceinline__ double f32_to_f64i(float v) {
  const uint32_t f = bit_as<uint32_t>(v);
  const uint32_t s = f & 0x80000000u, e = (f >> 23) & 0xffu, m = f & 0x7fffffu;
  uint32_t hi = s, lo = 0u;
  if (e == 255u) { hi = s | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u); lo = m << 29; }
  else if (e != 0u) { hi = s | ((e + 896u) << 20) | (m >> 3); lo = m << 29; }
  return bit_as<double>(((uint64_t)hi << 32) | lo);
}
// conversions between the arithmetic types of the FP32 / FP64 kernels
template <typename TO, typename TI>
__host__ __device__ __forceinline__ TO cvt_to(TI v) {
  if constexpr (sizeof(TO) == 4 && sizeof(TI) == 8) return f64_to_f32i(v);
  else if constexpr (sizeof(TO) == 8 && sizeof(TI) == 4) return f32_to_f64i(v);
  else return (TO)v;
}

// Target of the inner refinement loop (solver/pressure_schur.py:115).
__device__ __forceinline__ double inner_target(const SolveCtl* s) {
  double b = bits2d(s->bmax);
  double m = b > 1.0 ? b : 1.0;
  double t = 32 * 2.220446049250313e-16 * m;
  return t > 1e-10 ? t : 1e-10;
}
// Whether refinement sweep k (1 or 2) runs: the previous check exceeded the target.
__device__ __forceinline__ bool sweep_needed(const SolveCtl* s, int k) {
  double tg = inner_target(s);
  for (int c = 0; c < k; ++c)
    if (!(bits2d(s->rmax[c]) > tg)) return false;
  return true;
}
// index of the last residual check that ran, out of nchk launched checks
__device__ __forceinline__ int last_check(const SolveCtl* s, int nchk) {
  if (s->gk1) return s->gk1 - 1;
  double tg = inner_target(s);
  int k = 0;
  while (k + 1 < nchk && bits2d(s->rmax[k]) > tg) ++k;
  return k;
}

// Gate for conditionally executed kernels.
struct Gate {
  StepCtl* ctl;    // error flag lives here (nullptr: always run)
  int slot;        // solve slot for sweep gating
  int sweep;       // 0: unconditional, k: run only if sweep k is needed, -1: only while the
                   // case-indexed refinement loop marks the solve active
};
__device__ __forceinline__ bool gate_open_thread(const Gate& g) {
  if (!g.ctl) return true;
  if (g.sweep < 0) {  // both words read at once: one round trip
    const int err = *(volatile int*)&g.ctl->err;
    const int act = *(volatile int*)&g.ctl->solve[g.slot].act;
    return err == 0 && act != 0;
  }
  if (*(volatile int*)&g.ctl->err) return false;
  if (g.sweep == 0) return true;
  return sweep_needed(&g.ctl->solve[g.slot], g.sweep);
}
// Block-uniform gate: thread 0 decides, every thread of the block gets the same answer
// (the error word may change while the kernel runs).
__device__ __forceinline__ bool gate_open(const Gate& g) {
  // A kernel launched as a programmatic dependent of the previous kernel on its stream starts
  // before that kernel ends: wait for it (and its memory) before reading anything it wrote.
  // Without such a launch this returns at once.  (Triggering the dependents early, at block
  // start, was measured slower: the waiting blocks hold SM resources.)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ int open_flag;
  if (threadIdx.x == 0) open_flag = gate_open_thread(g) ? 1 : 0;
  __syncthreads();
  return open_flag != 0;
}
__device__ __forceinline__ void raise_gate(StepCtl* ctl, int err_class, int gate) {
  if (atomicCAS(&ctl->err, 0, err_class) == 0) ctl->gate = gate;
}

// Static geometry of one case on the device.
struct CaseDev {
  int nx, ny;
  double dx, dy, rho, nu;
  // reciprocals formed once on the host: GB300 issues FP64 at 1/64 of the FP32 rate, so
  // no per-point kernel divides (1/dx, 1/dy, 1/dx^2, 1/dy^2, (1/dx)/rho, (1/dy)/rho, 1/(dx dy), 1/rho)
  double idx, idy, idx2, idy2, gx, gy, iarea, irho;
  int64_t usize, vsize, psize;
  const uint8_t* cls_u;     // usize
  const uint8_t* cls_v;     // vsize
  const uint8_t* cls_p;     // psize
  double* inlet;            // ny (device, mutable by set_inlet)
  // ghost extension rows on the face grid (u rows then v rows, flat face-grid index)
  int n_ghost_f;
  const int64_t* gf_rows; const int64_t* gf_ptr; const int64_t* gf_col; const double* gf_val;
  int n_ghost_p;
  const int64_t* gp_rows; const int64_t* gp_ptr; const int64_t* gp_col; const double* gp_val;
  // irregular rows: pressure A (p grid), Helmholtz u (u grid), v (v grid)
  int n_irr[3];
  const int64_t* irr_rows[3]; const int64_t* irr_ptr[3]; const int64_t* irr_col[3]; const double* irr_val[3];
  const int32_t* irr_index[3];  // per grid point: row in the irregular CSR or -1
  const int32_t* a_nnz;     // psize: nnz of A rows (roundoff weights)
  // surface quadrature
  int n_surf;
  const int64_t* sp_ptr; const int64_t* sp_col; const double* sp_val;
  const int64_t* su_ptr; const int64_t* su_col; const double* su_val;
  const int64_t* sv_ptr; const int64_t* sv_col; const double* sv_val;
  const double* nwx; const double* nwy; const double* nxx; const double* nyy;
  double* surf_part;        // 4 * n_surf per-point force terms (k_forces scratch)
  unsigned* surf_ticket;    // blocks finished in k_forces (back to 0 after each launch)
  double D, U_ref;
  // FP32 copies of the stencil scalars for the FP32 kernels (a per-thread conversion would
  // issue on the FP64 pipe)
  float fdx, fdy, fidx2, fidy2, fiarea, fnu, fgx, fgy;
};

// Helmholtz coefficients (per dt)
struct HelmDev {
  double c;  // 0.5 * dt * nu
};

// ---- separable inverse on a rectangle view --------------------------------
struct RectView {
  int rows, cols;
  int64_t base, pitch;        // offset of (0,0) in the field grid and its row pitch
  const uint8_t* cls;         // class map of the field grid (mask for loads/stores)
};

// Chunk layout of the column systems of the y solve: inner rows [start[p], end[p]],
// interface row end[p] + 1 between chunk p and p + 1.
static constexpr int YCHUNK_MAX = 64;
struct YChunks {
  int P;
  int start[YCHUNK_MAX];
  int end[YCHUNK_MAX];
};

struct TransformTables {      // device tables of one rectangle kind (T = double or float)
  int n;                      // line length of the x transforms (columns)
  FftPlan plan_x;
  int tx_fwd, tx_inv;
  const void* Wx; const void* prex; const void* postx;
  const void* prex_inv; const void* postx_inv;
  // y direction: partitioned tridiagonal solve per x-mode
  YChunks ych;
  double gamma;               // constant off-diagonal of the column systems
  double yscale;              // 1 / (2 nx): normalisation of the inverse x transform
  const void* t0; const void* t1; const void* t2;  // rows x cols partition tables
  // band of the boundary Schur term: U c lives in rows bj0..bj1, C reads rows cj0..cj1
  int bj0, bj1, cj0, cj1;
  const void* bpiv;           // (bj1-bj0+1) x cols reciprocal pivots of the band systems
  const void* phi;            // bj0 x cols decay factors below the band
  const void* psi;            // (rows-1-bj1) x cols decay factors above the band
  // launch shapes (picked by timing candidates at set-up)
  int xg_threads, xg_pb;      // x pass: threads per line group, groups per block
  size_t smem_x;
  int lpb_y, threads_y;       // y solve: columns per block, threads
  size_t smem_y;
};

// spectral correction of the boundary term applied in the final x pass (see k_xpass)
template <typename T>
struct YCorr {
  const T* band;              // (j1-j0+1) x cols band solution; nullptr: no correction
  const T* phi;               // rows < j0: y[j][k] = phi[j][k] * band[0][k]
  const T* psi;               // rows > j1: y[j][k] = psi[j-j1-1][k] * band[j1-j0][k]
  int j0, j1;
};

// ---- flexible GMRES(50) with device-side control (kernels.cu) ---------------
struct GmresDev {             // the state of one solve, in device memory
  static constexpr int M = 50;
  double H[(M + 1) * M];      // R of the rotated Hessenberg matrix, row i column j at i M + j
  double cs[M], sn[M], g[M + 1], y[M];
  double tol, hscale;         // stop tolerance; scale of the next basis vector
  int jend, cycle, iterations, converged, stop;
};
struct GmresHandles {         // the conditions of the Arnoldi-step IF nodes of a cycle (count <= M)
  cudaGraphConditionalHandle step[GmresDev::M];
  int count;
};
// stop tolerance max(rtol ||b||, atol) (bn2 = ||b||^2 on the device)
void launch_gm_init(GmresDev* gd, const double* bn2, cudaGraphConditionalHandle cycle, cudaStream_t st,
                    double rtol = 1e-12, double atol = 1e-12);
void launch_gm_cycle_begin(GmresDev* gd, const double* beta2, const GmresHandles& hs, cudaStream_t st);
void launch_gm_scale(double* w, int64_t n, const GmresDev* gd, cudaStream_t st);
void launch_gm_step_end(GmresDev* gd, int j, const double* d1, const double* d2, const double* wn2,
                        cudaGraphConditionalHandle next, bool has_next, cudaStream_t st);
void launch_gm_cycle_end(GmresDev* gd, double* y, int* nv, cudaGraphConditionalHandle cycle, cudaStream_t st);
void launch_multiaxpy_dev(const double* V, int64_t ld, const int* nv, const double* coef, double* y, int64_t n,
                          cudaStream_t st);

// ---- tensor-core row transforms of the FP32 mode (rowgemm.cu) ---------------
// Transform matrices of the pressure rectangle in split TF32 (both directions) with their TMA
// descriptors, and the descriptors of the arrays the passes have read (cached per array).
struct RowGemm;
void row_gemm_free(RowGemm& g);
struct RowGemm {
  static constexpr int AMAPS = 8;
  alignas(64) unsigned char tmap[2][128];
  alignas(64) unsigned char amap[AMAPS][128];
  const void* aptr[AMAPS] = {};
  int aesz[AMAPS] = {};
  int namap = 0;
  float* mats = nullptr;
  int n = 0, rows = 0, np = 0, kp = 0;  // n = 0: not built (the FFT passes run)
  RowGemm() = default;
  RowGemm(const RowGemm&) = delete;
  RowGemm& operator=(const RowGemm&) = delete;
  ~RowGemm() { row_gemm_free(*this); }
};
struct RowGemmArgs {
  int M, N, K, np;
  float* sout;                 // forward: spectrum (row pitch N)
  double* xout;                // inverse: field, x[obase + m opitch + n]
  int64_t obase, opitch;
  const uint8_t* ocls;
  const double* add;
  const float* wcorr;          // inverse: boundary-term table W (M x N), band rows j0..j1
  int corr, j0, j1;
  Gate gate;
};
size_t row_gemm_smem_bytes();
// whether the passes can read (and write, for the spectrum) this array: a tensor map of it exists
bool row_gemm_ready(RowGemm& g, const void* ptr, int esize);
int row_gemm_build(RowGemm& g, int n, int rows, const double* tfwd, const double* tinv, size_t smem_optin,
                   cudaStream_t st);
template <typename TI>
bool launch_row_gemm_fwd(RowGemm& g, const TI* in, float* spec, const Gate& gate, cudaStream_t st);
bool launch_row_gemm_inv(RowGemm& g, const float* spec, const float* wcorr, int j0, int j1, double* x, int64_t obase,
                         int64_t opitch, const uint8_t* ocls, const double* add, const Gate& gate, cudaStream_t st);
// launch bookkeeping shared with the other translation units
void note_launch_ext();
void kt_mark_ext(int cls, cudaStream_t st, double bytes);
int pdl_mode_ext();
template <typename... KArgs, typename... Args>
inline void launch_pdl_ext(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                           Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_mode_ext();
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ---- launchers (kernels.cu) ------------------------------------------------
int configure_kernels(int smem_optin);
long long kernel_launch_count();
void kernel_launch_adjust(long long delta);
// per-launch event timing summed per kernel class (classes listed in kernels.cu)
static constexpr int KT_CLASSES = 13;
void ktimer_enable(int on);
void ktimer_collect();
bool ktimer_active();
void ktimer_read(int cls, double* total_ms, long long* count, double* bytes);
size_t xpass_smem_per_group(int type, int n, bool fp32);
size_t xpass_smem_tables(int type, int n, int plan_tw, bool fp32);  // twiddle tables staged once per block
size_t ysolve_smem(int rows, int lpb, bool fp32);
// Row transforms of rows r0..r0+nr-1: forward (tx_fwd) or inverse (tx_inv).  Element (r, e)
// is read at in[ibase + r*ipitch + e] (zero where icls marks the point inactive), minus the
// correction when corr.band is set, and written to out[obase + r*opitch + e] (zero where
// ocls marks the point inactive; add[.] + value when add is set).
template <typename T, typename TI, typename TO>
void launch_xpass(const TransformTables& tt, bool inverse, int r0, int nr, const TI* in, int64_t ibase,
                  int64_t ipitch, const uint8_t* icls, TO* out, int64_t obase, int64_t opitch, const uint8_t* ocls,
                  const double* add, const YCorr<T>& corr, const Gate& gate, cudaStream_t st);
// column solves of the spectral array S (rows x cols) in place, input scaled by 1/(2 nx)
template <typename T>
void launch_ysolve(const TransformTables& tt, int cols, int rows, T* S, const Gate& gate, cudaStream_t st);
// band column solves of B ((bj1-bj0+1) x cols) in place, input scaled by 1/(2 nx)
template <typename T>
void launch_yband(const TransformTables& tt, int cols, T* B, const Gate& gate, cudaStream_t st);
// Boundary term by direct sums (tables of the row transforms formed at set-up):
//   firstm[q] = sum_k binv[q][k] spec[mrow[q]][k]      (inverse row transform at the m points C reads)
template <typename T>
void launch_band_first(int m, int n, const int32_t* mrow, const T* binv, const T* spec, T* firstm, const Gate& gate,
                       cudaStream_t st);
//   c[r] = sum_q M[r][q] firstm[q]                      (FP64 GEMV, M = S^{-1} C, rows in band-row order)
template <typename T>
void launch_band_gemv(int rank, int m, const double* M, const T* firstm, double* c, const Gate& gate,
                      cudaStream_t st);
// or both at once with G = M binv folded on the host (rank x L, L = the spectrum rows the C rows
// read times n): part[r BAND_SPLIT + s] = slice s of G[r] . S, S = those spectrum rows
static constexpr int BAND_SPLIT = 4;
template <typename T>
void launch_band_direct(int rank, int L, const T* G, const T* S, double* part, const Gate& gate, cudaStream_t st);
//   band[j][k] = band solve of ( sum_{e in band row j} c[e] bfwd[e][k] ) per column k, with c[e]
//   the sum of its nsplit slices
template <typename T>
void launch_band_fwd_solve(const TransformTables& tt, int n, int rank, const int32_t* bptr, const double* c,
                           const T* bfwd, T* band, const Gate& gate, cudaStream_t st, int nsplit = 1);
// shared memory of launch_band_fwd_solve (the direct path needs it within the default 48 KB)
// and its blocks for n columns
size_t band_fwd_smem(int nb, int rank, bool fp32);
int band_fwd_blocks(int n);
// boundary Schur term c = M first[mcols] (M = S^{-1} C), written to w2 at the boundary rows
template <typename TF>
void launch_schur(const TF* first, int rank, int m, const int64_t* mcols, const double* M, const int64_t* rows,
                  double* w2, const Gate& gate, cudaStream_t st);

void launch_ghost(double* field, int n, const int64_t* rows, const int64_t* ptr, const int64_t* col,
                  const double* val, const Gate& gate, cudaStream_t st);

// residual of the operator of kind (0 pressure A, 1 Helmholtz u, 2 Helmholtz v)
// res = b - Op x on active points; reductions into sc at check index `check`
// (check < 0: the index sc->k maintained by launch_refine_decide)
// Host-formed coefficients of the regular rows of one operator: A x at a point is
//   cc[ic][jc] x + cw[ic] x_west + ce x_east + cy (x_south + x_north)
// with ic = 0 first column, 1 interior, 2 last column and jc = 0 wall row, 1 interior.
struct ResidualCoef {
  double cc[3][2];
  double cw[3];
  double ce, cy;
  float fcc[3][2], fcw[3], fce, fcy;  // FP32 copies (the FP32 mode's roundoff bound, in the residual)
};
void launch_residual(const CaseDev& c, const ResidualCoef& rc, int kind, const double* b, const double* x, void* res,
                     bool res_f32, SolveCtl* sc, int check, bool first_check, const Gate& gate, cudaStream_t st);
// FP32 Jacobi iterations of the Helmholtz systems (index 0: u, 1: v): 1 / diagonal of the
// regular rows per boundary class (as ResidualCoef::cc), and of every irregular row, with the
// irregular rows' entries in FP32 and their diagonal entry zeroed.
// Temporally blocked form (one launch per application): regular tiles of tw x th points read
// their tile and a halo of iters - 1 points (the reach of iters - 1 five-point iterations), and
// one body block covers the box [bj0, bj1) x [bi0, bi1) that holds every irregular row with
// iters - 1 points of margin; it loads the region [rj0, rj1) x [ri0, ri1) that the iterations
// of the box's points can reach through the regular and irregular stencils (found on the
// host), and sidx maps each irregular-row entry to its place in that region (-1 outside).
struct JacobiTiles {
  int tw, th, ntx, nty;
  int bj0, bj1, bi0, bi1;
  int rj0, rj1, ri0, ri1;
  int nrow, nnz;        // irregular rows of the grid and their entries (staged by the body block)
  const int32_t* sidx;  // per entry: place in the body region, -1 outside
  const int32_t* rpos;  // per irregular row: its place in the body region
};
struct HelmJacobi {
  float icc[2][3][2];
  const float* val[2];
  const float* idiag[2];
  int iters;
  JacobiTiles jt[2];
};
// d_out = D^{-1} (r - (H - D) d_in) on the u (kind 1) or v (kind 2) faces (d_in = nullptr:
// d_in = 0); with x set, x = [x +] that iterate instead of d_out (FP64).
template <typename TR>
void launch_helm_jacobi(const CaseDev& c, const ResidualCoef& rc, const HelmJacobi& hj, int kind, const TR* r,
                        const float* din, float* dout, double* x, bool accumulate, const Gate& gate, cudaStream_t st);
// All hj.iters iterations from d = 0 in one launch (temporal blocking): x = [x +] d.
template <typename TR>
void launch_helm_jacobi_tiled(const CaseDev& c, const ResidualCoef& rc, const HelmJacobi& hj, int kind, const TR* r,
                              double* x, bool accumulate, size_t smem, const Gate& gate, cudaStream_t st);
size_t helm_jacobi_tiled_smem(const JacobiTiles& t, int iters);
int helm_jacobi_tiled_optin(size_t smem);
// GMRES pieces on pressure-grid vectors: w = A z; out[i] = V_i . w (i < nv <= 64, V_i at V + i ld,
// part: multidot_blocks(n) * nv scratch); y = alpha y + sign sum_i coef[i] V_i
void launch_apply_pressure(const CaseDev& c, const ResidualCoef& rc, const double* z, double* w, const Gate& gate,
                           cudaStream_t st);
void launch_multidot(const double* V, int64_t ld, int nv, const double* w, int64_t n, double* part, double* out,
                     cudaStream_t st);
unsigned multidot_blocks(int64_t n);
// learned preconditioner glue: x = [v / s, mask] with s = max |v| (bits in *s_bits); z += s y
void launch_learned_prep(const CaseDev& c, const double* v, float* x, unsigned long long* s_bits, cudaStream_t st);
void launch_learned_apply(const CaseDev& c, const float* y, const unsigned long long* s_bits, double* z,
                          cudaStream_t st);
void launch_multiaxpy(const double* V, int64_t ld, int nv, const double* coef, double sign, double alpha, double* y,
                      int64_t n, cudaStream_t st);

// momentum right-hand side; mode 0 steady AB2, 1 start-up part A, 2 start-up part B
struct MomentumArgs {
  const double* U;        // unpacked velocity (face grid)
  const double* Uhalf;    // unpacked half-step velocity (mode 2)
  const double* P;        // pressure grid with ghost values
  const double* prev;     // previous advection (mode 0)
  double* now;            // advection output (modes 0, 1)
  double* out;            // rhs (modes 0, 2) or midpoint (mode 1)
  const float* U32;       // FP32 copies of U and P for the stencils (FP32 mode, mode 0)
  const float* P32;
  double dt, alpha;
  float dt32, alpha32;    // FP32 copies (set by the FP32 launcher)
  int mode;
};
void launch_momentum(const CaseDev& c, const MomentumArgs& a, const Gate& gate, cudaStream_t st);
// same with the stencil arithmetic in FP32 (outputs and q + increment in FP64); in mode 0 the
// stencils read the FP32 copies U32 / P32
void launch_momentum_f32(const CaseDev& c, const MomentumArgs& a, const Gate& gate, cudaStream_t st);
// FP32 copies of the face grid U (n_f points) and the pressure grid P (n_p points)
void launch_shadow(const double* U, float* U32, int64_t n_f, const double* P, float* P32, int64_t n_p,
                   const Gate& gate, cudaStream_t st);

// single operators on face grids (for the operator API)
void launch_advection(const CaseDev& c, const double* U, double* out, const Gate& gate, cudaStream_t st);
void launch_diffusion(const CaseDev& c, const double* U, double* out, bool with_inlet, double hdt, const Gate& gate,
                      cudaStream_t st);  // hdt==0: L U (+offset); else U - hdt*L U (H matvec)
void launch_gradient(const CaseDev& c, const double* P, double* out, const Gate& gate, cudaStream_t st);

// divergence at active p cells of an unpacked face grid: out = div / scale (div when scale is 0),
// max|div| -> *divmax (if divmax); a non-finite out raises the gate error when
// gate_on_nonfinite is set; sc is unused
void launch_divergence(const CaseDev& c, const double* U, double* out, double scale, SolveCtl* sc,
                       unsigned long long* divmax, int gate_on_nonfinite, const Gate& gate, cudaStream_t st);

// out = q - dt * G phi on active faces (phi grid ghost-filled); pressure gate of slot checked first
void launch_project_update(const CaseDev& c, const double* q, const double* phi, double dt, double* out,
                           const SolveCtl* psolve, const Gate& gate, cudaStream_t st);

// action = H result; proj = result + (rhs - action), H = I - c L of the CN solves with the
// residual's coefficients (rcu: u faces, rcv: v faces)
void launch_defect(const CaseDev& c, const ResidualCoef& rcu, const ResidualCoef& rcv, const double* result,
                   const double* rhs, double* action, double* proj, const Gate& gate, cudaStream_t st);

// half = p + inc; out = half + factor*inc (active p); coupled = max|action - rhs + dt G inc|
void launch_pressure_out(const CaseDev& c, const double* p, const double* inc, double factor, double dt,
                         const double* action, const double* rhs, double* half, double* pout,
                         unsigned long long* coupled, const Gate& gate, cudaStream_t st);

void launch_maxabs(const CaseDev& c, const double* U, unsigned long long* umax, unsigned long long* vmax,
                   const Gate& gate, cudaStream_t st);

// forces and coefficients; raises the force/step gates
void launch_forces(const CaseDev& c, const double* U, const double* P, double mu, double dt, StepCtl* ctl,
                   int check_gates, double* out6, const Gate& gate, cudaStream_t st);

// CN momentum gate (after both Helmholtz solves), nchk residual checks per solve
void launch_gate_momentum(StepCtl* ctl, int nchk, cudaStream_t st);
// projection divergence gate on div_max[k]
void launch_gate_projection(StepCtl* ctl, int k, cudaStream_t st);
// CFL screen: dt*(umax/dx + vmax/dy) > 0.5 -> error (values from a previous maxabs);
// screen = 1/0 runs/skips it, screen = -1 runs it when *counter % 100 == 0
void launch_cfl_screen(StepCtl* ctl, const unsigned long long* umax, const unsigned long long* vmax, double dt,
                       double dx, double dy, int screen, const long long* counter, cudaStream_t st);

void launch_gate_pressure(StepCtl* ctl, int slot, int nchk, cudaStream_t st);
// dst[k] = src[idx[k]] and dst[idx[k]] = src[k]
void launch_gather(const double* src, const int64_t* idx, int64_t n, double* dst, cudaStream_t st);
void launch_scatter(const double* src, const int64_t* idx, int64_t n, double* dst, cudaStream_t st);
// column col of (S - I): S[r*rank+col] = sum_e C[r,e] first[e]
void launch_schur_column(const double* first, const RectView& view, int rank, const int64_t* c_ptr,
                         const int64_t* c_col, const double* c_val, double* S, int col, cudaStream_t st);

// Refinement loop decision for a graph WHILE node: if check sc->k exceeded the inner
// target and another check is allowed, advance sc->k and set the condition to 1.
void launch_refine_decide(StepCtl* ctl, int slot, int nchk, cudaGraphConditionalHandle cond, cudaStream_t st);
// end of a step: if no gate failed, the new state's velocity maxima become the persistent
// ones; the step's control block is appended to ring[*ridx] and the step counter advances
void launch_step_end(StepCtl* ctl, unsigned long long* state_max, StepCtl* ring, int* ridx, long long* counter,
                     int cap, cudaStream_t st);

// zero/copy helpers
void launch_copy_active(const uint8_t* cls, int64_t n, const double* src, double* dst, const Gate& gate,
                        cudaStream_t st);

// set the inlet column of a face grid
void launch_set_inlet(const CaseDev& c, double* U, bool zero, cudaStream_t st);

// fluid-cell divergence statistics on a mask (mac_engine diagnostic)
void launch_divergence_stats(const CaseDev& c, const double* U, const uint8_t* mask, double* out5,
                             cudaStream_t st);

// ---- case-indexed launches (many cases of one grid shape per launch) --------
// The arguments of every case travel in the kernel's parameter space (up to GM_PACK cases);
// blockIdx.y selects the case and blocks past a case's own grid return at once.  Every case of
// one launch has the same block shape and shared-memory size (the cases of a batch group share
// nx, ny and the precision, and their launch shapes are made equal).
static constexpr int GM_PACK = 32;
template <typename A>
struct ArgPack {
  A a[GM_PACK];
};

template <typename T, typename TI, typename TO>
struct XpassArgs {
  int n, r0, nr, type;
  FftPlan plan;
  R2RTables<T> tb;
  const TI* in;
  int64_t ibase, ipitch;
  const uint8_t* icls;
  TO* out;
  int64_t obase, opitch;
  const uint8_t* ocls;
  const double* add;
  YCorr<T> corr;
  int gthreads, gpb;
  Gate gate;
  int nblk;
};
template <typename T>
struct YsolveArgs {
  int rows, cols;
  YChunks ch;
  T gamma, scale;
  const T* t0; const T* t1; const T* t2;
  T* S;
  Gate gate;
  int nblk;
};
template <typename T>
struct BandFirstArgs {
  int m, n;
  const int32_t* mrow;
  const T* binv;
  const T* spec;
  T* firstm;
  Gate gate;
};
template <typename T>
struct BandGemvArgs {
  int rank, m;
  const double* M;
  const T* firstm;
  double* c;
  Gate gate;
};
template <typename T>
struct BandFwdArgs {
  int nb, n, rank;
  const int32_t* bptr;
  const double* c;
  const T* bfwd;
  T gamma, scale;
  const T* bpiv;
  T* band;
  Gate gate;
  int nblk;
  int nsplit;   // slices per Schur value in c (1: c holds the values)
};
template <typename T>
struct BandDirectArgs {
  int rank, L;
  const T* G;
  const T* S;
  double* part;
  Gate gate;
};
struct ResidualArgs {
  CaseDev c;
  ResidualCoef rc;
  const double* b; const double* x;
  void* res;
  SolveCtl* sc;
  int check, first;
  Gate gate;
  int nblk;
};

// argument builders: the same conventions as the single-case launchers above
template <typename T, typename TI, typename TO>
XpassArgs<T, TI, TO> xpass_args(const TransformTables& tt, bool inverse, int r0, int nr, const TI* in, int64_t ibase,
                                int64_t ipitch, const uint8_t* icls, TO* out, int64_t obase, int64_t opitch,
                                const uint8_t* ocls, const double* add, const YCorr<T>& corr, const Gate& gate);
template <typename T>
YsolveArgs<T> ysolve_args(const TransformTables& tt, int cols, int rows, T* S, const Gate& gate);
ResidualArgs residual_args(const CaseDev& c, const ResidualCoef& rc, int kind, const double* b, const double* x,
                           void* res, bool res_f32, SolveCtl* sc, int check, bool first_check, const Gate& gate);
// launchers over the first n cases of a pack (tt0: the launch shape shared by the cases)
template <typename T, typename TI, typename TO>
void launch_xpass_multi(const ArgPack<XpassArgs<T, TI, TO>>& p, int n, const TransformTables& tt0, cudaStream_t st);
template <typename T>
void launch_ysolve_multi(const ArgPack<YsolveArgs<T>>& p, int n, const TransformTables& tt0, cudaStream_t st);
template <typename T>
void launch_band_first_multi(const ArgPack<BandFirstArgs<T>>& p, int n, cudaStream_t st);
template <typename T>
void launch_band_gemv_multi(const ArgPack<BandGemvArgs<T>>& p, int n, cudaStream_t st);
template <typename T>
void launch_band_fwd_solve_multi(const ArgPack<BandFwdArgs<T>>& p, int n, cudaStream_t st);
template <typename T>
void launch_band_direct_multi(const ArgPack<BandDirectArgs<T>>& p, int n, cudaStream_t st);
void launch_residual_multi(const ArgPack<ResidualArgs>& p, int n, int kind, bool res_f32, cudaStream_t st);
// Refinement decision of a WHILE node over n cases: each case whose check sc->k exceeded its
// inner target (and may refine again) advances sc->k and is marked active (SolveCtl::act); the
// condition is set while any case is active.  Kernels gated with Gate::sweep = -1 run for
// active cases only.
void launch_refine_decide_multi(const ArgPack<StepCtl*>& ctls, int n, int slot, int nchk,
                                cudaGraphConditionalHandle cond, cudaStream_t st);

}  // namespace gmk
