// Kernels of the ghost-cell AB2/CN step (sm_103a).  See kernels.cuh for the layout.
#include <algorithm>
#include <atomic>
#include <vector>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <utility>

#include "kernels.cuh"

namespace gmk {

static constexpr int TPB = 256;
static constexpr double EPS64 = 2.220446049250313e-16;

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Block-wide max of non-negative doubles (as bits) and optional sum; thread 0 commits atomically.
__device__ void block_commit_max(unsigned long long v, unsigned long long* dst) {
  __shared__ unsigned long long sm[32];
  v = warp_max_u64(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sm[lane] : 0ull;
    v = warp_max_u64(v);
    if (lane == 0 && v) atomicMax(dst, v);
  }
}
__device__ void block_commit_sum(double v, double* dst) {
  __shared__ double sm[32];
  v = warp_sum(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sm[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0 && v != 0.0) atomicAdd(dst, v);
  }
}
// FP32 variant for diagnostics sums of the FP32 mode (FP64 adds issue at 1/64 of the FP32 rate)
__device__ void block_commit_sum_f32(float v, double* dst) {
  __shared__ float smf[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smf[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? smf[lane] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0 && v != 0.0f) atomicAdd(dst, f32_to_f64i(v));
  }
}
// |v| as bits with the sign bit cleared, on the integer pipe.  Written as PTX, like the
// exponent test below, so that the compiler cannot turn either back into FP64 instructions
// (fabs, a compare).  With both in PTX the residual kernels measured 8-9 % faster on a GB300.
__device__ __forceinline__ unsigned long long absbits(double v) {
  unsigned long long r;
  asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(r) : "l"(dbits(v)));
  return r;
}
// |v| (the same value as fabs) on the integer pipe
__device__ __forceinline__ double absd(double v) { return bits2d(absbits(v)); }
// Inf or NaN, by the exponent bits (integer pipe, for the same reason)
__device__ __forceinline__ bool nonfinite_bits(double v) {
  unsigned long long r;
  asm("and.b64 %0, %1, 0x7ff0000000000000;" : "=l"(r) : "l"(dbits(v)));
  return r == 0x7ff0000000000000ull;
}

// Launch as a programmatic dependent of the previous kernel on the stream (its launch overlaps
// that kernel's end; the kernel's gate_open waits for it with griddepcontrol.wait before any
// read).  Used for every step kernel that begins with gate_open: the solve sweeps, the
// momentum right-hand side, the ghost rows, the projection, the defect, the pressure output,
// the maxima and the forces.
// GHOSTMAC_NO_PDL=1 launches them as ordinary stream successors.
static int pdl_mode() {
  static int mode = -1;
  if (mode < 0) {
    const char* e = std::getenv("GHOSTMAC_NO_PDL");
    mode = (e && e[0] == '1') ? 0 : 1;
  }
  return mode;
}
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_mode();
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

static inline unsigned blocks_for(int64_t n, int tpb = TPB) { return (unsigned)((n + tpb - 1) / tpb); }
// Grid of the reduction kernels: grid-stride loops over at most 4 blocks per SM of a GB300,
// so each block commits its partial max/sum with one atomic per quantity.
static inline unsigned reduce_blocks(int64_t n) {
  unsigned b = blocks_for(n);
  return b < 608u ? b : 608u;
}
// Blocks of the residual kernels.  Each block ends with its reductions (a warp-shuffle sum
// costs five adds per thread), so fewer, longer-striding blocks spend less on them.  Measured
// on the 800x820 case: the FP64 residual (sums in FP64) was fastest at 304 blocks, the
// FP32-mode residual (sums in FP32, and the FP64 stencil its only FP64 work) at 608.
static inline unsigned residual_blocks(int64_t n, bool res_f32) {
  const unsigned b = blocks_for(n), cap = res_f32 ? 608u : 304u;
  return b < cap ? b : cap;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// Host-side count of kernel launches issued by this library (all launchers call note_launch).
static std::atomic<long long> g_launches{0};
static inline void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long kernel_launch_count() { return g_launches.load(); }
// Graph capture records launches that have not run yet; the host corrects the count by the
// captured nodes and adds the nodes a graph replay executed.
void kernel_launch_adjust(long long delta) { g_launches.fetch_add(delta, std::memory_order_relaxed); }

// Optional CUDA-event timing of every launch, summed per kernel class (used by the
// benchmark for its per-class breakdown and the dominant kernel's launch time).  Classes:
// 1 x pass, 2 column solves, 3 momentum, 4 residual, 5 boundary chain / Schur GEMV, 6 projection pieces,
// 7 defect / pressure output, 8 ghost rows, 9 forces / maxima, 10 gates and loop control,
// 11 FP32 Jacobi sweeps of the Helmholtz systems, 12 row transforms on the tensor cores.
namespace {
struct KTimer {
  bool on = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> cls;
  int used = 0;
  std::vector<double> bytes;
  double total_ms[KT_CLASSES] = {};
  double total_bytes[KT_CLASSES] = {};
  long long count[KT_CLASSES] = {};
};
KTimer g_kt;
}  // namespace
// begin and end marks of one launch; the end mark carries the launch's algorithmic bytes
static inline void kt_mark(int cls, cudaStream_t st, double bytes = 0.0) {
  if (!g_kt.on || g_kt.used >= (int)g_kt.ev.size()) return;
  g_kt.cls[g_kt.used] = cls;
  g_kt.bytes[g_kt.used] = bytes;
  cudaEventRecord(g_kt.ev[g_kt.used++], st);
}
void ktimer_enable(int on) {
  if (g_kt.ev.empty()) {
    g_kt.ev.resize(4096);
    g_kt.cls.resize(4096);
    g_kt.bytes.resize(4096);
    for (auto& e : g_kt.ev) cudaEventCreate(&e);
  }
  g_kt.on = on != 0;
  g_kt.used = 0;
  for (int k = 0; k < KT_CLASSES; ++k) { g_kt.total_ms[k] = 0; g_kt.total_bytes[k] = 0; g_kt.count[k] = 0; }
}
// Folds the recorded pairs (begin and end of one launch are consecutive) into the totals;
// the streams must be synchronised.
void ktimer_collect() {
  for (int i = 0; i + 1 < g_kt.used; i += 2) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, g_kt.ev[i], g_kt.ev[i + 1]) == cudaSuccess) {
      const int c = g_kt.cls[i];
      if (c >= 0 && c < KT_CLASSES) {
        g_kt.total_ms[c] += ms;
        g_kt.total_bytes[c] += g_kt.bytes[i + 1];
        g_kt.count[c] += 1;
      }
    }
  }
  cudaGetLastError();
  g_kt.used = 0;
}
bool ktimer_active() { return g_kt.on; }
void note_launch_ext() { note_launch(); }
void kt_mark_ext(int cls, cudaStream_t st, double bytes) { kt_mark(cls, st, bytes); }
int pdl_mode_ext() { return pdl_mode(); }
void ktimer_read(int cls, double* total_ms, long long* count, double* bytes) {
  const bool ok = cls >= 0 && cls < KT_CLASSES;
  *total_ms = ok ? g_kt.total_ms[cls] : 0.0;
  *count = ok ? g_kt.count[cls] : 0;
  *bytes = ok ? g_kt.total_bytes[cls] : 0.0;
}

// ---------------------------------------------------------------------------
// separable inverse: x pass (rows) and y pass (columns with eigenvalue scaling)
// ---------------------------------------------------------------------------
// Row transforms.  A group of `gthreads` threads (one warp, or whole warps on a named
// barrier) transforms one line group -- two paired lines for the Makhoul and DST-I
// transforms, one line for the type-IV transforms -- and a block holds `gpb` groups.
// Rows r0 .. r0+nr-1 are transformed.  Masked load with the optional spectral correction
// of the boundary term (YCorr); masked store with the optional epilogue out = add + v.
// shared memory of one line group: the two FFT buffers (the real results go to the buffer the
// FFT does not end in)
template <typename T>
__host__ __device__ inline size_t xpass_group_smem(int type, int n) {
  const int lpw = r2r_paired(type) ? 2 : 1;
  return 2 * (size_t)r2r_buffer_elems(type, n, lpw) * sizeof(cplx<T>);
}
// lengths (complex entries) of the plan's twiddles, the pre- and the post-twiddles of a transform
__host__ __device__ inline int xpass_tw_len(int type, int n, int which, int plan_tw) {
  const int fam = r2r_family(type);
  if (which == 0) return plan_tw;
  if (which == 1) return fam == 2 ? n / 2 : 1;
  return fam == 2 ? n / 2 : (fam == 3 ? 1 : n);
}
template <typename T>
__host__ __device__ inline size_t xpass_tw_bytes(int type, int n, int plan_tw) {
  return ((size_t)(xpass_tw_len(type, n, 0, plan_tw) + xpass_tw_len(type, n, 1, plan_tw) +
                   xpass_tw_len(type, n, 2, plan_tw)) * sizeof(cplx<T>) + 15) / 16 * 16;
}
size_t xpass_smem_per_group(int type, int n, bool fp32) {
  return fp32 ? xpass_group_smem<float>(type, n) : xpass_group_smem<double>(type, n);
}
size_t xpass_smem_tables(int type, int n, int plan_tw, bool fp32) {
  return fp32 ? xpass_tw_bytes<float>(type, n, plan_tw) : xpass_tw_bytes<double>(type, n, plan_tw);
}

static constexpr int XB = 4;  // loads batched per thread in the row passes
static constexpr int XT = 8;  // table loads in flight per thread while the tables are staged
// Twiddle tables of one transform type staged into the block's shared memory (read by every
// stage of every group: a global load per stage would put an L2 round trip on each stage's
// critical path).  Each thread has XT loads in flight before its first store, so a table of
// up to XT * blockDim.x entries costs one round trip.  The tables are written once at set-up,
// never by a kernel, so the kernels stage them before waiting on the previous kernel of the
// stream.  Called by all threads of the block; ends with a block barrier.
template <typename T>
__device__ __forceinline__ R2RTables<T> xpass_stage_tables(int type, int n, const FftPlan& plan,
                                                           const R2RTables<T>& tb, unsigned char* smem_raw) {
  const int n0 = xpass_tw_len(type, n, 0, plan.tw_len), n1 = xpass_tw_len(type, n, 1, plan.tw_len);
  const int tot = n0 + n1 + xpass_tw_len(type, n, 2, plan.tw_len);
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  for (int q0 = threadIdx.x; q0 < tot; q0 += XT * blockDim.x) {
    cplx<T> v[XT];
#pragma unroll
    for (int u = 0; u < XT; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < tot) v[u] = q < n0 ? tb.W[q] : (q < n0 + n1 ? tb.pre[q - n0] : tb.post[q - n0 - n1]);
    }
#pragma unroll
    for (int u = 0; u < XT; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < tot) tw[q] = v[u];
    }
  }
  __syncthreads();
  return R2RTables<T>{tw, tw + n0, tw + n0 + n1};
}

// The line groups of (virtual) block bi: group grp of the block transforms lines
// (bi * gpb + grp) * lpw ... of rows r0 .. r0+nr-1.  Groups past the end return at once; every
// group synchronises on its own named barrier only, so a block may run this for several bi in turn.
template <typename T, typename TI, typename TO>
__device__ __forceinline__ void xpass_block(int bi, int n, int r0, int nr, int type, const FftPlan& plan,
                                            const R2RTables<T>& ts, const TI* __restrict__ in, int64_t ibase,
                                            int64_t ipitch, const uint8_t* __restrict__ icls, TO* __restrict__ out,
                                            int64_t obase, int64_t opitch, const uint8_t* __restrict__ ocls,
                                            const double* __restrict__ add, const YCorr<T>& corr, int gthreads,
                                            int gpb, unsigned char* smem_raw) {
  const int grp = threadIdx.x / gthreads, tid = threadIdx.x - grp * gthreads;
  const int lpw = r2r_paired(type) ? 2 : 1;
  const int l0 = (bi * gpb + grp) * lpw;
  if (grp >= gpb || l0 >= nr) return;
  const int nl = min(lpw, nr - l0);
  unsigned char* mine = smem_raw + xpass_tw_bytes<T>(type, n, plan.tw_len) + (size_t)grp * xpass_group_smem<T>(type, n);
  cplx<T>* a = reinterpret_cast<cplx<T>*>(mine);
  cplx<T>* b = a + r2r_buffer_elems(type, n, lpw);
  const Grp G{tid, gthreads, grp + 1};
  // per line (at most two): input row offset and the band correction (band row that scales or
  // is the correction, decay factors of this row: nullptr inside the band); scalars selected by
  // the line index, not an indexed array (that would go to local memory)
  int64_t irow0 = 0, irow1 = 0;
  const T *cb0 = nullptr, *cb1 = nullptr, *cf0 = nullptr, *cf1 = nullptr;
  for (int l = 0; l < nl; ++l) {
    const int r = r0 + l0 + l;
    const int64_t ir = ibase + (int64_t)r * ipitch;
    const T* cb = nullptr;
    const T* cf = nullptr;
    if (corr.band) {
      if (r < corr.j0) {
        cb = corr.band;
        cf = corr.phi + (int64_t)r * n;
      } else if (r > corr.j1) {
        cb = corr.band + (int64_t)(corr.j1 - corr.j0) * n;
        cf = corr.psi + (int64_t)(r - corr.j1 - 1) * n;
      } else {
        cb = corr.band + (int64_t)(r - corr.j0) * n;
      }
    }
    if (l == 0) { irow0 = ir; cb0 = cb; cf0 = cf; }
    else { irow1 = ir; cb1 = cb; cf1 = cf; }
  }
  // element e of line l: masked input minus the correction
  auto x = [&](int l, int e) -> T {
    const int64_t o = (l == 0 ? irow0 : irow1) + e;
    const T* cb = l == 0 ? cb0 : cb1;
    const T* cf = l == 0 ? cf0 : cf1;
    const TI v = in[o];
    const uint8_t mk = icls ? icls[o] : (uint8_t)CLS_ACTIVE;
    const T cv = cb ? (cf ? cf[e] * cb[e] : cb[e]) : (T)0;
    return ((mk & CLS_ACTIVE) ? cvt_to<T>(v) : (T)0) - cv;
  };
  const T* stage = r2r_lines<T>(type, n, nl, a, b, plan, ts, G, x);
  for (int l = 0; l < nl; ++l) {
    const int64_t row = obase + (int64_t)(r0 + l0 + l) * opitch;
    for (int e0 = tid; e0 < n; e0 += XB * gthreads) {
      uint8_t mk[XB];
      double ad[XB];
#pragma unroll
      for (int u = 0; u < XB; ++u) {
        const int64_t fo = row + e0 + u * gthreads;
        if (e0 + u * gthreads < n) {
          mk[u] = ocls ? ocls[fo] : (uint8_t)CLS_ACTIVE;
          ad[u] = add ? add[fo] : 0.0;
        }
      }
#pragma unroll
      for (int u = 0; u < XB; ++u) {
        const int e = e0 + u * gthreads;
        if (e >= n) continue;
        const int64_t fo = row + e;
        if (!(mk[u] & CLS_ACTIVE)) {
          out[fo] = (TO)0;
        } else {
          const T v = stage[l * n + e];
          out[fo] = add ? cvt_to<TO>(ad[u] + cvt_to<double>(v)) : cvt_to<TO>(v);
        }
      }
    }
  }
}

template <typename T, typename TI, typename TO>
__global__ void k_xpass(int n, int r0, int nr, int type, FftPlan plan, R2RTables<T> tb, const TI* __restrict__ in,
                        int64_t ibase, int64_t ipitch, const uint8_t* __restrict__ icls, TO* __restrict__ out,
                        int64_t obase, int64_t opitch, const uint8_t* __restrict__ ocls, const double* __restrict__ add,
                        YCorr<T> corr, int gthreads, int gpb, Gate gate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const R2RTables<T> ts = xpass_stage_tables<T>(type, n, plan, tb, smem_raw);
  if (!gate_open(gate)) return;
  xpass_block<T, TI, TO>(blockIdx.x, n, r0, nr, type, plan, ts, in, ibase, ipitch, icls, out, obase, opitch, ocls,
                         add, corr, gthreads, gpb, smem_raw);
}

template <typename T, typename TI, typename TO>
void launch_xpass(const TransformTables& tt, bool inverse, int r0, int nr, const TI* in, int64_t ibase,
                  int64_t ipitch, const uint8_t* icls, TO* out, int64_t obase, int64_t opitch, const uint8_t* ocls,
                  const double* add, const YCorr<T>& corr, const Gate& gate, cudaStream_t st) {
  if (nr <= 0) return;
  using C = cplx<T>;
  const int type = inverse ? tt.tx_inv : tt.tx_fwd;
  R2RTables<T> tb{(const C*)tt.Wx, (const C*)(inverse ? tt.prex_inv : tt.prex),
                  (const C*)(inverse ? tt.postx_inv : tt.postx)};
  const int lpw = r2r_paired(type) ? 2 : 1;
  const int per_block = tt.xg_pb * lpw;
  const unsigned grid = (unsigned)((nr + per_block - 1) / per_block);
  note_launch();
  kt_mark(1, st);
  launch_pdl(k_xpass<T, TI, TO>, dim3(grid), dim3(tt.xg_threads * tt.xg_pb), tt.smem_x, st, tt.n, r0, nr, type,
             tt.plan_x, tb, in, ibase, ipitch, icls, out, obase, opitch, ocls, add, corr, tt.xg_threads, tt.xg_pb,
             gate);
  // algorithmic bytes: one read and one write per point, class maps, the added field and the
  // correction band (tables of the decay factors once per point)
  kt_mark(1, st, (double)nr * tt.n * (sizeof(TI) + sizeof(TO) + (icls ? 1 : 0) + (ocls ? 1 : 0) + (add ? 8 : 0) +
                                      (corr.band ? sizeof(T) : 0)));
}
template void launch_xpass<double, double, double>(const TransformTables&, bool, int, int, const double*, int64_t,
                                                   int64_t, const uint8_t*, double*, int64_t, int64_t,
                                                   const uint8_t*, const double*, const YCorr<double>&, const Gate&,
                                                   cudaStream_t);
template void launch_xpass<float, double, float>(const TransformTables&, bool, int, int, const double*, int64_t,
                                                 int64_t, const uint8_t*, float*, int64_t, int64_t, const uint8_t*,
                                                 const double*, const YCorr<float>&, const Gate&, cudaStream_t);
template void launch_xpass<float, float, float>(const TransformTables&, bool, int, int, const float*, int64_t,
                                                int64_t, const uint8_t*, float*, int64_t, int64_t, const uint8_t*,
                                                const double*, const YCorr<float>&, const Gate&, cudaStream_t);
template void launch_xpass<float, float, double>(const TransformTables&, bool, int, int, const float*, int64_t,
                                                 int64_t, const uint8_t*, double*, int64_t, int64_t, const uint8_t*,
                                                 const double*, const YCorr<float>&, const Gate&, cudaStream_t);

// ---------------------------------------------------------------------------
// y direction of the separable inverse: for every x-mode kx the column system
// (L_y + lambda_x(kx)) z = s / (2 nx) (pressure) or ((1 - c lambda_x) - c L_y) z = s / (2 nx)
// (Helmholtz) is tridiagonal with a constant off-diagonal.  It is solved by a
// partition method: P chunks of inner rows separated by interface rows; each
// thread runs Thomas on one chunk with precomputed pivots, one thread per column
// solves the interface system, and the chunk solutions take the spike
// corrections.  Tables (rows x cols, same layout as the spectral array):
//   inner rows:     t0 = 1/pivot, t1 = left spike v, t2 = right spike w
//   interface rows: t0 = 1/pivot, t1 = sub-diagonal, t2 = sup/pivot of the interface system
// The data and every coefficient of the two recurrences are staged in shared memory
// first, so the dependent chains wait on shared-memory latency only.
// ---------------------------------------------------------------------------
template <typename T, int L>
__device__ __forceinline__ void ysolve_body(int n /*rows*/, int cols, const YChunks& ch, T gamma, T scale,
                                            const T* __restrict__ t0, const T* __restrict__ t1,
                                            const T* __restrict__ t2, T* __restrict__ S, int bid) {
  // L consecutive columns per block (L a power of two: thread -> (column, row/chunk) by shifts)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = n | 1;                                  // odd stride between the columns
  T* col = reinterpret_cast<T*>(smem_raw);              // L x ns values
  T* piv = col + (size_t)L * ns;                         // L x ns reciprocal pivots
  T* sl = piv + (size_t)L * ns;                          // L x ns left spikes (t1)
  T* sr = sl + (size_t)L * ns;                           // L x ns right spikes (t2)
  const int c0 = bid * L;
  const int P = ch.P;
  const int l = threadIdx.x & (L - 1);                   // column of this thread
  const int rsub = threadIdx.x / L;                      // row offset (load/store), chunk (solve)
  const int rstep = blockDim.x / L;
  const bool colok = c0 + l < cols;
  const int64_t cc = c0 + l;
  // load the column values and all three tables in one phase: 4 x 4 loads in flight per thread,
  // so the solve phases below wait on shared memory only
  for (int e0 = rsub; e0 < n; e0 += 4 * rstep) {
    T sv[4], pvv[4], v1[4], v2[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * rstep;
      if (colok && e < n) {
        const int64_t o = (int64_t)e * cols + cc;
        sv[u] = S[o];
        pvv[u] = t0[o];
        if (P > 1) {
          v1[u] = t1[o];
          v2[u] = t2[o];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * rstep;
      if (colok && e < n) {
        col[l * ns + e] = sv[u] * scale;
        piv[l * ns + e] = pvv[u];
        if (P > 1) {
          sl[l * ns + e] = v1[u];
          sr[l * ns + e] = v2[u];
        }
      }
    }
  }
  __syncthreads();
  const int p = rsub;
  const bool work = colok && p < P;
  int a = 0, b = -1;
  if (work) { a = ch.start[p]; b = ch.end[p]; }
  T* x = col + l * ns;
  const T* pv = piv + l * ns;
  const T* s1 = sl + l * ns;
  const T* s2 = sr + l * ns;
  // phase 1: chunk-local Thomas
  if (work) {
    T prev = 0;
    for (int j = a; j <= b; ++j) {
      prev = (x[j] - gamma * prev) * pv[j];
      x[j] = prev;
    }
    T next = x[b];
    for (int j = b - 1; j >= a; --j) {
      next = x[j] - (gamma * pv[j]) * next;
      x[j] = next;
    }
  }
  __syncthreads();
  // phase 2: interface system, one thread per column (its coefficients are the spike tables at
  // the interface rows)
  if (p == 0 && colok && P > 1) {
    T z = 0;
    for (int q = 0; q < P - 1; ++q) {
      const int e = ch.end[q] + 1;
      const T rhs = x[e] - gamma * x[e - 1] - gamma * x[e + 1];
      z = (rhs - s1[e] * z) * pv[e];
      x[e] = z;
    }
    T y = 0;
    for (int q = P - 2; q >= 0; --q) {
      const int e = ch.end[q] + 1;
      y = x[e] - s2[e] * y;
      x[e] = y;
    }
  }
  __syncthreads();
  // phase 3: spike corrections of the inner rows
  if (work && P > 1) {
    const T yl = p > 0 ? x[ch.end[p - 1] + 1] : (T)0;
    const T yr = p < P - 1 ? x[b + 1] : (T)0;
    for (int j = a; j <= b; ++j) x[j] = x[j] - yl * s1[j] - yr * s2[j];
  }
  __syncthreads();
  T* s_out = S + cc;
  if (colok)
    for (int e = rsub; e < n; e += rstep) s_out[(int64_t)e * cols] = col[l * ns + e];
}
template <typename T, int L>
__global__ void k_ysolve(int n /*rows*/, int cols, YChunks ch, T gamma, T scale, const T* __restrict__ t0,
                         const T* __restrict__ t1, const T* __restrict__ t2, T* __restrict__ S, Gate gate) {
  if (!gate_open(gate)) return;
  ysolve_body<T, L>(n, cols, ch, gamma, scale, t0, t1, t2, S, blockIdx.x);
}
size_t ysolve_smem(int rows, int lpb, bool fp32) {
  const size_t esz = fp32 ? 4 : 8;
  return (size_t)lpb * (rows | 1) * 4 * esz;  // values, pivots, left and right spikes
}

template <typename T>
void launch_ysolve(const TransformTables& tt, int cols, int rows, T* S, const Gate& gate, cudaStream_t st) {
  const unsigned gy = (unsigned)((cols + tt.lpb_y - 1) / tt.lpb_y);
  note_launch();
  kt_mark(2, st);
#define GM_YSOLVE(LL)                                                                                        \
  launch_pdl(k_ysolve<T, LL>, dim3(gy), dim3(tt.threads_y), tt.smem_y, st, rows, cols, tt.ych, (T)tt.gamma,     \
             (T)tt.yscale, (const T*)tt.t0, (const T*)tt.t1, (const T*)tt.t2, S, gate)
  switch (tt.lpb_y) {
    case 2: GM_YSOLVE(2); break;
    case 4: GM_YSOLVE(4); break;
    case 8: GM_YSOLVE(8); break;
    default: GM_YSOLVE(16); break;
  }
#undef GM_YSOLVE
  kt_mark(2, st, (double)rows * cols * sizeof(T) * 5);  // data in and out, three table entries per point
}
template void launch_ysolve<double>(const TransformTables&, int, int, double*, const Gate&, cudaStream_t);
template void launch_ysolve<float>(const TransformTables&, int, int, float*, const Gate&, cudaStream_t);

// Band solve of the boundary term: the x-transformed U c occupies rows j0..j1 only, so per
// x-mode its column solution is the band system (end pivots carry the elimination of the
// rows outside) followed by geometric decay outside the band (phi / psi tables, applied in
// the final x pass).  One thread per column; B holds nb x cols values in place.
template <typename T>
__global__ void k_yband(int nb, int cols, T gamma, T scale, const T* __restrict__ bpiv, T* __restrict__ B,
                        Gate gate) {
  if (!gate_open(gate)) return;
  // the block's columns of B and of the pivots are staged in shared memory first
  // (independent coalesced loads); then one thread per column runs the recurrences
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nc = blockDim.x;
  T* xb = reinterpret_cast<T*>(smem_raw);  // nb x nc
  T* pb = xb + (size_t)nb * nc;
  const int k0 = blockIdx.x * nc;
  const int kk = threadIdx.x;
  if (k0 + kk < cols) {
    for (int j0 = 0; j0 < nb; j0 += 8) {  // 8 rows in flight per thread
      T bv[8], pv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (j0 + u < nb) {
          const int64_t o = (int64_t)(j0 + u) * cols + k0 + kk;
          bv[u] = B[o];
          pv[u] = bpiv[o];
        }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (j0 + u < nb) {
          xb[(j0 + u) * nc + kk] = bv[u] * scale;
          pb[(j0 + u) * nc + kk] = pv[u];
        }
    }
  }
  __syncthreads();
  if (k0 + kk < cols) {
    T z = 0;
    for (int j = 0; j < nb; ++j) {
      z = (xb[j * nc + kk] - gamma * z) * pb[j * nc + kk];
      xb[j * nc + kk] = z;
    }
    T y = z;
    for (int j = nb - 2; j >= 0; --j) {
      y = xb[j * nc + kk] - (gamma * pb[j * nc + kk]) * y;
      xb[j * nc + kk] = y;
    }
  }
  if (k0 + kk < cols)
    for (int j = 0; j < nb; ++j) B[(int64_t)j * cols + k0 + kk] = xb[j * nc + kk];
}
template <typename T>
void launch_yband(const TransformTables& tt, int cols, T* B, const Gate& gate, cudaStream_t st) {
  const int nb = tt.bj1 - tt.bj0 + 1;
  if (nb <= 0) return;
  note_launch();
  kt_mark(2, st);
  // up to 32 columns per block (whole 128/256-byte row segments), shared memory 2 nb x nc values
  const int nc = (int)std::max<size_t>(1, std::min<size_t>(32, (48 * 1024) / (2 * (size_t)nb * sizeof(T))));
  k_yband<T><<<blocks_for(cols, nc), nc, (size_t)2 * nb * nc * sizeof(T), st>>>(nb, cols, (T)tt.gamma, (T)tt.yscale,
                                                                              (const T*)tt.bpiv, B, gate);
  kt_mark(2, st, (double)nb * cols * sizeof(T) * 3);
}
template void launch_yband<double>(const TransformTables&, int, double*, const Gate&, cudaStream_t);
template void launch_yband<float>(const TransformTables&, int, float*, const Gate&, cudaStream_t);

template <typename T, typename TI, typename TO>
__global__ void k_xpass_multi(const __grid_constant__ ArgPack<XpassArgs<T, TI, TO>> p);
template <typename T, int L>
__global__ void k_ysolve_multi(const __grid_constant__ ArgPack<YsolveArgs<T>> p);

// Opts the transform kernels into the large dynamic shared memory carve-out; returns the
// dynamic bytes every one of them may use (the opt-in limit minus their static shared memory).
template <typename K>
static int allow_dynamic_smem(K kernel, int optin) {
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, kernel) != cudaSuccess) return 0;
  int dyn = optin - (int)a.sharedSizeBytes;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) return 0;
  return dyn;
}
int configure_kernels(int smem_optin) {
  int d = smem_optin;
  d = std::min(d, allow_dynamic_smem(k_xpass<double, double, double>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass<float, double, float>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass<float, float, float>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass<float, float, double>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<double, 2>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<double, 4>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<double, 8>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<double, 16>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<float, 2>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<float, 4>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<float, 8>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve<float, 16>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass_multi<double, double, double>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass_multi<float, double, float>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass_multi<float, float, float>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_xpass_multi<float, float, double>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<double, 2>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<double, 4>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<double, 8>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<double, 16>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<float, 2>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<float, 4>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<float, 8>, smem_optin));
  d = std::min(d, allow_dynamic_smem(k_ysolve_multi<float, 16>, smem_optin));
  return d;
}

// ---------------------------------------------------------------------------
// boundary Schur correction: c = S^{-1} (C first), scattered into w2
// ---------------------------------------------------------------------------
static constexpr int SCHUR_ROWS = 4;
// c = M first[mcols] with M = S^{-1} C (rank x m, FP64), scattered to w2 at the boundary rows.
// Every block gathers the m points into shared memory (independent loads), then its warps
// take SCHUR_ROWS rows of the GEMV (lanes over the row, FP64 accumulation).
template <typename TF>
__global__ void k_schur(const TF* __restrict__ first, int rank, int m, const int64_t* __restrict__ mcols,
                        const double* __restrict__ M, const int64_t* __restrict__ rows, double* __restrict__ w2,
                        Gate gate) {
  if (!gate_open(gate)) return;
  extern __shared__ double gsh[];
  for (int q0 = threadIdx.x; q0 < m; q0 += 4 * blockDim.x) {
    int64_t ix[4];
    TF fv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (q0 + u * (int)blockDim.x < m) ix[u] = mcols[q0 + u * blockDim.x];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (q0 + u * (int)blockDim.x < m) fv[u] = first[ix[u]];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (q0 + u * (int)blockDim.x < m) gsh[q0 + u * blockDim.x] = cvt_to<double>(fv[u]);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int r0 = blockIdx.x * SCHUR_ROWS;
  for (int r = r0 + warp; r < min(rank, r0 + SCHUR_ROWS); r += nw) {
    const double* mr = M + (int64_t)r * m;
    double acc = 0.0;
#pragma unroll 8
    for (int q = lane; q < m; q += 32) acc += mr[q] * gsh[q];
    acc = warp_sum(acc);
    if (lane == 0) w2[rows[r]] = acc;
  }
}

template <typename TF>
void launch_schur(const TF* first, int rank, int m, const int64_t* mcols, const double* M, const int64_t* rows,
                  double* w2, const Gate& gate, cudaStream_t st) {
  if (rank <= 0) return;
  const unsigned g = (unsigned)((rank + SCHUR_ROWS - 1) / SCHUR_ROWS);
  note_launch();
  kt_mark(5, st);
  k_schur<TF><<<g, 32 * SCHUR_ROWS, (size_t)m * sizeof(double), st>>>(first, rank, m, mcols, M, rows, w2, gate);
  kt_mark(5, st, (double)m * (sizeof(TF) + 8) + (double)rank * m * 8 + rank * 16.0);
}
template void launch_schur<double>(const double*, int, int, const int64_t*, const double*, const int64_t*, double*,
                                   const Gate&, cudaStream_t);
template void launch_schur<float>(const float*, int, int, const int64_t*, const double*, const int64_t*, double*,
                                  const Gate&, cudaStream_t);

// ---------------------------------------------------------------------------
// boundary term by direct sums
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

static constexpr int BAND_TPB = 128;   // threads per output of the direct sums
static constexpr int BAND_ITEMS = 16;  // loads in flight per thread (n <= BAND_TPB * BAND_ITEMS per pass)

// Canonical order of the direct sums (every kernel that forms them uses it, so the single-case,
// fused and case-indexed paths agree bitwise): BAND_TPB threads per output, thread t adds its
// products at t, t + BAND_TPB, ... in order, then the warp sums, then the BAND_TPB / 32 warp
// partials in warp order.
template <typename TA, typename TB, typename TS>
__device__ __forceinline__ TS band_partial(const TA* __restrict__ a, const TB* __restrict__ b, int n, int t) {
  TS acc = 0;
  for (int k0 = t; k0 < n; k0 += BAND_TPB * BAND_ITEMS) {
    TA av[BAND_ITEMS];
    TB bv[BAND_ITEMS];
#pragma unroll
    for (int u = 0; u < BAND_ITEMS; ++u) {
      const int k = k0 + u * BAND_TPB;
      av[u] = k < n ? a[k] : (TA)0;
      bv[u] = k < n ? b[k] : (TB)0;
    }
#pragma unroll
    for (int u = 0; u < BAND_ITEMS; ++u) acc += cvt_to<TS>(av[u]) * cvt_to<TS>(bv[u]);
  }
  return acc;
}
// sum of a BAND_TPB-thread group's partials (part: BAND_TPB / 32 shared slots of this group);
// every thread of the block must call it (it holds block barriers)
template <typename T>
__device__ __forceinline__ T band_group_sum(T v, T* part, int t) {
  v = warp_sum_t<T>(v);
  __syncthreads();
  if ((t & 31) == 0) part[t >> 5] = v;
  __syncthreads();
  T s = 0;
#pragma unroll
  for (int w = 0; w < BAND_TPB / 32; ++w) s += part[w];
  return s;
}

// One block per point: the inverse row transform of its spectrum row evaluated at its column
// (coefficients in binv), all of a thread's products loaded before they are summed.
template <typename T>
__device__ __forceinline__ void band_first_body(int n, const int32_t* __restrict__ mrow, const T* __restrict__ binv,
                                                const T* __restrict__ spec, T* __restrict__ firstm, int q) {
  __shared__ T part[BAND_TPB / 32];
  const T v = band_group_sum<T>(
      band_partial<T, T, T>(binv + (int64_t)q * n, spec + (int64_t)mrow[q] * n, n, threadIdx.x), part, threadIdx.x);
  if (threadIdx.x == 0) firstm[q] = v;
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_first(int m, int n, const int32_t* __restrict__ mrow,
                                                         const T* __restrict__ binv, const T* __restrict__ spec,
                                                         T* __restrict__ firstm, Gate gate) {
  if (!gate_open(gate)) return;
  band_first_body<T>(n, mrow, binv, spec, firstm, blockIdx.x);
}

// One block per row of M: c[r] = M[r] . firstm (FP64 accumulation).
template <typename T>
__device__ __forceinline__ void band_gemv_body(int m, const double* __restrict__ M, const T* __restrict__ firstm,
                                               double* __restrict__ c, int r) {
  __shared__ double part[BAND_TPB / 32];
  const double v = band_group_sum<double>(band_partial<double, T, double>(M + (int64_t)r * m, firstm, m, threadIdx.x),
                                          part, threadIdx.x);
  if (threadIdx.x == 0) c[r] = v;
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_gemv(int rank, int m, const double* __restrict__ M,
                                                        const T* __restrict__ firstm, double* __restrict__ c,
                                                        Gate gate) {
  if (!gate_open(gate)) return;
  band_gemv_body<T>(m, M, firstm, c, blockIdx.x);
}

// The boundary term's Schur values in one sum per value: c[r] = G[r] . S[cj0 .. cj1 rows], with
// G = M binv folded on the host (G[r][(j - cj0) n + k] = sum over the points q of spectrum row j
// of M[r][q] binv[q][k]), so that the point values "first" are never formed.  Block (r, s) sums
// slice s of BAND_SPLIT slices (per-thread partials in T, the block's sum in FP64) and writes
// part[r BAND_SPLIT + s]; the band solve adds the slices in a fixed order.
template <typename T>
__device__ __forceinline__ void band_direct_body(int L, const T* __restrict__ G, const T* __restrict__ S,
                                                 double* __restrict__ part, int r, int sl) {
  __shared__ double dpart[BAND_TPB / 32];
  const int len = (L + BAND_SPLIT - 1) / BAND_SPLIT;
  const int i0 = sl * len, i1 = min(L, i0 + len);
  const T v = i1 > i0 ? band_partial<T, T, T>(G + (int64_t)r * L + i0, S + i0, i1 - i0, threadIdx.x) : (T)0;
  const double tot = band_group_sum<double>(cvt_to<double>(v), dpart, threadIdx.x);
  if (threadIdx.x == 0) part[r * BAND_SPLIT + sl] = tot;
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_direct(int L, const T* __restrict__ G, const T* __restrict__ S,
                                                          double* __restrict__ part, Gate gate) {
  if (!gate_open(gate)) return;
  band_direct_body<T>(L, G, S, part, blockIdx.x / BAND_SPLIT, blockIdx.x % BAND_SPLIT);
}

// Blocks of BAND_COLS columns x BAND_ROWT row threads.  Thread (kk, jt) forms the forward
// row transform of U c on band rows jt, jt + BAND_ROWT, ... of column k (a sum over that row's
// boundary values, c staged in shared memory), scaled; then one thread per column runs the band
// system (as k_yband) in shared memory, and all threads write the band back.
static constexpr int BAND_COLS = 16, BAND_ROWT = 16;
template <typename T>
__device__ __forceinline__ void band_fwd_solve_body(int nb, int n, int rank, const int32_t* __restrict__ bptr,
                                                    const double* __restrict__ c,
                                                    const T* __restrict__ bfwd, T gamma, T scale,
                                                    const T* __restrict__ bpiv, T* __restrict__ band, int bid,
                                                    int nsplit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* cs = reinterpret_cast<T*>(smem_raw);   // rank values c (band-row order, as the GEMV writes them)
  T* xb = cs + ((rank + 3) & ~3);           // nb x BAND_COLS
  T* pb = xb + (size_t)nb * BAND_COLS;      // nb x BAND_COLS
  int* ps = reinterpret_cast<int*>(pb + (size_t)nb * BAND_COLS);  // nb + 1 row pointers
  const int tid = threadIdx.x, kk = tid % BAND_COLS, jt = tid / BAND_COLS;
  // c[e], or the sum of its nsplit slices in slice order (k_band_direct)
  for (int e = tid; e < rank; e += blockDim.x) {
    double v = c[(int64_t)e * nsplit];
    for (int sl = 1; sl < nsplit; ++sl) v += c[(int64_t)e * nsplit + sl];
    cs[e] = cvt_to<T>(v);
  }
  for (int j = tid; j <= nb; j += blockDim.x) ps[j] = bptr[j];
  __syncthreads();
  const int k = bid * BAND_COLS + kk;
  if (k < n) {
    for (int j = jt; j < nb; j += BAND_ROWT) {
      const int e0 = ps[j], e1 = ps[j + 1];
      T z = 0;
      for (int e = e0; e < e1; e += 8) {
        T bv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) bv[u] = e + u < e1 ? bfwd[(int64_t)(e + u) * n + k] : (T)0;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (e + u < e1) z += cs[e + u] * bv[u];
      }
      xb[j * BAND_COLS + kk] = z * scale;
      pb[j * BAND_COLS + kk] = bpiv[(int64_t)j * n + k];
    }
  }
  __syncthreads();
  if (jt == 0 && k < n) {
    T z = 0;
    for (int j = 0; j < nb; ++j) {
      z = (xb[j * BAND_COLS + kk] - gamma * z) * pb[j * BAND_COLS + kk];
      xb[j * BAND_COLS + kk] = z;
    }
    T y = z;
    for (int j = nb - 2; j >= 0; --j) {
      y = xb[j * BAND_COLS + kk] - (gamma * pb[j * BAND_COLS + kk]) * y;
      xb[j * BAND_COLS + kk] = y;
    }
  }
  __syncthreads();
  if (k < n)
    for (int j = jt; j < nb; j += BAND_ROWT) band[(int64_t)j * n + k] = xb[j * BAND_COLS + kk];
}
template <typename T>
__global__ void __launch_bounds__(BAND_COLS * BAND_ROWT) k_band_fwd_solve(
    int nb, int n, int rank, const int32_t* __restrict__ bptr,
    const double* __restrict__ c, const T* __restrict__ bfwd, T gamma, T scale, const T* __restrict__ bpiv,
    T* __restrict__ band, Gate gate, int nsplit) {
  if (!gate_open(gate)) return;
  band_fwd_solve_body<T>(nb, n, rank, bptr, c, bfwd, gamma, scale, bpiv, band, blockIdx.x, nsplit);
}

int band_fwd_blocks(int n) { return (n + BAND_COLS - 1) / BAND_COLS; }
size_t band_fwd_smem(int nb, int rank, bool fp32) {
  const size_t esz = fp32 ? 4 : 8;
  return (size_t)((rank + 3) & ~3) * esz + (size_t)2 * nb * BAND_COLS * esz + (size_t)(nb + 1) * sizeof(int);
}

template <typename T>
void launch_band_first(int m, int n, const int32_t* mrow, const T* binv, const T* spec, T* firstm, const Gate& gate,
                       cudaStream_t st) {
  if (m <= 0) return;
  note_launch();
  kt_mark(5, st);
  launch_pdl(k_band_first<T>, dim3((unsigned)m), dim3(BAND_TPB), 0, st, m, n, mrow, binv, spec, firstm, gate);
  kt_mark(5, st, (double)m * n * 2 * sizeof(T));
}
template <typename T>
void launch_band_gemv(int rank, int m, const double* M, const T* firstm, double* c, const Gate& gate,
                      cudaStream_t st) {
  if (rank <= 0) return;
  note_launch();
  kt_mark(5, st);
  launch_pdl(k_band_gemv<T>, dim3((unsigned)rank), dim3(BAND_TPB), 0, st, rank, m, M, firstm, c, gate);
  kt_mark(5, st, (double)rank * m * 8 + (double)m * sizeof(T) + rank * 8.0);
}
template <typename T>
void launch_band_direct(int rank, int L, const T* G, const T* S, double* part, const Gate& gate, cudaStream_t st) {
  if (rank <= 0) return;
  note_launch();
  kt_mark(5, st);
  launch_pdl(k_band_direct<T>, dim3((unsigned)(rank * BAND_SPLIT)), dim3(BAND_TPB), 0, st, L, G, S, part, gate);
  // G read once, the spectrum rows once per value (L2), the slices written
  kt_mark(5, st, (double)rank * L * sizeof(T) + (double)L * sizeof(T) + rank * BAND_SPLIT * 8.0);
}
template <typename T>
void launch_band_fwd_solve(const TransformTables& tt, int n, int rank, const int32_t* bptr, const double* c,
                           const T* bfwd, T* band, const Gate& gate, cudaStream_t st, int nsplit) {
  const int nb = tt.bj1 - tt.bj0 + 1;
  if (nb <= 0) return;
  note_launch();
  kt_mark(5, st);
  launch_pdl(k_band_fwd_solve<T>, dim3((unsigned)((n + BAND_COLS - 1) / BAND_COLS)), dim3(BAND_COLS * BAND_ROWT),
             band_fwd_smem(nb, rank, sizeof(T) == 4), st, nb, n, rank, bptr, c, bfwd, (T)tt.gamma,
             (T)tt.yscale, (const T*)tt.bpiv, band, gate, nsplit);
  // the forward coefficients, the values c, the pivots and the band written once
  kt_mark(5, st, (double)rank * n * sizeof(T) + rank * 8.0 + (double)nb * n * 2 * sizeof(T));
}
template void launch_band_first<double>(int, int, const int32_t*, const double*, const double*, double*, const Gate&,
                                        cudaStream_t);
template void launch_band_first<float>(int, int, const int32_t*, const float*, const float*, float*, const Gate&,
                                       cudaStream_t);
template void launch_band_gemv<double>(int, int, const double*, const double*, double*, const Gate&, cudaStream_t);
template void launch_band_gemv<float>(int, int, const double*, const float*, double*, const Gate&, cudaStream_t);
template void launch_band_fwd_solve<double>(const TransformTables&, int, int, const int32_t*, const double*,
                                            const double*, double*, const Gate&, cudaStream_t, int);
template void launch_band_fwd_solve<float>(const TransformTables&, int, int, const int32_t*, const double*,
                                           const float*, float*, const Gate&, cudaStream_t, int);
template void launch_band_direct<double>(int, int, const double*, const double*, double*, const Gate&, cudaStream_t);
template void launch_band_direct<float>(int, int, const float*, const float*, double*, const Gate&, cudaStream_t);

// ---------------------------------------------------------------------------
// sparse rows with their loads batched: the column indices and values of up to CSR_B entries
// are loaded together, then the x values they point at, then the products are summed in entry
// order (the same sum as the one-entry-at-a-time loop, without an L2 round trip per entry)
// ---------------------------------------------------------------------------
template <int CSR_B = 8, typename F>
__device__ __forceinline__ void csr_row(const int64_t* __restrict__ col, const double* __restrict__ val, int64_t e0,
                                        int64_t e1, const double* __restrict__ x, int64_t xoff, F&& f) {
  for (int64_t e = e0; e < e1; e += CSR_B) {
    int64_t ci[CSR_B];
    double v[CSR_B], xv[CSR_B];
#pragma unroll
    for (int u = 0; u < CSR_B; ++u)
      if (e + u < e1) {
        ci[u] = col[e + u];
        v[u] = val[e + u];
      }
#pragma unroll
    for (int u = 0; u < CSR_B; ++u)
      if (e + u < e1) xv[u] = x[xoff + ci[u]];
#pragma unroll
    for (int u = 0; u < CSR_B; ++u)
      if (e + u < e1) f(v[u], xv[u]);
  }
}

// ---------------------------------------------------------------------------
// ghost extension rows
// ---------------------------------------------------------------------------
// Each ghost value is its row of interior values (the stencils read no ghost point).  A row's
// entries are spread over GHOST_LANES lanes, so its loads take one or two rounds instead of a
// serial chain through L2, and the lanes' partial sums are added in a fixed butterfly order.
constexpr int GHOST_LANES = 8;
__global__ void k_ghost(double* __restrict__ f, int n, const int64_t* __restrict__ rows, const int64_t* __restrict__ ptr,
                        const int64_t* __restrict__ col, const double* __restrict__ val, Gate gate) {
  if (!gate_open(gate)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = t / GHOST_LANES, l = t % GHOST_LANES;
  double acc = 0.0;
  if (r < n)
    for (int64_t e = ptr[r] + l, e1 = ptr[r + 1]; e < e1; e += GHOST_LANES) acc += val[e] * f[col[e]];
  for (int o = GHOST_LANES / 2; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (r < n && l == 0) f[rows[r]] = acc;
}

void launch_ghost(double* field, int n, const int64_t* rows, const int64_t* ptr, const int64_t* col,
                  const double* val, const Gate& gate, cudaStream_t st) {
  if (n <= 0) return;
  note_launch();
  kt_mark(8, st);
  launch_pdl(k_ghost, dim3(blocks_for((int64_t)n * GHOST_LANES, 128)), dim3(128), 0, st, field, n, rows, ptr, col, val, gate);
  kt_mark(8, st);
}

// ---------------------------------------------------------------------------
// stencils on the staggered grid
// ---------------------------------------------------------------------------
struct Grid {
  int nx, ny;
  int64_t usize;
  __device__ __forceinline__ int64_t u(int j, int i) const { return (int64_t)j * (nx + 1) + i; }
  __device__ __forceinline__ int64_t v(int j, int i) const { return usize + (int64_t)j * nx + i; }
  __device__ __forceinline__ int64_t p(int j, int i) const { return (int64_t)j * nx + i; }
};

// -N(u) at u face (j,i), i>=1, before /(dx dy) (solver/numba_kernels.py:17-74 with nu=0);
// arithmetic in T (double for the plain path, float in the FP32 mode)
template <typename T, typename S>
__device__ __forceinline__ T adv_u(const S* __restrict__ U, const Grid& g, int j, int i, T dx, T dy) {
  const int nx = g.nx, ny = g.ny;
  const T h = (T)0.5;
  auto fxy = [&](int jj, int ii) -> T {  // corner flux at (jj, ii), jj in [0, ny]
    if (jj == 0 || jj == ny) return (T)0;
    T vf;
    if (ii == 0) vf = (T)U[g.v(jj, 0)];
    else if (ii == nx) vf = (T)U[g.v(jj, nx - 1)];
    else vf = h * ((T)U[g.v(jj, ii - 1)] + (T)U[g.v(jj, ii)]);
    T ua = h * ((T)U[g.u(jj - 1, ii)] + (T)U[g.u(jj, ii)]);
    return -((vf * ua) * dx);
  };
  T uW = (T)U[g.u(j, i - 1)], uC = (T)U[g.u(j, i)];
  T fl = h * (uW + uC);
  T fxxW = -((fl * fl) * dy);
  if (i < nx) {
    T fr = h * (uC + (T)U[g.u(j, i + 1)]);
    T fxxE = -((fr * fr) * dy);
    return (fxxE - fxxW) + (fxy(j + 1, i) - fxy(j, i));
  }
  return (-uC * uC) * dy - fxxW + h * (fxy(j + 1, nx) - fxy(j, nx));
}

// -N(v) at v face (j,i), 1<=j<=ny-1 (solver/numba_kernels.py:77-142 with nu=0)
template <typename T, typename S>
__device__ __forceinline__ T adv_v(const S* __restrict__ U, const Grid& g, int j, int i, T dx, T dy) {
  const int nx = g.nx;
  const T h = (T)0.5;
  auto fyx = [&](int jj, int ii) -> T {  // corner flux at (jj, ii), ii in [0, nx]
    if (ii == 0) return (T)0;
    T uf = h * ((T)U[g.u(jj - 1, ii)] + (T)U[g.u(jj, ii)]);
    if (ii == nx) return (-uf * (T)U[g.v(jj, nx - 1)]) * dy;
    T va = h * ((T)U[g.v(jj, ii - 1)] + (T)U[g.v(jj, ii)]);
    return -((uf * va) * dy);
  };
  T vS = (T)U[g.v(j - 1, i)], vC = (T)U[g.v(j, i)], vN = (T)U[g.v(j + 1, i)];
  T fb = h * (vS + vC), ft = h * (vC + vN);
  T fyyS = -((fb * fb) * dx), fyyN = -((ft * ft) * dx);
  return (fyx(j, i + 1) - fyx(j, i)) + (fyyN - fyyS);
}

// raw_l (5-point with channel-wall, inlet and outlet rules) at a u face (solver/optimized_ghost_cell.py:116-120)
template <typename T, typename S, typename GR = Grid>
__device__ __forceinline__ T lap_u(const S* __restrict__ U, const GR& g, int j, int i, T idx2, T idy2,
                                   bool inlet) {
  const int nx = g.nx, ny = g.ny;
  T acc = 0;
  if (j > 0) acc += idy2 * (T)U[g.u(j - 1, i)];
  if (i > 1 || inlet) acc += (i == nx ? (T)2 * idx2 : idx2) * (T)U[g.u(j, i - 1)];
  acc += ((T)-2 * idx2 - ((j == 0 || j == ny - 1) ? (T)3 : (T)2) * idy2) * (T)U[g.u(j, i)];
  if (i < nx) acc += idx2 * (T)U[g.u(j, i + 1)];
  if (j < ny - 1) acc += idy2 * (T)U[g.u(j + 1, i)];
  return acc;
}
// at a v face (solver/optimized_ghost_cell.py:121-123); walls v=0 are stored as zeros
template <typename T, typename S, typename GR = Grid>
__device__ __forceinline__ T lap_v(const S* __restrict__ U, const GR& g, int j, int i, T idx2, T idy2) {
  const int nx = g.nx;
  T acc = idy2 * (T)U[g.v(j - 1, i)];
  if (i > 0) acc += idx2 * (T)U[g.v(j, i - 1)];
  acc += (-(i == 0 ? (T)3 : (i == nx - 1 ? (T)1 : (T)2)) * idx2 - (T)2 * idy2) * (T)U[g.v(j, i)];
  if (i < nx - 1) acc += idx2 * (T)U[g.v(j, i + 1)];
  acc += idy2 * (T)U[g.v(j + 1, i)];
  return acc;
}
// G p at faces from a pressure grid with ghost values (solver/optimized_ghost_cell.py:94-107)
template <typename T, typename S, typename GR = Grid>
__device__ __forceinline__ T grad_u(const S* __restrict__ P, const GR& g, int j, int i, T gx) {
  if (i < g.nx) return gx * (T)P[g.p(j, i)] - gx * (T)P[g.p(j, i - 1)];
  return ((T)-2 * gx) * (T)P[g.p(j, g.nx - 1)];
}
template <typename T, typename S, typename GR = Grid>
__device__ __forceinline__ T grad_v(const S* __restrict__ P, const GR& g, int j, int i, T gy) {
  return gy * (T)P[g.p(j, i)] - gy * (T)P[g.p(j - 1, i)];
}

// decode a face-grid thread index
// (face grids hold fewer than 2^31 points, checked at set-up: 32-bit division suffices)
__device__ __forceinline__ bool face_of(int64_t t, const Grid& g, int& comp, int& j, int& i) {
  if (t < g.usize) {
    const unsigned ut = (unsigned)t, w = (unsigned)(g.nx + 1);
    comp = 0; j = (int)(ut / w); i = (int)(ut - (unsigned)j * w);
    return true;
  }
  int64_t r = t - g.usize;
  if (r >= (int64_t)(g.ny + 1) * g.nx) return false;
  const unsigned ur = (unsigned)r;
  comp = 1; j = (int)(ur / (unsigned)g.nx); i = (int)(ur - (unsigned)j * g.nx);
  return true;
}

// T: stencil arithmetic; S: storage type the stencils read (double, or the FP32 copies)
template <typename T, typename S>
__global__ void k_momentum(CaseDev c, MomentumArgs a, const S* __restrict__ Us, const S* __restrict__ Ps, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) {
    double z = (comp == 0 && i == 0) ? c.inlet[j] : 0.0;
    if (a.mode != 2 && a.now) a.now[t] = 0.0;
    a.out[t] = a.mode == 1 ? z : 0.0;
    return;
  }
  constexpr bool F32 = sizeof(T) == 4;
  const T dx = F32 ? (T)c.fdx : (T)c.dx, dy = F32 ? (T)c.fdy : (T)c.dy;
  const T idx2 = F32 ? (T)c.fidx2 : (T)c.idx2, idy2 = F32 ? (T)c.fidy2 : (T)c.idy2;
  const T iarea = F32 ? (T)c.fiarea : (T)c.iarea, nu = F32 ? (T)c.fnu : (T)c.nu;
  const T dt = F32 ? (T)a.dt32 : (T)a.dt;
  const double q = a.U[t];
  T lq, gp, now = 0, off = 0;
  if (comp == 0) {
    lq = nu * lap_u<T>(Us, g, j, i, idx2, idy2, true);
    gp = grad_u<T>(Ps, g, j, i, F32 ? (T)c.fgx : (T)c.gx);
    if (a.mode != 2) {
      now = adv_u<T>(Us, g, j, i, dx, dy) * iarea;
      if (i == c.nx) now *= (T)2;
    }
    if (i == 1) off = nu * (idx2 * (T)c.inlet[j]);
  } else {
    lq = nu * lap_v<T>(Us, g, j, i, idx2, idy2);
    gp = grad_v<T>(Ps, g, j, i, F32 ? (T)c.fgy : (T)c.gy);
    if (a.mode != 2) now = adv_v<T>(Us, g, j, i, dx, dy) * iarea;
  }
  if (a.mode == 1) {
    a.now[t] = cvt_to<double>(now);
    a.out[t] = q + cvt_to<double>(((T)0.5 * dt) * ((now + lq) - gp));
    return;
  }
  T expl;
  if (a.mode == 0) {
    const T alpha = F32 ? (T)a.alpha32 : (T)a.alpha;
    expl = ((T)1 + alpha) * now - alpha * cvt_to<T>(a.prev[t]);
    a.now[t] = cvt_to<double>(now);
  } else {
    if (comp == 0) {
      expl = adv_u<T>(a.Uhalf, g, j, i, dx, dy) * iarea;
      if (i == c.nx) expl *= (T)2;
    } else {
      expl = adv_v<T>(a.Uhalf, g, j, i, dx, dy) * iarea;
    }
  }
  // rhs = q + dt (explicit + L q / 2 - G p) + dt/2 offset (solver/numba_kernels.py:596-601)
  if constexpr (sizeof(T) == 8)
    a.out[t] = (q + (double)(dt * (expl + (T)0.5 * lq - gp))) + (double)(((T)0.5 * dt) * off);
  else  // one FP64 add per face (the conversion runs on the integer pipe)
    a.out[t] = q + cvt_to<double>(dt * (expl + (T)0.5 * lq - gp) + ((T)0.5 * dt) * off);
}

// ---------------------------------------------------------------------------
// The AB2 momentum right-hand side (mode 0 of k_momentum) from a shared-memory tile.
//
// A block owns a TJ x TI patch of "points" (j, i), j in [0, ny], i in [0, nx]: point (j, i) is
// the u face (j, i) when j < ny and the v face (j, i) when i < nx.  It loads the u, v and p
// values its faces read (one halo row / column) once, with coalesced row loads, and forms each
// shared flux once instead of once per face that uses it:
//   corner products C = ua vf at the cell corners (jj, ii), 1 <= jj <= ny-1, 1 <= ii <= nx, where
//     ua = (u(jj-1, ii) + u(jj, ii)) / 2 and vf = (v(jj, ii-1) + v(jj, ii)) / 2 (v(jj, nx-1) at the
//     outlet); the u faces use -(C dx) (their fxy corner flux), the v faces -(C dy) (fyx): four
//     faces share each corner;
//   centre fluxes Xu = -((u(j, ii-1) + u(j, ii))^2 / 4 dy) of the u cells and
//     Yv = -((v(jj-1, i) + v(jj, i))^2 / 4 dx) of the v cells, two faces each
// (solver/numba_kernels.py:17-142: the same flux formulas as adv_u / adv_v).  The diffusion and
// pressure-gradient stencils read the tile through the same lap / grad functions as k_momentum.
// ---------------------------------------------------------------------------
static constexpr int MTI = 32, MTJ = 8;  // points per tile: 32 along x (one warp), 8 rows
// offsets of global (j, i) in the shared tiles: u and v tiles of (MTJ+2) x (MTI+2) (rows j0-1 ..
// j0+MTJ, columns i0-1 .. i0+MTI), the u tile first; the p tile (MTJ+1) x (MTI+1)
struct TileGrid {
  int nx, ny, j0, i0;
  static constexpr int W = MTI + 2, H = MTJ + 2, WP = MTI + 1;
  __device__ __forceinline__ int u(int j, int i) const { return (j - j0 + 1) * W + (i - i0 + 1); }
  __device__ __forceinline__ int v(int j, int i) const { return H * W + (j - j0 + 1) * W + (i - i0 + 1); }
  __device__ __forceinline__ int p(int j, int i) const { return (j - j0 + 1) * WP + (i - i0 + 1); }
};

template <typename T, typename S>
__global__ void __launch_bounds__(MTI * MTJ) k_momentum_tiled(CaseDev c, MomentumArgs a, const S* __restrict__ Us,
                                                              const S* __restrict__ Ps, Gate gate) {
  constexpr int W = TileGrid::W, H = TileGrid::H, WP = TileGrid::WP;
  __shared__ S suv[2 * H * W];
  __shared__ S sp[(MTJ + 1) * WP];
  __shared__ T fx[(MTJ + 1) * (MTI + 1)];  // -(C dx) at corner (j0 + r, i0 + q)
  __shared__ T fy[(MTJ + 1) * (MTI + 1)];  // -(C dy)
  __shared__ T xu[MTJ * (MTI + 1)];        // Xu at (j0 + r, i0 + q)
  __shared__ T yv[(MTJ + 1) * MTI];        // Yv at (j0 + r, i0 + q)
  if (!gate_open(gate)) return;
  const int nx = c.nx, ny = c.ny;
  const int j0 = blockIdx.y * MTJ, i0 = blockIdx.x * MTI;
  const int tid = threadIdx.y * MTI + threadIdx.x;
  const Grid g{nx, ny, c.usize};
  const TileGrid tg{nx, ny, j0, i0};
  // 1. the tiles (zero outside the grids; no stencil below reads those entries)
  for (int e = tid; e < H * W; e += MTI * MTJ) {
    const int r = e / W, q = e - r * W;
    const int j = j0 - 1 + r, i = i0 - 1 + q;
    suv[e] = (j >= 0 && j < ny && i >= 0 && i <= nx) ? Us[g.u(j, i)] : (S)0;
    suv[H * W + e] = (j >= 0 && j <= ny && i >= 0 && i < nx) ? Us[g.v(j, i)] : (S)0;
  }
  for (int e = tid; e < (MTJ + 1) * WP; e += MTI * MTJ) {
    const int r = e / WP, q = e - r * WP;
    const int j = j0 - 1 + r, i = i0 - 1 + q;
    sp[e] = (j >= 0 && j < ny && i >= 0 && i < nx) ? Ps[g.p(j, i)] : (S)0;
  }
  __syncthreads();
  constexpr bool F32 = sizeof(T) == 4;
  const T dx = F32 ? (T)c.fdx : (T)c.dx, dy = F32 ? (T)c.fdy : (T)c.dy;
  const T hh = (T)0.5;
  auto U = [&](int j, int i) -> T { return (T)suv[tg.u(j, i)]; };
  auto V = [&](int j, int i) -> T { return (T)suv[tg.v(j, i)]; };
  // 2. the shared fluxes
  for (int e = tid; e < (MTJ + 1) * (MTI + 1); e += MTI * MTJ) {
    const int r = e / (MTI + 1), q = e - r * (MTI + 1);
    const int jj = j0 + r, ii = i0 + q;
    T cx = (T)0, cy = (T)0;
    if (jj >= 1 && jj <= ny - 1 && ii >= 1 && ii <= nx) {
      const T vf = ii == nx ? V(jj, nx - 1) : hh * (V(jj, ii - 1) + V(jj, ii));
      const T ua = hh * (U(jj - 1, ii) + U(jj, ii));
      const T cc = vf * ua;
      cx = -(cc * dx);
      cy = -(cc * dy);
    }
    fx[e] = cx;
    fy[e] = cy;
  }
  for (int e = tid; e < MTJ * (MTI + 1); e += MTI * MTJ) {
    const int r = e / (MTI + 1), q = e - r * (MTI + 1);
    const int j = j0 + r, ii = i0 + q;
    T x = (T)0;
    if (j < ny && ii >= 1 && ii <= nx) {
      const T fl = hh * (U(j, ii - 1) + U(j, ii));
      x = -((fl * fl) * dy);
    }
    xu[e] = x;
  }
  for (int e = tid; e < (MTJ + 1) * MTI; e += MTI * MTJ) {
    const int r = e / MTI, q = e - r * MTI;
    const int jj = j0 + r, i = i0 + q;
    T y = (T)0;
    if (jj >= 1 && jj <= ny && i < nx) {
      const T fb = hh * (V(jj - 1, i) + V(jj, i));
      y = -((fb * fb) * dx);
    }
    yv[e] = y;
  }
  __syncthreads();
  const int r = threadIdx.y, q = threadIdx.x;
  const int j = j0 + r, i = i0 + q;
  const T idx2 = F32 ? (T)c.fidx2 : (T)c.idx2, idy2 = F32 ? (T)c.fidy2 : (T)c.idy2;
  const T iarea = F32 ? (T)c.fiarea : (T)c.iarea, nu = F32 ? (T)c.fnu : (T)c.nu;
  const T dt = F32 ? (T)a.dt32 : (T)a.dt;
  const T alpha = F32 ? (T)a.alpha32 : (T)a.alpha;
  auto FX = [&](int jj, int ii) -> T { return fx[(jj - j0) * (MTI + 1) + (ii - i0)]; };
  auto FY = [&](int jj, int ii) -> T { return fy[(jj - j0) * (MTI + 1) + (ii - i0)]; };
  auto XU = [&](int jj, int ii) -> T { return xu[(jj - j0) * (MTI + 1) + (ii - i0)]; };
  auto YV = [&](int jj, int ii) -> T { return yv[(jj - j0) * MTI + (ii - i0)]; };
  // 3. the faces of this point
  for (int comp = 0; comp < 2; ++comp) {
    if (comp == 0 ? (j >= ny || i > nx) : (j > ny || i >= nx)) continue;
    const int64_t t = comp == 0 ? g.u(j, i) : g.v(j, i);
    const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
    if (!(cls & CLS_ACTIVE)) {
      a.now[t] = 0.0;
      a.out[t] = 0.0;
      continue;
    }
    const double qv = a.U[t];
    T lq, gp, now, off = 0;
    if (comp == 0) {
      lq = nu * lap_u<T>(suv, tg, j, i, idx2, idy2, true);
      gp = grad_u<T>(sp, tg, j, i, F32 ? (T)c.fgx : (T)c.gx);
      T adv;
      if (i < nx) {
        adv = (XU(j, i + 1) - XU(j, i)) + (FX(j + 1, i) - FX(j, i));
      } else {
        const T uC = U(j, i);
        adv = (-uC * uC) * dy - XU(j, nx) + hh * (FX(j + 1, nx) - FX(j, nx));
      }
      now = adv * iarea;
      if (i == nx) now *= (T)2;
      if (i == 1) off = nu * (idx2 * (T)c.inlet[j]);
    } else {
      lq = nu * lap_v<T>(suv, tg, j, i, idx2, idy2);
      gp = grad_v<T>(sp, tg, j, i, F32 ? (T)c.fgy : (T)c.gy);
      now = ((FY(j, i + 1) - FY(j, i)) + (YV(j + 1, i) - YV(j, i))) * iarea;
    }
    const T expl = ((T)1 + alpha) * now - alpha * cvt_to<T>(a.prev[t]);
    a.now[t] = cvt_to<double>(now);
    if constexpr (sizeof(T) == 8)
      a.out[t] = (qv + (double)(dt * (expl + (T)0.5 * lq - gp))) + (double)(((T)0.5 * dt) * off);
    else
      a.out[t] = qv + cvt_to<double>(dt * (expl + (T)0.5 * lq - gp) + ((T)0.5 * dt) * off);
  }
}

// whether the AB2 right-hand side runs from shared-memory tiles (GHOSTMAC_MOMENTUM_TILED=0: the
// one-thread-per-face kernel; read at every launch, which graph replays do not repeat)
static bool momentum_tiled() {
  const char* e = std::getenv("GHOSTMAC_MOMENTUM_TILED");
  return !(e && e[0] == '0');
}
static dim3 momentum_tiles(const CaseDev& c) {
  return dim3((unsigned)((c.nx + 1 + MTI - 1) / MTI), (unsigned)((c.ny + 1 + MTJ - 1) / MTJ));
}

__global__ void k_shadow(const double* __restrict__ U, float* __restrict__ U32, int64_t nf,
                         const double* __restrict__ P, float* __restrict__ P32, int64_t np, Gate gate) {
  if (!gate_open(gate)) return;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf + np; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < nf) U32[t] = f64_to_f32i(U[t]);
    else P32[t - nf] = f64_to_f32i(P[t - nf]);
  }
}
void launch_shadow(const double* U, float* U32, int64_t n_f, const double* P, float* P32, int64_t n_p,
                   const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(3, st);
  launch_pdl(k_shadow, dim3(reduce_blocks(n_f + n_p)), dim3(TPB), 0, st, U, U32, n_f, P, P32, n_p, gate);
  kt_mark(3, st);
}

void launch_momentum(const CaseDev& c, const MomentumArgs& a, const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(3, st);
  if (a.mode == 0 && momentum_tiled())
    launch_pdl(k_momentum_tiled<double, double>, dim3(momentum_tiles(c)), dim3(dim3(MTI, MTJ)), 0, st, c, a, a.U, a.P, gate);
  else
    launch_pdl(k_momentum<double, double>, dim3(blocks_for(c.usize + c.vsize)), dim3(TPB), 0, st, c, a, a.U, a.P, gate);
  // algorithmic bytes: U, prev, class map read; now, out written; P read
  kt_mark(3, st, (double)(c.usize + c.vsize) * (8 * 4 + 1) + (double)c.psize * 8);
}
void launch_momentum_f32(const CaseDev& c, const MomentumArgs& a_in, const Gate& gate, cudaStream_t st) {
  MomentumArgs a = a_in;
  a.dt32 = (float)a.dt;
  a.alpha32 = (float)a.alpha;
  note_launch();
  kt_mark(3, st);
  if (a.mode == 0 && a.U32 && a.P32 && momentum_tiled())
    launch_pdl(k_momentum_tiled<float, float>, dim3(momentum_tiles(c)), dim3(dim3(MTI, MTJ)), 0, st, c, a, a.U32, a.P32, gate);
  else if (a.mode == 0 && a.U32 && a.P32)
    launch_pdl(k_momentum<float, float>, dim3(blocks_for(c.usize + c.vsize)), dim3(TPB), 0, st, c, a, a.U32, a.P32, gate);
  else
    launch_pdl(k_momentum<float, double>, dim3(blocks_for(c.usize + c.vsize)), dim3(TPB), 0, st, c, a, a.U, a.P, gate);
  kt_mark(3, st);
}

__global__ void k_advection(CaseDev c, const double* __restrict__ U, double* __restrict__ out, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) { out[t] = 0.0; return; }
  double r;
  if (comp == 0) {
    r = adv_u<double>(U, g, j, i, c.dx, c.dy) * c.iarea;
    if (i == c.nx) r *= 2;
  } else {
    r = adv_v<double>(U, g, j, i, c.dx, c.dy) * c.iarea;
  }
  out[t] = r;
}
void launch_advection(const CaseDev& c, const double* U, double* out, const Gate& gate, cudaStream_t st) {
  note_launch();
  k_advection<<<blocks_for(c.usize + c.vsize), TPB, 0, st>>>(c, U, out, gate);
}

__global__ void k_diffusion(CaseDev c, const double* __restrict__ U, double* __restrict__ out, int with_inlet,
                            double hdt, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) { out[t] = 0.0; return; }
  const double idx2 = c.idx2, idy2 = c.idy2;
  double l = comp == 0 ? c.nu * lap_u<double>(U, g, j, i, idx2, idy2, with_inlet != 0) : c.nu * lap_v<double>(U, g, j, i, idx2, idy2);
  out[t] = hdt == 0.0 ? l : U[t] - hdt * l;
}
void launch_diffusion(const CaseDev& c, const double* U, double* out, bool with_inlet, double hdt, const Gate& gate,
                      cudaStream_t st) {
  note_launch();
  k_diffusion<<<blocks_for(c.usize + c.vsize), TPB, 0, st>>>(c, U, out, with_inlet ? 1 : 0, hdt, gate);
}

__global__ void k_gradient(CaseDev c, const double* __restrict__ P, double* __restrict__ out, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) { out[t] = 0.0; return; }
  out[t] = comp == 0 ? grad_u<double>(P, g, j, i, c.gx) : grad_v<double>(P, g, j, i, c.gy);
}
void launch_gradient(const CaseDev& c, const double* P, double* out, const Gate& gate, cudaStream_t st) {
  note_launch();
  k_gradient<<<blocks_for(c.usize + c.vsize), TPB, 0, st>>>(c, P, out, gate);
}

// ---------------------------------------------------------------------------
// residual of the pressure operator A or the Helmholtz operators
// ---------------------------------------------------------------------------

// Residual res = b - A x of the pressure operator A (KIND 0, p grid) or the Helmholtz
// operators I - c L (KIND 1 u faces, KIND 2 v faces), with max |res| and sum res^2 per check.
// GB300 issues FP64 at 1/64 of the FP32 rate, so the regular rows use coefficients formed on
// the host (ResidualCoef): one add and four multiply-adds per point.  RES_F32: the residual
// is stored in FP32 (the input of the FP32 inverse).  Its max norm, which drives the
// refinement, is still taken from the FP64 residual; the diagnostic sums of res^2 and b^2 are
// FP32, so the only FP64 work left is the stencil.  The pressure gate's roundoff bound is formed
// in FP32 beside it.
// coefficient selection by value (indexing the parameter struct would copy it to local memory)
__device__ __forceinline__ double coef_cc(const ResidualCoef& rc, int ic, int jc) {
  const double c0 = jc ? rc.cc[0][1] : rc.cc[0][0];
  const double c1 = jc ? rc.cc[1][1] : rc.cc[1][0];
  const double c2 = jc ? rc.cc[2][1] : rc.cc[2][0];
  return ic == 0 ? c0 : (ic == 1 ? c1 : c2);
}
__device__ __forceinline__ double coef_cw(const ResidualCoef& rc, int ic) {
  return ic == 0 ? rc.cw[0] : (ic == 1 ? rc.cw[1] : rc.cw[2]);
}

template <int KIND, bool RES_F32>
__device__ __forceinline__ void residual_body(const CaseDev& c, const ResidualCoef& rc, const double* __restrict__ b,
                                              const double* __restrict__ x, void* __restrict__ res_out, SolveCtl* sc,
                                              int check, int first, int bid, int nblk) {
  if (check < 0) check = *(volatile int*)&sc->k;
  const int nx = c.nx, ny = c.ny;
  const int w = KIND == 1 ? nx + 1 : nx;            // row width of the grid
  const int64_t npts = KIND == 0 ? c.psize : (KIND == 1 ? c.usize : c.vsize);
  const int64_t base = KIND == 2 ? c.usize : 0;     // face-grid offset of the v field
  const uint8_t* cls = KIND == 0 ? c.cls_p : (KIND == 1 ? c.cls_u : c.cls_v);
  double* res64 = reinterpret_cast<double*>(res_out);
  float* res32 = reinterpret_cast<float*>(res_out);
  unsigned long long rm = 0, bm = 0, bd = 0, xb = 0;
  double rs = 0.0, bs = 0.0;
  float rs32 = 0.0f;  // RES_F32: sum of the stored FP32 residuals squared (diagnostics only)
  float bs32 = 0.0f;  // RES_F32: sum of the right-hand side squared in FP32 (diagnostics only)
  // RES_F32, pressure: the roundoff bound (2 nnz + 2) eps (|A| |x| + |b|) in FP32 and integer
  // arithmetic, beside the FP64 stencil (the FP64 pipe is this kernel's bound)
  constexpr bool BOUND32 = KIND == 0 && RES_F32;
  float bd32 = 0.0f;
  for (int64_t t = (int64_t)bid * blockDim.x + threadIdx.x; t < npts; t += (int64_t)nblk * blockDim.x) {
    const uint8_t k = cls[t];
    const int64_t f = base + t;
    if (!(k & CLS_ACTIVE)) {
      if (RES_F32) res32[f] = 0.0f; else res64[f] = 0.0;
      continue;
    }
    const double xv = x[f], bv = b[f];
    double r, aabs = 0.0;
    float aabs32 = 0.0f;
    int nnz = 0;
    const int row = (k & CLS_IRREG) ? c.irr_index[KIND][t] : -1;
    if (row >= 0) {
      const int64_t* cp = c.irr_ptr[KIND];
      double ax = 0.0;
      const int64_t e0 = cp[row], e1 = cp[row + 1];
      csr_row<4>(c.irr_col[KIND], c.irr_val[KIND], e0, e1, x, base, [&](double a, double xv2) {
        ax += a * xv2;
        if (KIND == 0 && !RES_F32) aabs += absd(a) * absd(xv2);
        if (BOUND32) aabs32 += fabsf(f64_to_f32i(a)) * fabsf(f64_to_f32i(xv2));
      });
      r = bv - ax;
      nnz = (int)(e1 - e0);
    } else {
      const int j = (int)((unsigned)t / (unsigned)w), i = (int)((unsigned)t - (unsigned)j * w);
      // neighbours outside the operator's stencil read as zero
      double xw = 0.0, xe = 0.0, xs = 0.0, xn = 0.0;
      int ic, jc;
      if (KIND == 0) {
        if (i > 0) xw = x[f - 1];
        if (i < nx - 1) xe = x[f + 1];
        if (j > 0) xs = x[f - w];
        if (j < ny - 1) xn = x[f + w];
        ic = i == 0 ? 0 : (i == nx - 1 ? 2 : 1);
        jc = (j == 0 || j == ny - 1) ? 0 : 1;
      } else if (KIND == 1) {
        if (i > 1) xw = x[f - 1];
        if (i < nx) xe = x[f + 1];
        if (j > 0) xs = x[f - w];
        if (j < ny - 1) xn = x[f + w];
        ic = i == nx ? 2 : 1;
        jc = (j == 0 || j == ny - 1) ? 0 : 1;
      } else {
        if (i > 0) xw = x[f - 1];
        if (i < nx - 1) xe = x[f + 1];
        if (j > 1) xs = x[f - w];
        if (j < ny - 1) xn = x[f + w];
        ic = i == 0 ? 0 : (i == nx - 1 ? 2 : 1);
        jc = 1;
      }
      // r = b - (cc x + cw xw + ce xe + cy (xs + xn)); Helmholtz rows carry the factors of
      // I - c L.  One add and four fused multiply-adds that subtract from b, written out so
      // that nothing else reaches the FP64 pipe; each rounding stays inside the
      // (2 nnz + 2) eps (|A| |x| + |b|) bound of the pressure gate.
      const double ccv = coef_cc(rc, ic, jc), cwv = coef_cw(rc, ic);
      r = fma(-rc.cy, xs + xn, fma(-rc.ce, xe, fma(-cwv, xw, fma(-ccv, xv, bv))));
      if (KIND == 0 && !RES_F32) {
        aabs = absd(ccv) * absd(xv) + rc.ce * (absd(xw) + absd(xe)) + rc.cy * (absd(xs) + absd(xn));
        nnz = c.a_nnz[t];
      }
      if (BOUND32) {
        const float c0 = jc ? rc.fcc[0][1] : rc.fcc[0][0], c1 = jc ? rc.fcc[1][1] : rc.fcc[1][0];
        const float c2 = jc ? rc.fcc[2][1] : rc.fcc[2][0];
        const float fcc = ic == 0 ? c0 : (ic == 1 ? c1 : c2);
        aabs32 = fabsf(fcc) * fabsf(f64_to_f32i(xv)) +
                 rc.fce * (fabsf(f64_to_f32i(xw)) + fabsf(f64_to_f32i(xe))) +
                 rc.fcy * (fabsf(f64_to_f32i(xs)) + fabsf(f64_to_f32i(xn)));
        nnz = c.a_nnz[t];
      }
    }
    rm = umax64(rm, absbits(r));
    if constexpr (RES_F32) {
      const float r32 = f64_to_f32i(r);
      res32[f] = r32;
      rs32 = fmaf(r32, r32, rs32);
    } else {
      res64[f] = r;
      rs += r * r;
    }
    if (KIND == 0 && !RES_F32) bd = umax64(bd, dbits((2.0 * nnz + 2.0) * EPS64 * (aabs + absd(bv))));
    if (BOUND32)
      bd32 = fmaxf(bd32, (2.0f * (float)nnz + 2.0f) * 2.220446049250313e-16f * (aabs32 + fabsf(f64_to_f32i(bv))));
    if (first) {
      bm = umax64(bm, absbits(bv));
      if constexpr (RES_F32) {
        const float b32 = f64_to_f32i(bv);
        bs32 = fmaf(b32, b32, bs32);
      } else {
        bs += bv * bv;
      }
    }
    if (nonfinite_bits(xv)) xb = 1;
  }
  block_commit_max(rm, &sc->rmax[check]);
  if constexpr (RES_F32) block_commit_sum_f32(rs32, &sc->rsq[check]);
  else block_commit_sum(rs, &sc->rsq[check]);
  if (KIND == 0 && !RES_F32) block_commit_max(bd, &sc->bound[check]);
  // the FP32 bound times 1 + 2^-20 (above its own rounding), as an FP64 value; non-negative
  // doubles order like their bits
  if (BOUND32) block_commit_max(dbits(f32_to_f64i(bd32 * 1.00000095367431640625f)), &sc->bound[check]);
  if (first) {
    block_commit_max(bm, &sc->bmax);
    if constexpr (RES_F32) block_commit_sum_f32(bs32, &sc->bsq);
    else block_commit_sum(bs, &sc->bsq);
  }
  block_commit_max(xb, &sc->xbad);
}
template <int KIND, bool RES_F32>
__global__ void k_residual(CaseDev c, ResidualCoef rc, const double* __restrict__ b, const double* __restrict__ x,
                           void* __restrict__ res_out, SolveCtl* sc, int check, int first, Gate gate) {
  if (!gate_open(gate)) return;
  residual_body<KIND, RES_F32>(c, rc, b, x, res_out, sc, check, first, blockIdx.x, gridDim.x);
}

void launch_residual(const CaseDev& c, const ResidualCoef& rc, int kind, const double* b, const double* x, void* res,
                     bool res_f32, SolveCtl* sc, int check, bool first_check, const Gate& gate, cudaStream_t st) {
  const int64_t n = kind == 0 ? c.psize : (kind == 1 ? c.usize : c.vsize);
  const unsigned g = residual_blocks(n, res_f32);
  const int fc = first_check ? 1 : 0;
  note_launch();
  kt_mark(4, st);
  if (res_f32) {
    if (kind == 0) launch_pdl(k_residual<0, true>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
    else if (kind == 1) launch_pdl(k_residual<1, true>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
    else launch_pdl(k_residual<2, true>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
  } else {
    if (kind == 0) launch_pdl(k_residual<0, false>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
    else if (kind == 1) launch_pdl(k_residual<1, false>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
    else launch_pdl(k_residual<2, false>, dim3(g), dim3(TPB), 0, st, c, rc, b, x, res, sc, check, fc, gate);
  }
  kt_mark(4, st, (double)n * (8 + 8 + (res_f32 ? 4 : 8) + 1));  // x, b, res, class map
}

// ---------------------------------------------------------------------------
// FP32 Jacobi sweeps of the CN Helmholtz systems (FP32 mode)
// ---------------------------------------------------------------------------
// The CN systems H = I - c L (c = dt nu / 2) are strongly diagonally dominant: the Jacobi
// iteration matrix has row-sum norm rho = max_i sum_{j != i} |H_ij| / |H_ii|, about 4 c / h^2
// (0.016 on the 800x820 Re 100 case), which the host computes from every row at set-up.  In
// the FP32 mode one application of the approximate inverse is then `iters` Jacobi
// iterations d <- D^{-1} (r - (H - D) d) from d = 0, in FP32, with the same regular-row
// coefficients and irregular rows as the residual kernel; x = [x +] d closes the last one.
// The FP64 residual and the refinement loop around it are those of the FFT inverse, so the
// answer meets the same residual targets; only the number of sweeps may differ.
static constexpr int JPT = 4;  // consecutive points per thread in the Jacobi iterations
template <int KIND, typename TR>
__global__ void __launch_bounds__(TPB) k_helm_jacobi(CaseDev c, ResidualCoef rc, HelmJacobi hj,
                                                    const TR* __restrict__ r, const float* __restrict__ din,
                                                    float* __restrict__ dout, double* __restrict__ x, int accumulate,
                                                    Gate gate) {
  if (!gate_open(gate)) return;
  const int nx = c.nx, ny = c.ny;
  const int w = KIND == 1 ? nx + 1 : nx;
  const int64_t npts = KIND == 1 ? c.usize : c.vsize;
  const int64_t base = KIND == 2 ? c.usize : 0;
  const uint8_t* cls = KIND == 1 ? c.cls_u : c.cls_v;
  const int64_t t0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * JPT;
  if (t0 >= npts) return;
  // every load of the thread's JPT points first (one round trip), then the arithmetic
  uint8_t k[JPT];
  float rv[JPT], dw[JPT], de[JPT], ds[JPT], dn[JPT];
#pragma unroll
  for (int u = 0; u < JPT; ++u) {
    const int64_t t = t0 + u;
    k[u] = 0;
    rv[u] = dw[u] = de[u] = ds[u] = dn[u] = 0.0f;
    if (t >= npts) continue;
    const int64_t f = base + t;
    k[u] = cls[t];
    if constexpr (sizeof(TR) == 8) rv[u] = f64_to_f32i(r[f]);
    else rv[u] = r[f];
    if (din) {
      const int j = (int)((unsigned)t / (unsigned)w), i = (int)((unsigned)t - (unsigned)j * w);
      if (KIND == 1) {
        if (i > 1) dw[u] = din[f - 1];
        if (i < nx) de[u] = din[f + 1];
        if (j > 0) ds[u] = din[f - w];
        if (j < ny - 1) dn[u] = din[f + w];
      } else {
        if (i > 0) dw[u] = din[f - 1];
        if (i < nx - 1) de[u] = din[f + 1];
        if (j > 1) ds[u] = din[f - w];
        if (j < ny - 1) dn[u] = din[f + w];
      }
    }
  }
#pragma unroll
  for (int u = 0; u < JPT; ++u) {
    const int64_t t = t0 + u;
    if (t >= npts) continue;
    const int64_t f = base + t;
    float d = 0.0f;
    if (k[u] & CLS_ACTIVE) {
      const int row = (k[u] & CLS_IRREG) ? c.irr_index[KIND][t] : -1;
      if (row >= 0) {
        float sum = 0.0f;
        if (din) {
          const int64_t* cp = c.irr_ptr[KIND];
          const int64_t* col = c.irr_col[KIND];
          const float* val = hj.val[KIND - 1];
          for (int64_t e = cp[row]; e < cp[row + 1]; ++e) sum = fmaf(val[e], din[base + col[e]], sum);
        }
        d = (rv[u] - sum) * hj.idiag[KIND - 1][row];
      } else {
        const int j = (int)((unsigned)t / (unsigned)w), i = (int)((unsigned)t - (unsigned)j * w);
        int ic, jc;
        if (KIND == 1) {
          ic = i == nx ? 2 : 1;
          jc = (j == 0 || j == ny - 1) ? 0 : 1;
        } else {
          ic = i == 0 ? 0 : (i == nx - 1 ? 2 : 1);
          jc = 1;
        }
        const float cwv = ic == 0 ? rc.fcw[0] : (ic == 1 ? rc.fcw[1] : rc.fcw[2]);
        const float i0 = jc ? hj.icc[KIND - 1][0][1] : hj.icc[KIND - 1][0][0];
        const float i1 = jc ? hj.icc[KIND - 1][1][1] : hj.icc[KIND - 1][1][0];
        const float i2 = jc ? hj.icc[KIND - 1][2][1] : hj.icc[KIND - 1][2][0];
        const float icc = ic == 0 ? i0 : (ic == 1 ? i1 : i2);
        const float off = fmaf(rc.fcy, ds[u] + dn[u], fmaf(rc.fce, de[u], cwv * dw[u]));
        d = (rv[u] - off) * icc;
      }
    }
    if (x) {
      // inactive points of the solution are zero
      x[f] = !(k[u] & CLS_ACTIVE) ? 0.0 : (accumulate ? x[f] + f32_to_f64i(d) : f32_to_f64i(d));
    } else {
      dout[f] = d;
    }
  }
}

template <typename TR>
void launch_helm_jacobi(const CaseDev& c, const ResidualCoef& rc, const HelmJacobi& hj, int kind, const TR* r,
                        const float* din, float* dout, double* x, bool accumulate, const Gate& gate, cudaStream_t st) {
  const int64_t n = kind == 1 ? c.usize : c.vsize;
  note_launch();
  kt_mark(11, st);
  const unsigned g = blocks_for((n + JPT - 1) / JPT);
  if (kind == 1)
    launch_pdl(k_helm_jacobi<1, TR>, dim3(g), dim3(TPB), 0, st, c, rc, hj, r, din, dout, x, accumulate ? 1 : 0, gate);
  else
    launch_pdl(k_helm_jacobi<2, TR>, dim3(g), dim3(TPB), 0, st, c, rc, hj, r, din, dout, x, accumulate ? 1 : 0, gate);
  // algorithmic bytes: r, the class map, the five-point iterate (read once per point) and the
  // new iterate (or x read and written by the last iteration)
  kt_mark(11, st, (double)n * (sizeof(TR) + 1 + (din ? 4 : 0) + (x ? (accumulate ? 16 : 8) : 4)));
}
template void launch_helm_jacobi<double>(const CaseDev&, const ResidualCoef&, const HelmJacobi&, int, const double*,
                                         const float*, float*, double*, bool, const Gate&, cudaStream_t);
template void launch_helm_jacobi<float>(const CaseDev&, const ResidualCoef&, const HelmJacobi&, int, const float*,
                                        const float*, float*, double*, bool, const Gate&, cudaStream_t);

// Temporally blocked Jacobi application: every block loads the class map and the right-hand
// side of its region once, runs the iterations in shared memory and writes its output box.
// A point's value after `iters` iterations depends only on points that iters - 1 stencil
// applications reach from it, so a tile with a halo of iters - 1 five-point steps reproduces
// the global iteration exactly outside the body box (whose margin keeps every irregular row
// iters - 1 points away), and the body block's region holds everything its box reaches.
// Points of a regular tile's halo may be irregular rows updated with the five-point formula:
// their values never reach the tile's outputs.
// Shared memory of a region of rh x rw points, stored with a border of one zero point on each
// side (every neighbour read is then in bounds and a missing neighbour reads zero): four float
// arrays (two iterates, the right-hand side and each point's multiplier: 1 / diagonal, or 0 on
// an inactive point) and the west coefficient of each column.
__host__ __device__ inline size_t jacobi_region_bytes(int rh, int rw) {
  const size_t n = (size_t)(rh + 2) * (rw + 2);
  return (n * 4 + (size_t)(rw + 2) + 3) / 4 * 4 * sizeof(float);
}
size_t helm_jacobi_tiled_smem(const JacobiTiles& t, int iters) {
  const int h = iters - 1;
  const size_t reg = jacobi_region_bytes(t.th + 2 * h, t.tw + 2 * h);
  size_t body = 0;
  if (t.bj1 > t.bj0)
    body = jacobi_region_bytes(t.rj1 - t.rj0, t.ri1 - t.ri0) + (size_t)t.nnz * 8 + (size_t)t.nrow * 12 + 4;
  return (std::max(reg, body) + 15) / 16 * 16;
}

// Block 0 is the body block (it starts first); the others are the regular tiles.  Threads walk
// the region in rows of 32 points per warp, so no per-point index division is needed.  The
// operator's excluded neighbours (the u inlet column, the v wall rows) are inactive points whose
// iterate is zero, and points outside the grid are the zero border, so the five-point update
// needs no neighbour tests.
// threads of a tile block: every tile's work is latency bound (few warps per SM at this grid
// size), so a tile takes more warps than the other kernels' blocks
constexpr int JTPB = 512;
template <int KIND, typename TR>
__global__ void __launch_bounds__(JTPB) k_helm_jacobi_tiled(CaseDev c, ResidualCoef rc, HelmJacobi hj,
                                                          const TR* __restrict__ r, double* __restrict__ x,
                                                          int accumulate, Gate gate) {
  extern __shared__ __align__(16) float jsm[];
  if (!gate_open(gate)) return;
  const JacobiTiles& T = hj.jt[KIND - 1];
  const int nx = c.nx, ny = c.ny;
  const int W = KIND == 1 ? nx + 1 : nx;
  const int R = KIND == 1 ? ny : ny + 1;
  const int64_t base = KIND == 2 ? c.usize : 0;
  const uint8_t* cls = KIND == 1 ? c.cls_u : c.cls_v;
  const int h = hj.iters - 1;
  const bool has_body = T.bj1 > T.bj0;
  const bool body = has_body && blockIdx.x == 0;
  int j0, j1, i0, i1, oj0, oj1, oi0, oi1;
  if (body) {
    j0 = T.rj0; j1 = T.rj1; i0 = T.ri0; i1 = T.ri1;
    oj0 = T.bj0; oj1 = T.bj1; oi0 = T.bi0; oi1 = T.bi1;
  } else {
    const int b = (int)blockIdx.x - (has_body ? 1 : 0);
    const int ty = b / T.ntx, tx = b - ty * T.ntx;
    oj0 = ty * T.th; oj1 = min(oj0 + T.th, R);
    oi0 = tx * T.tw; oi1 = min(oi0 + T.tw, W);
    j0 = max(oj0 - h, 0); j1 = min(oj1 + h, R);
    i0 = max(oi0 - h, 0); i1 = min(oi1 + h, W);
  }
  const int rw = i1 - i0, rh = j1 - j0, pw = rw + 2, np = pw * (rh + 2);
  float* cur = jsm;
  float* nxt = jsm + np;
  float* rr = jsm + 2 * np;
  float* mm = jsm + 3 * np;   // 1 / diagonal of the point's regular row, 0 on inactive points
  float* colw = jsm + 4 * np; // west coefficient of each region column
  unsigned char* stage = reinterpret_cast<unsigned char*>(jsm) + jacobi_region_bytes(rh, rw);
  float* sval = reinterpret_cast<float*>(stage);
  int32_t* ssidx = reinterpret_cast<int32_t*>(sval + (body ? T.nnz : 0));
  int32_t* sptr = ssidx + (body ? T.nnz : 0);
  int32_t* spos = sptr + (body ? T.nrow + 1 : 0);
  float* sidg = reinterpret_cast<float*>(spos + (body ? T.nrow : 0));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  // zero borders of both iterates; the right-hand side and the multiplier of every point, and
  // the west coefficient of every column, formed once for all the iterations
  for (int q = threadIdx.x; q < np; q += blockDim.x) { cur[q] = 0.0f; nxt[q] = 0.0f; }
  for (int pi = threadIdx.x; pi < rw; pi += blockDim.x) {
    const int ii = i0 + pi;
    const int icl = KIND == 1 ? (ii == nx ? 2 : 1) : (ii == 0 ? 0 : (ii == nx - 1 ? 2 : 1));
    colw[pi] = icl == 0 ? rc.fcw[0] : (icl == 1 ? rc.fcw[1] : rc.fcw[2]);
  }
  for (int pj = warp; pj < rh; pj += nwarp) {
    const int jj = j0 + pj;
    const int jc = KIND == 1 ? ((jj == 0 || jj == ny - 1) ? 0 : 1) : 1;
    const float ia = hj.icc[KIND - 1][0][jc], ib = hj.icc[KIND - 1][1][jc], ic2 = hj.icc[KIND - 1][2][jc];
    const int64_t row = (int64_t)jj * W + i0;
    for (int pi = lane; pi < rw; pi += 32) {
      const int q = (pj + 1) * pw + pi + 1;
      const int ii = i0 + pi;
      const int icl = KIND == 1 ? (ii == nx ? 2 : 1) : (ii == 0 ? 0 : (ii == nx - 1 ? 2 : 1));
      const bool act = (cls[row + pi] & CLS_ACTIVE) != 0;
      mm[q] = act ? (icl == 0 ? ia : (icl == 1 ? ib : ic2)) : 0.0f;
      float rv;
      if constexpr (sizeof(TR) == 8) rv = f64_to_f32i(r[base + row + pi]);
      else rv = r[base + row + pi];
      rr[q] = act ? rv : 0.0f;
    }
  }
  if (body) {
    const int64_t* cp = c.irr_ptr[KIND];
    for (int e = threadIdx.x; e < T.nnz; e += blockDim.x) {
      sval[e] = hj.val[KIND - 1][e];
      const int sx = T.sidx[e];  // place in the unpadded region
      ssidx[e] = sx < 0 ? -1 : (sx / rw + 1) * pw + (sx - (sx / rw) * rw) + 1;
    }
    for (int q = threadIdx.x; q <= T.nrow; q += blockDim.x) {
      sptr[q] = (int32_t)cp[q];
      if (q < T.nrow) {
        const int sx = T.rpos[q];
        spos[q] = (sx / rw + 1) * pw + (sx - (sx / rw) * rw) + 1;
        sidg[q] = hj.idiag[KIND - 1][q];
      }
    }
  }
  __syncthreads();
  // the regular rows: d = (r - (cw d_w + ce d_e + cy (d_s + d_n))) / diagonal, zero on inactive
  // points (the arithmetic of the untiled kernel, in the same order)
  const float fce = rc.fce, fcy = rc.fcy;
  for (int it = 0; it < hj.iters; ++it) {
    for (int pj = warp; pj < rh; pj += nwarp) {
      const int q0 = (pj + 1) * pw + 1;
      for (int pi = lane; pi < rw; pi += 32) {
        const int q = q0 + pi;
        const float m = mm[q];
        const float off = it > 0 ? fmaf(fcy, cur[q - pw] + cur[q + pw], fmaf(fce, cur[q + 1], colw[pi] * cur[q - 1]))
                                 : 0.0f;
        nxt[q] = m != 0.0f ? (rr[q] - off) * m : 0.0f;
      }
    }
    if (body) {
      // the irregular rows overwrite their places with the rows' own entries
      __syncthreads();
      for (int q = threadIdx.x; q < T.nrow; q += blockDim.x) {
        const int p = spos[q];
        float sum = 0.0f;
        if (it > 0)
          for (int e = sptr[q]; e < sptr[q + 1]; ++e) {
            const int sx = ssidx[e];
            if (sx >= 0) sum = fmaf(sval[e], cur[sx], sum);
          }
        nxt[p] = (rr[p] - sum) * sidg[q];
      }
    }
    __syncthreads();
    float* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  const int bj0 = T.bj0, bj1 = T.bj1, bi0 = T.bi0, bi1 = T.bi1;
  for (int pj = warp; pj < rh; pj += nwarp) {
    const int jj = j0 + pj;
    if (jj < oj0 || jj >= oj1) continue;
    const bool in_box_rows = has_body && jj >= bj0 && jj < bj1;
    const int64_t row = base + (int64_t)jj * W;
    for (int pi = lane; pi < rw; pi += 32) {
      const int ii = i0 + pi;
      if (ii < oi0 || ii >= oi1) continue;
      if (!body && in_box_rows && ii >= bi0 && ii < bi1) continue;
      const int q = (pj + 1) * pw + pi + 1;
      const int64_t f = row + ii;
      const float d = cur[q];
      x[f] = mm[q] == 0.0f ? 0.0 : (accumulate ? x[f] + f32_to_f64i(d) : f32_to_f64i(d));
    }
  }
}

// The kernels' dynamic shared-memory limit is a per-function, process-wide attribute shared by
// every case: it is raised to the device's opt-in maximum (never set to one case's size, which
// would make the launches of a larger case in the same process fail).
int helm_jacobi_tiled_optin(size_t smem) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  if (smem > (size_t)optin) return 1;
  const void* ks[4] = {(const void*)k_helm_jacobi_tiled<1, double>, (const void*)k_helm_jacobi_tiled<2, double>,
                       (const void*)k_helm_jacobi_tiled<1, float>, (const void*)k_helm_jacobi_tiled<2, float>};
  int e = 0;
  for (const void* k : ks) {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k) != cudaSuccess) { e = 1; continue; }
    const int dyn = optin - (int)a.sharedSizeBytes;
    if (smem > (size_t)dyn || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
      e = 1;
  }
  if (e) cudaGetLastError();
  return e;
}

template <typename TR>
void launch_helm_jacobi_tiled(const CaseDev& c, const ResidualCoef& rc, const HelmJacobi& hj, int kind, const TR* r,
                              double* x, bool accumulate, size_t smem, const Gate& gate, cudaStream_t st) {
  const JacobiTiles& T = hj.jt[kind - 1];
  const unsigned g = (unsigned)(T.ntx * T.nty + (T.bj1 > T.bj0 ? 1 : 0));
  const int64_t n = kind == 1 ? c.usize : c.vsize;
  note_launch();
  kt_mark(11, st);
  if (kind == 1)
    launch_pdl(k_helm_jacobi_tiled<1, TR>, dim3(g), dim3(JTPB), smem, st, c, rc, hj, r, x, accumulate ? 1 : 0, gate);
  else
    launch_pdl(k_helm_jacobi_tiled<2, TR>, dim3(g), dim3(JTPB), smem, st, c, rc, hj, r, x, accumulate ? 1 : 0, gate);
  // algorithmic bytes: r and the class map read, x written (read too when accumulating)
  kt_mark(11, st, (double)n * (sizeof(TR) + 1 + (accumulate ? 16 : 8)));
}
template void launch_helm_jacobi_tiled<double>(const CaseDev&, const ResidualCoef&, const HelmJacobi&, int,
                                               const double*, double*, bool, size_t, const Gate&, cudaStream_t);
template void launch_helm_jacobi_tiled<float>(const CaseDev&, const ResidualCoef&, const HelmJacobi&, int,
                                              const float*, double*, bool, size_t, const Gate&, cudaStream_t);


// ---------------------------------------------------------------------------
// flexible GMRES on the pressure grid (solver/pressure_schur.py:20-57, iterative branch):
// operator apply, block-deterministic multi-dot products and multi-axpy updates
// ---------------------------------------------------------------------------
// w = A z on the pressure grid (zero at inactive cells)
__global__ void k_apply_pressure(CaseDev c, ResidualCoef rc, const double* __restrict__ z, double* __restrict__ w,
                                 Gate gate) {
  if (!gate_open(gate)) return;
  const int nx = c.nx, ny = c.ny;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.psize; t += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t k = c.cls_p[t];
    if (!(k & CLS_ACTIVE)) {
      w[t] = 0.0;
      continue;
    }
    double ax;
    const int row = (k & CLS_IRREG) ? c.irr_index[0][t] : -1;
    if (row >= 0) {
      const int64_t* cp = c.irr_ptr[0];
      ax = 0.0;
      csr_row<4>(c.irr_col[0], c.irr_val[0], cp[row], cp[row + 1], z, 0, [&](double a, double zv) { ax += a * zv; });
    } else {
      const int j = (int)((unsigned)t / (unsigned)nx), i = (int)((unsigned)t - (unsigned)j * nx);
      const double xw = i > 0 ? z[t - 1] : 0.0, xe = i < nx - 1 ? z[t + 1] : 0.0;
      const double xs = j > 0 ? z[t - nx] : 0.0, xn = j < ny - 1 ? z[t + nx] : 0.0;
      const int ic = i == 0 ? 0 : (i == nx - 1 ? 2 : 1), jc = (j == 0 || j == ny - 1) ? 0 : 1;
      ax = coef_cc(rc, ic, jc) * z[t] + coef_cw(rc, ic) * xw + rc.ce * xe + rc.cy * (xs + xn);
    }
    w[t] = ax;
  }
}
void launch_apply_pressure(const CaseDev& c, const ResidualCoef& rc, const double* z, double* w, const Gate& gate,
                           cudaStream_t st) {
  note_launch();
  kt_mark(4, st);
  k_apply_pressure<<<reduce_blocks(c.psize), TPB, 0, st>>>(c, rc, z, w, gate);
  kt_mark(4, st, (double)c.psize * 17);
}

// Partial sums part[b * nv + i] = sum over block b's points of V_i[t] * w[t], i < nv (V_i at
// V + i * ld); the final pass sums the blocks in a fixed order (run-to-run identical).
static constexpr int GM_DOT_MAX = 64;
__global__ void k_multidot_part(const double* __restrict__ V, int64_t ld, int nv, const double* __restrict__ w,
                                int64_t n, double* __restrict__ part) {
  __shared__ double red[GM_DOT_MAX][TPB / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i0 = 0; i0 < nv; i0 += 8) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
      const double wt = w[t];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i0 + u < nv) acc[u] += V[(int64_t)(i0 + u) * ld + t] * wt;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const double sum = warp_sum(acc[u]);
      if (lane == 0 && i0 + u < nv) red[i0 + u][warp] = sum;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double sum = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum += red[i][q];
    part[(int64_t)blockIdx.x * nv + i] = sum;
  }
}
__global__ void k_multidot_final(const double* __restrict__ part, int nblocks, int nv, double* __restrict__ out) {
  const int i = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += 32) acc += part[(int64_t)b * nv + i];
  acc = warp_sum(acc);
  if (threadIdx.x == 0) out[i] = acc;
}
void launch_multidot(const double* V, int64_t ld, int nv, const double* w, int64_t n, double* part, double* out,
                     cudaStream_t st) {
  const unsigned nb = reduce_blocks(n);
  note_launch();
  kt_mark(6, st);
  k_multidot_part<<<nb, TPB, 0, st>>>(V, ld, nv, w, n, part);
  kt_mark(6, st, (double)n * 8 * (nv + 1));
  note_launch();
  k_multidot_final<<<nv, 32, 0, st>>>(part, (int)nb, nv, out);
}
unsigned multidot_blocks(int64_t n) { return reduce_blocks(n); }

// y[t] = alpha * y[t] + sign * sum_i coef[i] V_i[t]   (coef on the device)
__global__ void k_multiaxpy(const double* __restrict__ V, int64_t ld, int nv, const double* __restrict__ coef,
                            double sign, double alpha, double* __restrict__ y, int64_t n) {
  __shared__ double cf[GM_DOT_MAX + 1];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) cf[i] = coef[i];
  __syncthreads();
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < nv; ++i) acc += cf[i] * V[(int64_t)i * ld + t];
    y[t] = alpha * y[t] + sign * acc;
  }
}
void launch_multiaxpy(const double* V, int64_t ld, int nv, const double* coef, double sign, double alpha, double* y,
                      int64_t n, cudaStream_t st) {
  note_launch();
  kt_mark(6, st);
  k_multiaxpy<<<reduce_blocks(n), TPB, 0, st>>>(V, ld, nv, coef, sign, alpha, y, n);
  kt_mark(6, st, (double)n * 8 * (nv + 2));
}

// Learned preconditioner input / output on the pressure grid: x = [v / s, mask] (float32,
// 2 planes), s = max |v| over the active cells (computed by the first kernel into *s_bits);
// z += s y on the active cells.
__global__ void k_learned_max(CaseDev c, const double* __restrict__ v, unsigned long long* s_bits) {
  unsigned long long m = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.psize; t += (int64_t)gridDim.x * blockDim.x)
    if (c.cls_p[t] & CLS_ACTIVE) m = umax64(m, absbits(v[t]));
  block_commit_max(m, s_bits);
}
__global__ void k_learned_in(CaseDev c, const double* __restrict__ v, const unsigned long long* __restrict__ s_bits,
                             float* __restrict__ x) {
  const double s = bits2d(*s_bits);
  const double inv = s > 0 ? 1.0 / s : 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.psize; t += (int64_t)gridDim.x * blockDim.x) {
    const bool act = c.cls_p[t] & CLS_ACTIVE;
    x[t] = act ? (float)(v[t] * inv) : 0.f;
    x[c.psize + t] = act ? 1.f : 0.f;
  }
}
__global__ void k_learned_out(CaseDev c, const float* __restrict__ y, const unsigned long long* __restrict__ s_bits,
                              double* __restrict__ z) {
  const double s = bits2d(*s_bits);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.psize; t += (int64_t)gridDim.x * blockDim.x)
    if (c.cls_p[t] & CLS_ACTIVE) z[t] += s * (double)y[t];
}
void launch_learned_prep(const CaseDev& c, const double* v, float* x, unsigned long long* s_bits, cudaStream_t st) {
  note_launch();
  k_learned_max<<<reduce_blocks(c.psize), TPB, 0, st>>>(c, v, s_bits);
  note_launch();
  k_learned_in<<<reduce_blocks(c.psize), TPB, 0, st>>>(c, v, s_bits, x);
}
void launch_learned_apply(const CaseDev& c, const float* y, const unsigned long long* s_bits, double* z,
                          cudaStream_t st) {
  note_launch();
  k_learned_out<<<reduce_blocks(c.psize), TPB, 0, st>>>(c, y, s_bits, z);
}

// ---------------------------------------------------------------------------
// projection pieces
// ---------------------------------------------------------------------------
// D U at the active cells: its max |.| into divmax and/or, scaled, into out.  The scaled
// output takes its coefficients sx = idx s, sy = idy s from the host (s = 1/dt or 1), so it
// costs no more FP64 work than the divergence itself.
__global__ void k_divergence(CaseDev c, const double* __restrict__ U, double* __restrict__ out, double sx, double sy,
                             unsigned long long* divmax, int gate_nonfinite, StepCtl* ctl, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  unsigned long long dm = 0;
  bool bad = false;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.psize; t += (int64_t)gridDim.x * blockDim.x) {
    if (c.cls_p[t] & CLS_ACTIVE) {
      int j = (int)((unsigned)t / (unsigned)c.nx), i = (int)((unsigned)t - (unsigned)j * c.nx);
      const double du = U[g.u(j, i + 1)] - U[g.u(j, i)], dv = U[g.v(j + 1, i)] - U[g.v(j, i)];
      if (divmax) dm = umax64(dm, absbits(du * c.idx + dv * c.idy));
      if (out) {
        const double o = du * sx + dv * sy;
        out[t] = o;
        bad = bad || nonfinite_bits(o);
      }
    } else if (out) {
      out[t] = 0.0;
    }
  }
  if (gate_nonfinite && bad && ctl) raise_gate(ctl, 1, 4);
  if (divmax) block_commit_max(dm, divmax);
}
void launch_divergence(const CaseDev& c, const double* U, double* out, double scale, SolveCtl* sc,
                       unsigned long long* divmax, int gate_on_nonfinite, const Gate& gate, cudaStream_t st) {
  (void)sc;
  note_launch();
  kt_mark(6, st);
  const double s = scale != 0.0 ? 1.0 / scale : 1.0;
  launch_pdl(k_divergence, dim3(reduce_blocks(c.psize)), dim3(TPB), 0, st, c, U, out, c.idx * s, c.idy * s, divmax, gate_on_nonfinite,
                                                      gate.ctl, gate);
  kt_mark(6, st);
}

// out = q - dt G phi at the active faces, with dgx = dt gx and dgy = dt gy formed on the host:
// two fused multiply-adds per face (G phi is gx (phi_e - phi_w), at the outlet -2 gx phi_w)
__global__ void k_project_update(CaseDev c, const double* __restrict__ q, const double* __restrict__ phi, double dgx,
                                 double dgy, double* __restrict__ out, Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) {
    out[t] = (comp == 0 && i == 0) ? c.inlet[j] : 0.0;
    return;
  }
  if (comp == 1) out[t] = fma(dgy, phi[g.p(j - 1, i)], fma(-dgy, phi[g.p(j, i)], q[t]));
  else if (i < c.nx) out[t] = fma(dgx, phi[g.p(j, i - 1)], fma(-dgx, phi[g.p(j, i)], q[t]));
  else out[t] = fma(2.0 * dgx, phi[g.p(j, c.nx - 1)], q[t]);
}
void launch_project_update(const CaseDev& c, const double* q, const double* phi, double dt, double* out,
                           const SolveCtl* psolve, const Gate& gate, cudaStream_t st) {
  (void)psolve;
  note_launch();
  kt_mark(6, st);
  launch_pdl(k_project_update, dim3(blocks_for(c.usize + c.vsize)), dim3(TPB), 0, st, c, q, phi, dt * c.gx, dt * c.gy, out, gate);
  kt_mark(6, st);
}

// H r at an active u (KIND 1) or v (KIND 2) face t (index within its face grid) for the
// Helmholtz operator H = I - c L of the CN solves: the same rows as residual_body's, i.e. the
// host-formed coefficients on regular rows (one add, one multiply, three fused multiply-adds)
// and the folded sparse rows next to the body.
template <int KIND>
__device__ __forceinline__ double helm_action(const CaseDev& c, const ResidualCoef& rc, const double* __restrict__ x,
                                              int64_t t, uint8_t k) {
  const int nx = c.nx, ny = c.ny;
  const int w = KIND == 1 ? nx + 1 : nx;
  const int64_t base = KIND == 2 ? c.usize : 0;
  const int64_t f = base + t;
  const int row = (k & CLS_IRREG) ? c.irr_index[KIND][t] : -1;
  if (row >= 0) {
    const int64_t* cp = c.irr_ptr[KIND];
    double ax = 0.0;
    csr_row<4>(c.irr_col[KIND], c.irr_val[KIND], cp[row], cp[row + 1], x, base,
               [&](double a, double xv2) { ax += a * xv2; });
    return ax;
  }
  const int j = (int)((unsigned)t / (unsigned)w), i = (int)((unsigned)t - (unsigned)j * w);
  double xw = 0.0, xe = 0.0, xs = 0.0, xn = 0.0;
  int ic, jc;
  if (KIND == 1) {
    if (i > 1) xw = x[f - 1];
    if (i < nx) xe = x[f + 1];
    if (j > 0) xs = x[f - w];
    if (j < ny - 1) xn = x[f + w];
    ic = i == nx ? 2 : 1;
    jc = (j == 0 || j == ny - 1) ? 0 : 1;
  } else {
    if (i > 0) xw = x[f - 1];
    if (i < nx - 1) xe = x[f + 1];
    if (j > 1) xs = x[f - w];
    if (j < ny - 1) xn = x[f + w];
    ic = i == 0 ? 0 : (i == nx - 1 ? 2 : 1);
    jc = 1;
  }
  const double ccv = coef_cc(rc, ic, jc), cwv = coef_cw(rc, ic);
  return fma(rc.cy, xs + xn, fma(rc.ce, xe, fma(cwv, xw, ccv * x[f])));
}

// Defect correction of the CN velocity (solver/time_integration.py): action = H r and
// proj = r + (rhs - H r) at the active faces; inlet values and zeros elsewhere.
__global__ void k_defect(CaseDev c, ResidualCoef rcu, ResidualCoef rcv, const double* __restrict__ r,
                         const double* __restrict__ rhs, double* __restrict__ action, double* __restrict__ proj,
                         Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int comp, j, i;
  if (!face_of(t, g, comp, j, i)) return;
  const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
  if (!(cls & CLS_ACTIVE)) {
    action[t] = 0.0;
    proj[t] = (comp == 0 && i == 0) ? c.inlet[j] : 0.0;
    return;
  }
  const double hr = comp == 0 ? helm_action<1>(c, rcu, r, t, cls) : helm_action<2>(c, rcv, r, t - c.usize, cls);
  action[t] = hr;
  proj[t] = r[t] + (rhs[t] - hr);
}
void launch_defect(const CaseDev& c, const ResidualCoef& rcu, const ResidualCoef& rcv, const double* result,
                   const double* rhs, double* action, double* proj, const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(7, st);
  launch_pdl(k_defect, dim3(blocks_for(c.usize + c.vsize)), dim3(TPB), 0, st, c, rcu, rcv, result, rhs, action, proj, gate);
  kt_mark(7, st);
}

__global__ void k_pressure_out(CaseDev c, const double* __restrict__ p, const double* __restrict__ inc, double factor,
                               double dgx, double dgy, const double* __restrict__ action, const double* __restrict__ rhs,
                               double* __restrict__ half, double* __restrict__ pout, unsigned long long* coupled,
                               Gate gate) {
  if (!gate_open(gate)) return;
  const Grid g{c.nx, c.ny, c.usize};
  int64_t nf = c.usize + c.vsize;
  unsigned long long cm = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf + c.psize;
       t += (int64_t)gridDim.x * blockDim.x) {
  if (t < nf) {
    int comp, j, i;
    face_of(t, g, comp, j, i);
    const uint8_t cls = comp == 0 ? c.cls_u[t] : c.cls_v[t - c.usize];
    if (cls & CLS_ACTIVE) {
      // action - rhs + dt G inc, with dgx = dt gx and dgy = dt gy formed on the host
      const double a0 = action[t] - rhs[t];
      double r;
      if (comp == 1) r = fma(-dgy, inc[g.p(j - 1, i)], fma(dgy, inc[g.p(j, i)], a0));
      else if (i < c.nx) r = fma(-dgx, inc[g.p(j, i - 1)], fma(dgx, inc[g.p(j, i)], a0));
      else r = fma(-2.0 * dgx, inc[g.p(j, c.nx - 1)], a0);
      cm = umax64(cm, absbits(r));
    }
  } else {
    int64_t k = t - nf;
    if (c.cls_p[k] & CLS_ACTIVE) {
      double h = p[k] + inc[k];
      half[k] = h;
      pout[k] = h + factor * inc[k];
    } else {
      half[k] = 0.0;
      pout[k] = 0.0;
    }
  }
  }
  block_commit_max(cm, coupled);
}
void launch_pressure_out(const CaseDev& c, const double* p, const double* inc, double factor, double dt,
                         const double* action, const double* rhs, double* half, double* pout,
                         unsigned long long* coupled, const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(7, st);
  launch_pdl(k_pressure_out, dim3(reduce_blocks(c.usize + c.vsize + c.psize)), dim3(TPB), 0, st, c, p, inc, factor, dt * c.gx, dt * c.gy,
                                                                          action, rhs, half, pout, coupled, gate);
  kt_mark(7, st);
}

__global__ void k_maxabs(CaseDev c, const double* __restrict__ U, unsigned long long* umax, unsigned long long* vmax,
                         Gate gate) {
  if (!gate_open(gate)) return;
  unsigned long long a = 0, b = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c.usize + c.vsize;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < c.usize) a = umax64(a, absbits(U[t]));
    else b = umax64(b, absbits(U[t]));
  }
  block_commit_max(a, umax);
  block_commit_max(b, vmax);
}
void launch_maxabs(const CaseDev& c, const double* U, unsigned long long* umax, unsigned long long* vmax,
                   const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(9, st);
  launch_pdl(k_maxabs, dim3(reduce_blocks(c.usize + c.vsize)), dim3(TPB), 0, st, c, U, umax, vmax, gate);
  kt_mark(9, st);
}

// ---------------------------------------------------------------------------
// surface forces (solver/optimized_ghost_cell.py:280-286) and step gates (solver/main.py:401-415)
// ---------------------------------------------------------------------------
__global__ void k_forces(CaseDev c, const double* __restrict__ U, const double* __restrict__ P, double mu, double dt,
                         StepCtl* ctl, int check_gates, double* out6, Gate gate) {
  if (!gate_open(gate)) return;
  // one warp per quadrature point (lanes over the stencil nonzeros), the per-point terms go to
  // c.surf_part; the last block to finish sums them in a fixed order (deterministic)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int k = blockIdx.x * wpb + warp;
  if (k < c.n_surf) {
    double ps = 0, du = 0, dv = 0;
    for (int64_t e = c.sp_ptr[k] + lane; e < c.sp_ptr[k + 1]; e += 32) ps += c.sp_val[e] * P[c.sp_col[e]];
    for (int64_t e = c.su_ptr[k] + lane; e < c.su_ptr[k + 1]; e += 32) du += c.su_val[e] * U[c.su_col[e]];
    for (int64_t e = c.sv_ptr[k] + lane; e < c.sv_ptr[k + 1]; e += 32) dv += c.sv_val[e] * U[c.usize + c.sv_col[e]];
    ps = warp_sum(ps);
    du = warp_sum(du);
    dv = warp_sum(dv);
    if (lane == 0) {
      const double nxk = c.nxx[k], nyk = c.nyy[k];
      const double dn = du * nxk + dv * nyk;
      double* o = c.surf_part + 4 * (int64_t)k;
      o[0] = ps * c.nwx[k];
      o[1] = ps * c.nwy[k];
      o[2] = mu * (du + nxk * dn);
      o[3] = mu * (dv + nyk * dn);
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ int last;
  if (threadIdx.x == 0) last = atomicAdd(c.surf_ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[4];
  if (warp < 4) {
    double acc = 0.0;
    for (int q = lane; q < c.n_surf; q += 32) acc += __ldcg(c.surf_part + 4 * (int64_t)q + warp);
    acc = warp_sum(acc);
    if (lane == 0) red[warp] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *c.surf_ticket = 0u;
    const double PI = 3.141592653589793;
    double w = PI * c.D / c.n_surf;
    double fp[2] = {-red[0], -red[1]};
    double fv[2] = {red[2] * w, red[3] * w};
    double f6[6] = {fp[0] + fv[0], fp[1] + fv[1], fp[0], fp[1], fv[0], fv[1]};
    if (out6)
      for (int q = 0; q < 6; ++q) out6[q] = f6[q];
    if (ctl) {
      for (int q = 0; q < 6; ++q) ctl->forces[q] = f6[q];
      double denom = ((0.5 * c.rho) * (c.U_ref * c.U_ref)) * c.D;
      double cd = f6[0] / denom, cl = f6[1] / denom;
      ctl->cd = cd;
      ctl->cl = cl;
      if (check_gates) {
        if (!isfinite(cd) || !isfinite(cl)) {
          raise_gate(ctl, 3, 6);
        } else {
          double div = bits2d(ctl->div_max[1]);
          double cfl = dt * (bits2d(ctl->umax) / c.dx + bits2d(ctl->vmax) / c.dy);
          if (!(div < 1e-10) || !(cfl < 0.5)) raise_gate(ctl, 2, 5);
        }
      }
    }
  }
}
void launch_forces(const CaseDev& c, const double* U, const double* P, double mu, double dt, StepCtl* ctl,
                   int check_gates, double* out6, const Gate& gate, cudaStream_t st) {
  note_launch();
  kt_mark(9, st);
  const int wpb = 8;
  launch_pdl(k_forces, dim3((c.n_surf + wpb - 1) / wpb), dim3(32 * wpb), 0, st, c, U, P, mu, dt, ctl, check_gates, out6, gate);
  kt_mark(9, st);
}

__global__ void k_gate_momentum(StepCtl* ctl, int nchk) {
  if (ctl->err) return;
  double r = 0, bm = 0;
  bool bad = false;
  for (int s = 0; s < 2; ++s) {
    const SolveCtl* sc = &ctl->solve[s];
    double rr = bits2d(sc->rmax[last_check(sc, nchk)]);
    double bb = bits2d(sc->bmax);
    if (!(rr <= r)) r = rr;  // propagates NaN
    if (bb > bm) bm = bb;
    if (sc->xbad) bad = true;
  }
  double thr = 1e-10 * (bm > 1.0 ? bm : 1.0);
  if (bad || !(r <= thr)) raise_gate(ctl, 2, 2);
}
void launch_gate_momentum(StepCtl* ctl, int nchk, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_gate_momentum<<<1, 1, 0, st>>>(ctl, nchk);
  kt_mark(10, st);
}

__global__ void k_gate_pressure(StepCtl* ctl, int slot, int nchk) {
  if (ctl->err) return;
  const SolveCtl* sc = &ctl->solve[slot];
  int k = last_check(sc, nchk);
  double linf = bits2d(sc->rmax[k]), bound = bits2d(sc->bound[k]), bm = bits2d(sc->bmax);
  if (!isfinite(bm)) { raise_gate(ctl, 1, 4); return; }  // solver/pressure_schur.py:33-34
  double t = 64 * EPS64 * (bm > 1.0 ? bm : 1.0);
  t = t > 1e-10 ? t : 1e-10;
  t = bound > t ? bound : t;
  if (sc->xbad || !(linf <= t)) raise_gate(ctl, 2, 3);
}
void launch_gate_pressure(StepCtl* ctl, int slot, int nchk, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_gate_pressure<<<1, 1, 0, st>>>(ctl, slot, nchk);
  kt_mark(10, st);
}

__global__ void k_gate_projection(StepCtl* ctl, int k) {
  if (ctl->err) return;
  double d = bits2d(ctl->div_max[k]);
  if (!(d <= 1e-10)) raise_gate(ctl, 2, 1);
}
void launch_gate_projection(StepCtl* ctl, int k, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_gate_projection<<<1, 1, 0, st>>>(ctl, k);
  kt_mark(10, st);
}

// CFL screen of solver/main.py:273-278 (screen != 0) and the finite-field check of
// solver/time_integration.py:15-17 on the velocity maxima of the current state.
__global__ void k_cfl_screen(StepCtl* ctl, const unsigned long long* umax, const unsigned long long* vmax, double dt,
                             double dx, double dy, int screen, const long long* counter) {
  if (ctl->err) return;
  if (screen < 0) screen = (*counter % 100) == 0;
  double rate = bits2d(*umax) / dx + bits2d(*vmax) / dy;
  if (screen && (!isfinite(rate) || dt * rate > 0.5)) raise_gate(ctl, 2, 7);
  else if (!isfinite(rate)) raise_gate(ctl, 1, 8);
}
void launch_cfl_screen(StepCtl* ctl, const unsigned long long* umax, const unsigned long long* vmax, double dt,
                       double dx, double dy, int screen, const long long* counter, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_cfl_screen<<<1, 1, 0, st>>>(ctl, umax, vmax, dt, dx, dy, screen, counter);
  kt_mark(10, st);
}

// ---------------------------------------------------------------------------
// Flexible GMRES(50) with its control on the device (solver/pressure_schur.py:20-41): the
// Hessenberg column, the Givens rotations, the residual estimate, the convergence test and
// the least-squares update run in one-thread kernels on the device-resident GmresDev, and the
// loops are conditional graph nodes (restart cycles: WHILE; Arnoldi steps: one IF node per
// step, its condition set by the previous step).  The arithmetic is that of the host loop it
// replaces, in the same order.
// ---------------------------------------------------------------------------
__global__ void k_gm_init(GmresDev* gd, const double* __restrict__ bn2, cudaGraphConditionalHandle cycle,
                          double rtol, double atol) {
  gd->tol = fmax(rtol * sqrt(bn2[0]), atol);
  gd->iterations = 0;
  gd->converged = 0;
  gd->stop = 0;
  gd->cycle = 0;
  gd->jend = -1;
  cudaGraphSetConditional(cycle, 1u);
}
// beta = ||b - A x||; the cycle's first step runs while beta > tol
__global__ void k_gm_cycle_begin(GmresDev* gd, const double* __restrict__ beta2, GmresHandles hs) {
  const double beta = sqrt(beta2[0]);
  gd->jend = -1;
  bool go = beta > gd->tol;
  if (!go) {
    gd->converged = isfinite(beta) ? 1 : 0;
    gd->stop = 1;
    gd->hscale = 1.0;
  } else {
    for (int i = 0; i <= GmresDev::M; ++i) gd->g[i] = 0.0;
    gd->g[0] = beta;
    gd->hscale = 1.0 / beta;
  }
  for (int j = 0; j < hs.count; ++j) cudaGraphSetConditional(hs.step[j], (j == 0 && go) ? 1u : 0u);
}
// w *= hscale (the new basis vector, or V_0 at the start of a cycle)
__global__ void k_gm_scale(double* __restrict__ w, int64_t n, const GmresDev* __restrict__ gd) {
  const double s = gd->hscale;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    w[t] *= s;
}
// end of Arnoldi step j: column j of H from the two Gram-Schmidt passes and the norm, the
// rotations, the residual estimate g[j+1]; step j + 1 runs while it is finite and above tol
__global__ void k_gm_step_end(GmresDev* gd, int j, const double* __restrict__ d1, const double* __restrict__ d2,
                              const double* __restrict__ wn2, cudaGraphConditionalHandle next, int has_next) {
  double hc[GmresDev::M + 1];
  for (int i = 0; i <= j; ++i) hc[i] = d1[i] + d2[i];
  hc[j + 1] = sqrt(wn2[0]);
  gd->hscale = hc[j + 1] > 0 ? 1.0 / hc[j + 1] : 1.0;
  for (int i = 0; i < j; ++i) {
    const double a = gd->cs[i] * hc[i] + gd->sn[i] * hc[i + 1];
    hc[i + 1] = -gd->sn[i] * hc[i] + gd->cs[i] * hc[i + 1];
    hc[i] = a;
  }
  const double den = hypot(hc[j], hc[j + 1]);
  gd->cs[j] = den > 0 ? hc[j] / den : 1.0;
  gd->sn[j] = den > 0 ? hc[j + 1] / den : 0.0;
  hc[j] = den;
  gd->g[j + 1] = -gd->sn[j] * gd->g[j];
  gd->g[j] = gd->cs[j] * gd->g[j];
  for (int i = 0; i <= j; ++i) gd->H[i * GmresDev::M + j] = hc[i];
  gd->iterations += 1;
  gd->jend = j;
  const double r = gd->g[j + 1];
  bool go = true;
  if (!isfinite(r)) go = false;
  else if (fabs(r) <= gd->tol) { gd->converged = 1; go = false; }
  if (has_next) cudaGraphSetConditional(next, go ? 1u : 0u);
}
// end of a cycle: y = R^{-1} g (the solve of the host loop), nv = its length for x += Z y; the
// next cycle runs while not converged, a step was taken and fewer than 100 cycles ran
__global__ void k_gm_cycle_end(GmresDev* gd, double* __restrict__ y, int* __restrict__ nv,
                               cudaGraphConditionalHandle cycle) {
  const int jend = gd->jend;
  for (int i = jend; i >= 0; --i) {
    double acc = gd->g[i];
    for (int k = i + 1; k <= jend; ++k) acc -= gd->H[i * GmresDev::M + k] * gd->y[k];
    gd->y[i] = acc / gd->H[i * GmresDev::M + i];
  }
  for (int i = 0; i <= jend; ++i) y[i] = gd->y[i];
  *nv = jend + 1;
  gd->cycle += 1;
  const bool go = jend >= 0 && !gd->converged && !gd->stop && gd->cycle < 100;
  cudaGraphSetConditional(cycle, go ? 1u : 0u);
}
// y += sum_{i < *nv} coef[i] V_i (the count on the device)
__global__ void k_multiaxpy_dev(const double* __restrict__ V, int64_t ld, const int* __restrict__ nvp,
                                const double* __restrict__ coef, double* __restrict__ y, int64_t n) {
  __shared__ double cf[GM_DOT_MAX + 1];
  const int nv = *nvp;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) cf[i] = coef[i];
  __syncthreads();
  if (nv <= 0) return;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < nv; ++i) acc += cf[i] * V[(int64_t)i * ld + t];
    y[t] = 1.0 * y[t] + 1.0 * acc;
  }
}
void launch_gm_init(GmresDev* gd, const double* bn2, cudaGraphConditionalHandle cycle, cudaStream_t st, double rtol,
                    double atol) {
  note_launch();
  k_gm_init<<<1, 1, 0, st>>>(gd, bn2, cycle, rtol, atol);
}
void launch_gm_cycle_begin(GmresDev* gd, const double* beta2, const GmresHandles& hs, cudaStream_t st) {
  note_launch();
  k_gm_cycle_begin<<<1, 1, 0, st>>>(gd, beta2, hs);
}
void launch_gm_scale(double* w, int64_t n, const GmresDev* gd, cudaStream_t st) {
  note_launch();
  k_gm_scale<<<reduce_blocks(n), TPB, 0, st>>>(w, n, gd);
}
void launch_gm_step_end(GmresDev* gd, int j, const double* d1, const double* d2, const double* wn2,
                        cudaGraphConditionalHandle next, bool has_next, cudaStream_t st) {
  note_launch();
  k_gm_step_end<<<1, 1, 0, st>>>(gd, j, d1, d2, wn2, next, has_next ? 1 : 0);
}
void launch_gm_cycle_end(GmresDev* gd, double* y, int* nv, cudaGraphConditionalHandle cycle, cudaStream_t st) {
  note_launch();
  k_gm_cycle_end<<<1, 1, 0, st>>>(gd, y, nv, cycle);
}
void launch_multiaxpy_dev(const double* V, int64_t ld, const int* nv, const double* coef, double* y, int64_t n,
                          cudaStream_t st) {
  note_launch();
  k_multiaxpy_dev<<<reduce_blocks(n), TPB, 0, st>>>(V, ld, nv, coef, y, n);
}

__global__ void k_refine_decide(StepCtl* ctl, int slot, int nchk, cudaGraphConditionalHandle cond) {
  SolveCtl* sc = &ctl->solve[slot];
  int k = sc->k;
  bool need = false;
  if (!ctl->err) need = bits2d(sc->rmax[k]) > inner_target(sc) && k + 1 < nchk;
  if (need) sc->k = k + 1;
  cudaGraphSetConditional(cond, need ? 1u : 0u);
}
void launch_refine_decide(StepCtl* ctl, int slot, int nchk, cudaGraphConditionalHandle cond, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_refine_decide<<<1, 1, 0, st>>>(ctl, slot, nchk, cond);
  kt_mark(10, st);
}

__global__ void k_step_end(StepCtl* ctl, unsigned long long* state_max, StepCtl* ring, int* ridx, long long* counter,
                           int cap) {
  __shared__ int slot;
  if (threadIdx.x == 0) {
    slot = min(*ridx, cap - 1);
    if (!ctl->err) {
      state_max[0] = ctl->umax;
      state_max[1] = ctl->vmax;
    }
  }
  __syncthreads();
  const int* src = reinterpret_cast<const int*>(ctl);
  int* dst = reinterpret_cast<int*>(ring + slot);
  for (int i = threadIdx.x; i < (int)(sizeof(StepCtl) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    *ridx = slot + 1;
    *counter = *counter + 1;
  }
}
void launch_step_end(StepCtl* ctl, unsigned long long* state_max, StepCtl* ring, int* ridx, long long* counter,
                     int cap, cudaStream_t st) {
  note_launch();
  kt_mark(10, st);
  k_step_end<<<1, 128, 0, st>>>(ctl, state_max, ring, ridx, counter, cap);
  kt_mark(10, st);
}

__global__ void k_copy_active(const uint8_t* __restrict__ cls, int64_t n, const double* __restrict__ src,
                              double* __restrict__ dst, Gate gate) {
  if (!gate_open(gate)) return;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = (cls[t] & CLS_ACTIVE) ? src[t] : 0.0;
}
void launch_copy_active(const uint8_t* cls, int64_t n, const double* src, double* dst, const Gate& gate,
                        cudaStream_t st) {
  note_launch();
  launch_pdl(k_copy_active, dim3(blocks_for(n)), dim3(TPB), 0, st, cls, n, src, dst, gate);
}

__global__ void k_set_inlet(CaseDev c, double* U, int zero) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < c.ny) U[(int64_t)j * (c.nx + 1)] = zero ? 0.0 : c.inlet[j];
}
void launch_set_inlet(const CaseDev& c, double* U, bool zero, cudaStream_t st) {
  note_launch();
  kt_mark(6, st);
  k_set_inlet<<<blocks_for(c.ny, 128), 128, 0, st>>>(c, U, zero ? 1 : 0);
  kt_mark(6, st);
}

// mac_engine.calculate_mac_divergence_cpp (solver/src/bindings.cpp:343-390)
__global__ void k_div_stats(CaseDev c, const double* __restrict__ U, const uint8_t* __restrict__ mask, double* out5) {
  const Grid g{c.nx, c.ny, c.usize};
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m = 0;
  double s = 0, cs = 0, n = 0, cn = 0;
  if (t < c.psize && !mask[t]) {
    int j = (int)(t / c.nx), i = (int)(t % c.nx);
    double d = (U[g.u(j, i + 1)] - U[g.u(j, i)]) / c.dx + (U[g.v(j + 1, i)] - U[g.v(j, i)]) / c.dy;
    m = absbits(d);
    s = d * d;
    n = 1;
    bool core = true;
    if (i > 0 && mask[t - 1]) core = false;
    if (i < c.nx - 1 && mask[t + 1]) core = false;
    if (j > 0 && mask[t - c.nx]) core = false;
    if (j < c.ny - 1 && mask[t + c.nx]) core = false;
    if (core) { cs = d * d; cn = 1; }
  }
  block_commit_max(m, reinterpret_cast<unsigned long long*>(&out5[0]));
  block_commit_sum(s, &out5[1]);
  block_commit_sum(n, &out5[2]);
  block_commit_sum(cs, &out5[3]);
  block_commit_sum(cn, &out5[4]);
}
void launch_divergence_stats(const CaseDev& c, const double* U, const uint8_t* mask, double* out5, cudaStream_t st) {
  note_launch();
  k_div_stats<<<blocks_for(c.psize), TPB, 0, st>>>(c, U, mask, out5);
}

__global__ void k_gather(const double* __restrict__ src, const int64_t* __restrict__ idx, int64_t n,
                         double* __restrict__ dst) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = src[idx[t]];
}
__global__ void k_scatter(const double* __restrict__ src, const int64_t* __restrict__ idx, int64_t n,
                          double* __restrict__ dst) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[idx[t]] = src[t];
}
void launch_gather(const double* src, const int64_t* idx, int64_t n, double* dst, cudaStream_t st) {
  if (n > 0) {
    note_launch();
    k_gather<<<blocks_for(n), TPB, 0, st>>>(src, idx, n, dst);
  }
}
void launch_scatter(const double* src, const int64_t* idx, int64_t n, double* dst, cudaStream_t st) {
  if (n > 0) {
    note_launch();
    k_scatter<<<blocks_for(n), TPB, 0, st>>>(src, idx, n, dst);
  }
}

__global__ void k_schur_column(const double* __restrict__ first, RectView v, int rank, const int64_t* __restrict__ cp,
                               const int64_t* __restrict__ cc, const double* __restrict__ cv, double* __restrict__ S,
                               int col) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rank) return;
  double acc = 0.0;
  for (int64_t e = cp[r]; e < cp[r + 1]; ++e) acc += cv[e] * first[cc[e]];  // cc: field-grid flat indices
  S[(int64_t)r * rank + col] = acc;
}
void launch_schur_column(const double* first, const RectView& view, int rank, const int64_t* c_ptr,
                         const int64_t* c_col, const double* c_val, double* S, int col, cudaStream_t st) {
  if (rank > 0) {
    note_launch();
    k_schur_column<<<blocks_for(rank, 128), 128, 0, st>>>(first, view, rank, c_ptr, c_col, c_val, S, col);
  }
}

// ---------------------------------------------------------------------------
// case-indexed launches: blockIdx.y selects the case, its arguments come from the kernel's
// parameter space; blocks past the case's own grid return at once
// ---------------------------------------------------------------------------
template <typename T, typename TI, typename TO>
__global__ void k_xpass_multi(const __grid_constant__ ArgPack<XpassArgs<T, TI, TO>> p) {
  const XpassArgs<T, TI, TO>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.nblk) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const R2RTables<T> ts = xpass_stage_tables<T>(a.type, a.n, a.plan, a.tb, smem_raw);
  if (!gate_open(a.gate)) return;
  xpass_block<T, TI, TO>(blockIdx.x, a.n, a.r0, a.nr, a.type, a.plan, ts, a.in, a.ibase, a.ipitch, a.icls, a.out,
                         a.obase, a.opitch, a.ocls, a.add, a.corr, a.gthreads, a.gpb, smem_raw);
}
template <typename T, int L>
__global__ void k_ysolve_multi(const __grid_constant__ ArgPack<YsolveArgs<T>> p) {
  const YsolveArgs<T>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.nblk) return;
  if (!gate_open(a.gate)) return;
  ysolve_body<T, L>(a.rows, a.cols, a.ch, a.gamma, a.scale, a.t0, a.t1, a.t2, a.S, blockIdx.x);
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_first_multi(const __grid_constant__ ArgPack<BandFirstArgs<T>> p) {
  const BandFirstArgs<T>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.m) return;
  if (!gate_open(a.gate)) return;
  band_first_body<T>(a.n, a.mrow, a.binv, a.spec, a.firstm, blockIdx.x);
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_gemv_multi(const __grid_constant__ ArgPack<BandGemvArgs<T>> p) {
  const BandGemvArgs<T>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.rank) return;
  if (!gate_open(a.gate)) return;
  band_gemv_body<T>(a.m, a.M, a.firstm, a.c, blockIdx.x);
}
template <typename T>
__global__ void __launch_bounds__(BAND_TPB) k_band_direct_multi(const __grid_constant__ ArgPack<BandDirectArgs<T>> p) {
  const BandDirectArgs<T>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.rank * BAND_SPLIT) return;
  if (!gate_open(a.gate)) return;
  band_direct_body<T>(a.L, a.G, a.S, a.part, blockIdx.x / BAND_SPLIT, blockIdx.x % BAND_SPLIT);
}
template <typename T>
__global__ void __launch_bounds__(BAND_COLS * BAND_ROWT) k_band_fwd_solve_multi(
    const __grid_constant__ ArgPack<BandFwdArgs<T>> p) {
  const BandFwdArgs<T>& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.nblk) return;
  if (!gate_open(a.gate)) return;
  band_fwd_solve_body<T>(a.nb, a.n, a.rank, a.bptr, a.c, a.bfwd, a.gamma, a.scale, a.bpiv, a.band,
                         blockIdx.x, a.nsplit);
}
template <int KIND, bool RES_F32>
__global__ void k_residual_multi(const __grid_constant__ ArgPack<ResidualArgs> p) {
  const ResidualArgs& a = p.a[blockIdx.y];
  if ((int)blockIdx.x >= a.nblk) return;
  if (!gate_open(a.gate)) return;
  residual_body<KIND, RES_F32>(a.c, a.rc, a.b, a.x, a.res, a.sc, a.check, a.first, blockIdx.x, a.nblk);
}
__global__ void k_refine_decide_multi(const __grid_constant__ ArgPack<StepCtl*> ctls, int n, int slot, int nchk,
                                      cudaGraphConditionalHandle cond) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    StepCtl* ctl = ctls.a[c];
    SolveCtl* sc = &ctl->solve[slot];
    const int k = sc->k;
    bool need = false;
    if (!ctl->err) need = bits2d(sc->rmax[k]) > inner_target(sc) && k + 1 < nchk;
    if (need) {
      sc->k = k + 1;
      atomicOr(&any, 1);
    }
    sc->act = need ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) cudaGraphSetConditional(cond, any ? 1u : 0u);
}

template <typename T, typename TI, typename TO>
XpassArgs<T, TI, TO> xpass_args(const TransformTables& tt, bool inverse, int r0, int nr, const TI* in, int64_t ibase,
                                int64_t ipitch, const uint8_t* icls, TO* out, int64_t obase, int64_t opitch,
                                const uint8_t* ocls, const double* add, const YCorr<T>& corr, const Gate& gate) {
  using Cx = cplx<T>;
  XpassArgs<T, TI, TO> a{};
  a.n = tt.n;
  a.r0 = r0;
  a.nr = nr;
  a.type = inverse ? tt.tx_inv : tt.tx_fwd;
  a.plan = tt.plan_x;
  a.tb = R2RTables<T>{(const Cx*)tt.Wx, (const Cx*)(inverse ? tt.prex_inv : tt.prex),
                      (const Cx*)(inverse ? tt.postx_inv : tt.postx)};
  a.in = in;
  a.ibase = ibase;
  a.ipitch = ipitch;
  a.icls = icls;
  a.out = out;
  a.obase = obase;
  a.opitch = opitch;
  a.ocls = ocls;
  a.add = add;
  a.corr = corr;
  a.gthreads = tt.xg_threads;
  a.gpb = tt.xg_pb;
  a.gate = gate;
  const int per_block = tt.xg_pb * (r2r_paired(a.type) ? 2 : 1);
  a.nblk = (nr + per_block - 1) / per_block;
  return a;
}
template <typename T>
YsolveArgs<T> ysolve_args(const TransformTables& tt, int cols, int rows, T* S, const Gate& gate) {
  YsolveArgs<T> a{};
  a.rows = rows;
  a.cols = cols;
  a.ch = tt.ych;
  a.gamma = (T)tt.gamma;
  a.scale = (T)tt.yscale;
  a.t0 = (const T*)tt.t0;
  a.t1 = (const T*)tt.t1;
  a.t2 = (const T*)tt.t2;
  a.S = S;
  a.gate = gate;
  a.nblk = (cols + tt.lpb_y - 1) / tt.lpb_y;
  return a;
}
ResidualArgs residual_args(const CaseDev& c, const ResidualCoef& rc, int kind, const double* b, const double* x,
                           void* res, bool res_f32, SolveCtl* sc, int check, bool first_check, const Gate& gate) {
  ResidualArgs a{};
  a.c = c;
  a.rc = rc;
  a.b = b;
  a.x = x;
  a.res = res;
  a.sc = sc;
  a.check = check;
  a.first = first_check ? 1 : 0;
  a.gate = gate;
  a.nblk = (int)residual_blocks(kind == 0 ? c.psize : (kind == 1 ? c.usize : c.vsize), res_f32);
  return a;
}

static_assert(sizeof(ArgPack<ResidualArgs>) <= 32000 &&
                  sizeof(ArgPack<YsolveArgs<double>>) <= 32000 &&
                  sizeof(ArgPack<XpassArgs<double, double, double>>) <= 32000,
              "case-indexed argument packs must fit the kernel parameter space");
template <typename A>
static unsigned max_blocks(const ArgPack<A>& p, int n) {
  int m = 0;
  for (int c = 0; c < n; ++c) m = std::max(m, p.a[c].nblk);
  return (unsigned)std::max(m, 1);
}
template <typename T, typename TI, typename TO>
void launch_xpass_multi(const ArgPack<XpassArgs<T, TI, TO>>& p, int n, const TransformTables& tt0, cudaStream_t st) {
  if (n <= 0) return;
  note_launch();
  k_xpass_multi<T, TI, TO><<<dim3(max_blocks(p, n), (unsigned)n), tt0.xg_threads * tt0.xg_pb, tt0.smem_x, st>>>(p);
}
template <typename T>
void launch_ysolve_multi(const ArgPack<YsolveArgs<T>>& p, int n, const TransformTables& tt0, cudaStream_t st) {
  if (n <= 0) return;
  note_launch();
  const dim3 g(max_blocks(p, n), (unsigned)n);
  switch (tt0.lpb_y) {
    case 2: k_ysolve_multi<T, 2><<<g, tt0.threads_y, tt0.smem_y, st>>>(p); break;
    case 4: k_ysolve_multi<T, 4><<<g, tt0.threads_y, tt0.smem_y, st>>>(p); break;
    case 8: k_ysolve_multi<T, 8><<<g, tt0.threads_y, tt0.smem_y, st>>>(p); break;
    default: k_ysolve_multi<T, 16><<<g, tt0.threads_y, tt0.smem_y, st>>>(p); break;
  }
}
template <typename T>
void launch_band_first_multi(const ArgPack<BandFirstArgs<T>>& p, int n, cudaStream_t st) {
  if (n <= 0) return;
  int m = 1;
  for (int c = 0; c < n; ++c) m = std::max(m, p.a[c].m);
  note_launch();
  k_band_first_multi<T><<<dim3((unsigned)m, (unsigned)n), BAND_TPB, 0, st>>>(p);
}
template <typename T>
void launch_band_gemv_multi(const ArgPack<BandGemvArgs<T>>& p, int n, cudaStream_t st) {
  if (n <= 0) return;
  int r = 1;
  for (int c = 0; c < n; ++c) r = std::max(r, p.a[c].rank);
  note_launch();
  k_band_gemv_multi<T><<<dim3((unsigned)r, (unsigned)n), BAND_TPB, 0, st>>>(p);
}
template <typename T>
void launch_band_direct_multi(const ArgPack<BandDirectArgs<T>>& p, int n, cudaStream_t st) {
  if (n <= 0) return;
  int r = 1;
  for (int c = 0; c < n; ++c) r = std::max(r, p.a[c].rank);
  note_launch();
  k_band_direct_multi<T><<<dim3((unsigned)(r * BAND_SPLIT), (unsigned)n), BAND_TPB, 0, st>>>(p);
}
template <typename T>
void launch_band_fwd_solve_multi(const ArgPack<BandFwdArgs<T>>& p, int n, cudaStream_t st) {
  if (n <= 0) return;
  size_t smem = 0;
  for (int c = 0; c < n; ++c) smem = std::max(smem, band_fwd_smem(p.a[c].nb, p.a[c].rank, sizeof(T) == 4));
  note_launch();
  k_band_fwd_solve_multi<T><<<dim3(max_blocks(p, n), (unsigned)n), BAND_COLS * BAND_ROWT, smem, st>>>(p);
}
void launch_residual_multi(const ArgPack<ResidualArgs>& p, int n, int kind, bool res_f32, cudaStream_t st) {
  if (n <= 0) return;
  note_launch();
  const dim3 g(max_blocks(p, n), (unsigned)n);
  if (res_f32) {
    if (kind == 0) k_residual_multi<0, true><<<g, TPB, 0, st>>>(p);
    else if (kind == 1) k_residual_multi<1, true><<<g, TPB, 0, st>>>(p);
    else k_residual_multi<2, true><<<g, TPB, 0, st>>>(p);
  } else {
    if (kind == 0) k_residual_multi<0, false><<<g, TPB, 0, st>>>(p);
    else if (kind == 1) k_residual_multi<1, false><<<g, TPB, 0, st>>>(p);
    else k_residual_multi<2, false><<<g, TPB, 0, st>>>(p);
  }
}
void launch_refine_decide_multi(const ArgPack<StepCtl*>& ctls, int n, int slot, int nchk,
                                cudaGraphConditionalHandle cond, cudaStream_t st) {
  note_launch();
  k_refine_decide_multi<<<1, 32, 0, st>>>(ctls, n, slot, nchk, cond);
}

#define GM_XPASS_MULTI(T, TI, TO)                                                                                   \
  template XpassArgs<T, TI, TO> xpass_args<T, TI, TO>(const TransformTables&, bool, int, int, const TI*, int64_t, \
                                                      int64_t, const uint8_t*, TO*, int64_t, int64_t,             \
                                                      const uint8_t*, const double*, const YCorr<T>&, const Gate&); \
  template void launch_xpass_multi<T, TI, TO>(const ArgPack<XpassArgs<T, TI, TO>>&, int, const TransformTables&,   \
                                              cudaStream_t);
GM_XPASS_MULTI(double, double, double)
GM_XPASS_MULTI(float, double, float)
GM_XPASS_MULTI(float, float, float)
GM_XPASS_MULTI(float, float, double)
#undef GM_XPASS_MULTI
template YsolveArgs<double> ysolve_args<double>(const TransformTables&, int, int, double*, const Gate&);
template YsolveArgs<float> ysolve_args<float>(const TransformTables&, int, int, float*, const Gate&);
template void launch_ysolve_multi<double>(const ArgPack<YsolveArgs<double>>&, int, const TransformTables&,
                                          cudaStream_t);
template void launch_ysolve_multi<float>(const ArgPack<YsolveArgs<float>>&, int, const TransformTables&,
                                         cudaStream_t);
template void launch_band_first_multi<double>(const ArgPack<BandFirstArgs<double>>&, int, cudaStream_t);
template void launch_band_first_multi<float>(const ArgPack<BandFirstArgs<float>>&, int, cudaStream_t);
template void launch_band_gemv_multi<double>(const ArgPack<BandGemvArgs<double>>&, int, cudaStream_t);
template void launch_band_gemv_multi<float>(const ArgPack<BandGemvArgs<float>>&, int, cudaStream_t);
template void launch_band_direct_multi<double>(const ArgPack<BandDirectArgs<double>>&, int, cudaStream_t);
template void launch_band_direct_multi<float>(const ArgPack<BandDirectArgs<float>>&, int, cudaStream_t);
template void launch_band_fwd_solve_multi<double>(const ArgPack<BandFwdArgs<double>>&, int, cudaStream_t);
template void launch_band_fwd_solve_multi<float>(const ArgPack<BandFwdArgs<float>>&, int, cudaStream_t);

}  // namespace gmk
