// Snapshot POD (method of snapshots, postprocessing/modal_analysis.py:17-98) on the GPU.
//
// For M snapshots of N points (rows of X):
//   mean       the time average of every point, summed over the snapshots in order (the order
//              numpy's mean along axis 0 adds them), so it equals the reference bit for bit;
//   X'         X - mean, kept on the device;
//   C          X' X'^T / M, an M x M Gram matrix: 32 x 32 output tiles, the point range split
//              over blocks (each block accumulates its slice in FP64 from shared-memory tiles),
//              the slices then summed in a fixed order;
// the host takes the eigen-decomposition of C (M is small), and the device forms
//   phi_i      = X'^T v_i / sigma_i, one thread per point for all requested modes;
//   a_i        = X' phi_i, dot products over the points (per-block partials, fixed-order sums).
// All arithmetic is FP64.  Input snapshots may be host or device memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ghostmac.h"

namespace gmk {
void kernel_launch_adjust(long long delta);
}

struct gm_pod {
  int M = 0;
  int64_t N = 0;
  double* X = nullptr;       // M x N fluctuations
  double* mean = nullptr;    // N
  double* part = nullptr;    // Gram / coefficient partial sums
  size_t part_n = 0;
  double* C = nullptr;       // M x M
  double* V = nullptr;       // M x k eigenvector columns (row s: snapshot s)
  double* modes = nullptr;   // k x N
  double* coef = nullptr;    // k x M
  int kcap = 0;
  std::string err;
};

namespace {

constexpr int T = 32;             // Gram tile edge
constexpr int KCHUNK = 32;        // points per shared-memory stage
constexpr int SLICE = 16384;      // points per Gram block (its slice of the point range)
constexpr int MAXM = 4096;

__global__ void k_pod_mean(const double* __restrict__ X, int M, int64_t N, double* __restrict__ mean,
                           double* __restrict__ Xp) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  double s = 0.0;
  for (int i = 0; i < M; ++i) s += X[(int64_t)i * N + p];
  const double m = s / (double)M;
  mean[p] = m;
  for (int i = 0; i < M; ++i) Xp[(int64_t)i * N + p] = X[(int64_t)i * N + p] - m;
}

// part[slice][i][j] = sum over the slice's points of X'[i][p] X'[j][p], for the tile (bi, bj)
__global__ void __launch_bounds__(T * 8) k_pod_gram(const double* __restrict__ Xp, int M, int64_t N,
                                                    double* __restrict__ part) {
  __shared__ double a[T][KCHUNK + 1];
  __shared__ double b[T][KCHUNK + 1];
  const int bi = blockIdx.x, bj = blockIdx.y, sl = blockIdx.z;
  if (bj < bi) return;  // C is symmetric: the upper tiles only
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8: each thread 4 outputs (rows ty, ty+8, ...)
  const int64_t p0 = (int64_t)sl * SLICE, p1 = min((int64_t)N, p0 + SLICE);
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t k0 = p0; k0 < p1; k0 += KCHUNK) {
    for (int r = ty; r < T; r += 8) {
      const int gi = bi * T + r, gj = bj * T + r;
      const int64_t k = k0 + tx;
      a[r][tx] = (gi < M && k < p1) ? Xp[(int64_t)gi * N + k] : 0.0;
      b[r][tx] = (gj < M && k < p1) ? Xp[(int64_t)gj * N + k] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < KCHUNK; ++kk) {
      const double bv = b[tx][kk];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(a[ty + 8 * q][kk], bv, acc[q]);
    }
    __syncthreads();
  }
  const int nt = (M + T - 1) / T;
  for (int q = 0; q < 4; ++q) {
    const int i = bi * T + ty + 8 * q, j = bj * T + tx;
    if (i < M && j < M) part[((int64_t)sl * nt * nt + (int64_t)bi * nt + bj) * T * T + (ty + 8 * q) * T + tx] = acc[q];
  }
}

// C[i][j] = C[j][i] = (sum over slices in order) / M
__global__ void k_pod_gram_fold(const double* __restrict__ part, int M, int nslice, double* __restrict__ C) {
  const int i = blockIdx.y * blockDim.y + threadIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M || j >= M || j < i) return;
  const int nt = (M + T - 1) / T, bi = i / T, bj = j / T;
  double s = 0.0;
  for (int sl = 0; sl < nslice; ++sl) s += part[((int64_t)sl * nt * nt + (int64_t)bi * nt + bj) * T * T + (i % T) * T + (j % T)];
  const double c = s / (double)M;
  C[(int64_t)i * M + j] = c;
  C[(int64_t)j * M + i] = c;
}

// modes[q][p] = sum_s X'[s][p] V[s][q] / sigma[q] (zero where sigma <= 1e-12)
__global__ void k_pod_modes(const double* __restrict__ Xp, int M, int64_t N, const double* __restrict__ V, int k,
                            const double* __restrict__ inv_sigma, double* __restrict__ modes) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  for (int q = 0; q < k; ++q) {
    double s = 0.0;
    for (int i = 0; i < M; ++i) s += Xp[(int64_t)i * N + p] * V[(int64_t)i * k + q];
    modes[(int64_t)q * N + p] = inv_sigma[q] > 0 ? s * inv_sigma[q] : 0.0;
  }
}

// part[b][s][q] = sum over block b's points of X'[s][p] modes[q][p]
__global__ void k_pod_coef_part(const double* __restrict__ Xp, int M, int64_t N, const double* __restrict__ modes,
                                int k, double* __restrict__ part) {
  __shared__ double red[256 / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = 0; s < M; ++s)
    for (int q = 0; q < k; ++q) {
      double acc = 0.0;
      for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x)
        acc += Xp[(int64_t)s * N + p] * modes[(int64_t)q * N + p];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) red[warp] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        part[((int64_t)blockIdx.x * M + s) * k + q] = t;
      }
      __syncthreads();
    }
}
__global__ void k_pod_coef_fold(const double* __restrict__ part, int nb, int M, int k, double* __restrict__ coef) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M * k) return;
  const int s = e / k, q = e - s * k;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += part[((int64_t)b * M + s) * k + q];
  coef[(int64_t)q * M + s] = t;
}

bool is_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int fail(gm_pod* p, int code, const std::string& msg) {
  p->err = msg;
  return code;
}
int cuda_fail(gm_pod* p, cudaError_t e) {
  cudaGetLastError();
  return fail(p, GM_ECUDA, cudaGetErrorString(e));
}
template <typename Tp>
cudaError_t grow(Tp** ptr, size_t& have, size_t need) {
  if (have >= need && *ptr) return cudaSuccess;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(ptr, need * sizeof(Tp));
  if (e == cudaSuccess) have = need;
  return e;
}

}  // namespace

extern "C" {

int gm_pod_create(int32_t n_snapshots, int64_t n_points, gm_pod** out) {
  if (!out) return GM_EVALUE;
  *out = nullptr;
  if (n_snapshots < 1 || n_snapshots > MAXM || n_points < 1) return GM_EVALUE;
  gm_pod* p = new gm_pod();
  p->M = n_snapshots;
  p->N = n_points;
  cudaError_t e = cudaMalloc(&p->X, (size_t)p->M * p->N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&p->mean, (size_t)p->N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&p->C, (size_t)p->M * p->M * sizeof(double));
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (p->X) cudaFree(p->X);
    if (p->mean) cudaFree(p->mean);
    if (p->C) cudaFree(p->C);
    delete p;
    return GM_ECUDA;
  }
  *out = p;
  return GM_OK;
}

int gm_pod_destroy(gm_pod* p) {
  if (!p) return GM_OK;
  for (double* q : {p->X, p->mean, p->part, p->C, p->V, p->modes, p->coef})
    if (q) cudaFree(q);
  delete p;
  return GM_OK;
}

const char* gm_pod_last_error(const gm_pod* p) { return p ? p->err.c_str() : "null handle"; }

int gm_pod_gram(gm_pod* p, const double* snapshots, double* mean, double* gram, void* stream) {
  if (!p || !snapshots || !mean || !gram) return p ? fail(p, GM_EVALUE, "null argument") : GM_EVALUE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int M = p->M;
  const int64_t N = p->N;
  const size_t bytes = (size_t)M * N * sizeof(double);
  // the snapshots go through the fluctuation buffer: staged there first when they are host data
  const double* X = snapshots;
  if (!is_device(snapshots)) {
    if (cudaError_t e = cudaMemcpyAsync(p->X, snapshots, bytes, cudaMemcpyHostToDevice, st)) return cuda_fail(p, e);
    X = p->X;
  }
  k_pod_mean<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(X, M, N, p->mean, p->X);
  const int nt = (M + T - 1) / T;
  const int nslice = (int)((N + SLICE - 1) / SLICE);
  if (cudaError_t e = grow(&p->part, p->part_n, (size_t)nslice * nt * nt * T * T)) return cuda_fail(p, e);
  k_pod_gram<<<dim3(nt, nt, nslice), dim3(T, 8), 0, st>>>(p->X, M, N, p->part);
  k_pod_gram_fold<<<dim3(nt, nt), dim3(T, T), 0, st>>>(p->part, M, nslice, p->C);
  gmk::kernel_launch_adjust(3);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(p, e);
  cudaError_t e = cudaMemcpyAsync(mean, p->mean, N * sizeof(double), cudaMemcpyDefault, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gram, p->C, (size_t)M * M * sizeof(double), cudaMemcpyDefault, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(p, e);
  return GM_OK;
}

int gm_pod_modes(gm_pod* p, const double* eigvecs, const double* sigma, int32_t k, double* modes, double* coeffs,
                 void* stream) {
  if (!p || !eigvecs || !sigma || !modes || !coeffs) return p ? fail(p, GM_EVALUE, "null argument") : GM_EVALUE;
  if (k < 1 || k > p->M) return fail(p, GM_EVALUE, "mode count must be between 1 and the snapshot count");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int M = p->M;
  const int64_t N = p->N;
  if (k > p->kcap) {
    for (double** q : {&p->V, &p->modes, &p->coef})
      if (*q) { cudaFree(*q); *q = nullptr; }
    cudaError_t e = cudaMalloc(&p->V, ((size_t)M * k + k) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&p->modes, (size_t)k * N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&p->coef, (size_t)k * M * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(p, e);
    p->kcap = k;
  }
  std::vector<double> host((size_t)M * k + k);
  std::memcpy(host.data(), eigvecs, (size_t)M * k * sizeof(double));
  for (int q = 0; q < k; ++q) host[(size_t)M * k + q] = sigma[q] > 1e-12 ? 1.0 / sigma[q] : 0.0;
  if (cudaError_t e = cudaMemcpyAsync(p->V, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, st))
    return cuda_fail(p, e);
  k_pod_modes<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(p->X, M, N, p->V, k, p->V + (size_t)M * k, p->modes);
  const int nb = (int)std::min<int64_t>(304, (N + 255) / 256);
  if (cudaError_t e = grow(&p->part, p->part_n, (size_t)nb * M * k)) return cuda_fail(p, e);
  k_pod_coef_part<<<nb, 256, 0, st>>>(p->X, M, N, p->modes, k, p->part);
  k_pod_coef_fold<<<(unsigned)((M * k + 255) / 256), 256, 0, st>>>(p->part, nb, M, k, p->coef);
  gmk::kernel_launch_adjust(3);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(p, e);
  cudaError_t e = cudaMemcpyAsync(modes, p->modes, (size_t)k * N * sizeof(double), cudaMemcpyDefault, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(coeffs, p->coef, (size_t)k * M * sizeof(double), cudaMemcpyDefault, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(p, e);
  return GM_OK;
}

}  // extern "C"
