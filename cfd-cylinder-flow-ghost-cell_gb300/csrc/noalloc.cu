// Allocation-free fluid-cell divergence statistics.
//
// Some callers cannot call cudaMalloc at all: code that runs while another
// runtime owns the device memory pool (an embedding framework's fixed arena or
// a no-allocation steady-state loop), or a tool that only borrows device arrays
// from its host program.  gm_divergence_stats_noalloc serves them: it computes
// the same statistics as gm_divergence_stats (mac_engine's
// calculate_mac_divergence_cpp diagnostic) from caller-owned device arrays and
// keeps its only scratch, the per-block partial results, in the file-scope
// device array below.  Neither it nor anything it calls allocates.
//
// Limits and sharing:
//  * the grid may have at most GM_NOALLOC_MAX_CELLS pressure cells (larger
//    grids are rejected with GM_EVALUE);
//  * every GPU that loads this library holds the array (160 KiB) until exit;
//  * all calls share the array: calls that overlap on the GPU (different
//    streams, or host threads without ordering) race on it and must be
//    serialised by the caller;
//  * the first call on a device looks the array's device address up once for
//    that device; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/ghostmac.h"

namespace gmk {
void kernel_launch_adjust(long long delta);  // the library's launch counter (kernels.cu)
}

void gm_internal_set_error(const char* msg);  // defined in ghostmac.cu

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = GM_NOALLOC_MAX_CELLS / NA_THREADS;
constexpr int NA_FIELDS = 5;  // max |div|, sum div^2, count, core sum div^2, core count

// Per-block partials (written in full by every first pass, so nothing needs
// clearing between calls) and the 5 reduced values.
static __device__ __align__(256) double g_noalloc_scratch[NA_MAX_BLOCKS * NA_FIELDS + NA_FIELDS];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[MAX_DEVICES] = {};

__device__ __forceinline__ double warp_reduce(double v, bool is_max) {
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, w) : v + w;
  }
  return v;
}

// Pass 1: one partial record per block, in a fixed order of the block's threads.
__global__ void k_div_partials(const double* __restrict__ u, const double* __restrict__ v,
                               const unsigned char* __restrict__ mask, int nx, int ny, double dx, double dy,
                               double* __restrict__ scratch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)nx * ny;
  double r[NA_FIELDS] = {0, 0, 0, 0, 0};
  if (t < n && !mask[t]) {
    int j = (int)(t / nx), i = (int)(t % nx);
    double d = (u[(long long)j * (nx + 1) + i + 1] - u[(long long)j * (nx + 1) + i]) / dx +
               (v[(long long)(j + 1) * nx + i] - v[(long long)j * nx + i]) / dy;
    r[0] = fabs(d);
    r[1] = d * d;
    r[2] = 1;
    bool core = !(i > 0 && mask[t - 1]) && !(i < nx - 1 && mask[t + 1]) && !(j > 0 && mask[t - nx]) &&
                !(j < ny - 1 && mask[t + nx]);
    if (core) { r[3] = d * d; r[4] = 1; }
  }
  __shared__ double sm[NA_FIELDS][NA_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int f = 0; f < NA_FIELDS; ++f) {
    double w = warp_reduce(r[f], f == 0);
    if (lane == 0) sm[f][wid] = w;
  }
  __syncthreads();
  if (threadIdx.x < NA_FIELDS) {
    const int f = threadIdx.x;
    double acc = sm[f][0];
    for (int w = 1; w < NA_THREADS / 32; ++w) acc = f == 0 ? fmax(acc, sm[f][w]) : acc + sm[f][w];
    scratch[(long long)blockIdx.x * NA_FIELDS + f] = acc;
  }
}

// Pass 2: one block folds the partials of pass 1 in block order.
__global__ void k_div_final(int nblocks, double* __restrict__ scratch) {
  const int f = threadIdx.x;
  if (f >= NA_FIELDS) return;
  double acc = 0;
  for (int b = 0; b < nblocks; ++b) {
    double x = scratch[(long long)b * NA_FIELDS + f];
    acc = f == 0 ? fmax(acc, x) : acc + x;
  }
  scratch[(long long)NA_MAX_BLOCKS * NA_FIELDS + f] = acc;
}

int fail(int code, const char* msg) {
  gm_internal_set_error(msg);  // fixed buffer read by gm_last_error(NULL); no heap use
  return code;
}

// device (or managed) memory of the current device `dev`: arrays of another GPU would be
// read across the link, or fault without peer access
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

}  // namespace

extern "C" {

int gm_divergence_stats_noalloc(const double* u, const double* v, const uint8_t* mask, int32_t nx, int32_t ny,
                                double dx, double dy, double out[3], int64_t counts[2], void* stream) {
  if (!u || !v || !mask || !out || !counts) return fail(GM_EVALUE, "null argument");
  if (nx < 2 || ny < 2) return fail(GM_EVALUE, "mask must be a 2D grid with at least 2 cells per direction");
  if (!(std::isfinite(dx) && dx > 0 && std::isfinite(dy) && dy > 0))
    return fail(GM_EVALUE, "dx and dy must be finite and positive");
  if ((long long)nx * ny > GM_NOALLOC_MAX_CELLS)
    return fail(GM_EVALUE, "grid exceeds GM_NOALLOC_MAX_CELLS pressure cells of the static scratch");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    return fail(GM_ECUDA, "no CUDA device");
  }
  if (!on_device(u, dev) || !on_device(v, dev) || !on_device(mask, dev))
    return fail(GM_EVALUE, "u, v and mask must be device arrays of the current device");
  double* scratch = nullptr;
  {
    // set-up, once per device with that device current: device address of the static array
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GM_ECUDA, cudaGetErrorString(e));
      }
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long n = (long long)nx * ny;
  const int nblocks = (int)((n + NA_THREADS - 1) / NA_THREADS);
  gmk::kernel_launch_adjust(1);
  k_div_partials<<<nblocks, NA_THREADS, 0, st>>>(u, v, mask, nx, ny, dx, dy, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    gmk::kernel_launch_adjust(1);
    k_div_final<<<1, 32, 0, st>>>(nblocks, scratch);
    e = cudaGetLastError();
  }
  // a failed launch must not return the previous call's totals, which the shared array still holds
  if (e != cudaSuccess) return fail(GM_ECUDA, cudaGetErrorString(e));
  double r[NA_FIELDS];
  e = cudaMemcpyAsync(r, scratch + (long long)NA_MAX_BLOCKS * NA_FIELDS, sizeof r, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GM_ECUDA, cudaGetErrorString(e));
  }
  out[0] = r[0];
  out[1] = r[1];
  out[2] = r[3];
  counts[0] = (int64_t)std::llround(r[2]);
  counts[1] = (int64_t)std::llround(r[4]);
  return GM_OK;
}

}  // extern "C"
