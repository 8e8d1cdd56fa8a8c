// Learned pressure preconditioner: a 4-level convolutional U-Net on the pressure grid with
// BF16 weights and FP32 activations / accumulation; forward, backward (data and weight
// gradients) and Adam kernels.  It has no reference counterpart: it is the learned slot in
// the GMRES preconditioner (solver/pressure_schur.py:20-27, 39-41).
//
// Architecture (fixed): channels c = (16, 32, 64, 64) on levels 0..3 (level l has the grid
// coarsened 2^l times by 2x2 averaging).  Encoder: two 3x3 convolutions + ReLU per level
// (input: 2 channels, the normalised residual and the active mask).  Decoder: nearest 2x
// upsampling, concatenation with the encoder output of the level, one 3x3 convolution +
// ReLU.  Output: a 3x3 convolution to one channel (linear).  Twelve convolutions, 253,872
// weights and 465 biases.  Tensors are [batch][channel][height][width], zero padding.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ghostmac.h"

namespace gmk {
void kernel_launch_adjust(long long delta);  // the library's launch counter (kernels.cu)
}

namespace {

constexpr int NL = 12;
struct LayerDef {
  int cin, cout, level;
  bool relu;
};
constexpr LayerDef LAYERS[NL] = {{2, 16, 0, true},   {16, 16, 0, true},  {16, 32, 1, true}, {32, 32, 1, true},
                                 {32, 64, 2, true},  {64, 64, 2, true},  {64, 64, 3, true}, {64, 64, 3, true},
                                 {128, 64, 2, true}, {96, 32, 1, true},  {48, 16, 0, true}, {16, 1, 0, false}};

struct UnetError : std::exception {
  std::string msg;
  explicit UnetError(std::string m) : msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};
#define UN_CK(call)                                                                                \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) throw UnetError(std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

// ---- 3x3 convolution ------------------------------------------------------------------------
// forward:        out[b][co] = bias[co] + sum_ci sum_k W[co][ci][k] in[b][ci](p + d_k)
// transposed:     out[b][ci] = sum_co sum_k W[co][ci][k] in[b][co](p - d_k)      (data gradient)
// One thread per output pixel of a 32 x 8 tile, CO output channels per thread, the input tile
// (with its one-cell halo) and the CO x 9 weights of one input channel staged in shared memory.
constexpr int TW = 32, TH = 8, CO = 8;
template <bool TRANSPOSED>
__global__ void k_conv3(int B, int H, int W, int cin, int cout, const float* __restrict__ in,
                        const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias, float* __restrict__ out,
                        int relu) {
  __shared__ float tile[TH + 2][TW + 2];
  __shared__ float wt[CO][9];
  const int nco = (cout + CO - 1) / CO;
  const int b = blockIdx.z / nco, co0 = (blockIdx.z % nco) * CO;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  float acc[CO];
#pragma unroll
  for (int c = 0; c < CO; ++c) acc[c] = (!TRANSPOSED && bias && co0 + c < cout) ? bias[co0 + c] : 0.f;
  const size_t plane = (size_t)H * W;
  for (int ci = 0; ci < cin; ++ci) {
    const float* src = in + ((size_t)b * cin + ci) * plane;
    for (int t = ty * TW + tx; t < (TH + 2) * (TW + 2); t += TW * TH) {
      const int yy = t / (TW + 2), xx = t - yy * (TW + 2);
      const int gy = y0 + yy - 1, gx = x0 + xx - 1;
      tile[yy][xx] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? src[(size_t)gy * W + gx] : 0.f;
    }
    for (int t = ty * TW + tx; t < CO * 9; t += TW * TH) {
      const int c = t / 9, k = t - c * 9;
      float v = 0.f;
      if (co0 + c < cout) {
        // forward: W[co][ci][k]; transposed: the output channel is an input channel of the
        // layer (ci here runs over the layer's outputs) and the taps are mirrored
        v = TRANSPOSED ? __bfloat162float(w[((size_t)ci * cout + (co0 + c)) * 9 + (8 - k)])
                       : __bfloat162float(w[((size_t)(co0 + c) * cin + ci) * 9 + k]);
      }
      wt[c][k] = v;
    }
    __syncthreads();
    float v9[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v9[k] = tile[ty + k / 3][tx + k % 3];
#pragma unroll
    for (int c = 0; c < CO; ++c)
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[c] += wt[c][k] * v9[k];
    __syncthreads();
  }
  if (x < W && y < H) {
#pragma unroll
    for (int c = 0; c < CO; ++c) {
      if (co0 + c >= cout) break;
      float v = acc[c];
      if (relu && v < 0.f) v = 0.f;
      out[((size_t)b * cout + co0 + c) * plane + (size_t)y * W + x] = v;
    }
  }
}

// weight and bias gradients: dW[co][ci][k] += sum_b,p dz[b][co](p) in[b][ci](p + d_k),
// db[co] += sum dz.  Block: CO output channels x one input channel x a slice of rows.
__global__ void k_conv3_wgrad(int B, int H, int W, int cin, int cout, const float* __restrict__ in,
                              const float* __restrict__ dz, float* __restrict__ dw, float* __restrict__ db,
                              int row_slices) {
  const int nco = (cout + CO - 1) / CO;
  const int co0 = (blockIdx.x % nco) * CO, ci = blockIdx.x / nco;
  const int slice = blockIdx.y;
  const int rows_per = (H + row_slices - 1) / row_slices;
  const int ya = slice * rows_per, yb = min(H, ya + rows_per);
  float acc[CO][9];
  float bacc[CO];
#pragma unroll
  for (int c = 0; c < CO; ++c) {
    bacc[c] = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[c][k] = 0.f;
  }
  const size_t plane = (size_t)H * W;
  for (int b = 0; b < B; ++b) {
    const float* src = in + ((size_t)b * cin + ci) * plane;
    for (int t = threadIdx.x; t < (yb - ya) * W; t += blockDim.x) {
      const int y = ya + t / W, x = t % W;
      float v9[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const int gy = y + k / 3 - 1, gx = x + k % 3 - 1;
        v9[k] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? src[(size_t)gy * W + gx] : 0.f;
      }
#pragma unroll
      for (int c = 0; c < CO; ++c) {
        if (co0 + c >= cout) break;
        const float g = dz[((size_t)b * cout + co0 + c) * plane + (size_t)y * W + x];
        bacc[c] += g;
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[c][k] += g * v9[k];
      }
    }
  }
  // block reduction: warp shuffles, then one atomic per value from each warp
#pragma unroll
  for (int c = 0; c < CO; ++c) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float v = acc[c][k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0 && co0 + c < cout) atomicAdd(&dw[((size_t)(co0 + c) * cin + ci) * 9 + k], v);
    }
    float v = bacc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && ci == 0 && co0 + c < cout && db) atomicAdd(&db[co0 + c], v);
  }
}

// g *= (act > 0)   (ReLU backward on the layer output)
__global__ void k_relu_back(size_t n, const float* __restrict__ act, float* __restrict__ g) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    if (!(act[t] > 0.f)) g[t] = 0.f;
}
// 2x2 average pooling of C planes (H, W even) and its adjoint
__global__ void k_pool(int BC, int H, int W, const float* __restrict__ in, float* __restrict__ out) {
  const int h = H / 2, w = W / 2;
  const size_t n = (size_t)BC * h * w;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t pl = t / ((size_t)h * w);
    const int r = (int)(t - pl * h * w), y = r / w, x = r - y * w;
    const float* s = in + pl * H * W + (size_t)(2 * y) * W + 2 * x;
    out[t] = 0.25f * (s[0] + s[1] + s[W] + s[W + 1]);
  }
}
__global__ void k_pool_back(int BC, int H, int W, const float* __restrict__ dout, float* __restrict__ din, int add) {
  const int h = H / 2, w = W / 2;
  const size_t n = (size_t)BC * H * W;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t pl = t / ((size_t)H * W);
    const int r = (int)(t - pl * H * W), y = r / W, x = r - y * W;
    const float v = 0.25f * dout[pl * h * w + (size_t)(y / 2) * w + x / 2];
    din[t] = add ? din[t] + v : v;
  }
}
// nearest 2x upsampling of C planes into channels [0, C) of a wider tensor and its adjoint
__global__ void k_up(int B, int C, int Ctot, int h, int w, const float* __restrict__ in, float* __restrict__ out) {
  const int H = 2 * h, W = 2 * w;
  const size_t n = (size_t)B * C * H * W;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t pl = t / ((size_t)H * W);
    const int b = (int)(pl / C), c = (int)(pl - (size_t)b * C);
    const int r = (int)(t - pl * H * W), y = r / W, x = r - y * W;
    out[((size_t)b * Ctot + c) * H * W + r] = in[pl * h * w + (size_t)(y / 2) * w + x / 2];
  }
}
__global__ void k_up_back(int B, int C, int Ctot, int h, int w, const float* __restrict__ dout, float* __restrict__ din) {
  const int H = 2 * h, W = 2 * w;
  const size_t n = (size_t)B * C * h * w;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t pl = t / ((size_t)h * w);
    const int b = (int)(pl / C), c = (int)(pl - (size_t)b * C);
    const int r = (int)(t - pl * h * w), y = r / w, x = r - y * w;
    const float* s = dout + ((size_t)b * Ctot + c) * H * W + (size_t)(2 * y) * W + 2 * x;
    din[t] = s[0] + s[1] + s[W] + s[W + 1];
  }
}
// copy C planes per batch item between tensors of different channel counts
__global__ void k_copy_ch(int B, int C, size_t plane, const float* __restrict__ src, int csrc, int off_src,
                          float* __restrict__ dst, int cdst, int off_dst, int add) {
  const size_t n = (size_t)B * C * plane;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t pl = t / plane;
    const int b = (int)(pl / C), c = (int)(pl - (size_t)b * C);
    const size_t r = t - pl * plane;
    const float v = src[((size_t)b * csrc + off_src + c) * plane + r];
    float& d = dst[((size_t)b * cdst + off_dst + c) * plane + r];
    d = add ? d + v : v;
  }
}

unsigned gsz(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16); }

}  // namespace

struct gm_unet {
  int B = 0, H = 0, W = 0;
  // activations per layer output and the per-layer inputs that are not another layer's output
  float* act[NL] = {};     // outputs of the twelve convolutions
  float* pooled[3] = {};   // pool(e0), pool(e1), pool(e2)
  float* cat[3] = {};      // decoder inputs on levels 2, 1, 0
  float* x = nullptr;      // network input (2 channels)
  float* g_act[NL] = {};   // gradients of the layer outputs
  float* g_pooled[3] = {};
  float* g_cat[3] = {};
  std::vector<void*> allocs;
  std::string err;
  ~gm_unet() {
    for (void* p : allocs) cudaFree(p);
  }
  float* alloc(size_t n) {
    void* p = nullptr;
    UN_CK(cudaMalloc(&p, n * sizeof(float)));
    allocs.push_back(p);
    return (float*)p;
  }
  size_t plane(int level) const { return (size_t)(H >> level) * (W >> level); }
};

namespace {

// input tensor of layer k and its channel count
const float* layer_input(gm_unet* u, int k) {
  switch (k) {
    case 0: return u->x;
    case 2: return u->pooled[0];
    case 4: return u->pooled[1];
    case 6: return u->pooled[2];
    case 8: return u->cat[0];
    case 9: return u->cat[1];
    case 10: return u->cat[2];
    default: return u->act[k - 1];
  }
}
float* layer_input_grad(gm_unet* u, int k) {
  switch (k) {
    case 0: return nullptr;
    case 2: return u->g_pooled[0];
    case 4: return u->g_pooled[1];
    case 6: return u->g_pooled[2];
    case 8: return u->g_cat[0];
    case 9: return u->g_cat[1];
    case 10: return u->g_cat[2];
    default: return u->g_act[k - 1];
  }
}

void conv_fwd(gm_unet* u, int k, const __nv_bfloat16* w, const float* b, cudaStream_t st) {
  const LayerDef& L = LAYERS[k];
  const int H = u->H >> L.level, W = u->W >> L.level;
  dim3 grid((W + TW - 1) / TW, (H + TH - 1) / TH, u->B * ((L.cout + CO - 1) / CO)), block(TW, TH);
  gmk::kernel_launch_adjust(1);
  k_conv3<false><<<grid, block, 0, st>>>(u->B, H, W, L.cin, L.cout, layer_input(u, k), w, b, u->act[k], L.relu ? 1 : 0);
}

void forward(gm_unet* u, const __nv_bfloat16* const* w, const float* const* b, cudaStream_t st) {
  for (int k = 0; k < 8; ++k) {
    conv_fwd(u, k, w[k], b[k], st);
    if (k == 1 || k == 3 || k == 5) {
      const int l = LAYERS[k].level;
      gmk::kernel_launch_adjust(1);
      k_pool<<<gsz((size_t)u->B * LAYERS[k].cout * u->plane(l + 1)), 256, 0, st>>>(
          u->B * LAYERS[k].cout, u->H >> l, u->W >> l, u->act[k], u->pooled[k / 2]);
    }
  }
  // decoder: cat = [up(previous decoder output), encoder output of the level]
  const int skip[3] = {5, 3, 1}, prev[3] = {7, 8, 9};
  for (int d = 0; d < 3; ++d) {
    const int k = 8 + d, l = LAYERS[k].level;
    const int cu = LAYERS[prev[d]].cout, cs = LAYERS[skip[d]].cout, ct = cu + cs;
    gmk::kernel_launch_adjust(1);
    k_up<<<gsz((size_t)u->B * cu * u->plane(l)), 256, 0, st>>>(u->B, cu, ct, u->H >> (l + 1), u->W >> (l + 1),
                                                                 u->act[prev[d]], u->cat[d]);
    gmk::kernel_launch_adjust(1);
    k_copy_ch<<<gsz((size_t)u->B * cs * u->plane(l)), 256, 0, st>>>(u->B, cs, u->plane(l), u->act[skip[d]], cs, 0,
                                                                      u->cat[d], ct, cu, 0);
    conv_fwd(u, k, w[k], b[k], st);
  }
  conv_fwd(u, 11, w[11], b[11], st);
}

void backward(gm_unet* u, const __nv_bfloat16* const* w, float* const* dw, float* const* db, cudaStream_t st) {
  // g_act[11] holds dL/dy on entry; gradients accumulate into dw / db (zeroed by the caller)
  for (int k = 0; k < NL; ++k)
    if (k != 11) UN_CK(cudaMemsetAsync(u->g_act[k], 0, (size_t)u->B * LAYERS[k].cout * u->plane(LAYERS[k].level) * 4, st));
  for (int d = 0; d < 3; ++d) {
    const int l = LAYERS[8 + d].level;
    UN_CK(cudaMemsetAsync(u->g_cat[d], 0, (size_t)u->B * LAYERS[8 + d].cin * u->plane(l) * 4, st));
  }
  auto conv_back = [&](int k) {
    const LayerDef& L = LAYERS[k];
    const int H = u->H >> L.level, W = u->W >> L.level;
    const size_t n = (size_t)u->B * L.cout * H * W;
    if (L.relu) {
      gmk::kernel_launch_adjust(1);
      k_relu_back<<<gsz(n), 256, 0, st>>>(n, u->act[k], u->g_act[k]);
    }
    const int slices = std::max(1, std::min(64, H / 8));
    dim3 gw(((L.cout + CO - 1) / CO) * L.cin, slices);
    gmk::kernel_launch_adjust(1);
    k_conv3_wgrad<<<gw, 256, 0, st>>>(u->B, H, W, L.cin, L.cout, layer_input(u, k), u->g_act[k], dw[k], db[k], slices);
    float* gin = layer_input_grad(u, k);
    if (gin) {
      // the data gradient is written (not accumulated): every consumer tensor has exactly
      // one producing convolution, except the encoder outputs handled below
      dim3 grid((W + TW - 1) / TW, (H + TH - 1) / TH, u->B * ((L.cin + CO - 1) / CO)), block(TW, TH);
      gmk::kernel_launch_adjust(1);
      k_conv3<true><<<grid, block, 0, st>>>(u->B, H, W, L.cout, L.cin, u->g_act[k], w[k], nullptr, gin, 0);
    }
  };
  conv_back(11);
  const int skip[3] = {5, 3, 1}, prev[3] = {7, 8, 9};
  for (int d = 2; d >= 0; --d) {
    const int k = 8 + d, l = LAYERS[k].level;
    conv_back(k);
    const int cu = LAYERS[prev[d]].cout, cs = LAYERS[skip[d]].cout, ct = cu + cs;
    // split the concatenated gradient: upsampled part -> previous decoder output, skip part ->
    // encoder output (added: the encoder output also feeds the pooling / next conv)
    gmk::kernel_launch_adjust(1);
    k_up_back<<<gsz((size_t)u->B * cu * u->plane(l + 1)), 256, 0, st>>>(u->B, cu, ct, u->H >> (l + 1),
                                                                         u->W >> (l + 1), u->g_cat[d], u->g_act[prev[d]]);
    gmk::kernel_launch_adjust(1);
    k_copy_ch<<<gsz((size_t)u->B * cs * u->plane(l)), 256, 0, st>>>(u->B, cs, u->plane(l), u->g_cat[d], ct, cu,
                                                                      u->g_act[skip[d]], cs, 0, 1);
  }
  // encoder, top down: g_act[7] came from the decoder; g_act[5], [3], [1] hold their skip
  // gradients and receive the pooling path right after the next level's first conv
  for (int k = 7; k >= 0; --k) {
    if (k == 6 || k == 4 || k == 2) {
      conv_back(k);  // writes g_pooled
      const int src = k - 1, l = LAYERS[src].level;
      gmk::kernel_launch_adjust(1);
      k_pool_back<<<gsz((size_t)u->B * LAYERS[src].cout * u->plane(l)), 256, 0, st>>>(
          u->B * LAYERS[src].cout, u->H >> l, u->W >> l, u->g_pooled[k / 2 - 1], u->g_act[src], 1);
    } else {
      // k_conv3<true> writes its data gradient into g_act[k - 1]: for k = 7, 5, 3, 1 the input
      // is the previous conv's output, which has no other consumer
      conv_back(k);
    }
  }
}

std::string g_unet_error;

}  // namespace

extern "C" {

int gm_unet_layers(int32_t* n_layers, int32_t* cin, int32_t* cout) {
  if (n_layers) *n_layers = NL;
  for (int k = 0; k < NL; ++k) {
    if (cin) cin[k] = LAYERS[k].cin;
    if (cout) cout[k] = LAYERS[k].cout;
  }
  return GM_OK;
}

int gm_unet_create(int32_t batch, int32_t height, int32_t width, gm_unet** out) {
  if (!out) return GM_EVALUE;
  *out = nullptr;
  if (batch < 1 || height < 8 || width < 8 || height % 8 || width % 8) {
    g_unet_error = "the network needs batch >= 1 and a grid whose sides are multiples of 8";
    return GM_EVALUE;
  }
  auto u = std::make_unique<gm_unet>();
  u->B = batch;
  u->H = height;
  u->W = width;
  try {
    u->x = u->alloc((size_t)batch * 2 * u->plane(0));
    for (int k = 0; k < NL; ++k) {
      const size_t n = (size_t)batch * LAYERS[k].cout * u->plane(LAYERS[k].level);
      u->act[k] = u->alloc(n);
      u->g_act[k] = u->alloc(n);
    }
    for (int p = 0; p < 3; ++p) {
      const size_t n = (size_t)batch * LAYERS[2 * p + 1].cout * u->plane(p + 1);
      u->pooled[p] = u->alloc(n);
      u->g_pooled[p] = u->alloc(n);
    }
    for (int d = 0; d < 3; ++d) {
      const size_t n = (size_t)batch * LAYERS[8 + d].cin * u->plane(LAYERS[8 + d].level);
      u->cat[d] = u->alloc(n);
      u->g_cat[d] = u->alloc(n);
    }
  } catch (const std::exception& e) {
    g_unet_error = e.what();
    return GM_ECUDA;
  }
  *out = u.release();
  return GM_OK;
}

int gm_unet_destroy(gm_unet* u) {
  delete u;
  return GM_OK;
}

const char* gm_unet_last_error(const gm_unet* u) { return u ? u->err.c_str() : g_unet_error.c_str(); }

int gm_unet_input(gm_unet* u, float** x) {
  if (!u || !x) return GM_EVALUE;
  *x = u->x;
  return GM_OK;
}

int gm_unet_forward(gm_unet* u, const uint16_t* const* w_bf16, const float* const* bias, const float* x, float* y,
                    void* stream) {
  if (!u || !w_bf16 || !bias) return GM_EVALUE;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    if (x && x != u->x) UN_CK(cudaMemcpyAsync(u->x, x, (size_t)u->B * 2 * u->plane(0) * 4, cudaMemcpyDeviceToDevice, st));
    forward(u, reinterpret_cast<const __nv_bfloat16* const*>(w_bf16), bias, st);
    if (y) UN_CK(cudaMemcpyAsync(y, u->act[11], (size_t)u->B * u->plane(0) * 4, cudaMemcpyDeviceToDevice, st));
    UN_CK(cudaGetLastError());
  } catch (const std::exception& e) {
    u->err = e.what();
    return GM_ECUDA;
  }
  return GM_OK;
}

int gm_unet_backward(gm_unet* u, const uint16_t* const* w_bf16, const float* dy, float* const* dw, float* const* db,
                     void* stream) {
  if (!u || !w_bf16 || !dy || !dw || !db) return GM_EVALUE;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    UN_CK(cudaMemcpyAsync(u->g_act[11], dy, (size_t)u->B * u->plane(0) * 4, cudaMemcpyDeviceToDevice, st));
    backward(u, reinterpret_cast<const __nv_bfloat16* const*>(w_bf16), dw, db, st);
    UN_CK(cudaGetLastError());
  } catch (const std::exception& e) {
    u->err = e.what();
    return GM_ECUDA;
  }
  return GM_OK;
}

}  // extern "C"
