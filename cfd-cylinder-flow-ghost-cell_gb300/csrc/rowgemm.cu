// Row transforms of the FP32 mode's pressure inverse on the tensor cores (tcgen05, sm_103a).
//
// A row pass of the separable inverse (solver/rectangular_inverse.py:8-58: a DCT-IV, DST-III,
// DST-II or DST-IV along every row) is the product Y = X T^T of the rows X (rows x n) with the
// explicit n x n transform T.  T is formed on the host by running the FP64 FFT row pass on the
// rows of the identity, so this path applies exactly the transforms of the FFT path.
//
// Precision: split TF32.  T = T_hi + T_lo and X = X_hi + X_lo with every part rounded to TF32
// (11 significant bits), and Y = X_hi T_hi + X_hi T_lo + X_lo T_hi: three tcgen05 MMAs per
// k-step, each product exact in the FP32 accumulator; the dropped X_lo T_lo term and the
// representation error are about 2^-22 relative -- the accuracy of the FP32 FFT it replaces.
// The FP64 residual and the refinement sweeps around the inverse are unchanged.
//
// One CTA computes a 128 x 64 tile of Y with the accumulator in tensor memory (64 columns):
//   warp 8     TMA (cp.async.bulk.tensor): the raw 128 x 32 tile of X of every k block (and, in
//              the inverse pass, the same tile of the boundary-term table W), and the T_hi and
//              T_lo tiles (128-byte swizzle);
//   warps 0-7  split every raw tile into its TF32 parts (16 rows each) in the K-major
//              128-byte-swizzled layout the MMA reads; at the end each reads a 32 x 32 block of
//              the accumulator (tcgen05.ld), transposes it through shared memory and writes it
//              with coalesced row stores;
//   warp 9     allocates the tensor memory and issues the MMAs from one thread, committing
//              each stage back to its producers.
// Three MMA stages of 48 KB and two raw stages of 32 KB.  Every mbarrier wait gives up after
// two seconds of global time: the kernel then raises the device-wait gate (the step fails with
// an error), waits (bounded) for the copies and MMAs it issued, and frees its tensor memory.
//
// The inverse pass applies the boundary Schur term's spectral correction as it loads, with the
// arithmetic of the FFT pass: W holds the decay factors phi (rows < j0) and psi (rows > j1)
// around the band rows j0..j1, which the band solve writes into W itself; the loaded value is
// X - W * b0 (rows < j0), X - W (band rows) or X - W * b1 (rows > j1), where b0 and b1 are the
// first and last band rows.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "kernels.cuh"

namespace gmk {

namespace {

constexpr int BM = 128, BN = 64, BK = 32, STAGES = 3, RSTAGES = 2;
constexpr int CONV_WARPS = 8, TMA_WARP = CONV_WARPS, MMA_WARP = CONV_WARPS + 1;
constexpr int THREADS = (CONV_WARPS + 2) * 32;
constexpr int ROWS_PER_CONV = BM / CONV_WARPS;           // 16 rows of a raw tile per converter warp
constexpr uint32_t A_BYTES = BM * BK * 4;                // 16 KB per TF32 part
constexpr uint32_t B_BYTES = BN * BK * 4;                // 8 KB per TF32 part
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr uint32_t RAW_MAX = BM * BK * 8;                // raw tile: FP64 X, or FP32 X and FP32 W
constexpr uint32_t TMEM_COLS = BN;                       // FP32 accumulator, 128 lanes x 64 columns
constexpr int NMAX = 1024;                               // longest row (band rows b0, b1 staged whole)
constexpr unsigned long long WAIT_NS = 2000000000ull;    // bound of every mbarrier wait
constexpr int GATE_DEVICE_WAIT = 9;                      // gate id of a wait that ran out
constexpr uint32_t NBARS = 3 * STAGES + 2 * RSTAGES + 2;
constexpr size_t SMEM_BYTES =
    1024 + STAGES * STAGE_BYTES + RSTAGES * RAW_MAX + 2 * NMAX * 4 + 8 * NBARS + 16;
static_assert(SMEM_BYTES <= 226 * 1024, "row GEMM shared memory (with the gate's static word)");
static_assert(CONV_WARPS * 32 * 33 * 4 <= RSTAGES * RAW_MAX, "epilogue staging fits the raw ring");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// waits for the phase of the given parity to complete; false after WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const unsigned long long t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > WAIT_NS) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* tmap, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(tmap), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const void* tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}
// K-major operand tile with 128-byte swizzle: rows of 128 bytes, 8-row atoms of 1024 bytes
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused by swizzled K-major tiles)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: one 8-row atom
  d |= (uint64_t)1 << 46;             // descriptor version of sm_100 and later
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}
// instruction descriptor: kind::tf32, FP32 accumulator, A and B K-major, M = 128, N = 64
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// round to the 11 significant bits of TF32 (to nearest, ties away from zero)
__device__ __forceinline__ float tf32_round(float v) {
  return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
}
// v = hi + lo with hi and lo both TF32 (lo rounded too, so the MMA's truncation of its input
// mantissa drops nothing of it)
__device__ __forceinline__ void tf32_split(float v, float& hi, float& lo) {
  hi = tf32_round(v);
  lo = tf32_round(v - hi);
}
// byte offset of element (row r, k) of a 128 x 32 FP32 K-major swizzled tile
__device__ __forceinline__ uint32_t sw128_off(int r, int k) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + (k & 3) * 4);
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,"
      "%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// MODE 0: forward pass.  X = input rows (the FP32 residual or the FP64 right-hand side, zero off
//         the active set as every pressure right-hand side and residual here is); Y -> the FP32
//         spectrum (row pitch N).
// MODE 1: inverse pass.  X = spectrum minus the boundary-term correction; Y -> x = [x +] Y on the
//         active points, zero elsewhere (FP64).
template <int MODE, typename TI>
__global__ void __launch_bounds__(THREADS, 1) k_row_gemm(const __grid_constant__ CUtensorMap tmap_b,
                                                        const __grid_constant__ CUtensorMap tmap_x,
                                                        const __grid_constant__ CUtensorMap tmap_w, RowGemmArgs a) {
  extern __shared__ __align__(1024) unsigned char rg_smem[];
  constexpr uint32_t XBYTES = BM * BK * sizeof(TI);
  const bool corr = MODE == 1 && a.corr;
  const uint32_t raw_bytes = corr ? 2 * XBYTES : XBYTES;
  const uint32_t raw = smem_u32(rg_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  const uint32_t rbase = sbase + STAGES * STAGE_BYTES;          // raw ring
  const uint32_t bvec = rbase + RSTAGES * RAW_MAX;              // band rows b0, b1 (NMAX each)
  const uint32_t bars = bvec + 2 * NMAX * 4;                    // barriers
  auto full_a = [&](int s) { return bars + 8u * s; };
  auto full_b = [&](int s) { return bars + 8u * (STAGES + s); };
  auto empty = [&](int s) { return bars + 8u * (2 * STAGES + s); };
  auto raw_full = [&](int r) { return bars + 8u * (3 * STAGES + r); };
  auto raw_empty = [&](int r) { return bars + 8u * (3 * STAGES + RSTAGES + r); };
  const uint32_t done = bars + 8u * (3 * STAGES + 2 * RSTAGES);
  const uint32_t bvec_full = done + 8u;
  unsigned char* gsm = rg_smem + (sbase - raw);                 // generic pointer of sbase
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gsm + (bars + 8u * NBARS - sbase));
  const float* gbvec = reinterpret_cast<const float*>(gsm + (bvec - sbase));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int KB = (a.K + BK - 1) / BK;

  // set-up that reads nothing the previous kernel writes, before the dependent-launch wait
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_a(s), CONV_WARPS * 32);
      mbar_init(full_b(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int r = 0; r < RSTAGES; ++r) {
      mbar_init(raw_full(r), 1);
      mbar_init(raw_empty(r), CONV_WARPS * 32);
    }
    mbar_init(done, 1);
    mbar_init(bvec_full, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == TMA_WARP && lane == 0) {
    prefetch_tmap(&tmap_b);
    prefetch_tmap(&tmap_x);
    if (corr) prefetch_tmap(&tmap_w);
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  const bool open = gate_open(a.gate);  // waits for the previous kernel, then a block barrier
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);
  bool ok = true;
  if (open) {
    if (warp < CONV_WARPS) {
      // converters: lane = k within the block, the warp's 16 rows in turn
      if (corr && !mbar_wait(bvec_full, 0)) ok = false;
      for (int kb = 0; kb < KB && ok; ++kb) {
        const int s = kb % STAGES, r = kb % RSTAGES;
        if (!mbar_wait(raw_full(r), (kb / RSTAGES) & 1)) { ok = false; break; }
        if (kb >= STAGES && !mbar_wait(empty(s), ((kb / STAGES) & 1) ^ 1)) { ok = false; break; }
        const uint32_t ahi = sbase + s * STAGE_BYTES, alo = ahi + A_BYTES, src = rbase + r * RAW_MAX;
        float b0 = 0.0f, b1 = 0.0f;
        if (corr) {
          const int k = kb * BK + lane;
          if (k < a.K) {
            b0 = gbvec[k];
            b1 = gbvec[NMAX + k];
          }
        }
#pragma unroll 8
        for (int rr = 0; rr < ROWS_PER_CONV; ++rr) {
          const int rt = warp * ROWS_PER_CONV + rr;
          float v;
          if constexpr (sizeof(TI) == 8) {
            double d;
            asm volatile("ld.shared.f64 %0, [%1];" : "=d"(d) : "r"(src + (uint32_t)(rt * BK + lane) * 8u));
            v = f64_to_f32i(d);
          } else {
            asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(src + (uint32_t)(rt * BK + lane) * 4u));
          }
          if (corr) {
            float w;
            asm volatile("ld.shared.f32 %0, [%1];" : "=f"(w) : "r"(src + XBYTES + (uint32_t)(rt * BK + lane) * 4u));
            const int m = m0 + rt;  // warp-uniform
            v = m < a.j0 ? v - w * b0 : (m > a.j1 ? v - w * b1 : v - w);
          }
          float hi, lo;
          tf32_split(v, hi, lo);
          const uint32_t off = sw128_off(rt, lane);
          asm volatile("st.shared.f32 [%0], %1;" ::"r"(ahi + off), "f"(hi) : "memory");
          asm volatile("st.shared.f32 [%0], %1;" ::"r"(alo + off), "f"(lo) : "memory");
        }
        // the MMAs read the tile through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(raw_empty(r));
        mbar_arrive(full_a(s));
      }
    } else if (warp == TMA_WARP) {
      if (lane == 0) {
        int nraw = 0, nb = 0;
        if (corr) {
          mbar_expect_tx(bvec_full, (uint32_t)a.K * 8u);
          bulk_load(bvec, a.wcorr + (int64_t)a.j0 * a.K, (uint32_t)a.K * 4u, bvec_full);
          bulk_load(bvec + NMAX * 4, a.wcorr + (int64_t)a.j1 * a.K, (uint32_t)a.K * 4u, bvec_full);
        }
        // the raw X (and W) tile and the two parts of the transform tile of every k block
        for (int kb = 0; kb < KB && ok; ++kb) {
          const int s = kb % STAGES, r = kb % RSTAGES;
          if (kb >= RSTAGES && !mbar_wait(raw_empty(r), ((kb / RSTAGES) & 1) ^ 1)) { ok = false; break; }
          mbar_expect_tx(raw_full(r), raw_bytes);
          tma_load_2d(rbase + r * RAW_MAX, &tmap_x, kb * BK, m0, raw_full(r));
          if (corr) tma_load_2d(rbase + r * RAW_MAX + XBYTES, &tmap_w, kb * BK, m0, raw_full(r));
          ++nraw;
          if (kb >= STAGES && !mbar_wait(empty(s), ((kb / STAGES) & 1) ^ 1)) { ok = false; break; }
          const uint32_t bhi = sbase + s * STAGE_BYTES + 2 * A_BYTES, blo = bhi + B_BYTES;
          mbar_expect_tx(full_b(s), 2 * B_BYTES);
          tma_load_2d(bhi, &tmap_b, kb * BK, n0, full_b(s));
          tma_load_2d(blo, &tmap_b, kb * BK, a.np + n0, full_b(s));
          ++nb;
        }
        if (!ok) {
          // copies still in flight land before the block leaves: wait (bounded) for the last
          // phase armed on every stage
          for (int r = 0; r < RSTAGES && r < nraw; ++r) {
            const int last = nraw - 1 - ((nraw - 1 - r) % RSTAGES);
            mbar_wait(raw_full(last % RSTAGES), (last / RSTAGES) & 1);
          }
          for (int s = 0; s < STAGES && s < nb; ++s) {
            const int last = nb - 1 - ((nb - 1 - s) % STAGES);
            mbar_wait(full_b(last % STAGES), (last / STAGES) & 1);
          }
          if (corr) mbar_wait(bvec_full, 0);
        }
      }
    } else {
      if (lane == 0) {
        for (int kb = 0; kb < KB && ok; ++kb) {
          const int s = kb % STAGES;
          const uint32_t ph = (kb / STAGES) & 1;
          if (!mbar_wait(full_a(s), ph) || !mbar_wait(full_b(s), ph)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t ahi = sbase + s * STAGE_BYTES, alo = ahi + A_BYTES, bhi = alo + A_BYTES, blo = bhi + B_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 8; ++kk) {
            const uint32_t o = kk * 32;  // 8 TF32 values of K per MMA
            mma_tf32(tmem, sw128_desc(ahi + o), sw128_desc(bhi + o), (kb | kk) != 0);
            mma_tf32(tmem, sw128_desc(ahi + o), sw128_desc(blo + o), 1u);
            mma_tf32(tmem, sw128_desc(alo + o), sw128_desc(bhi + o), 1u);
          }
          mma_commit(empty(s));
        }
        // arrives once every MMA issued above has completed (also after a failed wait)
        mma_commit(done);
      }
    }
    if (warp < CONV_WARPS) {
      // the accumulator (and, after a failure, the end of the MMAs still reading shared memory)
      const bool fin = mbar_wait(done, 0);
      if (ok && !fin) ok = false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (ok) {
        // warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows) and columns 32 (w / 4) .. +31,
        // transposes the block through its own part of the (now idle) raw ring, and writes
        // each tile row with one coalesced store per warp
        const int quarter = warp & 3, half = warp >> 2;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * 32), v);
        const uint32_t stg = rbase + (uint32_t)warp * (32 * 33 * 4);
#pragma unroll
        for (int i = 0; i < 32; ++i)
          asm volatile("st.shared.f32 [%0], %1;" ::"r"(stg + (uint32_t)(lane * 33 + i) * 4u), "f"(v[i]) : "memory");
        __syncwarp();
        const int n = n0 + half * 32 + lane;
        const bool nok = n < a.N;
        if (MODE == 0) {
#pragma unroll 4
          for (int rr = 0; rr < 32; ++rr) {
            const int m = m0 + quarter * 32 + rr;
            if (m >= a.M) break;
            float y;
            asm volatile("ld.shared.f32 %0, [%1];" : "=f"(y) : "r"(stg + (uint32_t)(rr * 33 + lane) * 4u));
            if (nok) a.sout[(int64_t)m * a.N + n] = y;
          }
        } else {
          // loads of the class map and the added field first (8 rows in flight), then the stores
          for (int r0 = 0; r0 < 32; r0 += 8) {
            uint8_t mk[8];
            double ad[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int m = m0 + quarter * 32 + r0 + u;
              mk[u] = 0;
              ad[u] = 0.0;
              if (m < a.M && nok) {
                const int64_t o = a.obase + (int64_t)m * a.opitch + n;
                mk[u] = a.ocls ? a.ocls[o] : (uint8_t)CLS_ACTIVE;
                if (a.add) ad[u] = a.add[o];
              }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int m = m0 + quarter * 32 + r0 + u;
              if (m >= a.M || !nok) continue;
              const int64_t o = a.obase + (int64_t)m * a.opitch + n;
              float y;
              asm volatile("ld.shared.f32 %0, [%1];" : "=f"(y) : "r"(stg + (uint32_t)((r0 + u) * 33 + lane) * 4u));
              a.xout[o] = !(mk[u] & CLS_ACTIVE) ? 0.0 : (a.add ? ad[u] + f32_to_f64i(y) : f32_to_f64i(y));
            }
          }
        }
      }
    }
    if (!ok && a.gate.ctl) raise_gate(a.gate.ctl, 4, GATE_DEVICE_WAIT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    cudaGetLastError();
  }
  return fn;
}

float tf32_round_host(double v) {
  float f = (float)v;
  uint32_t b;
  std::memcpy(&b, &f, 4);
  b = (b + 0x1000u) & 0xFFFFE000u;
  std::memcpy(&f, &b, 4);
  return f;
}

bool encode_2d(void* out, CUtensorMapDataType type, size_t esize, void* base, int inner, int outer, int64_t pitch,
               int box_inner, int box_outer, CUtensorMapSwizzle sw) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * esize};
  const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  const cuuint32_t estr[2] = {1, 1};
  return enc(reinterpret_cast<CUtensorMap*>(out), type, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of the raw tiles of an array of `rows` rows of n values (row pitch n), cached per
// array; nullptr when none can be made (the caller keeps the FFT pass).
const void* row_gemm_amap(RowGemm& g, const void* ptr, int esize) {
  for (int i = 0; i < g.namap; ++i)
    if (g.aptr[i] == ptr && g.aesz[i] == esize) return g.amap[i];
  if (!ptr || g.namap >= RowGemm::AMAPS || (reinterpret_cast<uintptr_t>(ptr) & 15)) return nullptr;
  const int i = g.namap;
  if (!encode_2d(g.amap[i], esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, esize,
                 const_cast<void*>(ptr), g.n, g.rows, g.n, BK, BM, CU_TENSOR_MAP_SWIZZLE_NONE))
    return nullptr;
  g.aptr[i] = ptr;
  g.aesz[i] = esize;
  ++g.namap;
  return g.amap[i];
}

}  // namespace

size_t row_gemm_smem_bytes() { return SMEM_BYTES; }

bool row_gemm_ready(RowGemm& g, const void* ptr, int esize) { return g.n > 0 && row_gemm_amap(g, ptr, esize); }

void row_gemm_free(RowGemm& g) {
  if (g.mats) cudaFree(g.mats);
  g.mats = nullptr;
  g.n = 0;
  g.namap = 0;
}

// t[k * n + i]: output i of the transform of the unit vector e_k, for the forward (tfwd) and the
// inverse (tinv) pass.  The B operand of a direction is T with rows i (outputs) and columns k,
// stored as [T_hi; T_lo] (2 np rows of kp floats, zero padded) under one tensor map.  Needs n a
// multiple of 4 (row pitch of the TMA-loaded arrays a multiple of 16 bytes) and n <= 1024.
// Returns 0 when built, 1 when this path is unavailable (the caller keeps the FFT passes).
int row_gemm_build(RowGemm& g, int n, int rows, const double* tfwd, const double* tinv, size_t smem_optin,
                   cudaStream_t st) {
  row_gemm_free(g);
  if (n % 4 || n > NMAX || rows <= 0 || SMEM_BYTES > smem_optin || !encode_fn()) return 1;
  const void* ks[3] = {(const void*)k_row_gemm<0, float>, (const void*)k_row_gemm<0, double>,
                       (const void*)k_row_gemm<1, float>};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
  const int np = (n + BN - 1) / BN * BN, kp = (n + BK - 1) / BK * BK;
  const size_t per = (size_t)2 * np * kp;
  std::vector<float> host(2 * per, 0.0f);
  for (int d = 0; d < 2; ++d) {
    const double* t = d == 0 ? tfwd : tinv;
    float* hi = host.data() + d * per;
    float* lo = hi + (size_t)np * kp;
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) {
        const double v = t[(size_t)k * n + i];
        const float h = tf32_round_host(v);
        hi[(size_t)i * kp + k] = h;
        lo[(size_t)i * kp + k] = tf32_round_host(v - (double)h);
      }
  }
  if (cudaMalloc(&g.mats, host.size() * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    g.mats = nullptr;
    return 1;
  }
  if (cudaMemcpyAsync(g.mats, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    row_gemm_free(g);
    return 1;
  }
  static_assert(sizeof(CUtensorMap) <= sizeof(g.tmap[0]), "tensor map storage");
  for (int d = 0; d < 2; ++d)
    if (!encode_2d(g.tmap[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g.mats + d * per, kp, 2 * np, kp, BK, BN,
                   CU_TENSOR_MAP_SWIZZLE_128B)) {
      row_gemm_free(g);
      return 1;
    }
  g.n = n;
  g.rows = rows;
  g.np = np;
  g.kp = kp;
  return 0;
}

template <typename TI>
bool launch_row_gemm_fwd(RowGemm& g, const TI* in, float* spec, const Gate& gate, cudaStream_t st) {
  if (!g.n) return false;
  const void* am = row_gemm_amap(g, in, (int)sizeof(TI));
  if (!am) return false;
  RowGemmArgs a{};
  a.M = g.rows;
  a.N = a.K = g.n;
  a.np = g.np;
  a.sout = spec;
  a.gate = gate;
  const dim3 grid((unsigned)(g.np / BN), (unsigned)((g.rows + BM - 1) / BM));
  note_launch_ext();
  kt_mark_ext(12, st, 0.0);
  launch_pdl_ext(k_row_gemm<0, TI>, grid, dim3(THREADS), SMEM_BYTES, st,
                 *reinterpret_cast<const CUtensorMap*>(g.tmap[0]), *reinterpret_cast<const CUtensorMap*>(am),
                 *reinterpret_cast<const CUtensorMap*>(am), a);
  // algorithmic bytes: the input rows read once, the spectrum written once
  kt_mark_ext(12, st, (double)g.rows * g.n * (sizeof(TI) + 4));
  return true;
}
template bool launch_row_gemm_fwd<float>(RowGemm&, const float*, float*, const Gate&, cudaStream_t);
template bool launch_row_gemm_fwd<double>(RowGemm&, const double*, float*, const Gate&, cudaStream_t);

bool launch_row_gemm_inv(RowGemm& g, const float* spec, const float* wcorr, int j0, int j1, double* x, int64_t obase,
                         int64_t opitch, const uint8_t* ocls, const double* add, const Gate& gate, cudaStream_t st) {
  if (!g.n) return false;
  const void* am = row_gemm_amap(g, spec, 4);
  if (!am) return false;
  const bool corr = wcorr && j0 <= j1 && j0 >= 0 && j1 < g.rows;
  const void* wm = corr ? row_gemm_amap(g, wcorr, 4) : am;
  if (!wm) return false;
  RowGemmArgs a{};
  a.M = g.rows;
  a.N = a.K = g.n;
  a.np = g.np;
  a.xout = x;
  a.obase = obase;
  a.opitch = opitch;
  a.ocls = ocls;
  a.add = add;
  a.wcorr = wcorr;
  a.corr = corr ? 1 : 0;
  a.j0 = j0;
  a.j1 = j1;
  a.gate = gate;
  const dim3 grid((unsigned)(g.np / BN), (unsigned)((g.rows + BM - 1) / BM));
  note_launch_ext();
  kt_mark_ext(12, st, 0.0);
  launch_pdl_ext(k_row_gemm<1, float>, grid, dim3(THREADS), SMEM_BYTES, st,
                 *reinterpret_cast<const CUtensorMap*>(g.tmap[1]), *reinterpret_cast<const CUtensorMap*>(am),
                 *reinterpret_cast<const CUtensorMap*>(wm), a);
  // algorithmic bytes: the spectrum (and the correction table) read, the class map read, x read
  // (when accumulating) and written
  kt_mark_ext(12, st, (double)g.rows * g.n * (4 + (corr ? 4 : 0) + (ocls ? 1 : 0) + (add ? 16 : 8)));
  return true;
}

}  // namespace gmk
