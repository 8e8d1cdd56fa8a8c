// Real-to-real DCT/DST line transforms on shared memory for sm_103a.
//
// Every transform is reduced to a complex FFT (mixed-radix Stockham, natural
// order) with pre/post twiddles:
//   DCT-II  : Makhoul reordering, n-point complex FFT, two real lines packed
//             as real/imaginary parts of one FFT.
//   DCT-III : inverse of the above (Hermitian spectrum, inverse FFT, two lines).
//   DCT-IV  : n/2-point complex FFT of (x[2m] + i x[n-1-2m]) with twiddles.
//   DST-I   : odd extension, 2(n+1)-point complex FFT, two lines packed.
//   DST-II/III/IV: DCT-II/III/IV with sign flips and reversals.
// All transforms are unnormalised like scipy.fft with norm=None; the
// caller folds the 1/(2n) factors into its eigenvalue table.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gmk {

enum R2R : int { DCT2 = 0, DCT3 = 1, DCT4 = 2, DST1 = 3, DST2 = 4, DST3 = 5, DST4 = 6 };

// family of the complex FFT that carries a transform
__host__ __device__ inline int r2r_family(int t) {
  switch (t) {
    case DCT2: case DST2: return 0;  // Makhoul forward, paired lines, M = n
    case DCT3: case DST3: return 1;  // Makhoul inverse, paired lines, M = n
    case DCT4: case DST4: return 2;  // type IV, single line, M = n/2
    default: return 3;               // DST-I, paired lines, M = 2(n+1)
  }
}
__host__ __device__ inline int r2r_fft_length(int t, int n) {
  int f = r2r_family(t);
  return f == 2 ? n / 2 : (f == 3 ? 2 * (n + 1) : n);
}
__host__ __device__ inline bool r2r_paired(int t) { return r2r_family(t) != 2; }

template <typename T> struct cplx { T x, y; };

// The threads that cooperate on a set of lines: one warp (barrier __syncwarp), or a
// group of whole warps synchronised by the named barrier `bar` (1..15) over n threads.
// tid/n index the group's threads.
struct Grp {
  int tid, n, bar;
  __device__ __forceinline__ void sync() const {
    if (n == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(n) : "memory");
  }
};

template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) { return {a.x - b.x, a.y - b.y}; }

// FFT plan for one length: radices in stage order and the twiddle table
// W[t] = exp(-2*pi*i*t/M) (T precision), t < M.
struct FftPlan {
  int M;
  int nstages;
  int radix[20];
  unsigned ns_magic[20];  // ceil(2^32 / Ns) of stage s (Ns = product of the earlier radices; 0 when Ns = 1)
  int tw_off[20];         // offset of stage s's twiddles in the plan's twiddle table
  int tw_len;             // length (complex entries) of the plan's twiddle table
};
// The plan's twiddle table: for a radix-R stage (R in 2, 3, 4, 5, 8) the Ns x (R-1) entries
// W_M^(r k M/(Ns R)), k < Ns, r = 1..R-1, stored k-major so that one butterfly reads R-1
// consecutive entries; for any other radix the full table W_M^t, t < M.

// One radix-R butterfly on v[0..R) in place; dir = -1 forward, +1 inverse.
template <typename T, int R>
__device__ __forceinline__ void dft_small(cplx<T>* v, int dir);

template <typename T>
__device__ __forceinline__ void bfly2(cplx<T>& a, cplx<T>& b) {
  cplx<T> t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <typename T, int R>
__device__ __forceinline__ void dft_small(cplx<T>* v, int dir) {
  if constexpr (R == 2) {
    bfly2(v[0], v[1]);
  } else if constexpr (R == 3) {
    const T c = (T)-0.5, s = (T)dir * (T)0.86602540378443864676372317075294;
    cplx<T> a = v[0], b = v[1], d = v[2];
    cplx<T> sum = cadd(b, d), dif = csub(b, d);
    v[0] = cadd(a, sum);
    cplx<T> m = {a.x + c * sum.x, a.y + c * sum.y};
    cplx<T> r = {-s * dif.y, s * dif.x};
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
  } else if constexpr (R == 4) {
    cplx<T> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    cplx<T> b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
    // b1 * (dir * i)
    cplx<T> b1r = {-(T)dir * b1.y, (T)dir * b1.x};
    v[0] = cadd(a0, b0);
    v[2] = csub(a0, b0);
    v[1] = cadd(a1, b1r);
    v[3] = csub(a1, b1r);
  } else if constexpr (R == 5) {
    const T c1 = (T)0.30901699437494742410229341718282, c2 = (T)-0.80901699437494742410229341718282;
    const T s1 = (T)dir * (T)0.95105651629515357211643933337938, s2 = (T)dir * (T)0.58778525229247312916870595463907;
    cplx<T> a = v[0];
    cplx<T> p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]);
    cplx<T> p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
    v[0] = {a.x + p1.x + p2.x, a.y + p1.y + p2.y};
    cplx<T> q1 = {a.x + c1 * p1.x + c2 * p2.x, a.y + c1 * p1.y + c2 * p2.y};
    cplx<T> q2 = {a.x + c2 * p1.x + c1 * p2.x, a.y + c2 * p1.y + c1 * p2.y};
    // i * (s1 m1 + s2 m2), i * (s2 m1 - s1 m2)
    cplx<T> r1 = {-(s1 * m1.y + s2 * m2.y), s1 * m1.x + s2 * m2.x};
    cplx<T> r2 = {-(s2 * m1.y - s1 * m2.y), s2 * m1.x - s1 * m2.x};
    v[1] = cadd(q1, r1);
    v[4] = csub(q1, r1);
    v[2] = cadd(q2, r2);
    v[3] = csub(q2, r2);
  } else if constexpr (R == 8) {
    const T h = (T)0.70710678118654752440084436210485;
    // radix-2 over stride 4
    bfly2(v[0], v[4]); bfly2(v[1], v[5]); bfly2(v[2], v[6]); bfly2(v[3], v[7]);
    // twiddles w8^k on v[5], v[6], v[7] (w8 = exp(dir*i*pi/4))
    cplx<T> t5 = v[5];
    v[5] = {h * (t5.x - (T)dir * t5.y), h * (t5.y + (T)dir * t5.x)};
    cplx<T> t6 = v[6];
    v[6] = {-(T)dir * t6.y, (T)dir * t6.x};
    cplx<T> t7 = v[7];
    v[7] = {h * (-t7.x - (T)dir * t7.y), h * (-t7.y + (T)dir * t7.x)};
    // two radix-4 on (0,1,2,3) and (4,5,6,7) with natural-order interleave
    cplx<T> a[4] = {v[0], v[1], v[2], v[3]}, b[4] = {v[4], v[5], v[6], v[7]};
    dft_small<T, 4>(a, dir);
    dft_small<T, 4>(b, dir);
    v[0] = a[0]; v[2] = a[1]; v[4] = a[2]; v[6] = a[3];
    v[1] = b[0]; v[3] = b[1]; v[5] = b[2]; v[7] = b[3];
  }
}

// j / Ns for j < 2^16 and Ns <= 2^16 by one high multiply: floor(j * ceil(2^32/Ns) / 2^32)
// is exact there (the error term j * e / (Ns 2^32) stays below 1/Ns).
__device__ __forceinline__ int div_ns(int j, int Ns, unsigned magic) {
  return Ns == 1 ? j : (int)__umulhi((unsigned)j, magic);
}

// One Stockham stage for radix R and direction DIR (compile-time) over nfft transforms of
// length M; tw is this stage's twiddle table (k-major, R-1 entries per k).
template <typename T, int R, int DIR>
__device__ __forceinline__ void stage_fixed(const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out, int M,
                                            int nfft, int Ns, unsigned magic, const cplx<T>* __restrict__ tw,
                                            const Grp& G) {
  const int MR = M / R;
  for (int f = 0; f < nfft; ++f) {
    const cplx<T>* src = in + (size_t)f * M;
    cplx<T>* dst = out + (size_t)f * M;
    for (int j = G.tid; j < MR; j += G.n) {
      const int jq = div_ns(j, Ns, magic);
      const int k = j - jq * Ns;
      const cplx<T>* w = tw + k * (R - 1);
      cplx<T> v[R];
      v[0] = src[j];
#pragma unroll
      for (int r = 1; r < R; ++r) {
        cplx<T> ww = w[r - 1];
        if (DIR > 0) ww.y = -ww.y;
        v[r] = cmul(src[j + r * MR], ww);
      }
      dft_small<T, R>(v, DIR);
      const int base = jq * Ns * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) dst[base + q * Ns] = v[q];
    }
  }
}

// Generic odd radix (any R up to 64): direct R-point DFT per output; W is the full table.
template <typename T>
__device__ void stage_generic(const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out, int M, int nfft, int Ns,
                              unsigned magic, int R, const cplx<T>* __restrict__ W, int dir, const Grp& G) {
  const int MR = M / R;
  const int tws = M / (Ns * R);
  for (int f = 0; f < nfft; ++f) {
    const cplx<T>* src = in + (size_t)f * M;
    cplx<T>* dst = out + (size_t)f * M;
    for (int t = G.tid; t < MR * R; t += G.n) {
      const int j = t / R, q = t - j * R;
      const int jq = div_ns(j, Ns, magic);
      const int k = j - jq * Ns;
      cplx<T> acc = {0, 0};
      for (int r = 0; r < R; ++r) {
        cplx<T> a = src[j + r * MR];
        // combined twiddle exp(dir*2*pi*i*(r*k/(Ns R) + r*q/R)) = W[(r*k*tws + ((r*q)%R)*MR) % M]
        int e = (r * k * tws + ((r * q) % R) * MR) % M;
        cplx<T> w = W[e];
        if (dir > 0) w.y = -w.y;
        cplx<T> p = cmul(a, w);
        acc.x += p.x;
        acc.y += p.y;
      }
      dst[jq * Ns * R + k + q * Ns] = acc;
    }
  }
}

template <typename T, int DIR>
__device__ cplx<T>* fft_run_dir(cplx<T>* a, cplx<T>* b, const FftPlan& plan, int nfft, const cplx<T>* tw,
                               const Grp& G) {
  int Ns = 1;
  for (int s = 0; s < plan.nstages; ++s) {
    const int R = plan.radix[s];
    const unsigned mg = plan.ns_magic[s];
    const cplx<T>* ts = tw + plan.tw_off[s];
    switch (R) {
      case 2: stage_fixed<T, 2, DIR>(a, b, plan.M, nfft, Ns, mg, ts, G); break;
      case 3: stage_fixed<T, 3, DIR>(a, b, plan.M, nfft, Ns, mg, ts, G); break;
      case 4: stage_fixed<T, 4, DIR>(a, b, plan.M, nfft, Ns, mg, ts, G); break;
      case 5: stage_fixed<T, 5, DIR>(a, b, plan.M, nfft, Ns, mg, ts, G); break;
      case 8: stage_fixed<T, 8, DIR>(a, b, plan.M, nfft, Ns, mg, ts, G); break;
      default: stage_generic<T>(a, b, plan.M, nfft, Ns, mg, R, ts, DIR, G); break;
    }
    G.sync();
    cplx<T>* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// Runs the FFT on nfft transforms held in a (length M each); the result is in
// the returned buffer (a or b).  dir = -1 forward, +1 inverse (unnormalised).
template <typename T>
__device__ cplx<T>* fft_run(cplx<T>* a, cplx<T>* b, const FftPlan& plan, int nfft, const cplx<T>* tw, int dir,
                           const Grp& G) {
  return dir > 0 ? fft_run_dir<T, 1>(a, b, plan, nfft, tw, G) : fft_run_dir<T, -1>(a, b, plan, nfft, tw, G);
}

// Twiddle tables of one r2r transform of length n (T precision), device pointers.
template <typename T>
struct R2RTables {
  const cplx<T>* W;     // the plan's twiddle table (FftPlan)
  const cplx<T>* pre;   // type IV: exp(-i pi (4m+1)/(4n)), m < n/2
  const cplx<T>* post;  // DCT-II/III: (cos, sin)(pi k/(2n)), k < n; type IV: exp(-i pi k/n), k < n/2
};

// ---------------------------------------------------------------------------
// pre-processing: nl real lines of length n -> complex FFT inputs in buf.  x(l, i) gives
// element i of line l (the caller reads it from global memory with its masks, so the lines go
// to the FFT buffer without a staging pass); #pragma unroll keeps several lines' loads in
// flight per thread.
// ---------------------------------------------------------------------------
template <typename T, typename X>
__device__ __forceinline__ void r2r_pre(int type, int n, int nl, cplx<T>* buf, const R2RTables<T>& tb, const Grp& G,
                                        X&& x) {
  const int fam = r2r_family(type);
  if (fam == 2) {
    const int M = n / 2;
    const bool rev = type == DST4;
    for (int l = 0; l < nl; ++l) {
#pragma unroll 4
      for (int m = G.tid; m < M; m += G.n) {
        int i0 = 2 * m, i1 = n - 1 - 2 * m;
        T a = x(l, rev ? n - 1 - i0 : i0);
        T b = x(l, rev ? n - 1 - i1 : i1);
        cplx<T> w = tb.pre[m];
        buf[(size_t)l * M + m] = {a * w.x - b * w.y, b * w.x + a * w.y};
      }
    }
  } else if (fam == 0) {
    // Makhoul: v[m] = x[2m] (m < ceil(n/2)), v[n-1-m'] = x[2m'+1]
    const int npair = (nl + 1) / 2;
    const bool alt = type == DST2;  // DST-II: x'[m] = (-1)^m x[m]
    for (int pidx = 0; pidx < npair; ++pidx) {
#pragma unroll 4
      for (int m = G.tid; m < n; m += G.n) {
        int src = m < (n + 1) / 2 ? 2 * m : 2 * (n - 1 - m) + 1;
        T sgn = (alt && (src & 1)) ? (T)-1 : (T)1;
        int la = 2 * pidx, lb = 2 * pidx + 1;
        T a = sgn * x(la, src);
        T b = lb < nl ? sgn * x(lb, src) : (T)0;
        buf[(size_t)pidx * n + m] = {a, b};
      }
    }
  } else if (fam == 1) {
    // V[k] = e^{i pi k/(2n)} (X_k - i X_{n-k}), X_n = 0; two lines as V_A + i V_B
    const int npair = (nl + 1) / 2;
    const bool rev = type == DST3;  // DST-III: X'[k] = X[n-1-k]
    for (int pidx = 0; pidx < npair; ++pidx) {
#pragma unroll 4
      for (int k = G.tid; k < n; k += G.n) {
        int la = 2 * pidx, lb = 2 * pidx + 1;
        int ik = rev ? n - 1 - k : k;
        int ir = rev ? k - 1 : n - k;  // index of X_{n-k} in the stored line (valid when k > 0)
        cplx<T> cs = tb.post[k];       // (cos, sin)(pi k / (2n))
        T ak = x(la, ik);
        T ar = k > 0 ? x(la, ir) : (T)0;
        T bk = lb < nl ? x(lb, ik) : (T)0;
        T br = (lb < nl && k > 0) ? x(lb, ir) : (T)0;
        cplx<T> VA = {cs.x * ak + cs.y * ar, cs.y * ak - cs.x * ar};
        cplx<T> VB = {cs.x * bk + cs.y * br, cs.y * bk - cs.x * br};
        buf[(size_t)pidx * n + k] = {VA.x - VB.y, VA.y + VB.x};
      }
    }
  } else {
    // DST-I: odd extension of length 2(n+1)
    const int N = n + 1, M = 2 * N;
    const int npair = (nl + 1) / 2;
    for (int t = G.tid; t < npair * M; t += G.n) {
      int pidx = t / M, m = t - pidx * M;
      int la = 2 * pidx, lb = 2 * pidx + 1;
      cplx<T> z = {0, 0};
      if (m >= 1 && m <= n) {
        z.x = x(la, m - 1);
        z.y = lb < nl ? x(lb, m - 1) : (T)0;
      } else if (m >= N + 1) {
        int src = n - 1 - (m - N - 1);
        z.x = -x(la, src);
        z.y = lb < nl ? -x(lb, src) : (T)0;
      }
      buf[(size_t)pidx * M + m] = z;
    }
  }
}

// post-processing: FFT outputs in buf -> real lines in stage
template <typename T>
__device__ void r2r_post(int type, const cplx<T>* buf, int n, int nl, T* stage, const R2RTables<T>& tb, const Grp& G) {
  const int fam = r2r_family(type);
  if (fam == 2) {
    const int M = n / 2;
    const bool alt = type == DST4;  // y[k] *= (-1)^k
    for (int l = 0; l < nl; ++l)
    for (int k = G.tid; k < M; k += G.n) {
      cplx<T> z = cmul(buf[(size_t)l * M + k], tb.post[k]);
      T* y = stage + (size_t)l * n;
      int k0 = 2 * k, k1 = n - 1 - 2 * k;
      T y0 = (T)2 * z.x, y1 = (T)-2 * z.y;
      if (alt) {
        if (k0 & 1) y0 = -y0;
        if (k1 & 1) y1 = -y1;
      }
      y[k0] = y0;
      y[k1] = y1;
    }
  } else if (fam == 0) {
    const int npair = (nl + 1) / 2;
    const bool rev = type == DST2;  // DST-II: y[k] = Y'[n-1-k]
    for (int pidx = 0; pidx < npair; ++pidx)
    for (int k = G.tid; k < n; k += G.n) {
      cplx<T> Zk = buf[(size_t)pidx * n + k];
      cplx<T> Zc = buf[(size_t)pidx * n + (k == 0 ? 0 : n - k)];
      Zc.y = -Zc.y;
      cplx<T> cs = tb.post[k];
      cplx<T> s = cadd(Zk, Zc), d = csub(Zk, Zc);
      // Va = s/2, Vb = (d.y/2, -d.x/2); y = 2 (c Re + s Im)
      T ya = cs.x * s.x + cs.y * s.y;
      T yb = cs.x * d.y - cs.y * d.x;
      int out = rev ? n - 1 - k : k;
      int la = 2 * pidx, lb = 2 * pidx + 1;
      stage[(size_t)la * n + out] = ya;
      if (lb < nl) stage[(size_t)lb * n + out] = yb;
    }
  } else if (fam == 1) {
    const int npair = (nl + 1) / 2;
    const bool alt = type == DST3;  // DST-III: y[m] *= (-1)^m
    for (int pidx = 0; pidx < npair; ++pidx)
    for (int o = G.tid; o < n; o += G.n) {
      int src = (o & 1) ? n - 1 - (o - 1) / 2 : o / 2;
      cplx<T> z = buf[(size_t)pidx * n + src];
      T sgn = (alt && (o & 1)) ? (T)-1 : (T)1;
      int la = 2 * pidx, lb = 2 * pidx + 1;
      stage[(size_t)la * n + o] = sgn * z.x;
      if (lb < nl) stage[(size_t)lb * n + o] = sgn * z.y;
    }
  } else {
    const int N = n + 1, M = 2 * N;
    const int npair = (nl + 1) / 2;
    for (int t = G.tid; t < npair * n; t += G.n) {
      int pidx = t / n, k = t - pidx * n;
      cplx<T> z = buf[(size_t)pidx * M + k + 1];
      int la = 2 * pidx, lb = 2 * pidx + 1;
      stage[(size_t)la * n + k] = -z.y;
      if (lb < nl) stage[(size_t)lb * n + k] = z.x;
    }
  }
}

// Complex buffer length (elements) needed for nl lines of one transform.
__host__ __device__ inline int r2r_buffer_elems(int type, int n, int nl) {
  int M = r2r_fft_length(type, n);
  int nfft = r2r_paired(type) ? (nl + 1) / 2 : nl;
  return M * nfft;
}
__host__ __device__ inline int r2r_nfft(int type, int nl) { return r2r_paired(type) ? (nl + 1) / 2 : nl; }

// Full r2r transform of nl lines read through x(l, i) (see r2r_pre), through the FFT buffers
// a/b; the real results are left line-major (l * n + i) in the buffer the FFT does not end in,
// which is returned.
template <typename T, typename X>
__device__ __forceinline__ T* r2r_lines(int type, int n, int nl, cplx<T>* a, cplx<T>* b, const FftPlan& plan,
                                        const R2RTables<T>& tb, const Grp& G, X&& x) {
  const int fam = r2r_family(type);
  r2r_pre<T>(type, n, nl, a, tb, G, x);
  G.sync();
  cplx<T>* res = fft_run<T>(a, b, plan, r2r_nfft(type, nl), tb.W, fam == 1 ? +1 : -1, G);
  T* out = reinterpret_cast<T*>(res == a ? b : a);
  r2r_post<T>(type, res, n, nl, out, tb, G);
  G.sync();
  return out;
}

}  // namespace gmk
