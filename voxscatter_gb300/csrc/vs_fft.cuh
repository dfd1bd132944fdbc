// Mixed-radix Stockham FFT over lines held in shared memory.
//
// One CTA transforms a batch of lines cooperatively.  Element p of line b lives
// at buf[b*ls + p*es]; `lines_fast` selects the butterfly-to-thread mapping so
// that consecutive threads touch consecutive shared-memory words (lines
// contiguous along x: lines_fast=false, es=1; lines strided across an x-tile:
// lines_fast=true, ls=1).  Each radix-R stage reads R points at stride n/R,
// twiddles them by w_n^(r*k*n/(Ns*R)) (k = j mod Ns), does an R-point DFT and
// writes them at (j-k)*R + k + q*Ns, ping-ponging between two buffers (the
// autosort form of Stockham; output in natural order, no bit reversal).
// Radices 2,3,4,5,8 have closed-form butterflies, 7/11/13 use the twiddle
// table at compile-time size, any other prime up to FFT_MAX_GENERIC_RADIX uses
// a runtime O(R^2) DFT.  Forward = exp(-2 pi i/n) (MATLAB fft), inverse =
// exp(+2 pi i/n) without the 1/n factor (folded elsewhere).
#pragma once
#include "vs_common.cuh"
#include <vector>
#include <cmath>

namespace vs {

constexpr int FFT_MAX_STAGES = 16;
constexpr int FFT_MAX_GENERIC_RADIX = 128;

struct FftPlan {
  int n = 1;
  int nstages = 0;
  int radix[FFT_MAX_STAGES] = {};
};

inline FftPlan make_fft_plan(int n) {
  FftPlan p;
  p.n = n;
  int m = n;
  const int pref[] = {9, 8, 6, 5, 4, 3, 2, 7, 11, 13};
  for (int r : pref) {
    while (m % r == 0) {
      VS_REQUIRE(p.nstages < FFT_MAX_STAGES, "FFT length has too many factors");
      p.radix[p.nstages++] = r;
      m /= r;
    }
  }
  for (int f = 17; m > 1; f += 2) {
    while (m % f == 0) {
      VS_REQUIRE(f <= FFT_MAX_GENERIC_RADIX,
                 "FFT length " + std::to_string(n) + " has a prime factor above 128");
      VS_REQUIRE(p.nstages < FFT_MAX_STAGES, "FFT length has too many factors");
      p.radix[p.nstages++] = f;
      m /= f;
    }
  }
  return p;
}

// exp(-2 pi i t / n), t = 0..n-1, in double (reduced to the first octant so the
// table is accurate to the last bit of a double).
inline std::vector<double> twiddle_table(int n) {
  std::vector<double> t(2 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    // angle = 2*pi*k/n ; use symmetric reduction via integer arithmetic
    long long num = (long long)k * 8;  // in units of (2*pi/8)/n
    double c, s;
    long long q = num / n;  // octant index 0..7
    double rem = (double)(num - q * n) / (double)n;  // fraction within the octant
    double a = rem * (M_PI / 4);
    double ca = std::cos(a), sa = std::sin(a);
    double cb = std::cos(M_PI / 4 - a), sb = std::sin(M_PI / 4 - a);
    switch (q) {
      case 0: c = ca; s = sa; break;
      case 1: c = sb; s = cb; break;
      case 2: c = -sa; s = ca; break;
      case 3: c = -cb; s = sb; break;
      case 4: c = -ca; s = -sa; break;
      case 5: c = -sb; s = -cb; break;
      case 6: c = sa; s = -ca; break;
      default: c = cb; s = -sb; break;
    }
    t[2 * k] = c;
    t[2 * k + 1] = -s;
  }
  return t;
}

// Smallest m >= n whose prime factors are all in {2,3,5}: lengths the
// small-radix kernels (radices 2,3,4,5,8 only) transform.
inline int smooth_size(int n) {
  for (int m = n > 1 ? n : 1;; ++m) {
    int r = m;
    for (int f : {2, 3, 5})
      while (r % f == 0) r /= f;
    if (r == 1) return m;
  }
}

inline bool plan_is_small_radix(const FftPlan& p) {
  for (int s = 0; s < p.nstages; ++s) {
    const int r = p.radix[s];
    if (!(r == 2 || r == 3 || r == 4 || r == 5 || r == 6 || r == 8 || r == 9)) return false;
  }
  return true;
}

#if defined(__CUDACC__) || defined(VS_FFT_HOST_EMULATION)

// Dynamic shared memory of the calling kernel, typed.  All FFT buffers and
// the twiddle table are addressed as 32-bit offsets into it, so every access
// is a shared-memory access.
template <typename C>
__device__ __forceinline__ C* shmem() {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  return reinterpret_cast<C*>(smem_raw);
}

// Twiddle w_n^idx (conjugated for the inverse) from the table in shared memory.
template <bool INV, typename C>
__device__ __forceinline__ C twid(const C* tw, int idx) {
  C w = tw[idx];
  if (INV) w.y = -w.y;
  return w;
}

// multiply by -i (forward) or +i (inverse) as the sign of the 4-point DFT needs
template <bool INV, typename C>
__device__ __forceinline__ C rot90(C a) {
  C r;
  if (INV) { r.x = -a.y; r.y = a.x; }
  else { r.x = a.y; r.y = -a.x; }
  return r;
}

template <int R, bool INV, typename C>
struct Butterfly;

template <bool INV, typename C>
struct Butterfly<2, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV, typename C>
struct Butterfly<4, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) {
    C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    C s13 = cadd(v[1], v[3]), d13 = rot90<INV>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};

template <bool INV, typename C>
struct Butterfly<8, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C* tw, int n) {
    using T = decltype(v[0].x);
    const T h = (T)0.70710678118654752440;
    C u[4], w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      u[k] = cadd(v[k], v[k + 4]);
      w[k] = csub(v[k], v[k + 4]);
    }
    // w[k] *= exp(-+ 2 pi i k / 8)
    {
      C a = w[1];
      // forward: (1 - i)/sqrt2 ; inverse: (1 + i)/sqrt2
      if (INV) { w[1].x = (a.x - a.y) * h; w[1].y = (a.x + a.y) * h; }
      else { w[1].x = (a.x + a.y) * h; w[1].y = (a.y - a.x) * h; }
      w[2] = rot90<INV>(w[2]);
      C b = w[3];
      // forward: (-1 - i)/sqrt2 ; inverse: (-1 + i)/sqrt2
      if (INV) { w[3].x = (-b.x - b.y) * h; w[3].y = (b.x - b.y) * h; }
      else { w[3].x = (b.y - b.x) * h; w[3].y = (-b.x - b.y) * h; }
    }
    Butterfly<4, INV, C>::run(u, tw, n);
    Butterfly<4, INV, C>::run(w, tw, n);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = u[q];
      v[2 * q + 1] = w[q];
    }
  }
};

template <bool INV, typename C>
struct Butterfly<3, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) {
    using T = decltype(v[0].x);
    const T s3 = INV ? (T)0.86602540378443864676 : (T)-0.86602540378443864676;
    C t1 = cadd(v[1], v[2]);
    C t2 = make_c(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
    C d = csub(v[1], v[2]);
    // i*s3*d
    C t3 = make_c(-s3 * d.y, s3 * d.x);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
  __device__ __forceinline__ static C make_c(decltype(C().x) a, decltype(C().x) b) { C c; c.x = a; c.y = b; return c; }
};

template <bool INV, typename C>
struct Butterfly<5, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) {
    using T = decltype(v[0].x);
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
    const T sg = INV ? (T)1 : (T)-1;
    const T s1 = sg * (T)0.95105651629515357212, s2 = sg * (T)0.58778525229247312917;
    C b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]);
    C d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
    C a0 = v[0];
    C r1, r2, i1, i2;
    r1.x = a0.x + c1 * b1.x + c2 * b2.x; r1.y = a0.y + c1 * b1.y + c2 * b2.y;
    r2.x = a0.x + c2 * b1.x + c1 * b2.x; r2.y = a0.y + c2 * b1.y + c1 * b2.y;
    // i*(s1 d1 + s2 d2) and i*(s2 d1 - s1 d2)
    T e1x = s1 * d1.x + s2 * d2.x, e1y = s1 * d1.y + s2 * d2.y;
    T e2x = s2 * d1.x - s1 * d2.x, e2y = s2 * d1.y - s1 * d2.y;
    i1.x = -e1y; i1.y = e1x;
    i2.x = -e2y; i2.y = e2x;
    v[0] = cadd(a0, cadd(b1, b2));
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
  }
};

// 6 = 3 x 2: three-point DFTs over n = 2*n1 + n2, twiddles w6^(n2*k1), then
// two-point DFTs; output k = k1 + 3*k2.
template <bool INV, typename C>
struct Butterfly<6, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C* tw, int n) {
    using T = decltype(v[0].x);
    C a[3] = {v[0], v[2], v[4]}, b[3] = {v[1], v[3], v[5]};
    Butterfly<3, INV, C>::run(a, tw, n);
    Butterfly<3, INV, C>::run(b, tw, n);
    const T h = (T)0.5, s3 = INV ? (T)0.86602540378443864676 : (T)-0.86602540378443864676;
    // b1 *= w6 = (1/2, s3) ; b2 *= w6^2 = (-1/2, s3)
    C t1, t2;
    t1.x = h * b[1].x - s3 * b[1].y; t1.y = h * b[1].y + s3 * b[1].x;
    t2.x = -h * b[2].x - s3 * b[2].y; t2.y = -h * b[2].y + s3 * b[2].x;
    v[0] = cadd(a[0], b[0]); v[3] = csub(a[0], b[0]);
    v[1] = cadd(a[1], t1); v[4] = csub(a[1], t1);
    v[2] = cadd(a[2], t2); v[5] = csub(a[2], t2);
  }
};

// 9 = 3 x 3: three-point DFTs over n = 3*n1 + n2, twiddles w9^(n2*k1), then
// three-point DFTs over n2; output k = k1 + 3*k2.
template <bool INV, typename C>
struct Butterfly<9, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C* tw, int n) {
    using T = decltype(v[0].x);
    C y[3][3];
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2) {
      y[n2][0] = v[n2]; y[n2][1] = v[3 + n2]; y[n2][2] = v[6 + n2];
      Butterfly<3, INV, C>::run(y[n2], tw, n);
    }
    const T sg = INV ? (T)1 : (T)-1;
    // w9^1, w9^2, w9^4
    const T c1 = (T)0.76604444311897803520, s1 = sg * (T)0.64278760968653932632;
    const T c2 = (T)0.17364817766693034885, s2 = sg * (T)0.98480775301220805936;
    const T c4 = (T)-0.93969262078590838405, s4 = sg * (T)0.34202014332566873304;
    auto rot = [](C a, T c, T s) { C r; r.x = a.x * c - a.y * s; r.y = a.x * s + a.y * c; return r; };
    y[1][1] = rot(y[1][1], c1, s1);
    y[1][2] = rot(y[1][2], c2, s2);
    y[2][1] = rot(y[2][1], c2, s2);
    y[2][2] = rot(y[2][2], c4, s4);
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      C z[3] = {y[0][k1], y[1][k1], y[2][k1]};
      Butterfly<3, INV, C>::run(z, tw, n);
      v[k1] = z[0]; v[k1 + 3] = z[1]; v[k1 + 6] = z[2];
    }
  }
};

// cos(2 pi j/R), sin(2 pi j/R) for j = 1..(R-1)/2 of the odd prime radices
// (constant-folded once the butterfly loops are unrolled).
template <int R> __host__ __device__ constexpr double odd_cos(int j);
template <int R> __host__ __device__ constexpr double odd_sin(int j);
template <> __host__ __device__ constexpr double odd_cos<7>(int j) {
  return j == 1 ? 0.62348980185873359439 : j == 2 ? -0.22252093395631433737 : -0.90096886790241903498;
}
template <> __host__ __device__ constexpr double odd_sin<7>(int j) {
  return j == 1 ? 0.78183148246802980363 : j == 2 ? 0.97492791218182361934 : 0.43388373911755823142;
}
template <> __host__ __device__ constexpr double odd_cos<11>(int j) {
  return j == 1 ? 0.84125353283118120551 : j == 2 ? 0.41541501300188643508 : j == 3 ? -0.14231483827328500480 : j == 4 ? -0.65486073394528498959 : -0.95949297361449736865;
}
template <> __host__ __device__ constexpr double odd_sin<11>(int j) {
  return j == 1 ? 0.54064081745559755543 : j == 2 ? 0.90963199535451833011 : j == 3 ? 0.98982144188093279524 : j == 4 ? 0.75574957435425826890 : 0.28173255684142967104;
}
template <> __host__ __device__ constexpr double odd_cos<13>(int j) {
  return j == 1 ? 0.88545602565320991051 : j == 2 ? 0.56806474673115592289 : j == 3 ? 0.12053668025532300601 : j == 4 ? -0.35460488704253545489 : j == 5 ? -0.74851074817110119231 : -0.97094181742605201180;
}
template <> __host__ __device__ constexpr double odd_sin<13>(int j) {
  return j == 1 ? 0.46472317204376850652 : j == 2 ? 0.82298386589365635224 : j == 3 ? 0.99270887409805397272 : j == 4 ? 0.93501624268541483342 : j == 5 ? 0.66312265824079519305 : 0.23931566428755768339;
}

// Odd prime R by symmetric pairs: with s_r = v_r + v_{R-r}, d_r = v_r - v_{R-r},
//   out[k], out[R-k] = v_0 + sum_r cos(2 pi rk/R) s_r  -/+  i sum_r sin(2 pi rk/R) d_r
// (signs swapped for the inverse): (R-1)^2 real multiply-adds per R points
// instead of (R-1)^2 complex ones.
template <int R, bool INV, typename C>
struct OddButterfly {
  __device__ __forceinline__ static void run(C* v) {
    using T = decltype(v[0].x);
    constexpr int h = (R - 1) / 2;
    C sp[h], dm[h];
    C sum = v[0];
#pragma unroll
    for (int r = 0; r < h; ++r) {
      sp[r] = cadd(v[r + 1], v[R - 1 - r]);
      dm[r] = csub(v[r + 1], v[R - 1 - r]);
      sum = cadd(sum, sp[r]);
    }
    C out[R];
    out[0] = sum;
#pragma unroll
    for (int k = 1; k <= h; ++k) {
      C re = v[0];
      T imx = 0, imy = 0;
#pragma unroll
      for (int r = 1; r <= h; ++r) {
        const int m = (r * k) % R;
        const T ct = (T)(m <= h ? odd_cos<R>(m) : odd_cos<R>(R - m));
        const T st = (T)(m <= h ? odd_sin<R>(m) : -odd_sin<R>(R - m));
        re.x += ct * sp[r - 1].x;
        re.y += ct * sp[r - 1].y;
        imx += st * dm[r - 1].x;
        imy += st * dm[r - 1].y;
      }
      // forward: out[k] = re - i*im, out[R-k] = re + i*im ; inverse: swapped
      C a, b;
      a.x = re.x + imy; a.y = re.y - imx;  // re - i*im
      b.x = re.x - imy; b.y = re.y + imx;  // re + i*im
      out[k] = INV ? b : a;
      out[R - k] = INV ? a : b;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = out[q];
  }
};

template <bool INV, typename C>
struct Butterfly<7, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) { OddButterfly<7, INV, C>::run(v); }
};
template <bool INV, typename C>
struct Butterfly<11, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) { OddButterfly<11, INV, C>::run(v); }
};
template <bool INV, typename C>
struct Butterfly<13, INV, C> {
  __device__ __forceinline__ static void run(C* v, const C*, int) { OddButterfly<13, INV, C>::run(v); }
};

// Compile-time-size DFT for the remaining small primes, roots read from the
// length-n twiddle table: w_R^k = tw[k*n/R].
template <int R, bool INV, typename C>
struct Butterfly {
  __device__ __forceinline__ static void run(C* v, const C* tw, int n) {
    C y[R];
    const int st = n / R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      C acc = v[0];
#pragma unroll
      for (int r = 1; r < R; ++r) acc = cfma(v[r], twid<INV>(tw, ((r * q) % R) * st), acc);
      y[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = y[q];
  }
};

// Thread layout of a CTA of kFftThreads threads over a batch of lines: NL =
// 2^lg_nl line slots times NJ = kFftThreads/NL butterfly slots.  With
// lines_fast, consecutive threads take consecutive line slots (lines
// interleaved in shared memory, ls = 1); otherwise consecutive threads take
// consecutive butterflies of one line (lines contiguous, es = 1).  Lines
// beyond NL are handled by the same slot in steps of NL.
constexpr int kFftThreads = 256;

struct FftLayout {
  int lg_nl;       // log2 of the number of line slots
  bool lines_fast; // see above
  __host__ __device__ int nl() const { return 1 << lg_nl; }
};

// One radix-R Stockham stage over all lines for thread `t`.
// Buffers are offsets (in elements) into the kernel's shared memory: src, dst
// and the twiddle table tw (n entries of exp(-2 pi i k/n)).
// Butterfly j of a line reads R points at stride m = n/R, applies the twiddles
// w_n^(r*k*n/(Ns*R)) with k = j mod Ns, and writes the R outputs at
// (j - k)*R + k + q*Ns.  j advances by NJ per iteration; (j div Ns, j mod Ns)
// are advanced incrementally, so there is one runtime division per stage.
template <int R, bool INV, typename C>
__device__ __forceinline__ void fft_stage(int src, int dst, int n, int Ns, int nlines, int ls, int es, FftLayout lay,
                                          int tw, int t) {
  C* sm = shmem<C>();
  const C* twp = sm + tw;
  const int lg_nl = lay.lg_nl;
  const int NL = 1 << lg_nl;
  const int lg_nj = 8 - lg_nl;  // kFftThreads = 256
  const int NJ = 1 << lg_nj;
  const int lslot = lay.lines_fast ? (t & (NL - 1)) : (t >> lg_nj);
  const int jt = lay.lines_fast ? (t >> lg_nl) : (t & (NJ - 1));
  const int m = n / R;
  if (jt >= m) return;
  const int step = n / (Ns * R);
  const int q0 = jt / Ns, k0 = jt - q0 * Ns;
  const int dq = NJ / Ns, dk = NJ - dq * Ns;
  const int me = m * es, nse = Ns * es, rnse = R * nse;
  for (int line = lslot; line < nlines; line += NL) {
    const int s = src + line * ls;
    const int d = dst + line * ls;
    int q = q0, k = k0;
    for (int j = jt; j < m; j += NJ) {
      C v[R];
      const int sj = s + j * es;
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = sm[sj + r * me];
      if (Ns > 1) {
        const int ks = k * step;
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], twid<INV>(twp, r * ks));
      }
      Butterfly<R, INV, C>::run(v, twp, n);
      const int dd = d + q * rnse + k * es;
#pragma unroll
      for (int qq = 0; qq < R; ++qq) sm[dd + qq * nse] = v[qq];
      k += dk;
      q += dq;
      if (k >= Ns) { k -= Ns; ++q; }
    }
  }
}

// Stage of any radix R (primes without a closed-form butterfly, up to
// FFT_MAX_GENERIC_RADIX).  The work items are the (butterfly j, output q)
// pairs of a line, spread over all butterfly slots, so a long prime (one
// butterfly per line) is computed by every thread of the line rather than by
// one.  Output q of butterfly j (k = j mod Ns) is
//   sum_r x[j + r*m] * w_n^(r*k*step) * w_R^(r*q) = sum_r x[j + r*m] * w_n^(r*(k*step + q*n/R)),
// one table root per term with the index advanced modulo n.
template <bool INV, typename C>
__device__ __noinline__ void fft_stage_generic(int src, int dst, int n, int R, int Ns, int nlines, int ls, int es,
                                               FftLayout lay, int tw, int t) {
  C* sm = shmem<C>();
  const C* twp = sm + tw;
  const int lg_nl = lay.lg_nl;
  const int NL = 1 << lg_nl;
  const int lg_nj = 8 - lg_nl;
  const int NJ = 1 << lg_nj;
  const int lslot = lay.lines_fast ? (t & (NL - 1)) : (t >> lg_nj);
  const int jt = lay.lines_fast ? (t >> lg_nl) : (t & (NJ - 1));
  const int m = n / R;
  const int items = m * R;
  if (jt >= items) return;
  const int step = n / (Ns * R);
  const int st = n / R;
  for (int line = lslot; line < nlines; line += NL) {
    const int s = src + line * ls;
    const int d = dst + line * ls;
    for (int it = jt; it < items; it += NJ) {
      const int j = it / R, q = it - j * R;
      const int k = j % Ns;
      const int inc = k * step + q * st;  // < n
      C acc = sm[s + j * es];
      int idx = 0;
      for (int r = 1; r < R; ++r) {
        idx += inc;
        if (idx >= n) idx -= n;
        acc = cfma(sm[s + (j + r * m) * es], twid<INV>(twp, idx), acc);
      }
      sm[d + ((j - k) * R + k + q * Ns) * es] = acc;
    }
  }
}

// One stage for thread t; SMALL compiles only radices 2,3,4,5,6,8,9.
template <bool INV, typename C, bool SMALL>
__device__ __forceinline__ void fft_stage_any(int src, int dst, int n, int R, int Ns, int nlines, int ls, int es,
                                              FftLayout lay, int tw, int t) {
  switch (R) {
    case 2: fft_stage<2, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 3: fft_stage<3, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 4: fft_stage<4, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 5: fft_stage<5, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 6: fft_stage<6, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 8: fft_stage<8, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    case 9: fft_stage<9, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
    default:
      if (!SMALL) {
        switch (R) {
          case 7: fft_stage<7, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
          case 11: fft_stage<11, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
          case 13: fft_stage<13, INV, C>(src, dst, n, Ns, nlines, ls, es, lay, tw, t); break;
          default: fft_stage_generic<INV, C>(src, dst, n, R, Ns, nlines, ls, es, lay, tw, t); break;
        }
      }
      break;
  }
}

// Transforms `nlines` lines held at shared offset a (scratch at b, same
// shape; twiddle table at tw).  Element p of line l is at a + l*ls + p*es.
// The caller syncs before the call; the function ends with a __syncthreads()
// and returns the offset that holds the result.
template <bool INV, typename C, bool SMALL = false>
__device__ int fft_lines(int a, int b, const FftPlan& pl, int nlines, int ls, int es, FftLayout lay, int tw) {
  const int n = pl.n;
  int Ns = 1;
  for (int s = 0; s < pl.nstages; ++s) {
    const int R = pl.radix[s];
    fft_stage_any<INV, C, SMALL>(a, b, n, R, Ns, nlines, ls, es, lay, tw, (int)threadIdx.x);
    __syncthreads();
    const int tmp = a; a = b; b = tmp;
    Ns *= R;
  }
  return a;
}

// Copy the length-n twiddle table from global memory to shared offset tw
// (callers sync afterwards, together with their data loads).
template <typename C>
__device__ __forceinline__ void load_twiddles(const C* __restrict__ g, int n, int tw) {
  C* sm = shmem<C>();
  for (int i = threadIdx.x; i < n; i += blockDim.x) sm[tw + i] = __ldg(g + i);
}

#endif  // __CUDACC__ || VS_FFT_HOST_EMULATION

}  // namespace vs
