// Sequential host emulation of the device Stockham FFT (vs_fft.cuh).
// Every stage reads one buffer and writes the other, so running the 256
// threads of a CTA one after another, stage by stage, computes exactly what
// the CTA computes.  Compares forward and inverse transforms against a naive
// O(n^2) DFT in long double, for several thread layouts.
#include <cuda_runtime.h>
struct VsDim { unsigned x = 0, y = 0, z = 0; };
static VsDim threadIdx;
static VsDim blockDim = {1, 1, 1};
#define __syncthreads()
#define __noinline__
#define __ldg(p) (*(p))
#define VS_FFT_HOST_EMULATION 1
#include "../../voxscatter_gb300/csrc/vs_fft.cuh"

// The emulated CTA's dynamic shared memory (referenced by vs::shmem()).
namespace vs {
alignas(16) unsigned char smem_raw[1 << 22];
}
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

// Runs the stages of one CTA: shared buffers at offsets a and b, twiddles at tw.
template <bool INV, typename C, bool SMALL>
static int emulate(int a, int b, const vs::FftPlan& pl, int nlines, int ls, int es, vs::FftLayout lay, int tw) {
  int Ns = 1;
  for (int s = 0; s < pl.nstages; ++s) {
    for (int t = 0; t < vs::kFftThreads; ++t)
      vs::fft_stage_any<INV, C, SMALL>(a, b, pl.n, pl.radix[s], Ns, nlines, ls, es, lay, tw, t);
    const int tmp = a; a = b; b = tmp;
    Ns *= pl.radix[s];
  }
  return a;
}

template <typename T, bool INV>
static double check(int n, int nlines, bool lines_fast, int lg_nl = 0) {
  using C = vs::cplx_t<T>;
  vs::FftPlan pl = vs::make_fft_plan(n);
  std::vector<double> tw = vs::twiddle_table(n);
  C* sm = reinterpret_cast<C*>(vs::smem_raw);
  const int total = n * nlines;
  const int off_b = total, off_tw = 2 * total;
  for (int k = 0; k < n; ++k) { sm[off_tw + k].x = (T)tw[2 * k]; sm[off_tw + k].y = (T)tw[2 * k + 1]; }
  C* a = sm;
  std::vector<long double> in_re((size_t)n * nlines), in_im((size_t)n * nlines);
  srand(n * 7 + nlines);
  const int ls = lines_fast ? 1 : n, es = lines_fast ? nlines : 1;
  for (int l = 0; l < nlines; ++l)
    for (int p = 0; p < n; ++p) {
      double re = rand() / (double)RAND_MAX - 0.5, im = rand() / (double)RAND_MAX - 0.5;
      a[l * ls + p * es].x = (T)re; a[l * ls + p * es].y = (T)im;
      in_re[l * n + p] = (T)re; in_im[l * n + p] = (T)im;
    }
  const vs::FftLayout lay{lg_nl, lines_fast};
  const int roff = vs::plan_is_small_radix(pl) ? emulate<INV, C, true>(0, off_b, pl, nlines, ls, es, lay, off_tw)
                                               : emulate<INV, C, false>(0, off_b, pl, nlines, ls, es, lay, off_tw);
  const C* res = sm + roff;
  double err = 0, ref = 0;
  const long double sg = INV ? 1.0L : -1.0L;
  for (int l = 0; l < nlines; ++l)
    for (int q = 0; q < n; ++q) {
      long double sr = 0, si = 0;
      for (int p = 0; p < n; ++p) {
        long double ang = sg * 2.0L * 3.14159265358979323846264338327950288L * (long double)((long long)p * q % n) / n;
        long double c = cosl(ang), s = sinl(ang);
        sr += in_re[l * n + p] * c - in_im[l * n + p] * s;
        si += in_re[l * n + p] * s + in_im[l * n + p] * c;
      }
      const C o = res[l * ls + q * es];
      err += (double)((o.x - sr) * (o.x - sr) + (o.y - si) * (o.y - si));
      ref += (double)(sr * sr + si * si);
    }
  return std::sqrt(err / ref);
}

int main() {
  const int sizes[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 12, 13, 16, 17, 18, 23, 26, 27, 32, 36, 49, 52, 54, 56, 64, 72, 81,
                       53, 61, 68, 79, 91, 101, 105, 113, 121, 126, 128, 169, 182, 189, 192, 210, 127, 254, 256, 384,
                       512, 625, 1024};
  int bad = 0;
  for (int n : sizes) {
    for (int lf = 0; lf < 2; ++lf) {
      const int nl = lf ? 5 : 3;
      const int lg = (n % 3) + (lf ? 2 : 0);  // vary the number of line slots (1..16)
      double e1 = check<double, false>(n, nl, lf, lg), e2 = check<double, true>(n, nl, lf, lg);
      double e3 = check<float, false>(n, nl, lf, lg), e4 = check<float, true>(n, nl, lf, lg);
      const bool ok = e1 < 1e-14 && e2 < 1e-14 && e3 < 2e-6 && e4 < 2e-6;
      if (!ok) ++bad;
      printf("n=%5d lines_fast=%d  f64 %.2e %.2e  f32 %.2e %.2e %s\n", n, lf, e1, e2, e3, e4, ok ? "ok" : "BAD");
    }
  }
  printf(bad ? "FAILED %d\n" : "ALL OK\n", bad);
  return bad ? 1 : 0;
}
