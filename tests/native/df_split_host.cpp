// The FP64 <-> double-float conversions of vs_df.cuh (df_from_double,
// df_store) compiled for the host, with host stand-ins for the device
// intrinsics they use, against the FP64 conversions they replace:
// hi = (float)d, lo = (float)(d - (double)hi) bit for bit (round to nearest,
// ties to even) over random doubles of every exponent, exact ties and
// near-ties, zeros and the values outside the fast range; and df_store
// against (double)hi + (double)lo.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline long long __double_as_longlong(double d) { long long l; std::memcpy(&l, &d, 8); return l; }
static inline double __hiloint2double(int hi, int lo) {
  const unsigned long long b = ((unsigned long long)(unsigned)hi << 32) | (unsigned)lo;
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}
#include "../../voxscatter_gb300/csrc/vs_df.cuh"

static unsigned fbits(float f) { return __float_as_uint(f); }
static unsigned long long dbits(double d) { return (unsigned long long)__double_as_longlong(d); }

int main() {
  std::mt19937_64 rng(12345);
  std::vector<double> vals;
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-140, 140);
  for (int k = 0; k < 400000; ++k) vals.push_back(std::ldexp(u(rng), ex(rng)));
  // exact ties and near-ties of the float rounding, both signs
  for (int k = 0; k < 20000; ++k) {
    const float f = (float)std::ldexp(u(rng), ex(rng) / 2);
    const double h = (double)std::nextafter(f, 2.0f * std::fabs(f) + 1.0f) - (double)f;
    for (double d : {(double)f + h / 2, (double)f - h / 2, (double)f + h / 2 * (1 + std::ldexp(1.0, -28)),
                     (double)f + h / 2 * (1 - std::ldexp(1.0, -28)), -((double)f + h / 2)})
      vals.push_back(d);
  }
  for (double d : {0.0, -0.0, 1.0, -1.0, std::ldexp(1.0, -74), std::ldexp(1.0, -75), std::ldexp(1.0, 126),
                   std::ldexp(1.0, 127), 3.4e38, -3.4e38, 1e-300, -1e-300})
    vals.push_back(d);
  long bad = 0, fast = 0;
  for (double d : vals) {
    const vs::df a = vs::df_from_double(d);
    const float hr = (float)d;
    const float lr = (float)(d - (double)hr);
    const unsigned eb = (unsigned)(dbits(d) >> 52) & 0x7FFu;
    if (eb >= 949 && eb <= 1149) ++fast;
    if (fbits(a.hi) != fbits(hr) || fbits(a.lo) != fbits(lr)) {
      if (++bad < 5) std::printf("split mismatch at %.17g: %a %a vs %a %a\n", d, a.hi, a.lo, hr, lr);
    }
    const double back = vs::df_store(a), ref = (double)a.hi + (double)a.lo;
    if (dbits(back) != dbits(ref)) {
      if (++bad < 5) std::printf("store mismatch at %.17g\n", d);
    }
  }
  std::printf("%zu values (%ld on the fast path), %ld mismatches\n", vals.size(), fast, bad);
  if (bad == 0) std::printf("ALL OK\n");
  return bad == 0 ? 0 : 1;
}
