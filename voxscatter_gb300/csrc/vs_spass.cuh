// Two-level strided pass: FFT (forward) or IFFT (inverse) along a strided
// axis (y) of many lines, x tiles contiguous -- the y passes of the matvec and
// of the preconditioner apply.
//
// The line length is factored n = R1 * R2 (R1 <= 16, R2 <= 32, R1 near
// sqrt(n)).  With row = n1 + R1*n2 and k = k2 + R2*k1,
//   X[k2 + R2 k1] = sum_n1 w_R1^(n1 k1) w_n^(n1 k2) sum_n2 x[n1 + R1 n2] w_R2^(n2 k2).
// A CTA owns TX consecutive x columns of one plane:
//   forward  A : item (n1, x): rows n1 + R1*n2 (< n_in) straight from global
//                memory into registers, R2-point DFT, twiddle, one shared store;
//            B : item (k2, x): R1-point DFT of its column, outputs k2 + R2*k1
//                (< n_out) straight to global memory;
//   inverse  B': item (k2, x): rows k2 + R2*k1 from global memory, inverse
//                R1-point DFT, conjugate twiddle, one shared store;
//            A': item (n1, x): inverse R2-point DFT, rows n1 + R1*n2 (< n_out)
//                to global memory.
// Each element crosses shared memory once each way (the shared-memory
// Stockham kernel k_strided of vs_matvec.cu crosses it once per radix stage);
// the shared layout [n1][k2][x] is conflict-free in both stages.  Lengths
// outside the instantiated list use k_strided.  K is the arithmetic type: the
// storage type, or double-float (dfc) on FP64 data.  Instantiated per
// precision in vs_spass_c64.cu and vs_spass_c128.cu, in double-float in
// vs_df_spass_a.cu / vs_df_spass_b.cu (vs_df_passes.cuh).
#pragma once
#include "vs_zpass.cuh"

namespace vs {

// x columns per CTA: 16 (c64) / 8 (c128), doubled while TX*R2 leaves a partial
// warp and the CTA stays within 512 (c64) / 256 (c128) threads.
template <typename T, int R2>
constexpr int s2_tx() {
  const bool f = std::is_same<T, float>::value;
  int tx = f ? 16 : 8;
  while ((tx * R2) % 32 != 0 && 2 * tx * R2 <= (f ? 512 : 256)) tx *= 2;
  return tx;
}

// HO, inverse: n_out <= (R1 R2 + 1) / 2, so the outputs n2 >= lower_half_n2
// are never stored and never formed; forward (c64): n_in <= (R1 R2 + 1) / 2,
// so the inputs n2 >= lower_half_n2 are zeros the compiler folds out of the
// first DFT stage (the matvec's y pass has Q >= 2M - 1).
template <typename T, int R1, int R2, bool INV, typename K = cplx_t<T>, bool HO = false>
__global__ void __launch_bounds__(z2_threads(R2, s2_tx<T, R2>())) k_s2(StridedArgs<T> a) {
  using C = cplx_t<T>;  // storage
  static_assert(sizeof(K) == sizeof(C), "compute and storage elements share the shared-memory layout");
  constexpr int N = R1 * R2, TX = s2_tx<T, R2>(), NT = z2_threads(R2, TX);
  if (a.skip && a.skip[blockIdx.z * a.skip_stride]) return;
  a.prefetch_l2();
  K* S = shmem<K>();  // [R1][R2][TX]
  K* tw = S + N * TX;
  for (int i = threadIdx.x; i < N; i += NT) tw[i] = to_compute<K>(__ldg(a.tw + i));
  const int x0 = blockIdx.x * TX;
  int pa, pb;
  a.plane(pa, pb);
  const C* src = a.src + pa * a.s_a + pb * a.s_b + (int64_t)blockIdx.z * a.s_rhs;
  C* dst = a.dst + pa * a.d_a + pb * a.d_b + (int64_t)blockIdx.z * a.d_rhs;
  __syncthreads();
  if constexpr (!INV) {
    for (int it = threadIdx.x; it < R1 * TX; it += NT) {
      const int xl = it % TX, n1 = it / TX;
      const int x = x0 + xl;
      const bool xin = x < a.xext;
      K v[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) {
        const int row = n1 + R1 * n2;
        v[n2] = ((!HO || n2 < lower_half_n2(R1, R2)) && xin && row < a.n_in) ? to_compute<K>(src[row * a.s_row + x])
                                                                              : czero<K>();
      }
      reg_dft<R2, R2, 1, R1, false, K>(v, tw);
      K* s = S + (n1 * R2) * TX + xl;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) s[k2 * TX] = (k2 == 0 || n1 == 0) ? v[k2] : cmul(v[k2], tw[n1 * k2]);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < R2 * TX; it += NT) {
      const int xl = it % TX, k2 = it / TX;
      const int x = x0 + xl;
      K u[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) u[n1] = S[(n1 * R2 + k2) * TX + xl];
      reg_dft<R1, R1, 1, R2, false, K>(u, tw);
      if (x < a.xext) {
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) {
          const int row = k2 + R2 * k1;
          if (row < a.n_out) dst[row * a.d_row + x] = to_storage(u[k1], C{});
        }
      }
    }
  } else {
    for (int it = threadIdx.x; it < R2 * TX; it += NT) {
      const int xl = it % TX, k2 = it / TX;
      const int x = x0 + xl;
      const bool xin = x < a.xext;
      K u[R1];
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        const int row = k2 + R2 * k1;
        u[k1] = (xin && row < a.n_in) ? to_compute<K>(src[row * a.s_row + x]) : czero<K>();
      }
      reg_dft<R1, R1, 1, R2, true, K>(u, tw);
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1)
        S[(n1 * R2 + k2) * TX + xl] = (n1 == 0 || k2 == 0) ? u[n1] : cmul(u[n1], twid<true>(tw, n1 * k2));
    }
    __syncthreads();
    for (int it = threadIdx.x; it < R1 * TX; it += NT) {
      const int xl = it % TX, n1 = it / TX;
      const int x = x0 + xl;
      if (x >= a.xext || n1 >= a.n_out) continue;
      K v[R2];
      const K* s = S + (n1 * R2) * TX + xl;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) v[k2] = s[k2 * TX];
      reg_dft<R2, R2, 1, R1, true, K>(v, tw);
#pragma unroll
      for (int n2 = 0; n2 < (HO ? lower_half_n2(R1, R2) : R2); ++n2) {
        const int row = n1 + R1 * n2;
        if (row < a.n_out) dst[row * a.d_row + x] = to_storage(v[n2], C{});
      }
    }
  }
}

template <typename T, int R1, int R2, bool INV, typename K = cplx_t<T>>
static void launch_s2(const StridedArgs<T>& a, int nplanes, int nrhs, cudaStream_t st) {
  constexpr int TX = s2_tx<T, R2>(), NT = z2_threads(R2, TX);
  const size_t smem = (size_t)(R1 * R2 * TX + R1 * R2) * sizeof(cplx_t<T>);
  // the matvec's y passes read (forward) and keep (inverse) at most half the
  // line (Q >= 2M - 1)
  auto k = k_s2<T, R1, R2, INV, K>;
  if constexpr (INV) {
    if (2 * a.n_out - 1 <= R1 * R2) k = k_s2<T, R1, R2, INV, K, true>;
  } else if constexpr (std::is_same<T, float>::value) {
    if (2 * a.n_in - 1 <= R1 * R2) k = k_s2<T, R1, R2, INV, K, true>;
  }
  set_kernel_smem((const void*)k, smem);
  const dim3 grid(ceil_div(a.xext, TX), nplanes, nrhs);
  StridedArgs<T> b = a;
  if (b.pf) b.pf_per_cta = prefetch_share(b.pf_bytes, (uint64_t)grid.x * grid.y * grid.z);
  k<<<grid, NT, smem, st>>>(b);
  VS_LAUNCH_CHECK();
}

// Every instantiated two-level length (5-smooth 8..256, 288, 320, 384, 432,
// 480, 512, 91 = 7*13 and 105 = 7*15) with its split n = R1 * R2.
#define VS_S2_LIST(X)                                                                                      \
  X(2, 4) X(3, 3) X(2, 5) X(3, 4) X(3, 5) X(4, 4) X(3, 6) X(4, 5) X(4, 6) X(5, 5) X(3, 9) X(5, 6) X(4, 8)   \
  X(6, 6) X(5, 8) X(5, 9) X(6, 8) X(5, 10) X(6, 9) X(6, 10) X(8, 8) X(8, 9) X(5, 15) X(8, 10) X(9, 9)      \
  X(9, 10) X(8, 12) X(10, 10) X(9, 12) X(10, 12) X(5, 25) X(8, 16) X(9, 15) X(12, 12) X(10, 15) X(10, 16)  \
  X(9, 18) X(12, 15) X(12, 16) X(10, 20) X(12, 18) X(15, 15) X(12, 20) X(9, 27) X(10, 25) X(16, 16) X(7, 13)   \
  X(7, 15) X(12, 24) X(16, 20) X(16, 24) X(16, 27) X(16, 30) X(16, 32)

template <typename T, bool INV>
bool strided_two_level(const StridedArgs<T>& a, int nplanes, int nrhs, cudaStream_t st) {
  switch (a.plan.n) {
#define VS_S2_CASE(R1, R2)                            \
  case R1 * R2:                                       \
    launch_s2<T, R1, R2, INV>(a, nplanes, nrhs, st); \
    return true;
    VS_S2_LIST(VS_S2_CASE)
#undef VS_S2_CASE
    default: return false;
  }
}

}  // namespace vs
