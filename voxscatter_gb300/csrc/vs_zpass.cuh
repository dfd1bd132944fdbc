// Two-level z pass of the matvec: FFT_z, 6-component tensor multiply, IFFT_z.
//
// The z length is factored R = R1 * R2 (R1 <= 8, R2 <= 32).  With
// z = n1 + R1*n2 and kz = k2 + R2*k1,
//   X[k2 + R2 k1] = sum_n1 w_R1^(n1 k1) w_R^(n1 k2) sum_n2 x[n1 + R1 n2] w_R2^(n2 k2)
// and the inverse runs the same two levels in the opposite order.  A CTA owns
// TX consecutive x columns of one y frequency, all three components:
//   A  : item (c, n1, x): load the z points n1 + R1*n2 (< N) straight from
//        global memory into registers, R2-point DFT, twiddle w_R^(n1 k2),
//        one write to shared memory;
//   B  : item (k2, x): read the 3*R1 values of its k2 column, three R1-point
//        DFTs give all three components at the R1 frequencies k2 + R2*k1,
//        the symmetric tensor multiply with G, three inverse R1-point DFTs,
//        twiddle w_R^(-n1 k2), written back to the positions it read;
//   A' : item (c, n1, x): inverse R2-point DFT, store the first N z entries.
// Each element crosses shared memory twice each way instead of once per
// radix stage, and the shared layout [c][n1][k2][x] keeps every access of the
// three phases conflict-free (x is the fastest index in all of them).
// Lengths outside the instantiated list use the shared-memory Stockham kernel
// k_z of vs_matvec.cu; the operator picks its z length from this list.
// Instantiated per precision in vs_zpass_c64.cu and vs_zpass_c128.cu.
#pragma once
#include "vs_pipeline.cuh"
#include "vs_df.cuh"

namespace vs {

template <int R>
struct FirstRadixZ {
  static constexpr int v = R % 9 == 0 ? 9 : R % 8 == 0 ? 8 : R % 6 == 0 ? 6 : R % 5 == 0 ? 5
                         : R % 4 == 0 ? 4 : R % 3 == 0 ? 3 : R % 2 == 0 ? 2 : R;
};

// In-register Stockham DFT of length N (natural order in and out).  The
// twiddle table holds w_{N*TS}^m, so w_N^j is entry j*TS.
template <int N, int REM, int NS, int TS, bool INV, typename C>
__device__ __forceinline__ void reg_dft(C (&a)[N], const C* tw) {
  if constexpr (REM > 1) {
    constexpr int RD = FirstRadixZ<REM>::v;
    constexpr int m = N / RD;
    constexpr int step = N / (NS * RD);
    C b[N];
#pragma unroll
    for (int j = 0; j < m; ++j) {
      const int k = j % NS;
      C v[RD];
#pragma unroll
      for (int r = 0; r < RD; ++r) v[r] = a[j + r * m];
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < RD; ++r) v[r] = cmul(v[r], twid<INV>(tw, r * k * step * TS));
      }
      Butterfly<RD, INV, C>::run(v, tw, N);
      const int base = (j - k) * RD + k;
#pragma unroll
      for (int q = 0; q < RD; ++q) b[base + q * NS] = v[q];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = b[i];
    reg_dft<N, REM / RD, NS * RD, TS, INV, C>(a, tw);
  }
}

// x columns per CTA: 16 (c64) / 8 (c128), doubled while TX*R2 leaves a partial
// warp and the CTA stays within 512 (c64) / 256 (c128) threads.
template <typename T>
constexpr int z2_tx(int R2) {
  const bool f = std::is_same<T, float>::value;
  int tx = f ? 16 : 8;
  while ((tx * R2) % 32 != 0 && 2 * tx * R2 <= (f ? 512 : 256)) tx *= 2;
  return tx;
}

// One thread per stage-B item (TX * R2); stage A loops over its 3*R1*TX items.
constexpr int z2_threads(int R2, int tx) { return ((R2 * tx + 31) / 32) * 32; }

// CTAs per SM the capped variant holds the register allocation to: the live values of the
// larger of stage A (a line of R2 points and its Stockham copy) and stage B
// (3*R1 points and one tensor row of G) plus addressing, so that the compiler
// keeps several CTAs resident instead of hoisting all G loads of stage B.
template <typename T>
constexpr int z2_min_blocks(int R1, int R2) {
  const int cw = (int)(sizeof(T) / 4);
  const int a = 4 * R2 * cw, b = (6 * R1 + 12) * cw;
  const int need = (a > b ? a : b) + 24;
  const int nb = 65536 / (z2_threads(R2, z2_tx<T>(R2)) * need);
  return nb < 1 ? 1 : (nb > 8 ? 8 : nb);
}

// Entries n2 of a length-R1*R2 line (index n1 + R1 n2) that can be below an
// extent E when the length is at least 2E - 1 (the circulant embedding's
// bound): n2 < ((R1 R2 - 1) / 2) / R1 + 1.
constexpr int lower_half_n2(int R1, int R2) {
  return ((R1 * R2 - 1) / 2) / R1 + 1 < R2 ? ((R1 * R2 - 1) / 2) / R1 + 1 : R2;
}

template <typename T, int R1, int R2, bool CAP, typename K = cplx_t<T>>
__global__ void __launch_bounds__(z2_threads(R2, z2_tx<T>(R2)), CAP ? z2_min_blocks<T>(R1, R2) : 1)
    k_z2(PipeArgs<T> a, int sym) {
  using C = cplx_t<T>;  // storage
  static_assert(sizeof(K) == sizeof(C), "compute and storage elements share the shared-memory layout");
  constexpr int R = R1 * R2, TX = z2_tx<T>(R2), NT = z2_threads(R2, TX);
  if (a.skip && a.skip[blockIdx.z * a.skip_stride]) return;
  K* S = shmem<K>();  // [3][R1][R2][TX]
  K* tw = S + 3 * R * TX;
  for (int i = threadIdx.x; i < R; i += NT) tw[i] = to_compute<K>(__ldg(a.twR + i));
  const int x0 = blockIdx.x * TX, ky = blockIdx.y;
  const int64_t PQ = (int64_t)a.P * a.Q;
  const int64_t zs = PQ, cs = PQ * a.N;
  C* t2 = a.t2 + (int64_t)blockIdx.z * PQ * a.N * 3 + (int64_t)ky * a.P;
  const int N = a.N;
  __syncthreads();

  // A: forward over n2
  for (int it = threadIdx.x; it < 3 * R1 * TX; it += NT) {
    const int xl = it % TX, rest = it / TX;
    const int n1 = rest % R1, c = rest / R1;
    const int x = x0 + xl;
    const bool xin = x < a.P;
    K v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      const int z = n1 + R1 * n2;
      v[n2] = (n2 < lower_half_n2(R1, R2) && xin && z < N) ? to_compute<K>(t2[x + z * zs + c * cs]) : czero<K>();
    }
    reg_dft<R2, R2, 1, R1, false, K>(v, tw);
    K* s = S + ((c * R1 + n1) * R2) * TX + xl;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) s[k2 * TX] = k2 == 0 || n1 == 0 ? v[k2] : cmul(v[k2], tw[n1 * k2]);
  }
  __syncthreads();

  // B: forward over n1, tensor multiply, inverse over k1
  for (int it = threadIdx.x; it < R2 * TX; it += NT) {
    const int xl = it % TX, k2 = it / TX;
    const int x = x0 + xl;
    K u0[R1], u1[R1], u2[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      u0[n1] = S[((0 * R1 + n1) * R2 + k2) * TX + xl];
      u1[n1] = S[((1 * R1 + n1) * R2 + k2) * TX + xl];
      u2[n1] = S[((2 * R1 + n1) * R2 + k2) * TX + xl];
    }
    reg_dft<R1, R1, 1, R2, false, K>(u0, tw);
    reg_dft<R1, R1, 1, R2, false, K>(u1, tw);
    reg_dft<R1, R1, 1, R2, false, K>(u2, tw);
    if (x < a.P) {
      int gx = x, gy = ky, Pg = a.P, Qg = a.Q, Rg = R;
      bool fx = false, fy = false;
      if (sym) {
        Pg = a.P / 2 + 1; Qg = a.Q / 2 + 1; Rg = R / 2 + 1;
        if (x > a.P / 2) { gx = a.P - x; fx = true; }
        if (ky > a.Q / 2) { gy = a.Q - ky; fy = true; }
      }
      const int64_t PQg = (int64_t)Pg * Qg, PQRg = PQg * Rg;
      const C* G = a.G + gx + (int64_t)Pg * gy;
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        const int kz = k2 + R2 * k1;
        int gz = kz;
        bool fz = false;
        if (sym && kz > R / 2) { gz = R - kz; fz = true; }
        const int64_t gi = gz * PQg;
        const K g0 = to_compute<K>(__ldg(G + gi));
        K g1 = to_compute<K>(__ldg(G + PQRg + gi)), g2 = to_compute<K>(__ldg(G + 2 * PQRg + gi));
        const K g3 = to_compute<K>(__ldg(G + 3 * PQRg + gi));
        K g4 = to_compute<K>(__ldg(G + 4 * PQRg + gi));
        const K g5 = to_compute<K>(__ldg(G + 5 * PQRg + gi));
        if (fx != fy) { g1.x = -g1.x; g1.y = -g1.y; }
        if (fx != fz) { g2.x = -g2.x; g2.y = -g2.y; }
        if (fy != fz) { g4.x = -g4.x; g4.y = -g4.y; }
        const K v0 = u0[k1], v1 = u1[k1], v2 = u2[k1];
        K o0 = cmul(g0, v0); o0 = cfma(g1, v1, o0); o0 = cfma(g2, v2, o0);
        K o1 = cmul(g1, v0); o1 = cfma(g3, v1, o1); o1 = cfma(g4, v2, o1);
        K o2 = cmul(g2, v0); o2 = cfma(g4, v1, o2); o2 = cfma(g5, v2, o2);
        u0[k1] = o0;
        u1[k1] = o1;
        u2[k1] = o2;
      }
    }
    reg_dft<R1, R1, 1, R2, true, K>(u0, tw);
    reg_dft<R1, R1, 1, R2, true, K>(u1, tw);
    reg_dft<R1, R1, 1, R2, true, K>(u2, tw);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      const bool plain = n1 == 0 || k2 == 0;
      const K w = plain ? czero<K>() : twid<true>(tw, n1 * k2);
      S[((0 * R1 + n1) * R2 + k2) * TX + xl] = plain ? u0[n1] : cmul(u0[n1], w);
      S[((1 * R1 + n1) * R2 + k2) * TX + xl] = plain ? u1[n1] : cmul(u1[n1], w);
      S[((2 * R1 + n1) * R2 + k2) * TX + xl] = plain ? u2[n1] : cmul(u2[n1], w);
    }
  }
  __syncthreads();

  // A': inverse over k2, store the first N z entries.  The embedding has
  // R >= 2N - 1 (checked at operator creation), so only n2 < NZO can hold a
  // stored z = n1 + R1 n2 < N: the outputs above are never formed (the
  // compiler drops their share of the last butterfly stage).
  for (int it = threadIdx.x; it < 3 * R1 * TX; it += NT) {
    const int xl = it % TX, rest = it / TX;
    const int n1 = rest % R1, c = rest / R1;
    const int x = x0 + xl;
    if (x >= a.P || n1 >= N) continue;
    K v[R2];
    const K* s = S + ((c * R1 + n1) * R2) * TX + xl;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) v[k2] = s[k2 * TX];
    reg_dft<R2, R2, 1, R1, true, K>(v, tw);
#pragma unroll
    for (int n2 = 0; n2 < lower_half_n2(R1, R2); ++n2) {
      const int z = n1 + R1 * n2;
      if (z < N) t2[x + z * zs + c * cs] = to_storage(v[n2], C{});
    }
  }
}

// (R1, R2) of every instantiated z length; lengths are 5-smooth.
struct ZSplit {
  int R, R1, R2;
};
static constexpr ZSplit kZSplits[] = {
    {4, 2, 2},    {6, 2, 3},    {8, 2, 4},    {9, 3, 3},    {10, 2, 5},   {12, 3, 4},   {15, 3, 5},
    {16, 4, 4},   {18, 3, 6},   {20, 4, 5},   {24, 4, 6},   {27, 3, 9},   {30, 5, 6},   {32, 4, 8},
    {36, 6, 6},   {40, 5, 8},   {45, 5, 9},   {48, 6, 8},   {54, 6, 9},   {60, 6, 10},  {64, 8, 8},
    {72, 8, 9},   {80, 8, 10},  {90, 6, 15},  {96, 8, 12},  {108, 6, 18}, {120, 8, 15}, {128, 8, 16},
    {144, 8, 18}, {160, 8, 20}, {180, 6, 30}, {192, 8, 24}, {216, 8, 27}, {240, 8, 30}, {256, 8, 32}};

// K: the arithmetic type (the storage type, or double-float for FP64 storage;
// the double-float kernel is built only in its register-capped form).
template <typename T, int R1, int R2, typename K>
static void launch_z2(const PipeArgs<T>& a, int sym, bool cap, int nrhs, cudaStream_t st) {
  constexpr int TX = z2_tx<T>(R2), NT = z2_threads(R2, TX);
  const size_t smem = (3ull * R1 * R2 * TX + R1 * R2) * sizeof(cplx_t<T>);
  constexpr bool native = std::is_same<K, cplx_t<T>>::value;
  auto k = (cap || !native) ? k_z2<T, R1, R2, true, K> : k_z2<T, R1, R2, native ? false : true, K>;
  set_kernel_smem((const void*)k, smem);
  k<<<dim3(ceil_div(a.P, TX), a.Q, nrhs), NT, smem, st>>>(a, sym);
  VS_LAUNCH_CHECK();
}

template <typename T, typename K>
bool z_pass_two_level(const PipeArgs<T>& a, bool sym, bool cap, int nrhs, cudaStream_t st) {
  const int s = sym ? 1 : 0;
  switch (a.R) {
#define VS_Z2(R1, R2)                                        \
  case R1 * R2: launch_z2<T, R1, R2, K>(a, s, cap, nrhs, st); \
    return true;
    VS_Z2(2, 2) VS_Z2(2, 3) VS_Z2(2, 4) VS_Z2(3, 3) VS_Z2(2, 5) VS_Z2(3, 4) VS_Z2(3, 5)
    VS_Z2(4, 4) VS_Z2(3, 6) VS_Z2(4, 5) VS_Z2(4, 6) VS_Z2(3, 9) VS_Z2(5, 6) VS_Z2(4, 8)
    VS_Z2(6, 6) VS_Z2(5, 8) VS_Z2(5, 9) VS_Z2(6, 8) VS_Z2(6, 9) VS_Z2(6, 10) VS_Z2(8, 8)
    VS_Z2(8, 9) VS_Z2(8, 10) VS_Z2(6, 15) VS_Z2(8, 12) VS_Z2(6, 18) VS_Z2(8, 15) VS_Z2(8, 16)
    VS_Z2(8, 18) VS_Z2(8, 20) VS_Z2(6, 30) VS_Z2(8, 24) VS_Z2(8, 27) VS_Z2(8, 30) VS_Z2(8, 32)
#undef VS_Z2
    default: return false;
  }
}
}  // namespace vs
