// Register-resident z pass of the c64 matvec for short z transforms.
//
// For every 5-smooth z length R <= 54 except 48 (lengths whose line fits in
// registers without spilling; the library pads N <= 27 layers to these) a
// kernel is instantiated in which each thread holds one
// whole (component, x) line of the tile in registers and runs a fully unrolled
// mixed-radix Stockham FFT: all indices are compile-time constants, the
// twiddles are read from shared memory at constant offsets, and no barrier
// separates the stages.  The three components meet once in shared memory for
// the 6-component tensor multiply (first-octant spectrum with parity signs),
// then each thread transforms its output line back and stores the first N
// entries in place.  Same arithmetic as k_z in vs_matvec.cu.
#include "vs_pipeline.cuh"

namespace vs {

template <int R>
struct FirstRadix {
  static constexpr int v = R % 9 == 0 ? 9 : R % 8 == 0 ? 8 : R % 6 == 0 ? 6 : R % 5 == 0 ? 5
                         : R % 4 == 0 ? 4 : R % 3 == 0 ? 3 : R % 2 == 0 ? 2 : R;
};

template <int N, int REM, int NS, bool INV, typename C>
__device__ __forceinline__ void reg_fft_stages(C (&a)[N], const C* tw) {
  if constexpr (REM > 1) {
    constexpr int RD = FirstRadix<REM>::v;
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
        for (int r = 1; r < RD; ++r) v[r] = cmul(v[r], twid<INV>(tw, r * k * step));
      }
      Butterfly<RD, INV, C>::run(v, tw, N);
      const int base = (j - k) * RD + k;
#pragma unroll
      for (int q = 0; q < RD; ++q) b[base + q * NS] = v[q];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = b[i];
    reg_fft_stages<N, REM / RD, NS * RD, INV, C>(a, tw);
  }
}

constexpr int kZRegTx = 32;  // x columns per CTA; 3 warps (one per component)

template <int R>
__global__ void __launch_bounds__(3 * kZRegTx) k_z_reg(PipeArgs<float> a) {
  using C = float2;
  if (a.skip && a.skip[blockIdx.z * a.skip_stride]) return;
  __shared__ C xch[3 * R * kZRegTx];
  __shared__ C tw[R];
  for (int i = threadIdx.x; i < R; i += blockDim.x) tw[i] = __ldg(a.twR + i);
  const int c = threadIdx.x / kZRegTx, xl = threadIdx.x - c * kZRegTx;
  const int x = blockIdx.x * kZRegTx + xl;
  const int ky = blockIdx.y;
  const bool xin = x < a.P;
  const int64_t PQ = (int64_t)a.P * a.Q;
  C* t2 = a.t2 + (int64_t)blockIdx.z * PQ * a.N * 3 + (int64_t)ky * a.P + (int64_t)c * PQ * a.N + x;
  C v[R];
#pragma unroll
  for (int z = 0; z < R; ++z) v[z] = (z < a.N && xin) ? t2[z * PQ] : make_float2(0.f, 0.f);
  __syncthreads();
  reg_fft_stages<R, R, 1, false, C>(v, tw);
#pragma unroll
  for (int kz = 0; kz < R; ++kz) xch[(c * R + kz) * kZRegTx + xl] = v[kz];
  __syncthreads();
  if (xin) {
    // first-octant spectrum: mirrored frequencies with the parity signs
    const int Pg = a.P / 2 + 1, Qg = a.Q / 2 + 1, Rg = R / 2 + 1;
    const bool fx = x > a.P / 2, fy = ky > a.Q / 2;
    const int gx = fx ? a.P - x : x, gy = fy ? a.Q - ky : ky;
    const int64_t PQg = (int64_t)Pg * Qg, PQRg = PQg * Rg;
    const C* G = a.G + gx + (int64_t)Pg * gy;
    // components of row c of the symmetric tensor: (0: xx,xy,xz), (1: xy,yy,yz), (2: xz,yz,zz)
    const int c0 = c == 0 ? 0 : (c == 1 ? 1 : 2);
    const int c1 = c == 0 ? 1 : (c == 1 ? 3 : 4);
    const int c2 = c == 0 ? 2 : (c == 1 ? 4 : 5);
#pragma unroll
    for (int kz = 0; kz < R; ++kz) {
      const bool fz = kz > R / 2;
      const int64_t gi = (int64_t)(fz ? R - kz : kz) * PQg;
      C g0 = __ldg(G + c0 * PQRg + gi), g1 = __ldg(G + c1 * PQRg + gi), g2 = __ldg(G + c2 * PQRg + gi);
      // parity of each used component: xy (fx^fy), xz (fx^fz), yz (fy^fz)
      auto sgn = [&](int comp, C g) {
        const bool neg = (comp == 1 && fx != fy) || (comp == 2 && fx != fz) || (comp == 4 && fy != fz);
        return neg ? make_float2(-g.x, -g.y) : g;
      };
      g0 = sgn(c0, g0); g1 = sgn(c1, g1); g2 = sgn(c2, g2);
      const C i0 = xch[kz * kZRegTx + xl], i1 = xch[(R + kz) * kZRegTx + xl], i2 = xch[(2 * R + kz) * kZRegTx + xl];
      C o = cmul(g0, i0);
      o = cfma(g1, i1, o);
      o = cfma(g2, i2, o);
      v[kz] = o;
    }
    reg_fft_stages<R, R, 1, true, C>(v, tw);
#pragma unroll
    for (int z = 0; z < R; ++z)
      if (z < a.N) t2[z * PQ] = v[z];
  }
}

// Launches the register z pass when R has a register kernel; returns false otherwise.
bool z_pass_reg(const PipeArgs<float>& a, int nrhs, cudaStream_t st) {
  const dim3 grid(ceil_div(a.P, kZRegTx), a.Q, nrhs);
  const dim3 block(3 * kZRegTx);
  switch (a.R) {
#define VS_ZR(RR) \
  case RR: k_z_reg<RR><<<grid, block, 0, st>>>(a); break;
    VS_ZR(2) VS_ZR(3) VS_ZR(4) VS_ZR(5) VS_ZR(6) VS_ZR(8) VS_ZR(9) VS_ZR(10) VS_ZR(12) VS_ZR(15) VS_ZR(16)
    VS_ZR(18) VS_ZR(20) VS_ZR(24) VS_ZR(25) VS_ZR(27) VS_ZR(30) VS_ZR(32) VS_ZR(36) VS_ZR(40) VS_ZR(45)
    VS_ZR(50) VS_ZR(54)
#undef VS_ZR
    default: return false;
  }
  VS_LAUNCH_CHECK();
  return true;
}

}  // namespace vs
