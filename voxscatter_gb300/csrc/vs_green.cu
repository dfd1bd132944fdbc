// Operator setup on the device, FP64:
//  * Draine-Flatau tensor at every grid offset (getOPERATOR_DDA.m:29-119),
//  * parity-signed circulant embedding (circulant_nop_const.m:1-40 with the
//    sign table of gperiodic_coeff_nop.m:4-31) and its 3-D FFT
//    (fft_operator.m:1-8),
//  * the inverse: recovering the first-octant Toeplitz tensor from a given fN.
#include "vs_internal.h"
#include <cmath>

namespace vs {

// Per-axis parity of each component (xx,xy,xz,yy,yz,zz): -1 where the
// component is odd in that coordinate.  Products of these reproduce every row
// of gperiodic_coeff_nop.m (e.g. 'LM' = 'L' .* 'M').
__constant__ int c_par[3][6] = {{+1, -1, -1, +1, +1, +1},
                                {+1, -1, +1, +1, -1, +1},
                                {+1, +1, -1, +1, -1, +1}};

__constant__ double c_gl_x[10];
__constant__ double c_gl_w[10];

__device__ __forceinline__ void dda_tensor(double rx, double ry, double rz, double ko, double2* g) {
  const double r = sqrt(rx * rx + ry * ry + rz * rz);
  if (!(fabs(r) > 1e-15)) {
#pragma unroll
    for (int c = 0; c < 6; ++c) g[c] = make_double2(0, 0);
    return;
  }
  const double h[3] = {rx / r, ry / r, rz / r};
  double sn, cs;
  sincos(ko * r, &sn, &cs);
  // exp(i k r)/r
  const double2 pre = make_double2(cs / r, sn / r);
  const double c1 = ko * ko;
  // (i k r - 1)/r^2
  const double2 c2 = make_double2(-1.0 / (r * r), ko / r);
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const double I = (pa[c] == pb[c]) ? 1.0 : 0.0;
    const double rr = h[pa[c]] * h[pb[c]];
    const double t1 = c1 * (I - rr);
    const double t3 = I - 3.0 * rr;
    const double2 inner = make_double2(t1 + c2.x * t3, c2.y * t3);
    g[c] = cmul(pre, inner);
  }
}

__global__ void k_green(int L, int M, int N, const double* __restrict__ ox, const double* __restrict__ oy,
                        const double* __restrict__ oz, double ko, int near_quad, double2* __restrict__ toep) {
  const int64_t V = (int64_t)L * M * N;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(v % L);
    const int j = (int)((v / L) % M);
    const int k = (int)(v / ((int64_t)L * M));
    const double rx = ox[i], ry = oy[j], rz = oz[k];
    double2 g[6];
    const double rjk = sqrt(rx * rx + ry * ry + rz * rz);
    const double dx = L > 1 ? ox[1] : 0.0;
    if (near_quad && rjk < 5 * dx && rjk > 1e-15) {
      double2 acc[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[c] = make_double2(0, 0);
      for (int a = 0; a < 10; ++a)
        for (int b = 0; b < 10; ++b)
          for (int q = 0; q < 10; ++q) {
            double2 t[6];
            dda_tensor(rx + 0.5 * dx * c_gl_x[a], ry + 0.5 * dx * c_gl_x[b], rz + 0.5 * dx * c_gl_x[q], ko, t);
            const double w = 0.125 * c_gl_w[a] * c_gl_w[b] * c_gl_w[q];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              acc[c].x += w * t[c].x;
              acc[c].y += w * t[c].y;
            }
          }
#pragma unroll
      for (int c = 0; c < 6; ++c) g[c] = acc[c];
    } else {
      dda_tensor(rx, ry, rz, ko, g);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) toep[c * V + v] = g[c];
  }
}

// Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n
// (Golub & Welsch give the same rule; this is the classic recurrence form).
static void gauss_legendre(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-16) break;
    }
    x[i] = -z;
    w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

void green_dda_device(int L, int M, int N, const double* ox, const double* oy, const double* oz, double ko,
                      int near_quad, double2* toep, cudaStream_t st) {
  if (near_quad) {
    double x[10], w[10];
    gauss_legendre(10, x, w);
    VS_CUDA(cudaMemcpyToSymbolAsync(c_gl_x, x, sizeof(x), 0, cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyToSymbolAsync(c_gl_w, w, sizeof(w), 0, cudaMemcpyHostToDevice, st));
  }
  const int64_t V = (int64_t)L * M * N;
  const int blocks = (int)std::min<int64_t>(ceil_div(V, 128), 152 * 32);
  k_green<<<blocks, 128, 0, st>>>(L, M, N, ox, oy, oz, ko, near_quad, toep);
  VS_LAUNCH_CHECK();
}

// Source index and sign of circulant entry p along an axis of Toeplitz length
// n embedded in length Pn >= 2n-1: 0..n-1 direct, Pn-n+1..Pn-1 reflected, rest 0.
__device__ __forceinline__ int refl(int p, int n, int Pn, bool* flipped) {
  if (p < n) { *flipped = false; return p; }
  if (p >= Pn - n + 1) { *flipped = true; return Pn - p; }
  return -1;
}

__global__ void k_embed(int L, int M, int N, const double2* __restrict__ toep, int P, int Q, int R,
                        double2* __restrict__ out) {
  const int64_t PQR = (int64_t)P * Q * R;
  const int64_t V = (int64_t)L * M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * PQR; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / PQR);
    const int64_t g = e - c * PQR;
    const int p = (int)(g % P);
    const int q = (int)((g / P) % Q);
    const int r = (int)(g / ((int64_t)P * Q));
    bool fx, fy, fz;
    const int i = refl(p, L, P, &fx), j = refl(q, M, Q, &fy), k = refl(r, N, R, &fz);
    double2 v = make_double2(0, 0);
    if (i >= 0 && j >= 0 && k >= 0) {
      v = toep[c * V + i + (int64_t)L * (j + (int64_t)M * k)];
      int s = 1;
      if (fx) s *= c_par[0][c];
      if (fy) s *= c_par[1][c];
      if (fz) s *= c_par[2][c];
      if (s < 0) { v.x = -v.x; v.y = -v.y; }
    }
    out[e] = v;
  }
}

void embed_fft_device(int L, int M, int N, const double2* toep, int P, int Q, int R, double2* out, FftAxis* ax,
                      cudaStream_t st) {
  const int64_t PQR = (int64_t)P * Q * R;
  k_embed<<<(int)std::min<int64_t>(ceil_div(6 * PQR, 256), 152 * 32), 256, 0, st>>>(L, M, N, toep, P, Q, R, out);
  VS_LAUNCH_CHECK();
  fft_axis0<double, false>(out, P, (int64_t)Q * R * 6, ax[0], st);
  fft_strided<double, false>(out, P, Q, P, R, (int64_t)P * Q, 6, PQR, ax[1], st);
  fft_strided<double, false>(out, P, R, (int64_t)P * Q, Q, P, 6, PQR, ax[2], st);
}

__global__ void k_crop(int L, int M, int N, int P, int Q, int R, const double2* __restrict__ full, double scale,
                       double2* __restrict__ toep) {
  const int64_t V = (int64_t)L * M * N;
  const int64_t PQR = (int64_t)P * Q * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * V; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / V);
    const int64_t v = e - c * V;
    const int i = (int)(v % L);
    const int j = (int)((v / L) % M);
    const int k = (int)(v / ((int64_t)L * M));
    const double2 a = full[c * PQR + i + (int64_t)P * (j + (int64_t)Q * k)];
    toep[e] = make_double2(a.x * scale, a.y * scale);
  }
}

void toep_from_fN_device(int L, int M, int N, int P, int Q, int R, double2* fN, double2* toep, FftAxis* ax,
                         cudaStream_t st) {
  const int64_t PQR = (int64_t)P * Q * R;
  fft_axis0<double, true>(fN, P, (int64_t)Q * R * 6, ax[0], st);
  fft_strided<double, true>(fN, P, Q, P, R, (int64_t)P * Q, 6, PQR, ax[1], st);
  fft_strided<double, true>(fN, P, R, (int64_t)P * Q, Q, P, 6, PQR, ax[2], st);
  const int64_t V = (int64_t)L * M * N;
  k_crop<<<(int)std::min<int64_t>(ceil_div(6 * V, 256), 152 * 32), 256, 0, st>>>(L, M, N, P, Q, R, fN,
                                                                              1.0 / (double)PQR, toep);
  VS_LAUNCH_CHECK();
}

__global__ void k_finalize(const double2* __restrict__ in, int64_t n, double scale, double2* __restrict__ g64,
                           float2* __restrict__ g32) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = make_double2(in[e].x * scale, in[e].y * scale);
    if (g64) g64[e] = a;
    if (g32) g32[e] = make_float2((float)a.x, (float)a.y);
  }
}

// First-octant copy kx <= P/2, ky <= Q/2, kz <= R/2 of the scaled spectrum
// (the rest follows from the per-axis parity of each component).
__global__ void k_octant(const double2* __restrict__ in, int P, int Q, int R, double scale, double2* __restrict__ g64,
                         float2* __restrict__ g32) {
  const int Ph = P / 2 + 1, Qh = Q / 2 + 1, Rh = R / 2 + 1;
  const int64_t oct = (int64_t)Ph * Qh * Rh, PQR = (int64_t)P * Q * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * oct; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / oct);
    const int64_t g = e - c * oct;
    const int x = (int)(g % Ph);
    const int y = (int)((g / Ph) % Qh);
    const int z = (int)(g / ((int64_t)Ph * Qh));
    const double2 a = in[c * PQR + x + (int64_t)P * (y + (int64_t)Q * z)];
    const double2 v = make_double2(a.x * scale, a.y * scale);
    if (g64) g64[e] = v;
    if (g32) g32[e] = make_float2((float)v.x, (float)v.y);
  }
}

void octant_spectrum(const double2* fN, int P, int Q, int R, double scale, double2* g64, float2* g32, cudaStream_t st) {
  const int64_t oct = (int64_t)(P / 2 + 1) * (Q / 2 + 1) * (R / 2 + 1);
  k_octant<<<(int)std::min<int64_t>(ceil_div(6 * oct, 256), 152 * 32), 256, 0, st>>>(fN, P, Q, R, scale, g64, g32);
  VS_LAUNCH_CHECK();
}

// True when every odd tensor component vanishes exactly on its zero-offset
// plane: then the embedded tensor is exactly even/odd along each axis and its
// spectrum (and the circulant blocks) inherit that parity.
bool toeplitz_has_exact_parity(const double* toep, int L, int M, int N) {
  const int64_t V = (int64_t)L * M * N;
  // component -> odd along x / y / z (xx, xy, xz, yy, yz, zz)
  const bool ox[6] = {false, true, true, false, false, false};
  const bool oy[6] = {false, true, false, false, true, false};
  const bool oz[6] = {false, false, true, false, true, false};
  for (int c = 0; c < 6; ++c) {
    const double* t = toep + 2 * c * V;
    for (int k = 0; k < N; ++k)
      for (int j = 0; j < M; ++j)
        for (int i = 0; i < L; ++i) {
          if (!((ox[c] && i == 0) || (oy[c] && j == 0) || (oz[c] && k == 0))) continue;
          const int64_t e = 2 * (i + (int64_t)L * (j + (int64_t)M * k));
          if (t[e] != 0.0 || t[e + 1] != 0.0) return false;
        }
  }
  return true;
}

void finalize_spectrum(const double2* fN, int64_t total, double scale, double2* g64, float2* g32, cudaStream_t st) {
  k_finalize<<<(int)std::min<int64_t>(ceil_div(total, 256), 152 * 32), 256, 0, st>>>(fN, total, scale, g64, g32);
  VS_LAUNCH_CHECK();
}

}  // namespace vs
