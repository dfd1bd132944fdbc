// Excitation, extinction cross section and its gradient on the device.
//
//  * plane wave E0 exp(i k.r) evaluated at the operator's unknowns
//    (PlaneWavePointWise.m:7-19 followed by the Einc(idx3) gather of
//    main_DDA.m:81), FP64;
//  * C_ext = 4 pi ko dV / |E0|^2 sum_j Im(conj(Einc_j) . P_j) (Draine & Flatau,
//    JOSA A 11 (1994), eq. 8, with the dipole moment p = dV P of the
//    reference's unknown);
//  * dC_ext/d eps_j from the forward solution P and the adjoint solution lam of
//    A^T lam = conj(Einc): with A = diag(1/alpha_LDR(eps)) - dV G,
//    dC/d eps_j = -c Im/Re( d(1/alpha)/d eps_j * sum_comp lam_j P_j ).
#include "vs_internal.h"

namespace vs {

__global__ void k_plane_wave(const int* __restrict__ pos2grid, int64_t n3, int L, int M, int N,
                             const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                             double kx, double ky, double kz, double2 e0, double2 e1, double2 e2, double2* __restrict__ b) {
  const int64_t V = (int64_t)L * M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = pos2grid[e];
    const int c = (int)(g / V);
    const int64_t v = g - c * V;
    const int i = (int)(v % L), j = (int)((v / L) % M), k = (int)(v / ((int64_t)L * M));
    const double ph = kx * x[i] + ky * y[j] + kz * z[k];
    double sn, cs;
    sincos(ph, &sn, &cs);
    const double2 a = c == 0 ? e0 : (c == 1 ? e1 : e2);
    b[e] = make_double2(a.x * cs - a.y * sn, a.x * sn + a.y * cs);
  }
}

void plane_wave_device(const vs_op& op, const double* x, const double* y, const double* z, const double kvec[3],
                       const double2 E0[3], double2* b, cudaStream_t st) {
  k_plane_wave<<<(int)std::min<int64_t>(ceil_div(op.n3, 256), 152 * 16), 256, 0, st>>>(
      op.pos2grid.as<int>(), op.n3, op.L, op.M, op.N, x, y, z, kvec[0], kvec[1], kvec[2], E0[0], E0[1], E0[2], b);
  VS_LAUNCH_CHECK();
}

__global__ void k_conj(const double2* __restrict__ a, double2* __restrict__ b, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    b[e] = make_double2(a[e].x, -a[e].y);
}

void conj_device(const double2* a, double2* b, int64_t n, cudaStream_t st) {
  k_conj<<<(int)std::min<int64_t>(ceil_div(n, 256), 152 * 16), 256, 0, st>>>(a, b, n);
  VS_LAUNCH_CHECK();
}

// sum_e Im(conj(E_e) P_e) into out[blockIdx.x]; the host sums the partials.
__global__ void k_cext_partial(const double2* __restrict__ P, const double2* __restrict__ E, int64_t n,
                               double* __restrict__ out) {
  __shared__ double sm[256];
  double acc = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    acc += E[e].x * P[e].y - E[e].y * P[e].x;
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sm[0];
}

double cext_device(const double2* P, const double2* E, int64_t n, double scale, cudaStream_t st) {
  const int blocks = 256;
  DevBuf part;
  part.alloc(blocks * sizeof(double));
  k_cext_partial<<<blocks, 256, 0, st>>>(P, E, n, part.as<double>());
  VS_LAUNCH_CHECK();
  std::vector<double> h(blocks);
  VS_CUDA(cudaMemcpyAsync(h.data(), part.p, blocks * sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  double s = 0;
  for (double v : h) s += v;
  return s * scale;
}

// grad_re/grad_im[j] = -c Im/Re( dainv(eps_j) sum_comp lam P ), unknowns in idx3
// order [voxels; voxels; voxels].
__global__ void k_cext_grad(const double2* __restrict__ P, const double2* __restrict__ lam,
                            const double2* __restrict__ eps, int64_t nvox, double c, double bterm,
                            double* __restrict__ gre, double* __restrict__ gim) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nvox; j += (int64_t)gridDim.x * blockDim.x) {
    double2 lp = make_double2(0, 0);
#pragma unroll
    for (int k = 0; k < 3; ++k) lp = cadd(lp, cmul(lam[j + k * nvox], P[j + k * nvox]));
    // d(1/alpha_LDR)/d eps = -4 pi/(eps-1)^2 + (b2 + b3 S)(k d)^2
    const double2 em1 = make_double2(eps[j].x - 1.0, eps[j].y);
    const double2 sq = cmul(em1, em1);
    const double den = sq.x * sq.x + sq.y * sq.y;
    const double2 inv = make_double2(sq.x / den, -sq.y / den);
    const double2 da = make_double2(-4.0 * M_PI * inv.x + bterm, -4.0 * M_PI * inv.y);
    const double2 g = cmul(da, lp);
    gre[j] = -c * g.y;
    gim[j] = -c * g.x;
  }
}

void cext_grad_device(const double2* P, const double2* lam, const double2* eps, int64_t nvox, double c, double bterm,
                      double* gre, double* gim, cudaStream_t st) {
  k_cext_grad<<<(int)std::min<int64_t>(ceil_div(nvox, 256), 152 * 16), 256, 0, st>>>(P, lam, eps, nvox, c, bterm, gre,
                                                                                      gim);
  VS_LAUNCH_CHECK();
}

}  // namespace vs
