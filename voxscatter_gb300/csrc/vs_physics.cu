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


// ---- whole-domain field and far field ---------------------------------------

__global__ void k_iota(int* __restrict__ m, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    m[e] = (int)e;
}

const int* domain_map(vs_op& op, cudaStream_t st) {
  if (!op.map_all.p) {
    op.map_all.alloc(3 * op.V * sizeof(int));
    k_iota<<<(int)std::min<int64_t>(ceil_div(3 * op.V, 256), 152 * 16), 256, 0, st>>>(op.map_all.as<int>(), 3 * op.V);
    VS_LAUNCH_CHECK();
  }
  return op.map_all.as<int>();
}

// Pout(idx3) = vsol of main_DDA.m:136-138: the grid is cleared, then the
// unknowns are written to their grid entries (two launches).
template <typename C>
__global__ void k_zero_grid(int64_t ng, C* __restrict__ grid) {
  grid += blockIdx.y * ng;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x)
    grid[g] = C{0, 0};
}

template <typename C>
__global__ void k_fill_grid(const int* __restrict__ pos2grid, const C* __restrict__ x, int64_t n3, int64_t ng,
                            C* __restrict__ grid) {
  const int rhs = blockIdx.y;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3; e += (int64_t)gridDim.x * blockDim.x)
    grid[rhs * ng + pos2grid[e]] = x[rhs * n3 + e];
}

template <typename C>
void to_grid(const vs_op& op, const C* x, C* grid, int nrhs, cudaStream_t st) {
  const int64_t ng = 3 * op.V;
  const dim3 g1((unsigned)std::min<int64_t>(ceil_div(ng, 256), 152 * 8), nrhs);
  k_zero_grid<C><<<g1, 256, 0, st>>>(ng, grid);
  VS_LAUNCH_CHECK();
  const dim3 g2((unsigned)std::min<int64_t>(ceil_div(op.n3, 256), 152 * 8), nrhs);
  k_fill_grid<C><<<g2, 256, 0, st>>>(op.pos2grid.as<int>(), x, op.n3, ng, grid);
  VS_LAUNCH_CHECK();
}
template void to_grid<float2>(const vs_op&, const float2*, float2*, int, cudaStream_t);
template void to_grid<double2>(const vs_op&, const double2*, double2*, int, cudaStream_t);

// E = Einc - y + P / chi over the grid (main_DDA.m:139-148: Eout(idx3) = P/CHI,
// E = Einc - Etemp + Eout with Etemp the whole-domain MVP of Pout)
template <typename C>
__global__ void k_field_combine(const C* __restrict__ einc, const C* __restrict__ y, const C* __restrict__ pg,
                                double2 inv_chi, int64_t n, double2* __restrict__ e) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const double px = pg[g].x, py = pg[g].y;
    e[g] = make_double2((double)einc[g].x - (double)y[g].x + px * inv_chi.x - py * inv_chi.y,
                        (double)einc[g].y - (double)y[g].y + px * inv_chi.y + py * inv_chi.x);
  }
}

template <typename C>
void field_combine(const C* einc, const C* y, const C* pgrid, double2 inv_chi, int64_t n, double2* e,
                   cudaStream_t st) {
  k_field_combine<C><<<(int)std::min<int64_t>(ceil_div(n, 256), 152 * 16), 256, 0, st>>>(einc, y, pgrid, inv_chi,
                                                                                          n, e);
  VS_LAUNCH_CHECK();
}
template void field_combine<float2>(const float2*, const float2*, const float2*, double2, int64_t, double2*,
                                    cudaStream_t);
template void field_combine<double2>(const double2*, const double2*, const double2*, double2, int64_t, double2*,
                                     cudaStream_t);

// Far-field amplitude of the dipoles p_j = dV P_j in unit direction n:
//   F(n) = ko^2 dV (I - n n^T) sum_j P_j exp(-i ko n.r_j)
// (the far zone of the DDA Green tensor of getOPERATOR_DDA.m:99-113,
// E_sca -> exp(i ko r)/r F(n); Draine & Flatau, JOSA A 11 (1994) 1491).
// One CTA per (direction, right-hand side).  The phase factorises over the
// grid axes, so the CTA tabulates exp(-i ko n_x x_i), exp(-i ko n_y y_j) and
// exp(-i ko n_z z_k) once (FP64 sincos) and forms each voxel's phase with two
// complex products; sums in FP64, fixed-order tree reduction.
__global__ void __launch_bounds__(256) k_far_field(const int* __restrict__ pos2grid, const double2* __restrict__ P,
                                                   int64_t n3, int L, int M, int N, const double* __restrict__ xs,
                                                   const double* __restrict__ ys, const double* __restrict__ zs,
                                                   const double* __restrict__ dirs, double ko, double scale,
                                                   double2* __restrict__ F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* ph = reinterpret_cast<double2*>(smem_raw);  // [L + M + N]
  __shared__ double2 red[3][256];
  const int d = blockIdx.x, rhs = blockIdx.y;
  const double nx = dirs[3 * d], ny = dirs[3 * d + 1], nz = dirs[3 * d + 2];
  for (int i = threadIdx.x; i < L + M + N; i += blockDim.x) {
    const double arg = i < L ? -ko * nx * xs[i] : (i < L + M ? -ko * ny * ys[i - L] : -ko * nz * zs[i - L - M]);
    double sn, cs;
    sincos(arg, &sn, &cs);
    ph[i] = make_double2(cs, sn);
  }
  __syncthreads();
  const int64_t V = (int64_t)L * M * N;
  const double2* Pr = P + (int64_t)rhs * n3;
  double2 s[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  for (int64_t e = threadIdx.x; e < n3; e += blockDim.x) {
    const int64_t g = pos2grid[e];
    const int c = (int)(g / V);
    const int64_t v = g - c * V;
    const int i = (int)(v % L), j = (int)((v / L) % M), k = (int)(v / ((int64_t)L * M));
    const double2 a = ph[i], b = ph[L + j], w = ph[L + M + k];
    const double2 ab = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    const double2 p = make_double2(ab.x * w.x - ab.y * w.y, ab.x * w.y + ab.y * w.x);
    const double2 x = Pr[e];
    const double2 t = make_double2(x.x * p.x - x.y * p.y, x.x * p.y + x.y * p.x);
    s[c].x += t.x;
    s[c].y += t.y;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) red[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        red[c][threadIdx.x].x += red[c][threadIdx.x + h].x;
        red[c][threadIdx.x].y += red[c][threadIdx.x + h].y;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double2 a0 = red[0][0], a1 = red[1][0], a2 = red[2][0];
    const double ndr = nx * a0.x + ny * a1.x + nz * a2.x, ndi = nx * a0.y + ny * a1.y + nz * a2.y;
    double2* out = F + ((int64_t)rhs * gridDim.x + d) * 3;
    out[0] = make_double2(scale * (a0.x - nx * ndr), scale * (a0.y - nx * ndi));
    out[1] = make_double2(scale * (a1.x - ny * ndr), scale * (a1.y - ny * ndi));
    out[2] = make_double2(scale * (a2.x - nz * ndr), scale * (a2.y - nz * ndi));
  }
}

void far_field_device(const vs_op& op, const double2* P, int nrhs, const double* xs, const double* ys,
                      const double* zs, const double* dirs, int ndir, double ko, double dV, double2* F,
                      cudaStream_t st) {
  const size_t smem = (size_t)(op.L + op.M + op.N) * sizeof(double2);
  VS_REQUIRE(smem <= 160 * 1024, "grid too long for the far-field phase tables");
  set_kernel_smem((const void*)k_far_field, smem);
  k_far_field<<<dim3(ndir, nrhs), 256, smem, st>>>(op.pos2grid.as<int>(), P, op.n3, op.L, op.M, op.N, xs, ys, zs,
                                                   dirs, ko, ko * ko * dV, F);
  VS_LAUNCH_CHECK();
}

}  // namespace vs
