// Galerkin N-operator (JVIE) Toeplitz tensor on the device: the far- and
// medium-cell face-pair cubatures of assembly_nop_const.m:44-92 (the
// reference runs them as MATLAB parfor loops over mexcubature_nop_const,
// cubature_nop_const.cpp:8-124) and the projection onto the 6 tensor
// components (assembly_nop_const.m:150-165).  The singular near block
// (offsets < 2 per axis, assembly_nop_const.m:94-146) is supplied by the caller.
//
// One warp per offset m: for each of the 21 distinct (observation, source)
// face pairs the lanes stride over the Np*Np point pairs of the tensor
// Gauss-Legendre rule, summing w_p w_q exp(-i ko R)/R in FP64; a shuffle tree
// leaves every pair's sum in every lane, and lane c adds it into component c
// of G = sum_kl J_kl P_klc / (4 pi) with J = dx^4 I and I_kl the pair sum that
// entry (k, l) equals (the 15 copied entries folded into a per-pair
// projection).  Cells with every offset < 5 use the 10 x 10 rule, the others
// the 4 x 4 rule.
#include "vs_internal.h"

#include <vector>

namespace vs {

namespace {

constexpr int kNopPairs = 21;
constexpr int kNopFar = 4, kNopMedium = 10, kNopMediumCells = 5;

struct NopConst {
  double face[6][9];        // per face: vertex 1, edge 1->2, edge 1->4 (cube_faces.m)
  double proj[6][6][6];     // vector_projection.m
  double wf[16], uf[16], vf[16];     // 4 x 4 rule (gauss_2d.m)
  double wm[100], um[100], vm[100];  // 10 x 10 rule
  int obs[kNopPairs], src[kNopPairs];
  double pproj[kNopPairs][6];  // sum of proj[k][l][c] over the entries (k, l) that equal pair p
};
__constant__ NopConst c_nop;

// Sum over the np x np pairs of 2-D rule points (np = points per face).
__device__ __forceinline__ double2 nop_pair(int pr, const double* W, const double* U, const double* V, int np,
                                            const double rm[3], double ko) {
  const double* fo = c_nop.face[c_nop.obs[pr]];
  const double* fs = c_nop.face[c_nop.src[pr]];
  double re = 0, im = 0;
  const int n2 = np * np;
  for (int e = threadIdx.x & 31; e < n2; e += 32) {
    const int ip = e / np, iq = e - ip * np;
    double d2 = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double rp = fo[j] + fo[3 + j] * U[ip] + fo[6 + j] * V[ip] + rm[j];
      const double rq = fs[j] + fs[3 + j] * U[iq] + fs[6 + j] * V[iq];
      const double d = rq - rp;
      d2 += d * d;
    }
    const double R = sqrt(d2);
    double s, c;
    sincos(ko * R, &s, &c);
    const double wt = W[ip] * W[iq] / R;
    re += wt * c;
    im -= wt * s;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, off);
    im += __shfl_xor_sync(0xffffffffu, im, off);
  }
  return make_double2(re, im);
}

__global__ void __launch_bounds__(128) k_nop(int L, int M, int N, double ko, double dx, int nL, int nM, int nN,
                                             const double2* __restrict__ near, double2* __restrict__ G) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t V = (int64_t)L * M * N;
  if (w >= V) return;
  const int mx = (int)(w % L), my = (int)((w / L) % M), mz = (int)(w / ((int64_t)L * M));
  const int c = lane < 6 ? lane : 0;
  double re = 0, im = 0;
  if (mx < nL && my < nM && mz < nN) {
    if (near && lane < 6) {
      const int64_t nb = (int64_t)nL * nM * nN, cell = mx + (int64_t)nL * (my + (int64_t)nM * mz);
      for (int k = 0; k < 6; ++k)
        for (int l = 0; l < 6; ++l) {
          const double2 v = near[cell + nb * (k + 6 * l)];
          const double pk = c_nop.proj[k][l][c];
          re += v.x * pk;
          im += v.y * pk;
        }
    }
  } else {
    const bool medium = mx < kNopMediumCells && my < kNopMediumCells && mz < kNopMediumCells;
    const double* Wr = medium ? c_nop.wm : c_nop.wf;
    const double* Ur = medium ? c_nop.um : c_nop.uf;
    const double* Vr = medium ? c_nop.vm : c_nop.vf;
    const int np = medium ? kNopMedium * kNopMedium : kNopFar * kNopFar;  // 2-D points per face
    const double rm[3] = {mx * dx, my * dx, mz * dx};
    const double s4 = dx * dx * dx * dx;
    for (int pr = 0; pr < kNopPairs; ++pr) {
      const double2 v = nop_pair(pr, Wr, Ur, Vr, np, rm, ko);
      const double q = s4 * c_nop.pproj[pr][c];
      re += v.x * q;
      im += v.y * q;
    }
  }
  if (lane < 6) {
    const double s = 1.0 / (4.0 * M_PI);
    G[w + V * lane] = make_double2(re * s, im * s);
  }
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on the three-term
// recurrence, from the Chebyshev-like initial guesses).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0);
  w.assign(n, 0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double pn = n == 1 ? z : p1, pn1 = n == 1 ? 1 : p0;
      dp = n * (z * pn - pn1) / (z * z - 1);
      const double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2 / ((1 - z * z) * dp * dp);
  }
}

void rule_2d(int n, double* W, double* U, double* Vv) {
  std::vector<double> x, w;
  gauss_legendre(n, x, w);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      W[i * n + j] = w[i] * w[j] / 4;
      U[i * n + j] = (x[i] + 1) / 2;
      Vv[i * n + j] = (x[j] + 1) / 2;
    }
}

NopConst make_nop_const(double dx) {
  NopConst h{};
  // faces -x, +x, -y, +y, -z, +z: vertices 1, 2, 4 (cube_faces.m)
  const double v1[6][3] = {{0, 0, 0}, {dx, 0, 0}, {0, 0, 0}, {0, dx, 0}, {0, 0, 0}, {0, 0, dx}};
  const double v2[6][3] = {{0, dx, 0}, {dx, dx, 0}, {dx, 0, 0}, {dx, dx, 0}, {dx, 0, 0}, {dx, 0, dx}};
  const double v4[6][3] = {{0, 0, dx}, {dx, 0, dx}, {0, 0, dx}, {0, dx, dx}, {0, dx, 0}, {0, dx, dx}};
  for (int f = 0; f < 6; ++f)
    for (int j = 0; j < 3; ++j) {
      h.face[f][j] = v1[f][j];
      h.face[f][3 + j] = v2[f][j] - v1[f][j];
      h.face[f][6 + j] = v4[f][j] - v1[f][j];
    }
  // P(k,l,c) = (k x e_a).(l x e_b), k,l in {-x,+x,-y,+y,-z,+z}, c in (xx,xy,xz,yy,yz,zz)
  const int nrm[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  const int ab[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  auto cross = [](const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  for (int k = 0; k < 6; ++k)
    for (int l = 0; l < 6; ++l)
      for (int c = 0; c < 6; ++c) {
        const double kk[3] = {(double)nrm[k][0], (double)nrm[k][1], (double)nrm[k][2]};
        const double ll[3] = {(double)nrm[l][0], (double)nrm[l][1], (double)nrm[l][2]};
        double ea[3] = {0, 0, 0}, eb[3] = {0, 0, 0}, u[3], v[3];
        ea[ab[c][0]] = 1;
        eb[ab[c][1]] = 1;
        cross(kk, ea, u);
        cross(ll, eb, v);
        h.proj[k][l][c] = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
      }
  rule_2d(kNopFar, h.wf, h.uf, h.vf);
  rule_2d(kNopMedium, h.wm, h.um, h.vm);
  // the 21 distinct face pairs (cubature_nop_const.cpp:32-35) and the entries
  // copied from them (cubature_nop_const.cpp:100-118)
  const int obs[kNopPairs] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5};
  const int src[kNopPairs] = {0, 1, 2, 3, 4, 5, 0, 2, 3, 4, 5, 2, 3, 4, 5, 2, 4, 5, 4, 5, 4};
  int jidx[6][6];
  for (int k = 0; k < 6; ++k)
    for (int l = 0; l < 6; ++l) jidx[k][l] = -1;
  for (int p = 0; p < kNopPairs; ++p) {
    h.obs[p] = obs[p];
    h.src[p] = src[p];
    jidx[obs[p]][src[p]] = p;
  }
  const int cp[15][4] = {{1, 1, 0, 0}, {2, 0, 1, 3}, {2, 1, 0, 3}, {3, 0, 1, 2}, {3, 1, 0, 2},
                         {3, 3, 2, 2}, {4, 0, 1, 5}, {4, 1, 0, 5}, {4, 2, 3, 5}, {4, 3, 2, 5},
                         {5, 0, 1, 4}, {5, 1, 0, 4}, {5, 2, 3, 4}, {5, 3, 2, 4}, {5, 5, 4, 4}};
  for (const auto& c : cp) jidx[c[0]][c[1]] = jidx[c[2]][c[3]];
  for (int k = 0; k < 6; ++k)
    for (int l = 0; l < 6; ++l) {
      VS_REQUIRE(jidx[k][l] >= 0, "face-pair table incomplete");
      for (int c = 0; c < 6; ++c) h.pproj[jidx[k][l]][c] += h.proj[k][l][c];
    }
  return h;
}

}  // namespace

// The rule, face and projection tables live in one __constant__ block, so
// calls from concurrent host threads are serialised until their kernel is done.
void nop_assemble_device(int L, int M, int N, double ko, double dx, const double2* near, double2* G,
                         cudaStream_t st) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  const NopConst h = make_nop_const(dx);
  VS_CUDA(cudaMemcpyToSymbolAsync(c_nop, &h, sizeof(NopConst), 0, cudaMemcpyHostToDevice, st));
  const int64_t V = (int64_t)L * M * N;
  const int threads = 128;
  const int64_t blocks = (V * 32 + threads - 1) / threads;
  VS_REQUIRE(blocks < (1ll << 31), "grid too large");
  k_nop<<<(unsigned)blocks, threads, 0, st>>>(L, M, N, ko, dx, std::min(2, L), std::min(2, M), std::min(2, N),
                                             near, G);
  VS_LAUNCH_CHECK();
  VS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace vs
