// Chan-Olkin 2-level circulant preconditioner on the device.
//
// Build (FP64 up to the inversion):
//   level 1: T. Chan optimal-circulant average along x + FFT_x   (circ_1_level.m:5-90)
//   level 2: the same along y + FFT_y                              (circ_2_level.m:5-80)
//   blocks : per (i,j) the 3N x 3N matrix of N x N Toeplitz pieces  (circ_2_level.m:82-154)
//            shifted as shift*I - diag(d)*C                        (main_DDA.m:109,
//                                                                   scatteringHumanHead.m:181)
//            and inverted by Gauss-Jordan with partial pivoting in shared memory,
//            in FP32 (mixed path) and/or FP64.
// Apply (mvp_circ_2_level.m:4-22): gather + FFT_x, FFT_y, block GEMV, IFFT_y,
// IFFT_x + scatter.  The 1/(L*M) of the two inverse FFTs is folded into the
// stored inverse blocks.
#include "vs_pipeline.cuh"

namespace vs {

// sign of the (n+1-i)/n term per component, circ_1_level.m:14,29,42,55,69,84
__constant__ int c_s1[6] = {+1, -1, -1, +1, +1, +1};
// same for circ_2_level.m:14,27,38,51,63,76
__constant__ int c_s2[6] = {+1, -1, +1, +1, -1, +1};

__global__ void k_chan_x(const double2* __restrict__ A, double2* __restrict__ out, int L, int M, int N) {
  const int64_t V = (int64_t)L * M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * V; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / V);
    const int i = (int)((e - c * V) % L);
    double2 r;
    if (i == 0) {
      r = A[e];
    } else {
      const double w1 = c_s1[c] * (double)(L - i) / L, w2 = (double)i / L;
      const double2 a = A[e], b = A[e - i + (L - i)];
      r = make_double2(w1 * a.x + w2 * b.x, w1 * a.y + w2 * b.y);
    }
    out[e] = r;
  }
}

__global__ void k_chan_y(const double2* __restrict__ A, double2* __restrict__ out, int L, int M, int N) {
  const int64_t V = (int64_t)L * M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * V; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / V);
    const int j = (int)(((e - c * V) / L) % M);
    double2 r;
    if (j == 0) {
      r = A[e];
    } else {
      const double w1 = c_s2[c] * (double)(M - j) / M, w2 = (double)j / M;
      const double2 a = A[e], b = A[e + (int64_t)(M - 2 * j) * L];
      r = make_double2(w1 * a.x + w2 * b.x, w1 * a.y + w2 * b.y);
    }
    out[e] = r;
  }
}

void circ_levels_device(int L, int M, int N, const double2* toep, double2* lev1, double2* lev2, const FftAxis& axL,
                        const FftAxis& axM, cudaStream_t st) {
  const int64_t V = (int64_t)L * M * N;
  const int blocks = (int)std::min<int64_t>(ceil_div(6 * V, 256), 152 * 32);
  k_chan_x<<<blocks, 256, 0, st>>>(toep, lev1, L, M, N);
  VS_LAUNCH_CHECK();
  fft_axis0<double, false>(lev1, L, (int64_t)M * N * 6, axL, st);
  k_chan_y<<<blocks, 256, 0, st>>>(lev1, lev2, L, M, N);
  VS_LAUNCH_CHECK();
  fft_strided<double, false>(lev2, L, M, L, N * 6, (int64_t)L * M, 1, 0, axM, st);
}

__device__ __forceinline__ int comp_pair(int a, int b) {
  const int t[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  return t[a][b];
}

__host__ __device__ __forceinline__ float2 crecip(float2 a) {
  const float d = a.x * a.x + a.y * a.y;
  return make_float2(a.x / d, -a.y / d);
}
__host__ __device__ __forceinline__ double2 crecip(double2 a) {
  const double d = a.x * a.x + a.y * a.y;
  return make_double2(a.x / d, -a.y / d);
}

// Entry (p, q) of block (i, j): shift*[p==q] - d_p * C_ij(p, q), where C_ij is
// the 3x3 arrangement of N x N Toeplitz pieces of circ_2_level.m:82-154 (the
// (a, b) piece uses component comp_pair(a, b); entries above the diagonal of
// an xz / yz piece change sign).
__device__ __forceinline__ double2 block_entry(const double2* __restrict__ lev2, int L, int M, int N, int i, int j, int p,
                                               int q, double2 shift, const double2* __restrict__ dvec, double2 dscal) {
  const int a = p / N, zp = p - a * N, b = q / N, zq = q - b * N;
  const int c = comp_pair(a, b);
  const bool negcol = (a == 2) != (b == 2);
  int dz = zp - zq;
  double sg = 1.0;
  if (dz < 0) dz = -dz;
  else if (negcol && dz > 0) sg = -1.0;
  const double2 v = lev2[i + (int64_t)L * (j + (int64_t)M * (dz + (int64_t)N * c))];
  const double2 dd = dvec ? dvec[p] : dscal;
  double2 e = cmul(dd, v);
  e.x *= -sg;
  e.y *= -sg;
  if (p == q) { e.x += shift.x; e.y += shift.y; }
  return e;
}

// One CTA per block (i, j) = (blockIdx.x, blockIdx.y).  With invert = false
// the assembled matrix is stored as is (used to return circ_2_level's blocks).
template <typename T>
__global__ void __launch_bounds__(256) k_assemble_invert(const double2* __restrict__ lev2, int L, int M, int N,
                                                         double2 shift, const double2* __restrict__ dvec,
                                                         double2 dscal, int invert, int colmajor, double scale,
                                                         cplx_t<T>* __restrict__ out, int* __restrict__ status,
                                                         int Lb) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = 3 * N;
  C* A = reinterpret_cast<C*>(smem_raw);
  C* colk = A + n * n;
  int* perm = reinterpret_cast<int*>(colk + n);
  __shared__ int s_piv;
  __shared__ T s_pmag;
  const int i = blockIdx.x, j = blockIdx.y;
  for (int u = threadIdx.x; u < n * n; u += blockDim.x) {
    const int p = u / n, q = u - p * n;
    A[u] = ccast<C>(block_entry(lev2, L, M, N, i, j, p, q, shift, dvec, dscal));
  }
  __syncthreads();
  if (invert) {
    for (int k = 0; k < n; ++k) {
      if (threadIdx.x < 32) {
        T best = -1;
        int bi = k;
        for (int r = k + threadIdx.x; r < n; r += 32) {
          const C a = A[r * n + k];
          const T m = a.x * a.x + a.y * a.y;
          if (m > best) { best = m; bi = r; }
        }
        for (int off = 16; off; off >>= 1) {
          const T ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (threadIdx.x == 0) {
          s_piv = bi;
          s_pmag = best;
          perm[k] = bi;
        }
      }
      __syncthreads();
      const int p = s_piv;
      if (threadIdx.x == 0 && !(s_pmag > 0)) atomicOr(status, 1);
      if (p != k) {
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
          const C t = A[k * n + q];
          A[k * n + q] = A[p * n + q];
          A[p * n + q] = t;
        }
      }
      __syncthreads();
      for (int r = threadIdx.x; r < n; r += blockDim.x) colk[r] = A[r * n + k];
      __syncthreads();
      const C rinv = crecip(colk[k]);
      for (int q = threadIdx.x; q < n; q += blockDim.x) A[k * n + q] = (q == k) ? rinv : cmul(A[k * n + q], rinv);
      __syncthreads();
      for (int u = threadIdx.x; u < n * n; u += blockDim.x) {
        const int r = u / n;
        if (r == k) continue;
        const int q = u - r * n;
        const C base = (q == k) ? czero<C>() : A[u];
        A[u] = csub(base, cmul(colk[r], A[k * n + q]));
      }
      __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k) {
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
          const C t = A[r * n + k];
          A[r * n + k] = A[r * n + p];
          A[r * n + p] = t;
        }
      }
      __syncthreads();
    }
  }
  C* o = out + ((int64_t)i + (int64_t)Lb * j) * n * n;
  for (int u = threadIdx.x; u < n * n; u += blockDim.x) {
    const int p = u / n, q = u - p * n;
    const C a = A[u];
    if (!(isfinite(a.x) && isfinite(a.y))) atomicOr(status, 2);
    o[colmajor ? q * n + p : u] = cscale(a, (T)scale);
  }
}

size_t assemble_smem(int N, size_t csize) {
  const int n = 3 * N;
  return (size_t)n * n * csize + n * csize + n * sizeof(int) + 16;
}

// Element-wise assembly of all stored blocks, for any block size: entry (p, q)
// of block b = i + Lb*j goes to out[b*n*n + q*n + p] (colmajor) or
// out[b*n*n + p*n + q], times scale.
template <typename T>
__global__ void k_assemble(const double2* __restrict__ lev2, int L, int M, int N, double2 shift,
                           const double2* __restrict__ dvec, double2 dscal, int colmajor, double scale,
                           cplx_t<T>* __restrict__ out, int Lb, int Mb) {
  const int n = 3 * N;
  const int64_t nn = (int64_t)n * n, total = nn * Lb * Mb;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int u = (int)(e - b * nn);
    const int hi = u / n, lo = u - hi * n;
    const int p = colmajor ? lo : hi, q = colmajor ? hi : lo;
    const int j = (int)(b / Lb), i = (int)(b - (int64_t)j * Lb);
    const double2 v = block_entry(lev2, L, M, N, i, j, p, q, shift, dvec, dscal);
    out[e] = ccast<cplx_t<T>>(make_double2(v.x * scale, v.y * scale));
  }
}

// Blocked Gauss-Jordan inversion with partial pivoting of nmat row-major n x n
// matrices held in global memory, one CTA per matrix at a time (persistent
// over the batch).  For blocks too large for the shared-memory kernel.
//
// Columns are processed in panels of NB.  A panel (all n rows) is loaded into
// shared memory and reduced by the unblocked in-place steps (pivot search down
// the column among the rows not yet used, row swap, scale the pivot row,
// eliminate the column from every other row; the eliminated column is
// replaced by the corresponding column of the inverse).  Afterwards the panel
// holds [A_KK^-1 ; -A_OK A_KK^-1] for the pivot rows K of the panel and the
// other rows O, and every column c outside the panel transforms as
//     c_new = (c with rows K zeroed) + Panel * c_K,
// with the panel's row swaps applied to c first -- a rank-NB update done as a
// register-tiled complex GEMM over column tiles of TQ = 16*CN.  The swaps of
// one panel move only rows of K and rows swapped in from below the panel, and
// a row below the panel always receives a row of K, so each column tile
// gathers its new K rows and the changed rows below into shared memory before
// it is overwritten.  After the last panel the column interchanges are undone
// in one composed permutation, the result is scaled, and non-finite entries
// or a zero pivot set status bits 2 / 1.
template <typename T, int NB, int CN>
__global__ void __launch_bounds__(256) k_gj_blocked(cplx_t<T>* __restrict__ mats, int n, int64_t nmat, double scale,
                                                    int* __restrict__ status) {
  using C = cplx_t<T>;
  constexpr int TQ = 16 * CN, RM = 4, PS = NB + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* P = reinterpret_cast<C*>(smem_raw);  // [n][PS]
  C* Bsw = P + (size_t)n * PS;            // [NB][TQ]  new pivot rows of a column tile
  C* Osw = Bsw + NB * TQ;                 // [NB][TQ]  new rows below the panel that a swap changed
  C* colk = Osw + NB * TQ;                // [n]
  int* perm = reinterpret_cast<int*>(colk + n);
  int* rowsrc = perm + n;  // row r of the panel's result comes from row rowsrc[r]
  int* oidx = rowsrc + n;  // slot in Osw of a changed row below the panel, or -1
  int* olist = oidx + n;   // [NB]
  int* cmap = olist + NB;  // [n]
  __shared__ int s_piv, s_ocnt;
  __shared__ T s_pmag;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int64_t b = blockIdx.x; b < nmat; b += gridDim.x) {
    C* B = mats + b * (int64_t)n * n;
    for (int r = tid; r < n; r += blockDim.x) {
      rowsrc[r] = r;
      oidx[r] = -1;
    }
    for (int k0 = 0; k0 < n; k0 += NB) {
      const int nb = min(NB, n - k0);
      for (int u = tid; u < n * NB; u += blockDim.x) {
        const int r = u / NB, c = u - r * NB;
        P[r * PS + c] = c < nb ? B[(int64_t)r * n + k0 + c] : czero<C>();
      }
      __syncthreads();
      for (int kk = 0; kk < nb; ++kk) {
        const int k = k0 + kk;
        if (tid < 32) {
          T best = -1;
          int bi = k;
          for (int r = k + tid; r < n; r += 32) {
            const C a = P[r * PS + kk];
            const T m = a.x * a.x + a.y * a.y;
            if (m > best) { best = m; bi = r; }
          }
          for (int off = 16; off; off >>= 1) {
            const T ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
          }
          if (tid == 0) {
            s_piv = bi;
            s_pmag = best;
            perm[k] = bi;
            const int t = rowsrc[k];
            rowsrc[k] = rowsrc[bi];
            rowsrc[bi] = t;
          }
        }
        __syncthreads();
        const int p = s_piv;
        if (tid == 0 && !(s_pmag > 0)) atomicOr(status, 1);
        if (p != k && tid < NB) {
          const C t = P[k * PS + tid];
          P[k * PS + tid] = P[p * PS + tid];
          P[p * PS + tid] = t;
        }
        __syncthreads();
        for (int r = tid; r < n; r += blockDim.x) colk[r] = P[r * PS + kk];
        __syncthreads();
        const C rinv = crecip(colk[k]);
        if (tid < NB) P[k * PS + tid] = (tid == kk) ? rinv : cmul(P[k * PS + tid], rinv);
        __syncthreads();
        for (int u = tid; u < n * NB; u += blockDim.x) {
          const int r = u / NB, c = u - r * NB;
          if (r == k) continue;
          const C base = (c == kk) ? czero<C>() : P[r * PS + c];
          P[r * PS + c] = csub(base, cmul(colk[r], P[k * PS + c]));
        }
        __syncthreads();
      }
      if (tid == 0) {
        int cnt = 0;
        for (int kk = 0; kk < nb; ++kk) {
          const int p = perm[k0 + kk];
          if (p >= k0 + nb && oidx[p] < 0) {
            oidx[p] = cnt;
            olist[cnt++] = p;
          }
        }
        s_ocnt = cnt;
      }
      for (int u = tid; u < n * NB; u += blockDim.x) {
        const int r = u / NB, c = u - r * NB;
        if (c < nb) B[(int64_t)r * n + k0 + c] = P[r * PS + c];
      }
      __syncthreads();
      const int ocnt = s_ocnt, nrest = n - nb;
      for (int q0 = 0; q0 < nrest; q0 += TQ) {
        for (int u = tid; u < (nb + ocnt) * TQ; u += blockDim.x) {
          const int rr = u / TQ, qi = u - rr * TQ;
          const int qv = q0 + qi;
          if (qv >= nrest) continue;
          const int q = qv < k0 ? qv : qv + nb;
          if (rr < nb) Bsw[rr * TQ + qi] = B[(int64_t)rowsrc[k0 + rr] * n + q];
          else Osw[(rr - nb) * TQ + qi] = B[(int64_t)rowsrc[olist[rr - nb]] * n + q];
        }
        __syncthreads();
        for (int rs = 0; rs < n; rs += 16 * RM) {
          C acc[RM][CN];
#pragma unroll
          for (int m = 0; m < RM; ++m)
#pragma unroll
            for (int c = 0; c < CN; ++c) acc[m][c] = czero<C>();
#pragma unroll 4
          for (int kk = 0; kk < nb; ++kk) {
            C pv[RM], bv[CN];
#pragma unroll
            for (int m = 0; m < RM; ++m) {
              const int r = rs + ty + 16 * m;
              pv[m] = r < n ? P[r * PS + kk] : czero<C>();
            }
#pragma unroll
            for (int c = 0; c < CN; ++c) bv[c] = Bsw[kk * TQ + tx + 16 * c];
#pragma unroll
            for (int m = 0; m < RM; ++m)
#pragma unroll
              for (int c = 0; c < CN; ++c) acc[m][c] = cfma(pv[m], bv[c], acc[m][c]);
          }
#pragma unroll
          for (int m = 0; m < RM; ++m) {
            const int r = rs + ty + 16 * m;
            if (r >= n) continue;
            const bool inK = r >= k0 && r < k0 + nb;
            const int oi = oidx[r];
#pragma unroll
            for (int c = 0; c < CN; ++c) {
              const int qi = tx + 16 * c, qv = q0 + qi;
              if (qv >= nrest) continue;
              const int q = qv < k0 ? qv : qv + nb;
              C* dst = B + (int64_t)r * n + q;
              const C base = inK ? czero<C>() : (oi >= 0 ? Osw[oi * TQ + qi] : *dst);
              *dst = cadd(base, acc[m][c]);
            }
          }
        }
        __syncthreads();
      }
      for (int r = tid; r < n; r += blockDim.x) rowsrc[r] = r;
      if (tid < ocnt) oidx[olist[tid]] = -1;
      __syncthreads();
    }
    if (tid == 0) {
      for (int c = 0; c < n; ++c) cmap[c] = c;
      for (int k = n - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k) {
          const int t = cmap[k];
          cmap[k] = cmap[p];
          cmap[p] = t;
        }
      }
    }
    __syncthreads();
    for (int r0 = 0; r0 < n; r0 += PS) {
      const int nr = min(PS, n - r0);
      for (int u = tid; u < nr * n; u += blockDim.x) P[u] = B[(int64_t)r0 * n + u];
      __syncthreads();
      for (int u = tid; u < nr * n; u += blockDim.x) {
        const int rl = u / n, c = u - rl * n;
        const C a = cscale(P[rl * n + cmap[c]], (T)scale);
        if (!(isfinite(a.x) && isfinite(a.y))) atomicOr(status, 2);
        B[(int64_t)r0 * n + u] = a;
      }
      __syncthreads();
    }
  }
}

template <typename T>
constexpr int gj_cn() { return std::is_same<T, float>::value ? 4 : 2; }

size_t gj_blocked_smem(int n, size_t csize) {
  constexpr int NB = 32;
  const int TQ = 16 * (csize == sizeof(float2) ? 4 : 2);
  return ((size_t)n * (NB + 1) + 2ull * NB * TQ + n) * csize + (4ull * n + NB) * sizeof(int) + 64;
}

template <typename T>
void assemble_invert(const double2* lev2, int L, int M, int N, double2 shift, const double2* dvec, double2 dscal,
                     bool invert, bool colmajor, double scale, cplx_t<T>* out, int* status, cudaStream_t st,
                     bool sym, int lu) {
  const size_t smem = assemble_smem(N, sizeof(cplx_t<T>));
  const int Lb = sym ? L / 2 + 1 : L, Mb = sym ? M / 2 + 1 : M;
  const int n = 3 * N;
  const int64_t nmat = (int64_t)Lb * Mb;
  const bool fp32 = std::is_same<T, float>::value;
  // tensor cores when forced, and by default where the alternative is the
  // persistent CUDA-core kernel (blocks beyond the one-CTA shared-memory
  // kernel): measured faster there, slower than the shared-memory kernel below
  const bool use_tc = invert && fp32 && tc_invert_supported(n) &&
                      (lu == LU_TC || (lu == LU_AUTO && smem > 227 * 1024));
  if (use_tc) {
    VS_REQUIRE(colmajor, "tensor-core inversion produces column-major blocks");
    // the transposes assembled row-major; the inverse of A^T row-major is A^-1 column-major
    const int64_t total = nmat * n * n;
    const int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 152 * 64);
    k_assemble<T><<<blocks, 256, 0, st>>>(lev2, L, M, N, shift, dvec, dscal, 1, 1.0, out, Lb, Mb);
    VS_LAUNCH_CHECK();
    if constexpr (std::is_same<T, float>::value) invert_blocks_tc(out, n, nmat, scale, status, st);
    return;
  }
  if (!invert || smem > 227 * 1024) {
    // element-wise assembly; the inverse of A^T in row-major order is A^-1 in column-major order
    const int64_t total = nmat * n * n;
    const int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 152 * 64);
    k_assemble<T><<<blocks, 256, 0, st>>>(lev2, L, M, N, shift, dvec, dscal, (invert || colmajor) ? 1 : 0,
                                          invert ? 1.0 : scale, out, Lb, Mb);
    VS_LAUNCH_CHECK();
    if (!invert) return;
    VS_REQUIRE(colmajor, "large blocks are only produced column-major");
    const size_t gsm = gj_blocked_smem(n, sizeof(cplx_t<T>));
    if (gsm > 227 * 1024)
      throw Error(VS_ERR_UNSUPPORTED, "3N x 3N block of " + std::to_string(n) + " is too large to invert");
    auto k = k_gj_blocked<T, 32, gj_cn<T>()>;
    set_kernel_smem((const void*)k, gsm);
    int per_sm = 0;
    VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, gsm));
    int dev = 0, nsm = 0;
    VS_CUDA(cudaGetDevice(&dev));
    VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int grid = (int)std::min<int64_t>(nmat, (int64_t)nsm * std::max(per_sm, 1));
    k<<<grid, 256, gsm, st>>>(out, n, nmat, scale, status);
    VS_LAUNCH_CHECK();
    return;
  }
  auto k = k_assemble_invert<T>;
  set_kernel_smem((const void*)k, smem);
  k<<<dim3(Lb, Mb), 256, smem, st>>>(lev2, L, M, N, shift, dvec, dscal, invert ? 1 : 0, colmajor ? 1 : 0, scale, out,
                                     status, Lb);
  VS_LAUNCH_CHECK();
}
// In-place inversion of nmat n x n FP32 complex matrices already in device
// memory (either storage order: the inverse of the transpose is the
// transpose of the inverse), scaled by `scale`.
void invert_blocks_device(float2* mats, int n, int64_t nmat, int lu, double scale, int* status, cudaStream_t st) {
  if (nmat <= 0) return;
  if (lu != LU_CUDA && tc_invert_supported(n)) {
    invert_blocks_tc(mats, n, nmat, scale, status, st);
    return;
  }
  const size_t gsm = gj_blocked_smem(n, sizeof(float2));
  if (gsm > 227 * 1024)
    throw Error(VS_ERR_UNSUPPORTED, "block of " + std::to_string(n) + " is too large to invert");
  auto k = k_gj_blocked<float, 32, gj_cn<float>()>;
  set_kernel_smem((const void*)k, gsm);
  int per_sm = 0;
  VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, gsm));
  int dev = 0, nsm = 0;
  VS_CUDA(cudaGetDevice(&dev));
  VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)std::min<int64_t>(nmat, (int64_t)nsm * std::max(per_sm, 1));
  k<<<grid, 256, gsm, st>>>(mats, n, nmat, scale, status);
  VS_LAUNCH_CHECK();
}

template void assemble_invert<float>(const double2*, int, int, int, double2, const double2*, double2, bool, bool,
                                     double, float2*, int*, cudaStream_t, bool, int);
template void assemble_invert<double>(const double2*, int, int, int, double2, const double2*, double2, bool, bool,
                                      double, double2*, int*, cudaStream_t, bool, int);

// ---- apply: block GEMV on the (x,y)-frequency planes --------------------
// Inverse blocks are stored column-major (element (r, q) at q*n + r), so the
// threads that compute consecutive output rows read consecutive addresses of
// each column; each thread forms one full row sum, no cross-lane reduction.
// With sym, only blocks i <= L/2, j <= M/2 are stored; block (L-i, j) equals
// Dx B(i,j) Dx and (i, M-j) equals Dy B(i,j) Dy, Dx/Dy negating the x/y
// component entries, so the input and output entries of those components are
// negated around the product with the stored block.
template <typename T>
__global__ void __launch_bounds__(256) k_block_gemv(cplx_t<T>* __restrict__ t, const cplx_t<T>* __restrict__ inv, int L,
                                                    int M, int N, int ti, int64_t rhs_stride, const int* skip,
                                                    int sym, int skip_stride) {
  using C = cplx_t<T>;
  if (skip && skip[blockIdx.z * skip_stride]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = 3 * N;
  C* v = reinterpret_cast<C*>(smem_raw);
  C* o = v + ti * n;
  const int i0 = blockIdx.x * ti, j = blockIdx.y;
  C* tt = t + (int64_t)blockIdx.z * rhs_stride;
  const int64_t LM = (int64_t)L * M;
  const int Lb = sym ? L / 2 + 1 : L;
  const bool fy = sym && j > M / 2;
  const int js = fy ? M - j : j;
  for (int u = threadIdx.x; u < ti * n; u += blockDim.x) {
    const int s = u / ti, il = u - s * ti;
    const int i = i0 + il;
    // s = comp*N + z  ->  grid entry (i, j, z, comp)
    C val = (i < L) ? tt[i + (int64_t)L * j + LM * s] : czero<C>();
    const int comp = s / N;
    if ((comp == 0 && sym && i > L / 2) != (comp == 1 && fy)) { val.x = -val.x; val.y = -val.y; }
    v[il * n + s] = val;
  }
  __syncthreads();
  for (int rr = threadIdx.x; rr < ti * n; rr += blockDim.x) {
    const int il = rr / n, r = rr - il * n;
    const int i = i0 + il;
    if (i >= L) continue;
    const int is = (sym && i > L / 2) ? L - i : i;
    const C* A = inv + ((int64_t)is + (int64_t)Lb * js) * n * n + r;
    const C* x = v + il * n;
    C acc0 = czero<C>(), acc1 = czero<C>();
    int q = 0;
#pragma unroll 4
    for (; q + 1 < n; q += 2) {
      acc0 = cfma(__ldg(A + (int64_t)q * n), x[q], acc0);
      acc1 = cfma(__ldg(A + (int64_t)(q + 1) * n), x[q + 1], acc1);
    }
    if (q < n) acc0 = cfma(__ldg(A + (int64_t)q * n), x[q], acc0);
    C res = cadd(acc0, acc1);
    const int comp = r / N;
    if ((comp == 0 && sym && i > L / 2) != (comp == 1 && fy)) { res.x = -res.x; res.y = -res.y; }
    o[il * n + r] = res;
  }
  __syncthreads();
  for (int u = threadIdx.x; u < ti * n; u += blockDim.x) {
    const int s = u / ti, il = u - s * ti;
    const int i = i0 + il;
    if (i < L) tt[i + (int64_t)L * j + LM * s] = o[il * n + s];
  }
}

// Quadrant-symmetric apply: CTA (blockIdx.x, blockIdx.y, blockIdx.z) owns the
// stored blocks is = blockIdx.x*ti + il (il < ti), js = blockIdx.y, and the
// right-hand sides rhs = blockIdx.z*RG + rg (rg < RG).  Each stored block is
// applied to the up to four frequencies (is, js), (L-is, js), (is, M-js),
// (L-is, M-js) that share it, for all RG right-hand sides: W = 4*RG vectors
// per block, so every element of a stored block read from memory feeds W
// products.  Variant v has flips fx = v&1, fy = v>>1 (negate the x / y
// component entries of the input and of the output).
template <typename T, bool PAIR, int RG>
__global__ void __launch_bounds__(256) k_block_gemv_sym(cplx_t<T>* __restrict__ t, const cplx_t<T>* __restrict__ inv,
                                                        int L, int M, int N, int ti, int64_t rhs_stride, int nrhs,
                                                        const int* skip, int skip_stride) {
  using C = cplx_t<T>;
  constexpr int W = 4 * RG;
  constexpr int UNR = RG == 1 ? 4 : 2;  // column loads kept in flight per thread
  const int rhs0 = blockIdx.z * RG;
  const int nr = min(RG, nrhs - rhs0);
  if (skip) {
    bool all = true;
    for (int g = 0; g < nr; ++g) all = all && skip[(rhs0 + g) * skip_stride];
    if (all) return;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = 3 * N;
  const int Lb = L / 2 + 1;
  C* v = reinterpret_cast<C*>(smem_raw);  // [il][col = rg*4 + variant][n]
  C* o = v + ti * W * n;
  const int is0 = blockIdx.x * ti, js = blockIdx.y;
  const int64_t LM = (int64_t)L * M;
  const bool jmir = (js != 0) && (2 * js != M);
  for (int u = threadIdx.x; u < ti * W * n; u += blockDim.x) {
    const int s = u % n;
    const int rest = u / n;
    const int col = rest % W, il = rest / W;
    const int var = col & 3, rg = col >> 2;
    const int is = is0 + il;
    const bool imir = (is != 0) && (2 * is != L);
    const bool fx = var & 1, fy = var >> 1;
    C val = czero<C>();
    if (is < Lb && rg < nr && (!fx || imir) && (!fy || jmir)) {
      const int i = fx ? L - is : is, j = fy ? M - js : js;
      val = t[(int64_t)(rhs0 + rg) * rhs_stride + i + (int64_t)L * j + LM * s];
      const int comp = s / N;
      if ((comp == 0 && fx) != (comp == 1 && fy)) { val.x = -val.x; val.y = -val.y; }
    }
    v[u] = val;
  }
  __syncthreads();
  // output row r of column col, with the variant's output flips
  auto put = [&](int il, int r, int col, C a) {
    const int comp = r / N, var = col & 3;
    const bool neg = (comp == 0 && (var & 1)) || (comp == 1 && (var >> 1));
    o[(il * W + col) * n + r] = neg ? make_c<C>(-a.x, -a.y) : a;
  };
  if (PAIR) {
    const int h = n >> 1;
    for (int rr = threadIdx.x; rr < ti * h; rr += blockDim.x) {
      const int il = rr / h, r = 2 * (rr - il * h);
      const int is = is0 + il;
      if (is >= Lb) continue;
      const float4* A = reinterpret_cast<const float4*>(inv + ((int64_t)is + (int64_t)Lb * js) * n * n + r);
      const C* x = v + il * W * n;
      C a[W], b[W];
#pragma unroll
      for (int c = 0; c < W; ++c) { a[c] = czero<C>(); b[c] = czero<C>(); }
#pragma unroll UNR
      for (int q = 0; q < n; ++q) {
        const float4 mm = __ldg(A + (int64_t)q * h);
        const C m0 = make_c<C>(mm.x, mm.y), m1 = make_c<C>(mm.z, mm.w);
#pragma unroll
        for (int c = 0; c < W; ++c) {
          const C xv = x[c * n + q];
          a[c] = cfma(m0, xv, a[c]);
          b[c] = cfma(m1, xv, b[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < W; ++c) {
        put(il, r, c, a[c]);
        put(il, r + 1, c, b[c]);
      }
    }
  } else {
    for (int rr = threadIdx.x; rr < ti * n; rr += blockDim.x) {
      const int il = rr / n, r = rr - il * n;
      const int is = is0 + il;
      if (is >= Lb) continue;
      const C* A = inv + ((int64_t)is + (int64_t)Lb * js) * n * n + r;
      const C* x = v + il * W * n;
      C a[W];
#pragma unroll
      for (int c = 0; c < W; ++c) a[c] = czero<C>();
#pragma unroll UNR
      for (int q = 0; q < n; ++q) {
        const C m = __ldg(A + (int64_t)q * n);
#pragma unroll
        for (int c = 0; c < W; ++c) a[c] = cfma(m, x[c * n + q], a[c]);
      }
#pragma unroll
      for (int c = 0; c < W; ++c) put(il, r, c, a[c]);
    }
  }
  __syncthreads();
  for (int u = threadIdx.x; u < ti * W * n; u += blockDim.x) {
    const int s = u % n;
    const int rest = u / n;
    const int col = rest % W, il = rest / W;
    const int var = col & 3, rg = col >> 2;
    const int is = is0 + il;
    const bool imir = (is != 0) && (2 * is != L);
    const bool fx = var & 1, fy = var >> 1;
    if (is < Lb && rg < nr && (!fx || imir) && (!fy || jmir)) {
      const int i = fx ? L - is : is, j = fy ? M - js : js;
      t[(int64_t)(rhs0 + rg) * rhs_stride + i + (int64_t)L * j + LM * s] = o[u];
    }
  }
}

// ---- streamed quadrant-symmetric apply ------------------------------------
// Bulk asynchronous copies (cp.async.bulk) complete on an mbarrier; every wait
// is bounded and a wait that runs out sets status bit 4 and ends the CTA
// after its outstanding copies land (again with a bounded wait).
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_to_shared(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Bulk copy whose lines are the first candidates for L2 eviction (a one-pass
// stream that should not displace data the next passes re-read).
__device__ __forceinline__ void bulk_to_shared_stream(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar,
                                                      uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar), "l"(policy)
      : "memory");
}

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

constexpr int kGemvPolls = 1 << 20;  // default bound of every streamed-GEMV wait
// Stored blocks per CTA of the streamed GEMV that the forward y pass before it
// prefetches into L2 (gemv_first_bytes).
constexpr int kGemvPrefetchBlocks = 1;
// Each poll may suspend the waiting thread in hardware for up to this many
// nanoseconds (it resumes when the phase completes): waiting warps then stop
// taking issue slots from the warps that compute, and a wait still gives up
// after at most kGemvPolls polls (about a second).
constexpr uint32_t kGemvSuspendNs = 1000;

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int polls = kGemvPolls) {
  for (int i = 0; i < polls; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(kGemvSuspendNs)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Grid position of variant var (bit 0: mirror in x, bit 1: mirror in y) of the
// stored block (is, js); false when that mirror coincides with the block itself.
__device__ __forceinline__ bool mirror_of(int is, int js, int var, int L, int M, int& i, int& j) {
  const bool fx = var & 1, fy = var >> 1;
  if (fx && (is == 0 || 2 * is == L)) return false;
  if (fy && (js == 0 || 2 * js == M)) return false;
  i = fx ? L - is : is;
  j = fy ? M - js : js;
  return true;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Persistent apply over the stored blocks b = blockIdx.x + k*gridDim.x for the
// right-hand sides blockIdx.y*RG .. +RG, with three warp roles:
//  * producer warp (lane 0): streams the blocks (column-major 3N x 3N, in
//    chunks of cq columns) through a ring of nstage shared-memory stages with
//    bulk asynchronous copies, reusing a stage once every consumer warp has
//    arrived on its "empty" barrier;
//  * nv vector warps: gather the W = 4*RG vectors of a block (its four
//    mirrored frequencies per right-hand side, x/y component flips applied)
//    into one of two buffers [q][W] two blocks ahead of the consumers, and
//    after the consumers are done with a block add its G partial sums and
//    write the results (flips applied again) over the grid entries the
//    inputs came from;
//  * consumer warps: thread (g, rp) forms rows RW*rp .. +RW-1 (RW = 2 with
//    PAIR: one 16-byte load per column) over the chunk columns q = g (mod G)
//    and leaves its partial sums as [g][W][row].
// Block boundaries therefore never stop the stream.  Hand-offs use mbarriers:
// vfull[b] (vector warps -> consumers: buffer b holds the block's vectors),
// done[b] (consumers -> vector warps: the block's partial sums written, its
// vectors no longer needed) and rfree (vector warps -> consumers: the partial
// sums consumed).  The partial sums have one buffer: a block's are written
// after all of its chunks, by when the previous block's have long been
// reduced, so a second buffer would only take shared memory from the ring.  Ring positions and phases advance by
// counters (no divisions on the loops).  Every wait is bounded; a wait that
// runs out sets status bit 4 and the abort flag, every role leaves its loop,
// and the producer waits (bounded) for its last copies before the CTA ends.
// A chunk is fetched from the 16-byte boundary at or below its start, so with
// c64 elements and odd 3N the data may begin one element into the stage (the
// block buffers carry 64 bytes of tail padding for the rounded-up last copy);
// PAIR is used only when 3N is even, where every chunk starts aligned.
template <typename T, int RG, bool PAIR, bool PACKED = false>
__global__ void __launch_bounds__(384) k_block_gemv_stream(cplx_t<T>* __restrict__ t, const cplx_t<T>* __restrict__ inv,
                                                           int L, int M, int N, int64_t rhs_stride, int nrhs,
                                                           const int* skip, int skip_stride, int cq, int nstage,
                                                           int stage_elems, int G, int nc, int nv,
                                                           int* __restrict__ status, int polls) {
  using C = cplx_t<T>;
  constexpr int W = 4 * RG, RW = PAIR ? 2 : 1;
  const int rhs0 = blockIdx.y * RG;
  const int nr = min(RG, nrhs - rhs0);
  if (skip) {
    bool all = true;
    for (int g = 0; g < nr; ++g) all = all && skip[(rhs0 + g) * skip_stride];
    if (all) return;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);  // [8]
  uint64_t* empty = full + 8;                               // [8]
  uint64_t* vfull = empty + 8;                              // [2]
  uint64_t* done = vfull + 2;                               // [2]
  uint64_t* rfree = done + 2;                               // [1]
  volatile int* ctl = reinterpret_cast<volatile int*>(rfree + 2);  // [0] abort
  C* stg = reinterpret_cast<C*>(smem_raw + 256);
  const int n = 3 * N, Lb = L / 2 + 1, Mb = M / 2 + 1;
  C* vt0 = stg + (size_t)nstage * stage_elems;  // 2 x [n][W]
  C* red0 = vt0 + (size_t)2 * n * W;            // [G][W][n]
  const int64_t nblk = (int64_t)Lb * Mb, LM = (int64_t)L * M;
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t nmine = blockIdx.x < nblk ? (nblk - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int cpb = (n + cq - 1) / cq;
  const int64_t total = nmine * cpb;
  const int nW = n * W;
  const int ncw = nc / 32;
  if (tid == 0) {
    for (int s = 0; s < nstage; ++s) {
      mbar_init(smem_addr(full + s), 1);
      mbar_init(smem_addr(empty + s), ncw);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_addr(vfull + b), nv);
      mbar_init(smem_addr(done + b), ncw);
    }
    mbar_init(smem_addr(rfree), nv);
    ctl[0] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto fail = [&] {
    atomicOr(status, 4);
    ctl[0] = 1;
  };

  if (tid >= nc + 32) {  // vector warps: vthread vl of nv*32 handles elements vl, vl + nv*32, ...
    // vstride is a multiple of W (a power of two), so a thread keeps one
    // column col = (mirror var, right-hand side rg) and walks the rows q
    const int vl = tid - nc - 32, vstride = nv * 32;
    const int col = vl & (W - 1), var = col & 3, rg = col >> 2;
    const int q0 = vl / W, qstep = vstride / W;
    const bool fx = var & 1, fy = var >> 1;
    auto flip_at = [&](int q) { return q < N ? fx : (q < 2 * N ? fy : false); };
    // grid offset of this thread's mirror of block kb (-1: coincides with the block)
    auto base_of = [&](int64_t kb) -> int64_t {
      const int blk = (int)blockIdx.x + (int)kb * (int)gridDim.x;  // < Lb * Mb
      const int js = blk / Lb, is = blk - js * Lb;
      int i, j;
      return mirror_of(is, js, var, L, M, i, j) ? i + (int64_t)L * j : -1;
    };
    C* const trg = t + (int64_t)(rhs0 + rg) * rhs_stride;
    // load and store block kb in one go
    auto gather = [&](int64_t kb) {
      const int64_t base = base_of(kb);
      const bool on = rg < nr && base >= 0;
      const C* src = trg + (on ? base : 0);
      C* vt = vt0 + (size_t)(kb & 1) * nW + col;
      constexpr int B = 8;  // independent loads in flight per lane
      for (int q = q0; q < n; q += qstep * B) {
        C v[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
          const int qq = q + k * qstep;
          v[k] = (on && qq < n) ? src[LM * qq] : czero<C>();
        }
#pragma unroll
        for (int k = 0; k < B; ++k) {
          const int qq = q + k * qstep;
          if (qq >= n) break;
          C x = v[k];
          // packed blocks hold S = B D: D (negating the x and y components) on the input
          if (flip_at(qq) != (PACKED && qq < 2 * N)) { x.x = -x.x; x.y = -x.y; }
          vt[(size_t)qq * W] = x;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(vfull + (kb & 1)));
    };
    for (int64_t kb = 0; kb < nmine && kb < 2; ++kb) gather(kb);
    for (int64_t kb = 0; kb < nmine; ++kb) {
      const int b = (int)(kb & 1);
      bool ok = true;
      if (lane == 0) ok = !ctl[0] && mbar_wait(smem_addr(done + b), (uint32_t)((kb >> 1) & 1), polls);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) fail();
        break;
      }
      const int64_t base = base_of(kb);
      if (rg < nr && base >= 0) {
        const C* red = red0 + (size_t)col * n;
        C* dst = trg + base;
        for (int q = q0; q < n; q += qstep) {
          C sum = red[q];
          for (int gg = 1; gg < G; ++gg) sum = cadd(sum, red[(size_t)gg * nW + q]);
          if (flip_at(q)) { sum.x = -sum.x; sum.y = -sum.y; }
          dst[LM * q] = sum;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(rfree));
      if (kb + 2 < nmine) gather(kb + 2);
    }
    return;
  }

  if (tid >= nc) {  // producer warp
    if (lane == 0) {
      const uint64_t policy = l2_evict_first_policy();
      int64_t ch = 0, kb = 0;
      int s = 0, round = 0, cc = 0;
      for (; ch < total; ++ch) {
        if (ctl[0]) break;
        if (round > 0 && !mbar_wait(smem_addr(empty + s), (uint32_t)((round - 1) & 1), polls)) {
          fail();
          break;
        }
        const int c0 = cc * cq;
        const int ncols = min(cq, n - c0);
        // packed: one stage holds a whole padded block (stage_elems entries, 16-byte multiple)
        const C* src = PACKED ? inv + (blockIdx.x + kb * gridDim.x) * (int64_t)stage_elems
                              : inv + (blockIdx.x + kb * gridDim.x) * (int64_t)n * n + (int64_t)c0 * n;
        const uintptr_t a = reinterpret_cast<uintptr_t>(src), al = a & ~(uintptr_t)15;
        const uint32_t bytes = PACKED ? (uint32_t)(stage_elems * sizeof(C))
                                      : (uint32_t)(((a - al) + (size_t)ncols * n * sizeof(C) + 15) & ~(size_t)15);
        const uint32_t bar = smem_addr(full + s);
        mbar_expect_tx(bar, bytes);
        bulk_to_shared_stream(smem_addr(stg + (size_t)s * stage_elems), reinterpret_cast<const void*>(al), bytes, bar,
                              policy);
        if (++s == nstage) {
          s = 0;
          ++round;
        }
        if (++cc == cpb) {
          cc = 0;
          ++kb;
        }
      }
      // the copies still in flight land before the CTA may end
      for (int64_t k = ch > nstage ? ch - nstage : 0; k < ch; ++k)
        if (!mbar_wait(smem_addr(full + (k % nstage)), (uint32_t)((k / nstage) & 1))) atomicOr(status, 4);
    }
    return;
  }

  // consumer warps
  const int nrow = n / RW;
  const int nact = G * nrow;
  const int g = tid / nrow, rp = tid - g * nrow;
  int s = 0;
  uint32_t sph = 0;
  for (int64_t kb = 0; kb < nmine; ++kb) {
    const int b = (int)(kb & 1);
    bool ok = !ctl[0] && mbar_wait(smem_addr(vfull + b), (uint32_t)((kb >> 1) & 1), polls);
    const C* vt = vt0 + (size_t)b * nW;
    C acc[RW][W];
#pragma unroll
    for (int h = 0; h < RW; ++h)
#pragma unroll
      for (int c = 0; c < W; ++c) acc[h][c] = czero<C>();
    const C* blk = PACKED ? inv : inv + (blockIdx.x + kb * gridDim.x) * (int64_t)n * n;
    for (int cc = 0; cc < cpb && ok; ++cc) {
      ok = !ctl[0] && mbar_wait(smem_addr(full + s), sph, polls);
      if (!ok) break;
      if (PACKED && tid < nact) {
        // the lower triangle of S: column q (rows q..n-1) from q n - q (q - 1) / 2;
        // row rp over the columns q = g (mod G): q <= rp from column q, q > rp
        // from column rp
        const C* S = stg + (size_t)s * stage_elems;
        auto madd = [&](const C m, int q) {
          const C* xq = vt + (size_t)q * W;
          if constexpr (sizeof(C) == 8) {
#pragma unroll
            for (int c = 0; c < W; c += 2) {
              const float4 xx = *reinterpret_cast<const float4*>(xq + c);
              acc[0][c] = cfma(m, make_c<C>(xx.x, xx.y), acc[0][c]);
              acc[0][c + 1] = cfma(m, make_c<C>(xx.z, xx.w), acc[0][c + 1]);
            }
          } else {
#pragma unroll
            for (int c = 0; c < W; ++c) acc[0][c] = cfma(m, xq[c], acc[0][c]);
          }
        };
        int q = g;
        int o = g * n - g * (g - 1) / 2 + rp - g;
        const int gg2 = G * (G + 1) / 2;
        for (; q <= rp; q += G) {
          madd(S[o], q);
          o += G * (n - q) - gg2;
        }
        const int offp = rp * n - rp * (rp - 1) / 2 - rp;
        for (; q < n; q += G) madd(S[offp + q], q);
      } else if (tid < nact) {
        const int c0 = cc * cq;
        const int ncols = min(cq, n - c0);
        const int shift = (int)((reinterpret_cast<uintptr_t>(blk + (int64_t)c0 * n) & 15) / sizeof(C));
        const C* A = stg + (size_t)s * stage_elems + shift + RW * rp + (size_t)g * n;
        const C* xq = vt + (size_t)(c0 + g) * W;
#pragma unroll 2
        for (int ql = g; ql < ncols; ql += G, A += (size_t)G * n, xq += G * W) {  // column loop
          C m[RW];
          if constexpr (PAIR) {
            const float4 mm = *reinterpret_cast<const float4*>(A);
            m[0] = make_c<C>(mm.x, mm.y);
            m[1] = make_c<C>(mm.z, mm.w);
          } else {
            m[0] = *A;
          }
          if constexpr (sizeof(C) == 8) {
            // two vector entries per 16-byte load (W is a multiple of 4)
#pragma unroll
            for (int c = 0; c < W; c += 2) {
              const float4 xx = *reinterpret_cast<const float4*>(xq + c);
              const C x0 = make_c<C>(xx.x, xx.y), x1 = make_c<C>(xx.z, xx.w);
#pragma unroll
              for (int h = 0; h < RW; ++h) {
                acc[h][c] = cfma(m[h], x0, acc[h][c]);
                acc[h][c + 1] = cfma(m[h], x1, acc[h][c + 1]);
              }
            }
          } else {
#pragma unroll
            for (int c = 0; c < W; ++c) {
              const C xc = xq[c];
#pragma unroll
              for (int h = 0; h < RW; ++h) acc[h][c] = cfma(m[h], xc, acc[h][c]);
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(empty + s));
      if (++s == nstage) {
        s = 0;
        sph ^= 1;
      }
    }
    // the previous block's partial sums have been reduced (phase kb - 1 of rfree)
    if (ok && kb >= 1) ok = !ctl[0] && mbar_wait(smem_addr(rfree), (uint32_t)((kb - 1) & 1), polls);
    if (!ok) {
      if (lane == 0) fail();
      break;
    }
    if (tid < nact) {
      // partial sums as [g][W][row]: the RW rows of a thread are adjacent
      C* red = red0 + (size_t)g * W * n + RW * rp;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        if constexpr (PAIR) {
          *reinterpret_cast<float4*>(red + (size_t)c * n) = make_float4(acc[0][c].x, acc[0][c].y, acc[1][c].x, acc[1][c].y);
        } else {
          red[(size_t)c * n] = acc[0][c];
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_addr(done + b));
  }
}

// ---- packed symmetric blocks ---------------------------------------------
// With exact operator parity and a uniform block scaling, every inverse block
// B satisfies B^T = D B D, D = diag(-1 on the x and y components, +1 on z)
// (the 2-level circulant of a complex-symmetric Toeplitz operator: the block of
// frequency (-i, -j) is both B^T and D B D), so S = B D is complex symmetric
// and B x = S (D x).  Only the lower triangle of S is stored, column by column
// (column q holds rows q..n-1 from offset q n - q (q - 1) / 2), padded to a
// multiple of 16 entries per block: half the bytes of the full blocks.  The
// streamed kernel above applies them with PACKED set (one whole block per
// stage, D folded into the vector gather).

// Lower triangle of S = B D per stored block into the packed layout above.
template <typename T>
__global__ void k_pack_sym(const cplx_t<T>* __restrict__ inv, cplx_t<T>* __restrict__ pk, int n, int N,
                           int64_t nblk, int64_t pstride) {
  const int64_t tri = (int64_t)n * (n + 1) / 2;
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nblk * pstride;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = u / pstride, e = u - b * pstride;
    cplx_t<T> v = czero<cplx_t<T>>();
    if (e < tri) {
      // column q: the largest q with q n - q (q - 1) / 2 <= e
      int q = (int)((2.0 * n + 1 - sqrt((2.0 * n + 1) * (2.0 * n + 1) - 8.0 * (double)e)) / 2);
      while (q > 0 && (int64_t)q * n - (int64_t)q * (q - 1) / 2 > e) --q;
      while ((int64_t)(q + 1) * n - (int64_t)(q + 1) * q / 2 <= e) ++q;
      const int r = q + (int)(e - ((int64_t)q * n - (int64_t)q * (q - 1) / 2));
      v = inv[b * (int64_t)n * n + (int64_t)q * n + r];  // column-major B(r, q)
      if (q < 2 * N) { v.x = -v.x; v.y = -v.y; }           // S = B D
    }
    pk[u] = v;
  }
}

// Stream-kernel launch geometry: chunk columns, stages, stage size, column
// groups, consumer threads, shared memory and CTAs per SM.
struct GemvStream {
  int cq, nstage, stage_elems, G, nc, nv, ctas;
  size_t smem;
};

// Geometry for up to `ctas` CTAs per SM: the CTAs share the SM's 228 KB of
// shared memory (1 KB of each is reserved); when even two stages of one
// column do not fit beside the vectors, fewer CTAs per SM are tried, and
// cq = 0 when not even one CTA fits.
template <typename T>
static GemvStream gemv_stream_geometry(int n, int rg, int chunk_cols, bool pair, int ctas) {
  const size_t cs = sizeof(cplx_t<T>);
  GemvStream g{};
  const int nrow = pair ? n / 2 : n;
  g.G = std::max(1, std::min(4, 256 / nrow));
  g.nc = (g.G * nrow + 31) / 32 * 32;
  g.nv = std::max(1, std::min(4, (384 - g.nc - 32) / 32));
  const size_t vbytes = (size_t)n * 4 * rg * cs;
  const size_t fixed = 256 + (size_t)2 * vbytes + (size_t)g.G * vbytes;
  const size_t stage_target = 16 * 1024;
  auto stage_bytes = [&](int c) { return (((size_t)n * c + 2) * cs + 15) / 16 * 16; };
  for (int c = std::max(1, std::min(ctas, 4)); c >= 1; --c) {
    const size_t budget = c == 1 ? 220 * 1024 : (228 * 1024) / c - 1024;
    int cq = chunk_cols > 0 ? std::min(chunk_cols, n) : std::max(1, (int)(stage_target / ((size_t)n * cs)));
    cq = std::min(cq, n);
    while (cq > 1 && fixed + 2 * stage_bytes(cq) > budget) --cq;
    if (fixed + 2 * stage_bytes(cq) > budget) continue;
    g.cq = cq;
    g.stage_elems = (int)(stage_bytes(cq) / cs);
    g.nstage = 8;
    while (g.nstage > 2 && fixed + (size_t)g.nstage * stage_bytes(cq) > budget) --g.nstage;
    g.smem = fixed + (size_t)g.nstage * stage_bytes(cq);
    g.ctas = c;
    return g;
  }
  g.cq = 0;
  return g;
}

// ---- fused x/y passes of the preconditioner -----------------------------
// One CTA per (z, component) plane and right-hand side does both FFTs of the
// plane in shared memory (the whole L x M plane plus a Stockham scratch copy
// and the two twiddle tables), so the plane crosses global memory once each
// way instead of twice and one launch replaces two.  Forward: gather through
// map3, FFT along x (M rows of length L, rows contiguous), FFT along y (L
// columns of length M, columns interleaved), store the plane to t for the
// block GEMV; inverse: load the plane, inverse FFT along y then x, scatter to
// the unknowns.  Used when 2*L*M elements and the tables fit beside each
// other (c64 planes up to about 14,000 points).
template <typename T>
static size_t prec_plane_smem(int L, int M) {
  return (size_t)(2 * L * M + L + M) * sizeof(cplx_t<T>);
}

template <typename T>
static bool prec_plane_fits(int L, int M) {
  return prec_plane_smem<T>(L, M) <= 220 * 1024;
}

template <typename T, bool INV>
__global__ void __launch_bounds__(kFftThreads) k_prec_plane(const int* __restrict__ map3, const cplx_t<T>* __restrict__ x,
                                                           cplx_t<T>* __restrict__ y, cplx_t<T>* __restrict__ t,
                                                           const cplx_t<T>* __restrict__ twL,
                                                           const cplx_t<T>* __restrict__ twM, FftPlan pL, FftPlan pM,
                                                           int L, int M, int N, int64_t n3, const int* skip,
                                                           int skip_stride) {
  using C = cplx_t<T>;
  const int rhs = blockIdx.y;
  if (skip && skip[rhs * skip_stride]) return;
  C* sm = shmem<C>();
  const int LM = L * M, b1 = LM, tL = 2 * LM, tM = 2 * LM + L;
  load_twiddles(twL, L, tL);
  load_twiddles(twM, M, tM);
  const int plane = blockIdx.x;  // z + N * comp
  const int c = plane / N, z = plane - c * N;
  const int* map = map3 + ((int64_t)c * N + z) * LM;  // c*V + z*L*M
  C* tp = t + ((int64_t)rhs * 3 * N + plane) * LM;
  const FftLayout rows{4, false}, cols{5, true};
  if constexpr (!INV) {
    const C* xr = x + (int64_t)rhs * n3;
    for (int e = threadIdx.x; e < LM; e += kFftThreads) {
      const int pos = __ldg(map + e);
      sm[e] = pos >= 0 ? xr[pos] : czero<C>();
    }
    __syncthreads();
    int r = fft_lines<false, C, false>(0, b1, pL, M, L, 1, rows, tL);
    r = fft_lines<false, C, false>(r, r == 0 ? b1 : 0, pM, L, 1, L, cols, tM);
    for (int e = threadIdx.x; e < LM; e += kFftThreads) tp[e] = sm[r + e];
  } else {
    for (int e = threadIdx.x; e < LM; e += kFftThreads) sm[e] = tp[e];
    __syncthreads();
    int r = fft_lines<true, C, false>(0, b1, pM, L, 1, L, cols, tM);
    r = fft_lines<true, C, false>(r, r == 0 ? b1 : 0, pL, M, L, 1, rows, tL);
    C* yr = y + (int64_t)rhs * n3;
    for (int e = threadIdx.x; e < LM; e += kFftThreads) {
      const int pos = __ldg(map + e);
      if (pos >= 0) yr[pos] = sm[r + e];
    }
  }
}

template <typename T, bool INV>
static void launch_prec_plane(const vs_prec& pr, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, const int* skip,
                              int skip_stride, cudaStream_t st) {
  using C = cplx_t<T>;
  const size_t smem = prec_plane_smem<T>(pr.L, pr.M);
  auto k = k_prec_plane<T, INV>;
  set_kernel_smem((const void*)k, smem);
  k<<<dim3(3 * pr.N, nrhs), kFftThreads, smem, st>>>(pr.map3.as<int>(), x, y, (C*)pr.t.p, pr.axL.tw<T>(),
                                                      pr.axM.tw<T>(), pr.axL.plan, pr.axM.plan, pr.L, pr.M, pr.N,
                                                      pr.n3, skip, skip_stride);
  VS_LAUNCH_CHECK();
}

// Packed symmetric blocks: entries per block (the lower triangle padded to a
// multiple of 16, so every block starts on a 128-byte boundary for c64).
int64_t packed_stride(int n) { return ((int64_t)n * (n + 1) / 2 + 15) / 16 * 16; }

// Streamed-kernel geometry for packed blocks: one whole block per stage,
// nstage stages (2-8), up to `ctas` CTAs per SM; cq = 0 when two stages do not fit.
template <typename T>
static GemvStream gemv_packed_geometry(int n, int rg, int nstage, int ctas) {
  const size_t cs = sizeof(cplx_t<T>);
  GemvStream g{};
  g.G = std::max(1, std::min(4, 256 / n));
  g.nc = (g.G * n + 31) / 32 * 32;
  g.nv = std::max(1, std::min(4, (384 - g.nc - 32) / 32));
  const size_t vbytes = (size_t)n * 4 * rg * cs;
  const size_t fixed = 256 + (size_t)2 * vbytes + (size_t)g.G * vbytes;
  const size_t stage = (size_t)packed_stride(n) * cs;
  for (int c = std::max(1, std::min(ctas, 4)); c >= 1; --c) {
    const size_t budget = c == 1 ? 220 * 1024 : (228 * 1024) / c - 1024;
    int ns = std::min(std::max(nstage, 2), 8);
    while (ns > 2 && fixed + (size_t)ns * stage > budget) --ns;
    if (fixed + (size_t)ns * stage > budget) continue;
    g.cq = n;
    g.stage_elems = (int)packed_stride(n);
    g.nstage = ns;
    g.smem = fixed + (size_t)ns * stage;
    g.ctas = c;
    return g;
  }
  g.cq = 0;
  return g;
}

// Packed copies of the inverse blocks for the streamed kernel, in every
// precision the preconditioner holds whose two-stage ring fits in shared
// memory; only for quadrant-symmetric blocks with a uniform scaling (the
// caller's guarantee that S = B D is symmetric).
void pack_sym_blocks(vs_prec& pr, cudaStream_t st) {
  const int n = 3 * pr.N;
  if (!pr.sym || n > 256) return;
  const int64_t nblk = (int64_t)(pr.L / 2 + 1) * (pr.M / 2 + 1), ps = packed_stride(n);
  pr.pk_stride = ps;
  const int grid = (int)std::min<int64_t>(ceil_div(nblk * ps, 256), 152 * 32);
  if (pr.inv32.p && gemv_packed_geometry<float>(n, 1, 2, 1).cq > 0) {
    pr.pk32.alloc((size_t)nblk * ps * sizeof(float2));
    k_pack_sym<float><<<grid, 256, 0, st>>>(pr.inv32.as<float2>(), pr.pk32.as<float2>(), n, pr.N, nblk, ps);
    VS_LAUNCH_CHECK();
  }
  if (pr.inv64.p && gemv_packed_geometry<double>(n, 1, 2, 1).cq > 0) {
    pr.pk64.alloc((size_t)nblk * ps * sizeof(double2));
    k_pack_sym<double><<<grid, 256, 0, st>>>(pr.inv64.as<double2>(), pr.pk64.as<double2>(), n, pr.N, nblk, ps);
    VS_LAUNCH_CHECK();
  }
}

// Blocks of the full-block streamed GEMV that its CTAs read first (CTA c
// starts on stored block c, and the blocks lie in order), in bytes from the
// start of the block array; 0 when another GEMV form runs.  The forward y
// pass that precedes the GEMV prefetches them into L2 with bulk prefetches,
// which the y pass's idle DRAM cycles absorb: the GEMV's CTAs then start on
// L2 hits instead of all asking HBM for their first chunk at once.
template <typename T>
static uint64_t gemv_first_bytes(const vs_prec& pr, const PassShape& sh, int nrhs) {
  using C = cplx_t<T>;
  const int n = 3 * pr.N;
  const int rg_s = nrhs >= 4 ? 4 : 1;
  const C* pk = std::is_same<T, float>::value ? (const C*)pr.pk32.p : (const C*)pr.pk64.p;
  if (sh.gemv_mode == 2 && pk && pr.gemv_status.p && n <= 256) return 0;  // packed blocks
  const bool pair = std::is_same<T, float>::value && n % 2 == 0;
  const int want = sh.gemv_ti > 0 ? std::min(sh.gemv_ti, 4) : 2;
  const GemvStream g = gemv_stream_geometry<T>(n, rg_s, sh.gemv_chunk, pair, want);
  if (!(pr.sym && sh.gemv_mode != 0 && pr.gemv_status.p && n <= 192 && g.cq > 0)) return 0;
  int dev = 0, nsm = 0;
  VS_CUDA(cudaGetDevice(&dev));
  VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t nblk = (int64_t)(pr.L / 2 + 1) * (pr.M / 2 + 1);
  const int64_t first = std::min<int64_t>(nblk, (int64_t)nsm * std::max(1, g.ctas)) * kGemvPrefetchBlocks;
  return (uint64_t)(std::min(first, nblk) * n * n * (int64_t)sizeof(C)) & ~uint64_t(15);
}

template <typename T>
void prec_apply_pass(const vs_prec& pr, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, const int* skip,
                     cudaStream_t st, int pass, int skip_stride, const XFuse<T>* fz) {
  using C = cplx_t<T>;
  const int L = pr.L, M = pr.M, N = pr.N;
  const C* inv = std::is_same<T, float>::value ? (const C*)pr.inv32.p : (const C*)pr.inv64.p;
  VS_REQUIRE(inv != nullptr, "preconditioner was not built in this precision");
  C* t = (C*)pr.t.p;
  PipeArgs<T> a{};
  a.L = L; a.M = M; a.N = N; a.P = L; a.Q = M; a.R = N;
  a.V = pr.V; a.n3 = pr.n3;
  a.map3 = pr.map3.as<int>();
  a.x = x; a.y = y;
  a.t1 = t; a.t2 = t;
  a.twP = pr.axL.tw<T>();
  a.pP = pr.axL.plan;
  const PassShape& sh = pr.shape[std::is_same<T, float>::value ? 0 : 1];
  if (sh.lg_lpb_x >= 0) {
    a.lg_lpb = sh.lg_lpb_x;
  } else {
    int l = 8;
    while (l > 1 && 2ull * L * l * sizeof(C) > 48 * 1024) l >>= 1;
    int lg = 0;
    while ((1 << lg) < l) ++lg;
    a.lg_lpb = lg;
  }
  a.skip = skip;
  a.skip_stride = skip_stride;
  a.two_level = sh.x_reg == 1 ? 1 : 0;
  if (fz && pass == 0) {  // the forward x pass, whose gather is plain (MODE_PLAIN)
    VS_REQUIRE(a.two_level == 1 && sh.fuse_xy != 1 && x2_ctas(L, M * N * 3) > 0,
               "folded solver step needs the two-level x pass");
    a.fz = *fz;
  }
  StridedArgs<T> s{};
  s.src = t; s.dst = t;
  s.xext = L; s.n_in = M; s.n_out = M;
  if (sh.lg_tx_y >= 0) {
    s.lg_tx = sh.lg_tx_y;
  } else {
    int tx = 16;
    while (tx > 1 && 2ull * M * tx * sizeof(C) > 48 * 1024) tx >>= 1;
    int lg = 0;
    while ((1 << lg) < tx) ++lg;
    s.lg_tx = lg;
  }
  s.na = 3 * N;
  s.s_row = s.d_row = L;
  s.s_a = s.d_a = (int64_t)L * M;
  s.s_b = s.d_b = 0;
  s.s_rhs = s.d_rhs = (int64_t)L * M * N * 3;
  s.plan = pr.axM.plan;
  s.tw = pr.axM.tw<T>();
  s.skip = skip;
  s.skip_stride = skip_stride;
  s.two_level = sh.y_reg == 1 ? 1 : 0;
  // fused x/y planes: pass 0 does both forward FFTs, pass 4 both inverse ones
  const bool fuse = sh.fuse_xy == 1 && prec_plane_fits<T>(L, M);
  if (pass == 1 && !fuse) s.pf_bytes = gemv_first_bytes<T>(pr, sh, nrhs), s.pf = s.pf_bytes ? inv : nullptr;
  switch (pass) {
    case 0:
      if (fuse) launch_prec_plane<T, false>(pr, x, y, nrhs, skip, skip_stride, st);
      else launch_x_pass<T>(a, false, MODE_PLAIN, nrhs, st);
      break;
    case 1:
      if (!fuse) launch_strided_pass<T, false>(s, 3 * N, nrhs, st);
      break;
    case 2: {
      const int n = 3 * N;
      const int rg_s = nrhs >= 4 ? 4 : 1;
      const int polls = sh.wait_polls > 0 ? sh.wait_polls : (sh.wait_polls < 0 ? 0 : kGemvPolls);
      const C* pk = std::is_same<T, float>::value ? (const C*)pr.pk32.p : (const C*)pr.pk64.p;
      if (sh.gemv_mode == 2 && pk && pr.gemv_status.p && n <= 256) {
        // packed symmetric blocks through the streamed kernel; gemv_chunk is the ring depth here
        const GemvStream g = gemv_packed_geometry<T>(n, rg_s, sh.gemv_chunk, sh.gemv_ti > 0 ? sh.gemv_ti : 2);
        if (g.cq > 0) {
          auto k = rg_s == 4 ? k_block_gemv_stream<T, 4, false, true> : k_block_gemv_stream<T, 1, false, true>;
          set_kernel_smem((const void*)k, g.smem);
          int fit = 0, dev = 0, nsm = 0;
          const int nthr = g.nc + 32 + 32 * g.nv;
          VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k, nthr, g.smem));
          VS_CUDA(cudaGetDevice(&dev));
          VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
          const int64_t nblk = (int64_t)(L / 2 + 1) * (M / 2 + 1);
          const dim3 grid((unsigned)std::min<int64_t>(nblk, (int64_t)nsm * std::max(1, std::min(g.ctas, fit))),
                          ceil_div(nrhs, rg_s));
          k<<<grid, nthr, g.smem, st>>>(t, pk, L, M, N, (int64_t)L * M * N * 3, nrhs, skip, skip_stride, g.cq,
                                        g.nstage, g.stage_elems, g.G, g.nc, g.nv, pr.gemv_status.as<int>(), polls);
          VS_LAUNCH_CHECK();
          break;
        }
      }
      const bool pair = std::is_same<T, float>::value && n % 2 == 0;
      const int want = sh.gemv_ti > 0 ? std::min(sh.gemv_ti, 4) : 2;
      const GemvStream g = gemv_stream_geometry<T>(n, rg_s, sh.gemv_chunk, pair, want);
      if (pr.sym && sh.gemv_mode != 0 && pr.gemv_status.p && n <= 192 && g.cq > 0) {
        const int rg = rg_s;
        int dev = 0, nsm = 0;
        VS_CUDA(cudaGetDevice(&dev));
        VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        const int64_t nblk = (int64_t)(L / 2 + 1) * (M / 2 + 1);
        int* status = pr.gemv_status.as<int>();
#define VS_GS(RGV, PR)                                                                                        \
  {                                                                                                           \
    auto k = k_block_gemv_stream<T, RGV, PR>;                                                                 \
    set_kernel_smem((const void*)k, g.smem);                                                                  \
    int fit = 0;                                                                                              \
    VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k, g.nc + 32 + 32 * g.nv, g.smem));          \
    const dim3 grid((unsigned)std::min<int64_t>(nblk, (int64_t)nsm * std::max(1, std::min(g.ctas, fit))),   \
                    ceil_div(nrhs, rg));                                                                      \
    k<<<grid, g.nc + 32 + 32 * g.nv, g.smem, st>>>(t, inv, L, M, N, (int64_t)L * M * N * 3, nrhs, skip,        \
                                                   skip_stride, g.cq, g.nstage, g.stage_elems, g.G, g.nc,     \
                                                   g.nv, status, polls);                                      \
  }
        if constexpr (std::is_same<T, float>::value) {
          if (pair) {
            if (rg == 4) VS_GS(4, true) else VS_GS(1, true)
            VS_LAUNCH_CHECK();
            break;
          }
        }
        if (rg == 4) VS_GS(4, false) else VS_GS(1, false)
#undef VS_GS
        VS_LAUNCH_CHECK();
        break;
      }
      if (pr.sym) {
        const int Lb = L / 2 + 1, Mb = M / 2 + 1;
        const int nthr = sh.gemv_threads > 0 ? sh.gemv_threads : 256;
        int ti = sh.gemv_ti > 0 ? std::min(sh.gemv_ti, Lb) : std::min(Lb, 4);
        const bool pair = std::is_same<T, float>::value && n % 2 == 0;
        // right-hand sides per CTA: 4 when batching, so each block element feeds 16 products
        const int rg = nrhs >= 4 ? 4 : 1;
        while (ti > 1 && 2ull * ti * 4 * rg * n * sizeof(C) > 96 * 1024) --ti;
        const size_t smem = 2ull * ti * 4 * rg * n * sizeof(C);
        const dim3 grid(ceil_div(Lb, ti), Mb, ceil_div(nrhs, rg));
#define VS_GEMV(PR, RGV)                                                                              \
  {                                                                                                   \
    auto k = k_block_gemv_sym<T, PR, RGV>;                                                            \
    set_kernel_smem((const void*)k, smem);                                                            \
    k<<<grid, nthr, smem, st>>>(t, inv, L, M, N, ti, (int64_t)L * M * N * 3, nrhs, skip, skip_stride); \
  }
        if (pair) {
          if (rg == 4) VS_GEMV(true, 4) else VS_GEMV(true, 1)
        } else {
          if (rg == 4) VS_GEMV(false, 4) else VS_GEMV(false, 1)
        }
#undef VS_GEMV
        VS_LAUNCH_CHECK();
        break;
      }
      const int ti = std::min(L, 8);
      const size_t smem = 2ull * ti * n * sizeof(C);
      auto k = k_block_gemv<T>;
      set_kernel_smem((const void*)k, smem);
      k<<<dim3(ceil_div(L, ti), M, nrhs), 256, smem, st>>>(t, inv, L, M, N, ti, (int64_t)L * M * N * 3, skip, 0,
                                                            skip_stride);
      VS_LAUNCH_CHECK();
      break;
    }
    case 3:
      if (!fuse) launch_strided_pass<T, true>(s, 3 * N, nrhs, st);
      break;
    default:
      if (fuse) launch_prec_plane<T, true>(pr, x, y, nrhs, skip, skip_stride, st);
      else launch_x_pass<T>(a, true, MODE_PLAIN, nrhs, st);
      break;
  }
}

template <typename T>
int prec_launches(const vs_prec& pr) {
  const PassShape& sh = pr.shape[std::is_same<T, float>::value ? 0 : 1];
  return sh.fuse_xy == 1 && prec_plane_fits<T>(pr.L, pr.M) ? 3 : 5;
}
template int prec_launches<float>(const vs_prec&);
template int prec_launches<double>(const vs_prec&);

template <typename T>
void prec_apply(const vs_prec& pr, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, const int* skip, cudaStream_t st,
                int skip_stride) {
  for (int pass = 0; pass < 5; ++pass) prec_apply_pass<T>(pr, x, y, nrhs, skip, st, pass, skip_stride);
}
template <typename F>
static float time_ms_prec(cudaStream_t st, int reps, F&& f) {
  cudaEvent_t a, b;
  VS_CUDA(cudaEventCreate(&a));
  VS_CUDA(cudaEventCreate(&b));
  f();
  VS_CUDA(cudaEventRecord(a, st));
  for (int r = 0; r < reps; ++r) f();
  VS_CUDA(cudaEventRecord(b, st));
  VS_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  VS_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

// Autotune the preconditioner apply: lines per CTA of the x passes, x-tile of
// the y passes, and (symmetric storage) blocks per CTA and CTA size of the GEMV.
template <typename T>
void autotune_prec(vs_prec& pr, cudaStream_t st) {
  using C = cplx_t<T>;
  const int pi = std::is_same<T, float>::value ? 0 : 1;
  if ((pi == 0 && !pr.inv32.p) || (pi == 1 && !pr.inv64.p)) return;
  DevBuf xb, yb;
  xb.alloc(pr.n3 * sizeof(C));
  yb.alloc(pr.n3 * sizeof(C));
  fill_tuning_data(xb.p, pr.n3, std::is_same<T, double>::value, st);
  const C* x = xb.as<C>();
  C* y = yb.as<C>();
  const size_t cs = sizeof(C), lim = 227 * 1024;
  PassShape& sh = pr.shape[pi];
  const int reps = 3;
  // two rounds over the candidates, each candidate's best time kept: the
  // clocks may still be ramping up while the first candidates are timed
  auto best_of = [&](int* field, int lo, int hi, auto fits, auto run) {
    float t[8];
    for (int v = lo; v <= hi; ++v) t[v - lo] = 1e30f;
    for (int round = 0; round < 2; ++round)
      for (int v = lo; v <= hi; ++v) {
        if (!fits(v)) continue;
        *field = v;
        t[v - lo] = std::min(t[v - lo], time_ms_prec(st, reps, run));
      }
    int arg = -1;
    float best = 1e30f;
    for (int v = lo; v <= hi; ++v)
      if (fits(v) && t[v - lo] < best) { best = t[v - lo]; arg = v; }
    *field = arg;
  };
  sh.x_reg = 0;
  best_of(&sh.lg_lpb_x, 0, 4, [&](int v) { return (2ull * (1 << v) * pr.L + pr.L) * cs <= lim; },
          [&] {
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 0);
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 4);
          });
  best_of(&sh.x_reg, 0, 1, [&](int) { return true; },
          [&] {
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 0);
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 4);
          });
  sh.y_reg = 0;
  best_of(&sh.lg_tx_y, 1, 5, [&](int v) { return (2ull * pr.M * (1 << v) + pr.M) * cs <= lim; },
          [&] {
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 1);
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 3);
          });
  best_of(&sh.y_reg, 0, 1, [&](int) { return true; },
          [&] {
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 1);
            prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 3);
          });
  // the tuned separate x and y passes against the fused plane kernel
  sh.fuse_xy = 0;
  best_of(&sh.fuse_xy, 0, 1, [&](int v) { return v == 0 || prec_plane_fits<T>(pr.L, pr.M); },
          [&] {
            for (int pass : {0, 1, 3, 4}) prec_apply_pass<T>(pr, x, y, 1, nullptr, st, pass);
          });
  if (pr.sym) {
    // register-direct kernel over blocks per CTA and CTA size, against the
    // streamed kernel over CTAs per SM and chunk width
    float best = 1e30f;
    int bti = 0, bth = 0, bmode = 0, bchunk = 0;
    sh.gemv_mode = 0;
    for (int ti : {1, 2, 4}) {
      for (int th : {64, 128, 256}) {
        sh.gemv_ti = ti;
        sh.gemv_threads = th;
        const float t = time_ms_prec(st, reps, [&] { prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 2); });
        if (t < best) { best = t; bti = ti; bth = th; }
      }
    }
    sh.gemv_threads = 0;
    const int n = 3 * pr.N;
    sh.gemv_mode = 1;
    for (int ctas : {1, 2, 3, 4}) {
      for (int cq : {0, 16, 32, (n + 1) / 2}) {
        if (cq >= n) continue;
        sh.gemv_ti = ctas;
        sh.gemv_chunk = cq;
        const float t = time_ms_prec(st, reps, [&] { prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 2); });
        if (t < best) { best = t; bti = ctas; bth = 0; bmode = 1; bchunk = cq; }
      }
    }
    // the packed symmetric kernel over CTAs per SM and ring depth
    if ((pi == 0 ? pr.pk32.p : pr.pk64.p) != nullptr) {
      sh.gemv_mode = 2;
      for (int ctas : {1, 2, 3, 4}) {
        for (int ns : {2, 3, 4}) {
          const GemvStream pg = gemv_packed_geometry<T>(n, 1, ns, ctas);
          if (pg.cq == 0 || pg.nstage != ns || pg.ctas != ctas) continue;
          sh.gemv_ti = ctas;
          sh.gemv_chunk = ns;
          const float t = time_ms_prec(st, reps, [&] { prec_apply_pass<T>(pr, x, y, 1, nullptr, st, 2); });
          if (t < best) { best = t; bti = ctas; bth = 0; bmode = 2; bchunk = ns; }
        }
      }
    }
    sh.gemv_ti = bti;
    sh.gemv_threads = bth;
    sh.gemv_mode = bmode;
    sh.gemv_chunk = bchunk;
  }
  VS_CUDA(cudaStreamSynchronize(st));
}
template void autotune_prec<float>(vs_prec&, cudaStream_t);
template void autotune_prec<double>(vs_prec&, cudaStream_t);

template void prec_apply_pass<float>(const vs_prec&, const float2*, float2*, int, const int*, cudaStream_t, int, int,
                                     const XFuse<float>*);
template void prec_apply_pass<double>(const vs_prec&, const double2*, double2*, int, const int*, cudaStream_t, int,
                                      int, const XFuse<double>*);
template void prec_apply<float>(const vs_prec&, const float2*, float2*, int, const int*, cudaStream_t, int);
template void prec_apply<double>(const vs_prec&, const double2*, double2*, int, const int*, cudaStream_t, int);

}  // namespace vs
