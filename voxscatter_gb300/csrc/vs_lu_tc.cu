// Batched inversion of the 2-level circulant preconditioner's 3N x 3N blocks
// (the parfor of inv(...) at main_DDA.m:107-111, main_koch.m:114-118) with the
// trailing updates on the tensor cores.
//
// Blocked Gauss-Jordan with partial pivoting on nmat row-major n x n FP32
// complex matrices held in global memory, n <= 256, all matrices advancing
// one 32-column panel at a time:
//   1. k_tc_panel (one CTA per matrix, CUDA cores): the panel's n x nb columns
//      are reduced in shared memory by nb unblocked steps (pivot search among
//      the rows not yet used, row swap, pivot row scaled, column eliminated
//      from every other row), which leaves Panel = [A_KK^-1 ; -A_OK A_KK^-1]
//      for the pivot rows K and the other rows O.  The panel's row swaps are
//      applied to the columns outside it, and the rows K of those columns
//      (after the swaps) are copied to a scratch array V.
//   2. k_tc_update (tcgen05): every column c outside the panel becomes
//      c_new = (c with rows K zeroed) + Panel * c_K, a rank-nb complex update
//      D = Panel (n x nb) * V (nb x n).  Complex products run as real MMAs
//      with 2 x 2 blocks: output row 2r+e (e = 0 real, 1 imaginary part of
//      row r) and reduction index 2k+f give A~[2r, 2k..2k+1] = (Re, -Im),
//      A~[2r+1, 2k..2k+1] = (Im, Re) of Panel[r, k] and B~[q, 2k..2k+1] =
//      (Re, Im) of V[k, q], so one M = 128 MMA covers 64 complex rows with
//      real and imaginary parts interleaved in TMEM lanes.  Each FP32 operand
//      x is split into x_hi = tf32(x) and x_lo = x - x_hi and the product is
//      formed as A_hi B_hi + A_hi B_lo + A_lo B_hi (3xTF32), accumulated in
//      FP32 in TMEM, which keeps FP32 accuracy on the TF32 tensor pipe.
//   3. k_tc_finish: the column interchanges of all panels are undone in one
//      composed permutation, the result is scaled, non-finite entries flagged.
// Status bits: 1 zero pivot, 2 non-finite result, 8 an MMA completion wait ran
// out (the kernel then waits again, bounded, frees its TMEM and returns).
#include "vs_internal.h"
#include "vs_tc.cuh"

namespace vs {

namespace {

constexpr int kNB = 32;             // panel width (complex columns)
constexpr int kK = 2 * kNB;         // real reduction length of one panel
constexpr int kRowsPerTile = 64;    // complex rows per MMA tile (M = 128 real rows)
constexpr int kPanelThreads = 256;
constexpr int kUpdThreads = 128;
constexpr int kTQ = 64;             // column tile of the permutation in k_tc_panel
constexpr uint32_t kMmaPolls = 1u << 22;

__device__ __forceinline__ float2 crecipf(float2 a) {
  const float d = a.x * a.x + a.y * a.y;
  return make_float2(a.x / d, -a.y / d);
}

// Shared memory of k_tc_panel for blocks of n.
size_t panel_smem(int n) {
  return ((size_t)n * (kNB + 1) + (size_t)n + 2ull * kNB * kTQ) * sizeof(float2) + (3ull * n + kNB) * sizeof(int) +
         64;
}

__global__ void __launch_bounds__(kPanelThreads) k_tc_panel(float2* __restrict__ mats, int n, int64_t nmat, int k0,
                                                            float2* __restrict__ V, int* __restrict__ perm_all,
                                                            int* __restrict__ status) {
  constexpr int PS = kNB + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* P = reinterpret_cast<float2*>(smem_raw);  // [n][PS]
  float2* colk = P + (size_t)n * PS;                // [n]
  float2* buf = colk + n;                           // [2*NB][TQ]: old K rows, then old rows feeding O rows
  int* rowsrc = reinterpret_cast<int*>(buf + 2 * kNB * kTQ);  // new row r = old row rowsrc[r]
  int* oidx = rowsrc + n;                                     // slot of a changed row below the panel, or -1
  int* olist = oidx + n;                                      // [NB]
  int* piv = olist + kNB;                                     // [n] pivots of this panel (local copy)
  __shared__ int s_piv, s_ocnt;
  __shared__ float s_pmag;
  const int tid = threadIdx.x;
  const int nb = min(kNB, n - k0);
  for (int64_t b = blockIdx.x; b < nmat; b += gridDim.x) {
    float2* B = mats + b * (int64_t)n * n;
    int* perm = perm_all + b * (int64_t)n;
    for (int r = tid; r < n; r += blockDim.x) {
      rowsrc[r] = r;
      oidx[r] = -1;
    }
    for (int u = tid; u < n * kNB; u += blockDim.x) {
      const int r = u / kNB, c = u - r * kNB;
      P[r * PS + c] = c < nb ? B[(int64_t)r * n + k0 + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int kk = 0; kk < nb; ++kk) {
      const int k = k0 + kk;
      if (tid < 32) {
        float best = -1.f;
        int bi = k;
        for (int r = k + tid; r < n; r += 32) {
          const float2 a = P[r * PS + kk];
          const float m = a.x * a.x + a.y * a.y;
          if (m > best) { best = m; bi = r; }
        }
        for (int off = 16; off; off >>= 1) {
          const float ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (tid == 0) {
          s_piv = bi;
          s_pmag = best;
          piv[kk] = bi;
          const int t = rowsrc[k];
          rowsrc[k] = rowsrc[bi];
          rowsrc[bi] = t;
        }
      }
      __syncthreads();
      const int p = s_piv;
      if (tid == 0 && !(s_pmag > 0.f)) atomicOr(status, 1);
      if (p != k && tid < kNB) {
        const float2 t = P[k * PS + tid];
        P[k * PS + tid] = P[p * PS + tid];
        P[p * PS + tid] = t;
      }
      __syncthreads();
      for (int r = tid; r < n; r += blockDim.x) colk[r] = P[r * PS + kk];
      __syncthreads();
      const float2 rinv = crecipf(colk[k]);
      if (tid < kNB) P[k * PS + tid] = (tid == kk) ? rinv : cmul(P[k * PS + tid], rinv);
      __syncthreads();
      for (int u = tid; u < n * kNB; u += blockDim.x) {
        const int r = u / kNB, c = u - r * kNB;
        if (r == k) continue;
        const float2 base = (c == kk) ? make_float2(0.f, 0.f) : P[r * PS + c];
        P[r * PS + c] = csub(base, cmul(colk[r], P[k * PS + c]));
      }
      __syncthreads();
    }
    // the panel's final columns, and the bookkeeping of the rows below it
    // that a swap changed (each receives an old row of K)
    for (int u = tid; u < n * kNB; u += blockDim.x) {
      const int r = u / kNB, c = u - r * kNB;
      if (c < nb) B[(int64_t)r * n + k0 + c] = P[r * PS + c];
    }
    if (tid < nb) perm[k0 + tid] = piv[tid];
    if (tid == 0) {
      int cnt = 0;
      for (int kk = 0; kk < nb; ++kk) {
        const int p = piv[kk];
        if (p >= k0 + nb && oidx[p] < 0) {
          oidx[p] = cnt;
          olist[cnt++] = p;
        }
      }
      s_ocnt = cnt;
    }
    __syncthreads();
    // columns outside the panel: V <- old rows feeding K, changed rows below
    // the panel <- their old K row; zeros in V for the panel's own columns
    const int ocnt = s_ocnt;
    float2* Vb = V + b * (int64_t)kNB * n;
    for (int q0 = 0; q0 < n; q0 += kTQ) {
      for (int u = tid; u < (nb + ocnt) * kTQ; u += blockDim.x) {
        const int rr = u / kTQ, qi = u - rr * kTQ, q = q0 + qi;
        if (q >= n || (q >= k0 && q < k0 + nb)) continue;
        const int src = rr < nb ? rowsrc[k0 + rr] : rowsrc[olist[rr - nb]];
        buf[rr * kTQ + qi] = B[(int64_t)src * n + q];
      }
      __syncthreads();
      for (int u = tid; u < (kNB + ocnt) * kTQ; u += blockDim.x) {
        const int rr = u / kTQ, qi = u - rr * kTQ, q = q0 + qi;
        if (q >= n) continue;
        const bool inpanel = q >= k0 && q < k0 + nb;
        if (rr < kNB) {
          Vb[(int64_t)rr * n + q] = (rr < nb && !inpanel) ? buf[rr * kTQ + qi] : make_float2(0.f, 0.f);
        } else if (!inpanel) {
          B[(int64_t)olist[rr - kNB] * n + q] = buf[(nb + rr - kNB) * kTQ + qi];
        }
      }
      __syncthreads();
    }
  }
}

// Shared memory of k_tc_update: A_hi, A_lo (128 x K) and B_hi, B_lo (NT x K), FP32.
size_t update_smem(int NT) { return (2ull * 128 * kK + 2ull * NT * kK) * sizeof(float) + 1024; }

// One CTA per (matrix, 64-row tile); NT = MMA N (columns 0..NT-1 of the
// matrix, NT a multiple of 16 covering n).
__global__ void __launch_bounds__(kUpdThreads) k_tc_update(float2* __restrict__ mats, int n, int64_t nmat, int k0,
                                                           const float2* __restrict__ V, int NT, int tiles,
                                                           int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // 1024-byte alignment of the operand arrays (the descriptors need 16)
  unsigned char* base = smem_raw + ((1024u - (tc::smem_addr(smem_raw) & 1023u)) & 1023u);
  unsigned char* sAh = base;
  unsigned char* sAl = sAh + 128 * kK * 4;
  unsigned char* sBh = sAl + 128 * kK * 4;
  unsigned char* sBl = sBh + (size_t)NT * kK * 4;
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t b = blockIdx.x / tiles;
  const int tile = (int)(blockIdx.x - b * tiles);
  if (b >= nmat) return;
  float2* B = mats + b * (int64_t)n * n;
  const float2* Vb = V + b * (int64_t)kNB * n;
  const int r0 = tile * kRowsPerTile;
  const int nb = min(kNB, n - k0);
  // A~ (2x2 real blocks of the panel rows r0..r0+63): thread -> (row, k) with k fastest
  for (int u = tid; u < kRowsPerTile * kNB; u += kUpdThreads) {
    const int rl = u / kNB, kk = u - rl * kNB, r = r0 + rl;
    float2 w = make_float2(0.f, 0.f);
    if (r < n && kk < nb) w = B[(int64_t)r * n + k0 + kk];
    const float v[4] = {w.x, -w.y, w.y, w.x};  // (row 2rl: Re, -Im), (row 2rl+1: Im, Re)
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const float x = v[2 * e + f];
        const float hi = tc::to_tf32(x);
        const uint32_t off = tc::kmajor_offset(2 * rl + e, 2 * kk + f, kK);
        *reinterpret_cast<float*>(sAh + off) = hi;
        *reinterpret_cast<float*>(sAl + off) = x - hi;
      }
  }
  // B~ (columns q of V): thread -> (k, q) with q fastest
  for (int u = tid; u < kNB * NT; u += kUpdThreads) {
    const int kk = u / NT, q = u - kk * NT;
    const float2 w = (q < n && kk < nb) ? Vb[(int64_t)kk * n + q] : make_float2(0.f, 0.f);
    const float hx = tc::to_tf32(w.x), hy = tc::to_tf32(w.y);
    const uint32_t off = tc::kmajor_offset(q, 2 * kk, kK);  // (q, 2kk) and (q, 2kk+1) are adjacent
    *reinterpret_cast<float2*>(sBh + off) = make_float2(hx, hy);
    *reinterpret_cast<float2*>(sBl + off) = make_float2(w.x - hx, w.y - hy);
  }
  const uint32_t ncols = NT <= 32 ? 32u : NT <= 64 ? 64u : NT <= 128 ? 128u : 256u;
  if (warp == 0) tc::tmem_alloc(&s_tmem, ncols);
  if (tid == 0) tc::mbar_init(&s_bar, 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_tf32(128, NT);
    const uint32_t sbo = (kK / 4) * 128;
    const uint32_t ah = tc::smem_addr(sAh), al = tc::smem_addr(sAl), bh = tc::smem_addr(sBh),
                   bl = tc::smem_addr(sBl);
    const int steps = (2 * nb + 7) / 8;
    for (int s = 0; s < steps; ++s) {
      const uint32_t o = s * 256;
      tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, sbo), tc::smem_desc(bh + o, 128, sbo), idesc, s > 0 ? 1u : 0u);
      tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, sbo), tc::smem_desc(bl + o, 128, sbo), idesc, 1u);
      tc::mma_tf32(tmem, tc::smem_desc(al + o, 128, sbo), tc::smem_desc(bh + o, 128, sbo), idesc, 1u);
    }
    tc::mma_commit(&s_bar);
  }
  bool ok = tc::mbar_wait(&s_bar, 0, kMmaPolls);
  if (!ok) {
    if (lane == 0) atomicOr(status, 8);
    tc::mbar_wait(&s_bar, 0, kMmaPolls);  // let the MMAs in flight finish before TMEM is freed
  }
  tc::fence_after_sync();
  if (ok) {
    // warp w holds TMEM lanes 32w..32w+31: complex row r0 + 16w + lane/2,
    // real part in even lanes, imaginary part in odd lanes
    const int rl = 16 * warp + (lane >> 1), r = r0 + rl;
    const bool odd = lane & 1;
    const bool inK = r >= k0 && r < k0 + nb;
    for (int c = 0; c < NT; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + c, v);
      float2 d[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float send = odd ? v[i] : v[8 + i];
        const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
        d[i] = odd ? make_float2(recv, v[8 + i]) : make_float2(v[i], recv);
      }
      if (r < n) {
        const int q0 = c + (odd ? 8 : 0);
        float2* row = B + (int64_t)r * n;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = q0 + i;
          if (q >= n || (q >= k0 && q < k0 + nb)) continue;
          const float2 base0 = inK ? make_float2(0.f, 0.f) : row[q];
          row[q] = make_float2(base0.x + d[i].x, base0.y + d[i].y);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, ncols);
  }
}

// Undo the column interchanges (composed over all panels), scale, flag
// non-finite entries.  One CTA per matrix.
__global__ void __launch_bounds__(256) k_tc_finish(float2* __restrict__ mats, int n, int64_t nmat,
                                                   const int* __restrict__ perm_all, float scale,
                                                   int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* cmap = reinterpret_cast<int*>(smem_raw);
  float2* row = reinterpret_cast<float2*>(smem_raw + ((n * sizeof(int) + 15) & ~size_t(15)));
  for (int64_t b = blockIdx.x; b < nmat; b += gridDim.x) {
    float2* B = mats + b * (int64_t)n * n;
    const int* perm = perm_all + b * (int64_t)n;
    if (threadIdx.x == 0) {
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
    for (int r = 0; r < n; ++r) {
      float2* Br = B + (int64_t)r * n;
      for (int c = threadIdx.x; c < n; c += blockDim.x) row[c] = Br[c];
      __syncthreads();
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const float2 a = row[cmap[c]];
        const float2 o = make_float2(a.x * scale, a.y * scale);
        if (!(isfinite(o.x) && isfinite(o.y))) atomicOr(status, 2);
        Br[c] = o;
      }
      __syncthreads();
    }
  }
}

}  // namespace

bool tc_invert_supported(int n) { return n >= 2 && n <= 256; }

void invert_blocks_tc(float2* mats, int n, int64_t nmat, double scale, int* status, cudaStream_t st) {
  VS_REQUIRE(tc_invert_supported(n), "tensor-core inversion takes blocks of 2..256");
  if (nmat <= 0) return;
  const int NT = (n + 15) / 16 * 16;
  const int tiles = (n + kRowsPerTile - 1) / kRowsPerTile;
  int dev = 0, nsm = 0;
  VS_CUDA(cudaGetDevice(&dev));
  VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t psm = panel_smem(n), usm = update_smem(NT), fsm = n * sizeof(int) + 16 + n * sizeof(float2);
  set_kernel_smem((const void*)k_tc_panel, psm);
  set_kernel_smem((const void*)k_tc_update, usm);
  set_kernel_smem((const void*)k_tc_finish, fsm);
  int per_sm = 0;
  VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tc_panel, kPanelThreads, psm));
  // scratch V (32 rows of every matrix) bounded to ~512 MB: matrices in chunks
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nmat, (int64_t(512) << 20) / (kNB * n * 8)));
  DevBuf V, perm;
  V.alloc((size_t)chunk * kNB * n * sizeof(float2));
  perm.alloc((size_t)chunk * n * sizeof(int));
  for (int64_t m0 = 0; m0 < nmat; m0 += chunk) {
    const int64_t cm = std::min(chunk, nmat - m0);
    float2* mc = mats + m0 * (int64_t)n * n;
    const int pgrid = (int)std::min<int64_t>(cm, (int64_t)nsm * std::max(per_sm, 1));
    for (int k0 = 0; k0 < n; k0 += kNB) {
      k_tc_panel<<<pgrid, kPanelThreads, psm, st>>>(mc, n, cm, k0, V.as<float2>(), perm.as<int>(), status);
      VS_LAUNCH_CHECK();
      const int64_t ublocks = cm * tiles;
      VS_REQUIRE(ublocks < (int64_t(1) << 31), "too many blocks for one launch");
      k_tc_update<<<(unsigned)ublocks, kUpdThreads, usm, st>>>(mc, n, cm, k0, V.as<float2>(), NT, tiles, status);
      VS_LAUNCH_CHECK();
    }
    k_tc_finish<<<(int)std::min<int64_t>(cm, (int64_t)nsm * 8), 256, fsm, st>>>(mc, n, cm, perm.as<int>(),
                                                                                (float)scale, status);
    VS_LAUNCH_CHECK();
  }
  // V and perm are released when this returns: keep them until the work is done
  VS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace vs
