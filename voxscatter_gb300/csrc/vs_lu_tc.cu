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
constexpr int kUpdThreads = 256;
constexpr int kTQ = 64;             // column tile of the permutation in k_tc_panel
constexpr uint32_t kMmaPolls = 1u << 22;
constexpr int kMaxChunks = 4;       // 16-column chunks per warp of the update epilogue (NT <= 128)

__device__ __forceinline__ float2 crecipf(float2 a) {
  const float d = a.x * a.x + a.y * a.y;
  return make_float2(a.x / d, -a.y / d);
}

// Shared memory of k_tc_panel for blocks of n.
size_t panel_smem(int n) {
  return (2ull * kNB * kTQ + 3ull * kNB) * sizeof(float2) + (3ull * n + kNB + 2 * 8) * sizeof(int) + 64;
}

// The panel lives in registers: lane c holds column c of the panel for the
// warp's rows (8 warps, row r in warp r % 8 at slot r / 8, RPW >= n / 8 slots),
// so a row's column kk (the elimination multiplier) is one shuffle away and
// only the pivot search, the row swap and the scaled pivot row cross warps
// (three barriers per step).
template <int kPanelRows>
__global__ void __launch_bounds__(kPanelThreads) k_tc_panel(float2* __restrict__ mats, int n, int64_t nmat, int k0,
                                                            float2* __restrict__ V, int* __restrict__ perm_all,
                                                            int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);  // [2*NB][TQ]: old K rows, then old rows feeding O rows
  float2* prow = buf + 2 * kNB * kTQ;                  // [NB] scaled pivot row
  float2* swk = prow + kNB;                            // [NB] row k before the swap
  float2* swp = swk + kNB;                             // [NB] row p before the swap
  int* rowsrc = reinterpret_cast<int*>(swp + kNB);     // new row r = old row rowsrc[r]
  int* oidx = rowsrc + n;                              // slot of a changed row below the panel, or -1
  int* olist = oidx + n;                               // [NB]
  int* piv = olist + kNB;                              // [n]
  float* cand_m = reinterpret_cast<float*>(piv + n);   // [8] best magnitude per warp
  int* cand_i = reinterpret_cast<int*>(cand_m + 8);    // [8] its row
  __shared__ int s_ocnt;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nb = min(kNB, n - k0);
  const float2 z2 = make_float2(0.f, 0.f);
  for (int64_t b = blockIdx.x; b < nmat; b += gridDim.x) {
    float2* B = mats + b * (int64_t)n * n;
    int* perm = perm_all + b * (int64_t)n;
    for (int r = tid; r < n; r += blockDim.x) {
      rowsrc[r] = r;
      oidx[r] = -1;
    }
    float2 P[kPanelRows];
#pragma unroll
    for (int i = 0; i < kPanelRows; ++i) {
      const int r = warp + 8 * i;
      P[i] = (r < n && lane < nb) ? B[(int64_t)r * n + k0 + lane] : z2;
    }
    __syncthreads();
    for (int kk = 0; kk < nb; ++kk) {
      const int k = k0 + kk;
      // pivot search in column kk over rows >= k: per warp in lane kk, then
      // every thread reduces the eight candidates (same order, same result)
      float best = -1.f;
      int bi = k;
#pragma unroll
      for (int i = 0; i < kPanelRows; ++i) {
        const int r = warp + 8 * i;
        const float m = P[i].x * P[i].x + P[i].y * P[i].y;
        if (r >= k && r < n && m > best) { best = m; bi = r; }
      }
      if (lane == kk) {
        cand_m[warp] = best;
        cand_i[warp] = bi;
      }
      __syncthreads();
      float pm = cand_m[0];
      int p = cand_i[0];
      for (int w = 1; w < 8; ++w) {
        const float m = cand_m[w];
        const int ri = cand_i[w];
        if (m > pm || (m == pm && ri < p)) { pm = m; p = ri; }
      }
      if (p < k) p = k;  // no candidate (all below k): keep k, flagged as a zero pivot
      if (tid == 0) {
        if (!(pm > 0.f)) atomicOr(status, 1);
        piv[kk] = p;
        const int t = rowsrc[k];
        rowsrc[k] = rowsrc[p];
        rowsrc[p] = t;
      }
      // swap rows k and p through shared memory (selects over every slot,
      // so the slots stay in registers)
      const int ks = k >> 3, ps = p >> 3;
      if (p != k) {
        float2 tk = z2, tp = z2;
#pragma unroll
        for (int i = 0; i < kPanelRows; ++i) {
          tk = (i == ks) ? P[i] : tk;
          tp = (i == ps) ? P[i] : tp;
        }
        if (warp == (k & 7)) swk[lane] = tk;
        if (warp == (p & 7)) swp[lane] = tp;
      }
      __syncthreads();
      if (p != k) {
        const float2 nk = swp[lane], np = swk[lane];
        const bool wk = warp == (k & 7), wp = warp == (p & 7);
#pragma unroll
        for (int i = 0; i < kPanelRows; ++i) {
          P[i] = (wk && i == ks) ? nk : P[i];
          P[i] = (wp && i == ps) ? np : P[i];
        }
      }
      // scaled pivot row (row k's warp), broadcast through shared memory
      {
        float2 pk = z2;
#pragma unroll
        for (int i = 0; i < kPanelRows; ++i) pk = (i == ks) ? P[i] : pk;
        const float2 pv = make_float2(__shfl_sync(0xffffffffu, pk.x, kk), __shfl_sync(0xffffffffu, pk.y, kk));
        const float2 rinv = crecipf(pv);
        const float2 nv = (lane == kk) ? rinv : cmul(pk, rinv);
        if (warp == (k & 7)) prow[lane] = nv;
      }
      __syncthreads();
      const float2 pr = prow[lane];
#pragma unroll
      for (int i = 0; i < kPanelRows; ++i) {
        const int r = warp + 8 * i;
        const float2 ck = make_float2(__shfl_sync(0xffffffffu, P[i].x, kk), __shfl_sync(0xffffffffu, P[i].y, kk));
        const float2 base0 = (lane == kk) ? z2 : P[i];
        const float2 el = csub(base0, cmul(ck, pr));
        P[i] = (r == k) ? pr : (r < n ? el : P[i]);
      }
      // the next step's first barrier orders these register updates against
      // the shared buffers it rewrites
    }
    // the panel's final columns
#pragma unroll
    for (int i = 0; i < kPanelRows; ++i) {
      const int r = warp + 8 * i;
      if (r < n && lane < nb) B[(int64_t)r * n + k0 + lane] = P[i];
    }
    __syncthreads();
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
          Vb[(int64_t)rr * n + q] = (rr < nb && !inpanel) ? buf[rr * kTQ + qi] : z2;
        } else if (!inpanel) {
          B[(int64_t)olist[rr - kNB] * n + q] = buf[(nb + rr - kNB) * kTQ + qi];
        }
      }
      __syncthreads();
    }
  }
}

// Shared memory of k_tc_update: A_hi, A_lo (128 x K) and B_hi, B_lo (NT x K),
// FP32, plus alignment slack.
size_t update_smem(int NT) { return (2ull * 128 * kK + 2ull * NT * kK) * sizeof(float) + 128; }

// Column tiles of the update: at most 128 columns each (two CTAs per SM fit),
// NT a multiple of 16.
void update_tiling(int n, int* q_tiles, int* NT) {
  *q_tiles = (n + 127) / 128;
  const int w = (n + *q_tiles - 1) / *q_tiles;
  *NT = (w + 15) / 16 * 16;
}

// One CTA per (matrix, 64-row tile, NT-column tile).  Operands are staged
// with 16-byte stores, one row of a core matrix per thread and the rows of a
// core on consecutive threads, so each quarter-warp fills one 128-byte core
// without bank conflicts.
__global__ void __launch_bounds__(kUpdThreads) k_tc_update(float2* __restrict__ mats, int n, int64_t nmat, int k0,
                                                           const float2* __restrict__ V, int NT, int q_tiles,
                                                           int r_tiles, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((128u - (tc::smem_addr(smem_raw) & 127u)) & 127u);
  unsigned char* sAh = base;
  unsigned char* sAl = sAh + 128 * kK * 4;
  unsigned char* sBh = sAl + 128 * kK * 4;
  unsigned char* sBl = sBh + (size_t)NT * kK * 4;
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int per_mat = r_tiles * q_tiles;
  const int64_t b = blockIdx.x / per_mat;
  const int rem = (int)(blockIdx.x - b * per_mat);
  const int r0 = (rem / q_tiles) * kRowsPerTile, c0 = (rem % q_tiles) * NT;
  if (b >= nmat) return;
  float2* B = mats + b * (int64_t)n * n;
  const float2* Vb = V + b * (int64_t)kNB * n;
  const int nb = min(kNB, n - k0);
  const float2 z2 = make_float2(0.f, 0.f);
  // A~: real row R = 2 rl + e of panel row r0 + rl, K chunk c (panel columns
  // 2c, 2c+1): (Re, -Im) pairs for e = 0, (Im, Re) pairs for e = 1
  for (int u = tid; u < 128 * (kK / 4); u += kUpdThreads) {
    const int R = u & 127, c = u >> 7, rl = R >> 1, r = r0 + rl;
    float2 w0 = z2, w1 = z2;
    if (r < n) {
      const float2* rowp = B + (int64_t)r * n + k0;
      if (2 * c < nb) w0 = rowp[2 * c];
      if (2 * c + 1 < nb) w1 = rowp[2 * c + 1];
    }
    const float4 v = (R & 1) ? make_float4(w0.y, w0.x, w1.y, w1.x) : make_float4(w0.x, -w0.y, w1.x, -w1.y);
    const float4 h = make_float4(tc::to_tf32(v.x), tc::to_tf32(v.y), tc::to_tf32(v.z), tc::to_tf32(v.w));
    const uint32_t off = tc::kmajor_offset(R, 4 * c, kK);
    *reinterpret_cast<float4*>(sAh + off) = h;
    *reinterpret_cast<float4*>(sAl + off) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
  }
  // B~: row q of the column tile, K chunk c: (Re, Im) of V[2c, q], V[2c+1, q]
  for (int u = tid; u < NT * (kK / 4); u += kUpdThreads) {
    const int ql = u % NT, c = u / NT, q = c0 + ql;
    float2 w0 = z2, w1 = z2;
    if (q < n) {
      if (2 * c < nb) w0 = Vb[(int64_t)(2 * c) * n + q];
      if (2 * c + 1 < nb) w1 = Vb[(int64_t)(2 * c + 1) * n + q];
    }
    const float4 v = make_float4(w0.x, w0.y, w1.x, w1.y);
    const float4 h = make_float4(tc::to_tf32(v.x), tc::to_tf32(v.y), tc::to_tf32(v.z), tc::to_tf32(v.w));
    const uint32_t off = tc::kmajor_offset(ql, 4 * c, kK);
    *reinterpret_cast<float4*>(sBh + off) = h;
    *reinterpret_cast<float4*>(sBl + off) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
  }
  // epilogue mapping: warp w takes TMEM lanes 32 (w % 4).. (complex row
  // r0 + 16 (w % 4) + lane/2, real part in even lanes, imaginary part in odd
  // lanes) and, with warp w + 4, alternate 16-column chunks
  const int qd = warp & 3, half = warp >> 2;
  const int r_e = r0 + 16 * qd + (lane >> 1);
  const bool odd = lane & 1;
  const bool inK = r_e >= k0 && r_e < k0 + nb;
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
#pragma unroll
    for (int j = 0; j < kMaxChunks; ++j) {
      const int c = 16 * half + 32 * j;
      if (c >= NT) break;
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * qd) << 16) + c, v);
      float2 d[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float send = odd ? v[i] : v[8 + i];
        const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
        d[i] = odd ? make_float2(recv, v[8 + i]) : make_float2(v[i], recv);
      }
      if (r_e < n) {
        const int qb = c0 + c + (odd ? 8 : 0);
        float2* row = B + (int64_t)r_e * n;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = qb + i;
          if (q >= n || (q >= k0 && q < k0 + nb)) continue;
          const float2 base0 = inK ? z2 : row[q];
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
// non-finite entries.  One CTA per matrix; each warp permutes whole rows
// through its own shared-memory row buffer.
__global__ void __launch_bounds__(256) k_tc_finish(float2* __restrict__ mats, int n, int64_t nmat,
                                                   const int* __restrict__ perm_all, float scale,
                                                   int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* cmap = reinterpret_cast<int*>(smem_raw);
  float2* rows = reinterpret_cast<float2*>(smem_raw + ((n * sizeof(int) + 15) & ~size_t(15)));  // [8][n]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* row = rows + (size_t)warp * n;
  for (int64_t b = blockIdx.x; b < nmat; b += gridDim.x) {
    float2* B = mats + b * (int64_t)n * n;
    const int* perm = perm_all + b * (int64_t)n;
    __syncthreads();  // the previous matrix's cmap is no longer read
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
    for (int r = warp; r < n; r += 8) {
      float2* Br = B + (int64_t)r * n;
      for (int c = lane; c < n; c += 32) row[c] = Br[c];
      __syncwarp();
      for (int c = lane; c < n; c += 32) {
        const float2 a = row[cmap[c]];
        const float2 o = make_float2(a.x * scale, a.y * scale);
        if (!(isfinite(o.x) && isfinite(o.y))) atomicOr(status, 2);
        Br[c] = o;
      }
      __syncwarp();
    }
  }
}

}  // namespace

bool tc_invert_supported(int n) { return n >= 2 && n <= 256; }

void invert_blocks_tc(float2* mats, int n, int64_t nmat, double scale, int* status, cudaStream_t st) {
  VS_REQUIRE(tc_invert_supported(n), "tensor-core inversion takes blocks of 2..256");
  if (nmat <= 0) return;
  int q_tiles = 1, NT = 16;
  update_tiling(n, &q_tiles, &NT);
  const int r_tiles = (n + kRowsPerTile - 1) / kRowsPerTile;
  int dev = 0, nsm = 0;
  VS_CUDA(cudaGetDevice(&dev));
  VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t psm = panel_smem(n), usm = update_smem(NT), fsm = n * sizeof(int) + 16 + 8 * n * sizeof(float2);
  const int rpw = (n + 7) / 8;
  auto kp = rpw <= 4 ? k_tc_panel<4> : rpw <= 8 ? k_tc_panel<8> : rpw <= 16 ? k_tc_panel<16>
          : rpw <= 24 ? k_tc_panel<24> : k_tc_panel<32>;
  set_kernel_smem((const void*)kp, psm);
  set_kernel_smem((const void*)k_tc_update, usm);
  set_kernel_smem((const void*)k_tc_finish, fsm);
  int per_sm = 0;
  VS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, kPanelThreads, psm));
  // Matrices in chunks that stay resident in L2 across all panels of the
  // chunk (each panel re-reads and rewrites every matrix): one panel-kernel
  // wave, at most ~80 MB of matrices (the GB300's L2 is 129 MB).
  const int64_t l2_fit = std::max<int64_t>(1, (int64_t(80) << 20) / ((int64_t)n * n * 8));
  const int64_t wave = (int64_t)nsm * std::max(per_sm, 1);
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nmat, std::min(wave, l2_fit)));
  DevBuf V, perm;
  V.alloc((size_t)chunk * kNB * n * sizeof(float2));
  perm.alloc((size_t)chunk * n * sizeof(int));
  for (int64_t m0 = 0; m0 < nmat; m0 += chunk) {
    const int64_t cm = std::min(chunk, nmat - m0);
    float2* mc = mats + m0 * (int64_t)n * n;
    const int pgrid = (int)std::min<int64_t>(cm, (int64_t)nsm * std::max(per_sm, 1));
    for (int k0 = 0; k0 < n; k0 += kNB) {
      kp<<<pgrid, kPanelThreads, psm, st>>>(mc, n, cm, k0, V.as<float2>(), perm.as<int>(), status);
      VS_LAUNCH_CHECK();
      const int64_t ublocks = cm * r_tiles * q_tiles;
      VS_REQUIRE(ublocks < (int64_t(1) << 31), "too many blocks for one launch");
      k_tc_update<<<(unsigned)ublocks, kUpdThreads, usm, st>>>(mc, n, cm, k0, V.as<float2>(), NT, q_tiles, r_tiles,
                                                                status);
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
