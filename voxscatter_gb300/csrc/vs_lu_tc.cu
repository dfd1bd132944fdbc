// Batched inversion of the 2-level circulant preconditioner's 3N x 3N blocks
// (the parfor of inv(...) at main_DDA.m:107-111, main_koch.m:114-118) with the
// trailing updates on the tensor cores.
//
// Blocked Gauss-Jordan with partial pivoting on nmat row-major n x n FP32
// complex matrices in global memory, n <= 256, one persistent CTA per matrix
// at a time so that the matrix stays L2-resident across its panels.  Per
// 32-column panel:
//   * the panel's n x nb columns are reduced by nb unblocked steps held in
//     registers (pivot search among the rows not yet used, row swap, pivot
//     row scaled, column eliminated from every other row), which leaves
//     Panel = [A_KK^-1 ; -A_OK A_KK^-1] for the pivot rows K and the other
//     rows O;
//   * the panel's row swaps are applied to the other columns, whose rows K
//     (after the swaps) go straight into the MMA's B operand;
//   * every column c outside the panel becomes c_new = (c with rows K zeroed)
//     + Panel * c_K, a rank-nb complex update done one 64-row tile at a time
//     by tcgen05 MMAs.  Complex products run as real MMAs with 2 x 2 blocks:
//     output row 2r+e (e = 0 real, 1 imaginary part of row r) and reduction
//     index 2k+f give A~[2r, 2k..2k+1] = (Re, -Im), A~[2r+1, 2k..2k+1] =
//     (Im, Re) of Panel[r, k] and B~[q, 2k..2k+1] = (Re, Im) of the pivot row
//     k at column q, so one M = 128 MMA covers 64 complex rows with real and
//     imaginary parts interleaved in TMEM lanes.  Each FP32 operand x is split
//     into x_hi = tf32(x) and x_lo = x - x_hi and the product formed as
//     A_hi B_hi + A_hi B_lo + A_lo B_hi (3xTF32), accumulated in FP32 in TMEM,
//     which keeps FP32 accuracy on the TF32 tensor pipe.
// After the last panel the column interchanges are undone in one composed
// permutation, the result scaled and non-finite entries flagged.
// Status bits: 1 zero pivot, 2 non-finite result, 8 an MMA completion wait ran
// out (the CTA then waits again, bounded, frees its TMEM and stops).
#include "vs_internal.h"
#include "vs_tc.cuh"

namespace vs {

namespace {

constexpr int kNB = 32;             // panel width (complex columns)
constexpr int kK = 2 * kNB;         // real reduction length of one panel
constexpr int kRowsPerTile = 64;    // complex rows per MMA tile (M = 128 real rows)
constexpr int kTQ = 64;             // column tile of the row permutation (staging buffer [2 NB][TQ])
constexpr uint32_t kMmaPolls = 1u << 22;

__device__ __forceinline__ float2 crecipf(float2 a) {
  const float d = a.x * a.x + a.y * a.y;
  return make_float2(a.x / d, -a.y / d);
}

// nb unblocked Gauss-Jordan steps on a register-resident panel: lane c holds
// column c of the panel for the warp's rows (8 warps, row r in warp r % 8 at
// slot r / 8), so a row's column kk (the elimination multiplier) is one
// shuffle away and only the pivot search, the row swap and the scaled pivot
// row cross warps (three barriers per step).  Slot updates are selects over
// every slot, so the array stays in registers.  rowsrc / piv (thread 0) record
// the row interchanges; a zero pivot sets status bit 1.
template <int kPanelRows>
__device__ __forceinline__ void panel_steps(float2 (&P)[kPanelRows], int n, int k0, int nb, float2* prow, float2* swk,
                                            float2* swp, float* cand_m, int* cand_i, int* rowsrc, int* piv,
                                            int* status) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float2 z2 = make_float2(0.f, 0.f);
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
}

// Fused persistent inversion: one CTA per block at a time (grid-stride over
// the batch), the block staying L2-resident across all its panels.  Per
// 32-column panel: the register panel steps (panel_steps); the panel's row
// swaps applied to the other columns while the saved pivot rows are written
// straight into the MMA's B operand (hi/lo, K-major cores) -- no global
// scratch; then for every 64-row tile the A operand is staged from the
// panel's columns, 8 K-steps x 3 tcgen05 MMAs (3xTF32, N = NTB columns) run
// into TMEM, and the epilogue adds the product to the block in place (its old
// values loaded while the MMAs run).  TMEM is allocated once per CTA.  After
// the last panel the column interchanges are undone, the result scaled and
// checked.  Status bits as invert_blocks_tc; an MMA wait that runs out ends
// the CTA (after a second bounded wait) with bit 8 set.
size_t fused_smem(int n, int NTB) {
  return 128 + 2ull * 128 * kK * 4 + 2ull * NTB * kK * 4 + 3ull * kNB * sizeof(float2) +
         (5ull * n + 2 * kNB + 16) * sizeof(int);
}

constexpr int kFusedChunks = 8;  // 16-column chunks per warp of the epilogue (NTB <= 256)

template <int kPanelRows>
__global__ void __launch_bounds__(256, 1) k_tc_fused(float2* __restrict__ mats, int n, int64_t nmat, int NTB,
                                                     float scale, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((128u - (tc::smem_addr(smem_raw) & 127u)) & 127u);
  unsigned char* sAh = base;  // also the staging buffer of the swaps, [2*NB][TQ] complex (32 KB)
  unsigned char* sAl = sAh + 128 * kK * 4;
  unsigned char* sBh = sAl + 128 * kK * 4;  // also the row buffers of the final permutation
  unsigned char* sBl = sBh + (size_t)NTB * kK * 4;
  float2* prow = reinterpret_cast<float2*>(sBl + (size_t)NTB * kK * 4);
  float2* swk = prow + kNB;
  float2* swp = swk + kNB;
  int* rowsrc = reinterpret_cast<int*>(swp + kNB);
  int* oidx = rowsrc + n;
  int* olist = oidx + n;
  int* piv = olist + kNB;   // [NB] this panel
  int* perm = piv + kNB;    // [n] all panels
  int* cmap = perm + n;     // [n]
  float* cand_m = reinterpret_cast<float*>(cmap + n);
  int* cand_i = reinterpret_cast<int*>(cand_m + 8);
  float2* buf = reinterpret_cast<float2*>(sAh);
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_ocnt;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float2 z2 = make_float2(0.f, 0.f);
  const uint32_t ncols = NTB <= 128 ? 128u : 256u;
  if (warp == 0) tc::tmem_alloc(&s_tmem, ncols);
  if (tid == 0) tc::mbar_init(&s_bar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  uint32_t phase = 0;
  bool aborted = false;
  const int r_tiles = (n + kRowsPerTile - 1) / kRowsPerTile;
  const uint32_t idesc = tc::idesc_tf32(128, NTB);
  const uint32_t sbo = (kK / 4) * 128;
  const int qd = warp & 3, half = warp >> 2;
  const bool odd = lane & 1;
  for (int64_t b = blockIdx.x; b < nmat && !aborted; b += gridDim.x) {
    float2* B = mats + b * (int64_t)n * n;
    for (int r = tid; r < n; r += blockDim.x) {
      rowsrc[r] = r;
      oidx[r] = -1;
    }
    for (int k0 = 0; k0 < n && !aborted; k0 += kNB) {
      const int nb = min(kNB, n - k0);
      float2 P[kPanelRows];
#pragma unroll
      for (int i = 0; i < kPanelRows; ++i) {
        const int r = warp + 8 * i;
        P[i] = (r < n && lane < nb) ? B[(int64_t)r * n + k0 + lane] : z2;
      }
      __syncthreads();
      panel_steps<kPanelRows>(P, n, k0, nb, prow, swk, swp, cand_m, cand_i, rowsrc, piv, status);
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
      const int ocnt = s_ocnt;
      // the other columns: their old pivot rows into the B operand, the rows
      // below the panel that a swap changed receive their old pivot row
      for (int q0 = 0; q0 < NTB; q0 += kTQ) {
        for (int u = tid; u < (nb + ocnt) * kTQ; u += blockDim.x) {
          const int rr = u / kTQ, qi = u - rr * kTQ, q = q0 + qi;
          if (q >= n || (q >= k0 && q < k0 + nb)) continue;
          const int src = rr < nb ? rowsrc[k0 + rr] : rowsrc[olist[rr - nb]];
          buf[rr * kTQ + qi] = B[(int64_t)src * n + q];
        }
        __syncthreads();
        for (int u = tid; u < kTQ * (kK / 4); u += blockDim.x) {
          const int ql = u % kTQ, c = u / kTQ, q = q0 + ql;
          if (q >= NTB) continue;
          const bool on = q < n && !(q >= k0 && q < k0 + nb);
          const float2 w0 = (on && 2 * c < nb) ? buf[(2 * c) * kTQ + ql] : z2;
          const float2 w1 = (on && 2 * c + 1 < nb) ? buf[(2 * c + 1) * kTQ + ql] : z2;
          const float4 v = make_float4(w0.x, w0.y, w1.x, w1.y);
          const float4 h = make_float4(tc::to_tf32(v.x), tc::to_tf32(v.y), tc::to_tf32(v.z), tc::to_tf32(v.w));
          const uint32_t off = tc::kmajor_offset(q, 4 * c, kK);
          *reinterpret_cast<float4*>(sBh + off) = h;
          *reinterpret_cast<float4*>(sBl + off) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
        }
        for (int u = tid; u < ocnt * kTQ; u += blockDim.x) {
          const int o = u / kTQ, qi = u - o * kTQ, q = q0 + qi;
          if (q >= n || (q >= k0 && q < k0 + nb)) continue;
          B[(int64_t)olist[o] * n + q] = buf[(nb + o) * kTQ + qi];
        }
        __syncthreads();
      }
      // trailing update, one 64-row tile at a time
      for (int rt = 0; rt < r_tiles; ++rt) {
        const int r0 = rt * kRowsPerTile;
        for (int u = tid; u < 128 * (kK / 4); u += blockDim.x) {
          const int R = u & 127, c = u >> 7, r = r0 + (R >> 1);
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
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
          const uint32_t ah = tc::smem_addr(sAh), al = tc::smem_addr(sAl), bh = tc::smem_addr(sBh),
                         bl = tc::smem_addr(sBl);
          const int steps = (2 * nb + 7) / 8;
          for (int st = 0; st < steps; ++st) {
            const uint32_t o = st * 256;
            tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, sbo), tc::smem_desc(bh + o, 128, sbo), idesc,
                         st > 0 ? 1u : 0u);
            tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, sbo), tc::smem_desc(bl + o, 128, sbo), idesc, 1u);
            tc::mma_tf32(tmem, tc::smem_desc(al + o, 128, sbo), tc::smem_desc(bh + o, 128, sbo), idesc, 1u);
          }
          tc::mma_commit(&s_bar);
        }
        // the epilogue's old values, loaded while the MMAs run
        const int r_e = r0 + 16 * qd + (lane >> 1);
        const bool inK = r_e >= k0 && r_e < k0 + nb;
        float2 basev[kFusedChunks][8];
#pragma unroll
        for (int j = 0; j < kFusedChunks; ++j) {
          const int qb = 16 * half + 32 * j + (odd ? 8 : 0);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int q = qb + i;
            const bool ld = 16 * half + 32 * j < NTB && r_e < n && q < n && !inK && !(q >= k0 && q < k0 + nb);
            basev[j][i] = ld ? B[(int64_t)r_e * n + q] : z2;
          }
        }
        const bool ok = tc::mbar_wait(&s_bar, phase, kMmaPolls);
        const bool any_fail = __syncthreads_or(!ok);
        if (any_fail) {
          if (tid == 0) atomicOr(status, 8);
          tc::mbar_wait(&s_bar, phase, kMmaPolls);  // the MMAs in flight finish before TMEM is freed
          aborted = true;
          break;
        }
        phase ^= 1u;
        tc::fence_after_sync();
#pragma unroll
        for (int j = 0; j < kFusedChunks; ++j) {
          const int c = 16 * half + 32 * j;
          if (c >= NTB) break;
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
            const int qb = c + (odd ? 8 : 0);
            float2* row = B + (int64_t)r_e * n;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const int q = qb + i;
              if (q >= n || (q >= k0 && q < k0 + nb)) continue;
              row[q] = make_float2(basev[j][i].x + d[i].x, basev[j][i].y + d[i].y);
            }
          }
        }
        tc::fence_before_sync();
        __syncthreads();  // TMEM and the A operand are reused by the next tile
        tc::fence_after_sync();
      }
    }
    if (aborted) break;
    // undo the column interchanges, scale, flag non-finite entries
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
    float2* rowbuf = reinterpret_cast<float2*>(sBh) + (size_t)warp * n;
    for (int r = warp; r < n; r += 8) {
      float2* Br = B + (int64_t)r * n;
      for (int c = lane; c < n; c += 32) rowbuf[c] = Br[c];
      __syncwarp();
      for (int c = lane; c < n; c += 32) {
        const float2 a = rowbuf[cmap[c]];
        const float2 o = make_float2(a.x * scale, a.y * scale);
        if (!(isfinite(o.x) && isfinite(o.y))) atomicOr(status, 2);
        Br[c] = o;
      }
      __syncwarp();
    }
    __syncthreads();  // the row buffers are the next block's B operand
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, ncols);
  }
}

}  // namespace

bool tc_invert_supported(int n) { return n >= 2 && n <= 256; }

void invert_blocks_tc(float2* mats, int n, int64_t nmat, double scale, int* status, cudaStream_t st) {
  VS_REQUIRE(tc_invert_supported(n), "tensor-core inversion takes blocks of 2..256");
  if (nmat <= 0) return;
  {
    // the fused persistent kernel: one CTA per block at a time
    const int NTB = (n + 15) / 16 * 16;
    const size_t fsm = fused_smem(n, NTB);
    if (fsm <= 227 * 1024) {
      const int rpw = (n + 7) / 8;
      auto kf = rpw <= 4 ? k_tc_fused<4> : rpw <= 8 ? k_tc_fused<8> : rpw <= 16 ? k_tc_fused<16>
              : rpw <= 24 ? k_tc_fused<24> : k_tc_fused<32>;
      set_kernel_smem((const void*)kf, fsm);
      int dev = 0, nsm = 0;
      VS_CUDA(cudaGetDevice(&dev));
      VS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      kf<<<(int)std::min<int64_t>(nmat, nsm), 256, fsm, st>>>(mats, n, nmat, NTB, (float)scale, status);
      VS_LAUNCH_CHECK();
      return;
    }
  }
  throw Error(VS_ERR_UNSUPPORTED, "tensor-core inversion: block of " + std::to_string(n) + " does not fit");
}

}  // namespace vs
