// Argument blocks of the FFT passes shared by the matvec and the circulant
// preconditioner (kernels live in vs_matvec.cu).
#pragma once
#include "vs_internal.h"

namespace vs {

// Extra X-pass mode beyond vs_mode: plain gather / plain scatter (no diagonal).
constexpr int MODE_PLAIN = 3;

template <typename C>
struct DiagArg {
  const C* v;
  C s;
  __device__ __forceinline__ C at(int pos) const { return v ? v[pos] : s; }
};

// BiCGSTAB vector steps folded into an x pass (kind XF_NONE: none): the
// gather of the preconditioner's forward x pass forms the vector it
// transforms (XF_GATHER_P: p = r + beta (p - omega v), or p = r on the first
// iteration; XF_GATHER_S: s = r - alpha v, with ||s||^2) and writes it back,
// and the scatter of the matvec's inverse x pass adds the inner products of
// the vector it writes (XF_SCATTER_DOT: rt^H v; XF_SCATTER_OMEGA: t^H s and
// t^H t).  Scalars of right-hand side r are read at sbase + r * sstride +
// offset (bytes), in the storage precision (the solver keeps a float copy of
// each scalar for c64); each CTA writes its NV partial sums to part + r *
// pstride + blockIdx.x * NV (float-float pairs for c64, doubles for c128),
// which the solver adds up afterwards.
enum XFuseKind { XF_NONE = 0, XF_GATHER_P = 1, XF_GATHER_S = 2, XF_SCATTER_DOT = 3, XF_SCATTER_OMEGA = 4 };

template <typename T>
struct XFuse {
  using C = cplx_t<T>;
  int kind;
  const char* sbase;
  int64_t sstride;
  int off_a, off_b, off_iter;  // XF_GATHER_P: beta, omega, iteration counter; XF_GATHER_S: alpha
  const C* u;                  // r (gathers), rt (XF_SCATTER_DOT), s (XF_SCATTER_OMEGA)
  const C* v;                  // v (gathers)
  C* w;                        // p (XF_GATHER_P, read and written), s (XF_GATHER_S, written)
  double* part;
  int64_t pstride;
  // XF_GATHER_S with apart set: alpha = rho / (rt^H v) is taken by the pass
  // itself from the matvec's partial sums at apart + r * pstride (anb CTAs, 2
  // slots each), every CTA adding them in the same order (the same bits) and
  // its thread 0 dividing; CTA 0 stores alpha (FP64 at off_alpha, storage
  // precision at off_a) for the later steps.  A breakdown ends the iteration:
  // every CTA returns before touching a vector, and the last to count in on
  // the counter at off_counter writes the flag and the skip flag.
  const double* apart;
  int anb;
  int off_rho, off_alpha, off_flag, off_skip, off_counter;
  __device__ __forceinline__ C scalar(int rhs, int off) const {
    return *reinterpret_cast<const C*>(sbase + rhs * sstride + off);
  }
};

template <typename T>
struct PipeArgs {
  using C = cplx_t<T>;
  int L, M, N, P, Q, R;
  int64_t V, n3;
  const int* map3;
  const C* x;
  C* y;
  DiagArg<C> d1, d1c, d2;
  C* t1;
  C* t2;
  const C* G;
  const C* twP;
  const C* twQ;
  const C* twR;
  FftPlan pP, pQ, pR;
  int lg_lpb;  // log2 lines per block in the x passes
  int lg_tx;   // log2 x-tile width of the z pass
  const int* skip;   // right-hand side r is skipped when skip[r * skip_stride] != 0
  int skip_stride;
  int two_level;     // x passes: 1 two-level register kernel (vs_xpass.cuh) when P has one,
                     // 2 the same in double-float arithmetic (FP64 data only)
  // Gram of each right-hand side in place of the operator's (the reference
  // passes Gram to every MVP call; DDA's Gram = 1/alpha_LDR depends on the
  // incident direction and polarisation): Gram_r(pos) = grhs[r * grhs_per +
  // (grhs_per > 1 ? pos : 0)], and the diagonal term is Gram_r .* Mr.
  // nullptr: the operator's own d1 / d1c.
  const C* grhs;
  int64_t grhs_per;
  DiagArg<C> mr;
  XFuse<T> fz;  // folded solver step of the two-level x passes (kind XF_NONE: none)
};

// Diagonal coefficient of the XI epilogue at unknown `pos` of right-hand side
// `rhs`: Gram.*Mr, or Gram.*conj(Mr) for VS_CONJTRANSP (MVP.m:72-98 conjugates
// Mr but not Gram).
template <typename T>
__device__ __forceinline__ cplx_t<T> diag_term(const PipeArgs<T>& a, int pos, int rhs, bool conj_mr) {
  if (a.grhs == nullptr) return conj_mr ? a.d1c.at(pos) : a.d1.at(pos);
  const cplx_t<T> g = a.grhs[rhs * a.grhs_per + (a.grhs_per > 1 ? pos : 0)];
  const cplx_t<T> m = a.mr.at(pos);
  return cmul(g, conj_mr ? cconj(m) : m);
}

// ---- strided-axis pass (y of the pipeline; y and z of the setup FFTs) ----
// Lines run along a strided axis; a CTA owns an x-tile of `tx` columns of one
// plane.  Element (x, row) of plane (pa, pb) of the source is at
//   src + pa*s_a + pb*s_b + row*s_row + x      (same form for the destination).
// Rows [0, n_in) are loaded (zero pad up to n), rows [0, n_out) are stored.
// Bytes per CTA of an L2 prefetch of `bytes` over `nctas` CTAs (a multiple of 16).
inline uint64_t prefetch_share(uint64_t bytes, uint64_t nctas) {
  return ((bytes + nctas - 1) / nctas + 15) & ~uint64_t(15);
}

template <typename T>
struct StridedArgs {
  using C = cplx_t<T>;
  const C* src;
  C* dst;
  int xext, n_in, n_out, lg_tx, na;
  int64_t s_row, s_a, s_b, s_rhs;
  int64_t d_row, d_a, d_b, d_rhs;
  FftPlan plan;
  const C* tw;
  const int* skip;
  int skip_stride;
  int two_level;  // 1: two-level register kernel (vs_spass.cuh) when the length has one;
                  // 2: the same in double-float arithmetic (FP64 data only)
  unsigned na_mul;  // ceil(2^32 / na) for na >= 2, else 0 (set by launch_strided_pass)
  // L2 prefetch issued at the start (pf null: none): pf_bytes from pf, split
  // over the CTAs, pf_per_cta bytes each (multiples of 16; the launcher sets
  // pf_per_cta).  The preconditioner's forward y pass uses it for the blocks
  // the streamed GEMV that follows reads first.
  const void* pf;
  uint64_t pf_bytes, pf_per_cta;
  __device__ __forceinline__ void prefetch_l2() const {
    if (pf == nullptr || threadIdx.x != 0) return;
    const uint64_t id = blockIdx.x + (uint64_t)gridDim.x * (blockIdx.y + (uint64_t)gridDim.y * blockIdx.z);
    const uint64_t off = id * pf_per_cta;
    if (off >= pf_bytes) return;
    const uint64_t len = pf_bytes - off < pf_per_cta ? pf_bytes - off : pf_per_cta;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(static_cast<const char*>(pf) + off),
                 "r"((unsigned)len)
                 : "memory");
  }
  // plane (pa, pb) of blockIdx.y = pa + na * pb.  A division by a runtime
  // value goes through integer <-> float conversions, which GB300 runs on its
  // narrow FP64 pipe; the multiply-high by ceil(2^32 / na) is exact for
  // blockIdx.y < 2^16 and na <= 2^16 (the error of the reciprocal times
  // blockIdx.y stays below 1/na).
  __device__ __forceinline__ void plane(int& pa, int& pb) const {
    const unsigned y = blockIdx.y;
    const unsigned q = na_mul ? __umulhi(y, na_mul) : (na == 1 ? y : y / (unsigned)na);
    pb = (int)q;
    pa = (int)(y - q * (unsigned)na);
  }
};

// Two-level x pass (vs_xpass.cuh); false when P has no instantiation.
template <typename T, bool INV>
bool x_two_level(const PipeArgs<T>& a, int mode, int nrhs, cudaStream_t st);

// Two-level strided pass (vs_spass.cuh); false when the length has no instantiation.
template <typename T, bool INV>
bool strided_two_level(const StridedArgs<T>& a, int nplanes, int nrhs, cudaStream_t st);

// Two-level register z pass (vs_zpass.cuh); false when R has no instantiation.
template <typename T, typename K = cplx_t<T>>
bool z_pass_two_level(const PipeArgs<T>& a, bool sym, bool cap, int nrhs, cudaStream_t st);
// c128 storage, double-float arithmetic (vs_zpass_df.cu)
bool z_pass_two_level_df(const PipeArgs<double>& a, bool sym, int nrhs, cudaStream_t st);
// c128 storage, double-float arithmetic of the two-level x and strided passes
// (vs_df_xpass.cu, vs_df_spass.cu); false when the length has no instantiation.
bool x_two_level_df(const PipeArgs<double>& a, bool inverse, int mode, int nrhs, cudaStream_t st);
bool strided_two_level_df(const StridedArgs<double>& a, bool inverse, int nplanes, int nrhs, cudaStream_t st);
bool x_df_available(int P);
bool strided_df_available(int n);

template <typename T>
void launch_x_pass(const PipeArgs<T>& a, bool inverse, int mode, int nrhs, cudaStream_t st);
template <typename T, bool INV>
void launch_strided_pass(const StridedArgs<T>& a, int nplanes, int nrhs, cudaStream_t st);

}  // namespace vs
