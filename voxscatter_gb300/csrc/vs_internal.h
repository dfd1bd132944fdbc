// Internal objects behind the C-ABI handles.
#pragma once
#include "vs_common.cuh"
#include "vs_fft.cuh"
#include <memory>
#include <vector>
#include <string>
#include <atomic>

namespace vs {

// Owned device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    if (n <= bytes && p) return;
    release();
    if (n == 0) return;
    VS_CUDA(cudaMalloc(&p, n));
    bytes = n;
  }
  template <typename X> X* as() const { return reinterpret_cast<X*>(p); }
};

// One FFT axis: plan plus forward twiddle tables in both precisions.
struct FftAxis {
  FftPlan plan;
  DevBuf tw32, tw64;
  void init(int n, cudaStream_t st);
  template <typename T> const cplx_t<T>* tw() const;
};
template <> inline const float2* FftAxis::tw<float>() const { return tw32.as<float2>(); }
template <> inline const double2* FftAxis::tw<double>() const { return tw64.as<double2>(); }

// Launch shape of the FFT passes and of the block GEMV, chosen per operator /
// preconditioner and precision by the autotuner (log2 values; -1 = default).
struct PassShape {
  int lg_lpb_x = -1;   // x passes: lines per CTA
  int lg_tx_y = -1;    // y passes: x-tile width
  int y_reg = -1;      // y passes: 1 two-level register kernel, 0 shared-memory Stockham, -1 default (Stockham),
                       // 2 (operators' FP64 data) two-level in double-float arithmetic
  int x_reg = -1;      // x passes: as y_reg
  int lg_tx_z = -1;    // z pass: x-tile width
  int gemv_ti = 0;     // preconditioner GEMV: stored blocks per CTA (direct) or CTAs per SM (streamed); 0 = default
  int gemv_threads = 0;
  int gemv_mode = -1;  // 0 register-direct GEMV, 1 streamed through shared memory, 2 packed symmetric blocks,
                       // -1 default (streamed)
  int gemv_chunk = 0;  // streamed GEMV: block columns per bulk copy (0 = default)
  int z_reg = -1;      // z pass: 0 shared-memory Stockham, 1 two-level, 2 two-level with register cap, -1 default
  int fuse_xy = -1;    // preconditioner: 1 both x/y FFTs of a plane in one CTA (when it fits), 0/-1 separate passes
  int z_df = -1;       // c128 z pass: 1 double-float arithmetic on the FP64 data (two-level kernel only)
  int wait_polls = 0;  // streamed GEMV: polls before a wait on another warp role gives up (0: 2^20, -1: none)
};

// Gram of each right-hand side, in place of the operator's (the reference
// passes Gram to every MVP call, and the DDA drivers' Gram = 1/alpha_LDR
// depends on the incident direction and polarisation, getOPERATOR_DDA.m:14-26):
// nrhs x per complex values at the unknowns, per = 1 (a scalar per
// right-hand side) or n3.  Empty (g32 == g64 == nullptr): the operator's Gram.
struct RhsGram {
  const float2* g32 = nullptr;
  const double2* g64 = nullptr;
  int64_t per = 0;
  bool empty() const { return g32 == nullptr && g64 == nullptr; }
};

// Work vectors and device scalars of the Krylov solvers (vs_krylov.cu).
// A captured iteration graph and the buffers/settings it was captured with.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  std::vector<const void*> key;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key.clear();
  }
  ~GraphCache() { reset(); }
};

// CUDA events of an instrumented iteration graph, destroyed with the work
// area (after the graphs that record them: declared before them).
struct EventSet {
  std::vector<cudaEvent_t> ev;
  void ensure(size_t n) {
    while (ev.size() < n) {
      cudaEvent_t e;
      VS_CUDA(cudaEventCreate(&e));
      ev.push_back(e);
    }
  }
  EventSet() = default;
  EventSet(const EventSet&) = delete;
  EventSet& operator=(const EventSet&) = delete;
  ~EventSet() {
    for (auto e : ev) cudaEventDestroy(e);
  }
};

struct KrylovWork {
  EventSet prof_ev;                      // events of the profiled BiCGSTAB graph
  DevBuf r, rt, p, v_, s, t, ph, sh, x;  // in the inner solver's precision
  DevBuf r64, y64;                       // FP64 residual / matvec output
  DevBuf partials, state, scal, resvec;
  DevBuf xpart;                          // per-CTA partial sums of the folded BiCGSTAB steps
  GraphCache graph32, graph64;           // BiCGSTAB iteration graphs (c64 / c128)
  // GMRES(m): Krylov basis, Hessenberg (column-major, m+1 rows), rotations,
  // right-hand side g, solution y, pass coefficients, partial dots, state,
  // and the vectors w, tmp and the correction d.
  DevBuf gV, gH, gcs, gsn, gg, gy, ghp, gpart, gstate, gw, gtmp, gd;
  // GCRO-DR: the basis [C | V] in one array (C in the slots just below V),
  // recycled U, the next U and C, the solution in the preconditioned space,
  // the residual, the stacked [C^H A M V; Hessenberg] columns, partial and
  // final Gram products, combination coefficients.
  DevBuf rCV, rU, rU2, rC2, rz, rr, rBH, rgpart, rgram, rcoef;
  // Gram of each right-hand side of the current solve (empty: the operator's)
  DevBuf rg32, rg64;
  RhsGram rg;
  template <typename T> void ensure(int64_t n);
};

}  // namespace vs

// A context lives until vs_ctx_destroy has been called and the last operator
// or preconditioner created on it is destroyed (each holds a reference), so
// handles can be released in any order.
struct vs_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  vs::DevBuf stage;  // host<->device staging for the host-buffer entry points
  std::atomic<int> refs{1};
  // lockstep multi-particle solves: the auxiliary streams their graphs' branches
  // are captured on, the cached iteration graphs, and the device table of the
  // particles' states / rhs offsets / gathered skip flags
  std::vector<cudaStream_t> aux;
  vs::GraphCache pgraph32, pgraph64;
  vs::DevBuf pstates, poff, pskip;
};
void ctx_retain(vs_ctx* ctx);
void ctx_release(vs_ctx* ctx);
// Records a failure message where vs_last_error() reads it: on the context
// (if any) and as this thread's last error.
void record_error(vs_ctx* ctx, const char* msg);

// Diagonal coefficients of an operator at the n3 unknown positions.
struct VsDiagDev {
  bool arr = false;
  double2 s = {0, 0};
  vs::DevBuf v32, v64;
  template <typename T> const vs::cplx_t<T>* ptr() const;
};
template <> inline const float2* VsDiagDev::ptr<float>() const { return arr ? v32.as<float2>() : nullptr; }
template <> inline const double2* VsDiagDev::ptr<double>() const { return arr ? v64.as<double2>() : nullptr; }

struct vs_op {
  vs_ctx* ctx = nullptr;  // retained while the operator exists
  ~vs_op() { ctx_release(ctx); }
  int L = 0, M = 0, N = 0, P = 0, Q = 0, R = 0;
  int64_t V = 0, n3 = 0;
  vs::DevBuf map3;      // int32[3V]: unknown position of each grid entry, -1 if absent
  vs::DevBuf pos2grid;  // int32[n3]: grid entry of each unknown
  vs::DevBuf map_all;   // int32[3V]: identity map of whole-domain applies (built on first use)
  VsDiagDev d1, d1c, d2;  // Gram.*Mr, Gram.*conj(Mr), Mc at the unknowns
  VsDiagDev mr;           // Mr at the unknowns (with a Gram per right-hand side)
  bool gsym = false;    // G holds only the first octant (exact per-axis parity)
  vs::DevBuf G32, G64;  // spectrum of the embedded tensor / (P*Q*R): 6 x P*Q*R, or 6 x octant
  vs::DevBuf toep64;    // first-octant Toeplitz tensor, L*M*N*6 (double2)
  vs::FftAxis ax[3];
  vs::DevBuf t1, t2;    // pipeline intermediates
  vs::DevBuf xin, yout; // device staging for host-buffer applies
  vs::KrylovWork kw;    // solver state for vs_solve on this operator
  vs::PassShape shape[2];  // [0] c64, [1] c128 pipeline launch shapes
  bool std3 = false;    // idx3 = [idx; V+idx; 2V+idx] (the reference's idx3 form)
};

// 2-level circulant preconditioner: inverse blocks per (x,y) frequency.
struct vs_prec {
  vs_ctx* ctx = nullptr;    // retained while the preconditioner exists
  ~vs_prec() { ctx_release(ctx); }
  uint64_t id = 0;          // unique per preconditioner object (keys cached solver graphs)
  int L = 0, M = 0, N = 0;
  bool sym = false;         // blocks stored for i <= L/2, j <= M/2 only (parity of the operator)
  int64_t V = 0, n3 = 0;
  vs::DevBuf map3;          // int32[3V] unknown position of each grid entry (-1: absent)
  vs::DevBuf inv32, inv64;  // blocks of (3N)^2 (L*M, or (L/2+1)(M/2+1) when sym), column-major, / (L*M)
  vs::FftAxis axL, axM;
  vs::DevBuf t;             // apply scratch (L,M,N,3) per right-hand side
  vs::DevBuf xin, yout;
  int nrhs_cap = 0;
  vs::PassShape shape[2];   // [0] c64, [1] c128 apply launch shapes
  vs::DevBuf gemv_status;   // int: bit 4 set when a streamed-GEMV wait ran out
  // lower triangles of S = B D (D negates the x and y components), packed per
  // block with pk_stride entries; present when the blocks are symmetric so
  vs::DevBuf pk32, pk64;
  int64_t pk_stride = 0;
};

namespace vs {

template <typename T>
struct XFuse;  // a BiCGSTAB step folded into a two-level x pass (vs_pipeline.cuh)

// CTAs of a two-level x pass of length P over nlines lines (0: P has no
// two-level kernel); the solver sizes the folded steps' partial sums by it.
int x2_ctas(int P, int nlines);

// Launchers (vs_matvec.cu)
// rg: optional Gram of each right-hand side (nullptr or empty: the operator's).
// fz: optional solver step folded into the inverse x pass (pass 4).
template <typename T>
void matvec_pass(const vs_op& op, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, int mode, const int* skip,
                 cudaStream_t st, int pass, int skip_stride = 0, const RhsGram* rg = nullptr,
                 const XFuse<T>* fz = nullptr);
template <typename T>
void matvec_scratch(const vs_op& op, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, int mode, cplx_t<T>* t1,
                    cplx_t<T>* t2, cudaStream_t st);
// skip: optional device flags; right-hand side r is skipped (no work) when
// skip[r * skip_stride] != 0.
template <typename T>
void matvec(const vs_op& op, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, int mode, const int* skip,
            cudaStream_t st, int skip_stride = 0, const RhsGram* rg = nullptr);
void ensure_scratch(vs_op& op, int nrhs, size_t elem_bytes);
// Fills n complex values (c128 when dbl, else c64) with seeded values in
// [-0.5, 0.5): the autotuners time the passes on data like a solve's (the
// double-float kernels take a shorter path for zeros).
void fill_tuning_data(void* x, int64_t n, bool dbl, cudaStream_t st);
// Uploads a Gram per right-hand side (host, nrhs x gram_n complex with
// gram_n = 1 or L*M*N, a column-major grid) to g64 / g32 at op's unknowns and
// describes it in `out`.
void upload_rhs_gram(const vs_op& op, const double2* gram, int64_t nrhs, int64_t gram_n, DevBuf& g64, DevBuf& g32,
                     RhsGram& out, cudaStream_t st);

// Generic batched FFT passes (vs_matvec.cu)
template <typename T, bool INV>
void fft_axis0(cplx_t<T>* data, int n, int64_t nlines, const FftAxis& ax, cudaStream_t st);
template <typename T, bool INV>
void fft_strided(cplx_t<T>* data, int xext, int n, int64_t row_stride, int na, int64_t stride_a, int nb,
                 int64_t stride_b, const FftAxis& ax, cudaStream_t st);

// Green tensor and embedding (vs_green.cu)
void green_dda_device(int L, int M, int N, const double* ox, const double* oy, const double* oz, double ko,
                      int near_quad, double2* toep, cudaStream_t st);
void embed_fft_device(int L, int M, int N, const double2* toep, int P, int Q, int R, double2* out,
                      FftAxis* ax, cudaStream_t st);
void toep_from_fN_device(int L, int M, int N, int P, int Q, int R, double2* fN_inplace, double2* toep,
                         FftAxis* ax, cudaStream_t st);
void octant_spectrum(const double2* fN, int P, int Q, int R, double scale, double2* g64, float2* g32, cudaStream_t st);
bool toeplitz_has_exact_parity(const double* toep, int L, int M, int N);
void finalize_spectrum(const double2* fN, int64_t total, double scale, double2* g64, float2* g32,
                       cudaStream_t st);

// Preconditioner (vs_precond.cu)
void circ_levels_device(int L, int M, int N, const double2* toep, double2* lev1, double2* lev2, const FftAxis& axL,
                        const FftAxis& axM, cudaStream_t st);
// Galerkin N-operator Toeplitz tensor G (L, M, N, 6) on the device (vs_nop.cu);
// near: NULL or the (min(2,L), min(2,M), min(2,N), 6, 6) singular block.
void nop_assemble_device(int L, int M, int N, double ko, double dx, const double2* near, double2* G,
                         cudaStream_t st);

// Smallest instantiated two-level z length >= min_len (5-smooth beyond 256).
int z_pass_length(int min_len);
// lu: how FP32 blocks are inverted: LU_AUTO (one CTA per block in shared
// memory up to 3N = 168, then the tensor-core kernel up to 256, then the
// persistent CUDA-core blocked kernel: the fastest at each measured size),
// LU_TC (tensor-core trailing updates whenever 3N <= 256), LU_CUDA (CUDA-core
// kernels only).  FP64 blocks always use the CUDA-core kernels.
enum { LU_AUTO = 0, LU_TC = 1, LU_CUDA = 2 };
template <typename T>
void assemble_invert(const double2* lev2, int L, int M, int N, double2 shift, const double2* dvec, double2 dscal,
                     bool invert, bool colmajor, double scale, cplx_t<T>* out, int* status, cudaStream_t st,
                     bool sym = false, int lu = LU_AUTO);
// Batched in-place inversion of nmat row-major n x n FP32 complex matrices
// (n <= 256) by blocked Gauss-Jordan with tcgen05 trailing updates
// (vs_lu_tc.cu); results scaled by `scale`; status bits 1 zero pivot,
// 2 non-finite result, 8 an MMA wait ran out.
bool tc_invert_supported(int n);
void invert_blocks_tc(float2* mats, int n, int64_t nmat, double scale, int* status, cudaStream_t st);
// In-place inversion of nmat n x n FP32 complex matrices on the device: the
// tensor-core kernel (n <= 256 unless lu == LU_CUDA) or the blocked CUDA-core
// kernel.
void invert_blocks_device(float2* mats, int n, int64_t nmat, int lu, double scale, int* status, cudaStream_t st);
// fz: optional solver step folded into the forward x pass (pass 0).
template <typename T>
void prec_apply_pass(const vs_prec& pr, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, const int* skip,
                     cudaStream_t st, int pass, int skip_stride = 0, const XFuse<T>* fz = nullptr);
// kernel launches of one preconditioner apply (3 with fused x/y planes, else 5)
template <typename T>
int prec_launches(const vs_prec& pr);
template <typename T>
void prec_apply(const vs_prec& pr, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, const int* skip, cudaStream_t st,
                int skip_stride = 0);

// Physics (vs_physics.cu)
const int* domain_map(vs_op& op, cudaStream_t st);
template <typename T>
void matvec_domain(vs_op& op, const cplx_t<T>* x, cplx_t<T>* y, int nrhs, cplx_t<T> ca, cplx_t<T> cb,
                   cudaStream_t st);
template <typename C>
void to_grid(const vs_op& op, const C* x, C* grid, int nrhs, cudaStream_t st);
template <typename C>
void field_combine(const C* einc, const C* y, const C* pgrid, double2 inv_chi, int64_t n, double2* e,
                   cudaStream_t st);
void far_field_device(const vs_op& op, const double2* P, int nrhs, const double* xs, const double* ys,
                      const double* zs, const double* dirs, int ndir, double ko, double dV, double2* F,
                      cudaStream_t st);
void plane_wave_device(const vs_op& op, const double* x, const double* y, const double* z, const double kvec[3],
                       const double2 E0[3], double2* b, cudaStream_t st);
void conj_device(const double2* a, double2* b, int64_t n, cudaStream_t st);
double cext_device(const double2* P, const double2* E, int64_t n, double scale, cudaStream_t st);
void cext_grad_device(const double2* P, const double2* lam, const double2* eps, int64_t nvox, double c, double bterm,
                      double* gre, double* gim, cudaStream_t st);

// Autotuning of the launch shapes (vs_matvec.cu / vs_precond.cu): times a few
// candidate shapes of every pass with CUDA events and keeps the fastest.
template <typename T>
void autotune_op(vs_op& op, cudaStream_t st);
template <typename T>
void autotune_prec(vs_prec& pr, cudaStream_t st);
void pack_sym_blocks(vs_prec& pr, cudaStream_t st);

// Elementwise helpers (vs_matvec.cu)
void c128_to_c64(const double2* in, float2* out, int64_t n, cudaStream_t st);
void c64_to_c128(const float2* in, double2* out, int64_t n, cudaStream_t st);

}  // namespace vs
