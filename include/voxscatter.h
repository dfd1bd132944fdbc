/*
 * libvoxscatter: GB300 (sm_103a) FFT-accelerated DDA / Galerkin-JVIE solver.
 *
 * C ABI for the hot path of VoxScatter (MATLAB).  Every entry point returns an
 * int status (VS_OK = 0); on failure vs_last_error() gives the message.  All
 * complex arrays are interleaved (re, im) doubles, the layout of MATLAB
 * R2018a+ interleaved-complex mxArrays and of C99 double _Complex.  Grid arrays
 * are column-major (x fastest), exactly as MATLAB stores them.  Voxel and
 * unknown indices are 0-based (MATLAB's idx - 1).
 *
 * Host buffers are owned by the caller and only read or written during the
 * call.  Device objects (contexts, operators, preconditioners) are owned by
 * their handles.  A context owns one CUDA stream on one device; calls on one
 * context are serialised on that stream.  There is no CPU fallback: without a
 * usable sm_103a device, vs_ctx_create fails.
 */
#ifndef VOXSCATTER_H
#define VOXSCATTER_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum vs_status {
  VS_OK = 0,
  VS_ERR_ARG = 1,          /* invalid argument (sizes, null pointers, mode)        */
  VS_ERR_CUDA = 2,         /* CUDA runtime error                                   */
  VS_ERR_OOM = 3,          /* device allocation failed                             */
  VS_ERR_NONFINITE = 4,    /* NaN/Inf in an input vector                           */
  VS_ERR_UNSUPPORTED = 5,  /* size outside what the kernels support                */
  VS_ERR_TIMEOUT = 6       /* a bounded device-side wait gave up                   */
};

/* Apply modes of an operator (MVP.m transp_flag plus the plain transpose). */
enum vs_mode {
  VS_NOTRANSP = 0,   /* y = Gram.*Mr.*x - Mc.*N(x)                  MVP.m:101-131 */
  VS_TRANSP = 1,     /* y = Gram.*Mr.*x - N(Mc.*x)   (A^T, complex symmetric N)    */
  VS_CONJTRANSP = 2  /* y = Gram.*conj(Mr).*x - conj(N(Mc.*conj(x)))  MVP.m:65-98 */
};

/* Arithmetic of an apply. */
enum vs_precision { VS_C64 = 0, VS_C128 = 1 };

typedef struct vs_ctx vs_ctx;
typedef struct vs_op vs_op;

/* ---- context --------------------------------------------------------- */

/* Create a context on CUDA device `device` (one stream, owned). */
int vs_ctx_create(int device, vs_ctx** out);
int vs_ctx_destroy(vs_ctx* ctx);
/* Message of the last failure on `ctx` (or of the last failing call on this
 * thread when ctx is NULL).  Valid until the next call on the context. */
const char* vs_last_error(const vs_ctx* ctx);
/* Block until all work queued on the context's stream has finished. */
int vs_ctx_synchronize(vs_ctx* ctx);
/* The context's cudaStream_t, for callers that interleave their own work. */
int vs_ctx_stream(vs_ctx* ctx, void** stream);

/* ---- operator assembly (setup, FP64 on the device) ------------------- */

/* Draine-Flatau interaction tensor at every grid offset, 6 components
 * (xx,xy,xz,yy,yz,zz), G(0)=0.  Replaces the triple loop of
 * src/src_vie/src_operators/getOPERATOR_DDA.m:29-119.
 *   ox[L], oy[M], oz[N]: coordinate offsets r(i,1,1,1)-r(1,1,1,1), etc.
 *   near_quad: 0 = 'off' (point DDA); 1 = 'on' (10^3 Gauss-Legendre average of
 *   the kernel over the voxel for 0 < |R| < 5*ox[1], getOPERATOR_DDA.m:47-79).
 *   toep_out: L*M*N*6 complex, column-major (L,M,N,6). */
int vs_green_dda(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* ox, const double* oy,
                 const double* oz, double ko, int near_quad, double* toep_out);

/* LDR polarisability per element, getOPERATOR_DDA.m:7-26 (host arithmetic).
 *   m: n complex values, refractive index (is_eps = 0) or permittivity m^2
 *   (is_eps = 1).  alpha_out: n complex (dimensionless, i.e. divided by d^3). */
int vs_alpha_ldr(const double* m, int64_t n, int is_eps, double ko, double d, const double kvec[3],
                 const double E0[3], double* alpha_out);

/* Parity-signed circulant embedding of a Toeplitz tensor into a P x Q x R grid
 * followed by a forward 3-D FFT of each of the 6 components.  With
 * (P,Q,R) = (2L,2M,2N) this is circulant_nop_const.m:1-40 + fft_operator.m:1-8
 * (the reference's fN); any P >= 2L-1 (etc.) embeds the same operator.
 *   toep: L*M*N*6 complex; fN_out: P*Q*R*6 complex, column-major. */
int vs_circulant_fft(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, int64_t P,
                     int64_t Q, int64_t R, double* fN_out);

/* ---- operator (the MVP function handle) ------------------------------ */

/* Diagonal term of the operator, given as a scalar (n = 1) or per voxel
 * (n = L*M*N, column-major grid, like MVP.m's Mr/Mc/Gram arrays). */
typedef struct vs_diag {
  const double* v; /* complex values */
  int64_t n;       /* 1 or L*M*N     */
} vs_diag;

/* Operator A x = Gram.*Mr.*x - Mc.*N(x) on the unknowns idx3 (MVP.m:1-145).
 *   toep: the first-octant Toeplitz tensor L*M*N*6 (as from vs_green_dda); the
 *         library embeds it at the smallest 7-smooth P >= 2L-1 (etc.) unless
 *         P,Q,R > 0 are given.
 *   idx3: n3 0-based indices into the column-major (L,M,N,3) grid (MATLAB's
 *         idx3 - 1); each grid entry at most once.
 * The Toeplitz tensor is kept on the device for preconditioner builds. */
int vs_op_create(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, int64_t P, int64_t Q,
                 int64_t R, const int64_t* idx3, int64_t n3, vs_diag Mr, vs_diag Mc, vs_diag Gram,
                 vs_op** out);

/* Same operator from the reference's FFT'd circulant fN (P*Q*R*6 complex, as
 * passed to MVP.m).  The Toeplitz tensor is recovered on the device. */
int vs_op_create_fN(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* fN, int64_t P, int64_t Q,
                    int64_t R, const int64_t* idx3, int64_t n3, vs_diag Mr, vs_diag Mc, vs_diag Gram,
                    vs_op** out);

int vs_op_destroy(vs_op* op);

/* Sizes of an operator: L,M,N,P,Q,R and n3 (any pointer may be NULL). */
int vs_op_info(const vs_op* op, int64_t* LMN, int64_t* PQR, int64_t* n3);

/* y = op(x) for nrhs right-hand sides stored one after another (n3 each),
 * host buffers, complex double.  precision VS_C64 runs the fused c64 pipeline
 * (inputs rounded to c64, result widened); VS_C128 runs it in FP64.
 * Replaces MVP.m / mv_AN_const.m with GPU_flag = 0 or 1. */
int vs_op_apply(vs_op* op, const double* x, double* y, int64_t nrhs, int mode, int precision);

/* Same on device buffers already in the precision's type (float2 for VS_C64,
 * double2 for VS_C128), enqueued on the context's stream, no synchronisation. */
int vs_op_apply_device(vs_op* op, const void* x, void* y, int64_t nrhs, int mode, int precision);

#ifdef __cplusplus
}
#endif

#endif /* VOXSCATTER_H */
