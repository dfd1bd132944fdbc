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

/* Galerkin N-operator (JVIE) Toeplitz tensor, the far- and medium-cell part
 * of src/src_vie/src_operators/assembly_nop_const.m:44-92,150-165: face-pair
 * cubature of exp(-i ko R)/R (cubature_nop_const.cpp:8-124) over the 21
 * distinct pairs of the voxel faces, 4x4 Gauss-Legendre points per face for
 * all offsets, 10x10 for offsets < 5 per axis, projected onto the 6 tensor
 * components and divided by 4 pi.  FP64 on the device.
 *   near_J: NULL or the singular near block of assembly_nop_const.m:94-146
 *   (the caller's DIRECTFN/DEMCEM result), nL*nM*nN*6*6 complex, column-major
 *   (mx,my,mz,k,l), nL = min(2,L), nM = min(2,M), nN = min(2,N); with NULL
 *   those cells are zero.
 *   G_out: L*M*N*6 complex, column-major (L,M,N,6) -- the opToeplitz that
 *   vs_op_create takes. */
int vs_nop_assemble(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, double ko, double dx, const double* near_J,
                    double* G_out);

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

/* vs_op_apply with a Gram of each right-hand side in place of the operator's:
 * y_r = Gram_r.*Mr.*x_r - Mc.*N(x_r) (and the transposes as in vs_mode), i.e.
 * MVP.m:1-145 called with that right-hand side's Gram.  The DDA drivers pass
 * Gram = 1/alpha_LDR (main_DDA.m:75), which getOPERATOR_DDA.m:14-26 computes
 * from the incident direction and polarisation, so each (kvec, Eo) of a
 * particle has its own.  gram: nrhs * gram_n complex (host), gram_n = 1 or
 * L*M*N (column-major grid per right-hand side).  Host buffers as vs_op_apply. */
int vs_op_apply_gram(vs_op* op, const double* x, double* y, int64_t nrhs, int mode, int precision,
                     const double* gram, int64_t gram_n);

/* Same as vs_op_apply_device, but allocates nothing: for callers that cannot
 * call cudaMalloc when they apply the operator (services and plug-in hosts
 * that reserve their device memory at start-up and forbid allocation
 * afterwards, or that run inside a memory budget owned by another allocator,
 * such as a MEX function in MATLAB's GPU memory pool).  No counterpart in the
 * reference (its MVP.m allocates freely).  The pipeline intermediates
 * (P*M*N*3 + P*Q*N*3 elements per right-hand side, plus 256 bytes of
 * alignment) live in a 64 MiB array the library reserves on every device that
 * loads it, until the process exits; larger requests return
 * VS_ERR_UNSUPPORTED.  The first call on a device looks up the array's address
 * and caches it for the process (do not reset the device meanwhile): make that
 * first call before any stream capture.  All calls share the array: calls whose
 * GPU work overlaps race and must be serialised. */
int vs_op_apply_device_noalloc(vs_op* op, const void* x, void* y, int64_t nrhs, int mode, int precision);

/* ---- 2-level circulant preconditioner ------------------------------- */

typedef struct vs_prec vs_prec;

/* Bit mask of the precisions a preconditioner is built for, and how the
 * FP32 (VS_BUILD_C64) blocks are inverted.  By default: one CTA per block in
 * shared memory up to 3N = 168; for 168 < 3N <= 256 a persistent blocked
 * Gauss-Jordan whose rank-32 trailing updates are tcgen05 3xTF32 MMAs (each
 * block L2-resident in one CTA); beyond that the same on the CUDA cores.
 * VS_BUILD_LU_TC forces the tensor-core kernel for any 3N <= 256,
 * VS_BUILD_LU_CUDA the CUDA-core kernels.  FP64 blocks are always inverted
 * on the CUDA cores. */
enum vs_prec_mask { VS_BUILD_C64 = 1, VS_BUILD_C128 = 2, VS_BUILD_LU_TC = 4, VS_BUILD_LU_CUDA = 8 };

/* circ_1_level (on_off = 'off') followed by circ_2_level on the device, FP64:
 * src/src_preconditioning/circ_1_level.m:1-93 and circ_2_level.m:1-155.
 *   toep: L*M*N*6 complex.  Outputs (any may be NULL):
 *   circL_out: circ_L_opToep, L*M*N*6;  circM_out: circ_M_opToep, L*M*N*6;
 *   blocks_out: the cell circ{i,j} as L*M blocks (block index i + L*j), each
 *   3N x 3N column-major. */
int vs_circ_levels(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, double* circL_out,
                   double* circM_out, double* blocks_out);

/* Face vector of the JVIE 2-level preconditioner from the relative
 * permittivity grid (scatteringHumanHead.m:157-177): the mean of eps_r over x
 * and then y in each z layer, face_2(k) = (t_k - 1) / t_k, and
 * face3 = [face_2; face_2; face_2] (3N complex) -- the d argument of
 * vs_prec_create with shift = Gram.  eps_r: L*M*N complex, column-major.
 * Host arithmetic. */
int vs_eps_layer_average(int64_t L, int64_t M, int64_t N, const double* eps_r, double* face3);

/* Preconditioner inv(shift*I - diag(d)*C_ij) for every (x,y) frequency of the
 * 2-level circulant approximation of op's Toeplitz tensor:
 * main_DDA.m:98-116 (shift = 1/alpha_LDR, d = dV) and
 * scatteringHumanHead.m:132-184 (shift = Gram, d = face3_2, a 3N vector).
 *   shift: 1 complex; d: nd complex with nd = 1 or 3N;
 *   precisions: VS_BUILD_C64 | VS_BUILD_C128 (inversions in FP32 / FP64).
 * Returns VS_ERR_ARG if a block is singular.  The preconditioner copies op's
 * unknown indices and does not reference op afterwards. */
int vs_prec_create(vs_op* op, const double* shift, const double* d, int64_t nd, int precisions, vs_prec** out);

/* Preconditioner from caller-supplied inverse blocks (the inv_blocks cell of
 * mvp_circ_2_level.m:2): L*M blocks (index i + L*j), each 3N x 3N column-major
 * complex; idx3: n3 0-based unknown indices into the (L,M,N,3) grid. */
int vs_prec_create_blocks(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* inv_blocks,
                          const int64_t* idx3, int64_t n3, int precisions, vs_prec** out);

/* Batched inversion of nmat complex n x n matrices in device memory, in place,
 * FP32 (float2), column-major or row-major alike: the parfor of inv() over the
 * preconditioner blocks at main_DDA.m:107-111 (main_koch.m:114-118), e.g. for
 * inverse blocks handed to vs_prec_create_blocks.  method: 0 (tensor-core
 * trailing updates for n <= 256, else the CUDA cores), VS_BUILD_LU_TC
 * (tensor cores, n <= 256), VS_BUILD_LU_CUDA (persistent blocked
 * Gauss-Jordan on the CUDA cores).  Enqueued on the
 * context's stream; returns after it completes, VS_ERR_ARG if a matrix is
 * singular or its inverse is not finite. */
int vs_invert_blocks_device(vs_ctx* ctx, void* mats, int64_t n, int64_t nmat, int method);

int vs_prec_destroy(vs_prec* prec);

/* y = M^-1 x (mvp_circ_2_level.m:1-23) for nrhs right-hand sides, host
 * buffers, complex double; precision VS_C64 or VS_C128 (must have been built). */
int vs_prec_apply(vs_prec* prec, const double* x, double* y, int64_t nrhs, int precision);

/* Same on device buffers of the precision's type, enqueued, no synchronisation. */
int vs_prec_apply_device(vs_prec* prec, const void* x, void* y, int64_t nrhs, int precision);

/* Copy out the inverse blocks of one precision as complex double, in the
 * layout of vs_prec_create_blocks. */
int vs_prec_get_blocks(vs_prec* prec, int precision, double* out);

/* ---- Krylov solve ---------------------------------------------------- */

/* VS_BICGSTAB: MATLAB bicgstab(A, b, tol, maxit, M1) (right preconditioned);
 * VS_GMRES: MATLAB gmres(A, b, restart, tol, maxit, M1) (left preconditioned,
 * restarted); VS_GMRES_DR: the reference's pgmresDR(A, b, restart, tol,
 * maxit, ritz, [], [], M) (src/src_numeric/src_iterative/pgmresDR.m:73,
 * called by JVIE_Solver_const_GPU.m:400-447): GCRO-DR, right preconditioned,
 * each restart recycling the `ritz` harmonic Ritz vectors of smallest
 * magnitude.  Each is the inner solver of the FP64 refinement loop. */
enum vs_solve_method { VS_BICGSTAB = 0, VS_GMRES = 1, VS_GMRES_DR = 2 };
enum vs_solve_precision {
  VS_SOLVE_MIXED = 0, /* c64 inner solve on the c64 pipeline inside FP64 iterative refinement */
  VS_SOLVE_FP64 = 1   /* the same Krylov method on the c128 pipeline throughout               */
};

typedef struct vs_solve_opts {
  int method;          /* VS_BICGSTAB                                                        */
  int precision;       /* VS_SOLVE_MIXED or VS_SOLVE_FP64                                    */
  double tol;          /* stop when ||b - A x|| <= tol ||b|| (FP64 true residual for MIXED)  */
  int maxit;           /* maximum (inner) iterations in total                                */
  double inner_tol;    /* MIXED: relative tolerance of each inner solve, 0 = automatic       */
  int max_refine;      /* MIXED: maximum refinement steps                                    */
  int iters_per_graph; /* iterations captured per CUDA graph launch (host polls in between)  */
  double* resvec;      /* optional: relative residual norms at every half step               */
  int64_t resvec_cap;  /* capacity of resvec                                                 */
  int transpose;       /* 0: solve A x = b; 1: solve A^T x = b (plain transpose, adjoints)   */
  int restart;         /* VS_GMRES: restart length (Krylov basis size); VS_GMRES_DR: 2..256   */
  int ritz;            /* VS_GMRES_DR: recycled harmonic Ritz vectors, 1..restart-1           */
  /* Gram of each right-hand side in place of the operator's, as the drivers
   * pass Gram to every MVP call: NULL = the operator's; else nrhs * gram_n
   * complex, gram_n = 1 (one value per right-hand side) or L*M*N (a
   * column-major grid per right-hand side).  DDA: Gram = 1/alpha_LDR of each
   * incident direction and polarisation (getOPERATOR_DDA.m:14-26 with the
   * kvec, Eo of main_DDA.m:61-62).  A preconditioner passed with it stays the
   * one it was built for (it only changes the convergence, not the solution). */
  const double* gram;
  int64_t gram_n;
  /* Optional, VS_BICGSTAB: 16 floats that receive durations inside this solve
   * (ms), from CUDA events recorded between the launches of the captured
   * iterations (graph launches after which every right-hand side was still
   * iterating): [0..4] the preconditioner's five passes, [5..9] the matvec's
   * five passes, each averaged over its launches; [10] the solver's own
   * kernels per iteration; [11] iterations averaged; [12] the FP64 residuals
   * b - A x, average per call; [13] their calls; [14..15] 0.  The
   * instrumented iteration graph replaces the plain one (later plain solves
   * capture it again), and its event nodes add a little time: time solves
   * without it.  NULL: no profile. */
  float* profile_ms;
  /* VS_BICGSTAB: 0 (default) folds the vector steps of an iteration into the
   * x passes (p and s formed in the preconditioner's forward x pass, the
   * inner products of v and t added in the matvec's inverse x pass, one-CTA
   * kernels for alpha, ||s|| and omega) wherever both x passes run the
   * two-level kernels; 1 keeps them as separate kernels.  The two agree to
   * the rounding of the inner products' summation order. */
  int unfused;
} vs_solve_opts;

typedef struct vs_solve_info {
  int flag;        /* 0 converged, 1 maxit reached, 4 breakdown, 5 non-finite (MATLAB flags) */
  double relres;   /* final ||b - A x|| / ||b||, computed in FP64 on the c128 pipeline       */
  double iter;     /* iterations (BiCGSTAB counts half steps as 0.5); inner total for MIXED  */
  int refinements; /* MIXED: refinement steps taken                                          */
  int64_t n_resvec;
  double time_ms;  /* wall time of the call                                                  */
  int64_t kernel_launches; /* kernels this call launched (each node of a graph launch counts) */
} vs_solve_info;

/* Fill opts with defaults: BiCGSTAB, MIXED, tol 1e-6, maxit 2000, automatic
 * inner tolerance, 10 refinements, 4 iterations per graph, no resvec, no
 * transpose, GMRES restart 50, 10 recycled vectors for GMRES-DR, the
 * operator's Gram, no profile, folded vector steps. */
void vs_solve_opts_default(vs_solve_opts* opts);

/* Solve A x = b with the (optional, may be NULL) preconditioner, right
 * preconditioned as MATLAB's bicgstab(A, b, tol, maxit, M1) at
 * main_DDA.m:82,120-121.  b: n3 complex (host); x: in = initial guess,
 * out = solution.  Non-convergence is not an error: it is reported in
 * info->flag, as MATLAB does. */
int vs_solve(vs_op* op, vs_prec* prec, const double* b, double* x, const vs_solve_opts* opts, vs_solve_info* info);

/* Same with b and x in device memory (double2, n3 each). */
int vs_solve_device(vs_op* op, vs_prec* prec, const void* b, void* x, const vs_solve_opts* opts, vs_solve_info* info);

/* nrhs right-hand sides of the same operator (incident directions and
 * polarisations of one particle), stored one after another (n3 each); infos
 * has nrhs entries and opts->resvec, if given, holds resvec_cap entries per
 * right-hand side.  BiCGSTAB solves the batch together: every pipeline launch
 * serves all right-hand sides (the Green spectrum and the preconditioner
 * blocks are read once per launch), each right-hand side keeping its own
 * scalars and convergence test.  GMRES solves them one after another. */
int vs_solve_batch(vs_op* op, vs_prec* prec, const double* b, double* x, int64_t nrhs, const vs_solve_opts* opts,
                   vs_solve_info* infos);
int vs_solve_batch_device(vs_op* op, vs_prec* prec, const void* b, void* x, int64_t nrhs, const vs_solve_opts* opts,
                          vs_solve_info* infos);

/* Several particles at once (the reference solves its particles, incident
 * directions and polarisations in a loop of bicgstab calls, main_DDA.m:61-82):
 * nparticles operators, each with its own preconditioner (precs may be NULL,
 * or hold NULL entries), right-hand sides b[i] and solutions x[i] (device,
 * double2, nrhs[i] * n3 each, as vs_solve_batch_device).  Operators created on
 * different contexts are solved concurrently, one host thread per context,
 * each on its context's stream; operators that share a context run one after
 * another.  infos holds sum(nrhs) entries, particle by particle.  Returns the
 * first failing particle's status (its message in vs_last_error(NULL) and in
 * its context); the other particles still run.  A preconditioner shared by
 * particles on different contexts is rejected (VS_ERR_ARG) before any work. */
int vs_solve_particles_device(int64_t nparticles, vs_op* const* ops, vs_prec* const* precs, const void* const* b,
                              void* const* x, const int64_t* nrhs, const vs_solve_opts* opts, vs_solve_info* infos);

/* Several particles solved in lockstep on one context (the loop of bicgstab
 * calls over particles, incident directions and polarisations of
 * main_DDA.m:61-82): every inner BiCGSTAB iteration of all particles is one
 * CUDA graph launch whose branches -- one per particle, with its own operator,
 * preconditioner and per-rhs Gram -- the GPU runs concurrently; the FP64
 * refinement steps of all particles run together.  ops: distinct operators,
 * all on one context; precs: NULL or distinct preconditioners (or NULL
 * entries); b[i], x[i]: device double2, nrhs[i] * n3 each (x starts from 0);
 * gram: NULL or per particle NULL / nrhs[i] * gram_n[i] complex (host), the
 * Gram of each right-hand side as in vs_solve_opts.gram.  opts: BiCGSTAB,
 * MIXED or FP64; opts->gram and opts->resvec must be NULL.  infos: sum(nrhs)
 * entries, particle by particle. */
int vs_solve_particles(int64_t nparticles, vs_op* const* ops, vs_prec* const* precs, const void* const* b,
                       void* const* x, const int64_t* nrhs, const double* const* gram, const int64_t* gram_n,
                       const vs_solve_opts* opts, vs_solve_info* infos);

/* ---- excitation, extinction cross section, gradient ------------------- */

/* Plane wave E0 .* exp(1i k.r) at op's unknowns: PlaneWavePointWise.m:7-19
 * followed by the Einc(idx3) gather of main_DDA.m:81, FP64 on the device.
 *   x[L], y[M], z[N]: voxel-centre coordinates (grid3d.m:41-61); E0: 3
 *   complex.  b_out: n3 complex (host). */
int vs_plane_wave(vs_op* op, const double* x, const double* y, const double* z, const double kvec[3],
                  const double* E0, double* b_out);

/* Extinction cross section of a DDA solution P (n3 complex, the reference's
 * dipole moment per volume) under the incident field Einc at the same
 * unknowns: C_ext = 4 pi ko dV / |E0|^2 sum Im(conj(Einc) P) (Draine &
 * Flatau 1994, eq. 8).  Absent from the reference (README.md:35). */
int vs_cext(vs_op* op, const double* P, const double* Einc, double ko, double dV, double e0norm2, double* cext);

/* Whole-domain apply over every entry of the (L,M,N,3) grid (column-major,
 * 3*L*M*N complex per right-hand side, zeros where there is no material):
 *   y = a x + b crop(G * x),   a, b complex scalars,
 * with op's operator spectrum.  Replaces the MVP_eval handle of
 * main_DDA.m:142-145 (MVP over idxAll with Mr = 1, Mc = dV, Gram = 1/alpha:
 * a = 1/alpha, b = -dV) and mv_L_const.m:1-80 as called by
 * E_field_Nop_const.m:76-84 (JOut = crop(fN * J) - Gram J: a = -Gram, b = 1).
 * Host buffers, complex double; precision VS_C64 or VS_C128. */
int vs_op_apply_domain(vs_op* op, const double* x_grid, double* y_grid, int64_t nrhs, const double a[2],
                       const double b[2], int precision);

/* Total field on the whole grid after a DDA solve (main_DDA.m:136-148):
 *   Pout = P on op's unknowns, 0 elsewhere;  E = Einc - (Pout/alpha - dV crop(G * Pout)) + Pout/chi.
 *   P: n3 per right-hand side; Einc_grid, E_grid: 3*L*M*N per right-hand side
 *   (the incident field on the whole grid, PlaneWavePointWise.m over r);
 *   alpha, chi: complex scalars (alpha_LDR and (m^2-1)/(4 pi) of main_DDA.m:139). */
int vs_field_dda(vs_op* op, const double* P, const double* Einc_grid, int64_t nrhs, const double alpha[2],
                 double dV, const double chi[2], double* E_grid, int precision);

/* Far-field amplitude of the dipoles p_j = dV P_j in ndir unit directions n:
 *   F(n) = ko^2 dV (I - n n^T) sum_j P_j exp(-i ko n . r_j),   E_sca -> exp(i ko r)/r F(n)
 * (far zone of the DDA Green tensor of getOPERATOR_DDA.m:99-113; Draine &
 * Flatau 1994).  The reference has no far-field routine (README.md:35).  With
 * F(k_inc) the optical theorem gives C_ext = 4 pi / ko Im(conj(E0) . F) / |E0|^2.
 *   P: n3 per right-hand side; x, y, z: the grid axes (as vs_plane_wave);
 *   dirs: ndir x 3 unit vectors; F: nrhs x ndir x 3 complex.  FP64. */
int vs_far_field(vs_op* op, const double* P, int64_t nrhs, const double* x, const double* y, const double* z,
                 double ko, double dV, const double* dirs, int64_t ndir, double* F);

/* C_ext and its gradient with respect to each voxel's permittivity by the
 * adjoint method: solves A P = Einc and A^T lam = conj(Einc) with opts (the
 * operator must carry Gram = 1/alpha_LDR(eps) per voxel and Mc = dV, the DDA
 * system of main_DDA.m:75), then dC/d eps_j = -c Im/Re(d(1/alpha)/d eps_j *
 * sum_comp lam_j P_j).  eps: one complex per voxel in idx order (n3/3);
 * grad_re/grad_im: dC/dRe(eps_j), dC/dIm(eps_j); P_out optional (n3).
 * Requires idx3 in the [idx; V+idx; 2V+idx] form. */
int vs_cext_grad(vs_op* op, vs_prec* prec, const double* Einc, const double* eps, double ko, double d,
                 const double kvec[3], const double E0[3], const vs_solve_opts* opts, double* cext, double* grad_re,
                 double* grad_im, double* P_out, vs_solve_info* info_fwd, vs_solve_info* info_adj);

/* Orientation-averaged extinction cross section (random-orientation averaging,
 * listed as a to-do at README.md:37).  The particle stays fixed on op's grid
 * and the incident plane wave takes ndir orientations: a unit direction k
 * (dirs, ndir x 3) and an angle psi (NULL: 0) turning the polarisation pair
 * b1 = k x z / |k x z| (k x x when k is along z), b2 = k x b1 about k, giving
 * e1 = cos(psi) b1 + sin(psi) b2 and e2 = k x e1 -- the three Euler angles of
 * a particle orientation (rotating the particle is rotating the incident wave
 * the other way).  Every (orientation, polarisation) is solved with its own
 * LDR polarisability (Gram = 1/alpha_LDR(m, k, e), getOPERATOR_DDA.m:7-26)
 * on op's Toeplitz operator, 8 orientations per batched solve; C_ext (vs_cext,
 * |E0| = 1) is averaged over the two polarisations (unpolarised incidence)
 * and then over the orientations with the weights (NULL: equal weights;
 * normalised by their sum).  The LDR polarisability depends on the
 * polarisation, so the two-polarisation average depends on psi: a random
 * orientation average samples psi as well as k.
 *   op: the DDA operator (Mr = 1, Mc = dV; idx3 in the [idx; V+idx; 2V+idx]
 *   form); m: refractive index, 1 value or n3/3 in idx order; x, y, z: grid
 *   axes (as vs_plane_wave); ko, d: wavenumber and dipole spacing; opts: the
 *   solver (opts->gram NULL, no transpose).  Outputs: cext_avg; cext_each
 *   (optional, ndir x 2: per orientation and polarisation); infos (optional,
 *   ndir x 2). */
int vs_orientation_average(vs_op* op, vs_prec* prec, const double* m, int64_t nm, const double* x, const double* y,
                           const double* z, double ko, double d, const double* dirs, const double* psi,
                           const double* weights, int64_t ndir, const vs_solve_opts* opts, double* cext_avg,
                           double* cext_each, vs_solve_info* infos);

/* ---- diagnostics ----------------------------------------------------- */

/* Launch shape of an operator's pipeline in one precision, as chosen by the
 * autotuner at creation (log2 values, -1 = built-in default).  Setting it pins
 * the shape, e.g. for reproducible timings. */
typedef struct vs_shape {
  int lg_lines_x;  /* x passes: log2 lines per CTA                                 */
  int lg_tile_y;   /* y passes: log2 x-tile width                                  */
  int lg_tile_z;   /* z pass (shared-memory kernel): log2 x-tile width             */
  int z_reg;       /* z pass: 0 shared-memory Stockham, 1 two-level registers,
                      2 two-level with a register cap for occupancy          */
  int y_reg;       /* y passes: 0 shared-memory Stockham, 1 two-level registers,
                      2 (VS_C128 only) two-level in double-float arithmetic,
                      where the length has that kernel (else as 1)        */
  int x_reg;       /* x passes: as y_reg                                    */
  int z_df;        /* VS_C128 only: 1 runs the two-level z pass in double-float
                      arithmetic (pairs of floats, about 48 bits) on the FP64
                      data; 0 / -1 FP64 arithmetic                            */
} vs_shape;
int vs_op_get_shape(const vs_op* op, int precision, vs_shape* shape);
int vs_op_set_shape(vs_op* op, int precision, const vs_shape* shape);

/* Launch shape of a preconditioner apply: x/y tiles of its FFT passes and
 * the block GEMV.  gemv_mode 0 is the register-direct GEMV (gemv_blocks
 * stored blocks per CTA, gemv_threads per CTA); gemv_mode 1 streams each block
 * through shared memory with bulk asynchronous copies (gemv_blocks CTAs per SM, 1-4,
 * gemv_chunk block columns per copy); gemv_mode 2 streams the packed lower
 * triangles of the symmetric blocks S = B D (D negating the x and y
 * components; built by vs_prec_create when the operator has exact parity and
 * d is one scalar, VS_ERR_UNSUPPORTED otherwise), one whole block per copy
 * (gemv_blocks CTAs per SM, gemv_chunk = ring depth 2-8).  0 / -1 select the
 * defaults. */
typedef struct vs_prec_shape {
  int lg_lines_x;
  int lg_tile_y;
  int gemv_blocks;
  int gemv_threads;
  int gemv_mode;
  int gemv_chunk;
  int y_reg;       /* y passes: 0 shared-memory Stockham, 1 two-level registers */
  int x_reg;       /* x passes: 0 shared-memory Stockham, 1 two-level registers */
  int fuse_xy;     /* 1: both FFTs of each (z, component) plane in one CTA when the
                      plane fits in shared memory; 0 / -1: separate x and y passes */
  int wait_polls;  /* streamed GEMV (gemv_mode 1, 2): polls before a wait on another
                      warp role gives up (0 = 2^20; -1 = none, every such wait
                      gives up at once, for exercising the failure path).  A
                      wait that runs out ends the CTA's work and the apply fails
                      with VS_ERR_TIMEOUT; the wait for the CTA's own copies
                      still in flight always keeps the full bound. */
} vs_prec_shape;
int vs_prec_get_shape(const vs_prec* prec, int precision, vs_prec_shape* shape);
int vs_prec_set_shape(vs_prec* prec, int precision, const vs_prec_shape* shape);

/* Time each of the 5 launches of one apply (matvec: X-forward gather, Y
 * forward, Z FFT x tensor x inverse, Y inverse, X inverse + diagonal; the
 * preconditioner: X-forward gather, Y forward, block GEMV, Y inverse, X
 * inverse) with CUDA events on the context's stream, averaged over nrep
 * back-to-back applies of nrhs right-hand sides.  ms_out receives 5 floats
 * (milliseconds per launch).  Device buffers x, y of the precision's type. */
int vs_op_time_passes(vs_op* op, const void* x, void* y, int64_t nrhs, int precision, int nrep, float* ms_out);
int vs_prec_time_passes(vs_prec* prec, const void* x, void* y, int64_t nrhs, int precision, int nrep, float* ms_out);

#ifdef __cplusplus
}
#endif

#endif /* VOXSCATTER_H */
