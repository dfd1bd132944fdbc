// Device Krylov state and solver entry (vs_krylov.cu).
#pragma once
#include "vs_internal.h"

namespace vs {


// Scalars of one Krylov iteration, resident in device memory.
struct KState {
  double2 rho, rho_prev, alpha, omega, beta;
  float2 alpha32, omega32, beta32;  // float copies for the c64 kernels (written with the doubles)
  double tol_abs, res, res_scale;
  double best_res;  // smallest full-step residual so far (stagnation guard)
  double* partials;
  double* resvec;
  unsigned counter;
  int skip, flag, half_pending, iter2, maxit, nres, resvec_cap;
  int best_iter2;   // half-step count at best_res
  int stag_window;  // stop with flag 3 after this many iterations without a 1% improvement (0: off)
};

// Scalars of one GMRES cycle, resident in device memory.
struct GState {
  double tol_abs;    // stop when the preconditioned residual estimate |g_{k+1}| <= tol_abs
  double res;        // current estimate
  double res_scale;  // resvec entries are res * res_scale
  double* resvec;
  int k;             // Arnoldi steps done in this cycle
  int m;             // restart length
  int skip, flag, nres, resvec_cap;
};

// Durations inside a BiCGSTAB solve, from CUDA events recorded between the
// launches of its captured iterations (only graph launches after which every
// right-hand side was still iterating count), plus the FP64 residuals.
struct SolveProfile {
  double pass_ms[10] = {};  // preconditioner passes 0..4, matvec passes 0..4 (sum over iters)
  double vec_ms = 0;        // the solver's own kernels (sum over iters)
  int64_t iters = 0;        // iterations summed
  double resid_ms = 0;      // FP64 residuals b - A x (sum)
  int64_t resid_calls = 0;
};

struct SolveParams {
  SolveProfile* profile = nullptr;  // non-null: record the in-solve durations
  bool fold_steps = true;           // BiCGSTAB: fold the vector steps into the x passes where possible
  int mode = 0;  // 0 mixed, 1 fp64
  double tol = 1e-6;
  int maxit = 2000;
  double inner_tol = 0;  // 0: automatic
  double inner_floor = 1e-7;
  int max_refine = 10;
  int per_graph = 4;
  int resvec_cap = 0;
  double* resvec_host = nullptr;
  int op_mode = 0;  // VS_NOTRANSP: solve A x = b; VS_TRANSP: solve A^T x = b
  int restart = 50; // GMRES restart length
  int ritz = 10;     // GCRO-DR: recycled harmonic Ritz vectors
  // Gram of each right-hand side (host, nrhs x gram_n complex, gram_n = 1 or
  // L*M*N) in place of the operator's; nullptr: the operator's
  const double2* gram_host = nullptr;
  int64_t gram_n = 0;
};

struct SolveResult {
  int flag = 1;
  double relres = 0, iter = 0, inner_iters = 0;
  int refinements = 0;
  int64_t n_resvec = 0;
  int64_t launches = 0;  // kernels launched by the solve (graph nodes count per graph launch)
};

void solve_bicgstab(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                    cudaStream_t st);
void solve_bicgstab_batch(vs_op& op, vs_prec* pr, const double2* b, double2* x, int nrhs, const SolveParams& prm,
                          std::vector<SolveResult>& out, cudaStream_t st);
// One particle of a lockstep multi-particle BiCGSTAB solve (device b and x,
// nrhs * n3 each; gram: host Gram per rhs or nullptr).
struct PartJob {
  vs_op* op = nullptr;
  vs_prec* pr = nullptr;
  const double2* b = nullptr;
  double2* x = nullptr;
  int nrhs = 0;
  const double2* gram = nullptr;
  int64_t gram_n = 0;
  std::vector<SolveResult> out;
};
// All particles' operators on ctx (one stream), distinct operators and
// preconditioners; x starts from zero.
void solve_bicgstab_particles(vs_ctx* ctx, std::vector<PartJob>& jobs, const SolveParams& prm, cudaStream_t st);
void solve_gmres(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                 cudaStream_t st);
void solve_gmres_dr(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                    cudaStream_t st);

}  // namespace vs
