/*
 * voxscatter_mex.c -- MATLAB MEX gateway onto libvoxscatter (include/voxscatter.h).
 *
 * Build (MATLAB R2018a or later, interleaved complex API):
 *   mex -R2018a -I<repo>/include voxscatter_mex.c -L<repo>/voxscatter_gb300 -lvoxscatter
 *
 * The reference's drivers build function handles around MVP / mv_AN_const
 * (src/src_vie/src_mvp/MVP.m:1), mvp_circ_2_level
 * (src/src_preconditioning/mvp_circ_2_level.m:2) and the Krylov calls
 * (main_DDA.m:82-129, pgmresDR.m:73); the .m shims beside this file keep those
 * signatures and call this gateway.  One command per call:
 *
 *   op   = voxscatter_mex('op_create', Toep, Mr, Mc, Gram, idx3)            vs_op_create
 *   op   = voxscatter_mex('op_create_fN', fN, L, M, N, Mr, Mc, Gram, idx3)  vs_op_create_fN
 *   y    = voxscatter_mex('op_apply', op, x, mode, precision)              vs_op_apply
 *   y    = voxscatter_mex('op_apply_gram', op, x, gram, mode, precision)   vs_op_apply_gram
 *          voxscatter_mex('op_destroy', op)
 *   pr   = voxscatter_mex('prec_create', op, shift, d, precisions)         vs_prec_create
 *   pr   = voxscatter_mex('prec_create_blocks', inv_blocks, L, M, N, idx3) vs_prec_create_blocks
 *   y    = voxscatter_mex('prec_apply', pr, x, precision)                  vs_prec_apply
 *          voxscatter_mex('prec_destroy', pr)
 *   [x, flag, relres, iter, resvec] = voxscatter_mex('solve', op, pr, b, x0, opts)          vs_solve(_batch)
 *   E    = voxscatter_mex('field_dda', op, P, Einc, alpha, dV, chi, precision)              vs_field_dda
 *   [cext, g_re, g_im, P] = voxscatter_mex('cext_grad', op, pr, Einc, eps, ko, d, kvec, E0, opts)
 *   [cavg, ceach] = voxscatter_mex('orientation_average', op, pr, m, x, y, z, ko, d, dirs, psi, w, opts)
 *
 * Arguments: idx3 is MATLAB's 1-based index vector (converted to 0-based
 * here); x, b are n3 x nrhs complex; mode is 'notransp', 'transp' (the
 * reference's conjugate transpose) or 'plain_transp'; precision 'c64' or
 * 'c128'; pr may be [] (no preconditioner); opts is a struct whose fields
 * (all optional) are method ('bicgstab' | 'gmres' | 'gmresdr'), precision
 * ('mixed' | 'fp64'), tol, maxit, restart, ritz, inner_tol, max_refine,
 * transpose, gram.  Handles are uint64 scalars; the gateway keeps a table of
 * the live ones and rejects any other value.  Library failures are raised
 * as MATLAB errors with the library's message; non-convergence is the flag
 * output, as in MATLAB.  Every handle and the context are released when the
 * MEX file is cleared.
 */
#include <stdint.h>
#include <string.h>

#include "mex.h"
#include "voxscatter.h"

#define VS_MAX_HANDLES 4096

static vs_ctx* g_ctx = NULL;
static void* g_handles[VS_MAX_HANDLES];
static int g_kinds[VS_MAX_HANDLES]; /* 1 operator, 2 preconditioner */

static void release_all(void) {
  int i;
  for (i = 0; i < VS_MAX_HANDLES; ++i) {
    if (g_kinds[i] == 1) vs_op_destroy((vs_op*)g_handles[i]);
    if (g_kinds[i] == 2) vs_prec_destroy((vs_prec*)g_handles[i]);
    g_handles[i] = NULL;
    g_kinds[i] = 0;
  }
  if (g_ctx) vs_ctx_destroy(g_ctx);
  g_ctx = NULL;
}

static void check(int status) {
  if (status != VS_OK) mexErrMsgIdAndTxt("voxscatter:library", "libvoxscatter status %d: %s", status,
                                         vs_last_error(g_ctx));
}

static void fail(const char* what) { mexErrMsgIdAndTxt("voxscatter:argument", "%s", what); }

static mxArray* new_handle(void* p, int kind) {
  int i;
  for (i = 0; i < VS_MAX_HANDLES; ++i)
    if (g_kinds[i] == 0) {
      mxArray* h = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
      g_handles[i] = p;
      g_kinds[i] = kind;
      *(uint64_t*)mxGetData(h) = (uint64_t)(uintptr_t)p;
      return h;
    }
  fail("too many live voxscatter handles");
  return NULL;
}

/* the live handle of this kind held by a, or NULL for [] when optional */
static void* get_handle(const mxArray* a, int kind, int optional, int* slot) {
  uint64_t v;
  int i;
  if (optional && mxGetNumberOfElements(a) == 0) return NULL;
  if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1) fail("expected a voxscatter handle (uint64 scalar)");
  v = *(uint64_t*)mxGetData(a);
  for (i = 0; i < VS_MAX_HANDLES; ++i)
    if (g_kinds[i] == kind && (uint64_t)(uintptr_t)g_handles[i] == v) {
      if (slot) *slot = i;
      return g_handles[i];
    }
  fail("not a live voxscatter handle of the expected kind");
  return NULL;
}

/* interleaved complex data of a double array (real arrays are rejected:
 * pass complex(x) so no conversion copy is hidden here) */
static double* cplx(const mxArray* a, const char* name) {
  if (!mxIsDouble(a) || !mxIsComplex(a)) {
    static char msg[128];
    strncpy(msg, name, 64);
    msg[64] = 0;
    strcat(msg, " must be a complex double array");
    fail(msg);
  }
  return (double*)mxGetComplexDoubles(a);
}

static vs_diag diag_arg(const mxArray* a, const char* name) {
  vs_diag d;
  d.v = cplx(a, name);
  d.n = (int64_t)mxGetNumberOfElements(a);
  return d;
}

/* 1-based double index vector -> 0-based int64 (mxMalloc'd) */
static int64_t* idx_arg(const mxArray* a, int64_t* n) {
  const double* v;
  int64_t* out;
  int64_t e;
  if (!mxIsDouble(a) || mxIsComplex(a)) fail("idx3 must be a real double vector of 1-based indices");
  *n = (int64_t)mxGetNumberOfElements(a);
  v = mxGetDoubles(a);
  out = (int64_t*)mxMalloc((size_t)(*n > 0 ? *n : 1) * sizeof(int64_t));
  for (e = 0; e < *n; ++e) out[e] = (int64_t)v[e] - 1;
  return out;
}

static int mode_arg(const mxArray* a) {
  char s[16];
  if (mxGetString(a, s, sizeof s)) fail("mode must be 'notransp', 'transp' or 'plain_transp'");
  if (!strcmp(s, "notransp")) return VS_NOTRANSP;
  if (!strcmp(s, "transp")) return VS_CONJTRANSP;
  if (!strcmp(s, "plain_transp")) return VS_TRANSP;
  fail("mode must be 'notransp', 'transp' or 'plain_transp'");
  return 0;
}

static int precision_arg(const mxArray* a) {
  char s[8];
  if (mxGetString(a, s, sizeof s)) fail("precision must be 'c64' or 'c128'");
  if (!strcmp(s, "c64")) return VS_C64;
  if (!strcmp(s, "c128")) return VS_C128;
  fail("precision must be 'c64' or 'c128'");
  return 0;
}

static double field_or(const mxArray* s, const char* f, double dflt) {
  const mxArray* v = mxGetField(s, 0, f);
  return (v && mxGetNumberOfElements(v) > 0) ? mxGetScalar(v) : dflt;
}

/* vs_solve_opts from a struct (fields optional); gram, if given, must stay
 * alive while the options are used */
static void opts_arg(const mxArray* s, vs_solve_opts* o, int64_t V) {
  const mxArray* f;
  char buf[16];
  vs_solve_opts_default(o);
  if (!s || mxGetNumberOfElements(s) == 0) return;
  if (!mxIsStruct(s)) fail("opts must be a struct");
  if ((f = mxGetField(s, 0, "method")) != NULL && !mxGetString(f, buf, sizeof buf)) {
    if (!strcmp(buf, "bicgstab")) o->method = VS_BICGSTAB;
    else if (!strcmp(buf, "gmres")) o->method = VS_GMRES;
    else if (!strcmp(buf, "gmresdr")) o->method = VS_GMRES_DR;
    else fail("opts.method must be 'bicgstab', 'gmres' or 'gmresdr'");
  }
  if ((f = mxGetField(s, 0, "precision")) != NULL && !mxGetString(f, buf, sizeof buf))
    o->precision = strcmp(buf, "fp64") ? VS_SOLVE_MIXED : VS_SOLVE_FP64;
  o->tol = field_or(s, "tol", o->tol);
  o->maxit = (int)field_or(s, "maxit", o->maxit);
  o->restart = (int)field_or(s, "restart", o->restart);
  o->ritz = (int)field_or(s, "ritz", o->ritz);
  o->inner_tol = field_or(s, "inner_tol", o->inner_tol);
  o->max_refine = (int)field_or(s, "max_refine", o->max_refine);
  o->transpose = (int)field_or(s, "transpose", o->transpose);
  if ((f = mxGetField(s, 0, "gram")) != NULL && mxGetNumberOfElements(f) > 0) {
    o->gram = cplx(f, "opts.gram");
    o->gram_n = (mxGetM(f) == (size_t)V) ? V : 1;
  }
}

static int is(const char* cmd, const char* name) { return !strcmp(cmd, name); }

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  char cmd[32];
  if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof cmd)) fail("first argument: a command string");
  if (!g_ctx) {
    check(vs_ctx_create(0, &g_ctx));
    mexAtExit(release_all);
  }
  (void)nlhs;

  if (is(cmd, "op_create")) { /* op = ('op_create', Toep, Mr, Mc, Gram, idx3) */
    const mwSize* d;
    int64_t n3, *idx;
    vs_op* op;
    if (nrhs != 6) fail("op_create: Toep, Mr, Mc, Gram, idx3");
    if (mxGetNumberOfDimensions(prhs[1]) != 4) fail("Toep must be L x M x N x 6");
    d = mxGetDimensions(prhs[1]);
    idx = idx_arg(prhs[5], &n3);
    check(vs_op_create(g_ctx, (int64_t)d[0], (int64_t)d[1], (int64_t)d[2], cplx(prhs[1], "Toep"), 0, 0, 0, idx, n3,
                       diag_arg(prhs[2], "Mr"), diag_arg(prhs[3], "Mc"), diag_arg(prhs[4], "Gram"), &op));
    mxFree(idx);
    plhs[0] = new_handle(op, 1);
  } else if (is(cmd, "op_create_fN")) { /* op = ('op_create_fN', fN, L, M, N, Mr, Mc, Gram, idx3) */
    const mwSize* d;
    int64_t n3, *idx;
    vs_op* op;
    if (nrhs != 9) fail("op_create_fN: fN, L, M, N, Mr, Mc, Gram, idx3");
    if (mxGetNumberOfDimensions(prhs[1]) != 4) fail("fN must be P x Q x R x 6");
    d = mxGetDimensions(prhs[1]);
    idx = idx_arg(prhs[8], &n3);
    check(vs_op_create_fN(g_ctx, (int64_t)mxGetScalar(prhs[2]), (int64_t)mxGetScalar(prhs[3]),
                          (int64_t)mxGetScalar(prhs[4]), cplx(prhs[1], "fN"), (int64_t)d[0], (int64_t)d[1],
                          (int64_t)d[2], idx, n3, diag_arg(prhs[5], "Mr"), diag_arg(prhs[6], "Mc"),
                          diag_arg(prhs[7], "Gram"), &op));
    mxFree(idx);
    plhs[0] = new_handle(op, 1);
  } else if (is(cmd, "op_apply") || is(cmd, "op_apply_gram")) {
    /* y = ('op_apply', op, x, mode, precision) / ('op_apply_gram', op, x, gram, mode, precision) */
    const int g = is(cmd, "op_apply_gram");
    vs_op* op;
    int64_t n3, L3[3];
    size_t cols;
    if (nrhs != (g ? 6 : 5)) fail(g ? "op_apply_gram: op, x, gram, mode, precision" : "op_apply: op, x, mode, precision");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    check(vs_op_info(op, L3, NULL, &n3));
    if (mxGetM(prhs[2]) != (size_t)n3) fail("x must have n3 rows");
    cols = mxGetN(prhs[2]);
    plhs[0] = mxCreateDoubleMatrix((mwSize)n3, (mwSize)cols, mxCOMPLEX);
    if (g) {
      const int64_t V = L3[0] * L3[1] * L3[2];
      const int64_t gn = (mxGetNumberOfElements(prhs[3]) == cols) ? 1 : V;
      if (mxGetNumberOfElements(prhs[3]) != (size_t)(gn * (int64_t)cols)) fail("gram: nrhs values or L*M*N x nrhs");
      check(vs_op_apply_gram(op, cplx(prhs[2], "x"), (double*)mxGetComplexDoubles(plhs[0]), (int64_t)cols,
                             mode_arg(prhs[4]), precision_arg(prhs[5]), cplx(prhs[3], "gram"), gn));
    } else {
      check(vs_op_apply(op, cplx(prhs[2], "x"), (double*)mxGetComplexDoubles(plhs[0]), (int64_t)cols,
                        mode_arg(prhs[3]), precision_arg(prhs[4])));
    }
  } else if (is(cmd, "op_destroy") || is(cmd, "prec_destroy")) {
    const int kind = is(cmd, "op_destroy") ? 1 : 2;
    int slot = -1;
    void* h;
    if (nrhs != 2) fail("destroy: one handle");
    h = get_handle(prhs[1], kind, 0, &slot);
    check(kind == 1 ? vs_op_destroy((vs_op*)h) : vs_prec_destroy((vs_prec*)h));
    g_handles[slot] = NULL;
    g_kinds[slot] = 0;
  } else if (is(cmd, "prec_create")) { /* pr = ('prec_create', op, shift, d, precisions) */
    vs_op* op;
    vs_prec* pr;
    char pm[16] = "both";
    int mask = VS_BUILD_C64 | VS_BUILD_C128;
    if (nrhs < 4 || nrhs > 5) fail("prec_create: op, shift, d[, 'c64'|'c128'|'both']");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    if (nrhs == 5 && !mxGetString(prhs[4], pm, sizeof pm)) {
      if (!strcmp(pm, "c64")) mask = VS_BUILD_C64;
      else if (!strcmp(pm, "c128")) mask = VS_BUILD_C128;
    }
    check(vs_prec_create(op, cplx(prhs[2], "shift"), cplx(prhs[3], "d"), (int64_t)mxGetNumberOfElements(prhs[3]),
                         mask, &pr));
    plhs[0] = new_handle(pr, 2);
  } else if (is(cmd, "prec_create_blocks")) {
    /* pr = ('prec_create_blocks', inv_blocks, L, M, N, idx3); inv_blocks: 3N x 3N x L x M
       (cat(4, ...) of the reference's cell, block (i, j) at (:, :, i, j)) */
    int64_t L, M, N, n3, *idx;
    vs_prec* pr;
    if (nrhs != 6) fail("prec_create_blocks: inv_blocks, L, M, N, idx3");
    L = (int64_t)mxGetScalar(prhs[2]);
    M = (int64_t)mxGetScalar(prhs[3]);
    N = (int64_t)mxGetScalar(prhs[4]);
    if (mxGetNumberOfElements(prhs[1]) != (size_t)(9 * N * N * L * M)) fail("inv_blocks must be 3N x 3N x L x M");
    idx = idx_arg(prhs[5], &n3);
    check(vs_prec_create_blocks(g_ctx, L, M, N, cplx(prhs[1], "inv_blocks"), idx, n3, VS_BUILD_C64 | VS_BUILD_C128,
                                &pr));
    mxFree(idx);
    plhs[0] = new_handle(pr, 2);
  } else if (is(cmd, "prec_apply")) { /* y = ('prec_apply', pr, x, precision) */
    vs_prec* pr;
    if (nrhs != 4) fail("prec_apply: pr, x, precision");
    pr = (vs_prec*)get_handle(prhs[1], 2, 0, NULL);
    plhs[0] = mxCreateDoubleMatrix(mxGetM(prhs[2]), mxGetN(prhs[2]), mxCOMPLEX);
    check(vs_prec_apply(pr, cplx(prhs[2], "x"), (double*)mxGetComplexDoubles(plhs[0]), (int64_t)mxGetN(prhs[2]),
                        precision_arg(prhs[3])));
  } else if (is(cmd, "solve")) {
    /* [x, flag, relres, iter, resvec] = ('solve', op, pr, b, x0, opts); b: n3 x nrhs */
    vs_op* op;
    vs_prec* pr;
    vs_solve_opts o;
    int64_t n3, L3[3], cols, r, cap;
    vs_solve_info* infos;
    double* x;
    double* rv = NULL;
    if (nrhs != 6) fail("solve: op, pr, b, x0, opts");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    pr = (vs_prec*)get_handle(prhs[2], 2, 1, NULL);
    check(vs_op_info(op, L3, NULL, &n3));
    if (mxGetM(prhs[3]) != (size_t)n3) fail("b must have n3 rows");
    cols = (int64_t)mxGetN(prhs[3]);
    opts_arg(prhs[5], &o, L3[0] * L3[1] * L3[2]);
    plhs[0] = mxCreateDoubleMatrix((mwSize)n3, (mwSize)cols, mxCOMPLEX);
    x = (double*)mxGetComplexDoubles(plhs[0]);
    if (mxGetNumberOfElements(prhs[4]) > 0) {
      if (mxGetNumberOfElements(prhs[4]) != (size_t)(n3 * cols)) fail("x0 must be n3 x nrhs or []");
      memcpy(x, cplx(prhs[4], "x0"), (size_t)(n3 * cols) * 2 * sizeof(double));
    } else {
      memset(x, 0, (size_t)(n3 * cols) * 2 * sizeof(double));
    }
    cap = 4 * (int64_t)o.maxit + 64;
    if (cols == 1) {
      rv = (double*)mxMalloc((size_t)cap * sizeof(double));
      o.resvec = rv;
      o.resvec_cap = cap;
    }
    infos = (vs_solve_info*)mxMalloc((size_t)cols * sizeof(vs_solve_info));
    if (cols == 1) check(vs_solve(op, pr, cplx(prhs[3], "b"), x, &o, infos));
    else check(vs_solve_batch(op, pr, cplx(prhs[3], "b"), x, cols, &o, infos));
    plhs[1] = mxCreateDoubleMatrix(1, (mwSize)cols, mxREAL);
    plhs[2] = mxCreateDoubleMatrix(1, (mwSize)cols, mxREAL);
    plhs[3] = mxCreateDoubleMatrix(1, (mwSize)cols, mxREAL);
    for (r = 0; r < cols; ++r) {
      mxGetDoubles(plhs[1])[r] = infos[r].flag;
      mxGetDoubles(plhs[2])[r] = infos[r].relres;
      mxGetDoubles(plhs[3])[r] = infos[r].iter;
    }
    if (rv) {
      plhs[4] = mxCreateDoubleMatrix((mwSize)infos[0].n_resvec, 1, mxREAL);
      memcpy(mxGetDoubles(plhs[4]), rv, (size_t)infos[0].n_resvec * sizeof(double));
      mxFree(rv);
    } else {
      plhs[4] = mxCreateDoubleMatrix(0, 1, mxREAL);
    }
    mxFree(infos);
  } else if (is(cmd, "field_dda")) {
    /* E = ('field_dda', op, P, Einc, alpha, dV, chi, precision); Einc on the whole grid (3LMN) */
    vs_op* op;
    if (nrhs != 8) fail("field_dda: op, P, Einc, alpha, dV, chi, precision");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    plhs[0] = mxCreateDoubleMatrix(mxGetNumberOfElements(prhs[3]), 1, mxCOMPLEX);
    check(vs_field_dda(op, cplx(prhs[2], "P"), cplx(prhs[3], "Einc"), 1, cplx(prhs[4], "alpha"),
                       mxGetScalar(prhs[5]), cplx(prhs[6], "chi"), (double*)mxGetComplexDoubles(plhs[0]),
                       precision_arg(prhs[7])));
  } else if (is(cmd, "cext_grad")) {
    /* [cext, g_re, g_im, P] = ('cext_grad', op, pr, Einc, eps, ko, d, kvec, E0, opts) */
    vs_op* op;
    vs_prec* pr;
    vs_solve_opts o;
    vs_solve_info fi, ai;
    int64_t n3, L3[3];
    double cext = 0;
    size_t nvox;
    if (nrhs != 10) fail("cext_grad: op, pr, Einc, eps, ko, d, kvec, E0, opts");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    pr = (vs_prec*)get_handle(prhs[2], 2, 1, NULL);
    check(vs_op_info(op, L3, NULL, &n3));
    if (mxGetNumberOfElements(prhs[7]) != 3 || mxGetNumberOfElements(prhs[8]) != 3) fail("kvec and E0: 3 values");
    opts_arg(prhs[9], &o, L3[0] * L3[1] * L3[2]);
    nvox = mxGetNumberOfElements(prhs[4]);
    plhs[1] = mxCreateDoubleMatrix((mwSize)nvox, 1, mxREAL);
    plhs[2] = mxCreateDoubleMatrix((mwSize)nvox, 1, mxREAL);
    plhs[3] = mxCreateDoubleMatrix((mwSize)n3, 1, mxCOMPLEX);
    check(vs_cext_grad(op, pr, cplx(prhs[3], "Einc"), cplx(prhs[4], "eps"), mxGetScalar(prhs[5]),
                       mxGetScalar(prhs[6]), mxGetDoubles(prhs[7]), mxGetDoubles(prhs[8]), &o, &cext,
                       mxGetDoubles(plhs[1]), mxGetDoubles(plhs[2]), (double*)mxGetComplexDoubles(plhs[3]), &fi,
                       &ai));
    plhs[0] = mxCreateDoubleScalar(cext);
  } else if (is(cmd, "orientation_average")) {
    /* [cavg, ceach] = ('orientation_average', op, pr, m, x, y, z, ko, d, dirs, psi, w, opts);
       dirs: ndir x 3 (row j = direction j), psi and w: ndir or [] */
    vs_op* op;
    vs_prec* pr;
    vs_solve_opts o;
    int64_t L3[3], ndir, j, q;
    double cavg = 0, *dirs;
    if (nrhs != 13) fail("orientation_average: op, pr, m, x, y, z, ko, d, dirs, psi, w, opts");
    op = (vs_op*)get_handle(prhs[1], 1, 0, NULL);
    pr = (vs_prec*)get_handle(prhs[2], 2, 1, NULL);
    check(vs_op_info(op, L3, NULL, NULL));
    opts_arg(prhs[12], &o, L3[0] * L3[1] * L3[2]);
    ndir = (int64_t)mxGetM(prhs[9]);
    if (mxGetN(prhs[9]) != 3) fail("dirs must be ndir x 3");
    dirs = (double*)mxMalloc((size_t)(3 * ndir) * sizeof(double)); /* column-major -> row per direction */
    for (j = 0; j < ndir; ++j)
      for (q = 0; q < 3; ++q) dirs[3 * j + q] = mxGetDoubles(prhs[9])[j + ndir * q];
    plhs[1] = mxCreateDoubleMatrix(2, (mwSize)ndir, mxREAL);
    check(vs_orientation_average(op, pr, cplx(prhs[3], "m"), (int64_t)mxGetNumberOfElements(prhs[3]),
                                 mxGetDoubles(prhs[4]), mxGetDoubles(prhs[5]), mxGetDoubles(prhs[6]),
                                 mxGetScalar(prhs[7]), mxGetScalar(prhs[8]), dirs,
                                 mxGetNumberOfElements(prhs[10]) ? mxGetDoubles(prhs[10]) : NULL,
                                 mxGetNumberOfElements(prhs[11]) ? mxGetDoubles(prhs[11]) : NULL, ndir, &o, &cavg,
                                 mxGetDoubles(plhs[1]), NULL));
    mxFree(dirs);
    plhs[0] = mxCreateDoubleScalar(cavg);
  } else {
    fail("unknown command");
  }
}
