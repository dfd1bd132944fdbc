// C-ABI entry points (include/voxscatter.h).  Each entry validates its
// arguments, runs on the context's stream and converts exceptions into a
// status code plus a message readable through vs_last_error().
#include "vs_internal.h"
#include "vs_krylov.h"
#include <chrono>
#include <atomic>
#include <thread>
#include <complex>
#include <cstring>
#include <cmath>
#include <set>

namespace {

thread_local std::string g_last_error;

uint64_t next_object_id() {
  static std::atomic<uint64_t> counter{1};
  return counter.fetch_add(1);
}

template <typename F>
int guarded(vs_ctx* ctx, F&& f) {
  try {
    if (ctx) VS_CUDA(cudaSetDevice(ctx->device));
    f();
    return VS_OK;
  } catch (const vs::Error& e) {
    g_last_error = e.what();
    if (ctx) ctx->err = e.what();
    return e.status;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    if (ctx) ctx->err = e.what();
    return VS_ERR_CUDA;
  }
}

using cd = std::complex<double>;

// Host view of a vs_diag.
struct HostDiag {
  const cd* v;
  int64_t n;
  cd at(int64_t vox) const { return n == 1 ? v[0] : v[vox]; }
};

HostDiag check_diag(const vs_diag& d, int64_t V, const char* name) {
  VS_REQUIRE(d.v != nullptr, std::string(name) + " is NULL");
  VS_REQUIRE(d.n == 1 || d.n == V, std::string(name) + " must have 1 or L*M*N entries");
  return HostDiag{reinterpret_cast<const cd*>(d.v), d.n};
}

void upload_diag(VsDiagDev& dst, const std::vector<cd>& vals, cudaStream_t st) {
  bool uniform = true;
  for (size_t e = 1; e < vals.size(); ++e)
    if (vals[e] != vals[0]) { uniform = false; break; }
  if (uniform) {
    dst.arr = false;
    const cd s = vals.empty() ? cd(0, 0) : vals[0];
    dst.s = make_double2(s.real(), s.imag());
    return;
  }
  dst.arr = true;
  const size_t n = vals.size();
  std::vector<float2> f(n);
  for (size_t e = 0; e < n; ++e) f[e] = make_float2((float)vals[e].real(), (float)vals[e].imag());
  dst.v64.alloc(n * sizeof(double2));
  dst.v32.alloc(n * sizeof(float2));
  VS_CUDA(cudaMemcpyAsync(dst.v64.p, vals.data(), n * sizeof(double2), cudaMemcpyHostToDevice, st));
  VS_CUDA(cudaMemcpyAsync(dst.v32.p, f.data(), n * sizeof(float2), cudaMemcpyHostToDevice, st));
  VS_CUDA(cudaStreamSynchronize(st));
}

void check_grid(int64_t L, int64_t M, int64_t N) {
  VS_REQUIRE(L >= 1 && M >= 1 && N >= 1, "L, M, N must be >= 1");
  VS_REQUIRE(L <= 2048 && M <= 2048 && N <= 2048, "grid extent above 2048");
  VS_REQUIRE(3 * L * M * N < (int64_t(1) << 31), "3*L*M*N must fit in int32");
}

void check_fft_len(int64_t P, int64_t L, const char* name) {
  VS_REQUIRE(P >= 2 * L - 1, std::string(name) + " must be >= 2*extent-1 for an exact circulant embedding");
  VS_REQUIRE(P <= 4096, std::string(name) + " above 4096");
}

// Shared tail of the two operator constructors: index maps, diagonals, FFT
// axes, spectrum (from fN_full, P*Q*R*6 unscaled), scratch.
void op_common(vs_op* op, const int64_t* idx3, int64_t n3, vs_diag Mr, vs_diag Mc, vs_diag Gram) {
  cudaStream_t st = op->ctx->stream;
  const int64_t V = op->V;
  VS_REQUIRE(idx3 != nullptr || n3 == 0, "idx3 is NULL");
  VS_REQUIRE(n3 >= 1 && n3 <= 3 * V, "n3 must be in [1, 3*L*M*N]");
  std::vector<int> map3(3 * V, -1);
  std::vector<int> p2g(n3);
  for (int64_t e = 0; e < n3; ++e) {
    const int64_t g = idx3[e];
    VS_REQUIRE(g >= 0 && g < 3 * V, "idx3 entry out of range [0, 3*L*M*N)");
    VS_REQUIRE(map3[g] < 0, "idx3 has a repeated entry");
    map3[g] = (int)e;
    p2g[e] = (int)g;
  }
  op->n3 = n3;
  op->std3 = (n3 % 3 == 0);
  for (int64_t e = 0; op->std3 && e < n3 / 3; ++e)
    op->std3 = idx3[e] < V && idx3[e + n3 / 3] == idx3[e] + V && idx3[e + 2 * n3 / 3] == idx3[e] + 2 * V;
  op->map3.alloc(map3.size() * sizeof(int));
  op->pos2grid.alloc(p2g.size() * sizeof(int));
  VS_CUDA(cudaMemcpyAsync(op->map3.p, map3.data(), map3.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  VS_CUDA(cudaMemcpyAsync(op->pos2grid.p, p2g.data(), p2g.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  HostDiag mr = check_diag(Mr, V, "Mr"), mc = check_diag(Mc, V, "Mc"), gr = check_diag(Gram, V, "Gram");
  std::vector<cd> d1(n3), d1c(n3), d2(n3), dmr(n3);
  for (int64_t e = 0; e < n3; ++e) {
    const int64_t vox = idx3[e] % V;
    d1[e] = gr.at(vox) * mr.at(vox);
    d1c[e] = gr.at(vox) * std::conj(mr.at(vox));
    d2[e] = mc.at(vox);
    dmr[e] = mr.at(vox);
  }
  upload_diag(op->d1, d1, st);
  upload_diag(op->d1c, d1c, st);
  upload_diag(op->d2, d2, st);
  upload_diag(op->mr, dmr, st);
  VS_CUDA(cudaStreamSynchronize(st));
}

void axes_init(vs_op* op) {
  cudaStream_t st = op->ctx->stream;
  op->ax[0].init(op->P, st);
  op->ax[1].init(op->Q, st);
  op->ax[2].init(op->R, st);
}

void spectrum_from_full(vs_op* op, const double2* full) {
  const int64_t PQR = (int64_t)op->P * op->Q * op->R;
  if (op->gsym) {
    const int64_t oct = (int64_t)(op->P / 2 + 1) * (op->Q / 2 + 1) * (op->R / 2 + 1);
    op->G64.alloc(6 * oct * sizeof(double2));
    op->G32.alloc(6 * oct * sizeof(float2));
    vs::octant_spectrum(full, op->P, op->Q, op->R, 1.0 / (double)PQR, op->G64.as<double2>(), op->G32.as<float2>(),
                        op->ctx->stream);
    return;
  }
  op->G64.alloc(6 * PQR * sizeof(double2));
  op->G32.alloc(6 * PQR * sizeof(float2));
  vs::finalize_spectrum(full, 6 * PQR, 1.0 / (double)PQR, op->G64.as<double2>(), op->G32.as<float2>(),
                        op->ctx->stream);
}

// Caller blocks <-> device blocks (both column-major; device copies carry the 1/(L*M) of the inverse FFTs).
__global__ void k_blocks_in(const double2* __restrict__ in, int64_t total, double scale, double2* o64,
                            float2* o32) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = make_double2(in[e].x * scale, in[e].y * scale);
    if (o64) o64[e] = v;
    if (o32) o32[e] = make_float2((float)v.x, (float)v.y);
  }
}

// Expands stored blocks to the full L*M set; with sym, block (i, j) comes from
// the stored (min(i, L-i), min(j, M-j)) with the parity signs of the x/y
// component rows and columns.
__global__ void k_blocks_out(const double2* __restrict__ i64, const float2* __restrict__ i32, int L, int M, int N,
                             int sym, double scale, double2* __restrict__ out) {
  const int n = 3 * N;
  const int64_t nn = (int64_t)n * n, total = (int64_t)L * M * nn;
  const int Lb = sym ? L / 2 + 1 : L;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn, r = e - b * nn;
    const int i = (int)(b % L), j = (int)(b / L);
    const int q = (int)(r / n), p = (int)(r - (int64_t)q * n);  // column-major (p, q)
    const bool fx = sym && i > L / 2, fy = sym && j > M / 2;
    const int is = fx ? L - i : i, js = fy ? M - j : j;
    const int64_t src = ((int64_t)is + (int64_t)Lb * js) * nn + r;
    const double2 a = i64 ? i64[src] : make_double2(i32[src].x, i32[src].y);
    const int cp = p / N, cq = q / N;
    const bool fp = (cp == 0 && fx) != (cp == 1 && fy);
    const bool fq = (cq == 0 && fx) != (cq == 1 && fy);
    const double sg = (fp != fq) ? -scale : scale;
    out[e] = make_double2(a.x * sg, a.y * sg);
  }
}

void prec_common_impl(vs_prec* pr, int precisions) {
  VS_REQUIRE((precisions & 3) != 0 && (precisions & ~15) == 0,
             "precisions must be VS_BUILD_C64 and/or VS_BUILD_C128 (optionally one of VS_BUILD_LU_TC, VS_BUILD_LU_CUDA)");
  VS_REQUIRE((precisions & 12) != 12, "VS_BUILD_LU_TC and VS_BUILD_LU_CUDA exclude each other");
  cudaStream_t st = pr->ctx->stream;
  pr->axL.init(pr->L, st);
  pr->axM.init(pr->M, st);
  pr->t.alloc((size_t)pr->L * pr->M * pr->N * 3 * sizeof(double2));
  pr->nrhs_cap = 1;
  pr->gemv_status.alloc(sizeof(int));
  VS_CUDA(cudaMemsetAsync(pr->gemv_status.p, 0, sizeof(int), st));
}

// Raises if a streamed-GEMV wait of this preconditioner ever ran out (the
// stream must be idle).
void check_prec_status(vs_prec* pr) {
  if (!pr || !pr->gemv_status.p) return;
  int hs = 0;
  VS_CUDA(cudaMemcpy(&hs, pr->gemv_status.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (hs != 0) {
    // reported once: the next apply starts from a clear status
    VS_CUDA(cudaMemset(pr->gemv_status.p, 0, sizeof(int)));
    throw vs::Error(VS_ERR_TIMEOUT, "a streamed preconditioner GEMV wait ran out (its result is not valid)");
  }
}

void prec_scratch_impl(vs_prec* pr, int64_t nrhs) {
  if (nrhs > pr->nrhs_cap) {
    pr->t.alloc((size_t)pr->L * pr->M * pr->N * 3 * sizeof(double2) * nrhs);
    pr->nrhs_cap = (int)nrhs;
  }
}

template <typename F>
void time_passes(cudaStream_t st, int nrep, float* ms_out, F&& launch) {
  cudaEvent_t ev[6];
  for (auto& e : ev) VS_CUDA(cudaEventCreate(&e));
  float acc[5] = {0, 0, 0, 0, 0};
  try {
    for (int r = 0; r < nrep; ++r) {
      VS_CUDA(cudaEventRecord(ev[0], st));
      for (int p = 0; p < 5; ++p) {
        launch(p);
        VS_CUDA(cudaEventRecord(ev[p + 1], st));
      }
      VS_CUDA(cudaEventSynchronize(ev[5]));
      for (int p = 0; p < 5; ++p) {
        float ms = 0;
        VS_CUDA(cudaEventElapsedTime(&ms, ev[p], ev[p + 1]));
        acc[p] += ms;
      }
    }
  } catch (...) {
    for (auto& e : ev) cudaEventDestroy(e);
    throw;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int p = 0; p < 5; ++p) ms_out[p] = acc[p] / nrep;
}

vs::SolveParams solve_params(vs_op* op, vs_prec* prec, const vs_solve_opts* o) {
  VS_REQUIRE(o, "NULL argument");
  VS_REQUIRE(o->method == VS_BICGSTAB || o->method == VS_GMRES || o->method == VS_GMRES_DR, "unsupported method");
  VS_REQUIRE(o->method != VS_GMRES || (o->restart >= 1 && o->restart <= 2048), "GMRES restart must be in [1, 2048]");
  VS_REQUIRE(o->method != VS_GMRES_DR || (o->restart >= 2 && o->restart <= 256),
             "GMRES-DR restart must be in [2, 256]");
  VS_REQUIRE(o->method != VS_GMRES_DR || (o->ritz >= 1 && o->ritz < o->restart),
             "GMRES-DR ritz must be in [1, restart - 1]");
  VS_REQUIRE(o->precision == VS_SOLVE_MIXED || o->precision == VS_SOLVE_FP64, "bad precision");
  VS_REQUIRE(o->tol > 0 && o->maxit >= 0 && o->iters_per_graph >= 1 && o->iters_per_graph <= 64, "bad options");
  VS_REQUIRE(!prec || (prec->L == op->L && prec->M == op->M && prec->N == op->N && prec->n3 == op->n3),
             "preconditioner does not match the operator");
  VS_REQUIRE(!prec || (o->precision == VS_SOLVE_MIXED ? prec->inv32.p != nullptr : prec->inv64.p != nullptr),
             "preconditioner not built in the precision this solve needs");
  VS_REQUIRE(o->transpose == 0 || o->transpose == 1, "transpose must be 0 or 1");
  vs::SolveParams prm;
  prm.mode = o->precision;
  prm.tol = o->tol;
  prm.maxit = o->maxit;
  prm.inner_tol = o->inner_tol;
  prm.max_refine = o->max_refine;
  prm.per_graph = o->iters_per_graph;
  prm.resvec_cap = (int)std::min<int64_t>(o->resvec ? o->resvec_cap : 0, 1 << 30);
  prm.resvec_host = o->resvec;
  prm.op_mode = o->transpose ? VS_TRANSP : VS_NOTRANSP;
  prm.restart = o->restart;
  prm.ritz = o->ritz;
  VS_REQUIRE(o->gram == nullptr || o->gram_n == 1 || o->gram_n == op->V,
             "gram_n must be 1 or L*M*N when a Gram per right-hand side is given");
  prm.gram_host = reinterpret_cast<const double2*>(o->gram);
  prm.gram_n = o->gram ? o->gram_n : 0;
  VS_REQUIRE(o->unfused == 0 || o->unfused == 1, "unfused must be 0 or 1");
  prm.fold_steps = o->unfused == 0;
  return prm;
}

void fill_info(const vs::SolveResult& r, vs_solve_info* info) {
  info->flag = r.flag;
  info->relres = r.relres;
  info->iter = r.iter;
  info->refinements = r.refinements;
  info->n_resvec = r.n_resvec;
  info->kernel_launches = r.launches;
}

// The 16 floats of vs_solve_opts.profile_ms from a solve's profile.
void write_profile(const vs::SolveProfile& p, float* out) {
  for (int i = 0; i < 16; ++i) out[i] = 0.0f;
  if (p.iters > 0) {
    // every pass runs twice per iteration
    for (int i = 0; i < 10; ++i) out[i] = (float)(p.pass_ms[i] / (2.0 * p.iters));
    out[10] = (float)(p.vec_ms / p.iters);
  }
  out[11] = (float)p.iters;
  if (p.resid_calls > 0) out[12] = (float)(p.resid_ms / p.resid_calls);
  out[13] = (float)p.resid_calls;
}

void solve_impl(vs_op* op, vs_prec* prec, const double2* b, double2* x, const vs_solve_opts* o,
                vs_solve_info* info) {
  VS_REQUIRE(info, "NULL argument");
  vs::SolveParams prm = solve_params(op, prec, o);
  vs::SolveProfile prof;
  if (o->profile_ms) prm.profile = &prof;
  vs::SolveResult r;
  if (o->method == VS_GMRES) vs::solve_gmres(*op, prec, b, x, prm, r, op->ctx->stream);
  else if (o->method == VS_GMRES_DR) vs::solve_gmres_dr(*op, prec, b, x, prm, r, op->ctx->stream);
  else vs::solve_bicgstab(*op, prec, b, x, prm, r, op->ctx->stream);
  check_prec_status(prec);
  fill_info(r, info);
  if (o->profile_ms) write_profile(prof, o->profile_ms);
}

// nrhs right-hand sides: BiCGSTAB runs them as one batch (every launch serves
// all of them); GMRES runs them one after another.
void solve_batch_impl(vs_op* op, vs_prec* prec, const double2* b, double2* x, int64_t nrhs, const vs_solve_opts* o,
                      vs_solve_info* infos) {
  VS_REQUIRE(infos, "NULL argument");
  VS_REQUIRE(nrhs >= 1 && nrhs <= 4096, "nrhs must be in [1, 4096]");
  vs::SolveParams prm = solve_params(op, prec, o);
  const int64_t n = op->n3;
  if (o->method == VS_GMRES || o->method == VS_GMRES_DR) {
    for (int64_t r = 0; r < nrhs; ++r) {
      vs::SolveParams p1 = prm;
      p1.resvec_host = prm.resvec_host ? prm.resvec_host + r * prm.resvec_cap : nullptr;
      p1.gram_host = prm.gram_host ? prm.gram_host + r * prm.gram_n : nullptr;
      vs::SolveResult res;
      if (o->method == VS_GMRES) vs::solve_gmres(*op, prec, b + r * n, x + r * n, p1, res, op->ctx->stream);
      else vs::solve_gmres_dr(*op, prec, b + r * n, x + r * n, p1, res, op->ctx->stream);
      fill_info(res, infos + r);
    }
    check_prec_status(prec);
    return;
  }
  vs::SolveProfile prof;
  if (o->profile_ms) prm.profile = &prof;
  std::vector<vs::SolveResult> res;
  vs::solve_bicgstab_batch(*op, prec, b, x, (int)nrhs, prm, res, op->ctx->stream);
  check_prec_status(prec);
  for (int64_t r = 0; r < nrhs; ++r) fill_info(res[r], infos + r);
  if (o->profile_ms) write_profile(prof, o->profile_ms);
}

// S = sum_j (k_hat_j e_hat_j)^2 of the LDR polarisability (getOPERATOR_DDA.m:14-20).
double ldr_S(const double kvec[3], const double E0[3]) {
  const double nk = std::sqrt(kvec[0] * kvec[0] + kvec[1] * kvec[1] + kvec[2] * kvec[2]);
  const double ne = std::sqrt(E0[0] * E0[0] + E0[1] * E0[1] + E0[2] * E0[2]);
  VS_REQUIRE(nk > 0 && ne > 0, "kvec and E0 must be non-zero");
  double S = 0;
  for (int j = 0; j < 3; ++j) {
    const double t = (kvec[j] / nk) * (E0[j] / ne);
    S += t * t;
  }
  return S;
}

// Two orthonormal polarisations of a unit incident direction k:
// e1 = k x z / |k x z| (k x x when k is along z), e2 = k x e1.
void polarisation_basis(const double k[3], double e1[3], double e2[3]) {
  double a[3] = {k[1], -k[0], 0.0};  // k x z
  double na = std::sqrt(a[0] * a[0] + a[1] * a[1]);
  if (na < 1e-6) {
    a[0] = 0.0; a[1] = k[2]; a[2] = -k[1];  // k x x
    na = std::sqrt(a[1] * a[1] + a[2] * a[2]);
  }
  for (int j = 0; j < 3; ++j) e1[j] = a[j] / na;
  e2[0] = k[1] * e1[2] - k[2] * e1[1];
  e2[1] = k[2] * e1[0] - k[0] * e1[2];
  e2[2] = k[0] * e1[1] - k[1] * e1[0];
}

// alpha_LDR of one element (getOPERATOR_DDA.m:7-26), dimensionless.
cd alpha_ldr_one(cd m, bool is_eps, double kd, double S) {
  const double b1 = -1.8915316, b2 = 0.1648469, b3 = -1.7700004;
  const cd msqr = is_eps ? m : m * m;
  const cd aCM = 3.0 / (4.0 * M_PI) * (msqr - 1.0) / (msqr + 2.0);
  return aCM / (1.0 + aCM * ((b1 + msqr * b2 + msqr * b3 * S) * kd * kd - cd(0, 2.0 / 3.0) * kd * kd * kd));
}

}  // namespace

void record_error(vs_ctx* ctx, const char* msg) {
  g_last_error = msg;
  if (ctx) ctx->err = msg;
}

void ctx_retain(vs_ctx* ctx) {
  if (ctx) ctx->refs.fetch_add(1);
}

void ctx_release(vs_ctx* ctx) {
  if (!ctx || ctx->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(ctx->device);
  ctx->pgraph32.reset();
  ctx->pgraph64.reset();
  for (cudaStream_t a : ctx->aux) cudaStreamDestroy(a);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// host complex double -> device buffer of the precision's type
static void upload_as(const double* h, int64_t n, bool c64, vs::DevBuf& stage, vs::DevBuf& out, cudaStream_t st) {
  if (c64) {
    stage.alloc(n * sizeof(double2));
    out.alloc(n * sizeof(float2));
    VS_CUDA(cudaMemcpyAsync(stage.p, h, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    vs::c128_to_c64(stage.as<double2>(), out.as<float2>(), n, st);
  } else {
    out.alloc(n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(out.p, h, n * sizeof(double2), cudaMemcpyHostToDevice, st));
  }
}

extern "C" {

int vs_ctx_create(int device, vs_ctx** out) {
  return guarded(nullptr, [&] {
    VS_REQUIRE(out != nullptr, "out is NULL");
    int n = 0;
    VS_CUDA(cudaGetDeviceCount(&n));
    VS_REQUIRE(device >= 0 && device < n, "no such CUDA device");
    VS_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    VS_CUDA(cudaGetDeviceProperties(&prop, device));
    if (!(prop.major == 10 && prop.minor == 3))
      throw vs::Error(VS_ERR_UNSUPPORTED, std::string("libvoxscatter is built for sm_103a; device is ") + prop.name +
                                              " sm_" + std::to_string(prop.major) + std::to_string(prop.minor));
    auto* c = new vs_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      throw vs::Error(VS_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = c;
  });
}

int vs_ctx_destroy(vs_ctx* ctx) {
  if (!ctx) return VS_OK;
  int st = guarded(ctx, [&] { VS_CUDA(cudaStreamSynchronize(ctx->stream)); });
  ctx_release(ctx);
  return st;
}

const char* vs_last_error(const vs_ctx* ctx) { return ctx ? ctx->err.c_str() : g_last_error.c_str(); }

int vs_ctx_synchronize(vs_ctx* ctx) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] { VS_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int vs_ctx_stream(vs_ctx* ctx, void** stream) {
  if (!ctx || !stream) return VS_ERR_ARG;
  *stream = (void*)ctx->stream;
  return VS_OK;
}

int vs_alpha_ldr(const double* m, int64_t n, int is_eps, double ko, double d, const double kvec[3],
                            const double E0[3], double* alpha_out) {
  return guarded(nullptr, [&] {
    VS_REQUIRE(m && alpha_out && kvec && E0 && n >= 0, "NULL argument");
    const double S = ldr_S(kvec, E0);
    const cd* mm = reinterpret_cast<const cd*>(m);
    cd* out = reinterpret_cast<cd*>(alpha_out);
    for (int64_t e = 0; e < n; ++e) out[e] = alpha_ldr_one(mm[e], is_eps != 0, ko * d, S);
  });
}

int vs_eps_layer_average(int64_t L, int64_t M, int64_t N, const double* eps_r, double* face3) {
  return guarded(nullptr, [&] {
    VS_REQUIRE(eps_r && face3, "NULL argument");
    VS_REQUIRE(L >= 1 && M >= 1 && N >= 1, "L, M, N must be positive");
    const cd* e = reinterpret_cast<const cd*>(eps_r);
    cd* f = reinterpret_cast<cd*>(face3);
    for (int64_t k = 0; k < N; ++k) {
      // mean over x, then over y (the order of the reference's two averages)
      cd sy = 0;
      for (int64_t j = 0; j < M; ++j) {
        cd sx = 0;
        for (int64_t i = 0; i < L; ++i) sx += e[i + L * (j + M * k)];
        sy += sx / (double)L;
      }
      const cd t = sy / (double)M;
      VS_REQUIRE(std::abs(t) > 0, "layer-average permittivity is zero");
      const cd fk = (t - 1.0) / t;
      f[k] = fk;
      f[N + k] = fk;
      f[2 * N + k] = fk;
    }
  });
}

int vs_green_dda(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* ox, const double* oy,
                 const double* oz, double ko, int near_quad, double* toep_out) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(ox && oy && oz && toep_out, "NULL argument");
    cudaStream_t st = ctx->stream;
    const int64_t V = L * M * N;
    vs::DevBuf dox, doy, doz, dt;
    dox.alloc(L * sizeof(double)); doy.alloc(M * sizeof(double)); doz.alloc(N * sizeof(double));
    dt.alloc(6 * V * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dox.p, ox, L * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(doy.p, oy, M * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(doz.p, oz, N * sizeof(double), cudaMemcpyHostToDevice, st));
    vs::green_dda_device((int)L, (int)M, (int)N, dox.as<double>(), doy.as<double>(), doz.as<double>(), ko,
                         near_quad, dt.as<double2>(), st);
    VS_CUDA(cudaMemcpyAsync(toep_out, dt.p, 6 * V * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_nop_assemble(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, double ko, double dx, const double* near_J,
                    double* G_out) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(G_out, "G_out is NULL");
    VS_REQUIRE(dx > 0 && std::isfinite(dx) && std::isfinite(ko), "dx must be positive and ko finite");
    cudaStream_t st = ctx->stream;
    const int64_t V = L * M * N;
    const int64_t nb = std::min<int64_t>(2, L) * std::min<int64_t>(2, M) * std::min<int64_t>(2, N);
    vs::DevBuf g, nj;
    g.alloc(6 * V * sizeof(double2));
    if (near_J) {
      nj.alloc(36 * nb * sizeof(double2));
      VS_CUDA(cudaMemcpyAsync(nj.p, near_J, 36 * nb * sizeof(double2), cudaMemcpyHostToDevice, st));
    }
    vs::nop_assemble_device((int)L, (int)M, (int)N, ko, dx, near_J ? nj.as<double2>() : nullptr,
                            g.as<double2>(), st);
    VS_CUDA(cudaMemcpyAsync(G_out, g.p, 6 * V * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_circulant_fft(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, int64_t P, int64_t Q,
                     int64_t R, double* fN_out) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] {
    check_grid(L, M, N);
    check_fft_len(P, L, "P"); check_fft_len(Q, M, "Q"); check_fft_len(R, N, "R");
    VS_REQUIRE(toep && fN_out, "NULL argument");
    cudaStream_t st = ctx->stream;
    const int64_t V = L * M * N, PQR = P * Q * R;
    vs::DevBuf dt, df;
    dt.alloc(6 * V * sizeof(double2));
    df.alloc(6 * PQR * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dt.p, toep, 6 * V * sizeof(double2), cudaMemcpyHostToDevice, st));
    vs::FftAxis ax[3];
    ax[0].init((int)P, st); ax[1].init((int)Q, st); ax[2].init((int)R, st);
    vs::embed_fft_device((int)L, (int)M, (int)N, dt.as<double2>(), (int)P, (int)Q, (int)R, df.as<double2>(), ax, st);
    VS_CUDA(cudaMemcpyAsync(fN_out, df.p, 6 * PQR * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_op_create(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, int64_t P, int64_t Q, int64_t R,
                 const int64_t* idx3, int64_t n3, vs_diag Mr, vs_diag Mc, vs_diag Gram, vs_op** out) {
  if (!ctx) return VS_ERR_ARG;
  vs_op* op = nullptr;
  int s = guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(toep && out, "NULL argument");
    if (P <= 0) P = vs::smooth_size((int)(2 * L - 1));
    if (Q <= 0) Q = vs::smooth_size((int)(2 * M - 1));
    if (R <= 0) R = vs::z_pass_length((int)(2 * N - 1));
    check_fft_len(P, L, "P"); check_fft_len(Q, M, "Q"); check_fft_len(R, N, "R");
    op = new vs_op();
    op->ctx = ctx;
    ctx_retain(ctx);
    op->L = (int)L; op->M = (int)M; op->N = (int)N;
    op->P = (int)P; op->Q = (int)Q; op->R = (int)R;
    op->V = L * M * N;
    op_common(op, idx3, n3, Mr, Mc, Gram);
    op->gsym = vs::toeplitz_has_exact_parity(toep, op->L, op->M, op->N);
    cudaStream_t st = ctx->stream;
    op->toep64.alloc(6 * op->V * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(op->toep64.p, toep, 6 * op->V * sizeof(double2), cudaMemcpyHostToDevice, st));
    axes_init(op);
    const int64_t PQR = P * Q * R;
    vs::DevBuf full;
    full.alloc(6 * PQR * sizeof(double2));
    vs::embed_fft_device(op->L, op->M, op->N, op->toep64.as<double2>(), op->P, op->Q, op->R, full.as<double2>(),
                         op->ax, st);
    spectrum_from_full(op, full.as<double2>());
    vs::ensure_scratch(*op, 1, sizeof(float2));
    vs::autotune_op<float>(*op, st);
    vs::autotune_op<double>(*op, st);
    VS_CUDA(cudaStreamSynchronize(st));
    *out = op;
  });
  if (s != VS_OK) delete op;
  return s;
}

int vs_op_create_fN(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* fN, int64_t P, int64_t Q,
                    int64_t R, const int64_t* idx3, int64_t n3, vs_diag Mr, vs_diag Mc, vs_diag Gram,
                    vs_op** out) {
  if (!ctx) return VS_ERR_ARG;
  vs_op* op = nullptr;
  int s = guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(fN && out, "NULL argument");
    check_fft_len(P, L, "P"); check_fft_len(Q, M, "Q"); check_fft_len(R, N, "R");
    op = new vs_op();
    op->ctx = ctx;
    ctx_retain(ctx);
    op->L = (int)L; op->M = (int)M; op->N = (int)N;
    op->P = (int)P; op->Q = (int)Q; op->R = (int)R;
    op->V = L * M * N;
    op_common(op, idx3, n3, Mr, Mc, Gram);
    cudaStream_t st = ctx->stream;
    axes_init(op);
    const int64_t PQR = P * Q * R;
    vs::DevBuf full;
    full.alloc(6 * PQR * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(full.p, fN, 6 * PQR * sizeof(double2), cudaMemcpyHostToDevice, st));
    spectrum_from_full(op, full.as<double2>());
    op->toep64.alloc(6 * op->V * sizeof(double2));
    vs::toep_from_fN_device(op->L, op->M, op->N, op->P, op->Q, op->R, full.as<double2>(), op->toep64.as<double2>(),
                            op->ax, st);
    vs::ensure_scratch(*op, 1, sizeof(float2));
    vs::autotune_op<float>(*op, st);
    vs::autotune_op<double>(*op, st);
    VS_CUDA(cudaStreamSynchronize(st));
    *out = op;
  });
  if (s != VS_OK) delete op;
  return s;
}

int vs_op_destroy(vs_op* op) {
  if (!op) return VS_OK;
  int s = guarded(op->ctx, [&] { VS_CUDA(cudaStreamSynchronize(op->ctx->stream)); });
  delete op;
  return s;
}

int vs_op_info(const vs_op* op, int64_t* LMN, int64_t* PQR, int64_t* n3) {
  if (!op) return VS_ERR_ARG;
  if (LMN) { LMN[0] = op->L; LMN[1] = op->M; LMN[2] = op->N; }
  if (PQR) { PQR[0] = op->P; PQR[1] = op->Q; PQR[2] = op->R; }
  if (n3) *n3 = op->n3;
  return VS_OK;
}

int vs_op_apply_device(vs_op* op, const void* x, void* y, int64_t nrhs, int mode, int precision) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x && y, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    VS_REQUIRE(mode >= VS_NOTRANSP && mode <= VS_CONJTRANSP, "bad mode");
    cudaStream_t st = op->ctx->stream;
    if (precision == VS_C64) {
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      vs::matvec<float>(*op, (const float2*)x, (float2*)y, (int)nrhs, mode, nullptr, st);
    } else {
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      vs::matvec<double>(*op, (const double2*)x, (double2*)y, (int)nrhs, mode, nullptr, st);
    }
  });
}

int vs_op_apply(vs_op* op, const double* x, double* y, int64_t nrhs, int mode, int precision) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x && y, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    VS_REQUIRE(mode >= VS_NOTRANSP && mode <= VS_CONJTRANSP, "bad mode");
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n3 * nrhs;
    op->xin.alloc(n * sizeof(double2) * (precision == VS_C64 ? 1 : 1));
    op->yout.alloc(n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(op->xin.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if (precision == VS_C64) {
      vs::DevBuf x32, y32;
      x32.alloc(n * sizeof(float2));
      y32.alloc(n * sizeof(float2));
      vs::c128_to_c64(op->xin.as<double2>(), x32.as<float2>(), n, st);
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      vs::matvec<float>(*op, x32.as<float2>(), y32.as<float2>(), (int)nrhs, mode, nullptr, st);
      vs::c64_to_c128(y32.as<float2>(), op->yout.as<double2>(), n, st);
      VS_CUDA(cudaMemcpyAsync(y, op->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VS_CUDA(cudaStreamSynchronize(st));
    } else {
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      vs::matvec<double>(*op, op->xin.as<double2>(), op->yout.as<double2>(), (int)nrhs, mode, nullptr, st);
      VS_CUDA(cudaMemcpyAsync(y, op->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VS_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int vs_op_apply_gram(vs_op* op, const double* x, double* y, int64_t nrhs, int mode, int precision,
                     const double* gram, int64_t gram_n) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x && y && gram, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    VS_REQUIRE(mode >= VS_NOTRANSP && mode <= VS_CONJTRANSP, "bad mode");
    cudaStream_t st = op->ctx->stream;
    vs::DevBuf g64, g32, stage, xd, yd, y64;
    vs::RhsGram rg;
    vs::upload_rhs_gram(*op, reinterpret_cast<const double2*>(gram), nrhs, gram_n, g64, g32, rg, st);
    const int64_t n = op->n3 * nrhs;
    const bool c64 = precision == VS_C64;
    upload_as(x, n, c64, stage, xd, st);
    if (c64) {
      yd.alloc(n * sizeof(float2));
      y64.alloc(n * sizeof(double2));
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      vs::matvec<float>(*op, xd.as<float2>(), yd.as<float2>(), (int)nrhs, mode, nullptr, st, 0, &rg);
      vs::c64_to_c128(yd.as<float2>(), y64.as<double2>(), n, st);
      VS_CUDA(cudaMemcpyAsync(y, y64.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    } else {
      yd.alloc(n * sizeof(double2));
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      vs::matvec<double>(*op, xd.as<double2>(), yd.as<double2>(), (int)nrhs, mode, nullptr, st, 0, &rg);
      VS_CUDA(cudaMemcpyAsync(y, yd.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

// ---- preconditioner ---------------------------------------------------

int vs_circ_levels(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* toep, double* circL_out,
                   double* circM_out, double* blocks_out) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(toep, "toep is NULL");
    cudaStream_t st = ctx->stream;
    const int64_t V = L * M * N;
    vs::DevBuf dt, l1, l2, blk, status;
    dt.alloc(6 * V * sizeof(double2));
    l1.alloc(6 * V * sizeof(double2));
    l2.alloc(6 * V * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dt.p, toep, 6 * V * sizeof(double2), cudaMemcpyHostToDevice, st));
    vs::FftAxis axL, axM;
    axL.init((int)L, st);
    axM.init((int)M, st);
    vs::circ_levels_device((int)L, (int)M, (int)N, dt.as<double2>(), l1.as<double2>(), l2.as<double2>(), axL, axM, st);
    if (circL_out) VS_CUDA(cudaMemcpyAsync(circL_out, l1.p, 6 * V * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (circM_out) {
      VS_CUDA(cudaMemcpyAsync(circM_out, l2.p, 6 * V * sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    if (blocks_out) {
      const int64_t n = 3 * N;
      blk.alloc(L * M * n * n * sizeof(double2));
      status.alloc(sizeof(int));
      VS_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
      vs::assemble_invert<double>(l2.as<double2>(), (int)L, (int)M, (int)N, make_double2(0, 0), nullptr,
                                  make_double2(-1, 0), false, true, 1.0, blk.as<double2>(), status.as<int>(), st);
      VS_CUDA(cudaMemcpyAsync(blocks_out, blk.p, L * M * n * n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    VS_CUDA(cudaStreamSynchronize(st));
    if (circM_out) {  // circ_2_level.m:44 stores -CC3 for the xz component
      double* c3 = circM_out + 2 * 2 * V;
      for (int64_t e = 0; e < 2 * V; ++e) c3[e] = -c3[e];
    }
  });
}


int vs_prec_create(vs_op* op, const double* shift, const double* d, int64_t nd, int precisions, vs_prec** out) {
  if (!op) return VS_ERR_ARG;
  vs_prec* pr = nullptr;
  int s = guarded(op->ctx, [&] {
    VS_REQUIRE(shift && d && out, "NULL argument");
    VS_REQUIRE(nd == 1 || nd == 3 * (int64_t)op->N, "d must have 1 or 3N entries");
    pr = new vs_prec();
    pr->id = next_object_id();
    pr->ctx = op->ctx;
    ctx_retain(pr->ctx);
    pr->L = op->L; pr->M = op->M; pr->N = op->N;
    pr->V = op->V; pr->n3 = op->n3;
    cudaStream_t st = op->ctx->stream;
    pr->map3.alloc(3 * op->V * sizeof(int));
    VS_CUDA(cudaMemcpyAsync(pr->map3.p, op->map3.p, 3 * op->V * sizeof(int), cudaMemcpyDeviceToDevice, st));
    prec_common_impl(pr, precisions);
    const int64_t V = op->V, n = 3 * op->N, LM = (int64_t)op->L * op->M;
    vs::DevBuf l1, l2, dv, status;
    l1.alloc(6 * V * sizeof(double2));
    l2.alloc(6 * V * sizeof(double2));
    status.alloc(sizeof(int));
    VS_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
    vs::circ_levels_device(op->L, op->M, op->N, op->toep64.as<double2>(), l1.as<double2>(), l2.as<double2>(), pr->axL,
                           pr->axM, st);
    const double2 sh = make_double2(shift[0], shift[1]);
    double2 ds = make_double2(d[0], d[1]);
    const double2* dptr = nullptr;
    if (nd > 1) {
      dv.alloc(nd * sizeof(double2));
      VS_CUDA(cudaMemcpyAsync(dv.p, d, nd * sizeof(double2), cudaMemcpyHostToDevice, st));
      dptr = dv.as<double2>();
    }
    const double scale = 1.0 / (double)LM;
    pr->sym = op->gsym;  // exact parity of the Toeplitz tensor: quadrant storage suffices
    const int64_t nblk = pr->sym ? (int64_t)(op->L / 2 + 1) * (op->M / 2 + 1) : LM;
    if (precisions & VS_BUILD_C64) {
      pr->inv32.alloc(nblk * n * n * sizeof(float2) + 64);
      const int lu = (precisions & VS_BUILD_LU_TC) ? vs::LU_TC : (precisions & VS_BUILD_LU_CUDA) ? vs::LU_CUDA
                                                                                                  : vs::LU_AUTO;
      vs::assemble_invert<float>(l2.as<double2>(), op->L, op->M, op->N, sh, dptr, ds, true, true, scale,
                                 pr->inv32.as<float2>(), status.as<int>(), st, pr->sym, lu);
    }
    if (precisions & VS_BUILD_C128) {
      pr->inv64.alloc(nblk * n * n * sizeof(double2) + 64);
      vs::assemble_invert<double>(l2.as<double2>(), op->L, op->M, op->N, sh, dptr, ds, true, true, scale,
                                  pr->inv64.as<double2>(), status.as<int>(), st, pr->sym);
    }
    int hs = 0;
    VS_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    if (hs & 8) throw vs::Error(VS_ERR_TIMEOUT, "a tensor-core MMA of the block inversion did not complete in time");
    VS_REQUIRE(hs == 0, "a preconditioner block is singular or its inverse is not finite");
    // with a uniform scaling d every block is symmetric up to the x/y sign flips
    if (nd == 1) vs::pack_sym_blocks(*pr, st);
    prec_scratch_impl(pr, 1);
    vs::autotune_prec<float>(*pr, st);
    vs::autotune_prec<double>(*pr, st);
    *out = pr;
  });
  if (s != VS_OK) delete pr;
  return s;
}

int vs_prec_create_blocks(vs_ctx* ctx, int64_t L, int64_t M, int64_t N, const double* inv_blocks,
                          const int64_t* idx3, int64_t n3, int precisions, vs_prec** out) {
  if (!ctx) return VS_ERR_ARG;
  vs_prec* pr = nullptr;
  int s = guarded(ctx, [&] {
    check_grid(L, M, N);
    VS_REQUIRE(inv_blocks && idx3 && out, "NULL argument");
    pr = new vs_prec();
    pr->id = next_object_id();
    pr->ctx = ctx;
    ctx_retain(ctx);
    pr->L = (int)L; pr->M = (int)M; pr->N = (int)N;
    pr->V = L * M * N;
    cudaStream_t st = ctx->stream;
    const int64_t V = pr->V;
    VS_REQUIRE(n3 >= 1 && n3 <= 3 * V, "n3 must be in [1, 3*L*M*N]");
    std::vector<int> map3(3 * V, -1);
    for (int64_t e = 0; e < n3; ++e) {
      const int64_t g = idx3[e];
      VS_REQUIRE(g >= 0 && g < 3 * V, "idx3 entry out of range [0, 3*L*M*N)");
      VS_REQUIRE(map3[g] < 0, "idx3 has a repeated entry");
      map3[g] = (int)e;
    }
    pr->n3 = n3;
    pr->map3.alloc(3 * V * sizeof(int));
    VS_CUDA(cudaMemcpyAsync(pr->map3.p, map3.data(), 3 * V * sizeof(int), cudaMemcpyHostToDevice, st));
    prec_common_impl(pr, precisions);
    const int64_t n = 3 * N, LM = L * M;
    vs::DevBuf raw;
    raw.alloc(LM * n * n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(raw.p, inv_blocks, LM * n * n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if (precisions & VS_BUILD_C64) pr->inv32.alloc(LM * n * n * sizeof(float2) + 64);
    if (precisions & VS_BUILD_C128) pr->inv64.alloc(LM * n * n * sizeof(double2) + 64);
    const int64_t tot = LM * n * n;
    k_blocks_in<<<(int)std::min<int64_t>(vs::ceil_div(tot, 256), 152 * 32), 256, 0, st>>>(
        raw.as<double2>(), tot, 1.0 / (double)LM, (precisions & VS_BUILD_C128) ? pr->inv64.as<double2>() : nullptr,
        (precisions & VS_BUILD_C64) ? pr->inv32.as<float2>() : nullptr);
    VS_LAUNCH_CHECK();
    VS_CUDA(cudaStreamSynchronize(st));
    *out = pr;
  });
  if (s != VS_OK) delete pr;
  return s;
}

int vs_invert_blocks_device(vs_ctx* ctx, void* mats, int64_t n, int64_t nmat, int method) {
  if (!ctx) return VS_ERR_ARG;
  return guarded(ctx, [&] {
    VS_REQUIRE(mats, "NULL argument");
    VS_REQUIRE(n >= 1 && n <= 4096 && nmat >= 0, "n must be in [1, 4096] and nmat >= 0");
    VS_REQUIRE(method == 0 || method == VS_BUILD_LU_TC || method == VS_BUILD_LU_CUDA, "bad method");
    VS_REQUIRE(method != VS_BUILD_LU_TC || vs::tc_invert_supported((int)n), "tensor-core inversion takes n <= 256");
    cudaStream_t st = ctx->stream;
    vs::DevBuf status;
    status.alloc(sizeof(int));
    VS_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
    vs::invert_blocks_device((float2*)mats, (int)n, nmat, method == VS_BUILD_LU_CUDA ? vs::LU_CUDA : vs::LU_TC, 1.0,
                             status.as<int>(), st);
    int hs = 0;
    VS_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    if (hs & 8) throw vs::Error(VS_ERR_TIMEOUT, "a tensor-core MMA of the block inversion did not complete in time");
    VS_REQUIRE(hs == 0, "a matrix is singular or its inverse is not finite");
  });
}

int vs_prec_destroy(vs_prec* prec) {
  if (!prec) return VS_OK;
  int s = guarded(prec->ctx, [&] { VS_CUDA(cudaStreamSynchronize(prec->ctx->stream)); });
  delete prec;
  return s;
}


int vs_prec_apply_device(vs_prec* prec, const void* x, void* y, int64_t nrhs, int precision) {
  if (!prec) return VS_ERR_ARG;
  return guarded(prec->ctx, [&] {
    VS_REQUIRE(x && y, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "bad precision");
    prec_scratch_impl(prec, nrhs);
    cudaStream_t st = prec->ctx->stream;
    if (precision == VS_C64) vs::prec_apply<float>(*prec, (const float2*)x, (float2*)y, (int)nrhs, nullptr, st);
    else vs::prec_apply<double>(*prec, (const double2*)x, (double2*)y, (int)nrhs, nullptr, st);
  });
}

int vs_prec_apply(vs_prec* prec, const double* x, double* y, int64_t nrhs, int precision) {
  if (!prec) return VS_ERR_ARG;
  return guarded(prec->ctx, [&] {
    VS_REQUIRE(x && y, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "bad precision");
    prec_scratch_impl(prec, nrhs);
    cudaStream_t st = prec->ctx->stream;
    const int64_t n = prec->n3 * nrhs;
    prec->xin.alloc(n * sizeof(double2));
    prec->yout.alloc(n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(prec->xin.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if (precision == VS_C64) {
      vs::DevBuf x32, y32;
      x32.alloc(n * sizeof(float2));
      y32.alloc(n * sizeof(float2));
      vs::c128_to_c64(prec->xin.as<double2>(), x32.as<float2>(), n, st);
      vs::prec_apply<float>(*prec, x32.as<float2>(), y32.as<float2>(), (int)nrhs, nullptr, st);
      vs::c64_to_c128(y32.as<float2>(), prec->yout.as<double2>(), n, st);
      VS_CUDA(cudaMemcpyAsync(y, prec->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VS_CUDA(cudaStreamSynchronize(st));
    } else {
      vs::prec_apply<double>(*prec, prec->xin.as<double2>(), prec->yout.as<double2>(), (int)nrhs, nullptr, st);
      VS_CUDA(cudaMemcpyAsync(y, prec->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VS_CUDA(cudaStreamSynchronize(st));
    }
    check_prec_status(prec);
  });
}

int vs_prec_get_blocks(vs_prec* prec, int precision, double* out) {
  if (!prec) return VS_ERR_ARG;
  return guarded(prec->ctx, [&] {
    VS_REQUIRE(out, "NULL argument");
    VS_REQUIRE((precision == VS_C64 && prec->inv32.p) || (precision == VS_C128 && prec->inv64.p),
               "preconditioner not built in that precision");
    cudaStream_t st = prec->ctx->stream;
    const int64_t n = 3 * prec->N, LM = (int64_t)prec->L * prec->M;
    vs::DevBuf o;
    o.alloc(LM * n * n * sizeof(double2));
    k_blocks_out<<<(int)std::min<int64_t>(vs::ceil_div(LM * n * n, 256), 152 * 32), 256, 0, st>>>(
        precision == VS_C128 ? prec->inv64.as<double2>() : nullptr,
        precision == VS_C64 ? prec->inv32.as<float2>() : nullptr, prec->L, prec->M, prec->N, prec->sym ? 1 : 0,
        (double)LM, o.as<double2>());
    VS_LAUNCH_CHECK();
    VS_CUDA(cudaMemcpyAsync(out, o.p, LM * n * n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

// ---- solve --------------------------------------------------------------

void vs_solve_opts_default(vs_solve_opts* o) {
  if (!o) return;
  o->method = VS_BICGSTAB;
  o->precision = VS_SOLVE_MIXED;
  o->tol = 1e-6;
  o->maxit = 2000;
  o->inner_tol = 0;
  o->max_refine = 10;
  o->iters_per_graph = 4;
  o->resvec = nullptr;
  o->resvec_cap = 0;
  o->transpose = 0;
  o->restart = 50;
  o->ritz = 10;
  o->gram = nullptr;
  o->gram_n = 0;
  o->profile_ms = nullptr;
  o->unfused = 0;
}


int vs_solve_device(vs_op* op, vs_prec* prec, const void* b, void* x, const vs_solve_opts* opts, vs_solve_info* info) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(b && x, "NULL argument");
    const auto t0 = std::chrono::steady_clock::now();
    solve_impl(op, prec, (const double2*)b, (double2*)x, opts, info);
    info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  });
}

int vs_solve(vs_op* op, vs_prec* prec, const double* b, double* x, const vs_solve_opts* opts, vs_solve_info* info) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(b && x, "NULL argument");
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n3;
    op->xin.alloc(n * sizeof(double2));
    op->yout.alloc(n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(op->xin.p, b, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(op->yout.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    solve_impl(op, prec, op->xin.as<double2>(), op->yout.as<double2>(), opts, info);
    VS_CUDA(cudaMemcpyAsync(x, op->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  });
}

// ---- diagnostics ----------------------------------------------------------

int vs_op_get_shape(const vs_op* op, int precision, vs_shape* shape) {
  if (!op || !shape || (precision != VS_C64 && precision != VS_C128)) return VS_ERR_ARG;
  const vs::PassShape& s = op->shape[precision == VS_C64 ? 0 : 1];
  shape->lg_lines_x = s.lg_lpb_x;
  shape->lg_tile_y = s.lg_tx_y;
  shape->lg_tile_z = s.lg_tx_z;
  shape->z_reg = s.z_reg;
  shape->y_reg = s.y_reg;
  shape->x_reg = s.x_reg;
  shape->z_df = s.z_df;
  return VS_OK;
}

int vs_prec_get_shape(const vs_prec* prec, int precision, vs_prec_shape* shape) {
  if (!prec || !shape || (precision != VS_C64 && precision != VS_C128)) return VS_ERR_ARG;
  const vs::PassShape& s = prec->shape[precision == VS_C64 ? 0 : 1];
  shape->lg_lines_x = s.lg_lpb_x;
  shape->lg_tile_y = s.lg_tx_y;
  shape->gemv_blocks = s.gemv_ti;
  shape->gemv_threads = s.gemv_threads;
  shape->gemv_mode = s.gemv_mode;
  shape->gemv_chunk = s.gemv_chunk;
  shape->y_reg = s.y_reg;
  shape->x_reg = s.x_reg;
  shape->fuse_xy = s.fuse_xy;
  shape->wait_polls = s.wait_polls;
  return VS_OK;
}

int vs_prec_set_shape(vs_prec* prec, int precision, const vs_prec_shape* shape) {
  if (!prec) return VS_ERR_ARG;
  return guarded(prec->ctx, [&] {
    VS_REQUIRE(shape && (precision == VS_C64 || precision == VS_C128), "bad argument");
    const size_t cs = precision == VS_C64 ? sizeof(float2) : sizeof(double2);
    const size_t lim = 227 * 1024;
    VS_REQUIRE(shape->lg_lines_x >= -1 && shape->lg_lines_x <= 8 && shape->lg_tile_y >= -1 && shape->lg_tile_y <= 8,
               "tile out of range");
    VS_REQUIRE(shape->lg_lines_x < 0 || (2ull * (1 << shape->lg_lines_x) * prec->L + prec->L) * cs <= lim,
               "x tile exceeds shared memory");
    VS_REQUIRE(shape->lg_tile_y < 0 || (2ull * prec->M * (1 << shape->lg_tile_y) + prec->M) * cs <= lim,
               "y tile exceeds shared memory");
    VS_REQUIRE(shape->gemv_blocks >= 0 && shape->gemv_blocks <= 64, "gemv_blocks out of range");
    VS_REQUIRE(shape->gemv_threads == 0 || (shape->gemv_threads >= 32 && shape->gemv_threads <= 256 &&
                                            shape->gemv_threads % 32 == 0),
               "gemv_threads must be 0 or a multiple of 32 in [32, 256]");
    vs::PassShape& s = prec->shape[precision == VS_C64 ? 0 : 1];
    s.lg_lpb_x = shape->lg_lines_x;
    s.lg_tx_y = shape->lg_tile_y;
    VS_REQUIRE(shape->gemv_mode >= -1 && shape->gemv_mode <= 2, "gemv_mode must be -1, 0, 1 or 2");
    if (shape->gemv_mode == 2 && (precision == VS_C64 ? prec->pk32.p : prec->pk64.p) == nullptr)
      throw vs::Error(VS_ERR_UNSUPPORTED, "packed symmetric blocks are not available for this preconditioner");
    VS_REQUIRE(shape->gemv_chunk >= 0 && shape->gemv_chunk <= 3 * prec->N, "gemv_chunk out of range");
    VS_REQUIRE(shape->gemv_mode < 1 || shape->gemv_blocks <= 4, "streamed GEMV takes 1 to 4 CTAs per SM");
    s.gemv_ti = shape->gemv_blocks;
    s.gemv_threads = shape->gemv_threads;
    VS_REQUIRE(shape->y_reg >= -1 && shape->y_reg <= 1, "y_reg must be -1, 0 or 1");
    s.gemv_mode = shape->gemv_mode;
    VS_REQUIRE(shape->x_reg >= -1 && shape->x_reg <= 1, "x_reg must be -1, 0 or 1");
    VS_REQUIRE(shape->fuse_xy >= -1 && shape->fuse_xy <= 1, "fuse_xy must be -1, 0 or 1");
    s.gemv_chunk = shape->gemv_chunk;
    s.y_reg = shape->y_reg;
    s.x_reg = shape->x_reg;
    s.fuse_xy = shape->fuse_xy;
    VS_REQUIRE(shape->wait_polls >= -1, "wait_polls must be >= -1");
    s.wait_polls = shape->wait_polls;
  });
}

int vs_op_set_shape(vs_op* op, int precision, const vs_shape* shape) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(shape && (precision == VS_C64 || precision == VS_C128), "bad argument");
    const size_t cs = precision == VS_C64 ? sizeof(float2) : sizeof(double2);
    const size_t lim = 227 * 1024;
    VS_REQUIRE(shape->lg_lines_x >= -1 && shape->lg_lines_x <= 8, "lg_lines_x out of range");
    VS_REQUIRE(shape->lg_tile_y >= -1 && shape->lg_tile_y <= 8, "lg_tile_y out of range");
    VS_REQUIRE(shape->lg_tile_z >= -1 && shape->lg_tile_z <= 8, "lg_tile_z out of range");
    VS_REQUIRE(shape->lg_lines_x < 0 || (2ull * (1 << shape->lg_lines_x) * op->P + op->P) * cs <= lim,
               "x tile exceeds shared memory");
    VS_REQUIRE(shape->lg_tile_y < 0 || (2ull * op->Q * (1 << shape->lg_tile_y) + op->Q) * cs <= lim,
               "y tile exceeds shared memory");
    VS_REQUIRE(shape->lg_tile_z < 0 || (2ull * op->R * 3 * (1 << shape->lg_tile_z) + op->R) * cs <= lim,
               "z tile exceeds shared memory");
    VS_REQUIRE(shape->z_reg >= -1 && shape->z_reg <= 2, "z_reg must be -1, 0, 1 or 2");
    VS_REQUIRE(shape->y_reg >= -1 && shape->y_reg <= 2, "y_reg must be -1, 0, 1 or 2");
    VS_REQUIRE(shape->x_reg >= -1 && shape->x_reg <= 2, "x_reg must be -1, 0, 1 or 2");
    VS_REQUIRE((shape->y_reg != 2 && shape->x_reg != 2) || precision == VS_C128,
               "x_reg / y_reg 2 (double-float arithmetic) apply to VS_C128 only");
    VS_REQUIRE(shape->z_df >= -1 && shape->z_df <= 1, "z_df must be -1, 0 or 1");
    VS_REQUIRE(shape->z_df != 1 || precision == VS_C128, "z_df applies to VS_C128 only");
    vs::PassShape& s = op->shape[precision == VS_C64 ? 0 : 1];
    s.lg_lpb_x = shape->lg_lines_x;
    s.lg_tx_y = shape->lg_tile_y;
    s.lg_tx_z = shape->lg_tile_z;
    s.z_reg = shape->z_reg;
    s.y_reg = shape->y_reg;
    s.x_reg = shape->x_reg;
    s.z_df = shape->z_df;
    op->kw.graph32.reset();
    op->kw.graph64.reset();
  });
}

int vs_op_time_passes(vs_op* op, const void* x, void* y, int64_t nrhs, int precision, int nrep, float* ms_out) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x && y && ms_out && nrep >= 1, "bad argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    cudaStream_t st = op->ctx->stream;
    if (precision == VS_C64) {
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      time_passes(st, nrep, ms_out, [&](int p) {
        vs::matvec_pass<float>(*op, (const float2*)x, (float2*)y, (int)nrhs, VS_NOTRANSP, nullptr, st, p);
      });
    } else {
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      time_passes(st, nrep, ms_out, [&](int p) {
        vs::matvec_pass<double>(*op, (const double2*)x, (double2*)y, (int)nrhs, VS_NOTRANSP, nullptr, st, p);
      });
    }
  });
}

int vs_prec_time_passes(vs_prec* prec, const void* x, void* y, int64_t nrhs, int precision, int nrep,
                        float* ms_out) {
  if (!prec) return VS_ERR_ARG;
  return guarded(prec->ctx, [&] {
    VS_REQUIRE(x && y && ms_out && nrep >= 1, "bad argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    prec_scratch_impl(prec, nrhs);
    cudaStream_t st = prec->ctx->stream;
    if (precision == VS_C64)
      time_passes(st, nrep, ms_out, [&](int p) {
        vs::prec_apply_pass<float>(*prec, (const float2*)x, (float2*)y, (int)nrhs, nullptr, st, p);
      });
    else
      time_passes(st, nrep, ms_out, [&](int p) {
        vs::prec_apply_pass<double>(*prec, (const double2*)x, (double2*)y, (int)nrhs, nullptr, st, p);
      });
  });
}

// ---- excitation, extinction, gradient --------------------------------------

int vs_plane_wave(vs_op* op, const double* x, const double* y, const double* z, const double kvec[3],
                  const double* E0, double* b_out) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x && y && z && kvec && E0 && b_out, "NULL argument");
    cudaStream_t st = op->ctx->stream;
    vs::DevBuf dx, dy, dz, db;
    dx.alloc(op->L * sizeof(double)); dy.alloc(op->M * sizeof(double)); dz.alloc(op->N * sizeof(double));
    db.alloc(op->n3 * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dx.p, x, op->L * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dy.p, y, op->M * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dz.p, z, op->N * sizeof(double), cudaMemcpyHostToDevice, st));
    const double2 e[3] = {make_double2(E0[0], E0[1]), make_double2(E0[2], E0[3]), make_double2(E0[4], E0[5])};
    vs::plane_wave_device(*op, dx.as<double>(), dy.as<double>(), dz.as<double>(), kvec, e, db.as<double2>(), st);
    VS_CUDA(cudaMemcpyAsync(b_out, db.p, op->n3 * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_op_apply_domain(vs_op* op, const double* x_grid, double* y_grid, int64_t nrhs, const double* a,
                       const double* b, int precision) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(x_grid && y_grid && a && b, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    cudaStream_t st = op->ctx->stream;
    const int64_t n = 3 * op->V * nrhs;
    const bool c64 = precision == VS_C64;
    vs::DevBuf stage, xd, yd, y64;
    upload_as(x_grid, n, c64, stage, xd, st);
    if (c64) {
      yd.alloc(n * sizeof(float2));
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      vs::matvec_domain<float>(*op, xd.as<float2>(), yd.as<float2>(), (int)nrhs, make_float2((float)a[0], (float)a[1]),
                               make_float2((float)b[0], (float)b[1]), st);
      y64.alloc(n * sizeof(double2));
      vs::c64_to_c128(yd.as<float2>(), y64.as<double2>(), n, st);
      VS_CUDA(cudaMemcpyAsync(y_grid, y64.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    } else {
      yd.alloc(n * sizeof(double2));
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      vs::matvec_domain<double>(*op, xd.as<double2>(), yd.as<double2>(), (int)nrhs, make_double2(a[0], a[1]),
                                make_double2(b[0], b[1]), st);
      VS_CUDA(cudaMemcpyAsync(y_grid, yd.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_field_dda(vs_op* op, const double* P, const double* Einc_grid, int64_t nrhs, const double* alpha, double dV,
                 const double* chi, double* E_grid, int precision) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(P && Einc_grid && alpha && chi && E_grid, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    const double a2 = alpha[0] * alpha[0] + alpha[1] * alpha[1], c2 = chi[0] * chi[0] + chi[1] * chi[1];
    VS_REQUIRE(a2 > 0 && c2 > 0, "alpha and chi must be nonzero");
    cudaStream_t st = op->ctx->stream;
    const int64_t ng = 3 * op->V * nrhs, np = op->n3 * nrhs;
    const bool c64 = precision == VS_C64;
    const double ia_re = alpha[0] / a2, ia_im = -alpha[1] / a2;  // 1/alpha
    const double2 inv_chi = make_double2(chi[0] / c2, -chi[1] / c2);
    vs::DevBuf stage, stage2, pd, pg, yd, ed, ein;
    upload_as(P, np, c64, stage, pd, st);
    ed.alloc(ng * sizeof(double2));
    if (c64) {
      pg.alloc(ng * sizeof(float2));
      yd.alloc(ng * sizeof(float2));
      vs::to_grid<float2>(*op, pd.as<float2>(), pg.as<float2>(), (int)nrhs, st);
      vs::ensure_scratch(*op, (int)nrhs, sizeof(float2));
      vs::matvec_domain<float>(*op, pg.as<float2>(), yd.as<float2>(), (int)nrhs, make_float2((float)ia_re, (float)ia_im),
                               make_float2((float)-dV, 0.f), st);
      upload_as(Einc_grid, ng, true, stage2, ein, st);
      vs::field_combine<float2>(ein.as<float2>(), yd.as<float2>(), pg.as<float2>(), inv_chi, ng, ed.as<double2>(), st);
    } else {
      pg.alloc(ng * sizeof(double2));
      yd.alloc(ng * sizeof(double2));
      vs::to_grid<double2>(*op, pd.as<double2>(), pg.as<double2>(), (int)nrhs, st);
      vs::ensure_scratch(*op, (int)nrhs, sizeof(double2));
      vs::matvec_domain<double>(*op, pg.as<double2>(), yd.as<double2>(), (int)nrhs, make_double2(ia_re, ia_im),
                                make_double2(-dV, 0.0), st);
      upload_as(Einc_grid, ng, false, stage2, ein, st);
      vs::field_combine<double2>(ein.as<double2>(), yd.as<double2>(), pg.as<double2>(), inv_chi, ng, ed.as<double2>(),
                                 st);
    }
    VS_CUDA(cudaMemcpyAsync(E_grid, ed.p, ng * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_far_field(vs_op* op, const double* P, int64_t nrhs, const double* x, const double* y, const double* z,
                 double ko, double dV, const double* dirs, int64_t ndir, double* F) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(P && x && y && z && dirs && F, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(ndir >= 1 && ndir <= (int64_t)1 << 30, "ndir must be in [1, 2^30]");
    cudaStream_t st = op->ctx->stream;
    vs::DevBuf dp, dx, dy, dz, dd, df;
    dp.alloc(op->n3 * nrhs * sizeof(double2));
    dx.alloc(op->L * sizeof(double)); dy.alloc(op->M * sizeof(double)); dz.alloc(op->N * sizeof(double));
    dd.alloc(ndir * 3 * sizeof(double));
    df.alloc(nrhs * ndir * 3 * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dp.p, P, op->n3 * nrhs * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dx.p, x, op->L * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dy.p, y, op->M * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dz.p, z, op->N * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dd.p, dirs, ndir * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
    vs::far_field_device(*op, dp.as<double2>(), (int)nrhs, dx.as<double>(), dy.as<double>(), dz.as<double>(),
                         dd.as<double>(), (int)ndir, ko, dV, df.as<double2>(), st);
    VS_CUDA(cudaMemcpyAsync(F, df.p, nrhs * ndir * 3 * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_cext(vs_op* op, const double* P, const double* Einc, double ko, double dV, double e0norm2, double* cext) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(P && Einc && cext && e0norm2 > 0, "bad argument");
    cudaStream_t st = op->ctx->stream;
    vs::DevBuf dp, de;
    dp.alloc(op->n3 * sizeof(double2));
    de.alloc(op->n3 * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(dp.p, P, op->n3 * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(de.p, Einc, op->n3 * sizeof(double2), cudaMemcpyHostToDevice, st));
    *cext = vs::cext_device(dp.as<double2>(), de.as<double2>(), op->n3, 4.0 * M_PI * ko * dV / e0norm2, st);
  });
}

int vs_cext_grad(vs_op* op, vs_prec* prec, const double* Einc, const double* eps, double ko, double d,
                 const double kvec[3], const double E0[3], const vs_solve_opts* opts, double* cext, double* grad_re,
                 double* grad_im, double* P_out, vs_solve_info* info_fwd, vs_solve_info* info_adj) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(Einc && eps && kvec && E0 && opts && cext && grad_re && grad_im && info_fwd && info_adj,
               "NULL argument");
    VS_REQUIRE(op->std3, "the gradient needs idx3 in the reference's [idx; V+idx; 2V+idx] form");
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n3, nvox = n / 3;
    vs::DevBuf de, dc, dP, dl, deps, dgr, dgi;
    de.alloc(n * sizeof(double2)); dc.alloc(n * sizeof(double2));
    dP.alloc(n * sizeof(double2)); dl.alloc(n * sizeof(double2));
    deps.alloc(nvox * sizeof(double2));
    dgr.alloc(nvox * sizeof(double)); dgi.alloc(nvox * sizeof(double));
    VS_CUDA(cudaMemcpyAsync(de.p, Einc, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(deps.p, eps, nvox * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemsetAsync(dP.p, 0, n * sizeof(double2), st));
    VS_CUDA(cudaMemsetAsync(dl.p, 0, n * sizeof(double2), st));
    vs_solve_opts o = *opts;
    o.transpose = 0;
    const auto t0 = std::chrono::steady_clock::now();
    solve_impl(op, prec, de.as<double2>(), dP.as<double2>(), &o, info_fwd);
    const auto t1 = std::chrono::steady_clock::now();
    info_fwd->time_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    vs::conj_device(de.as<double2>(), dc.as<double2>(), n, st);
    o.transpose = 1;
    solve_impl(op, prec, dc.as<double2>(), dl.as<double2>(), &o, info_adj);
    info_adj->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
    const double e2 = E0[0] * E0[0] + E0[1] * E0[1] + E0[2] * E0[2];
    const double c = 4.0 * M_PI * ko * d * d * d / e2;
    *cext = vs::cext_device(dP.as<double2>(), de.as<double2>(), n, c, st);
    const double nk = std::sqrt(kvec[0] * kvec[0] + kvec[1] * kvec[1] + kvec[2] * kvec[2]);
    const double ne = std::sqrt(e2);
    double S = 0;
    for (int j = 0; j < 3; ++j) S += (kvec[j] / nk * E0[j] / ne) * (kvec[j] / nk * E0[j] / ne);
    const double bterm = (0.1648469 + -1.7700004 * S) * (ko * d) * (ko * d);
    vs::cext_grad_device(dP.as<double2>(), dl.as<double2>(), deps.as<double2>(), nvox, c, bterm, dgr.as<double>(),
                         dgi.as<double>(), st);
    VS_CUDA(cudaMemcpyAsync(grad_re, dgr.p, nvox * sizeof(double), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaMemcpyAsync(grad_im, dgi.p, nvox * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (P_out) VS_CUDA(cudaMemcpyAsync(P_out, dP.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
  });
}

int vs_solve_batch_device(vs_op* op, vs_prec* prec, const void* b, void* x, int64_t nrhs, const vs_solve_opts* opts,
                          vs_solve_info* infos) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(b && x, "NULL argument");
    const auto t0 = std::chrono::steady_clock::now();
    solve_batch_impl(op, prec, (const double2*)b, (double2*)x, nrhs, opts, infos);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int64_t r = 0; r < nrhs; ++r) infos[r].time_ms = ms;
  });
}

int vs_solve_particles_device(int64_t nparticles, vs_op* const* ops, vs_prec* const* precs, const void* const* b,
                              void* const* x, const int64_t* nrhs, const vs_solve_opts* opts, vs_solve_info* infos) {
  if (nparticles < 1 || !ops || !b || !x || !nrhs || !opts || !infos) {
    g_last_error = "vs_solve_particles_device: NULL argument or no particles";
    return VS_ERR_ARG;
  }
  if (opts->gram) {
    g_last_error = "vs_solve_particles_device: opts->gram must be NULL (a Gram per right-hand side belongs to one particle)";
    return VS_ERR_ARG;
  }
  // particles grouped by context: one host thread per context
  std::vector<vs_ctx*> ctxs;
  std::vector<std::vector<int64_t>> groups;
  std::vector<int64_t> first(nparticles);
  int64_t off = 0;
  for (int64_t i = 0; i < nparticles; ++i) {
    if (!ops[i] || nrhs[i] < 1) {
      g_last_error = "vs_solve_particles_device: NULL operator or nrhs < 1 for particle " + std::to_string(i);
      return VS_ERR_ARG;
    }
    first[i] = off;
    off += nrhs[i];
    size_t g = 0;
    while (g < ctxs.size() && ctxs[g] != ops[i]->ctx) ++g;
    if (g == ctxs.size()) {
      ctxs.push_back(ops[i]->ctx);
      groups.emplace_back();
    }
    groups[g].push_back(i);
  }
  // a preconditioner keeps per-apply scratch, so one used by particles on two
  // contexts would be applied by two threads at once
  if (precs)
    for (int64_t i = 0; i < nparticles; ++i)
      for (int64_t j = i + 1; j < nparticles; ++j)
        if (precs[i] && precs[i] == precs[j] && ops[i]->ctx != ops[j]->ctx) {
          g_last_error = "vs_solve_particles_device: particles " + std::to_string(i) + " and " + std::to_string(j) +
                         " share a preconditioner but not a context";
          return VS_ERR_ARG;
        }
  std::vector<int> status(groups.size(), VS_OK);
  std::vector<int64_t> failed(groups.size(), -1);
  auto run_group = [&](size_t g) {
    for (int64_t i : groups[g]) {
      const int st = vs_solve_batch_device(ops[i], precs ? precs[i] : nullptr, b[i], x[i], nrhs[i], opts,
                                           infos + first[i]);
      if (st != VS_OK && status[g] == VS_OK) {
        status[g] = st;
        failed[g] = i;
      }
    }
  };
  std::vector<std::thread> threads;
  try {
    for (size_t g = 1; g < groups.size(); ++g) threads.emplace_back(run_group, g);
  } catch (const std::exception& e) {  // no thread could be started: run the rest here
    for (size_t g = threads.size() + 1; g < groups.size(); ++g) run_group(g);
  }
  run_group(0);
  for (auto& t : threads) t.join();
  for (size_t g = 0; g < groups.size(); ++g)
    if (status[g] != VS_OK) {
      g_last_error = "particle " + std::to_string(failed[g]) + ": " + ops[failed[g]]->ctx->err;
      return status[g];
    }
  return VS_OK;
}

int vs_solve_particles(int64_t nparticles, vs_op* const* ops, vs_prec* const* precs, const void* const* b,
                       void* const* x, const int64_t* nrhs, const double* const* gram, const int64_t* gram_n,
                       const vs_solve_opts* opts, vs_solve_info* infos) {
  if (nparticles < 1 || !ops || !ops[0]) {
    g_last_error = "vs_solve_particles: no particles or NULL operator";
    return VS_ERR_ARG;
  }
  vs_ctx* ctx = ops[0]->ctx;
  return guarded(ctx, [&] {
    VS_REQUIRE(b && x && nrhs && opts && infos, "vs_solve_particles: NULL argument");
    VS_REQUIRE(nparticles <= 65536, "vs_solve_particles: at most 65536 particles");
    VS_REQUIRE(opts->method == VS_BICGSTAB, "vs_solve_particles runs BiCGSTAB");
    VS_REQUIRE(opts->gram == nullptr, "vs_solve_particles takes the Gram per right-hand side in `gram`, not opts");
    VS_REQUIRE(opts->resvec == nullptr, "vs_solve_particles returns no residual history (opts->resvec must be NULL)");
    std::vector<vs::PartJob> jobs(nparticles);
    std::set<const void*> seen_op, seen_pr;
    int64_t total = 0;
    for (int64_t i = 0; i < nparticles; ++i) {
      vs_op* op = ops[i];
      VS_REQUIRE(op != nullptr, "vs_solve_particles: NULL operator for particle " + std::to_string(i));
      VS_REQUIRE(op->ctx == ctx, "vs_solve_particles: all operators must be on one context");
      VS_REQUIRE(seen_op.insert(op).second, "vs_solve_particles: an operator appears twice");
      vs_prec* pr = precs ? precs[i] : nullptr;
      if (pr) VS_REQUIRE(seen_pr.insert(pr).second, "vs_solve_particles: a preconditioner appears twice");
      VS_REQUIRE(b[i] && x[i], "vs_solve_particles: NULL b or x for particle " + std::to_string(i));
      VS_REQUIRE(nrhs[i] >= 1 && nrhs[i] <= 4096, "vs_solve_particles: nrhs must be in [1, 4096]");
      vs::SolveParams chk = solve_params(op, pr, opts);  // precision, tolerance and preconditioner checks
      (void)chk;
      const double* g = gram ? gram[i] : nullptr;
      if (g) VS_REQUIRE(gram_n && (gram_n[i] == 1 || gram_n[i] == op->V),
                        "vs_solve_particles: gram_n[i] must be 1 or L*M*N");
      jobs[i].op = op;
      jobs[i].pr = pr;
      jobs[i].b = (const double2*)b[i];
      jobs[i].x = (double2*)x[i];
      jobs[i].nrhs = (int)nrhs[i];
      jobs[i].gram = reinterpret_cast<const double2*>(g);
      jobs[i].gram_n = g ? gram_n[i] : 0;
      total += nrhs[i];
    }
    const auto t0 = std::chrono::steady_clock::now();
    vs::SolveParams prm = solve_params(ops[0], jobs[0].pr, opts);
    vs::solve_bicgstab_particles(ctx, jobs, prm, ctx->stream);
    for (auto& j : jobs) check_prec_status(j.pr);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int64_t at = 0;
    for (auto& j : jobs)
      for (auto& r : j.out) {
        fill_info(r, infos + at);
        infos[at++].time_ms = ms;
      }
    (void)total;
  });
}

int vs_solve_batch(vs_op* op, vs_prec* prec, const double* b, double* x, int64_t nrhs, const vs_solve_opts* opts,
                   vs_solve_info* infos) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(b && x, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 4096, "nrhs must be in [1, 4096]");
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n3 * nrhs;
    op->xin.alloc(n * sizeof(double2));
    op->yout.alloc(n * sizeof(double2));
    VS_CUDA(cudaMemcpyAsync(op->xin.p, b, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(op->yout.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    solve_batch_impl(op, prec, op->xin.as<double2>(), op->yout.as<double2>(), nrhs, opts, infos);
    VS_CUDA(cudaMemcpyAsync(x, op->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int64_t r = 0; r < nrhs; ++r) infos[r].time_ms = ms;
  });
}

int vs_orientation_average(vs_op* op, vs_prec* prec, const double* m, int64_t nm, const double* x, const double* y,
                           const double* z, double ko, double d, const double* dirs, const double* psi,
                           const double* weights, int64_t ndir, const vs_solve_opts* opts, double* cext_avg,
                           double* cext_each, vs_solve_info* infos) {
  if (!op) return VS_ERR_ARG;
  return guarded(op->ctx, [&] {
    VS_REQUIRE(m && x && y && z && dirs && opts && cext_avg, "NULL argument");
    VS_REQUIRE(ndir >= 1 && ndir <= (int64_t(1) << 20), "ndir must be in [1, 2^20]");
    VS_REQUIRE(op->std3, "orientation averaging needs idx3 in the [idx; V+idx; 2V+idx] form");
    VS_REQUIRE(opts->gram == nullptr, "the Gram of every direction is formed here: opts->gram must be NULL");
    VS_REQUIRE(opts->transpose == 0, "orientation averaging solves A x = b (opts->transpose must be 0)");
    VS_REQUIRE(ko > 0 && d > 0, "ko and d must be positive");
    const int64_t n = op->n3, nvox = n / 3, V = op->V;
    VS_REQUIRE(nm == 1 || nm == nvox, "m must have 1 or n3/3 entries");
    cudaStream_t st = op->ctx->stream;
    const cd* mm = reinterpret_cast<const cd*>(m);
    // grid voxel of each idx entry (the x-component unknowns), for a per-voxel m
    std::vector<int> vox;
    if (nm > 1) {
      vox.resize(nvox);
      VS_CUDA(cudaMemcpyAsync(vox.data(), op->pos2grid.p, nvox * sizeof(int), cudaMemcpyDeviceToHost, st));
      VS_CUDA(cudaStreamSynchronize(st));
    }
    std::vector<double> w(ndir, 1.0);
    double wsum = 0;
    for (int64_t j = 0; j < ndir; ++j) {
      if (weights) w[j] = weights[j];
      VS_REQUIRE(std::isfinite(w[j]) && w[j] >= 0, "weights must be finite and non-negative");
      wsum += w[j];
    }
    VS_REQUIRE(wsum > 0, "the weights sum to zero");
    vs::DevBuf dx, dy, dz;
    dx.alloc(op->L * sizeof(double)); dy.alloc(op->M * sizeof(double)); dz.alloc(op->N * sizeof(double));
    VS_CUDA(cudaMemcpyAsync(dx.p, x, op->L * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dy.p, y, op->M * sizeof(double), cudaMemcpyHostToDevice, st));
    VS_CUDA(cudaMemcpyAsync(dz.p, z, op->N * sizeof(double), cudaMemcpyHostToDevice, st));
    // directions in batches of 8 (16 right-hand sides: every pipeline launch serves all of them)
    constexpr int64_t kDirChunk = 8;
    const int64_t cap = std::min<int64_t>(ndir, kDirChunk) * 2;
    vs::DevBuf B, X;
    B.alloc(cap * n * sizeof(double2));
    X.alloc(cap * n * sizeof(double2));
    std::vector<cd> gram(nm > 1 ? cap * V : cap);
    vs::SolveParams prm = solve_params(op, prec, opts);
    const double kd = ko * d, scale = 4.0 * M_PI * ko * d * d * d;  // |E0| = 1
    double acc = 0;
    for (int64_t c0 = 0; c0 < ndir; c0 += kDirChunk) {
      const int64_t nd = std::min(kDirChunk, ndir - c0), nr = 2 * nd;
      for (int64_t j = 0; j < nd; ++j) {
        const double* dj = dirs + 3 * (c0 + j);
        const double nk = std::sqrt(dj[0] * dj[0] + dj[1] * dj[1] + dj[2] * dj[2]);
        VS_REQUIRE(nk > 0 && std::isfinite(nk), "a direction is zero or not finite");
        const double k[3] = {dj[0] / nk, dj[1] / nk, dj[2] / nk};
        double b1[3], b2[3], e[2][3];
        polarisation_basis(k, b1, b2);
        const double ps = psi ? psi[c0 + j] : 0.0;
        VS_REQUIRE(std::isfinite(ps), "psi must be finite");
        const double cp = std::cos(ps), sp = std::sin(ps);
        for (int q = 0; q < 3; ++q) {
          e[0][q] = cp * b1[q] + sp * b2[q];
          e[1][q] = -sp * b1[q] + cp * b2[q];
        }
        const double kvec[3] = {ko * k[0], ko * k[1], ko * k[2]};
        for (int pol = 0; pol < 2; ++pol) {
          const int64_t r = 2 * j + pol;
          const double2 E0[3] = {make_double2(e[pol][0], 0), make_double2(e[pol][1], 0), make_double2(e[pol][2], 0)};
          vs::plane_wave_device(*op, dx.as<double>(), dy.as<double>(), dz.as<double>(), kvec, E0,
                                B.as<double2>() + r * n, st);
          const double S = ldr_S(kvec, e[pol]);
          if (nm == 1) {
            gram[r] = 1.0 / alpha_ldr_one(mm[0], false, kd, S);
          } else {
            cd* g = gram.data() + r * V;
            std::fill(g, g + V, cd(1.0, 0.0));  // entries off the particle are never read
            for (int64_t v = 0; v < nvox; ++v) g[vox[v]] = 1.0 / alpha_ldr_one(mm[v], false, kd, S);
          }
        }
      }
      vs::SolveParams pc = prm;
      pc.gram_host = reinterpret_cast<const double2*>(gram.data());
      pc.gram_n = nm == 1 ? 1 : V;
      VS_CUDA(cudaMemsetAsync(X.p, 0, nr * n * sizeof(double2), st));
      std::vector<vs::SolveResult> res(nr);
      if (opts->method == VS_BICGSTAB) {
        vs::solve_bicgstab_batch(*op, prec, B.as<double2>(), X.as<double2>(), (int)nr, pc, res, st);
      } else {
        for (int64_t r = 0; r < nr; ++r) {
          vs::SolveParams p1 = pc;
          p1.gram_host = pc.gram_host + r * pc.gram_n;
          p1.resvec_host = nullptr;
          p1.resvec_cap = 0;
          if (opts->method == VS_GMRES)
            vs::solve_gmres(*op, prec, B.as<double2>() + r * n, X.as<double2>() + r * n, p1, res[r], st);
          else
            vs::solve_gmres_dr(*op, prec, B.as<double2>() + r * n, X.as<double2>() + r * n, p1, res[r], st);
        }
      }
      check_prec_status(prec);
      for (int64_t r = 0; r < nr; ++r) {
        const double c = vs::cext_device(X.as<double2>() + r * n, B.as<double2>() + r * n, n, scale, st);
        const int64_t j = c0 + r / 2;
        if (cext_each) cext_each[2 * j + (r & 1)] = c;
        if (infos) fill_info(res[r], infos + 2 * j + (r & 1));
        acc += w[j] * 0.5 * c;
      }
    }
    *cext_avg = acc / wsum;
  });
}

}  // extern "C"
