// C-ABI entry points (include/voxscatter.h).  Each entry validates its
// arguments, runs on the context's stream and converts exceptions into a
// status code plus a message readable through vs_last_error().
#include "vs_internal.h"
#include <complex>
#include <cstring>
#include <cmath>

namespace {

thread_local std::string g_last_error;

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
  op->map3.alloc(map3.size() * sizeof(int));
  op->pos2grid.alloc(p2g.size() * sizeof(int));
  VS_CUDA(cudaMemcpyAsync(op->map3.p, map3.data(), map3.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  VS_CUDA(cudaMemcpyAsync(op->pos2grid.p, p2g.data(), p2g.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  HostDiag mr = check_diag(Mr, V, "Mr"), mc = check_diag(Mc, V, "Mc"), gr = check_diag(Gram, V, "Gram");
  std::vector<cd> d1(n3), d1c(n3), d2(n3);
  for (int64_t e = 0; e < n3; ++e) {
    const int64_t vox = idx3[e] % V;
    d1[e] = gr.at(vox) * mr.at(vox);
    d1c[e] = gr.at(vox) * std::conj(mr.at(vox));
    d2[e] = mc.at(vox);
  }
  upload_diag(op->d1, d1, st);
  upload_diag(op->d1c, d1c, st);
  upload_diag(op->d2, d2, st);
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
  op->G64.alloc(6 * PQR * sizeof(double2));
  op->G32.alloc(6 * PQR * sizeof(float2));
  vs::finalize_spectrum(full, 6 * PQR, 1.0 / (double)PQR, op->G64.as<double2>(), op->G32.as<float2>(),
                        op->ctx->stream);
}

}  // namespace

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
  cudaStreamDestroy(ctx->stream);
  delete ctx;
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
    const double b1 = -1.8915316, b2 = 0.1648469, b3 = -1.7700004;
    const double nk = std::sqrt(kvec[0] * kvec[0] + kvec[1] * kvec[1] + kvec[2] * kvec[2]);
    const double ne = std::sqrt(E0[0] * E0[0] + E0[1] * E0[1] + E0[2] * E0[2]);
    VS_REQUIRE(nk > 0 && ne > 0, "kvec and E0 must be non-zero");
    double S = 0;
    for (int j = 0; j < 3; ++j) {
      const double t = (kvec[j] / nk) * (E0[j] / ne);
      S += t * t;
    }
    const cd* mm = reinterpret_cast<const cd*>(m);
    cd* out = reinterpret_cast<cd*>(alpha_out);
    const double kd = ko * d;
    for (int64_t e = 0; e < n; ++e) {
      const cd msqr = is_eps ? mm[e] : mm[e] * mm[e];
      const cd aCM = 3.0 / (4.0 * M_PI) * (msqr - 1.0) / (msqr + 2.0);
      out[e] = aCM / (1.0 + aCM * ((b1 + msqr * b2 + msqr * b3 * S) * kd * kd - cd(0, 2.0 / 3.0) * kd * kd * kd));
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
    if (R <= 0) R = vs::smooth_size((int)(2 * N - 1));
    check_fft_len(P, L, "P"); check_fft_len(Q, M, "Q"); check_fft_len(R, N, "R");
    op = new vs_op();
    op->ctx = ctx;
    op->L = (int)L; op->M = (int)M; op->N = (int)N;
    op->P = (int)P; op->Q = (int)Q; op->R = (int)R;
    op->V = L * M * N;
    op_common(op, idx3, n3, Mr, Mc, Gram);
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

}  // extern "C"
