// Krylov solvers on the device.
//
// BiCGSTAB (van der Vorst 1992, preconditioned form of Barrett et al. 1994)
// with MATLAB bicgstab's conventions (main_DDA.m:82,120): the preconditioner
// applies M^-1, convergence is tested on the recurrence residual at every half
// step, iter may be a half integer, resvec holds ||r|| at every half step.
// All scalars (rho, alpha, omega, norms) live in device memory and are formed
// by deterministic two-level reductions (per-CTA partials summed in a fixed
// order by the last CTA to finish) with FP64 accumulation, so one iteration is
// a fixed launch sequence that is captured once in a CUDA graph; a device
// `skip` flag turns every launch into a no-op once the iteration has converged
// or broken down, and the host polls the state once per graph launch.
//
// Mixed precision: the inner solve runs on the c64 pipeline; an outer loop
// forms the true residual r = b - A x with the c128 pipeline and compensated
// (Ogita-Rump-Oishi Dot2) FP64 norms, solves A d = r/||r|| in c64 and updates
// x += ||r|| d in FP64 until ||r||/||b|| <= tol.
#include "vs_krylov.h"

#include <chrono>
#include <cmath>
#include <vector>

namespace vs {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 2 * 152;

// FP64 double-double accumulation (TwoSum / TwoProd by fma) for the c128 path.
struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, double b) {
  const double s = a.hi + b;
  const double bb = s - a.hi;
  const double err = (a.hi - (s - bb)) + (b - bb);
  return DD{s, a.lo + err};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD r = dd_add(a, b.hi);
  r.lo += b.lo;
  return r;
}
__device__ __forceinline__ DD dd_fma(DD a, double x, double y) {
  const double p = x * y;
  const double e = fma(x, y, -p);
  DD r = dd_add(a, p);
  r.lo += e;
  return r;
}

// Accumulators: float inputs accumulate exactly-rounded products in double.
template <typename T>
struct Acc {
  double re = 0, im = 0;
  __device__ __forceinline__ void dot(cplx_t<T> u, cplx_t<T> v) {  // += conj(u) v
    re = fma((double)u.x, (double)v.x, re);
    re = fma((double)u.y, (double)v.y, re);
    im = fma((double)u.x, (double)v.y, im);
    im = fma(-(double)u.y, (double)v.x, im);
  }
  __device__ __forceinline__ void norm2(cplx_t<T> u) {
    re = fma((double)u.x, (double)u.x, re);
    re = fma((double)u.y, (double)u.y, re);
  }
  __device__ __forceinline__ double2 value() const { return make_double2(re, im); }
};
template <>
struct Acc<double> {
  DD re{0, 0}, im{0, 0};
  __device__ __forceinline__ void dot(double2 u, double2 v) {
    re = dd_fma(re, u.x, v.x);
    re = dd_fma(re, u.y, v.y);
    im = dd_fma(im, u.x, v.y);
    im = dd_fma(im, -u.y, v.x);
  }
  __device__ __forceinline__ void norm2(double2 u) {
    re = dd_fma(re, u.x, u.x);
    re = dd_fma(re, u.y, u.y);
  }
  __device__ __forceinline__ double2 value() const { return make_double2(re.hi + re.lo, im.hi + im.lo); }
};

// Block reduction of NV doubles; returns true in the last CTA to finish, with
// the grid totals in `tot` (all threads of that CTA).  Partials are summed in
// CTA order, so the result does not depend on scheduling.
template <int NV>
__device__ bool grid_reduce(double (&v)[NV], double* __restrict__ partials, unsigned* __restrict__ counter,
                            double (&tot)[NV]) {
  __shared__ double sm[NV][kRedThreads / 32];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
#pragma unroll
    for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += sm[k][w];
      partials[blockIdx.x * NV + k] = x;
    }
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) x += ((volatile double*)partials)[b * NV + k];
#pragma unroll
    for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += sm[k][w];
    tot[k] = x;
  }
  if (threadIdx.x == 0) *counter = 0;
  return true;
}

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ bool cz(double2 a) { return a.x == 0.0 && a.y == 0.0; }
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

#define GRID_LOOP(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// rho = rt^H r ; beta = (rho/rho_prev)(alpha/omega)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_rho(const cplx_t<T>* rt, const cplx_t<T>* r, int64_t n, KState* s) {
  if (s->skip) return;
  Acc<T> a;
  GRID_LOOP(i, n) a.dot(rt[i], r[i]);
  double v[2] = {a.value().x, a.value().y}, t[2];
  if (grid_reduce<2>(v, s->partials, &s->counter, t) && threadIdx.x == 0) {
    const double2 rho = make_double2(t[0], t[1]);
    if (cz(rho) || !cfinite(rho)) {
      s->flag = cfinite(rho) ? 4 : 5;
      s->skip = 1;
      return;
    }
    if (s->iter2 > 0) s->beta = cmul(cdiv(rho, s->rho_prev), cdiv(s->alpha, s->omega));
    s->rho = rho;
  }
}

// p = r (first iteration) or r + beta (p - omega v)
template <typename T>
__global__ void k_bicg_p(cplx_t<T>* p, const cplx_t<T>* r, const cplx_t<T>* v, int64_t n, const KState* s) {
  using C = cplx_t<T>;
  if (s->skip) return;
  if (s->iter2 == 0) {
    GRID_LOOP(i, n) p[i] = r[i];
    return;
  }
  const C beta = ccast<C>(s->beta), om = ccast<C>(s->omega);
  GRID_LOOP(i, n) p[i] = cfma(beta, csub(p[i], cmul(om, v[i])), r[i]);
}

// alpha = rho / (rt^H v)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_alpha(const cplx_t<T>* rt, const cplx_t<T>* v, int64_t n, KState* s) {
  if (s->skip) return;
  Acc<T> a;
  GRID_LOOP(i, n) a.dot(rt[i], v[i]);
  double w[2] = {a.value().x, a.value().y}, t[2];
  if (grid_reduce<2>(w, s->partials, &s->counter, t) && threadIdx.x == 0) {
    const double2 d = make_double2(t[0], t[1]);
    if (cz(d) || !cfinite(d)) {
      s->flag = cfinite(d) ? 4 : 5;
      s->skip = 1;
      return;
    }
    s->alpha = cdiv(s->rho, d);
  }
}

// s = r - alpha v ; ||s|| ; half-step convergence test
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_s(cplx_t<T>* sv, const cplx_t<T>* r, const cplx_t<T>* v, int64_t n, KState* s) {
  using C = cplx_t<T>;
  if (s->skip) return;
  const C al = ccast<C>(s->alpha);
  Acc<T> a;
  GRID_LOOP(i, n) {
    const C x = csub(r[i], cmul(al, v[i]));
    sv[i] = x;
    a.norm2(x);
  }
  double w[1] = {a.value().x}, t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) {
    const double res = sqrt(t[0]);
    const int k = s->iter2 + 1;
    if (k < s->resvec_cap) s->resvec[k] = res * s->res_scale;
    s->nres = k + 1;
    s->res = res;
    if (!isfinite(res)) {
      s->flag = 5;
      s->skip = 1;
    } else if (res <= s->tol_abs) {
      s->half_pending = 1;
      s->flag = 0;
      s->iter2 = k;
      s->skip = 1;
    }
  }
}

// x += alpha ph when the half step converged (runs regardless of skip).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_xhalf(cplx_t<T>* x, const cplx_t<T>* ph, int64_t n, KState* s) {
  using C = cplx_t<T>;
  __shared__ int s_go;
  __shared__ bool s_last;
  if (threadIdx.x == 0) s_go = s->half_pending;
  __syncthreads();
  if (!s_go) return;
  const C al = ccast<C>(s->alpha);
  GRID_LOOP(i, n) x[i] = cfma(al, ph[i], x[i]);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(&s->counter, 1u);
    s_last = (t == gridDim.x - 1);
    if (s_last) {
      s->half_pending = 0;
      s->counter = 0;
    }
  }
}

// omega = (t^H s)/(t^H t)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_omega(const cplx_t<T>* t, const cplx_t<T>* sv, int64_t n, KState* s) {
  if (s->skip) return;
  Acc<T> a, b;
  GRID_LOOP(i, n) {
    a.dot(t[i], sv[i]);
    b.norm2(t[i]);
  }
  double w[3] = {a.value().x, a.value().y, b.value().x}, tt[3];
  if (grid_reduce<3>(w, s->partials, &s->counter, tt) && threadIdx.x == 0) {
    const double2 ts = make_double2(tt[0], tt[1]);
    const double t2 = tt[2];
    if (!(t2 > 0) || !cfinite(ts)) {
      s->flag = (t2 == 0) ? 4 : 5;
      s->skip = 1;
      return;
    }
    const double2 om = make_double2(ts.x / t2, ts.y / t2);
    if (cz(om)) {
      s->flag = 4;
      s->skip = 1;
      return;
    }
    s->omega = om;
  }
}

// x += alpha ph + omega sh ; r = s - omega t ; ||r|| ; full-step test
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_xr(cplx_t<T>* x, cplx_t<T>* r, const cplx_t<T>* ph, const cplx_t<T>* sh,
                                                        const cplx_t<T>* sv, const cplx_t<T>* t, int64_t n, KState* s) {
  using C = cplx_t<T>;
  if (s->skip) return;
  const C al = ccast<C>(s->alpha), om = ccast<C>(s->omega);
  Acc<T> a;
  GRID_LOOP(i, n) {
    x[i] = cfma(om, sh[i], cfma(al, ph[i], x[i]));
    const C ri = csub(sv[i], cmul(om, t[i]));
    r[i] = ri;
    a.norm2(ri);
  }
  double w[1] = {a.value().x}, tt[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, tt) && threadIdx.x == 0) {
    const double res = sqrt(tt[0]);
    const int k = s->iter2 + 2;
    if (k < s->resvec_cap) s->resvec[k] = res * s->res_scale;
    s->nres = k + 1;
    s->iter2 = k;
    s->res = res;
    s->rho_prev = s->rho;
    if (res < 0.99 * s->best_res) {
      s->best_res = res;
      s->best_iter2 = k;
    }
    if (!isfinite(res)) {
      s->flag = 5;
      s->skip = 1;
    } else if (res <= s->tol_abs) {
      s->flag = 0;
      s->skip = 1;
    } else if (k >= 2 * s->maxit) {
      s->flag = 1;
      s->skip = 1;
    } else if (s->stag_window > 0 && k - s->best_iter2 >= 2 * s->stag_window) {
      s->flag = 3;  // stagnated (MATLAB flag 3)
      s->skip = 1;
    }
  }
}

// ||u||^2 into s->aux (and u^H v optional) -- used for the initial residual.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_norm(const cplx_t<T>* u, int64_t n, KState* s, double* out) {
  Acc<T> a;
  GRID_LOOP(i, n) a.norm2(u[i]);
  double w[1] = {a.value().x}, t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) *out = sqrt(t[0]);
}

template <typename T>
__global__ void k_copy(cplx_t<T>* dst, const cplx_t<T>* src, int64_t n) {
  GRID_LOOP(i, n) dst[i] = src[i];
}
template <typename T>
__global__ void k_zero(cplx_t<T>* dst, int64_t n) {
  GRID_LOOP(i, n) dst[i] = czero<cplx_t<T>>();
}

// r64 = b - y64 and its compensated norm
__global__ void __launch_bounds__(kRedThreads) k_resid64(const double2* b, const double2* y, double2* r, int64_t n, KState* s,
                                                        double* out) {
  Acc<double> a;
  GRID_LOOP(i, n) {
    const double2 v = csub(b[i], y[i]);
    r[i] = v;
    a.norm2(v);
  }
  double w[1] = {a.value().x}, t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) *out = sqrt(t[0]);
}

// r32 = r64 * sc
__global__ void k_scale_down(const double2* r, float2* o, int64_t n, double sc) {
  GRID_LOOP(i, n) o[i] = make_float2((float)(r[i].x * sc), (float)(r[i].y * sc));
}
// x64 += sc * d32
__global__ void k_update64(double2* x, const float2* d, int64_t n, double sc) {
  GRID_LOOP(i, n) {
    x[i].x = fma(sc, (double)d[i].x, x[i].x);
    x[i].y = fma(sc, (double)d[i].y, x[i].y);
  }
}

// Inner (c64) solves stop when the residual has not improved by 1% for this
// many iterations: the c64 recurrence has reached its floor and the FP64
// refinement takes over.
constexpr int kStagnationWindow = 8;

static int vec_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), kRedBlocks)); }

// ---- host driver ---------------------------------------------------------

template <typename T>
void KrylovWork::ensure(int64_t n) {
  using C = cplx_t<T>;
  const size_t b = n * sizeof(C);
  DevBuf* v[] = {&r, &rt, &p, &v_, &s, &t, &ph, &sh, &x};
  for (DevBuf* d : v) d->alloc(b);
}

static void upload_state(KState* d, const KState& h, cudaStream_t st) {
  VS_CUDA(cudaMemcpyAsync(d, &h, sizeof(KState), cudaMemcpyHostToDevice, st));
}

// One BiCGSTAB iteration (two half steps) as a fixed launch sequence.
template <typename T>
static void bicg_iteration(const vs_op& op, const vs_prec* pr, KrylovWork& w, KState* s, int64_t n, int mode,
                           cudaStream_t st) {
  using C = cplx_t<T>;
  C* r = w.r.as<C>();
  C* rt = w.rt.as<C>();
  C* p = w.p.as<C>();
  C* v = w.v_.as<C>();
  C* sv = w.s.as<C>();
  C* t = w.t.as<C>();
  C* ph = w.ph.as<C>();
  C* sh = w.sh.as<C>();
  C* x = w.x.as<C>();
  const int g = vec_grid(n);
  const int* skip = &s->skip;
  k_bicg_rho<T><<<g, kRedThreads, 0, st>>>(rt, r, n, s);
  k_bicg_p<T><<<g, 256, 0, st>>>(p, r, v, n, s);
  if (pr) prec_apply<T>(*pr, p, ph, 1, skip, st);
  else k_copy<T><<<g, 256, 0, st>>>(ph, p, n);
  matvec<T>(op, ph, v, 1, mode, skip, st);
  k_bicg_alpha<T><<<g, kRedThreads, 0, st>>>(rt, v, n, s);
  k_bicg_s<T><<<g, kRedThreads, 0, st>>>(sv, r, v, n, s);
  k_bicg_xhalf<T><<<g, kRedThreads, 0, st>>>(x, ph, n, s);
  if (pr) prec_apply<T>(*pr, sv, sh, 1, skip, st);
  else k_copy<T><<<g, 256, 0, st>>>(sh, sv, n);
  matvec<T>(op, sh, t, 1, mode, skip, st);
  k_bicg_omega<T><<<g, kRedThreads, 0, st>>>(t, sv, n, s);
  k_bicg_xr<T><<<g, kRedThreads, 0, st>>>(x, r, ph, sh, sv, t, n, s);
  VS_LAUNCH_CHECK();
}

// Kernels in one bicg_iteration: 7 solver kernels, 2 matvecs of 5 passes, and
// 2 preconditioner applies of 5 passes (or 2 copies without preconditioner).
static int kernels_per_iteration(const vs_prec* pr) { return 7 + 10 + (pr ? 10 : 2); }

// Runs BiCGSTAB on w.x (initial guess already there) for A x = w.r0-based
// system: the caller has put the initial residual in w.r.  Returns the final
// state.  Iterations are launched as a CUDA graph of `per_graph` iterations.
template <typename T>
static KState bicgstab_core(const vs_op& op, const vs_prec* pr, KrylovWork& w, int64_t n, double bnorm, double tol,
                            int maxit, double res_scale, double* resvec_dev, int resvec_cap, int per_graph,
                            cudaStream_t st, int64_t* launches, int stag_window, int mode) {
  using C = cplx_t<T>;
  KState h{};
  h.tol_abs = tol * bnorm;
  h.maxit = maxit;
  h.res_scale = res_scale;
  h.resvec = resvec_dev;
  h.resvec_cap = resvec_cap;
  h.partials = w.partials.as<double>();
  h.flag = 1;
  h.stag_window = stag_window;
  h.best_res = INFINITY;
  KState* s = w.state.as<KState>();
  // r0 norm
  upload_state(s, h, st);
  const int g = vec_grid(n);
  k_copy<T><<<g, 256, 0, st>>>(w.rt.as<C>(), w.r.as<C>(), n);
  k_norm<T><<<g, kRedThreads, 0, st>>>(w.r.as<C>(), n, s, w.scal.as<double>());
  *launches += 2;
  double r0 = 0;
  VS_CUDA(cudaMemcpyAsync(&r0, w.scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  if (resvec_dev && resvec_cap > 0) {
    const double v0 = r0 * res_scale;
    VS_CUDA(cudaMemcpyAsync(resvec_dev, &v0, sizeof(double), cudaMemcpyHostToDevice, st));
  }
  h.res = r0;
  h.nres = 1;
  if (!(r0 > h.tol_abs) || maxit <= 0) {
    h.flag = (r0 <= h.tol_abs) ? 0 : 1;
    return h;
  }
  h.best_res = r0;
  // The iteration graph depends only on the buffers, the preconditioner and
  // the graph length (scalars live in the device state), so it is captured
  // once and reused by later solves on this operator.
  GraphCache& gc = std::is_same<T, float>::value ? w.graph32 : w.graph64;
  std::vector<const void*> key = {w.r.p, w.rt.p, w.p.p, w.v_.p, w.s.p, w.t.p, w.ph.p, w.sh.p, w.x.p,
                                  w.state.p, w.partials.p, op.t1.p, op.t2.p,
                                  (const void*)(uintptr_t)(pr ? pr->id : 0), pr ? pr->t.p : nullptr,
                                  (const void*)(uintptr_t)per_graph, (const void*)(uintptr_t)mode};
  if (gc.exec == nullptr || gc.key != key) {
    gc.reset();
    // One launch sequence with skip set, outside capture: every kernel returns
    // at once, but first-use attribute calls happen here rather than in the
    // capture.
    KState idle = h;
    idle.skip = 1;
    upload_state(s, idle, st);
    bicg_iteration<T>(op, pr, w, s, n, mode, st);
    *launches += kernels_per_iteration(pr);
    cudaGraph_t graph = nullptr;
    VS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      for (int k = 0; k < per_graph; ++k) bicg_iteration<T>(op, pr, w, s, n, mode, st);
    } catch (...) {
      cudaStreamEndCapture(st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    VS_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&gc.exec, graph, 0);
    cudaGraphDestroy(graph);
    VS_CUDA(e);
    gc.key = key;
  }
  upload_state(s, h, st);
  KState cur{};
  const int max_launch = (maxit + per_graph - 1) / per_graph + 1;
  for (int it = 0; it < max_launch; ++it) {
    VS_CUDA(cudaGraphLaunch(gc.exec, st));
    *launches += (int64_t)per_graph * kernels_per_iteration(pr);
    VS_CUDA(cudaMemcpyAsync(&cur, s, sizeof(KState), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    if (cur.skip) break;
  }
  if (!cur.skip) cur.flag = 1;
  return cur;
}

static double norm64(KrylovWork& w, const double2* u, int64_t n, cudaStream_t st, int64_t* launches) {
  *launches += 1;
  KState* s = w.state.as<KState>();
  k_norm<double><<<vec_grid(n), kRedThreads, 0, st>>>(u, n, s, w.scal.as<double>());
  VS_LAUNCH_CHECK();
  double h = 0;
  VS_CUDA(cudaMemcpyAsync(&h, w.scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  return h;
}

// r64 = b - A x64 (c128 pipeline); returns ||r64||.
static double residual64(const vs_op& op, KrylovWork& w, const double2* b, const double2* x, double2* r, int64_t n,
                         cudaStream_t st, int64_t* launches, int mode) {
  *launches += 6;
  KState* s = w.state.as<KState>();
  double2* y = w.y64.as<double2>();
  matvec<double>(op, x, y, 1, mode, nullptr, st);
  k_resid64<<<vec_grid(n), kRedThreads, 0, st>>>(b, y, r, n, s, w.scal.as<double>());
  VS_LAUNCH_CHECK();
  double h = 0;
  VS_CUDA(cudaMemcpyAsync(&h, w.scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  return h;
}

void solve_bicgstab(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                    cudaStream_t st) {
  const int64_t n = op.n3;
  KrylovWork& w = op.kw;
  w.partials.alloc(kRedBlocks * 4 * sizeof(double));
  w.state.alloc(sizeof(KState));
  w.scal.alloc(4 * sizeof(double));
  VS_CUDA(cudaMemsetAsync(w.partials.p, 0, kRedBlocks * 4 * sizeof(double), st));
  KState zero{};
  zero.partials = w.partials.as<double>();  // every reduction needs its partial-sum buffer
  upload_state(w.state.as<KState>(), zero, st);
  const int cap = prm.resvec_cap;
  w.resvec.alloc(std::max(1, cap) * sizeof(double));
  double* rv = cap > 0 ? w.resvec.as<double>() : nullptr;
  ensure_scratch(op, 1, sizeof(double2));
  int64_t launches = 0;
  const double bnorm = norm64(w, b, n, st, &launches);
  if (!std::isfinite(bnorm)) throw Error(VS_ERR_NONFINITE, "right-hand side has NaN or Inf entries");
  out = SolveResult{};
  if (bnorm == 0) {
    VS_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double2), st));
    VS_CUDA(cudaStreamSynchronize(st));
    out.flag = 0;
    return;
  }
  if (prm.mode == VS_SOLVE_FP64) {
    w.ensure<double>(n);
    w.y64.alloc(n * sizeof(double2));
    // x0 -> w.x ; r = b - A x0
    k_copy<double><<<vec_grid(n), 256, 0, st>>>(w.x.as<double2>(), x, n);
    if (norm64(w, x, n, st, &launches) == 0.0) {  // x0 = 0: r = b exactly, no matvec
      k_copy<double><<<vec_grid(n), 256, 0, st>>>(w.r.as<double2>(), b, n);
      VS_LAUNCH_CHECK();
      launches += 1;
    } else {
      residual64(op, w, b, x, w.r.as<double2>(), n, st, &launches, prm.op_mode);
    }
    launches += 1;
    KState fs = bicgstab_core<double>(op, pr, w, n, bnorm, prm.tol, prm.maxit, 1.0 / bnorm, rv, cap, prm.per_graph, st,
                                      &launches, 0, prm.op_mode);
    launches += 1;
    k_copy<double><<<vec_grid(n), 256, 0, st>>>(x, w.x.as<double2>(), n);
    VS_LAUNCH_CHECK();
    out.flag = fs.flag;
    out.iter = fs.iter2 * 0.5;
    out.inner_iters = fs.iter2 * 0.5;
    out.n_resvec = std::min<int64_t>(fs.nres, cap);
    const double rn = residual64(op, w, b, x, w.r.as<double2>(), n, st, &launches, prm.op_mode);
    out.relres = rn / bnorm;
    if (out.flag == 0 && out.relres > prm.tol) out.flag = 1;
  } else {
    // mixed: c64 inner BiCGSTAB inside FP64 refinement
    w.ensure<float>(n);
    w.y64.alloc(n * sizeof(double2));
    w.r64.alloc(n * sizeof(double2));
    double2* r64 = w.r64.as<double2>();
    double rn;
    if (norm64(w, x, n, st, &launches) == 0.0) {  // x0 = 0: r = b exactly, no matvec
      k_copy<double><<<vec_grid(n), 256, 0, st>>>(r64, b, n);
      VS_LAUNCH_CHECK();
      launches += 1;
      rn = bnorm;
    } else {
      rn = residual64(op, w, b, x, r64, n, st, &launches, prm.op_mode);
    }
    int inner_total2 = 0;
    int64_t nres = 0;
    int flag = 1;
    int refine = 0;
    for (; refine <= prm.max_refine; ++refine) {
      if (rn <= prm.tol * bnorm) {
        flag = 0;
        break;
      }
      if (refine == prm.max_refine || inner_total2 >= 2 * prm.maxit) break;
      // Aim one inner solve at the whole remaining reduction (with margin for
      // the c64 rounding of the operator), but not below what c64 can reach.
      double itol = prm.inner_tol > 0 ? prm.inner_tol : std::max(0.3 * prm.tol * bnorm / rn, prm.inner_floor);
      itol = std::min(itol, 0.5);
      k_scale_down<<<vec_grid(n), 256, 0, st>>>(r64, w.r.as<float2>(), n, 1.0 / rn);
      k_zero<float><<<vec_grid(n), 256, 0, st>>>(w.x.as<float2>(), n);
      VS_LAUNCH_CHECK();
      double* rvk = (rv && nres < cap) ? rv + nres : nullptr;
      const int capk = rv ? (int)(cap - nres) : 0;
      KState fs = bicgstab_core<float>(op, pr, w, n, 1.0, itol, prm.maxit - inner_total2 / 2, rn / bnorm, rvk, capk,
                                       prm.per_graph, st, &launches, kStagnationWindow, prm.op_mode);
      launches += 2;
      inner_total2 += fs.iter2;
      nres += std::min<int64_t>(fs.nres, capk);
      if (fs.flag >= 4 && fs.iter2 == 0) {
        flag = fs.flag;
        break;
      }
      k_update64<<<vec_grid(n), 256, 0, st>>>(x, w.x.as<float2>(), n, rn);
      VS_LAUNCH_CHECK();
      launches += 1;
      rn = residual64(op, w, b, x, r64, n, st, &launches, prm.op_mode);
    }
    out.flag = (rn <= prm.tol * bnorm) ? 0 : (flag >= 4 ? flag : 1);
    out.relres = rn / bnorm;
    out.iter = inner_total2 * 0.5;
    out.inner_iters = inner_total2 * 0.5;
    out.refinements = refine;
    out.n_resvec = nres;
  }
  out.launches = launches;
  if (cap > 0 && prm.resvec_host && out.n_resvec > 0)
    VS_CUDA(cudaMemcpyAsync(prm.resvec_host, rv, out.n_resvec * sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace vs

// ===========================================================================
// GMRES(m), left preconditioned as MATLAB's gmres(A, b, restart, tol, maxit, M1)
// (main_DDA.m:89,128-129; Saad & Schultz 1986): Arnoldi with classical
// Gram-Schmidt and one reorthogonalisation pass (two batched dot/axpy passes
// per step), Givens rotations and the small triangular solve on the device.
// Convergence is tested on the preconditioned residual estimate |g_{k+1}|
// relative to ||M^-1 r0||.  It runs as the inner solver of the FP64 refinement
// loop below (c64 or c128 pipeline), so the reported relres is always the
// true FP64 residual.
// ===========================================================================
namespace vs {

constexpr int kDotChunk = 4096;  // elements per CTA of the batched dots

template <typename T>
__global__ void __launch_bounds__(256) k_gm_dots(const cplx_t<T>* __restrict__ V, const cplx_t<T>* __restrict__ w,
                                                 int64_t n, double2* __restrict__ part, int nchunk,
                                                 const GState* st) {
  if (st->skip) return;
  const int j = blockIdx.y;
  const cplx_t<T>* v = V + (int64_t)j * n;
  const int64_t i0 = (int64_t)blockIdx.x * kDotChunk;
  const int64_t i1 = (n < i0 + kDotChunk) ? n : i0 + kDotChunk;
  Acc<T> a;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) a.dot(v[i], w[i]);
  __shared__ double sre[8], sim[8];
  double re = a.value().x, im = a.value().y;
  for (int off = 16; off; off >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, off);
    im += __shfl_xor_sync(0xffffffffu, im, off);
  }
  if ((threadIdx.x & 31) == 0) { sre[threadIdx.x >> 5] = re; sim[threadIdx.x >> 5] = im; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0, q = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { r += sre[k]; q += sim[k]; }
    part[(int64_t)j * nchunk + blockIdx.x] = make_double2(r, q);
  }
}

// hp[j] = sum of the partials of vector j; H(:,k) += hp (column k of the Hessenberg)
__global__ void k_gm_dots_final(const double2* __restrict__ part, int nchunk, double2* __restrict__ hp,
                                double2* __restrict__ Hcol, GState* st) {
  if (st->skip) return;
  const int j = blockIdx.x;
  double r = 0, q = 0;
  for (int c = threadIdx.x; c < nchunk; c += blockDim.x) { r += part[(int64_t)j * nchunk + c].x; q += part[(int64_t)j * nchunk + c].y; }
  for (int off = 16; off; off >>= 1) {
    r += __shfl_xor_sync(0xffffffffu, r, off);
    q += __shfl_xor_sync(0xffffffffu, q, off);
  }
  __shared__ double sr[8], sq[8];
  if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = r; sq[threadIdx.x >> 5] = q; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += sr[k]; b += sq[k]; }
    hp[j] = make_double2(a, b);
    Hcol[j].x += a;
    Hcol[j].y += b;
  }
}

// w -= sum_j hp[j] V_j
template <typename T>
__global__ void k_gm_axpy(const cplx_t<T>* __restrict__ V, cplx_t<T>* __restrict__ w, int64_t n, int kk,
                          const double2* __restrict__ hp, const GState* st) {
  using C = cplx_t<T>;
  if (st->skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* h = reinterpret_cast<C*>(smem_raw);
  for (int j = threadIdx.x; j < kk; j += blockDim.x) h[j] = ccast<C>(hp[j]);
  __syncthreads();
  GRID_LOOP(i, n) {
    C acc = w[i];
    for (int j = 0; j < kk; ++j) {
      const C v = V[(int64_t)j * n + i];
      acc = csub(acc, cmul(h[j], v));
    }
    w[i] = acc;
  }
}

// H(k+1,k) = ||w|| (grid reduction; the last CTA writes it)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_gm_norm(const cplx_t<T>* w, int64_t n, double* partials,
                                                         unsigned* counter, double2* Hk1, const GState* st) {
  if (st->skip) return;
  Acc<T> a;
  GRID_LOOP(i, n) a.norm2(w[i]);
  double v[1] = {a.value().x}, t[1];
  if (grid_reduce<1>(v, partials, counter, t) && threadIdx.x == 0) *Hk1 = make_double2(sqrt(t[0]), 0.0);
}

// V_{k+1} = w / H(k+1,k)
template <typename T>
__global__ void k_gm_scale(const cplx_t<T>* __restrict__ w, cplx_t<T>* __restrict__ vnext, int64_t n,
                           const double2* Hk1, const GState* st) {
  if (st->skip) return;
  const double h = Hk1->x;
  const T s = (T)(h > 0 ? 1.0 / h : 0.0);
  GRID_LOOP(i, n) vnext[i] = cscale(w[i], s);
}

// Apply the previous rotations to column k, form rotation k, update g and the
// residual estimate (one thread).
__global__ void k_gm_givens(GState* st, double2* H, double* cs, double2* sn, double2* g) {
  if (st->skip || threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = st->k, m1 = st->m + 1;
  double2* h = H + (int64_t)k * m1;
  for (int j = 0; j < k; ++j) {
    const double2 a = h[j], b = h[j + 1];
    // [c s; -conj(s) c] [a; b]
    const double2 t = cadd(cscale(a, cs[j]), cmul(sn[j], b));
    const double2 u = csub(cscale(b, cs[j]), cmul(cconj(sn[j]), a));
    h[j] = t;
    h[j + 1] = u;
  }
  const double2 a = h[k], b = h[k + 1];
  const double na = sqrt(a.x * a.x + a.y * a.y), nb = sqrt(b.x * b.x + b.y * b.y);
  const double den = sqrt(na * na + nb * nb);
  double c;
  double2 s;
  if (na == 0.0) {
    c = 0.0;
    s = make_double2(1.0, 0.0);
  } else {
    c = na / den;
    s = cscale(cmul(make_double2(a.x / na, a.y / na), cconj(b)), 1.0 / den);
  }
  cs[k] = c;
  sn[k] = s;
  h[k] = cadd(cscale(a, c), cmul(s, b));
  h[k + 1] = make_double2(0, 0);
  const double2 gk = g[k];
  g[k + 1] = cscale(cmul(cconj(s), gk), -1.0);
  g[k] = cscale(gk, c);
  const double res = sqrt(g[k + 1].x * g[k + 1].x + g[k + 1].y * g[k + 1].y);
  st->res = res;
  st->k = k + 1;
  if (st->nres < st->resvec_cap) st->resvec[st->nres] = res * st->res_scale;
  st->nres += 1;
  if (!isfinite(res)) {
    st->flag = 5;
    st->skip = 1;
  } else if (res <= st->tol_abs) {
    st->flag = 0;
    st->skip = 1;
  } else if (st->k >= st->m) {
    st->skip = 1;  // cycle complete; the host restarts
  }
}

// Back substitution H(0:k,0:k) y = g(0:k) (upper triangular after the rotations).
__global__ void k_gm_solve(const GState* st, const double2* H, const double2* g, double2* y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = st->k, m1 = st->m + 1;
  for (int i = k - 1; i >= 0; --i) {
    double2 acc = g[i];
    for (int j = i + 1; j < k; ++j) acc = csub(acc, cmul(H[(int64_t)j * m1 + i], y[j]));
    const double2 d = H[(int64_t)i * m1 + i];
    const double dd = d.x * d.x + d.y * d.y;
    y[i] = dd > 0 ? make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd)
                  : make_double2(0, 0);
  }
}

// d += sum_j y[j] V_j
template <typename T>
__global__ void k_gm_xupdate(cplx_t<T>* __restrict__ d, const cplx_t<T>* __restrict__ V, int64_t n, int k,
                             const double2* __restrict__ y) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* ys = reinterpret_cast<C*>(smem_raw);
  for (int j = threadIdx.x; j < k; j += blockDim.x) ys[j] = ccast<C>(y[j]);
  __syncthreads();
  GRID_LOOP(i, n) {
    C acc = d[i];
    for (int j = 0; j < k; ++j) acc = cfma(ys[j], V[(int64_t)j * n + i], acc);
    d[i] = acc;
  }
}

// r - A d  (T precision), into out
template <typename T>
__global__ void k_sub(const cplx_t<T>* __restrict__ a, const cplx_t<T>* __restrict__ b, cplx_t<T>* __restrict__ o,
                      int64_t n) {
  GRID_LOOP(i, n) o[i] = csub(a[i], b[i]);
}

template <typename T>
__global__ void k_scale_by(const cplx_t<T>* __restrict__ a, cplx_t<T>* __restrict__ o, int64_t n, const double* nrm) {
  const double h = *nrm;
  const T s = (T)(h > 0 ? 1.0 / h : 0.0);
  GRID_LOOP(i, n) o[i] = cscale(a[i], s);
}

__global__ void k_r64_to(const double2* r, float2* o, int64_t n, double sc) {
  GRID_LOOP(i, n) o[i] = make_float2((float)(r[i].x * sc), (float)(r[i].y * sc));
}
__global__ void k_r64_to(const double2* r, double2* o, int64_t n, double sc) {
  GRID_LOOP(i, n) o[i] = make_double2(r[i].x * sc, r[i].y * sc);
}
__global__ void k_update64_from(double2* x, const float2* d, int64_t n, double sc) {
  GRID_LOOP(i, n) {
    x[i].x = fma(sc, (double)d[i].x, x[i].x);
    x[i].y = fma(sc, (double)d[i].y, x[i].y);
  }
}
__global__ void k_update64_from(double2* x, const double2* d, int64_t n, double sc) {
  GRID_LOOP(i, n) {
    x[i].x = fma(sc, d[i].x, x[i].x);
    x[i].y = fma(sc, d[i].y, x[i].y);
  }
}

// Inner GMRES on A d = rin (rin, d in precision T; d starts at 0).  Returns
// the number of Arnoldi steps and sets *flag (0 converged, 1 not).
template <typename T>
static int gmres_core(const vs_op& op, const vs_prec* pr, KrylovWork& w, int64_t n, const cplx_t<T>* rin,
                      cplx_t<T>* d, double itol, int m, int maxit, int op_mode, double res_scale, double* resvec_dev,
                      int resvec_cap, int64_t* nres_out, int* flag, cudaStream_t st, int64_t* launches) {
  using C = cplx_t<T>;
  const int g = vec_grid(n);
  const int nchunk = ceil_div(n, kDotChunk);
  C* V = w.gV.as<C>();
  C* wv = w.gw.as<C>();
  C* tmp = w.gtmp.as<C>();
  double2* H = w.gH.as<double2>();
  double2* hp = w.ghp.as<double2>();
  double2* part = w.gpart.as<double2>();
  GState* gs = w.gstate.as<GState>();
  KState* ks = w.state.as<KState>();
  auto minv = [&](const C* in, C* out) {
    if (pr) prec_apply<T>(*pr, in, out, 1, &gs->skip, st);
    else k_copy<T><<<g, 256, 0, st>>>(out, in, n);
    *launches += pr ? 5 : 1;
  };
  VS_CUDA(cudaMemsetAsync(d, 0, n * sizeof(C), st));
  GState h{};
  h.m = m;
  h.resvec = resvec_dev;
  h.resvec_cap = resvec_cap;
  h.res_scale = res_scale;
  int steps = 0;
  *flag = 1;
  double beta0 = -1;
  int64_t nres = 0;
  for (int cycle = 0; steps < maxit; ++cycle) {
    // z = M^-1 (rin - A d) into V_0 (un-normalised), beta = ||z||
    h.skip = 0;
    VS_CUDA(cudaMemcpyAsync(gs, &h, sizeof(GState), cudaMemcpyHostToDevice, st));
    if (cycle == 0) {
      minv(rin, V);
    } else {
      matvec<T>(op, d, tmp, 1, op_mode, nullptr, st);
      k_sub<T><<<g, 256, 0, st>>>(rin, tmp, tmp, n);
      minv(tmp, V);
      *launches += 6;
    }
    k_norm<T><<<g, kRedThreads, 0, st>>>(V, n, ks, w.scal.as<double>());
    double beta = 0;
    VS_CUDA(cudaMemcpyAsync(&beta, w.scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    *launches += 1;
    if (beta0 < 0) {
      beta0 = beta;
      h.tol_abs = itol * beta0;
      if (resvec_dev && resvec_cap > 0) {
        const double v0 = beta * res_scale;
        VS_CUDA(cudaMemcpyAsync(resvec_dev, &v0, sizeof(double), cudaMemcpyHostToDevice, st));
      }
      nres = 1;
    }
    if (!(beta > h.tol_abs)) {
      *flag = 0;
      break;
    }
    k_scale_by<T><<<g, 256, 0, st>>>(V, V, n, w.scal.as<double>());
    // fresh Hessenberg and g = [beta, 0, ...]
    VS_CUDA(cudaMemsetAsync(H, 0, (size_t)(m + 1) * m * sizeof(double2), st));
    VS_CUDA(cudaMemsetAsync(w.gg.p, 0, (m + 1) * sizeof(double2), st));
    const double2 g0 = make_double2(beta, 0);
    VS_CUDA(cudaMemcpyAsync(w.gg.p, &g0, sizeof(double2), cudaMemcpyHostToDevice, st));
    h.k = 0;
    h.skip = 0;
    h.flag = 1;
    h.res = beta;
    h.nres = (int)nres;
    VS_CUDA(cudaMemcpyAsync(gs, &h, sizeof(GState), cudaMemcpyHostToDevice, st));
    *launches += 1;
    const int kmax = std::min(m, maxit - steps);
    GState cur{};
    int issued = 0;
    for (int k = 0; k < kmax; ++k) {
      const C* vk = V + (int64_t)k * n;
      matvec<T>(op, vk, tmp, 1, op_mode, &gs->skip, st);
      minv(tmp, wv);
      double2* Hcol = H + (int64_t)k * (m + 1);
      for (int pass = 0; pass < 2; ++pass) {
        k_gm_dots<T><<<dim3(nchunk, k + 1), 256, 0, st>>>(V, wv, n, part, nchunk, gs);
        k_gm_dots_final<<<k + 1, 256, 0, st>>>(part, nchunk, hp, Hcol, gs);
        k_gm_axpy<T><<<g, 256, (k + 1) * sizeof(C), st>>>(V, wv, n, k + 1, hp, gs);
      }
      // partial sums and counter of the shared reduction state (device addresses)
      k_gm_norm<T><<<g, kRedThreads, 0, st>>>(wv, n, w.partials.as<double>(), &ks->counter, Hcol + k + 1, gs);
      k_gm_scale<T><<<g, 256, 0, st>>>(wv, V + (int64_t)(k + 1) * n, n, Hcol + k + 1, gs);
      k_gm_givens<<<1, 32, 0, st>>>(gs, H, w.gcs.as<double>(), w.gsn.as<double2>(), w.gg.as<double2>());
      VS_LAUNCH_CHECK();
      *launches += 5 + 9;
      ++issued;
      if (issued % 4 == 0 || k == kmax - 1) {
        VS_CUDA(cudaMemcpyAsync(&cur, gs, sizeof(GState), cudaMemcpyDeviceToHost, st));
        VS_CUDA(cudaStreamSynchronize(st));
        if (cur.skip) break;
      }
    }
    VS_CUDA(cudaMemcpyAsync(&cur, gs, sizeof(GState), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    const int kd = cur.k;
    steps += kd;
    nres = cur.nres;
    if (kd > 0) {
      k_gm_solve<<<1, 32, 0, st>>>(gs, H, w.gg.as<double2>(), w.gy.as<double2>());
      k_gm_xupdate<T><<<g, 256, kd * sizeof(C), st>>>(d, V, n, kd, w.gy.as<double2>());
      VS_LAUNCH_CHECK();
      *launches += 2;
    }
    if (cur.flag == 0) {
      *flag = 0;
      break;
    }
    if (cur.flag == 5 || kd == 0) {
      *flag = cur.flag == 5 ? 5 : 4;
      break;
    }
  }
  *nres_out = std::min<int64_t>(nres, resvec_cap);
  return steps;
}

template <typename T>
static void gmres_buffers(KrylovWork& w, int64_t n, int m) {
  using C = cplx_t<T>;
  w.gV.alloc((size_t)(m + 1) * n * sizeof(C));
  w.gw.alloc(n * sizeof(C));
  w.gtmp.alloc(n * sizeof(C));
  w.gd.alloc(n * sizeof(C));
  w.r.alloc(n * sizeof(C));
  w.gH.alloc((size_t)(m + 1) * m * sizeof(double2));
  w.gcs.alloc(m * sizeof(double));
  w.gsn.alloc(m * sizeof(double2));
  w.gg.alloc((m + 1) * sizeof(double2));
  w.gy.alloc(m * sizeof(double2));
  w.ghp.alloc((m + 1) * sizeof(double2));
  w.gpart.alloc((size_t)(m + 1) * ceil_div(n, kDotChunk) * sizeof(double2));
  w.gstate.alloc(sizeof(GState));
}

template <typename T>
static void gmres_refine(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm,
                         SolveResult& out, cudaStream_t st, double bnorm, int64_t& launches, double* rv, int cap) {
  using C = cplx_t<T>;
  KrylovWork& w = op.kw;
  const int64_t n = op.n3;
  const int m = std::max(1, std::min(prm.restart, prm.maxit));
  gmres_buffers<T>(w, n, m);
  w.y64.alloc(n * sizeof(double2));
  w.r64.alloc(n * sizeof(double2));
  double2* r64 = w.r64.as<double2>();
  double rn;
  if (norm64(w, x, n, st, &launches) == 0.0) {
    k_copy<double><<<vec_grid(n), 256, 0, st>>>(r64, b, n);
    VS_LAUNCH_CHECK();
    launches += 1;
    rn = bnorm;
  } else {
    rn = residual64(op, w, b, x, r64, n, st, &launches, prm.op_mode);
  }
  const bool fp64 = std::is_same<T, double>::value;
  int steps = 0, flag = 1, refine = 0;
  int64_t nres = 0;
  for (; refine <= prm.max_refine; ++refine) {
    if (rn <= prm.tol * bnorm) {
      flag = 0;
      break;
    }
    if (refine == prm.max_refine || steps >= prm.maxit) break;
    double itol = prm.inner_tol > 0 ? prm.inner_tol
                                    : std::max((fp64 ? 0.5 : 0.3) * prm.tol * bnorm / rn, fp64 ? 1e-15 : prm.inner_floor);
    itol = std::min(itol, 0.5);
    k_r64_to<<<vec_grid(n), 256, 0, st>>>(r64, w.r.as<C>(), n, 1.0 / rn);
    VS_LAUNCH_CHECK();
    launches += 1;
    double* rvk = (rv && nres < cap) ? rv + nres : nullptr;
    const int capk = rv ? (int)(cap - nres) : 0;
    int64_t nk = 0;
    int f = 1;
    steps += gmres_core<T>(op, pr, w, n, w.r.as<C>(), w.gd.as<C>(), itol, m, prm.maxit - steps, prm.op_mode,
                           rn / bnorm, rvk, capk, &nk, &f, st, &launches);
    nres += nk;
    k_update64_from<<<vec_grid(n), 256, 0, st>>>(x, w.gd.as<C>(), n, rn);
    VS_LAUNCH_CHECK();
    launches += 1;
    rn = residual64(op, w, b, x, r64, n, st, &launches, prm.op_mode);
    if (f == 5) {
      flag = 5;
      break;
    }
  }
  out.flag = (rn <= prm.tol * bnorm) ? 0 : (flag >= 4 ? flag : 1);
  out.relres = rn / bnorm;
  out.iter = steps;
  out.inner_iters = steps;
  out.refinements = refine;
  out.n_resvec = nres;
}

void solve_gmres(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                 cudaStream_t st) {
  const int64_t n = op.n3;
  KrylovWork& w = op.kw;
  w.partials.alloc(kRedBlocks * 4 * sizeof(double));
  w.state.alloc(sizeof(KState));
  w.scal.alloc(4 * sizeof(double));
  KState zero{};
  zero.partials = w.partials.as<double>();
  upload_state(w.state.as<KState>(), zero, st);
  const int cap = prm.resvec_cap;
  w.resvec.alloc(std::max(1, cap) * sizeof(double));
  double* rv = cap > 0 ? w.resvec.as<double>() : nullptr;
  ensure_scratch(op, 1, sizeof(double2));
  int64_t launches = 0;
  const double bnorm = norm64(w, b, n, st, &launches);
  if (!std::isfinite(bnorm)) throw Error(VS_ERR_NONFINITE, "right-hand side has NaN or Inf entries");
  out = SolveResult{};
  if (bnorm == 0) {
    VS_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double2), st));
    VS_CUDA(cudaStreamSynchronize(st));
    out.flag = 0;
    return;
  }
  if (prm.mode == VS_SOLVE_FP64) gmres_refine<double>(op, pr, b, x, prm, out, st, bnorm, launches, rv, cap);
  else gmres_refine<float>(op, pr, b, x, prm, out, st, bnorm, launches, rv, cap);
  out.launches = launches;
  if (cap > 0 && prm.resvec_host && out.n_resvec > 0)
    VS_CUDA(cudaMemcpyAsync(prm.resvec_host, rv, out.n_resvec * sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace vs
