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
#include "vs_dense.h"
#include "vs_reduce.cuh"
#include "vs_pipeline.cuh"

#include <chrono>
#include <cmath>
#include <vector>
#include <memory>

namespace vs {

// The reduction kernels (dots and norms with a grid-wide sum): two CTAs of
// 256 threads per SM.  Each CTA ends with a fence and one atomic on the
// right-hand side's counter, and those serialise (eight CTAs per SM made the
// kernels slower; one CTA of 1024 per SM was no faster).
constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 2 * 152;

// Grid sum of NV per-thread values (FF2 for the c64 kernels, double for
// c128); returns true in the last CTA to finish, with the grid totals in
// `tot` (all threads of that CTA).  Each CTA adds its threads' values
// (cta_partials: warp trees, then warp 0 over the warps) into one slot per
// value, and warp 0 of the last CTA adds the slots in CTA order, so the
// result does not depend on scheduling.  GB300 runs FP64 at a small fraction
// of its FP32 rate (an FP64 instruction that every thread of a 300-CTA grid
// executed cost about 0.1 us), so the c64 sums stay float-float on the FP32
// pipes and one lane widens each total to double.
template <int NV, typename V>
__device__ bool grid_reduce(const V (&v)[NV], double* __restrict__ partials, unsigned* __restrict__ counter,
                            double (&tot)[NV]) {
  __shared__ double stot[NV];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  cta_partials<NV>(v, partials + (int64_t)blockIdx.x * NV);  // written by thread 0
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  if (warp == 0) {
    V x[NV];
    slot_sums<NV, (kRedBlocks + 31) / 32, true>(partials, (int)gridDim.x, lane, 32, x);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const V y = warp_sum_v(x[k]);
      if (lane == 0) stot[k] = widen(y);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = stot[k];
  if (threadIdx.x == 0) *counter = 0;
  return true;
}


#define GRID_LOOP(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// Grid-stride walk over [0, n) in chunks of kChunk elements per thread: the
// loads of a chunk (ld(i), each predicated on i < n) are all issued before
// its first use (use(i, loaded)), so a thread waits about one memory latency
// per chunk rather than one per element.  Elements are used in increasing i,
// as in a plain grid-stride loop, so per-thread sums keep their order.
constexpr int kChunk = 4;
template <typename Ld, typename Use>
__device__ __forceinline__ void grid_chunks(int64_t n, Ld ld, Use use) {
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < n; b += kChunk * st) {
    decltype(ld(b)) v[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u)
      if (b + u * st < n) v[u] = ld(b + u * st);
#pragma unroll
    for (int u = 0; u < kChunk; ++u)
      if (b + u * st < n) use(b + u * st, v[u]);
  }
}
template <typename C, int K>
struct Loaded {
  C e[K];
};

// All BiCGSTAB kernels below run on a batch of right-hand sides sharing one
// operator: blockIdx.y is the right-hand side, its vectors start at
// rhs * n, and its scalars live in states[rhs] (each state carries its own
// reduction partials and counter).  A kernel of more than one CTA writes a
// state only from the last CTA to count in on that counter, after every
// thread of every CTA has read the skip flag, so a CTA never splits over it.

// The scalars in the kernels' precision: the float copies for c64.
template <typename C>
__device__ __forceinline__ C scal(const double2& d, const float2& f);
template <>
__device__ __forceinline__ float2 scal<float2>(const double2&, const float2& f) { return f; }
template <>
__device__ __forceinline__ double2 scal<double2>(const double2& d, const float2&) { return d; }
__device__ __forceinline__ float2 to_f2(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ void set_alpha(KState* s, double2 v) { s->alpha = v; s->alpha32 = to_f2(v); }
__device__ __forceinline__ void set_omega(KState* s, double2 v) { s->omega = v; s->omega32 = to_f2(v); }
__device__ __forceinline__ void set_beta(KState* s, double2 v) { s->beta = v; s->beta32 = to_f2(v); }

// The scalar steps of BiCGSTAB, from the grid totals (one thread):
// alpha = rho / (rt^H v) with its breakdown test (alpha_step);
__device__ __forceinline__ void finish_alpha(KState* s, const double (&t)[2]) {
  double2 al;
  const int f = alpha_step(s->rho, t, al);
  if (f >= 0) {
    s->flag = f;
    s->skip = 1;
    return;
  }
  set_alpha(s, al);
}
// ||s|| (t = ||s||^2) and the half-step convergence test;
__device__ __forceinline__ void finish_s(KState* s, const double (&t)[1]) {
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
// omega = (t^H s)/(t^H t) (tt = t^H s, t^H t) with its breakdown tests:
// the flag that ends the iteration (4 breakdown, 5 not finite), or -1 and
// omega in om.
__device__ __forceinline__ int omega_step(const double (&tt)[3], double2& om) {
  const double2 ts = make_double2(tt[0], tt[1]);
  const double t2 = tt[2];
  if (!(t2 > 0) || !cfinite(ts)) return (t2 == 0) ? 4 : 5;
  om = make_double2(ts.x / t2, ts.y / t2);
  return cz(om) ? 4 : -1;
}
__device__ __forceinline__ void finish_omega(KState* s, const double (&tt)[3]) {
  double2 om;
  const int f = omega_step(tt, om);
  if (f >= 0) {
    s->flag = f;
    s->skip = 1;
    return;
  }
  set_omega(s, om);
}

// Folded steps (vs_pipeline.cuh XFuse): a two-level x pass left nb per-CTA
// partial sums (NV slots each, slot form V) of a right-hand side at part; a
// CTA of kFinThreads adds them in a fixed order (each thread a few slots, all
// loaded before the first add, then the warp and CTA trees; float-float for
// c64), so every CTA that adds the same slots gets the same bits; thread 0
// widens the totals to double, and every thread gets them in tot.  (One warp
// walking all partials waited on one L2 load per partial: 5-8 us per step.)
constexpr int kFinThreads = 256;
static_assert(kFinThreads == kRedThreads, "the merged kernels add partials with their own CTAs");
template <int NV, typename V>
__device__ __forceinline__ void sum_cta_partials(const double* __restrict__ part, int nb, double (&tot)[NV]) {
  __shared__ double slot[NV];
  V x[NV];
  slot_sums<NV, 4, false>(part, nb, (int)threadIdx.x, kFinThreads, x);
  cta_partials<NV>(x, slot);  // thread 0 writes the CTA's sums in slot form
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      V y;
      get_slot<false>(slot + k, y);
      slot[k] = widen(y);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = slot[k];
}
// rho = rt^H r ; beta = (rho/rho_prev)(alpha/omega)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_rho(const cplx_t<T>* __restrict__ rt,
                                                         const cplx_t<T>* __restrict__ r, int64_t n,
                                                         KState* states) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  if (s->skip) return;
  rt += blockIdx.y * n; r += blockIdx.y * n;
  Acc<T> a;
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{rt[i], r[i]}}; },
              [&](int64_t, const Loaded<C, 2>& l) { a.dot(l.e[0], l.e[1]); });
  const SlotV<T> v[2] = {a.vre(), a.vim()};
  double t[2];
  if (grid_reduce<2>(v, s->partials, &s->counter, t) && threadIdx.x == 0) {
    const double2 rho = make_double2(t[0], t[1]);
    if (cz(rho) || !cfinite(rho)) {
      s->flag = cfinite(rho) ? 4 : 5;
      s->skip = 1;
      return;
    }
    if (s->iter2 > 0) set_beta(s, cmul(cdiv(rho, s->rho_prev), cdiv(s->alpha, s->omega)));
    s->rho = rho;
  }
}

// p = r (first iteration) or r + beta (p - omega v)
template <typename T>
__global__ void k_bicg_p(cplx_t<T>* __restrict__ p, const cplx_t<T>* __restrict__ r,
                         const cplx_t<T>* __restrict__ v, int64_t n, const KState* states) {
  using C = cplx_t<T>;
  const KState* s = states + blockIdx.y;
  if (s->skip) return;
  p += blockIdx.y * n; r += blockIdx.y * n; v += blockIdx.y * n;
  if (s->iter2 == 0) {
    grid_chunks(n, [&](int64_t i) { return r[i]; }, [&](int64_t i, C x) { p[i] = x; });
    return;
  }
  const C beta = scal<C>(s->beta, s->beta32), om = scal<C>(s->omega, s->omega32);
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 3>{{p[i], v[i], r[i]}}; },
              [&](int64_t i, const Loaded<C, 3>& l) { p[i] = cfma(beta, csub(l.e[0], cmul(om, l.e[1])), l.e[2]); });
}

// alpha = rho / (rt^H v)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_alpha(const cplx_t<T>* __restrict__ rt,
                                                           const cplx_t<T>* __restrict__ v, int64_t n,
                                                           KState* states) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  if (s->skip) return;
  rt += blockIdx.y * n; v += blockIdx.y * n;
  Acc<T> a;
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{rt[i], v[i]}}; },
              [&](int64_t, const Loaded<C, 2>& l) { a.dot(l.e[0], l.e[1]); });
  const SlotV<T> w[2] = {a.vre(), a.vim()};
  double t[2];
  if (grid_reduce<2>(w, s->partials, &s->counter, t) && threadIdx.x == 0) finish_alpha(s, t);
}

// s = r - alpha v ; ||s|| ; half-step convergence test
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_s(cplx_t<T>* __restrict__ sv, const cplx_t<T>* __restrict__ r,
                                                       const cplx_t<T>* __restrict__ v, int64_t n, KState* states) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  if (s->skip) return;
  sv += blockIdx.y * n; r += blockIdx.y * n; v += blockIdx.y * n;
  const C al = scal<C>(s->alpha, s->alpha32);
  Acc<T> a;
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{r[i], v[i]}}; },
              [&](int64_t i, const Loaded<C, 2>& l) {
                const C x = csub(l.e[0], cmul(al, l.e[1]));
                sv[i] = x;
                a.norm2(x);
              });
  const SlotV<T> w[1] = {a.vre()};
  double t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) finish_s(s, t);
}

// x += alpha ph when the half step converged (runs regardless of skip).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_xhalf(cplx_t<T>* __restrict__ x,
                                                           const cplx_t<T>* __restrict__ ph, int64_t n,
                                                           KState* states) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  __shared__ int s_go;
  if (threadIdx.x == 0) s_go = s->half_pending;
  __syncthreads();
  if (!s_go) return;
  x += blockIdx.y * n; ph += blockIdx.y * n;
  const C al = scal<C>(s->alpha, s->alpha32);
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{x[i], ph[i]}}; },
              [&](int64_t i, const Loaded<C, 2>& l) { x[i] = cfma(al, l.e[1], l.e[0]); });
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&s->counter, 1u) == gridDim.x - 1) {
      s->half_pending = 0;
      s->counter = 0;
    }
  }
}

// Folded steps, after the second preconditioner apply's forward x pass left
// the partial sums of ||s||^2 at part (nb per right-hand side): every CTA
// adds them (same order, same bits) and its thread 0 takes the half-step
// test; every CTA adds its share of alpha ph to x when the half step
// converged, and the last CTA to finish -- after every CTA has read the skip
// flag -- writes the half-step state (finish_s).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_shalf(cplx_t<T>* __restrict__ x,
                                                           const cplx_t<T>* __restrict__ ph, int64_t n,
                                                           KState* states, const double* __restrict__ part,
                                                           int64_t pstride, int nb) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  __shared__ int s_conv;
  if (s->skip) return;
  double t[1];
  sum_cta_partials<1, SlotV<T>>(part + blockIdx.y * pstride, nb, t);
  if (threadIdx.x == 0) {
    const double res = sqrt(t[0]);
    s_conv = isfinite(res) && res <= s->tol_abs;
  }
  __syncthreads();
  if (s_conv) {
    x += blockIdx.y * n; ph += blockIdx.y * n;
    const C al = scal<C>(s->alpha, s->alpha32);
    grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{x[i], ph[i]}}; },
                [&](int64_t i, const Loaded<C, 2>& l) { x[i] = cfma(al, l.e[1], l.e[0]); });
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&s->counter, 1u) == gridDim.x - 1) {
      finish_s(s, t);
      s->half_pending = 0;
      s->counter = 0;
    }
  }
}

// omega = (t^H s)/(t^H t)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_omega(const cplx_t<T>* __restrict__ t,
                                                           const cplx_t<T>* __restrict__ sv, int64_t n,
                                                           KState* states) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  if (s->skip) return;
  t += blockIdx.y * n; sv += blockIdx.y * n;
  Acc<T> a, b;
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 2>{{t[i], sv[i]}}; },
              [&](int64_t, const Loaded<C, 2>& l) {
                a.dot(l.e[0], l.e[1]);
                b.norm2(l.e[0]);
              });
  const SlotV<T> w[3] = {a.vre(), a.vim(), b.vre()};
  double tt[3];
  if (grid_reduce<3>(w, s->partials, &s->counter, tt) && threadIdx.x == 0) finish_omega(s, tt);
}

// x += alpha ph + omega sh ; r = s - omega t ; ||r|| ; full-step test ; and,
// when the iteration continues, the next rho = rt^H r with its breakdown test
// and beta = (rho_new/rho)(alpha/omega) (the first rho comes from k_bicg_rho).
// omega: from the state (k_bicg_omega), or, with folded steps (opart
// non-null), from the partial sums of t^H s and t^H t that the matvec's
// inverse x pass left at opart (nb per right-hand side), added by every CTA
// in the same order and divided by its thread 0; a breakdown there ends the
// iteration (every CTA returns, the last to finish writes the flag), else the
// last CTA stores omega with the rest.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_bicg_xr(cplx_t<T>* __restrict__ x, cplx_t<T>* __restrict__ r,
                                                        const cplx_t<T>* __restrict__ ph,
                                                        const cplx_t<T>* __restrict__ sh,
                                                        const cplx_t<T>* __restrict__ sv,
                                                        const cplx_t<T>* __restrict__ t,
                                                        const cplx_t<T>* __restrict__ rt, int64_t n, KState* states,
                                                        const double* __restrict__ opart, int64_t pstride, int nb) {
  using C = cplx_t<T>;
  KState* s = states + blockIdx.y;
  __shared__ double2 s_om;
  __shared__ float2 s_om32;
  __shared__ int s_flag;
  if (s->skip) return;
  if (opart) {
    double tt[3];
    sum_cta_partials<3, SlotV<T>>(opart + blockIdx.y * pstride, nb, tt);
    if (threadIdx.x == 0) {
      double2 om = make_double2(0, 0);
      s_flag = omega_step(tt, om);
      s_om = om;
      s_om32 = to_f2(om);
    }
    __syncthreads();
    if (s_flag >= 0) {
      // every CTA sees the breakdown; the last one to count in writes it
      // (no state is written while a CTA may still read the skip flag)
      if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&s->counter, 1u) == gridDim.x - 1) {
          s->flag = s_flag;
          s->skip = 1;
          s->counter = 0;
        }
      }
      return;
    }
  } else if (threadIdx.x == 0) {
    s_om = s->omega;
    s_om32 = s->omega32;
  }
  __syncthreads();
  const int64_t o = blockIdx.y * n;
  x += o; r += o; ph += o; sh += o; sv += o; t += o; rt += o;
  const C al = scal<C>(s->alpha, s->alpha32), om = scal<C>(s_om, s_om32);
  Acc<T> a, d;
  grid_chunks(n, [&](int64_t i) { return Loaded<C, 6>{{x[i], ph[i], sh[i], sv[i], t[i], rt[i]}}; },
              [&](int64_t i, const Loaded<C, 6>& l) {
                x[i] = cfma(om, l.e[2], cfma(al, l.e[1], l.e[0]));
                const C ri = csub(l.e[3], cmul(om, l.e[4]));
                r[i] = ri;
                a.norm2(ri);
                d.dot(l.e[5], ri);
              });
  const SlotV<T> w[3] = {a.vre(), d.vre(), d.vim()};
  double tt[3];
  if (grid_reduce<3>(w, s->partials, &s->counter, tt) && threadIdx.x == 0) {
    const double2 omd = s_om;
    set_omega(s, omd);
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
    if (!s->skip) {
      const double2 rho = make_double2(tt[1], tt[2]);
      if (cz(rho) || !cfinite(rho)) {
        s->flag = cfinite(rho) ? 4 : 5;
        s->skip = 1;
      } else {
        set_beta(s, cmul(cdiv(rho, s->rho), cdiv(s->alpha, omd)));
        s->rho = rho;
      }
    }
  }
}

// out[rhs] = ||u_rhs|| (states supply the reduction buffers)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_norm(const cplx_t<T>* u, int64_t n, KState* states, double* out) {
  KState* s = states + blockIdx.y;
  u += blockIdx.y * n;
  Acc<T> a;
  grid_chunks(n, [&](int64_t i) { return u[i]; }, [&](int64_t, cplx_t<T> x) { a.norm2(x); });
  const SlotV<T> w[1] = {a.vre()};
  double t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) out[blockIdx.y] = sqrt(t[0]);
}

template <typename T>
__global__ void k_copy(cplx_t<T>* dst, const cplx_t<T>* src, int64_t n) {
  GRID_LOOP(i, n) dst[i] = src[i];
}
template <typename T>
__global__ void k_zero(cplx_t<T>* dst, int64_t n) {
  GRID_LOOP(i, n) dst[i] = czero<cplx_t<T>>();
}

// r64 = b - y64 and its compensated norm, per right-hand side
__global__ void __launch_bounds__(kRedThreads) k_resid64(const double2* b, const double2* y, double2* r, int64_t n,
                                                        KState* states, double* out) {
  KState* s = states + blockIdx.y;
  const int64_t o = blockIdx.y * n;
  b += o; y += o; r += o;
  Acc<double> a;
  GRID_LOOP(i, n) {
    const double2 v = csub(b[i], y[i]);
    r[i] = v;
    a.norm2(v);
  }
  const double w[1] = {a.vre()};
  double t[1];
  if (grid_reduce<1>(w, s->partials, &s->counter, t) && threadIdx.x == 0) out[blockIdx.y] = sqrt(t[0]);
}

// r32 = r64 * sc[rhs]
__global__ void k_scale_down(const double2* r, float2* o, int64_t n, const double* sc) {
  const int64_t off = blockIdx.y * n;
  const double f = sc[blockIdx.y];
  GRID_LOOP(i, n) o[off + i] = make_float2((float)(r[off + i].x * f), (float)(r[off + i].y * f));
}
// x64 += sc[rhs] * d32
__global__ void k_update64(double2* x, const float2* d, int64_t n, const double* sc) {
  const int64_t off = blockIdx.y * n;
  const double f = sc[blockIdx.y];
  GRID_LOOP(i, n) {
    x[off + i].x = fma(f, (double)d[off + i].x, x[off + i].x);
    x[off + i].y = fma(f, (double)d[off + i].y, x[off + i].y);
  }
}

// Inner (c64) solves stop when the residual has not improved by 1% for this
// many iterations: the c64 recurrence has reached its floor and the FP64
// refinement takes over.
constexpr int kStagnationWindow = 8;

// CTAs of the element-wise kernels (256 threads, no grid-wide sum)
static int vec_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 8 * 152)); }
// CTAs of the reduction kernels (kRedThreads threads; at most kRedBlocks partials)
static int red_grid(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kRedThreads), kRedBlocks));
}

// The Gram per right-hand side of the current solve, or nullptr (the operator's).
static const RhsGram* rgp(const KrylovWork& w) { return w.rg.empty() ? nullptr : &w.rg; }

// Installs the solve's Gram per right-hand side (if any) on the work buffers
// for the duration of one solve.
struct RhsGramScope {
  KrylovWork& w;
  RhsGramScope(const vs_op& op, KrylovWork& wk, const SolveParams& prm, int nrhs, cudaStream_t st) : w(wk) {
    w.rg = RhsGram{};
    if (prm.gram_host) upload_rhs_gram(op, prm.gram_host, nrhs, prm.gram_n, w.rg64, w.rg32, w.rg, st);
  }
  ~RhsGramScope() { w.rg = RhsGram{}; }
};

// ---- host driver ---------------------------------------------------------

template <typename T>
void KrylovWork::ensure(int64_t n) {
  using C = cplx_t<T>;
  const size_t b = n * sizeof(C);
  DevBuf* v[] = {&r, &rt, &p, &v_, &s, &t, &ph, &sh, &x};
  for (DevBuf* d : v) d->alloc(b);
}

// Per-rhs reduction buffers: kRedBlocks * 4 doubles each.
static void reduction_buffers(KrylovWork& w, int nrhs) {
  w.partials.alloc((size_t)nrhs * kRedBlocks * 4 * sizeof(double));
  w.state.alloc((size_t)nrhs * sizeof(KState));
  w.scal.alloc((size_t)std::max(4, nrhs) * sizeof(double));
}

static void upload_states(KrylovWork& w, std::vector<KState>& h, cudaStream_t st) {
  for (size_t r = 0; r < h.size(); ++r) {
    h[r].partials = w.partials.as<double>() + r * kRedBlocks * 4;
    h[r].counter = 0;
  }
  VS_CUDA(cudaMemcpyAsync(w.state.p, h.data(), h.size() * sizeof(KState), cudaMemcpyHostToDevice, st));
}

static std::vector<double> read_scal(KrylovWork& w, int nrhs, cudaStream_t st) {
  std::vector<double> v(nrhs);
  VS_CUDA(cudaMemcpyAsync(v.data(), w.scal.p, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  return v;
}

// Events recorded by one profiled iteration (kIterMarks per iteration): 0
// before it, 1 after the direction update, 2..6 after the five passes of the
// first preconditioner apply, 7..11 after the matvec's five, 12 after the
// alpha / s / half-step kernels (with folded steps none: 12 follows 11),
// 13..17 and 18..22 the second apply and matvec, 23 after the omega / x, r
// kernels; with folded steps, 24 after the half-step kernel (between 13 and
// 14).
constexpr int kIterMarks = 25;

// BiCGSTAB's vector steps folded into the x passes (XFuse): the
// preconditioner's forward x pass forms p (first apply) and s with ||s||^2
// (second apply), the matvec's inverse x pass adds rt^H v (first) and t^H s,
// t^H t (second); the partial sums of nb_mv / nb_pr CTAs per right-hand side
// go to part (pstride doubles each).  alpha, the half-step test and omega
// are taken by every CTA of the kernels that use them (the second apply's
// forward x pass, k_bicg_shalf, k_bicg_xr).  Four streaming vector kernels
// and three scalar kernels of the iteration are gone.
struct FoldPlan {
  int nb_mv = 0, nb_pr = 0;
  int64_t pstride = 0;
  double* part = nullptr;
};

// Whether both x passes of this precision run the two-level kernel (the one
// with the folded steps).
template <typename T>
static bool can_fold(const vs_op& op, const vs_prec* pr) {
  if (!pr) return false;
  const int pi = std::is_same<T, float>::value ? 0 : 1;
  const PassShape& sp = pr->shape[pi];
  const PassShape& so = op.shape[pi];
  if (sp.x_reg != 1 || sp.fuse_xy == 1 || so.x_reg < 1) return false;
  const int nl = op.M * op.N * 3;
  return x2_ctas(pr->L, nl) > 0 && x2_ctas(op.P, nl) > 0 && pr->L == op.L && pr->M == op.M && pr->N == op.N;
}

// The fold plan of an operator / preconditioner pair and nrhs right-hand
// sides, its partial sums in w.xpart; false when the steps cannot be folded.
template <typename T>
static bool make_fold_plan(const vs_op& op, const vs_prec* pr, KrylovWork& w, int nrhs, FoldPlan& plan) {
  if (!can_fold<T>(op, pr)) return false;
  const int nl = op.M * op.N * 3;
  plan.nb_mv = x2_ctas(op.P, nl);
  plan.nb_pr = x2_ctas(pr->L, nl);
  plan.pstride = 3 * (int64_t)std::max(plan.nb_mv, plan.nb_pr);
  const size_t need = (size_t)nrhs * plan.pstride * sizeof(double);
  if (w.xpart.bytes < need) w.xpart.alloc(need);
  plan.part = w.xpart.as<double>();
  return true;
}

// One BiCGSTAB iteration (two half steps) for all right-hand sides as a fixed
// launch sequence; mk (kIterMarks events) records the marks above.
template <typename T>
static void bicg_iteration(const vs_op& op, const vs_prec* pr, KrylovWork& w, KState* s, int64_t n, int nrhs,
                           int mode, cudaStream_t st, cudaEvent_t* mk = nullptr, const FoldPlan* fold = nullptr) {
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
  const dim3 g(vec_grid(n), nrhs), gr(red_grid(n), nrhs);
  const int* skip = &s->skip;
  const int ss = (int)(sizeof(KState) / sizeof(int));
  // an external record: a node of the captured graph (a plain record inside
  // a capture only orders streams)
  auto mark = [&](int i) {
    if (mk) VS_CUDA(cudaEventRecordWithFlags(mk[i], st, cudaEventRecordExternal));
  };
  // M^-1 u -> o then A o -> y, one event after each pass when profiled
  auto prec_then_matvec = [&](const C* u, C* o, C* y, int m0) {
    for (int pass = 0; pass < 5; ++pass) {
      if (pr) prec_apply_pass<T>(*pr, u, o, nrhs, skip, st, pass, ss);
      else if (pass == 0) k_copy<T><<<dim3(vec_grid(n * nrhs)), 256, 0, st>>>(o, u, n * nrhs);
      mark(m0 + pass);
    }
    for (int pass = 0; pass < 5; ++pass) {
      matvec_pass<T>(op, o, y, nrhs, mode, skip, st, pass, ss, rgp(w));
      mark(m0 + 5 + pass);
    }
  };
  if (fold) {
    XFuse<T> f{};
    f.sbase = reinterpret_cast<const char*>(s);
    f.sstride = (int64_t)sizeof(KState);
    f.part = fold->part;
    f.pstride = fold->pstride;
    XFuse<T> fp = f, fsv = f, fd = f, fo = f;
    // the passes read the scalars in their own precision (float copies for c64)
    constexpr bool c64 = std::is_same<T, float>::value;
    fp.kind = XF_GATHER_P;
    fp.off_a = c64 ? (int)offsetof(KState, beta32) : (int)offsetof(KState, beta);
    fp.off_b = c64 ? (int)offsetof(KState, omega32) : (int)offsetof(KState, omega);
    fp.off_iter = (int)offsetof(KState, iter2);
    fp.u = r; fp.v = v; fp.w = p;
    fsv.kind = XF_GATHER_S;
    fsv.off_a = c64 ? (int)offsetof(KState, alpha32) : (int)offsetof(KState, alpha);
    fsv.u = r; fsv.v = v; fsv.w = sv;
    // alpha from the first matvec's partial sums, taken by the gather itself
    fsv.apart = fold->part;
    fsv.anb = fold->nb_mv;
    fsv.off_rho = (int)offsetof(KState, rho);
    fsv.off_alpha = (int)offsetof(KState, alpha);
    fsv.off_flag = (int)offsetof(KState, flag);
    fsv.off_skip = (int)offsetof(KState, skip);
    fsv.off_counter = (int)offsetof(KState, counter);
    fd.kind = XF_SCATTER_DOT;
    fd.u = rt;
    fo.kind = XF_SCATTER_OMEGA;
    fo.u = sv;
    mark(0);
    mark(1);
    // p = r + beta (p - omega v) in the first apply's forward x pass
    for (int pass = 0; pass < 5; ++pass) {
      prec_apply_pass<T>(*pr, p, ph, nrhs, skip, st, pass, ss, pass == 0 ? &fp : nullptr);
      mark(2 + pass);
    }
    // rt^H v in the matvec's inverse x pass
    for (int pass = 0; pass < 5; ++pass) {
      matvec_pass<T>(op, ph, v, nrhs, mode, skip, st, pass, ss, rgp(w), pass == 4 ? &fd : nullptr);
      mark(7 + pass);
    }
    mark(12);
    // alpha, then s = r - alpha v and ||s||^2, in the second apply's forward
    // x pass; the half-step test (and x += alpha ph if it converged), then
    // the rest of the apply
    prec_apply_pass<T>(*pr, sv, sh, nrhs, skip, st, 0, ss, &fsv);
    mark(13);
    k_bicg_shalf<T><<<gr, kRedThreads, 0, st>>>(x, ph, n, s, fold->part, fold->pstride, fold->nb_pr);
    mark(24);
    for (int pass = 1; pass < 5; ++pass) {
      prec_apply_pass<T>(*pr, sv, sh, nrhs, skip, st, pass, ss);
      mark(13 + pass);
    }
    // t^H s, t^H t in the matvec's inverse x pass; omega, x and r
    for (int pass = 0; pass < 5; ++pass) {
      matvec_pass<T>(op, sh, t, nrhs, mode, skip, st, pass, ss, rgp(w), pass == 4 ? &fo : nullptr);
      mark(18 + pass);
    }
    k_bicg_xr<T><<<gr, kRedThreads, 0, st>>>(x, r, ph, sh, sv, t, rt, n, s, fold->part, fold->pstride, fold->nb_mv);
    mark(23);
    VS_LAUNCH_CHECK();
    return;
  }
  mark(0);
  k_bicg_p<T><<<g, 256, 0, st>>>(p, r, v, n, s);
  mark(1);
  prec_then_matvec(p, ph, v, 2);
  k_bicg_alpha<T><<<gr, kRedThreads, 0, st>>>(rt, v, n, s);
  k_bicg_s<T><<<gr, kRedThreads, 0, st>>>(sv, r, v, n, s);
  k_bicg_xhalf<T><<<gr, kRedThreads, 0, st>>>(x, ph, n, s);
  mark(12);
  prec_then_matvec(sv, sh, t, 13);
  k_bicg_omega<T><<<gr, kRedThreads, 0, st>>>(t, sv, n, s);
  k_bicg_xr<T><<<gr, kRedThreads, 0, st>>>(x, r, ph, sh, sv, t, rt, n, s, nullptr, 0, 0);
  mark(23);
  VS_LAUNCH_CHECK();
}

// Adds the durations between the marks of `iters` profiled iterations.
static void add_iteration_profile(const cudaEvent_t* ev, int iters, SolveProfile* prof, bool folded) {
  auto dt = [&](int it, int a, int b) {
    float ms = 0;
    VS_CUDA(cudaEventElapsedTime(&ms, ev[it * kIterMarks + a], ev[it * kIterMarks + b]));
    return (double)ms;
  };
  for (int it = 0; it < iters; ++it) {
    prof->vec_ms += dt(it, 0, 1) + dt(it, 11, 12) + dt(it, 22, 23) + (folded ? dt(it, 13, 24) : 0.0);
    for (int p = 0; p < 10; ++p)
      prof->pass_ms[p] += dt(it, 1 + p, 2 + p) + ((folded && p == 1) ? dt(it, 24, 14) : dt(it, 12 + p, 13 + p));
  }
  prof->iters += iters;
}

// Kernels in one bicg_iteration: 6 solver kernels, 2 matvecs of 5 passes, and
// 2 preconditioner applies (or 2 copies without preconditioner); with folded
// steps 2 solver kernels (the half-step test with x after a converged half
// step; omega with x and r) and 20 passes.
template <typename T>
static int kernels_per_iteration(const vs_prec* pr, bool folded = false) {
  return folded ? 22 : 6 + 10 + (pr ? 2 * prec_launches<T>(*pr) : 2);
}

// BiCGSTAB on w.x (initial guesses already there) with initial residuals in
// w.r, for nrhs right-hand sides.  The absolute tolerance of rhs r is
// tol * bnorm[r].  Iterations are launched as a CUDA graph of `per_graph`
// iterations; the host polls the states between graph launches.
template <typename T>
static std::vector<KState> bicgstab_core(const vs_op& op, const vs_prec* pr, KrylovWork& w, int64_t n, int nrhs,
                                         const std::vector<double>& bnorm, double tol, int maxit,
                                         const std::vector<double>& res_scale, double* resvec_dev, int resvec_cap,
                                         int per_graph, cudaStream_t st, int64_t* launches, int stag_window,
                                         int mode, SolveProfile* prof = nullptr, bool fold_steps = false) {
  using C = cplx_t<T>;
  std::vector<KState> h(nrhs);
  for (int r = 0; r < nrhs; ++r) {
    KState& k = h[r];
    k = KState{};
    k.tol_abs = tol * bnorm[r];
    k.maxit = maxit;
    k.res_scale = res_scale[r];
    k.resvec = resvec_dev ? resvec_dev + (int64_t)r * resvec_cap : nullptr;
    k.resvec_cap = resvec_dev ? resvec_cap : 0;
    k.flag = 1;
    k.stag_window = stag_window;
    k.best_res = INFINITY;
  }
  KState* s = w.state.as<KState>();
  upload_states(w, h, st);
  const int gn = vec_grid(n * nrhs);
  k_copy<T><<<gn, 256, 0, st>>>(w.rt.as<C>(), w.r.as<C>(), n * nrhs);
  k_norm<T><<<dim3(red_grid(n), nrhs), kRedThreads, 0, st>>>(w.r.as<C>(), n, s, w.scal.as<double>());
  *launches += 2;
  const std::vector<double> r0 = read_scal(w, nrhs, st);
  bool any_active = false;
  for (int r = 0; r < nrhs; ++r) {
    if (h[r].resvec && resvec_cap > 0) {
      const double v0 = r0[r] * res_scale[r];
      VS_CUDA(cudaMemcpyAsync(h[r].resvec, &v0, sizeof(double), cudaMemcpyHostToDevice, st));
    }
    h[r].res = r0[r];
    h[r].nres = 1;
    h[r].best_res = r0[r];
    if (!(r0[r] > h[r].tol_abs) || maxit <= 0) {
      h[r].flag = (r0[r] <= h[r].tol_abs) ? 0 : 1;
      h[r].skip = 1;
    } else {
      any_active = true;
    }
  }
  if (!any_active) return h;
  // The iteration graph depends only on the buffers, the preconditioner, the
  // batch size and the graph length (scalars live in the device states), so
  // it is captured once and reused by later solves on this operator.
  GraphCache& gc = std::is_same<T, float>::value ? w.graph32 : w.graph64;
  FoldPlan plan;
  const FoldPlan* fold = fold_steps && make_fold_plan<T>(op, pr, w, nrhs, plan) ? &plan : nullptr;
  std::vector<const void*> key = {w.r.p, w.rt.p, w.p.p, w.v_.p, w.s.p, w.t.p, w.ph.p, w.sh.p, w.x.p,
                                  w.state.p, w.partials.p, op.t1.p, op.t2.p,
                                  (const void*)(uintptr_t)(pr ? pr->id : 0), pr ? pr->t.p : nullptr,
                                  (const void*)(uintptr_t)per_graph, (const void*)(uintptr_t)mode,
                                  (const void*)(uintptr_t)nrhs, w.rg.g32, w.rg.g64, (const void*)(uintptr_t)w.rg.per,
                                  (const void*)(uintptr_t)(prof ? 1 : 0), (const void*)(uintptr_t)(fold ? 1 : 0),
                                  fold ? w.xpart.p : nullptr};
  if (prof) w.prof_ev.ensure((size_t)per_graph * kIterMarks);
  if (gc.exec == nullptr || gc.key != key) {
    gc.reset();
    // One launch sequence with every rhs skipped, outside capture: all
    // kernels return at once, but first-use attribute calls happen here
    // rather than in the capture.
    std::vector<KState> idle = h;
    for (auto& k : idle) k.skip = 1;
    upload_states(w, idle, st);
    bicg_iteration<T>(op, pr, w, s, n, nrhs, mode, st, nullptr, fold);
    *launches += kernels_per_iteration<T>(pr, fold != nullptr);
    cudaGraph_t graph = nullptr;
    VS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      for (int k = 0; k < per_graph; ++k)
        bicg_iteration<T>(op, pr, w, s, n, nrhs, mode, st, prof ? w.prof_ev.ev.data() + k * kIterMarks : nullptr,
                          fold);
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
  upload_states(w, h, st);
  // rho of the initial residual; later ones come out of k_bicg_xr
  k_bicg_rho<T><<<dim3(red_grid(n), nrhs), kRedThreads, 0, st>>>(w.rt.as<C>(), w.r.as<C>(), n, s);
  VS_LAUNCH_CHECK();
  *launches += 1;
  std::vector<KState> cur(nrhs);
  const int max_launch = (maxit + per_graph - 1) / per_graph + 1;
  for (int it = 0; it < max_launch; ++it) {
    VS_CUDA(cudaGraphLaunch(gc.exec, st));
    *launches += (int64_t)per_graph * kernels_per_iteration<T>(pr, fold != nullptr);
    VS_CUDA(cudaMemcpyAsync(cur.data(), s, nrhs * sizeof(KState), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    bool all = true, none = true;
    for (int r = 0; r < nrhs; ++r) {
      all = all && cur[r].skip;
      none = none && !cur[r].skip;
    }
    // every iteration of this launch ran for every rhs: a profile sample
    if (prof && none) add_iteration_profile(w.prof_ev.ev.data(), per_graph, prof, fold != nullptr);
    if (all) break;
  }
  for (int r = 0; r < nrhs; ++r)
    if (!cur[r].skip) cur[r].flag = 1;
  return cur;
}

// ||u_r|| for every rhs (compensated for c128)
static std::vector<double> norms64(KrylovWork& w, const double2* u, int64_t n, int nrhs, cudaStream_t st,
                                   int64_t* launches) {
  std::vector<KState> h(nrhs);
  upload_states(w, h, st);
  k_norm<double><<<dim3(red_grid(n), nrhs), kRedThreads, 0, st>>>(u, n, w.state.as<KState>(), w.scal.as<double>());
  VS_LAUNCH_CHECK();
  *launches += 1;
  return read_scal(w, nrhs, st);
}

// r64 = b - A x64 (c128 pipeline); returns ||r64|| per rhs.
static std::vector<double> residuals64(const vs_op& op, KrylovWork& w, const double2* b, const double2* x, double2* r,
                                       int64_t n, int nrhs, cudaStream_t st, int64_t* launches, int mode,
                                       SolveProfile* prof = nullptr) {
  std::vector<KState> h(nrhs);
  upload_states(w, h, st);
  double2* y = w.y64.as<double2>();
  if (prof) {
    w.prof_ev.ensure(2);
    VS_CUDA(cudaEventRecord(w.prof_ev.ev[0], st));
  }
  matvec<double>(op, x, y, nrhs, mode, nullptr, st, 0, rgp(w));
  k_resid64<<<dim3(red_grid(n), nrhs), kRedThreads, 0, st>>>(b, y, r, n, w.state.as<KState>(), w.scal.as<double>());
  VS_LAUNCH_CHECK();
  *launches += 6;
  if (prof) VS_CUDA(cudaEventRecord(w.prof_ev.ev[1], st));
  std::vector<double> out = read_scal(w, nrhs, st);
  if (prof) {
    float ms = 0;
    VS_CUDA(cudaEventElapsedTime(&ms, w.prof_ev.ev[0], w.prof_ev.ev[1]));
    prof->resid_ms += ms;
    prof->resid_calls += 1;
  }
  return out;
}

// Single-rhs helpers used by GMRES.
static double norm64(KrylovWork& w, const double2* u, int64_t n, cudaStream_t st, int64_t* launches) {
  return norms64(w, u, n, 1, st, launches)[0];
}
static double residual64(const vs_op& op, KrylovWork& w, const double2* b, const double2* x, double2* r, int64_t n,
                         cudaStream_t st, int64_t* launches, int mode) {
  return residuals64(op, w, b, x, r, n, 1, st, launches, mode)[0];
}

void solve_bicgstab_batch(vs_op& op, vs_prec* pr, const double2* b, double2* x, int nrhs, const SolveParams& prm,
                          std::vector<SolveResult>& out, cudaStream_t st) {
  const int64_t n = op.n3;
  KrylovWork& w = op.kw;
  RhsGramScope gram_scope(op, w, prm, nrhs, st);
  reduction_buffers(w, nrhs);
  const int cap = prm.resvec_cap;
  w.resvec.alloc((size_t)std::max(1, cap) * nrhs * sizeof(double));
  double* rv = cap > 0 ? w.resvec.as<double>() : nullptr;
  ensure_scratch(op, nrhs, sizeof(double2));
  if (pr) {
    const size_t need = (size_t)pr->L * pr->M * pr->N * 3 * sizeof(double2) * nrhs;
    if (pr->t.bytes < need) pr->t.alloc(need);
  }
  int64_t launches = 0;
  const std::vector<double> bnorm = norms64(w, b, n, nrhs, st, &launches);
  out.assign(nrhs, SolveResult{});
  for (int r = 0; r < nrhs; ++r)
    if (!std::isfinite(bnorm[r])) throw Error(VS_ERR_NONFINITE, "right-hand side has NaN or Inf entries");
  // zero right-hand sides: x = 0, converged
  std::vector<double> bsafe(nrhs);
  for (int r = 0; r < nrhs; ++r) {
    bsafe[r] = bnorm[r] > 0 ? bnorm[r] : 1.0;
    if (bnorm[r] == 0) VS_CUDA(cudaMemsetAsync(x + r * n, 0, n * sizeof(double2), st));
  }
  const std::vector<double> xn = norms64(w, x, n, nrhs, st, &launches);
  bool x0zero = true;
  for (double v : xn) x0zero = x0zero && v == 0.0;
  std::vector<double> rn;
  std::vector<int> inner2(nrhs, 0), flag(nrhs, 1), refine(nrhs, 0);
  std::vector<int64_t> nres(nrhs, 0);
  if (prm.mode == VS_SOLVE_FP64) {
    w.ensure<double>(n * nrhs);
    w.y64.alloc(n * nrhs * sizeof(double2));
    k_copy<double><<<vec_grid(n * nrhs), 256, 0, st>>>(w.x.as<double2>(), x, n * nrhs);
    if (x0zero) k_copy<double><<<vec_grid(n * nrhs), 256, 0, st>>>(w.r.as<double2>(), b, n * nrhs);
    else residuals64(op, w, b, x, w.r.as<double2>(), n, nrhs, st, &launches, prm.op_mode, prm.profile);
    launches += 2;
    std::vector<double> sc(nrhs);
    for (int r = 0; r < nrhs; ++r) sc[r] = 1.0 / bsafe[r];
    std::vector<KState> fs = bicgstab_core<double>(op, pr, w, n, nrhs, bsafe, prm.tol, prm.maxit, sc, rv, cap,
                                                   prm.per_graph, st, &launches, 0, prm.op_mode, prm.profile,
                                                   prm.fold_steps);
    k_copy<double><<<vec_grid(n * nrhs), 256, 0, st>>>(x, w.x.as<double2>(), n * nrhs);
    VS_LAUNCH_CHECK();
    launches += 1;
    rn = residuals64(op, w, b, x, w.r.as<double2>(), n, nrhs, st, &launches, prm.op_mode, prm.profile);
    for (int r = 0; r < nrhs; ++r) {
      out[r].flag = fs[r].flag;
      out[r].iter = fs[r].iter2 * 0.5;
      out[r].inner_iters = out[r].iter;
      out[r].n_resvec = std::min<int64_t>(fs[r].nres, cap);
      out[r].relres = bnorm[r] > 0 ? rn[r] / bnorm[r] : 0.0;
      if (bnorm[r] == 0) out[r].flag = 0;
      else if (out[r].flag == 0 && out[r].relres > prm.tol) out[r].flag = 1;
    }
  } else {
    // mixed: c64 inner BiCGSTAB inside FP64 refinement, all rhs together
    w.ensure<float>(n * nrhs);
    w.y64.alloc(n * nrhs * sizeof(double2));
    w.r64.alloc(n * nrhs * sizeof(double2));
    double2* r64 = w.r64.as<double2>();
    if (x0zero) {
      k_copy<double><<<vec_grid(n * nrhs), 256, 0, st>>>(r64, b, n * nrhs);
      VS_LAUNCH_CHECK();
      launches += 1;
      rn = bnorm;
    } else {
      rn = residuals64(op, w, b, x, r64, n, nrhs, st, &launches, prm.op_mode, prm.profile);
    }
    DevBuf scd;
    scd.alloc(nrhs * sizeof(double));
    for (int step = 0; step <= prm.max_refine; ++step) {
      bool all_done = true;
      for (int r = 0; r < nrhs; ++r) {
        const bool done = rn[r] <= prm.tol * bnorm[r] || flag[r] >= 4;
        if (rn[r] <= prm.tol * bnorm[r]) flag[r] = 0;
        all_done = all_done && done;
      }
      if (all_done || step == prm.max_refine) break;
      int used = 0;
      for (int r = 0; r < nrhs; ++r) used = std::max(used, inner2[r]);
      if (used >= 2 * prm.maxit) break;
      // per-rhs inner tolerance relative to the scaled residual (norm 1);
      // converged rhs get tol 1 (they stop at iteration 0)
      std::vector<double> scale(nrhs), one(nrhs, 1.0), rscale(nrhs), itol(nrhs);
      for (int r = 0; r < nrhs; ++r) {
        const bool done = rn[r] <= prm.tol * bnorm[r] || flag[r] >= 4;
        scale[r] = rn[r] > 0 ? 1.0 / rn[r] : 0.0;
        double t = prm.inner_tol > 0 ? prm.inner_tol : std::max(0.3 * prm.tol * bnorm[r] / rn[r], prm.inner_floor);
        itol[r] = done ? 2.0 : std::min(t, 0.5);
        rscale[r] = bnorm[r] > 0 ? rn[r] / bnorm[r] : 0.0;
        refine[r] += done ? 0 : 1;
      }
      VS_CUDA(cudaMemcpyAsync(scd.p, scale.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, st));
      k_scale_down<<<dim3(vec_grid(n), nrhs), 256, 0, st>>>(r64, w.r.as<float2>(), n, scd.as<double>());
      k_zero<float><<<vec_grid(n * nrhs), 256, 0, st>>>(w.x.as<float2>(), n * nrhs);
      VS_LAUNCH_CHECK();
      launches += 2;
      // one inner solve with a common tolerance: use the tightest active one,
      // expressed per rhs through bnorm = itol_r / itol_min
      double tmin = 1.0;
      for (int r = 0; r < nrhs; ++r) tmin = std::min(tmin, itol[r]);
      std::vector<double> bn(nrhs);
      for (int r = 0; r < nrhs; ++r) bn[r] = itol[r] / tmin;
      double* rvk = nullptr;
      int capk = 0;
      if (rv && nrhs == 1 && nres[0] < cap) {
        rvk = rv + nres[0];
        capk = (int)(cap - nres[0]);
      }
      std::vector<KState> fs = bicgstab_core<float>(op, pr, w, n, nrhs, bn, tmin, prm.maxit - used / 2, rscale, rvk,
                                                    capk, prm.per_graph, st, &launches, kStagnationWindow,
                                                    prm.op_mode, prm.profile, prm.fold_steps);
      bool progressed = false;
      for (int r = 0; r < nrhs; ++r) {
        inner2[r] += fs[r].iter2;
        if (nrhs == 1) nres[0] += std::min<int64_t>(fs[0].nres, capk);
        if (fs[r].flag >= 4 && fs[r].iter2 == 0 && !(rn[r] <= prm.tol * bnorm[r])) flag[r] = fs[r].flag;
        progressed = progressed || fs[r].iter2 > 0;
      }
      VS_CUDA(cudaMemcpyAsync(scd.p, rn.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, st));
      k_update64<<<dim3(vec_grid(n), nrhs), 256, 0, st>>>(x, w.x.as<float2>(), n, scd.as<double>());
      VS_LAUNCH_CHECK();
      launches += 1;
      rn = residuals64(op, w, b, x, r64, n, nrhs, st, &launches, prm.op_mode, prm.profile);
      if (!progressed) break;
    }
    for (int r = 0; r < nrhs; ++r) {
      out[r].flag = (rn[r] <= prm.tol * bnorm[r]) ? 0 : (flag[r] >= 4 ? flag[r] : 1);
      out[r].relres = bnorm[r] > 0 ? rn[r] / bnorm[r] : 0.0;
      out[r].iter = inner2[r] * 0.5;
      out[r].inner_iters = out[r].iter;
      out[r].refinements = refine[r];
      out[r].n_resvec = nrhs == 1 ? nres[0] : 0;
      if (bnorm[r] == 0) out[r].flag = 0;
    }
  }
  for (auto& o : out) o.launches = launches;
  if (cap > 0 && prm.resvec_host) {
    for (int r = 0; r < nrhs; ++r)
      if (out[r].n_resvec > 0)
        VS_CUDA(cudaMemcpyAsync(prm.resvec_host + (int64_t)r * cap, rv + (int64_t)r * cap,
                                out[r].n_resvec * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  VS_CUDA(cudaStreamSynchronize(st));
}

void solve_bicgstab(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                    cudaStream_t st) {
  std::vector<SolveResult> r;
  solve_bicgstab_batch(op, pr, b, x, 1, prm, r, st);
  out = r[0];
}

// ===========================================================================
// Lockstep BiCGSTAB over several particles (the reference solves each
// particle, incident direction and polarisation with its own bicgstab call,
// main_DDA.m:61-82).  Every particle keeps its own operator, preconditioner,
// work buffers and per-rhs states; an inner iteration of all particles is one
// CUDA graph whose branches (one per particle, forked to auxiliary streams
// during capture) the GPU runs concurrently, so the small particles' launches
// overlap instead of queueing.  A last node gathers every right-hand side's
// skip flag, so the host polls all particles with one copy per graph launch.
// Converged right-hand sides keep costing nothing but empty CTAs (skip flag),
// and a particle whose right-hand sides all converged skips whole launches.
// The FP64 refinement steps run in lockstep too (one host synchronisation per
// phase for all particles).
// ===========================================================================

// out[off[p] + r] = states_p[r].skip
__global__ void k_gather_skip(const KState* const* states, const int* off, int nparts, int* out) {
  for (int p = blockIdx.x; p < nparts; p += gridDim.x)
    for (int r = threadIdx.x; r < off[p + 1] - off[p]; r += blockDim.x) out[off[p] + r] = states[p][r].skip;
}

namespace {

constexpr int kMaxAuxStreams = 16;

// Per-particle bookkeeping of a lockstep solve.
struct PartState {
  PartJob* job = nullptr;
  int64_t n = 0;
  std::unique_ptr<RhsGramScope> gram;
  std::vector<double> bnorm, bsafe, rn, scal;
  std::vector<int> inner2, flag, refine;
  std::vector<double> tolr, rscale;  // inner solve: tolerance factor and resvec scale per rhs
  std::vector<KState> h, cur;
};

// Enqueue ||u_r|| (FP64, compensated) of every particle into its w.scal.
void enqueue_norms(std::vector<PartState>& ps, const std::vector<const double2*>& u, cudaStream_t st) {
  for (size_t i = 0; i < ps.size(); ++i) {
    PartState& p = ps[i];
    KrylovWork& w = p.job->op->kw;
    p.h.assign(p.job->nrhs, KState{});
    upload_states(w, p.h, st);
    k_norm<double><<<dim3(red_grid(p.n), p.job->nrhs), kRedThreads, 0, st>>>(u[i], p.n, w.state.as<KState>(),
                                                                             w.scal.as<double>());
  }
  VS_LAUNCH_CHECK();
}

// r64 = b - A x64 for every particle (its Gram per rhs), norms into w.scal.
void enqueue_residuals(std::vector<PartState>& ps, const std::vector<double2*>& xs, std::vector<double2*>& rs,
                       int mode, cudaStream_t st) {
  for (size_t i = 0; i < ps.size(); ++i) {
    PartState& p = ps[i];
    vs_op& op = *p.job->op;
    KrylovWork& w = op.kw;
    p.h.assign(p.job->nrhs, KState{});
    upload_states(w, p.h, st);
    matvec<double>(op, xs[i], w.y64.as<double2>(), p.job->nrhs, mode, nullptr, st, 0, rgp(w));
    k_resid64<<<dim3(red_grid(p.n), p.job->nrhs), kRedThreads, 0, st>>>(p.job->b, w.y64.as<double2>(), rs[i], p.n,
                                                                       w.state.as<KState>(), w.scal.as<double>());
  }
  VS_LAUNCH_CHECK();
}

// Copy every particle's w.scal (nrhs doubles) to p.scal; one synchronisation.
void read_all_scal(std::vector<PartState>& ps, cudaStream_t st) {
  for (auto& p : ps) {
    p.scal.resize(p.job->nrhs);
    VS_CUDA(cudaMemcpyAsync(p.scal.data(), p.job->op->kw.scal.p, p.job->nrhs * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  }
  VS_CUDA(cudaStreamSynchronize(st));
}

// Lockstep inner BiCGSTAB on every particle's w.x / w.r (precision T): rhs r
// of particle p stops at ||r|| <= tol * p.tolr[r], resvec entries scaled by
// p.rscale[r].  Returns with p.cur holding the final states.
template <typename T>
void bicgstab_lockstep(vs_ctx* ctx, std::vector<PartState>& ps, double tol, int maxit, int per_graph, int stag,
                       int mode, cudaStream_t st, int64_t* launches, bool fold_steps) {
  using C = cplx_t<T>;
  const int np = (int)ps.size();
  bool any_active = false;
  for (auto& p : ps) {
    const int nrhs = p.job->nrhs;
    KrylovWork& w = p.job->op->kw;
    p.h.assign(nrhs, KState{});
    for (int r = 0; r < nrhs; ++r) {
      KState& k = p.h[r];
      k.tol_abs = tol * p.tolr[r];
      k.maxit = maxit;
      k.res_scale = p.rscale[r];
      k.flag = 1;
      k.stag_window = stag;
      k.best_res = INFINITY;
    }
    upload_states(w, p.h, st);
    k_copy<T><<<vec_grid(p.n * nrhs), 256, 0, st>>>(w.rt.as<C>(), w.r.as<C>(), p.n * nrhs);
    k_norm<T><<<dim3(red_grid(p.n), nrhs), kRedThreads, 0, st>>>(w.r.as<C>(), p.n, w.state.as<KState>(),
                                                                 w.scal.as<double>());
    *launches += 2;
  }
  VS_LAUNCH_CHECK();
  read_all_scal(ps, st);
  for (auto& p : ps) {
    for (int r = 0; r < p.job->nrhs; ++r) {
      KState& k = p.h[r];
      k.res = p.scal[r];
      k.nres = 1;
      k.best_res = p.scal[r];
      if (!(p.scal[r] > k.tol_abs) || maxit <= 0) {
        k.flag = (p.scal[r] <= k.tol_abs) ? 0 : 1;
        k.skip = 1;
      } else {
        any_active = true;
      }
    }
    p.cur = p.h;
  }
  if (!any_active) return;
  // the graph: every particle's iterations as a branch, then the skip gather;
  // each particle folds its vector steps into its x passes where it can
  GraphCache& gc = std::is_same<T, float>::value ? ctx->pgraph32 : ctx->pgraph64;
  std::vector<FoldPlan> plans(np);
  std::vector<const FoldPlan*> folds(np, nullptr);
  for (int i = 0; i < np; ++i)
    if (fold_steps && make_fold_plan<T>(*ps[i].job->op, ps[i].job->pr, ps[i].job->op->kw, ps[i].job->nrhs, plans[i]))
      folds[i] = &plans[i];
  std::vector<const void*> key = {(const void*)(uintptr_t)per_graph, (const void*)(uintptr_t)mode,
                                  (const void*)(uintptr_t)np, ctx->pskip.p, ctx->pstates.p, ctx->poff.p};
  for (int i = 0; i < np; ++i) key.push_back(folds[i] ? folds[i]->part : nullptr);
  for (auto& p : ps) {
    const vs_op& op = *p.job->op;
    const KrylovWork& w = op.kw;
    const vs_prec* pr = p.job->pr;
    const void* bufs[] = {w.r.p, w.rt.p, w.p.p, w.v_.p, w.s.p, w.t.p, w.ph.p, w.sh.p, w.x.p, w.state.p,
                          w.partials.p, op.t1.p, op.t2.p, (const void*)w.rg.g32, (const void*)w.rg.g64};
    for (const void* v : bufs) key.push_back(v);
    key.push_back((const void*)(uintptr_t)w.rg.per);
    key.push_back((const void*)(uintptr_t)p.job->nrhs);
    key.push_back((const void*)(uintptr_t)(pr ? pr->id : 0));
    key.push_back(pr ? pr->t.p : nullptr);
  }
  if (gc.exec == nullptr || gc.key != key) {
    gc.reset();
    // one idle launch sequence per particle outside capture (first-use attribute calls)
    for (int i = 0; i < np; ++i) {
      PartState& p = ps[i];
      KrylovWork& w = p.job->op->kw;
      std::vector<KState> idle = p.h;
      for (auto& k : idle) k.skip = 1;
      upload_states(w, idle, st);
      bicg_iteration<T>(*p.job->op, p.job->pr, w, w.state.as<KState>(), p.n, p.job->nrhs, mode, st, nullptr,
                        folds[i]);
      *launches += kernels_per_iteration<T>(p.job->pr, folds[i] != nullptr);
    }
    VS_CUDA(cudaStreamSynchronize(st));
    const int naux = std::min(np, kMaxAuxStreams);
    while ((int)ctx->aux.size() < naux) {
      cudaStream_t a;
      VS_CUDA(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
      ctx->aux.push_back(a);
    }
    std::vector<cudaEvent_t> ev(np + 1, nullptr);
    auto destroy_events = [&] {
      for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    };
    cudaGraph_t graph = nullptr;
    try {
      for (auto& e : ev) VS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      VS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        VS_CUDA(cudaEventRecord(ev[np], st));
        for (int i = 0; i < np; ++i) {
          cudaStream_t si = ctx->aux[i % naux];
          VS_CUDA(cudaStreamWaitEvent(si, ev[np], 0));
          PartState& p = ps[i];
          KrylovWork& w = p.job->op->kw;
          for (int k = 0; k < per_graph; ++k)
            bicg_iteration<T>(*p.job->op, p.job->pr, w, w.state.as<KState>(), p.n, p.job->nrhs, mode, si, nullptr,
                              folds[i]);
          VS_CUDA(cudaEventRecord(ev[i], si));
        }
        for (int i = 0; i < np; ++i) VS_CUDA(cudaStreamWaitEvent(st, ev[i], 0));
        k_gather_skip<<<std::min(np, 152), 32, 0, st>>>(ctx->pstates.as<const KState*>(), ctx->poff.as<int>(), np,
                                                          ctx->pskip.as<int>());
        VS_LAUNCH_CHECK();
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
    } catch (...) {
      destroy_events();
      throw;
    }
    destroy_events();
  }
  for (auto& p : ps) {
    KrylovWork& w = p.job->op->kw;
    upload_states(w, p.h, st);
    k_bicg_rho<T><<<dim3(red_grid(p.n), p.job->nrhs), kRedThreads, 0, st>>>(w.rt.as<C>(), w.r.as<C>(), p.n,
                                                                           w.state.as<KState>());
    *launches += 1;
  }
  VS_LAUNCH_CHECK();
  int total = 0;
  for (auto& p : ps) total += p.job->nrhs;
  std::vector<int> skip(total);
  int64_t per_launch = 1;
  for (int i = 0; i < np; ++i)
    per_launch += (int64_t)per_graph * kernels_per_iteration<T>(ps[i].job->pr, folds[i] != nullptr);
  const int max_launch = (maxit + per_graph - 1) / per_graph + 1;
  for (int it = 0; it < max_launch; ++it) {
    VS_CUDA(cudaGraphLaunch(gc.exec, st));
    *launches += per_launch;
    VS_CUDA(cudaMemcpyAsync(skip.data(), ctx->pskip.p, total * sizeof(int), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    bool all = true;
    for (int v : skip) all = all && v;
    if (all) break;
  }
  for (auto& p : ps) {
    p.cur.resize(p.job->nrhs);
    VS_CUDA(cudaMemcpyAsync(p.cur.data(), p.job->op->kw.state.p, p.job->nrhs * sizeof(KState),
                            cudaMemcpyDeviceToHost, st));
  }
  VS_CUDA(cudaStreamSynchronize(st));
  for (auto& p : ps)
    for (auto& k : p.cur)
      if (!k.skip) k.flag = 1;
}

}  // namespace

void solve_bicgstab_particles(vs_ctx* ctx, std::vector<PartJob>& jobs, const SolveParams& prm, cudaStream_t st) {
  const int np = (int)jobs.size();
  std::vector<PartState> ps(np);
  std::vector<int> off(np + 1, 0);
  std::vector<const KState*> sp(np);
  int64_t launches = 0;
  for (int i = 0; i < np; ++i) {
    PartState& p = ps[i];
    p.job = &jobs[i];
    vs_op& op = *jobs[i].op;
    KrylovWork& w = op.kw;
    const int nrhs = jobs[i].nrhs;
    p.n = op.n3;
    SolveParams pi = prm;
    pi.gram_host = jobs[i].gram;
    pi.gram_n = jobs[i].gram_n;
    p.gram.reset(new RhsGramScope(op, w, pi, nrhs, st));
    reduction_buffers(w, nrhs);
    ensure_scratch(op, nrhs, sizeof(double2));
    if (jobs[i].pr) {
      vs_prec& pr = *jobs[i].pr;
      const size_t need = (size_t)pr.L * pr.M * pr.N * 3 * sizeof(double2) * nrhs;
      if (pr.t.bytes < need) pr.t.alloc(need);
    }
    if (prm.mode == VS_SOLVE_FP64) w.ensure<double>(p.n * nrhs);
    else w.ensure<float>(p.n * nrhs);
    w.y64.alloc(p.n * nrhs * sizeof(double2));
    w.r64.alloc(p.n * nrhs * sizeof(double2));
    off[i + 1] = off[i] + nrhs;
    sp[i] = w.state.as<KState>();
    jobs[i].out.assign(nrhs, SolveResult{});
  }
  ctx->pstates.alloc(np * sizeof(KState*));
  ctx->poff.alloc((np + 1) * sizeof(int));
  ctx->pskip.alloc(std::max(1, off[np]) * sizeof(int));
  VS_CUDA(cudaMemcpyAsync(ctx->pstates.p, sp.data(), np * sizeof(KState*), cudaMemcpyHostToDevice, st));
  VS_CUDA(cudaMemcpyAsync(ctx->poff.p, off.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  // ||b||, and a zero initial guess (the particles entry starts from x = 0)
  std::vector<const double2*> bs(np);
  for (int i = 0; i < np; ++i) bs[i] = jobs[i].b;
  enqueue_norms(ps, bs, st);
  read_all_scal(ps, st);
  for (int i = 0; i < np; ++i) {
    PartState& p = ps[i];
    const int nrhs = jobs[i].nrhs;
    p.bnorm = p.scal;
    p.bsafe.resize(nrhs);
    for (int r = 0; r < nrhs; ++r) {
      if (!std::isfinite(p.bnorm[r])) throw Error(VS_ERR_NONFINITE, "right-hand side has NaN or Inf entries");
      p.bsafe[r] = p.bnorm[r] > 0 ? p.bnorm[r] : 1.0;
    }
    VS_CUDA(cudaMemsetAsync(jobs[i].x, 0, p.n * nrhs * sizeof(double2), st));
    p.inner2.assign(nrhs, 0);
    p.flag.assign(nrhs, 1);
    p.refine.assign(nrhs, 0);
  }
  std::vector<double2*> xs(np), r64s(np), rws(np);
  for (int i = 0; i < np; ++i) {
    xs[i] = jobs[i].x;
    r64s[i] = jobs[i].op->kw.r64.as<double2>();
  }
  if (prm.mode == VS_SOLVE_FP64) {
    for (int i = 0; i < np; ++i) {
      PartState& p = ps[i];
      KrylovWork& w = jobs[i].op->kw;
      const int64_t m = p.n * jobs[i].nrhs;
      k_zero<double><<<vec_grid(m), 256, 0, st>>>(w.x.as<double2>(), m);
      k_copy<double><<<vec_grid(m), 256, 0, st>>>(w.r.as<double2>(), jobs[i].b, m);
      p.tolr = p.bsafe;
      p.rscale.resize(jobs[i].nrhs);
      for (int r = 0; r < jobs[i].nrhs; ++r) p.rscale[r] = 1.0 / p.bsafe[r];
    }
    bicgstab_lockstep<double>(ctx, ps, prm.tol, prm.maxit, prm.per_graph, 0, prm.op_mode, st, &launches,
                              prm.fold_steps);
    for (int i = 0; i < np; ++i) {
      KrylovWork& w = jobs[i].op->kw;
      const int64_t m = ps[i].n * jobs[i].nrhs;
      k_copy<double><<<vec_grid(m), 256, 0, st>>>(jobs[i].x, w.x.as<double2>(), m);
    }
    enqueue_residuals(ps, xs, r64s, prm.op_mode, st);
    read_all_scal(ps, st);
    for (int i = 0; i < np; ++i) {
      PartState& p = ps[i];
      for (int r = 0; r < jobs[i].nrhs; ++r) {
        SolveResult& o = jobs[i].out[r];
        o.flag = p.cur[r].flag;
        o.iter = o.inner_iters = p.cur[r].iter2 * 0.5;
        o.relres = p.bnorm[r] > 0 ? p.scal[r] / p.bnorm[r] : 0.0;
        if (p.bnorm[r] == 0) o.flag = 0;
        else if (o.flag == 0 && o.relres > prm.tol) o.flag = 1;
      }
    }
  } else {
    // mixed: c64 inner solves of all particles in lockstep inside FP64 refinement
    for (int i = 0; i < np; ++i) {
      const int64_t m = ps[i].n * jobs[i].nrhs;
      k_copy<double><<<vec_grid(m), 256, 0, st>>>(r64s[i], jobs[i].b, m);
      ps[i].rn = ps[i].bnorm;
    }
    VS_LAUNCH_CHECK();
    DevBuf scd;
    int maxr = 1;
    for (auto& j : jobs) maxr = std::max(maxr, j.nrhs);
    std::vector<DevBuf> scales(np);
    for (int step = 0; step <= prm.max_refine; ++step) {
      bool all_done = true;
      int used = 0;
      for (auto& p : ps)
        for (int r = 0; r < p.job->nrhs; ++r) {
          const bool done = p.rn[r] <= prm.tol * p.bnorm[r] || p.flag[r] >= 4;
          if (p.rn[r] <= prm.tol * p.bnorm[r]) p.flag[r] = 0;
          all_done = all_done && done;
          used = std::max(used, p.inner2[r]);
        }
      if (all_done || step == prm.max_refine || used >= 2 * prm.maxit) break;
      // per-rhs inner tolerance relative to the scaled residual; one common
      // inner tolerance tmin, expressed per rhs through tolr = itol / tmin
      double tmin = 1.0;
      std::vector<std::vector<double>> itol(np);
      for (int i = 0; i < np; ++i) {
        PartState& p = ps[i];
        const int nrhs = jobs[i].nrhs;
        itol[i].resize(nrhs);
        std::vector<double> scale(nrhs);
        p.rscale.resize(nrhs);
        for (int r = 0; r < nrhs; ++r) {
          const bool done = p.rn[r] <= prm.tol * p.bnorm[r] || p.flag[r] >= 4;
          scale[r] = p.rn[r] > 0 ? 1.0 / p.rn[r] : 0.0;
          const double t = prm.inner_tol > 0 ? prm.inner_tol
                                             : std::max(0.3 * prm.tol * p.bnorm[r] / p.rn[r], prm.inner_floor);
          itol[i][r] = done ? 2.0 : std::min(t, 0.5);
          p.rscale[r] = p.bnorm[r] > 0 ? p.rn[r] / p.bnorm[r] : 0.0;
          p.refine[r] += done ? 0 : 1;
          tmin = std::min(tmin, itol[i][r]);
        }
        KrylovWork& w = jobs[i].op->kw;
        scales[i].alloc(nrhs * sizeof(double));
        VS_CUDA(cudaMemcpyAsync(scales[i].p, scale.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, st));
        k_scale_down<<<dim3(vec_grid(p.n), nrhs), 256, 0, st>>>(r64s[i], w.r.as<float2>(), p.n, scales[i].as<double>());
        k_zero<float><<<vec_grid(p.n * nrhs), 256, 0, st>>>(w.x.as<float2>(), p.n * nrhs);
        launches += 2;
      }
      for (int i = 0; i < np; ++i) {
        ps[i].tolr.resize(jobs[i].nrhs);
        for (int r = 0; r < jobs[i].nrhs; ++r) ps[i].tolr[r] = itol[i][r] / tmin;
      }
      bicgstab_lockstep<float>(ctx, ps, tmin, prm.maxit - used / 2, prm.per_graph, kStagnationWindow, prm.op_mode, st,
                               &launches, prm.fold_steps);
      bool progressed = false;
      for (int i = 0; i < np; ++i) {
        PartState& p = ps[i];
        const int nrhs = jobs[i].nrhs;
        for (int r = 0; r < nrhs; ++r) {
          p.inner2[r] += p.cur[r].iter2;
          if (p.cur[r].flag >= 4 && p.cur[r].iter2 == 0 && !(p.rn[r] <= prm.tol * p.bnorm[r])) p.flag[r] = p.cur[r].flag;
          progressed = progressed || p.cur[r].iter2 > 0;
        }
        KrylovWork& w = jobs[i].op->kw;
        VS_CUDA(cudaMemcpyAsync(scales[i].p, p.rn.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, st));
        k_update64<<<dim3(vec_grid(p.n), nrhs), 256, 0, st>>>(jobs[i].x, w.x.as<float2>(), p.n, scales[i].as<double>());
        launches += 1;
      }
      VS_LAUNCH_CHECK();
      enqueue_residuals(ps, xs, r64s, prm.op_mode, st);
      read_all_scal(ps, st);
      for (auto& p : ps) p.rn = p.scal;
      if (!progressed) break;
    }
    for (int i = 0; i < np; ++i) {
      PartState& p = ps[i];
      for (int r = 0; r < jobs[i].nrhs; ++r) {
        SolveResult& o = jobs[i].out[r];
        o.flag = (p.rn[r] <= prm.tol * p.bnorm[r]) ? 0 : (p.flag[r] >= 4 ? p.flag[r] : 1);
        o.relres = p.bnorm[r] > 0 ? p.rn[r] / p.bnorm[r] : 0.0;
        o.iter = o.inner_iters = p.inner2[r] * 0.5;
        o.refinements = p.refine[r];
        if (p.bnorm[r] == 0) o.flag = 0;
      }
    }
  }
  for (auto& j : jobs)
    for (auto& o : j.out) o.launches = launches;
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

// A complex chunk partial in its 16-byte slot: the float-float real and
// imaginary parts as float4 (hi, lo, hi, lo) for c64, a double2 for c128.
// The c64 sums stay on the FP32 pipes until one thread widens the total
// (GB300 runs FP64 at a small fraction of its FP32 rate).
__device__ __forceinline__ void put_cslot(double2* p, FF2 re, FF2 im) {
  *reinterpret_cast<float4*>(p) = make_float4(re.hi, re.lo, im.hi, im.lo);
}
__device__ __forceinline__ void put_cslot(double2* p, double re, double im) { *p = make_double2(re, im); }
__device__ __forceinline__ void get_cslot(const double2* p, FF2& re, FF2& im) {
  const float4 f = *reinterpret_cast<const float4*>(p);
  re = FF2{f.x, f.y};
  im = FF2{f.z, f.w};
}
__device__ __forceinline__ void get_cslot(const double2* p, double& re, double& im) {
  const double2 d = *p;
  re = d.x;
  im = d.y;
}
// CTA sum of one complex value per thread (blockDim.x <= 256): warp trees,
// then thread 0 adds the warps in order; the total in thread 0.
template <typename V>
__device__ __forceinline__ void cta_csum(V& re, V& im) {
  __shared__ V sre[8], sim[8];
  re = warp_sum_v(re);
  im = warp_sum_v(im);
  if ((threadIdx.x & 31) == 0) {
    sre[threadIdx.x >> 5] = re;
    sim[threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    re = sre[0];
    im = sim[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      add_slot(re, sre[k]);
      add_slot(im, sim[k]);
    }
  }
}
// Per-thread x^H y over [i0, i1) with stride blockDim.x, four elements'
// loads issued together.
template <typename T>
__device__ __forceinline__ void chunk_dot(const cplx_t<T>* __restrict__ x, const cplx_t<T>* __restrict__ y,
                                          int64_t i0, int64_t i1, Acc<T>& a) {
  using C = cplx_t<T>;
  const int64_t st = blockDim.x;
  for (int64_t b = i0 + threadIdx.x; b < i1; b += 4 * st) {
    C u[4], v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (b + k * st < i1) {
        u[k] = x[b + k * st];
        v[k] = y[b + k * st];
      }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (b + k * st < i1) a.dot(u[k], v[k]);
  }
}

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
  chunk_dot<T>(v, w, i0, i1, a);
  SlotV<T> re = a.vre(), im = a.vim();
  cta_csum(re, im);
  if (threadIdx.x == 0) put_cslot(part + (int64_t)j * nchunk + blockIdx.x, re, im);
}

// Sum of the nchunk complex slots at part (one CTA), widened to double in thread 0.
template <typename T>
__device__ __forceinline__ double2 sum_cslots(const double2* __restrict__ part, int nchunk) {
  using V = SlotV<T>;
  V r{}, q{};
  for (int c = threadIdx.x; c < nchunk; c += blockDim.x) {
    V a, b;
    get_cslot(part + c, a, b);
    add_slot(r, a);
    add_slot(q, b);
  }
  cta_csum(r, q);
  return threadIdx.x == 0 ? make_double2(widen(r), widen(q)) : make_double2(0, 0);
}

// hp[j] = sum of the partials of vector j; H(:,k) += hp (column k of the Hessenberg)
template <typename T>
__global__ void k_gm_dots_final(const double2* __restrict__ part, int nchunk, double2* __restrict__ hp,
                                double2* __restrict__ Hcol, GState* st) {
  if (st->skip) return;
  const int j = blockIdx.x;
  const double2 t = sum_cslots<T>(part + (int64_t)j * nchunk, nchunk);
  if (threadIdx.x == 0) {
    hp[j] = t;
    Hcol[j].x += t.x;
    Hcol[j].y += t.y;
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
  const SlotV<T> v[1] = {a.vre()};
  double t[1];
  if (grid_reduce<1>(v, partials, counter, t) && threadIdx.x == 0) *Hk1 = make_double2(sqrt(t[0]), 0.0);
}

// V_{k+1} = w / H(k+1,k) (the reciprocal taken once per CTA)
template <typename T>
__global__ void k_gm_scale(const cplx_t<T>* __restrict__ w, cplx_t<T>* __restrict__ vnext, int64_t n,
                           const double2* Hk1, const GState* st) {
  if (st->skip) return;
  __shared__ T s_s;
  if (threadIdx.x == 0) {
    const double h = Hk1->x;
    s_s = (T)(h > 0 ? 1.0 / h : 0.0);
  }
  __syncthreads();
  const T s = s_s;
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
  __shared__ T s_s;
  if (threadIdx.x == 0) {
    const double h = *nrm;
    s_s = (T)(h > 0 ? 1.0 / h : 0.0);
  }
  __syncthreads();
  const T s = s_s;
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
    *launches += pr ? prec_launches<T>(*pr) : 1;
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
      matvec<T>(op, d, tmp, 1, op_mode, nullptr, st, 0, rgp(w));
      k_sub<T><<<g, 256, 0, st>>>(rin, tmp, tmp, n);
      minv(tmp, V);
      *launches += 6;
    }
    k_norm<T><<<red_grid(n), kRedThreads, 0, st>>>(V, n, ks, w.scal.as<double>());
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
      matvec<T>(op, vk, tmp, 1, op_mode, &gs->skip, st, 0, rgp(w));
      minv(tmp, wv);
      double2* Hcol = H + (int64_t)k * (m + 1);
      for (int pass = 0; pass < 2; ++pass) {
        k_gm_dots<T><<<dim3(nchunk, k + 1), 256, 0, st>>>(V, wv, n, part, nchunk, gs);
        k_gm_dots_final<T><<<k + 1, 256, 0, st>>>(part, nchunk, hp, Hcol, gs);
        k_gm_axpy<T><<<g, 256, (k + 1) * sizeof(C), st>>>(V, wv, n, k + 1, hp, gs);
      }
      // partial sums and counter of the shared reduction state (device addresses)
      k_gm_norm<T><<<red_grid(n), kRedThreads, 0, st>>>(wv, n, w.partials.as<double>(), &ks->counter, Hcol + k + 1, gs);
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

// ===========================================================================
// GCRO-DR, MATLAB-style pgmresDR(A, b, restart, tol, maxit, ritz, [], [], M)
// (src/src_numeric/src_iterative/pgmresDR.m:73-281, pgmresDR_iter.m:1-142,
// getHarmVecs1.m, getHarmVecs2.m; Parks, de Sturler, Mackey, Johnson and
// Maiti, SIAM J. Sci. Comput. 28 (2006) 1651-1674), right preconditioned as
// the JVIE solvers call it (JVIE_Solver_const_GPU.m:400-427).  Each cycle runs
// up to `restart` Arnoldi steps on (I - C C^H) A M; after it the `ritz`
// harmonic Ritz vectors of smallest magnitude span the recycled space U with
// C = A M U orthonormal, which the next cycle deflates.  The Arnoldi steps
// and their residual estimate reuse the GMRES kernels above (classical
// Gram-Schmidt against [C | V] at once, C stored just below V, applied twice;
// C is orthogonal to V, so this equals projecting against C and then V as
// pgmresDR_iter.m:99-107 does); the unrotated Hessenberg
// is kept for the harmonic Ritz problems.  Between cycles the host solves the
// small least-squares, QR and eigen problems (vs_dense.cu) from Gram products
// formed on the device, and tall-skinny combinations on the device form the
// solution update, the new residual and the next U and C.
// ===========================================================================

// Partial dots X_i^H Y_j over one chunk of kDotChunk entries, X = [Xa (na
// vectors) | Xb], Y (ny vectors), all of stride n; grid (nchunk, nx, ny).
template <typename T>
__global__ void __launch_bounds__(256) k_dr_gram(const cplx_t<T>* __restrict__ Xa, int na,
                                                 const cplx_t<T>* __restrict__ Xb, const cplx_t<T>* __restrict__ Y,
                                                 int64_t n, double2* __restrict__ part, int nchunk) {
  const int i = blockIdx.y, j = blockIdx.z;
  const cplx_t<T>* x = i < na ? Xa + (int64_t)i * n : Xb + (int64_t)(i - na) * n;
  const cplx_t<T>* y = Y + (int64_t)j * n;
  const int64_t i0 = (int64_t)blockIdx.x * kDotChunk;
  const int64_t i1 = (n < i0 + kDotChunk) ? n : i0 + kDotChunk;
  Acc<T> a;
  chunk_dot<T>(x, y, i0, i1, a);
  SlotV<T> re = a.vre(), im = a.vim();
  cta_csum(re, im);
  if (threadIdx.x == 0) put_cslot(part + ((int64_t)i * gridDim.z + j) * nchunk + blockIdx.x, re, im);
}

// G(i, j) (column-major, nx rows) = sum of the chunk partials of pair (i, j);
// one CTA per pair, block b = i * ny + j.
template <typename T>
__global__ void k_dr_gram_final(const double2* __restrict__ part, int nchunk, int nx, int ny, double2* __restrict__ G) {
  const int b = blockIdx.x, i = b / ny, j = b - i * ny;
  const double2 t = sum_cslots<T>(part + (int64_t)b * nchunk, nchunk);
  if (threadIdx.x == 0) G[i + (int64_t)j * nx] = t;
}

// out_c = (accumulate ? out_c : 0) + sum_j X_j coef(j, c) for c < ncol, with
// X = [Xa (na vectors) | Xb (nb vectors)] and coef column-major (na + nb rows);
// blockIdx.y picks a tile of 4 output columns, so each X entry is read once
// per tile.
template <typename T>
__global__ void __launch_bounds__(256) k_dr_combine(const cplx_t<T>* __restrict__ Xa, int na,
                                                    const cplx_t<T>* __restrict__ Xb, int nb,
                                                    const double2* __restrict__ coef, int ncol,
                                                    cplx_t<T>* __restrict__ out, int64_t n, int accumulate) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* cs = reinterpret_cast<C*>(smem_raw);  // [na + nb][4]
  const int nx = na + nb, c0 = blockIdx.y * 4;
  for (int u = threadIdx.x; u < nx * 4; u += blockDim.x) {
    const int j = u >> 2, t = u & 3;
    cs[u] = (c0 + t < ncol) ? ccast<C>(coef[j + (int64_t)(c0 + t) * nx]) : czero<C>();
  }
  __syncthreads();
  const int nt = min(4, ncol - c0);
  GRID_LOOP(e, n) {
    C acc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) acc[t] = (accumulate && t < nt) ? out[(int64_t)(c0 + t) * n + e] : czero<C>();
    for (int j = 0; j < nx; ++j) {
      const C v = j < na ? Xa[(int64_t)j * n + e] : Xb[(int64_t)(j - na) * n + e];
#pragma unroll
      for (int t = 0; t < 4; ++t) acc[t] = cfma(cs[j * 4 + t], v, acc[t]);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (t < nt) out[(int64_t)(c0 + t) * n + e] = acc[t];
  }
}

// Column k of the unrotated Hessenberg (len entries) into the copy that the
// Givens kernel rotates.
__global__ void k_dr_copycol(const GState* st, const double2* __restrict__ src, double2* __restrict__ dst, int len) {
  if (st->skip) return;
  for (int i = threadIdx.x; i < len; i += blockDim.x) dst[i] = src[i];
}

using dense::cd;

// G = [Xa | Xb]^H Y on the host ((na + nb) x ny, column-major).
template <typename T>
static std::vector<cd> dr_gram(KrylovWork& w, const cplx_t<T>* Xa, int na, const cplx_t<T>* Xb, int nb,
                               const cplx_t<T>* Y, int ny, int64_t n, cudaStream_t st, int64_t* launches) {
  const int nx = na + nb;
  std::vector<cd> G((size_t)nx * ny, 0);
  if (nx == 0 || ny == 0) return G;
  const int nchunk = ceil_div(n, kDotChunk);
  w.rgpart.alloc((size_t)nx * ny * nchunk * sizeof(double2));
  w.rgram.alloc((size_t)nx * ny * sizeof(double2));
  k_dr_gram<T><<<dim3(nchunk, nx, ny), 256, 0, st>>>(Xa, na, nb ? Xb : Xa, Y, n, w.rgpart.as<double2>(), nchunk);
  k_dr_gram_final<T><<<nx * ny, 256, 0, st>>>(w.rgpart.as<double2>(), nchunk, nx, ny, w.rgram.as<double2>());
  VS_LAUNCH_CHECK();
  *launches += 2;
  std::vector<double2> h((size_t)nx * ny);
  VS_CUDA(cudaMemcpyAsync(h.data(), w.rgram.p, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
  for (size_t i = 0; i < h.size(); ++i) G[i] = cd(h[i].x, h[i].y);
  return G;
}

// out (ncol vectors) (+)= [Xa | Xb] coef, coef (na + nb) x ncol column-major.
template <typename T>
static void dr_combine(KrylovWork& w, const cplx_t<T>* Xa, int na, const cplx_t<T>* Xb, int nb,
                       const std::vector<cd>& coef, int ncol, cplx_t<T>* out, int64_t n, bool accumulate,
                       cudaStream_t st, int64_t* launches) {
  const int nx = na + nb;
  if (nx == 0 || ncol == 0) return;
  std::vector<double2> h((size_t)nx * ncol);
  for (size_t i = 0; i < h.size(); ++i) h[i] = make_double2(coef[i].real(), coef[i].imag());
  // stream-ordered after the previous combine that read the coefficients; the
  // copy from pageable memory is staged before the call returns
  w.rcoef.alloc(h.size() * sizeof(double2));
  VS_CUDA(cudaMemcpyAsync(w.rcoef.p, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
  const size_t smem = (size_t)nx * 4 * sizeof(cplx_t<T>);
  k_dr_combine<T><<<dim3(vec_grid(n), ceil_div(ncol, 4)), 256, smem, st>>>(
      Xa, na, nb ? Xb : Xa, nb, w.rcoef.as<double2>(), ncol, out, n, accumulate ? 1 : 0);
  VS_LAUNCH_CHECK();
  *launches += 1;
}

template <typename T>
static void gcrodr_buffers(KrylovWork& w, int64_t n, int m, int kr) {
  using C = cplx_t<T>;
  const size_t kv = (size_t)std::max(kr, 1) * n * sizeof(C);
  w.rCV.alloc((size_t)(kr + m + 1) * n * sizeof(C));
  w.rU.alloc(kv);
  w.rU2.alloc(kv);
  w.rC2.alloc(kv);
  w.rz.alloc(n * sizeof(C));
  w.rr.alloc(n * sizeof(C));
  w.rBH.alloc((size_t)(kr + m + 1) * m * sizeof(double2));
  // the Gram-Schmidt pass covers up to kr + m vectors of [C | V]
  w.ghp.alloc((size_t)(kr + m + 1) * sizeof(double2));
  w.gpart.alloc((size_t)(kr + m + 1) * ceil_div(n, kDotChunk) * sizeof(double2));
}

// Inner GCRO-DR on A d = rin (precision T, d overwritten), right
// preconditioned: A M z = rin, d = M z.  Convergence: the Arnoldi residual
// estimate <= itol * ||rin||.  Returns the Arnoldi steps taken; *flag 0
// converged, 1 not, 4 breakdown, 5 non-finite.
template <typename T>
static int gcrodr_core(const vs_op& op, const vs_prec* pr, KrylovWork& w, int64_t n, const cplx_t<T>* rin,
                       cplx_t<T>* d, double itol, int m, int kr, int maxit, int op_mode, double res_scale,
                       double* resvec_dev, int resvec_cap, int64_t* nres_out, int* flag, cudaStream_t st,
                       int64_t* launches) {
  using C = cplx_t<T>;
  const int g = vec_grid(n);
  const int nchunk = ceil_div(n, kDotChunk);
  // [C | V]: the kc recycled C vectors sit in the slots just below V, so one
  // Gram-Schmidt pass projects against both
  C* V = w.rCV.as<C>() + (int64_t)kr * n;
  C* wv = w.gw.as<C>();
  C* tmp = w.gtmp.as<C>();
  C* U = w.rU.as<C>();
  C* U2 = w.rU2.as<C>();
  C* C2 = w.rC2.as<C>();
  C* z = w.rz.as<C>();
  C* r = w.rr.as<C>();
  double2* H = w.gH.as<double2>();
  double2* BH = w.rBH.as<double2>();
  double2* hp = w.ghp.as<double2>();
  double2* part = w.gpart.as<double2>();
  GState* gs = w.gstate.as<GState>();
  KState* ks = w.state.as<KState>();
  auto rprec = [&](const C* in, C* out, const int* skip) {
    if (pr) prec_apply<T>(*pr, in, out, 1, skip, st);
    else k_copy<T><<<g, 256, 0, st>>>(out, in, n);
    *launches += pr ? prec_launches<T>(*pr) : 1;
  };
  auto norm_dev = [&](const C* u) {
    k_norm<T><<<red_grid(n), kRedThreads, 0, st>>>(u, n, ks, w.scal.as<double>());
    double v = 0;
    VS_CUDA(cudaMemcpyAsync(&v, w.scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    *launches += 1;
    return v;
  };
  k_copy<T><<<g, 256, 0, st>>>(r, rin, n);
  VS_CUDA(cudaMemsetAsync(z, 0, n * sizeof(C), st));
  *launches += 1;
  const double bn = norm_dev(r);
  const double tol_abs = itol * bn;
  if (resvec_dev && resvec_cap > 0) {
    const double v0 = bn * res_scale;
    VS_CUDA(cudaMemcpyAsync(resvec_dev, &v0, sizeof(double), cudaMemcpyHostToDevice, st));
  }
  int64_t nres = 1;
  *flag = 1;
  int steps = 0, kc = 0;
  C* Cm = V;  // first of the kc recycled vectors (none yet)
  for (;;) {
    const double beta = norm_dev(r);
    if (!std::isfinite(beta)) {
      *flag = 5;
      break;
    }
    if (!(beta > tol_abs)) {
      *flag = 0;
      break;
    }
    if (steps >= maxit) break;
    k_scale_by<T><<<g, 256, 0, st>>>(r, V, n, w.scal.as<double>());
    // column k of BH (leading dimension ld): rows 0..kc-1 = C^H A M v_k,
    // rows kc..kc+k+1 = the unrotated Hessenberg column
    const int ld = kc + m + 1;
    VS_CUDA(cudaMemsetAsync(H, 0, (size_t)(m + 1) * m * sizeof(double2), st));
    VS_CUDA(cudaMemsetAsync(BH, 0, (size_t)ld * m * sizeof(double2), st));
    VS_CUDA(cudaMemsetAsync(w.gg.p, 0, (m + 1) * sizeof(double2), st));
    const double2 g0 = make_double2(beta, 0);
    VS_CUDA(cudaMemcpyAsync(w.gg.p, &g0, sizeof(double2), cudaMemcpyHostToDevice, st));
    GState h{};
    h.m = m;
    h.resvec = resvec_dev;
    h.resvec_cap = resvec_cap;
    h.res_scale = res_scale;
    h.tol_abs = tol_abs;
    h.k = 0;
    h.skip = 0;
    h.flag = 1;
    h.res = beta;
    h.nres = (int)nres;
    VS_CUDA(cudaMemcpyAsync(gs, &h, sizeof(GState), cudaMemcpyHostToDevice, st));
    *launches += 1;
    const int kmax = std::min(m, maxit - steps);
    GState cur{};
    for (int k = 0; k < kmax; ++k) {
      rprec(V + (int64_t)k * n, tmp, &gs->skip);
      matvec<T>(op, tmp, wv, 1, op_mode, &gs->skip, st, 0, rgp(w));
      *launches += 5;
      double2* col = BH + (int64_t)k * ld;
      const int nb = kc + k + 1;  // C_0..C_kc-1, V_0..V_k
      for (int pass = 0; pass < 2; ++pass) {
        k_gm_dots<T><<<dim3(nchunk, nb), 256, 0, st>>>(Cm, wv, n, part, nchunk, gs);
        k_gm_dots_final<T><<<nb, 256, 0, st>>>(part, nchunk, hp, col, gs);
        k_gm_axpy<T><<<g, 256, nb * sizeof(C), st>>>(Cm, wv, n, nb, hp, gs);
      }
      double2* Hcol = col + kc;
      k_gm_norm<T><<<red_grid(n), kRedThreads, 0, st>>>(wv, n, w.partials.as<double>(), &ks->counter, Hcol + k + 1, gs);
      k_gm_scale<T><<<g, 256, 0, st>>>(wv, V + (int64_t)(k + 1) * n, n, Hcol + k + 1, gs);
      k_dr_copycol<<<1, 64, 0, st>>>(gs, Hcol, H + (int64_t)k * (m + 1), k + 2);
      k_gm_givens<<<1, 32, 0, st>>>(gs, H, w.gcs.as<double>(), w.gsn.as<double2>(), w.gg.as<double2>());
      VS_LAUNCH_CHECK();
      *launches += 10;
      if ((k + 1) % 4 == 0 || k == kmax - 1) {
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
    if (cur.flag == 5) {
      *flag = 5;
      break;
    }
    if (kd == 0) {
      *flag = 4;
      break;
    }
    const bool conv = cur.flag == 0;
    const bool more = !conv && steps < maxit;
    // the small dense problems of the cycle; one that fails (a rank-deficient
    // least-squares matrix, a harmonic Ritz problem whose QR iteration does not
    // converge) ends the solve as a breakdown, flag 4, keeping the iterate so far
    try {
    // B = C^H A M V (kc x kd) and the unrotated Hessenberg ((kd+1) x kd) on the host
    std::vector<double2> bhh((size_t)ld * kd);
    VS_CUDA(cudaMemcpyAsync(bhh.data(), BH, bhh.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VS_CUDA(cudaStreamSynchronize(st));
    std::vector<cd> Hh((size_t)(kd + 1) * kd);
    for (int j = 0; j < kd; ++j)
      for (int i = 0; i <= kd; ++i) {
        const double2 e = bhh[kc + i + (size_t)j * ld];
        Hh[i + (size_t)j * (kd + 1)] = cd(e.x, e.y);
      }
    auto bh = [&](int i, int j) { return cd(bhh[i + (size_t)j * ld].x, bhh[i + (size_t)j * ld].y); };
    if (kc == 0) {
      // first cycle (pgmresDR.m:190-221)
      std::vector<cd> rhs(kd + 1, 0);
      rhs[0] = beta;
      const std::vector<cd> y = dense::lstsq(Hh, kd + 1, kd, rhs);
      dr_combine<T>(w, V, kd, nullptr, 0, y, 1, z, n, true, st, launches);
      std::vector<cd> t(kd + 1, 0);
      for (int j = 0; j < kd; ++j)
        for (int i = 0; i <= kd; ++i) t[i] -= Hh[i + (size_t)j * (kd + 1)] * y[j];
      dr_combine<T>(w, V, kd + 1, nullptr, 0, t, 1, r, n, true, st, launches);
      const int kk = std::min(kr, kd - 1);
      if (more && kk >= 1) {
        const dense::Mat P = dense::harm_vecs1(kd, kk, Hh);
        dense::Mat HP((size_t)(kd + 1) * kk, 0), Q, R;
        for (int c = 0; c < kk; ++c)
          for (int j = 0; j < kd; ++j)
            for (int i = 0; i <= kd; ++i) HP[i + (size_t)c * (kd + 1)] += Hh[i + (size_t)j * (kd + 1)] * P[j + (size_t)c * kd];
        dense::qr_econ(HP, kd + 1, kk, Q, R);
        const dense::Mat cu = dense::right_div_upper(P, kd, kk, R);
        dr_combine<T>(w, V, kd, nullptr, 0, cu, kk, U2, n, false, st, launches);
        dr_combine<T>(w, V, kd + 1, nullptr, 0, Q, kk, C2, n, false, st, launches);
        std::swap(U, U2);
        Cm = V - (int64_t)kk * n;
        VS_CUDA(cudaMemcpyAsync(Cm, C2, (size_t)kk * n * sizeof(C), cudaMemcpyDeviceToDevice, st));
        kc = kk;
      }
    } else {
      // later cycles (pgmresDR.m:236-258): U scaled to unit columns by D
      const int mm = kc + kd;
      const std::vector<cd> G = dr_gram<T>(w, Cm, kc, V, kd + 1, U, kc, n, st, launches);     // [C V]^H U
      const std::vector<cd> Gr = dr_gram<T>(w, Cm, kc, V, kd + 1, r, 1, n, st, launches);     // [C V]^H r
      const std::vector<cd> UU = dr_gram<T>(w, U, kc, nullptr, 0, U, kc, n, st, launches);    // U^H U
      std::vector<double> Dv(kc);
      for (int i = 0; i < kc; ++i) Dv[i] = 1.0 / std::sqrt(UU[i + (size_t)i * kc].real());
      dense::Mat H2((size_t)(mm + 1) * mm, 0);
      for (int i = 0; i < kc; ++i) H2[i + (size_t)i * (mm + 1)] = Dv[i];
      for (int j = 0; j < kd; ++j) {
        for (int i = 0; i < kc; ++i) H2[i + (size_t)(kc + j) * (mm + 1)] = bh(i, j);
        for (int i = 0; i <= kd; ++i) H2[kc + i + (size_t)(kc + j) * (mm + 1)] = Hh[i + (size_t)j * (kd + 1)];
      }
      const std::vector<cd> y = dense::lstsq(H2, mm + 1, mm, Gr);
      std::vector<cd> cx(y);
      for (int i = 0; i < kc; ++i) cx[i] *= Dv[i];
      dr_combine<T>(w, U, kc, V, kd, cx, 1, z, n, true, st, launches);
      std::vector<cd> t(mm + 1, 0);
      for (int j = 0; j < mm; ++j)
        for (int i = 0; i <= mm; ++i) t[i] -= H2[i + (size_t)j * (mm + 1)] * y[j];
      dr_combine<T>(w, Cm, kc, V, kd + 1, t, 1, r, n, true, st, launches);
      if (more) {
        dense::Mat Wm((size_t)(mm + 1) * mm, 0);
        for (int j = 0; j < kc; ++j)
          for (int i = 0; i <= mm; ++i) Wm[i + (size_t)j * (mm + 1)] = G[i + (size_t)j * (mm + 1)] * Dv[j];
        for (int j = kc; j < mm; ++j) Wm[j + (size_t)j * (mm + 1)] = 1;
        const dense::Mat P = dense::harm_vecs2(mm, kc, H2, Wm);
        dense::Mat HP((size_t)(mm + 1) * kc, 0), Q, R;
        for (int c = 0; c < kc; ++c)
          for (int j = 0; j < mm; ++j)
            for (int i = 0; i <= mm; ++i) HP[i + (size_t)c * (mm + 1)] += H2[i + (size_t)j * (mm + 1)] * P[j + (size_t)c * mm];
        dense::qr_econ(HP, mm + 1, kc, Q, R);
        dense::Mat cu = dense::right_div_upper(P, mm, kc, R);
        for (int c = 0; c < kc; ++c)
          for (int i = 0; i < kc; ++i) cu[i + (size_t)c * mm] *= Dv[i];
        dr_combine<T>(w, U, kc, V, kd, cu, kc, U2, n, false, st, launches);
        dr_combine<T>(w, Cm, kc, V, kd + 1, Q, kc, C2, n, false, st, launches);
        std::swap(U, U2);
        VS_CUDA(cudaMemcpyAsync(Cm, C2, (size_t)kc * n * sizeof(C), cudaMemcpyDeviceToDevice, st));
      }
    }
    } catch (const dense::Failure&) {
      *flag = 4;
      break;
    }
    if (conv) {
      *flag = 0;
      break;
    }
    if (steps >= maxit) break;
  }
  rprec(z, d, nullptr);
  VS_LAUNCH_CHECK();
  *nres_out = std::min<int64_t>(nres, resvec_cap);
  return steps;
}

// FP64 iterative refinement around the inner GMRES(m) (DR false) or GCRO-DR
// (DR true) solve in precision T.
template <typename T, bool DR = false>
static void gmres_refine(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm,
                         SolveResult& out, cudaStream_t st, double bnorm, int64_t& launches, double* rv, int cap) {
  using C = cplx_t<T>;
  KrylovWork& w = op.kw;
  const int64_t n = op.n3;
  const int m = std::max(1, std::min(prm.restart, prm.maxit));
  const int kr = std::max(0, std::min(prm.ritz, m - 1));
  gmres_buffers<T>(w, n, m);
  if (DR) gcrodr_buffers<T>(w, n, m, kr);
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
    if (DR)
      steps += gcrodr_core<T>(op, pr, w, n, w.r.as<C>(), w.gd.as<C>(), itol, m, kr, prm.maxit - steps, prm.op_mode,
                              rn / bnorm, rvk, capk, &nk, &f, st, &launches);
    else
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

template <bool DR>
static void solve_gmres_impl(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm,
                             SolveResult& out, cudaStream_t st) {
  const int64_t n = op.n3;
  KrylovWork& w = op.kw;
  RhsGramScope gram_scope(op, w, prm, 1, st);
  reduction_buffers(w, 1);
  std::vector<KState> zero(1);
  upload_states(w, zero, st);
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
  if (prm.mode == VS_SOLVE_FP64) gmres_refine<double, DR>(op, pr, b, x, prm, out, st, bnorm, launches, rv, cap);
  else gmres_refine<float, DR>(op, pr, b, x, prm, out, st, bnorm, launches, rv, cap);
  out.launches = launches;
  if (cap > 0 && prm.resvec_host && out.n_resvec > 0)
    VS_CUDA(cudaMemcpyAsync(prm.resvec_host, rv, out.n_resvec * sizeof(double), cudaMemcpyDeviceToHost, st));
  VS_CUDA(cudaStreamSynchronize(st));
}

void solve_gmres(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                 cudaStream_t st) {
  solve_gmres_impl<false>(op, pr, b, x, prm, out, st);
}

void solve_gmres_dr(vs_op& op, vs_prec* pr, const double2* b, double2* x, const SolveParams& prm, SolveResult& out,
                    cudaStream_t st) {
  solve_gmres_impl<true>(op, pr, b, x, prm, out, st);
}

}  // namespace vs
