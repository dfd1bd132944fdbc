// Two-level x passes: gather + zero-pad + FFT along x (XF), and IFFT along x
// + crop + diagonal term + scatter (XI), for lines of length P = R1 * R2
// (R1 <= 16, R2 <= 32, R1 near sqrt(P)).  Same arithmetic as k_xf /
// k_xi in vs_matvec.cu (which handle the lengths not instantiated here).
//
// A CTA owns NL = 256 / R2 lines (line = (j, k, comp), x contiguous):
//   XF A : item (n1, line): x points n1 + R1*n2 (< L) gathered through map3
//          (with the mode's conjugation / diagonal) into registers, R2-point
//          DFT, twiddle, one shared store;
//      B : item (k2, line): R1-point DFT, outputs k2 + R2*k1 stored to T1;
//   XI B': item (k2, line): T1 entries k2 + R2*k1, inverse R1-point DFT,
//          conjugate twiddle, one shared store;
//      A': item (n1, line): inverse R2-point DFT, entries n1 + R1*n2 (< L)
//          combined with the diagonal term and scattered through map3.
// Shared layout [line][n1][k2] with an odd row stride R2 | 1, so consecutive
// n1 (stage A, A') and consecutive k2 (stage B, B') are both conflict-free
// while the global accesses of every stage run along x.  The inter-stage
// twiddles w^(n1*k2) come from a second table laid out along the index the
// threads vary (conflict-free, unlike the strided 1-D table), and the first
// stage issues its global loads before the tables are filled, so the fill
// and the barrier overlap their latency.  Every thread holds at most one item
// of a stage (R1 <= R2).  K is the arithmetic type: the storage type, or
// double-float (dfc) on FP64 data, whose DFTs then run on the FP32 pipes and
// whose results are rounded back to FP64 at the global stores.
// Instantiated per precision in vs_xpass_c64.cu and vs_xpass_c128.cu, in
// double-float in vs_df_xpass_a.cu / vs_df_xpass_b.cu (vs_df_passes.cuh).
#pragma once
#include "vs_spass.cuh"
#include "vs_reduce.cuh"

namespace vs {

constexpr int kX2Threads = 256;
constexpr int X2C = 4;  // elements per chunk of the cooperative gather and scatter

template <typename T>
__device__ __forceinline__ cplx_t<T> x2_gather(const PipeArgs<T>& a, const cplx_t<T>* x, int pos, int mode) {
  using C = cplx_t<T>;
  if (pos < 0) return czero<C>();
  C v = x[pos];
  if (mode == VS_TRANSP) v = cmul(a.d2.at(pos), v);
  else if (mode == VS_CONJTRANSP) v = cmul(a.d2.at(pos), cconj(v));
  return v;
}

// The folded gather's alpha step (XFuse::apart): every CTA adds the
// matvec's partial sums of rt^H v in the same order and its thread 0 forms
// alpha = rho / (rt^H v) and the breakdown test; false (every thread) on a
// breakdown, after the last CTA to count in has written the flags.
template <typename T>
__device__ __noinline__ bool x2_alpha_step(const XFuse<T>& f, int rhs, cplx_t<T>& sa) {
  using C = cplx_t<T>;
  __shared__ double tot[2];
  __shared__ C s_al;
  __shared__ int s_flag;
  SlotV<T> x[2];
  slot_sums<2, 4, false>(f.apart + rhs * f.pstride, f.anb, (int)threadIdx.x, (int)blockDim.x, x);
  cta_partials<2>(x, tot);  // thread 0 writes the CTA's sums in slot form
  char* st = const_cast<char*>(f.sbase) + rhs * f.sstride;
  if (threadIdx.x == 0) {
    double t[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      SlotV<T> y;
      get_slot<false>(tot + k, y);
      t[k] = widen(y);
    }
    double2 al = make_double2(0.0, 0.0);
    s_flag = alpha_step(*reinterpret_cast<const double2*>(st + f.off_rho), t, al);
    C c;
    c.x = (decltype(c.x))al.x;
    c.y = (decltype(c.y))al.y;
    s_al = c;
    if (s_flag < 0 && blockIdx.x == 0) {
      *reinterpret_cast<double2*>(st + f.off_alpha) = al;
      *reinterpret_cast<C*>(st + f.off_a) = c;
    }
  }
  __syncthreads();
  if (s_flag >= 0) {
    if (threadIdx.x == 0) {
      __threadfence();
      unsigned* counter = reinterpret_cast<unsigned*>(st + f.off_counter);
      if (atomicAdd(counter, 1u) == gridDim.x - 1) {
        *reinterpret_cast<int*>(st + f.off_flag) = s_flag;
        *reinterpret_cast<int*>(st + f.off_skip) = 1;
        *counter = 0;
      }
    }
    return false;
  }
  sa = s_al;
  return true;
}

// Component of x line `line` (< 3 MN) by two compares: a division by the
// runtime MN goes through integer <-> float conversions, which GB300 runs on
// its narrow FP64 pipe.
__device__ __forceinline__ int comp_of(int line, int MN) { return (line >= MN) + (line >= 2 * MN); }

// HO (inverse only): L <= (R1 R2 + 1) / 2, so the outputs n2 >=
// lower_half_n2 are never scattered and never formed.
template <typename T, int R1, int R2, bool INV, typename K = cplx_t<T>, bool HO = false>
__global__ void __launch_bounds__(kX2Threads, (std::is_same<T, float>::value && R2 <= 18) ? 4 : 1) k_x2(PipeArgs<T> a, int mode) {
  using C = cplx_t<T>;  // storage
  static_assert(sizeof(K) == sizeof(C), "compute and storage elements share the shared-memory layout");
  constexpr int P = R1 * R2, NL = kX2Threads / R2, RS = R2 | 1;
  static_assert(R1 <= R2, "one stage item per thread");
  if (a.skip && a.skip[blockIdx.y * a.skip_stride]) return;
  K* S = shmem<K>();  // [NL][R1][RS]
  K* tw = S + NL * R1 * RS;
  // w^(n1*k2) laid out with the index the threads of a stage vary fastest:
  // [k2][n1] for XF stage A, [n1][k2] for XI stage B'
  K* tw2 = tw + P;
  const int rhs = blockIdx.y;
  const C* x = a.x + (int64_t)rhs * a.n3;
  const int64_t t1off = (int64_t)rhs * P * a.M * a.N * 3;
  const int nlines = a.M * a.N * 3, MN = a.M * a.N;
  const int line0 = blockIdx.x * NL;
  const int it = threadIdx.x;
  if constexpr (!INV) {
    C* t1 = a.t1 + t1off;
    // stage A loads first: the table fill and the barrier overlap their latency
    const int n1 = it % R1, l = it / R1, line = line0 + l;
    const bool act = it < R1 * NL;
    K v[R2];
    const bool fused = a.fz.kind == XF_GATHER_P || a.fz.kind == XF_GATHER_S;
    Acc<T> acc;
    auto fill_tables = [&] {
      for (int i = it; i < P; i += kX2Threads) {
        tw[i] = to_compute<K>(__ldg(a.twP + i));
        const int k2 = i / R1, m1 = i - k2 * R1;
        tw2[i] = to_compute<K>(__ldg(a.twP + m1 * k2));
      }
    };
    if (fused) {
      // (only the preconditioner's forward pass folds a step, and its gather
      // is plain: no diagonal or conjugation applies to the formed element)
      // Every thread of the CTA forms elements of its NL lines (element e =
      // l P + i, i < L; zeros up to P) into S in stage A's input layout
      // [l][n1][n2] (i = n1 + R1 n2), in chunks of X2C: indices, then the
      // solver's vectors, then the formed elements written back, so a chunk's
      // loads are in flight together.  (Stage A's R1 NL threads alone, R2
      // elements each, waited on twice as many rounds of dependent loads.)
      const int64_t off = (int64_t)rhs * a.n3;
      const bool pk = a.fz.kind == XF_GATHER_P;
      C sa;
      if (!pk && a.fz.apart) {
        if (!x2_alpha_step(a.fz, rhs, sa)) return;  // breakdown: no vector is touched
      } else {
        sa = a.fz.scalar(rhs, a.fz.off_a);
      }
      const C sb = pk ? a.fz.scalar(rhs, a.fz.off_b) : czero<C>();
      const bool first = pk && *reinterpret_cast<const int*>(a.fz.sbase + rhs * a.fz.sstride + a.fz.off_iter) == 0;
      const C* __restrict__ fu = a.fz.u + off;
      const C* __restrict__ fv = a.fz.v + off;
      C* __restrict__ fw = a.fz.w + off;
      constexpr int NE = NL * P, NCH = (NE + kX2Threads - 1) / kX2Threads;
#pragma unroll
      for (int c0 = 0; c0 < NCH; c0 += X2C) {
        int pos[X2C], sidx[X2C];
        C val[X2C];
#pragma unroll
        for (int j = 0; j < X2C; ++j) {
          const int e = it + kX2Threads * (c0 + j);
          const int le = e / P, i = e - le * P, linee = line0 + le;
          sidx[j] = (c0 + j < NCH && e < NE) ? (le * R1 + i % R1) * RS + i / R1 : -1;
          pos[j] = -1;
          if (sidx[j] >= 0 && i < a.L && linee < nlines) {
            const int ce = comp_of(linee, MN), jke = linee - ce * MN;
            pos[j] = __ldg(a.map3 + (int64_t)ce * a.V + (int64_t)jke * a.L + i);
          }
        }
#pragma unroll
        for (int j = 0; j < X2C; ++j) {
          val[j] = czero<C>();
          if (pos[j] >= 0) {
            const C r = fu[pos[j]], vv = fv[pos[j]];
            if (pk) val[j] = first ? r : cfma(sa, csub(fw[pos[j]], cmul(sb, vv)), r);
            else val[j] = csub(r, cmul(sa, vv));
          }
        }
#pragma unroll
        for (int j = 0; j < X2C; ++j) {
          if (sidx[j] >= 0) S[sidx[j]] = to_compute<K>(val[j]);
          if (pos[j] >= 0) {
            fw[pos[j]] = val[j];
            if (!pk) acc.norm2(val[j]);
          }
        }
      }
      fill_tables();
      __syncthreads();
      // each stage-A thread reads its own row, which it alone rewrites below
      if (act) {
        const K* s = S + (l * R1 + n1) * RS;
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) v[n2] = s[n2];
      }
    } else {
      if (act && line < nlines) {
        const int c = comp_of(line, MN), jk = line - c * MN;
        const int* map = a.map3 + (int64_t)c * a.V + (int64_t)jk * a.L;
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
          const int i = n1 + R1 * n2;
          v[n2] = i < a.L ? to_compute<K>(x2_gather(a, x, __ldg(map + i), mode)) : czero<K>();
        }
      } else {
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) v[n2] = czero<K>();
      }
      fill_tables();
      __syncthreads();
    }
    if (act) {
      reg_dft<R2, R2, 1, R1, false, K>(v, tw);
      K* s = S + (l * R1 + n1) * RS;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) s[k2] = (k2 == 0 || n1 == 0) ? v[k2] : cmul(v[k2], tw2[k2 * R1 + n1]);
    }
    __syncthreads();
    {
      const int k2 = it % R2, lb = it / R2, lineb = line0 + lb;
      if (it < R2 * NL && lineb < nlines) {
        K u[R1];
#pragma unroll
        for (int m1 = 0; m1 < R1; ++m1) u[m1] = S[(lb * R1 + m1) * RS + k2];
        reg_dft<R1, R1, 1, R2, false, K>(u, tw);
        C* out = t1 + (int64_t)lineb * P;
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) out[k2 + R2 * k1] = to_storage(u[k1], C{});
      }
    }
    if (a.fz.kind == XF_GATHER_S) {  // the CTA's ||s||^2 (every thread takes part)
      const decltype(acc.vre()) w[1] = {acc.vre()};
      cta_partials<1>(w, a.fz.part + rhs * a.fz.pstride + blockIdx.x);
    }
  } else {
    const C* t1 = a.t1 + t1off;
    C* y = a.y + (int64_t)rhs * a.n3;
    // stage B' loads first
    const int k2 = it % R2, l = it / R2, line = line0 + l;
    const bool act = it < R2 * NL;
    K u[R1];
    {
      const C* in = t1 + (int64_t)line * P;
      const bool ld = act && line < nlines;
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) u[k1] = ld ? to_compute<K>(in[k2 + R2 * k1]) : czero<K>();
    }
    // With a folded inner product, the solver vector read at the scatter (rt
    // or s) was last touched an iteration or a preconditioner apply ago and is
    // mostly out of L2: the stage-A' threads prefetch it (and the input) into
    // L2 at the unknowns of the CTA's lines, so the latency overlaps the
    // first DFT stage instead of the scatter.
    if (a.fz.kind == XF_SCATTER_DOT || a.fz.kind == XF_SCATTER_OMEGA) {
      const int pn1 = it % R1, pla = it / R1, pline = line0 + pla;
      if (it < R1 * NL && pline < nlines && pn1 < a.L) {
        const int c = comp_of(pline, MN), jk = pline - c * MN;
        const int* map = a.map3 + (int64_t)c * a.V + (int64_t)jk * a.L;
        const C* fu = a.fz.u + (int64_t)rhs * a.n3;
        const C* xin = a.x + (int64_t)rhs * a.n3;
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
          const int i = pn1 + R1 * n2;
          if (i >= a.L) continue;
          const int p = __ldg(map + i);
          if (p < 0) continue;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(fu + p));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(xin + p));
        }
      }
    }
    for (int i = it; i < P; i += kX2Threads) {
      tw[i] = to_compute<K>(__ldg(a.twP + i));
      const int m1 = i / R2, j2 = i - m1 * R2;
      tw2[i] = to_compute<K>(__ldg(a.twP + m1 * j2));
    }
    __syncthreads();
    if (act) {
      reg_dft<R1, R1, 1, R2, true, K>(u, tw);
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1)
        S[(l * R1 + n1) * RS + k2] = (n1 == 0 || k2 == 0) ? u[n1] : cmul(u[n1], cconj(tw2[n1 * R2 + k2]));
    }
    __syncthreads();
    const int n1 = it % R1, la = it / R1, linea = line0 + la;
    constexpr int NO = HO ? lower_half_n2(R1, R2) : R2;  // outputs formed per row
    // stage A' by R1 NL threads: the row's outputs i = n1 + R1 n2 back into
    // its own row of S
    if (it < R1 * NL && linea < nlines && n1 < a.L) {
      K v[R2];
      K* s = S + (la * R1 + n1) * RS;
#pragma unroll
      for (int j2 = 0; j2 < R2; ++j2) v[j2] = s[j2];
      reg_dft<R2, R2, 1, R1, true, K>(v, tw);
#pragma unroll
      for (int n2 = 0; n2 < NO; ++n2) s[n2] = v[n2];
    }
    __syncthreads();
    // The scatter, by every thread of the CTA: element e = l IH + i of its NL
    // lines (outputs i < L; IH bounds the formed outputs), in chunks of X2C
    // (indices, then the inputs, then the outputs).  (Stage A''s R1 NL
    // threads alone, R2 outputs each, waited on more rounds of dependent
    // loads.)
    constexpr int IH = (R1 * NO < P) ? R1 * NO : P;
    constexpr int NE = NL * IH, NCH = (NE + kX2Threads - 1) / kX2Threads;
    Acc<T> acc, acc2;
    const int fk = a.fz.kind;
    // the output never aliases the input or the solver's vectors: with the
    // pointers restrict-qualified a chunk's loads need not wait for the
    // previous chunk's stores
    const C* __restrict__ xr = x;
    C* __restrict__ yr = y;
    const C* __restrict__ fu = fk != XF_NONE ? a.fz.u + (int64_t)rhs * a.n3 : nullptr;
#pragma unroll
    for (int c0 = 0; c0 < NCH; c0 += X2C) {
      int pos[X2C], sidx[X2C];
#pragma unroll
      for (int j = 0; j < X2C; ++j) {
        const int e = it + kX2Threads * (c0 + j);
        const int le = e / IH, i = e - le * IH, linee = line0 + le;
        pos[j] = -1;
        sidx[j] = (le * R1 + i % R1) * RS + i / R1;
        if (c0 + j < NCH && e < NE && i < a.L && linee < nlines) {
          const int ce = comp_of(linee, MN), jke = linee - ce * MN;
          pos[j] = __ldg(a.map3 + (int64_t)ce * a.V + (int64_t)jke * a.L + i);
        }
      }
      C xv[X2C], fv[X2C];
#pragma unroll
      for (int j = 0; j < X2C; ++j) {
        if (pos[j] >= 0) {
          if (mode != MODE_PLAIN) xv[j] = xr[pos[j]];
          if (fk != XF_NONE) fv[j] = fu[pos[j]];
        }
      }
#pragma unroll
      for (int j = 0; j < X2C; ++j) {
        const int p = pos[j];
        if (p < 0) continue;
        const C conv = to_storage(S[sidx[j]], C{});
        C out;
        if (mode == MODE_PLAIN) {
          out = conv;
        } else {
          if (mode == VS_NOTRANSP) out = csub(cmul(diag_term(a, p, rhs, false), xv[j]), cmul(a.d2.at(p), conv));
          else if (mode == VS_TRANSP) out = csub(cmul(diag_term(a, p, rhs, false), xv[j]), conv);
          else out = csub(cmul(diag_term(a, p, rhs, true), xv[j]), cconj(conv));
        }
        yr[p] = out;
        if (fk == XF_SCATTER_DOT) {
          acc.dot(fv[j], out);  // rt^H v
        } else if (fk == XF_SCATTER_OMEGA) {
          acc.dot(out, fv[j]);  // t^H s
          acc2.norm2(out);      // t^H t
        }
      }
    }
    // the CTA's inner products (every thread takes part)
    using V = decltype(acc.vre());
    if (fk == XF_SCATTER_DOT) {
      const V w[2] = {acc.vre(), acc.vim()};
      cta_partials<2>(w, a.fz.part + rhs * a.fz.pstride + (int64_t)blockIdx.x * 2);
    } else if (fk == XF_SCATTER_OMEGA) {
      const V w[3] = {acc.vre(), acc.vim(), acc2.vre()};
      cta_partials<3>(w, a.fz.part + rhs * a.fz.pstride + (int64_t)blockIdx.x * 3);
    }
  }
}

template <typename T, int R1, int R2, bool INV, typename K = cplx_t<T>>
static void launch_x2(const PipeArgs<T>& a, int mode, int nrhs, cudaStream_t st) {
  constexpr int NL = kX2Threads / R2, RS = R2 | 1;
  const size_t smem = (size_t)(NL * R1 * RS + 2 * R1 * R2) * sizeof(cplx_t<T>);
  // the matvec's inverse x pass keeps at most half the line (P >= 2L - 1)
  auto k = k_x2<T, R1, R2, INV, K>;
  if constexpr (INV) {
    if (2 * a.L - 1 <= R1 * R2) k = k_x2<T, R1, R2, INV, K, true>;
  }
  set_kernel_smem((const void*)k, smem);
  const int nlines = a.M * a.N * 3;
  k<<<dim3(ceil_div(nlines, NL), nrhs), kX2Threads, smem, st>>>(a, mode);
  VS_LAUNCH_CHECK();
}

template <typename T, bool INV>
bool x_two_level(const PipeArgs<T>& a, int mode, int nrhs, cudaStream_t st) {
  switch (a.P) {
#define VS_X2_CASE(R1, R2)                      \
  case R1 * R2:                                 \
    launch_x2<T, R1, R2, INV>(a, mode, nrhs, st); \
    return true;
    VS_S2_LIST(VS_X2_CASE)
#undef VS_X2_CASE
    default: return false;
  }
}

}  // namespace vs
