// Small dense complex linear algebra on the host for the GCRO-DR cycle
// (pgmresDR.m:190-258, getHarmVecs1.m, getHarmVecs2.m): the reference calls
// MATLAB's backslash, qr(.,0) and eig on matrices of the cycle's size; these
// are the same operations written out (Householder QR, Gaussian elimination
// with partial pivoting, Hessenberg reduction + shifted QR to the Schur form,
// Golub & Van Loan, "Matrix Computations", 4th ed., 5.1-5.2, 7.4-7.5).
#include "vs_dense.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

namespace vs {
namespace dense {

namespace {

inline cd phase(cd z) {
  const double a = std::abs(z);
  return a > 0 ? z / a : cd(1, 0);
}

// x^H y over n entries
inline cd dotc(const cd* x, const cd* y, int n) {
  cd s = 0;
  for (int i = 0; i < n; ++i) s += std::conj(x[i]) * y[i];
  return s;
}

// Solve A x = b (n x n, general) by Gaussian elimination with partial pivoting.
std::vector<cd> lu_solve(Mat A, int n, std::vector<cd> b) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::abs(A[k + (size_t)k * n]);
    for (int i = k + 1; i < n; ++i)
      if (std::abs(A[i + (size_t)k * n]) > best) {
        best = std::abs(A[i + (size_t)k * n]);
        p = i;
      }
    if (!(best > 0)) throw Failure("singular matrix in a GCRO-DR least-squares step");
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k + (size_t)j * n], A[p + (size_t)j * n]);
      std::swap(b[k], b[p]);
    }
    const cd piv = A[k + (size_t)k * n];
    for (int i = k + 1; i < n; ++i) {
      const cd f = A[i + (size_t)k * n] / piv;
      if (f == cd(0)) continue;
      for (int j = k + 1; j < n; ++j) A[i + (size_t)j * n] -= f * A[k + (size_t)j * n];
      b[i] -= f * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    cd s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[i + (size_t)j * n] * b[j];
    b[i] = s / A[i + (size_t)i * n];
  }
  return b;
}

// R^-1 B for R (c x c) upper triangular, B (c x nc)
Mat left_div_upper(const Mat& R, int c, const Mat& B, int nc) {
  Mat X = B;
  for (int col = 0; col < nc; ++col) {
    cd* x = X.data() + (size_t)col * c;
    for (int i = c - 1; i >= 0; --i) {
      cd s = x[i];
      for (int j = i + 1; j < c; ++j) s -= R[i + (size_t)j * c] * x[j];
      x[i] = s / R[i + (size_t)i * c];
    }
  }
  return X;
}

// eigen-pairs ordered by ascending |lambda| (stable for ties), as MATLAB's
// sortrows on [abs(lambda) vecs'] orders them
void sorted_eig(const Mat& A, int n, std::vector<cd>& lam, Mat& X) {
  std::vector<cd> l0;
  Mat X0;
  eig(A, n, l0, X0);
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return std::abs(l0[a]) < std::abs(l0[b]); });
  lam.resize(n);
  X.assign((size_t)n * n, 0);
  for (int j = 0; j < n; ++j) {
    lam[j] = l0[ord[j]];
    std::copy(X0.begin() + (size_t)ord[j] * n, X0.begin() + (size_t)(ord[j] + 1) * n, X.begin() + (size_t)j * n);
  }
}

}  // namespace

void qr_econ(const Mat& A, int r, int c, Mat& Q, Mat& R) {
  if (r < c) throw Failure("qr_econ needs rows >= columns");
  Mat W = A;
  std::vector<std::vector<cd>> refl(c);
  for (int j = 0; j < c; ++j) {
    const int len = r - j;
    cd* x = W.data() + j + (size_t)j * r;
    double nx = 0;
    for (int i = 0; i < len; ++i) nx += std::norm(x[i]);
    nx = std::sqrt(nx);
    std::vector<cd> v(x, x + len);
    const cd alpha = -phase(x[0]) * nx;
    v[0] -= alpha;
    double vn = 0;
    for (int i = 0; i < len; ++i) vn += std::norm(v[i]);
    if (vn > 0) {
      vn = std::sqrt(vn);
      for (auto& e : v) e /= vn;
      for (int l = j; l < c; ++l) {
        cd* col = W.data() + j + (size_t)l * r;
        const cd s = dotc(v.data(), col, len);
        for (int i = 0; i < len; ++i) col[i] -= 2.0 * s * v[i];
      }
    } else {
      std::fill(v.begin(), v.end(), cd(0));
    }
    refl[j] = std::move(v);
  }
  R.assign((size_t)c * c, 0);
  for (int l = 0; l < c; ++l)
    for (int i = 0; i <= l; ++i) R[i + (size_t)l * c] = W[i + (size_t)l * r];
  Q.assign((size_t)r * c, 0);
  for (int l = 0; l < c; ++l) Q[l + (size_t)l * r] = 1;
  for (int j = c - 1; j >= 0; --j) {
    const auto& v = refl[j];
    const int len = r - j;
    for (int l = 0; l < c; ++l) {
      cd* col = Q.data() + j + (size_t)l * r;
      const cd s = dotc(v.data(), col, len);
      if (s == cd(0)) continue;
      for (int i = 0; i < len; ++i) col[i] -= 2.0 * s * v[i];
    }
  }
}

std::vector<cd> lstsq(const Mat& A, int r, int c, const std::vector<cd>& rhs) {
  Mat Q, R;
  qr_econ(A, r, c, Q, R);
  std::vector<cd> y(c);
  for (int j = 0; j < c; ++j) y[j] = dotc(Q.data() + (size_t)j * r, rhs.data(), r);
  for (int i = 0; i < c; ++i)
    if (!(std::abs(R[i + (size_t)i * c]) > 0)) throw Failure("rank-deficient GCRO-DR least-squares matrix");
  Mat Y(y.begin(), y.end());
  Y = left_div_upper(R, c, Y, 1);
  return std::vector<cd>(Y.begin(), Y.end());
}

Mat right_div_upper(const Mat& B, int r, int c, const Mat& R) {
  for (int j = 0; j < c; ++j)
    if (!(std::abs(R[j + (size_t)j * c]) > 0)) throw Failure("singular triangle in a GCRO-DR basis update");
  Mat X((size_t)r * c, 0);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) {
      cd s = B[i + (size_t)j * r];
      for (int l = 0; l < j; ++l) s -= X[i + (size_t)l * r] * R[l + (size_t)j * c];
      X[i + (size_t)j * r] = s / R[j + (size_t)j * c];
    }
  return X;
}

void eig(const Mat& A, int n, std::vector<cd>& lam, Mat& X) {
  Mat H = A, Z((size_t)n * n, 0);
  auto h = [&](int i, int j) -> cd& { return H[i + (size_t)j * n]; };
  auto z = [&](int i, int j) -> cd& { return Z[i + (size_t)j * n]; };
  for (int i = 0; i < n; ++i) z(i, i) = 1;
  double hnorm = 0;
  for (const auto& e : H) hnorm = std::max(hnorm, std::abs(e));
  if (!std::isfinite(hnorm)) throw Failure("non-finite matrix in a harmonic Ritz eigenproblem");
  // Householder reduction to upper Hessenberg form, H = Z^H A Z
  for (int k = 0; k + 2 < n; ++k) {
    const int len = n - k - 1;
    std::vector<cd> v(len);
    double nx = 0;
    for (int i = 0; i < len; ++i) {
      v[i] = h(k + 1 + i, k);
      nx += std::norm(v[i]);
    }
    nx = std::sqrt(nx);
    if (nx == 0) continue;
    v[0] -= -phase(v[0]) * nx;
    double vn = 0;
    for (const auto& e : v) vn += std::norm(e);
    if (!(vn > 0)) continue;
    vn = std::sqrt(vn);
    for (auto& e : v) e /= vn;
    for (int j = k; j < n; ++j) {
      cd s = 0;
      for (int i = 0; i < len; ++i) s += std::conj(v[i]) * h(k + 1 + i, j);
      for (int i = 0; i < len; ++i) h(k + 1 + i, j) -= 2.0 * s * v[i];
    }
    for (int i = 0; i < n; ++i) {
      cd s = 0, t = 0;
      for (int l = 0; l < len; ++l) {
        s += h(i, k + 1 + l) * v[l];
        t += z(i, k + 1 + l) * v[l];
      }
      for (int l = 0; l < len; ++l) {
        h(i, k + 1 + l) -= 2.0 * s * std::conj(v[l]);
        z(i, k + 1 + l) -= 2.0 * t * std::conj(v[l]);
      }
    }
    for (int i = k + 2; i < n; ++i) h(i, k) = 0;
  }
  // shifted QR iteration to the complex Schur form H = Z^H A Z (upper triangular)
  const double eps = 2.220446049250313e-16;
  std::vector<double> cs(n);
  std::vector<cd> sn(n);
  int hi = n - 1, iter = 0, total = 0;
  while (hi > 0) {
    int l = hi;
    for (; l > 0; --l) {
      double s = std::abs(h(l - 1, l - 1)) + std::abs(h(l, l));
      if (s == 0) s = hnorm;
      if (std::abs(h(l, l - 1)) <= eps * s) break;
    }
    if (l > 0) h(l, l - 1) = 0;
    if (l == hi) {
      --hi;
      iter = 0;
      continue;
    }
    if (++total > 60 * n) throw Failure("harmonic Ritz eigenproblem: QR iteration did not converge");
    ++iter;
    cd mu;
    const cd a = h(hi - 1, hi - 1), b = h(hi - 1, hi), c = h(hi, hi - 1), d = h(hi, hi);
    if (iter % 11 == 0) {
      mu = d + std::abs(c) * 0.75;  // exceptional shift
    } else {
      const cd tr2 = 0.5 * (a + d), disc = std::sqrt(0.25 * (a - d) * (a - d) + b * c);
      const cd m1 = tr2 + disc, m2 = tr2 - disc;
      mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
    }
    for (int i = l; i <= hi; ++i) h(i, i) -= mu;
    for (int k = l; k < hi; ++k) {
      const cd x = h(k, k), y = h(k + 1, k);
      const double ax = std::abs(x), r = std::hypot(ax, std::abs(y));
      double c0;
      cd s0;
      if (r == 0) {
        c0 = 1;
        s0 = 0;
      } else if (ax == 0) {
        c0 = 0;
        s0 = 1;
      } else {
        c0 = ax / r;
        s0 = (x / ax) * std::conj(y) / r;
      }
      cs[k] = c0;
      sn[k] = s0;
      for (int j = k; j < n; ++j) {
        const cd u = h(k, j), v = h(k + 1, j);
        h(k, j) = c0 * u + s0 * v;
        h(k + 1, j) = -std::conj(s0) * u + c0 * v;
      }
    }
    for (int k = l; k < hi; ++k) {
      const double c0 = cs[k];
      const cd s0 = sn[k];
      for (int i = 0; i <= k + 1; ++i) {
        const cd u = h(i, k), v = h(i, k + 1);
        h(i, k) = c0 * u + std::conj(s0) * v;
        h(i, k + 1) = -s0 * u + c0 * v;
      }
      for (int i = 0; i < n; ++i) {
        const cd u = z(i, k), v = z(i, k + 1);
        z(i, k) = c0 * u + std::conj(s0) * v;
        z(i, k + 1) = -s0 * u + c0 * v;
      }
    }
    for (int i = l; i <= hi; ++i) h(i, i) += mu;
  }
  // eigenvectors of the triangle by back substitution, mapped back through Z
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = h(i, i);
  X.assign((size_t)n * n, 0);
  const double small = std::max(hnorm, 1e-300) * eps;
  std::vector<cd> y(n);
  for (int i = 0; i < n; ++i) {
    std::fill(y.begin(), y.end(), cd(0));
    y[i] = 1;
    for (int j = i - 1; j >= 0; --j) {
      cd s = 0;
      for (int l = j + 1; l <= i; ++l) s += h(j, l) * y[l];
      cd den = h(j, j) - lam[i];
      if (std::abs(den) < small) den = small;
      y[j] = -s / den;
    }
    double nrm = 0;
    cd* x = X.data() + (size_t)i * n;
    for (int r = 0; r < n; ++r) {
      cd s = 0;
      for (int l = 0; l <= i; ++l) s += z(r, l) * y[l];
      x[r] = s;
      nrm += std::norm(s);
    }
    nrm = std::sqrt(nrm);
    for (int r = 0; r < n; ++r) x[r] /= nrm;
  }
}

Mat harm_vecs1(int m, int k, const Mat& H) {
  const int ld = m + 1;
  Mat Hm((size_t)m * m), HmH((size_t)m * m);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) {
      Hm[i + (size_t)j * m] = H[i + (size_t)j * ld];
      HmH[j + (size_t)i * m] = std::conj(H[i + (size_t)j * ld]);
    }
  std::vector<cd> em(m, 0);
  em[m - 1] = 1;
  const std::vector<cd> f = lu_solve(HmH, m, em);
  const cd h = H[m + (size_t)(m - 1) * ld];
  for (int i = 0; i < m; ++i) Hm[i + (size_t)(m - 1) * m] += h * h * f[i];
  std::vector<cd> lam;
  Mat X;
  sorted_eig(Hm, m, lam, X);
  return Mat(X.begin(), X.begin() + (size_t)k * m);
}

Mat harm_vecs2(int m, int k, const Mat& H2, const Mat& W) {
  Mat Q, R;
  qr_econ(H2, m + 1, m, Q, R);
  Mat Y((size_t)m * m);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) Y[i + (size_t)j * m] = dotc(Q.data() + (size_t)i * (m + 1), W.data() + (size_t)j * (m + 1), m + 1);
  const Mat Mx = left_div_upper(R, m, Y, m);
  std::vector<cd> lam;
  Mat X;
  sorted_eig(Mx, m, lam, X);
  return Mat(X.begin() + (size_t)(m - k) * m, X.end());
}

}  // namespace dense
}  // namespace vs

// Test hooks (not part of the public interface): the host routines above on
// interleaved complex column-major arrays, so the CPU tests can compare them
// with LAPACK through NumPy without a GPU.  Return 0, or -1 on failure.
namespace {
vs::dense::Mat to_mat(const double* a, size_t count) {
  vs::dense::Mat m(count);
  for (size_t i = 0; i < count; ++i) m[i] = vs::dense::cd(a[2 * i], a[2 * i + 1]);
  return m;
}
void from_mat(const vs::dense::Mat& m, double* out) {
  for (size_t i = 0; i < m.size(); ++i) {
    out[2 * i] = m[i].real();
    out[2 * i + 1] = m[i].imag();
  }
}
}  // namespace

extern "C" int vsx_dense_eig(int n, const double* A, double* lam, double* X) {
  try {
    std::vector<vs::dense::cd> l;
    vs::dense::Mat x;
    vs::dense::eig(to_mat(A, (size_t)n * n), n, l, x);
    from_mat(vs::dense::Mat(l.begin(), l.end()), lam);
    from_mat(x, X);
    return 0;
  } catch (...) {
    return -1;
  }
}

extern "C" int vsx_dense_harm_vecs1(int m, int k, const double* H, double* P) {
  try {
    from_mat(vs::dense::harm_vecs1(m, k, to_mat(H, (size_t)(m + 1) * m)), P);
    return 0;
  } catch (...) {
    return -1;
  }
}

extern "C" int vsx_dense_harm_vecs2(int m, int k, const double* H2, const double* W, double* P) {
  try {
    from_mat(vs::dense::harm_vecs2(m, k, to_mat(H2, (size_t)(m + 1) * m), to_mat(W, (size_t)(m + 1) * m)), P);
    return 0;
  } catch (...) {
    return -1;
  }
}

extern "C" int vsx_dense_lstsq(int r, int c, const double* A, const double* rhs, double* y) {
  try {
    const auto v = vs::dense::lstsq(to_mat(A, (size_t)r * c), r, c, to_mat(rhs, (size_t)r));
    from_mat(vs::dense::Mat(v.begin(), v.end()), y);
    return 0;
  } catch (...) {
    return -1;
  }
}
