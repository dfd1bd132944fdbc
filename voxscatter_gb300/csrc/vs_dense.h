// Small dense complex linear algebra on the host (vs_dense.cu): the
// least-squares solves, economy QR and harmonic Ritz eigenproblems of the
// GCRO-DR cycle.  Matrices are column-major std::vector<cd> with the row
// count as leading dimension; sizes are those of one Krylov cycle (<= a few
// hundred), so plain O(n^3) loops are used.
#pragma once
#include <complex>
#include <stdexcept>
#include <vector>

namespace vs {
namespace dense {

using cd = std::complex<double>;
using Mat = std::vector<cd>;

// A numerical failure of one of these routines (singular or rank-deficient
// matrix, QR iteration without convergence, non-finite input).
struct Failure : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Economy QR of A (r x c, r >= c) by Householder reflections: Q (r x c) with
// orthonormal columns, R (c x c) upper triangular, A = Q R.
void qr_econ(const Mat& A, int r, int c, Mat& Q, Mat& R);

// Least-squares solution of min ||A y - rhs|| for A (r x c) of full column rank.
std::vector<cd> lstsq(const Mat& A, int r, int c, const std::vector<cd>& rhs);

// X = B R^-1 for B (r x c) and R (c x c) upper triangular (MATLAB's B / R).
Mat right_div_upper(const Mat& B, int r, int c, const Mat& R);

// Eigenvalues lam and eigenvectors X (columns of unit 2-norm) of a general
// complex n x n matrix: Householder Hessenberg reduction, shifted QR to the
// complex Schur form (Wilkinson shifts), back-substitution on the triangle.
// Throws if the QR iteration does not converge.
void eig(const Mat& A, int n, std::vector<cd>& lam, Mat& X);

// getHarmVecs1.m: the k harmonic Ritz vectors of smallest |theta| of the
// (m+1) x m Arnoldi Hessenberg H, eig(H_m + h_{m+1,m}^2 H_m^-H e_m e_m^T).
// Returns P (m x k).
Mat harm_vecs1(int m, int k, const Mat& H);

// getHarmVecs2.m: eig(H2^H W, H2^H H2) for H2, W ((m+1) x m), solved as the
// standard problem R^-1 Q^H W with H2 = Q R; the k eigenvectors of largest
// |lambda|.  Returns P (m x k).
Mat harm_vecs2(int m, int k, const Mat& H2, const Mat& W);

}  // namespace dense
}  // namespace vs
