// C entry point over the reference's face-pair cubature
// (src/src_vie/src_operators/mexcubatures/cubature_nop_const.cpp:8), for the
// oracle tests only: the same argument conversion its MEX gateway performs
// (cubature_nop_const_mex.cpp:40-75) -- MATLAB's column-major R_faces(3,4,6)
// into the C array [3][4][6], and I_mn back as a column-major 6x6 complex
// matrix (interleaved re/im here).  Compiled together with the reference
// source by oracle/build_ref.py into oracle/_ref/libref_nop.so.
#include <complex>

void cubature_nop(const int Np, const double w[], const double u[], const double v[], const double r_m[3],
                  const double r_n[3], const double R_faces[3][4][6], const double ko, const double dx,
                  std::complex<double> I_mn[6][6]);

extern "C" void ref_cubature_nop(int np, const double* w, const double* u, const double* v, const double* r_m,
                                 const double* r_n, const double* faces_colmajor, double ko, double dx,
                                 double* out) {
  double faces[3][4][6];
  for (int f = 0; f < 6; ++f)
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 3; ++i) faces[i][j][f] = faces_colmajor[i + 3 * j + 12 * f];
  std::complex<double> I[6][6];
  cubature_nop(np, w, u, v, r_m, r_n, faces, ko, dx, I);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      out[2 * (i + 6 * j)] = I[i][j].real();
      out[2 * (i + 6 * j) + 1] = I[i][j].imag();
    }
}
