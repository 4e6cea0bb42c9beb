// Stand-in for the sphericart::SphericalHarmonics<T> API that libsymmetrix calls
// (libsymmetrix/source/mace.cpp:118-148, spherical_harmonic.cpp:45-101).  The real
// library is lab-cosmo/sphericart, an un-vendored git submodule
// (libsymmetrix/external/sphericart, version not pinned in the reference tree).
//
// Test infrastructure only.  Restated from the published definition of the
// orthonormal real spherical harmonics of the unit vector u = x/|x| (no
// Condon-Shortley phase: Y_1,-1 ~ y, Y_1,0 ~ z, Y_1,1 ~ x), which is also the
// convention of libsymmetrix/source/spherical_harmonic.cpp:38-43.  Gradients are
// with respect to the raw Cartesian input x.  Layouts follow the reference call
// sites: sph[n][lm], dsph[n][3][lm] with lm = l*(l+1)+m.
//
// Each Y_lm is written as P_lm(x)/|x|^l with P_lm a homogeneous polynomial, so
// dY_lm/dx = grad P_lm(u)/|x| - l Y_lm u/|x|.  l_max <= 3.
#pragma once

#include <cmath>
#include <stdexcept>
#include <vector>

namespace sphericart {

template <typename T>
class SphericalHarmonics {
 public:
  explicit SphericalHarmonics(size_t l_max) : l_max_(static_cast<int>(l_max)) {
    if (l_max_ > 3) throw std::invalid_argument("sphericart stand-in supports l_max <= 3");
  }

  void compute(const std::vector<T>& xyz, std::vector<T>& sph) {
    const size_t n = xyz.size() / 3, nlm = (l_max_ + 1) * (l_max_ + 1);
    if (sph.size() < n * nlm) sph.resize(n * nlm);
    T Y[16], G[3][16];
    for (size_t i = 0; i < n; ++i) {
      eval(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], Y, G, false);
      for (size_t lm = 0; lm < nlm; ++lm) sph[i * nlm + lm] = Y[lm];
    }
  }

  void compute_with_gradients(const std::vector<T>& xyz, std::vector<T>& sph, std::vector<T>& dsph) {
    const size_t n = xyz.size() / 3, nlm = (l_max_ + 1) * (l_max_ + 1);
    if (sph.size() < n * nlm) sph.resize(n * nlm);
    if (dsph.size() < 3 * n * nlm) dsph.resize(3 * n * nlm);
    T Y[16], G[3][16];
    for (size_t i = 0; i < n; ++i) {
      eval(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], Y, G, true);
      for (size_t lm = 0; lm < nlm; ++lm) {
        sph[i * nlm + lm] = Y[lm];
        for (int a = 0; a < 3; ++a) dsph[(3 * i + a) * nlm + lm] = G[a][lm];
      }
    }
  }

 private:
  int l_max_;

  void eval(T x, T y, T z, T* Y, T (*G)[16], bool grad) const {
    const T pi = T(3.14159265358979323846);
    const T r = std::sqrt(x * x + y * y + z * z);
    const T X = x / r, Yy = y / r, Z = z / r;
    // P[lm] and dP/d(X,Y,Z)[lm] of the homogeneous polynomials at the unit vector
    T P[16], dP[3][16];
    const T c0 = T(0.5) / std::sqrt(pi);
    const T c1 = std::sqrt(T(3) / (T(4) * pi));
    const T c2a = T(0.5) * std::sqrt(T(15) / pi), c2b = T(0.25) * std::sqrt(T(5) / pi),
            c2c = T(0.25) * std::sqrt(T(15) / pi);
    const T c3a = T(0.25) * std::sqrt(T(35) / (T(2) * pi)), c3b = T(0.5) * std::sqrt(T(105) / pi),
            c3c = T(0.25) * std::sqrt(T(21) / (T(2) * pi)), c3d = T(0.25) * std::sqrt(T(7) / pi),
            c3e = T(0.25) * std::sqrt(T(105) / pi);
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 16; ++k) dP[a][k] = 0;
    const T XX = X * X, YY = Yy * Yy, ZZ = Z * Z, RR = XX + YY + ZZ;
    P[0] = c0;
    P[1] = c1 * Yy; dP[1][1] = c1;
    P[2] = c1 * Z;  dP[2][2] = c1;
    P[3] = c1 * X;  dP[0][3] = c1;
    // l = 2 : xy, yz, 3z^2 - r^2, xz, x^2 - y^2
    P[4] = c2a * X * Yy; dP[0][4] = c2a * Yy; dP[1][4] = c2a * X;
    P[5] = c2a * Yy * Z; dP[1][5] = c2a * Z;  dP[2][5] = c2a * Yy;
    P[6] = c2b * (T(3) * ZZ - RR);
    dP[0][6] = -T(2) * c2b * X; dP[1][6] = -T(2) * c2b * Yy; dP[2][6] = T(4) * c2b * Z;
    P[7] = c2a * X * Z; dP[0][7] = c2a * Z; dP[2][7] = c2a * X;
    P[8] = c2c * (XX - YY); dP[0][8] = T(2) * c2c * X; dP[1][8] = -T(2) * c2c * Yy;
    // l = 3 : y(3x^2-y^2), xyz, y(5z^2-r^2), z(5z^2-3r^2), x(5z^2-r^2), z(x^2-y^2), x(x^2-3y^2)
    P[9] = c3a * Yy * (T(3) * XX - YY);
    dP[0][9] = c3a * T(6) * X * Yy; dP[1][9] = c3a * (T(3) * XX - T(3) * YY);
    P[10] = c3b * X * Yy * Z;
    dP[0][10] = c3b * Yy * Z; dP[1][10] = c3b * X * Z; dP[2][10] = c3b * X * Yy;
    P[11] = c3c * Yy * (T(5) * ZZ - RR);
    dP[0][11] = c3c * (-T(2) * X * Yy); dP[1][11] = c3c * (T(5) * ZZ - RR - T(2) * YY);
    dP[2][11] = c3c * (T(8) * Yy * Z);
    P[12] = c3d * Z * (T(5) * ZZ - T(3) * RR);
    dP[0][12] = c3d * (-T(6) * X * Z); dP[1][12] = c3d * (-T(6) * Yy * Z);
    dP[2][12] = c3d * (T(15) * ZZ - T(3) * RR - T(6) * ZZ);
    P[13] = c3c * X * (T(5) * ZZ - RR);
    dP[0][13] = c3c * (T(5) * ZZ - RR - T(2) * XX); dP[1][13] = c3c * (-T(2) * X * Yy);
    dP[2][13] = c3c * (T(8) * X * Z);
    P[14] = c3e * Z * (XX - YY);
    dP[0][14] = c3e * T(2) * X * Z; dP[1][14] = -c3e * T(2) * Yy * Z; dP[2][14] = c3e * (XX - YY);
    P[15] = c3a * X * (XX - T(3) * YY);
    dP[0][15] = c3a * (T(3) * XX - T(3) * YY); dP[1][15] = -c3a * T(6) * X * Yy;
    const int nlm = (l_max_ + 1) * (l_max_ + 1);
    for (int lm = 0; lm < nlm; ++lm) Y[lm] = P[lm];
    if (!grad) return;
    const T u[3] = {X, Yy, Z};
    for (int l = 0; l <= l_max_; ++l)
      for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm)
        for (int a = 0; a < 3; ++a) G[a][lm] = (dP[a][lm] - T(l) * P[lm] * u[a]) / r;
  }
};

}  // namespace sphericart
