// Host-side static data: quadrature rules, modal basis, reference tables, grid incidence maps
// and Taylor mass blocks.  Compiled with -ffp-contract=off so that every expression rounds as
// written (the same operation order as the reference's formulas).
#include "dgadv_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace dgadv {

// ---------------------------------------------------------------------------------------------
// quadRule1D (core/quadRule1D.m:48-95): Gauss-Legendre on [-1,1] mapped to [0,1].
bool quad_rule_1d(int qOrd, Rule1D &out) {
  std::vector<double> Q, W;
  if (qOrd == 0 || qOrd == 1) {
    Q = {0.0}; W = {2.0};
  } else if (qOrd == 2 || qOrd == 3) {
    const double s = std::sqrt(1.0 / 3.0);
    Q = {-s, s}; W = {1.0, 1.0};
  } else if (qOrd == 4 || qOrd == 5) {
    const double s = std::sqrt(3.0 / 5.0);
    Q = {-s, 0.0 * s, s};
    W = {1.0 / 9.0 * 5.0, 1.0 / 9.0 * 8.0, 1.0 / 9.0 * 5.0};
  } else if (qOrd == 6 || qOrd == 7) {
    const double c = 2.0 / 7.0 * std::sqrt(6.0 / 5.0);
    const double sg[4] = {-1, -1, 1, 1}, pm[4] = {1, -1, -1, 1};
    const double s30 = std::sqrt(30.0), wm[4] = {-1, 1, 1, -1};
    for (int i = 0; i < 4; ++i) {
      Q.push_back(sg[i] * std::sqrt(3.0 / 7.0 + pm[i] * c));
      W.push_back(1.0 / 36.0 * (18.0 + s30 * wm[i]));
    }
  } else if (qOrd == 8 || qOrd == 9) {
    const double c = std::sqrt(10.0 / 7.0), s70 = std::sqrt(70.0);
    const double sg[5] = {-1, -1, 0, 1, 1}, pm[5] = {2, -2, 0, -2, 2};
    const double wm[5] = {-1, 1, 0, 1, -1}, wa[5] = {0, 0, 190, 0, 0};
    for (int i = 0; i < 5; ++i) {
      Q.push_back(sg[i] * std::sqrt(5.0 + pm[i] * c) / 3.0);
      W.push_back(1.0 / 900.0 * (322.0 + 13.0 * s70 * wm[i] + wa[i]));
    }
  } else {
    return false;
  }
  out.Q.resize(Q.size()); out.W.resize(W.size());
  for (size_t i = 0; i < Q.size(); ++i) { out.Q[i] = (Q[i] + 1.0) / 2.0; out.W[i] = W[i] / 2.0; }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Gauss rules from the three-term recurrence of the orthonormal polynomials (Golub-Welsch
// eigenvalues by cyclic Jacobi rotations, then Newton refinement and Christoffel weights).
namespace {

void jacobi_eigenvalues(std::vector<double> A, int n, std::vector<double> &ev) {
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    if (off < 1e-300) break;
    for (int pI = 0; pI < n; ++pI)
      for (int q = pI + 1; q < n; ++q) {
        const double apq = A[pI * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[pI * n + pI], aqq = A[q * n + q];
        const double th = (aqq - app) / (2 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[k * n + pI], akq = A[k * n + q];
          A[k * n + pI] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[pI * n + k], aqk = A[q * n + k];
          A[pI * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
      }
  }
  ev.resize(n);
  for (int i = 0; i < n; ++i) ev[i] = A[i * n + i];
  std::sort(ev.begin(), ev.end());
}

// Gauss rule for the weight (1-x)^al (1+x)^be on [-1,1], n points ascending.
void gauss_jacobi(int n, double al, double be, std::vector<double> &x, std::vector<double> &w) {
  std::vector<double> a(n + 1), b(n + 1, 0.0);
  for (int k = 0; k <= n; ++k) {
    const double s = 2.0 * k + al + be;
    a[k] = (k == 0) ? (be - al) / (al + be + 2) : (be * be - al * al) / (s * (s + 2));
    if (k >= 1) {
      const double num = 4.0 * k * (k + al) * (k + be) * (k + al + be);
      const double den = s * s * (s + 1) * (s - 1);
      b[k] = std::sqrt(num / den);
    }
  }
  const double mu0 = std::pow(2.0, al + be + 1) * std::tgamma(al + 1) * std::tgamma(be + 1) /
                     std::tgamma(al + be + 2);
  std::vector<double> J(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    J[i * n + i] = a[i];
    if (i + 1 < n) J[i * n + i + 1] = J[(i + 1) * n + i] = b[i + 1];
  }
  jacobi_eigenvalues(J, n, x);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double xi = x[i];
    for (int it = 0; it < 6; ++it) {  // Newton on the orthonormal p_n
      double pm1 = 0, p0 = 1 / std::sqrt(mu0), dm1 = 0, d0 = 0;
      for (int k = 0; k < n; ++k) {
        const double p1 = ((xi - a[k]) * p0 - b[k] * pm1) / b[k + 1];
        const double d1 = (p0 + (xi - a[k]) * d0 - b[k] * dm1) / b[k + 1];
        pm1 = p0; p0 = p1; dm1 = d0; d0 = d1;
      }
      if (d0 == 0) break;
      const double dx = p0 / d0;
      xi -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    x[i] = xi;
    double pm1 = 0, p0 = 1 / std::sqrt(mu0), s = p0 * p0;
    for (int k = 0; k + 1 < n; ++k) {
      const double p1 = ((xi - a[k]) * p0 - b[k] * pm1) / b[k + 1];
      pm1 = p0; p0 = p1; s += p0 * p0;
    }
    w[i] = 1.0 / s;
  }
}

}  // namespace

// quadRule2D (core/quadRule2D.m:64-109).  Orders >= 7: collapsed-square product rule
// (the rule of core/triquad.m, re-derived: Gauss-Jacobi(0,1) in s, Gauss-Legendre in t,
// (x1,x2) = (s(1-t), s t), s fastest).
bool quad_rule_2d(int qOrd, Rule2D &r) {
  r.Q1.clear(); r.Q2.clear(); r.W.clear();
  if (qOrd == 0 || qOrd == 1) {
    r.Q1 = {1.0 / 3.0}; r.Q2 = {1.0 / 3.0}; r.W = {1.0 / 2.0};
  } else if (qOrd == 2) {
    r.Q1 = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0}; r.Q2 = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
    r.W = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0};
  } else if (qOrd == 3) {
    const double a1 = (3 + std::sqrt(3.0)) / 6, a2 = (3 - std::sqrt(3.0)) / 6;
    const double b1 = (6 + std::sqrt(6.0)) / 10, b2 = (6 - std::sqrt(6.0)) / 10;
    const double w1 = 1.0 / 8 + std::sqrt(6.0) / 72, w2 = 1.0 / 8 - std::sqrt(6.0) / 72;
    r.Q1 = {a1 * b1, a2 * b1, a1 * b2, a2 * b2};
    r.Q2 = {a2 * b1, a1 * b1, a2 * b2, a1 * b2};
    r.W = {w1, w1, w2, w2};
  } else if (qOrd == 4) {
    r.Q1 = {0.445948490915965, 0.108103018168070, 0.445948490915965,
            0.091576213509771, 0.816847572980458, 0.091576213509771};
    r.Q2 = {0.108103018168070, 0.445948490915965, 0.445948490915965,
            0.816847572980458, 0.091576213509771, 0.091576213509771};
    r.W = {0.111690794839005, 0.111690794839005, 0.111690794839005,
           0.054975871827661, 0.054975871827661, 0.054975871827661};
  } else if (qOrd == 5) {
    const double a1 = (6 - std::sqrt(15.0)) / 21, a2 = (6 + std::sqrt(15.0)) / 21;
    const double w1 = (155 - std::sqrt(15.0)) / 2400, w2 = (155 + std::sqrt(15.0)) / 2400;
    r.Q1 = {1.0 / 3, a1, 1 - 2 * a1, a1, a2, 1 - 2 * a2, a2};
    r.Q2 = {1.0 / 3, 1 - 2 * a1, a1, a1, 1 - 2 * a2, a2, a2};
    r.W = {9.0 / 80, w1, w1, w1, w2, w2, w2};
  } else if (qOrd == 6) {
    r.Q1 = {0.063089014491502, 0.873821971016996, 0.063089014491502,
            0.249286745170910, 0.501426509658179, 0.249286745170910,
            0.310352451033785, 0.053145049844816, 0.636502499121399,
            0.053145049844816, 0.636502499121399, 0.310352451033785};
    r.Q2 = {0.063089014491502, 0.063089014491502, 0.873821971016996,
            0.249286745170910, 0.249286745170910, 0.501426509658179,
            0.053145049844816, 0.310352451033785, 0.053145049844816,
            0.636502499121399, 0.310352451033785, 0.636502499121399};
    r.W = {0.025422453185103, 0.025422453185103, 0.025422453185103,
           0.058393137863189, 0.058393137863189, 0.058393137863189,
           0.041425537809187, 0.041425537809187, 0.041425537809187,
           0.041425537809187, 0.041425537809187, 0.041425537809187};
  } else if (qOrd >= 7 && qOrd <= 20) {
    const int n = qOrd;
    std::vector<double> X, wJ, Y, wL;
    gauss_jacobi(n, 0.0, 1.0, X, wJ);
    gauss_jacobi(n, 0.0, 0.0, Y, wL);
    for (int j = 0; j < n; ++j) {
      const double t = (1 + Y[j]) / 2, wt = wL[j] / 2;
      for (int i = 0; i < n; ++i) {
        const double s = (X[i] + 1) / 2, ws = wJ[i] / 4;
        const double yy = t * s;
        r.Q1.push_back(s - yy);
        r.Q2.push_back(yy);
        r.W.push_back(ws * wt);
      }
    }
  } else {
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Orthonormal modal basis on the reference triangle (core/phi.m:40-61, core/gradPhi.m:42-87).
double phi(int i, double x, double y) {
  const double s2 = std::sqrt(2.0), s3 = std::sqrt(3.0), s5 = std::sqrt(5.0), s6 = std::sqrt(6.0);
  const double s10 = std::sqrt(10.0), s14 = std::sqrt(14.0), s30 = std::sqrt(30.0);
  const double s70 = std::sqrt(70.0);
  switch (i) {
    case 0: return s2 * 1.0;
    case 1: return 2 - 6 * x;
    case 2: return 2 * s3 * (1 - x - 2 * y);
    case 3: return s6 * ((10 * x - 8) * x + 1);
    case 4: return s3 * ((5 * x - 4) * x + (-15 * y + 12) * y - 1);
    case 5: return 3 * s5 * ((3 * x + 8 * y - 4) * x + (3 * y - 4) * y + 1);
    case 6: return 2 * s2 * (-1 + (15 + (-45 + 35 * x) * x) * x);
    case 7: return 2 * s6 * (-1 + (13 + (-33 + 21 * x) * x) * x + (2 + (-24 + 42 * x) * x) * y);
    case 8: return 2 * s10 * (-1 + (9 + (-15 + 7 * x) * x) * x +
                              (6 + (-48 + 42 * x) * x + (-6 + 42 * x) * y) * y);
    case 9: return 2 * s14 * (-1 + (3 + (-3 + x) * x) * x +
                              (12 + (-24 + 12 * x) * x + (-30 + 30 * x + 20 * y) * y) * y);
    case 10: return s10 * (1 + (-24 + (126 + (-224 + 126 * x) * x) * x) * x);
    case 11: return s30 * (1 + (-22 + (105 + (-168 + 84 * x) * x) * x) * x +
                           (-2 + (42 + (-168 + 168 * x) * x) * x) * y);
    case 12: return 5 * s2 * (1 + (-18 + (69 + (-88 + 36 * x) * x) * x) * x +
                              (-6 + (102 + (-312 + 216 * x) * x) * x +
                               (6 + (-96 + 216 * x) * x) * y) * y);
    case 13: return s70 * (1 + (-12 + (30 + (-28 + 9 * x) * x) * x) * x +
                           (-12 + (132 + (-228 + 108 * x) * x) * x +
                            (30 + (-300 + 270 * x) * x + (-20 + 180 * x) * y) * y) * y);
    case 14: return 3 * s10 * (1 + (-4 + (6 + (-4 + x) * x) * x) * x +
                               (-20 + (60 + (-60 + 20 * x) * x) * x +
                                (90 + (-180 + 90 * x) * x + (-140 + 140 * x + 70 * y) * y) * y) * y);
  }
  return 0.0;
}

double grad_phi(int i, int m, double x, double y) {
  const double s2 = std::sqrt(2.0), s3 = std::sqrt(3.0), s5 = std::sqrt(5.0), s6 = std::sqrt(6.0);
  const double s10 = std::sqrt(10.0), s14 = std::sqrt(14.0), s30 = std::sqrt(30.0);
  const double s70 = std::sqrt(70.0);
  if (m == 0) {
    switch (i) {
      case 0: return 0.0;
      case 1: return -6 * 1.0;
      case 2: return -2 * s3 * 1.0;
      case 3: return s6 * (20 * x - 8);
      case 4: return s3 * (10 * x - 4);
      case 5: return 6 * s5 * (3 * x + 4 * y - 2);
      case 6: return 2 * s2 * (15 + (-90 + 105 * x) * x);
      case 7: return 2 * s6 * (13 + (-66 + 63 * x) * x + (-24 + 84 * x) * y);
      case 8: return 2 * s10 * (9 + (-30 + 21 * x) * x + (-48 + 84 * x + 42 * y) * y);
      case 9: return 2 * s14 * (3 + (-6 + 3 * x) * x + (-24 + 24 * x + 30 * y) * y);
      case 10: return s10 * (-24 + (252 + (-672 + 504 * x) * x) * x);
      case 11: return s30 * (-22 + (210 + (-504 + 336 * x) * x) * x + (42 + (-336 + 504 * x) * x) * y);
      case 12: return 5 * s2 * (-18 + (138 + (-264 + 144 * x) * x) * x +
                                (102 + (-624 + 648 * x) * x + (-96 + 432 * x) * y) * y);
      case 13: return s70 * (-12 + (60 + (-84 + 36 * x) * x) * x +
                             (132 + (-456 + 324 * x) * x + (-300 + 540 * x + 180 * y) * y) * y);
      case 14: return 3 * s10 * (-4 + (12 + (-12 + 4 * x) * x) * x +
                                 (60 + (-120 + 60 * x) * x + (-180 + 180 * x + 140 * y) * y) * y);
    }
  } else {
    switch (i) {
      case 0: return 0.0;
      case 1: return 0.0;
      case 2: return -4 * s3 * 1.0;
      case 3: return 0.0;
      case 4: return 2 * s3 * (-15 * y + 6);
      case 5: return 6 * s5 * (4 * x + 3 * y - 2);
      case 6: return 0.0;
      case 7: return 2 * s6 * (2 + (-24 + 42 * x) * x);
      case 8: return 2 * s10 * (6 + (-48 + 42 * x) * x + (-12 + 84 * x) * y);
      case 9: return 2 * s14 * (12 + (-24 + 12 * x) * x + (-60 + 60 * x + 60 * y) * y);
      case 10: return 0.0;
      case 11: return s30 * (-2 + (42 + (-168 + 168 * x) * x) * x);
      case 12: return 5 * s2 * (-6 + (102 + (-312 + 216 * x) * x) * x + (12 + (-192 + 432 * x) * x) * y);
      case 13: return s70 * (-12 + (132 + (-228 + 108 * x) * x) * x +
                             (60 + (-600 + 540 * x) * x + (-60 + 540 * x) * y) * y);
      case 14: return 3 * s10 * (-20 + (60 + (-60 + 20 * x) * x) * x +
                                 (180 + (-360 + 180 * x) * x + (-420 + 420 * x + 280 * y) * y) * y);
    }
  }
  return 0.0;
}

// ---------------------------------------------------------------------------------------------
// Small dense inverse (Gauss-Jordan with partial pivoting), row-major n x n.
static bool invert(const std::vector<double> &A, int n, std::vector<double> &inv) {
  std::vector<double> M(A);
  inv.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[r * n + c]) > std::fabs(M[piv * n + c])) piv = r;
    if (M[piv * n + c] == 0.0) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) { std::swap(M[c * n + k], M[piv * n + k]); std::swap(inv[c * n + k], inv[piv * n + k]); }
    const double d = M[c * n + c];
    for (int k = 0; k < n; ++k) { M[c * n + k] /= d; inv[c * n + k] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) { M[r * n + k] -= f * M[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
  return true;
}

static void matmul(const std::vector<double> &A, const std::vector<double> &B, int n,
                   std::vector<double> &C) {
  C.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0;
      for (int k = 0; k < n; ++k) s += A[i * n + k] * B[k * n + j];
      C[i * n + j] = s;
    }
}

// ---------------------------------------------------------------------------------------------
// Taylor basis (core/phiTaylorPhy.m:70-135) of one element, evaluated at offsets (dx,dy) from
// the barycentre.  The mean corrections use, for a function of degree d, quadRule2D(d) mapped
// into the element (offsets mx, my of the rule's points from the barycentre).
struct TaylorElem {
  double dX;                 // 2 / sqrt(2 |T|)
  double mean[15];           // correction subtracted before scaling (index = basis function)
};

static double seq_dot(const std::vector<double> &a, const std::vector<double> &w) {
  double s = 0;
  for (size_t r = 0; r < a.size(); ++r) s = s + a[r] * w[r];
  return s;
}

// offsets of the points of quadRule2D(qOrd) from the barycentre: X = (B1 Q1 + B2 Q2) + a1 - b
static void rule_offsets(int qOrd, const double Bm[4], const double a1[2], const double b[2],
                         std::vector<double> &mx, std::vector<double> &my, std::vector<double> &W) {
  Rule2D r;
  quad_rule_2d(qOrd, r);
  const size_t R = r.W.size();
  mx.resize(R); my.resize(R); W = r.W;
  for (size_t q = 0; q < R; ++q) {
    mx[q] = (Bm[0] * r.Q1[q] + Bm[1] * r.Q2[q]) + a1[0] * 1.0 - b[0];
    my[q] = (Bm[2] * r.Q1[q] + Bm[3] * r.Q2[q]) + a1[1] * 1.0 - b[1];
  }
}

static void taylor_elem_setup(int N, const double Bm[4], const double a1[2], const double b[2],
                              double areaT, TaylorElem &te) {
  te.dX = 2 / std::sqrt(2 * areaT);
  std::fill(te.mean, te.mean + 15, 0.0);
  std::vector<double> mx, my, W, tmp;
  if (N > 3) {
    rule_offsets(2, Bm, a1, b, mx, my, W);
    tmp.resize(W.size());
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = mx[r] * mx[r];
    te.mean[3] = seq_dot(tmp, W);
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = 2 * (mx[r] * my[r]);
    te.mean[4] = seq_dot(tmp, W);
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = my[r] * my[r];
    te.mean[5] = seq_dot(tmp, W);
  }
  if (N > 6) {
    rule_offsets(3, Bm, a1, b, mx, my, W);
    tmp.resize(W.size());
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = std::pow(mx[r], 3);
    te.mean[6] = seq_dot(tmp, W) / 3;
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = mx[r] * mx[r] * my[r];
    te.mean[7] = seq_dot(tmp, W);
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = mx[r] * (my[r] * my[r]);
    te.mean[8] = seq_dot(tmp, W);
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = std::pow(my[r], 3);
    te.mean[9] = seq_dot(tmp, W) / 3;
  }
  if (N > 10) {
    rule_offsets(4, Bm, a1, b, mx, my, W);
    tmp.resize(W.size());
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = std::pow(mx[r], 4);
    te.mean[10] = seq_dot(tmp, W) / 12;
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = std::pow(mx[r], 3) * my[r];
    te.mean[11] = seq_dot(tmp, W) / 3;
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = mx[r] * mx[r] * (my[r] * my[r]);
    te.mean[12] = seq_dot(tmp, W) / 2;
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = mx[r] * std::pow(my[r], 3);
    te.mean[13] = seq_dot(tmp, W) / 3;
    for (size_t r = 0; r < W.size(); ++r) tmp[r] = std::pow(my[r], 4);
    te.mean[14] = seq_dot(tmp, W) / 12;
  }
}

static double taylor_eval(int j, double dx, double dy, const TaylorElem &te) {
  const double d = te.dX, d2 = d * d;
  switch (j) {
    case 0: return 1.0;
    case 1: return dx * d;
    case 2: return dy * d;
    case 3: return (0.5 * (dx * dx) - te.mean[3]) * d2;
    case 4: return (dx * dy - te.mean[4]) * d2;
    case 5: return (0.5 * (dy * dy) - te.mean[5]) * d2;
    case 6: return (std::pow(dx, 3) / 6 - te.mean[6]) * std::pow(d, 3);
    case 7: return (0.5 * (dx * dx) * dy - te.mean[7]) * std::pow(d, 3);
    case 8: return (0.5 * dx * (dy * dy) - te.mean[8]) * std::pow(d, 3);
    case 9: return (std::pow(dy, 3) / 6 - te.mean[9]) * std::pow(d, 3);
    case 10: return (std::pow(dx, 4) / 24 - te.mean[10]) * std::pow(d, 4);
    case 11: return (std::pow(dx, 3) * dy / 6 - te.mean[11]) * std::pow(d, 4);
    case 12: return ((dx * dx) * (dy * dy) / 4 - te.mean[12]) * std::pow(d, 4);
    case 13: return (dx * std::pow(dy, 3) / 6 - te.mean[13]) * std::pow(d, 4);
    case 14: return (std::pow(dy, 4) / 24 - te.mean[14]) * std::pow(d, 4);
  }
  return 0.0;
}

// ---------------------------------------------------------------------------------------------
bool build_ref_tables(int p, RefTables &t, std::string &err, int volOrder) {
  if (p < 0 || p > kMaxPHost) { err = "p must be in 0..4"; return false; }
  const int N = N_of_p(p);
  t.p = p; t.N = N;
  const int qv = volOrder > 0 ? volOrder : std::max(2 * p, 1);
  quad_rule_2d(qv, t.vol);
  quad_rule_1d(2 * p + 1, t.edge);
  t.Q = (int)t.vol.W.size();
  t.R = (int)t.edge.W.size();
  const int Q = t.Q, R = t.R;
  t.phiQ.resize(Q * N); t.gradQ.resize(2 * Q * N);
  for (int q = 0; q < Q; ++q)
    for (int i = 0; i < N; ++i) {
      t.phiQ[q * N + i] = phi(i, t.vol.Q1[q], t.vol.Q2[q]);
      t.gradQ[q * N + i] = grad_phi(i, 0, t.vol.Q1[q], t.vol.Q2[q]);
      t.gradQ[Q * N + q * N + i] = grad_phi(i, 1, t.vol.Q1[q], t.vol.Q2[q]);
    }
  // edge traces: gammaMap(n, s) = (1-s, s), (0, 1-s), (s, 0)          core/gammaMap.m:50-57
  t.phi1D.resize(3 * R * N);
  for (int n = 0; n < 3; ++n)
    for (int r = 0; r < R; ++r) {
      const double s = t.edge.Q[r];
      double x = 0, y = 0;
      if (n == 0) { x = 1 - s; y = s; } else if (n == 1) { x = 0; y = 1 - s; } else { x = s; y = 0; }
      for (int i = 0; i < N; ++i) t.phi1D[(n * R + r) * N + i] = phi(i, x, y);
    }
  // neighbour traces: theta_{nn,np} applied to gamma_nn(s)              core/theta.m:109-133
  t.thetaPhi.resize(9 * R * N);
  for (int nn = 0; nn < 3; ++nn)
    for (int np = 0; np < 3; ++np)
      for (int r = 0; r < R; ++r) {
        const double s = t.edge.Q[r];
        double X1 = 0, X2 = 0;
        if (nn == 0) { X1 = 1 - s; X2 = s; } else if (nn == 1) { X1 = 0; X2 = 1 - s; } else { X1 = s; X2 = 0; }
        double P1 = 0, P2 = 0;
        if (nn == 0) {
          if (np == 0) { P1 = 1 - X1; P2 = 1 - X2; } else if (np == 1) { P1 = 0; P2 = X2; } else { P1 = X1; P2 = 0; }
        } else if (nn == 1) {
          if (np == 0) { P1 = 1 - X2; P2 = X2; } else if (np == 1) { P1 = 0; P2 = 1 - X2; } else { P1 = X2; P2 = 0; }
        } else {
          if (np == 0) { P1 = X1; P2 = 1 - X1; } else if (np == 1) { P1 = 0; P2 = X1; } else { P1 = 1 - X1; P2 = 0; }
        }
        for (int i = 0; i < N; ++i) t.thetaPhi[((nn * 3 + np) * R + r) * N + i] = phi(i, P1, P2);
      }
  // hatM with the volume rule (core/integrateRefElemPhiPhi.m:49-59)
  t.hatM.resize(N * N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0;
      for (int q = 0; q < Q; ++q) s = s + t.vol.W[q] * t.phiQ[q * N + i] * t.phiQ[q * N + j];
      t.hatM[i * N + j] = s;
    }
  if (!invert(t.hatM, N, t.hatMinv)) { err = "hatM is singular"; return false; }
  // Taylor map on the reference element itself (B = I): T_ref(i,j) = int phi_i phiT_j with the
  // rule of order 2p+1 (core/assembleMatElemPhiDiscPhiTaylor.m:68-77 with 2|T| = 1).
  // For an element with Jacobian B the Taylor coefficients of a modal vector c are
  // cT = S_B D hatM c with D = S_I^-1 T_ref^-1, where S_B maps reference derivatives at the
  // barycentre to physical ones scaled by dX^-|a|.  DM = D hatM, DMinv = hatM^-1 T_ref S_I.
  {
    Rule2D r;
    quad_rule_2d(std::max(2 * p + 1, 1), r);
    const double Bm[4] = {1.0, 0.0, 0.0, 1.0}, a1[2] = {0.0, 0.0};
    const double b[2] = {(0.0 + 1.0 + 0.0) / 3, (0.0 + 0.0 + 1.0) / 3};
    TaylorElem te;
    taylor_elem_setup(N, Bm, a1, b, 0.5, te);
    std::vector<double> T(N * N);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double s = 0;
        for (size_t q = 0; q < r.W.size(); ++q) {
          const double dx = (Bm[0] * r.Q1[q] + Bm[1] * r.Q2[q]) + a1[0] - b[0];
          const double dy = (Bm[2] * r.Q1[q] + Bm[3] * r.Q2[q]) + a1[1] - b[1];
          s = s + phi(i, r.Q1[q], r.Q2[q]) * taylor_eval(j, dx, dy, te) * r.W[q];
        }
        T[i * N + j] = 2 * 0.5 * s;
      }
    std::vector<double> Tinv;
    if (!invert(T, N, Tinv)) { err = "Taylor map singular"; return false; }
    std::vector<double> SI(N, 1.0);  // dX^|a| with dX = 2 on the reference element
    for (int d = 0, idx = 0; d <= p; ++d)
      for (int m = 0; m <= d; ++m, ++idx) SI[idx] = std::pow(2.0, d);
    std::vector<double> D(N * N), TS(N * N);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        D[i * N + j] = SI[i] * Tinv[i * N + j];     // S_I^-1 = diag(dX^|a|)
        TS[i * N + j] = T[i * N + j] / SI[j];       // T_ref S_I
      }
    matmul(D, t.hatM, N, t.DM);
    matmul(t.hatMinv, TS, N, t.DMinv);
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// generateGridData (core/generateGridData.m:130-198).
bool build_grid(int numV, const double *coordV, int numT, const int32_t *V0Tc, Grid &g,
                std::string &err) {
  if (numV <= 0 || numT <= 0 || !coordV || !V0Tc) { err = "empty mesh"; return false; }
  g.numT = numT; g.numV = numV;
  g.coordV.resize(2 * (size_t)numV);
  for (int v = 0; v < numV; ++v) { g.coordV[2 * v] = coordV[v]; g.coordV[2 * v + 1] = coordV[numV + v]; }
  g.V0T.resize(3 * (size_t)numT);
  for (int t = 0; t < numT; ++t)
    for (int n = 0; n < 3; ++n) {
      const int32_t v = V0Tc[(size_t)n * numT + t];
      if (v < 0 || v >= numV) { err = "V0T holds a vertex id out of range"; return false; }
      g.V0T[3 * (size_t)t + n] = v;
    }
  // undirected edges numbered like find(triu(V2T + V2T')): ascending column (larger vertex),
  // then ascending row (smaller vertex)
  struct DE { int64_t key; int32_t t; int8_t n; };
  std::vector<DE> de(3 * (size_t)numT);
  for (int t = 0; t < numT; ++t)
    for (int n = 0; n < 3; ++n) {
      const int a = g.V0T[3 * (size_t)t + n], b = g.V0T[3 * (size_t)t + (n + 1) % 3];
      if (a == b) { err = "degenerate triangle"; return false; }
      const int lo = std::min(a, b), hi = std::max(a, b);
      de[3 * (size_t)t + n] = {(int64_t)hi * numV + lo, t, (int8_t)n};
    }
  std::vector<int64_t> keys(de.size());
  for (size_t i = 0; i < de.size(); ++i) keys[i] = de[i].key;
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  const int numE = (int)keys.size();
  g.numE = numE;
  auto edge_of = [&](int a, int b) -> int {
    const int lo = std::min(a, b), hi = std::max(a, b);
    const int64_t k = (int64_t)hi * numV + lo;
    return (int)(std::lower_bound(keys.begin(), keys.end(), k) - keys.begin());
  };
  g.T0E.assign(2 * (size_t)numE, -1);
  g.V0E.assign(2 * (size_t)numE, -1);
  std::vector<int32_t> cnt(numE, 0);
  // first owner = smallest element index (the last writer of the reversed loop)
  for (int t = 0; t < numT; ++t)
    for (int n = 0; n < 3; ++n) {
      const int a = g.V0T[3 * (size_t)t + n], b = g.V0T[3 * (size_t)t + (n + 1) % 3];
      const int e = edge_of(a, b);
      if (cnt[e] == 0) {
        g.T0E[2 * (size_t)e] = t; g.V0E[2 * (size_t)e] = a; g.V0E[2 * (size_t)e + 1] = b;
      } else if (cnt[e] == 1) {
        if (g.V0E[2 * (size_t)e] != b || g.V0E[2 * (size_t)e + 1] != a) {
          err = "edge shared with equal orientation (mesh not consistently counter-clockwise)";
          return false;
        }
        g.T0E[2 * (size_t)e + 1] = t;
      } else {
        err = "edge shared by more than two triangles";
        return false;
      }
      ++cnt[e];
    }
  g.E0T.resize(3 * (size_t)numT);
  for (int t = 0; t < numT; ++t)
    for (int n = 0; n < 3; ++n)
      g.E0T[3 * (size_t)t + n] = edge_of(g.V0T[3 * (size_t)t + (n + 1) % 3], g.V0T[3 * (size_t)t + (n + 2) % 3]);
  g.E0E.assign(2 * (size_t)numE, -1);
  for (int t = 0; t < numT; ++t)
    for (int n = 0; n < 3; ++n) {
      const int e = g.E0T[3 * (size_t)t + n];
      if (g.T0E[2 * (size_t)e] == t) g.E0E[2 * (size_t)e] = n; else g.E0E[2 * (size_t)e + 1] = n;
    }
  const double *X = g.coordV.data();
  g.areaE.resize(numE); g.nuE.resize(2 * (size_t)numE); g.baryE.resize(2 * (size_t)numE);
  for (int e = 0; e < numE; ++e) {
    const int a = g.V0E[2 * (size_t)e], b = g.V0E[2 * (size_t)e + 1];
    const double vx = X[2 * b] - X[2 * a], vy = X[2 * b + 1] - X[2 * a + 1];
    const double len = std::sqrt(vx * vx + vy * vy);
    g.areaE[e] = len;
    g.nuE[2 * (size_t)e] = (vx * 0.0 + vy * 1.0) / len;
    g.nuE[2 * (size_t)e + 1] = (vx * -1.0 + vy * 0.0) / len;
    g.baryE[2 * (size_t)e] = 0.5 * (X[2 * a] + X[2 * b]);
    g.baryE[2 * (size_t)e + 1] = 0.5 * (X[2 * a + 1] + X[2 * b + 1]);
  }
  g.areaT.resize(numT); g.baryT.resize(2 * (size_t)numT); g.B.resize(4 * (size_t)numT);
  g.areaE0T.resize(3 * (size_t)numT); g.nuE0T.resize(6 * (size_t)numT);
  g.coordV0T.resize(6 * (size_t)numT); g.detJ0T.resize(numT);
  for (int t = 0; t < numT; ++t) {
    const int v1 = g.V0T[3 * (size_t)t], v2 = g.V0T[3 * (size_t)t + 1], v3 = g.V0T[3 * (size_t)t + 2];
    const double x1 = X[2 * v1], y1 = X[2 * v1 + 1], x2 = X[2 * v2], y2 = X[2 * v2 + 1];
    const double x3 = X[2 * v3], y3 = X[2 * v3 + 1];
    const double area = (x1 * y2 + x2 * y3 + x3 * y1 - x1 * y3 - x2 * y1 - x3 * y2) / 2;
    if (!(area > 0)) { err = "triangle with non-positive area (vertices must be counter-clockwise)"; return false; }
    g.areaT[t] = area;
    g.detJ0T[t] = 2 * area;
    g.baryT[2 * (size_t)t] = (x1 + x2 + x3) / 3;
    g.baryT[2 * (size_t)t + 1] = (y1 + y2 + y3) / 3;
    const double c[3][2] = {{x1, y1}, {x2, y2}, {x3, y3}};
    for (int n = 0; n < 3; ++n)
      for (int m = 0; m < 2; ++m) g.coordV0T[6 * (size_t)t + 2 * n + m] = c[n][m];
    g.B[4 * (size_t)t + 0] = x2 - x1;   // B(:,1,1)
    g.B[4 * (size_t)t + 1] = x3 - x1;   // B(:,1,2)
    g.B[4 * (size_t)t + 2] = y2 - y1;   // B(:,2,1)
    g.B[4 * (size_t)t + 3] = y3 - y1;   // B(:,2,2)
    for (int n = 0; n < 3; ++n) {
      const int e = g.E0T[3 * (size_t)t + n];
      const double sig = (g.T0E[2 * (size_t)e + 1] == t) ? -1.0 : 1.0;
      g.areaE0T[3 * (size_t)t + n] = g.areaE[e];
      g.nuE0T[6 * (size_t)t + 2 * n] = g.nuE[2 * (size_t)e] * sig;
      g.nuE0T[6 * (size_t)t + 2 * n + 1] = g.nuE[2 * (size_t)e + 1] * sig;
    }
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Taylor mass blocks (core/assembleMatElemPhiTaylorPhiTaylor.m:50-64), packed upper triangle.
void taylor_mass_packed(const Grid &g, int p, std::vector<double> &out) {
  const int N = N_of_p(p);
  const int P = N * (N + 1) / 2;
  Rule2D r;
  quad_rule_2d(std::max(2 * p, 1), r);
  const size_t R = r.W.size();
  out.assign((size_t)g.numT * P, 0.0);
  std::vector<double> val(R * N);
  for (int t = 0; t < g.numT; ++t) {
    const double *Bm = &g.B[4 * (size_t)t];
    const double a1[2] = {g.coordV0T[6 * (size_t)t], g.coordV0T[6 * (size_t)t + 1]};
    const double b[2] = {g.baryT[2 * (size_t)t], g.baryT[2 * (size_t)t + 1]};
    TaylorElem te;
    taylor_elem_setup(N, Bm, a1, b, g.areaT[t], te);
    for (size_t q = 0; q < R; ++q) {
      const double dx = (Bm[0] * r.Q1[q] + Bm[1] * r.Q2[q]) + a1[0] * 1.0 - b[0];
      const double dy = (Bm[2] * r.Q1[q] + Bm[3] * r.Q2[q]) + a1[1] * 1.0 - b[1];
      for (int j = 0; j < N; ++j) val[q * N + j] = taylor_eval(j, dx, dy, te);
    }
    size_t o = (size_t)t * P;
    for (int i = 0; i < N; ++i)
      for (int j = i; j < N; ++j) {
        double s = 0;
        for (size_t q = 0; q < R; ++q) s = s + val[q * N + i] * val[q * N + j] * r.W[q];
        out[o++] = 2 * g.areaT[t] * s;
      }
  }
}

// Coefficients of (a + b z)^(D-m) (c + e z)^m in z^j (row m, column j).
static void deriv_block_host(double a, double b, double c, double e, int D, std::vector<double> &S) {
  S.assign((D + 1) * (D + 1), 0.0);
  for (int m = 0; m <= D; ++m) {
    std::vector<double> poly(D + 1, 0.0);
    poly[0] = 1.0;
    for (int r = 0; r < D; ++r) {
      const bool first = r < D - m;
      const double x0 = first ? a : c, x1 = first ? b : e;
      for (int j = D; j >= 0; --j) poly[j] = poly[j] * x0 + (j > 0 ? poly[j - 1] * x1 : 0.0);
    }
    for (int j = 0; j <= D; ++j) S[m * (D + 1) + j] = poly[j];
  }
}

void taylor_correction(const Grid &g, int p, const RefTables &t, std::vector<double> &out) {
  const int N = N_of_p(p), P = N * (N + 1) / 2;
  std::vector<double> mt;
  taylor_mass_packed(g, p, mt);
  out.assign((size_t)g.numT * N * (N - 1), 0.0);
  std::vector<double> S(N * N), Si(N * N), M(N * N), W(N * N), blk;
  for (int k = 0; k < g.numT; ++k) {
    const double B11 = g.B[4 * (size_t)k], B12 = g.B[4 * (size_t)k + 1];
    const double B21 = g.B[4 * (size_t)k + 2], B22 = g.B[4 * (size_t)k + 3];
    const double det = B11 * B22 - B12 * B21;
    const double A11 = B22 / det, A12 = -B12 / det, A21 = -B21 / det, A22 = B11 / det;
    const double dX = 2 / std::sqrt(g.detJ0T[k]);
    std::fill(S.begin(), S.end(), 0.0);
    std::fill(Si.begin(), Si.end(), 0.0);
    S[0] = 1.0; Si[0] = 1.0;
    for (int d = 1; d <= p; ++d) {
      const int off = d * (d + 1) / 2;
      deriv_block_host(A11, A21, A12, A22, d, blk);
      for (int m = 0; m <= d; ++m)
        for (int j = 0; j <= d; ++j) S[(off + m) * N + off + j] = blk[m * (d + 1) + j] / std::pow(dX, d);
      deriv_block_host(B11, B21, B12, B22, d, blk);
      for (int m = 0; m <= d; ++m)
        for (int j = 0; j <= d; ++j) Si[(off + m) * N + off + j] = blk[m * (d + 1) + j] * std::pow(dX, d);
    }
    // Mcorr from the packed Taylor mass block
    const double *pk = &mt[(size_t)k * P];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        const int a = std::min(i, j), b = std::max(i, j);
        M[i * N + j] = pk[a * N - a * (a - 1) / 2 + (b - a)];
      }
    for (int i = 0; i < N; ++i) {
      const double dii = M[i * N + i];
      for (int j = 0; j < N; ++j) W[i * N + j] = M[i * N + j] / dii;
    }
    std::vector<double> T1, T2;
    matmul(Si, W, N, T1);     // S^-1 Mcorr
    matmul(T1, S, N, T2);     // S^-1 Mcorr S
    for (int i = 0; i < N; ++i) T2[i * N + i] -= 1.0;
    std::vector<double> Qk;
    matmul(t.DMinv, T2, N, Qk);
    for (int i = 0; i < N; ++i)
      for (int j = 1; j < N; ++j) out[((size_t)k * N + i) * (N - 1) + (j - 1)] = Qk[i * N + j];
  }
}

}  // namespace dgadv
