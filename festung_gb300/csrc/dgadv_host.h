// Host-side static data shared by the C-ABI entry points and the device solver.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace dgadv {

constexpr int kMaxP = 3;           // highest degree with device kernels
constexpr int kMaxPHost = 4;       // highest degree of the host tables (reference limit)

inline int N_of_p(int p) { return (p + 1) * (p + 2) / 2; }

struct Rule1D { std::vector<double> Q, W; };
struct Rule2D { std::vector<double> Q1, Q2, W; };

bool quad_rule_1d(int qOrd, Rule1D &out);
bool quad_rule_2d(int qOrd, Rule2D &out);

double phi(int i, double x, double y);             // i is 0-based
double grad_phi(int i, int m, double x, double y);

// Reference-element tables of degree p (all row-major, 0-based).
struct RefTables {
  int p = 0, N = 0, Q = 0, R = 0, QM = 0;
  Rule2D vol;                      // quadRule2D(max(2p,1)): volume term and hatM
  Rule1D edge;                     // quadRule1D(2p+1): edge term
  std::vector<double> phiQ;        // Q x N
  std::vector<double> gradQ;       // 2 x Q x N
  std::vector<double> phi1D;       // 3 x R x N
  std::vector<double> thetaPhi;    // 3 x 3 x R x N  (edge nn, neighbour edge np)
  std::vector<double> hatM;        // N x N
  std::vector<double> hatMinv;     // N x N
  std::vector<double> DM;          // N x N   Taylor-derivative map times hatM
  std::vector<double> DMinv;       // N x N   its inverse
};
// volOrder: order of the volume rule (0: max(2p, 1), the explicit problem's; the implicit
// problem integrates with 2p + 1, advection_implicit/preprocessProblem.m)
bool build_ref_tables(int p, RefTables &t, std::string &err, int volOrder = 0);

// Grid data with generateGridData semantics (row-major per element / edge, 0-based ids).
struct Grid {
  int numT = 0, numV = 0, numE = 0;
  std::vector<int32_t> V0T;        // numT x 3
  std::vector<int32_t> V0E;        // numE x 2
  std::vector<int32_t> T0E;        // numE x 2, 0-based element or -1
  std::vector<int32_t> E0T;        // numT x 3
  std::vector<int32_t> E0E;        // numE x 2, 0-based local edge or -1
  std::vector<double> coordV;      // numV x 2
  std::vector<double> areaE, nuE, baryE, areaT, baryT, B, areaE0T, nuE0T, coordV0T, detJ0T;
  // B: numT x 4 as (B11, B12, B21, B22); nuE0T: numT x 3 x 2; coordV0T numT x 3 x 2
};
bool build_grid(int numV, const double *coordV_colmajor, int numT, const int32_t *V0T_colmajor,
                Grid &g, std::string &err);

// Taylor mass matrix blocks M_T(k) as assembleMatElemPhiTaylorPhiTaylor, packed upper
// triangle (i <= j) row by row, for every element.  Size numT x N(N+1)/2.
void taylor_mass_packed(const Grid &g, int p, std::vector<double> &out);

// Time-derivative limiting correction of the linear limiter in reference-derivative
// coordinates: Q_k = DM^-1 (S_k^-1 Mcorr_k S_k - I), columns 1..N-1, for every element
// (numT x N x (N-1), row-major per element).  S_k maps reference derivatives at the barycentre
// to the element's Taylor coefficients; Mcorr_k = diag(1/diag(M_T)) M_T.
void taylor_correction(const Grid &g, int p, const RefTables &t, std::vector<double> &out);

}  // namespace dgadv
