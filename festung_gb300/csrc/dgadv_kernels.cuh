// Shared types of the device kernels.  One thread owns one element; all per-element arrays are
// structure-of-arrays with leading dimension Kp (coalesced loads across a warp).
//
// Stage pipeline (stage s of an SSP-RK step, advection/solveSubStep.m:57-99):
//   limiter off:          k_stage_op  (volume + upwind flux + mass + SSP)            -> c^(s)
//   linear limiter:       k_stage_op  -> c^(s) (p = 1) or cDot (p >= 2), element means scattered
//                         to the vertex min / max keys with atomics
//                         k_limit_dot_lin (p >= 2: limit cDot, Taylor mass correction, SSP)
//                         k_limit_lin  -> limited modal c^(s)
//   hierarchical limiter: the same passes on Taylor coefficients (k_limit_dot, k_limit)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dgadv {

template <int P> struct Dims {
  static constexpr int N = (P + 1) * (P + 2) / 2;
  static constexpr int Q = P == 0 ? 1 : (P == 1 ? 3 : (P == 2 ? 6 : 12));   // quadRule2D(max(2p,1))
  static constexpr int R = P + 1;                                            // quadRule1D(2p+1)
  static constexpr int NMT = N * (N + 1) / 2;                                // packed Taylor mass
  static constexpr int NC_HIER = P * (P + 1) / 2;                            // hierarchical sub-limiters
};

template <typename T, int P> struct Tab {
  static constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  T phiQ[Q][N];       // phi_j at the volume points
  T g1[Q][N];         // d/dx1 phi_i at the volume points
  T g2[Q][N];         // d/dx2 phi_i at the volume points
  T phi1D[3][R][N];   // phi_j at the edge points of edge n
  T thetaPhi[3][3][R][N];  // phi_j of the neighbour at the same points (theta_{n,np} o gamma_n)
  T hatMinv[N][N];
  T DM[N][N];         // modal -> reference derivatives at the barycentre (times hatM)
  T DMinv[N][N];
  T Gr[N][N];         // Gram matrix of the reference-derivative basis, DM^-T hatM DM^-1 (the
                      // Taylor mass block of an element is 2|T| S^-T Gr S^-1)
  // adjoint: the transposed mass solve folded into the test-function tables,
  // Hg1[q][j] = sum_i g1[q][i] hatMinv[i][j] (likewise Hg2, Hphi), or the tables themselves
  // where the forward path uses hatM = I (FP32)
  T Hg1[Q][N];
  T Hg2[Q][N];
  T Hphi[3][R][N];
  // forward: the mass solve folded into the volume and flux test functions,
  // Fg1[q][i] = sum_j hatMinv[i][j] g1[q][j] (likewise Fg2, Fphi), or the tables themselves
  // where the forward path uses hatM = I (FP32)
  T Fg1[Q][N];
  T Fg2[Q][N];
  T Fphi[3][R][N];
};

// Static per-element data of one mesh (device pointers, SoA with stride Kp).
template <typename T> struct Geo {
  int K, Kp, numV, Vp;
  const T *F;        // 2Q x Kp  volume flux factors W_q (B22 u1 - B12 u2)/detJ, W_q (B11 u2 - B21 u1)/detJ
  const T *Vn;       // 3R x Kp  markNotN * |E| * w_r * (u.nu)_r / detJ
  const T *Aop;      // N^2 x Kp the element operator (FP64 without source terms; null: none):
                     //          volume term and own outflow, hatM^-1 folded in
  const int *nbr;    // 3 x Kp   neighbour element across edge n, -1 on the boundary
  const int *code;   // Kp       bits 2n..2n+1: neighbour's local edge; bit 6+n: outflow counted;
                     //          bit 9+n: local vertex n lies on a Dirichlet edge
  const T *Bm;       // 4 x Kp   B11, B12, B21, B22
  const T *MT;       // time-derivative limiting: NMT x Kp packed Taylor mass blocks
                     // (hierarchical / strict) or N(N-1) x Kp rows of Q_k (linear)
  int mtOnTheFly;    // forward kernels rebuild the Taylor mass correction from B and Gr instead
                     // of reading MT (the limiter adjoint still reads MT)
  const int *V0T;    // 3 x Kp   vertex ids
  const int *vptr;   // numV+1   CSR vertex -> elements
  const int *vidx;
  const T *rhs;      // nTerms x N x Kp   (L - K_D - K_N)_m / detJ
  const T *cDV0T;    // nTerms x 3 x Kp   boundary values at the vertices
  int nTerms;
  int timeFn[4];
  const int *instOf; // ensembles: instance of each block of kBlock elements (null: one instance)
  const int *permv;  // Kp       caller's index of each element (ties of the limiter adjoint)
  int nInst;         // instances; each has its own global-extreme slots
};

struct LimArgs {
  int type;              // 0 linear, 1 hierarchical vertex
  int nc;                // number of centroid quantities
  int shift;             // replicate the reference's global shift
  const unsigned long long *gmm;   // 2 x nc encoded global min / max
};

}  // namespace dgadv
