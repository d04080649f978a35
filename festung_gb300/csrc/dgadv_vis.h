// Solution output: the VTK (.vtu) and Tecplot (.plt) text files of core/visualizeDataLagr.m for
// one scalar field given at the Lagrange nodes of each triangle (core/projectDataDisc2DataLagr.m).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace dgadv {

enum { kVisVtk = 1, kVisTec = 2 };

// Values phi_i(node_j) (numP x N, row j) at the Lagrange nodes of degree p
// (core/projectDataDisc2DataLagr.m:49-53); returns numP (1, 3 or 6).
int lagrange_table(int p, int N, double *phiAtNodes);

// Element corner coordinates of a mesh (caller's element order) and the text of the parts of
// the files that do not change between outputs, built on first use.
class VisMesh {
 public:
  VisMesh() = default;
  // coordV: numV x 2 row-major pairs; V0T: numT x 3 row-major, 0-based.
  bool init(int numT, int numV, const double *coordV, const int32_t *V0T, std::string &err);
  bool empty() const { return K == 0; }
  // dataLagr: K x numP column-major with numP in {1, 3, 6}; writes <base>.<tLvl>.vtu and / or
  // <base>.<tLvl>.plt.  Returns false with err set if a file cannot be written.
  bool write(const double *dataLagr, int numP, const char *varName, const char *baseName, int tLvl,
             int types, std::string &err);

 private:
  int K = 0;
  std::vector<double> cx, cy;        // 3 corners per element, in element order
  std::string vtkGeo[2], tecGeo[2];  // cached geometry text, [0]: 3 points, [1]: 6 points
  size_t tecConnStart[2] = {0, 0};   // offset of the connectivity in tecGeo
  void point(int k, int j, double &x, double &y) const;
  const std::string &vtk_geometry(int numP);
  const std::string &tec_geometry(int numP);
};

}  // namespace dgadv
