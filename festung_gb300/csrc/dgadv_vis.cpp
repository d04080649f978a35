// Solution output files (core/visualizeDataLagr.m:114-291, scalar data): text formatted in
// parallel on the host cores, geometry text cached per mesh.
#include "dgadv_guard.h"
#include "dgadv_vis.h"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>

#include "../../include/dgadv.h"
#include "dgadv_host.h"

namespace dgadv {

namespace {

// Lagrange nodes (L1, L2) on the reference triangle: centroid (p = 0), vertices (p = 1),
// vertices then the midpoints of edges 1, 2, 3 (p >= 2)   core/projectDataDisc2DataLagr.m:49-53
const double kL1[6] = {0.0, 1.0, 0.0, 0.5, 0.0, 0.5};
const double kL2[6] = {0.0, 0.0, 1.0, 0.5, 0.5, 0.0};
// Node of the file's point j of a quadratic element: VTK / Tecplot list the vertices, then the
// midpoints of the edges 1-2, 2-3, 3-1 (core/visualizeDataLagr.m:216-217, columns [1,2,3,6,4,5]).
const int kNode6[6] = {0, 1, 2, 5, 3, 4};

constexpr size_t kItemChars = 96;      // longest formatted item ("%.12e %.12e %.1e\n" + indent)
constexpr size_t kChunkItems = 1 << 15;

// Formats items 0..n-1 (item i written by f(i, buf), returning its length) into consecutive
// parts, in parallel over host threads for large n.
template <class F>
std::vector<std::string> format_parts(size_t n, F f) {
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), (n + kChunkItems - 1) / kChunkItems);
  std::vector<std::string> parts(std::max<size_t>(nt, 1));
  auto run = [&](size_t t) {
    const size_t i0 = n * t / parts.size(), i1 = n * (t + 1) / parts.size();
    std::string &s = parts[t];
    s.reserve((i1 - i0) * 24);
    char buf[kItemChars];
    for (size_t i = i0; i < i1; ++i) s.append(buf, f(i, buf));
  };
  if (parts.size() == 1) {
    run(0);
  } else {
    std::vector<std::thread> th;
    for (size_t t = 1; t < parts.size(); ++t) th.emplace_back(run, t);
    run(0);
    for (auto &x : th) x.join();
  }
  return parts;
}

std::string join(const std::vector<std::string> &parts) {
  size_t n = 0;
  for (const auto &s : parts) n += s.size();
  std::string out;
  out.reserve(n);
  for (const auto &s : parts) out += s;
  return out;
}

// MATLAB fprintf cycling a format of `per` conversions separated by spaces and ended by a
// newline: value i is followed by '\n' if it ends a line, else by ' ' (also the last value).
inline char cycle_sep(size_t i, size_t per) { return (i % per == per - 1) ? '\n' : ' '; }

class File {
 public:
  explicit File(const std::string &path) : fp_(std::fopen(path.c_str(), "wb")), path_(path) {}
  ~File() { if (fp_) std::fclose(fp_); }
  bool ok() const { return fp_ != nullptr && !bad_; }
  void put(const std::string &s) { put(s.data(), s.size()); }
  void put(const char *s) { put(s, std::strlen(s)); }
  void put(const char *s, size_t n) {
    if (fp_ && !bad_ && n && std::fwrite(s, 1, n, fp_) != n) bad_ = true;
  }
  void parts(const std::vector<std::string> &v) { for (const auto &s : v) put(s); }
  void printf(const char *fmt, ...) __attribute__((format(printf, 2, 3))) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    const int n = std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (n > 0) put(buf, std::min<size_t>((size_t)n, sizeof buf - 1));
  }
  bool close() {
    if (!fp_) return false;
    const bool good = !bad_ && std::fclose(fp_) == 0;
    fp_ = nullptr;
    return good;
  }

 private:
  FILE *fp_;
  std::string path_;
  bool bad_ = false;
};

// mkdir -p of the directory part of `base` (core/visualizeDataLagr.m:100-103).
bool make_parent_dirs(const std::string &base, std::string &err) {
  const size_t slash = base.find_last_of('/');
  if (slash == std::string::npos || slash == 0) return true;
  const std::string dir = base.substr(0, slash);
  for (size_t pos = 1; pos <= dir.size(); ++pos) {
    if (pos != dir.size() && dir[pos] != '/') continue;
    const std::string d = dir.substr(0, pos);
    struct stat st;
    if (stat(d.c_str(), &st) == 0) {
      if (!S_ISDIR(st.st_mode)) { err = "not a directory: " + d; return false; }
      continue;
    }
    if (mkdir(d.c_str(), 0777) != 0 && errno != EEXIST) {
      err = "cannot create directory " + d + ": " + std::strerror(errno);
      return false;
    }
  }
  return true;
}

}  // namespace

int lagrange_table(int p, int N, double *phiAtNodes) {
  const int numP = p == 0 ? 1 : (p == 1 ? 3 : 6);
  for (int j = 0; j < numP; ++j) {
    const double x = p == 0 ? 1.0 / 3.0 : kL1[j], y = p == 0 ? 1.0 / 3.0 : kL2[j];
    for (int i = 0; i < N; ++i) phiAtNodes[(size_t)j * N + i] = phi(i, x, y);
  }
  return numP;
}

bool VisMesh::init(int numT, int numV, const double *coordV, const int32_t *V0T, std::string &err) {
  if (numT <= 0 || numV <= 0 || !coordV || !V0T) { err = "empty mesh"; return false; }
  K = numT;
  cx.resize(3 * (size_t)K);
  cy.resize(3 * (size_t)K);
  for (size_t i = 0; i < 3 * (size_t)K; ++i) {
    const int v = V0T[i];
    if (v < 0 || v >= numV) { err = "V0T holds a vertex id out of range"; K = 0; return false; }
    cx[i] = coordV[2 * (size_t)v];
    cy[i] = coordV[2 * (size_t)v + 1];
  }
  for (auto &s : vtkGeo) s.clear();
  for (auto &s : tecGeo) s.clear();
  return true;
}

// Point j of element k in file order: the corners, then (6 points) the midpoints of edges 3, 1, 2
// of the reference's numbering (edge n opposite corner n), each 0.5 * (a + b) as g.baryE
// (core/generateGridData.m:161).
void VisMesh::point(int k, int j, double &x, double &y) const {
  const size_t b = 3 * (size_t)k;
  if (j < 3) { x = cx[b + j]; y = cy[b + j]; return; }
  const int a = j - 3, c = (j - 2) % 3;   // 3: corners 0-1, 4: 1-2, 5: 2-0
  x = 0.5 * (cx[b + a] + cx[b + c]);
  y = 0.5 * (cy[b + a] + cy[b + c]);
}

// <Piece> through </Cells> of the .vtu file (core/visualizeDataLagr.m:139-152).
const std::string &VisMesh::vtk_geometry(int numP) {
  std::string &g = vtkGeo[numP == 6];
  if (!g.empty()) return g;
  const size_t nPts = (size_t)K * numP;
  char head[256];
  std::snprintf(head, sizeof head,
                "    <Piece NumberOfPoints=\"%zu\" NumberOfCells=\"%d\">\n      <Points>\n"
                "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n",
                nPts, K);
  g = head;
  g += join(format_parts(nPts, [&](size_t i, char *b) {
    double x, y;
    point((int)(i / numP), (int)(i % numP), x, y);
    return std::snprintf(b, kItemChars, "          %.12e %.12e %.1e\n", x, y, 0.0);
  }));
  g += "        </DataArray>\n      </Points>\n      <Cells>\n"
       "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n           ";
  g += join(format_parts(nPts, [](size_t i, char *b) { return std::snprintf(b, kItemChars, "%zu ", i); }));
  g += "\n        </DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
  g += join(format_parts((size_t)K, [&](size_t i, char *b) {
    return std::snprintf(b, kItemChars, "           %zu\n", (i + 1) * numP);
  }));
  g += "        </DataArray>\n        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
  const int id = numP == 6 ? 22 : 5;   // VTK_QUADRATIC_TRIANGLE / VTK_TRIANGLE
  g += join(format_parts((size_t)K, [&](size_t, char *b) {
    return std::snprintf(b, kItemChars, "           %d\n", id);
  }));
  g += "        </DataArray>\n      </Cells>\n";
  return g;
}

// Coordinate blocks and connectivity of the .plt file (core/visualizeDataLagr.m:279-290); the
// zone header and the data go between them.
const std::string &VisMesh::tec_geometry(int numP) {
  std::string &g = tecGeo[numP == 6];
  if (!g.empty()) return g;
  const size_t nPts = (size_t)K * numP;
  for (int m = 0; m < 2; ++m) {
    g += join(format_parts(nPts, [&](size_t i, char *b) {
      double x, y;
      point((int)(i / numP), (int)(i % numP), x, y);
      const int n = std::snprintf(b, kItemChars, "%.12e", m == 0 ? x : y);
      b[n] = cycle_sep(i, 5);
      return n + 1;
    }));
    g += "\n\n";
  }
  // connectivity: 1-based point ids, three per line; a quadratic element splits into four
  // triangles (corner 1, 2, 3 with their adjacent midpoints, then the midpoint triangle)
  static const int sub[12] = {1, 4, 6, 2, 5, 4, 3, 6, 5, 4, 5, 6};
  const size_t nIds = numP == 6 ? 12 * (size_t)K : 3 * (size_t)K;
  tecConnStart[numP == 6] = g.size();
  g += join(format_parts(nIds, [&](size_t i, char *b) {
    const size_t id = numP == 6 ? 6 * (i / 12) + sub[i % 12] : i + 1;
    return std::snprintf(b, kItemChars, "%zu%c", id, cycle_sep(i, 3));
  }));
  return g;
}

bool VisMesh::write(const double *dataLagr, int numP, const char *varName, const char *baseName, int tLvl,
                    int types, std::string &err) {
  if (K == 0 || !dataLagr || !varName || !baseName || (numP != 1 && numP != 3 && numP != 6) ||
      (types & ~(kVisVtk | kVisTec)) || !types) {
    err = "invalid output arguments";
    return false;
  }
  if (!make_parent_dirs(baseName, err)) return false;
  const int nodesP = numP == 6 ? 6 : 3;
  const size_t nPts = (size_t)K * nodesP;
  // point values in file order (core/visualizeDataLagr.m:209-218)
  auto value = [&](size_t i) {
    const size_t k = i / nodesP, j = i % nodesP;
    if (numP == 1) return dataLagr[k];
    return dataLagr[(size_t)(numP == 6 ? kNode6[j] : (int)j) * K + k];
  };
  const std::string base = std::string(baseName) + "." + std::to_string(tLvl);
  if (types & kVisVtk) {
    const std::string path = base + ".vtu";
    File f(path);
    if (!f.ok()) { err = "cannot open " + path + ": " + std::strerror(errno); return false; }
    f.put("<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" "
          "byte_order=\"LittleEndian\" compressor=\"vtkZLibDataCompressor\">\n  <UnstructuredGrid>\n");
    f.put(vtk_geometry(nodesP));
    f.printf("      <PointData Scalars=\"%s\">\n", varName);
    f.printf("        <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"1\" format=\"ascii\">\n", varName);
    f.parts(format_parts(nPts, [&](size_t i, char *b) { return std::snprintf(b, kItemChars, "          %.9e\n", value(i)); }));
    f.put("        </DataArray>\n      </PointData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n");
    if (!f.close()) { err = "cannot write " + path; return false; }
  }
  if (types & kVisTec) {
    const std::string path = base + ".plt";
    File f(path);
    if (!f.ok()) { err = "cannot open " + path + ": " + std::strerror(errno); return false; }
    const std::string &g = tec_geometry(nodesP);
    const size_t split = tecConnStart[nodesP == 6];
    f.put("TITLE=\"FESTUNG output file\"\n");
    f.printf("VARIABLES=X, Y, \"%s\"\n", varName);
    f.printf("ZONE T=\"Time=%.3e\", N=%zu, E=%zu, ET=TRIANGLE, F=FEBLOCK, SOLUTIONTIME=%.3e\n\n", (double)tLvl, nPts,
             nodesP == 6 ? 4 * (size_t)K : (size_t)K, (double)tLvl);
    f.put(g.data(), split);
    f.parts(format_parts(nPts, [&](size_t i, char *b) {
      const int n = std::snprintf(b, kItemChars, "%.9e", value(i));
      b[n] = cycle_sep(i, 5);
      return n + 1;
    }));
    f.put("\n");
    f.put(g.data() + split, g.size() - split);
    if (!f.close()) { err = "cannot write " + path; return false; }
  }
  return true;
}

}  // namespace dgadv

extern "C" int dgadv_write_lagrange(int32_t numT, int32_t numV, const double *coordV, const int32_t *V0T,
                                    int32_t numP, const double *dataLagr, const char *varName,
                                    const char *fileName, int32_t tLvl, int32_t fileTypes) {
  return dgadv::guarded(nullptr, [&]() -> int {
  if (numT <= 0 || numV <= 0 || !coordV || !V0T || !dataLagr || !varName || !fileName ||
      (numP != 1 && numP != 3 && numP != 6) || !fileTypes || (fileTypes & ~(DGADV_OUT_VTK | DGADV_OUT_TEC)))
    return DGADV_EINVAL;
  std::vector<double> xy(2 * (size_t)numV);
  for (int v = 0; v < numV; ++v) { xy[2 * (size_t)v] = coordV[v]; xy[2 * (size_t)v + 1] = coordV[(size_t)numV + v]; }
  std::vector<int32_t> t(3 * (size_t)numT);
  for (int k = 0; k < numT; ++k)
    for (int n = 0; n < 3; ++n) t[3 * (size_t)k + n] = V0T[(size_t)n * numT + k];
  dgadv::VisMesh mesh;
  std::string err;
  if (!mesh.init(numT, numV, xy.data(), t.data(), err)) return DGADV_EMESH;
  return mesh.write(dataLagr, numP, varName, fileName, tLvl, fileTypes, err) ? DGADV_OK : DGADV_EIO;
  });
}
