// Field post-processing of an edge solution: E at points or tetrahedron
// centroids (src/edge_basis.cpp:131-193, computed on the GPU by
// efgk_edge_field) and the VTK exports built on it (src/io/vtk_export.cpp).
#include <cmath>
#include <fstream>
#include <iomanip>
#include <stdexcept>

#include "device.hpp"
#include "edgefem.hpp"
#include "edgefem_gb300_kernels.h"

namespace edgefem {

namespace {

struct TetArrays {
  std::vector<double> xyz;
  std::vector<int32_t> nodes, edges;
  std::vector<std::uint8_t> signs;
};

TetArrays tet_arrays(const Mesh &mesh) {
  TetArrays a;
  a.xyz.resize(3 * mesh.nodes.size());
  for (std::size_t i = 0; i < mesh.nodes.size(); ++i) {
    a.xyz[3 * i] = mesh.nodes[i].xyz.x;
    a.xyz[3 * i + 1] = mesh.nodes[i].xyz.y;
    a.xyz[3 * i + 2] = mesh.nodes[i].xyz.z;
  }
  const std::size_t T = mesh.tets.size();
  a.nodes.resize(4 * T);
  a.edges.resize(6 * T);
  a.signs.resize(T);
  for (std::size_t t = 0; t < T; ++t) {
    const Element &el = mesh.tets[t];
    std::uint8_t bits = 0;
    for (int k = 0; k < 4; ++k) a.nodes[4 * t + k] = mesh.nodeIndex.at(el.conn[k]);
    for (int k = 0; k < 6; ++k) {
      a.edges[6 * t + k] = el.edges[k];
      if (el.edge_orient[k] < 0) bits |= static_cast<std::uint8_t>(1u << k);
    }
    a.signs[t] = bits;
  }
  return a;
}

std::vector<Vec3C> run_field(const TetArrays &a, const VecC &x, const std::vector<int> *tet_of,
                             const std::vector<Vec3> *pts, std::size_t nq) {
  std::vector<Vec3C> out(nq);
  if (nq == 0) return out;
  CUstream_st *s = stream();
  DevBuf xyz = to_device(a.xyz, s), tn = to_device(a.nodes, s), te = to_device(a.edges, s),
         ts = to_device(a.signs, s), xd = to_device(x, s);
  DevBuf to, pd;
  if (tet_of) to = to_device(*tet_of, s);
  if (pts) {
    std::vector<double> p(3 * pts->size());
    for (std::size_t i = 0; i < pts->size(); ++i)
      p[3 * i] = (*pts)[i].x, p[3 * i + 1] = (*pts)[i].y, p[3 * i + 2] = (*pts)[i].z;
    pd = to_device(p, s);
  }
  DevBuf E(nq * 3 * sizeof(cplx));
  cuda_check(efgk_edge_field(static_cast<int64_t>(nq), xyz.as<double>(), tn.as<int32_t>(), ts.as<std::uint8_t>(),
                             te.as<int32_t>(), tet_of ? to.as<int32_t>() : nullptr,
                             pts ? pd.as<double>() : nullptr, xd.as<double>(), E.as<double>(), s),
             "efgk_edge_field");
  E.download(out.data(), nq * 3 * sizeof(cplx), s);
  return out;
}

void check_solution(const Mesh &mesh, const VecC &x) {
  if (x.size() != mesh.edges.size())
    throw std::invalid_argument("solution has " + std::to_string(x.size()) + " entries, the mesh " +
                                std::to_string(mesh.edges.size()) + " edges");
}

double norm3(const Vec3C &e) { return std::sqrt(std::norm(e[0]) + std::norm(e[1]) + std::norm(e[2])); }

// Phase of the largest-magnitude component (the first one on ties).
double dominant_phase(const Vec3C &e) {
  double best = 0.0, ph = 0.0;
  for (int j = 0; j < 3; ++j) {
    const double m = std::abs(e[j]);
    if (m > best) best = m, ph = std::arg(e[j]);
  }
  return ph;
}

}  // namespace

std::array<double, 4> compute_barycentric(const std::array<Vec3, 4> &v, const Vec3 &p) {
  // src/edge_basis.cpp:131-151: lambda_0..2 = B^-1 (p - v3), lambda_3 = 1 - sum.
  // Host arithmetic on one tetrahedron (a 3x3 solve by Cramer's rule).
  const double c[3][3] = {{v[0].x - v[3].x, v[1].x - v[3].x, v[2].x - v[3].x},
                          {v[0].y - v[3].y, v[1].y - v[3].y, v[2].y - v[3].y},
                          {v[0].z - v[3].z, v[1].z - v[3].z, v[2].z - v[3].z}};
  const double r[3] = {p.x - v[3].x, p.y - v[3].y, p.z - v[3].z};
  auto det3 = [](const double m[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  };
  const double d = det3(c);
  std::array<double, 4> lam{};
  for (int k = 0; k < 3; ++k) {
    double m[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) m[i][j] = j == k ? r[i] : c[i][j];
    lam[k] = det3(m) / d;
  }
  lam[3] = 1.0 - lam[0] - lam[1] - lam[2];
  return lam;
}

Vec3C evaluate_edge_field(const std::array<Vec3, 4> &vertices, const std::array<int, 6> &edge_orient,
                          const std::array<cplx, 6> &edge_dofs, const Vec3 &point) {
  // src/edge_basis.cpp:162-193, one point, through the same GPU kernel as the
  // bulk evaluation (a one-tetrahedron mesh whose edges are its local edges).
  TetArrays a;
  for (const Vec3 &v : vertices) a.xyz.insert(a.xyz.end(), {v.x, v.y, v.z});
  a.nodes = {0, 1, 2, 3};
  a.edges = {0, 1, 2, 3, 4, 5};
  std::uint8_t bits = 0;
  for (int k = 0; k < 6; ++k)
    if (edge_orient[k] < 0) bits |= static_cast<std::uint8_t>(1u << k);
  a.signs = {bits};
  const std::vector<int> tet_of{0};
  const std::vector<Vec3> pts{point};
  return run_field(a, VecC(edge_dofs.begin(), edge_dofs.end()), &tet_of, &pts, 1)[0];
}

std::vector<Vec3C> evaluate_field_at_points(const Mesh &mesh, const VecC &solution, const std::vector<int> &tet_of,
                                            const std::vector<Vec3> &points) {
  check_solution(mesh, solution);
  if (tet_of.size() != points.size()) throw std::invalid_argument("tet_of and points differ in length");
  for (int t : tet_of)
    if (t < 0 || static_cast<std::size_t>(t) >= mesh.tets.size())
      throw std::invalid_argument("tet index out of range: " + std::to_string(t));
  return run_field(tet_arrays(mesh), solution, &tet_of, &points, points.size());
}

std::vector<Vec3C> evaluate_field_at_centroids(const Mesh &mesh, const VecC &solution) {
  check_solution(mesh, solution);
  return run_field(tet_arrays(mesh), solution, nullptr, nullptr, mesh.tets.size());
}

void export_fields_vtk(const Mesh &mesh, const VecC &solution, const std::string &filename,
                       const VTKExportOptions &options) {
  // src/io/vtk_export.cpp:44-200: XML unstructured grid, fields at the tet
  // centroids as cell data.  The reference's stream turns to scientific
  // notation with 8 digits at its first point coordinate and stays so.
  const std::vector<Vec3C> E = evaluate_field_at_centroids(mesh, solution);
  std::ofstream f(filename);
  if (!f.is_open()) throw std::runtime_error("Cannot open file for VTK export: " + filename);
  const std::size_t T = mesh.tets.size(), NN = mesh.nodes.size();
  f << "<?xml version=\"1.0\"?>\n";
  f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  f << "  <UnstructuredGrid>\n";
  f << "    <Piece NumberOfPoints=\"" << NN << "\" NumberOfCells=\"" << T << "\">\n";
  f << "      <Points>\n";
  f << "        <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
  for (const Node &n : mesh.nodes)
    f << "          " << std::scientific << std::setprecision(8) << n.xyz.x << " " << n.xyz.y << " " << n.xyz.z
      << "\n";
  f << "        </DataArray>\n";
  f << "      </Points>\n";
  f << "      <Cells>\n";
  f << "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n";
  for (const Element &el : mesh.tets) {
    f << "          ";
    for (int k = 0; k < 4; ++k) f << mesh.nodeIndex.at(el.conn[k]) << " ";
    f << "\n";
  }
  f << "        </DataArray>\n";
  f << "        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
  f << "          ";
  for (std::size_t i = 1; i <= T; ++i) {
    f << (i * 4) << " ";
    if (i % 20 == 0) f << "\n          ";
  }
  f << "\n        </DataArray>\n";
  f << "        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
  f << "          ";
  for (std::size_t i = 0; i < T; ++i) {
    f << "10 ";
    if ((i + 1) % 30 == 0) f << "\n          ";
  }
  f << "\n        </DataArray>\n";
  f << "      </Cells>\n";
  f << "      <CellData>\n";
  auto vec_array = [&](const char *name, bool imag) {
    f << "        <DataArray type=\"Float64\" Name=\"" << name << "\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (const Vec3C &e : E) {
      f << "          " << std::scientific;
      for (int j = 0; j < 3; ++j) f << (imag ? e[j].imag() : e[j].real()) << (j < 2 ? " " : "\n");
    }
    f << "        </DataArray>\n";
  };
  if (options.export_magnitude) {
    f << "        <DataArray type=\"Float64\" Name=\"E_magnitude\" format=\"ascii\">\n";
    for (const Vec3C &e : E) f << "          " << std::scientific << norm3(e) << "\n";
    f << "        </DataArray>\n";
  }
  if (options.export_phase) {
    f << "        <DataArray type=\"Float64\" Name=\"E_phase_rad\" format=\"ascii\">\n";
    for (const Vec3C &e : E) f << "          " << std::scientific << dominant_phase(e) << "\n";
    f << "        </DataArray>\n";
  }
  if (options.export_real) vec_array("E_real", false);
  if (options.export_imag) vec_array("E_imag", true);
  if (options.export_vector) vec_array("E_vector", false);
  f << "        <DataArray type=\"Int32\" Name=\"PhysicalTag\" format=\"ascii\">\n";
  f << "          ";
  for (std::size_t i = 0; i < T; ++i) {
    f << mesh.tets[i].phys << " ";
    if ((i + 1) % 20 == 0) f << "\n          ";
  }
  f << "\n        </DataArray>\n";
  f << "      </CellData>\n";
  f << "    </Piece>\n";
  f << "  </UnstructuredGrid>\n";
  f << "</VTKFile>\n";
}

void export_fields_vtk_legacy(const Mesh &mesh, const VecC &solution, const std::string &filename,
                              const VTKExportOptions &options) {
  // src/io/vtk_export.cpp:202-272: legacy ASCII VTK, magnitude and real
  // vector at the centroids.
  const std::vector<Vec3C> E = evaluate_field_at_centroids(mesh, solution);
  std::ofstream f(filename);
  if (!f.is_open()) throw std::runtime_error("Cannot open file for VTK export: " + filename);
  const std::size_t T = mesh.tets.size(), NN = mesh.nodes.size();
  f << "# vtk DataFile Version 3.0\nEdgeFEM Field Export\nASCII\nDATASET UNSTRUCTURED_GRID\n";
  f << "POINTS " << NN << " double\n";
  for (const Node &n : mesh.nodes)
    f << std::scientific << std::setprecision(8) << n.xyz.x << " " << n.xyz.y << " " << n.xyz.z << "\n";
  f << "CELLS " << T << " " << (T * 5) << "\n";
  for (const Element &el : mesh.tets) {
    f << "4";
    for (int k = 0; k < 4; ++k) f << " " << mesh.nodeIndex.at(el.conn[k]);
    f << "\n";
  }
  f << "CELL_TYPES " << T << "\n";
  for (std::size_t i = 0; i < T; ++i) f << "10\n";
  f << "CELL_DATA " << T << "\n";
  if (options.export_magnitude) {
    f << "SCALARS E_magnitude double 1\nLOOKUP_TABLE default\n";
    for (const Vec3C &e : E) f << std::scientific << norm3(e) << "\n";
  }
  if (options.export_vector) {
    f << "VECTORS E_vector double\n";
    for (const Vec3C &e : E)
      f << std::scientific << e[0].real() << " " << e[1].real() << " " << e[2].real() << "\n";
  }
}

}  // namespace edgefem
