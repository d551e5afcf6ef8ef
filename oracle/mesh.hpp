// Oracle (test infrastructure only): restatement of RS's structured mesh
// generator, its topology index lists, hexahedral/quadrilateral geometry and
// the O-method multi-point flux approximation (MPFA-O) that fills the Darcy
// transmissibility lists Connection.MD.
//
// Reference files (under rs/src/no/uib/cipr/rs/):
//   meshgen/structured/CartesianTopology.java:44-80 (build loops)
//   meshgen/structured/CartesianTopology{2D,3D}.java (index formulas)
//   meshgen/structured/NaturalIJKOrdering.java:39-104 (element iteration)
//   geometry/Topology.java:181-247 (LinkedHashSet insertion orders)
//   meshgen/structured/StructuredGeometry{2D,3D}.java, HexCell.java,
//   QuadCell.java, BilinearMap.java:48-102, TrilinearMap.java:41-146
//   geometry/Mesh.java:64-190, geometry/Connection.java:61-107
//   geometry/flux/O_MPFA.java:55-457, geometry/flux/MPFA.java:30-354
#pragma once
#include <vector>

#include "mtj.hpp"

namespace orc {

struct Vec3 {
  double x = 0, y = 0, z = 0;
};

struct MDEntry {
  int element;
  double k;
};

struct Mesh {
  int dim = 3, ni = 0, nj = 0, nk = 0;
  // corner points
  std::vector<Vec3> point;
  std::vector<std::vector<int>> pointInterfaces, pointElements;
  // interfaces
  std::vector<Vec3> inormal, icenter;
  std::vector<double> iarea;
  std::vector<char> iboundary;
  std::vector<std::vector<int>> interfacePoints;
  std::vector<int> interfaceElement, interfaceConnection;
  // elements
  std::vector<Vec3> ecenter;
  std::vector<double> evolume;
  std::vector<std::vector<int>> elementPoints, elementInterfaces;
  // neighbour connections (RS has no non-neighbour connections here)
  std::vector<int> connHereIntf, connThereIntf, connHere, connThere;
  std::vector<double> connMult;
  // rock: permeability tensor xx, yy, zz, xy, xz, yz per element
  std::vector<double> K6;
  // Darcy transmissibilities per connection (Connection.MD order)
  std::vector<std::vector<MDEntry>> MD;

  int numElements() const { return (int)ecenter.size(); }
  int numConnections() const { return (int)connHere.size(); }
  int numPoints() const { return (int)point.size(); }
};

// Builds the structured mesh.  `coords` holds 3 doubles per corner point in
// linear point order (i fastest); pass nullptr to use the untransformed
// tensor grid x0 + sum(dx), y0 + sum(dy), z0 + sum(dz) (dz < 0).
// For dim == 2, nk must be 0 and z is 0.
Mesh build_structured_mesh(int dim, int ni, int nj, int nk, const double* coords, double x0, double y0,
                           double z0, double dx, double dy, double dz);

// O_MPFA.calculateTransmissibilities followed by
// Connection.setDarcyTransmissibilities for every neighbour connection.
void compute_mpfa_o(Mesh& mesh, double continuity);

// L_MPFA.calculateTransmissibilities (geometry/flux/L_MPFA.java:52-74, the
// L-method of L interaction regions with a two-point flux on boundary
// points), 3-D, then Connection.setDarcyTransmissibilities.
void compute_mpfa_l(Mesh& mesh);

// TPFA (geometry/flux/TPFA.java:50-72), including its quirk of using the
// "there" normal conductivity twice in the harmonic mean.
void compute_tpfa(Mesh& mesh);

// LinearSolver.determineSparsityPattern (numerics/LinearSolver.java:111-155)
// followed by CompRowMatrix.construct: the diagonal plus every MD element on
// the rows of both sides of each connection, sorted.
CompRowMatrix pressure_pattern(const Mesh& mesh);

// PotentialCalculator.determineSparsityPattern (numerics/PotentialCalculator.java:347-373):
// as above but without the explicit diagonal.
CompRowMatrix potential_pattern(const Mesh& mesh);

// Cell-wise consistency checks of Mesh.testMesh that concern the data the
// hot path reads (outward unit normals, neighbouring areas and normals).
void test_mesh(const Mesh& mesh);

}  // namespace orc
