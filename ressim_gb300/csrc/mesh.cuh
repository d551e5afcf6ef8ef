// Structured RS mesh on the GPU: closed-form topology, geometry arrays and
// the Darcy transmissibility lists (Connection.MD) produced by MPFA-O.
#pragma once
#include "linalg.cuh"

namespace rsg {

struct Grid {
  int dim, ni, nj, nk;  // nk = 0 in 2D
  int npi, npj, npk;
  int nel, nfacepe, nintf, nconn, npts;
};

struct Mesh {
  Context* ctx = nullptr;
  Grid g;
  DeviceBuffer<double> pts;          // 3 per corner point
  DeviceBuffer<double> perm;         // 6 per element (xx yy zz xy xz yz)
  DeviceBuffer<double> ecenter, evol;   // 3n, n
  DeviceBuffer<double> iarea, icenter, inormal;
  DeviceBuffer<int> conn;            // 2 per connection (here, there)
  // MD lists
  int maxmd = 18;
  int64_t nmd = 0;
  DeviceBuffer<int> md_ptr, md_elem;
  DeviceBuffer<double> md_k;
  std::vector<int> h_md_ptr, h_md_elem, h_conn;
  bool have_md = false;
  double continuity = 1.0;           // continuity point used by the last MPFA-O computation
  bool tpfa = false;                 // MD lists from the two-point approximation
  bool lmethod = false;              // MD lists from the L-method
  // pressure pattern (LinearSolver) and potential pattern (PotentialCalculator)
  std::vector<int> h_prow, h_pcol, h_qrow, h_qcol;
  // per MD entry: CSR position in the here row and in the there row of the
  // pressure pattern; per cell: incident connections (ascending) with side
  DeviceBuffer<int> md_pos_here, md_pos_there, cell_conn_ptr, cell_conn;
  void build_patterns();
};

// d(sum_k mu_k^T T phi_k)/d log K per element (scale times the sum over the
// npairs pairs; mu_k per connection, phi_k per element, all device arrays),
// written to out or added to it.
void mpfa_adjoint(Mesh& m, int npairs, const double* mu, const double* phi, double scale, bool accumulate,
                  double* out);

}  // namespace rsg

struct rsg_mesh {
  rsg::Mesh m;
};
