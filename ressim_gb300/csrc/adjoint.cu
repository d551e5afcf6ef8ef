// Discrete adjoint: reverse-mode gradients with respect to per-element
// log-permeability through the MPFA-O transmissibilities, with the transposed
// linear systems solved by the same GPU Krylov stack as the forward runs.
// This capability has no counterpart in the reference; the forward problems
// it differentiates are PotentialCalculator's steady potential problem
// (rs/src/no/uib/cipr/rs/numerics/PotentialCalculator.java:319-333) and the
// pressure step of Discretisation (numerics/Discretisation.java:280-919).
#include <vector>

#include "mesh.cuh"

namespace rsg {

namespace {

// mu_c = lambda~_here - lambda~_there with the fixed rows' lambda taken as 0
__global__ void k_conn_difference(int nconn, const int* __restrict__ conn, const double* __restrict__ lam,
                                  const int* __restrict__ fixed_mask, double* __restrict__ mu) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nconn) return;
  const int h = conn[2 * c], t = conn[2 * c + 1];
  const double lh = fixed_mask[h] ? 0.0 : lam[h];
  const double lt = fixed_mask[t] ? 0.0 : lam[t];
  mu[c] = lh - lt;
}

}  // namespace

}  // namespace rsg

using rsg::guarded;

extern "C" {

rsg_status rsg_mesh_transmissibility_adjoint(rsg_mesh* mh, int32_t npairs, const double* conn_weights,
                                             const double* cell_potentials, double* dlogk) {
  if (!mh || npairs < 0 || !dlogk || (npairs > 0 && (!conn_weights || !cell_potentials))) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    rsg::Context& c = *m.ctx;
    const int nel = m.g.nel, ncn = m.g.nconn;
    rsg::DeviceBuffer<double> mu((size_t)std::max(npairs * ncn, 1)), phi((size_t)std::max(npairs * nel, 1)),
        out(nel);
    if (npairs) {
      RSG_CUDA(cudaMemcpyAsync(mu.get(), conn_weights, sizeof(double) * npairs * ncn, cudaMemcpyHostToDevice,
                               c.stream));
      RSG_CUDA(cudaMemcpyAsync(phi.get(), cell_potentials, sizeof(double) * npairs * nel, cudaMemcpyHostToDevice,
                               c.stream));
    }
    rsg::mpfa_adjoint(m, npairs, mu.get(), phi.get(), 1.0, false, out.get());
    RSG_CUDA(cudaMemcpyAsync(dlogk, out.get(), sizeof(double) * nel, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
  });
}

rsg_status rsg_potential_adjoint(rsg_mesh* mh, rsg_solver* solver, rsg_csr* A, int32_t nfixed, const int32_t* fixed,
                                 const double* p, const double* dJdp, double* lambda, double* dJ_dlogk,
                                 rsg_solve_info* info) {
  if (!mh || !solver || !A || !p || !dJdp || !dJ_dlogk || nfixed < 0 || (nfixed > 0 && !fixed)) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    rsg::Context& c = *m.ctx;
    const int n = m.g.nel;
    if (!m.have_md) throw rsg::Error(RSG_BAD_ARG, "transmissibilities have not been computed");
    if (A->m.n != n) throw rsg::Error(RSG_BAD_ARG, "matrix size differs from the mesh's element count");
    std::vector<int> mask(n, 0);
    for (int q = 0; q < nfixed; ++q) {
      if (fixed[q] < 0 || fixed[q] >= n) throw rsg::Error(RSG_BAD_ARG, "fixed row out of range");
      mask[fixed[q]] = 1;
    }
    rsg::CsrTranspose tr;
    tr.update(A->m);
    rsg::DeviceBuffer<double> dp(n), w(n), lam(n), mu(m.g.nconn), out(n);
    rsg::DeviceBuffer<int> dmask(n);
    RSG_CUDA(cudaMemcpyAsync(dp.get(), p, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(w.get(), dJdp, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(dmask.get(), mask.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemsetAsync(lam.get(), 0, sizeof(double) * n, c.stream));
    // the transpose lives only for this call: the solver must not keep it
    struct Forget {
      rsg::Solver& s;
      ~Forget() { rsg::solver_forget_matrix(s); }
    } forget{*solver->s};
    rsg::solver_setup(*solver->s, tr.AT);
    rsg::solver_solve(*solver->s, tr.AT, w.get(), lam.get(), info);
    RSG_LAUNCH(c, "conn_difference", rsg::k_conn_difference, rsg::blocks_for(m.g.nconn, 256), 256, 0, m.g.nconn,
               m.conn.get(), lam.get(), dmask.get(), mu.get());
    rsg::mpfa_adjoint(m, 1, mu.get(), dp.get(), -1.0, false, out.get());
    if (lambda) RSG_CUDA(cudaMemcpyAsync(lambda, lam.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    RSG_CUDA(cudaMemcpyAsync(dJ_dlogk, out.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
  });
}

}  // extern "C"
