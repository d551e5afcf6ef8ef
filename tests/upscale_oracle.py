"""The upscaling pipeline of ressim_gb300.upscale run on the CPU oracle (its
meshes, MPFA, PressureDiscretisation restatement and connection fluxes),
with the same host-side classification: the checker of the GPU pipeline."""
import numpy as np

from oracle import oracle as O
from ressim_gb300 import upscale as U


def here_interface(dim, ni, nj, conn):
    """Interface index (element * faces + face) of each connection's here
    side: the forward face that points to the there element."""
    h, t = conn[:, 0].astype(np.int64), conn[:, 1].astype(np.int64)
    d = t - h
    if dim == 3:
        face = np.where(d == 1, 5, np.where(d == ni, 3, 1))
        return h * 6 + face
    face = np.where(d == 1, 3, 1)
    return h * 4 + face


def lognormal_perm(n, seed, anis=0.1):
    """Per-cell (xx, yy, zz, xy, xz, yz) with log10 kxx ~ N(0, 0.5)."""
    g = np.random.Generator(np.random.PCG64(seed))
    k = 10.0 ** (0.5 * g.standard_normal(n))
    perm = np.zeros((n, 6))
    perm[:, 0] = k
    perm[:, 1] = k
    perm[:, 2] = anis * k
    return perm


def perturbed_coords(dim, ni, nj, nk, seed, amp=0.1):
    """Corner points of a unit-spaced grid (dz = -1), each interior-free
    coordinate moved by U(-amp, amp) in x and y."""
    c = U._tensor_coords(dim, ni, nj, nk, 0.0, 0.0, 0.0, 1.0, 1.0, -1.0)
    g = np.random.Generator(np.random.PCG64(seed))
    c[:, :2] += g.uniform(-amp, amp, (len(c), 2))
    return c


def oracle_upscale(dim, ni, nj, nk, coords, perm, domains, bc_type="Open", method="mpfa"):
    fine = O.Mesh(dim, ni, nj, nk if dim == 3 else 0, coords=coords, perm=perm)
    geo = fine.geometry()
    conn = fine.connections()
    icen = geo["icenter"][here_interface(dim, ni, nj, conn)]
    centers = geo["centers"]
    out = []
    for d in domains:
        elements, bnd, innerc = U.classify(d, centers, conn, icen)
        dims, local, pts, pm = U.domain_box(dim, ni, nj, nk if dim == 3 else 0, coords, perm, elements)
        m = O.Mesh(dim, *dims, coords=pts, perm=pm)
        m.mpfa(tpfa=(method == "tpfa"), lmethod=(method == "lmpfa"))
        lbnd, lin = U.local_numbering(conn, local, m.connections(), bnd, innerc)
        bx, by = U.pressure_bc(d, centers[local], lbnd, bc_type)
        px, itx, _, _ = O.pressure_discretisation(m, bx)
        py, ity, _, _ = O.pressure_discretisation(m, by)
        ux, uy = O.connection_flux(m, px), O.connection_flux(m, py)
        tensor, k21 = U.flow_rate_tensor(d, ux, uy, lin)
        out.append(dict(index=d.index, tensor=tensor, k21=k21, iterations=(itx, ity), px=px, py=py, ux=ux, uy=uy,
                        inner=lin, bc=(bx, by), elements=len(local)))
    return out, dict(centers=centers, conn=conn, icenters=icen)
