"""Flow-based permeability upscaling over the GPU pressure solver: the
reference's upscale package (rs/src/no/uib/cipr/rs/upscale/*.java) and the
partition geometry it reads (rs/src/no/uib/cipr/rs/meshgen/partition/*.java).

A structured fine grid is cut into coarse domains (Partition2D); each domain
is its coarse cell grown by a border.  Fine elements are classified by their
centres (Region2D's winding-number test), connections by the centre of their
here interface (closest segment), as PartitionData.partition does.  On each
domain's own mesh (the fine cells of the domain, MPFA-O or TPFA recomputed on
it, as SubdomainMeshGenerator + meshgen/Main do) two pressure problems are
solved on the GPU (rsg_upscale_pressure, PressureDiscretisation.java) with
the linear Dirichlet data of PressureBC, the connection fluxes come from
rsg_mesh_connection_flux, and LocalFlowRateAverage turns the flow through the
inner box's sides into a coarse tensor.

Two choices differ from the reference's file-driven pipeline, neither
changing a formula: a domain's elements must form an index box of the fine
grid (SubdomainMeshGenerator builds a general mesh from any subset; an
index box keeps the element order, i fastest, that the reference's
ascending global numbering gives), and the coarse flow rates are summed in
ascending connection order (the reference iterates a HashSet).
"""
import numpy as np

from . import abi, api
from .api import RSGError

FRONT, RIGHT, BACK, LEFT = "FRONT", "RIGHT", "BACK", "LEFT"
# Orientation.getOrientations2D (meshgen/structured/Orientation.java)
ORIENTATIONS_2D = (FRONT, BACK, LEFT, RIGHT)


class Region2D:
    """A closed rectangular region (meshgen/partition/Region2D.java:12-108):
    oriented segments front p0->p1, right p1->p2, back p2->p3, left p3->p0."""

    def __init__(self, p0, p1, p2, p3):
        p = [np.asarray(q, dtype=np.float64) for q in (p0, p1, p2, p3)]
        self.segments = ((p[0], p[1], FRONT), (p[1], p[2], RIGHT), (p[2], p[3], BACK), (p[3], p[0], LEFT))

    @staticmethod
    def _is_left(v1, v2, pts):
        return (v2[0] - v1[0]) * (pts[:, 1] - v1[1]) - (pts[:, 0] - v1[0]) * (v2[1] - v1[1])

    def contains(self, pts):
        """pointInRegion (:33-59): winding number of the segments around each point."""
        pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
        wn = np.zeros(len(pts), np.int64)
        for v1, v2, _ in self.segments:
            up = (v1[1] <= pts[:, 1]) & (v2[1] > pts[:, 1])
            down = (v1[1] > pts[:, 1]) & (v2[1] <= pts[:, 1])
            il = self._is_left(v1, v2, pts)
            wn += (up & (il > 0.0)).astype(np.int64)
            wn -= (down & (il < 0.0)).astype(np.int64)
        return wn != 0

    @staticmethod
    def _distance(p0, p1, pts):
        """Segment3D.distanceToPoint (meshgen/partition/Segment3D.java:45-66)."""
        v = p1 - p0
        w = pts - p0
        c1 = w @ v
        c2 = v @ v
        d_first = np.sqrt(np.einsum("ij,ij->i", w, w))
        t = pts - p1
        d_second = np.sqrt(np.einsum("ij,ij->i", t, t))
        b = c1 / c2 if c2 != 0 else np.zeros_like(c1)
        pb = p0 + np.outer(b, v)
        t = pts - pb
        d_mid = np.sqrt(np.einsum("ij,ij->i", t, t))
        return np.where(c1 <= 0.0, d_first, np.where(c2 <= c1, d_second, d_mid))

    def closest(self, pts):
        """getClosestSegment (:61-75): the first segment at the smallest
        distance (front, right, back, left order), as orientation names."""
        pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
        d = np.stack([self._distance(a, b, pts) for a, b, _ in self.segments], axis=1)
        names = np.array([s[2] for s in self.segments])
        return names[np.argmin(d, axis=1)]


class Domain2D:
    """A coarse domain (meshgen/partition/Domain2D.java:22-110): the inner
    rectangle p0..p3 and the domain grown by border b on every side."""

    def __init__(self, p0, p1, p2, p3, border, index):
        self.index = index
        self.x0, self.y0 = float(p0[0]), float(p0[1])
        self.x1, self.y1 = float(p2[0]), float(p2[1])
        b = float(border)
        self.inner = Region2D(p0, p1, p2, p3)
        off = lambda p, dx, dy: (p[0] + dx, p[1] + dy, p[2])  # noqa: E731
        self.domain = Region2D(off(p0, -b, -b), off(p1, b, -b), off(p2, b, b), off(p3, -b, b))


def _expanded_points(x0, counts, deltas):
    """ArrayData.getExpanded + getExpandedPoints: each delta repeated its
    count, then the running sum from x0."""
    d = np.repeat(np.asarray(deltas, np.float64), np.asarray(counts, np.int64))
    return np.concatenate([[x0], x0 + np.cumsum(d)])


def partition2d(x0, y0, nx, dx, ny, dy, border):
    """Partition2D (meshgen/partition/Partition2D.java:49-97): the coarse
    domains of a Cartesian partition, numbered i fastest."""
    if len(nx) != len(dx) or len(ny) != len(dy):
        raise ValueError("the number of Nx and Dx (Ny and Dy) values must agree")
    if any(v <= 0 for v in nx) or any(v <= 0 for v in ny) or any(v <= 0 for v in dx) or any(v <= 0 for v in dy):
        raise ValueError("Nx, Ny, Dx and Dy must be positive")
    xs = _expanded_points(float(x0), nx, dx)
    ys = _expanded_points(float(y0), ny, dy)
    out = []
    for j in range(len(ys) - 1):
        for i in range(len(xs) - 1):
            p0 = (xs[i], ys[j], 0.0)
            p1 = (xs[i + 1], ys[j], 0.0)
            p2 = (xs[i + 1], ys[j + 1], 0.0)
            p3 = (xs[i], ys[j + 1], 0.0)
            out.append(Domain2D(p0, p1, p2, p3, border, len(out)))
    return out


def classify(domain, centers, conn, icenters):
    """PartitionData.partition (meshgen/partition/PartitionData.java:285-384)
    for one domain: the elements whose centres lie in the domain, the
    boundary elements per side (in the domain, with a neighbour outside, side
    = closest domain segment to the here interface's centre) and the inner
    connections per side (one end in the inner box, the other in the border
    ring, side = closest inner segment).  Global indices."""
    in_dom = domain.domain.contains(centers[:, :2])
    in_inner = domain.inner.contains(centers[:, :2])
    h, t = conn[:, 0], conn[:, 1]
    bnd = {o: set() for o in ORIENTATIONS_2D}
    innerc = {o: [] for o in ORIENTATIONS_2D}
    one = in_dom[h] != in_dom[t]
    if one.any():
        sides = domain.domain.closest(icenters[one])
        inside = np.where(in_dom[h[one]], h[one], t[one])
        for e, o in zip(inside.tolist(), sides.tolist()):
            bnd[o].add(e)
    both = in_dom[h] & in_dom[t] & (in_inner[h] != in_inner[t])
    if both.any():
        idx = np.flatnonzero(both)
        sides = domain.inner.closest(icenters[idx])
        for c, o in zip(idx.tolist(), sides.tolist()):
            innerc[o].append(c)
    return np.flatnonzero(in_dom), {o: np.array(sorted(v), np.int64) for o, v in bnd.items()}, \
        {o: np.array(v, np.int64) for o, v in innerc.items()}


def pressure_bc(domain, centers, boundary, bc_type="Open"):
    """PressureBC (upscale/PressureBC.java:24-100): Dirichlet values 1 -
    (x - x0) / L1 (x direction) and 1 - (y - y0) / L2 (y direction) on the
    boundary elements of every side ("Open") or of the two sides facing the
    flow ("Closed").  centers: of the elements the maps are keyed by."""
    if bc_type.lower() == "open":
        sx = sy = ORIENTATIONS_2D
    elif bc_type.lower() == "closed":
        sx, sy = (RIGHT, LEFT), (FRONT, BACK)
    else:
        raise ValueError("BoundaryConditions must be of either Open or Closed type")
    L1, L2 = domain.x1 - domain.x0, domain.y1 - domain.y0
    bx, by = {}, {}
    for o in sx:
        for e in boundary[o].tolist():
            bx[e] = 1.0 - (centers[e, 0] - domain.x0) / L1
    for o in sy:
        for e in boundary[o].tolist():
            by[e] = 1 - (centers[e, 1] - domain.y0) / L2
    return bx, by


class PressureDiscretisation:
    """upscale/PressureDiscretisation(mesh, bc) on the GPU: assembles the
    potential matrix with the boundary rows and solves it with GMRES(30) +
    ILU(0) (rsg_upscale_pressure).  bc: {element: pressure}.  Raises
    RSGError with the solver's status if it does not converge (the
    reference throws IterativeSolverNotConvergedException)."""

    def __init__(self, mesh, bc):
        n = mesh.counts()["elements"]
        cells = np.fromiter(bc.keys(), dtype=np.int32, count=len(bc))
        vals = np.fromiter(bc.values(), dtype=np.float64, count=len(bc))
        self.x = np.zeros(n)
        self.info = abi.rsg_solve_info()
        st = api.lib().rsg_upscale_pressure(mesh.h, len(cells), abi.iptr(cells), abi.dptr(vals), abi.dptr(self.x),
                                            self.info)
        if st != 0:
            raise RSGError(st, "PressureDiscretisation")

    def get_solution(self, i=None):
        return self.x if i is None else self.x[i]


def _tensor_coords(dim, ni, nj, nk, x0, y0, z0, dx, dy, dz):
    """Corner points of a tensor grid, linear point order (i fastest)."""
    xs = x0 + dx * np.arange(ni + 1)
    ys = y0 + dy * np.arange(nj + 1)
    zs = z0 + dz * np.arange((nk if dim == 3 else 0) + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def domain_box(dim, ni, nj, nk, coords, perm, elements):
    """A domain's elements as an index box of the fine grid (else RSGError
    UNSUPPORTED): ((ni, nj, nk) of the box, global element ids in the box's
    own order, i fastest, its corner points and its permeabilities)."""
    elements = np.asarray(elements, np.int64)
    i, j, k = elements % ni, (elements // ni) % nj, elements // (ni * nj)
    i0, i1, j0, j1, k0, k1 = i.min(), i.max() + 1, j.min(), j.max() + 1, k.min(), k.max() + 1
    sni, snj, snk = int(i1 - i0), int(j1 - j0), int(k1 - k0)
    if sni * snj * snk != len(elements):
        raise RSGError(abi.UNSUPPORTED, "domain elements do not form an index box of the fine grid")
    kk, jj, ii = np.meshgrid(np.arange(k0, k1), np.arange(j0, j1), np.arange(i0, i1), indexing="ij")
    local = (ii + ni * (jj + nj * kk)).ravel()
    npi, npj = ni + 1, nj + 1
    pk = np.arange(k0, k1 + 1) if dim == 3 else np.arange(1)
    pk_, pj_, pi_ = np.meshgrid(pk, np.arange(j0, j1 + 1), np.arange(i0, i1 + 1), indexing="ij")
    pts = np.ascontiguousarray(coords[(pi_ + npi * (pj_ + npj * pk_)).ravel()])
    return (sni, snj, snk if dim == 3 else 0), local, pts, np.ascontiguousarray(perm[local])


def flow_rate_tensor(domain, ux, uy, inner):
    """LocalFlowRateAverage.postProcessX/YDirection (:86-121) and
    computeAveragedPermeability (:48-83): q11 (RIGHT) and q21 (BACK) of the x
    solve's fluxes, q22 (BACK) and q12 (LEFT) of the y solve's, dp = 1,
    k11 = q11 L1 / (L2 dp), k21 = q21 / dp, k22 = q22 L2 / (L1 dp),
    k12 = q12 / dp.  Returns (Tensor3D(k11, k22, 0, k12, 0, 0) as (xx, yy,
    zz, xy, xz, yz), k21)."""
    L1, L2, dp = domain.x1 - domain.x0, domain.y1 - domain.y0, 1.0
    q11, q21 = ux[inner[RIGHT]].sum(), ux[inner[BACK]].sum()
    q22, q12 = uy[inner[BACK]].sum(), uy[inner[LEFT]].sum()
    k11, k21 = q11 * L1 / (L2 * dp), q21 / dp
    k22, k12 = q22 * L2 / (L1 * dp), q12 / dp
    return np.array([k11, k22, 0.0, k12, 0.0, 0.0]), k21


def local_numbering(conn, local, local_conn, boundary, innerc):
    """The classification's global element and connection ids in the
    domain mesh's numbering (connections matched by their element pair)."""
    g2l = {int(g): q for q, g in enumerate(np.asarray(local).tolist())}
    pair = {(int(a), int(b)): q for q, (a, b) in enumerate(np.asarray(local_conn).tolist())}
    lbnd = {o: np.array([g2l[int(e)] for e in v], np.int64) for o, v in boundary.items()}
    lin = {o: np.array([pair[(g2l[int(conn[c, 0])], g2l[int(conn[c, 1])])] for c in v], np.int64)
           for o, v in innerc.items()}
    return lbnd, lin


class StructuredUpscaler:
    """Upscaling of a structured fine grid (dim 2 or 3, ni x nj x nk cells,
    corner coordinates in linear point order, 6 permeability components per
    cell) over the coarse domains of `partition2d`.  The fine mesh supplies
    the geometry for the classification; each domain gets its own mesh with
    MPFA-O ("mpfa"), TPFA ("tpfa") or L-method ("lmpfa", 3-D) lists."""

    def __init__(self, ctx, dim, ni, nj, nk, perm, coords=None, method="mpfa", continuity=1.0, **tensor):
        self.ctx, self.dim = ctx, dim
        self.ni, self.nj, self.nk = ni, nj, (nk if dim == 3 else 0)
        self.perm = np.ascontiguousarray(perm, dtype=np.float64).reshape(-1, 6)
        if coords is None:
            t = dict(x0=0.0, y0=0.0, z0=0.0, dx=1.0, dy=1.0, dz=-1.0)
            t.update(tensor)
            coords = _tensor_coords(dim, ni, nj, nk, **t)
        self.coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        self.method, self.continuity = method, continuity
        fine = api.Mesh(ctx, dim, ni, nj, self.nk, self.perm, coords=self.coords)
        try:
            self.centers, _ = fine.geometry()
            self.conn = fine.connections()
            self.icenters = fine.interface_centers()
        finally:
            fine.release()

    def domain_mesh(self, elements):
        """The domain's own mesh on the GPU with its transmissibilities.
        Returns (mesh, global element ids in local order)."""
        dims, local, pts, perm = domain_box(self.dim, self.ni, self.nj, self.nk, self.coords, self.perm, elements)
        m = api.Mesh(self.ctx, self.dim, *dims, perm, coords=pts)
        if self.method == "tpfa":
            m.compute_tpfa()
        elif self.method == "lmpfa":
            m.compute_lmpfa()
        else:
            m.compute_mpfa(self.continuity)
        return m, local

    def local_flow_rate_average(self, domains, bc_type="Open"):
        """LocalFlowRateAverage (upscale/LocalFlowRateAverage.java:30-181) for
        every domain: x- and y-direction pressure solves, connection fluxes,
        q11 (RIGHT) and q21 (BACK) of the x solve, q22 (BACK) and q12 (LEFT) of
        the y solve, k11 = q11 L1 / (L2 dp), k21 = q21 / dp, k22 = q22 L2 /
        (L1 dp), k12 = q12 / dp with dp = 1.  Returns one dict per domain:
        tensor (xx, yy, zz, xy, xz, yz) = (k11, k22, 0, k12, 0, 0) as
        Tensor3D(K(0,0), K(1,1), 0, K(0,1), 0, 0), the k21 it does not use, and
        the two solves' iteration counts."""
        out = []
        for d in domains:
            elements, boundary, innerc = classify(d, self.centers, self.conn, self.icenters)
            mesh, local = self.domain_mesh(elements)
            try:
                lbnd, lin = local_numbering(self.conn, local, mesh.connections(), boundary, innerc)
                bx, by = pressure_bc(d, self.centers[local], lbnd, bc_type)
                px = PressureDiscretisation(mesh, bx)
                py = PressureDiscretisation(mesh, by)
                ux = mesh.connection_flux(px.get_solution())
                uy = mesh.connection_flux(py.get_solution())
                tensor, k21 = flow_rate_tensor(d, ux, uy, lin)
                out.append(dict(index=d.index, tensor=tensor, k21=k21,
                                iterations=(px.info.iterations, py.info.iterations), elements=len(local),
                                px=px.get_solution(), py=py.get_solution(), ux=ux, uy=uy, inner=lin, bc=(bx, by)))
            finally:
                mesh.release()
        return out
