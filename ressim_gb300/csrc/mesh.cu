// Structured mesh geometry and MPFA-O transmissibilities on the GPU.
//
// Topology follows RS's StructuredMeshGenerator numbering in closed form
// (rs/src/no/uib/cipr/rs/meshgen/structured/CartesianTopology3D.java:41-286,
// CartesianTopology2D.java:38-228, NaturalIJKOrdering.java:57-104,
// geometry/Topology.java:207-247): the interface and element lists of a
// corner point come in the order RS's LinkedHashSets produce them, which
// fixes the local numbering of each interaction region and therefore the
// pivoting of its LU factorisation.
//
// Geometry restates HexCell/QuadCell/BilinearMap/TrilinearMap; MPFA-O
// restates geometry/flux/O_MPFA.java:55-457 and MPFA.java:43-354 with the
// dense LU of netlib dgesv (dgetf2 + dgetrs) and dgemm, one thread per corner
// point.  Everything is compiled without fused multiply-add so each product
// and sum rounds as the Java code does.
#include <algorithm>
#include <numeric>

#include "mesh.cuh"

namespace rsg {

namespace {

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 vmul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 vcross(V3 a, V3 v) {
  return {a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x};
}
__device__ __forceinline__ double vdot(V3 a, V3 v) { return a.x * v.x + a.y * v.y + a.z * v.z; }
__device__ __forceinline__ double vnorm(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ double vcomp(V3 a, int c) { return c == 1 ? a.x : (c == 2 ? a.y : a.z); }
__device__ __forceinline__ V3 ld3(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ void st3(double* p, int64_t i, V3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

__host__ __device__ __forceinline__ int EL(const Grid& g, int i, int j, int k) { return i + j * g.ni + k * g.ni * g.nj; }
__host__ __device__ __forceinline__ int PT(const Grid& g, int i, int j, int k) {
  return i + j * g.npi + k * g.npi * g.npj;
}
__host__ __device__ __forceinline__ bool valid(const Grid& g, int i, int j, int k) {
  if (i < 0 || i > g.ni - 1 || j < 0 || j > g.nj - 1) return false;
  if (g.dim == 3) return k >= 0 && k <= g.nk - 1;
  return k == 0;
}
__host__ __device__ __forceinline__ void el_ijk(const Grid& g, int e, int& i, int& j, int& k) {
  i = e % g.ni;
  j = (e / g.ni) % g.nj;
  k = e / (g.ni * g.nj);
}

// Neighbour across face o of element (i,j,k); returns false on the boundary.
__host__ __device__ bool face_neighbour(const Grid& g, int i, int j, int k, int o, int& ne, int& no) {
  int di = 0, dj = 0, dk = 0, opp;
  if (g.dim == 3) {
    switch (o) {
      case 0: dk = -1; opp = 1; break;
      case 1: dk = 1; opp = 0; break;
      case 2: dj = -1; opp = 3; break;
      case 3: dj = 1; opp = 2; break;
      case 4: di = -1; opp = 5; break;
      default: di = 1; opp = 4; break;
    }
  } else {
    switch (o) {
      case 0: dj = -1; opp = 1; break;
      case 1: dj = 1; opp = 0; break;
      case 2: di = -1; opp = 3; break;
      default: di = 1; opp = 2; break;
    }
  }
  if (!valid(g, i + di, j + dj, k + dk)) return false;
  ne = EL(g, i + di, j + dj, k + dk);
  no = opp;
  return true;
}

// Connection index of an interior face (CartesianTopology3D.getLinearConnection :104-130,
// CartesianTopology2D :103-119); forward faces (odd o) are the "here" side.
__host__ __device__ int face_connection(const Grid& g, int i, int j, int k, int o) {
  if (!(o & 1)) {
    int ne, no;
    face_neighbour(g, i, j, k, o, ne, no);
    int a, b, c;
    el_ijk(g, ne, a, b, c);
    i = a;
    j = b;
    k = c;
    o = no;
  }
  const int ni = g.ni, nj = g.nj, nk = g.nk;
  if (g.dim == 3) {
    if (o == 1) return i + j * ni + k * ni * nj;
    if (o == 3) return i + j * ni + k * ni * (nj - 1) + ni * nj * (nk - 1);
    return i + j * (ni - 1) + k * (ni - 1) * nj + ni * (nj - 1) * nk + ni * nj * (nk - 1);
  }
  if (o == 1) return i + j * ni;
  return i + j * (ni - 1) + ni * (nj - 1);
}

__host__ __device__ void elem_points(const Grid& g, int i, int j, int k, int* cp) {
  if (g.dim == 3) {
    cp[0] = PT(g, i, j, k);
    cp[1] = cp[0] + 1;
    cp[2] = PT(g, i, j + 1, k) + 1;
    cp[3] = cp[2] - 1;
    cp[4] = PT(g, i, j, k + 1);
    cp[5] = cp[4] + 1;
    cp[6] = PT(g, i, j + 1, k + 1) + 1;
    cp[7] = cp[6] - 1;
  } else {
    cp[0] = PT(g, i, j, 0);
    cp[1] = cp[0] + 1;
    cp[2] = PT(g, i, j + 1, 0) + 1;
    cp[3] = cp[2] - 1;
  }
}

// getInterfacePoints (3D :267-286, 2D :213-228)
__host__ __device__ int face_points(const Grid& g, const int* cp, int o, int* ip) {
  if (g.dim == 3) {
    const int t[6][4] = {{0, 1, 2, 3}, {7, 6, 5, 4}, {4, 5, 1, 0}, {6, 7, 3, 2}, {7, 4, 0, 3}, {5, 6, 2, 1}};
    for (int a = 0; a < 4; ++a) ip[a] = cp[t[o][a]];
    return 4;
  }
  const int t2[4][2] = {{1, 0}, {3, 2}, {0, 3}, {2, 1}};
  ip[0] = cp[t2[o][0]];
  ip[1] = cp[t2[o][1]];
  return 2;
}

// Corner point topology: elements in NaturalIJKOrdering iteration order,
// interfaces grouped by element in orientation order.
struct PointTopo {
  int ne, nf, nconn;
  int el[8];
  int eijk[8][3];
  int face[24];     // global interface index
  int fel[24];      // position of the owning element in el[]
  int fo[24];       // orientation
  int lidx[24];     // local connection index (intfMap)
  char boundary[24];
};

__device__ void point_topology(const Grid& g, int p, PointTopo& t) {
  const int pi = p % g.npi, pj = (p / g.npi) % g.npj, pk = p / (g.npi * g.npj);
  t.ne = 0;
  t.nf = 0;
  const int nfe = g.dim == 3 ? 6 : 4;
  for (int di = -1; di <= 0; ++di)
    for (int dj = -1; dj <= 0; ++dj)
      for (int dk = (g.dim == 3 ? -1 : 0); dk <= 0; ++dk) {
        int i = pi + di, j = pj + dj, k = pk + dk;
        if (!valid(g, i, j, k)) continue;
        int a = t.ne++;
        int e = EL(g, i, j, k);
        t.el[a] = e;
        t.eijk[a][0] = i;
        t.eijk[a][1] = j;
        t.eijk[a][2] = k;
        int os[3], no = 0;
        if (g.dim == 3) os[no++] = (pk == k) ? 0 : 1;
        if (g.dim == 3) os[no++] = (pj == j) ? 2 : 3;
        else os[no++] = (pj == j) ? 0 : 1;
        if (g.dim == 3) os[no++] = (pi == i) ? 4 : 5;
        else os[no++] = (pi == i) ? 2 : 3;
        for (int q = 0; q < no; ++q) {
          int f = t.nf++;
          t.face[f] = e * nfe + os[q];
          t.fel[f] = a;
          t.fo[f] = os[q];
          int ne_, no_;
          t.boundary[f] = !face_neighbour(g, i, j, k, os[q], ne_, no_);
        }
      }
  // createLocalInterfaceMap (O_MPFA.java:142-153)
  t.nconn = 0;
  for (int f = 0; f < t.nf; ++f) {
    int idx = -1;
    if (!t.boundary[f]) {
      int a = t.fel[f];
      int ne_, no_;
      face_neighbour(g, t.eijk[a][0], t.eijk[a][1], t.eijk[a][2], t.fo[f], ne_, no_);
      int nb = ne_ * nfe + no_;
      for (int q = 0; q < f; ++q)
        if (t.face[q] == nb) {
          idx = t.lidx[q];
          break;
        }
    }
    t.lidx[f] = idx >= 0 ? idx : t.nconn++;
  }
}

// ---------------------------------------------------------- geometry ----
struct Bilin {
  V3 p0, p1, p2, p3, normal;
  double area;
};
__device__ Bilin bilinear(V3 a, V3 b, V3 c, V3 d) {
  // BilinearMap.computeAreaNormal (:79-102)
  Bilin m{a, b, c, d, {0, 0, 0}, 0};
  V3 x1 = a, x2 = b, x3 = c, x4 = d;
  V3 A = vcross(vsub(x2, x1), vsub(x3, x1));
  V3 B = vcross(vsub(x2, x1), vsub(x4, x2));
  V3 C = vcross(vsub(x4, x3), vsub(x3, x1));
  V3 D = vcross(vsub(x4, x3), vsub(x4, x2));
  V3 n = vmul(vadd(A, vadd(B, vadd(C, D))), .25);
  double length = vnorm(n);
  m.area = length;
  m.normal = (length < 1.0e-9) ? V3{0, 0, 0} : vmul(n, 1.0 / length);
  return m;
}
__device__ V3 bilin_point(const Bilin& m, double a, double b) {
  double k0 = (1 - a) * (1 - b), k1 = a * (1 - b), k2 = (1 - a) * b, k3 = a * b;
  return {k0 * m.p0.x + k1 * m.p1.x + k2 * m.p2.x + k3 * m.p3.x, k0 * m.p0.y + k1 * m.p1.y + k2 * m.p2.y + k3 * m.p3.y,
          k0 * m.p0.z + k1 * m.p1.z + k2 * m.p2.z + k3 * m.p3.z};
}

__device__ double tri_coord(const V3* x, double a, double b, double c, int d) {
  // TrilinearMap.getPoint (:41-64); x[0..7] = x1..x8
  double v1 = vcomp(x[0], d), v2 = vcomp(x[1], d), v3 = vcomp(x[2], d), v4 = vcomp(x[3], d);
  double v5 = vcomp(x[4], d), v6 = vcomp(x[5], d), v7 = vcomp(x[6], d), v8 = vcomp(x[7], d);
  return c * (b * (a * v4 + (1 - a) * v3) + (1 - b) * (a * v2 + (1 - a) * v1)) +
         (1 - c) * (b * (a * v8 + (1 - a) * v7) + (1 - b) * (a * v6 + (1 - a) * v5));
}

__device__ double tri_volume(const V3* x) {
  // TrilinearMap.getVolume (:76-146) including the running sign flip
  V3 r1 = x[2], r2 = x[3], r3 = x[0], r4 = x[1], r5 = x[6], r6 = x[7], r7 = x[4], r8 = x[5];
  V3 C[2][2][2];
  C[0][0][0] = r1;
  C[1][0][0] = vsub(r2, r1);
  C[0][1][0] = vsub(r3, r1);
  C[0][0][1] = vsub(r5, r1);
  C[1][1][0] = vsub(vadd(r4, r1), vadd(r3, r2));
  C[0][1][1] = vsub(vadd(r7, r1), vadd(r5, r3));
  C[1][0][1] = vsub(vadd(r6, r1), vadd(r5, r2));
  C[1][1][1] = vsub(vadd(r8, vadd(r5, vadd(r3, r2))), vadd(r7, vadd(r6, vadd(r4, r1))));
  const int perm[6][3] = {{1, 2, 3}, {1, 3, 2}, {2, 1, 3}, {2, 3, 1}, {3, 1, 2}, {3, 2, 1}};
  double volume = 0.0;
  for (int q = 0; q < 6; ++q) {
    const int a = perm[q][0], b = perm[q][1], c = perm[q][2];
    for (int pb = 0; pb <= 1; pb++)
      for (int pc = 0; pc <= 1; pc++)
        for (int qa = 0; qa <= 1; qa++)
          for (int qc = 0; qc <= 1; qc++)
            for (int ra = 0; ra <= 1; ra++)
              for (int rb = 0; rb <= 1; rb++) {
                double e = vcomp(C[1][pb][pc], a) * vcomp(C[qa][1][qc], b) * vcomp(C[ra][rb][1], c);
                double d = (double)((qa + ra + 1) * (pb + rb + 1) * (pc + qc + 1));
                volume += e / d;
              }
    int s = 0;
    for (int i = 0; i < 3; i++)
      for (int l = 0; l < i; l++)
        if (perm[q][l] > i) s += 1;
    volume = ((s & 1) ? -1.0 : 1.0) * volume;
  }
  return volume;
}

__global__ void k_geometry(Grid g, const double* __restrict__ pts, double* ecenter, double* evol, double* iarea,
                           double* icenter, double* inormal) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel) return;
  int i, j, k;
  el_ijk(g, e, i, j, k);
  int cp[8];
  elem_points(g, i, j, k, cp);
  if (g.dim == 3) {
    // HexCell (:26-51): right-hand ordering -> volume/area ordering
    V3 x[8] = {ld3(pts, cp[0]), ld3(pts, cp[1]), ld3(pts, cp[3]), ld3(pts, cp[2]),
               ld3(pts, cp[4]), ld3(pts, cp[5]), ld3(pts, cp[7]), ld3(pts, cp[6])};
    evol[e] = tri_volume(x);
    st3(ecenter, e, V3{tri_coord(x, 0.5, 0.5, 0.5, 1), tri_coord(x, 0.5, 0.5, 0.5, 2), tri_coord(x, 0.5, 0.5, 0.5, 3)});
    const int fidx[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 2, 4, 6}, {1, 3, 5, 7}};
    const double scale[6] = {1.0, -1.0, -1.0, 1.0, 1.0, -1.0};
    for (int o = 0; o < 6; ++o) {
      Bilin b = bilinear(x[fidx[o][0]], x[fidx[o][1]], x[fidx[o][2]], x[fidx[o][3]]);
      int64_t f = (int64_t)e * 6 + o;
      iarea[f] = b.area;
      st3(icenter, f, bilin_point(b, .5, .5));
      st3(inormal, f, vmul(b.normal, scale[o]));
    }
  } else {
    // QuadCell (:27-95)
    V3 p0 = ld3(pts, cp[0]), p1 = ld3(pts, cp[1]), p2 = ld3(pts, cp[2]), p3 = ld3(pts, cp[3]);
    Bilin b = bilinear(p0, p1, p3, p2);
    st3(ecenter, e, bilin_point(b, .5, .5));
    evol[e] = b.area;
    V3 ends[4][2] = {{p0, p1}, {p2, p3}, {p3, p0}, {p1, p2}};
    for (int o = 0; o < 4; ++o) {
      V3 a = ends[o][0], c = ends[o][1];
      double x_ = c.x - a.x, y_ = c.y - a.y;
      V3 n{y_, -x_, 0};
      n = vmul(n, 1 / vnorm(n));
      int64_t f = (int64_t)e * 4 + o;
      st3(inormal, f, n);
      iarea[f] = vnorm(vsub(c, a));
      st3(icenter, f, vmul(vadd(a, c), 0.5));
    }
  }
}

__global__ void k_connections(Grid g, int* conn) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel) return;
  int i, j, k;
  el_ijk(g, e, i, j, k);
  const int nfe = g.dim == 3 ? 6 : 4;
  for (int o = 1; o < nfe; o += 2) {
    int ne, no;
    if (!face_neighbour(g, i, j, k, o, ne, no)) continue;
    int c = face_connection(g, i, j, k, o);
    conn[2 * c] = e;
    conn[2 * c + 1] = ne;
  }
}

// ------------------------------------------------------------ dense LU ----
// netlib dgesv: dgetf2 (idamax pivot, reciprocal scaling, dger update) then
// dgetrs (dlaswp, unit-lower and non-unit-upper dtrsm with zero skips).
__device__ int d_dgesv(int n, int nrhs, double* A, int lda, double* B, int ldb) {
  int ipiv[12];
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = fabs(A[j + j * lda]);
    for (int i = j + 1; i < n; ++i) {
      double a = fabs(A[i + j * lda]);
      if (a > amax) {
        amax = a;
        jp = i;
      }
    }
    ipiv[j] = jp;
    if (A[jp + j * lda] != 0.0) {
      if (jp != j)
        for (int c = 0; c < n; ++c) {
          double t = A[j + c * lda];
          A[j + c * lda] = A[jp + c * lda];
          A[jp + c * lda] = t;
        }
      if (j < n - 1) {
        double rp = 1.0 / A[j + j * lda];
        for (int i = j + 1; i < n; ++i) A[i + j * lda] *= rp;
      }
    } else if (info == 0)
      info = j + 1;
    if (j < n - 1)
      for (int c = j + 1; c < n; ++c) {
        double yv = A[j + c * lda];
        if (yv != 0.0) {
          double temp = -1.0 * yv;
          for (int i = j + 1; i < n; ++i) A[i + c * lda] += A[i + j * lda] * temp;
        }
      }
  }
  if (info) return info;
  for (int j = 0; j < n; ++j)
    if (ipiv[j] != j)
      for (int c = 0; c < nrhs; ++c) {
        double t = B[j + c * ldb];
        B[j + c * ldb] = B[ipiv[j] + c * ldb];
        B[ipiv[j] + c * ldb] = t;
      }
  for (int c = 0; c < nrhs; ++c) {
    double* bc = B + c * ldb;
    for (int k = 0; k < n; ++k)
      if (bc[k] != 0.0)
        for (int i = k + 1; i < n; ++i) bc[i] -= bc[k] * A[i + k * lda];
    for (int k = n - 1; k >= 0; --k)
      if (bc[k] != 0.0) {
        bc[k] = bc[k] / A[k + k * lda];
        for (int i = 0; i < k; ++i) bc[i] -= bc[k] * A[i + k * lda];
      }
  }
  return 0;
}

constexpr int TLD = 12;  // leading dimension of the per-point T store
constexpr int TSZ = 96;  // 12 local connections x 8 elements

// MPFA.calculateNormalArea (:314-354) for the face at position f of point p
__device__ V3 normal_area(const Grid& g, const PointTopo& t, int f, int p, const double* pts, const double* inormal,
                          const double* iarea) {
  const int face = t.face[f];
  if (g.dim == 2) return vmul(ld3(inormal, face), -iarea[face] / 2);
  int cp[8], ip[4];
  const int a = t.fel[f];
  elem_points(g, t.eijk[a][0], t.eijk[a][1], t.eijk[a][2], cp);
  face_points(g, cp, t.fo[f], ip);
  int i = 0;
  for (int q = 0; q < 4; ++q)
    if (ip[q] == p) {
      i = q;
      break;
    }
  V3 x1 = ld3(pts, ip[i]);
  V3 x2 = ld3(pts, ip[i == 0 ? 3 : (i - 1) % 4]);
  V3 x3 = ld3(pts, ip[(i + 1) % 4]);
  V3 x4 = ld3(pts, ip[(i + 2) % 4]);
  V3 v21 = vsub(x2, x1), v31 = vsub(x3, x1), v42 = vsub(x4, x2), v43 = vsub(x4, x3);
  V3 n1 = vmul(vcross(v21, v31), 9);
  V3 n2 = vmul(vcross(v21, v42), 3);
  V3 n3 = vmul(vcross(v43, v31), 3);
  V3 n4 = vcross(v43, v42);
  return vmul(vadd(vadd(vadd(n1, n2), n3), n4), 1. / 64.);
}

// OmethodInteractionRegion.calculateT (O_MPFA.java:193-239) per corner point;
// stores T = C (A\B) - D (column major, ld 12) and flags singular regions.
__global__ void __launch_bounds__(128) k_mpfa_point(Grid g, const double* __restrict__ pts,
                                                    const double* __restrict__ perm, const double* __restrict__ ecenter,
                                                    const double* __restrict__ icenter,
                                                    const double* __restrict__ inormal,
                                                    const double* __restrict__ iarea, double continuity,
                                                    double* __restrict__ Tstore, int* flag) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  PointTopo t;
  point_topology(g, p, t);
  const int nc = t.nconn, ne = t.ne;
  double A[TLD * TLD], B[TLD * 8], C[TLD * TLD], D[TLD * 8];
  for (int q = 0; q < TLD * TLD; ++q) A[q] = C[q] = 0;
  for (int q = 0; q < TLD * 8; ++q) B[q] = D[q] = 0;
  const V3 corner = ld3(pts, p);
  const int per = g.dim == 3 ? 3 : 2;  // interfaces of one element at the point
  for (int a = 0; a < ne; ++a) {
    const int el = t.el[a];
    const int f0 = a * per;  // faces of element a occupy positions f0..f0+per-1
    const int n = per + 1;
    double Ab[16], Psi[16];
    for (int q = 0; q < 16; ++q) Ab[q] = Psi[q] = 0;
    V3 ec = ld3(ecenter, el);
    Ab[0] = 1;
    Ab[0 + 1 * n] = ec.x;
    Ab[0 + 2 * n] = ec.y;
    if (n == 4) Ab[0 + 3 * n] = ec.z;
    for (int i = 0; i < per; ++i) {
      V3 cp = ld3(icenter, t.face[f0 + i]);
      if (continuity != 1)
        cp = {(cp.x - corner.x) * continuity + corner.x, (cp.y - corner.y) * continuity + corner.y,
              (cp.z - corner.z) * continuity + corner.z};
      Ab[(i + 1)] = 1;
      Ab[(i + 1) + 1 * n] = cp.x;
      Ab[(i + 1) + 2 * n] = cp.y;
      if (n == 4) Ab[(i + 1) + 3 * n] = cp.z;
    }
    for (int i = 0; i < n; ++i) Psi[i + i * n] = 1;
    if (d_dgesv(n, n, Ab, n, Psi, n) != 0) {
      atomicCAS(flag, 0, 1);
      return;
    }
    V3 grad[4];
    for (int i = 0; i < n; ++i) grad[i] = {Psi[1 + i * n], Psi[2 + i * n], n == 4 ? Psi[3 + i * n] : 0.0};
    const double* K = perm + 6 * (int64_t)el;
    const double kxx = K[0], kyy = K[1], kzz = K[2], kxy = K[3], kxz = K[4], kyz = K[5];
    V3 Kn[3];
    for (int i = 0; i < per; ++i) {
      V3 v = normal_area(g, t, f0 + i, p, pts, inormal, iarea);
      Kn[i] = {kxx * v.x + kxy * v.y + kxz * v.z, kxy * v.x + kyy * v.y + kyz * v.z, kxz * v.x + kyz * v.y + kzz * v.z};
    }
    // assembleElementContribution (O_MPFA.java:422-457)
    for (int i = 0; i < per; ++i) {
      double f = vdot(Kn[i], grad[0]);
      const int fi = f0 + i;
      const int is = t.lidx[fi];
      const bool isHere = t.boundary[fi] ? true : (t.fo[fi] & 1);
      B[is + a * TLD] += -f;
      if (isHere) D[is + a * TLD] += -f;
      for (int j = 1; j < per + 1; j++) {
        f = vdot(Kn[i], grad[j]);
        const int js = t.lidx[f0 + j - 1];
        A[is + js * TLD] += f;
        if (isHere) C[is + js * TLD] += f;
      }
    }
  }
  // T = C * (A \ B) - D (MPFA.java:43-54)
  if (d_dgesv(nc, ne, A, TLD, B, TLD) != 0) {
    atomicCAS(flag, 0, 2);
    return;
  }
  double* T = Tstore + (int64_t)p * TSZ;
  for (int j = 0; j < ne; ++j)
    for (int i = 0; i < nc; ++i) {
      double acc = D[i + j * TLD] * -1;
      T[i + j * TLD] = acc;
    }
  for (int j = 0; j < ne; ++j)
    for (int l = 0; l < nc; ++l) {
      double bl = B[l + j * TLD];
      if (bl != 0.0) {
        double temp = 1.0 * bl;
        for (int i = 0; i < nc; ++i) T[i + j * TLD] += temp * C[i + l * TLD];
      }
    }
}

// ------------------------------------------------------------- adjoint ----
// LU with partial pivoting in dgetf2's order, keeping the pivots so that the
// adjoint can solve with both A and A^T of one interaction region.
__device__ int d_getrf(int n, double* A, int lda, int* ipiv) {
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = fabs(A[j + j * lda]);
    for (int i = j + 1; i < n; ++i)
      if (fabs(A[i + j * lda]) > amax) {
        amax = fabs(A[i + j * lda]);
        jp = i;
      }
    ipiv[j] = jp;
    if (A[jp + j * lda] == 0.0) return j + 1;
    if (jp != j)
      for (int c = 0; c < n; ++c) {
        double t = A[j + c * lda];
        A[j + c * lda] = A[jp + c * lda];
        A[jp + c * lda] = t;
      }
    const double rp = 1.0 / A[j + j * lda];
    for (int i = j + 1; i < n; ++i) A[i + j * lda] *= rp;
    for (int c = j + 1; c < n; ++c) {
      const double yv = A[j + c * lda];
      if (yv != 0.0)
        for (int i = j + 1; i < n; ++i) A[i + c * lda] -= A[i + j * lda] * yv;
    }
  }
  return 0;
}

// x = A^{-1} x with P A = L U from d_getrf
__device__ void d_getrs_n(int n, const double* LU, int lda, const int* ipiv, double* x) {
  for (int j = 0; j < n; ++j)
    if (ipiv[j] != j) {
      double t = x[j];
      x[j] = x[ipiv[j]];
      x[ipiv[j]] = t;
    }
  for (int k = 0; k < n; ++k)
    for (int i = k + 1; i < n; ++i) x[i] -= x[k] * LU[i + k * lda];
  for (int k = n - 1; k >= 0; --k) {
    x[k] /= LU[k + k * lda];
    for (int i = 0; i < k; ++i) x[i] -= x[k] * LU[i + k * lda];
  }
}

// x = A^{-T} x: A^T = U^T L^T P, so solve U^T, then L^T, then undo the swaps
__device__ void d_getrs_t(int n, const double* LU, int lda, const int* ipiv, double* x) {
  for (int k = 0; k < n; ++k) {
    double s = x[k];
    for (int i = 0; i < k; ++i) s -= LU[i + k * lda] * x[i];
    x[k] = s / LU[k + k * lda];
  }
  for (int k = n - 1; k >= 0; --k) {
    double s = x[k];
    for (int i = k + 1; i < n; ++i) s -= LU[i + k * lda] * x[i];
    x[k] = s;
  }
  for (int j = n - 1; j >= 0; --j)
    if (ipiv[j] != j) {
      double t = x[j];
      x[j] = x[ipiv[j]];
      x[ipiv[j]] = t;
    }
}

// Reverse-mode derivative of the corner-point transmissibilities
// T = C A^{-1} B - D (O_MPFA.java:193-239) with respect to the logarithm of
// each element's permeability tensor.  Every local matrix is a sum of element
// contributions linear in that element's K, so d(.)/d log K_a is element a's
// own contribution (A_a, B_a, C_a, D_a), and
//   dT/dlogK_a = C_a X - D_a + C A^{-1} (B_a - A_a X),   X = A^{-1} B.
// For npairs weight/potential pairs (mu_k per connection, phi_k per element)
// the kernel forms  G_a = sum_k mu_k^T (dT/dlogK_a) phi_k  without building
// dT: with y = X phi and nu = A^{-T} C^T mu,
//   G_a = sum_{faces i of a} (here_i mu_i - nu_i) s_i,
// s_i being the flux of element a's linear potential through face i.  The
// result goes to corner slot (di + 2 dj + 4 dk) of element a, one writer per
// slot, so the per-element sum is deterministic.
__global__ void __launch_bounds__(128) k_mpfa_adjoint_point(
    Grid g, const double* __restrict__ pts, const double* __restrict__ perm, const double* __restrict__ ecenter,
    const double* __restrict__ icenter, const double* __restrict__ inormal, const double* __restrict__ iarea,
    double continuity, int npairs, const double* __restrict__ mu, const double* __restrict__ phi,
    double* __restrict__ Gcorner, int* flag) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  PointTopo t;
  point_topology(g, p, t);
  const int nc = t.nconn, ne = t.ne;
  const int per = g.dim == 3 ? 3 : 2;
  double A[TLD * TLD], C[TLD * TLD], fv[8][3][4];
  for (int q = 0; q < TLD * TLD; ++q) A[q] = C[q] = 0;
  const V3 corner = ld3(pts, p);
  for (int a = 0; a < ne; ++a) {
    const int el = t.el[a];
    const int f0 = a * per;
    const int n = per + 1;
    double Ab[16], Psi[16];
    for (int q = 0; q < 16; ++q) Ab[q] = Psi[q] = 0;
    V3 ec = ld3(ecenter, el);
    Ab[0] = 1;
    Ab[0 + 1 * n] = ec.x;
    Ab[0 + 2 * n] = ec.y;
    if (n == 4) Ab[0 + 3 * n] = ec.z;
    for (int i = 0; i < per; ++i) {
      V3 cp = ld3(icenter, t.face[f0 + i]);
      if (continuity != 1)
        cp = {(cp.x - corner.x) * continuity + corner.x, (cp.y - corner.y) * continuity + corner.y,
              (cp.z - corner.z) * continuity + corner.z};
      Ab[(i + 1)] = 1;
      Ab[(i + 1) + 1 * n] = cp.x;
      Ab[(i + 1) + 2 * n] = cp.y;
      if (n == 4) Ab[(i + 1) + 3 * n] = cp.z;
    }
    for (int i = 0; i < n; ++i) Psi[i + i * n] = 1;
    if (d_dgesv(n, n, Ab, n, Psi, n) != 0) {
      atomicCAS(flag, 0, 1);
      return;
    }
    V3 grad[4];
    for (int i = 0; i < n; ++i) grad[i] = {Psi[1 + i * n], Psi[2 + i * n], n == 4 ? Psi[3 + i * n] : 0.0};
    const double* K = perm + 6 * (int64_t)el;
    const double kxx = K[0], kyy = K[1], kzz = K[2], kxy = K[3], kxz = K[4], kyz = K[5];
    for (int i = 0; i < per; ++i) {
      V3 v = normal_area(g, t, f0 + i, p, pts, inormal, iarea);
      V3 Kn = {kxx * v.x + kxy * v.y + kxz * v.z, kxy * v.x + kyy * v.y + kyz * v.z, kxz * v.x + kyz * v.y + kzz * v.z};
      const int fi = f0 + i;
      const int is = t.lidx[fi];
      const bool isHere = t.boundary[fi] ? true : (t.fo[fi] & 1);
      for (int j = 0; j < per + 1; j++) {
        const double f = vdot(Kn, grad[j]);
        fv[a][i][j] = f;
        if (j == 0) continue;
        const int js = t.lidx[f0 + j - 1];
        A[is + js * TLD] += f;
        if (isHere) C[is + js * TLD] += f;
      }
    }
  }
  int ipiv[TLD];
  if (d_getrf(nc, A, TLD, ipiv) != 0) {
    atomicCAS(flag, 0, 2);
    return;
  }
  double G[8];
  for (int a = 0; a < ne; ++a) G[a] = 0;
  for (int k = 0; k < npairs; ++k) {
    const double* muk = mu + (int64_t)k * g.nconn;
    const double* phik = phi + (int64_t)k * g.nel;
    double m[TLD], y[TLD], v[TLD], ph[8];
    for (int i = 0; i < nc; ++i) m[i] = y[i] = 0;
    // connection weights on the local rows: the here-side face of each
    // interior local connection names its connection
    for (int f = 0; f < t.nf; ++f)
      if (!t.boundary[f] && (t.fo[f] & 1)) {
        const int a = t.fel[f];
        m[t.lidx[f]] = muk[face_connection(g, t.eijk[a][0], t.eijk[a][1], t.eijk[a][2], t.fo[f])];
      }
    for (int a = 0; a < ne; ++a) {
      ph[a] = phik[t.el[a]];
      for (int i = 0; i < per; ++i) y[t.lidx[a * per + i]] -= fv[a][i][0] * ph[a];  // B phi
    }
    d_getrs_n(nc, A, TLD, ipiv, y);
    for (int j = 0; j < nc; ++j) {
      double s = 0;
      for (int i = 0; i < nc; ++i) s += C[i + j * TLD] * m[i];
      v[j] = s;
    }
    d_getrs_t(nc, A, TLD, ipiv, v);
    for (int a = 0; a < ne; ++a)
      for (int i = 0; i < per; ++i) {
        const int fi = a * per + i;
        const int is = t.lidx[fi];
        const bool isHere = t.boundary[fi] ? true : (t.fo[fi] & 1);
        double s = fv[a][i][0] * ph[a];
        for (int j = 1; j < per + 1; ++j) s += fv[a][i][j] * y[t.lidx[a * per + j - 1]];
        G[a] += ((isHere ? m[is] : 0.0) - v[is]) * s;
      }
  }
  const int pi = p % g.npi, pj = (p / g.npi) % g.npj, pk = p / (g.npi * g.npj);
  for (int a = 0; a < ne; ++a) {
    const int slot = (pi - t.eijk[a][0]) + 2 * (pj - t.eijk[a][1]) + (g.dim == 3 ? 4 * (pk - t.eijk[a][2]) : 0);
    Gcorner[8 * (int64_t)t.el[a] + slot] = G[a];
  }
}

// dJ/dlogK per element: scale * sum of its corner slots (+ out when accumulating)
__global__ void k_corner_sum(int nel, int ncorner, const double* __restrict__ Gcorner, double scale, int accumulate,
                             double* __restrict__ out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double s = 0;
  for (int q = 0; q < ncorner; ++q) s += Gcorner[8 * (int64_t)e + q];
  out[e] = (accumulate ? out[e] : 0.0) + scale * s;
}

// storeTransmissibilities (O_MPFA.java:88-112) gathered per connection over
// its corner points in ascending point order, then Connection.check
// (geometry/Connection.java:80-107).
__global__ void k_mpfa_gather(Grid g, int maxmd, const double* __restrict__ Tstore, const int* __restrict__ conn,
                              int* md_len, int* md_elem, double* md_k, int* flag) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nconn) return;
  const int here = conn[2 * c], there = conn[2 * c + 1];
  int i, j, k;
  el_ijk(g, here, i, j, k);
  const int nfe = g.dim == 3 ? 6 : 4;
  int o = -1;
  for (int q = 1; q < nfe; q += 2) {
    int ne, no;
    if (face_neighbour(g, i, j, k, q, ne, no) && ne == there) {
      o = q;
      break;
    }
  }
  const int fh = here * nfe + o;
  int cp[8], ip[4];
  elem_points(g, i, j, k, cp);
  const int np = face_points(g, cp, o, ip);
  // ascending point order
  for (int a = 1; a < np; ++a)
    for (int b = a; b > 0 && ip[b] < ip[b - 1]; --b) {
      int tmp = ip[b];
      ip[b] = ip[b - 1];
      ip[b - 1] = tmp;
    }
  int el[18];
  double kk[18];
  int n = 0;
  PointTopo t;
  for (int a = 0; a < np; ++a) {
    const int p = ip[a];
    point_topology(g, p, t);
    int li = -1;
    for (int f = 0; f < t.nf; ++f)
      if (t.face[f] == fh) {
        li = t.lidx[f];
        break;
      }
    if (li < 0 || li >= TLD) {
      atomicCAS(flag, 0, 5);
      return;
    }
    const double* T = Tstore + (int64_t)p * TSZ;
    for (int e = 0; e < t.ne; ++e) {
      double tk = T[li + e * TLD];
      bool found = false;
      for (int q = 0; q < n; ++q)
        if (el[q] == t.el[e]) {
          found = true;
          kk[q] += tk;
          break;
        }
      if (!found && tk != 0) {
        if (n >= maxmd) {
          atomicCAS(flag, 0, 3);
          return;
        }
        el[n] = t.el[e];
        kk[n] = tk;
        n++;
      }
    }
  }
  double sum = 0;
  bool hasHere = false, hasThere = false;
  for (int q = 0; q < n; ++q) {
    sum += kk[q];
    hasHere |= el[q] == here;
    hasThere |= el[q] == there;
  }
  if (fabs(sum) > 1.0e-6 || !hasHere || !hasThere) atomicCAS(flag, 0, 4);
  md_len[c] = n;
  for (int q = 0; q < n; ++q) {
    md_elem[(int64_t)c * maxmd + q] = el[q];
    md_k[(int64_t)c * maxmd + q] = kk[q] * 1.0;  // connection multiplier (1 on structured grids)
  }
}

// ------------------------------------------------------------ L-method ----
// MPFA.getHalfEdgePoints (MPFA.java:165-201) for the face at position f of
// point p: the midpoints of the face's two edges at p, the one towards the
// next point of the face's circular point list first.
__device__ void half_edge_points(const Grid& g, const PointTopo& t, int f, int p, const double* pts, V3& e1,
                                 V3& e2) {
  int cp[8], ip[4];
  const int a = t.fel[f];
  elem_points(g, t.eijk[a][0], t.eijk[a][1], t.eijk[a][2], cp);
  face_points(g, cp, t.fo[f], ip);
  int i = 0;
  for (int q = 0; q < 4; ++q)
    if (ip[q] == p) {
      i = q;
      break;
    }
  const V3 c1 = ld3(pts, p), c2 = ld3(pts, ip[(i + 1) % 4]), c3 = ld3(pts, ip[i == 0 ? 3 : i - 1]);
  e1 = vmul(vadd(c1, c2), 0.5);
  e2 = vmul(vadd(c1, c3), 0.5);
}

// position in t of the face across face position f (the other side of its connection)
__device__ int across(const Grid& g, const PointTopo& t, int f) {
  const int a = t.fel[f];
  int ne_, no_;
  if (!face_neighbour(g, t.eijk[a][0], t.eijk[a][1], t.eijk[a][2], t.fo[f], ne_, no_)) return -1;
  const int nb = ne_ * (g.dim == 3 ? 6 : 4) + no_;
  for (int q = 0; q < t.nf; ++q)
    if (t.face[q] == nb) return q;
  return -1;
}

// Linear basis functions through four points: column i of A^-1 holds
// c1..c4 of the function that is 1 at point i (L_MPFA.java:406-447, 659-758)
__device__ bool basis4(const V3* q, double* Psi) {
  double Ab[16];
  for (int r = 0; r < 4; ++r) {
    Ab[r] = 1;
    Ab[r + 4] = q[r].x;
    Ab[r + 8] = q[r].y;
    Ab[r + 12] = q[r].z;
  }
  for (int k = 0; k < 16; ++k) Psi[k] = 0;
  for (int i = 0; i < 4; ++i) Psi[i + i * 4] = 1;
  return d_dgesv(4, 4, Ab, 4, Psi, 4) == 0;
}
__device__ __forceinline__ V3 bgrad(const double* Psi, int i) { return {Psi[1 + i * 4], Psi[2 + i * 4], Psi[3 + i * 4]}; }
__device__ __forceinline__ double bval(const double* Psi, int i, V3 x) {
  return Psi[0 + i * 4] + Psi[1 + i * 4] * x.x + Psi[2 + i * 4] * x.y + Psi[3 + i * 4] * x.z;
}
__device__ __forceinline__ V3 kmult6(const double* K, V3 v) {
  return {K[0] * v.x + K[3] * v.y + K[4] * v.z, K[3] * v.x + K[1] * v.y + K[5] * v.z,
          K[4] * v.x + K[5] * v.y + K[2] * v.z};
}

// L_MPFA per interior corner point of a 3-D grid: for each of the 8 elements
// at the point, the T matrix (3 x 4, column major, at slot 12 a) of its L
// interaction region (LmethodInteractionRegion.calculateT, L_MPFA.java:580-657
// and 760-866): rows are the element's faces at the point in the point's
// face order, columns the element, then the elements across those faces.
// Boundary points keep no T (their sub-faces take a two-point flux).
__global__ void __launch_bounds__(128) k_lmpfa_point(Grid g, const double* __restrict__ pts,
                                                     const double* __restrict__ perm,
                                                     const double* __restrict__ ecenter,
                                                     const double* __restrict__ icenter,
                                                     const double* __restrict__ inormal,
                                                     const double* __restrict__ iarea, double* __restrict__ Tstore,
                                                     int* flag) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  PointTopo t;
  point_topology(g, p, t);
  for (int f = 0; f < t.nf; ++f)
    if (t.boundary[f]) return;
  const V3 corner = ld3(pts, p);
  for (int a = 0; a < t.ne; ++a) {
    const int el = t.el[a], f0 = 3 * a;
    double A[9] = {0}, B[12] = {0}, C[9] = {0}, D[12] = {0}, Pp[16], Ps[16];
    // primary: basis through its centre and its three face centres
    V3 q[4] = {ld3(ecenter, el), ld3(icenter, t.face[f0]), ld3(icenter, t.face[f0 + 1]), ld3(icenter, t.face[f0 + 2])};
    if (!basis4(q, Pp)) {
      atomicCAS(flag, 0, 1);
      return;
    }
    for (int i = 0; i < 3; ++i) {
      const V3 kn = kmult6(perm + 6 * (int64_t)el, normal_area(g, t, f0 + i, p, pts, inormal, iarea));
      double fl = vdot(kn, bgrad(Pp, 0));
      B[i] += -fl;
      for (int j = 1; j < 4; ++j) {
        fl = vdot(kn, bgrad(Pp, j));
        A[i + (j - 1) * 3] += fl;
      }
    }
    // secondaries: basis through the centre, the face centre, the corner
    // point and the face's first half-edge point
    for (int i = 0; i < 3; ++i) {
      const int fs = across(g, t, f0 + i);
      if (fs < 0) {
        atomicCAS(flag, 0, 5);
        return;
      }
      const int es = t.el[t.fel[fs]];
      V3 e1, e2;
      half_edge_points(g, t, fs, p, pts, e1, e2);
      V3 qs[4] = {ld3(ecenter, es), ld3(icenter, t.face[fs]), corner, e1};
      if (!basis4(qs, Ps)) {
        atomicCAS(flag, 0, 1);
        return;
      }
      const V3 kn = kmult6(perm + 6 * (int64_t)es, normal_area(g, t, fs, p, pts, inormal, iarea));
      double fl = vdot(kn, bgrad(Ps, 0));
      B[i + (i + 1) * 3] += -fl;
      D[i + (i + 1) * 3] += -fl;
      fl = vdot(kn, bgrad(Ps, 1));
      A[i + i * 3] += fl;
      C[i + i * 3] += fl;
      const V3 at[2] = {corner, e1};
      for (int w = 0; w < 2; ++w) {
        fl = vdot(kn, bgrad(Ps, 2 + w));
        double psik = bval(Pp, 0, at[w]);
        B[i] += -fl * psik;
        D[i] += -fl * psik;
        for (int k = 1; k < 4; ++k) {
          psik = bval(Pp, k, at[w]);
          A[i + (k - 1) * 3] += fl * psik;
          C[i + (k - 1) * 3] += fl * psik;
        }
      }
    }
    // T = C (A \ B) - D (MPFA.java:43-54)
    if (d_dgesv(3, 4, A, 3, B, 3) != 0) {
      atomicCAS(flag, 0, 2);
      return;
    }
    double* T = Tstore + (int64_t)p * TSZ + 12 * a;
    for (int k = 0; k < 12; ++k) T[k] = D[k] * -1;
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 3; ++l) {
        const double bl = B[l + j * 3];
        if (bl != 0.0) {
          const double temp = 1.0 * bl;
          for (int i = 0; i < 3; ++i) T[i + j * 3] += temp * C[i + l * 3];
        }
      }
  }
}

// The L-method's MD lists gathered per connection over its corner points in
// ascending point order: at an interior point the L region (here or there
// element as primary) whose primary coefficient on the connection's sub-face
// is smaller in magnitude, the second on a tie (chooseTransmissibilities,
// L_MPFA.java:170-212), stored with storeLTransmissibilities' sign and
// zero rules (:218-249); at a boundary point the two-point flux over the
// sub-face (calculateBoundaryTransmissibilities, :77-126).  Then
// Connection.check.
__global__ void k_lmpfa_gather(Grid g, int maxmd, const double* __restrict__ Tstore, const int* __restrict__ conn,
                               const double* __restrict__ pts, const double* __restrict__ perm,
                               const double* __restrict__ ecenter, const double* __restrict__ icenter,
                               const double* __restrict__ inormal, int* md_len, int* md_elem, double* md_k,
                               int* flag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nconn) return;
  const int here = conn[2 * c], there = conn[2 * c + 1];
  int i, j, k;
  el_ijk(g, here, i, j, k);
  int o = -1, ot = -1;
  for (int q = 1; q < 6; q += 2) {
    int ne_, no_;
    if (face_neighbour(g, i, j, k, q, ne_, no_) && ne_ == there) {
      o = q;
      ot = no_;
      break;
    }
  }
  const int fh = here * 6 + o, ft = there * 6 + ot;
  int cp[8], ip[4];
  elem_points(g, i, j, k, cp);
  face_points(g, cp, o, ip);
  for (int a = 1; a < 4; ++a)
    for (int b = a; b > 0 && ip[b] < ip[b - 1]; --b) {
      const int tmp = ip[b];
      ip[b] = ip[b - 1];
      ip[b - 1] = tmp;
    }
  int el[18];
  double kk[18];
  int n = 0;
  auto add = [&](int e, double tk, bool keep) {
    for (int q = 0; q < n; ++q)
      if (el[q] == e) {
        kk[q] += tk;
        return true;
      }
    if (tk != 0 || keep) {
      if (n >= maxmd) return false;
      el[n] = e;
      kk[n] = tk;
      n++;
    }
    return true;
  };
  PointTopo t;
  for (int a = 0; a < 4; ++a) {
    const int p = ip[a];
    point_topology(g, p, t);
    bool onb = false;
    for (int f = 0; f < t.nf; ++f) onb |= t.boundary[f] != 0;
    int ph = -1, pt = -1;
    for (int f = 0; f < t.nf; ++f) {
      if (t.face[f] == fh) ph = f;
      if (t.face[f] == ft) pt = f;
    }
    if (ph < 0 || pt < 0) {
      atomicCAS(flag, 0, 5);
      return;
    }
    if (onb) {
      const V3 ki = kmult6(perm + 6 * (int64_t)here, ld3(inormal, fh));
      const V3 kj = kmult6(perm + 6 * (int64_t)there, ld3(inormal, ft));
      const double Kin = sqrt(ki.x * ki.x + ki.y * ki.y + ki.z * ki.z);
      const double Kjn = sqrt(kj.x * kj.x + kj.y * kj.y + kj.z * kj.z);
      // MPFA.computeSubFaceArea (MPFA.java:131-160)
      V3 e1, e2;
      half_edge_points(g, t, ph, p, pts, e1, e2);
      const V3 fa = ld3(icenter, fh), fb = ld3(pts, p);
      const V3 ab = vsub(fb, fa), ac = vsub(e1, fa), ad = vsub(e2, fa);
      const double A1 = 0.5 * vnorm(vcross(ab, ac));
      const double A2 = 0.5 * vnorm(vcross(ab, ad));
      const double A = A1 + A2;
      double tt = 0;
      if (Kin != 0 && Kjn != 0)
        tt = Kin * Kjn * A /
             (Kjn * vnorm(vsub(fa, ld3(ecenter, here))) + Kjn * vnorm(vsub(ld3(icenter, ft), ld3(ecenter, there))));
      if (!add(here, tt, false) || !add(there, -tt, false)) {
        atomicCAS(flag, 0, 3);
        return;
      }
      continue;
    }
    // the two candidate regions: here and there element as primary; the
    // sub-face's row is the primary's own face on the connection
    const int aH = t.fel[ph], aT = t.fel[pt];
    const int rH = ph - 3 * aH, rT = pt - 3 * aT;
    const double* TH = Tstore + (int64_t)p * TSZ + 12 * aH;
    const double* TT = Tstore + (int64_t)p * TSZ + 12 * aT;
    const bool pickH = fabs(TH[rH]) < fabs(TT[rT]);
    const int ap = pickH ? aH : aT, row = pickH ? rH : rT;
    const double* T = pickH ? TH : TT;
    const int prim = t.el[ap];
    for (int jj = 0; jj < 4; ++jj) {
      int e = prim;
      if (jj > 0) {
        const int fs = across(g, t, 3 * ap + jj - 1);
        if (fs < 0) {
          atomicCAS(flag, 0, 5);
          return;
        }
        e = t.el[t.fel[fs]];
      }
      double tk = T[row + jj * 3];
      if (prim == here) tk *= -1;
      if (!add(e, tk, e == here || e == there)) {
        atomicCAS(flag, 0, 3);
        return;
      }
    }
  }
  double sum = 0;
  bool hasHere = false, hasThere = false;
  for (int q = 0; q < n; ++q) {
    sum += kk[q];
    hasHere |= el[q] == here;
    hasThere |= el[q] == there;
  }
  if (fabs(sum) > 1.0e-6 || !hasHere || !hasThere) atomicCAS(flag, 0, 4);
  md_len[c] = n;
  for (int q = 0; q < n; ++q) {
    md_elem[(int64_t)c * maxmd + q] = el[q];
    md_k[(int64_t)c * maxmd + q] = kk[q] * 1.0;  // connection multiplier (1 on structured grids)
  }
}

__global__ void k_md_compact(int nconn, int maxmd, const int* __restrict__ ptr, const int* __restrict__ el_in,
                             const double* __restrict__ k_in, int* el_out, double* k_out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nconn) return;
  for (int q = ptr[c]; q < ptr[c + 1]; ++q) {
    el_out[q] = el_in[(int64_t)c * maxmd + (q - ptr[c])];
    k_out[q] = k_in[(int64_t)c * maxmd + (q - ptr[c])];
  }
}

// cell -> incident connections, ascending
__global__ void k_cell_conns(Grid g, int* cptr_fixed /* nel * 6 */, int* ccount) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel) return;
  int i, j, k;
  el_ijk(g, e, i, j, k);
  const int nfe = g.dim == 3 ? 6 : 4;
  int cs[6], n = 0;
  for (int o = 0; o < nfe; ++o) {
    int ne, no;
    if (!face_neighbour(g, i, j, k, o, ne, no)) continue;
    int c = face_connection(g, i, j, k, o);
    // side flag in the sign bit region: store c*2 + (here ? 0 : 1)
    cs[n++] = 2 * c + ((o & 1) ? 0 : 1);
  }
  for (int a = 1; a < n; ++a)
    for (int b = a; b > 0 && cs[b] < cs[b - 1]; --b) {
      int tmp = cs[b];
      cs[b] = cs[b - 1];
      cs[b - 1] = tmp;
    }
  for (int a = 0; a < 6; ++a) cptr_fixed[(int64_t)e * 6 + a] = a < n ? cs[a] : -1;
  ccount[e] = n;
}

// Row pattern: diagonal (optional) plus MD elements of incident connections.
template <bool FILL>
__global__ void k_rows(int nel, int with_diag, const int* __restrict__ cc, const int* __restrict__ ccount,
                       const int* __restrict__ md_ptr, const int* __restrict__ md_el, int* row_len,
                       const int* __restrict__ row_ptr, int* col) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int buf[128];
  int n = 0;
  if (with_diag) buf[n++] = e;
  for (int a = 0; a < ccount[e]; ++a) {
    int c = cc[(int64_t)e * 6 + a] >> 1;
    for (int q = md_ptr[c]; q < md_ptr[c + 1] && n < 128; ++q) buf[n++] = md_el[q];
  }
  for (int a = 1; a < n; ++a)
    for (int b = a; b > 0 && buf[b] < buf[b - 1]; --b) {
      int tmp = buf[b];
      buf[b] = buf[b - 1];
      buf[b - 1] = tmp;
    }
  int m = 0;
  for (int a = 0; a < n; ++a)
    if (a == 0 || buf[a] != buf[a - 1]) {
      if (FILL) col[row_ptr[e] + m] = buf[a];
      m++;
    }
  if (!FILL) row_len[e] = m;
}

// TPFA.calculateTransmissibility (geometry/flux/TPFA.java:50-72), with its
// use of ||K_j n_j|| for both distances: MD = {(here, t), (there, -t)}.
__global__ void k_tpfa(Grid g, const int* __restrict__ conn, const double* __restrict__ perm,
                       const double* __restrict__ ecenter, const double* __restrict__ iarea,
                       const double* __restrict__ icenter, const double* __restrict__ inormal, int* md_ptr, int* md_el,
                       double* md_k) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) md_ptr[g.nconn] = 2 * g.nconn;
  if (c >= g.nconn) return;
  const int ei = conn[2 * c], ej = conn[2 * c + 1];
  int i, j, k;
  el_ijk(g, ei, i, j, k);
  const int nfe = g.dim == 3 ? 6 : 4;
  int o = -1, oj = -1;
  for (int q = 1; q < nfe; q += 2) {
    int ne, no;
    if (face_neighbour(g, i, j, k, q, ne, no) && ne == ej) {
      o = q;
      oj = no;
      break;
    }
  }
  const int is = ei * nfe + o, js = ej * nfe + oj;
  auto mult_norm = [&](int el, V3 v) {
    const double* K = perm + 6 * (int64_t)el;
    const double xx = K[0], yy = K[1], zz = K[2], xy = K[3], xz = K[4], yz = K[5];
    const double x = xx * v.x + xy * v.y + xz * v.z;
    const double y = xy * v.x + yy * v.y + yz * v.z;
    const double z = xz * v.x + yz * v.y + zz * v.z;
    return sqrt(x * x + y * y + z * z);
  };
  const double Kin = mult_norm(ei, ld3(inormal, is));
  const double Kjn = mult_norm(ej, ld3(inormal, js));
  const double A = iarea[is];
  double t = 0;
  if (Kin != 0 && Kjn != 0)
    t = Kin * Kjn * A /
        (Kjn * vnorm(vsub(ld3(icenter, is), ld3(ecenter, ei))) + Kjn * vnorm(vsub(ld3(icenter, js), ld3(ecenter, ej))));
  md_ptr[c] = 2 * c;
  md_el[2 * c] = ei;
  md_k[2 * c] = t * 1.0;  // connection multiplier (1 on structured grids)
  md_el[2 * c + 1] = ej;
  md_k[2 * c + 1] = -t * 1.0;
}

// Adjoint of the TPFA transmissibilities: t_c = ||K_here n|| A / (d_here + d_there)
// (||K_there n|| cancels), so d t_c / d log K_here = t_c and the there side
// has no derivative: out[e] (+)= scale * sum_k sum_{c here at e} mu_k,c F_k,c.
__global__ void k_tpfa_adjoint(int nel, int nconn, int npairs, const int* __restrict__ cc,
                               const int* __restrict__ ccount, const int* __restrict__ conn,
                               const double* __restrict__ md_k, const double* __restrict__ mu,
                               const double* __restrict__ phi, double scale, int accumulate, double* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double s = 0;
  for (int a = 0; a < ccount[e]; ++a) {
    const int code = cc[(int64_t)e * 6 + a];
    if (code & 1) continue;  // there side
    const int c = code >> 1;
    const int t = conn[2 * c + 1];
    for (int k = 0; k < npairs; ++k)
      s += mu[(int64_t)k * nconn + c] * md_k[2 * c] * (phi[(int64_t)k * nel + e] - phi[(int64_t)k * nel + t]);
  }
  out[e] = (accumulate ? out[e] : 0.0) + scale * s;
}

__device__ int bsearch_pos(const int* col, int lo, int hi, int key) {
  hi -= 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int v = col[mid];
    if (v < key) lo = mid + 1;
    else if (v > key) hi = mid - 1;
    else return mid;
  }
  return -1;
}

__global__ void k_md_pos(int nconn, const int* __restrict__ conn, const int* __restrict__ md_ptr,
                         const int* __restrict__ md_el, const int* __restrict__ rp, const int* __restrict__ col,
                         int* pos_here, int* pos_there) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nconn) return;
  int h = conn[2 * c], t = conn[2 * c + 1];
  for (int q = md_ptr[c]; q < md_ptr[c + 1]; ++q) {
    pos_here[q] = bsearch_pos(col, rp[h], rp[h + 1], md_el[q]);
    pos_there[q] = bsearch_pos(col, rp[t], rp[t + 1], md_el[q]);
  }
}

// PotentialCalculator.discretizeFlux, gathered per row in connection order.
__global__ void k_potential_rows(int nel, const int* __restrict__ cc, const int* __restrict__ ccount,
                                 const int* __restrict__ md_ptr, const int* __restrict__ md_el,
                                 const double* __restrict__ md_k, const int* __restrict__ rp,
                                 const int* __restrict__ col, double* val) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  for (int q = rp[e]; q < rp[e + 1]; ++q) val[q] = 0;
  for (int a = 0; a < ccount[e]; ++a) {
    int code = cc[(int64_t)e * 6 + a];
    int c = code >> 1;
    bool here = !(code & 1);
    for (int q = md_ptr[c]; q < md_ptr[c + 1]; ++q) {
      int pos = bsearch_pos(col, rp[e], rp[e + 1], md_el[q]);
      if (pos >= 0) val[pos] += here ? md_k[q] : -md_k[q];
    }
  }
}

// flux[c] = sum_k t_k p[el_k] over connection c's MD list, in list order
// (PotentialCalculator.calculateFlux, numerics/PotentialCalculator.java:265-280;
// LocalFlowRateAverage.computeDarcyFlux, upscale/LocalFlowRateAverage.java:123-137).
__global__ void k_connection_flux(int nconn, const int* __restrict__ md_ptr, const int* __restrict__ md_el,
                                  const double* __restrict__ md_k, const double* __restrict__ p, double* flux) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nconn) return;
  double f = 0;
  for (int q = md_ptr[c]; q < md_ptr[c + 1]; ++q) f += md_k[q] * p[md_el[q]];
  flux[c] = f;
}

// Centre of each connection's here interface (the here element's face that
// points to the there element): Connection.hereInterface().center.
__global__ void k_connection_icenter(Grid g, const int* __restrict__ conn, const double* __restrict__ icenter,
                                     double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nconn) return;
  const int ei = conn[2 * c], ej = conn[2 * c + 1];
  int i, j, k;
  el_ijk(g, ei, i, j, k);
  const int nfe = g.dim == 3 ? 6 : 4;
  int o = 1;
  for (int q = 0; q < nfe; ++q) {
    int ne, no;
    if (face_neighbour(g, i, j, k, q, ne, no) && ne == ej) {
      o = q;
      break;
    }
  }
  for (int a = 0; a < 3; ++a) out[3 * (int64_t)c + a] = icenter[3 * ((int64_t)ei * nfe + o) + a];
}

}  // namespace

static void make_grid(Grid& g, int dim, int ni, int nj, int nk) {
  g.dim = dim;
  g.ni = ni;
  g.nj = nj;
  g.nk = dim == 3 ? nk : 0;
  g.npi = ni + 1;
  g.npj = nj + 1;
  g.npk = dim == 3 ? nk + 1 : 1;
  g.npts = g.npi * g.npj * g.npk;
  g.nel = dim == 3 ? ni * nj * nk : ni * nj;
  g.nfacepe = dim == 3 ? 6 : 4;
  g.nintf = g.nel * g.nfacepe;
  g.nconn = dim == 3 ? 3 * ni * nj * nk - ni * nj - ni * nk - nj * nk : 2 * ni * nj - ni - nj;
}

static void scan_lengths(const std::vector<int>& len, std::vector<int>& ptr) {
  ptr.assign(len.size() + 1, 0);
  for (size_t i = 0; i < len.size(); ++i) ptr[i + 1] = ptr[i] + len[i];
}

// MD lists gathered per connection (fixed stride maxmd) into the mesh's CSR
// form, after the gather kernel's status flag is checked
static void install_md(Mesh& m, DeviceBuffer<int>& flag, DeviceBuffer<int>& mdlen, DeviceBuffer<int>& mdel,
                       DeviceBuffer<double>& mdk) {
  Context& c = *m.ctx;
  const Grid& g = m.g;
  int hf = 0;
  std::vector<int> hl(g.nconn);
  RSG_CUDA(cudaMemcpyAsync(&hf, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  if (g.nconn > 0)
    RSG_CUDA(cudaMemcpyAsync(hl.data(), mdlen.get(), sizeof(int) * g.nconn, cudaMemcpyDeviceToHost, c.stream));
  c.sync();
  if (hf == 1) throw Error(RSG_SINGULAR, "Severe grid distortion (singular basis system)");
  if (hf == 2) throw Error(RSG_SINGULAR, "Conductivity tensor does not appear to be symmetrical, positive definite");
  if (hf == 3) throw Error(RSG_BAD_ARG, "too many transmissibilities on a connection");
  if (hf == 4) throw Error(RSG_BAD_ARG, "Transmissibilities on a connection fail the consistency check");
  if (hf == 5) throw Error(RSG_BAD_ARG, "interaction region lookup failed");
  scan_lengths(hl, m.h_md_ptr);
  m.nmd = m.h_md_ptr[g.nconn];
  m.md_ptr.resize(g.nconn + 1);
  m.md_elem.resize(std::max<int64_t>(m.nmd, 1));
  m.md_k.resize(std::max<int64_t>(m.nmd, 1));
  RSG_CUDA(cudaMemcpyAsync(m.md_ptr.get(), m.h_md_ptr.data(), sizeof(int) * (g.nconn + 1), cudaMemcpyHostToDevice,
                           c.stream));
  RSG_LAUNCH(c, "md_compact", k_md_compact, blocks_for(std::max(g.nconn, 1), 256), 256, 0, g.nconn, m.maxmd,
             m.md_ptr.get(), mdel.get(), mdk.get(), m.md_elem.get(), m.md_k.get());
  m.h_md_elem.resize(m.nmd);
  RSG_CUDA(cudaMemcpyAsync(m.h_md_elem.data(), m.md_elem.get(), sizeof(int) * m.nmd, cudaMemcpyDeviceToHost,
                           c.stream));
  c.sync();
  m.have_md = true;
  m.build_patterns();
}

void mpfa_adjoint(Mesh& m, int npairs, const double* mu, const double* phi, double scale, bool accumulate,
                  double* out) {
  if (!m.have_md) throw Error(RSG_BAD_ARG, "transmissibilities have not been computed");
  if (m.lmethod) throw Error(RSG_UNSUPPORTED, "the adjoint is built for MPFA-O and TPFA transmissibilities");
  Context& c = *m.ctx;
  const Grid& g = m.g;
  if (m.tpfa) {
    RSG_LAUNCH(c, "tpfa_adjoint", k_tpfa_adjoint, blocks_for(g.nel, 128), 128, 0, g.nel, g.nconn, npairs,
               m.cell_conn.get(), m.cell_conn_ptr.get(), m.conn.get(), m.md_k.get(), mu, phi, scale,
               accumulate ? 1 : 0, out);
    c.sync();
    return;
  }
  DeviceBuffer<double> corner((size_t)g.nel * 8);
  DeviceBuffer<int> flag(1);
  RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), c.stream));
  RSG_CUDA(cudaMemsetAsync(corner.get(), 0, sizeof(double) * g.nel * 8, c.stream));
  RSG_LAUNCH(c, "mpfa_adjoint_point", k_mpfa_adjoint_point, blocks_for(g.npts, 128), 128, 0, g, m.pts.get(),
             m.perm.get(), m.ecenter.get(), m.icenter.get(), m.inormal.get(), m.iarea.get(), m.continuity, npairs, mu,
             phi, corner.get(), flag.get());
  RSG_LAUNCH(c, "corner_sum", k_corner_sum, blocks_for(g.nel, 128), 128, 0, g.nel, g.dim == 3 ? 8 : 4, corner.get(),
             scale, accumulate ? 1 : 0, out);
  int hf = 0;
  RSG_CUDA(cudaMemcpyAsync(&hf, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  c.sync();
  if (hf) throw Error(RSG_SINGULAR, "singular interaction region in the transmissibility adjoint");
}

void Mesh::build_patterns() {
  Context& c = *ctx;
  const int n = g.nel;
  DeviceBuffer<int> cc((size_t)n * 6), ccount(n);
  RSG_LAUNCH(c, "cell_conns", k_cell_conns, blocks_for(n, 256), 256, 0, g, cc.get(), ccount.get());
  DeviceBuffer<int> len(n);
  auto one = [&](int with_diag, std::vector<int>& hrow, std::vector<int>& hcol, DeviceBuffer<int>& drow,
                 DeviceBuffer<int>& dcol) {
    RSG_LAUNCH(c, "pattern_rows", k_rows<false>, blocks_for(n, 128), 128, 0, n, with_diag, cc.get(), ccount.get(),
               md_ptr.get(), md_elem.get(), len.get(), (const int*)nullptr, (int*)nullptr);
    std::vector<int> hl(n);
    RSG_CUDA(cudaMemcpyAsync(hl.data(), len.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    scan_lengths(hl, hrow);
    drow.resize(n + 1);
    dcol.resize(std::max(hrow[n], 1));
    RSG_CUDA(cudaMemcpyAsync(drow.get(), hrow.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, c.stream));
    RSG_LAUNCH(c, "pattern_rows", k_rows<true>, blocks_for(n, 128), 128, 0, n, with_diag, cc.get(), ccount.get(),
               md_ptr.get(), md_elem.get(), len.get(), drow.get(), dcol.get());
    hcol.resize(hrow[n]);
    RSG_CUDA(cudaMemcpyAsync(hcol.data(), dcol.get(), sizeof(int) * hrow[n], cudaMemcpyDeviceToHost, c.stream));
    c.sync();
  };
  DeviceBuffer<int> prow, pcol, qrow, qcol;
  one(1, h_prow, h_pcol, prow, pcol);
  one(0, h_qrow, h_qcol, qrow, qcol);
  md_pos_here.resize(std::max<int64_t>(nmd, 1));
  md_pos_there.resize(std::max<int64_t>(nmd, 1));
  RSG_LAUNCH(c, "md_pos", k_md_pos, blocks_for(g.nconn, 128), 128, 0, g.nconn, conn.get(), md_ptr.get(),
             md_elem.get(), prow.get(), pcol.get(), md_pos_here.get(), md_pos_there.get());
  cell_conn_ptr = std::move(ccount);
  cell_conn = std::move(cc);
  c.sync();
}

}  // namespace rsg

using rsg::guarded;

extern "C" {

rsg_status rsg_mesh_create_structured(rsg_ctx* ctx, int32_t dim, int32_t ni, int32_t nj, int32_t nk,
                                      const double* coords, double x0, double y0, double z0, double dx, double dy,
                                      double dz, const double* perm, rsg_mesh** out) {
  if (!ctx || !out || !perm) return RSG_BAD_ARG;
  if ((dim != 2 && dim != 3) || ni <= 0 || nj <= 0 || (dim == 3 && nk <= 0)) return RSG_BAD_ARG;
  *out = nullptr;
  rsg_mesh* h = new rsg_mesh();
  rsg_status st = guarded(&ctx->c, [&] {
    rsg::Mesh& m = h->m;
    m.ctx = &ctx->c;
    rsg::make_grid(m.g, dim, ni, nj, nk);
    const rsg::Grid& g = m.g;
    if ((int64_t)g.nel * 6 > INT32_MAX) throw rsg::Error(RSG_UNSUPPORTED, "grid too large");
    m.maxmd = dim == 3 ? 18 : 6;
    std::vector<double> p((size_t)g.npts * 3);
    if (coords) std::copy(coords, coords + p.size(), p.begin());
    else
      for (int k = 0; k < g.npk; ++k)
        for (int j = 0; j < g.npj; ++j)
          for (int i = 0; i < g.npi; ++i) {
            double x = x0, y = y0, z = (dim == 3) ? z0 : 0.0;
            for (int a = 0; a < i; ++a) x += dx;
            for (int a = 0; a < j; ++a) y += dy;
            if (dim == 3)
              for (int a = 0; a < k; ++a) z += dz;
            size_t q = (size_t)i + (size_t)j * g.npi + (size_t)k * g.npi * g.npj;
            p[3 * q] = x;
            p[3 * q + 1] = y;
            p[3 * q + 2] = z;
          }
    rsg::Context& c = ctx->c;
    m.pts.resize(p.size());
    m.perm.resize((size_t)g.nel * 6);
    RSG_CUDA(cudaMemcpyAsync(m.pts.get(), p.data(), sizeof(double) * p.size(), cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(m.perm.get(), perm, sizeof(double) * g.nel * 6, cudaMemcpyHostToDevice, c.stream));
    m.ecenter.resize((size_t)g.nel * 3);
    m.evol.resize(g.nel);
    m.iarea.resize(g.nintf);
    m.icenter.resize((size_t)g.nintf * 3);
    m.inormal.resize((size_t)g.nintf * 3);
    m.conn.resize((size_t)g.nconn * 2);
    RSG_LAUNCH(c, "geometry", rsg::k_geometry, rsg::blocks_for(g.nel, 128), 128, 0, g, m.pts.get(), m.ecenter.get(),
               m.evol.get(), m.iarea.get(), m.icenter.get(), m.inormal.get());
    RSG_LAUNCH(c, "connections", rsg::k_connections, rsg::blocks_for(g.nel, 256), 256, 0, g, m.conn.get());
    m.h_conn.resize((size_t)g.nconn * 2);
    RSG_CUDA(cudaMemcpyAsync(m.h_conn.data(), m.conn.get(), sizeof(int) * m.h_conn.size(), cudaMemcpyDeviceToHost,
                             c.stream));
    c.sync();
  });
  if (st != RSG_OK) {
    delete h;
    return st;
  }
  *out = h;
  return RSG_OK;
}

rsg_status rsg_mesh_destroy(rsg_mesh* m) {
  if (!m) return RSG_BAD_ARG;
  if (m->m.ctx) cudaStreamSynchronize(m->m.ctx->stream);
  delete m;
  return RSG_OK;
}

rsg_status rsg_mesh_compute_mpfa(rsg_mesh* mh, double continuity) {
  if (!mh) return RSG_BAD_ARG;
  if (continuity > 1 || continuity <= 0) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    rsg::Context& c = *m.ctx;
    const rsg::Grid& g = m.g;
    m.continuity = continuity;
    rsg::DeviceBuffer<double> T((size_t)g.npts * rsg::TSZ);
    rsg::DeviceBuffer<int> flag(1), mdlen(g.nconn), mdel((size_t)g.nconn * m.maxmd);
    rsg::DeviceBuffer<double> mdk((size_t)g.nconn * m.maxmd);
    RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), c.stream));
    RSG_LAUNCH(c, "mpfa_point", rsg::k_mpfa_point, rsg::blocks_for(g.npts, 128), 128, 0, g, m.pts.get(), m.perm.get(),
               m.ecenter.get(), m.icenter.get(), m.inormal.get(), m.iarea.get(), continuity, T.get(), flag.get());
    RSG_LAUNCH(c, "mpfa_gather", rsg::k_mpfa_gather, rsg::blocks_for(g.nconn, 128), 128, 0, g, m.maxmd, T.get(),
               m.conn.get(), mdlen.get(), mdel.get(), mdk.get(), flag.get());
    rsg::install_md(m, flag, mdlen, mdel, mdk);
    m.tpfa = false;
    m.lmethod = false;
  });
}

// L_MPFA.calculateTransmissibilities (geometry/flux/L_MPFA.java:52-74) on the GPU
rsg_status rsg_mesh_compute_lmpfa(rsg_mesh* mh) {
  if (!mh) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (m.g.dim != 3) return RSG_UNSUPPORTED;
  return guarded(m.ctx, [&] {
    rsg::Context& c = *m.ctx;
    const rsg::Grid& g = m.g;
    rsg::DeviceBuffer<double> T((size_t)g.npts * rsg::TSZ);
    rsg::DeviceBuffer<int> flag(1), mdlen(g.nconn), mdel((size_t)g.nconn * m.maxmd);
    rsg::DeviceBuffer<double> mdk((size_t)g.nconn * m.maxmd);
    RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), c.stream));
    RSG_LAUNCH(c, "lmpfa_point", rsg::k_lmpfa_point, rsg::blocks_for(g.npts, 128), 128, 0, g, m.pts.get(),
               m.perm.get(), m.ecenter.get(), m.icenter.get(), m.inormal.get(), m.iarea.get(), T.get(), flag.get());
    RSG_LAUNCH(c, "lmpfa_gather", rsg::k_lmpfa_gather, rsg::blocks_for(std::max(g.nconn, 1), 128), 128, 0, g,
               m.maxmd, T.get(), m.conn.get(), m.pts.get(), m.perm.get(), m.ecenter.get(), m.icenter.get(),
               m.inormal.get(), mdlen.get(), mdel.get(), mdk.get(), flag.get());
    rsg::install_md(m, flag, mdlen, mdel, mdk);
    m.tpfa = false;
    m.lmethod = true;
  });
}

rsg_status rsg_mesh_compute_tpfa(rsg_mesh* mh) {
  if (!mh) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    rsg::Context& c = *m.ctx;
    const rsg::Grid& g = m.g;
    m.nmd = 2 * (int64_t)g.nconn;
    m.md_ptr.resize(g.nconn + 1);
    m.md_elem.resize(std::max<int64_t>(m.nmd, 1));
    m.md_k.resize(std::max<int64_t>(m.nmd, 1));
    RSG_LAUNCH(c, "tpfa", rsg::k_tpfa, rsg::blocks_for(std::max(g.nconn, 1), 128), 128, 0, g, m.conn.get(),
               m.perm.get(), m.ecenter.get(), m.iarea.get(), m.icenter.get(), m.inormal.get(), m.md_ptr.get(),
               m.md_elem.get(), m.md_k.get());
    m.h_md_ptr.resize(g.nconn + 1);
    m.h_md_elem.resize(m.nmd);
    RSG_CUDA(cudaMemcpyAsync(m.h_md_ptr.data(), m.md_ptr.get(), sizeof(int) * (g.nconn + 1), cudaMemcpyDeviceToHost,
                             c.stream));
    RSG_CUDA(cudaMemcpyAsync(m.h_md_elem.data(), m.md_elem.get(), sizeof(int) * m.nmd, cudaMemcpyDeviceToHost,
                             c.stream));
    c.sync();
    m.have_md = true;
    m.tpfa = true;
    m.lmethod = false;
    m.build_patterns();
  });
}

rsg_status rsg_mesh_get_counts(rsg_mesh* mh, int64_t* counts) {
  if (!mh || !counts) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  counts[0] = m.g.nel;
  counts[1] = m.g.nconn;
  counts[2] = m.nmd;
  counts[3] = m.g.npts;
  counts[4] = m.h_pcol.size();
  return RSG_OK;
}

rsg_status rsg_mesh_get_geometry(rsg_mesh* mh, double* centers, double* volumes) {
  if (!mh) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    if (centers)
      RSG_CUDA(cudaMemcpyAsync(centers, m.ecenter.get(), sizeof(double) * 3 * m.g.nel, cudaMemcpyDeviceToHost,
                               m.ctx->stream));
    if (volumes)
      RSG_CUDA(cudaMemcpyAsync(volumes, m.evol.get(), sizeof(double) * m.g.nel, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_mesh_get_connections(rsg_mesh* mh, int32_t* conn) {
  if (!mh || !conn) return RSG_BAD_ARG;
  std::copy(mh->m.h_conn.begin(), mh->m.h_conn.end(), conn);
  return RSG_OK;
}

rsg_status rsg_mesh_get_transmissibilities(rsg_mesh* mh, int32_t* md_ptr, int32_t* md_elem, double* md_k) {
  if (!mh) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (!m.have_md) return RSG_BAD_ARG;
  return guarded(m.ctx, [&] {
    if (md_ptr) std::copy(m.h_md_ptr.begin(), m.h_md_ptr.end(), md_ptr);
    if (md_elem) std::copy(m.h_md_elem.begin(), m.h_md_elem.end(), md_elem);
    if (md_k)
      RSG_CUDA(cudaMemcpyAsync(md_k, m.md_k.get(), sizeof(double) * m.nmd, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_mesh_get_pattern(rsg_mesh* mh, int32_t which, int32_t* row_ptr, int32_t* col, int64_t* nnz) {
  if (!mh || (which != 0 && which != 1)) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (!m.have_md) return RSG_BAD_ARG;
  const auto& r = which == 0 ? m.h_prow : m.h_qrow;
  const auto& c = which == 0 ? m.h_pcol : m.h_qcol;
  if (nnz) *nnz = (int64_t)c.size();
  if (row_ptr) std::copy(r.begin(), r.end(), row_ptr);
  if (col) std::copy(c.begin(), c.end(), col);
  return RSG_OK;
}

rsg_status rsg_mesh_connection_flux(rsg_mesh* mh, const double* p, double* flux) {
  if (!mh || !p || !flux) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (!m.have_md) return RSG_BAD_ARG;
  return guarded(m.ctx, [&] {
    rsg::DeviceBuffer<double> dp(m.g.nel), df(std::max(m.g.nconn, 1));
    RSG_CUDA(cudaMemcpyAsync(dp.get(), p, sizeof(double) * m.g.nel, cudaMemcpyHostToDevice, m.ctx->stream));
    if (m.g.nconn > 0)
      RSG_LAUNCH(*m.ctx, "connection_flux", rsg::k_connection_flux, rsg::blocks_for(m.g.nconn, 256), 256, 0,
                 m.g.nconn, m.md_ptr.get(), m.md_elem.get(), m.md_k.get(), (const double*)dp.get(), df.get());
    RSG_CUDA(cudaMemcpyAsync(flux, df.get(), sizeof(double) * m.g.nconn, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_mesh_get_interface_centers(rsg_mesh* mh, double* centers) {
  if (!mh || !centers) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  return guarded(m.ctx, [&] {
    rsg::DeviceBuffer<double> d((size_t)3 * std::max(m.g.nconn, 1));
    if (m.g.nconn > 0)
      RSG_LAUNCH(*m.ctx, "connection_icenter", rsg::k_connection_icenter, rsg::blocks_for(m.g.nconn, 256), 256, 0,
                 m.g, m.conn.get(), m.icenter.get(), d.get());
    RSG_CUDA(cudaMemcpyAsync(centers, d.get(), sizeof(double) * 3 * m.g.nconn, cudaMemcpyDeviceToHost,
                             m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_upscale_pressure(rsg_mesh* mh, int32_t nbc, const int32_t* cells, const double* values, double* x,
                                rsg_solve_info* info) {
  if (!mh || !x || nbc < 0 || (nbc > 0 && (!cells || !values))) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (!m.have_md) return RSG_BAD_ARG;
  const int n = m.g.nel;
  for (int q = 0; q < nbc; ++q)
    if (cells[q] < 0 || cells[q] >= n) return RSG_BAD_ARG;
  // the matrix and the solver of PressureDiscretisation(mesh, bc)
  // (PressureDiscretisation.java:59-87): pattern without the explicit
  // diagonal, GMRES(30) + ILU(0), DefaultIterationMonitor with
  // maxIterations 10000, rtol 1e-50, atol 1e-10, dtol 1e5, x = 0
  rsg_csr A;
  rsg_solver S;
  rsg_status st = guarded(m.ctx, [&] {
    A.m.build(m.ctx, n, (int32_t)m.h_qcol.size(), m.h_qrow.data(), m.h_qcol.data());
    S.s = rsg::make_solver(m.ctx, RSG_GMRES, RSG_PC_ILU, 1e-50, 1e-10, 1e5, 10000, 30);
  });
  // assemble(): A(here,k) += t_k, A(there,k) -= t_k; then for each boundary
  // cell b_i = p_i and row i := e_i (Matrices.zeroRows(A, 1.0, {i}))
  if (st == RSG_OK) st = rsg_mesh_assemble_potential(mh, &A);
  if (st == RSG_OK && nbc > 0) st = rsg_csr_zero_rows(&A, 1.0, nbc, cells);
  if (st == RSG_OK) st = rsg_solver_setup(&S, &A);
  if (st == RSG_OK) {
    std::vector<double> b(n, 0.0);
    for (int q = 0; q < nbc; ++q) b[cells[q]] = values[q];
    std::fill(x, x + n, 0.0);
    rsg_solve_info local{};
    st = rsg_solver_solve(&S, &A, b.data(), x, info ? info : &local);
  }
  cudaStreamSynchronize(m.ctx->stream);
  return st;
}

rsg_status rsg_mesh_assemble_potential(rsg_mesh* mh, rsg_csr* A) {
  if (!mh || !A) return RSG_BAD_ARG;
  rsg::Mesh& m = mh->m;
  if (!m.have_md) return RSG_BAD_ARG;
  return guarded(m.ctx, [&] {
    if (A->m.n != m.g.nel || A->m.h_col != m.h_qcol)
      throw rsg::Error(RSG_OUT_OF_PATTERN, "matrix does not have the potential pattern of this mesh");
    RSG_LAUNCH(*m.ctx, "potential_rows", rsg::k_potential_rows, rsg::blocks_for(m.g.nel, 128), 128, 0, m.g.nel,
               m.cell_conn.get(), m.cell_conn_ptr.get(), m.md_ptr.get(), m.md_elem.get(), m.md_k.get(),
               A->m.rowptr.get(), A->m.col.get(), A->m.val.get());
    A->m.sell_dirty = true;
    m.ctx->sync();
  });
}

}  // extern "C"
