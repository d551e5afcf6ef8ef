// Oracle (test infrastructure only): structured mesh, geometry and MPFA-O.
#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <unordered_map>

namespace orc {

namespace {

// Vector3D arithmetic in the Java evaluation order (geometry/Vector3D.java).
inline Vec3 sub(const Vec3& a, const Vec3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 add(const Vec3& a, const Vec3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 mul(const Vec3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline Vec3 cross(const Vec3& a, const Vec3& v) {
  return {a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x};
}
inline double vdot(const Vec3& a, const Vec3& v) { return a.x * v.x + a.y * v.y + a.z * v.z; }
inline double vnorm(const Vec3& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double comp(const Vec3& a, int c) { return c == 1 ? a.x : (c == 2 ? a.y : a.z); }

// Insertion-ordered set of ints (java.util.LinkedHashSet<Integer>).
struct OrderedSet {
  std::vector<int> v;
  void add(int x) {
    for (int y : v)
      if (y == x) return;
    v.push_back(x);
  }
};

// BilinearMap (meshgen/structured/BilinearMap.java:31-102)
struct Bilinear {
  Vec3 p0, p1, p2, p3, normal;
  double area;
  Bilinear(Vec3 a, Vec3 b, Vec3 c, Vec3 d) : p0(a), p1(b), p2(c), p3(d) {
    Vec3 x1 = p0, x2 = p1, x3 = p2, x4 = p3;
    Vec3 A = cross(sub(x2, x1), sub(x3, x1));
    Vec3 B = cross(sub(x2, x1), sub(x4, x2));
    Vec3 C = cross(sub(x4, x3), sub(x3, x1));
    Vec3 D = cross(sub(x4, x3), sub(x4, x2));
    Vec3 n = mul(add(A, add(B, add(C, D))), .25);
    double length = vnorm(n);
    area = length;
    if (length < 1.0e-9) normal = {0, 0, 0};
    else normal = mul(n, 1.0 / length);
  }
  Vec3 point(double a, double b) const {
    double k0 = (1 - a) * (1 - b), k1 = a * (1 - b), k2 = (1 - a) * b, k3 = a * b;
    return {k0 * p0.x + k1 * p1.x + k2 * p2.x + k3 * p3.x, k0 * p0.y + k1 * p1.y + k2 * p2.y + k3 * p3.y,
            k0 * p0.z + k1 * p1.z + k2 * p2.z + k3 * p3.z};
  }
};

// TrilinearMap (meshgen/structured/TrilinearMap.java:17-146)
struct Trilinear {
  Vec3 x1, x2, x3, x4, x5, x6, x7, x8;
  Vec3 point(double a, double b, double c) const {
    auto f = [&](int d) {
      double v1 = comp(x1, d), v2 = comp(x2, d), v3 = comp(x3, d), v4 = comp(x4, d);
      double v5 = comp(x5, d), v6 = comp(x6, d), v7 = comp(x7, d), v8 = comp(x8, d);
      return c * (b * (a * v4 + (1 - a) * v3) + (1 - b) * (a * v2 + (1 - a) * v1)) +
             (1 - c) * (b * (a * v8 + (1 - a) * v7) + (1 - b) * (a * v6 + (1 - a) * v5));
    };
    return {f(1), f(2), f(3)};
  }
  double volume() const {
    // Multipole expansion with RS's signature rule and its running sign flip
    // of the accumulated sum after every permutation (:139-141).
    Vec3 r1 = x3, r2 = x4, r3 = x1, r4 = x2, r5 = x7, r6 = x8, r7 = x5, r8 = x6;
    Vec3 C[2][2][2];
    C[0][0][0] = r1;
    C[1][0][0] = sub(r2, r1);
    C[0][1][0] = sub(r3, r1);
    C[0][0][1] = sub(r5, r1);
    C[1][1][0] = sub(add(r4, r1), add(r3, r2));
    C[0][1][1] = sub(add(r7, r1), add(r5, r3));
    C[1][0][1] = sub(add(r6, r1), add(r5, r2));
    C[1][1][1] = sub(add(r8, add(r5, add(r3, r2))), add(r7, add(r6, add(r4, r1))));
    static const int perm[6][3] = {{1, 2, 3}, {1, 3, 2}, {2, 1, 3}, {2, 3, 1}, {3, 1, 2}, {3, 2, 1}};
    double volume = 0.0;
    for (int q = 0; q < 6; ++q) {
      int a = perm[q][0], b = perm[q][1], c = perm[q][2];
      for (int pb = 0; pb <= 1; pb++)
        for (int pc = 0; pc <= 1; pc++)
          for (int qa = 0; qa <= 1; qa++)
            for (int qc = 0; qc <= 1; qc++)
              for (int ra = 0; ra <= 1; ra++)
                for (int rb = 0; rb <= 1; rb++) {
                  double e = comp(C[1][pb][pc], a) * comp(C[qa][1][qc], b) * comp(C[ra][rb][1], c);
                  double d = (double)((qa + ra + 1) * (pb + rb + 1) * (pc + qc + 1));
                  volume += e / d;
                }
      // Permutation3.computeSignature (:165-174)
      int s = 0;
      for (int i = 0; i < 3; i++)
        for (int l = 0; l < i; l++)
          if (perm[q][l] > i) s += 1;
      double mult = (s % 2 == 0) ? 1.0 : -1.0;
      volume = mult * volume;
    }
    return volume;
  }
};

}  // namespace

Mesh build_structured_mesh(int dim, int ni, int nj, int nk, const double* coords, double x0, double y0, double z0,
                           double dx, double dy, double dz) {
  if (dim != 2 && dim != 3) throw Failure(ST_BAD_ARG, "dimension must be 2 or 3");
  if (ni <= 0 || nj <= 0 || (dim == 3 && nk <= 0)) throw Failure(ST_BAD_ARG, "grid sizes must be positive");
  if (dim == 2) nk = 0;
  Mesh m;
  m.dim = dim;
  m.ni = ni;
  m.nj = nj;
  m.nk = nk;
  const int npi = ni + 1, npj = nj + 1, npk = (dim == 3) ? nk + 1 : 1;
  const int nPoints = npi * npj * npk;
  const int nEl = (dim == 3) ? ni * nj * nk : ni * nj;
  const int nFace = (dim == 3) ? 6 : 4;
  const int nIntf = nEl * nFace;
  const int nConn = (dim == 3) ? 3 * ni * nj * nk - ni * nj - ni * nk - nj * nk : 2 * ni * nj - ni - nj;

  auto P = [&](int i, int j, int k) { return i + j * npi + k * npi * npj; };  // NaturalIJKOrdering points
  auto E = [&](int i, int j, int k) { return i + j * ni + k * ni * nj; };
  auto valid = [&](int i, int j, int k) {
    if (i < 0 || i > ni - 1) return false;
    if (j < 0 || j > nj - 1) return false;
    if (dim == 3) {
      if (k < 0 || k > nk - 1) return false;
    } else if (k != 0)
      return false;
    return true;
  };

  // geometry: points (StructuredGeometry{2D,3D}.java, ArrayData.getExpandedPoints)
  m.point.resize(nPoints);
  for (int k = 0; k < npk; ++k)
    for (int j = 0; j < npj; ++j)
      for (int i = 0; i < npi; ++i) {
        int p = P(i, j, k);
        if (coords) m.point[p] = {coords[3 * p], coords[3 * p + 1], coords[3 * p + 2]};
        else {
          double x = x0, y = y0, z = (dim == 3) ? z0 : 0.0;
          for (int a = 0; a < i; ++a) x += dx;
          for (int a = 0; a < j; ++a) y += dy;
          if (dim == 3)
            for (int a = 0; a < k; ++a) z += dz;
          m.point[p] = {x, y, z};
        }
      }

  // topology (CartesianTopology.construct + Topology.build*)
  std::vector<OrderedSet> pI(nPoints), pE(nPoints), iP(nIntf), eP(nEl), eI(nEl);
  m.interfaceElement.assign(nIntf, -1);
  m.interfaceConnection.assign(nIntf, -1);
  m.iboundary.assign(nIntf, 1);

  // element corner points (CartesianTopology3D.getElementPoints :219-237 / 2D :172-183)
  auto elemPoints = [&](int i, int j, int k, int* cp) {
    if (dim == 3) {
      cp[0] = P(i, j, k);
      cp[1] = cp[0] + 1;
      cp[2] = P(i, j + 1, k) + 1;
      cp[3] = cp[2] - 1;
      cp[4] = P(i, j, k + 1);
      cp[5] = cp[4] + 1;
      cp[6] = P(i, j + 1, k + 1) + 1;
      cp[7] = cp[6] - 1;
    } else {
      cp[0] = P(i, j, 0);
      cp[1] = cp[0] + 1;
      cp[2] = P(i, j + 1, 0) + 1;
      cp[3] = cp[2] - 1;
    }
  };
  // interface points per orientation (3D :267-286 TOP,BOTTOM,FRONT,BACK,LEFT,RIGHT;
  // 2D :213-228 FRONT,BACK,LEFT,RIGHT)
  auto intfPoints = [&](const int* cp, int o, int* ip) -> int {
    if (dim == 3) {
      static const int tab[6][4] = {{0, 1, 2, 3}, {7, 6, 5, 4}, {4, 5, 1, 0}, {6, 7, 3, 2}, {7, 4, 0, 3}, {5, 6, 2, 1}};
      for (int a = 0; a < 4; ++a) ip[a] = cp[tab[o][a]];
      return 4;
    }
    static const int tab2[4][2] = {{1, 0}, {3, 2}, {0, 3}, {2, 1}};
    ip[0] = cp[tab2[o][0]];
    ip[1] = cp[tab2[o][1]];
    return 2;
  };

  // element iteration order of NaturalIJKOrdering.getIJK: i outer, then j, then k
  const int kmax = (dim == 3) ? nk : 1;
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < kmax; ++k) {
        int e = E(i, j, k);
        int cp[8];
        elemPoints(i, j, k, cp);
        for (int o = 0; o < nFace; ++o) {
          int f = e * nFace + o;
          int ip[4];
          int np = intfPoints(cp, o, ip);
          for (int a = 0; a < np; ++a) {
            iP[f].add(ip[a]);
            pI[ip[a]].add(f);
          }
        }
        for (int o = 0; o < nFace; ++o) {
          int f = e * nFace + o;
          eI[e].add(f);
          m.interfaceElement[f] = e;
          for (int p : iP[f].v) {
            eP[e].add(p);
            pE[p].add(e);
          }
        }
      }

  // neighbour connections (forward orientations: 3D BOTTOM,BACK,RIGHT; 2D BACK,RIGHT)
  m.connHereIntf.assign(nConn, -1);
  m.connThereIntf.assign(nConn, -1);
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < kmax; ++k) {
        int e = E(i, j, k);
        if (dim == 3) {
          // BOTTOM (local 1) -> neighbour (i,j,k+1) TOP (0)
          if (valid(i, j, k + 1)) {
            int c = i + j * ni + k * ni * nj;
            m.connHereIntf[c] = e * 6 + 1;
            m.connThereIntf[c] = E(i, j, k + 1) * 6 + 0;
          }
          // BACK (3) -> (i,j+1,k) FRONT (2)
          if (valid(i, j + 1, k)) {
            int c = i + j * ni + k * ni * (nj - 1) + ni * nj * (nk - 1);
            m.connHereIntf[c] = e * 6 + 3;
            m.connThereIntf[c] = E(i, j + 1, k) * 6 + 2;
          }
          // RIGHT (5) -> (i+1,j,k) LEFT (4)
          if (valid(i + 1, j, k)) {
            int c = i + j * (ni - 1) + k * (ni - 1) * nj + ni * (nj - 1) * nk + ni * nj * (nk - 1);
            m.connHereIntf[c] = e * 6 + 5;
            m.connThereIntf[c] = E(i + 1, j, k) * 6 + 4;
          }
        } else {
          // BACK (1) -> (i,j+1) FRONT (0)
          if (valid(i, j + 1, 0)) {
            int c = i + j * ni;
            m.connHereIntf[c] = e * 4 + 1;
            m.connThereIntf[c] = E(i, j + 1, 0) * 4 + 0;
          }
          // RIGHT (3) -> (i+1,j) LEFT (2)
          if (valid(i + 1, j, 0)) {
            int c = i + j * (ni - 1) + ni * (nj - 1);
            m.connHereIntf[c] = e * 4 + 3;
            m.connThereIntf[c] = E(i + 1, j, 0) * 4 + 2;
          }
        }
      }
  m.connHere.resize(nConn);
  m.connThere.resize(nConn);
  m.connMult.assign(nConn, 1.0);
  for (int c = 0; c < nConn; ++c) {
    if (m.connHereIntf[c] < 0) throw Failure(ST_BAD_ARG, "connection numbering incomplete");
    m.interfaceConnection[m.connHereIntf[c]] = c;
    m.interfaceConnection[m.connThereIntf[c]] = c;
    m.iboundary[m.connHereIntf[c]] = 0;
    m.iboundary[m.connThereIntf[c]] = 0;
    m.connHere[c] = m.interfaceElement[m.connHereIntf[c]];
    m.connThere[c] = m.interfaceElement[m.connThereIntf[c]];
  }

  m.pointInterfaces.resize(nPoints);
  m.pointElements.resize(nPoints);
  for (int p = 0; p < nPoints; ++p) {
    m.pointInterfaces[p] = pI[p].v;
    m.pointElements[p] = pE[p].v;
  }
  m.interfacePoints.resize(nIntf);
  for (int f = 0; f < nIntf; ++f) m.interfacePoints[f] = iP[f].v;
  m.elementPoints.resize(nEl);
  m.elementInterfaces.resize(nEl);
  for (int e = 0; e < nEl; ++e) {
    m.elementPoints[e] = eP[e].v;
    m.elementInterfaces[e] = eI[e].v;
  }

  // element and interface geometry
  m.ecenter.resize(nEl);
  m.evolume.resize(nEl);
  m.inormal.resize(nIntf);
  m.icenter.resize(nIntf);
  m.iarea.resize(nIntf);
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < kmax; ++k) {
        int e = E(i, j, k);
        int cp[8];
        elemPoints(i, j, k, cp);
        if (dim == 3) {
          // HexCell.java:26-51
          const Vec3* g = m.point.data();
          Vec3 p0 = g[cp[0]], p1 = g[cp[1]], p2 = g[cp[3]], p3 = g[cp[2]];
          Vec3 p4 = g[cp[4]], p5 = g[cp[5]], p6 = g[cp[7]], p7 = g[cp[6]];
          Trilinear t{p0, p1, p2, p3, p4, p5, p6, p7};
          m.evolume[e] = t.volume();
          m.ecenter[e] = t.point(0.5, 0.5, 0.5);
          Bilinear faces[6] = {Bilinear(p0, p1, p2, p3), Bilinear(p4, p5, p6, p7), Bilinear(p0, p1, p4, p5),
                               Bilinear(p2, p3, p6, p7), Bilinear(p0, p2, p4, p6), Bilinear(p1, p3, p5, p7)};
          static const double scale[6] = {1.0, -1.0, -1.0, 1.0, 1.0, -1.0};
          for (int o = 0; o < 6; ++o) {
            int f = e * 6 + o;
            m.iarea[f] = faces[o].area;
            m.icenter[f] = faces[o].point(.5, .5);
            m.inormal[f] = mul(faces[o].normal, scale[o]);
          }
        } else {
          // QuadCell.java:27-95
          const Vec3* g = m.point.data();
          Vec3 p0 = g[cp[0]], p1 = g[cp[1]], p2 = g[cp[2]], p3 = g[cp[3]];
          Bilinear b(p0, p1, p3, p2);
          m.ecenter[e] = b.point(.5, .5);
          m.evolume[e] = b.area;
          Vec3 ends[4][2] = {{p0, p1}, {p2, p3}, {p3, p0}, {p1, p2}};
          for (int o = 0; o < 4; ++o) {
            int f = e * 4 + o;
            Vec3 a = ends[o][0], c = ends[o][1];
            double x = c.x - a.x, y = c.y - a.y;
            Vec3 n{y, -x, 0};
            n = mul(n, 1 / vnorm(n));
            m.inormal[f] = n;
            m.iarea[f] = vnorm(sub(c, a));
            m.icenter[f] = mul(add(a, c), 0.5);
          }
        }
      }

  m.K6.assign((size_t)6 * nEl, 0.0);
  m.MD.assign(nConn, {});
  return m;
}

void test_mesh(const Mesh& m) {
  // geometry/Mesh.java:620-660
  for (size_t f = 0; f < m.iarea.size(); ++f) {
    if (std::fabs(1.0 - vnorm(m.inormal[f])) > 1.0e-6) throw Failure(ST_BAD_ARG, "Normal should have unit length");
    Vec3 ei = sub(m.icenter[f], m.ecenter[m.interfaceElement[f]]);
    Vec3 en = add(ei, mul(m.inormal[f], 1.0e-6));
    if (vnorm(en) <= vnorm(ei)) throw Failure(ST_BAD_ARG, "Normal does not point outwards");
  }
  for (int c = 0; c < m.numConnections(); ++c) {
    int a = m.connHereIntf[c], b = m.connThereIntf[c];
    if (!(std::fabs(m.iarea[a] - m.iarea[b]) < 1.0e-9))
      throw Failure(ST_BAD_ARG, "Neighbouring interfaces should have same area");
    if (vdot(m.inormal[a], m.inormal[b]) >= 0)
      throw Failure(ST_BAD_ARG, "Neighbouring interfaces must have opposite normals");
  }
}

// ----------------------------------------------------------------- MPFA ----
namespace {

// Tensor3D.mult (geometry/Tensor3D.java:62-68)
inline Vec3 kmult(const double* K, const Vec3& v) {
  double xx = K[0], yy = K[1], zz = K[2], xy = K[3], xz = K[4], yz = K[5];
  return {xx * v.x + xy * v.y + xz * v.z, xy * v.x + yy * v.y + yz * v.z, xz * v.x + yz * v.y + zz * v.z};
}

// MPFA.calculateNormalArea (geometry/flux/MPFA.java:314-354)
Vec3 normal_area(const Mesh& m, int intf, int p) {
  const auto& pts = m.interfacePoints[intf];
  int n = (int)pts.size();
  if (n == 2) return mul(m.inormal[intf], -m.iarea[intf] / 2);
  if (n == 3) return mul(m.inormal[intf], -m.iarea[intf] / 3);
  if (n > 4) throw Failure(ST_UNSUPPORTED, "general polygon interfaces are not used by structured meshes");
  int i = 0;
  for (int q : pts)
    if (q == p) break;
    else i++;
  Vec3 x1 = m.point[pts[i]];
  Vec3 x2 = m.point[pts[i == 0 ? 3 : (i - 1) % 4]];
  Vec3 x3 = m.point[pts[(i + 1) % 4]];
  Vec3 x4 = m.point[pts[(i + 2) % 4]];
  Vec3 v21 = sub(x2, x1), v31 = sub(x3, x1), v42 = sub(x4, x2), v43 = sub(x4, x3);
  Vec3 n1 = mul(cross(v21, v31), 9);
  Vec3 n2 = mul(cross(v21, v42), 3);
  Vec3 n3 = mul(cross(v43, v31), 3);
  Vec3 n4 = cross(v43, v42);
  return mul(add(add(add(n1, n2), n3), n4), 1. / 64.);
}

int neighbour_interface(const Mesh& m, int intf) {
  int c = m.interfaceConnection[intf];
  return m.connHereIntf[c] == intf ? m.connThereIntf[c] : m.connHereIntf[c];
}

}  // namespace

static void finish_md(Mesh& m, std::vector<std::vector<MDEntry>>& M);

void compute_mpfa_o(Mesh& m, double continuity) {
  if (continuity > 1 || continuity <= 0) throw Failure(ST_BAD_ARG, "continuity must be in (0,1]");
  std::vector<std::vector<MDEntry>> M(m.numConnections());
  std::vector<double> A, B, C, D, AiB, T, Aloc;
  std::vector<int> ipiv;
  for (int p = 0; p < m.numPoints(); ++p) {
    const auto& pints = m.pointInterfaces[p];
    const auto& pels = m.pointElements[p];
    // OmethodInteractionRegion (O_MPFA.java:131-167)
    std::unordered_map<int, int> elMap, intfMap;
    for (size_t a = 0; a < pels.size(); ++a) elMap[pels[a]] = (int)a;
    int numConnections = 0;
    for (int f : pints) {
      if (!m.iboundary[f] && intfMap.count(neighbour_interface(m, f))) intfMap[f] = intfMap[neighbour_interface(m, f)];
      else intfMap[f] = numConnections++;
    }
    const int nc = numConnections, ne = (int)pels.size();
    A.assign((size_t)nc * nc, 0.0);
    B.assign((size_t)nc * ne, 0.0);
    C.assign((size_t)nc * nc, 0.0);
    D.assign((size_t)nc * ne, 0.0);
    // calculateT (O_MPFA.java:193-239)
    for (int el : pels) {
      std::vector<int> inter;
      for (int f : pints)
        for (int g : m.elementInterfaces[el])
          if (f == g) inter.push_back(f);
      const int ni = (int)inter.size();
      if (ni != 2 && ni != 3) throw Failure(ST_BAD_ARG, "Interaction region has too many interfaces");
      const int n = ni + 1;
      // calculateBasisFunctions2D/3D (:271-401): solve A * Psi = I by dgesv
      double Ab[16] = {0}, Psi[16] = {0};
      int piv[4];
      const Vec3 ec = m.ecenter[el];
      Ab[0 + 0 * n] = 1;
      Ab[0 + 1 * n] = ec.x;
      Ab[0 + 2 * n] = ec.y;
      if (n == 4) Ab[0 + 3 * n] = ec.z;
      for (int i = 0; i < ni; ++i) {
        Vec3 cp = m.icenter[inter[i]];
        if (continuity != 1) {
          Vec3 corner = m.point[p];
          cp = {(cp.x - corner.x) * continuity + corner.x, (cp.y - corner.y) * continuity + corner.y,
                (cp.z - corner.z) * continuity + corner.z};
        }
        Ab[(i + 1) + 0 * n] = 1;
        Ab[(i + 1) + 1 * n] = cp.x;
        Ab[(i + 1) + 2 * n] = cp.y;
        if (n == 4) Ab[(i + 1) + 3 * n] = cp.z;
      }
      for (int i = 0; i < n; ++i) Psi[i + i * n] = 1;
      if (dgesv(n, n, Ab, n, piv, Psi, n) != 0) throw Failure(ST_SINGULAR, "Severe grid distortion at element");
      Vec3 grad[4];
      for (int i = 0; i < n; ++i) grad[i] = {Psi[1 + i * n], Psi[2 + i * n], n == 4 ? Psi[3 + i * n] : 0.0};
      // calculateLocalConductivityDirections (MPFA.java:109-120)
      Vec3 Kn[3];
      for (int i = 0; i < ni; ++i) Kn[i] = kmult(&m.K6[6 * (size_t)el], normal_area(m, inter[i], p));
      // assembleElementContribution (O_MPFA.java:422-457)
      for (int i = 0; i < ni; ++i) {
        double f = vdot(Kn[i], grad[0]);
        int intf = inter[i];
        int is = intfMap[intf];
        int ei = elMap[m.interfaceElement[intf]];
        bool isHere = m.iboundary[intf] ? true : (intf == m.connHereIntf[m.interfaceConnection[intf]]);
        B[is + (size_t)ei * nc] += -f;
        if (isHere) D[is + (size_t)ei * nc] += -f;
        for (int j = 1; j < ni + 1; j++) {
          f = vdot(Kn[i], grad[j]);
          int js = intfMap[inter[j - 1]];
          A[is + (size_t)js * nc] += f;
          if (isHere) C[is + (size_t)js * nc] += f;
        }
      }
    }
    // MPFA.calculateTmatrix (MPFA.java:43-54): T = C * (A \ B) - D
    AiB = B;
    Aloc = A;
    ipiv.assign(nc, 0);
    if (dgesv(nc, ne, Aloc.data(), nc, ipiv.data(), AiB.data(), nc) != 0)
      throw Failure(ST_SINGULAR, "Conductivity tensor does not appear to be symmetrical, positive definite");
    T.assign((size_t)nc * ne, 0.0);
    for (size_t a = 0; a < T.size(); ++a) T[a] = D[a] * -1;
    dgemm_nn_add(nc, ne, nc, C.data(), nc, AiB.data(), nc, T.data(), nc);
    // storeTransmissibilities for each neighbour connection at p (O_MPFA.java:88-112)
    std::set<int> conns;
    for (int f : pints)
      if (!m.iboundary[f]) conns.insert(m.interfaceConnection[f]);
    for (int c : conns) {
      int i = intfMap[m.connHereIntf[c]];
      auto& Mi = M[c];
      for (int el : pels) {
        int j = elMap[el];
        double tk = T[i + (size_t)j * nc];
        bool found = false;
        for (auto& tp : Mi)
          if (tp.element == el) {
            found = true;
            tp.k += tk;
            break;
          }
        if (!found && tk != 0) Mi.push_back({el, tk});
      }
    }
  }
  finish_md(m, M);
}

// Connection.setDarcyTransmissibilities / check (geometry/Connection.java:61-107)
static void finish_md(Mesh& m, std::vector<std::vector<MDEntry>>& M) {
  for (int c = 0; c < m.numConnections(); ++c) {
    double sum = 0;
    bool hasHere = false, hasThere = false;
    std::set<int> seen;
    for (auto& t : M[c]) {
      sum += t.k;
      if (!seen.insert(t.element).second) throw Failure(ST_BAD_ARG, "Duplicate transmissibility over connection");
      hasHere |= t.element == m.connHere[c];
      hasThere |= t.element == m.connThere[c];
    }
    if (std::fabs(sum) > 1.0e-6) throw Failure(ST_BAD_ARG, "Transmissibilities on connection do not sum to zero");
    if (!hasHere || !hasThere) throw Failure(ST_BAD_ARG, "Transmissibilities do not include both sides");
    for (auto& t : M[c]) t.k *= m.connMult[c];
  }
  m.MD = std::move(M);
}

namespace {

// MPFA.getHalfEdgePoints (geometry/flux/MPFA.java:165-201): the midpoints of
// the two edges of interface intf at corner point p, next one first
void half_edge_points(const Mesh& m, int p, int intf, Vec3& cp1, Vec3& cp2) {
  const auto& pts = m.interfacePoints[intf];
  const int n = (int)pts.size();
  int i = 0;
  while (i < n && pts[i] != p) ++i;
  const int j = (i + 1) % n, k = i == 0 ? n - 1 : i - 1;
  const Vec3 c1 = m.point[p], c2 = m.point[pts[j]], c3 = m.point[pts[k]];
  cp1 = mul(add(c1, c2), 0.5);
  cp2 = mul(add(c1, c3), 0.5);
}

// MPFA.computeSubFaceArea (geometry/flux/MPFA.java:131-160)
double sub_face_area(const Mesh& m, int intf, int p) {
  Vec3 c, d;
  half_edge_points(m, p, intf, c, d);
  const Vec3 a = m.icenter[intf], b = m.point[p];
  const Vec3 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a);
  const double A1 = 0.5 * vnorm(cross(ab, ac));
  const double A2 = 0.5 * vnorm(cross(ab, ad));
  return A1 + A2;
}

// A linear function c1 + c2 x + c3 y + c4 z through four points (one basis
// function per point, the columns of A^-1; L_MPFA.java:406-447, 659-758)
struct Basis4 {
  double c[4][4];  // c[i] = (c1, c2, c3, c4) of basis function i
  Vec3 grad(int i) const { return {c[i][1], c[i][2], c[i][3]}; }
  double psi(int i, const Vec3& q) const { return c[i][0] + c[i][1] * q.x + c[i][2] * q.y + c[i][3] * q.z; }
};

Basis4 basis4(const Vec3* q) {
  double Ab[16] = {0}, Psi[16] = {0};
  int piv[4];
  for (int r = 0; r < 4; ++r) {
    Ab[r + 0 * 4] = 1;
    Ab[r + 1 * 4] = q[r].x;
    Ab[r + 2 * 4] = q[r].y;
    Ab[r + 3 * 4] = q[r].z;
  }
  for (int i = 0; i < 4; ++i) Psi[i + i * 4] = 1;
  if (dgesv(4, 4, Ab, 4, piv, Psi, 4) != 0) throw Failure(ST_SINGULAR, "Error computing basis functions");
  Basis4 b;
  for (int i = 0; i < 4; ++i)
    for (int r = 0; r < 4; ++r) b.c[i][r] = Psi[r + i * 4];
  return b;
}

// LmethodInteractionRegion(p, primary) and calculateT (L_MPFA.java:495-657,
// 760-866): T (3 x 4, column major) over the region's elements, primary
// first, then the neighbours across the primary's three interfaces at p, in
// their order.  prim: the primary's interfaces at p.
void l_region_T(const Mesh& m, int p, int primary, const std::vector<int>& prim, int* els, double* T) {
  double A[9] = {0}, B[12] = {0}, C[9] = {0}, D[12] = {0};
  els[0] = primary;
  int sec_intf[3];
  for (int i = 0; i < 3; ++i) {
    sec_intf[i] = neighbour_interface(m, prim[i]);
    els[i + 1] = m.interfaceElement[sec_intf[i]];
  }
  // primary element: basis through its centre and its three interface centres
  Vec3 q[4] = {m.ecenter[primary], m.icenter[prim[0]], m.icenter[prim[1]], m.icenter[prim[2]]};
  const Basis4 pp = basis4(q);
  for (int i = 0; i < 3; ++i) {
    const Vec3 kn = kmult(&m.K6[6 * (size_t)primary], normal_area(m, prim[i], p));
    double f = vdot(kn, pp.grad(0));
    B[i + 0 * 3] += -f;
    for (int j = 1; j < 4; ++j) {
      f = vdot(kn, pp.grad(j));
      A[i + (j - 1) * 3] += f;
    }
  }
  // secondary elements: basis through the centre, the interface centre, the
  // corner point and the interface's first half-edge point
  for (int i = 0; i < 3; ++i) {
    const int el = els[i + 1], jntf = sec_intf[i];
    Vec3 e1, e2;
    half_edge_points(m, p, jntf, e1, e2);
    Vec3 qs[4] = {m.ecenter[el], m.icenter[jntf], m.point[p], e1};
    const Basis4 ps = basis4(qs);
    const Vec3 kn = kmult(&m.K6[6 * (size_t)el], normal_area(m, jntf, p));
    double f = vdot(kn, ps.grad(0));
    B[i + (i + 1) * 3] += -f;
    D[i + (i + 1) * 3] += -f;
    f = vdot(kn, ps.grad(1));
    A[i + i * 3] += f;
    C[i + i * 3] += f;
    // assembleFullPotentialContribution at the corner point, then the edge point
    const Vec3 at[2] = {m.point[p], e1};
    for (int w = 0; w < 2; ++w) {
      f = vdot(kn, ps.grad(2 + w));
      double psik = pp.psi(0, at[w]);
      B[i + 0 * 3] += -f * psik;
      D[i + 0 * 3] += -f * psik;
      for (int k = 1; k < 4; ++k) {
        psik = pp.psi(k, at[w]);
        A[i + (k - 1) * 3] += f * psik;
        C[i + (k - 1) * 3] += f * psik;
      }
    }
  }
  // MPFA.calculateTmatrix: T = C (A \ B) - D
  double AiB[12];
  int piv[3];
  for (int a = 0; a < 12; ++a) AiB[a] = B[a];
  if (dgesv(3, 4, A, 3, piv, AiB, 3) != 0)
    throw Failure(ST_SINGULAR, "Conductivity tensor does not appear to be symmetrical, positive definite");
  for (int a = 0; a < 12; ++a) T[a] = D[a] * -1;
  dgemm_nn_add(3, 4, 3, C, 3, AiB, 3, T, 3);
}

void md_add(std::vector<MDEntry>& Mi, int el, double tk, bool keep_zero) {
  for (auto& tp : Mi)
    if (tp.element == el) {
      tp.k += tk;
      return;
    }
  if (tk != 0 || keep_zero) Mi.push_back({el, tk});
}

}  // namespace

// L_MPFA.calculateTransmissibilities (geometry/flux/L_MPFA.java:52-74) on
// 3-D hexahedral meshes.  The reference iterates a point's connections and a
// region's elements through hash sets, whose order Java leaves open; here
// connections go in ascending index and a region's elements primary first,
// which fixes the order of each MD list (the values do not depend on it).
void compute_mpfa_l(Mesh& m) {
  if (m.dim != 3) throw Failure(ST_UNSUPPORTED, "the L-method is built for 3-D hexahedral meshes");
  std::vector<std::vector<MDEntry>> M(m.numConnections());
  for (int p = 0; p < m.numPoints(); ++p) {
    const auto& pints = m.pointInterfaces[p];
    bool onBoundary = false;
    std::set<int> conns;
    for (int f : pints) {
      if (m.iboundary[f]) onBoundary = true;
      else conns.insert(m.interfaceConnection[f]);
    }
    if (onBoundary) {
      // calculateBoundaryTransmissibilities (:77-126): two-point fluxes over
      // the sub-faces at p, with TPFA's distance weighting
      for (int c : conns) {
        const int is = m.connHereIntf[c], js = m.connThereIntf[c];
        const int ei = m.interfaceElement[is], ej = m.interfaceElement[js];
        const Vec3 ki = kmult(&m.K6[6 * (size_t)ei], m.inormal[is]);
        const Vec3 kj = kmult(&m.K6[6 * (size_t)ej], m.inormal[js]);
        const double Kin = std::sqrt(ki.x * ki.x + ki.y * ki.y + ki.z * ki.z);
        const double Kjn = std::sqrt(kj.x * kj.x + kj.y * kj.y + kj.z * kj.z);
        const double A = sub_face_area(m, is, p);
        double t = 0;
        if (Kin != 0 && Kjn != 0)
          t = Kin * Kjn * A /
              (Kjn * vnorm(sub(m.icenter[is], m.ecenter[ei])) + Kjn * vnorm(sub(m.icenter[js], m.ecenter[ej])));
        md_add(M[c], m.connHere[c], t, false);
        md_add(M[c], m.connThere[c], -t, false);
      }
      continue;
    }
    // getElementInterfaces: each element's interfaces at p, in p's order
    std::map<int, std::vector<int>> elIntf;
    for (int el : m.pointElements[p]) elIntf[el];
    for (int f : pints) elIntf[m.interfaceElement[f]].push_back(f);
    for (int c : conns) {
      const int here = m.connHere[c], there = m.connThere[c], hi = m.connHereIntf[c];
      const int nuHere = (int)elIntf[here].size(), nuThere = (int)elIntf[there].size();
      int prim[2], np = 0;
      if (nuHere == 3) prim[np++] = here;
      if (nuThere == 3) prim[np++] = there;
      if (np == 0) throw Failure(ST_BAD_ARG, "Illegal local vertex degree for point");
      int els[2][4], row[2];
      double T[2][12];
      for (int r = 0; r < np; ++r) {
        const auto& pi = elIntf[prim[r]];
        l_region_T(m, p, prim[r], pi, els[r], T[r]);
        // the row of c's here interface: the primary's interface or its neighbour
        row[r] = -1;
        for (int i = 0; i < 3; ++i)
          if (pi[i] == hi || neighbour_interface(m, pi[i]) == hi) row[r] = i;
      }
      // chooseTransmissibilities (:170-212): the smaller |t| of the primary's
      // coefficient on c's sub-face; the second candidate on a tie
      int pick = 0;
      if (np == 2) pick = std::fabs(T[0][row[0]]) < std::fabs(T[1][row[1]]) ? 0 : 1;
      // storeLTransmissibilities (:218-249)
      for (int j = 0; j < 4; ++j) {
        const int el = els[pick][j];
        double tk = T[pick][row[pick] + j * 3];
        if (prim[pick] == here) tk *= -1;
        md_add(M[c], el, tk, el == here || el == there);
      }
    }
  }
  finish_md(m, M);
}

void compute_tpfa(Mesh& m) {
  auto multNorm = [](const double* K, const Vec3& v) {
    Vec3 r = kmult(K, v);
    return std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
  };
  m.MD.assign(m.numConnections(), {});
  for (int c = 0; c < m.numConnections(); ++c) {
    int is = m.connHereIntf[c], js = m.connThereIntf[c];
    int ei = m.interfaceElement[is], ej = m.interfaceElement[js];
    double Kin = multNorm(&m.K6[6 * (size_t)ei], m.inormal[is]);
    double Kjn = multNorm(&m.K6[6 * (size_t)ej], m.inormal[js]);
    double A = m.iarea[is];
    double t = 0;
    if (Kin != 0 && Kjn != 0)
      t = Kin * Kjn * A / (Kjn * vnorm(sub(m.icenter[is], m.ecenter[ei])) + Kjn * vnorm(sub(m.icenter[js], m.ecenter[ej])));
    m.MD[c] = {{m.connHere[c], t * m.connMult[c]}, {m.connThere[c], -t * m.connMult[c]}};
  }
}

static CompRowMatrix pattern_impl(const Mesh& m, bool diag) {
  const int n = m.numElements();
  std::vector<std::set<int>> nz(n);
  if (diag)
    for (int e = 0; e < n; ++e) nz[e].insert(e);
  for (int c = 0; c < m.numConnections(); ++c)
    for (auto& t : m.MD[c]) {
      nz[m.connHere[c]].insert(t.element);
      nz[m.connThere[c]].insert(t.element);
    }
  std::vector<std::vector<int>> rows(n);
  for (int e = 0; e < n; ++e) rows[e].assign(nz[e].begin(), nz[e].end());
  return CompRowMatrix::from_rows(n, rows);
}

CompRowMatrix pressure_pattern(const Mesh& m) { return pattern_impl(m, true); }
CompRowMatrix potential_pattern(const Mesh& m) { return pattern_impl(m, false); }

}  // namespace orc
