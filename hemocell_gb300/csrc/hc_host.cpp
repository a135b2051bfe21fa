// Host-side precompute: meshes, rest-state constants, units, placement, packing.
#include "hc_host.h"

#include <algorithm>
#include <fstream>
#include <sstream>
#include <iterator>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>

namespace hcg {
namespace {

inline Vec3 sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 add(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 mul(Vec3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline Vec3 divv(Vec3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline Vec3 crs(Vec3 a, Vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dt3(Vec3 a, Vec3 b) {
  double r = 0;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
inline double nrm(Vec3 a) { return std::sqrt(dt3(a, a)); }
inline Vec3 unit_normal(Vec3 a, Vec3 b, Vec3 c) {
  Vec3 n = crs(sub(b, a), sub(c, a));
  double l = nrm(n);
  return l != 0 ? divv(n, l) : Vec3{0, 0, 0};
}

typedef std::array<Vec3, 3> Tri;

// Triangle soup of the refined icosahedron.  The 12 vertices and 20 faces
// are the reference's table (helper/meshGeneratingFunctions.hh:43-102), kept
// identical so the refinement yields the same soup; refinement replaces each
// face by its middle triangle and appends the three corner triangles
// (:108-141), with midpoints projected back onto the unit sphere.
std::vector<Tri> icosphere_soup(int min_triangles) {
  const double a = -0.8506508084, b = -0.5257311121;
  const Vec3 P[12] = {{a, b, 0},  {-a, b, 0}, {-a, -b, 0}, {a, -b, 0}, {b, 0, a},  {b, 0, -a},
                      {-b, 0, -a}, {-b, 0, a}, {0, a, b},   {0, -a, b}, {0, -a, -b}, {0, a, -b}};
  // 1-based corner indices of the 20 faces
  static const int F[20][3] = {{5, 8, 9},  {5, 10, 8}, {6, 12, 7}, {6, 7, 11}, {1, 4, 5},
                               {1, 6, 4},  {3, 2, 8},  {3, 7, 2},  {9, 12, 1}, {9, 2, 12},
                               {10, 4, 11}, {10, 11, 3}, {9, 1, 5}, {12, 6, 1}, {5, 4, 10},
                               {6, 11, 4}, {8, 2, 9},  {7, 12, 2}, {8, 10, 3}, {7, 3, 11}};
  std::vector<Tri> soup;
  for (const auto& f : F) soup.push_back({P[f[0] - 1], P[f[1] - 1], P[f[2] - 1]});
  auto mid = [](Vec3 p, Vec3 q) {
    Vec3 m = mul(add(p, q), 0.5);
    return divv(m, nrm(m));
  };
  size_t size;
  while ((int)(size = soup.size()) < min_triangles) {
    for (size_t i = 0; i < size; ++i) {
      const Vec3 va = soup[i][0], vb = soup[i][1], vc = soup[i][2];
      const Vec3 vd = mid(va, vb), ve = mid(vb, vc), vf = mid(vc, va);
      soup[i] = {vd, ve, vf};
      soup.push_back({va, vd, vf});
      soup.push_back({vd, vb, ve});
      soup.push_back({vf, ve, vc});
    }
  }
  return soup;
}

// Merge bit-identical corners, numbering vertices by first appearance.
Mesh merge_soup(const std::vector<Tri>& soup) {
  Mesh m;
  std::map<std::array<uint64_t, 3>, int> id;
  for (const Tri& t : soup) {
    std::array<int, 3> tri;
    for (int c = 0; c < 3; ++c) {
      std::array<uint64_t, 3> key;
      std::memcpy(&key[0], &t[c].x, 8);
      std::memcpy(&key[1], &t[c].y, 8);
      std::memcpy(&key[2], &t[c].z, 8);
      auto it = id.find(key);
      if (it == id.end()) {
        it = id.emplace(key, (int)m.v.size()).first;
        m.v.push_back(t[c]);
      }
      tri[c] = it->second;
    }
    m.t.push_back(tri);
  }
  return m;
}

inline int sgn(double v) { return (0.0 < v) - (v < 0.0); }

}  // namespace

Units derive_units(double dx, double dt, double nu_p, double rho_p, double kBT_p, double tau_override) {
  Units u;
  if (tau_override > 0) {
    u.tau = tau_override;
    u.nu_lbm = 1.0 / 3.0 * (u.tau - 0.5);
  } else {
    u.nu_lbm = nu_p * dt / (dx * dx);
    u.tau = 3.0 * u.nu_lbm + 0.5;
  }
  u.dm = rho_p * (dx * dx * dx);
  u.df = u.dm * dx / (dt * dt);
  u.kBT_lbm = kBT_p / (u.df * dx);
  u.f_limit = 50.0 / 1.0e12 / u.df;  // FORCE_LIMIT 50 pN, config/constant_defaults.h:73-75
  return u;
}

ModelK scale_material(int model, int nfaces, const Units& u, double dx, double dt, const double* mat) {
  ModelK k;
  const double plc = 7.5e-9 / dx;  // persistence length
  const double eqL = 5e-7 / dx;
  const double nfs = 1280.0 / nfaces;
  k.k_link = mat[0] * u.kBT_lbm / plc;
  k.k_bend = mat[1] * u.kBT_lbm / eqL;
  k.k_volume = mat[2] * nfs * u.kBT_lbm / eqL;
  k.k_area = mat[3] * nfs * u.kBT_lbm / eqL;
  k.eta_m = mat[4] * dx / dt / u.df;
  const bool wbc = model == 2;
  k.k_inner_rigid = wbc ? mat[5] / u.df : 0.0;
  k.k_cyto = wbc ? mat[6] / u.df : 0.0;
  k.core_radius = wbc ? mat[7] / dx : 0.0;
  k.radius = wbc ? mat[8] / dx : 0.0;
  return k;
}

Mesh icosphere(int min_triangles, double radius) {
  Mesh m = merge_soup(icosphere_soup(min_triangles));
  for (Vec3& p : m.v) p = mul(p, radius);
  return m;
}

// The shape constructors' fixed rotation TriangleSet::rotate(pi/2 + a0,
// pi/2 + a1, a2) with a0 = a1 = a2 = 0 (HemoCellField passes zero Euler
// angles, core/hemoCellField.cpp:59-66; helper/meshGeneratingFunctions.hh:223-238).
// The Euler angles are read in the "x-convention" (rotation by phi about z,
// theta about the new x, psi about the new z) and applied to point
// coordinates as p' = A p with Goldstein's matrix A = B(psi) C(theta) D(phi).
// With (pi/2, pi/2, 0) it takes (x, y, z) to (y, z, x) up to cos(pi/2)
// rounding: the biconcave disc's axis ends on y, which the reference's
// stretch validation relies on (its cell is placed with angles (90, 0, 0)
// and measured across x and y, tests/validation/stretch_cell).
struct Euler {
  double a[3][3];
  Euler(double phi, double theta, double psi) {
    const double cf = std::cos(phi), sf = std::sin(phi), ct = std::cos(theta), st = std::sin(theta);
    const double cp = std::cos(psi), sp = std::sin(psi);
    a[0][0] = cp * cf - ct * sf * sp;
    a[0][1] = cp * sf + ct * cf * sp;
    a[0][2] = sp * st;
    a[1][0] = -sp * cf - ct * sf * cp;
    a[1][1] = -sp * sf + ct * cf * cp;
    a[1][2] = cp * st;
    a[2][0] = st * sf;
    a[2][1] = -st * cf;
    a[2][2] = ct;
  }
  Vec3 operator()(Vec3 p) const {
    return {a[0][0] * p.x + a[0][1] * p.y + a[0][2] * p.z, a[1][0] * p.x + a[1][1] * p.y + a[1][2] * p.z,
            a[2][0] * p.x + a[2][1] * p.y + a[2][2] * p.z};
  }
};
const Euler& shape_rotation() {
  static const Euler R(M_PI / 2.0, M_PI / 2.0, 0.0);
  return R;
}

// RBC_FROM_SPHERE (helper/meshGeneratingFunctions.hh:153-168, :213-241): the
// unit icosphere rotated, spherePointToRBCPoint with R = 1, scale(radius),
// the same rotation again.  Palabos's inflate() of the finished mesh
// (helper/meshGeneratingFunctions.h:89-93) is not in the reference tree and
// is not applied.
Mesh rbc_from_sphere(int min_triangles, double radius) {
  Mesh m = merge_soup(icosphere_soup(min_triangles));
  const Euler& R = shape_rotation();
  const double C0 = 0.054322, C2 = 1.001279, C4 = -0.561381;
  for (Vec3& p : m.v) {
    p = R(p);
    double r2 = p.x * p.x + p.y * p.y;
    const int s = sgn(p.z);
    if (1 - r2 < 0) r2 = 1;
    Vec3 q = {p.x, p.y, s * std::sqrt(1 - r2) * (C0 + C2 * r2 + C4 * r2 * r2)};
    p = R(mul(q, radius));
  }
  return m;
}

// ELLIPSOID_FROM_SPHERE (helper/meshGeneratingFunctions.hh:170-183, :244-271):
// rotated unit icosphere, spherePointToEllipsoidPoint, the same rotation.
Mesh ellipsoid_from_sphere(int min_triangles, double radius, double aspect) {
  Mesh m = merge_soup(icosphere_soup(min_triangles));
  const Euler& R = shape_rotation();
  for (Vec3& p : m.v) {
    p = R(p);
    double r2 = p.x * p.x + p.y * p.y;
    const int s = sgn(p.z);
    if (1 - r2 < 0) r2 = 1;
    p = R(Vec3{p.x * radius, p.y * radius, s * aspect * radius * std::sqrt(1 - r2)});
  }
  return m;
}

std::vector<std::array<int, 2>> antipodal_pairs(const std::vector<Vec3>& v) {
  std::vector<std::array<int, 2>> out;
  double scale = 0;
  for (const Vec3& p : v) scale = std::max(scale, nrm(p));
  const double tol = 1e-9 * std::max(scale, 1.0);
  for (size_t i = 0; i < v.size(); ++i)
    for (size_t j = i + 1; j < v.size(); ++j)
      if (nrm(add(v[i], v[j])) < tol) {
        out.push_back({(int)i, (int)j});
        break;
      }
  return out;
}

std::string build_constants(TypeConstants& tc, int model, const std::vector<Vec3>& P,
                            const std::vector<std::array<int, 3>>& tris,
                            const std::vector<std::array<int, 2>>& inner) {
  tc = TypeConstants();
  tc.model = model;
  tc.nv = (int)P.size();
  tc.nf = (int)tris.size();
  tc.rest = P;
  if (tc.nv < 4 || tc.nf < 4) return "mesh too small";
  // directed edge -> triangle
  std::unordered_map<uint64_t, int> dir;
  dir.reserve(tris.size() * 4);
  auto key = [](int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
  for (int k = 0; k < tc.nf; ++k) {
    for (int c = 0; c < 3; ++c) {
      const int a = tris[k][c], b = tris[k][(c + 1) % 3];
      if (a < 0 || a >= tc.nv || b < 0 || b >= tc.nv) return "triangle index out of range";
      if (!dir.emplace(key(a, b), k).second) return "mesh is not an oriented 2-manifold";
    }
    for (int c = 0; c < 3; ++c) tc.tris.push_back(tris[k][c]);
  }
  for (const auto& d : dir) {
    const int a = (int)(d.first >> 32), b = (int)(d.first & 0xffffffffu);
    if (!dir.count(key(b, a))) return "mesh is not closed";
  }
  // edges i<j in triangle order (commonCellConstants.cpp:81-93)
  for (int k = 0; k < tc.nf; ++k) {
    const auto& t = tris[k];
    if (t[0] < t[1]) { tc.edges.push_back(t[0]); tc.edges.push_back(t[1]); }
    if (t[1] < t[2]) { tc.edges.push_back(t[1]); tc.edges.push_back(t[2]); }
    if (t[2] < t[0]) { tc.edges.push_back(t[2]); tc.edges.push_back(t[0]); }
  }
  tc.ne = (int)tc.edges.size() / 2;
  auto third = [&](int k, int a, int b) {
    for (int c = 0; c < 3; ++c)
      if (tris[k][c] != a && tris[k][c] != b) return tris[k][c];
    return -1;
  };
  for (int e = 0; e < tc.ne; ++e) {
    const int a = tc.edges[2 * e], b = tc.edges[2 * e + 1];
    tc.edge_l0.push_back(nrm(sub(P[b], P[a])));
    const int t0 = dir.at(key(b, a)), t1 = dir.at(key(a, b));
    tc.bend_tris.push_back(t0);
    tc.bend_tris.push_back(t1);
    tc.bend_outer.push_back(third(t0, a, b));
    tc.bend_outer.push_back(third(t1, a, b));
    const Vec3 V1 = unit_normal(P[tris[t0][0]], P[tris[t0][1]], P[tris[t0][2]]);
    const Vec3 V2 = unit_normal(P[tris[t1][0]], P[tris[t1][1]], P[tris[t1][2]]);
    const Vec3 ev = sub(P[b], P[a]);
    const Vec3 uv = divv(ev, nrm(ev));
    tc.edge_angle0.push_back(std::atan2(dt3(crs(V1, V2), uv), dt3(V1, V2)));
  }
  for (const auto& e : inner) {
    if (e[0] < 0 || e[0] >= tc.nv || e[1] < 0 || e[1] >= tc.nv) return "inner edge index out of range";
    tc.inner.push_back(e[0]);
    tc.inner.push_back(e[1]);
    tc.inner_l0.push_back(nrm(sub(P[e[1]], P[e[0]])));
  }
  tc.ni = (int)inner.size();
  for (int k = 0; k < tc.nf; ++k) {
    const Vec3 n = crs(sub(P[tris[k][1]], P[tris[k][0]]), sub(P[tris[k][2]], P[tris[k][0]]));
    tc.tri_a0.push_back(0.5 * nrm(n));
  }
  // volume_eq as MeshMetrics: each triangle once per corner, ascending ids per vertex
  {
    std::vector<std::vector<int>> vt(tc.nv);
    for (int k = 0; k < tc.nf; ++k)
      for (int c = 0; c < 3; ++c) vt[tris[k][c]].push_back(k);
    double vol = 0;
    for (int v = 0; v < tc.nv; ++v)
      for (int k : vt[v]) {
        const double t6 = dt3(P[tris[k][0]], crs(P[tris[k][1]], P[tris[k][2]]));
        vol += t6 / 6.0 / 3.0;
      }
    tc.volume_eq = vol;
  }
  double s = 0;
  for (double a : tc.tri_a0) s += a;
  tc.area_mean_eq = s / tc.nf;
  s = 0;
  for (double l : tc.edge_l0) s += l;
  tc.edge_mean_eq = s / tc.ne;
  s = 0;
  for (double a : tc.edge_angle0) s += a;
  tc.angle_mean_eq = s / tc.ne;
  // 1-ring: first entry from the edge list, then walk the directed edges
  tc.ring.assign(6 * tc.nv, -1);
  tc.ring_n.assign(tc.nv, 0);
  std::vector<int> first(tc.nv, -1), valence(tc.nv, 0);
  for (int e = 0; e < tc.ne; ++e) {
    const int a = tc.edges[2 * e], b = tc.edges[2 * e + 1];
    if (first[a] < 0) first[a] = b;
    if (first[b] < 0) first[b] = a;
    valence[a]++;
    valence[b]++;
  }
  for (int v = 0; v < tc.nv; ++v) {
    if (valence[v] > 6) return "vertex valence above 6 (the 1-ring holds at most 6)";
    if (valence[v] < 3) return "vertex valence below 3";
    tc.ring_n[v] = valence[v];
    int cur = first[v];
    tc.ring[6 * v] = cur;
    for (int n = 1; n < valence[v]; ++n) {
      const int k = dir.at(key(v, cur));
      cur = third(k, v, cur);
      tc.ring[6 * v + n] = cur;
    }
  }
  // per-vertex adjacency (slot j: ring neighbour ring[j], face (i, r_j, r_j+1))
  {
    std::unordered_map<uint64_t, int> eid;
    for (int e = 0; e < tc.ne; ++e) eid[key(tc.edges[2 * e], tc.edges[2 * e + 1])] = e;
    auto edge_of = [&](int a, int b) { return eid.at(a < b ? key(a, b) : key(b, a)); };
    tc.vface.assign(6 * tc.nv, -1);
    tc.vedge.assign(6 * tc.nv, -1);
    tc.vopp.assign(6 * tc.nv, -1);
    for (int v = 0; v < tc.nv; ++v) {
      const int rn = tc.ring_n[v];
      for (int j = 0; j < rn; ++j) {
        const int r = tc.ring[6 * v + j], r1 = tc.ring[6 * v + (j + 1) % rn];
        tc.vface[6 * v + j] = dir.at(key(v, r));
        tc.vedge[6 * v + j] = edge_of(v, r);
        tc.vopp[6 * v + j] = edge_of(r, r1);
      }
    }
    tc.slot_rot.assign(6 * tc.nv, 0);
    tc.slot_a0.assign(6 * tc.nv, 0.0);
    tc.slot_l0.assign(6 * tc.nv, 0.0);
    for (int v = 0; v < tc.nv; ++v)
      for (int j = 0; j < tc.ring_n[v]; ++j) {
        const int k = tc.vface[6 * v + j];
        tc.slot_rot[6 * v + j] = tris[k][0] == v ? 0 : (tris[k][1] == v ? 1 : 2);
        tc.slot_a0[6 * v + j] = tc.tri_a0[k];
        tc.slot_l0[6 * v + j] = tc.edge_l0[tc.vedge[6 * v + j]];
      }
    tc.vinner_off.assign(tc.nv + 1, 0);
    for (int e = 0; e < tc.ni; ++e) {
      tc.vinner_off[tc.inner[2 * e] + 1]++;
      tc.vinner_off[tc.inner[2 * e + 1] + 1]++;
    }
    for (int v = 0; v < tc.nv; ++v) tc.vinner_off[v + 1] += tc.vinner_off[v];
    tc.vinner.assign(tc.vinner_off[tc.nv], -1);
    std::vector<int> fill(tc.vinner_off.begin(), tc.vinner_off.end() - 1);
    for (int e = 0; e < tc.ni; ++e) {
      tc.vinner[fill[tc.inner[2 * e]]++] = e;
      tc.vinner[fill[tc.inner[2 * e + 1]]++] = e;
    }
  }
  // surface patch centre distance (commonCellConstants.cpp:284-314)
  for (int i = 0; i < tc.nv; ++i) {
    const int rn = tc.ring_n[i];
    Vec3 sum = {0, 0, 0};
    for (int j = 0; j < rn; ++j) sum = add(sum, P[tc.ring[6 * i + j]]);
    const Vec3 mid = divv(sum, (double)rn);
    const Vec3 x = P[i];
    const Vec3 dev = sub(mid, x);
    Vec3 pn = {0, 0, 0};
    for (int j = 0; j < rn; ++j) {
      Vec3 t = crs(sub(P[tc.ring[6 * i + j]], x), sub(P[tc.ring[6 * i + (j + 1) % rn]], x));
      pn = add(pn, divv(t, nrm(t)));
    }
    pn = divv(pn, nrm(pn));
    tc.patch_d0.push_back(dt3(pn, dev));
  }
  return "";
}

// loadParticles' placement of one cell (io/readPositionsBloodCells.cpp:290-361),
// in the reference's order of operations: the template is translated by minus
// its bounding-box centre (:316); meshRotation (:111-118) translates by minus
// the centre of the new bounding box, applies rotateTriangularMeshXYZ
// (:39-109: Rz * (Ry * Rx) of the column-first factors) and translates back;
// positionCellInParticleField (:120-124) adds the starting point.
void place_cell(const std::vector<Vec3>& rest, const double centre[3], const double ang[3],
                std::vector<double>& out) {
  auto bbox_mid = [](const std::vector<std::array<double, 3>>& v, double c[3], bool half_sum) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (const auto& q : v)
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], q[a]);
        hi[a] = std::max(hi[a], q[a]);
      }
    for (int a = 0; a < 3; ++a) c[a] = half_sum ? (hi[a] + lo[a]) * 0.5 : -(lo[a] + hi[a]) / 2.0;
  };
  std::vector<std::array<double, 3>> v(rest.size());
  for (size_t i = 0; i < rest.size(); ++i) v[i] = {rest[i].x, rest[i].y, rest[i].z};
  double t0[3], c2[3];
  bbox_mid(v, t0, false);
  for (auto& q : v)
    for (int a = 0; a < 3; ++a) q[a] = q[a] + t0[a];
  bbox_mid(v, c2, true);
  const double A[3][3] = {{1, 0, 0}, {0, std::cos(ang[0]), std::sin(ang[0])}, {0, -std::sin(ang[0]), std::cos(ang[0])}};
  const double B[3][3] = {{std::cos(ang[1]), 0, -std::sin(ang[1])}, {0, 1, 0}, {std::sin(ang[1]), 0, std::cos(ang[1])}};
  const double Cz[3][3] = {{std::cos(ang[2]), std::sin(ang[2]), 0}, {-std::sin(ang[2]), std::cos(ang[2]), 0}, {0, 0, 1}};
  double BA[3][3], M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      BA[i][j] = 0;
      for (int k = 0; k < 3; ++k) BA[i][j] += B[i][k] * A[k][j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      M[i][j] = 0;
      for (int k = 0; k < 3; ++k) M[i][j] += Cz[i][k] * BA[k][j];
    }
  for (const auto& p : v) {
    const double q[3] = {p[0] + -c2[0], p[1] + -c2[1], p[2] + -c2[2]};
    for (int i = 0; i < 3; ++i) {
      double r = 0;
      for (int j = 0; j < 3; ++j) r += M[i][j] * q[j];
      out.push_back(centre[i] + (r + c2[i]));
    }
  }
}

namespace {
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Nodes covered by a placed closed mesh: its vertices' nearest nodes plus
// every node inside the surface, found by scanline parity along z over the
// (x, y) columns the triangles cover.  Returns false if a non-periodic axis
// is left.
struct Raster {
  std::vector<std::pair<long, double>> hits;  // (column key, z crossing)
};

bool rasterize(const std::vector<double>& xyz, const std::vector<std::array<int, 3>>& tris, int nx, int ny, int nz,
               const int* per, std::vector<long>& nodes, Raster& R) {
  nodes.clear();
  R.hits.clear();
  const int dims[3] = {nx, ny, nz};
  bool ok = true;
  auto wrap = [&](long q, int a) -> long {
    if (q < 0 || q >= dims[a]) {
      if (per[a]) return ((q % dims[a]) + dims[a]) % dims[a];
      ok = false;
    }
    return q;
  };
  const int nv = (int)xyz.size() / 3;
  for (int i = 0; i < nv; ++i) {
    long q[3];
    for (int a = 0; a < 3; ++a) q[a] = wrap((long)std::floor(xyz[3 * i + a] + 0.5), a);
    if (!ok) return false;
    nodes.push_back(q[0] + (long)nx * (q[1] + (long)ny * q[2]));
  }
  const long OFF = 1 << 20;  // column keys of unwrapped (x, y)
  for (const auto& t : tris) {
    const double* p0 = &xyz[3 * t[0]];
    const double* p1 = &xyz[3 * t[1]];
    const double* p2 = &xyz[3 * t[2]];
    const double x0 = std::min({p0[0], p1[0], p2[0]}), x1 = std::max({p0[0], p1[0], p2[0]});
    const double y0 = std::min({p0[1], p1[1], p2[1]}), y1 = std::max({p0[1], p1[1], p2[1]});
    const double det = (p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]);
    if (std::fabs(det) < 1e-14) continue;
    for (long X = (long)std::ceil(x0); X <= (long)std::floor(x1); ++X)
      for (long Y = (long)std::ceil(y0); Y <= (long)std::floor(y1); ++Y) {
        const double px = X + 1e-7, py = Y + 2.3e-7;
        const double l1 = ((px - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (py - p0[1])) / det;
        const double l2 = ((p1[0] - p0[0]) * (py - p0[1]) - (px - p0[0]) * (p1[1] - p0[1])) / det;
        if (l1 < 0 || l2 < 0 || l1 + l2 > 1) continue;
        R.hits.push_back({(X + OFF) * (2 * OFF) + (Y + OFF), p0[2] + l1 * (p1[2] - p0[2]) + l2 * (p2[2] - p0[2])});
      }
  }
  std::sort(R.hits.begin(), R.hits.end());
  for (size_t k = 0; k + 1 < R.hits.size();) {
    size_t e = k;
    while (e < R.hits.size() && R.hits[e].first == R.hits[k].first) ++e;
    const long X = R.hits[k].first / (2 * OFF) - OFF, Y = R.hits[k].first % (2 * OFF) - OFF;
    for (size_t j = k; j + 1 < e; j += 2)
      for (long Z = (long)std::ceil(R.hits[j].second); Z <= (long)std::floor(R.hits[j + 1].second); ++Z) {
        long q[3] = {wrap(X, 0), wrap(Y, 1), wrap(Z, 2)};
        if (!ok) return false;
        nodes.push_back(q[0] + (long)nx * (q[1] + (long)ny * q[2]));
      }
    k = e;
  }
  std::sort(nodes.begin(), nodes.end());
  nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
  return true;
}

struct Packed {
  int type;
  double cen[3], ang[3];
  std::vector<long> nodes;
};

// uniform random rotation as reference-convention angles: the reference
// matrices rotate by the negated angles, Rz(c)Ry(b)Rx(a) with b = asin(2u-1)
void random_angles(SplitMix64& rng, double* ang) {
  const double a = (2 * rng.uniform() - 1) * M_PI;
  const double b = std::asin(2 * rng.uniform() - 1);
  const double g = (2 * rng.uniform() - 1) * M_PI;
  ang[0] = -a;
  ang[1] = -b;
  ang[2] = -g;
}

double gauss(SplitMix64& rng) {
  double u1 = std::max(rng.uniform(), 1e-300), u2 = rng.uniform();
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2 * M_PI * u2);
}
}  // namespace

// Seeded packing: random sequential addition (largest shapes first); a cell
// that finds no free spot within a few hundred tries is put where it
// overlaps least, and a Monte-Carlo relaxation then moves overlapping cells
// (small displacements and rotations, accepted when the overlap does not
// grow) until no node is shared.  Solid nodes dilated by `margin` are never
// entered.  Returns the number of cells placed without overlap (all of them
// on success).
int pack_cells(int nx, int ny, int nz, const int* per, const uint8_t* solid, int ntypes,
               const std::vector<Mesh>& shapes, const int* counts, double margin, unsigned long long seed,
               int max_attempts, double* centres, double* angles, int* types) {
  const long N = (long)nx * ny * nz;
  std::vector<uint8_t> blocked(N, 0);
  std::vector<uint16_t> occ(N, 0);
  const int m = (int)std::ceil(std::max(margin, 0.0));
  const int dims[3] = {nx, ny, nz};
  if (solid) {
    for (long Z = 0; Z < nz; ++Z)
      for (long Y = 0; Y < ny; ++Y)
        for (long X = 0; X < nx; ++X) {
          if (!solid[X + nx * (Y + (long)ny * Z)]) continue;
          for (int dz = -m; dz <= m; ++dz)
            for (int dy = -m; dy <= m; ++dy)
              for (int dx = -m; dx <= m; ++dx) {
                if (dx * dx + dy * dy + dz * dz > margin * margin + 1e-9) continue;
                long q[3] = {X + dx, Y + dy, Z + dz};
                bool ok = true;
                for (int a = 0; a < 3; ++a)
                  if (q[a] < 0 || q[a] >= dims[a]) {
                    if (per[a]) q[a] = (q[a] + dims[a]) % dims[a];
                    else ok = false;
                  }
                if (ok) blocked[q[0] + nx * (q[1] + (long)ny * q[2])] = 1;
              }
        }
  }
  std::vector<int> order(ntypes);
  for (int t = 0; t < ntypes; ++t) order[t] = t;
  std::vector<double> extent(ntypes, 0);
  for (int t = 0; t < ntypes; ++t)
    for (const Vec3& p : shapes[t].v) extent[t] = std::max(extent[t], std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z));
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return extent[a] > extent[b]; });
  SplitMix64 rng{seed};
  Raster R;
  std::vector<double> xyz;
  std::vector<Packed> cells;
  // candidate: returns overlap count (>=0) or -1 if invalid (wall / outside)
  auto evaluate = [&](int t, const double* cen, const double* ang, std::vector<long>& out) -> long {
    xyz.clear();
    place_cell(shapes[t].v, cen, ang, xyz);
    if (!rasterize(xyz, shapes[t].t, nx, ny, nz, per, out, R)) return -1;
    long ov = 0;
    for (long n : out) {
      if (blocked[n]) return -1;
      ov += occ[n];
    }
    return ov;
  };
  const int rsa_tries = std::max(1, std::min(max_attempts, 300));
  for (int t : order) {
    for (int c = 0; c < counts[t]; ++c) {
      Packed best;
      long best_ov = -1;
      for (int att = 0; att < rsa_tries; ++att) {
        Packed cand;
        cand.type = t;
        for (int a = 0; a < 3; ++a) cand.cen[a] = rng.uniform() * dims[a] - 0.5;
        random_angles(rng, cand.ang);
        long ov = evaluate(t, cand.cen, cand.ang, cand.nodes);
        if (ov < 0) continue;
        if (best_ov < 0 || ov < best_ov) {
          best = cand;
          best_ov = ov;
        }
        if (ov == 0) break;
      }
      if (best_ov < 0) return (int)cells.size();  // nowhere valid at all
      for (long n : best.nodes) occ[n]++;
      cells.push_back(std::move(best));
    }
  }
  // Monte-Carlo relaxation of the overlaps
  auto overlap_of = [&](const Packed& p) {
    long ov = 0;
    for (long n : p.nodes) ov += occ[n] - 1;
    return ov;
  };
  const long max_moves = (long)std::max(1, max_attempts) * (long)std::max<size_t>(cells.size(), 1);
  long moves = 0;
  std::vector<int> bad;
  while (moves < max_moves) {
    bad.clear();
    for (int i = 0; i < (int)cells.size(); ++i)
      if (overlap_of(cells[i]) > 0) bad.push_back(i);
    if (bad.empty()) break;
    for (int k = (int)bad.size() - 1; k > 0; --k) std::swap(bad[k], bad[rng.next() % (k + 1)]);
    for (int i : bad) {
      Packed& p = cells[i];
      long cur = overlap_of(p);
      if (cur == 0) continue;
      for (long n : p.nodes) occ[n]--;
      for (int tries = 0; tries < 8 && cur > 0; ++tries, ++moves) {
        Packed cand = p;
        const double step = 0.5 + 1.5 * rng.uniform();
        for (int a = 0; a < 3; ++a) cand.cen[a] = p.cen[a] + step * gauss(rng);
        if (rng.uniform() < 0.2) random_angles(rng, cand.ang);
        else
          for (int a = 0; a < 3; ++a) cand.ang[a] = p.ang[a] + 0.3 * gauss(rng);
        long ov = evaluate(p.type, cand.cen, cand.ang, cand.nodes);
        if (ov >= 0 && ov <= cur) {
          p = std::move(cand);
          cur = ov;
        }
      }
      for (long n : p.nodes) occ[n]++;
    }
  }
  int placed = 0;
  for (const Packed& p : cells) {
    if (overlap_of(p) > 0) continue;
    for (int a = 0; a < 3; ++a) {
      double c = p.cen[a];
      // keep centres inside the periodic box
      if (per[a]) c = std::fmod(std::fmod(c + 0.5, (double)dims[a]) + dims[a], (double)dims[a]) - 0.5;
      centres[3 * placed + a] = c;
      angles[3 * placed + a] = p.ang[a];
    }
    types[placed] = p.type;
    placed++;
  }
  return placed;
}

// ---------------------------------------------------------------------------
// STL geometry (helper/voxelizeDomain.cpp:74-152, getFlagMatrixFromSTL).

std::string read_stl(const std::string& path, std::vector<std::array<Vec3, 3>>& tris) {
  tris.clear();
  std::ifstream in(path, std::ios::binary);
  if (!in) return "cannot open " + path;
  std::vector<char> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  // binary: 80-byte header, uint32 count, 50 bytes per triangle
  if (data.size() >= 84) {
    uint32_t n = 0;
    std::memcpy(&n, data.data() + 80, 4);
    if (data.size() == 84 + 50 * (size_t)n) {
      for (uint32_t k = 0; k < n; ++k) {
        const char* r = data.data() + 84 + 50 * (size_t)k + 12;  // skip the normal
        std::array<Vec3, 3> t;
        for (int c = 0; c < 3; ++c) {
          float v[3];
          std::memcpy(v, r + 12 * c, 12);
          t[c] = {v[0], v[1], v[2]};
        }
        tris.push_back(t);
      }
      return "";
    }
  }
  // ASCII: "vertex x y z" lines, three per facet
  std::istringstream ss(std::string(data.begin(), data.end()));
  std::string word;
  std::vector<Vec3> verts;
  while (ss >> word) {
    if (word == "vertex") {
      Vec3 v;
      if (!(ss >> v.x >> v.y >> v.z)) return "malformed vertex in " + path;
      verts.push_back(v);
    }
  }
  if (verts.empty() || verts.size() % 3 != 0) return path + " is neither a binary nor an ASCII STL file";
  for (size_t k = 0; k < verts.size(); k += 3) tris.push_back({verts[k], verts[k + 1], verts[k + 2]});
  return "";
}

std::string voxelize(const std::vector<std::array<Vec3, 3>>& tris_in, int ref_dir, double ref_length, int margin,
                     bool open_ends, int dims[3], std::vector<uint8_t>& flags) {
  if (tris_in.empty()) return "no triangles";
  if (ref_dir < 0 || ref_dir > 2 || !(ref_length > 0) || margin < 0) return "bad voxelisation parameters";
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (const auto& t : tris_in)
    for (const auto& v : t) {
      const double c[3] = {v.x, v.y, v.z};
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], c[a]);
        hi[a] = std::max(hi[a], c[a]);
      }
    }
  const double ext = hi[ref_dir] - lo[ref_dir];
  if (!(ext > 0)) return "the mesh has no extent along the reference direction";
  // scale: the mesh spans ref_length lattice units along ref_dir; it starts
  // `margin` nodes into the lattice on every axis
  const double sc = ref_length / ext;
  for (int a = 0; a < 3; ++a) dims[a] = (int)std::ceil((hi[a] - lo[a]) * sc - 1e-9) + 1 + 2 * margin;
  const long long N = (long long)dims[0] * dims[1] * dims[2];
  if (N <= 0 || N > (1LL << 33)) return "voxelised lattice too large";
  std::vector<std::array<Vec3, 3>> tris(tris_in.size());
  for (size_t k = 0; k < tris.size(); ++k)
    for (int c = 0; c < 3; ++c)
      tris[k][c] = {(tris_in[k][c].x - lo[0]) * sc + margin, (tris_in[k][c].y - lo[1]) * sc + margin,
                    (tris_in[k][c].z - lo[2]) * sc + margin};
  // parity of crossings along +x for every (y, z) row of nodes; the row is
  // nudged off the node lattice so that it never runs through an edge
  const double ey = 1.234567e-6, ez = 2.345678e-6;
  std::vector<std::vector<int>> rows((size_t)dims[1] * dims[2]);
  for (size_t k = 0; k < tris.size(); ++k) {
    double y0 = 1e300, y1 = -1e300, z0 = 1e300, z1 = -1e300;
    for (const auto& v : tris[k]) {
      y0 = std::min(y0, v.y);
      y1 = std::max(y1, v.y);
      z0 = std::min(z0, v.z);
      z1 = std::max(z1, v.z);
    }
    for (int Z = std::max(0, (int)std::floor(z0)); Z <= std::min(dims[2] - 1, (int)std::ceil(z1)); ++Z)
      for (int Y = std::max(0, (int)std::floor(y0)); Y <= std::min(dims[1] - 1, (int)std::ceil(y1)); ++Y)
        rows[(size_t)Z * dims[1] + Y].push_back((int)k);
  }
  flags.assign(N, 1);
  std::vector<double> xs;
  for (int Z = 0; Z < dims[2]; ++Z)
    for (int Y = 0; Y < dims[1]; ++Y) {
      const double py = Y + ey, pz = Z + ez;
      xs.clear();
      for (int k : rows[(size_t)Z * dims[1] + Y]) {
        const Vec3 &A = tris[k][0], &B = tris[k][1], &C = tris[k][2];
        // barycentric coordinates of (py, pz) in the triangle's (y, z) projection
        const double d = (B.y - A.y) * (C.z - A.z) - (C.y - A.y) * (B.z - A.z);
        if (d == 0.0) continue;
        const double u = ((py - A.y) * (C.z - A.z) - (C.y - A.y) * (pz - A.z)) / d;
        const double v = ((B.y - A.y) * (pz - A.z) - (py - A.y) * (B.z - A.z)) / d;
        if (u < 0 || v < 0 || u + v > 1) continue;
        xs.push_back(A.x + u * (B.x - A.x) + v * (C.x - A.x));
      }
      std::sort(xs.begin(), xs.end());
      for (size_t k = 0; k + 1 < xs.size(); k += 2)
        for (int X = std::max(0, (int)std::ceil(xs[k])); X <= std::min(dims[0] - 1, (int)std::floor(xs[k + 1])); ++X)
          flags[X + (size_t)dims[0] * (Y + (size_t)dims[1] * Z)] = 0;
    }
  if (open_ends && dims[0] >= 3) {
    // the domain is closed: open both x ends by copying the slice next to them
    auto copy_slice = [&](int dst, int src) {
      for (int Z = 0; Z < dims[2]; ++Z)
        for (int Y = 0; Y < dims[1]; ++Y)
          flags[dst + (size_t)dims[0] * (Y + (size_t)dims[1] * Z)] = flags[src + (size_t)dims[0] * (Y + (size_t)dims[1] * Z)];
    };
    const int src0 = std::min(margin + 1, dims[0] - 1), src1 = std::max(dims[0] - 2 - margin, 0);
    for (int X = 0; X < src0; ++X) copy_slice(X, src0);
    for (int X = dims[0] - 1; X > src1; --X) copy_slice(X, src1);
  }
  return "";
}

}  // namespace hcg
